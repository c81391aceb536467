// k_ilut.cu -- ILUT / MILUT factorisation on the GPU.
//
// ilut (src/Utilities/Libraries/sparskit2/ilut.f90:48-462, Saad's dual
// threshold ILU with MODFLOW's relaxation of the dropped sum and its pivot
// guard) restated for one thread per row.  Row ii depends only on the U rows
// of the earlier rows it eliminates, and those are known only once its own
// elimination reaches them (fill brings new ones), so rows are not levelled
// ahead of time: every thread claims the next row from a counter and, before
// it eliminates row jrow, waits for jrow's completion word.  Rows are claimed
// in increasing order, so the lowest unfinished claimed row never waits on an
// unclaimed one and every wait ends; each wait is still bounded (kWaitCycles) and
// gives up when the attempt is void (a pivot failed, an error was raised).
//
// The working row follows the reference's bookkeeping where it decides the
// result: the elimination takes the smallest remaining column each time; the
// multipliers are kept in elimination order, the U candidates in the order
// they entered the row (the row's own upper entries in JA order, then the
// fill as it appears); dropped terms are summed in the reference's order; the
// lfil largest multipliers and the lfil - 1 largest U entries are chosen by
// the same partial quick-sort (qsplit, :519-581), whose output order is the
// storage order and so the summation order of the triangular solves.  Every
// operation is rounded on its own (no FMA), as in the CPU code.
//
// Output: per row, in padded slots (lfil L entries, lfil - 1 U entries), the
// kept columns and values, their counts and the inverse pivot.  The host
// turns the counts into the IAPC/JAPC layout of the ILU0 preconditioner and
// k_ilut_scatter moves the values there, so the level-scheduled sweeps apply
// ILUT unchanged (lusol, :465-516, is the ilu0a pair of sweeps).
#include "gbims_internal.cuh"
#include "k_llword.cuh"
#include <algorithm>
#include <climits>

namespace gb {
namespace {

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release_u32(unsigned *p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ bool attempt_void(const IlutStatus *s) {
  const volatile IlutStatus *vs = s;
  return vs->pivot_fail != INT_MAX || vs->err != 0;
}

__device__ __forceinline__ void raise_error(IlutStatus *s, int code, int row) {
  if (atomicCAS(&s->err, 0, code) == 0) atomicExch(&s->err_row, row);
}

// Waits until row r of this factorisation is complete.  False when the
// attempt became void or the wait ran out (then an error is raised).
__device__ bool wait_row(const IlutDev &I, int r) {
  if (ld_acquire_u32(I.rdone + r) == I.epoch) return true;
  const unsigned long long t0 = wclock();
  for (;;) {
    __nanosleep(64);
    if (ld_acquire_u32(I.rdone + r) == I.epoch) return true;
    if (attempt_void(I.stat)) return false;
    if (wclock() - t0 > kWaitCycles) {
      raise_error(I.stat, kIlutErrWait, r);
      return false;
    }
  }
}

// Partial quick-sort by decreasing magnitude around the ncut-th entry
// (1-based): the arrangement qsplit leaves, entry for entry.
__device__ void split_by_magnitude(int n, double *a, int *ind, int ncut) {
  int first = 0, last = n - 1;
  const int cut = ncut - 1;
  if (cut < first || cut > last) return;
  for (;;) {
    int mid = first;
    const double key = fabs(a[mid]);
    for (int j = first + 1; j <= last; ++j) {
      if (fabs(a[j]) > key) {
        ++mid;
        const double t = a[mid];
        a[mid] = a[j];
        a[j] = t;
        const int it = ind[mid];
        ind[mid] = ind[j];
        ind[j] = it;
      }
    }
    const double t = a[mid];
    a[mid] = a[first];
    a[first] = t;
    const int it = ind[mid];
    ind[mid] = ind[first];
    ind[first] = it;
    if (mid == cut) return;
    if (mid > cut) last = mid - 1;
    else first = mid + 1;
  }
}

__global__ void __launch_bounds__(128) k_ilut_factor(IlutDev I, const int *__restrict__ ia,
                                                     const int *__restrict__ ja,
                                                     const double *__restrict__ a, double droptol,
                                                     double relax, double delta, int izero) {
  // the working row: L candidates (multipliers in front, live entries after
  // the elimination cursor) and U candidates in the order they entered
  int Lc[kIlutCap], Uc[kIlutCap];
  double Lv[kIlutCap], Uv[kIlutCap];
  const int lfil = I.lfil;
  for (;;) {
    if (attempt_void(I.stat)) return;
    const unsigned long long claim = atomicAdd(&I.stat->next, 1ULL);
    if (claim >= (unsigned long long)I.n) return;
    const int row = (int)claim;
    const int j1 = ia[row], j2 = ia[row + 1];
    double tnorm = 0.0;
    for (int k = j1; k < j2; ++k) tnorm = __dadd_rn(tnorm, fabs(a[k]));
    if (tnorm == 0.0) {
      raise_error(I.stat, kIlutErrZeroRow, row);
      return;
    }
    tnorm = __ddiv_rn(tnorm, (double)(j2 - j1));
    int lenl = 0, nu = 0;
    double wd = 0.0;
    for (int j = j1; j < j2; ++j) {
      const int c = ja[j];
      const double t = a[j];
      if (c < row) {
        if (lenl == kIlutCap) { raise_error(I.stat, kIlutErrCap, row); return; }
        Lc[lenl] = c;
        Lv[lenl] = t;
        ++lenl;
      } else if (c == row) {
        wd = t;
      } else {
        if (nu == kIlutCap) { raise_error(I.stat, kIlutErrCap, row); return; }
        Uc[nu] = c;
        Uv[nu] = t;
        ++nu;
      }
    }
    double dropsum = 0.0;
    int ilen = 0;
    for (int jj = 0; jj < lenl; ++jj) {
      int jrow = Lc[jj], k = jj;
      for (int j = jj + 1; j < lenl; ++j)
        if (Lc[j] < jrow) {
          jrow = Lc[j];
          k = j;
        }
      if (k != jj) {
        Lc[k] = Lc[jj];
        Lc[jj] = jrow;
        const double s = Lv[jj];
        Lv[jj] = Lv[k];
        Lv[k] = s;
      }
      if (!wait_row(I, jrow)) return;
      const double fact = __dmul_rn(Lv[jj], __ldcg(I.dinv + jrow));
      if (fabs(fact) <= droptol) {
        dropsum = __dadd_rn(dropsum, Lv[jj]);
        continue;
      }
      const int nuj = __ldcg(I.nu + jrow);
      const size_t ub = (size_t)jrow * I.su;
      for (int q = 0; q < nuj; ++q) {
        const double s = __dmul_rn(fact, __ldcg(I.uval + ub + q));
        const int c = __ldcg(I.ucol + ub + q);
        if (c == row) {
          wd = __dsub_rn(wd, s);
        } else if (c > row) {
          int p = -1;
          for (int t = 0; t < nu; ++t)
            if (Uc[t] == c) { p = t; break; }
          if (p >= 0) {
            Uv[p] = __dsub_rn(Uv[p], s);
          } else {
            if (nu == kIlutCap) { raise_error(I.stat, kIlutErrCap, row); return; }
            Uc[nu] = c;
            Uv[nu] = -s;
            ++nu;
          }
        } else {
          // columns below jrow were eliminated already and never come back
          int p = -1;
          for (int t = jj + 1; t < lenl; ++t)
            if (Lc[t] == c) { p = t; break; }
          if (p >= 0) {
            Lv[p] = __dsub_rn(Lv[p], s);
          } else {
            if (lenl == kIlutCap) { raise_error(I.stat, kIlutErrCap, row); return; }
            Lc[lenl] = c;
            Lv[lenl] = -s;
            ++lenl;
          }
        }
      }
      Lv[ilen] = fact;
      Lc[ilen] = jrow;
      ++ilen;
    }
    // L: the lfil largest multipliers
    const int nkeep = min(ilen, lfil);
    split_by_magnitude(ilen, Lv, Lc, nkeep);
    const size_t lb = (size_t)row * I.sl;
    for (int k = 0; k < nkeep; ++k) {
      I.lcol[lb + k] = Lc[k];
      I.lval[lb + k] = Lv[k];
    }
    // U: drop below droptol x tnorm, then the lfil - 1 largest
    const double tol = __dmul_rn(droptol, tnorm);
    int m = 0;
    for (int k = 0; k < nu; ++k) {
      if (fabs(Uv[k]) > tol) {
        Uv[m] = Uv[k];
        Uc[m] = Uc[k];
        ++m;
      } else {
        dropsum = __dadd_rn(dropsum, Uv[k]);
      }
    }
    const int ulen = min(m + 1, lfil);
    split_by_magnitude(m, Uv, Uc, ulen);
    const int ukeep = ulen > 0 ? ulen - 1 : 0;
    const size_t ubr = (size_t)row * I.su;
    for (int k = 0; k < ukeep; ++k) {
      I.ucol[ubr + k] = Uc[k];
      I.uval[ubr + k] = Uv[k];
    }
    // the pivot, guarded against a sign change or zero
    double dw = __dadd_rn(__dmul_rn(__dadd_rn(1.0, delta), wd), __dmul_rn(relax, dropsum));
    if (copysign(fabs(wd), dw) != wd) {
      if (izero > 1) {
        dw = __dmul_rn(__dmul_rn(copysign(1.0, wd), __dadd_rn(1.0e-4, droptol)), tnorm);
      } else {
        atomicMin(&I.stat->pivot_fail, row);
        return;
      }
    }
    if (fabs(dw) == 0.0) {
      if (izero > 1) {
        dw = __dmul_rn(__dmul_rn(copysign(1.0, wd), __dadd_rn(1.0e-4, droptol)), tnorm);
      } else {
        atomicMin(&I.stat->pivot_fail, row);
        return;
      }
    }
    I.dinv[row] = __drcp_rn(dw);
    I.nl[row] = nkeep;
    I.nu[row] = ukeep;
    st_release_u32(I.rdone + row, I.epoch);
  }
}

// Values from the padded rows into the IAPC/JAPC/APC layout.
__global__ void k_ilut_scatter(IlutDev I, const int *__restrict__ iapc,
                               const int *__restrict__ japc, double *__restrict__ apc) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= I.n) return;
  apc[row] = I.dinv[row];
  const int l0 = iapc[row], u0 = japc[row];
  const int nl = I.nl[row], nu = I.nu[row];
  const size_t lb = (size_t)row * I.sl, ub = (size_t)row * I.su;
  for (int k = 0; k < nl; ++k) apc[l0 + k] = I.lval[lb + k];
  for (int k = 0; k < nu; ++k) apc[u0 + k] = I.uval[ub + k];
}

}  // namespace

int ilut_grid() {
  static int blocks = -1;
  if (blocks < 0) {
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_ilut_factor, 128, 0);
    blocks = std::max(1, per_sm) * kNumSM;
  }
  return blocks;
}

void launch_ilut_factor(const IlutDev &I, const int *d_ia, const int *d_ja, const double *d_amat,
                        double droptol, double relax, double delta, int izero, cudaStream_t st) {
  const int grid = std::max(1, std::min(ilut_grid(), (I.n + 127) / 128));
  k_ilut_factor<<<grid, 128, 0, st>>>(I, d_ia, d_ja, d_amat, droptol, relax, delta, izero);
}

void launch_ilut_scatter(const IlutDev &I, const int *d_iapc, const int *d_japc, double *d_apc,
                         cudaStream_t st) {
  k_ilut_scatter<<<(I.n + 255) / 256, 256, 0, st>>>(I, d_iapc, d_japc, d_apc);
}

}  // namespace gb
