// k_xt3d.cuh -- the arithmetic of XT3D (Xt3dInterface.f90, Xt3dAlgorithm.f90)
// on the device: the connection geometry of a cell and its neighbours
// (xt3d_load), the local (c, d, e) frame of a connection (getrot), the
// weights of the neighbouring connections (abwts), the one-sided flux
// coefficients (abhats) and their blend into the "conductances" of the
// connection (qconds).
//
// Every operation is rounded on its own (__dadd_rn, __dmul_rn, __ddiv_rn,
// __dsqrt_rn; no FMA) and every sum keeps the reference's order, so the
// coefficients are bit for bit those of the Fortran compiled without
// contraction.  A neighbour slot holds its cell number, or -1 for an
// inactive neighbour (the Fortran's 0).
#pragma once
#include "k_gwf.cuh"

namespace gb {

#define XADD __dadd_rn
#define XSUB __dsub_rn
#define XMUL __dmul_rn
#define XDIV __ddiv_rn

struct XtCell {
  int nnbr;
  bool allhc;                 // every active connection horizontal
  int nb[kXtNb];
  double vc[kXtNb][3];        // unit vector from the cell to the neighbour's centre
  double vn[kXtNb][3];        // unit normal of the shared face
  double dl[kXtNb], dln[kXtNb];
};

// xt3d_load (Xt3dInterface.f90:1211-1275) with the grid's connection_normal
// and connection_vector (Dis.f90:1039-1160, Disv.f90:979-1080,
// Disu.f90:1062-1164; line_unit_vector DisvGeom.f90:473-496); the
// displacements and normals come from x.geo
__device__ inline void xt_load(const NpfDev &g, const Xt3dDev &x, const int *ibound,
                               const double *sat, int n, XtCell &c) {
  c.nnbr = g.ia[n + 1] - g.ia[n] - 1;
  c.allhc = true;
  for (int il = 0; il < c.nnbr; ++il) {
    const int ii = g.ia[n] + 1 + il;
    const int jj = g.ja[ii], jjs = g.jas[ii];
    if (ibound[jj] == 0) {
      c.nb[il] = -1;
      continue;
    }
    c.nb[il] = jj;
    const int ihc = g.ihc[jjs];
    double dltot;
    if (ihc == 0) {
      const double z = (jj < n) ? 1.0 : -1.0;
      c.vn[il][0] = 0.0;
      c.vn[il][1] = 0.0;
      c.vn[il][2] = z;
      const double z1 = XADD(g.bot[n], XMUL(0.5, XSUB(g.top[n], g.bot[n])));
      const double z2 = XADD(g.bot[jj], XMUL(0.5, XSUB(g.top[jj], g.bot[jj])));
      if (x.vcentre) {
        // DISU: between the cell centres (line_unit_vector)
        const double *gg = x.geo + 8 * (size_t)jjs + ((jj > n) ? 0 : 4);
        const double dx = gg[0], dy = gg[1], dz = XSUB(z2, z1);
        const double vmag = __dsqrt_rn(XADD(XADD(XMUL(dx, dx), XMUL(dy, dy)), XMUL(dz, dz)));
        c.vc[il][0] = XDIV(dx, vmag);
        c.vc[il][1] = XDIV(dy, vmag);
        c.vc[il][2] = XDIV(dz, vmag);
        dltot = vmag;
      } else {
        c.vc[il][0] = 0.0;
        c.vc[il][1] = 0.0;
        c.vc[il][2] = z;
        dltot = fabs(XSUB(z2, z1));
      }
    } else {
      // x.geo: per connection n < m, from n to m then from m to n
      const double *gg = x.geo + 8 * (size_t)jjs + ((jj > n) ? 0 : 4);
      const double dx = gg[0], dy = gg[1];
      c.vn[il][0] = gg[2];
      c.vn[il][1] = gg[3];
      c.vn[il][2] = 0.0;
      double z1 = 0.0, z2 = 0.0;
      if (!x.nozee) {
        z1 = XADD(g.bot[n], XMUL(XMUL(0.5, sat[n]), XSUB(g.top[n], g.bot[n])));
        z2 = XADD(g.bot[jj], XMUL(XMUL(0.5, sat[jj]), XSUB(g.top[jj], g.bot[jj])));
      }
      const double dz = XSUB(z2, z1);
      const double vmag = __dsqrt_rn(XADD(XADD(XMUL(dx, dx), XMUL(dy, dy)), XMUL(dz, dz)));
      c.vc[il][0] = XDIV(dx, vmag);
      c.vc[il][1] = XDIV(dy, vmag);
      c.vc[il][2] = XDIV(dz, vmag);
      dltot = vmag;
    }
    double cl1n, cl2n;
    if (jj > n) {
      cl1n = g.cl1[jjs];
      cl2n = g.cl2[jjs];
    } else {
      cl1n = g.cl2[jjs];
      cl2n = g.cl1[jjs];
    }
    const double oo = XDIV(1.0, XADD(cl1n, cl2n));
    c.dl[il] = XMUL(XMUL(dltot, cl1n), oo);
    c.dln[il] = XMUL(XMUL(dltot, cl2n), oo);
    if (ihc == 0) c.allhc = false;
  }
}

// getrot (Xt3dAlgorithm.f90:283-357); returns iml0 (-1: none)
__device__ inline int xt_getrot(const XtCell &c, int il01, double r[3][3]) {
  const double vcc[3] = {c.vc[il01][0], c.vc[il01][1], c.vc[il01][2]};
  double acmpmn = 1.0 - 1e-10, cmpmn = 0.0;
  int iml0 = -1;
  for (int il = 0; il < c.nnbr; ++il) {
    if (il == il01 || c.nb[il] < 0) continue;
    const double cmp =
        XADD(XADD(XMUL(c.vc[il][0], vcc[0]), XMUL(c.vc[il][1], vcc[1])), XMUL(c.vc[il][2], vcc[2]));
    const double acmp = fabs(cmp);
    if (acmp < acmpmn) {
      cmpmn = cmp;
      acmpmn = acmp;
      iml0 = il;
    }
  }
  if (iml0 < 0) {
    for (int i = 0; i < 3; ++i) r[i][0] = vcc[i];
    return -1;
  }
  double vcd[3], vce[3];
  for (int i = 0; i < 3; ++i) vcd[i] = XSUB(c.vc[iml0][i], XMUL(cmpmn, vcc[i]));
  const double s = __dsqrt_rn(XSUB(1.0, XMUL(cmpmn, cmpmn)));
  for (int i = 0; i < 3; ++i) vcd[i] = XDIV(vcd[i], s);
  vce[0] = XSUB(XMUL(vcc[1], vcd[2]), XMUL(vcc[2], vcd[1]));
  vce[1] = XSUB(XMUL(vcc[2], vcd[0]), XMUL(vcc[0], vcd[2]));
  vce[2] = XSUB(XMUL(vcc[0], vcd[1]), XMUL(vcc[1], vcd[0]));
  for (int i = 0; i < 3; ++i) {
    r[i][0] = vcc[i];
    r[i][1] = vcd[i];
    r[i][2] = vce[i];
  }
  return iml0;
}

// abwts (Xt3dAlgorithm.f90:389-490); nde1 1 (d) or 2 (e), 0-based
__device__ inline void xt_abwts(const XtCell &c, int il01, int nde1, const double vccde[][3],
                                double vcthresh, double &acd, double &add, double &aed,
                                double *bd) {
  const int nde2 = 3 - nde1;
  double omwt[kXtNb];
  double dsum = 0.0, vcmx = 0.0;
  for (int il = 0; il < c.nnbr; ++il) omwt[il] = 0.0;
  for (int il = 0; il < c.nnbr; ++il) {
    if (il == il01 || c.nb[il] < 0) continue;
    const double a = fabs(vccde[il][nde1]);
    vcmx = (a > vcmx) ? a : vcmx;
    const double dlm = XMUL(0.5, XADD(c.dl[il], c.dln[il]));
    const double cosang = vccde[il][0];
    const double dl4wt =
        __dsqrt_rn(XSUB(XADD(XMUL(dlm, dlm), XMUL(c.dl[il01], c.dl[il01])),
                        XMUL(XMUL(XMUL(2.0, dlm), c.dl[il01]), cosang)));
    omwt[il] = XMUL(fabs(vccde[il][nde1]), dl4wt);
    dsum = XADD(dsum, omwt[il]);
  }
  dsum = XADD(dsum, XMUL(1e-10, dsum));
  for (int il = 0; il < c.nnbr; ++il) {
    if (il == il01 || c.nb[il] < 0) continue;
    const double fact = XSUB(dsum, omwt[il]);
    omwt[il] = XMUL(fact, fabs(vccde[il][nde1]));
  }
  for (int il = 0; il < c.nnbr; ++il) bd[il] = 0.0;
  dsum = 0.0;
  for (int il = 0; il < c.nnbr; ++il) {
    if (il == il01 || c.nb[il] < 0) continue;
    bd[il] = XMUL(omwt[il], copysign(1.0, vccde[il][nde1]));
    dsum = XADD(dsum, XMUL(omwt[il], fabs(vccde[il][nde1])));
  }
  const double oodsum = XDIV(1.0, dsum);
  for (int il = 0; il < c.nnbr; ++il) {
    if (il == il01 || c.nb[il] < 0) continue;
    bd[il] = XMUL(bd[il], oodsum);
  }
  add = 1.0;
  acd = 0.0;
  aed = 0.0;
  for (int il = 0; il < c.nnbr; ++il) {
    if (il == il01 || c.nb[il] < 0) continue;
    acd = XADD(acd, XMUL(bd[il], vccde[il][0]));
    aed = XADD(aed, XMUL(bd[il], vccde[il][nde2]));
  }
  if (vcmx < vcthresh) {
    const double fatten = XDIV(vcmx, vcthresh);
    acd = XMUL(acd, fatten);
    aed = XMUL(aed, fatten);
    for (int il = 0; il < c.nnbr; ++il) bd[il] = XMUL(bd[il], fatten);
  }
}

// abhats (Xt3dAlgorithm.f90:127-272); bhat has kXtNb entries
__device__ inline void xt_abhats(const XtCell &c, int il01, const double *ck, double vcthresh,
                                 double ar01, double &ahat, double *bhat) {
  double rmat[3][3];
  const int iml0 = xt_getrot(c, il01, rmat);
  for (int il = 0; il < kXtNb; ++il) bhat[il] = 0.0;
  if (iml0 < 0) {
    double w[3];
    for (int i = 0; i < 3; ++i) {
      double s = 0.0;
      for (int k = 0; k < 3; ++k) s = XADD(s, XMUL(ck[3 * i + k], rmat[k][0]));
      w[i] = s;
    }
    double sigma1 = 0.0;
    for (int i = 0; i < 3; ++i) sigma1 = XADD(sigma1, XMUL(c.vn[il01][i], w[i]));
    ahat = XDIV(sigma1, c.dl[il01]);
  } else {
    double vccde[kXtNb][3];
    for (int il = 0; il < c.nnbr; ++il)
      for (int j = 0; j < 3; ++j) {
        double s = 0.0;
        for (int i = 0; i < 3; ++i) s = XADD(s, XMUL(rmat[i][j], c.vc[il][i]));
        vccde[il][j] = s;
      }
    double acd, add, aed, bd[kXtNb];
    xt_abwts(c, il01, 1, vccde, vcthresh, acd, add, aed, bd);
    double ace = 0.0, aee = 1.0, ade = 0.0, be[kXtNb];
    bool zero_e = true;
    if (!c.allhc) {
      bool iscomp = false;
      for (int il = 0; il < c.nnbr; ++il) {
        if (il == il01 || c.nb[il] < 0) continue;
        if (fabs(vccde[il][2]) > 1e-10) {
          iscomp = true;
          break;
        }
      }
      if (iscomp) {
        xt_abwts(c, il01, 2, vccde, vcthresh, ace, aee, ade, be);
        zero_e = false;
      }
    }
    if (zero_e) {
      ace = 0.0;
      aee = 1.0;
      ade = 0.0;
      for (int il = 0; il < c.nnbr; ++il) be[il] = 0.0;
    }
    const double determ = XSUB(XMUL(add, aee), XMUL(ade, aed));
    const double oodet = XDIV(1.0, determ);
    const double alphad = XMUL(XSUB(XMUL(acd, aee), XMUL(ace, aed)), oodet);
    const double alphae = XMUL(XSUB(XMUL(ace, add), XMUL(acd, ade)), oodet);
    double cr[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double s = 0.0;
        for (int k = 0; k < 3; ++k) s = XADD(s, XMUL(ck[3 * i + k], rmat[k][j]));
        cr[i][j] = s;
      }
    double sigma[3];
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int i = 0; i < 3; ++i) s = XADD(s, XMUL(c.vn[il01][i], cr[i][j]));
      sigma[j] = s;
    }
    ahat = XDIV(XSUB(XSUB(sigma[0], XMUL(sigma[1], alphad)), XMUL(sigma[2], alphae)), c.dl[il01]);
    for (int il = 0; il < c.nnbr; ++il) {
      if (il == il01 || c.nb[il] < 0) continue;
      const double betad = XMUL(XSUB(XMUL(bd[il], aee), XMUL(be[il], aed)), oodet);
      const double betae = XMUL(XSUB(XMUL(be[il], add), XMUL(bd[il], ade)), oodet);
      const double dl0il = XADD(c.dl[il], c.dln[il]);
      bhat[il] = XDIV(XADD(XMUL(sigma[1], betad), XMUL(sigma[2], betae)), dl0il);
    }
    bhat[il01] = 0.0;
  }
  ahat = XMUL(ahat, ar01);
  for (int il = 0; il < c.nnbr; ++il) bhat[il] = XMUL(bhat[il], ar01);
}

// qconds (Xt3dAlgorithm.f90:47-121); chati0 and chat1j have kXtNb entries
__device__ inline void xt_qconds(const XtCell &c0, int il01, const double *ck0, const XtCell &c1,
                                 int il10, const double *ck1, double ar01, double ar10,
                                 double vcthresh, double &chat01, double *chati0,
                                 double *chat1j) {
  if (ar01 == 0.0) {
    chat01 = 0.0;
    for (int i = 0; i < kXtNb; ++i) {
      chati0[i] = 0.0;
      chat1j[i] = 0.0;
    }
    return;
  }
  double ahat0, ahat1, bhat0[kXtNb], bhat1[kXtNb];
  xt_abhats(c0, il01, ck0, vcthresh, ar01, ahat0, bhat0);
  xt_abhats(c1, il10, ck1, vcthresh, ar10, ahat1, bhat1);
  const double denom = XADD(ahat0, ahat1);
  const double wght1 = (fabs(denom) > 2.220446049250313e-16) ? XDIV(ahat0, XADD(ahat0, ahat1)) : 1.0;
  const double wght0 = XSUB(1.0, wght1);
  chat01 = XMUL(wght1, ahat1);
  for (int i = 0; i < kXtNb; ++i) {
    chati0[i] = XMUL(wght0, bhat0[i]);
    chat1j[i] = XMUL(wght1, bhat1[i]);
  }
}

// position of column col in solution row r (sia[r]-relative), or -1
__device__ __forceinline__ int xt_pos(const Xt3dDev &x, int s0, int len, int col) {
  for (int k = 0; k < len; ++k)
    if (x.sja[s0 + k] == col) return k;
  return -1;
}

}  // namespace gb
