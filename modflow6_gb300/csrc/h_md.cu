// h_md.cu -- REORDERING_METHOD MD: the minimum-degree numbering IMS takes
// from the Yale sparse matrix package (ims_odrv with path 1,
// src/Solution/LinearMethods/ImsReordering.f90:7-772: md, mdi, mdm, mdp,
// mdu), on the host once per matrix structure.  As in the package, the
// quotient graph lives in two linked arrays v/l: v(1:n) holds each vertex's
// mark and v(n+1:) the list entries; last/next encode the degree lists
// (last < 0: head of the list of degree -last), an eliminated vertex's
// order (next = -k) and, for elements, their list length (last).  The work
// length is the one IMS gives, nsp = 3 NEQ + 4 NJA (ImsLinearBase.f90:585).
// Indices are 1-based inside (0 is the null link).
#include "gbims_internal.cuh"

namespace gb {
namespace {

struct MdWork {
  int n, mmax;
  std::vector<int> v, l, head, last, next;
  int *mark;         // v(1:n)
  bool bad = false;  // a degree out of range (malformed input)
  MdWork(int n_, int mmax_)
      : n(n_), mmax(mmax_), v(mmax_ + 1, 0), l(mmax_ + 1, 0), head(2 * n_ + 2, 0),
        last(n_ + 1, 0), next(n_ + 1, 0), mark(v.data()) {}

  // mdi: vertex lists of the symmetric pattern, then the degree lists.
  int init(const std::vector<int> &ia, const std::vector<int> &ja) {
    for (int u = 1; u <= n; ++u) {
      mark[u] = 1;
      l[u] = 0;
      head[u] = 0;
    }
    int sfs = n + 1;
    for (int u = 1; u <= n; ++u) {
      for (int j = ia[u - 1]; j < ia[u]; ++j) {
        const int w = ja[j] + 1;
        if (w == u) continue;
        bool known = false;
        if (w < u) {  // already linked from w's own row?
          int p = u;
          for (int c = mark[u] - 1; c > 0; --c) {
            p = l[p];
            if (v[p] == w) {
              known = true;
              break;
            }
          }
        }
        if (known) continue;
        if (sfs >= mmax) return 9 * n + u;
        ++mark[u];
        v[sfs] = w;
        l[sfs] = l[u];
        l[u] = sfs++;
        ++mark[w];
        v[sfs] = u;
        l[sfs] = l[w];
        l[w] = sfs++;
      }
    }
    for (int u = 1; u <= n; ++u) {
      const int d = mark[u];
      next[u] = head[d];
      head[d] = u;
      last[u] = -d;
      if (next[u] > 0) last[next[u]] = u;
      mark[u] = 0;
    }
    return 0;
  }

  // mdm: the uneliminated vertices reachable from the new element ek,
  // directly or through the elements it absorbs, chained from ek.
  int merge(int ek) {
    const int tag = mark[ek];
    int tail = ek;
    for (int s = l[ek]; s != 0;) {
      const int cur = s;
      s = l[cur];
      const int w = v[cur];
      if (next[w] >= 0) {
        mark[w] = tag;
        l[tail] = cur;
        tail = cur;
        continue;
      }
      int b = l[w];
      for (int c = last[w]; c > 0; --c) {
        const int nb = b;
        b = l[nb];
        const int vb = v[nb];
        if (mark[vb] >= tag) continue;
        mark[vb] = tag;
        l[tail] = nb;
        tail = nb;
      }
      mark[w] = tag;
    }
    l[tail] = 0;
    return tail;
  }

  // mdp: takes the reachable vertices off their degree lists, drops the
  // absorbed elements from their lists, eliminates those left with no
  // element but ek, and flags the ones whose only other element is single.
  void purge(int &k, int ek, int tail) {
    const int tag = mark[ek];
    int li = ek, freed = 0;
    for (int c = last[ek]; c > 0; --c) {
      const int i = li;
      li = l[i];
      const int w = v[li];
      if (last[w] != 0) {
        if (last[w] > 0) next[last[w]] = next[w];
        else head[-last[w]] = next[w];
        if (next[w] > 0) last[next[w]] = last[w];
      }
      for (int s = w, ls = l[s]; ls != 0; ls = l[s]) {
        if (mark[v[ls]] >= tag) {
          freed = ls;
          l[s] = l[ls];
        } else {
          s = ls;
        }
      }
      const int lw = l[w];
      if (lw == 0) {
        l[i] = l[li];
        li = i;
        next[w] = -(++k);
        --last[ek];
        continue;
      }
      const int ew = v[lw];
      if (l[lw] == 0 && next[ew] < 0) {
        if (mark[ew] >= 0) {
          last[w] = ew;
          mark[ew] = -1;
          l[tail] = li;
          tail = li;
          l[i] = l[li];
          li = i;
        } else {
          last[w] = 0;
          --mark[ew];
        }
      } else {
        last[w] = -ek;
      }
      v[freed] = ek;
      l[freed] = l[w];
      l[w] = freed;
    }
    l[tail] = 0;
  }

  // mdu: external degrees of the reachable vertices, back onto the lists.
  void update(int ek, int &dmin) {
    int tag = mark[ek] - last[ek];
    int i = ek;
    for (int c = last[ek]; c > 0; --c) {
      i = l[i];
      const int w = v[i];
      if (last[w] == 0) continue;
      int d;
      if (last[w] > 0) {
        const int e = last[w];
        d = last[ek] + last[e] + mark[e];
        mark[e] = 0;
      } else {
        ++tag;
        d = last[ek];
        bool outmatched = false;
        for (int s = l[l[w]]; s != 0; s = l[s]) {
          const int x = v[s];
          if (next[x] >= 0) {
            mark[x] = tag;
            ++d;
            continue;
          }
          if (mark[x] < 0) {
            last[w] = 0;
            --mark[x];
            for (int t = l[s]; t != 0; t = l[t])
              if (mark[v[t]] < 0) --mark[v[t]];
            outmatched = true;
            break;
          }
          int b = x;
          for (int cb = last[x]; cb > 0; --cb) {
            b = l[b];
            const int vb = v[b];
            if (mark[vb] >= tag) continue;
            mark[vb] = tag;
            ++d;
          }
        }
        if (outmatched) continue;
      }
      if (d < 1 || d > 2 * n) {  // a degree no quotient graph of n nodes has
        bad = true;
        return;
      }
      next[w] = head[d];
      head[d] = w;
      last[w] = -d;
      if (next[w] > 0) last[next[w]] = w;
      if (d < dmin) dmin = d;
    }
  }
};

}  // namespace

int md_order(int n, const std::vector<int> &ia, const std::vector<int> &ja,
             std::vector<int> &lorder) {
  lorder.assign(n, 0);
  const long long nsp = 3LL * n + 4LL * ia[n];
  const long long mmax = (nsp - n) / 2;
  if (mmax < n) return 10 * n + 1;
  if (mmax > INT_MAX - 1) return 9 * n + 1;
  MdWork W(n, (int)mmax);
  if (int flag = W.init(ia, ja)) return flag;
  int k = 0, dmin = 1, tag = 0;
  while (k < n) {
    while (dmin < 2 * n + 1 && W.head[dmin] <= 0) ++dmin;
    if (W.head[dmin] <= 0) return 8 * n + 1;  // no vertex left on any degree list
    const int ek = W.head[dmin];
    W.head[dmin] = W.next[ek];
    if (W.head[dmin] > 0) W.last[W.head[dmin]] = -dmin;
    W.next[ek] = -(++k);
    W.last[ek] = dmin - 1;
    tag += W.last[ek];
    W.mark[ek] = tag;
    const int tail = W.merge(ek);
    W.purge(k, ek, tail);
    W.update(ek, dmin);
    if (W.bad) return 8 * n + 2;
  }
  for (int u = 1; u <= n; ++u) lorder[-W.next[u] - 1] = u - 1;
  return 0;
}

}  // namespace gb
