// h_rcm.cu -- REORDERING_METHOD RCM: the reverse Cuthill-McKee numbering
// that IMS computes once per matrix structure (ims_base_calc_order,
// src/Solution/LinearMethods/ImsLinearBase.f90:556-610, calling genrcm of
// src/Utilities/Libraries/rcm/rcm.f90:1003-1107), on the host beside the
// other structure work of gbims_create.  The numbering depends only on the
// pattern, and the solve's arithmetic depends on the numbering, so every
// step follows the vendored routines: the pseudo-peripheral root search
// (root_find :3121-3316 over level_set :2188-2330), the unmasked-degree
// count (degree :853-1001, the diagonal counted as IMS passes it), the
// breadth-first numbering with each node's new neighbours insertion-sorted
// by degree -- the vendored loop never compares against the first new
// neighbour -- and the reversal (rcm :2899-3120).
#include "gbims_internal.cuh"

namespace gb {
namespace {

struct RcmWork {
  const std::vector<int> &ia, &ja;
  std::vector<int> mask, deg, level, level_row;
  std::vector<char> seen;
  RcmWork(int n, const std::vector<int> &ia_, const std::vector<int> &ja_)
      : ia(ia_), ja(ja_), mask(n, 1), deg(n, 0), level(n), level_row(n + 1), seen(n, 0) {}

  // Rooted level structure of root's component (unmasked nodes); returns
  // the number of levels.  The component's mask is restored on exit.
  int level_set(int root) {
    mask[root] = 0;
    level[0] = root;
    int nl = 0, end = 0, count = 1;
    for (;;) {
      const int begin = end;
      end = count;
      level_row[nl++] = begin;
      for (int i = begin; i < end; ++i) {
        const int node = level[i];
        for (int j = ia[node]; j < ia[node + 1]; ++j) {
          const int nb = ja[j];
          if (mask[nb] != 0) {
            level[count++] = nb;
            mask[nb] = 0;
          }
        }
      }
      if (count - end <= 0) break;
    }
    level_row[nl] = end;
    for (int i = 0; i < count; ++i) mask[level[i]] = 1;
    return nl;
  }

  // A pseudo-peripheral node of root's component.
  int root_find(int root) {
    int nl = level_set(root);
    const int size = level_row[nl];
    if (nl == 1 || nl == size) return root;
    for (;;) {
      int mindeg = size;
      const int last = level_row[nl - 1];
      root = level[last];
      if (last < size - 1) {
        for (int j = last; j < size; ++j) {
          const int node = level[j];
          int d = 0;
          for (int k = ia[node]; k < ia[node + 1]; ++k)
            if (0 < mask[ja[k]]) ++d;
          if (d < mindeg) {
            root = node;
            mindeg = d;
          }
        }
      }
      const int nl2 = level_set(root);
      if (nl2 <= nl) break;
      nl = nl2;
      if (size <= nl) break;
    }
    return root;
  }

  // Numbers root's component into out[0..size) and returns its size.
  int number(int root, int *out) {
    // the component and the unmasked degree of each of its nodes
    out[0] = root;
    seen[root] = 1;
    int size = 1, end = 0;
    for (;;) {
      const int begin = end;
      end = size;
      for (int i = begin; i < end; ++i) {
        const int node = out[i];
        int d = 0;
        for (int j = ia[node]; j < ia[node + 1]; ++j) {
          const int nb = ja[j];
          if (mask[nb] != 0) {
            ++d;
            if (!seen[nb]) {
              seen[nb] = 1;
              out[size++] = nb;
            }
          }
        }
        deg[node] = d;
      }
      if (size - end == 0) break;
    }
    for (int i = 0; i < size; ++i) seen[out[i]] = 0;
    mask[root] = 0;
    if (size == 1) return 1;
    // breadth-first numbering; p(i) is the 1-based position i of the list
    auto p = [&](int i) -> int & { return out[i - 1]; };
    int lvlend = 0, lnbr = 1;
    while (lvlend < lnbr) {
      const int lbegin = lvlend + 1;
      lvlend = lnbr;
      for (int i = lbegin; i <= lvlend; ++i) {
        const int node = p(i);
        const int fnbr = lnbr + 1;
        for (int j = ia[node]; j < ia[node + 1]; ++j) {
          const int nb = ja[j];
          if (mask[nb] != 0) {
            ++lnbr;
            mask[nb] = 0;
            p(lnbr) = nb;
          }
        }
        if (lnbr <= fnbr) continue;
        for (int k = fnbr; k < lnbr;) {
          int l = k;
          ++k;
          const int nb = p(k);
          while (fnbr < l) {
            const int lp = p(l);
            if (deg[lp] <= deg[nb]) break;
            p(l + 1) = lp;
            --l;
          }
          p(l + 1) = nb;
        }
      }
    }
    for (int i = 0; i < size / 2; ++i) std::swap(out[i], out[size - 1 - i]);
    return size;
  }
};

}  // namespace

void rcm_order(int n, const std::vector<int> &ia, const std::vector<int> &ja,
               std::vector<int> &lorder) {
  lorder.assign(n, 0);
  RcmWork w(n, ia, ja);
  int placed = 0;
  for (int i = 0; i < n && placed < n; ++i) {
    if (w.mask[i] == 0) continue;
    const int root = w.root_find(i);
    placed += w.number(root, lorder.data() + placed);
  }
}

}  // namespace gb
