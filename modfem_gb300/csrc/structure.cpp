// Host-side structure build for a mesh given to the library (the job
// sir_create does in ModFEM, sid_mkb/sis_mkb_intf.c:396-1690):
//  * DOF numbering by first appearance of each vertex over the elements in
//    order (utr_get_list_dof_ent, utd_util/uts_ls_intf.c:182-300; block ids
//    keep that order, sis_mkb_intf.c:1019);
//  * CRS rows holding every DOF that shares an element with the row DOF,
//    columns ascending with the diagonal included (sis_mkb_intf.c:1128,
//    lad_crs/las_crs_intf.c:72-300);
//  * per-element assembly tables, n*n value positions then n rhs positions
//    (lar_fill_assembly_table_int_ent_crs, las_crs_intf.c:354-438);
//  * a breadth-first first-fit colouring of the elements that share a DOF
//    (utd_util/uts_coloring.cpp:61-150) for the deterministic scatter mode.
// Multi-threaded with std::thread over row and element ranges.

#include <algorithm>
#include <thread>

#include "gbfem_internal.h"

namespace gbfem {

template <typename F>
static void parallel_for(int n, F f) {
  unsigned nt = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
  if (n < 20000) nt = 1;
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nt; t++) {
    int lo = (int)((long long)n * t / nt), hi = (int)((long long)n * (t + 1) / nt);
    th.emplace_back([=]() { f(lo, hi); });
  }
  for (auto &x : th) x.join();
}

int build_host_structure(int nno, int nel, int nv, const int *el_nodes, int nfa, const int *fa_el,
                         const int *fa_side, HostStructure &hs) {
  (void)nfa; (void)fa_el; (void)fa_side;
  // 1. first-appearance DOF order
  hs.dof_of_node.assign(nno, -1);
  int nd = 0;
  for (long long i = 0; i < (long long)nel * nv; i++) {
    int n = el_nodes[i];
    if (n < 0 || n >= nno) {
      set_error("element vertex index out of range");
      return -2;
    }
    if (hs.dof_of_node[n] < 0) hs.dof_of_node[n] = nd++;
  }
  hs.ndof = nd;
  std::vector<int> el_dofs((size_t)nel * nv);
  for (size_t i = 0; i < el_dofs.size(); i++) el_dofs[i] = hs.dof_of_node[el_nodes[i]];

  // 2. dof -> element incidence
  std::vector<int> inc_ptr(nd + 1, 0);
  for (int d : el_dofs) inc_ptr[d + 1]++;
  for (int r = 0; r < nd; r++) inc_ptr[r + 1] += inc_ptr[r];
  std::vector<int> inc(inc_ptr[nd]);
  {
    std::vector<int> fill(inc_ptr.begin(), inc_ptr.end() - 1);
    for (int e = 0; e < nel; e++)
      for (int j = 0; j < nv; j++) inc[fill[el_dofs[(size_t)e * nv + j]]++] = e;
  }

  // 3. CRS rows (count, then fill), each thread with its own scratch
  hs.row_ptr.assign(nd + 1, 0);
  auto row_cols = [&](int r, std::vector<int> &tmp) {
    tmp.clear();
    for (int k = inc_ptr[r]; k < inc_ptr[r + 1]; k++) {
      const int *ed = &el_dofs[(size_t)inc[k] * nv];
      for (int j = 0; j < nv; j++) tmp.push_back(ed[j]);
    }
    std::sort(tmp.begin(), tmp.end());
    tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
  };
  std::vector<int> rowlen(nd);
  parallel_for(nd, [&](int lo, int hi) {
    std::vector<int> tmp;
    for (int r = lo; r < hi; r++) {
      row_cols(r, tmp);
      rowlen[r] = (int)tmp.size();
    }
  });
  long long nnz = 0;
  for (int r = 0; r < nd; r++) {
    hs.row_ptr[r] = (int)nnz;
    nnz += rowlen[r];
  }
  if (nnz > 2147483647LL) {
    set_error("matrix too large for 32-bit CRS indices");
    return -2;
  }
  hs.row_ptr[nd] = (int)nnz;
  hs.col_ind.assign(nnz, 0);
  parallel_for(nd, [&](int lo, int hi) {
    std::vector<int> tmp;
    for (int r = lo; r < hi; r++) {
      row_cols(r, tmp);
      std::copy(tmp.begin(), tmp.end(), hs.col_ind.begin() + hs.row_ptr[r]);
    }
  });

  // 4. element tables
  const int tl = nv * nv + nv;
  hs.el_table.assign((size_t)nel * tl, 0);
  parallel_for(nel, [&](int lo, int hi) {
    for (int e = lo; e < hi; e++) {
      const int *ed = &el_dofs[(size_t)e * nv];
      int *t = &hs.el_table[(size_t)e * tl];
      for (int j = 0; j < nv; j++) {
        const int r = ed[j];
        const int *b = hs.col_ind.data() + hs.row_ptr[r], *en = hs.col_ind.data() + hs.row_ptr[r + 1];
        for (int i = 0; i < nv; i++) t[j + i * nv] = (int)(std::lower_bound(b, en, ed[i]) - hs.col_ind.data());
        t[nv * nv + j] = r;
      }
    }
  });

  // 5. colourings: elements sharing a dof; boundary faces through the dofs of
  //    their element (a superset of the face's own dofs)
  color_entities(nel, nv, el_dofs, nd, hs.el_color_ptr, hs.el_perm);
  std::vector<int> fa_dofs((size_t)nfa * nv);
  for (int f = 0; f < nfa; f++)
    for (int j = 0; j < nv; j++) fa_dofs[(size_t)f * nv + j] = el_dofs[(size_t)fa_el[f] * nv + j];
  color_entities(nfa, nv, fa_dofs, nd, hs.fa_color_ptr, hs.fa_perm);
  return 0;
}

// Breadth-first first-fit colouring (utd_util/uts_coloring.cpp:61-150):
// entities sharing a dof are neighbours; each entity taken from the front of
// the breadth-first walk gets the smallest colour unused by its coloured
// neighbours.  Returns colour ranges over a permutation of the entities.
void color_entities(int nent, int nv, const std::vector<int> &ent_dofs, int nd, std::vector<int> &color_ptr,
                    std::vector<int> &perm) {
  std::vector<int> inc_ptr(nd + 1, 0);
  for (int d : ent_dofs) inc_ptr[d + 1]++;
  for (int r = 0; r < nd; r++) inc_ptr[r + 1] += inc_ptr[r];
  std::vector<int> inc(inc_ptr[nd]);
  {
    std::vector<int> fill(inc_ptr.begin(), inc_ptr.end() - 1);
    for (int e = 0; e < nent; e++)
      for (int j = 0; j < nv; j++) inc[fill[ent_dofs[(size_t)e * nv + j]]++] = e;
  }
  std::vector<int> color(nent, -1), queue;
  queue.reserve(nent);
  std::vector<char> seen(nent, 0);
  std::vector<int> used(64, -1);
  int ncol = 0, start = 0, done = 0;
  size_t qh = 0;
  while (done < nent) {
    if (qh == queue.size()) {
      while (start < nent && color[start] >= 0) start++;
      if (start >= nent) break;
      queue.push_back(start);
      seen[start] = 1;
    }
    const int cur = queue[qh++];
    for (int j = 0; j < nv; j++) {
      const int d = ent_dofs[(size_t)cur * nv + j];
      for (int k = inc_ptr[d]; k < inc_ptr[d + 1]; k++) {
        const int nb = inc[k];
        if (nb == cur) continue;
        if (color[nb] >= 0) used[color[nb]] = cur;
        if (!seen[nb]) {
          seen[nb] = 1;
          queue.push_back(nb);
        }
      }
    }
    int c = 0;
    while (c < ncol && used[c] == cur) c++;
    if (c == ncol) {
      ncol++;
      if (ncol >= (int)used.size()) used.resize(used.size() * 2, -1);
    }
    color[cur] = c;
    done++;
  }
  color_ptr.assign(ncol + 1, 0);
  for (int e = 0; e < nent; e++) color_ptr[color[e] + 1]++;
  for (int c = 0; c < ncol; c++) color_ptr[c + 1] += color_ptr[c];
  perm.assign(nent, 0);
  std::vector<int> fill(color_ptr.begin(), color_ptr.end() - 1);
  for (int e = 0; e < nent; e++) perm[fill[color[e]]++] = e;
}

}  // namespace gbfem
