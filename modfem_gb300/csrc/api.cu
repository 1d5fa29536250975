// C ABI of libmodfem_gb300 (declared in include/modfem_gb300.h).

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <chrono>
#include <functional>
#include <mutex>

#include "gbfem_internal.h"

namespace gbfem {
static thread_local std::string g_err;
void set_error(const std::string &msg) { g_err = msg; }
}  // namespace gbfem

using gbfem::DevBuf;
using gbfem::set_error;


template <typename T>
static int upload(gbfem_ctx c, DevBuf<T> &d, const T *h, size_t n) {
  GB_TRY(d.alloc(n));
  if (n) GB_CUDA(cudaMemcpyAsync(d.p, h, n * sizeof(T), cudaMemcpyHostToDevice, c->stream));
  return 0;
}

// Pieces of a coordinate (b = 0) or coefficient (b = 1) upload: up_stream
// first waits for the work queued on the context stream (which may still
// read the old values), then copies nitems x width doubles in 8 pieces with
// an event after each.
static int piece_upload(gbfem_ctx c, int b, double *dst, const double *src, long long nitems, int width) {
  if (!c->up_stream) {
    GB_CUDA(cudaStreamCreateWithFlags(&c->up_stream, cudaStreamNonBlocking));
    GB_CUDA(cudaEventCreateWithFlags(&c->up_now, cudaEventDisableTiming));
    for (auto &row : c->up_ev)
      for (auto &ev : row) GB_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  }
  GB_CUDA(cudaEventRecord(c->up_now, c->stream));
  GB_CUDA(cudaStreamWaitEvent(c->up_stream, c->up_now, 0));
  const int P = 8;
  const long long per = std::max(1LL, (nitems + P - 1) / P);
  for (int p = 0; p < P; p++) {
    const long long lo = std::min(nitems, p * per), hi = std::min(nitems, lo + per);
    if (hi > lo)
      GB_CUDA(cudaMemcpyAsync(dst + lo * width, src + lo * width, (size_t)(hi - lo) * width * sizeof(double),
                              cudaMemcpyHostToDevice, c->up_stream));
    GB_CUDA(cudaEventRecord(c->up_ev[b][p], c->up_stream));
  }
  c->up_np[b] = P;
  c->up_per[b] = per;
  c->up_pending = true;
  return 0;
}

// The context stream waits for every piece still in flight.
static int settle_uploads(gbfem_ctx c) {
  if (!c->up_pending) return 0;
  for (int b = 0; b < 2; b++)
    if (c->up_np[b] > 0) GB_CUDA(cudaStreamWaitEvent(c->stream, c->up_ev[b][c->up_np[b] - 1], 0));
  c->up_np[0] = c->up_np[1] = 0;
  c->up_pending = false;
  return 0;
}

// Before a buffer the pieces write is freed or reallocated: they are done.
static int drain_uploads(gbfem_ctx c) {
  GB_TRY(settle_uploads(c));
  if (c->up_stream) GB_CUDA(cudaStreamSynchronize(c->up_stream));
  return 0;
}

static const int kDgNs[5] = {0, 6, 18, 40, 75};
static const int kDgTetNs[5] = {0, 4, 10, 20, 35};
static inline bool el_is_tet(gbfem_ctx c, int e) { return c->mixed ? c->h_el_tet[e] != 0 : c->nv == GBFEM_TETRA; }
static inline int el_nverts(gbfem_ctx c, int e) { return el_is_tet(c, e) ? 4 : 6; }
// functions of DG element e: tensor basis on prisms, complete basis on
// tetrahedra
static inline int dg_ns_el(gbfem_ctx c, int e) {
  return el_is_tet(c, e) ? kDgTetNs[c->dg_p[e]] : kDgNs[c->dg_p[e]];
}
// element class of the DG kernels: 1..4 prisms of degree p, 5..8 tetrahedra
static inline int dg_cls(gbfem_ctx c, int e) { return c->dg_p[e] + (el_is_tet(c, e) ? 4 : 0); }
// the tetrahedron kernels' vertex array (4 per element)
static inline const int *tet_nodes(gbfem_ctx c) { return c->mixed ? c->el_nodes4.p : c->el_nodes.p; }

// The host copies of a device-built structure (dof of each node, CRS rows
// and columns, element tables), downloaded once on first use after a build.
static int fetch_host_structure(gbfem_ctx c) {
  if (!c->hs_stale) return 0;
  const int nd = c->ndof;
  c->hs.dof_of_node.resize(c->nno);
  c->hs.row_ptr.resize((size_t)nd + 1);
  c->hs.col_ind.resize((size_t)c->nnz);
  // sized by the current structure, never by a buffer's grown capacity
  const size_t ntab = (size_t)c->nel * (c->nv * c->nv + c->nv);
  c->hs.el_table.resize(ntab);
  GB_CUDA(cudaMemcpyAsync(c->hs.dof_of_node.data(), c->dof_of_node.p, (size_t)c->nno * sizeof(int),
                          cudaMemcpyDeviceToHost, c->stream));
  GB_CUDA(cudaMemcpyAsync(c->hs.row_ptr.data(), c->row_ptr.p, ((size_t)nd + 1) * sizeof(int), cudaMemcpyDeviceToHost,
                          c->stream));
  GB_CUDA(cudaMemcpyAsync(c->hs.col_ind.data(), c->col_ind.p, (size_t)c->nnz * sizeof(int), cudaMemcpyDeviceToHost,
                          c->stream));
  GB_CUDA(cudaMemcpyAsync(c->hs.el_table.data(), c->el_table.p, ntab * sizeof(int), cudaMemcpyDeviceToHost,
                          c->stream));
  GB_CUDA(cudaStreamSynchronize(c->stream));
  c->hs_stale = false;
  return 0;
}

// Block SpMV over all DG block rows, one launch per element class (1..4:
// prisms of degree 1..4, 5..8: tetrahedra of degree 1..4).
static int dg_spmv(gbfem_ctx c, int mode, const double *x, const double *b, double *out) {
  int n = 0;
  for (int cls = 1; cls <= 8; cls++) {
    if (!c->dg_list[cls].p) continue;
    if (mode == 2 && c->dg_residual_dd) {
      const int r = gbfem::launch_dg_block_residual_dd(c->stream, cls, (int)c->dg_list[cls].n, c->dg_list[cls].p,
                                                       c->dg_roff_d.p, c->dg_row_val_d.p, c->dg_cx_off_d.p,
                                                       c->dg_colx_d.p, c->dg_val.p, x, b, out);
      if (r < 0) return r;
      n += r;
      continue;
    }
    const int r = gbfem::launch_dg_block_spmv(c->stream, mode, cls, (int)c->dg_list[cls].n, c->dg_list[cls].p,
                                              c->dg_roff_d.p, c->dg_row_val_d.p, c->dg_cx_off_d.p, c->dg_colx_d.p,
                                              c->dg_val.p, c->dg_dinv_off_d.p, c->dg_dinv.p, x, b, out);
    if (r < 0) return r;
    n += r;
  }
  return n;
}

extern "C" {

int gbfem_version(void) { return 1; }

const char *gbfem_last_error(void) { return gbfem::g_err.c_str(); }

int gbfem_create(gbfem_ctx *ctx, int device) { return gbfem::create_context(ctx, device, 0); }

}  // extern "C"

// A context whose stream has the given CUDA priority (0: the default).
int gbfem::create_context(gbfem_ctx *ctx, int device, int priority) {
  GB_CHECK(ctx != nullptr, "null context pointer");
  int ndev = 0;
  GB_CUDA(cudaGetDeviceCount(&ndev));
  GB_CHECK(device >= 0 && device < ndev, "no such CUDA device");
  GB_CUDA(cudaSetDevice(device));
  gbfem_ctx c = new gbfem_ctx_s();
  c->device = device;
  if (cudaStreamCreateWithPriority(&c->stream, cudaStreamNonBlocking, priority) != cudaSuccess ||
      cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess ||
      cudaEventCreate(&c->ev2) != cudaSuccess || cudaEventCreate(&c->ev3) != cudaSuccess) {
    delete c;
    set_error("stream/event creation failed");
    return -1;
  }
  if (c->err.alloc(1) < 0) {
    delete c;
    return -1;
  }
  cudaMemset(c->err.p, 0, sizeof(int));
  {
    // scratch taken with cudaMallocAsync (the device structure build) stays
    // in the device's default pool between builds, up to 1 GB, instead of
    // going back at every synchronisation (a setting of this process only)
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
      uint64_t thr = 1ULL << 30;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
  }
  *ctx = c;
  return 0;
}

extern "C" {

int gbfem_destroy(gbfem_ctx c) {
  if (!c) return 0;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  if (c->up_stream) {
    cudaStreamSynchronize(c->up_stream);
    cudaStreamDestroy(c->up_stream);
    cudaEventDestroy(c->up_now);
    for (auto &row : c->up_ev)
      for (auto &ev : row)
        if (ev) cudaEventDestroy(ev);
  }
  if (c->elem_stream) {
    cudaStreamSynchronize(c->elem_stream);
    cudaStreamDestroy(c->elem_stream);
    cudaEventDestroy(c->elem_ev0);
  }
  if (c->copy_stream) {
    cudaStreamSynchronize(c->copy_stream);
    cudaStreamDestroy(c->copy_stream);
    for (auto &ev : c->pipe_ev)
      if (ev) cudaEventDestroy(ev);
  }
  c->row_last.release();
  if (c->gm_graph) cudaGraphExecDestroy(c->gm_graph);
  c->sell_off.release();
  c->sell_col.release();
  c->sell_col16.release();
  c->sell_val.release();
  c->sell_valdw.release();
  c->gm_xdw.release();
  c->gm_small.release();
  c->gm_npart.release();
  c->gm_cnt.release();
  if (c->side_stream) {
    cudaStreamSynchronize(c->side_stream);
    cudaStreamDestroy(c->side_stream);
    for (auto &ev : c->side_ev)
      if (ev) cudaEventDestroy(ev);
  }
  DevBuf<double> *dbufs[] = {&c->xyz, &c->k_el, &c->D_el, &c->val, &c->rhs, &c->dinv, &c->V,
                             &c->w, &c->tmp, &c->x, &c->b, &c->partial, &c->hcol};
  for (auto *b : dbufs) b->release();
  DevBuf<int> *ibufs[] = {&c->el_nodes, &c->fa_el, &c->fa_side, &c->row_ptr, &c->col_ind, &c->dof_of_node,
                          &c->el_table, &c->el_perm, &c->fa_perm, &c->fa_map, &c->err, &c->in_id,
                          &c->in_pos, &c->in_table, &c->dg_roff_d};
  for (auto *b : ibufs) b->release();
  for (int cls = 0; cls < 9; cls++) {
    c->dg_list[cls].release();
    c->dg_mlist[cls].release();
  }
  for (int p = 0; p < 5; p++) {
    c->dg_flist_tc[p].release();
    c->dg_flist_64[p].release();
  }
  c->dg_mhf_ptr.release();
  c->dg_mhf.release();
  c->el_nodes4.release();
  c->dg_boff_diag_d.release();
  c->dg_val.release();
  c->dg_rhs.release();
  c->dg_hf_ptr.release();
  c->dg_p_d.release();
  c->dg_hf.release();
  c->dg_dinv.release();
  c->dg_dinv_off_d.release();
  c->dg_bptr_d.release();
  c->dg_bcol_d.release();
  c->dg_boff_d.release();
  c->dg_val32.release();
  c->dg_dinv32.release();
  c->ir_x.release();
  c->ir_r.release();
  c->dg_colx_d.release();
  c->dg_row_val_d.release();
  c->dg_cx_off_d.release();
  c->dg_fcfg.release();
  c->dg_ftab_off.release();
  c->dg_ftab.release();
  c->dg_tcface.release();
  c->dg_fgeo.release();
  c->dg_fshare.release();
  cudaEventDestroy(c->ev0);
  cudaEventDestroy(c->ev1);
  cudaEventDestroy(c->ev2);
  cudaEventDestroy(c->ev3);
  cudaStreamDestroy(c->stream);
  delete c;
  return 0;
}

long long gbfem_device_bytes(gbfem_ctx c) {
  if (!c) return 0;
  long long s = 0;
  const DevBuf<double> *dbufs[] = {&c->xyz, &c->k_el, &c->D_el, &c->val, &c->rhs, &c->dinv, &c->V,
                                   &c->w, &c->tmp, &c->x, &c->b, &c->partial, &c->hcol};
  for (auto *b : dbufs) s += b->bytes();
  const DevBuf<int> *ibufs[] = {&c->el_nodes, &c->fa_el, &c->fa_side, &c->row_ptr, &c->col_ind,
                                &c->dof_of_node, &c->el_table, &c->el_perm, &c->fa_perm, &c->fa_map,
                                &c->err, &c->in_id, &c->in_pos, &c->in_table};
  for (auto *b : ibufs) s += b->bytes();
  s += c->dg_val.bytes() + c->dg_rhs.bytes() + c->dg_dinv.bytes() + c->dg_hf.bytes() + c->dg_boff_d.bytes() +
       c->dg_boff_diag_d.bytes() + c->dg_dinv_off_d.bytes() + c->dg_bptr_d.bytes() + c->dg_bcol_d.bytes() +
       c->dg_hf_ptr.bytes() + c->dg_p_d.bytes() + c->dg_roff_d.bytes() + c->dg_colx_d.bytes() +
       c->dg_row_val_d.bytes() + c->dg_cx_off_d.bytes();
  for (int cls = 0; cls < 9; cls++) s += c->dg_list[cls].bytes() + c->dg_mlist[cls].bytes();
  for (int p = 0; p < 5; p++) s += c->dg_flist_tc[p].bytes() + c->dg_flist_64[p].bytes();
  s += c->dg_mhf_ptr.bytes() + c->dg_mhf.bytes() + c->el_nodes4.bytes();
  return s;
}

static void forget_dropin_tables(gbfem_ctx c);

int gbfem_set_option(gbfem_ctx c, int option, long long value) {
  GB_CHECK(c, "null context");
  if (option == GBFEM_OPT_CACHE_TABLES) {
    c->cache_tables = value ? 1 : 0;
    forget_dropin_tables(c);
    return 0;
  }
  if (option == GBFEM_OPT_DG_SPMV_ARITH) {
    GB_CHECK(value == GBFEM_STD_FP64 || value == GBFEM_STD_DWORD, "DG SpMV arithmetic must be FP64 or DWORD");
    c->dg_spmv_dword = value == GBFEM_STD_DWORD;
    return 0;
  }
  if (option == GBFEM_OPT_STD_SPMV_ARITH) {
    GB_CHECK(value == GBFEM_STD_FP64 || value == GBFEM_STD_DWORD, "std SpMV arithmetic must be FP64 or DWORD");
    c->std_spmv_dword = value == GBFEM_STD_DWORD;
    return 0;
  }
  if (option == GBFEM_OPT_DG_RESIDUAL) {
    GB_CHECK(value == GBFEM_RESIDUAL_FP64 || value == GBFEM_RESIDUAL_COMPENSATED,
             "DG residual arithmetic must be FP64 or COMPENSATED");
    c->dg_residual_dd = value == GBFEM_RESIDUAL_COMPENSATED;
    return 0;
  }
  if (option == GBFEM_OPT_STD_ARITH) {
    GB_CHECK(value == GBFEM_STD_FP64 || value == GBFEM_STD_DWORD, "std arithmetic must be FP64 or DWORD");
    c->std_dword = value == GBFEM_STD_DWORD;
    return 0;
  }
  set_error("unknown option");
  return -2;
}

static void clear_constraints(gbfem_ctx c) {
  c->ncon = 0;
  c->con_gen++;
  c->h_con_node.clear();
  c->h_con_par.clear();
  c->h_el_con.clear();
  c->con_split_key[0] = c->con_split_key[1] = nullptr;
}

int gbfem_set_mesh(gbfem_ctx c, int nno, const double *node_xyz, int nel, int nv, const int *el_nodes,
                   int nfa, const int *fa_id, const int *fa_el, const int *fa_side, const int *fa_bc) {
  GB_CHECK(c, "null context");
  GB_CHECK(nno > 0 && nel > 0 && node_xyz && el_nodes, "empty mesh");
  GB_CHECK(nv == GBFEM_PRISM || nv == GBFEM_TETRA, "nv must be 6 (prism) or 4 (tetrahedron)");
  GB_CHECK(nfa >= 0, "negative face count");
  GB_CHECK(nfa == 0 || (fa_el && fa_side), "face arrays missing");
  GB_CHECK(nv == GBFEM_PRISM || nfa == 0, "boundary faces are supported for prisms only");
  GB_CUDA(cudaSetDevice(c->device));
  GB_TRY(drain_uploads(c));
  for (long long i = 0; i < (long long)nel * nv; i++)
    GB_CHECK(el_nodes[i] >= 0 && el_nodes[i] < nno, "element vertex index out of range");
  for (int f = 0; f < nfa; f++) {
    GB_CHECK(fa_el[f] >= 0 && fa_el[f] < nel, "face element out of range");
    GB_CHECK(fa_side[f] >= 0 && fa_side[f] <= 4, "face side out of range");
    if (fa_bc) GB_CHECK(fa_bc[f] > 0 && fa_bc[f] < 10, "only Dirichlet faces (0<bc<10) are integrated");
  }
  c->nno = nno;
  c->nel = nel;
  c->nv = nv;
  c->nfa = nfa;
  c->mixed = false;
  c->pipe_e0 = c->pipe_e1 = -1;  // the download plan reads the element vertices
  clear_constraints(c);
  c->h_el_tet.clear();
  c->el_nodes4.release();
  c->h_el_nodes.assign(el_nodes, el_nodes + (size_t)nel * nv);
  c->h_fa_el.assign(fa_el, fa_el + nfa);
  c->h_fa_side.assign(fa_side, fa_side + nfa);
  c->h_fa_id.clear();
  int maxid = 0;
  if (fa_id) {
    c->h_fa_id.assign(fa_id, fa_id + nfa);
    for (int f = 0; f < nfa; f++) maxid = std::max(maxid, fa_id[f]);
  }
  c->max_fa_id = maxid;
  c->fa_index_of_id.assign(maxid + 1, -1);
  for (int f = 0; f < (int)c->h_fa_id.size(); f++) c->fa_index_of_id[c->h_fa_id[f]] = f;
  GB_TRY(upload(c, c->xyz, node_xyz, (size_t)nno * 3));
  GB_TRY(upload(c, c->el_nodes, el_nodes, (size_t)nel * nv));
  GB_TRY(upload(c, c->fa_el, fa_el, (size_t)nfa));
  GB_TRY(upload(c, c->fa_side, fa_side, (size_t)nfa));
  GB_TRY(upload(c, c->fa_map, c->fa_index_of_id.data(), c->fa_index_of_id.size()));
  c->have_structure = c->have_tables = false;
  GB_CUDA(cudaStreamSynchronize(c->stream));
  return 0;
}

int gbfem_set_mesh_mixed(gbfem_ctx c, int nno, const double *node_xyz, int nel, const int *el_nv,
                         const int *el_nodes) {
  GB_CHECK(c, "null context");
  GB_TRY(drain_uploads(c));
  GB_CHECK(nno > 0 && nel > 0 && node_xyz && el_nodes && el_nv, "empty mesh");
  GB_CUDA(cudaSetDevice(c->device));
  std::vector<int> en((size_t)nel * 6), en4((size_t)nel * 4);
  std::vector<unsigned char> tet(nel);
  for (int e = 0; e < nel; e++) {
    GB_CHECK(el_nv[e] == GBFEM_PRISM || el_nv[e] == GBFEM_TETRA,
             "element " + std::to_string(e) + ": vertex count must be 6 (prism) or 4 (tetrahedron)");
    tet[e] = el_nv[e] == GBFEM_TETRA;
    for (int k = 0; k < el_nv[e]; k++)
      GB_CHECK(el_nodes[6 * (size_t)e + k] >= 0 && el_nodes[6 * (size_t)e + k] < nno,
               "element vertex index out of range");
    // unused slots of a tetrahedron repeat its first vertex: every slot is
    // a valid node
    for (int k = 0; k < 6; k++) en[6 * (size_t)e + k] = el_nodes[6 * (size_t)e + (k < el_nv[e] ? k : 0)];
    for (int k = 0; k < 4; k++) en4[4 * (size_t)e + k] = el_nodes[6 * (size_t)e + k];
  }
  c->nno = nno;
  c->nel = nel;
  c->nv = GBFEM_PRISM;  // element slots
  c->nfa = 0;
  c->mixed = true;
  clear_constraints(c);
  c->h_el_tet.swap(tet);
  c->h_el_nodes.swap(en);
  c->h_fa_el.clear();
  c->h_fa_side.clear();
  c->h_fa_id.clear();
  c->max_fa_id = 0;
  c->fa_index_of_id.assign(1, -1);
  GB_TRY(upload(c, c->xyz, node_xyz, (size_t)nno * 3));
  GB_TRY(upload(c, c->el_nodes, c->h_el_nodes.data(), c->h_el_nodes.size()));
  GB_TRY(upload(c, c->el_nodes4, en4.data(), en4.size()));
  GB_TRY(upload(c, c->fa_map, c->fa_index_of_id.data(), c->fa_index_of_id.size()));
  c->fa_el.release();
  c->fa_side.release();
  c->have_structure = c->have_tables = false;
  c->dg_p.clear();
  c->dg_nfa = -1;
  c->dg_ready = false;
  GB_CUDA(cudaStreamSynchronize(c->stream));
  return 0;
}

int gbfem_set_node_coords(gbfem_ctx c, const double *node_xyz) {
  GB_CHECK(c && c->nno > 0, "mesh not set");
  GB_CHECK(node_xyz, "null coordinates");
  if (c->cache_tables) return piece_upload(c, 0, c->xyz.p, node_xyz, c->nno, 3);
  GB_TRY(settle_uploads(c));
  GB_CUDA(cudaMemcpyAsync(c->xyz.p, node_xyz, (size_t)c->nno * 3 * sizeof(double), cudaMemcpyHostToDevice,
                          c->stream));
  return 0;
}

int gbfem_set_coefficients(gbfem_ctx c, const double *k_el, const double *D_el, double f, double g,
                           double penalty) {
  GB_CHECK(c && c->nel > 0, "mesh not set");
  GB_CHECK(!(k_el && D_el), "give either k_el or D_el");
  // the buffers are kept while their sizes stay: pieces in flight into them
  // need waiting for only when one is freed or reallocated
  const bool keep = (k_el ? c->k_el.p && c->k_el.n >= (size_t)c->nel : !c->k_el.p) &&
                    (D_el ? c->D_el.p && c->D_el.n >= (size_t)9 * c->nel : !c->D_el.p);
  if (!keep) GB_TRY(drain_uploads(c));
  if (!c->cache_tables) GB_TRY(settle_uploads(c));
  if (k_el) {
    GB_TRY(c->k_el.alloc(c->nel));
    if (c->cache_tables)
      GB_TRY(piece_upload(c, 1, c->k_el.p, k_el, c->nel, 1));
    else
      GB_CUDA(cudaMemcpyAsync(c->k_el.p, k_el, (size_t)c->nel * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  } else {
    c->k_el.release();
  }
  if (D_el) {
    GB_TRY(c->D_el.alloc((size_t)9 * c->nel));
    if (c->cache_tables)
      GB_TRY(piece_upload(c, 1, c->D_el.p, D_el, c->nel, 9));
    else
      GB_CUDA(cudaMemcpyAsync(c->D_el.p, D_el, (size_t)9 * c->nel * sizeof(double), cudaMemcpyHostToDevice,
                              c->stream));
    c->aniso = 1;
  } else {
    c->D_el.release();
    c->aniso = 0;
  }
  c->f = f;
  c->g = g;
  c->penalty = penalty;
  return 0;
}

static int alloc_matrix(gbfem_ctx c) {
  GB_TRY(c->val.alloc((size_t)c->nnz));
  GB_TRY(c->rhs.alloc((size_t)c->ndof));
  return 0;
}

// A new structure voids the drop-in's cached tables and download plan
// (they index the old row_ptr / values), whatever pointers the caller passes.
static void forget_dropin_tables(gbfem_ctx c) {
  for (int i = 0; i < 3; i++) {
    c->cache_key[i] = nullptr;
    c->cache_len[i] = 0;
    c->cache_sig[i] = 0;
  }
  c->pipe_e0 = c->pipe_e1 = -1;
  c->table_generation++;
}

int gbfem_invalidate_tables(gbfem_ctx c) {
  GB_CHECK(c, "null context");
  forget_dropin_tables(c);
  return 0;
}

int gbfem_table_cache_stats(gbfem_ctx c, long long *generation, long long *uploads) {
  GB_CHECK(c, "null context");
  if (generation) *generation = c->table_generation;
  if (uploads) *uploads = c->table_uploads;
  return 0;
}

int gbfem_set_constraints(gbfem_ctx c, int n, const int *vertex, const int *nr_constr, const int *constr_id) {
  GB_CHECK(c && c->nno > 0, "mesh not set");
  GB_CHECK(!c->mixed && c->nv == GBFEM_PRISM, "constrained vertices are supported on std prism meshes");
  GB_CHECK(n >= 0 && n <= c->nno, "constrained vertex count out of range");
  GB_CHECK(n == 0 || (vertex && nr_constr && constr_id), "missing constraint arrays");
  GB_CUDA(cudaSetDevice(c->device));
  std::vector<int> node(c->nno, -1), par((size_t)4 * std::max(n, 1), -1);
  for (int k = 0; k < n; k++) {
    const int v = vertex[k], cnt = nr_constr[k];
    GB_CHECK(v >= 0 && v < c->nno, "constrained vertex index out of range");
    GB_CHECK(node[v] < 0, "vertex " + std::to_string(v) + " listed twice");
    GB_CHECK(cnt == 2 || cnt == 4, "a constrained vertex has 2 (mid-edge) or 4 (mid-face) constraining vertices");
    for (int j = 0; j < cnt; j++) {
      const int p = constr_id[4 * (size_t)k + j];
      GB_CHECK(p >= 0 && p < c->nno && p != v, "constraining vertex index out of range");
      par[4 * (size_t)k + j] = p;
    }
    node[v] = k;
  }
  // one level of constraints, as on the reference's 1-irregular meshes
  // (apr_get_stiff_mat_data expands a constrained vertex once)
  for (int k = 0; k < 4 * n; k++)
    GB_CHECK(par[k] < 0 || node[par[k]] < 0, "a constraining vertex is itself constrained");
  clear_constraints(c);
  std::vector<unsigned char> el_con(c->nel, 0);
  if (n > 0)
    for (long long i = 0; i < (long long)c->nel * c->nv; i++)
      if (node[c->h_el_nodes[i]] >= 0) el_con[i / c->nv] = 1;
  GB_TRY(upload(c, c->con_node, node.data(), node.size()));
  GB_TRY(upload(c, c->con_par, par.data(), par.size()));
  c->h_con_node.swap(node);
  c->h_con_par.swap(par);
  c->h_el_con.swap(el_con);
  c->ncon = n;
  GB_CUDA(cudaStreamSynchronize(c->stream));
  return 0;
}

// length of the expanded vertex list of an element (its table block holds
// n x n + n entries)
static int constrained_list_length(gbfem_ctx c, int el) {
  int n = 0;
  for (int j = 0; j < c->nv; j++) {
    const int k = c->ncon ? c->h_con_node[c->h_el_nodes[(size_t)el * c->nv + j]] : -1;
    n += k < 0 ? 1 : (c->h_con_par[4 * (size_t)k + 2] >= 0 ? 4 : 2);
  }
  return n;
}

int gbfem_set_crs_structure(gbfem_ctx c, int ndof, const int *dof_of_node, long long nnz, const int *row_ptr,
                            const int *col_ind) {
  GB_CHECK(c && c->nno > 0, "mesh not set");
  GB_CHECK(!c->mixed, "meshes of prisms and tetrahedra together are for the DG path (gbfem_dg_*)");
  GB_CHECK(ndof > 0 && nnz > 0 && nnz < 2147483647LL && row_ptr && col_ind, "bad CRS structure");
  GB_CHECK(row_ptr[0] == 0 && row_ptr[ndof] == nnz, "row_ptr inconsistent with nnz");
  c->ndof = ndof;
  c->nnz = nnz;
  c->hs_stale = false;
  c->hs.ndof = ndof;
  c->hs.row_ptr.assign(row_ptr, row_ptr + ndof + 1);
  c->hs.col_ind.assign(col_ind, col_ind + nnz);
  if (dof_of_node) {
    // a vertex of an element without a dof is a constrained (hanging) vertex
    // (apr_get_ent_pdeg(...) == 0, apd_std_lin/aps_std_lin_intf.c:2998): its
    // element's contributions take the constraint rewrite of
    // apr_get_stiff_mat_data (:2995-3170), which needs its constraining
    // vertices (gbfem_set_constraints, called before this)
    for (long long i = 0; i < (long long)c->nel * c->nv; i++) {
      const int v = c->h_el_nodes[i], d = dof_of_node[v];
      const bool constrained = c->ncon && c->h_con_node[v] >= 0;
      GB_CHECK(constrained || (d >= 0 && d < ndof),
               "element " + std::to_string(i / c->nv) + " has a vertex without a dof (a constrained / hanging "
               "vertex) that gbfem_set_constraints did not name");
      GB_CHECK(!constrained || d < 0, "a constrained vertex carries a dof");
    }
    c->hs.dof_of_node.assign(dof_of_node, dof_of_node + c->nno);
  }
  GB_TRY(upload(c, c->row_ptr, row_ptr, (size_t)ndof + 1));
  GB_TRY(upload(c, c->col_ind, col_ind, (size_t)nnz));
  if (dof_of_node) GB_TRY(upload(c, c->dof_of_node, dof_of_node, (size_t)c->nno));
  GB_TRY(alloc_matrix(c));
  forget_dropin_tables(c);
  c->have_structure = true;
  c->sell_ready = false;
  c->have_tables = false;
  GB_CUDA(cudaStreamSynchronize(c->stream));
  return 0;
}

int gbfem_build_structure(gbfem_ctx c, int *ndof, long long *nnz, int *nr_colors) {
  GB_CHECK(c && c->nno > 0, "mesh not set");
  GB_CHECK(c->ncon == 0, "constrained vertices: the structure and tables come from the caller "
                         "(gbfem_set_crs_structure, gbfem_create_assemble_stiff_mat)");
  GB_CHECK(!c->mixed, "meshes of prisms and tetrahedra together are for the DG path (gbfem_dg_*)");
  GB_TRY(gbfem::build_host_structure(c->nno, c->nel, c->nv, c->h_el_nodes.data(), c->nfa, c->h_fa_el.data(),
                                     c->h_fa_side.data(), c->hs));
  c->hs_stale = false;
  c->ndof = c->hs.ndof;
  c->nnz = (long long)c->hs.col_ind.size();
  GB_TRY(upload(c, c->row_ptr, c->hs.row_ptr.data(), c->hs.row_ptr.size()));
  GB_TRY(upload(c, c->col_ind, c->hs.col_ind.data(), c->hs.col_ind.size()));
  GB_TRY(upload(c, c->dof_of_node, c->hs.dof_of_node.data(), c->hs.dof_of_node.size()));
  GB_TRY(upload(c, c->el_table, c->hs.el_table.data(), c->hs.el_table.size()));
  GB_TRY(upload(c, c->el_perm, c->hs.el_perm.data(), c->hs.el_perm.size()));
  GB_TRY(upload(c, c->fa_perm, c->hs.fa_perm.data(), c->hs.fa_perm.size()));
  c->h_el_color_ptr = c->hs.el_color_ptr;
  c->h_fa_color_ptr = c->hs.fa_color_ptr;
  c->el_colour_pending = false;
  c->have_inc = false;
  GB_TRY(alloc_matrix(c));
  forget_dropin_tables(c);
  c->have_structure = c->have_tables = true;
  c->sell_ready = false;
  GB_CUDA(cudaStreamSynchronize(c->stream));
  if (ndof) *ndof = c->ndof;
  if (nnz) *nnz = c->nnz;
  if (nr_colors) *nr_colors = (int)c->h_el_color_ptr.size() - 1;
  return 0;
}

int gbfem_build_structure_device(gbfem_ctx c, int *ndof, long long *nnz) {
  GB_CHECK(c && c->nno > 0, "mesh not set");
  GB_CHECK(!c->mixed, "meshes of prisms and tetrahedra together are for the DG path (gbfem_dg_*)");
  GB_CHECK(c->ncon == 0, "constrained vertices: the structure and tables come from the caller "
                         "(gbfem_set_crs_structure, gbfem_create_assemble_stiff_mat)");
  GB_CUDA(cudaSetDevice(c->device));
  GB_CUDA(cudaMemsetAsync(c->err.p, 0, sizeof(int), c->stream));
  int nd = 0;
  long long nz = 0;
  GB_TRY(gbfem::build_device_structure(c->stream, c->nno, c->nel, c->nv, c->el_nodes.p, c->dof_of_node, c->row_ptr,
                                       c->col_ind, c->el_table, c->err.p, &nd, &nz));
  // the element colouring is made by the first colour scatter that needs it
  c->h_el_color_ptr.clear();
  c->el_colour_pending = true;
  c->have_inc = false;
  c->ndof = nd;
  c->nnz = nz;
  // the host copies (for the getters and the drop-in's chunked download) are
  // fetched when first needed: at 2M prisms the columns and element tables
  // are 420 MB, most of the build's time if copied every build
  c->hs.ndof = nd;
  c->hs.dof_of_node.clear();
  c->hs.row_ptr.clear();
  c->hs.col_ind.clear();
  c->hs.el_table.clear();
  c->hs_stale = true;
  // boundary faces (few): first-fit colouring on the host over the dofs of
  // their elements, as the host build does
  c->h_fa_color_ptr.clear();
  if (c->nfa > 0) {
    // only the dof of each node is needed here (the other host copies stay
    // on the device until something asks for them)
    std::vector<int> dn(c->nno);
    GB_CUDA(cudaMemcpyAsync(dn.data(), c->dof_of_node.p, (size_t)c->nno * sizeof(int), cudaMemcpyDeviceToHost,
                            c->stream));
    GB_CUDA(cudaStreamSynchronize(c->stream));
    std::vector<int> fa_dofs((size_t)c->nfa * c->nv), perm;
    for (int f = 0; f < c->nfa; f++)
      for (int j = 0; j < c->nv; j++)
        fa_dofs[(size_t)f * c->nv + j] = dn[c->h_el_nodes[(size_t)c->h_fa_el[f] * c->nv + j]];
    gbfem::color_entities(c->nfa, c->nv, fa_dofs, nd, c->h_fa_color_ptr, perm);
    GB_TRY(upload(c, c->fa_perm, perm.data(), perm.size()));
  }
  GB_TRY(alloc_matrix(c));
  forget_dropin_tables(c);
  c->have_structure = c->have_tables = true;
  c->sell_ready = false;
  GB_CUDA(cudaStreamSynchronize(c->stream));
  if (ndof) *ndof = nd;
  if (nnz) *nnz = nz;
  return 0;
}

int gbfem_get_crs_structure(gbfem_ctx c, int *dof_of_node, int *row_ptr, int *col_ind) {
  GB_CHECK(c && c->have_structure, "structure not set");
  GB_TRY(fetch_host_structure(c));
  if (dof_of_node && !c->hs.dof_of_node.empty())
    memcpy(dof_of_node, c->hs.dof_of_node.data(), c->hs.dof_of_node.size() * sizeof(int));
  if (row_ptr) memcpy(row_ptr, c->hs.row_ptr.data(), c->hs.row_ptr.size() * sizeof(int));
  if (col_ind) memcpy(col_ind, c->hs.col_ind.data(), c->hs.col_ind.size() * sizeof(int));
  return 0;
}

int gbfem_get_element_tables(gbfem_ctx c, int *tables) {
  GB_CHECK(c && c->have_tables, "structure not built (gbfem_build_structure)");
  GB_CHECK(tables, "null output");
  GB_TRY(fetch_host_structure(c));
  memcpy(tables, c->hs.el_table.data(), c->hs.el_table.size() * sizeof(int));
  return 0;
}

static int check_err_flag(gbfem_ctx c) {
  int h = 0;
  GB_CUDA(cudaMemcpyAsync(&h, c->err.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  GB_CUDA(cudaStreamSynchronize(c->stream));
  if (h) {
    cudaMemsetAsync(c->err.p, 0, sizeof(int), c->stream);
    set_error(h == 1   ? "integration entity list names an element outside the mesh"
              : h == 9 ? "the element incidence does not match the element tables"
                       : "integration entity list names a face that is not a boundary face of the mesh");
    return -3;
  }
  return 0;
}

// Fingerprint of a host int array from 257 entries spread over it (the
// first, the last and 255 at equal strides; FNV-1a over index and value).
static unsigned long long table_signature(const int *h, long long n) {
  unsigned long long s = 1469598103934665603ULL ^ (unsigned long long)n;
  if (n <= 0) return s;
  const int kSamples = 256;
  for (int i = 0; i <= kSamples; i++) {
    const long long j = i == kSamples ? n - 1 : (n * i) / kSamples;
    s = (s ^ (unsigned long long)(unsigned)j) * 1099511628211ULL;
    s = (s ^ (unsigned long long)(unsigned)h[j]) * 1099511628211ULL;
  }
  return s;
}

// Copies one drop-in input unless the tables are cached and this slot holds
// the same pointer and length with the same sampled contents; any upload
// voids the download plan, which depends on the tables.
static int stage_input(gbfem_ctx c, int slot, DevBuf<int> &d, const int *h, long long n) {
  const unsigned long long sig = c->cache_tables ? table_signature(h, n) : 0;
  if (c->cache_tables && c->cache_key[slot] == h && c->cache_len[slot] == n && c->cache_sig[slot] == sig &&
      d.n >= (size_t)n)
    return 0;
  GB_TRY(upload(c, d, h, (size_t)n));
  c->cache_key[slot] = h;
  c->cache_len[slot] = n;
  c->cache_sig[slot] = sig;
  c->pipe_e0 = c->pipe_e1 = -1;
  c->table_uploads++;
  return 0;
}

// The penalty faces with atomic scatter on a second stream, after the work
// already queued on the context stream (the memsets), beside the element
// kernel; join_side makes the context stream wait for them.  Atomic sums
// commute, so the order against the elements does not matter.
static int ensure_side(gbfem_ctx c) {
  if (!c->side_stream) {
    GB_CUDA(cudaStreamCreateWithFlags(&c->side_stream, cudaStreamNonBlocking));
    for (auto &ev : c->side_ev) GB_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  }
  return 0;
}
static int launch_faces_beside(gbfem_ctx c, int count, const int *ent_fa, const int *fa_map, int fa_map_len,
                               const int *ent_pos, const int *tab, int do_sm, int do_rhs, int *launches,
                               cudaStream_t after = nullptr, cudaEvent_t coords_ready = nullptr) {
  GB_TRY(ensure_side(c));
  GB_CUDA(cudaEventRecord(c->side_ev[0], after ? after : c->stream));
  GB_CUDA(cudaStreamWaitEvent(c->side_stream, c->side_ev[0], 0));
  if (coords_ready) GB_CUDA(cudaStreamWaitEvent(c->side_stream, coords_ready, 0));
  const int r = gbfem::launch_prism_faces(c->side_stream, true, count, ent_fa, 0, fa_map, fa_map_len,
                                          ent_pos, c->nfa, c->fa_el.p, c->fa_side.p, c->el_nodes.p, c->xyz.p,
                                          c->penalty, c->g, tab, c->val.p, c->rhs.p, do_sm, do_rhs, c->err.p);
  GB_TRY(r);
  *launches += r;
  GB_CUDA(cudaEventRecord(c->side_ev[1], c->side_stream));
  return 0;
}
static int join_side(gbfem_ctx c, cudaStream_t st) {
  GB_CUDA(cudaStreamWaitEvent(st, c->side_ev[1], 0));
  return 0;
}

// last element (position within the element range) touching each row: the
// rows of an element's rhs positions and of its value positions (found in
// row_ptr); entries outside the structure are left to the element kernels
__global__ void row_last_kernel(int count, const int *__restrict__ pos, const int *__restrict__ table, int nv,
                                int ndof, const int *__restrict__ row_ptr, int *row_last) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const int *t = table + pos[i];
  const int nnz = row_ptr[ndof];
  for (int j = 0; j < nv; j++) {
    const int r = t[nv * nv + j];
    if (r >= 0 && r < ndof) atomicMax(row_last + r, i);
  }
  for (int j = 0; j < nv * nv; j++) {
    const int q = t[j];
    if (q < 0 || q >= nnz) continue;
    int lo = 0, hi = ndof;  // row_ptr[lo] <= q < row_ptr[hi]
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (row_ptr[mid] <= q) lo = mid;
      else hi = mid;
    }
    atomicMax(row_last + lo, i);
  }
}

// Chunks of the element range and, per chunk, the number of leading rows that
// no later element touches (dof order by first appearance makes rows finish
// roughly in element order); built once per cached set of tables.
static int build_pipe_plan(gbfem_ctx c, int e0, int e1) {
  const int count = e1 - e0, nd = c->ndof;
  GB_TRY(c->row_last.alloc((size_t)nd));
  GB_CUDA(cudaMemsetAsync(c->row_last.p, 0xFF, (size_t)nd * sizeof(int), c->stream));
  row_last_kernel<<<(count + 255) / 256, 256, 0, c->stream>>>(count, c->in_pos.p + e0, c->in_table.p, c->nv, nd,
                                                              c->row_ptr.p, c->row_last.p);
  GB_CUDA(cudaGetLastError());
  std::vector<int> last(nd);
  GB_CUDA(cudaMemcpyAsync(last.data(), c->row_last.p, (size_t)nd * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  GB_CUDA(cudaStreamSynchronize(c->stream));
  for (int r = 1; r < nd; r++) last[r] = std::max(last[r], last[r - 1]);  // prefix maximum
  // chunks of whole waves of resident element threads (128-thread blocks,
  // five per SM for the FP64 kernel, three for the double-word one), at
  // most eight
  int nsm = 152;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device);
  const long long wave = (long long)nsm * (c->std_dword ? 3 : 5) * 128;
  const long long chunk = std::max(wave, (count / 8 + wave) / wave * wave);
  const int K = (int)((count + chunk - 1) / chunk);
  c->pipe_el.assign(K + 1, 0);
  c->pipe_rows.assign(K, nd);
  for (int k = 0; k <= K; k++) c->pipe_el[k] = (int)std::min<long long>(count, chunk * k);
  for (int k = 0; k + 1 < K; k++)
    c->pipe_rows[k] = (int)(std::upper_bound(last.begin(), last.end(), c->pipe_el[k + 1] - 1) - last.begin());
  // (the chunks' largest node and element indices are found when a call
  // first overlaps uploads with them: pipe_chunk_reach)
  c->pipe_maxnode.clear();
  c->pipe_maxel.clear();
  if (!c->copy_stream) {
    GB_CUDA(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
    for (auto &ev : c->pipe_ev) GB_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  }
  for (int i = 0; i < 3; i++) {
    c->pipe_key[i] = c->cache_key[i];
    c->pipe_len[i] = c->cache_len[i];
  }
  c->pipe_e0 = e0;
  c->pipe_e1 = e1;
  c->pipe_dword = c->std_dword;
  return 0;
}

// The largest node and element index each chunk of the download plan reads
// (which pieces of a coordinate / coefficient upload it waits for), from the
// entity ids the plan's tables were cached with; ids outside the mesh are
// the kernel's to report.
static void pipe_chunk_reach(gbfem_ctx c, int e0, const int *h_ent_id) {
  const int K = (int)c->pipe_el.size() - 1;
  c->pipe_maxnode.assign(K, c->nno - 1);
  c->pipe_maxel.assign(K, c->nel - 1);
  for (int k = 0; k < K; k++) {
    int mn = 0, me = 0;
    for (int i = e0 + c->pipe_el[k]; i < e0 + c->pipe_el[k + 1]; i++) {
      const int el = h_ent_id[i] - 1;
      if (el < 0 || el >= c->nel) continue;
      me = std::max(me, el);
      for (int j = 0; j < c->nv; j++) mn = std::max(mn, c->h_el_nodes[(size_t)el * c->nv + j]);
    }
    c->pipe_maxnode[k] = mn;
    c->pipe_maxel[k] = me;
  }
}

// Splits the drop-in's element range [e0, e1) and face range [f0, f1) into
// entities without and with constrained vertices and uploads the lists
// (element ids and table positions, face ids and positions) to con_lists:
// plain elements (ids, positions: e1 - e0 slots each), plain faces (f1 - f0
// slots each), then the constrained elements' ids and positions and the
// constrained faces' (con_split_n: the four counts).  Kept while the tables
// are cached and nothing it depends on changed.
static int split_constrained(gbfem_ctx c, const int *ent_id, const int *ent_pos, int n_ent, int e0, int e1, int f0,
                             int f1) {
  const long long sig[7] = {n_ent, e0, e1, f0, f1, c->con_gen, c->table_generation};
  bool same = c->cache_tables && c->con_split_key[0] == ent_id && c->con_split_key[1] == ent_pos;
  for (int i = 0; i < 7; i++) same = same && c->con_split_sig[i] == sig[i];
  if (same) return 0;
  const int ne = e1 - e0, nf = f1 - f0;
  std::vector<int> lists(2 * (size_t)(ne + nf) + 2 * (size_t)(ne + nf));
  std::vector<int> ce, cf;
  int nfe = 0, nff = 0;
  for (int i = e0; i < e1; i++) {
    const int el = ent_id[i] - 1;
    if (el >= 0 && el < c->nel && c->h_el_con[el]) {
      ce.push_back(i);
    } else {  // (ids outside the mesh reach the plain kernel, which reports them)
      lists[nfe] = ent_id[i];
      lists[ne + nfe] = ent_pos[i];
      nfe++;
    }
  }
  for (int i = f0; i < f1; i++) {
    const int id = ent_id[i];
    const int fa = (id >= 0 && id < (int)c->fa_index_of_id.size()) ? c->fa_index_of_id[id] : -1;
    if (fa >= 0 && c->h_el_con[c->h_fa_el[fa]]) {
      cf.push_back(i);
    } else {
      lists[2 * (size_t)ne + nff] = id;
      lists[2 * (size_t)ne + nf + nff] = ent_pos[i];
      nff++;
    }
  }
  const size_t b = 2 * (size_t)(ne + nf);
  const int nce = (int)ce.size(), ncf = (int)cf.size();
  for (int k = 0; k < nce; k++) {
    lists[b + k] = ent_id[ce[k]];
    lists[b + nce + k] = ent_pos[ce[k]];
  }
  for (int k = 0; k < ncf; k++) {
    lists[b + 2 * nce + k] = ent_id[cf[k]];
    lists[b + 2 * nce + ncf + k] = ent_pos[cf[k]];
  }
  GB_TRY(upload(c, c->con_lists, lists.data(), std::max<size_t>(b + 2 * (size_t)(nce + ncf), 1)));
  c->con_split_n[0] = nfe;
  c->con_split_n[1] = nce;
  c->con_split_n[2] = nff;
  c->con_split_n[3] = ncf;
  c->con_split_key[0] = ent_id;
  c->con_split_key[1] = ent_pos;
  for (int i = 0; i < 7; i++) c->con_split_sig[i] = sig[i];
  return 0;
}

int gbfem_create_assemble_stiff_mat(gbfem_ctx c, int Level_id, int Comp_type, const int *Pdeg_coarse_p,
                                    int Nr_int_ent, const int *L_int_ent_type, const int *L_int_ent_id,
                                    int Nr_colors_elems, const int *L_color_index_elems, int Nr_colors_faces,
                                    const int *L_color_index_faces, const int *Asse_pos_first_dof_int_ent,
                                    const int *Assembly_table, int Max_dofs_int_ent, double *crs_val,
                                    double *rhs) {
  GB_CHECK(c && c->have_structure, "structure not set (gbfem_set_crs_structure)");
  GB_CHECK(Level_id == 0, "only the finest (single) level is supported");
  GB_CHECK(Pdeg_coarse_p == nullptr || *Pdeg_coarse_p == -10, "coarse-level degrees are not supported");
  GB_CHECK(Comp_type >= GBFEM_COMP_SM && Comp_type <= GBFEM_COMP_BOTH, "Comp_type must be SM, RHS or BOTH");
  GB_CHECK(Nr_int_ent >= 0 && L_int_ent_id && Asse_pos_first_dof_int_ent && Assembly_table,
           "missing entity lists or assembly table");
  if (c->ncon == 0) {
    GB_CHECK(Max_dofs_int_ent <= c->nv,
             "Max_dofs_int_ent exceeds the element vertex count: an entity's dof list holds the constraining "
             "vertices of a constrained (hanging) vertex; name them with gbfem_set_constraints");
    GB_CHECK(Max_dofs_int_ent == c->nv, "Max_dofs_int_ent must equal the element vertex count");
  } else {
    // an expanded list holds up to 4 constraining vertices per vertex
    GB_CHECK(Max_dofs_int_ent >= c->nv && Max_dofs_int_ent <= 4 * c->nv,
             "Max_dofs_int_ent out of range for a mesh with constrained vertices");
  }
  GB_CUDA(cudaSetDevice(c->device));
  // element and face ranges in the entity lists
  int e0, e1, f0, f1;
  if (L_color_index_elems && Nr_colors_elems > 0) {
    e0 = L_color_index_elems[0];
    e1 = L_color_index_elems[Nr_colors_elems];
  } else {
    e0 = 0;
    e1 = 0;
    while (e1 < Nr_int_ent && L_int_ent_type[e1] == GBFEM_ELEMENT) e1++;
  }
  if (L_color_index_faces && Nr_colors_faces > 0) {
    f0 = L_color_index_faces[0];
    f1 = L_color_index_faces[Nr_colors_faces];
  } else {
    f0 = e1;
    f1 = Nr_int_ent;
  }
  GB_CHECK(0 <= e0 && e0 <= e1 && e1 <= Nr_int_ent && 0 <= f0 && f0 <= f1 && f1 <= Nr_int_ent,
           "colour index ranges outside the entity list");
  if (L_int_ent_type) {
    // the lists keep elements and faces in separate contiguous ranges
    if (e1 > e0) GB_CHECK(L_int_ent_type[e0] == GBFEM_ELEMENT && L_int_ent_type[e1 - 1] == GBFEM_ELEMENT,
                          "element range holds non-element entities");
    if (f1 > f0) GB_CHECK(L_int_ent_type[f0] == GBFEM_FACE && L_int_ent_type[f1 - 1] == GBFEM_FACE,
                          "face range holds non-face entities");
  }
  long long tlen = 0;
  {
    // table length: last entity's position + n*n + n (n: its dof count,
    // longer than nv where its element has constrained vertices)
    for (int i : {e1 - 1, f1 - 1}) {
      if (i < 0) continue;
      int n = c->nv;
      if (c->ncon) {
        int el = -1;
        if (i < e1 && i >= e0) {
          el = L_int_ent_id[i] - 1;
        } else {
          const int id = L_int_ent_id[i];
          const int fa = (id >= 0 && id < (int)c->fa_index_of_id.size()) ? c->fa_index_of_id[id] : -1;
          el = fa >= 0 ? c->h_fa_el[fa] : -1;
        }
        if (el >= 0 && el < c->nel) n = constrained_list_length(c, el);
      }
      tlen = std::max(tlen, (long long)Asse_pos_first_dof_int_ent[i] + (long long)n * n + n);
    }
  }
  cudaEventRecord(c->ev0, c->stream);
  const long long uploads0 = c->table_uploads;
  GB_TRY(stage_input(c, 0, c->in_id, L_int_ent_id, Nr_int_ent));
  GB_TRY(stage_input(c, 1, c->in_pos, Asse_pos_first_dof_int_ent, Nr_int_ent));
  GB_TRY(stage_input(c, 2, c->in_table, Assembly_table, tlen));
  const int do_sm = Comp_type != GBFEM_COMP_RHS, do_rhs = Comp_type != GBFEM_COMP_SM;
  // with cached tables and host outputs: element chunks, each chunk's
  // finished rows downloaded while the next chunk runs (plain meshes)
  const bool pipe = c->cache_tables && (crs_val || rhs) && e1 > e0 && c->ncon == 0;
  if (pipe) {
    bool same = c->pipe_e0 == e0 && c->pipe_e1 == e1 && c->pipe_dword == c->std_dword;
    for (int i = 0; i < 3; i++) same = same && c->pipe_key[i] == c->cache_key[i] && c->pipe_len[i] == c->cache_len[i];
    if (!same) GB_TRY(build_pipe_plan(c, e0, e1));
  }
  // coordinates / coefficients still going up in pieces (set while the
  // tables are cached) overlap the element chunks, which run on their own
  // stream after the work queued on the context stream and wait for the
  // pieces they read; otherwise everything waits for the whole uploads
  const bool overlap = pipe && c->up_pending && c->table_uploads == uploads0;
  if (!overlap) GB_TRY(settle_uploads(c));
  if (overlap && c->pipe_maxnode.size() + 1 != c->pipe_el.size()) pipe_chunk_reach(c, e0, L_int_ent_id);
  cudaStream_t est = c->stream;
  if (overlap) {
    if (!c->elem_stream) {
      GB_CUDA(cudaStreamCreateWithFlags(&c->elem_stream, cudaStreamNonBlocking));
      GB_CUDA(cudaEventCreateWithFlags(&c->elem_ev0, cudaEventDisableTiming));
    }
    GB_CUDA(cudaEventRecord(c->elem_ev0, c->stream));
    GB_CUDA(cudaStreamWaitEvent(c->elem_stream, c->elem_ev0, 0));
    est = c->elem_stream;
  }
  if (do_sm) GB_CUDA(cudaMemsetAsync(c->val.p, 0, (size_t)c->nnz * sizeof(double), est));
  if (do_rhs) GB_CUDA(cudaMemsetAsync(c->rhs.p, 0, (size_t)c->ndof * sizeof(double), est));
  int launches = 0, r;
  // with constrained vertices: the entities whose element has one are split
  // off (their tables are n x n + n with the expanded lists) to the rewrite
  // kernels; the others keep the plain kernels
  const int *fe_id = c->in_id.p + e0, *fe_pos = c->in_pos.p + e0;
  const int *ff_id = c->in_id.p + f0, *ff_pos = c->in_pos.p + f0;
  int nfe = e1 - e0, nff = f1 - f0, nce = 0, ncf = 0;
  if (c->ncon) {
    GB_TRY(split_constrained(c, L_int_ent_id, Asse_pos_first_dof_int_ent, Nr_int_ent, e0, e1, f0, f1));
    const int *L = c->con_lists.p;
    nfe = c->con_split_n[0];
    nce = c->con_split_n[1];
    nff = c->con_split_n[2];
    ncf = c->con_split_n[3];
    const int ne = e1 - e0;
    fe_id = L;
    fe_pos = L + ne;
    ff_id = L + 2 * ne;
    ff_pos = L + 2 * ne + (f1 - f0);
  }
  const bool side = nff > 0;  // the faces run beside the element chunks
  if (side)
    GB_TRY(launch_faces_beside(c, nff, ff_id, c->fa_map.p, (int)c->fa_map.n, ff_pos, c->in_table.p, do_sm, do_rhs,
                               &launches, est, overlap && c->up_np[0] > 0 ? c->up_ev[0][c->up_np[0] - 1] : nullptr));
  cudaEventRecord(c->ev2, est);
  GB_CHECK(c->nv == GBFEM_PRISM || !c->aniso, "std tetrahedra take an isotropic k_el (tensors: prisms and DG)");
  // elements a..b of the (plain) element list
  auto elements = [&](int a, int b) -> int {
    if (b <= a) return 0;
    if (c->nv == GBFEM_PRISM)
      return gbfem::launch_prism_elements(est, true, c->aniso, b - a, fe_id + a, 1, fe_pos + a, c->nel,
                                          c->el_nodes.p, c->xyz.p, c->k_el.p, c->D_el.p, c->f, c->in_table.p,
                                          c->val.p, c->rhs.p, do_sm, do_rhs, c->err.p, c->std_dword);
    return gbfem::launch_tet_elements(est, true, b - a, fe_id + a, 1, fe_pos + a, c->nel, c->el_nodes.p,
                                      c->xyz.p, c->k_el.p, c->f, c->in_table.p, c->val.p, c->rhs.p, do_sm, do_rhs,
                                      c->err.p);
  };
  // the entities with constrained vertices, after the plain elements
  auto constrained = [&]() -> int {
    int n = 0;
    if (!c->ncon) return 0;
    const int ne = e1 - e0, nf = f1 - f0;
    const int *L = c->con_lists.p;
    for (int fc = 0; fc < 2; fc++) {
      const int cnt = fc ? ncf : nce;
      if (cnt == 0) continue;
      const int *ids = fc ? L + 2 * ne + 2 * nf + 2 * nce : L + 2 * ne + 2 * nf;
      const int r2 = gbfem::launch_prism_constrained(
          c->stream, fc == 1, c->aniso, cnt, ids, ids + cnt, c->nel, c->fa_map.p, (int)c->fa_map.n, c->nfa,
          c->fa_el.p, c->fa_side.p, c->el_nodes.p, c->xyz.p, c->k_el.p, c->D_el.p, c->f, c->penalty, c->g,
          c->con_node.p, c->con_par.p, c->in_table.p, c->val.p, c->rhs.p, do_sm, do_rhs, c->err.p);
      if (r2 < 0) return r2;
      n += r2;
    }
    return n;
  };
  if (pipe) {
    GB_TRY(fetch_host_structure(c));
    const int K = (int)c->pipe_el.size() - 1;
    const int *rp = c->hs.row_ptr.data();
    // all chunks first: a copy into pageable memory returns only when done
    for (int k = 0; k < K; k++) {
      if (overlap)
        for (int b = 0; b < 2; b++) {
          if (c->up_np[b] == 0) continue;
          const long long item = b == 0 ? c->pipe_maxnode[k] : c->pipe_maxel[k];
          const int piece = (int)std::min<long long>(c->up_np[b] - 1, item / c->up_per[b]);
          GB_CUDA(cudaStreamWaitEvent(est, c->up_ev[b][piece], 0));
        }
      GB_TRY(r = elements(c->pipe_el[k], c->pipe_el[k + 1]));
      launches += r;
      GB_CUDA(cudaEventRecord(c->pipe_ev[k], est));
    }
    cudaEventRecord(c->ev3, est);
    if (side) GB_TRY(join_side(c, c->copy_stream));  // face rows are final before any download
    int rprev = 0;
    for (int k = 0; k < K; k++) {
      GB_CUDA(cudaStreamWaitEvent(c->copy_stream, c->pipe_ev[k], 0));
      const int r1 = k + 1 < K ? c->pipe_rows[k] : c->ndof;
      if (r1 > rprev) {
        if (crs_val)
          GB_CUDA(cudaMemcpyAsync(crs_val + rp[rprev], c->val.p + rp[rprev], (size_t)(rp[r1] - rp[rprev]) * sizeof(double),
                                  cudaMemcpyDeviceToHost, c->copy_stream));
        if (rhs)
          GB_CUDA(cudaMemcpyAsync(rhs + rprev, c->rhs.p + rprev, (size_t)(r1 - rprev) * sizeof(double),
                                  cudaMemcpyDeviceToHost, c->copy_stream));
        rprev = r1;
      }
    }
    GB_CUDA(cudaEventRecord(c->pipe_ev[K], c->copy_stream));
    GB_CUDA(cudaStreamWaitEvent(c->stream, c->pipe_ev[K], 0));
    // (the copy stream waited for every chunk and the faces; the context
    // stream now also waits for every piece of the uploads)
    if (overlap) GB_TRY(settle_uploads(c));
  } else {
    GB_TRY(r = elements(0, nfe));
    launches += r;
    GB_TRY(r = constrained());
    launches += r;
    cudaEventRecord(c->ev3, c->stream);
    if (side) GB_TRY(join_side(c, c->stream));
    if (crs_val) GB_CUDA(cudaMemcpyAsync(crs_val, c->val.p, (size_t)c->nnz * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    if (rhs) GB_CUDA(cudaMemcpyAsync(rhs, c->rhs.p, (size_t)c->ndof * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  }
  cudaEventRecord(c->ev1, c->stream);
  GB_TRY(check_err_flag(c));
  cudaEventElapsedTime(&c->last_ms, c->ev0, c->ev1);
  cudaEventElapsedTime(&c->last_el_ms, c->ev2, c->ev3);
  c->last_launches = launches;
  return 0;
}

int gbfem_assemble(gbfem_ctx c, int scatter_mode) {
  GB_CHECK(c && c->have_tables, "structure not built (gbfem_build_structure)");
  GB_CHECK(c->ncon == 0, "constrained vertices: assemble through gbfem_create_assemble_stiff_mat with the "
                         "caller's tables");
  GB_CHECK(c->nv == GBFEM_PRISM || !c->aniso, "std tetrahedra take an isotropic k_el (tensors: prisms and DG)");
  GB_CHECK(scatter_mode == GBFEM_SCATTER_ATOMIC || scatter_mode == GBFEM_SCATTER_COLOR ||
               scatter_mode == GBFEM_SCATTER_GATHER,
           "bad scatter mode");
  GB_CHECK(scatter_mode != GBFEM_SCATTER_GATHER || (c->nv == GBFEM_PRISM && !c->std_dword),
           "the gather scatter takes std prisms in FP64 element arithmetic");
  GB_CUDA(cudaSetDevice(c->device));
  GB_TRY(settle_uploads(c));
  const bool atomic = scatter_mode == GBFEM_SCATTER_ATOMIC;
  const bool gather = scatter_mode == GBFEM_SCATTER_GATHER;
  if (!atomic && !c->have_inc && (gather || c->el_colour_pending)) {
    GB_TRY(gbfem::build_device_incidence(c->stream, c->nel, c->nv, c->el_table.p, c->ndof, c->inc_ptr, c->inc));
    c->have_inc = true;
  }
  if (scatter_mode == GBFEM_SCATTER_COLOR && c->el_colour_pending) {
    GB_CUDA(cudaMemsetAsync(c->err.p, 0, sizeof(int), c->stream));
    GB_TRY(gbfem::build_device_colouring(c->stream, c->nel, c->nv, c->el_table.p, c->inc_ptr.p, c->inc.p,
                                         c->el_perm, c->h_el_color_ptr, c->err.p));
    c->el_colour_pending = false;
  }
  if (gather) GB_TRY(c->ek.alloc((size_t)c->nel * 42));
  cudaEventRecord(c->ev0, c->stream);
  GB_CUDA(cudaMemsetAsync(c->val.p, 0, (size_t)c->nnz * sizeof(double), c->stream));
  GB_CUDA(cudaMemsetAsync(c->rhs.p, 0, (size_t)c->ndof * sizeof(double), c->stream));
  int launches = 0, r;
  // boundary faces, then elements (utd_util/uts_ls_intf.c:3629-3858,
  // 4103-4290); with atomic scatter the faces run beside the elements
  const bool side = atomic && c->nfa > 0;
  if (c->nfa > 0) {
    if (atomic) {
      GB_TRY(launch_faces_beside(c, c->nfa, nullptr, nullptr, 0, nullptr, c->el_table.p, 1, 1, &launches));
    } else {
      // the colour permutation lists face indices: feed them as "ids" through an identity map
      for (size_t k = 0; k + 1 < c->h_fa_color_ptr.size(); k++) {
        const int lo = c->h_fa_color_ptr[k], hi = c->h_fa_color_ptr[k + 1];
        r = gbfem::launch_prism_faces(c->stream, false, hi - lo, c->fa_perm.p + lo, 0, nullptr, -1, nullptr,
                                      c->nfa, c->fa_el.p, c->fa_side.p, c->el_nodes.p, c->xyz.p, c->penalty,
                                      c->g, c->el_table.p, c->val.p, c->rhs.p, 1, 1, c->err.p);
        GB_TRY(r);
        launches += r;
      }
    }
  }
  cudaEventRecord(c->ev2, c->stream);
  if (atomic) {
    if (c->nv == GBFEM_PRISM)
      r = gbfem::launch_prism_elements(c->stream, true, c->aniso, c->nel, nullptr, 0, nullptr, c->nel,
                                       c->el_nodes.p, c->xyz.p, c->k_el.p, c->D_el.p, c->f, c->el_table.p,
                                       c->val.p, c->rhs.p, 1, 1, c->err.p, c->std_dword);
    else
      r = gbfem::launch_tet_elements(c->stream, true, c->nel, nullptr, 0, nullptr, c->nel, c->el_nodes.p,
                                     c->xyz.p, c->k_el.p, c->f, c->el_table.p, c->val.p, c->rhs.p, 1, 1,
                                     c->err.p);
    GB_TRY(r);
    launches += r;
  } else if (gather) {
    r = gbfem::launch_std_gather(c->stream, c->aniso, c->nel, c->ndof, c->el_nodes.p, c->xyz.p, c->k_el.p,
                                 c->D_el.p, c->f, c->inc_ptr.p, c->inc.p, c->el_table.p, c->ek.p, c->val.p,
                                 c->rhs.p, c->err.p);
    GB_TRY(r);
    launches += r;
  } else {
    for (size_t k = 0; k + 1 < c->h_el_color_ptr.size(); k++) {
      const int lo = c->h_el_color_ptr[k], hi = c->h_el_color_ptr[k + 1];
      if (c->nv == GBFEM_PRISM)
        r = gbfem::launch_prism_elements(c->stream, false, c->aniso, hi - lo, c->el_perm.p + lo, 0, nullptr,
                                         c->nel, c->el_nodes.p, c->xyz.p, c->k_el.p, c->D_el.p, c->f,
                                         c->el_table.p, c->val.p, c->rhs.p, 1, 1, c->err.p, c->std_dword);
      else
        r = gbfem::launch_tet_elements(c->stream, false, hi - lo, c->el_perm.p + lo, 0, nullptr, c->nel,
                                       c->el_nodes.p, c->xyz.p, c->k_el.p, c->f, c->el_table.p, c->val.p,
                                       c->rhs.p, 1, 1, c->err.p);
      GB_TRY(r);
      launches += r;
    }
  }
  cudaEventRecord(c->ev3, c->stream);
  if (side) GB_TRY(join_side(c, c->stream));
  cudaEventRecord(c->ev1, c->stream);
  GB_TRY(check_err_flag(c));
  cudaEventElapsedTime(&c->last_ms, c->ev0, c->ev1);
  cudaEventElapsedTime(&c->last_el_ms, c->ev2, c->ev3);
  c->last_launches = launches;
  return 0;
}

// ---------------------------------------------------------------------------
// DG prisms
// ---------------------------------------------------------------------------
int gbfem_dg_set_degrees(gbfem_ctx c, const int *p_el) {
  GB_CHECK(c && c->nel > 0, "DG needs a mesh (gbfem_set_mesh)");
  GB_CHECK(p_el, "null degree array");
  for (int e = 0; e < c->nel; e++) GB_CHECK(p_el[e] >= 1 && p_el[e] <= 4, "DG degree must be 1..4");
  c->dg_p.assign(p_el, p_el + c->nel);
  c->dg_ready = false;
  return 0;
}

int gbfem_dg_set_faces(gbfem_ctx c, int nfa, const int *fa_type, const int *fa_bc, const int *fa_el,
                       const int *fa_side, const int *fa_nodes) {
  GB_CHECK(c && c->nel > 0, "DG needs a mesh (gbfem_set_mesh)");
  GB_CHECK(nfa >= 0, "negative face count");
  GB_CHECK(nfa == 0 || (fa_type && fa_bc && fa_el && fa_side && fa_nodes), "face arrays missing");
  const int nel = c->nel, stride = c->nv;
  const int *en = c->h_el_nodes.data();
  for (int f = 0; f < nfa; f++) {
    const int t = fa_type[f], e1 = fa_el[2 * f], e2 = fa_el[2 * f + 1], sd = fa_side[f];
    GB_CHECK(t == 3 || t == 4, "face type must be 3 (triangle) or 4 (quadrilateral)");
    GB_CHECK(e1 >= 0 && e1 < nel, "face neighbour out of range");
    GB_CHECK(e2 == -1 || (e2 >= 0 && e2 < nel && e2 != e1), "second face neighbour out of range");
    if (el_is_tet(c, e1))
      GB_CHECK(t == 3 && sd >= 0 && sd <= 3, "tetrahedron faces are triangles on sides 0..3");
    else
      GB_CHECK(sd >= 0 && sd <= 4 && (sd < 2) == (t == 3), "face side does not match the face type");
    GB_CHECK(e2 < 0 || el_is_tet(c, e1) == el_is_tet(c, e2) || t == 3,
             "a face between a prism and a tetrahedron must be a triangle");
    GB_CHECK(e2 >= 0 || (fa_bc[f] > 0 && fa_bc[f] < 10),
             "boundary faces must carry a Dirichlet flag (0 < bc < 10)");
    const int nv1 = el_nverts(c, e1), nv2 = e2 >= 0 ? el_nverts(c, e2) : 0;
    for (int i = 0; i < t; i++) {
      const int v = fa_nodes[4 * f + i];
      bool in1 = false, in2 = e2 < 0;
      for (int k = 0; k < nv1; k++) in1 = in1 || en[stride * (size_t)e1 + k] == v;
      for (int k = 0; k < nv2; k++) in2 = in2 || en[stride * (size_t)e2 + k] == v;
      GB_CHECK(in1 && in2, "face vertex is not a vertex of its neighbours");
    }
  }
  c->dg_nfa = nfa;
  c->dg_fa_type.assign(fa_type, fa_type + nfa);
  c->dg_fa_bc.assign(fa_bc, fa_bc + nfa);
  c->dg_fa_el.assign(fa_el, fa_el + 2 * (size_t)nfa);
  c->dg_fa_side.assign(fa_side, fa_side + nfa);
  c->dg_fa_nodes.assign(fa_nodes, fa_nodes + 4 * (size_t)nfa);
  c->dg_ready = false;
  return 0;
}

int gbfem_dg_set_volume_kernel(gbfem_ctx c, int mode) {
  GB_CHECK(c, "null context");
  GB_CHECK(mode == GBFEM_DG_VOLUME_FP64 || mode == GBFEM_DG_VOLUME_TC || mode == GBFEM_DG_VOLUME_TF32 ||
               mode == GBFEM_DG_VOLUME_DWORD || mode == GBFEM_DG_VOLUME_TC_DWORD,
           "unknown DG volume kernel");
  c->dg_volume_mode = mode;
  return 0;
}

int gbfem_dg_set_face_kernel(gbfem_ctx c, int mode) {
  GB_CHECK(c, "null context");
  GB_CHECK(mode == GBFEM_DG_FACE_FP64 || mode == GBFEM_DG_FACE_TC || mode == GBFEM_DG_FACE_DWORD ||
               mode == GBFEM_DG_FACE_TC_DWORD,
           "unknown DG face kernel");
  c->dg_face_mode = mode;
  return 0;
}

int gbfem_dg_set_penalty(gbfem_ctx c, double pen) {
  GB_CHECK(c, "null context");
  GB_CHECK(pen > 0.0, "penalty must be positive");
  c->dg_pen = pen;
  return 0;
}

int gbfem_dg_build_structure(gbfem_ctx c, int *ndof, long long *nval) {
  GB_CHECK(c && !c->dg_p.empty(), "DG degrees not set (gbfem_dg_set_degrees)");
  GB_CUDA(cudaSetDevice(c->device));
  const int nel = c->nel;
  const int nfa = c->dg_nfa < 0 ? 0 : c->dg_nfa;
  // dof blocks in element order (utr_get_list_ent, DG branch: one dof entity
  // per element, uts_ls_intf.c:640-700)
  c->dg_roff.assign(nel + 1, 0);
  for (int e = 0; e < nel; e++) c->dg_roff[e + 1] = c->dg_roff[e] + dg_ns_el(c, e);
  c->dg_ndof = c->dg_roff[nel];
  // block row e: the element and its face neighbours, ascending (the sorted
  // neighbour lists of sir_create, sis_mkb_intf.c:1100-1146)
  std::vector<int> cnt(nel + 1, 1);
  for (int f = 0; f < nfa; f++) {
    const int e1 = c->dg_fa_el[2 * f], e2 = c->dg_fa_el[2 * f + 1];
    if (e2 >= 0) {
      cnt[e1]++;
      cnt[e2]++;
    }
  }
  c->dg_bptr.assign(nel + 1, 0);
  for (int e = 0; e < nel; e++) c->dg_bptr[e + 1] = c->dg_bptr[e] + cnt[e];
  c->dg_bcol.assign(c->dg_bptr[nel], 0);
  std::vector<int> fill(c->dg_bptr.begin(), c->dg_bptr.end() - 1);
  for (int e = 0; e < nel; e++) c->dg_bcol[fill[e]++] = e;
  for (int f = 0; f < nfa; f++) {
    const int e1 = c->dg_fa_el[2 * f], e2 = c->dg_fa_el[2 * f + 1];
    if (e2 >= 0) {
      c->dg_bcol[fill[e1]++] = e2;
      c->dg_bcol[fill[e2]++] = e1;
    }
  }
  for (int e = 0; e < nel; e++) {
    auto b0 = c->dg_bcol.begin() + c->dg_bptr[e], b1 = c->dg_bcol.begin() + c->dg_bptr[e + 1];
    std::sort(b0, b1);
    GB_CHECK(std::adjacent_find(b0, b1) == b1, "two faces join the same pair of elements");
  }
  const int nblk = c->dg_bptr[nel];
  c->dg_boff.assign(nblk + 1, 0);
  std::vector<long long> diag(nel), dinv_off(nel + 1, 0);
  for (int e = 0; e < nel; e++) {
    const long long ne = dg_ns_el(c, e);
    for (int k = c->dg_bptr[e]; k < c->dg_bptr[e + 1]; k++) {
      const int col = c->dg_bcol[k];
      if (col == e) diag[e] = c->dg_boff[k];
      c->dg_boff[k + 1] = c->dg_boff[k] + ne * dg_ns_el(c, col);
    }
    dinv_off[e + 1] = dinv_off[e] + ne * ne;
  }
  c->dg_nval = c->dg_boff[nblk];
  auto block_of = [&](int row, int col) -> long long {
    auto b0 = c->dg_bcol.begin() + c->dg_bptr[row], b1 = c->dg_bcol.begin() + c->dg_bptr[row + 1];
    return c->dg_boff[std::lower_bound(b0, b1, col) - c->dg_bcol.begin()];
  };
  // face incidences per owner, faces in table order (the reference integrates
  // faces in face order after the elements); faces between a prism and a
  // tetrahedron go to a second table of their own
  auto is_mixed_face = [&](int f) {
    const int e1 = c->dg_fa_el[2 * f], e2 = c->dg_fa_el[2 * f + 1];
    return e2 >= 0 && el_is_tet(c, e1) != el_is_tet(c, e2);
  };
  std::vector<int> hcnt(nel + 1, 0), mcnt(nel + 1, 0);
  for (int f = 0; f < nfa; f++) {
    std::vector<int> &cn = is_mixed_face(f) ? mcnt : hcnt;
    cn[c->dg_fa_el[2 * f]]++;
    if (c->dg_fa_el[2 * f + 1] >= 0) cn[c->dg_fa_el[2 * f + 1]]++;
  }
  std::vector<int> hptr(nel + 1, 0), mptr(nel + 1, 0);
  for (int e = 0; e < nel; e++) {
    hptr[e + 1] = hptr[e] + hcnt[e];
    mptr[e + 1] = mptr[e] + mcnt[e];
  }
  std::vector<gbfem::DgHalfFace> hf(hptr[nel]), mhf(mptr[nel]);
  std::vector<int> hfill(hptr.begin(), hptr.end() - 1), mfill(mptr.begin(), mptr.end() - 1);
  const int *en = c->h_el_nodes.data();
  const int stride = c->nv;  // element slots in h_el_nodes (6 on mixed meshes)
  // face-point configurations (vertex count, local vertex order) of the
  // tensor-core face kernel's basis tables (faces between prisms)
  std::vector<unsigned char> cfgs;
  auto cfg_of = [&](int nfv, const unsigned char *loc) -> int {
    const int ncfg = (int)cfgs.size() / 5;
    for (int k = 0; k < ncfg; k++)
      if (cfgs[5 * k] == nfv && memcmp(&cfgs[5 * k + 1], loc, nfv) == 0) return k;
    if (ncfg >= gbfem::DG_TF_MAXCFG) return 255;
    cfgs.push_back((unsigned char)nfv);
    for (int i = 0; i < 4; i++) cfgs.push_back(i < nfv ? loc[i] : 0);
    return ncfg;
  };
  std::vector<int> face_rep(nfa, -1);  // the first neighbour's record of each face between prisms
  for (int f = 0; f < nfa; f++) {
    gbfem::DgHalfFace h;
    memset(&h, 0, sizeof(h));
    h.el1 = c->dg_fa_el[2 * f];
    h.el2 = c->dg_fa_el[2 * f + 1];
    h.side1 = c->dg_fa_side[f];
    h.nfv = c->dg_fa_type[f];
    h.face = f;
    const int nv1 = el_nverts(c, h.el1), nv2 = h.el2 >= 0 ? el_nverts(c, h.el2) : 0;
    for (int i = 0; i < h.nfv; i++) {
      const int v = c->dg_fa_nodes[4 * f + i];
      for (int k = 0; k < nv1; k++)
        if (en[stride * (size_t)h.el1 + k] == v) h.loc1[i] = (unsigned char)k;
      for (int k = 0; k < nv2; k++)
        if (en[stride * (size_t)h.el2 + k] == v) h.loc2[i] = (unsigned char)k;
    }
    const bool mixedf = is_mixed_face(f);
    if (!mixedf && !el_is_tet(c, h.el1)) {
      h.cfg1 = (unsigned char)cfg_of(h.nfv, h.loc1);
      h.cfg2 = h.el2 >= 0 ? (unsigned char)cfg_of(h.nfv, h.loc2) : 0;
    }
    h.owner_is_2 = 0;
    h.blk = h.el2 >= 0 ? block_of(h.el1, h.el2) : -1;
    if (mixedf) {
      mhf[mfill[h.el1]++] = h;
      h.owner_is_2 = 1;
      h.blk = block_of(h.el2, h.el1);
      mhf[mfill[h.el2]++] = h;
      continue;
    }
    if (!el_is_tet(c, h.el1)) face_rep[f] = hfill[h.el1];
    hf[hfill[h.el1]++] = h;
    if (h.el2 >= 0) {
      h.owner_is_2 = 1;
      h.blk = block_of(h.el2, h.el1);
      hf[hfill[h.el2]++] = h;
    }
  }
  // tables and face list for the tensor-core face kernel (faces between
  // prisms, at most DG_TF_MAXCFG configurations; otherwise that kernel is
  // not used)
  c->dg_ftab_ok = false;
  c->dg_tcface.release();
  if (!cfgs.empty() && (int)cfgs.size() / 5 < gbfem::DG_TF_MAXCFG) {
    const int ncfg = (int)cfgs.size() / 5;
    std::vector<long long> toff((size_t)ncfg * 9);
    const long long tsize = gbfem::dg_face_table_size(ncfg, cfgs.data(), toff.data());
    std::vector<int> tcf;  // faces whose sides both have degree <= 3
    for (int f = 0; f < nfa; f++) {
      const int e1 = c->dg_fa_el[2 * f], e2 = c->dg_fa_el[2 * f + 1];
      if (face_rep[f] >= 0 && c->dg_p[e1] <= 3 && (e2 < 0 || c->dg_p[e2] <= 3)) tcf.push_back(face_rep[f]);
    }
    GB_TRY(upload(c, c->dg_fcfg, cfgs.data(), cfgs.size()));
    GB_TRY(upload(c, c->dg_ftab_off, toff.data(), toff.size()));
    GB_TRY(c->dg_ftab.alloc((size_t)tsize));
    GB_TRY(gbfem::launch_dg_face_tables(c->stream, ncfg, c->dg_fcfg.p, c->dg_ftab_off.p, c->dg_ftab.p));
    if (!tcf.empty()) GB_TRY(upload(c, c->dg_tcface, tcf.data(), tcf.size()));
    c->dg_ftab_ok = true;
  }
  // per block row: value offset, and the dof index of each of its columns
  std::vector<long long> row_val(nel), cx_off(nel + 1, 0);
  for (int e = 0; e < nel; e++) {
    row_val[e] = c->dg_boff[c->dg_bptr[e]];
    long long nct = 0;
    for (int k = c->dg_bptr[e]; k < c->dg_bptr[e + 1]; k++) nct += dg_ns_el(c, c->dg_bcol[k]);
    cx_off[e + 1] = cx_off[e] + nct;
  }
  std::vector<int> colx(cx_off[nel]);
  for (int e = 0; e < nel; e++) {
    long long t = cx_off[e];
    for (int k = c->dg_bptr[e]; k < c->dg_bptr[e + 1]; k++) {
      const int col = c->dg_bcol[k];
      for (int j = c->dg_roff[col]; j < c->dg_roff[col + 1]; j++) colx[t++] = j;
    }
  }
  // elements per class (1..4 prisms, 5..8 tetrahedra of degree 1..4),
  // ordered by their row's column count so that the rows a warp multiplies
  // together take the same number of steps; the owners of faces between a
  // prism and a tetrahedron per class
  for (int cls = 1; cls <= 8; cls++) {
    std::vector<int> lst, mlst;
    for (int e = 0; e < nel; e++)
      if (dg_cls(c, e) == cls) {
        lst.push_back(e);
        if (mcnt[e]) mlst.push_back(e);
      }
    c->dg_list[cls].release();
    c->dg_mlist[cls].release();
    if (lst.empty()) continue;
    std::stable_sort(lst.begin(), lst.end(), [&](int a, int b) {
      return cx_off[a + 1] - cx_off[a] > cx_off[b + 1] - cx_off[b];
    });
    GB_TRY(upload(c, c->dg_list[cls], lst.data(), lst.size()));
    if (!mlst.empty()) GB_TRY(upload(c, c->dg_mlist[cls], mlst.data(), mlst.size()));
  }
  // prism face owners of degree <= 3 whose neighbours across faces between
  // prisms all have degree <= 3 suit the tensor-core face kernel; the others
  // keep the FP64 one
  for (int p = 1; p <= 4; p++) {
    std::vector<int> tcl, fpl;
    for (int e = 0; e < nel; e++) {
      if (c->dg_p[e] != p || el_is_tet(c, e)) continue;
      bool ok = p <= 3;
      for (int h = hptr[e]; ok && h < hptr[e + 1]; h++) {
        const int nb = hf[h].owner_is_2 ? hf[h].el1 : hf[h].el2;
        if (nb >= 0 && c->dg_p[nb] > 3) ok = false;
      }
      (ok ? tcl : fpl).push_back(e);
    }
    c->dg_flist_tc[p].release();
    c->dg_flist_64[p].release();
    if (!tcl.empty()) GB_TRY(upload(c, c->dg_flist_tc[p], tcl.data(), tcl.size()));
    if (!fpl.empty()) GB_TRY(upload(c, c->dg_flist_64[p], fpl.data(), fpl.size()));
  }
  GB_TRY(upload(c, c->dg_row_val_d, row_val.data(), row_val.size()));
  GB_TRY(upload(c, c->dg_cx_off_d, cx_off.data(), cx_off.size()));
  GB_TRY(upload(c, c->dg_colx_d, colx.data(), colx.size()));
  GB_TRY(upload(c, c->dg_roff_d, c->dg_roff.data(), c->dg_roff.size()));
  GB_TRY(upload(c, c->dg_boff_diag_d, diag.data(), diag.size()));
  GB_TRY(upload(c, c->dg_p_d, c->dg_p.data(), c->dg_p.size()));
  GB_TRY(upload(c, c->dg_hf_ptr, hptr.data(), hptr.size()));
  if (!hf.empty())
    GB_TRY(upload(c, c->dg_hf, hf.data(), hf.size()));
  else
    c->dg_hf.release();
  if (!mhf.empty()) {
    GB_TRY(upload(c, c->dg_mhf_ptr, mptr.data(), mptr.size()));
    GB_TRY(upload(c, c->dg_mhf, mhf.data(), mhf.size()));
  } else {
    c->dg_mhf_ptr.release();
    c->dg_mhf.release();
  }
  GB_TRY(upload(c, c->dg_bptr_d, c->dg_bptr.data(), c->dg_bptr.size()));
  GB_TRY(upload(c, c->dg_bcol_d, c->dg_bcol.data(), c->dg_bcol.size()));
  GB_TRY(upload(c, c->dg_boff_d, c->dg_boff.data(), c->dg_boff.size()));
  GB_TRY(upload(c, c->dg_dinv_off_d, dinv_off.data(), dinv_off.size()));
  c->dg_ninv = dinv_off[nel];
  GB_TRY(c->dg_val.alloc((size_t)c->dg_nval));
  GB_TRY(c->dg_rhs.alloc((size_t)c->dg_ndof));
  GB_CUDA(cudaStreamSynchronize(c->stream));
  c->dg_ready = true;
  if (ndof) *ndof = c->dg_ndof;
  if (nval) *nval = c->dg_nval;
  return 0;
}

int gbfem_dg_get_structure(gbfem_ctx c, int *dof_off, int *bptr, int *bcol, long long *boff) {
  GB_CHECK(c && c->dg_ready, "DG structure not built");
  if (dof_off) memcpy(dof_off, c->dg_roff.data(), c->dg_roff.size() * sizeof(int));
  if (bptr) memcpy(bptr, c->dg_bptr.data(), c->dg_bptr.size() * sizeof(int));
  if (bcol) memcpy(bcol, c->dg_bcol.data(), c->dg_bcol.size() * sizeof(int));
  if (boff) memcpy(boff, c->dg_boff.data(), c->dg_boff.size() * sizeof(long long));
  return (int)c->dg_bcol.size();
}

int gbfem_dg_assemble(gbfem_ctx c) {
  GB_CHECK(c && c->dg_ready, "DG structure not built (gbfem_dg_build_structure)");
  GB_TRY(settle_uploads(c));
  GB_CUDA(cudaSetDevice(c->device));
  int launches = 0;
  // volume terms write every diagonal block and the rhs; the face kernel then
  // adds to those and writes every off-diagonal block: nothing to clear
  const bool tc = c->dg_volume_mode == GBFEM_DG_VOLUME_TC || c->dg_volume_mode == GBFEM_DG_VOLUME_TF32 ||
                  c->dg_volume_mode == GBFEM_DG_VOLUME_TC_DWORD;
  // double-word stiffness sums: for every degree, or for those the tensor
  // cores do not cover
  const bool dwv = c->dg_volume_mode == GBFEM_DG_VOLUME_DWORD || c->dg_volume_mode == GBFEM_DG_VOLUME_TC_DWORD;
  if (tc) GB_CUDA(cudaMemsetAsync(c->err.p, 0, sizeof(int), c->stream));
  const bool tcf = c->dg_face_mode == GBFEM_DG_FACE_TC || c->dg_face_mode == GBFEM_DG_FACE_TC_DWORD;
  // Tensor-core faces beside a volume kernel on the CUDA cores (FP64 or
  // double word): the face kernel runs on the side stream from the start,
  // its diagonal-block and rhs shares go to scratch and are added once both
  // are done (the result is the same as in sequence: volume block + share).
  // The face kernel is latency bound at two CTAs per SM (its TMEM), which
  // leaves room for a volume CTA beside them.
  const bool overlap = tcf && !tc && c->dg_ftab_ok && c->dg_hf.p && c->nv == GBFEM_PRISM;
  long long share_off[5] = {0, 0, 0, 0, 0};
  if (overlap) {
    GB_TRY(ensure_side(c));
    GB_CUDA(cudaMemsetAsync(c->err.p, 0, sizeof(int), c->stream));
    long long tot = 0;
    for (int p = 1; p <= 3; p++) {
      share_off[p] = tot;
      const long long ns = kDgNs[p];
      tot += (long long)c->dg_flist_tc[p].n * (ns * ns + ns);
    }
    GB_TRY(c->dg_fshare.alloc((size_t)std::max(tot, 1LL)));
    GB_TRY(c->dg_fgeo.alloc((size_t)c->dg_nfa * 16 * 8));
  }
  cudaEventRecord(c->ev0, c->stream);
  if (overlap) {
    GB_CUDA(cudaEventRecord(c->side_ev[0], c->stream));
    GB_CUDA(cudaStreamWaitEvent(c->side_stream, c->side_ev[0], 0));
    int r = gbfem::launch_dg_face_geometry(c->side_stream, (int)c->dg_tcface.n, c->dg_tcface.p, c->dg_hf.p,
                                           c->dg_p_d.p, c->el_nodes.p, c->xyz.p, c->k_el.p, c->D_el.p, c->dg_pen,
                                           c->dg_fgeo.p);
    GB_TRY(r);
    launches += r;
    for (int p = 1; p <= 3; p++) {
      if (!c->dg_flist_tc[p].p) continue;
      r = gbfem::launch_dg_tc_faces(c->side_stream, p, (int)c->dg_flist_tc[p].n, c->dg_flist_tc[p].p,
                                    c->dg_hf_ptr.p, c->dg_hf.p, c->dg_p_d.p, c->dg_fgeo.p, c->dg_ftab.p,
                                    c->dg_ftab_off.p, c->g, c->dg_boff_diag_d.p, c->dg_roff_d.p, c->dg_val.p,
                                    c->dg_rhs.p, c->err.p, c->dg_fshare.p + share_off[p]);
      GB_TRY(r);
      launches += r;
    }
    GB_CUDA(cudaEventRecord(c->side_ev[1], c->side_stream));
  }
  for (int cls = 5; cls <= 8; cls++) {
    if (!c->dg_list[cls].p) continue;
    const int r = gbfem::launch_dg_tet_elements(c->stream, c->device, cls - 4, (int)c->dg_list[cls].n,
                                                c->dg_list[cls].p, tet_nodes(c), c->xyz.p, c->k_el.p, c->D_el.p,
                                                c->f, c->dg_boff_diag_d.p, c->dg_roff_d.p, c->dg_val.p,
                                                c->dg_rhs.p);
    GB_TRY(r);
    launches += r;
  }
  for (int p = 1; p <= 4; p++) {
    if (!c->dg_list[p].p) continue;
    int r;
    if (tc && gbfem::dg_tc_supported(p))  // TC_DWORD: split BF16 on the tensor cores
      r = gbfem::launch_dg_tc_volume(c->stream, c->device, p, (int)c->dg_list[p].n, c->dg_list[p].p, c->el_nodes.p,
                                     c->xyz.p, c->k_el.p, c->D_el.p, c->f, c->dg_boff_diag_d.p, c->dg_roff_d.p,
                                     c->dg_val.p, c->dg_rhs.p, c->err.p,
                                     c->dg_volume_mode == GBFEM_DG_VOLUME_TF32 ? 1 : 0);
    else
      r = gbfem::launch_dg_prism_elements(c->stream, c->device, p, (int)c->dg_list[p].n, c->dg_list[p].p,
                                          c->el_nodes.p, c->xyz.p, c->k_el.p, c->D_el.p, c->f,
                                          c->dg_boff_diag_d.p, c->dg_roff_d.p, c->dg_val.p, c->dg_rhs.p,
                                          c->dg_var_vol[p], dwv);
    GB_TRY(r);
    launches += r;
  }
  cudaEventRecord(c->ev2, c->stream);
  bool geo_done = false;
  if (overlap) {
    // the shares of the tensor-core owners, then the other owners below
    GB_CUDA(cudaStreamWaitEvent(c->stream, c->side_ev[1], 0));
    for (int p = 1; p <= 3; p++) {
      const int r = gbfem::launch_dg_face_share_add(c->stream, p, (int)c->dg_flist_tc[p].n, c->dg_flist_tc[p].p,
                                                    c->dg_fshare.p + share_off[p], c->dg_boff_diag_d.p,
                                                    c->dg_roff_d.p, c->dg_val.p, c->dg_rhs.p);
      GB_TRY(r);
      launches += r;
    }
  }
  const bool mixed_faces = c->dg_mhf.p != nullptr;
  if (mixed_faces && !tc && !(tcf && c->dg_hf.p) && !overlap)
    GB_CUDA(cudaMemsetAsync(c->err.p, 0, sizeof(int), c->stream));
  if (c->dg_hf.p) {
    if (tcf && !tc && !overlap) GB_CUDA(cudaMemsetAsync(c->err.p, 0, sizeof(int), c->stream));
    for (int cls = 5; cls <= 8; cls++) {
      if (!c->dg_list[cls].p) continue;
      const int r = gbfem::launch_dg_tet_faces(c->stream, cls - 4, (int)c->dg_list[cls].n, c->dg_list[cls].p,
                                               c->dg_hf_ptr.p, c->dg_hf.p, c->dg_p_d.p, tet_nodes(c), c->xyz.p,
                                               c->k_el.p, c->D_el.p, c->dg_pen, c->g, c->dg_boff_diag_d.p,
                                               c->dg_roff_d.p, c->dg_val.p, c->dg_rhs.p,
                                               c->dg_face_mode == GBFEM_DG_FACE_DWORD ||
                                                   c->dg_face_mode == GBFEM_DG_FACE_TC_DWORD);
      GB_TRY(r);
      launches += r;
    }
    for (int p = 1; p <= 4; p++) {
      if (!c->dg_list[p].p) continue;
      if (tcf && c->dg_ftab_ok) {
        // tensor-core eligible owners (done above when overlapped), then the
        // rest on the FP64 (or, in TC_DWORD mode, the double-word) kernel;
        // running those two side by side on disjoint owners was slower (167
        // vs 157 ms at p = 3, 432k)
        if (!overlap && !geo_done) {
          // per-point geometry of every face between degree <= 3 elements,
          // once per face (both owners read it)
          GB_TRY(c->dg_fgeo.alloc((size_t)c->dg_nfa * 16 * 8));
          const int r = gbfem::launch_dg_face_geometry(c->stream, (int)c->dg_tcface.n, c->dg_tcface.p, c->dg_hf.p,
                                                       c->dg_p_d.p, c->el_nodes.p, c->xyz.p, c->k_el.p, c->D_el.p,
                                                       c->dg_pen, c->dg_fgeo.p);
          GB_TRY(r);
          launches += r;
          geo_done = true;
        }
        int r = 0;
        if (!overlap) {
          r = gbfem::launch_dg_tc_faces(c->stream, p, (int)c->dg_flist_tc[p].n, c->dg_flist_tc[p].p,
                                        c->dg_hf_ptr.p, c->dg_hf.p, c->dg_p_d.p, c->dg_fgeo.p, c->dg_ftab.p,
                                        c->dg_ftab_off.p, c->g, c->dg_boff_diag_d.p, c->dg_roff_d.p,
                                        c->dg_val.p, c->dg_rhs.p, c->err.p, nullptr);
          GB_TRY(r);
          launches += r;
        }
        r = gbfem::launch_dg_prism_faces(c->stream, p, (int)c->dg_flist_64[p].n, c->dg_flist_64[p].p, c->dg_hf_ptr.p,
                                         c->dg_hf.p, c->dg_p_d.p, c->el_nodes.p, c->xyz.p, c->k_el.p, c->D_el.p,
                                         c->dg_pen, c->g, c->dg_boff_diag_d.p, c->dg_roff_d.p, c->dg_val.p,
                                         c->dg_rhs.p, c->dg_var_face[p], c->dg_face_mode == GBFEM_DG_FACE_TC_DWORD);
        GB_TRY(r);
        launches += r;
        continue;
      }
      // owners whose neighbourhood has degrees <= 3 on the compact tables
      // (more CTAs per SM), the others on the full ones; same results
      const bool dwf = c->dg_face_mode == GBFEM_DG_FACE_DWORD;
      for (int low = 1; low >= 0; low--) {
        const gbfem::DevBuf<int> &lst = low ? c->dg_flist_tc[p] : c->dg_flist_64[p];
        if (!lst.p) continue;
        const int r = gbfem::launch_dg_prism_faces(c->stream, p, (int)lst.n, lst.p, c->dg_hf_ptr.p, c->dg_hf.p,
                                                   c->dg_p_d.p, c->el_nodes.p, c->xyz.p, c->k_el.p, c->D_el.p,
                                                   c->dg_pen, c->g, c->dg_boff_diag_d.p, c->dg_roff_d.p,
                                                   c->dg_val.p, c->dg_rhs.p, c->dg_var_face[p], dwf, low != 0);
        GB_TRY(r);
        launches += r;
      }
    }
  }
  // faces between a prism and a tetrahedron, after every other face kernel
  // (their owners add to the diagonal blocks directly); FP64 in every mode
  for (int cls = 1; mixed_faces && cls <= 8; cls++) {
    if (!c->dg_mlist[cls].p) continue;
    const int r = gbfem::launch_dg_mixed_faces(c->stream, cls, (int)c->dg_mlist[cls].n, c->dg_mlist[cls].p,
                                               c->dg_mhf_ptr.p, c->dg_mhf.p, c->dg_p_d.p, c->el_nodes.p,
                                               tet_nodes(c), c->xyz.p, c->k_el.p, c->D_el.p, c->dg_pen,
                                               c->dg_boff_diag_d.p, c->dg_val.p, c->err.p);
    GB_TRY(r);
    launches += r;
  }
  cudaEventRecord(c->ev1, c->stream);
  GB_CUDA(cudaEventSynchronize(c->ev1));
  cudaEventElapsedTime(&c->last_ms, c->ev0, c->ev1);
  cudaEventElapsedTime(&c->last_el_ms, c->ev0, c->ev2);
  cudaEventElapsedTime(&c->last_fa_ms, c->ev2, c->ev1);
  if (tc || (tcf && c->dg_hf.p) || mixed_faces) {
    int herr = 0;
    GB_CUDA(cudaMemcpy(&herr, c->err.p, sizeof(int), cudaMemcpyDeviceToHost));
    GB_CHECK(herr != 5, "tensor-core volume kernel: a pipeline wait expired");
    GB_CHECK(herr != 6, "tensor-core face kernel: an MMA completion wait expired");
    GB_CHECK(herr != 7, "tensor-core face kernel: an owner with a degree-4 neighbour reached it");
    GB_CHECK(herr != 8, "prism-tetrahedron face kernel: a face record does not match its owner class");
    GB_CHECK(herr == 0, "DG assembly kernel error " + std::to_string(herr));
  }
  c->last_launches = launches;
  return 0;
}

int gbfem_dg_set_variants(gbfem_ctx c, const int *vol, const int *face) {
  GB_CHECK(c, "null context");
  for (int p = 1; p <= 4; p++) {
    if (vol) GB_CHECK(vol[p] >= 0 && vol[p] < 3, "volume variant out of range");
    if (face) GB_CHECK(face[p] >= 0 && face[p] < 2, "face variant out of range");
  }
  for (int p = 1; p <= 4; p++) {
    if (vol) c->dg_var_vol[p] = vol[p];
    if (face) c->dg_var_face[p] = face[p];
  }
  return 0;
}

// Times every launch-shape variant of the FP64 volume kernel and of the face
// kernel per degree class on up to `sample` elements of the class (the
// matrix is overwritten: assemble afterwards) and keeps the fastest.
int gbfem_dg_autotune(gbfem_ctx c, int sample, int *vol_out, int *face_out, double *ms_out) {
  GB_CHECK(c && c->dg_ready, "DG structure not built (gbfem_dg_build_structure)");
  GB_TRY(settle_uploads(c));
  GB_CHECK(c->nv == GBFEM_PRISM, "the launch-shape autotuner covers the prism kernels");
  GB_CUDA(cudaSetDevice(c->device));
  if (sample <= 0) sample = 16384;
  cudaStream_t st = c->stream;
  auto time_it = [&](const std::function<int()> &launch, float *best) -> int {
    *best = 1e30f;
    GB_TRY(launch());  // warm-up (module load, caches)
    for (int rep = 0; rep < 3; rep++) {
      cudaEventRecord(c->ev2, st);
      GB_TRY(launch());
      cudaEventRecord(c->ev3, st);
      GB_CUDA(cudaEventSynchronize(c->ev3));
      float ms = 0.f;
      cudaEventElapsedTime(&ms, c->ev2, c->ev3);
      *best = std::min(*best, ms);
    }
    return 0;
  };
  for (int p = 1; p <= 4; p++) {
    if (!c->dg_list[p].p) continue;
    const int cnt = (int)std::min<size_t>(c->dg_list[p].n, (size_t)sample);
    float bv = 1e30f, bf = 1e30f;
    for (int v = 0; v < 3; v++) {
      float ms;
      GB_TRY(time_it([&] {
        return gbfem::launch_dg_prism_elements(st, c->device, p, cnt, c->dg_list[p].p, c->el_nodes.p, c->xyz.p,
                                               c->k_el.p, c->D_el.p, c->f, c->dg_boff_diag_d.p, c->dg_roff_d.p,
                                               c->dg_val.p, c->dg_rhs.p, v);
      }, &ms));
      if (ms_out) ms_out[(p - 1) * 5 + v] = ms;
      if (ms < bv) {
        bv = ms;
        c->dg_var_vol[p] = v;
      }
    }
    if (c->dg_hf.p)
      for (int v = 0; v < 2; v++) {
        float ms;
        GB_TRY(time_it([&] {
          return gbfem::launch_dg_prism_faces(st, p, cnt, c->dg_list[p].p, c->dg_hf_ptr.p, c->dg_hf.p, c->dg_p_d.p,
                                              c->el_nodes.p, c->xyz.p, c->k_el.p, c->D_el.p, c->dg_pen, c->g,
                                              c->dg_boff_diag_d.p, c->dg_roff_d.p, c->dg_val.p, c->dg_rhs.p, v);
        }, &ms));
        if (ms_out) ms_out[(p - 1) * 5 + 3 + v] = ms;
        if (ms < bf) {
          bf = ms;
          c->dg_var_face[p] = v;
        }
      }
  }
  for (int p = 1; p <= 4; p++) {
    if (vol_out) vol_out[p] = c->dg_var_vol[p];
    if (face_out) face_out[p] = c->dg_var_face[p];
  }
  return 0;
}

int gbfem_dg_last_timing(gbfem_ctx c, double *total_ms, double *volume_ms, double *face_ms, int *launches) {
  GB_CHECK(c, "null context");
  if (total_ms) *total_ms = c->last_ms;
  if (volume_ms) *volume_ms = c->last_el_ms;
  if (face_ms) *face_ms = c->last_fa_ms;
  if (launches) *launches = c->last_launches;
  return 0;
}

int gbfem_dg_get_matrix(gbfem_ctx c, double *vals, double *rhs) {
  GB_CHECK(c && c->dg_ready, "DG structure not built");
  if (vals) GB_CUDA(cudaMemcpyAsync(vals, c->dg_val.p, (size_t)c->dg_nval * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (rhs) GB_CUDA(cudaMemcpyAsync(rhs, c->dg_rhs.p, (size_t)c->dg_ndof * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  GB_CUDA(cudaStreamSynchronize(c->stream));
  return 0;
}

int gbfem_dg_set_matrix(gbfem_ctx c, const double *vals, const double *rhs) {
  GB_CHECK(c && c->dg_ready, "DG structure not built");
  if (vals) GB_CUDA(cudaMemcpyAsync(c->dg_val.p, vals, (size_t)c->dg_nval * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  if (rhs) GB_CUDA(cudaMemcpyAsync(c->dg_rhs.p, rhs, (size_t)c->dg_ndof * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GB_CUDA(cudaStreamSynchronize(c->stream));
  return 0;
}

int gbfem_dg_compute_residual(gbfem_ctx c, int Use_rhs, int Ini_zero, int Ndof, const double *X, const double *B,
                              double *V) {
  GB_CHECK(c && c->dg_ready, "DG structure not built");
  GB_CHECK(Ndof == c->dg_ndof, "Ndof differs from the matrix size");
  GB_CHECK(V != nullptr, "null output vector");
  GB_CUDA(cudaSetDevice(c->device));
  const size_t nb = (size_t)Ndof * sizeof(double);
  GB_TRY(c->x.alloc(Ndof));
  GB_TRY(c->tmp.alloc(Ndof));
  if (Ini_zero || X == nullptr)
    GB_CUDA(cudaMemsetAsync(c->x.p, 0, nb, c->stream));
  else
    GB_CUDA(cudaMemcpyAsync(c->x.p, X, nb, cudaMemcpyHostToDevice, c->stream));
  const double *bd = nullptr;
  if (Use_rhs) {
    if (B) {
      GB_TRY(c->b.alloc(Ndof));
      GB_CUDA(cudaMemcpyAsync(c->b.p, B, nb, cudaMemcpyHostToDevice, c->stream));
      bd = c->b.p;
    } else {
      bd = c->dg_rhs.p;
    }
  }
  GB_TRY(dg_spmv(c, 2, c->x.p, bd, c->tmp.p));
  GB_CUDA(cudaMemcpyAsync(V, c->tmp.p, nb, cudaMemcpyDeviceToHost, c->stream));
  GB_CUDA(cudaStreamSynchronize(c->stream));
  return 0;
}

int gbfem_last_assembly_timing(gbfem_ctx c, double *total_ms, double *element_ms, int *launches) {
  GB_CHECK(c, "null context");
  if (total_ms) *total_ms = c->last_ms;
  if (element_ms) *element_ms = c->last_el_ms;
  if (launches) *launches = c->last_launches;
  return 0;
}

int gbfem_last_solve_timing(gbfem_ctx c, double *total_ms, double *spmv_ms, int *spmv_count, int *launches) {
  GB_CHECK(c, "null context");
  if (total_ms) *total_ms = c->last_solve_ms;
  if (spmv_ms) *spmv_ms = c->last_spmv_ms;
  if (spmv_count) *spmv_count = c->last_spmv_count;
  if (launches) *launches = c->last_solve_kernels;
  return 0;
}

void *gbfem_host_alloc(long long bytes) {
  void *p = nullptr;
  if (bytes <= 0 || cudaHostAlloc(&p, (size_t)bytes, cudaHostAllocPortable) != cudaSuccess) {
    set_error("cudaHostAlloc failed");
    return nullptr;
  }
  return p;
}

int gbfem_host_free(void *ptr) {
  if (ptr) GB_CUDA(cudaFreeHost(ptr));
  return 0;
}

int gbfem_measure_fp64_peak(gbfem_ctx c, double *tflops) {
  GB_CHECK(c && tflops, "null argument");
  GB_CUDA(cudaSetDevice(c->device));
  double v = 0.0;
  GB_TRY(gbfem::measure_fp64_peak(c->stream, c->device, &v));
  *tflops = v;
  return 0;
}

int gbfem_get_matrix(gbfem_ctx c, double *crs_val, double *rhs) {
  GB_CHECK(c && c->have_structure, "structure not set");
  if (crs_val) GB_CUDA(cudaMemcpyAsync(crs_val, c->val.p, (size_t)c->nnz * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (rhs) GB_CUDA(cudaMemcpyAsync(rhs, c->rhs.p, (size_t)c->ndof * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  GB_CUDA(cudaStreamSynchronize(c->stream));
  return 0;
}

int gbfem_set_matrix(gbfem_ctx c, const double *crs_val, const double *rhs) {
  GB_CHECK(c && c->have_structure, "structure not set");
  if (crs_val) GB_CUDA(cudaMemcpyAsync(c->val.p, crs_val, (size_t)c->nnz * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  if (rhs) GB_CUDA(cudaMemcpyAsync(c->rhs.p, rhs, (size_t)c->ndof * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GB_CUDA(cudaStreamSynchronize(c->stream));
  return 0;
}

int gbfem_compute_residual(gbfem_ctx c, int Use_rhs, int Ini_zero, int Ndof, const double *X, const double *B,
                           double *V) {
  GB_CHECK(c && c->have_structure, "structure not set");
  GB_CHECK(Ndof == c->ndof, "Ndof differs from the matrix size");
  GB_CHECK(V != nullptr, "null output vector");
  GB_CUDA(cudaSetDevice(c->device));
  const size_t nb = (size_t)Ndof * sizeof(double);
  GB_TRY(c->x.alloc(Ndof));
  GB_TRY(c->tmp.alloc(Ndof));
  if (Ini_zero || X == nullptr)
    GB_CUDA(cudaMemsetAsync(c->x.p, 0, nb, c->stream));
  else
    GB_CUDA(cudaMemcpyAsync(c->x.p, X, nb, cudaMemcpyHostToDevice, c->stream));
  const double *bd = nullptr;
  if (Use_rhs) {
    if (B) {
      GB_TRY(c->b.alloc(Ndof));
      GB_CUDA(cudaMemcpyAsync(c->b.p, B, nb, cudaMemcpyHostToDevice, c->stream));
      bd = c->b.p;
    } else {
      bd = c->rhs.p;
    }
  }
  GB_TRY(gbfem::launch_spmv(c->stream, 0, Ndof, c->row_ptr.p, c->col_ind.p, c->val.p, c->x.p, bd, nullptr,
                            c->tmp.p));
  GB_CUDA(cudaMemcpyAsync(V, c->tmp.p, nb, cudaMemcpyDeviceToHost, c->stream));
  GB_CUDA(cudaStreamSynchronize(c->stream));
  return 0;
}

}  // extern "C"

// Restarted GMRES(m) on a device-resident operator (lss_mkb_core.c:2317-2660):
// left preconditioned, classical Gram-Schmidt, Givens rotations, stopping on
// the preconditioned residual with the reference's 1e-12 floors
// (:2377-2378).  Vectors live on the device; the (m+1)x(m+1) Hessenberg
// matrix and the rotations live on the host (one small device-to-host copy
// per Arnoldi step).  op(0, in, out): out = M^-1 (b - A in);
// op(1, in, out): out = M^-1 A in; both return the number of kernels they
// launched.  Returns the iteration count.
using GmresOp = std::function<int(int, const double *, double *)>;

static int gmres_run(gbfem_ctx c, int n, int krylov, int max_iter, double tol_rel, int ini_zero, double *x,
                     double *res_out, double *res_rel_out, const GmresOp &op) {
  int kernels = 0;
#define GB_COUNT(x)          \
  do {                       \
    int r_ = (x);            \
    if (r_ < 0) return r_;   \
    kernels += r_;           \
  } while (0)
  const int m = krylov;
  const long long ld = n;
  GB_TRY(c->V.alloc((size_t)n * (m + 1)));
  GB_TRY(c->x.alloc(n));
  GB_TRY(c->tmp.alloc(n));
  GB_TRY(c->hcol.alloc(m + 2));
  const int nb = gbfem::reduction_blocks(n);
  GB_TRY(c->partial.alloc((size_t)nb * (m + 2)));
  cudaStream_t st = c->stream;
  // x == NULL: the solution stays in c->x (zeroed when ini_zero)
  if (ini_zero)
    GB_CUDA(cudaMemsetAsync(c->x.p, 0, (size_t)n * sizeof(double), st));
  else if (x)
    GB_CUDA(cudaMemcpyAsync(c->x.p, x, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, st));
  double tol_abs = 1e-12;
  if (tol_rel < 1e-12) tol_rel = 1e-12;
  std::vector<double> H((size_t)(m + 1) * (m + 1), 0.0), cs(m + 1), sn(m + 1), s(m + 2), hh(m + 2);
  double beta0 = -1.0, resid = 0.0;
  int it = 0;
  float spmv_ms = 0.f;
  int spmv_n = 0;
  cudaEventRecord(c->ev0, st);
  for (;;) {
    // v0 = M^-1 (b - A x)
    GB_COUNT(op(0, c->x.p, c->tmp.p));
    GB_COUNT(gbfem::launch_multidot(st, n, 1, c->tmp.p, ld, c->tmp.p, c->partial.p, c->hcol.p, 1));
    double rn = 0.0;
    GB_CUDA(cudaMemcpyAsync(&rn, c->hcol.p, sizeof(double), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    if (beta0 < 0) beta0 = rn;
    resid = rn;
    if (rn < tol_abs || (beta0 > 0 && rn / beta0 < tol_rel) || it >= max_iter) break;
    GB_COUNT(gbfem::launch_scale(st, n, c->hcol.p, 1, c->tmp.p, c->V.p));
    s[0] = rn;
    for (int i = 1; i <= m; i++) s[i] = 0.0;
    int done = 0;
    for (int j = 0; j < m; j++) {
      double *vj = c->V.p + (size_t)j * n, *w = c->V.p + (size_t)(j + 1) * n;
      it++;
      // w = M^-1 A v_j
      cudaEventRecord(c->ev2, st);
      GB_COUNT(op(1, vj, w));
      cudaEventRecord(c->ev3, st);
      // classical Gram-Schmidt: h = V^T w, w -= V h, h_{j+1} = |w|
      GB_COUNT(gbfem::launch_multidot(st, n, j + 1, c->V.p, ld, w, c->partial.p, c->hcol.p, 0));
      GB_COUNT(gbfem::launch_multiaxpy(st, n, j + 1, c->hcol.p, -1.0, c->V.p, ld, w));
      GB_COUNT(gbfem::launch_multidot(st, n, 1, w, ld, w, c->partial.p, c->hcol.p + j + 1, 1));
      GB_CUDA(cudaMemcpyAsync(hh.data(), c->hcol.p, (j + 2) * sizeof(double), cudaMemcpyDeviceToHost, st));
      GB_COUNT(gbfem::launch_scale(st, n, c->hcol.p + j + 1, 1, w, w));
      GB_CUDA(cudaStreamSynchronize(st));
      {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->ev2, c->ev3);
        spmv_ms += ms;
        spmv_n++;
      }
      for (int k = 0; k <= j + 1; k++) H[k + (size_t)j * (m + 1)] = hh[k];
      for (int k = 0; k < j; k++) {
        const double a = H[k + (size_t)j * (m + 1)], b = H[k + 1 + (size_t)j * (m + 1)];
        H[k + (size_t)j * (m + 1)] = cs[k] * a + sn[k] * b;
        H[k + 1 + (size_t)j * (m + 1)] = cs[k] * b - sn[k] * a;
      }
      {
        const double a = H[j + (size_t)j * (m + 1)], b = H[j + 1 + (size_t)j * (m + 1)];
        const double rr = std::hypot(a, b);
        cs[j] = a / rr;
        sn[j] = b / rr;
        H[j + (size_t)j * (m + 1)] = rr;
        H[j + 1 + (size_t)j * (m + 1)] = 0.0;
        const double s0 = s[j];
        s[j] = cs[j] * s0;
        s[j + 1] = -sn[j] * s0;
      }
      resid = std::fabs(s[j + 1]);
      if (j == m - 1 || it >= max_iter || resid < tol_abs || resid / beta0 < tol_rel) {
        done = j + 1;
        break;
      }
    }
    // y = H^-1 s, x += V y
    for (int k = done - 1; k >= 0; k--) {
      double t = s[k];
      for (int i = k + 1; i < done; i++) t -= H[k + (size_t)i * (m + 1)] * s[i];
      s[k] = t / H[k + (size_t)k * (m + 1)];
    }
    GB_CUDA(cudaMemcpyAsync(c->hcol.p, s.data(), done * sizeof(double), cudaMemcpyHostToDevice, st));
    GB_COUNT(gbfem::launch_multiaxpy(st, n, done, c->hcol.p, 1.0, c->V.p, ld, c->x.p));
    GB_CUDA(cudaStreamSynchronize(st));
    if (resid < tol_abs || resid / beta0 < tol_rel || it >= max_iter) break;
  }
  cudaEventRecord(c->ev1, st);
  if (x) GB_CUDA(cudaMemcpyAsync(x, c->x.p, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  cudaEventElapsedTime(&c->last_solve_ms, c->ev0, c->ev1);
  c->last_spmv_ms = spmv_ms;
  c->last_spmv_count = spmv_n;
  c->last_solve_kernels += kernels;
  if (res_out) *res_out = resid;
  if (res_rel_out) *res_rel_out = beta0 > 0 ? resid / beta0 : 0.0;
  return it;
#undef GB_COUNT
}

extern "C" {

// CRS matrix with point Jacobi (lar_fill_preconditioner_crs: 1 / a_ii,
// las_crs_intf.c:707).
int gbfem_solve(gbfem_ctx c, int krylov, int max_iter, double tol_rel, int ini_zero, double *x, double *res_out,
                double *res_rel_out) {
  GB_CHECK(c && c->have_structure, "structure not set");
  GB_CHECK(krylov > 0 && krylov <= 256, "krylov must be in 1..256");
  GB_CHECK(max_iter >= 0, "negative iteration limit");
  GB_CHECK(x != nullptr, "null solution vector");
  GB_CUDA(cudaSetDevice(c->device));
  return gbfem::gmres_device_std(c, krylov, max_iter, tol_rel, ini_zero, x, res_out, res_rel_out);
}

// DG block matrix with block Jacobi (inverted diagonal blocks).
int gbfem_dg_solve(gbfem_ctx c, int krylov, int max_iter, double tol_rel, int ini_zero, double *x, double *res_out,
                   double *res_rel_out) {
  GB_CHECK(c && c->dg_ready, "DG structure not built");
  GB_CHECK(krylov > 0 && krylov <= 256, "krylov must be in 1..256");
  GB_CHECK(x != nullptr, "null solution vector");
  GB_CUDA(cudaSetDevice(c->device));
  const int n = c->dg_ndof;
  cudaStream_t st = c->stream;
  GB_TRY(c->dg_dinv.alloc((size_t)c->dg_ninv));
  GB_CUDA(cudaMemsetAsync(c->err.p, 0, sizeof(int), st));
  GB_TRY(gbfem::launch_dg_block_inverse(st, c->nel, c->dg_roff_d.p, c->dg_boff_diag_d.p, c->dg_val.p,
                                        c->dg_dinv_off_d.p, c->dg_dinv.p, c->err.p));
  int herr = 0;
  GB_CUDA(cudaMemcpyAsync(&herr, c->err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  GB_CHECK(herr == 0, "singular diagonal block in the DG block Jacobi preconditioner");
  c->last_solve_kernels = 1;
  if (c->dg_spmv_dword) {
    // double-word copies of the matrix and of the inverted diagonal blocks
    // for the Arnoldi products; the restart residuals stay FP64
    GB_TRY(c->dg_valdw.alloc((size_t)c->dg_nval));
    GB_TRY(c->dg_dinvdw.alloc((size_t)c->dg_ninv));
    GB_TRY(gbfem::launch_to_dw(st, c->dg_nval, c->dg_val.p, c->dg_valdw.p));
    GB_TRY(gbfem::launch_to_dw(st, c->dg_ninv, c->dg_dinv.p, c->dg_dinvdw.p));
    c->last_solve_kernels += 2;
  }
  GmresOp op = [&](int mode, const double *in, double *out) -> int {
    if (mode == 1 && c->dg_spmv_dword) {
      int nl = 0;
      for (int cls = 1; cls <= 8; cls++) {
        if (!c->dg_list[cls].p) continue;
        const int r = gbfem::launch_dg_block_spmv_dw(c->stream, mode, cls, (int)c->dg_list[cls].n,
                                                     c->dg_list[cls].p, c->dg_roff_d.p, c->dg_row_val_d.p,
                                                     c->dg_cx_off_d.p, c->dg_colx_d.p, c->dg_valdw.p,
                                                     c->dg_dinv_off_d.p, c->dg_dinvdw.p, in, nullptr, out);
        if (r < 0) return r;
        nl += r;
      }
      return nl;
    }
    return dg_spmv(c, mode, in, mode == 0 ? c->dg_rhs.p : nullptr, out);
  };
  return gmres_run(c, n, krylov, max_iter, tol_rel, ini_zero, x, res_out, res_rel_out, op);
}

// DG iterative refinement: FP64 outer loop on the true residual, inner
// GMRES on FP32 copies of the matrix and of the inverted diagonal blocks.
static int dg_spmv32(gbfem_ctx c, int mode, const double *x, const double *b, double *out) {
  int n = 0;
  for (int cls = 1; cls <= 8; cls++) {
    if (!c->dg_list[cls].p) continue;
    const int r = gbfem::launch_dg_block_spmv32(c->stream, mode, cls, (int)c->dg_list[cls].n, c->dg_list[cls].p,
                                                c->dg_roff_d.p, c->dg_row_val_d.p, c->dg_cx_off_d.p,
                                                c->dg_colx_d.p, c->dg_val32.p, c->dg_dinv_off_d.p, c->dg_dinv32.p,
                                                x, b, out);
    if (r < 0) return r;
    n += r;
  }
  return n;
}

int gbfem_dg_solve_ir(gbfem_ctx c, int krylov, int max_iter, double tol_rel, double inner_tol, double *x,
                      int *outer_steps, double *rel_res) {
  GB_CHECK(c && c->dg_ready, "DG structure not built");
  GB_CHECK(krylov > 0 && krylov <= 256, "krylov must be in 1..256");
  GB_CHECK(x != nullptr, "null solution vector");
  GB_CHECK(tol_rel > 0 && inner_tol > 0 && inner_tol < 1, "tolerances must be positive (inner < 1)");
  GB_CUDA(cudaSetDevice(c->device));
  const int n = c->dg_ndof;
  cudaStream_t st = c->stream;
  // preconditioner in FP64, then FP32 copies of it and of the matrix
  GB_TRY(c->dg_dinv.alloc((size_t)c->dg_ninv));
  GB_CUDA(cudaMemsetAsync(c->err.p, 0, sizeof(int), st));
  GB_TRY(gbfem::launch_dg_block_inverse(st, c->nel, c->dg_roff_d.p, c->dg_boff_diag_d.p, c->dg_val.p,
                                        c->dg_dinv_off_d.p, c->dg_dinv.p, c->err.p));
  GB_TRY(c->dg_val32.alloc((size_t)c->dg_nval));
  GB_TRY(c->dg_dinv32.alloc((size_t)c->dg_ninv));
  GB_TRY(gbfem::launch_to_float(st, c->dg_nval, c->dg_val.p, c->dg_val32.p));
  GB_TRY(gbfem::launch_to_float(st, c->dg_ninv, c->dg_dinv.p, c->dg_dinv32.p));
  int herr = 0;
  GB_CUDA(cudaMemcpyAsync(&herr, c->err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  GB_CHECK(herr == 0, "singular diagonal block in the DG block Jacobi preconditioner");
  GB_TRY(c->ir_x.alloc(n));
  GB_TRY(c->ir_r.alloc(n));
  GB_TRY(c->hcol.alloc(krylov + 2));
  const int nb = gbfem::reduction_blocks(n);
  GB_TRY(c->partial.alloc((size_t)nb * (krylov + 2)));
  GB_TRY(c->b.alloc(2));
  const double one = 1.0;
  GB_CUDA(cudaMemcpyAsync(c->b.p, &one, sizeof(double), cudaMemcpyHostToDevice, st));
  GB_CUDA(cudaMemsetAsync(c->ir_x.p, 0, (size_t)n * sizeof(double), st));
  auto norm = [&](const double *v, double *out) -> int {
    const int r = gbfem::launch_multidot(st, n, 1, v, n, v, c->partial.p, c->hcol.p, 1);
    if (r < 0) return r;
    if (cudaMemcpyAsync(out, c->hcol.p, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
      gbfem::set_error("norm copy failed");
      return -1;
    }
    return 0;
  };
  double bn = 0.0;
  GB_TRY(norm(c->dg_rhs.p, &bn));
  const double *r_dev = c->ir_r.p;
  GmresOp op32 = [&](int mode, const double *in, double *out) -> int {
    return dg_spmv32(c, mode, in, mode == 0 ? r_dev : nullptr, out);
  };
  const auto t0 = std::chrono::steady_clock::now();
  int inner_total = 0, k = 0;
  double rel = 1.0, dprev = 0.0;
  bool converged_x = false;
  for (; k < 100; k++) {
    // true residual in FP64 (or with compensated sums)
    GB_TRY(dg_spmv(c, 2, c->ir_x.p, c->dg_rhs.p, c->ir_r.p));
    double rn = 0.0;
    GB_TRY(norm(c->ir_r.p, &rn));
    rel = bn > 0 ? rn / bn : 0.0;
    if (rel <= tol_rel || inner_total >= max_iter || converged_x) break;
    // correction from the FP32 operator (x0 = 0, result in c->x)
    // each correction: at most 10 restart cycles (the FP32 operator's own
    // rounding floor stops progress long before a tight inner tolerance)
    const int cap = std::min(max_iter - inner_total, 10 * krylov);
    const int it = gmres_run(c, n, krylov, cap, inner_tol, 1, nullptr, nullptr, nullptr, op32);
    GB_TRY(it);
    inner_total += it;
    GB_TRY(gbfem::launch_multiaxpy(st, n, 1, c->b.p, 1.0, c->x.p, n, c->ir_x.p));
    if (c->dg_residual_dd) {
      // with an accurate residual the solution converges to FP64 rounding
      // while the FP64-rounded residual stalls at its floor, so the steps
      // also stop on the corrections: once one is at the rounding level of
      // x, or, once the corrections are small (below 1e-10 of x: the inner
      // solves have reached the operator's accuracy), when one stops
      // contracting (Demmel et al., extra-precise iterative refinement,
      // ACM TOMS 32, 2006)
      double dn = 0.0, xn = 0.0;
      GB_TRY(norm(c->x.p, &dn));
      GB_TRY(norm(c->ir_x.p, &xn));
      if (dn <= 4.0 * 2.220446049250313e-16 * xn || (k >= 1 && dn > 0.5 * dprev && dn < 1e-10 * xn))
        converged_x = true;
      dprev = dn;
    }
  }
  GB_CUDA(cudaMemcpyAsync(x, c->ir_x.p, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  c->last_solve_ms = (float)std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (outer_steps) *outer_steps = k;
  if (rel_res) *rel_res = rel;
  return inner_total;
}

}  // extern "C"
