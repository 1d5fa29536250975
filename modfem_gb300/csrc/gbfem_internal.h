// Internal declarations shared by the CUDA translation units of libmodfem_gb300.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/modfem_gb300.h"

namespace gbfem {

void set_error(const std::string &msg);

#define GB_CUDA(call)                                                                        \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess) {                                                                 \
      ::gbfem::set_error(std::string(#call) + ": " + cudaGetErrorString(e_));                \
      return -1;                                                                             \
    }                                                                                        \
  } while (0)

#define GB_CHECK(cond, msg)                                                                  \
  do {                                                                                       \
    if (!(cond)) {                                                                           \
      ::gbfem::set_error(msg);                                                               \
      return -2;                                                                             \
    }                                                                                        \
  } while (0)

// propagates a negative status
#define GB_TRY(x)            \
  do {                       \
    int r_ = (x);            \
    if (r_ < 0) return r_;   \
  } while (0)

// Device buffer with explicit size tracking (no torch, no allocator layers).
template <typename T>
struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  int alloc(size_t count) {
    if (count <= n && p) return 0;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    if (count == 0) return 0;
    if (cudaMalloc(&p, count * sizeof(T)) != cudaSuccess) {
      set_error("cudaMalloc failed for " + std::to_string(count * sizeof(T)) + " bytes");
      return -1;
    }
    n = count;
    return 0;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  size_t bytes() const { return n * sizeof(T); }
};

// Per-degree DG prism tables on a device (dg_kernels.cu): D[q][a][u]
// reference derivatives, PHI[q][u] values, QP (xi, eta, zeta, w) per point.
struct DgDeviceTables {
  const double *D[5];
  const double *PHI[5];
  const double *QP[5];
  const float2 *Ddw[5];  // D as double words (h, l) for the double-word volume kernel
};
int dg_tables_for_device(int device, DgDeviceTables **out);

// Host-side structure built from the mesh (DOF order, CRS, tables, colours).
struct HostStructure {
  int ndof = 0;
  std::vector<int> dof_of_node;
  std::vector<int> row_ptr;
  std::vector<int> col_ind;
  std::vector<int> el_table;      // 42 (prism) or 20 (tet) ints per element
  std::vector<int> fa_table;      // per bc face: 16 value positions + 4 rhs (unused slots -1)
  std::vector<int> el_color_ptr;  // colour c holds el_perm[el_color_ptr[c] .. el_color_ptr[c+1])
  std::vector<int> el_perm;
  std::vector<int> fa_color_ptr;  // same for the boundary faces
  std::vector<int> fa_perm;
};

int build_host_structure(int nno, int nel, int nv, const int *el_nodes, int nfa, const int *fa_el,
                         const int *fa_side, HostStructure &hs);
// el_perm / el_color_ptr (may be null): a deterministic element colouring
// for the colour-batched scatter
int build_device_structure(cudaStream_t st, int nno, int nel, int nv, const int *el_nodes, DevBuf<int> &dof_of_node,
                           DevBuf<int> &row_ptr, DevBuf<int> &col_ind, DevBuf<int> &el_table, int *err,
                           int *ndof_out, long long *nnz_out);
// DOF -> element incidence from the element tables, each list in element order
int build_device_incidence(cudaStream_t st, int nel, int nv, const int *el_table, int nd, DevBuf<int> &inc_ptr,
                           DevBuf<int> &inc);
// elements-sharing-a-DOF colouring (Jones-Plassmann) from the tables and incidence
int build_device_colouring(cudaStream_t st, int nel, int nv, const int *el_table, const int *inc_ptr,
                           const int *inc, DevBuf<int> &el_perm, std::vector<int> &el_color_ptr, int *err);
void color_entities(int nent, int nv, const std::vector<int> &ent_dofs, int nd, std::vector<int> &color_ptr,
                    std::vector<int> &perm);

// kernel launchers (return the number of kernels launched, < 0 on error)
// gbfem_create with a CUDA stream priority for the context's stream
int create_context(gbfem_ctx *ctx, int device, int priority);
int launch_prism_elements(cudaStream_t st, bool atomic, bool aniso, int count, const int *ent_el,
                          int el_base, const int *ent_pos, int nel, const int *el_nodes,
                          const double *xyz, const double *k_el, const double *D_el, double f,
                          const int *tab, double *val, double *rhs, int do_sm, int do_rhs, int *err,
                          bool dword = false);
int launch_prism_faces(cudaStream_t st, bool atomic, int count, const int *ent_fa, int fa_base,
                       const int *fa_map, int fa_map_len, const int *ent_pos, int nfa,
                       const int *fa_el, const int *fa_side, const int *el_nodes,
                       const double *xyz, double penalty, double g, const int *tab, double *val,
                       double *rhs, int do_sm, int do_rhs, int *err);
// Prism elements by the deterministic gather scatter: local matrices stored
// to ek (42 doubles an element), then one thread a row over the incidence
int launch_std_gather(cudaStream_t st, bool aniso, int nel, int nd, const int *el_nodes, const double *xyz,
                      const double *k_el, const double *D_el, double f, const int *inc_ptr, const int *inc,
                      const int *tab, double *ek, double *val, double *rhs, int *err);
// Elements (faces = false, 1-based element ids) or boundary faces (mesh face
// ids through fa_map) whose element has constrained vertices: local matrices
// rewritten for the constraints and scattered through n x n + n tables.
int launch_prism_constrained(cudaStream_t st, bool faces, bool aniso, int count, const int *ent_id,
                             const int *ent_pos, int nel, const int *fa_map, int fa_map_len, int nfa,
                             const int *fa_el, const int *fa_side, const int *el_nodes, const double *xyz,
                             const double *k_el, const double *D_el, double f, double penalty, double g,
                             const int *con_node, const int *con_par, const int *tab, double *val, double *rhs,
                             int do_sm, int do_rhs, int *err);
int launch_tet_elements(cudaStream_t st, bool atomic, int count, const int *ent_el, int el_base,
                        const int *ent_pos, int nel, const int *el_nodes, const double *xyz,
                        const double *k_el, double f, const int *tab, double *val, double *rhs,
                        int do_sm, int do_rhs, int *err);
int launch_spmv(cudaStream_t st, int mode, int n, const int *row_ptr, const int *col_ind, const double *val,
                const double *x, const double *b, const double *scale, double *v);
int launch_jacobi_diag(cudaStream_t st, int n, const int *row_ptr, const int *col_ind, const double *val,
                       double *dinv);
int reduction_blocks(int n);
int launch_multidot(cudaStream_t st, int n, int m, const double *base, long long ld, const double *w,
                    double *partial, double *out, int sqrt_out);
int launch_multiaxpy(cudaStream_t st, int n, int m, const double *c, double sign, const double *base,
                     long long ld, double *y);
int launch_scale(cudaStream_t st, int n, const double *alpha, int invert, const double *x, double *y);
int launch_mul(cudaStream_t st, int n, const double *a, double *y);
int measure_fp64_peak(cudaStream_t st, int device, double *tflops);
// restarted GMRES with point Jacobi on the context's CRS matrix, all of it on
// the device (gmres_dev.cu); returns the iteration count
int gmres_device_std(gbfem_ctx c, int krylov, int max_iter, double tol_rel, int ini_zero, double *x,
                     double *res_out, double *res_rel_out);
// One (element, face) incidence of the DG face assembly, built on the host:
// the face's two neighbours (el2 = -1 on a Dirichlet boundary face), the side
// of el1 the face lies on, its vertex count, the local vertex index in el1 /
// el2 of each face vertex (face order), which neighbour owns this record, the
// value offset of the owner's off-diagonal block (owner, other), the
// face-point configurations of both sides (index of the (vertex count, local
// vertex order) pair in the basis tables of the tensor-core face kernel) and
// the face's index in the caller's face table.
struct DgHalfFace {
  int el1, el2;
  int side1, nfv;
  long long blk;
  unsigned char loc1[4], loc2[4];
  unsigned char owner_is_2, cfg1, cfg2, spare;
  int face;
};
static_assert(sizeof(DgHalfFace) == 40, "half-face record layout");

int launch_dg_tet_elements(cudaStream_t st, int device, int p, int count, const int *ent_el, const int *el_nodes,
                           const double *xyz, const double *k_el, const double *D_el, double f,
                           const long long *boff, const int *roff, double *val, double *rhs);
int launch_dg_tet_faces(cudaStream_t st, int p, int count, const int *ent_el, const int *hf_ptr,
                        const DgHalfFace *hf, const int *el_p, const int *el_nodes, const double *xyz,
                        const double *k_el, const double *D_el, double pen, double g, const long long *boff_diag,
                        const int *roff, double *val, double *rhs, bool dword = false);
// Faces between a prism and a tetrahedron (dg_mixed_faces.cu): owners of
// class cls (1..4 prisms of degree cls, 5..8 tetrahedra of degree cls - 4),
// their mixed half-faces mhf[mhf_ptr[e] .. mhf_ptr[e + 1]); prism vertices
// from el_nodes6 (6 per element), tetrahedron vertices from el_nodes4 (4 per
// element).  Runs after the same-type face kernels on the same stream.
int launch_dg_mixed_faces(cudaStream_t st, int cls, int count, const int *ent_el, const int *mhf_ptr,
                          const DgHalfFace *mhf, const int *el_p, const int *el_nodes6, const int *el_nodes4,
                          const double *xyz, const double *k_el, const double *D_el, double pen,
                          const long long *boff_diag, double *val, int *err);
bool dg_tc_faces_supported(int p);
// Face-point configurations of the tensor-core face kernel: cfg[5 c ..]
// = (vertex count, local vertex of each face vertex); tables of the reference
// basis (value and xi / eta / zeta derivatives, [point][function][4]) at the
// face points of every configuration c, rule degree pr and basis degree pb
// (1..3) from tab_off[(3 c + pr - 1) 3 + pb - 1]
constexpr int DG_TF_MAXCFG = 64;
long long dg_face_table_size(int ncfg, const unsigned char *cfg, long long *tab_off);
int launch_dg_face_tables(cudaStream_t st, int ncfg, const unsigned char *cfg, const long long *tab_off,
                          double *tab);
// Per-point geometry of the faces in `faces` (one half-face record each):
// geo[(face * 16 + q) * 8 ..] = (f a, c a, v1, v2) with f = 0.5 interior / 1
// boundary, a = |ds| w_q, c = pen p / sqrt(area), v_s = J_s^-1 A_s^T n
int launch_dg_face_geometry(cudaStream_t st, int count, const int *faces_hf, const DgHalfFace *hf,
                            const int *el_p, const int *el_nodes, const double *xyz, const double *k_el,
                            const double *D_el, double pen, double *geo);
// share == NULL: each owner's diagonal-block and rhs shares are added to its
// block and rows; else they are stored in the owner's slot of share (NS^2 +
// NS values, list order) for launch_dg_face_share_add, so that the kernel may
// run beside the volume kernel that writes those blocks
int launch_dg_tc_faces(cudaStream_t st, int p, int count, const int *ent_el, const int *hf_ptr,
                       const DgHalfFace *hf, const int *el_p, const double *geo, const double *ftab,
                       const long long *ftab_off, double g, const long long *boff_diag, const int *roff,
                       double *val, double *rhs, int *err, double *share);
int launch_dg_face_share_add(cudaStream_t st, int p, int count, const int *ent_el, const double *share,
                             const long long *boff_diag, const int *roff, double *val, double *rhs);
int launch_dg_prism_faces(cudaStream_t st, int p, int count, const int *ent_el, const int *hf_ptr,
                          const DgHalfFace *hf, const int *el_p, const int *el_nodes, const double *xyz,
                          const double *k_el, const double *D_el, double pen, double g, const long long *boff_diag,
                          const int *roff, double *val, double *rhs, int variant, bool dword = false, bool low = false);
// Variable-block CRS (one block row per DG element, dense column-major
// blocks with the row block's size as leading dimension) and block Jacobi.
int launch_dg_block_inverse(cudaStream_t st, int nel, const int *roff, const long long *boff_diag,
                            const double *val, const long long *dinv_off, double *dinv, int *err);
// mode 0: out = Minv (b - A x) (b may be NULL), 1: out = Minv A x,
// 2: out = (b ? b : 0) - A x (Minv unused); rows of the count elements of
// degree p listed in ent_el.  row_val[e]: value offset of block row e (its
// blocks are consecutive); colx[cx_off[e] ..]: dof index of each column.
int launch_dg_block_spmv(cudaStream_t st, int mode, int p, int count, const int *ent_el, const int *roff,
                         const long long *row_val, const long long *cx_off, const int *colx, const double *val,
                         const long long *dinv_off, const double *dinv, const double *x, const double *b,
                         double *out);
// The same with the matrix and the arithmetic in FP32 (inner solves of
// iterative refinement); vectors stay FP64.
int launch_dg_block_spmv32(cudaStream_t st, int mode, int p, int count, const int *ent_el, const int *roff,
                           const long long *row_val, const long long *cx_off, const int *colx, const float *val,
                           const long long *dinv_off, const float *dinv, const double *x, const double *b,
                           double *out);
// out = b - A x (b may be NULL) with compensated (two-word) sums
int launch_dg_block_residual_dd(cudaStream_t st, int p, int count, const int *ent_el, const int *roff,
                                const long long *row_val, const long long *cx_off, const int *colx,
                                const double *val, const double *x, const double *b, double *out);
int launch_to_float(cudaStream_t st, long long n, const double *a, float *b);
// double -> double word (h, l float pairs, 8 bytes each) and the block SpMV
// on double-word copies of the matrix and of the inverted diagonal blocks
int launch_to_dw(cudaStream_t st, long long n, const double *a, void *b);
int launch_dg_block_spmv_dw(cudaStream_t st, int mode, int p, int count, const int *ent_el, const int *roff,
                           const long long *row_val, const long long *cx_off, const int *colx, const void *val,
                           const long long *dinv_off, const void *dinv, const double *x, const double *b,
                           double *out);
// Tensor-core (tcgen05, split BF16) DG volume integrals, FP64-equivalent.
bool dg_tc_supported(int p);
int launch_dg_tc_volume(cudaStream_t st, int device, int p, int count, const int *ent_el, const int *el_nodes,
                        const double *xyz, const double *k_el, const double *D_el, double f, const long long *boff,
                        const int *roff, double *val, double *rhs, int *err, int mode);
int launch_dg_prism_elements(cudaStream_t st, int device, int p, int count, const int *ent_el, const int *el_nodes,
                             const double *xyz, const double *k_el, const double *D_el, double f,
                             const long long *boff, const int *roff, double *val, double *rhs, int variant, bool dword = false);

}  // namespace gbfem

struct gbfem_ctx_s {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr, ev3 = nullptr;
  // mesh
  int nno = 0, nel = 0, nv = 0, nfa = 0;  // nv: vertices per element (6 per element slot on mixed meshes)
  int max_fa_id = 0;
  gbfem::DevBuf<double> xyz;
  gbfem::DevBuf<int> el_nodes;
  // meshes of prisms and tetrahedra together (gbfem_set_mesh_mixed, DG
  // only): el_nodes holds 6 slots per element, el_nodes4 the first 4 of each
  // (the tetrahedron kernels' layout); h_el_tet marks the tetrahedra
  bool mixed = false;
  std::vector<unsigned char> h_el_tet;
  gbfem::DevBuf<int> el_nodes4;
  gbfem::DevBuf<int> fa_el, fa_side;
  std::vector<int> h_fa_id, h_fa_el, h_fa_side, h_el_nodes;
  std::vector<int> fa_index_of_id;  // reference face id -> bc face index (-1 none)
  // constrained (hanging) vertices (gbfem_set_constraints): per vertex -1 or
  // the index k of its constraining vertices con_par[4k..4k+3] (-1 padded);
  // h_el_con marks the elements with a constrained vertex
  int ncon = 0;
  long long con_gen = 0;
  std::vector<int> h_con_node, h_con_par;
  std::vector<unsigned char> h_el_con;
  gbfem::DevBuf<int> con_node, con_par;
  // the drop-in's entity lists split into entities with and without
  // constrained vertices (element ids, positions; face ids, positions)
  gbfem::DevBuf<int> con_lists;
  int con_split_n[4] = {0, 0, 0, 0};
  const void *con_split_key[2] = {nullptr, nullptr};
  long long con_split_sig[7] = {-1, -1, -1, -1, -1, -1, -1};
  // coefficients
  gbfem::DevBuf<double> k_el, D_el;
  int aniso = 0;
  double f = 1.0, g = 0.0, penalty = 1.0e7;
  // structure
  int ndof = 0;
  long long nnz = 0;
  gbfem::DevBuf<int> row_ptr, col_ind, dof_of_node;
  gbfem::DevBuf<int> el_table, el_perm, fa_perm, fa_map;
  // the device build leaves the element colouring to the first colour
  // scatter; the DOF -> element incidence (gather scatter) is built on demand
  bool el_colour_pending = false, have_inc = false;
  gbfem::DevBuf<int> inc_ptr, inc;
  gbfem::DevBuf<double> ek;  // local matrices of the gather scatter
  std::vector<int> h_el_color_ptr, h_fa_color_ptr;
  gbfem::HostStructure hs;
  // the device build leaves the host copies in hs to be fetched on first use
  // (getters, the drop-in's chunked download), not downloaded every build
  bool hs_stale = false;
  bool have_structure = false, have_tables = false;
  // matrix
  gbfem::DevBuf<double> val, rhs, dinv;
  gbfem::DevBuf<int> err;
  // drop-in staging (kept between calls when table caching is on)
  gbfem::DevBuf<int> in_id, in_pos, in_table;
  const void *cache_key[3] = {nullptr, nullptr, nullptr};
  long long cache_len[3] = {0, 0, 0};
  unsigned long long cache_sig[3] = {0, 0, 0};  // sampled contents at upload
  long long table_generation = 0;  // bumped whenever the cached tables are voided
  long long table_uploads = 0;     // drop-in inputs copied to the device (cache misses)
  int cache_tables = 0;
  bool std_dword = false;  // std prism elements in double-word arithmetic
  // pipelined download of the drop-in call while the tables are cached:
  // element chunks, and per chunk the rows no later element touches, copied
  // on copy_stream while the next chunk runs
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t pipe_ev[9] = {};
  gbfem::DevBuf<int> row_last;
  const void *pipe_key[3] = {nullptr, nullptr, nullptr};
  long long pipe_len[3] = {0, 0, 0};
  int pipe_e0 = -1, pipe_e1 = -1;
  bool pipe_dword = false;
  // the boundary-face kernel runs beside the element kernel (atomic scatter)
  cudaStream_t side_stream = nullptr;
  cudaEvent_t side_ev[2] = {};
  std::vector<int> pipe_el, pipe_rows;
  std::vector<int> pipe_maxnode, pipe_maxel;  // largest node / element index an element chunk reads
  // node coordinates and coefficients set while the tables are cached go up
  // in pieces on up_stream (events per piece), so that the drop-in's element
  // chunks (on elem_stream) start as soon as the pieces they read are there;
  // every other user of these arrays first makes the context stream wait
  // for all pieces (settle_uploads)
  cudaStream_t up_stream = nullptr, elem_stream = nullptr;
  cudaEvent_t up_ev[2][8] = {}, up_now = nullptr, elem_ev0 = nullptr;
  bool up_pending = false;
  int up_np[2] = {0, 0};        // pieces in flight: [0] coordinates, [1] k_el or D_el
  long long up_per[2] = {1, 1};  // nodes / elements a piece
  // Krylov workspace
  gbfem::DevBuf<double> V, w, tmp, x, b, partial, hcol;
  // device-resident std GMRES (gmres_dev.cu): sliced-ELL copy of the CRS
  // matrix, small arrays and state, the captured restart cycle
  gbfem::DevBuf<int> sell_off, sell_col;
  gbfem::DevBuf<double> sell_val, gm_small, gm_npart;
  gbfem::DevBuf<unsigned> gm_cnt;
  gbfem::DevBuf<float2> sell_valdw, gm_xdw;
  gbfem::DevBuf<short> sell_col16;  // columns relative to the row, where they fit in 16 bits
  bool sell_ready = false, std_spmv_dword = false, sell_cols16 = false;
  int sell_n = 0;
  long long sell_nnz = 0, sell_total = 0;
  cudaGraphExec_t gm_graph = nullptr;
  int gm_key_n = 0, gm_key_m = 0, gm_kernels = 0;
  bool gm_key_dw = false;
  unsigned char gm_key_args[256] = {};
  // DG prisms: per-element degree, block-CRS structure (block row = element)
  std::vector<int> dg_p, dg_roff, dg_bptr, dg_bcol;
  std::vector<long long> dg_boff;
  long long dg_nval = 0, dg_ninv = 0;
  int dg_ndof = 0;
  bool dg_ready = false;
  // elements per class: 1..4 prisms of degree 1..4, 5..8 tetrahedra of
  // degree 1..4
  gbfem::DevBuf<int> dg_list[9], dg_roff_d;
  gbfem::DevBuf<int> dg_flist_tc[5], dg_flist_64[5];  // prism face owners: tensor-core eligible / FP64
  // faces between a prism and a tetrahedron: half-face records per owner
  // and the owners per class that have any
  gbfem::DevBuf<int> dg_mhf_ptr, dg_mlist[9];
  gbfem::DevBuf<gbfem::DgHalfFace> dg_mhf;
  gbfem::DevBuf<long long> dg_boff_diag_d;
  gbfem::DevBuf<double> dg_val, dg_rhs;
  // DG faces: the caller's face table and the per-element incidences
  std::vector<int> dg_fa_type, dg_fa_bc, dg_fa_el, dg_fa_side, dg_fa_nodes;
  int dg_nfa = -1;  // -1: no face table (volume terms only)
  double dg_pen = 10.0;
  int dg_volume_mode = 0;  // GBFEM_DG_VOLUME_FP64 / _TC / _TF32
  int dg_face_mode = 0;    // GBFEM_DG_FACE_FP64 / _TC
  int dg_var_vol[5] = {0, 0, 0, 0, 0}, dg_var_face[5] = {0, 0, 0, 0, 0};  // launch-shape variants per degree
  gbfem::DevBuf<int> dg_hf_ptr, dg_p_d;
  gbfem::DevBuf<gbfem::DgHalfFace> dg_hf;
  // tensor-core faces: face-point configurations, basis tables at the face
  // points, faces between degree <= 3 elements (a record of each) and their
  // per-point geometry
  gbfem::DevBuf<unsigned char> dg_fcfg;
  gbfem::DevBuf<long long> dg_ftab_off;
  gbfem::DevBuf<double> dg_ftab, dg_fgeo, dg_fshare;
  gbfem::DevBuf<int> dg_tcface;
  bool dg_ftab_ok = false;
  // DG block Jacobi: inverted diagonal blocks, block e at dg_dinv_off_d[e]
  gbfem::DevBuf<double> dg_dinv;
  gbfem::DevBuf<float> dg_val32, dg_dinv32;  // FP32 copies for iterative refinement
  gbfem::DevBuf<float2> dg_valdw, dg_dinvdw;  // double-word copies for the GMRES operator
  bool dg_spmv_dword = false;
  bool dg_residual_dd = false;  // true residuals (IR, gbfem_dg_compute_residual) with compensated sums
  gbfem::DevBuf<double> ir_x, ir_r;
  gbfem::DevBuf<long long> dg_dinv_off_d;
  gbfem::DevBuf<int> dg_bptr_d, dg_bcol_d, dg_colx_d;
  gbfem::DevBuf<long long> dg_boff_d, dg_row_val_d, dg_cx_off_d;
  // timing
  float last_ms = 0.f, last_el_ms = 0.f, last_fa_ms = 0.f, last_solve_ms = 0.f, last_spmv_ms = 0.f;
  int last_spmv_count = 0, last_solve_kernels = 0;
  int last_launches = 0;
};
