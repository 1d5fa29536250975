/*
 * modfem_gb300.h - C ABI of the GB300 (sm_103a) integrate / assemble / SpMV /
 * GMRES path for ModFEM's convection-diffusion problem module.
 *
 * Plain C types only (pointers, sizes); every call returns >= 0 on success
 * and < 0 on error, the ModFEM convention (include/pdh_intf.h: "returns: >=0 -
 * success code, <0 - error code"); gbfem_last_error() gives the message.
 *
 * One context holds one problem on one GPU: its mesh geometry, coefficients,
 * CRS structure and assembly tables, the assembled matrix and the Krylov
 * workspace, all resident in device memory.  Host pointers passed to the calls
 * are read or written before the call returns.  Calls on one context are not
 * thread safe; different contexts may be used from different threads.
 *
 * Numbering follows ModFEM: local element matrices are column-major
 * (Stiff_mat[u*n + w], u = trial/column, w = test/row), assembly tables give
 * for each integration entity n*n CRS value positions (entry j + i*n is row
 * dof j, column dof i) followed by n rhs positions
 * (lsd_mkb/lad_crs/las_crs_intf.c:354-438).
 */
#ifndef MODFEM_GB300_H
#define MODFEM_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gbfem_ctx_s *gbfem_ctx;

/* integration entity types (include/aph_intf.h:134-135: APC_ELEMENT, APC_FACE) */
#define GBFEM_ELEMENT 4
#define GBFEM_FACE 3
/* Comp_type (include/pdh_intf.h PDC_COMP_*): what to assemble */
#define GBFEM_COMP_SM 1
#define GBFEM_COMP_RHS 2
#define GBFEM_COMP_BOTH 3
/* element types */
#define GBFEM_PRISM 6
#define GBFEM_TETRA 4
/* scatter modes of gbfem_assemble */
#define GBFEM_SCATTER_ATOMIC 0 /* one launch, FP64 atomics (summation order varies) */
#define GBFEM_SCATTER_COLOR 1  /* one launch per colour, plain adds (deterministic) */
#define GBFEM_SCATTER_GATHER 2 /* local matrices stored, then one thread a row sums them over
                                  the incident elements in element order (deterministic, no
                                  colouring; std prisms, FP64 element arithmetic) */

/* ---------------------------------------------------------------------- */
/* context                                                                  */
/* ---------------------------------------------------------------------- */
int gbfem_version(void);
const char *gbfem_last_error(void);
/* Creates a context on CUDA device `device` with its own stream. */
int gbfem_create(gbfem_ctx *ctx, int device);
int gbfem_destroy(gbfem_ctx ctx);
/* Bytes of device memory the context holds. */
long long gbfem_device_bytes(gbfem_ctx ctx);

/* Options (no reference counterpart).
 * GBFEM_OPT_CACHE_TABLES = 1: gbfem_create_assemble_stiff_mat keeps the
 * device copies of the entity lists and assembly table between calls and
 * skips their upload while the caller passes the same pointers and sizes and
 * a sample of 257 entries of each array (first, last, equal strides) reads
 * the same as at upload.  The caller promises not to change their contents,
 * as holds in ModFEM between sir_create and sir_free; the sample catches most
 * violations (new tables at a reused address), gbfem_invalidate_tables voids
 * the cache explicitly (call it after sir_free / a new sir_create), and a new
 * structure (gbfem_set_crs_structure, gbfem_build_structure*) or setting this
 * option again voids it too.  With the cache on, the call also downloads each
 * element chunk's finished rows while the next chunk runs.
 * GBFEM_OPT_STD_ARITH: arithmetic of the std prism element matrices with an
 * isotropic coefficient (gbfem_assemble and the drop-in), GBFEM_STD_FP64
 * (default) or GBFEM_STD_DWORD: double-word float pairs on the FP32 pipe
 * (about 48 significant bits; entries within about 1e-14 of the FP64 ones,
 * vertex differences and the global assembly sums stay FP64).  Tensor
 * coefficients and tetrahedra always take FP64.
 * GBFEM_OPT_DG_SPMV_ARITH: arithmetic of the preconditioned block SpMV in
 * the Arnoldi steps of gbfem_dg_solve, GBFEM_STD_FP64 (default) or
 * GBFEM_STD_DWORD: double-word copies of the matrix and of the inverted
 * diagonal blocks, products summed on the FP32 pipes (the FP64 form is bound
 * by the FP64 pipe below HBM bandwidth); the restart residuals stay FP64.
 * GBFEM_OPT_DG_RESIDUAL: arithmetic of the DG true residual b - A x in
 * gbfem_dg_compute_residual and the outer steps of gbfem_dg_solve_ir:
 * GBFEM_RESIDUAL_FP64 (default) or GBFEM_RESIDUAL_COMPENSATED, FP64 products and sums with their rounding
 * errors carried in a second FP64 word (as accurate as twice the working
 * precision): refinement then reaches a solution accurate to about FP64
 * rounding even where the FP64 residual of a penalty-scaled system stalls
 * near 1e-11 relative.
 * GBFEM_OPT_STD_SPMV_ARITH: arithmetic of the preconditioned SpMV in the
 * Arnoldi steps of gbfem_solve, GBFEM_STD_FP64 (default) or GBFEM_STD_DWORD:
 * a double-word copy of the matrix (float pairs, 8 bytes a value like FP64)
 * with the products on the FP32 pipes; the restart residuals stay FP64. */
#define GBFEM_OPT_CACHE_TABLES 1
#define GBFEM_OPT_STD_ARITH 2
#define GBFEM_OPT_DG_SPMV_ARITH 3
#define GBFEM_OPT_DG_RESIDUAL 4
#define GBFEM_OPT_STD_SPMV_ARITH 5
#define GBFEM_STD_FP64 0
#define GBFEM_STD_DWORD 1
#define GBFEM_RESIDUAL_FP64 0
#define GBFEM_RESIDUAL_COMPENSATED 1
int gbfem_set_option(gbfem_ctx ctx, int option, long long value);
/* Voids the drop-in table cache (GBFEM_OPT_CACHE_TABLES): the next
 * gbfem_create_assemble_stiff_mat uploads its lists and table again.  No
 * reference counterpart (ModFEM frees its tables in sir_free). */
int gbfem_invalidate_tables(gbfem_ctx ctx);
/* Cache bookkeeping: how often the cache was voided, and how many drop-in
 * input arrays were copied to the device (cache misses). */
int gbfem_table_cache_stats(gbfem_ctx ctx, long long *generation, long long *uploads);

/* ---------------------------------------------------------------------- */
/* problem data                                                             */
/* ---------------------------------------------------------------------- */
/* Mesh geometry, the data the reference approximation module reads through
 * mmr_el_node_coor (mmd_prism/mms_prism_datstr.c:365) and mmr_fa_* for every
 * element and boundary face.  el_nodes: nv vertex indices (0-based) per
 * element in mmr_el_node_coor order (prism: bottom triangle then top,
 * nv = 6; tetrahedron nv = 4).  Boundary faces with a Dirichlet flag
 * (0 < bc < 10, pdr_get_bc_type in pds_conv_diff_weakform.c:1240-1252) carry
 * the reference face id (for the entity lists of the drop-in call), the
 * 0-based element and the element side (0 bottom, 1 top, 2..4 lateral over
 * triangle edge 0..2). */
int gbfem_set_mesh(gbfem_ctx ctx, int nno, const double *node_xyz, int nel, int nv,
                   const int *el_nodes, int nfa, const int *fa_id, const int *fa_el,
                   const int *fa_side, const int *fa_bc);
/* A mesh of prisms and tetrahedra together, for the DG path (gbfem_dg_*):
 * el_nv[e] = 6 (prism) or 4 (tetrahedron), the vertex count
 * mmr_el_node_coor returns in nodes[0] (mmd_prism/mms_prism_datstr.c:365);
 * el_nodes: 6 slots per element, the element's vertices first in
 * mmr_el_node_coor order (a tetrahedron's slots 4 and 5 are ignored).  The
 * DG face table (gbfem_dg_set_faces) then joins any two elements; a face
 * between a prism and a tetrahedron is a triangle (the prism's bottom or
 * top).  The std path refuses such a mesh.  No reference counterpart for the
 * DG system on it: the reference's DG module is prism-only. */
int gbfem_set_mesh_mixed(gbfem_ctx ctx, int nno, const double *node_xyz, int nel, const int *el_nv,
                         const int *el_nodes);
/* Updates node coordinates only (same topology), e.g. a moved mesh. */
int gbfem_set_node_coords(gbfem_ctx ctx, const double *node_xyz);

/* PDE coefficients in place of the per-quadrature-point callback
 * pdr_el_coeff (include/pdh_intf.h:513-612): -div(K grad u) = f with
 * K = k_el[e]*I (k_el != NULL) or the full tensor D_el[9e..9e+8] (row-major
 * a_ij multiplying d_i(test) d_j(trial), pds_conv_diff_weakform.c:757);
 * Dirichlet value g imposed by the penalty face integral with factor
 * `penalty` (1e7 in pds_conv_diff_weakform_std.c:480). */
int gbfem_set_coefficients(gbfem_ctx ctx, const double *k_el, const double *D_el, double f,
                           double g, double penalty);

/* Constrained (hanging) vertices of a refined std prism mesh, replacing
 * apr_get_constr_data (apd_std_lin/aps_std_util.c:358-395) for the
 * assembly: vertex[k] (0-based) carries no dof and stands for its
 * nr_constr[k] = 2 (mid-edge) or 4 (mid-face) constraining vertices
 * constr_id[4k..4k+nr_constr[k]-1] (the order of apr_get_constr_data),
 * each with coefficient 1/2 or 1/4.  An element with such a vertex has the
 * expanded dof list of apr_get_stiff_mat_data (aps_std_lin_intf.c:2978-
 * 3035; a constrained vertex replaced in place by its constraining vertices)
 * and gbfem_create_assemble_stiff_mat rewrites its element and boundary-face
 * matrices as that function does (:3077-3160) before the table-driven
 * scatter; its table block then holds n x n + n entries, n the expanded
 * length.  Constraining vertices are themselves unconstrained (1-irregular
 * meshes).  Call after gbfem_set_mesh (which clears them) and before
 * gbfem_set_crs_structure; n = 0 clears.  The library's own structure
 * builds and gbfem_assemble refuse a mesh with constraints: ModFEM's
 * sir_create supplies the structure and tables. */
int gbfem_set_constraints(gbfem_ctx ctx, int n, const int *vertex, const int *nr_constr, const int *constr_id);

/* CRS structure as sir_create leaves it (sid_mkb/sis_mkb_intf.c:396-1690,
 * lad_crs/las_crs_intf.c:72-300): dof index of each node (-1 if none), row
 * pointers and ascending column indices with the diagonal included. */
int gbfem_set_crs_structure(gbfem_ctx ctx, int ndof, const int *dof_of_node, long long nnz,
                            const int *row_ptr, const int *col_ind);
/* Builds the same structure in the library (first-appearance dof order over
 * the elements, utd_util/uts_ls_intf.c:182-300; sorted neighbour columns) and
 * the element/face assembly tables and colours used by gbfem_assemble. */
int gbfem_build_structure(gbfem_ctx ctx, int *ndof, long long *nnz, int *nr_colors);
/* The same structure built on the device (first-appearance ranks by an
 * atomicMin and a scan, incidence lists, per-row sorted unique columns,
 * binary-searched tables): identical arrays, no host pass over the mesh.
 * The boundary faces are coloured on the host; the elements are coloured on
 * the device by the first colour-batched gbfem_assemble (Jones-Plassmann
 * with hashed priorities: deterministic, more colours than the host's
 * first-fit walk), and the gather scatter builds its DOF -> element
 * incidence on its first call, so all scatter modes work after either
 * build; the colour and gather modes sum in a fixed order. */
int gbfem_build_structure_device(gbfem_ctx ctx, int *ndof, long long *nnz);
/* Copies the structure out (any pointer may be NULL). */
int gbfem_get_crs_structure(gbfem_ctx ctx, int *dof_of_node, int *row_ptr, int *col_ind);
/* Copies out the element assembly tables gbfem_build_structure made, in the
 * layout of lar_fill_assembly_table_int_ent_crs (las_crs_intf.c:354-438):
 * nv*nv + nv ints per element, elements in mesh order. */
int gbfem_get_element_tables(gbfem_ctx ctx, int *tables);

/* ---------------------------------------------------------------------- */
/* the hot path                                                             */
/* ---------------------------------------------------------------------- */
/* Drop-in for pdr_create_assemble_stiff_mat (include/pdh_intf.h:230-249,
 * pdd_conv_diff/linear_solver_interface/pds_conv_diff_ls_intf.c:253;
 * driver utr_create_assemble_stiff_mat, utd_util/uts_ls_intf.c:3368-4322):
 * integrates every element and boundary face in the lists and adds the
 * results into the CRS values and rhs through the given assembly tables.
 * The lists, colours and tables are the ones sir_create built; they are
 * copied to the device on every call.  crs_val (nnz) and rhs (ndof) are host
 * arrays in the caller's CRS storage (itv_crs_matrices, lad_crs/lah_crs.h);
 * when crs_val/rhs are NULL the result stays on the device for
 * gbfem_compute_residual / gbfem_solve.  The matrix is cleared first
 * (lsr_mkb_clear_matrix, sis_mkb_intf.c:2043).  Pdeg_coarse_p and Level_id
 * must describe the finest (only) level. */
int gbfem_create_assemble_stiff_mat(gbfem_ctx ctx, int Level_id, int Comp_type,
                                    const int *Pdeg_coarse_p, int Nr_int_ent,
                                    const int *L_int_ent_type, const int *L_int_ent_id,
                                    int Nr_colors_elems, const int *L_color_index_elems,
                                    int Nr_colors_faces, const int *L_color_index_faces,
                                    const int *Asse_pos_first_dof_int_ent,
                                    const int *Assembly_table, int Max_dofs_int_ent,
                                    double *crs_val, double *rhs);

/* Device-resident integrate + assemble with the tables gbfem_build_structure
 * made (no host transfers): clears and fills the device CRS values and rhs.
 * scatter_mode: GBFEM_SCATTER_ATOMIC, _COLOR or _GATHER (see above). */
int gbfem_assemble(gbfem_ctx ctx, int scatter_mode);
/* Copies the device CRS values / rhs to host arrays (either may be NULL). */
int gbfem_get_matrix(gbfem_ctx ctx, double *crs_val, double *rhs);
/* Uploads CRS values / rhs (either may be NULL), e.g. a matrix assembled elsewhere. */
int gbfem_set_matrix(gbfem_ctx ctx, const double *crs_val, const double *rhs);

/* ---------------------------------------------------------------------- */
/* DG prisms (apd_dg_prism)                                                 */
/* ---------------------------------------------------------------------- */
/* Per-element degree p = 1..4 of the tensor monomial DG basis on prisms
 * (ModFEM pdeg 101 p, (p+1)^2(p+2)/2 = 6/18/40/75 functions;
 * apr_get_el_pdeg_numshap, apd_dg_prism/aps_dg_prism_intf.c:725-775).  On
 * tetrahedra (of a tetrahedral or a mixed mesh) the complete monomial basis xi^a eta^b zeta^c,
 * a+b+c <= p, (p+1)(p+2)(p+3)/6 = 4/10/20/35 functions (no reference
 * counterpart: apd_dg_prism is prism-only), with the same weak form.
 * Coefficients from gbfem_set_coefficients (a tensor must be symmetric). */
int gbfem_dg_set_degrees(gbfem_ctx ctx, const int *p_el);
/* Face table of the mesh (tetrahedra: triangles, side k = the face
 * opposite local vertex k; on a mesh of prisms and tetrahedra each face's
 * side is that of its first neighbour's type), the data the DG weak form reads per face through
 * mmr_fa_type (mmd_prism/mms_prism_datstr.c:969), mmr_fa_bc (:993),
 * mmr_fa_eq_neig (:1140) and mmr_fa_node_coor (:1488): type 3 (triangle) or
 * 4 (quadrilateral); bc flag; two neighbours per face (0-based, second -1 on
 * the boundary, where the flag must be Dirichlet, 0 < bc < 10); the side of
 * the first neighbour the face lies on (0 bottom, 1 top, 2..4 lateral over
 * triangle edge 0..2; the normal points out of that element); four vertex
 * indices per face in mmr_fa_node_coor order (fourth -1 on triangles).
 * Without a face table only volume terms are assembled. */
int gbfem_dg_set_faces(gbfem_ctx ctx, int nfa, const int *fa_type, const int *fa_bc, const int *fa_el,
                       const int *fa_side, const int *fa_nodes);
/* Volume-integral kernel (no reference counterpart): GBFEM_DG_VOLUME_FP64
 * (FP64 pipe) or GBFEM_DG_VOLUME_TC, the tensor cores with split BF16
 * products (ten 6-bit slices per operand, exact FP32 slice sums, FP64
 * recombination), both giving the reference's element matrices to FP64
 * accuracy; or GBFEM_DG_VOLUME_TF32, the tensor cores with TF32 hi/lo
 * operands and FP32 accumulation (about 1e-6 of the entry scale: an
 * approximate matrix, for comparison).  The tensor-core kernels cover
 * p = 1..3; p = 4 elements keep the FP64 kernel.  GBFEM_DG_VOLUME_DWORD:
 * the FP64 kernel's algebra with each stiffness entry summed in double-word
 * (float pair) arithmetic on the FP32 pipes (errors of order 2^-48 of the
 * summed magnitudes), all degrees; GBFEM_DG_VOLUME_TC_DWORD: split BF16 on
 * the tensor cores for p = 1..3 and the double-word kernel for p = 4. */
#define GBFEM_DG_VOLUME_FP64 0
#define GBFEM_DG_VOLUME_TC 1
#define GBFEM_DG_VOLUME_TF32 2
#define GBFEM_DG_VOLUME_DWORD 3
#define GBFEM_DG_VOLUME_TC_DWORD 4
int gbfem_dg_set_volume_kernel(gbfem_ctx ctx, int mode);
/* Face-integral kernel (no reference counterpart): GBFEM_DG_FACE_FP64 or
 * GBFEM_DG_FACE_TC, the tensor cores with split BF16 products (seven 8-bit
 * slices per operand, exact FP32 slice sums, recombination rounded once to
 * FP64: the reference's face matrices to FP64 accuracy) for owners of degree
 * <= 3 whose neighbours all have degree <= 3; other owners keep the FP64
 * kernel; or GBFEM_DG_FACE_DWORD, the FP64 kernel's algebra with the point
 * tables in double-word (float pair) form and every entry summed on the
 * FP32 pipes by exact products and sums (errors of order 2^-48 of the summed
 * magnitudes), all degrees, prisms and tetrahedra; or
 * GBFEM_DG_FACE_TC_DWORD: the tensor cores where they apply (prisms) and the
 * double-word kernel for the other owners. */
#define GBFEM_DG_FACE_FP64 0
#define GBFEM_DG_FACE_TC 1
#define GBFEM_DG_FACE_DWORD 2
#define GBFEM_DG_FACE_TC_DWORD 3
int gbfem_dg_set_face_kernel(gbfem_ctx ctx, int mode);
/* Interior-penalty factor, pdr_ctrl_d_params(problem, 12) in the DG weak
 * form (pds_conv_diff_weakform_dg.c:516-531); default 10. */
int gbfem_dg_set_penalty(gbfem_ctx ctx, double penalty);
/* Block-CRS structure of the DG matrix (the device form of the reference's
 * lad_block storage, lsd_mkb/lad_block/lah_block.h): one dof block per
 * element in element order (the reference's DG dof entities,
 * utd_util/uts_ls_intf.c:640-700); block row e holds the element and its
 * face neighbours in ascending order; dense blocks ns_r x ns_c, column-major
 * with leading dimension ns_r (Dia / Aux of las_block_intf.c:362-520).
 * Returns the dof count and the number of stored values. */
int gbfem_dg_build_structure(gbfem_ctx ctx, int *ndof, long long *nval);
/* dof_off[nel+1] first dof of each element; bptr[nel+1], bcol[nblk] block
 * rows/columns; boff[nblk+1] value offsets.  Returns nblk. */
int gbfem_dg_get_structure(gbfem_ctx ctx, int *dof_off, int *bptr, int *bcol, long long *boff);
/* Integrates all elements (apr_num_int_el of apd_dg_prism,
 * aps_dg_prism_intf.c:1239-1728) and all faces of the face table
 * (pdr_conv_diff_comp_fa_stiff_mat_app, pds_conv_diff_weakform_dg.c:
 * 232-1140: interior penalty on interior faces, the Dirichlet form with the
 * value g of gbfem_set_coefficients on boundary faces) into the block matrix
 * and the rhs, each block entry written by one thread in a fixed order. */
int gbfem_dg_assemble(gbfem_ctx ctx);
/* Launch-shape autotuner (no reference counterpart): per degree class,
 * times the FP64 volume kernel's three shapes (threads per CTA, points per
 * shared-memory chunk) and the face kernel's two (threads per CTA) on up to
 * `sample` elements (<= 0: 16384) of the current mesh and keeps the fastest
 * for later assemblies.  Every shape sums each matrix entry in the same
 * order, so the choice never changes the results.  Overwrites the matrix:
 * assemble afterwards.  vol[5], face[5] (index = degree) receive the choices
 * and ms[20] (5 per degree: three volume, two face shapes) the timings; any
 * may be NULL. */
int gbfem_dg_autotune(gbfem_ctx ctx, int sample, int *vol, int *face, double *ms);
/* Sets the shapes explicitly (vol[p] in 0..2, face[p] in 0..1, index p = 1..4). */
int gbfem_dg_set_variants(gbfem_ctx ctx, const int *vol, const int *face);
/* Times (ms) of the last gbfem_dg_assemble: total, volume and face kernels. */
int gbfem_dg_last_timing(gbfem_ctx ctx, double *total_ms, double *volume_ms, double *face_ms, int *launches);
int gbfem_dg_get_matrix(gbfem_ctx ctx, double *vals, double *rhs);
int gbfem_dg_set_matrix(gbfem_ctx ctx, const double *vals, const double *rhs);
/* lar_compute_residual for the block storage (lar_compute_residual_block,
 * lsd_mkb/lad_block/las_block_intf.c:2266): V = (Use_rhs ? B : 0) - A*X,
 * host arrays of Ndof entries in dof-block order (B NULL: the assembled rhs). */
int gbfem_dg_compute_residual(gbfem_ctx ctx, int Use_rhs, int Ini_zero, int Ndof, const double *X,
                              const double *B, double *V);
/* GMRES(krylov) on the DG matrix (lsr_mkb_core_gmres, lsd_mkb/lsd_mkb_core/
 * lss_mkb_core.c:2317) with the reference's block Jacobi preconditioner for
 * block storage (the inverse of every diagonal block,
 * lar_fill_preconditioner_block, las_block_intf.c:1224-1330), stopping on
 * the preconditioned residual relative to the initial one (floors 1e-12).
 * x: host array of ndof (initial guess unless ini_zero; solution on return).
 * Returns the iteration count. */
int gbfem_dg_solve(gbfem_ctx ctx, int krylov, int max_iter, double tol_rel, int ini_zero, double *x,
                   double *res, double *res_rel);
/* No reference counterpart.  Mixed-precision solve of the same system:
 * FP64 iterative refinement (true residual b - A x and correction in FP64)
 * around GMRES(krylov) whose block SpMV and block-Jacobi product use FP32
 * copies of the matrix and of the inverted diagonal blocks in FP32
 * arithmetic (Arnoldi orthogonalisation stays FP64).  Each inner solve stops
 * at inner_tol relative to its initial preconditioned residual or after 10
 * restart cycles (10 krylov iterations); the loop
 * stops when ||b - A x|| <= tol_rel ||b|| or max_iter inner iterations were
 * spent.  With GBFEM_OPT_DG_RESIDUAL = GBFEM_RESIDUAL_COMPENSATED the true
 * residual carries twice the working precision and the loop also stops once
 * a correction is below 4 ulp of ||x||, or is below 1e-10 ||x|| and no
 * longer halves the previous one:
 * x is then accurate to about FP64 rounding (tol_rel below the FP64 residual
 * floor asks for exactly that).  Returns the inner iterations; *outer_steps
 * refinement steps, *rel_res the final relative true residual. */
int gbfem_dg_solve_ir(gbfem_ctx ctx, int krylov, int max_iter, double tol_rel, double inner_tol, double *x,
                      int *outer_steps, double *rel_res);

/* Drop-in for lar_compute_residual (lsd_mkb/las_intf.c:771,
 * lad_crs/las_crs_intf.c:788-856): V = (Use_rhs ? B : 0) - A*X, X, B, V host
 * arrays of Ndof entries (B NULL: the assembled rhs); Ini_zero != 0 treats X
 * as zero. */
int gbfem_compute_residual(gbfem_ctx ctx, int Use_rhs, int Ini_zero, int Ndof, const double *X,
                           const double *B, double *V);

/* No counterpart in the reference.  The same residual as
 * gbfem_compute_residual for callers that cannot let the library allocate
 * device memory: a host application whose own memory manager has already
 * claimed the GPU's memory (so a cudaMalloc would fail or steal from its
 * pool), or one calling from a latency-critical loop where the device-wide
 * synchronisation a cudaMalloc/cudaFree may imply is not acceptable.  This call
 * allocates nothing: the device copies of X and B and the result V are staged
 * in one file-scope __device__ array of 3 * GBFEM_NOALLOC_MAX_NDOF doubles
 * (6 MiB) that every GPU loading the library holds until the process exits.
 * Ndof above GBFEM_NOALLOC_MAX_NDOF is rejected with an error.  The first call
 * on a device looks up the array's device address (cudaGetSymbolAddress) with
 * that device current; make that first call before any stream capture.  All
 * calls on a device share the one array, so calls whose work overlaps on the
 * GPU (two contexts or threads on the same device at once) race and must be
 * serialised by the caller.  The matrix is the context's device-resident one,
 * set up beforehand.  The call runs on the context's device and leaves the
 * caller's current device as it found it. */
#define GBFEM_NOALLOC_MAX_NDOF 262144
int gbfem_compute_residual_noalloc(gbfem_ctx ctx, int Use_rhs, int Ini_zero, int Ndof, const double *X,
                                   const double *B, double *V);

/* Replaces lsr_mkb_core_gmres with the point-Jacobi preconditioner
 * (lsd_mkb_core/lss_mkb_core.c:2317-2660, lad_crs/las_crs_intf.c:707,857):
 * restarted GMRES(krylov), classical Gram-Schmidt, Givens rotations, stop
 * when the preconditioned residual falls below max(tol_rel*initial, 1e-12)
 * or after max_iter iterations.  x (host, ndof) holds the initial guess if
 * ini_zero == 0 and receives the solution.  Returns the iteration count. */
int gbfem_solve(gbfem_ctx ctx, int krylov, int max_iter, double tol_rel, int ini_zero, double *x,
                double *res_out, double *res_rel_out);

/* Timing of the last integrate+assemble call, from CUDA events on the
 * context stream (no reference counterpart; the reference prints wall times
 * under TIME_TEST, utd_util/uts_ls_intf.c:4312-4318): total_ms covers the
 * whole call on the device timeline (uploads, clearing, kernels, downloads),
 * element_ms only the element-integration kernel launches; launches counts
 * the library's kernels in the call. */
int gbfem_last_assembly_timing(gbfem_ctx ctx, double *total_ms, double *element_ms, int *launches);

/* Timing of the last gbfem_solve from CUDA events (no reference
 * counterpart; the reference prints its iteration time under
 * MKB_SOLVE_TIME_TEST, sid_mkb/sis_mkb_intf.c:2162-2172): the whole solve, the
 * preconditioned SpMV launches alone and how many there were, and the
 * library's kernel launches. */
int gbfem_last_solve_timing(gbfem_ctx ctx, double *total_ms, double *spmv_ms, int *spmv_count, int *launches);

/* Page-locked host memory for fast transfers (no reference counterpart). */
void *gbfem_host_alloc(long long bytes);
int gbfem_host_free(void *ptr);

/* Measures the device's FP64 FMA throughput in TFLOP/s with a register-only
 * FMA-chain kernel (no reference counterpart; the roofline denominator of the
 * FP64-bound integration kernels). */
int gbfem_measure_fp64_peak(gbfem_ctx ctx, double *tflops);

/* ---------------------------------------------------------------------- */
/* file formats (host only; no GPU needed)                                  */
/* ---------------------------------------------------------------------- */
/* Reads a jk ("gradmesh") prism mesh as mmr_import_mesh_grad does
 * (mmd_prism/mms_prism_input_gradmesh.c:30-420), in the reference's
 * numbering: sizes[3] = nno, nel, nfa (call with NULL arrays first);
 * xyz[3 nno]; el_nodes[6 nel] (0-based, mmr_el_node_coor order); the face
 * table of gbfem_dg_set_faces (type, bc, two neighbours, first neighbour's
 * side, four vertices in mmr_fa_node_coor order) in face-id order. */
int gbfem_read_jk(const char *path, int *sizes, double *xyz, int *el_nodes, int *fa_type, int *fa_bc, int *fa_el,
                  int *fa_side, int *fa_nodes);
/* field.dmp of a std scalar field as apr_write_field writes it
 * (apd_std_lin/aps_std_lin_intf.c:539-680): x indexed by dof_of_node. */
int gbfem_write_field_std(const char *path, int nno, const int *dof_of_node, const double *x);
/* field.dmp of a DG field (apd_dg_prism/aps_dg_prism_intf.c:459-560):
 * degrees p_el (1..4, written as -101 p), coefficients of element e at
 * x[dof_off[e] .. dof_off[e+1]).  uniform != 0 writes one degree line (the
 * first element's), as the reference does for a field created with one
 * degree (its field_p->uniform), whatever the element degrees are later;
 * uniform == 0 one line per element. */
int gbfem_write_field_dg(const char *path, int nel, const int *p_el, const int *dof_off, const double *x,
                         int uniform);

/* ---------------------------------------------------------------------- */
/* batched DG volume integrals of mixed element types and degrees          */
/* ---------------------------------------------------------------------- */
/* One persistent kernel, replayed as a CUDA graph, integrates the element
 * matrices and load vectors of any mix of DG prisms (tensor basis, as
 * apr_num_int_el of apd_dg_prism, aps_dg_prism_intf.c:1239-1728) and affine
 * DG tetrahedra (complete monomial basis xi^a eta^b zeta^c, a+b+c <= p, on
 * the reference tetrahedron; no reference counterpart, apd_dg_prism is
 * prism-only) of degrees 1..4: -div(A grad u) = f, volume terms.  The blocks
 * are stored prisms first, then tetrahedra, each ns x ns column-major
 * (ns = 6, 18, 40, 75 for prisms; 4, 10, 20, 35 for tetrahedra), load
 * vectors likewise.  The prism blocks and load vectors equal, bit for bit,
 * the diagonal blocks and rhs gbfem_dg_assemble produces without a face
 * table. */
typedef struct gbfem_batch_s *gbfem_batch;
int gbfem_batch_create(gbfem_batch *batch, int device);
int gbfem_batch_destroy(gbfem_batch batch);
/* prism_xyz[18 np] (mmr_el_node_coor order), prism_A[9 np] row-major
 * symmetric tensors, prism_p[np]; tet_xyz[12 nt], tet_A[9 nt], tet_p[nt].
 * nval, nrhs: output sizes of the default layout. */
int gbfem_batch_set(gbfem_batch batch, int np, const double *prism_xyz, const double *prism_A, const int *prism_p,
                    int nt, const double *tet_xyz, const double *tet_A, const int *tet_p, double f, long long *nval,
                    long long *nrhs);
/* Scatter target: element e (prisms first, then tetrahedra) writes its block
 * at val_off[e] of a value array of nval entries and its load vector at
 * rhs_off[e] of an rhs of nrhs, e.g. the diagonal blocks of a block-CRS
 * matrix (gbfem_dg_get_structure's layout); entries no element writes stay
 * zero. */
int gbfem_batch_set_layout(gbfem_batch batch, const long long *val_off, const int *rhs_off, long long nval,
                           long long nrhs);
/* Launch variant per degree (index 1..4): prisms 0..2 (threads per element,
 * quadrature points per shared-memory chunk), tetrahedra 0..4 (8 << v
 * elements per tile).  Either pointer may be NULL.  Every variant gives the
 * same bits. */
int gbfem_batch_set_variants(gbfem_batch batch, const int *prism_v, const int *tet_v);
/* Arithmetic of the prism stiffness sums: 0 FP64 (default), 1 double word
 * (float pairs on the FP32 pipes, exact products and TwoSum chains; entries
 * within about 2^-48 of the summed magnitudes).  Tetrahedra (6 FMAs per
 * entry against exact reference matrices) stay FP64. */
int gbfem_batch_set_arith(gbfem_batch batch, int dword);
/* Times every variant of every (type, degree) class present on up to
 * `sample` of its elements (<= 0: 16384), keeps the fastest.  prism_v[5],
 * tet_v[5] receive the choices, ms[50] the timings ((type*5 + p)*5 + v,
 * -1 where not timed); any may be NULL.  Overwrites the output: run after. */
int gbfem_batch_autotune(gbfem_batch batch, int sample, int *prism_v, int *tet_v, double *ms);
/* Replays the graph; ms: device time of the launch.  Returns the tiles. */
int gbfem_batch_run(gbfem_batch batch, double *ms);
int gbfem_batch_get(gbfem_batch batch, double *vals, double *rhs);

/* ---------------------------------------------------------------------- */
/* serving (no counterpart in the reference)                                */
/* ---------------------------------------------------------------------- */
/* A server takes independent heat problems as they arrive and integrates,
 * assembles and solves them on one GPU with continuous batching.  std and DG
 * requests run in two lanes, each with its own FIFO queue, half of the
 * max_active slots (more while the other lane has nobody waiting), CUDA
 * stream and step graph, so std requests neither wait for DG requests'
 * solves nor queue behind them; a request is admitted when its lane has a
 * slot and its device footprint fits in the shared HBM budget.  Worker
 * threads upload, build, integrate and assemble each admitted request on its
 * own stream (std requests before DG ones) while the engine thread advances
 * each lane's requests in the solve phase together, one GMRES iteration per
 * step with batched kernels and the GMRES scalar logic on the device; large
 * std requests are solved alone on their own stream instead
 * (GBFEM_SERVE_OPT_SOLO_DOFS, GBFEM_SERVE_OPT_STD_PRECEDENCE).  A request's
 * result does not depend on the other requests in the mix (bit-identical
 * alone and together).  The numerics per request are those of
 * gbfem_assemble + gbfem_solve (std) and gbfem_dg_assemble + gbfem_dg_solve
 * (DG): same assembly, same GMRES(krylov) with (block) Jacobi, stopping on the
 * preconditioned residual relative to the initial one. */
#define GBFEM_SERVE_STD 0
#define GBFEM_SERVE_DG 1
typedef struct gbfem_server_s *gbfem_server;
typedef struct {
  int kind;               /* GBFEM_SERVE_STD or GBFEM_SERVE_DG */
  int dg_p;               /* DG degree of every element (1..4) */
  int nno;                /* nodes, node_xyz[3 nno] */
  const double *node_xyz;
  int nel;                /* prisms, el_nodes[6 nel] (0-based) */
  const int *el_nodes;
  const double *k_el;     /* isotropic coefficient per element */
  double f, g;            /* source, Dirichlet value */
  int nbf;                /* std: Dirichlet boundary faces (element, side) */
  const int *bf_el, *bf_side;
  int nfa;                /* DG: face table as gbfem_dg_set_faces */
  const int *fa_type, *fa_bc, *fa_el, *fa_side, *fa_nodes;
  double dg_penalty;      /* <= 0: 10 */
  int krylov, max_iter;   /* GMRES(krylov), krylov <= 64 */
  double tol_rel;
} gbfem_serve_request;
/* hbm_budget <= 0: 85% of the free device memory; max_active: requests in
 * preparation or solve at once (<= 64); prep_threads: host workers. */
int gbfem_server_create(gbfem_server *srv, int device, long long hbm_budget, int max_active, int prep_threads);
/* Finishes the requests being prepared or solved, drops the queued ones. */
int gbfem_server_destroy(gbfem_server srv);
/* Copies the request's inputs; returns its id (>= 0) or < 0. */
long long gbfem_server_submit(gbfem_server srv, const gbfem_serve_request *req);
/* 1 finished, 0 timed out (timeout_s < 0 waits without limit), < 0 failed. */
int gbfem_server_wait(gbfem_server srv, long long id, double timeout_s);
/* Solution (dof order of the library's structure), GMRES iterations,
 * relative preconditioned residual and times[5] in seconds: queued,
 * preparation, waiting for a solve slot, solve, submit-to-done latency.
 * Returns the solution length. */
int gbfem_server_result(gbfem_server srv, long long id, double *x, long long nx, int *iters, double *rel_res,
                        double *times);
/* Forgets a finished request's result. */
int gbfem_server_release(gbfem_server srv, long long id);
/* Cancels a request: a queued or prepared one leaves at once, one being
 * prepared or solved at the end of its preparation or at the engine's next
 * poll; its device memory returns to the budget and gbfem_server_wait then
 * reports it failed ("cancelled").  Returns 0, or 1 when the request had
 * already finished, failed or been cancelled. */
int gbfem_server_cancel(gbfem_server srv, long long id);
/* GBFEM_SERVE_OPT_STEPS_PER_POLL: engine steps launched between two host
 * reads of the requests' phases (1..64, default 4): fewer host round trips
 * against up to that many idle steps for a request that has finished.
 * GBFEM_SERVE_OPT_FAIL_PREPARATIONS: the next `value` request preparations
 * fail as a device allocation would ("injected allocation failure"), before
 * any device work; for testing how callers and the admission accounting
 * handle failed requests (the failure is made on the host). */
#define GBFEM_SERVE_OPT_STEPS_PER_POLL 1
#define GBFEM_SERVE_OPT_FAIL_PREPARATIONS 2
/* GBFEM_SERVE_OPT_SOLO_DOFS: std requests with at least this many dofs
 * (default 40,000; 0: none) are not batched into the engine's steps: they
 * are admitted on the HBM budget alone (no lane slot), prepared first, and
 * solved by one of eight solo threads with gbfem_solve's device-resident
 * GMRES (sliced-ELL SpMV, restart cycles as a CUDA graph) on the request's
 * own highest-priority stream, beside the batched lanes.  Same stopping
 * rule; the result does not depend on the other requests either way. */
#define GBFEM_SERVE_OPT_SOLO_DOFS 3
/* GBFEM_SERVE_OPT_STD_PRECEDENCE: 1 (default): while a solo-sized std
 * request is being prepared or solved, the engine launches no new DG-lane
 * steps (DG steps already in flight finish), so the large latency-bound std
 * requests have the GPU to themselves and the DG requests, whose solves run
 * for seconds, wait for those windows; 0: both lanes always step. */
#define GBFEM_SERVE_OPT_STD_PRECEDENCE 4
int gbfem_server_set_option(gbfem_server srv, int option, long long value);
/* stats[8]: engine steps, kernel launches, peak active requests, peak
 * bytes charged, budget, bytes charged now, queued, active. */
int gbfem_server_stats(gbfem_server srv, long long *stats);
/* Device bytes a request is charged at admission (host estimate). */
long long gbfem_serve_footprint(const gbfem_serve_request *req);

#ifdef __cplusplus
}
#endif
#endif
