/*
 * oracle.h - CPU restatement of ModFEM's integrate / assemble / solve path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg use this library, and only as the checker or
 * the timed CPU baseline; the product never links or calls it.
 *
 * Parity pinning: the restatement is checked against the reference ModFEM
 * sources compiled in this tree (oracle/ref -> oracle/_ref) through golden
 * fixtures under tests/golden (element matrices, CRS structure, assembly
 * tables, assembled values, GMRES solutions).
 */
#ifndef MODFEM_ORACLE_H
#define MODFEM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* element integrals (column-major local matrices: sm[u*n + w], u = trial/column, w = test/row) */
void orc_std_prism_element(const double *X /*18*/, const double *A /*9, a_ij row-major*/,
                           double f, double *sm /*36*/, double *rhs /*6*/);
void orc_std_prism_face(const double *X /*18*/, int side, double penalty, double g,
                        double *sm /*36*/, double *rhs /*6*/);
void orc_std_tet_element(const double *X /*12*/, const double *A /*9*/, double f,
                         double *sm /*16*/, double *rhs /*4*/);

/* first-appearance DOF numbering and CRS structure */
int orc_std_dof_order(int nel, int nv, const int *el_nodes, int nno, int *dof_of_node);
long orc_std_crs_structure(int nel, int nv, const int *el_nodes, const int *dof_of_node, int ndof,
                           int *row_ptr /*ndof+1*/, int *col_ind /*may be NULL to count*/);
/* assembly table of one integration entity: n*n value positions (table[j+i*n] for
   row j, column i) followed by n rhs positions */
void orc_crs_table(int n, const int *dofs, const int *row_ptr, const int *col_ind, int *table);

/* breadth-first first-fit colouring of integration entities sharing a DOF */
int orc_color_entities(int nent, int nv, const int *ent_dofs, int ndof, int *color);

/* whole-mesh integrate + assemble of the std prism problem (elements then
   bc faces), colour-parallel with OpenMP when nthreads > 1.  Values are
   added to val[] and rhs[] (cleared by the caller).  Returns seconds. */
double orc_std_prism_assemble(int nel, const int *el_nodes, const double *coords, const double *k_el,
                              const double *D_el, double f, int nfa, const int *fa_el,
                              const int *fa_side, double penalty, double g,
                              const int *dof_of_node, const int *row_ptr, const int *col_ind,
                              const int *el_color_ptr, const int *el_perm, int nthreads,
                              double *val, double *rhs);

/* makes orc_std_prism_assemble add |entries| (error scale for parity checks) */
void orc_set_accumulate_abs(int on);

/* v = (use_rhs ? b : 0) - A x  (CRS) */
void orc_crs_residual(int n, const int *row_ptr, const int *col_ind, const double *val,
                      int use_rhs, const double *b, const double *x, double *v);

/* left-Jacobi-preconditioned restarted GMRES(m), classical Gram-Schmidt,
   Givens rotations; stops when the preconditioned residual norm drops below
   max(tol_rel*initial, 1e-12) or after max_iter iterations.  Returns the
   number of iterations; *res_out gets the final preconditioned residual. */
int orc_gmres_jacobi(int n, const int *row_ptr, const int *col_ind, const double *val,
                     const double *b, double *x, int krylov, int max_iter, double tol_rel,
                     double *res_out, double *res_rel_out);

/* DG prisms, tensor basis of degree p = 1..4 (pdeg 101 p): ns x ns column-major
   matrix and ns load vector; returns ns (< 0 for an unsupported p) */
int orc_dg_nshape(int p);
int orc_dg_face_rule(int p, int ti, double *out);
int orc_dg_exponents(int p, int *out);
int orc_dg_prism_element(const double *X /*18*/, const double *A /*9*/, double f, int p, double *sm,
                         double *rhs);

/* DG face (interior: X2 != NULL; Dirichlet boundary: X2 == NULL); see oracle.c */
int orc_dg_face(int ftype, const double *X1, const int *loc1, int p1, const double *A1, int side1,
                const double *X2, const int *loc2, int p2, const double *A2, double pen, double g,
                double *sm, double *rhs);

#ifdef __cplusplus
}
#endif
#endif
