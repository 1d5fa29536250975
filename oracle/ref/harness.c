/*
 * harness.c - test infrastructure only.
 *
 * Links the reference ModFEM sources (mesh module mmd_prism, approximation
 * module apd_std_lin or apd_dg_prism, the conv-diff weak forms, the MKB solver
 * interface sid_mkb and the solver library lsd_mkb, plus the assembly driver in
 * utd_util/uts_ls_intf.c) into one shared library that the parity tests and the
 * golden-fixture generator call through ctypes.  Nothing in this file is part
 * of the product; it plays the role of ModFEM's problem-dependent module
 * (pdr_* callbacks), supplies BLAS/LAPACK routines, and stubs out I/O.
 *
 * The problem it states is the steady Poisson/heat problem
 *     -div(K grad u) = f   in the mesh domain,   u = g on faces with 0<bc<10,
 * with K an isotropic scalar k per element (or a full 3x3 tensor per element)
 * and f, g constants, Dirichlet data imposed by the reference's own 1e7
 * penalty face integrals (pdd_conv_diff/weak_formulation/approx_std/
 * pds_conv_diff_weakform_std.c:480).
 *
 * Callback shapes follow pdd_conv_diff/linear_solver_interface/
 * pds_conv_diff_ls_intf.c:253-620 (pdr_create_assemble_stiff_mat,
 * pdr_assemble_local_stiff_mat[_with_table], pdr_comp_stiff_mat,
 * pdr_select_el_coeff_vect, pdr_el_coeff) and include/pdh_intf.h.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <time.h>

#include "mmh_intf.h"
#include "aph_intf.h"
#include "sih_intf.h"
#include "pdh_intf.h"
#include "uth_intf.h"
#include "sih_mkb.h"
#include "lah_crs.h"

/* ------------------------------------------------------------------ */
/* problem-module constants (same values as pds_conv_diff_ls_intf.c)   */
/* ------------------------------------------------------------------ */
const int PDC_ELEMENT = APC_ELEMENT;
const int PDC_FACE = APC_FACE;
const int PDC_EDGE = APC_EDGE;
const int PDC_VERTEX = APC_VERTEX;
const int PDC_NO_COMP = APC_NO_COMP;
const int PDC_COMP_SM = APC_COMP_SM;
const int PDC_COMP_RHS = APC_COMP_RHS;
const int PDC_COMP_BOTH = APC_COMP_BOTH;

int pdv_conv_diff_current_problem_id = 1;
FILE *utv_log_out = NULL;

/* ------------------------------------------------------------------ */
/* harness state                                                       */
/* ------------------------------------------------------------------ */
static int h_mesh_id = 0, h_field_id = 0, h_solver_id = -1;
static int h_nel_coef = 0;
static double *h_k = NULL;      /* [max_el+1] isotropic coefficient per element */
static double *h_D = NULL;      /* [9*(max_el+1)] tensor per element (row-major a_ij) */
static int h_aniso = 0;
static double h_f = 1.0;        /* source */
static double h_g = 0.0;        /* Dirichlet value */
static double h_dg_penalty = 10.0;
static double *h_sol = NULL;    /* solution dofs per dof entity id (nrdofs each) */
static int h_sol_stride = 1, h_sol_cap = 0;
static double h_last_assembly_s = 0.0;

static double wall(void)
{
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

/* ------------------------------------------------------------------ */
/* utilities normally provided by utd_system / utd_util C++ files      */
/* ------------------------------------------------------------------ */
static double h_t0 = -1.0;
void time_init(void) { h_t0 = wall(); }
double time_clock(void)
{
  if (h_t0 < 0) time_init();
  return wall() - h_t0;
}
const char *utr_log_pre(void) { return ""; }

/* ------------------------------------------------------------------ */
/* Element colouring.  utd_util/uts_coloring.cpp is Boost-based C++;   */
/* its selected routine utr_first_fit_coloring_with_front             */
/* (uts_coloring.cpp:61, chosen at :254-268) is a breadth-first walk   */
/* that gives each visited element the smallest colour unused by its   */
/* already coloured neighbours.  Restated here in plain C.             */
/* ------------------------------------------------------------------ */
int utr_generate_int_ent_coloring(const int nElems, int **elem2elem, int *Elem_colors)
{
  int i, nr_color = 0, colored = 0;
  int *queue = (int *)malloc((nElems + 1) * sizeof(int));
  char *seen = (char *)calloc(nElems + 1, 1);
  int cap = 64;
  char *used = (char *)calloc(cap, 1);
  int qh = 0, qt = 0;
  for (i = 0; i < nElems; i++) Elem_colors[i] = -1;
  if (nElems == 0) { free(queue); free(seen); free(used); return 0; }
  int start = 0;
  while (colored < nElems) {
    if (qh == qt) {
      while (start < nElems && Elem_colors[start] != -1) start++;
      if (start >= nElems) break;
      queue[qt++] = start;
      seen[start] = 1;
    }
    int cur = queue[qh++];
    for (i = 1; i <= elem2elem[cur][0]; i++) {
      int nb = elem2elem[cur][i];
      if (Elem_colors[nb] >= 0) used[Elem_colors[nb]] = 1;
      if (!seen[nb]) { seen[nb] = 1; queue[qt++] = nb; }
    }
    int c = 0;
    while (c < nr_color && used[c]) c++;
    if (c == nr_color) {
      nr_color++;
      if (nr_color >= cap) { used = (char *)realloc(used, 2 * cap); memset(used + cap, 0, cap); cap *= 2; }
    }
    Elem_colors[cur] = c;
    colored++;
    for (i = 1; i <= elem2elem[cur][0]; i++) {
      int nb = elem2elem[cur][i];
      if (Elem_colors[nb] >= 0) used[Elem_colors[nb]] = 0;
    }
  }
  free(queue); free(seen); free(used);
  return nr_color;
}

/* ------------------------------------------------------------------ */
/* BLAS / LAPACK, written from the netlib reference definitions       */
/* (column-major, Fortran calling convention).                         */
/* ------------------------------------------------------------------ */
double ddot_(int *n, double *x, int *incx, double *y, int *incy)
{
  double s = 0.0; int i;
  for (i = 0; i < *n; i++) s += x[i * (*incx)] * y[i * (*incy)];
  return s;
}
double dnrm2_(int *n, double *x, int *incx)
{
  double scale = 0.0, ssq = 1.0; int i;
  if (*n < 1) return 0.0;
  for (i = 0; i < *n; i++) {
    double v = x[i * (*incx)];
    if (v != 0.0) {
      double a = fabs(v);
      if (scale < a) { ssq = 1.0 + ssq * (scale / a) * (scale / a); scale = a; }
      else ssq += (a / scale) * (a / scale);
    }
  }
  return scale * sqrt(ssq);
}
void daxpy_(int *n, double *a, double *x, int *incx, double *y, int *incy)
{
  int i;
  if (*a == 0.0) return;
  for (i = 0; i < *n; i++) y[i * (*incy)] += (*a) * x[i * (*incx)];
}
void dscal_(int *n, double *a, double *x, int *incx)
{
  int i;
  for (i = 0; i < *n; i++) x[i * (*incx)] *= *a;
}
void dcopy_(int *n, double *x, int *incx, double *y, int *incy)
{
  int i;
  for (i = 0; i < *n; i++) y[i * (*incy)] = x[i * (*incx)];
}
void drot_(int *n, double *x, int *incx, double *y, int *incy, double *c, double *s)
{
  int i;
  for (i = 0; i < *n; i++) {
    double xv = x[i * (*incx)], yv = y[i * (*incy)];
    x[i * (*incx)] = (*c) * xv + (*s) * yv;
    y[i * (*incy)] = (*c) * yv - (*s) * xv;
  }
}
void drotg_(double *a, double *b, double *c, double *s)
{
  double roe = (fabs(*a) > fabs(*b)) ? *a : *b;
  double scale = fabs(*a) + fabs(*b), r, z;
  if (scale == 0.0) { *c = 1.0; *s = 0.0; r = 0.0; z = 0.0; }
  else {
    double as = *a / scale, bs = *b / scale;
    r = scale * sqrt(as * as + bs * bs);
    if (roe < 0) r = -r;
    *c = *a / r; *s = *b / r;
    z = 1.0;
    if (fabs(*a) > fabs(*b)) z = *s;
    if (fabs(*b) >= fabs(*a) && *c != 0.0) z = 1.0 / *c;
  }
  *a = r; *b = z;
}
static int lsame(const char *a, char b) { return (a[0] | 32) == (b | 32); }
void dtrsv_(char *uplo, char *trans, char *diag, int *n, double *A, int *lda, double *x, int *incx)
{
  int N = *n, L = *lda, ix = *incx, i, j;
  int up = lsame(uplo, 'U'), tr = !lsame(trans, 'N'), unit = lsame(diag, 'U');
#define AA(i, j) A[(i) + (size_t)(j) * L]
  if (!tr) {
    if (up) {
      for (j = N - 1; j >= 0; j--) {
        if (!unit) x[j * ix] /= AA(j, j);
        for (i = j - 1; i >= 0; i--) x[i * ix] -= x[j * ix] * AA(i, j);
      }
    } else {
      for (j = 0; j < N; j++) {
        if (!unit) x[j * ix] /= AA(j, j);
        for (i = j + 1; i < N; i++) x[i * ix] -= x[j * ix] * AA(i, j);
      }
    }
  } else {
    if (up) {
      for (j = 0; j < N; j++) {
        double t = x[j * ix];
        for (i = 0; i < j; i++) t -= AA(i, j) * x[i * ix];
        if (!unit) t /= AA(j, j);
        x[j * ix] = t;
      }
    } else {
      for (j = N - 1; j >= 0; j--) {
        double t = x[j * ix];
        for (i = N - 1; i > j; i--) t -= AA(i, j) * x[i * ix];
        if (!unit) t /= AA(j, j);
        x[j * ix] = t;
      }
    }
  }
#undef AA
}
void dgemv_(char *trans, int *m, int *n, double *alpha, double *A, int *lda, double *x, int *incx,
            double *beta, double *y, int *incy)
{
  int M = *m, N = *n, L = *lda, i, j;
  int tr = !lsame(trans, 'N');
  int leny = tr ? N : M, lenx = tr ? M : N;
  (void)lenx;
  for (i = 0; i < leny; i++) y[i * (*incy)] = (*beta == 0.0) ? 0.0 : (*beta) * y[i * (*incy)];
  if (*alpha == 0.0) return;
  if (!tr) {
    for (j = 0; j < N; j++) {
      double t = (*alpha) * x[j * (*incx)];
      for (i = 0; i < M; i++) y[i * (*incy)] += t * A[i + (size_t)j * L];
    }
  } else {
    for (j = 0; j < N; j++) {
      double t = 0.0;
      for (i = 0; i < M; i++) t += A[i + (size_t)j * L] * x[i * (*incx)];
      y[j * (*incy)] += (*alpha) * t;
    }
  }
}
void dgemm_(char *ta, char *tb, int *m, int *n, int *k, double *alpha, double *A, int *lda,
            double *B, int *ldb, double *beta, double *C, int *ldc)
{
  int M = *m, N = *n, K = *k, i, j, l;
  int tA = !lsame(ta, 'N'), tB = !lsame(tb, 'N');
  for (j = 0; j < N; j++)
    for (i = 0; i < M; i++) {
      double s = 0.0;
      for (l = 0; l < K; l++) {
        double a = tA ? A[l + (size_t)i * (*lda)] : A[i + (size_t)l * (*lda)];
        double b = tB ? B[j + (size_t)l * (*ldb)] : B[l + (size_t)j * (*ldb)];
        s += a * b;
      }
      C[i + (size_t)j * (*ldc)] = (*alpha) * s + ((*beta == 0.0) ? 0.0 : (*beta) * C[i + (size_t)j * (*ldc)]);
    }
}
void dgetrf_(int *m, int *n, double *A, int *lda, int *ipiv, int *info)
{
  int M = *m, N = *n, L = *lda, i, j, k;
  int mn = M < N ? M : N;
  *info = 0;
  for (k = 0; k < mn; k++) {
    int p = k; double mx = fabs(A[k + (size_t)k * L]);
    for (i = k + 1; i < M; i++) if (fabs(A[i + (size_t)k * L]) > mx) { mx = fabs(A[i + (size_t)k * L]); p = i; }
    ipiv[k] = p + 1;
    if (A[p + (size_t)k * L] == 0.0) { if (*info == 0) *info = k + 1; continue; }
    if (p != k) for (j = 0; j < N; j++) { double t = A[k + (size_t)j * L]; A[k + (size_t)j * L] = A[p + (size_t)j * L]; A[p + (size_t)j * L] = t; }
    for (i = k + 1; i < M; i++) A[i + (size_t)k * L] /= A[k + (size_t)k * L];
    for (j = k + 1; j < N; j++) {
      double t = A[k + (size_t)j * L];
      if (t != 0.0) for (i = k + 1; i < M; i++) A[i + (size_t)j * L] -= A[i + (size_t)k * L] * t;
    }
  }
}
void dgetrs_(char *trans, int *n, int *nrhs, double *A, int *lda, int *ipiv, double *B, int *ldb, int *info)
{
  int N = *n, r, i;
  *info = 0;
  int one = 1;
  for (r = 0; r < *nrhs; r++) {
    double *b = B + (size_t)r * (*ldb);
    if (lsame(trans, 'N')) {
      for (i = 0; i < N; i++) { int p = ipiv[i] - 1; if (p != i) { double t = b[i]; b[i] = b[p]; b[p] = t; } }
      dtrsv_("L", "N", "U", n, A, lda, b, &one);
      dtrsv_("U", "N", "N", n, A, lda, b, &one);
    } else {
      dtrsv_("U", "T", "N", n, A, lda, b, &one);
      dtrsv_("L", "T", "U", n, A, lda, b, &one);
      for (i = N - 1; i >= 0; i--) { int p = ipiv[i] - 1; if (p != i) { double t = b[i]; b[i] = b[p]; b[p] = t; } }
    }
  }
}
void dgetri_(int *n, double *A, int *lda, int *ipiv, double *work, int *lwork, int *info)
{
  int N = *n, L = *lda, i, j;
  double *inv = (double *)calloc((size_t)N * N, sizeof(double));
  (void)work; (void)lwork;
  for (i = 0; i < N; i++) inv[i + (size_t)i * N] = 1.0;
  dgetrs_("N", n, n, A, lda, ipiv, inv, n, info);
  for (j = 0; j < N; j++) for (i = 0; i < N; i++) A[i + (size_t)j * L] = inv[i + (size_t)j * N];
  free(inv);
}

/* ------------------------------------------------------------------ */
/* pdr_* callbacks                                                      */
/* ------------------------------------------------------------------ */
int pdr_ctrl_i_params(int Problem_id, int Num)
{
  (void)Problem_id;
  switch (Num) {
    case 2: return h_mesh_id;
    case 3: return h_field_id;
    case 4: return 1;   /* number of solution vectors */
    case 5: return 1;   /* nreq */
    case 6: return h_solver_id;
    default: return 0;
  }
}
double pdr_ctrl_d_params(int Problem_id, int Num)
{
  (void)Problem_id;
  if (Num == 12) return h_dg_penalty;
  return 0.0;
}
/* time-integration parameters: steady problem, fully implicit (index 2 is the
   implicitness parameter the DG face terms scale by, index 4 the time) */
double pdr_time_d_params(int Problem_id, int Num)
{
  (void)Problem_id;
  if (Num == 2) return 1.0;
  return 0.0;
}
int pdr_problem_name(int Problem_id, char *Name) { (void)Problem_id; strcpy(Name, "GB300_POISSON"); return 1; }

int pdr_get_bc_type(int Fa_bc)
{
  if (Fa_bc <= 0) return PDC_INTERIOR;
  else if (Fa_bc < PDC_MAXBCVAL) return PDC_BC_DIRI;
  else if (Fa_bc < 2 * PDC_MAXBCVAL) return PDC_BC_NEUM;
  else return PDC_BC_MIXED;
}

void pdr_fa_coeff(int Face, int BC_flag, int Elem, int Mat_num, double Hsize, double Time, int Pdeg,
                  double *Xcoor, double *Vec_norm, double *U_val, double *U_x, double *U_y, double *U_z,
                  double *Anx, double *Any, double *Anz, double *Bn, double *Fval, double *Gval,
                  double *Qn, double *Vel_norm)
{
  /* normal diffusion An_j = sum_i a_ij n_i of the element's coefficient, as
     pdr_fa_coeff builds it (pds_conv_diff_weakform.c:654-695); Dirichlet data */
  double a[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  (void)Face; (void)Mat_num; (void)Hsize; (void)Time; (void)Pdeg; (void)Xcoor;
  (void)U_val; (void)U_x; (void)U_y; (void)U_z;
  if (h_aniso && h_D != NULL && Elem >= 0 && Elem <= h_nel_coef) {
    memcpy(a, h_D + 9 * (size_t)Elem, 9 * sizeof(double));
  } else {
    double k = (h_k != NULL && Elem >= 0 && Elem <= h_nel_coef) ? h_k[Elem] : 1.0;
    a[0] = a[4] = a[8] = k;
  }
  Anx[0] = a[0] * Vec_norm[0] + a[3] * Vec_norm[1] + a[6] * Vec_norm[2];
  Any[0] = a[1] * Vec_norm[0] + a[4] * Vec_norm[1] + a[7] * Vec_norm[2];
  Anz[0] = a[2] * Vec_norm[0] + a[5] * Vec_norm[1] + a[8] * Vec_norm[2];
  Bn[0] = 0.0; Fval[0] = 0.0; Gval[0] = 0.0; Qn[0] = 0.0; Vel_norm[0] = 0.0;
  if (pdr_get_bc_type(BC_flag) == PDC_BC_DIRI) Fval[0] = h_g;
}

int pdr_select_el_coeff_vect(int Problem_id, int *Coeff_vect_ind)
{
  int i;
  (void)Problem_id;
  for (i = 0; i <= 22; i++) Coeff_vect_ind[i] = 0;
  Coeff_vect_ind[0] = 1;
  if (h_aniso) {
    for (i = 2; i <= 10; i++) Coeff_vect_ind[i] = 1;
  } else {
    /* the same selection as the reference's DIFF_IN_CUBE problem
       (pds_conv_diff_weakform.c:103-115): axx, ayy, azz, sval */
    Coeff_vect_ind[2] = 1; Coeff_vect_ind[6] = 1; Coeff_vect_ind[10] = 1;
  }
  Coeff_vect_ind[22] = 1;
  return 1;
}


int pdr_el_coeff(int Problem_id, int Elem, int Mat_num, double Hsize, int Pdeg, double *X_loc,
                 double *Base_phi, double *Base_dphix, double *Base_dphiy, double *Base_dphiz,
                 double *Xcoor, double *Uk_val, double *Uk_x, double *Uk_y, double *Uk_z,
                 double *Un_val, double *Un_x, double *Un_y, double *Un_z,
                 double *Mval, double *Axx, double *Axy, double *Axz, double *Ayx, double *Ayy, double *Ayz,
                 double *Azx, double *Azy, double *Azz, double *Bx, double *By, double *Bz,
                 double *Tx, double *Ty, double *Tz, double *Cval, double *Lval,
                 double *Qx, double *Qy, double *Qz, double *Sval)
{
  (void)Problem_id; (void)Mat_num; (void)Hsize; (void)Pdeg; (void)X_loc; (void)Base_phi;
  (void)Base_dphix; (void)Base_dphiy; (void)Base_dphiz; (void)Xcoor; (void)Uk_val; (void)Uk_x;
  (void)Uk_y; (void)Uk_z; (void)Un_val; (void)Un_x; (void)Un_y; (void)Un_z;
  double k = 1.0;
  if (h_k != NULL && Elem >= 0 && Elem <= h_nel_coef) k = h_k[Elem];
  Mval[0] = 0.0;
  Axx[0] = Ayy[0] = Azz[0] = k;
  Axy[0] = Axz[0] = Ayx[0] = Ayz[0] = Azx[0] = Azy[0] = 0.0;
  if (h_aniso && h_D != NULL && Elem >= 0 && Elem <= h_nel_coef) {
    const double *D = h_D + 9 * (size_t)Elem;
    Axx[0] = D[0]; Axy[0] = D[1]; Axz[0] = D[2];
    Ayx[0] = D[3]; Ayy[0] = D[4]; Ayz[0] = D[5];
    Azx[0] = D[6]; Azy[0] = D[7]; Azz[0] = D[8];
  }
  Bx[0] = By[0] = Bz[0] = 0.0;
  Tx[0] = Ty[0] = Tz[0] = 0.0;
  Cval[0] = 0.0; Lval[0] = 0.0;
  Qx[0] = Qy[0] = Qz[0] = 0.0;
  Sval[0] = h_f;
  return 0;
}

/* weak-form entry points compiled from the reference (std or dg variant) */
extern int pdr_conv_diff_comp_el_stiff_mat_app(int, int, int, int, int *, int *, int *, int *, int *,
                                               double *, double *, char *);
extern int pdr_conv_diff_comp_fa_stiff_mat_app(int, int, int, int, int *, int *, int *, int *, int *,
                                               double *, double *, char *);

int pdr_comp_stiff_mat(int Problem_id, int Int_ent_type, int Int_ent_id, int Comp_sm, int *Pdeg_vec,
                       int *Nr_dof_ent, int *List_dof_ent_type, int *List_dof_ent_id,
                       int *List_dof_ent_nrdof, int *Nrdofs_loc, double *Stiff_mat,
                       double *Rhs_vect, char *Rewr_dofs)
{
  int pdeg = (Pdeg_vec == NULL) ? -10 : Pdeg_vec[0];
  if (Int_ent_type == PDC_ELEMENT)
    pdr_conv_diff_comp_el_stiff_mat_app(Problem_id, Int_ent_id, Comp_sm, pdeg, Nr_dof_ent,
                                        List_dof_ent_type, List_dof_ent_id, List_dof_ent_nrdof,
                                        Nrdofs_loc, Stiff_mat, Rhs_vect, Rewr_dofs);
  else if (Int_ent_type == PDC_FACE)
    pdr_conv_diff_comp_fa_stiff_mat_app(Problem_id, Int_ent_id, Comp_sm, pdeg, Nr_dof_ent,
                                        List_dof_ent_type, List_dof_ent_id, List_dof_ent_nrdof,
                                        Nrdofs_loc, Stiff_mat, Rhs_vect, Rewr_dofs);
  else { fprintf(stderr, "wrong integration entity type\n"); exit(-1); }
  return 1;
}

int pdr_assemble_local_stiff_mat(int Problem_id, int Level_id, int Comp_type, int Nr_dof_ent,
                                 int *L_dof_ent_type, int *L_dof_ent_id, int *L_dof_ent_nrdofs,
                                 double *Stiff_mat, double *Rhs_vect, char *Rewr_dofs)
{
  (void)Problem_id;
  sir_assemble_local_stiff_mat(h_solver_id, Level_id, Comp_type, Nr_dof_ent, L_dof_ent_type,
                               L_dof_ent_id, L_dof_ent_nrdofs, Stiff_mat, Rhs_vect, Rewr_dofs);
  return 1;
}
int pdr_assemble_local_stiff_mat_with_table(int Problem_id, int Level_id, int Comp_type, int Nr_dof_ent,
                                            int *Assembly_table_int_ent, double *Stiff_mat,
                                            double *Rhs_vect, char *Rewr_dofs)
{
  (void)Problem_id;
  sir_assemble_local_stiff_mat_with_table(h_solver_id, Level_id, Comp_type, Nr_dof_ent,
                                          Assembly_table_int_ent, Stiff_mat, Rhs_vect, Rewr_dofs);
  return 1;
}

#ifndef HARNESS_GB300_SHIM
/* the reference's CPU driver; the GB300 shim build takes
   modfem_gb300/modfem_side/pds_gb300_ls_intf.c's function instead */
int pdr_create_assemble_stiff_mat(int Problem_id, int Level_id, int Comp_type, int *Pdeg_coarse_p,
                                  int Nr_int_ent, int *L_int_ent_type, int *L_int_ent_id,
                                  int Nr_colors_elems, int *L_color_index_elems, int Nr_colors_faces,
                                  int *L_color_index_faces, int *Asse_pos_first_dof_int_ent,
                                  int *Assembly_table, int Max_dofs_int_ent)
{
  double t = wall();
  utr_create_assemble_stiff_mat(Problem_id, Level_id, Comp_type, Pdeg_coarse_p, Nr_int_ent,
                                L_int_ent_type, L_int_ent_id, Nr_colors_elems, L_color_index_elems,
                                Nr_colors_faces, L_color_index_faces, Asse_pos_first_dof_int_ent,
                                Assembly_table, Max_dofs_int_ent);
  h_last_assembly_s = wall() - t;
  return 1;
}
#endif

int pdr_get_list_ent(int Problem_id, int *Nr_int_ent, int **List_int_ent_type, int **List_int_ent_id,
                     int *Nr_dof_ent, int **List_dof_ent_type, int **List_dof_ent_id,
                     int **List_dof_ent_nrdofs, int *Nrdofs_glob, int *Max_dofs_per_dof_ent)
{
  return utr_get_list_ent(Problem_id, Nr_int_ent, List_int_ent_type, List_int_ent_id, Nr_dof_ent,
                          List_dof_ent_type, List_dof_ent_id, List_dof_ent_nrdofs, Nrdofs_glob,
                          Max_dofs_per_dof_ent);
}
int pdr_exchange_dofs(int a, int b, int c, double *d) { (void)a; (void)b; (void)c; (void)d; return 1; }
double pdr_vec_norm(int Problem_id, int Solver_id, int Level_id, int Nrdof, double *Vector)
{
  int one = 1; (void)Problem_id; (void)Solver_id; (void)Level_id;
  return dnrm2_(&Nrdof, Vector, &one);
}
double pdr_sc_prod(int Problem_id, int Solver_id, int Level_id, int Nrdof, double *V1, double *V2)
{
  int one = 1; (void)Problem_id; (void)Solver_id; (void)Level_id;
  return ddot_(&Nrdof, V1, &one, V2, &one);
}
int pdr_get_ent_pdeg(int Problem_id, int Ent_type, int Ent_id)
{
  (void)Problem_id;
  return apr_get_ent_pdeg(h_field_id, Ent_type, Ent_id);
}
int pdr_read_sol_dofs(int Problem_id, int Dof_ent_type, int Dof_ent_id, int Nrdofs, double *Vect_dofs)
{
  int i; (void)Problem_id; (void)Dof_ent_type;
  for (i = 0; i < Nrdofs; i++)
    Vect_dofs[i] = (h_sol && Dof_ent_id < h_sol_cap) ? h_sol[(size_t)Dof_ent_id * h_sol_stride + i] : 0.0;
  return 1;
}
int pdr_write_sol_dofs(int Problem_id, int Dof_ent_type, int Dof_ent_id, int Nrdofs, double *Vect_dofs)
{
  int i; (void)Problem_id; (void)Dof_ent_type;
  if (h_sol && Dof_ent_id < h_sol_cap)
    for (i = 0; i < Nrdofs && i < h_sol_stride; i++) h_sol[(size_t)Dof_ent_id * h_sol_stride + i] = Vect_dofs[i];
  return 1;
}

/* ------------------------------------------------------------------ */
/* harness API (called from Python through ctypes)                     */
/* ------------------------------------------------------------------ */
int refh_load_jk(const char *path)
{
  if (utv_log_out == NULL) utv_log_out = stderr;
  h_mesh_id = mmr_init_mesh(MMC_GRADMESH_DATA, (char *)path, stdout);
  return h_mesh_id;
}

int refh_mesh_sizes(int *nno, int *max_node_id, int *nel, int *max_el_id, int *nfa, int *max_fa_id)
{
  *nno = mmr_get_nr_node(h_mesh_id);
  *max_node_id = mmr_get_max_node_id(h_mesh_id);
  *nel = mmr_get_nr_elem(h_mesh_id);
  *max_el_id = mmr_get_max_elem_id(h_mesh_id);
  *nfa = mmr_get_nr_face(h_mesh_id);
  *max_fa_id = mmr_get_max_face_id(h_mesh_id);
  return 0;
}

/* node coordinates for ids 1..max_node_id, written at xyz[3*(id-1)] */
int refh_node_coords(double *xyz)
{
  int n = mmr_get_max_node_id(h_mesh_id), i;
  for (i = 1; i <= n; i++) mmr_node_coor(h_mesh_id, i, &xyz[3 * (i - 1)]);
  return n;
}

/* moves every node to the given coordinates (mmr_move_node takes a displacement) */
int refh_set_node_coords(const double *xyz)
{
  int n = mmr_get_max_node_id(h_mesh_id), i;
  for (i = 1; i <= n; i++) {
    double c[3], d[3];
    mmr_node_coor(h_mesh_id, i, c);
    d[0] = xyz[3 * (i - 1)] - c[0];
    d[1] = xyz[3 * (i - 1) + 1] - c[1];
    d[2] = xyz[3 * (i - 1) + 2] - c[2];
    mmr_move_node(h_mesh_id, i, d);
  }
  return n;
}

/* element vertex ids in mmr_el_node_coor order: nodes[nv*(el-1)+j] */
int refh_el_nodes(int nv, int *nodes)
{
  int nmax = mmr_get_max_elem_id(h_mesh_id), el, j;
  for (el = 1; el <= nmax; el++) {
    int l[MMC_MAXELVNO + 1];
    mmr_el_node_coor(h_mesh_id, el, l, NULL);
    for (j = 0; j < nv; j++) nodes[nv * (el - 1) + j] = (j < l[0]) ? l[j + 1] : 0;
  }
  return nmax;
}

/* boundary faces with bc>0 in mmr order: face id, bc flag, neighbour element */
int refh_bc_faces(int *fa_id, int *fa_bc, int *fa_el)
{
  int nfa = 0, cnt = 0;
  while ((nfa = mmr_get_next_face_all(h_mesh_id, nfa)) != 0) {
    if (mmr_fa_status(h_mesh_id, nfa) == MMC_ACTIVE && mmr_fa_bc(h_mesh_id, nfa) > 0) {
      int neig[2];
      mmr_fa_eq_neig(h_mesh_id, nfa, neig, NULL, NULL);
      if (fa_id) { fa_id[cnt] = nfa; fa_bc[cnt] = mmr_fa_bc(h_mesh_id, nfa); fa_el[cnt] = abs(neig[0]); }
      cnt++;
    }
  }
  return cnt;
}

int refh_init_field(int field_type, int pdeg)
{
  h_field_id = apr_init_field((char)field_type, APC_ZERO, h_mesh_id, 1, 1, pdeg, NULL, NULL);
  return h_field_id;
}

int refh_set_coeffs(int nel, const double *k, const double *D, double f, double g, int aniso)
{
  free(h_k); free(h_D);
  h_k = NULL; h_D = NULL;
  h_nel_coef = nel;
  if (k) { h_k = (double *)malloc((nel + 1) * sizeof(double)); h_k[0] = 1.0; memcpy(h_k + 1, k, nel * sizeof(double)); }
  if (D) { h_D = (double *)calloc(9 * (size_t)(nel + 1), sizeof(double)); memcpy(h_D + 9, D, 9 * (size_t)nel * sizeof(double)); }
  h_f = f; h_g = g; h_aniso = aniso;
  return 0;
}

void refh_set_dg_penalty(double p) { h_dg_penalty = p; }

/* element (type=APC_ELEMENT) or face (APC_FACE) stiffness matrix and load
   vector, column-major, with the dof entity list */
int refh_int_ent_stiff(int type, int id, double *sm, double *rhs, int *nrdofs, int *nr_dof_ent,
                       int *dof_type, int *dof_id, int *dof_nrdofs)
{
  int n = APC_MAXELSD, ne = PDC_MAX_DOF_PER_INT;
  char rewr;
  pdr_comp_stiff_mat(1, type, id, PDC_COMP_BOTH, NULL, &ne, dof_type, dof_id, dof_nrdofs, &n, sm, rhs, &rewr);
  *nrdofs = n; *nr_dof_ent = ne;
  return n;
}

int refh_solver_create(const char *mkb_dat)
{
  h_solver_id = sir_init(1, SIC_SEQUENTIAL, 1, (char *)mkb_dat, -1, -1, -1.0, -1);
  sir_create(h_solver_id, 1);
  return h_solver_id;
}

int refh_level_sizes(int *nrdofs, int *nr_int_ent, int *nr_dof_ent, int *nr_colors_elems, int *nr_colors_faces,
                     int *len_asse_pos, int *max_dofs_int_ent, int *nnz)
{
  sit_levels *lv = &siv_solver[h_solver_id].level[0];
  int i, tot = 0;
  *nrdofs = lv->nrdofs_glob;
  *nr_int_ent = lv->nr_int_ent;
  *nr_dof_ent = lv->nr_dof_ent;
  *nr_colors_elems = lv->nr_colors_elems;
  *nr_colors_faces = lv->nr_colors_faces;
  *len_asse_pos = lv->nr_asse_blocks_all_int_ent;
  *max_dofs_int_ent = lv->max_dofs_int_ent;
  /* length of the assembly table: sum over int ents of (n*n + n) */
  for (i = 0; i < lv->nr_int_ent; i++) {
    int ne = PDC_MAX_DOF_PER_INT, n = APC_MAXELSD;
    int t[PDC_MAX_DOF_PER_INT], id[PDC_MAX_DOF_PER_INT], nd[PDC_MAX_DOF_PER_INT];
    pdr_comp_stiff_mat(1, lv->l_int_ent_type[i], lv->l_int_ent_id[i], PDC_NO_COMP, NULL, &ne, t, id, nd, NULL, NULL, NULL, NULL);
    int j, s = 0;
    for (j = 0; j < ne; j++) s += nd[j];
    tot += s * s + s;
  }
  *nnz = itv_crs_matrices[0].Nnz;
  return tot;
}

int refh_level_lists(int *int_ent_type, int *int_ent_id, int *color_elems, int *color_faces,
                     int *asse_pos, int *assembly_table, int table_len,
                     int *dof_ent_type, int *dof_ent_id, int *dof_posglob, int *dof_block_id)
{
  sit_levels *lv = &siv_solver[h_solver_id].level[0];
  int i;
  for (i = 0; i < lv->nr_int_ent; i++) { int_ent_type[i] = lv->l_int_ent_type[i]; int_ent_id[i] = lv->l_int_ent_id[i]; }
  for (i = 0; i <= lv->nr_colors_elems; i++) color_elems[i] = lv->l_color_index_elems ? lv->l_color_index_elems[i] : 0;
  for (i = 0; i <= lv->nr_colors_faces; i++) color_faces[i] = lv->l_color_index_faces ? lv->l_color_index_faces[i] : 0;
  for (i = 0; i < lv->nr_int_ent; i++) asse_pos[i] = lv->asse_pos_first_dof_int_ent ? lv->asse_pos_first_dof_int_ent[i] : 0;
  if (lv->assembly_table) for (i = 0; i < table_len; i++) assembly_table[i] = lv->assembly_table[i];
  for (i = 0; i < lv->nr_dof_ent; i++) {
    dof_ent_type[i] = lv->l_dof_struct[i].dof_ent_type;
    dof_ent_id[i] = lv->l_dof_struct[i].dof_ent_id;
    dof_posglob[i] = lv->l_dof_struct[i].posglob;
    dof_block_id[i] = lv->l_dof_struct[i].block_id;
  }
  return lv->nr_int_ent;
}

int refh_crs_get(int *row_ptr, int *col_ind, double *val, double *rhs)
{
  itt_crs_matrices *m = &itv_crs_matrices[0];
  int i;
  if (row_ptr) for (i = 0; i <= m->Nrdofgl; i++) row_ptr[i] = m->crs_row_ptr[i];
  if (col_ind) for (i = 0; i < m->Nnz; i++) col_ind[i] = m->crs_col_ind[i];
  if (val) for (i = 0; i < m->Nnz; i++) val[i] = m->crs_val[i];
  if (rhs) for (i = 0; i < m->Nrdofgl; i++) rhs[i] = m->rhs[i];
  return m->Nnz;
}

/* clears the matrix and runs the reference assembly driver exactly as
   sir_solve does for the table-driven path (sis_mkb_intf.c:2043-2076) */
double refh_assemble(void)
{
  sit_levels *lv = &siv_solver[h_solver_id].level[0];
  int pdeg_coarse = -10;
  lsr_mkb_clear_matrix(h_solver_id, 0, SIC_SOLVE);
  pdr_create_assemble_stiff_mat(1, 0, PDC_COMP_BOTH, &pdeg_coarse, lv->nr_int_ent, lv->l_int_ent_type,
                                lv->l_int_ent_id, lv->nr_colors_elems, lv->l_color_index_elems,
                                lv->nr_colors_faces, lv->l_color_index_faces,
                                lv->asse_pos_first_dof_int_ent, lv->assembly_table, lv->max_dofs_int_ent);
  return h_last_assembly_s;
}

/* reference residual V = B - A X through the lar_ boundary (las_intf.c:771) */
void refh_residual(int use_rhs, int ini_zero, int ndof, double *x, double *b, double *v)
{
  lar_compute_residual(0, use_rhs, ini_zero, ndof, x, b, v);
}

/* full sir_solve: assemble, precondition, GMRES; solution per dof entity id.
   sol must hold stride*(max dof entity id + 1) doubles. */
int refh_solve(int max_iter, double tol, int monitor, double *sol, int sol_cap, int stride,
               double *conv_meas_out, double *times)
{
  int nit = max_iter;
  double meas = tol, rate = 0.0, t0;
  h_sol = sol; h_sol_cap = sol_cap; h_sol_stride = stride;
  t0 = wall();
  sir_solve(h_solver_id, SIC_SOLVE, 0, monitor, &nit, &meas, &rate);
  if (times) { times[0] = wall() - t0; times[1] = h_last_assembly_s; }
  h_sol = NULL;
  *conv_meas_out = meas;
  return nit;
}

int refh_solver_free(void)
{
  sir_free(h_solver_id);
  sir_destroy(h_solver_id);
  h_solver_id = -1;
  return 0;
}

#ifdef HARNESS_STD
/* One adaptation step as utr_adapt runs it for refinement only
   (utd_util/uts_adapt.c:1458-1539): mmr_init_ref, apr_refine of each listed
   active element (which also refines neighbours to keep the mesh 1-irregular,
   aps_std_lin_intf.c:4007-4190), apr_proj_dof_ref (which creates the
   constraint data of the hanging vertices, aps_std_lin_intf.c:3440-3615) and
   mmr_final_ref.  The mesh's adaptation limits are set first: max_gen
   generations, generation difference 1 (1-irregular meshes).  Returns the
   number of active elements. */
int refh_refine(int n, const int *el_ids, int max_gen)
{
  int nmno = mmr_get_max_node_id(h_mesh_id), nmed = mmr_get_max_edge_id(h_mesh_id);
  int nmfa = mmr_get_max_face_id(h_mesh_id), nmel = mmr_get_max_elem_id(h_mesh_id), i;
  if (n <= 0) return mmr_get_nr_elem(h_mesh_id);
  mmr_set_max_gen(h_mesh_id, max_gen);
  mmr_set_max_gen_diff(h_mesh_id, 1);
  mmr_init_ref(h_mesh_id);
  for (i = 0; i < n; i++)
    if (mmr_el_status(h_mesh_id, el_ids[i]) == MMC_ACTIVE) apr_refine(h_field_id, el_ids[i]);
  apr_proj_dof_ref(h_field_id, n > 1 ? -3 : el_ids[0], nmel, nmfa, nmed, nmno);
  mmr_final_ref(h_mesh_id);
  return mmr_get_nr_elem(h_mesh_id);
}

/* status of elements 1..max_el_id (1 active, -1 refined, 0 free) */
int refh_el_status(int *st)
{
  int nmax = mmr_get_max_elem_id(h_mesh_id), el;
  for (el = 1; el <= nmax; el++) st[el - 1] = mmr_el_status(h_mesh_id, el);
  return nmax;
}

/* per node 1..max_node_id: cnt[id-1] = 0 for a node with dofs (or free
   space), else the number of constraining vertices (2 mid-edge, 4 mid-face)
   with their ids in par[4*(id-1) ...] (apr_get_constr_data) */
int refh_constr(int *cnt, int *par)
{
  int nmax = mmr_get_max_node_id(h_mesh_id), v, j, ncon = 0;
  for (v = 1; v <= nmax; v++) {
    int c[5] = {0, 0, 0, 0, 0};
    cnt[v - 1] = 0;
    for (j = 0; j < 4; j++) par[4 * (v - 1) + j] = 0;
    if (mmr_node_status(h_mesh_id, v) != MMC_ACTIVE) continue;
    if (apr_get_ent_pdeg(h_field_id, APC_VERTEX, v) != 0) continue;
    apr_get_constr_data(h_field_id, v, APC_VERTEX, c, NULL);
    cnt[v - 1] = c[0];
    for (j = 0; j < c[0] && j < 4; j++) par[4 * (v - 1) + j] = c[j + 1];
    ncon++;
  }
  return ncon;
}

/* side (0..4, position in mmr_el_faces) of each boundary face of
   refh_bc_faces in its element */
int refh_bc_face_sides(int n, const int *fa_id, const int *fa_el, int *side)
{
  int i, j;
  for (i = 0; i < n; i++) {
    int faces[MMC_MAXELFAC + 1];
    mmr_el_faces(h_mesh_id, fa_el[i], faces, NULL);
    side[i] = -1;
    for (j = 1; j <= faces[0]; j++)
      if (faces[j] == fa_id[i]) side[i] = j - 1;
  }
  return n;
}
#endif

#ifdef HARNESS_STD
/* Std linear tetrahedron through the reference's own element calculations:
   apr_set_quadr_3D (aps_std_util.c:1335) and apr_elem_calc_3D with the
   tetra base (aps_std_util.c:869), accumulated with the 9-term diffusion and
   source loops of apr_num_int_el (aps_std_lin_intf.c:2113-2134, 2785-2791).
   The tet mesh module (mmd_t4_prism) needs Boost and is not linked, so the
   element loop is driven here with given vertex coordinates. */
extern int apr_set_quadr_3D(int Base_type, int *Pdeg_vec, int *Ngauss, double *Xg, double *Wg);
extern double apr_elem_calc_3D(int Control, int Nreq, int *Pdeg_vec, int Base_type, double *Eta,
                               double *Node_coor, double *Sol_dofs, double *Base_phi, double *Base_dphix,
                               double *Base_dphiy, double *Base_dphiz, double *Xcoor, double *Sol,
                               double *Dsolx, double *Dsoly, double *Dsolz, double *Vec_nor);
void apr_gauss_init(void);

int refh_tet_element(const double *Xin, const double *A, double f, double *sm, double *rhs)
{
  static int init = 0;
  int pdeg = 1, ng, q, u, w;
  double xg[3000], wg[1000], X[12];
  if (!init) { apr_gauss_init(); init = 1; }
  memcpy(X, Xin, 12 * sizeof(double));
  apr_set_quadr_3D(APC_BASE_TETRA_STD, &pdeg, &ng, xg, wg);
  for (u = 0; u < 16; u++) sm[u] = 0.0;
  for (u = 0; u < 4; u++) rhs[u] = 0.0;
  for (q = 0; q < ng; q++) {
    double phi[APC_MAXELVD], gx[APC_MAXELVD], gy[APC_MAXELVD], gz[APC_MAXELVD], xc[3];
    double det = apr_elem_calc_3D(2, 1, &pdeg, APC_BASE_TETRA_STD, &xg[3 * q], X, NULL, phi, gx, gy, gz, xc,
                                  NULL, NULL, NULL, NULL, NULL);
    double vol = det * wg[q];
    for (u = 0; u < 4; u++)
      for (w = 0; w < 4; w++)
        sm[u * 4 + w] += (A[0] * gx[u] * gx[w] + A[1] * gy[u] * gx[w] + A[2] * gz[u] * gx[w] +
                          A[3] * gx[u] * gy[w] + A[4] * gy[u] * gy[w] + A[5] * gz[u] * gy[w] +
                          A[6] * gx[u] * gz[w] + A[7] * gy[u] * gz[w] + A[8] * gz[u] * gz[w]) * vol;
    for (w = 0; w < 4; w++) rhs[w] += f * phi[w] * vol;
  }
  return ng;
}
#endif

#ifdef HARNESS_DG
/* DG prism approximation (apd_dg_prism) helpers: basis values, quadrature
   rules and per-element degrees straight from the reference module. */
extern int apr_shape_fun_3D(int Base_type, int Pdeg, double *Eta, double *Base_phi, double *Base_dphix,
                            double *Base_dphiy, double *Base_dphiz);
extern int apr_set_quadr_3D(int Base_type, int *Pdeg_vec, int *Ngauss, double *Xg, double *Wg);
extern int apr_set_quadr_2D(int Fa_type, int Base_type, int *Pdeg_vec, int *Ngauss, double *Xg, double *Wg);
void apr_gauss_init(void);

int refh_dg_basis(int pdeg, const double *eta, double *phi, double *dx, double *dy, double *dz)
{
  double e[3] = {eta[0], eta[1], eta[2]};
  return apr_shape_fun_3D(APC_BASE_TENSOR_DG, pdeg, e, phi, dx, dy, dz);
}

int refh_dg_quadrature(int pdeg, double *xg, double *wg)
{
  static int init = 0;
  int ng = 0, p = pdeg;
  if (!init) { apr_gauss_init(); init = 1; }
  apr_set_quadr_3D(APC_BASE_TENSOR_DG, &p, &ng, xg, wg);
  return ng;
}

int refh_dg_face_quadrature(int fa_type, int pdeg, double *xg, double *wg)
{
  static int init = 0;
  int ng = 0, p = pdeg;
  if (!init) { apr_gauss_init(); init = 1; }
  apr_set_quadr_2D(fa_type, APC_BASE_TENSOR_DG, &p, &ng, xg, wg);
  return ng;
}

int refh_set_el_pdeg(int el, int pdeg)
{
  return apr_set_ent_pdeg(h_field_id, APC_ELEMENT, el, pdeg);
}
#endif

/* Every active face in mmr order: out[10*i ..] = id, type, bc, neig1, neig2
   (signed, 0 = boundary), side1, side2, then up to 4 vertex ids in
   mmr_fa_node_coor order (padded with 0); returns the count. */
int refh_all_faces(int *out)
{
  int nfa = 0, cnt = 0;
  while ((nfa = mmr_get_next_face_all(h_mesh_id, nfa)) != 0) {
    if (mmr_fa_status(h_mesh_id, nfa) != MMC_ACTIVE) continue;
    if (out) {
      int neig[2] = {0, 0}, sides[2] = {0, 0}, shift = 0, gen = 0, nodes[MMC_MAXFAVNO + 1], j;
      double ac[4], bc[2];
      mmr_fa_neig(h_mesh_id, nfa, neig, sides, &shift, &gen, ac, bc);
      mmr_fa_node_coor(h_mesh_id, nfa, nodes, NULL);
      int *o = out + 10 * cnt;
      o[0] = nfa; o[1] = mmr_fa_type(h_mesh_id, nfa); o[2] = mmr_fa_bc(h_mesh_id, nfa);
      o[3] = neig[0]; o[4] = neig[1]; o[5] = sides[0]; o[6] = sides[1];
      for (j = 0; j < 4; j++) o[6 + j] = 0;
      for (j = 0; j < nodes[0] && j < 3; j++) o[7 + j] = nodes[j + 1];
      /* the fourth vertex of a quad does not fit: store it in slot 6 after sides */
      if (nodes[0] == 4) { o[6] = sides[1] * 1000 + nodes[4]; }
    }
    cnt++;
  }
  return cnt;
}

/* Field dump through the reference's own writer (apr_write_field): the
 * values are first stored in the field with apr_write_ent_dofs, per vertex
 * (std: vals[n] for vertex n+1, NaN = vertex without dofs) or per element
 * (DG: vals + off[e] .. off[e+1]). */
int refh_write_field(const char *path, int ent_type, int nent, const double *vals, const int *off)
{
  int i;
  for (i = 0; i < nent; i++) {
    if (ent_type == APC_VERTEX) {
      double v = vals[i];
      if (v != v) continue;
      apr_write_ent_dofs(h_field_id, APC_VERTEX, i + 1, 1, 1, &v);
    } else {
      apr_write_ent_dofs(h_field_id, APC_ELEMENT, i + 1, off[i + 1] - off[i], 1, (double *)vals + off[i]);
    }
  }
  return apr_write_field(h_field_id, 1, 1, 0.0, (char *)path);
}
