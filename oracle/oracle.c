/*
 * oracle.c - CPU restatement of ModFEM's std-linear integrate / assemble /
 * GMRES path.  TEST INFRASTRUCTURE ONLY (see oracle.h): the checker for the
 * CUDA path and the timed CPU baseline; never linked into the product.
 *
 * Each routine states which reference routine it follows.  Reference paths
 * are relative to the ModFEM source tree (modfem2017/src).
 */
#include "oracle.h"
#include "../modfem_gb300/csrc/dg_tables.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static double now_s(void)
{
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

/* Gauss-Legendre 2-point line rule and the 3-point triangle rule with the
   15-digit values the reference tabulates (apd_std_lin/aps_gauss_util_std.c:
   apr_gauss_init, Xg_1d[1], Xg_2d[1], Wg_2d[1]). */
static const double G2 = 0.577350269189626;
static const double T3_XI[3] = {0.166666666666667, 0.166666666666667, 0.666666666666667};
static const double T3_ETA[3] = {0.166666666666667, 0.666666666666667, 0.166666666666667};
static const double T3_W = 0.333333333333333;

/* 3x3 inverse and determinant in the reference's formula order
   (apd_std_lin/aps_std_util.c:2770-2824, ut_mat3_inv). */
static double mat3_inv(const double *m, double *mi)
{
  double rjac = m[0] * (m[4] * m[8] - m[7] * m[5]) + m[3] * (m[7] * m[2] - m[1] * m[8]) +
                m[6] * (m[1] * m[5] - m[4] * m[2]);
  double r = 1.0 / rjac;
  mi[0] = (m[4] * m[8] - m[7] * m[5]) * r;
  mi[3] = (-m[3] * m[8] + m[6] * m[5]) * r;
  mi[6] = (m[3] * m[7] - m[6] * m[4]) * r;
  mi[1] = (m[7] * m[2] - m[1] * m[8]) * r;
  mi[4] = (m[0] * m[8] - m[6] * m[2]) * r;
  mi[7] = (-m[0] * m[7] + m[6] * m[1]) * r;
  mi[2] = (m[1] * m[5] - m[4] * m[2]) * r;
  mi[5] = (-m[0] * m[5] + m[3] * m[2]) * r;
  mi[8] = (m[0] * m[4] - m[3] * m[1]) * r;
  return rjac;
}

/* Linear prism shape functions on the reference prism (triangle x [-1,1])
   and their local derivatives (aps_std_util.c:463-510). */
static void prism_shape(const double *e, double *phi, double *dx, double *dy, double *dz)
{
  double lo = (1.0 - e[2]) / 2.0, hi = (1.0 + e[2]) / 2.0, l0 = 1.0 - e[0] - e[1];
  phi[0] = lo * l0; phi[1] = lo * e[0]; phi[2] = lo * e[1];
  phi[3] = hi * l0; phi[4] = hi * e[0]; phi[5] = hi * e[1];
  dx[0] = -lo; dx[1] = lo; dx[2] = 0.0; dx[3] = -hi; dx[4] = hi; dx[5] = 0.0;
  dy[0] = -lo; dy[1] = 0.0; dy[2] = lo; dy[3] = -hi; dy[4] = 0.0; dy[5] = hi;
  dz[0] = -0.5 * l0; dz[1] = -0.5 * e[0]; dz[2] = -0.5 * e[1];
  dz[3] = 0.5 * l0; dz[4] = 0.5 * e[0]; dz[5] = 0.5 * e[1];
}

/* Jacobian matrix dx/deta (row-major: dxdeta[3*i+j] = d x_i / d eta_j) of the
   geometrically linear prism (aps_std_util.c:650-672). */
static void prism_jacobian(const double *X, const double *dx, const double *dy, const double *dz,
                           double *J)
{
  int i;
  for (i = 0; i < 9; i++) J[i] = 0.0;
  for (i = 0; i < 6; i++) {
    J[0] += X[3 * i] * dx[i]; J[1] += X[3 * i] * dy[i]; J[2] += X[3 * i] * dz[i];
    J[3] += X[3 * i + 1] * dx[i]; J[4] += X[3 * i + 1] * dy[i]; J[5] += X[3 * i + 1] * dz[i];
    J[6] += X[3 * i + 2] * dx[i]; J[7] += X[3 * i + 2] * dy[i]; J[8] += X[3 * i + 2] * dz[i];
  }
}

/* Shared quadrature-point body of apr_num_int_el for nreq=1 with the 9-term
   diffusion branch and the source term (apd_std_lin/aps_std_lin_intf.c:
   2113-2134 and 2785-2791). */
static void accumulate_qp(int ns, const double *phi, const double *gx, const double *gy,
                          const double *gz, const double *A, double f, double vol, double *sm,
                          double *rhs)
{
  int u, w;
  for (u = 0; u < ns; u++)
    for (w = 0; w < ns; w++)
      sm[u * ns + w] += (A[0] * gx[u] * gx[w] + A[1] * gy[u] * gx[w] + A[2] * gz[u] * gx[w] +
                         A[3] * gx[u] * gy[w] + A[4] * gy[u] * gy[w] + A[5] * gz[u] * gy[w] +
                         A[6] * gx[u] * gz[w] + A[7] * gy[u] * gz[w] + A[8] * gz[u] * gz[w]) * vol;
  for (w = 0; w < ns; w++) rhs[w] += f * phi[w] * vol;
}

/* apr_num_int_el for the std linear prism (aps_std_lin_intf.c:1537-2880):
   quadrature of apr_set_quadr_3D (aps_std_util.c:1335-1440) - outer loop over
   the two Gauss line points, inner over the three triangle points, weight
   0.5*w_tri*w_line - element calculations of apr_elem_calc_3D_prism
   (aps_std_util.c:520-820). */
void orc_std_prism_element(const double *X, const double *A, double f, double *sm, double *rhs)
{
  int iz, it, i;
  memset(sm, 0, 36 * sizeof(double));
  memset(rhs, 0, 6 * sizeof(double));
  for (iz = 0; iz < 2; iz++) {
    for (it = 0; it < 3; it++) {
      double e[3] = {T3_XI[it], T3_ETA[it], iz == 0 ? -G2 : G2};
      double w = 0.5 * T3_W * 1.0;
      double phi[6], dx[6], dy[6], dz[6], J[9], Ji[9], gx[6], gy[6], gz[6];
      prism_shape(e, phi, dx, dy, dz);
      prism_jacobian(X, dx, dy, dz, J);
      double det = fabs(mat3_inv(J, Ji));
      for (i = 0; i < 6; i++) {
        gx[i] = dx[i] * Ji[0] + dy[i] * Ji[3] + dz[i] * Ji[6];
        gy[i] = dx[i] * Ji[1] + dy[i] * Ji[4] + dz[i] * Ji[7];
        gz[i] = dx[i] * Ji[2] + dy[i] * Ji[5] + dz[i] * Ji[8];
      }
      accumulate_qp(6, phi, gx, gy, gz, A, f, det * w, sm, rhs);
    }
  }
}

/* Boundary penalty integral of the std conv-diff weak form
   (pdd_conv_diff/weak_formulation/approx_std/pds_conv_diff_weakform_std.c:
   253-630): K += penalty*phi_j*phi_i*|dS|*w, R += penalty*g*phi_i*|dS|*w over
   the face rule of apr_set_quadr_2D (aps_std_util.c:1445-1500): 3-point
   triangle rule with weights 0.5*w for sides 0/1, 2x2 Gauss with weights
   0.5*w1*w2 on [-1,1]^2 mapped to edge parameter (s+1)/2 for lateral sides.
   |dS| follows the side cases of apr_elem_calc_3D_prism (aps_std_util.c:
   770-805). */
void orc_std_prism_face(const double *X, int side, double penalty, double g, double *sm, double *rhs)
{
  int q, i, j, nq;
  double pts[4][3], wq[4];
  memset(sm, 0, 36 * sizeof(double));
  memset(rhs, 0, 6 * sizeof(double));
  if (side <= 1) {
    nq = 3;
    for (q = 0; q < 3; q++) {
      pts[q][0] = T3_XI[q]; pts[q][1] = T3_ETA[q]; pts[q][2] = side == 0 ? -1.0 : 1.0;
      wq[q] = 0.5 * T3_W;
    }
  } else {
    nq = 4;
    for (q = 0; q < 4; q++) {
      double s = (q / 2 == 0) ? -G2 : G2, t = (q % 2 == 0) ? -G2 : G2;
      double u = (s + 1.0) / 2.0;
      if (side == 2) { pts[q][0] = u; pts[q][1] = 0.0; }
      else if (side == 3) { pts[q][0] = 1.0 - u; pts[q][1] = u; }
      else { pts[q][0] = 0.0; pts[q][1] = 1.0 - u; }
      pts[q][2] = t;
      wq[q] = 0.5 * 1.0 * 1.0;
    }
  }
  for (q = 0; q < nq; q++) {
    double phi[6], dx[6], dy[6], dz[6], J[9], ds[3];
    prism_shape(pts[q], phi, dx, dy, dz);
    prism_jacobian(X, dx, dy, dz, J);
    if (side == 0) {
      ds[0] = -J[3] * J[7] + J[6] * J[4]; ds[1] = -J[6] * J[1] + J[0] * J[7]; ds[2] = -J[0] * J[4] + J[3] * J[1];
    } else if (side == 1) {
      ds[0] = J[3] * J[7] - J[6] * J[4]; ds[1] = J[6] * J[1] - J[0] * J[7]; ds[2] = J[0] * J[4] - J[3] * J[1];
    } else if (side == 2) {
      ds[0] = J[3] * J[8] - J[6] * J[5]; ds[1] = J[6] * J[2] - J[0] * J[8]; ds[2] = J[0] * J[5] - J[3] * J[2];
    } else if (side == 3) {
      ds[0] = (J[4] - J[3]) * J[8] - (J[7] - J[6]) * J[5];
      ds[1] = (J[7] - J[6]) * J[2] - (J[1] - J[0]) * J[8];
      ds[2] = (J[1] - J[0]) * J[5] - (J[4] - J[3]) * J[2];
    } else {
      ds[0] = J[5] * J[7] - J[8] * J[4]; ds[1] = J[8] * J[1] - J[2] * J[7]; ds[2] = J[2] * J[4] - J[5] * J[1];
    }
    double area = sqrt(ds[0] * ds[0] + ds[1] * ds[1] + ds[2] * ds[2]) * wq[q];
    for (j = 0; j < 6; j++)
      for (i = 0; i < 6; i++) sm[j * 6 + i] += penalty * phi[j] * phi[i] * area;
    for (i = 0; i < 6; i++) rhs[i] += penalty * g * phi[i] * area;
  }
}

/* Linear tetrahedron (apr_elem_calc_3D_tetra, aps_std_util.c:869-1130):
   constant Jacobian from edge vectors, |det|/6 volume factor; 4-point rule
   of order 2 with weights 1/4 in the point order apr_set_quadr_3D produces
   (aps_std_util.c:1360-1375 reading Xg_3d[1] with a stride of 3). */
void orc_std_tet_element(const double *X, const double *A, double f, double *sm, double *rhs)
{
  static const double a = 0.585410196624969, b = 0.138196601125011;
  const double P[4][3] = {{a, b, b}, {b, b, a}, {b, b, b}, {b, a, b}};
  double J[9], Ji[9], gx[4], gy[4], gz[4], phi[4];
  const double dx[4] = {-1.0, 1.0, 0.0, 0.0}, dy[4] = {-1.0, 0.0, 1.0, 0.0}, dz[4] = {-1.0, 0.0, 0.0, 1.0};
  int q, i;
  memset(sm, 0, 16 * sizeof(double));
  memset(rhs, 0, 4 * sizeof(double));
  J[0] = X[3] - X[0]; J[3] = X[4] - X[1]; J[6] = X[5] - X[2];
  J[1] = X[6] - X[0]; J[4] = X[7] - X[1]; J[7] = X[8] - X[2];
  J[2] = X[9] - X[0]; J[5] = X[10] - X[1]; J[8] = X[11] - X[2];
  double det = fabs(mat3_inv(J, Ji) * 0.16666666666666666666666666666667);
  for (i = 0; i < 4; i++) {
    gx[i] = dx[i] * Ji[0] + dy[i] * Ji[3] + dz[i] * Ji[6];
    gy[i] = dx[i] * Ji[1] + dy[i] * Ji[4] + dz[i] * Ji[7];
    gz[i] = dx[i] * Ji[2] + dy[i] * Ji[5] + dz[i] * Ji[8];
  }
  for (q = 0; q < 4; q++) {
    phi[0] = 1.0 - P[q][0] - P[q][1] - P[q][2]; phi[1] = P[q][0]; phi[2] = P[q][1]; phi[3] = P[q][2];
    accumulate_qp(4, phi, gx, gy, gz, A, f, det * 0.25, sm, rhs);
  }
}

/* DOF entities in order of first appearance over the integration entities'
   element DOF lists (utd_util/uts_ls_intf.c:259-300, utr_get_list_dof_ent);
   the solver keeps that order as block ids (sid_mkb/sis_mkb_intf.c:1019). */
int orc_std_dof_order(int nel, int nv, const int *el_nodes, int nno, int *dof_of_node)
{
  int e, j, nd = 0;
  for (j = 0; j < nno; j++) dof_of_node[j] = -1;
  for (e = 0; e < nel; e++)
    for (j = 0; j < nv; j++) {
      int nd_id = el_nodes[(size_t)e * nv + j];
      if (dof_of_node[nd_id] < 0) dof_of_node[nd_id] = nd++;
    }
  return nd;
}

static int cmp_int(const void *a, const void *b)
{
  int x = *(const int *)a, y = *(const int *)b;
  return (x > y) - (x < y);
}

/* CRS structure: row r holds every DOF that shares an element with r,
   diagonal included, in ascending column order (neighbour lists sorted in
   sir_create, sid_mkb/sis_mkb_intf.c:1128; diagonal inserted in order,
   lsd_mkb/lad_crs/las_crs_intf.c:196-245). */
long orc_std_crs_structure(int nel, int nv, const int *el_nodes, const int *dof_of_node, int ndof,
                           int *row_ptr, int *col_ind)
{
  /* node -> element incidence */
  int *cnt = (int *)calloc(ndof + 1, sizeof(int));
  int e, j, r;
  for (e = 0; e < nel; e++)
    for (j = 0; j < nv; j++) cnt[dof_of_node[el_nodes[(size_t)e * nv + j]] + 1]++;
  for (r = 0; r < ndof; r++) cnt[r + 1] += cnt[r];
  int *inc = (int *)malloc((size_t)cnt[ndof] * sizeof(int));
  int *fill = (int *)calloc((size_t)ndof + 1, sizeof(int));
  for (e = 0; e < nel; e++)
    for (j = 0; j < nv; j++) {
      int d = dof_of_node[el_nodes[(size_t)e * nv + j]];
      inc[cnt[d] + fill[d]++] = e;
    }
  int *mark = (int *)malloc(ndof * sizeof(int));
  for (r = 0; r < ndof; r++) mark[r] = -1;
  int *tmp = (int *)malloc(64 * nv * sizeof(int) + 64);
  int tcap = 64 * nv + 16;
  long nnz = 0;
  row_ptr[0] = 0;
  for (r = 0; r < ndof; r++) {
    int nt = 0, k;
    for (k = cnt[r]; k < cnt[r + 1]; k++) {
      int el = inc[k];
      for (j = 0; j < nv; j++) {
        int c = dof_of_node[el_nodes[(size_t)el * nv + j]];
        if (mark[c] != r) {
          mark[c] = r;
          if (nt >= tcap) { tcap *= 2; tmp = (int *)realloc(tmp, tcap * sizeof(int)); }
          tmp[nt++] = c;
        }
      }
    }
    qsort(tmp, nt, sizeof(int), cmp_int);
    if (col_ind) memcpy(col_ind + nnz, tmp, nt * sizeof(int));
    nnz += nt;
    row_ptr[r + 1] = (int)nnz;
  }
  free(cnt); free(inc); free(fill); free(mark); free(tmp);
  return nnz;
}

static int find_col(const int *col_ind, int lo, int hi, int c)
{
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (col_ind[mid] < c) lo = mid + 1; else hi = mid;
  }
  return lo;
}

/* Assembly table of one integration entity (lar_fill_assembly_table_int_ent_crs,
   lsd_mkb/lad_crs/las_crs_intf.c:354-438): entry j + i*n is the CRS position
   of (row dofs[j], column dofs[i]); entry n*n + j is the rhs position. */
void orc_crs_table(int n, const int *dofs, const int *row_ptr, const int *col_ind, int *table)
{
  int i, j;
  for (i = 0; i < n; i++)
    for (j = 0; j < n; j++) {
      int r = dofs[j];
      table[j + i * n] = find_col(col_ind, row_ptr[r], row_ptr[r + 1], dofs[i]);
    }
  for (j = 0; j < n; j++) table[n * n + j] = dofs[j];
}

/* Breadth-first first-fit colouring (utd_util/uts_coloring.cpp:61-150,
   utr_first_fit_coloring_with_front): entities that share a DOF are
   neighbours; each entity taken from the front gets the smallest colour
   not used by an already coloured neighbour. */
int orc_color_entities(int nent, int nv, const int *ent_dofs, int ndof, int *color)
{
  int *cnt = (int *)calloc(ndof + 1, sizeof(int));
  int e, j, k;
  for (e = 0; e < nent; e++)
    for (j = 0; j < nv; j++) cnt[ent_dofs[(size_t)e * nv + j] + 1]++;
  for (k = 0; k < ndof; k++) cnt[k + 1] += cnt[k];
  int *inc = (int *)malloc((size_t)cnt[ndof] * sizeof(int) + 4);
  int *fill = (int *)calloc((size_t)ndof + 1, sizeof(int));
  for (e = 0; e < nent; e++)
    for (j = 0; j < nv; j++) { int d = ent_dofs[(size_t)e * nv + j]; inc[cnt[d] + fill[d]++] = e; }
  int *queue = (int *)malloc((nent + 1) * sizeof(int));
  char *seen = (char *)calloc(nent + 1, 1);
  int ncol = 0, cap = 256, qh = 0, qt = 0, start = 0, done = 0;
  int *used = (int *)malloc(cap * sizeof(int));
  for (k = 0; k < cap; k++) used[k] = -1;
  for (e = 0; e < nent; e++) color[e] = -1;
  while (done < nent) {
    if (qh == qt) {
      while (start < nent && color[start] >= 0) start++;
      if (start >= nent) break;
      queue[qt++] = start; seen[start] = 1;
    }
    int cur = queue[qh++];
    for (j = 0; j < nv; j++) {
      int d = ent_dofs[(size_t)cur * nv + j];
      for (k = cnt[d]; k < cnt[d + 1]; k++) {
        int nb = inc[k];
        if (nb == cur) continue;
        if (color[nb] >= 0) used[color[nb]] = cur;
        if (!seen[nb]) { seen[nb] = 1; queue[qt++] = nb; }
      }
    }
    int c = 0;
    while (c < ncol && used[c] == cur) c++;
    if (c == ncol) {
      ncol++;
      if (ncol >= cap) {
        used = (int *)realloc(used, 2 * cap * sizeof(int));
        for (k = cap; k < 2 * cap; k++) used[k] = -1;
        cap *= 2;
      }
    }
    color[cur] = c;
    done++;
  }
  free(cnt); free(inc); free(fill); free(queue); free(seen); free(used);
  return ncol;
}

/* Elements, then boundary faces, integrated and added into the CRS arrays
   through per-entity tables, one colour at a time (uts_ls_intf.c:4103-4290
   element loop; lar_assemble_SM_and_LV_with_table_crs,
   las_crs_intf.c:440-518).  Faces are assembled serially before the
   elements. */
/* when set, the assemble routine adds |entries| instead of entries: the sum
   of absolute contributions that bounds the rounding error of every assembled
   value, used as the error scale of the parity tests */
static int g_accumulate_abs = 0;
void orc_set_accumulate_abs(int on) { g_accumulate_abs = on; }

double orc_std_prism_assemble(int nel, const int *el_nodes, const double *coords, const double *k_el,
                              const double *D_el, double f, int nfa, const int *fa_el,
                              const int *fa_side, double penalty, double g,
                              const int *dof_of_node, const int *row_ptr, const int *col_ind,
                              const int *el_color_ptr, const int *el_perm, int nthreads,
                              double *val, double *rhs)
{
  double t0 = now_s();
  int ifa;
  for (ifa = 0; ifa < nfa; ifa++) {
    int e = fa_el[ifa], j, dofs[6], table[42];
    double X[18], sm[36], r[6];
    for (j = 0; j < 6; j++) {
      int nd = el_nodes[(size_t)e * 6 + j];
      X[3 * j] = coords[3 * (size_t)nd]; X[3 * j + 1] = coords[3 * (size_t)nd + 1]; X[3 * j + 2] = coords[3 * (size_t)nd + 2];
      dofs[j] = dof_of_node[nd];
    }
    orc_std_prism_face(X, fa_side[ifa], penalty, g, sm, r);
    orc_crs_table(6, dofs, row_ptr, col_ind, table);
    for (j = 0; j < 36; j++) val[table[j]] += g_accumulate_abs ? fabs(sm[j]) : sm[j];
    for (j = 0; j < 6; j++) rhs[table[36 + j]] += g_accumulate_abs ? fabs(r[j]) : r[j];
  }
  int ncol = el_color_ptr ? 1 : 0, c;
  if (el_color_ptr) { while (el_color_ptr[ncol] < nel) ncol++; }
  if (!el_color_ptr) ncol = 1;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  for (c = 0; c < ncol; c++) {
    int lo = el_color_ptr ? el_color_ptr[c] : 0, hi = el_color_ptr ? el_color_ptr[c + 1] : nel;
    int ii;
#pragma omp parallel for schedule(static) if (nthreads > 1 && el_color_ptr)
    for (ii = lo; ii < hi; ii++) {
      int e = el_perm ? el_perm[ii] : ii, j, dofs[6], table[42];
      double X[18], sm[36], r[6], A[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
      for (j = 0; j < 6; j++) {
        int nd = el_nodes[(size_t)e * 6 + j];
        X[3 * j] = coords[3 * (size_t)nd]; X[3 * j + 1] = coords[3 * (size_t)nd + 1]; X[3 * j + 2] = coords[3 * (size_t)nd + 2];
        dofs[j] = dof_of_node[nd];
      }
      if (D_el) { for (j = 0; j < 9; j++) A[j] = D_el[9 * (size_t)e + j]; }
      else { double k = k_el ? k_el[e] : 1.0; A[0] = A[4] = A[8] = k; }
      orc_std_prism_element(X, A, f, sm, r);
      orc_crs_table(6, dofs, row_ptr, col_ind, table);
      for (j = 0; j < 36; j++) val[table[j]] += g_accumulate_abs ? fabs(sm[j]) : sm[j];
      for (j = 0; j < 6; j++) rhs[table[36 + j]] += g_accumulate_abs ? fabs(r[j]) : r[j];
    }
  }
  return now_s() - t0;
}

/* lar_compute_residual_crs (lsd_mkb/lad_crs/las_crs_intf.c:788-856). */
void orc_crs_residual(int n, const int *row_ptr, const int *col_ind, const double *val,
                      int use_rhs, const double *b, const double *x, double *v)
{
  int r;
#pragma omp parallel for schedule(static)
  for (r = 0; r < n; r++) {
    double s = use_rhs ? b[r] : 0.0;
    int k;
    for (k = row_ptr[r]; k < row_ptr[r + 1]; k++) s -= val[k] * x[col_ind[k]];
    v[r] = s;
  }
}

static double dot(int n, const double *a, const double *b)
{
  double s = 0.0; int i;
  for (i = 0; i < n; i++) s += a[i] * b[i];
  return s;
}

/* Restarted left-preconditioned GMRES with classical Gram-Schmidt and Givens
   rotations (lsd_mkb/lsd_mkb_core/lss_mkb_core.c:2317-2660,
   lsr_mkb_core_gmres) with the point-Jacobi preconditioner 1/a_ii
   (lar_fill_preconditioner_crs, las_crs_intf.c:707).  The preconditioned
   operator is applied as D^-1 A v directly (the reference goes through one
   Jacobi smoothing sweep, lss_mkb_core.c:2003-2055, which equals it up to
   rounding). */
int orc_gmres_jacobi(int n, const int *row_ptr, const int *col_ind, const double *val,
                     const double *b, double *x, int krylov, int max_iter, double tol_rel,
                     double *res_out, double *res_rel_out)
{
  int m = krylov, i, k, r;
  double *dinv = (double *)malloc(n * sizeof(double));
  double *V = (double *)malloc((size_t)n * (m + 1) * sizeof(double));
  double *H = (double *)calloc((size_t)(m + 1) * (m + 1), sizeof(double));
  double *cs = (double *)malloc((m + 1) * sizeof(double)), *sn = (double *)malloc((m + 1) * sizeof(double));
  double *s = (double *)malloc((m + 2) * sizeof(double));
  double *tmp = (double *)malloc(n * sizeof(double));
  for (r = 0; r < n; r++) {
    int kk;
    dinv[r] = 1.0;
    for (kk = row_ptr[r]; kk < row_ptr[r + 1]; kk++)
      if (col_ind[kk] == r) dinv[r] = 1.0 / val[kk];
  }
  double tol_abs = 1e-12, beta0 = -1.0, resid = 0.0;
  int it = 0;
  if (tol_rel < 1e-12) tol_rel = 1e-12;
  for (;;) {
    orc_crs_residual(n, row_ptr, col_ind, val, 1, b, x, tmp);
    for (i = 0; i < n; i++) V[i] = dinv[i] * tmp[i];
    double rn = sqrt(dot(n, V, V));
    if (beta0 < 0) beta0 = rn;
    resid = rn;
    if (rn < tol_abs || (beta0 > 0 && rn / beta0 < tol_rel) || it >= max_iter) break;
    for (i = 0; i < n; i++) V[i] /= rn;
    s[0] = rn;
    for (i = 1; i <= m; i++) s[i] = 0.0;
    int j, done = 0;
    for (j = 0; j < m; j++) {
      double *w = V + (size_t)(j + 1) * n;
      it++;
      orc_crs_residual(n, row_ptr, col_ind, val, 0, NULL, V + (size_t)j * n, tmp);
      for (i = 0; i < n; i++) w[i] = -dinv[i] * tmp[i];
      for (k = 0; k <= j; k++) H[k + j * (m + 1)] = dot(n, V + (size_t)k * n, w);
      for (k = 0; k <= j; k++) {
        double h = H[k + j * (m + 1)];
        double *vk = V + (size_t)k * n;
        for (i = 0; i < n; i++) w[i] -= h * vk[i];
      }
      double hn = sqrt(dot(n, w, w));
      H[j + 1 + j * (m + 1)] = hn;
      for (i = 0; i < n; i++) w[i] /= hn;
      for (k = 0; k < j; k++) {
        double a = H[k + j * (m + 1)], bb = H[k + 1 + j * (m + 1)];
        H[k + j * (m + 1)] = cs[k] * a + sn[k] * bb;
        H[k + 1 + j * (m + 1)] = cs[k] * bb - sn[k] * a;
      }
      {
        double a = H[j + j * (m + 1)], bb = H[j + 1 + j * (m + 1)];
        double rr = hypot(a, bb);
        cs[j] = a / rr; sn[j] = bb / rr;
        H[j + j * (m + 1)] = rr; H[j + 1 + j * (m + 1)] = 0.0;
        double s0 = s[j];
        s[j] = cs[j] * s0; s[j + 1] = -sn[j] * s0;
      }
      resid = fabs(s[j + 1]);
      if (j == m - 1 || it >= max_iter || resid < tol_abs || resid / beta0 < tol_rel) { done = j + 1; break; }
    }
    /* y = H^-1 s (upper triangular), x += V y */
    for (k = done - 1; k >= 0; k--) {
      double t = s[k];
      for (i = k + 1; i < done; i++) t -= H[k + i * (m + 1)] * s[i];
      s[k] = t / H[k + k * (m + 1)];
    }
    for (k = 0; k < done; k++) {
      double *vk = V + (size_t)k * n;
      for (i = 0; i < n; i++) x[i] += s[k] * vk[i];
    }
    if (resid < tol_abs || resid / beta0 < tol_rel || it >= max_iter) break;
  }
  *res_out = resid;
  *res_rel_out = beta0 > 0 ? resid / beta0 : 0.0;
  free(dinv); free(V); free(H); free(cs); free(sn); free(s); free(tmp);
  return it;
}

/* ------------------------------------------------------------------ */
/* DG prism elements (apd_dg_prism)                                    */
/* ------------------------------------------------------------------ */

/* Tensor DG basis of degree p (pdeg = 101 p): monomials xi^a eta^b zeta^c in
   the reference's order (apr_shape_fun_3D, apd_dg_prism/aps_dg_util.c:408-995;
   ordering table in dg_tables.h) and their local derivatives. */
static int dg_shape(int p, const double *e, double *phi, double *dx, double *dy, double *dz)
{
  int ns = GB_DG_NS[p], i;
  double px[8], py[8], pz[8];
  px[0] = py[0] = pz[0] = 1.0;
  for (i = 1; i <= p; i++) { px[i] = px[i - 1] * e[0]; py[i] = py[i - 1] * e[1]; pz[i] = pz[i - 1] * e[2]; }
  for (i = 0; i < ns; i++) {
    int a = GB_DG_EXP[p - 1][i][0], b = GB_DG_EXP[p - 1][i][1], c = GB_DG_EXP[p - 1][i][2];
    phi[i] = px[a] * py[b] * pz[c];
    dx[i] = a ? a * px[a - 1] * py[b] * pz[c] : 0.0;
    dy[i] = b ? b * px[a] * py[b - 1] * pz[c] : 0.0;
    dz[i] = c ? c * px[a] * py[b] * pz[c - 1] : 0.0;
  }
  return ns;
}

int orc_dg_nshape(int p) { return (p >= 1 && p <= GB_DG_PMAX) ? GB_DG_NS[p] : -1; }

/* the DG face rule of degree p (apr_set_quadr_2D of the DG module, ti 0
   triangle, 1 quadrilateral): (s, t, w) per point; returns the point count */
int orc_dg_face_rule(int p, int ti, double *out)
{
  int q, nq;
  if (p < 1 || p > GB_DG_PMAX || ti < 0 || ti > 1) return -1;
  nq = GB_DG_NQF[p][ti];
  for (q = 0; q < nq; q++) {
    out[3 * q] = GB_DG_FQ[p - 1][ti][q][0];
    out[3 * q + 1] = GB_DG_FQ[p - 1][ti][q][1];
    out[3 * q + 2] = GB_DG_FQ[p - 1][ti][q][2];
  }
  return nq;
}

/* the tensor basis exponents (a, b, c) of degree p in the reference's order */
int orc_dg_exponents(int p, int *out)
{
  int i;
  if (p < 1 || p > GB_DG_PMAX) return -1;
  for (i = 0; i < GB_DG_NS[p]; i++) {
    out[3 * i] = GB_DG_EXP[p - 1][i][0];
    out[3 * i + 1] = GB_DG_EXP[p - 1][i][1];
    out[3 * i + 2] = GB_DG_EXP[p - 1][i][2];
  }
  return GB_DG_NS[p];
}

/* apr_num_int_el of the DG module (apd_dg_prism/aps_dg_prism_intf.c:1239-1728)
   for nreq = 1: the volume rule of apr_set_quadr_3D (aps_dg_util.c:1415-1480),
   the prism geometry of apr_elem_calc_3D (aps_dg_util.c:112-400), the 9-term
   diffusion (:1582-1606) and the source term (:1680-1715). */
int orc_dg_prism_element(const double *X, const double *A, double f, int p, double *sm, double *rhs)
{
  int ns, nq, q, i;
  if (p < 1 || p > GB_DG_PMAX) return -1;
  ns = GB_DG_NS[p];
  nq = GB_DG_NQ[p];
  memset(sm, 0, (size_t)ns * ns * sizeof(double));
  memset(rhs, 0, (size_t)ns * sizeof(double));
  for (q = 0; q < nq; q++) {
    const double *qp = GB_DG_QP[p - 1][q];
    double phi[GB_DG_MAXNS], dx[GB_DG_MAXNS], dy[GB_DG_MAXNS], dz[GB_DG_MAXNS];
    double gx[GB_DG_MAXNS], gy[GB_DG_MAXNS], gz[GB_DG_MAXNS];
    double e[3] = {qp[0], qp[1], qp[2]};
    double ph6[6], d6x[6], d6y[6], d6z[6], J[9], Ji[9];
    dg_shape(p, e, phi, dx, dy, dz);
    prism_shape(e, ph6, d6x, d6y, d6z);
    prism_jacobian(X, d6x, d6y, d6z, J);
    double det = fabs(mat3_inv(J, Ji));
    for (i = 0; i < ns; i++) {
      gx[i] = dx[i] * Ji[0] + dy[i] * Ji[3] + dz[i] * Ji[6];
      gy[i] = dx[i] * Ji[1] + dy[i] * Ji[4] + dz[i] * Ji[7];
      gz[i] = dx[i] * Ji[2] + dy[i] * Ji[5] + dz[i] * Ji[8];
    }
    accumulate_qp(ns, phi, gx, gy, gz, A, f, det * qp[3], sm, rhs);
  }
  return ns;
}

/* ------------------------------------------------------------------ */
/* DG prism faces                                                      */
/* ------------------------------------------------------------------ */

/* local coordinates of the six prism vertices */
static const double PRISM_VLOC[6][3] = {{0, 0, -1}, {1, 0, -1}, {0, 1, -1}, {0, 0, 1}, {1, 0, 1}, {0, 1, 1}};

/* |ds| and the outward normal on element side `side` at local point e
   (apr_elem_calc_3D control 3 + side; the same side formulas as the std
   prism, aps_std_util.c:770-805) */
static double prism_side_ds(const double *X, int side, const double *e, double *nrm)
{
  double phi[6], dx[6], dy[6], dz[6], J[9], ds[3];
  prism_shape(e, phi, dx, dy, dz);
  prism_jacobian(X, dx, dy, dz, J);
  if (side == 0) {
    ds[0] = -J[3] * J[7] + J[6] * J[4]; ds[1] = -J[6] * J[1] + J[0] * J[7]; ds[2] = -J[0] * J[4] + J[3] * J[1];
  } else if (side == 1) {
    ds[0] = J[3] * J[7] - J[6] * J[4]; ds[1] = J[6] * J[1] - J[0] * J[7]; ds[2] = J[0] * J[4] - J[3] * J[1];
  } else if (side == 2) {
    ds[0] = J[3] * J[8] - J[6] * J[5]; ds[1] = J[6] * J[2] - J[0] * J[8]; ds[2] = J[0] * J[5] - J[3] * J[2];
  } else if (side == 3) {
    ds[0] = (J[4] - J[3]) * J[8] - (J[7] - J[6]) * J[5];
    ds[1] = (J[7] - J[6]) * J[2] - (J[1] - J[0]) * J[8];
    ds[2] = (J[1] - J[0]) * J[5] - (J[4] - J[3]) * J[2];
  } else {
    ds[0] = J[5] * J[7] - J[8] * J[4]; ds[1] = J[8] * J[1] - J[2] * J[7]; ds[2] = J[2] * J[4] - J[5] * J[1];
  }
  double d = sqrt(ds[0] * ds[0] + ds[1] * ds[1] + ds[2] * ds[2]);
  nrm[0] = ds[0] / d; nrm[1] = ds[1] / d; nrm[2] = ds[2] / d;
  return d;
}

/* basis values and global gradients of a DG element at local point e */
static void dg_eval(const double *X, int p, const double *e, double *phi, double *gx, double *gy, double *gz)
{
  double dx[GB_DG_MAXNS], dy[GB_DG_MAXNS], dz[GB_DG_MAXNS], ph6[6], d6x[6], d6y[6], d6z[6], J[9], Ji[9];
  int i, ns = dg_shape(p, e, phi, dx, dy, dz);
  prism_shape(e, ph6, d6x, d6y, d6z);
  prism_jacobian(X, d6x, d6y, d6z, J);
  mat3_inv(J, Ji);
  for (i = 0; i < ns; i++) {
    gx[i] = dx[i] * Ji[0] + dy[i] * Ji[3] + dz[i] * Ji[6];
    gy[i] = dx[i] * Ji[1] + dy[i] * Ji[4] + dz[i] * Ji[7];
    gz[i] = dx[i] * Ji[2] + dy[i] * Ji[5] + dz[i] * Ji[8];
  }
}

/* mmr_fa_area (mmd_prism/mms_prism_datstr.c:1732-1790) from the face vertices
   in face order: triangle 0.5|a x b|, quadrilateral 0.5(|a x b| + |c x d|) */
static double face_area(const double *V, int nfv)
{
  double a[3], b[3], e[3];
  int i;
  for (i = 0; i < 3; i++) { a[i] = V[3 + i] - V[i]; b[i] = V[6 + i] - V[3 + i]; }
  e[0] = a[1] * b[2] - a[2] * b[1]; e[1] = a[2] * b[0] - a[0] * b[2]; e[2] = a[0] * b[1] - a[1] * b[0];
  double s = sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
  if (nfv == 3) return 0.5 * s;
  double c[3], d[3], f[3];
  for (i = 0; i < 3; i++) { c[i] = V[9 + i] - V[6 + i]; d[i] = V[i] - V[9 + i]; }
  f[0] = c[1] * d[2] - c[2] * d[1]; f[1] = c[2] * d[0] - c[0] * d[2]; f[2] = c[0] * d[1] - c[1] * d[0];
  return 0.5 * (s + sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]));
}

/* DG face integral of the conv-diff weak form for nreq = 1, steady
   (implicitness 1), no convection (pdd_conv_diff/weak_formulation/approx_dg/
   pds_conv_diff_weakform_dg.c:232-1140): interior faces give the four blocks
   of the non-symmetric interior penalty form with the normal diffusion
   An = A^T n of each side and penalty pen * min(p1, p2) / sqrt(face area);
   Dirichlet faces give the boundary form with penalty pen * p1 and data g.
   Face rule: the DG face quadrature of the side with more points
   (apr_set_quadr_2D, aps_dg_util.c); a face point is placed in each element
   by the weights of the face's vertices (barycentric on triangles, bilinear
   on quadrilaterals), which is how both elements' maps restrict to the face.
   loc1/loc2: local vertex index in each element of the face vertices in face
   order.  sm: (ns1+ns2)^2 column-major, rhs: ns1+ns2.  Returns ns1+ns2. */
int orc_dg_face(int ftype, const double *X1, const int *loc1, int p1, const double *A1, int side1,
                const double *X2, const int *loc2, int p2, const double *A2, double pen, double g,
                double *sm, double *rhs)
{
  int nfv = ftype == 4 ? 4 : 3, i, j, q;
  int ns1 = GB_DG_NS[p1], ns2 = X2 ? GB_DG_NS[p2] : 0, n = ns1 + ns2;
  int ti = ftype == 4 ? 1 : 0;
  int pr = p1;
  if (X2 && GB_DG_NQF[p2][ti] > GB_DG_NQF[p1][ti]) pr = p2;
  int nq = GB_DG_NQF[pr][ti];
  double V[12];
  for (i = 0; i < nfv; i++) for (j = 0; j < 3; j++) V[3 * i + j] = X1[3 * loc1[i] + j];
  double hf = sqrt(face_area(V, nfv));
  double penalty = pen * (X2 ? (p1 < p2 ? p1 : p2) : p1);
  memset(sm, 0, (size_t)n * n * sizeof(double));
  memset(rhs, 0, (size_t)n * sizeof(double));
  for (q = 0; q < nq; q++) {
    const double *fq = GB_DG_FQ[pr - 1][ti][q];
    double w[4];
    if (nfv == 3) { w[0] = 1.0 - fq[0] - fq[1]; w[1] = fq[0]; w[2] = fq[1]; }
    else {
      double u = (fq[0] + 1.0) / 2.0, v = (fq[1] + 1.0) / 2.0;
      w[0] = (1.0 - u) * (1.0 - v); w[1] = u * (1.0 - v); w[2] = u * v; w[3] = (1.0 - u) * v;
    }
    double e1[3] = {0, 0, 0}, e2[3] = {0, 0, 0};
    for (i = 0; i < nfv; i++)
      for (j = 0; j < 3; j++) {
        e1[j] += w[i] * PRISM_VLOC[loc1[i]][j];
        if (X2) e2[j] += w[i] * PRISM_VLOC[loc2[i]][j];
      }
    double nrm[3];
    double area = prism_side_ds(X1, side1, e1, nrm) * fq[2];
    double phi1[GB_DG_MAXNS], gx1[GB_DG_MAXNS], gy1[GB_DG_MAXNS], gz1[GB_DG_MAXNS], g1[GB_DG_MAXNS];
    double phi2[GB_DG_MAXNS], gx2[GB_DG_MAXNS], gy2[GB_DG_MAXNS], gz2[GB_DG_MAXNS], g2[GB_DG_MAXNS];
    dg_eval(X1, p1, e1, phi1, gx1, gy1, gz1);
    double an1[3] = {A1[0] * nrm[0] + A1[3] * nrm[1] + A1[6] * nrm[2], A1[1] * nrm[0] + A1[4] * nrm[1] + A1[7] * nrm[2],
                     A1[2] * nrm[0] + A1[5] * nrm[1] + A1[8] * nrm[2]};
    for (i = 0; i < ns1; i++) g1[i] = an1[0] * gx1[i] + an1[1] * gy1[i] + an1[2] * gz1[i];
    if (X2) {
      dg_eval(X2, p2, e2, phi2, gx2, gy2, gz2);
      double an2[3] = {A2[0] * nrm[0] + A2[3] * nrm[1] + A2[6] * nrm[2],
                       A2[1] * nrm[0] + A2[4] * nrm[1] + A2[7] * nrm[2],
                       A2[2] * nrm[0] + A2[5] * nrm[1] + A2[8] * nrm[2]};
      for (i = 0; i < ns2; i++) g2[i] = an2[0] * gx2[i] + an2[1] * gy2[i] + an2[2] * gz2[i];
      /* columns j (trial), rows i (test) */
      for (j = 0; j < ns1; j++)
        for (i = 0; i < ns1; i++)
          sm[(size_t)j * n + i] += ((phi1[j] * g1[i] - phi1[i] * g1[j]) * 0.5 * 1.0 + penalty * phi1[j] * phi1[i] / hf) * area;
      for (j = 0; j < ns2; j++)
        for (i = 0; i < ns1; i++)
          sm[(size_t)(ns1 + j) * n + i] += ((-phi2[j] * g1[i] - phi1[i] * g2[j]) * 0.5 * 1.0 - penalty * phi2[j] * phi1[i] / hf) * area;
      for (j = 0; j < ns1; j++)
        for (i = 0; i < ns2; i++)
          sm[(size_t)j * n + ns1 + i] += ((phi1[j] * g2[i] + phi2[i] * g1[j]) * 0.5 * 1.0 - penalty * phi1[j] * phi2[i] / hf) * area;
      for (j = 0; j < ns2; j++)
        for (i = 0; i < ns2; i++)
          sm[(size_t)(ns1 + j) * n + ns1 + i] += ((-phi2[j] * g2[i] + phi2[i] * g2[j]) * 0.5 * 1.0 + penalty * phi2[j] * phi2[i] / hf) * area;
    } else {
      for (j = 0; j < ns1; j++)
        for (i = 0; i < ns1; i++)
          sm[(size_t)j * n + i] += ((g1[i] * phi1[j] - g1[j] * phi1[i]) * 1.0 + penalty * phi1[j] * phi1[i] / hf) * area;
      for (i = 0; i < ns1; i++) rhs[i] += (g1[i] * g + penalty * g * phi1[i] / hf) * area;
    }
  }
  return n;
}
