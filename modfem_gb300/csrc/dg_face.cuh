// DG prism face integrals (interior penalty and Dirichlet boundary forms),
// shared by the CUDA face kernel and a host-compiled check against the oracle.
//
// Reference: pdr_conv_diff_comp_fa_stiff_mat_app of the DG weak form
// (pdd_conv_diff/weak_formulation/approx_dg/pds_conv_diff_weakform_dg.c:
// 232-1140) for nreq = 1, steady, no convection:
//   interior face, normal n outward from the first neighbour (side 1), An_s =
//   A_s^T n, g_s = An_s . grad phi_s, c = pen min(p1, p2) / sqrt(face area):
//     K11 += a [ 0.5 (phi1_j g1_i - phi1_i g1_j) + c phi1_j phi1_i ]
//     K12 += a [ 0.5 (-phi2_j g1_i - phi1_i g2_j) - c phi2_j phi1_i ]
//     K21 += a [ 0.5 (phi1_j g2_i + phi2_i g1_j) - c phi1_j phi2_i ]
//     K22 += a [ 0.5 (-phi2_j g2_i + phi2_i g2_j) + c phi2_j phi2_i ]
//   (row i test, column j trial, a = |ds| w_q);
//   Dirichlet face with data g: the same K11 with factor 1 instead of 0.5 and
//   c = pen p1 / sqrt(area), and R1_i += a (g1_i g + c g phi1_i).
//
// Every block is a sum over points of two rank-one products.  For the rows of
// side o (the element that owns them) define per point
//     L_i = f a g_i + s_o c a phi_i,   M_i = -s_o f a phi_i
// (f = 0.5 interior / 1 boundary, s_1 = +1, s_2 = -1) and for the columns of
// side t: Phi_j = s_t phi_j, Gam_j = g_j.  Then every block row of the face is
//     K[i][j] = sum_q L_i Phi_j + M_i Gam_j,
// and the Dirichlet load is R_i = g sum_q L_i.  One element can therefore
// integrate its own rows of every face it touches (its diagonal block and its
// off-diagonal block of that face) without the neighbour's rows: two FP64 FMA
// per matrix entry and point.
#pragma once

#include "dg_tables.h"
#include "prism_std.cuh"

namespace gbfem {

// local coordinates of the prism vertices (bottom triangle, then top)
GB_HD v3 prism_vertex_local(int i) {
  const double xi = (i == 1 || i == 4) ? 1.0 : 0.0;
  const double eta = (i == 2 || i == 5) ? 1.0 : 0.0;
  return {xi, eta, i < 3 ? -1.0 : 1.0};
}

// Columns j_a = dx/dxi_a of the Jacobian of the linear prism at local point e.
GB_HD void prism_jacobian_columns(const double *X, v3 e, v3 &j1, v3 &j2, v3 &j3) {
  const double lo = (1.0 - e.z) / 2.0, hi = (1.0 + e.z) / 2.0, l0 = 1.0 - e.x - e.y;
  const double dx[6] = {-lo, lo, 0.0, -hi, hi, 0.0};
  const double dy[6] = {-lo, 0.0, lo, -hi, 0.0, hi};
  const double dz[6] = {-0.5 * l0, -0.5 * e.x, -0.5 * e.y, 0.5 * l0, 0.5 * e.x, 0.5 * e.y};
  j1 = {0, 0, 0};
  j2 = {0, 0, 0};
  j3 = {0, 0, 0};
#pragma unroll
  for (int i = 0; i < 6; i++) {
    const v3 x = {X[3 * i], X[3 * i + 1], X[3 * i + 2]};
    j1 = v3_fma(dx[i], x, j1);
    j2 = v3_fma(dy[i], x, j2);
    j3 = v3_fma(dz[i], x, j3);
  }
}

// Outward side vector (|.| = surface Jacobian) of prism side 0 (bottom),
// 1 (top), 2..4 (lateral over triangle edges 0..2), the side formulas of
// apr_elem_calc_3D (apd_std_lin/aps_std_util.c:770-805).
GB_HD v3 prism_side_vector(int side, v3 j1, v3 j2, v3 j3) {
  switch (side) {
    case 0: return v3_scale(-1.0, v3_cross(j1, j2));
    case 1: return v3_cross(j1, j2);
    case 2: return v3_cross(j1, j3);
    case 3: return v3_cross(v3_sub(j2, j1), j3);
    default: return v3_cross(j3, j2);
  }
}

// mmr_fa_area (mmd_prism/mms_prism_datstr.c:1732-1790) from the face vertices
// in face order: triangle |a x b| / 2, quadrilateral (|a x b| + |c x d|) / 2.
GB_HD double dg_face_area(const v3 *V, int nfv) {
  const v3 a = v3_sub(V[1], V[0]), b = v3_sub(V[2], V[1]);
  const double s = sqrt(v3_dot(v3_cross(a, b), v3_cross(a, b)));
  if (nfv == 3) return 0.5 * s;
  const v3 c = v3_sub(V[3], V[2]), d = v3_sub(V[0], V[3]);
  const v3 cd = v3_cross(c, d);
  return 0.5 * (s + sqrt(v3_dot(cd, cd)));
}

// Geometry of one face point: the point in each neighbour's local
// coordinates (through the face-vertex weights: barycentric on triangles,
// bilinear on quadrilaterals), the area weight a = |ds| w and, per side, the
// vector v = J^-1 A^T n so that g_i = An . grad phi_i = v . dphi_i/dxi.
struct DgFacePoint {
  v3 e1, e2, v1, v2;
  double a;
};

GB_HD v3 dg_face_v(const double *X, v3 e, const double *A, v3 n) {
  v3 j1, j2, j3;
  prism_jacobian_columns(X, e, j1, j2, j3);
  const v3 c1 = v3_cross(j2, j3), c2 = v3_cross(j3, j1), c3 = v3_cross(j1, j2);
  const double rdet = 1.0 / v3_dot(j1, c1);
  // An = A^T n with A row-major (a_ij multiplies d_i(test) d_j(trial))
  const v3 an = {A[0] * n.x + A[3] * n.y + A[6] * n.z, A[1] * n.x + A[4] * n.y + A[7] * n.z,
                 A[2] * n.x + A[5] * n.y + A[8] * n.z};
  return {v3_dot(c1, an) * rdet, v3_dot(c2, an) * rdet, v3_dot(c3, an) * rdet};
}

// fq = (s, t, w) of the face rule; loc: local vertex index in each neighbour
// of the face vertices in face order.  X2/A2 NULL on the boundary.
GB_HD DgFacePoint dg_face_point(int nfv, const double *fq, const double *X1, const unsigned char *loc1,
                                int side1, const double *A1, const double *X2, const unsigned char *loc2,
                                const double *A2) {
  double w[4];
  if (nfv == 3) {
    w[0] = 1.0 - fq[0] - fq[1];
    w[1] = fq[0];
    w[2] = fq[1];
    w[3] = 0.0;
  } else {
    const double u = (fq[0] + 1.0) / 2.0, v = (fq[1] + 1.0) / 2.0;
    w[0] = (1.0 - u) * (1.0 - v);
    w[1] = u * (1.0 - v);
    w[2] = u * v;
    w[3] = (1.0 - u) * v;
  }
  DgFacePoint P;
  P.e1 = {0, 0, 0};
  P.e2 = {0, 0, 0};
#pragma unroll
  for (int i = 0; i < 4; i++) {
    if (i >= nfv) break;
    P.e1 = v3_fma(w[i], prism_vertex_local(loc1[i]), P.e1);
    if (X2) P.e2 = v3_fma(w[i], prism_vertex_local(loc2[i]), P.e2);
  }
  v3 j1, j2, j3;
  prism_jacobian_columns(X1, P.e1, j1, j2, j3);
  const v3 ds = prism_side_vector(side1, j1, j2, j3);
  const double d = sqrt(v3_dot(ds, ds));
  const v3 n = v3_scale(1.0 / d, ds);  // one division, three products
  P.a = d * fq[2];
  P.v1 = dg_face_v(X1, P.e1, A1, n);
  P.v2 = X2 ? dg_face_v(X2, P.e2, A2, n) : v3{0, 0, 0};
  return P;
}

// local coordinates of the tetrahedron vertices (0,0,0), (1,0,0), (0,1,0), (0,0,1)
GB_HD v3 tet_vertex_local(int k) { return {k == 1 ? 1.0 : 0.0, k == 2 ? 1.0 : 0.0, k == 3 ? 1.0 : 0.0}; }

// v = J^-1 A^T n for the affine tetrahedron X[12] (J constant: columns
// X1-X0, X2-X0, X3-X0)
GB_HD v3 tet_face_v(const double *X, const double *A, v3 n) {
  const v3 x0 = {X[0], X[1], X[2]};
  const v3 j1 = v3_sub(v3{X[3], X[4], X[5]}, x0), j2 = v3_sub(v3{X[6], X[7], X[8]}, x0),
           j3 = v3_sub(v3{X[9], X[10], X[11]}, x0);
  const v3 c1 = v3_cross(j2, j3), c2 = v3_cross(j3, j1), c3 = v3_cross(j1, j2);
  const double rdet = 1.0 / v3_dot(j1, c1);
  const v3 an = {A[0] * n.x + A[3] * n.y + A[6] * n.z, A[1] * n.x + A[4] * n.y + A[7] * n.z,
                 A[2] * n.x + A[5] * n.y + A[8] * n.z};
  return {v3_dot(c1, an) * rdet, v3_dot(c2, an) * rdet, v3_dot(c3, an) * rdet};
}

// Per point and side, the monomial factors of the basis: powers
// T[k][m] = x_k^m and the gradient factors T[3 + k][m] = m x_k^(m-1) v_k
// (m = 0..4, k = xi, eta, zeta), so that for xi^a eta^b zeta^c
//   phi = T0[a] T1[b] T2[c],
//   g = v . grad_xi phi = T3[a] T1[b] T2[c] + T0[a] (T4[b] T2[c] + T1[b] T5[c]),
// six FP64 operations per function instead of forming powers per function.
GB_HD void dg_point_factors(v3 e, v3 v, double *T /* [6][5] */) {
  const double x[3] = {e.x, e.y, e.z}, w[3] = {v.x, v.y, v.z};
  for (int k = 0; k < 3; k++) {
    double p = 1.0, q = 0.0;  // x^m and m x^(m-1)
    for (int m = 0; m <= GB_DG_PMAX; m++) {
      T[5 * k + m] = p;
      T[5 * (3 + k) + m] = q * w[k];
      q = fma(q, x[k], p);
      p *= x[k];
    }
  }
}

GB_HD void dg_basis_from_factors(const double *T, int a, int b, int c, double &phi, double &g) {
  const double u = T[5 + b] * T[10 + c];
  phi = T[a] * u;
  const double t = fma(T[5 + b], T[25 + c], T[20 + b] * T[10 + c]);
  g = fma(T[15 + a], u, T[a] * t);
}

// Row (L, M) and column (Phi, Gam) values of basis function (a, b, c) of
// side `side` (1 or 2) at one point; fac 0.5 interior / 1 boundary;
// cpen = penalty / sqrt(area).  L and M are used when the function's own
// element owns the rows, Phi and Gam in every block of the face.
GB_HD void dg_face_values(int a, int b, int c, int side, v3 e, v3 v, double area_w, double fac, double cpen,
                          double &L, double &M, double &Phi, double &Gam) {
  double T[30], phi, g;
  dg_point_factors(e, v, T);
  dg_basis_from_factors(T, a, b, c, phi, g);
  const double s = side == 1 ? 1.0 : -1.0;
  L = fma(fac * area_w, g, s * cpen * area_w * phi);
  M = -s * fac * area_w * phi;
  Phi = s * phi;
  Gam = g;
}

}  // namespace gbfem
