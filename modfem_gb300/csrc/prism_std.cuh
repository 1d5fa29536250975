// Element math of the standard linear prism, shared by the CUDA kernels and
// by a host-compiled check against the oracle (functions are host+device).
//
// Reference: apr_num_int_el (apd_std_lin/aps_std_lin_intf.c:1537-2880) with
// apr_elem_calc_3D_prism (aps_std_util.c:520-820) and the quadrature of
// apr_set_quadr_3D (aps_std_util.c:1380-1438; constants aps_gauss_util_std.c):
// two Gauss line points (zeta = -+0.577350269189626) x three triangle points
// ((1/6,1/6), (1/6,2/3), (2/3,1/6)), weight 0.5 * (1/3) each.
//
// FP64 instruction economy (GB300's FP64 rate is 1/64 of FP32):
//  * dx/dxi = m1 + zeta d1 and dx/deta = m2 + zeta d2 depend on zeta only,
//    dx/dzeta = c0 + xi d1 + eta d2 on (xi, eta) only;
//  * gradients are written with the adjugate rows c1 = j2 x j3, c2 = j3 x j1,
//    c3 = j1 x j2 (c3 per Gauss line point), no 3x3 inverse, and only their
//    dot products are formed (Binet-Cauchy, from the Jacobian's inner
//    products);
//  * shape-function derivative patterns make every unscaled gradient
//    g_{t,s} = h_s e_t + sigma_s (L_t/2) c3 with e = (-(c1+c2), c1, c2),
//    so the stiffness needs only the six products s*ci.cj per quadrature point
//    (s = k w / |det|); the 21 matrix entries are then linear combinations of
//    quadrature sums of those products with compile-time weights h_s(zeta),
//    L_t(xi, eta);
//  * the six determinants share one reciprocal (running products).
#pragma once

#include <math.h>

#if defined(__CUDACC__)
#define GB_HD __host__ __device__ __forceinline__
#else
#define GB_HD inline
#endif

namespace gbfem {

struct v3 {
  double x, y, z;
};
GB_HD v3 v3_add(v3 a, v3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
GB_HD v3 v3_sub(v3 a, v3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
GB_HD v3 v3_scale(double s, v3 a) { return {s * a.x, s * a.y, s * a.z}; }
GB_HD v3 v3_fma(double s, v3 a, v3 b) { return {fma(s, a.x, b.x), fma(s, a.y, b.y), fma(s, a.z, b.z)}; }
GB_HD v3 v3_cross(v3 a, v3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
GB_HD double v3_dot(v3 a, v3 b) { return fma(a.x, b.x, fma(a.y, b.y, a.z * b.z)); }

#define GB_PRISM_G2 0.577350269189626
#define GB_PRISM_T1 0.166666666666667
#define GB_PRISM_T2 0.666666666666667
#define GB_PRISM_TW 0.333333333333333

// Packed upper triangle of the 6x6 matrix: index of (u, w), u <= w, local
// vertex i = t + 3 s (t triangle vertex, s = 0 bottom / 1 top).
GB_HD int packed_index(int u, int w) { return u * 6 - (u * (u - 1)) / 2 + (w - u); }

// Isotropic coefficient kk: K (21 packed entries, K[u][w] = integral of
// kk grad phi_u . grad phi_w) and R (6, integral of f phi_w).
//
// Works with J' = 2J (columns j1' = M1 + zeta D1, j2' = M2 + zeta D2,
// j3' = C0 + xi D1 + eta D2 from plain vertex differences): det' = 8 det and
// the adjugate rows c' = 4c, so the stiffness scale k w / |det| on c.c
// becomes (k w / 2) / |det'| on c'.c', and the load scale w |det| becomes
// (w / 8) |det'|.  The adjugate rows enter only through their dot products,
// which the Binet-Cauchy identity (a x b).(c x d) = (a.c)(b.d) - (a.d)(b.c)
// gives from the six inner products a_ij = j_i'.j_j' in two operations each;
// det' = j3'.(j1' x j2').
// Pieces written for an arithmetic type T with +, -, *, unary -, t_fma,
// t_abs, construction from a double constant and a prism_recip6 overload
// (found by argument-dependent lookup).  The element below is instantiated
// for double; the double-word element (prism_dw.cuh) reuses the vector
// helpers with float pairs and restructures the quadrature sums.
GB_HD double t_fma(double a, double b, double c) { return fma(a, b, c); }
GB_HD double t_abs(double a) { return fabs(a); }

template <typename T>
struct vec3 {
  T x, y, z;
};
template <typename T>
GB_HD vec3<T> q_add(vec3<T> a, vec3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <typename T>
GB_HD vec3<T> q_sub(vec3<T> a, vec3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <typename T>
GB_HD vec3<T> q_fma(T s, vec3<T> a, vec3<T> b) { return {t_fma(s, a.x, b.x), t_fma(s, a.y, b.y), t_fma(s, a.z, b.z)}; }
template <typename T>
GB_HD vec3<T> q_cross(vec3<T> a, vec3<T> b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <typename T>
GB_HD T q_dot(vec3<T> a, vec3<T> b) { return t_fma(a.x, b.x, t_fma(a.y, b.y, a.z * b.z)); }

// inv[q] = 1/a[q] for the six determinants: one division and running
// products (FP64 division is a long instruction sequence)
GB_HD void prism_recip6(const double (&a)[6], double (&inv)[6]) {
  double pre[6];
  pre[0] = a[0];
#pragma unroll
  for (int q = 1; q < 6; q++) pre[q] = pre[q - 1] * a[q];
  double r = 1.0 / pre[5];
#pragma unroll
  for (int q = 5; q > 0; q--) {
    inv[q] = r * pre[q - 1];
    r = r * a[q];
  }
  inv[0] = r;
}

// Element math from the five vertex-difference vectors
// ea = X1 - X0, eb = X4 - X3, fa = X2 - X0, fb = X5 - X3, C0 = X3 - X0.
template <typename T>
GB_HD void prism_std_element_t(vec3<T> ea, vec3<T> eb, vec3<T> fa, vec3<T> fb, vec3<T> C0, T kk, T f,
                               T (&K)[21], T (&R)[6]) {
  const vec3<T> M1 = q_add(ea, eb), D1 = q_sub(eb, ea);
  const vec3<T> M2 = q_add(fa, fb), D2 = q_sub(fb, fa);
  const double wq = 0.5 * GB_PRISM_TW * 1.0;
  const double XI[3] = {GB_PRISM_T1, GB_PRISM_T1, GB_PRISM_T2};
  const double ETA[3] = {GB_PRISM_T1, GB_PRISM_T2, GB_PRISM_T1};

  // zeta-only quantities
  vec3<T> j1[2], j2[2], c3[2];
  T a11[2], a12[2], a22[2], c33[2];
#pragma unroll
  for (int z = 0; z < 2; z++) {
    const T zeta(z == 0 ? -GB_PRISM_G2 : GB_PRISM_G2);
    j1[z] = q_fma(zeta, D1, M1);
    j2[z] = q_fma(zeta, D2, M2);
    c3[z] = q_cross(j1[z], j2[z]);
    a11[z] = q_dot(j1[z], j1[z]);
    a12[z] = q_dot(j1[z], j2[z]);
    a22[z] = q_dot(j2[z], j2[z]);
    c33[z] = t_fma(a11[z], a22[z], -a12[z] * a12[z]);
  }
  // (xi, eta)-only quantities
  vec3<T> j3[3];
  T a33[3];
#pragma unroll
  for (int p = 0; p < 3; p++) {
    j3[p] = q_fma(T(ETA[p]), D2, q_fma(T(XI[p]), D1, C0));
    a33[p] = q_dot(j3[p], j3[p]);
  }
  T adet[6], a13[6], a23[6];
#pragma unroll
  for (int q = 0; q < 6; q++) {
    const int z = q / 3, p = q % 3;
    adet[q] = t_abs(q_dot(j3[p], c3[z]));
    a13[q] = q_dot(j1[z], j3[p]);
    a23[q] = q_dot(j2[z], j3[p]);
  }
  T inv[6];
  prism_recip6(adet, inv);

  // quadrature sums of the scaled adjugate products
  const T kw = T(0.5 * wq) * kk;
  T S11[2], S12[2], S22[2];  // sum over triangle points of s c1.c1, s c1.c2, s c2.c2
  T M[2][2][3];              // M[z][a][t'] = sum_p L_t'(p) s c_a.c3   (a: c1, c2)
  T F[3];                    // F[p] = sum_z s c3.c3
  T RA[2][3];                // RA[z][t] = sum_p L_t(p) |det'|
#pragma unroll
  for (int p = 0; p < 3; p++) F[p] = T(0.0);
#pragma unroll
  for (int z = 0; z < 2; z++) {
    S11[z] = S12[z] = S22[z] = T(0.0);
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
      for (int t = 0; t < 3; t++) M[z][a][t] = T(0.0);
#pragma unroll
    for (int t = 0; t < 3; t++) RA[z][t] = T(0.0);
#pragma unroll
    for (int p = 0; p < 3; p++) {
      const int q = 3 * z + p;
      const double L[3] = {1.0 - XI[p] - ETA[p], XI[p], ETA[p]};
      const T s = kw * inv[q];
      // Binet-Cauchy: c1 = j2 x j3, c2 = j3 x j1, c3 = j1 x j2
      const T c11 = t_fma(a22[z], a33[p], -a23[q] * a23[q]);
      const T c12 = t_fma(a23[q], a13[q], -a12[z] * a33[p]);
      const T c22 = t_fma(a33[p], a11[z], -a13[q] * a13[q]);
      const T c13 = t_fma(a12[z], a23[q], -a22[z] * a13[q]);
      const T c23 = t_fma(a13[q], a12[z], -a23[q] * a11[z]);
      S11[z] = t_fma(s, c11, S11[z]);
      S12[z] = t_fma(s, c12, S12[z]);
      S22[z] = t_fma(s, c22, S22[z]);
      const T g13 = s * c13, g23 = s * c23;
#pragma unroll
      for (int t = 0; t < 3; t++) {
        M[z][0][t] = t_fma(T(L[t]), g13, M[z][0][t]);
        M[z][1][t] = t_fma(T(L[t]), g23, M[z][1][t]);
        RA[z][t] = t_fma(T(L[t]), adet[q], RA[z][t]);
      }
      F[p] = t_fma(s, c33[z], F[p]);
    }
  }

  // A[ss'][tt'] = sum_z h_s h_s' E_tt'(z), E = sums of s e_t.e_t' with
  // e = (-(c1+c2), c1, c2); N[s][t][t'] = 1/2 sum_z h_s(z) M_tt'(z)
  T A[3][6];
  T N[2][3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 6; j++) A[i][j] = T(0.0);
#pragma unroll
  for (int s = 0; s < 2; s++)
#pragma unroll
    for (int t = 0; t < 3; t++)
#pragma unroll
      for (int u = 0; u < 3; u++) N[s][t][u] = T(0.0);
#pragma unroll
  for (int z = 0; z < 2; z++) {
    const double zeta = z == 0 ? -GB_PRISM_G2 : GB_PRISM_G2;
    const double h[2] = {(1.0 - zeta) / 2.0, (1.0 + zeta) / 2.0};
    // packed symmetric 3x3: (00, 01, 02, 11, 12, 22)
    const T e01 = -(S11[z] + S12[z]), e02 = -(S12[z] + S22[z]);
    const T E[6] = {-(e01 + e02), e01, e02, S11[z], S12[z], S22[z]};
    const double H[3] = {h[0] * h[0], h[0] * h[1], h[1] * h[1]};
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 6; j++) A[i][j] = t_fma(T(H[i]), E[j], A[i][j]);
#pragma unroll
    for (int u = 0; u < 3; u++) {
      const T m1t = M[z][0][u], m2t = M[z][1][u];
      const T mt[3] = {-(m1t + m2t), m1t, m2t};
#pragma unroll
      for (int s = 0; s < 2; s++)
#pragma unroll
        for (int t = 0; t < 3; t++) N[s][t][u] = t_fma(T(0.5 * h[s]), mt[t], N[s][t][u]);
    }
  }
  // fold P_tt' = 1/4 sum_p L_t L_t' F(p) into A with the sign sigma_s sigma_s'
  // (+ for ss' = 00 and 11, - for 01)
  {
    const int tt[6][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2}};
#pragma unroll
    for (int j = 0; j < 6; j++) {
      T acc = T(0.0);
#pragma unroll
      for (int p = 0; p < 3; p++) {
        const double L[3] = {1.0 - XI[p] - ETA[p], XI[p], ETA[p]};
        acc = t_fma(T(0.25 * L[tt[j][0]] * L[tt[j][1]]), F[p], acc);
      }
      A[0][j] += acc;
      A[1][j] -= acc;
      A[2][j] += acc;
    }
  }
  // K entries: u = t + 3s, w = t' + 3s'
#pragma unroll
  for (int u = 0; u < 6; u++) {
#pragma unroll
    for (int w = u; w < 6; w++) {
      const int t = u % 3, s = u / 3, tp = w % 3, sp = w / 3;
      const int a = t < tp ? t : tp, b = t < tp ? tp : t;
      const int sym = a == 0 ? b : (a == 1 ? 2 + b : 5);  // packed 3x3 symmetric index
      const int ss = s + sp;                              // 0: 00, 1: 01, 2: 11
      T v = A[ss][sym];
      v = sp == 0 ? v - N[s][t][tp] : v + N[s][t][tp];
      v = s == 0 ? v - N[sp][tp][t] : v + N[sp][tp][t];
      K[packed_index(u, w)] = v;
    }
  }
  // R_{t,s} = f w sum_z h_s(z) sum_p L_t(p) |det|,  |det| = |det'| / 8
  const T fw = T(0.125 * wq) * f;
#pragma unroll
  for (int t = 0; t < 3; t++) {
    const double hlo0 = (1.0 + GB_PRISM_G2) / 2.0, hlo1 = (1.0 - GB_PRISM_G2) / 2.0;  // h_0 at z = 0, 1
    R[t] = fw * t_fma(T(hlo0), RA[0][t], T(hlo1) * RA[1][t]);
    R[t + 3] = fw * t_fma(T(hlo1), RA[0][t], T(hlo0) * RA[1][t]);
  }
}

GB_HD void prism_std_element(const v3 (&X)[6], double kk, double f, double (&K)[21], double (&R)[6]) {
  const v3 ea = v3_sub(X[1], X[0]), eb = v3_sub(X[4], X[3]);
  const v3 fa = v3_sub(X[2], X[0]), fb = v3_sub(X[5], X[3]);
  const v3 C0 = v3_sub(X[3], X[0]);
  prism_std_element_t<double>({ea.x, ea.y, ea.z}, {eb.x, eb.y, eb.z}, {fa.x, fa.y, fa.z}, {fb.x, fb.y, fb.z},
                              {C0.x, C0.y, C0.z}, kk, f, K, R);
}

}  // namespace gbfem
