// Integrate + scatter kernels for standard linear prisms and tetrahedra (FP64).
//
// One thread integrates one element (or one boundary face) and adds its local
// stiffness matrix and load vector straight into the CRS values / rhs through
// the element's assembly table, so element matrices never reach HBM.  On
// GB300 the FP64 pipe (about 1.2 TFLOP/s, 1/58 of the FP32 rate) bounds
// these kernels, not HBM, so the arithmetic is arranged to minimise FP64
// instructions; the isotropic prism math lives in prism_std.cuh (see there).
// The full-tensor variant below integrates per quadrature point:
//  * the Jacobian of the linear prism splits into ζ-only columns
//    (dx/dξ = m1 + ζ d1, dx/dη = m2 + ζ d2) and a (ξ,η)-only column
//    (dx/dζ = c0 + ξ d1 + η d2);
//  * gradients use the adjugate rows (no 3x3 inverse), det and the weight
//    fold into one scale w/|det| applied once per shape function.
// Both equal the reference's apr_num_int_el (apd_std_lin/
// aps_std_lin_intf.c:1537-2880 with apr_elem_calc_3D_prism, aps_std_util.c:
// 520-820) up to rounding.

#include "gbfem_internal.h"
#include "prism_dw.cuh"
#include "prism_std.cuh"

namespace gbfem {

struct d3 {
  double x, y, z;
};
__device__ __forceinline__ d3 operator+(d3 a, d3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ d3 operator-(d3 a, d3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ d3 operator*(double s, d3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ d3 fma3(double s, d3 a, d3 b) {
  return {fma(s, a.x, b.x), fma(s, a.y, b.y), fma(s, a.z, b.z)};
}
__device__ __forceinline__ d3 cross(d3 a, d3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ double dot(d3 a, d3 b) { return fma(a.x, b.x, fma(a.y, b.y, a.z * b.z)); }

__device__ __forceinline__ d3 load_node(const double *__restrict__ xyz, int n) {
  const double *p = xyz + 3 * (size_t)n;
  return {__ldg(p), __ldg(p + 1), __ldg(p + 2)};
}

// Quadrature of apr_set_quadr_3D for the std prism (aps_std_util.c:1380-1438)
// with the reference's tabulated constants (aps_gauss_util_std.c, Xg_1d[1],
// Xg_2d[1], Wg_2d[1]): two Gauss line points x three triangle points,
// weight 0.5 * (1/3) * 1.
#define GB_G2 0.577350269189626
#define GB_T1 0.166666666666667
#define GB_T2 0.666666666666667
#define GB_TW 0.333333333333333

template <bool ATOMIC>
__device__ __forceinline__ void add_val(double *__restrict__ a, int i, double v) {
  if (ATOMIC)
    atomicAdd(a + i, v);
  else
    a[i] += v;
}

// Adds one symmetric 6x6 local matrix (upper triangle K[u][w], u<=w, packed
// row by row) and a load vector through an assembly table (table[w + 6u] is
// the CRS position of row w, column u; table[36 + w] the rhs row).
template <bool ATOMIC>
__device__ __forceinline__ void scatter6(const int *__restrict__ tab, const double (&K)[21],
                                         const double (&R)[6], double *__restrict__ val,
                                         double *__restrict__ rhs, bool do_sm, bool do_rhs) {
  int t[42];
  const int2 *t2 = reinterpret_cast<const int2 *>(tab);
#pragma unroll
  for (int i = 0; i < 21; i++) {
    int2 v = __ldg(t2 + i);
    t[2 * i] = v.x;
    t[2 * i + 1] = v.y;
  }
  if (do_sm) {
    int k = 0;
#pragma unroll
    for (int u = 0; u < 6; u++)
#pragma unroll
      for (int w = u; w < 6; w++, k++) {
        add_val<ATOMIC>(val, t[w + 6 * u], K[k]);
        if (w != u) add_val<ATOMIC>(val, t[u + 6 * w], K[k]);
      }
  }
  if (do_rhs) {
#pragma unroll
    for (int w = 0; w < 6; w++) add_val<ATOMIC>(rhs, t[36 + w], R[w]);
  }
}

// Same with a full coefficient tensor A (a_ij multiplies d_i(test) d_j(trial));
// all 36 entries are integrated (A need not be symmetric).
__device__ __forceinline__ void prism_element_aniso(const d3 (&X)[6], const double *__restrict__ A,
                                                    double f, double (&K)[36], double (&R)[6]) {
  const d3 a0 = X[0], a1 = X[1], a2 = X[2], b0 = X[3], b1 = X[4], b2 = X[5];
  const d3 ea = a1 - a0, eb = b1 - b0, fa = a2 - a0, fb = b2 - b0;
  const d3 m1 = 0.5 * (ea + eb), d1 = 0.5 * (eb - ea);
  const d3 m2 = 0.5 * (fa + fb), d2 = 0.5 * (fb - fa);
  const d3 c0 = 0.5 * (b0 - a0);
  double a[9];
#pragma unroll
  for (int i = 0; i < 9; i++) a[i] = __ldg(A + i);
#pragma unroll
  for (int i = 0; i < 36; i++) K[i] = 0.0;
#pragma unroll
  for (int i = 0; i < 6; i++) R[i] = 0.0;
  const double wq = 0.5 * GB_TW * 1.0;
#pragma unroll
  for (int iz = 0; iz < 2; iz++) {
    const double zeta = iz == 0 ? -GB_G2 : GB_G2;
    const double hlo = (1.0 - zeta) / 2.0, hhi = (1.0 + zeta) / 2.0;
    const d3 j1 = fma3(zeta, d1, m1), j2 = fma3(zeta, d2, m2);
    const d3 c3 = cross(j1, j2);
#pragma unroll
    for (int it = 0; it < 3; it++) {
      const double xi = it == 2 ? GB_T2 : GB_T1;
      const double eta = it == 1 ? GB_T2 : GB_T1;
      const double L0 = 1.0 - xi - eta;
      const d3 j3 = fma3(eta, d2, fma3(xi, d1, c0));
      const d3 c1 = cross(j2, j3), c2 = cross(j3, j1);
      const double adet = fabs(dot(j1, c1));
      const double s = wq / adet;
      const double fv = f * wq * adet;
      const d3 e0 = -1.0 * (c1 + c2);
      const double hL0 = 0.5 * L0, hL1 = 0.5 * xi, hL2 = 0.5 * eta;
      d3 g[6];
      g[0] = fma3(hlo, e0, -hL0 * c3);
      g[1] = fma3(hlo, c1, -hL1 * c3);
      g[2] = fma3(hlo, c2, -hL2 * c3);
      g[3] = fma3(hhi, e0, hL0 * c3);
      g[4] = fma3(hhi, c1, hL1 * c3);
      g[5] = fma3(hhi, c2, hL2 * c3);
#pragma unroll
      for (int u = 0; u < 6; u++) {
        // p = s * A g_u  (row i of A dotted with the trial gradient)
        const d3 q = s * g[u];
        const d3 p = {fma(a[0], q.x, fma(a[1], q.y, a[2] * q.z)), fma(a[3], q.x, fma(a[4], q.y, a[5] * q.z)),
                      fma(a[6], q.x, fma(a[7], q.y, a[8] * q.z))};
#pragma unroll
        for (int w = 0; w < 6; w++)
          K[u * 6 + w] = fma(p.x, g[w].x, fma(p.y, g[w].y, fma(p.z, g[w].z, K[u * 6 + w])));
      }
      const double flo = fv * hlo, fhi = fv * hhi;
      R[0] = fma(flo, L0, R[0]);
      R[1] = fma(flo, xi, R[1]);
      R[2] = fma(flo, eta, R[2]);
      R[3] = fma(fhi, L0, R[3]);
      R[4] = fma(fhi, xi, R[4]);
      R[5] = fma(fhi, eta, R[5]);
    }
  }
}

// Elements: for i in [0, count): element e = ent_el ? ent_el[i] - el_base : i,
// table at tab + (ent_pos ? ent_pos[i] : 42*e).  Entity ids outside
// [0, nel) set *err and are skipped.
template <bool ATOMIC, bool ANISO, bool DWORD>
__global__ void __launch_bounds__(128) prism_elements_kernel(
    int count, const int *__restrict__ ent_el, int el_base, const int *__restrict__ ent_pos, int nel,
    const int *__restrict__ el_nodes, const double *__restrict__ xyz, const double *__restrict__ k_el,
    const double *__restrict__ D_el, double f, const int *__restrict__ tab, double *__restrict__ val,
    double *__restrict__ rhs, int do_sm, int do_rhs, int *__restrict__ err) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  int e = ent_el ? __ldg(ent_el + i) - el_base : i;
  if (e < 0 || e >= nel) {
    atomicExch(err, 1);
    return;
  }
  const int *tb = tab + (ent_pos ? (size_t)__ldg(ent_pos + i) : (size_t)42 * e);
  const int2 *n2 = reinterpret_cast<const int2 *>(el_nodes + 6 * (size_t)e);
  int2 na = __ldg(n2), nb = __ldg(n2 + 1), nc = __ldg(n2 + 2);
  d3 X[6] = {load_node(xyz, na.x), load_node(xyz, na.y), load_node(xyz, nb.x),
             load_node(xyz, nb.y), load_node(xyz, nc.x), load_node(xyz, nc.y)};
  double R[6];
  if (!ANISO) {
    double K[21];
    const v3 Xv[6] = {{X[0].x, X[0].y, X[0].z}, {X[1].x, X[1].y, X[1].z}, {X[2].x, X[2].y, X[2].z},
                      {X[3].x, X[3].y, X[3].z}, {X[4].x, X[4].y, X[4].z}, {X[5].x, X[5].y, X[5].z}};
    prism_std_element(Xv, k_el ? __ldg(k_el + e) : 1.0, f, K, R);
    scatter6<ATOMIC>(tb, K, R, val, rhs, do_sm, do_rhs);
  } else {
    double K[36];
    prism_element_aniso(X, D_el + 9 * (size_t)e, f, K, R);
    int t[42];
    const int2 *t2 = reinterpret_cast<const int2 *>(tb);
#pragma unroll
    for (int j = 0; j < 21; j++) {
      int2 v = __ldg(t2 + j);
      t[2 * j] = v.x;
      t[2 * j + 1] = v.y;
    }
    if (do_sm) {
#pragma unroll
      for (int u = 0; u < 6; u++)
#pragma unroll
        for (int w = 0; w < 6; w++) add_val<ATOMIC>(val, t[w + 6 * u], K[u * 6 + w]);
    }
    if (do_rhs) {
#pragma unroll
      for (int w = 0; w < 6; w++) add_val<ATOMIC>(rhs, t[36 + w], R[w]);
    }
  }
}

// Isotropic std prisms in double-word arithmetic (prism_dw.cuh): each thread
// keeps its intermediate values in kPrismDwSlots float2 slots of shared
// memory (thread-major stride, conflict-free 8-byte accesses) and scatters
// each entry as soon as it is formed.
constexpr int kDwThreads = 128;
__constant__ DwPairCodes kDwPairs = dw_pair_codes();
template <bool ATOMIC>
__global__ void __launch_bounds__(kDwThreads, 3) prism_elements_dw_kernel(
    int count, const int *__restrict__ ent_el, int el_base, const int *__restrict__ ent_pos, int nel,
    const int *__restrict__ el_nodes, const double *__restrict__ xyz, const double *__restrict__ k_el, double f,
    const int *__restrict__ tab, double *__restrict__ val, double *__restrict__ rhs, int do_sm, int do_rhs,
    int *__restrict__ err) {
  extern __shared__ float2 dw_slots[];
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  int e = ent_el ? __ldg(ent_el + i) - el_base : i;
  if (e < 0 || e >= nel) {
    atomicExch(err, 1);
    return;
  }
  const int *tb = tab + (ent_pos ? (size_t)__ldg(ent_pos + i) : (size_t)42 * e);
  // the table row (168 bytes) is read only after the element math: start
  // bringing its lines into L2 now
  asm volatile("prefetch.global.L2 [%0];" ::"l"(tb));
  asm volatile("prefetch.global.L2 [%0];" ::"l"(tb + 21));
  asm volatile("prefetch.global.L2 [%0];" ::"l"(tb + 41));
  const int2 *n2 = reinterpret_cast<const int2 *>(el_nodes + 6 * (size_t)e);
  const int2 na = __ldg(n2), nb = __ldg(n2 + 1), nc = __ldg(n2 + 2);
  const int nodes[6] = {na.x, na.y, nb.x, nb.y, nc.x, nc.y};
  v3 X[6];
#pragma unroll
  for (int j = 0; j < 6; j++) {
    const d3 x = load_node(xyz, nodes[j]);
    X[j] = {x.x, x.y, x.z};
  }
  const DwSlots sl{dw_slots + threadIdx.x, kDwThreads};
  prism_std_element_dw(X, k_el ? __ldg(k_el + e) : 1.0, f, sl);
  if (do_sm) {
    // the next entry's two table positions are loaded one iteration ahead
    int c0 = kDwPairs.c[0];
    int p1 = __ldg(tb + (c0 & 0xFF)), p2 = p1;
#pragma unroll 1
    for (int k = 0; k < 21; k++) {
      const int c1 = kDwPairs.c[2 * k + 1];
      const int c0n = k + 1 < 21 ? kDwPairs.c[2 * k + 2] : c0;
      const int q1 = __ldg(tb + (c0n & 0xFF)), q2 = __ldg(tb + ((c0n >> 8) & 0xFF));
      const double v = prism_dw_entry(sl, c0, c1);
      add_val<ATOMIC>(val, p1, v);
      if (!(c0 >> 24)) add_val<ATOMIC>(val, p2, v);
      c0 = c0n;
      p1 = q1;
      p2 = q2;
    }
  }
  if (do_rhs) {
    const int2 *r2 = reinterpret_cast<const int2 *>(tb + 36);
    const int2 ra = __ldg(r2), rb = __ldg(r2 + 1), rc = __ldg(r2 + 2);
    const int rows[6] = {ra.x, ra.y, rb.x, rb.y, rc.x, rc.y};
#pragma unroll
    for (int j = 0; j < 6; j++) add_val<ATOMIC>(rhs, rows[j], prism_dw_load(sl, j));
  }
}

// The penalty face integrals of one boundary face (side 0..4 of its prism,
// vertices X): K over the face's own vertices loc[0..nloc) (upper triangle
// of a 4x4 block packed row by row), R their load entries.
__device__ __forceinline__ void prism_face_local(const d3 (&X)[6], int side, double penalty, double g,
                                                 int (&loc)[4], int &nloc, double (&K)[10], double (&Rl)[4]) {
  const d3 a0 = X[0], a1 = X[1], a2 = X[2], b0 = X[3], b1 = X[4], b2 = X[5];
  const d3 ea = a1 - a0, eb = b1 - b0, fa_ = a2 - a0, fb = b2 - b0;
  const d3 m1 = 0.5 * (ea + eb), d1 = 0.5 * (eb - ea);
  const d3 m2 = 0.5 * (fa_ + fb), d2 = 0.5 * (fb - fa_);
  const d3 c0 = 0.5 * (b0 - a0);
  if (side == 0) { loc[0] = 0; loc[1] = 1; loc[2] = 2; nloc = 3; }
  else if (side == 1) { loc[0] = 3; loc[1] = 4; loc[2] = 5; nloc = 3; }
  else {
    int a = side - 2, b = (side - 1) % 3;
    loc[0] = a; loc[1] = b; loc[2] = a + 3; loc[3] = b + 3; nloc = 4;
  }
#pragma unroll
  for (int j = 0; j < 10; j++) K[j] = 0.0;
#pragma unroll
  for (int j = 0; j < 4; j++) Rl[j] = 0.0;
  const int nq = side <= 1 ? 3 : 4;
  for (int q = 0; q < nq; q++) {
    double xi, eta, zeta, w;
    if (side <= 1) {
      xi = q == 2 ? GB_T2 : GB_T1;
      eta = q == 1 ? GB_T2 : GB_T1;
      zeta = side == 0 ? -1.0 : 1.0;
      w = 0.5 * GB_TW;
    } else {
      const double s = (q >> 1) == 0 ? -GB_G2 : GB_G2, t = (q & 1) == 0 ? -GB_G2 : GB_G2;
      const double u = (s + 1.0) / 2.0;
      if (side == 2) { xi = u; eta = 0.0; }
      else if (side == 3) { xi = 1.0 - u; eta = u; }
      else { xi = 0.0; eta = 1.0 - u; }
      zeta = t;
      w = 0.5;
    }
    const d3 j1 = fma3(zeta, d1, m1), j2 = fma3(zeta, d2, m2);
    const d3 j3 = fma3(eta, d2, fma3(xi, d1, c0));
    d3 ds;
    if (side <= 1) ds = cross(j1, j2);
    else if (side == 2) ds = cross(j1, j3);
    else if (side == 3) ds = cross(j2 - j1, j3);
    else ds = cross(j3, j2);
    const double area = sqrt(dot(ds, ds)) * w;
    const double hlo = (1.0 - zeta) / 2.0, hhi = (1.0 + zeta) / 2.0, L0 = 1.0 - xi - eta;
    const double phi6[6] = {hlo * L0, hlo * xi, hlo * eta, hhi * L0, hhi * xi, hhi * eta};
    double ph[4];
    for (int j = 0; j < nloc; j++) ph[j] = phi6[loc[j]];
    const double pa = penalty * area;
    int k = 0;
    for (int a = 0; a < 4; a++)
      for (int b = a; b < 4; b++, k++)
        if (a < nloc && b < nloc) K[k] = fma(pa * ph[a], ph[b], K[k]);
    for (int a = 0; a < nloc; a++) Rl[a] = fma(pa * g, ph[a], Rl[a]);
  }
}

// Boundary penalty faces of the std weak form (pdd_conv_diff/weak_formulation/
// approx_std/pds_conv_diff_weakform_std.c:253-630):
// K_ij += penalty phi_i phi_j |dS| w, R_i += penalty g phi_i |dS| w, with the
// face rule of apr_set_quadr_2D (aps_std_util.c:1445-1500) and |dS| of the
// side cases of apr_elem_calc_3D_prism (aps_std_util.c:770-805).  Only the
// face's own vertices get non-zero entries.
template <bool ATOMIC>
__global__ void __launch_bounds__(128) prism_faces_kernel(
    int count, const int *__restrict__ ent_fa, int fa_base, const int *__restrict__ fa_map,
    int fa_map_len, const int *__restrict__ ent_pos, int nfa, const int *__restrict__ fa_el,
    const int *__restrict__ fa_side, const int *__restrict__ el_nodes, const double *__restrict__ xyz,
    double penalty, double g, const int *__restrict__ tab, double *__restrict__ val,
    double *__restrict__ rhs, int do_sm, int do_rhs, int *__restrict__ err) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  // face index: i, or ent_fa[i] (a face index when fa_map is null, else a
  // mesh face id translated through fa_map)
  int fa = i;
  if (ent_fa) {
    int id = __ldg(ent_fa + i) - fa_base;
    if (fa_map)
      fa = (id >= 0 && id < fa_map_len) ? __ldg(fa_map + id) : -1;
    else
      fa = id;
  }
  if (fa < 0 || fa >= nfa) {
    atomicExch(err, 2);
    return;
  }
  const int e = __ldg(fa_el + fa), side = __ldg(fa_side + fa);
  const int *tb = tab + (ent_pos ? (size_t)__ldg(ent_pos + i) : (size_t)42 * e);
  const int *nd = el_nodes + 6 * (size_t)e;
  d3 X[6];
#pragma unroll
  for (int j = 0; j < 6; j++) X[j] = load_node(xyz, __ldg(nd + j));
  int loc[4], nloc;
  double K[10], Rl[4];
  prism_face_local(X, side, penalty, g, loc, nloc, K, Rl);
  if (do_sm) {
    int k = 0;
    for (int a = 0; a < 4; a++)
      for (int b = a; b < 4; b++, k++) {
        if (a >= nloc || b >= nloc) continue;
        const int u = loc[a], wv = loc[b];
        add_val<ATOMIC>(val, __ldg(tb + wv + 6 * u), K[k]);
        if (a != b) add_val<ATOMIC>(val, __ldg(tb + u + 6 * wv), K[k]);
      }
  }
  if (do_rhs && g != 0.0) {
    for (int a = 0; a < nloc; a++) add_val<ATOMIC>(rhs, __ldg(tb + 36 + loc[a]), Rl[a]);
  }
}

// Std linear tetrahedra (apr_elem_calc_3D_tetra, aps_std_util.c:869-1130):
// constant Jacobian, volume |det|/6, 4-point order-2 rule with weights 1/4;
// tables hold 20 ints (16 values + 4 rhs).
template <bool ATOMIC>
__global__ void __launch_bounds__(128) tet_elements_kernel(
    int count, const int *__restrict__ ent_el, int el_base, const int *__restrict__ ent_pos, int nel,
    const int *__restrict__ el_nodes, const double *__restrict__ xyz, const double *__restrict__ k_el,
    double f, const int *__restrict__ tab, double *__restrict__ val, double *__restrict__ rhs,
    int do_sm, int do_rhs, int *__restrict__ err) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  int e = ent_el ? __ldg(ent_el + i) - el_base : i;
  if (e < 0 || e >= nel) {
    atomicExch(err, 1);
    return;
  }
  const int *tb = tab + (ent_pos ? (size_t)__ldg(ent_pos + i) : (size_t)20 * e);
  const int4 n4 = __ldg(reinterpret_cast<const int4 *>(el_nodes + 4 * (size_t)e));
  const d3 x0 = load_node(xyz, n4.x), x1 = load_node(xyz, n4.y), x2 = load_node(xyz, n4.z),
           x3 = load_node(xyz, n4.w);
  const d3 j1 = x1 - x0, j2 = x2 - x0, j3 = x3 - x0;
  const d3 c1 = cross(j2, j3), c2 = cross(j3, j1), c3 = cross(j1, j2);
  const double det = dot(j1, c1);
  const double adet = fabs(det * 0.16666666666666666666666666666667);  // |det|/6
  const double kk = k_el ? __ldg(k_el + e) : 1.0;
  // k * vol / det^2 with vol = |det|/6 summed over the 4 weights 1/4
  const double s = kk * adet / (det * det);
  d3 g[4] = {-1.0 * (c1 + c2 + c3), c1, c2, c3};
  if (do_sm) {
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const d3 p = s * g[u];
#pragma unroll
      for (int w = u; w < 4; w++) {
        const double v = dot(p, g[w]);
        add_val<ATOMIC>(val, __ldg(tb + w + 4 * u), v);
        if (w != u) add_val<ATOMIC>(val, __ldg(tb + u + 4 * w), v);
      }
    }
  }
  if (do_rhs) {
    const double a = 0.585410196624969, b = 0.138196601125011;
    // quadrature point order of apr_set_quadr_3D: (a,b,b), (b,b,a), (b,b,b), (b,a,b)
    const double P[4][3] = {{a, b, b}, {b, b, a}, {b, b, b}, {b, a, b}};
    double R[4] = {0, 0, 0, 0};
    const double fv = f * adet * 0.25;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      R[0] = fma(fv, 1.0 - P[q][0] - P[q][1] - P[q][2], R[0]);
      R[1] = fma(fv, P[q][0], R[1]);
      R[2] = fma(fv, P[q][1], R[2]);
      R[3] = fma(fv, P[q][2], R[3]);
    }
#pragma unroll
    for (int w = 0; w < 4; w++) add_val<ATOMIC>(rhs, __ldg(tb + 16 + w), R[w]);
  }
}

// The deterministic gather scatter: each element's local matrix and load
// vector are stored (ek[e*42 + a*6 + b] = row a, column b; ek[e*42 + 36 + a]
// = load entry a), then one thread a row adds its row's entries over the
// incident elements in element order, through the elements' tables.  Every
// CRS entry and rhs row has one writer and a fixed summation order, without
// the colouring the colour scatter needs.
template <bool ANISO>
__global__ void __launch_bounds__(128) prism_elements_store_kernel(
    int nel, const int *__restrict__ el_nodes, const double *__restrict__ xyz, const double *__restrict__ k_el,
    const double *__restrict__ D_el, double f, double *__restrict__ ek) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nel) return;
  const int2 *n2 = reinterpret_cast<const int2 *>(el_nodes + 6 * (size_t)e);
  const int2 na = __ldg(n2), nb = __ldg(n2 + 1), nc = __ldg(n2 + 2);
  d3 X[6] = {load_node(xyz, na.x), load_node(xyz, na.y), load_node(xyz, nb.x),
             load_node(xyz, nb.y), load_node(xyz, nc.x), load_node(xyz, nc.y)};
  double *o = ek + 42 * (size_t)e;
  double R[6];
  if (!ANISO) {
    double K[21];
    const v3 Xv[6] = {{X[0].x, X[0].y, X[0].z}, {X[1].x, X[1].y, X[1].z}, {X[2].x, X[2].y, X[2].z},
                      {X[3].x, X[3].y, X[3].z}, {X[4].x, X[4].y, X[4].z}, {X[5].x, X[5].y, X[5].z}};
    prism_std_element(Xv, k_el ? __ldg(k_el + e) : 1.0, f, K, R);
    int k = 0;
#pragma unroll
    for (int u = 0; u < 6; u++)
#pragma unroll
      for (int w = u; w < 6; w++, k++) {
        o[u * 6 + w] = K[k];
        if (w != u) o[w * 6 + u] = K[k];
      }
  } else {
    double K[36];
    prism_element_aniso(X, D_el + 9 * (size_t)e, f, K, R);
    // K[u * 6 + w] is (row w, column u)
#pragma unroll
    for (int a = 0; a < 6; a++)
#pragma unroll
      for (int b = 0; b < 6; b++) o[a * 6 + b] = K[b * 6 + a];
  }
#pragma unroll
  for (int a = 0; a < 6; a++) o[36 + a] = R[a];
}

__global__ void __launch_bounds__(128) std_gather_kernel(int nd, int nv, const int *__restrict__ inc_ptr,
                                                         const int *__restrict__ inc, const int *__restrict__ tab,
                                                         const double *__restrict__ ek, double *__restrict__ val,
                                                         double *__restrict__ rhs, int *__restrict__ err) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nd) return;
  const int tl = nv * nv + nv;
  double racc = 0.0;
  for (int k = __ldg(inc_ptr + r); k < __ldg(inc_ptr + r + 1); k++) {
    const int e = __ldg(inc + k);
    const int *tb = tab + (size_t)e * tl;
    int a = -1;
    for (int j = 0; j < nv; j++)
      if (__ldg(tb + nv * nv + j) == r) a = j;
    if (a < 0) {  // the incidence does not match the tables
      atomicExch(err, 9);
      return;
    }
    const double *ke = ek + (size_t)e * tl + a * nv;
    for (int b = 0; b < nv; b++) val[__ldg(tb + a + nv * b)] += __ldg(ke + b);
    racc += __ldg(ek + (size_t)e * tl + nv * nv + a);
  }
  rhs[r] += racc;
}

// Elements and boundary faces whose element has constrained (hanging)
// vertices: the local 6x6 matrix and load vector are rewritten as
// apr_get_stiff_mat_data does (apd_std_lin/aps_std_lin_intf.c:2978-3160)
// and scattered through the entity's assembly table of n x n + n entries,
// n the length of the expanded vertex list: in vertex order a real vertex
// stands for itself with coefficient 1, a constrained vertex for its 2
// (mid-edge) or 4 (mid-face) constraining vertices with coefficient 1/2 or
// 1/4; entry (a, b) = c_a c_b K[i(a)][i(b)], rhs entry a = c_a R[i(a)].
// con_node[v] is -1 for a vertex with a dof, else the index k of its
// constraining vertices con_par[4k..4k+3] (-1 padded).  These entities lie
// along refinement interfaces only: one thread an entity, FP64 arithmetic.
__device__ __forceinline__ int con_expand(const int (&nodes)[6], const int *__restrict__ con_node,
                                          const int *__restrict__ con_par, unsigned char (&src)[24],
                                          double (&cf)[24]) {
  int n = 0;
#pragma unroll
  for (int v = 0; v < 6; v++) {
    const int k = __ldg(con_node + nodes[v]);
    if (k < 0) {
      src[n] = (unsigned char)v;
      cf[n++] = 1.0;
    } else {
      const int cnt = __ldg(con_par + 4 * (size_t)k + 2) >= 0 ? 4 : 2;
      const double c = cnt == 2 ? 0.5 : 0.25;
      for (int j = 0; j < cnt; j++) {
        src[n] = (unsigned char)v;
        cf[n++] = c;
      }
    }
  }
  return n;
}

template <bool ANISO, bool FACE>
__global__ void __launch_bounds__(128) prism_constrained_kernel(
    int count, const int *__restrict__ ent_id, const int *__restrict__ ent_pos, int nel,
    const int *__restrict__ fa_map, int fa_map_len, int nfa, const int *__restrict__ fa_el,
    const int *__restrict__ fa_side, const int *__restrict__ el_nodes, const double *__restrict__ xyz,
    const double *__restrict__ k_el, const double *__restrict__ D_el, double f, double penalty, double g,
    const int *__restrict__ con_node, const int *__restrict__ con_par, const int *__restrict__ tab,
    double *__restrict__ val, double *__restrict__ rhs, int do_sm, int do_rhs, int *__restrict__ err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  int e, side = 0;
  if (FACE) {
    const int id = __ldg(ent_id + i);
    const int fa = (id >= 0 && id < fa_map_len) ? __ldg(fa_map + id) : -1;
    if (fa < 0 || fa >= nfa) {
      atomicExch(err, 2);
      return;
    }
    e = __ldg(fa_el + fa);
    side = __ldg(fa_side + fa);
  } else {
    e = __ldg(ent_id + i) - 1;
    if (e < 0 || e >= nel) {
      atomicExch(err, 1);
      return;
    }
  }
  int nodes[6];
  d3 X[6];
#pragma unroll
  for (int j = 0; j < 6; j++) {
    nodes[j] = __ldg(el_nodes + 6 * (size_t)e + j);
    X[j] = load_node(xyz, nodes[j]);
  }
  // the local matrix, K[u * 6 + w] = (row w, column u), and load vector
  double K[36], R[6];
  if (FACE) {
    int loc[4], nloc;
    double Kf[10], Rl[4];
    prism_face_local(X, side, penalty, g, loc, nloc, Kf, Rl);
#pragma unroll
    for (int j = 0; j < 36; j++) K[j] = 0.0;
#pragma unroll
    for (int j = 0; j < 6; j++) R[j] = 0.0;
    int k = 0;
    for (int a = 0; a < 4; a++)
      for (int b = a; b < 4; b++, k++) {
        if (a >= nloc || b >= nloc) continue;
        K[loc[a] * 6 + loc[b]] = Kf[k];
        K[loc[b] * 6 + loc[a]] = Kf[k];
      }
    for (int a = 0; a < nloc; a++) R[loc[a]] = Rl[a];
  } else if (ANISO) {
    prism_element_aniso(X, D_el + 9 * (size_t)e, f, K, R);
  } else {
    double Ks[21];
    const v3 Xv[6] = {{X[0].x, X[0].y, X[0].z}, {X[1].x, X[1].y, X[1].z}, {X[2].x, X[2].y, X[2].z},
                      {X[3].x, X[3].y, X[3].z}, {X[4].x, X[4].y, X[4].z}, {X[5].x, X[5].y, X[5].z}};
    prism_std_element(Xv, k_el ? __ldg(k_el + e) : 1.0, f, Ks, R);
    int k = 0;
#pragma unroll
    for (int u = 0; u < 6; u++)
#pragma unroll
      for (int w = u; w < 6; w++, k++) {
        K[u * 6 + w] = Ks[k];
        K[w * 6 + u] = Ks[k];
      }
  }
  unsigned char src[24];
  double cf[24];
  const int n = con_expand(nodes, con_node, con_par, src, cf);
  const int *tb = tab + __ldg(ent_pos + i);
  if (do_sm) {
    for (int b = 0; b < n; b++)
      for (int a = 0; a < n; a++) {
        const double kv = K[src[b] * 6 + src[a]];
        if (kv != 0.0) atomicAdd(val + __ldg(tb + a + n * b), cf[b] * cf[a] * kv);
      }
  }
  if (do_rhs) {
    for (int a = 0; a < n; a++) {
      const double rv = R[src[a]];
      if (rv != 0.0) atomicAdd(rhs + __ldg(tb + n * n + a), cf[a] * rv);
    }
  }
}

// ---------------------------------------------------------------------------
// host-side launchers
// ---------------------------------------------------------------------------
static inline unsigned nblk(long long n, int t) { return (unsigned)((n + t - 1) / t); }

int launch_prism_elements(cudaStream_t st, bool atomic, bool aniso, int count, const int *ent_el,
                          int el_base, const int *ent_pos, int nel, const int *el_nodes,
                          const double *xyz, const double *k_el, const double *D_el, double f,
                          const int *tab, double *val, double *rhs, int do_sm, int do_rhs, int *err,
                          bool dword) {
  if (count <= 0) return 0;
  const int T = 128;
#define GB_LAUNCH(A, B, W)                                                                        \
  prism_elements_kernel<A, B, W><<<nblk(count, T), T, 0, st>>>(count, ent_el, el_base, ent_pos, nel, \
                                                               el_nodes, xyz, k_el, D_el, f, tab,   \
                                                               val, rhs, do_sm, do_rhs, err)
  if (aniso) {
    if (atomic) GB_LAUNCH(true, true, false);
    else GB_LAUNCH(false, true, false);
  } else if (dword) {
    const size_t sm = (size_t)kPrismDwSlots * kDwThreads * sizeof(float2);
    if (atomic)
      prism_elements_dw_kernel<true><<<nblk(count, kDwThreads), kDwThreads, sm, st>>>(
          count, ent_el, el_base, ent_pos, nel, el_nodes, xyz, k_el, f, tab, val, rhs, do_sm, do_rhs, err);
    else
      prism_elements_dw_kernel<false><<<nblk(count, kDwThreads), kDwThreads, sm, st>>>(
          count, ent_el, el_base, ent_pos, nel, el_nodes, xyz, k_el, f, tab, val, rhs, do_sm, do_rhs, err);
  } else {
    if (atomic) GB_LAUNCH(true, false, false);
    else GB_LAUNCH(false, false, false);
  }
#undef GB_LAUNCH
  GB_CUDA(cudaGetLastError());
  return 1;
}

int launch_prism_faces(cudaStream_t st, bool atomic, int count, const int *ent_fa, int fa_base,
                       const int *fa_map, int fa_map_len, const int *ent_pos, int nfa,
                       const int *fa_el, const int *fa_side, const int *el_nodes,
                       const double *xyz, double penalty, double g, const int *tab, double *val,
                       double *rhs, int do_sm, int do_rhs, int *err) {
  if (count <= 0) return 0;
  const int T = 128;
  if (atomic)
    prism_faces_kernel<true><<<nblk(count, T), T, 0, st>>>(count, ent_fa, fa_base, fa_map, fa_map_len,
                                                           ent_pos, nfa, fa_el, fa_side, el_nodes, xyz,
                                                           penalty, g, tab, val, rhs, do_sm, do_rhs, err);
  else
    prism_faces_kernel<false><<<nblk(count, T), T, 0, st>>>(count, ent_fa, fa_base, fa_map, fa_map_len,
                                                            ent_pos, nfa, fa_el, fa_side, el_nodes, xyz,
                                                            penalty, g, tab, val, rhs, do_sm, do_rhs, err);
  GB_CUDA(cudaGetLastError());
  return 1;
}

int launch_std_gather(cudaStream_t st, bool aniso, int nel, int nd, const int *el_nodes, const double *xyz,
                      const double *k_el, const double *D_el, double f, const int *inc_ptr, const int *inc,
                      const int *tab, double *ek, double *val, double *rhs, int *err) {
  if (nel <= 0) return 0;
  const int T = 128;
  if (aniso)
    prism_elements_store_kernel<true><<<nblk(nel, T), T, 0, st>>>(nel, el_nodes, xyz, k_el, D_el, f, ek);
  else
    prism_elements_store_kernel<false><<<nblk(nel, T), T, 0, st>>>(nel, el_nodes, xyz, k_el, D_el, f, ek);
  std_gather_kernel<<<nblk(nd, T), T, 0, st>>>(nd, 6, inc_ptr, inc, tab, ek, val, rhs, err);
  GB_CUDA(cudaGetLastError());
  return 2;
}

int launch_prism_constrained(cudaStream_t st, bool faces, bool aniso, int count, const int *ent_id,
                             const int *ent_pos, int nel, const int *fa_map, int fa_map_len, int nfa,
                             const int *fa_el, const int *fa_side, const int *el_nodes, const double *xyz,
                             const double *k_el, const double *D_el, double f, double penalty, double g,
                             const int *con_node, const int *con_par, const int *tab, double *val, double *rhs,
                             int do_sm, int do_rhs, int *err) {
  if (count <= 0) return 0;
  const int T = 128;
#define GB_LAUNCH(A, F)                                                                                         \
  prism_constrained_kernel<A, F><<<nblk(count, T), T, 0, st>>>(count, ent_id, ent_pos, nel, fa_map, fa_map_len, \
                                                              nfa, fa_el, fa_side, el_nodes, xyz, k_el, D_el, f, \
                                                              penalty, g, con_node, con_par, tab, val, rhs,      \
                                                              do_sm, do_rhs, err)
  if (faces) GB_LAUNCH(false, true);
  else if (aniso) GB_LAUNCH(true, false);
  else GB_LAUNCH(false, false);
#undef GB_LAUNCH
  GB_CUDA(cudaGetLastError());
  return 1;
}

int launch_tet_elements(cudaStream_t st, bool atomic, int count, const int *ent_el, int el_base,
                        const int *ent_pos, int nel, const int *el_nodes, const double *xyz,
                        const double *k_el, double f, const int *tab, double *val, double *rhs,
                        int do_sm, int do_rhs, int *err) {
  if (count <= 0) return 0;
  const int T = 128;
  if (atomic)
    tet_elements_kernel<true><<<nblk(count, T), T, 0, st>>>(count, ent_el, el_base, ent_pos, nel, el_nodes,
                                                            xyz, k_el, f, tab, val, rhs, do_sm, do_rhs, err);
  else
    tet_elements_kernel<false><<<nblk(count, T), T, 0, st>>>(count, ent_el, el_base, ent_pos, nel, el_nodes,
                                                             xyz, k_el, f, tab, val, rhs, do_sm, do_rhs, err);
  GB_CUDA(cudaGetLastError());
  return 1;
}

}  // namespace gbfem
