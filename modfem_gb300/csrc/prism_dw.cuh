// Standard linear prism element in double-word arithmetic (float pairs on
// the FP32 pipe; the FP64 pipe only forms the 15 vertex differences).
//
// Same integrals as prism_std_element_t (apr_num_int_el of
// apd_std_lin/aps_std_lin_intf.c:1537-2880 with the 2 x 3 point prism rule of
// apr_set_quadr_3D, aps_std_util.c:1380-1438), reorganised for a compact
// instruction stream: a fully unrolled double-word element is several times
// the size of the FP64 one and stalls on instruction fetch, so the work runs
// in three short phases with per-thread shared-memory slots between them:
//
//  1. a loop over the two Gauss line points z (three triangle points p
//     unrolled): Jacobian inner products, Binet-Cauchy adjugate products,
//     one Newton-refined reciprocal per point; seven values per (z, p) go to
//     the slots: s c1.c1, s c1.c2, s c2.c2, s c1.c3, s c2.c3, |det'|, s c3.c3
//     (s = k w / (2 |det'|), J' = 2 J as in the FP64 form);
//  2. straight-line combination into A[ss'][tt'] and N[s][t][t'] using the
//     structure of the rule's weights: every triangle weight is
//     L_t(p) = 1/6 + 1/2 [p = p_t] (p_0 = 0, p_1 = 2, p_2 = 1), and the line
//     weights at z = 0, 1 are (h_0, h_1) = (alpha, beta), (beta, alpha), so
//     sums over z become sums and differences of the two points' values;
//  3. the caller's loop over the 21 packed entries K[u][w] = A +- N +- N
//     (prism_dw_entry, converted to double) and the 6 loads (prism_dw_load).
#pragma once

#include "dword.cuh"
#include "prism_std.cuh"

#if defined(__CUDACC__)
#include <vector_types.h>
#endif

namespace gbfem {

// one double word per slot: slot i of this thread at base[i * stride]
struct DwSlots {
  float2 *base;
  int stride;
  DW_HD dw get(int i) const {
    const float2 v = base[(size_t)i * stride];
    return dw(v.x, v.y);
  }
  DW_HD void put(int i, dw x) const {
    float2 v;
    v.x = x.h;
    v.y = x.l;
    base[(size_t)i * stride] = v;
  }
};

// Slots: phase 1 writes value f of point q = 3 z + p to slot 7 q + f; phase 2
// reuses them once read: A[ss][j] in 7 j + ss (the f = 0..2 slots), N (index
// n = 9 s + 3 t + t') in the f = 3, 4 slots for n < 12 and the f = 6 slots
// after, R[w] in 7 w + 5.
constexpr int kPrismDwSlots = 42;
DW_CX int dw_slot_a(int ss, int j) { return 7 * j + ss; }
DW_CX int dw_slot_n(int n) { return n < 12 ? 7 * (n >> 1) + 3 + (n & 1) : 7 * (n - 12) + 6; }
DW_CX int dw_slot_r(int w) { return 7 * w + 5; }

DW_HD dw dw_scale2(dw x, float s) { return dw(f_mul(x.h, s), f_mul(x.l, s)); }  // s a power of two

DW_HD vec3<dw> dw_diff3(v3 a, v3 b) {
  return {dw_from_double(a.x - b.x), dw_from_double(a.y - b.y), dw_from_double(a.z - b.z)};
}

DW_HD dw dw_dot(const vec3<dw> &a, const vec3<dw> &b) { return dw_dot3(a.x, b.x, a.y, b.y, a.z, b.z); }
DW_HD vec3<dw> dw_cross(const vec3<dw> &a, const vec3<dw> &b) {
  return {dw_fms(a.y, b.z, a.z, b.y), dw_fms(a.z, b.x, a.x, b.z), dw_fms(a.x, b.y, a.y, b.x)};
}

// phase 1 for Gauss line point z (runtime 0 or 1)
DW_HD void prism_dw_phase1(int z, vec3<dw> M1, vec3<dw> D1, vec3<dw> M2, vec3<dw> D2, const vec3<dw> (&j3)[3],
                           const dw (&a33)[3], dw kw, const DwSlots &sl) {
  const dw zeta = z == 0 ? dw(-GB_PRISM_G2) : dw(GB_PRISM_G2);
  const vec3<dw> j1 = q_fma(zeta, D1, M1), j2 = q_fma(zeta, D2, M2);
  const vec3<dw> c3 = dw_cross(j1, j2);
  const dw a11 = dw_dot(j1, j1), a12 = dw_dot(j1, j2), a22 = dw_dot(j2, j2);
  const dw c33 = dw_fms(a11, a22, a12, a12);
#pragma unroll
  for (int p = 0; p < 3; p++) {
    const dw adet = t_abs(dw_dot(j3[p], c3));
    const dw a13 = dw_dot(j1, j3[p]), a23 = dw_dot(j2, j3[p]);
    const dw s = kw * dw_recip(adet);
    // Binet-Cauchy: c1 = j2 x j3, c2 = j3 x j1, c3 = j1 x j2
    const dw c11 = dw_fms(a22, a33[p], a23, a23);
    const dw c12 = dw_fms(a23, a13, a12, a33[p]);
    const dw c22 = dw_fms(a33[p], a11, a13, a13);
    const dw c13 = dw_fms(a12, a23, a22, a13);
    const dw c23 = dw_fms(a13, a12, a23, a11);
    const int o = 7 * (3 * z + p);
    sl.put(o + 0, s * c11);
    sl.put(o + 1, s * c12);
    sl.put(o + 2, s * c22);
    sl.put(o + 3, s * c13);
    sl.put(o + 4, s * c23);
    sl.put(o + 5, adet);
    sl.put(o + 6, s * c33);
  }
}

// phase 2: A, N and R into the slots (each slot written after its phase-1
// value was read)
DW_HD void prism_dw_phase2(const DwSlots &sl, dw fw) {
  constexpr double AL = (1.0 + GB_PRISM_G2) / 2.0, BE = (1.0 - GB_PRISM_G2) / 2.0;  // h_0 at z = 0, 1
  constexpr double CP = (AL * AL + BE * BE) / 2.0, CQ = (AL * AL - BE * BE) / 2.0, CA1 = AL * BE;
  constexpr double NQ = 0.25 * (AL - BE);
  const int pt[3] = {0, 2, 1};  // p_t: the point where L_t = 2/3
  auto at = [&](int z, int p, int f) { return sl.get(7 * (3 * z + p) + f); };
  // E_j(z) over z: sums P and differences Q of S11, S12, S22
  dw SP[3], SQ[3];
#pragma unroll
  for (int f = 0; f < 3; f++) {
    const dw s0 = at(0, 0, f) + at(0, 1, f) + at(0, 2, f);
    const dw s1 = at(1, 0, f) + at(1, 1, f) + at(1, 2, f);
    SP[f] = s0 + s1;
    SQ[f] = s0 - s1;
  }
  // E = (-(e01 + e02), e01, e02, S11, S12, S22), e01 = -(S11 + S12), e02 = -(S12 + S22)
  auto E6 = [](const dw (&S)[3], dw (&E)[6]) {
    const dw e01 = -(S[0] + S[1]), e02 = -(S[1] + S[2]);
    E[0] = -(e01 + e02);
    E[1] = e01;
    E[2] = e02;
    E[3] = S[0];
    E[4] = S[1];
    E[5] = S[2];
  };
  dw EP[6], EQ[6];
  E6(SP, EP);
  E6(SQ, EQ);
  // P_tt' = 1/4 sum_p L_t L_t' F(p), F(p) = s c3.c3 summed over z
  dw F[3];
#pragma unroll
  for (int p = 0; p < 3; p++) F[p] = at(0, p, 6) + at(1, p, 6);
  const dw Fb = dw(0.25 * GB_PRISM_T1 * GB_PRISM_T1) * (F[0] + F[1] + F[2]);
  const int tt[6][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2}};
#pragma unroll
  for (int j = 0; j < 6; j++) {
    const int a = tt[j][0], b = tt[j][1];
    const dw acc = a == b ? t_fma(dw(0.25 * GB_PRISM_T1 + 0.0625), F[pt[a]], Fb)
                          : t_fma(dw(0.125 * GB_PRISM_T1), F[pt[a]] + F[pt[b]], Fb);
    const dw cp = dw(CP) * EP[j], cq = dw(CQ) * EQ[j];
    sl.put(dw_slot_a(0, j), cp + cq + acc);
    sl.put(dw_slot_a(1, j), dw(CA1) * EP[j] - acc);
    sl.put(dw_slot_a(2, j), (cp - cq) + acc);
  }
  // N[s][t][u] = 1/2 sum_z h_s(z) mt_t(z, u), mt = (-(m1 + m2), m1, m2),
  // m_a(z, u) = sum_p L_u(p) s c_a.c3 = 1/6 sum_p g_a(z, p) + 1/2 g_a(z, p_u)
  dw PM[3][3], QM[3][3];  // [t][u]
#pragma unroll
  for (int a = 0; a < 2; a++) {
    dw GP[3], GQ[3];
#pragma unroll
    for (int p = 0; p < 3; p++) {
      const dw g0 = at(0, p, 3 + a), g1 = at(1, p, 3 + a);
      GP[p] = g0 + g1;
      GQ[p] = g0 - g1;
    }
    const dw sp = dw(GB_PRISM_T1) * (GP[0] + GP[1] + GP[2]);
    const dw sq = dw(GB_PRISM_T1) * (GQ[0] + GQ[1] + GQ[2]);
#pragma unroll
    for (int u = 0; u < 3; u++) {
      PM[1 + a][u] = sp + dw_scale2(GP[pt[u]], 0.5f);
      QM[1 + a][u] = sq + dw_scale2(GQ[pt[u]], 0.5f);
    }
  }
#pragma unroll
  for (int u = 0; u < 3; u++) {
    PM[0][u] = -(PM[1][u] + PM[2][u]);
    QM[0][u] = -(QM[1][u] + QM[2][u]);
  }
#pragma unroll
  for (int t = 0; t < 3; t++)
#pragma unroll
    for (int u = 0; u < 3; u++) {
      const dw p = dw_scale2(PM[t][u], 0.25f), q = dw(NQ) * QM[t][u];  // (alpha + beta) = 1
      sl.put(dw_slot_n(3 * t + u), p + q);
      sl.put(dw_slot_n(9 + 3 * t + u), p - q);
    }
  // R_{t,s} = f w sum_z h_s(z) sum_p L_t(p) |det|, |det| = |det'| / 8
  dw AP[3], AQ[3];
#pragma unroll
  for (int p = 0; p < 3; p++) {
    const dw d0 = at(0, p, 5), d1 = at(1, p, 5);
    AP[p] = d0 + d1;
    AQ[p] = d0 - d1;
  }
  const dw rp = dw(GB_PRISM_T1) * (AP[0] + AP[1] + AP[2]), rq = dw(GB_PRISM_T1) * (AQ[0] + AQ[1] + AQ[2]);
#pragma unroll
  for (int t = 0; t < 3; t++) {
    const dw P = dw_scale2(rp + dw_scale2(AP[pt[t]], 0.5f), 0.5f);  // (alpha + beta) / 2
    const dw Q = dw(GB_PRISM_G2 / 2.0) * (rq + dw_scale2(AQ[pt[t]], 0.5f));
    sl.put(dw_slot_r(t), fw * (P + Q));
    sl.put(dw_slot_r(t + 3), fw * (P - Q));
  }
}

// Phases 1 and 2 of one element: afterwards the slots hold A, N and R, read
// by prism_dw_entry / prism_dw_load.
DW_HD void prism_std_element_dw(const v3 (&X)[6], double kk, double f, const DwSlots &sl) {
  const vec3<dw> ea = dw_diff3(X[1], X[0]), eb = dw_diff3(X[4], X[3]);
  const vec3<dw> fa = dw_diff3(X[2], X[0]), fb = dw_diff3(X[5], X[3]);
  const vec3<dw> C0 = dw_diff3(X[3], X[0]);
  const vec3<dw> M1 = q_add(ea, eb), D1 = q_sub(eb, ea);
  const vec3<dw> M2 = q_add(fa, fb), D2 = q_sub(fb, fa);
  // j3 at the triangle points: C0 + (D1 + D2)/6, then + D2/2 (p = 1), + D1/2 (p = 2)
  vec3<dw> j3[3];
  const dw sixth = dw(GB_PRISM_T1);
  j3[0] = {t_fma(sixth, D1.x + D2.x, C0.x), t_fma(sixth, D1.y + D2.y, C0.y), t_fma(sixth, D1.z + D2.z, C0.z)};
  j3[1] = {j3[0].x + dw_scale2(D2.x, 0.5f), j3[0].y + dw_scale2(D2.y, 0.5f), j3[0].z + dw_scale2(D2.z, 0.5f)};
  j3[2] = {j3[0].x + dw_scale2(D1.x, 0.5f), j3[0].y + dw_scale2(D1.y, 0.5f), j3[0].z + dw_scale2(D1.z, 0.5f)};
  dw a33[3];
#pragma unroll
  for (int p = 0; p < 3; p++) a33[p] = dw_dot(j3[p], j3[p]);
  const double wq = 0.5 * GB_PRISM_TW * 1.0;
  const dw kw = dw(0.5 * wq) * dw_from_double(kk);
#pragma unroll 1
  for (int z = 0; z < 2; z++) prism_dw_phase1(z, M1, D1, M2, D2, j3, a33, kw, sl);
  prism_dw_phase2(sl, dw(0.125 * wq) * dw_from_double(f));
}

// The 21 packed entries K[u][w] = A[s+s'][tt'] +- N[s][t][t'] +- N[s'][t'][t]
// (u = t + 3 s <= w = t' + 3 s'), two codes each:
//   c[2k]     table offsets w + 6u and u + 6w (bits 0-7, 8-15), slot of A
//             (16-23), u == w (24);
//   c[2k + 1] slots of the two N terms (0-7, 8-15), their signs (16, 17:
//             set for minus, i.e. s' = 0 and s = 0).
struct DwPairCodes {
  int c[42];
};
DW_CX DwPairCodes dw_pair_codes() {
  DwPairCodes r{};
  int k = 0;
  for (int u = 0; u < 6; u++)
    for (int w = u; w < 6; w++, k++) {
      const int t = u % 3, s = u / 3, tp = w % 3, sp = w / 3;
      const int a = t < tp ? t : tp, b = t < tp ? tp : t;
      const int sym = a == 0 ? b : (a == 1 ? 2 + b : 5);  // packed 3x3 symmetric index
      r.c[2 * k] = (w + 6 * u) | (u + 6 * w) << 8 | dw_slot_a(s + sp, sym) << 16 | (u == w ? 1 : 0) << 24;
      r.c[2 * k + 1] = dw_slot_n(9 * s + 3 * t + tp) | dw_slot_n(9 * sp + 3 * tp + t) << 8 | (sp == 0 ? 1 : 0) << 16 |
                       (s == 0 ? 1 : 0) << 17;
    }
  return r;
}

DW_HD dw dw_flip(dw x, unsigned sgn) { return dw(f_from_bits(f_bits(x.h) ^ sgn), f_from_bits(f_bits(x.l) ^ sgn)); }

// entry of codes (c0, c1) as a double
DW_HD double prism_dw_entry(const DwSlots &sl, int c0, int c1) {
  const dw v = sl.get((c0 >> 16) & 0xFF);
  const dw n1 = dw_flip(sl.get(c1 & 0xFF), (unsigned)(c1 >> 16 & 1) << 31);
  const dw n2 = dw_flip(sl.get((c1 >> 8) & 0xFF), (unsigned)(c1 >> 17 & 1) << 31);
  return dw_to_double((v + n1) + n2);
}

// R[w] as a double
DW_HD double prism_dw_load(const DwSlots &sl, int w) { return dw_to_double(sl.get(dw_slot_r(w))); }

}  // namespace gbfem
