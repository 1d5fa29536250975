// Volume integral of one DG tensor-basis prism of degree P (FP64), shared by
// the per-degree kernel and the persistent mixed kernel.
//
// Reference: apr_num_int_el of apd_dg_prism (aps_dg_prism_intf.c:1239-1728):
// K_uw = sum_q vol_q sum_ij a_ij d_i phi_w d_j phi_u, R_w = sum_q vol_q f phi_w.
// With the adjugate rows c_a of the Jacobian every point contributes
// D_q^T G_q D_q (D_q: 3 x ns reference derivatives, G_q = (w_q/|det|) C^T A C,
// 6 entries for symmetric A).  A group of THR threads (tid = 0..THR-1) of the
// calling CTA integrates one element: it has written the vertex coordinates to
// sX[18] and the tensor to sA[9] (shared memory); the body synchronises the
// whole CTA before reading them, so every group of the CTA runs the same body
// (same P, THR, QC) the same number of times; a group without an element
// passes write = false and computes on whatever sX/sA hold.
#pragma once

#include "dword.cuh"
#include "prism_std.cuh"

namespace gbfem {

template <int P, int THR, int QC>
struct DgDims {
  static constexpr int NS = P == 1 ? 6 : P == 2 ? 18 : P == 3 ? 40 : 75;
  static constexpr int NQ = P == 1 ? 6 : P == 2 ? 18 : P == 3 ? 48 : 80;
  static constexpr int THREADS = THR;
  static constexpr int QCHUNK = QC;
  static constexpr int NSYM = NS * (NS + 1) / 2;
  static constexpr int PER_THREAD = (NSYM + THREADS - 1) / THREADS;
};

// Geometric factors G_q, V_q at the points and the load vector (both forms)
template <int P, int THR, int QC>
__device__ __forceinline__ void dg_volume_points(const double *sX, const double *sA, double f,
                                                 const double *__restrict__ PHItab,
                                                 const double *__restrict__ QPtab, double *rhs_out,
                                                 double (*sG)[6], double *sV, int tid, bool write) {
  using Dm = DgDims<P, THR, QC>;
  constexpr int NS = Dm::NS, NQ = Dm::NQ, DG_THREADS = Dm::THREADS;
  __syncthreads();
  // geometric factors at the points
  for (int q = tid; q < NQ; q += DG_THREADS) {
    const double xi = QPtab[4 * q], eta = QPtab[4 * q + 1], zeta = QPtab[4 * q + 2], w = QPtab[4 * q + 3];
    const double lo = (1.0 - zeta) / 2.0, hi = (1.0 + zeta) / 2.0, l0 = 1.0 - xi - eta;
    // d x / d(xi, eta, zeta) of the linear prism (apr_elem_calc_3D geometry)
    const double dx[6] = {-lo, lo, 0.0, -hi, hi, 0.0};
    const double dy[6] = {-lo, 0.0, lo, -hi, 0.0, hi};
    const double dz[6] = {-0.5 * l0, -0.5 * xi, -0.5 * eta, 0.5 * l0, 0.5 * xi, 0.5 * eta};
    v3 j1 = {0, 0, 0}, j2 = {0, 0, 0}, j3 = {0, 0, 0};
#pragma unroll
    for (int i = 0; i < 6; i++) {
      const v3 x = {sX[3 * i], sX[3 * i + 1], sX[3 * i + 2]};
      j1 = v3_fma(dx[i], x, j1);
      j2 = v3_fma(dy[i], x, j2);
      j3 = v3_fma(dz[i], x, j3);
    }
    const v3 c1 = v3_cross(j2, j3), c2 = v3_cross(j3, j1), c3 = v3_cross(j1, j2);
    const double adet = fabs(v3_dot(j1, c1));
    const double s = w / adet;
    // A c_b for b = 1..3, then G_ab = s c_a . (A c_b)
    const v3 cb[3] = {c1, c2, c3};
    v3 Ac[3];
#pragma unroll
    for (int b = 0; b < 3; b++)
      Ac[b] = {fma(sA[0], cb[b].x, fma(sA[1], cb[b].y, sA[2] * cb[b].z)),
               fma(sA[3], cb[b].x, fma(sA[4], cb[b].y, sA[5] * cb[b].z)),
               fma(sA[6], cb[b].x, fma(sA[7], cb[b].y, sA[8] * cb[b].z))};
    // G_ab = s (A c_b) . c_a: the tensor a_ij multiplies d_i(test) d_j(trial),
    // so with test index a and trial index b: G_ab = s c_a^T A c_b
    sG[q][0] = s * v3_dot(cb[0], Ac[0]);
    sG[q][1] = s * v3_dot(cb[0], Ac[1]);
    sG[q][2] = s * v3_dot(cb[0], Ac[2]);
    sG[q][3] = s * v3_dot(cb[1], Ac[1]);
    sG[q][4] = s * v3_dot(cb[1], Ac[2]);
    sG[q][5] = s * v3_dot(cb[2], Ac[2]);
    sV[q] = w * adet;
  }
  __syncthreads();
  // load vector
  for (int u = tid; u < NS; u += DG_THREADS) {
    double r = 0.0;
    for (int q = 0; q < NQ; q++) r = fma(PHItab[(size_t)q * NS + u], sV[q], r);
    if (write) rhs_out[u] = f * r;
  }
}

// upper entry k of an NS x NS block as (u, w), u <= w (row u holds (u, u..NS-1))
template <int NS>
__device__ __forceinline__ void dg_upper_entry(int k, int &u, int &w) {
  u = 0;
  while (k >= NS - u) {
    k -= NS - u;
    u++;
  }
  w = u + k;
}

// shared scratch: sG[NQ][6], sV[NQ], sT[QC][3][NS]
template <int P, int THR, int QC>
__device__ __forceinline__ void dg_prism_volume_body(const double *sX, const double *sA, double f,
                                                     const double *__restrict__ Dtab,
                                                     const double *__restrict__ PHItab,
                                                     const double *__restrict__ QPtab, double *blk,
                                                     double *rhs_out, double (*sG)[6], double *sV,
                                                     double (*sT)[3][DgDims<P, THR, QC>::NS], int tid,
                                                     bool write) {
  using Dm = DgDims<P, THR, QC>;
  constexpr int NS = Dm::NS, NQ = Dm::NQ, DG_THREADS = Dm::THREADS, DG_QCHUNK = Dm::QCHUNK;
  dg_volume_points<P, THR, QC>(sX, sA, f, PHItab, QPtab, rhs_out, sG, sV, tid, write);
  // stiffness: upper entries k = tid + j * DG_THREADS
  double acc[Dm::PER_THREAD];
  int uu[Dm::PER_THREAD], ww[Dm::PER_THREAD];
#pragma unroll
  for (int j = 0; j < Dm::PER_THREAD; j++) {
    acc[j] = 0.0;
    int k = tid + j * DG_THREADS;
    int u = 0;
    if (k < Dm::NSYM) {
      // row u holds entries (u, u..NS-1): find u with k in [off(u), off(u+1))
      while (k >= NS - u) {
        k -= NS - u;
        u++;
      }
      uu[j] = u;
      ww[j] = u + k;
    } else {
      uu[j] = 0;
      ww[j] = -1;
    }
  }
  for (int q0 = 0; q0 < NQ; q0 += DG_QCHUNK) {
    const int qn = NQ - q0 < DG_QCHUNK ? NQ - q0 : DG_QCHUNK;
    __syncthreads();
    // T_q[a][w] = sum_b G_q[a][b] D_q[b][w]
    for (int t = tid; t < qn * NS; t += DG_THREADS) {
      const int ql = t / NS, w = t % NS, q = q0 + ql;
      const double *Dq = Dtab + (size_t)q * 3 * NS;
      const double d0 = Dq[w], d1 = Dq[NS + w], d2 = Dq[2 * NS + w];
      const double *g = sG[q];
      sT[ql][0][w] = fma(g[0], d0, fma(g[1], d1, g[2] * d2));
      sT[ql][1][w] = fma(g[1], d0, fma(g[3], d1, g[4] * d2));
      sT[ql][2][w] = fma(g[2], d0, fma(g[4], d1, g[5] * d2));
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < Dm::PER_THREAD; j++) {
      if (ww[j] < 0) continue;
      const int u = uu[j], w = ww[j];
      double a = acc[j];
      for (int ql = 0; ql < qn; ql++) {
        const double *Dq = Dtab + (size_t)(q0 + ql) * 3 * NS;
        a = fma(__ldg(Dq + u), sT[ql][0][w], a);
        a = fma(__ldg(Dq + NS + u), sT[ql][1][w], a);
        a = fma(__ldg(Dq + 2 * NS + u), sT[ql][2][w], a);
      }
      acc[j] = a;
    }
  }
  // K_uw (test w, trial u) is column-major in the block: blk[w + NS u]
  if (!write) return;
#pragma unroll
  for (int j = 0; j < Dm::PER_THREAD; j++) {
    if (ww[j] < 0) continue;
    const int u = uu[j], w = ww[j];
    blk[w + (size_t)NS * u] = acc[j];
    if (u != w) blk[u + (size_t)NS * w] = acc[j];
  }
}

// Double-word form of the stiffness (the points and the load vector as
// above): T_q = G_q D_q formed in FP64 and stored as double words, every
// upper entry a sum over the points of 3 products of double words (D from
// the double-word table) by exact products and TwoSum chains (DwAcc), the
// entries of a thread interleaved point by point.  Entries within about
// 2^-48 of the summed magnitudes; the FP64 pipe keeps only the geometry and
// the T_q (9 FMAs per point and function).
template <int P, int THR, int QC>
__device__ __forceinline__ void dg_prism_volume_body_dw(const double *sX, const double *sA, double f,
                                                        const double *__restrict__ Dtab,
                                                        const float2 *__restrict__ Ddw,
                                                        const double *__restrict__ PHItab,
                                                        const double *__restrict__ QPtab, double *blk,
                                                        double *rhs_out, double (*sG)[6], double *sV,
                                                        float2 (*sT)[3][DgDims<P, THR, QC>::NS], int tid,
                                                        bool write = true) {
  using Dm = DgDims<P, THR, QC>;
  constexpr int NS = Dm::NS, NQ = Dm::NQ, DG_THREADS = Dm::THREADS, DG_QCHUNK = Dm::QCHUNK;
  constexpr int PER = Dm::PER_THREAD;
  dg_volume_points<P, THR, QC>(sX, sA, f, PHItab, QPtab, rhs_out, sG, sV, tid, write);
  DwAcc acc[PER];
  int uu[PER], ww[PER];
#pragma unroll
  for (int j = 0; j < PER; j++) {
    acc[j] = DwAcc{0.0f, 0.0f, 0.0f};
    const int k = tid + j * DG_THREADS;
    if (k < Dm::NSYM) {
      dg_upper_entry<NS>(k, uu[j], ww[j]);
    } else {
      uu[j] = 0;
      ww[j] = -1;
    }
  }
  for (int q0 = 0; q0 < NQ; q0 += DG_QCHUNK) {
    const int qn = NQ - q0 < DG_QCHUNK ? NQ - q0 : DG_QCHUNK;
    __syncthreads();
    for (int t = tid; t < qn * NS; t += DG_THREADS) {
      const int ql = t / NS, w = t % NS, q = q0 + ql;
      const double *Dq = Dtab + (size_t)q * 3 * NS;
      const double d0 = Dq[w], d1 = Dq[NS + w], d2 = Dq[2 * NS + w];
      const double *g = sG[q];
      sT[ql][0][w] = dw_f2(fma(g[0], d0, fma(g[1], d1, g[2] * d2)));
      sT[ql][1][w] = dw_f2(fma(g[1], d0, fma(g[3], d1, g[4] * d2)));
      sT[ql][2][w] = dw_f2(fma(g[2], d0, fma(g[4], d1, g[5] * d2)));
    }
    __syncthreads();
    for (int ql = 0; ql < qn; ql++) {
      const float2 *Dq = Ddw + (size_t)(q0 + ql) * 3 * NS;
#pragma unroll
      for (int j = 0; j < PER; j++) {
        if (ww[j] < 0) continue;
        const int u = uu[j], w = ww[j];
        dwacc_prod(acc[j], __ldg(Dq + u), sT[ql][0][w]);
        dwacc_prod(acc[j], __ldg(Dq + NS + u), sT[ql][1][w]);
        dwacc_prod(acc[j], __ldg(Dq + 2 * NS + u), sT[ql][2][w]);
      }
      if (ql & 1) {
#pragma unroll
        for (int j = 0; j < PER; j++) dwacc_fold(acc[j]);
      }
    }
#pragma unroll
    for (int j = 0; j < PER; j++) dwacc_fold(acc[j]);
  }
  if (!write) return;
#pragma unroll
  for (int j = 0; j < PER; j++) {
    if (ww[j] < 0) continue;
    const int u = uu[j], w = ww[j];
    const double v = dwacc_value(acc[j]);
    blk[w + (size_t)NS * u] = v;
    if (u != w) blk[u + (size_t)NS * w] = v;
  }
}

}  // namespace gbfem
