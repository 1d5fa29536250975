// DG prism volume integrals (tensor monomial basis, p = 1..4), FP64.
//
// Reference: apr_num_int_el of apd_dg_prism (aps_dg_prism_intf.c:1239-1728):
// K_uw = sum_q vol_q sum_ij a_ij d_i phi_w d_j phi_u, R_w = sum_q vol_q f phi_w,
// basis and rules as in dg_tables.h.
//
// With the adjugate rows c_a of the Jacobian (grad phi = (1/det) sum_a
// dphi/dxi_a c_a) every point contributes D_q^T G_q D_q with D_q the 3 x ns
// reference derivatives (element independent, a per-degree table) and
// G_q = (w_q / |det|) C^T A C, a 3x3 matrix (6 entries for symmetric A).
// One CTA integrates one element: threads first build G_q for all points,
// then per chunk of points T_q = G_q D_q (3 x ns) in shared memory, then each
// thread accumulates its share of the ns(ns+1)/2 upper entries
// K_uw += sum_a D_q[a][u] T_q[a][w].  FP64 per element:
// nq (9 ns + 3 ns (ns+1)/2) FMA (p=3: 135k).  On GB300 the FP64 pipe issues
// 2 FMA/clk/SM while shared memory serves 16 doubles/clk/SM, so the kernel is
// FP64-bound, not shared-memory bound.
//
// The element's own matrix is its diagonal block in the block-CRS storage
// (dense ns x ns, column-major, offset boff[e]); no other element writes
// there, so no atomics are needed for volume terms.

#include "gbfem_internal.h"
#include "dg_tables.h"
#include "prism_std.cuh"

namespace gbfem {

// per-degree device tables: D[q][a][u] reference derivatives, PHI[q][u] values
struct DgDeviceTables {
  const double *D[GB_DG_PMAX + 1];
  const double *PHI[GB_DG_PMAX + 1];
  const double *QP[GB_DG_PMAX + 1];  // (xi, eta, zeta, w) per point
};

static DgDeviceTables g_dg_tables[64];
static bool g_dg_tables_ready[64] = {false};

// Builds D and PHI for degree p on the host from the monomial exponents.
static void host_dg_tables(int p, std::vector<double> &D, std::vector<double> &PHI, std::vector<double> &QP) {
  const int ns = GB_DG_NS[p], nq = GB_DG_NQ[p];
  D.assign((size_t)nq * 3 * ns, 0.0);
  PHI.assign((size_t)nq * ns, 0.0);
  QP.assign((size_t)nq * 4, 0.0);
  for (int q = 0; q < nq; q++) {
    const double *e = GB_DG_QP[p - 1][q];
    for (int k = 0; k < 4; k++) QP[q * 4 + k] = e[k];
    double px[8], py[8], pz[8];
    px[0] = py[0] = pz[0] = 1.0;
    for (int i = 1; i <= p; i++) {
      px[i] = px[i - 1] * e[0];
      py[i] = py[i - 1] * e[1];
      pz[i] = pz[i - 1] * e[2];
    }
    for (int u = 0; u < ns; u++) {
      const int a = GB_DG_EXP[p - 1][u][0], b = GB_DG_EXP[p - 1][u][1], c = GB_DG_EXP[p - 1][u][2];
      PHI[(size_t)q * ns + u] = px[a] * py[b] * pz[c];
      D[((size_t)q * 3 + 0) * ns + u] = a ? a * px[a - 1] * py[b] * pz[c] : 0.0;
      D[((size_t)q * 3 + 1) * ns + u] = b ? b * px[a] * py[b - 1] * pz[c] : 0.0;
      D[((size_t)q * 3 + 2) * ns + u] = c ? c * px[a] * py[b] * pz[c - 1] : 0.0;
    }
  }
}

int dg_tables_for_device(int device, DgDeviceTables **out) {
  GB_CHECK(device >= 0 && device < 64, "device index out of range");
  if (!g_dg_tables_ready[device]) {
    for (int p = 1; p <= GB_DG_PMAX; p++) {
      std::vector<double> D, PHI, QP;
      host_dg_tables(p, D, PHI, QP);
      double *d = nullptr, *ph = nullptr, *qp = nullptr;
      GB_CUDA(cudaMalloc(&d, D.size() * sizeof(double)));
      GB_CUDA(cudaMalloc(&ph, PHI.size() * sizeof(double)));
      GB_CUDA(cudaMalloc(&qp, QP.size() * sizeof(double)));
      GB_CUDA(cudaMemcpy(d, D.data(), D.size() * sizeof(double), cudaMemcpyHostToDevice));
      GB_CUDA(cudaMemcpy(ph, PHI.data(), PHI.size() * sizeof(double), cudaMemcpyHostToDevice));
      GB_CUDA(cudaMemcpy(qp, QP.data(), QP.size() * sizeof(double), cudaMemcpyHostToDevice));
      g_dg_tables[device].D[p] = d;
      g_dg_tables[device].PHI[p] = ph;
      g_dg_tables[device].QP[p] = qp;
    }
    g_dg_tables_ready[device] = true;
  }
  *out = &g_dg_tables[device];
  return 0;
}

// Launch shapes (threads per CTA, quadrature points per shared-memory
// chunk) per degree; the autotuner times them on the mesh at hand.  Thread
// counts near a multiple of the NS(NS+1)/2 upper entries keep the FP64 lanes
// busy (21 / 32, 171 / 192, 820 / 864 = 3 x 288, 2850 / 2880 = 10 x 288).
// Every variant sums each entry over the points in the same order: identical
// results.
constexpr int DG_VOL_VARIANTS = 3;
__host__ __device__ constexpr int dg_vol_threads(int p, int v) {
  return p == 1 ? (v == 0 ? 32 : 64) : p == 2 ? (v == 0 ? 192 : v == 1 ? 96 : 192)
                                       : (v == 0 ? 288 : v == 1 ? 224 : 288);
}
__host__ __device__ constexpr int dg_vol_qchunk(int p, int v) { return v == 2 ? 16 : 8; }

template <int P, int THR, int QC>
struct DgDims {
  static constexpr int NS = P == 1 ? 6 : P == 2 ? 18 : P == 3 ? 40 : 75;
  static constexpr int NQ = P == 1 ? 6 : P == 2 ? 18 : P == 3 ? 48 : 80;
  static constexpr int THREADS = THR;
  static constexpr int QCHUNK = QC;
  static constexpr int NSYM = NS * (NS + 1) / 2;
  static constexpr int PER_THREAD = (NSYM + THREADS - 1) / THREADS;
};

// Elements of degree P: ent_el[i] (0-based), matrix block at val + boff[e],
// rhs rows at rhs + roff[e].  A (tensor, 9 per element) or k (isotropic).
template <int P, int THR, int QC>
__global__ void __launch_bounds__(THR) dg_prism_elements_kernel(
    int count, const int *__restrict__ ent_el, const int *__restrict__ el_nodes, const double *__restrict__ xyz,
    const double *__restrict__ k_el, const double *__restrict__ D_el, double f, const double *__restrict__ Dtab,
    const double *__restrict__ PHItab, const double *__restrict__ QPtab, const long long *__restrict__ boff,
    const int *__restrict__ roff, double *__restrict__ val, double *__restrict__ rhs) {
  using Dm = DgDims<P, THR, QC>;
  constexpr int NS = Dm::NS, NQ = Dm::NQ, DG_THREADS = Dm::THREADS, DG_QCHUNK = Dm::QCHUNK;
  __shared__ double sG[NQ][6];        // w/|det| C^T A C (symmetric, packed 00 01 02 11 12 22)
  __shared__ double sV[NQ];           // w |det|
  __shared__ double sT[DG_QCHUNK][3][NS];
  __shared__ double sX[18];
  __shared__ double sA[9];
  const int bi = blockIdx.x;
  if (bi >= count) return;
  const int e = ent_el[bi];
  const int tid = threadIdx.x;
  if (tid < 6) {
    const int n = el_nodes[6 * (size_t)e + tid];
    sX[3 * tid] = xyz[3 * (size_t)n];
    sX[3 * tid + 1] = xyz[3 * (size_t)n + 1];
    sX[3 * tid + 2] = xyz[3 * (size_t)n + 2];
  }
  if (tid < 9) {
    if (D_el)
      sA[tid] = D_el[9 * (size_t)e + tid];
    else
      sA[tid] = (tid == 0 || tid == 4 || tid == 8) ? (k_el ? k_el[e] : 1.0) : 0.0;
  }
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
    rhs[roff[e] + u] = f * r;
  }
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
  // K_uw (test w, trial u) is column-major in the block: val[w + NS u]
  double *blk = val + boff[e];
#pragma unroll
  for (int j = 0; j < Dm::PER_THREAD; j++) {
    if (ww[j] < 0) continue;
    const int u = uu[j], w = ww[j];
    blk[w + (size_t)NS * u] = acc[j];
    if (u != w) blk[u + (size_t)NS * w] = acc[j];
  }
}

int launch_dg_prism_elements(cudaStream_t st, int device, int p, int count, const int *ent_el, const int *el_nodes,
                             const double *xyz, const double *k_el, const double *D_el, double f,
                             const long long *boff, const int *roff, double *val, double *rhs, int variant) {
  if (count <= 0) return 0;
  GB_CHECK(p >= 1 && p <= GB_DG_PMAX, "DG degree must be 1..4");
  GB_CHECK(variant >= 0 && variant < DG_VOL_VARIANTS, "volume kernel variant out of range");
  DgDeviceTables *tb = nullptr;
  int r = dg_tables_for_device(device, &tb);
  if (r < 0) return r;
#define GB_DG_LAUNCH(PP, VV)                                                                               \
  dg_prism_elements_kernel<PP, dg_vol_threads(PP, VV), dg_vol_qchunk(PP, VV)>                             \
      <<<count, dg_vol_threads(PP, VV), 0, st>>>(count, ent_el, el_nodes, xyz, k_el, D_el, f, tb->D[PP],    \
                                                 tb->PHI[PP], tb->QP[PP], boff, roff, val, rhs)
#define GB_DG_P(PP)                  \
  switch (variant) {                 \
    case 0: GB_DG_LAUNCH(PP, 0); break; \
    case 1: GB_DG_LAUNCH(PP, 1); break; \
    default: GB_DG_LAUNCH(PP, 2); break; \
  }
  switch (p) {
    case 1: GB_DG_P(1); break;
    case 2: GB_DG_P(2); break;
    case 3: GB_DG_P(3); break;
    default: GB_DG_P(4); break;
  }
#undef GB_DG_P
#undef GB_DG_LAUNCH
  GB_CUDA(cudaGetLastError());
  return 1;
}

}  // namespace gbfem
