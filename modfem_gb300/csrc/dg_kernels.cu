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
#include "dg_volume.cuh"
#include "prism_std.cuh"

namespace gbfem {

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
      std::vector<float2> Dw(D.size());
      for (size_t i = 0; i < D.size(); i++) {
        const float h = (float)D[i];
        Dw[i] = make_float2(h, (float)(D[i] - (double)h));
      }
      float2 *dw = nullptr;
      GB_CUDA(cudaMalloc(&dw, Dw.size() * sizeof(float2)));
      GB_CUDA(cudaMemcpy(dw, Dw.data(), Dw.size() * sizeof(float2), cudaMemcpyHostToDevice));
      g_dg_tables[device].D[p] = d;
      g_dg_tables[device].PHI[p] = ph;
      g_dg_tables[device].QP[p] = qp;
      g_dg_tables[device].Ddw[p] = dw;
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
// The double-word kernel is bound by issue and latency, not by the FP64
// pipe: at p = 4 it takes 720 threads (four of the 2,850 entries each) so
// that more warps share the SM; the other degrees keep the FP64 shapes.
__host__ __device__ constexpr int dg_vol_threads_dw(int p, int v) { return p == 4 ? 720 : dg_vol_threads(p, v); }


// Elements of degree P: ent_el[i] (0-based), matrix block at val + boff[e],
// rhs rows at rhs + roff[e].  A (tensor, 9 per element) or k (isotropic).
template <int P, int THR, int QC>
__global__ void __launch_bounds__(THR) dg_prism_elements_kernel(
    int count, const int *__restrict__ ent_el, const int *__restrict__ el_nodes, const double *__restrict__ xyz,
    const double *__restrict__ k_el, const double *__restrict__ D_el, double f, const double *__restrict__ Dtab,
    const double *__restrict__ PHItab, const double *__restrict__ QPtab, const long long *__restrict__ boff,
    const int *__restrict__ roff, double *__restrict__ val, double *__restrict__ rhs) {
  using Dm = DgDims<P, THR, QC>;
  __shared__ double sG[Dm::NQ][6];  // w/|det| C^T A C (symmetric, packed 00 01 02 11 12 22)
  __shared__ double sV[Dm::NQ];     // w |det|
  __shared__ double sT[QC][3][Dm::NS];
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
  dg_prism_volume_body<P, THR, QC>(sX, sA, f, Dtab, PHItab, QPtab, val + boff[e], rhs + roff[e], sG, sV, sT, tid,
                                   true);
}

// The same elements with the stiffness summed in double-word arithmetic
// (dg_prism_volume_body_dw).
template <int P, int THR, int QC>
__global__ void __launch_bounds__(THR) dg_prism_elements_dw_kernel(
    int count, const int *__restrict__ ent_el, const int *__restrict__ el_nodes, const double *__restrict__ xyz,
    const double *__restrict__ k_el, const double *__restrict__ D_el, double f, const double *__restrict__ Dtab,
    const float2 *__restrict__ Ddw, const double *__restrict__ PHItab, const double *__restrict__ QPtab,
    const long long *__restrict__ boff, const int *__restrict__ roff, double *__restrict__ val,
    double *__restrict__ rhs) {
  using Dm = DgDims<P, THR, QC>;
  __shared__ double sG[Dm::NQ][6];
  __shared__ double sV[Dm::NQ];
  __shared__ float2 sT[QC][3][Dm::NS];
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
  dg_prism_volume_body_dw<P, THR, QC>(sX, sA, f, Dtab, Ddw, PHItab, QPtab, val + boff[e], rhs + roff[e], sG, sV, sT,
                                      tid);
}

int launch_dg_prism_elements(cudaStream_t st, int device, int p, int count, const int *ent_el, const int *el_nodes,
                             const double *xyz, const double *k_el, const double *D_el, double f,
                             const long long *boff, const int *roff, double *val, double *rhs, int variant,
                             bool dword) {
  if (count <= 0) return 0;
  GB_CHECK(p >= 1 && p <= GB_DG_PMAX, "DG degree must be 1..4");
  GB_CHECK(variant >= 0 && variant < DG_VOL_VARIANTS, "volume kernel variant out of range");
  DgDeviceTables *tb = nullptr;
  int r = dg_tables_for_device(device, &tb);
  if (r < 0) return r;
#define GB_DG_LAUNCH(PP, VV)                                                                                 \
  if (dword)                                                                                                 \
    dg_prism_elements_dw_kernel<PP, dg_vol_threads_dw(PP, VV), dg_vol_qchunk(PP, VV)>                        \
        <<<count, dg_vol_threads_dw(PP, VV), 0, st>>>(count, ent_el, el_nodes, xyz, k_el, D_el, f, tb->D[PP], \
                                                   tb->Ddw[PP], tb->PHI[PP], tb->QP[PP], boff, roff, val, rhs); \
  else                                                                                                       \
    dg_prism_elements_kernel<PP, dg_vol_threads(PP, VV), dg_vol_qchunk(PP, VV)>                              \
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
