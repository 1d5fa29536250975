// Batched DG volume integrals of elements of mixed type and degree (tensor-
// basis prisms and complete-basis tetrahedra, p = 1..4, from any number of
// meshes) in one persistent launch replayed as a CUDA graph.  No reference
// counterpart for the batching; prisms follow apr_num_int_el of apd_dg_prism
// (aps_dg_prism_intf.c:1239-1728) through dg_volume.cuh.
//
// DG tetrahedra (the reference has none: apd_dg_prism is prism-only) use the
// complete monomial basis xi^a eta^b zeta^c, a + b + c <= p, on the
// reference tetrahedron (0,0,0), (1,0,0), (0,1,0), (0,0,1), ordered by total
// degree d, then a descending, then b descending: (p+1)(p+2)(p+3)/6 = 4, 10,
// 20, 35 functions.  An affine tetrahedron has a constant Jacobian, so
//   K = sum_c G_c T_c,  G = C^T A C / |det|  (6 entries, c = 00 01 02 11 12 22),
//   T_aa = S_aa, T_ab = S_ab + S_ba,  S_ab[i][j] = int_ref d_a phi_i d_b phi_j,
//   R_i = f |det| int_ref phi_i,
// with the reference matrices integrated exactly on the host from the
// monomial moments int_ref xi^a eta^b zeta^c = a! b! c! / (a+b+c+3)!.
//
// Work: tiles of (type, degree, first element, count) sorted heaviest first;
// persistent CTAs (one per SM, 256 threads) take tiles from an atomic
// counter.  A prism tile is one element (the CTA integrates it as the
// per-degree kernel does, bit-identical); a tetrahedron tile is `tet_tile`
// elements, threads over (element, upper entry).

#include <cmath>
#include <cstring>
#include <vector>

#include "dg_tables.h"
#include "dg_volume.cuh"
#include "gbfem_internal.h"

namespace gbfem {

constexpr int DGB_THREADS = 256;
constexpr int DGB_QC = 8;

__host__ __device__ constexpr int tet_ns(int p) { return (p + 1) * (p + 2) * (p + 3) / 6; }

struct DgBatchTile {
  int type;   // 0 prism, 1 tetrahedron
  int p;
  int first;  // first element of the tile within its type's arrays
  int count;
};

struct DgBatchTables {
  const double *D[GB_DG_PMAX + 1], *PHI[GB_DG_PMAX + 1], *QP[GB_DG_PMAX + 1];  // prisms
  const double *T[GB_DG_PMAX + 1];    // tets: 6 x (ns(ns+1)/2) packed upper entries
  const double *MOM[GB_DG_PMAX + 1];  // tets: int_ref phi_i
};

template <int P>
__device__ void dgb_prism(const DgBatchTables &tb, int e, const double *__restrict__ X, const double *__restrict__ A,
                          double f, const long long *__restrict__ off, const int *__restrict__ roff,
                          double *__restrict__ val, double *__restrict__ rhs, double *smem) {
  using Dm = DgDims<P, DGB_THREADS, DGB_QC>;
  double *sX = smem, *sA = smem + 18;
  double(*sG)[6] = (double(*)[6])(smem + 32);
  double *sV = smem + 32 + 6 * Dm::NQ;
  double(*sT)[3][Dm::NS] = (double(*)[3][Dm::NS])(smem + 32 + 7 * Dm::NQ);
  const int tid = threadIdx.x;
  __syncthreads();  // the previous tile is done with the scratch
  if (tid < 18) sX[tid] = X[18 * (size_t)e + tid];
  if (tid < 9) sA[tid] = A[9 * (size_t)e + tid];
  dg_prism_volume_body<P, DGB_THREADS, DGB_QC>(sX, sA, f, tb.D[P], tb.PHI[P], tb.QP[P], val + off[e], rhs + roff[e],
                                                sG, sV, sT);
}

template <int P>
__device__ void dgb_tets(const DgBatchTables &tb, int first, int count, const double *__restrict__ X,
                         const double *__restrict__ A, double f, const long long *__restrict__ off,
                         const int *__restrict__ roff, double *__restrict__ val, double *__restrict__ rhs,
                         double *smem) {
  constexpr int NS = tet_ns(P), NSYM = NS * (NS + 1) / 2;
  double *sGc = smem;  // [count][7]: 6 G entries, |det|
  const int tid = threadIdx.x;
  __syncthreads();
  for (int el = tid; el < count; el += DGB_THREADS) {
    const double *x = X + 12 * (size_t)(first + el), *a = A + 9 * (size_t)(first + el);
    const v3 x0 = {x[0], x[1], x[2]};
    const v3 j1 = v3_sub(v3{x[3], x[4], x[5]}, x0), j2 = v3_sub(v3{x[6], x[7], x[8]}, x0),
             j3 = v3_sub(v3{x[9], x[10], x[11]}, x0);
    const v3 cb[3] = {v3_cross(j2, j3), v3_cross(j3, j1), v3_cross(j1, j2)};
    const double adet = fabs(v3_dot(j1, cb[0]));
    v3 Ac[3];
#pragma unroll
    for (int b = 0; b < 3; b++)
      Ac[b] = {fma(a[0], cb[b].x, fma(a[1], cb[b].y, a[2] * cb[b].z)),
               fma(a[3], cb[b].x, fma(a[4], cb[b].y, a[5] * cb[b].z)),
               fma(a[6], cb[b].x, fma(a[7], cb[b].y, a[8] * cb[b].z))};
    const double s = 1.0 / adet;
    double *g = sGc + 7 * el;
    g[0] = s * v3_dot(cb[0], Ac[0]);
    g[1] = s * v3_dot(cb[0], Ac[1]);
    g[2] = s * v3_dot(cb[0], Ac[2]);
    g[3] = s * v3_dot(cb[1], Ac[1]);
    g[4] = s * v3_dot(cb[1], Ac[2]);
    g[5] = s * v3_dot(cb[2], Ac[2]);
    g[6] = adet;
  }
  __syncthreads();
  const double *T = tb.T[P];
  for (int t = tid; t < count * NSYM; t += DGB_THREADS) {
    const int el = t / NSYM, k0 = t % NSYM;
    int k = k0, u = 0;
    while (k >= NS - u) {
      k -= NS - u;
      u++;
    }
    const int w = u + k;
    const double *g = sGc + 7 * el;
    double v = 0.0;
#pragma unroll
    for (int c = 0; c < 6; c++) v = fma(g[c], __ldg(T + c * NSYM + k0), v);
    double *blk = val + off[first + el];
    blk[w + NS * u] = v;
    if (u != w) blk[u + NS * w] = v;
  }
  for (int t = tid; t < count * NS; t += DGB_THREADS) {
    const int el = t / NS, i = t % NS;
    rhs[roff[first + el] + i] = f * sGc[7 * el + 6] * __ldg(tb.MOM[P] + i);
  }
}

__global__ void __launch_bounds__(DGB_THREADS) dg_batch_kernel(
    int ntiles, const DgBatchTile *__restrict__ tiles, int *counter, DgBatchTables tb, double f,
    const double *__restrict__ pX, const double *__restrict__ pA, const long long *__restrict__ poff,
    const int *__restrict__ proff, const double *__restrict__ tX, const double *__restrict__ tA,
    const long long *__restrict__ toff, const int *__restrict__ troff, double *__restrict__ val,
    double *__restrict__ rhs) {
  extern __shared__ double smem[];
  __shared__ int s_tile;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_tile = atomicAdd(counter, 1);
    __syncthreads();
    const int t = s_tile;
    if (t >= ntiles) return;
    const DgBatchTile T = tiles[t];
    if (T.type == 0) {
      switch (T.p) {
        case 1: dgb_prism<1>(tb, T.first, pX, pA, f, poff, proff, val, rhs, smem); break;
        case 2: dgb_prism<2>(tb, T.first, pX, pA, f, poff, proff, val, rhs, smem); break;
        case 3: dgb_prism<3>(tb, T.first, pX, pA, f, poff, proff, val, rhs, smem); break;
        default: dgb_prism<4>(tb, T.first, pX, pA, f, poff, proff, val, rhs, smem); break;
      }
    } else {
      switch (T.p) {
        case 1: dgb_tets<1>(tb, T.first, T.count, tX, tA, f, toff, troff, val, rhs, smem); break;
        case 2: dgb_tets<2>(tb, T.first, T.count, tX, tA, f, toff, troff, val, rhs, smem); break;
        case 3: dgb_tets<3>(tb, T.first, T.count, tX, tA, f, toff, troff, val, rhs, smem); break;
        default: dgb_tets<4>(tb, T.first, T.count, tX, tA, f, toff, troff, val, rhs, smem); break;
      }
    }
  }
}

// ------------------------------------------------------------------ host
// exact reference-tetrahedron matrices for degree p
static void tet_tables(int p, std::vector<double> &T, std::vector<double> &MOM, std::vector<int> &EXP) {
  const int ns = tet_ns(p), nsym = ns * (ns + 1) / 2;
  EXP.clear();
  for (int d = 0; d <= p; d++)
    for (int a = d; a >= 0; a--)
      for (int b = d - a; b >= 0; b--) {
        EXP.push_back(a);
        EXP.push_back(b);
        EXP.push_back(d - a - b);
      }
  std::vector<double> fact(3 * p + 8, 1.0);
  for (size_t i = 1; i < fact.size(); i++) fact[i] = fact[i - 1] * (double)i;
  auto mom = [&](int a, int b, int c) { return fact[a] * fact[b] * fact[c] / fact[a + b + c + 3]; };
  MOM.assign(ns, 0.0);
  for (int i = 0; i < ns; i++) MOM[i] = mom(EXP[3 * i], EXP[3 * i + 1], EXP[3 * i + 2]);
  // S_ab[i][j] = int d_a phi_i d_b phi_j
  auto S = [&](int a, int b, int i, int j) {
    int ei[3] = {EXP[3 * i], EXP[3 * i + 1], EXP[3 * i + 2]}, ej[3] = {EXP[3 * j], EXP[3 * j + 1], EXP[3 * j + 2]};
    if (ei[a] == 0 || ej[b] == 0) return 0.0;
    const double coef = (double)ei[a] * ej[b];
    ei[a]--;
    ej[b]--;
    return coef * mom(ei[0] + ej[0], ei[1] + ej[1], ei[2] + ej[2]);
  };
  const int pa[6] = {0, 0, 0, 1, 1, 2}, pb[6] = {0, 1, 2, 1, 2, 2};
  T.assign(6 * (size_t)nsym, 0.0);
  for (int c = 0; c < 6; c++) {
    int k = 0;
    for (int u = 0; u < ns; u++)
      for (int w = u; w < ns; w++, k++)
        T[(size_t)c * nsym + k] = pa[c] == pb[c] ? S(pa[c], pa[c], u, w) : S(pa[c], pb[c], u, w) + S(pb[c], pa[c], u, w);
  }
}

static DgBatchTables g_bt[64];
static bool g_bt_ready[64];

int dg_batch_tables(int device, DgBatchTables *out) {
  GB_CHECK(device >= 0 && device < 64, "device index out of range");
  if (!g_bt_ready[device]) {
    DgDeviceTables *pt = nullptr;
    const int r = dg_tables_for_device(device, &pt);
    if (r < 0) return r;
    for (int p = 1; p <= GB_DG_PMAX; p++) {
      g_bt[device].D[p] = pt->D[p];
      g_bt[device].PHI[p] = pt->PHI[p];
      g_bt[device].QP[p] = pt->QP[p];
      std::vector<double> T, MOM;
      std::vector<int> EXP;
      tet_tables(p, T, MOM, EXP);
      double *dT = nullptr, *dM = nullptr;
      GB_CUDA(cudaMalloc(&dT, T.size() * sizeof(double)));
      GB_CUDA(cudaMalloc(&dM, MOM.size() * sizeof(double)));
      GB_CUDA(cudaMemcpy(dT, T.data(), T.size() * sizeof(double), cudaMemcpyHostToDevice));
      GB_CUDA(cudaMemcpy(dM, MOM.data(), MOM.size() * sizeof(double), cudaMemcpyHostToDevice));
      g_bt[device].T[p] = dT;
      g_bt[device].MOM[p] = dM;
    }
    g_bt_ready[device] = true;
  }
  *out = g_bt[device];
  return 0;
}

}  // namespace gbfem

// ------------------------------------------------------------------ C ABI
using gbfem::DevBuf;
using gbfem::DgBatchTile;

struct gbfem_batch_s {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int np = 0, nt = 0, tet_tile = 32, ntiles = 0;
  double f = 1.0;
  long long nval = 0, nrhs = 0;
  DevBuf<double> pX, pA, tX, tA, val, rhs;
  DevBuf<long long> poff, toff;
  DevBuf<int> proff, troff, counter;
  DevBuf<DgBatchTile> tiles;
  std::vector<int> pp, tp;
  cudaGraphExec_t graph = nullptr;
  float last_ms = 0.f;
};

static int batch_build(gbfem_batch b) {
  // tiles: heaviest first (prisms p4 .. p1, then tets p4 .. p1)
  std::vector<DgBatchTile> tiles;
  std::vector<int> order_p, order_t;
  for (int p = 4; p >= 1; p--)
    for (int e = 0; e < b->np; e++)
      if (b->pp[e] == p) tiles.push_back({0, p, e, 1});
  for (int p = 4; p >= 1; p--) {
    int run = -1, cnt = 0;
    for (int e = 0; e <= b->nt; e++) {
      const bool in = e < b->nt && b->tp[e] == p;
      // consecutive elements of one degree form tiles of up to tet_tile
      if (in && run >= 0 && cnt < b->tet_tile && e == run + cnt) {
        cnt++;
        continue;
      }
      if (run >= 0) tiles.push_back({1, p, run, cnt});
      run = in ? e : -1;
      cnt = in ? 1 : 0;
    }
  }
  b->ntiles = (int)tiles.size();
  if (b->tiles.alloc(std::max<size_t>(tiles.size(), 1)) < 0) return -1;
  if (!tiles.empty())
    GB_CUDA(cudaMemcpy(b->tiles.p, tiles.data(), tiles.size() * sizeof(DgBatchTile), cudaMemcpyHostToDevice));
  // capture memset + persistent kernel as a graph
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  gbfem::DgBatchTables tb;
  if (gbfem::dg_batch_tables(b->device, &tb) < 0) return -1;
  int sms = 0, occ = 0;
  GB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device));
  const size_t smem = sizeof(double) * std::max(32 + 7 * 80 + gbfem::DGB_QC * 3 * 75, 7 * b->tet_tile);
  GB_CUDA(cudaFuncSetAttribute(gbfem::dg_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, gbfem::dg_batch_kernel, gbfem::DGB_THREADS, smem));
  const int grid = sms * std::max(occ, 1);
  cudaGraph_t g = nullptr;
  GB_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  cudaMemsetAsync(b->counter.p, 0, sizeof(int), b->stream);
  gbfem::dg_batch_kernel<<<grid, gbfem::DGB_THREADS, smem, b->stream>>>(
      b->ntiles, b->tiles.p, b->counter.p, tb, b->f, b->pX.p, b->pA.p, b->poff.p, b->proff.p, b->tX.p, b->tA.p,
      b->toff.p, b->troff.p, b->val.p, b->rhs.p);
  GB_CUDA(cudaStreamEndCapture(b->stream, &g));
  const cudaError_t e = cudaGraphInstantiate(&b->graph, g, 0);
  cudaGraphDestroy(g);
  GB_CUDA(e);
  return 0;
}

extern "C" {

int gbfem_batch_create(gbfem_batch *out, int device) {
  GB_CHECK(out, "null pointer");
  GB_CUDA(cudaSetDevice(device));
  gbfem_batch b = new gbfem_batch_s();
  b->device = device;
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&b->e0) != cudaSuccess || cudaEventCreate(&b->e1) != cudaSuccess || b->counter.alloc(1) < 0) {
    delete b;
    gbfem::set_error("batch creation failed");
    return -1;
  }
  *out = b;
  return 0;
}

int gbfem_batch_destroy(gbfem_batch b) {
  if (!b) return 0;
  cudaSetDevice(b->device);
  cudaStreamSynchronize(b->stream);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  DevBuf<double> *d[] = {&b->pX, &b->pA, &b->tX, &b->tA, &b->val, &b->rhs};
  for (auto *x : d) x->release();
  b->poff.release();
  b->toff.release();
  b->proff.release();
  b->troff.release();
  b->counter.release();
  b->tiles.release();
  cudaEventDestroy(b->e0);
  cudaEventDestroy(b->e1);
  cudaStreamDestroy(b->stream);
  delete b;
  return 0;
}

int gbfem_batch_set(gbfem_batch b, int np, const double *prism_xyz, const double *prism_A, const int *prism_p,
                    int nt, const double *tet_xyz, const double *tet_A, const int *tet_p, double f, int tet_tile,
                    long long *nval, long long *nrhs) {
  GB_CHECK(b, "null batch");
  GB_CHECK(np >= 0 && nt >= 0 && np + nt > 0, "empty batch");
  GB_CHECK(np == 0 || (prism_xyz && prism_A && prism_p), "prism arrays missing");
  GB_CHECK(nt == 0 || (tet_xyz && tet_A && tet_p), "tetrahedron arrays missing");
  GB_CHECK(tet_tile >= 1 && tet_tile <= 256, "tet_tile must be 1..256");
  GB_CUDA(cudaSetDevice(b->device));
  b->np = np;
  b->nt = nt;
  b->f = f;
  b->tet_tile = tet_tile;
  b->pp.assign(prism_p, prism_p + np);
  b->tp.assign(tet_p, tet_p + nt);
  // output: prism blocks, then tet blocks, each ns x ns column-major
  std::vector<long long> poff(np), toff(nt);
  std::vector<int> proff(np), troff(nt);
  long long v = 0;
  int r = 0;
  for (int e = 0; e < np; e++) {
    GB_CHECK(prism_p[e] >= 1 && prism_p[e] <= 4, "degree must be 1..4");
    const int ns = GB_DG_NS[prism_p[e]];
    poff[e] = v;
    proff[e] = r;
    v += (long long)ns * ns;
    r += ns;
  }
  for (int e = 0; e < nt; e++) {
    GB_CHECK(tet_p[e] >= 1 && tet_p[e] <= 4, "degree must be 1..4");
    const int ns = gbfem::tet_ns(tet_p[e]);
    toff[e] = v;
    troff[e] = r;
    v += (long long)ns * ns;
    r += ns;
  }
  b->nval = v;
  b->nrhs = r;
  auto up = [&](auto &buf, const auto *h, size_t n) -> int {
    if (buf.alloc(std::max<size_t>(n, 1)) < 0) return -1;
    if (n) GB_CUDA(cudaMemcpy(buf.p, h, n * sizeof(*h), cudaMemcpyHostToDevice));
    return 0;
  };
  if (up(b->pX, prism_xyz, 18 * (size_t)np) < 0 || up(b->pA, prism_A, 9 * (size_t)np) < 0 ||
      up(b->tX, tet_xyz, 12 * (size_t)nt) < 0 || up(b->tA, tet_A, 9 * (size_t)nt) < 0 ||
      up(b->poff, poff.data(), poff.size()) < 0 || up(b->toff, toff.data(), toff.size()) < 0 ||
      up(b->proff, proff.data(), proff.size()) < 0 || up(b->troff, troff.data(), troff.size()) < 0 ||
      b->val.alloc((size_t)v) < 0 || b->rhs.alloc((size_t)r) < 0)
    return -1;
  if (batch_build(b) < 0) return -1;
  if (nval) *nval = v;
  if (nrhs) *nrhs = r;
  return 0;
}

int gbfem_batch_run(gbfem_batch b, double *ms) {
  GB_CHECK(b && b->graph, "batch not set");
  GB_CUDA(cudaSetDevice(b->device));
  cudaEventRecord(b->e0, b->stream);
  GB_CUDA(cudaGraphLaunch(b->graph, b->stream));
  cudaEventRecord(b->e1, b->stream);
  GB_CUDA(cudaEventSynchronize(b->e1));
  cudaEventElapsedTime(&b->last_ms, b->e0, b->e1);
  if (ms) *ms = b->last_ms;
  return b->ntiles;
}

int gbfem_batch_get(gbfem_batch b, double *vals, double *rhs) {
  GB_CHECK(b && b->graph, "batch not set");
  if (vals) GB_CUDA(cudaMemcpy(vals, b->val.p, (size_t)b->nval * sizeof(double), cudaMemcpyDeviceToHost));
  if (rhs) GB_CUDA(cudaMemcpy(rhs, b->rhs.p, (size_t)b->nrhs * sizeof(double), cudaMemcpyDeviceToHost));
  return 0;
}

}  // extern "C"
