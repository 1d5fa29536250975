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
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "dg_tables.h"
#include "dg_volume.cuh"
#include "gbfem_internal.h"

namespace gbfem {

constexpr int DGB_THREADS = 256;
__host__ __device__ constexpr int tet_ns(int p) { return (p + 1) * (p + 2) * (p + 3) / 6; }

// Work: tiles of one (type, degree, launch variant) class, listed heaviest
// class first; persistent CTAs (256 threads, as many as fit on the SMs) take
// tiles from an atomic counter.  A prism tile holds 256 / THR elements, each
// integrated by a group of THR threads exactly as the per-degree kernel does
// (bit-identical for every variant); a tetrahedron tile holds `tile`
// elements, threads over (element, block entry).  The variant of each class
// (prism: threads per element, points per shared-memory chunk; tetrahedron:
// elements per tile) is chosen by gbfem_batch_autotune.

constexpr int DGB_VARIANTS = 3;    // prism variants per degree
constexpr int DGB_TET_VARIANTS = 5;
__host__ __device__ constexpr int dgb_prism_thr(int p, int v) {
  return p == 1 ? (v == 0 ? 32 : v == 1 ? 64 : 128)
       : p == 2 ? (v == 0 ? 64 : v == 1 ? 128 : 256)
       : p == 3 ? (v == 2 ? 128 : 256)
                : 256;
}
__host__ __device__ constexpr int dgb_prism_qc(int p, int v) {
  return p == 3 ? (v == 1 ? 16 : 8) : p == 4 ? (v == 0 ? 8 : v == 1 ? 16 : 4) : 8;
}
__host__ __device__ constexpr int dgb_tet_tile(int v) { return 8 << v; }  // 8 .. 128
// shared doubles of one prism group
__host__ __device__ constexpr int dgb_prism_group_smem(int p, int v) {
  return 32 + 7 * (p == 1 ? 6 : p == 2 ? 18 : p == 3 ? 48 : 80) +
         dgb_prism_qc(p, v) * 3 * (p == 1 ? 6 : p == 2 ? 18 : p == 3 ? 40 : 75);
}

struct DgBatchTile {
  unsigned char type;  // 0 prism, 1 tetrahedron
  unsigned char p;
  unsigned char variant;
  unsigned char pad;
  int start;  // elements order[start .. start + count)
  int count;
  int pad2;
};

struct DgBatchTables {
  const double *D[GB_DG_PMAX + 1], *PHI[GB_DG_PMAX + 1], *QP[GB_DG_PMAX + 1];  // prisms
  const float2 *Ddw[GB_DG_PMAX + 1];  // prisms, D as double words
  const double *T[GB_DG_PMAX + 1];    // tets: 6 x (ns(ns+1)/2) packed upper entries
  const double *MOM[GB_DG_PMAX + 1];  // tets: int_ref phi_i
};

struct DgBatchArgs {
  const DgBatchTile *tiles;
  const int *order;
  const double *pX, *pA, *tX, *tA;  // gathered vertices (18 / 12) and tensors (9) per element
  const long long *poff, *toff;     // value offset of each element's block
  const int *proff, *troff;         // rhs offset
  double *val, *rhs;
  double f;
  int dword;  // prism stiffness sums in double-word arithmetic
};

template <int P, int THR, int QC>
__device__ void dgb_prism(const DgBatchTables &tb, const DgBatchArgs &a, const DgBatchTile &T, double *smem) {
  using Dm = DgDims<P, THR, QC>;
  constexpr int GROUP = 32 + 7 * Dm::NQ + QC * 3 * Dm::NS;
  const int g = threadIdx.x / THR, lt = threadIdx.x % THR;
  const bool valid = g < T.count;
  const int e = a.order[T.start + (valid ? g : T.count - 1)];
  double *base = smem + g * GROUP;
  double *sX = base, *sA = base + 18;
  double(*sG)[6] = (double(*)[6])(base + 32);
  double *sV = base + 32 + 6 * Dm::NQ;
  double(*sT)[3][Dm::NS] = (double(*)[3][Dm::NS])(base + 32 + 7 * Dm::NQ);
  if (lt < 18) sX[lt] = a.pX[18 * (size_t)e + lt];
  if (lt < 9) sA[lt] = a.pA[9 * (size_t)e + lt];
  if (a.dword)  // uniform over the launch; the float2 slices fill the same scratch
    dg_prism_volume_body_dw<P, THR, QC>(sX, sA, a.f, tb.D[P], tb.Ddw[P], tb.PHI[P], tb.QP[P], a.val + a.poff[e],
                                        a.rhs + a.proff[e], sG, sV, (float2(*)[3][Dm::NS])sT, lt, valid);
  else
    dg_prism_volume_body<P, THR, QC>(sX, sA, a.f, tb.D[P], tb.PHI[P], tb.QP[P], a.val + a.poff[e],
                                     a.rhs + a.proff[e], sG, sV, sT, lt, valid);
}

// The 6 geometric factors G = C^T A C / |det| (00 01 02 11 12 22) and |det|
// of an affine tetrahedron from its vertices x[12] and tensor A[9]
__device__ __forceinline__ void dg_tet_geometry(const double *x, const double *A, double *g) {
  const v3 x0 = {x[0], x[1], x[2]};
  const v3 j1 = v3_sub(v3{x[3], x[4], x[5]}, x0), j2 = v3_sub(v3{x[6], x[7], x[8]}, x0),
           j3 = v3_sub(v3{x[9], x[10], x[11]}, x0);
  const v3 cb[3] = {v3_cross(j2, j3), v3_cross(j3, j1), v3_cross(j1, j2)};
  const double adet = fabs(v3_dot(j1, cb[0]));
  v3 Ac[3];
#pragma unroll
  for (int b = 0; b < 3; b++)
    Ac[b] = {fma(A[0], cb[b].x, fma(A[1], cb[b].y, A[2] * cb[b].z)),
             fma(A[3], cb[b].x, fma(A[4], cb[b].y, A[5] * cb[b].z)),
             fma(A[6], cb[b].x, fma(A[7], cb[b].y, A[8] * cb[b].z))};
  const double s = 1.0 / adet;
  g[0] = s * v3_dot(cb[0], Ac[0]);
  g[1] = s * v3_dot(cb[0], Ac[1]);
  g[2] = s * v3_dot(cb[0], Ac[2]);
  g[3] = s * v3_dot(cb[1], Ac[1]);
  g[4] = s * v3_dot(cb[1], Ac[2]);
  g[5] = s * v3_dot(cb[2], Ac[2]);
  g[6] = adet;
}

template <int P>
__device__ void dgb_tets(const DgBatchTables &tb, const DgBatchArgs &a, const DgBatchTile &T, double *smem) {
  constexpr int NS = tet_ns(P), NSYM = NS * (NS + 1) / 2;
  static_assert(NSYM > 0, "degree");
  double *sGc = smem;  // [count][7]: 6 G entries, |det|
  int *sE = (int *)(smem + 7 * 128);
  const int tid = threadIdx.x, count = T.count;
  for (int el = tid; el < count; el += DGB_THREADS) {
    const int e = a.order[T.start + el];
    sE[el] = e;
    dg_tet_geometry(a.tX + 12 * (size_t)e, a.tA + 9 * (size_t)e, sGc + 7 * el);
  }
  __syncthreads();
  // every entry of the tile's blocks once, column-major within a block, so
  // consecutive threads write consecutive addresses (6 FMAs per entry from
  // the packed upper triangle of the reference matrices)
  const double *Tt = tb.T[P];
  for (int t = tid; t < count * NS * NS; t += DGB_THREADS) {
    const int el = t / (NS * NS), r = t % (NS * NS), u = r / NS, w = r % NS;
    const int lo = u < w ? u : w, hi = u < w ? w : u;
    const int k0 = lo * NS - lo * (lo - 1) / 2 + (hi - lo);
    const double *g = sGc + 7 * el;
    double v = 0.0;
#pragma unroll
    for (int c = 0; c < 6; c++) v = fma(g[c], __ldg(Tt + c * NSYM + k0), v);
    a.val[a.toff[sE[el]] + r] = v;
  }
  for (int t = tid; t < count * NS; t += DGB_THREADS) {
    const int el = t / NS, i = t % NS;
    a.rhs[a.troff[sE[el]] + i] = a.f * sGc[7 * el + 6] * __ldg(tb.MOM[P] + i);
  }
}

template <int P>
__device__ __forceinline__ void dgb_prism_variant(const DgBatchTables &tb, const DgBatchArgs &a,
                                                  const DgBatchTile &T, double *smem) {
  switch (T.variant) {
    case 0: dgb_prism<P, dgb_prism_thr(P, 0), dgb_prism_qc(P, 0)>(tb, a, T, smem); break;
    case 1: dgb_prism<P, dgb_prism_thr(P, 1), dgb_prism_qc(P, 1)>(tb, a, T, smem); break;
    default: dgb_prism<P, dgb_prism_thr(P, 2), dgb_prism_qc(P, 2)>(tb, a, T, smem); break;
  }
}

// Tetrahedra of degree P of a DG context (one CTA per 32 elements): vertex
// coordinates through el_nodes, tensor D_el (9 per element) or k_el I; block
// ns x ns column-major at val + boff[e], load vector at rhs + roff[e].  The
// same arithmetic as the batch tiles.
template <int P>
__global__ void __launch_bounds__(DGB_THREADS) dg_tet_elements_kernel(
    int count, const int *__restrict__ ent_el, const int *__restrict__ el_nodes, const double *__restrict__ xyz,
    const double *__restrict__ k_el, const double *__restrict__ D_el, double f, const double *__restrict__ Tt,
    const double *__restrict__ MOM, const long long *__restrict__ boff, const int *__restrict__ roff,
    double *__restrict__ val, double *__restrict__ rhs) {
  constexpr int NS = tet_ns(P), NSYM = NS * (NS + 1) / 2, TILE = 32;
  __shared__ double sGc[TILE][7];
  __shared__ int sE[TILE];
  const int tid = threadIdx.x, first = blockIdx.x * TILE;
  const int n = count - first < TILE ? count - first : TILE;
  if (tid < n) {
    const int e = ent_el[first + tid];
    sE[tid] = e;
    double x[12], A[9];
#pragma unroll
    for (int v = 0; v < 4; v++) {
      const int node = el_nodes[4 * (size_t)e + v];
#pragma unroll
      for (int d = 0; d < 3; d++) x[3 * v + d] = xyz[3 * (size_t)node + d];
    }
#pragma unroll
    for (int r = 0; r < 9; r++) A[r] = D_el ? D_el[9 * (size_t)e + r] : ((r % 4 == 0) ? (k_el ? k_el[e] : 1.0) : 0.0);
    dg_tet_geometry(x, A, sGc[tid]);
  }
  __syncthreads();
  for (int t = tid; t < n * NS * NS; t += DGB_THREADS) {
    const int el = t / (NS * NS), r = t % (NS * NS), u = r / NS, w = r % NS;
    const int lo = u < w ? u : w, hi = u < w ? w : u;
    const int k0 = lo * NS - lo * (lo - 1) / 2 + (hi - lo);
    double v = 0.0;
#pragma unroll
    for (int c = 0; c < 6; c++) v = fma(sGc[el][c], __ldg(Tt + c * NSYM + k0), v);
    val[boff[sE[el]] + r] = v;
  }
  for (int t = tid; t < n * NS; t += DGB_THREADS) {
    const int el = t / NS, i = t % NS;
    rhs[roff[sE[el]] + i] = f * sGc[el][6] * __ldg(MOM + i);
  }
}

__global__ void __launch_bounds__(DGB_THREADS) dg_batch_kernel(int ntiles, int *counter, DgBatchTables tb,
                                                               DgBatchArgs a) {
  extern __shared__ double smem[];
  __shared__ int s_tile;
  for (;;) {
    __syncthreads();  // the previous tile is done with s_tile and the scratch
    if (threadIdx.x == 0) s_tile = atomicAdd(counter, 1);
    __syncthreads();
    const int t = s_tile;
    if (t >= ntiles) return;
    const DgBatchTile T = a.tiles[t];
    if (T.type == 0) {
      switch (T.p) {
        case 1: dgb_prism_variant<1>(tb, a, T, smem); break;
        case 2: dgb_prism_variant<2>(tb, a, T, smem); break;
        case 3: dgb_prism_variant<3>(tb, a, T, smem); break;
        default: dgb_prism_variant<4>(tb, a, T, smem); break;
      }
    } else {
      switch (T.p) {
        case 1: dgb_tets<1>(tb, a, T, smem); break;
        case 2: dgb_tets<2>(tb, a, T, smem); break;
        case 3: dgb_tets<3>(tb, a, T, smem); break;
        default: dgb_tets<4>(tb, a, T, smem); break;
      }
    }
  }
}

// ------------------------------------------------------------------ host
// exact reference-tetrahedron matrices for degree p
static void tet_tables(int p, std::vector<double> &T, std::vector<double> &MOM) {
  const int ns = tet_ns(p), nsym = ns * (ns + 1) / 2;
  std::vector<int> EXP;
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

static int dg_batch_tables(int device, DgBatchTables *out) {
  GB_CHECK(device >= 0 && device < 64, "device index out of range");
  if (!g_bt_ready[device]) {
    DgDeviceTables *pt = nullptr;
    const int r = dg_tables_for_device(device, &pt);
    if (r < 0) return r;
    for (int p = 1; p <= GB_DG_PMAX; p++) {
      g_bt[device].D[p] = pt->D[p];
      g_bt[device].PHI[p] = pt->PHI[p];
      g_bt[device].QP[p] = pt->QP[p];
      g_bt[device].Ddw[p] = pt->Ddw[p];
      std::vector<double> T, MOM;
      tet_tables(p, T, MOM);
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

int launch_dg_tet_elements(cudaStream_t st, int device, int p, int count, const int *ent_el, const int *el_nodes,
                           const double *xyz, const double *k_el, const double *D_el, double f,
                           const long long *boff, const int *roff, double *val, double *rhs) {
  if (count <= 0) return 0;
  GB_CHECK(p >= 1 && p <= 4, "DG degree must be 1..4");
  DgBatchTables tb;
  const int r = dg_batch_tables(device, &tb);
  if (r < 0) return r;
  const int grid = (count + 31) / 32;
#define GB_TET_LAUNCH(PP)                                                                                       \
  dg_tet_elements_kernel<PP><<<grid, DGB_THREADS, 0, st>>>(count, ent_el, el_nodes, xyz, k_el, D_el, f, tb.T[PP], \
                                                           tb.MOM[PP], boff, roff, val, rhs)
  switch (p) {
    case 1: GB_TET_LAUNCH(1); break;
    case 2: GB_TET_LAUNCH(2); break;
    case 3: GB_TET_LAUNCH(3); break;
    default: GB_TET_LAUNCH(4); break;
  }
#undef GB_TET_LAUNCH
  GB_CUDA(cudaGetLastError());
  return 1;
}

// dynamic shared memory covering every class and variant
static size_t dgb_smem_bytes() {
  int m = 7 * 128 + 128;  // tets: G and |det| per element, element ids
  for (int p = 1; p <= 4; p++)
    for (int v = 0; v < DGB_VARIANTS; v++)
      m = std::max(m, (DGB_THREADS / dgb_prism_thr(p, v)) * dgb_prism_group_smem(p, v));
  return sizeof(double) * (size_t)m;
}

}  // namespace gbfem

// ------------------------------------------------------------------ C ABI
using gbfem::DevBuf;
using gbfem::DgBatchTile;

struct gbfem_batch_s {
  int device = 0, sms = 0, grid = 0;
  size_t smem = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int np = 0, nt = 0, ntiles = 0;
  int var_prism[5] = {0, 0, 0, 0, 0}, var_tet[5] = {2, 2, 2, 2, 2};
  double f = 1.0;
  int dword = 0;
  long long nval = 0, nrhs = 0;
  DevBuf<double> pX, pA, tX, tA, val, rhs;
  DevBuf<long long> poff, toff;
  DevBuf<int> proff, troff, counter, order;
  DevBuf<DgBatchTile> tiles;
  std::vector<int> pp, tp, order_h;
  std::vector<int> cls_start[2][5];  // element order of each class
  gbfem::DgBatchTables tb{};
  cudaGraphExec_t graph = nullptr;
  float last_ms = 0.f;
};

// order: elements grouped by class (prisms p = 1..4, then tets p = 1..4),
// input order within a class; cls_start[t][p] = {begin, end}
static void batch_order(gbfem_batch b) {
  b->order_h.clear();
  for (int t = 0; t < 2; t++)
    for (int p = 1; p <= 4; p++) {
      const std::vector<int> &deg = t == 0 ? b->pp : b->tp;
      const int begin = (int)b->order_h.size();
      for (int e = 0; e < (int)deg.size(); e++)
        if (deg[e] == p) b->order_h.push_back(e);
      b->cls_start[t][p] = {begin, (int)b->order_h.size()};
    }
}

// tiles of the classes in `sel` (bit t*5+p), up to `limit` elements per class
static void batch_tiles(gbfem_batch b, unsigned sel, int limit, std::vector<DgBatchTile> &tiles) {
  tiles.clear();
  for (int p = 4; p >= 1; p--)  // heaviest classes first
    for (int t = 0; t < 2; t++) {
      if (!(sel & (1u << (t * 5 + p)))) continue;
      const int begin = b->cls_start[t][p][0], end = std::min(b->cls_start[t][p][1], begin + limit);
      const int v = t == 0 ? b->var_prism[p] : b->var_tet[p];
      const int per = t == 0 ? gbfem::DGB_THREADS / gbfem::dgb_prism_thr(p, v) : gbfem::dgb_tet_tile(v);
      for (int s = begin; s < end; s += per) {
        DgBatchTile T{};
        T.type = (unsigned char)t;
        T.p = (unsigned char)p;
        T.variant = (unsigned char)v;
        T.start = s;
        T.count = std::min(per, end - s);
        tiles.push_back(T);
      }
    }
}

static gbfem::DgBatchArgs batch_args(gbfem_batch b) {
  gbfem::DgBatchArgs a;
  a.tiles = b->tiles.p;
  a.order = b->order.p;
  a.pX = b->pX.p;
  a.pA = b->pA.p;
  a.tX = b->tX.p;
  a.tA = b->tA.p;
  a.poff = b->poff.p;
  a.toff = b->toff.p;
  a.proff = b->proff.p;
  a.troff = b->troff.p;
  a.val = b->val.p;
  a.rhs = b->rhs.p;
  a.f = b->f;
  a.dword = b->dword;
  return a;
}

static int batch_upload_tiles(gbfem_batch b, const std::vector<DgBatchTile> &tiles) {
  if (b->tiles.alloc(std::max<size_t>(tiles.size(), 1)) < 0) return -1;
  if (!tiles.empty())
    GB_CUDA(cudaMemcpy(b->tiles.p, tiles.data(), tiles.size() * sizeof(DgBatchTile), cudaMemcpyHostToDevice));
  return 0;
}

static int batch_launch(gbfem_batch b, int ntiles) {
  GB_CUDA(cudaMemsetAsync(b->counter.p, 0, sizeof(int), b->stream));
  gbfem::dg_batch_kernel<<<b->grid, gbfem::DGB_THREADS, b->smem, b->stream>>>(ntiles, b->counter.p, b->tb,
                                                                             batch_args(b));
  GB_CUDA(cudaGetLastError());
  return 0;
}

// full tile list with the current variants, captured with its counter reset
static int batch_build(gbfem_batch b) {
  std::vector<DgBatchTile> tiles;
  batch_tiles(b, ~0u, 1 << 30, tiles);
  b->ntiles = (int)tiles.size();
  if (batch_upload_tiles(b, tiles) < 0) return -1;
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  cudaGraph_t g = nullptr;
  GB_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  const int rl = batch_launch(b, b->ntiles);
  const cudaError_t ec = cudaStreamEndCapture(b->stream, &g);
  if (rl < 0) return rl;
  GB_CUDA(ec);
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
  b->smem = gbfem::dgb_smem_bytes();
  int occ = 0;
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&b->e0) != cudaSuccess || cudaEventCreate(&b->e1) != cudaSuccess || b->counter.alloc(1) < 0 ||
      cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      cudaFuncSetAttribute(gbfem::dg_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b->smem) !=
          cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, gbfem::dg_batch_kernel, gbfem::DGB_THREADS, b->smem) !=
          cudaSuccess ||
      gbfem::dg_batch_tables(device, &b->tb) < 0) {
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    gbfem::set_error("batch creation failed");
    return -1;
  }
  b->grid = b->sms * std::max(occ, 1);
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
  b->order.release();
  b->tiles.release();
  cudaEventDestroy(b->e0);
  cudaEventDestroy(b->e1);
  cudaStreamDestroy(b->stream);
  delete b;
  return 0;
}

int gbfem_batch_set(gbfem_batch b, int np, const double *prism_xyz, const double *prism_A, const int *prism_p,
                    int nt, const double *tet_xyz, const double *tet_A, const int *tet_p, double f, long long *nval,
                    long long *nrhs) {
  GB_CHECK(b, "null batch");
  GB_CHECK(np >= 0 && nt >= 0 && np + nt > 0, "empty batch");
  GB_CHECK(np == 0 || (prism_xyz && prism_A && prism_p), "prism arrays missing");
  GB_CHECK(nt == 0 || (tet_xyz && tet_A && tet_p), "tetrahedron arrays missing");
  for (int e = 0; e < np; e++) GB_CHECK(prism_p[e] >= 1 && prism_p[e] <= 4, "degree must be 1..4");
  for (int e = 0; e < nt; e++) GB_CHECK(tet_p[e] >= 1 && tet_p[e] <= 4, "degree must be 1..4");
  GB_CUDA(cudaSetDevice(b->device));
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  b->np = np;
  b->nt = nt;
  b->f = f;
  b->pp.assign(prism_p, prism_p + np);
  b->tp.assign(tet_p, tet_p + nt);
  // default layout: prism blocks, then tet blocks, each ns x ns column-major
  std::vector<long long> poff(np), toff(nt);
  std::vector<int> proff(np), troff(nt);
  long long v = 0;
  int r = 0;
  for (int e = 0; e < np; e++) {
    const int ns = GB_DG_NS[prism_p[e]];
    poff[e] = v;
    proff[e] = r;
    v += (long long)ns * ns;
    r += ns;
  }
  for (int e = 0; e < nt; e++) {
    const int ns = gbfem::tet_ns(tet_p[e]);
    toff[e] = v;
    troff[e] = r;
    v += (long long)ns * ns;
    r += ns;
  }
  b->nval = v;
  b->nrhs = r;
  batch_order(b);
  auto up = [&](auto &buf, const auto *h, size_t n) -> int {
    if (buf.alloc(std::max<size_t>(n, 1)) < 0) return -1;
    if (n) GB_CUDA(cudaMemcpy(buf.p, h, n * sizeof(*h), cudaMemcpyHostToDevice));
    return 0;
  };
  if (up(b->pX, prism_xyz, 18 * (size_t)np) < 0 || up(b->pA, prism_A, 9 * (size_t)np) < 0 ||
      up(b->tX, tet_xyz, 12 * (size_t)nt) < 0 || up(b->tA, tet_A, 9 * (size_t)nt) < 0 ||
      up(b->poff, poff.data(), poff.size()) < 0 || up(b->toff, toff.data(), toff.size()) < 0 ||
      up(b->proff, proff.data(), proff.size()) < 0 || up(b->troff, troff.data(), troff.size()) < 0 ||
      up(b->order, b->order_h.data(), b->order_h.size()) < 0 || b->val.alloc((size_t)v) < 0 ||
      b->rhs.alloc((size_t)r) < 0)
    return -1;
  if (batch_build(b) < 0) return -1;
  if (nval) *nval = v;
  if (nrhs) *nrhs = r;
  return 0;
}

int gbfem_batch_set_layout(gbfem_batch b, const long long *val_off, const int *rhs_off, long long nval,
                           long long nrhs) {
  GB_CHECK(b && b->np + b->nt > 0, "batch not set");
  GB_CHECK(val_off && rhs_off, "null argument");
  const int n = b->np + b->nt;
  for (int e = 0; e < n; e++) {
    const int p = e < b->np ? b->pp[e] : b->tp[e - b->np];
    const long long ns = e < b->np ? GB_DG_NS[p] : gbfem::tet_ns(p);
    GB_CHECK(val_off[e] >= 0 && val_off[e] + ns * ns <= nval, "block offset out of range");
    GB_CHECK(rhs_off[e] >= 0 && rhs_off[e] + ns <= nrhs, "rhs offset out of range");
  }
  GB_CHECK(nrhs < (1ll << 31), "rhs too long");
  GB_CUDA(cudaSetDevice(b->device));
  if (b->poff.alloc(std::max(b->np, 1)) < 0 || b->toff.alloc(std::max(b->nt, 1)) < 0 ||
      b->proff.alloc(std::max(b->np, 1)) < 0 || b->troff.alloc(std::max(b->nt, 1)) < 0)
    return -1;
  if (b->np) {
    GB_CUDA(cudaMemcpy(b->poff.p, val_off, b->np * sizeof(long long), cudaMemcpyHostToDevice));
    GB_CUDA(cudaMemcpy(b->proff.p, rhs_off, b->np * sizeof(int), cudaMemcpyHostToDevice));
  }
  if (b->nt) {
    GB_CUDA(cudaMemcpy(b->toff.p, val_off + b->np, b->nt * sizeof(long long), cudaMemcpyHostToDevice));
    GB_CUDA(cudaMemcpy(b->troff.p, rhs_off + b->np, b->nt * sizeof(int), cudaMemcpyHostToDevice));
  }
  if (b->val.alloc((size_t)nval) < 0 || b->rhs.alloc((size_t)nrhs) < 0) return -1;
  GB_CUDA(cudaMemset(b->val.p, 0, (size_t)nval * sizeof(double)));
  GB_CUDA(cudaMemset(b->rhs.p, 0, (size_t)nrhs * sizeof(double)));
  b->nval = nval;
  b->nrhs = nrhs;
  return batch_build(b);
}

int gbfem_batch_set_variants(gbfem_batch b, const int *prism_v, const int *tet_v) {
  GB_CHECK(b, "null batch");
  for (int p = 1; p <= 4; p++) {
    GB_CHECK(!prism_v || (prism_v[p] >= 0 && prism_v[p] < gbfem::DGB_VARIANTS), "prism variant out of range");
    GB_CHECK(!tet_v || (tet_v[p] >= 0 && tet_v[p] < gbfem::DGB_TET_VARIANTS), "tetrahedron variant out of range");
  }
  for (int p = 1; p <= 4; p++) {
    if (prism_v) b->var_prism[p] = prism_v[p];
    if (tet_v) b->var_tet[p] = tet_v[p];
  }
  GB_CUDA(cudaSetDevice(b->device));
  return b->np + b->nt > 0 ? batch_build(b) : 0;
}

int gbfem_batch_set_arith(gbfem_batch b, int dword) {
  GB_CHECK(b, "null batch");
  GB_CHECK(dword == 0 || dword == 1, "arithmetic must be 0 (FP64) or 1 (double word)");
  b->dword = dword;
  GB_CUDA(cudaSetDevice(b->device));
  return b->np + b->nt > 0 ? batch_build(b) : 0;
}

int gbfem_batch_autotune(gbfem_batch b, int sample, int *prism_v, int *tet_v, double *ms) {
  GB_CHECK(b && b->np + b->nt > 0, "batch not set");
  GB_CUDA(cudaSetDevice(b->device));
  if (sample <= 0) sample = 16384;
  if (ms)
    for (int i = 0; i < 2 * 5 * 5; i++) ms[i] = -1.0;
  std::vector<DgBatchTile> tiles;
  for (int t = 0; t < 2; t++)
    for (int p = 1; p <= 4; p++) {
      if (b->cls_start[t][p][1] == b->cls_start[t][p][0]) continue;
      int *var = t == 0 ? b->var_prism : b->var_tet;
      const int nv = t == 0 ? gbfem::DGB_VARIANTS : gbfem::DGB_TET_VARIANTS;
      double best = 1e30;
      int bestv = var[p];
      for (int v = 0; v < nv; v++) {
        var[p] = v;
        batch_tiles(b, 1u << (t * 5 + p), sample, tiles);
        if (batch_upload_tiles(b, tiles) < 0) return -1;
        float tmin = 1e30f;
        for (int rep = 0; rep < 3; rep++) {
          cudaEventRecord(b->e0, b->stream);
          if (batch_launch(b, (int)tiles.size()) < 0) return -1;
          cudaEventRecord(b->e1, b->stream);
          GB_CUDA(cudaEventSynchronize(b->e1));
          float x = 0.f;
          cudaEventElapsedTime(&x, b->e0, b->e1);
          if (rep > 0) tmin = std::min(tmin, x);
        }
        if (ms) ms[(t * 5 + p) * 5 + v] = tmin;
        if (tmin < best) {
          best = tmin;
          bestv = v;
        }
      }
      var[p] = bestv;
    }
  for (int p = 0; p < 5; p++) {
    if (prism_v) prism_v[p] = b->var_prism[p];
    if (tet_v) tet_v[p] = b->var_tet[p];
  }
  return batch_build(b);
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
  GB_CUDA(cudaSetDevice(b->device));
  if (vals) GB_CUDA(cudaMemcpy(vals, b->val.p, (size_t)b->nval * sizeof(double), cudaMemcpyDeviceToHost));
  if (rhs) GB_CUDA(cudaMemcpy(rhs, b->rhs.p, (size_t)b->nrhs * sizeof(double), cudaMemcpyDeviceToHost));
  return 0;
}

}  // extern "C"
