// DG prism face integrals on the device, one CTA per element (the owner of a
// block row), FP64.
//
// Reference: pdr_conv_diff_comp_fa_stiff_mat_app of the DG weak form
// (pds_conv_diff_weakform_dg.c:232-1140), assembled by lar_assemble_SM_and_LV_
// block (lsd_mkb/lad_block/las_block_intf.c:362-520).  The face math and the
// row form it is evaluated in are in dg_face.cuh.
//
// Ownership instead of atomics: the CTA of element e integrates, for every
// face of e, only the rows of e: the face's part of the diagonal block (e, e)
// (summed in registers over the faces and added once to the block the volume
// kernel wrote) and the whole off-diagonal block (e, neighbour), which no
// other face touches and which is written with plain coalesced stores.  Each
// entry of every block is therefore produced by exactly one thread, in a fixed
// order: the assembly is deterministic and the off-diagonal blocks need no
// clearing.  The price is that both neighbours evaluate the face basis of
// both sides (a few percent of the FP64 work; the block products dominate).

#include "dg_face.cuh"
#include "gbfem_internal.h"

namespace gbfem {

__device__ const double d_dg_fq[GB_DG_PMAX][2][GB_DG_MAXNQF][3] = GB_DG_FQ_INIT;
__device__ const unsigned char d_dg_exp[GB_DG_PMAX][GB_DG_MAXNS][3] = GB_DG_EXP_INIT;
__device__ const int d_dg_ns[GB_DG_PMAX + 1] = GB_DG_NS_INIT;
__device__ const int d_dg_nqf[GB_DG_PMAX + 1][2] = GB_DG_NQF_INIT;

constexpr int DGF_NQ = GB_DG_MAXNQF;  // points of the largest face rule
constexpr int DGF_GEO = 16;           // e1, e2, v1, v2, a, then the owner-row scales
constexpr int DGF_FAC = 30;           // monomial factors per point and side

// Threads per CTA per degree (variant 0 fills the thread slots of the
// NS x NS diagonal block evenly or nearly: 36 / 64, 324 / 384 = 2 x 192,
// 1600 / 1600 = 5 x 320, 5625 / 5632 = 22 x 256; the products are FP64-bound,
// so idle lanes are lost FP64 issue); the autotuner times the alternatives.
// Every variant sums each entry over the points in the same order.
constexpr int DG_FACE_VARIANTS = 2;
__host__ __device__ constexpr int dg_face_threads(int p, int v) {
  return p == 1 ? (v == 0 ? 64 : 128) : p == 2 ? (v == 0 ? 192 : 128) : p == 3 ? (v == 0 ? 320 : 160)
                                                                              : (v == 0 ? 256 : 384);
}

template <int P, int THR>
struct DgFaceDims {
  static constexpr int NS = P == 1 ? 6 : P == 2 ? 18 : P == 3 ? 40 : 75;
  static constexpr int THREADS = THR;
  static constexpr int NCOL = NS + GB_DG_MAXNS;  // own + neighbour columns
  static constexpr int PER = (NS * NS + THREADS - 1) / THREADS;
  static constexpr int SMEM_DOUBLES =
      2 * DGF_NQ * NS + 2 * DGF_NQ * NCOL + 36 + 18 + DGF_NQ * DGF_GEO + 2 * DGF_NQ * DGF_FAC + 1;
};

template <int P, int THR>
__global__ void __launch_bounds__(THR) dg_prism_faces_kernel(
    int count, const int *__restrict__ ent_el, const int *__restrict__ hf_ptr, const DgHalfFace *__restrict__ hf,
    const int *__restrict__ el_p, const int *__restrict__ el_nodes, const double *__restrict__ xyz,
    const double *__restrict__ k_el, const double *__restrict__ D_el, double pen, double gval,
    const long long *__restrict__ boff_diag, const int *__restrict__ roff, double *__restrict__ val,
    double *__restrict__ rhs) {
  using Dm = DgFaceDims<P, THR>;
  constexpr int NS = Dm::NS, NCOL = Dm::NCOL, DGF_THREADS = Dm::THREADS;
  static_assert(DGF_THREADS >= 54 && DGF_THREADS - 1 >= DGF_NQ, "loader and penalty threads");
  extern __shared__ double smem[];
  double *sL = smem;                       // [DGF_NQ][NS]   owner rows
  double *sM = sL + DGF_NQ * NS;           // [DGF_NQ][NS]
  double *sPhi = sM + DGF_NQ * NS;         // [DGF_NQ][NCOL] columns, side 1 then side 2
  double *sGam = sPhi + DGF_NQ * NCOL;     // [DGF_NQ][NCOL]
  double *sX = sGam + DGF_NQ * NCOL;       // [2][18] vertex coordinates of both sides
  double *sA = sX + 36;                    // [2][9] coefficient tensors
  double *sGeo = sA + 18;                  // [DGF_NQ][DGF_GEO]
  double *sFac = sGeo + DGF_NQ * DGF_GEO;  // [DGF_NQ][2][DGF_FAC]
  double *sPen = sFac + 2 * DGF_NQ * DGF_FAC;  // penalty / sqrt(face area)
  const int bi = blockIdx.x;
  if (bi >= count) return;
  const int e = ent_el[bi];
  const int tid = threadIdx.x;
  double acc[Dm::PER];
#pragma unroll
  for (int m = 0; m < Dm::PER; m++) acc[m] = 0.0;
  double racc = 0.0;
  const int h0 = hf_ptr[e], h1 = hf_ptr[e + 1];
  for (int h = h0; h < h1; h++) {
    const DgHalfFace F = hf[h];
    const bool interior = F.el2 >= 0;
    const int own2 = F.owner_is_2;
    const int p1 = el_p[F.el1], p2 = interior ? el_p[F.el2] : 1;
    const int ns1 = d_dg_ns[p1], ns2 = interior ? d_dg_ns[p2] : 0;
    const int ti = F.nfv == 4 ? 1 : 0;
    int pr = p1;
    if (interior && d_dg_nqf[p2][ti] > d_dg_nqf[p1][ti]) pr = p2;
    const int nq = d_dg_nqf[pr][ti];
    __syncthreads();  // shared arrays of the previous face are free
    if (tid < 36) {
      const int s = tid / 18, r = tid % 18;
      if (s == 0 || interior) {
        const int el = s ? F.el2 : F.el1;
        const int node = el_nodes[6 * (size_t)el + r / 3];
        sX[tid] = xyz[3 * (size_t)node + r % 3];
      }
    } else if (tid < 54) {
      const int t = tid - 36, s = t / 9, r = t % 9;
      if (s == 0 || interior) {
        const int el = s ? F.el2 : F.el1;
        sA[t] = D_el ? D_el[9 * (size_t)el + r] : ((r % 4 == 0) ? (k_el ? k_el[el] : 1.0) : 0.0);
      }
    }
    __syncthreads();
    if (tid < nq) {
      const DgFacePoint Pq = dg_face_point(F.nfv, d_dg_fq[pr - 1][ti][tid], sX, F.loc1, F.side1, sA,
                                           interior ? sX + 18 : nullptr, F.loc2, sA + 9);
      double *G = sGeo + tid * DGF_GEO;
      G[0] = Pq.e1.x; G[1] = Pq.e1.y; G[2] = Pq.e1.z;
      G[3] = Pq.e2.x; G[4] = Pq.e2.y; G[5] = Pq.e2.z;
      G[6] = Pq.v1.x; G[7] = Pq.v1.y; G[8] = Pq.v1.z;
      G[9] = Pq.v2.x; G[10] = Pq.v2.y; G[11] = Pq.v2.z;
      G[12] = Pq.a;
    } else if (tid == DGF_THREADS - 1) {
      v3 V[4];
#pragma unroll
      for (int i = 0; i < 4; i++) {
        const int l = i < F.nfv ? F.loc1[i] : 0;
        V[i] = {sX[3 * l], sX[3 * l + 1], sX[3 * l + 2]};
      }
      const int pp = interior ? (p1 < p2 ? p1 : p2) : p1;
      sPen[0] = pen * pp / sqrt(dg_face_area(V, F.nfv));
    }
    __syncthreads();
    const double fac = interior ? 0.5 : 1.0;
    const int nsum = ns1 + ns2;
    // monomial factors per (point, side); the owner-row scales per point:
    // L = alpha g + beta phi, M = gamma phi (alpha = f a, beta = s_o c a,
    // gamma = -s_o f a)
    for (int t = tid; t < 2 * nq; t += DGF_THREADS) {
      const int q = t >> 1, sd = t & 1;
      if (sd == 1 && !interior) continue;
      const double *G = sGeo + q * DGF_GEO;
      dg_point_factors(v3{G[3 * sd], G[3 * sd + 1], G[3 * sd + 2]}, v3{G[6 + 3 * sd], G[7 + 3 * sd], G[8 + 3 * sd]},
                       sFac + (2 * q + sd) * DGF_FAC);
      if (sd == 0) {
        const double aw = G[12], so = own2 ? -1.0 : 1.0;
        sGeo[q * DGF_GEO + 13] = fac * aw;
        sGeo[q * DGF_GEO + 14] = so * sPen[0] * aw;
        sGeo[q * DGF_GEO + 15] = -so * fac * aw;
      }
    }
    __syncthreads();
    for (int t = tid; t < nq * nsum; t += DGF_THREADS) {
      const int q = t / nsum, j = t - q * nsum;
      const int side = j < ns1 ? 1 : 2, jj = side == 1 ? j : j - ns1, p = side == 1 ? p1 : p2;
      const unsigned char *ex = d_dg_exp[p - 1][jj];
      double phi, g;
      dg_basis_from_factors(sFac + (2 * q + side - 1) * DGF_FAC, ex[0], ex[1], ex[2], phi, g);
      // Phi = s_t phi: the sign flip on the integer side, not the FP64 pipe
      sPhi[q * NCOL + j] = __longlong_as_double(__double_as_longlong(phi) ^ (side == 2 ? (long long)1 << 63 : 0));
      sGam[q * NCOL + j] = g;
      if ((side == 2) == (own2 != 0)) {
        const double *G = sGeo + q * DGF_GEO;
        sL[q * NS + jj] = fma(G[13], g, G[14] * phi);
        sM[q * NS + jj] = G[15] * phi;
      }
    }
    __syncthreads();
    // the face's share of the diagonal block: entry k = i + NS j
    const int own_lo = own2 ? ns1 : 0;
#pragma unroll
    for (int m = 0; m < Dm::PER; m++) {
      const int k = tid + m * DGF_THREADS;
      if (k < NS * NS) {
        const int i = k % NS, j = k / NS + own_lo;
        double a = acc[m];
        for (int q = 0; q < nq; q++) a = fma(sL[q * NS + i], sPhi[q * NCOL + j], fma(sM[q * NS + i], sGam[q * NCOL + j], a));
        acc[m] = a;
      }
    }
    if (interior) {
      // block (e, neighbour): NS x ns_nb, column-major, leading dimension NS
      const int nb_lo = own2 ? 0 : ns1, ns_nb = own2 ? ns1 : ns2;
      double *blk = val + F.blk;
      for (int k = tid; k < NS * ns_nb; k += DGF_THREADS) {
        const int i = k % NS, j = k / NS + nb_lo;
        double a = 0.0;
        for (int q = 0; q < nq; q++) a = fma(sL[q * NS + i], sPhi[q * NCOL + j], fma(sM[q * NS + i], sGam[q * NCOL + j], a));
        blk[k] = a;
      }
    } else if (tid < NS) {
      double s = 0.0;
      for (int q = 0; q < nq; q++) s += sL[q * NS + tid];
      racc = fma(gval, s, racc);
    }
  }
  if (h1 == h0) return;
  double *dblk = val + boff_diag[e];
#pragma unroll
  for (int m = 0; m < Dm::PER; m++) {
    const int k = tid + m * DGF_THREADS;
    if (k < NS * NS) dblk[k] += acc[m];
  }
  if (tid < NS) rhs[roff[e] + tid] += racc;
}

int launch_dg_prism_faces(cudaStream_t st, int p, int count, const int *ent_el, const int *hf_ptr,
                          const DgHalfFace *hf, const int *el_p, const int *el_nodes, const double *xyz,
                          const double *k_el, const double *D_el, double pen, double g, const long long *boff_diag,
                          const int *roff, double *val, double *rhs, int variant) {
  if (count <= 0) return 0;
  GB_CHECK(p >= 1 && p <= GB_DG_PMAX, "DG degree must be 1..4");
  GB_CHECK(variant >= 0 && variant < DG_FACE_VARIANTS, "face kernel variant out of range");
#define GB_DGF_LAUNCH(PP, VV)                                                                                   \
  {                                                                                                             \
    constexpr int T_ = dg_face_threads(PP, VV);                                                                 \
    const size_t smem = sizeof(double) * DgFaceDims<PP, T_>::SMEM_DOUBLES;                                      \
    GB_CUDA(cudaFuncSetAttribute(dg_prism_faces_kernel<PP, T_>, cudaFuncAttributeMaxDynamicSharedMemorySize,   \
                                 (int)smem));                                                                   \
    dg_prism_faces_kernel<PP, T_><<<count, T_, smem, st>>>(count, ent_el, hf_ptr, hf, el_p, el_nodes, xyz, k_el, \
                                                           D_el, pen, g, boff_diag, roff, val, rhs);            \
  }
#define GB_DGF_P(PP)                                     \
  if (variant == 0) GB_DGF_LAUNCH(PP, 0) else GB_DGF_LAUNCH(PP, 1)
  switch (p) {
    case 1: GB_DGF_P(1); break;
    case 2: GB_DGF_P(2); break;
    case 3: GB_DGF_P(3); break;
    default: GB_DGF_P(4); break;
  }
#undef GB_DGF_P
#undef GB_DGF_LAUNCH
  GB_CUDA(cudaGetLastError());
  return 1;
}

}  // namespace gbfem
