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
#include "dword.cuh"
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
// The double-word form at p = 4 keeps 22 float-triple accumulators a thread
// at 256 threads (255 registers, one CTA of 8 warps per SM); 512 threads
// halve them (128 registers, 16 warps): 87 ms instead of 103 (92 at 384) for
// a 128k-prism mixed-degree mesh.  Other degrees as the FP64 form.
__host__ __device__ constexpr int dg_face_threads_dw(int p, int v) {
  return p == 4 ? (v == 0 ? 512 : 384) : dg_face_threads(p, v);
}

// LOW: the owner and all its neighbours have degree <= 3, so a face has at
// most 16 points and a neighbour at most 40 functions: the point tables
// shrink to 16 rows and NS + 40 columns (p = 3: 51 KB of shared memory
// instead of 92, four CTAs per SM instead of two).  Same operations in the
// same order: bit-identical results.
template <int P, int THR, bool LOW = false>
struct DgFaceDims {
  static constexpr int NS = P == 1 ? 6 : P == 2 ? 18 : P == 3 ? 40 : 75;
  static constexpr int THREADS = THR;
  static constexpr int NQ = LOW ? 16 : DGF_NQ;             // points of the largest face rule met
  static constexpr int NCOL = NS + (LOW ? 40 : GB_DG_MAXNS);  // own + neighbour columns
  static constexpr int PER = (NS * NS + THREADS - 1) / THREADS;
  // degree <= 3: the coordinates, tensors, point geometry and penalty of all
  // (up to 5) faces are prepared at once before the face loop (the long FP64
  // chains of the face points then run side by side instead of on a few
  // threads per face); degree 4 keeps one face at a time (shared memory)
  static constexpr bool ALLF = P <= 3;
  static constexpr int NFG = ALLF ? 5 : 1;
  static constexpr int SMEM_DOUBLES =
      2 * NQ * NS + 2 * NQ * NCOL + NFG * (36 + 18 + NQ * DGF_GEO + 1) + 2 * NQ * DGF_FAC;
};

// Double-word form (DW = true): the point tables hold float pairs
// (converted from the FP64 basis values) and each entry is a dot product of
// length 2 nq on the FP32 pipes: per product an exact TwoProd (with the cross
// terms of the low words), the high parts summed by TwoSum, every rounding
// error collected in a float and folded back every four points.  The error
// stays of order u^2 = 2^-48 of the summed magnitudes, against the FP64
// kernel's 2 nq FP64 FMAs per entry at 1/64 of the FP32 issue rate
// (accumulator: DwAcc, dword.cuh).

template <int P, int THR, bool DW, bool LOW>
__global__ void __launch_bounds__(THR) dg_prism_faces_kernel(
    int count, const int *__restrict__ ent_el, const int *__restrict__ hf_ptr, const DgHalfFace *__restrict__ hf,
    const int *__restrict__ el_p, const int *__restrict__ el_nodes, const double *__restrict__ xyz,
    const double *__restrict__ k_el, const double *__restrict__ D_el, double pen, double gval,
    const long long *__restrict__ boff_diag, const int *__restrict__ roff, double *__restrict__ val,
    double *__restrict__ rhs) {
  using Dm = DgFaceDims<P, THR, LOW>;
  constexpr int NS = Dm::NS, NCOL = Dm::NCOL, DGF_THREADS = Dm::THREADS, NQ = Dm::NQ;
  static_assert(DGF_THREADS >= 54 && DGF_THREADS - 1 >= NQ, "loader and penalty threads");
  extern __shared__ double smem[];
  double *sL = smem;                       // [NQ][NS]   owner rows
  double *sM = sL + NQ * NS;               // [NQ][NS]
  double *sPhi = sM + NQ * NS;             // [NQ][NCOL] columns, side 1 then side 2
  double *sGam = sPhi + NQ * NCOL;         // [NQ][NCOL]
  constexpr int NFG = Dm::NFG;
  double *sX0 = sGam + NQ * NCOL;              // [NFG][2][18] vertex coordinates of both sides
  double *sA0 = sX0 + NFG * 36;                // [NFG][2][9] coefficient tensors
  double *sGeo0 = sA0 + NFG * 18;              // [NFG][NQ][DGF_GEO]
  double *sFac = sGeo0 + NFG * NQ * DGF_GEO;   // [NQ][2][DGF_FAC]
  double *sPen0 = sFac + 2 * NQ * DGF_FAC;     // [NFG] penalty / sqrt(face area)
  const int bi = blockIdx.x;
  if (bi >= count) return;
  const int e = ent_el[bi];
  const int tid = threadIdx.x;
  double acc[Dm::PER];
  DwAcc dacc[DW ? Dm::PER : 1];
#pragma unroll
  for (int m = 0; m < Dm::PER; m++) acc[m] = 0.0;
#pragma unroll
  for (int m = 0; m < (DW ? Dm::PER : 1); m++) dacc[m] = DwAcc{0.0f, 0.0f, 0.0f};
  double racc = 0.0;
  // p = 4 double word: register tiles of block entries (dwacc_face_tile):
  // the diagonal share in 3 x 5 tiles (375 of them, one a thread), kept over
  // the faces; the off-diagonal blocks in 3 x 3 tiles
  constexpr bool TILED = DW && P == 4;
  constexpr int DTI = 3, DTJ = 5, NDI = NS / DTI, NDJ = NS / DTJ, OTI = 3, OTJ = 3, NOI = NS / OTI;
  static_assert(!TILED || (NS % DTI == 0 && NS % DTJ == 0 && NS % OTI == 0 && NDI * NDJ <= DGF_THREADS),
                "tiles of the p = 4 diagonal block");
  DwAcc dtile[TILED ? DTI : 1][TILED ? DTJ : 1];
#pragma unroll
  for (int x = 0; x < (TILED ? DTI : 1); x++)
#pragma unroll
    for (int y = 0; y < (TILED ? DTJ : 1); y++) dtile[x][y] = DwAcc{0.0f, 0.0f, 0.0f};
  const int dti = tid % NDI, dtj = tid / NDI;  // this thread's diagonal tile (tid < NDI NDJ)
  float2 *fL = reinterpret_cast<float2 *>(sL), *fM = reinterpret_cast<float2 *>(sM);
  float2 *fPhi = reinterpret_cast<float2 *>(sPhi), *fGam = reinterpret_cast<float2 *>(sGam);
  const int h0 = hf_ptr[e], h1 = hf_ptr[e + 1];
  // the point rule of a face: the larger of its two sides' rules
  auto face_rule = [&](const DgHalfFace &F, int &pr, int &ti) {
    const bool interior = F.el2 >= 0;
    const int p1 = el_p[F.el1], p2 = interior ? el_p[F.el2] : 1;
    ti = F.nfv == 4 ? 1 : 0;
    pr = p1;
    if (interior && d_dg_nqf[p2][ti] > d_dg_nqf[p1][ti]) pr = p2;
  };
  auto face_geometry = [&](const DgHalfFace &F, int q, const double *X, const double *A, double *G) {
    int pr, ti;
    face_rule(F, pr, ti);
    const bool interior = F.el2 >= 0;
    const DgFacePoint Pq = dg_face_point(F.nfv, d_dg_fq[pr - 1][ti][q], X, F.loc1, F.side1, A,
                                         interior ? X + 18 : nullptr, F.loc2, A + 9);
    G[0] = Pq.e1.x; G[1] = Pq.e1.y; G[2] = Pq.e1.z;
    G[3] = Pq.e2.x; G[4] = Pq.e2.y; G[5] = Pq.e2.z;
    G[6] = Pq.v1.x; G[7] = Pq.v1.y; G[8] = Pq.v1.z;
    G[9] = Pq.v2.x; G[10] = Pq.v2.y; G[11] = Pq.v2.z;
    G[12] = Pq.a;
  };
  auto face_penalty = [&](const DgHalfFace &F, const double *X) {
    const bool interior = F.el2 >= 0;
    const int p1 = el_p[F.el1], p2 = interior ? el_p[F.el2] : 1;
    v3 V[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const int l = i < F.nfv ? F.loc1[i] : 0;
      V[i] = {X[3 * l], X[3 * l + 1], X[3 * l + 2]};
    }
    const int pp = interior ? (p1 < p2 ? p1 : p2) : p1;
    return pen * pp / sqrt(dg_face_area(V, F.nfv));
  };
  auto load_face = [&](const DgHalfFace &F, int c, double *X, double *A) {  // c in [0, 54)
    const bool interior = F.el2 >= 0;
    if (c < 36) {
      const int s = c / 18, r = c % 18;
      if (s == 0 || interior) {
        const int el = s ? F.el2 : F.el1;
        X[c] = xyz[3 * (size_t)el_nodes[6 * (size_t)el + r / 3] + r % 3];
      }
    } else {
      const int t = c - 36, s = t / 9, r = t % 9;
      if (s == 0 || interior) {
        const int el = s ? F.el2 : F.el1;
        A[t] = D_el ? D_el[9 * (size_t)el + r] : ((r % 4 == 0) ? (k_el ? k_el[el] : 1.0) : 0.0);
      }
    }
  };
  const int nf = h1 - h0;
  const bool allf = Dm::ALLF && nf <= NFG;  // uniform over the CTA
  if (allf) {
    for (int t = tid; t < nf * 54; t += DGF_THREADS) {
      const int f = t / 54;
      load_face(hf[h0 + f], t % 54, sX0 + 36 * f, sA0 + 18 * f);
    }
    __syncthreads();
    for (int t = tid; t < nf * NQ; t += DGF_THREADS) {
      const int f = t / NQ, q = t % NQ;
      const DgHalfFace F = hf[h0 + f];
      int pr, ti;
      face_rule(F, pr, ti);
      if (q < d_dg_nqf[pr][ti]) face_geometry(F, q, sX0 + 36 * f, sA0 + 18 * f, sGeo0 + (f * NQ + q) * DGF_GEO);
    }
    for (int f = tid; f < nf; f += DGF_THREADS) sPen0[f] = face_penalty(hf[h0 + f], sX0 + 36 * f);
  }
  for (int h = h0; h < h1; h++) {
    const DgHalfFace F = hf[h];
    const bool interior = F.el2 >= 0;
    const int own2 = F.owner_is_2;
    const int p1 = el_p[F.el1], p2 = interior ? el_p[F.el2] : 1;
    const int ns1 = d_dg_ns[p1], ns2 = interior ? d_dg_ns[p2] : 0;
    int pr, ti;
    face_rule(F, pr, ti);
    const int nq = d_dg_nqf[pr][ti];
    const int fo = allf ? h - h0 : 0;
    double *sX = sX0 + 36 * fo, *sA = sA0 + 18 * fo, *sGeo = sGeo0 + fo * NQ * DGF_GEO, *sPen = sPen0 + fo;
    __syncthreads();  // shared arrays of the previous face are free (and the prepared faces written)
    if (!allf) {  // this face only
      if (tid < 54) load_face(F, tid, sX, sA);
      __syncthreads();
      if (tid < nq) {
        face_geometry(F, tid, sX, sA, sGeo + tid * DGF_GEO);
      } else if (tid == DGF_THREADS - 1) {
        sPen[0] = face_penalty(F, sX);
      }
      __syncthreads();
    }
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
      const double Phi = __longlong_as_double(__double_as_longlong(phi) ^ (side == 2 ? (long long)1 << 63 : 0));
      if (DW) {
        fPhi[q * NCOL + j] = dw_f2(Phi);
        fGam[q * NCOL + j] = dw_f2(g);
      } else {
        sPhi[q * NCOL + j] = Phi;
        sGam[q * NCOL + j] = g;
      }
      if ((side == 2) == (own2 != 0)) {
        const double *G = sGeo + q * DGF_GEO;
        const double L = fma(G[13], g, G[14] * phi), M = G[15] * phi;
        if (DW) {
          fL[q * NS + jj] = dw_f2(L);
          fM[q * NS + jj] = dw_f2(M);
        } else {
          sL[q * NS + jj] = L;
          sM[q * NS + jj] = M;
        }
      }
    }
    __syncthreads();
    // the face's share of the diagonal block: entry k = i + NS j
    const int own_lo = own2 ? ns1 : 0;
    if (TILED) {
      if (tid < NDI * NDJ)
        dwacc_face_tile<NS, (TILED ? DTI : 1), (TILED ? DTJ : 1)>(dtile, fL, fM, fPhi, fGam, nq, NCOL, dti * DTI,
                                                                 dtj * DTJ, NS, own_lo);
    } else if (DW) {
      dwacc_face_block<NS, THR, (DW ? Dm::PER : 1)>(dacc, fL, fM, fPhi, fGam, nq, NCOL, tid, NS * NS, own_lo);
    } else {
#pragma unroll
      for (int m = 0; m < Dm::PER; m++) {
        const int k = tid + m * DGF_THREADS;
        if (k < NS * NS) {
          const int i = k % NS, j = k / NS + own_lo;
          double a = acc[m];
          for (int q = 0; q < nq; q++)
            a = fma(sL[q * NS + i], sPhi[q * NCOL + j], fma(sM[q * NS + i], sGam[q * NCOL + j], a));
          acc[m] = a;
        }
      }
    }
    if (interior) {
      // block (e, neighbour): NS x ns_nb, column-major, leading dimension NS
      const int nb_lo = own2 ? 0 : ns1, ns_nb = own2 ? ns1 : ns2;
      double *blk = val + F.blk;
      if (TILED) {
        const int noj = (ns_nb + OTJ - 1) / OTJ;
        for (int t = tid; t < NOI * noj; t += DGF_THREADS) {
          const int oi = t % NOI, oj = t / NOI;
          DwAcc o[TILED ? OTI : 1][TILED ? OTJ : 1];
#pragma unroll
          for (int x = 0; x < (TILED ? OTI : 1); x++)
#pragma unroll
            for (int y = 0; y < (TILED ? OTJ : 1); y++) o[x][y] = DwAcc{0.0f, 0.0f, 0.0f};
          dwacc_face_tile<NS, (TILED ? OTI : 1), (TILED ? OTJ : 1)>(o, fL, fM, fPhi, fGam, nq, NCOL, oi * OTI,
                                                                   oj * OTJ, ns_nb, nb_lo);
#pragma unroll
          for (int x = 0; x < (TILED ? OTI : 1); x++)
#pragma unroll
            for (int y = 0; y < (TILED ? OTJ : 1); y++) {
              const int j = oj * OTJ + y;
              if (j < ns_nb) blk[oi * OTI + x + (size_t)NS * j] = dwacc_value(o[x][y]);
            }
        }
      } else if (DW) {
        constexpr int PB = DW ? Dm::PER : 1;
        for (int k0 = tid; k0 < NS * ns_nb; k0 += PB * DGF_THREADS) {
          DwAcc a[PB];
#pragma unroll
          for (int m = 0; m < PB; m++) a[m] = DwAcc{0.0f, 0.0f, 0.0f};
          dwacc_face_block<NS, THR, PB>(a, fL, fM, fPhi, fGam, nq, NCOL, k0, NS * ns_nb, nb_lo);
#pragma unroll
          for (int m = 0; m < PB; m++)
            if (k0 + m * DGF_THREADS < NS * ns_nb) blk[k0 + m * DGF_THREADS] = dwacc_value(a[m]);
        }
      } else {
        for (int k = tid; k < NS * ns_nb; k += DGF_THREADS) {
          const int i = k % NS, j = k / NS + nb_lo;
          double a = 0.0;
          for (int q = 0; q < nq; q++)
            a = fma(sL[q * NS + i], sPhi[q * NCOL + j], fma(sM[q * NS + i], sGam[q * NCOL + j], a));
          blk[k] = a;
        }
      }
    } else if (tid < NS) {
      double s = 0.0;
      for (int q = 0; q < nq; q++) {
        if (DW) {
          const float2 v = fL[q * NS + tid];
          s += dw_to_double(dw(v.x, v.y));
        } else {
          s += sL[q * NS + tid];
        }
      }
      racc = fma(gval, s, racc);
    }
  }
  if (h1 == h0) return;
  double *dblk = val + boff_diag[e];
  if (TILED) {
    if (tid < NDI * NDJ) {
#pragma unroll
      for (int x = 0; x < (TILED ? DTI : 1); x++)
#pragma unroll
        for (int y = 0; y < (TILED ? DTJ : 1); y++)
          dblk[dti * DTI + x + (size_t)NS * (dtj * DTJ + y)] += dwacc_value(dtile[x][y]);
    }
  } else {
#pragma unroll
    for (int m = 0; m < Dm::PER; m++) {
      const int k = tid + m * DGF_THREADS;
      if (k < NS * NS) dblk[k] += DW ? dwacc_value(dacc[DW ? m : 0]) : acc[m];
    }
  }
  if (tid < NS) rhs[roff[e] + tid] += racc;
}

int launch_dg_prism_faces(cudaStream_t st, int p, int count, const int *ent_el, const int *hf_ptr,
                          const DgHalfFace *hf, const int *el_p, const int *el_nodes, const double *xyz,
                          const double *k_el, const double *D_el, double pen, double g, const long long *boff_diag,
                          const int *roff, double *val, double *rhs, int variant, bool dword, bool low) {
  if (count <= 0) return 0;
  GB_CHECK(p >= 1 && p <= GB_DG_PMAX, "DG degree must be 1..4");
  GB_CHECK(variant >= 0 && variant < DG_FACE_VARIANTS, "face kernel variant out of range");
#define GB_DGF_LAUNCH(PP, VV, WW, LL)                                                                          \
  {                                                                                                             \
    constexpr int T_ = WW ? dg_face_threads_dw(PP, VV) : dg_face_threads(PP, VV);                               \
    const size_t smem = sizeof(double) * DgFaceDims<PP, T_, LL>::SMEM_DOUBLES;                                  \
    GB_CUDA(cudaFuncSetAttribute(dg_prism_faces_kernel<PP, T_, WW, LL>,                                        \
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));                      \
    dg_prism_faces_kernel<PP, T_, WW, LL><<<count, T_, smem, st>>>(count, ent_el, hf_ptr, hf, el_p, el_nodes,   \
                                                                   xyz, k_el, D_el, pen, g, boff_diag, roff,    \
                                                                   val, rhs);                                   \
  }
#define GB_DGF_W(PP, LL)                                 \
  if (dword) {                                           \
    if (variant == 0) GB_DGF_LAUNCH(PP, 0, true, LL)     \
    else GB_DGF_LAUNCH(PP, 1, true, LL)                  \
  } else {                                               \
    if (variant == 0) GB_DGF_LAUNCH(PP, 0, false, LL)    \
    else GB_DGF_LAUNCH(PP, 1, false, LL)                 \
  }
#define GB_DGF_P(PP)        \
  if (low) GB_DGF_W(PP, true) \
  else GB_DGF_W(PP, false)
  GB_CHECK(!low || p <= 3, "the compact face tables need degrees <= 3");
  switch (p) {
    case 1: GB_DGF_P(1); break;
    case 2: GB_DGF_P(2); break;
    case 3: GB_DGF_P(3); break;
    default: GB_DGF_W(4, false); break;
  }
#undef GB_DGF_P
#undef GB_DGF_W
#undef GB_DGF_LAUNCH
  GB_CUDA(cudaGetLastError());
  return 1;
}

}  // namespace gbfem
