// DG tetrahedron face integrals on the device, one CTA per owner element,
// FP64.  The reference's DG module is prism-only (apd_dg_prism); this is the
// interior-penalty form of its weak form (pds_conv_diff_weakform_dg.c:
// 232-1140) with the algebra of the prism face kernel (dg_face.cuh,
// dg_faces.cu) on affine tetrahedra:
//   rows i of e (side s_i), columns j of both sides (side s_j), per point q
//   of the face rule: a_q [ s_j phi_j (f g_i + s_i c phi_i) - s_i f phi_i g_j ],
// g = (A^T n) . grad phi = v . grad_xi phi with v = J^-1 A^T n constant per
// side (affine map), f = 1/2 inside and 1 on the Dirichlet boundary,
// c = pen min(p1, p2) / sqrt(area) (pen p1 / sqrt(area) on the boundary),
// n the unit normal out of the first neighbour, a_q = |ds| w_q.  The face
// rule is the triangle rule of the prism kernel for max(p1, p2) (order
// 2 max(p1, p2)); the point in each neighbour's reference coordinates comes
// through the face-vertex weights.  Basis: complete monomials xi^a eta^b
// zeta^c, a + b + c <= p, ordered by total degree, then a, then b
// descending.  Ownership as in the prism kernel: e's CTA writes e's rows of
// the off-diagonal blocks and adds its share of the diagonal block once.

#include "dg_face.cuh"
#include "dword.cuh"
#include "gbfem_internal.h"

namespace gbfem {

static __device__ const double tt_fq[GB_DG_PMAX][2][GB_DG_MAXNQF][3] = GB_DG_FQ_INIT;
static __device__ const int tt_nqf[GB_DG_PMAX + 1][2] = GB_DG_NQF_INIT;

// threads per CTA by the owner's degree: the diagonal share has NS^2 = 16,
// 100, 400, 1225 entries
__host__ __device__ constexpr int tt_threads(int p) { return p == 1 ? 32 : p == 2 ? 64 : p == 3 ? 128 : 256; }
constexpr int TT_NQ = 16;   // points of the triangle rule for p = 4
constexpr int TT_NS = 35;   // functions for p = 4
constexpr int TT_NCOL = 2 * TT_NS;

__host__ __device__ constexpr int tt_ns(int p) { return (p + 1) * (p + 2) * (p + 3) / 6; }

// DW: the point tables as double words and every entry summed by exact
// products and TwoSum chains (DwAcc, dword.cuh), as in the prism face kernel.
template <int P, bool DW, int TT_THREADS = tt_threads(P)>
__global__ void __launch_bounds__(TT_THREADS) dg_tet_faces_kernel(
    int count, const int *__restrict__ ent_el, const int *__restrict__ hf_ptr, const DgHalfFace *__restrict__ hf,
    const int *__restrict__ el_p, const int *__restrict__ el_nodes, const double *__restrict__ xyz,
    const double *__restrict__ k_el, const double *__restrict__ D_el, double pen, double gval,
    const long long *__restrict__ boff_diag, const int *__restrict__ roff, double *__restrict__ val,
    double *__restrict__ rhs) {
  constexpr int NS = tt_ns(P), PER = (NS * NS + TT_THREADS - 1) / TT_THREADS;
  __shared__ double sL[TT_NQ][NS], sM[TT_NQ][NS];
  __shared__ double sPhi[TT_NQ][TT_NCOL], sGam[TT_NQ][TT_NCOL];
  __shared__ double sX[2][12], sA[2][9], sV[2][3], sAw[TT_NQ], sC[2];  // sC: |ds|, penalty factor
  __shared__ unsigned char sExp[TT_NS][3];
  __shared__ double sFac[TT_NQ][2][30];  // monomial factors per point and side (dg_point_factors)
  const int bi = blockIdx.x;
  if (bi >= count) return;
  const int e = ent_el[bi];
  const int tid = threadIdx.x;
  if (tid == 0) {
    int k = 0;
    for (int d = 0; d <= GB_DG_PMAX; d++)
      for (int a = d; a >= 0; a--)
        for (int b = d - a; b >= 0; b--, k++) {
          sExp[k][0] = (unsigned char)a;
          sExp[k][1] = (unsigned char)b;
          sExp[k][2] = (unsigned char)(d - a - b);
        }
  }
  double acc[PER];
  DwAcc dacc[DW ? PER : 1];
#pragma unroll
  for (int m = 0; m < PER; m++) acc[m] = 0.0;
#pragma unroll
  for (int m = 0; m < (DW ? PER : 1); m++) dacc[m] = DwAcc{0.0f, 0.0f, 0.0f};
  double racc = 0.0;
  float2 *fL = reinterpret_cast<float2 *>(&sL[0][0]), *fM = reinterpret_cast<float2 *>(&sM[0][0]);
  float2 *fPhi = reinterpret_cast<float2 *>(&sPhi[0][0]), *fGam = reinterpret_cast<float2 *>(&sGam[0][0]);
  const int h0 = hf_ptr[e], h1 = hf_ptr[e + 1];
  for (int h = h0; h < h1; h++) {
    const DgHalfFace F = hf[h];
    const bool interior = F.el2 >= 0;
    const int own2 = F.owner_is_2;
    const int p1 = el_p[F.el1], p2 = interior ? el_p[F.el2] : 1;
    const int ns1 = tt_ns(p1), ns2 = interior ? tt_ns(p2) : 0;
    const int pr = interior && p2 > p1 ? p2 : p1;
    const int nq = tt_nqf[pr][0];
    __syncthreads();  // shared arrays of the previous face are free
    for (int t = tid; t < 42; t += TT_THREADS) {
      if (t < 24) {
        const int s = t / 12, r = t % 12;
        if (s == 0 || interior) {
          const int el = s ? F.el2 : F.el1;
          sX[s][r] = xyz[3 * (size_t)el_nodes[4 * (size_t)el + r / 3] + r % 3];
        }
      } else {
        const int u = t - 24, s = u / 9, r = u % 9;
        if (s == 0 || interior) {
          const int el = s ? F.el2 : F.el1;
          sA[s][r] = D_el ? D_el[9 * (size_t)el + r] : ((r % 4 == 0) ? (k_el ? k_el[el] : 1.0) : 0.0);
        }
      }
    }
    __syncthreads();
    if (tid < 2) {
      // face vertices in face order from the first neighbour; the normal
      // points away from its vertex off the face (local index side1)
      const double *X1 = sX[0];
      const int la = F.loc1[0], lb = F.loc1[1], lc = F.loc1[2];
      const v3 va = {X1[3 * la], X1[3 * la + 1], X1[3 * la + 2]};
      const v3 vb = {X1[3 * lb], X1[3 * lb + 1], X1[3 * lb + 2]};
      const v3 vc = {X1[3 * lc], X1[3 * lc + 1], X1[3 * lc + 2]};
      const v3 ds = v3_cross(v3_sub(vb, va), v3_sub(vc, va));
      const double d = sqrt(v3_dot(ds, ds));
      v3 n = v3_scale(1.0 / d, ds);
      const v3 vo = {X1[3 * F.side1], X1[3 * F.side1 + 1], X1[3 * F.side1 + 2]};
      if (v3_dot(n, v3_sub(vo, va)) > 0.0) n = v3_scale(-1.0, n);
      if (tid == 0) {
        const v3 v1 = tet_face_v(sX[0], sA[0], n);
        sV[0][0] = v1.x;
        sV[0][1] = v1.y;
        sV[0][2] = v1.z;
        sC[0] = d;
        const int pp = interior ? (p1 < p2 ? p1 : p2) : p1;
        sC[1] = pen * pp / sqrt(0.5 * d);
      } else if (interior) {
        const v3 v2 = tet_face_v(sX[1], sA[1], n);
        sV[1][0] = v2.x;
        sV[1][1] = v2.y;
        sV[1][2] = v2.z;
      }
    }
    __syncthreads();
    for (int q = tid; q < nq; q += TT_THREADS) sAw[q] = sC[0] * tt_fq[pr - 1][0][q][2];
    // per (point, side): the point in that side's reference coordinates and
    // the factor table x_k^m, m x_k^(m-1) v_k
    for (int t = tid; t < 2 * nq; t += TT_THREADS) {
      const int q = t >> 1, sd = t & 1;
      if (sd == 1 && !interior) continue;
      const double *fq = tt_fq[pr - 1][0][q];
      const double w[3] = {1.0 - fq[0] - fq[1], fq[0], fq[1]};
      const unsigned char *loc = sd == 0 ? F.loc1 : F.loc2;
      v3 ev = {0, 0, 0};
#pragma unroll
      for (int i = 0; i < 3; i++) ev = v3_fma(w[i], tet_vertex_local(loc[i]), ev);
      dg_point_factors(ev, v3{sV[sd][0], sV[sd][1], sV[sd][2]}, sFac[q][sd]);
    }
    const double fac = interior ? 0.5 : 1.0;
    const int nsum = ns1 + ns2;
    __syncthreads();
    for (int t = tid; t < nq * nsum; t += TT_THREADS) {
      const int q = t / nsum, j = t - q * nsum;
      const int side = j < ns1 ? 0 : 1, jj = side == 0 ? j : j - ns1;
      double phi, g;
      dg_basis_from_factors(sFac[q][side], sExp[jj][0], sExp[jj][1], sExp[jj][2], phi, g);
      const double Phi = side == 1 ? -phi : phi;
      if (DW) {
        fPhi[q * TT_NCOL + j] = dw_f2(Phi);
        fGam[q * TT_NCOL + j] = dw_f2(g);
      } else {
        sPhi[q][j] = Phi;
        sGam[q][j] = g;
      }
      if (side == own2) {
        const double aw = sAw[q], so = own2 ? -1.0 : 1.0;
        const double L = aw * fma(fac, g, so * sC[1] * phi), M = -so * fac * aw * phi;
        if (DW) {
          fL[q * NS + jj] = dw_f2(L);
          fM[q * NS + jj] = dw_f2(M);
        } else {
          sL[q][jj] = L;
          sM[q][jj] = M;
        }
      }
    }
    __syncthreads();
    // the face's share of the diagonal block: entry k = i + NS j
    const int own_lo = own2 ? ns1 : 0;
    if (DW) {
      dwacc_face_block<NS, TT_THREADS, (DW ? PER : 1)>(dacc, fL, fM, fPhi, fGam, nq, TT_NCOL, tid, NS * NS, own_lo);
    } else {
#pragma unroll
      for (int m = 0; m < PER; m++) {
        const int k = tid + m * TT_THREADS;
        if (k < NS * NS) {
          const int i = k % NS, j = k / NS + own_lo;
          double s = acc[m];
          for (int q = 0; q < nq; q++) s = fma(sL[q][i], sPhi[q][j], fma(sM[q][i], sGam[q][j], s));
          acc[m] = s;
        }
      }
    }
    if (interior) {
      // block (e, neighbour): NS x ns_nb, column-major, leading dimension NS
      const int nb_lo = own2 ? 0 : ns1, ns_nb = own2 ? ns1 : ns2;
      double *blk = val + F.blk;
      if (DW) {
        constexpr int PB = DW ? PER : 1;
        for (int k0 = tid; k0 < NS * ns_nb; k0 += PB * TT_THREADS) {
          DwAcc a[PB];
#pragma unroll
          for (int m = 0; m < PB; m++) a[m] = DwAcc{0.0f, 0.0f, 0.0f};
          dwacc_face_block<NS, TT_THREADS, PB>(a, fL, fM, fPhi, fGam, nq, TT_NCOL, k0, NS * ns_nb, nb_lo);
#pragma unroll
          for (int m = 0; m < PB; m++)
            if (k0 + m * TT_THREADS < NS * ns_nb) blk[k0 + m * TT_THREADS] = dwacc_value(a[m]);
        }
      } else {
        for (int k = tid; k < NS * ns_nb; k += TT_THREADS) {
          const int i = k % NS, j = k / NS + nb_lo;
          double s = 0.0;
          for (int q = 0; q < nq; q++) s = fma(sL[q][i], sPhi[q][j], fma(sM[q][i], sGam[q][j], s));
          blk[k] = s;
        }
      }
    } else if (tid < NS) {
      double s = 0.0;
      for (int q = 0; q < nq; q++) {
        if (DW) {
          const float2 v = fL[q * NS + tid];
          s += dw_to_double(dw(v.x, v.y));
        } else {
          s += sL[q][tid];
        }
      }
      racc = fma(gval, s, racc);
    }
  }
  if (h1 == h0) return;
  double *dblk = val + boff_diag[e];
#pragma unroll
  for (int m = 0; m < PER; m++) {
    const int k = tid + m * TT_THREADS;
    if (k < NS * NS) dblk[k] += DW ? dwacc_value(dacc[DW ? m : 0]) : acc[m];
  }
  if (tid < NS) rhs[roff[e] + tid] += racc;
}

int launch_dg_tet_faces(cudaStream_t st, int p, int count, const int *ent_el, const int *hf_ptr,
                        const DgHalfFace *hf, const int *el_p, const int *el_nodes, const double *xyz,
                        const double *k_el, const double *D_el, double pen, double g, const long long *boff_diag,
                        const int *roff, double *val, double *rhs, bool dword) {
  if (count <= 0) return 0;
  GB_CHECK(p >= 1 && p <= GB_DG_PMAX, "DG degree must be 1..4");
#define GB_TT_LAUNCH(PP)                                                                                        \
  if (dword)                                                                                                    \
    dg_tet_faces_kernel<PP, true><<<count, tt_threads(PP), 0, st>>>(count, ent_el, hf_ptr, hf, el_p, el_nodes,  \
                                                                    xyz, k_el, D_el, pen, g, boff_diag, roff,  \
                                                                    val, rhs);                                 \
  else                                                                                                          \
    dg_tet_faces_kernel<PP, false><<<count, tt_threads(PP), 0, st>>>(count, ent_el, hf_ptr, hf, el_p, el_nodes, \
                                                                     xyz, k_el, D_el, pen, g, boff_diag, roff, \
                                                                     val, rhs)
  switch (p) {
    case 1: GB_TT_LAUNCH(1); break;
    case 2: GB_TT_LAUNCH(2); break;
    case 3: GB_TT_LAUNCH(3); break;
    default: GB_TT_LAUNCH(4); break;
  }
#undef GB_TT_LAUNCH
  GB_CUDA(cudaGetLastError());
  return 1;
}

}  // namespace gbfem
