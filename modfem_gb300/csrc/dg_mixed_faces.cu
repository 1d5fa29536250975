// DG face integrals between a prism and a tetrahedron, one CTA per owner
// element, FP64.  The reference's DG module is prism-only (apd_dg_prism); a
// mesh of prisms and tetrahedra together meets such faces where a prism's
// bottom or top triangle is a tetrahedron's face.  The form is the interior
// penalty form of the prism face kernel (dg_face.cuh: the reference's
// pdr_conv_diff_comp_fa_stiff_mat_app, pds_conv_diff_weakform_dg.c:232-1140)
// with each side's own basis:
//   rows i of the owner o, columns j of both sides t, per point q of the
//   triangle rule of degree max(p1, p2):
//     K[i][j] += a_q [ (f g_i + c Phi_i) Phi_j - f Phi_i g_j ],
//   Phi = s phi (s = +1 on the first neighbour, -1 on the second), g = (A^T
//   n) . grad phi = v . grad_xi phi with v = J^-1 A^T n (per point on the
//   prism side, constant on the affine tetrahedron), f = 1/2, c = pen
//   min(p1, p2) / sqrt(area), n the unit normal of the flat face pointing
//   away from the first neighbour's vertex centroid, a_q = |ds| w_q.
// Each side's local point comes from the face-vertex weights (barycentric)
// and that side's local vertex coordinates; prisms take the tensor basis in
// the reference's order, tetrahedra the complete basis (total degree, then
// a, then b descending).
//
// The kernel runs after the face kernels of the same-type faces, on the same
// stream: the owner's CTA is then the only writer of its diagonal block and
// adds each face's share to it directly; it writes the whole off-diagonal
// block (owner, neighbour), which no other face touches.  These faces lie on
// the interface between the two element regions only, so the kernel is
// sized for simplicity: every table in shared memory, 128 threads.

#include "dg_face.cuh"
#include "gbfem_internal.h"

namespace gbfem {

static __device__ const double mf_fq[GB_DG_PMAX][2][GB_DG_MAXNQF][3] = GB_DG_FQ_INIT;
static __device__ const int mf_nqf[GB_DG_PMAX + 1][2] = GB_DG_NQF_INIT;
static __device__ const unsigned char mf_pexp[GB_DG_PMAX][GB_DG_MAXNS][3] = GB_DG_EXP_INIT;

constexpr int MF_THREADS = 128;
constexpr int MF_NQ = 16;                 // points of the triangle rule of degree 4
constexpr int MF_NCOL = 2 * GB_DG_MAXNS;  // columns of both sides
constexpr int MF_TET_NS = 35;

__host__ __device__ constexpr int mf_ns(bool tet, int p) {
  return tet ? (p + 1) * (p + 2) * (p + 3) / 6 : (p == 1 ? 6 : p == 2 ? 18 : p == 3 ? 40 : 75);
}

template <int P, bool OTET>
__global__ void __launch_bounds__(MF_THREADS) dg_mixed_faces_kernel(
    int count, const int *__restrict__ ent_el, const int *__restrict__ mhf_ptr, const DgHalfFace *__restrict__ mhf,
    const int *__restrict__ el_p, const int *__restrict__ el_nodes6, const int *__restrict__ el_nodes4,
    const double *__restrict__ xyz, const double *__restrict__ k_el, const double *__restrict__ D_el, double pen,
    const long long *__restrict__ boff_diag, double *__restrict__ val, int *__restrict__ err) {
  constexpr int NS = mf_ns(OTET, P);
  __shared__ double sPhi[MF_NQ][MF_NCOL], sGam[MF_NQ][MF_NCOL];
  __shared__ double sFac[MF_NQ][2][30];  // monomial factors per point and side (dg_point_factors)
  __shared__ double sX[2][18], sA[2][9], sAw[MF_NQ], sN[3], sC;
  __shared__ unsigned char sTexp[MF_TET_NS][3];
  const int bi = blockIdx.x;
  if (bi >= count) return;
  const int e = ent_el[bi];
  const int tid = threadIdx.x;
  if (tid == 0) {
    int k = 0;
    for (int d = 0; d <= GB_DG_PMAX; d++)
      for (int a = d; a >= 0; a--)
        for (int b = d - a; b >= 0; b--, k++) {
          sTexp[k][0] = (unsigned char)a;
          sTexp[k][1] = (unsigned char)b;
          sTexp[k][2] = (unsigned char)(d - a - b);
        }
  }
  double *dblk = val + boff_diag[e];
  const int h0 = mhf_ptr[e], h1 = mhf_ptr[e + 1];
  for (int h = h0; h < h1; h++) {
    const DgHalfFace F = mhf[h];
    const int own2 = F.owner_is_2;
    // record side 0 is the first neighbour, side 1 the second; the owner is
    // of type OTET, the other side of the other type
    const bool tet1 = own2 ? !OTET : OTET;
    // (uniform over the CTA: every thread leaves together)
    if (F.el2 < 0 || F.nfv != 3 || el_p[own2 ? F.el2 : F.el1] != P) {
      if (tid == 0) atomicExch(err, 8);
      return;
    }
    const int p1 = el_p[F.el1], p2 = el_p[F.el2];
    const int ns1 = mf_ns(tet1, p1), ns2 = mf_ns(!tet1, p2), nsum = ns1 + ns2;
    const int pr = p2 > p1 ? p2 : p1;
    const int nq = mf_nqf[pr][0];
    __syncthreads();  // shared tables of the previous face are free
    for (int t = tid; t < 2 * 18 + 2 * 9; t += MF_THREADS) {
      if (t < 36) {
        const int s = t / 18, r = t % 18;
        const bool tet = s == 0 ? tet1 : !tet1;
        const int el = s ? F.el2 : F.el1;
        if (r < (tet ? 12 : 18))
          sX[s][r] = xyz[3 * (size_t)(tet ? el_nodes4[4 * (size_t)el + r / 3] : el_nodes6[6 * (size_t)el + r / 3]) +
                         r % 3];
      } else {
        const int u = t - 36, s = u / 9, r = u % 9;
        const int el = s ? F.el2 : F.el1;
        sA[s][r] = D_el ? D_el[9 * (size_t)el + r] : ((r % 4 == 0) ? (k_el ? k_el[el] : 1.0) : 0.0);
      }
    }
    __syncthreads();
    if (tid == 0) {
      // face vertices in face order from the first neighbour; the normal
      // points away from its vertex centroid
      const double *X1 = sX[0];
      const int nv1 = tet1 ? 4 : 6;
      v3 V[3], cen = {0, 0, 0}, vm = {0, 0, 0};
      for (int i = 0; i < 3; i++) {
        const int l = F.loc1[i];
        V[i] = {X1[3 * l], X1[3 * l + 1], X1[3 * l + 2]};
        vm = v3_fma(1.0 / 3.0, V[i], vm);
      }
      for (int k = 0; k < nv1; k++) cen = v3_fma(1.0 / nv1, v3{X1[3 * k], X1[3 * k + 1], X1[3 * k + 2]}, cen);
      const v3 ds = v3_cross(v3_sub(V[1], V[0]), v3_sub(V[2], V[0]));
      const double d = sqrt(v3_dot(ds, ds));
      v3 n = v3_scale(1.0 / d, ds);
      if (v3_dot(n, v3_sub(vm, cen)) < 0.0) n = v3_scale(-1.0, n);
      sN[0] = n.x;
      sN[1] = n.y;
      sN[2] = n.z;
      sC = pen * (p1 < p2 ? p1 : p2) / sqrt(0.5 * d);
      for (int q = 0; q < nq; q++) sAw[q] = d * mf_fq[pr - 1][0][q][2];
    }
    __syncthreads();
    // per (point, side): the point in that side's local coordinates, v and
    // the factor table
    for (int t = tid; t < 2 * nq; t += MF_THREADS) {
      const int q = t >> 1, sd = t & 1;
      const bool tet = sd == 0 ? tet1 : !tet1;
      const double *fq = mf_fq[pr - 1][0][q];
      const double w[3] = {1.0 - fq[0] - fq[1], fq[0], fq[1]};
      const unsigned char *loc = sd == 0 ? F.loc1 : F.loc2;
      v3 ev = {0, 0, 0};
#pragma unroll
      for (int i = 0; i < 3; i++) ev = v3_fma(w[i], tet ? tet_vertex_local(loc[i]) : prism_vertex_local(loc[i]), ev);
      const v3 n = {sN[0], sN[1], sN[2]};
      const v3 v = tet ? tet_face_v(sX[sd], sA[sd], n) : dg_face_v(sX[sd], ev, sA[sd], n);
      dg_point_factors(ev, v, sFac[q][sd]);
    }
    __syncthreads();
    for (int t = tid; t < nq * nsum; t += MF_THREADS) {
      const int q = t / nsum, j = t - q * nsum;
      const int side = j < ns1 ? 0 : 1, jj = side == 0 ? j : j - ns1;
      const bool tet = side == 0 ? tet1 : !tet1;
      const int ps = side == 0 ? p1 : p2;
      const unsigned char *ex = tet ? sTexp[jj] : mf_pexp[ps - 1][jj];
      double phi, g;
      dg_basis_from_factors(sFac[q][side], ex[0], ex[1], ex[2], phi, g);
      sPhi[q][j] = side == 1 ? -phi : phi;
      sGam[q][j] = g;
    }
    __syncthreads();
    const double fac = 0.5, cp = sC;
    const int own_lo = own2 ? ns1 : 0;
    // the face's share of the diagonal block, entry i + NS j
    for (int k = tid; k < NS * NS; k += MF_THREADS) {
      const int i = k % NS + own_lo, j = k / NS + own_lo;
      double s = 0.0;
      for (int q = 0; q < nq; q++)
        s = fma(sAw[q], fma(fma(fac, sGam[q][i], cp * sPhi[q][i]), sPhi[q][j], -fac * sPhi[q][i] * sGam[q][j]), s);
      dblk[k] += s;
    }
    // block (owner, neighbour): NS x ns_nb, column-major, leading dimension NS
    const int nb_lo = own2 ? 0 : ns1, ns_nb = own2 ? ns1 : ns2;
    double *blk = val + F.blk;
    for (int k = tid; k < NS * ns_nb; k += MF_THREADS) {
      const int i = k % NS + own_lo, j = k / NS + nb_lo;
      double s = 0.0;
      for (int q = 0; q < nq; q++)
        s = fma(sAw[q], fma(fma(fac, sGam[q][i], cp * sPhi[q][i]), sPhi[q][j], -fac * sPhi[q][i] * sGam[q][j]), s);
      blk[k] = s;
    }
  }
}

int launch_dg_mixed_faces(cudaStream_t st, int cls, int count, const int *ent_el, const int *mhf_ptr,
                          const DgHalfFace *mhf, const int *el_p, const int *el_nodes6, const int *el_nodes4,
                          const double *xyz, const double *k_el, const double *D_el, double pen,
                          const long long *boff_diag, double *val, int *err) {
  if (count <= 0) return 0;
  GB_CHECK(cls >= 1 && cls <= 2 * GB_DG_PMAX, "DG element class must be 1..8");
#define GB_MF_LAUNCH(PP, TT)                                                                                   \
  dg_mixed_faces_kernel<PP, TT><<<count, MF_THREADS, 0, st>>>(count, ent_el, mhf_ptr, mhf, el_p, el_nodes6,  \
                                                              el_nodes4, xyz, k_el, D_el, pen, boff_diag, val, \
                                                              err)
  switch (cls) {
    case 1: GB_MF_LAUNCH(1, false); break;
    case 2: GB_MF_LAUNCH(2, false); break;
    case 3: GB_MF_LAUNCH(3, false); break;
    case 4: GB_MF_LAUNCH(4, false); break;
    case 5: GB_MF_LAUNCH(1, true); break;
    case 6: GB_MF_LAUNCH(2, true); break;
    case 7: GB_MF_LAUNCH(3, true); break;
    default: GB_MF_LAUNCH(4, true); break;
  }
#undef GB_MF_LAUNCH
  GB_CUDA(cudaGetLastError());
  return 1;
}

}  // namespace gbfem
