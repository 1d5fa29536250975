// Host-side instantiation of the DG face math of the CUDA face kernel: the
// full face matrix composed from the per-owner row form (each side's rows
// against both sides' columns), for comparison with the oracle on the CPU.
#include "../../modfem_gb300/csrc/dg_face.cuh"

using namespace gbfem;

// sm: (ns1+ns2)^2 column-major (entry row + n col), rhs: ns1+ns2.
extern "C" int host_dg_face(int ftype, const double *X1, const int *loc1i, int p1, const double *A1, int side1,
                            const double *X2, const int *loc2i, int p2, const double *A2, double pen, double g,
                            double *sm, double *rhs) {
  const int nfv = ftype == 4 ? 4 : 3, ti = ftype == 4 ? 1 : 0;
  const bool interior = X2 != nullptr;
  const int ns1 = GB_DG_NS[p1], ns2 = interior ? GB_DG_NS[p2] : 0, n = ns1 + ns2;
  unsigned char loc1[4] = {0, 0, 0, 0}, loc2[4] = {0, 0, 0, 0};
  for (int i = 0; i < nfv; i++) {
    loc1[i] = (unsigned char)loc1i[i];
    if (interior) loc2[i] = (unsigned char)loc2i[i];
  }
  int pr = p1;
  if (interior && GB_DG_NQF[p2][ti] > GB_DG_NQF[p1][ti]) pr = p2;
  const int nq = GB_DG_NQF[pr][ti];
  v3 V[4];
  for (int i = 0; i < nfv; i++) V[i] = {X1[3 * loc1[i]], X1[3 * loc1[i] + 1], X1[3 * loc1[i] + 2]};
  const double hf = sqrt(dg_face_area(V, nfv));
  const double fac = interior ? 0.5 : 1.0;
  const double cpen = pen * (interior ? (p1 < p2 ? p1 : p2) : p1) / hf;
  for (int i = 0; i < n * n; i++) sm[i] = 0.0;
  for (int i = 0; i < n; i++) rhs[i] = 0.0;
  for (int q = 0; q < nq; q++) {
    const DgFacePoint P = dg_face_point(nfv, GB_DG_FQ[pr - 1][ti][q], X1, loc1, side1, A1, interior ? X2 : nullptr,
                                        loc2, A2);
    double L[150], M[150], Phi[150], Gam[150];
    for (int j = 0; j < n; j++) {
      const int side = j < ns1 ? 1 : 2, jj = j < ns1 ? j : j - ns1, p = side == 1 ? p1 : p2;
      const unsigned char *ex = GB_DG_EXP[p - 1][jj];
      dg_face_values(ex[0], ex[1], ex[2], side, side == 1 ? P.e1 : P.e2, side == 1 ? P.v1 : P.v2, P.a, fac, cpen,
                     L[j], M[j], Phi[j], Gam[j]);
    }
    for (int j = 0; j < n; j++)
      for (int i = 0; i < n; i++) sm[(size_t)j * n + i] = fma(L[i], Phi[j], fma(M[i], Gam[j], sm[(size_t)j * n + i]));
    if (!interior)
      for (int i = 0; i < n; i++) rhs[i] += g * L[i];
  }
  return n;
}
