// Host-side instantiation of the element math the CUDA kernels use, so the
// CPU test suite can check it against the oracle without a GPU.  Build with
// -Xcompiler -ffp-contract=off: the double-word operations rely on every
// float operation being rounded on its own.
#include "../../modfem_gb300/csrc/prism_dw.cuh"

extern "C" void host_prism_std_element(const double *X18, double k, double f, double *K21, double *R6) {
  gbfem::v3 X[6];
  for (int i = 0; i < 6; i++) X[i] = {X18[3 * i], X18[3 * i + 1], X18[3 * i + 2]};
  double K[21], R[6];
  gbfem::prism_std_element(X, k, f, K, R);
  for (int i = 0; i < 21; i++) K21[i] = K[i];
  for (int i = 0; i < 6; i++) R6[i] = R[i];
}

extern "C" void host_prism_std_element_dw(const double *X18, double k, double f, double *K21, double *R6) {
  gbfem::v3 X[6];
  for (int i = 0; i < 6; i++) X[i] = {X18[3 * i], X18[3 * i + 1], X18[3 * i + 2]};
  float2 slots[gbfem::kPrismDwSlots];
  const gbfem::DwSlots sl{slots, 1};
  gbfem::prism_std_element_dw(X, k, f, sl);
  constexpr gbfem::DwPairCodes codes = gbfem::dw_pair_codes();
  for (int k = 0; k < 21; k++) {
    const int c0 = codes.c[2 * k], u = (c0 >> 8) & 0xFF;  // u + 6 w, u <= w
    K21[gbfem::packed_index(u % 6, u / 6)] = gbfem::prism_dw_entry(sl, c0, codes.c[2 * k + 1]);
  }
  for (int w = 0; w < 6; w++) R6[w] = gbfem::prism_dw_load(sl, w);
}

// double-word conversions, both directions
extern "C" void host_dw_roundtrip(const double *x, int n, float *hl, double *back) {
  for (int i = 0; i < n; i++) {
    const gbfem::dw d = gbfem::dw_from_double(x[i]);
    hl[2 * i] = d.h;
    hl[2 * i + 1] = d.l;
    back[i] = gbfem::dw_to_double(d);
  }
}
