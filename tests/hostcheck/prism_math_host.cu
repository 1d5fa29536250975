// Host-side instantiation of the element math the CUDA kernels use, so the
// CPU test suite can check it against the oracle without a GPU.
#include "../../modfem_gb300/csrc/prism_std.cuh"

extern "C" void host_prism_std_element(const double *X18, double k, double f, double *K21, double *R6) {
  gbfem::v3 X[6];
  for (int i = 0; i < 6; i++) X[i] = {X18[3 * i], X18[3 * i + 1], X18[3 * i + 2]};
  double K[21], R[6];
  gbfem::prism_std_element(X, k, f, K, R);
  for (int i = 0; i < 21; i++) K21[i] = K[i];
  for (int i = 0; i < 6; i++) R6[i] = R[i];
}
