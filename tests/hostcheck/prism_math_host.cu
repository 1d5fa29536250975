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

// double-word operations on double inputs (converted to float pairs),
// results widened back: op 0 product, 1 sum, 2 fused a b + c, 3 a b - c d,
// 4 reciprocal of a, 5 dot3 (a, b, c) . (d, d, d)
extern "C" void host_dw_ops(int op, int n, const double *a, const double *b, const double *c, const double *d,
                            double *out) {
  using namespace gbfem;
  for (int i = 0; i < n; i++) {
    const dw x = dw_from_double(a[i]), y = dw_from_double(b[i]), z = dw_from_double(c[i]), w = dw_from_double(d[i]);
    dw r;
    switch (op) {
      case 0: r = x * y; break;
      case 1: r = x + y; break;
      case 2: r = t_fma(x, y, z); break;
      case 3: r = dw_fms(x, y, z, w); break;
      case 4: r = dw_recip(x); break;
      default: r = dw_dot3(x, w, y, w, z, w); break;
    }
    out[i] = dw_to_double(r);
  }
}

// sum_k x_k y_k through the long-sum accumulator, folded every `fold` terms
extern "C" double host_dwacc_dot(int n, const double *x, const double *y, int fold) {
  using namespace gbfem;
  DwAcc a{0.0f, 0.0f, 0.0f};
  for (int k = 0; k < n; k++) {
    const float2 u = dw_f2(x[k]), v = dw_f2(y[k]);
    dwacc_prod(a, u, v);
    if (fold > 0 && k % fold == fold - 1) dwacc_fold(a);
  }
  return dwacc_value(a);
}
