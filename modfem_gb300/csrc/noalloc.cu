// gbfem_compute_residual_noalloc: the residual V = (Use_rhs ? B : 0) - A*X of
// gbfem_compute_residual, for callers that must not have the library
// allocate device memory.  The device copies of X and B and the result V live
// in one file-scope __device__ array instead of context buffers grown with
// cudaMalloc.

#include <mutex>

#include "gbfem_internal.h"

#define GB_TRY_NOALLOC(x)  \
  do {                     \
    int r_ = (x);          \
    if (r_ < 0) return r_; \
  } while (0)

// Three vectors of GBFEM_NOALLOC_MAX_NDOF doubles: X, B, V (6 MiB per device,
// held by every GPU that loads the library until the process exits).
static __device__ __align__(256) double g_residual_scratch[3 * GBFEM_NOALLOC_MAX_NDOF];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double *g_scratch_addr[kMaxDevices] = {nullptr};

// Device address of the scratch array on the current device.  The host-side
// symbol is only a stand-in for the device array; the kernel must get the
// address cudaGetSymbolAddress reports for this device, looked up once per
// device on the first call made with that device current.
int scratch_for_device(int device, double **out) {
  GB_CHECK(device >= 0 && device < kMaxDevices, "device index out of range for the no-alloc scratch table");
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[device]) {
    void *p = nullptr;
    GB_CUDA(cudaGetSymbolAddress(&p, g_residual_scratch));
    g_scratch_addr[device] = static_cast<double *>(p);
  }
  *out = g_scratch_addr[device];
  return 0;
}

// Makes the context's device current for the call and puts the caller's
// current device back on every return.
struct DeviceGuard {
  int saved = -1;
  ~DeviceGuard() {
    if (saved >= 0) cudaSetDevice(saved);
  }
};

int residual_on_device(gbfem_ctx c, int Use_rhs, int Ini_zero, int Ndof, const double *X, const double *B,
                       double *V);

}  // namespace

extern "C" int gbfem_compute_residual_noalloc(gbfem_ctx c, int Use_rhs, int Ini_zero, int Ndof, const double *X,
                                              const double *B, double *V) {
  GB_CHECK(c && c->have_structure, "structure not set");
  GB_CHECK(Ndof == c->ndof, "Ndof differs from the matrix size");
  GB_CHECK(V != nullptr, "null output vector");
  GB_CHECK(Ndof <= GBFEM_NOALLOC_MAX_NDOF,
           "Ndof exceeds GBFEM_NOALLOC_MAX_NDOF (262144), the size of the no-alloc scratch; use "
           "gbfem_compute_residual");
  DeviceGuard guard;
  GB_CUDA(cudaGetDevice(&guard.saved));
  if (guard.saved == c->device) guard.saved = -1;  // nothing to restore
  GB_CUDA(cudaSetDevice(c->device));
  return residual_on_device(c, Use_rhs, Ini_zero, Ndof, X, B, V);
}

namespace {

int residual_on_device(gbfem_ctx c, int Use_rhs, int Ini_zero, int Ndof, const double *X, const double *B,
                       double *V) {
  double *scratch = nullptr;
  GB_TRY_NOALLOC(scratch_for_device(c->device, &scratch));
  double *xd = scratch, *bd = scratch + GBFEM_NOALLOC_MAX_NDOF, *vd = scratch + 2 * GBFEM_NOALLOC_MAX_NDOF;
  const size_t nb = (size_t)Ndof * sizeof(double);
  // the array keeps the previous call's contents: X must read as zero when
  // Ini_zero is set, everything else is overwritten below
  if (Ini_zero || X == nullptr)
    GB_CUDA(cudaMemsetAsync(xd, 0, nb, c->stream));
  else
    GB_CUDA(cudaMemcpyAsync(xd, X, nb, cudaMemcpyHostToDevice, c->stream));
  const double *b = nullptr;
  if (Use_rhs) {
    if (B) {
      GB_CUDA(cudaMemcpyAsync(bd, B, nb, cudaMemcpyHostToDevice, c->stream));
      b = bd;
    } else {
      b = c->rhs.p;
    }
  }
  GB_TRY_NOALLOC(gbfem::launch_spmv(c->stream, 0, Ndof, c->row_ptr.p, c->col_ind.p, c->val.p, xd, b, nullptr, vd));
  GB_CUDA(cudaMemcpyAsync(V, vd, nb, cudaMemcpyDeviceToHost, c->stream));
  GB_CUDA(cudaStreamSynchronize(c->stream));
  return 0;
}

}  // namespace
