// Serving engine: independent FE problems (std linear or DG prisms) arriving
// over time are integrated, assembled and solved on one GPU with continuous
// batching.  No counterpart in the reference (ModFEM solves one problem per
// process); the per-request numerics are the library's own
// (gbfem_assemble / gbfem_dg_assemble, GMRES with Jacobi / block Jacobi).
//
// Pipeline:
//  * two lanes, std and DG requests, each with its own FIFO admission queue,
//    slot quota, CUDA stream (std at the highest priority, DG at the lowest),
//    step graph and state readback, polled independently: a std request
//    never waits for a DG request's FP64-bound block SpMVs, nor behind DG
//    requests in the queue;
//  * admission: FIFO per lane; a request starts when its lane has a free slot
//    (half of max_active, or more while the other lane has nobody waiting)
//    and its estimated device footprint fits in the shared HBM budget
//    (replaced by the measured footprint once it is built).  Std requests of
//    GBFEM_SERVE_OPT_SOLO_DOFS dofs or more never enter the engine's lanes:
//    they are admitted on the budget alone;
//  * preparation (worker threads, one CUDA stream each, std requests' at a
//    high priority, solo-sized ones' at the highest; solo-sized std
//    requests taken first, then the other
//    std ones, then DG): upload, structure (built on the device for std
//    requests), integrate + assemble, preconditioner; overlaps with
//    the solves running.  Solo-sized requests are then solved by one of eight
//    solo threads, alone on their stream, with the device-resident GMRES of
//    gbfem_solve;
//  * solve (engine thread, one stream per lane): every step of a lane
//    advances each of its active requests by one GMRES iteration with
//    batched kernels over all of them - one CRS SpMV launch for all std
//    requests, one launch per degree class for each DG request, and one
//    launch each for the Gram-Schmidt dot products, updates and norms.  The scalar GMRES logic
//    (Hessenberg column, Givens rotations, convergence test, restart and the
//    small triangular solve) runs on the device per request, so a step needs
//    no host round trip per request; the host reads the requests' phases once
//    per step to retire finished ones and admit new ones between steps.
//
// Assembly is deterministic (the gather scatter for std requests, one
// owning thread per block entry for DG) and every request's reductions are
// partitioned by its own size only and summed in a fixed order, so its result
// does not depend on which other requests share the steps: a request gives
// the same bits alone and in a mix.
//
// The kernel sequence of a lane's step depends only on its set of active
// requests (their state lives on the device), so it is captured once per
// change of that set as a CUDA graph and replayed every step.

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "dg_spmv.cuh"
#include "gbfem_internal.h"

namespace gbfem {

constexpr int SRV_MAXSLOTS = 64;
constexpr int SRV_MMAX = 64;              // largest Krylov dimension of a served request
constexpr int SRV_PART = SRV_MMAX + 2;    // per reduction block: dots 0..m, norm at SRV_MMAX + 1
constexpr int SRV_T = 256;
constexpr int SRV_PER = 8;
constexpr int SRV_CHUNK = SRV_T * SRV_PER;  // vector entries per BLAS-1 block
constexpr int SRV_SPMV_LANES = 4;
constexpr int SRV_SPMV_ROWS = SRV_T / SRV_SPMV_LANES;

enum { PH_RESTART = 0, PH_ARNOLDI = 1, PH_DONE = 2 };

// host-written description of an active request
struct SrvDesc {
  int kind;  // 0 std CRS (point Jacobi), 1 DG blocks (block Jacobi)
  int n, m, max_iter;
  double tol_rel, tol_abs;
  const int *row_ptr, *col_ind;
  const double *val, *dinv;
  const int *roff, *colx;
  const long long *row_val, *cx_off, *dinv_off;
  const double *dgval, *dgdinv;
  const double *b;
  double *x, *V, *tmp, *H, *cs, *sn, *s, *y, *hcol;
  int red_first, red_nb;
};

// device-written GMRES state of a request
struct SrvState {
  int phase, j, it, done_cols, final_flag, fresh, wscale, widx;
  double beta0, resid, beta, hn;
};

__device__ __forceinline__ double srv_block_sum(double s) {
  __shared__ double sh[SRV_T / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  s = 0.0;
  if (threadIdx.x < 32) {
    s = threadIdx.x < SRV_T / 32 ? sh[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  }
  return s;  // valid in thread 0
}

// x += V[:, :done] y at a restart
__global__ void __launch_bounds__(SRV_T) srv_update_x(const int2 *map, const SrvDesc *dd, const SrvState *ss) {
  const int2 mp = map[blockIdx.x];
  const SrvDesc &D = dd[mp.x];
  const SrvState &S = ss[mp.x];
  if (S.phase != PH_RESTART || S.done_cols == 0) return;
  for (int t = 0; t < SRV_PER; t++) {
    const long long i = (long long)mp.y + t * SRV_T + threadIdx.x;
    if (i >= D.n) break;
    double a = 0.0;
    for (int k = 0; k < S.done_cols; k++) a = fma(D.y[k], D.V[(size_t)k * D.n + i], a);
    D.x[i] = fma(1.0, a, D.x[i]);
  }
}

// CRS rows of the std requests: MODE 0 tmp = dinv (b - A x) for restarting
// requests, MODE 1 V[j+1] = dinv A V[j] for requests in an Arnoldi step.
template <int MODE>
__global__ void __launch_bounds__(SRV_T) srv_crs_spmv(const int2 *map, const SrvDesc *dd, const SrvState *ss) {
  const int2 mp = map[blockIdx.x];
  const SrvDesc &D = dd[mp.x];
  const SrvState &S = ss[mp.x];
  const bool act = MODE == 0 ? (S.phase == PH_RESTART && !S.final_flag) : S.phase == PH_ARNOLDI;
  if (!act) return;  // uniform over the block
  const int lane = threadIdx.x & (SRV_SPMV_LANES - 1);
  const long long r = (long long)mp.y + threadIdx.x / SRV_SPMV_LANES;
  const bool valid = r < D.n;
  const double *x = MODE == 0 ? D.x : D.V + (size_t)S.j * D.n;
  double *out = MODE == 0 ? D.tmp : D.V + (size_t)(S.j + 1) * D.n;
  const int lo = valid ? D.row_ptr[r] : 0, hi = valid ? D.row_ptr[r + 1] : 0;
  double s = 0.0;
  for (int k = lo + lane; k < hi; k += SRV_SPMV_LANES) s = fma(D.val[k], x[D.col_ind[k]], s);
#pragma unroll
  for (int o = SRV_SPMV_LANES / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, SRV_SPMV_LANES);
  if (valid && lane == 0) out[r] = MODE == 0 ? (D.b[r] - s) * D.dinv[r] : D.dinv[r] * s;
}

// the block rows of degree P of one DG request (same two modes)
template <int P, int MODE>
__global__ void __launch_bounds__(DGS_THREADS) srv_dg_spmv(int slot, int count, const int *ent_el,
                                                           const SrvDesc *dd, const SrvState *ss) {
  __shared__ double sv[DGS_ROWS][DgSpmvDims<P>::NS];
  const SrvDesc &D = dd[slot];
  const SrvState &S = ss[slot];
  const bool act = MODE == 0 ? (S.phase == PH_RESTART && !S.final_flag) : S.phase == PH_ARNOLDI;
  if (!act) return;
  const double *x = MODE == 0 ? D.x : D.V + (size_t)S.j * D.n;
  double *out = MODE == 0 ? D.tmp : D.V + (size_t)(S.j + 1) * D.n;
  dg_block_row_spmv<P>(MODE == 0 ? 0 : 1, count, ent_el, D.roff, D.row_val, D.cx_off, D.colx, D.dgval, D.dinv_off,
                       D.dgdinv, x, MODE == 0 ? D.b : nullptr, out, sv);
}

// per-block sum of squares: WHICH 0 the restart residual tmp, 1 the new
// Arnoldi vector V[j+1]
template <int WHICH>
__global__ void __launch_bounds__(SRV_T) srv_norm_partial(const int2 *map, const SrvDesc *dd, const SrvState *ss,
                                                          double *partial) {
  const int2 mp = map[blockIdx.x];
  const SrvDesc &D = dd[mp.x];
  const SrvState &S = ss[mp.x];
  const bool act = WHICH == 0 ? (S.phase == PH_RESTART && !S.final_flag) : S.phase == PH_ARNOLDI;
  if (!act) return;
  const double *v = WHICH == 0 ? D.tmp : D.V + (size_t)(S.j + 1) * D.n;
  double s = 0.0;
  for (int t = 0; t < SRV_PER; t++) {
    const long long i = (long long)mp.y + t * SRV_T + threadIdx.x;
    if (i < D.n) s = fma(v[i], v[i], s);
  }
  s = srv_block_sum(s);
  if (threadIdx.x == 0) partial[(size_t)(D.red_first + mp.y / SRV_CHUNK) * SRV_PART + SRV_MMAX + 1] = s;
}

// Gram-Schmidt dot products of V[k] (k = blockIdx.y <= j) with V[j+1]
__global__ void __launch_bounds__(SRV_T) srv_dot_partial(const int2 *map, const SrvDesc *dd, const SrvState *ss,
                                                         double *partial) {
  const int2 mp = map[blockIdx.x];
  const int k = blockIdx.y;
  const SrvDesc &D = dd[mp.x];
  const SrvState &S = ss[mp.x];
  if (S.phase != PH_ARNOLDI || k > S.j) return;
  const double *a = D.V + (size_t)k * D.n, *w = D.V + (size_t)(S.j + 1) * D.n;
  double s = 0.0;
  for (int t = 0; t < SRV_PER; t++) {
    const long long i = (long long)mp.y + t * SRV_T + threadIdx.x;
    if (i < D.n) s = fma(a[i], w[i], s);
  }
  s = srv_block_sum(s);
  if (threadIdx.x == 0) partial[(size_t)(D.red_first + mp.y / SRV_CHUNK) * SRV_PART + k] = s;
}

// hcol[k] = sum over the request's blocks (fixed order), one CTA per request
__global__ void srv_dot_sum(const int *act, const SrvDesc *dd, const SrvState *ss, const double *partial) {
  const int slot = act[blockIdx.x];
  const SrvDesc &D = dd[slot];
  const SrvState &S = ss[slot];
  if (S.phase != PH_ARNOLDI) return;
  for (int k = threadIdx.x; k <= S.j; k += blockDim.x) {
    double s = 0.0;
    for (int b = 0; b < D.red_nb; b++) s += partial[(size_t)(D.red_first + b) * SRV_PART + k];
    D.hcol[k] = s;
  }
}

// V[j+1] -= V[:, :j+1] hcol
__global__ void __launch_bounds__(SRV_T) srv_orthogonalize(const int2 *map, const SrvDesc *dd, const SrvState *ss) {
  const int2 mp = map[blockIdx.x];
  const SrvDesc &D = dd[mp.x];
  const SrvState &S = ss[mp.x];
  if (S.phase != PH_ARNOLDI) return;
  double *w = D.V + (size_t)(S.j + 1) * D.n;
  for (int t = 0; t < SRV_PER; t++) {
    const long long i = (long long)mp.y + t * SRV_T + threadIdx.x;
    if (i >= D.n) break;
    double a = 0.0;
    for (int k = 0; k <= S.j; k++) a = fma(D.hcol[k], D.V[(size_t)k * D.n + i], a);
    w[i] = fma(-1.0, a, w[i]);
  }
}

__device__ double srv_norm_from_partial(const SrvDesc &D, const double *partial) {
  double s = 0.0;
  for (int b = 0; b < D.red_nb; b++) s += partial[(size_t)(D.red_first + b) * SRV_PART + SRV_MMAX + 1];
  return sqrt(s);
}

// restart: x is up to date, tmp = M^-1 (b - A x); start a new cycle or stop
// (lss_mkb_core.c:2377-2400 tests, as gbfem_solve)
__global__ void srv_logic_restart(int nact, const int *act, const SrvDesc *dd, SrvState *ss, const double *partial) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nact) return;
  const int slot = act[t];
  const SrvDesc &D = dd[slot];
  SrvState &S = ss[slot];
  S.fresh = 0;
  S.wscale = 0;
  if (S.phase != PH_RESTART) return;
  if (S.final_flag) {
    S.phase = PH_DONE;
    return;
  }
  const double rn = srv_norm_from_partial(D, partial);
  if (S.beta0 < 0) S.beta0 = rn;
  S.resid = rn;
  if (rn < D.tol_abs || (S.beta0 > 0 && rn / S.beta0 < D.tol_rel) || S.it >= D.max_iter) {
    S.phase = PH_DONE;
    return;
  }
  D.s[0] = rn;
  for (int i = 1; i <= D.m; i++) D.s[i] = 0.0;
  S.beta = rn;
  S.j = 0;
  S.done_cols = 0;
  S.fresh = 1;
  S.phase = PH_ARNOLDI;
}

__global__ void __launch_bounds__(SRV_T) srv_start_cycle(const int2 *map, const SrvDesc *dd, const SrvState *ss) {
  const int2 mp = map[blockIdx.x];
  const SrvDesc &D = dd[mp.x];
  const SrvState &S = ss[mp.x];
  if (!S.fresh) return;
  for (int t = 0; t < SRV_PER; t++) {
    const long long i = (long long)mp.y + t * SRV_T + threadIdx.x;
    if (i < D.n) D.V[i] = D.tmp[i] / S.beta;
  }
}

// one Arnoldi column: Hessenberg entries, Givens rotations, residual
// estimate, and at the end of a cycle the triangular solve for y
__global__ void srv_logic_arnoldi(int nact, const int *act, const SrvDesc *dd, SrvState *ss,
                                  const double *partial) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nact) return;
  const int slot = act[t];
  const SrvDesc &D = dd[slot];
  SrvState &S = ss[slot];
  if (S.phase != PH_ARNOLDI) return;
  const int m = D.m, j = S.j, ld = m + 1;
  const double hn = srv_norm_from_partial(D, partial);
  double *H = D.H;
  for (int k = 0; k <= j; k++) H[k + (size_t)j * ld] = D.hcol[k];
  H[j + 1 + (size_t)j * ld] = hn;
  for (int k = 0; k < j; k++) {
    const double a = H[k + (size_t)j * ld], b = H[k + 1 + (size_t)j * ld];
    H[k + (size_t)j * ld] = D.cs[k] * a + D.sn[k] * b;
    H[k + 1 + (size_t)j * ld] = D.cs[k] * b - D.sn[k] * a;
  }
  {
    const double a = H[j + (size_t)j * ld], b = H[j + 1 + (size_t)j * ld];
    const double rr = hypot(a, b);
    D.cs[j] = a / rr;
    D.sn[j] = b / rr;
    H[j + (size_t)j * ld] = rr;
    H[j + 1 + (size_t)j * ld] = 0.0;
    const double s0 = D.s[j];
    D.s[j] = D.cs[j] * s0;
    D.s[j + 1] = -D.sn[j] * s0;
  }
  S.it++;
  S.resid = fabs(D.s[j + 1]);
  S.hn = hn;
  S.widx = j + 1;
  S.wscale = 1;
  const bool conv = S.resid < D.tol_abs || S.resid / S.beta0 < D.tol_rel;
  if (j == m - 1 || S.it >= D.max_iter || conv) {
    const int done = j + 1;
    for (int k = done - 1; k >= 0; k--) {
      double v = D.s[k];
      for (int i = k + 1; i < done; i++) v -= H[k + (size_t)i * ld] * D.y[i];
      D.y[k] = v / H[k + (size_t)k * ld];
    }
    S.done_cols = done;
    S.final_flag = (conv || S.it >= D.max_iter) ? 1 : 0;
    S.phase = PH_RESTART;
  } else {
    S.j = j + 1;
  }
}

__global__ void __launch_bounds__(SRV_T) srv_normalize(const int2 *map, const SrvDesc *dd, const SrvState *ss) {
  const int2 mp = map[blockIdx.x];
  const SrvDesc &D = dd[mp.x];
  const SrvState &S = ss[mp.x];
  if (!S.wscale) return;
  double *w = D.V + (size_t)S.widx * D.n;
  for (int t = 0; t < SRV_PER; t++) {
    const long long i = (long long)mp.y + t * SRV_T + threadIdx.x;
    if (i < D.n) w[i] = w[i] / S.hn;
  }
}

}  // namespace gbfem

using gbfem::DevBuf;
using gbfem::SrvDesc;
using gbfem::SrvState;

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

const int kNs[5] = {0, 6, 18, 40, 75};

struct SrvRequest {
  long long id = 0;
  int kind = 0, p = 1, krylov = 30, max_iter = 1000;
  double tol = 1e-8, f = 1.0, g = 0.0, pen = 10.0;
  int nno = 0, nel = 0, nbf = 0, nfa = 0;
  std::vector<double> xyz, k;
  std::vector<int> el, bf_el, bf_side, fa_type, fa_bc, fa_el, fa_side, fa_nodes;
  long long footprint = 0, charged = 0;
  double t_submit = 0, t_admit = 0, t_ready = 0, t_start = 0, t_done = 0;
  int status = 0;  // 0 queued, 1 preparing, 2 ready, 3 solving, 4 done, -1 failed, -2 cancelled
  bool cancel = false;  // cancellation asked while preparing or solving
  bool solo = false;    // large std request: solved alone by a solo thread
  bool solo_admit = false;  // admitted as a solo request, outside the lane's slots
  std::string err;
  gbfem_ctx ctx = nullptr;
  DevBuf<double> kry;
  int n = 0, slot = -1;
  std::vector<double> x;
  int iters = 0;
  double rel = 0.0;
};

using ReqPtr = std::shared_ptr<SrvRequest>;

}  // namespace

long long gbfem_serve_footprint_impl(int kind, int p, int nno, int nel, int nbf, int nfa, int krylov) {
  const long long m1 = krylov + 1;
  long long b = 24LL * nno + 24LL * nel + 8LL * nel + 16LL * nbf + (1LL << 20);
  if (kind == 0) {
    const long long n = nno, nnz = 27LL * nno;  // prism meshes hold about 21 entries per row
    b += 12LL * nnz + 4LL * (n + 1) + 4LL * nno + 168LL * nel + 8LL * nel + 16LL * nbf;  // CRS, tables, colours
    b += 336LL * nel + 24LL * nel + 4LL * (n + 1);  // gather scatter: local matrices, incidence
    b += 8LL * n * (m1 + 4) + 8LL * m1 * m1;                                           // Krylov
  } else {
    const long long ns = kNs[p], n = ns * nel, blocks = nel + 2LL * nfa;
    b += 8LL * ns * ns * blocks + 8LL * ns * ns * nel + 4LL * ns * blocks + 64LL * nel + 48LL * 2 * nfa;
    b += 8LL * n * (m1 + 4) + 8LL * m1 * m1;
  }
  return b;
}

// One lane of the engine: the active requests of one kind and what their
// batched steps need.
struct SrvLane {
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;  // recorded after a poll's steps and state readback
  bool busy = false, changed = false;
  std::deque<ReqPtr> waitq;    // admission queue of this kind
  int held = 0;                // admitted and not yet retired
  std::vector<int> act;        // slots
  DevBuf<int2> d_map_vec, d_map_crs;
  DevBuf<int> d_act;
  DevBuf<double> d_partial;
  SrvState *h_state = nullptr;  // pinned readback of the last poll
  int n_vec = 0, n_crs = 0, max_m1 = 1;
  cudaGraphExec_t graph = nullptr;
  int graph_kernels = 0;
};

struct gbfem_server_s {
  int device = 0;
  long long budget = 0, in_use = 0, peak_in_use = 0;
  int max_active = 0;
  std::mutex mu;
  std::condition_variable cv_engine, cv_prep, cv_done, cv_solo;
  std::deque<ReqPtr> prepq, readyq;
  // prepared solo requests, solved by the solo threads (so that a long solve
  // does not hold a preparation worker)
  std::deque<ReqPtr> soloq;
  std::vector<std::thread> solo_workers;
  std::map<long long, ReqPtr> reqs;
  long long next_id = 0;
  int n_preparing = 0, n_active = 0;
  bool stop = false;
  std::vector<std::thread> workers;
  std::thread engine;
  // contexts and Krylov spaces of finished requests, freed by the reaper
  // thread: a cudaFree synchronises the device, which on the engine thread
  // would hold every lane until all GPU work drained
  std::deque<std::pair<gbfem_ctx, double *>> reapq;
  std::condition_variable cv_reap;
  bool reap_stop = false;
  std::thread reaper;
  // engine-owned
  SrvLane lanes[2];  // 0: std requests, 1: DG requests
  ReqPtr slots[gbfem::SRV_MAXSLOTS];
  DevBuf<SrvDesc> d_desc;
  DevBuf<SrvState> d_state;
  SrvState *h_init = nullptr;  // pinned: initial states of newly started requests
  SrvDesc *h_desc = nullptr;
  long long steps = 0, launches = 0;
  int peak_active = 0;
  int steps_per_poll = 4;
  int inject_prep_failures = 0;  // GBFEM_SERVE_OPT_FAIL_PREPARATIONS
  int solo_dofs = 40000;         // GBFEM_SERVE_OPT_SOLO_DOFS
  int std_precedence = 1;        // GBFEM_SERVE_OPT_STD_PRECEDENCE
  std::atomic<int> n_solo{0};    // solo requests admitted and not finished
  int prio_std = 0;              // stream priority of std requests' contexts
  int prio_solo = 0;             // of solo-sized std requests' contexts (the greatest)
  std::string fatal;
};

namespace {

// Hands a finished request's context and Krylov space to the reaper (no
// device work of it may be in flight).
void reap(gbfem_server s, SrvRequest &r) {
  double *kry = r.kry.p;
  r.kry.p = nullptr;  // ownership passes to the reaper
  r.kry.n = 0;
  gbfem_ctx c = r.ctx;
  r.ctx = nullptr;
  if (!c && !kry) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->reapq.emplace_back(c, kry);
  }
  s->cv_reap.notify_one();
}

void reaper_loop(gbfem_server s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    s->cv_reap.wait(lk, [&] { return s->reap_stop || !s->reapq.empty(); });
    if (s->reapq.empty()) return;  // stop, and nothing left
    const auto item = s->reapq.front();
    s->reapq.pop_front();
    lk.unlock();
    if (item.first) gbfem_destroy(item.first);
    if (item.second) cudaFree(item.second);
    lk.lock();
  }
}

// A lane may hold half of max_active requests, or more while the other lane
// has nobody waiting; the HBM budget is shared.
void try_admit(gbfem_server s) {  // caller holds s->mu
  const int share = std::max(1, s->max_active / 2);
  // std requests of at least solo_dofs dofs (one per vertex) are solved by
  // their preparation worker on their own stream, not in the engine's
  // lanes: they take no lane slot, only their share of the HBM budget
  if (s->solo_dofs > 0) {
    auto &q = s->lanes[0].waitq;
    for (auto it = q.begin(); it != q.end();) {
      ReqPtr r = *it;
      if (r->nno < s->solo_dofs) {
        ++it;
        continue;
      }
      if (s->in_use + r->footprint > s->budget && s->in_use > 0) break;
      it = q.erase(it);
      r->solo_admit = true;
      s->n_solo++;
      s->in_use += r->footprint;
      r->charged = r->footprint;
      s->peak_in_use = std::max(s->peak_in_use, s->in_use);
      r->status = 1;
      r->t_admit = now_s();
      s->n_preparing++;
      s->prepq.push_back(r);
      s->cv_prep.notify_one();
    }
  }
  for (int L = 0; L < 2; L++) {
    SrvLane &ln = s->lanes[L], &other = s->lanes[1 - L];
    while (!ln.waitq.empty()) {
      ReqPtr r = ln.waitq.front();
      if (ln.held + other.held >= s->max_active) break;
      if (ln.held >= share && !other.waitq.empty()) break;
      if (s->in_use + r->footprint > s->budget && s->in_use > 0) break;
      ln.waitq.pop_front();
      ln.held++;
      s->in_use += r->footprint;
      r->charged = r->footprint;
      s->peak_in_use = std::max(s->peak_in_use, s->in_use);
      r->status = 1;
      r->t_admit = now_s();
      s->n_preparing++;
      s->prepq.push_back(r);
      s->cv_prep.notify_one();
    }
  }
}

int prepare(gbfem_server s, SrvRequest &r) {
  {
    // host-side fault injection: this preparation fails as a device
    // allocation would, before any device work
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->inject_prep_failures > 0) {
      s->inject_prep_failures--;
      gbfem::set_error("injected allocation failure (GBFEM_SERVE_OPT_FAIL_PREPARATIONS)");
      return -1;
    }
  }
  gbfem_ctx c = nullptr;
  // std requests' preparation and solo solves at the std lane's priority:
  // the DG lane's long block SpMVs (lowest priority) do not hold them up
  int rc = gbfem::create_context(&c, s->device, r.kind == 0 ? (r.solo_admit ? s->prio_solo : s->prio_std) : 0);
  if (rc < 0) return rc;
  r.ctx = c;
  std::vector<int> fid, fbc;
  if (r.kind == 0) {
    fbc.assign(r.nbf, 1);
    rc = gbfem_set_mesh(c, r.nno, r.xyz.data(), r.nel, GBFEM_PRISM, r.el.data(), r.nbf, nullptr, r.bf_el.data(),
                        r.bf_side.data(), fbc.data());
  } else {
    rc = gbfem_set_mesh(c, r.nno, r.xyz.data(), r.nel, GBFEM_PRISM, r.el.data(), 0, nullptr, nullptr, nullptr,
                        nullptr);
  }
  if (rc < 0) return rc;
  rc = gbfem_set_coefficients(c, r.k.data(), nullptr, r.f, r.g, 1.0e7);
  if (rc < 0) return rc;
  if (r.kind == 0) {
    int nd = 0;
    long long nnz = 0;
    // structure on the device
    if ((rc = gbfem_build_structure_device(c, &nd, &nnz)) < 0) return rc;
    // the gather scatter: the same summation order every time (no element
    // colouring needed), so a request's matrix (and result) does not depend
    // on when it runs
    if ((rc = gbfem_assemble(c, GBFEM_SCATTER_GATHER)) < 0) return rc;
    r.n = nd;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      r.solo = r.solo_admit || (s->solo_dofs > 0 && nd >= s->solo_dofs);
    }
    if (r.solo) {
      // solved by the preparation worker with the device-resident GMRES
      if (cudaStreamSynchronize(c->stream) != cudaSuccess) {
        gbfem::set_error("preparation failed on the device");
        return -1;
      }
      return 0;
    }
    if ((rc = c->dinv.alloc(nd)) < 0) return rc;
    if ((rc = gbfem::launch_jacobi_diag(c->stream, nd, c->row_ptr.p, c->col_ind.p, c->val.p, c->dinv.p)) < 0)
      return rc;
  } else {
    std::vector<int> pe(r.nel, r.p);
    if ((rc = gbfem_dg_set_degrees(c, pe.data())) < 0) return rc;
    if ((rc = gbfem_dg_set_faces(c, r.nfa, r.fa_type.data(), r.fa_bc.data(), r.fa_el.data(), r.fa_side.data(),
                                 r.fa_nodes.data())) < 0)
      return rc;
    if ((rc = gbfem_dg_set_penalty(c, r.pen)) < 0) return rc;
    int nd = 0;
    long long nv = 0;
    if ((rc = gbfem_dg_build_structure(c, &nd, &nv)) < 0) return rc;
    if ((rc = gbfem_dg_assemble(c)) < 0) return rc;
    r.n = nd;
    if ((rc = c->dg_dinv.alloc((size_t)c->dg_ninv)) < 0) return rc;
    cudaMemsetAsync(c->err.p, 0, sizeof(int), c->stream);
    if ((rc = gbfem::launch_dg_block_inverse(c->stream, c->nel, c->dg_roff_d.p, c->dg_boff_diag_d.p, c->dg_val.p,
                                             c->dg_dinv_off_d.p, c->dg_dinv.p, c->err.p)) < 0)
      return rc;
    int herr = 0;
    cudaMemcpyAsync(&herr, c->err.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess || herr != 0) {
      gbfem::set_error("DG block Jacobi: singular diagonal block");
      return -2;
    }
  }
  // Krylov workspace: x, tmp, V (m+1 columns), H, cs, sn, s, y, hcol
  const long long n = r.n, m1 = r.krylov + 1;
  if ((rc = r.kry.alloc((size_t)(n * (m1 + 2) + m1 * m1 + 5 * (m1 + 1)))) < 0) return rc;
  if (cudaMemsetAsync(r.kry.p, 0, r.kry.bytes(), c->stream) != cudaSuccess) return -1;
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) {
    gbfem::set_error("preparation failed on the device");
    return -1;
  }
  return 0;
}

void prep_worker(gbfem_server s) {
  cudaSetDevice(s->device);
  for (;;) {
    ReqPtr r;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_prep.wait(lk, [&] { return s->stop || !s->prepq.empty(); });
      if (s->prepq.empty()) return;
      // solo-sized std requests first (the longest latency-bound path:
      // preparation, then a device GMRES of hundreds of iterations), then
      // the other std requests (short preparation, latency-bound solve),
      // then DG, each in admission order
      auto it = std::find_if(s->prepq.begin(), s->prepq.end(), [](const ReqPtr &q) { return q->solo_admit; });
      if (it == s->prepq.end())
        it = std::find_if(s->prepq.begin(), s->prepq.end(), [](const ReqPtr &q) { return q->kind == 0; });
      if (it == s->prepq.end()) it = s->prepq.begin();
      r = *it;
      s->prepq.erase(it);
    }
    const int rc = prepare(s, *r);
    std::unique_lock<std::mutex> lk(s->mu);
    s->n_preparing--;
    r->t_ready = now_s();
    if (rc < 0 || r->cancel) {
      r->status = rc < 0 ? -1 : -2;
      r->err = rc < 0 ? gbfem_last_error() : "cancelled";
      lk.unlock();
      reap(s, *r);
      lk.lock();
      s->in_use -= r->charged;
      r->charged = 0;
      r->t_done = now_s();
      if (!r->solo_admit) s->lanes[r->kind].held--;
      if (r->solo_admit) s->n_solo--;
      try_admit(s);
      s->cv_done.notify_all();
      continue;
    }
    if (r->solo) {
      // a large std request: solved by a solo thread on its own stream
      r->status = 3;
      s->soloq.push_back(r);
      s->cv_solo.notify_one();
      continue;
    }
    // replace the estimate by what the request holds
    const long long actual = gbfem_device_bytes(r->ctx) + (long long)r->kry.bytes();
    s->in_use += actual - r->charged;
    r->charged = actual;
    s->peak_in_use = std::max(s->peak_in_use, s->in_use);
    r->status = 2;
    s->readyq.push_back(r);
    s->cv_engine.notify_one();
    try_admit(s);
  }
}

// Solo requests (large std): gbfem_solve's device GMRES on the request's own
// stream and restart-cycle graph, beside the engine's batched lanes; the
// estimate (which includes the Krylov space) stays charged until done.
void solo_worker(gbfem_server s) {
  cudaSetDevice(s->device);
  for (;;) {
    ReqPtr r;
    bool skip = false;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_solo.wait(lk, [&] { return s->stop || !s->soloq.empty(); });
      if (s->soloq.empty()) return;
      r = s->soloq.front();
      s->soloq.pop_front();
      s->n_active++;
      r->t_start = now_s();
      skip = r->cancel;
    }
    r->x.assign(r->n, 0.0);
    double res = 0.0, rel = 0.0;
    // (cancelled while queued here: not solved)
    const int it = skip ? 0
                        : gbfem::gmres_device_std(r->ctx, r->krylov, r->max_iter, r->tol, 1, r->x.data(), &res,
                                                       &rel);
    const std::string err = it < 0 ? std::string(gbfem_last_error()) : std::string();
    reap(s, *r);
    std::lock_guard<std::mutex> lk(s->mu);
    r->iters = it < 0 ? 0 : it;
    r->rel = rel;
    s->in_use -= r->charged;
    r->charged = 0;
    r->status = it < 0 ? -1 : (r->cancel ? -2 : 4);
    if (it < 0) r->err = err;
    if (r->cancel && it >= 0) r->err = "cancelled";
    r->t_done = now_s();
    s->n_active--;
    if (!r->solo_admit) s->lanes[r->kind].held--;
    if (r->solo_admit) s->n_solo--;
    try_admit(s);
    s->cv_done.notify_all();
  }
}

void fill_desc(SrvDesc &d, SrvRequest &r) {
  memset(&d, 0, sizeof(d));
  gbfem_ctx c = r.ctx;
  const long long n = r.n, m1 = r.krylov + 1;
  d.kind = r.kind;
  d.n = r.n;
  d.m = r.krylov;
  d.max_iter = r.max_iter;
  d.tol_rel = r.tol < 1e-12 ? 1e-12 : r.tol;
  d.tol_abs = 1e-12;
  if (r.kind == 0) {
    d.row_ptr = c->row_ptr.p;
    d.col_ind = c->col_ind.p;
    d.val = c->val.p;
    d.dinv = c->dinv.p;
    d.b = c->rhs.p;
  } else {
    d.roff = c->dg_roff_d.p;
    d.colx = c->dg_colx_d.p;
    d.row_val = c->dg_row_val_d.p;
    d.cx_off = c->dg_cx_off_d.p;
    d.dinv_off = c->dg_dinv_off_d.p;
    d.dgval = c->dg_val.p;
    d.dgdinv = c->dg_dinv.p;
    d.b = c->dg_rhs.p;
  }
  double *w = r.kry.p;
  d.x = w;
  d.tmp = w + n;
  d.V = w + 2 * n;
  d.H = d.V + n * m1;
  d.cs = d.H + m1 * m1;
  d.sn = d.cs + (m1 + 1);
  d.s = d.sn + (m1 + 1);
  d.y = d.s + (m1 + 1);
  d.hcol = d.y + (m1 + 1);
}

// rebuild a lane's block maps and its requests' descriptors after its
// active set changed (the lane is idle: nothing of it is in flight)
int rebuild(gbfem_server s, SrvLane &ln, int L) {
  std::vector<int2> mv, mc;
  int red = 0;
  ln.act.clear();
  ln.max_m1 = 1;
  for (int i = 0; i < gbfem::SRV_MAXSLOTS; i++) {
    if (!s->slots[i] || s->slots[i]->kind != L) continue;
    SrvRequest &r = *s->slots[i];
    ln.act.push_back(i);
    SrvDesc &d = s->h_desc[i];
    const int nb = (r.n + gbfem::SRV_CHUNK - 1) / gbfem::SRV_CHUNK;
    d.red_first = red;
    d.red_nb = nb;
    red += nb;
    for (int b = 0; b < nb; b++) mv.push_back(make_int2(i, b * gbfem::SRV_CHUNK));
    if (r.kind == 0)
      for (int r0 = 0; r0 < r.n; r0 += gbfem::SRV_SPMV_ROWS) mc.push_back(make_int2(i, r0));
    ln.max_m1 = std::max(ln.max_m1, r.krylov + 1);
  }
  ln.n_vec = (int)mv.size();
  ln.n_crs = (int)mc.size();
  if (ln.d_map_vec.alloc(std::max<size_t>(mv.size(), 1)) < 0 || ln.d_map_crs.alloc(std::max<size_t>(mc.size(), 1)) < 0 ||
      ln.d_act.alloc(std::max<size_t>(ln.act.size(), 1)) < 0 ||
      ln.d_partial.alloc((size_t)std::max(red, 1) * gbfem::SRV_PART) < 0)
    return -1;
  if (!mv.empty())
    GB_CUDA(cudaMemcpyAsync(ln.d_map_vec.p, mv.data(), mv.size() * sizeof(int2), cudaMemcpyHostToDevice, ln.stream));
  if (!mc.empty())
    GB_CUDA(cudaMemcpyAsync(ln.d_map_crs.p, mc.data(), mc.size() * sizeof(int2), cudaMemcpyHostToDevice, ln.stream));
  if (!ln.act.empty())
    GB_CUDA(cudaMemcpyAsync(ln.d_act.p, ln.act.data(), ln.act.size() * sizeof(int), cudaMemcpyHostToDevice, ln.stream));
  // only this lane's descriptors: the other lane's kernels read theirs meanwhile
  for (int i : ln.act)
    GB_CUDA(cudaMemcpyAsync(s->d_desc.p + i, s->h_desc + i, sizeof(SrvDesc), cudaMemcpyHostToDevice, ln.stream));
  // the host copies (maps, descriptors) are rewritten by the next rebuild
  GB_CUDA(cudaStreamSynchronize(ln.stream));
  return 0;
}

int step(gbfem_server s, SrvLane &ln) {
  using namespace gbfem;
  cudaStream_t st = ln.stream;
  const int nact = (int)ln.act.size();
  const int lt = 128, lb = (nact + lt - 1) / lt;
  int L = 0;
  const int2 *mv = ln.d_map_vec.p, *mc = ln.d_map_crs.p;
  SrvDesc *dd = s->d_desc.p;
  SrvState *ss = s->d_state.p;
  double *part = ln.d_partial.p;
  auto dg_spmv = [&](int mode) {
    for (int i : ln.act) {
      SrvRequest &r = *s->slots[i];
      if (r.kind != 1) continue;
      for (int p = 1; p <= 4; p++) {
        const int cnt = (int)r.ctx->dg_list[p].n;
        if (!r.ctx->dg_list[p].p || cnt == 0) continue;
        const int grid = (cnt + DGS_ROWS - 1) / DGS_ROWS;
        const int *lst = r.ctx->dg_list[p].p;
#define GB_SRV_DG(PP)                                                                          \
  if (mode == 0)                                                                               \
    srv_dg_spmv<PP, 0><<<grid, DGS_THREADS, 0, st>>>(i, cnt, lst, dd, ss);                    \
  else                                                                                         \
    srv_dg_spmv<PP, 1><<<grid, DGS_THREADS, 0, st>>>(i, cnt, lst, dd, ss)
        switch (p) {
          case 1: GB_SRV_DG(1); break;
          case 2: GB_SRV_DG(2); break;
          case 3: GB_SRV_DG(3); break;
          default: GB_SRV_DG(4); break;
        }
#undef GB_SRV_DG
        L++;
      }
    }
  };
  // restart: x += V y, residual, its norm, new cycle or stop
  srv_update_x<<<ln.n_vec, SRV_T, 0, st>>>(mv, dd, ss);
  if (ln.n_crs) srv_crs_spmv<0><<<ln.n_crs, SRV_T, 0, st>>>(mc, dd, ss);
  dg_spmv(0);
  srv_norm_partial<0><<<ln.n_vec, SRV_T, 0, st>>>(mv, dd, ss, part);
  srv_logic_restart<<<lb, lt, 0, st>>>(nact, ln.d_act.p, dd, ss, part);
  srv_start_cycle<<<ln.n_vec, SRV_T, 0, st>>>(mv, dd, ss);
  // one Arnoldi step
  if (ln.n_crs) srv_crs_spmv<1><<<ln.n_crs, SRV_T, 0, st>>>(mc, dd, ss);
  dg_spmv(1);
  srv_dot_partial<<<dim3(ln.n_vec, ln.max_m1), SRV_T, 0, st>>>(mv, dd, ss, part);
  srv_dot_sum<<<nact, 64, 0, st>>>(ln.d_act.p, dd, ss, part);
  srv_orthogonalize<<<ln.n_vec, SRV_T, 0, st>>>(mv, dd, ss);
  srv_norm_partial<1><<<ln.n_vec, SRV_T, 0, st>>>(mv, dd, ss, part);
  srv_logic_arnoldi<<<lb, lt, 0, st>>>(nact, ln.d_act.p, dd, ss, part);
  srv_normalize<<<ln.n_vec, SRV_T, 0, st>>>(mv, dd, ss);
  L += 11 + (ln.n_crs ? 2 : 0);
  GB_CUDA(cudaGetLastError());
  return L;
}

// capture a lane's step for its current active set
int capture(gbfem_server s, SrvLane &ln) {
  if (ln.graph) {
    cudaGraphExecDestroy(ln.graph);
    ln.graph = nullptr;
  }
  if (ln.act.empty()) return 0;
  cudaGraph_t g = nullptr;
  GB_CUDA(cudaStreamBeginCapture(ln.stream, cudaStreamCaptureModeThreadLocal));
  const int L = step(s, ln);
  cudaGraph_t gg = nullptr;
  const cudaError_t e = cudaStreamEndCapture(ln.stream, &gg);
  if (L < 0) return L;
  GB_CUDA(e);
  g = gg;
  const cudaError_t ei = cudaGraphInstantiate(&ln.graph, g, 0);
  cudaGraphDestroy(g);
  GB_CUDA(ei);
  ln.graph_kernels = L;
  return 0;
}

// A finished (or cancelled) request leaves its slot; the lane is idle here
// (its last poll completed), so nothing of it is in flight.
void retire(gbfem_server s, SrvLane &ln, int i, bool cancelled = false) {
  ReqPtr r = s->slots[i];
  const SrvState &S = ln.h_state[i];
  if (!cancelled) {
    r->x.resize(r->n);
    cudaMemcpyAsync(r->x.data(), r->kry.p, (size_t)r->n * sizeof(double), cudaMemcpyDeviceToHost, ln.stream);
    cudaStreamSynchronize(ln.stream);
    r->iters = S.it;
    r->rel = S.beta0 > 0 ? S.resid / S.beta0 : 0.0;
  }
  reap(s, *r);
  s->slots[i].reset();
  std::lock_guard<std::mutex> lk(s->mu);
  s->in_use -= r->charged;
  r->charged = 0;
  r->status = cancelled ? -2 : 4;
  if (cancelled) r->err = "cancelled";
  r->t_done = now_s();
  s->n_active--;
  ln.held--;
  try_admit(s);
  s->cv_done.notify_all();
}

void engine_fail(gbfem_server s, const std::string &msg) {
  std::lock_guard<std::mutex> lk(s->mu);
  s->fatal = msg;
  s->stop = true;
  s->cv_done.notify_all();
}

void engine_loop(gbfem_server s) {
  cudaSetDevice(s->device);
  for (;;) {
    {
      std::unique_lock<std::mutex> lk(s->mu);
      const bool idle = s->lanes[0].act.empty() && s->lanes[1].act.empty() && !s->lanes[0].busy &&
                        !s->lanes[1].busy;
      if (idle && s->readyq.empty()) {
        s->cv_engine.wait(lk, [&] { return s->stop || !s->readyq.empty(); });
        if (s->stop && s->readyq.empty()) return;
      }
      while (!s->readyq.empty()) {
        int i = 0;
        while (i < gbfem::SRV_MAXSLOTS && s->slots[i]) i++;
        if (i == gbfem::SRV_MAXSLOTS) break;
        ReqPtr r = s->readyq.front();
        s->readyq.pop_front();
        SrvLane &ln = s->lanes[r->kind];
        r->slot = i;
        r->status = 3;
        r->t_start = now_s();
        s->slots[i] = r;
        s->n_active++;
        fill_desc(s->h_desc[i], *r);
        SrvState init;
        memset(&init, 0, sizeof(init));
        init.phase = gbfem::PH_RESTART;
        init.beta0 = -1.0;
        s->h_init[i] = init;
        // behind the lane's work in flight (which does not touch slot i)
        cudaMemcpyAsync(s->d_state.p + i, s->h_init + i, sizeof(SrvState), cudaMemcpyHostToDevice, ln.stream);
        ln.changed = true;
      }
      s->peak_active = std::max(s->peak_active, s->n_active);
    }
    bool progressed = false;
    for (int L = 0; L < 2; L++) {
      SrvLane &ln = s->lanes[L];
      if (ln.busy) {
        const cudaError_t q = cudaEventQuery(ln.done);
        if (q == cudaErrorNotReady) continue;
        if (q != cudaSuccess) {
          engine_fail(s, std::string("serving step failed: ") + cudaGetErrorString(q));
          return;
        }
        ln.busy = false;
        progressed = true;
        for (int i : std::vector<int>(ln.act)) {
          bool cancelled;
          {
            std::lock_guard<std::mutex> lk(s->mu);
            cancelled = s->slots[i]->cancel;
          }
          if (ln.h_state[i].phase == gbfem::PH_DONE || cancelled) {
            retire(s, ln, i, cancelled);
            ln.changed = true;
          }
        }
      }
      if (ln.changed) {
        if (rebuild(s, ln, L) < 0 || capture(s, ln) < 0) {
          engine_fail(s, gbfem_last_error());
          return;
        }
        ln.changed = false;
      }
      if (ln.act.empty()) continue;
      // std precedence: no new DG steps while a solo request is in flight
      if (L == 1 && s->std_precedence && s->n_solo.load() > 0) continue;
      // several steps per poll: a finished request's kernels are no-ops until
      // it is retired, so the extra steps only cost their launch
      cudaError_t ge = cudaSuccess;
      for (int k = 0; k < s->steps_per_poll && ge == cudaSuccess; k++) {
        ge = cudaGraphLaunch(ln.graph, ln.stream);
        s->steps++;
        s->launches += ln.graph_kernels;
      }
      if (ge != cudaSuccess ||
          cudaMemcpyAsync(ln.h_state, s->d_state.p, sizeof(SrvState) * gbfem::SRV_MAXSLOTS, cudaMemcpyDeviceToHost,
                          ln.stream) != cudaSuccess ||
          cudaEventRecord(ln.done, ln.stream) != cudaSuccess) {
        engine_fail(s, std::string("serving step failed: ") + cudaGetErrorString(cudaGetLastError()));
        return;
      }
      ln.busy = true;
      progressed = true;
    }
    if (!progressed) std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
}

}  // namespace

extern "C" {

long long gbfem_serve_footprint(const gbfem_serve_request *q) {
  if (!q) return -2;
  return gbfem_serve_footprint_impl(q->kind, q->dg_p, q->nno, q->nel, q->nbf, q->nfa, q->krylov);
}

int gbfem_server_create(gbfem_server *out, int device, long long hbm_budget, int max_active, int prep_threads) {
  GB_CHECK(out, "null server pointer");
  GB_CHECK(max_active >= 1 && max_active <= gbfem::SRV_MAXSLOTS, "max_active must be 1..64");
  GB_CHECK(prep_threads >= 1 && prep_threads <= 16, "prep_threads must be 1..16");
  GB_CUDA(cudaSetDevice(device));
  gbfem_server s = new gbfem_server_s();
  s->device = device;
  s->max_active = max_active;
  if (hbm_budget <= 0) {
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    hbm_budget = (long long)(0.85 * (double)fr);
  }
  s->budget = hbm_budget;
  bool ok = s->d_desc.alloc(gbfem::SRV_MAXSLOTS) >= 0 && s->d_state.alloc(gbfem::SRV_MAXSLOTS) >= 0 &&
            cudaHostAlloc(&s->h_init, sizeof(SrvState) * gbfem::SRV_MAXSLOTS, cudaHostAllocPortable) == cudaSuccess &&
            cudaHostAlloc(&s->h_desc, sizeof(SrvDesc) * gbfem::SRV_MAXSLOTS, cudaHostAllocPortable) == cudaSuccess;
  // the std lane's short steps get a high stream priority (below only the
  // solo-sized std requests' streams), the DG lane's long FP64-bound SpMVs
  // the lowest: when both lanes have work queued the block scheduler starts
  // std blocks first
  int prio_least = 0, prio_greatest = 0;
  cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
  // solo-sized std requests above every other stream, the other std work
  // (preparations, the std lane) next, the DG lane last (greatest is the
  // numerically smallest priority)
  s->prio_solo = prio_greatest;
  s->prio_std = prio_greatest < prio_least ? prio_greatest + 1 : prio_greatest;
  for (int L = 0; L < 2 && ok; L++) {
    SrvLane &ln = s->lanes[L];
    ok = cudaStreamCreateWithPriority(&ln.stream, cudaStreamNonBlocking, L == 0 ? s->prio_std : prio_least) ==
             cudaSuccess &&
         cudaEventCreateWithFlags(&ln.done, cudaEventDisableTiming) == cudaSuccess &&
         cudaHostAlloc(&ln.h_state, sizeof(SrvState) * gbfem::SRV_MAXSLOTS, cudaHostAllocPortable) == cudaSuccess;
    if (ok) memset(ln.h_state, 0, sizeof(SrvState) * gbfem::SRV_MAXSLOTS);
  }
  if (!ok) {
    gbfem::set_error("server allocation failed");
    for (SrvLane &ln : s->lanes) {
      if (ln.h_state) cudaFreeHost(ln.h_state);
      if (ln.done) cudaEventDestroy(ln.done);
      if (ln.stream) cudaStreamDestroy(ln.stream);
    }
    if (s->h_init) cudaFreeHost(s->h_init);
    if (s->h_desc) cudaFreeHost(s->h_desc);
    delete s;
    return -1;
  }
  memset(s->h_init, 0, sizeof(SrvState) * gbfem::SRV_MAXSLOTS);
  memset(s->h_desc, 0, sizeof(SrvDesc) * gbfem::SRV_MAXSLOTS);
  cudaMemset(s->d_state.p, 0, sizeof(SrvState) * gbfem::SRV_MAXSLOTS);
  for (int i = 0; i < prep_threads; i++) s->workers.emplace_back(prep_worker, s);
  for (int i = 0; i < 8; i++) s->solo_workers.emplace_back(solo_worker, s);
  s->engine = std::thread(engine_loop, s);
  s->reaper = std::thread(reaper_loop, s);
  *out = s;
  return 0;
}

int gbfem_server_destroy(gbfem_server s) {
  if (!s) return 0;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    for (SrvLane &ln : s->lanes) ln.waitq.clear();
  }
  s->cv_prep.notify_all();
  s->cv_engine.notify_all();
  for (auto &t : s->workers) t.join();
  // the solo threads solve what is queued for them, then return
  s->cv_solo.notify_all();
  for (auto &t : s->solo_workers) t.join();
  // the engine finishes the requests it holds, then returns
  if (s->engine.joinable()) s->engine.join();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->reap_stop = true;
  }
  s->cv_reap.notify_all();
  if (s->reaper.joinable()) s->reaper.join();  // after freeing what was queued
  cudaSetDevice(s->device);
  for (auto &kv : s->reqs) {
    if (kv.second->ctx) gbfem_destroy(kv.second->ctx);
    kv.second->kry.release();
  }
  for (auto &r : s->readyq) {
    if (r->ctx) gbfem_destroy(r->ctx);
    r->kry.release();
  }
  for (SrvLane &ln : s->lanes) {
    if (ln.stream) cudaStreamSynchronize(ln.stream);
    if (ln.graph) cudaGraphExecDestroy(ln.graph);
    ln.d_map_vec.release();
    ln.d_map_crs.release();
    ln.d_act.release();
    ln.d_partial.release();
    if (ln.h_state) cudaFreeHost(ln.h_state);
    if (ln.done) cudaEventDestroy(ln.done);
    if (ln.stream) cudaStreamDestroy(ln.stream);
  }
  s->d_desc.release();
  s->d_state.release();
  if (s->h_init) cudaFreeHost(s->h_init);
  if (s->h_desc) cudaFreeHost(s->h_desc);
  delete s;
  return 0;
}

long long gbfem_server_submit(gbfem_server s, const gbfem_serve_request *q) {
  GB_CHECK(s && q, "null argument");
  GB_CHECK(q->kind == GBFEM_SERVE_STD || q->kind == GBFEM_SERVE_DG, "kind must be GBFEM_SERVE_STD or _DG");
  GB_CHECK(q->nno > 0 && q->nel > 0 && q->node_xyz && q->el_nodes && q->k_el, "empty request");
  GB_CHECK(q->krylov >= 1 && q->krylov <= gbfem::SRV_MMAX, "krylov must be 1..64 for served requests");
  GB_CHECK(q->max_iter >= 1, "max_iter must be positive");
  if (q->kind == GBFEM_SERVE_DG) {
    GB_CHECK(q->dg_p >= 1 && q->dg_p <= 4, "DG degree must be 1..4");
    GB_CHECK(q->nfa > 0 && q->fa_type && q->fa_bc && q->fa_el && q->fa_side && q->fa_nodes, "DG needs a face table");
  } else {
    GB_CHECK(q->nbf == 0 || (q->bf_el && q->bf_side), "boundary face arrays missing");
  }
  auto r = std::make_shared<SrvRequest>();
  r->kind = q->kind;
  r->p = q->dg_p;
  r->krylov = q->krylov;
  r->max_iter = q->max_iter;
  r->tol = q->tol_rel;
  r->f = q->f;
  r->g = q->g;
  r->pen = q->dg_penalty > 0 ? q->dg_penalty : 10.0;
  r->nno = q->nno;
  r->nel = q->nel;
  r->xyz.assign(q->node_xyz, q->node_xyz + 3 * (size_t)q->nno);
  r->el.assign(q->el_nodes, q->el_nodes + 6 * (size_t)q->nel);
  r->k.assign(q->k_el, q->k_el + q->nel);
  if (q->kind == GBFEM_SERVE_STD) {
    r->nbf = q->nbf;
    r->bf_el.assign(q->bf_el, q->bf_el + q->nbf);
    r->bf_side.assign(q->bf_side, q->bf_side + q->nbf);
  } else {
    r->nfa = q->nfa;
    r->fa_type.assign(q->fa_type, q->fa_type + q->nfa);
    r->fa_bc.assign(q->fa_bc, q->fa_bc + q->nfa);
    r->fa_el.assign(q->fa_el, q->fa_el + 2 * (size_t)q->nfa);
    r->fa_side.assign(q->fa_side, q->fa_side + q->nfa);
    r->fa_nodes.assign(q->fa_nodes, q->fa_nodes + 4 * (size_t)q->nfa);
  }
  r->footprint = gbfem_serve_footprint(q);
  std::lock_guard<std::mutex> lk(s->mu);
  GB_CHECK(!s->stop, "server is stopping");
  GB_CHECK(s->fatal.empty(), s->fatal.c_str());
  r->id = s->next_id++;
  r->t_submit = now_s();
  s->reqs[r->id] = r;
  s->lanes[r->kind].waitq.push_back(r);
  try_admit(s);
  return r->id;
}

int gbfem_server_wait(gbfem_server s, long long id, double timeout_s) {
  GB_CHECK(s, "null server");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  GB_CHECK(it != s->reqs.end(), "unknown request id");
  ReqPtr r = it->second;
  auto pred = [&] { return r->status == 4 || r->status < 0 || !s->fatal.empty(); };
  if (timeout_s < 0)
    s->cv_done.wait(lk, pred);
  else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred))
    return 0;
  if (!s->fatal.empty()) {
    gbfem::set_error(s->fatal);
    return -1;
  }
  if (r->status < 0) {
    gbfem::set_error("request failed: " + r->err);
    return -2;
  }
  return 1;
}

int gbfem_server_result(gbfem_server s, long long id, double *x, long long nx, int *iters, double *rel_res,
                        double *times) {
  GB_CHECK(s, "null server");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  GB_CHECK(it != s->reqs.end(), "unknown request id");
  SrvRequest &r = *it->second;
  GB_CHECK(r.status == 4, "request not finished");
  if (x) {
    GB_CHECK(nx >= (long long)r.x.size(), "solution buffer too small");
    memcpy(x, r.x.data(), r.x.size() * sizeof(double));
  }
  if (iters) *iters = r.iters;
  if (rel_res) *rel_res = r.rel;
  if (times) {
    times[0] = r.t_admit - r.t_submit;  // queued for admission
    times[1] = r.t_ready - r.t_admit;   // upload, structure, integrate + assemble, preconditioner
    times[2] = r.t_start - r.t_ready;   // waiting for an engine slot
    times[3] = r.t_done - r.t_start;    // batched GMRES
    times[4] = r.t_done - r.t_submit;   // latency
  }
  return (int)r.x.size();
}

int gbfem_server_cancel(gbfem_server s, long long id) {
  GB_CHECK(s, "null server");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  GB_CHECK(it != s->reqs.end(), "unknown request id");
  ReqPtr r = it->second;
  if (r->status == 4 || r->status < 0) return 1;  // finished, failed or cancelled already
  if (r->status == 0) {  // queued: leaves the queue now
    auto &q = s->lanes[r->kind].waitq;
    q.erase(std::remove(q.begin(), q.end(), r), q.end());
  } else if (r->status == 2) {  // prepared, waiting for an engine slot: freed now
    s->readyq.erase(std::remove(s->readyq.begin(), s->readyq.end(), r), s->readyq.end());
    if (r->ctx) gbfem_destroy(r->ctx);
    r->ctx = nullptr;
    r->kry.release();
    s->in_use -= r->charged;
    r->charged = 0;
    if (!r->solo_admit) s->lanes[r->kind].held--;
    try_admit(s);
  } else {  // preparing or solving: its worker or the engine retires it
    r->cancel = true;
    return 0;
  }
  r->status = -2;
  r->err = "cancelled";
  r->t_done = now_s();
  s->cv_done.notify_all();
  return 0;
}

int gbfem_server_release(gbfem_server s, long long id) {
  GB_CHECK(s, "null server");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  GB_CHECK(it != s->reqs.end(), "unknown request id");
  GB_CHECK(it->second->status == 4 || it->second->status < 0, "request not finished");
  s->reqs.erase(it);
  return 0;
}

int gbfem_server_set_option(gbfem_server s, int option, long long value) {
  GB_CHECK(s, "null server");
  if (option == GBFEM_SERVE_OPT_STEPS_PER_POLL) {
    GB_CHECK(value >= 1 && value <= 64, "steps per poll must be 1..64");
    std::lock_guard<std::mutex> lk(s->mu);
    s->steps_per_poll = (int)value;
    return 0;
  }
  if (option == GBFEM_SERVE_OPT_SOLO_DOFS) {
    GB_CHECK(value >= 0 && value <= 2000000000LL, "solo threshold out of range");
    std::lock_guard<std::mutex> lk(s->mu);
    s->solo_dofs = (int)value;
    return 0;
  }
  if (option == GBFEM_SERVE_OPT_STD_PRECEDENCE) {
    GB_CHECK(value == 0 || value == 1, "std precedence is 0 or 1");
    std::lock_guard<std::mutex> lk(s->mu);
    s->std_precedence = (int)value;
    return 0;
  }
  if (option == GBFEM_SERVE_OPT_FAIL_PREPARATIONS) {
    GB_CHECK(value >= 0 && value <= 1000000, "injected failure count out of range");
    std::lock_guard<std::mutex> lk(s->mu);
    s->inject_prep_failures = (int)value;
    return 0;
  }
  gbfem::set_error("unknown server option");
  return -2;
}

int gbfem_server_stats(gbfem_server s, long long *st) {
  GB_CHECK(s && st, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  st[0] = s->steps;
  st[1] = s->launches;
  st[2] = s->peak_active;
  st[3] = s->peak_in_use;
  st[4] = s->budget;
  st[5] = s->in_use;
  st[6] = (long long)(s->lanes[0].waitq.size() + s->lanes[1].waitq.size());
  st[7] = s->n_active;
  return 0;
}

}  // extern "C"
