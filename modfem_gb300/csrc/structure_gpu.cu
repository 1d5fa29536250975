// Device-side structure build for std meshes: the same DOF order, CRS and
// assembly tables as the host build (and as the reference's sir_create),
// made with kernels so that a new mesh (a served request) needs no host pass.
//
//  1. first appearance of each vertex: first[n] = min over its incidences of
//     (element * nv + local vertex) (atomicMin); the DOF of n is the number
//     of used vertices whose first appearance comes earlier = an exclusive
//     scan of a 0/1 mark at every first-appearance position
//     (utr_get_list_dof_ent, utd_util/uts_ls_intf.c:182-300);
//  2. DOF -> element incidence lists (count, scan, fill in any order);
//  3. CRS rows: the DOFs of the incident elements of each row, sorted and
//     deduplicated per row (two passes: lengths, scan, columns), diagonal
//     included (sis_mkb_intf.c:1128, lad_crs/las_crs_intf.c:72-300);
//  4. element tables: for every (row dof j, column dof i) of an element the
//     position found by binary search in row j, then the rhs rows
//     (lar_fill_assembly_table_int_ent_crs, las_crs_intf.c:354-438).
// Every output is independent of thread scheduling, so it equals the host
// build bit for bit.  Built on demand from the element tables (whichever
// build made them): the DOF -> element incidence with each list in element
// order (the deterministic gather scatter reads it), and the
// elements-sharing-a-DOF colouring of the colour scatter.

#include <algorithm>
#include <climits>

#include "gbfem_internal.h"

namespace gbfem {

constexpr int SG_T = 256;
constexpr int SG_PER = 8;
constexpr int SG_CHUNK = SG_T * SG_PER;
constexpr int SG_MAXROW = 256;  // candidate column slots per row (6 x incident elements)

__device__ __forceinline__ int sg_block_exclusive(int v, int *total) {
  __shared__ int ws[SG_T / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[w] = x;
  __syncthreads();
  if (w == 0) {
    int s = lane < SG_T / 32 ? ws[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < SG_T / 32) ws[lane] = s;
  }
  __syncthreads();
  const int before = (w > 0 ? ws[w - 1] : 0) + x - v;
  *total = ws[SG_T / 32 - 1];
  __syncthreads();
  return before;
}

// exclusive scan, three kernels: chunk sums, scan of the sums, chunk scans
__global__ void sg_chunk_sums(long long n, const int *__restrict__ in, int *__restrict__ sums) {
  long long base = (long long)blockIdx.x * SG_CHUNK;
  int s = 0;
  for (int t = 0; t < SG_PER; t++) {
    const long long i = base + (long long)t * SG_T + threadIdx.x;
    if (i < n) s += in[i];
  }
  int tot;
  sg_block_exclusive(s, &tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void sg_scan_sums(int nb, int *sums, int *total) {
  // one CTA: each thread scans a contiguous range sequentially
  const int per = (nb + SG_T - 1) / SG_T, lo = threadIdx.x * per, hi = min(nb, lo + per);
  int s = 0;
  for (int i = lo; i < hi; i++) s += sums[i];
  int tot;
  int off = sg_block_exclusive(s, &tot);
  for (int i = lo; i < hi; i++) {
    const int v = sums[i];
    sums[i] = off;
    off += v;
  }
  if (threadIdx.x == 0) *total = tot;
}

__global__ void sg_chunk_scan(long long n, const int *__restrict__ in, const int *__restrict__ sums,
                              int *__restrict__ out) {
  long long base = (long long)blockIdx.x * SG_CHUNK + (long long)threadIdx.x * SG_PER;
  int v[SG_PER], s = 0;
#pragma unroll
  for (int t = 0; t < SG_PER; t++) {
    const long long i = base + t;
    v[t] = i < n ? in[i] : 0;
    s += v[t];
  }
  int tot;
  int off = sums[blockIdx.x] + sg_block_exclusive(s, &tot);
#pragma unroll
  for (int t = 0; t < SG_PER; t++) {
    const long long i = base + t;
    if (i < n) out[i] = off;
    off += v[t];
  }
}

// Scratch of one build, allocated and freed in the build stream's order
// (cudaMallocAsync / cudaFreeAsync, used on that stream only): unlike
// cudaFree, nothing here synchronises the device, so a build running beside
// other streams (the serving engine's) does not wait for their work.
template <typename T>
struct SgTemp {
  T *p = nullptr;
  size_t n = 0;
  cudaStream_t st = nullptr;
  explicit SgTemp(cudaStream_t s) : st(s) {}
  SgTemp(const SgTemp &) = delete;
  SgTemp &operator=(const SgTemp &) = delete;
  ~SgTemp() { release(); }
  int alloc(size_t count) {
    if (count <= n && p) return 0;
    release();
    if (count == 0) return 0;
    if (cudaMallocAsync(reinterpret_cast<void **>(&p), count * sizeof(T), st) != cudaSuccess) {
      p = nullptr;
      set_error("cudaMallocAsync failed for " + std::to_string(count * sizeof(T)) + " bytes");
      return -1;
    }
    n = count;
    return 0;
  }
  void release() {
    if (p) cudaFreeAsync(p, st);
    p = nullptr;
    n = 0;
  }
};

// out[i] = sum_{k < i} in[k] for i <= n (out has n + 1 entries); total in out[n]
static int sg_scan(cudaStream_t st, long long n, const int *in, int *out, SgTemp<int> &tmp) {
  const int nb = (int)((n + SG_CHUNK - 1) / SG_CHUNK);
  GB_CHECK(nb <= SG_T * 4096, "scan too long");
  if (tmp.alloc((size_t)nb + 1) < 0) return -1;
  if (nb > 0) {
    sg_chunk_sums<<<nb, SG_T, 0, st>>>(n, in, tmp.p);
    sg_scan_sums<<<1, SG_T, 0, st>>>(nb, tmp.p, out + n);
    sg_chunk_scan<<<nb, SG_T, 0, st>>>(n, in, tmp.p, out);
  } else {
    GB_CUDA(cudaMemsetAsync(out, 0, sizeof(int), st));
  }
  GB_CUDA(cudaGetLastError());
  return 0;
}

__global__ void sg_fill(int n, int v, int *a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = v;
}

__global__ void sg_first(long long m, int nv, const int *__restrict__ el_nodes, int *first) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m; i += (long long)gridDim.x * blockDim.x)
    atomicMin(first + el_nodes[i], (int)i);
}

__global__ void sg_mark(int nno, const int *__restrict__ first, int *mark) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n < nno && first[n] != INT_MAX) mark[first[n]] = 1;
}

__global__ void sg_dofs(int nno, const int *__restrict__ first, const int *__restrict__ rank, int *dof_of_node) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n < nno) dof_of_node[n] = first[n] == INT_MAX ? -1 : rank[first[n]];
}

__global__ void sg_el_dofs(long long m, const int *__restrict__ el_nodes, const int *__restrict__ dof_of_node,
                           int *el_dofs, int *inc_cnt) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m; i += (long long)gridDim.x * blockDim.x) {
    const int d = dof_of_node[el_nodes[i]];
    el_dofs[i] = d;
    atomicAdd(inc_cnt + d, 1);
  }
}

__global__ void sg_inc_fill(long long m, int nv, const int *__restrict__ el_dofs, int *cursor, int *inc) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m; i += (long long)gridDim.x * blockDim.x)
    inc[atomicAdd(cursor + el_dofs[i], 1)] = (int)(i / nv);
}

// sorted unique columns of row r into buf (returns the count, or -1 if the
// row has more candidates than SG_MAXROW)
__device__ int sg_row(int r, int nv, const int *__restrict__ inc_ptr, const int *__restrict__ inc,
                      const int *__restrict__ el_dofs, int *buf) {
  int n = 0;
  for (int k = inc_ptr[r]; k < inc_ptr[r + 1]; k++) {
    const int *ed = el_dofs + (size_t)inc[k] * nv;
    for (int j = 0; j < nv; j++) {
      if (n >= SG_MAXROW) return -1;
      // insertion into the sorted prefix, skipping duplicates
      const int v = ed[j];
      int p = n;
      while (p > 0 && buf[p - 1] > v) p--;
      if (p > 0 && buf[p - 1] == v) continue;
      for (int q = n; q > p; q--) buf[q] = buf[q - 1];
      buf[p] = v;
      n++;
    }
  }
  return n;
}

__global__ void sg_row_len(int nd, int nv, const int *__restrict__ inc_ptr, const int *__restrict__ inc,
                           const int *__restrict__ el_dofs, int *len, int *err) {
  int buf[SG_MAXROW];
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nd) return;
  const int n = sg_row(r, nv, inc_ptr, inc, el_dofs, buf);
  if (n < 0) {
    atomicExch(err, 7);
    len[r] = 0;
  } else {
    len[r] = n;
  }
}

__global__ void sg_row_fill(int nd, int nv, const int *__restrict__ inc_ptr, const int *__restrict__ inc,
                            const int *__restrict__ el_dofs, const int *__restrict__ row_ptr, int *col_ind) {
  int buf[SG_MAXROW];
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nd) return;
  const int n = sg_row(r, nv, inc_ptr, inc, el_dofs, buf);
  for (int i = 0; i < n && row_ptr[r] + i < row_ptr[r + 1]; i++) col_ind[row_ptr[r] + i] = buf[i];
}

__global__ void sg_tables(int nel, int nv, const int *__restrict__ el_dofs, const int *__restrict__ row_ptr,
                          const int *__restrict__ col_ind, int *table) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nel) return;
  const int tl = nv * nv + nv;
  const int *ed = el_dofs + (size_t)e * nv;
  int *t = table + (size_t)e * tl;
  for (int j = 0; j < nv; j++) {
    const int r = ed[j];
    for (int i = 0; i < nv; i++) {
      int lo = row_ptr[r], hi = row_ptr[r + 1];  // first position with col >= ed[i]
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (col_ind[mid] < ed[i])
          lo = mid + 1;
        else
          hi = mid;
      }
      t[j + i * nv] = lo;
    }
    t[nv * nv + j] = r;
  }
}

// Element colouring for the deterministic colour-batched scatter: elements
// sharing a dof must differ.  Jones-Plassmann with hashed priorities: in
// round r an uncoloured element whose priority beats every neighbour not
// coloured in an earlier round takes the smallest colour its earlier-coloured
// neighbours leave free.  Two neighbours never both win a round, and every
// decision reads only what earlier rounds fixed, so the colouring does not
// depend on thread scheduling.  state = (round << 8) | colour, -1 uncoloured.
__device__ __forceinline__ unsigned sg_prio(int e) {
  unsigned h = (unsigned)e * 0x9E3779B1u;
  h ^= h >> 16;
  h *= 0x85EBCA6Bu;
  h ^= h >> 13;
  return h;
}

__global__ void sg_jp_round(int nel, int nv, int rnd, const int *__restrict__ el_dofs, int stride,
                            const int *__restrict__ inc_ptr, const int *__restrict__ inc, int *state,
                            int *remaining, int *err) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nel || state[e] >= 0) return;
  const unsigned pe = sg_prio(e);
  unsigned long long used = 0;
  bool wins = true;
  for (int j = 0; j < nv && wins; j++) {
    const int d = el_dofs[(size_t)e * stride + j];
    for (int k = inc_ptr[d]; k < inc_ptr[d + 1]; k++) {
      const int f = inc[k];
      if (f == e) continue;
      const int sf = ((volatile int *)state)[f];
      if (sf >= 0 && (sf >> 8) < rnd) {
        used |= 1ULL << (sf & 63);
      } else {
        const unsigned pf = sg_prio(f);
        if (pf > pe || (pf == pe && f > e)) {
          wins = false;
          break;
        }
      }
    }
  }
  if (!wins) {
    atomicAdd(remaining, 1);
    return;
  }
  const int c = __ffsll((long long)~used) - 1;
  if (c < 0 || c >= 64) {
    atomicExch(err, 2);
    return;
  }
  state[e] = (rnd << 8) | c;
}

__global__ void sg_color_count(int nel, const int *__restrict__ state, int *cnt) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < nel) atomicAdd(cnt + (state[e] & 63), 1);
}

__global__ void sg_color_fill(int nel, const int *__restrict__ state, int *cursor, int *perm) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < nel) perm[atomicAdd(cursor + (state[e] & 63), 1)] = e;
}

int build_device_structure(cudaStream_t st, int nno, int nel, int nv, const int *el_nodes, DevBuf<int> &dof_of_node,
                           DevBuf<int> &row_ptr, DevBuf<int> &col_ind, DevBuf<int> &el_table, int *err,
                           int *ndof_out, long long *nnz_out) {
  const long long m = (long long)nel * nv;
  SgTemp<int> first(st), mark(st), rank(st), el_dofs(st), inc_cnt(st), inc_ptr(st), inc(st), len(st), tmp(st);
  auto cleanup = [&]() {
    first.release(); mark.release(); rank.release(); el_dofs.release(); inc_cnt.release();
    inc_ptr.release(); inc.release(); len.release(); tmp.release();
  };
  auto fail = [&](int r) { cleanup(); return r; };
  const int g1 = 152 * 8;
  if (first.alloc(nno) < 0 || mark.alloc(m + 1) < 0 || rank.alloc(m + 1) < 0 || dof_of_node.alloc(nno) < 0 ||
      el_dofs.alloc(m) < 0)
    return fail(-1);
  // 1. DOF order
  sg_fill<<<(nno + 255) / 256, 256, 0, st>>>(nno, INT_MAX, first.p);  // unused vertices keep INT_MAX
  sg_first<<<g1, 256, 0, st>>>(m, nv, el_nodes, first.p);
  GB_CUDA(cudaMemsetAsync(mark.p, 0, (size_t)(m + 1) * sizeof(int), st));
  sg_mark<<<(nno + 255) / 256, 256, 0, st>>>(nno, first.p, mark.p);
  if (sg_scan(st, m, mark.p, rank.p, tmp) < 0) return fail(-1);
  sg_dofs<<<(nno + 255) / 256, 256, 0, st>>>(nno, first.p, rank.p, dof_of_node.p);
  int nd = 0;
  GB_CUDA(cudaMemcpyAsync(&nd, rank.p + m, sizeof(int), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  // 2. incidence
  if (inc_cnt.alloc((size_t)nd + 1) < 0 || inc_ptr.alloc((size_t)nd + 1) < 0 || inc.alloc(m) < 0) return fail(-1);
  GB_CUDA(cudaMemsetAsync(inc_cnt.p, 0, (size_t)(nd + 1) * sizeof(int), st));
  sg_el_dofs<<<g1, 256, 0, st>>>(m, el_nodes, dof_of_node.p, el_dofs.p, inc_cnt.p);
  if (sg_scan(st, nd, inc_cnt.p, inc_ptr.p, tmp) < 0) return fail(-1);
  GB_CUDA(cudaMemcpyAsync(inc_cnt.p, inc_ptr.p, (size_t)nd * sizeof(int), cudaMemcpyDeviceToDevice, st));
  sg_inc_fill<<<g1, 256, 0, st>>>(m, nv, el_dofs.p, inc_cnt.p, inc.p);
  // 3. rows
  if (len.alloc((size_t)nd + 1) < 0 || row_ptr.alloc((size_t)nd + 1) < 0) return fail(-1);
  sg_row_len<<<(nd + 127) / 128, 128, 0, st>>>(nd, nv, inc_ptr.p, inc.p, el_dofs.p, len.p, err);
  if (sg_scan(st, nd, len.p, row_ptr.p, tmp) < 0) return fail(-1);
  int nnz = 0, herr = 0;
  GB_CUDA(cudaMemcpyAsync(&nnz, row_ptr.p + nd, sizeof(int), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  if (herr) {
    cleanup();
    GB_CHECK(false, "a vertex has more neighbours than the device structure build supports");
  }
  if (col_ind.alloc((size_t)nnz) < 0) return fail(-1);
  sg_row_fill<<<(nd + 127) / 128, 128, 0, st>>>(nd, nv, inc_ptr.p, inc.p, el_dofs.p, row_ptr.p, col_ind.p);
  // 4. element tables
  if (el_table.alloc((size_t)nel * (nv * nv + nv)) < 0) return fail(-1);
  sg_tables<<<(nel + 127) / 128, 128, 0, st>>>(nel, nv, el_dofs.p, row_ptr.p, col_ind.p, el_table.p);
  GB_CUDA(cudaGetLastError());
  GB_CUDA(cudaStreamSynchronize(st));
  cleanup();
  *ndof_out = nd;
  *nnz_out = nnz;
  return 0;
}


// Incidence from the element tables (the rhs rows t[nv*nv + j] are the
// element's dofs): count, scan, fill, then each list sorted by element.
__global__ void sg_inc_count_tab(int nel, int nv, const int *__restrict__ table, int *cnt) {
  const long long m = (long long)nel * nv, tl = nv * nv + nv;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m; i += (long long)gridDim.x * blockDim.x)
    atomicAdd(cnt + table[(i / nv) * tl + nv * nv + i % nv], 1);
}

__global__ void sg_inc_fill_tab(int nel, int nv, const int *__restrict__ table, int *cursor, int *inc) {
  const long long m = (long long)nel * nv, tl = nv * nv + nv;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m; i += (long long)gridDim.x * blockDim.x)
    inc[atomicAdd(cursor + table[(i / nv) * tl + nv * nv + i % nv], 1)] = (int)(i / nv);
}

__global__ void sg_inc_sort(int nd, const int *__restrict__ inc_ptr, int *inc) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nd) return;
  int *a = inc + inc_ptr[r];
  const int n = inc_ptr[r + 1] - inc_ptr[r];
  for (int i = 1; i < n; i++) {
    const int v = a[i];
    int j = i;
    while (j > 0 && a[j - 1] > v) {
      a[j] = a[j - 1];
      j--;
    }
    a[j] = v;
  }
}

int build_device_incidence(cudaStream_t st, int nel, int nv, const int *el_table, int nd, DevBuf<int> &inc_ptr,
                           DevBuf<int> &inc) {
  const long long m = (long long)nel * nv;
  SgTemp<int> cnt(st), tmp(st);
  if (cnt.alloc((size_t)nd + 1) < 0 || inc_ptr.alloc((size_t)nd + 1) < 0 || inc.alloc((size_t)std::max(m, 1LL)) < 0)
    return -1;
  const int g1 = 152 * 8;
  GB_CUDA(cudaMemsetAsync(cnt.p, 0, ((size_t)nd + 1) * sizeof(int), st));
  sg_inc_count_tab<<<g1, 256, 0, st>>>(nel, nv, el_table, cnt.p);
  if (sg_scan(st, nd, cnt.p, inc_ptr.p, tmp) < 0) return -1;
  GB_CUDA(cudaMemcpyAsync(cnt.p, inc_ptr.p, (size_t)nd * sizeof(int), cudaMemcpyDeviceToDevice, st));
  sg_inc_fill_tab<<<g1, 256, 0, st>>>(nel, nv, el_table, cnt.p, inc.p);
  sg_inc_sort<<<(nd + 127) / 128, 128, 0, st>>>(nd, inc_ptr.p, inc.p);
  GB_CUDA(cudaGetLastError());
  // the scratch is released in stream order: nothing here waits for the device
  return 0;
}

// The colouring of the colour scatter (Jones-Plassmann, sg_jp_round), from
// the element tables and the incidence.
int build_device_colouring(cudaStream_t st, int nel, int nv, const int *el_table, const int *inc_ptr,
                           const int *inc, DevBuf<int> &el_perm, std::vector<int> &el_color_ptr, int *err) {
  // rounds in batches of SG_JP_BATCH between host reads of the last round's
  // count of elements left (a round after the last one colours nothing and
  // returns at once), each round with its own counter
  constexpr int SG_JP_BATCH = 8;
  const int tl = nv * nv + nv;
  const int *el_dofs = el_table + nv * nv;
  SgTemp<int> state(st), cnt(st);
  if (state.alloc(nel) < 0 || cnt.alloc(64 + SG_JP_BATCH) < 0 || el_perm.alloc(nel) < 0) return -1;
  sg_fill<<<(nel + 255) / 256, 256, 0, st>>>(nel, -1, state.p);
  int remaining = nel, rnd = 0, herr = 0;
  while (remaining > 0) {
    GB_CUDA(cudaMemsetAsync(cnt.p + 64, 0, SG_JP_BATCH * sizeof(int), st));
    for (int b = 0; b < SG_JP_BATCH; b++, rnd++)
      sg_jp_round<<<(nel + 255) / 256, 256, 0, st>>>(nel, nv, rnd, el_dofs, tl, inc_ptr, inc, state.p,
                                                    cnt.p + 64 + b, err);
    GB_CUDA(cudaMemcpyAsync(&remaining, cnt.p + 64 + SG_JP_BATCH - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    if (rnd > (1 << 22)) break;  // cannot happen: every round colours the top-priority element left
  }
  GB_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaMemsetAsync(cnt.p, 0, 64 * sizeof(int), st));
  sg_color_count<<<(nel + 255) / 256, 256, 0, st>>>(nel, state.p, cnt.p);
  std::vector<int> counts(64);
  GB_CUDA(cudaMemcpyAsync(counts.data(), cnt.p, 64 * sizeof(int), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  GB_CHECK(!herr && remaining == 0, "device colouring needs more than 64 colours");
  int ncol = 64;
  while (ncol > 0 && counts[ncol - 1] == 0) ncol--;
  el_color_ptr.assign(ncol + 1, 0);
  for (int c = 0; c < ncol; c++) el_color_ptr[c + 1] = el_color_ptr[c] + counts[c];
  GB_CUDA(cudaMemcpyAsync(cnt.p, el_color_ptr.data(), ncol * sizeof(int), cudaMemcpyHostToDevice, st));
  sg_color_fill<<<(nel + 255) / 256, 256, 0, st>>>(nel, state.p, cnt.p, el_perm.p);
  GB_CUDA(cudaGetLastError());
  GB_CUDA(cudaStreamSynchronize(st));
  return 0;
}

}  // namespace gbfem
