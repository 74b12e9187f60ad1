// SELL-32 construction and the sliced sparse product used by every apply.
//
// One thread per (block) row, one warp per 32-row slice, entries stored
// column-major inside the slice: the 32 lanes read 32 consecutive column
// indices and, for each block component, 32 consecutive values.  Every FP64
// instruction has all lanes busy (FP64 is the scarce unit on GB300); the row
// sum uses two interleaved accumulators to halve the dependent-FMA chain.

#include <atomic>
#include <cstdlib>
#include <cstdarg>
#include <cstdio>
#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "gbpc_common.cuh"
#include "gbpc_internal.h"

// ---------------------------------------------------------------------------
// Error reporting (thread-local message).

static thread_local std::string g_last_error = "no error";

void gbpc_set_error(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
}

void gbpc_set_error_cuda(cudaError_t e, const char* expr, const char* file, int line) {
  gbpc_set_error("CUDA error %s (%s) in %s at %s:%d", cudaGetErrorName(e), cudaGetErrorString(e),
                 expr, file, line);
}

extern "C" const char* gbpc_last_error(void) { return g_last_error.c_str(); }
extern "C" int gbpc_version(void) { return 1; }

extern "C" int gbpc_device_bytes(size_t* live_host) {
  if (!live_host) {
    gbpc_set_error("gbpc_device_bytes: null output");
    return GBPC_ERR_ARG;
  }
  *live_host = gbpc::device_bytes_live();
  return GBPC_OK;
}

namespace gbpc {

size_t dtype_size(int dtype) {
  switch (dtype) {
    case GBPC_F64: return 8;
    case GBPC_F32: return 4;
    case GBPC_BF16: return 2;
    default: return 0;
  }
}

bool valid_value_dtype(int d) { return d == GBPC_F64 || d == GBPC_F32 || d == GBPC_BF16; }

namespace {
std::atomic<size_t> g_live_bytes{0};
thread_local size_t* t_tally = nullptr;
thread_local bool t_pdl = false;
}  // namespace

bool pdl_active() {
  static const bool enabled = [] {
    const char* e = std::getenv("GBPC_PDL");
    return !(e && e[0] == '0');
  }();
  return t_pdl && enabled;
}
PdlScope::PdlScope(bool on) : prev(t_pdl) { t_pdl = on; }
PdlScope::~PdlScope() { t_pdl = prev; }

size_t* current_tally() { return t_tally; }
size_t device_bytes_live() { return g_live_bytes.load(); }

void note_release(size_t n, size_t* tally) {
  g_live_bytes.fetch_sub(n);
  if (tally) *tally -= n;
}

ByteTally::ByteTally(size_t* counter) : prev(t_tally) { t_tally = counter; }
ByteTally::~ByteTally() { t_tally = prev; }

int DevBuf::alloc(size_t n) {
  release();
  if (n == 0) n = 16;
  cudaError_t e = cudaMalloc(&p, n);
  if (e != cudaSuccess) {
    p = nullptr;
    gbpc_set_error("device allocation of %zu bytes failed: %s", n, cudaGetErrorString(e));
    return GBPC_ERR_NOMEM;
  }
  bytes = n;
  tally = t_tally;
  if (tally) *tally += n;
  g_live_bytes.fetch_add(n);
  return GBPC_OK;
}

int ReduceBuf::init(cudaStream_t st) {
  int rc = partials.alloc(sizeof(double) * kMaxCtas);
  if (rc) return rc;
  rc = counter.alloc(sizeof(unsigned int));
  if (rc) return rc;
  GBPC_CUDA_TRY(cudaMemsetAsync(counter.p, 0, sizeof(unsigned int), st));
  return GBPC_OK;
}

int vec_copy(void* dst, const void* src, size_t bytes, cudaStream_t st) {
  if (dst == src || bytes == 0) return GBPC_OK;
  GBPC_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, st));
  return GBPC_OK;
}

// ---------------------------------------------------------------------------
// SELL construction.

__device__ __forceinline__ bool keep_entry(int part, int src_row, int c) {
  return part == 0 || (part == 1 && c < src_row) || (part == 2 && c > src_row);
}

// Stored entries of each output row after the build filters.
__global__ void sell_length_kernel(int nrow, const int32_t* __restrict__ off,
                                   const int32_t* __restrict__ col, const int32_t* rows,
                                   const int32_t* colmap, int part, int32_t* len) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrow) return;
  const int src = rows ? rows[r] : r;
  int count = 0;
  if (colmap == nullptr && part == 0) {
    count = off[src + 1] - off[src];
  } else {
    for (int e = off[src]; e < off[src + 1]; ++e) {
      const int c = col[e];
      if (!keep_entry(part, src, c)) continue;
      if (colmap && colmap[c] < 0) continue;
      ++count;
    }
  }
  len[r] = count;
}

// Rows ordered by decreasing length inside windows of `window` rows (a stable
// counting sort per window, one thread per window), so that each 32-row slice
// holds rows of similar length and padding stays small.
// Rows are sorted by length inside windows when the plain layout would pad
// more than this fraction.
constexpr double kSortPadding = 0.10;
constexpr int kSortWindow = 256;

// Stable sort of each window's rows by length, longest first: one CTA per
// window, the thread of row r places it at its rank (rows longer than r, or
// as long and earlier).
__global__ void __launch_bounds__(kSortWindow)
window_sort_kernel(int nrow, const int32_t* __restrict__ len, int32_t* perm) {
  __shared__ int sl[kSortWindow];
  const int lo = blockIdx.x * kSortWindow;
  const int hi = min(nrow, lo + kSortWindow);
  const int k = threadIdx.x;
  sl[k] = lo + k < hi ? len[lo + k] : -1;
  __syncthreads();
  if (lo + k >= hi) return;
  const int mine = sl[k];
  int rank = 0;
  for (int q = 0; q < hi - lo; ++q) {
    const int o = sl[q];
    rank += (o > mine) || (o == mine && q < k);
  }
  perm[lo + rank] = lo + k;
}

__global__ void sell_width_kernel(int nrow, int nslices, const int32_t* __restrict__ len,
                                  const int32_t* perm, int64_t* slice_entries) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nslices) return;
  int width = 0;
  for (int l = 0; l < kSlice; ++l) {
    const int k = s * kSlice + l;
    if (k >= nrow) break;
    width = max(width, len[perm ? perm[k] : k]);
  }
  slice_entries[s] = (int64_t)width * kSlice;
}

__global__ void max_kernel(int n, const int32_t* __restrict__ v, int32_t* out) {
  int m = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    m = max(m, v[i]);
  atomicMax(out, m);
}

// Exclusive scan of int64 counts by a single CTA (setup only).
__global__ void scan_i64_kernel(const int64_t* in, int64_t* out, int n) {
  __shared__ int64_t carry;
  __shared__ int64_t buf[1024];
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < n; base += 1024) {
    const int i = base + threadIdx.x;
    const int64_t v = (i < n) ? in[i] : 0;
    buf[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
      const int64_t t = (threadIdx.x >= o) ? buf[threadIdx.x - o] : 0;
      __syncthreads();
      buf[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < n) out[i] = carry + buf[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == 1023) carry += buf[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[n] = carry;
}

template <typename VI, typename VO>
__device__ __forceinline__ VO convert_value(VI v);
template <> __device__ __forceinline__ double convert_value<double, double>(double v) { return v; }
template <> __device__ __forceinline__ float convert_value<double, float>(double v) { return __double2float_rn(v); }
template <> __device__ __forceinline__ __nv_bfloat16 convert_value<double, __nv_bfloat16>(double v) {
  return __float2bfloat16_rn(__double2float_rn(v));
}
template <> __device__ __forceinline__ float convert_value<float, float>(float v) { return v; }
template <> __device__ __forceinline__ double convert_value<float, double>(float v) { return (double)v; }
template <> __device__ __forceinline__ __nv_bfloat16 convert_value<float, __nv_bfloat16>(float v) {
  return __float2bfloat16_rn(v);
}
template <> __device__ __forceinline__ __nv_bfloat16 convert_value<__nv_bfloat16, __nv_bfloat16>(__nv_bfloat16 v) {
  return v;
}

template <typename VI, typename VO>
__global__ void sell_fill_kernel(int nrow, int nslices, int B, const int32_t* __restrict__ off,
                                 const int32_t* __restrict__ col, const VI* __restrict__ val,
                                 const int32_t* rows, const int32_t* colmap, int part,
                                 const VI* row_scale, const int32_t* perm,
                                 const int64_t* __restrict__ slice_ptr, int32_t* cols_out,
                                 VO* vals_out) {
  const int k_row = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = k_row / kSlice;
  if (s >= nslices) return;
  const int lane = k_row % kSlice;
  const int64_t base = slice_ptr[s];
  const int width = (int)((slice_ptr[s + 1] - base) / kSlice);
  const int BB = B * B;
  int k = 0;
  if (k_row < nrow) {
    const int r = perm ? perm[k_row] : k_row;
    const int src = rows ? rows[r] : r;
    for (int e = off[src]; e < off[src + 1]; ++e) {
      int c = col[e];
      if (!keep_entry(part, src, c)) continue;
      if (colmap) {
        c = colmap[c];
        if (c < 0) continue;
      }
      if (k >= width) break;  // never for the pattern the layout was built from
      const int64_t E = base + (int64_t)k * kSlice + lane;
      cols_out[E] = c;
      for (int q = 0; q < BB; ++q) {
        VI v = val[(int64_t)e * BB + q];
        if (row_scale) v = v * row_scale[src];
        vals_out[base * BB + ((int64_t)k * BB + q) * kSlice + lane] = convert_value<VI, VO>(v);
      }
      ++k;
    }
  }
  for (; k < width; ++k) {
    const int64_t E = base + (int64_t)k * kSlice + lane;
    cols_out[E] = -1;
    for (int q = 0; q < BB; ++q)
      vals_out[base * BB + ((int64_t)k * BB + q) * kSlice + lane] = convert_value<double, VO>(0.0);
  }
}

template <typename VI, typename VO>
static void launch_fill(const Sell& s, int B, const int32_t* off, const int32_t* col,
                        const void* val, const SellBuild& opt, cudaStream_t st) {
  const int threads = s.nslices * kSlice;
  sell_fill_kernel<VI, VO><<<grid_for(threads, kThreads), kThreads, 0, st>>>(
      s.nrow, s.nslices, B, off, col, (const VI*)val, opt.rows, opt.colmap, opt.part,
      (const VI*)opt.row_scale, s.perm.p ? s.perm.as<int32_t>() : nullptr,
      s.slice_ptr.as<int64_t>(), s.cols.as<int32_t>(), s.vals.as<VO>());
}

// Product schedule: the slices by width descending (stable), each entry
// {slice, width, first entry} as an int4, built on the host from slice_ptr.
// Rows still sum their entries in storage order; the schedule only decides
// which warp takes which slice (and so the order of a fused dot product's
// per-thread partial sums).
static int build_schedule(Sell& s, cudaStream_t st) {
  s.sched.release();
  if (s.nslices == 0) return GBPC_OK;
  std::vector<int64_t> ptr((size_t)s.nslices + 1);
  GBPC_CUDA_TRY(cudaMemcpyAsync(ptr.data(), s.slice_ptr.p, sizeof(int64_t) * ptr.size(),
                                cudaMemcpyDeviceToHost, st));
  GBPC_CUDA_TRY(cudaStreamSynchronize(st));
  std::vector<int> order((size_t)s.nslices);
  for (int i = 0; i < s.nslices; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return ptr[a + 1] - ptr[a] > ptr[b + 1] - ptr[b];
  });
  std::vector<int32_t> tasks((size_t)4 * s.nslices);
  for (int i = 0; i < s.nslices; ++i) {
    const int sl = order[i];
    const int64_t base = ptr[sl];
    const uint64_t ubase = (uint64_t)base;
    tasks[4 * (size_t)i] = sl;
    tasks[4 * (size_t)i + 1] = (int32_t)((ptr[sl + 1] - base) / kSlice);
    tasks[4 * (size_t)i + 2] = (int32_t)(uint32_t)(ubase & 0xffffffffu);
    tasks[4 * (size_t)i + 3] = (int32_t)(uint32_t)(ubase >> 32);
  }
  int rc = s.sched.alloc(sizeof(int32_t) * tasks.size());
  if (rc) return rc;
  if ((rc = s.err.alloc(sizeof(int32_t)))) return rc;
  GBPC_CUDA_TRY(cudaMemsetAsync(s.err.p, 0, sizeof(int32_t), st));
  GBPC_CUDA_TRY(cudaMemcpyAsync(s.sched.p, tasks.data(), sizeof(int32_t) * tasks.size(),
                                cudaMemcpyHostToDevice, st));
  GBPC_CUDA_TRY(cudaStreamSynchronize(st));
  return GBPC_OK;
}

int sell_build(Sell& s, int nrow_out, int ncol, int B, const int32_t* off, const int32_t* col,
               const void* val, int in_dtype, int out_dtype, const SellBuild& opt,
               cudaStream_t st) {
  if (B < 1 || B > 4) {
    gbpc_set_error("block size must be 1..4, got %d", B);
    return GBPC_ERR_ARG;
  }
  if (!valid_value_dtype(in_dtype) || !valid_value_dtype(out_dtype) ||
      (in_dtype == GBPC_BF16 && out_dtype != GBPC_BF16)) {
    gbpc_set_error("unsupported value dtype %d -> %d", in_dtype, out_dtype);
    return GBPC_ERR_ARG;
  }
  s.nrow = nrow_out;
  s.ncol = ncol;
  s.B = B;
  s.vdtype = out_dtype;
  s.nslices = (nrow_out + kSlice - 1) / kSlice;
  s.perm.release();
  int rc = s.slice_ptr.alloc(sizeof(int64_t) * (s.nslices + 1));
  if (rc) return rc;
  DevBuf counts, len, scratch;
  if ((rc = counts.alloc(sizeof(int64_t) * (s.nslices + 1)))) return rc;
  if ((rc = len.alloc(sizeof(int32_t) * (nrow_out + 1)))) return rc;
  if ((rc = scratch.alloc(sizeof(int32_t) * 2))) return rc;
  GBPC_CUDA_TRY(cudaMemsetAsync(scratch.p, 0, sizeof(int32_t) * 2, st));
  if (nrow_out > 0) {
    sell_length_kernel<<<grid_for(nrow_out, kThreads), kThreads, 0, st>>>(
        nrow_out, off, col, opt.rows, opt.colmap, opt.part, len.as<int32_t>());
    sell_width_kernel<<<grid_for(s.nslices, kThreads), kThreads, 0, st>>>(
        nrow_out, s.nslices, len.as<int32_t>(), nullptr, counts.as<int64_t>());
  }
  scan_i64_kernel<<<1, 1024, 0, st>>>(counts.as<int64_t>(), s.slice_ptr.as<int64_t>(), s.nslices);
  GBPC_CUDA_TRY(cudaGetLastError());
  if (nrow_out > 0)
    max_kernel<<<std::min(grid_for(nrow_out, kThreads), 1024), kThreads, 0, st>>>(
        nrow_out, len.as<int32_t>(), scratch.as<int32_t>());
  GBPC_CUDA_TRY(cudaGetLastError());
  int32_t maxlen = 0;
  GBPC_CUDA_TRY(cudaMemcpyAsync(&s.nent, s.slice_ptr.as<int64_t>() + s.nslices, sizeof(int64_t),
                                cudaMemcpyDeviceToHost, st));
  GBPC_CUDA_TRY(cudaMemcpyAsync(&maxlen, scratch.p, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  GBPC_CUDA_TRY(cudaStreamSynchronize(st));
  // Try rows sorted by length inside windows; keep that layout when it saves
  // more than kSortPadding of the stored entries.
  if (nrow_out > kSlice && maxlen > 0) {
    DevBuf perm, counts2, ptr2;
    if ((rc = perm.alloc(sizeof(int32_t) * nrow_out))) return rc;
    if ((rc = counts2.alloc(sizeof(int64_t) * (s.nslices + 1)))) return rc;
    if ((rc = ptr2.alloc(sizeof(int64_t) * (s.nslices + 1)))) return rc;
    const int nwin = (nrow_out + kSortWindow - 1) / kSortWindow;
    window_sort_kernel<<<nwin, kSortWindow, 0, st>>>(nrow_out, len.as<int32_t>(),
                                                    perm.as<int32_t>());
    sell_width_kernel<<<grid_for(s.nslices, kThreads), kThreads, 0, st>>>(
        nrow_out, s.nslices, len.as<int32_t>(), perm.as<int32_t>(), counts2.as<int64_t>());
    scan_i64_kernel<<<1, 1024, 0, st>>>(counts2.as<int64_t>(), ptr2.as<int64_t>(), s.nslices);
    GBPC_CUDA_TRY(cudaGetLastError());
    int64_t nent2 = 0;
    GBPC_CUDA_TRY(cudaMemcpyAsync(&nent2, ptr2.as<int64_t>() + s.nslices, sizeof(int64_t),
                                  cudaMemcpyDeviceToHost, st));
    GBPC_CUDA_TRY(cudaStreamSynchronize(st));
    if ((double)nent2 < (double)s.nent * (1.0 - kSortPadding)) {
      std::swap(s.perm.p, perm.p);
      std::swap(s.perm.bytes, perm.bytes);
      std::swap(s.slice_ptr.p, ptr2.p);
      std::swap(s.slice_ptr.bytes, ptr2.bytes);
      s.nent = nent2;
    }
  }
  if ((rc = build_schedule(s, st))) return rc;
  if ((rc = s.cols.alloc(sizeof(int32_t) * s.nent))) return rc;
  if ((rc = s.vals.alloc(dtype_size(out_dtype) * s.nent * B * B))) return rc;
  if (s.nslices > 0) {
    if (in_dtype == GBPC_BF16) {
      launch_fill<__nv_bfloat16, __nv_bfloat16>(s, B, off, col, val, opt, st);
    } else if (in_dtype == GBPC_F64) {
      if (out_dtype == GBPC_F64) launch_fill<double, double>(s, B, off, col, val, opt, st);
      else if (out_dtype == GBPC_F32) launch_fill<double, float>(s, B, off, col, val, opt, st);
      else launch_fill<double, __nv_bfloat16>(s, B, off, col, val, opt, st);
    } else {
      if (out_dtype == GBPC_F64) launch_fill<float, double>(s, B, off, col, val, opt, st);
      else if (out_dtype == GBPC_F32) launch_fill<float, float>(s, B, off, col, val, opt, st);
      else launch_fill<float, __nv_bfloat16>(s, B, off, col, val, opt, st);
    }
  }
  GBPC_CUDA_TRY(cudaGetLastError());
  GBPC_CUDA_TRY(cudaStreamSynchronize(st));
  return GBPC_OK;
}

// Rows whose stored length exceeds the width of their slice.
__global__ void sell_fits_kernel(int nrow, const int32_t* __restrict__ len,
                                 const int32_t* __restrict__ perm,
                                 const int64_t* __restrict__ slice_ptr, int32_t* bad) {
  const int k_row = blockIdx.x * blockDim.x + threadIdx.x;
  if (k_row >= nrow) return;
  const int sl = k_row / kSlice;
  const int r = perm ? perm[k_row] : k_row;
  const int64_t width = (slice_ptr[sl + 1] - slice_ptr[sl]) / kSlice;
  if (len[r] > width) atomicAdd(bad, 1);
}

// New values for an unchanged pattern: the fill pass again over the existing
// layout (slices, row order, columns), writing vals in place, so captured
// products see them.  Rejects a pattern whose rows do not fit the layout.
int sell_refill(Sell& s, const int32_t* off, const int32_t* col, const void* val, int in_dtype,
                const SellBuild& opt, cudaStream_t st) {
  const int out_dtype = s.vdtype;
  if (!valid_value_dtype(in_dtype) || (in_dtype == GBPC_BF16 && out_dtype != GBPC_BF16)) {
    gbpc_set_error("unsupported value dtype %d -> %d", in_dtype, out_dtype);
    return GBPC_ERR_ARG;
  }
  if (s.nrow > 0) {
    DevBuf len, bad;
    int rc;
    if ((rc = len.alloc(sizeof(int32_t) * (s.nrow + 1)))) return rc;
    if ((rc = bad.alloc(sizeof(int32_t)))) return rc;
    GBPC_CUDA_TRY(cudaMemsetAsync(bad.p, 0, sizeof(int32_t), st));
    sell_length_kernel<<<grid_for(s.nrow, kThreads), kThreads, 0, st>>>(
        s.nrow, off, col, opt.rows, opt.colmap, opt.part, len.as<int32_t>());
    sell_fits_kernel<<<grid_for(s.nrow, kThreads), kThreads, 0, st>>>(
        s.nrow, len.as<int32_t>(), s.perm.p ? s.perm.as<int32_t>() : nullptr,
        s.slice_ptr.as<int64_t>(), bad.as<int32_t>());
    GBPC_CUDA_TRY(cudaGetLastError());
    int32_t h = 0;
    GBPC_CUDA_TRY(cudaMemcpyAsync(&h, bad.p, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    GBPC_CUDA_TRY(cudaStreamSynchronize(st));
    if (h) {
      gbpc_set_error("refill: %d rows do not fit the operator's layout (pattern changed)", h);
      return GBPC_ERR_ARG;
    }
  }
  if (s.nslices > 0) {
    if (in_dtype == GBPC_BF16) {
      launch_fill<__nv_bfloat16, __nv_bfloat16>(s, s.B, off, col, val, opt, st);
    } else if (in_dtype == GBPC_F64) {
      if (out_dtype == GBPC_F64) launch_fill<double, double>(s, s.B, off, col, val, opt, st);
      else if (out_dtype == GBPC_F32) launch_fill<double, float>(s, s.B, off, col, val, opt, st);
      else launch_fill<double, __nv_bfloat16>(s, s.B, off, col, val, opt, st);
    } else {
      if (out_dtype == GBPC_F64) launch_fill<float, double>(s, s.B, off, col, val, opt, st);
      else if (out_dtype == GBPC_F32) launch_fill<float, float>(s, s.B, off, col, val, opt, st);
      else launch_fill<float, __nv_bfloat16>(s, s.B, off, col, val, opt, st);
    }
  }
  GBPC_CUDA_TRY(cudaGetLastError());
  return GBPC_OK;
}

// ---------------------------------------------------------------------------
// Product entry point (kernels in gbpc_spmv.cuh, instantiated per vector type
// in gbpc_spmv_f64.cu and gbpc_spmv_f32.cu).

int spmv_f64(const Sell& m, const void* x, const void* y, void* z, double alpha, double beta,
             const int* guard, const EpiHost& ep, const Reduction& red, cudaStream_t st);
int spmv_f32(const Sell& m, const void* x, const void* y, void* z, double alpha, double beta,
             const int* guard, const EpiHost& ep, const Reduction& red, cudaStream_t st);

int sell_spmv(const Sell& m, int adtype, const void* x, const void* y, void* z, double alpha,
              double beta, const int* guard, const EpiHost& ep, const DotSpec* dot,
              cudaStream_t st) {
  Reduction red{};
  if (dot != nullptr && dot->w != nullptr) {
    // The weight is float64 whatever the product's vectors; a float32
    // output is widened before it is multiplied (the float32-applied
    // preconditioner inside the float64 CG loop).
    red.w = dot->w;
    red.partials = dot->rb->partials.as<double>();
    red.counter = dot->rb->counter.as<unsigned int>();
    red.mode = dot->mode;
    red.ks = (KrylovScalars*)dot->ks;
    red.out = dot->out;
  }
  int rc;
  if (adtype == GBPC_F64) rc = spmv_f64(m, x, y, z, alpha, beta, guard, ep, red, st);
  else if (adtype == GBPC_F32) rc = spmv_f32(m, x, y, z, alpha, beta, guard, ep, red, st);
  else {
    gbpc_set_error("vector dtype must be float64 or float32");
    return GBPC_ERR_ARG;
  }
  if (rc) return rc;
  GBPC_CUDA_TRY(cudaGetLastError());
  return GBPC_OK;
}

// Kernel variants timed by the autotuner (scalar rows; must match
// launch_variant in gbpc_spmv.cuh).
constexpr int kNumVariants = 6;

// The software-pipelined variant is the default: inside Krylov iterations
// (matrix streamed from HBM, input vector warm) it was the fastest or within
// 2 % on every product of the 70^3 biharmonic solve (forward and backward
// factored operator, G, G^T).  Another variant replaces it only when it is
// clearly faster (kSwitchMargin) in the timing below, as can happen on rows
// much wider than these.
constexpr int kDefaultVariant = 4;
constexpr float kSwitchMargin = 0.90f;

int sell_autotune(Sell& m, int adtype, cudaStream_t st) {
  // Blocked rows: 2 x 2 and 3 x 3 blocks choose between the one-slice
  // kernel (0) and the pipelined blocked kernel (4); other sizes run 0.
  const bool blocked = m.B != 1;
  if (m.nslices == 0 || m.B > 3) {
    m.variant = 0;
    return GBPC_OK;
  }
  // GBPC_SPMV_VARIANT=0..kNumVariants-1 fixes the variant (tests and
  // tuning); every variant gives the same results.  Blocked rows run
  // variant 4 as the pipelined blocked kernel and 1..3 as 0.
  if (const char* e = std::getenv("GBPC_SPMV_VARIANT")) {
    if (e[0] >= '0' && e[0] <= '9' && e[1] == '\0' && e[0] - '0' < kNumVariants) {
      m.variant = e[0] - '0';
      return GBPC_OK;
    }
  }
  // Fewer slices than warps in one grid (kSms CTAs of kThreads): the
  // product is launch-latency-bound and timing the variants measures noise,
  // so the default stands without the timed launches.
  if (m.nslices < kSms * (kThreads / 32)) {
    m.variant = blocked ? 0 : kDefaultVariant;
    return GBPC_OK;
  }
  const size_t vs = dtype_size(adtype);
  DevBuf x, z;
  int rc;
  // Scalar lengths: nrow and ncol count B x B blocks.
  const size_t xbytes = vs * (size_t)std::max(m.ncol, 1) * m.B;
  const size_t zbytes = vs * (size_t)std::max(m.nrow, 1) * m.B;
  if ((rc = x.alloc(xbytes))) return rc;
  if ((rc = z.alloc(zbytes))) return rc;
  GBPC_CUDA_TRY(cudaMemsetAsync(x.p, 0, xbytes, st));
  cudaEvent_t e0, e1;
  GBPC_CUDA_TRY(cudaEventCreate(&e0));
  GBPC_CUDA_TRY(cudaEventCreate(&e1));
  float ms[kNumVariants];
  for (int v = 0; v < kNumVariants && !rc; ++v) {
    ms[v] = 1e30f;
    if (blocked && v != 0 && v != 4) continue;
    if (v == 5) continue;  // the bulk-copy variant runs only when GBPC_SPMV_VARIANT=5 selects it
    m.variant = v;
    for (int w = 0; w < 2 && !rc; ++w)
      rc = sell_spmv(m, adtype, x.p, nullptr, z.p, 1.0, 0.0, nullptr, EpiHost{}, nullptr, st);
    cudaEventRecord(e0, st);
    for (int w = 0; w < 5 && !rc; ++w)
      rc = sell_spmv(m, adtype, x.p, nullptr, z.p, 1.0, 0.0, nullptr, EpiHost{}, nullptr, st);
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    ms[v] = 0.f;
    cudaEventElapsedTime(&ms[v], e0, e1);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  int best_v = kDefaultVariant;
  if (blocked) {
    best_v = ms[4] < ms[0] ? 4 : 0;
  } else {
    for (int v = 0; v < kNumVariants && !rc; ++v)
      if (ms[v] < kSwitchMargin * ms[kDefaultVariant] && ms[v] < ms[best_v]) best_v = v;
  }
  m.variant = best_v;
  if (rc) return rc;
  GBPC_CUDA_TRY(cudaGetLastError());
  return GBPC_OK;
}

}  // namespace gbpc
