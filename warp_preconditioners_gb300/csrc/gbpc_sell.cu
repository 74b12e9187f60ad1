// SELL-32 construction and the sliced sparse product used by every apply.
//
// One thread per (block) row, one warp per 32-row slice, entries stored
// column-major inside the slice: the 32 lanes read 32 consecutive column
// indices and, for each block component, 32 consecutive values.  Every FP64
// instruction has all lanes busy (FP64 is the scarce unit on GB300); the row
// sum uses two interleaved accumulators to halve the dependent-FMA chain.

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

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

__global__ void sell_width_kernel(int nrow, int nslices, const int32_t* __restrict__ off,
                                  const int32_t* __restrict__ col, const int32_t* rows,
                                  const int32_t* colmap, int part, int64_t* slice_entries) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nslices) return;
  int width = 0;
  for (int l = 0; l < kSlice; ++l) {
    const int r = s * kSlice + l;
    if (r >= nrow) break;
    const int src = rows ? rows[r] : r;
    int count = 0;
    if (rows == nullptr && colmap == nullptr && part == 0) {
      count = off[src + 1] - off[src];
    } else {
      for (int e = off[src]; e < off[src + 1]; ++e) {
        const int c = col[e];
        if (!keep_entry(part, src, c)) continue;
        if (colmap && colmap[c] < 0) continue;
        ++count;
      }
    }
    width = max(width, count);
  }
  slice_entries[s] = (int64_t)width * kSlice;
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
                                 const VI* row_scale, const int64_t* __restrict__ slice_ptr,
                                 int32_t* cols_out, VO* vals_out) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = r / kSlice;
  if (s >= nslices) return;
  const int lane = r % kSlice;
  const int64_t base = slice_ptr[s];
  const int width = (int)((slice_ptr[s + 1] - base) / kSlice);
  const int BB = B * B;
  int k = 0;
  if (r < nrow) {
    const int src = rows ? rows[r] : r;
    for (int e = off[src]; e < off[src + 1]; ++e) {
      int c = col[e];
      if (!keep_entry(part, src, c)) continue;
      if (colmap) {
        c = colmap[c];
        if (c < 0) continue;
      }
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
      (const VI*)opt.row_scale, s.slice_ptr.as<int64_t>(), s.cols.as<int32_t>(), s.vals.as<VO>());
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
  int rc = s.slice_ptr.alloc(sizeof(int64_t) * (s.nslices + 1));
  if (rc) return rc;
  DevBuf counts;
  if ((rc = counts.alloc(sizeof(int64_t) * (s.nslices + 1)))) return rc;
  if (s.nslices > 0) {
    sell_width_kernel<<<grid_for(s.nslices, kThreads), kThreads, 0, st>>>(
        nrow_out, s.nslices, off, col, opt.rows, opt.colmap, opt.part, counts.as<int64_t>());
  }
  scan_i64_kernel<<<1, 1024, 0, st>>>(counts.as<int64_t>(), s.slice_ptr.as<int64_t>(), s.nslices);
  GBPC_CUDA_TRY(cudaGetLastError());
  GBPC_CUDA_TRY(cudaMemcpyAsync(&s.nent, s.slice_ptr.as<int64_t>() + s.nslices, sizeof(int64_t),
                                cudaMemcpyDeviceToHost, st));
  GBPC_CUDA_TRY(cudaStreamSynchronize(st));
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
  return GBPC_OK;
}

// ---------------------------------------------------------------------------
// The sliced product.
//
// One warp per slice, slices distributed over a grid that fills the GPU.  For
// each chunk of entries the warp first issues every column-index load, then
// every value load and x gather, then the FMAs, so each lane keeps a whole
// chunk of independent memory requests in flight.  alpha/beta tests are
// uniform integer flags computed on the host: FP64 compares would take FP64
// issue slots, the scarce resource on this GPU.

template <typename A>
struct EpiDev {
  const A* aux0;
  const A* aux1;
};

template <typename A>
__device__ __forceinline__ A fma_t(A a, A b, A c);
template <> __device__ __forceinline__ double fma_t<double>(double a, double b, double c) { return fma(a, b, c); }
template <> __device__ __forceinline__ float fma_t<float>(float a, float b, float c) { return fmaf(a, b, c); }

enum SpmvFlags : int { F_ALPHA_ZERO = 1, F_ALPHA_ONE = 2, F_BETA_ZERO = 4 };

template <int B> struct Chunk { static constexpr int value = 8; };
template <> struct Chunk<2> { static constexpr int value = 4; };
template <> struct Chunk<3> { static constexpr int value = 2; };
template <> struct Chunk<4> { static constexpr int value = 2; };

template <int B, typename V, typename A, int EPI, bool DOT>
__global__ void __launch_bounds__(kThreads)
sell_spmv_kernel(SellView<V> m, const A* x, const A* y, A* z, A alpha, A beta, int flags,
                 const int* guard, EpiDev<A> ep, Reduction red) {
  if (guard_off(guard)) return;
  constexpr int BB = B * B;
  constexpr int CH = Chunk<B>::value;
  const bool run = (EPI == EPI_TRI_LOWER || EPI == EPI_TRI_UPPER) || !(flags & F_ALPHA_ZERO);
  const bool alpha_one = (flags & F_ALPHA_ONE) != 0;
  const bool beta_zero = (flags & F_BETA_ZERO) != 0;
  const int lane = threadIdx.x & 31;
  const int warps_total = gridDim.x * (kThreads / 32);
  double dot_part = 0.0;
  for (int s = blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5); s < m.nslices; s += warps_total) {
    const int row = s * kSlice + lane;
    const int64_t base = __ldg(m.slice_ptr + s);
    const int width = (int)((__ldg(m.slice_ptr + s + 1) - base) >> 5);
    A acc[B];
#pragma unroll
    for (int r = 0; r < B; ++r) acc[r] = A(0);
    if (run) {
      const int32_t* cp = m.cols + base + lane;
      const V* vp = m.vals + base * BB + lane;
      for (int k0 = 0; k0 < width; k0 += CH) {
        int c[CH];
#pragma unroll
        for (int j = 0; j < CH; ++j)
          c[j] = (k0 + j < width) ? __ldg(cp + (int64_t)(k0 + j) * kSlice) : -1;
        A xv[CH][B];
        V vv[CH][BB];
#pragma unroll
        for (int j = 0; j < CH; ++j) {
#pragma unroll
          for (int q = 0; q < B; ++q) xv[j][q] = (c[j] >= 0) ? __ldg(x + (int64_t)c[j] * B + q) : A(0);
#pragma unroll
          for (int q = 0; q < BB; ++q)
            vv[j][q] = (k0 + j < width) ? __ldg(vp + ((int64_t)(k0 + j) * BB + q) * kSlice)
                                        : static_cast<V>(0.0f);
        }
#pragma unroll
        for (int j = 0; j < CH; ++j) {
          if (k0 + j < width) {  // uniform across the warp
#pragma unroll
            for (int r = 0; r < B; ++r)
#pragma unroll
              for (int q = 0; q < B; ++q) acc[r] = fma_t<A>(widen<A, V>(vv[j][r * B + q]), xv[j][q], acc[r]);
          }
        }
      }
    }
    if (row < m.nrow) {
      A out[B];
#pragma unroll
      for (int r = 0; r < B; ++r) {
        const int64_t idx = (int64_t)row * B + r;
        if (EPI == EPI_AXPBY) {
          A v = alpha_one ? acc[r] : alpha * acc[r];
          if (!beta_zero) v = fma_t<A>(beta, y[idx], v);
          out[r] = v;
        } else if (EPI == EPI_SQLAP_BWD) {
          A v = A(0);
          if (run) {
            v = fma_t<A>(ep.aux0[idx], ep.aux1[idx], acc[r]);
            if (!alpha_one) v = alpha * v;
          }
          if (!beta_zero) v = fma_t<A>(beta, y[idx], v);
          out[r] = v;
        } else if (EPI == EPI_SQLAP_FWD) {
          out[r] = ep.aux0[idx] * acc[r];
        } else {
          out[r] = ep.aux0[idx] - acc[r];
        }
      }
      if (EPI == EPI_TRI_UPPER) {
        A t[B];
#pragma unroll
        for (int r = 0; r < B; ++r) {
          A s2 = A(0);
#pragma unroll
          for (int q = 0; q < B; ++q) s2 = fma_t<A>(ep.aux1[(int64_t)row * BB + r * B + q], out[q], s2);
          t[r] = s2;
        }
#pragma unroll
        for (int r = 0; r < B; ++r) out[r] = t[r];
      }
#pragma unroll
      for (int r = 0; r < B; ++r) {
        const int64_t idx = (int64_t)row * B + r;
        z[idx] = out[r];
        if (DOT) dot_part = fma((double)out[r], red.w[idx], dot_part);
      }
    }
  }
  if (DOT) reduce_and_finalize(red, dot_part);
}

static int spmv_grid(int nslices) {
  // One slice per warp, at most one wave of resident CTAs.
  const int warps_per_cta = kThreads / 32;
  int g = (nslices + warps_per_cta - 1) / warps_per_cta;
  if (g < 1) g = 1;
  if (g > kMaxCtas) g = kMaxCtas;
  return g;
}

static int spmv_flags(double alpha, double beta) {
  int f = 0;
  if (alpha == 0.0) f |= F_ALPHA_ZERO;
  if (alpha == 1.0) f |= F_ALPHA_ONE;
  if (beta == 0.0) f |= F_BETA_ZERO;
  return f;
}

template <int B, typename V, typename A, int EPI>
static void launch_spmv(const Sell& m, const void* x, const void* y, void* z, double alpha,
                        double beta, const int* guard, const EpiHost& ep, const Reduction& red,
                        cudaStream_t st) {
  SellView<V> view{m.nrow, m.nslices, m.slice_ptr.as<int64_t>(), m.cols.as<int32_t>(),
                   m.vals.as<V>()};
  EpiDev<A> e{(const A*)ep.aux0, (const A*)ep.aux1};
  const int flags = spmv_flags(alpha, beta);
  if (red.w != nullptr)
    sell_spmv_kernel<B, V, A, EPI, true><<<spmv_grid(m.nslices), kThreads, 0, st>>>(
        view, (const A*)x, (const A*)y, (A*)z, (A)alpha, (A)beta, flags, guard, e, red);
  else
    sell_spmv_kernel<B, V, A, EPI, false><<<spmv_grid(m.nslices), kThreads, 0, st>>>(
        view, (const A*)x, (const A*)y, (A*)z, (A)alpha, (A)beta, flags, guard, e, red);
}

template <int B, typename V, typename A>
static int dispatch_epi(const Sell& m, const void* x, const void* y, void* z, double alpha,
                        double beta, const int* guard, const EpiHost& ep, const Reduction& red,
                        cudaStream_t st) {
  switch (ep.kind) {
    case EPI_AXPBY: launch_spmv<B, V, A, EPI_AXPBY>(m, x, y, z, alpha, beta, guard, ep, red, st); break;
    case EPI_TRI_LOWER: launch_spmv<B, V, A, EPI_TRI_LOWER>(m, x, y, z, alpha, beta, guard, ep, red, st); break;
    case EPI_TRI_UPPER: launch_spmv<B, V, A, EPI_TRI_UPPER>(m, x, y, z, alpha, beta, guard, ep, red, st); break;
    case EPI_SQLAP_FWD:
      if (B != 1) return GBPC_ERR_ARG;
      launch_spmv<1, V, A, EPI_SQLAP_FWD>(m, x, y, z, alpha, beta, guard, ep, red, st);
      break;
    case EPI_SQLAP_BWD:
      if (B != 1) return GBPC_ERR_ARG;
      launch_spmv<1, V, A, EPI_SQLAP_BWD>(m, x, y, z, alpha, beta, guard, ep, red, st);
      break;
    default: return GBPC_ERR_ARG;
  }
  return GBPC_OK;
}

template <int B, typename A>
static int dispatch_v(const Sell& m, const void* x, const void* y, void* z, double alpha,
                      double beta, const int* guard, const EpiHost& ep, const Reduction& red,
                      cudaStream_t st) {
  switch (m.vdtype) {
    case GBPC_F64:
      if (sizeof(A) == 4) break;  // float64 storage needs float64 vectors
      return dispatch_epi<B, double, A>(m, x, y, z, alpha, beta, guard, ep, red, st);
    case GBPC_F32: return dispatch_epi<B, float, A>(m, x, y, z, alpha, beta, guard, ep, red, st);
    case GBPC_BF16: return dispatch_epi<B, __nv_bfloat16, A>(m, x, y, z, alpha, beta, guard, ep, red, st);
  }
  gbpc_set_error("unsupported storage/vector dtype combination %d/%d", m.vdtype, (int)sizeof(A));
  return GBPC_ERR_ARG;
}

int sell_spmv(const Sell& m, int adtype, const void* x, const void* y, void* z, double alpha,
              double beta, const int* guard, const EpiHost& ep, const DotSpec* dot,
              cudaStream_t st) {
  Reduction red{};
  if (dot != nullptr && dot->w != nullptr) {
    red.w = dot->w;
    red.partials = dot->rb->partials.as<double>();
    red.counter = dot->rb->counter.as<unsigned int>();
    red.mode = dot->mode;
    red.ks = (KrylovScalars*)dot->ks;
    red.out = dot->out;
  }
  int rc;
  if (adtype == GBPC_F64) {
    switch (m.B) {
      case 1: rc = dispatch_v<1, double>(m, x, y, z, alpha, beta, guard, ep, red, st); break;
      case 2: rc = dispatch_v<2, double>(m, x, y, z, alpha, beta, guard, ep, red, st); break;
      case 3: rc = dispatch_v<3, double>(m, x, y, z, alpha, beta, guard, ep, red, st); break;
      case 4: rc = dispatch_v<4, double>(m, x, y, z, alpha, beta, guard, ep, red, st); break;
      default: rc = GBPC_ERR_ARG;
    }
  } else if (adtype == GBPC_F32) {
    if (dot != nullptr && dot->w != nullptr) {
      gbpc_set_error("fused dot products need float64 vectors");
      return GBPC_ERR_ARG;
    }
    switch (m.B) {
      case 1: rc = dispatch_v<1, float>(m, x, y, z, alpha, beta, guard, ep, red, st); break;
      case 2: rc = dispatch_v<2, float>(m, x, y, z, alpha, beta, guard, ep, red, st); break;
      case 3: rc = dispatch_v<3, float>(m, x, y, z, alpha, beta, guard, ep, red, st); break;
      case 4: rc = dispatch_v<4, float>(m, x, y, z, alpha, beta, guard, ep, red, st); break;
      default: rc = GBPC_ERR_ARG;
    }
  } else {
    gbpc_set_error("vector dtype must be float64 or float32");
    return GBPC_ERR_ARG;
  }
  if (rc) return rc;
  GBPC_CUDA_TRY(cudaGetLastError());
  return GBPC_OK;
}

}  // namespace gbpc
