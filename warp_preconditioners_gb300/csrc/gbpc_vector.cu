// Vector utilities behind the host-side helpers that the reference gets from
// Warp: seeded Rademacher probes (FSAI.quality), z = alpha x + beta y and a
// deterministic dot product (the Krylov loop for operators defined in
// Python, and float32 systems), plus an FP64 FMA throughput probe that the
// benchmark divides by.
//
// All entry points are stream-ordered and allocate nothing; the dot product
// takes a caller-owned work array of gbpc_vec_dot_work_size() doubles.

#include <algorithm>

#include "gbpc_common.cuh"
#include "gbpc_internal.h"

namespace gbpc {
namespace {

// The PCG hash of Jarzynski and Olano ("Hash Functions for GPU Rendering",
// JCGT 9(3), 2020), on which Warp's rand_init / randi streams are built: a
// state seeded from (seed, offset) as pcg(seed + pcg(offset)), and each draw
// replaces the state by its hash.
__device__ __forceinline__ uint32_t pcg_hash(uint32_t v) {
  const uint32_t state = v * 747796405u + 2891336453u;
  const uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
  return (word >> 22u) ^ word;
}

// out[i] = 2 randi(rand_init(seed, i), 0, 2) - 1, the probe of
// warp_preconditioners/fsai_reuse.py:143-147 (randi(state, lo, hi) draws
// lo + state % (hi - lo) from the advanced unsigned state).
template <typename T>
__global__ void rademacher_kernel(int64_t n, uint32_t seed, T* out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t state = pcg_hash(seed + pcg_hash((uint32_t)i));
    const uint32_t draw = pcg_hash(state);
    out[i] = (T)(2 * (int)(draw % 2u) - 1);
  }
}

template <typename T>
__global__ void axpby_kernel(int64_t n, T alpha, const T* x, T beta, const T* y, T* z, int flags) {
  // flags: 1 = alpha is zero (x never read), 2 = beta is zero (y never read)
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    T v = T(0);
    if (!(flags & 1)) v = alpha * x[i];
    if (!(flags & 2)) v = (flags & 1) ? beta * y[i] : v + beta * y[i];
    z[i] = v;
  }
}

constexpr int kDotCtas = 2 * kSms;
constexpr int kDotThreads = 512;

// Per-CTA partial sums in double (fixed grid, fixed tree), then one CTA adds
// the partials in index order: the same result on every run.
template <typename T>
__global__ void __launch_bounds__(kDotThreads)
dot_partials_kernel(int64_t n, const T* x, const T* y, double* partials) {
  __shared__ double sh[kDotThreads / 32];
  double part = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kDotThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kDotThreads)
    part = fma((double)x[i], (double)y[i], part);
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = part;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < kDotThreads / 32 ? sh[threadIdx.x] : 0.0;
    for (int o = 8; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) partials[blockIdx.x] = v;
  }
}

__global__ void dot_final_kernel(const double* partials, int count, double* out) {
  double v = 0.0;
  for (int i = threadIdx.x; i < count; i += 32) v += partials[i];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (threadIdx.x == 0) *out = v;
}

// Eight independent FMA chains per thread, `iters` rounds: 8 * iters FMAs a
// thread.  The chains' inputs come from the thread index, so nothing is
// known at compile time, and the sum is stored so nothing is dropped.
__global__ void __launch_bounds__(256) fma_probe_kernel(int64_t iters, double* out) {
  const double t = 1.0 + 1e-9 * (double)(blockIdx.x * blockDim.x + threadIdx.x);
  double a0 = t, a1 = t + 1, a2 = t + 2, a3 = t + 3, a4 = t + 4, a5 = t + 5, a6 = t + 6, a7 = t + 7;
  const double m = 0.999999999, c = 1e-12;
  for (int64_t k = 0; k < iters; ++k) {
    a0 = fma(a0, m, c);
    a1 = fma(a1, m, c);
    a2 = fma(a2, m, c);
    a3 = fma(a3, m, c);
    a4 = fma(a4, m, c);
    a5 = fma(a5, m, c);
    a6 = fma(a6, m, c);
    a7 = fma(a7, m, c);
  }
  const double s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
  if (s == 12345.0) out[0] = s;  // practically never; keeps the chains live
  if (blockIdx.x == 0 && threadIdx.x == 0) out[1] = s;
}

int grid_for_vec(int64_t n) {
  int64_t g = (n + 255) / 256;
  if (g > 4 * kSms) g = 4 * kSms;
  return g < 1 ? 1 : (int)g;
}

}  // namespace
}  // namespace gbpc

using namespace gbpc;

extern "C" int gbpc_rademacher(int64_t n, int seed, int dtype, void* out, void* stream) {
  if (n < 0 || (n > 0 && !out) || (dtype != GBPC_F64 && dtype != GBPC_F32)) {
    gbpc_set_error("gbpc_rademacher: bad arguments");
    return GBPC_ERR_ARG;
  }
  if (n == 0) return GBPC_OK;
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == GBPC_F64)
    rademacher_kernel<double><<<grid_for_vec(n), 256, 0, st>>>(n, (uint32_t)seed, (double*)out);
  else
    rademacher_kernel<float><<<grid_for_vec(n), 256, 0, st>>>(n, (uint32_t)seed, (float*)out);
  GBPC_CUDA_TRY(cudaGetLastError());
  return GBPC_OK;
}

extern "C" int gbpc_vec_axpby(int64_t n, int dtype, double alpha, const void* x, double beta,
                              const void* y, void* z, void* stream) {
  const int flags = (alpha == 0.0 ? 1 : 0) | (beta == 0.0 ? 2 : 0);
  if (n < 0 || (n > 0 && (!z || (!(flags & 1) && !x) || (!(flags & 2) && !y))) ||
      (dtype != GBPC_F64 && dtype != GBPC_F32)) {
    gbpc_set_error("gbpc_vec_axpby: bad arguments");
    return GBPC_ERR_ARG;
  }
  if (n == 0) return GBPC_OK;
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == GBPC_F64)
    axpby_kernel<double><<<grid_for_vec(n), 256, 0, st>>>(n, alpha, (const double*)x, beta,
                                                          (const double*)y, (double*)z, flags);
  else
    axpby_kernel<float><<<grid_for_vec(n), 256, 0, st>>>(n, (float)alpha, (const float*)x,
                                                         (float)beta, (const float*)y, (float*)z,
                                                         flags);
  GBPC_CUDA_TRY(cudaGetLastError());
  return GBPC_OK;
}

extern "C" int gbpc_vec_dot_work_size(void) { return kDotCtas; }

extern "C" int gbpc_vec_dot(int64_t n, int dtype, const void* x, const void* y, double* work,
                            double* result, void* stream) {
  if (n < 0 || !work || !result || (n > 0 && (!x || !y)) ||
      (dtype != GBPC_F64 && dtype != GBPC_F32)) {
    gbpc_set_error("gbpc_vec_dot: bad arguments");
    return GBPC_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  int g = (int)std::min<int64_t>((n + kDotThreads - 1) / kDotThreads, kDotCtas);
  if (g < 1) g = 1;
  if (dtype == GBPC_F64)
    dot_partials_kernel<double><<<g, kDotThreads, 0, st>>>(n, (const double*)x, (const double*)y,
                                                           work);
  else
    dot_partials_kernel<float><<<g, kDotThreads, 0, st>>>(n, (const float*)x, (const float*)y,
                                                          work);
  GBPC_CUDA_TRY(cudaGetLastError());
  dot_final_kernel<<<1, 32, 0, st>>>(work, g, result);
  GBPC_CUDA_TRY(cudaGetLastError());
  return GBPC_OK;
}

extern "C" int gbpc_fma_probe(int64_t iters, int ctas, double* out, void* stream) {
  if (iters < 1 || ctas < 1 || !out) {
    gbpc_set_error("gbpc_fma_probe: bad arguments");
    return GBPC_ERR_ARG;
  }
  fma_probe_kernel<<<ctas, 256, 0, (cudaStream_t)stream>>>(iters, out);
  GBPC_CUDA_TRY(cudaGetLastError());
  return GBPC_OK;
}
