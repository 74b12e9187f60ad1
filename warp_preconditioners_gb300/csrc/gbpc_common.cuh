// Shared device-side definitions for the GB300 preconditioned-Krylov library.
//
// Storage formats
//   * CSR / BSR: the reference's canonical compact layout (sorted, unique
//     column indices per row; b x b blocks stored row-major).
//   * SELL-32: "sliced ELL" with 32 (block) rows per slice, stored
//     column-major inside each slice so that the 32 lanes of a warp read 32
//     consecutive words.  Padding slots carry column -1 and are skipped, so a
//     NaN in x behind a padding slot never leaks into a row sum.
//
// Arithmetic notes for GB300 (sm_103a): FP64 issues at 1/64 of the FP32 rate
// and an FP64 warp instruction costs the same whether 1 or 32 lanes are
// active, so FP64 kernels keep all lanes busy (one row per thread) and keep
// reductions short.  Reductions are deterministic: per-CTA partials summed in
// a fixed order by the last CTA to finish.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include "../../include/gbpc.h"

namespace gbpc {

constexpr int kSlice = 32;     // rows per SELL slice (one warp)
constexpr int kThreads = 1024;  // threads per CTA for streaming kernels
// Resident 1024-thread CTAs per SM for kernels within 32 registers per thread;
// streaming grids are capped at this many CTAs per SM so reductions combine
// few partial sums.
constexpr int kCtasPerSm = 2;
constexpr int kSms = 152;

// ---------------------------------------------------------------------------
// Value conversion helpers.

template <typename T> __device__ __forceinline__ double to_double(T v) { return (double)v; }
template <> __device__ __forceinline__ double to_double<__nv_bfloat16>(__nv_bfloat16 v) {
  return (double)__bfloat162float(v);
}
template <typename T> __device__ __forceinline__ float to_float(T v) { return (float)v; }
template <> __device__ __forceinline__ float to_float<__nv_bfloat16>(__nv_bfloat16 v) {
  return __bfloat162float(v);
}
template <typename A, typename S> __device__ __forceinline__ A widen(S v);
template <> __device__ __forceinline__ double widen<double, double>(double v) { return v; }
template <> __device__ __forceinline__ double widen<double, float>(float v) { return (double)v; }
template <> __device__ __forceinline__ double widen<double, __nv_bfloat16>(__nv_bfloat16 v) {
  return (double)__bfloat162float(v);
}
template <> __device__ __forceinline__ float widen<float, float>(float v) { return v; }
template <> __device__ __forceinline__ float widen<float, __nv_bfloat16>(__nv_bfloat16 v) {
  return __bfloat162float(v);
}
template <> __device__ __forceinline__ float widen<float, double>(double v) { return (float)v; }

// ---------------------------------------------------------------------------
// SELL-32 view (device pointers).  Slice s covers block rows [32 s, 32 s + 32)
// and entries [slice_ptr[s], slice_ptr[s+1]); entry (k, lane) of slice s is at
// E = slice_ptr[s] + 32 k + lane.  Its column is cols[E]; component q of its
// B x B block is vals[slice_ptr[s] * B * B + (k * B * B + q) * 32 + lane].
template <typename V>
struct SellView {
  int nrow;        // block rows
  int nslices;
  const int64_t* slice_ptr;
  const int32_t* cols;
  const V* vals;
  const int32_t* perm;  // stored row k is matrix row perm[k] (nullptr: identity)
  const int4* sched;    // SliceTask[nslices], slices by width descending
  int reverse;          // walk each warp's passes last to first (see warp_slice)
  int* err;             // set to 1 by a kernel whose bounded wait gave up (nullable)
};

// One entry of a sliced-ELL product schedule: slice s, its width (entries
// per lane) and the offset of its first entry.  Stored as an int4
// {s, width, base low word, base high word} so a warp reads it in one load.
struct SliceTask {
  int s;
  int width;
  int64_t base;
};

__device__ __forceinline__ SliceTask load_task(const int4* sched, int64_t idx) {
  const int4 t = __ldg(sched + idx);
  return SliceTask{t.x, t.y, (int64_t)(((uint64_t)(uint32_t)t.w << 32) | (uint32_t)t.z)};
}

// Schedule position of a warp's pass i: passes alternate direction over the
// width-sorted slices (t forward, then W - 1 - t, ...), so a warp that took
// one of the widest slices of a pass takes one of the narrowest of the next.
__device__ __forceinline__ int64_t sched_index(int i, int t, int warps_total) {
  return (int64_t)i * warps_total + ((i & 1) ? warps_total - 1 - t : t);
}

// Schedule position of warp t's k-th slice (k = 0, 1, ...), or -1 when it
// has no k-th slice.  Forward: passes 0, 1, ...  Reverse: the same passes
// last to first (a partial last pass that misses warp t is skipped), so a
// product that follows another over the same matrix starts with the slices
// that product touched last, which are the ones most likely still in L2.
// Each warp takes the same set of slices either way; only a fused dot
// product's summation order would change, so reverse walks are used for
// products without one.
__device__ __forceinline__ int64_t warp_slice(int k, int t, int warps_total, int64_t nslices,
                                              bool reverse) {
  if (!reverse) {
    const int64_t idx = sched_index(k, t, warps_total);
    return idx < nslices ? idx : -1;
  }
  const int passes = (int)((nslices + warps_total - 1) / warps_total);
  const bool has_last = passes > 0 && sched_index(passes - 1, t, warps_total) < nslices;
  const int pass = passes - 1 - k - (has_last ? 0 : 1);
  return pass >= 0 ? sched_index(pass, t, warps_total) : -1;
}

// ---------------------------------------------------------------------------
// Krylov scalars, resident on the device for the whole solve.
struct KrylovScalars {
  double bb;       // b.b
  double atol_sq;  // max(atol, tol |b|)^2
  double rr;       // recursive r.r
  double rz;       // CG: r.z   | CR: z.Az
  double rz_new;
  double denom;    // CG: p.Ap  | CR: y.Ap
  double alpha;
  double beta;
  int it;
  int maxiter;
  int active;
  int pad;
  unsigned long long cond_handle;  // cudaGraphConditionalHandle (0 = none)
  double tol;
  double atol;
  double* hist;    // residual history: hist[k] = |r_k| for k < hist_len (nullptr: none)
  int hist_len;
  int pad2;
};

// What the last CTA does with a finished reduction.
enum FinMode : int {
  FIN_NONE = 0,
  FIN_STORE = 1,       // *out = total
  FIN_INIT_BB = 2,     // bb = total
  FIN_INIT_RR = 3,     // rr = total; atol_sq; active; graph condition
  FIN_CG_ALPHA = 4,    // denom = total; alpha = rz / denom
  FIN_RR = 5,          // rr = total
  FIN_CG_BETA = 6,     // beta = total / rz; rz = total; it++; active
  FIN_INIT_RZ = 7,     // rz = total
  FIN_CR_ALPHA = 8,    // denom = total; alpha = rz / denom  (rz holds z.Az)
};

struct Reduction {
  const double* w;         // dot(w, out) with the kernel's output (nullptr: no dot)
  double* partials;        // per-CTA partial sums (>= gridDim.x entries)
  unsigned int* counter;   // arrival counter, zero between uses
  int mode;                // FinMode
  KrylovScalars* ks;
  double* out;             // FIN_STORE destination
};

// Programmatic dependent launch.  Kernels of the Krylov loop body are
// launched with cudaLaunchAttributeProgrammaticStreamSerialization, so the
// next kernel is scheduled while this one drains instead of after it; every
// such kernel first waits (in hardware, no polling) until its predecessor
// has completed and its writes are visible.  Launched without the attribute,
// both instructions do nothing.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_launch_dependents() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

__device__ __forceinline__ bool guard_off(const int* guard) {
  return guard != nullptr && *(volatile const int*)guard == 0;
}

// Sum of one double per thread over a CTA of kThreads threads with few FP64
// instructions: transpose through shared memory so warp 0 adds kThreads/32
// values per lane with full lanes, then a 5-step shuffle tree.  Result valid
// in thread 0.
__device__ __forceinline__ double block_sum(double v, double* smem /*kThreads*/) {
  static_assert(kThreads % 128 == 0, "block_sum expects a multiple of 128 threads");
  smem[threadIdx.x] = v;
  __syncthreads();
  // 128 threads add kThreads/128 values each (each reads only its own
  // column of smem before writing its own slot), then warp 0 adds 4 values
  // per lane and finishes with a shuffle tree.
  if (threadIdx.x < 128) {
    double s = smem[threadIdx.x];
#pragma unroll
    for (int k = 1; k < kThreads / 128; ++k) s += smem[threadIdx.x + 128 * k];
    smem[threadIdx.x] = s;
  }
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x < 32) {
    s = smem[threadIdx.x] + smem[threadIdx.x + 32];
    s += smem[threadIdx.x + 64] + smem[threadIdx.x + 96];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  }
  __syncthreads();
  return s;
}

// Krylov bookkeeping done by one thread once a reduction is complete.  The
// stopping rule mirrors warp.optim.linear: continue while r.r > atol^2 and
// fewer than maxiter iterations have run.
__device__ __forceinline__ void set_active(KrylovScalars* ks) {
  const int active = (ks->rr > ks->atol_sq) && (ks->it < ks->maxiter);
  ks->active = active;
  if (ks->cond_handle != 0ull)
    cudaGraphSetConditional((cudaGraphConditionalHandle)ks->cond_handle, active ? 1u : 0u);
}

__device__ __forceinline__ void finalize(const Reduction& red, double total) {
  KrylovScalars* ks = red.ks;
  switch (red.mode) {
    case FIN_STORE:
      *red.out = total;
      break;
    case FIN_INIT_BB:
      ks->bb = total;
      break;
    case FIN_INIT_RR: {
      ks->rr = total;
      const double a = fmax(ks->atol, ks->tol * sqrt(ks->bb));
      ks->atol_sq = a * a;
      ks->it = 0;
      if (ks->hist && ks->hist_len > 0) ks->hist[0] = sqrt(total);
      set_active(ks);
      break;
    }
    case FIN_INIT_RZ:
      ks->rz = total;
      break;
    case FIN_CG_ALPHA:
    case FIN_CR_ALPHA:
      ks->denom = total;
      ks->alpha = ks->rz / total;
      break;
    case FIN_RR:
      ks->rr = total;
      // The iteration count is advanced later in the same iteration.
      if (ks->hist && ks->it + 1 < ks->hist_len) ks->hist[ks->it + 1] = sqrt(total);
      break;
    case FIN_CG_BETA:
      ks->rz_new = total;
      ks->beta = total / ks->rz;
      ks->rz = total;
      ks->it += 1;
      set_active(ks);
      break;
    default:
      break;
  }
}

// Every thread of the CTA calls this with its partial; the last CTA to arrive
// sums all CTA partials and applies the finalize action.  That final sum is
// one warp's: lane l adds partials l, l + 32, ... (loads issued kFinLoads at
// a time), then a fixed butterfly — fewer barriers and dependent FP64 adds
// on the critical path than a whole-CTA sum, and the same order every run.
constexpr int kFinLoads = 10;  // 320 partials per pass: every grid of kSms * kCtasPerSm CTAs

__device__ __forceinline__ void reduce_and_finalize(const Reduction& red, double v) {
  __shared__ double smem[kThreads];
  __shared__ bool am_last;
  const double s = block_sum(v, smem);
  if (threadIdx.x == 0) {
    red.partials[blockIdx.x] = s;
    __threadfence();
    const unsigned int t = atomicAdd(red.counter, 1u);
    am_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (am_last && threadIdx.x < 32) {
    __threadfence();
    const unsigned lane = threadIdx.x, count = gridDim.x;
    double acc = 0.0;
    for (unsigned b = 0; b < count; b += 32 * kFinLoads) {
      double p[kFinLoads];
#pragma unroll
      for (int q = 0; q < kFinLoads; ++q) {
        const unsigned k = b + lane + 32 * q;
        p[q] = k < count ? __ldcg(red.partials + k) : 0.0;
      }
#pragma unroll
      for (int q = 0; q < kFinLoads; ++q) acc += p[q];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) {
      *red.counter = 0u;
      finalize(red, acc);
    }
  }
}

// True while a PdlScope is open on this thread (and GBPC_PDL is not "0").
bool pdl_active();

// Kernel launch that adds the programmatic-serialisation attribute while
// pdl_active(); the kernel must call pdl_wait() before reading anything its
// predecessor wrote.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_k(void (*kernel)(KArgs...), int grid, int block, size_t smem,
                            cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl_active() ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

inline int grid_for(int64_t items, int per_cta) {
  int64_t g = (items + per_cta - 1) / per_cta;
  if (g < 1) g = 1;
  if (g > 0x7fffffff) g = 0x7fffffff;
  return (int)g;
}

}  // namespace gbpc

#define GBPC_CUDA_TRY(expr)                         \
  do {                                              \
    cudaError_t _e = (expr);                        \
    if (_e != cudaSuccess) {                        \
      gbpc_set_error_cuda(_e, #expr, __FILE__, __LINE__); \
      return GBPC_ERR_CUDA;                         \
    }                                               \
  } while (0)

void gbpc_set_error(const char* fmt, ...);
void gbpc_set_error_cuda(cudaError_t e, const char* expr, const char* file, int line);
