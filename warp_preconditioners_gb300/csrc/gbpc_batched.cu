// Multi-right-hand-side operators, batched PCG and mixed-precision iterative
// refinement.
//
// Vectors hold k <= 32 right-hand sides per row, row-major (row i of X is
// X[i*k .. i*k+k)).  A warp works on 32/KP consecutive rows at once, each on
// a group of KP lanes (KP = k rounded up to a power of two) with lane j of the
// group on right-hand side j.  A group reads each stored entry of its row once
// (a coalesced load of up to KP entries, then shuffles inside the group) and
// gathers the k values of x's row in one access, so matrix bytes are shared by
// all right-hand sides, and the FP64 instructions issued per right-hand side
// are those of k/KP single-vector products (the warp-wide FP64 issue rate does
// not depend on how many lanes are active).
//
// Dots are accumulated in float64 per right-hand side, folded across the row
// groups of a warp, reduced per CTA through shared memory and combined in
// index order by the last CTA to finish (deterministic for a given k).  Every
// right-hand side has its own CG scalars and stopping test; finished ones are
// masked out while the rest continue.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <type_traits>
#include <vector>

#include "gbpc_common.cuh"
#include "gbpc_internal.h"

namespace gbpc {
namespace {

constexpr int kB = 32;            // lanes = right-hand sides per warp
constexpr int kBThreads = 512;    // 16 warps per CTA
constexpr int kBWarps = kBThreads / 32;
constexpr int kBMaxCtas = 152 * 4;

struct BatchScalars {
  double bb[kB], atol_sq[kB], rr[kB], rz[kB], denom[kB], alpha[kB], beta[kB];
  int it[kB], active[kB];
  int any_active, maxiter, k, pad;
  double tol, atol;
  unsigned long long cond_handle;
};

enum BFin : int {
  BF_NONE = 0,
  BF_BB = 1,      // bb_j = total_j
  BF_INIT_RR = 2, // rr_j, atol_sq_j, active_j
  BF_INIT_RZ = 3, // rz_j
  BF_ALPHA = 4,   // denom_j, alpha_j = active ? rz_j / denom_j : 0
  BF_RR = 5,      // rr_j
  BF_BETA = 6,    // beta_j, rz_j, it_j, active_j, any_active
  BF_STORE = 7,   // out[j] = total_j
};

struct BRed {
  const void* w;     // dot(w, out) per right-hand side (nullptr: none); same type as out
  double* partials;  // [gridDim.x][kB]
  unsigned int* counter;
  int mode;
  BatchScalars* bs;
  double* out;
  int w_f64;         // w is float64 although out is float32 (float32 preconditioner)
};

template <typename T> __device__ __forceinline__ T fma_bt(T a, T b, T c);
template <> __device__ __forceinline__ float fma_bt<float>(float a, float b, float c) { return fmaf(a, b, c); }
template <> __device__ __forceinline__ double fma_bt<double>(double a, double b, double c) { return fma(a, b, c); }

template <typename T, typename V> __device__ __forceinline__ T cvt(V v);
template <> __device__ __forceinline__ float cvt<float, float>(float v) { return v; }
template <> __device__ __forceinline__ float cvt<float, __nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }
template <> __device__ __forceinline__ float cvt<float, double>(double v) { return (float)v; }
template <> __device__ __forceinline__ double cvt<double, double>(double v) { return v; }
template <> __device__ __forceinline__ double cvt<double, float>(float v) { return (double)v; }
template <> __device__ __forceinline__ double cvt<double, __nv_bfloat16>(__nv_bfloat16 v) {
  return (double)__bfloat162float(v);
}

// Lanes per row group for k right-hand sides (k rounded up to a power of 2).
static inline int kp_for(int k) {
  int kp = 1;
  while (kp < k) kp <<= 1;
  return kp;
}

// Per right-hand-side total over the row groups of a warp: lanes with the
// same index inside their group are summed (a fixed butterfly); lane j < KP
// returns the total for right-hand side j, the other lanes 0.
template <int KP>
__device__ __forceinline__ double b_fold(double v) {
#pragma unroll
  for (int o = KP; o < 32; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return (threadIdx.x & 31) < KP ? v : 0.0;
}

__device__ __forceinline__ void b_set_active(BatchScalars* bs, int j, bool valid) {
  const int a = valid && (bs->rr[j] > bs->atol_sq[j]) && (bs->it[j] < bs->maxiter);
  bs->active[j] = a;
}

// Per-RHS finalize, executed by lane j of warp 0 of the last CTA.
__device__ __forceinline__ void b_finalize(const BRed& red, int j, double total) {
  BatchScalars* bs = red.bs;
  const bool valid = j < bs->k;
  switch (red.mode) {
    case BF_BB: bs->bb[j] = total; break;
    case BF_INIT_RR: {
      bs->rr[j] = total;
      const double a = fmax(bs->atol, bs->tol * sqrt(bs->bb[j]));
      bs->atol_sq[j] = a * a;
      bs->it[j] = 0;
      b_set_active(bs, j, valid);
      break;
    }
    case BF_INIT_RZ: bs->rz[j] = total; break;
    case BF_ALPHA:
      bs->denom[j] = total;
      bs->alpha[j] = bs->active[j] ? bs->rz[j] / total : 0.0;
      break;
    case BF_RR: bs->rr[j] = total; break;
    case BF_BETA:
      if (bs->active[j]) {
        bs->beta[j] = total / bs->rz[j];
        bs->rz[j] = total;
        bs->it[j] += 1;
      } else {
        bs->beta[j] = 0.0;
      }
      b_set_active(bs, j, valid);
      break;
    case BF_STORE:
      if (red.out) red.out[j] = total;
      break;
  }
  if (red.mode == BF_INIT_RR || red.mode == BF_BETA) {
    const unsigned any = __ballot_sync(0xffffffffu, bs->active[j] != 0);
    if (j == 0) {
      bs->any_active = any != 0u;
      if (bs->cond_handle != 0ull)
        cudaGraphSetConditional((cudaGraphConditionalHandle)bs->cond_handle, any ? 1u : 0u);
    }
  }
}

// Every thread calls this with its lane's partial (lane = RHS).  Warps are
// reduced through shared memory, CTAs through `partials` in index order.
__device__ __forceinline__ void b_reduce(const BRed& red, double v) {
  __shared__ double sm[kBWarps][kB];
  __shared__ bool am_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  sm[warp][lane] = v;
  __syncthreads();
  if (warp == 0) {
    double s = sm[0][lane];
#pragma unroll
    for (int w = 1; w < kBWarps; ++w) s += sm[w][lane];
    red.partials[(size_t)blockIdx.x * kB + lane] = s;
    __threadfence();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned int t = atomicAdd(red.counter, 1u);
    am_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (am_last) {
    // All warps of the last CTA sum a fixed subset of the CTA partials, then
    // warp 0 adds the warp sums in order: deterministic and short.
    __threadfence();
    double s = 0.0;
    unsigned int c = warp;
    // Eight CTA partials loaded together (zero past the last CTA), added in
    // the same order as one at a time: the loads no longer wait on each
    // other, including the last, partial group.
    for (; c < gridDim.x; c += 8 * kBWarps) {
      double v[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const unsigned int k = c + q * kBWarps;
        v[q] = k < gridDim.x ? __ldcg(red.partials + (size_t)k * kB + lane) : 0.0;
      }
#pragma unroll
      for (int q = 0; q < 8; ++q) s += v[q];
    }
    sm[warp][lane] = s;
    __syncthreads();
    if (warp == 0) {
      double t = sm[0][lane];
#pragma unroll
      for (int w = 1; w < kBWarps; ++w) t += sm[w][lane];
      b_finalize(red, lane, t);
      if (lane == 0) *red.counter = 0u;
    }
  }
}

enum BEpi : int { BE_AXPBY = 0, BE_SQLAP_BWD = 1 };

// Z = alpha * A X + beta * Y (or the factored backward epilogue).  A warp
// handles 32/KP consecutive rows, one per group of KP lanes; lane j of a
// group works on right-hand side j.  Row-scaled forward products pass the
// scaled matrix.  Each row sums its entries in storage order, whatever KP.
// UNIT: alpha == 1 and beta == 0 known at compile time (the Krylov loops'
// products), so no scaling or Y term is issued.
template <typename V, typename T, int EPI, bool DOT, int KP, bool UNIT = false>
__global__ void __launch_bounds__(kBThreads, 2)
bspmm_kernel(int nrow, int k, const int32_t* __restrict__ off, const int32_t* __restrict__ col,
             const V* __restrict__ val, const T* X, const T* Y, T* Z, double alpha, double beta,
             int alpha_zero, int alpha_one, int beta_zero, const T* wm, const T* X2,
             const int* guard, BRed red) {
  if constexpr (UNIT) {
    alpha_zero = 0;
    alpha_one = 1;
    beta_zero = 1;
  }
  pdl_wait();
  pdl_launch_dependents();
  if (guard_off(guard)) return;
  constexpr int GR = 32 / KP;
  const int lane = threadIdx.x & 31;
  const int grp = lane / KP, j = lane % KP;
  const int64_t warps_total = (int64_t)gridDim.x * kBWarps;
  const bool on = j < k;
  double dot = 0.0;
  for (int64_t wb = (int64_t)(threadIdx.x >> 5) * gridDim.x + blockIdx.x; wb * GR < nrow;
       wb += warps_total) {
    const int row = (int)(wb * GR) + grp;
    const bool live = row < nrow;
    T acc = T(0);
    if (!alpha_zero) {
      int e0 = 0, len = 0;
      if (live) {
        e0 = __ldg(off + row);
        len = __ldg(off + row + 1) - e0;
      }
      int maxlen = len;
#pragma unroll
      for (int o = KP; o < 32; o <<= 1) maxlen = max(maxlen, __shfl_xor_sync(0xffffffffu, maxlen, o));
      // Gathers of a chunk are issued together, then the FMAs run in
      // storage order (the same sum as one entry at a time).  The FMA loops
      // stop at the chunk's last entry in any row of the warp (a uniform
      // exit): an FP64 instruction costs its full issue slot even with every
      // lane predicated off.
      if constexpr (KP == 1) {
        constexpr int U = 4;
        for (int base = 0; base < maxlen; base += U) {
          T xv[U], vv[U];
#pragma unroll
          for (int e = 0; e < U; ++e) {
            const bool in = base + e < len;
            vv[e] = in ? cvt<T, V>(__ldg(val + e0 + base + e)) : T(0);
            xv[e] = in ? X[(int64_t)__ldg(col + e0 + base + e) * k] : T(0);
          }
#pragma unroll
          for (int e = 0; e < U; ++e) {
            if (base + e >= maxlen) break;
            if (base + e < len) acc = fma_bt<T>(vv[e], xv[e], acc);
          }
        }
      } else if constexpr (KP >= 16) {
        // Wide groups: enough independent work per warp already; one
        // entry at a time (the batched form measured slower and spills).
        for (int base = 0; base < maxlen; base += KP) {
          int c_l = 0;
          T v_l = T(0);
          if (base + j < len) {
            c_l = __ldg(col + e0 + base + j);
            v_l = cvt<T, V>(__ldg(val + e0 + base + j));
          }
          const int cnt = min(KP, maxlen - base);
          for (int e = 0; e < cnt; ++e) {
            const int c = __shfl_sync(0xffffffffu, c_l, e, KP);
            const T v = __shfl_sync(0xffffffffu, v_l, e, KP);
            if (on && base + e < len) acc = fma_bt<T>(v, X[(int64_t)c * k + j], acc);
          }
        }
      } else {
        constexpr int SUB = KP;  // all the chunk's gathers in flight per lane
        for (int base = 0; base < maxlen; base += KP) {
          int c_l = 0;
          T v_l = T(0);
          if (base + j < len) {
            c_l = __ldg(col + e0 + base + j);
            v_l = cvt<T, V>(__ldg(val + e0 + base + j));
          }
          const int cnt = min(KP, maxlen - base);
#pragma unroll
          for (int s0 = 0; s0 < KP; s0 += SUB) {
            if (s0 >= cnt) break;
            T xv[SUB], vv[SUB];
#pragma unroll
            for (int e = 0; e < SUB; ++e) {
              const int c = __shfl_sync(0xffffffffu, c_l, s0 + e, KP);
              vv[e] = __shfl_sync(0xffffffffu, v_l, s0 + e, KP);
              xv[e] = (on && base + s0 + e < len) ? X[(int64_t)c * k + j] : T(0);
            }
#pragma unroll
            for (int e = 0; e < SUB; ++e) {
              if (s0 + e >= cnt) break;
              if (on && base + s0 + e < len) acc = fma_bt<T>(vv[e], xv[e], acc);
            }
          }
        }
      }
    }
    if (on && live) {
      const int64_t idx = (int64_t)row * k + j;
      T out;
      if (EPI == BE_SQLAP_BWD) {
        out = T(0);
        if (!alpha_zero) {
          out = fma_bt<T>(wm[row], X2[idx], acc);
          if (!alpha_one) out = (T)alpha * out;
        }
      } else {
        out = alpha_one ? acc : (T)alpha * acc;
      }
      if (!beta_zero) out = fma_bt<T>((T)beta, Y[idx], out);
      Z[idx] = out;
      if (DOT) {
        const double wv = (!std::is_same<T, double>::value && red.w_f64)
                              ? ((const double*)red.w)[idx]
                              : (double)((const T*)red.w)[idx];
        dot = fma((double)out, wv, dot);
      }
    }
  }
  if (DOT) b_reduce(red, b_fold<KP>(dot));
}

// ---------------------------------------------------------------------------
// Batched CG kernels (vectors T, scalars float64).

// Rows of the elementwise kernels follow the same groups as the product.
#define B_ROWS(KP)                                                                     \
  constexpr int GR = 32 / (KP);                                                       \
  const int lane = threadIdx.x & 31;                                                  \
  const int grp = lane / (KP), j = lane % (KP);                                       \
  const int64_t warps_total = (int64_t)gridDim.x * kBWarps;                           \
  (void)grp;

template <typename T, int KP>
__global__ void __launch_bounds__(kBThreads)
bdot_kernel(int64_t n, int k, const T* a, const T* b, BRed red) {
  B_ROWS(KP);
  double s = 0.0;
  if (j < k)
    for (int64_t wb = (int64_t)(threadIdx.x >> 5) * gridDim.x + blockIdx.x; wb * GR < n;
         wb += warps_total) {
      const int64_t row = wb * GR + grp;
      if (row < n) s = fma((double)a[row * k + j], (double)b[row * k + j], s);
    }
  b_reduce(red, b_fold<KP>(s));
}

// X += alpha_j P; R -= alpha_j AP; reduce r.r  (inactive RHS untouched).
// R32 != nullptr: also R32 = (float) R, the input of a float32
// preconditioner inside the float64 loop.
template <typename T, int KP>
__global__ void __launch_bounds__(kBThreads)
bcg_update_kernel(int64_t n, int k, BatchScalars* bs, T* X, T* R, const T* P, const T* AP,
                  float* R32, BRed red) {
  pdl_wait();
  pdl_launch_dependents();
  if (*(volatile int*)&bs->any_active == 0) return;
  B_ROWS(KP);
  const bool on = j < k && bs->active[j];
  const T a = on ? (T)bs->alpha[j] : T(0);
  double s = 0.0;
  if (j < k)
    for (int64_t wb = (int64_t)(threadIdx.x >> 5) * gridDim.x + blockIdx.x; wb * GR < n;
         wb += warps_total) {
      const int64_t row = wb * GR + grp;
      if (row >= n) continue;
      const int64_t idx = row * k + j;
      T r = R[idx];
      if (on) {
        X[idx] = fma_bt<T>(a, P[idx], X[idx]);
        r = fma_bt<T>(-a, AP[idx], r);
        R[idx] = r;
        if (R32) R32[idx] = (float)r;
      }
      s = fma((double)r, (double)r, s);
    }
  b_reduce(red, b_fold<KP>(s));
}

// P = Z + beta_j P  (active RHS only); Z may be float32 (widened).
template <typename T, int KP, typename ZT = T>
__global__ void __launch_bounds__(kBThreads)
bxpay_kernel(int64_t n, int k, const BatchScalars* bs, const ZT* Zv, T* P) {
  pdl_wait();
  pdl_launch_dependents();
  if (*(volatile const int*)&bs->any_active == 0) return;
  B_ROWS(KP);
  if (j >= k || !bs->active[j]) return;
  const T b = (T)bs->beta[j];
  for (int64_t wb = (int64_t)(threadIdx.x >> 5) * gridDim.x + blockIdx.x; wb * GR < n;
       wb += warps_total) {
    const int64_t row = wb * GR + grp;
    if (row >= n) continue;
    const int64_t idx = row * k + j;
    P[idx] = fma_bt<T>(b, P[idx], (T)Zv[idx]);
  }
}

// Calls f(std::integral_constant<int, KP>{}) for the group width of k.
template <typename F>
static void with_kp(int k, F&& f) {
  switch (kp_for(k)) {
    case 1: f(std::integral_constant<int, 1>{}); break;
    case 2: f(std::integral_constant<int, 2>{}); break;
    case 4: f(std::integral_constant<int, 4>{}); break;
    case 8: f(std::integral_constant<int, 8>{}); break;
    case 16: f(std::integral_constant<int, 16>{}); break;
    default: f(std::integral_constant<int, 32>{}); break;
  }
}

__global__ void bset_kernel(BatchScalars* bs, int k, double tol, double atol, int maxiter,
                            unsigned long long handle) {
  const int j = threadIdx.x;
  if (j < kB) {
    bs->it[j] = 0;
    bs->active[j] = 0;
    bs->alpha[j] = 0.0;
    bs->beta[j] = 0.0;
  }
  if (j == 0) {
    bs->k = k;
    bs->tol = tol;
    bs->atol = atol;
    bs->maxiter = maxiter;
    bs->any_active = 1;
    bs->cond_handle = handle;
  }
}

__global__ void bcopy_outputs_kernel(const BatchScalars* bs, int k, int32_t* nit, double* rr) {
  const int j = threadIdx.x;
  if (j < k) {
    if (nit) nit[j] = bs->it[j];
    if (rr) rr[j] = bs->rr[j];
  }
}

// Y = (T) X   (precision change of a block of vectors)
template <typename TO, typename TI>
__global__ void convert_kernel(int64_t count, const TI* x, TO* y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = (TO)x[i];
}

// X64 += (double) D; per RHS max |D| and max |X| into dmax[k], xmax[k]
// (non-negative doubles order like their bit patterns: integer atomicMax).
template <typename T>
__global__ void accumulate_kernel(int64_t n, int k, const T* D, double* X, unsigned long long* dmax,
                                  unsigned long long* xmax) {
  const int64_t count = n * k;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(i % k);
    const double d = (double)D[i];
    const double x = X[i] + d;
    X[i] = x;
    atomicMax(dmax + j, (unsigned long long)__double_as_longlong(fabs(d)));
    atomicMax(xmax + j, (unsigned long long)__double_as_longlong(fabs(x)));
  }
}

// Zero the RHS columns that have converged (mask[j] != 0).
template <typename T>
__global__ void mask_columns_kernel(int64_t n, int k, const int* mask, T* X) {
  const int64_t count = n * k;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x)
    if (mask[i % k]) X[i] = T(0);
}

// CTAs for nrow rows at 32/KP rows per warp (a function of k only through KP).
int b_grid(int64_t nrow, int kp) {
  const int64_t rows_per_cta = (int64_t)kBWarps * (32 / kp);
  const int64_t g = (nrow + rows_per_cta - 1) / rows_per_cta;
  return (int)std::max<int64_t>(1, std::min<int64_t>(g, kBMaxCtas));
}

int e_grid(int64_t count) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((count + 255) / 256, 152 * 8));
}

}  // namespace

// ---------------------------------------------------------------------------
// Batched operators.

struct BCsr {
  int nrow = 0, ncol = 0;
  int vdtype = GBPC_F64;
  DevBuf off, col, val;
};

static int bcsr_copy(BCsr& m, int nrow, int ncol, const int32_t* off, const int32_t* col,
                     const void* val, int in_dtype, int out_dtype, const void* row_scale,
                     cudaStream_t st);

struct BOp {
  virtual ~BOp() = default;
  size_t device_bytes = 0;  // DevBuf bytes held (declared first: released last)
  int64_t rows = 0;
  int vdtype = GBPC_F64;  // vector dtype
  int max_rhs = kB;       // capacity of the scratch blocks
  virtual int apply(int k, const void* X, const void* Y, void* Z, double alpha, double beta,
                    const int* guard, const BRed* dot, cudaStream_t st) = 0;
};

template <typename V, typename T, int EPI>
static void launch_bspmm(const BCsr& m, int k, const void* X, const void* Y, void* Z, double alpha,
                         double beta, const void* wm, const void* X2, const int* guard,
                         const BRed* dot, cudaStream_t st) {
  BRed red{};
  if (dot) red = *dot;
  const int az = alpha == 0.0, a1 = alpha == 1.0, bz = beta == 0.0;
  with_kp(k, [&](auto kpc) {
    constexpr int KP = decltype(kpc)::value;
    const int g = b_grid(m.nrow, KP);
    auto go = [&](auto kern) {
      launch_k(kern, g, kBThreads, 0, st, m.nrow, k, (const int32_t*)m.off.as<int32_t>(),
               (const int32_t*)m.col.as<int32_t>(), (const V*)m.val.as<V>(), (const T*)X,
               (const T*)Y, (T*)Z, alpha, beta, az, a1, bz, (const T*)wm, (const T*)X2, guard,
               red);
    };
    const bool unit = !az && a1 && bz;
    if (dot && dot->w) {
      if (unit) go(bspmm_kernel<V, T, EPI, true, KP, true>);
      else go(bspmm_kernel<V, T, EPI, true, KP>);
    } else {
      if (unit) go(bspmm_kernel<V, T, EPI, false, KP, true>);
      else go(bspmm_kernel<V, T, EPI, false, KP>);
    }
  });
}

template <int EPI>
static int bspmm(const BCsr& m, int vdtype, int k, const void* X, const void* Y, void* Z,
                 double alpha, double beta, const void* wm, const void* X2, const int* guard,
                 const BRed* dot, cudaStream_t st) {
  if (vdtype == GBPC_F64) {
    if (m.vdtype == GBPC_F64) launch_bspmm<double, double, EPI>(m, k, X, Y, Z, alpha, beta, wm, X2, guard, dot, st);
    else if (m.vdtype == GBPC_F32) launch_bspmm<float, double, EPI>(m, k, X, Y, Z, alpha, beta, wm, X2, guard, dot, st);
    else launch_bspmm<__nv_bfloat16, double, EPI>(m, k, X, Y, Z, alpha, beta, wm, X2, guard, dot, st);
  } else {
    if (m.vdtype == GBPC_F64) {
      gbpc_set_error("float64 storage needs float64 vectors");
      return GBPC_ERR_ARG;
    }
    if (m.vdtype == GBPC_F32) launch_bspmm<float, float, EPI>(m, k, X, Y, Z, alpha, beta, wm, X2, guard, dot, st);
    else launch_bspmm<__nv_bfloat16, float, EPI>(m, k, X, Y, Z, alpha, beta, wm, X2, guard, dot, st);
  }
  GBPC_CUDA_TRY(cudaGetLastError());
  return GBPC_OK;
}

struct BSparseOp : BOp {
  BCsr a;
  int apply(int k, const void* X, const void* Y, void* Z, double alpha, double beta,
            const int* guard, const BRed* dot, cudaStream_t st) override {
    return bspmm<BE_AXPBY>(a, vdtype, k, X, Y, Z, alpha, beta, nullptr, nullptr, guard, dot, st);
  }
};

struct BFsaiOp : BOp {
  BCsr g, gt;
  DevBuf tmp;  // rows * max_rhs vectors
  int apply(int k, const void* X, const void* Y, void* Z, double alpha, double beta,
            const int* guard, const BRed* dot, cudaStream_t st) override {
    int rc;
    if (alpha != 0.0 &&
        (rc = bspmm<BE_AXPBY>(g, vdtype, k, X, nullptr, tmp.p, 1.0, 0.0, nullptr, nullptr, guard,
                              nullptr, st)))
      return rc;
    return bspmm<BE_AXPBY>(gt, vdtype, k, tmp.p, Y, Z, alpha, beta, nullptr, nullptr, guard, dot, st);
  }
};

struct BSqlapOp : BOp {
  BCsr fwd, bwd;  // M^-1 L and L (all vertices free)
  DevBuf wmass, tmp;
  int apply(int k, const void* X, const void* Y, void* Z, double alpha, double beta,
            const int* guard, const BRed* dot, cudaStream_t st) override {
    int rc;
    if (alpha != 0.0 &&
        (rc = bspmm<BE_AXPBY>(fwd, vdtype, k, X, nullptr, tmp.p, 1.0, 0.0, nullptr, nullptr, guard,
                              nullptr, st)))
      return rc;
    return bspmm<BE_SQLAP_BWD>(bwd, vdtype, k, tmp.p, Y, Z, alpha, beta, wmass.p, X, guard, dot, st);
  }
};

template <typename VI, typename VO>
__global__ void bcsr_fill_kernel(int nrow, const int32_t* __restrict__ off, const int32_t* __restrict__ col,
                                 const VI* __restrict__ val, const VI* row_scale, int32_t* ocol,
                                 VO* oval) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrow) return;
  for (int e = off[i]; e < off[i + 1]; ++e) {
    ocol[e] = col[e];
    VI v = val[e];
    if (row_scale) v = v * row_scale[i];
    oval[e] = (VO)v;
  }
}

template <typename VI>
__global__ void bcsr_fill_bf16_kernel(int nrow, const int32_t* __restrict__ off,
                                      const int32_t* __restrict__ col, const VI* __restrict__ val,
                                      const VI* row_scale, int32_t* ocol, __nv_bfloat16* oval) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrow) return;
  for (int e = off[i]; e < off[i + 1]; ++e) {
    ocol[e] = col[e];
    VI v = val[e];
    if (row_scale) v = v * row_scale[i];
    oval[e] = __float2bfloat16_rn((float)v);
  }
}

static int bcsr_copy(BCsr& m, int nrow, int ncol, const int32_t* off, const int32_t* col,
                     const void* val, int in_dtype, int out_dtype, const void* row_scale,
                     cudaStream_t st) {
  if (!(in_dtype == GBPC_F64 || in_dtype == GBPC_F32) || !valid_value_dtype(out_dtype) ||
      (in_dtype == GBPC_F32 && out_dtype == GBPC_F64)) {
    gbpc_set_error("batched operator: unsupported dtype %d -> %d", in_dtype, out_dtype);
    return GBPC_ERR_ARG;
  }
  m.nrow = nrow;
  m.ncol = ncol;
  m.vdtype = out_dtype;
  int32_t nnz = 0;
  GBPC_CUDA_TRY(cudaMemcpyAsync(&nnz, off + nrow, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  GBPC_CUDA_TRY(cudaStreamSynchronize(st));
  int rc;
  if ((rc = m.off.alloc(sizeof(int32_t) * (nrow + 1)))) return rc;
  if ((rc = m.col.alloc(sizeof(int32_t) * std::max(nnz, 1)))) return rc;
  if ((rc = m.val.alloc(dtype_size(out_dtype) * std::max(nnz, 1)))) return rc;
  GBPC_CUDA_TRY(cudaMemcpyAsync(m.off.p, off, sizeof(int32_t) * (nrow + 1), cudaMemcpyDeviceToDevice, st));
  const int g = grid_for(std::max(nrow, 1), 256);
  if (nrow > 0) {
    if (in_dtype == GBPC_F64) {
      if (out_dtype == GBPC_F64)
        bcsr_fill_kernel<double, double><<<g, 256, 0, st>>>(nrow, off, col, (const double*)val,
                                                          (const double*)row_scale, m.col.as<int32_t>(), m.val.as<double>());
      else if (out_dtype == GBPC_F32)
        bcsr_fill_kernel<double, float><<<g, 256, 0, st>>>(nrow, off, col, (const double*)val,
                                                         (const double*)row_scale, m.col.as<int32_t>(), m.val.as<float>());
      else
        bcsr_fill_bf16_kernel<double><<<g, 256, 0, st>>>(nrow, off, col, (const double*)val,
                                                        (const double*)row_scale, m.col.as<int32_t>(), m.val.as<__nv_bfloat16>());
    } else {
      if (out_dtype == GBPC_F32)
        bcsr_fill_kernel<float, float><<<g, 256, 0, st>>>(nrow, off, col, (const float*)val,
                                                        (const float*)row_scale, m.col.as<int32_t>(), m.val.as<float>());
      else
        bcsr_fill_bf16_kernel<float><<<g, 256, 0, st>>>(nrow, off, col, (const float*)val,
                                                       (const float*)row_scale, m.col.as<int32_t>(), m.val.as<__nv_bfloat16>());
    }
  }
  GBPC_CUDA_TRY(cudaGetLastError());
  return GBPC_OK;
}

// ---------------------------------------------------------------------------
// Batched PCG (device loop in one CUDA graph, per-RHS stopping).

struct BSolver {
  size_t device_bytes = 0;  // DevBuf bytes held (declared first: released last)
  BOp* A = nullptr;
  BOp* M = nullptr;
  int64_t n = 0;
  int vdtype = GBPC_F32;
  int max_rhs = kB;
  // Float64 loop with a float32 preconditioner (A float64, M float32): the
  // update kernel writes R32, M maps R32 to Z32 with the float64 dot r.z,
  // and the direction update widens Z32.
  bool mixed_m = false;
  DevBuf R, Zv, P, AP, bs, partials, counter, R32, Z32;
  // Graph being built (moved into `graphs` once instantiated).
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphConditionalHandle handle = 0;
  // Instantiated graphs by (B, X, k), least recently used dropped first.
  struct Cached {
    cudaGraph_t graph;
    cudaGraphExec_t exec;
    cudaGraphConditionalHandle handle;
    const void* b;
    void* x;
    int k;
    uint64_t used;
  };
  static constexpr size_t kMaxGraphs = 8;
  std::vector<Cached> graphs;
  uint64_t clock = 0;
  int unroll = 8;
  bool use_pdl = true;  // programmatic dependent launches inside the loop body

  ~BSolver() {
    drop();
    for (auto& c : graphs) {
      cudaGraphExecDestroy(c.exec);
      cudaGraphDestroy(c.graph);
    }
  }
  void drop() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
  }
  BatchScalars* S() { return bs.as<BatchScalars>(); }
  BRed red(const void* w, int mode) {
    BRed r{};
    r.w = w;
    r.partials = partials.as<double>();
    r.counter = counter.as<unsigned int>();
    r.mode = mode;
    r.bs = S();
    return r;
  }
  size_t vbytes(int k) const { return dtype_size(vdtype) * (size_t)n * k; }

  template <typename T>
  int record_init(int k, const void* B, void* X, cudaStream_t st) {
    int rc;
    GBPC_CUDA_TRY(cudaMemsetAsync(counter.p, 0, sizeof(unsigned int), st));
    BRed rbb = red(B, BF_BB);
    with_kp(k, [&](auto kpc) {
      constexpr int KP = decltype(kpc)::value;
      bdot_kernel<T, KP><<<b_grid(n, KP), kBThreads, 0, st>>>(n, k, (const T*)B, (const T*)B, rbb);
    });
    GBPC_CUDA_TRY(cudaGetLastError());
    BRed rrr = red(R.p, BF_INIT_RR);
    if ((rc = A->apply(k, X, B, R.p, -1.0, 1.0, nullptr, &rrr, st))) return rc;
    BRed rrz = red(R.p, BF_INIT_RZ);
    if (mixed_m) {
      const int64_t count = n * k;
      convert_kernel<float, double><<<e_grid(count), 256, 0, st>>>(count, R.as<double>(),
                                                                   R32.as<float>());
      GBPC_CUDA_TRY(cudaGetLastError());
      rrz.w_f64 = 1;
      if ((rc = M->apply(k, R32.p, nullptr, Z32.p, 1.0, 0.0, nullptr, &rrz, st))) return rc;
      convert_kernel<double, float><<<e_grid(count), 256, 0, st>>>(count, Z32.as<float>(),
                                                                   P.as<double>());
      GBPC_CUDA_TRY(cudaGetLastError());
      return GBPC_OK;
    }
    if ((rc = M->apply(k, R.p, nullptr, Zv.p, 1.0, 0.0, nullptr, &rrz, st))) return rc;
    GBPC_CUDA_TRY(cudaMemcpyAsync(P.p, Zv.p, vbytes(k), cudaMemcpyDeviceToDevice, st));
    return GBPC_OK;
  }

  template <typename T>
  int record_iteration(int k, void* X, cudaStream_t st) {
    int rc;
    const int* guard = &S()->any_active;
    BRed ra = red(P.p, BF_ALPHA);
    if ((rc = A->apply(k, P.p, nullptr, AP.p, 1.0, 0.0, guard, &ra, st))) return rc;
    BRed rr = red(R.p, BF_RR);
    float* r32 = mixed_m ? R32.as<float>() : nullptr;
    with_kp(k, [&](auto kpc) {
      constexpr int KP = decltype(kpc)::value;
      launch_k(bcg_update_kernel<T, KP>, b_grid(n, KP), kBThreads, 0, st, n, k, S(), (T*)X,
               (T*)R.p, (const T*)P.p, (const T*)AP.p, r32, rr);
    });
    GBPC_CUDA_TRY(cudaGetLastError());
    BRed rb = red(R.p, BF_BETA);
    if (mixed_m) {
      rb.w_f64 = 1;
      if ((rc = M->apply(k, R32.p, nullptr, Z32.p, 1.0, 0.0, guard, &rb, st))) return rc;
      with_kp(k, [&](auto kpc) {
        constexpr int KP = decltype(kpc)::value;
        launch_k(bxpay_kernel<T, KP, float>, b_grid(n, KP), kBThreads, 0, st, n, k,
                 (const BatchScalars*)S(), (const float*)Z32.p, (T*)P.p);
      });
      GBPC_CUDA_TRY(cudaGetLastError());
      return GBPC_OK;
    }
    if ((rc = M->apply(k, R.p, nullptr, Zv.p, 1.0, 0.0, guard, &rb, st))) return rc;
    with_kp(k, [&](auto kpc) {
      constexpr int KP = decltype(kpc)::value;
      launch_k(bxpay_kernel<T, KP>, b_grid(n, KP), kBThreads, 0, st, n, k,
               (const BatchScalars*)S(), (const T*)Zv.p, (T*)P.p);
    });
    GBPC_CUDA_TRY(cudaGetLastError());
    return GBPC_OK;
  }

  template <typename T>
  int build(int k, const void* B, void* X, cudaStream_t st) {
    drop();
    GBPC_CUDA_TRY(cudaGraphCreate(&graph, 0));
    GBPC_CUDA_TRY(cudaGraphConditionalHandleCreate(&handle, graph, 0, cudaGraphCondAssignDefault));
    cudaStream_t cs;
    GBPC_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    int rc = GBPC_OK;
    do {
      if (cudaStreamBeginCaptureToGraph(cs, graph, nullptr, nullptr, 0,
                                        cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        rc = GBPC_ERR_CUDA;
        break;
      }
      rc = record_init<T>(k, B, X, cs);
      cudaGraph_t g2 = nullptr;
      cudaError_t e = cudaStreamEndCapture(cs, &g2);
      if (rc) break;
      if (e != cudaSuccess) {
        gbpc_set_error_cuda(e, "capture batched init", __FILE__, __LINE__);
        rc = GBPC_ERR_CUDA;
        break;
      }
      size_t count = 0;
      cudaGraphGetNodes(graph, nullptr, &count);
      std::vector<cudaGraphNode_t> nodes(count);
      cudaGraphGetNodes(graph, nodes.data(), &count);
      cudaGraphNode_t tail = nullptr;
      for (auto nd : nodes) {
        size_t outs = 0;
        cudaGraphNodeGetDependentNodes(nd, nullptr, nullptr, &outs);
        if (outs == 0) tail = nd;
      }
      cudaGraphNodeParams cp = {};
      cp.type = cudaGraphNodeTypeConditional;
      cp.conditional.handle = handle;
      cp.conditional.type = cudaGraphCondTypeWhile;
      cp.conditional.size = 1;
      cudaGraphNode_t cnode;
      e = cudaGraphAddNode(&cnode, graph, tail ? &tail : nullptr, nullptr, tail ? 1 : 0, &cp);
      if (e != cudaSuccess) {
        gbpc_set_error_cuda(e, "add conditional node", __FILE__, __LINE__);
        rc = GBPC_ERR_CUDA;
        break;
      }
      cudaGraph_t body = cp.conditional.phGraph_out[0];
      if (cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0,
                                        cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        rc = GBPC_ERR_CUDA;
        break;
      }
      {
        PdlScope scope(use_pdl);
        for (int u = 0; u < unroll && !rc; ++u) rc = record_iteration<T>(k, X, cs);
      }
      e = cudaStreamEndCapture(cs, &g2);
      if (rc) break;
      if (e != cudaSuccess || cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) {
        gbpc_set_error("batched solver: graph capture/instantiate failed");
        rc = GBPC_ERR_CUDA;
        break;
      }
    } while (0);
    cudaStreamDestroy(cs);
    if (rc) {
      drop();
      cudaGetLastError();
      return rc;
    }
    if (graphs.size() >= kMaxGraphs) {
      auto lru = std::min_element(graphs.begin(), graphs.end(),
                                  [](const Cached& a, const Cached& b) { return a.used < b.used; });
      cudaGraphExecDestroy(lru->exec);
      cudaGraphDestroy(lru->graph);
      graphs.erase(lru);
    }
    graphs.push_back(Cached{graph, exec, handle, B, X, k, ++clock});
    graph = nullptr;
    exec = nullptr;
    return GBPC_OK;
  }

  int run(int k, const void* B, void* X, double tol, double atol, int maxiter, int32_t* nit,
          double* rr, cudaStream_t st) {
    if (maxiter <= 0) maxiter = (int)std::min<int64_t>(n, 0x7fffffff);
    if (k > max_rhs || k > A->max_rhs || k > M->max_rhs) {
      gbpc_set_error("batched solver: %d right-hand sides exceed the capacity (%d)", k,
                     std::min(max_rhs, std::min(A->max_rhs, M->max_rhs)));
      return GBPC_ERR_ARG;
    }
    int rc;
    Cached* hit = nullptr;
    for (auto& c : graphs)
      if (c.b == B && c.x == X && c.k == k) hit = &c;
    if (!hit) {
      rc = (vdtype == GBPC_F64) ? build<double>(k, B, X, st) : build<float>(k, B, X, st);
      if (rc && use_pdl) {  // capture without programmatic launches instead
        use_pdl = false;
        rc = (vdtype == GBPC_F64) ? build<double>(k, B, X, st) : build<float>(k, B, X, st);
      }
      if (rc) return rc;
      hit = &graphs.back();
    }
    hit->used = ++clock;
    bset_kernel<<<1, kB, 0, st>>>(S(), k, tol, atol, maxiter, (unsigned long long)hit->handle);
    GBPC_CUDA_TRY(cudaGetLastError());
    GBPC_CUDA_TRY(cudaGraphLaunch(hit->exec, st));
    if (nit || rr) bcopy_outputs_kernel<<<1, kB, 0, st>>>(S(), k, nit, rr);
    GBPC_CUDA_TRY(cudaGetLastError());
    return GBPC_OK;
  }
};

}  // namespace gbpc

using namespace gbpc;

struct gbpc_bop {
  std::unique_ptr<BOp> impl;
};
struct gbpc_bsolver {
  BSolver s;
};

#define GBPC_BOP_OUT(ptr)       \
  do {                          \
    gbpc_bop* h = new gbpc_bop; \
    h->impl.reset(ptr);         \
    *out = h;                   \
  } while (0)

static int bop_vdtype_ok(int value_dtype, int vector_dtype) {
  if (vector_dtype != GBPC_F64 && vector_dtype != GBPC_F32) {
    gbpc_set_error("batched operators use float64 or float32 vectors");
    return GBPC_ERR_ARG;
  }
  if (value_dtype == GBPC_F64 && vector_dtype != GBPC_F64) {
    gbpc_set_error("float64 storage needs float64 vectors");
    return GBPC_ERR_ARG;
  }
  return GBPC_OK;
}

extern "C" int gbpc_bop_sparse(int n, const int32_t* off, const int32_t* col, const void* val,
                               int in_dtype, int value_dtype, int vector_dtype, void* stream,
                               gbpc_bop** out) {
  int rc = bop_vdtype_ok(value_dtype, vector_dtype);
  if (rc) return rc;
  if (!out || n < 0 || !off) {
    gbpc_set_error("gbpc_bop_sparse: bad arguments");
    return GBPC_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  auto* op = new BSparseOp;
  ByteTally tally(&op->device_bytes);
  op->rows = n;
  op->vdtype = vector_dtype;
  rc = bcsr_copy(op->a, n, n, off, col, val, in_dtype, value_dtype, nullptr, st);
  if (!rc && cudaStreamSynchronize(st) != cudaSuccess) rc = GBPC_ERR_CUDA;
  if (rc) {
    delete op;
    return rc;
  }
  GBPC_BOP_OUT(op);
  return GBPC_OK;
}

extern "C" int gbpc_bop_fsai(int n, const int32_t* g_off, const int32_t* g_col, const void* g_val,
                             const int32_t* gt_off, const int32_t* gt_col, const void* gt_val,
                             int in_dtype, int value_dtype, int vector_dtype, int max_rhs,
                             void* stream, gbpc_bop** out) {
  int rc = bop_vdtype_ok(value_dtype, vector_dtype);
  if (rc) return rc;
  if (!out || n < 0 || !g_off || !gt_off || max_rhs < 1 || max_rhs > kB) {
    gbpc_set_error("gbpc_bop_fsai: bad arguments");
    return GBPC_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  auto* op = new BFsaiOp;
  ByteTally tally(&op->device_bytes);
  op->rows = n;
  op->vdtype = vector_dtype;
  op->max_rhs = max_rhs;
  rc = bcsr_copy(op->g, n, n, g_off, g_col, g_val, in_dtype, value_dtype, nullptr, st);
  if (!rc) rc = bcsr_copy(op->gt, n, n, gt_off, gt_col, gt_val, in_dtype, value_dtype, nullptr, st);
  if (!rc) rc = op->tmp.alloc(dtype_size(vector_dtype) * std::max(n, 1) * max_rhs);
  if (!rc && cudaStreamSynchronize(st) != cudaSuccess) rc = GBPC_ERR_CUDA;
  if (rc) {
    delete op;
    return rc;
  }
  GBPC_BOP_OUT(op);
  return GBPC_OK;
}

template <typename T>
__global__ void bsqlap_prep_kernel(int n, const double* mass, double w, T* inv, T* wm) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  inv[i] = (T)(1.0 / mass[i]);
  wm[i] = (T)(w * mass[i]);
}

extern "C" int gbpc_bop_sqlap(int n, const int32_t* off, const int32_t* col, const void* val,
                              int in_dtype, int value_dtype, int vector_dtype, const double* mass,
                              double mass_weight, int max_rhs, void* stream, gbpc_bop** out) {
  int rc = bop_vdtype_ok(value_dtype, vector_dtype);
  if (rc) return rc;
  if (!out || n < 0 || !off || !mass || !std::isfinite(mass_weight) || mass_weight < 0 ||
      max_rhs < 1 || max_rhs > kB) {
    gbpc_set_error("gbpc_bop_sqlap: bad arguments");
    return GBPC_ERR_ARG;
  }
  if (in_dtype != GBPC_F64) {
    gbpc_set_error("gbpc_bop_sqlap: pass float64 L values (converted on the device)");
    return GBPC_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  auto* op = new BSqlapOp;
  ByteTally tally(&op->device_bytes);
  op->rows = n;
  op->vdtype = vector_dtype;
  op->max_rhs = max_rhs;
  DevBuf inv64, wm64;
  rc = inv64.alloc(sizeof(double) * std::max(n, 1));
  if (!rc) rc = op->wmass.alloc(dtype_size(vector_dtype) * std::max(n, 1));
  if (!rc) rc = wm64.alloc(sizeof(double) * std::max(n, 1));
  if (!rc && n > 0) {
    bsqlap_prep_kernel<double><<<grid_for(n, 256), 256, 0, st>>>(n, mass, mass_weight,
                                                                 inv64.as<double>(), wm64.as<double>());
    if (vector_dtype == GBPC_F64)
      cudaMemcpyAsync(op->wmass.p, wm64.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, st);
    else
      convert_kernel<float, double><<<e_grid(n), 256, 0, st>>>(n, wm64.as<double>(), op->wmass.as<float>());
  }
  // Forward matrix M^-1 L (rows scaled in float64 before narrowing), backward L.
  if (!rc) rc = bcsr_copy(op->fwd, n, n, off, col, val, GBPC_F64, value_dtype, inv64.p, st);
  if (!rc) rc = bcsr_copy(op->bwd, n, n, off, col, val, GBPC_F64, value_dtype, nullptr, st);
  if (!rc) rc = op->tmp.alloc(dtype_size(vector_dtype) * std::max(n, 1) * max_rhs);
  if (!rc && cudaStreamSynchronize(st) != cudaSuccess) rc = GBPC_ERR_CUDA;
  if (rc) {
    delete op;
    return rc;
  }
  GBPC_BOP_OUT(op);
  return GBPC_OK;
}

extern "C" int gbpc_bop_apply(gbpc_bop* op, int k, const void* X, const void* Y, void* Z,
                              double alpha, double beta, void* stream) {
  if (!op || k < 1 || k > op->impl->max_rhs) {
    gbpc_set_error("gbpc_bop_apply: k must be 1..%d", op ? op->impl->max_rhs : kB);
    return GBPC_ERR_ARG;
  }
  if (X == Z && alpha != 0.0) {
    gbpc_set_error("gbpc_bop_apply: X must not alias Z");
    return GBPC_ERR_ARG;
  }
  return op->impl->apply(k, X, Y, Z, alpha, beta, nullptr, nullptr, (cudaStream_t)stream);
}

extern "C" int gbpc_bop_device_bytes(const gbpc_bop* op, size_t* bytes_host) {
  if (!op || !bytes_host) {
    gbpc_set_error("gbpc_bop_device_bytes: bad arguments");
    return GBPC_ERR_ARG;
  }
  *bytes_host = op->impl->device_bytes;
  return GBPC_OK;
}

extern "C" int gbpc_bop_destroy(gbpc_bop* op) {
  if (!op) return GBPC_OK;
  cudaDeviceSynchronize();
  delete op;
  return GBPC_OK;
}

extern "C" int gbpc_bsolver_create(gbpc_bop* A, gbpc_bop* M, int unroll, int max_rhs,
                                   void* stream, gbpc_bsolver** out) {
  // Vector dtypes: equal, or a float64 operator with a float32 preconditioner
  // (the loop stays float64; only M runs in float32).
  const bool mixed_m = A && M && A->impl->vdtype == GBPC_F64 && M->impl->vdtype == GBPC_F32;
  if (!out || !A || !M || A->impl->rows != M->impl->rows ||
      (A->impl->vdtype != M->impl->vdtype && !mixed_m)) {
    gbpc_set_error("gbpc_bsolver_create: operator and preconditioner must match in size and "
                   "vector dtype (or pair a float64 operator with a float32 preconditioner)");
    return GBPC_ERR_ARG;
  }
  if (max_rhs < 1 || max_rhs > kB) {
    gbpc_set_error("gbpc_bsolver_create: max_rhs must be 1..%d", kB);
    return GBPC_ERR_ARG;
  }
  auto* h = new gbpc_bsolver;
  BSolver& s = h->s;
  ByteTally tally(&s.device_bytes);
  s.max_rhs = max_rhs;
  s.A = A->impl.get();
  s.M = M->impl.get();
  s.n = A->impl->rows;
  s.vdtype = A->impl->vdtype;
  if (unroll > 0) s.unroll = std::min(unroll, 64);
  const size_t bytes = dtype_size(s.vdtype) * std::max<int64_t>(s.n, 1) * max_rhs;
  int rc = s.R.alloc(bytes);
  if (!rc) rc = s.Zv.alloc(bytes);
  if (!rc) rc = s.P.alloc(bytes);
  if (!rc) rc = s.AP.alloc(bytes);
  s.mixed_m = mixed_m;
  if (!rc && mixed_m) rc = s.R32.alloc(sizeof(float) * std::max<int64_t>(s.n, 1) * max_rhs);
  if (!rc && mixed_m) rc = s.Z32.alloc(sizeof(float) * std::max<int64_t>(s.n, 1) * max_rhs);
  if (!rc) rc = s.bs.alloc(sizeof(BatchScalars));
  if (!rc) rc = s.partials.alloc(sizeof(double) * kBMaxCtas * kB);
  if (!rc) rc = s.counter.alloc(sizeof(unsigned int));
  if (!rc && (cudaMemsetAsync(s.bs.p, 0, sizeof(BatchScalars), (cudaStream_t)stream) != cudaSuccess ||
              cudaMemsetAsync(s.counter.p, 0, sizeof(unsigned int), (cudaStream_t)stream) != cudaSuccess))
    rc = GBPC_ERR_CUDA;
  if (rc) {
    delete h;
    return rc;
  }
  *out = h;
  return GBPC_OK;
}

extern "C" int gbpc_bsolver_run(gbpc_bsolver* h, int k, const void* B, void* X, double tol,
                                double atol, int maxiter, int32_t* nit_dev, double* rr_dev,
                                void* stream) {
  NvtxRange nvtx_range("gbpc_bsolver_run");
  if (!h || k < 1 || k > h->s.max_rhs || !B || !X) {
    gbpc_set_error("gbpc_bsolver_run: bad arguments (k must be 1..%d)", h ? h->s.max_rhs : kB);
    return GBPC_ERR_ARG;
  }
  return h->s.run(k, B, X, tol, atol, maxiter, nit_dev, rr_dev, (cudaStream_t)stream);
}

extern "C" int gbpc_bsolver_device_bytes(const gbpc_bsolver* h, size_t* bytes_host) {
  if (!h || !bytes_host) {
    gbpc_set_error("gbpc_bsolver_device_bytes: bad arguments");
    return GBPC_ERR_ARG;
  }
  *bytes_host = h->s.device_bytes;
  return GBPC_OK;
}

extern "C" int gbpc_bsolver_destroy(gbpc_bsolver* h) {
  if (!h) return GBPC_OK;
  cudaDeviceSynchronize();
  delete h;
  return GBPC_OK;
}

// Mixed-precision iterative refinement for k right-hand sides of one system:
// the residual r = b - A64 x is formed in float64, the correction is solved
// with the batched PCG of `inner` (typically float32 operator and a float32 /
// bfloat16 FSAI factor) to relative tolerance tol_inner, and x += d in
// float64.  A right-hand side stops once max|d| <= tol_outer * max|x|.
extern "C" int gbpc_refine(gbpc_bop* A64, gbpc_bsolver* inner, int k, const double* B, double* X,
                           double tol_outer, double tol_inner, int max_outer, int max_inner,
                           int32_t* outer_host, int32_t* inner_host, void* stream) {
  if (!A64 || !inner || k < 1 || k > kB || k > A64->impl->max_rhs || !B || !X ||
      A64->impl->vdtype != GBPC_F64 || A64->impl->rows != inner->s.n) {
    gbpc_set_error("gbpc_refine: bad arguments");
    return GBPC_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  BSolver& s = inner->s;
  const int64_t n = s.n;
  const int64_t count = n * k;
  DevBuf R64, Rin, D, stats, mask, nit;
  int rc;
  if ((rc = R64.alloc(sizeof(double) * std::max<int64_t>(count, 1)))) return rc;
  if ((rc = Rin.alloc(dtype_size(s.vdtype) * std::max<int64_t>(count, 1)))) return rc;
  if ((rc = D.alloc(dtype_size(s.vdtype) * std::max<int64_t>(count, 1)))) return rc;
  if ((rc = stats.alloc(sizeof(unsigned long long) * 2 * kB))) return rc;
  if ((rc = mask.alloc(sizeof(int) * kB))) return rc;
  if ((rc = nit.alloc(sizeof(int32_t) * kB))) return rc;
  std::vector<int> done(kB, 0);
  std::vector<int32_t> outer_it(k, 0), inner_it(k, 0);
  GBPC_CUDA_TRY(cudaMemsetAsync(X, 0, sizeof(double) * count, st));
  GBPC_CUDA_TRY(cudaMemcpyAsync(R64.p, B, sizeof(double) * count, cudaMemcpyDeviceToDevice, st));
  for (int outer = 0; outer < max_outer; ++outer) {
    GBPC_CUDA_TRY(cudaMemcpyAsync(mask.p, done.data(), sizeof(int) * kB, cudaMemcpyHostToDevice, st));
    if (s.vdtype == GBPC_F32)
      convert_kernel<float, double><<<e_grid(count), 256, 0, st>>>(count, R64.as<double>(), Rin.as<float>());
    else
      GBPC_CUDA_TRY(cudaMemcpyAsync(Rin.p, R64.p, sizeof(double) * count, cudaMemcpyDeviceToDevice, st));
    if (s.vdtype == GBPC_F32)
      mask_columns_kernel<float><<<e_grid(count), 256, 0, st>>>(n, k, mask.as<int>(), Rin.as<float>());
    else
      mask_columns_kernel<double><<<e_grid(count), 256, 0, st>>>(n, k, mask.as<int>(), Rin.as<double>());
    GBPC_CUDA_TRY(cudaMemsetAsync(D.p, 0, dtype_size(s.vdtype) * count, st));
    if ((rc = s.run(k, Rin.p, D.p, tol_inner, 0.0, max_inner, nit.as<int32_t>(), nullptr, st))) return rc;
    GBPC_CUDA_TRY(cudaMemsetAsync(stats.p, 0, sizeof(unsigned long long) * 2 * kB, st));
    if (s.vdtype == GBPC_F32)
      accumulate_kernel<float><<<e_grid(count), 256, 0, st>>>(n, k, D.as<float>(), X,
                                                              stats.as<unsigned long long>(),
                                                              stats.as<unsigned long long>() + kB);
    else
      accumulate_kernel<double><<<e_grid(count), 256, 0, st>>>(n, k, D.as<double>(), X,
                                                               stats.as<unsigned long long>(),
                                                               stats.as<unsigned long long>() + kB);
    GBPC_CUDA_TRY(cudaGetLastError());
    if ((rc = A64->impl->apply(k, X, B, R64.p, -1.0, 1.0, nullptr, nullptr, st))) return rc;
    unsigned long long h[2 * kB];
    int32_t its[kB];
    GBPC_CUDA_TRY(cudaMemcpyAsync(h, stats.p, sizeof(h), cudaMemcpyDeviceToHost, st));
    GBPC_CUDA_TRY(cudaMemcpyAsync(its, nit.p, sizeof(int32_t) * k, cudaMemcpyDeviceToHost, st));
    GBPC_CUDA_TRY(cudaStreamSynchronize(st));
    bool all = true;
    for (int j = 0; j < k; ++j) {
      if (done[j]) continue;
      inner_it[j] += its[j];
      outer_it[j] += 1;
      double dm, xm;
      memcpy(&dm, &h[j], sizeof(double));
      memcpy(&xm, &h[kB + j], sizeof(double));
      if (dm <= tol_outer * xm) done[j] = 1;
      if (!done[j]) all = false;
    }
    if (all) break;
  }
  if (outer_host) memcpy(outer_host, outer_it.data(), sizeof(int32_t) * k);
  if (inner_host) memcpy(inner_host, inner_it.data(), sizeof(int32_t) * k);
  return GBPC_OK;
}
