// Restarted, right-preconditioned GMRES(m) with the whole loop on the device.
//
// warp.optim.linear.gmres (warp-lang, not vendored) is what the reference's
// lifted-biharmonic and indefinite call sites use (tests/test_biharmonic.py:32,
// tests/test_indefinite.py:130, benchmarks/indefinite.py:192-225).  Its exact
// iterates are not pinned by the reference; this is the textbook method:
// Arnoldi on A M with classical Gram-Schmidt applied twice (each pass one
// multi-dot and one multi-axpy over the basis), Givens rotations on the
// Hessenberg column, the residual norm |g_{j+1}| as the stopping quantity
// (stop when it is <= max(atol, tol |b|) or after maxiter steps), and at the
// end of a cycle x += M (V y) with H y = g solved by back-substitution.
//
// One CUDA graph: initialisation (r = b - A x, v_0 = r/|r|), then a
// conditional while-node whose body is one Arnoldi step followed by a
// conditional if-node holding the end-of-cycle update (back-substitution,
// solution update, new residual).  Every reduction is deterministic: per-CTA
// partials, combined in a fixed order by the last CTA to finish.
//
// FP64 throughput, not memory, bounds the Gram-Schmidt kernels on this part
// (about 1.7 FP64 operations per clock per SM, the same for a warp
// instruction whatever its active lanes), so their reductions are laid out
// to spend as few FP64 warp instructions as possible: a reduce-scatter
// butterfly across the lanes, cluster-level sums through distributed shared
// memory, and final sums with one coefficient per lane.

#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "gbpc_common.cuh"
#include "gbpc_internal.h"

namespace gbpc {

int copy_with_dot(int64_t n, const double* x, double* z, const int* guard, const Reduction& red,
                  cudaStream_t st);

namespace {

namespace cg = cooperative_groups;

constexpr int kGT = 256;          // threads per CTA
constexpr int kGMaxK = 65;        // basis vectors (restart <= 64)
constexpr int kGCtas = 152 * 4;   // CTAs of the vector kernels (at most)
constexpr int kGChunk = 16;       // basis vectors per pass over the rows
constexpr int kGCluster = 8;      // CTAs per cluster of the multi-dot
constexpr int kMdotCtas = 152 * 2;  // multi-dot CTAs (at most; a multiple of kGCluster)
constexpr int kMdotClusters = kMdotCtas / kGCluster;
static_assert(kMdotCtas % kGCluster == 0, "multi-dot grid must hold whole clusters");
static_assert(kMdotClusters <= kGCtas, "multi-dot partials fit the partials buffer");

struct GmresState {
  int m, j, it, maxiter;
  int done, not_done, restart, resid;  // flags (ints: operator guards point at them)
  double tol, atol, atol_sq, bb, beta2, ww, res, inv;
  unsigned long long while_handle, if_handle;
};

// Hessenberg workspace: H column-major (m+1) x m, rotations, g, y, the
// current column and the coefficients of the last Gram-Schmidt pass.
struct GmresWork {
  double* H;
  double* cs;
  double* sn;
  double* g;
  double* y;
  double* hcol;
  double* coef;
};

__device__ __forceinline__ void set_cond(unsigned long long h, bool v) {
  if (h != 0ull) cudaGraphSetConditional((cudaGraphConditionalHandle)h, v ? 1u : 0u);
}

int g_grid(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + kGT - 1) / kGT, kGCtas)); }

// Multi-dot grid: whole clusters, at most two CTAs per SM (fewer partials
// for the final sum; a thread takes one or two rows).
int mdot_grid(int64_t n) {
  int64_t g = (n + kGT - 1) / kGT;
  g = (g + kGCluster - 1) / kGCluster * kGCluster;
  return (int)std::max<int64_t>(kGCluster, std::min<int64_t>(g, kMdotCtas));
}

// Sum of a value over the CTA (kGT threads), valid in thread 0.
__device__ __forceinline__ double cta_sum(double v, double* sm) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kGT / 32; ++w) s += sm[w];
  __syncthreads();
  return s;
}

// Total of count (<= kGCtas) partials by the whole CTA: thread t adds the
// partials t, t + kGT, ... (every load issued before the adds), then
// cta_sum.  Deterministic for a given count; valid in thread 0.
__device__ __forceinline__ double cta_total(const double* p, unsigned count, double* sm) {
  constexpr int L = (kGCtas + kGT - 1) / kGT;
  double v[L];
#pragma unroll
  for (int q = 0; q < L; ++q) {
    const unsigned c = threadIdx.x + q * kGT;
    v[q] = c < count ? __ldcg(p + c) : 0.0;
  }
  double t = 0.0;
#pragma unroll
  for (int q = 0; q < L; ++q) t += v[q];
  return cta_sum(t, sm);
}

// Last of `arrivals` CTAs to arrive gets true (after its partial is visible).
__device__ __forceinline__ bool arrive_last(unsigned int* counter, unsigned arrivals) {
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == arrivals - 1;
  __syncthreads();
  if (last) __threadfence();
  return last;
}

__global__ void gm_setup_kernel(GmresState* s, int m, double tol, double atol, int maxiter,
                                unsigned long long while_handle, unsigned long long if_handle) {
  s->m = m;
  s->j = 0;
  s->it = 0;
  s->maxiter = maxiter;
  s->done = 0;
  s->not_done = 1;
  s->restart = 0;
  s->resid = 1;
  s->tol = tol;
  s->atol = atol;
  s->res = 0.0;
  s->while_handle = while_handle;
  s->if_handle = if_handle;
}

// bb = b.b, then atol_sq = max(atol, tol |b|)^2.
__global__ void __launch_bounds__(kGT)
gm_bnorm_kernel(int64_t n, const double* b, GmresState* s, double* partials,
                unsigned int* counter) {
  __shared__ double sm[kGT / 32];
  double acc = 0.0;
  for (int64_t r = (int64_t)blockIdx.x * kGT + threadIdx.x; r < n; r += (int64_t)gridDim.x * kGT)
    acc = fma(b[r], b[r], acc);
  const double cs = cta_sum(acc, sm);
  if (threadIdx.x == 0) partials[blockIdx.x] = cs;
  if (arrive_last(counter, gridDim.x)) {
    const double t = cta_total(partials, gridDim.x, sm);
    if (threadIdx.x == 0) {
      s->bb = t;
      const double a = fmax(s->atol, s->tol * sqrt(t));
      s->atol_sq = a * a;
      *counter = 0u;
    }
  }
}

// Reduce-scatter of C (<= 16) per-lane values across the warp, padded to
// P = 2^p with zeros: level l trades half of the remaining values with the
// lane 16 >> l away and adds, so after p levels lane L holds a partial of
// value L >> (5 - p); 5 - p plain butterfly levels complete it.  P - 1 + 5 - p
// adds per lane against 5 C for C separate shuffle trees.
template <int C>
struct Scatter {
  static constexpr int P = C <= 1 ? 1 : C <= 2 ? 2 : C <= 4 ? 4 : C <= 8 ? 8 : 16;
  static constexpr int p = P == 1 ? 0 : P == 2 ? 1 : P == 4 ? 2 : P == 8 ? 3 : 4;
  static constexpr int low = 5 - p;  // lanes sharing a value: 1 << low
};

template <int C>
__device__ __forceinline__ double scatter_sum(const double (&a)[C]) {
  constexpr int P = Scatter<C>::P, p = Scatter<C>::p;
  const int lane = threadIdx.x & 31;
  double v[P];
#pragma unroll
  for (int q = 0; q < P; ++q) v[q] = q < C ? a[q] : 0.0;
#pragma unroll
  for (int l = 0; l < p; ++l) {
    const int half = P >> (l + 1), off = 16 >> l;
    const bool up = (lane & off) != 0;
#pragma unroll
    for (int q = 0; q < half; ++q) {
      const double send = up ? v[q] : v[q + half];
      const double keep = up ? v[q + half] : v[q];
      v[q] = keep + __shfl_xor_sync(0xffffffffu, send, off);
    }
  }
  double t = v[0];
#pragma unroll
  for (int off = 16 >> p; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
  return t;
}

// One pass over the rows for basis vectors i0 .. i0 + C - 1 (C independent
// loads per row), leaving each warp's sums in sm[warp][i0 + c].
template <int C>
__device__ __forceinline__ void mdot_pass(int64_t n, const double* __restrict__ V,
                                          const double* __restrict__ w, int i0,
                                          double (*sm)[kGMaxK]) {
  double acc[C];
#pragma unroll
  for (int q = 0; q < C; ++q) acc[q] = 0.0;
  const double* Vi = V + (size_t)i0 * n;
  for (int64_t r = (int64_t)blockIdx.x * kGT + threadIdx.x; r < n; r += (int64_t)gridDim.x * kGT) {
    const double wr = w[r];
    double t[C];
#pragma unroll
    for (int q = 0; q < C; ++q) t[q] = Vi[(size_t)q * n + r];
#pragma unroll
    for (int q = 0; q < C; ++q) acc[q] = fma(t[q], wr, acc[q]);
  }
  const double total = scatter_sum<C>(acc);
  constexpr int low = Scatter<C>::low;
  const int lane = threadIdx.x & 31, c = lane >> low;
  if ((lane & ((1 << low) - 1)) == 0 && c < C) sm[threadIdx.x >> 5][i0 + c] = total;
}

// The last rem (< 16) basis vectors with a pass of exactly that width.
template <int C>
__device__ __forceinline__ void mdot_rest(int rem, int64_t n, const double* V, const double* w,
                                          int i0, double (*sm)[kGMaxK]) {
  if constexpr (C > 0) {
    if (rem == C) mdot_pass<C>(n, V, w, i0, sm);
    else mdot_rest<C - 1>(rem, n, V, w, i0, sm);
  }
}

// coef[i] = V_i . w for i <= j (this pass); hcol accumulates the passes.
// Warp sums (scatter_sum) -> CTA sums -> cluster sums in the cluster's
// first CTA, read through distributed shared memory -> per-cluster partials
// -> the last cluster to finish adds them, one coefficient per lane.
__global__ void __cluster_dims__(kGCluster, 1, 1) __launch_bounds__(kGT)
gm_mdot_kernel(int64_t n, const double* V, const double* w, GmresState* s, GmresWork wk,
               int accumulate, double* partials, unsigned int* counter) {
  pdl_wait();
  pdl_launch_dependents();
  // Uniform over the grid (nothing writes it during this kernel), so a whole
  // cluster returns together and no CTA is left at a cluster barrier.
  if (*(volatile int*)&s->not_done == 0) return;
  __shared__ double sm[kGT / 32][kGMaxK];
  __shared__ double cta[kGMaxK];
  const int k = s->j + 1;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int i0 = 0;
  for (; i0 + kGChunk <= k; i0 += kGChunk) mdot_pass<kGChunk>(n, V, w, i0, sm);
  mdot_rest<kGChunk - 1>(k - i0, n, V, w, i0, sm);
  __syncthreads();
  if (threadIdx.x < k) {
    double t = 0.0;
#pragma unroll
    for (int q = 0; q < kGT / 32; ++q) t += sm[q][threadIdx.x];
    cta[threadIdx.x] = t;
  }
  cg::cluster_group cluster = cg::this_cluster();
  cluster.sync();
  const bool leader = cluster.block_rank() == 0;
  if (leader && threadIdx.x < k) {
    double v[kGCluster];
#pragma unroll
    for (int q = 0; q < kGCluster; ++q) v[q] = cluster.map_shared_rank(cta, q)[threadIdx.x];
    double t = 0.0;
#pragma unroll
    for (int q = 0; q < kGCluster; ++q) t += v[q];
    partials[(size_t)(blockIdx.x / kGCluster) * kGMaxK + threadIdx.x] = t;
  }
  cluster.sync();  // the leader's remote reads are done before any CTA exits
  if (!leader) return;
  const unsigned nc = gridDim.x / kGCluster;
  if (arrive_last(counter, nc)) {
    // Warp w adds clusters w, w + 8, ... for coefficients lane, lane + 32, ...
    constexpr int L = (kMdotClusters + kGT / 32 - 1) / (kGT / 32);
    for (int i = lane; i < k; i += 32) {
      double v[L];
#pragma unroll
      for (int q = 0; q < L; ++q) {
        const unsigned c = warp + q * (kGT / 32);
        v[q] = c < nc ? __ldcg(partials + (size_t)c * kGMaxK + i) : 0.0;
      }
      double t = 0.0;
#pragma unroll
      for (int q = 0; q < L; ++q) t += v[q];
      sm[warp][i] = t;
    }
    __syncthreads();
    if (threadIdx.x < k) {
      double t = 0.0;
#pragma unroll
      for (int q = 0; q < kGT / 32; ++q) t += sm[q][threadIdx.x];
      wk.coef[threadIdx.x] = t;
      wk.hcol[threadIdx.x] = accumulate ? wk.hcol[threadIdx.x] + t : t;
    }
    if (threadIdx.x == 0) *counter = 0u;
  }
}

// Givens update of column j and the stopping test, by one full warp.
// Applying rotations 0..j-1 to the new column is the affine recurrence
// a_{i+1} = -s_i a_i + c_i h_{i+1} (a_0 = h_0) with H[i] = c_i a_i + s_i h_{i+1};
// the lanes compose the maps with a shuffle scan (5 levels per 32 rotations)
// instead of one thread stepping through them.
__device__ void gm_step_finalize(GmresState* s, GmresWork wk, double ww) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int j = s->j, m = s->m;
  double* H = wk.H + (size_t)j * (m + 1);
  double carry = wk.hcol[0];  // a_i at the start of the current block of 32
  for (int b0 = 0; b0 < j; b0 += 32) {
    const int i = b0 + lane;
    const bool on = i < j;
    const double c = on ? wk.cs[i] : 1.0;
    const double sn = on ? wk.sn[i] : 0.0;
    const double h1 = on ? wk.hcol[i + 1] : 0.0;
    double al = on ? -sn : 1.0, be = on ? c * h1 : 0.0;  // identity past j
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {  // lane i: maps b0..i composed, i's last
      const double pal = __shfl_up_sync(full, al, o), pbe = __shfl_up_sync(full, be, o);
      if (lane >= o) {
        be = fma(al, pbe, be);
        al = al * pal;
      }
    }
    double pal = __shfl_up_sync(full, al, 1), pbe = __shfl_up_sync(full, be, 1);
    if (lane == 0) {
      pal = 1.0;
      pbe = 0.0;
    }
    const double ai = fma(pal, carry, pbe);
    if (on) H[i] = fma(c, ai, sn * h1);
    carry = fma(__shfl_sync(full, al, 31), carry, __shfl_sync(full, be, 31));
  }
  if (lane != 0) return;
  const double hn = sqrt(ww);
  const double a = carry, b = hn;
  double c = 1.0, sn = 0.0;
  if (b != 0.0) {
    if (fabs(b) > fabs(a)) {
      const double t = a / b;
      sn = 1.0 / sqrt(1.0 + t * t);
      c = sn * t;
    } else {
      const double t = b / a;
      c = 1.0 / sqrt(1.0 + t * t);
      sn = c * t;
    }
  }
  wk.cs[j] = c;
  wk.sn[j] = sn;
  H[j] = c * a + sn * b;
  H[j + 1] = 0.0;
  const double gj = wk.g[j];
  wk.g[j + 1] = -sn * gj;
  wk.g[j] = c * gj;
  s->res = fabs(wk.g[j + 1]);
  s->it += 1;
  const bool breakdown = !(hn > 0.0) || !isfinite(hn);
  s->inv = breakdown ? 0.0 : 1.0 / hn;
  const bool conv = s->res * s->res <= s->atol_sq;
  const bool stop = conv || s->it >= s->maxiter;
  const bool restart = stop || breakdown || (j + 1 == m);
  s->done = stop;
  s->not_done = !stop;
  s->restart = restart;
  s->resid = restart && !stop;
  set_cond(s->if_handle, restart);
  set_cond(s->while_handle, !stop);
}

// v - sum_q cf[q] V_{i0+q}[r] for C basis vectors, loads issued together,
// FMAs in basis order.
template <int C>
__device__ __forceinline__ double update_pass(double v, const double* __restrict__ Vi, int64_t n,
                                              int64_t r, const double* cf) {
  double t[C];
#pragma unroll
  for (int q = 0; q < C; ++q) t[q] = Vi[(size_t)q * n + r];
#pragma unroll
  for (int q = 0; q < C; ++q) v = fma(-cf[q], t[q], v);
  return v;
}

template <int C>
__device__ __forceinline__ double update_rest(int rem, double v, const double* Vi, int64_t n,
                                              int64_t r, const double* cf) {
  if constexpr (C > 0) {
    if (rem == C) return update_pass<C>(v, Vi, n, r, cf);
    return update_rest<C - 1>(rem, v, Vi, n, r, cf);
  }
  return v;
}

// w -= sum_i coef[i] V_i; with `norm`, ww = w.w and the step finalize.
__global__ void __launch_bounds__(kGT)
gm_update_kernel(int64_t n, const double* V, double* w, GmresState* s, GmresWork wk, int norm,
                 double* partials, unsigned int* counter) {
  pdl_wait();
  pdl_launch_dependents();
  if (*(volatile int*)&s->not_done == 0) return;
  __shared__ double sm[kGT / 32];
  __shared__ double cf[kGMaxK];
  const int k = s->j + 1;
  if (threadIdx.x < k) cf[threadIdx.x] = wk.coef[threadIdx.x];
  __syncthreads();
  double acc = 0.0;
  for (int64_t r = (int64_t)blockIdx.x * kGT + threadIdx.x; r < n; r += (int64_t)gridDim.x * kGT) {
    double v = w[r];
    int i = 0;
    for (; i + kGChunk <= k; i += kGChunk)
      v = update_pass<kGChunk>(v, V + (size_t)i * n, n, r, cf + i);
    v = update_rest<kGChunk - 1>(k - i, v, V + (size_t)i * n, n, r, cf + i);
    w[r] = v;
    acc = fma(v, v, acc);
  }
  if (!norm) return;
  const double c = cta_sum(acc, sm);
  if (threadIdx.x == 0) partials[blockIdx.x] = c;
  if (arrive_last(counter, gridDim.x)) {
    const double t = cta_total(partials, gridDim.x, sm);
    if (threadIdx.x < 32) {
      const double ww = __shfl_sync(0xffffffffu, t, 0);
      if (threadIdx.x == 0) {
        s->ww = ww;
        *counter = 0u;
      }
      gm_step_finalize(s, wk, ww);
    }
  }
}

// v_{j+1} = w / h_{j+1} into the basis and the fixed current vector, then j++
// (the last CTA, after every CTA has read j).
__global__ void __launch_bounds__(kGT)
gm_next_kernel(int64_t n, double* V, const double* w, double* vcur, GmresState* s,
               unsigned int* counter) {
  pdl_wait();
  pdl_launch_dependents();
  if (*(volatile int*)&s->restart != 0 || *(volatile int*)&s->not_done == 0) return;
  const int j1 = s->j + 1;
  const double inv = s->inv;
  double* Vn = V + (size_t)j1 * n;
  for (int64_t r = (int64_t)blockIdx.x * kGT + threadIdx.x; r < n; r += (int64_t)gridDim.x * kGT) {
    const double v = w[r] * inv;
    Vn[r] = v;
    vcur[r] = v;
  }
  if (arrive_last(counter, gridDim.x) && threadIdx.x == 0) {
    s->j = j1;
    *counter = 0u;
  }
}

// End of a cycle: H y = g by back-substitution, one warp.  Column-oriented:
// once y_i is known every lane removes H[r, i] y_i from its rows r < i, so
// each step is one multiply and one FMA across the lanes; the diagonal
// reciprocals are formed up front in parallel.
__global__ void gm_solve_kernel(GmresState* s, GmresWork wk) {
  if (*(volatile int*)&s->restart == 0) return;
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int k = s->j + 1, m = s->m;  // k <= 64
  double t0 = 0.0, t1 = 0.0, r0 = 0.0, r1 = 0.0;  // rows lane and lane + 32
  if (lane < k) {
    t0 = wk.g[lane];
    const double d = wk.H[(size_t)lane * (m + 1) + lane];
    r0 = d != 0.0 ? 1.0 / d : 0.0;
  }
  if (lane + 32 < k) {
    t1 = wk.g[lane + 32];
    const double d = wk.H[(size_t)(lane + 32) * (m + 1) + lane + 32];
    r1 = d != 0.0 ? 1.0 / d : 0.0;
  }
  for (int i = k - 1; i >= 0; --i) {
    const bool hi = i >= 32;
    const double ti = __shfl_sync(full, hi ? t1 : t0, i & 31);
    const double ri = __shfl_sync(full, hi ? r1 : r0, i & 31);
    const double yi = ti * ri;
    if (lane == (i & 31)) wk.y[i] = yi;
    const double* col = wk.H + (size_t)i * (m + 1);
    if (lane < i) t0 = fma(-col[lane], yi, t0);
    if (lane + 32 < i) t1 = fma(-col[lane + 32], yi, t1);
  }
}

// t = sum_i y_i V_i
__global__ void __launch_bounds__(kGT)
gm_combine_kernel(int64_t n, const double* V, double* t, const GmresState* s, GmresWork wk) {
  if (*(volatile const int*)&s->restart == 0) return;
  __shared__ double yy[kGMaxK];
  const int k = s->j + 1;
  if (threadIdx.x < k) yy[threadIdx.x] = wk.y[threadIdx.x];
  __syncthreads();
  for (int64_t r = (int64_t)blockIdx.x * kGT + threadIdx.x; r < n; r += (int64_t)gridDim.x * kGT) {
    double v = 0.0;
    for (int i = 0; i < k; ++i) v = fma(yy[i], V[(size_t)i * n + r], v);
    t[r] = v;
  }
}

// x += d
__global__ void __launch_bounds__(kGT)
gm_xupdate_kernel(int64_t n, double* x, const double* d, const GmresState* s) {
  if (*(volatile const int*)&s->restart == 0) return;
  for (int64_t r = (int64_t)blockIdx.x * kGT + threadIdx.x; r < n; r += (int64_t)gridDim.x * kGT)
    x[r] += d[r];
}

// After r = b - A x with beta2 = r.r: start a cycle (or stop).
__global__ void gm_begin_kernel(GmresState* s, GmresWork wk) {
  if (*(volatile int*)&s->resid == 0) return;
  const double beta = sqrt(s->beta2);
  for (int i = 0; i <= s->m; ++i) wk.g[i] = 0.0;
  wk.g[0] = beta;
  s->res = beta;
  s->j = 0;
  const bool conv = s->beta2 <= s->atol_sq;
  const bool stop = conv || !(beta > 0.0) || !isfinite(beta) || s->it >= s->maxiter;
  s->inv = stop ? 0.0 : 1.0 / beta;
  s->done = stop;
  s->not_done = !stop;
  s->restart = 0;
  set_cond(s->while_handle, !stop);
}

// v_0 = r / |r|
__global__ void __launch_bounds__(kGT)
gm_first_kernel(int64_t n, double* V, const double* r, double* vcur, const GmresState* s) {
  if (*(volatile const int*)&s->not_done == 0) return;
  const double inv = s->inv;
  for (int64_t i = (int64_t)blockIdx.x * kGT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kGT) {
    const double v = r[i] * inv;
    V[i] = v;
    vcur[i] = v;
  }
}

__global__ void gm_outputs_kernel(const GmresState* s, int32_t* nit, double* res, double* target) {
  if (nit) *nit = s->it;
  if (res) *res = s->res;
  if (target) *target = sqrt(s->atol_sq);
}

}  // namespace

struct Gmres {
  size_t device_bytes = 0;  // DevBuf bytes held (declared first: released last)
  Operator* A = nullptr;
  Operator* M = nullptr;
  int64_t n = 0;
  int m = 31;
  DevBuf V, w, t, d, vcur, state, work, partials, counter;
  ReduceBuf rb;
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphConditionalHandle while_h = 0, if_h = 0;
  const double* last_b = nullptr;
  double* last_x = nullptr;

  ~Gmres() { drop(); }
  void drop() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
    last_b = nullptr;
    last_x = nullptr;
  }
  GmresState* S() { return state.as<GmresState>(); }
  GmresWork W() {
    double* base = work.as<double>();
    GmresWork wk;
    wk.H = base;
    wk.cs = wk.H + (size_t)(m + 1) * m;
    wk.sn = wk.cs + m;
    wk.g = wk.sn + m;
    wk.y = wk.g + (m + 1);
    wk.hcol = wk.y + m;
    wk.coef = wk.hcol + (m + 1);
    return wk;
  }
  static size_t work_doubles(int m) { return (size_t)(m + 1) * m + 2 * (size_t)m + 2 * (size_t)(m + 1) + m + (m + 1); }

  int precondition(const double* in, double* out, const int* guard, cudaStream_t st) {
    if (M) return M->apply(in, nullptr, out, 1.0, 0.0, guard, nullptr, st);
    GBPC_CUDA_TRY(cudaMemcpyAsync(out, in, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    return GBPC_OK;
  }

  // r = b - A x into w with beta2, then start a cycle.
  int record_residual(const double* b, double* x, const int* guard, cudaStream_t st) {
    DotSpec dot;
    dot.w = w.as<double>();
    dot.rb = &rb;
    dot.mode = FIN_STORE;
    dot.out = &S()->beta2;
    int rc;
    if ((rc = A->apply(x, b, w.p, -1.0, 1.0, guard, &dot, st))) return rc;
    gm_begin_kernel<<<1, 1, 0, st>>>(S(), W());
    gm_first_kernel<<<g_grid(n), kGT, 0, st>>>(n, V.as<double>(), w.as<double>(),
                                                vcur.as<double>(), S());
    GBPC_CUDA_TRY(cudaGetLastError());
    return GBPC_OK;
  }

  int record_init(const double* b, double* x, cudaStream_t st) {
    GBPC_CUDA_TRY(cudaMemsetAsync(counter.p, 0, sizeof(unsigned int), st));
    gm_bnorm_kernel<<<g_grid(n), kGT, 0, st>>>(n, b, S(), partials.as<double>(),
                                                counter.as<unsigned int>());
    GBPC_CUDA_TRY(cudaGetLastError());
    return record_residual(b, x, nullptr, st);
  }

  // One Arnoldi step: w = A M v_j, two Gram-Schmidt passes, Givens, v_{j+1}.
  int record_step(cudaStream_t st) {
    const int* guard = &S()->not_done;
    int rc;
    const double* in = vcur.as<double>();
    if (M) {
      if ((rc = M->apply(vcur.p, nullptr, t.p, 1.0, 0.0, guard, nullptr, st))) return rc;
      in = t.as<double>();
    }
    if ((rc = A->apply(in, nullptr, w.p, 1.0, 0.0, guard, nullptr, st))) return rc;
    for (int pass = 0; pass < 2; ++pass) {
      GBPC_CUDA_TRY(launch_k(gm_mdot_kernel, mdot_grid(n), kGT, 0, st, n,
                             (const double*)V.as<double>(), (const double*)w.as<double>(), S(), W(),
                             pass, partials.as<double>(), counter.as<unsigned int>()));
      GBPC_CUDA_TRY(launch_k(gm_update_kernel, g_grid(n), kGT, 0, st, n,
                             (const double*)V.as<double>(), w.as<double>(), S(), W(), pass,
                             partials.as<double>(), counter.as<unsigned int>()));
    }
    GBPC_CUDA_TRY(launch_k(gm_next_kernel, g_grid(n), kGT, 0, st, n, V.as<double>(),
                           (const double*)w.as<double>(), vcur.as<double>(), S(),
                           counter.as<unsigned int>()));
    return GBPC_OK;
  }

  // End of a cycle: y, x += M (V y), and (unless finished) the next residual.
  int record_cycle_end(const double* b, double* x, cudaStream_t st) {
    int rc;
    gm_solve_kernel<<<1, 32, 0, st>>>(S(), W());
    gm_combine_kernel<<<g_grid(n), kGT, 0, st>>>(n, V.as<double>(), t.as<double>(), S(), W());
    GBPC_CUDA_TRY(cudaGetLastError());
    const double* dx = t.as<double>();
    if (M) {
      if ((rc = M->apply(t.p, nullptr, d.p, 1.0, 0.0, &S()->restart, nullptr, st))) return rc;
      dx = d.as<double>();
    }
    gm_xupdate_kernel<<<g_grid(n), kGT, 0, st>>>(n, x, dx, S());
    GBPC_CUDA_TRY(cudaGetLastError());
    return record_residual(b, x, &S()->resid, st);
  }

  static int tail_of(cudaGraph_t g, cudaGraphNode_t* tail) {
    size_t count = 0;
    cudaGraphGetNodes(g, nullptr, &count);
    std::vector<cudaGraphNode_t> nodes(count);
    cudaGraphGetNodes(g, nodes.data(), &count);
    *tail = nullptr;
    for (auto nd : nodes) {
      size_t outs = 0;
      cudaGraphNodeGetDependentNodes(nd, nullptr, nullptr, &outs);
      if (outs == 0) *tail = nd;
    }
    return GBPC_OK;
  }

  int build_graph(const double* b, double* x, cudaStream_t st) {
    (void)st;
    drop();
    GBPC_CUDA_TRY(cudaGraphCreate(&graph, 0));
    GBPC_CUDA_TRY(cudaGraphConditionalHandleCreate(&while_h, graph, 0, cudaGraphCondAssignDefault));
    cudaStream_t cs;
    GBPC_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    int rc = GBPC_OK;
    cudaGraph_t g2 = nullptr;
    do {
      if (cudaStreamBeginCaptureToGraph(cs, graph, nullptr, nullptr, 0,
                                        cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        rc = GBPC_ERR_CUDA;
        break;
      }
      rc = record_init(b, x, cs);
      cudaError_t e = cudaStreamEndCapture(cs, &g2);
      if (rc) break;
      if (e != cudaSuccess) {
        gbpc_set_error_cuda(e, "capture GMRES init", __FILE__, __LINE__);
        rc = GBPC_ERR_CUDA;
        break;
      }
      cudaGraphNode_t tail = nullptr;
      tail_of(graph, &tail);
      cudaGraphNodeParams wp = {};
      wp.type = cudaGraphNodeTypeConditional;
      wp.conditional.handle = while_h;
      wp.conditional.type = cudaGraphCondTypeWhile;
      wp.conditional.size = 1;
      cudaGraphNode_t wnode;
      e = cudaGraphAddNode(&wnode, graph, tail ? &tail : nullptr, nullptr, tail ? 1 : 0, &wp);
      if (e != cudaSuccess) {
        gbpc_set_error_cuda(e, "add GMRES while node", __FILE__, __LINE__);
        rc = GBPC_ERR_CUDA;
        break;
      }
      cudaGraph_t body = wp.conditional.phGraph_out[0];
      if ((e = cudaGraphConditionalHandleCreate(&if_h, body, 0, cudaGraphCondAssignDefault)) !=
          cudaSuccess) {
        gbpc_set_error_cuda(e, "GMRES if handle", __FILE__, __LINE__);
        rc = GBPC_ERR_CUDA;
        break;
      }
      if (cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0,
                                        cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        rc = GBPC_ERR_CUDA;
        break;
      }
      {
        PdlScope scope(true);
        rc = record_step(cs);
      }
      e = cudaStreamEndCapture(cs, &g2);
      if (rc) break;
      if (e != cudaSuccess) {
        gbpc_set_error_cuda(e, "capture GMRES step", __FILE__, __LINE__);
        rc = GBPC_ERR_CUDA;
        break;
      }
      tail_of(body, &tail);
      cudaGraphNodeParams ip = {};
      ip.type = cudaGraphNodeTypeConditional;
      ip.conditional.handle = if_h;
      ip.conditional.type = cudaGraphCondTypeIf;
      ip.conditional.size = 1;
      cudaGraphNode_t inode;
      e = cudaGraphAddNode(&inode, body, tail ? &tail : nullptr, nullptr, tail ? 1 : 0, &ip);
      if (e != cudaSuccess) {
        gbpc_set_error_cuda(e, "add GMRES if node", __FILE__, __LINE__);
        rc = GBPC_ERR_CUDA;
        break;
      }
      cudaGraph_t ibody = ip.conditional.phGraph_out[0];
      if (cudaStreamBeginCaptureToGraph(cs, ibody, nullptr, nullptr, 0,
                                        cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        rc = GBPC_ERR_CUDA;
        break;
      }
      rc = record_cycle_end(b, x, cs);
      e = cudaStreamEndCapture(cs, &g2);
      if (rc) break;
      if (e != cudaSuccess) {
        gbpc_set_error_cuda(e, "capture GMRES cycle end", __FILE__, __LINE__);
        rc = GBPC_ERR_CUDA;
        break;
      }
      e = cudaGraphInstantiate(&exec, graph, 0);
      if (e != cudaSuccess) {
        gbpc_set_error_cuda(e, "instantiate GMRES", __FILE__, __LINE__);
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
    last_b = b;
    last_x = x;
    return GBPC_OK;
  }

  int run(const double* b, double* x, double tol, double atol, int maxiter, bool use_graph,
          int32_t* nit, double* res, double* target, cudaStream_t st) {
    if (maxiter <= 0) maxiter = (int)std::min<int64_t>(std::max<int64_t>(n, 1), 0x7fffffff);
    int rc;
    if (use_graph) {
      if (!exec || last_b != b || last_x != x) {
        if ((rc = build_graph(b, x, st))) return rc;
      }
      gm_setup_kernel<<<1, 1, 0, st>>>(S(), m, tol, atol, maxiter, (unsigned long long)while_h,
                                       (unsigned long long)if_h);
      GBPC_CUDA_TRY(cudaGetLastError());
      GBPC_CUDA_TRY(cudaGraphLaunch(exec, st));
    } else {
      // Host-driven loop of the same kernels (every kernel checks the flags).
      gm_setup_kernel<<<1, 1, 0, st>>>(S(), m, tol, atol, maxiter, 0ull, 0ull);
      if ((rc = record_init(b, x, st))) return rc;
      int flags[2] = {1, 0};  // not_done, restart
      for (int step = 0; step < maxiter + 1 && flags[0]; ++step) {
        if ((rc = record_step(st))) return rc;
        GBPC_CUDA_TRY(cudaMemcpyAsync(flags + 1, &S()->restart, sizeof(int), cudaMemcpyDeviceToHost, st));
        GBPC_CUDA_TRY(cudaStreamSynchronize(st));
        if (flags[1] && (rc = record_cycle_end(b, x, st))) return rc;
        GBPC_CUDA_TRY(cudaMemcpyAsync(flags, &S()->not_done, sizeof(int), cudaMemcpyDeviceToHost, st));
        GBPC_CUDA_TRY(cudaStreamSynchronize(st));
      }
    }
    gm_outputs_kernel<<<1, 1, 0, st>>>(S(), nit, res, target);
    GBPC_CUDA_TRY(cudaGetLastError());
    return GBPC_OK;
  }
};

}  // namespace gbpc

using namespace gbpc;

struct gbpc_gmres {
  Gmres g;
};

extern "C" int gbpc_gmres_create(gbpc_op* A, gbpc_op* M, int restart, void* stream,
                                 gbpc_gmres** out) {
  if (!out || !A || !A->impl || restart < 1 || restart > kGMaxK - 1) {
    gbpc_set_error("gbpc_gmres_create: bad arguments (restart must be 1..%d)", kGMaxK - 1);
    return GBPC_ERR_ARG;
  }
  Operator* a = A->impl.get();
  Operator* m = (M && M->impl) ? M->impl.get() : nullptr;
  if (a->vdtype != GBPC_F64 || (m && m->vdtype != GBPC_F64)) {
    gbpc_set_error("GMRES runs on float64 vectors");
    return GBPC_ERR_ARG;
  }
  if (m && m->rows != a->rows) {
    gbpc_set_error("operator and preconditioner sizes differ (%lld vs %lld)", (long long)a->rows,
                   (long long)m->rows);
    return GBPC_ERR_ARG;
  }
  auto* h = new gbpc_gmres;
  Gmres& g = h->g;
  ByteTally tally(&g.device_bytes);
  g.A = a;
  g.M = m;
  g.n = a->rows;
  g.m = restart;
  const size_t vec = sizeof(double) * std::max<int64_t>(g.n, 1);
  int rc = g.V.alloc(vec * (restart + 1));
  if (!rc) rc = g.w.alloc(vec);
  if (!rc) rc = g.t.alloc(vec);
  if (!rc) rc = g.d.alloc(vec);
  if (!rc) rc = g.vcur.alloc(vec);
  if (!rc) rc = g.state.alloc(sizeof(GmresState));
  if (!rc) rc = g.work.alloc(sizeof(double) * Gmres::work_doubles(restart));
  if (!rc) rc = g.partials.alloc(sizeof(double) * (size_t)kGCtas * kGMaxK);
  if (!rc) rc = g.counter.alloc(sizeof(unsigned int));
  if (!rc) rc = g.rb.init((cudaStream_t)stream);
  cudaStream_t st = (cudaStream_t)stream;
  if (!rc && (cudaMemsetAsync(g.counter.p, 0, sizeof(unsigned int), st) != cudaSuccess ||
              cudaMemsetAsync(g.work.p, 0, sizeof(double) * Gmres::work_doubles(restart), st) !=
                  cudaSuccess ||
              cudaMemsetAsync(g.state.p, 0, sizeof(GmresState), st) != cudaSuccess ||
              cudaStreamSynchronize(st) != cudaSuccess))
    rc = GBPC_ERR_CUDA;
  if (rc) {
    delete h;
    return rc;
  }
  *out = h;
  return GBPC_OK;
}

extern "C" int gbpc_gmres_run(gbpc_gmres* h, const double* b, double* x, double tol, double atol,
                              int maxiter, int use_graph, int32_t* nit_dev, double* res_dev,
                              double* target_dev, void* stream) {
  NvtxRange nvtx_range("gbpc_gmres_run");
  if (!h || !b || !x) {
    gbpc_set_error("gbpc_gmres_run: bad arguments");
    return GBPC_ERR_ARG;
  }
  return h->g.run(b, x, tol, atol, maxiter, use_graph != 0, nit_dev, res_dev, target_dev,
                  (cudaStream_t)stream);
}

extern "C" int gbpc_gmres_device_bytes(const gbpc_gmres* h, size_t* bytes_host) {
  if (!h || !bytes_host) {
    gbpc_set_error("gbpc_gmres_device_bytes: bad arguments");
    return GBPC_ERR_ARG;
  }
  *bytes_host = h->g.device_bytes;
  return GBPC_OK;
}

extern "C" int gbpc_gmres_destroy(gbpc_gmres* h) {
  if (!h) return GBPC_OK;
  cudaDeviceSynchronize();
  delete h;
  return GBPC_OK;
}
