// The sliced sparse product (SELL-32) shared by the per-vector-type
// translation units gbpc_spmv_f64.cu and gbpc_spmv_f32.cu.
#pragma once

#include <type_traits>

#include "gbpc_common.cuh"
#include "gbpc_internal.h"

namespace gbpc {

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
template <> struct Chunk<4> { static constexpr int value = 1; };

// Epilogue of one row: z[row] from the accumulated product (and the fused
// dot contribution, in row order of the calling thread).
template <int B, typename V, typename A, int EPI, bool DOT>
__device__ __forceinline__ void spmv_finish(const SellView<V>& m, int row, const A (&acc)[B],
                                            const A* y, A* z, A alpha, A beta, bool run,
                                            bool alpha_one, bool beta_zero, const EpiDev<A>& ep,
                                            const Reduction& red, double& dot_part) {
  constexpr int BB = B * B;
  if (row < m.nrow) {
    const int orow = m.perm ? __ldg(m.perm + row) : row;
    A out[B];
#pragma unroll
    for (int r = 0; r < B; ++r) {
      const int64_t idx = (int64_t)orow * B + r;
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
        for (int q = 0; q < B; ++q) s2 = fma_t<A>(ep.aux1[(int64_t)orow * BB + r * B + q], out[q], s2);
        t[r] = s2;
      }
#pragma unroll
      for (int r = 0; r < B; ++r) out[r] = t[r];
    }
#pragma unroll
    for (int r = 0; r < B; ++r) {
      const int64_t idx = (int64_t)orow * B + r;
      z[idx] = out[r];
      if (DOT) dot_part = fma((double)out[r], red.w[idx], dot_part);
    }
  }
}

template <int B, typename V, typename A, int EPI, bool DOT, int CH, int MINB, bool UNIT = false>
__global__ void __launch_bounds__(kThreads, MINB)
sell_spmv_kernel(SellView<V> m, const A* x, const A* y, A* z, A alpha, A beta, int flags,
                 const int* guard, EpiDev<A> ep, Reduction red) {
  pdl_wait();
  pdl_launch_dependents();
  if (guard_off(guard)) return;
  constexpr int BB = B * B;
  const bool run =
      UNIT || (EPI == EPI_TRI_LOWER || EPI == EPI_TRI_UPPER) || !(flags & F_ALPHA_ZERO);
  const bool alpha_one = UNIT || (flags & F_ALPHA_ONE) != 0;
  const bool beta_zero = UNIT || (flags & F_BETA_ZERO) != 0;
  const int lane = threadIdx.x & 31;
  const int warps_total = gridDim.x * (kThreads / 32);
  double dot_part = 0.0;
  // Warp w of CTA c is schedule lane t = w * gridDim.x + c (a CTA's warps
  // sit far apart in the schedule) and takes one slice per pass, passes
  // alternating direction over the slices sorted by width: every warp gets a
  // mix of wide and narrow slices, and the slowest warp, which the kernel
  // waits for, carries close to the average work.
  const int t = (threadIdx.x >> 5) * gridDim.x + blockIdx.x;
  for (int i = 0;; ++i) {
    const int64_t idx = warp_slice(i, t, warps_total, m.nslices, !DOT && m.reverse);
    if (idx < 0) break;  // later passes lie further out
    const SliceTask task = load_task(m.sched, idx);
    const int row = task.s * kSlice + lane;
    const int64_t base = task.base;
    const int width = task.width;
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
    spmv_finish<B, V, A, EPI, DOT>(m, row, acc, y, z, alpha, beta, run, alpha_one, beta_zero, ep,
                                   red, dot_part);
  }
  if (DOT) reduce_and_finalize(red, dot_part);
}

// Scalar rows, two slices at once: the slices of passes i and i + 1 that the
// loop above would take one after the other are read together, so
// every lane keeps two independent FMA chains and twice the loads in flight.
// Each row still sums its entries in storage order, and the dot product
// receives the rows in the same order, so the result equals the one-slice
// kernel's bit for bit.
template <typename V, typename A, int EPI, bool DOT, int CH, bool UNIT = false>
__global__ void __launch_bounds__(kThreads, 1)
sell_spmv2_kernel(SellView<V> m, const A* x, const A* y, A* z, A alpha, A beta, int flags,
                  const int* guard, EpiDev<A> ep, Reduction red) {
  pdl_wait();
  pdl_launch_dependents();
  if (guard_off(guard)) return;
  const bool run =
      UNIT || (EPI == EPI_TRI_LOWER || EPI == EPI_TRI_UPPER) || !(flags & F_ALPHA_ZERO);
  const bool alpha_one = UNIT || (flags & F_ALPHA_ONE) != 0;
  const bool beta_zero = UNIT || (flags & F_BETA_ZERO) != 0;
  const int lane = threadIdx.x & 31;
  const int warps_total = gridDim.x * (kThreads / 32);
  double dot_part = 0.0;
  // Passes i and i + 1 of the one-slice kernel's schedule together.
  const int t = (threadIdx.x >> 5) * gridDim.x + blockIdx.x;
  for (int i = 0; (int64_t)i * warps_total < m.nslices; i += 2) {
    const int64_t idx1 = sched_index(i, t, warps_total);
    if (idx1 >= m.nslices) break;
    const int64_t idx2 = sched_index(i + 1, t, warps_total);
    const bool has2 = idx2 < m.nslices;  // uniform across the warp
    const SliceTask t1 = load_task(m.sched, idx1);
    const int s = t1.s;
    const int64_t base1 = t1.base;
    const int width1 = t1.width;
    int s2 = 0;
    int64_t base2 = 0;
    int width2 = 0;
    if (has2) {
      const SliceTask t2 = load_task(m.sched, idx2);
      s2 = t2.s;
      base2 = t2.base;
      width2 = t2.width;
    }
    A acc1[1] = {A(0)}, acc2[1] = {A(0)};
    if (run) {
      const int32_t* cp1 = m.cols + base1 + lane;
      const V* vp1 = m.vals + base1 + lane;
      const int32_t* cp2 = m.cols + base2 + lane;
      const V* vp2 = m.vals + base2 + lane;
      const int wmax = max(width1, width2);
      for (int k0 = 0; k0 < wmax; k0 += CH) {
        int c1[CH], c2[CH];
#pragma unroll
        for (int j = 0; j < CH; ++j) {
          c1[j] = (k0 + j < width1) ? __ldg(cp1 + (int64_t)(k0 + j) * kSlice) : -1;
          c2[j] = (k0 + j < width2) ? __ldg(cp2 + (int64_t)(k0 + j) * kSlice) : -1;
        }
        A x1[CH], x2[CH];
        V v1[CH], v2[CH];
#pragma unroll
        for (int j = 0; j < CH; ++j) {
          x1[j] = (c1[j] >= 0) ? __ldg(x + c1[j]) : A(0);
          x2[j] = (c2[j] >= 0) ? __ldg(x + c2[j]) : A(0);
          v1[j] = (k0 + j < width1) ? __ldg(vp1 + (int64_t)(k0 + j) * kSlice) : static_cast<V>(0.0f);
          v2[j] = (k0 + j < width2) ? __ldg(vp2 + (int64_t)(k0 + j) * kSlice) : static_cast<V>(0.0f);
        }
#pragma unroll
        for (int j = 0; j < CH; ++j) {
          if (k0 + j < width1) acc1[0] = fma_t<A>(widen<A, V>(v1[j]), x1[j], acc1[0]);
          if (k0 + j < width2) acc2[0] = fma_t<A>(widen<A, V>(v2[j]), x2[j], acc2[0]);
        }
      }
    }
    spmv_finish<1, V, A, EPI, DOT>(m, s * kSlice + lane, acc1, y, z, alpha, beta, run, alpha_one,
                                   beta_zero, ep, red, dot_part);
    if (has2)
      spmv_finish<1, V, A, EPI, DOT>(m, s2 * kSlice + lane, acc2, y, z, alpha, beta, run,
                                     alpha_one, beta_zero, ep, red, dot_part);
  }
  if (DOT) reduce_and_finalize(red, dot_part);
}

// Chunk ch (CH entries per lane) of a slice into registers: column -1 and
// value 0 past the slice's width (the same padding the other variants use).
template <typename V, int CH>
__device__ __forceinline__ void load_chunk(const SellView<V>& m, const SliceTask& task, int k0,
                                           int lane, int (&c)[CH], V (&v)[CH]) {
  const int32_t* cp = m.cols + task.base + lane;
  const V* vp = m.vals + task.base + lane;
#pragma unroll
  for (int j = 0; j < CH; ++j) {
    const bool in = k0 + j < task.width;
    c[j] = in ? __ldg(cp + (int64_t)(k0 + j) * kSlice) : -1;
    v[j] = in ? __ldg(vp + (int64_t)(k0 + j) * kSlice) : static_cast<V>(0.0f);
  }
}

// Scalar rows, software-pipelined: a warp walks the chunks of its slices
// (same schedule as above) as one stream and loads chunk c + 1's columns and
// values, which come from DRAM, before it gathers x for chunk c (mostly L2
// hits) and issues chunk c's FMAs, so a warp's own FMAs cover part of its
// DRAM latency and a slice costs one dependent round trip instead of three.
// The FMAs, their order and the padding treatment are those of the
// one-slice kernel, so the results are identical bit for bit.
// UNIT: alpha == 1 and beta == 0 known at compile time (every product of
// the Krylov loops), so the epilogue carries no scaling or y term at all.
template <typename V, typename A, int EPI, bool DOT, int CH, bool UNIT = false>
__global__ void __launch_bounds__(kThreads, 1)
sell_spmv_pipe_kernel(SellView<V> m, const A* x, const A* y, A* z, A alpha, A beta, int flags,
                      const int* guard, EpiDev<A> ep, Reduction red) {
  const bool run =
      UNIT || (EPI == EPI_TRI_LOWER || EPI == EPI_TRI_UPPER) || !(flags & F_ALPHA_ZERO);
  const bool alpha_one = UNIT || (flags & F_ALPHA_ONE) != 0;
  const bool beta_zero = UNIT || (flags & F_BETA_ZERO) != 0;
  const int lane = threadIdx.x & 31;
  const int warps_total = gridDim.x * (kThreads / 32);
  const int t = (threadIdx.x >> 5) * gridDim.x + blockIdx.x;
  // The matrix does not change while a solve runs (it is written only by
  // builds and refills, which complete before any product that follows them
  // starts), so the warp's first schedule entries and first chunk are read
  // before the wait on the previous kernel: under programmatic dependent
  // launch these loads overlap that kernel's tail.  Only x, y and the guard
  // come from the previous kernel.
  const bool rev = !DOT && m.reverse;
  const int64_t idx = warp_slice(0, t, warps_total, m.nslices, rev);
  const bool any = idx >= 0;
  SliceTask cur{-1, 0, 0}, nxt{-1, 0, 0};
  int pc[CH];
  V pv[CH];
  bool have = false;  // pc/pv hold the first chunk of cur
  if (any) {
    cur = load_task(m.sched, idx);
    const int64_t nidx = warp_slice(1, t, warps_total, m.nslices, rev);
    if (nidx >= 0) nxt = load_task(m.sched, nidx);
    if (run) {
      load_chunk<V, CH>(m, cur, 0, lane, pc, pv);
      have = true;
    }
  }
  pdl_wait();
  pdl_launch_dependents();
  if (guard_off(guard)) return;
  double dot_part = 0.0;
  if (any) {
    int i = 0;
    while (true) {
      A acc[1] = {A(0)};
      if (run) {
        if (!have) load_chunk<V, CH>(m, cur, 0, lane, pc, pv);
        have = false;
        for (int k0 = 0; k0 < cur.width; k0 += CH) {  // uniform across the warp
          int c[CH];
          V v[CH];
#pragma unroll
          for (int j = 0; j < CH; ++j) {
            c[j] = pc[j];
            v[j] = pv[j];
          }
          if (k0 + CH < cur.width) {
            load_chunk<V, CH>(m, cur, k0 + CH, lane, pc, pv);
          } else if (nxt.s >= 0) {
            load_chunk<V, CH>(m, nxt, 0, lane, pc, pv);
            have = true;
          }
          A xv[CH];
#pragma unroll
          for (int j = 0; j < CH; ++j) xv[j] = (c[j] >= 0) ? __ldg(x + c[j]) : A(0);
#pragma unroll
          for (int j = 0; j < CH; ++j)
            if (k0 + j < cur.width) acc[0] = fma_t<A>(widen<A, V>(v[j]), xv[j], acc[0]);
        }
      }
      spmv_finish<1, V, A, EPI, DOT>(m, cur.s * kSlice + lane, acc, y, z, alpha, beta, run,
                                     alpha_one, beta_zero, ep, red, dot_part);
      if (nxt.s < 0) break;
      cur = nxt;
      ++i;
      const int64_t nidx = warp_slice(i + 1, t, warps_total, m.nslices, rev);
      nxt = nidx >= 0 ? load_task(m.sched, nidx) : SliceTask{-1, 0, 0};
    }
  }
  if (DOT) reduce_and_finalize(red, dot_part);
}

// Blocked rows (B x B blocks), software-pipelined like the scalar kernel
// above: chunk c + 1's block columns and B*B values are loaded before chunk
// c's x gathers and FMAs.  The FMAs run in sell_spmv_kernel's order (entry,
// then block row r, then column q), so the results equal the one-slice
// blocked kernel's bit for bit.  CH = 2 for 2 x 2 blocks, 1 for 3 x 3 (the
// 64-register budget).
template <typename V, int B, int CH>
__device__ __forceinline__ void load_chunk_b(const SellView<V>& m, const SliceTask& task, int k0,
                                             int lane, int (&c)[CH], V (&v)[CH][B * B]) {
  constexpr int BB = B * B;
  const int32_t* cp = m.cols + task.base + lane;
  const V* vp = m.vals + task.base * BB + lane;
#pragma unroll
  for (int j = 0; j < CH; ++j) {
    const bool in = k0 + j < task.width;
    c[j] = in ? __ldg(cp + (int64_t)(k0 + j) * kSlice) : -1;
#pragma unroll
    for (int q = 0; q < BB; ++q)
      v[j][q] = in ? __ldg(vp + ((int64_t)(k0 + j) * BB + q) * kSlice) : static_cast<V>(0.0f);
  }
}

template <int B, typename V, typename A, int EPI, bool DOT, int CH, bool UNIT = false>
__global__ void __launch_bounds__(kThreads, 1)
sell_spmv_bpipe_kernel(SellView<V> m, const A* x, const A* y, A* z, A alpha, A beta, int flags,
                       const int* guard, EpiDev<A> ep, Reduction red) {
  constexpr int BB = B * B;
  const bool run =
      UNIT || (EPI == EPI_TRI_LOWER || EPI == EPI_TRI_UPPER) || !(flags & F_ALPHA_ZERO);
  const bool alpha_one = UNIT || (flags & F_ALPHA_ONE) != 0;
  const bool beta_zero = UNIT || (flags & F_BETA_ZERO) != 0;
  const int lane = threadIdx.x & 31;
  const int warps_total = gridDim.x * (kThreads / 32);
  const int t = (threadIdx.x >> 5) * gridDim.x + blockIdx.x;
  // First schedule entries and chunk before the wait (the matrix is not
  // written while a solve runs; see the scalar kernel).
  const int64_t idx = sched_index(0, t, warps_total);
  const bool any = idx < m.nslices;
  SliceTask cur{-1, 0, 0}, nxt{-1, 0, 0};
  int pc[CH];
  V pv[CH][BB];
  bool have = false;
  if (any) {
    cur = load_task(m.sched, idx);
    const int64_t nidx = sched_index(1, t, warps_total);
    if (nidx < m.nslices) nxt = load_task(m.sched, nidx);
    if (run) {
      load_chunk_b<V, B, CH>(m, cur, 0, lane, pc, pv);
      have = true;
    }
  }
  pdl_wait();
  pdl_launch_dependents();
  if (guard_off(guard)) return;
  double dot_part = 0.0;
  if (any) {
    int i = 0;
    while (true) {
      A acc[B];
#pragma unroll
      for (int r = 0; r < B; ++r) acc[r] = A(0);
      if (run) {
        if (!have) load_chunk_b<V, B, CH>(m, cur, 0, lane, pc, pv);
        have = false;
        for (int k0 = 0; k0 < cur.width; k0 += CH) {  // uniform across the warp
          int c[CH];
          V v[CH][BB];
#pragma unroll
          for (int j = 0; j < CH; ++j) {
            c[j] = pc[j];
#pragma unroll
            for (int q = 0; q < BB; ++q) v[j][q] = pv[j][q];
          }
          if (k0 + CH < cur.width) {
            load_chunk_b<V, B, CH>(m, cur, k0 + CH, lane, pc, pv);
          } else if (nxt.s >= 0) {
            load_chunk_b<V, B, CH>(m, nxt, 0, lane, pc, pv);
            have = true;
          }
          A xv[CH][B];
#pragma unroll
          for (int j = 0; j < CH; ++j)
#pragma unroll
            for (int q = 0; q < B; ++q)
              xv[j][q] = (c[j] >= 0) ? __ldg(x + (int64_t)c[j] * B + q) : A(0);
#pragma unroll
          for (int j = 0; j < CH; ++j) {
            if (k0 + j < cur.width) {
#pragma unroll
              for (int r = 0; r < B; ++r)
#pragma unroll
                for (int q = 0; q < B; ++q)
                  acc[r] = fma_t<A>(widen<A, V>(v[j][r * B + q]), xv[j][q], acc[r]);
            }
          }
        }
      }
      spmv_finish<B, V, A, EPI, DOT>(m, cur.s * kSlice + lane, acc, y, z, alpha, beta, run,
                                     alpha_one, beta_zero, ep, red, dot_part);
      if (nxt.s < 0) break;
      cur = nxt;
      ++i;
      const int64_t nidx = sched_index(i + 1, t, warps_total);
      nxt = nidx < m.nslices ? load_task(m.sched, nidx) : SliceTask{-1, 0, 0};
    }
  }
  if (DOT) reduce_and_finalize(red, dot_part);
}

// ---------------------------------------------------------------------------
// Scalar rows with the matrix streamed by the bulk-copy engine.
//
// A slice's entries are contiguous (column-major inside the slice), so a
// chunk of CH entries per lane is one block of 128 CH bytes of columns and
// one of 32 CH sizeof(V) bytes of values.  Each warp owns a ring of NS
// shared-memory stages; lane 0 keeps the next NS chunks of the warp's slice
// sequence in flight with cp.async.bulk (completion counted in bytes on an
// mbarrier per stage), so the DRAM stream no longer costs registers or
// waits on the warp.  The warp reads a stage into registers, hands it back
// to the copy engine at once, issues that chunk's x gathers, and only then
// multiplies the previous chunk, whose gathers have been in flight for a
// whole step.  Rows still sum their entries in storage order, slices are
// finished in the schedule order of the other variants and the grid is the
// same, so results (fused dot included) are identical to theirs bit for bit.
// Every mbarrier wait is bounded: a wait that gives up sets *m.err, waits
// (bounded) for the warp's copies in flight and leaves the kernel.

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void bulk_to_smem(void* dst, const void* src, uint32_t bytes,
                                             uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

constexpr int kBulkCH = 4;                 // entries per lane per stage
constexpr int kBulkStageBytesMax = 6144;   // shared memory per warp for its ring
constexpr uint32_t kBulkSpinLimit = 1u << 20;  // try_wait rounds before giving up

template <typename V>
struct BulkCfg {
  static constexpr int kColBytes = kBulkCH * kSlice * 4;
  static constexpr int kValBytes = kBulkCH * kSlice * (int)sizeof(V);
  static constexpr int kStage = kColBytes + kValBytes;
  static constexpr int NS = kBulkStageBytesMax / kStage;  // 4 (double), 6 (float), 8 (bf16)
  static constexpr int kWarpBytes = NS * kStage;
  static constexpr size_t kSmem = (size_t)(kThreads / 32) * (kWarpBytes + NS * 8);
};

// The warp's chunk sequence: its slices in schedule order, CH entries of
// each at a time, slices of width 0 skipped (they have no entries to copy).
struct ChunkCursor {
  int i;          // schedule pass of the current slice
  SliceTask task;
  int k0;
  bool done;
};

template <typename V>
__device__ __forceinline__ void cursor_seek(ChunkCursor& c, const SellView<V>& m, int t, int W,
                                            bool rev) {
  // From pass c.i onward, the first slice with entries.
  while (true) {
    const int64_t idx = warp_slice(c.i, t, W, m.nslices, rev);
    if (idx < 0) {
      c.done = true;
      return;
    }
    c.task = load_task(m.sched, idx);
    c.k0 = 0;
    if (c.task.width > 0) return;
    ++c.i;
  }
}

template <typename V>
__device__ __forceinline__ void cursor_next(ChunkCursor& c, const SellView<V>& m, int t, int W,
                                            bool rev) {
  c.k0 += kBulkCH;
  if (c.k0 < c.task.width) return;
  ++c.i;
  cursor_seek(c, m, t, W, rev);
}

template <typename V>
__device__ __forceinline__ void issue_chunk(const ChunkCursor& c, const SellView<V>& m,
                                            unsigned char* stage, uint64_t* bar) {
  using Cfg = BulkCfg<V>;
  const int nk = min(kBulkCH, c.task.width - c.k0);
  const int64_t first = c.task.base + (int64_t)c.k0 * kSlice;
  const uint32_t cb = (uint32_t)nk * kSlice * 4;
  const uint32_t vb = (uint32_t)nk * kSlice * (uint32_t)sizeof(V);
  mbar_arrive_expect_tx(bar, cb + vb);
  bulk_to_smem(stage, m.cols + first, cb, bar);
  bulk_to_smem(stage + Cfg::kColBytes, m.vals + first, vb, bar);
}

template <typename V, typename A, int EPI, bool DOT, bool UNIT = false>
__global__ void __launch_bounds__(kThreads, 1)
sell_spmv_bulk_kernel(SellView<V> m, const A* x, const A* y, A* z, A alpha, A beta, int flags,
                      const int* guard, EpiDev<A> ep, Reduction red) {
  using Cfg = BulkCfg<V>;
  constexpr int NS = Cfg::NS;
  extern __shared__ __align__(128) unsigned char bulk_smem[];
  const bool run =
      UNIT || (EPI == EPI_TRI_LOWER || EPI == EPI_TRI_UPPER) || !(flags & F_ALPHA_ZERO);
  const bool alpha_one = UNIT || (flags & F_ALPHA_ONE) != 0;
  const bool beta_zero = UNIT || (flags & F_BETA_ZERO) != 0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int W = gridDim.x * (kThreads / 32);
  const int t = warp * gridDim.x + blockIdx.x;
  const bool rev = !DOT && m.reverse;
  unsigned char* ring = bulk_smem + (size_t)warp * Cfg::kWarpBytes;
  uint64_t* bars =
      reinterpret_cast<uint64_t*>(bulk_smem + (size_t)(kThreads / 32) * Cfg::kWarpBytes) + warp * NS;

  // The matrix is not written while a solve runs, so the ring is filled
  // before the wait on the previous kernel (see sell_spmv_pipe_kernel).
  ChunkCursor prod{0, SliceTask{-1, 0, 0}, 0, false};
  uint32_t issued = 0;  // chunks handed to the copy engine (uniform over the warp)
  if (run) {
    if (lane == 0) {
#pragma unroll
      for (int st = 0; st < NS; ++st) mbar_init(bars + st, 1);
      fence_mbar_init();
    }
    __syncwarp();
    cursor_seek(prod, m, t, W, rev);
    for (int st = 0; st < NS && !prod.done; ++st) {
      if (lane == 0) issue_chunk(prod, m, ring + (size_t)st * Cfg::kStage, bars + st);
      cursor_next(prod, m, t, W, rev);
      ++issued;
    }
  }
  pdl_wait();
  pdl_launch_dependents();
  bool off = guard_off(guard);
  double dot_part = 0.0;
  bool failed = false;
  uint32_t q = 0;  // chunks consumed
  // Pending chunk: the chunk whose x gathers went out last step; its values
  // are read from its stage when it is multiplied, and the stage goes back
  // to the copy engine after that.
  A px[kBulkCH];
  int pn = 0;          // its entry count (0: none pending)
  int pst = 0;         // its stage
  bool plast = false;  // it is the last chunk of its slice
  int prow = 0;        // row (of the slice) it belongs to
  A acc = A(0);
  auto multiply_pending = [&]() {
    // Exactly pn multiply-adds, in entry order: pn is the same on every lane,
    // so a slice's short last chunk issues no predicated-off FP64
    // instructions (each would still take an issue slot).
    static_assert(kBulkCH == 4, "the cases below spell out chunks of 4");
    const V* sv = reinterpret_cast<const V*>(ring + (size_t)pst * Cfg::kStage + Cfg::kColBytes) +
                  lane;
    if (pn == 4) {
      acc = fma_t<A>(widen<A, V>(sv[0]), px[0], acc);
      acc = fma_t<A>(widen<A, V>(sv[kSlice]), px[1], acc);
      acc = fma_t<A>(widen<A, V>(sv[2 * kSlice]), px[2], acc);
      acc = fma_t<A>(widen<A, V>(sv[3 * kSlice]), px[3], acc);
    } else if (pn == 3) {
      acc = fma_t<A>(widen<A, V>(sv[0]), px[0], acc);
      acc = fma_t<A>(widen<A, V>(sv[kSlice]), px[1], acc);
      acc = fma_t<A>(widen<A, V>(sv[2 * kSlice]), px[2], acc);
    } else if (pn == 2) {
      acc = fma_t<A>(widen<A, V>(sv[0]), px[0], acc);
      acc = fma_t<A>(widen<A, V>(sv[kSlice]), px[1], acc);
    } else {
      acc = fma_t<A>(widen<A, V>(sv[0]), px[0], acc);
    }
    if (plast) {
      A a1[1] = {acc};
      spmv_finish<1, V, A, EPI, DOT>(m, prow, a1, y, z, alpha, beta, run, alpha_one, beta_zero,
                                     ep, red, dot_part);
      acc = A(0);
    }
    pn = 0;
    // Every lane's reads of the stage precede the refill (the warp barrier
    // is the release / acquire the mbarrier pipelines rely on).
    __syncwarp();
    if (!prod.done) {
      if (lane == 0) issue_chunk(prod, m, ring + (size_t)pst * Cfg::kStage, bars + pst);
      cursor_next(prod, m, t, W, rev);
      ++issued;
    }
  };
  if (!off) {
    for (int i = 0;; ++i) {
      const int64_t idx = warp_slice(i, t, W, m.nslices, rev);
      if (idx < 0) break;
      const SliceTask task = load_task(m.sched, idx);
      const int row = task.s * kSlice + lane;
      if (!run || task.width == 0) {
        if (pn) multiply_pending();
        A a1[1] = {A(0)};
        spmv_finish<1, V, A, EPI, DOT>(m, row, a1, y, z, alpha, beta, run, alpha_one, beta_zero,
                                       ep, red, dot_part);
        continue;
      }
      for (int k0 = 0; k0 < task.width; k0 += kBulkCH, ++q) {
        const int st = (int)(q % NS);
        const uint32_t parity = (q / NS) & 1u;
        uint32_t spins = 0;
        while (!mbar_try_wait(bars + st, parity)) {
          if (++spins == kBulkSpinLimit) {
            failed = true;
            break;
          }
        }
        if (__any_sync(0xffffffffu, failed)) {
          failed = true;
          break;
        }
        const int32_t* sc =
            reinterpret_cast<const int32_t*>(ring + (size_t)st * Cfg::kStage) + lane;
        const int nk = min(kBulkCH, task.width - k0);
        A xv[kBulkCH];
#pragma unroll
        for (int j = 0; j < kBulkCH; ++j) {
          const int c = j < nk ? sc[j * kSlice] : -1;
          xv[j] = c >= 0 ? __ldg(x + c) : A(0);
        }
        if (pn) multiply_pending();
#pragma unroll
        for (int j = 0; j < kBulkCH; ++j) px[j] = xv[j];
        pn = nk;
        pst = st;
        plast = k0 + kBulkCH >= task.width;
        prow = row;
      }
      if (failed) break;
    }
    if (!failed && pn) multiply_pending();
  }
  if (failed || off) {
    // Leave no copy running into this CTA's shared memory: wait (bounded)
    // for every chunk issued and not yet consumed.
    if (failed && lane == 0) atomicExch(m.err, 1);
    if (run) {
      for (uint32_t r = q; r < issued; ++r) {
        const int st = (int)(r % NS);
        uint32_t spins = 0;
        while (!mbar_try_wait(bars + st, (r / NS) & 1u) && ++spins < kBulkSpinLimit) {
        }
      }
    }
    if (off) return;
  }
  if (DOT) reduce_and_finalize(red, dot_part);
}

// Launch configuration of a variant: CTAs resident per SM times SMs, with
// slices spread over the warps by a grid stride.
// Every variant launches the same grid (one 1024-thread CTA per SM at most),
// so the CTA partials of a fused dot product, and therefore its rounding, do
// not depend on which variant the autotuner picked: results are identical
// whatever the timing (and whatever else shares the GPU).
static int spmv_grid(int nslices, int /*minb*/) {
  const int warps_per_cta = kThreads / 32;
  int g = (nslices + warps_per_cta - 1) / warps_per_cta;
  if (g < 1) g = 1;
  if (g > kSms) g = kSms;
  return g;
}

static int spmv_flags(double alpha, double beta) {
  int f = 0;
  if (alpha == 0.0) f |= F_ALPHA_ZERO;
  if (alpha == 1.0) f |= F_ALPHA_ONE;
  if (beta == 0.0) f |= F_BETA_ZERO;
  return f;
}

// Product kernel variants for scalar rows: entries loaded per chunk 8, 16,
// 4, 3 on each of two slices at once, 4 software-pipelined, and 5 streamed
// by the bulk-copy engine; all have a 64-register budget (one 1024-thread
// CTA per SM).  Blocked rows use one variant.
constexpr int kNumVariants = 6;

// Products with alpha == 1 and beta == 0 (all of the Krylov loops') run an
// instantiation that knows it: no scaling or y term is issued (an FP64
// instruction costs its issue slot even with every lane predicated off).
constexpr int kUnitFlags = F_ALPHA_ONE | F_BETA_ZERO;

template <typename V, typename A, int EPI, bool DOT, bool UNIT>
static void launch_bulk(const SellView<V>& view, const void* x, const void* y, void* z,
                        double alpha, double beta, int flags, const int* guard,
                        const EpiDev<A>& e, const Reduction& red, int nslices, cudaStream_t st) {
  auto kern = sell_spmv_bulk_kernel<V, A, EPI, DOT, UNIT>;
  static bool ready = false;  // the opt-in shared memory size, once per instantiation
  if (!ready) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)BulkCfg<V>::kSmem);
    ready = true;
  }
  launch_k(kern, spmv_grid(nslices, 1), kThreads, BulkCfg<V>::kSmem, st, view, (const A*)x,
           (const A*)y, (A*)z, (A)alpha, (A)beta, flags, guard, e, red);
}

template <int B, typename V, typename A, int EPI, bool DOT, int CH, int MINB>
static void launch_one(const SellView<V>& view, const void* x, const void* y, void* z,
                       double alpha, double beta, int flags, const int* guard, const EpiDev<A>& e,
                       const Reduction& red, int nslices, cudaStream_t st) {
  if (flags == kUnitFlags)
    launch_k(sell_spmv_kernel<B, V, A, EPI, DOT, CH, MINB, true>, spmv_grid(nslices, MINB),
             kThreads, 0, st, view, (const A*)x, (const A*)y, (A*)z, (A)alpha, (A)beta, flags,
             guard, e, red);
  else
    launch_k(sell_spmv_kernel<B, V, A, EPI, DOT, CH, MINB>, spmv_grid(nslices, MINB), kThreads, 0,
             st, view, (const A*)x, (const A*)y, (A*)z, (A)alpha, (A)beta, flags, guard, e, red);
}

template <int B, typename V, typename A, int EPI, bool DOT>
static void launch_variant(int variant, const SellView<V>& view, const void* x, const void* y,
                           void* z, double alpha, double beta, int flags, const int* guard,
                           const EpiDev<A>& e, const Reduction& red, int nslices,
                           cudaStream_t st) {
  if constexpr (B == 1) {
    switch (variant) {
      case 1:
        launch_one<B, V, A, EPI, DOT, 16, 1>(view, x, y, z, alpha, beta, flags, guard, e, red,
                                             nslices, st);
        return;
      case 2:
        launch_one<B, V, A, EPI, DOT, 4, 1>(view, x, y, z, alpha, beta, flags, guard, e, red,
                                            nslices, st);
        return;
      case 3:
        if (flags == kUnitFlags)
          launch_k(sell_spmv2_kernel<V, A, EPI, DOT, 3, true>, spmv_grid(nslices, 1), kThreads, 0,
                   st, view, (const A*)x, (const A*)y, (A*)z, (A)alpha, (A)beta, flags, guard, e,
                   red);
        else
          launch_k(sell_spmv2_kernel<V, A, EPI, DOT, 3>, spmv_grid(nslices, 1), kThreads, 0, st,
                   view, (const A*)x, (const A*)y, (A*)z, (A)alpha, (A)beta, flags, guard, e, red);
        return;
      case 4:
        if (flags == kUnitFlags)
          launch_k(sell_spmv_pipe_kernel<V, A, EPI, DOT, 4, true>, spmv_grid(nslices, 1), kThreads,
                   0, st, view, (const A*)x, (const A*)y, (A*)z, (A)alpha, (A)beta, flags, guard, e,
                   red);
        else
          launch_k(sell_spmv_pipe_kernel<V, A, EPI, DOT, 4>, spmv_grid(nslices, 1), kThreads, 0,
                   st, view, (const A*)x, (const A*)y, (A*)z, (A)alpha, (A)beta, flags, guard, e,
                   red);
        return;
      case 5:
        if (flags == kUnitFlags)
          launch_bulk<V, A, EPI, DOT, true>(view, x, y, z, alpha, beta, flags, guard, e, red,
                                            nslices, st);
        else
          launch_bulk<V, A, EPI, DOT, false>(view, x, y, z, alpha, beta, flags, guard, e, red,
                                             nslices, st);
        return;
      default:
        break;
    }
  }
  if constexpr (B == 2 || B == 3) {
    if (variant == 4) {
      constexpr int CH = (B == 2) ? 2 : 1;
      if (flags == kUnitFlags)
        launch_k(sell_spmv_bpipe_kernel<B, V, A, EPI, DOT, CH, true>, spmv_grid(nslices, 1),
                 kThreads, 0, st, view, (const A*)x, (const A*)y, (A*)z, (A)alpha, (A)beta, flags,
                 guard, e, red);
      else
        launch_k(sell_spmv_bpipe_kernel<B, V, A, EPI, DOT, CH>, spmv_grid(nslices, 1), kThreads,
                 0, st, view, (const A*)x, (const A*)y, (A*)z, (A)alpha, (A)beta, flags, guard,
                 e, red);
      return;
    }
  }
  launch_one<B, V, A, EPI, DOT, Chunk<B>::value, 1>(view, x, y, z, alpha, beta, flags, guard, e,
                                                    red, nslices, st);
}

template <int B, typename V, typename A, int EPI>
static void launch_spmv(const Sell& m, const void* x, const void* y, void* z, double alpha,
                        double beta, const int* guard, const EpiHost& ep, const Reduction& red,
                        cudaStream_t st) {
  SellView<V> view{m.nrow, m.nslices, m.slice_ptr.as<int64_t>(), m.cols.as<int32_t>(),
                   m.vals.as<V>(), m.perm.p ? m.perm.as<int32_t>() : nullptr,
                   m.sched.as<int4>(), ep.reverse ? 1 : 0, m.err.as<int>()};
  EpiDev<A> e{(const A*)ep.aux0, (const A*)ep.aux1};
  const int flags = spmv_flags(alpha, beta);
  if (red.w != nullptr)
    launch_variant<B, V, A, EPI, true>(m.variant, view, x, y, z, alpha, beta, flags, guard, e,
                                       red, m.nslices, st);
  else
    launch_variant<B, V, A, EPI, false>(m.variant, view, x, y, z, alpha, beta, flags, guard, e,
                                        red, m.nslices, st);
}

// Epilogue dispatch.  Triangular-sweep epilogues exist only for V == A,
// the factored-operator epilogue only for scalar rows.
template <int B, typename V, typename A>
static int dispatch_epi(const Sell& m, const void* x, const void* y, void* z, double alpha,
                        double beta, const int* guard, const EpiHost& ep, const Reduction& red,
                        cudaStream_t st) {
  switch (ep.kind) {
    case EPI_AXPBY:
      launch_spmv<B, V, A, EPI_AXPBY>(m, x, y, z, alpha, beta, guard, ep, red, st);
      return GBPC_OK;
    case EPI_TRI_LOWER:
    case EPI_TRI_UPPER:
      if constexpr (std::is_same<V, A>::value) {
        if (ep.kind == EPI_TRI_LOWER)
          launch_spmv<B, V, A, EPI_TRI_LOWER>(m, x, y, z, alpha, beta, guard, ep, red, st);
        else
          launch_spmv<B, V, A, EPI_TRI_UPPER>(m, x, y, z, alpha, beta, guard, ep, red, st);
        return GBPC_OK;
      }
      break;
    case EPI_SQLAP_BWD:
      if constexpr (B == 1 && std::is_same<V, A>::value) {
        launch_spmv<1, V, A, EPI_SQLAP_BWD>(m, x, y, z, alpha, beta, guard, ep, red, st);
        return GBPC_OK;
      }
      break;
    case EPI_SQLAP_FWD:
      if constexpr (B == 1 && std::is_same<V, A>::value) {
        launch_spmv<1, V, A, EPI_SQLAP_FWD>(m, x, y, z, alpha, beta, guard, ep, red, st);
        return GBPC_OK;
      }
      break;
    default:
      break;
  }
  gbpc_set_error("unsupported product epilogue %d for this block size / dtype", ep.kind);
  return GBPC_ERR_ARG;
}

// All products whose vectors have type A.
template <typename A>
static int spmv_dispatch(const Sell& m, const void* x, const void* y, void* z, double alpha,
                         double beta, const int* guard, const EpiHost& ep, const Reduction& red,
                         cudaStream_t st) {
  auto by_block = [&](auto vtag) -> int {
    using V = decltype(vtag);
    switch (m.B) {
      case 1: return dispatch_epi<1, V, A>(m, x, y, z, alpha, beta, guard, ep, red, st);
      case 2: return dispatch_epi<2, V, A>(m, x, y, z, alpha, beta, guard, ep, red, st);
      case 3: return dispatch_epi<3, V, A>(m, x, y, z, alpha, beta, guard, ep, red, st);
      case 4: return dispatch_epi<4, V, A>(m, x, y, z, alpha, beta, guard, ep, red, st);
    }
    gbpc_set_error("block size must be 1..4");
    return GBPC_ERR_ARG;
  };
  switch (m.vdtype) {
    case GBPC_F64:
      if constexpr (std::is_same<A, double>::value) return by_block(double{});
      break;
    case GBPC_F32:
      return by_block(float{});
    case GBPC_BF16:
      return by_block(__nv_bfloat16{});
  }
  gbpc_set_error("unsupported storage/vector dtype combination %d/%d", m.vdtype, (int)sizeof(A));
  return GBPC_ERR_ARG;
}

int spmv_f64(const Sell& m, const void* x, const void* y, void* z, double alpha, double beta,
             const int* guard, const EpiHost& ep, const Reduction& red, cudaStream_t st);
int spmv_f32(const Sell& m, const void* x, const void* y, void* z, double alpha, double beta,
             const int* guard, const EpiHost& ep, const Reduction& red, cudaStream_t st);

}  // namespace gbpc
