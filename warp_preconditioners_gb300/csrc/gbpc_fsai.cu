// Adaptive FSAI setup on GB300.
//
// Two builds of the same rows: by rounds (every row's growth steps in
// lock step, a scoring launch and a factor launch per step; the default),
// and one warp per row through all its steps (rows whose candidate table
// overflows in the first, and every row with GBPC_FSAI_ROUNDS=0).
//
// Follows warp_preconditioners/fsai.py:44-176 operation for operation so that
// the selected supports and the factor values are bit-identical to a
// non-contracting evaluation of the reference (this file is compiled with
// -fmad=false; every product and sum is rounded separately, divisions and
// square roots are IEEE-exact).
//
// What differs from the reference is the work distribution, not arithmetic:
//   * candidate scores are accumulated by walking the rows of the current
//     support in support order (q = 0, 1, ...), reading the transposed entry
//     A[c, S_q] through a precomputed transpose position, into a per-warp
//     shared-memory hash table keyed by column.  Each candidate's residual is
//     therefore summed in exactly the reference's order (absent terms are
//     exact zeros and are skipped), but without one binary search per term;
//   * equilibrated entries (a_ij * s_i) * s_j are computed once per nonzero;
//   * the top-`step` selection is a warp-wide arg-max on the IEEE bit pattern
//     of |residual| (non-negative doubles order like their bit patterns), with
//     the reference's tie-break (higher score, then lower column);
//   * the warp-per-row bordered Cholesky forward solve runs column-oriented
//     across lanes, which performs the same subtraction sequence per entry
//     as the reference's row-oriented loop.
// The transpose-position lookup needs a structurally symmetric matrix (any
// SPD input assembled by summation is); other inputs are rejected.

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <vector>

#include "gbpc_common.cuh"
#include "gbpc_internal.h"

namespace gbpc {

namespace {

constexpr int kEmpty = -1;
constexpr int kTomb = -2;

template <typename T> struct Bits;
template <> struct Bits<double> {
  using U = unsigned long long;
  static __device__ __forceinline__ U abs_bits(double v) {
    return (U)__double_as_longlong(v) & 0x7fffffffffffffffull;
  }
  static constexpr U kInf = 0x7ff0000000000000ull;
};
template <> struct Bits<float> {
  using U = unsigned int;
  static __device__ __forceinline__ U abs_bits(float v) { return (U)__float_as_uint(v) & 0x7fffffffu; }
  static constexpr U kInf = 0x7f800000u;
};

__device__ __forceinline__ unsigned int hash_col(int c) { return (unsigned int)c * 2654435761u; }

__device__ __forceinline__ int lower_bound_row(const int32_t* col, int lo, int hi, int j) {
  while (lo < hi) {
    const int mid = (lo + hi) / 2;
    if (col[mid] < j) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// fsai.py:44-57: s_i = 1/sqrt(a_ii) or a counted failure.
template <typename T>
__global__ void fsai_diag_kernel(int n, const int32_t* __restrict__ off,
                                 const int32_t* __restrict__ col, const T* __restrict__ val,
                                 T* scale, int32_t* status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int lo = lower_bound_row(col, off[i], off[i + 1], i);
  T d = T(0);
  if (lo < off[i + 1] && col[lo] == i) d = val[lo];
  if (d > T(0) && isfinite(d)) {
    scale[i] = T(1) / sqrt(d);
  } else {
    scale[i] = T(0);
    atomicAdd(status + 0, 1);
  }
}

// Equilibrated entries and transposed equilibrated entries:
//   ahat[e]  = (a_ij * s_i) * s_j            for e = (i, j)
//   ahatT[e] = (a_ji * s_j) * s_i            (the entry (j, i) seen from row i)
// status[3] counts entries without a stored transpose; status[4] is the
// longest row.
template <typename T>
__global__ void fsai_prep_kernel(int n, const int32_t* __restrict__ off,
                                 const int32_t* __restrict__ col, const T* __restrict__ val,
                                 const T* __restrict__ scale, T* ahat, T* ahatT, int32_t* status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int b = off[i], e_end = off[i + 1];
  atomicMax(status + 4, e_end - b);
  const T si = scale[i];
  int missing = 0;
  for (int e = b; e < e_end; ++e) {
    const int j = col[e];
    const T sj = scale[j];
    const T t = val[e] * si;
    ahat[e] = t * sj;
    const int t_pos = lower_bound_row(col, off[j], off[j + 1], i);
    if (t_pos < off[j + 1] && col[t_pos] == i) {
      const T u = val[t_pos] * sj;
      ahatT[e] = u * si;
    } else {
      ahatT[e] = T(0);
      ++missing;
    }
  }
  if (missing) atomicAdd(status + 3, missing);
}

struct BuildParams {
  int n;
  int width;      // W <= 64
  int step;       // S <= 64
  int hsize;      // candidate table slots (power of 2)
  int hbits;
  int psize;      // pattern table slots (power of 2, >= 2W)
  int pbits;
  const int32_t* rows;   // optional row list (fallback pass)
  int nrows_list;
  int32_t* overflow_list;
  int32_t* overflow_count;
};

// Bytes of one warp's shared-memory slice, rounded to 16 so that every
// warp's floating-point arrays start 16-byte aligned.
template <typename T>
__host__ __device__ constexpr size_t warp_smem_bytes(int W, int S, int H, int PH) {
  return (sizeof(T) * ((size_t)W * (W + 1) / 2 + 4 * (size_t)W + (size_t)H) +
          sizeof(int) * ((size_t)W + 2 * (size_t)PH + (size_t)H + (size_t)S) + 15) &
         ~(size_t)15;
}

__device__ __forceinline__ int plookup(const int* pkey, const int* ppos, int pmask, int pbits, int c) {
  unsigned int s = hash_col(c) >> (32 - pbits);
  for (int probe = 0; probe <= pmask; ++probe) {
    const int k = pkey[s];
    if (k == c) return ppos[s];
    if (k == kEmpty) return -1;
    s = (s + 1) & pmask;
  }
  return -1;
}

__device__ __forceinline__ void pinsert(int* pkey, int* ppos, int pmask, int pbits, int c, int pos) {
  unsigned int s = hash_col(c) >> (32 - pbits);
  for (int probe = 0; probe <= pmask; ++probe) {
    if (pkey[s] == kEmpty) {
      pkey[s] = c;
      ppos[s] = pos;
      return;
    }
    s = (s + 1) & pmask;
  }
}

// Find or insert column c in the candidate table; -1 when the table is full.
__device__ __forceinline__ int hfind_insert(int* hkey, int hmask, int hbits, int c) {
  unsigned int s = hash_col(c) >> (32 - hbits);
  for (int probe = 0; probe <= hmask; ++probe) {
    int k = hkey[s];
    if (k == c) return (int)s;
    if (k == kEmpty) {
      k = atomicCAS(hkey + s, kEmpty, c);
      if (k == kEmpty || k == c) return (int)s;
    }
    s = (s + 1) & hmask;
  }
  return -1;
}

// fsai.py:60-176, one warp per row (see the file comment).
template <typename T>
__global__ void __launch_bounds__(256)
fsai_build_kernel(BuildParams P, const int32_t* __restrict__ off, const int32_t* __restrict__ col,
                  const T* __restrict__ ahat, const T* __restrict__ ahatT,
                  const T* __restrict__ scale, T tolerance, T pivot_floor, int32_t* ell_cols,
                  T* ell_vals, int32_t* row_counts, int32_t* status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  using BitsT = Bits<T>;
  using U = typename BitsT::U;
  const int W = P.width, S = P.step, H = P.hsize, PH = P.psize;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int gw = blockIdx.x * (blockDim.x >> 5) + warp;
  const int total = P.rows ? P.nrows_list : P.n;
  if (gw >= total) return;
  const int i = P.rows ? P.rows[gw] : gw;

  unsigned char* base = smem_raw + (size_t)warp * warp_smem_bytes<T>(W, S, H, PH);
  T* chol = reinterpret_cast<T*>(base);          // column-major packed lower triangle
  T* z = chol + (size_t)W * (W + 1) / 2;
  T* v = z + W;
  T* a = v + W;
  T* wv = a + W;
  T* hacc = wv + W;
  int* pattern = reinterpret_cast<int*>(hacc + H);
  int* pkey = pattern + W;
  int* ppos = pkey + PH;
  int* hkey = ppos + PH;
  int* cand = hkey + H;
  const int hmask = H - 1, pmask = PH - 1;
  // Column p of L starts at cs(p) = p*W - p*(p-1)/2 and holds rows p..W-1.
  auto L = [&](int r, int p) -> T& { return chol[p * W - (p * (p - 1)) / 2 + (r - p)]; };

  for (int s = lane; s < PH; s += 32) pkey[s] = kEmpty;
  for (int s = lane; s < H; s += 32) hkey[s] = kEmpty;
  __syncwarp();
  if (lane == 0) {
    pattern[0] = i;
    pinsert(pkey, ppos, pmask, P.pbits, i, 0);
    L(0, 0) = T(1);
    z[0] = T(1);
    v[0] = T(1);
  }
  __syncwarp();
  int size = 1;
  bool stopped = false;
  bool truncated = false;
  while (size < W) {
    // Candidate residuals, summed in support order.
    for (int s = lane; s < H; s += 32) hacc[s] = T(0);
    __syncwarp();
    bool overflow = false;
    for (int q = 0; q < size; ++q) {
      const int pq = pattern[q];
      const T zq = z[q];
      const int e_end = off[pq + 1];
      for (int e = off[pq] + lane; e < e_end; e += 32) {
        const int c = col[e];
        if (c < i && plookup(pkey, ppos, pmask, P.pbits, c) < 0) {
          const int slot = hfind_insert(hkey, hmask, P.hbits, c);
          if (slot < 0) {
            overflow = true;
          } else {
            const T t = ahatT[e] * zq;
            hacc[slot] = hacc[slot] + t;
          }
        }
      }
      __syncwarp();
    }
    if (__any_sync(0xffffffffu, overflow)) {
      if (lane == 0) {
        const int k = atomicAdd(P.overflow_count, 1);
        P.overflow_list[k] = i;
      }
      return;
    }
    // Top-`step` distinct candidates: higher score, then lower column.
    int nsel = 0;
    for (int r = 0; r < S; ++r) {
      U best_bits = 0;
      int best_col = 0x7fffffff;
      int best_slot = -1;
      for (int s = lane; s < H; s += 32) {
        const int k = hkey[s];
        if (k < 0) continue;
        const U bits = BitsT::abs_bits(hacc[s]);
        if (bits == 0 || bits > BitsT::kInf) continue;  // zero or NaN: never selected
        if (bits > best_bits || (bits == best_bits && k < best_col)) {
          best_bits = bits;
          best_col = k;
          best_slot = s;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const U ob = __shfl_xor_sync(0xffffffffu, best_bits, o);
        const int oc = __shfl_xor_sync(0xffffffffu, best_col, o);
        const int os = __shfl_xor_sync(0xffffffffu, best_slot, o);
        if (ob > best_bits || (ob == best_bits && oc < best_col)) {
          best_bits = ob;
          best_col = oc;
          best_slot = os;
        }
      }
      if (best_slot < 0) break;
      if (lane == 0) {
        cand[r] = best_col;
        hkey[best_slot] = kTomb;
      }
      __syncwarp();
      ++nsel;
    }
    if (nsel == 0) break;
    const T old_z0 = z[0];
    for (int r = 0; r < nsel; ++r) {
      if (size == W) break;
      const int best = cand[r];
      // a[p] = (A[best, S_p] * s_best) * s_{S_p}, zero when not stored.
      for (int p = lane; p < size; p += 32) a[p] = T(0);
      __syncwarp();
      {
        const int e_end = off[best + 1];
        for (int e = off[best] + lane; e < e_end; e += 32) {
          const int pos = plookup(pkey, ppos, pmask, P.pbits, col[e]);
          if (pos >= 0 && pos < size) a[pos] = ahat[e];
        }
      }
      __syncwarp();
      T a0 = (lane < size) ? a[lane] : T(0);
      T a1 = (lane + 32 < size) ? a[lane + 32] : T(0);
      T pivot = T(1);
      T rhs = T(0);
      for (int p = 0; p < size; ++p) {
        const int owner = p & 31;
        T wl = T(0);
        if (lane == owner) wl = ((p < 32) ? a0 : a1) / L(p, p);
        const T wp = __shfl_sync(0xffffffffu, wl, owner);
        if (lane == 0) wv[p] = wp;
        const T sq = wp * wp;
        pivot = pivot - sq;
        const T pr = wp * v[p];
        rhs = rhs - pr;
        if (lane > p && lane < size) {
          const T t = L(lane, p) * wp;
          a0 = a0 - t;
        }
        if (lane + 32 > p && lane + 32 < size) {
          const T t = L(lane + 32, p) * wp;
          a1 = a1 - t;
        }
      }
      __syncwarp();
      if (pivot <= pivot_floor || !isfinite(pivot)) {
        truncated = true;
        stopped = true;
        break;
      }
      for (int p = lane; p < size; p += 32) L(size, p) = wv[p];
      if (lane == 0) {
        pattern[size] = best;
        pinsert(pkey, ppos, pmask, P.pbits, best, size);
        const T d = sqrt(pivot);
        L(size, size) = d;
        v[size] = rhs / d;
      }
      __syncwarp();
      ++size;
    }
    // L^T z = v, in the reference's order.
    if (lane == 0) {
      for (int rev = 0; rev < size; ++rev) {
        const int p = size - 1 - rev;
        T acc = v[p];
        for (int q = p + 1; q < size; ++q) {
          const T t = L(q, p) * z[q];
          acc = acc - t;
        }
        z[p] = acc / L(p, p);
      }
    }
    __syncwarp();
    if (stopped) break;
    if (tolerance > T(0)) {
      const T ratio = old_z0 / z[0];
      if (T(1) - ratio <= tolerance) break;
    }
  }
  // Normalise, validate, sort by column, write the ELL row.
  const T norm = sqrt(z[0]);
  bool valid = true;
  int my_col[2];
  T my_val[2];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int p = lane + 32 * h;
    my_col[h] = -1;
    my_val[h] = T(0);
    if (p < size) {
      const int c = pattern[p];
      const T t = z[p] / norm;
      const T val = t * scale[c];
      my_col[h] = c;
      my_val[h] = val;
      if (!isfinite(val)) valid = false;
      if (p == 0 && !(val > T(0))) valid = false;
    }
  }
  const bool all_valid = __all_sync(0xffffffffu, valid);
  int32_t* oc = ell_cols + (size_t)i * W;
  T* ov = ell_vals + (size_t)i * W;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int p = lane + 32 * h;
    if (p < size) {
      int rank = 0;
      for (int q = 0; q < size; ++q) rank += (pattern[q] < my_col[h]);
      oc[rank] = my_col[h];
      ov[rank] = my_val[h];
    } else if (p < W) {
      oc[p] = -1;
      ov[p] = T(0);
    }
  }
  if (lane == 0) {
    row_counts[i] = size;
    if (truncated) atomicAdd(status + 1, 1);
    if (!all_valid) atomicAdd(status + 2, 1);
  }
}

// ---------------------------------------------------------------------------
// The build by rounds.  A round is one growth step of every row still
// growing, in two launches:
//   * scoring, a warp per row: the row's support goes into a shared-memory
//     hash table (marked with its position), the frontier's residuals are
//     summed in support order as above, the step's candidates are selected,
//     and each candidate's entries against the support (and against the
//     candidates selected before it) are gathered from its own row;
//   * factoring, a thread per row: the bordered Cholesky step for each
//     candidate, then L^T z = v, and the stop tests.
// The row's factor (packed by rows: L(r, p) at r(r+1)/2 + p), v and the
// gathered entries live in device memory as structures of arrays over the
// rows of a chunk, so the threads of a warp read consecutive words; w and z
// live in shared memory, one column per thread.  The scoring tables alone
// set how many warps fit on an SM, and the factor arithmetic, sequential
// within a row, runs 32 rows to a warp.  The bordering's sums are the
// reference's own left-looking loop (row p of L against w); every product
// and sum is the reference's, in its order.  Rows still growing are kept in
// a device list, rebuilt by the factor launch each round, so no round waits
// on the host.

template <typename T>
struct RoundState {
  int nc;           // rows in the chunk
  int r0;           // first row of the chunk
  int W, S;         // width; candidates per round (<= W)
  int H, hbits;     // scoring table slots
  int32_t* size;    // [nc] support size
  int32_t* nsel;    // [nc] candidates selected this round
  int32_t* flags;   // [nc] bit 0: truncated; bit 1: table overflow
  int32_t* pat;     // [nc][W] support in insertion order
  int32_t* lo;      // [nc][W] end of the entries of row pat[p] in columns < the row
  int32_t* cand;    // [nc][S]
  T* z;             // [nc][W]
  T* v;             // [W][nc]
  T* L;             // [W(W+1)/2][nc]
  T* a;             // [S][W][nc]: entries of candidate k against position p
  int32_t* list0;   // rows still growing (chunk-local), two lists used in turn
  int32_t* list1;
  int32_t* count;   // [2] lengths of the lists
};

__host__ __device__ constexpr size_t round_smem_per_warp(int T_size, int H) {
  return ((size_t)H * (T_size + sizeof(int) + sizeof(unsigned short) + 1) + 15) & ~(size_t)15;
}

template <typename T>
__global__ void fsai_round_init_kernel(RoundState<T> R, const int32_t* __restrict__ off,
                                       const int32_t* __restrict__ col) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j == 0) {
    R.count[0] = R.nc;
    R.count[1] = 0;
  }
  if (j >= R.nc) return;
  const int i = R.r0 + j;
  R.size[j] = 1;
  R.nsel[j] = 0;
  R.flags[j] = 0;
  R.pat[(size_t)j * R.W] = i;
  R.lo[(size_t)j * R.W] = lower_bound_row(col, off[i], off[i + 1], i);
  R.z[(size_t)j * R.W] = T(1);
  R.v[j] = T(1);
  R.L[j] = T(1);
  R.list0[j] = j;
}

// Find or insert column c; `fresh` tells whether this call inserted it.
__device__ __forceinline__ int hfind_insert_fresh(int* hkey, int hmask, int hbits, int c,
                                                  bool& fresh) {
  unsigned int s = hash_col(c) >> (32 - hbits);
  fresh = false;
  for (int probe = 0; probe <= hmask; ++probe) {
    int k = hkey[s];
    if (k == c) return (int)s;
    if (k == kEmpty) {
      k = atomicCAS(hkey + s, kEmpty, c);
      if (k == kEmpty) {
        fresh = true;
        return (int)s;
      }
      if (k == c) return (int)s;
    }
    s = (s + 1) & hmask;
  }
  return -1;
}

__device__ __forceinline__ int hfind(const int* hkey, int hmask, int hbits, int c) {
  unsigned int s = hash_col(c) >> (32 - hbits);
  for (int probe = 0; probe <= hmask; ++probe) {
    const int k = hkey[s];
    if (k == c) return (int)s;
    if (k == kEmpty) return -1;
    s = (s + 1) & hmask;
  }
  return -1;
}

// Per-warp scoring table: residuals, columns, the marks below and the list
// of occupied slots (so that selection and clearing visit only those).
template <typename T>
struct ScoreTable {
  T* acc;
  int* key;
  signed char* pos;  // 0 a candidate; p + 1 the support column at position p;
                     // -(k + 1) the k-th candidate selected this round
  unsigned short* used;
  int nused;         // the same in every lane
  int mask, bits;

  // Note slot s, newly taken by the lanes whose `fresh` is set.
  __device__ __forceinline__ void note(bool fresh, int s, int lane) {
    const unsigned m = __ballot_sync(0xffffffffu, fresh);
    if (fresh) used[nused + __popc(m & ((1u << lane) - 1u))] = (unsigned short)s;
    nused += __popc(m);
  }
};

template <typename T>
__global__ void __launch_bounds__(128)
fsai_round_score_kernel(RoundState<T> R, int cur, const int32_t* __restrict__ off,
                        const int32_t* __restrict__ col, const T* __restrict__ ahat,
                        const T* __restrict__ ahatT, int32_t* overflow_list,
                        int32_t* overflow_count) {
  extern __shared__ __align__(16) unsigned char round_smem[];
  using BitsT = Bits<T>;
  using U = typename BitsT::U;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int W = R.W, S = R.S, H = R.H;
  const int64_t nc = R.nc;
  unsigned char* base = round_smem + (size_t)warp * round_smem_per_warp((int)sizeof(T), H);
  ScoreTable<T> tb;
  tb.acc = reinterpret_cast<T*>(base);
  tb.key = reinterpret_cast<int*>(tb.acc + H);
  tb.used = reinterpret_cast<unsigned short*>(tb.key + H);
  tb.pos = reinterpret_cast<signed char*>(tb.used + H);
  tb.nused = 0;
  tb.mask = H - 1;
  tb.bits = R.hbits;
  if (blockIdx.x == 0 && threadIdx.x == 0) R.count[cur ^ 1] = 0;
  const int count = R.count[cur];
  const int32_t* list = cur ? R.list1 : R.list0;
  for (int s = lane; s < H; s += 32) tb.key[s] = kEmpty;
  __syncwarp();
  for (int idx = blockIdx.x * nw + warp; idx < count; idx += gridDim.x * nw) {
    const int j = list[idx];
    const int i = R.r0 + j;
    const int size = R.size[j];
    // The support, its z and its rows' extents, two positions per lane.
    int pc[2], ob[2], oe[2];
    T zv[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int p = lane + 32 * h;
      pc[h] = -1;
      ob[h] = oe[h] = 0;
      zv[h] = T(0);
      if (p < size) {
        pc[h] = R.pat[(size_t)j * W + p];
        zv[h] = R.z[(size_t)j * W + p];
        ob[h] = off[pc[h]];
        oe[h] = R.lo[(size_t)j * W + p];  // rows are sorted: columns < i come first
      }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      bool fresh = false;
      int s = -1;
      if (pc[h] >= 0) {
        s = hfind_insert_fresh(tb.key, tb.mask, tb.bits, pc[h], fresh);
        if (s >= 0) tb.pos[s] = (signed char)(lane + 32 * h + 1);  // H > W: always found
      }
      tb.note(fresh, s, lane);
    }
    __syncwarp();
    // Frontier residuals, summed in support order.  Only the entries of a
    // support row in columns < i can score; the work is a sequence of
    // (support position, 32 of those entries) items, and the next item's
    // entries are loaded before the current one is summed.
    bool overflow = false;
    auto item_row = [&](int q, int& b, int& e, T& zq) {
      const int h = q >> 5, src = q & 31;
      b = __shfl_sync(0xffffffffu, h ? ob[1] : ob[0], src);
      e = __shfl_sync(0xffffffffu, h ? oe[1] : oe[0], src);
      zq = __shfl_sync(0xffffffffu, h ? zv[1] : zv[0], src);
    };
    int q = 0, e0, qe;
    T zq;
    item_row(0, e0, qe, zq);
    int cc = -1;
    T tt = T(0);
    if (e0 + lane < qe) {
      cc = col[e0 + lane];
      tt = ahatT[e0 + lane];
    }
    while (q < size) {
      int nq = q, ne0 = e0 + 32, nqe = qe;
      T nzq = zq;
      if (ne0 >= qe) {
        nq = q + 1;
        if (nq < size) item_row(nq, ne0, nqe, nzq);
      }
      int ncc = -1;
      T ntt = T(0);
      if (nq < size && ne0 + lane < nqe) {
        ncc = col[ne0 + lane];
        ntt = ahatT[ne0 + lane];
      }
      bool fresh = false;
      int s = -1;
      if (cc >= 0) {
        const T t = tt * zq;
        s = hfind_insert_fresh(tb.key, tb.mask, tb.bits, cc, fresh);
        if (s < 0) {
          overflow = true;
        } else if (fresh) {
          tb.pos[s] = 0;
          tb.acc[s] = t;  // 0 + t: the same magnitude, all the score reads
        } else if (tb.pos[s] == 0) {
          tb.acc[s] = tb.acc[s] + t;
        }
      }
      tb.note(fresh, s, lane);
      __syncwarp();
      q = nq;
      e0 = ne0;
      qe = nqe;
      zq = nzq;
      cc = ncc;
      tt = ntt;
    }
    int ns = 0;
    if (__any_sync(0xffffffffu, overflow)) {
      if (lane == 0) {
        R.flags[j] |= 2;
        overflow_list[atomicAdd(overflow_count, 1)] = i;
      }
    } else {
      // Top candidates: higher score, then lower column.
      const int want = min(S, W - size);
      for (int k = 0; k < want; ++k) {
        U best_bits = 0;
        int best_col = 0x7fffffff;
        int best_slot = -1;
        for (int t = lane; t < tb.nused; t += 32) {
          const int s = tb.used[t];
          if (tb.pos[s] != 0) continue;
          const int kk = tb.key[s];
          const U bits = BitsT::abs_bits(tb.acc[s]);
          if (bits == 0 || bits > BitsT::kInf) continue;  // zero or NaN: never selected
          if (bits > best_bits || (bits == best_bits && kk < best_col)) {
            best_bits = bits;
            best_col = kk;
            best_slot = s;
          }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          const U ob2 = __shfl_xor_sync(0xffffffffu, best_bits, o);
          const int oc = __shfl_xor_sync(0xffffffffu, best_col, o);
          const int os = __shfl_xor_sync(0xffffffffu, best_slot, o);
          if (ob2 > best_bits || (ob2 == best_bits && oc < best_col)) {
            best_bits = ob2;
            best_col = oc;
            best_slot = os;
          }
        }
        if (best_slot < 0) break;
        if (lane == 0) {
          tb.pos[best_slot] = (signed char)(-(k + 1));
          R.cand[(size_t)j * S + k] = best_col;
        }
        __syncwarp();
        ++ns;
      }
      // Entries of each candidate against the support and the candidates
      // selected before it; zero where the matrix stores none.
      for (int k = 0; k < ns; ++k)
        for (int p = lane; p < size + k; p += 32) R.a[((size_t)k * W + p) * nc + j] = T(0);
      __syncwarp();
      for (int k = 0; k < ns; ++k) {
        const int best = R.cand[(size_t)j * S + k];
        const int e_beg = off[best], e_end = off[best + 1];
        int below = 0;  // entries of the candidate's row in columns < i
        for (int e0 = e_beg; e0 < e_end; e0 += 32) {
          const int e = e0 + lane;
          const int c = e < e_end ? col[e] : 0x7fffffff;
          below += __popc(__ballot_sync(0xffffffffu, c < i));
          const int s = e < e_end ? hfind(tb.key, tb.mask, tb.bits, c) : -1;
          if (s < 0) continue;
          const int hp = tb.pos[s];
          int pos = -1;
          if (hp > 0) pos = hp - 1;
          else if (hp < 0 && -hp - 1 < k) pos = size + (-hp - 1);
          if (pos >= 0) R.a[((size_t)k * W + pos) * nc + j] = ahat[e];
        }
        if (lane == 0) R.lo[(size_t)j * W + size + k] = e_beg + below;
      }
    }
    if (lane == 0) R.nsel[j] = ns;
    // Empty the slots this row used.
    __syncwarp();
    for (int t = lane; t < tb.nused; t += 32) tb.key[tb.used[t]] = kEmpty;
    tb.nused = 0;
    __syncwarp();
  }
}

template <typename T>
__global__ void __launch_bounds__(128)
fsai_round_factor_kernel(RoundState<T> R, int cur, T tolerance, T pivot_floor) {
  extern __shared__ __align__(16) unsigned char round_fsmem[];
  T* ws = reinterpret_cast<T*>(round_fsmem);  // [W][blockDim.x]: w, then z
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31;
  const int W = R.W, S = R.S;
  const int64_t nc = R.nc;
  const int count = R.count[cur];
  const int32_t* list = cur ? R.list1 : R.list0;
  int32_t* next = cur ? R.list0 : R.list1;
  T* w = ws + tid;
  for (int wbase = blockIdx.x * nt + (tid & ~31); wbase < count; wbase += gridDim.x * nt) {
    const int idx = wbase + lane;
    bool keep = false;
    int j = -1;
    if (idx < count) {
      j = list[idx];
      const int ns = R.nsel[j];
      if (ns > 0) {
        int size = R.size[j];
        T* Lj = R.L + j;
        const T* vj = R.v + j;
        auto L = [&](int r, int p) -> T& { return Lj[((size_t)(r * (r + 1) / 2 + p)) * nc]; };
        const T old_z0 = R.z[(size_t)j * W];
        bool stopped = false;
        for (int k = 0; k < ns; ++k) {
          if (size == W) break;
          const T* ak = R.a + (size_t)k * W * nc + j;
          T pivot = T(1);
          T rhs = T(0);
          for (int p = 0; p < size; ++p) {
            T acc = ak[(size_t)p * nc];
            const T* Lrow = Lj + (size_t)(p * (p + 1) / 2) * nc;  // L(p, q) at Lrow[q nc]
            const T dp = Lrow[(size_t)p * nc];
            int q = 0;
            // Loads in batches of 8 ahead of the (sequential) subtractions.
            for (; q + 8 <= p; q += 8) {
              T l[8];
#pragma unroll
              for (int u = 0; u < 8; ++u) l[u] = Lrow[(size_t)(q + u) * nc];
#pragma unroll
              for (int u = 0; u < 8; ++u) {
                const T t = l[u] * w[(q + u) * nt];
                acc = acc - t;
              }
            }
            for (; q < p; ++q) {
              const T t = Lrow[(size_t)q * nc] * w[q * nt];
              acc = acc - t;
            }
            const T wp = acc / dp;
            w[p * nt] = wp;
            const T sq = wp * wp;
            pivot = pivot - sq;
            const T pr = wp * vj[(size_t)p * nc];
            rhs = rhs - pr;
          }
          if (pivot <= pivot_floor || !isfinite(pivot)) {
            stopped = true;
            break;
          }
          for (int p = 0; p < size; ++p) L(size, p) = w[p * nt];
          R.pat[(size_t)j * W + size] = R.cand[(size_t)j * S + k];
          const T d = sqrt(pivot);
          L(size, size) = d;
          R.v[(size_t)size * nc + j] = rhs / d;
          ++size;
        }
        // L^T z = v, in the reference's order.
        for (int p = size - 1; p >= 0; --p) {
          T acc = vj[(size_t)p * nc];
          const T dp = L(p, p);
          int q = p + 1;
          int k0 = q * (q + 1) / 2 + p;  // packed index of L(q, p)
          for (; q + 8 <= size; q += 8) {
            T l[8];
            int kk = k0;
#pragma unroll
            for (int u = 0; u < 8; ++u) {
              l[u] = Lj[(size_t)kk * nc];
              kk += q + u + 1;
            }
            k0 = kk;
#pragma unroll
            for (int u = 0; u < 8; ++u) {
              const T t = l[u] * w[(q + u) * nt];
              acc = acc - t;
            }
          }
          for (; q < size; ++q) {
            const T t = Lj[(size_t)k0 * nc] * w[q * nt];
            acc = acc - t;
            k0 += q + 1;
          }
          w[p * nt] = acc / dp;
        }
        for (int p = 0; p < size; ++p) R.z[(size_t)j * W + p] = w[p * nt];
        R.size[j] = size;
        if (stopped) {
          R.flags[j] |= 1;
        } else if (tolerance > T(0) && T(1) - old_z0 / w[0] <= tolerance) {
          // converged
        } else {
          keep = size < W;
        }
      }
    }
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    int at = 0;
    if (lane == 0 && m) at = atomicAdd(R.count + (cur ^ 1), __popc(m));
    at = __shfl_sync(0xffffffffu, at, 0);
    if (keep) next[at + __popc(m & ((1u << lane) - 1u))] = j;
  }
}

// Normalise, validate, sort by column and write the ELL rows of a chunk;
// a warp per row.
template <typename T>
__global__ void __launch_bounds__(256)
fsai_round_finish_kernel(RoundState<T> R, const T* __restrict__ scale, int32_t* ell_cols,
                         T* ell_vals, int32_t* row_counts, int32_t* status) {
  const int lane = threadIdx.x & 31;
  const int j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (j >= R.nc) return;
  const int flags = R.flags[j];
  if (flags & 2) return;  // rerun by the warp-per-row kernel
  const int W = R.W, i = R.r0 + j, size = R.size[j];
  const T norm = sqrt(R.z[(size_t)j * W]);
  int my_col[2];
  T my_val[2];
  bool valid = true;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int p = lane + 32 * h;
    my_col[h] = -1;
    my_val[h] = T(0);
    if (p < size) {
      const int c = R.pat[(size_t)j * W + p];
      const T t = R.z[(size_t)j * W + p] / norm;
      const T val = t * scale[c];
      my_col[h] = c;
      my_val[h] = val;
      if (!isfinite(val)) valid = false;
      if (p == 0 && !(val > T(0))) valid = false;
    }
  }
  const bool all_valid = __all_sync(0xffffffffu, valid);
  int rank[2] = {0, 0};
  for (int q = 0; q < size; ++q) {
    const int cq = __shfl_sync(0xffffffffu, q < 32 ? my_col[0] : my_col[1], q & 31);
    rank[0] += (cq < my_col[0]);
    rank[1] += (cq < my_col[1]);
  }
  int32_t* oc = ell_cols + (size_t)i * W;
  T* ov = ell_vals + (size_t)i * W;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int p = lane + 32 * h;
    if (p < size) {
      oc[rank[h]] = my_col[h];
      ov[rank[h]] = my_val[h];
    } else if (p < W) {
      oc[p] = -1;
      ov[p] = T(0);
    }
  }
  if (lane == 0) {
    row_counts[i] = size;
    if (flags & 1) atomicAdd(status + 1, 1);
    if (!all_valid) atomicAdd(status + 2, 1);
  }
}

// ---------------------------------------------------------------------------
// Scans, packing, transpose, scalarise, conversion.

// Exclusive scan of int32 counts into out[0..n] (out[n] = total), 1024 per CTA.
__global__ void scan_block_kernel(const int32_t* in, int32_t* out, int64_t* block_sums, int n) {
  __shared__ int64_t buf[1024];
  const int i = blockIdx.x * 1024 + threadIdx.x;
  const int64_t v = (i < n) ? in[i] : 0;
  buf[threadIdx.x] = v;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    const int64_t t = (threadIdx.x >= o) ? buf[threadIdx.x - o] : 0;
    __syncthreads();
    buf[threadIdx.x] += t;
    __syncthreads();
  }
  if (i < n) out[i] = (int32_t)(buf[threadIdx.x] - v);
  if (threadIdx.x == 1023) block_sums[blockIdx.x] = buf[1023];
}

__global__ void scan_sums_kernel(int64_t* sums, int nb, int32_t* out_total, int n) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int64_t run = 0;
  for (int b = 0; b < nb; ++b) {
    const int64_t t = sums[b];
    sums[b] = run;
    run += t;
  }
  out_total[n] = (int32_t)run;
}

__global__ void scan_add_kernel(int32_t* out, const int64_t* sums, int n) {
  const int i = blockIdx.x * 1024 + threadIdx.x;
  if (i < n) out[i] = (int32_t)(out[i] + sums[blockIdx.x]);
}

}  // namespace

int scan_exclusive_i32(const int32_t* in, int32_t* out, int n, cudaStream_t st) {
  const int nb = (n + 1023) / 1024;
  DevBuf sums;
  int rc = sums.alloc(sizeof(int64_t) * (nb + 1));
  if (rc) return rc;
  if (n > 0) scan_block_kernel<<<nb, 1024, 0, st>>>(in, out, sums.as<int64_t>(), n);
  scan_sums_kernel<<<1, 32, 0, st>>>(sums.as<int64_t>(), nb, out, n);
  if (n > 0) scan_add_kernel<<<nb, 1024, 0, st>>>(out, sums.as<int64_t>(), n);
  GBPC_CUDA_TRY(cudaGetLastError());
  GBPC_CUDA_TRY(cudaStreamSynchronize(st));  // `sums` is released on return
  return GBPC_OK;
}

namespace {

template <typename T>
__global__ void pack_kernel(int n, int width, const int32_t* __restrict__ ell_cols,
                            const T* __restrict__ ell_vals, const int32_t* __restrict__ offsets,
                            int32_t* columns, T* values) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int b = offsets[i], e_end = offsets[i + 1];
  for (int e = b; e < e_end; ++e) {
    const size_t p = (size_t)i * width + (e - b);
    columns[e] = ell_cols[p];
    values[e] = ell_vals[p];
  }
}

__global__ void count_columns_kernel(int nrow, const int32_t* __restrict__ off,
                                     const int32_t* __restrict__ col, int32_t* counts) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrow) return;
  for (int e = off[i]; e < off[i + 1]; ++e) atomicAdd(counts + col[e], 1);
}

template <typename T>
__global__ void scatter_transpose_kernel(int nrow, const int32_t* __restrict__ off,
                                         const int32_t* __restrict__ col, const T* __restrict__ val,
                                         int32_t* cursor, int32_t* t_col, T* t_val) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrow) return;
  for (int e = off[i]; e < off[i + 1]; ++e) {
    const int dst = atomicAdd(cursor + col[e], 1);
    t_col[dst] = i;
    t_val[dst] = val[e];
  }
}

// Insertion sort of each row by column (rows of a transpose are short).
template <typename T>
__global__ void sort_rows_kernel(int nrow, const int32_t* __restrict__ off, int32_t* cols, T* vals) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrow) return;
  const int b = off[r], e_end = off[r + 1];
  for (int e = b + 1; e < e_end; ++e) {
    const int c = cols[e];
    const T v = vals[e];
    int q = e;
    while (q > b && cols[q - 1] > c) {
      cols[q] = cols[q - 1];
      vals[q] = vals[q - 1];
      --q;
    }
    cols[q] = c;
    vals[q] = v;
  }
}

// fsai_pack.py:74-107.
template <typename T>
__global__ void scalarize_kernel(int nrow_blocks, int b, const int32_t* __restrict__ off,
                                 const int32_t* __restrict__ col, const T* __restrict__ val,
                                 int32_t* out_off, int32_t* out_col, T* out_val) {
  const int n = nrow_blocks * b;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int r = i / b, component = i % b;
  const int start = off[r];
  const int count = off[r + 1] - start;
  const int64_t base = (int64_t)start * b * b + (int64_t)component * count * b;
  out_off[i] = (int32_t)base;
  for (int p = 0; p < count; ++p)
    for (int c = 0; c < b; ++c) {
      const int64_t dest = base + (int64_t)p * b + c;
      out_col[dest] = col[start + p] * b + c;
      out_val[dest] = val[((int64_t)start + p) * b * b + (int64_t)component * b + c];
    }
  if (i == n - 1) out_off[i + 1] = (int32_t)(base + (int64_t)count * b);
}

template <typename TI, typename TO>
__device__ __forceinline__ TO narrow(TI v);
template <> __device__ __forceinline__ float narrow<double, float>(double v) { return __double2float_rn(v); }
template <> __device__ __forceinline__ __nv_bfloat16 narrow<double, __nv_bfloat16>(double v) {
  return __float2bfloat16_rn(__double2float_rn(v));
}
template <> __device__ __forceinline__ __nv_bfloat16 narrow<float, __nv_bfloat16>(float v) {
  return __float2bfloat16_rn(v);
}
template <> __device__ __forceinline__ double narrow<double, double>(double v) { return v; }
template <> __device__ __forceinline__ float narrow<float, float>(float v) { return v; }

// fsai.py:181-196: finite values and a positive diagonal after conversion.
template <typename TI, typename TO>
__global__ void convert_factor_kernel(int n, const int32_t* __restrict__ off,
                                      const int32_t* __restrict__ col, const TI* __restrict__ src,
                                      TO* dst, int32_t* invalid) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= n) return;
  bool bad = false;
  for (int e = off[row]; e < off[row + 1]; ++e) {
    const TO v = narrow<TI, TO>(src[e]);
    dst[e] = v;
    const float f = to_float(v);
    if (!isfinite(f)) bad = true;
    if (col[e] == row && !(f > 0.0f)) bad = true;
  }
  if (bad) atomicAdd(invalid, 1);
}

// ---------------------------------------------------------------------------
// Fixed-support numeric refit (fsai_reuse.py:75-149, kernel `refit`), one
// warp per row.
//
// Row i keeps its support S (the sorted columns of G's row i, diagonal
// last).  The scaled local matrix A_S = diag(s) A[S,S] diag(s) is factored
// A_S = L L^T, z = A_S^-1 e_i by a forward and a backward substitution, and
// g_i[S] = z / sqrt(z_i) * s[S].  Every value is formed with the reference's
// operations in the reference's order: the right-looking factorisation
// applies the subtractions of each element in the same k order as the
// reference's row-by-row loop, the forward substitution runs column by
// column across lanes in the same order, and the backward substitution runs
// on one lane because its sums run in increasing column order.  With
// contraction disabled the factor is bit-identical to a sequential
// evaluation of the reference loop.  Pivots <= floor or non-finite are
// replaced by 1 and the row is counted invalid, as in the reference.

constexpr int kRefitWarps = 4;

__device__ __forceinline__ int tri_index(int p, int q) { return p * (p + 1) / 2 + q; }

// (p, q), q <= p, of lower-triangle index t (row-major).
__device__ __forceinline__ void tri_decode(int t, int& p, int& q) {
  p = (int)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
  while (p > 0 && tri_index(p, 0) > t) --p;
  while (tri_index(p + 1, 0) <= t) ++p;
  q = t - tri_index(p, 0);
}

__device__ __forceinline__ bool finite_value(double v) { return isfinite(v); }
__device__ __forceinline__ bool finite_value(float v) { return isfinite(v); }
__device__ __forceinline__ bool finite_value(__nv_bfloat16 v) { return isfinite(__bfloat162float(v)); }
__device__ __forceinline__ bool nonpositive(double v) { return v <= 0.0; }
__device__ __forceinline__ bool nonpositive(float v) { return v <= 0.0f; }
__device__ __forceinline__ bool nonpositive(__nv_bfloat16 v) { return __bfloat162float(v) <= 0.0f; }

template <typename T, typename S>
__global__ void __launch_bounds__(32 * kRefitWarps)
fsai_refit_kernel(int n, const int32_t* __restrict__ a_off, const int32_t* __restrict__ a_col,
                  const T* __restrict__ a_val, const T* __restrict__ scale,
                  const int32_t* __restrict__ g_off, const int32_t* __restrict__ g_col, int width,
                  T floor, S* out, int32_t* bad) {
  extern __shared__ __align__(16) unsigned char refit_smem[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int row = blockIdx.x * kRefitWarps + w;
  const int tri_len = tri_index(width, 0);
  T* tri = reinterpret_cast<T*>(refit_smem) + (size_t)w * (tri_len + width);
  T* z = tri + tri_len;
  if (row >= n) return;
  const int start = g_off[row];
  const int s = g_off[row + 1] - start;
  if (s < 1 || s > width) {
    if (lane == 0) atomicAdd(bad, 1);
    return;
  }
  // Scaled local matrix, lower triangle: (a_rc * s_r) * s_c.
  for (int t = lane; t < tri_index(s, 0); t += 32) {
    int p, q;
    tri_decode(t, p, q);
    const int r = g_col[start + p], c = g_col[start + q];
    const int lo = lower_bound_row(a_col, a_off[r], a_off[r + 1], c);
    T a = T(0);
    if (lo < a_off[r + 1] && a_col[lo] == c) a = a_val[lo] * scale[r] * scale[c];
    tri[t] = a;
  }
  __syncwarp();
  bool valid = true;
  for (int k = 0; k < s; ++k) {
    T d = tri[tri_index(k, k)];
    if (d <= floor || !isfinite(d)) {
      valid = false;
      d = T(1);
    }
    const T ckk = sqrt(d);
    __syncwarp();
    if (lane == 0) tri[tri_index(k, k)] = ckk;
    for (int p = k + 1 + lane; p < s; p += 32) tri[tri_index(p, k)] = tri[tri_index(p, k)] / ckk;
    __syncwarp();
    const int m = s - k - 1;
    for (int t = lane; t < tri_index(m, 0); t += 32) {
      int pp, qq;
      tri_decode(t, pp, qq);
      const int p = k + 1 + pp, q = k + 1 + qq;
      tri[tri_index(p, q)] = tri[tri_index(p, q)] - tri[tri_index(p, k)] * tri[tri_index(q, k)];
    }
    __syncwarp();
  }
  // Forward substitution L y = e_i, column by column (rows lane, lane + 32).
  T a0 = (lane < s && g_col[start + lane] == row) ? T(1) : T(0);
  T a1 = (lane + 32 < s && g_col[start + lane + 32] == row) ? T(1) : T(0);
  for (int q = 0; q < s; ++q) {
    if (q == lane) z[q] = a0 / tri[tri_index(q, q)];
    if (q == lane + 32) z[q] = a1 / tri[tri_index(q, q)];
    __syncwarp();
    const T zq = z[q];
    if (lane > q && lane < s) a0 = a0 - tri[tri_index(lane, q)] * zq;
    if (lane + 32 > q && lane + 32 < s) a1 = a1 - tri[tri_index(lane + 32, q)] * zq;
  }
  __syncwarp();
  // Backward substitution L^T z = y, one lane (sums in increasing q).
  if (lane == 0) {
    for (int p = s - 1; p >= 0; --p) {
      T a = z[p];
      for (int q = p + 1; q < s; ++q) a = a - tri[tri_index(q, p)] * z[q];
      z[p] = a / tri[tri_index(p, p)];
    }
  }
  __syncwarp();
  const T norm = sqrt(z[s - 1]);
  bool ok = true;
  for (int p = lane; p < s; p += 32) {
    const S v = narrow<T, S>(z[p] / norm * scale[g_col[start + p]]);
    out[start + p] = v;
    if (!finite_value(v)) ok = false;
    if (p == s - 1 && nonpositive(v)) ok = false;
  }
  ok = __all_sync(0xffffffffu, ok) && valid;
  if (lane == 0 && !ok) atomicAdd(bad, 1);
}

// The same refit with one thread per row, for supports of at most W entries:
// the reference's loop itself (fsai_reuse.py:97-149), so every lane issues
// useful FP64 work.  On this GPU an FP64 warp instruction costs the same
// however many lanes are active, which makes the warp-per-row version's
// one-lane steps (substitutions, divisions) its bottleneck for small
// supports; wider supports stay with it, because per-thread arrays of
// W(W+1)/2 words would need a large local-memory reservation.
template <typename T, typename S, int W>
__global__ void __launch_bounds__(128)
fsai_refit_row_kernel(int n, const int32_t* __restrict__ a_off, const int32_t* __restrict__ a_col,
                      const T* __restrict__ a_val, const T* __restrict__ scale,
                      const int32_t* __restrict__ g_off, const int32_t* __restrict__ g_col,
                      T floor, S* out, int32_t* bad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int start = g_off[i];
  const int size = g_off[i + 1] - start;
  if (size < 1 || size > W) {
    atomicAdd(bad, 1);
    return;
  }
  T chol[W * (W + 1) / 2];
  T z[W];
  bool valid = true;
  for (int p = 0; p < size; ++p) {
    const int r = g_col[start + p];
    const int rlo = a_off[r], rhi = a_off[r + 1];
    for (int q = 0; q <= p; ++q) {
      const int c = g_col[start + q];
      const int lo = lower_bound_row(a_col, rlo, rhi, c);
      T a = T(0);
      if (lo < rhi && a_col[lo] == c) a = a_val[lo] * scale[r] * scale[c];
      for (int k = 0; k < q; ++k) a = a - chol[tri_index(p, k)] * chol[tri_index(q, k)];
      if (p == q) {
        if (a <= floor || !isfinite(a)) {
          valid = false;
          a = T(1);
        }
        chol[tri_index(p, p)] = sqrt(a);
      } else {
        chol[tri_index(p, q)] = a / chol[tri_index(q, q)];
      }
    }
  }
  for (int p = 0; p < size; ++p) {
    T a = (g_col[start + p] == i) ? T(1) : T(0);
    for (int q = 0; q < p; ++q) a = a - chol[tri_index(p, q)] * z[q];
    z[p] = a / chol[tri_index(p, p)];
  }
  for (int p = size - 1; p >= 0; --p) {
    T a = z[p];
    for (int q = p + 1; q < size; ++q) a = a - chol[tri_index(q, p)] * z[q];
    z[p] = a / chol[tri_index(p, p)];
  }
  const T norm = sqrt(z[size - 1]);
  for (int p = 0; p < size; ++p) {
    const S v = narrow<T, S>(z[p] / norm * scale[g_col[start + p]]);
    out[start + p] = v;
    if (!finite_value(v)) valid = false;
    if (p == size - 1 && nonpositive(v)) valid = false;
  }
  if (!valid) atomicAdd(bad, 1);
}

// The same refit for wider supports, one thread per row: the local factor
// lives in device memory as a structure of arrays over the rows of a chunk
// (L(p, q) of the k-th row at L[(p(p+1)/2 + q) stride + k], so the threads
// of a warp read consecutive words) and z in shared memory.  Rows are taken
// in order of support size (`order`), so the threads of a warp run loops of
// the same length.  A[r, S] is gathered by merging the sorted row r with the
// sorted support.  Operations and their order are the reference's.
template <typename T, typename S>
__global__ void __launch_bounds__(128)
fsai_refit_wide_kernel(int count, const int32_t* __restrict__ order, int64_t stride, T* L,
                       const int32_t* __restrict__ a_off, const int32_t* __restrict__ a_col,
                       const T* __restrict__ a_val, const T* __restrict__ scale,
                       const int32_t* __restrict__ g_off, const int32_t* __restrict__ g_col,
                       int W, T floor, S* out, int32_t* bad) {
  extern __shared__ __align__(16) unsigned char refit_wide_smem[];
  T* z = reinterpret_cast<T*>(refit_wide_smem) + threadIdx.x;  // z[p] at z[p * blockDim.x]
  const int nt = blockDim.x;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const int i = order[k];
  const int start = g_off[i];
  const int size = g_off[i + 1] - start;
  if (size < 1 || size > W) {
    atomicAdd(bad, 1);
    return;
  }
  T* Lk = L + k;
  auto at = [&](int p, int q) -> T& { return Lk[(size_t)(p * (p + 1) / 2 + q) * stride]; };
  bool valid = true;
  for (int p = 0; p < size; ++p) {
    const int r = g_col[start + p];
    const T sr = scale[r];
    int e = a_off[r];
    const int rhi = a_off[r + 1];
    const T* Lp = Lk + (size_t)(p * (p + 1) / 2) * stride;  // row p: Lp[q stride]
    for (int q = 0; q <= p; ++q) {
      const int c = g_col[start + q];
      while (e < rhi && a_col[e] < c) ++e;
      T a = T(0);
      if (e < rhi && a_col[e] == c) a = a_val[e] * sr * scale[c];
      const T* Lq = Lk + (size_t)(q * (q + 1) / 2) * stride;
      int t = 0;
      for (; t + 8 <= q; t += 8) {
        T x[8], y[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          x[u] = Lp[(size_t)(t + u) * stride];
          y[u] = Lq[(size_t)(t + u) * stride];
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) a = a - x[u] * y[u];
      }
      for (; t < q; ++t) a = a - Lp[(size_t)t * stride] * Lq[(size_t)t * stride];
      if (p == q) {
        if (a <= floor || !isfinite(a)) {
          valid = false;
          a = T(1);
        }
        at(p, p) = sqrt(a);
      } else {
        at(p, q) = a / Lq[(size_t)q * stride];
      }
    }
  }
  for (int p = 0; p < size; ++p) {
    T a = (g_col[start + p] == i) ? T(1) : T(0);
    const T* Lp = Lk + (size_t)(p * (p + 1) / 2) * stride;
    for (int q = 0; q < p; ++q) a = a - Lp[(size_t)q * stride] * z[q * nt];
    z[p * nt] = a / Lp[(size_t)p * stride];
  }
  for (int p = size - 1; p >= 0; --p) {
    T a = z[p * nt];
    int kk = (p + 1) * (p + 2) / 2 + p;  // packed index of L(p + 1, p)
    for (int q = p + 1; q < size; ++q) {
      a = a - Lk[(size_t)kk * stride] * z[q * nt];
      kk += q + 1;
    }
    z[p * nt] = a / at(p, p);
  }
  const T norm = sqrt(z[(size - 1) * nt]);
  for (int p = 0; p < size; ++p) {
    const S v = narrow<T, S>(z[p * nt] / norm * scale[g_col[start + p]]);
    out[start + p] = v;
    if (!finite_value(v)) valid = false;
    if (p == size - 1 && nonpositive(v)) valid = false;
  }
  if (!valid) atomicAdd(bad, 1);
}

// Rows ordered by support size (counting sort; the order within a size is
// immaterial, every row is computed on its own).
__global__ void support_size_count_kernel(int n, const int32_t* __restrict__ g_off, int W,
                                          int32_t* bins) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int s = min(max(g_off[i + 1] - g_off[i], 0), W);
  atomicAdd(bins + s, 1);
}

__global__ void support_size_scan_kernel(int W, int32_t* bins) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int acc = 0;
  for (int s = 0; s <= W; ++s) {
    const int c = bins[s];
    bins[s] = acc;
    acc += c;
  }
}

__global__ void support_size_scatter_kernel(int n, const int32_t* __restrict__ g_off, int W,
                                            int32_t* cursor, int32_t* order) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int s = min(max(g_off[i + 1] - g_off[i], 0), W);
  order[atomicAdd(cursor + s, 1)] = i;
}

// map[e] = position of entry (i, j) of a CSR matrix in its transpose's row j.
__global__ void transpose_map_kernel(int nrow, const int32_t* __restrict__ off,
                                     const int32_t* __restrict__ col,
                                     const int32_t* __restrict__ t_off,
                                     const int32_t* __restrict__ t_col, int32_t* map,
                                     int32_t* missing) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrow) return;
  for (int e = off[i]; e < off[i + 1]; ++e) {
    const int j = col[e];
    const int pos = lower_bound_row(t_col, t_off[j], t_off[j + 1], i);
    if (pos < t_off[j + 1] && t_col[pos] == i) {
      map[e] = pos;
    } else {
      map[e] = -1;
      atomicAdd(missing, 1);
    }
  }
}

template <typename V>
__global__ void scatter_values_kernel(int64_t count, const V* __restrict__ src,
                                      const int32_t* __restrict__ map, V* dst) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < count;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int32_t m = map[e];
    if (m >= 0) dst[m] = src[e];
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// Host entry points.

// GBPC_FSAI_CHUNK_ROWS=m caps the rows whose device state the build by
// rounds and the wide refit hold at once (read on every call; the tests use
// it to run several chunks on small matrices).
static int64_t chunk_rows_limit() {
  const char* e = std::getenv("GBPC_FSAI_CHUNK_ROWS");
  const long long v = e ? std::atoll(e) : 0;
  return v >= 32 ? (int64_t)v : INT64_MAX;
}

// GBPC_FSAI_ROUNDS=0 selects the warp-per-row build for every row (the two
// builds give identical factors; the switch exists to compare them).
static bool rounds_build_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("GBPC_FSAI_ROUNDS");
    return !(e && e[0] == '0');
  }();
  return on;
}

template <typename T>
static int fsai_setup_t(int n, const int32_t* off, const int32_t* col, const T* val, int W,
                        int S, double kap, double floor_, int32_t* ell_cols, T* ell_vals,
                        int32_t* counts, T* scale, int32_t* status_host, cudaStream_t st) {
  int64_t nnz = 0;
  {
    int32_t last = 0;
    GBPC_CUDA_TRY(cudaMemcpyAsync(&last, off + n, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    GBPC_CUDA_TRY(cudaStreamSynchronize(st));
    nnz = last;
  }
  DevBuf ahat, ahatT, status, ovl;
  int rc;
  if ((rc = ahat.alloc(sizeof(T) * std::max<int64_t>(nnz, 1)))) return rc;
  if ((rc = ahatT.alloc(sizeof(T) * std::max<int64_t>(nnz, 1)))) return rc;
  if ((rc = status.alloc(sizeof(int32_t) * 8))) return rc;
  if ((rc = ovl.alloc(sizeof(int32_t) * std::max(n, 1)))) return rc;
  GBPC_CUDA_TRY(cudaMemsetAsync(status.p, 0, sizeof(int32_t) * 8, st));
  int32_t* stat = status.as<int32_t>();
  if (n > 0) {
    fsai_diag_kernel<T><<<grid_for(n, 256), 256, 0, st>>>(n, off, col, val, scale, stat);
    fsai_prep_kernel<T><<<grid_for(n, 256), 256, 0, st>>>(n, off, col, val, scale, ahat.as<T>(),
                                                          ahatT.as<T>(), stat);
  }
  GBPC_CUDA_TRY(cudaGetLastError());
  int32_t h[8];
  GBPC_CUDA_TRY(cudaMemcpyAsync(h, stat, sizeof(h), cudaMemcpyDeviceToHost, st));
  GBPC_CUDA_TRY(cudaStreamSynchronize(st));
  if (h[3] != 0) {
    gbpc_set_error("FSAI setup requires a structurally symmetric matrix (%d entries lack a "
                   "stored transpose)", h[3]);
    return GBPC_ERR_UNSUPPORTED;
  }
  const int maxrow = std::max(h[4], 1);
  int PH = 1, pbits = 0;
  while (PH < 2 * W) { PH <<= 1; ++pbits; }
  if (pbits == 0) { PH = 2; pbits = 1; }
  // Distinct candidates never exceed W * maxrow; a table larger than that
  // cannot overflow.  First pass uses a smaller table for occupancy.
  int64_t bound = (int64_t)W * maxrow + 1;
  int Hfull = 32, hbits_full = 5;
  while (Hfull < bound) { Hfull <<= 1; ++hbits_full; }
  int Hfirst = Hfull, hbits_first = hbits_full;
  const int Hcap = (W <= 16) ? 512 : 1024;
  while (Hfirst > Hcap) { Hfirst >>= 1; --hbits_first; }

  int smem_optin = 0, dev = 0;
  GBPC_CUDA_TRY(cudaGetDevice(&dev));
  GBPC_CUDA_TRY(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));

  auto launch = [&](int H, int hbits, const int32_t* rows, int nrows) -> int {
    const size_t per_warp = warp_smem_bytes<T>(W, S, H, PH);
    if (per_warp > (size_t)smem_optin) {
      gbpc_set_error("FSAI setup: rows too long for shared memory (%zu bytes per warp)", per_warp);
      return GBPC_ERR_UNSUPPORTED;
    }
    int warps = (int)std::min<size_t>(8, std::max<size_t>(1, (100 * 1024) / per_warp));
    while ((size_t)warps * per_warp > (size_t)smem_optin) --warps;
    const size_t smem = (size_t)warps * per_warp;
    GBPC_CUDA_TRY(cudaFuncSetAttribute(fsai_build_kernel<T>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    BuildParams P;
    P.n = n;
    P.width = W;
    P.step = S;
    P.hsize = H;
    P.hbits = hbits;
    P.psize = PH;
    P.pbits = pbits;
    P.rows = rows;
    P.nrows_list = nrows;
    P.overflow_list = ovl.as<int32_t>();
    P.overflow_count = stat + 5;
    const int items = rows ? nrows : n;
    if (items > 0)
      fsai_build_kernel<T><<<grid_for(items, warps), warps * 32, smem, st>>>(
          P, off, col, ahat.as<T>(), ahatT.as<T>(), scale, (T)kap, (T)floor_, ell_cols, ell_vals,
          counts, stat);
    GBPC_CUDA_TRY(cudaGetLastError());
    return GBPC_OK;
  };
  // First pass: the build by rounds (see fsai_round_score_kernel).
  auto launch_rounds = [&](int H, int hbits) -> int {
    const int SE = std::min(S, W);
    const size_t per_warp = round_smem_per_warp((int)sizeof(T), H);
    const int wpc = 4;
    const size_t score_smem = per_warp * wpc;
    const int ft = 128;
    const size_t factor_smem = sizeof(T) * (size_t)W * ft;
    if (score_smem > (size_t)smem_optin || factor_smem > (size_t)smem_optin) return -1;
    // Device state per row of a chunk: the factor, v, z, the gathered
    // entries, the support and its rows' ends, the candidates and five
    // counters.
    const size_t per_row = sizeof(T) * ((size_t)W * (W + 1) / 2 + 2 * (size_t)W + (size_t)SE * W) +
                           sizeof(int32_t) * (2 * (size_t)W + SE + 5);
    // One chunk when the state fits in a quarter of the free memory (8 GB
    // at most): the last rounds, when few rows still grow, are latency
    // bound, and each chunk pays them once.
    size_t free_b = 0, total_b = 0;
    GBPC_CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    const size_t budget = std::min<size_t>(free_b / 4, (size_t)8 << 30);
    const int64_t cap = std::max<int64_t>(4096, (int64_t)(budget / per_row));
    const int nc = (int)std::min<int64_t>(n, std::min<int64_t>(cap, chunk_rows_limit()));
    DevBuf b_size, b_nsel, b_flags, b_pat, b_lo, b_cand, b_z, b_v, b_L, b_a, b_l0, b_l1, b_count;
    if ((rc = b_size.alloc(sizeof(int32_t) * nc)) || (rc = b_nsel.alloc(sizeof(int32_t) * nc)) ||
        (rc = b_flags.alloc(sizeof(int32_t) * nc)) ||
        (rc = b_pat.alloc(sizeof(int32_t) * (size_t)nc * W)) ||
        (rc = b_lo.alloc(sizeof(int32_t) * (size_t)nc * W)) ||
        (rc = b_cand.alloc(sizeof(int32_t) * (size_t)nc * SE)) ||
        (rc = b_z.alloc(sizeof(T) * (size_t)nc * W)) || (rc = b_v.alloc(sizeof(T) * (size_t)nc * W)) ||
        (rc = b_L.alloc(sizeof(T) * (size_t)nc * W * (W + 1) / 2)) ||
        (rc = b_a.alloc(sizeof(T) * (size_t)nc * W * SE)) ||
        (rc = b_l0.alloc(sizeof(int32_t) * nc)) || (rc = b_l1.alloc(sizeof(int32_t) * nc)) ||
        (rc = b_count.alloc(sizeof(int32_t) * 2)))
      return rc;
    RoundState<T> R;
    R.W = W;
    R.S = SE;
    R.H = H;
    R.hbits = hbits;
    R.size = b_size.as<int32_t>();
    R.nsel = b_nsel.as<int32_t>();
    R.flags = b_flags.as<int32_t>();
    R.pat = b_pat.as<int32_t>();
    R.lo = b_lo.as<int32_t>();
    R.cand = b_cand.as<int32_t>();
    R.z = b_z.as<T>();
    R.v = b_v.as<T>();
    R.L = b_L.as<T>();
    R.a = b_a.as<T>();
    R.list0 = b_l0.as<int32_t>();
    R.list1 = b_l1.as<int32_t>();
    R.count = b_count.as<int32_t>();
    GBPC_CUDA_TRY(cudaFuncSetAttribute(fsai_round_score_kernel<T>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)score_smem));
    GBPC_CUDA_TRY(cudaFuncSetAttribute(fsai_round_factor_kernel<T>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)factor_smem));
    int sms = 0, occ_s = 0, occ_f = 0;
    GBPC_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    GBPC_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &occ_s, fsai_round_score_kernel<T>, 32 * wpc, score_smem));
    GBPC_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &occ_f, fsai_round_factor_kernel<T>, ft, factor_smem));
    const int grid_s = sms * std::max(occ_s, 1), grid_f = sms * std::max(occ_f, 1);
    for (int r0 = 0; r0 < n; r0 += nc) {
      R.r0 = r0;
      R.nc = std::min(nc, n - r0);
      fsai_round_init_kernel<T><<<grid_for(R.nc, 256), 256, 0, st>>>(R, off, col);
      // Every round adds an entry to each row still growing, or ends it.
      for (int round = 0; round < W - 1; ++round) {
        const int cur = round & 1;
        fsai_round_score_kernel<T><<<grid_s, 32 * wpc, score_smem, st>>>(
            R, cur, off, col, ahat.as<T>(), ahatT.as<T>(), ovl.as<int32_t>(), stat + 5);
        fsai_round_factor_kernel<T><<<grid_f, ft, factor_smem, st>>>(R, cur, (T)kap, (T)floor_);
      }
      fsai_round_finish_kernel<T><<<grid_for(R.nc, 8), 256, 0, st>>>(R, scale, ell_cols, ell_vals,
                                                                     counts, stat);
      GBPC_CUDA_TRY(cudaGetLastError());
    }
    return GBPC_OK;
  };
  int rr = -1;
  // The scoring tables of the build by rounds: 512 slots unless the
  // longest row makes fewer enough.  (A tet-mesh biharmonic row at width 48
  // meets ~170 distinct columns, 330 at most; rows that find more rerun
  // below with a table that cannot overflow.)
  int Hr = Hfull, hbits_r = hbits_full;
  while (Hr > 512) { Hr >>= 1; --hbits_r; }
  if (rounds_build_enabled() && (rr = launch_rounds(Hr, hbits_r)) > 0) return rr;
  if (rr != 0 && (rc = launch(Hfirst, hbits_first, nullptr, n))) return rc;
  GBPC_CUDA_TRY(cudaMemcpyAsync(h, stat, sizeof(h), cudaMemcpyDeviceToHost, st));
  GBPC_CUDA_TRY(cudaStreamSynchronize(st));
  if (h[5] > 0) {
    // Rows whose frontier overflowed the first table: rerun them exactly
    // with a table that cannot overflow.
    const int nover = h[5];
    DevBuf list;
    if ((rc = list.alloc(sizeof(int32_t) * nover))) return rc;
    GBPC_CUDA_TRY(cudaMemcpyAsync(list.p, ovl.p, sizeof(int32_t) * nover, cudaMemcpyDeviceToDevice, st));
    GBPC_CUDA_TRY(cudaMemsetAsync(stat + 5, 0, sizeof(int32_t), st));
    if ((rc = launch(Hfull, hbits_full, list.as<int32_t>(), nover))) return rc;
    GBPC_CUDA_TRY(cudaMemcpyAsync(h, stat, sizeof(h), cudaMemcpyDeviceToHost, st));
    GBPC_CUDA_TRY(cudaStreamSynchronize(st));
    if (h[5] > 0) {
      gbpc_set_error("FSAI setup: candidate table overflow");
      return GBPC_ERR_UNSUPPORTED;
    }
  }
  if (status_host) {
    status_host[0] = h[0];
    status_host[1] = h[1];
    status_host[2] = h[2];
  }
  if (h[0]) {
    gbpc_set_error("FSAI requires finite positive diagonals (%d invalid rows)", h[0]);
    return GBPC_ERR_DIAGONAL;
  }
  if (h[2]) {
    gbpc_set_error("FSAI factor lost finite entries or a positive diagonal");
    return GBPC_ERR_FACTOR;
  }
  return GBPC_OK;
}

}  // namespace gbpc

using namespace gbpc;

extern "C" int gbpc_fsai_setup(int n, const int32_t* offsets, const int32_t* columns,
                               const void* values, int dtype, int width, int step,
                               double kap_tolerance, double pivot_floor, int32_t* ell_cols,
                               void* ell_vals, int32_t* row_counts, void* scale,
                               int32_t* status_host, void* stream) {
  NvtxRange nvtx_range("gbpc_fsai_setup");
  if (n < 0 || !offsets || (n > 0 && (!columns || !values || !ell_cols || !ell_vals ||
                                      !row_counts || !scale))) {
    gbpc_set_error("gbpc_fsai_setup: null or negative argument");
    return GBPC_ERR_ARG;
  }
  if (width < 1 || width > 64) {
    gbpc_set_error("max_row_size must be an integer in [1, 64]");
    return GBPC_ERR_ARG;
  }
  if (step < 1 || step > 64) {
    gbpc_set_error("max_step_size must be an integer in [1, 64]");
    return GBPC_ERR_ARG;
  }
  if (!(kap_tolerance >= 0.0 && kap_tolerance < 1.0)) {
    gbpc_set_error("kap_tolerance must be in [0, 1)");
    return GBPC_ERR_ARG;
  }
  if (!(pivot_floor > 0.0 && pivot_floor < 1.0)) {
    gbpc_set_error("pivot_floor must be in (0, 1)");
    return GBPC_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == GBPC_F64)
    return fsai_setup_t<double>(n, offsets, columns, (const double*)values, width, step,
                                kap_tolerance, pivot_floor, ell_cols, (double*)ell_vals,
                                row_counts, (double*)scale, status_host, st);
  if (dtype == GBPC_F32)
    return fsai_setup_t<float>(n, offsets, columns, (const float*)values, width, step,
                               kap_tolerance, pivot_floor, ell_cols, (float*)ell_vals,
                               row_counts, (float*)scale, status_host, st);
  gbpc_set_error("FSAI supports float32 and float64 matrices");
  return GBPC_ERR_ARG;
}

extern "C" int gbpc_fsai_pack(int n, int width, const int32_t* ell_cols, const void* ell_vals,
                              const int32_t* row_counts, int dtype, int32_t* offsets_out,
                              int32_t* columns_out, void* values_out, int64_t* nnz_host,
                              void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  if (n < 0 || !offsets_out || (n > 0 && !row_counts)) {
    gbpc_set_error("gbpc_fsai_pack: bad arguments");
    return GBPC_ERR_ARG;
  }
  if (columns_out == nullptr) {
    int rc = scan_exclusive_i32(row_counts, offsets_out, n, st);
    if (rc) return rc;
    int32_t total = 0;
    GBPC_CUDA_TRY(cudaMemcpyAsync(&total, offsets_out + n, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    GBPC_CUDA_TRY(cudaStreamSynchronize(st));
    if (nnz_host) *nnz_host = total;
    return GBPC_OK;
  }
  if (n == 0) return GBPC_OK;
  if (dtype == GBPC_F64)
    pack_kernel<double><<<grid_for(n, 256), 256, 0, st>>>(n, width, ell_cols, (const double*)ell_vals,
                                                         offsets_out, columns_out, (double*)values_out);
  else if (dtype == GBPC_F32)
    pack_kernel<float><<<grid_for(n, 256), 256, 0, st>>>(n, width, ell_cols, (const float*)ell_vals,
                                                        offsets_out, columns_out, (float*)values_out);
  else {
    gbpc_set_error("gbpc_fsai_pack: dtype must be float64 or float32");
    return GBPC_ERR_ARG;
  }
  GBPC_CUDA_TRY(cudaGetLastError());
  return GBPC_OK;
}

template <typename T>
static int transpose_t(int nrow, int ncol, const int32_t* off, const int32_t* col, const T* val,
                       int32_t* t_off, int32_t* t_col, T* t_val, cudaStream_t st) {
  DevBuf counts, cursor;
  int rc;
  if ((rc = counts.alloc(sizeof(int32_t) * (ncol + 1)))) return rc;
  if ((rc = cursor.alloc(sizeof(int32_t) * (ncol + 1)))) return rc;
  GBPC_CUDA_TRY(cudaMemsetAsync(counts.p, 0, sizeof(int32_t) * (ncol + 1), st));
  if (nrow > 0) count_columns_kernel<<<grid_for(nrow, 256), 256, 0, st>>>(nrow, off, col, counts.as<int32_t>());
  GBPC_CUDA_TRY(cudaGetLastError());
  if ((rc = scan_exclusive_i32(counts.as<int32_t>(), t_off, ncol, st))) return rc;
  GBPC_CUDA_TRY(cudaMemcpyAsync(cursor.p, t_off, sizeof(int32_t) * (ncol + 1), cudaMemcpyDeviceToDevice, st));
  if (nrow > 0)
    scatter_transpose_kernel<T><<<grid_for(nrow, 256), 256, 0, st>>>(nrow, off, col, val,
                                                                    cursor.as<int32_t>(), t_col, t_val);
  if (ncol > 0) sort_rows_kernel<T><<<grid_for(ncol, 256), 256, 0, st>>>(ncol, t_off, t_col, t_val);
  GBPC_CUDA_TRY(cudaGetLastError());
  GBPC_CUDA_TRY(cudaStreamSynchronize(st));
  return GBPC_OK;
}

extern "C" int gbpc_csr_transpose(int nrow, int ncol, const int32_t* offsets,
                                  const int32_t* columns, const void* values, int dtype,
                                  int32_t* t_off, int32_t* t_col, void* t_val, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  if (nrow < 0 || ncol < 0 || !offsets || !t_off) {
    gbpc_set_error("gbpc_csr_transpose: bad arguments");
    return GBPC_ERR_ARG;
  }
  switch (dtype) {
    case GBPC_F64:
      return transpose_t<double>(nrow, ncol, offsets, columns, (const double*)values, t_off, t_col,
                                 (double*)t_val, st);
    case GBPC_F32:
      return transpose_t<float>(nrow, ncol, offsets, columns, (const float*)values, t_off, t_col,
                                (float*)t_val, st);
    case GBPC_BF16:
      return transpose_t<__nv_bfloat16>(nrow, ncol, offsets, columns, (const __nv_bfloat16*)values,
                                        t_off, t_col, (__nv_bfloat16*)t_val, st);
  }
  gbpc_set_error("gbpc_csr_transpose: bad dtype");
  return GBPC_ERR_ARG;
}

extern "C" int gbpc_scalarize(int nrow_blocks, int b, const int32_t* offsets,
                              const int32_t* columns, const void* values, int dtype,
                              int32_t* out_off, int32_t* out_col, void* out_val, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  if (nrow_blocks < 0 || b < 1 || b > 8 || !offsets || !out_off) {
    gbpc_set_error("gbpc_scalarize: bad arguments");
    return GBPC_ERR_ARG;
  }
  const int n = nrow_blocks * b;
  if (n == 0) {
    GBPC_CUDA_TRY(cudaMemsetAsync(out_off, 0, sizeof(int32_t), st));
    return GBPC_OK;
  }
  if (dtype == GBPC_F64)
    scalarize_kernel<double><<<grid_for(n, 256), 256, 0, st>>>(nrow_blocks, b, offsets, columns,
                                                              (const double*)values, out_off,
                                                              out_col, (double*)out_val);
  else if (dtype == GBPC_F32)
    scalarize_kernel<float><<<grid_for(n, 256), 256, 0, st>>>(nrow_blocks, b, offsets, columns,
                                                             (const float*)values, out_off, out_col,
                                                             (float*)out_val);
  else {
    gbpc_set_error("gbpc_scalarize: dtype must be float64 or float32");
    return GBPC_ERR_ARG;
  }
  GBPC_CUDA_TRY(cudaGetLastError());
  return GBPC_OK;
}

extern "C" int gbpc_convert_factor(int n, const int32_t* offsets, const int32_t* columns,
                                   const void* src, int src_dtype, void* dst, int dst_dtype,
                                   int32_t* invalid_host, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  DevBuf bad;
  int rc;
  if ((rc = bad.alloc(sizeof(int32_t)))) return rc;
  GBPC_CUDA_TRY(cudaMemsetAsync(bad.p, 0, sizeof(int32_t), st));
  if (n > 0) {
    const int g = grid_for(n, 256);
    if (src_dtype == GBPC_F64 && dst_dtype == GBPC_F32)
      convert_factor_kernel<double, float><<<g, 256, 0, st>>>(n, offsets, columns, (const double*)src,
                                                             (float*)dst, bad.as<int32_t>());
    else if (src_dtype == GBPC_F64 && dst_dtype == GBPC_BF16)
      convert_factor_kernel<double, __nv_bfloat16><<<g, 256, 0, st>>>(
          n, offsets, columns, (const double*)src, (__nv_bfloat16*)dst, bad.as<int32_t>());
    else if (src_dtype == GBPC_F32 && dst_dtype == GBPC_BF16)
      convert_factor_kernel<float, __nv_bfloat16><<<g, 256, 0, st>>>(
          n, offsets, columns, (const float*)src, (__nv_bfloat16*)dst, bad.as<int32_t>());
    else if (src_dtype == dst_dtype && src_dtype == GBPC_F64)
      convert_factor_kernel<double, double><<<g, 256, 0, st>>>(n, offsets, columns, (const double*)src,
                                                              (double*)dst, bad.as<int32_t>());
    else if (src_dtype == dst_dtype && src_dtype == GBPC_F32)
      convert_factor_kernel<float, float><<<g, 256, 0, st>>>(n, offsets, columns, (const float*)src,
                                                            (float*)dst, bad.as<int32_t>());
    else {
      gbpc_set_error("gbpc_convert_factor: unsupported conversion %d -> %d", src_dtype, dst_dtype);
      return GBPC_ERR_ARG;
    }
  }
  GBPC_CUDA_TRY(cudaGetLastError());
  int32_t h = 0;
  GBPC_CUDA_TRY(cudaMemcpyAsync(&h, bad.p, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  GBPC_CUDA_TRY(cudaStreamSynchronize(st));
  if (invalid_host) *invalid_host = h;
  if (h) {
    gbpc_set_error("factor_dtype conversion lost finite entries or a positive diagonal");
    return GBPC_ERR_CONVERSION;
  }
  return GBPC_OK;
}


// ---------------------------------------------------------------------------
// Fixed-support refit entry points (fsai_reuse.py:157-245).

namespace gbpc {
// GBPC_FSAI_REFIT_WIDE=0 keeps supports wider than 16 on the warp-per-row
// refit (the two give identical values; the switch exists to compare them).
static bool refit_wide_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("GBPC_FSAI_REFIT_WIDE");
    return !(e && e[0] == '0');
  }();
  return on;
}

template <typename T, typename S>
static int refit_t(int n, const int32_t* a_off, const int32_t* a_col, const T* a_val,
                   const int32_t* g_off, const int32_t* g_col, int width, double floor_, S* out,
                   int32_t* status_host, cudaStream_t st) {
  DevBuf scale, status;
  int rc;
  if ((rc = scale.alloc(sizeof(T) * std::max(n, 1)))) return rc;
  if ((rc = status.alloc(sizeof(int32_t) * 2))) return rc;
  GBPC_CUDA_TRY(cudaMemsetAsync(status.p, 0, sizeof(int32_t) * 2, st));
  int32_t* stat = status.as<int32_t>();
  if (n > 0) {
    fsai_diag_kernel<T><<<grid_for(n, 256), 256, 0, st>>>(n, a_off, a_col, a_val, scale.as<T>(),
                                                          stat);
    if (width <= 8) {
      fsai_refit_row_kernel<T, S, 8><<<grid_for(n, 128), 128, 0, st>>>(
          n, a_off, a_col, a_val, scale.as<T>(), g_off, g_col, (T)floor_, out, stat + 1);
    } else if (width <= 16) {
      fsai_refit_row_kernel<T, S, 16><<<grid_for(n, 128), 128, 0, st>>>(
          n, a_off, a_col, a_val, scale.as<T>(), g_off, g_col, (T)floor_, out, stat + 1);
    } else if (refit_wide_enabled()) {
      // Thread per row, rows in order of support size, the local factors of
      // a chunk of rows in device memory (a quarter of the free memory, 8 GB
      // at most).
      const int ft = 128;
      const size_t tri = (size_t)width * (width + 1) / 2;
      size_t free_b = 0, total_b = 0;
      GBPC_CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
      const size_t budget = std::min<size_t>(free_b / 4, (size_t)8 << 30);
      const int nc = (int)std::min<int64_t>(
          n, std::min<int64_t>(std::max<int64_t>(4096, (int64_t)(budget / (sizeof(T) * tri))),
                               chunk_rows_limit()));
      DevBuf bins, order, lbuf;
      if ((rc = bins.alloc(sizeof(int32_t) * (width + 1))) ||
          (rc = order.alloc(sizeof(int32_t) * n)) || (rc = lbuf.alloc(sizeof(T) * tri * nc)))
        return rc;
      GBPC_CUDA_TRY(cudaMemsetAsync(bins.p, 0, sizeof(int32_t) * (width + 1), st));
      support_size_count_kernel<<<grid_for(n, 256), 256, 0, st>>>(n, g_off, width,
                                                                  bins.as<int32_t>());
      support_size_scan_kernel<<<1, 32, 0, st>>>(width, bins.as<int32_t>());
      support_size_scatter_kernel<<<grid_for(n, 256), 256, 0, st>>>(
          n, g_off, width, bins.as<int32_t>(), order.as<int32_t>());
      const size_t smem = sizeof(T) * (size_t)width * ft;
      GBPC_CUDA_TRY(cudaFuncSetAttribute(fsai_refit_wide_kernel<T, S>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      for (int k0 = 0; k0 < n; k0 += nc) {
        const int cnt = std::min(nc, n - k0);
        fsai_refit_wide_kernel<T, S><<<grid_for(cnt, ft), ft, smem, st>>>(
            cnt, order.as<int32_t>() + k0, (int64_t)cnt, lbuf.as<T>(), a_off, a_col, a_val,
            scale.as<T>(), g_off, g_col, width, (T)floor_, out, stat + 1);
      }
    } else {
      const size_t smem = sizeof(T) * (size_t)(width * (width + 1) / 2 + width) * kRefitWarps;
      GBPC_CUDA_TRY(cudaFuncSetAttribute(fsai_refit_kernel<T, S>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      fsai_refit_kernel<T, S><<<(n + kRefitWarps - 1) / kRefitWarps, 32 * kRefitWarps, smem,
                                st>>>(n, a_off, a_col, a_val, scale.as<T>(), g_off, g_col, width,
                                      (T)floor_, out, stat + 1);
    }
  }
  GBPC_CUDA_TRY(cudaGetLastError());
  GBPC_CUDA_TRY(cudaMemcpyAsync(status_host, stat, sizeof(int32_t) * 2, cudaMemcpyDeviceToHost, st));
  GBPC_CUDA_TRY(cudaStreamSynchronize(st));
  return GBPC_OK;
}
}  // namespace gbpc

extern "C" int gbpc_fsai_refit(int n, const int32_t* a_off, const int32_t* a_col,
                               const void* a_val, int dtype, const int32_t* g_off,
                               const int32_t* g_col, int width, double pivot_floor, void* out,
                               int factor_dtype, int32_t* status_host, void* stream) {
  NvtxRange nvtx_range("gbpc_fsai_refit");
  if (n < 0 || width < 1 || width > 64 || !status_host ||
      (n > 0 && (!a_off || !a_col || !a_val || !g_off || !g_col || !out)) ||
      !(pivot_floor > 0.0 && pivot_floor < 1.0)) {
    gbpc_set_error("gbpc_fsai_refit: bad arguments");
    return GBPC_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == GBPC_F64) {
    if (factor_dtype == GBPC_F64)
      return refit_t<double, double>(n, a_off, a_col, (const double*)a_val, g_off, g_col, width,
                                     pivot_floor, (double*)out, status_host, st);
    if (factor_dtype == GBPC_F32)
      return refit_t<double, float>(n, a_off, a_col, (const double*)a_val, g_off, g_col, width,
                                    pivot_floor, (float*)out, status_host, st);
    if (factor_dtype == GBPC_BF16)
      return refit_t<double, __nv_bfloat16>(n, a_off, a_col, (const double*)a_val, g_off, g_col,
                                            width, pivot_floor, (__nv_bfloat16*)out, status_host,
                                            st);
  } else if (dtype == GBPC_F32) {
    if (factor_dtype == GBPC_F32)
      return refit_t<float, float>(n, a_off, a_col, (const float*)a_val, g_off, g_col, width,
                                   pivot_floor, (float*)out, status_host, st);
    if (factor_dtype == GBPC_BF16)
      return refit_t<float, __nv_bfloat16>(n, a_off, a_col, (const float*)a_val, g_off, g_col,
                                           width, pivot_floor, (__nv_bfloat16*)out, status_host,
                                           st);
  }
  gbpc_set_error("gbpc_fsai_refit: unsupported matrix / factor dtype pair (%d, %d)", dtype,
                 factor_dtype);
  return GBPC_ERR_ARG;
}

extern "C" int gbpc_transpose_map(int nrow, const int32_t* offsets, const int32_t* columns,
                                  const int32_t* t_offsets, const int32_t* t_columns,
                                  int32_t* map_out, void* stream) {
  if (nrow < 0 || (nrow > 0 && (!offsets || !columns || !t_offsets || !t_columns || !map_out))) {
    gbpc_set_error("gbpc_transpose_map: bad arguments");
    return GBPC_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  DevBuf missing;
  int rc = missing.alloc(sizeof(int32_t));
  if (rc) return rc;
  GBPC_CUDA_TRY(cudaMemsetAsync(missing.p, 0, sizeof(int32_t), st));
  if (nrow > 0)
    transpose_map_kernel<<<grid_for(nrow, 256), 256, 0, st>>>(nrow, offsets, columns, t_offsets,
                                                              t_columns, map_out,
                                                              missing.as<int32_t>());
  GBPC_CUDA_TRY(cudaGetLastError());
  int32_t h = 0;
  GBPC_CUDA_TRY(cudaMemcpyAsync(&h, missing.p, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  GBPC_CUDA_TRY(cudaStreamSynchronize(st));
  if (h) {
    gbpc_set_error("gbpc_transpose_map: %d entries have no transposed counterpart", h);
    return GBPC_ERR_ARG;
  }
  return GBPC_OK;
}

extern "C" int gbpc_scatter_values(int64_t count, const void* src, const int32_t* map, void* dst,
                                   int dtype, void* stream) {
  if (count < 0 || (count > 0 && (!src || !map || !dst)) || !valid_value_dtype(dtype)) {
    gbpc_set_error("gbpc_scatter_values: bad arguments");
    return GBPC_ERR_ARG;
  }
  if (count == 0) return GBPC_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const int g = (int)std::min<int64_t>((count + 255) / 256, 152 * 8);
  if (dtype == GBPC_F64)
    scatter_values_kernel<double><<<g, 256, 0, st>>>(count, (const double*)src, map, (double*)dst);
  else if (dtype == GBPC_F32)
    scatter_values_kernel<float><<<g, 256, 0, st>>>(count, (const float*)src, map, (float*)dst);
  else
    scatter_values_kernel<__nv_bfloat16><<<g, 256, 0, st>>>(count, (const __nv_bfloat16*)src, map,
                                                            (__nv_bfloat16*)dst);
  GBPC_CUDA_TRY(cudaGetLastError());
  return GBPC_OK;
}
