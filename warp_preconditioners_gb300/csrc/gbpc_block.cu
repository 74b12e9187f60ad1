// Block preconditioner setup kernels: block Jacobi inverses, synchronous
// block ILU(0) sweeps, block-row adaptive FSAI, plus BSR format helpers.
//
// warp_preconditioners/block_ilu.py:17-210 and
// benchmarks/block_fsai_candidate.py:22-178, restated per block row / per
// stored block.  Setup only: the apply side of these preconditioners runs
// through the SELL product (gbpc_sell.cu).

#include <algorithm>

#include "gbpc_common.cuh"
#include "gbpc_internal.h"

namespace gbpc {

int scan_exclusive_i32(const int32_t* in, int32_t* out, int n, cudaStream_t st);

namespace {

template <typename T>
__device__ T det_n(const T* a, int b) {
  if (b == 1) return a[0];
  if (b == 2) return a[0] * a[3] - a[1] * a[2];
  if (b == 3)
    return a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) +
           a[2] * (a[3] * a[7] - a[4] * a[6]);
  T total = T(0);
  for (int c = 0; c < 4; ++c) {
    T m[9];
    int k = 0;
    for (int r = 1; r < 4; ++r)
      for (int cc = 0; cc < 4; ++cc)
        if (cc != c) m[k++] = a[r * 4 + cc];
    const T cof = m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
                  m[2] * (m[3] * m[7] - m[4] * m[6]);
    total = (c % 2 == 0) ? total + a[c] * cof : total - a[c] * cof;
  }
  return total;
}

template <typename T>
__device__ T minor_det(const T* a, int b, int skip_r, int skip_c) {
  T m[9];
  int k = 0;
  for (int rr = 0; rr < b; ++rr)
    for (int cc = 0; cc < b; ++cc)
      if (rr != skip_r && cc != skip_c) m[k++] = a[rr * b + cc];
  return det_n(m, b - 1);
}

// block_ilu.py:17-43: max-abs scaling, determinant threshold, adjugate inverse.
template <typename T>
__device__ int safe_inverse(const T* a, int b, T tolerance, T* inverse) {
  int bad = 0;
  T scale = T(0);
  for (int k = 0; k < b * b; ++k) scale = fmax(scale, fabs(a[k]));
  for (int k = 0; k < b * b; ++k) inverse[k] = T(0);
  if (scale > T(0) && isfinite(scale)) {
    T normalized[16];
    for (int k = 0; k < b * b; ++k) normalized[k] = a[k] / scale;
    const T det = det_n(normalized, b);
    if (isfinite(det) && fabs(det) > tolerance) {
      if (b == 1) {
        inverse[0] = T(1) / a[0];
      } else {
        for (int r = 0; r < b; ++r)
          for (int c = 0; c < b; ++c) {
            const T mnr = minor_det(normalized, b, c, r);
            inverse[r * b + c] = ((((r + c) & 1) ? -mnr : mnr) / det) / scale;
          }
      }
    } else {
      bad = 1;
    }
  } else {
    bad = 1;
  }
  for (int k = 0; k < b * b; ++k)
    if (!isfinite(inverse[k])) bad += 1;
  return bad;
}

// block_ilu.py:76-104 (`diagonal_only`).
template <typename T>
__global__ void block_diag_inverse_kernel(int nrow, int b, const int32_t* __restrict__ off,
                                          const int32_t* __restrict__ col, const T* __restrict__ val,
                                          T tolerance, T* inverse, int32_t* bad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrow) return;
  int lo = off[i], hi = off[i + 1];
  const int end = hi;
  while (lo < hi) {
    const int mid = (lo + hi) / 2;
    if (col[mid] < i) lo = mid + 1; else hi = mid;
  }
  int nb;
  T inv[16];
  if (lo < end && col[lo] == i) {
    nb = safe_inverse(val + (size_t)lo * b * b, b, tolerance, inv);
  } else {
    nb = 1;
    for (int k = 0; k < b * b; ++k) inv[k] = T(0);
  }
  for (int k = 0; k < b * b; ++k) inverse[(size_t)i * b * b + k] = inv[k];
  if (nb) atomicAdd(bad, nb);
}

// block_ilu.py:46-61 (`topology`).
__global__ void topology_kernel(int nrow, const int32_t* __restrict__ off,
                                const int32_t* __restrict__ col, int32_t* rows, int32_t* diag,
                                int32_t* bad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrow) return;
  int found = -1;
  for (int e = off[i]; e < off[i + 1]; ++e) {
    rows[e] = i;
    if (col[e] == i) found = e;
  }
  diag[i] = found;
  if (found < 0) atomicAdd(bad, 1);
}

// block_ilu.py:63-73 (`invert`).
template <typename T>
__global__ void invert_kernel(int nrow, int b, const T* __restrict__ values,
                              const int32_t* __restrict__ diag, T* inverse, T tolerance,
                              int32_t* bad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrow || diag[i] < 0) return;
  T inv[16];
  const int nb = safe_inverse(values + (size_t)diag[i] * b * b, b, tolerance, inv);
  for (int k = 0; k < b * b; ++k) inverse[(size_t)i * b * b + k] = inv[k];
  if (nb) atomicAdd(bad, nb);
}

template <typename T>
__device__ __forceinline__ void matmul_n(const T* a, const T* m, int b, T* out) {
  for (int r = 0; r < b; ++r)
    for (int c = 0; c < b; ++c) {
      T s = T(0);
      for (int k = 0; k < b; ++k) s = s + a[r * b + k] * m[k * b + c];
      out[r * b + c] = s;
    }
}

// block_ilu.py:106-118 (`initialize`).
template <typename T>
__global__ void initialize_kernel(int64_t nnz, int b, const int32_t* __restrict__ rows,
                                  const int32_t* __restrict__ col, const T* __restrict__ val,
                                  const T* __restrict__ inverse, T* factors) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nnz) return;
  const int bb = b * b;
  if (col[e] < rows[e]) {
    matmul_n(val + e * bb, inverse + (size_t)col[e] * bb, b, factors + e * bb);
  } else {
    for (int q = 0; q < bb; ++q) factors[e * bb + q] = val[e * bb + q];
  }
}

// block_ilu.py:120-150 (`sweep`): one synchronous ILU(0) update of every
// stored block from the previous sweep's factors.
template <typename T>
__global__ void sweep_kernel(int64_t nnz, int b, const int32_t* __restrict__ off,
                             const int32_t* __restrict__ col, const int32_t* __restrict__ rows,
                             const T* __restrict__ val, const T* __restrict__ old,
                             const T* __restrict__ inverse, T* out, T relaxation) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nnz) return;
  const int bb = b * b;
  const int i = rows[e], j = col[e];
  T value[16], prod[16];
  for (int q = 0; q < bb; ++q) value[q] = val[e * bb + q];
  const int kmax = min(i, j);
  for (int ik = off[i]; ik < off[i + 1]; ++ik) {
    const int k = col[ik];
    if (k >= kmax) break;
    int lo = off[k], hi = off[k + 1];
    while (lo < hi) {
      const int mid = (lo + hi) / 2;
      if (col[mid] < j) lo = mid + 1; else hi = mid;
    }
    if (lo < off[k + 1] && col[lo] == j) {
      matmul_n(old + (size_t)ik * bb, old + (size_t)lo * bb, b, prod);
      for (int q = 0; q < bb; ++q) value[q] = value[q] - prod[q];
    }
  }
  if (j < i) {
    matmul_n(value, inverse + (size_t)j * bb, b, prod);
    for (int q = 0; q < bb; ++q) value[q] = prod[q];
  }
  for (int q = 0; q < bb; ++q)
    out[e * bb + q] = (T(1) - relaxation) * old[e * bb + q] + relaxation * value[q];
}

template <typename T>
__global__ void validate_kernel(int64_t count, const T* __restrict__ values, int32_t* bad) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  if (!isfinite(values[k])) atomicAdd(bad, 1);
}

// benchmarks/block_fsai_candidate.py:22-43 (`entry`).
template <typename T>
__device__ __forceinline__ T block_entry(const int32_t* off, const int32_t* col, const T* val,
                                         int b, int i, int j) {
  int lo = off[i / b], hi = off[i / b + 1];
  const int end = hi;
  while (lo < hi) {
    const int mid = (lo + hi) / 2;
    if (col[mid] < j / b) lo = mid + 1; else hi = mid;
  }
  T result = T(0);
  if (lo < end && col[lo] == j / b) result = val[(size_t)lo * b * b + (i % b) * b + (j % b)];
  return result;
}

// benchmarks/block_fsai_candidate.py:45-59 (`diagonal`).
template <typename T>
__global__ void block_fsai_diag_kernel(int n, int b, const int32_t* __restrict__ off,
                                       const int32_t* __restrict__ col, const T* __restrict__ val,
                                       T* scale, int32_t* status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const T d = block_entry(off, col, val, b, i, i);
  if (d > T(0) && isfinite(d)) {
    scale[i] = T(1) / sqrt(d);
  } else {
    atomicAdd(status, 1);
    scale[i] = T(0);
  }
}

// benchmarks/block_fsai_candidate.py:61-176 (`build`), one thread per block
// row with the local system in thread-private memory (width <= 16), then the
// rows of the block sorted by column (fsai_pack.py:15-39) with counts.
constexpr int kBfMaxWidth = 16;
template <typename T>
__global__ void block_fsai_build_kernel(int nrow, int b, int max_blocks,
                                        const int32_t* __restrict__ off,
                                        const int32_t* __restrict__ col, const T* __restrict__ val,
                                        const T* __restrict__ scale, int32_t* cols, T* vals,
                                        int32_t* counts, int32_t* status, int refit) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrow) return;
  const int width = b * max_blocks;
  int pattern[4];
  T chol[kBfMaxWidth * kBfMaxWidth];
  T z[kBfMaxWidth * 4];
  for (int p = 0; p < 4; ++p) pattern[p] = -1;
  pattern[0] = i;
  int size = 1;
  if (refit) {
    for (int p = 0; p < max_blocks; ++p) {
      const int c = cols[((size_t)i * b) * width + p * b];
      if (c >= 0 && c / b != i) pattern[size++] = c / b;
    }
  }
  for (int k = 0; k < kBfMaxWidth * 4; ++k) z[k] = T(0);
  int bad = 0;
  for (int stepi = 0; stepi < max_blocks; ++stepi) {
    for (int k = 0; k < kBfMaxWidth * kBfMaxWidth; ++k) chol[k] = T(0);
    const int count = size * b;
    for (int p = 0; p < count; ++p) {
      const int r = pattern[p / b] * b + p % b;
      for (int q = 0; q <= p; ++q) {
        const int c = pattern[q / b] * b + q % b;
        T v = (block_entry(off, col, val, b, r, c) * scale[r]) * scale[c];
        for (int k = 0; k < q; ++k) v = v - chol[p * kBfMaxWidth + k] * chol[q * kBfMaxWidth + k];
        if (p == q) {
          if (v <= T(0) || !isfinite(v)) {
            ++bad;
            v = T(1);
          }
          chol[p * kBfMaxWidth + q] = sqrt(v);
        } else {
          chol[p * kBfMaxWidth + q] = v / chol[q * kBfMaxWidth + q];
        }
      }
    }
    for (int c = 0; c < b; ++c) {
      for (int p = 0; p < count; ++p) {
        T v = (p == c) ? T(1) : T(0);
        for (int q = 0; q < p; ++q) v = v - chol[p * kBfMaxWidth + q] * z[q * 4 + c];
        z[p * 4 + c] = v / chol[p * kBfMaxWidth + p];
      }
      for (int rev = 0; rev < count; ++rev) {
        const int p = count - rev - 1;
        T v = z[p * 4 + c];
        for (int q = p + 1; q < count; ++q) v = v - chol[q * kBfMaxWidth + p] * z[q * 4 + c];
        z[p * 4 + c] = v / chol[p * kBfMaxWidth + p];
      }
    }
    if (refit || stepi == max_blocks - 1) break;
    int best = -1;
    T best_score = T(0);
    for (int p = 0; p < size; ++p) {
      const int row = pattern[p];
      for (int e = off[row]; e < off[row + 1]; ++e) {
        const int candidate = col[e];
        bool selected = candidate >= i;
        for (int q = 0; q < size; ++q)
          if (pattern[q] == candidate) selected = true;
        if (selected) continue;
        T score = T(0);
        for (int r = 0; r < b; ++r) {
          const int cr = candidate * b + r;
          for (int c = 0; c < b; ++c) {
            T residual = T(0);
            for (int q = 0; q < count; ++q) {
              const int j = pattern[q / b] * b + q % b;
              residual = residual +
                         ((block_entry(off, col, val, b, cr, j) * scale[cr]) * scale[j]) * z[q * 4 + c];
            }
            score = score + residual * residual;
          }
        }
        if (score > best_score || (score == best_score && candidate < best)) {
          best = candidate;
          best_score = score;
        }
      }
    }
    if (best < 0 || best_score == T(0)) break;
    pattern[size++] = best;
  }
  // Block-row normalisation G = chol(Z_ii)^-1 Z^T D^-1/2.
  T norm[16];
  for (int k = 0; k < 16; ++k) norm[k] = T(0);
  for (int r = 0; r < b; ++r)
    for (int c = 0; c <= r; ++c) {
      T v = z[r * 4 + c];
      for (int k = 0; k < c; ++k) v = v - norm[r * 4 + k] * norm[c * 4 + k];
      if (r == c) norm[r * 4 + c] = sqrt(v);
      else norm[r * 4 + c] = v / norm[c * 4 + c];
    }
  for (int q = 0; q < size * b; ++q)
    for (int r = 0; r < b; ++r) {
      T v = z[q * 4 + r];
      for (int k = 0; k < r; ++k) v = v - norm[r * 4 + k] * z[q * 4 + k];
      z[q * 4 + r] = v / norm[r * 4 + r];
    }
  // Emit each scalar row sorted by column: blocks in ascending block column.
  int order[4];
  for (int p = 0; p < size; ++p) order[p] = p;
  for (int p = 1; p < size; ++p) {
    const int t = order[p];
    int q = p;
    while (q > 0 && pattern[order[q - 1]] > pattern[t]) {
      order[q] = order[q - 1];
      --q;
    }
    order[q] = t;
  }
  for (int r = 0; r < b; ++r) {
    const size_t rowbase = ((size_t)i * b + r) * width;
    int k = 0;
    for (int p = 0; p < size; ++p) {
      const int blk = order[p];
      for (int c = 0; c < b; ++c) {
        const int qq = blk * b + c;
        const int j = pattern[blk] * b + c;
        cols[rowbase + k] = j;
        vals[rowbase + k] = z[qq * 4 + r] * scale[j];
        ++k;
      }
    }
    for (; k < width; ++k) {
      cols[rowbase + k] = -1;
      vals[rowbase + k] = T(0);
    }
    counts[(size_t)i * b + r] = size * b;
  }
  if (bad) atomicAdd(status, bad);
}

// Scalar CSR (b rows per block row, each row sorted) -> b x b BSR.
// Phase 0 counts distinct block columns per block row; phase 1 fills.
template <typename T>
__global__ void csr_to_bsr_kernel(int nrow_blocks, int b, const int32_t* __restrict__ off,
                                  const int32_t* __restrict__ col, const T* __restrict__ val,
                                  int phase, int32_t* counts, const int32_t* __restrict__ boff,
                                  int32_t* bcol, T* bval) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= nrow_blocks) return;
  int cursor[8];
  for (int r = 0; r < b; ++r) cursor[r] = off[I * b + r];
  int nblk = 0;
  const int bb = b * b;
  while (true) {
    int next = 0x7fffffff;
    for (int r = 0; r < b; ++r)
      if (cursor[r] < off[I * b + r + 1]) next = min(next, col[cursor[r]] / b);
    if (next == 0x7fffffff) break;
    if (phase == 1) {
      const int dst = boff[I] + nblk;
      bcol[dst] = next;
      for (int q = 0; q < bb; ++q) bval[(size_t)dst * bb + q] = T(0);
      for (int r = 0; r < b; ++r)
        while (cursor[r] < off[I * b + r + 1] && col[cursor[r]] / b == next) {
          bval[(size_t)dst * bb + r * b + col[cursor[r]] % b] = val[cursor[r]];
          ++cursor[r];
        }
    } else {
      for (int r = 0; r < b; ++r)
        while (cursor[r] < off[I * b + r + 1] && col[cursor[r]] / b == next) ++cursor[r];
    }
    ++nblk;
  }
  if (phase == 0) counts[I] = nblk;
}

__global__ void count_block_columns_kernel(int nrow, const int32_t* __restrict__ off,
                                           const int32_t* __restrict__ col, int32_t* counts) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrow) return;
  for (int e = off[i]; e < off[i + 1]; ++e) atomicAdd(counts + col[e], 1);
}

// Block transpose: block (J, I) of the result is the transpose of block (I, J).
template <typename T>
__global__ void bsr_scatter_transpose_kernel(int nrow, int b, const int32_t* __restrict__ off,
                                             const int32_t* __restrict__ col,
                                             const T* __restrict__ val, int32_t* cursor,
                                             int32_t* t_col, T* t_val) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrow) return;
  const int bb = b * b;
  for (int e = off[i]; e < off[i + 1]; ++e) {
    const int dst = atomicAdd(cursor + col[e], 1);
    t_col[dst] = i;
    for (int r = 0; r < b; ++r)
      for (int c = 0; c < b; ++c) t_val[(size_t)dst * bb + c * b + r] = val[(size_t)e * bb + r * b + c];
  }
}

template <typename T>
__global__ void bsr_sort_rows_kernel(int nrow, int b, const int32_t* __restrict__ off, int32_t* cols,
                                     T* vals) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrow) return;
  const int bb = b * b;
  const int s = off[r], e_end = off[r + 1];
  for (int e = s + 1; e < e_end; ++e) {
    const int c = cols[e];
    T v[16];
    for (int q = 0; q < bb; ++q) v[q] = vals[(size_t)e * bb + q];
    int q = e;
    while (q > s && cols[q - 1] > c) {
      cols[q] = cols[q - 1];
      for (int k = 0; k < bb; ++k) vals[(size_t)q * bb + k] = vals[(size_t)(q - 1) * bb + k];
      --q;
    }
    cols[q] = c;
    for (int k = 0; k < bb; ++k) vals[(size_t)q * bb + k] = v[k];
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// Host helpers used by the operator constructors (gbpc_ops.cu).

int block_diag_inverse(int nrow, int b, const int32_t* off, const int32_t* col, const void* val,
                       int dtype, double tol, void* inverse, int32_t* bad_host, cudaStream_t st) {
  DevBuf bad;
  int rc;
  if ((rc = bad.alloc(sizeof(int32_t)))) return rc;
  GBPC_CUDA_TRY(cudaMemsetAsync(bad.p, 0, sizeof(int32_t), st));
  if (nrow > 0) {
    if (dtype == GBPC_F64)
      block_diag_inverse_kernel<double><<<grid_for(nrow, 128), 128, 0, st>>>(
          nrow, b, off, col, (const double*)val, tol, (double*)inverse, bad.as<int32_t>());
    else
      block_diag_inverse_kernel<float><<<grid_for(nrow, 128), 128, 0, st>>>(
          nrow, b, off, col, (const float*)val, (float)tol, (float*)inverse, bad.as<int32_t>());
  }
  GBPC_CUDA_TRY(cudaGetLastError());
  GBPC_CUDA_TRY(cudaMemcpyAsync(bad_host, bad.p, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  GBPC_CUDA_TRY(cudaStreamSynchronize(st));
  return GBPC_OK;
}

template <typename T>
static int bilu0_setup_t(int nrow, int b, const int32_t* off, const int32_t* col, const T* val,
                         int64_t nnz, int factor_sweeps, T relaxation, T tol, T* factors,
                         T* inverse, int32_t* bad_host, cudaStream_t st) {
  DevBuf rows, diag, bad, other;
  int rc;
  const int bb = b * b;
  if ((rc = rows.alloc(sizeof(int32_t) * std::max<int64_t>(nnz, 1)))) return rc;
  if ((rc = diag.alloc(sizeof(int32_t) * std::max(nrow, 1)))) return rc;
  if ((rc = bad.alloc(sizeof(int32_t)))) return rc;
  if ((rc = other.alloc(sizeof(T) * std::max<int64_t>(nnz, 1) * bb))) return rc;
  GBPC_CUDA_TRY(cudaMemsetAsync(bad.p, 0, sizeof(int32_t), st));
  GBPC_CUDA_TRY(cudaMemsetAsync(inverse, 0, sizeof(T) * (size_t)std::max(nrow, 1) * bb, st));
  int32_t* pb = bad.as<int32_t>();
  if (nrow > 0) {
    topology_kernel<<<grid_for(nrow, 128), 128, 0, st>>>(nrow, off, col, rows.as<int32_t>(),
                                                         diag.as<int32_t>(), pb);
    invert_kernel<T><<<grid_for(nrow, 128), 128, 0, st>>>(nrow, b, val, diag.as<int32_t>(),
                                                          inverse, tol, pb);
  }
  GBPC_CUDA_TRY(cudaGetLastError());
  GBPC_CUDA_TRY(cudaMemcpyAsync(bad_host, pb, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  GBPC_CUDA_TRY(cudaStreamSynchronize(st));
  if (*bad_host) return GBPC_OK;
  T* cur = factors;
  T* nxt = other.as<T>();
  if (nnz > 0) {
    initialize_kernel<T><<<grid_for(nnz, 128), 128, 0, st>>>(nnz, b, rows.as<int32_t>(), col, val,
                                                            inverse, cur);
    for (int s = 0; s < factor_sweeps; ++s) {
      sweep_kernel<T><<<grid_for(nnz, 128), 128, 0, st>>>(nnz, b, off, col, rows.as<int32_t>(), val,
                                                          cur, inverse, nxt, relaxation);
      std::swap(cur, nxt);
      invert_kernel<T><<<grid_for(nrow, 128), 128, 0, st>>>(nrow, b, cur, diag.as<int32_t>(),
                                                            inverse, tol, pb);
    }
    if (cur != factors)
      GBPC_CUDA_TRY(cudaMemcpyAsync(factors, cur, sizeof(T) * nnz * bb, cudaMemcpyDeviceToDevice, st));
    validate_kernel<T><<<grid_for(nnz * bb, 256), 256, 0, st>>>(nnz * bb, factors, pb);
  }
  GBPC_CUDA_TRY(cudaGetLastError());
  GBPC_CUDA_TRY(cudaMemcpyAsync(bad_host, pb, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  GBPC_CUDA_TRY(cudaStreamSynchronize(st));
  return GBPC_OK;
}

int bilu0_setup(int nrow, int b, const int32_t* off, const int32_t* col, const void* val,
                int dtype, int64_t nnz, int factor_sweeps, double relaxation, double tol,
                void* factors, void* inverse, int32_t* bad_host, cudaStream_t st) {
  if (dtype == GBPC_F64)
    return bilu0_setup_t<double>(nrow, b, off, col, (const double*)val, nnz, factor_sweeps,
                                 relaxation, tol, (double*)factors, (double*)inverse, bad_host, st);
  return bilu0_setup_t<float>(nrow, b, off, col, (const float*)val, nnz, factor_sweeps,
                              (float)relaxation, (float)tol, (float*)factors, (float*)inverse,
                              bad_host, st);
}

}  // namespace gbpc

using namespace gbpc;

extern "C" int gbpc_block_fsai_setup(int nrow, int block, int max_blocks, const int32_t* offsets,
                                     const int32_t* columns, const void* values, int refit,
                                     int32_t* ell_cols, void* ell_vals, int32_t* row_counts,
                                     void* scale, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  if (nrow < 0 || block < 2 || block > 4 || max_blocks < 1 || max_blocks > 4 ||
      block * max_blocks > kBfMaxWidth) {
    gbpc_set_error("block FSAI supports blocks of 2..4 and max_blocks 1..4 (width <= %d)",
                   kBfMaxWidth);
    return GBPC_ERR_ARG;
  }
  DevBuf status;
  int rc;
  if ((rc = status.alloc(sizeof(int32_t)))) return rc;
  GBPC_CUDA_TRY(cudaMemsetAsync(status.p, 0, sizeof(int32_t), st));
  const int n = nrow * block;
  if (nrow > 0) {
    block_fsai_diag_kernel<double><<<grid_for(n, 128), 128, 0, st>>>(
        n, block, offsets, columns, (const double*)values, (double*)scale, status.as<int32_t>());
    block_fsai_build_kernel<double><<<grid_for(nrow, 64), 64, 0, st>>>(
        nrow, block, max_blocks, offsets, columns, (const double*)values, (const double*)scale,
        ell_cols, (double*)ell_vals, row_counts, status.as<int32_t>(), refit);
  }
  GBPC_CUDA_TRY(cudaGetLastError());
  int32_t h = 0;
  GBPC_CUDA_TRY(cudaMemcpyAsync(&h, status.p, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  GBPC_CUDA_TRY(cudaStreamSynchronize(st));
  if (h) {
    gbpc_set_error("Nonpositive block FSAI pivot");
    return GBPC_ERR_BLOCK_PIVOT;
  }
  return GBPC_OK;
}

template <typename T>
static int csr_to_bsr_t(int nrow_blocks, int b, const int32_t* off, const int32_t* col,
                        const T* val, int32_t* boff, int32_t* bcol, T* bval, int64_t* nnzb_host,
                        cudaStream_t st) {
  if (bcol == nullptr) {
    DevBuf counts;
    int rc;
    if ((rc = counts.alloc(sizeof(int32_t) * (nrow_blocks + 1)))) return rc;
    if (nrow_blocks > 0)
      csr_to_bsr_kernel<T><<<grid_for(nrow_blocks, 128), 128, 0, st>>>(
          nrow_blocks, b, off, col, val, 0, counts.as<int32_t>(), nullptr, nullptr, nullptr);
    GBPC_CUDA_TRY(cudaGetLastError());
    if ((rc = scan_exclusive_i32(counts.as<int32_t>(), boff, nrow_blocks, st))) return rc;
    int32_t total = 0;
    GBPC_CUDA_TRY(cudaMemcpyAsync(&total, boff + nrow_blocks, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    GBPC_CUDA_TRY(cudaStreamSynchronize(st));
    if (nnzb_host) *nnzb_host = total;
    return GBPC_OK;
  }
  if (nrow_blocks > 0)
    csr_to_bsr_kernel<T><<<grid_for(nrow_blocks, 128), 128, 0, st>>>(nrow_blocks, b, off, col, val,
                                                                    1, nullptr, boff, bcol, bval);
  GBPC_CUDA_TRY(cudaGetLastError());
  return GBPC_OK;
}

extern "C" int gbpc_csr_to_bsr(int nrow_blocks, int block, const int32_t* offsets,
                               const int32_t* columns, const void* values, int dtype,
                               int32_t* b_off, int32_t* b_col, void* b_val, int64_t* nnzb_host,
                               void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  if (nrow_blocks < 0 || block < 1 || block > 4 || !offsets || !b_off) {
    gbpc_set_error("gbpc_csr_to_bsr: bad arguments");
    return GBPC_ERR_ARG;
  }
  if (dtype == GBPC_F64)
    return csr_to_bsr_t<double>(nrow_blocks, block, offsets, columns, (const double*)values, b_off,
                                b_col, (double*)b_val, nnzb_host, st);
  if (dtype == GBPC_F32)
    return csr_to_bsr_t<float>(nrow_blocks, block, offsets, columns, (const float*)values, b_off,
                               b_col, (float*)b_val, nnzb_host, st);
  gbpc_set_error("gbpc_csr_to_bsr: dtype must be float64 or float32");
  return GBPC_ERR_ARG;
}

template <typename T>
static int bsr_transpose_t(int nrow, int ncol, int b, const int32_t* off, const int32_t* col,
                           const T* val, int32_t* t_off, int32_t* t_col, T* t_val, cudaStream_t st) {
  DevBuf counts, cursor;
  int rc;
  if ((rc = counts.alloc(sizeof(int32_t) * (ncol + 1)))) return rc;
  if ((rc = cursor.alloc(sizeof(int32_t) * (ncol + 1)))) return rc;
  GBPC_CUDA_TRY(cudaMemsetAsync(counts.p, 0, sizeof(int32_t) * (ncol + 1), st));
  if (nrow > 0)
    count_block_columns_kernel<<<grid_for(nrow, 256), 256, 0, st>>>(nrow, off, col, counts.as<int32_t>());
  GBPC_CUDA_TRY(cudaGetLastError());
  if ((rc = scan_exclusive_i32(counts.as<int32_t>(), t_off, ncol, st))) return rc;
  GBPC_CUDA_TRY(cudaMemcpyAsync(cursor.p, t_off, sizeof(int32_t) * (ncol + 1), cudaMemcpyDeviceToDevice, st));
  if (nrow > 0)
    bsr_scatter_transpose_kernel<T><<<grid_for(nrow, 256), 256, 0, st>>>(
        nrow, b, off, col, val, cursor.as<int32_t>(), t_col, t_val);
  if (ncol > 0)
    bsr_sort_rows_kernel<T><<<grid_for(ncol, 128), 128, 0, st>>>(ncol, b, t_off, t_col, t_val);
  GBPC_CUDA_TRY(cudaGetLastError());
  GBPC_CUDA_TRY(cudaStreamSynchronize(st));
  return GBPC_OK;
}

extern "C" int gbpc_bsr_transpose(int nrow, int ncol, int block, const int32_t* offsets,
                                  const int32_t* columns, const void* values, int dtype,
                                  int32_t* t_off, int32_t* t_col, void* t_val, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  if (nrow < 0 || ncol < 0 || block < 1 || block > 4 || !offsets || !t_off) {
    gbpc_set_error("gbpc_bsr_transpose: bad arguments");
    return GBPC_ERR_ARG;
  }
  if (dtype == GBPC_F64)
    return bsr_transpose_t<double>(nrow, ncol, block, offsets, columns, (const double*)values, t_off,
                                   t_col, (double*)t_val, st);
  if (dtype == GBPC_F32)
    return bsr_transpose_t<float>(nrow, ncol, block, offsets, columns, (const float*)values, t_off,
                                  t_col, (float*)t_val, st);
  gbpc_set_error("gbpc_bsr_transpose: dtype must be float64 or float32");
  return GBPC_ERR_ARG;
}
