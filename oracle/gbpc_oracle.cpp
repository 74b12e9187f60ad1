// CPU oracle for the preconditioned-Krylov path of warp-preconditioners.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, in plain sequential C++, the
// algorithms of the reference package (alecjacobson/warp-preconditioners) so
// that the CUDA path can be checked against it.  Only the tests, the smoke
// check and the CPU-baseline leg of bench.py load it; the product never does.
//
// Arithmetic rules: IEEE-754 binary64/binary32, round to nearest, and NO
// multiply-add contraction (the build passes -ffp-contract=off on x86 and Arm
// alike).  Every loop keeps the reference's operation order, so the FSAI
// supports and values produced here are bit-for-bit those of a non-contracting
// evaluation of the reference kernels.
//
// Each function cites the reference file and lines it follows.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

template <typename T>
inline bool finite(T v) { return std::isfinite(v); }

// warp_preconditioners/fsai.py:21-41 (`entry`): lower-bound binary search of
// column j in the sorted CSR row i; zero when absent.
template <typename T>
inline T entry(const int32_t* off, const int32_t* col, const T* val, int i, int j) {
  int lo = off[i], hi = off[i + 1];
  const int end = hi;
  while (lo < hi) {
    const int mid = (lo + hi) / 2;
    if (col[mid] < j) lo = mid + 1; else hi = mid;
  }
  T result = T(0);
  if (lo < end && col[lo] == j) result = val[lo];
  return result;
}

// Whether row i stores column j (operation counting only).
inline bool stored(const int32_t* off, const int32_t* col, int i, int j) {
  const int32_t* b = col + off[i];
  const int32_t* e = col + off[i + 1];
  const int32_t* p = std::lower_bound(b, e, j);
  return p != e && *p == j;
}

// warp_preconditioners/fsai.py:44-57 (`diagonal`).
template <typename T>
void fsai_diagonal(int n, const int32_t* off, const int32_t* col, const T* val, T* scale,
                   int32_t* status) {
  int32_t bad = 0;
#pragma omp parallel for reduction(+ : bad) schedule(static)
  for (int i = 0; i < n; ++i) {
    const T d = entry(off, col, val, i, i);
    if (d > T(0) && finite(d)) {
      scale[i] = T(1) / std::sqrt(d);
    } else {
      scale[i] = T(0);
      bad += 1;
    }
  }
  status[0] += bad;
}

// warp_preconditioners/fsai.py:60-176 (`build`): adaptive support growth with
// bordered Cholesky, one row at a time.  Returns status increments through
// `truncated` (status[1]) and `invalid` (status[2]).
//
// With COUNT, `flops` accumulates the row's floating-point operations: every
// separately rounded multiply, add/subtract, divide and square root counts
// one (the reference evaluates without contraction, so there are no fused
// multiply-adds); comparisons and fabs count none.  A candidate's score term
// for a support row that does not store the candidate's column is a product
// with the lookup's zero: it is not counted, since it contributes nothing
// and a sparse implementation skips it; the small dense Cholesky updates are
// counted in full.
//
// The row's width slots are written at output row `out_row` (row i itself
// when every row is built; its position in the list when only some are).
template <typename T, bool COUNT = false>
void fsai_build_row(int i, const int32_t* off, const int32_t* col, const T* val, const T* scale,
                    T tolerance, T pivot_floor, int width, int step, int32_t* cols_out,
                    T* vals_out, int& truncated, int& invalid, std::vector<int>& pattern,
                    std::vector<T>& chol, std::vector<T>& z, std::vector<T>& v, std::vector<T>& w,
                    std::vector<int>& cand, std::vector<T>& sc, int64_t& flops, int out_row = -1) {
  if (out_row < 0) out_row = i;
  std::fill(pattern.begin(), pattern.end(), -1);
  std::fill(chol.begin(), chol.end(), T(0));
  std::fill(z.begin(), z.end(), T(0));
  std::fill(v.begin(), v.end(), T(0));
  auto L = [&](int r, int c) -> T& { return chol[(size_t)r * width + c]; };
  pattern[0] = i;
  L(0, 0) = T(1);
  z[0] = T(1);
  v[0] = T(1);
  int size = 1;
  while (size < width) {
    std::fill(cand.begin(), cand.end(), -1);
    std::fill(sc.begin(), sc.end(), T(0));
    for (int p = 0; p < size; ++p) {
      const int row = pattern[p];
      for (int e = off[row]; e < off[row + 1]; ++e) {
        const int c = col[e];
        bool selected = c >= i;
        for (int q = 0; q < size; ++q)
          if (pattern[q] == c) selected = true;
        for (int q = 0; q < step; ++q)
          if (cand[q] == c) selected = true;
        if (selected) continue;
        T residual = T(0);
        for (int q = 0; q < size; ++q) {
          const int j = pattern[q];
          if constexpr (COUNT) flops += stored(off, col, c, j) ? 4 : 0;
          // ((a * s_c) * s_j) * z_q, then the running sum: no contraction.
          const T a = entry(off, col, val, c, j);
          const T t1 = a * scale[c];
          const T t2 = t1 * scale[j];
          const T t3 = t2 * z[q];
          residual = residual + t3;
        }
        const T score = std::fabs(residual);
        for (int rank = 0; rank < step; ++rank) {
          if (score > sc[rank] || (score == sc[rank] && c < cand[rank])) {
            for (int dest = step - 1; dest > rank; --dest) {
              cand[dest] = cand[dest - 1];
              sc[dest] = sc[dest - 1];
            }
            cand[rank] = c;
            sc[rank] = score;
            break;
          }
        }
      }
    }
    if (cand[0] < 0) break;
    const T old_z0 = z[0];
    bool stopped = false;
    for (int rank = 0; rank < step; ++rank) {
      const int best = cand[rank];
      if (best < 0 || size == width) break;
      // Border the Cholesky factor of the selected principal submatrix.
      T pivot = T(1);
      // per p: 2 scalings, p multiply-subtracts, a divide, a square and its subtraction
      if constexpr (COUNT) flops += 5 * (int64_t)size + (int64_t)size * (size - 1);
      for (int p = 0; p < size; ++p) {
        const T e0 = entry(off, col, val, best, pattern[p]);
        T a = (e0 * scale[best]) * scale[pattern[p]];
        for (int q = 0; q < p; ++q) {
          const T prod = L(p, q) * w[q];
          a = a - prod;
        }
        w[p] = a / L(p, p);
        const T sq = w[p] * w[p];
        pivot = pivot - sq;
      }
      if (pivot <= pivot_floor || !finite(pivot)) {
        truncated += 1;
        stopped = true;
        break;
      }
      pattern[size] = best;
      for (int p = 0; p < size; ++p) L(size, p) = w[p];
      if constexpr (COUNT) flops += 1 + 2 * (int64_t)size + 1;  // sqrt, rhs, divide
      L(size, size) = std::sqrt(pivot);
      T rhs = T(0);
      for (int p = 0; p < size; ++p) {
        const T prod = w[p] * v[p];
        rhs = rhs - prod;
      }
      v[size] = rhs / L(size, size);
      size += 1;
    }
    // A[S,S] z = e_0 through L^T z = v.
    if constexpr (COUNT) flops += (int64_t)size + (int64_t)size * (size - 1);
    for (int rev = 0; rev < size; ++rev) {
      const int p = size - 1 - rev;
      T a = v[p];
      for (int q = p + 1; q < size; ++q) {
        const T prod = L(q, p) * z[q];
        a = a - prod;
      }
      z[p] = a / L(p, p);
    }
    if (stopped) break;
    if (tolerance > T(0)) {
      if constexpr (COUNT) flops += 2;
      const T ratio = old_z0 / z[0];
      if (T(1) - ratio <= tolerance) break;
    }
  }
  const T norm = std::sqrt(z[0]);
  if constexpr (COUNT) flops += 1 + 2 * (int64_t)size;
  bool valid = true;
  for (int p = 0; p < width; ++p) {
    const size_t e = (size_t)out_row * width + p;
    cols_out[e] = -1;
    vals_out[e] = T(0);
    if (p < size) {
      cols_out[e] = pattern[p];
      vals_out[e] = (z[p] / norm) * scale[pattern[p]];
      if (!finite(vals_out[e])) valid = false;
      if (p == 0 && vals_out[e] <= T(0)) valid = false;
    }
  }
  if (!valid) invalid += 1;
}

template <typename T, bool COUNT = false>
void fsai_setup(int n, const int32_t* off, const int32_t* col, const T* val, int width, int step,
                T tolerance, T pivot_floor, int32_t* cols_out, T* vals_out, T* scale,
                int32_t* status, int64_t* flops_out = nullptr) {
  fsai_diagonal(n, off, col, val, scale, status);
  int truncated = 0, invalid = 0;
  int64_t flops = COUNT ? 2 * (int64_t)n : 0;  // 1 / sqrt(a_ii) per row
#pragma omp parallel reduction(+ : truncated, invalid, flops)
  {
    std::vector<int> pattern(width), cand(step);
    std::vector<T> chol((size_t)width * width), z(width), v(width), w(width), sc(step);
#pragma omp for schedule(dynamic, 256)
    for (int i = 0; i < n; ++i)
      fsai_build_row<T, COUNT>(i, off, col, val, scale, tolerance, pivot_floor, width, step,
                               cols_out, vals_out, truncated, invalid, pattern, chol, z, v, w,
                               cand, sc, flops);
  }
  status[1] += truncated;
  status[2] += invalid;
  if (flops_out) *flops_out = flops;
}

// The same build for the listed rows only (every row of the reference's
// build is independent, so any subset gives exactly those rows of the full
// factor): row rows[k] is written to output row k.  Scales are computed for
// all rows, since a row's scores read its candidates' scales.
template <typename T>
void fsai_setup_rows(int n, const int32_t* off, const int32_t* col, const T* val, int width,
                     int step, T tolerance, T pivot_floor, int nrows, const int32_t* rows,
                     int32_t* cols_out, T* vals_out, int32_t* status) {
  std::vector<T> scale((size_t)std::max(n, 1));
  fsai_diagonal(n, off, col, val, scale.data(), status);
  int truncated = 0, invalid = 0;
  int64_t flops = 0;
#pragma omp parallel reduction(+ : truncated, invalid)
  {
    std::vector<int> pattern(width), cand(step);
    std::vector<T> chol((size_t)width * width), z(width), v(width), w(width), sc(step);
#pragma omp for schedule(dynamic, 16)
    for (int k = 0; k < nrows; ++k)
      fsai_build_row<T, false>(rows[k], off, col, val, scale.data(), tolerance, pivot_floor,
                               width, step, cols_out, vals_out, truncated, invalid, pattern,
                               chol, z, v, w, cand, sc, flops, k);
  }
  status[1] += truncated;
  status[2] += invalid;
}

// warp_preconditioners/fsai_pack.py:15-71 (`sort_rows`, `array_scan`, `pack`).
// Sorts each width-slot row by column in place, then compacts to CSR.
template <typename T>
int64_t fsai_pack(int n, int width, int32_t* ell_cols, T* ell_vals, int32_t* g_off,
                  int32_t* g_col, T* g_val) {
  std::vector<int32_t> counts((size_t)n + 1, 0);
#pragma omp parallel
  {
    std::vector<int> cols(width);
    std::vector<T> vals(width);
#pragma omp for schedule(static)
    for (int i = 0; i < n; ++i) {
      int size = 0;
      for (int p = 0; p < width; ++p) {
        const int c = ell_cols[(size_t)i * width + p];
        if (c < 0) continue;
        const T vv = ell_vals[(size_t)i * width + p];
        int q = size;
        while (q > 0) {
          if (cols[q - 1] <= c) break;
          cols[q] = cols[q - 1];
          vals[q] = vals[q - 1];
          --q;
        }
        cols[q] = c;
        vals[q] = vv;
        ++size;
      }
      counts[(size_t)i + 1] = size;
      for (int p = 0; p < size; ++p) {
        ell_cols[(size_t)i * width + p] = cols[p];
        ell_vals[(size_t)i * width + p] = vals[p];
      }
    }
  }
  // Inclusive scan of counts (counts[0] == 0) gives the row offsets.
  int64_t running = 0;
  for (int i = 0; i <= n; ++i) {
    running += counts[i];
    g_off[i] = (int32_t)running;
  }
  if (g_col != nullptr) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i)
      for (int e = g_off[i]; e < g_off[i + 1]; ++e) {
        const size_t p = (size_t)i * width + (e - g_off[i]);
        g_col[e] = ell_cols[p];
        g_val[e] = ell_vals[p];
      }
  }
  return running;
}

// Explicit transpose of a canonical CSR matrix: rows of the result list the
// source rows in increasing order (warp.sparse.bsr_transposed semantics for
// scalar blocks, called from warp_preconditioners/fsai.py:356).
template <typename T>
void csr_transpose(int nrow, int ncol, const int32_t* off, const int32_t* col, const T* val,
                   int32_t* t_off, int32_t* t_col, T* t_val) {
  std::vector<int32_t> count((size_t)ncol + 1, 0);
  for (int i = 0; i < nrow; ++i)
    for (int e = off[i]; e < off[i + 1]; ++e) count[(size_t)col[e] + 1] += 1;
  t_off[0] = 0;
  for (int j = 0; j < ncol; ++j) t_off[j + 1] = t_off[j] + count[(size_t)j + 1];
  std::vector<int32_t> cursor(t_off, t_off + ncol);
  for (int i = 0; i < nrow; ++i)
    for (int e = off[i]; e < off[i + 1]; ++e) {
      const int32_t dst = cursor[col[e]]++;
      t_col[dst] = i;
      t_val[dst] = val[e];
    }
}

// warp_preconditioners/fsai_pack.py:74-107 (`scalarize`): canonical b x b BSR
// to scalar CSR, keeping numerical zeros stored inside blocks.
template <typename T>
void scalarize(int nrow_blocks, int b, const int32_t* off, const int32_t* col, const T* val,
               int32_t* out_off, int32_t* out_col, T* out_val) {
  const int n = nrow_blocks * b;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) {
    const int r = i / b, component = i % b;
    const int start = off[r];
    const int count = off[r + 1] - start;
    const int64_t base = (int64_t)start * b * b + (int64_t)component * count * b;
    out_off[i] = (int32_t)base;
    for (int p = 0; p < count; ++p)
      for (int c = 0; c < b; ++c) {
        const int64_t dest = base + (int64_t)p * b + c;
        out_col[dest] = col[start + p] * b + c;
        out_val[dest] = val[((size_t)start + p) * b * b + (size_t)component * b + c];
      }
    if (i == n - 1) out_off[i + 1] = (int32_t)(base + (int64_t)count * b);
  }
  if (n == 0) out_off[0] = 0;
}

// z = alpha * A x + beta * y for scalar CSR with storage type S and arithmetic
// type A.  warp_preconditioners/sparse_operator.py:64-87 (`_mixed_kernel`): the
// row sum runs in stored order; alpha == 0 never reads x, beta == 0 never
// reads y.  x must not alias z (callers copy, sparse_operator.py:119-121).
template <typename S, typename A>
void csr_spmv(int n, const int32_t* off, const int32_t* col, const S* val, const A* x,
              const A* y, A* z, A alpha, A beta) {
#pragma omp parallel for schedule(static)
  for (int row = 0; row < n; ++row) {
    A result = A(0);
    if (alpha != A(0)) {
      for (int e = off[row]; e < off[row + 1]; ++e) {
        const A prod = A(val[e]) * x[col[e]];
        result = result + prod;
      }
      result = result * alpha;
    }
    if (beta != A(0)) {
      const A t = beta * y[row];
      result = result + t;
    }
    z[row] = result;
  }
}

// Block CSR product, b x b blocks stored row-major
// (benchmarks/block_fsai_candidate.py:264-293 `block_product`).
template <typename S, typename A>
void bsr_spmv(int nrow, int b, const int32_t* off, const int32_t* col, const S* val, const A* x,
              const A* y, A* z, A alpha, A beta) {
#pragma omp parallel for schedule(static)
  for (int row = 0; row < nrow; ++row) {
    A result[4] = {A(0), A(0), A(0), A(0)};
    if (alpha != A(0)) {
      for (int e = off[row]; e < off[row + 1]; ++e) {
        const A* xx = x + (size_t)col[e] * b;
        const S* blk = val + (size_t)e * b * b;
        for (int r = 0; r < b; ++r)
          for (int c = 0; c < b; ++c) {
            const A prod = A(blk[r * b + c]) * xx[c];
            result[r] = result[r] + prod;
          }
      }
    }
    for (int r = 0; r < b; ++r) {
      A value = result[r] * alpha;
      if (beta != A(0)) value = value + beta * y[(size_t)row * b + r];
      z[(size_t)row * b + r] = value;
    }
  }
}

// warp_preconditioners/squared_laplacian.py:37-101 (`forward`, `backward`):
// z = alpha * ((L M^-1 L + w M)[free, free] x) + beta * y, or with
// boundary=true the eliminated right-hand side product of rhs().
template <typename T>
void sqlap_apply(int n, const int32_t* off, const int32_t* col, const T* val,
                 const T* inverse_mass, const T* mass, const int32_t* free, int nfree,
                 const int32_t* index, T mass_weight, const T* x, const T* y, T* z, T alpha,
                 T beta, bool boundary, T* tmp) {
#pragma omp parallel for schedule(static)
  for (int row = 0; row < n; ++row) {
    T acc = T(0);
    for (int e = off[row]; e < off[row + 1]; ++e) {
      const int c_full = col[e];
      const int c = index[c_full];
      if (boundary) {
        if (c < 0) acc = acc + val[e] * x[c_full];
      } else {
        if (c >= 0) acc = acc + val[e] * x[c];
      }
    }
    tmp[row] = inverse_mass[row] * acc;
  }
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nfree; ++i) {
    T acc = T(0);
    const int row = free[i];
    if (alpha != T(0))
      for (int e = off[row]; e < off[row + 1]; ++e) acc = acc + val[e] * tmp[col[e]];
    if (mass_weight != T(0) && alpha != T(0)) acc = acc + (mass_weight * mass[free[i]]) * x[i];
    acc = acc * alpha;
    if (beta != T(0)) acc = acc + beta * y[i];
    z[i] = acc;
  }
}

// Small dense helpers for warp_preconditioners/block_ilu.py:17-43
// (`safe_inverse`): determinant and adjugate inverse of 1..4 square blocks.
template <typename T>
T det_n(const T* a, int b) {
  if (b == 1) return a[0];
  if (b == 2) return a[0] * a[3] - a[1] * a[2];
  if (b == 3)
    return a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) +
           a[2] * (a[3] * a[7] - a[4] * a[6]);
  // 4x4 by cofactor expansion along the first row.
  T total = T(0);
  for (int c = 0; c < 4; ++c) {
    T m[9];
    int k = 0;
    for (int r = 1; r < 4; ++r)
      for (int cc = 0; cc < 4; ++cc)
        if (cc != c) m[k++] = a[r * 4 + cc];
    const T cof = det_n(m, 3);
    total = (c % 2 == 0) ? total + a[c] * cof : total - a[c] * cof;
  }
  return total;
}

template <typename T>
void inverse_n(const T* a, int b, T* out) {
  const T det = det_n(a, b);
  if (b == 1) {
    out[0] = T(1) / a[0];
    return;
  }
  for (int r = 0; r < b; ++r)
    for (int c = 0; c < b; ++c) {
      // adj[r][c] = (-1)^(r+c) * minor(c, r)
      T m[9];
      int k = 0;
      for (int rr = 0; rr < b; ++rr)
        for (int cc = 0; cc < b; ++cc)
          if (rr != c && cc != r) m[k++] = a[rr * b + cc];
      const T minor = det_n(m, b - 1);
      out[r * b + c] = (((r + c) % 2) ? -minor : minor) / det;
    }
}

template <typename T>
int safe_inverse(const T* a, int b, T tolerance, T* inverse) {
  int bad = 0;
  T scale = T(0);
  for (int k = 0; k < b * b; ++k) scale = std::max(scale, (T)std::fabs(a[k]));
  for (int k = 0; k < b * b; ++k) inverse[k] = T(0);
  if (scale > T(0) && finite(scale)) {
    T normalized[16];
    for (int k = 0; k < b * b; ++k) normalized[k] = a[k] / scale;
    const T det = det_n(normalized, b);
    if (finite(det) && std::fabs(det) > tolerance) {
      if (b == 1) {
        inverse[0] = T(1) / a[0];
      } else {
        inverse_n(normalized, b, inverse);
        for (int k = 0; k < b * b; ++k) inverse[k] = inverse[k] / scale;
      }
    } else {
      bad += 1;
    }
  } else {
    bad += 1;
  }
  for (int k = 0; k < b * b; ++k)
    if (!finite(inverse[k])) bad += 1;
  return bad;
}

// warp_preconditioners/block_ilu.py:76-104 (`diagonal_only`).
template <typename T>
int block_diag_inverse(int nrow, int b, const int32_t* off, const int32_t* col, const T* val,
                       T tolerance, T* inverse) {
  int bad = 0;
#pragma omp parallel for reduction(+ : bad) schedule(static)
  for (int i = 0; i < nrow; ++i) {
    int lo = off[i], hi = off[i + 1];
    const int end = hi;
    while (lo < hi) {
      const int mid = (lo + hi) / 2;
      if (col[mid] < i) lo = mid + 1; else hi = mid;
    }
    if (lo < end && col[lo] == i)
      bad += safe_inverse(val + (size_t)lo * b * b, b, tolerance, inverse + (size_t)i * b * b);
    else
      bad += 1;
  }
  return bad;
}

template <typename T>
inline void matmul(const T* a, const T* bm, int b, T* out) {
  for (int r = 0; r < b; ++r)
    for (int c = 0; c < b; ++c) {
      T s = T(0);
      for (int k = 0; k < b; ++k) s = s + a[r * b + k] * bm[k * b + c];
      out[r * b + c] = s;
    }
}

// warp_preconditioners/block_ilu.py:362-402 with kernels :46-150, :205-210:
// topology, diagonal inversion, initialisation, `factor_sweeps` synchronous
// sweeps (each followed by re-inversion of the factor diagonal), validation.
template <typename T>
int bilu0_setup(int nrow, int b, const int32_t* off, const int32_t* col, const T* val,
                int factor_sweeps, T relaxation, T tolerance, T* factors, T* inverse) {
  const int bb = b * b;
  const int64_t nnz = off[nrow];
  std::vector<int32_t> rows(nnz), diag(nrow);
  int bad = 0;
  for (int i = 0; i < nrow; ++i) {
    int found = -1;
    for (int e = off[i]; e < off[i + 1]; ++e) {
      rows[e] = i;
      if (col[e] == i) found = e;
    }
    diag[i] = found;
    if (found < 0) bad += 1;
  }
  auto invert = [&](const T* values) {
    int nb = 0;
#pragma omp parallel for reduction(+ : nb) schedule(static)
    for (int i = 0; i < nrow; ++i)
      if (diag[i] >= 0)
        nb += safe_inverse(values + (size_t)diag[i] * bb, b, tolerance, inverse + (size_t)i * bb);
    return nb;
  };
  bad += invert(val);
  if (bad) return bad;
  std::vector<T> other((size_t)nnz * bb);
  T* cur = factors;
  T* nxt = other.data();
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < nnz; ++e) {
    if (col[e] < rows[e]) matmul(val + e * bb, inverse + (size_t)col[e] * bb, b, cur + e * bb);
    else std::memcpy(cur + e * bb, val + e * bb, sizeof(T) * bb);
  }
  for (int s = 0; s < factor_sweeps; ++s) {
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < nnz; ++e) {
      const int i = rows[e], j = col[e];
      T value[16], prod[16], out[16];
      std::memcpy(value, val + e * bb, sizeof(T) * bb);
      for (int ik = off[i]; ik < off[i + 1]; ++ik) {
        const int k = col[ik];
        if (k >= std::min(i, j)) break;
        int lo = off[k], hi = off[k + 1];
        while (lo < hi) {
          const int mid = (lo + hi) / 2;
          if (col[mid] < j) lo = mid + 1; else hi = mid;
        }
        if (lo < off[k + 1] && col[lo] == j) {
          matmul(cur + (size_t)ik * bb, cur + (size_t)lo * bb, b, prod);
          for (int q = 0; q < bb; ++q) value[q] = value[q] - prod[q];
        }
      }
      if (j < i) {
        matmul(value, inverse + (size_t)j * bb, b, out);
        std::memcpy(value, out, sizeof(T) * bb);
      }
      for (int q = 0; q < bb; ++q)
        nxt[e * bb + q] = (T(1) - relaxation) * cur[e * bb + q] + relaxation * value[q];
    }
    std::swap(cur, nxt);
    bad += invert(cur);
  }
  if (cur != factors) std::memcpy(factors, cur, sizeof(T) * (size_t)nnz * bb);
  for (int64_t k = 0; k < nnz * bb; ++k)
    if (!finite(factors[k])) bad += 1;
  return bad;
}

// warp_preconditioners/block_ilu.py:404-450 (`_apply`) with `triangular`
// (:153-171) and `combine` (:174-185), and :188-202 for alpha == 0.
template <typename T>
void bilu0_apply(int nrow, int b, const int32_t* off, const int32_t* col, const T* factors,
                 const T* inverse, int solve_sweeps, const T* x, const T* y, T* z, T alpha,
                 T beta) {
  const int bb = b * b;
  const size_t n = (size_t)nrow * b;
  if (alpha == T(0)) {
    for (size_t k = 0; k < n; ++k) z[k] = (beta != T(0)) ? beta * y[k] : T(0);
    return;
  }
  std::vector<T> a(n, T(0)), bbuf(n), c(n, T(0)), d(n);
  auto sweep = [&](const T* rhs, const T* old, T* out, bool lower) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nrow; ++i) {
      T value[4];
      for (int r = 0; r < b; ++r) value[r] = rhs[(size_t)i * b + r];
      for (int e = off[i]; e < off[i + 1]; ++e) {
        const int j = col[e];
        if ((lower && j < i) || (!lower && j > i)) {
          const T* f = factors + (size_t)e * bb;
          for (int r = 0; r < b; ++r) {
            T s = T(0);
            for (int k = 0; k < b; ++k) s = s + f[r * b + k] * old[(size_t)j * b + k];
            value[r] = value[r] - s;
          }
        }
      }
      if (!lower) {
        T tmp[4];
        const T* inv = inverse + (size_t)i * bb;
        for (int r = 0; r < b; ++r) {
          T s = T(0);
          for (int k = 0; k < b; ++k) s = s + inv[r * b + k] * value[k];
          tmp[r] = s;
        }
        for (int r = 0; r < b; ++r) value[r] = tmp[r];
      }
      for (int r = 0; r < b; ++r) out[(size_t)i * b + r] = value[r];
    }
  };
  T* pa = a.data();
  T* pb = bbuf.data();
  for (int s = 0; s < solve_sweeps; ++s) {
    sweep(x, pa, pb, true);
    std::swap(pa, pb);
  }
  T* pc = c.data();
  T* pd = d.data();
  for (int s = 0; s < solve_sweeps; ++s) {
    sweep(pa, pc, pd, false);
    std::swap(pc, pd);
  }
  for (size_t k = 0; k < n; ++k) {
    T value = alpha * pc[k];
    if (beta != T(0)) value = value + beta * y[k];
    z[k] = value;
  }
}

// block_ilu.py:188-202 (`diagonal_apply`): z = alpha D^-1 x + beta y.
template <typename T>
void block_jacobi_apply(int nrow, int b, const T* inverse, const T* x, const T* y, T* z, T alpha,
                        T beta) {
  const int bb = b * b;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nrow; ++i) {
    T value[4] = {T(0), T(0), T(0), T(0)};
    if (alpha != T(0))
      for (int r = 0; r < b; ++r) {
        T s = T(0);
        for (int k = 0; k < b; ++k) s = s + inverse[(size_t)i * bb + r * b + k] * x[(size_t)i * b + k];
        value[r] = alpha * s;
      }
    for (int r = 0; r < b; ++r) {
      if (beta != T(0)) value[r] = value[r] + beta * y[(size_t)i * b + r];
      z[(size_t)i * b + r] = value[r];
    }
  }
}

// benchmarks/block_fsai_candidate.py:22-59 (`entry`, `diagonal`) on b x b BSR.
template <typename T>
inline T block_entry(const int32_t* off, const int32_t* col, const T* val, int b, int i, int j) {
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

// benchmarks/block_fsai_candidate.py:61-176 (`build`): block-row greedy
// growth with a full local Cholesky per step, b right-hand sides, and the
// block-row normalisation G = chol(Z_ii)^-1 Z^T D^-1/2.  Output: scalar ELL
// rows of width b*max_blocks.
template <typename T>
int block_fsai_setup(int nrow, int b, int max_blocks, const int32_t* off, const int32_t* col,
                     const T* val, int32_t* cols_out, T* vals_out, T* scale, bool refit) {
  const int n = nrow * b;
  const int width = b * max_blocks;
  int bad = 0;
#pragma omp parallel for reduction(+ : bad) schedule(static)
  for (int i = 0; i < n; ++i) {
    const T d = block_entry(off, col, val, b, i, i);
    if (d > T(0) && finite(d)) {
      scale[i] = T(1) / std::sqrt(d);
    } else {
      bad += 1;
      scale[i] = T(0);
    }
  }
#pragma omp parallel reduction(+ : bad)
  {
    std::vector<int> pattern(max_blocks);
    std::vector<T> chol((size_t)width * width), z((size_t)width * b);
#pragma omp for schedule(dynamic, 64)
    for (int i = 0; i < nrow; ++i) {
      std::fill(pattern.begin(), pattern.end(), -1);
      pattern[0] = i;
      int size = 1;
      if (refit) {
        for (int p = 0; p < max_blocks; ++p) {
          const int c = cols_out[(size_t)i * b * width + p * b];
          if (c >= 0 && c / b != i) pattern[size++] = c / b;
        }
      }
      std::fill(z.begin(), z.end(), T(0));
      auto Z = [&](int p, int c) -> T& { return z[(size_t)p * b + c]; };
      for (int stepi = 0; stepi < max_blocks; ++stepi) {
        std::fill(chol.begin(), chol.end(), T(0));
        auto L = [&](int p, int q) -> T& { return chol[(size_t)p * width + q]; };
        const int count = size * b;
        for (int p = 0; p < count; ++p) {
          const int r = pattern[p / b] * b + p % b;
          for (int q = 0; q <= p; ++q) {
            const int c = pattern[q / b] * b + q % b;
            T vv = (block_entry(off, col, val, b, r, c) * scale[r]) * scale[c];
            for (int k = 0; k < q; ++k) vv = vv - L(p, k) * L(q, k);
            if (p == q) {
              if (vv <= T(0) || !finite(vv)) {
                bad += 1;
                vv = T(1);
              }
              L(p, q) = std::sqrt(vv);
            } else {
              L(p, q) = vv / L(q, q);
            }
          }
        }
        for (int c = 0; c < b; ++c) {
          for (int p = 0; p < count; ++p) {
            T vv = (p == c) ? T(1) : T(0);
            for (int q = 0; q < p; ++q) vv = vv - L(p, q) * Z(q, c);
            Z(p, c) = vv / L(p, p);
          }
          for (int rev = 0; rev < count; ++rev) {
            const int p = count - rev - 1;
            T vv = Z(p, c);
            for (int q = p + 1; q < count; ++q) vv = vv - L(q, p) * Z(q, c);
            Z(p, c) = vv / L(p, p);
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
                             ((block_entry(off, col, val, b, cr, j) * scale[cr]) * scale[j]) * Z(q, c);
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
      // Block-row normalisation.
      T norm[16] = {};
      for (int r = 0; r < b; ++r)
        for (int c = 0; c <= r; ++c) {
          T vv = Z(r, c);
          for (int k = 0; k < c; ++k) vv = vv - norm[r * b + k] * norm[c * b + k];
          if (r == c) norm[r * b + c] = std::sqrt(vv);
          else norm[r * b + c] = vv / norm[c * b + c];
        }
      for (int q = 0; q < size * b; ++q)
        for (int r = 0; r < b; ++r) {
          T vv = Z(q, r);
          for (int k = 0; k < r; ++k) vv = vv - norm[r * b + k] * Z(q, k);
          Z(q, r) = vv / norm[r * b + r];
        }
      for (int r = 0; r < b; ++r)
        for (int q = 0; q < width; ++q) {
          const size_t e = ((size_t)i * b + r) * width + q;
          cols_out[e] = -1;
          vals_out[e] = T(0);
          if (q < size * b) {
            const int j = pattern[q / b] * b + q % b;
            cols_out[e] = j;
            vals_out[e] = Z(q, r) * scale[j];
          }
        }
    }
  }
  return bad;
}

// ---------------------------------------------------------------------------
// Krylov solvers.  The reference calls warp.optim.linear.cg / cr (warp-lang,
// not vendored; call sites benchmarks/block_challenge.py:131-139,
// visualization/solve_fields.py:121-124).  These are the textbook
// preconditioned conjugate gradient and conjugate residual recurrences with
// the same stopping rule: the recursive residual r.r <= max(atol, tol*|b|)^2,
// tested before every iteration, and at most maxiter iterations.

struct Operator {
  // kind 0: identity; 1: scalar CSR; 2: b x b BSR; 3: factored squared
  // Laplacian (all free); 4: FSAI G^T G with explicit G and GT (CSR, f64 or
  // f32 storage); 5: diagonal scaling z = alpha*d*x; 6: block Jacobi
  // (inverse blocks); 7: block ILU(0).
  int kind;
  int n;     // scalar length of the vectors
  int nrow;  // rows of the (block) matrix
  int b;
  const int32_t* off;
  const int32_t* col;
  const void* val;
  int val_f32;  // storage is float32
  const int32_t* off2;
  const int32_t* col2;
  const void* val2;
  const double* mass;
  const double* inv_mass;
  double mass_weight;
  const double* diag;  // kind 5 scaling, kind 6/7 inverse blocks
  const double* factors;
  int sweeps;
};

void op_apply(const Operator& op, const double* x, const double* y, double* z, double alpha,
              double beta, std::vector<double>& tmp) {
  switch (op.kind) {
    case 0:
#pragma omp parallel for schedule(static)
      for (int k = 0; k < op.n; ++k) z[k] = alpha * x[k] + (beta != 0.0 ? beta * y[k] : 0.0);
      break;
    case 1:
      if (op.val_f32)
        csr_spmv<float, double>(op.n, op.off, op.col, (const float*)op.val, x, y, z, alpha, beta);
      else
        csr_spmv<double, double>(op.n, op.off, op.col, (const double*)op.val, x, y, z, alpha, beta);
      break;
    case 2:
      if (op.val_f32)
        bsr_spmv<float, double>(op.nrow, op.b, op.off, op.col, (const float*)op.val, x, y, z, alpha, beta);
      else
        bsr_spmv<double, double>(op.nrow, op.b, op.off, op.col, (const double*)op.val, x, y, z, alpha, beta);
      break;
    case 3: {
      tmp.resize(op.n);
      const double* L = (const double*)op.val;
#pragma omp parallel for schedule(static)
      for (int row = 0; row < op.n; ++row) {
        double acc = 0.0;
        for (int e = op.off[row]; e < op.off[row + 1]; ++e) acc = acc + L[e] * x[op.col[e]];
        tmp[row] = op.inv_mass[row] * acc;
      }
#pragma omp parallel for schedule(static)
      for (int row = 0; row < op.n; ++row) {
        double acc = 0.0;
        for (int e = op.off[row]; e < op.off[row + 1]; ++e) acc = acc + L[e] * tmp[op.col[e]];
        if (op.mass_weight != 0.0) acc = acc + (op.mass_weight * op.mass[row]) * x[row];
        acc = acc * alpha;
        if (beta != 0.0) acc = acc + beta * y[row];
        z[row] = acc;
      }
      break;
    }
    case 4: {
      tmp.resize(op.n);
      if (op.val_f32) {
        csr_spmv<float, double>(op.n, op.off, op.col, (const float*)op.val, x, tmp.data(), tmp.data(), 1.0, 0.0);
        csr_spmv<float, double>(op.n, op.off2, op.col2, (const float*)op.val2, tmp.data(), y, z, alpha, beta);
      } else {
        csr_spmv<double, double>(op.n, op.off, op.col, (const double*)op.val, x, tmp.data(), tmp.data(), 1.0, 0.0);
        csr_spmv<double, double>(op.n, op.off2, op.col2, (const double*)op.val2, tmp.data(), y, z, alpha, beta);
      }
      break;
    }
    case 5:
#pragma omp parallel for schedule(static)
      for (int k = 0; k < op.n; ++k) {
        double v = alpha * (x[k] * op.diag[k]);
        if (beta != 0.0) v = v + beta * y[k];
        z[k] = v;
      }
      break;
    case 6:
      block_jacobi_apply<double>(op.nrow, op.b, op.diag, x, y, z, alpha, beta);
      break;
    case 7:
      bilu0_apply<double>(op.nrow, op.b, op.off, op.col, op.factors, op.diag, op.sweeps, x, y, z, alpha, beta);
      break;
  }
}

double dot(int n, const double* a, const double* b) {
  double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (int k = 0; k < n; ++k) s = s + a[k] * b[k];
  return s;
}

}  // namespace

namespace {

// warp_preconditioners/fsai_reuse.py:18-31 (`find`): slot of column j in the
// sorted CSR row i, or -1.
inline int find_slot(const int32_t* off, const int32_t* col, int i, int j) {
  int lo = off[i], hi = off[i + 1];
  const int end = hi;
  while (lo < hi) {
    const int mid = (lo + hi) / 2;
    if (col[mid] < j) lo = mid + 1; else hi = mid;
  }
  return (lo < end && col[lo] == j) ? lo : -1;
}

// warp_preconditioners/fsai_reuse.py:75-149 (`refit`): on each row's fixed
// support, the row-by-row Cholesky of the Jacobi-scaled local matrix, a
// forward and a backward substitution for the unit vector of the row, and
// the normalisation z / sqrt(z_i) * s.  Returns the number of invalid rows
// (pivot <= floor or non-finite, non-finite value, non-positive diagonal).
template <typename T, typename S>
int32_t fsai_refit(int n, const int32_t* off, const int32_t* col, const T* val, const T* scale,
                   const int32_t* goff, const int32_t* gcol, T floor_, S* out) {
  int32_t bad = 0;
#pragma omp parallel for reduction(+ : bad) schedule(dynamic, 64)
  for (int i = 0; i < n; ++i) {
    const int start = goff[i];
    const int size = goff[i + 1] - start;
    if (size < 1) {
      bad += 1;
      continue;
    }
    std::vector<T> chol((size_t)size * size, T(0)), z(size, T(0));
    bool valid = true;
    for (int p = 0; p < size; ++p) {
      const int r = gcol[start + p];
      for (int q = 0; q <= p; ++q) {
        const int c = gcol[start + q];
        const int slot = find_slot(off, col, r, c);
        T a = T(0);
        if (slot >= 0) a = val[slot] * scale[r] * scale[c];
        for (int k = 0; k < q; ++k) a -= chol[(size_t)p * size + k] * chol[(size_t)q * size + k];
        if (p == q) {
          if (a <= floor_ || !finite(a)) {
            valid = false;
            a = T(1);
          }
          chol[(size_t)p * size + q] = std::sqrt(a);
        } else {
          chol[(size_t)p * size + q] = a / chol[(size_t)q * size + q];
        }
      }
    }
    for (int p = 0; p < size; ++p) {
      T a = (gcol[start + p] == i) ? T(1) : T(0);
      for (int q = 0; q < p; ++q) a -= chol[(size_t)p * size + q] * z[q];
      z[p] = a / chol[(size_t)p * size + p];
    }
    for (int rev = 0; rev < size; ++rev) {
      const int p = size - 1 - rev;
      T a = z[p];
      for (int q = p + 1; q < size; ++q) a -= chol[(size_t)q * size + p] * z[q];
      z[p] = a / chol[(size_t)p * size + p];
    }
    const T norm = std::sqrt(z[size - 1]);
    for (int p = 0; p < size; ++p) {
      const S value = S(z[p] / norm * scale[gcol[start + p]]);
      out[start + p] = value;
      if (!finite(value)) valid = false;
      if (p == size - 1 && value <= S(0)) valid = false;
    }
    if (!valid) bad += 1;
  }
  return bad;
}

}  // namespace

namespace {

// SciPy's csr_matmat (scipy/sparse/sparsetools/csr.h) as used by the
// reference's host assembly K @ diags(d) @ K + diags(e).  csr_matmat emits
// each row in reverse insertion order (a linked list of touched columns), so
// the intermediate K diags(d) holds row i in decreasing column order and the
// second product accumulates the contributions A_ij d_j B_jk into C_ik over
// j DEcreasing, from zero (without d, A @ B walks sorted A rows: j
// increasing); then e_i is added to the diagonal; exact zeros are dropped
// and rows sorted.
// Returns nnz; with c_col == nullptr only c_off is filled.
int64_t spgemm(int nrow, int ncol, const int32_t* a_off, const int32_t* a_col, const double* a_val,
               const double* d, const int32_t* b_off, const int32_t* b_col, const double* b_val,
               const double* e, int32_t* c_off, int32_t* c_col, double* c_val) {
  std::vector<double> sums(ncol, 0.0);
  std::vector<char> used(ncol, 0);
  std::vector<int> cols;
  int64_t nnz = 0;
  c_off[0] = 0;
  for (int i = 0; i < nrow; ++i) {
    cols.clear();
    const int len = a_off[i + 1] - a_off[i];
    for (int t = 0; t < len; ++t) {
      const int jj = d ? a_off[i + 1] - 1 - t : a_off[i] + t;
      const int j = a_col[jj];
      const double v = d ? a_val[jj] * d[j] : a_val[jj];
      for (int kk = b_off[j]; kk < b_off[j + 1]; ++kk) {
        const int k = b_col[kk];
        if (!used[k]) {
          used[k] = 1;
          cols.push_back(k);
        }
        sums[k] += v * b_val[kk];
      }
    }
    if (e) {
      if (!used[i]) {
        used[i] = 1;
        cols.push_back(i);
      }
      sums[i] += e[i];
    }
    std::sort(cols.begin(), cols.end());
    for (int k : cols) {
      if (sums[k] != 0.0) {
        if (c_col) {
          c_col[nnz] = k;
          c_val[nnz] = sums[k];
        }
        ++nnz;
      }
      sums[k] = 0.0;
      used[k] = 0;
    }
    c_off[i + 1] = (int32_t)nnz;
  }
  return nnz;
}

}  // namespace

extern "C" {

int or_num_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void or_set_num_threads(int t) {
#ifdef _OPENMP
  if (t > 0) omp_set_num_threads(t);
#else
  (void)t;
#endif
}

void or_fsai_setup_f64(int n, const int32_t* off, const int32_t* col, const double* val,
                       int width, int step, double tol, double floor_, int32_t* cols_out,
                       double* vals_out, double* scale, int32_t* status) {
  fsai_setup<double>(n, off, col, val, width, step, tol, floor_, cols_out, vals_out, scale, status);
}
void or_fsai_setup_rows_f64(int n, const int32_t* off, const int32_t* col, const double* val,
                            int width, int step, double tol, double floor_, int nrows,
                            const int32_t* rows, int32_t* cols_out, double* vals_out,
                            int32_t* status) {
  fsai_setup_rows<double>(n, off, col, val, width, step, tol, floor_, nrows, rows, cols_out,
                          vals_out, status);
}
// FSAI setup that also counts its floating-point operations.
int64_t or_fsai_setup_flops_f64(int n, const int32_t* off, const int32_t* col, const double* val,
                                int width, int step, double tol, double floor_, int32_t* cols_out,
                                double* vals_out, double* scale, int32_t* status) {
  int64_t flops = 0;
  fsai_setup<double, true>(n, off, col, val, width, step, tol, floor_, cols_out, vals_out, scale,
                           status, &flops);
  return flops;
}
void or_fsai_setup_f32(int n, const int32_t* off, const int32_t* col, const float* val, int width,
                       int step, float tol, float floor_, int32_t* cols_out, float* vals_out,
                       float* scale, int32_t* status) {
  fsai_setup<float>(n, off, col, val, width, step, tol, floor_, cols_out, vals_out, scale, status);
}
int64_t or_fsai_pack_f64(int n, int width, int32_t* ell_cols, double* ell_vals, int32_t* g_off,
                         int32_t* g_col, double* g_val) {
  return fsai_pack<double>(n, width, ell_cols, ell_vals, g_off, g_col, g_val);
}
int64_t or_fsai_pack_f32(int n, int width, int32_t* ell_cols, float* ell_vals, int32_t* g_off,
                         int32_t* g_col, float* g_val) {
  return fsai_pack<float>(n, width, ell_cols, ell_vals, g_off, g_col, g_val);
}
void or_csr_transpose_f64(int nrow, int ncol, const int32_t* off, const int32_t* col,
                          const double* val, int32_t* t_off, int32_t* t_col, double* t_val) {
  csr_transpose<double>(nrow, ncol, off, col, val, t_off, t_col, t_val);
}
void or_csr_transpose_f32(int nrow, int ncol, const int32_t* off, const int32_t* col,
                          const float* val, int32_t* t_off, int32_t* t_col, float* t_val) {
  csr_transpose<float>(nrow, ncol, off, col, val, t_off, t_col, t_val);
}
void or_scalarize_f64(int nrow_blocks, int b, const int32_t* off, const int32_t* col,
                      const double* val, int32_t* out_off, int32_t* out_col, double* out_val) {
  scalarize<double>(nrow_blocks, b, off, col, val, out_off, out_col, out_val);
}
void or_scalarize_f32(int nrow_blocks, int b, const int32_t* off, const int32_t* col,
                      const float* val, int32_t* out_off, int32_t* out_col, float* out_val) {
  scalarize<float>(nrow_blocks, b, off, col, val, out_off, out_col, out_val);
}
void or_csr_spmv_f64(int n, const int32_t* off, const int32_t* col, const double* val,
                     const double* x, const double* y, double* z, double alpha, double beta) {
  csr_spmv<double, double>(n, off, col, val, x, y, z, alpha, beta);
}
void or_csr_spmv_f32(int n, const int32_t* off, const int32_t* col, const float* val,
                     const float* x, const float* y, float* z, float alpha, float beta) {
  csr_spmv<float, float>(n, off, col, val, x, y, z, alpha, beta);
}
void or_csr_spmv_f32s_f64a(int n, const int32_t* off, const int32_t* col, const float* val,
                           const double* x, const double* y, double* z, double alpha,
                           double beta) {
  csr_spmv<float, double>(n, off, col, val, x, y, z, alpha, beta);
}
void or_bsr_spmv_f64(int nrow, int b, const int32_t* off, const int32_t* col, const double* val,
                     const double* x, const double* y, double* z, double alpha, double beta) {
  bsr_spmv<double, double>(nrow, b, off, col, val, x, y, z, alpha, beta);
}
void or_bsr_spmv_f32s_f64a(int nrow, int b, const int32_t* off, const int32_t* col,
                           const float* val, const double* x, const double* y, double* z,
                           double alpha, double beta) {
  bsr_spmv<float, double>(nrow, b, off, col, val, x, y, z, alpha, beta);
}
void or_sqlap_apply_f64(int n, const int32_t* off, const int32_t* col, const double* val,
                        const double* inverse_mass, const double* mass, const int32_t* free_,
                        int nfree, const int32_t* index, double mass_weight, const double* x,
                        const double* y, double* z, double alpha, double beta, int boundary,
                        double* tmp) {
  sqlap_apply<double>(n, off, col, val, inverse_mass, mass, free_, nfree, index, mass_weight, x, y,
                      z, alpha, beta, boundary != 0, tmp);
}
void or_sqlap_apply_f32(int n, const int32_t* off, const int32_t* col, const float* val,
                        const float* inverse_mass, const float* mass, const int32_t* free_,
                        int nfree, const int32_t* index, float mass_weight, const float* x,
                        const float* y, float* z, float alpha, float beta, int boundary,
                        float* tmp) {
  sqlap_apply<float>(n, off, col, val, inverse_mass, mass, free_, nfree, index, mass_weight, x, y,
                     z, alpha, beta, boundary != 0, tmp);
}
int or_block_diag_inverse_f64(int nrow, int b, const int32_t* off, const int32_t* col,
                              const double* val, double tol, double* inverse) {
  return block_diag_inverse<double>(nrow, b, off, col, val, tol, inverse);
}
int or_block_diag_inverse_f32(int nrow, int b, const int32_t* off, const int32_t* col,
                              const float* val, float tol, float* inverse) {
  return block_diag_inverse<float>(nrow, b, off, col, val, tol, inverse);
}
int or_bilu0_setup_f64(int nrow, int b, const int32_t* off, const int32_t* col, const double* val,
                       int factor_sweeps, double relaxation, double tol, double* factors,
                       double* inverse) {
  return bilu0_setup<double>(nrow, b, off, col, val, factor_sweeps, relaxation, tol, factors, inverse);
}
int or_bilu0_setup_f32(int nrow, int b, const int32_t* off, const int32_t* col, const float* val,
                       int factor_sweeps, float relaxation, float tol, float* factors,
                       float* inverse) {
  return bilu0_setup<float>(nrow, b, off, col, val, factor_sweeps, relaxation, tol, factors, inverse);
}
void or_bilu0_apply_f64(int nrow, int b, const int32_t* off, const int32_t* col,
                        const double* factors, const double* inverse, int solve_sweeps,
                        const double* x, const double* y, double* z, double alpha, double beta) {
  bilu0_apply<double>(nrow, b, off, col, factors, inverse, solve_sweeps, x, y, z, alpha, beta);
}
void or_bilu0_apply_f32(int nrow, int b, const int32_t* off, const int32_t* col,
                        const float* factors, const float* inverse, int solve_sweeps,
                        const float* x, const float* y, float* z, float alpha, float beta) {
  bilu0_apply<float>(nrow, b, off, col, factors, inverse, solve_sweeps, x, y, z, alpha, beta);
}
void or_block_jacobi_apply_f64(int nrow, int b, const double* inverse, const double* x,
                               const double* y, double* z, double alpha, double beta) {
  block_jacobi_apply<double>(nrow, b, inverse, x, y, z, alpha, beta);
}
int or_block_fsai_setup_f64(int nrow, int b, int max_blocks, const int32_t* off,
                            const int32_t* col, const double* val, int32_t* cols_out,
                            double* vals_out, double* scale, int refit) {
  return block_fsai_setup<double>(nrow, b, max_blocks, off, col, val, cols_out, vals_out, scale,
                                  refit != 0);
}

// Preconditioned CG (method 0) or CR (method 1) on float64 vectors.
// Returns the iteration count; *out_rr receives the final recursive r.r and
// *out_atol_sq the squared absolute threshold.
int or_krylov_f64(int method, const Operator* A, const Operator* M, const double* b, double* x,
                  double tol, double atol, int maxiter, double* out_rr, double* out_atol_sq) {
  const int n = A->n;
  std::vector<double> r(n), z(n), p(n), Ap(n), tmpA, tmpM, Az, y;
  op_apply(*A, x, b, r.data(), -1.0, 1.0, tmpA);  // r = b - A x
  const double bb = dot(n, b, b);
  const double atol_eff = std::max(atol, tol * std::sqrt(bb));
  const double atol_sq = atol_eff * atol_eff;
  *out_atol_sq = atol_sq;
  double rr = dot(n, r.data(), r.data());
  const bool has_m = M != nullptr && M->kind != 0;
  auto precondition = [&](const double* in, double* out) {
    if (has_m) op_apply(*M, in, out, out, 1.0, 0.0, tmpM);
    else std::memcpy(out, in, sizeof(double) * n);
  };
  int it = 0;
  if (method == 0) {
    precondition(r.data(), z.data());
    double rz = dot(n, r.data(), z.data());
    p = z;
    while (it < maxiter && rr > atol_sq) {
      op_apply(*A, p.data(), Ap.data(), Ap.data(), 1.0, 0.0, tmpA);
      const double pAp = dot(n, p.data(), Ap.data());
      const double alpha = rz / pAp;
#pragma omp parallel for schedule(static)
      for (int k = 0; k < n; ++k) {
        x[k] = x[k] + alpha * p[k];
        r[k] = r[k] - alpha * Ap[k];
      }
      precondition(r.data(), z.data());
      const double rz_new = dot(n, r.data(), z.data());
      rr = dot(n, r.data(), r.data());
      const double beta = rz_new / rz;
      rz = rz_new;
#pragma omp parallel for schedule(static)
      for (int k = 0; k < n; ++k) p[k] = z[k] + beta * p[k];
      ++it;
    }
  } else {
    Az.resize(n);
    y.resize(n);
    precondition(r.data(), z.data());
    op_apply(*A, z.data(), Az.data(), Az.data(), 1.0, 0.0, tmpA);
    p = z;
    Ap = Az;
    double zAz = dot(n, z.data(), Az.data());
    while (it < maxiter && rr > atol_sq) {
      precondition(Ap.data(), y.data());
      const double yAp = dot(n, Ap.data(), y.data());
      const double alpha = zAz / yAp;
#pragma omp parallel for schedule(static)
      for (int k = 0; k < n; ++k) {
        x[k] = x[k] + alpha * p[k];
        r[k] = r[k] - alpha * Ap[k];
        z[k] = z[k] - alpha * y[k];
      }
      op_apply(*A, z.data(), Az.data(), Az.data(), 1.0, 0.0, tmpA);
      const double zAz_new = dot(n, z.data(), Az.data());
      rr = dot(n, r.data(), r.data());
      const double beta = zAz_new / zAz;
      zAz = zAz_new;
#pragma omp parallel for schedule(static)
      for (int k = 0; k < n; ++k) {
        p[k] = z[k] + beta * p[k];
        Ap[k] = Az[k] + beta * Ap[k];
      }
      ++it;
    }
  }
  *out_rr = rr;
  return it;
}

int or_operator_size() { return (int)sizeof(Operator); }

void or_operator_apply(const Operator* op, const double* x, const double* y, double* z,
                       double alpha, double beta) {
  std::vector<double> tmp;
  op_apply(*op, x, y, z, alpha, beta, tmp);
}


void or_fsai_diagonal_f64(int n, const int32_t* off, const int32_t* col, const double* val,
                          double* scale, int32_t* status) {
  fsai_diagonal<double>(n, off, col, val, scale, status);
}
void or_fsai_diagonal_f32(int n, const int32_t* off, const int32_t* col, const float* val,
                          float* scale, int32_t* status) {
  fsai_diagonal<float>(n, off, col, val, scale, status);
}
int32_t or_fsai_refit_f64_f64(int n, const int32_t* off, const int32_t* col, const double* val,
                              const double* scale, const int32_t* goff, const int32_t* gcol,
                              double floor_, double* out) {
  return fsai_refit<double, double>(n, off, col, val, scale, goff, gcol, floor_, out);
}
int32_t or_fsai_refit_f64_f32(int n, const int32_t* off, const int32_t* col, const double* val,
                              const double* scale, const int32_t* goff, const int32_t* gcol,
                              double floor_, float* out) {
  return fsai_refit<double, float>(n, off, col, val, scale, goff, gcol, floor_, out);
}
int32_t or_fsai_refit_f32_f32(int n, const int32_t* off, const int32_t* col, const float* val,
                              const float* scale, const int32_t* goff, const int32_t* gcol,
                              float floor_, float* out) {
  return fsai_refit<float, float>(n, off, col, val, scale, goff, gcol, floor_, out);
}
int64_t or_spgemm(int nrow, int ncol, const int32_t* a_off, const int32_t* a_col,
                  const double* a_val, const double* d, const int32_t* b_off,
                  const int32_t* b_col, const double* b_val, const double* e, int32_t* c_off,
                  int32_t* c_col, double* c_val) {
  return spgemm(nrow, ncol, a_off, a_col, a_val, d, b_off, b_col, b_val, e, c_off, c_col, c_val);
}
}  // extern "C"
