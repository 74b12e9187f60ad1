// Linear operators behind the C ABI: sparse products, FSAI G^T G, the
// factored squared Laplacian, scalar Jacobi, block Jacobi, block ILU(0).
//
// Every operator keeps its matrices in SELL-32 (gbpc_sell.cu) and applies
// z = alpha * Op * x + beta * y with the reference's conventions (aliasing
// allowed, beta == 0 never reads y, alpha == 0 never reads x).  The last
// kernel of each apply can fuse a dot product with its output, which the
// Krylov loops use to avoid separate reduction launches.

#include <algorithm>
#include <cmath>
#include <vector>

#include "gbpc_common.cuh"
#include "gbpc_internal.h"

namespace gbpc {

int block_diag_inverse(int nrow, int b, const int32_t* off, const int32_t* col, const void* val,
                       int dtype, double tol, void* inverse, int32_t* bad_host, cudaStream_t st);
int bilu0_setup(int nrow, int b, const int32_t* off, const int32_t* col, const void* val,
                int dtype, int64_t nnz, int factor_sweeps, double relaxation, double tol,
                void* factors, void* inverse, int32_t* bad_host, cudaStream_t st);

namespace {

// ---------------------------------------------------------------------------
// Elementwise kernels.

// z = alpha * (d .* x) + beta * y   (d == nullptr: d = 1), optional dot(w, z).
// UNIT: alpha == 1 and beta == 0 known at compile time (1 * t == t).
template <typename A, bool UNIT = false>
__global__ void __launch_bounds__(kThreads, kCtasPerSm)
scale_axpby_kernel(int64_t n, const A* d, const A* x, const A* y, A* z, A alpha, A beta,
                   const int* guard, Reduction red) {
  if (guard_off(guard)) return;
  double part = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kThreads) {
    A v = A(0);
    if (UNIT) v = d ? d[i] * x[i] : x[i];
    else if (alpha != A(0)) v = alpha * (d ? d[i] * x[i] : x[i]);
    if (!UNIT && beta != A(0)) v = v + beta * y[i];
    z[i] = v;
    if (red.w) part = fma((double)v, red.w[i], part);
  }
  if (red.w) reduce_and_finalize(red, part);
}

// Block diagonal apply: z_i = alpha * inv_i x_i + beta y_i (block_ilu.py:188-202).
// UNIT: alpha == 1 and beta == 0 known at compile time (inside the Krylov
// loops), so neither the scaling (1 * s == s) nor the y term is issued.
template <typename A, int B, bool UNIT = false>
__global__ void __launch_bounds__(kThreads, kCtasPerSm)
block_diag_apply_kernel(int nrow, const A* __restrict__ inv, const A* x, const A* y, A* z, A alpha,
                        A beta, const int* guard, Reduction red) {
  if constexpr (UNIT) {
    alpha = A(1);
    beta = A(0);
  }
  if (guard_off(guard)) return;
  double part = 0.0;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < nrow; i += gridDim.x * kThreads) {
    A xi[B], v[B];
#pragma unroll
    for (int q = 0; q < B; ++q) {
      xi[q] = (alpha != A(0)) ? x[(int64_t)i * B + q] : A(0);
      v[q] = A(0);
    }
    if (alpha != A(0)) {
#pragma unroll
      for (int r = 0; r < B; ++r) {
        A s = A(0);
#pragma unroll
        for (int q = 0; q < B; ++q) s = fma(inv[(int64_t)i * B * B + r * B + q], xi[q], s);
        v[r] = UNIT ? s : alpha * s;
      }
    }
#pragma unroll
    for (int r = 0; r < B; ++r) {
      const int64_t idx = (int64_t)i * B + r;
      if (beta != A(0)) v[r] = v[r] + beta * y[idx];
      z[idx] = v[r];
      if (red.w) part = fma((double)v[r], red.w[idx], part);
    }
  }
  if (red.w) reduce_and_finalize(red, part);
}

// squared_laplacian.py:11-35: free -> compact index with duplicate detection,
// and 1/mass with validity.
__global__ void index_free_kernel(int nfree, const int32_t* __restrict__ free_idx, int n,
                                  int32_t* index, int32_t* status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nfree) return;
  const int j = free_idx[i];
  if (j != i) atomicAdd(status + 3, 1);  // not the identity selection
  if (j < 0 || j >= n) {
    atomicAdd(status + 0, 1);
  } else {
    const int old = atomicCAS(index + j, -1, i);
    if (old != -1) atomicAdd(status + 1, 1);
  }
}

template <typename T>
__global__ void mass_inverse_kernel(int n, const T* __restrict__ mass, T* inverse, int32_t* status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const T m = mass[i];
  if (m > T(0) && isfinite(m)) {
    inverse[i] = T(1) / m;
  } else {
    inverse[i] = T(0);
    atomicAdd(status + 2, 1);
  }
}

template <typename T>
__global__ void gather_scaled_kernel(int nfree, const int32_t* __restrict__ free_idx,
                                     const T* __restrict__ mass, T weight, T* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nfree) return;
  out[i] = weight * mass[free_idx[i]];
}

// Boundary column map: c -> c when c is constrained (index[c] < 0), else -1.
__global__ void boundary_map_kernel(int n, const int32_t* __restrict__ index, int32_t* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = (index[i] < 0) ? i : -1;
}

// Scalar diagonal of a BSR matrix and its inverse (zero diagonal -> 1).
template <typename T>
__global__ void scalar_diag_kernel(int nrow, int b, const int32_t* __restrict__ off,
                                   const int32_t* __restrict__ col, const T* __restrict__ val,
                                   double* inv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrow) return;
  double d[4] = {0.0, 0.0, 0.0, 0.0};
  for (int e = off[i]; e < off[i + 1]; ++e)
    if (col[e] == i)
      for (int r = 0; r < b; ++r) d[r] = (double)val[(int64_t)e * b * b + r * b + r];
  for (int r = 0; r < b; ++r) inv[(int64_t)i * b + r] = (d[r] != 0.0) ? 1.0 / d[r] : 1.0;
}

template <typename A>
__global__ void to_vector_dtype_kernel(int64_t n, const double* in, A* out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (A)in[i];
}

int elementwise_grid(int64_t n) { return std::min<int64_t>(grid_for(n, kThreads), kSms * kCtasPerSm); }

Reduction make_reduction(const DotSpec* dot) {
  Reduction red{};
  if (dot != nullptr && dot->w != nullptr) {
    red.w = dot->w;
    red.partials = dot->rb->partials.as<double>();
    red.counter = dot->rb->counter.as<unsigned int>();
    red.mode = dot->mode;
    red.ks = (KrylovScalars*)dot->ks;
    red.out = dot->out;
  }
  return red;
}

int scale_axpby(int vdtype, int64_t n, const void* d, const void* x, const void* y, void* z,
                double alpha, double beta, const int* guard, const DotSpec* dot, cudaStream_t st) {
  const Reduction red = make_reduction(dot);
  if (vdtype == GBPC_F64 && alpha == 1.0 && beta == 0.0)
    scale_axpby_kernel<double, true><<<elementwise_grid(n), kThreads, 0, st>>>(
        n, (const double*)d, (const double*)x, (const double*)y, (double*)z, alpha, beta, guard, red);
  else if (vdtype == GBPC_F64)
    scale_axpby_kernel<double><<<elementwise_grid(n), kThreads, 0, st>>>(
        n, (const double*)d, (const double*)x, (const double*)y, (double*)z, alpha, beta, guard, red);
  else
    scale_axpby_kernel<float><<<elementwise_grid(n), kThreads, 0, st>>>(
        n, (const float*)d, (const float*)x, (const float*)y, (float*)z, (float)alpha, (float)beta,
        guard, red);
  GBPC_CUDA_TRY(cudaGetLastError());
  return GBPC_OK;
}

// Float32 preconditioner behind a float64 interface (LowPrecisionOp).
// out = (float) x, guarded like the products.
__global__ void __launch_bounds__(kThreads, kCtasPerSm)
narrow_kernel(int64_t n, const double* __restrict__ x, float* __restrict__ out, const int* guard) {
  pdl_wait();
  pdl_launch_dependents();
  if (guard_off(guard)) return;
  for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kThreads)
    out[i] = (float)x[i];
}

// z = alpha * (double) v + beta * y (beta == 0 never reads y), with the
// fused dot(w, z) in float64.
template <bool UNIT>
__global__ void __launch_bounds__(kThreads, kCtasPerSm)
widen_axpby_kernel(int64_t n, const float* __restrict__ v, const double* y, double* z,
                   double alpha, double beta, int beta_zero, const int* guard, Reduction red) {
  pdl_wait();
  pdl_launch_dependents();
  if (guard_off(guard)) return;
  double part = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kThreads) {
    double o = (double)v[i];
    if (!UNIT) {
      o = alpha * o;
      if (!beta_zero) o = fma(beta, y[i], o);
    }
    z[i] = o;
    if (red.w) part = fma(o, red.w[i], part);
  }
  if (red.w) reduce_and_finalize(red, part);
}

// ---------------------------------------------------------------------------
// Operators.

struct SparseOp : Operator {
  Sell m;
  int apply(const void* x, const void* y, void* z, double alpha, double beta, const int* guard,
            const DotSpec* dot, cudaStream_t st) override {
    return sell_spmv(m, vdtype, x, y, z, alpha, beta, guard, EpiHost{}, dot, st);
  }
  int scalar_products(const Sell** out, int max) const override {
    if (max < 1 || m.B != 1 || m.vdtype != GBPC_F64 || vdtype != GBPC_F64) return 0;
    out[0] = &m;
    return 1;
  }
};

struct FsaiOp : Operator {
  Sell g, gt;
  DevBuf tmp;
  int apply(const void* x, const void* y, void* z, double alpha, double beta, const int* guard,
            const DotSpec* dot, cudaStream_t st) override {
    int rc;
    // x is fully consumed into tmp before z is written, so x, y, z may alias.
    if (alpha != 0.0) {
      rc = sell_spmv(g, vdtype, x, nullptr, tmp.p, 1.0, 0.0, guard, EpiHost{}, nullptr, st);
      if (rc) return rc;
    }
    return sell_spmv(gt, vdtype, tmp.p, y, z, alpha, beta, guard, EpiHost{}, dot, st);
  }
  bool gathers_x() const override { return false; }
  int scalar_products(const Sell** out, int max) const override {
    if (max < 2 || g.B != 1 || g.vdtype != GBPC_F64 || gt.vdtype != GBPC_F64 ||
        vdtype != GBPC_F64)
      return 0;
    out[0] = &g;
    out[1] = &gt;
    return 2;
  }
};

struct SqlapOp : Operator {
  int n = 0, nfree = 0;
  // free_indices == 0, 1, ..., n - 1: L[free, :] is L itself and compact
  // column indices are L's, so one stored copy of L serves both products.
  bool identity_free = false;
  Sell fwd;       // L with columns mapped to compact free indices (not built when identity_free)
  Sell bwd;       // rows L[free, :]
  Sell bnd;       // L with only constrained columns (rhs)
  DevBuf inv_mass, wmass, tmp, index, free_idx, zeros;
  int apply(const void* x, const void* y, void* z, double alpha, double beta, const int* guard,
            const DotSpec* dot, cudaStream_t st) override {
    int rc;
    if (alpha != 0.0) {
      // tmp = (M^-1 L) x.  It walks its slices in reverse so that the
      // backward product, which walks L forward, starts on the slices read
      // last (with one copy of L they are still in L2), and the next
      // forward product starts on the slices the backward one read last.
      EpiHost f;
      f.reverse = true;
      if (identity_free) {
        // tmp[i] = (1 / mass[i]) * (L x)[i], the reference's order
        // (squared_laplacian.py:37-64).
        f.kind = EPI_SQLAP_FWD;
        f.aux0 = inv_mass.p;
        rc = sell_spmv(bwd, vdtype, x, nullptr, tmp.p, 1.0, 0.0, guard, f, nullptr, st);
      } else {
        // The row scaling is folded into fwd's stored values.
        rc = sell_spmv(fwd, vdtype, x, nullptr, tmp.p, 1.0, 0.0, guard, f, nullptr, st);
      }
      if (rc) return rc;
    }
    EpiHost b{EPI_SQLAP_BWD, wmass.p, x};
    return sell_spmv(bwd, vdtype, tmp.p, y, z, alpha, beta, guard, b, dot, st);
  }
  bool gathers_x() const override { return false; }
  bool factored_parts(const Sell** L, const void** im, const void** wm) const override {
    if (!identity_free || vdtype != GBPC_F64 || bwd.B != 1 || bwd.vdtype != GBPC_F64) return false;
    *L = &bwd;
    *im = inv_mass.p;
    *wm = wmass.p;
    return true;
  }
  int rhs(const void* u, void* out, cudaStream_t st) {
    int rc = sell_spmv(bnd, vdtype, u, nullptr, tmp.p, 1.0, 0.0, nullptr, EpiHost{}, nullptr, st);
    if (rc) return rc;
    EpiHost b{EPI_SQLAP_BWD, zeros.p, zeros.p};
    return sell_spmv(bwd, vdtype, tmp.p, nullptr, out, -1.0, 0.0, nullptr, b, nullptr, st);
  }
};

struct DiagOp : Operator {
  DevBuf inv;  // vector dtype
  int apply(const void* x, const void* y, void* z, double alpha, double beta, const int* guard,
            const DotSpec* dot, cudaStream_t st) override {
    return scale_axpby(vdtype, rows, inv.p, x, y, z, alpha, beta, guard, dot, st);
  }
  bool gathers_x() const override { return false; }
};

struct BlockJacobiOp : Operator {
  int nrow = 0, B = 1;
  DevBuf inv;  // [nrow][B][B], vector dtype
  int apply(const void* x, const void* y, void* z, double alpha, double beta, const int* guard,
            const DotSpec* dot, cudaStream_t st) override {
    const Reduction red = make_reduction(dot);
    const int g = elementwise_grid(nrow);
    const bool unit = alpha == 1.0 && beta == 0.0;
#define GBPC_BJ(Bv)                                                                            \
  if (vdtype == GBPC_F64 && unit)                                                              \
    block_diag_apply_kernel<double, Bv, true><<<g, kThreads, 0, st>>>(                         \
        nrow, inv.as<double>(), (const double*)x, (const double*)y, (double*)z, alpha, beta,    \
        guard, red);                                                                           \
  else if (vdtype == GBPC_F64)                                                                 \
    block_diag_apply_kernel<double, Bv><<<g, kThreads, 0, st>>>(                               \
        nrow, inv.as<double>(), (const double*)x, (const double*)y, (double*)z, alpha, beta,    \
        guard, red);                                                                           \
  else                                                                                         \
    block_diag_apply_kernel<float, Bv><<<g, kThreads, 0, st>>>(                                \
        nrow, inv.as<float>(), (const float*)x, (const float*)y, (float*)z, (float)alpha,       \
        (float)beta, guard, red);
    switch (B) {
      case 1: GBPC_BJ(1) break;
      case 2: GBPC_BJ(2) break;
      case 3: GBPC_BJ(3) break;
      case 4: GBPC_BJ(4) break;
    }
#undef GBPC_BJ
    GBPC_CUDA_TRY(cudaGetLastError());
    return GBPC_OK;
  }
  bool gathers_x() const override { return false; }
};

struct Bilu0Op : Operator {
  int nrow = 0, B = 1, sweeps = 1;
  Sell lower, upper;
  DevBuf inv;         // [nrow][B][B], vector dtype
  DevBuf buf[4];      // a, b, c, d
  int apply(const void* x, const void* y, void* z, double alpha, double beta, const int* guard,
            const DotSpec* dot, cudaStream_t st) override {
    // alpha == 0 takes the block-diagonal path of the reference, z = beta * y
    // (block_ilu.py:404-406).
    if (alpha == 0.0) return scale_axpby(vdtype, rows, nullptr, x, y, z, 0.0, beta, guard, dot, st);
    const size_t bytes = dtype_size(vdtype) * rows;
    void* a = buf[0].p;
    void* b = buf[1].p;
    GBPC_CUDA_TRY(cudaMemsetAsync(a, 0, bytes, st));
    int rc;
    for (int s = 0; s < sweeps; ++s) {
      EpiHost e{EPI_TRI_LOWER, x, nullptr};
      if ((rc = sell_spmv(lower, vdtype, a, nullptr, b, 1.0, 0.0, guard, e, nullptr, st))) return rc;
      std::swap(a, b);
    }
    void* c = buf[2].p;
    void* d = buf[3].p;
    GBPC_CUDA_TRY(cudaMemsetAsync(c, 0, bytes, st));
    for (int s = 0; s < sweeps; ++s) {
      EpiHost e{EPI_TRI_UPPER, a, inv.p};
      if ((rc = sell_spmv(upper, vdtype, c, nullptr, d, 1.0, 0.0, guard, e, nullptr, st))) return rc;
      std::swap(c, d);
    }
    return scale_axpby(vdtype, rows, nullptr, c, y, z, alpha, beta, guard, dot, st);
  }
  bool gathers_x() const override { return false; }
};

}  // namespace

int LowPrecisionOp::apply(const void* x, const void* y, void* z, double alpha, double beta,
                          const int* guard, const DotSpec* dot, cudaStream_t st) {
  // alpha == 0: z = beta * y without reading x (the operator contract).
  if (alpha == 0.0) return scale_axpby(GBPC_F64, rows, nullptr, x, y, z, 0.0, beta, guard, dot, st);
  const int g = elementwise_grid(rows);
  // x is consumed into in32 before z is written, so x, y, z may alias.
  GBPC_CUDA_TRY(launch_k(narrow_kernel, g, kThreads, 0, st, rows, (const double*)x,
                         in32.as<float>(), guard));
  int rc = inner->apply(in32.p, nullptr, out32.p, 1.0, 0.0, guard, nullptr, st);
  if (rc) return rc;
  const Reduction red = make_reduction(dot);
  const bool unit = alpha == 1.0 && beta == 0.0;
  if (unit)
    GBPC_CUDA_TRY(launch_k(widen_axpby_kernel<true>, g, kThreads, 0, st, rows,
                           (const float*)out32.as<float>(), (const double*)y, (double*)z, alpha,
                           beta, 1, guard, red));
  else
    GBPC_CUDA_TRY(launch_k(widen_axpby_kernel<false>, g, kThreads, 0, st, rows,
                           (const float*)out32.as<float>(), (const double*)y, (double*)z, alpha,
                           beta, (int)(beta == 0.0), guard, red));
  return GBPC_OK;
}

namespace {

int check_dtypes(int value_dtype, int vector_dtype) {
  if (!valid_value_dtype(value_dtype)) {
    gbpc_set_error("value dtype must be float64, float32 or bfloat16");
    return GBPC_ERR_ARG;
  }
  if (vector_dtype != GBPC_F64 && vector_dtype != GBPC_F32) {
    gbpc_set_error("vector dtype must be float64 or float32");
    return GBPC_ERR_ARG;
  }
  if (value_dtype == GBPC_F64 && vector_dtype == GBPC_F32) {
    gbpc_set_error("float64 storage needs float64 vectors");
    return GBPC_ERR_ARG;
  }
  return GBPC_OK;
}

// Input arrays are passed in their storage dtype.
int input_dtype(int value_dtype) { return value_dtype; }

}  // namespace
}  // namespace gbpc

using namespace gbpc;

#define GBPC_OUT_OP(op_ptr)                 \
  do {                                      \
    gbpc_op* h = new gbpc_op;               \
    h->impl.reset(op_ptr);                  \
    *out = h;                               \
  } while (0)

extern "C" int gbpc_op_sparse(int nrow, int ncol, int block, const int32_t* offsets,
                              const int32_t* columns, const void* values, int value_dtype,
                              int vector_dtype, void* stream, gbpc_op** out) {
  if (!out || nrow < 0 || ncol < 0 || !offsets) {
    gbpc_set_error("gbpc_op_sparse: bad arguments");
    return GBPC_ERR_ARG;
  }
  if (value_dtype == GBPC_BF16) {
    gbpc_set_error("gbpc_op_sparse: pass float32 or float64 values (bfloat16 is a storage option "
                   "of gbpc_op_fsai)");
    return GBPC_ERR_ARG;
  }
  int rc = check_dtypes(value_dtype, vector_dtype);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  auto* op = new SparseOp;
  ByteTally tally(&op->device_bytes);
  op->rows = (int64_t)nrow * block;
  op->vdtype = vector_dtype;
  rc = sell_build(op->m, nrow, ncol, block, offsets, columns, values, value_dtype, value_dtype,
                  SellBuild{}, st);
  if (!rc) rc = sell_autotune(op->m, vector_dtype, st);
  if (!rc) rc = op->alias_scratch.alloc(dtype_size(vector_dtype) * std::max<int64_t>(op->rows, 1));
  if (rc) {
    delete op;
    return rc;
  }
  cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    delete op;
    gbpc_set_error_cuda(e, "sync", __FILE__, __LINE__);
    return GBPC_ERR_CUDA;
  }
  GBPC_OUT_OP(op);
  return GBPC_OK;
}

extern "C" int gbpc_op_fsai(int nrow, int block, const int32_t* g_off, const int32_t* g_col,
                            const void* g_val, const int32_t* gt_off, const int32_t* gt_col,
                            const void* gt_val, int value_dtype, int vector_dtype, void* stream,
                            gbpc_op** out) {
  NvtxRange nvtx_range("gbpc_op_fsai");
  if (!out || nrow < 0 || !g_off || !gt_off || block < 1 || block > 4) {
    gbpc_set_error("gbpc_op_fsai: bad arguments");
    return GBPC_ERR_ARG;
  }
  const bool low = vector_dtype == GBPC_F32_APPLY;
  if (low && value_dtype != GBPC_F32 && value_dtype != GBPC_BF16) {
    gbpc_set_error("float32 application needs float32 or bfloat16 factor storage");
    return GBPC_ERR_ARG;
  }
  int rc = check_dtypes(value_dtype, low ? GBPC_F32 : vector_dtype);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  if (low) {
    // The float32 operator, wrapped behind float64 vectors.
    gbpc_op* inner = nullptr;
    rc = gbpc_op_fsai(nrow, block, g_off, g_col, g_val, gt_off, gt_col, gt_val, value_dtype,
                      GBPC_F32, stream, &inner);
    if (rc) return rc;
    auto* w = new LowPrecisionOp;
    w->inner = std::move(inner->impl);
    delete inner;
    w->device_bytes = w->inner->device_bytes;
    {
      ByteTally tally(&w->device_bytes);
      w->rows = (int64_t)nrow * block;
      w->vdtype = GBPC_F64;
      rc = w->in32.alloc(sizeof(float) * std::max<int64_t>(w->rows, 1));
      if (!rc) rc = w->out32.alloc(sizeof(float) * std::max<int64_t>(w->rows, 1));
    }
    if (rc) {
      delete w;
      return rc;
    }
    GBPC_OUT_OP(w);
    return GBPC_OK;
  }
  auto* op = new FsaiOp;
  ByteTally tally(&op->device_bytes);
  op->rows = (int64_t)nrow * block;
  op->vdtype = vector_dtype;
  const int in = input_dtype(value_dtype);
  rc = sell_build(op->g, nrow, nrow, block, g_off, g_col, g_val, in, value_dtype, SellBuild{}, st);
  if (!rc) rc = sell_build(op->gt, nrow, nrow, block, gt_off, gt_col, gt_val, in, value_dtype, SellBuild{}, st);
  if (!rc) rc = sell_autotune(op->g, vector_dtype, st);
  if (!rc) rc = sell_autotune(op->gt, vector_dtype, st);
  if (!rc) rc = op->tmp.alloc(dtype_size(vector_dtype) * std::max<int64_t>(op->rows, 1));
  if (!rc) {
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      gbpc_set_error_cuda(e, "sync", __FILE__, __LINE__);
      rc = GBPC_ERR_CUDA;
    }
  }
  if (rc) {
    delete op;
    return rc;
  }
  GBPC_OUT_OP(op);
  return GBPC_OK;
}

extern "C" int gbpc_op_fsai_refill(gbpc_op* h, const int32_t* g_off, const int32_t* g_col,
                                   const void* g_val, const int32_t* gt_off,
                                   const int32_t* gt_col, const void* gt_val, int value_dtype,
                                   void* stream) {
  Operator* base = h ? h->impl.get() : nullptr;
  if (auto* low = dynamic_cast<LowPrecisionOp*>(base)) base = low->inner.get();
  auto* op = dynamic_cast<FsaiOp*>(base);
  if (!op || !g_off || !gt_off || !valid_value_dtype(value_dtype)) {
    gbpc_set_error("gbpc_op_fsai_refill: needs an FSAI operator and its factor arrays");
    return GBPC_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const int in = input_dtype(value_dtype);
  int rc = sell_refill(op->g, g_off, g_col, g_val, in, SellBuild{}, st);
  if (!rc) rc = sell_refill(op->gt, gt_off, gt_col, gt_val, in, SellBuild{}, st);
  return rc;
}

extern "C" int gbpc_op_sqlap(int n, const int32_t* offsets, const int32_t* columns,
                             const void* values, int dtype, const void* mass,
                             const int32_t* free_indices, int nfree, double mass_weight,
                             void* stream, gbpc_op** out) {
  NvtxRange nvtx_range("gbpc_op_sqlap");
  if (!out || n < 0 || nfree < 0 || !offsets || (nfree > 0 && !free_indices) || (n > 0 && !mass)) {
    gbpc_set_error("gbpc_op_sqlap: bad arguments");
    return GBPC_ERR_ARG;
  }
  if (dtype != GBPC_F64 && dtype != GBPC_F32) {
    gbpc_set_error("L must use float32 or float64");
    return GBPC_ERR_ARG;
  }
  if (!std::isfinite(mass_weight) || mass_weight < 0) {
    gbpc_set_error("mass_weight must be finite and nonnegative");
    return GBPC_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  auto* op = new SqlapOp;
  ByteTally tally(&op->device_bytes);
  op->rows = nfree;
  op->vdtype = dtype;
  op->n = n;
  op->nfree = nfree;
  const size_t vs = dtype_size(dtype);
  int rc = GBPC_OK;
  DevBuf status, bmap;
  auto fail = [&](int code) {
    delete op;
    return code;
  };
  if ((rc = status.alloc(sizeof(int32_t) * 4))) return fail(rc);
  if ((rc = op->index.alloc(sizeof(int32_t) * std::max(n, 1)))) return fail(rc);
  if ((rc = op->free_idx.alloc(sizeof(int32_t) * std::max(nfree, 1)))) return fail(rc);
  if ((rc = op->inv_mass.alloc(vs * std::max(n, 1)))) return fail(rc);
  if ((rc = op->wmass.alloc(vs * std::max(nfree, 1)))) return fail(rc);
  if ((rc = op->zeros.alloc(vs * std::max(nfree, 1)))) return fail(rc);
  if ((rc = op->tmp.alloc(vs * std::max(n, 1)))) return fail(rc);
  if ((rc = bmap.alloc(sizeof(int32_t) * std::max(n, 1)))) return fail(rc);
  if (cudaMemsetAsync(status.p, 0, sizeof(int32_t) * 4, st) != cudaSuccess ||
      cudaMemsetAsync(op->index.p, 0xff, sizeof(int32_t) * std::max(n, 1), st) != cudaSuccess ||
      cudaMemsetAsync(op->zeros.p, 0, vs * std::max(nfree, 1), st) != cudaSuccess) {
    gbpc_set_error("gbpc_op_sqlap: memset failed");
    return fail(GBPC_ERR_CUDA);
  }
  if (nfree > 0) {
    cudaMemcpyAsync(op->free_idx.p, free_indices, sizeof(int32_t) * nfree, cudaMemcpyDeviceToDevice, st);
    index_free_kernel<<<grid_for(nfree, 256), 256, 0, st>>>(nfree, free_indices, n,
                                                            op->index.as<int32_t>(), status.as<int32_t>());
  }
  if (n > 0) {
    if (dtype == GBPC_F64)
      mass_inverse_kernel<double><<<grid_for(n, 256), 256, 0, st>>>(
          n, (const double*)mass, op->inv_mass.as<double>(), status.as<int32_t>());
    else
      mass_inverse_kernel<float><<<grid_for(n, 256), 256, 0, st>>>(
          n, (const float*)mass, op->inv_mass.as<float>(), status.as<int32_t>());
  }
  int32_t h[4] = {0, 0, 0, 0};
  cudaMemcpyAsync(h, status.p, sizeof(h), cudaMemcpyDeviceToHost, st);
  cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    gbpc_set_error_cuda(e, "sqlap setup", __FILE__, __LINE__);
    return fail(GBPC_ERR_CUDA);
  }
  if (h[0] || h[1]) {
    gbpc_set_error("free_indices must be distinct and in bounds");
    return fail(GBPC_ERR_FREE_INDEX);
  }
  if (h[2]) {
    gbpc_set_error("mass entries must be finite and positive");
    return fail(GBPC_ERR_MASS);
  }
  if (nfree > 0) {
    if (dtype == GBPC_F64)
      gather_scaled_kernel<double><<<grid_for(nfree, 256), 256, 0, st>>>(
          nfree, free_indices, (const double*)mass, mass_weight, op->wmass.as<double>());
    else
      gather_scaled_kernel<float><<<grid_for(nfree, 256), 256, 0, st>>>(
          nfree, free_indices, (const float*)mass, (float)mass_weight, op->wmass.as<float>());
  }
  if (n > 0)
    boundary_map_kernel<<<grid_for(n, 256), 256, 0, st>>>(n, op->index.as<int32_t>(), bmap.as<int32_t>());
  SellBuild fo;
  fo.colmap = op->index.as<int32_t>();
  fo.row_scale = op->inv_mass.p;
  SellBuild bo;
  bo.rows = op->free_idx.as<int32_t>();
  SellBuild bd;
  bd.colmap = bmap.as<int32_t>();
  bd.row_scale = op->inv_mass.p;
  op->identity_free = nfree == n && h[3] == 0;
  if (!op->identity_free &&
      (rc = sell_build(op->fwd, n, nfree, 1, offsets, columns, values, dtype, dtype, fo, st)))
    return fail(rc);
  if ((rc = sell_build(op->bwd, nfree, n, 1, offsets, columns, values, dtype, dtype, bo, st))) return fail(rc);
  if ((rc = sell_build(op->bnd, n, n, 1, offsets, columns, values, dtype, dtype, bd, st))) return fail(rc);
  if (!op->identity_free && (rc = sell_autotune(op->fwd, dtype, st))) return fail(rc);
  if ((rc = sell_autotune(op->bwd, dtype, st))) return fail(rc);
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    gbpc_set_error_cuda(e, "sqlap setup", __FILE__, __LINE__);
    return fail(GBPC_ERR_CUDA);
  }
  GBPC_OUT_OP(op);
  return GBPC_OK;
}

extern "C" int gbpc_sqlap_rhs(gbpc_op* h, const void* boundary_values, void* out, void* stream) {
  if (!h) {
    gbpc_set_error("gbpc_sqlap_rhs: null operator");
    return GBPC_ERR_ARG;
  }
  auto* op = dynamic_cast<SqlapOp*>(h->impl.get());
  if (!op) {
    gbpc_set_error("gbpc_sqlap_rhs: not a squared-Laplacian operator");
    return GBPC_ERR_ARG;
  }
  return op->rhs(boundary_values, out, (cudaStream_t)stream);
}

extern "C" int gbpc_op_diagonal(int nrow, int block, const int32_t* offsets,
                                const int32_t* columns, const void* values, int dtype,
                                void* stream, gbpc_op** out) {
  if (!out || nrow < 0 || block < 1 || block > 4 || (dtype != GBPC_F64 && dtype != GBPC_F32)) {
    gbpc_set_error("gbpc_op_diagonal: bad arguments");
    return GBPC_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  auto* op = new DiagOp;
  ByteTally tally(&op->device_bytes);
  op->rows = (int64_t)nrow * block;
  op->vdtype = dtype;
  DevBuf tmp;
  int rc = tmp.alloc(sizeof(double) * std::max<int64_t>(op->rows, 1));
  if (!rc) rc = op->inv.alloc(dtype_size(dtype) * std::max<int64_t>(op->rows, 1));
  if (rc) {
    delete op;
    return rc;
  }
  if (nrow > 0) {
    if (dtype == GBPC_F64)
      scalar_diag_kernel<double><<<grid_for(nrow, 256), 256, 0, st>>>(
          nrow, block, offsets, columns, (const double*)values, op->inv.as<double>());
    else {
      scalar_diag_kernel<float><<<grid_for(nrow, 256), 256, 0, st>>>(
          nrow, block, offsets, columns, (const float*)values, tmp.as<double>());
      to_vector_dtype_kernel<float><<<grid_for(op->rows, 256), 256, 0, st>>>(
          op->rows, tmp.as<double>(), op->inv.as<float>());
    }
  }
  cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    delete op;
    gbpc_set_error_cuda(e, "diagonal setup", __FILE__, __LINE__);
    return GBPC_ERR_CUDA;
  }
  GBPC_OUT_OP(op);
  return GBPC_OK;
}

extern "C" int gbpc_op_block_jacobi(int nrow, int block, const int32_t* offsets,
                                    const int32_t* columns, const void* values, int dtype,
                                    double pivot_tolerance, void* inverse_out, void* stream,
                                    gbpc_op** out) {
  NvtxRange nvtx_range("gbpc_op_block_jacobi");
  if (!out || nrow < 0 || block < 1 || block > 4 || (dtype != GBPC_F64 && dtype != GBPC_F32)) {
    gbpc_set_error("BlockJacobi requires square blocks of size 1 through 4");
    return GBPC_ERR_ARG;
  }
  if (!std::isfinite(pivot_tolerance) || pivot_tolerance < 0) {
    gbpc_set_error("pivot_tolerance must be finite and nonnegative");
    return GBPC_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  auto* op = new BlockJacobiOp;
  ByteTally tally(&op->device_bytes);
  op->rows = (int64_t)nrow * block;
  op->vdtype = dtype;
  op->nrow = nrow;
  op->B = block;
  int rc = op->inv.alloc(dtype_size(dtype) * std::max<int64_t>((int64_t)nrow * block * block, 1));
  if (rc) {
    delete op;
    return rc;
  }
  int32_t bad = 0;
  rc = block_diag_inverse(nrow, block, offsets, columns, values, dtype, pivot_tolerance, op->inv.p,
                          &bad, st);
  if (!rc && bad) {
    gbpc_set_error("Missing, nonfinite or singular/near-singular block pivot");
    rc = GBPC_ERR_PIVOT;
  }
  if (!rc && inverse_out)
    if (cudaMemcpyAsync(inverse_out, op->inv.p, dtype_size(dtype) * (size_t)nrow * block * block,
                        cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
      gbpc_set_error("gbpc_op_block_jacobi: copy failed");
      rc = GBPC_ERR_CUDA;
    }
  if (rc) {
    delete op;
    return rc;
  }
  GBPC_OUT_OP(op);
  return GBPC_OK;
}

extern "C" int gbpc_op_block_jacobi_update(gbpc_op* h, int nrow, int block,
                                           const int32_t* offsets, const int32_t* columns,
                                           const void* values, int dtype, double pivot_tolerance,
                                           void* inverse_out, void* stream) {
  auto* op = h ? dynamic_cast<BlockJacobiOp*>(h->impl.get()) : nullptr;
  if (!op || nrow != op->nrow || block != op->B || dtype != op->vdtype) {
    gbpc_set_error("gbpc_op_block_jacobi_update: needs a BlockJacobi operator of the same "
                   "shape and dtype");
    return GBPC_ERR_ARG;
  }
  if (!std::isfinite(pivot_tolerance) || pivot_tolerance < 0) {
    gbpc_set_error("pivot_tolerance must be finite and nonnegative");
    return GBPC_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const size_t bytes = dtype_size(dtype) * (size_t)nrow * block * block;
  DevBuf cand;
  int rc = cand.alloc(std::max<size_t>(bytes, 16));
  if (rc) return rc;
  int32_t bad = 0;
  rc = block_diag_inverse(nrow, block, offsets, columns, values, dtype, pivot_tolerance, cand.p,
                          &bad, st);
  if (rc) return rc;
  if (bad) {  // the previous inverse stays in place
    gbpc_set_error("Missing, nonfinite or singular/near-singular block pivot");
    return GBPC_ERR_PIVOT;
  }
  if (bytes) {
    GBPC_CUDA_TRY(cudaMemcpyAsync(op->inv.p, cand.p, bytes, cudaMemcpyDeviceToDevice, st));
    if (inverse_out)
      GBPC_CUDA_TRY(cudaMemcpyAsync(inverse_out, cand.p, bytes, cudaMemcpyDeviceToDevice, st));
  }
  GBPC_CUDA_TRY(cudaStreamSynchronize(st));
  return GBPC_OK;
}

extern "C" int gbpc_op_bilu0(int nrow, int block, const int32_t* offsets, const int32_t* columns,
                             const void* values, int dtype, int factor_sweeps, int solve_sweeps,
                             double relaxation, double pivot_tolerance, void* factors_out,
                             void* inverse_out, void* stream, gbpc_op** out) {
  NvtxRange nvtx_range("gbpc_op_bilu0");
  if (!out || nrow < 0 || block < 1 || block > 4 || (dtype != GBPC_F64 && dtype != GBPC_F32)) {
    gbpc_set_error("BlockILU0 requires square blocks of size 1 through 4");
    return GBPC_ERR_ARG;
  }
  if (factor_sweeps < 0) {
    gbpc_set_error("factor_sweeps must be a nonnegative integer");
    return GBPC_ERR_ARG;
  }
  if (solve_sweeps < 1) {
    gbpc_set_error("solve_sweeps must be a positive integer");
    return GBPC_ERR_ARG;
  }
  if (!std::isfinite(relaxation) || !(relaxation > 0 && relaxation <= 1)) {
    gbpc_set_error("relaxation must be in (0,1]");
    return GBPC_ERR_ARG;
  }
  if (!std::isfinite(pivot_tolerance) || pivot_tolerance < 0) {
    gbpc_set_error("pivot_tolerance must be finite and nonnegative");
    return GBPC_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  int32_t nnz32 = 0;
  if (cudaMemcpy(&nnz32, offsets + nrow, sizeof(int32_t), cudaMemcpyDeviceToHost) != cudaSuccess) {
    gbpc_set_error("gbpc_op_bilu0: cannot read offsets");
    return GBPC_ERR_CUDA;
  }
  const int64_t nnz = nnz32;
  const size_t vs = dtype_size(dtype);
  const int bb = block * block;
  auto* op = new Bilu0Op;
  ByteTally tally(&op->device_bytes);
  op->rows = (int64_t)nrow * block;
  op->vdtype = dtype;
  op->nrow = nrow;
  op->B = block;
  op->sweeps = solve_sweeps;
  DevBuf factors;
  int rc = factors.alloc(vs * std::max<int64_t>(nnz, 1) * bb);
  if (!rc) rc = op->inv.alloc(vs * std::max<int64_t>((int64_t)nrow * bb, 1));
  for (int k = 0; k < 4 && !rc; ++k) rc = op->buf[k].alloc(vs * std::max<int64_t>(op->rows, 1));
  int32_t bad = 0;
  if (!rc)
    rc = bilu0_setup(nrow, block, offsets, columns, values, dtype, nnz, factor_sweeps, relaxation,
                     pivot_tolerance, factors.p, op->inv.p, &bad, st);
  if (!rc && bad) {
    gbpc_set_error("Missing, nonfinite or singular/near-singular block pivot");
    rc = GBPC_ERR_PIVOT;
  }
  SellBuild lo, up;
  lo.part = 1;
  up.part = 2;
  if (!rc) rc = sell_build(op->lower, nrow, nrow, block, offsets, columns, factors.p, dtype, dtype, lo, st);
  if (!rc) rc = sell_build(op->upper, nrow, nrow, block, offsets, columns, factors.p, dtype, dtype, up, st);
  if (!rc && factors_out)
    if (cudaMemcpyAsync(factors_out, factors.p, vs * nnz * bb, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
      rc = GBPC_ERR_CUDA;
  if (!rc && inverse_out)
    if (cudaMemcpyAsync(inverse_out, op->inv.p, vs * (size_t)nrow * bb, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
      rc = GBPC_ERR_CUDA;
  if (!rc && cudaStreamSynchronize(st) != cudaSuccess) rc = GBPC_ERR_CUDA;
  if (rc) {
    if (rc == GBPC_ERR_CUDA) gbpc_set_error("gbpc_op_bilu0: CUDA failure");
    delete op;
    return rc;
  }
  GBPC_OUT_OP(op);
  return GBPC_OK;
}

extern "C" int gbpc_op_apply(gbpc_op* h, const void* x, const void* y, void* z, double alpha,
                             double beta, void* stream) {
  NvtxRange nvtx_range("gbpc_op_apply");
  if (!h || !h->impl) {
    gbpc_set_error("gbpc_op_apply: null operator");
    return GBPC_ERR_ARG;
  }
  Operator* op = h->impl.get();
  cudaStream_t st = (cudaStream_t)stream;
  if (op->gathers_x() && x == z && alpha != 0.0) {
    int rc = vec_copy(op->alias_scratch.p, x, dtype_size(op->vdtype) * op->rows, st);
    if (rc) return rc;
    x = op->alias_scratch.p;
  }
  return op->apply(x, y, z, alpha, beta, nullptr, nullptr, st);
}

extern "C" int gbpc_op_device_bytes(const gbpc_op* h, size_t* bytes_host) {
  if (!h || !h->impl || !bytes_host) {
    gbpc_set_error("gbpc_op_device_bytes: bad arguments");
    return GBPC_ERR_ARG;
  }
  *bytes_host = h->impl->device_bytes;
  return GBPC_OK;
}

extern "C" int gbpc_op_rows(const gbpc_op* h, int64_t* rows_host) {
  if (!h || !h->impl || !rows_host) {
    gbpc_set_error("gbpc_op_rows: bad arguments");
    return GBPC_ERR_ARG;
  }
  *rows_host = h->impl->rows;
  return GBPC_OK;
}

extern "C" int gbpc_op_destroy(gbpc_op* h) {
  if (!h) return GBPC_OK;
  cudaDeviceSynchronize();
  delete h;
  return GBPC_OK;
}
