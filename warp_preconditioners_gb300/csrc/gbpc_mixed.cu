// Preconditioners of the mixed (indefinite) harmonic systems
// (warp_preconditioners/mixed.py:283-427): MatchingSchur (block elimination
// with repeated approximate inverses of H = K + alpha^(1/p) M) and
// ShiftedBlock (the first-order block approximation).  Vectors interleave
// `order` unknowns per vertex; K is a scalar CSR matrix (sliced-ELL product),
// H^-1 any operator of this library (normally FSAI(H)).  Each apply is a
// fixed sequence of kernels on the caller's stream, capturable in graphs.

#include <algorithm>
#include <cmath>

#include "gbpc_common.cuh"
#include "gbpc_internal.h"

namespace gbpc {

int copy_with_dot(int64_t n, const double* x, double* z, const int* guard, const Reduction& red,
                  cudaStream_t st);

namespace {

constexpr int kMT = 256;

int m_grid(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + kMT - 1) / kMT, 152 * 16)); }

#define FOR_ROWS(i, n)                                                                   \
  for (int64_t i = (int64_t)blockIdx.x * kMT + threadIdx.x; i < (n); i += (int64_t)gridDim.x * kMT)

// mixed.py:75-80 (`scaled_component`): out = x[:, c] / mass
template <typename T>
__global__ void scaled_component_kernel(int64_t n, int order, const T* x, int c, const T* mass,
                                        T* out, const int* guard) {
  if (guard_off(guard)) return;
  FOR_ROWS(i, n) out[i] = x[i * order + c] / mass[i];
}

// mixed.py:113-116 (`divide`): out = x / mass
template <typename T>
__global__ void divide_kernel(int64_t n, const T* x, const T* mass, T* out, const int* guard) {
  if (guard_off(guard)) return;
  FOR_ROWS(i, n) out[i] = x[i] / mass[i];
}

// mixed.py:82-87 (`multiply_mass`): out = mass * x
template <typename T>
__global__ void multiply_mass_kernel(int64_t n, const T* x, const T* mass, T* out,
                                     const int* guard) {
  if (guard_off(guard)) return;
  FOR_ROWS(i, n) out[i] = mass[i] * x[i];
}

// mixed.py:89-100 (`rhs`): out = x[:, 0] - k1 (+ k2 for order 3)
template <typename T>
__global__ void schur_rhs_kernel(int64_t n, int order, const T* x, const T* k1, const T* k2,
                                 T* out, const int* guard) {
  if (guard_off(guard)) return;
  FOR_ROWS(i, n) {
    T v = x[i * order] - k1[i];
    if (order == 3) v += k2[i];
    out[i] = v;
  }
}

// mixed.py:102-111 (`auxiliary`): out = -(ku + x[:, c]) / mass
template <typename T>
__global__ void auxiliary_kernel(int64_t n, int order, const T* x, int c, const T* ku,
                                 const T* mass, T* out, const int* guard) {
  if (guard_off(guard)) return;
  FOR_ROWS(i, n) out[i] = -(ku[i] + x[i * order + c]) / mass[i];
}

// mixed.py:118-141 (`finish`): z = alpha (u, a[, lam]) + beta y
template <typename T>
__global__ void schur_finish_kernel(int64_t n, int order, const T* u, const T* a, const T* lam,
                                    const T* y, T* z, T alpha, T beta, const int* guard) {
  if (guard_off(guard)) return;
  FOR_ROWS(i, n) {
    T v[3] = {u[i], a[i], order == 3 ? lam[i] : T(0)};
    for (int c = 0; c < order; ++c) {
      T w = (alpha == T(0)) ? T(0) : v[c] * alpha;
      if (beta != T(0)) w += beta * y[i * order + c];
      z[i * order + c] = w;
    }
  }
}

// mixed.py:341-356 (`unpack`)
template <typename T>
__global__ void shifted_unpack_kernel(int64_t n, int order, const T* x, T* a, T* b, T* c, T scale,
                                      const int* guard) {
  if (guard_off(guard)) return;
  FOR_ROWS(i, n) {
    if (order == 2) {
      const T x0 = x[i * 2], x1 = x[i * 2 + 1];
      a[i] = (x0 / scale - scale * x1) * T(0.5);
      b[i] = (-x0 / scale - scale * x1) * T(0.5);
    } else {
      a[i] = -x[i * 3 + 2];
      b[i] = -x[i * 3 + 1];
      c[i] = -x[i * 3];
    }
  }
}

// mixed.py:358-383 (`finish`)
template <typename T>
__global__ void shifted_finish_kernel(int64_t n, int order, const T* a, const T* b, const T* c,
                                      const T* y, T* z, T scale, T alpha, T beta,
                                      const int* guard) {
  if (guard_off(guard)) return;
  FOR_ROWS(i, n) {
    T v[3];
    if (order == 2) {
      v[0] = a[i] / scale;
      v[1] = b[i] * scale;
      v[2] = T(0);
    } else {
      v[0] = a[i];
      v[1] = b[i];
      v[2] = c[i];
    }
    for (int q = 0; q < order; ++q) {
      T w = (alpha == T(0)) ? T(0) : v[q] * alpha;
      if (beta != T(0)) w += beta * y[i * order + q];
      z[i * order + q] = w;
    }
  }
}

}  // namespace

// Shared pieces of the two preconditioners.
struct MixedBase : Operator {
  int order = 2;
  int64_t n = 0;  // vertices
  Operator* hinv = nullptr;  // not owned
  DevBuf buf[7];
  ReduceBuf rb;

  template <typename T> T* B(int k) { return buf[k].as<T>(); }

  int init_buffers(int count) {
    int rc;
    for (int k = 0; k < count; ++k)
      if ((rc = buf[k].alloc(dtype_size(vdtype) * std::max<int64_t>(n, 1)))) return rc;
    return GBPC_OK;
  }

  // Fused dot(w, z) after the apply (the Krylov loops use it for M).
  int finish_dot(void* z, const int* guard, const DotSpec* dot, cudaStream_t st) {
    if (!dot || !dot->w) return GBPC_OK;
    if (vdtype != GBPC_F64) {
      gbpc_set_error("fused dot products need float64 vectors");
      return GBPC_ERR_ARG;
    }
    Reduction red{};
    red.w = dot->w;
    red.partials = dot->rb->partials.as<double>();
    red.counter = dot->rb->counter.as<unsigned int>();
    red.mode = dot->mode;
    red.ks = (KrylovScalars*)dot->ks;
    red.out = dot->out;
    return copy_with_dot(rows, (const double*)z, (double*)z, guard, red, st);
  }
};

struct MatchingSchurOp : MixedBase {
  Sell k;  // scalar K (float64 or float32 values, vectors of the same type)

  int kmv(const void* in, void* out, const int* guard, cudaStream_t st) {
    return sell_spmv(k, vdtype, in, nullptr, out, 1.0, 0.0, guard, EpiHost{}, nullptr, st);
  }

  template <typename T>
  int apply_t(const T* x, const T* y, T* z, double alpha, double beta, const int* guard,
              const DotSpec* dot, cudaStream_t st) {
    const T* mass = B<T>(6);
    T *t = B<T>(0), *v = B<T>(1), *w = B<T>(2), *g = B<T>(3), *u = B<T>(4), *a = B<T>(5);
    T* lam = t;  // order 3: t is free again when lam is formed
    const int G = m_grid(n);
    int rc;
    scaled_component_kernel<T><<<G, kMT, 0, st>>>(n, order, x, 1, mass, t, guard);
    if ((rc = kmv(t, v, guard, st))) return rc;
    if (order == 3) {
      scaled_component_kernel<T><<<G, kMT, 0, st>>>(n, order, x, 2, mass, t, guard);
      if ((rc = kmv(t, w, guard, st))) return rc;
      divide_kernel<T><<<G, kMT, 0, st>>>(n, w, mass, t, guard);
      if ((rc = kmv(t, w, guard, st))) return rc;
    }
    schur_rhs_kernel<T><<<G, kMT, 0, st>>>(n, order, x, v, w, g, guard);
    if ((rc = hinv->apply(g, nullptr, u, 1.0, 0.0, guard, nullptr, st))) return rc;
    for (int step = 0; step < order - 1; ++step) {
      multiply_mass_kernel<T><<<G, kMT, 0, st>>>(n, u, mass, t, guard);
      const double sgn = (order == 3 && step == 1) ? -1.0 : 1.0;
      if ((rc = hinv->apply(t, nullptr, u, sgn, 0.0, guard, nullptr, st))) return rc;
    }
    if ((rc = kmv(u, v, guard, st))) return rc;
    auxiliary_kernel<T><<<G, kMT, 0, st>>>(n, order, x, order == 2 ? 1 : 2, v, mass, a, guard);
    if (order == 3) {
      if ((rc = kmv(a, v, guard, st))) return rc;
      auxiliary_kernel<T><<<G, kMT, 0, st>>>(n, order, x, 1, v, mass, lam, guard);
    }
    schur_finish_kernel<T><<<G, kMT, 0, st>>>(n, order, u, a, lam, y, z, (T)alpha, (T)beta, guard);
    GBPC_CUDA_TRY(cudaGetLastError());
    return finish_dot(z, guard, dot, st);
  }

  int apply(const void* x, const void* y, void* z, double alpha, double beta, const int* guard,
            const DotSpec* dot, cudaStream_t st) override {
    if (vdtype == GBPC_F64)
      return apply_t<double>((const double*)x, (const double*)y, (double*)z, alpha, beta, guard,
                             dot, st);
    return apply_t<float>((const float*)x, (const float*)y, (float*)z, alpha, beta, guard, dot,
                          st);
  }
  bool gathers_x() const override { return false; }  // x is consumed before z is written
};

struct ShiftedBlockOp : MixedBase {
  double scale = 1.0;

  template <typename T>
  int apply_t(const T* x, const T* y, T* z, double alpha, double beta, const int* guard,
              const DotSpec* dot, cudaStream_t st) {
    T *a = B<T>(0), *b = B<T>(1), *c = B<T>(2), *u = B<T>(3), *v = B<T>(4), *w = B<T>(5);
    const int G = m_grid(n);
    int rc;
    shifted_unpack_kernel<T><<<G, kMT, 0, st>>>(n, order, x, a, b, c, (T)scale, guard);
    if ((rc = hinv->apply(a, nullptr, u, 1.0, 0.0, guard, nullptr, st))) return rc;
    if ((rc = hinv->apply(b, nullptr, v, 1.0, 0.0, guard, nullptr, st))) return rc;
    if (order == 3 && (rc = hinv->apply(c, nullptr, w, 1.0, 0.0, guard, nullptr, st))) return rc;
    shifted_finish_kernel<T><<<G, kMT, 0, st>>>(n, order, u, v, w, y, z, (T)scale, (T)alpha,
                                                (T)beta, guard);
    GBPC_CUDA_TRY(cudaGetLastError());
    return finish_dot(z, guard, dot, st);
  }

  int apply(const void* x, const void* y, void* z, double alpha, double beta, const int* guard,
            const DotSpec* dot, cudaStream_t st) override {
    if (vdtype == GBPC_F64)
      return apply_t<double>((const double*)x, (const double*)y, (double*)z, alpha, beta, guard,
                             dot, st);
    return apply_t<float>((const float*)x, (const float*)y, (float*)z, alpha, beta, guard, dot,
                          st);
  }
  bool gathers_x() const override { return false; }
};

}  // namespace gbpc

using namespace gbpc;

static int mixed_check(int order, int n, gbpc_op* hinv, int dtype) {
  if ((order != 2 && order != 3) || n < 0 || !hinv || !hinv->impl ||
      (dtype != GBPC_F64 && dtype != GBPC_F32)) {
    gbpc_set_error("mixed preconditioner: order must be 2 or 3 with an H^-1 operator");
    return GBPC_ERR_ARG;
  }
  if (hinv->impl->rows != n || hinv->impl->vdtype != dtype) {
    gbpc_set_error("H_inverse must match H");
    return GBPC_ERR_ARG;
  }
  return GBPC_OK;
}

extern "C" int gbpc_op_matching_schur(int order, int n, const int32_t* k_off, const int32_t* k_col,
                                      const void* k_val, int dtype, const void* mass,
                                      gbpc_op* hinv, void* stream, gbpc_op** out) {
  int rc = mixed_check(order, n, hinv, dtype);
  if (rc) return rc;
  if (!out || !k_off || (n > 0 && !mass)) {
    gbpc_set_error("gbpc_op_matching_schur: bad arguments");
    return GBPC_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  auto* op = new MatchingSchurOp;
  ByteTally tally(&op->device_bytes);
  op->order = order;
  op->n = n;
  op->rows = (int64_t)n * order;
  op->vdtype = dtype;
  op->hinv = hinv->impl.get();
  rc = op->init_buffers(7);
  if (!rc && n > 0)
    rc = (cudaMemcpyAsync(op->buf[6].p, mass, dtype_size(dtype) * n, cudaMemcpyDeviceToDevice,
                          st) == cudaSuccess) ? GBPC_OK : GBPC_ERR_CUDA;
  if (!rc) rc = sell_build(op->k, n, n, 1, k_off, k_col, k_val, dtype, dtype, SellBuild{}, st);
  if (!rc) rc = sell_autotune(op->k, dtype, st);
  if (!rc && cudaStreamSynchronize(st) != cudaSuccess) rc = GBPC_ERR_CUDA;
  if (rc) {
    delete op;
    return rc;
  }
  gbpc_op* h = new gbpc_op;
  h->impl.reset(op);
  *out = h;
  return GBPC_OK;
}

extern "C" int gbpc_op_shifted_block(int order, int n, double scale, int dtype, gbpc_op* hinv,
                                     void* stream, gbpc_op** out) {
  int rc = mixed_check(order, n, hinv, dtype);
  if (rc) return rc;
  if (!out || !std::isfinite(scale) || !(scale > 0.0)) {
    gbpc_set_error("gbpc_op_shifted_block: bad arguments");
    return GBPC_ERR_ARG;
  }
  (void)stream;
  auto* op = new ShiftedBlockOp;
  ByteTally tally(&op->device_bytes);
  op->order = order;
  op->n = n;
  op->rows = (int64_t)n * order;
  op->vdtype = dtype;
  op->hinv = hinv->impl.get();
  op->scale = scale;
  rc = op->init_buffers(6);
  if (rc) {
    delete op;
    return rc;
  }
  gbpc_op* h = new gbpc_op;
  h->impl.reset(op);
  *out = h;
  return GBPC_OK;
}
