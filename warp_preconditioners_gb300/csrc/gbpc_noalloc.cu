// FSAI application without any device allocation.
//
// gbpc_fsai_apply_noalloc computes z = alpha * G^T (G x) + beta * y straight
// from the CSR arrays of G and G^T.  The intermediate G x lives in a
// fixed-size array in the library's own device memory instead of a buffer
// from cudaMalloc, so callers that must not allocate device memory (see the
// declaration in include/gbpc.h) can still apply the preconditioner.
//
// The array is a file-scope __device__ variable of kNoAllocMaxRows doubles
// (4 MiB).  CUDA loads this translation unit's module lazily, so the array is
// reserved on a device by the first call of gbpc_fsai_apply_noalloc there
// (a call with n == 0 does only that), and it stays reserved until the
// process exits.  Host code only ever passes the array's device address,
// obtained with cudaGetSymbolAddress; the host-side symbol itself is not a
// device address.

#include <mutex>

#include "gbpc_common.cuh"
#include "gbpc_internal.h"

namespace gbpc {
namespace {

constexpr int kNoAllocMaxRows = 1 << 19;  // 524,288 rows of float64 scratch
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocMaxRows];

std::mutex g_scratch_mutex;
double* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device.  Outside stream
// capture it is looked up on every call (cheap once the module is loaded, and
// never stale after a device reset recreated the context); the first lookup
// on a device loads the module and reserves the array.  Under stream capture
// the address cached by the last uncaptured call on that device is used, so
// the first call on each device must come before any capture.
int scratch_address(cudaStream_t st, double** out) {
  int dev = 0;
  GBPC_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    gbpc_set_error("gbpc_fsai_apply_noalloc: device ordinal %d out of range", dev);
    return GBPC_ERR_ARG;
  }
  cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
  GBPC_CUDA_TRY(cudaStreamIsCapturing(st, &capture));
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (capture == cudaStreamCaptureStatusNone) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      gbpc_set_error_cuda(e, "cudaGetSymbolAddress(g_noalloc_scratch)", __FILE__, __LINE__);
      return GBPC_ERR_CUDA;
    }
    g_scratch_ptr[dev] = static_cast<double*>(p);
  } else if (g_scratch_ptr[dev] == nullptr) {
    gbpc_set_error("gbpc_fsai_apply_noalloc: first call on device %d made under stream "
                   "capture; call it once (n = 0 is enough) before capturing",
                   dev);
    return GBPC_ERR_ARG;
  }
  *out = g_scratch_ptr[dev];
  return GBPC_OK;
}

// One thread per row of a scalar CSR matrix: out = alpha * A v + beta * y
// (beta == 0 never reads y, alpha == 0 never reads v).
template <typename S>
__global__ void __launch_bounds__(kThreads, kCtasPerSm)
csr_rows_kernel(int n, const int32_t* __restrict__ off, const int32_t* __restrict__ col,
                const S* __restrict__ val, const double* v, const double* y, double* out,
                double alpha, double beta, int alpha_zero, int beta_zero) {
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= n) return;
  double acc = 0.0;
  if (!alpha_zero) {
    const int e_end = off[i + 1];
    for (int e = off[i]; e < e_end; ++e) acc = fma((double)val[e], v[col[e]], acc);
    acc = alpha * acc;
  }
  if (!beta_zero) acc = fma(beta, y[i], acc);
  out[i] = acc;
}

template <typename S>
int apply_t(int n, const int32_t* g_off, const int32_t* g_col, const S* g_val,
            const int32_t* gt_off, const int32_t* gt_col, const S* gt_val, const double* x,
            const double* y, double* z, double alpha, double beta, cudaStream_t st) {
  double* tmp = nullptr;
  int rc = scratch_address(st, &tmp);
  if (rc) return rc;
  const int grid = grid_for(n, kThreads);
  const int alpha_zero = alpha == 0.0;
  // tmp = G x is written in full for every row before it is read, so the
  // array's previous contents never matter.
  if (!alpha_zero)
    csr_rows_kernel<S><<<grid, kThreads, 0, st>>>(n, g_off, g_col, g_val, x, nullptr, tmp, 1.0,
                                                  0.0, 0, 1);
  csr_rows_kernel<S><<<grid, kThreads, 0, st>>>(n, gt_off, gt_col, gt_val, tmp, y, z, alpha, beta,
                                                alpha_zero, beta == 0.0);
  GBPC_CUDA_TRY(cudaGetLastError());
  return GBPC_OK;
}

}  // namespace
}  // namespace gbpc

using namespace gbpc;

extern "C" int gbpc_fsai_apply_noalloc_max_rows(void) { return kNoAllocMaxRows; }

extern "C" int gbpc_fsai_apply_noalloc(int n, const int32_t* g_off, const int32_t* g_col,
                                       const void* g_val, const int32_t* gt_off,
                                       const int32_t* gt_col, const void* gt_val,
                                       int value_dtype, const double* x, const double* y,
                                       double* z, double alpha, double beta, void* stream) {
  if (n < 0 || n > kNoAllocMaxRows) {
    gbpc_set_error("gbpc_fsai_apply_noalloc: n = %d rows exceeds the fixed scratch of %d rows "
                   "(use gbpc_op_fsai + gbpc_op_apply for larger factors)",
                   n, kNoAllocMaxRows);
    return GBPC_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (n == 0) {
    // Nothing to compute; the call still reserves the scratch array on the
    // current device, so a host can make it at start-up, before it takes a
    // fixed memory pool.
    double* tmp = nullptr;
    return scratch_address(st, &tmp);
  }
  if (!g_off || !g_col || !g_val || !gt_off || !gt_col || !gt_val || !z ||
      (alpha != 0.0 && !x) || (beta != 0.0 && !y)) {
    gbpc_set_error("gbpc_fsai_apply_noalloc: null array argument");
    return GBPC_ERR_ARG;
  }
  if (value_dtype == GBPC_F64)
    return apply_t<double>(n, g_off, g_col, (const double*)g_val, gt_off, gt_col,
                           (const double*)gt_val, x, y, z, alpha, beta, st);
  if (value_dtype == GBPC_F32)
    return apply_t<float>(n, g_off, g_col, (const float*)g_val, gt_off, gt_col,
                          (const float*)gt_val, x, y, z, alpha, beta, st);
  gbpc_set_error("gbpc_fsai_apply_noalloc: factor values must be float64 or float32");
  return GBPC_ERR_ARG;
}
