// Sparse product C = A diag(d) B + diag(e) on the device, for the assembled
// smoothing operator Q = alpha M + K M^-1 K (A = B = K, d = 1/mass,
// e = alpha mass).  The reference assembles Q on the host with SciPy
// (results/dirichlet-tuning/README.md:72-77) as K @ diags(d) @ K + diags(e);
// this is the same product in the same order.  SciPy's csr_matmat emits each
// row in reverse insertion order, so its intermediate K diags(d) holds row i
// with columns decreasing, and the contributions A_ij d_j B_jk reach entry
// (i, k) in DEcreasing j, starting from zero (a plain A B, whose A rows are
// sorted, sums over j increasing); e_i is added to the diagonal last; exact zeros are dropped and each row is written sorted by column.
// Compiled without multiply-add contraction, so the values are those of a
// separately rounded evaluation of that sum (SciPy's own on x86-64).
//
// One warp per row: the lanes take the entries of B's row j, each column
// k of C has at most one contribution per j, and a shared-memory hash table
// (sized from the longest rows of A and B) accumulates the row.  Two passes:
// counts (for the offsets), then the sorted columns and values.

#include <algorithm>
#include <vector>

#include "gbpc_common.cuh"
#include "gbpc_internal.h"

namespace gbpc {
namespace {

constexpr int kSgWarps = 4;
constexpr int kSgEmpty = -1;

__device__ __forceinline__ unsigned int sg_hash(int c) { return (unsigned int)c * 2654435761u; }

__device__ __forceinline__ int sg_insert(int* keys, int mask, int bits, int c) {
  unsigned int s = sg_hash(c) >> (32 - bits);
  for (int probe = 0; probe <= mask; ++probe) {
    int k = keys[s];
    if (k == c) return (int)s;
    if (k == kSgEmpty) {
      k = atomicCAS(keys + s, kSgEmpty, c);
      if (k == kSgEmpty || k == c) return (int)s;
    }
    s = (s + 1) & mask;
  }
  return -1;
}

__global__ void row_max_kernel(int n, const int32_t* __restrict__ off, int32_t* out) {
  int m = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    m = max(m, off[i + 1] - off[i]);
  atomicMax(out, m);
}

// pass 0: counts[i] = live entries of row i; pass 1: write the sorted row.
template <int PASS>
__global__ void __launch_bounds__(32 * kSgWarps)
spgemm_kernel(int nrow, const int32_t* __restrict__ a_off, const int32_t* __restrict__ a_col,
              const double* __restrict__ a_val, const double* __restrict__ d,
              const int32_t* __restrict__ b_off, const int32_t* __restrict__ b_col,
              const double* __restrict__ b_val, const double* __restrict__ e, int H, int hbits,
              int32_t* counts, const int32_t* __restrict__ c_off, int32_t* c_col, double* c_val,
              int32_t* overflow) {
  extern __shared__ __align__(16) unsigned char sg_smem[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int i = blockIdx.x * kSgWarps + w;
  // Per warp: vals[H], list values[H/2] (doubles), then keys[H], list columns[H/2].
  double* dbase = reinterpret_cast<double*>(sg_smem);
  double* vals = dbase + (size_t)w * H;
  double* lval = dbase + (size_t)kSgWarps * H + (size_t)w * (H / 2);
  int* ibase = reinterpret_cast<int*>(dbase + (size_t)kSgWarps * (H + H / 2));
  int* keys = ibase + (size_t)w * H;
  int* lcol = ibase + (size_t)kSgWarps * H + (size_t)w * (H / 2);
  if (i >= nrow) return;
  const int mask = H - 1;
  for (int s = lane; s < H; s += 32) {
    keys[s] = kSgEmpty;
    vals[s] = 0.0;
  }
  __syncwarp();
  bool over = false;
  const int len = a_off[i + 1] - a_off[i];
  for (int t = 0; t < len; ++t) {
    const int jj = d ? a_off[i + 1] - 1 - t : a_off[i] + t;
    const int j = a_col[jj];
    const double v = d ? a_val[jj] * d[j] : a_val[jj];
    for (int kk = b_off[j] + lane; kk < b_off[j + 1]; kk += 32) {
      const int slot = sg_insert(keys, mask, hbits, b_col[kk]);
      if (slot < 0) {
        over = true;
      } else {
        const double p = v * b_val[kk];
        vals[slot] = vals[slot] + p;
      }
    }
    __syncwarp();
  }
  if (e && lane == 0) {
    const int slot = sg_insert(keys, mask, hbits, i);
    if (slot < 0) over = true;
    else vals[slot] = vals[slot] + e[i];
  }
  __syncwarp();
  if (__any_sync(0xffffffffu, over)) {
    if (lane == 0) atomicAdd(overflow, 1);
    return;
  }
  // Compact the nonzero entries (at most H/2: the table holds <= H/2 keys).
  int nlive = 0;
  for (int s0 = 0; s0 < H; s0 += 32) {
    const int s = s0 + lane;
    const bool live = keys[s] != kSgEmpty && vals[s] != 0.0;
    const unsigned m = __ballot_sync(0xffffffffu, live);
    if (live) {
      const int pos = nlive + __popc(m & ((1u << lane) - 1u));
      lcol[pos] = keys[s];
      lval[pos] = vals[s];
    }
    nlive += __popc(m);
  }
  __syncwarp();
  if (PASS == 0) {
    if (lane == 0) counts[i] = nlive;
  } else {
    const int base = c_off[i];
    for (int t = lane; t < nlive; t += 32) {
      const int k = lcol[t];
      int rank = 0;
      for (int u = 0; u < nlive; ++u) rank += (lcol[u] < k);
      c_col[base + rank] = k;
      c_val[base + rank] = lval[t];
    }
  }
}

}  // namespace

int scan_exclusive_i32(const int32_t* in, int32_t* out, int n, cudaStream_t st);

}  // namespace gbpc

using namespace gbpc;

extern "C" int gbpc_spgemm(int nrow, int ncol, const int32_t* a_off, const int32_t* a_col,
                           const double* a_val, const double* col_scale, int b_nrow,
                           const int32_t* b_off, const int32_t* b_col, const double* b_val,
                           const double* add_diag, int32_t* c_off, int32_t* c_col, double* c_val,
                           int64_t* nnz_host, void* stream) {
  NvtxRange nvtx_range("gbpc_spgemm");
  if (nrow < 0 || b_nrow < 0 || ncol < 0 || !c_off || !a_off || !b_off ||
      (add_diag && nrow > ncol)) {
    gbpc_set_error("gbpc_spgemm: bad arguments");
    return GBPC_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  DevBuf stat;
  int rc = stat.alloc(sizeof(int32_t) * 3);
  if (rc) return rc;
  GBPC_CUDA_TRY(cudaMemsetAsync(stat.p, 0, sizeof(int32_t) * 3, st));
  int32_t* s = stat.as<int32_t>();
  if (nrow > 0) row_max_kernel<<<std::min(grid_for(nrow, 256), 1024), 256, 0, st>>>(nrow, a_off, s);
  if (b_nrow > 0)
    row_max_kernel<<<std::min(grid_for(b_nrow, 256), 1024), 256, 0, st>>>(b_nrow, b_off, s + 1);
  GBPC_CUDA_TRY(cudaGetLastError());
  int32_t h[3];
  GBPC_CUDA_TRY(cudaMemcpyAsync(h, s, sizeof(h), cudaMemcpyDeviceToHost, st));
  GBPC_CUDA_TRY(cudaStreamSynchronize(st));
  // Distinct columns of a row of C never exceed maxA * maxB (+1 diagonal).
  const int64_t bound = (int64_t)h[0] * h[1] + 1;
  int smem_optin = 0, dev = 0;
  GBPC_CUDA_TRY(cudaGetDevice(&dev));
  GBPC_CUDA_TRY(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  // Table sizes are powers of two from 64 up; the largest one that fits the
  // opt-in shared memory ends the search, so H never overflows.
  int64_t H64 = 64;
  int hbits = 6;
  while (H64 < 2 * bound &&
         (size_t)kSgWarps * (H64 + H64 / 2) * (sizeof(double) + sizeof(int)) <= (size_t)smem_optin) {
    H64 <<= 1;
    ++hbits;
  }
  const size_t smem = (size_t)kSgWarps * (H64 + H64 / 2) * (sizeof(double) + sizeof(int));
  const int H = (int)std::min<int64_t>(H64, 1 << 30);
  if (H64 < 2 * bound || smem > (size_t)smem_optin) {
    gbpc_set_error("gbpc_spgemm: rows too long (%lld candidate columns per row)", (long long)bound);
    return GBPC_ERR_UNSUPPORTED;
  }
  const int grid = (nrow + kSgWarps - 1) / kSgWarps;
  if (c_col == nullptr) {
    DevBuf counts;
    if ((rc = counts.alloc(sizeof(int32_t) * std::max(nrow, 1)))) return rc;
    if (nrow > 0) {
      GBPC_CUDA_TRY(cudaFuncSetAttribute(spgemm_kernel<0>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      spgemm_kernel<0><<<grid, 32 * kSgWarps, smem, st>>>(
          nrow, a_off, a_col, a_val, col_scale, b_off, b_col, b_val, add_diag, H, hbits,
          counts.as<int32_t>(), nullptr, nullptr, nullptr, s + 2);
      GBPC_CUDA_TRY(cudaGetLastError());
    }
    if ((rc = scan_exclusive_i32(counts.as<int32_t>(), c_off, nrow, st))) return rc;
    int32_t tail[2] = {0, 0};
    GBPC_CUDA_TRY(cudaMemcpyAsync(&tail[0], c_off + nrow, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    GBPC_CUDA_TRY(cudaMemcpyAsync(&tail[1], s + 2, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    GBPC_CUDA_TRY(cudaStreamSynchronize(st));
    if (tail[1]) {
      gbpc_set_error("gbpc_spgemm: row accumulator overflow");
      return GBPC_ERR_UNSUPPORTED;
    }
    if (nnz_host) *nnz_host = tail[0];
    return GBPC_OK;
  }
  if (nrow > 0) {
    GBPC_CUDA_TRY(cudaFuncSetAttribute(spgemm_kernel<1>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    spgemm_kernel<1><<<grid, 32 * kSgWarps, smem, st>>>(
        nrow, a_off, a_col, a_val, col_scale, b_off, b_col, b_val, add_diag, H, hbits, nullptr,
        c_off, c_col, c_val, s + 2);
    GBPC_CUDA_TRY(cudaGetLastError());
  }
  GBPC_CUDA_TRY(cudaStreamSynchronize(st));
  return GBPC_OK;
}
