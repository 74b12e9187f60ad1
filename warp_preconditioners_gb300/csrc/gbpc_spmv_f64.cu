// Sliced products with float64 vectors (float64, float32 or bfloat16 storage).
#include "gbpc_spmv.cuh"

namespace gbpc {

int spmv_f64(const Sell& m, const void* x, const void* y, void* z, double alpha, double beta,
             const int* guard, const EpiHost& ep, const Reduction& red, cudaStream_t st) {
  return spmv_dispatch<double>(m, x, y, z, alpha, beta, guard, ep, red, st);
}

}  // namespace gbpc
