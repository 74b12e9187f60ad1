// Host-side internals shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <memory>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/gbpc.h"

namespace gbpc {

// An NVTX range around a setup, apply or solve entry point (visible in
// Nsight timelines; costs nothing measurable when no tool is attached).
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

constexpr int kMaxCtas = 152 * 8;  // partial-sum capacity of every reduction buffer

size_t dtype_size(int dtype);
bool valid_value_dtype(int d);

// Bookkeeping of device bytes held by DevBuf allocations: a process-wide
// live total, and per object a tally.  While a ByteTally scope is open on a
// thread, every DevBuf that thread allocates adds its bytes to the scope's
// counter and takes them back when released, so an operator or solver built
// inside such a scope knows the device bytes it holds.
void note_release(size_t bytes, size_t* tally);
size_t* current_tally();
size_t device_bytes_live();
struct ByteTally {
  size_t* prev;
  explicit ByteTally(size_t* counter);
  ~ByteTally();
  ByteTally(const ByteTally&) = delete;
  ByteTally& operator=(const ByteTally&) = delete;
};

// While open, kernels launched through launch_k on this thread carry the
// programmatic dependent launch attribute (gbpc_common.cuh).
struct PdlScope {
  bool prev;
  explicit PdlScope(bool on);
  ~PdlScope();
  PdlScope(const PdlScope&) = delete;
  PdlScope& operator=(const PdlScope&) = delete;
};

// Owned device allocation.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  size_t* tally = nullptr;  // counter charged with `bytes` (nullable)
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) {
      cudaFree(p);
      note_release(bytes, tally);
    }
    p = nullptr;
    bytes = 0;
    tally = nullptr;
  }
  int alloc(size_t n);
  template <typename T> T* as() const { return static_cast<T*>(p); }
};

// Sliced ELL matrix (32 block rows per slice) with owned storage.
struct Sell {
  int nrow = 0;     // block rows
  int ncol = 0;     // block columns
  int B = 1;        // block size
  int nslices = 0;
  int vdtype = GBPC_F64;
  int64_t nent = 0;  // entries including padding
  DevBuf slice_ptr;  // int64[nslices + 1]
  DevBuf cols;       // int32[nent]
  DevBuf vals;       // vdtype[nent * B * B]
  DevBuf perm;       // int32[nrow] when rows are stored sorted by length
  DevBuf sched;      // int4[nslices]: product schedule, slices by width descending
  DevBuf err;        // int32[1]: set by a product kernel whose bounded wait gave up
  int variant = 0;   // product kernel variant chosen by sell_autotune
  int64_t nnz = 0;   // stored entries without padding
};

// Build options: output row k reads source row rows[k] (rows == nullptr:
// k itself); columns are remapped through colmap (entries whose image is
// negative are dropped); `part` keeps all (0), strictly lower (1) or strictly
// upper (2) blocks relative to the source row index; `row_scale` multiplies
// every value of source row r by row_scale[r] (bf16 input: unsupported).
struct SellBuild {
  const int32_t* rows = nullptr;
  const int32_t* colmap = nullptr;
  int part = 0;
  const void* row_scale = nullptr;  // optional per-source-row factor (input value dtype)
};

// Rewrites the values of a Sell built from the same pattern (off, col, opt).
int sell_refill(Sell& s, const int32_t* off, const int32_t* col, const void* val, int in_dtype,
                const SellBuild& opt, cudaStream_t st);
int sell_build(Sell& s, int nrow_out, int ncol, int B, const int32_t* off, const int32_t* col,
               const void* val, int in_dtype, int out_dtype, const SellBuild& opt,
               cudaStream_t st);

// Time the product kernel variants on `m` (vectors of dtype adtype) and keep
// the fastest.  All variants sum each row in the same order, so the choice
// never changes results.
int sell_autotune(Sell& m, int adtype, cudaStream_t st);

// Epilogues of the SELL product (see gbpc_sell.cu).
enum EpiKind : int {
  EPI_AXPBY = 0,      // z = alpha * acc + beta * y
  EPI_SQLAP_FWD = 1,  // z = aux0 * acc                      (aux0 = 1/mass)
  EPI_SQLAP_BWD = 2,  // z = alpha * (acc + aux0 * aux1) + beta * y  (aux0 = w*mass[free], aux1 = x)
  EPI_TRI_LOWER = 3,  // z = aux0 - acc                      (aux0 = rhs)
  EPI_TRI_UPPER = 4,  // z = inv_block(aux1) * (aux0 - acc)  (aux0 = rhs, aux1 = inverse blocks)
};

struct EpiHost {
  int kind = EPI_AXPBY;
  const void* aux0 = nullptr;
  const void* aux1 = nullptr;
  // Walk the slices in reverse pass order (products without a fused dot;
  // the result is the same either way): the second of two back-to-back
  // products over one matrix then starts on the first one's most recently
  // read slices.
  bool reverse = false;
};

struct ReductionHost;  // defined in gbpc_common.cuh as gbpc::Reduction

// Scratch for one deterministic reduction: partials + arrival counter.
struct ReduceBuf {
  DevBuf partials;  // double[kMaxCtas]
  DevBuf counter;   // unsigned int[1], zero between uses
  int init(cudaStream_t st);
};

// z = alpha * A x + beta * y over a SELL matrix with vector type adtype.
// red_w != nullptr adds dot(red_w, z) reduced into `rb` with finalize mode
// `fin_mode` acting on `ks` (or storing to `fin_out`).
struct DotSpec {
  const double* w = nullptr;
  ReduceBuf* rb = nullptr;
  int mode = 0;
  void* ks = nullptr;
  double* out = nullptr;
};

int sell_spmv(const Sell& m, int adtype, const void* x, const void* y, void* z, double alpha,
              double beta, const int* guard, const EpiHost& ep, const DotSpec* dot,
              cudaStream_t st);

// Vector helpers (float64 unless stated).
int vec_copy(void* dst, const void* src, size_t bytes, cudaStream_t st);

// ---------------------------------------------------------------------------
// Operators.

struct Operator {
  virtual ~Operator() = default;
  size_t device_bytes = 0;  // DevBuf bytes held (declared first: released last)
  int64_t rows = 0;        // scalar vector length
  int vdtype = GBPC_F64;   // vector dtype
  // z = alpha Op x + beta y.  `guard` (nullable device int) skips all work
  // when zero.  `dot` (nullable) reduces dot(dot->w, z) in the final kernel.
  virtual int apply(const void* x, const void* y, void* z, double alpha, double beta,
                    const int* guard, const DotSpec* dot, cudaStream_t st) = 0;
  // True when x may not alias z in apply (the generic entry copies x first).
  virtual bool gathers_x() const { return true; }
  // The scalar float64 sliced-ELL matrices whose products in this order
  // are the whole apply (z = M_k ... M_1 x, no epilogue), or 0 when the
  // operator is not of that form.  Lets a solver run them itself.
  virtual int scalar_products(const Sell** out, int max) const {
    (void)out;
    (void)max;
    return 0;
  }
  // The factored squared Laplacian with every vertex free, float64: its L,
  // 1/m and w m (apply = L((1/m) o (L x)) + (w m) o x), or false.
  virtual bool factored_parts(const Sell** L, const void** inv_mass, const void** wmass) const {
    (void)L;
    (void)inv_mass;
    (void)wmass;
    return false;
  }
  DevBuf alias_scratch;  // copy of x when x aliases z
};

// A preconditioner applied in float32 behind a float64 interface
// (GBPC_F32_APPLY): apply() narrows x into in32, runs `inner` (float32
// vectors) into out32 and widens alpha * out32 + beta * y into z with the
// fused dot.  The CG solver writes in32 and reads out32 itself, so inside
// its loop only `inner` runs.
struct LowPrecisionOp : Operator {
  std::unique_ptr<Operator> inner;
  DevBuf in32, out32;
  int apply(const void* x, const void* y, void* z, double alpha, double beta, const int* guard,
            const DotSpec* dot, cudaStream_t st) override;
  bool gathers_x() const override { return false; }
};

}  // namespace gbpc

struct gbpc_op {
  std::unique_ptr<gbpc::Operator> impl;
};
