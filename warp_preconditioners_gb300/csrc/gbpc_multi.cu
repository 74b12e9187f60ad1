// Many independent systems of uneven size in one solve: preconditioned CG on
// a block-diagonal operator whose diagonal blocks are the systems (segments
// of consecutive rows), with every Krylov scalar, dot product and stopping
// test kept per segment.
//
// The operator and the preconditioner are ordinary libgbpc operators over
// the concatenated vectors (a block-diagonal BSR matrix, a factored
// squared-Laplacian operator over concatenated meshes, FSAI of the
// block-diagonal matrix, which equals the per-system FSAI factors row for
// row because the adaptive search never leaves a row's pattern), so each
// product is one launch for all systems.  The vector updates and dot
// products run over tiles of at most kTile rows that never straddle two
// segments; a segment's dot product is the sum of its tiles' partials in
// tile order.  Nothing a segment computes depends on the other segments, so
// a system's iterates are the same bit for bit whether it is solved alone
// or with any others.
//
// Per iteration:  Ap = A p;  tile partials of p.Ap
//                 alpha_s = rz_s / (p.Ap)_s;  x += alpha p, r -= alpha Ap
//                   (tiles of active segments)  [+ tile partials of r.r]
//                 z = M r;  tile partials of r.z
//                 per segment: rr, beta = rz_new / rz, it++, active?
//                 p = z + beta p  (active segments)
// The loop (one CUDA graph with a conditional while-node) runs while any
// segment is active; converged segments keep their x, r and counters.
// No reference counterpart: the reference solves one system per call.

#include <algorithm>
#include <vector>

#include "gbpc_common.cuh"
#include "gbpc_internal.h"

namespace gbpc {
namespace {

constexpr int kTile = 4096;         // rows per tile
constexpr int kMThreads = 512;      // threads per CTA of the tile kernels
constexpr int kMMaxCtas = 4 * kSms;
constexpr int kFinThreads = 256;    // one warp per segment in the finalize kernel

struct SegScalars {
  double bb, atol_sq, rr, rz, beta;
  int it, active, maxiter, pad;
};

struct MultiCtl {
  double tol, atol;
  unsigned long long cond_handle;
  int nseg, any_active;
  unsigned int active_count, done_ctas;
};

struct Tiles {
  int ntiles;
  const int32_t* seg;     // segment of tile t
  const int64_t* begin;   // first row of tile t
  const int64_t* end;     // one past its last row
  const int32_t* seg_off; // tiles of segment s: [seg_off[s], seg_off[s + 1])
};

__device__ __forceinline__ bool ctl_off(const MultiCtl* c) {
  return *(volatile const int*)&c->any_active == 0;
}

// Sum over a 512-thread CTA in a fixed order; valid in warp 0.
__device__ __forceinline__ double cta_sum(double v, double* sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (warp == 0) {
    t = lane < kMThreads / 32 ? sh[lane] : 0.0;
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  }
  __syncthreads();
  return t;
}

// A segment's total: its tiles' partials, lane-strided, then a fixed
// butterfly (called by one full warp; every lane returns the total).
__device__ __forceinline__ double seg_total(const double* partials, int lo, int hi) {
  const int lane = threadIdx.x & 31;
  double v = 0.0;
  for (int t = lo + lane; t < hi; t += 32) v += __ldcg(partials + t);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// partials[t] = x.y over tile t (0 for tiles of inactive segments when
// skip_inactive).
__global__ void __launch_bounds__(kMThreads)
tile_dot_kernel(Tiles tl, const SegScalars* segs, const MultiCtl* ctl, bool skip_inactive,
                const double* x, const double* y, double* partials) {
  __shared__ double sh[kMThreads / 32];
  if (skip_inactive && ctl_off(ctl)) return;
  for (int t = blockIdx.x; t < tl.ntiles; t += gridDim.x) {
    const int s = tl.seg[t];
    double part = 0.0;
    if (!skip_inactive || segs[s].active) {
      const int64_t e = tl.end[t];
      for (int64_t i = tl.begin[t] + threadIdx.x; i < e; i += kMThreads)
        part = fma(x[i], y[i], part);
    }
    const double tot = cta_sum(part, sh);
    if (threadIdx.x == 0) partials[t] = tot;
  }
}

// x += alpha_s p; r -= alpha_s Ap on the tiles of active segments, with
// alpha_s = rz_s / (p.Ap)_s from the p.Ap tile partials; rr partials.
__global__ void __launch_bounds__(kMThreads)
tile_update_kernel(Tiles tl, const SegScalars* segs, const MultiCtl* ctl, const double* pap,
                   double* x, double* r, const double* p, const double* Ap, double* rr_part) {
  __shared__ double sh[kMThreads / 32];
  __shared__ double alpha_sh;
  if (ctl_off(ctl)) return;
  for (int t = blockIdx.x; t < tl.ntiles; t += gridDim.x) {
    const int s = tl.seg[t];
    if (!segs[s].active) continue;  // uniform over the CTA
    if (threadIdx.x < 32) {
      const double den = seg_total(pap, tl.seg_off[s], tl.seg_off[s + 1]);
      if (threadIdx.x == 0) alpha_sh = segs[s].rz / den;
    }
    __syncthreads();
    const double alpha = alpha_sh;
    double part = 0.0;
    const int64_t e = tl.end[t];
    for (int64_t i = tl.begin[t] + threadIdx.x; i < e; i += kMThreads) {
      x[i] = fma(alpha, p[i], x[i]);
      const double ri = fma(-alpha, Ap[i], r[i]);
      r[i] = ri;
      part = fma(ri, ri, part);
    }
    const double tot = cta_sum(part, sh);
    if (threadIdx.x == 0) rr_part[t] = tot;
  }
}

// p = z + beta_s p on the tiles of active segments.
__global__ void __launch_bounds__(kMThreads)
tile_xpay_kernel(Tiles tl, const SegScalars* segs, const MultiCtl* ctl, const double* z,
                 double* p) {
  if (ctl_off(ctl)) return;
  for (int t = blockIdx.x; t < tl.ntiles; t += gridDim.x) {
    const int s = tl.seg[t];
    if (!segs[s].active) continue;
    const double beta = segs[s].beta;
    const int64_t e = tl.end[t];
    for (int64_t i = tl.begin[t] + threadIdx.x; i < e; i += kMThreads) p[i] = fma(beta, p[i], z[i]);
  }
}

enum MFin : int { MF_INIT = 0, MF_INIT_RZ = 1, MF_BETA = 2 };

// One warp per segment: MF_INIT (a = b.b, b = r.r partials) sets bb, rr,
// atol_sq, it = 0, active; MF_INIT_RZ (a = r.z) sets rz; MF_BETA (a = r.r,
// b = r.z partials) finishes an iteration of the active segments.  The last
// CTA to finish publishes whether any segment is still active (and sets the
// while-node's condition).
__global__ void __launch_bounds__(kFinThreads)
seg_finalize_kernel(int mode, Tiles tl, SegScalars* segs, MultiCtl* ctl, const double* pa,
                    const double* pb, bool guarded) {
  __shared__ bool am_last;
  if (guarded && ctl_off(ctl)) return;
  const int lane = threadIdx.x & 31;
  const int s = blockIdx.x * (kFinThreads / 32) + (threadIdx.x >> 5);
  unsigned int active = 0;
  if (s < ctl->nseg) {
    const int lo = tl.seg_off[s], hi = tl.seg_off[s + 1];
    const double a = seg_total(pa, lo, hi);
    const double b = pb ? seg_total(pb, lo, hi) : 0.0;
    SegScalars& g = segs[s];
    if (lane == 0) {
      if (mode == MF_INIT) {
        g.bb = a;
        g.rr = b;
        const double at = fmax(ctl->atol, ctl->tol * sqrt(a));
        g.atol_sq = at * at;
        g.it = 0;
        g.beta = 0.0;
        g.active = (g.rr > g.atol_sq) && (g.it < g.maxiter);
      } else if (mode == MF_INIT_RZ) {
        g.rz = a;
      } else if (g.active) {
        g.rr = a;
        g.beta = b / g.rz;
        g.rz = b;
        g.it += 1;
        g.active = (g.rr > g.atol_sq) && (g.it < g.maxiter);
      }
      active = g.active ? 1u : 0u;
    }
  }
  if (mode == MF_INIT_RZ) return;
  if (lane == 0 && active) atomicAdd(&ctl->active_count, 1u);
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) am_last = atomicAdd(&ctl->done_ctas, 1u) == gridDim.x - 1;
  __syncthreads();
  if (am_last && threadIdx.x == 0) {
    __threadfence();
    const unsigned int count = atomicAdd(&ctl->active_count, 0u);
    ctl->any_active = count > 0u;
    ctl->active_count = 0u;
    ctl->done_ctas = 0u;
    if (ctl->cond_handle != 0ull)
      cudaGraphSetConditional((cudaGraphConditionalHandle)ctl->cond_handle, count ? 1u : 0u);
  }
}

__global__ void mset_kernel(MultiCtl* ctl, SegScalars* segs, const int64_t* seg_rows, int nseg,
                            double tol, double atol, int maxiter, unsigned long long handle) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s == 0) {
    ctl->tol = tol;
    ctl->atol = atol;
    ctl->cond_handle = handle;
    ctl->nseg = nseg;
    ctl->any_active = 1;
    ctl->active_count = 0u;
    ctl->done_ctas = 0u;
  }
  if (s < nseg) {
    const int64_t rows = seg_rows[s + 1] - seg_rows[s];
    segs[s].maxiter = maxiter > 0 ? maxiter : (rows < 0x7fffffff ? (int)rows : 0x7fffffff);
  }
}

__global__ void mcopy_outputs_kernel(const SegScalars* segs, int nseg, int32_t* nit, double* rr,
                                     double* atol_sq) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  if (nit) nit[s] = segs[s].it;
  if (rr) rr[s] = segs[s].rr;
  if (atol_sq) atol_sq[s] = segs[s].atol_sq;
}

}  // namespace

struct MultiSolver {
  Operator* A = nullptr;
  Operator* M = nullptr;
  int64_t n = 0;
  int nseg = 0, ntiles = 0, unroll = 4;
  bool use_graph = true;
  size_t device_bytes = 0;
  DevBuf r, z, p, Ap, pa, pb, pc, segs, ctl, tile_seg, tile_begin, tile_end, seg_tiles, seg_rows;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraphConditionalHandle handle = 0;
  const double* last_b = nullptr;
  double* last_x = nullptr;

  ~MultiSolver() { drop_graph(); }
  void drop_graph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
  }
  Tiles tiles() const {
    return Tiles{ntiles, tile_seg.as<int32_t>(), tile_begin.as<int64_t>(), tile_end.as<int64_t>(),
                 seg_tiles.as<int32_t>()};
  }
  SegScalars* S() const { return segs.as<SegScalars>(); }
  MultiCtl* C() const { return ctl.as<MultiCtl>(); }
  int tile_grid() const { return std::max(1, std::min(ntiles, kMMaxCtas)); }
  int fin_grid() const { return std::max(1, (nseg + kFinThreads / 32 - 1) / (kFinThreads / 32)); }

  int precondition(const double* in, double* out, const int* guard, cudaStream_t st) {
    if (M) return M->apply(in, nullptr, out, 1.0, 0.0, guard, nullptr, st);
    // Identity: a plain copy (it also runs once every segment has converged;
    // nothing reads z then).
    GBPC_CUDA_TRY(cudaMemcpyAsync(out, in, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    return GBPC_OK;
  }

  int record_init(const double* b, double* x, cudaStream_t st) {
    int rc;
    const Tiles tl = tiles();
    if ((rc = A->apply(x, b, r.p, -1.0, 1.0, nullptr, nullptr, st))) return rc;
    tile_dot_kernel<<<tile_grid(), kMThreads, 0, st>>>(tl, S(), C(), false, b, b, pa.as<double>());
    tile_dot_kernel<<<tile_grid(), kMThreads, 0, st>>>(tl, S(), C(), false, r.as<double>(),
                                                       r.as<double>(), pb.as<double>());
    seg_finalize_kernel<<<fin_grid(), kFinThreads, 0, st>>>(MF_INIT, tl, S(), C(), pa.as<double>(),
                                                            pb.as<double>(), false);
    GBPC_CUDA_TRY(cudaGetLastError());
    if ((rc = precondition(r.as<double>(), z.as<double>(), nullptr, st))) return rc;
    tile_dot_kernel<<<tile_grid(), kMThreads, 0, st>>>(tl, S(), C(), false, r.as<double>(),
                                                       z.as<double>(), pa.as<double>());
    seg_finalize_kernel<<<fin_grid(), kFinThreads, 0, st>>>(MF_INIT_RZ, tl, S(), C(),
                                                            pa.as<double>(), nullptr, false);
    GBPC_CUDA_TRY(cudaGetLastError());
    GBPC_CUDA_TRY(cudaMemcpyAsync(p.p, z.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    return GBPC_OK;
  }

  int record_iteration(double* x, cudaStream_t st) {
    int rc;
    const Tiles tl = tiles();
    const int* guard = &C()->any_active;
    if ((rc = A->apply(p.p, nullptr, Ap.p, 1.0, 0.0, guard, nullptr, st))) return rc;
    tile_dot_kernel<<<tile_grid(), kMThreads, 0, st>>>(tl, S(), C(), true, p.as<double>(),
                                                       Ap.as<double>(), pa.as<double>());
    tile_update_kernel<<<tile_grid(), kMThreads, 0, st>>>(tl, S(), C(), pa.as<double>(), x,
                                                          r.as<double>(), p.as<double>(),
                                                          Ap.as<double>(), pb.as<double>());
    GBPC_CUDA_TRY(cudaGetLastError());
    if ((rc = precondition(r.as<double>(), z.as<double>(), guard, st))) return rc;
    tile_dot_kernel<<<tile_grid(), kMThreads, 0, st>>>(tl, S(), C(), true, r.as<double>(),
                                                       z.as<double>(), pc.as<double>());
    seg_finalize_kernel<<<fin_grid(), kFinThreads, 0, st>>>(MF_BETA, tl, S(), C(), pb.as<double>(),
                                                            pc.as<double>(), true);
    tile_xpay_kernel<<<tile_grid(), kMThreads, 0, st>>>(tl, S(), C(), z.as<double>(),
                                                        p.as<double>());
    GBPC_CUDA_TRY(cudaGetLastError());
    return GBPC_OK;
  }

  int build_graph(const double* b, double* x, cudaStream_t st) {
    drop_graph();
    GBPC_CUDA_TRY(cudaGraphCreate(&graph, 0));
    GBPC_CUDA_TRY(cudaGraphConditionalHandleCreate(&handle, graph, 0, cudaGraphCondAssignDefault));
    cudaStream_t cs;
    GBPC_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    int rc = GBPC_OK;
    do {
      if (cudaStreamBeginCaptureToGraph(cs, graph, nullptr, nullptr, 0,
                                        cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        gbpc_set_error("multi-system solver: begin capture failed");
        rc = GBPC_ERR_CUDA;
        break;
      }
      rc = record_init(b, x, cs);
      cudaGraph_t g2 = nullptr;
      cudaError_t e = cudaStreamEndCapture(cs, &g2);
      if (rc) break;
      if (e != cudaSuccess) {
        gbpc_set_error_cuda(e, "capture init", __FILE__, __LINE__);
        rc = GBPC_ERR_CUDA;
        break;
      }
      size_t count = 0;
      cudaGraphGetNodes(graph, nullptr, &count);
      std::vector<cudaGraphNode_t> nodes(count);
      cudaGraphGetNodes(graph, nodes.data(), &count);
      cudaGraphNode_t tail = nullptr;
      for (auto nd : nodes) {
        size_t outs = 0;
        cudaGraphNodeGetDependentNodes(nd, nullptr, nullptr, &outs);
        if (outs == 0) tail = nd;
      }
      cudaGraphNodeParams cp = {};
      cp.type = cudaGraphNodeTypeConditional;
      cp.conditional.handle = handle;
      cp.conditional.type = cudaGraphCondTypeWhile;
      cp.conditional.size = 1;
      cudaGraphNode_t cnode;
      e = cudaGraphAddNode(&cnode, graph, tail ? &tail : nullptr, nullptr, tail ? 1 : 0, &cp);
      if (e != cudaSuccess) {
        gbpc_set_error_cuda(e, "add conditional node", __FILE__, __LINE__);
        rc = GBPC_ERR_CUDA;
        break;
      }
      cudaGraph_t body = cp.conditional.phGraph_out[0];
      if (cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0,
                                        cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        gbpc_set_error("multi-system solver: begin body capture failed");
        rc = GBPC_ERR_CUDA;
        break;
      }
      for (int u = 0; u < unroll && !rc; ++u) rc = record_iteration(x, cs);
      e = cudaStreamEndCapture(cs, &g2);
      if (rc) break;
      if (e != cudaSuccess) {
        gbpc_set_error_cuda(e, "capture body", __FILE__, __LINE__);
        rc = GBPC_ERR_CUDA;
        break;
      }
      e = cudaGraphInstantiate(&exec, graph, 0);
      if (e != cudaSuccess) {
        gbpc_set_error_cuda(e, "instantiate", __FILE__, __LINE__);
        rc = GBPC_ERR_CUDA;
      }
    } while (false);
    cudaStreamDestroy(cs);
    if (rc) {
      drop_graph();
      cudaGetLastError();
      return rc;
    }
    last_b = b;
    last_x = x;
    return GBPC_OK;
  }

  int run(const double* b, double* x, double tol, double atol, int maxiter, int32_t* nit_dev,
          double* rr_dev, double* atol_sq_dev, cudaStream_t st) {
    int rc;
    if (use_graph) {
      if (!exec || last_b != b || last_x != x)
        if ((rc = build_graph(b, x, st))) return rc;
      mset_kernel<<<grid_for(nseg, 256), 256, 0, st>>>(C(), S(), seg_rows.as<int64_t>(), nseg, tol,
                                                       atol, maxiter, (unsigned long long)handle);
      GBPC_CUDA_TRY(cudaGetLastError());
      GBPC_CUDA_TRY(cudaGraphLaunch(exec, st));
    } else {
      mset_kernel<<<grid_for(nseg, 256), 256, 0, st>>>(C(), S(), seg_rows.as<int64_t>(), nseg, tol,
                                                       atol, maxiter, 0ull);
      GBPC_CUDA_TRY(cudaGetLastError());
      if ((rc = record_init(b, x, st))) return rc;
      int active = 1;
      while (active) {
        for (int k = 0; k < 16; ++k)
          if ((rc = record_iteration(x, st))) return rc;
        GBPC_CUDA_TRY(cudaMemcpyAsync(&active, &C()->any_active, sizeof(int),
                                      cudaMemcpyDeviceToHost, st));
        GBPC_CUDA_TRY(cudaStreamSynchronize(st));
      }
    }
    if (nit_dev || rr_dev || atol_sq_dev)
      mcopy_outputs_kernel<<<grid_for(nseg, 256), 256, 0, st>>>(S(), nseg, nit_dev, rr_dev,
                                                                atol_sq_dev);
    GBPC_CUDA_TRY(cudaGetLastError());
    return GBPC_OK;
  }
};

}  // namespace gbpc

using namespace gbpc;

struct gbpc_msolver {
  MultiSolver s;
};

extern "C" int gbpc_msolver_create(gbpc_op* A, gbpc_op* M, int nseg, const int64_t* seg_rows_host,
                                   int use_graph, int unroll, void* stream, gbpc_msolver** out) {
  if (!out || !A || !A->impl || nseg < 1 || !seg_rows_host) {
    gbpc_set_error("gbpc_msolver_create: bad arguments");
    return GBPC_ERR_ARG;
  }
  Operator* a = A->impl.get();
  Operator* m = (M && M->impl) ? M->impl.get() : nullptr;
  if (a->vdtype != GBPC_F64 || (m && m->vdtype != GBPC_F64)) {
    gbpc_set_error("the multi-system solver runs on float64 vectors");
    return GBPC_ERR_ARG;
  }
  if (m && m->rows != a->rows) {
    gbpc_set_error("operator and preconditioner sizes differ (%lld vs %lld)", (long long)a->rows,
                   (long long)m->rows);
    return GBPC_ERR_ARG;
  }
  if (seg_rows_host[0] != 0 || seg_rows_host[nseg] != a->rows) {
    gbpc_set_error("segment offsets must start at 0 and end at the operator's %lld rows",
                   (long long)a->rows);
    return GBPC_ERR_ARG;
  }
  // Tiles: each segment cut into pieces of at most kTile rows.
  std::vector<int32_t> tseg, stile(nseg + 1, 0);
  std::vector<int64_t> tbeg, tend;
  for (int s = 0; s < nseg; ++s) {
    const int64_t lo = seg_rows_host[s], hi = seg_rows_host[s + 1];
    if (hi < lo) {
      gbpc_set_error("segment offsets must be nondecreasing (segment %d)", s);
      return GBPC_ERR_ARG;
    }
    for (int64_t b = lo; b < hi; b += kTile) {
      tseg.push_back(s);
      tbeg.push_back(b);
      tend.push_back(std::min<int64_t>(b + kTile, hi));
    }
    if (tseg.size() > 0x7fffffff) {
      gbpc_set_error("too many tiles");
      return GBPC_ERR_ARG;
    }
    stile[s + 1] = (int32_t)tseg.size();
  }
  cudaStream_t st = (cudaStream_t)stream;
  auto* h = new gbpc_msolver;
  MultiSolver& s = h->s;
  ByteTally tally(&s.device_bytes);
  s.A = a;
  s.M = m;
  s.n = a->rows;
  s.nseg = nseg;
  s.ntiles = (int)tseg.size();
  s.use_graph = use_graph != 0;
  if (unroll > 0) s.unroll = std::min(unroll, 64);
  const size_t vb = sizeof(double) * std::max<int64_t>(s.n, 1);
  const size_t tb = sizeof(double) * std::max(s.ntiles, 1);
  int rc = GBPC_OK;
  for (DevBuf* d : {&s.r, &s.z, &s.p, &s.Ap})
    if (!rc) rc = d->alloc(vb);
  for (DevBuf* d : {&s.pa, &s.pb, &s.pc})
    if (!rc) rc = d->alloc(tb);
  if (!rc) rc = s.segs.alloc(sizeof(SegScalars) * nseg);
  if (!rc) rc = s.ctl.alloc(sizeof(MultiCtl));
  if (!rc) rc = s.tile_seg.alloc(sizeof(int32_t) * std::max(s.ntiles, 1));
  if (!rc) rc = s.tile_begin.alloc(sizeof(int64_t) * std::max(s.ntiles, 1));
  if (!rc) rc = s.tile_end.alloc(sizeof(int64_t) * std::max(s.ntiles, 1));
  if (!rc) rc = s.seg_tiles.alloc(sizeof(int32_t) * (nseg + 1));
  if (!rc) rc = s.seg_rows.alloc(sizeof(int64_t) * (nseg + 1));
  if (!rc) {
    cudaError_t e = cudaMemsetAsync(s.segs.p, 0, sizeof(SegScalars) * nseg, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(s.ctl.p, 0, sizeof(MultiCtl), st);
    if (e == cudaSuccess && s.ntiles > 0) {
      e = cudaMemcpyAsync(s.tile_seg.p, tseg.data(), sizeof(int32_t) * s.ntiles,
                          cudaMemcpyHostToDevice, st);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(s.tile_begin.p, tbeg.data(), sizeof(int64_t) * s.ntiles,
                            cudaMemcpyHostToDevice, st);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(s.tile_end.p, tend.data(), sizeof(int64_t) * s.ntiles,
                            cudaMemcpyHostToDevice, st);
    }
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(s.seg_tiles.p, stile.data(), sizeof(int32_t) * (nseg + 1),
                          cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(s.seg_rows.p, seg_rows_host, sizeof(int64_t) * (nseg + 1),
                          cudaMemcpyHostToDevice, st);
    // The host vectors above are pageable and go out of scope: finish the copies.
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      gbpc_set_error_cuda(e, "gbpc_msolver_create", __FILE__, __LINE__);
      rc = GBPC_ERR_CUDA;
    }
  }
  if (rc) {
    delete h;
    return rc;
  }
  *out = h;
  return GBPC_OK;
}

extern "C" int gbpc_msolver_run(gbpc_msolver* h, const double* b, double* x, double tol,
                                double atol, int maxiter, int32_t* nit_dev, double* rr_dev,
                                double* atol_sq_dev, void* stream) {
  NvtxRange nvtx_range("gbpc_msolver_run");
  if (!h || (h->s.n > 0 && (!b || !x))) {
    gbpc_set_error("gbpc_msolver_run: bad arguments");
    return GBPC_ERR_ARG;
  }
  return h->s.run(b, x, tol, atol, maxiter, nit_dev, rr_dev, atol_sq_dev, (cudaStream_t)stream);
}

extern "C" int gbpc_msolver_device_bytes(const gbpc_msolver* h, size_t* bytes_host) {
  if (!h || !bytes_host) {
    gbpc_set_error("gbpc_msolver_device_bytes: bad arguments");
    return GBPC_ERR_ARG;
  }
  *bytes_host = h->s.device_bytes;
  return GBPC_OK;
}

extern "C" int gbpc_msolver_destroy(gbpc_msolver* h) {
  if (!h) return GBPC_OK;
  cudaDeviceSynchronize();
  delete h;
  return GBPC_OK;
}
