// Preconditioned CG and CR with the whole loop on the device.
//
// The reference runs warp.optim.linear.cg / cr (warp-lang, not vendored) with
// check_every=0 inside a captured CUDA graph whose while-condition is the
// recursive residual test.  Here one CUDA graph holds the initialisation and
// a conditional while-node whose body is one iteration; the last kernel of
// each iteration decides whether the loop continues (r.r > max(atol,
// tol |b|)^2 and it < maxiter), so a solve is a single graph launch with no
// host round trip.  Every reduction is fused into the kernel that produces
// the vector being reduced and is summed deterministically.
//
// Per iteration (PCG):  Ap = A p  [+ p.Ap -> alpha]
//                       x += alpha p, r -= alpha Ap  [+ r.r]
//                       z = M r  [+ r.z -> beta, it++, continue?]
//                       p = z + beta p
// Per iteration (PCR):  y = M Ap  [+ Ap.y -> alpha]
//                       x += alpha p, r -= alpha Ap, z -= alpha y  [+ r.r]
//                       Az = A z  [+ z.Az -> beta, it++, continue?]
//                       p = z + beta p, Ap = Az + beta Ap

#include <algorithm>
#include <vector>

#include "gbpc_common.cuh"
#include "gbpc_internal.h"

namespace gbpc {

int copy_with_dot(int64_t n, const double* x, double* z, const int* guard, const Reduction& red,
                  cudaStream_t st);

namespace {

__device__ __forceinline__ bool inactive(const KrylovScalars* ks) {
  return *(volatile const int*)&ks->active == 0;
}

// x += alpha p; r -= alpha Ap; reduce r.r.  R32: also r32 = (float) r, the
// input of a float32-applied preconditioner (no separate conversion pass).
template <bool R32>
__global__ void __launch_bounds__(kThreads, kCtasPerSm)
cg_update_kernel(int64_t n, KrylovScalars* ks, double* x, double* r, const double* p,
                 const double* Ap, float* r32, Reduction red) {
  // x and p are not written by the previous kernel (the operator apply that
  // produced Ap), so a thread's first row of them is read before the wait.
  const int64_t i0 = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  double x0 = 0.0, p0 = 0.0;
  if (i0 < n) {
    x0 = x[i0];
    p0 = p[i0];
  }
  pdl_wait();
  pdl_launch_dependents();
  if (inactive(ks)) return;
  const double alpha = ks->alpha;
  double part = 0.0;
  for (int64_t i = i0; i < n; i += (int64_t)gridDim.x * kThreads) {
    const bool first = i == i0;
    x[i] = fma(alpha, first ? p0 : p[i], first ? x0 : x[i]);
    const double ri = fma(-alpha, Ap[i], r[i]);
    r[i] = ri;
    if (R32) r32[i] = (float)ri;
    part = fma(ri, ri, part);
  }
  reduce_and_finalize(red, part);
}

// x += alpha p; r -= alpha Ap; z -= alpha y; reduce r.r
__global__ void __launch_bounds__(kThreads, kCtasPerSm)
cr_update_kernel(int64_t n, KrylovScalars* ks, double* x, double* r, double* z, const double* p,
                 const double* Ap, const double* y, Reduction red) {
  pdl_wait();
  pdl_launch_dependents();
  if (inactive(ks)) return;
  const double alpha = ks->alpha;
  double part = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kThreads) {
    x[i] = fma(alpha, p[i], x[i]);
    const double ri = fma(-alpha, Ap[i], r[i]);
    r[i] = ri;
    z[i] = fma(-alpha, y[i], z[i]);
    part = fma(ri, ri, part);
  }
  reduce_and_finalize(red, part);
}

// p = z + beta p  (and q = w + beta q with Q: CR).  Q is a template
// parameter so that CG issues no FP64 instruction for the absent q.  Z is
// float for a float32-applied preconditioner (z widened on the fly).
template <bool Q, typename Z = double>
__global__ void __launch_bounds__(kThreads, kCtasPerSm)
xpay_kernel(int64_t n, const KrylovScalars* ks, const Z* z, double* p, const double* w,
            double* q) {
  // p (and q) were last written an iteration ago, not by the previous
  // kernel: a thread's first row of them is read before the wait.
  const int64_t i0 = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  double p0 = 0.0, q0 = 0.0;
  if (i0 < n) {
    p0 = p[i0];
    if (Q) q0 = q[i0];
  }
  pdl_wait();
  pdl_launch_dependents();
  if (inactive(ks)) return;
  const double beta = ks->beta;
  for (int64_t i = i0; i < n; i += (int64_t)gridDim.x * kThreads) {
    const bool first = i == i0;
    p[i] = fma(beta, first ? p0 : p[i], (double)z[i]);
    if (Q) q[i] = fma(beta, first ? q0 : q[i], w[i]);
  }
}

// dot(a, b) into the reduction's finalize action (initialisation only).
__global__ void __launch_bounds__(kThreads, kCtasPerSm)
dot_kernel(int64_t n, const double* a, const double* b, Reduction red) {
  double part = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kThreads)
    part = fma(a[i], b[i], part);
  reduce_and_finalize(red, part);
}

// r32 = (float) r (initialisation of the float32-preconditioned loop).
__global__ void narrow_copy_kernel(int64_t n, const double* r, float* r32) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    r32[i] = (float)r[i];
}

// p = (double) z32.
__global__ void widen_copy_kernel(int64_t n, const float* z32, double* p) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    p[i] = (double)z32[i];
}

__global__ void set_scalars_kernel(KrylovScalars* ks, double tol, double atol, int maxiter,
                                   unsigned long long handle, double* hist, int hist_len) {
  ks->tol = tol;
  ks->atol = atol;
  ks->maxiter = maxiter;
  ks->it = 0;
  ks->active = 1;
  ks->cond_handle = handle;
  ks->hist = hist;
  ks->hist_len = hist ? hist_len : 0;
}

__global__ void copy_outputs_kernel(const KrylovScalars* ks, int32_t* nit, double* rr,
                                    double* atol_sq) {
  if (nit) *nit = ks->it;
  if (rr) *rr = ks->rr;
  if (atol_sq) *atol_sq = ks->atol_sq;
}

int vec_grid(int64_t n) { return std::min<int64_t>(grid_for(n, kThreads), kSms * kCtasPerSm); }

}  // namespace

struct Solver {
  size_t device_bytes = 0;  // DevBuf bytes held (declared first: released last)
  int method = GBPC_CG;
  Operator* A = nullptr;
  Operator* M = nullptr;
  // M applied in float32 behind a float64 interface: CG writes its float32
  // input (low->in32) in the update kernel and reads its float32 output
  // (low->out32) in the direction update, so only low->inner runs per
  // iteration (CR uses M's own float64 interface).
  LowPrecisionOp* low = nullptr;
  int64_t n = 0;
  bool use_graph = true;
  int unroll = 8;  // iterations per pass of the device loop (measured: 1 -> 8 saves ~4 us/iteration)
  double* hist = nullptr;  // residual history of the next runs (gbpc_solver_set_history)
  int hist_len = 0;
  bool use_pdl = true;  // programmatic dependent launches inside the loop body
  DevBuf r, z, p, Ap, Az, y, ks, zeros;
  ReduceBuf rb;
  // Cached graph for the last (b, x) pair.
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphConditionalHandle handle = 0;
  const double* last_b = nullptr;
  double* last_x = nullptr;

  ~Solver() { drop_graph(); }
  void drop_graph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
    last_b = nullptr;
    last_x = nullptr;
  }

  KrylovScalars* K() { return ks.as<KrylovScalars>(); }

  DotSpec dot(const double* w, int mode) {
    DotSpec d;
    d.w = w;
    d.rb = &rb;
    d.mode = mode;
    d.ks = K();
    return d;
  }

  // z = M r (identity when M is null), with the fused dot(w, z).
  int precondition(const double* in, double* out, const int* guard, const DotSpec* d,
                   cudaStream_t st) {
    if (M) return M->apply(in, nullptr, out, 1.0, 0.0, guard, d, st);
    Reduction red{};
    if (d) {
      red.w = d->w;
      red.partials = rb.partials.as<double>();
      red.counter = rb.counter.as<unsigned int>();
      red.mode = d->mode;
      red.ks = K();
    }
    // Identity preconditioner: out = in with the fused dot.
    return copy_with_dot(n, in, out, guard, red, st);
  }

  // Initialisation: r = b - A x, bb, rr, z = M r, rz (or zAz for CR), p, Ap.
  int record_init(const double* b, double* x, cudaStream_t st) {
    int rc;
    GBPC_CUDA_TRY(cudaMemsetAsync(rb.counter.p, 0, sizeof(unsigned int), st));
    Reduction rbb{};
    rbb.partials = rb.partials.as<double>();
    rbb.counter = rb.counter.as<unsigned int>();
    rbb.mode = FIN_INIT_BB;
    rbb.ks = K();
    rbb.w = b;
    dot_kernel<<<vec_grid(n), kThreads, 0, st>>>(n, b, b, rbb);
    GBPC_CUDA_TRY(cudaGetLastError());
    DotSpec drr = dot(r.as<double>(), FIN_INIT_RR);
    if ((rc = A->apply(x, b, r.p, -1.0, 1.0, nullptr, &drr, st))) return rc;
    // z = M r, rz = r.z   (set_active already ran; inactive solves still
    // compute these harmless initial quantities).
    if (method == GBPC_CG && low) {
      DotSpec drz = dot(r.as<double>(), FIN_INIT_RZ);
      narrow_copy_kernel<<<vec_grid(n), kThreads, 0, st>>>(n, r.as<double>(), low->in32.as<float>());
      GBPC_CUDA_TRY(cudaGetLastError());
      if ((rc = low->inner->apply(low->in32.p, nullptr, low->out32.p, 1.0, 0.0, nullptr, &drz, st)))
        return rc;
      widen_copy_kernel<<<vec_grid(n), kThreads, 0, st>>>(n, low->out32.as<float>(), p.as<double>());
      GBPC_CUDA_TRY(cudaGetLastError());
    } else if (method == GBPC_CG) {
      DotSpec drz = dot(r.as<double>(), FIN_INIT_RZ);
      if ((rc = precondition(r.as<double>(), z.as<double>(), nullptr, &drz, st))) return rc;
      GBPC_CUDA_TRY(cudaMemcpyAsync(p.p, z.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    } else {
      if ((rc = precondition(r.as<double>(), z.as<double>(), nullptr, nullptr, st))) return rc;
      DotSpec dza = dot(z.as<double>(), FIN_INIT_RZ);
      if ((rc = A->apply(z.p, nullptr, Az.p, 1.0, 0.0, nullptr, &dza, st))) return rc;
      GBPC_CUDA_TRY(cudaMemcpyAsync(p.p, z.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
      GBPC_CUDA_TRY(cudaMemcpyAsync(Ap.p, Az.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    }
    return GBPC_OK;
  }

  int record_iteration(double* x, cudaStream_t st) {
    int rc;
    const int* guard = &K()->active;
    Reduction rrr{};
    rrr.partials = rb.partials.as<double>();
    rrr.counter = rb.counter.as<unsigned int>();
    rrr.mode = FIN_RR;
    rrr.ks = K();
    rrr.w = r.as<double>();
    if (method == GBPC_CG && low) {
      DotSpec da = dot(p.as<double>(), FIN_CG_ALPHA);
      if ((rc = A->apply(p.p, nullptr, Ap.p, 1.0, 0.0, guard, &da, st))) return rc;
      GBPC_CUDA_TRY(launch_k(cg_update_kernel<true>, vec_grid(n), kThreads, 0, st, n, K(), x,
                             r.as<double>(), (const double*)p.as<double>(),
                             (const double*)Ap.as<double>(), low->in32.as<float>(), rrr));
      DotSpec db = dot(r.as<double>(), FIN_CG_BETA);
      if ((rc = low->inner->apply(low->in32.p, nullptr, low->out32.p, 1.0, 0.0, guard, &db, st)))
        return rc;
      GBPC_CUDA_TRY(launch_k(xpay_kernel<false, float>, vec_grid(n), kThreads, 0, st, n,
                             (const KrylovScalars*)K(), (const float*)low->out32.as<float>(),
                             p.as<double>(), (const double*)nullptr, (double*)nullptr));
    } else if (method == GBPC_CG) {
      DotSpec da = dot(p.as<double>(), FIN_CG_ALPHA);
      if ((rc = A->apply(p.p, nullptr, Ap.p, 1.0, 0.0, guard, &da, st))) return rc;
      GBPC_CUDA_TRY(launch_k(cg_update_kernel<false>, vec_grid(n), kThreads, 0, st, n, K(), x,
                             r.as<double>(), (const double*)p.as<double>(),
                             (const double*)Ap.as<double>(), (float*)nullptr, rrr));
      DotSpec db = dot(r.as<double>(), FIN_CG_BETA);
      if ((rc = precondition(r.as<double>(), z.as<double>(), guard, &db, st))) return rc;
      GBPC_CUDA_TRY(launch_k(xpay_kernel<false>, vec_grid(n), kThreads, 0, st, n,
                             (const KrylovScalars*)K(), (const double*)z.as<double>(),
                             p.as<double>(), (const double*)nullptr, (double*)nullptr));
    } else {
      DotSpec da = dot(Ap.as<double>(), FIN_CR_ALPHA);
      if ((rc = precondition(Ap.as<double>(), y.as<double>(), guard, &da, st))) return rc;
      GBPC_CUDA_TRY(launch_k(cr_update_kernel, vec_grid(n), kThreads, 0, st, n, K(), x,
                             r.as<double>(), z.as<double>(), (const double*)p.as<double>(),
                             (const double*)Ap.as<double>(), (const double*)y.as<double>(), rrr));
      DotSpec db = dot(z.as<double>(), FIN_CG_BETA);
      if ((rc = A->apply(z.p, nullptr, Az.p, 1.0, 0.0, guard, &db, st))) return rc;
      GBPC_CUDA_TRY(launch_k(xpay_kernel<true>, vec_grid(n), kThreads, 0, st, n,
                             (const KrylovScalars*)K(), (const double*)z.as<double>(),
                             p.as<double>(), (const double*)Az.as<double>(), Ap.as<double>()));
    }
    GBPC_CUDA_TRY(cudaGetLastError());
    return GBPC_OK;
  }

  int build_graph(const double* b, double* x, cudaStream_t st) {
    drop_graph();
    GBPC_CUDA_TRY(cudaGraphCreate(&graph, 0));
    GBPC_CUDA_TRY(cudaGraphConditionalHandleCreate(&handle, graph, 0, cudaGraphCondAssignDefault));
    // Capture the initialisation into the parent graph on a private stream.
    cudaStream_t cs;
    GBPC_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    int rc = GBPC_OK;
    cudaGraphNode_t init_tail = nullptr;
    do {
      if (cudaStreamBeginCaptureToGraph(cs, graph, nullptr, nullptr, 0,
                                        cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
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
      // The captured nodes form a chain; find its sink.
      size_t count = 0;
      cudaGraphGetNodes(graph, nullptr, &count);
      std::vector<cudaGraphNode_t> nodes(count);
      cudaGraphGetNodes(graph, nodes.data(), &count);
      for (auto nd : nodes) {
        size_t outs = 0;
        cudaGraphNodeGetDependentNodes(nd, nullptr, nullptr, &outs);
        if (outs == 0) init_tail = nd;
      }
      cudaGraphNodeParams cp = {};
      cp.type = cudaGraphNodeTypeConditional;
      cp.conditional.handle = handle;
      cp.conditional.type = cudaGraphCondTypeWhile;
      cp.conditional.size = 1;
      cudaGraphNode_t cnode;
      e = cudaGraphAddNode(&cnode, graph, init_tail ? &init_tail : nullptr, nullptr,
                           init_tail ? 1 : 0, &cp);
      if (e != cudaSuccess) {
        gbpc_set_error_cuda(e, "add conditional node", __FILE__, __LINE__);
        rc = GBPC_ERR_CUDA;
        break;
      }
      cudaGraph_t body = cp.conditional.phGraph_out[0];
      if (cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0,
                                        cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        rc = GBPC_ERR_CUDA;
        break;
      }
      // `unroll` guarded iterations per pass of the while-node: the loop
      // condition is evaluated once per pass, and iterations after
      // convergence inside a pass return immediately from every kernel.
      {
        PdlScope scope(use_pdl);
        for (int u = 0; u < unroll && !rc; ++u) rc = record_iteration(x, cs);
      }
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
        break;
      }
    } while (0);
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
    if (maxiter <= 0) maxiter = (int)std::min<int64_t>(n, 0x7fffffff);
    int rc;
    if (use_graph) {
      if (!exec || last_b != b || last_x != x) {
        rc = build_graph(b, x, st);
        if (rc && use_pdl) {  // capture without programmatic launches instead
          use_pdl = false;
          rc = build_graph(b, x, st);
        }
        if (rc) return rc;
      }
      set_scalars_kernel<<<1, 1, 0, st>>>(K(), tol, atol, maxiter, (unsigned long long)handle,
                                          hist, hist_len);
      GBPC_CUDA_TRY(cudaGetLastError());
      GBPC_CUDA_TRY(cudaGraphLaunch(exec, st));
    } else {
      set_scalars_kernel<<<1, 1, 0, st>>>(K(), tol, atol, maxiter, 0ull, hist, hist_len);
      if ((rc = record_init(b, x, st))) return rc;
      // Host-driven loop: chunks of iterations, then read the flag.
      int active = 1;
      int done = 0;
      while (active && done < maxiter) {
        const int chunk = std::min(16, maxiter - done);
        for (int k = 0; k < chunk; ++k)
          if ((rc = record_iteration(x, st))) return rc;
        done += chunk;
        GBPC_CUDA_TRY(cudaMemcpyAsync(&active, &K()->active, sizeof(int), cudaMemcpyDeviceToHost, st));
        GBPC_CUDA_TRY(cudaStreamSynchronize(st));
      }
    }
    if (nit_dev || rr_dev || atol_sq_dev)
      copy_outputs_kernel<<<1, 1, 0, st>>>(K(), nit_dev, rr_dev, atol_sq_dev);
    GBPC_CUDA_TRY(cudaGetLastError());
    return GBPC_OK;
  }
};

// Identity preconditioner helper (defined here to keep the reduction local).
__global__ void __launch_bounds__(kThreads, kCtasPerSm)
copy_dot_kernel(int64_t n, const double* x, double* z, const int* guard, Reduction red) {
  if (guard_off(guard)) return;
  double part = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kThreads) {
    const double v = x[i];
    z[i] = v;
    if (red.w) part = fma(v, red.w[i], part);
  }
  if (red.w) reduce_and_finalize(red, part);
}

int copy_with_dot(int64_t n, const double* x, double* z, const int* guard, const Reduction& red,
                  cudaStream_t st) {
  copy_dot_kernel<<<vec_grid(n), kThreads, 0, st>>>(n, x, z, guard, red);
  GBPC_CUDA_TRY(cudaGetLastError());
  return GBPC_OK;
}

}  // namespace gbpc

using namespace gbpc;

struct gbpc_solver {
  Solver s;
};

extern "C" int gbpc_solver_create(int method, gbpc_op* A, gbpc_op* M, int use_graph, int unroll,
                                  void* stream, gbpc_solver** out) {
  if (!out || !A || !A->impl || (method != GBPC_CG && method != GBPC_CR)) {
    gbpc_set_error("gbpc_solver_create: bad arguments");
    return GBPC_ERR_ARG;
  }
  Operator* a = A->impl.get();
  Operator* m = (M && M->impl) ? M->impl.get() : nullptr;
  if (a->vdtype != GBPC_F64 || (m && m->vdtype != GBPC_F64)) {
    gbpc_set_error("the Krylov solvers run on float64 vectors");
    return GBPC_ERR_ARG;
  }
  if (m && m->rows != a->rows) {
    gbpc_set_error("operator and preconditioner sizes differ (%lld vs %lld)", (long long)a->rows,
                   (long long)m->rows);
    return GBPC_ERR_ARG;
  }
  auto* h = new gbpc_solver;
  Solver& s = h->s;
  ByteTally tally(&s.device_bytes);
  s.method = method;
  s.A = a;
  s.M = m;
  s.low = dynamic_cast<LowPrecisionOp*>(m);
  s.n = a->rows;
  s.use_graph = use_graph != 0;
  if (unroll > 0) s.unroll = unroll > 64 ? 64 : unroll;
  const size_t bytes = sizeof(double) * std::max<int64_t>(s.n, 1);
  int rc = s.r.alloc(bytes);
  if (!rc) rc = s.z.alloc(bytes);
  if (!rc) rc = s.p.alloc(bytes);
  if (!rc) rc = s.Ap.alloc(bytes);
  if (!rc && method == GBPC_CR) rc = s.Az.alloc(bytes);
  if (!rc && method == GBPC_CR) rc = s.y.alloc(bytes);
  if (!rc) rc = s.ks.alloc(sizeof(KrylovScalars));
  if (!rc) rc = s.rb.init((cudaStream_t)stream);
  if (!rc && cudaMemsetAsync(s.ks.p, 0, sizeof(KrylovScalars), (cudaStream_t)stream) != cudaSuccess)
    rc = GBPC_ERR_CUDA;
  if (rc) {
    delete h;
    return rc;
  }
  *out = h;
  return GBPC_OK;
}

extern "C" int gbpc_solver_run(gbpc_solver* h, const double* b, double* x, double tol, double atol,
                               int maxiter, int32_t* nit_dev, double* rr_dev, double* atol_sq_dev,
                               void* stream) {
  NvtxRange nvtx_range("gbpc_solver_run");
  if (!h || !b || !x) {
    gbpc_set_error("gbpc_solver_run: bad arguments");
    return GBPC_ERR_ARG;
  }
  return h->s.run(b, x, tol, atol, maxiter, nit_dev, rr_dev, atol_sq_dev, (cudaStream_t)stream);
}

extern "C" int gbpc_solver_set_history(gbpc_solver* h, double* hist, int hist_len) {
  if (!h || hist_len < 0 || (hist_len > 0 && !hist)) {
    gbpc_set_error("gbpc_solver_set_history: bad arguments");
    return GBPC_ERR_ARG;
  }
  h->s.hist = hist_len > 0 ? hist : nullptr;
  h->s.hist_len = hist_len;
  return GBPC_OK;
}

extern "C" int gbpc_solver_device_bytes(const gbpc_solver* h, size_t* bytes_host) {
  if (!h || !bytes_host) {
    gbpc_set_error("gbpc_solver_device_bytes: bad arguments");
    return GBPC_ERR_ARG;
  }
  *bytes_host = h->s.device_bytes;
  return GBPC_OK;
}

extern "C" int gbpc_solver_destroy(gbpc_solver* h) {
  if (!h) return GBPC_OK;
  cudaDeviceSynchronize();
  delete h;
  return GBPC_OK;
}

extern "C" int gbpc_krylov(int method, gbpc_op* A, gbpc_op* M, const double* b, double* x,
                           double tol, double atol, int maxiter, int use_graph, int32_t* nit_dev,
                           double* rr_dev, double* atol_sq_dev, int32_t* nit_host,
                           double* rr_host, double* atol_sq_host, void* stream) {
  gbpc_solver* s = nullptr;
  int rc = gbpc_solver_create(method, A, M, use_graph, 0, stream, &s);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  DevBuf outs;
  const bool want_host = nit_host || rr_host || atol_sq_host;
  if (want_host && (rc = outs.alloc(32))) {
    gbpc_solver_destroy(s);
    return rc;
  }
  int32_t* nd = nit_dev;
  double* rd = rr_dev;
  double* ad = atol_sq_dev;
  rc = gbpc_solver_run(s, b, x, tol, atol, maxiter, nd, rd, ad, stream);
  if (!rc && want_host) {
    copy_outputs_kernel<<<1, 1, 0, st>>>(s->s.K(), (int32_t*)outs.p, (double*)outs.p + 1,
                                         (double*)outs.p + 2);
    unsigned char hbuf[32];
    if (cudaMemcpyAsync(hbuf, outs.p, 32, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
      gbpc_set_error("gbpc_krylov: readback failed");
      rc = GBPC_ERR_CUDA;
    } else {
      if (nit_host) *nit_host = *(int32_t*)hbuf;
      if (rr_host) *rr_host = ((double*)hbuf)[1];
      if (atol_sq_host) *atol_sq_host = ((double*)hbuf)[2];
    }
  }
  gbpc_solver_destroy(s);
  return rc;
}
