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

#include <cooperative_groups.h>

#include <algorithm>
#include <cstdlib>
#include <type_traits>
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

// ---------------------------------------------------------------------------
// Small systems: the whole PCG solve as one cooperative kernel.
//
// Below a few tens of thousands of rows an iteration of the graph loop is a
// handful of tiny kernels, each paying its launch and drain (~28 us per
// iteration on the 64 x 64 Laplacian against ~2 us of arithmetic).  For a
// scalar sparse operator and an FSAI (or no) preconditioner, one
// cooperative launch runs every iteration instead: the grid syncs between
// the dependent phases (5 per iteration), every CTA adds the per-CTA
// partial sums of a dot product in the same order (so every CTA holds the
// same alpha, beta and stopping decision), and the loop ends at the same
// test as the graph loop (r.r <= max(atol, tol |b|)^2 or maxiter).  Rows
// sum their entries in storage order, as in the sliced-ELL kernels.

namespace coop {

namespace cgr = cooperative_groups;

constexpr int kThreadsC = 256;  // 8 warps per CTA
// A system whose CG iteration needs at most this many multiply-adds (stored
// entries of every product, padding included, plus the vector updates)
// runs on one thread-block cluster of 16 CTAs (8 where 16 cannot be
// scheduled): the cluster's FP64 rate covers it in a few microseconds, less
// than the launches of the graph loop it replaces.  Measured: the 64 x 64
// Laplacian with FSAI w8 (~114k) runs 13.7 against 27.7 us per iteration;
// biharmonic systems of 15k-50k rows (0.7-2.2 M) ran slower on a cluster
// than on the whole GPU.
constexpr int64_t kClusterWork = 600000;

struct Mat {
  int nrow, nslices;
  const int64_t* slice_ptr;
  const int32_t* cols;
  const double* vals;
  const int32_t* perm;
};

struct Args {
  Mat A, G, GT;  // G.nslices < 0: no preconditioner
  // inv_mass != nullptr: A is the factored squared Laplacian with every
  // vertex free, A x = L ((1/m) o (L x)) + (w m) o x with L = A above.
  const double* inv_mass;
  const double* wmass;
  int64_t n;
  const double* b;
  double* x;
  double *r, *z, *p, *Ap, *t, *u;
  KrylovScalars* ks;
};

// Row epilogues of `product`, those of the sliced-ELL kernels: plain,
// (1/m) o acc, acc + (w m) o x.
enum CoopEpi : int { CE_PLAIN = 0, CE_SCALE = 1, CE_MASS = 2 };

// z = m x (one warp per slice, rows in storage order); dot_part += z . w.
__device__ __forceinline__ void product(const Mat& m, const double* x, double* z, const double* w,
                                        double& dot_part, int cta, int ncta,
                                        int epi = CE_PLAIN, const double* aux0 = nullptr,
                                        const double* aux1 = nullptr) {
  const int lane = threadIdx.x & 31;
  const int nwarps = ncta * (kThreadsC / 32);
  for (int s = cta * (kThreadsC / 32) + (threadIdx.x >> 5); s < m.nslices; s += nwarps) {
    const int64_t base = m.slice_ptr[s];
    const int width = (int)((m.slice_ptr[s + 1] - base) / kSlice);
    double acc = 0.0;
    // Chunks of 8 entries: all column and value loads, then all x gathers,
    // then the multiply-adds in entry order (one dependent round trip per
    // chunk instead of two per entry).
    for (int k0 = 0; k0 < width; k0 += 8) {
      int c[8];
      double v[8], xv[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int64_t e = base + (int64_t)(k0 + j) * kSlice + lane;
        const bool in = k0 + j < width;
        c[j] = in ? m.cols[e] : -1;
        v[j] = in ? m.vals[e] : 0.0;
      }
#pragma unroll
      for (int j = 0; j < 8; ++j) xv[j] = c[j] >= 0 ? x[c[j]] : 0.0;
#pragma unroll
      for (int j = 0; j < 8; ++j)
        if (c[j] >= 0) acc = fma(v[j], xv[j], acc);
    }
    const int row = s * kSlice + lane;
    if (row < m.nrow) {
      const int orow = m.perm ? m.perm[row] : row;
      double out = acc;
      if (epi == CE_SCALE) out = aux0[orow] * acc;
      else if (epi == CE_MASS) out = fma(aux0[orow], aux1[orow], acc);
      z[orow] = out;
      if (w) dot_part = fma(out, w[orow], dot_part);
    }
  }
}

// CTA sum of one value per thread, in thread 0 (fixed order).
__device__ __forceinline__ double cta_sum(double v, double* sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  double c = 0.0;
  if (threadIdx.x == 0)
    for (int w2 = 0; w2 < kThreadsC / 32; ++w2) c += sh[w2];
  return c;
}

// Synchronisation and the exchange of per-CTA sums.  Every CTA gets the
// same total: the CTA sums added in CTA order (lanes take them strided,
// then a fixed butterfly).  Two slots alternate, so a CTA that runs ahead
// never overwrites sums another CTA is still reading.
//
// ClusterSync: the grid is one thread-block cluster; syncs are the
// cluster's hardware barrier and every CTA reads the others' sums from
// their shared memory (distributed shared memory), no global round trip.
struct ClusterSync {
  cgr::cluster_group c;
  double* xch;  // this CTA's shared [2] exchange slots
  __device__ ClusterSync(double* x) : c(cgr::this_cluster()), xch(x) {}
  __device__ void sync() { c.sync(); }
  __device__ double total(double v, int slot, double* sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const double cs = cta_sum(v, sh);
    if (threadIdx.x == 0) xch[slot] = cs;
    c.sync();
    if (warp == 0) {
      const unsigned int ranks = c.num_blocks();
      double a = 0.0;
      for (unsigned int q = lane; q < ranks; q += 32) a += *c.map_shared_rank(xch + slot, q);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
      if (lane == 0) sh[kThreadsC / 32] = a;
    }
    __syncthreads();
    const double t = sh[kThreadsC / 32];
    __syncthreads();
    return t;
  }
  // No CTA leaves while another may still read its shared memory.
  __device__ void finish() { c.sync(); }
};

// Ap = A x with dot_part += Ap . w: one product, or the factored squared
// Laplacian's two with a sync between them.
template <class S>
__device__ __forceinline__ void apply_a(S& grid, const Args& a, const double* x, double* out,
                                        const double* w, double& dot_part, int cta, int ncta) {
  if (a.inv_mass) {
    double d0 = 0.0;
    product(a.A, x, a.u, nullptr, d0, cta, ncta, CE_SCALE, a.inv_mass);
    grid.sync();
    product(a.A, a.u, out, w, dot_part, cta, ncta, CE_MASS, a.wmass, x);
  } else {
    product(a.A, x, out, w, dot_part, cta, ncta);
  }
}

// z = M r (G then G^T, a sync between them; or z = r); returns this
// thread's share of r.z.
template <class S>
__device__ __forceinline__ double precondition(S& grid, const Args& a, bool precond, int64_t gt,
                                               int64_t gs, int cta, int ncta) {
  double prz = 0.0;
  if (precond) {
    double d0 = 0.0;
    product(a.G, a.r, a.t, nullptr, d0, cta, ncta);
    grid.sync();
    product(a.GT, a.t, a.z, a.r, prz, cta, ncta);
  } else {
    for (int64_t i = gt; i < a.n; i += gs) {
      const double ri = a.r[i];
      a.z[i] = ri;
      prz = fma(ri, ri, prz);
    }
  }
  return prz;
}

// One system's PCG solve on CTAs cta = 0..ncta-1 of a grid or a cluster.
template <class S>
__device__ void pcg_body(const Args& a, S& grid, int cta, int ncta, double* sh) {
  KrylovScalars* ks = a.ks;
  const int64_t n = a.n;
  const int64_t gt = (int64_t)cta * kThreadsC + threadIdx.x;
  const int64_t gs = (int64_t)ncta * kThreadsC;
  const bool precond = a.G.nslices >= 0;
  int slot = 0;
  const double tol = ks->tol, atol = ks->atol;
  const int maxiter = ks->maxiter;
  double* hist = ks->hist;
  const int hist_len = ks->hist_len;
  // r = b - A x; b.b and r.r.
  double dummy = 0.0;
  apply_a(grid, a, a.x, a.Ap, nullptr, dummy, cta, ncta);
  grid.sync();
  double pbb = 0.0, prr = 0.0;
  for (int64_t i = gt; i < n; i += gs) {
    const double bi = a.b[i];
    const double ri = bi - a.Ap[i];
    a.r[i] = ri;
    pbb = fma(bi, bi, pbb);
    prr = fma(ri, ri, prr);
  }
  const double bb = grid.total(pbb, slot, sh);
  slot ^= 1;
  double rr = grid.total(prr, slot, sh);
  slot ^= 1;
  const double at = fmax(atol, tol * sqrt(bb));
  const double atol_sq = at * at;
  if (gt == 0 && hist && hist_len > 0) hist[0] = sqrt(rr);
  // z = M r, rz = r.z, p = z.
  double prz = precondition(grid, a, precond, gt, gs, cta, ncta);
  double rz = grid.total(prz, slot, sh);
  slot ^= 1;
  for (int64_t i = gt; i < n; i += gs) a.p[i] = a.z[i];
  grid.sync();
  int it = 0;
  double alpha = 0.0, beta = 0.0, pap = 0.0;
  while (rr > atol_sq && it < maxiter) {
    double ppap = 0.0;
    apply_a(grid, a, a.p, a.Ap, a.p, ppap, cta, ncta);
    pap = grid.total(ppap, slot, sh);
    slot ^= 1;
    alpha = rz / pap;
    double prr2 = 0.0;
    for (int64_t i = gt; i < n; i += gs) {
      a.x[i] = fma(alpha, a.p[i], a.x[i]);
      const double ri = fma(-alpha, a.Ap[i], a.r[i]);
      a.r[i] = ri;
      prr2 = fma(ri, ri, prr2);
    }
    rr = grid.total(prr2, slot, sh);
    slot ^= 1;
    if (gt == 0 && hist && it + 1 < hist_len) hist[it + 1] = sqrt(rr);
    const double prz2 = precondition(grid, a, precond, gt, gs, cta, ncta);
    const double rz_new = grid.total(prz2, slot, sh);
    slot ^= 1;
    beta = rz_new / rz;
    rz = rz_new;
    ++it;
    for (int64_t i = gt; i < n; i += gs) a.p[i] = fma(beta, a.p[i], a.z[i]);
    grid.sync();
  }
  grid.finish();
  if (gt == 0) {
    ks->bb = bb;
    ks->atol_sq = atol_sq;
    ks->rr = rr;
    ks->rz = rz;
    ks->denom = pap;
    ks->alpha = alpha;
    ks->beta = beta;
    ks->it = it;
    ks->active = 0;
  }
}

// One system on one cluster (the grid is that cluster).
__global__ void __launch_bounds__(kThreadsC) pcg_kernel(Args a) {
  __shared__ double sh[kThreadsC / 32 + 1];
  __shared__ double xch[2];
  ClusterSync grid(xch);
  pcg_body(a, grid, blockIdx.x, gridDim.x, sh);
}

// Many systems in one launch: cluster c (CTAs c*C .. c*C+C-1 of a 1-D grid
// of nsys clusters of C CTAs) solves system c with its own operator,
// preconditioner, vectors and scalars.  Clusters never wait on each other:
// each leaves when its own system has converged.
__global__ void __launch_bounds__(kThreadsC) multi_cluster_kernel(const Args* systems, int nsys) {
  __shared__ double sh[kThreadsC / 32 + 1];
  __shared__ double xch[2];
  cgr::cluster_group cl = cgr::this_cluster();
  const int C = (int)cl.num_blocks();
  const int sys = blockIdx.x / C;
  if (sys >= nsys) return;  // uniform over a cluster
  const Args a = systems[sys];
  ClusterSync sync(xch);
  pcg_body(a, sync, (int)cl.block_rank(), C, sh);
}

// tol, atol, maxiter (<= 0: the system's size) of every system, no history.
__global__ void multi_set_kernel(const Args* systems, int nsys, double tol, double atol,
                                 int maxiter) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsys) return;
  KrylovScalars* ks = systems[s].ks;
  ks->tol = tol;
  ks->atol = atol;
  const int64_t n = systems[s].n;
  ks->maxiter = maxiter > 0 ? maxiter : (n < 0x7fffffff ? (int)n : 0x7fffffff);
  ks->it = 0;
  ks->active = 1;
  ks->cond_handle = 0ull;
  ks->hist = nullptr;
  ks->hist_len = 0;
}

__global__ void multi_outputs_kernel(const Args* systems, int nsys, int32_t* nit, double* rr,
                                     double* atol_sq) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsys) return;
  const KrylovScalars* ks = systems[s].ks;
  if (nit) nit[s] = ks->it;
  if (rr) rr[s] = ks->rr;
  if (atol_sq) atol_sq[s] = ks->atol_sq;
}

Mat mat_of(const Sell& m) {
  return Mat{m.nrow, m.nslices, m.slice_ptr.as<int64_t>(), m.cols.as<int32_t>(),
             m.vals.as<double>(), m.perm.p ? m.perm.as<int32_t>() : nullptr};
}

bool enabled() {
  static const bool on = [] {
    const char* e = std::getenv("GBPC_COOP");
    return !(e && e[0] == '0');
  }();
  return on;
}

// Cluster size both cluster kernels run with: 16 CTAs when such a cluster
// of either kernel can be scheduled, else 8, else 0 (no cluster path).
// One size for both, so a system gives the same bits alone and in a group.
int cluster_size() {
  static int chosen = -1;
  if (chosen >= 0) return chosen;
  chosen = 0;
  const void* kerns[2] = {(const void*)pcg_kernel, (const void*)multi_cluster_kernel};
  for (const void* k : kerns)
    if (cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)
      cudaGetLastError();
  for (int c : {16, 8}) {
    bool ok = true;
    for (const void* k : kerns) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(c);
      cfg.blockDim = dim3(kThreadsC);
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = c;
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      int clusters = 0;
      if (cudaOccupancyMaxActiveClusters(&clusters, k, &cfg) != cudaSuccess || clusters < 1) {
        cudaGetLastError();
        ok = false;
      }
    }
    if (ok) {
      chosen = c;
      break;
    }
  }
  return chosen;
}

}  // namespace coop

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
  // Small systems (coop::kClusterWork) with a sparse or factored operator
  // and an FSAI or no preconditioner run as one kernel on one cluster.
  bool coop = false;
  int coop_cluster = 0;  // CTAs of that cluster
  coop::Args cargs{};
  DevBuf r, z, p, Ap, Az, y, ks, zeros, t, u;
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

  // Decide whether this solver runs as one cooperative kernel (small
  // scalar CG with a sparse operator and an FSAI or no preconditioner, the
  // graph loop requested) and size its grid: enough CTAs for one slice per
  // warp, at most what can be resident at once.
  int setup_coop() {
    coop = false;
    if (!coop::enabled() || method != GBPC_CG || !use_graph || low || n < 1) return GBPC_OK;
    const Sell* pa[1] = {nullptr};
    const Sell* pm[2] = {nullptr, nullptr};
    const void* inv_mass = nullptr;
    const void* wmass = nullptr;
    if (A->scalar_products(pa, 1) != 1 && !A->factored_parts(pa, &inv_mass, &wmass))
      return GBPC_OK;
    if (M && M->scalar_products(pm, 2) != 2) return GBPC_OK;
    const int64_t work = (inv_mass ? 2 : 1) * pa[0]->nent +
                         (M ? pm[0]->nent + pm[1]->nent : 0) + 8 * n;
    if (work > coop::kClusterWork) return GBPC_OK;
    coop_cluster = coop::cluster_size();
    if (coop_cluster == 0) return GBPC_OK;
    int rc;
    if ((rc = t.alloc(sizeof(double) * n))) return rc;
    if (inv_mass && (rc = u.alloc(sizeof(double) * n))) return rc;
    cargs = coop::Args{};
    cargs.A = coop::mat_of(*pa[0]);
    cargs.inv_mass = (const double*)inv_mass;
    cargs.wmass = (const double*)wmass;
    cargs.u = inv_mass ? u.as<double>() : nullptr;
    if (M) {
      cargs.G = coop::mat_of(*pm[0]);
      cargs.GT = coop::mat_of(*pm[1]);
    } else {
      cargs.G.nslices = -1;
      cargs.GT.nslices = -1;
    }
    cargs.n = n;
    cargs.r = r.as<double>();
    cargs.z = z.as<double>();
    cargs.p = p.as<double>();
    cargs.Ap = Ap.as<double>();
    cargs.t = t.as<double>();
    cargs.ks = K();
    coop = true;
    return GBPC_OK;
  }

  int run(const double* b, double* x, double tol, double atol, int maxiter, int32_t* nit_dev,
          double* rr_dev, double* atol_sq_dev, cudaStream_t st) {
    if (maxiter <= 0) maxiter = (int)std::min<int64_t>(n, 0x7fffffff);
    int rc;
    if (coop) {
      set_scalars_kernel<<<1, 1, 0, st>>>(K(), tol, atol, maxiter, 0ull, hist, hist_len);
      GBPC_CUDA_TRY(cudaGetLastError());
      coop::Args a = cargs;
      a.b = b;
      a.x = x;
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(coop_cluster);
      cfg.blockDim = dim3(coop::kThreadsC);
      cfg.stream = st;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = coop_cluster;
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      GBPC_CUDA_TRY(cudaLaunchKernelEx(&cfg, coop::pcg_kernel, a));
    } else if (use_graph) {
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
  if (!rc) rc = s.setup_coop();
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

extern "C" int gbpc_solver_cluster(const gbpc_solver* h, int* cluster_host) {
  if (!h || !cluster_host) {
    gbpc_set_error("gbpc_solver_cluster: bad arguments");
    return GBPC_ERR_ARG;
  }
  *cluster_host = h->s.coop ? h->s.coop_cluster : 0;
  return GBPC_OK;
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

// ---------------------------------------------------------------------------
// Many independent small systems in one launch, one thread-block cluster per
// system (coop::multi_cluster_kernel).  Unlike gbpc_msolver, the systems keep
// their own operators (nothing is concatenated), each cluster leaves as soon
// as its system has converged, and a system's iterates are those of the
// single-system cluster kernel of the same cluster size.


struct gbpc_csolver {
  size_t device_bytes = 0;  // declared first: released last
  int nsys = 0;
  int cluster = 0;
  std::vector<coop::Args> host_args;
  gbpc::DevBuf args, vecs, scalars;
};

extern "C" int gbpc_csolver_create(int nsys, gbpc_op* const* A, gbpc_op* const* M, void* stream,
                                   gbpc_csolver** out) {
  if (!out || nsys < 1 || !A) {
    gbpc_set_error("gbpc_csolver_create: bad arguments");
    return GBPC_ERR_ARG;
  }
  const int C = coop::cluster_size();
  if (C == 0) {
    gbpc_set_error("gbpc_csolver_create: no thread-block cluster of 8 or 16 CTAs can be scheduled");
    return GBPC_ERR_UNSUPPORTED;
  }
  struct Parts {
    const Sell* a;
    const void* im;
    const void* wm;
    const Sell* g;
    const Sell* gt;
    int64_t n;
  };
  std::vector<Parts> parts((size_t)nsys);
  size_t doubles = 0;
  for (int s = 0; s < nsys; ++s) {
    if (!A[s] || !A[s]->impl) {
      gbpc_set_error("gbpc_csolver_create: system %d has no operator", s);
      return GBPC_ERR_ARG;
    }
    Operator* a = A[s]->impl.get();
    Operator* m = (M && M[s] && M[s]->impl) ? M[s]->impl.get() : nullptr;
    Parts p{};
    const Sell* pa[1] = {nullptr};
    const Sell* pm[2] = {nullptr, nullptr};
    if (a->scalar_products(pa, 1) != 1 && !a->factored_parts(pa, &p.im, &p.wm)) {
      gbpc_set_error("gbpc_csolver_create: system %d: the operator must be a float64 scalar sparse "
                     "product or the factored squared Laplacian with every vertex free", s);
      return GBPC_ERR_UNSUPPORTED;
    }
    if (m && m->scalar_products(pm, 2) != 2) {
      gbpc_set_error("gbpc_csolver_create: system %d: the preconditioner must be a float64 "
                     "scalar FSAI or none", s);
      return GBPC_ERR_UNSUPPORTED;
    }
    if (m && m->rows != a->rows) {
      gbpc_set_error("gbpc_csolver_create: system %d: operator and preconditioner sizes differ", s);
      return GBPC_ERR_ARG;
    }
    p.a = pa[0];
    p.g = pm[0];
    p.gt = pm[1];
    p.n = a->rows;
    doubles += (size_t)p.n * (p.im ? 6 : 5);
    parts[s] = p;
  }
  auto* h = new gbpc_csolver;
  ByteTally tally(&h->device_bytes);
  h->nsys = nsys;
  h->cluster = C;
  int rc = h->vecs.alloc(sizeof(double) * std::max<size_t>(doubles, 1));
  if (!rc) rc = h->scalars.alloc(sizeof(KrylovScalars) * nsys);
  if (!rc) rc = h->args.alloc(sizeof(coop::Args) * nsys);
  if (!rc && cudaMemsetAsync(h->scalars.p, 0, sizeof(KrylovScalars) * nsys, (cudaStream_t)stream) !=
                 cudaSuccess)
    rc = GBPC_ERR_CUDA;
  if (rc) {
    delete h;
    return rc;
  }
  h->host_args.resize((size_t)nsys);
  double* v = h->vecs.as<double>();
  for (int s = 0; s < nsys; ++s) {
    const Parts& p = parts[s];
    coop::Args& g = h->host_args[s];
    g = coop::Args{};
    g.A = coop::mat_of(*p.a);
    if (p.g) {
      g.G = coop::mat_of(*p.g);
      g.GT = coop::mat_of(*p.gt);
    } else {
      g.G.nslices = -1;
      g.GT.nslices = -1;
    }
    g.inv_mass = (const double*)p.im;
    g.wmass = (const double*)p.wm;
    g.n = p.n;
    g.r = v;
    g.z = v + p.n;
    g.p = v + 2 * p.n;
    g.Ap = v + 3 * p.n;
    g.t = v + 4 * p.n;
    g.u = p.im ? v + 5 * p.n : nullptr;
    v += (size_t)p.n * (p.im ? 6 : 5);
    g.ks = h->scalars.as<KrylovScalars>() + s;
  }
  *out = h;
  return GBPC_OK;
}

extern "C" int gbpc_csolver_run(gbpc_csolver* h, int count, const double* const* b_host,
                                double* const* x_host, double tol, double atol, int maxiter,
                                int32_t* nit_dev, double* rr_dev, double* atol_sq_dev,
                                void* stream) {
  NvtxRange nvtx_range("gbpc_csolver_run");
  if (!h || !b_host || !x_host || count < 1 || count > h->nsys) {
    gbpc_set_error("gbpc_csolver_run: bad arguments");
    return GBPC_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  for (int s = 0; s < count; ++s) {
    if (h->host_args[s].n > 0 && (!b_host[s] || !x_host[s])) {
      gbpc_set_error("gbpc_csolver_run: system %d has no right-hand side or solution vector", s);
      return GBPC_ERR_ARG;
    }
    h->host_args[s].b = b_host[s];
    h->host_args[s].x = x_host[s];
  }
  // Pageable source: the copy is staged before the call returns.
  GBPC_CUDA_TRY(cudaMemcpyAsync(h->args.p, h->host_args.data(), sizeof(coop::Args) * count,
                                cudaMemcpyHostToDevice, st));
  const coop::Args* dargs = h->args.as<coop::Args>();
  coop::multi_set_kernel<<<grid_for(count, 128), 128, 0, st>>>(dargs, count, tol, atol, maxiter);
  GBPC_CUDA_TRY(cudaGetLastError());
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)count * h->cluster);
  cfg.blockDim = dim3(coop::kThreadsC);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = h->cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  GBPC_CUDA_TRY(cudaLaunchKernelEx(&cfg, coop::multi_cluster_kernel, dargs, count));
  if (nit_dev || rr_dev || atol_sq_dev) {
    coop::multi_outputs_kernel<<<grid_for(count, 128), 128, 0, st>>>(dargs, count, nit_dev,
                                                                     rr_dev, atol_sq_dev);
    GBPC_CUDA_TRY(cudaGetLastError());
  }
  return GBPC_OK;
}

extern "C" int gbpc_csolver_cluster_size(const gbpc_csolver* h, int* cluster_host) {
  if (!h || !cluster_host) {
    gbpc_set_error("gbpc_csolver_cluster_size: bad arguments");
    return GBPC_ERR_ARG;
  }
  *cluster_host = h->cluster;
  return GBPC_OK;
}

extern "C" int gbpc_csolver_device_bytes(const gbpc_csolver* h, size_t* bytes_host) {
  if (!h || !bytes_host) {
    gbpc_set_error("gbpc_csolver_device_bytes: bad arguments");
    return GBPC_ERR_ARG;
  }
  *bytes_host = h->device_bytes;
  return GBPC_OK;
}

extern "C" int gbpc_csolver_destroy(gbpc_csolver* h) {
  if (!h) return GBPC_OK;
  cudaDeviceSynchronize();
  delete h;
  return GBPC_OK;
}
