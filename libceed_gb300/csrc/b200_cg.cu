// Conjugate gradients on the fused operator: plain FP64 CG, and FP32 CG inside FP64 iterative refinement.
//
// There is no solver inside libCEED; this mirrors the KSPCG use of CeedOperatorApply in the reference's PETSc
// benchmark driver (examples/petsc/bps.c, "DoFs/Sec in CG" at :287), with homogeneous Dirichlet conditions through a
// mask (1 on free nodes, 0 on the box boundary): the solver works with m * A(m * x).
//
// All scalars (alpha, beta, r.r) stay on the device, so a block of `check_every` iterations is one CUDA graph and the
// host only reads r.r between blocks.  Dot products and norms use a fixed-order two-pass reduction: each thread sums
// in FP64 for FP64 vectors and in float-float (about 48 bits, on the FP32 pipe) for FP32 vectors, and the per-block
// and final passes add in FP64.  Mixed mode (defect correction): r = m(b - A64 x) in FP64; FP32 CG solves
// A32 d = r to a relative tolerance; x += d in FP64; repeat until |r| / |b| <= rtol.
#include "b200_internal.cuh"
#include "b200_reduce.cuh"

#include <cmath>

namespace b200 {

// Device scalars: [0] r.z of the current iterate, [1] p.w, [2] r.z after the update, [3] r.r after the update
// (z = M r with the Jacobi preconditioner M = diag(A)^-1, or z = r without one, when [2] is r.r itself).
enum { kRR = 0, kPW = 1, kRRNew = 2, kRes = 3 };

// The reduction kernels run on a fixed grid of two blocks per SM (so that their sums are reproducible), which leaves
// few threads to keep HBM busy: each thread therefore loads kUnroll<T> elements (at i, i + stride, ...) before using
// any of them.  Partial sums are still accumulated in index order i, i + stride, ..., as a plain loop would.
template <typename T>
constexpr int kUnroll = sizeof(T) == 4 ? 16 : 8;

// p.w (the operator output w unmasked: p is zero on the Dirichlet nodes, so p.w = p.(m w) term by term).
template <typename T>
__global__ void __launch_bounds__(kReduceThreads) k_cg_pdot(int64_t n, const T *__restrict__ p, const T *__restrict__ w, double *__restrict__ partial) {
  constexpr int U      = kUnroll<T>;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t       i      = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  typename AccFor<T>::type acc;
  for (; i + (U - 1) * stride < n; i += U * stride) {
    T wv[U], pv[U];
#pragma unroll
    for (int k = 0; k < U; k++) {
      wv[k] = w[i + k * stride];
      pv[k] = p[i + k * stride];
    }
#pragma unroll
    for (int k = 0; k < U; k++) acc.add_prod(pv[k], wv[k]);
  }
  for (; i < n; i += stride) acc.add_prod(p[i], w[i]);
  const double sum = block_reduce(kRedDot, acc.value());
  if (threadIdx.x == 0) partial[blockIdx.x] = sum;
}

// x += alpha p, r = m (r - alpha w), and the partial sums of r.r.  The mask (0 or 1) applied here is the m of m A(m x):
// r stays zero on the Dirichlet nodes.
template <typename T>
__global__ void __launch_bounds__(kReduceThreads) k_cg_update(int64_t n, const double *__restrict__ s, const T *__restrict__ mask, T *__restrict__ x,
                                                                T *__restrict__ r, const T *__restrict__ p, const T *__restrict__ w,
                                                                double *__restrict__ partial) {
  constexpr int U      = kUnroll<T>;
  const double  pw     = s[kPW];
  const T       alpha  = (T)(pw != 0.0 ? s[kRR] / pw : 0.0);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t       i      = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  typename AccFor<T>::type acc;
  for (; i + (U - 1) * stride < n; i += U * stride) {
    T xv[U], pv[U], rv[U], wv[U], mv[U];
#pragma unroll
    for (int k = 0; k < U; k++) {
      xv[k] = x[i + k * stride];
      pv[k] = p[i + k * stride];
      rv[k] = r[i + k * stride];
      wv[k] = w[i + k * stride];
      mv[k] = mask[i + k * stride];
    }
#pragma unroll
    for (int k = 0; k < U; k++) {
      x[i + k * stride] = xv[k] + alpha * pv[k];
      const T ri        = mv[k] * (rv[k] - alpha * wv[k]);
      r[i + k * stride] = ri;
      acc.add_prod(ri, ri);
    }
  }
  for (; i < n; i += stride) {
    x[i] += alpha * p[i];
    const T ri = mask[i] * (r[i] - alpha * w[i]);
    r[i]       = ri;
    acc.add_prod(ri, ri);
  }
  const double sum = block_reduce(kRedSumSq, acc.value());
  if (threadIdx.x == 0) partial[blockIdx.x] = sum;
}

// Preconditioned update: also z = M r, with partial sums of r.z (partial) and r.r (partial2).
template <typename T>
__global__ void __launch_bounds__(kReduceThreads) k_pcg_update(int64_t n, const double *__restrict__ s, const T *__restrict__ mask, T *__restrict__ x,
                                                                 T *__restrict__ r, T *__restrict__ z, const T *__restrict__ inv_diag,
                                                                 const T *__restrict__ p, const T *__restrict__ w, double *__restrict__ partial,
                                                                 double *__restrict__ partial2) {
  constexpr int U      = kUnroll<T>;
  const double  pw     = s[kPW];
  const T       alpha  = (T)(pw != 0.0 ? s[kRR] / pw : 0.0);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t       i      = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  typename AccFor<T>::type rz, rr;
  for (; i + (U - 1) * stride < n; i += U * stride) {
    T xv[U], pv[U], rv[U], wv[U], dv[U], mv[U];
#pragma unroll
    for (int k = 0; k < U; k++) {
      xv[k] = x[i + k * stride];
      pv[k] = p[i + k * stride];
      rv[k] = r[i + k * stride];
      wv[k] = w[i + k * stride];
      dv[k] = inv_diag[i + k * stride];
      mv[k] = mask[i + k * stride];
    }
#pragma unroll
    for (int k = 0; k < U; k++) {
      x[i + k * stride] = xv[k] + alpha * pv[k];
      const T ri        = mv[k] * (rv[k] - alpha * wv[k]);
      const T zi        = dv[k] * ri;
      r[i + k * stride] = ri;
      z[i + k * stride] = zi;
      rz.add_prod(ri, zi);
      rr.add_prod(ri, ri);
    }
  }
  for (; i < n; i += stride) {
    x[i] += alpha * p[i];
    const T ri = mask[i] * (r[i] - alpha * w[i]);
    const T zi = inv_diag[i] * ri;
    r[i]       = ri;
    z[i]       = zi;
    rz.add_prod(ri, zi);
    rr.add_prod(ri, ri);
  }
  const double rz_sum = block_reduce(kRedDot, rz.value());
  __syncthreads();
  const double rr_sum = block_reduce(kRedSumSq, rr.value());
  if (threadIdx.x == 0) {
    partial[blockIdx.x]  = rz_sum;
    partial2[blockIdx.x] = rr_sum;
  }
}

// p = src + beta p, src = r (plain CG) or z (preconditioned).
template <typename T>
__global__ void k_cg_direction(int64_t n, const double *__restrict__ s, const T *__restrict__ src, T *__restrict__ p) {
  constexpr int U      = 4;
  const double  rr     = s[kRR];
  const T       beta   = (T)(rr != 0.0 ? s[kRRNew] / rr : 0.0);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t       i      = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  for (; i + (U - 1) * stride < n; i += U * stride) {
    T sv[U], pv[U];
#pragma unroll
    for (int k = 0; k < U; k++) {
      sv[k] = src[i + k * stride];
      pv[k] = p[i + k * stride];
    }
#pragma unroll
    for (int k = 0; k < U; k++) p[i + k * stride] = sv[k] + beta * pv[k];
  }
  for (; i < n; i += stride) p[i] = src[i] + beta * p[i];
}

// Start of a preconditioned solve: z = p = M r.
template <typename T>
__global__ void k_pcg_start(int64_t n, const T *__restrict__ inv_diag, const T *__restrict__ r, T *__restrict__ z, T *__restrict__ p) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const T zi = inv_diag[i] * r[i];
    z[i]       = zi;
    p[i]       = zi;
  }
}

// Final pass of a reduction into s[dst]; optionally first retire r.r (s[kRR] = s[kRRNew]).
__global__ void __launch_bounds__(kReduceThreads) k_cg_final(int blocks, const double *__restrict__ partial, double *__restrict__ s, int dst,
                                                               int retire) {
  double acc = 0.0;
  for (int i = threadIdx.x; i < blocks; i += blockDim.x) acc += partial[i];
  acc = block_reduce(kRedDot, acc);
  if (threadIdx.x == 0) {
    if (retire) s[kRR] = s[kRRNew];
    s[dst] = acc;
  }
}

// r = m (b - r) and its squared norm (r holds A x on entry).
__global__ void __launch_bounds__(kReduceThreads) k_residual(int64_t n, const double *__restrict__ mask, const double *__restrict__ b,
                                                               double *__restrict__ r, double *__restrict__ partial) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t       i      = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double        acc    = 0.0;
  for (; i + (kUnroll<double> - 1) * stride < n; i += kUnroll<double> * stride) {
    double mv[kUnroll<double>], bv[kUnroll<double>], rv[kUnroll<double>];
#pragma unroll
    for (int k = 0; k < kUnroll<double>; k++) {
      mv[k] = mask[i + k * stride];
      bv[k] = b[i + k * stride];
      rv[k] = r[i + k * stride];
    }
#pragma unroll
    for (int k = 0; k < kUnroll<double>; k++) {
      const double ri   = mv[k] * (bv[k] - rv[k]);
      r[i + k * stride] = ri;
      acc += ri * ri;
    }
  }
  for (; i < n; i += stride) {
    const double ri = mask[i] * (b[i] - r[i]);
    r[i]            = ri;
    acc += ri * ri;
  }
  acc = block_reduce(kRedSumSq, acc);
  if (threadIdx.x == 0) partial[blockIdx.x] = acc;
}

// Start of a CG solve: x = 0, r = p = rhs (masked already), and s[kRR] = s[kRRNew] = r.r.  rhs may be r itself (the
// FP64 start scales r in place), so neither is __restrict__.
template <typename T, typename S>
__global__ void k_cg_start(int64_t n, const S *rhs, double scale, T *__restrict__ x, T *r, T *__restrict__ p) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const T v = (T)((double)rhs[i] * scale);
    x[i]      = 0;
    r[i]      = v;
    p[i]      = v;
  }
}

__global__ void k_copy_scalar(double *s, int dst, int src) { s[dst] = s[src]; }

__global__ void k_add_correction(int64_t n, double scale, const float *__restrict__ d, double *__restrict__ x) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) x[i] += scale * (double)d[i];
}

template <typename T>
__global__ void k_to_prec(int64_t n, const double *__restrict__ src, T *__restrict__ dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) dst[i] = (T)src[i];
}

}  // namespace b200

using namespace b200;

struct CgWork {
  b200_ctx ctx;
  int64_t  n;
  int      blocks;
  double  *partial, *partial2, *s, *s_host;
  double  *dot_partial;  // per-block p.w of the fused apply (persistent FP32 operator), dot_blocks of them, then its scratch
  int      dot_blocks;
  double  *r64, *p64, *w64, *z64;
  float   *x32, *r32, *p32, *w32, *z32, *mask32, *inv32;
  const double *inv64;  // Jacobi preconditioner (masked 1/diag) or nullptr
  cudaEvent_t   e0, e1;  // device time of the solve
};

template <typename T>
static int cg_iterations(CgWork &wk, b200_op op, const void *qdata, const T *mask, T *x, T *r, T *p, T *w, T *z, const T *inv, int count) {
  b200_ctx  ctx = wk.ctx;
  const int g   = wk.blocks;
  // The persistent FP32 operator sums p.w = p.(A p) element by element inside the apply, which saves the pass over p and w.
  const int db = wk.dot_partial ? op_dot_blocks(op, nullptr) : 0;
  for (int it = 0; it < count; it++) {
    if (db > 0) {
      int st = op_apply_dot(op, p, w, qdata, wk.dot_partial);
      if (st) return st;
      k_cg_final<<<1, kReduceThreads, 0, ctx->stream>>>(db, wk.dot_partial, wk.s, kPW, 1);
      B200_LAUNCHED(ctx, "cg_final");
    } else {
      int st = b200_op_apply(op, p, w, qdata, nullptr, 0);
      if (st) return st;
      k_cg_pdot<T><<<g, kReduceThreads, 0, ctx->stream>>>(wk.n, p, w, wk.partial);
      B200_LAUNCHED(ctx, "cg_pdot");
      k_cg_final<<<1, kReduceThreads, 0, ctx->stream>>>(g, wk.partial, wk.s, kPW, 1);
      B200_LAUNCHED(ctx, "cg_final");
    }
    if (inv) {
      k_pcg_update<T><<<g, kReduceThreads, 0, ctx->stream>>>(wk.n, wk.s, mask, x, r, z, inv, p, w, wk.partial, wk.partial2);
      B200_LAUNCHED(ctx, "pcg_update");
      k_cg_final<<<1, kReduceThreads, 0, ctx->stream>>>(g, wk.partial2, wk.s, kRes, 0);
      B200_LAUNCHED(ctx, "cg_final");
    } else {
      k_cg_update<T><<<g, kReduceThreads, 0, ctx->stream>>>(wk.n, wk.s, mask, x, r, p, w, wk.partial);
      B200_LAUNCHED(ctx, "cg_update");
    }
    k_cg_final<<<1, kReduceThreads, 0, ctx->stream>>>(g, wk.partial, wk.s, kRRNew, 0);
    B200_LAUNCHED(ctx, "cg_final");
    k_cg_direction<T><<<stride_grid(ctx, wk.n, 256), 256, 0, ctx->stream>>>(wk.n, wk.s, inv ? z : r, p);
    B200_LAUNCHED(ctx, "cg_direction");
  }
  return B200_SUCCESS;
}

// Run CG iterations in blocks of `every` (one CUDA graph per block when use_graph) until sqrt(r.r) <= stop or
// max_it.  On entry s[kRR] = s[kRRNew] = r.r of the start vector.
template <typename T>
static int cg_loop(CgWork &wk, b200_op op, const void *qdata, const T *mask, T *x, T *r, T *p, T *w, T *z, const T *inv, double stop, int max_it,
                   int every, int use_graph, int *iters, double *rr_out) {
  const int conv = inv ? kRes : kRRNew;  // index of r.r
  b200_ctx        ctx   = wk.ctx;
  cudaGraphExec_t exec  = nullptr;
  int64_t         per_graph = 0;  // kernels one graph launch runs
  int             done  = 0;
  double          rr    = 0.0;
  int             st    = B200_SUCCESS;
  B200_CUDA(cudaMemcpyAsync(wk.s_host, wk.s + conv, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  B200_CUDA(cudaStreamSynchronize(ctx->stream));
  rr = wk.s_host[0];
  while (done < max_it && !(sqrt(rr) <= stop)) {
    const int count = every < max_it - done ? every : max_it - done;
    if (use_graph && count == every) {
      if (!exec) {
        // Failures below leave the loop with st set, so the graph and its executable are always destroyed.
        cudaGraph_t     graph = nullptr;
        cudaGraphExec_t ge    = nullptr;
        const int64_t   l0    = ctx->launches;
        st = cuda_status(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture", __FILE__, __LINE__);
        if (st) break;
        st                = cg_iterations<T>(wk, op, qdata, mask, x, r, p, w, z, inv, count);
        const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
        if (!st) st = cuda_status(ce, "cudaStreamEndCapture", __FILE__, __LINE__);
        if (!st) st = cuda_status(cudaGraphInstantiate(&ge, graph, 0), "cudaGraphInstantiate", __FILE__, __LINE__);
        if (graph) cudaGraphDestroy(graph);
        if (st) break;
        exec          = ge;
        per_graph     = ctx->launches - l0;
        ctx->launches = l0;  // captured, not yet run
      }
      st = cuda_status(cudaGraphLaunch(exec, ctx->stream), "cudaGraphLaunch", __FILE__, __LINE__);
      if (st) break;
      ctx->launches += per_graph;
    } else {
      st = cg_iterations<T>(wk, op, qdata, mask, x, r, p, w, z, inv, count);
      if (st) break;
    }
    done += count;
    st = cuda_status(cudaMemcpyAsync(wk.s_host, wk.s + conv, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync", __FILE__,
                     __LINE__);
    if (!st) st = cuda_status(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize", __FILE__, __LINE__);
    if (st) break;
    rr = wk.s_host[0];
    if (!std::isfinite(rr)) {
      set_error("CG diverged (r.r = %g after %d iterations)", rr, done);
      st = B200_ERROR_BACKEND;
      break;
    }
  }
  if (exec) cudaGraphExecDestroy(exec);
  *iters  = done;
  *rr_out = rr;
  return st;
}

// After r = p = rhs: with a preconditioner, z = p = M r; s[kRR] = s[kRRNew] = r.z and s[kRes] = r.r.
template <typename T>
static int pcg_start(CgWork &wk, T *r, T *z, T *p, const T *inv, int prec) {
  b200_ctx ctx = wk.ctx;
  int      st  = reduce_to_device(ctx, prec, kRedSumSq, wk.n, r, nullptr, wk.s + kRes);
  if (st) return st;
  if (inv) {
    k_pcg_start<T><<<stride_grid(ctx, wk.n, 256), 256, 0, ctx->stream>>>(wk.n, inv, r, z, p);
    B200_LAUNCHED(ctx, "pcg_start");
    st = reduce_to_device(ctx, prec, kRedDot, wk.n, r, z, wk.s + kRRNew);
  } else {
    st = reduce_to_device(ctx, prec, kRedSumSq, wk.n, r, nullptr, wk.s + kRRNew);
  }
  if (st) return st;
  k_copy_scalar<<<1, 1, 0, ctx->stream>>>(wk.s, kRR, kRRNew);
  B200_LAUNCHED(ctx, "cg_copy");
  return B200_SUCCESS;
}

// r64 = m (b - A64 x), returns |r64|.
static int outer_residual(CgWork &wk, b200_op op64, const void *qdata64, const double *mask, const double *b, const double *x, double *norm) {
  b200_ctx ctx = wk.ctx;
  int      st  = b200_op_apply(op64, x, wk.r64, qdata64, nullptr, 0);
  if (st) return st;
  k_residual<<<wk.blocks, kReduceThreads, 0, ctx->stream>>>(wk.n, mask, b, wk.r64, wk.partial);
  B200_LAUNCHED(ctx, "cg_residual");
  k_cg_final<<<1, kReduceThreads, 0, ctx->stream>>>(wk.blocks, wk.partial, wk.s, kRRNew, 0);
  B200_LAUNCHED(ctx, "cg_final");
  B200_CUDA(cudaMemcpyAsync(wk.s_host, wk.s + kRRNew, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  B200_CUDA(cudaStreamSynchronize(ctx->stream));
  *norm = sqrt(wk.s_host[0]);
  return B200_SUCCESS;
}

static int cg_solve_on_stream(b200_ctx ctx, b200_op op64, b200_op op32, const void *qdata64, const void *qdata32, const double *mask,
                              const double *b, double *x, int64_t n, const b200_cg_opts *opts, b200_cg_stats *stats);

extern "C" int b200_cg_solve(b200_ctx ctx, b200_op op64, b200_op op32, const void *qdata64, const void *qdata32, const double *mask, const double *b,
                             double *x, int64_t n, const b200_cg_opts *opts, b200_cg_stats *stats) {
  B200_CHECK(op64 && qdata64 && mask && b && x && opts && stats, B200_ERROR_INCOMPLETE, "b200_cg_solve: missing argument");
  B200_CHECK(!opts->mixed || (op32 && qdata32), B200_ERROR_INCOMPLETE, "mixed-precision CG needs the FP32 operator and qdata");
  // The solve runs on a private non-blocking stream (a legacy default stream cannot be captured into a graph),
  // ordered after the work already queued on the context's stream and before anything queued after the call.
  cudaStream_t user_stream = ctx->stream, solve_stream;
  cudaEvent_t  fork, join;
  B200_CUDA(cudaStreamCreateWithFlags(&solve_stream, cudaStreamNonBlocking));
  B200_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
  B200_CUDA(cudaEventCreateWithFlags(&join, cudaEventDisableTiming));
  B200_CUDA(cudaEventRecord(fork, user_stream));
  B200_CUDA(cudaStreamWaitEvent(solve_stream, fork, 0));
  ctx->stream = solve_stream;
  const int st_solve = cg_solve_on_stream(ctx, op64, op32, qdata64, qdata32, mask, b, x, n, opts, stats);
  cudaEventRecord(join, solve_stream);
  cudaStreamWaitEvent(user_stream, join, 0);
  ctx->stream = user_stream;
  cudaStreamSynchronize(solve_stream);
  cudaStreamDestroy(solve_stream);
  cudaEventDestroy(fork);
  cudaEventDestroy(join);
  return st_solve;
}

// The solve proper; every array and event it creates is recorded in wk, which the caller releases on every path.
static int cg_run(CgWork &wk, b200_ctx ctx, b200_op op64, b200_op op32, const void *qdata64, const void *qdata32, const double *mask,
                  const double *b, double *x, int64_t n, const b200_cg_opts *opts, b200_cg_stats *stats) {
  wk.ctx    = ctx;
  wk.n      = n;
  wk.blocks = reduce_blocks(ctx->num_sms);
  const int every = opts->check_every > 0 ? opts->check_every : 10;
  *stats          = b200_cg_stats{};
  int st          = B200_SUCCESS;
  wk.inv64 = opts->jacobi;
  B200_CUDA(cudaMalloc(&wk.partial, sizeof(double) * (size_t)(wk.blocks + 8)));
  B200_CUDA(cudaMalloc(&wk.partial2, sizeof(double) * (size_t)(wk.blocks + 8)));
  B200_CUDA(cudaMalloc(&wk.s, sizeof(double) * 8));
  if (wk.inv64) B200_CUDA(cudaMalloc(&wk.z64, sizeof(double) * (size_t)n));
  B200_CUDA(cudaMallocHost(&wk.s_host, sizeof(double) * 8));
  B200_CUDA(cudaMalloc(&wk.r64, sizeof(double) * (size_t)n));
  B200_CUDA(cudaMalloc(&wk.p64, sizeof(double) * (size_t)n));
  B200_CUDA(cudaMalloc(&wk.w64, sizeof(double) * (size_t)n));
  if (opts->mixed) {
    size_t dot_len = 0;
    wk.dot_blocks  = opts->separate_pdot ? 0 : op_dot_blocks(op32, &dot_len);
    if (wk.dot_blocks > 0) B200_CUDA(cudaMalloc(&wk.dot_partial, sizeof(double) * dot_len));
    B200_CUDA(cudaMalloc(&wk.x32, sizeof(float) * (size_t)n));
    B200_CUDA(cudaMalloc(&wk.r32, sizeof(float) * (size_t)n));
    B200_CUDA(cudaMalloc(&wk.p32, sizeof(float) * (size_t)n));
    B200_CUDA(cudaMalloc(&wk.w32, sizeof(float) * (size_t)n));
    B200_CUDA(cudaMalloc(&wk.mask32, sizeof(float) * (size_t)n));
    k_to_prec<float><<<stride_grid(ctx, n, 256), 256, 0, ctx->stream>>>(n, mask, wk.mask32);
    B200_LAUNCHED(ctx, "to_f32");
    if (wk.inv64) {
      B200_CUDA(cudaMalloc(&wk.z32, sizeof(float) * (size_t)n));
      B200_CUDA(cudaMalloc(&wk.inv32, sizeof(float) * (size_t)n));
      k_to_prec<float><<<stride_grid(ctx, n, 256), 256, 0, ctx->stream>>>(n, wk.inv64, wk.inv32);
      B200_LAUNCHED(ctx, "to_f32");
    }
  }
  double bnorm = 0.0;
  st           = reduce_to_device(ctx, B200_F64, kRedSumSq, n, b, nullptr, wk.s + kRRNew);
  if (!st) {
    B200_CUDA(cudaMemcpyAsync(wk.s_host, wk.s + kRRNew, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    B200_CUDA(cudaStreamSynchronize(ctx->stream));
    bnorm = sqrt(wk.s_host[0]);
  }
  const int64_t launches0 = ctx->launches;
  B200_CUDA(cudaEventCreate(&wk.e0));
  B200_CUDA(cudaEventCreate(&wk.e1));
  B200_CUDA(cudaEventRecord(wk.e0, ctx->stream));
  const double target = opts->rtol * bnorm;
  double       rnorm  = 0.0;
  int          total  = 0;
  if (!st && !opts->mixed) {
    // FP64 CG from x = 0: r = p = m b.
    st = b200_vec_pointwise_mult(ctx, B200_F64, n, wk.r64, mask, b);
    if (!st) {
      k_cg_start<double, double><<<stride_grid(ctx, n, 256), 256, 0, ctx->stream>>>(n, wk.r64, 1.0, x, wk.r64, wk.p64);
      st = check_launch(ctx, "cg_start", __FILE__, __LINE__);
    }
    if (!st) st = pcg_start<double>(wk, wk.r64, wk.z64, wk.p64, wk.inv64, B200_F64);
    double rr = 0.0;
    if (!st)
      st = cg_loop<double>(wk, op64, qdata64, mask, x, wk.r64, wk.p64, wk.w64, wk.z64, wk.inv64, target, opts->max_it, every, opts->use_graph,
                           &total, &rr);
    if (!st) st = outer_residual(wk, op64, qdata64, mask, b, x, &rnorm);
    stats->outer = 1;
  } else if (!st) {
    B200_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * (size_t)n, ctx->stream));
    st = outer_residual(wk, op64, qdata64, mask, b, x, &rnorm);
    int outer = 0;
    while (!st && !(rnorm <= target) && outer < opts->max_outer && total < opts->max_it) {
      // Inner FP32 CG on A d = r / |r| (scaled to unit norm), from d = 0.
      const double scale = rnorm > 0 ? 1.0 / rnorm : 1.0;
      k_cg_start<float, double><<<stride_grid(ctx, n, 256), 256, 0, ctx->stream>>>(n, wk.r64, scale, wk.x32, wk.r32, wk.p32);
      st = check_launch(ctx, "cg_start", __FILE__, __LINE__);
      if (!st) st = pcg_start<float>(wk, wk.r32, wk.z32, wk.p32, wk.inv32, B200_F32);
      int    it = 0;
      double rr = 0.0;
      if (!st)
        st = cg_loop<float>(wk, op32, qdata32, wk.mask32, wk.x32, wk.r32, wk.p32, wk.w32, wk.z32, wk.inv32, opts->inner_rtol, opts->max_it - total,
                            every, opts->use_graph, &it, &rr);
      total += it;
      if (st) break;
      k_add_correction<<<stride_grid(ctx, n, 256), 256, 0, ctx->stream>>>(n, rnorm, wk.x32, x);
      st = check_launch(ctx, "cg_correct", __FILE__, __LINE__);
      if (!st) st = outer_residual(wk, op64, qdata64, mask, b, x, &rnorm);
      outer++;
    }
    stats->outer = outer;
  }
  if (!st) {
    B200_CUDA(cudaEventRecord(wk.e1, ctx->stream));
    B200_CUDA(cudaEventSynchronize(wk.e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, wk.e0, wk.e1);
    stats->seconds = ms * 1e-3;
  }
  stats->iterations   = total;
  stats->rel_residual = bnorm > 0 ? rnorm / bnorm : rnorm;
  stats->converged    = !st && rnorm <= target;
  stats->launches     = ctx->launches - launches0;
  return st;
}

static int cg_solve_on_stream(b200_ctx ctx, b200_op op64, b200_op op32, const void *qdata64, const void *qdata32, const double *mask,
                              const double *b, double *x, int64_t n, const b200_cg_opts *opts, b200_cg_stats *stats) {
  CgWork    wk{};
  const int st = cg_run(wk, ctx, op64, op32, qdata64, qdata32, mask, b, x, n, opts, stats);
  cudaStreamSynchronize(ctx->stream);  // nothing queued may still use the arrays freed below
  if (wk.e0) cudaEventDestroy(wk.e0);
  if (wk.e1) cudaEventDestroy(wk.e1);
  cudaFree(wk.partial);
  cudaFree(wk.partial2);
  cudaFree(wk.dot_partial);
  cudaFree(wk.z64);
  cudaFree(wk.z32);
  cudaFree(wk.inv32);
  cudaFree(wk.s);
  cudaFreeHost(wk.s_host);
  cudaFree(wk.r64);
  cudaFree(wk.p64);
  cudaFree(wk.w64);
  cudaFree(wk.x32);
  cudaFree(wk.r32);
  cudaFree(wk.p32);
  cudaFree(wk.w32);
  cudaFree(wk.mask32);
  return st;
}
