/*
 * libceed_b200: the C ABI of the GB300 (sm_103a) operator-apply backend.
 *
 * These are the entry points that the libCEED backend `/gpu/cuda/b200` (host code in C, see
 * libceed_gb300/backend/) binds: plain pointers, sizes and POD descriptors, an `int` status on every
 * call (0 = success), and no CPU fallback.  Each entry point names the reference interface whose
 * work it takes over.  References are paths inside the libCEED source tree.
 *
 * Data layouts chosen by this backend (published to libCEED through CeedElemRestrictionSetELayout):
 *   L-vector   component k of the node at offset o lives at o + k*comp_stride
 *   E-vector   [comp][elem][node]   (ELayout {1, num_elem*elem_size, elem_size})
 *   Q-vector   [eval-dim][comp][elem][qpt]
 *   qdata      strided E-vector with backend strides: [comp][elem][qpt]
 *   offsets    int32 [elem][node], device memory
 *   1D matrices row-major Q x P (interp, grad) and Q x Q (collocated grad), host memory at create time
 *
 * Precision: B200_F64 kernels compute in double; B200_F32 kernels compute and accumulate in float.  B200_F64X (fused
 * operator only) reads and writes double vectors but computes in float-float (a pair of floats, ~48-bit significand)
 * on the FP32 pipes; its results agree with B200_F64 to ~1e-13 relative.  Every other call treats B200_F64X as B200_F64.
 * Every call is asynchronous on the context's stream unless it returns a host value.
 */
#ifndef CEED_B200_H
#define CEED_B200_H

#ifndef __CUDACC_RTC__
#include <stddef.h>
#include <stdint.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes mirror include/ceed/types.h CeedErrorType. */
enum {
  B200_SUCCESS            = 0,
  B200_ERROR_MINOR        = 1,
  B200_ERROR_DIMENSION    = 2,
  B200_ERROR_INCOMPLETE   = 3,
  B200_ERROR_INCOMPATIBLE = 4,
  B200_ERROR_ACCESS       = 5,
  B200_ERROR_UNSUPPORTED  = -2,
  B200_ERROR_BACKEND      = -1,
};

enum { B200_F64 = 0, B200_F32 = 1, B200_F64X = 2 };
enum { B200_NOTRANSPOSE = 0, B200_TRANSPOSE = 1 };                                             /* CeedTransposeMode */
enum { B200_EVAL_NONE = 0, B200_EVAL_INTERP = 1, B200_EVAL_GRAD = 2, B200_EVAL_WEIGHT = 16 }; /* CeedEvalMode */
enum { B200_NORM_1 = 0, B200_NORM_2 = 1, B200_NORM_MAX = 2 };                                  /* CeedNormType */
enum { B200_COPY_H2D = 1, B200_COPY_D2H = 2, B200_COPY_D2D = 3 };
enum { B200_SCATTER_ATOMIC = 0, B200_SCATTER_DETERMINISTIC = 1 };

/* Pointwise kernels of the fused operator: the gallery QFunctions of the path
 * (include/ceed/jit-source/gallery/ *.h) plus the kappa-weighted diffusion. */
enum {
  B200_QF_MASS           = 0, /* MassApply:             u, qdata(1)            -> v      */
  B200_QF_POISSON        = 1, /* Poisson3DApply:        du, qdata(6)           -> dv     */
  B200_QF_VECMASS        = 2, /* Vector3MassApply:      u(3), qdata(1)         -> v(3)   */
  B200_QF_VECPOISSON     = 3, /* Vector3Poisson3DApply: du(3), qdata(6)        -> dv(3)  */
  B200_QF_POISSON_KAPPA  = 4, /* Poisson3DApply with qdata scaled by kappa[elem][qpt]     */
};

typedef struct b200_ctx_s   *b200_ctx;
typedef struct b200_basis_s *b200_basis;
typedef struct b200_plan_s  *b200_plan;
typedef struct b200_op_s    *b200_op;

/* Message of the last failing call on this thread. */
const char *b200_last_error(void);

/* ---- Context: one per Ceed.  Replaces CeedInit_Cuda device selection (backends/cuda/ceed-cuda-common.c:19-35)
 *      and CeedSetStream (interface/ceed.c:1408). ---------------------------------------------------------------- */
int b200_ctx_create(int device_id, b200_ctx *ctx);
int b200_ctx_set_stream(b200_ctx ctx, void *cuda_stream);
int b200_ctx_get_stream(b200_ctx ctx, void **cuda_stream);
int b200_ctx_sync(b200_ctx ctx);
int b200_ctx_destroy(b200_ctx ctx);
/* Number of kernels this library launched on the context (all entry points). */
int b200_ctx_launch_count(b200_ctx ctx, int64_t *count);
/* Device status word of the context, read and cleared (synchronizes the stream).  0, or an OR of B200_STATUS_* bits
 * set by kernels whose bounded wait on an asynchronous copy gave up (their results are then invalid).  No counterpart
 * in the reference (its kernels do not wait on asynchronous copies). */
enum { B200_STATUS_COPY_TIMEOUT = 1 };
int b200_ctx_status(b200_ctx ctx, int *status);

/* ---- Device memory of CeedVector arrays.  Replaces the device half of CeedVectorCreate_Cuda / SetArray /
 *      SyncArray (backends/cuda-ref/ceed-cuda-ref-vector.c:97-262). ------------------------------------------------ */
int b200_alloc(b200_ctx ctx, size_t bytes, void **dptr);
int b200_free(b200_ctx ctx, void *dptr);
int b200_copy(b200_ctx ctx, void *dst, const void *src, size_t bytes, int kind);

/* ---- Vector BLAS-1.  Replaces backends/cuda-ref/kernels/cuda-ref-vector.cu:14-220 and the cuBLAS norm calls of
 *      backends/cuda-ref/ceed-cuda-ref-vector.c:487-640 (CeedVectorSetValue/Scale/AXPY/AXPBY/PointwiseMult/
 *      Reciprocal/Norm, interface/ceed-vector.c:377-953).  b200_vec_dot has no CeedVector counterpart (the CG
 *      driver needs it); b200_vec_convert copies between precisions. -------------------------------------------- */
int b200_vec_set_value(b200_ctx ctx, int prec, int64_t n, void *x, double value);
int b200_vec_scale(b200_ctx ctx, int prec, int64_t n, void *x, double alpha);
int b200_vec_axpy(b200_ctx ctx, int prec, int64_t n, double alpha, const void *x, void *y);
int b200_vec_axpby(b200_ctx ctx, int prec, int64_t n, double alpha, double beta, const void *x, void *y);
int b200_vec_pointwise_mult(b200_ctx ctx, int prec, int64_t n, void *w, const void *x, const void *y);
int b200_vec_reciprocal(b200_ctx ctx, int prec, int64_t n, void *x);
int b200_vec_norm(b200_ctx ctx, int prec, int64_t n, const void *x, int norm_type, double *norm);
int b200_vec_dot(b200_ctx ctx, int prec, int64_t n, const void *x, const void *y, double *dot);
int b200_vec_convert(b200_ctx ctx, int64_t n, int src_prec, const void *src, int dst_prec, void *dst);

/* ---- Strided vector access.  Replaces CeedVectorSetValueStrided / CeedVectorCopyStrided
 *      (interface/ceed-vector.c:412, :300) and their device kernels setValueStridedK / copyStridedK
 *      (backends/cuda-ref/kernels/cuda-ref-vector.cu:14-80): entries start, start + step, ... below stop, with
 *      stop = -1 meaning `length` (for the copy, the shorter of the two vectors' lengths).  stop outside [-1, length],
 *      start outside [0, stop] or step <= 0 return B200_ERROR_ACCESS before anything runs. */
int b200_vec_set_value_strided(b200_ctx ctx, int prec, int64_t length, int64_t start, int64_t stop, int64_t step, void *x, double value);
int b200_vec_copy_strided(b200_ctx ctx, int prec, int64_t length, int64_t start, int64_t stop, int64_t step, const void *x, void *y);

/* ---- Element restriction.  Offset form replaces OffsetNoTranspose / OffsetTranspose
 *      (include/ceed/jit-source/cuda/cuda-ref-restriction-offset.h:15-67, host side
 *      backends/cuda-ref/ceed-cuda-ref-restriction.c); strided form replaces cuda-ref-restriction-strided.h.
 *      Gather: e = E l (bit-exact copy).  Scatter: l += E^T e, atomic (any order) or deterministic (fixed
 *      per-node order from the inverse-offset plan, bit-reproducible run to run). ------------------------------- */
int b200_rstr_gather(b200_ctx ctx, int prec, int64_t num_elem, int elem_size, int num_comp, int64_t comp_stride, int64_t l_size,
                     const int32_t *offsets, const void *l_vec, void *e_vec);
int b200_rstr_scatter_atomic(b200_ctx ctx, int prec, int64_t num_elem, int elem_size, int num_comp, int64_t comp_stride, int64_t l_size,
                             const int32_t *offsets, const void *e_vec, void *l_vec);
/* Inverse-offset plan for the deterministic scatter: replaces the host CSR build of
 * backends/cuda-ref/ceed-cuda-ref-restriction.c:416-493.  offsets_host may be NULL when offsets_dev is given. */
int b200_plan_create(b200_ctx ctx, int64_t num_elem, int elem_size, int num_comp, int64_t comp_stride, int64_t l_size,
                     const int32_t *offsets_host, const int32_t *offsets_dev, b200_plan *plan);
int b200_plan_destroy(b200_plan plan);
/* l = E^T e (add = 0; entries the restriction does not reach become 0) or l += E^T e (add = 1), summing each node's
 * entries in ascending E-index order. */
int b200_rstr_scatter_det(b200_ctx ctx, b200_plan plan, int prec, const void *e_vec, void *l_vec, int add);
int b200_rstr_strided_gather(b200_ctx ctx, int prec, int64_t num_elem, int elem_size, int num_comp, const int64_t strides[3],
                             const void *l_vec, void *e_vec);
int b200_rstr_strided_scatter(b200_ctx ctx, int prec, int64_t num_elem, int elem_size, int num_comp, const int64_t strides[3],
                              const void *e_vec, void *l_vec);

/* ---- Tensor H1 basis (dim 1..3, P, Q <= 16).  Replaces CeedBasisCreateTensorH1_Cuda and the Interp/Grad/Weight
 *      kernels of include/ceed/jit-source/cuda/cuda-ref-basis-tensor.h (CeedBasisApply / ApplyAdd,
 *      interface/ceed-basis.c:2083-2111).  add = 1 accumulates into v (TRANSPOSE only, as ApplyAdd). ------------ */
int b200_basis_create(b200_ctx ctx, int dim, int P_1d, int Q_1d, int num_comp, const double *interp_1d, const double *grad_1d,
                      const double *q_weight_1d, b200_basis *basis);
int b200_basis_apply(b200_basis basis, int prec, int64_t num_elem, int t_mode, int eval_mode, int add, const void *u, void *v);
int b200_basis_destroy(b200_basis basis);

/* ---- Gallery QFunctions on Q-vectors (unfused path).  Replaces CeedQFunctionApply_Cuda with the JIT'd gallery
 *      sources (backends/cuda-ref/ceed-cuda-ref-qfunction.c).  in/out are arrays of device pointers in the order of
 *      the gallery field lists; kappa-weighted diffusion takes (du, qdata, kappa). ------------------------------ */
int b200_qf_apply(b200_ctx ctx, int prec, int qf_kind, int64_t num_points, const void *const *in, void *const *out);

/* ---- Geometric factors.  Replaces the setup operator with gallery Mass3DBuild / Poisson3DBuild
 *      (include/ceed/jit-source/gallery/ceed-mass3dbuild.h, ceed-poisson3dbuild.h) on a trilinear coordinate field:
 *      coords has 3 components at comp_stride, x_offsets are [elem][8] vertex offsets.  qdata (FP64) is written in
 *      the backend layout [comp][elem][qpt] with 1 (mass) or 6 (Poisson, Voigt order) components. ------------- */
int b200_qdata_build(b200_ctx ctx, int poisson, int64_t num_elem, int Q_1d, const double *x_interp_1d, const double *x_grad_1d,
                     const double *q_weight_1d, const int32_t *x_offsets, int64_t x_comp_stride, const double *coords, double *qdata);

/* ---- Fused operator apply (the hot path).  Replaces CeedOperatorApplyAdd_Cuda_gen and its generated kernel
 *      (backends/cuda-gen/ceed-cuda-gen-operator.c:105-300, ceed-cuda-gen-operator-build.cpp:1158-1680) and the
 *      ref backend's element loop (backends/ref/ceed-ref-operator.c:381-476): gather -> interp/grad -> pointwise
 *      kernel -> transposes -> scatter in one kernel per element batch. -------------------------------------------- */
typedef struct {
  int            qf;          /* B200_QF_* */
  int            prec;        /* B200_F64, B200_F32 or B200_F64X (centro-symmetric bases) */
  int            P_1d, Q_1d;  /* Q_1d = P_1d + 1 for the compiled kernels, P_1d in 2..9 */
  int            num_comp;    /* 1, or 3 for the vector QFunctions */
  int            scatter;     /* B200_SCATTER_ATOMIC or B200_SCATTER_DETERMINISTIC */
  int64_t        num_elem;
  int64_t        l_size;      /* length of u and v */
  int64_t        comp_stride; /* component stride of the L-vector */
  const int32_t *offsets;     /* device, [elem][P^3] */
  const double  *interp_1d;   /* host, Q x P */
  const double  *grad_1d;     /* host, Q x P */
  int            elems_per_block; /* 0: tuned default */
  int            staging;         /* 0: default, 1: registers, 2: shared memory, 3: persistent pipelined,
                                     4: point (Q^3-thread) mapping, 5: bulk-copy (TMA) qdata slabs,
                                     6: none (qdata read from global memory in the pointwise stage),
                                     7: persistent blocks with bulk-copy staging one batch ahead (FP32, one component) */
} b200_op_desc;

int b200_op_create(b200_ctx ctx, const b200_op_desc *desc, b200_op *op);
/* v = A u (add = 0, CeedOperatorApply) or v += A u (add = 1, CeedOperatorApplyAdd).  qdata: [comp][elem][qpt] in
 * the operator's storage precision (double for B200_F64 and B200_F64X); kappa: [elem][qpt] or NULL.  With no elements
 * Apply zeroes v and ApplyAdd leaves it; u and qdata may then be NULL. */
int b200_op_apply(b200_op op, const void *u, void *v, const void *qdata, const void *kappa, int add);
/* v = A u together with u . (A u), for CG-type solvers (no counterpart in the reference, whose solvers take the dot
 * product in a separate pass).  Only for operators whose kernel is the persistent FP32 one (staging 7) with the atomic
 * scatter: b200_op_dot_len sets *blocks to the number of per-block partial sums (0: not available for this operator, and
 * b200_op_apply_dot returns B200_ERROR_UNSUPPORTED) and *doubles to the length of the device array `partial` that
 * b200_op_apply_dot needs (at least *blocks).  After the apply, partial[0 .. *blocks) hold the per-block sums (FP64; the
 * kernel sums each thread's quadrature-point terms (grad u)^T D (grad u), or u q u for the mass, in float-float).
 * Their sum, in order, is u . (A u) (exact for the assembled operator: u . A u = sum over elements of u_e . A_e u_e). */
int b200_op_dot_len(b200_op op, int *blocks, int64_t *doubles);
int b200_op_apply_dot(b200_op op, const void *u, void *v, const void *qdata, double *partial);
/* Algorithmic bytes and FLOPs of one apply (for roofline reporting). */
int b200_op_cost(b200_op op, double *bytes, double *flops);
/* The reference's FLOP model of one apply of a fused operator, CeedOperatorGetFlopsEstimate
 * (interface/ceed-operator.c:1834-1960, with CeedBasisGetFlopsEstimate at interface/ceed-basis.c:954 and
 * CeedElemRestrictionGetFlopsEstimate at interface/ceed-elemrestriction.c:576, and the gallery QFunctions' estimates:
 * Poisson 15, mass 1, times the components for the vector ones; the kappa-weighted Poisson, not in the gallery, 21).
 * Pure host arithmetic (no GPU). */
int b200_flops_estimate(int qf, int P_1d, int Q_1d, int num_comp, int64_t num_elem, int64_t *flops);
/* Launch shape in use: elements per block and threads per block. */
int b200_op_get_tile(b200_op op, int *elems_per_block, int *threads_per_block, int *staging);
int b200_op_set_tile(b200_op op, int elems_per_block, int staging);
/* Largest elements-per-block the kernel of a staging mode can launch with (threads and shared memory). */
int b200_op_tile_limits(b200_op op, int staging, int *max_elems_per_block);
/* Device time of one v += A u with the current tile, averaged over reps launches (CUDA events; used by the
 * autotuner, which sweeps elements per block, thread mapping and qdata staging per (P, Q, components, precision)).
 * No counterpart in the reference, whose cuda-gen backend sizes blocks by a heuristic
 * (backends/cuda-gen/ceed-cuda-gen-operator.c:40-97). */
int b200_op_time(b200_op op, const void *u, void *v, const void *qdata, const void *kappa, int reps, double *ms_per_apply);
int b200_op_destroy(b200_op op);

/* ---- Diagonal assembly.  Replaces CeedOperatorLinearAssembleDiagonal (interface/ceed-preconditioning.c:2395) and
 *      include/ceed/jit-source/cuda/cuda-ref-operator-assemble-diagonal.h for the mass (poisson = 0, qdata 1 comp) and
 *      diffusion (poisson = 1, qdata 6 comps, optional kappa [elem][qpt]) operators: diag = sum_e E^T diag(A_e), FP64.
 *      The same diagonal serves every component of a vector field (num_comp, comp_stride).  det_plan (from
 *      b200_plan_create on the same offsets) makes the sum deterministic; NULL uses atomics. */
int b200_assemble_diagonal(b200_ctx ctx, int poisson, int P_1d, int Q_1d, int64_t num_elem, int num_comp, int64_t comp_stride, int64_t l_size,
                           const double *interp_1d, const double *grad_1d, const int32_t *offsets, const double *qdata, const double *kappa,
                           double *diag, b200_plan det_plan);

/* ---- QFunctions compiled at run time.  Replaces the NVRTC QFunction path of the reference
 *      (backends/cuda/ceed-cuda-compile.cpp:70-240, backends/cuda-gen/ceed-cuda-gen-operator-build.cpp:1343-1361): the
 *      QFunction source ("file.h:Name" of CeedQFunctionCreateInterior, split into path and name) is compiled with NVRTC
 *      for sm_103a into the fused kernel template, with CeedScalar = the operator's precision.  One active
 *      one-component field (CEED_EVAL_INTERP or CEED_EVAL_GRAD in and out); every other input is passive with
 *      CEED_EVAL_NONE through a backend-strided restriction ([comp][elem][qpt]). */
typedef struct {
  const char *source_path;   /* file holding the CEED_QFUNCTION */
  const char *name;          /* its name */
  int         num_inputs;    /* QFunction inputs, in declaration order (at most 8) */
  int         input_size[8]; /* field sizes (3 for a GRAD scalar field, 1 for INTERP, qdata sizes ...) */
  int         active_input;  /* index of the active input */
  int         eval_in;       /* B200_EVAL_INTERP or B200_EVAL_GRAD */
  int         eval_out;      /* B200_EVAL_INTERP or B200_EVAL_GRAD (the single output is active) */
  const char *include_dirs;  /* extra include directories, ':'-separated, or NULL */
} b200_jit_qfunction;

int b200_op_create_jit(b200_ctx ctx, const b200_op_desc *desc, const b200_jit_qfunction *qf, b200_op *op);
/* Compile the fused kernel for a QFunction source without loading it (no GPU needed): returns the NVRTC log through
 * b200_last_error on failure. */
int b200_jit_compile_check(const b200_jit_qfunction *qf, int prec, int P_1d);
/* passive: device pointers of the passive inputs in QFunction order (skipping the active one); qf_ctx: the
 * QFunction context data in device memory, or NULL. */
int b200_op_apply_jit(b200_op op, const void *u, void *v, const void *const *passive, void *qf_ctx, int add);

/* Adjoint of the kappa-weighted diffusion with respect to kappa: g[elem][qpt] = grad(w) . D grad(u), recomputing the
 * gradients from u and w (no stored E-vectors).  Both in the operator's precision. */
int b200_op_kappa_grad(b200_op op, const void *u, const void *w, const void *qdata, void *g);

/* ---- Conjugate gradients on the fused operator (no libCEED counterpart: the reference solves with PETSc KSPCG around
 *      CeedOperatorApply in examples/petsc/bps.c).  Homogeneous Dirichlet conditions through mask (exactly 1 free, 0 fixed):
 *      solves m A(m x) = m b from x = 0.  mixed = 0: FP64 CG.  mixed = 1: FP32 CG (op32, qdata32) on the defect
 *      r = m(b - A64 x), computed in FP64, until |r| / |b| <= rtol.  Dot products and norms are summed per thread in FP64
 *      (FP64 vectors) or float-float (FP32 vectors), then in FP64, in a fixed order.
 *      Blocks of check_every iterations run as one CUDA graph when use_graph = 1.  b, x, mask: FP64 device arrays
 *      of length n.  With jacobi set (e.g. from b200_assemble_diagonal), the iterations are Jacobi-preconditioned. */
typedef struct {
  double rtol;        /* target |m(b - A x)| / |b| */
  int    max_it;      /* cap on CG iterations (all inner iterations in mixed mode) */
  int    mixed;       /* 0: FP64 CG, 1: FP32 CG inside FP64 refinement */
  double inner_rtol;  /* mixed: relative residual reduction of each inner solve */
  int    max_outer;   /* mixed: cap on refinement steps */
  int    use_graph;   /* capture iteration blocks in CUDA graphs */
  int    check_every; /* iterations between convergence checks (graph size) */
  const double *jacobi; /* Jacobi preconditioner: masked 1/diag(A) (FP64, device, length n), or NULL for plain CG */
  int    separate_pdot; /* mixed: 1 takes p.(A p) in a pass over p and A p even where the FP32 operator's persistent kernel
                           sums it element by element during the apply (0, the default) */
} b200_cg_opts;

typedef struct {
  int     iterations;   /* CG iterations (summed over refinement steps) */
  int     outer;        /* refinement steps (1 for FP64 CG) */
  int     converged;
  double  rel_residual; /* final |m(b - A64 x)| / |b|, recomputed in FP64 */
  double  seconds;      /* device time of the solve (CUDA events) */
  int64_t launches;     /* kernels run by the solve */
} b200_cg_stats;

/* ---- Dot product that allocates nothing.  No counterpart in the reference: for callers that cannot allocate device
 *      memory when they need the reduction (an application allocator that owns all device memory, or a loop that must
 *      not call cudaMalloc/cudaFree because they can synchronize the device).  Same arithmetic as b200_vec_dot (FP64
 *      accumulation, fixed order), but the partial sums live in a 128 KiB array inside this library that every GPU
 *      loading it keeps until exit, and the result goes to `result`, one double in device memory, asynchronously on
 *      `cuda_stream`; no b200_ctx is needed.  n is limited to 134,217,728 entries (B200_ERROR_DIMENSION beyond).  All
 *      calls share the array: calls that overlap on the GPU race, so order them on one stream.  The first call on a
 *      device looks up the array's address with that device current; make it before any stream capture. */
int b200_vec_dot_static(int prec, int64_t n, const void *x, const void *y, double *result, void *cuda_stream);

int b200_cg_solve(b200_ctx ctx, b200_op op64, b200_op op32, const void *qdata64, const void *qdata32, const double *mask, const double *b,
                  double *x, int64_t n, const b200_cg_opts *opts, b200_cg_stats *stats);

/* ---- Pipe throughput probe.  No counterpart in the reference: measures the fused multiply-add rate of the FP64
 *      (prec B200_F64) or FP32 (B200_F32) pipe of the context's GPU with independent FMA chains on every SM, so that
 *      compute-bound kernels report a fraction of a measured peak.  Blocks the host; *tflops = 2 * FMAs / s / 1e12. */
int b200_fma_peak(b200_ctx ctx, int prec, double *tflops);

/* ---- FP64 tensor-core probe.  No counterpart in the reference: *dmma_tflops is the FP64 rate of the tensor-core
 *      instruction mma.sync m8n8k4 (DMMA) alone; *mixed_tflops the total FP64 rate when every warp interleaves DMMA
 *      chains with DFMA chains.  A mixed rate no higher than the larger single rate means the two share one FP64 unit,
 *      so moving contractions of the FP64 kernels onto the tensor path cannot raise their bound.  Blocks the host. */
int b200_fp64_tensor_peak(b200_ctx ctx, double *dmma_tflops, double *mixed_tflops);

/* ---- Bounded-wait self-test.  No counterpart in the reference: one block waits, with the bounded mbarrier wait of the
 *      bulk-copy kernels and at most max_polls polls (1..65536), on a barrier that nothing completes, and records the
 *      give-up in the context's status word (B200_STATUS_COPY_TIMEOUT, read with b200_ctx_status), so that this path
 *      is exercised without a fault; the context stays usable.  Blocks the host. */
int b200_wait_selftest(b200_ctx ctx, int max_polls);

#ifdef __cplusplus
}
#endif
#endif
