// Host-side launchers of the fused operator kernels and the table that maps (precision, QFunction, P, staging) to
// a compiled instance.  Instances are spread over several translation units (b200_op_inst_*.cu) so the build runs in
// parallel.
#pragma once

#include "b200_internal.cuh"
#include "b200_op_kernels.cuh"

namespace b200 {

constexpr int kOpPMin = 2, kOpPMax = 9;  // compiled range of P_1d (Q_1d = P_1d + 1)

// Untyped launch request; pointers are reinterpreted in the instance's precision.
struct OpLaunch {
  int64_t        num_elem, comp_stride;
  int            epb, det;
  const int32_t *offsets;
  const void    *u, *qdata, *kappa, *w;  // w: second field of the kappa gradient
  void          *v, *e_out, *g;
  const double  *B, *G;  // host 1D matrices, Q x P and Q x Q
};

using OpLauncher = int (*)(b200_ctx ctx, const OpLaunch &req);
using OpSmemFn   = size_t (*)(int epb);

struct OpInstance {
  OpLauncher launch;
  OpSmemFn   smem;
  int        max_threads;  // from cudaFuncGetAttributes (register-limited)
};

template <typename T, int P, int Q>
inline OpMats<T, P, Q> make_mats(const double *B, const double *G) {
  OpMats<T, P, Q> m;
  for (int i = 0; i < Q * P; i++) m.B[i] = (T)B[i];
  for (int i = 0; i < Q * Q; i++) m.G[i] = (T)G[i];
  return m;
}

template <typename T>
inline OpArgs<T> make_args(const OpLaunch &r) {
  OpArgs<T> a;
  a.num_elem    = r.num_elem;
  a.comp_stride = r.comp_stride;
  a.epb         = r.epb;
  a.det         = r.det;
  a.offsets     = r.offsets;
  a.u           = (const T *)r.u;
  a.v           = (T *)r.v;
  a.e_out       = (T *)r.e_out;
  a.qdata       = (const T *)r.qdata;
  a.kappa       = (const T *)r.kappa;
  return a;
}

template <typename T, int P, int QF, int STAGE>
size_t op_smem(int epb) {
  return sizeof(T) * (size_t)epb * OpShape<T, P, P + 1, QF, STAGE>::team_smem;
}

template <typename T, int P, int QF, int STAGE>
int op_launch(b200_ctx ctx, const OpLaunch &r) {
  constexpr int Q    = P + 1;
  auto          kern = k_op_apply<T, P, Q, QF, STAGE>;
  const size_t  smem = op_smem<T, P, QF, STAGE>(r.epb);
  if (smem > 48 * 1024) B200_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t grid = ceil_div(r.num_elem, r.epb);
  kern<<<(unsigned)grid, r.epb * Q * Q, smem, ctx->stream>>>(make_args<T>(r), make_mats<T, P, Q>(r.B, r.G));
  B200_LAUNCHED(ctx, "op_apply");
  return B200_SUCCESS;
}

template <typename T, int P>
int kgrad_launch(b200_ctx ctx, const OpLaunch &r) {
  constexpr int Q    = P + 1;
  auto          kern = k_kappa_grad<T, P, Q>;
  const size_t  smem = sizeof(T) * (size_t)r.epb * 3 * Q * Q * Q;
  if (smem > 48 * 1024) B200_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t grid = ceil_div(r.num_elem, r.epb);
  kern<<<(unsigned)grid, r.epb * Q * Q, smem, ctx->stream>>>(make_args<T>(r), (const T *)r.w, (T *)r.g, make_mats<T, P, Q>(r.B, r.G));
  B200_LAUNCHED(ctx, "op_kappa_grad");
  return B200_SUCCESS;
}

template <typename T, int P, int QF, int STAGE>
OpInstance op_instance() {
  OpInstance       inst{op_launch<T, P, QF, STAGE>, op_smem<T, P, QF, STAGE>, 1024};
  cudaFuncAttributes attr;
  if (cudaFuncGetAttributes(&attr, k_op_apply<T, P, P + 1, QF, STAGE>) == cudaSuccess) inst.max_threads = attr.maxThreadsPerBlock;
  return inst;
}

// Lookup implemented by the instance translation units.  Returns false when no instance exists.
bool op_lookup(int prec, int qf, int P, int stage, OpInstance *out);
bool kgrad_lookup(int prec, int P, OpLauncher *out);

}  // namespace b200

// Instantiate the table slice for one (T, QF): P = 2..9, both staging modes.
#define B200_OP_TABLE(T, QF, FN)                                                                                              \
  namespace b200 {                                                                                                            \
  bool FN(int P, int stage, OpInstance *out) {                                                                                \
    switch (P * 4 + stage) {                                                                                                  \
      case 2 * 4 + kStageReg: *out = op_instance<T, 2, QF, kStageReg>(); return true;                                         \
      case 2 * 4 + kStageSmem: *out = op_instance<T, 2, QF, kStageSmem>(); return true;                                       \
      case 3 * 4 + kStageReg: *out = op_instance<T, 3, QF, kStageReg>(); return true;                                         \
      case 3 * 4 + kStageSmem: *out = op_instance<T, 3, QF, kStageSmem>(); return true;                                       \
      case 4 * 4 + kStageReg: *out = op_instance<T, 4, QF, kStageReg>(); return true;                                         \
      case 4 * 4 + kStageSmem: *out = op_instance<T, 4, QF, kStageSmem>(); return true;                                       \
      case 5 * 4 + kStageReg: *out = op_instance<T, 5, QF, kStageReg>(); return true;                                         \
      case 5 * 4 + kStageSmem: *out = op_instance<T, 5, QF, kStageSmem>(); return true;                                       \
      case 6 * 4 + kStageReg: *out = op_instance<T, 6, QF, kStageReg>(); return true;                                         \
      case 6 * 4 + kStageSmem: *out = op_instance<T, 6, QF, kStageSmem>(); return true;                                       \
      case 7 * 4 + kStageReg: *out = op_instance<T, 7, QF, kStageReg>(); return true;                                         \
      case 7 * 4 + kStageSmem: *out = op_instance<T, 7, QF, kStageSmem>(); return true;                                       \
      case 8 * 4 + kStageReg: *out = op_instance<T, 8, QF, kStageReg>(); return true;                                         \
      case 8 * 4 + kStageSmem: *out = op_instance<T, 8, QF, kStageSmem>(); return true;                                       \
      case 9 * 4 + kStageReg: *out = op_instance<T, 9, QF, kStageReg>(); return true;                                         \
      case 9 * 4 + kStageSmem: *out = op_instance<T, 9, QF, kStageSmem>(); return true;                                       \
      default: return false;                                                                                                  \
    }                                                                                                                         \
  }                                                                                                                           \
  }
