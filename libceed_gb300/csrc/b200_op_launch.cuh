// Host-side launchers of the fused operator kernels and the table that maps (precision, QFunction, P, variant) to a
// compiled instance.  Instances are spread over several translation units (b200_op_inst_*.cu) so the build runs in
// parallel.
#pragma once

#include "b200_internal.cuh"
#include "b200_op_kernels.cuh"

namespace b200 {

constexpr int kOpPMin = 2, kOpPMax = 9;  // compiled range of P_1d (Q_1d = P_1d + 1)

// Kernel variants: qdata staging x contraction form.
enum {
  kVarReg = 0, kVarSmem = 1, kVarRegEO = 2, kVarSmemEO = 3, kVarPipeEO = 4, kVar3D = 5, kVarTma = 6, kVarTmaEO = 7, kVarLate = 8, kVarLateEO = 9,
  kVarPTma = 10, kVarPTmaEO = 11, kNumVariants = 12
};

// Untyped launch request; pointers are reinterpreted in the instance's precision.
struct OpLaunch {
  int64_t        num_elem, comp_stride;
  int            epb, det;
  int            grid;  // persistent variant: number of blocks
  const int32_t *offsets;
  const void    *u, *qdata, *kappa, *w;  // w: second field of the kappa gradient
  void          *v, *e_out, *g;
  const double  *B, *G;  // host 1D matrices, Q x P and Q x Q
  int           *status;  // device status word of the context
  double        *dot;     // persistent FP32 kernel: per-block sums of u . (A u) (one per block of the grid), or nullptr
};

using OpLauncher  = int (*)(b200_ctx ctx, const OpLaunch &req);
using OpSmemFn    = size_t (*)(int epb);
using OpOccupancy = int (*)(int epb);  // resident blocks per SM

struct OpInstance {
  OpLauncher  launch;
  OpSmemFn    smem;
  OpOccupancy occupancy;
  int         max_threads;  // from cudaFuncGetAttributes (register-limited)
  bool        persistent;
  OpOccupancy dot_occupancy = nullptr;  // persistent FP32 kernel: blocks per SM of its form that also sums u . (A u)
};

// Even-odd form of a row-major J x K matrix M with parity par (+1 or -1).
template <typename T, int J, int K>
inline void make_eo(const double *M, int par, EOMat<T, J, K> &out) {
  constexpr int Jh = J / 2, Kh = K / 2;
  for (int j = 0; j < Jh; j++)
    for (int k = 0; k < Kh; k++) {
      out.E[j * Kh + k] = (T)(0.5 * (M[j * K + k] + M[j * K + K - 1 - k]));
      out.O[j * Kh + k] = (T)(0.5 * (M[j * K + k] - M[j * K + K - 1 - k]));
    }
  for (int j = 0; j <= Jh; j++) out.C[j] = (T)((K % 2 && j < Jh) ? M[j * K + Kh] : 0.0);
  for (int k = 0; k <= Kh; k++) out.R[k] = (T)0.0;
  if (J % 2) {
    const double *row = M + Jh * K;
    for (int k = 0; k < Kh; k++) out.R[k] = (T)(par > 0 ? 0.5 * (row[k] + row[K - 1 - k]) : 0.5 * (row[k] - row[K - 1 - k]));
    if (K % 2 && par > 0) out.R[Kh] = (T)row[Kh];
  }
}

template <typename T, int P, int Q>
inline OpMats<T, P, Q> make_mats(const double *B, const double *G) {
  OpMats<T, P, Q> m;
  double          Bt[P * Q], Gt[Q * Q];
  for (int i = 0; i < Q * P; i++) m.B[i] = (T)B[i];
  for (int i = 0; i < Q * Q; i++) m.G[i] = (T)G[i];
  for (int i = 0; i < Q; i++)
    for (int j = 0; j < P; j++) Bt[j * Q + i] = B[i * P + j];
  for (int i = 0; i < Q; i++)
    for (int j = 0; j < Q; j++) Gt[j * Q + i] = G[i * Q + j];
  make_eo<T, Q, P>(B, 1, m.Be);
  make_eo<T, P, Q>(Bt, 1, m.Bte);
  make_eo<T, Q, Q>(G, -1, m.Ge);
  make_eo<T, Q, Q>(Gt, -1, m.Gte);
  return m;
}

template <typename T>
inline OpArgs<typename Store<T>::type> make_args(const OpLaunch &r) {
  using S = typename Store<T>::type;
  OpArgs<S> a;
  a.num_elem    = r.num_elem;
  a.comp_stride = r.comp_stride;
  a.epb         = r.epb;
  a.det         = r.det;
  a.offsets     = r.offsets;
  a.u           = (const S *)r.u;
  a.v           = (S *)r.v;
  a.e_out       = (S *)r.e_out;
  a.qdata       = (const S *)r.qdata;
  a.kappa       = (const S *)r.kappa;
  a.status      = r.status;
  a.dot         = r.dot;
  return a;
}

template <typename T, int P, int QF, int STAGE>
size_t op_smem(int epb) {
  constexpr int Q = P + 1;
  size_t        prefix = 0;
  if constexpr (STAGE == kStageTma) prefix = tma_prefix_bytes<typename Store<T>::type, Q, QFTraits<QF>::nqk>(epb);
  if constexpr (TileMap<T, Q, STAGE>::tuned) return prefix + sizeof(T) * 3 * (size_t)TileMap<T, Q, STAGE>::region(epb);
  return prefix + sizeof(T) * (size_t)epb * OpShape<T, P, Q, QF, STAGE>::team_smem;
}

template <typename K>
inline int blocks_per_sm(K kern, int threads, size_t smem) {
  int n = 0;
  if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, threads, smem) != cudaSuccess) return 0;
  return n;
}

template <typename T, int P, int QF, int STAGE, bool EO>
int op_launch(b200_ctx ctx, const OpLaunch &r) {
  constexpr int Q    = P + 1;
  auto          kern = k_op_apply<T, P, Q, QF, STAGE, EO>;
  const size_t  smem = op_smem<T, P, QF, STAGE>(r.epb);
  if (smem > 48 * 1024) B200_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t grid = ceil_div(r.num_elem, r.epb);
  kern<<<(unsigned)grid, r.epb * Q * Q, smem, ctx->stream>>>(make_args<T>(r), make_mats<T, P, Q>(r.B, r.G));
  B200_LAUNCHED(ctx, "op_apply");
  return B200_SUCCESS;
}

template <typename T, int P, int QF>
int op_launch_pipe(b200_ctx ctx, const OpLaunch &r) {
  constexpr int Q    = P + 1;
  auto          kern = k_op_apply_pipe<T, P, Q, QF>;
  const size_t  smem = op_smem<T, P, QF, kStagePipe>(r.epb);
  if (smem > 48 * 1024) B200_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t nbatch = ceil_div(r.num_elem, r.epb);
  const int64_t grid   = r.grid < nbatch ? r.grid : nbatch;
  kern<<<(unsigned)(grid > 0 ? grid : 1), r.epb * Q * Q, smem, ctx->stream>>>(make_args<T>(r), make_mats<T, P, Q>(r.B, r.G));
  B200_LAUNCHED(ctx, "op_apply_pipe");
  return B200_SUCCESS;
}

template <typename T, int P, int QF>
size_t op_smem_3d(int epb) {
  using SH = Op3DShape<T, P, P + 1>;
  return sizeof(T) * ((size_t)SH::mats + (size_t)epb * SH::team);
}

template <typename T, int P, int QF>
int op_launch_3d(b200_ctx ctx, const OpLaunch &r) {
  constexpr int Q    = P + 1;
  auto          kern = k_op_apply_3d<T, P, Q, QF>;
  const size_t  smem = op_smem_3d<T, P, QF>(r.epb);
  if (smem > 48 * 1024) B200_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t grid = ceil_div(r.num_elem, r.epb);
  kern<<<(unsigned)grid, r.epb * Q * Q * Q, smem, ctx->stream>>>(make_args<T>(r), make_mats<T, P, Q>(r.B, r.G));
  B200_LAUNCHED(ctx, "op_apply_3d");
  return B200_SUCCESS;
}

template <typename T, int P, int QF>
int op_occupancy_3d(int epb) {
  return blocks_per_sm(k_op_apply_3d<T, P, P + 1, QF>, epb * (P + 1) * (P + 1) * (P + 1), op_smem_3d<T, P, QF>(epb));
}

template <typename T, int P, int QF>
OpInstance op_instance_3d() {
  OpInstance         inst{op_launch_3d<T, P, QF>, op_smem_3d<T, P, QF>, op_occupancy_3d<T, P, QF>, 1024, false};
  cudaFuncAttributes attr;
  if (cudaFuncGetAttributes(&attr, k_op_apply_3d<T, P, P + 1, QF>) == cudaSuccess) inst.max_threads = attr.maxThreadsPerBlock;
  return inst;
}

template <typename T, int P>
int kgrad_launch(b200_ctx ctx, const OpLaunch &r) {
  constexpr int Q    = P + 1;
  auto          kern = k_kappa_grad<T, P, Q>;
  const size_t  smem = sizeof(T) * (size_t)r.epb * tile_team_stride(Q, 0);
  if (smem > 48 * 1024) B200_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t grid = ceil_div(r.num_elem, r.epb);
  kern<<<(unsigned)grid, r.epb * Q * Q, smem, ctx->stream>>>(make_args<T>(r), (const T *)r.w, (T *)r.g, make_mats<T, P, Q>(r.B, r.G));
  B200_LAUNCHED(ctx, "op_kappa_grad");
  return B200_SUCCESS;
}

template <typename T, int P, int QF, int STAGE, bool EO>
int op_occupancy(int epb) {
  return blocks_per_sm(k_op_apply<T, P, P + 1, QF, STAGE, EO>, epb * (P + 1) * (P + 1), op_smem<T, P, QF, STAGE>(epb));
}

template <typename T, int P, int QF>
int op_occupancy_pipe(int epb) {
  return blocks_per_sm(k_op_apply_pipe<T, P, P + 1, QF>, epb * (P + 1) * (P + 1), op_smem<T, P, QF, kStagePipe>(epb));
}

template <typename T, int P, int QF, int STAGE, bool EO>
OpInstance op_instance() {
  OpInstance         inst{op_launch<T, P, QF, STAGE, EO>, op_smem<T, P, QF, STAGE>, op_occupancy<T, P, QF, STAGE, EO>, 1024, false};
  cudaFuncAttributes attr;
  if (cudaFuncGetAttributes(&attr, k_op_apply<T, P, P + 1, QF, STAGE, EO>) == cudaSuccess) inst.max_threads = attr.maxThreadsPerBlock;
  return inst;
}

template <typename T, int P, int QF>
OpInstance op_instance_pipe() {
  OpInstance         inst{op_launch_pipe<T, P, QF>, op_smem<T, P, QF, kStagePipe>, op_occupancy_pipe<T, P, QF>, 1024, true};
  cudaFuncAttributes attr;
  if (cudaFuncGetAttributes(&attr, k_op_apply_pipe<T, P, P + 1, QF>) == cudaSuccess) inst.max_threads = attr.maxThreadsPerBlock;
  return inst;
}

// The persistent FP32 kernel: the 64-register instance at P = 5.
template <typename T, int P, int QF, bool EO, bool DOT = false>
constexpr auto ptma_kernel() {
  if constexpr (P == 5) return k_op_apply_ptma_r64<T, P, P + 1, QF, EO, DOT>;
  else return k_op_apply_ptma<T, P, P + 1, QF, EO, DOT>;
}

// The DOT form keeps each thread's running float-float sum (two floats) after the tile buffers.
template <typename T, int P, int QF, bool DOT>
size_t op_smem_ptma(int epb) {
  return op_smem<T, P, QF, kStageTma>(epb) + (DOT ? (size_t)epb * (P + 1) * (P + 1) * 2 * sizeof(float) : 0);
}

// With r.dot set, the DOT instance also writes one partial sum of u . (A u) per block, r.grid of them (blocks past
// the last batch write 0).
template <typename T, int P, int QF, bool EO>
int op_launch_ptma(b200_ctx ctx, const OpLaunch &r) {
  constexpr int Q    = P + 1;
  auto          kern = r.dot ? ptma_kernel<T, P, QF, EO, true>() : ptma_kernel<T, P, QF, EO>();
  const size_t  smem = r.dot ? op_smem_ptma<T, P, QF, true>(r.epb) : op_smem_ptma<T, P, QF, false>(r.epb);
  if (smem > 48 * 1024) B200_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t nbatch = ceil_div(r.num_elem, r.epb);
  const int64_t grid   = r.dot ? r.grid : (r.grid < nbatch ? r.grid : nbatch);
  if (grid <= 0) return B200_SUCCESS;
  kern<<<(unsigned)grid, r.epb * Q * Q, smem, ctx->stream>>>(make_args<T>(r), make_mats<T, P, Q>(r.B, r.G));
  B200_LAUNCHED(ctx, "op_apply_ptma");
  return B200_SUCCESS;
}

template <typename T, int P, int QF, bool EO, bool DOT>
int op_occupancy_ptma(int epb) {
  return blocks_per_sm(ptma_kernel<T, P, QF, EO, DOT>(), epb * (P + 1) * (P + 1), op_smem_ptma<T, P, QF, DOT>(epb));
}

template <typename T, int P, int QF, bool EO>
OpInstance op_instance_ptma() {
  OpInstance inst{op_launch_ptma<T, P, QF, EO>, op_smem<T, P, QF, kStageTma>, op_occupancy_ptma<T, P, QF, EO, false>, 1024, true,
                  op_occupancy_ptma<T, P, QF, EO, true>};
  cudaFuncAttributes attr;
  if (cudaFuncGetAttributes(&attr, ptma_kernel<T, P, QF, EO>()) == cudaSuccess) inst.max_threads = attr.maxThreadsPerBlock;
  return inst;
}

template <typename T, int P, int QF>
bool op_variant(int variant, OpInstance *out) {
  if constexpr (__is_same(T, dfloat)) {
    // Float-float: only the even-odd kernels (half the multiply-adds, which cost ~15 FP32 operations each).
    if (variant == kVarRegEO) *out = op_instance<T, P, QF, kStageReg, true>();
    else if (variant == kVarSmemEO) *out = op_instance<T, P, QF, kStageSmem, true>();
    else if (variant == kVarTmaEO) *out = op_instance<T, P, QF, kStageTma, true>();
    else if (variant == kVarLateEO) *out = op_instance<T, P, QF, kStageLate, true>();
    else if (variant == kVar3D) *out = op_instance_3d<T, P, QF>();
    else return false;
    return true;
  } else {
    switch (variant) {
      case kVarReg: *out = op_instance<T, P, QF, kStageReg, false>(); return true;
      case kVarSmem: *out = op_instance<T, P, QF, kStageSmem, false>(); return true;
      case kVarRegEO: *out = op_instance<T, P, QF, kStageReg, true>(); return true;
      case kVarSmemEO: *out = op_instance<T, P, QF, kStageSmem, true>(); return true;
      case kVarPipeEO:
        if constexpr (QFTraits<QF>::nc == 1) {
          *out = op_instance_pipe<T, P, QF>();
          return true;
        } else {
          return false;
        }
      case kVar3D: *out = op_instance_3d<T, P, QF>(); return true;
      case kVarTma: *out = op_instance<T, P, QF, kStageTma, false>(); return true;
      case kVarTmaEO: *out = op_instance<T, P, QF, kStageTma, true>(); return true;
      case kVarLate: *out = op_instance<T, P, QF, kStageLate, false>(); return true;
      case kVarLateEO: *out = op_instance<T, P, QF, kStageLate, true>(); return true;
      case kVarPTma:
      case kVarPTmaEO:
        if constexpr (__is_same(T, float) && QFTraits<QF>::nc == 1) {
          *out = variant == kVarPTma ? op_instance_ptma<T, P, QF, false>() : op_instance_ptma<T, P, QF, true>();
          return true;
        } else {
          return false;
        }
      default: return false;
    }
  }
}

// Lookup implemented by the instance translation units.  Returns false when no instance exists.
bool op_lookup(int prec, int qf, int P, int variant, OpInstance *out);
bool kgrad_lookup(int prec, int P, OpLauncher *out);

}  // namespace b200

// Instantiate the table slice for one (T, QF): P = 2..9, every variant.
#define B200_OP_TABLE(T, QF, FN)                                           \
  namespace b200 {                                                         \
  bool FN(int P, int variant, OpInstance *out) {                           \
    switch (P) {                                                           \
      case 2: return op_variant<T, 2, QF>(variant, out);                  \
      case 3: return op_variant<T, 3, QF>(variant, out);                  \
      case 4: return op_variant<T, 4, QF>(variant, out);                  \
      case 5: return op_variant<T, 5, QF>(variant, out);                  \
      case 6: return op_variant<T, 6, QF>(variant, out);                  \
      case 7: return op_variant<T, 7, QF>(variant, out);                  \
      case 8: return op_variant<T, 8, QF>(variant, out);                  \
      case 9: return op_variant<T, 9, QF>(variant, out);                  \
      default: return false;                                               \
    }                                                                      \
  }                                                                        \
  }
