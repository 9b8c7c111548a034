// Fused operator apply: object lifetime, launch-shape selection and the deterministic scatter.
//
// Takes over CeedOperatorApplyAdd_Cuda_gen / ApplyAddCore (backends/cuda-gen/ceed-cuda-gen-operator.c:105-300):
// one fused kernel launch per apply, block shape chosen per (precision, P, Q, components) instead of the reference's
// occupancy-and-waste heuristic (:40-97).  With the deterministic scatter the fused kernel writes the element results
// and the inverse-offset plan sums them in a fixed order.
#include "b200_internal.cuh"
#include "b200_jit.cuh"
#include "b200_op_launch.cuh"
#include "b200_plan.cuh"

#include <cmath>
#include <cstdlib>
#include <vector>

namespace b200 {
constexpr int kJitMaxFieldsHost = 8;  // kJitMaxFields of b200_jit_kernel.cuh
bool op_table_f64_mass(int, int, OpInstance *);
bool op_table_f64_poisson(int, int, OpInstance *);
bool op_table_f64_vecmass(int, int, OpInstance *);
bool op_table_f64_vecpoisson(int, int, OpInstance *);
bool op_table_f64_kappa(int, int, OpInstance *);
bool op_table_f32_mass(int, int, OpInstance *);
bool op_table_f32_poisson(int, int, OpInstance *);
bool op_table_f32_vecmass(int, int, OpInstance *);
bool op_table_f32_vecpoisson(int, int, OpInstance *);
bool op_table_f32_kappa(int, int, OpInstance *);
bool op_table_f64x_mass(int, int, OpInstance *);
bool op_table_f64x_poisson(int, int, OpInstance *);
bool op_table_f64x_vecmass(int, int, OpInstance *);
bool op_table_f64x_vecpoisson(int, int, OpInstance *);
bool op_table_f64x_kappa(int, int, OpInstance *);
bool kgrad_table_f64(int, OpLauncher *);
bool kgrad_table_f32(int, OpLauncher *);

bool op_lookup(int prec, int qf, int P, int variant, OpInstance *out) {
  if (P < kOpPMin || P > kOpPMax) return false;
  if (prec == B200_F64) {
    switch (qf) {
      case B200_QF_MASS: return op_table_f64_mass(P, variant, out);
      case B200_QF_POISSON: return op_table_f64_poisson(P, variant, out);
      case B200_QF_VECMASS: return op_table_f64_vecmass(P, variant, out);
      case B200_QF_VECPOISSON: return op_table_f64_vecpoisson(P, variant, out);
      case B200_QF_POISSON_KAPPA: return op_table_f64_kappa(P, variant, out);
    }
  } else if (prec == B200_F32) {
    switch (qf) {
      case B200_QF_MASS: return op_table_f32_mass(P, variant, out);
      case B200_QF_POISSON: return op_table_f32_poisson(P, variant, out);
      case B200_QF_VECMASS: return op_table_f32_vecmass(P, variant, out);
      case B200_QF_VECPOISSON: return op_table_f32_vecpoisson(P, variant, out);
      case B200_QF_POISSON_KAPPA: return op_table_f32_kappa(P, variant, out);
    }
  } else if (prec == B200_F64X) {
    switch (qf) {
      case B200_QF_MASS: return op_table_f64x_mass(P, variant, out);
      case B200_QF_POISSON: return op_table_f64x_poisson(P, variant, out);
      case B200_QF_VECMASS: return op_table_f64x_vecmass(P, variant, out);
      case B200_QF_VECPOISSON: return op_table_f64x_vecpoisson(P, variant, out);
      case B200_QF_POISSON_KAPPA: return op_table_f64x_kappa(P, variant, out);
    }
  }
  return false;
}

// Element type of the vectors in HBM: B200_F64X stores double.
static int storage_prec(int prec) { return prec == B200_F32 ? B200_F32 : B200_F64; }
static size_t storage_bytes(int prec) { return prec == B200_F32 ? 4 : 8; }

// True when M (J x K, row-major) satisfies M[J-1-j][K-1-k] = par * M[j][k] to rounding.
static bool centro(const double *M, int J, int K, int par) {
  double scale = 0.0;
  for (int i = 0; i < J * K; i++) scale = fmax(scale, fabs(M[i]));
  for (int j = 0; j < J; j++)
    for (int k = 0; k < K; k++)
      if (fabs(M[(J - 1 - j) * K + (K - 1 - k)] - par * M[j * K + k]) > 1e-12 * scale) return false;
  return true;
}

bool kgrad_lookup(int prec, int P, OpLauncher *out) {
  if (P < kOpPMin || P > kOpPMax) return false;
  return prec == B200_F64 ? kgrad_table_f64(P, out) : prec == B200_F32 ? kgrad_table_f32(P, out) : false;
}

// Householder reflection A <- (I - b v v^T) A on an m x n block (row stride `row`, column stride `col`), v[0] = 1 implied.
static void householder_reflect(double *A, const double *v, double b, int m, int n, int row, int col) {
  for (int j = 0; j < n; j++) {
    double w = A[j * col];
    for (int i = 1; i < m; i++) w += v[i] * A[i * row + j * col];
    A[j * col] -= b * w;
    for (int i = 1; i < m; i++) A[i * row + j * col] -= b * w * v[i];
  }
}

// Collocated derivative G_c = G B^+ (Q x Q).  B^+ is formed as CeedBasisGetCollocatedGrad forms it
// (interface/ceed-basis.c:750-772 with CeedMatrixPseudoinverse, :1188-1300): Householder QR of B (Q x P), Q^T applied
// to the identity, back substitution with R; then G B^+ with ascending sums.  The same operations in the same order
// (host code built without multiply-add contraction), so G_c is bitwise the reference's table.  Returns false when B
// is rank deficient.
static bool collocated_grad(int P, int Q, const double *B, const double *G, double *Gc) {
  const int           m = Q, n = P;
  std::vector<double> a(B, B + (size_t)m * n), tau((size_t)m, 0.0), id((size_t)m * m, 0.0), v((size_t)m, 0.0), pinv((size_t)n * m, 0.0);
  for (int i = 0; i < n && i < m - 1; i++) {
    double sigma = 0.0;
    v[i]         = a[i + n * i];
    for (int j = i + 1; j < m; j++) {
      v[j] = a[i + n * j];
      sigma += v[j] * v[j];
    }
    const double norm = sqrt(v[i] * v[i] + sigma), r_ii = -copysign(norm, v[i]);
    if (norm == 0.0) return false;
    v[i] -= r_ii;
    tau[i] = 2 * v[i] * v[i] / (v[i] * v[i] + sigma);
    for (int j = i + 1; j < m; j++) v[j] /= v[i];
    householder_reflect(&a[(size_t)i * n + i + 1], &v[i], tau[i], m - i, n - i - 1, n, 1);
    a[i + n * i] = r_ii;
    for (int j = i + 1; j < m; j++) a[i + n * j] = v[j];
  }
  for (int i = 0; i < m; i++) id[(size_t)i * m + i] = 1.0;
  for (int i = 0; i < n; i++) {
    for (int j = i + 1; j < m; j++) v[j] = a[(size_t)j * n + i];
    householder_reflect(&id[(size_t)i * m], &v[i], tau[i], m - i, m, m, 1);
  }
  if (fabs(a[(size_t)n * n - 1]) < 1e-300) return false;
  for (int j = 0; j < m; j++) {
    pinv[j + m * (n - 1)] = id[j + m * (n - 1)] / a[(size_t)n * n - 1];
    for (int i = n - 2; i >= 0; i--) {
      pinv[j + m * i] = id[j + m * i];
      for (int k = i + 1; k < n; k++) pinv[j + m * i] -= a[k + n * i] * pinv[j + m * k];
      pinv[j + m * i] /= a[i + n * i];
    }
  }
  for (int i = 0; i < Q; i++)
    for (int j = 0; j < Q; j++) {
      double s = 0.0;
      for (int k = 0; k < P; k++) s += G[k + i * P] * pinv[j + k * Q];
      Gc[j + i * Q] = s;
    }
  return true;
}

}  // namespace b200

using namespace b200;

struct b200_op_s {
  b200_ctx            ctx;
  b200_op_desc        d;
  std::vector<double> B, Gc;  // host copies: Q x P interp, Q x Q collocated gradient
  OpInstance          inst;
  int                 stage, epb, variant;
  int                 grid;       // persistent variant: blocks
  int                 dot_grid;   // persistent FP32 kernel: blocks of its form that also sums u . (A u), else 0
  bool                symmetric;  // B centro-symmetric and G_c centro-antisymmetric: even-odd kernels apply
  b200_plan           plan;     // deterministic scatter only
  void               *e_work;   // element results for the deterministic scatter, [comp][elem][node]
  // Run-time compiled QFunction (b200_op_create_jit)
  bool                jit;
  cudaKernel_t        jit_kernel;
  int                 jit_num_passive;
  std::vector<char>   jit_mats;
};

static int op_variant_of(b200_op op, int stage, int *variant) {
  const bool eo = op->symmetric;
  if (stage == kStageReg) *variant = eo ? kVarRegEO : kVarReg;
  else if (stage == kStageSmem) *variant = eo ? kVarSmemEO : kVarSmem;
  else if (stage == kStagePipe) {
    B200_CHECK(eo && op->d.num_comp == 1, B200_ERROR_UNSUPPORTED,
               "the pipelined kernel needs one component and a centro-symmetric basis (Lagrange on Gauss-Lobatto nodes, Gauss points)");
    *variant = kVarPipeEO;
  } else if (stage == kStage3D) {
    *variant = kVar3D;
  } else if (stage == kStageTma) {
    *variant = eo ? kVarTmaEO : kVarTma;
  } else if (stage == kStageLate) {
    *variant = eo ? kVarLateEO : kVarLate;
  } else if (stage == kStagePTma) {
    B200_CHECK(op->d.prec == B200_F32 && op->d.num_comp == 1, B200_ERROR_UNSUPPORTED,
               "the persistent bulk-copy kernel is FP32 with one component");
    *variant = eo ? kVarPTmaEO : kVarPTma;
  } else {
    B200_CHECK(false, B200_ERROR_UNSUPPORTED, "unknown qdata staging %d", stage);
  }
  return B200_SUCCESS;
}

// Default launch shape per precision and QFunction, from autotuner sweeps on GB300 (n^3 boxes of ~17M DoF, atomic
// scatter, every staging and elements-per-block candidate).  Indexed by P_1d - 2; {staging, elements per block}.  The
// autotuner refines it per problem.
struct TileDefault {
  int stage, epb;
};
static const TileDefault kTileF64Grad[8]  = {{1, 32}, {4, 5}, {6, 14}, {6, 8}, {6, 7}, {6, 5}, {6, 3}, {6, 5}};
static const TileDefault kTileF64Mass[8]  = {{1, 32}, {1, 24}, {1, 24}, {1, 16}, {1, 8}, {1, 5}, {5, 3}, {1, 3}};
static const TileDefault kTileF32Grad[8]  = {{5, 28}, {1, 10}, {5, 5}, {7, 6}, {7, 5}, {7, 2}, {7, 3}, {7, 1}};
static const TileDefault kTileF32Mass[8]  = {{7, 32}, {1, 10}, {5, 10}, {7, 7}, {7, 5}, {7, 2}, {7, 3}, {5, 2}};
static const TileDefault kTileF64XGrad[8] = {{1, 14}, {1, 20}, {1, 10}, {1, 7}, {6, 8}, {6, 4}, {6, 7}, {6, 5}};
static const TileDefault kTileF64XMass[8] = {{1, 14}, {1, 16}, {1, 6}, {1, 7}, {1, 5}, {1, 6}, {5, 4}, {5, 3}};
static const TileDefault kTileVector[8]   = {{1, 14}, {1, 8}, {1, 7}, {1, 7}, {1, 2}, {1, 1}, {1, 1}, {1, 1}};
// Three-component fields at the degrees the vector sweep covers (2, 4, 6: P = 3, 5, 7), per precision and QFunction
// ({0, 0}: fall back to kTileVector).  Indexed [P = 3, 5, 7].
static const TileDefault kTileVecF64Grad[3]  = {{4, 4}, {4, 1}, {6, 3}};
static const TileDefault kTileVecF64Mass[3]  = {{1, 32}, {2, 14}, {5, 5}};
static const TileDefault kTileVecF32Grad[3]  = {{1, 10}, {5, 3}, {5, 2}};
static const TileDefault kTileVecF32Mass[3]  = {{1, 7}, {5, 7}, {5, 2}};
static const TileDefault kTileVecF64XGrad[3] = {{6, 32}, {6, 10}, {6, 4}};
static const TileDefault kTileVecF64XMass[3] = {{2, 10}, {6, 8}, {6, 7}};

static void op_default_tile(b200_op op, int *epb, int *stage) {
  const int   Q = op->d.Q_1d, P = op->d.P_1d;
  TileDefault t{kStageReg, 256 / (Q * Q) > 0 ? 256 / (Q * Q) : 1};
  if (P >= kOpPMin && P <= kOpPMax) {
    const bool mass = op->d.qf == B200_QF_MASS || op->d.qf == B200_QF_VECMASS;
    if (op->d.num_comp > 1) {
      t = kTileVector[P - 2];
      if (P == 3 || P == 5 || P == 7) {
        const int         i = (P - 3) / 2;
        const TileDefault v = op->d.prec == B200_F64    ? (mass ? kTileVecF64Mass : kTileVecF64Grad)[i]
                              : op->d.prec == B200_F64X ? (mass ? kTileVecF64XMass : kTileVecF64XGrad)[i]
                                                        : (mass ? kTileVecF32Mass : kTileVecF32Grad)[i];
        t = v;
      }
    }
    else if (op->d.prec == B200_F64) t = (mass ? kTileF64Mass : kTileF64Grad)[P - 2];
    else if (op->d.prec == B200_F64X) t = (mass ? kTileF64XMass : kTileF64XGrad)[P - 2];
    else t = (mass ? kTileF32Mass : kTileF32Grad)[P - 2];
  }
  // The pipelined kernel needs a centro-symmetric basis: without one the default falls back to register staging.
  if (t.stage == kStagePipe && !op->symmetric) t = {kStageReg, t.epb};
  if (*stage <= 0) *stage = t.stage;
  if (*epb <= 0) {
    if (*stage == t.stage) *epb = t.epb;
    else if (*stage == kStagePipe) *epb = 128 / (Q * Q) > 0 ? 128 / (Q * Q) : 1;
    else if (*stage == kStage3D) *epb = 512 / (Q * Q * Q) > 0 ? 512 / (Q * Q * Q) : 1;
    else *epb = 256 / (Q * Q) > 0 ? 256 / (Q * Q) : 1;
  }
}

// Threads per element of a staging choice: Q^2 (line mapping) or Q^3 (point mapping).
static int team_threads(const b200_op_desc &d, int stage) { return stage == kStage3D ? d.Q_1d * d.Q_1d * d.Q_1d : d.Q_1d * d.Q_1d; }

static int op_select(b200_op op, int epb, int stage) {
  op_default_tile(op, &epb, &stage);
  const int Q2 = team_threads(op->d, stage);
  int variant;
  int st = op_variant_of(op, stage, &variant);
  if (st) return st;
  OpInstance inst;
  B200_CHECK(op_lookup(op->d.prec, op->d.qf, op->d.P_1d, variant, &inst), B200_ERROR_UNSUPPORTED,
             "no compiled fused kernel for prec=%d qf=%d P=%d Q=%d variant=%d", op->d.prec, op->d.qf, op->d.P_1d, op->d.Q_1d, variant);
  const int max_epb_threads = inst.max_threads / Q2;
  int       max_epb_smem    = 1;
  while (max_epb_smem < 64 && inst.smem(max_epb_smem + 1) <= 200 * 1024) max_epb_smem++;
  if (epb > max_epb_threads) epb = max_epb_threads;
  if (epb > max_epb_smem) epb = max_epb_smem;
  B200_CHECK(epb >= 1 && inst.smem(epb) <= 227 * 1024, B200_ERROR_UNSUPPORTED, "fused kernel P=%d does not fit one element per block", op->d.P_1d);
  int grid = 0, dot_grid = 0;
  if (inst.persistent) {
    const int occ = inst.occupancy(epb);
    B200_CHECK(occ >= 1, B200_ERROR_UNSUPPORTED, "pipelined kernel P=%d with %d elements per block cannot be resident", op->d.P_1d, epb);
    grid = occ * op->ctx->num_sms;
    if (inst.dot_occupancy) dot_grid = inst.dot_occupancy(epb) * op->ctx->num_sms;
  }
  op->inst    = inst;
  op->stage   = stage;
  op->epb     = epb;
  op->variant = variant;
  op->grid    = grid;
  op->dot_grid = dot_grid;
  return B200_SUCCESS;
}

extern "C" int b200_op_create(b200_ctx ctx, const b200_op_desc *desc, b200_op *out) {
  const b200_op_desc &d = *desc;
  B200_CHECK(d.prec == B200_F64 || d.prec == B200_F32 || d.prec == B200_F64X, B200_ERROR_UNSUPPORTED, "unknown precision %d", d.prec);
  B200_CHECK(d.Q_1d == d.P_1d + 1, B200_ERROR_UNSUPPORTED, "fused kernels are compiled for Q_1d = P_1d + 1 (got P=%d, Q=%d)", d.P_1d, d.Q_1d);
  B200_CHECK(d.P_1d >= kOpPMin && d.P_1d <= kOpPMax, B200_ERROR_UNSUPPORTED, "fused kernels cover P_1d in %d..%d (got %d)", kOpPMin, kOpPMax, d.P_1d);
  const int nc_expected = (d.qf == B200_QF_VECMASS || d.qf == B200_QF_VECPOISSON) ? 3 : 1;
  B200_CHECK(d.num_comp == nc_expected, B200_ERROR_DIMENSION, "QFunction %d needs %d components (got %d)", d.qf, nc_expected, d.num_comp);
  B200_CHECK((d.offsets || d.num_elem == 0) && d.interp_1d && d.grad_1d, B200_ERROR_INCOMPLETE, "b200_op_create: offsets and 1D matrices are required");
  B200_CHECK(d.scatter == B200_SCATTER_ATOMIC || d.scatter == B200_SCATTER_DETERMINISTIC, B200_ERROR_UNSUPPORTED, "unknown scatter mode %d",
             d.scatter);
  B200_CHECK(d.num_elem >= 0 && d.num_elem <= (int64_t)INT32_MAX * 64, B200_ERROR_DIMENSION, "num_elem %lld out of range", (long long)d.num_elem);
  b200_op op = new b200_op_s();
  op->ctx    = ctx;
  op->d      = d;
  op->plan   = nullptr;
  op->e_work = nullptr;
  const int P = d.P_1d, Q = d.Q_1d;
  op->B.assign(d.interp_1d, d.interp_1d + Q * P);
  op->Gc.assign((size_t)Q * Q, 0.0);
  if (!collocated_grad(P, Q, d.interp_1d, d.grad_1d, op->Gc.data())) {
    delete op;
    set_error("collocated gradient: interpolation matrix is rank deficient");
    return B200_ERROR_BACKEND;
  }
  op->symmetric = centro(op->B.data(), Q, P, 1) && centro(op->Gc.data(), Q, Q, -1) && !getenv("CEED_B200_NO_EVEN_ODD");
  if (d.prec == B200_F64X && !op->symmetric) {
    delete op;
    set_error("float-float kernels need a centro-symmetric basis (Lagrange on Gauss-Lobatto nodes, Gauss points)");
    return B200_ERROR_UNSUPPORTED;
  }
  int st = op_select(op, d.elems_per_block, d.staging);
  if (!st && d.scatter == B200_SCATTER_DETERMINISTIC && d.num_elem > 0) {
    st = b200_plan_create(ctx, d.num_elem, P * P * P, d.num_comp, d.comp_stride, d.l_size, nullptr, d.offsets, &op->plan);
    const size_t esz = storage_bytes(d.prec) * (size_t)d.num_elem * P * P * P * d.num_comp;
    if (!st) st = cuda_status(cudaMalloc(&op->e_work, esz), "cudaMalloc(e_work)", __FILE__, __LINE__);
  }
  if (st) {
    b200_op_destroy(op);
    return st;
  }
  *out = op;
  return B200_SUCCESS;
}

extern "C" int b200_op_set_tile(b200_op op, int elems_per_block, int staging) { return op_select(op, elems_per_block, staging); }

extern "C" int b200_op_get_tile(b200_op op, int *elems_per_block, int *threads_per_block, int *staging) {
  if (elems_per_block) *elems_per_block = op->epb;
  if (threads_per_block) *threads_per_block = op->epb * team_threads(op->d, op->stage);
  if (staging) *staging = op->stage;
  return B200_SUCCESS;
}

static int op_apply_impl(b200_op op, const void *u, void *v, const void *qdata, const void *kappa, int add, double *dot) {
  b200_ctx            ctx = op->ctx;
  const b200_op_desc &d   = op->d;
  B200_CHECK(!op->jit, B200_ERROR_INCOMPATIBLE, "operator has a run-time compiled QFunction: use b200_op_apply_jit");
  B200_CHECK(v || d.l_size == 0, B200_ERROR_INCOMPLETE, "b200_op_apply: v is required");
  const size_t tsz = storage_bytes(d.prec);
  if (d.num_elem == 0) {  // no elements: Apply zeroes v, ApplyAdd leaves it
    if (!add && d.l_size > 0) B200_CUDA(cudaMemsetAsync(v, 0, tsz * (size_t)d.l_size, ctx->stream));
    return B200_SUCCESS;
  }
  B200_CHECK(u && qdata, B200_ERROR_INCOMPLETE, "b200_op_apply: u and qdata are required");
  B200_CHECK(d.qf != B200_QF_POISSON_KAPPA || kappa, B200_ERROR_INCOMPLETE, "kappa-weighted diffusion needs kappa");
  OpLaunch r{};
  r.num_elem    = d.num_elem;
  r.comp_stride = d.comp_stride;
  r.epb         = op->epb;
  r.grid        = dot ? op->dot_grid : op->grid;
  r.det         = d.scatter == B200_SCATTER_DETERMINISTIC;
  r.offsets     = d.offsets;
  r.u           = u;
  r.qdata       = qdata;
  r.kappa       = kappa;
  r.v           = v;
  r.e_out       = op->e_work;
  r.B           = op->B.data();
  r.G           = op->Gc.data();
  r.status      = ctx->d_status;
  r.dot         = dot;
  if (!r.det && !add) B200_CUDA(cudaMemsetAsync(v, 0, tsz * (size_t)d.l_size, ctx->stream));
  int st = op->inst.launch(ctx, r);
  if (st) return st;
  if (r.det) st = plan_scatter(op->plan, storage_prec(d.prec), op->e_work, v, add);
  return st;
}

extern "C" int b200_op_apply(b200_op op, const void *u, void *v, const void *qdata, const void *kappa, int add) {
  return op_apply_impl(op, u, v, qdata, kappa, add, nullptr);
}

namespace b200 {
int op_dot_blocks(b200_op op, size_t *doubles) {
  const b200_op_desc &d = op->d;
  const bool ok = !op->jit && op->stage == kStagePTma && op->dot_grid > 0 && d.scatter != B200_SCATTER_DETERMINISTIC && d.num_elem > 0 &&
                  d.qf != B200_QF_POISSON_KAPPA;
  if (doubles) *doubles = ok ? (size_t)op->dot_grid : 0;
  return ok ? op->dot_grid : 0;
}
int op_apply_dot(b200_op op, const void *u, void *v, const void *qdata, double *partial) {
  B200_CHECK(partial && op_dot_blocks(op, nullptr) > 0, B200_ERROR_UNSUPPORTED, "op_apply_dot needs a persistent FP32 operator with the atomic scatter");
  return op_apply_impl(op, u, v, qdata, nullptr, 0, partial);
}
}  // namespace b200

extern "C" int b200_op_dot_len(b200_op op, int *blocks, int64_t *doubles) {
  size_t    len = 0;
  const int nb  = op_dot_blocks(op, &len);
  if (blocks) *blocks = nb;
  if (doubles) *doubles = (int64_t)len;
  return B200_SUCCESS;
}

extern "C" int b200_op_apply_dot(b200_op op, const void *u, void *v, const void *qdata, double *partial) {
  return op_apply_dot(op, u, v, qdata, partial);
}

extern "C" int b200_op_kappa_grad(b200_op op, const void *u, const void *w, const void *qdata, void *g) {
  b200_ctx            ctx = op->ctx;
  const b200_op_desc &d   = op->d;
  B200_CHECK(d.qf == B200_QF_POISSON_KAPPA && d.prec != B200_F64X, B200_ERROR_INCOMPATIBLE, "kappa gradient needs the kappa-weighted diffusion operator");
  if (d.num_elem == 0) return B200_SUCCESS;
  OpLauncher launch;
  B200_CHECK(kgrad_lookup(d.prec, d.P_1d, &launch), B200_ERROR_UNSUPPORTED, "no kappa-gradient kernel for P=%d", d.P_1d);
  OpLaunch r{};
  r.num_elem    = d.num_elem;
  r.comp_stride = d.comp_stride;
  const int Q   = d.Q_1d;
  r.epb         = 256 / (Q * Q) > 0 ? 256 / (Q * Q) : 1;
  while (r.epb > 1 && (size_t)storage_bytes(d.prec) * r.epb * tile_team_stride(Q, 0) > 96 * 1024) r.epb--;
  r.offsets = d.offsets;
  r.u       = u;
  r.w       = w;
  r.qdata   = qdata;
  r.g       = g;
  r.B       = op->B.data();
  r.G       = op->Gc.data();
  r.status  = ctx->d_status;
  return launch(ctx, r);
}

extern "C" int b200_op_cost(b200_op op, double *bytes, double *flops) {
  const b200_op_desc &d  = op->d;
  const double        P  = d.P_1d, Q = d.Q_1d, ne = (double)d.num_elem, nc = d.num_comp;
  const double        ts = (double)storage_bytes(d.prec);
  const bool          grad = d.qf == B200_QF_POISSON || d.qf == B200_QF_VECPOISSON || d.qf == B200_QF_POISSON_KAPPA;
  const double        nqd  = grad ? 6.0 : 1.0;
  // Algorithmic bytes: read u, write v, read offsets, read qdata (and kappa) once each.
  if (bytes) *bytes = ts * (2.0 * (double)d.l_size) + 4.0 * ne * P * P * P + ts * ne * Q * Q * Q * (nqd + (d.qf == B200_QF_POISSON_KAPPA ? 1 : 0));
  if (flops) {
    const double interp = 2.0 * (P * P * P * Q + P * P * Q * Q + P * Q * Q * Q);  // one direction set, one way
    const double gradc  = 3.0 * 2.0 * Q * Q * Q * Q;                              // collocated derivatives, one way
    const double qf     = grad ? (15.0 + (d.qf == B200_QF_POISSON_KAPPA ? 6.0 : 0.0)) * Q * Q * Q : 1.0 * Q * Q * Q;
    const double per_c  = 2.0 * interp + (grad ? 2.0 * gradc + 2.0 * Q * Q * Q : 0.0);
    *flops              = ne * (nc * per_c + (grad ? nc * 15.0 * Q * Q * Q : nc * Q * Q * Q) + (qf - (grad ? 15.0 : 1.0) * Q * Q * Q));
  }
  return B200_SUCCESS;
}

// Tensor contraction FLOPs of one element and component block, as CeedBasisGetFlopsEstimate counts them
// (interface/ceed-basis.c:971-977): sum over directions of 2 * pre * P * post * Q.
static int64_t tensor_flops(int dim, int num_comp, int P, int Q) {
  int64_t f = 0, pre = num_comp, post = 1;
  for (int d = 0; d < dim - 1; d++) pre *= P;
  for (int d = 0; d < dim; d++) {
    f += 2 * pre * P * post * Q;
    pre /= P;
    post *= Q;
  }
  return f;
}

extern "C" int b200_flops_estimate(int qf, int P_1d, int Q_1d, int num_comp, int64_t num_elem, int64_t *flops) {
  B200_CHECK(flops && P_1d >= 1 && Q_1d >= 1 && num_comp >= 1 && num_elem >= 0, B200_ERROR_DIMENSION, "b200_flops_estimate: bad arguments");
  int64_t qf_flops = 0;
  bool    grad     = true;
  switch (qf) {
    case B200_QF_MASS: qf_flops = 1, grad = false; break;
    case B200_QF_POISSON: qf_flops = 15; break;
    case B200_QF_VECMASS: qf_flops = num_comp, grad = false; break;
    case B200_QF_VECPOISSON: qf_flops = 15 * num_comp; break;
    case B200_QF_POISSON_KAPPA: qf_flops = 21; break;
    default: B200_CHECK(false, B200_ERROR_UNSUPPORTED, "unknown QFunction %d", qf);
  }
  const int     dim  = 3;
  const int64_t Q3   = (int64_t)Q_1d * Q_1d * Q_1d, P3 = (int64_t)P_1d * P_1d * P_1d;
  const int64_t mult = grad ? 2 : 1;  // CEED_EVAL_GRAD counts twice the interpolation's tensor FLOPs
  // The transposed basis counts with both 1D sizes set to Q_1d, as the reference's estimate does (its swap assigns
  // P_1d = Q_1d and then Q_1d = P_1d).
  const int64_t per_elem = mult * tensor_flops(dim, num_comp, P_1d, Q_1d) + Q3 * qf_flops + mult * tensor_flops(dim, num_comp, Q_1d, Q_1d) +
                           P3 * num_comp;  // transposed restriction: one add per E-vector entry
  *flops = num_elem ? num_elem * per_elem : 0;
  return B200_SUCCESS;
}

extern "C" int b200_op_time(b200_op op, const void *u, void *v, const void *qdata, const void *kappa, int reps, double *ms_per_apply) {
  b200_ctx    ctx = op->ctx;
  cudaEvent_t e0, e1;
  B200_CHECK(reps > 0, B200_ERROR_DIMENSION, "reps must be positive");
  int st = b200_op_apply(op, u, v, qdata, kappa, 1);  // warm (and fail early on a bad tile)
  if (st) return st;
  B200_CUDA(cudaEventCreate(&e0));
  B200_CUDA(cudaEventCreate(&e1));
  B200_CUDA(cudaEventRecord(e0, ctx->stream));
  for (int i = 0; i < reps && !st; i++) st = b200_op_apply(op, u, v, qdata, kappa, 1);
  B200_CUDA(cudaEventRecord(e1, ctx->stream));
  B200_CUDA(cudaEventSynchronize(e1));
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms_per_apply = ms / reps;
  return st;
}

extern "C" int b200_op_tile_limits(b200_op op, int staging, int *max_elems_per_block) {
  OpInstance inst;
  const int  Q2 = team_threads(op->d, staging);
  int        variant;
  *max_elems_per_block = 0;
  if (op_variant_of(op, staging, &variant)) return B200_SUCCESS;  // staging not available for this operator: no tiles
  if (!op_lookup(op->d.prec, op->d.qf, op->d.P_1d, variant, &inst)) return B200_SUCCESS;  // no instance for this staging
  int m = inst.max_threads / Q2;
  while (m > 1 && inst.smem(m) > 200 * 1024) m--;
  *max_elems_per_block = m < 1 ? 0 : m;
  return B200_SUCCESS;
}

// Shared part of b200_op_create and b200_op_create_jit: validation of the layout fields, collocated gradient, symmetry,
// deterministic plan.
static int op_common_init(b200_ctx ctx, const b200_op_desc &d, b200_op op) {
  B200_CHECK(d.prec == B200_F64 || d.prec == B200_F32, B200_ERROR_UNSUPPORTED, "unknown precision %d", d.prec);
  B200_CHECK(d.Q_1d == d.P_1d + 1, B200_ERROR_UNSUPPORTED, "fused kernels are compiled for Q_1d = P_1d + 1 (got P=%d, Q=%d)", d.P_1d, d.Q_1d);
  B200_CHECK(d.P_1d >= kOpPMin && d.P_1d <= kOpPMax, B200_ERROR_UNSUPPORTED, "fused kernels cover P_1d in %d..%d (got %d)", kOpPMin, kOpPMax, d.P_1d);
  B200_CHECK((d.offsets || d.num_elem == 0) && d.interp_1d && d.grad_1d, B200_ERROR_INCOMPLETE, "offsets and 1D matrices are required");
  B200_CHECK(d.scatter == B200_SCATTER_ATOMIC || d.scatter == B200_SCATTER_DETERMINISTIC, B200_ERROR_UNSUPPORTED, "unknown scatter mode %d",
             d.scatter);
  op->ctx    = ctx;
  op->d      = d;
  op->plan   = nullptr;
  op->e_work = nullptr;
  const int P = d.P_1d, Q = d.Q_1d;
  op->B.assign(d.interp_1d, d.interp_1d + Q * P);
  op->Gc.assign((size_t)Q * Q, 0.0);
  B200_CHECK(collocated_grad(P, Q, d.interp_1d, d.grad_1d, op->Gc.data()), B200_ERROR_BACKEND, "collocated gradient: interpolation matrix is rank deficient");
  op->symmetric = centro(op->B.data(), Q, P, 1) && centro(op->Gc.data(), Q, Q, -1) && !getenv("CEED_B200_NO_EVEN_ODD");
  if (d.scatter == B200_SCATTER_DETERMINISTIC && d.num_elem > 0) {
    int st = b200_plan_create(ctx, d.num_elem, P * P * P, d.num_comp, d.comp_stride, d.l_size, nullptr, d.offsets, &op->plan);
    if (st) return st;
    const size_t esz = storage_bytes(d.prec) * (size_t)d.num_elem * P * P * P * d.num_comp;
    B200_CUDA(cudaMalloc(&op->e_work, esz));
  }
  return B200_SUCCESS;
}

extern "C" int b200_op_create_jit(b200_ctx ctx, const b200_op_desc *desc, const b200_jit_qfunction *qf, b200_op *out) {
  B200_CHECK(desc && qf && qf->source_path && qf->name, B200_ERROR_INCOMPLETE, "b200_op_create_jit: missing descriptor");
  B200_CHECK(desc->num_comp == 1, B200_ERROR_UNSUPPORTED, "run-time compiled QFunctions: one-component active field only");
  B200_CHECK(qf->num_inputs >= 1 && qf->num_inputs <= 8 && qf->active_input >= 0 && qf->active_input < qf->num_inputs, B200_ERROR_DIMENSION,
             "QFunction inputs: %d with active input %d", qf->num_inputs, qf->active_input);
  B200_CHECK((qf->eval_in == B200_EVAL_INTERP || qf->eval_in == B200_EVAL_GRAD) && (qf->eval_out == B200_EVAL_INTERP || qf->eval_out == B200_EVAL_GRAD),
             B200_ERROR_UNSUPPORTED, "active fields must use CEED_EVAL_INTERP or CEED_EVAL_GRAD");
  B200_CHECK(qf->input_size[qf->active_input] == (qf->eval_in == B200_EVAL_GRAD ? 3 : 1), B200_ERROR_DIMENSION,
             "active input size %d does not match its eval mode", qf->input_size[qf->active_input]);
  b200_op op = new b200_op_s();
  int     st = op_common_init(ctx, *desc, op);
  if (!st) {
    JitRequest r;
    r.source_path  = qf->source_path;
    r.qf_name      = qf->name;
    r.prec         = desc->prec;
    r.P            = desc->P_1d;
    r.eval_in      = qf->eval_in;
    r.eval_out     = qf->eval_out;
    r.eo           = op->symmetric;
    r.num_inputs   = qf->num_inputs;
    r.active_input = qf->active_input;
    for (int i = 0; i < 8; i++) r.input_size[i] = i < qf->num_inputs ? qf->input_size[i] : 0;
    if (qf->include_dirs) {
      std::string dirs(qf->include_dirs);
      size_t      pos = 0;
      while (pos <= dirs.size()) {
        const size_t next = dirs.find(':', pos);
        const auto   item = dirs.substr(pos, next == std::string::npos ? std::string::npos : next - pos);
        if (!item.empty()) r.include_dirs.push_back(item);
        if (next == std::string::npos) break;
        pos = next + 1;
      }
    }
    std::string key;
    st = jit_compile(r, &op->jit_kernel, &key);
    if (!st) st = jit_mats_blob(desc->prec, desc->P_1d, op->B.data(), op->Gc.data(), &op->jit_mats);
  }
  if (st) {
    b200_op_destroy(op);
    return st;
  }
  op->jit             = true;
  op->jit_num_passive = qf->num_inputs - 1;
  const int Q         = desc->Q_1d;
  op->epb             = desc->elems_per_block > 0 ? desc->elems_per_block : (256 / (Q * Q) > 0 ? 256 / (Q * Q) : 1);
  op->stage           = 0;
  op->variant         = -1;
  op->grid            = 0;
  op->dot_grid        = 0;
  *out                = op;
  return B200_SUCCESS;
}

extern "C" int b200_op_apply_jit(b200_op op, const void *u, void *v, const void *const *passive, void *qf_ctx, int add) {
  b200_ctx            ctx = op->ctx;
  const b200_op_desc &d   = op->d;
  B200_CHECK(op->jit, B200_ERROR_INCOMPATIBLE, "operator has a compiled pointwise kernel: use b200_op_apply");
  B200_CHECK(u && v, B200_ERROR_INCOMPLETE, "b200_op_apply_jit: u and v are required");
  const size_t tsz = storage_bytes(d.prec);
  if (!add && d.scatter == B200_SCATTER_ATOMIC) B200_CUDA(cudaMemsetAsync(v, 0, tsz * (size_t)d.l_size, ctx->stream));
  if (d.num_elem == 0) return B200_SUCCESS;
  // Kernel arguments: OpArgs<T>, JitFields<T>, OpMats<T, P, Q> (bytes prepared at create).
  struct ArgsBlob {
    int64_t        num_elem, comp_stride;
    int            epb, det;
    const int32_t *offsets;
    const void    *u;
    void          *v, *e_out;
    const void    *qdata, *kappa;
    int           *status;
    double        *dot;
  } a{d.num_elem, d.comp_stride, op->epb, d.scatter == B200_SCATTER_DETERMINISTIC, d.offsets, u, v, op->e_work, nullptr, nullptr, ctx->d_status,
      nullptr};
  static_assert(sizeof(ArgsBlob) == sizeof(OpArgs<double>), "argument layout");
  struct FieldsBlob {
    const void *passive[kJitMaxFieldsHost];
    void       *ctx;
  } f{};
  for (int i = 0; i < op->jit_num_passive && i < kJitMaxFieldsHost; i++) f.passive[i] = passive ? passive[i] : nullptr;
  f.ctx                 = qf_ctx;
  void        *params[] = {&a, &f, op->jit_mats.data()};
  const int    Q        = d.Q_1d;
  const size_t smem     = tsz * (size_t)op->epb * tile_team_stride(Q, 0);
  if (smem > 48 * 1024) B200_CUDA(cudaFuncSetAttribute((const void *)op->jit_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t grid = ceil_div(d.num_elem, op->epb);
  B200_CUDA(cudaLaunchKernel((const void *)op->jit_kernel, dim3((unsigned)grid), dim3(op->epb * Q * Q), params, smem, ctx->stream));
  B200_LAUNCHED(ctx, "op_apply_jit");
  if (d.scatter == B200_SCATTER_DETERMINISTIC) return plan_scatter(op->plan, storage_prec(d.prec), op->e_work, v, add);
  return B200_SUCCESS;
}

extern "C" int b200_op_destroy(b200_op op) {
  if (!op) return B200_SUCCESS;
  if (op->plan) b200_plan_destroy(op->plan);
  if (op->e_work) cudaFree(op->e_work);
  delete op;
  return B200_SUCCESS;
}
