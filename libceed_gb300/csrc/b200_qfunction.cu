// Gallery QFunctions on Q-vectors (the unfused path, CeedQFunctionApply) and the geometric-factor setup
// (Mass3DBuild / Poisson3DBuild through a trilinear coordinate field).
//
// Point kernels follow include/ceed/jit-source/gallery/ceed-massapply.h, ceed-poisson3dapply.h,
// ceed-vectormassapply.h, ceed-vectorpoisson3dapply.h, ceed-mass3dbuild.h and ceed-poisson3dbuild.h.  Q-vectors hold
// field component k of point i at k * num_points + i (the layout libCEED's QFunction interface uses,
// include/ceed/ceed.h:363-377).
#include "b200_internal.cuh"
#include "b200_pointwise.cuh"

namespace b200 {

template <typename T, int QF>
__global__ void k_qf_apply(int64_t n, const T *__restrict__ in0, const T *__restrict__ in1, const T *__restrict__ in2, T *__restrict__ out0) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if (QF == B200_QF_MASS) {
      out0[i] = in0[i] * in1[i];
    } else if (QF == B200_QF_VECMASS) {
      const T q = in1[i];
      for (int c = 0; c < 3; c++) out0[c * n + i] = in0[c * n + i] * q;
    } else {
      T D[6];
      for (int k = 0; k < 6; k++) D[k] = in1[k * n + i];
      if (QF == B200_QF_POISSON_KAPPA) {
        const T kap = in2[i];
        for (int k = 0; k < 6; k++) D[k] *= kap;
      }
      const int nc = QF == B200_QF_VECPOISSON ? 3 : 1;
      for (int c = 0; c < nc; c++) {
        T vg[3];
        poisson_point(D, in0[(0 * nc + c) * n + i], in0[(1 * nc + c) * n + i], in0[(2 * nc + c) * n + i], vg);
        for (int d = 0; d < 3; d++) out0[(d * nc + c) * n + i] = vg[d];
      }
    }
  }
}

// One thread per quadrature point; 8 vertex coordinates per element through the trilinear basis (P = 2).
// x_interp / x_grad are the Q x 2 1D matrices of the coordinate basis.
__global__ void k_qdata_build(int poisson, int64_t num_elem, int Q, const double *__restrict__ x_interp, const double *__restrict__ x_grad,
                              const double *__restrict__ q_weight, const int32_t *__restrict__ x_offsets, int64_t x_comp_stride,
                              const double *__restrict__ coords, double *__restrict__ qdata) {
  const int     Q3 = Q * Q * Q;
  const int64_t n  = num_elem * Q3;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e  = i / Q3;
    const int     q  = (int)(i % Q3);
    const int     qx = q % Q, qy = (q / Q) % Q, qz = q / (Q * Q);
    double        X[3][8];
    for (int v = 0; v < 8; v++) {
      const int64_t o = x_offsets[e * 8 + v];
      for (int c = 0; c < 3; c++) X[c][v] = coords[o + c * x_comp_stride];
    }
    // J[d][c] = d x_c / d xi_d (the GRAD Q-vector layout [dim][comp]).
    double J[3][3];
    for (int d = 0; d < 3; d++) {
      const double *Mx = d == 0 ? x_grad : x_interp, *My = d == 1 ? x_grad : x_interp, *Mz = d == 2 ? x_grad : x_interp;
      for (int c = 0; c < 3; c++) {
        double s = 0.0;
        for (int vz = 0; vz < 2; vz++)
          for (int vy = 0; vy < 2; vy++)
            for (int vx = 0; vx < 2; vx++) s += Mz[qz * 2 + vz] * My[qy * 2 + vy] * Mx[qx * 2 + vx] * X[c][vx + 2 * (vy + 2 * vz)];
        J[d][c] = s;
      }
    }
    const double w = q_weight[qz] * (q_weight[qy] * (q_weight[qx] * 1.0));
    if (poisson) {
      double qd[6];
      poisson3d_build_point(J, w, qd);
      for (int k = 0; k < 6; k++) qdata[(k * num_elem + e) * Q3 + q] = qd[k];
    } else {
      qdata[e * Q3 + q] = mass3d_build_point(J, w);
    }
  }
}

}  // namespace b200

using namespace b200;

extern "C" int b200_qf_apply(b200_ctx ctx, int prec, int qf_kind, int64_t num_points, const void *const *in, void *const *out) {
  if (num_points <= 0) return B200_SUCCESS;
  const int g = stride_grid(ctx, num_points, 256);
#define QF_CASE(T, K)                                                                                                              \
  case K:                                                                                                                          \
    k_qf_apply<T, K><<<g, 256, 0, ctx->stream>>>(num_points, (const T *)in[0], (const T *)in[1],                                 \
                                                 K == B200_QF_POISSON_KAPPA ? (const T *)in[2] : nullptr, (T *)out[0]);           \
    break;
  if (prec == B200_F64) {
    switch (qf_kind) {
      QF_CASE(double, B200_QF_MASS)
      QF_CASE(double, B200_QF_POISSON)
      QF_CASE(double, B200_QF_VECMASS)
      QF_CASE(double, B200_QF_VECPOISSON)
      QF_CASE(double, B200_QF_POISSON_KAPPA)
      default: B200_CHECK(false, B200_ERROR_UNSUPPORTED, "unknown QFunction kind %d", qf_kind);
    }
  } else if (prec == B200_F32) {
    switch (qf_kind) {
      QF_CASE(float, B200_QF_MASS)
      QF_CASE(float, B200_QF_POISSON)
      QF_CASE(float, B200_QF_VECMASS)
      QF_CASE(float, B200_QF_VECPOISSON)
      QF_CASE(float, B200_QF_POISSON_KAPPA)
      default: B200_CHECK(false, B200_ERROR_UNSUPPORTED, "unknown QFunction kind %d", qf_kind);
    }
  } else {
    B200_CHECK(false, B200_ERROR_UNSUPPORTED, "unknown precision %d", prec);
  }
#undef QF_CASE
  B200_LAUNCHED(ctx, "qf_apply");
  return B200_SUCCESS;
}

extern "C" int b200_qdata_build(b200_ctx ctx, int poisson, int64_t num_elem, int Q_1d, const double *x_interp_1d, const double *x_grad_1d,
                                const double *q_weight_1d, const int32_t *x_offsets, int64_t x_comp_stride, const double *coords, double *qdata) {
  B200_CHECK(Q_1d >= 1 && Q_1d <= 16, B200_ERROR_UNSUPPORTED, "Q_1d = %d not in 1..16", Q_1d);
  if (num_elem <= 0) return B200_SUCCESS;
  // The 1D tables are tiny: stage them in device memory owned by this call's stream order.
  double *mats = nullptr;
  const size_t nb = sizeof(double) * (size_t)(5 * Q_1d);
  B200_CUDA(cudaMallocAsync((void **)&mats, nb, ctx->stream));
  double host[5 * 16];
  for (int i = 0; i < 2 * Q_1d; i++) host[i] = x_interp_1d[i], host[2 * Q_1d + i] = x_grad_1d[i];
  for (int i = 0; i < Q_1d; i++) host[4 * Q_1d + i] = q_weight_1d[i];
  B200_CUDA(cudaMemcpyAsync(mats, host, nb, cudaMemcpyHostToDevice, ctx->stream));
  const int64_t n = num_elem * Q_1d * Q_1d * Q_1d;
  k_qdata_build<<<stride_grid(ctx, n, 128), 128, 0, ctx->stream>>>(poisson, num_elem, Q_1d, mats, mats + 2 * Q_1d, mats + 4 * Q_1d, x_offsets,
                                                                   x_comp_stride, coords, qdata);
  B200_LAUNCHED(ctx, "qdata_build");
  B200_CUDA(cudaStreamSynchronize(ctx->stream));
  B200_CUDA(cudaFreeAsync(mats, ctx->stream));
  return B200_SUCCESS;
}
