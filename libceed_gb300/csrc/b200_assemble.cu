// Diagonal of the fused operator (CeedOperatorLinearAssembleDiagonal), for Jacobi preconditioning.
//
// Takes over the diagonal assembly of interface/ceed-preconditioning.c:2395 and its GPU kernel
// include/ceed/jit-source/cuda/cuda-ref-operator-assemble-diagonal.h.  For basis function i = (ix, iy, iz) of an
// element, the gradient at quadrature point q is (G B B, B G B, B B G)(q, i) with the 1D tables B and G, so
//   A_e[i][i] = sum_q sum_{d,d'} g_d(i,q) D_dd'(q) g_d'(i,q)
// factors into six (three for the diagonal of D, three for the symmetric off-diagonal, counted twice) separable sums
// sum_q D_dd'(q) W_x[qx][ix] W_y[qy][iy] W_z[qz][iz], with W a product of two 1D tables (G*G, G*B or B*B).  Each is
// evaluated by sum factorization (Q^3 -> P^3 in three 1D passes).  The mass operator uses W = B*B with qdata.  Element
// diagonals are added into the L-vector with atomics (or written per element for a deterministic sum).
#include "b200_internal.cuh"
#include "b200_plan.cuh"

#include <vector>

namespace b200 {

constexpr int kDiagThreads = 128;

// out[(iz, iy, ix)] (P^3) = sum_q in[q] Wx[qx][ix] Wy[qy][iy] Wz[qz][iz]; in is Q^3 in shared memory; t1, t2 scratch.
__device__ void separable_sum(int P, int Q, const double *in, const double *Wx, const double *Wy, const double *Wz, double *t1, double *t2,
                              double *out, bool add) {
  // x: t1[qz][qy][ix]
  for (int k = threadIdx.x; k < Q * Q * P; k += blockDim.x) {
    const int ix = k % P, qy = (k / P) % Q, qz = k / (P * Q);
    double    s = 0;
    for (int qx = 0; qx < Q; qx++) s += Wx[qx * P + ix] * in[(qz * Q + qy) * Q + qx];
    t1[k] = s;
  }
  __syncthreads();
  // y: t2[qz][iy][ix]
  for (int k = threadIdx.x; k < Q * P * P; k += blockDim.x) {
    const int ix = k % P, iy = (k / P) % P, qz = k / (P * P);
    double    s = 0;
    for (int qy = 0; qy < Q; qy++) s += Wy[qy * P + iy] * t1[(qz * Q + qy) * P + ix];
    t2[k] = s;
  }
  __syncthreads();
  // z: out[iz][iy][ix]
  for (int k = threadIdx.x; k < P * P * P; k += blockDim.x) {
    const int ix = k % P, iy = (k / P) % P, iz = k / (P * P);
    double    s = 0;
    for (int qz = 0; qz < Q; qz++) s += Wz[qz * P + iz] * t2[(qz * P + iy) * P + ix];
    out[k] = add ? out[k] + s : s;
  }
  __syncthreads();
}

// One block per element.  W tables in global memory: BB, GB, GG (each Q x P), products of the 1D tables.
__global__ void __launch_bounds__(kDiagThreads) k_assemble_diag(int poisson, int P, int Q, int64_t num_elem, int num_comp, int64_t comp_stride,
                                                                  const double *__restrict__ W,
                                                                  const double *__restrict__ qdata, const double *__restrict__ kappa,
                                                                  const int32_t *__restrict__ offsets, double *__restrict__ diag_l,
                                                                  double *__restrict__ diag_e) {
  extern __shared__ double sm[];
  const int Q3 = Q * Q * Q, P3 = P * P * P;
  double   *sD = sm, *t1 = sD + Q3, *t2 = t1 + Q * Q * P, *acc = t2 + Q * P * P, *sW = acc + P3;
  for (int i = threadIdx.x; i < 3 * Q * P; i += blockDim.x) sW[i] = W[i];
  const double *BB = sW, *GB = sW + Q * P, *GG = sW + 2 * Q * P;
  __syncthreads();
  for (int64_t e = blockIdx.x; e < num_elem; e += gridDim.x) {
    if (!poisson) {
      for (int q = threadIdx.x; q < Q3; q += blockDim.x) sD[q] = qdata[e * Q3 + q];
      __syncthreads();
      separable_sum(P, Q, sD, BB, BB, BB, t1, t2, acc, false);
    } else {
      // Voigt components 0..5 = xx, yy, zz, yz, xz, xy; off-diagonal ones count twice.
      const int     voigt_d[6] = {0, 1, 2, 1, 0, 0}, voigt_e[6] = {0, 1, 2, 2, 2, 1};
      for (int c = 0; c < 6; c++) {
        const double f = c < 3 ? 1.0 : 2.0;
        for (int q = threadIdx.x; q < Q3; q += blockDim.x)
          sD[q] = f * qdata[((int64_t)c * num_elem + e) * Q3 + q] * (kappa ? kappa[e * Q3 + q] : 1.0);
        __syncthreads();
        // Direction dir gets GG if both derivatives act on it, GB if one does, BB otherwise.
        const double *Wd[3];
        for (int dir = 0; dir < 3; dir++) {
          const int n = (voigt_d[c] == dir) + (voigt_e[c] == dir);
          Wd[dir]     = n == 2 ? GG : n == 1 ? GB : BB;
        }
        separable_sum(P, Q, sD, Wd[0], Wd[1], Wd[2], t1, t2, acc, c > 0);
      }
    }
    for (int i = threadIdx.x; i < P3; i += blockDim.x)
      for (int c = 0; c < num_comp; c++) {
        if (diag_e) diag_e[((int64_t)c * num_elem + e) * P3 + i] = acc[i];
        else atomicAdd(&diag_l[(int64_t)offsets[e * P3 + i] + c * comp_stride], acc[i]);
      }
    __syncthreads();
  }
}

}  // namespace b200

using namespace b200;

extern "C" int b200_assemble_diagonal(b200_ctx ctx, int poisson, int P_1d, int Q_1d, int64_t num_elem, int num_comp, int64_t comp_stride,
                                      int64_t l_size, const double *interp_1d, const double *grad_1d, const int32_t *offsets, const double *qdata,
                                      const double *kappa, double *diag, b200_plan det_plan) {
  B200_CHECK(P_1d >= 2 && P_1d <= 16 && Q_1d >= 1 && Q_1d <= 16, B200_ERROR_UNSUPPORTED, "P=%d, Q=%d not supported", P_1d, Q_1d);
  const int           P = P_1d, Q = Q_1d;
  std::vector<double> W(3 * Q * P);
  for (int i = 0; i < Q * P; i++) {
    W[i]             = interp_1d[i] * interp_1d[i];
    W[Q * P + i]     = grad_1d[i] * interp_1d[i];
    W[2 * Q * P + i] = grad_1d[i] * grad_1d[i];
  }
  double *dW = nullptr, *e_diag = nullptr;
  B200_CUDA(cudaMallocAsync((void **)&dW, sizeof(double) * W.size(), ctx->stream));
  B200_CUDA(cudaMemcpyAsync(dW, W.data(), sizeof(double) * W.size(), cudaMemcpyHostToDevice, ctx->stream));
  if (det_plan) B200_CUDA(cudaMallocAsync((void **)&e_diag, sizeof(double) * (size_t)num_elem * P * P * P * num_comp, ctx->stream));
  else B200_CUDA(cudaMemsetAsync(diag, 0, sizeof(double) * (size_t)l_size, ctx->stream));
  const size_t smem = sizeof(double) * (size_t)(Q * Q * Q + Q * Q * P + Q * P * P + P * P * P + 3 * Q * P);
  const int    grid = (int)(num_elem < (int64_t)ctx->num_sms * 16 ? num_elem : (int64_t)ctx->num_sms * 16);
  if (num_elem > 0) {
    if (smem > 48 * 1024) B200_CUDA(cudaFuncSetAttribute(k_assemble_diag, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_assemble_diag<<<grid, kDiagThreads, smem, ctx->stream>>>(poisson, P, Q, num_elem, num_comp, comp_stride, dW, qdata, kappa, offsets, diag,
                                                               e_diag);
    B200_LAUNCHED(ctx, "assemble_diag");
  }
  int st = B200_SUCCESS;
  if (det_plan && num_elem > 0) st = plan_scatter(det_plan, B200_F64, e_diag, diag, 0);
  cudaFreeAsync(dW, ctx->stream);
  if (e_diag) cudaFreeAsync(e_diag, ctx->stream);
  return st;
}
