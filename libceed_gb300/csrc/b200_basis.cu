// Standalone tensor-product H1 basis (CeedBasisApply / ApplyAdd for INTERP, GRAD and WEIGHT, dim 1..3).
//
// Takes over the Interp / Grad / Weight kernels of include/ceed/jit-source/cuda/cuda-ref-basis-tensor.h.  One block
// per element; each 1D contraction is a pass through shared memory.  Gradients use dim^2 contractions (the derivative
// matrix in one direction, interpolation in the others), which is exact for any P and Q.  This entry point serves the
// unfused path and the reference's standalone basis tests; the fused operator has its own kernels.
#include "b200_internal.cuh"

#include <vector>

struct b200_basis_s {
  b200_ctx ctx;
  int      dim, P, Q, num_comp;
  double  *mats_f64;  // device: interp (Q*P) | grad (Q*P) | qweight (Q)
  float   *mats_f32;
};

namespace b200 {

constexpr int kBasisMax = 16;  // P, Q <= 16
constexpr int kBasisThreads = 256;

// v[pre][j][post] = sum_b M(j, b) u[pre][b][post], M(j,b) = mat[j*B + b] or mat[b*J + j] (transpose).
template <typename T>
__device__ void contract(int pre, int B, int post, int J, const T *mat, bool transpose, const T *u, T *v) {
  const int n = pre * J * post;
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const int c = k % post, j = (k / post) % J, a = k / (post * J);
    T         s = 0;
    for (int b = 0; b < B; b++) s += (transpose ? mat[b * J + j] : mat[j * B + b]) * u[(a * B + b) * post + c];
    v[k] = s;
  }
  __syncthreads();
}

template <typename T>
__global__ void __launch_bounds__(kBasisThreads) k_basis(int dim, int P, int Q, int num_comp, int64_t num_elem, int t_mode, int eval_mode, int add,
                                                         int big, const T *__restrict__ mats, const T *__restrict__ u, T *__restrict__ v) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T        *s_mat = reinterpret_cast<T *>(smem_raw);  // interp | grad | qweight, then three work buffers of `big`
  T        *buf0 = s_mat + 2 * Q * P + Q, *buf1 = buf0 + big, *buf2 = buf1 + big;
  for (int i = threadIdx.x; i < 2 * Q * P + Q; i += blockDim.x) s_mat[i] = mats[i];
  __syncthreads();
  const T *B = s_mat, *G = s_mat + Q * P, *W = s_mat + 2 * Q * P;
  int      nn = 1, nq = 1;
  for (int d = 0; d < dim; d++) nn *= P, nq *= Q;
  const bool tr = t_mode == B200_TRANSPOSE;

  for (int64_t e = blockIdx.x; e < num_elem; e += gridDim.x) {
    if (eval_mode == B200_EVAL_WEIGHT) {
      for (int k = threadIdx.x; k < nq; k += blockDim.x) {
        T   w = 1;
        int r = k;
        for (int d = 0; d < dim; d++) {
          w = W[r % Q] * w;
          r /= Q;
        }
        v[e * nq + k] = w;
      }
      continue;
    }
    const int qc = eval_mode == B200_EVAL_GRAD ? dim : 1;
    for (int comp = 0; comp < num_comp; comp++) {
      if (!tr) {
        // E [comp][elem][node] -> Q [d][comp][elem][qpt]
        for (int p = 0; p < qc; p++) {
          const T *in = u + ((int64_t)comp * num_elem + e) * nn;
          for (int k = threadIdx.x; k < nn; k += blockDim.x) buf0[k] = in[k];
          __syncthreads();
          int pre = nn, post = 1;
          T  *src = buf0;
          for (int d = 0; d < dim; d++) {
            pre /= P;
            const T *M   = (eval_mode == B200_EVAL_GRAD && d == p) ? G : B;
            T       *dst = src == buf0 ? buf1 : buf0;
            contract(pre, P, post, Q, M, false, src, dst);
            post *= Q;
            src = dst;
          }
          T *out = v + (((int64_t)p * num_comp + comp) * num_elem + e) * nq;
          for (int k = threadIdx.x; k < nq; k += blockDim.x) out[k] = src[k];
          __syncthreads();
        }
      } else {
        // Q [d][comp][elem][qpt] -> E [comp][elem][node], summed over d
        for (int k = threadIdx.x; k < nn; k += blockDim.x) buf2[k] = 0;
        for (int p = 0; p < qc; p++) {
          const T *in = u + (((int64_t)p * num_comp + comp) * num_elem + e) * nq;
          for (int k = threadIdx.x; k < nq; k += blockDim.x) buf0[k] = in[k];
          __syncthreads();
          int pre = nq, post = 1;
          T  *src = buf0, *dst = buf1;
          for (int d = 0; d < dim; d++) {
            pre /= Q;
            const T *M = (eval_mode == B200_EVAL_GRAD && d == p) ? G : B;
            contract(pre, Q, post, P, M, true, src, dst);
            post *= P;
            T *t = src;
            src  = dst;
            dst  = t;
          }
          for (int k = threadIdx.x; k < nn; k += blockDim.x) buf2[k] += src[k];
          __syncthreads();
        }
        T *out = v + ((int64_t)comp * num_elem + e) * nn;
        for (int k = threadIdx.x; k < nn; k += blockDim.x) out[k] = add ? out[k] + buf2[k] : buf2[k];
        __syncthreads();
      }
    }
  }
}

}  // namespace b200

using namespace b200;

extern "C" int b200_basis_create(b200_ctx ctx, int dim, int P_1d, int Q_1d, int num_comp, const double *interp_1d, const double *grad_1d,
                                 const double *q_weight_1d, b200_basis *out) {
  B200_CHECK(dim >= 1 && dim <= 3, B200_ERROR_DIMENSION, "tensor basis dimension %d not in 1..3", dim);
  B200_CHECK(P_1d >= 1 && P_1d <= kBasisMax && Q_1d >= 1 && Q_1d <= kBasisMax, B200_ERROR_UNSUPPORTED, "P_1d=%d, Q_1d=%d: at most %d supported",
             P_1d, Q_1d, kBasisMax);
  B200_CHECK(num_comp >= 1, B200_ERROR_DIMENSION, "num_comp %d < 1", num_comp);
  const int           n = 2 * Q_1d * P_1d + Q_1d;
  std::vector<double> h(n, 0.0);
  for (int i = 0; i < Q_1d * P_1d; i++) {
    h[i]                   = interp_1d ? interp_1d[i] : 0.0;
    h[Q_1d * P_1d + i]     = grad_1d ? grad_1d[i] : 0.0;
  }
  for (int i = 0; i < Q_1d; i++) h[2 * Q_1d * P_1d + i] = q_weight_1d ? q_weight_1d[i] : 0.0;
  std::vector<float> hf(h.begin(), h.end());
  b200_basis         b = new b200_basis_s();
  b->ctx = ctx, b->dim = dim, b->P = P_1d, b->Q = Q_1d, b->num_comp = num_comp;
  cudaError_t err = cudaMalloc(&b->mats_f64, sizeof(double) * n);  // b is value-initialised: a partial basis frees cleanly
  if (err == cudaSuccess) err = cudaMalloc(&b->mats_f32, sizeof(float) * n);
  if (err == cudaSuccess) err = cudaMemcpy(b->mats_f64, h.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMemcpy(b->mats_f32, hf.data(), sizeof(float) * n, cudaMemcpyHostToDevice);
  if (err != cudaSuccess) {
    b200_basis_destroy(b);
    return cuda_status(err, "b200_basis_create", __FILE__, __LINE__);
  }
  *out = b;
  return B200_SUCCESS;
}

extern "C" int b200_basis_apply(b200_basis b, int prec, int64_t num_elem, int t_mode, int eval_mode, int add, const void *u, void *v) {
  b200_ctx ctx = b->ctx;
  B200_CHECK(eval_mode == B200_EVAL_INTERP || eval_mode == B200_EVAL_GRAD || eval_mode == B200_EVAL_WEIGHT, B200_ERROR_UNSUPPORTED,
             "eval mode %d not supported by the tensor H1 basis", eval_mode);
  B200_CHECK(!(eval_mode == B200_EVAL_WEIGHT && t_mode == B200_TRANSPOSE), B200_ERROR_BACKEND, "CEED_EVAL_WEIGHT incompatible with CEED_TRANSPOSE");
  B200_CHECK(!(add && t_mode != B200_TRANSPOSE), B200_ERROR_UNSUPPORTED, "CeedBasisApplyAdd only supports CEED_TRANSPOSE");
  B200_CHECK(eval_mode == B200_EVAL_WEIGHT || u, B200_ERROR_BACKEND, "An input vector is required for this CeedEvalMode");
  if (num_elem <= 0) return B200_SUCCESS;
  const int mx = b->P > b->Q ? b->P : b->Q;
  int       big = 1;
  for (int d = 0; d < b->dim; d++) big *= mx;
  const int grid = (int)(num_elem < (int64_t)ctx->num_sms * 16 ? num_elem : (int64_t)ctx->num_sms * 16);
  if (prec == B200_F64) {
    const size_t smem = sizeof(double) * (2 * b->Q * b->P + b->Q + 3 * big);
    B200_CUDA(cudaFuncSetAttribute(k_basis<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_basis<double><<<grid, kBasisThreads, smem, ctx->stream>>>(b->dim, b->P, b->Q, b->num_comp, num_elem, t_mode, eval_mode, add, big, b->mats_f64,
                                                                (const double *)u, (double *)v);
  } else if (prec == B200_F32) {
    const size_t smem = sizeof(float) * (2 * b->Q * b->P + b->Q + 3 * big);
    B200_CUDA(cudaFuncSetAttribute(k_basis<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_basis<float><<<grid, kBasisThreads, smem, ctx->stream>>>(b->dim, b->P, b->Q, b->num_comp, num_elem, t_mode, eval_mode, add, big, b->mats_f32,
                                                               (const float *)u, (float *)v);
  } else {
    B200_CHECK(false, B200_ERROR_UNSUPPORTED, "unknown precision %d", prec);
  }
  B200_LAUNCHED(ctx, "basis_apply");
  return B200_SUCCESS;
}

extern "C" int b200_basis_destroy(b200_basis b) {
  if (!b) return B200_SUCCESS;
  cudaFree(b->mats_f64);
  cudaFree(b->mats_f32);
  delete b;
  return B200_SUCCESS;
}
