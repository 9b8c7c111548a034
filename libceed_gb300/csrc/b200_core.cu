// Context, device memory, vector BLAS-1 and reductions of libceed_b200.
//
// Vector kernels take over backends/cuda-ref/kernels/cuda-ref-vector.cu (setValueK, scaleValueK, axpyValueK,
// axpbyValueK, pointwiseMultValueK, rcpValueK) and the cuBLAS norm calls of
// backends/cuda-ref/ceed-cuda-ref-vector.c:487-640.  Reductions are two-pass with a fixed grid and a fixed tree, so
// a norm or dot product is bit-reproducible from run to run; FP32 vectors are reduced in FP64.
#include "b200_internal.cuh"
#include "b200_reduce.cuh"

#include <cmath>
#include <cstring>

namespace b200 {

static thread_local char g_last_error[1024] = "";

void set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof g_last_error, fmt, ap);
  va_end(ap);
}

int cuda_status(cudaError_t err, const char *what, const char *file, int line) {
  if (err == cudaSuccess) return B200_SUCCESS;
  set_error("CUDA error %s (%s) in %s at %s:%d", cudaGetErrorName(err), cudaGetErrorString(err), what, file, line);
  return B200_ERROR_BACKEND;
}

// ---------------------------------------------------------------------------------------------------------------
// Elementwise kernels (grid-stride; 64-bit indices)
// ---------------------------------------------------------------------------------------------------------------
template <typename T>
__global__ void k_set_value(int64_t n, T *__restrict__ x, T value) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) x[i] = value;
}
template <typename T>
__global__ void k_scale(int64_t n, T *__restrict__ x, T alpha) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) x[i] *= alpha;
}
template <typename T>
__global__ void k_axpy(int64_t n, T alpha, const T *__restrict__ x, T *__restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) y[i] += alpha * x[i];
}
template <typename T>
__global__ void k_axpby(int64_t n, T alpha, T beta, const T *__restrict__ x, T *__restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = alpha * x[i] + beta * y[i];
}
template <typename T>
__global__ void k_pointwise_mult(int64_t n, T *__restrict__ w, const T *__restrict__ x, const T *__restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) w[i] = x[i] * y[i];
}
template <typename T>
__global__ void k_reciprocal(int64_t n, T *__restrict__ x) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (fabs((double)x[i]) > 1e-16) x[i] = (T)1 / x[i];  // as rcpValueK: entries below CEED_EPSILON are left alone
}
// Strided forms: entry start + j * step for j < count (count already clipped to the range on the host).
template <typename T>
__global__ void k_set_value_strided(int64_t count, int64_t start, int64_t step, T *__restrict__ x, T value) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < count; j += (int64_t)gridDim.x * blockDim.x)
    x[start + j * step] = value;
}
template <typename T>
__global__ void k_copy_strided(int64_t count, int64_t start, int64_t step, const T *__restrict__ x, T *__restrict__ y) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < count; j += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = start + j * step;
    y[i]            = x[i];
  }
}
template <typename S, typename D>
__global__ void k_convert(int64_t n, const S *__restrict__ src, D *__restrict__ dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) dst[i] = (D)src[i];
}

}  // namespace b200

using namespace b200;

// ---------------------------------------------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------------------------------------------
extern "C" const char *b200_last_error(void) { return g_last_error; }

extern "C" int b200_ctx_create(int device_id, b200_ctx *out) {
  int n = 0;
  B200_CUDA(cudaGetDeviceCount(&n));
  B200_CHECK(device_id >= 0 && device_id < n, B200_ERROR_BACKEND, "device_id %d out of range (%d devices)", device_id, n);
  B200_CUDA(cudaSetDevice(device_id));
  cudaDeviceProp prop;
  B200_CUDA(cudaGetDeviceProperties(&prop, device_id));
  B200_CHECK(prop.major == 10 && prop.minor == 3, B200_ERROR_UNSUPPORTED,
             "libceed_b200 is built for sm_103a (GB300); device %d is sm_%d%d", device_id, prop.major, prop.minor);
  b200_ctx ctx = new b200_ctx_s();
  ctx->device   = device_id;
  ctx->num_sms  = prop.multiProcessorCount;
  ctx->stream   = 0;
  ctx->launches = 0;
  ctx->red_blocks = reduce_blocks(ctx->num_sms);
  cudaError_t err = cudaMalloc(&ctx->red_partial, sizeof(double) * (size_t)(2 * ctx->red_blocks + 8));  // pointers start null
  if (err == cudaSuccess) err = cudaMallocHost(&ctx->red_result_host, sizeof(double) * 8);
  if (err == cudaSuccess) err = cudaMalloc(&ctx->d_status, sizeof(int));
  if (err == cudaSuccess) err = cudaMemset(ctx->d_status, 0, sizeof(int));
  if (err != cudaSuccess) {
    b200_ctx_destroy(ctx);
    return cuda_status(err, "b200_ctx_create", __FILE__, __LINE__);
  }
  *out = ctx;
  return B200_SUCCESS;
}

extern "C" int b200_ctx_set_stream(b200_ctx ctx, void *stream) {
  ctx->stream = (cudaStream_t)stream;
  return B200_SUCCESS;
}

extern "C" int b200_ctx_get_stream(b200_ctx ctx, void **stream) {
  *stream = (void *)ctx->stream;
  return B200_SUCCESS;
}

extern "C" int b200_ctx_sync(b200_ctx ctx) {
  B200_CUDA(cudaStreamSynchronize(ctx->stream));
  return B200_SUCCESS;
}

extern "C" int b200_ctx_launch_count(b200_ctx ctx, int64_t *count) {
  *count = ctx->launches;
  return B200_SUCCESS;
}

extern "C" int b200_ctx_status(b200_ctx ctx, int *status) {
  int h = 0;
  B200_CUDA(cudaMemcpyAsync(&h, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  B200_CUDA(cudaStreamSynchronize(ctx->stream));
  B200_CUDA(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream));
  *status = h;
  return B200_SUCCESS;
}

extern "C" int b200_ctx_destroy(b200_ctx ctx) {
  if (!ctx) return B200_SUCCESS;
  cudaStreamSynchronize(ctx->stream);
  cudaFree(ctx->d_status);
  cudaFree(ctx->red_partial);
  cudaFreeHost(ctx->red_result_host);
  delete ctx;
  return B200_SUCCESS;
}

extern "C" int b200_alloc(b200_ctx ctx, size_t bytes, void **dptr) {
  (void)ctx;
  *dptr = nullptr;
  if (bytes == 0) return B200_SUCCESS;
  B200_CUDA(cudaMalloc(dptr, bytes));
  return B200_SUCCESS;
}

extern "C" int b200_free(b200_ctx ctx, void *dptr) {
  (void)ctx;
  if (dptr) B200_CUDA(cudaFree(dptr));
  return B200_SUCCESS;
}

extern "C" int b200_copy(b200_ctx ctx, void *dst, const void *src, size_t bytes, int kind) {
  cudaMemcpyKind k = kind == B200_COPY_H2D ? cudaMemcpyHostToDevice : kind == B200_COPY_D2H ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  B200_CHECK(kind >= 1 && kind <= 3, B200_ERROR_BACKEND, "b200_copy: bad copy kind %d", kind);
  if (bytes == 0) return B200_SUCCESS;
  B200_CUDA(cudaMemcpyAsync(dst, src, bytes, k, ctx->stream));
  return B200_SUCCESS;
}

#define B200_PREC_DISPATCH(prec, T, ...)                                                         \
  do {                                                                                            \
    if ((prec) == B200_F64) {                                                                     \
      using T = double;                                                                           \
      __VA_ARGS__;                                                                                       \
    } else if ((prec) == B200_F32) {                                                              \
      using T = float;                                                                            \
      __VA_ARGS__;                                                                                       \
    } else {                                                                                      \
      set_error("unknown precision %d", (int)(prec));                                             \
      return B200_ERROR_UNSUPPORTED;                                                              \
    }                                                                                             \
  } while (0)

extern "C" int b200_vec_set_value(b200_ctx ctx, int prec, int64_t n, void *x, double value) {
  if (n <= 0) return B200_SUCCESS;
  B200_PREC_DISPATCH(prec, T, {
    k_set_value<T><<<stride_grid(ctx, n, 256), 256, 0, ctx->stream>>>(n, (T *)x, (T)value);
    B200_LAUNCHED(ctx, "set_value");
  });
  return B200_SUCCESS;
}

extern "C" int b200_vec_scale(b200_ctx ctx, int prec, int64_t n, void *x, double alpha) {
  if (n <= 0) return B200_SUCCESS;
  B200_PREC_DISPATCH(prec, T, {
    k_scale<T><<<stride_grid(ctx, n, 256), 256, 0, ctx->stream>>>(n, (T *)x, (T)alpha);
    B200_LAUNCHED(ctx, "scale");
  });
  return B200_SUCCESS;
}

extern "C" int b200_vec_axpy(b200_ctx ctx, int prec, int64_t n, double alpha, const void *x, void *y) {
  if (n <= 0) return B200_SUCCESS;
  B200_PREC_DISPATCH(prec, T, {
    k_axpy<T><<<stride_grid(ctx, n, 256), 256, 0, ctx->stream>>>(n, (T)alpha, (const T *)x, (T *)y);
    B200_LAUNCHED(ctx, "axpy");
  });
  return B200_SUCCESS;
}

extern "C" int b200_vec_axpby(b200_ctx ctx, int prec, int64_t n, double alpha, double beta, const void *x, void *y) {
  if (n <= 0) return B200_SUCCESS;
  B200_PREC_DISPATCH(prec, T, {
    k_axpby<T><<<stride_grid(ctx, n, 256), 256, 0, ctx->stream>>>(n, (T)alpha, (T)beta, (const T *)x, (T *)y);
    B200_LAUNCHED(ctx, "axpby");
  });
  return B200_SUCCESS;
}

extern "C" int b200_vec_pointwise_mult(b200_ctx ctx, int prec, int64_t n, void *w, const void *x, const void *y) {
  if (n <= 0) return B200_SUCCESS;
  B200_PREC_DISPATCH(prec, T, {
    k_pointwise_mult<T><<<stride_grid(ctx, n, 256), 256, 0, ctx->stream>>>(n, (T *)w, (const T *)x, (const T *)y);
    B200_LAUNCHED(ctx, "pointwise_mult");
  });
  return B200_SUCCESS;
}

extern "C" int b200_vec_reciprocal(b200_ctx ctx, int prec, int64_t n, void *x) {
  if (n <= 0) return B200_SUCCESS;
  B200_PREC_DISPATCH(prec, T, {
    k_reciprocal<T><<<stride_grid(ctx, n, 256), 256, 0, ctx->stream>>>(n, (T *)x);
    B200_LAUNCHED(ctx, "reciprocal");
  });
  return B200_SUCCESS;
}

// Checks the range of the strided forms as CeedVectorCopyStrided / CeedVectorSetValueStrided do
// (interface/ceed-vector.c:300-325, :412-425): stop in [-1, length] with -1 meaning length, start in [0, length] and
// not past stop (CEED_ERROR_ACCESS otherwise); step must be positive (the reference's host loop never ends for
// step <= 0).  *count is the number of entries start, start + step, ... below stop.
static int strided_count(const char *who, int64_t length, int64_t start, int64_t stop, int64_t step, int64_t *count) {
  *count = 0;
  B200_CHECK(length >= 0, B200_ERROR_DIMENSION, "%s: negative length %lld", who, (long long)length);
  B200_CHECK(stop >= -1 && stop <= length, B200_ERROR_ACCESS, "%s: invalid value for stop %lld, must be in the range [-1, %lld]", who,
             (long long)stop, (long long)length);
  if (stop == -1) stop = length;
  B200_CHECK(start >= 0 && start <= stop, B200_ERROR_ACCESS, "%s: invalid value for start %lld, must be in the range [0, %lld]", who,
             (long long)start, (long long)stop);
  B200_CHECK(step > 0, B200_ERROR_ACCESS, "%s: step %lld must be positive", who, (long long)step);
  *count = ceil_div(stop - start, step);
  return B200_SUCCESS;
}

extern "C" int b200_vec_set_value_strided(b200_ctx ctx, int prec, int64_t length, int64_t start, int64_t stop, int64_t step, void *x,
                                          double value) {
  int64_t count = 0;
  int     st    = strided_count("b200_vec_set_value_strided", length, start, stop, step, &count);
  if (st) return st;
  if (count == 0) return B200_SUCCESS;
  B200_PREC_DISPATCH(prec, T, {
    k_set_value_strided<T><<<stride_grid(ctx, count, 256), 256, 0, ctx->stream>>>(count, start, step, (T *)x, (T)value);
    B200_LAUNCHED(ctx, "set_value_strided");
  });
  return B200_SUCCESS;
}

extern "C" int b200_vec_copy_strided(b200_ctx ctx, int prec, int64_t length, int64_t start, int64_t stop, int64_t step, const void *x,
                                     void *y) {
  int64_t count = 0;
  int     st    = strided_count("b200_vec_copy_strided", length, start, stop, step, &count);
  if (st) return st;
  if (count == 0) return B200_SUCCESS;
  B200_PREC_DISPATCH(prec, T, {
    k_copy_strided<T><<<stride_grid(ctx, count, 256), 256, 0, ctx->stream>>>(count, start, step, (const T *)x, (T *)y);
    B200_LAUNCHED(ctx, "copy_strided");
  });
  return B200_SUCCESS;
}

extern "C" int b200_vec_convert(b200_ctx ctx, int64_t n, int src_prec, const void *src, int dst_prec, void *dst) {
  if (n <= 0) return B200_SUCCESS;
  int g = stride_grid(ctx, n, 256);
  if (src_prec == B200_F64 && dst_prec == B200_F32) k_convert<double, float><<<g, 256, 0, ctx->stream>>>(n, (const double *)src, (float *)dst);
  else if (src_prec == B200_F32 && dst_prec == B200_F64) k_convert<float, double><<<g, 256, 0, ctx->stream>>>(n, (const float *)src, (double *)dst);
  else if (src_prec == B200_F64 && dst_prec == B200_F64) k_convert<double, double><<<g, 256, 0, ctx->stream>>>(n, (const double *)src, (double *)dst);
  else if (src_prec == B200_F32 && dst_prec == B200_F32) k_convert<float, float><<<g, 256, 0, ctx->stream>>>(n, (const float *)src, (float *)dst);
  else B200_CHECK(false, B200_ERROR_UNSUPPORTED, "b200_vec_convert: bad precisions %d -> %d", src_prec, dst_prec);
  B200_LAUNCHED(ctx, "convert");
  return B200_SUCCESS;
}

// Reductions: results land in ctx->red_partial[2*red_blocks] on the device, then in pinned host memory.
namespace b200 {
int reduce_to_device(b200_ctx ctx, int prec, int kind, int64_t n, const void *x, const void *y, double *result_dev) {
  const int blocks = ctx->red_blocks;
  if (prec == B200_F64) {
    k_reduce_partial<double><<<blocks, kReduceThreads, 0, ctx->stream>>>(kind, n, (const double *)x, (const double *)y, ctx->red_partial);
  } else if (prec == B200_F32) {
    k_reduce_partial<float><<<blocks, kReduceThreads, 0, ctx->stream>>>(kind, n, (const float *)x, (const float *)y, ctx->red_partial);
  } else {
    set_error("unknown precision %d", prec);
    return B200_ERROR_UNSUPPORTED;
  }
  B200_LAUNCHED(ctx, "reduce_partial");
  k_reduce_final<<<1, kReduceThreads, 0, ctx->stream>>>(kind, blocks, ctx->red_partial, result_dev);
  B200_LAUNCHED(ctx, "reduce_final");
  return B200_SUCCESS;
}

static int reduce_to_host(b200_ctx ctx, int prec, int kind, int64_t n, const void *x, const void *y, double *out) {
  double *res_dev = ctx->red_partial + 2 * ctx->red_blocks;
  int     st      = reduce_to_device(ctx, prec, kind, n, x, y, res_dev);
  if (st) return st;
  B200_CUDA(cudaMemcpyAsync(ctx->red_result_host, res_dev, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  B200_CUDA(cudaStreamSynchronize(ctx->stream));
  *out = ctx->red_result_host[0];
  return B200_SUCCESS;
}
}  // namespace b200

extern "C" int b200_vec_norm(b200_ctx ctx, int prec, int64_t n, const void *x, int norm_type, double *norm) {
  B200_CHECK(norm_type >= B200_NORM_1 && norm_type <= B200_NORM_MAX, B200_ERROR_UNSUPPORTED, "unknown norm type %d", norm_type);
  const int kind = norm_type == B200_NORM_1 ? kRedAbsSum : norm_type == B200_NORM_2 ? kRedSumSq : kRedMaxAbs;
  int       st   = reduce_to_host(ctx, prec, kind, n, x, nullptr, norm);
  if (!st && norm_type == B200_NORM_2) *norm = sqrt(*norm);
  return st;
}

extern "C" int b200_vec_dot(b200_ctx ctx, int prec, int64_t n, const void *x, const void *y, double *dot) {
  return reduce_to_host(ctx, prec, kRedDot, n, x, y, dot);
}
