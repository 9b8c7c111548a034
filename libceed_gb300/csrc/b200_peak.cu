// FMA-rate probe (b200_fma_peak): the denominator of the compute roofline of the fused FP64 and FP32 kernels.
#include "b200_internal.cuh"

namespace b200 {

constexpr int kPeakChains = 8, kPeakUnroll = 16;

// Eight independent chains x <- x*a + b per thread; the result is stored only if it takes an impossible value so the
// chains stay live without memory traffic.
template <typename T>
__global__ void k_fma_peak(T *out, int iters, T a, T b) {
  T x[kPeakChains];
  for (int c = 0; c < kPeakChains; c++) x[c] = (T)(threadIdx.x + c);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < kPeakUnroll; k++)
#pragma unroll
      for (int c = 0; c < kPeakChains; c++) x[c] = x[c] * a + b;
  }
  T s = 0;
  for (int c = 0; c < kPeakChains; c++) s += x[c];
  if (s == (T)-1.25) out[threadIdx.x] = s;
}

template <typename T>
static int fma_peak(b200_ctx ctx, int iters, double *tflops) {
  const int blocks = ctx->num_sms * 8, threads = 256;
  T        *out    = nullptr;
  B200_CUDA(cudaMallocAsync((void **)&out, sizeof(T) * threads, ctx->stream));
  cudaEvent_t e0, e1;
  B200_CUDA(cudaEventCreate(&e0));
  B200_CUDA(cudaEventCreate(&e1));
  k_fma_peak<T><<<blocks, threads, 0, ctx->stream>>>(out, iters / 8 + 1, (T)0.999, (T)0.001);  // warm-up
  double best = 0;
  for (int rep = 0; rep < 3; rep++) {
    B200_CUDA(cudaEventRecord(e0, ctx->stream));
    k_fma_peak<T><<<blocks, threads, 0, ctx->stream>>>(out, iters, (T)0.999, (T)0.001);
    B200_CUDA(cudaEventRecord(e1, ctx->stream));
    B200_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    const double t = 2.0 * blocks * threads * (double)iters * kPeakUnroll * kPeakChains / (ms * 1e-3) / 1e12;
    best           = t > best ? t : best;
  }
  B200_LAUNCHED(ctx, "fma_peak");
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(out, ctx->stream);
  *tflops = best;
  return B200_SUCCESS;
}

}  // namespace b200

using namespace b200;

extern "C" int b200_fma_peak(b200_ctx ctx, int prec, double *tflops) {
  B200_CHECK(tflops, B200_ERROR_INCOMPLETE, "b200_fma_peak: tflops is required");
  if (prec == B200_F64) return fma_peak<double>(ctx, 256, tflops);
  if (prec == B200_F32) return fma_peak<float>(ctx, 4096, tflops);
  B200_CHECK(false, B200_ERROR_UNSUPPORTED, "unknown precision %d", prec);
}
