// FMA-rate probe (b200_fma_peak): the denominator of the compute roofline of the fused FP64 and FP32 kernels.
#include "b200_internal.cuh"
#include "b200_op_kernels.cuh"

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

// FP64 tensor-core probe: chains of mma.sync m8n8k4 (the only FP64 tensor-core instruction of sm_103a; tcgen05 has
// no FP64 kind), alone (mode 0) or interleaved in every warp with as many DFMA chains as the DFMA probe (mode 1), to
// tell whether the tensor path adds FP64 throughput to the FMA pipe or shares it.  No memory traffic: the result is
// stored only if it takes an impossible value.
__device__ __forceinline__ void dmma_8x8x4(double &d0, double &d1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n" : "+d"(d0), "+d"(d1) : "d"(a), "d"(b));
}

__global__ void k_dmma_peak(double *out, int iters, int mode, double a, double b) {
  double x[kPeakChains], y[kPeakChains], f[kPeakChains];
  for (int c = 0; c < kPeakChains; c++) {
    x[c] = threadIdx.x + c;
    y[c] = c;
    f[c] = threadIdx.x * 0.5 + c;
  }
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int c = 0; c < kPeakChains; c++) dmma_8x8x4(x[c], y[c], a, b);
    if (mode == 1) {
#pragma unroll
      for (int k = 0; k < 4; k++)
#pragma unroll
        for (int c = 0; c < kPeakChains; c++) f[c] = f[c] * a + b;
    }
  }
  double s = 0;
  for (int c = 0; c < kPeakChains; c++) s += x[c] + y[c] + f[c];
  if (s == -1.25) out[threadIdx.x] = s;
}

static int dmma_peak(b200_ctx ctx, int iters, double *dmma_tflops, double *mixed_tflops) {
  const int blocks = ctx->num_sms * 4, threads = 256;
  double   *out    = nullptr;
  B200_CUDA(cudaMallocAsync((void **)&out, sizeof(double) * threads, ctx->stream));
  cudaEvent_t e0, e1;
  B200_CUDA(cudaEventCreate(&e0));
  B200_CUDA(cudaEventCreate(&e1));
  const double warps = (double)blocks * threads / 32;
  for (int mode = 0; mode < 2; mode++) {
    k_dmma_peak<<<blocks, threads, 0, ctx->stream>>>(out, iters / 8 + 1, mode, 0.999, 0.001);  // warm-up
    float best = 0;
    for (int rep = 0; rep < 3; rep++) {
      B200_CUDA(cudaEventRecord(e0, ctx->stream));
      k_dmma_peak<<<blocks, threads, 0, ctx->stream>>>(out, iters, mode, 0.999, 0.001);
      B200_CUDA(cudaEventRecord(e1, ctx->stream));
      B200_CUDA(cudaEventSynchronize(e1));
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      best = (rep == 0 || ms < best) ? ms : best;
    }
    const double mma_flops = warps * iters * kPeakChains * 512.0;                        // 2 * 8 * 8 * 4 per warp MMA
    const double fma_flops = mode == 1 ? warps * 32.0 * iters * 4 * kPeakChains * 2.0 : 0.0;
    const double tflops    = (mma_flops + fma_flops) / (best * 1e-3) / 1e12;
    if (mode == 0) *dmma_tflops = tflops;
    else *mixed_tflops = tflops;
  }
  B200_LAUNCHED(ctx, "dmma_peak");
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(out, ctx->stream);
  return B200_SUCCESS;
}

// Give-up path of the bounded mbarrier wait: every thread of one block waits, with the wait of the bulk-copy kernels and
// a bound of max_polls, on a barrier whose phase nothing completes (no copy is issued and no thread arrives), then the
// first thread records the give-up in the context's status word, as the kernels do.
__global__ void k_wait_selftest(int *status, int max_polls) {
  __shared__ __align__(8) unsigned long long bar;
  if (threadIdx.x == 0) mbar_init(&bar, 1);
  __syncthreads();
  const bool done = mbar_wait(&bar, 0, max_polls);
  __syncthreads();
  if (!done && threadIdx.x == 0) atomicOr(status, B200_STATUS_COPY_TIMEOUT);
}

}  // namespace b200

using namespace b200;

extern "C" int b200_wait_selftest(b200_ctx ctx, int max_polls) {
  B200_CHECK(max_polls >= 1 && max_polls <= (1 << 16), B200_ERROR_DIMENSION, "b200_wait_selftest: max_polls must be in [1, 65536]");
  k_wait_selftest<<<1, 64, 0, ctx->stream>>>(ctx->d_status, max_polls);
  B200_LAUNCHED(ctx, "wait_selftest");
  B200_CUDA(cudaStreamSynchronize(ctx->stream));
  return B200_SUCCESS;
}

extern "C" int b200_fp64_tensor_peak(b200_ctx ctx, double *dmma_tflops, double *mixed_tflops) {
  B200_CHECK(dmma_tflops && mixed_tflops, B200_ERROR_INCOMPLETE, "b200_fp64_tensor_peak: both outputs are required");
  return dmma_peak(ctx, 1000, dmma_tflops, mixed_tflops);
}

extern "C" int b200_fma_peak(b200_ctx ctx, int prec, double *tflops) {
  B200_CHECK(tflops, B200_ERROR_INCOMPLETE, "b200_fma_peak: tflops is required");
  if (prec == B200_F64) return fma_peak<double>(ctx, 256, tflops);
  if (prec == B200_F32) return fma_peak<float>(ctx, 4096, tflops);
  B200_CHECK(false, B200_ERROR_UNSUPPORTED, "unknown precision %d", prec);
}
