// Deterministic two-pass reductions (sum of squares, |x| sum, max |x|, dot product), accumulated in FP64.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "b200_internal.cuh"

namespace b200 {

enum { kRedSumSq = 0, kRedAbsSum = 1, kRedMaxAbs = 2, kRedDot = 3 };
constexpr int kReduceThreads = 256;

// Fixed grid: two blocks per SM.  The result of a reduction depends only on n and the grid, never on timing.
inline int reduce_blocks(int num_sms) { return 2 * num_sms; }

__device__ __forceinline__ double red_combine(int kind, double a, double b) { return kind == kRedMaxAbs ? fmax(a, b) : a + b; }

// Block-wide combine in a fixed tree: warp shuffles, then the warp leaders.
__device__ __forceinline__ double block_reduce(int kind, double v) {
  __shared__ double s_warp[kReduceThreads / 32];
  for (int off = 16; off > 0; off >>= 1) v = red_combine(kind, v, __shfl_down_sync(0xffffffffu, v, off));
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) s_warp[warp] = v;
  __syncthreads();
  v = threadIdx.x < kReduceThreads / 32 ? s_warp[threadIdx.x] : 0.0;
  if (warp == 0)
    for (int off = 16; off > 0; off >>= 1) v = red_combine(kind, v, __shfl_down_sync(0xffffffffu, v, off));
  return v;
}

__device__ __forceinline__ double red_term(int kind, double acc, double xi, double yi) {
  switch (kind) {
    case kRedSumSq: return acc + xi * xi;
    case kRedAbsSum: return acc + fabs(xi);
    case kRedMaxAbs: return fmax(acc, fabs(xi));
    default: return acc + xi * yi;
  }
}

// The fixed grid leaves few threads per SM, so each thread loads 8 elements (i, i + stride, ...) before combining
// them; the combination order is the plain loop's, so the result does not depend on the unrolling.
template <typename T>
__global__ void __launch_bounds__(kReduceThreads) k_reduce_partial(int kind, int64_t n, const T *__restrict__ x, const T *__restrict__ y,
                                                                   double *__restrict__ partial) {
  constexpr int U      = 8;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t       i      = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double        acc    = 0.0;
  for (; i + (U - 1) * stride < n; i += U * stride) {
    T xv[U], yv[U];
#pragma unroll
    for (int k = 0; k < U; k++) {
      xv[k] = x[i + k * stride];
      yv[k] = kind == kRedDot ? y[i + k * stride] : T(0);
    }
#pragma unroll
    for (int k = 0; k < U; k++) acc = red_term(kind, acc, (double)xv[k], (double)yv[k]);
  }
  for (; i < n; i += stride) acc = red_term(kind, acc, (double)x[i], kind == kRedDot ? (double)y[i] : 0.0);
  acc = block_reduce(kind, acc);
  if (threadIdx.x == 0) partial[blockIdx.x] = acc;
}

static __global__ void __launch_bounds__(kReduceThreads) k_reduce_final(int kind, int blocks, const double *__restrict__ partial,
                                                                 double *__restrict__ result) {
  double acc = 0.0;
  for (int i = threadIdx.x; i < blocks; i += blockDim.x) acc = red_combine(kind, acc, partial[i]);
  acc = block_reduce(kind, acc);
  if (threadIdx.x == 0) result[0] = acc;
}

// Reduce into result_dev (device memory) on the context stream, without a host round trip.
int reduce_to_device(b200_ctx ctx, int prec, int kind, int64_t n, const void *x, const void *y, double *result_dev);

}  // namespace b200
