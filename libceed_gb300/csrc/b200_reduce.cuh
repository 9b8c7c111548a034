// Deterministic two-pass reductions (sum of squares, |x| sum, max |x|, dot product); the per-block and final passes add
// in FP64.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "b200_dfloat.cuh"
#include "b200_internal.cuh"

namespace b200 {

enum { kRedSumSq = 0, kRedAbsSum = 1, kRedMaxAbs = 2, kRedDot = 3 };
constexpr int kReduceThreads = 256;

// Fixed grid: two blocks per SM.  The result of a reduction depends only on n and the grid, never on timing.
inline int reduce_blocks(int num_sms) { return 2 * num_sms; }

__device__ __forceinline__ double red_combine(int kind, double a, double b) { return kind == kRedMaxAbs ? fmax(a, b) : a + b; }

// Per-thread accumulators.  FP64 data: a double.  FP32 data: F2Acc (float-float on the FP32 pipe) instead of
// converting every value to double, which on this GPU puts two conversions and a multiply-add per element on the FP64
// pipe (1/60 of the FP32 rate) and bounded the FP32 CG's dot products at a fifth of the HBM rate.
struct DAcc {
  double                            s = 0.0;
  __device__ __forceinline__ void   add(double v) { s += v; }
  __device__ __forceinline__ void   add_prod(double a, double b) { s += a * b; }
  __device__ __forceinline__ double value() const { return s; }
};
template <typename T>
struct AccFor {
  using type = DAcc;
};
template <>
struct AccFor<float> {
  using type = F2Acc;
};

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

// The fixed grid leaves few threads per SM, so each thread loads 8 elements (i, i + stride, ...) before combining
// them; the combination order is the plain loop's, so the result does not depend on the unrolling.
template <typename T>
__global__ void __launch_bounds__(kReduceThreads) k_reduce_partial(int kind, int64_t n, const T *__restrict__ x, const T *__restrict__ y,
                                                                   double *__restrict__ partial) {
  constexpr int U      = 8;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t       i      = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  // The vector API's norms and dots keep FP64 sums for FP32 data too, so that squares above the FP32 range (|x| > 1.8e19)
  // do not overflow; the CG kernels, whose vectors are scaled to unit norm, use the FP32-pipe accumulator.
  DAcc sum;           // kRedSumSq, kRedAbsSum, kRedDot
  T    mx = T(0);     // kRedMaxAbs
  auto term = [&](T xi, T yi) {
    const T ax = xi < T(0) ? -xi : xi;
    if (kind == kRedSumSq) sum.add_prod((double)xi, (double)xi);
    else if (kind == kRedAbsSum) sum.add((double)ax);
    else if (kind == kRedMaxAbs) mx = ax > mx ? ax : mx;
    else sum.add_prod((double)xi, (double)yi);
  };
  for (; i + (U - 1) * stride < n; i += U * stride) {
    T xv[U], yv[U];
#pragma unroll
    for (int k = 0; k < U; k++) {
      xv[k] = x[i + k * stride];
      yv[k] = kind == kRedDot ? y[i + k * stride] : T(0);
    }
#pragma unroll
    for (int k = 0; k < U; k++) term(xv[k], yv[k]);
  }
  for (; i < n; i += stride) term(x[i], kind == kRedDot ? y[i] : T(0));
  const double acc = block_reduce(kind, kind == kRedMaxAbs ? (double)mx : sum.value());
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
