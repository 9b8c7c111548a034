// b200_vec_dot_static: a dot product that allocates nothing.
//
// Some callers of this library cannot allocate device memory at the moment they need a reduction: a host
// application whose memory manager owns every device allocation (pooled allocators in large simulation codes), or a
// time-critical loop that must not call cudaMalloc/cudaFree because those calls can synchronize the device.  This
// entry point serves them.  It is the two-pass FP64-accumulated dot product of b200_vec_dot, but its per-block
// partial sums live in a fixed array in device memory that is part of this library (g_dot_scratch below, 128 KiB,
// held by every GPU that loads the library until the process exits), and it writes the result to device memory the
// caller provides.  It needs no b200_ctx.
//
// Limits and sharing rules:
//  * n may be at most kStaticDotSlots * kStaticDotChunk = 134,217,728 entries; longer vectors are rejected with
//    B200_ERROR_DIMENSION before anything runs.
//  * All calls share g_dot_scratch, which keeps the last call's contents.  Each call writes every slot it later reads,
//    so nothing has to start at zero.  Calls whose kernels overlap on the GPU (different streams, or different host
//    threads, without ordering between them) race on the array and give wrong results: order them on one stream.
//  * The first call on a device looks up the array's device address (cudaGetSymbolAddress, with that device current)
//    and caches it; make that first call before any stream capture.
#include <atomic>

#include "b200_internal.cuh"
#include "b200_reduce.cuh"

namespace b200 {

constexpr int     kStaticDotSlots   = 16384;                     // partial sums: 16384 doubles = 128 KiB
constexpr int     kStaticDotChunk   = kReduceThreads * 32;       // entries summed by one block
constexpr int64_t kStaticDotMaxN    = (int64_t)kStaticDotSlots * kStaticDotChunk;
constexpr int     kStaticMaxDevices = 64;

static __device__ __align__(256) double g_dot_scratch[kStaticDotSlots];

// Device address of g_dot_scratch per device, filled on the first call with that device current.  The array's name in
// host code is only a host-side stand-in, so kernels are always given this address.
static std::atomic<double *> g_scratch_addr[kStaticMaxDevices];

// Block b sums x[i]*y[i] over its chunk [b*chunk, min((b+1)*chunk, n)) in a fixed order.
template <typename T>
__global__ void __launch_bounds__(kReduceThreads) k_dot_chunks(int64_t n, const T *__restrict__ x, const T *__restrict__ y,
                                                                 double *__restrict__ partial) {
  const int64_t beg = (int64_t)blockIdx.x * kStaticDotChunk;
  const int64_t end = beg + kStaticDotChunk < n ? beg + kStaticDotChunk : n;
  double        acc = 0.0;
  for (int64_t i = beg + threadIdx.x; i < end; i += kReduceThreads) acc += (double)x[i] * (double)y[i];
  acc = block_reduce(kRedDot, acc);
  if (threadIdx.x == 0) partial[blockIdx.x] = acc;
}

__global__ void __launch_bounds__(kReduceThreads) k_dot_chunks_final(int blocks, const double *__restrict__ partial, double *__restrict__ result) {
  double acc = 0.0;
  for (int i = threadIdx.x; i < blocks; i += kReduceThreads) acc += partial[i];
  acc = block_reduce(kRedDot, acc);
  if (threadIdx.x == 0) result[0] = acc;
}

static int static_scratch(double **out) {
  int dev = 0;
  B200_CUDA(cudaGetDevice(&dev));
  B200_CHECK(dev >= 0 && dev < kStaticMaxDevices, B200_ERROR_UNSUPPORTED, "device %d beyond the %d devices b200_vec_dot_static supports", dev,
             kStaticMaxDevices);
  double *ptr = g_scratch_addr[dev].load(std::memory_order_acquire);
  if (!ptr) {
    B200_CUDA(cudaGetSymbolAddress((void **)&ptr, g_dot_scratch));
    B200_CHECK(ptr != nullptr, B200_ERROR_BACKEND, "cudaGetSymbolAddress returned no address for the static scratch");
    g_scratch_addr[dev].store(ptr, std::memory_order_release);
  }
  *out = ptr;
  return B200_SUCCESS;
}

}  // namespace b200

using namespace b200;

extern "C" int b200_vec_dot_static(int prec, int64_t n, const void *x, const void *y, double *result, void *cuda_stream) {
  B200_CHECK(n >= 0 && n <= kStaticDotMaxN, B200_ERROR_DIMENSION,
             "b200_vec_dot_static: n = %lld exceeds its static scratch limit of %lld entries (use b200_vec_dot)", (long long)n,
             (long long)kStaticDotMaxN);
  B200_CHECK(prec == B200_F64 || prec == B200_F32, B200_ERROR_UNSUPPORTED, "unknown precision %d", prec);
  B200_CHECK(result && (n == 0 || (x && y)), B200_ERROR_INCOMPLETE, "b200_vec_dot_static: missing input or output pointer");
  double *scratch = nullptr;
  int     st      = static_scratch(&scratch);
  if (st) return st;
  cudaStream_t stream = (cudaStream_t)cuda_stream;
  const int    blocks = (int)ceil_div(n, kStaticDotChunk);
  if (blocks > 0) {
    if (prec == B200_F64) k_dot_chunks<double><<<blocks, kReduceThreads, 0, stream>>>(n, (const double *)x, (const double *)y, scratch);
    else k_dot_chunks<float><<<blocks, kReduceThreads, 0, stream>>>(n, (const float *)x, (const float *)y, scratch);
    B200_CUDA(cudaGetLastError());
  }
  k_dot_chunks_final<<<1, kReduceThreads, 0, stream>>>(blocks, scratch, result);
  B200_CUDA(cudaGetLastError());
  return B200_SUCCESS;
}
