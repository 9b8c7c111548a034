// Shared internals of libceed_b200: context, error reporting and launch bookkeeping.
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/ceed-b200.h"

struct b200_ctx_s {
  int          device;
  int          num_sms;
  cudaStream_t stream;
  int64_t      launches;  // kernels launched through this context
  // Reduction scratch: per-block partial sums and the host-visible result.
  double      *red_partial;
  double      *red_result_host;  // pinned
  int          red_blocks;
  int         *d_status;  // device: kernels OR in B200_STATUS_* bits (a bounded wait that gave up)
};

namespace b200 {

void set_error(const char *fmt, ...);
int  cuda_status(cudaError_t err, const char *what, const char *file, int line);

inline int check_launch(b200_ctx ctx, const char *what, const char *file, int line) {
  ctx->launches++;
  return cuda_status(cudaGetLastError(), what, file, line);
}

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Grid for a grid-stride elementwise kernel: a multiple of the SM count, bounded.
inline int stride_grid(b200_ctx ctx, int64_t n, int threads) {
  int64_t want = ceil_div(n, threads);
  int64_t cap  = (int64_t)ctx->num_sms * 8;
  if (want < 1) want = 1;
  return (int)(want < cap ? want : cap);
}

// Fused w = A u and u . (A u) for the CG (persistent FP32 operators with the atomic scatter): op_dot_blocks returns
// how many per-block partial sums op_apply_dot writes at the start of `partial`, or 0 when the operator's kernel has no
// such form, and sets *doubles to the length `partial` needs (the partial sums, then the kernel's per-thread scratch).
int op_dot_blocks(b200_op op, size_t *doubles);
int op_apply_dot(b200_op op, const void *u, void *v, const void *qdata, double *partial);

}  // namespace b200

#define B200_CUDA(call)                                                                  \
  do {                                                                                   \
    int _st = b200::cuda_status((call), #call, __FILE__, __LINE__);                      \
    if (_st) return _st;                                                                 \
  } while (0)

#define B200_LAUNCHED(ctx, name)                                                         \
  do {                                                                                   \
    int _st = b200::check_launch((ctx), name, __FILE__, __LINE__);                       \
    if (_st) return _st;                                                                 \
  } while (0)

#define B200_CHECK(cond, code, ...)                                                      \
  do {                                                                                   \
    if (!(cond)) {                                                                       \
      b200::set_error(__VA_ARGS__);                                                      \
      return (code);                                                                     \
    }                                                                                    \
  } while (0)
