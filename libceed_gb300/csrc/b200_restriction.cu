// Element restriction kernels: offset gather (L -> E), atomic scatter-add (E -> L), the deterministic inverse-offset
// scatter, and the strided forms used for qdata.
//
// The offset kernels take over include/ceed/jit-source/cuda/cuda-ref-restriction-offset.h (OffsetNoTranspose,
// OffsetTranspose in its atomic and deterministic forms); the inverse-offset plan takes over the host CSR build of
// backends/cuda-ref/ceed-cuda-ref-restriction.c:416-493.  E-vectors use the layout [comp][elem][node].
#include "b200_internal.cuh"

#include <algorithm>
#include <vector>

#include "b200_plan.cuh"

struct b200_plan_s {
  b200_ctx ctx;
  int64_t  num_elem;
  int      elem_size;
  int64_t  num_unique;    // distinct offsets
  int32_t *l_indices;     // [num_unique] distinct offsets, ascending
  int32_t *t_start;       // [num_unique + 1] CSR row starts into t_indices
  int32_t *t_indices;     // [num_elem * elem_size] E-node index e*elem_size + i, ascending within a row
  int      num_comp;
  int64_t  comp_stride;
  int64_t  l_size;
  bool     covers_all;    // every L entry in [0, l_size) is hit (then add = 0 needs no zeroing)
};

namespace b200 {

template <typename T>
__global__ void k_gather(int64_t num_entries, int64_t e_comp_stride, int num_comp, int64_t comp_stride, const int32_t *__restrict__ offsets,
                         const T *__restrict__ l_vec, T *__restrict__ e_vec) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < num_entries; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t o = offsets[i];
    for (int c = 0; c < num_comp; c++) e_vec[c * e_comp_stride + i] = l_vec[o + c * comp_stride];
  }
}

template <typename T>
__global__ void k_scatter_atomic(int64_t num_entries, int64_t e_comp_stride, int num_comp, int64_t comp_stride,
                                 const int32_t *__restrict__ offsets, const T *__restrict__ e_vec, T *__restrict__ l_vec) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < num_entries; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t o = offsets[i];
    for (int c = 0; c < num_comp; c++) atomicAdd(&l_vec[o + c * comp_stride], e_vec[c * e_comp_stride + i]);
  }
}

// One thread per distinct node: sum its E entries in ascending E-index order, then write (or add) once.
template <typename T>
__global__ void k_scatter_det(int64_t num_unique, int64_t e_comp_stride, int num_comp, int64_t comp_stride, const int32_t *__restrict__ l_indices,
                              const int32_t *__restrict__ t_start, const int32_t *__restrict__ t_indices, const T *__restrict__ e_vec,
                              T *__restrict__ l_vec, int add) {
  for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < num_unique; u += (int64_t)gridDim.x * blockDim.x) {
    const int32_t beg = t_start[u], end = t_start[u + 1];
    const int64_t o   = l_indices[u];
    for (int c = 0; c < num_comp; c++) {
      T s = 0;
      for (int32_t k = beg; k < end; k++) s += e_vec[c * e_comp_stride + t_indices[k]];
      T *dst = &l_vec[o + c * comp_stride];
      *dst   = add ? *dst + s : s;
    }
  }
}

template <typename T>
__global__ void k_strided_gather(int64_t num_elem, int elem_size, int num_comp, int64_t s0, int64_t s1, int64_t s2, const T *__restrict__ l_vec,
                                 T *__restrict__ e_vec) {
  const int64_t n = num_elem * elem_size;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = i / elem_size, node = i % elem_size;
    for (int c = 0; c < num_comp; c++) e_vec[c * n + i] = l_vec[node * s0 + c * s1 + e * s2];
  }
}

template <typename T>
__global__ void k_strided_scatter(int64_t num_elem, int elem_size, int num_comp, int64_t s0, int64_t s1, int64_t s2, const T *__restrict__ e_vec,
                                  T *__restrict__ l_vec) {
  const int64_t n = num_elem * elem_size;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = i / elem_size, node = i % elem_size;
    for (int c = 0; c < num_comp; c++) l_vec[node * s0 + c * s1 + e * s2] += e_vec[c * n + i];
  }
}

}  // namespace b200

using namespace b200;

#define PREC_SWITCH(prec, T, ...)                                                                       \
  do {                                                                                                   \
    if ((prec) == B200_F64) {                                                                            \
      using T = double;                                                                                  \
      __VA_ARGS__;                                                                                              \
    } else if ((prec) == B200_F32) {                                                                     \
      using T = float;                                                                                   \
      __VA_ARGS__;                                                                                              \
    } else {                                                                                             \
      set_error("unknown precision %d", (int)(prec));                                                    \
      return B200_ERROR_UNSUPPORTED;                                                                     \
    }                                                                                                    \
  } while (0)

extern "C" int b200_rstr_gather(b200_ctx ctx, int prec, int64_t num_elem, int elem_size, int num_comp, int64_t comp_stride, int64_t l_size,
                                const int32_t *offsets, const void *l_vec, void *e_vec) {
  (void)l_size;
  const int64_t n = num_elem * elem_size;
  if (n <= 0) return B200_SUCCESS;
  PREC_SWITCH(prec, T, {
    k_gather<T><<<stride_grid(ctx, n, 256), 256, 0, ctx->stream>>>(n, n, num_comp, comp_stride, offsets, (const T *)l_vec, (T *)e_vec);
    B200_LAUNCHED(ctx, "rstr_gather");
  });
  return B200_SUCCESS;
}

extern "C" int b200_rstr_scatter_atomic(b200_ctx ctx, int prec, int64_t num_elem, int elem_size, int num_comp, int64_t comp_stride, int64_t l_size,
                                        const int32_t *offsets, const void *e_vec, void *l_vec) {
  (void)l_size;
  const int64_t n = num_elem * elem_size;
  if (n <= 0) return B200_SUCCESS;
  PREC_SWITCH(prec, T, {
    k_scatter_atomic<T><<<stride_grid(ctx, n, 256), 256, 0, ctx->stream>>>(n, n, num_comp, comp_stride, offsets, (const T *)e_vec, (T *)l_vec);
    B200_LAUNCHED(ctx, "rstr_scatter_atomic");
  });
  return B200_SUCCESS;
}

extern "C" int b200_plan_create(b200_ctx ctx, int64_t num_elem, int elem_size, int num_comp, int64_t comp_stride, int64_t l_size,
                                const int32_t *offsets_host, const int32_t *offsets_dev, b200_plan *out) {
  const int64_t        n = num_elem * elem_size;
  std::vector<int32_t> off_copy;
  B200_CHECK(n < (int64_t)INT32_MAX, B200_ERROR_UNSUPPORTED, "deterministic plan: %lld E entries exceed int32 indexing", (long long)n);
  if (!offsets_host) {
    B200_CHECK(offsets_dev, B200_ERROR_INCOMPLETE, "b200_plan_create: no offsets given");
    off_copy.resize((size_t)n);
    B200_CUDA(cudaMemcpy(off_copy.data(), offsets_dev, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost));
    offsets_host = off_copy.data();
  }
  int32_t max_off = -1;
  for (int64_t i = 0; i < n; i++) {
    B200_CHECK(offsets_host[i] >= 0, B200_ERROR_DIMENSION, "offset %lld is negative (%d)", (long long)i, offsets_host[i]);
    max_off = std::max(max_off, offsets_host[i]);
  }
  // Counting sort by offset: rows in ascending offset order, entries in ascending E index within a row.
  std::vector<int32_t> count((size_t)max_off + 2, 0);
  for (int64_t i = 0; i < n; i++) count[(size_t)offsets_host[i] + 1]++;
  std::vector<int32_t> l_idx, t_start;
  l_idx.reserve((size_t)n);
  t_start.reserve((size_t)n + 1);
  std::vector<int32_t> pos((size_t)max_off + 1, 0);
  int32_t              acc = 0;
  for (int64_t o = 0; o <= max_off; o++) {
    const int32_t c = count[(size_t)o + 1];
    pos[(size_t)o]  = acc;
    if (c > 0) {
      l_idx.push_back((int32_t)o);
      t_start.push_back(acc);
    }
    acc += c;
  }
  t_start.push_back(acc);
  std::vector<int32_t> t_idx((size_t)n);
  for (int64_t i = 0; i < n; i++) t_idx[(size_t)pos[(size_t)offsets_host[i]]++] = (int32_t)i;

  B200_CHECK((int64_t)max_off + (int64_t)(num_comp - 1) * comp_stride < l_size, B200_ERROR_DIMENSION,
             "offsets reach %lld, beyond the L-vector length %lld", (long long)max_off + (long long)(num_comp - 1) * comp_stride, (long long)l_size);

  b200_plan p    = new b200_plan_s();  // value-initialised: device pointers start null, so b200_plan_destroy frees a partial plan
  p->ctx         = ctx;
  p->num_elem    = num_elem;
  p->elem_size   = elem_size;
  p->num_unique  = (int64_t)l_idx.size();
  p->num_comp    = num_comp;
  p->comp_stride = comp_stride;
  p->l_size      = l_size;
  // A valid restriction maps distinct (offset, component) pairs to distinct entries, so it writes every entry of the
  // L-vector exactly when the pairs are as many as the entries.
  p->covers_all  = p->num_unique * num_comp == l_size;
  cudaError_t err = cudaMalloc(&p->l_indices, sizeof(int32_t) * l_idx.size());
  if (err == cudaSuccess) err = cudaMalloc(&p->t_start, sizeof(int32_t) * t_start.size());
  if (err == cudaSuccess) err = cudaMalloc(&p->t_indices, sizeof(int32_t) * t_idx.size());
  if (err == cudaSuccess) err = cudaMemcpy(p->l_indices, l_idx.data(), sizeof(int32_t) * l_idx.size(), cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMemcpy(p->t_start, t_start.data(), sizeof(int32_t) * t_start.size(), cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMemcpy(p->t_indices, t_idx.data(), sizeof(int32_t) * t_idx.size(), cudaMemcpyHostToDevice);
  if (err != cudaSuccess) {
    b200_plan_destroy(p);
    return cuda_status(err, "b200_plan_create", __FILE__, __LINE__);
  }
  *out = p;
  return B200_SUCCESS;
}

extern "C" int b200_plan_destroy(b200_plan p) {
  if (!p) return B200_SUCCESS;
  cudaFree(p->l_indices);
  cudaFree(p->t_start);
  cudaFree(p->t_indices);
  delete p;
  return B200_SUCCESS;
}

namespace b200 {
int plan_scatter(b200_plan p, int prec, const void *e_vec, void *l_vec, int add) {
  b200_ctx      ctx = p->ctx;
  const int     num_comp = p->num_comp;
  const int64_t comp_stride = p->comp_stride, l_size = p->l_size;
  const int64_t n   = p->num_elem * p->elem_size;
  if (!add && !p->covers_all) {
    int st = b200_vec_set_value(ctx, prec, l_size, l_vec, 0.0);
    if (st) return st;
  }
  if (p->num_unique == 0) return B200_SUCCESS;
  PREC_SWITCH(prec, T, {
    k_scatter_det<T><<<stride_grid(ctx, p->num_unique, 256), 256, 0, ctx->stream>>>(p->num_unique, n, num_comp, comp_stride, p->l_indices, p->t_start,
                                                                                    p->t_indices, (const T *)e_vec, (T *)l_vec,
                                                                                    add || !p->covers_all);
    B200_LAUNCHED(ctx, "rstr_scatter_det");
  });
  return B200_SUCCESS;
}
}  // namespace b200

extern "C" int b200_rstr_scatter_det(b200_ctx ctx, b200_plan plan, int prec, const void *e_vec, void *l_vec, int add) {
  B200_CHECK(plan && plan->ctx == ctx, B200_ERROR_INCOMPATIBLE, "b200_rstr_scatter_det: plan belongs to another context");
  return plan_scatter(plan, prec, e_vec, l_vec, add);
}

extern "C" int b200_rstr_strided_gather(b200_ctx ctx, int prec, int64_t num_elem, int elem_size, int num_comp, const int64_t strides[3],
                                        const void *l_vec, void *e_vec) {
  const int64_t n = num_elem * elem_size;
  if (n <= 0) return B200_SUCCESS;
  PREC_SWITCH(prec, T, {
    k_strided_gather<T><<<stride_grid(ctx, n, 256), 256, 0, ctx->stream>>>(num_elem, elem_size, num_comp, strides[0], strides[1], strides[2],
                                                                          (const T *)l_vec, (T *)e_vec);
    B200_LAUNCHED(ctx, "rstr_strided_gather");
  });
  return B200_SUCCESS;
}

extern "C" int b200_rstr_strided_scatter(b200_ctx ctx, int prec, int64_t num_elem, int elem_size, int num_comp, const int64_t strides[3],
                                         const void *e_vec, void *l_vec) {
  const int64_t n = num_elem * elem_size;
  if (n <= 0) return B200_SUCCESS;
  PREC_SWITCH(prec, T, {
    k_strided_scatter<T><<<stride_grid(ctx, n, 256), 256, 0, ctx->stream>>>(num_elem, elem_size, num_comp, strides[0], strides[1], strides[2],
                                                                           (const T *)e_vec, (T *)l_vec);
    B200_LAUNCHED(ctx, "rstr_strided_scatter");
  });
  return B200_SUCCESS;
}
