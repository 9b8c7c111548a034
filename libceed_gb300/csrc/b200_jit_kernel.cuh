// Fused operator kernel for QFunctions compiled at run time (NVRTC, -arch=sm_103a).
//
// The user's QFunction source is included into the program together with a small generated glue function,
// b200_jit_point(), that gathers the QFunction's passive inputs at one quadrature point, arranges the active field's
// values in libCEED's per-point layout (component k of field i at in[i][k], CEED_Q_VLA = 1, Q = 1 per call) and calls
// the user function.  This mirrors how the reference inlines QFunctions into its generated kernel
// (backends/cuda-gen/ceed-cuda-gen-operator-build.cpp:1343-1361), but here the surrounding kernel is a fixed template:
// one active field in (CEED_EVAL_INTERP or CEED_EVAL_GRAD) and out, any passive CEED_EVAL_NONE inputs through
// backend-strided restrictions, one component.
#pragma once

#include "b200_op_kernels.cuh"

namespace b200 {

constexpr int kJitMaxFields = 8;

template <typename T>
struct JitFields {
  const T *passive[kJitMaxFields];  // passive inputs in QFunction order (skipping the active one), [comp][elem][qpt]
  void    *ctx;                     // QFunction context data (device memory) or nullptr
};

#define B200_IDX(x, y, z) ((x) + Q * (y) + tile_plane(Q) * (z))
#define B200_QLIN(x, y, z) ((x) + Q * ((y) + Q * (z)))

template <typename T, int P, int Q, int EVAL_IN, int EVAL_OUT, bool EO>
__global__ void k_op_jit(const OpArgs<typename Store<T>::type> args, const JitFields<T> F, const OpMats<T, P, Q> M) {
  using C                 = Contract<T, P, Q, EO>;
  constexpr int  Q2       = Q * Q, Q3 = Q * Q * Q, P3 = P * P * P;
  constexpr bool GRAD_IN  = EVAL_IN == B200_EVAL_GRAD;
  constexpr bool GRAD_OUT = EVAL_OUT == B200_EVAL_GRAD;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int     tid = threadIdx.x % Q2, slot = threadIdx.x / Q2;
  const int     a = tid % Q, b = tid / Q;
  const int64_t e      = (int64_t)blockIdx.x * args.epb + slot;
  const bool    active = e < args.num_elem;
  const int64_t ne     = args.num_elem;
  T *s0 = reinterpret_cast<T *>(smem_raw) + slot * tile_team_stride(Q, 0), *s1 = s0 + tile_buf(Q), *s2 = s1 + tile_buf(Q);

  for (int i = tid; i < P3; i += Q2) {
    const int x = i % P, y = (i / P) % P, z = i / (P * P);
    s0[B200_IDX(x, y, z)] = active ? args.u[args.offsets[e * P3 + i]] : T(0);
  }
  __syncthreads();
  if (a < P && b < P) {
    T in[P], o[Q];
#pragma unroll
    for (int k = 0; k < P; k++) in[k] = s0[B200_IDX(k, a, b)];
    C::interp(M, in, o);
#pragma unroll
    for (int j = 0; j < Q; j++) s1[B200_IDX(j, a, b)] = o[j];
  }
  __syncthreads();
  if (b < P) {
    T in[P], o[Q];
#pragma unroll
    for (int k = 0; k < P; k++) in[k] = s1[B200_IDX(a, k, b)];
    C::interp(M, in, o);
#pragma unroll
    for (int j = 0; j < Q; j++) s0[B200_IDX(a, j, b)] = o[j];
  }
  __syncthreads();
  T U[Q], dz[Q];
  {
    T in[P];
#pragma unroll
    for (int k = 0; k < P; k++) in[k] = s0[B200_IDX(a, b, k)];
    C::interp(M, in, U);
  }
  if constexpr (GRAD_IN) {
#pragma unroll
    for (int j = 0; j < Q; j++) s1[B200_IDX(a, b, j)] = U[j];
    C::grad(M, U, dz);
    __syncthreads();
    {
      T in[Q], o[Q];
#pragma unroll
      for (int k = 0; k < Q; k++) in[k] = s1[B200_IDX(k, a, b)];
      C::grad(M, in, o);
#pragma unroll
      for (int j = 0; j < Q; j++) s0[B200_IDX(j, a, b)] = o[j];
#pragma unroll
      for (int k = 0; k < Q; k++) in[k] = s1[B200_IDX(a, k, b)];
      C::grad(M, in, o);
#pragma unroll
      for (int j = 0; j < Q; j++) s2[B200_IDX(a, j, b)] = o[j];
    }
    __syncthreads();
  }
  // ---- the user's QFunction at each point of the thread's z-line ----------------------------------------------------
  T w[Q];
#pragma unroll 1
  for (int z = 0; z < Q; z++) {
    const int q = B200_IDX(a, b, z), qg = B200_QLIN(a, b, z);
    T         act_in[GRAD_IN ? 3 : 1], act_out[GRAD_OUT ? 3 : 1];
    if constexpr (GRAD_IN) {
      act_in[0] = s0[q];
      act_in[1] = s2[q];
      act_in[2] = dz[z];
    } else {
      act_in[0] = U[z];
    }
    if (active) b200_jit_point(F, ne, e, qg, act_in, act_out);
    else
      for (int k = 0; k < (GRAD_OUT ? 3 : 1); k++) act_out[k] = T(0);
    if constexpr (GRAD_OUT) {
      s0[q] = act_out[0];  // each thread rewrites only its own z-line here
      s2[q] = act_out[1];
      w[z]  = act_out[2];
    } else {
      w[z] = act_out[0];
    }
  }
  if constexpr (GRAD_OUT) {
    __syncthreads();
    {
      T in[Q], o[Q];
#pragma unroll
      for (int k = 0; k < Q; k++) in[k] = s0[B200_IDX(k, a, b)];
      C::grad_t(M, in, o);
#pragma unroll
      for (int j = 0; j < Q; j++) s1[B200_IDX(j, a, b)] = o[j];
    }
    __syncthreads();
    {
      T in[Q], o[Q];
#pragma unroll
      for (int k = 0; k < Q; k++) in[k] = s2[B200_IDX(a, k, b)];
      C::grad_t(M, in, o);
#pragma unroll
      for (int j = 0; j < Q; j++) s1[B200_IDX(a, j, b)] += o[j];
    }
    __syncthreads();
    T wz[Q];
    C::grad_t(M, w, wz);
#pragma unroll
    for (int j = 0; j < Q; j++) w[j] = wz[j] + s1[B200_IDX(a, b, j)];
  }
  {
    T o[P];
    C::interp_t(M, w, o);
    // Every thread rewrites only its own z-line of s0 here (the points it read in the QFunction stage).
#pragma unroll
    for (int p = 0; p < P; p++) s0[B200_IDX(a, b, p)] = o[p];
  }
  __syncthreads();
  if (b < P) {
    T in[Q], o[P];
#pragma unroll
    for (int k = 0; k < Q; k++) in[k] = s0[B200_IDX(a, k, b)];
    C::interp_t(M, in, o);
#pragma unroll
    for (int p = 0; p < P; p++) s1[B200_IDX(a, p, b)] = o[p];
  }
  __syncthreads();
  if (a < P && b < P && active) {
    T in[Q], out[P];
#pragma unroll
    for (int k = 0; k < Q; k++) in[k] = s1[B200_IDX(k, a, b)];
    C::interp_t(M, in, out);
    scatter_line<T, P>(args, e, 0, args.offsets + e * P3 + P * (a + P * b), a, b, out);
  }
}

#undef B200_IDX
#undef B200_QLIN

}  // namespace b200
