// Fused operator-apply kernels for tensor-product H1 hexahedra (the hot path).
//
// One kernel does, per element: offset gather of u -> sum-factorized interpolation to the Q^3 Gauss points ->
// collocated gradient -> pointwise QFunction -> transposed gradient and interpolation -> scatter-add into v (atomic),
// or a write of the element result for the deterministic inverse-offset scatter.  This is the work the reference
// splits across CeedOperatorApplyAdd_Ref's element loop (backends/ref/ceed-ref-operator.c:381-476) and fuses in the
// string-generated cuda-gen kernel (backends/cuda-gen/ceed-cuda-gen-operator-build.cpp:1158-1680).
//
// Thread layout ("line" mapping): a team of Q*Q threads per element, team thread (a, b).  In each 1D contraction a
// thread owns one line of the element tile along the contracted direction: it loads the line from shared memory into
// registers, applies the 1D matrix (held in the kernel's parameter space, so every FMA reads it as a constant
// operand) and writes the line back.  The z-direction lines stay in registers across stages.  A block holds
// `epb` teams; the element tile buffers live in dynamic shared memory.
//
// Gradient: collocated, dX = G_c (B u) with G_c = G B^+ (Q x Q); the transpose applies G_c^T then B^T.
// Staging of qdata: kStageReg prefetches the thread's z-line of qdata into registers at kernel entry (the loads are
// in flight during the interpolation stages); kStageSmem copies the element's qdata slab into shared memory at entry
// (reused by all components of a vector field).
#pragma once

#include <cstdint>

#include "b200_pointwise.cuh"

namespace b200 {

enum { kStageReg = 1, kStageSmem = 2 };

template <typename T, int P, int Q>
struct OpMats {
  T B[Q * P];  // interp, row-major Q x P
  T G[Q * Q];  // collocated gradient, row-major Q x Q
};

template <typename T>
struct OpArgs {
  int64_t        num_elem;
  int64_t        comp_stride;  // L-vector component stride
  int            epb;          // elements per block
  int            det;          // 1: write the element result to e_out (deterministic scatter follows)
  const int32_t *offsets;
  const T       *u;
  T             *v;      // L-vector (atomic scatter)
  T             *e_out;  // E-vector [comp][elem][node] (deterministic scatter)
  const T       *qdata;  // [qcomp][elem][qpt]
  const T       *kappa;  // [elem][qpt] or nullptr
};

template <int QF>
struct QFTraits {
  static constexpr bool grad  = QF == B200_QF_POISSON || QF == B200_QF_VECPOISSON || QF == B200_QF_POISSON_KAPPA;
  static constexpr int  nc    = (QF == B200_QF_VECMASS || QF == B200_QF_VECPOISSON) ? 3 : 1;
  static constexpr int  nqd   = grad ? 6 : 1;
  static constexpr bool kappa = QF == B200_QF_POISSON_KAPPA;
};

template <typename T, int P, int Q, int QF, int STAGE>
struct OpShape {
  static constexpr int Q2 = Q * Q, Q3 = Q * Q * Q, P3 = P * P * P;
  // Per-team shared memory in elements of T: three Q^3 tile buffers, plus the qdata slab when staged in smem.
  static constexpr int team_smem = 3 * Q3 + (STAGE == kStageSmem ? (QFTraits<QF>::nqd + (QFTraits<QF>::kappa ? 1 : 0)) * Q3 : 0);
};

// out[j] = sum_k M[j*K + k] in[k], j < J
template <typename T, int J, int K>
__device__ __forceinline__ void mat_apply(const T *M, const T (&in)[K], T (&out)[J]) {
#pragma unroll
  for (int j = 0; j < J; j++) {
    T s = M[j * K] * in[0];
#pragma unroll
    for (int k = 1; k < K; k++) s = fma(M[j * K + k], in[k], s);
    out[j] = s;
  }
}

// out[k] = sum_j M[j*K + k] in[j], k < K  (transpose of a J x K matrix)
template <typename T, int J, int K>
__device__ __forceinline__ void mat_apply_t(const T *M, const T (&in)[J], T (&out)[K]) {
#pragma unroll
  for (int k = 0; k < K; k++) {
    T s = M[k] * in[0];
#pragma unroll
    for (int j = 1; j < J; j++) s = fma(M[j * K + k], in[j], s);
    out[k] = s;
  }
}

template <typename T, int P, int Q, int QF, int STAGE>
__global__ void k_op_apply(const OpArgs<T> args, const OpMats<T, P, Q> M) {
  using TR            = QFTraits<QF>;
  using SH            = OpShape<T, P, Q, QF, STAGE>;
  constexpr int Q2    = SH::Q2, Q3 = SH::Q3, P3 = SH::P3, NC = TR::nc, NQD = TR::nqd;
  constexpr bool GRAD = TR::grad;
#define IDX(x, y, z) (((z) * Q + (y)) * Q + (x))

  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int     tid = threadIdx.x % Q2, slot = threadIdx.x / Q2;
  const int     a = tid % Q, b = tid / Q;
  const int64_t e      = (int64_t)blockIdx.x * args.epb + slot;
  const bool    active = e < args.num_elem;
  const int64_t ne     = args.num_elem;
  T *s0 = reinterpret_cast<T *>(smem_raw) + slot * SH::team_smem, *s1 = s0 + Q3, *s2 = s1 + Q3, *sq = s2 + Q3;

  // ---- qdata staging ----------------------------------------------------------------------------------------
  constexpr int RQ = STAGE == kStageReg ? NQD : 1, RZ = STAGE == kStageReg ? Q : 1, RK = (STAGE == kStageReg && TR::kappa) ? Q : 1;
  T rq[RQ][RZ], rk[RK];
  if constexpr (STAGE == kStageReg) {
#pragma unroll
    for (int z = 0; z < Q; z++) {
#pragma unroll
      for (int k = 0; k < NQD; k++) rq[k][z] = active ? args.qdata[((int64_t)k * ne + e) * Q3 + IDX(a, b, z)] : T(0);
      if constexpr (TR::kappa) rk[z] = active ? args.kappa[e * Q3 + IDX(a, b, z)] : T(0);
    }
  } else {
    for (int i = tid; i < NQD * Q3; i += Q2) {
      const int k = i / Q3, q = i % Q3;
      sq[i]       = active ? args.qdata[((int64_t)k * ne + e) * Q3 + q] : T(0);
    }
    if constexpr (TR::kappa)
      for (int q = tid; q < Q3; q += Q2) sq[NQD * Q3 + q] = active ? args.kappa[e * Q3 + q] : T(0);
  }

#pragma unroll 1
  for (int c = 0; c < NC; c++) {
    if (c > 0) __syncthreads();
    // ---- gather u into s0[z][y][x] ------------------------------------------------------------------------------
    for (int i = tid; i < P3; i += Q2) {
      const int x = i % P, y = (i / P) % P, z = i / (P * P);
      s0[IDX(x, y, z)] = active ? args.u[(int64_t)args.offsets[e * P3 + i] + c * args.comp_stride] : T(0);
    }
    __syncthreads();
    // ---- X interpolation: lines (y, z) < P ------------------------------------------------------------------------
    if (a < P && b < P) {
      T in[P], out[Q];
#pragma unroll
      for (int k = 0; k < P; k++) in[k] = s0[IDX(k, a, b)];
      mat_apply<T, Q, P>(M.B, in, out);
#pragma unroll
      for (int j = 0; j < Q; j++) s1[IDX(j, a, b)] = out[j];
    }
    __syncthreads();
    // ---- Y interpolation: lines (x < Q, z < P) --------------------------------------------------------------------
    if (b < P) {
      T in[P], out[Q];
#pragma unroll
      for (int k = 0; k < P; k++) in[k] = s1[IDX(a, k, b)];
      mat_apply<T, Q, P>(M.B, in, out);
#pragma unroll
      for (int j = 0; j < Q; j++) s0[IDX(a, j, b)] = out[j];
    }
    __syncthreads();
    // ---- Z interpolation (+ Z derivative): lines (x, y) ------------------------------------------------------------
    T U[Q], dz[GRAD ? Q : 1];
    {
      T in[P];
#pragma unroll
      for (int k = 0; k < P; k++) in[k] = s0[IDX(a, b, k)];
      mat_apply<T, Q, P>(M.B, in, U);
    }
    if constexpr (GRAD) {
#pragma unroll
      for (int j = 0; j < Q; j++) s1[IDX(a, b, j)] = U[j];
      mat_apply<T, Q, Q>(M.G, U, dz);
      __syncthreads();
      // ---- X and Y derivatives of the interpolated values -----------------------------------------------------------
      {
        T in[Q], out[Q];
#pragma unroll
        for (int k = 0; k < Q; k++) in[k] = s1[IDX(k, a, b)];
        mat_apply<T, Q, Q>(M.G, in, out);
#pragma unroll
        for (int j = 0; j < Q; j++) s0[IDX(j, a, b)] = out[j];
#pragma unroll
        for (int k = 0; k < Q; k++) in[k] = s1[IDX(a, k, b)];
        mat_apply<T, Q, Q>(M.G, in, out);
#pragma unroll
        for (int j = 0; j < Q; j++) s2[IDX(a, j, b)] = out[j];
      }
      __syncthreads();
      // ---- pointwise QFunction on the z-line (x = a, y = b) ----------------------------------------------------------
#pragma unroll
      for (int z = 0; z < Q; z++) {
        T D[6];
#pragma unroll
        for (int k = 0; k < 6; k++) {
          if constexpr (STAGE == kStageReg) D[k] = rq[k][z];
          else D[k] = sq[k * Q3 + IDX(a, b, z)];
        }
        if constexpr (TR::kappa) {
          T kap;
          if constexpr (STAGE == kStageReg) kap = rk[z];
          else kap = sq[NQD * Q3 + IDX(a, b, z)];
#pragma unroll
          for (int k = 0; k < 6; k++) D[k] *= kap;
        }
        T vg[3];
        poisson_point(D, s0[IDX(a, b, z)], s2[IDX(a, b, z)], dz[z], vg);
        s0[IDX(a, b, z)] = vg[0];
        s2[IDX(a, b, z)] = vg[1];
        dz[z]            = vg[2];
      }
      __syncthreads();
      // ---- X derivative, transposed: lines (y, z) --------------------------------------------------------------------
      {
        T in[Q], out[Q];
#pragma unroll
        for (int k = 0; k < Q; k++) in[k] = s0[IDX(k, a, b)];
        mat_apply_t<T, Q, Q>(M.G, in, out);
#pragma unroll
        for (int j = 0; j < Q; j++) s1[IDX(j, a, b)] = out[j];
      }
      __syncthreads();
      // ---- Y derivative, transposed, accumulated: lines (x, z) ---------------------------------------------------------
      {
        T in[Q], out[Q];
#pragma unroll
        for (int k = 0; k < Q; k++) in[k] = s2[IDX(a, k, b)];
        mat_apply_t<T, Q, Q>(M.G, in, out);
#pragma unroll
        for (int j = 0; j < Q; j++) s1[IDX(a, j, b)] += out[j];
      }
      __syncthreads();
      // ---- Z derivative transposed + sum, then Z interpolation transposed: lines (x, y) ---------------------------------
      {
        T w[Q], out[P];
        mat_apply_t<T, Q, Q>(M.G, dz, w);
#pragma unroll
        for (int j = 0; j < Q; j++) w[j] += s1[IDX(a, b, j)];
        mat_apply_t<T, Q, P>(M.B, w, out);
#pragma unroll
        for (int p = 0; p < P; p++) s0[IDX(a, b, p)] = out[p];
      }
    } else {
      // ---- mass: pointwise product on the z-line, then Z interpolation transposed ------------------------------------------
      // Each thread reads and rewrites only its own z-line of s0, so no barrier is needed here.
      T w[Q], out[P];
#pragma unroll
      for (int z = 0; z < Q; z++) {
        if constexpr (STAGE == kStageReg) w[z] = U[z] * rq[0][z];
        else w[z] = U[z] * sq[IDX(a, b, z)];
      }
      mat_apply_t<T, Q, P>(M.B, w, out);
#pragma unroll
      for (int p = 0; p < P; p++) s0[IDX(a, b, p)] = out[p];
    }
    __syncthreads();
    // ---- Y interpolation transposed: lines (x < Q, z < P) ------------------------------------------------------------------
    if (b < P) {
      T in[Q], out[P];
#pragma unroll
      for (int k = 0; k < Q; k++) in[k] = s0[IDX(a, k, b)];
      mat_apply_t<T, Q, P>(M.B, in, out);
#pragma unroll
      for (int p = 0; p < P; p++) s1[IDX(a, p, b)] = out[p];
    }
    __syncthreads();
    // ---- X interpolation transposed and scatter: lines (y, z) < P ----------------------------------------------------------
    if (a < P && b < P && active) {
      T in[Q], out[P];
#pragma unroll
      for (int k = 0; k < Q; k++) in[k] = s1[IDX(k, a, b)];
      mat_apply_t<T, Q, P>(M.B, in, out);
      const int base = P * (a + P * b);
      if (args.det) {
        T *dst = args.e_out + ((int64_t)c * ne + e) * P3 + base;
#pragma unroll
        for (int p = 0; p < P; p++) dst[p] = out[p];
      } else {
#pragma unroll
        for (int p = 0; p < P; p++) atomicAdd(&args.v[(int64_t)args.offsets[e * P3 + base + p] + c * args.comp_stride], out[p]);
      }
    }
  }
#undef IDX
}

// Gradient of the kappa-weighted diffusion with respect to kappa: g[e][q] = grad(w)_q . D_q grad(u)_q, both gradients
// recomputed from the L-vectors (no stored E-vectors).
template <typename T, int P, int Q>
__global__ void k_kappa_grad(const OpArgs<T> args, const T *__restrict__ w_vec, T *__restrict__ g, const OpMats<T, P, Q> M) {
  constexpr int Q2 = Q * Q, Q3 = Q * Q * Q, P3 = P * P * P;
#define IDX(x, y, z) (((z) * Q + (y)) * Q + (x))
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int     tid = threadIdx.x % Q2, slot = threadIdx.x / Q2;
  const int     a = tid % Q, b = tid / Q;
  const int64_t e      = (int64_t)blockIdx.x * args.epb + slot;
  const bool    active = e < args.num_elem;
  const int64_t ne     = args.num_elem;
  T *s0 = reinterpret_cast<T *>(smem_raw) + slot * 3 * Q3, *s1 = s0 + Q3, *s2 = s1 + Q3;
  T  gu[3][Q];
#pragma unroll 1
  for (int pass = 0; pass < 2; pass++) {
    const T *src = pass == 0 ? args.u : w_vec;
    if (pass) __syncthreads();
    for (int i = tid; i < P3; i += Q2) {
      const int x = i % P, y = (i / P) % P, z = i / (P * P);
      s0[IDX(x, y, z)] = active ? src[args.offsets[e * P3 + i]] : T(0);
    }
    __syncthreads();
    if (a < P && b < P) {
      T in[P], out[Q];
#pragma unroll
      for (int k = 0; k < P; k++) in[k] = s0[IDX(k, a, b)];
      mat_apply<T, Q, P>(M.B, in, out);
#pragma unroll
      for (int j = 0; j < Q; j++) s1[IDX(j, a, b)] = out[j];
    }
    __syncthreads();
    if (b < P) {
      T in[P], out[Q];
#pragma unroll
      for (int k = 0; k < P; k++) in[k] = s1[IDX(a, k, b)];
      mat_apply<T, Q, P>(M.B, in, out);
#pragma unroll
      for (int j = 0; j < Q; j++) s0[IDX(a, j, b)] = out[j];
    }
    __syncthreads();
    T U[Q], dz[Q];
    {
      T in[P];
#pragma unroll
      for (int k = 0; k < P; k++) in[k] = s0[IDX(a, b, k)];
      mat_apply<T, Q, P>(M.B, in, U);
    }
#pragma unroll
    for (int j = 0; j < Q; j++) s1[IDX(a, b, j)] = U[j];
    mat_apply<T, Q, Q>(M.G, U, dz);
    __syncthreads();
    {
      T in[Q], out[Q];
#pragma unroll
      for (int k = 0; k < Q; k++) in[k] = s1[IDX(k, a, b)];
      mat_apply<T, Q, Q>(M.G, in, out);
#pragma unroll
      for (int j = 0; j < Q; j++) s0[IDX(j, a, b)] = out[j];
#pragma unroll
      for (int k = 0; k < Q; k++) in[k] = s1[IDX(a, k, b)];
      mat_apply<T, Q, Q>(M.G, in, out);
#pragma unroll
      for (int j = 0; j < Q; j++) s2[IDX(a, j, b)] = out[j];
    }
    __syncthreads();
    if (pass == 0) {
#pragma unroll
      for (int z = 0; z < Q; z++) {
        T D[6];
#pragma unroll
        for (int k = 0; k < 6; k++) D[k] = active ? args.qdata[((int64_t)k * ne + e) * Q3 + IDX(a, b, z)] : T(0);
        T vg[3];
        poisson_point(D, s0[IDX(a, b, z)], s2[IDX(a, b, z)], dz[z], vg);
        gu[0][z] = vg[0];
        gu[1][z] = vg[1];
        gu[2][z] = vg[2];
      }
    } else if (active) {
#pragma unroll
      for (int z = 0; z < Q; z++) g[e * Q3 + IDX(a, b, z)] = s0[IDX(a, b, z)] * gu[0][z] + s2[IDX(a, b, z)] * gu[1][z] + dz[z] * gu[2][z];
    }
  }
#undef IDX
}

}  // namespace b200
