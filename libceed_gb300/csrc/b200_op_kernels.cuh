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
// operand) and writes the line back.  The z-direction lines stay in registers across stages.
//
// Gradient: collocated, dX = G_c (B u) with G_c = G B^+ (Q x Q); the transpose applies G_c^T then B^T.
//
// Even-odd contractions (EO = true): the interpolation matrix of a Lagrange basis on Gauss-Lobatto nodes evaluated at
// Gauss points is centro-symmetric (B[Q-1-i][P-1-j] = B[i][j]) and the collocated derivative is centro-antisymmetric,
// so each 1D contraction splits into an even and an odd half on (in[k] +- in[K-1-k]); this removes ~17% (degree 4)
// to ~30% (degree 8) of the multiply-adds, which is what bounds the FP64 kernels on this GPU.  The host checks the
// symmetry before choosing an EO kernel.
//
// Kernel variants:
//   k_op_apply<.., kStageReg>  qdata z-line prefetched into registers at entry (loads in flight during interpolation)
//   k_op_apply<.., kStageSmem> qdata slab of the element copied into shared memory at entry (vector fields reuse it)
//   k_op_apply_pipe            persistent blocks looping over element batches with a two-deep software pipeline:
//                              while batch i is computed, batch i+1's qdata streams into a second shared-memory buffer
//                              (cp.async) and its u values and batch i+2's offsets are loaded into registers.
//   k_op_apply<.., kStageTma>  the block's elements are consecutive, so each qdata component of the block is one
//                              contiguous range: warp 0 issues cp.async.bulk copies at entry (one per element and
//                              component into bank-aligned slabs when elements start on 16 bytes, else one per
//                              component), completing on an mbarrier that the threads wait on (bounded) just before the
//                              pointwise stage, so the copy overlaps the gather and the interpolation without registers
//                              or load instructions.  FP32: coalesced gather and scatter, per-epoch tile layouts.
//   k_op_apply<.., kStageLate> nothing staged: the pointwise stage loads each point's qdata from global memory (after an
//                              L2 prefetch of the block's qdata at entry).
//   k_op_apply_ptma            FP32, one component: persistent blocks looping over element batches with the bulk-copy
//                              staging, the next batch's copies and gathered values in flight during the current one.
//   k_op_apply_3d              "point" mapping: a team of Q^3 threads per element, one thread per output point of
//                              each stage (Q*P*P, Q*Q*P, Q^3, ... threads active), the 1D matrices in shared memory
//                              and the thread's own qdata in registers (one coalesced load per component).
#pragma once

#ifndef __CUDACC_RTC__
#include <cstdint>
#endif

#include "b200_dfloat.cuh"
#include "b200_pointwise.cuh"

namespace b200 {

// kStage3D: point mapping (k_op_apply_3d); kStageTma: the block's qdata slabs arrive by bulk copy (TMA engine)
// kStageLate: nothing is staged; the pointwise stage reads each point's qdata from global memory when it needs it, so the
// kernel holds neither the qdata registers of kStageReg nor the slabs of kStageTma (higher occupancy where those limit it)
// kStagePTma: persistent blocks over element batches, bulk-copy staging one batch ahead (FP32, one component)
enum { kStageReg = 1, kStageSmem = 2, kStagePipe = 3, kStage3D = 4, kStageTma = 5, kStageLate = 6, kStagePTma = 7 };

// Shared-memory layout of an element tile: point (x, y, z) at x + Q*y + tile_plane(Q)*z, three tiles per team
// (tile_buf each), and a team stride that is fixed modulo 32 words.  The plane padding and the team stride residue
// were chosen with a model of this kernel's shared-memory accesses (every stage's line reads and writes, per warp,
// 4-byte words on 32 banks) to minimise the number of wavefronts; e.g. at Q = 6 the model counts 35% fewer than the
// unpadded Q^3 layout, at Q = 4 a factor 2.7 fewer.  Global arrays (qdata, kappa) keep the linear point order.
__host__ __device__ constexpr int tile_plane_pad(int Q) {
  return Q == 3 ? 27 : Q == 4 ? 11 : Q == 5 ? 13 : Q == 6 ? 3 : Q == 7 ? 7 : Q == 8 ? 9 : Q == 9 ? 0 : Q == 10 ? 9 : 0;
}
__host__ __device__ constexpr int tile_team_mod(int Q) {  // team stride modulo 32 (in elements)
  return ((3 * Q * (Q * Q + tile_plane_pad(Q))) + (Q == 3 ? 5 : Q == 4 ? 12 : Q == 5 ? 31 : Q == 6 ? 6 : Q == 7 ? 25 : Q == 8 ? 0
                                                              : Q == 9 ? 6 : Q == 10 ? 30 : 0)) % 32;
}
__host__ __device__ constexpr int tile_plane(int Q) { return Q * Q + tile_plane_pad(Q); }
__host__ __device__ constexpr int tile_buf(int Q) { return Q * tile_plane(Q); }
// Team stride (elements of T) for `extra` elements of staging space after the three tiles.
__host__ __device__ constexpr int tile_team_stride(int Q, int extra) {
  return 3 * tile_buf(Q) + extra + ((tile_team_mod(Q) - (3 * tile_buf(Q) + extra) % 32) % 32 + 32) % 32;
}

// Per-epoch tile layouts.  An epoch is the life of one tile buffer's contents, from the stage that writes it to the
// last stage that reads it; its layout places point (x, y, z) of team `slot` at slot*sg + x*sx + y*sy + z*sz within the
// buffer's region.  Lanes of one warp are consecutive team threads, and each stage's accesses run along one direction
// (x-lines, y-lines, z-lines, or the element's nodes in lexicographic order for the coalesced gather and scatter), so a
// layout can be conflict-free for the writer's direction and the reader's direction together where one fixed layout
// cannot serve all three.  The FP32 bulk-copy kernels (coalesced gather and scatter) use layouts chosen per (Q, epoch)
// by a search over axis orders, paddings and team strides that minimises a model of the shared-memory wavefronts (32
// four-byte banks) of every stage at the default tile, with extents within 12% of Q^3: e.g. at Q = 6 the model counts
// 16% fewer wavefronts than the single padded layout, at Q = 8 32% fewer (measured: 0-4% faster applies; the address
// arithmetic costs registers, which is why the register-staged kernels, limited by occupancy, keep the single layout
// above, as do the FP64 and float-float kernels).
enum { kEpGather = 0, kEpXY, kEpYZ, kEpU, kEpDX, kEpDY, kEpT, kEpZT, kEpYT, kEpScatter, kNumEp };

struct TileLay {
  int sx, sy, sz, sg, ext;  // strides of x, y, z and of the team slot; extent of one team's tile
};

// Epoch order: gather (nodes -> X interpolation), X -> Y interpolation, Y -> Z interpolation, interpolated values ->
// X and Y derivatives, X derivative -> QFunction -> transposed X derivative, the same for Y, transposed X -> Y -> Z
// derivatives, transposed Z -> Y interpolation, transposed Y -> X interpolation, X-line results -> scatter.
__host__ __device__ constexpr TileLay tile_lay_f32(int Q, int ep) {
  constexpr TileLay t[8][kNumEp] = {
      {{1, 3, 9, 27, 27}, {1, 10, 3, 38, 29}, {3, 1, 9, 27, 27}, {1, 3, 9, 27, 27}, {1, 3, 9, 27, 27},
       {3, 1, 9, 27, 27}, {3, 1, 9, 27, 27}, {3, 1, 9, 27, 27}, {1, 10, 3, 38, 29}, {1, 3, 9, 27, 27}},  // Q = 3
      {{1, 4, 17, 67, 67}, {1, 17, 4, 76, 67}, {4, 1, 17, 80, 67}, {1, 4, 18, 80, 70}, {1, 4, 17, 80, 67},
       {4, 1, 17, 80, 67}, {1, 18, 4, 80, 70}, {4, 1, 17, 80, 67}, {1, 17, 4, 76, 67}, {1, 4, 17, 67, 67}},  // Q = 4
      {{5, 25, 1, 132, 125}, {5, 1, 25, 132, 125}, {5, 25, 1, 125, 125}, {26, 1, 5, 153, 129}, {26, 1, 5, 153, 129},
       {5, 1, 25, 125, 125}, {5, 1, 25, 125, 125}, {5, 25, 1, 125, 125}, {5, 1, 25, 132, 125}, {5, 25, 1, 132, 125}},  // Q = 5
      {{6, 1, 37, 221, 221}, {37, 6, 1, 224, 221}, {1, 6, 38, 228, 226}, {37, 1, 6, 228, 221}, {1, 6, 37, 228, 221},
       {1, 6, 38, 228, 226}, {1, 39, 6, 260, 231}, {1, 6, 38, 228, 226}, {37, 6, 1, 224, 221}, {6, 1, 37, 221, 221}},  // Q = 6
      {{1, 7, 49, 358, 343}, {52, 1, 7, 362, 361}, {7, 1, 49, 343, 343}, {1, 52, 7, 369, 361}, {1, 7, 49, 343, 343},
       {7, 1, 49, 343, 343}, {1, 52, 7, 369, 361}, {7, 1, 49, 343, 343}, {52, 1, 7, 362, 361}, {1, 7, 49, 358, 343}},  // Q = 7
      {{1, 71, 8, 561, 561}, {1, 65, 8, 519, 519}, {1, 8, 72, 568, 568}, {67, 1, 8, 533, 533}, {68, 1, 8, 540, 540},
       {1, 8, 72, 568, 568}, {67, 1, 8, 533, 533}, {1, 8, 72, 568, 568}, {1, 65, 8, 519, 519}, {1, 71, 8, 561, 561}},  // Q = 8
      {{84, 1, 9, 753, 753}, {1, 84, 9, 753, 753}, {1, 81, 9, 729, 729}, {1, 9, 81, 729, 729}, {1, 9, 81, 729, 729},
       {1, 9, 81, 729, 729}, {1, 9, 81, 729, 729}, {1, 81, 9, 729, 729}, {1, 84, 9, 753, 753}, {84, 1, 9, 753, 753}},  // Q = 9
      {{100, 1, 10, 1008, 1000}, {1, 113, 10, 1117, 1117}, {1, 10, 106, 1060, 1054}, {1, 113, 10, 1124, 1117},
       {1, 10, 101, 1028, 1009}, {1, 10, 106, 1060, 1054}, {1, 113, 10, 1124, 1117}, {1, 10, 106, 1060, 1054},
       {1, 113, 10, 1117, 1117}, {100, 1, 10, 1008, 1000}},  // Q = 10
  };
  return t[Q - 3][ep];
}

template <typename A, typename B>
struct SameType {
  static constexpr bool value = false;
};
template <typename A>
struct SameType<A, A> {
  static constexpr bool value = true;
};

template <typename T, int Q, int STAGE>
struct TileMap {
  static constexpr bool tuned = SameType<T, float>::value && Q >= 3 && Q <= 10 && STAGE == kStageTma;
  __host__ __device__ static constexpr TileLay lay(int ep) {
    return tuned ? tile_lay_f32(Q, ep) : TileLay{1, Q, tile_plane(Q), 0, tile_buf(Q)};
  }
  __host__ __device__ static constexpr bool same(int e1, int e2) {
    return lay(e1).sx == lay(e2).sx && lay(e1).sy == lay(e2).sy && lay(e1).sz == lay(e2).sz && lay(e1).sg == lay(e2).sg;
  }
  // Values of T in one buffer region of epb teams (tuned layouts; a multiple of 4 so regions start on 16 bytes).
  __host__ __device__ static constexpr int region(int epb) {
    int r = 0;
    for (int ep = 0; ep < kNumEp; ep++) {
      const int v = (epb - 1) * lay(ep).sg + lay(ep).ext;
      r           = v > r ? v : r;
    }
    return (r + 3) / 4 * 4;
  }
};

// The three tile buffers of the block's teams.  `base` is the block's tile area.  Tuned layouts: buffer b's region
// starts at b * bst and the team offset comes from the epoch's layout.  Otherwise a team's three tiles are bst =
// tile_buf(Q) apart and teams `tst` apart.  at() addresses the thread's own team (slot); at_team() another one.
template <typename T, int Q, int STAGE>
struct TileSet {
  using Map = TileMap<T, Q, STAGE>;
  T  *base;
  int bst, slot, tst;
  __host__ __device__ static constexpr bool same(int e1, int e2) { return Map::same(e1, e2); }
  template <int EP>
  __device__ __forceinline__ T &at_team(int buf, int x, int y, int z, int team) const {
    constexpr TileLay L = Map::lay(EP);
    return base[buf * bst + (Map::tuned ? L.sg : tst) * team + L.sx * x + L.sy * y + L.sz * z];
  }
  template <int EP>
  __device__ __forceinline__ T &at(int buf, int x, int y, int z) const {
    return at_team<EP>(buf, x, y, z, slot);
  }
};

// Owner of one line in the stages that work on fewer than Q^2 lines per element: the X interpolation and its transpose
// (x-lines (y, z), y, z < P) and the Y interpolation and its transpose (y-lines (x, z), x < Q, z < P).  Packed form:
// the block's threads take the active lines of all its teams in order (thread t of the block: team t / lines, line
// t % lines), so whole warps are idle in these stages instead of lanes of every warp; otherwise thread (a, b) of team
// `slot` owns line (a, b) when it is active.
struct LineOwner {
  int  u, w, team;  // line coordinates (y, z) for x-lines, (x, z) for y-lines
  bool on;
};
template <int P, int Q, bool PACK>
__device__ __forceinline__ LineOwner x_line_owner(int a, int b, int slot, int epb) {
  if constexpr (PACK) {
    const int t = threadIdx.x, team = t / (P * P), r = t % (P * P);
    return LineOwner{r % P, r / P, team, team < epb};
  } else {
    return LineOwner{a, b, slot, a < P && b < P};
  }
}
template <int P, int Q, bool PACK>
__device__ __forceinline__ LineOwner y_line_owner(int a, int b, int slot, int epb) {
  if constexpr (PACK) {
    const int t = threadIdx.x, team = t / (Q * P), r = t % (Q * P);
    return LineOwner{r % Q, r / Q, team, team < epb};
  } else {
    return LineOwner{a, b, slot, b < P};
  }
}

// Even-odd form of a J x K matrix with parity +1 (centro-symmetric) or -1 (centro-antisymmetric).
template <typename T, int J, int K>
struct EOMat {
  static constexpr int Jh = J / 2, Kh = K / 2;
  T E[Jh * Kh];  // (M[j][k] + M[j][K-1-k]) / 2
  T O[Jh * Kh];  // (M[j][k] - M[j][K-1-k]) / 2
  T C[Jh + 1];   // middle input column M[j][Kh] (K odd)
  T R[Kh + 1];   // middle output row (J odd): even part (parity +1) or odd part (parity -1), then M[Jh][Kh]
};

template <typename T, int P, int Q>
struct OpMats {
  T B[Q * P];  // interp, row-major Q x P
  T G[Q * Q];  // collocated gradient, row-major Q x Q
  EOMat<T, Q, P> Be;   // B   (Q x P), parity +1
  EOMat<T, P, Q> Bte;  // B^T (P x Q), parity +1
  EOMat<T, Q, Q> Ge;   // G   (Q x Q), parity -1
  EOMat<T, Q, Q> Gte;  // G^T (Q x Q), parity -1
};

template <typename T>
struct OpArgs {
  int64_t        num_elem;
  int64_t        comp_stride;  // L-vector component stride
  int            epb;          // elements per block (teams per block)
  int            det;          // 1: write the element result to e_out (deterministic scatter follows)
  const int32_t *offsets;
  const T       *u;
  T             *v;      // L-vector (atomic scatter)
  T             *e_out;  // E-vector [comp][elem][node] (deterministic scatter)
  const T       *qdata;  // [qcomp][elem][qpt]
  const T       *kappa;  // [elem][qpt] or nullptr
  int           *status; // device status word (B200_STATUS_* bits)
  double        *dot;    // persistent FP32 kernel: per-block sums of u . (A u) over its elements, or nullptr
};

template <int QF>
struct QFTraits {
  static constexpr bool grad  = QF == B200_QF_POISSON || QF == B200_QF_VECPOISSON || QF == B200_QF_POISSON_KAPPA;
  static constexpr int  nc    = (QF == B200_QF_VECMASS || QF == B200_QF_VECPOISSON) ? 3 : 1;
  static constexpr int  nqd   = grad ? 6 : 1;
  static constexpr bool kappa = QF == B200_QF_POISSON_KAPPA;
  static constexpr int  nqk   = nqd + (kappa ? 1 : 0);  // staged qdata components, kappa last
};

template <typename T, int P, int Q, int QF, int STAGE>
struct OpShape {
  static constexpr int Q2 = Q * Q, Q3 = Q * Q * Q, P3 = P * P * P;
  // Per-team shared memory in elements of T: three Q^3 tile buffers, plus the qdata slab (smem staging) or two
  // qdata slabs and the element's offsets (pipelined).
  static constexpr int extra     = (STAGE == kStageSmem ? QFTraits<QF>::nqk * Q3 : 0) +
                               (STAGE == kStagePipe ? 2 * QFTraits<QF>::nqk * Q3 + (P3 * 4 + (int)sizeof(T) - 1) / (int)sizeof(T) : 0);
  static constexpr int team_smem = tile_team_stride(Q, extra);
};

// ---- bulk copies (TMA engine) completing on an mbarrier ---------------------------------------------------------------
__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count) : "memory");
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");  // make the initialised barrier visible to the copy engine
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
// dst (shared) and src (global) 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(smem_addr(dst)), "l"(src),
               "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}
// Prefetch [src, src + bytes) from global memory into L2 (src 16-byte aligned, bytes a multiple of 16); no completion.
__device__ __forceinline__ void bulk_prefetch_l2(const void *src, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;\n" ::"l"(src), "r"(bytes) : "memory");
}
// Wait for phase `parity` of the barrier to complete, giving up after a bounded number of polls (each try_wait also
// suspends for a bounded time).  Returns false on give-up.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity, int max_polls = 1 << 22) {
  for (int i = 0; i < max_polls; i++) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Element stride (storage values) of a bulk-copy qdata slab copied element by element: the smallest stride >= Q^3 that
// is a multiple of 16 bytes and that continues the team's point index Q^2 modulo the bank width (32 four-byte banks;
// 8-byte values go in half-warps over 16 bank pairs).  Then a warp whose lanes span two teams reads consecutive banks in
// the pointwise stage instead of two overlapping runs.
template <typename S, int Q>
__host__ __device__ constexpr int tma_elem_stride() {
  constexpr int W = 128 / (int)sizeof(S), A = 16 / (int)sizeof(S);
  if ((Q * Q) % A != 0) return Q * Q * Q;  // no such stride (odd Q: elements are not 16-byte aligned either)
  int sq = Q * Q * Q;
  while (sq % A != 0 || (sq - Q * Q) % W != 0) sq++;
  return sq;
}
// Shared-memory prefix of the bulk-copy staging: an mbarrier (16 bytes) and one slab per staged qdata component of
// epb elements (element stride tma_elem_stride) plus 16 bytes of alignment slack on each side.
template <typename S, int Q>
__host__ __device__ constexpr size_t tma_slab_bytes(int epb) {
  return ((size_t)epb * tma_elem_stride<S, Q>() * sizeof(S) + 32 + 15) / 16 * 16;
}
template <typename S, int Q, int NQK>
__host__ __device__ constexpr size_t tma_prefix_bytes(int epb) {
  return 16 + NQK * tma_slab_bytes<S, Q>(epb);
}

struct NoWait {
  __device__ void operator()() const {}
};
// Per-point hook of op_stages: receives each quadrature point's term of u . (A u) (grad u . D grad u, or u q u).
struct NoDot {
  __device__ void operator()(float) const {}
  __device__ void operator()(double) const {}
};

// out[j] = sum_k M[j*K + k] in[k], j < J
template <typename T, int J, int K>
__device__ __forceinline__ void mat_apply(const T *M, const T (&in)[K], T (&out)[J]) {
#pragma unroll
  for (int j = 0; j < J; j++) {
    Dot<T> s;
    s.first(M[j * K], in[0]);
#pragma unroll
    for (int k = 1; k < K; k++) s.add(M[j * K + k], in[k]);
    out[j] = s.value();
  }
}

// out[k] = sum_j M[j*K + k] in[j], k < K  (transpose of a J x K matrix)
template <typename T, int J, int K>
__device__ __forceinline__ void mat_apply_t(const T *M, const T (&in)[J], T (&out)[K]) {
#pragma unroll
  for (int k = 0; k < K; k++) {
    Dot<T> s;
    s.first(M[k], in[0]);
#pragma unroll
    for (int j = 1; j < J; j++) s.add(M[j * K + k], in[j]);
    out[k] = s.value();
  }
}

// out = M in through the even-odd form (M is J x K with parity PAR).
template <typename T, int J, int K, int PAR>
__device__ __forceinline__ void eo_apply(const EOMat<T, J, K> &M, const T (&in)[K], T (&out)[J]) {
  constexpr int  Jh = J / 2, Kh = K / 2;
  constexpr bool Km = K % 2, Jm = J % 2;
  T              ie[Kh], io[Kh];
#pragma unroll
  for (int k = 0; k < Kh; k++) {
    ie[k] = in[k] + in[K - 1 - k];
    io[k] = in[k] - in[K - 1 - k];
  }
#pragma unroll
  for (int j = 0; j < Jh; j++) {
    Dot<T> de, dd;
    de.first(M.E[j * Kh], ie[0]);
    dd.first(M.O[j * Kh], io[0]);
#pragma unroll
    for (int k = 1; k < Kh; k++) {
      de.add(M.E[j * Kh + k], ie[k]);
      dd.add(M.O[j * Kh + k], io[k]);
    }
    if constexpr (Km) de.add(M.C[j], in[Kh]);
    const T e = de.value(), o = dd.value();
    out[j]         = e + o;
    out[J - 1 - j] = PAR > 0 ? e - o : o - e;
  }
  if constexpr (Jm) {
    Dot<T> r;
    if constexpr (PAR > 0) {
      r.first(M.R[0], ie[0]);
#pragma unroll
      for (int k = 1; k < Kh; k++) r.add(M.R[k], ie[k]);
      if constexpr (Km) r.add(M.R[Kh], in[Kh]);
    } else {
      r.first(M.R[0], io[0]);
#pragma unroll
      for (int k = 1; k < Kh; k++) r.add(M.R[k], io[k]);
    }
    out[Jh] = r.value();
  }
}

template <typename T, int P, int Q, bool EO>
struct Contract {
  static __device__ __forceinline__ void interp(const OpMats<T, P, Q> &M, const T (&in)[P], T (&out)[Q]) {
    if constexpr (EO) eo_apply<T, Q, P, 1>(M.Be, in, out);
    else mat_apply<T, Q, P>(M.B, in, out);
  }
  static __device__ __forceinline__ void interp_t(const OpMats<T, P, Q> &M, const T (&in)[Q], T (&out)[P]) {
    if constexpr (EO) eo_apply<T, P, Q, 1>(M.Bte, in, out);
    else mat_apply_t<T, Q, P>(M.B, in, out);
  }
  static __device__ __forceinline__ void grad(const OpMats<T, P, Q> &M, const T (&in)[Q], T (&out)[Q]) {
    if constexpr (EO) eo_apply<T, Q, Q, -1>(M.Ge, in, out);
    else mat_apply<T, Q, Q>(M.G, in, out);
  }
  static __device__ __forceinline__ void grad_t(const OpMats<T, P, Q> &M, const T (&in)[Q], T (&out)[Q]) {
    if constexpr (EO) eo_apply<T, Q, Q, -1>(M.Gte, in, out);
    else mat_apply_t<T, Q, Q>(M.G, in, out);
  }
};

#define B200_IDX(x, y, z) ((x) + Q * (y) + tile_plane(Q) * (z))  // shared-memory tile position
#define B200_QLIN(x, y, z) ((x) + Q * ((y) + Q * (z)))         // linear point index of global arrays

// The element pipeline from the gathered element values to the x-line owners' output lines.  Thread (a, b) of its team
// owns z-line (a, b) in the Z stages, the derivatives and the QFunction; lx and ly name the lines it owns in the X and
// Y stages.  On entry either (XREG) the x-line owners (lx.on) hold in xin[p] the element value at node (p, lx.u, lx.w)
// of team lx.team, or buffer 0 holds the element values (x, y, z < P) in the layout of epoch kEpGather and every
// thread has passed a barrier after writing them; qd(k, z) returns qdata component k (kappa already applied) at point
// (a, b, z), after qwait() has returned; qafter() runs once all threads are past their last qdata read.  On exit the
// x-line owners hold in out[p] the element result at node (p, lx.u, lx.w) of team lx.team.  Uses the three tile buffers
// of `tl` (each epoch in its own layout) and block-wide barriers.  qdot(t) receives each of the thread's quadrature
// points' terms of u . (A u) = sum over points of (grad u)^T D (grad u) (mass: u q u).
template <typename T, int P, int Q, int QF, bool EO, bool XREG, typename TL, typename QD, typename QW = NoWait, typename QA = NoWait,
          typename QP = NoDot>
__device__ __forceinline__ void op_stages(const TL &tl, const OpMats<T, P, Q> &M, int a, int b, const LineOwner &lx, const LineOwner &ly,
                                          const T (&xin)[P], QD qd, T (&out)[P], QW qwait = QW{}, QA qafter = QA{}, QP qdot = QP{}) {
  using C             = Contract<T, P, Q, EO>;
  constexpr bool GRAD = QFTraits<QF>::grad;
  // ---- X interpolation: lines (y, z) < P, owner lx ------------------------------------------------------------------
  if (lx.on) {
    T in[P], o[Q];
#pragma unroll
    for (int k = 0; k < P; k++) in[k] = XREG ? xin[k] : tl.template at_team<kEpGather>(0, k, lx.u, lx.w, lx.team);
    C::interp(M, in, o);
#pragma unroll
    for (int j = 0; j < Q; j++) tl.template at_team<kEpXY>(1, j, lx.u, lx.w, lx.team) = o[j];
  }
  __syncthreads();
  // ---- Y interpolation: lines (x < Q, z < P), owner ly ------------------------------------------------------------
  if (ly.on) {
    T in[P], o[Q];
#pragma unroll
    for (int k = 0; k < P; k++) in[k] = tl.template at_team<kEpXY>(1, ly.u, k, ly.w, ly.team);
    C::interp(M, in, o);
#pragma unroll
    for (int j = 0; j < Q; j++) tl.template at_team<kEpYZ>(0, ly.u, j, ly.w, ly.team) = o[j];
  }
  __syncthreads();
  // ---- Z interpolation (+ Z derivative): lines (x, y) --------------------------------------------------------------
  T U[Q];
  {
    T in[P];
#pragma unroll
    for (int k = 0; k < P; k++) in[k] = tl.template at<kEpYZ>(0, a, b, k);
    C::interp(M, in, U);
  }
  if constexpr (GRAD) {
    T dz[Q];
#pragma unroll
    for (int j = 0; j < Q; j++) tl.template at<kEpU>(1, a, b, j) = U[j];
    C::grad(M, U, dz);
    __syncthreads();
    // ---- X and Y derivatives of the interpolated values ------------------------------------------------------------
    {
      T in[Q], o[Q];
#pragma unroll
      for (int k = 0; k < Q; k++) in[k] = tl.template at<kEpU>(1, k, a, b);
      C::grad(M, in, o);
#pragma unroll
      for (int j = 0; j < Q; j++) tl.template at<kEpDX>(0, j, a, b) = o[j];
#pragma unroll
      for (int k = 0; k < Q; k++) in[k] = tl.template at<kEpU>(1, a, k, b);
      C::grad(M, in, o);
#pragma unroll
      for (int j = 0; j < Q; j++) tl.template at<kEpDY>(2, a, j, b) = o[j];
    }
    __syncthreads();
    // ---- pointwise QFunction on the z-line (x = a, y = b) ------------------------------------------------------------
    qwait();
#pragma unroll
    for (int z = 0; z < Q; z++) {
      T D[6];
#pragma unroll
      for (int k = 0; k < 6; k++) D[k] = qd(k, z);
      T       vg[3];
      const T gx = tl.template at<kEpDX>(0, a, b, z), gy = tl.template at<kEpDY>(2, a, b, z);
      poisson_point(D, gx, gy, dz[z], vg);
      if constexpr (!SameType<QP, NoDot>::value) qdot(gx * vg[0] + gy * vg[1] + dz[z] * vg[2]);
      tl.template at<kEpDX>(0, a, b, z) = vg[0];
      tl.template at<kEpDY>(2, a, b, z) = vg[1];
      dz[z]                 = vg[2];
    }
    __syncthreads();
    // ---- X derivative, transposed: lines (y, z) --------------------------------------------------------------------
    {
      T in[Q], o[Q];
#pragma unroll
      for (int k = 0; k < Q; k++) in[k] = tl.template at<kEpDX>(0, k, a, b);
      C::grad_t(M, in, o);
#pragma unroll
      for (int j = 0; j < Q; j++) tl.template at<kEpT>(1, j, a, b) = o[j];
    }
    __syncthreads();
    // ---- Y derivative, transposed, accumulated: lines (x, z) ---------------------------------------------------------
    {
      T in[Q], o[Q];
#pragma unroll
      for (int k = 0; k < Q; k++) in[k] = tl.template at<kEpDY>(2, a, k, b);
      C::grad_t(M, in, o);
#pragma unroll
      for (int j = 0; j < Q; j++) tl.template at<kEpT>(1, a, j, b) += o[j];
    }
    __syncthreads();
    // ---- Z derivative transposed + sum, then Z interpolation transposed: lines (x, y) --------------------------------
    {
      T w[Q], o[P];
      C::grad_t(M, dz, w);
#pragma unroll
      for (int j = 0; j < Q; j++) w[j] += tl.template at<kEpT>(1, a, b, j);
      C::interp_t(M, w, o);
#pragma unroll
      for (int p = 0; p < P; p++) tl.template at<kEpZT>(0, a, b, p) = o[p];
    }
  } else {
    // ---- mass: pointwise product on the z-line, then Z interpolation transposed ----------------------------------------
    // With one layout for both epochs each thread reads and rewrites only its own z-line of buffer 0, so no barrier is
    // needed here; otherwise the Z interpolation's reads must finish first.
    T w[Q], o[P];
    qwait();
#pragma unroll
    for (int z = 0; z < Q; z++) {
      w[z] = U[z] * qd(0, z);
      if constexpr (!SameType<QP, NoDot>::value) qdot(U[z] * w[z]);
    }
    C::interp_t(M, w, o);
    if constexpr (!TL::same(kEpYZ, kEpZT)) __syncthreads();
#pragma unroll
    for (int p = 0; p < P; p++) tl.template at<kEpZT>(0, a, b, p) = o[p];
  }
  __syncthreads();
  qafter();  // every thread is past its last qdata read
  // ---- Y interpolation transposed: lines (x < Q, z < P), owner ly ----------------------------------------------------
  if (ly.on) {
    T in[Q], o[P];
#pragma unroll
    for (int k = 0; k < Q; k++) in[k] = tl.template at_team<kEpZT>(0, ly.u, k, ly.w, ly.team);
    C::interp_t(M, in, o);
#pragma unroll
    for (int p = 0; p < P; p++) tl.template at_team<kEpYT>(1, ly.u, p, ly.w, ly.team) = o[p];
  }
  __syncthreads();
  // ---- X interpolation transposed: lines (y, z) < P, owner lx ----------------------------------------------------------
  if (lx.on) {
    T in[Q];
#pragma unroll
    for (int k = 0; k < Q; k++) in[k] = tl.template at_team<kEpYT>(1, k, lx.u, lx.w, lx.team);
    C::interp_t(M, in, out);
  }
}

// Scatter the thread's output line (nodes (p, a, b)) of element e, component c.
template <typename T, int P>
__device__ __forceinline__ void scatter_line(const OpArgs<typename Store<T>::type> &args, int64_t e, int c, const int32_t *off_line, int a, int b,
                                             const T (&out)[P]) {
  using S = typename Store<T>::type;
  constexpr int P3   = P * P * P;
  const int     base = P * (a + P * b);
  if (args.det) {
    S *dst = args.e_out + ((int64_t)c * args.num_elem + e) * P3 + base;
#pragma unroll
    for (int p = 0; p < P; p++) dst[p] = (S)out[p];
  } else {
#pragma unroll
    for (int p = 0; p < P; p++) atomicAdd(&args.v[(int64_t)off_line[p] + c * args.comp_stride], (S)out[p]);
  }
}

template <typename T, int P, int Q, int QF, int STAGE, bool EO>
__global__ void k_op_apply(const OpArgs<typename Store<T>::type> args, const OpMats<T, P, Q> M) {
  using TR         = QFTraits<QF>;
  using SH         = OpShape<T, P, Q, QF, STAGE>;
  constexpr int Q2 = SH::Q2, Q3 = SH::Q3, P3 = SH::P3, NC = TR::nc, NQD = TR::nqd;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int     tid = threadIdx.x % Q2, slot = threadIdx.x / Q2;
  const int     a = tid % Q, b = tid / Q;
  const int64_t e      = (int64_t)blockIdx.x * args.epb + slot;
  const bool    active = e < args.num_elem;
  const int64_t ne     = args.num_elem;
  using S              = typename Store<T>::type;
  constexpr int NQK    = TR::nqk;
  // Bulk-copy staging: [mbarrier][NQK slabs][team tiles]; the other stagings start with the team tiles.
  const size_t       prefix = STAGE == kStageTma ? tma_prefix_bytes<S, Q, NQK>(args.epb) : 0;
  unsigned long long *bar   = reinterpret_cast<unsigned long long *>(smem_raw);
  using TM          = TileMap<T, Q, STAGE>;
  T *const tiles    = reinterpret_cast<T *>(smem_raw + prefix);
  T *const sq       = tiles + slot * SH::team_smem + 3 * tile_buf(Q);  // shared-memory qdata staging (legacy team layout)
  const TileSet<T, Q, STAGE> tl{tiles, TM::tuned ? TM::region(args.epb) : tile_buf(Q), slot, TM::tuned ? 0 : SH::team_smem};

  // ---- qdata staging ------------------------------------------------------------------------------------------------
  // Register staging keeps the loaded storage values (S) and converts at first use, so that the loads stay in flight
  // through the interpolation stages also when T is not the storage type.
  // When T is the storage type kappa multiplies the qdata at load; otherwise it is kept apart and multiplied in T.
  constexpr int  RQ = STAGE == kStageReg ? NQD : 1, RZ = STAGE == kStageReg ? Q : 1;
  constexpr bool KSEP = TR::kappa && !__is_same(S, T);
  S              rq[RQ][RZ];
  S              rk[KSEP ? RZ : 1];
  if constexpr (STAGE == kStageReg) {
#pragma unroll
    for (int z = 0; z < Q; z++) {
      S kap = S(1);
      if constexpr (TR::kappa) kap = active ? args.kappa[e * Q3 + B200_QLIN(a, b, z)] : S(0);
      if constexpr (KSEP) rk[z] = kap;
#pragma unroll
      for (int k = 0; k < NQD; k++) {
        rq[k][z] = active ? args.qdata[((int64_t)k * ne + e) * Q3 + B200_QLIN(a, b, z)] : S(0);
        if constexpr (TR::kappa && !KSEP) rq[k][z] *= kap;
      }
    }
  } else if constexpr (STAGE == kStageSmem) {
    for (int i = tid; i < NQD * Q3; i += Q2) {
      const int k = i / Q3, q = i % Q3;
      sq[i]       = active ? T(args.qdata[((int64_t)k * ne + e) * Q3 + q]) : T(0);
    }
    if constexpr (TR::kappa)
      for (int q = tid; q < Q3; q += Q2) sq[NQD * Q3 + q] = active ? T(args.kappa[e * Q3 + q]) : T(0);
  }
  // Bulk-copy staging: slab k holds component k (kappa last) of the block's elements e0 .. e0 + nb - 1.  When every
  // element's range starts on 16 bytes (Q^3 values of 16-byte multiple size, aligned arrays) each element is copied on
  // its own to a padded element stride (tma_elem_stride: consecutive banks for warps spanning two teams); the lanes of
  // warp 0 share the nqk * nb copies.  Otherwise each component is one copy of the block's contiguous range, widened to
  // the enclosing 16-byte chunks (each chunk holds array data, so it lies on a mapped page); qoff[k] is then the offset,
  // in storage values, of element e0 within slab k.
  const int64_t  e0    = (int64_t)blockIdx.x * args.epb;
  const int      nb    = (int)((ne - e0) < args.epb ? (ne - e0) : args.epb);
  const size_t   slab  = tma_slab_bytes<S, Q>(args.epb);
  constexpr int  SQ    = tma_elem_stride<S, Q>();
  const bool     split = (Q3 * sizeof(S)) % 16 == 0 && (((size_t)args.qdata | (size_t)args.kappa) & 15) == 0;
  const int      estr  = split ? SQ : Q3;  // element stride within a slab
  int            qoff[STAGE == kStageTma ? NQK : 1];
  auto           comp_src = [&](int k, int64_t el) -> const S * {
    return (TR::kappa && k == NQD) ? args.kappa + el * Q3 : args.qdata + ((int64_t)k * ne + el) * Q3;
  };
  if constexpr (STAGE == kStageLate) {
    // Unstaged: at entry the first lanes ask the copy engine to prefetch each qdata component of the block's elements
    // into L2 (widened to 16-byte chunks, as above), so that the pointwise stage's loads find them there.
    if (threadIdx.x < NQK) {
      const S     *src = comp_src(threadIdx.x, e0);
      const size_t lo = (size_t)src & ~(size_t)15, hi = ((size_t)(src + (size_t)nb * Q3) + 15) & ~(size_t)15;
      bulk_prefetch_l2((const void *)lo, (unsigned)(hi - lo));
    }
  }
  if constexpr (STAGE == kStageTma) {
#pragma unroll
    for (int k = 0; k < NQK; k++) qoff[k] = split ? 0 : (int)(((size_t)comp_src(k, e0) & 15) / sizeof(S));
    if (split) {
      if (threadIdx.x < 32) {
        if (threadIdx.x == 0) {
          mbar_init(bar, 1);
          mbar_arrive_expect_tx(bar, (unsigned)(NQK * nb * Q3 * sizeof(S)));
        }
        __syncwarp();
        for (int i = threadIdx.x; i < NQK * nb; i += 32) {
          const int k = i / nb, el = i % nb;
          bulk_copy_g2s(smem_raw + 16 + k * slab + (size_t)el * SQ * sizeof(S), comp_src(k, e0 + el), (unsigned)(Q3 * sizeof(S)), bar);
        }
      }
    } else if (threadIdx.x == 0) {
      mbar_init(bar, 1);
      unsigned total = 0;
      for (int k = 0; k < NQK; k++) {
        const S     *src = comp_src(k, e0);
        const size_t lo = (size_t)src & ~(size_t)15, hi = ((size_t)(src + (size_t)nb * Q3) + 15) & ~(size_t)15;
        total += (unsigned)(hi - lo);
      }
      mbar_arrive_expect_tx(bar, total);
      for (int k = 0; k < NQK; k++) {
        const S     *src = comp_src(k, e0);
        const size_t lo = (size_t)src & ~(size_t)15, hi = ((size_t)(src + (size_t)nb * Q3) + 15) & ~(size_t)15;
        bulk_copy_g2s(smem_raw + 16 + k * slab, (const void *)lo, (unsigned)(hi - lo), bar);
      }
    }
  }
  auto qwait = [&]() {
    if constexpr (STAGE == kStageTma) {
      if (!mbar_wait(bar, 0) && threadIdx.x == 0) atomicOr(args.status, B200_STATUS_COPY_TIMEOUT);
    }
  };
  auto qd = [&](int k, int z) -> T {
    if constexpr (STAGE == kStageLate) {
      const int64_t q = e * Q3 + B200_QLIN(a, b, z);
      if (!active) return T(0);
      if constexpr (TR::kappa) return T(args.qdata[(int64_t)k * ne * Q3 + q]) * T(args.kappa[q]);
      else return T(args.qdata[(int64_t)k * ne * Q3 + q]);
    } else if constexpr (STAGE == kStageReg) {
      if constexpr (KSEP) return T(rq[k][z]) * T(rk[z]);
      else return T(rq[k][z]);
    } else if constexpr (STAGE == kStageTma) {
      const S  *sl  = reinterpret_cast<const S *>(smem_raw + 16);
      const int q   = slot * estr + B200_QLIN(a, b, z);
      const int st  = (int)(slab / sizeof(S));
      if constexpr (TR::kappa) return T(sl[k * st + qoff[k] + q]) * T(sl[NQD * st + qoff[NQD] + q]);
      else return T(sl[k * st + qoff[k] + q]);
    } else {
      const int q = B200_QLIN(a, b, z);
      if constexpr (TR::kappa) return sq[k * Q3 + q] * sq[NQD * Q3 + q];
      else return sq[k * Q3 + q];
    }
  };

  // Coalesced gather and scatter (FP32, bulk-copy staging): team thread tid handles the element's nodes i = tid + r Q^2
  // in lexicographic order, so a warp's loads and atomics touch runs of consecutive nodes; the values pass through
  // shared memory on the way to and from the x-line owners.  This pays where the L1 data pipe is the bound (the FP32
  // kernels); the FP64 and float-float kernels, bound by their arithmetic, keep the other form: thread (a, b),
  // a, b < P, gathers and later scatters the element's x-line of nodes (p, a, b), which feeds the X interpolation from
  // registers.  Either way the thread's offsets stay in registers from the gather to the scatter.
  // The X and Y stages take packed line owners in the kernels with the single tile layout (the per-epoch layouts were
  // chosen for the thread (a, b) owners).
  constexpr bool CG = STAGE == kStageTma && __is_same(T, float);
  constexpr bool PACK = !TM::tuned;
  constexpr int  PU = (P3 + Q2 - 1) / Q2;  // nodes per thread in the coalesced form
  const LineOwner lx = x_line_owner<P, Q, PACK>(a, b, slot, args.epb), ly = y_line_owner<P, Q, PACK>(a, b, slot, args.epb);
  const int64_t   ex = e0 + lx.team;  // element of the thread's x-line
  const bool      xact = lx.on && ex < ne;
  int32_t         off_line[CG ? PU : P];
  if constexpr (CG) {
#pragma unroll
    for (int r = 0; r < PU; r++) off_line[r] = (active && tid + r * Q2 < P3) ? args.offsets[e * P3 + tid + r * Q2] : 0;
  } else {
#pragma unroll
    for (int p = 0; p < P; p++) off_line[p] = xact ? args.offsets[ex * P3 + P * (lx.u + P * lx.w) + p] : 0;
  }

  // The barrier at the top of each later component protects the tiles still being read by the previous one.
#pragma unroll 1
  for (int c = 0; c < NC; c++) {
    if (c > 0) __syncthreads();
    T xin[P], out[P];
    if constexpr (CG) {
#pragma unroll
      for (int r = 0; r < PU; r++) {
        const int i = tid + r * Q2;
        if (i < P3) tl.template at<kEpGather>(0, i % P, (i / P) % P, i / (P * P)) = active ? T(args.u[(int64_t)off_line[r] + c * args.comp_stride]) : T(0);
      }
      __syncthreads();
      if (c == 0) op_stages<T, P, Q, QF, EO, false>(tl, M, a, b, lx, ly, xin, qd, out, qwait);
      else op_stages<T, P, Q, QF, EO, false>(tl, M, a, b, lx, ly, xin, qd, out);
      // Buffer 0 was last read by the Y interpolation (transposed), before the barrier that preceded the X stage.
      if (lx.on) {
#pragma unroll
        for (int p = 0; p < P; p++) tl.template at_team<kEpScatter>(0, p, lx.u, lx.w, lx.team) = out[p];
      }
      __syncthreads();
      if (active) {
        using S = typename Store<T>::type;
#pragma unroll
        for (int r = 0; r < PU; r++) {
          const int i = tid + r * Q2;
          if (i < P3) {
            const T val = tl.template at<kEpScatter>(0, i % P, (i / P) % P, i / (P * P));
            if (args.det) args.e_out[((int64_t)c * ne + e) * P3 + i] = (S)val;
            else atomicAdd(&args.v[(int64_t)off_line[r] + c * args.comp_stride], (S)val);
          }
        }
      }
    } else {
#pragma unroll
      for (int p = 0; p < P; p++) xin[p] = xact ? T(args.u[(int64_t)off_line[p] + c * args.comp_stride]) : T(0);
      if (c == 0) op_stages<T, P, Q, QF, EO, true>(tl, M, a, b, lx, ly, xin, qd, out, qwait);
      else op_stages<T, P, Q, QF, EO, true>(tl, M, a, b, lx, ly, xin, qd, out);
      if (xact) scatter_line<T, P>(args, ex, c, off_line, lx.u, lx.w, out);
    }
  }
}

// Persistent form of the FP32 bulk-copy kernel (one component).  Block i handles element batches i, i + gridDim.x, ...
// with the same stages, layouts and coalesced gather and scatter as k_op_apply<float, ..., kStageTma>, and works one
// batch ahead: while batch j is computed, the values of batch j + 1 are loaded into registers (their offsets were loaded
// one batch earlier still), and once every thread is past its last qdata read of batch j the bulk copies of batch j + 1's
// qdata are issued into the same slabs, completing on the same mbarrier (phase parity alternating with the batch count).
// Every copy issued is waited for, so none is in flight when a block exits.
// DOT: also write to args.dot[blockIdx.x] the block's share of u . (A u), summed per thread in float-float over the
// quadrature points of its active elements (in two floats per thread after the tile buffers) and then per block in
// FP64, in a fixed order (a CG step's p . A p without a
// second pass over the vectors; exact for the assembled operator, since u . (A u) = sum over elements of u_e . (A_e u_e)).
template <typename T, int P, int Q, int QF, bool EO, bool DOT>
__device__ __forceinline__ void op_apply_ptma(const OpArgs<typename Store<T>::type> &args, const OpMats<T, P, Q> &M) {
  static_assert(SameType<T, float>::value && QFTraits<QF>::nc == 1, "the persistent bulk-copy kernel is FP32, one component");
  using TR         = QFTraits<QF>;
  using TM         = TileMap<T, Q, kStageTma>;
  constexpr int Q2 = Q * Q, Q3 = Q * Q * Q, P3 = P * P * P, NQD = TR::nqd, NQK = TR::nqk;
  constexpr int PU = (P3 + Q2 - 1) / Q2;  // nodes per thread in the coalesced gather and scatter
  using S          = T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int     tid = threadIdx.x % Q2, slot = threadIdx.x / Q2;
  const int     a = tid % Q, b = tid / Q;
  const int64_t ne     = args.num_elem;
  const int64_t nbatch = (ne + args.epb - 1) / args.epb;
  const size_t  prefix = tma_prefix_bytes<S, Q, NQK>(args.epb);
  const size_t  slab   = tma_slab_bytes<S, Q>(args.epb);
  constexpr int SQ     = tma_elem_stride<S, Q>();
  unsigned long long *bar = reinterpret_cast<unsigned long long *>(smem_raw);
  T *const             tiles = reinterpret_cast<T *>(smem_raw + prefix);
  const TileSet<T, Q, kStageTma> tl{tiles, TM::region(args.epb), slot, 0};
  const LineOwner lx = x_line_owner<P, Q, false>(a, b, slot, args.epb), ly = y_line_owner<P, Q, false>(a, b, slot, args.epb);
  const bool      split = (Q3 * sizeof(S)) % 16 == 0 && (((size_t)args.qdata | (size_t)args.kappa) & 15) == 0;
  const int       estr  = split ? SQ : Q3;
  auto comp_src = [&](int k, int64_t el) -> const S * {
    return (TR::kappa && k == NQD) ? args.kappa + el * Q3 : args.qdata + ((int64_t)k * ne + el) * Q3;
  };
  // Bulk copies of one batch's qdata (warp 0; lane 0 arms the barrier for the batch's bytes first).
  auto issue = [&](int64_t batch) {
    if (threadIdx.x >= 32) return;
    // The slabs were last read by the threads (generic proxy) before a barrier; order those reads before the copy
    // engine's writes (async proxy).
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    const int64_t e0 = batch * args.epb;
    const int     nb = (int)((ne - e0) < args.epb ? (ne - e0) : args.epb);
    if (split) {
      if (threadIdx.x == 0) mbar_arrive_expect_tx(bar, (unsigned)(NQK * nb * Q3 * sizeof(S)));
      __syncwarp();
      for (int i = threadIdx.x; i < NQK * nb; i += 32) {
        const int k = i / nb, el = i % nb;
        bulk_copy_g2s(smem_raw + 16 + k * slab + (size_t)el * SQ * sizeof(S), comp_src(k, e0 + el), (unsigned)(Q3 * sizeof(S)), bar);
      }
    } else if (threadIdx.x == 0) {
      unsigned total = 0;
      for (int k = 0; k < NQK; k++) {
        const S     *src = comp_src(k, e0);
        const size_t lo = (size_t)src & ~(size_t)15, hi = ((size_t)(src + (size_t)nb * Q3) + 15) & ~(size_t)15;
        total += (unsigned)(hi - lo);
      }
      mbar_arrive_expect_tx(bar, total);
      for (int k = 0; k < NQK; k++) {
        const S     *src = comp_src(k, e0);
        const size_t lo = (size_t)src & ~(size_t)15, hi = ((size_t)(src + (size_t)nb * Q3) + 15) & ~(size_t)15;
        bulk_copy_g2s(smem_raw + 16 + k * slab, (const void *)lo, (unsigned)(hi - lo), bar);
      }
    }
  };
  auto load_offsets = [&](int64_t batch, int32_t (&o)[PU]) {
    const int64_t e = batch * args.epb + slot;
#pragma unroll
    for (int r = 0; r < PU; r++) o[r] = (batch < nbatch && e < ne && tid + r * Q2 < P3) ? args.offsets[e * P3 + tid + r * Q2] : 0;
  };
  auto load_u = [&](int64_t batch, const int32_t (&o)[PU], T (&uv)[PU]) {
    const int64_t e = batch * args.epb + slot;
#pragma unroll
    for (int r = 0; r < PU; r++) uv[r] = (batch < nbatch && e < ne && tid + r * Q2 < P3) ? args.u[o[r]] : T(0);
  };

  int64_t batch = blockIdx.x;
  if (batch >= nbatch) {
    if (DOT && threadIdx.x == 0) args.dot[blockIdx.x] = 0.0;
    return;
  }
  // DOT: the running sums (registers held across the loop spill at 64 per thread); each thread only touches its own.
  auto dot_slot = [&]() -> float * { return reinterpret_cast<float *>(tiles + 3 * TM::region(args.epb)) + 2 * threadIdx.x; };
  if (DOT) dot_slot()[0] = dot_slot()[1] = 0.f;
  if (threadIdx.x == 0) mbar_init(bar, 1);
  __syncthreads();
  issue(batch);
  int32_t o_cur[PU], o_nxt[PU], o_nn[PU];
  T       u_cur[PU], u_nxt[PU];
  load_offsets(batch, o_cur);
  load_u(batch, o_cur, u_cur);
  load_offsets(batch + gridDim.x, o_nxt);
  unsigned parity = 0;
#pragma unroll 1
  for (; batch < nbatch; batch += gridDim.x, parity ^= 1) {
    const int64_t e0 = batch * args.epb, e = e0 + slot;
    const bool    active = e < ne;
    const int64_t next = batch + gridDim.x;
    __syncthreads();  // the previous batch's scatter reads of buffer 0 are done
#pragma unroll
    for (int r = 0; r < PU; r++) {
      const int i = tid + r * Q2;
      if (i < P3) tl.template at<kEpGather>(0, i % P, (i / P) % P, i / (P * P)) = u_cur[r];
    }
    // The next batch's values and the offsets of the one after: in flight while this batch is computed.
    load_u(next, o_nxt, u_nxt);
    load_offsets(next + gridDim.x, o_nn);
    __syncthreads();
    int qoff[NQK];
#pragma unroll
    for (int k = 0; k < NQK; k++) qoff[k] = split ? 0 : (int)(((size_t)comp_src(k, e0) & 15) / sizeof(S));
    auto qwait = [&]() {
      if (!mbar_wait(bar, parity) && threadIdx.x == 0) atomicOr(args.status, B200_STATUS_COPY_TIMEOUT);
    };
    auto qafter = [&]() {
      if (next < nbatch) issue(next);
    };
    auto qd = [&](int k, int z) -> T {
      const S  *sl = reinterpret_cast<const S *>(smem_raw + 16);
      const int q  = slot * estr + B200_QLIN(a, b, z);
      const int st = (int)(slab / sizeof(S));
      if constexpr (TR::kappa) return T(sl[k * st + qoff[k] + q]) * T(sl[NQD * st + qoff[NQD] + q]);
      else return T(sl[k * st + qoff[k] + q]);
    };
    T none[P], out[P];
    T pts = T(0);  // DOT: this batch's points
    if constexpr (DOT) {
      auto qdot = [&](T t) { pts += t; };
      op_stages<T, P, Q, QF, EO, false>(tl, M, a, b, lx, ly, none, qd, out, qwait, qafter, qdot);
    } else {
      op_stages<T, P, Q, QF, EO, false>(tl, M, a, b, lx, ly, none, qd, out, qwait, qafter);
    }
    // Buffer 0 was last read by the Y interpolation (transposed), before the barrier that preceded the X stage.
    if (lx.on) {
#pragma unroll
      for (int p = 0; p < P; p++) tl.template at_team<kEpScatter>(0, p, lx.u, lx.w, lx.team) = out[p];
    }
    __syncthreads();
    if (active) {
#pragma unroll
      for (int r = 0; r < PU; r++) {
        const int i = tid + r * Q2;
        if (i < P3) {
          const T val = tl.template at<kEpScatter>(0, i % P, (i / P) % P, i / (P * P));
          if (args.det) args.e_out[e * P3 + i] = (S)val;
          else atomicAdd(&args.v[o_cur[r]], (S)val);
        }
      }
    }
#pragma unroll
    for (int r = 0; r < PU; r++) {
      o_cur[r] = o_nxt[r];
      o_nxt[r] = o_nn[r];
      u_cur[r] = u_nxt[r];
    }
    if (DOT && active) {  // inactive teams hold stale qdata: their sum is dropped
      float *sl = dot_slot();
      F2Acc  acc;
      acc.hi = sl[0], acc.lo = sl[1];
      acc.add(pts);
      sl[0] = acc.hi, sl[1] = acc.lo;
    }
  }
  if constexpr (DOT) {
    // Block sum through the (now free) tile buffers: thread t < 32 adds entries t, t + 32, ... (only thread t touches
    // entry t), then thread 0 adds those 32.
    double *red = reinterpret_cast<double *>(tiles);
    F2Acc   acc;
    acc.hi = dot_slot()[0], acc.lo = dot_slot()[1];
    __syncthreads();
    red[threadIdx.x] = acc.value();
    __syncthreads();
    if (threadIdx.x < 32) {
      double t = 0.0;
      for (int i = threadIdx.x; i < (int)blockDim.x; i += 32) t += red[i];
      red[threadIdx.x] = t;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int i = 0; i < 32 && i < (int)blockDim.x; i++) t += red[i];
      args.dot[blockIdx.x] = t;
    }
  }
}

template <typename T, int P, int Q, int QF, bool EO, bool DOT>
__global__ void k_op_apply_ptma(const OpArgs<typename Store<T>::type> args, const OpMats<T, P, Q> M) {
  op_apply_ptma<T, P, Q, QF, EO, DOT>(args, M);
}
// The same kernel capped at 64 registers, used at P = 5: one more block resides per SM (measured: +3.5 % at degree 4;
// at higher degrees the cap costs more than it gains).
template <typename T, int P, int Q, int QF, bool EO, bool DOT>
__global__ void __maxnreg__(64) k_op_apply_ptma_r64(const OpArgs<typename Store<T>::type> args, const OpMats<T, P, Q> M) {
  op_apply_ptma<T, P, Q, QF, EO, DOT>(args, M);
}

// Asynchronous global -> shared copy of one 4- or 8-byte value (completes at cp.async.wait_group).
template <typename T>
__device__ __forceinline__ void cp_async_scalar(T *dst, const T *src) {
  const unsigned saddr = (unsigned)__cvta_generic_to_shared(dst);
  if constexpr (sizeof(T) == 8) asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(saddr), "l"(src) : "memory");
  else asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(saddr), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Persistent, software-pipelined variant (one component; even-odd contractions).  Block i handles element batches
// i, i + gridDim.x, ...; a batch is `epb` consecutive elements, one per team.  Per team: tiles s0..s2, two qdata
// slabs (qbuf[2][nqk * Q^3]) filled by cp.async one batch ahead, and the batch's offsets (soff) for the scatter.
template <typename T, int P, int Q, int QF>
__global__ void k_op_apply_pipe(const OpArgs<typename Store<T>::type> args, const OpMats<T, P, Q> M) {
  static_assert(sizeof(typename Store<T>::type) == sizeof(T) && !__is_same(T, dfloat), "the pipelined kernel stages storage values as T");
  using TR         = QFTraits<QF>;
  using SH         = OpShape<T, P, Q, QF, kStagePipe>;
  constexpr int Q2 = SH::Q2, Q3 = SH::Q3, P3 = SH::P3, NQD = TR::nqd, NQK = TR::nqk;
  constexpr int PU = (P3 + Q2 - 1) / Q2;  // gathered values per thread
  static_assert(TR::nc == 1, "the pipelined kernel handles one component");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int     tid = threadIdx.x % Q2, slot = threadIdx.x / Q2;
  const int     a = tid % Q, b = tid / Q;
  const int64_t ne     = args.num_elem;
  const int64_t nbatch = (ne + args.epb - 1) / args.epb;
  T            *s0 = reinterpret_cast<T *>(smem_raw) + slot * SH::team_smem, *s1 = s0 + tile_buf(Q), *s2 = s1 + tile_buf(Q);
  T            *qbuf[2] = {s2 + tile_buf(Q), s2 + tile_buf(Q) + NQK * Q3};
  int32_t      *soff    = reinterpret_cast<int32_t *>(s2 + tile_buf(Q) + 2 * NQK * Q3);

  auto elem_of      = [&](int64_t batch) -> int64_t { return batch * args.epb + slot; };
  auto load_offsets = [&](int64_t batch, int32_t (&o)[PU]) {
    const int64_t e = elem_of(batch);
#pragma unroll
    for (int r = 0; r < PU; r++) {
      const int i = tid + r * Q2;
      o[r]        = (batch < nbatch && e < ne && i < P3) ? args.offsets[e * P3 + i] : 0;
    }
  };
  auto load_u = [&](int64_t batch, const int32_t (&o)[PU], T (&uv)[PU]) {
    const int64_t e = elem_of(batch);
#pragma unroll
    for (int r = 0; r < PU; r++) {
      const int i = tid + r * Q2;
      uv[r]       = (batch < nbatch && e < ne && i < P3) ? args.u[o[r]] : T(0);
    }
  };
  auto stage_qdata = [&](int64_t batch, T *dst) {
    const int64_t e = elem_of(batch);
    if (batch < nbatch && e < ne) {
      for (int i = tid; i < NQK * Q3; i += Q2) {
        const int k = i / Q3, q = i % Q3;
        const T  *src = (TR::kappa && k == NQD) ? args.kappa + e * Q3 + q : args.qdata + ((int64_t)k * ne + e) * Q3 + q;
        cp_async_scalar(dst + i, src);
      }
    }
    cp_async_commit();
  };

  int64_t batch = blockIdx.x;
  int32_t o_cur[PU], o_next[PU];
  T       u_cur[PU];
  // Prologue: the first batch's offsets and u, its qdata in flight, and the next batch's offsets.
  load_offsets(batch, o_cur);
  load_u(batch, o_cur, u_cur);
  stage_qdata(batch, qbuf[0]);
  load_offsets(batch + gridDim.x, o_next);
  int buf = 0;
#pragma unroll 1
  for (; batch < nbatch; batch += gridDim.x) {
    const int64_t e      = elem_of(batch);
    const bool    active = e < ne;
    __syncthreads();  // the previous batch's last reads of s0, s1 and soff are done
#pragma unroll
    for (int r = 0; r < PU; r++) {
      const int i = tid + r * Q2;
      if (i < P3) {
        const int x = i % P, y = (i / P) % P, z = i / (P * P);
        s0[B200_IDX(x, y, z)] = u_cur[r];
        soff[i]               = o_cur[r];
      }
    }
    // Issue the next batch's loads; they complete while this batch is computed.
    const int64_t nb = batch + gridDim.x;
#pragma unroll
    for (int r = 0; r < PU; r++) o_cur[r] = o_next[r];
    load_u(nb, o_cur, u_cur);
    load_offsets(nb + gridDim.x, o_next);
    stage_qdata(nb, qbuf[buf ^ 1]);
    cp_async_wait<1>();  // this batch's qdata group has landed (the next one may still be in flight)
    __syncthreads();
    const T *sq = qbuf[buf];
    auto     qd = [&](int k, int z) -> T {
      const int q = B200_QLIN(a, b, z);
      if constexpr (TR::kappa) return sq[k * Q3 + q] * sq[NQD * Q3 + q];
      else return sq[k * Q3 + q];
    };
    T out[P], none[P];
    const LineOwner lx = x_line_owner<P, Q, false>(a, b, slot, args.epb), ly = y_line_owner<P, Q, false>(a, b, slot, args.epb);
    op_stages<T, P, Q, QF, true, false>(TileSet<T, Q, kStagePipe>{reinterpret_cast<T *>(smem_raw), tile_buf(Q), slot, SH::team_smem}, M, a, b, lx, ly,
                                        none, qd, out);
    if (a < P && b < P && active) scatter_line<T, P>(args, e, 0, soff + P * (a + P * b), a, b, out);
    buf ^= 1;
  }
  cp_async_wait<0>();
}

// Shared memory of the point-mapped kernel: the 1D matrices (B, then G_c), padded to 32 elements, then one team of
// three tiles per element.
template <typename T, int P, int Q>
struct Op3DShape {
  static constexpr int mats = (Q * P + Q * Q + 31) / 32 * 32;
  static constexpr int team = tile_team_stride(Q, 0);
};

// Point ("3D") thread mapping.  Team thread t is point (x, y, z) = (t % Q, t / Q % Q, t / Q^2) of the element's Q^3
// grid; each stage of the sum factorization lets the first (outputs of the stage) threads compute one output each as
// a length-P or length-Q dot product over a shared tile.  Same stages and result as k_op_apply (general, not even-odd
// contractions); every thread reads its own point's qdata once.
template <typename T, int P, int Q, int QF>
__global__ void k_op_apply_3d(const OpArgs<typename Store<T>::type> args, const OpMats<T, P, Q> M) {
  using TR         = QFTraits<QF>;
  using SH         = Op3DShape<T, P, Q>;
  constexpr int Q2 = Q * Q, Q3 = Q * Q * Q, P2 = P * P, P3 = P * P * P, NC = TR::nc, NQD = TR::nqd;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T            *sB = reinterpret_cast<T *>(smem_raw), *sG = sB + Q * P;
  const int     t = threadIdx.x % Q3, slot = threadIdx.x / Q3;
  const int64_t e      = (int64_t)blockIdx.x * args.epb + slot;
  const bool    active = e < args.num_elem;
  const int64_t ne     = args.num_elem;
  T            *s0 = sB + SH::mats + slot * SH::team, *s1 = s0 + tile_buf(Q), *s2 = s1 + tile_buf(Q);
  for (int i = threadIdx.x; i < Q * P; i += blockDim.x) sB[i] = M.B[i];
  for (int i = threadIdx.x; i < Q * Q; i += blockDim.x) sG[i] = M.G[i];
  const int x = t % Q, y = (t / Q) % Q, z = t / Q2;
  T         D[NQD];
  {
    T kap = T(1);
    if constexpr (TR::kappa) kap = active ? T(args.kappa[e * Q3 + t]) : T(0);
#pragma unroll
    for (int k = 0; k < NQD; k++) D[k] = active ? T(args.qdata[((int64_t)k * ne + e) * Q3 + t]) * kap : T(0);
  }
  const int32_t my_off = (active && t < P3) ? args.offsets[e * P3 + t] : 0;

#pragma unroll 1
  for (int c = 0; c < NC; c++) {
    __syncthreads();  // matrices in place (c = 0), tiles free again (c > 0)
    if (t < P3) s0[B200_IDX(t % P, (t / P) % P, t / P2)] = active ? T(args.u[(int64_t)my_off + c * args.comp_stride]) : T(0);
    __syncthreads();
    if (t < Q * P2) {  // X interpolation: (i < Q, j < P, k < P)
      const int i = t % Q, j = (t / Q) % P, k = t / (Q * P);
      Dot<T>    s;
      s.first(sB[i * P], s0[B200_IDX(0, j, k)]);
#pragma unroll
      for (int m = 1; m < P; m++) s.add(sB[i * P + m], s0[B200_IDX(m, j, k)]);
      s1[B200_IDX(i, j, k)] = s.value();
    }
    __syncthreads();
    if (t < Q2 * P) {  // Y interpolation: (i < Q, j < Q, k < P)
      const int i = t % Q, j = (t / Q) % Q, k = t / Q2;
      Dot<T>    s;
      s.first(sB[j * P], s1[B200_IDX(i, 0, k)]);
#pragma unroll
      for (int m = 1; m < P; m++) s.add(sB[j * P + m], s1[B200_IDX(i, m, k)]);
      s0[B200_IDX(i, j, k)] = s.value();
    }
    __syncthreads();
    T U;  // Z interpolation: every point
    {
      Dot<T> s;
      s.first(sB[z * P], s0[B200_IDX(x, y, 0)]);
#pragma unroll
      for (int m = 1; m < P; m++) s.add(sB[z * P + m], s0[B200_IDX(x, y, m)]);
      U = s.value();
    }
    T w;
    if constexpr (TR::grad) {
      s1[B200_IDX(x, y, z)] = U;
      __syncthreads();
      Dot<T> d0, d1, d2;
      d0.first(sG[x * Q], s1[B200_IDX(0, y, z)]);
      d1.first(sG[y * Q], s1[B200_IDX(x, 0, z)]);
      d2.first(sG[z * Q], s1[B200_IDX(x, y, 0)]);
#pragma unroll
      for (int m = 1; m < Q; m++) {
        d0.add(sG[x * Q + m], s1[B200_IDX(m, y, z)]);
        d1.add(sG[y * Q + m], s1[B200_IDX(x, m, z)]);
        d2.add(sG[z * Q + m], s1[B200_IDX(x, y, m)]);
      }
      T vg[3];
      poisson_point(D, d0.value(), d1.value(), d2.value(), vg);
      __syncthreads();
      s0[B200_IDX(x, y, z)] = vg[0];
      s1[B200_IDX(x, y, z)] = vg[1];
      s2[B200_IDX(x, y, z)] = vg[2];
      __syncthreads();
      Dot<T> dw;
      dw.first(sG[x], s0[B200_IDX(0, y, z)]);
      dw.add(sG[y], s1[B200_IDX(x, 0, z)]);
      dw.add(sG[z], s2[B200_IDX(x, y, 0)]);
#pragma unroll
      for (int m = 1; m < Q; m++) {
        dw.add(sG[m * Q + x], s0[B200_IDX(m, y, z)]);
        dw.add(sG[m * Q + y], s1[B200_IDX(x, m, z)]);
        dw.add(sG[m * Q + z], s2[B200_IDX(x, y, m)]);
      }
      w = dw.value();
    } else {
      w = U * D[0];
    }
    __syncthreads();
    s0[B200_IDX(x, y, z)] = w;
    __syncthreads();
    if (t < Q2 * P) {  // Z interpolation transposed: (i < Q, j < Q, k < P)
      const int i = t % Q, j = (t / Q) % Q, k = t / Q2;
      Dot<T>    s;
      s.first(sB[k], s0[B200_IDX(i, j, 0)]);
#pragma unroll
      for (int m = 1; m < Q; m++) s.add(sB[m * P + k], s0[B200_IDX(i, j, m)]);
      s1[B200_IDX(i, j, k)] = s.value();
    }
    __syncthreads();
    if (t < Q * P2) {  // Y interpolation transposed: (i < Q, j < P, k < P)
      const int i = t % Q, j = (t / Q) % P, k = t / (Q * P);
      Dot<T>    s;
      s.first(sB[j], s1[B200_IDX(i, 0, k)]);
#pragma unroll
      for (int m = 1; m < Q; m++) s.add(sB[m * P + j], s1[B200_IDX(i, m, k)]);
      s0[B200_IDX(i, j, k)] = s.value();
    }
    __syncthreads();
    if (t < P3 && active) {  // X interpolation transposed and scatter: node (i, j, k) = t
      const int i = t % P, j = (t / P) % P, k = t / P2;
      Dot<T>    s;
      s.first(sB[i], s0[B200_IDX(0, j, k)]);
#pragma unroll
      for (int m = 1; m < Q; m++) s.add(sB[m * P + i], s0[B200_IDX(m, j, k)]);
      using S = typename Store<T>::type;
      if (args.det) args.e_out[((int64_t)c * ne + e) * P3 + t] = (S)s.value();
      else atomicAdd(&args.v[(int64_t)my_off + c * args.comp_stride], (S)s.value());
    }
  }
}

// Gradient of the kappa-weighted diffusion with respect to kappa: g[e][q] = grad(w)_q . D_q grad(u)_q, both gradients
// recomputed from the L-vectors (no stored E-vectors).
template <typename T, int P, int Q>
__global__ void k_kappa_grad(const OpArgs<typename Store<T>::type> args, const T *__restrict__ w_vec, T *__restrict__ g, const OpMats<T, P, Q> M) {
  using C          = Contract<T, P, Q, false>;
  constexpr int Q2 = Q * Q, Q3 = Q * Q * Q, P3 = P * P * P;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int     tid = threadIdx.x % Q2, slot = threadIdx.x / Q2;
  const int     a = tid % Q, b = tid / Q;
  const int64_t e      = (int64_t)blockIdx.x * args.epb + slot;
  const bool    active = e < args.num_elem;
  const int64_t ne     = args.num_elem;
  T *s0 = reinterpret_cast<T *>(smem_raw) + slot * tile_team_stride(Q, 0), *s1 = s0 + tile_buf(Q), *s2 = s1 + tile_buf(Q);
  T  gu[3][Q];
#pragma unroll 1
  for (int pass = 0; pass < 2; pass++) {
    const T *src = pass == 0 ? args.u : w_vec;
    if (pass) __syncthreads();
    for (int i = tid; i < P3; i += Q2) {
      const int x = i % P, y = (i / P) % P, z = i / (P * P);
      s0[B200_IDX(x, y, z)] = active ? src[args.offsets[e * P3 + i]] : T(0);
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
    if (pass == 0) {
#pragma unroll
      for (int z = 0; z < Q; z++) {
        T D[6];
#pragma unroll
        for (int k = 0; k < 6; k++) D[k] = active ? args.qdata[((int64_t)k * ne + e) * Q3 + B200_QLIN(a, b, z)] : T(0);
        T vg[3];
        poisson_point(D, s0[B200_IDX(a, b, z)], s2[B200_IDX(a, b, z)], dz[z], vg);
        gu[0][z] = vg[0];
        gu[1][z] = vg[1];
        gu[2][z] = vg[2];
      }
    } else if (active) {
#pragma unroll
      for (int z = 0; z < Q; z++)
        g[e * Q3 + B200_QLIN(a, b, z)] = s0[B200_IDX(a, b, z)] * gu[0][z] + s2[B200_IDX(a, b, z)] * gu[1][z] + dz[z] * gu[2][z];
    }
  }
}

#undef B200_IDX
#undef B200_QLIN

}  // namespace b200
