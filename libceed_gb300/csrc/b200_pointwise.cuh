// Pointwise bodies of the gallery QFunctions on this path, one quadrature point per call.
// Voigt order of the symmetric 3x3 geometric factor: index 0..5 = xx, yy, zz, yz, xz, xy, i.e. the matrix
//   [0 5 4]
//   [5 1 3]
//   [4 3 2]
// as in include/ceed/jit-source/gallery/ceed-poisson3dbuild.h and ceed-poisson3dapply.h.
#pragma once

#include "b200_dfloat.cuh"

namespace b200 {

// vg_j = sum_i ug_i D_ij  (Poisson3DApply), accumulated left to right like the gallery source.
template <typename T>
__device__ __forceinline__ void poisson_point(const T D[6], T gx, T gy, T gz, T vg[3]) {
  vg[0] = mad(gz, D[4], mad(gy, D[5], gx * D[0]));
  vg[1] = mad(gz, D[3], mad(gy, D[1], gx * D[5]));
  vg[2] = mad(gz, D[2], mad(gy, D[3], gx * D[4]));
}

// qdata = w * det(J)  (Mass3DBuild); J[d][c] = d x_c / d xi_d.
__device__ __forceinline__ double mass3d_build_point(const double J[3][3], double w) {
  return (J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
          J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0])) *
         w;
}

// qdata = w / det(J) * adj(J) adj(J)^T in Voigt order  (Poisson3DBuild).
__device__ __forceinline__ void poisson3d_build_point(const double J[3][3], double w, double qd[6]) {
  double A[3][3];
  for (int j = 0; j < 3; j++)
    for (int k = 0; k < 3; k++)
      A[k][j] = J[(k + 1) % 3][(j + 1) % 3] * J[(k + 2) % 3][(j + 2) % 3] - J[(k + 2) % 3][(j + 1) % 3] * J[(k + 1) % 3][(j + 2) % 3];
  const double qw = w / (J[0][0] * A[0][0] + J[0][1] * A[0][1] + J[0][2] * A[0][2]);
  qd[0]           = qw * (A[0][0] * A[0][0] + A[0][1] * A[0][1] + A[0][2] * A[0][2]);
  qd[1]           = qw * (A[1][0] * A[1][0] + A[1][1] * A[1][1] + A[1][2] * A[1][2]);
  qd[2]           = qw * (A[2][0] * A[2][0] + A[2][1] * A[2][1] + A[2][2] * A[2][2]);
  qd[3]           = qw * (A[1][0] * A[2][0] + A[1][1] * A[2][1] + A[1][2] * A[2][2]);
  qd[4]           = qw * (A[0][0] * A[2][0] + A[0][1] * A[2][1] + A[0][2] * A[2][2]);
  qd[5]           = qw * (A[0][0] * A[1][0] + A[0][1] * A[1][1] + A[0][2] * A[1][2]);
}

}  // namespace b200
