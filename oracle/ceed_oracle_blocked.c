/* CPU baseline: a restatement of libCEED's /cpu/self/opt/blocked operator apply for tensor-H1 hexahedra.
 *
 * TEST AND BENCHMARK INFRASTRUCTURE ONLY: the benchmark times it as the CPU baseline and the tests check it against
 * the serial oracle (ceed_oracle.c); the product library never links it.
 *
 * It follows the reference's blocked operator (backends/opt/ceed-opt-operator.c:443-505, block size 8 from
 * backends/opt/ceed-opt-blocked.c:48): elements are processed in blocks of eight whose values are interleaved with the
 * element index innermost, so every tensor contraction runs its innermost loop over eight elements at once
 * (backends/opt/ceed-opt-tensor.c:16-34, called with post = num_elem as in backends/ref/ceed-ref-basis.c); per block the
 * input restriction (backends/ref/ceed-ref-restriction.c:59-75, offsets padded with the last element), the basis, the
 * QFunction over Q^3 * 8 points, the transposed basis and the output restriction, which adds node by node and within a
 * node position element by element (backends/ref/ceed-ref-restriction.c:219-240), skipping padding elements.  Every
 * element's arithmetic is the serial oracle's; only the order in which the scatter adds the contributions of elements
 * of one block to a shared node differs (rounding differences of one ulp in such sums).
 *
 * Built with -O3 -ffp-contract=off: the inner element loops vectorise, no multiply-add is contracted. */
#include <stdlib.h>
#include <string.h>

#include "ceed_oracle.h"

#define ORC_BLK 8

/* v[a][j][c] (+)= sum_b t[j,b] u[a][b][c], loop order of backends/opt/ceed-opt-tensor.c:16-34 (c innermost). */
static void blk_contract(int A, int B, int C, int J, const double *restrict t, int t_mode, int add, const double *restrict u,
                         double *restrict v) {
  const int s0 = t_mode == ORC_TRANSPOSE ? 1 : B, s1 = t_mode == ORC_TRANSPOSE ? J : 1;

  if (!add)
    for (int q = 0; q < A * J * C; q++) v[q] = 0.0;
  for (int a = 0; a < A; a++)
    for (int b = 0; b < B; b++)
      for (int j = 0; j < J; j++) {
        const double  tq = t[j * s0 + b * s1];
        double       *vv = v + (a * J + j) * C;
        const double *uu = u + (a * B + b) * C;

        for (int c = 0; c < C; c++) vv[c] += tq * uu[c];
      }
}

/* Basis of one block (interp for mass, collocated gradient for Poisson); values [qcomp][comp][node or point][8]. */
static void blk_basis(int P_1d, int Q_1d, int nc, const double *interp, const double *colo, int t_mode, int grad, const double *u, double *v,
                      double *t0, double *t1, double *ib) {
  double   *tmp[2] = {t0, t1};
  const int nq     = Q_1d * Q_1d * Q_1d;

  if (!grad) {
    int P = P_1d, Q = Q_1d;

    if (t_mode == ORC_TRANSPOSE) P = Q_1d, Q = P_1d;
    int pre = nc * P * P, post = ORC_BLK;

    for (int d = 0; d < 3; d++) {
      blk_contract(pre, P, post, Q, interp, t_mode, t_mode == ORC_TRANSPOSE && d == 2, d == 0 ? u : tmp[d % 2], d == 2 ? v : tmp[(d + 1) % 2]);
      pre /= P;
      post *= Q;
    }
    return;
  }
  if (t_mode == ORC_NOTRANSPOSE) {
    int pre = nc * P_1d * P_1d, post = ORC_BLK;

    for (int d = 0; d < 3; d++) {
      blk_contract(pre, P_1d, post, Q_1d, interp, ORC_NOTRANSPOSE, 0, d == 0 ? u : tmp[d % 2], d == 2 ? ib : tmp[(d + 1) % 2]);
      pre /= P_1d;
      post *= Q_1d;
    }
    pre = nc * Q_1d * Q_1d, post = ORC_BLK;
    for (int d = 0; d < 3; d++) {
      blk_contract(pre, Q_1d, post, Q_1d, colo, ORC_NOTRANSPOSE, 0, ib, &v[(size_t)d * nq * nc * ORC_BLK]);
      pre /= Q_1d;
      post *= Q_1d;
    }
  } else {
    int pre = nc * Q_1d * Q_1d, post = ORC_BLK;

    for (int d = 0; d < 3; d++) {
      blk_contract(pre, Q_1d, post, Q_1d, colo, ORC_TRANSPOSE, d > 0, &u[(size_t)d * nq * nc * ORC_BLK], ib);
      pre /= Q_1d;
      post *= Q_1d;
    }
    pre = nc * Q_1d * Q_1d, post = ORC_BLK;
    for (int d = 0; d < 3; d++) {
      blk_contract(pre, Q_1d, post, P_1d, interp, ORC_TRANSPOSE, d == 2, d == 0 ? ib : tmp[d % 2], d == 2 ? v : tmp[(d + 1) % 2]);
      pre /= Q_1d;
      post *= P_1d;
    }
  }
}

int orc_operator_apply_blocked(const orc_operator *op, const double *u, double *v, int add) {
  const int     P = op->P, Q = op->Q, P3 = P * P * P, Q3 = Q * Q * Q, nc = op->num_comp;
  const int     grad = op->qf == ORC_QF_POISSON3D_APPLY || op->qf == ORC_QF_VECPOISSON3D_APPLY || op->qf == ORC_QF_POISSON3D_KAPPA;
  const int     qc = grad ? 3 : 1, nqd = grad ? 6 : 1;
  const int64_t ne = op->num_elem;
  const int     mx = P > Q ? P : Q;
  const size_t  work = (size_t)nc * mx * mx * mx * ORC_BLK;
  double       *e_in = malloc(sizeof(double) * (size_t)nc * P3 * ORC_BLK), *e_out = malloc(sizeof(double) * (size_t)nc * P3 * ORC_BLK);
  double       *uq = malloc(sizeof(double) * (size_t)qc * nc * Q3 * ORC_BLK), *vq = malloc(sizeof(double) * (size_t)qc * nc * Q3 * ORC_BLK);
  double       *qd = malloc(sizeof(double) * (size_t)nqd * Q3 * ORC_BLK), *kp = malloc(sizeof(double) * (size_t)Q3 * ORC_BLK);
  double       *t0 = malloc(sizeof(double) * work), *t1 = malloc(sizeof(double) * work), *ib = malloc(sizeof(double) * work);
  double       *colo = malloc(sizeof(double) * (size_t)Q * Q);
  int           rc = 0;

  if (!e_in || !e_out || !uq || !vq || !qd || !kp || !t0 || !t1 || !ib || !colo || Q < P) rc = 1;
  if (!rc && grad) rc = orc_collocated_grad(P, Q, op->interp_1d, op->grad_1d, colo);
  if (!rc) {
    if (!add)
      for (int64_t i = 0; i < op->l_size; i++) v[i] = 0.0;
    for (int64_t e0 = 0; e0 < ne; e0 += ORC_BLK) {
      const int nb = ne - e0 < ORC_BLK ? (int)(ne - e0) : ORC_BLK;

      /* Input restriction of the block; padding elements repeat the last element. */
      for (int k = 0; k < nc; k++)
        for (int n = 0; n < P3; n++)
          for (int j = 0; j < ORC_BLK; j++) {
            const int64_t e = e0 + (j < nb ? j : nb - 1);

            e_in[((size_t)k * P3 + n) * ORC_BLK + j] = u[op->offsets[e * P3 + n] + k * op->comp_stride];
          }
      /* Passive inputs (qdata, kappa) through the blocked strided restriction. */
      for (int k = 0; k < nqd; k++)
        for (int q = 0; q < Q3; q++)
          for (int j = 0; j < ORC_BLK; j++) {
            const int64_t e = e0 + (j < nb ? j : nb - 1);

            qd[((size_t)k * Q3 + q) * ORC_BLK + j] = op->qdata[(e * nqd + k) * Q3 + q];
            if (k == 0 && op->kappa) kp[(size_t)q * ORC_BLK + j] = op->kappa[e * Q3 + q];
          }
      blk_basis(P, Q, nc, op->interp_1d, colo, ORC_NOTRANSPOSE, grad, e_in, uq, t0, t1, ib);
      /* QFunction over Q^3 * 8 points (the gallery kernels, as in the serial oracle). */
      const int nq = Q3 * ORC_BLK;

      if (!grad) {
        for (int c = 0; c < nc; c++)
          for (int i = 0; i < nq; i++) vq[(size_t)c * nq + i] = uq[(size_t)c * nq + i] * qd[i];
      } else {
        for (int i = 0; i < nq; i++) {
          double d6[6];

          for (int k = 0; k < 6; k++) d6[k] = qd[(size_t)k * nq + i];
          if (op->qf == ORC_QF_POISSON3D_KAPPA)
            for (int k = 0; k < 6; k++) d6[k] *= kp[i];
          for (int c = 0; c < nc; c++) {
            const double g0 = uq[(size_t)(0 * nc + c) * nq + i], g1 = uq[(size_t)(1 * nc + c) * nq + i], g2 = uq[(size_t)(2 * nc + c) * nq + i];

            /* ceed-poisson3dapply.h: D symmetric in Voigt order [0 5 4; 5 1 3; 4 3 2] */
            vq[(size_t)(0 * nc + c) * nq + i] = g0 * d6[0] + g1 * d6[5] + g2 * d6[4];
            vq[(size_t)(1 * nc + c) * nq + i] = g0 * d6[5] + g1 * d6[1] + g2 * d6[3];
            vq[(size_t)(2 * nc + c) * nq + i] = g0 * d6[4] + g1 * d6[3] + g2 * d6[2];
          }
        }
      }
      for (size_t i = 0; i < (size_t)nc * P3 * ORC_BLK; i++) e_out[i] = 0.0;
      blk_basis(P, Q, nc, op->interp_1d, colo, ORC_TRANSPOSE, grad, vq, e_out, t0, t1, ib);
      /* Output restriction: component, node position, then element within the block; padding skipped. */
      for (int k = 0; k < nc; k++)
        for (int n = 0; n < P3; n++)
          for (int j = 0; j < nb; j++) v[op->offsets[(e0 + j) * P3 + n] + k * op->comp_stride] += e_out[((size_t)k * P3 + n) * ORC_BLK + j];
    }
  }
  free(e_in);
  free(e_out);
  free(uq);
  free(vq);
  free(qd);
  free(kp);
  free(t0);
  free(t1);
  free(ib);
  free(colo);
  return rc;
}
