// QFunctions written the way libCEED users write them (CEED_QFUNCTION, CEED_Q_VLA, component-major Q arrays), used to
// test run-time compilation into the fused kernel.
#include <ceed/types.h>

// Variable-coefficient diffusion: vg = kappa * D ug with D the 6-entry symmetric geometric factor (Voigt order).
CEED_QFUNCTION(DiffusionKappa)(void *ctx, const CeedInt Q, const CeedScalar *const *in, CeedScalar *const *out) {
  const CeedScalar(*ug)[CEED_Q_VLA] = (const CeedScalar(*)[CEED_Q_VLA])in[0], (*qd)[CEED_Q_VLA] = (const CeedScalar(*)[CEED_Q_VLA])in[1];
  const CeedScalar *kappa = in[2];
  CeedScalar(*vg)[CEED_Q_VLA] = (CeedScalar(*)[CEED_Q_VLA])out[0];

  CeedPragmaSIMD for (CeedInt i = 0; i < Q; i++) {
    const CeedScalar k = kappa[i];
    const CeedScalar D[3][3] = {
        {qd[0][i] * k, qd[5][i] * k, qd[4][i] * k},
        {qd[5][i] * k, qd[1][i] * k, qd[3][i] * k},
        {qd[4][i] * k, qd[3][i] * k, qd[2][i] * k}
    };
    for (CeedInt j = 0; j < 3; j++) vg[j][i] = ug[0][i] * D[0][j] + ug[1][i] * D[1][j] + ug[2][i] * D[2][j];
  }
  return CEED_ERROR_SUCCESS;
}

struct ScaledMassContext {
  CeedScalar scale;
};

// Mass operator scaled by a context value: v = scale * qdata * u (qdata listed first to test input ordering).
CEED_QFUNCTION(ScaledMass)(void *ctx, const CeedInt Q, const CeedScalar *const *in, CeedScalar *const *out) {
  const struct ScaledMassContext *c = (const struct ScaledMassContext *)ctx;
  const CeedScalar               *qd = in[0], *u = in[1];
  CeedScalar                     *v = out[0];

  CeedPragmaSIMD for (CeedInt i = 0; i < Q; i++) v[i] = c->scale * qd[i] * u[i];
  return CEED_ERROR_SUCCESS;
}
