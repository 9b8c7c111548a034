// Drop-in check of `/gpu/cuda/b200` through the stock libCEED API: the same problems are set up on `/gpu/cuda/b200`
// and on `/cpu/self/ref/serial` in one process and the applies compared (relative l-infinity, tolerance 1e-12):
//   1. gallery Poisson3DBuild + Poisson3DApply on a perturbed box of hexahedra (fused compiled kernel);
//      and its assembled diagonal (CeedOperatorLinearAssembleDiagonal);
//      the same with the resource option ":arithmetic=float-float" (float-float kernels on double vectors);
//   2. gallery Mass3DBuild + the user QFunction ScaledMass from tests/qfunctions/user-qfunctions.h with a context
//      (NVRTC-compiled on /gpu/cuda/b200, the function pointer on the CPU backend);
//   3. CeedVectorSetValueStrided and CeedVectorCopyStrided (device kernels on /gpu/cuda/b200), compared bitwise.
// Needs a GPU and a libCEED build; prints nothing on success, like the reference's tests/t*.c.
#include <ceed.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "user-qfunctions.h"

int CeedB200Register(void);

static void ApplyUserMass(const char *resource, int n, int P, const double *coords, const CeedInt *xoff, const CeedInt *uoff, const double *u,
                          double *v) {
  const int            Q = P + 1, ne = n * n * n, nv = (n + 1) * (n + 1) * (n + 1), nd = n * (P - 1) + 1, N = nd * nd * nd;
  Ceed                 ceed;
  CeedVector           X, U, V, QD;
  CeedBasis            bx, bu;
  CeedElemRestriction  rx, ru, rq;
  CeedQFunction        qf_b, qf_a;
  CeedQFunctionContext qctx;
  CeedOperator         op_b, op_a;
  struct ScaledMassContext c = {0.75};

  CeedInit(resource, &ceed);
  CeedElemRestrictionCreate(ceed, ne, 8, 3, nv, 3 * nv, CEED_MEM_HOST, CEED_COPY_VALUES, xoff, &rx);
  CeedElemRestrictionCreate(ceed, ne, P * P * P, 1, 1, N, CEED_MEM_HOST, CEED_COPY_VALUES, uoff, &ru);
  CeedElemRestrictionCreateStrided(ceed, ne, Q * Q * Q, 1, ne * Q * Q * Q, CEED_STRIDES_BACKEND, &rq);
  CeedBasisCreateTensorH1Lagrange(ceed, 3, 3, 2, Q, CEED_GAUSS, &bx);
  CeedBasisCreateTensorH1Lagrange(ceed, 3, 1, P, Q, CEED_GAUSS, &bu);
  CeedVectorCreate(ceed, 3 * nv, &X);
  CeedVectorSetArray(X, CEED_MEM_HOST, CEED_COPY_VALUES, (double *)coords);
  CeedVectorCreate(ceed, ne * Q * Q * Q, &QD);
  CeedVectorCreate(ceed, N, &U);
  CeedVectorCreate(ceed, N, &V);
  CeedVectorSetArray(U, CEED_MEM_HOST, CEED_COPY_VALUES, (double *)u);
  CeedQFunctionCreateInteriorByName(ceed, "Mass3DBuild", &qf_b);
  CeedOperatorCreate(ceed, qf_b, CEED_QFUNCTION_NONE, CEED_QFUNCTION_NONE, &op_b);
  CeedOperatorSetField(op_b, "dx", rx, bx, CEED_VECTOR_ACTIVE);
  CeedOperatorSetField(op_b, "weights", CEED_ELEMRESTRICTION_NONE, bx, CEED_VECTOR_NONE);
  CeedOperatorSetField(op_b, "qdata", rq, CEED_BASIS_NONE, CEED_VECTOR_ACTIVE);
  CeedOperatorApply(op_b, X, QD, CEED_REQUEST_IMMEDIATE);
  CeedQFunctionCreateInterior(ceed, 1, ScaledMass, USER_QF_PATH ":ScaledMass", &qf_a);
  CeedQFunctionAddInput(qf_a, "qdata", 1, CEED_EVAL_NONE);
  CeedQFunctionAddInput(qf_a, "u", 1, CEED_EVAL_INTERP);
  CeedQFunctionAddOutput(qf_a, "v", 1, CEED_EVAL_INTERP);
  CeedQFunctionContextCreate(ceed, &qctx);
  CeedQFunctionContextSetData(qctx, CEED_MEM_HOST, CEED_COPY_VALUES, sizeof c, &c);
  CeedQFunctionSetContext(qf_a, qctx);
  CeedOperatorCreate(ceed, qf_a, CEED_QFUNCTION_NONE, CEED_QFUNCTION_NONE, &op_a);
  CeedOperatorSetField(op_a, "qdata", rq, CEED_BASIS_NONE, QD);
  CeedOperatorSetField(op_a, "u", ru, bu, CEED_VECTOR_ACTIVE);
  CeedOperatorSetField(op_a, "v", ru, bu, CEED_VECTOR_ACTIVE);
  CeedOperatorApply(op_a, U, V, CEED_REQUEST_IMMEDIATE);
  {
    const double *a;

    CeedVectorGetArrayRead(V, CEED_MEM_HOST, &a);
    for (int i = 0; i < N; i++) v[i] = a[i];
    CeedVectorRestoreArrayRead(V, &a);
  }
  CeedOperatorDestroy(&op_a);
  CeedOperatorDestroy(&op_b);
  CeedQFunctionContextDestroy(&qctx);
  CeedQFunctionDestroy(&qf_a);
  CeedQFunctionDestroy(&qf_b);
  CeedElemRestrictionDestroy(&rx);
  CeedElemRestrictionDestroy(&ru);
  CeedElemRestrictionDestroy(&rq);
  CeedBasisDestroy(&bx);
  CeedBasisDestroy(&bu);
  CeedVectorDestroy(&X);
  CeedVectorDestroy(&U);
  CeedVectorDestroy(&V);
  CeedVectorDestroy(&QD);
  CeedDestroy(&ceed);
}

static void Apply(const char *resource, int n, int P, const double *coords, const CeedInt *xoff, const CeedInt *uoff, const double *u, double *v,
                  double *diag) {
  const int     Q = P + 1, ne = n * n * n, nv = (n + 1) * (n + 1) * (n + 1), nd = n * (P - 1) + 1, N = nd * nd * nd;
  Ceed          ceed;
  CeedVector    X, U, V, QD;
  CeedBasis     bx, bu;
  CeedElemRestriction rx, ru, rq;
  CeedQFunction qf_b, qf_a;
  CeedOperator  op_b, op_a;

  CeedInit(resource, &ceed);
  CeedElemRestrictionCreate(ceed, ne, 8, 3, nv, 3 * nv, CEED_MEM_HOST, CEED_COPY_VALUES, xoff, &rx);
  CeedElemRestrictionCreate(ceed, ne, P * P * P, 1, 1, N, CEED_MEM_HOST, CEED_COPY_VALUES, uoff, &ru);
  CeedElemRestrictionCreateStrided(ceed, ne, Q * Q * Q, 6, 6 * ne * Q * Q * Q, CEED_STRIDES_BACKEND, &rq);
  CeedBasisCreateTensorH1Lagrange(ceed, 3, 3, 2, Q, CEED_GAUSS, &bx);
  CeedBasisCreateTensorH1Lagrange(ceed, 3, 1, P, Q, CEED_GAUSS, &bu);
  CeedVectorCreate(ceed, 3 * nv, &X);
  CeedVectorSetArray(X, CEED_MEM_HOST, CEED_COPY_VALUES, (double *)coords);
  CeedVectorCreate(ceed, 6 * ne * Q * Q * Q, &QD);
  CeedVectorCreate(ceed, N, &U);
  CeedVectorCreate(ceed, N, &V);
  CeedVectorSetArray(U, CEED_MEM_HOST, CEED_COPY_VALUES, (double *)u);
  CeedQFunctionCreateInteriorByName(ceed, "Poisson3DBuild", &qf_b);
  CeedOperatorCreate(ceed, qf_b, CEED_QFUNCTION_NONE, CEED_QFUNCTION_NONE, &op_b);
  CeedOperatorSetField(op_b, "dx", rx, bx, CEED_VECTOR_ACTIVE);
  CeedOperatorSetField(op_b, "weights", CEED_ELEMRESTRICTION_NONE, bx, CEED_VECTOR_NONE);
  CeedOperatorSetField(op_b, "qdata", rq, CEED_BASIS_NONE, CEED_VECTOR_ACTIVE);
  CeedOperatorApply(op_b, X, QD, CEED_REQUEST_IMMEDIATE);
  CeedQFunctionCreateInteriorByName(ceed, "Poisson3DApply", &qf_a);
  CeedOperatorCreate(ceed, qf_a, CEED_QFUNCTION_NONE, CEED_QFUNCTION_NONE, &op_a);
  CeedOperatorSetField(op_a, "du", ru, bu, CEED_VECTOR_ACTIVE);
  CeedOperatorSetField(op_a, "qdata", rq, CEED_BASIS_NONE, QD);
  CeedOperatorSetField(op_a, "dv", ru, bu, CEED_VECTOR_ACTIVE);
  CeedOperatorApply(op_a, U, V, CEED_REQUEST_IMMEDIATE);
  {
    const double *a;

    CeedVectorGetArrayRead(V, CEED_MEM_HOST, &a);
    for (int i = 0; i < N; i++) v[i] = a[i];
    CeedVectorRestoreArrayRead(V, &a);
  }
  CeedOperatorLinearAssembleDiagonal(op_a, V, CEED_REQUEST_IMMEDIATE);
  {
    const double *a;

    CeedVectorGetArrayRead(V, CEED_MEM_HOST, &a);
    for (int i = 0; i < N; i++) diag[i] = a[i];
    CeedVectorRestoreArrayRead(V, &a);
  }
  CeedOperatorDestroy(&op_a);
  CeedOperatorDestroy(&op_b);
  CeedQFunctionDestroy(&qf_a);
  CeedQFunctionDestroy(&qf_b);
  CeedElemRestrictionDestroy(&rx);
  CeedElemRestrictionDestroy(&ru);
  CeedElemRestrictionDestroy(&rq);
  CeedBasisDestroy(&bx);
  CeedBasisDestroy(&bu);
  CeedVectorDestroy(&X);
  CeedVectorDestroy(&U);
  CeedVectorDestroy(&V);
  CeedVectorDestroy(&QD);
  CeedDestroy(&ceed);
}

// x = u, then x[3:N:7] = -2.5, then y = 0 with y[1:-1:5] = x[1:-1:5]; returns x followed by y in out[2N].
static void Strided(const char *resource, int N, const double *u, double *out) {
  Ceed       ceed;
  CeedVector x, y;

  CeedInit(resource, &ceed);
  CeedVectorCreate(ceed, N, &x);
  CeedVectorCreate(ceed, N, &y);
  CeedVectorSetArray(x, CEED_MEM_HOST, CEED_COPY_VALUES, (double *)u);
  CeedVectorSetValue(y, 0.0);
  CeedVectorSetValueStrided(x, 3, N, 7, -2.5);
  CeedVectorCopyStrided(x, 1, -1, 5, y);
  const double *a;
  CeedVectorGetArrayRead(x, CEED_MEM_HOST, &a);
  for (int i = 0; i < N; i++) out[i] = a[i];
  CeedVectorRestoreArrayRead(x, &a);
  CeedVectorGetArrayRead(y, CEED_MEM_HOST, &a);
  for (int i = 0; i < N; i++) out[N + i] = a[i];
  CeedVectorRestoreArrayRead(y, &a);
  CeedVectorDestroy(&x);
  CeedVectorDestroy(&y);
  CeedDestroy(&ceed);
}

int main(void) {
  const int n = 3, P = 5, nv = (n + 1) * (n + 1) * (n + 1), nd = n * (P - 1) + 1, N = nd * nd * nd, ne = n * n * n;
  double   *coords = malloc(sizeof(double) * 3 * nv), *u = malloc(sizeof(double) * N), *v_gpu = malloc(sizeof(double) * N),
         *v_ref = malloc(sizeof(double) * N);
  CeedInt  *xoff = malloc(sizeof(CeedInt) * ne * 8), *uoff = malloc(sizeof(CeedInt) * ne * P * P * P);

  for (int k = 0; k <= n; k++)
    for (int j = 0; j <= n; j++)
      for (int i = 0; i <= n; i++) {
        const int v = i + (n + 1) * (j + (n + 1) * k), in = i > 0 && i < n && j > 0 && j < n && k > 0 && k < n;
        coords[v]          = (double)i / n + (in ? 0.04 * sin(7.0 * v) / n : 0.0);
        coords[nv + v]     = (double)j / n + (in ? 0.04 * cos(5.0 * v) / n : 0.0);
        coords[2 * nv + v] = (double)k / n;
      }
  for (int e = 0; e < ne; e++) {
    const int ex = e % n, ey = (e / n) % n, ez = e / (n * n);
    for (int l = 0; l < 8; l++) xoff[e * 8 + l] = (ex + (l & 1)) + (n + 1) * ((ey + ((l >> 1) & 1)) + (n + 1) * (ez + (l >> 2)));
    for (int lz = 0; lz < P; lz++)
      for (int ly = 0; ly < P; ly++)
        for (int lx = 0; lx < P; lx++)
          uoff[e * P * P * P + lx + P * (ly + P * lz)] = (ex * (P - 1) + lx) + nd * ((ey * (P - 1) + ly) + nd * (ez * (P - 1) + lz));
  }
  for (int i = 0; i < N; i++) u[i] = sin(0.37 * i);
  CeedB200Register();
  double *d_gpu = malloc(sizeof(double) * N), *d_ref = malloc(sizeof(double) * N);
  Apply("/gpu/cuda/b200", n, P, coords, xoff, uoff, u, v_gpu, d_gpu);
  Apply("/cpu/self/ref/serial", n, P, coords, xoff, uoff, u, v_ref, d_ref);
  double err = 0, scale = 0;
  for (int i = 0; i < N; i++) err = fmax(err, fabs(v_gpu[i] - v_ref[i])), scale = fmax(scale, fabs(v_ref[i]));
  if (err > 1e-12 * scale) printf("Error: /gpu/cuda/b200 differs from /cpu/self/ref/serial by %e (relative)\n", err / scale);
  int fail = err > 1e-12 * scale;
  err = 0, scale = 0;
  for (int i = 0; i < N; i++) err = fmax(err, fabs(d_gpu[i] - d_ref[i])), scale = fmax(scale, fabs(d_ref[i]));
  if (err > 1e-12 * scale) printf("Error: assembled diagonal on /gpu/cuda/b200 differs by %e (relative)\n", err / scale);
  fail |= err > 1e-12 * scale;
  Apply("/gpu/cuda/b200:arithmetic=float-float", n, P, coords, xoff, uoff, u, v_gpu, d_gpu);
  err = 0, scale = 0;
  for (int i = 0; i < N; i++) err = fmax(err, fabs(v_gpu[i] - v_ref[i])), scale = fmax(scale, fabs(v_ref[i]));
  if (err > 1e-12 * scale) printf("Error: float-float apply on /gpu/cuda/b200 differs by %e (relative)\n", err / scale);
  fail |= err > 1e-12 * scale;
  free(d_gpu), free(d_ref);
  ApplyUserMass("/gpu/cuda/b200", n, P, coords, xoff, uoff, u, v_gpu);
  ApplyUserMass("/cpu/self/ref/serial", n, P, coords, xoff, uoff, u, v_ref);
  err = 0, scale = 0;
  for (int i = 0; i < N; i++) err = fmax(err, fabs(v_gpu[i] - v_ref[i])), scale = fmax(scale, fabs(v_ref[i]));
  if (err > 1e-12 * scale) printf("Error: user QFunction on /gpu/cuda/b200 differs from /cpu/self/ref/serial by %e (relative)\n", err / scale);
  fail |= err > 1e-12 * scale;
  double *s_gpu = malloc(sizeof(double) * 2 * N), *s_ref = malloc(sizeof(double) * 2 * N);
  Strided("/gpu/cuda/b200", N, u, s_gpu);
  Strided("/cpu/self/ref/serial", N, u, s_ref);
  int strided_diff = 0;
  for (int i = 0; i < 2 * N; i++) strided_diff += s_gpu[i] != s_ref[i];
  if (strided_diff) printf("Error: strided set/copy on /gpu/cuda/b200 differs in %d entries\n", strided_diff);
  fail |= strided_diff != 0;
  free(s_gpu), free(s_ref);
  free(coords), free(u), free(v_gpu), free(v_ref), free(xoff), free(uoff);
  return fail;
}
