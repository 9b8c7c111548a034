/*
 * Golden-vector generator: drives the reference libCEED (interface + /cpu/self/ref/serial + gallery, built from the
 * reference sources by oracle/Makefile into oracle/_ref/) through its public C API and writes the arrays that pin the
 * oracle and the GPU backend.  TEST INFRASTRUCTURE ONLY.
 *
 * Usage: ref_harness <out_dir> [resource]
 * Writes <out_dir>/<name>.bin (raw little-endian) and <out_dir>/manifest.txt ("name dtype count" per line).
 *
 * Meshes and random inputs come from the oracle's own generators (ceed_oracle.c: counter-based splitmix64, box
 * mesh), so the tests can regenerate every input bit-for-bit without the reference.
 */
#include <ceed.h>
#include <ceed/backend.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ceed_oracle.h"

static FILE       *g_manifest;
static const char *g_dir;

static void dump(const char *name, const char *dtype, const void *data, size_t count) {
  char   path[1024];
  size_t esize = strcmp(dtype, "f64") == 0 ? 8 : 4;

  snprintf(path, sizeof path, "%s/%s.bin", g_dir, name);
  FILE *f = fopen(path, "wb");

  if (!f || fwrite(data, esize, count, f) != count) {
    fprintf(stderr, "write failed: %s\n", path);
    exit(1);
  }
  fclose(f);
  fprintf(g_manifest, "%s %s %zu\n", name, dtype, count);
}

static void dump_vec(const char *name, CeedVector v) {
  CeedSize          n;
  const CeedScalar *a;

  CeedVectorGetLength(v, &n);
  CeedVectorGetArrayRead(v, CEED_MEM_HOST, &a);
  dump(name, "f64", a, (size_t)n);
  CeedVectorRestoreArrayRead(v, &a);
}

/* 1D basis tables for P = 2..10 with Q = P+1 Gauss points, plus the P = Q = 4 tables of tests/output/t300-basis.out. */
static void case_basis(Ceed ceed) {
  char name[128];

  for (int P = 2; P <= 10; P++) {
    for (int mode = 0; mode < 2; mode++) {
      const int         Q = mode == 0 ? P + 1 : P;
      CeedBasis         b;
      const CeedScalar *interp, *grad, *qref, *qw;
      CeedScalar        colo[16 * 16];

      if (mode == 1 && P != 4) continue;
      CeedBasisCreateTensorH1Lagrange(ceed, 1, 1, P, Q, mode == 0 ? CEED_GAUSS : CEED_GAUSS_LOBATTO, &b);
      CeedBasisGetInterp1D(b, &interp);
      CeedBasisGetGrad1D(b, &grad);
      CeedBasisGetQRef(b, &qref);
      CeedBasisGetQWeights(b, &qw);
      snprintf(name, sizeof name, "basis_P%d_Q%d_%s_interp", P, Q, mode == 0 ? "gauss" : "lobatto");
      dump(name, "f64", interp, (size_t)(P * Q));
      snprintf(name, sizeof name, "basis_P%d_Q%d_%s_grad", P, Q, mode == 0 ? "gauss" : "lobatto");
      dump(name, "f64", grad, (size_t)(P * Q));
      snprintf(name, sizeof name, "basis_P%d_Q%d_%s_qref", P, Q, mode == 0 ? "gauss" : "lobatto");
      dump(name, "f64", qref, (size_t)Q);
      snprintf(name, sizeof name, "basis_P%d_Q%d_%s_qweight", P, Q, mode == 0 ? "gauss" : "lobatto");
      dump(name, "f64", qw, (size_t)Q);
      if (mode == 0) {
        CeedBasisGetCollocatedGrad(b, colo);
        snprintf(name, sizeof name, "basis_P%d_Q%d_gauss_colograd", P, Q);
        dump(name, "f64", colo, (size_t)(Q * Q));
      }
      CeedBasisDestroy(&b);
    }
  }
}

/* Standalone 3D basis applies on a few elements: INTERP and GRAD, both transpose modes (one element per call,
 * as the ref operator uses them). */
static void case_basis_apply(Ceed ceed) {
  const int P = 4, Q = 5, ncomp = 2, P3 = 64, Q3 = 125;
  char      name[128];
  CeedBasis b;

  CeedBasisCreateTensorH1Lagrange(ceed, 3, ncomp, P, Q, CEED_GAUSS, &b);
  for (int emode = 0; emode < 2; emode++) {
    const CeedEvalMode em = emode == 0 ? CEED_EVAL_INTERP : CEED_EVAL_GRAD;
    const int          qc = emode == 0 ? 1 : 3;
    CeedVector         u, v, ut, vt;
    double            *buf_u = malloc(sizeof(double) * P3 * ncomp), *buf_q = malloc(sizeof(double) * Q3 * ncomp * qc);

    orc_fill_uniform(100 + emode, P3 * ncomp, -1, 1, buf_u);
    orc_fill_uniform(200 + emode, Q3 * ncomp * qc, -1, 1, buf_q);
    CeedVectorCreate(ceed, P3 * ncomp, &u);
    CeedVectorCreate(ceed, Q3 * ncomp * qc, &v);
    CeedVectorCreate(ceed, Q3 * ncomp * qc, &ut);
    CeedVectorCreate(ceed, P3 * ncomp, &vt);
    CeedVectorSetArray(u, CEED_MEM_HOST, CEED_COPY_VALUES, buf_u);
    CeedVectorSetArray(ut, CEED_MEM_HOST, CEED_COPY_VALUES, buf_q);
    CeedBasisApply(b, 1, CEED_NOTRANSPOSE, em, u, v);
    CeedBasisApply(b, 1, CEED_TRANSPOSE, em, ut, vt);
    snprintf(name, sizeof name, "bapply_%s_u", emode == 0 ? "interp" : "grad");
    dump_vec(name, u);
    snprintf(name, sizeof name, "bapply_%s_v", emode == 0 ? "interp" : "grad");
    dump_vec(name, v);
    snprintf(name, sizeof name, "bapply_%s_ut", emode == 0 ? "interp" : "grad");
    dump_vec(name, ut);
    snprintf(name, sizeof name, "bapply_%s_vt", emode == 0 ? "interp" : "grad");
    dump_vec(name, vt);
    CeedVectorDestroy(&u);
    CeedVectorDestroy(&v);
    CeedVectorDestroy(&ut);
    CeedVectorDestroy(&vt);
    free(buf_u);
    free(buf_q);
  }
  {
    CeedVector w;

    CeedVectorCreate(ceed, Q3, &w);
    CeedBasisApply(b, 1, CEED_NOTRANSPOSE, CEED_EVAL_WEIGHT, CEED_VECTOR_NONE, w);
    dump_vec("bapply_weight", w);
    CeedVectorDestroy(&w);
  }
  CeedBasisDestroy(&b);
}

typedef struct {
  const char *tag;
  int         n, P, Q, ncomp, poisson;
  double      noise;
  uint64_t    seed;
  int         kappa; /* kappa-weighted diffusion with its gradient */
} op_case;

/* Source string of the kappa QFunction: the ref backend calls the function pointer; the path is only recorded. */
CEED_QFUNCTION(PoissonKappaApply)(void *ctx, const CeedInt Q, const CeedScalar *const *in, CeedScalar *const *out) {
  const CeedScalar *ug = in[0], *qd = in[1], *kap = in[2];
  CeedScalar       *vg = out[0];

  for (CeedInt i = 0; i < Q; i++) {
    double D[3][3], u3[3] = {ug[i], ug[Q + i], ug[2 * Q + i]};
    double d6[6];

    for (int k = 0; k < 6; k++) d6[k] = qd[k * Q + i] * kap[i];
    D[0][0] = d6[0], D[0][1] = d6[5], D[0][2] = d6[4];
    D[1][0] = d6[5], D[1][1] = d6[1], D[1][2] = d6[3];
    D[2][0] = d6[4], D[2][1] = d6[3], D[2][2] = d6[2];
    for (int j = 0; j < 3; j++) vg[j * Q + i] = (u3[0] * D[0][j] + u3[1] * D[1][j] + u3[2] * D[2][j]);
  }
  return 0;
}

/* g = grad(w) . D grad(u) per point: the kappa-gradient of 1/2|A(kappa)u - f|^2 with w = A(kappa)u - f. */
CEED_QFUNCTION(PoissonKappaGrad)(void *ctx, const CeedInt Q, const CeedScalar *const *in, CeedScalar *const *out) {
  const CeedScalar *ug = in[0], *wg = in[1], *qd = in[2];
  CeedScalar       *g = out[0];

  for (CeedInt i = 0; i < Q; i++) {
    double D[3][3], u3[3] = {ug[i], ug[Q + i], ug[2 * Q + i]}, v3[3];

    D[0][0] = qd[0 * Q + i], D[0][1] = qd[5 * Q + i], D[0][2] = qd[4 * Q + i];
    D[1][0] = qd[5 * Q + i], D[1][1] = qd[1 * Q + i], D[1][2] = qd[3 * Q + i];
    D[2][0] = qd[4 * Q + i], D[2][1] = qd[3 * Q + i], D[2][2] = qd[2 * Q + i];
    for (int j = 0; j < 3; j++) v3[j] = (u3[0] * D[0][j] + u3[1] * D[1][j] + u3[2] * D[2][j]);
    g[i] = wg[i] * v3[0] + wg[Q + i] * v3[1] + wg[2 * Q + i] * v3[2];
  }
  return 0;
}

static void case_operator(Ceed ceed, const op_case *c) {
  const int     n = c->n, P = c->P, Q = c->Q, nc = c->ncomp, P3 = P * P * P, Q3 = Q * Q * Q;
  const int64_t ne = (int64_t)n * n * n, nv = (int64_t)(n + 1) * (n + 1) * (n + 1), nd = (int64_t)(n * (P - 1) + 1);
  const int64_t nnodes = nd * nd * nd, lsize = nnodes * nc, qcomp = c->poisson ? 6 : 1;
  char          name[160];
  double       *coords = malloc(sizeof(double) * 3 * nv);
  int32_t      *off_x = malloc(sizeof(int32_t) * ne * 8), *off_u = malloc(sizeof(int32_t) * ne * P3);
  double       *ubuf = malloc(sizeof(double) * lsize);

  orc_box_vertices(n, n, n, c->noise, c->seed, coords);
  orc_box_offsets(n, n, n, 2, 1, off_x);
  orc_box_offsets(n, n, n, P, nc, off_u);
  orc_fill_uniform(c->seed + 1, lsize, -1.0, 1.0, ubuf);

  CeedElemRestriction rx, ru, rq, rk;
  CeedBasis           bx, bu;
  CeedVector          X, U, V, QD, KAP = NULL, E;
  CeedQFunction       qf_build, qf_apply;
  CeedOperator        op_build, op_apply;

  CeedElemRestrictionCreate(ceed, ne, 8, 3, nv, 3 * nv, CEED_MEM_HOST, CEED_COPY_VALUES, off_x, &rx);
  CeedElemRestrictionCreate(ceed, ne, P3, nc, nc == 1 ? nnodes : 1, lsize, CEED_MEM_HOST, CEED_COPY_VALUES, off_u, &ru);
  CeedElemRestrictionCreateStrided(ceed, ne, Q3, qcomp, qcomp * ne * Q3, CEED_STRIDES_BACKEND, &rq);
  CeedBasisCreateTensorH1Lagrange(ceed, 3, 3, 2, Q, CEED_GAUSS, &bx);
  CeedBasisCreateTensorH1Lagrange(ceed, 3, nc, P, Q, CEED_GAUSS, &bu);
  CeedVectorCreate(ceed, 3 * nv, &X);
  CeedVectorSetArray(X, CEED_MEM_HOST, CEED_COPY_VALUES, coords);
  CeedVectorCreate(ceed, qcomp * ne * Q3, &QD);
  CeedVectorCreate(ceed, lsize, &U);
  CeedVectorCreate(ceed, lsize, &V);
  CeedVectorSetArray(U, CEED_MEM_HOST, CEED_COPY_VALUES, ubuf);

  /* Setup operator: geometric factors */
  CeedQFunctionCreateInteriorByName(ceed, c->poisson ? "Poisson3DBuild" : "Mass3DBuild", &qf_build);
  CeedOperatorCreate(ceed, qf_build, CEED_QFUNCTION_NONE, CEED_QFUNCTION_NONE, &op_build);
  CeedOperatorSetField(op_build, "dx", rx, bx, CEED_VECTOR_ACTIVE);
  CeedOperatorSetField(op_build, "weights", CEED_ELEMRESTRICTION_NONE, bx, CEED_VECTOR_NONE);
  CeedOperatorSetField(op_build, "qdata", rq, CEED_BASIS_NONE, CEED_VECTOR_ACTIVE);
  CeedOperatorApply(op_build, X, QD, CEED_REQUEST_IMMEDIATE);

  /* Apply operator */
  if (c->kappa) {
    CeedVectorCreate(ceed, ne * Q3, &KAP);
    double *kbuf = malloc(sizeof(double) * ne * Q3);

    for (int64_t i = 0; i < ne * Q3; i++) kbuf[i] = exp(0.5 * orc_uniform(c->seed + 2, (uint64_t)i, -1.0, 1.0));
    CeedVectorSetArray(KAP, CEED_MEM_HOST, CEED_COPY_VALUES, kbuf);
    free(kbuf);
    CeedElemRestrictionCreateStrided(ceed, ne, Q3, 1, ne * Q3, CEED_STRIDES_BACKEND, &rk);
    CeedQFunctionCreateInterior(ceed, 1, PoissonKappaApply, PoissonKappaApply_loc, &qf_apply);
    CeedQFunctionAddInput(qf_apply, "du", 3, CEED_EVAL_GRAD);
    CeedQFunctionAddInput(qf_apply, "qdata", 6, CEED_EVAL_NONE);
    CeedQFunctionAddInput(qf_apply, "kappa", 1, CEED_EVAL_NONE);
    CeedQFunctionAddOutput(qf_apply, "dv", 3, CEED_EVAL_GRAD);
  } else if (c->poisson) {
    CeedQFunctionCreateInteriorByName(ceed, nc == 1 ? "Poisson3DApply" : "Vector3Poisson3DApply", &qf_apply);
  } else {
    CeedQFunctionCreateInteriorByName(ceed, nc == 1 ? "MassApply" : "Vector3MassApply", &qf_apply);
  }
  CeedOperatorCreate(ceed, qf_apply, CEED_QFUNCTION_NONE, CEED_QFUNCTION_NONE, &op_apply);
  CeedOperatorSetField(op_apply, c->poisson ? "du" : "u", ru, bu, CEED_VECTOR_ACTIVE);
  CeedOperatorSetField(op_apply, "qdata", rq, CEED_BASIS_NONE, QD);
  if (c->kappa) CeedOperatorSetField(op_apply, "kappa", rk, CEED_BASIS_NONE, KAP);
  CeedOperatorSetField(op_apply, c->poisson ? "dv" : "v", ru, bu, CEED_VECTOR_ACTIVE);
  CeedOperatorApply(op_apply, U, V, CEED_REQUEST_IMMEDIATE);
  if (!c->kappa) {  // the reference's FLOP model (gallery QFunctions carry their estimates)
    CeedSize flops = 0;
    double   f;

    CeedOperatorGetFlopsEstimate(op_apply, &flops);
    f = (double)flops;
    snprintf(name, sizeof name, "%s_flops", c->tag);
    dump(name, "f64", &f, 1);
  }

  snprintf(name, sizeof name, "%s_coords", c->tag);
  dump(name, "f64", coords, (size_t)(3 * nv));
  snprintf(name, sizeof name, "%s_offsets", c->tag);
  dump(name, "i32", off_u, (size_t)(ne * P3));
  snprintf(name, sizeof name, "%s_qdata", c->tag);
  dump_vec(name, QD);
  snprintf(name, sizeof name, "%s_u", c->tag);
  dump_vec(name, U);
  snprintf(name, sizeof name, "%s_v", c->tag);
  dump_vec(name, V);

  /* Restriction gather of u, E-vector in the ref layout [elem][comp][node], and its transpose. */
  CeedElemRestrictionCreateVector(ru, NULL, &E);
  CeedElemRestrictionApply(ru, CEED_NOTRANSPOSE, U, E, CEED_REQUEST_IMMEDIATE);
  snprintf(name, sizeof name, "%s_egather", c->tag);
  dump_vec(name, E);
  CeedVectorSetValue(V, 0.0);
  CeedElemRestrictionApply(ru, CEED_TRANSPOSE, E, V, CEED_REQUEST_IMMEDIATE);
  snprintf(name, sizeof name, "%s_escatter", c->tag);
  dump_vec(name, V);
  CeedVectorDestroy(&E);

  if (c->kappa) {
    /* w = A(kappa)u - f, f seeded; gradient g = grad(w).D grad(u) per point, assembled on this backend. */
    CeedVector    W, G;
    CeedQFunction qf_g;
    CeedOperator  op_g;
    double       *fbuf = malloc(sizeof(double) * lsize);
    CeedScalar   *w;

    CeedOperatorApply(op_apply, U, V, CEED_REQUEST_IMMEDIATE);
    orc_fill_uniform(c->seed + 3, lsize, -1.0, 1.0, fbuf);
    CeedVectorCreate(ceed, lsize, &W);
    CeedVectorCopy(V, W);
    CeedVectorGetArray(W, CEED_MEM_HOST, &w);
    for (int64_t i = 0; i < lsize; i++) w[i] -= fbuf[i];
    CeedVectorRestoreArray(W, &w);
    CeedVectorCreate(ceed, ne * Q3, &G);
    CeedQFunctionCreateInterior(ceed, 1, PoissonKappaGrad, PoissonKappaGrad_loc, &qf_g);
    CeedQFunctionAddInput(qf_g, "du", 3, CEED_EVAL_GRAD);
    CeedQFunctionAddInput(qf_g, "dw", 3, CEED_EVAL_GRAD);
    CeedQFunctionAddInput(qf_g, "qdata", 6, CEED_EVAL_NONE);
    CeedQFunctionAddOutput(qf_g, "g", 1, CEED_EVAL_NONE);
    CeedOperatorCreate(ceed, qf_g, CEED_QFUNCTION_NONE, CEED_QFUNCTION_NONE, &op_g);
    CeedOperatorSetField(op_g, "du", ru, bu, U);
    CeedOperatorSetField(op_g, "dw", ru, bu, CEED_VECTOR_ACTIVE);
    CeedOperatorSetField(op_g, "qdata", rq, CEED_BASIS_NONE, QD);
    CeedOperatorSetField(op_g, "g", rk, CEED_BASIS_NONE, CEED_VECTOR_ACTIVE);
    CeedOperatorApply(op_g, W, G, CEED_REQUEST_IMMEDIATE);
    snprintf(name, sizeof name, "%s_kappa", c->tag);
    dump_vec(name, KAP);
    snprintf(name, sizeof name, "%s_f", c->tag);
    dump(name, "f64", fbuf, (size_t)lsize);
    snprintf(name, sizeof name, "%s_kgrad", c->tag);
    dump_vec(name, G);
    free(fbuf);
    CeedVectorDestroy(&W);
    CeedVectorDestroy(&G);
    CeedQFunctionDestroy(&qf_g);
    CeedOperatorDestroy(&op_g);
    CeedElemRestrictionDestroy(&rk);
    CeedVectorDestroy(&KAP);
  }

  CeedOperatorDestroy(&op_build);
  CeedOperatorDestroy(&op_apply);
  CeedQFunctionDestroy(&qf_build);
  CeedQFunctionDestroy(&qf_apply);
  CeedElemRestrictionDestroy(&rx);
  CeedElemRestrictionDestroy(&ru);
  CeedElemRestrictionDestroy(&rq);
  CeedBasisDestroy(&bx);
  CeedBasisDestroy(&bu);
  CeedVectorDestroy(&X);
  CeedVectorDestroy(&U);
  CeedVectorDestroy(&V);
  CeedVectorDestroy(&QD);
  free(coords);
  free(off_x);
  free(off_u);
  free(ubuf);
}

int main(int argc, char **argv) {
  Ceed        ceed;
  char        path[1024];
  const char *resource = argc > 2 ? argv[2] : "/cpu/self/ref/serial";

  if (argc < 2) {
    fprintf(stderr, "usage: %s <out_dir> [resource]\n", argv[0]);
    return 1;
  }
  g_dir = argv[1];
  snprintf(path, sizeof path, "%s/manifest.txt", g_dir);
  g_manifest = fopen(path, "w");
  if (!g_manifest) return 1;
  CeedInit(resource, &ceed);

  case_basis(ceed);
  case_basis_apply(ceed);
  /* Mass operator of the CPU parity configuration: 8^3 hexes, P=4, Q=5, +-0.1h noise. */
  const op_case mass = {"mass_n8_p3", 8, 4, 5, 1, 0, 0.1, 1001, 0};
  case_operator(ceed, &mass);
  /* Poisson at degrees 1..8 on small boxes with +-0.05h noise. */
  const int nper[9] = {0, 6, 4, 3, 3, 2, 2, 2, 2};

  for (int p = 1; p <= 8; p++) {
    op_case c;
    char   *tag = malloc(32);

    snprintf(tag, 32, "poisson_n%d_p%d", nper[p], p);
    c = (op_case){tag, nper[p], p + 1, p + 2, 1, 1, 0.05, (uint64_t)(2000 + p), 0};
    case_operator(ceed, &c);
  }
  /* Three-component interlaced vector Poisson and mass at degrees 2 and 4. */
  const op_case vp2 = {"vpoisson_n4_p2", 4, 3, 4, 3, 1, 0.05, 3002, 0};
  const op_case vp4 = {"vpoisson_n3_p4", 3, 5, 6, 3, 1, 0.05, 3004, 0};
  const op_case vm4 = {"vmass_n3_p4", 3, 5, 6, 3, 0, 0.05, 3104, 0};
  case_operator(ceed, &vp2);
  case_operator(ceed, &vp4);
  case_operator(ceed, &vm4);
  /* Kappa-weighted diffusion at degree 3 with its kappa-gradient. */
  const op_case kap = {"kappa_n3_p3", 3, 4, 5, 1, 1, 0.05, 4003, 1};
  case_operator(ceed, &kap);

  fclose(g_manifest);
  CeedDestroy(&ceed);
  return 0;
}
