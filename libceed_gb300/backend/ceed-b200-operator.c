// CeedOperator for `/gpu/cuda/b200`: the fused apply of tensor-H1 hexahedral operators.
//
// CeedOperatorApply / ApplyAdd (interface/ceed-operator.c:2271-2410) land here.  On first use the operator is matched
// against the pattern the fused kernels implement:
//   apply:  active input/output through one offset restriction and one 3D tensor H1 basis with Q = P + 1, a gallery
//           pointwise kernel (MassApply, Poisson3DApply, Vector3MassApply, Vector3Poisson3DApply), and qdata as a
//           passive CEED_EVAL_NONE field through a strided restriction with backend strides -> b200_op_apply;
//   setup:  Mass3DBuild / Poisson3DBuild with a trilinear coordinate field -> b200_qdata_build;
//   user:   a QFunction from a source file with one active input (CEED_EVAL_INTERP or GRAD) and one active output
//           through one offset restriction and 3D tensor basis with Q = P + 1, passive inputs CEED_EVAL_NONE through
//           backend-strided restrictions -> NVRTC-compiled fused kernel (b200_op_create_jit / b200_op_apply_jit), as
//           the reference's cuda-gen backend compiles its generated kernel (backends/cuda/ceed-cuda-compile.cpp).
// Anything else returns CEED_ERROR_UNSUPPORTED: this backend has no CPU fallback and no delegate.
#include <string.h>

#include "ceed-b200-backend.h"

static int FieldParts(CeedOperatorField f, CeedElemRestriction *r, CeedBasis *b, CeedVector *v) {
  CeedCallBackend(CeedOperatorFieldGetElemRestriction(f, r));
  CeedCallBackend(CeedOperatorFieldGetBasis(f, b));
  CeedCallBackend(CeedOperatorFieldGetVector(f, v));
  return CEED_ERROR_SUCCESS;
}

// Fill the parts of the fused-operator descriptor that come from the active restriction and basis.
static int ActiveDesc(Ceed ceed, CeedElemRestriction ru, CeedBasis bu, b200_op_desc *d) {
  CeedInt                   dim, P, Q, nc, ne, comp_stride;
  CeedSize                  l_size;
  bool                      is_tensor, det;
  const CeedScalar         *interp, *grad;
  CeedRestrictionType       type;
  CeedElemRestriction_B200 *r_impl;

  CeedCallBackend(CeedElemRestrictionGetType(ru, &type));
  CeedCallBackend(CeedBasisIsTensor(bu, &is_tensor));
  CeedCallBackend(CeedBasisGetDimension(bu, &dim));
  CeedCallBackend(CeedBasisGetNumNodes1D(bu, &P));
  CeedCallBackend(CeedBasisGetNumQuadraturePoints1D(bu, &Q));
  CeedCheck(type == CEED_RESTRICTION_STANDARD && is_tensor && dim == 3 && Q == P + 1, ceed, CEED_ERROR_UNSUPPORTED,
            "fused apply needs an offset restriction and a 3D tensor basis with Q = P + 1");
  CeedCallBackend(CeedElemRestrictionGetNumComponents(ru, &nc));
  CeedCallBackend(CeedElemRestrictionGetNumElements(ru, &ne));
  CeedCallBackend(CeedElemRestrictionGetCompStride(ru, &comp_stride));
  CeedCallBackend(CeedElemRestrictionGetLVectorSize(ru, &l_size));
  CeedCallBackend(CeedBasisGetInterp1D(bu, &interp));
  CeedCallBackend(CeedBasisGetGrad1D(bu, &grad));
  CeedCallBackend(CeedIsDeterministic(ceed, &det));
  CeedCallBackend(CeedElemRestrictionGetData(ru, &r_impl));
  memset(d, 0, sizeof *d);
  d->prec        = B200_F64;
  d->P_1d        = P;
  d->Q_1d        = Q;
  d->num_comp    = nc;
  d->scatter     = det ? B200_SCATTER_DETERMINISTIC : B200_SCATTER_ATOMIC;
  d->num_elem    = ne;
  d->l_size      = l_size;
  d->comp_stride = comp_stride;
  d->offsets     = r_impl->d_offsets;
  d->interp_1d   = interp;
  d->grad_1d     = grad;
  return CEED_ERROR_SUCCESS;
}

// User QFunction: match the field pattern, compile with NVRTC, keep the passive vectors.
static int OperatorAnalyseJit_B200(CeedOperator op, CeedQFunction qf, CeedInt n_in, CeedOperatorField *in, CeedInt n_out,
                                   CeedOperatorField *out) {
  Ceed                 ceed = CeedOperatorReturnCeed(op);
  CeedOperator_B200   *impl;
  CeedQFunctionField  *qf_in, *qf_out;
  CeedInt              qf_n_in, qf_n_out, active = -1, num_roots = 0;
  CeedElemRestriction  ru = NULL, ro = NULL;
  CeedBasis            bu = NULL, bo = NULL;
  CeedVector           vo;
  b200_op_desc         d;
  b200_jit_qfunction   j;
  const char          *name, *source, **roots = NULL;
  char                 dirs[4096] = "";
  b200_ctx             ctx;

  CeedCallBackend(CeedOperatorGetData(op, &impl));
  CeedCallBackend(CeedGetB200Context(ceed, &ctx));
  CeedCallBackend(CeedQFunctionGetFields(qf, &qf_n_in, &qf_in, &qf_n_out, &qf_out));
  CeedCheck(n_in >= 1 && n_in <= 8 && n_out == 1, ceed, CEED_ERROR_UNSUPPORTED, "run-time compiled QFunctions: 1 to 8 inputs and one output");
  memset(&j, 0, sizeof j);
  j.num_inputs = n_in;
  impl->num_passive = 0;
  for (CeedInt i = 0; i < n_in; i++) {
    CeedElemRestriction r;
    CeedBasis           b;
    CeedVector          v;
    CeedEvalMode        mode;
    CeedInt             size;

    CeedCallBackend(FieldParts(in[i], &r, &b, &v));
    CeedCallBackend(CeedQFunctionFieldGetSize(qf_in[i], &size));
    CeedCallBackend(CeedQFunctionFieldGetEvalMode(qf_in[i], &mode));
    j.input_size[i] = size;
    if (v == CEED_VECTOR_ACTIVE) {
      CeedCheck(active < 0 && (mode == CEED_EVAL_INTERP || mode == CEED_EVAL_GRAD), ceed, CEED_ERROR_UNSUPPORTED,
                "run-time compiled QFunctions: one active input with CEED_EVAL_INTERP or CEED_EVAL_GRAD");
      active    = i;
      j.eval_in = mode == CEED_EVAL_GRAD ? B200_EVAL_GRAD : B200_EVAL_INTERP;
      ru        = r;
      bu        = b;
    } else {
      bool strided = false, backend_strides = false;

      CeedCallBackend(CeedElemRestrictionIsStrided(r, &strided));
      if (strided) CeedCallBackend(CeedElemRestrictionHasBackendStrides(r, &backend_strides));
      CeedCheck(mode == CEED_EVAL_NONE && backend_strides && v != CEED_VECTOR_NONE, ceed, CEED_ERROR_UNSUPPORTED,
                "run-time compiled QFunctions: passive inputs use CEED_EVAL_NONE through backend-strided restrictions");
      impl->passive[impl->num_passive++] = v;  // reference kept until destroy
      CeedCallBackend(CeedElemRestrictionDestroy(&r));
      CeedCallBackend(CeedBasisDestroy(&b));
    }
  }
  CeedCheck(active >= 0, ceed, CEED_ERROR_UNSUPPORTED, "run-time compiled QFunctions need an active input");
  {
    CeedEvalMode mode;

    CeedCallBackend(FieldParts(out[0], &ro, &bo, &vo));
    CeedCallBackend(CeedQFunctionFieldGetEvalMode(qf_out[0], &mode));
    j.eval_out = mode == CEED_EVAL_GRAD ? B200_EVAL_GRAD : B200_EVAL_INTERP;
    CeedCheck(vo == CEED_VECTOR_ACTIVE && ro == ru && bo == bu && (mode == CEED_EVAL_INTERP || mode == CEED_EVAL_GRAD), ceed,
              CEED_ERROR_UNSUPPORTED, "run-time compiled QFunctions: the active output uses the active input's restriction and basis");
  }
  CeedCallBackend(ActiveDesc(ceed, ru, bu, &d));
  d.qf = -1;
  CeedCallBackend(CeedQFunctionGetKernelName(qf, &name));
  CeedCallBackend(CeedQFunctionGetSourcePath(qf, &source));
  CeedCallBackend(CeedGetJitSourceRoots(ceed, &num_roots, &roots));
  for (CeedInt i = 0; i < num_roots; i++) {
    if (strlen(dirs) + strlen(roots[i]) + 2 >= sizeof dirs) break;
    if (dirs[0]) strcat(dirs, ":");
    strcat(dirs, roots[i]);
  }
  j.source_path  = source;
  j.name         = name;
  j.active_input = active;
  j.include_dirs = dirs;
  CeedCallB200(ceed, b200_op_create_jit(ctx, &d, &j, &impl->op));
  CeedCallBackend(CeedRestoreJitSourceRoots(ceed, &roots));
  {
    CeedQFunctionContext qf_ctx = NULL;

    CeedCallBackend(CeedQFunctionGetContext(qf, &qf_ctx));
    impl->ctx_size = 0;
    if (qf_ctx) CeedCallBackend(CeedQFunctionContextGetContextSize(qf_ctx, &impl->ctx_size));
    if (impl->ctx_size) CeedCallB200(ceed, b200_alloc(ctx, impl->ctx_size, &impl->d_ctx));
  }
  impl->kind = 3;
  CeedCallBackend(CeedElemRestrictionDestroy(&ru));
  CeedCallBackend(CeedElemRestrictionDestroy(&ro));
  CeedCallBackend(CeedBasisDestroy(&bu));
  CeedCallBackend(CeedBasisDestroy(&bo));
  return CEED_ERROR_SUCCESS;
}

static int OperatorAnalyse_B200(CeedOperator op) {
  Ceed                ceed = CeedOperatorReturnCeed(op);
  CeedOperator_B200  *impl;
  CeedQFunction       qf;
  CeedQFunction_B200 *qf_impl;
  CeedInt             n_in, n_out;
  CeedOperatorField  *in, *out;
  b200_ctx            ctx;

  CeedCallBackend(CeedOperatorGetData(op, &impl));
  if (impl->kind) return CEED_ERROR_SUCCESS;
  impl->kind = -1;
  CeedCallBackend(CeedGetB200Context(ceed, &ctx));
  CeedCallBackend(CeedOperatorGetQFunction(op, &qf));
  CeedCallBackend(CeedQFunctionGetData(qf, &qf_impl));
  CeedCallBackend(CeedOperatorGetFields(op, &n_in, &in, &n_out, &out));
  if (qf_impl->qf_kind == -1) {
    // Geometric factors: fields "dx" (GRAD of coordinates), "weights" (WEIGHT), output "qdata".
    CeedElemRestriction rx, rq;
    CeedBasis           bx, bq;
    CeedVector          vx, vq;
    CeedInt             P, dim, nc, esize;
    bool                backend_strides = false, strided;

    CeedCallBackend(FieldParts(in[0], &rx, &bx, &vx));
    CeedCallBackend(FieldParts(out[0], &rq, &bq, &vq));
    CeedCallBackend(CeedBasisGetDimension(bx, &dim));
    CeedCallBackend(CeedBasisGetNumNodes1D(bx, &P));
    CeedCallBackend(CeedElemRestrictionGetNumComponents(rx, &nc));
    CeedCallBackend(CeedElemRestrictionGetElementSize(rx, &esize));
    CeedCallBackend(CeedElemRestrictionIsStrided(rq, &strided));
    if (strided) CeedCallBackend(CeedElemRestrictionHasBackendStrides(rq, &backend_strides));
    CeedCheck(dim == 3 && P == 2 && nc == 3 && esize == 8 && backend_strides, ceed, CEED_ERROR_UNSUPPORTED,
              "geometric factors on /gpu/cuda/b200 need a trilinear 3-component coordinate field and backend-strided qdata");
    impl->rstr_x  = rx;
    impl->basis_x = bx;
    impl->kind    = 2;
    CeedCallBackend(CeedElemRestrictionDestroy(&rq));
    CeedCallBackend(CeedBasisDestroy(&bq));
    if (vx != CEED_VECTOR_ACTIVE && vx != CEED_VECTOR_NONE) CeedCallBackend(CeedVectorDestroy(&vx));
    if (vq != CEED_VECTOR_ACTIVE && vq != CEED_VECTOR_NONE) CeedCallBackend(CeedVectorDestroy(&vq));
    CeedCallBackend(CeedQFunctionDestroy(&qf));
    return CEED_ERROR_SUCCESS;
  }
  if (qf_impl->qf_kind == CEED_B200_QF_JIT) {
    CeedCallBackend(OperatorAnalyseJit_B200(op, qf, n_in, in, n_out, out));
    CeedCallBackend(CeedQFunctionDestroy(&qf));
    return CEED_ERROR_SUCCESS;
  }
  CeedCheck(qf_impl->qf_kind >= 0, ceed, CEED_ERROR_UNSUPPORTED, "QFunction is not one of the pointwise kernels compiled for /gpu/cuda/b200");
  {
    CeedElemRestriction ru, rq, ro;
    CeedBasis           bu, bq, bo;
    CeedVector          vu, vq, vo;
    CeedInt             dim, P, Q, nc, ne, comp_stride;
    CeedSize            l_size;
    bool                is_tensor, strided, backend_strides = false, det;
    b200_op_desc        d;
    const CeedScalar   *interp, *grad;
    CeedRestrictionType type;

    CeedCallBackend(FieldParts(in[0], &ru, &bu, &vu));
    CeedCallBackend(FieldParts(in[1], &rq, &bq, &vq));
    CeedCallBackend(FieldParts(out[0], &ro, &bo, &vo));
    CeedCheck(vu == CEED_VECTOR_ACTIVE && vo == CEED_VECTOR_ACTIVE && ru == ro && bu == bo && vq != CEED_VECTOR_ACTIVE && vq != CEED_VECTOR_NONE, ceed,
              CEED_ERROR_UNSUPPORTED, "fused apply needs the active field in and out through one restriction and basis, qdata passive");
    CeedCallBackend(CeedElemRestrictionGetType(ru, &type));
    CeedCallBackend(CeedBasisIsTensor(bu, &is_tensor));
    CeedCallBackend(CeedBasisGetDimension(bu, &dim));
    CeedCallBackend(CeedBasisGetNumNodes1D(bu, &P));
    CeedCallBackend(CeedBasisGetNumQuadraturePoints1D(bu, &Q));
    CeedCallBackend(CeedElemRestrictionIsStrided(rq, &strided));
    if (strided) CeedCallBackend(CeedElemRestrictionHasBackendStrides(rq, &backend_strides));
    CeedCheck(type == CEED_RESTRICTION_STANDARD && is_tensor && dim == 3 && Q == P + 1 && backend_strides, ceed, CEED_ERROR_UNSUPPORTED,
              "fused apply needs an offset restriction, a 3D tensor basis with Q = P + 1 and backend-strided qdata");
    CeedCallBackend(CeedElemRestrictionGetNumComponents(ru, &nc));
    CeedCallBackend(CeedElemRestrictionGetNumElements(ru, &ne));
    CeedCallBackend(CeedElemRestrictionGetCompStride(ru, &comp_stride));
    CeedCallBackend(CeedElemRestrictionGetLVectorSize(ru, &l_size));
    CeedCallBackend(CeedBasisGetInterp1D(bu, &interp));
    CeedCallBackend(CeedBasisGetGrad1D(bu, &grad));
    CeedCallBackend(CeedIsDeterministic(ceed, &det));
    {
      CeedElemRestriction_B200 *r_impl;

      CeedCallBackend(CeedElemRestrictionGetData(ru, &r_impl));
      memset(&d, 0, sizeof d);
      d.qf          = qf_impl->qf_kind;
      d.prec        = B200_F64;
      d.P_1d        = P;
      d.Q_1d        = Q;
      d.num_comp    = nc;
      d.scatter     = det ? B200_SCATTER_DETERMINISTIC : B200_SCATTER_ATOMIC;
      d.num_elem    = ne;
      d.l_size      = l_size;
      d.comp_stride = comp_stride;
      d.offsets     = r_impl->d_offsets;
      d.interp_1d   = interp;
      d.grad_1d     = grad;
    }
    {
      Ceed_B200 *data;

      CeedCallBackend(CeedGetData(ceed, &data));
      // Float-float arithmetic where its kernels exist (centro-symmetric bases); FP64 else.
      if (data->float_float) {
        d.prec = B200_F64X;
        if (b200_op_create(ctx, &d, &impl->op)) d.prec = B200_F64;
      }
    }
    if (d.prec == B200_F64) CeedCallB200(ceed, b200_op_create(ctx, &d, &impl->op));
    impl->qdata   = vq;  // reference kept until destroy
    impl->kind    = 1;
    impl->qf_kind = qf_impl->qf_kind;
    impl->desc    = d;
    CeedCallBackend(CeedElemRestrictionReferenceCopy(ru, &impl->rstr_u));
    CeedCallBackend(CeedElemRestrictionDestroy(&ru));
    CeedCallBackend(CeedElemRestrictionDestroy(&rq));
    CeedCallBackend(CeedElemRestrictionDestroy(&ro));
    CeedCallBackend(CeedBasisDestroy(&bu));
    CeedCallBackend(CeedBasisDestroy(&bq));
    CeedCallBackend(CeedBasisDestroy(&bo));
  }
  CeedCallBackend(CeedQFunctionDestroy(&qf));
  return CEED_ERROR_SUCCESS;
}

static int OperatorApplyCore_B200(CeedOperator op, CeedVector in_vec, CeedVector out_vec, bool add) {
  Ceed               ceed = CeedOperatorReturnCeed(op);
  CeedOperator_B200 *impl;
  const CeedScalar  *du, *dv, *dq;
  b200_ctx           ctx;

  CeedCallBackend(OperatorAnalyse_B200(op));
  CeedCallBackend(CeedOperatorGetData(op, &impl));
  CeedCallBackend(CeedGetB200Context(ceed, &ctx));
  CeedCallBackend(CeedVectorGetDevice_B200(in_vec, false, &du));
  CeedCallBackend(CeedVectorGetDevice_B200(out_vec, true, &dv));
  if (impl->kind == 1) {
    CeedCallBackend(CeedVectorGetDevice_B200(impl->qdata, false, &dq));
    CeedCallB200(ceed, b200_op_apply(impl->op, du, (void *)dv, dq, NULL, add ? 1 : 0));
  } else if (impl->kind == 3) {
    const void *passive[8] = {NULL};

    for (CeedInt i = 0; i < impl->num_passive; i++) CeedCallBackend(CeedVectorGetDevice_B200(impl->passive[i], false, (const CeedScalar **)&passive[i]));
    if (impl->ctx_size) {
      CeedQFunction qf;
      const void   *h_ctx;

      CeedCallBackend(CeedOperatorGetQFunction(op, &qf));
      CeedCallBackend(CeedQFunctionGetInnerContextData(qf, CEED_MEM_HOST, &h_ctx));
      CeedCallB200(ceed, b200_copy(ctx, impl->d_ctx, h_ctx, impl->ctx_size, B200_COPY_H2D));
      CeedCallBackend(CeedQFunctionRestoreInnerContextData(qf, &h_ctx));
      CeedCallBackend(CeedQFunctionDestroy(&qf));
    }
    CeedCallB200(ceed, b200_op_apply_jit(impl->op, du, (void *)dv, passive, impl->d_ctx, add ? 1 : 0));
  } else if (impl->kind == 2) {
    CeedQFunction             qf;
    CeedQFunction_B200       *qf_impl;
    CeedElemRestriction_B200 *rx;
    const CeedScalar         *interp, *grad, *qw;
    CeedInt                   ne, Q, comp_stride;

    CeedCheck(!add, ceed, CEED_ERROR_UNSUPPORTED, "geometric factors are computed with CeedOperatorApply");
    CeedCallBackend(CeedOperatorGetQFunction(op, &qf));
    CeedCallBackend(CeedQFunctionGetData(qf, &qf_impl));
    CeedCallBackend(CeedElemRestrictionGetData(impl->rstr_x, &rx));
    CeedCallBackend(CeedElemRestrictionGetNumElements(impl->rstr_x, &ne));
    CeedCallBackend(CeedElemRestrictionGetCompStride(impl->rstr_x, &comp_stride));
    CeedCallBackend(CeedBasisGetNumQuadraturePoints1D(impl->basis_x, &Q));
    CeedCallBackend(CeedBasisGetInterp1D(impl->basis_x, &interp));
    CeedCallBackend(CeedBasisGetGrad1D(impl->basis_x, &grad));
    CeedCallBackend(CeedBasisGetQWeights(impl->basis_x, &qw));
    CeedCallB200(ceed, b200_qdata_build(ctx, qf_impl->build_poisson, ne, Q, interp, grad, qw, rx->d_offsets, comp_stride, du, (double *)dv));
    CeedCallBackend(CeedQFunctionDestroy(&qf));
  } else {
    return CeedError(ceed, CEED_ERROR_UNSUPPORTED, "operator not supported by /gpu/cuda/b200");
  }
  return CEED_ERROR_SUCCESS;
}

static int CeedOperatorApply_B200(CeedOperator op, CeedVector in_vec, CeedVector out_vec, CeedRequest *request) {
  (void)request;
  return OperatorApplyCore_B200(op, in_vec, out_vec, false);
}

static int CeedOperatorApplyAdd_B200(CeedOperator op, CeedVector in_vec, CeedVector out_vec, CeedRequest *request) {
  (void)request;
  return OperatorApplyCore_B200(op, in_vec, out_vec, true);
}

// CeedOperatorLinearAssembleAddDiagonal (interface/ceed-preconditioning.c:2395) for the fused gallery operators:
// diag += the operator's diagonal, by b200_assemble_diagonal (deterministic through the restriction's inverse-offset
// plan when the Ceed is deterministic).
static int CeedOperatorLinearAssembleAddDiagonal_B200(CeedOperator op, CeedVector assembled, CeedRequest *request) {
  Ceed                      ceed = CeedOperatorReturnCeed(op);
  CeedOperator_B200        *impl;
  CeedElemRestriction_B200 *r_impl;
  const CeedScalar         *dq, *dd;
  b200_ctx                  ctx;
  void                     *tmp = NULL;
  bool                      det;
  int                       poisson;

  (void)request;
  CeedCallBackend(OperatorAnalyse_B200(op));
  CeedCallBackend(CeedOperatorGetData(op, &impl));
  CeedCheck(impl->kind == 1, ceed, CEED_ERROR_UNSUPPORTED, "diagonal assembly on /gpu/cuda/b200 covers the fused gallery operators");
  CeedCallBackend(CeedGetB200Context(ceed, &ctx));
  CeedCallBackend(CeedIsDeterministic(ceed, &det));
  CeedCallBackend(CeedElemRestrictionGetData(impl->rstr_u, &r_impl));
  const b200_op_desc *d = &impl->desc;
  if (det && !r_impl->plan) {
    CeedInt elem_size;

    CeedCallBackend(CeedElemRestrictionGetElementSize(impl->rstr_u, &elem_size));
    CeedCallB200(ceed, b200_plan_create(ctx, d->num_elem, elem_size, d->num_comp, d->comp_stride, d->l_size, r_impl->h_offsets, r_impl->d_offsets,
                                        &r_impl->plan));
  }
  poisson = impl->qf_kind == B200_QF_POISSON || impl->qf_kind == B200_QF_VECPOISSON;
  CeedCallBackend(CeedVectorGetDevice_B200(impl->qdata, false, &dq));
  CeedCallBackend(CeedVectorGetDevice_B200(assembled, true, &dd));
  CeedCallB200(ceed, b200_alloc(ctx, sizeof(double) * (size_t)d->l_size, &tmp));
  int st = b200_assemble_diagonal(ctx, poisson, d->P_1d, d->Q_1d, d->num_elem, d->num_comp, d->comp_stride, d->l_size, d->interp_1d, d->grad_1d,
                                  d->offsets, dq, NULL, (double *)tmp, det ? r_impl->plan : NULL);
  if (!st) st = b200_vec_axpy(ctx, B200_F64, d->l_size, 1.0, tmp, (void *)dd);
  b200_free(ctx, tmp);
  CeedCheck(!st, ceed, CEED_ERROR_BACKEND, "b200_assemble_diagonal: %s", b200_last_error());
  return CEED_ERROR_SUCCESS;
}

static int CeedOperatorDestroy_B200(CeedOperator op) {
  CeedOperator_B200 *impl;

  CeedCallBackend(CeedOperatorGetData(op, &impl));
  if (impl->op) b200_op_destroy(impl->op);
  if (impl->qdata) CeedCallBackend(CeedVectorDestroy(&impl->qdata));
  for (CeedInt i = 0; i < impl->num_passive; i++) CeedCallBackend(CeedVectorDestroy(&impl->passive[i]));
  if (impl->d_ctx) {
    Ceed     ceed = CeedOperatorReturnCeed(op);
    b200_ctx ctx;

    CeedCallBackend(CeedGetB200Context(ceed, &ctx));
    b200_free(ctx, impl->d_ctx);
  }
  if (impl->rstr_x) CeedCallBackend(CeedElemRestrictionDestroy(&impl->rstr_x));
  if (impl->rstr_u) CeedCallBackend(CeedElemRestrictionDestroy(&impl->rstr_u));
  if (impl->basis_x) CeedCallBackend(CeedBasisDestroy(&impl->basis_x));
  CeedCallBackend(CeedFree(&impl));
  return CEED_ERROR_SUCCESS;
}

int CeedOperatorCreate_B200(CeedOperator op) {
  Ceed               ceed;
  CeedOperator_B200 *impl;

  CeedCallBackend(CeedOperatorGetCeed(op, &ceed));
  CeedCallBackend(CeedCalloc(1, &impl));
  CeedCallBackend(CeedOperatorSetData(op, impl));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Operator", op, "Apply", CeedOperatorApply_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Operator", op, "ApplyAdd", CeedOperatorApplyAdd_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Operator", op, "LinearAssembleAddDiagonal", CeedOperatorLinearAssembleAddDiagonal_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Operator", op, "Destroy", CeedOperatorDestroy_B200));
  CeedCallBackend(CeedDestroy(&ceed));
  return CEED_ERROR_SUCCESS;
}
