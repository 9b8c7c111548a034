// Tensor H1 CeedBasis for `/gpu/cuda/b200` (dim 1..3): INTERP, GRAD and WEIGHT through b200_basis_apply.
// Non-tensor, H(div) and H(curl) bases are not created (CEED_ERROR_UNSUPPORTED from the frontend).
#include "ceed-b200-backend.h"

static int BasisApplyCore(CeedBasis basis, bool add, CeedInt num_elem, CeedTransposeMode t_mode, CeedEvalMode eval_mode, CeedVector u,
                          CeedVector v) {
  CeedBasis_B200   *impl;
  Ceed              ceed = CeedBasisReturnCeed(basis);
  const CeedScalar *du = NULL, *dv;
  int               em;

  CeedCallBackend(CeedBasisGetData(basis, &impl));
  switch (eval_mode) {
    case CEED_EVAL_INTERP: em = B200_EVAL_INTERP; break;
    case CEED_EVAL_GRAD: em = B200_EVAL_GRAD; break;
    case CEED_EVAL_WEIGHT: em = B200_EVAL_WEIGHT; break;
    default: return CeedError(ceed, CEED_ERROR_BACKEND, "%s not supported by the tensor H1 basis", CeedEvalModes[eval_mode]);
  }
  if (u != CEED_VECTOR_NONE) CeedCallBackend(CeedVectorGetDevice_B200(u, false, &du));
  CeedCallBackend(CeedVectorGetDevice_B200(v, true, &dv));
  CeedCallB200(ceed, b200_basis_apply(impl->basis, B200_F64, num_elem, t_mode == CEED_TRANSPOSE ? B200_TRANSPOSE : B200_NOTRANSPOSE, em, add ? 1 : 0,
                                      du, (void *)dv));
  return CEED_ERROR_SUCCESS;
}

static int CeedBasisApply_B200(CeedBasis basis, CeedInt num_elem, CeedTransposeMode t_mode, CeedEvalMode eval_mode, CeedVector u, CeedVector v) {
  return BasisApplyCore(basis, false, num_elem, t_mode, eval_mode, u, v);
}

static int CeedBasisApplyAdd_B200(CeedBasis basis, CeedInt num_elem, CeedTransposeMode t_mode, CeedEvalMode eval_mode, CeedVector u, CeedVector v) {
  return BasisApplyCore(basis, true, num_elem, t_mode, eval_mode, u, v);
}

static int CeedBasisDestroy_B200(CeedBasis basis) {
  CeedBasis_B200 *impl;

  CeedCallBackend(CeedBasisGetData(basis, &impl));
  b200_basis_destroy(impl->basis);
  CeedCallBackend(CeedFree(&impl));
  return CEED_ERROR_SUCCESS;
}

int CeedBasisCreateTensorH1_B200(CeedInt dim, CeedInt P_1d, CeedInt Q_1d, const CeedScalar *interp_1d, const CeedScalar *grad_1d,
                                 const CeedScalar *q_ref_1d, const CeedScalar *q_weight_1d, CeedBasis basis) {
  Ceed            ceed;
  CeedBasis_B200 *impl;
  CeedInt         num_comp;
  b200_ctx        ctx;

  CeedCallBackend(CeedBasisGetCeed(basis, &ceed));
  CeedCallBackend(CeedGetB200Context(ceed, &ctx));
  CeedCallBackend(CeedBasisGetNumComponents(basis, &num_comp));
  CeedCallBackend(CeedCalloc(1, &impl));
  CeedCallB200(ceed, b200_basis_create(ctx, dim, P_1d, Q_1d, num_comp, interp_1d, grad_1d, q_weight_1d, &impl->basis));
  (void)q_ref_1d;
  CeedCallBackend(CeedBasisSetData(basis, impl));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Basis", basis, "Apply", CeedBasisApply_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Basis", basis, "ApplyAdd", CeedBasisApplyAdd_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Basis", basis, "Destroy", CeedBasisDestroy_B200));
  CeedCallBackend(CeedDestroy(&ceed));
  return CEED_ERROR_SUCCESS;
}
