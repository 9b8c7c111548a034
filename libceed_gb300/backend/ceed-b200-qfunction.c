// CeedQFunction and CeedQFunctionContext for `/gpu/cuda/b200`.
//
// The pointwise kernels of this backend are compiled in: the gallery QFunctions of the hot path, recognised by kernel
// name (MassApply, Poisson3DApply, Vector3MassApply, Vector3Poisson3DApply; Mass3DBuild and Poisson3DBuild run as the
// geometric-factor setup).  Any other QFunction created from a source file (CeedQFunctionCreateInterior with
// "file.h:Name") is compiled at run time with NVRTC into the fused operator kernel when an operator using it is first
// applied (b200_op_create_jit).  Standalone CeedQFunctionApply on Q-vectors calls b200_qf_apply for the gallery
// kernels; for user QFunctions it returns CEED_ERROR_UNSUPPORTED (no CPU fallback).  Contexts hold host data; the
// operator copies the context to the device before each run-time compiled apply.
#include <stdlib.h>
#include <string.h>

#include "ceed-b200-backend.h"

static int QFunctionKind(const char *name, int *kind, int *build_poisson) {
  *build_poisson = 0;
  if (!strcmp(name, "MassApply")) *kind = B200_QF_MASS;
  else if (!strcmp(name, "Poisson3DApply")) *kind = B200_QF_POISSON;
  else if (!strcmp(name, "Vector3MassApply")) *kind = B200_QF_VECMASS;
  else if (!strcmp(name, "Vector3Poisson3DApply")) *kind = B200_QF_VECPOISSON;
  else if (!strcmp(name, "Mass3DBuild")) *kind = -1;
  else if (!strcmp(name, "Poisson3DBuild")) *kind = -1, *build_poisson = 1;
  else *kind = -2;
  return CEED_ERROR_SUCCESS;
}

static int CeedQFunctionApply_B200(CeedQFunction qf, CeedInt Q, CeedVector *U, CeedVector *V) {
  CeedQFunction_B200 *impl;
  Ceed                ceed = CeedQFunctionReturnCeed(qf);
  b200_ctx            ctx;
  CeedInt             num_in, num_out;
  const void         *in[3] = {NULL, NULL, NULL};
  void               *out[1];

  CeedCallBackend(CeedQFunctionGetData(qf, &impl));
  CeedCallBackend(CeedGetB200Context(ceed, &ctx));
  CeedCheck(impl->qf_kind >= 0, ceed, CEED_ERROR_UNSUPPORTED, "/gpu/cuda/b200 cannot apply this QFunction on Q-vectors");
  CeedCallBackend(CeedQFunctionGetNumArgs(qf, &num_in, &num_out));
  for (CeedInt i = 0; i < num_in && i < 3; i++) CeedCallBackend(CeedVectorGetDevice_B200(U[i], false, (const CeedScalar **)&in[i]));
  CeedCallBackend(CeedVectorGetDevice_B200(V[0], true, (const CeedScalar **)&out[0]));
  CeedCallB200(ceed, b200_qf_apply(ctx, B200_F64, impl->qf_kind, Q, in, out));
  return CEED_ERROR_SUCCESS;
}

static int CeedQFunctionDestroy_B200(CeedQFunction qf) {
  CeedQFunction_B200 *impl;

  CeedCallBackend(CeedQFunctionGetData(qf, &impl));
  CeedCallBackend(CeedFree(&impl));
  return CEED_ERROR_SUCCESS;
}

int CeedQFunctionCreate_B200(CeedQFunction qf) {
  Ceed                ceed;
  CeedQFunction_B200 *impl;
  const char         *name;

  CeedCallBackend(CeedQFunctionGetCeed(qf, &ceed));
  CeedCallBackend(CeedCalloc(1, &impl));
  CeedCallBackend(CeedQFunctionGetKernelName(qf, &name));
  CeedCallBackend(QFunctionKind(name, &impl->qf_kind, &impl->build_poisson));
  if (impl->qf_kind == -2) {
    const char *source = NULL;

    CeedCallBackend(CeedQFunctionGetSourcePath(qf, &source));
    if (source && source[0]) impl->qf_kind = CEED_B200_QF_JIT;
  }
  CeedCallBackend(CeedQFunctionSetData(qf, impl));
  CeedCallBackend(CeedSetBackendFunction(ceed, "QFunction", qf, "Apply", CeedQFunctionApply_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "QFunction", qf, "Destroy", CeedQFunctionDestroy_B200));
  CeedCallBackend(CeedDestroy(&ceed));
  return CEED_ERROR_SUCCESS;
}

// ---- QFunctionContext: host memory only ---------------------------------------------------------------------------
typedef struct {
  void *data, *owned, *borrowed;
} CeedQFunctionContext_B200;

static int CtxHasValidData(CeedQFunctionContext ctx, bool *valid) {
  CeedQFunctionContext_B200 *impl;

  CeedCallBackend(CeedQFunctionContextGetBackendData(ctx, &impl));
  *valid = impl->data != NULL;
  return CEED_ERROR_SUCCESS;
}

static int CtxHasBorrowed(CeedQFunctionContext ctx, CeedMemType mem_type, bool *has) {
  CeedQFunctionContext_B200 *impl;

  CeedCallBackend(CeedQFunctionContextGetBackendData(ctx, &impl));
  *has = mem_type == CEED_MEM_HOST && impl->borrowed != NULL;
  return CEED_ERROR_SUCCESS;
}

static int CtxSetData(CeedQFunctionContext ctx, CeedMemType mem_type, CeedCopyMode copy_mode, void *data) {
  CeedQFunctionContext_B200 *impl;
  size_t                     size;

  CeedCallBackend(CeedQFunctionContextGetBackendData(ctx, &impl));
  CeedCheck(mem_type == CEED_MEM_HOST, CeedQFunctionContextReturnCeed(ctx), CEED_ERROR_UNSUPPORTED, "contexts live in host memory on /gpu/cuda/b200");
  CeedCallBackend(CeedQFunctionContextGetContextSize(ctx, &size));
  CeedCallBackend(CeedFree(&impl->owned));
  impl->borrowed = NULL;
  if (copy_mode == CEED_COPY_VALUES) {
    CeedCallBackend(CeedMallocArray(1, size ? size : 1, &impl->owned));
    memcpy(impl->owned, data, size);
    impl->data = impl->owned;
  } else if (copy_mode == CEED_OWN_POINTER) {
    impl->owned = impl->data = data;
  } else {
    impl->borrowed = impl->data = data;
  }
  return CEED_ERROR_SUCCESS;
}

static int CtxTakeData(CeedQFunctionContext ctx, CeedMemType mem_type, void *data) {
  CeedQFunctionContext_B200 *impl;

  CeedCallBackend(CeedQFunctionContextGetBackendData(ctx, &impl));
  *(void **)data = impl->borrowed;
  impl->borrowed = impl->data = NULL;
  (void)mem_type;
  return CEED_ERROR_SUCCESS;
}

static int CtxGetData(CeedQFunctionContext ctx, CeedMemType mem_type, void *data) {
  CeedQFunctionContext_B200 *impl;

  CeedCallBackend(CeedQFunctionContextGetBackendData(ctx, &impl));
  CeedCheck(mem_type == CEED_MEM_HOST, CeedQFunctionContextReturnCeed(ctx), CEED_ERROR_UNSUPPORTED, "contexts live in host memory on /gpu/cuda/b200");
  *(void **)data = impl->data;
  return CEED_ERROR_SUCCESS;
}

static int CtxRestoreData(CeedQFunctionContext ctx) { return CEED_ERROR_SUCCESS; }

static int CtxDestroy(CeedQFunctionContext ctx) {
  CeedQFunctionContext_B200 *impl;

  CeedCallBackend(CeedQFunctionContextGetBackendData(ctx, &impl));
  CeedCallBackend(CeedFree(&impl->owned));
  CeedCallBackend(CeedFree(&impl));
  return CEED_ERROR_SUCCESS;
}

int CeedQFunctionContextCreate_B200(CeedQFunctionContext ctx) {
  CeedQFunctionContext_B200 *impl;
  Ceed                       ceed;

  CeedCallBackend(CeedQFunctionContextGetCeed(ctx, &ceed));
  CeedCallBackend(CeedCalloc(1, &impl));
  CeedCallBackend(CeedQFunctionContextSetBackendData(ctx, impl));
  CeedCallBackend(CeedSetBackendFunction(ceed, "QFunctionContext", ctx, "HasValidData", CtxHasValidData));
  CeedCallBackend(CeedSetBackendFunction(ceed, "QFunctionContext", ctx, "HasBorrowedDataOfType", CtxHasBorrowed));
  CeedCallBackend(CeedSetBackendFunction(ceed, "QFunctionContext", ctx, "SetData", CtxSetData));
  CeedCallBackend(CeedSetBackendFunction(ceed, "QFunctionContext", ctx, "TakeData", CtxTakeData));
  CeedCallBackend(CeedSetBackendFunction(ceed, "QFunctionContext", ctx, "GetData", CtxGetData));
  CeedCallBackend(CeedSetBackendFunction(ceed, "QFunctionContext", ctx, "GetDataRead", CtxGetData));
  CeedCallBackend(CeedSetBackendFunction(ceed, "QFunctionContext", ctx, "RestoreData", CtxRestoreData));
  CeedCallBackend(CeedSetBackendFunction(ceed, "QFunctionContext", ctx, "RestoreDataRead", CtxRestoreData));
  CeedCallBackend(CeedSetBackendFunction(ceed, "QFunctionContext", ctx, "Destroy", CtxDestroy));
  CeedCallBackend(CeedDestroy(&ceed));
  return CEED_ERROR_SUCCESS;
}
