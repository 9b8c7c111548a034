// Registration and initialization of the libCEED backend `/gpu/cuda/b200`.
//
// Registered through CeedRegister (include/ceed/backend.h:248) like backends/cuda-ref/ceed-cuda-ref.c:72, either from
// a `CEED_BACKEND(CeedRegister_B200, 1, "/gpu/cuda/b200")` line in backends/ceed-backend-list-b200.h or by calling
// CeedRegister_B200() before CeedInit.  There is no delegate and no fallback Ceed: anything the backend cannot run
// returns CEED_ERROR_UNSUPPORTED.
#include <stdlib.h>
#include <string.h>

#include "ceed-b200-backend.h"

int CeedGetB200Context(Ceed ceed, b200_ctx *ctx) {
  Ceed_B200 *data;

  CeedCallBackend(CeedGetData(ceed, &data));
  *ctx = data->ctx;
  return CEED_ERROR_SUCCESS;
}

static int CeedGetPreferredMemType_B200(CeedMemType *mem_type) {
  *mem_type = CEED_MEM_DEVICE;
  return CEED_ERROR_SUCCESS;
}

static int CeedSetStream_B200(Ceed ceed, void *stream) {
  b200_ctx ctx;

  CeedCallBackend(CeedGetB200Context(ceed, &ctx));
  CeedCallB200(ceed, b200_ctx_set_stream(ctx, stream));
  return CEED_ERROR_SUCCESS;
}

static int CeedDestroy_B200(Ceed ceed) {
  Ceed_B200 *data;

  CeedCallBackend(CeedGetData(ceed, &data));
  if (data->ctx) b200_ctx_destroy(data->ctx);
  CeedCallBackend(CeedFree(&data));
  return CEED_ERROR_SUCCESS;
}

static int CeedInit_B200(const char *resource, Ceed ceed) {
  char      *resource_root;
  Ceed_B200 *data;
  int        device_id = 0;

  CeedCallBackend(CeedGetResourceRoot(ceed, resource, ":", &resource_root));
  CeedCheck(!strcmp(resource_root, "/gpu/cuda/b200"), ceed, CEED_ERROR_BACKEND, "B200 backend cannot use resource: %s", resource);
  CeedCallBackend(CeedFree(&resource_root));
  const char *dev = strstr(resource, ":device_id=");
  if (dev) device_id = atoi(dev + strlen(":device_id="));
  // ":arithmetic=float-float": fused applies on centro-symmetric bases run the float-float (B200_F64X) kernels on the
  // same double vectors (within ~1e-13 relative of FP64); every other operator keeps FP64.
  const char *arith = strstr(resource, ":arithmetic=");
  CeedCheck(!arith || !strncmp(arith + strlen(":arithmetic="), "float-float", 11) || !strncmp(arith + strlen(":arithmetic="), "fp64", 4), ceed,
            CEED_ERROR_BACKEND, "B200 backend: arithmetic must be fp64 or float-float (resource %s)", resource);

  CeedCallBackend(CeedCalloc(1, &data));
  data->device_id   = device_id;
  data->float_float = arith && !strncmp(arith + strlen(":arithmetic="), "float-float", 11);
  if (b200_ctx_create(device_id, &data->ctx)) {
    CeedCallBackend(CeedFree(&data));
    return CeedError(ceed, CEED_ERROR_BACKEND, "b200_ctx_create: %s", b200_last_error());
  }
  CeedCallBackend(CeedSetData(ceed, data));
  // The deterministic inverse-offset scatter is available; atomics are the default (CeedSetDeterministic is for
  // backends whose every apply is reproducible, so it stays unset).
  CeedCallBackend(CeedSetBackendFunction(ceed, "Ceed", ceed, "GetPreferredMemType", CeedGetPreferredMemType_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Ceed", ceed, "SetStream", CeedSetStream_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Ceed", ceed, "VectorCreate", CeedVectorCreate_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Ceed", ceed, "ElemRestrictionCreate", CeedElemRestrictionCreate_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Ceed", ceed, "BasisCreateTensorH1", CeedBasisCreateTensorH1_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Ceed", ceed, "QFunctionCreate", CeedQFunctionCreate_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Ceed", ceed, "QFunctionContextCreate", CeedQFunctionContextCreate_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Ceed", ceed, "OperatorCreate", CeedOperatorCreate_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Ceed", ceed, "Destroy", CeedDestroy_B200));
  return CEED_ERROR_SUCCESS;
}

// Priority 30: `/gpu/cuda` keeps resolving to the reference's own CUDA backends; `/gpu/cuda/b200` selects this one.
CEED_INTERN int CeedRegister_B200(void) { return CeedRegister("/gpu/cuda/b200", CeedInit_B200, 30); }

// Out-of-tree registration: a program linked against a stock libCEED calls this once before CeedInit.
int CeedB200Register(void) { return CeedRegister_B200(); }
