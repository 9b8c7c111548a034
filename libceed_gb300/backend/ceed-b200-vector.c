// CeedVector for `/gpu/cuda/b200`: a host mirror and a device array with validity flags; arithmetic runs on the device
// through b200_vec_* (replacing backends/cuda-ref/ceed-cuda-ref-vector.c and kernels/cuda-ref-vector.cu).
#include <stdlib.h>
#include <string.h>

#include "ceed-b200-backend.h"

static int VecData(CeedVector vec, CeedVector_B200 **impl, b200_ctx *ctx, CeedSize *n) {
  Ceed ceed;

  CeedCallBackend(CeedVectorGetData(vec, impl));
  CeedCallBackend(CeedVectorGetCeed(vec, &ceed));
  CeedCallBackend(CeedGetB200Context(ceed, ctx));
  CeedCallBackend(CeedDestroy(&ceed));
  if (n) CeedCallBackend(CeedVectorGetLength(vec, n));
  return CEED_ERROR_SUCCESS;
}

static int SyncD2H(CeedVector vec) {
  CeedVector_B200 *impl;
  b200_ctx         ctx;
  CeedSize         n;

  CeedCallBackend(VecData(vec, &impl, &ctx, &n));
  if (!impl->h_array) {
    CeedCallBackend(CeedMalloc(n ? n : 1, &impl->h_owned));
    impl->h_array = impl->h_owned;
  }
  if (impl->d_valid && !impl->h_valid) {
    if (b200_copy(ctx, impl->h_array, impl->d_array, sizeof(CeedScalar) * (size_t)n, B200_COPY_D2H) || b200_ctx_sync(ctx))
      return CeedError(CeedVectorReturnCeed(vec), CEED_ERROR_BACKEND, "%s", b200_last_error());
  }
  impl->h_valid = true;
  return CEED_ERROR_SUCCESS;
}

static int SyncH2D(CeedVector vec) {
  CeedVector_B200 *impl;
  b200_ctx         ctx;
  CeedSize         n;

  CeedCallBackend(VecData(vec, &impl, &ctx, &n));
  if (!impl->d_array) {
    if (b200_alloc(ctx, sizeof(CeedScalar) * (size_t)(n ? n : 1), (void **)&impl->d_owned))
      return CeedError(CeedVectorReturnCeed(vec), CEED_ERROR_BACKEND, "%s", b200_last_error());
    impl->d_array = impl->d_owned;
  }
  if (impl->h_valid && !impl->d_valid) {
    if (b200_copy(ctx, impl->d_array, impl->h_array, sizeof(CeedScalar) * (size_t)n, B200_COPY_H2D))
      return CeedError(CeedVectorReturnCeed(vec), CEED_ERROR_BACKEND, "%s", b200_last_error());
  }
  impl->d_valid = true;
  return CEED_ERROR_SUCCESS;
}

static int CeedVectorHasValidArray_B200(CeedVector vec, bool *has_valid_array) {
  CeedVector_B200 *impl;

  CeedCallBackend(CeedVectorGetData(vec, &impl));
  *has_valid_array = impl->h_valid || impl->d_valid;
  return CEED_ERROR_SUCCESS;
}

static int CeedVectorHasBorrowedArrayOfType_B200(CeedVector vec, CeedMemType mem_type, bool *has) {
  CeedVector_B200 *impl;

  CeedCallBackend(CeedVectorGetData(vec, &impl));
  *has = mem_type == CEED_MEM_HOST ? impl->h_borrowed != NULL : impl->d_borrowed != NULL;
  return CEED_ERROR_SUCCESS;
}

static int CeedVectorSetArray_B200(CeedVector vec, CeedMemType mem_type, CeedCopyMode copy_mode, CeedScalar *array) {
  CeedVector_B200 *impl;
  b200_ctx         ctx;
  CeedSize         n;

  CeedCallBackend(VecData(vec, &impl, &ctx, &n));
  impl->h_valid = impl->d_valid = false;
  if (mem_type == CEED_MEM_HOST) {
    if (copy_mode == CEED_COPY_VALUES) {
      if (!impl->h_owned) CeedCallBackend(CeedMalloc(n ? n : 1, &impl->h_owned));
      impl->h_borrowed = NULL;
      impl->h_array    = impl->h_owned;
      if (array) memcpy(impl->h_array, array, sizeof(CeedScalar) * (size_t)n);
    } else {
      CeedCallBackend(CeedFree(&impl->h_owned));
      if (copy_mode == CEED_OWN_POINTER) {
        impl->h_owned    = array;
        impl->h_borrowed = NULL;
      } else {
        impl->h_borrowed = array;
      }
      impl->h_array = array;
    }
    impl->h_valid = array != NULL;
  } else {
    if (copy_mode == CEED_COPY_VALUES) {
      if (!impl->d_owned && b200_alloc(ctx, sizeof(CeedScalar) * (size_t)(n ? n : 1), (void **)&impl->d_owned))
        return CeedError(CeedVectorReturnCeed(vec), CEED_ERROR_BACKEND, "%s", b200_last_error());
      impl->d_borrowed = NULL;
      impl->d_array    = impl->d_owned;
      if (array) CeedCallB200(CeedVectorReturnCeed(vec), b200_copy(ctx, impl->d_array, array, sizeof(CeedScalar) * (size_t)n, B200_COPY_D2D));
    } else {
      if (impl->d_owned) b200_free(ctx, impl->d_owned);
      impl->d_owned = NULL;
      if (copy_mode == CEED_OWN_POINTER) {
        impl->d_owned    = array;
        impl->d_borrowed = NULL;
      } else {
        impl->d_borrowed = array;
      }
      impl->d_array = array;
    }
    impl->d_valid = array != NULL;
  }
  return CEED_ERROR_SUCCESS;
}

static int CeedVectorTakeArray_B200(CeedVector vec, CeedMemType mem_type, CeedScalar **array) {
  CeedVector_B200 *impl;

  CeedCallBackend(CeedVectorGetData(vec, &impl));
  if (mem_type == CEED_MEM_HOST) {
    CeedCallBackend(SyncD2H(vec));
    *array           = impl->h_borrowed;
    impl->h_borrowed = impl->h_array = NULL;
    impl->h_valid    = false;
  } else {
    CeedCallBackend(SyncH2D(vec));
    *array           = impl->d_borrowed;
    impl->d_borrowed = impl->d_array = NULL;
    impl->d_valid    = false;
  }
  return CEED_ERROR_SUCCESS;
}

static int CeedVectorSyncArray_B200(CeedVector vec, CeedMemType mem_type) {
  return mem_type == CEED_MEM_HOST ? SyncD2H(vec) : SyncH2D(vec);
}

static int GetArrayCore(CeedVector vec, CeedMemType mem_type, bool write_only, bool read_only, CeedScalar **array) {
  CeedVector_B200 *impl;

  CeedCallBackend(CeedVectorGetData(vec, &impl));
  if (mem_type == CEED_MEM_HOST) {
    if (write_only) {
      CeedSize n;
      CeedCallBackend(CeedVectorGetLength(vec, &n));
      if (!impl->h_array) {
        CeedCallBackend(CeedMalloc(n ? n : 1, &impl->h_owned));
        impl->h_array = impl->h_owned;
      }
      impl->h_valid = true;
    } else {
      CeedCallBackend(SyncD2H(vec));
    }
    if (!read_only) impl->d_valid = false;
    *array = impl->h_array;
  } else {
    if (write_only) {
      CeedVector_B200 *i2;
      b200_ctx         ctx;
      CeedSize         n;
      CeedCallBackend(VecData(vec, &i2, &ctx, &n));
      if (!impl->d_array) {
        CeedCallB200(CeedVectorReturnCeed(vec), b200_alloc(ctx, sizeof(CeedScalar) * (size_t)(n ? n : 1), (void **)&impl->d_owned));
        impl->d_array = impl->d_owned;
      }
      impl->d_valid = true;
    } else {
      CeedCallBackend(SyncH2D(vec));
    }
    if (!read_only) impl->h_valid = false;
    *array = impl->d_array;
  }
  return CEED_ERROR_SUCCESS;
}

static int CeedVectorGetArray_B200(CeedVector vec, CeedMemType mem_type, CeedScalar **array) { return GetArrayCore(vec, mem_type, false, false, array); }
static int CeedVectorGetArrayRead_B200(CeedVector vec, CeedMemType mem_type, const CeedScalar **array) {
  return GetArrayCore(vec, mem_type, false, true, (CeedScalar **)array);
}
static int CeedVectorGetArrayWrite_B200(CeedVector vec, CeedMemType mem_type, CeedScalar **array) { return GetArrayCore(vec, mem_type, true, false, array); }
static int CeedVectorRestoreArray_B200(CeedVector vec) { return CEED_ERROR_SUCCESS; }
static int CeedVectorRestoreArrayRead_B200(CeedVector vec) { return CEED_ERROR_SUCCESS; }

// Device pointer for kernels; write = true invalidates the host mirror.
int CeedVectorGetDevice_B200(CeedVector vec, bool write, const CeedScalar **d_array) {
  return GetArrayCore(vec, CEED_MEM_DEVICE, false, !write, (CeedScalar **)d_array);
}

static int CeedVectorSetValue_B200(CeedVector vec, CeedScalar value) {
  CeedVector_B200 *impl;
  b200_ctx         ctx;
  CeedSize         n;
  CeedScalar      *d;

  CeedCallBackend(VecData(vec, &impl, &ctx, &n));
  CeedCallBackend(GetArrayCore(vec, CEED_MEM_DEVICE, true, false, &d));
  CeedCallB200(CeedVectorReturnCeed(vec), b200_vec_set_value(ctx, B200_F64, n, d, value));
  return CEED_ERROR_SUCCESS;
}

// Strided set and copy keep the entries outside the range, so the vector must hold data already (as
// backends/cuda-ref/ceed-cuda-ref-vector.c:243-375 requires); stop = -1 is resolved by b200_vec_*_strided.
static int CeedVectorSetValueStrided_B200(CeedVector vec, CeedSize start, CeedSize stop, CeedSize step, CeedScalar value) {
  CeedVector_B200  *impl;
  b200_ctx          ctx;
  CeedSize          n;
  const CeedScalar *d;

  CeedCallBackend(VecData(vec, &impl, &ctx, &n));
  CeedCheck(impl->h_valid || impl->d_valid, CeedVectorReturnCeed(vec), CEED_ERROR_BACKEND, "CeedVector must have valid data set");
  CeedCallBackend(CeedVectorGetDevice_B200(vec, true, &d));
  CeedCallB200(CeedVectorReturnCeed(vec), b200_vec_set_value_strided(ctx, B200_F64, n, start, stop, step, (void *)d, value));
  return CEED_ERROR_SUCCESS;
}

static int CeedVectorCopyStrided_B200(CeedVector vec, CeedSize start, CeedSize stop, CeedSize step, CeedVector vec_copy) {
  CeedVector_B200  *impl, *impl_copy;
  b200_ctx          ctx;
  CeedSize          n, n_copy;
  const CeedScalar *dx, *dy;

  CeedCallBackend(VecData(vec, &impl, &ctx, &n));
  CeedCallBackend(CeedVectorGetData(vec_copy, &impl_copy));
  CeedCallBackend(CeedVectorGetLength(vec_copy, &n_copy));
  CeedCheck(impl->h_valid || impl->d_valid, CeedVectorReturnCeed(vec), CEED_ERROR_BACKEND, "CeedVector must have valid data set");
  CeedCheck(impl_copy->h_valid || impl_copy->d_valid, CeedVectorReturnCeed(vec_copy), CEED_ERROR_BACKEND,
            "CeedVector must have valid data set");
  CeedCallBackend(CeedVectorGetDevice_B200(vec, false, &dx));
  CeedCallBackend(CeedVectorGetDevice_B200(vec_copy, true, &dy));
  CeedCallB200(CeedVectorReturnCeed(vec), b200_vec_copy_strided(ctx, B200_F64, n < n_copy ? n : n_copy, start, stop, step, dx, (void *)dy));
  return CEED_ERROR_SUCCESS;
}

static int CeedVectorNorm_B200(CeedVector vec, CeedNormType type, CeedScalar *norm) {
  CeedVector_B200  *impl;
  b200_ctx          ctx;
  CeedSize          n;
  const CeedScalar *d;

  CeedCallBackend(VecData(vec, &impl, &ctx, &n));
  CeedCallBackend(CeedVectorGetDevice_B200(vec, false, &d));
  const int t = type == CEED_NORM_1 ? B200_NORM_1 : type == CEED_NORM_2 ? B200_NORM_2 : B200_NORM_MAX;
  CeedCallB200(CeedVectorReturnCeed(vec), b200_vec_norm(ctx, B200_F64, n, d, t, norm));
  return CEED_ERROR_SUCCESS;
}

static int CeedVectorScale_B200(CeedVector vec, CeedScalar alpha) {
  CeedVector_B200  *impl;
  b200_ctx          ctx;
  CeedSize          n;
  const CeedScalar *d;

  CeedCallBackend(VecData(vec, &impl, &ctx, &n));
  CeedCallBackend(CeedVectorGetDevice_B200(vec, true, &d));
  CeedCallB200(CeedVectorReturnCeed(vec), b200_vec_scale(ctx, B200_F64, n, (void *)d, alpha));
  return CEED_ERROR_SUCCESS;
}

static int CeedVectorAXPY_B200(CeedVector y, CeedScalar alpha, CeedVector x) {
  CeedVector_B200  *impl;
  b200_ctx          ctx;
  CeedSize          n;
  const CeedScalar *dx, *dy;

  CeedCallBackend(VecData(y, &impl, &ctx, &n));
  CeedCallBackend(CeedVectorGetDevice_B200(x, false, &dx));
  CeedCallBackend(CeedVectorGetDevice_B200(y, true, &dy));
  CeedCallB200(CeedVectorReturnCeed(y), b200_vec_axpy(ctx, B200_F64, n, alpha, dx, (void *)dy));
  return CEED_ERROR_SUCCESS;
}

static int CeedVectorAXPBY_B200(CeedVector y, CeedScalar alpha, CeedScalar beta, CeedVector x) {
  CeedVector_B200  *impl;
  b200_ctx          ctx;
  CeedSize          n;
  const CeedScalar *dx, *dy;

  CeedCallBackend(VecData(y, &impl, &ctx, &n));
  CeedCallBackend(CeedVectorGetDevice_B200(x, false, &dx));
  CeedCallBackend(CeedVectorGetDevice_B200(y, true, &dy));
  CeedCallB200(CeedVectorReturnCeed(y), b200_vec_axpby(ctx, B200_F64, n, alpha, beta, dx, (void *)dy));
  return CEED_ERROR_SUCCESS;
}

static int CeedVectorPointwiseMult_B200(CeedVector w, CeedVector x, CeedVector y) {
  CeedVector_B200  *impl;
  b200_ctx          ctx;
  CeedSize          n;
  const CeedScalar *dx, *dy, *dw;

  CeedCallBackend(VecData(w, &impl, &ctx, &n));
  CeedCallBackend(CeedVectorGetDevice_B200(x, false, &dx));
  CeedCallBackend(CeedVectorGetDevice_B200(y, false, &dy));
  CeedCallBackend(CeedVectorGetDevice_B200(w, true, &dw));
  CeedCallB200(CeedVectorReturnCeed(w), b200_vec_pointwise_mult(ctx, B200_F64, n, (void *)dw, dx, dy));
  return CEED_ERROR_SUCCESS;
}

static int CeedVectorReciprocal_B200(CeedVector vec) {
  CeedVector_B200  *impl;
  b200_ctx          ctx;
  CeedSize          n;
  const CeedScalar *d;

  CeedCallBackend(VecData(vec, &impl, &ctx, &n));
  CeedCallBackend(CeedVectorGetDevice_B200(vec, true, &d));
  CeedCallB200(CeedVectorReturnCeed(vec), b200_vec_reciprocal(ctx, B200_F64, n, (void *)d));
  return CEED_ERROR_SUCCESS;
}

static int CeedVectorDestroy_B200(CeedVector vec) {
  CeedVector_B200 *impl;
  b200_ctx         ctx;

  CeedCallBackend(VecData(vec, &impl, &ctx, NULL));
  if (impl->d_owned) b200_free(ctx, impl->d_owned);
  CeedCallBackend(CeedFree(&impl->h_owned));
  CeedCallBackend(CeedFree(&impl));
  return CEED_ERROR_SUCCESS;
}

int CeedVectorCreate_B200(CeedSize n, CeedVector vec) {
  CeedVector_B200 *impl;
  Ceed             ceed;

  CeedCallBackend(CeedVectorGetCeed(vec, &ceed));
  CeedCallBackend(CeedCalloc(1, &impl));
  CeedCallBackend(CeedVectorSetData(vec, impl));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Vector", vec, "HasValidArray", CeedVectorHasValidArray_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Vector", vec, "HasBorrowedArrayOfType", CeedVectorHasBorrowedArrayOfType_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Vector", vec, "SetArray", CeedVectorSetArray_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Vector", vec, "TakeArray", CeedVectorTakeArray_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Vector", vec, "SyncArray", CeedVectorSyncArray_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Vector", vec, "GetArray", CeedVectorGetArray_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Vector", vec, "GetArrayRead", CeedVectorGetArrayRead_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Vector", vec, "GetArrayWrite", CeedVectorGetArrayWrite_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Vector", vec, "RestoreArray", CeedVectorRestoreArray_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Vector", vec, "RestoreArrayRead", CeedVectorRestoreArrayRead_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Vector", vec, "SetValue", CeedVectorSetValue_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Vector", vec, "SetValueStrided", CeedVectorSetValueStrided_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Vector", vec, "CopyStrided", CeedVectorCopyStrided_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Vector", vec, "Norm", CeedVectorNorm_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Vector", vec, "Scale", CeedVectorScale_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Vector", vec, "AXPY", CeedVectorAXPY_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Vector", vec, "AXPBY", CeedVectorAXPBY_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Vector", vec, "PointwiseMult", CeedVectorPointwiseMult_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Vector", vec, "Reciprocal", CeedVectorReciprocal_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "Vector", vec, "Destroy", CeedVectorDestroy_B200));
  CeedCallBackend(CeedDestroy(&ceed));
  (void)n;
  return CEED_ERROR_SUCCESS;
}
