// CeedElemRestriction for `/gpu/cuda/b200`: offset (standard) and strided restrictions on the device.  E-vector layout
// [comp][elem][node], published through CeedElemRestrictionSetELayout as backends/cuda-ref/ceed-cuda-ref-restriction.c
// does; transposes use the atomic scatter, or the inverse-offset plan when the Ceed is deterministic.
#include <stdlib.h>
#include <string.h>

#include "ceed-b200-backend.h"

static int RstrCtx(CeedElemRestriction rstr, CeedElemRestriction_B200 **impl, b200_ctx *ctx) {
  Ceed ceed;

  CeedCallBackend(CeedElemRestrictionGetData(rstr, impl));
  CeedCallBackend(CeedElemRestrictionGetCeed(rstr, &ceed));
  CeedCallBackend(CeedGetB200Context(ceed, ctx));
  CeedCallBackend(CeedDestroy(&ceed));
  return CEED_ERROR_SUCCESS;
}

static int CeedElemRestrictionApply_B200(CeedElemRestriction rstr, CeedTransposeMode t_mode, CeedVector u, CeedVector v, CeedRequest *request) {
  CeedElemRestriction_B200 *impl;
  b200_ctx                  ctx;
  CeedInt                   num_elem, elem_size, num_comp, comp_stride = 1;
  CeedSize                  l_size;
  const CeedScalar         *du, *dv;
  Ceed                      ceed = CeedElemRestrictionReturnCeed(rstr);
  bool                      is_det;

  CeedCallBackend(RstrCtx(rstr, &impl, &ctx));
  CeedCallBackend(CeedElemRestrictionGetNumElements(rstr, &num_elem));
  CeedCallBackend(CeedElemRestrictionGetElementSize(rstr, &elem_size));
  CeedCallBackend(CeedElemRestrictionGetNumComponents(rstr, &num_comp));
  CeedCallBackend(CeedElemRestrictionGetLVectorSize(rstr, &l_size));
  if (!impl->strided) CeedCallBackend(CeedElemRestrictionGetCompStride(rstr, &comp_stride));
  CeedCallBackend(CeedVectorGetDevice_B200(u, false, &du));
  CeedCallBackend(CeedVectorGetDevice_B200(v, true, &dv));
  if (impl->strided) {
    if (t_mode == CEED_NOTRANSPOSE) CeedCallB200(ceed, b200_rstr_strided_gather(ctx, B200_F64, num_elem, elem_size, num_comp, impl->strides, du, (void *)dv));
    else CeedCallB200(ceed, b200_rstr_strided_scatter(ctx, B200_F64, num_elem, elem_size, num_comp, impl->strides, du, (void *)dv));
  } else if (t_mode == CEED_NOTRANSPOSE) {
    CeedCallB200(ceed, b200_rstr_gather(ctx, B200_F64, num_elem, elem_size, num_comp, comp_stride, l_size, impl->d_offsets, du, (void *)dv));
  } else {
    CeedCallBackend(CeedIsDeterministic(ceed, &is_det));
    if (is_det) {
      if (!impl->plan)
        CeedCallB200(ceed, b200_plan_create(ctx, num_elem, elem_size, num_comp, comp_stride, l_size, impl->h_offsets, impl->d_offsets, &impl->plan));
      CeedCallB200(ceed, b200_rstr_scatter_det(ctx, impl->plan, B200_F64, du, (void *)dv, 1));
    } else {
      CeedCallB200(ceed, b200_rstr_scatter_atomic(ctx, B200_F64, num_elem, elem_size, num_comp, comp_stride, l_size, impl->d_offsets, du, (void *)dv));
    }
  }
  if (request != CEED_REQUEST_IMMEDIATE && request != CEED_REQUEST_ORDERED) *request = NULL;
  return CEED_ERROR_SUCCESS;
}

static int CeedElemRestrictionGetOffsets_B200(CeedElemRestriction rstr, CeedMemType mem_type, const CeedInt **offsets) {
  CeedElemRestriction_B200 *impl;

  CeedCallBackend(CeedElemRestrictionGetData(rstr, &impl));
  *offsets = mem_type == CEED_MEM_HOST ? impl->h_offsets : (const CeedInt *)impl->d_offsets;
  return CEED_ERROR_SUCCESS;
}

static int CeedElemRestrictionDestroy_B200(CeedElemRestriction rstr) {
  CeedElemRestriction_B200 *impl;
  b200_ctx                  ctx;

  CeedCallBackend(RstrCtx(rstr, &impl, &ctx));
  if (impl->plan) b200_plan_destroy(impl->plan);
  if (impl->d_offsets) b200_free(ctx, impl->d_offsets);
  CeedCallBackend(CeedFree(&impl->h_offsets));
  CeedCallBackend(CeedFree(&impl));
  return CEED_ERROR_SUCCESS;
}

int CeedElemRestrictionCreate_B200(CeedMemType mem_type, CeedCopyMode copy_mode, const CeedInt *offsets, const bool *orients,
                                   const CeedInt8 *curl_orients, CeedElemRestriction rstr) {
  Ceed                      ceed;
  CeedElemRestriction_B200 *impl;
  CeedRestrictionType       type;
  CeedInt                   num_elem, elem_size, num_comp;
  CeedSize                  l_size;
  b200_ctx                  ctx;

  CeedCallBackend(CeedElemRestrictionGetCeed(rstr, &ceed));
  CeedCallBackend(CeedGetB200Context(ceed, &ctx));
  CeedCallBackend(CeedElemRestrictionGetType(rstr, &type));
  CeedCheck(type == CEED_RESTRICTION_STANDARD || type == CEED_RESTRICTION_STRIDED, ceed, CEED_ERROR_UNSUPPORTED,
            "/gpu/cuda/b200 supports offset and strided restrictions only");
  CeedCallBackend(CeedElemRestrictionGetNumElements(rstr, &num_elem));
  CeedCallBackend(CeedElemRestrictionGetElementSize(rstr, &elem_size));
  CeedCallBackend(CeedElemRestrictionGetNumComponents(rstr, &num_comp));
  CeedCallBackend(CeedElemRestrictionGetLVectorSize(rstr, &l_size));
  CeedCallBackend(CeedCalloc(1, &impl));
  {
    CeedInt layout[3] = {1, num_elem * elem_size, elem_size};  // [comp][elem][node]
    CeedCallBackend(CeedElemRestrictionSetELayout(rstr, layout));
  }
  if (type == CEED_RESTRICTION_STRIDED) {
    bool    backend_strides;
    CeedInt s[3];

    impl->strided = true;
    CeedCallBackend(CeedElemRestrictionHasBackendStrides(rstr, &backend_strides));
    if (backend_strides) {
      impl->strides[0] = 1, impl->strides[1] = (int64_t)num_elem * elem_size, impl->strides[2] = elem_size;
    } else {
      CeedCallBackend(CeedElemRestrictionGetStrides(rstr, s));
      impl->strides[0] = s[0], impl->strides[1] = s[1], impl->strides[2] = s[2];
    }
  } else {
    const size_t n = (size_t)num_elem * elem_size;

    CeedCallBackend(CeedMalloc(n ? n : 1, &impl->h_offsets));
    if (mem_type == CEED_MEM_HOST) {
      memcpy(impl->h_offsets, offsets, sizeof(CeedInt) * n);
    } else {
      CeedCallB200(ceed, b200_copy(ctx, impl->h_offsets, offsets, sizeof(CeedInt) * n, B200_COPY_D2H));
      CeedCallB200(ceed, b200_ctx_sync(ctx));
    }
    for (size_t i = 0; i < n; i++)
      CeedCheck(impl->h_offsets[i] >= 0 && impl->h_offsets[i] < l_size, ceed, CEED_ERROR_DIMENSION, "offset %zu (%d) outside the L-vector", i,
                impl->h_offsets[i]);
    CeedCallB200(ceed, b200_alloc(ctx, sizeof(int32_t) * (n ? n : 1), (void **)&impl->d_offsets));
    CeedCallB200(ceed, b200_copy(ctx, impl->d_offsets, impl->h_offsets, sizeof(int32_t) * n, B200_COPY_H2D));
    if (copy_mode == CEED_OWN_POINTER && mem_type == CEED_MEM_HOST) free((void *)offsets);
  }
  (void)orients;
  (void)curl_orients;
  (void)num_comp;
  CeedCallBackend(CeedElemRestrictionSetData(rstr, impl));
  CeedCallBackend(CeedSetBackendFunction(ceed, "ElemRestriction", rstr, "Apply", CeedElemRestrictionApply_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "ElemRestriction", rstr, "ApplyUnsigned", CeedElemRestrictionApply_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "ElemRestriction", rstr, "ApplyUnoriented", CeedElemRestrictionApply_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "ElemRestriction", rstr, "GetOffsets", CeedElemRestrictionGetOffsets_B200));
  CeedCallBackend(CeedSetBackendFunction(ceed, "ElemRestriction", rstr, "Destroy", CeedElemRestrictionDestroy_B200));
  CeedCallBackend(CeedDestroy(&ceed));
  return CEED_ERROR_SUCCESS;
}
