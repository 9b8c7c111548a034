// libCEED backend `/gpu/cuda/b200`: private data of each object.  Host code in C; all device work goes through
// the C ABI of libceed_b200 (include/ceed-b200.h).
#pragma once

#include <ceed.h>
#include <ceed/backend.h>
#include <stdbool.h>

#include "ceed-b200.h"  // the C ABI (include/ceed-b200.h)

#define CeedCallB200(ceed, call)                                                                          \
  do {                                                                                                   \
    int b200_status_ = (call);                                                                           \
    if (b200_status_) return CeedError((ceed), CEED_ERROR_BACKEND, "%s: %s", #call, b200_last_error()); \
  } while (0)

typedef struct {
  b200_ctx ctx;
  int      device_id;
  bool     float_float;  // resource option ":arithmetic=float-float"
} Ceed_B200;

// Host and device mirrors of a CeedVector (the copy-mode rules of backends/cuda/ceed-cuda-common.c:53-80).
typedef struct {
  CeedScalar *h_array, *h_owned, *h_borrowed;
  CeedScalar *d_array, *d_owned, *d_borrowed;
  bool        h_valid, d_valid;
} CeedVector_B200;

typedef struct {
  int32_t  *d_offsets;  // device, [elem][node]
  CeedInt  *h_offsets;  // host copy (GetOffsets)
  b200_plan plan;       // deterministic transpose, created on first use
  bool      strided;
  int64_t   strides[3];
} CeedElemRestriction_B200;

typedef struct {
  b200_basis basis;
} CeedBasis_B200;

#define CEED_B200_QF_JIT (-3)  // user QFunction from a source file, compiled at run time with NVRTC

typedef struct {
  int qf_kind;  // B200_QF_*, -1 for the geometric-factor builds, CEED_B200_QF_JIT, -2 unsupported
  int build_poisson;
} CeedQFunction_B200;

typedef struct {
  b200_op     op;
  int         kind;  // 0 not analysed, 1 fused apply, 2 geometric-factor build, 3 run-time compiled QFunction, -1 unsupported
  CeedVector  qdata, kappa;
  CeedElemRestriction rstr_u, rstr_x;  // rstr_u: active restriction of the fused apply (diagonal assembly)
  CeedBasis   basis_x;
  // kind 3: passive inputs in QFunction order (without the active one) and the device copy of the context
  CeedInt     num_passive;
  CeedVector  passive[8];
  void       *d_ctx;
  size_t      ctx_size;
  int         qf_kind;  // kind 1: B200_QF_* of the fused apply
  b200_op_desc desc;    // kind 1: the fused operator's descriptor (diagonal assembly)
} CeedOperator_B200;

CEED_INTERN int CeedVectorCreate_B200(CeedSize n, CeedVector vec);
CEED_INTERN int CeedElemRestrictionCreate_B200(CeedMemType mem_type, CeedCopyMode copy_mode, const CeedInt *offsets, const bool *orients,
                                               const CeedInt8 *curl_orients, CeedElemRestriction rstr);
CEED_INTERN int CeedBasisCreateTensorH1_B200(CeedInt dim, CeedInt P_1d, CeedInt Q_1d, const CeedScalar *interp_1d, const CeedScalar *grad_1d,
                                             const CeedScalar *q_ref_1d, const CeedScalar *q_weight_1d, CeedBasis basis);
CEED_INTERN int CeedQFunctionCreate_B200(CeedQFunction qf);
CEED_INTERN int CeedQFunctionContextCreate_B200(CeedQFunctionContext ctx);
CEED_INTERN int CeedOperatorCreate_B200(CeedOperator op);
CEED_INTERN int CeedVectorGetDevice_B200(CeedVector vec, bool write, const CeedScalar **d_array);
CEED_INTERN int CeedGetB200Context(Ceed ceed, b200_ctx *ctx);
