// Compiled instances of the fused operator kernel: float, B200_QF_VECPOISSON, P_1d = 2..9, register and shared-memory qdata staging.
#include "b200_op_launch.cuh"

B200_OP_TABLE(float, B200_QF_VECPOISSON, op_table_f32_vecpoisson)
