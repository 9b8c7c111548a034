// Compiled instances of the fused operator kernel: double, B200_QF_POISSON, P_1d = 2..9, register and shared-memory qdata staging.
#include "b200_op_launch.cuh"

B200_OP_TABLE(double, B200_QF_POISSON, op_table_f64_poisson)
