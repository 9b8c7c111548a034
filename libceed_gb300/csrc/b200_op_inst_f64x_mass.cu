// Compiled instances of the fused operator kernel in float-float arithmetic (B200_F64X): B200_QF_MASS, P_1d = 2..9,
// even-odd contractions with register, shared-memory or bulk-copy qdata staging.  Vectors and qdata stay double in HBM.
#include "b200_op_launch.cuh"

B200_OP_TABLE(dfloat, B200_QF_MASS, op_table_f64x_mass)
