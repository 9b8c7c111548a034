// Compiled instances of the fused operator kernel: float, B200_QF_POISSON_KAPPA, P_1d = 2..9, register and shared-memory qdata staging.
#include "b200_op_launch.cuh"

B200_OP_TABLE(float, B200_QF_POISSON_KAPPA, op_table_f32_kappa)

namespace b200 {
// Kappa-gradient instances, P_1d = 2..9.
bool kgrad_table_f32(int P, OpLauncher *out) {
  switch (P) {
    case 2: *out = kgrad_launch<float, 2>; return true;
    case 3: *out = kgrad_launch<float, 3>; return true;
    case 4: *out = kgrad_launch<float, 4>; return true;
    case 5: *out = kgrad_launch<float, 5>; return true;
    case 6: *out = kgrad_launch<float, 6>; return true;
    case 7: *out = kgrad_launch<float, 7>; return true;
    case 8: *out = kgrad_launch<float, 8>; return true;
    case 9: *out = kgrad_launch<float, 9>; return true;
    default: return false;
  }
}
}  // namespace b200
