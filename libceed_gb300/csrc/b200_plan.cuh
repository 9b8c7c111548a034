// Deterministic scatter through an inverse-offset plan (used by the restriction and the fused operator).
#pragma once

#include "b200_internal.cuh"

namespace b200 {
// l (+)= E^T e with e in the layout [comp][elem][node]; fixed summation order per node.
int plan_scatter(b200_plan plan, int prec, const void *e_vec, void *l_vec, int add);
}  // namespace b200
