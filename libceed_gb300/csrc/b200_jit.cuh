// Run-time compilation of fused operator kernels for user QFunctions (internal interface).
#pragma once

#include <string>
#include <vector>

#include "b200_internal.cuh"

namespace b200 {

struct JitRequest {
  std::string              source_path, qf_name;
  int                      prec, P, eval_in, eval_out;
  bool                     eo;
  int                      num_inputs, active_input;
  int                      input_size[8];
  std::vector<std::string> include_dirs;
};

// Compile (or fetch from the cache) k_op_jit for the request; returns the loaded kernel.
int jit_compile(const JitRequest &r, cudaKernel_t *kernel, std::string *key, bool load = true);
// OpMats<T, P, P+1> of the interpolation and collocated-gradient matrices, as bytes for the kernel parameters.
int jit_mats_blob(int prec, int P, const double *B, const double *G, std::vector<char> *blob);

}  // namespace b200
