// Run-time compilation of fused operator kernels for user QFunctions (NVRTC, -arch=sm_103a).
//
// The reference JIT-compiles every CUDA kernel with NVRTC for the device's sm_XY and includes the QFunction source
// into its generated operator kernel (backends/cuda/ceed-cuda-compile.cpp:70-240,
// backends/cuda-gen/ceed-cuda-gen-operator-build.cpp:1343-1361).  Here the gallery kernels of the path are compiled
// ahead of time; a QFunction given as source ("file.h:Name") is compiled here into the fixed kernel template of
// b200_jit_kernel.cuh, for the architecture-specific target sm_103a, and loaded with cudaLibraryLoadData.  NVRTC is
// loaded with dlopen on first use, so the library itself has no link-time dependency on it.
#include <dlfcn.h>
#include <nvrtc.h>

#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "b200_internal.cuh"
#include "b200_jit.cuh"
#include "b200_op_launch.cuh"

namespace b200 {

namespace {

struct Nvrtc {
  void *handle = nullptr;
  nvrtcResult (*create)(nvrtcProgram *, const char *, const char *, int, const char *const *, const char *const *);
  nvrtcResult (*compile)(nvrtcProgram, int, const char *const *);
  nvrtcResult (*log_size)(nvrtcProgram, size_t *);
  nvrtcResult (*log)(nvrtcProgram, char *);
  nvrtcResult (*cubin_size)(nvrtcProgram, size_t *);
  nvrtcResult (*cubin)(nvrtcProgram, char *);
  nvrtcResult (*add_name)(nvrtcProgram, const char *);
  nvrtcResult (*lowered)(nvrtcProgram, const char *, const char **);
  nvrtcResult (*destroy)(nvrtcProgram *);
  const char *(*error_string)(nvrtcResult);
};

std::mutex g_jit_mutex;
Nvrtc      g_nvrtc;
std::map<std::string, cudaKernel_t> g_kernel_cache;
std::vector<cudaLibrary_t>          g_libraries;

int load_nvrtc() {
  if (g_nvrtc.handle) return B200_SUCCESS;
  const char *names[] = {"libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13", "/usr/local/cuda/lib64/libnvrtc.so"};
  void       *h       = nullptr;
  for (const char *n : names)
    if ((h = dlopen(n, RTLD_NOW | RTLD_LOCAL))) break;
  B200_CHECK(h, B200_ERROR_BACKEND, "NVRTC (libnvrtc.so.13) could not be loaded: %s", dlerror());
#define B200_SYM(field, sym)                                                                           \
  g_nvrtc.field = reinterpret_cast<decltype(g_nvrtc.field)>(dlsym(h, sym));                           \
  B200_CHECK(g_nvrtc.field, B200_ERROR_BACKEND, "NVRTC symbol %s missing", sym);
  B200_SYM(create, "nvrtcCreateProgram");
  B200_SYM(compile, "nvrtcCompileProgram");
  B200_SYM(log_size, "nvrtcGetProgramLogSize");
  B200_SYM(log, "nvrtcGetProgramLog");
  B200_SYM(cubin_size, "nvrtcGetCUBINSize");
  B200_SYM(cubin, "nvrtcGetCUBIN");
  B200_SYM(add_name, "nvrtcAddNameExpression");
  B200_SYM(lowered, "nvrtcGetLoweredName");
  B200_SYM(destroy, "nvrtcDestroyProgram");
  B200_SYM(error_string, "nvrtcGetErrorString");
#undef B200_SYM
  g_nvrtc.handle = h;
  return B200_SUCCESS;
}

// Directory holding this shared library (…/libceed_gb300/lib); kernel sources are found relative to it.
std::string library_dir() {
  Dl_info info;
  if (dladdr((void *)&load_nvrtc, &info) && info.dli_fname) {
    std::string p(info.dli_fname);
    const auto  s = p.rfind('/');
    return s == std::string::npos ? "." : p.substr(0, s);
  }
  return ".";
}

bool read_file(const std::string &path, std::string *out) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  std::stringstream ss;
  ss << f.rdbuf();
  *out = ss.str();
  return true;
}

// The subset of libCEED's QFunction header that a QFunction source needs inside the fused kernel.
const char *kCeedTypesShim = R"(#pragma once
#ifndef B200_JIT_CEED_TYPES
#define B200_JIT_CEED_TYPES
typedef int CeedInt;
typedef long long CeedSize;
typedef signed char CeedInt8;
typedef B200_JIT_SCALAR CeedScalar;
#define CEED_QFUNCTION(name) static __device__ __forceinline__ int name
#define CEED_QFUNCTION_HELPER static __device__ __forceinline__
#define CEED_QFUNCTION_ATTR
#define CEED_Q_VLA 1
#define CeedPragmaSIMD
#define CEED_ERROR_SUCCESS 0
#define CEED_EPSILON 1e-16
#endif
)";

}  // namespace

int jit_compile(const JitRequest &r, cudaKernel_t *kernel, std::string *key_out, bool load) {
  std::lock_guard<std::mutex> lock(g_jit_mutex);
  int                         st = load_nvrtc();
  if (st) return st;
  std::string user_src;
  B200_CHECK(read_file(r.source_path, &user_src), B200_ERROR_BACKEND, "cannot read QFunction source %s", r.source_path.c_str());
  const char *scalar = r.prec == B200_F64 ? "double" : "float";
  std::ostringstream key;
  key << r.source_path << ':' << r.qf_name << '|' << scalar << '|' << r.P << '|' << r.eval_in << r.eval_out << r.eo << '|' << r.active_input;
  for (int i = 0; i < r.num_inputs; i++) key << ',' << r.input_size[i];
  key << '|' << std::hash<std::string>()(user_src);
  if (key_out) *key_out = key.str();
  auto hit = g_kernel_cache.find(key.str());
  if (load && hit != g_kernel_cache.end()) {
    *kernel = hit->second;
    return B200_SUCCESS;
  }

  // Kernel template sources, shipped in-tree next to the compiled library.
  const std::string dir = library_dir();
  std::string       hdr_abi, hdr_kernels, hdr_point, hdr_jit, hdr_df;
  B200_CHECK(read_file(dir + "/../../include/ceed-b200.h", &hdr_abi) && read_file(dir + "/../csrc/b200_op_kernels.cuh", &hdr_kernels) &&
                 read_file(dir + "/../csrc/b200_pointwise.cuh", &hdr_point) && read_file(dir + "/../csrc/b200_jit_kernel.cuh", &hdr_jit) &&
                 read_file(dir + "/../csrc/b200_dfloat.cuh", &hdr_df),
             B200_ERROR_BACKEND, "kernel template sources not found next to %s", dir.c_str());

  // Glue: gather the passive inputs at one point and call the user's QFunction with Q = 1.
  const int          Q3 = (r.P + 1) * (r.P + 1) * (r.P + 1);
  std::ostringstream src;
  src << "typedef long long int64_t;\ntypedef int int32_t;\ntypedef unsigned long long uint64_t;\ntypedef unsigned int uint32_t;\n"
      << "typedef decltype(sizeof(0)) size_t;\n#define B200_JIT_SCALAR " << scalar << "\n#include \"ceed-b200.h\"\n#include \"ceed/types.h\"\n"
      << "#include \"b200_jit_kernel.cuh\"\n#include \"b200_user_qfunction.h\"\nnamespace b200 {\n"
      << "__device__ __forceinline__ void b200_jit_point(const JitFields<CeedScalar> &F, int64_t ne, int64_t e, int q, const CeedScalar *act_in, "
         "CeedScalar *act_out) {\n";
  int passive = 0;
  for (int i = 0; i < r.num_inputs; i++) {
    if (i == r.active_input) continue;
    src << "  CeedScalar p" << i << "[" << r.input_size[i] << "];\n  for (int k = 0; k < " << r.input_size[i] << "; k++) p" << i << "[k] = F.passive["
        << passive << "][((int64_t)k * ne + e) * " << Q3 << " + q];\n";
    passive++;
  }
  src << "  const CeedScalar *in[" << r.num_inputs << "] = {";
  for (int i = 0; i < r.num_inputs; i++) src << (i ? ", " : "") << (i == r.active_input ? std::string("act_in") : "p" + std::to_string(i));
  src << "};\n  CeedScalar *out[1] = {act_out};\n  ::" << r.qf_name << "(F.ctx, 1, in, out);\n}\n}  // namespace b200\n";
  std::ostringstream name;
  name << "b200::k_op_jit<" << scalar << ", " << r.P << ", " << r.P + 1 << ", " << r.eval_in << ", " << r.eval_out << ", "
       << (r.eo ? "true" : "false") << ">";
  // The user's source is a header of the program; includes beside it resolve through -I.
  const char *headers[]   = {hdr_abi.c_str(), hdr_kernels.c_str(), hdr_point.c_str(), hdr_jit.c_str(), hdr_df.c_str(),
                             kCeedTypesShim,  kCeedTypesShim,      "",                user_src.c_str()};
  const char *hdr_names[] = {"ceed-b200.h",  "b200_op_kernels.cuh", "b200_pointwise.cuh", "b200_jit_kernel.cuh", "b200_dfloat.cuh",
                             "ceed/types.h", "ceed.h",              "math.h",             "b200_user_qfunction.h"};
  std::string              src_dir = r.source_path.substr(0, r.source_path.rfind('/') == std::string::npos ? 0 : r.source_path.rfind('/'));
  std::vector<std::string> opts    = {"-arch=sm_103a", "-std=c++17", "-default-device", "-DB200_JIT=1"};
  if (!src_dir.empty()) opts.push_back("-I" + src_dir);
  for (const auto &d : r.include_dirs) opts.push_back("-I" + d);
  std::vector<const char *> copts;
  for (const auto &o : opts) copts.push_back(o.c_str());

  nvrtcProgram prog;
  nvrtcResult  nr = g_nvrtc.create(&prog, src.str().c_str(), "b200_jit_operator.cu", 9, headers, hdr_names);
  B200_CHECK(nr == NVRTC_SUCCESS, B200_ERROR_BACKEND, "nvrtcCreateProgram: %s", g_nvrtc.error_string(nr));
  g_nvrtc.add_name(prog, name.str().c_str());
  nr = g_nvrtc.compile(prog, (int)copts.size(), copts.data());
  if (nr != NVRTC_SUCCESS) {
    size_t n = 0;
    g_nvrtc.log_size(prog, &n);
    std::string log(n, '\0');
    g_nvrtc.log(prog, &log[0]);
    g_nvrtc.destroy(&prog);
    set_error("NVRTC could not compile QFunction %s from %s:\n%s", r.qf_name.c_str(), r.source_path.c_str(), log.c_str());
    return B200_ERROR_BACKEND;
  }
  const char *lowered = nullptr;
  g_nvrtc.lowered(prog, name.str().c_str(), &lowered);
  std::string lowered_name = lowered ? lowered : "";
  size_t      cubin_size   = 0;
  g_nvrtc.cubin_size(prog, &cubin_size);
  std::vector<char> cubin(cubin_size);
  g_nvrtc.cubin(prog, cubin.data());
  g_nvrtc.destroy(&prog);
  B200_CHECK(!lowered_name.empty() && cubin_size > 0, B200_ERROR_BACKEND, "NVRTC produced no kernel for %s", name.str().c_str());
  if (!load) return B200_SUCCESS;
  cudaLibrary_t lib;
  B200_CUDA(cudaLibraryLoadData(&lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0));
  B200_CUDA(cudaLibraryGetKernel(kernel, lib, lowered_name.c_str()));
  g_libraries.push_back(lib);
  g_kernel_cache[key.str()] = *kernel;
  return B200_SUCCESS;
}

// OpMats<T, P, P+1> bytes for the kernel's parameter space.
int jit_mats_blob(int prec, int P, const double *B, const double *G, std::vector<char> *blob) {
  auto put = [&](const auto &m) {
    blob->resize(sizeof(m));
    memcpy(blob->data(), &m, sizeof(m));
  };
#define B200_MATS_CASE(PP)                                                                          \
  case PP:                                                                                          \
    if (prec == B200_F64) put(make_mats<double, PP, PP + 1>(B, G));                                 \
    else put(make_mats<float, PP, PP + 1>(B, G));                                                   \
    return B200_SUCCESS;
  switch (P) {
    B200_MATS_CASE(2)
    B200_MATS_CASE(3)
    B200_MATS_CASE(4)
    B200_MATS_CASE(5)
    B200_MATS_CASE(6)
    B200_MATS_CASE(7)
    B200_MATS_CASE(8)
    B200_MATS_CASE(9)
  }
#undef B200_MATS_CASE
  set_error("JIT kernels cover P_1d in 2..9 (got %d)", P);
  return B200_ERROR_UNSUPPORTED;
}

}  // namespace b200

using namespace b200;

extern "C" int b200_jit_compile_check(const b200_jit_qfunction *qf, int prec, int P_1d) {
  B200_CHECK(qf && qf->source_path && qf->name, B200_ERROR_INCOMPLETE, "b200_jit_compile_check: missing descriptor");
  B200_CHECK(prec == B200_F64 || prec == B200_F32, B200_ERROR_UNSUPPORTED, "unknown precision %d", prec);
  B200_CHECK(P_1d >= 2 && P_1d <= 9, B200_ERROR_UNSUPPORTED, "JIT kernels cover P_1d in 2..9 (got %d)", P_1d);
  JitRequest r;
  r.source_path  = qf->source_path;
  r.qf_name      = qf->name;
  r.prec         = prec;
  r.P            = P_1d;
  r.eval_in      = qf->eval_in;
  r.eval_out     = qf->eval_out;
  r.eo           = true;
  r.num_inputs   = qf->num_inputs;
  r.active_input = qf->active_input;
  for (int i = 0; i < 8; i++) r.input_size[i] = i < qf->num_inputs ? qf->input_size[i] : 0;
  cudaKernel_t unused;
  return jit_compile(r, &unused, nullptr, false);
}
