// Status reporting and library-wide counters of the C-ABI.
#include <cuda_runtime.h>

#include <string>

#include "common.cuh"

namespace pt {

static thread_local std::string g_last_error;
static uint64_t g_launches = 0;

uint64_t* launch_counter() { return &g_launches; }

void set_error(const std::string& msg) { g_last_error = msg; }

int fail(int code, const std::string& msg) {
  set_error(msg);
  return code;
}

int check_cuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return PT_OK;
  return fail(PT_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

int check_launch(const char* what) { return check_cuda(cudaGetLastError(), what); }

}  // namespace pt

extern "C" int pt_version(void) { return 100; }

extern "C" const char* pt_last_error(void) { return pt::g_last_error.c_str(); }

extern "C" uint64_t pt_launch_count(void) {
  return __atomic_load_n(pt::launch_counter(), __ATOMIC_RELAXED);
}
