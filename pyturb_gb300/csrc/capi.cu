// Status reporting and library-wide counters of the C-ABI.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

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

// ---------------------------------------------------------------- profiling
struct ProfRec {
  const char* name;
  cudaEvent_t a, b;
};
static std::mutex g_prof_mu;
static bool g_prof_on = false;
static std::vector<ProfRec> g_prof;
static std::vector<cudaEvent_t> g_pool;

static cudaEvent_t pool_get() {
  if (!g_pool.empty()) {
    cudaEvent_t e = g_pool.back();
    g_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

ProfScope::ProfScope(const char* name, cudaStream_t s) : name_(name), s_(s), a_(nullptr), on_(false) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  if (!g_prof_on) return;
  on_ = true;
  a_ = pool_get();
  cudaEventRecord(a_, s_);
}

ProfScope::~ProfScope() {
  if (!on_) return;
  std::lock_guard<std::mutex> lk(g_prof_mu);
  cudaEvent_t b = pool_get();
  cudaEventRecord(b, s_);
  g_prof.push_back(ProfRec{name_, a_, b});
}

}  // namespace pt

extern "C" int pt_version(void) { return 100; }

extern "C" const char* pt_last_error(void) { return pt::g_last_error.c_str(); }

extern "C" int pt_prof_enable(int on) {
  std::lock_guard<std::mutex> lk(pt::g_prof_mu);
  pt::g_prof_on = on != 0;
  return PT_OK;
}

extern "C" int pt_prof_report(char* buf, size_t len) {
  if (!buf || len == 0) return pt::fail(PT_ERR_ARG, "pt_prof_report: empty buffer");
  if (int rc = pt::check_cuda(cudaDeviceSynchronize(), "pt_prof_report: sync")) return rc;
  std::lock_guard<std::mutex> lk(pt::g_prof_mu);
  std::map<std::string, std::pair<long, double>> agg;
  for (auto& r : pt::g_prof) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, r.a, r.b);
    auto& e = agg[r.name];
    e.first += 1;
    e.second += ms;
    pt::g_pool.push_back(r.a);
    pt::g_pool.push_back(r.b);
  }
  pt::g_prof.clear();
  std::string out;
  char line[256];
  for (auto& kv : agg) {
    std::snprintf(line, sizeof line, "%s %ld %.6f\n", kv.first.c_str(), kv.second.first,
                  kv.second.second);
    out += line;
  }
  if (out.size() + 1 > len) return pt::fail(PT_ERR_ARG, "pt_prof_report: buffer too small");
  std::memcpy(buf, out.c_str(), out.size() + 1);
  return PT_OK;
}

extern "C" uint64_t pt_launch_count(void) {
  return __atomic_load_n(pt::launch_counter(), __ATOMIC_RELAXED);
}
