// Shared device helpers for the pyturb_gb300 kernels: complex arithmetic,
// status reporting, the Philox4x32-10 counter-based generator and the
// Box-Muller normal transform.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

#include "../../include/pyturb_gb300.h"

namespace pt {

// ---------------------------------------------------------------- status
// The last error message of the calling host thread (C-ABI contract: every
// entry point returns a status code and leaves a readable message here).
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int check_cuda(cudaError_t e, const char* what);
int check_launch(const char* what);

// ---------------------------------------------------------------- profiling
// Optional per-kernel timing with CUDA events recorded on the launching
// stream (pt_prof_enable / pt_prof_report). Off by default: a disabled scope
// costs one branch.
class ProfScope {
 public:
  ProfScope(const char* name, cudaStream_t s);
  ~ProfScope();

 private:
  const char* name_;
  cudaStream_t s_;
  cudaEvent_t a_;
  bool on_;
};

// ---------------------------------------------------------------- complex
__host__ __device__ __forceinline__ float2 cadd(float2 a, float2 b) {
  return make_float2(a.x + b.x, a.y + b.y);
}
__host__ __device__ __forceinline__ float2 csub(float2 a, float2 b) {
  return make_float2(a.x - b.x, a.y - b.y);
}
__host__ __device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// a * conj(b)
__host__ __device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.y, b.x, -a.x * b.y));
}
__host__ __device__ __forceinline__ float2 cscale(float2 a, float s) {
  return make_float2(a.x * s, a.y * s);
}
__host__ __device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
// acc += a * b
__host__ __device__ __forceinline__ float2 cfma(float2 a, float2 b, float2 acc) {
  acc.x = fmaf(a.x, b.x, fmaf(-a.y, b.y, acc.x));
  acc.y = fmaf(a.x, b.y, fmaf(a.y, b.x, acc.y));
  return acc;
}
// multiply by +i
__host__ __device__ __forceinline__ float2 cmul_i(float2 a) { return make_float2(-a.y, a.x); }

// ---------------------------------------------------------------- Philox
// Philox4x32 with 10 rounds (Salmon, Moraes, Dror & Shaw, SC'11,
// "Parallel random numbers: as easy as 1, 2, 3"): a bijection of a 128-bit
// counter under a 64-bit key, so every noise element is addressed directly
// by (key, counter) with no generator state.
struct u32x4 {
  uint32_t x, y, z, w;
};

__device__ __forceinline__ void philox_round(u32x4& c, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  uint32_t hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
  uint32_t hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
  u32x4 r;
  r.x = hi1 ^ c.y ^ k0;
  r.y = lo1;
  r.z = hi0 ^ c.w ^ k1;
  r.w = lo0;
  c = r;
}

__device__ __forceinline__ u32x4 philox4x32_10(u32x4 c, uint64_t key) {
  uint32_t k0 = (uint32_t)key, k1 = (uint32_t)(key >> 32);
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    philox_round(c, k0, k1);
    k0 += W0;
    k1 += W1;
  }
  philox_round(c, k0, k1);
  return c;
}

// Two independent N(0,1) draws from two 32-bit uniforms (Box-Muller).
// u1 is mapped to (0, 1] so the logarithm is finite. The radius and angle use
// the hardware approximations (log2, sqrt, sin/cos on [-pi, pi)): absolute
// errors near 1e-6, far below the statistical scatter of the draws, at a
// fraction of the instructions of the correctly rounded functions.
__device__ __forceinline__ float sqrt_approx(float x) {
  float r;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float2 box_muller(uint32_t a, uint32_t b) {
  const float u1 = ((float)(a >> 8) + 1.0f) * (1.0f / 16777216.0f);
  const float u2 = (float)(b >> 8) * (1.0f / 16777216.0f) - 0.5f;  // [-0.5, 0.5)
  // -2 ln u1 = -2 ln 2 log2 u1 >= 0
  const float r = sqrt_approx(-1.3862943611198906f * __log2f(u1));
  float s, c;
  __sincosf(6.283185307179586f * u2, &s, &c);
  // angle 2 pi u2 - pi: negate to keep the orientation of 2 pi (u2 + 0.5)
  return make_float2(-r * c, -r * s);
}

// Noise domains keep the streams of different consumers disjoint.
enum NoiseDomain : uint32_t {
  kDomainScreen = 0x11u,      // main FFT-grid noise of PhaseScreen.generate
  kDomainSub = 0x22u,         // subharmonic 3x3 noise
  kDomainLayer = 0x33u,       // frozen-flow layer spectra
  kDomainLayerSub = 0x44u,    // frozen-flow layer subharmonics
  kDomainExtrude = 0x55u,     // extrusion row noise
  kDomainBoil = 0x66u,        // boiling AR(1) innovations
  kDomainBoilSeed = 0x77u,    // seed rows of extrusion boiling's fresh windows
};

// Complex N(0,1)+iN(0,1) pair for element `idx` of stream (`key`, `call`, `domain`).
__device__ __forceinline__ float2 philox_cnormal(uint64_t key, uint64_t idx, uint64_t call,
                                                 uint32_t domain) {
  u32x4 c;
  c.x = (uint32_t)idx;
  c.y = (uint32_t)(idx >> 32);
  c.z = (uint32_t)call;
  c.w = ((uint32_t)(call >> 32) & 0x00FFFFFFu) | (domain << 24);
  u32x4 r = philox4x32_10(c, key);
  return box_muller(r.x, r.y);
}

// Both complex pairs of one Philox call: (x, y) -> lo, (z, w) -> hi. The screen
// noise of a row of length N uses counter (row * H + ky mod H), H = ceil(N/2),
// lo for ky < H and hi for ky >= H, so the elements ky and ky + H share a
// call (the register FFT path owns both in one thread).
__device__ __forceinline__ void philox_cnormal2(uint64_t key, uint64_t idx, uint64_t call,
                                                uint32_t domain, float2& lo, float2& hi) {
  u32x4 c;
  c.x = (uint32_t)idx;
  c.y = (uint32_t)(idx >> 32);
  c.z = (uint32_t)call;
  c.w = ((uint32_t)(call >> 32) & 0x00FFFFFFu) | (domain << 24);
  const u32x4 r = philox4x32_10(c, key);
  lo = box_muller(r.x, r.y);
  hi = box_muller(r.z, r.w);
}
__device__ __forceinline__ float2 screen_normal(uint64_t key, uint64_t row, int ky, int N,
                                                uint64_t call) {
  const int H = (N + 1) / 2;
  const bool upper = ky >= H;
  float2 lo, hi;
  philox_cnormal2(key, row * (uint64_t)H + (uint64_t)(upper ? ky - H : ky), call, kDomainScreen,
                  lo, hi);
  return upper ? hi : lo;
}

// ---------------------------------------------------------------- L2 policy
// An L2 evict-last policy (createpolicy) and read-only loads that carry it,
// for tables every CTA re-reads (filters, operators).
__device__ __forceinline__ uint64_t l2_evict_last() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ float ld_keep(const float* p, uint64_t pol) {
  float v;
  asm("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(pol));
  return v;
}

// ---------------------------------------------------------------- fixed point phase
// Shift-theorem phases are formed as k * u (mod 1) with u = frac(s * df)
// held as a 64-bit binary fraction, so the product wraps exactly and the
// phase error does not grow with the travel s.
__device__ __forceinline__ uint64_t phase_fixed(double u) {
  double f = u - floor(u);
  return (uint64_t)__double2ull_rz(f * 18446744073709551616.0);
}
__device__ __forceinline__ float2 phasor_from_fixed(uint64_t p) {
  // signed fraction of a turn in [-0.5, 0.5): the high word as a signed
  // integer times 2^-32 plus the low word times 2^-64, all in float (FP64
  // conversions run at a small fraction of the FP32 rate on this part). The
  // float result matches the correctly rounded value to about an ulp; the
  // absolute phase error stays below 2^-33 turn.
  const float hi = (float)(int32_t)(uint32_t)(p >> 32);
  const float lo = (float)(uint32_t)p;
  const float cyc = fmaf(lo, 5.421010862427522e-20f, hi * 2.3283064365386963e-10f);
  float s, c;
  sincospif(2.0f * cyc, &s, &c);
  return make_float2(c, s);
}

}  // namespace pt
