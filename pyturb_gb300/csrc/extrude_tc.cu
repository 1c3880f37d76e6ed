// Tensor-core (tcgen05) form of the Assemat-Wilson extrusion product, and a
// one-tile self-test of the tcgen05 path.
//
// The extrusion step is new_row = [A | B_unit] [stencil ; bscale * beta] for
// every screen that needs a row (_ExtrudeLayer._extrude_one,
// src/pyturb/extrude.py:424-430): a GEMM with M = W output pixels, N = screens
// and K = (m + 1) W. Here both operands are split into bf16 terms, x = x_hi +
// x_lo (+ x_mid), and the products accumulate in fp32 in tensor memory.

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "common.cuh"
#include "tc.cuh"

namespace pt {
uint64_t* launch_counter();
static inline void count_launch_t(int k = 1) {
  __atomic_add_fetch(launch_counter(), (uint64_t)k, __ATOMIC_RELAXED);
}

__device__ int g_tc_error;

// One tile: D (128 x N) = A (128 x K) B (N x K)^T, bf16 operands (row-major,
// K contiguous), fp32 D row-major. 128 threads; N, K multiples of 16, N <= 256.
__global__ void __launch_bounds__(128)
k_tc_probe(int N, int K, const uint16_t* __restrict__ A, const uint16_t* __restrict__ B,
           float* __restrict__ D) {
  extern __shared__ uint8_t smraw[];
  __shared__ uint64_t bar;
  __shared__ uint32_t tslot;
  uint8_t* base = (uint8_t*)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  uint8_t* sA = base;
  uint8_t* sB = base + (size_t)128 * K * 2;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int i = tid; i < 128 * K; i += blockDim.x)
    *(uint16_t*)(sA + tc::core_offset(i / K, i % K, K)) = A[i];
  for (int i = tid; i < N * K; i += blockDim.x)
    *(uint16_t*)(sB + tc::core_offset(i / K, i % K, K)) = B[i];
  if (warp == 0) tc::tmem_alloc(&tslot, 256);
  if (tid == 0) {
    tc::mbar_init(&bar, 1);
    tc::fence_mbar_init();
  }
  tc::fence_proxy_async_smem();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tslot;
  if (tid == 0) {
    const uint32_t idesc = tc::idesc_bf16(128, N);
    const uint32_t a0 = tc::smem_u32(sA), b0 = tc::smem_u32(sB);
    for (int ks = 0; ks < K / 16; ++ks) {
      const uint64_t ad = tc::smem_desc(a0 + ks * 256, 128, K * 16);
      const uint64_t bd = tc::smem_desc(b0 + ks * 256, 128, K * 16);
      tc::mma_bf16(tmem, ad, bd, idesc, ks > 0 ? 1u : 0u);
    }
    tc::mma_commit(&bar);
  }
  bool ok = tc::mbar_wait(&bar, 0, &g_tc_error);
  ok = __all_sync(0xffffffffu, ok);
  tc::tc_fence_after();
  if (ok) {
    const int row = warp * 32 + lane;
    for (int c0 = 0; c0 < N; c0 += 16) {
      float v[16];
      tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
      for (int i = 0; i < 16; ++i) D[(size_t)row * N + c0 + i] = v[i];
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 256);
}

int tc_device_error(int* out, int clear) {
  int v = 0;
  if (int rc = check_cuda(cudaMemcpyFromSymbol(&v, g_tc_error, sizeof(int)), "tc error word"))
    return rc;
  if (clear) {
    const int z = 0;
    if (int rc = check_cuda(cudaMemcpyToSymbol(g_tc_error, &z, sizeof(int)), "tc error word"))
      return rc;
  }
  *out = v;
  return PT_OK;
}

}  // namespace pt

using namespace pt;

extern "C" int pt_tc_probe(int N, int K, const uint16_t* A, const uint16_t* B, float* D,
                           void* stream) {
  if (N < 16 || N > 256 || N % 16 || K < 16 || K > 256 || K % 16)
    return fail(PT_ERR_ARG, "pt_tc_probe: N and K must be multiples of 16 in [16, 256]");
  if (!A || !B || !D) return fail(PT_ERR_ARG, "pt_tc_probe: NULL pointer");
  const size_t smem = (size_t)(128 + N) * K * 2 + 1024;
  if (int rc = check_cuda(cudaFuncSetAttribute(k_tc_probe, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)smem), "pt_tc_probe"))
    return rc;
  cudaStream_t s = (cudaStream_t)stream;
  k_tc_probe<<<1, 128, smem, s>>>(N, K, A, B, D);
  count_launch_t();
  if (int rc = check_launch("pt_tc_probe")) return rc;
  if (int rc = check_cuda(cudaStreamSynchronize(s), "pt_tc_probe")) return rc;
  int err = 0;
  if (int rc = tc_device_error(&err, 1)) return rc;
  if (err) return fail(PT_ERR_CUDA, "pt_tc_probe: an mbarrier wait timed out");
  return PT_OK;
}
