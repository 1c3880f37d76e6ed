// Tensor-core (tcgen05) form of the Assemat-Wilson extrusion product, and a
// one-tile self-test of the tcgen05 path.
//
// The extrusion step is new_row = [A | B_unit] [stencil ; bscale * beta] for
// every screen that needs a row (_ExtrudeLayer._extrude_one,
// src/pyturb/extrude.py:424-430): a GEMM with M = W output pixels, N = screens
// and K = (m + 1) W plus any sparse stencil points. Here both operands are
// split into bf16 terms, x = x_hi + x_lo (+ x_mid), and the products
// accumulate in fp32 in tensor memory.

#include <cuda_bf16.h>
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

// ------------------------------------------------------------------ extrusion GEMM
// Operand tiles: 128 (A) or NP (B) rows x kTcKc columns of one bf16 term in
// the core-matrix layout (SBO = kTcKc * 16 B). The terms of one
// (row tile, K chunk) are contiguous, so one bulk copy stages all of them.
using tc::kTcKc;
constexpr int kTcM = 128;
constexpr int kTcTileA = kTcM * kTcKc * 2;  // bytes of one A term tile
constexpr size_t kTcSmemMax = 227 * 1024;
constexpr int kTcMaxStages = 6;

__device__ __forceinline__ void split_bf16(float x, int terms, uint16_t* t) {
  float r = x;
  for (int i = 0; i < terms; ++i) {
    const __nv_bfloat16 h = __float2bfloat16_rn(r);
    t[i] = __bfloat16_as_ushort(h);
    r -= __bfloat162float(h);
  }
}

// tiles[(((g * MT + mt) * nkc + kc) * terms + t) * kTcTileA + core(r % 128, k % kTcKc)]
__global__ void k_tc_prepare(int W, int K, int G, int MT, int nkc, int terms,
                             const float* __restrict__ M, uint8_t* __restrict__ tiles) {
  const size_t cols = (size_t)nkc * kTcKc;
  const size_t total = (size_t)G * MT * kTcM * cols;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(i % cols);
    const size_t rg = i / cols;
    const int r = (int)(rg % ((size_t)MT * kTcM));
    const int g = (int)(rg / ((size_t)MT * kTcM));
    const float x = (r < W && k < K) ? M[((size_t)g * W + r) * K + k] : 0.f;
    uint16_t t[3];
    split_bf16(x, terms, t);
    const int mt = r / kTcM, kc = k / kTcKc;
    uint8_t* blk = tiles + (((size_t)g * MT + mt) * nkc + kc) * terms * kTcTileA;
    const uint32_t off = tc::core_offset(r % kTcM, k % kTcKc, kTcKc);
    for (int q = 0; q < terms; ++q) *(uint16_t*)(blk + (size_t)q * kTcTileA + off) = t[q];
  }
}

// partial[z][j][r] = sum over K chunks [z cps, (z + 1) cps) of sum over term
// products of A_ta[r][k] X_tb[j][k]: one 128-row tile per CTA, the job
// columns (NP <= 256) in one TMEM accumulator. Thread 0 drives a STAGES-deep
// bulk-copy pipeline and issues the MMAs; all four warps read TMEM back.
template <int TERMS>
__global__ void __launch_bounds__(128)
k_tc_gemm(int W, int J, int NP, int nkc, int cps, int stages, const uint8_t* __restrict__ At,
          const uint8_t* __restrict__ Bt, float* __restrict__ partial) {
  constexpr int NPROD = TERMS == 1 ? 1 : (TERMS == 2 ? 3 : 6);
  constexpr int pa[6] = {0, 0, 1, 0, 2, 1};
  constexpr int pb[6] = {0, 1, 0, 2, 0, 1};
  extern __shared__ uint8_t smraw[];
  __shared__ uint64_t full[kTcMaxStages], empty[kTcMaxStages], done;
  __shared__ uint32_t tslot;
  uint8_t* base = (uint8_t*)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int mt = blockIdx.x, z = blockIdx.y;
  const int MT = gridDim.x;
  const int kc0 = z * cps, kc1 = min(nkc, kc0 + cps);
  const int n = kc1 - kc0;
  const uint32_t bytesA = TERMS * kTcTileA, bytesB = TERMS * NP * kTcKc * 2;
  const uint32_t stage_bytes = bytesA + bytesB;
  if (warp == 0) tc::tmem_alloc(&tslot, 256);
  if (tid == 0) {
    for (int q = 0; q < stages; ++q) {
      tc::mbar_init(&full[q], 1);
      tc::mbar_init(&empty[q], 1);
    }
    tc::mbar_init(&done, 1);
    tc::fence_mbar_init();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tslot;
  // lane 0 of warp 0 drives the copies and MMAs; its warp-mates park at the
  // __syncwarp below instead of spinning on `done` in the same warp
  if (tid == 0 && n > 0) {
    const uint8_t* a_src = At + ((size_t)mt * nkc) * TERMS * kTcTileA;
    const uint8_t* b_src = Bt;
    // the operator is re-read every row step: keep it in L2 ahead of the
    // per-step operand and partials
    const uint64_t keep = tc::policy_evict_last();
    auto load = [&](int c) {  // chunk c (relative) into stage c % stages
      uint8_t* st = base + (size_t)(c % stages) * stage_bytes;
      uint64_t* fb = &full[c % stages];
      tc::mbar_expect_tx(fb, stage_bytes);
      tc::bulk_g2s_hint(st, a_src + (size_t)(kc0 + c) * TERMS * kTcTileA, bytesA, fb, keep);
      tc::bulk_g2s(st + bytesA, b_src + (size_t)(kc0 + c) * bytesB, bytesB, fb);
    };
    // all stages filled up front; afterwards the stage of chunk i - 1 is
    // refilled with chunk i - 1 + stages once chunk i's MMAs are queued, so
    // the wait for chunk i - 1 overlaps chunk i on the tensor pipe
    for (int c = 0; c < min(stages, n); ++c) load(c);
    const uint32_t idesc = tc::idesc_bf16(kTcM, NP);
    for (int i = 0; i < n; ++i) {
      if (!tc::mbar_wait(&full[i % stages], (i / stages) & 1, &g_tc_error)) break;
      tc::tc_fence_after();
      const uint32_t sa = tc::smem_u32(base + (size_t)(i % stages) * stage_bytes);
      const uint32_t sb = sa + bytesA;
#pragma unroll
      for (int ks = 0; ks < kTcKc / 16; ++ks)
#pragma unroll
        for (int p = 0; p < NPROD; ++p) {
          const uint64_t ad = tc::smem_desc(sa + pa[p] * kTcTileA + ks * 256, 128, kTcKc * 16);
          const uint64_t bd = tc::smem_desc(sb + pb[p] * NP * kTcKc * 2 + ks * 256, 128,
                                            kTcKc * 16);
          tc::mma_bf16(tmem, ad, bd, idesc, (i | ks | p) ? 1u : 0u);
        }
      tc::mma_commit(&empty[i % stages]);
      const int prev = i - 1, next = i - 1 + stages;
      if (prev >= 0 && next < n) {
        if (!tc::mbar_wait(&empty[prev % stages], (prev / stages) & 1, &g_tc_error)) break;
        load(next);
      }
    }
    tc::mma_commit(&done);
  }
  if (warp == 0) __syncwarp();
  bool ok = n > 0 ? tc::mbar_wait(&done, 0, &g_tc_error) : true;
  ok = __all_sync(0xffffffffu, ok);
  tc::tc_fence_after();
  if (ok) {
    const int r = mt * kTcM + warp * 32 + lane;
    float* pz = partial + (size_t)z * J * W;
    for (int c0 = 0; c0 < NP; c0 += 16) {
      float v[16];
      tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
      if (r < W) {
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const int j = c0 + q;
          if (j < J) __stcs(pz + (size_t)j * W + r, n > 0 ? v[q] : 0.f);  // read once
        }
      }
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 256);
  (void)MT;
}

// Geometry shared by the host side.
struct TcShape {
  int K, MT, nkc, NP, cps, nz, stages;
  size_t stage_bytes;
};
TcShape tc_shape(int W, int K, int J, int terms) {
  TcShape t{};
  t.K = K;
  t.MT = (W + kTcM - 1) / kTcM;
  t.nkc = (t.K + kTcKc - 1) / kTcKc;
  t.NP = std::max(16, (J + 15) / 16 * 16);
  const int want = std::max(1, 148 / t.MT);  // about one CTA per SM
  t.cps = (t.nkc + want - 1) / want;
  t.nz = (t.nkc + t.cps - 1) / t.cps;
  t.stage_bytes = (size_t)terms * (kTcTileA + (size_t)t.NP * kTcKc * 2);
  // one CTA per SM with as many stages as fit in 227 KB (less static shared
  // memory and the 1 KB alignment pad)
  t.stages = (int)std::min<size_t>(kTcMaxStages, (kTcSmemMax - 2048) / t.stage_bytes);
  return t;
}
int tc_max_jobs(int terms) { return terms == 3 ? 160 : 192; }
size_t tc_operator_bytes(int W, int K, int G, int terms) {
  const TcShape t = tc_shape(W, K, 1, terms);
  return (size_t)G * t.MT * t.nkc * terms * kTcTileA;
}
size_t tc_btile_bytes(int W, int K, int J, int terms) {
  const TcShape t = tc_shape(W, K, J, terms);
  return (size_t)t.nkc * terms * t.NP * kTcKc * 2;
}

size_t tc_partial_floats(int W, int K, int J, int terms) {
  const TcShape t = tc_shape(W, K, J, terms);
  return (size_t)t.nz * J * W;
}

int tc_prepare_launch(int W, int K, int G, const float* M, int terms, void* tiles,
                      cudaStream_t s) {
  const TcShape t = tc_shape(W, K, 1, terms);
  const size_t total = (size_t)G * t.MT * kTcM * t.nkc * kTcKc;
  const int blocks = (int)std::min<size_t>((total + 255) / 256, 152 * 16);
  k_tc_prepare<<<blocks, 256, 0, s>>>(W, t.K, G, t.MT, t.nkc, terms, M, (uint8_t*)tiles);
  count_launch_t();
  return check_launch("pt_extrude_tc_prepare");
}

int tc_gemm_launch(int W, int K, int J, int terms, const uint8_t* At, const uint8_t* Bt,
                   float* partial, int* nz_out, cudaStream_t s) {
  const TcShape t = tc_shape(W, K, J, terms);
  if (t.stages < 2) return fail(PT_ERR_UNSUPPORTED, "extrusion tensor-core form: too many jobs");
  const size_t smem = (size_t)t.stages * t.stage_bytes + 1024;
  dim3 grid(t.MT, t.nz);
  if (terms == 1) {  // the float32 form's operator correction
    ProfScope ps("k_tc_gemm_lo", s);
    static bool attr = false;
    if (!attr) {
      if (int rc = check_cuda(cudaFuncSetAttribute(k_tc_gemm<1>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)(kTcSmemMax - 1024)), "k_tc_gemm"))
        return rc;
      attr = true;
    }
    k_tc_gemm<1><<<grid, 128, smem, s>>>(W, J, t.NP, t.nkc, t.cps, t.stages, At, Bt, partial);
    count_launch_t();
    *nz_out = t.nz;
    return check_launch("k_tc_gemm");
  }
  ProfScope ps("k_tc_gemm", s);
  if (terms == 2) {
    static bool attr = false;
    if (!attr) {
      if (int rc = check_cuda(cudaFuncSetAttribute(k_tc_gemm<2>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)(kTcSmemMax - 1024)), "k_tc_gemm"))
        return rc;
      attr = true;
    }
    k_tc_gemm<2><<<grid, 128, smem, s>>>(W, J, t.NP, t.nkc, t.cps, t.stages, At, Bt, partial);
  } else {
    static bool attr = false;
    if (!attr) {
      if (int rc = check_cuda(cudaFuncSetAttribute(k_tc_gemm<3>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)(kTcSmemMax - 1024)), "k_tc_gemm"))
        return rc;
      attr = true;
    }
    k_tc_gemm<3><<<grid, 128, smem, s>>>(W, J, t.NP, t.nkc, t.cps, t.stages, At, Bt, partial);
  }
  count_launch_t();
  *nz_out = t.nz;
  return check_launch("k_tc_gemm");
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
