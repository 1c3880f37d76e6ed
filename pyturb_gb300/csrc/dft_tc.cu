// Tensor-core (tcgen05) form of the 512-point inverse DFT, the transform under
// PhaseScreen.generate (src/pyturb/fourier.py:259) and Atmosphere._integrate
// (src/pyturb/atmosphere.py:918), as a four-step DFT of two small matrix
// products instead of an FFT.
//
// n = 16 n1 + n2 (n1 < 32, n2 < 16), k = k1 + 32 k2 (k1 < 32, k2 < 16):
//   X[k1 + 32 k2] = sum_{n2} W16^{n2 k2} W512^{n2 k1} sum_{n1} W32^{n1 k1} x[16 n1 + n2],
// W_N = e^{+2 pi i / N} (the unnormalised inverse transform of numpy.fft.ifft * N).
//
// A CTA of 128 threads transforms 8 lines (rows, or columns with a stride).
// Stage 1: the 128 jobs (line, n2) times the real 64 x 64 block form of the
// 32-point DFT, M = 128, N = 64, K = 64. Then a twiddle multiply in
// registers. Stage 2: the 256 jobs (line, k1) times the 32 x 32 block form of
// the 16-point DFT, two M = 128 tiles, N = 32, K = 32. Operands are split
// into three bf16 terms (x = hi + mid + lo, 24 bits); the six products with
// term indices summing to at most 2 accumulate in fp32 in tensor memory. The
// lines are staged through shared memory, so loads and stores coalesce for
// both the row and the column pass.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "common.cuh"
#include "tc.cuh"

namespace pt {
uint64_t* launch_counter();
static inline void count_launch_d(int k = 1) {
  __atomic_add_fetch(launch_counter(), (uint64_t)k, __ATOMIC_RELAXED);
}

// bounded mbarrier waits that run out record it here (the kernel then skips
// its remaining work and still frees its tensor memory)
static __device__ int g_dft_error;

namespace dft {
constexpr int N = 512, N1 = 32, N2 = 16, LINES = 8;
constexpr int A1_TILE = 128 * 64 * 2;   // bytes of one bf16 term of a stage-1 A tile
constexpr int B1_TILE = 64 * 64 * 2;    // stage-1 B (the 32-point DFT block matrix)
constexpr int A2_TILE = 128 * 32 * 2;   // one stage-2 A tile, one term
constexpr int B2_TILE = 32 * 32 * 2;    // stage-2 B (the 16-point DFT block matrix)
constexpr int TERMS = 3;
// shared memory: staged lines (fp32 complex) | A (stage 1, reused by stage 2) | B1 | B2
constexpr int OFF_X = 0;
constexpr int OFF_A = OFF_X + LINES * N * 8;                       // 32 KB
constexpr int OFF_B1 = OFF_A + TERMS * A1_TILE;                    // + 48 KB
constexpr int OFF_B2 = OFF_B1 + TERMS * B1_TILE;                   // + 24 KB
constexpr int SMEM = OFF_B2 + TERMS * B2_TILE + 1024;              // + 6 KB + alignment
static_assert(2 * TERMS * A2_TILE <= TERMS * A1_TILE, "stage-2 tiles reuse the stage-1 space");

__device__ __forceinline__ void split3(float v, uint16_t* t) {
  float r = v;
#pragma unroll
  for (int i = 0; i < TERMS; ++i) {
    const __nv_bfloat16 h = __float2bfloat16_rn(r);
    t[i] = __bfloat16_as_ushort(h);
    r -= __bfloat162float(h);
  }
}

// e^{+2 pi i num / den} from the exact fraction (num reduced mod den)
__device__ __forceinline__ float2 unit(int num, int den) {
  float s, c;
  sincospif(2.0f * (float)(num % den) / (float)den, &s, &c);
  return make_float2(c, s);
}

// The real block form [[C, -S], [S, C]] of the M-point DFT (M = 32 or 16) as
// a (2M x 2M) B operand: row o (output: re k for o < M, im k - M above),
// column kk (input: re n for kk < M, im n - M above).
template <int M>
__device__ void build_dft_b(uint8_t* sb, int tile_bytes) {
  constexpr int K = 2 * M;
  for (int e = threadIdx.x; e < K * K; e += blockDim.x) {
    const int o = e / K, kk = e % K;
    const int k = o % M, n = kk % M;
    const float2 w = unit(k * n, M);
    float v;
    if (o < M) v = kk < M ? w.x : -w.y;
    else v = kk < M ? w.y : w.x;
    uint16_t t[TERMS];
    split3(v, t);
    const uint32_t off = tc::core_offset(o, kk, K);
#pragma unroll
    for (int q = 0; q < TERMS; ++q) *(uint16_t*)(sb + q * tile_bytes + off) = t[q];
  }
}
}  // namespace dft

// lines [8 blockIdx.x, +8) of `lines`; line L: image L / 512, index j = L % 512;
// element n of line (b, j) at in[b * img + j * ls + n * es] (complex units).
// in and out may alias: a CTA reads all of its lines before it writes them,
// and no two CTAs touch the same line.
__global__ void __launch_bounds__(128)
k_dft512_tc(const float2* in, float2* out, int lines, long long img, int ls, int es) {
  using namespace dft;
  extern __shared__ uint8_t smraw[];
  __shared__ uint64_t bar;
  __shared__ uint32_t tslot;
  uint8_t* base = (uint8_t*)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  float2* xs = (float2*)(base + OFF_X);
  uint8_t* sA = base + OFF_A;
  uint8_t* sB1 = base + OFF_B1;
  uint8_t* sB2 = base + OFF_B2;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int L0 = blockIdx.x * LINES;
  if (L0 >= lines) return;
  const long long b = L0 / N;
  const int j0 = L0 % N;
  const float2* src = in + b * img + (long long)j0 * ls;
  float2* dst = out + b * img + (long long)j0 * ls;

  if (warp == 0) tc::tmem_alloc(&tslot, 128);
  if (tid == 0) {
    tc::mbar_init(&bar, 1);
    tc::fence_mbar_init();
  }
  // stage the 8 lines: along the line when it is contiguous, else across the lines
  if (es == 1) {
    for (int e = tid; e < LINES * N; e += 128) xs[e] = src[(long long)(e / N) * ls + e % N];
  } else {
    for (int e = tid; e < LINES * N; e += 128) {
      const int n = e / LINES, r = e % LINES;
      xs[r * N + n] = src[(long long)n * es + (long long)r * ls];
    }
  }
  build_dft_b<N1>(sB1, B1_TILE);
  build_dft_b<N2>(sB2, B2_TILE);
  __syncthreads();
  // stage-1 A: job q = 16 r + n2, K = [re x[16 n1 + n2] (n1 < 32) | im ...]
  {
    const int q = tid, r = q >> 4, n2 = q & 15;
    for (int g = 0; g < 8; ++g) {  // 8 groups of 8 K values
      uint32_t w4[TERMS][4];
#pragma unroll
      for (int h = 0; h < 4; ++h) {
        uint16_t ta[TERMS], tb[TERMS];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const int kk = 8 * g + 2 * h + u;
          const int n1 = kk & 31;
          const float2 x = xs[r * N + 16 * n1 + n2];
          split3(kk < 32 ? x.x : x.y, u ? tb : ta);
        }
#pragma unroll
        for (int t = 0; t < TERMS; ++t) w4[t][h] = (uint32_t)ta[t] | ((uint32_t)tb[t] << 16);
      }
      const uint32_t off = tc::core_offset(q, 8 * g, 64);
#pragma unroll
      for (int t = 0; t < TERMS; ++t)
        *(uint4*)(sA + t * A1_TILE + off) = make_uint4(w4[t][0], w4[t][1], w4[t][2], w4[t][3]);
    }
  }
  tc::fence_proxy_async_smem();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tslot;
  constexpr int pa[6] = {0, 0, 1, 0, 2, 1};
  constexpr int pb[6] = {0, 1, 0, 2, 0, 1};
  if (tid == 0) {
    const uint32_t idesc = tc::idesc_bf16(128, 64);
    const uint32_t a0 = tc::smem_u32(sA), b0 = tc::smem_u32(sB1);
    for (int p = 0; p < 6; ++p)
      for (int ks = 0; ks < 4; ++ks) {
        const uint64_t ad = tc::smem_desc(a0 + pa[p] * A1_TILE + ks * 256, 128, 64 * 16);
        const uint64_t bd = tc::smem_desc(b0 + pb[p] * B1_TILE + ks * 256, 128, 64 * 16);
        tc::mma_bf16(tmem, ad, bd, idesc, (p | ks) ? 1u : 0u);
      }
    tc::mma_commit(&bar);
  }
  bool ok = tc::mbar_wait(&bar, 0, &g_dft_error);
  ok = __all_sync(0xffffffffu, ok);
  tc::tc_fence_after();
  __syncthreads();  // every thread is past the wait before stage-1 A is overwritten
  if (ok) {
    // row q of D1: Y[r][n2][k1] for k1 < 32 (re in columns 0..31, im 32..63);
    // twiddle W512^{n2 k1}, then stage-2 A: job (r, k1) -> tile r / 4, row
    // 32 (r % 4) + k1, K = [re (n2 < 16) | im]
    const int q = 32 * warp + lane, r = q >> 4, n2 = q & 15;
    float re[32], im[32];
    const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
    tc::tmem_ld16(trow + 0, re);
    tc::tmem_ld16(trow + 16, re + 16);
    tc::tmem_ld16(trow + 32, im);
    tc::tmem_ld16(trow + 48, im + 16);
    uint8_t* tile = sA + (r >> 2) * (TERMS * A2_TILE);
#pragma unroll
    for (int k1 = 0; k1 < 32; ++k1) {
      const float2 w = dft::unit(n2 * k1, N);
      const float yr = re[k1] * w.x - im[k1] * w.y;
      const float yi = re[k1] * w.y + im[k1] * w.x;
      uint16_t tr[TERMS], ti[TERMS];
      dft::split3(yr, tr);
      dft::split3(yi, ti);
      const int row = 32 * (r & 3) + k1;
      const uint32_t o_re = tc::core_offset(row, n2, 32), o_im = tc::core_offset(row, 16 + n2, 32);
#pragma unroll
      for (int t = 0; t < TERMS; ++t) {
        *(uint16_t*)(tile + t * A2_TILE + o_re) = tr[t];
        *(uint16_t*)(tile + t * A2_TILE + o_im) = ti[t];
      }
    }
  }
  tc::fence_proxy_async_smem();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  if (tid == 0 && ok) {
    const uint32_t idesc = tc::idesc_bf16(128, 32);
    const uint32_t b0 = tc::smem_u32(sB2);
    for (int m = 0; m < 2; ++m) {
      const uint32_t a0 = tc::smem_u32(sA + m * (TERMS * A2_TILE));
      for (int p = 0; p < 6; ++p)
        for (int ks = 0; ks < 2; ++ks) {
          const uint64_t ad = tc::smem_desc(a0 + pa[p] * A2_TILE + ks * 256, 128, 32 * 16);
          const uint64_t bd = tc::smem_desc(b0 + pb[p] * B2_TILE + ks * 256, 128, 32 * 16);
          tc::mma_bf16(tmem + 64 + 32 * m, ad, bd, idesc, (p | ks) ? 1u : 0u);
        }
    }
    tc::mma_commit(&bar);
  }
  bool ok2 = ok ? tc::mbar_wait(&bar, 1, &g_dft_error) : false;
  ok2 = __all_sync(0xffffffffu, ok2);
  tc::tc_fence_after();
  if (ok2) {
    // tile m, row 32 warp + lane = job (r = 4 m + warp, k1 = lane): X[r][k1 + 32 k2]
    const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
    for (int m = 0; m < 2; ++m) {
      float v[32];
      tc::tmem_ld16(trow + 64 + 32 * m, v);
      tc::tmem_ld16(trow + 64 + 32 * m + 16, v + 16);
      const int r = 4 * m + warp, k1 = lane;
#pragma unroll
      for (int k2 = 0; k2 < 16; ++k2) xs[r * N + k1 + 32 * k2] = make_float2(v[k2], v[16 + k2]);
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (ok2) {
    if (es == 1) {
      for (int e = tid; e < LINES * N; e += 128) dst[(long long)(e / N) * ls + e % N] = xs[e];
    } else {
      for (int e = tid; e < LINES * N; e += 128) {
        const int n = e / LINES, r = e % LINES;
        dst[(long long)n * es + (long long)r * ls] = xs[r * N + n];
      }
    }
  }
  if (warp == 0) tc::tmem_dealloc(tmem, 128);
}

}  // namespace pt

using namespace pt;

// Unnormalised inverse 2-D DFT of `batch` complex 512 x 512 images on the
// tensor cores (in and out may alias): a row pass, then a column pass in
// place. No reference counterpart beyond the transform it replaces.
extern "C" int pt_ifft2_tc(int ns, const float* in, float* out, int batch, void* stream) {
  if (ns != dft::N) return fail(PT_ERR_UNSUPPORTED, "pt_ifft2_tc: the tensor-core DFT is built for ns = 512");
  if (!in || !out || batch < 0) return fail(PT_ERR_ARG, "pt_ifft2_tc: bad arguments");
  if (batch == 0) return PT_OK;
  if ((long long)batch * dft::N / dft::LINES > 0x7fffffffLL)
    return fail(PT_ERR_ARG, "pt_ifft2_tc: batch too large");
  cudaStream_t s = (cudaStream_t)stream;
  static bool attr = false;
  if (!attr) {
    if (int rc = check_cuda(cudaFuncSetAttribute(k_dft512_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 dft::SMEM),
                            "pt_ifft2_tc: shared memory"))
      return rc;
    attr = true;
  }
  const int lines = batch * dft::N;
  const long long img = (long long)dft::N * dft::N;
  const dim3 grid((unsigned)(lines / dft::LINES));
  {
    ProfScope ps("k_dft512_tc", s);
    k_dft512_tc<<<grid, 128, dft::SMEM, s>>>((const float2*)in, (float2*)out, lines, img, dft::N, 1);
    k_dft512_tc<<<grid, 128, dft::SMEM, s>>>((const float2*)out, (float2*)out, lines, img, 1,
                                             dft::N);
  }
  count_launch_d(2);
  return check_launch("pt_ifft2_tc");
}
