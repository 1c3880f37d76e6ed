// Tensor-core (tcgen05) form of the 512-point inverse DFT, the transform under
// PhaseScreen.generate (src/pyturb/fourier.py:259) and Atmosphere._integrate
// (src/pyturb/atmosphere.py:918), as a four-step DFT of two small matrix
// products instead of an FFT.
//
// n = 16 n1 + n2 (n1 < 32, n2 < 16), k = k1 + 32 k2 (k1 < 32, k2 < 16):
//   X[k1 + 32 k2] = sum_{n2} W16^{n2 k2} W512^{n2 k1} sum_{n1} W32^{n1 k1} x[16 n1 + n2],
// W_N = e^{+2 pi i / N} (the unnormalised inverse transform of numpy.fft.ifft * N).
//
// A persistent CTA of 256 threads (two per SM) transforms 8 lines at a time
// (rows, or columns with a stride). Stage 1: the 128 jobs (line, n2) times
// the real 64 x 64 block form of the 32-point DFT, M = 128, N = 64, K = 64
// (A K-major). Then a twiddle multiply in registers. Stage 2: the 256 jobs
// (line, k1) times the 32 x 32 block form of the 16-point DFT, two M = 128
// tiles, N = 32, K = 32 (A MN-major, so that a thread's 8 consecutive k1 rows
// are one 16-byte store). Operands are split into two fp16 terms (x = hi +
// lo + O(2^-24 x)) after each line is scaled by a power of two that keeps
// them in fp16 range; the three products hi hi, hi lo, lo hi accumulate in
// fp32 in tensor memory, and the scale is undone on the way out. The lines
// are staged through shared memory, so loads and stores coalesce for both
// the row and the column pass.
#include <cuda_fp16.h>
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
constexpr int N = 512, N1 = 32, N2 = 16, LINES = 8, THREADS = 256;
constexpr int A1_TILE = 128 * 64 * 2;   // bytes of one fp16 term of a stage-1 A tile
constexpr int B1_TILE = 64 * 64 * 2;    // stage-1 B (the 32-point DFT block matrix)
constexpr int A2_TILE = 128 * 32 * 2;   // one stage-2 A tile, one term
constexpr int B2_TILE = 32 * 32 * 2;    // stage-2 B (the 16-point DFT block matrix)
constexpr int TERMS = 2;
// shared memory: staged lines (fp32 complex) | A (stage 1, reused by stage 2) |
// B1 | B2, 92 KB, two CTAs an SM (the twiddles live in registers).
// Unswizzled operands need 16-byte alignment; the base is rounded up to 128
// bytes.
// The staged lines: rows as xs[r * N + n]; columns as xs[n * XCS + r], so
// that a row index's 8 lines (64 bytes in memory) arrive in 16-byte copies
// and the stage-1 reads stay free of bank conflicts (a stride of 10 float2).
constexpr int XCS = 10;
constexpr int OFF_X = 0;
constexpr int OFF_A = OFF_X + N * XCS * 8;                         // 40 KB
constexpr int OFF_B1 = OFF_A + TERMS * A1_TILE;                    // + 32 KB
constexpr int OFF_B2 = OFF_B1 + TERMS * B1_TILE;                   // + 16 KB
constexpr int SMEM = OFF_B2 + TERMS * B2_TILE + 128;               // + 4 KB + alignment
static_assert(2 * TERMS * A2_TILE <= TERMS * A1_TILE, "stage-2 tiles reuse the stage-1 space");
static_assert(LINES * N * 8 <= TERMS * A1_TILE, "the output lines are staged in the operand space");
// The stage-1 operand of a line is scaled by a power of two so that its
// largest component is below 2^kScaleExp: the fp16 terms then stay in range
// through the 32-point stage (|Y| <= 32 sqrt(2) 2^9 < 65504).
constexpr int kScaleExp = 9;

// two values as fp16 hi and lo terms (v = hi + lo + O(2^-24 v), round to
// nearest twice), packed in pairs (a at the lower address)
__device__ __forceinline__ void split2h(float a, float b, uint32_t& hi, uint32_t& lo) {
  const __half2 h = __floats2half2_rn(a, b);
  const float2 hf = __half22float2(h);
  const __half2 l = __floats2half2_rn(a - hf.x, b - hf.y);
  hi = *reinterpret_cast<const uint32_t*>(&h);
  lo = *reinterpret_cast<const uint32_t*>(&l);
}

// Element n of line r of the staged group.
template <bool kCols>
__device__ __forceinline__ int xat(int r, int n) { return kCols ? n * XCS + r : r * N + n; }

// Issue the asynchronous copies of group grp's 8 lines into xs: rows are one
// contiguous 32 KB block, columns 64 bytes a row index; 16-byte copies.
template <bool kCols>
__device__ __forceinline__ void stage_group(const float2* in, long long img, int grp, float2* xs) {
  const int L0 = grp * LINES;
  const float2* src = in + (L0 / N) * img + (long long)(L0 % N) * (kCols ? 1 : N);
  if (!kCols) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int c = threadIdx.x + THREADS * i;  // 16-byte chunk
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                       (uint32_t)__cvta_generic_to_shared(xs + 2 * c)),
                   "l"(src + 2 * c)
                   : "memory");
    }
  } else {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int c = threadIdx.x + THREADS * i, n = c >> 2, r = 2 * (c & 3);  // lines r, r + 1
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                       (uint32_t)__cvta_generic_to_shared(xs + n * XCS + r)),
                   "l"(src + (long long)n * N + r)
                   : "memory");
    }
  }
  asm volatile("cp.async.commit_group;" ::: "memory");
}

// Instruction descriptor of kind::f16 with fp16 A and B (format 0), fp32 D,
// K-major unless kMajorMN_A.
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N) {
  return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// The stage-2 A tiles are MN-major without swizzle: 8 consecutive rows (M) of
// one K index make a 16-byte core-matrix row, 8 K indices a core matrix; core
// matrices are 128 bytes apart along M and A2_KCORE apart along K.
constexpr int A2_KCORE = 16 * 128;
constexpr uint32_t kMajorMN_A = 1u << 15;  // instruction descriptor: A is MN-major
__device__ __forceinline__ uint32_t mn_offset(int mcore, int k) {
  return (uint32_t)(mcore * 128 + (k >> 3) * A2_KCORE + (k & 7) * 16);
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
    const __half h = __float2half_rn(v);
    const __half l = __float2half_rn(v - __half2float(h));
    const uint32_t off = tc::core_offset(o, kk, K);
    *(__half*)(sb + off) = h;
    *(__half*)(sb + tile_bytes + off) = l;
  }
}
}  // namespace dft

// Persistent CTAs of 256 threads: groups of 8 lines g = blockIdx.x, +
// gridDim.x, ...; line L: image L / 512, index j = L % 512; element n of line
// (b, j) at in[b * img + j * 512 + n] (rows) or in[b * img + n * 512 + j]
// (kCols), complex units. in and out may alias: a CTA reads all of a group's
// lines before it writes them, and no two CTAs touch the same line. The DFT
// matrices and the twiddles are built once per CTA. Each phase splits its
// 128 rows (stage-1 jobs, tensor-memory lanes) between the two halves of the
// CTA by columns.
template <bool kCols>
__global__ void __launch_bounds__(dft::THREADS, 2)
k_dft512_tc(const float2* in, float2* out, int lines, long long img) {
  constexpr int ls = kCols ? 1 : dft::N;  // line stride (complex units)
  using namespace dft;
  extern __shared__ uint8_t smraw[];
  __shared__ uint64_t bar;
  __shared__ uint32_t tslot;
  __shared__ float sc[LINES], isc[LINES];  // per-line power-of-two scale and its inverse
  uint8_t* base = (uint8_t*)(((uintptr_t)smraw + 127) & ~(uintptr_t)127);
  float2* xs = (float2*)(base + OFF_X);
  uint8_t* sA = base + OFF_A;
  float2* ob = (float2*)sA;  // the transformed lines, staged in the dead operand space
  uint8_t* sB1 = base + OFF_B1;
  uint8_t* sB2 = base + OFF_B2;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int q = tid & 127, half = tid >> 7;  // row (job / TMEM lane) and column half
  const int groups = lines / LINES;
  if ((int)blockIdx.x >= groups) return;

  if (warp == 0) tc::tmem_alloc(&tslot, 128);
  if (tid == 0) {
    tc::mbar_init(&bar, 1);
    tc::fence_mbar_init();
  }
  build_dft_b<N1>(sB1, B1_TILE);
  build_dft_b<N2>(sB2, B2_TILE);
  // the twiddles W512^{n2 k1} of this thread's stage-1 row (n2 = q % 16) and
  // column half (k1 in [16 half, 16 half + 16))
  float twr[16], twi[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    const float2 w = unit((q & 15) * (16 * half + i), N);
    twr[i] = w.x;
    twi[i] = w.y;
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tslot;
  // this warp's tensor-memory lane quarter
  const uint32_t trow = tmem + ((uint32_t)((warp & 3) * 32) << 16);
  constexpr int NPROD = 3;  // hi hi, hi lo, lo hi
  constexpr int pa[NPROD] = {0, 0, 1};
  constexpr int pb[NPROD] = {0, 1, 0};
  bool alive = true;
  // the first group's lines; every later group is prefetched while the one
  // before it is transformed (xs is free once the stage-1 operand is built)
  stage_group<kCols>(in, img, blockIdx.x, xs);
  for (int grp = blockIdx.x; grp < groups && alive; grp += gridDim.x) {
    const int L0 = grp * LINES;
    const long long b = L0 / N;
    const int j0 = L0 % N;
    float2* dst = out + b * img + (long long)j0 * ls;
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    __syncthreads();
    {
      // line r = warp: the power of two that puts its largest component below 2^kScaleExp
      float mx = 0.f;
#pragma unroll
      for (int i = 0; i < N / 32; ++i) {
        const float2 v = xs[xat<kCols>(warp, lane + 32 * i)];
        mx = fmaxf(mx, fmaxf(fabsf(v.x), fabsf(v.y)));
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
      if (lane == 0) {
        int ex = 0;
        if (mx > 0.f) frexpf(mx, &ex);  // mx < 2^ex
        sc[warp] = ldexpf(1.f, kScaleExp - ex);
        isc[warp] = ldexpf(1.f, ex - kScaleExp);
      }
    }
    __syncthreads();
    // stage-1 A (K-major): job q = 16 r + n2, K = [re x[16 n1 + n2] (n1 < 32) | im ...],
    // scaled by the line's sc; this half: n1 in [16 half, 16 half + 16)
    {
      const int r = q >> 4, n2 = q & 15;
      const float s1 = sc[r];
#pragma unroll
      for (int gg = 0; gg < 2; ++gg) {
        const int g = 2 * half + gg;  // n1 in [8 g, 8 g + 8): K groups g (re) and g + 4 (im)
        uint32_t wr[TERMS][4], wi[TERMS][4];
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          const float2 xa = xs[xat<kCols>(r, 16 * (8 * g + 2 * h) + n2)];
          const float2 xb = xs[xat<kCols>(r, 16 * (8 * g + 2 * h + 1) + n2)];
          split2h(xa.x * s1, xb.x * s1, wr[0][h], wr[1][h]);
          split2h(xa.y * s1, xb.y * s1, wi[0][h], wi[1][h]);
        }
        const uint32_t o_re = tc::core_offset(q, 8 * g, 64), o_im = tc::core_offset(q, 32 + 8 * g, 64);
#pragma unroll
        for (int t = 0; t < TERMS; ++t) {
          *(uint4*)(sA + t * A1_TILE + o_re) = make_uint4(wr[t][0], wr[t][1], wr[t][2], wr[t][3]);
          *(uint4*)(sA + t * A1_TILE + o_im) = make_uint4(wi[t][0], wi[t][1], wi[t][2], wi[t][3]);
        }
      }
    }
    tc::fence_proxy_async_smem();
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    if (grp + (int)gridDim.x < groups) stage_group<kCols>(in, img, grp + gridDim.x, xs);
    if (tid == 0) {
      const uint32_t idesc = idesc_f16(128, 64);
      const uint32_t a0 = tc::smem_u32(sA), b0 = tc::smem_u32(sB1);
      for (int p = 0; p < NPROD; ++p)
        for (int ks = 0; ks < 4; ++ks) {
          const uint64_t ad = tc::smem_desc(a0 + pa[p] * A1_TILE + ks * 256, 128, 64 * 16);
          const uint64_t bd = tc::smem_desc(b0 + pb[p] * B1_TILE + ks * 256, 128, 64 * 16);
          tc::mma_bf16(tmem, ad, bd, idesc, (p | ks) ? 1u : 0u);
        }
      tc::mma_commit(&bar);
    }
    bool ok = true;  // one warp polls the barrier; the others sleep in the CTA barrier
    if (warp == 0) ok = tc::mbar_wait(&bar, 0, &g_dft_error);
    ok = __syncthreads_and(ok);  // also: every thread is past the wait before A is rewritten
    tc::tc_fence_after();
    if (!ok) {
      alive = false;
      break;
    }
    {
      // row q of D1: Y[r][n2][k1] (re in columns k1, im in 32 + k1), this
      // half's k1 in [16 half, +16); twiddle W512^{n2 k1}, then stage-2 A
      // (MN-major): job (r, k1) -> tile r / 4, row 32 (r % 4) + k1, K = [re
      // (n2 < 16) | im]; 8 consecutive k1 make one 16-byte store
      const int r = q >> 4, n2 = q & 15;
      float re[16], im[16];
      tc::tmem_ld16(trow + 16 * half, re);
      tc::tmem_ld16(trow + 32 + 16 * half, im);
      uint8_t* tile = sA + (r >> 2) * (TERMS * A2_TILE);
#pragma unroll
      for (int jj = 0; jj < 2; ++jj) {  // rows 32 (r % 4) + 8 j .. + 7, j = 2 half + jj
        uint32_t wr[TERMS][4], wi[TERMS][4];
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          const int ka = 8 * jj + 2 * h, kb = ka + 1;
          split2h(re[ka] * twr[ka] - im[ka] * twi[ka], re[kb] * twr[kb] - im[kb] * twi[kb],
                  wr[0][h], wr[1][h]);
          split2h(re[ka] * twi[ka] + im[ka] * twr[ka], re[kb] * twi[kb] + im[kb] * twr[kb],
                  wi[0][h], wi[1][h]);
        }
        const int mc = 4 * (r & 3) + 2 * half + jj;  // core matrix along M
        const uint32_t o_re = mn_offset(mc, n2), o_im = mn_offset(mc, 16 + n2);
#pragma unroll
        for (int t = 0; t < TERMS; ++t) {
          *(uint4*)(tile + t * A2_TILE + o_re) = make_uint4(wr[t][0], wr[t][1], wr[t][2], wr[t][3]);
          *(uint4*)(tile + t * A2_TILE + o_im) = make_uint4(wi[t][0], wi[t][1], wi[t][2], wi[t][3]);
        }
      }
    }
    tc::fence_proxy_async_smem();
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    if (tid == 0) {
      const uint32_t idesc = idesc_f16(128, 32) | kMajorMN_A;
      const uint32_t b0 = tc::smem_u32(sB2);
      for (int m = 0; m < 2; ++m) {
        const uint32_t a0 = tc::smem_u32(sA + m * (TERMS * A2_TILE));
        for (int p = 0; p < NPROD; ++p)
          for (int ks = 0; ks < 2; ++ks) {
            const uint64_t ad = tc::smem_desc(a0 + pa[p] * A2_TILE + ks * 2 * A2_KCORE, A2_KCORE, 128);
            const uint64_t bd = tc::smem_desc(b0 + pb[p] * B2_TILE + ks * 256, 128, 32 * 16);
            tc::mma_bf16(tmem + 64 + 32 * m, ad, bd, idesc, (p | ks) ? 1u : 0u);
          }
      }
      tc::mma_commit(&bar);
    }
    bool ok2 = true;
    if (warp == 0) ok2 = tc::mbar_wait(&bar, 1, &g_dft_error);
    ok2 = __syncthreads_and(ok2);
    tc::tc_fence_after();
    if (!ok2) {
      alive = false;
      break;
    }
    {
      // tile m = half, row 32 (warp % 4) + lane = job (r = 4 m + warp % 4, k1 = lane):
      // X[r][k1 + 32 k2], re in columns k2, im in 16 + k2
      float v[32];
      tc::tmem_ld16(trow + 64 + 32 * half, v);
      tc::tmem_ld16(trow + 64 + 32 * half + 16, v + 16);
      const int r = 4 * half + (warp & 3), k1 = lane;
      const float u = isc[r];
#pragma unroll
      for (int k2 = 0; k2 < 16; ++k2)
        ob[r * N + k1 + 32 * k2] = make_float2(v[k2] * u, v[16 + k2] * u);
    }
    tc::tc_fence_before();
    __syncthreads();
#pragma unroll 4
    for (int i = 0; i < 8; ++i) {
      const int e4 = tid + THREADS * i;
      if (kCols) {
        const int n = e4 >> 2, r = 2 * (e4 & 3);
        const float2 u = ob[r * N + n], w = ob[(r + 1) * N + n];
        *(float4*)(dst + (e4 >> 2) * N + r) = make_float4(u.x, u.y, w.x, w.y);
      } else {
        *(float4*)(dst + (e4 >> 8) * N + 2 * (e4 & 255)) = *(const float4*)(ob + 2 * e4);
      }
    }
    __syncthreads();
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 128);
}

// The tensor-core DFT's error word (bounded waits that ran out), for
// pt_device_error.
int dft_device_error(int* out, int clear) {
  int v = 0;
  if (int rc = check_cuda(cudaMemcpyFromSymbol(&v, g_dft_error, sizeof(int)), "dft error word"))
    return rc;
  if (clear) {
    const int z = 0;
    if (int rc = check_cuda(cudaMemcpyToSymbol(g_dft_error, &z, sizeof(int)), "dft error word"))
      return rc;
  }
  *out = v;
  return PT_OK;
}

}  // namespace pt

using namespace pt;

// Unnormalised inverse 2-D DFT of `batch` complex 512 x 512 images on the
// tensor cores (in and out may alias): a row pass, then a column pass in
// place. No reference counterpart beyond the transform it replaces.
extern "C" int pt_ifft2_tc(int ns, const float* in, float* out, int batch, void* stream) {
  if (ns != dft::N) return fail(PT_ERR_UNSUPPORTED, "pt_ifft2_tc: the tensor-core DFT is built for ns = 512");
  if (!in || !out || batch < 0) return fail(PT_ERR_ARG, "pt_ifft2_tc: bad arguments");
  if ((uintptr_t)in % 16 || (uintptr_t)out % 16)
    return fail(PT_ERR_ARG, "pt_ifft2_tc: in and out must be 16-byte aligned");
  if (batch == 0) return PT_OK;
  if ((long long)batch * dft::N > 0x7fffffffLL)
    return fail(PT_ERR_ARG, "pt_ifft2_tc: batch too large");
  cudaStream_t s = (cudaStream_t)stream;
  static int resident = 0;  // CTAs of k_dft512_tc the device holds at once
  if (!resident) {
    int dev = 0;
    if (int rc = check_cuda(cudaGetDevice(&dev), "pt_ifft2_tc: device")) return rc;
    cudaDeviceProp prop;
    if (int rc = check_cuda(cudaGetDeviceProperties(&prop, dev), "pt_ifft2_tc: properties")) return rc;
    // CTAs per SM from the SM's shared memory and registers (the occupancy
    // calculator does not follow the carveout preference)
    int per_sm = 4;
    for (const void* f : {(const void*)k_dft512_tc<false>, (const void*)k_dft512_tc<true>}) {
      if (int rc = check_cuda(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, dft::SMEM),
                              "pt_ifft2_tc: shared memory"))
        return rc;
      if (int rc = check_cuda(cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout,
                                                   (int)cudaSharedmemCarveoutMaxShared),
                              "pt_ifft2_tc: carveout"))
        return rc;
      cudaFuncAttributes fa;
      if (int rc = check_cuda(cudaFuncGetAttributes(&fa, f), "pt_ifft2_tc: attributes")) return rc;
      const size_t per_cta = (size_t)dft::SMEM + fa.sharedSizeBytes + prop.reservedSharedMemPerBlock;
      per_sm = std::min(per_sm, (int)(prop.sharedMemPerMultiprocessor / per_cta));
      per_sm = std::min(per_sm, prop.regsPerMultiprocessor / std::max(1, fa.numRegs * dft::THREADS));
    }
    if (per_sm < 1) return fail(PT_ERR_UNSUPPORTED, "pt_ifft2_tc: the kernel does not fit on an SM");
    resident = prop.multiProcessorCount * per_sm;
  }
  const int lines = batch * dft::N;
  const long long img = (long long)dft::N * dft::N;
  // persistent: one wave of resident CTAs, each over many groups of 8 lines
  const dim3 grid((unsigned)std::min(lines / dft::LINES, resident));
  {
    ProfScope ps("k_dft512_tc", s);
    k_dft512_tc<false><<<grid, dft::THREADS, dft::SMEM, s>>>((const float2*)in, (float2*)out, lines, img);
    k_dft512_tc<true><<<grid, dft::THREADS, dft::SMEM, s>>>((const float2*)out, (float2*)out, lines, img);
  }
  count_launch_d(2);
  return check_launch("pt_ifft2_tc");
}
