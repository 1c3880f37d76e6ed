// Column pass fed by the Tensor Memory Accelerator (included by spectral.cu
// inside namespace pt, after frames_fast.cuh).
//
// Persistent over frame pairs: a CTA owns C columns and walks the pairs
// pl = blockIdx.y, blockIdx.y + gridDim.y, ... Each pair's C x N column tile
// (64 B x 512 rows at N = 512) is brought into shared memory by
// cp.async.bulk.tensor loads that complete on an mbarrier; two tile buffers
// alternate, so the next-but-one pair's tile is in flight while this pair is
// transformed and written out. Waits on the mbarrier are bounded: after
// kWaitLimit polls the CTA records kErrWaitTimeout in the device error word
// and proceeds, so a lost transfer is reported, never hangs.
#pragma once

constexpr int kErrWaitTimeout = 1;
constexpr long long kWaitLimit = 1ll << 22;

__device__ int g_pt_device_error;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

// Poll the barrier's phase with an upper bound; false (and the device error
// word set) when the bound is exhausted.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity,
                                                  long long limit) {
  const uint32_t addr = smem_u32(bar);
  for (long long it = 0; it < limit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(addr), "r"(parity)
        : "memory");
    if (done) return true;
  }
  atomicOr(&g_pt_device_error, kErrWaitTimeout);
  return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

template <int N>
struct TmaCfg {
  static constexpr int C = RegCfg<N>::C;
  static constexpr int BOXR = N < 256 ? N : 256;  // rows per TMA box (<= 256)
  static constexpr int NBOX = N / BOXR;
  static constexpr uint32_t TILE_BYTES = (uint32_t)N * C * sizeof(float2);
};

template <int N>
__device__ __forceinline__ void issue_tile(const CUtensorMap* map, float2* dst, int y0, int pair,
                                           uint64_t* bar) {
  using Cfg = TmaCfg<N>;
  mbar_arrive_expect_tx(bar, Cfg::TILE_BYTES);
#pragma unroll
  for (int b = 0; b < Cfg::NBOX; ++b)
    tma_load_2d(dst + (size_t)b * Cfg::BOXR * Cfg::C, map, y0, pair * N + b * Cfg::BOXR, bar);
}

template <int N>
__global__ void __launch_bounds__(RegCfg<N>::THREADS, 2)
k_pair_cols_tma(const __grid_constant__ CUtensorMap map, const float2* __restrict__ tw, int npair,
                int pair0, PairStore st) {
  constexpr int T = RegCfg<N>::T, C = RegCfg<N>::C;
  extern __shared__ __align__(128) float2 smf[];
  float2* tiles = smf;                 // 2 x N*C, TMA destinations
  float2* buf = smf + 2 * N * C;       // N*C FFT scratch (column-interleaved)
  float2* stw = buf + N * C;           // stage twiddles
  float2* mtab = stw + N;              // (2, 3P, C)
  uint64_t* bars = reinterpret_cast<uint64_t*>(mtab + 2 * 3 * (st.P > 0 ? st.P : 1) * C);
  const int c = threadIdx.x % C, j = threadIdx.x / C;
  const ColLayout<C> s{buf + c};
  const int y0 = blockIdx.x * C;
  const int y = y0 + c;
  const int P = st.P;
  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    fence_proxy_async();
  }
  load_stage_tw<N>(stw, tw);
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 0; k < 2; ++k) {
      const int pl = blockIdx.y + k * gridDim.y;
      if (pl < npair) issue_tile<N>(&map, tiles + (size_t)k * N * C, y0, pl, &bars[k]);
    }
  }
  const size_t plane = (size_t)st.n_out * st.n_out;
  const int yo = y - st.crop;
  for (int k = 0, pl = blockIdx.y; pl < npair; ++k, pl += gridDim.y) {
    const int b = k & 1;
    const uint32_t parity = (uint32_t)(k >> 1) & 1u;
    const int pair = pair0 + pl;
    const int img_re = pair * st.re_mul + st.re_add;
    const int img_im = pair * st.im_mul + st.im_add;
    const bool do_re = img_re < st.count, do_im = img_im < st.count;
    const int row_re = pl * st.crow_mul + st.crow_re, row_im = pl * st.crow_mul + st.crow_im;
    // subharmonic per-column table of this pair
    for (int i = threadIdx.x; i < 2 * 3 * P * C; i += blockDim.x) {
      const int cc = i % C;
      const int pi = (i / C) % (3 * P);
      const int o = i / (C * 3 * P);
      const bool take = o == 0 ? do_re : do_im;
      const int row = o == 0 ? row_re : row_im;
      float2 m = make_float2(0.f, 0.f);
      if (take) {
        const int p = pi / 3, ii = pi % 3;
        const float2* cf = st.coef + ((size_t)row * P + p) * 9 + ii * 3;
#pragma unroll
        for (int jj = 0; jj < 3; ++jj)
          m = cfma(cf[jj], st.basis[((size_t)p * 3 + jj) * N + y0 + cc], m);
      }
      mtab[i] = m;
    }
    mbar_wait_bounded(&bars[b], parity, kWaitLimit);
    float2 x[8];
    const float2* tile = tiles + (size_t)b * N * C;
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = tile[(j + T * i) * C + c];
    __syncthreads();  // tile b consumed; mtab ready
    if (threadIdx.x == 0) {
      const int nxt = pl + 2 * gridDim.y;
      if (nxt < npair) {
        fence_proxy_async();
        issue_tile<N>(&map, tiles + (size_t)b * N * C, y0, nxt, &bars[b]);
      }
    }
    float k0 = 0.f, k1 = 0.f;
    if (st.sym) {
      for (int p = 0; p < P; ++p) {
        k0 += mtab[(0 * 3 * P + 3 * p + 1) * C + c].x;
        k1 += mtab[(1 * 3 * P + 3 * p + 1) * C + c].x;
      }
      if (P > 0 && do_re) k0 -= st.mean[row_re];
      if (P > 0 && do_im) k1 -= st.mean[row_im];
    }
    reg_fft<N>(x, j, stw, s);
    if (yo >= 0 && yo < st.n_out) {
      const float mre = (P > 0 && do_re) ? st.mean[row_re] : 0.f;
      const float mim = (P > 0 && do_im) ? st.mean[row_im] : 0.f;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int xr = j + T * i;
        const int xo = xr - st.crop;
        if (xo < 0 || xo >= st.n_out) continue;
        float lre, lim;
        if (st.sym) {
          lre = k0;
          lim = k1;
          for (int p = 0; p < P; ++p) {
            const float2 bb = st.basis[(size_t)(3 * p) * N + xr];
            const float2 m00 = mtab[(0 * 3 * P + 3 * p) * C + c];
            const float2 m02 = mtab[(0 * 3 * P + 3 * p + 2) * C + c];
            const float2 m10 = mtab[(1 * 3 * P + 3 * p) * C + c];
            const float2 m12 = mtab[(1 * 3 * P + 3 * p + 2) * C + c];
            lre = fmaf(bb.x, m00.x + m02.x, fmaf(bb.y, m02.y - m00.y, lre));
            lim = fmaf(bb.x, m10.x + m12.x, fmaf(bb.y, m12.y - m10.y, lim));
          }
        } else {
          lre = -mre;
          lim = -mim;
          for (int pi = 0; pi < 3 * P; ++pi) {
            const float2 bb = st.basis[(size_t)pi * N + xr];
            const float2 m0 = mtab[(0 * 3 * P + pi) * C + c];
            const float2 m1 = mtab[(1 * 3 * P + pi) * C + c];
            lre = fmaf(bb.x, m0.x, fmaf(-bb.y, m0.y, lre));
            lim = fmaf(bb.x, m1.x, fmaf(-bb.y, m1.y, lim));
          }
        }
        const size_t o = (size_t)xo * st.n_out + yo;
        if (do_re) {
          const float val = img_scale_of(st, img_re) * (x[i].x + lre);
          float* dst = st.out + (size_t)img_re * plane + o;
          *dst = st.accumulate ? *dst + val : val;
        }
        if (do_im) {
          const float val = img_scale_of(st, img_im) * (x[i].y + lim);
          float* dst = st.out + (size_t)img_im * plane + o;
          *dst = st.accumulate ? *dst + val : val;
        }
      }
    }
    __syncthreads();  // mtab and buf reused by the next pair
  }
}

// Failure-path self-test of the bounded wait: one CTA expects bytes that no
// copy will ever deliver, so the wait must run out after `limit` polls,
// record kErrWaitTimeout and let the kernel finish.
__global__ void k_selftest_wait_timeout(long long limit, int* result) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_proxy_async();
  }
  __syncthreads();
  if (threadIdx.x == 0) mbar_arrive_expect_tx(&bar, 16);  // nothing will complete it
  const bool ok = mbar_wait_bounded(&bar, 0, limit);
  if (threadIdx.x == 0) *result = ok ? 0 : 1;
}
