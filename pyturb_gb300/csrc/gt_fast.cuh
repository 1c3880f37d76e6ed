// Register-resident transforms of length N = R1 * M (R1 odd, M a power of
// two; here R1 = 3, M = 64..512: N = 192, 384, 768, 1536) for generate,
// included by spectral.cu inside namespace pt after the power-of-two fast
// path.
//
// Good-Thomas (prime factor) decomposition: with gcd(R1, M) = 1 the
// N-point DFT is a 2-D R1 x M DFT without twiddles,
//   x[n1, n2] = x[(M n1 + R1 n2) mod N],
//   X[(k1 M u + k2 R1 v) mod N] = sum_n1 w_R1^(n1 k1) sum_n2 w_M^(n2 k2) x[n1, n2],
// u = M^-1 mod R1, v = R1^-1 mod M. A team of T = M / 8 threads holds R1
// sub-vectors of 8 elements per thread (n2 = j + T i), runs the R1 M-point
// register transforms in lockstep (fft_reg.cuh, one barrier per exchange for
// all of them), and the R1-point DFTs are then thread-local: thread j holds
// every n1 for its k2 = j + T i. Elements n2 and n2 + M / 2 of a sub-vector
// are n and n + N / 2, the two halves of one screen-noise Philox call.
#pragma once

// a^-1 mod m by search (a and m are small and coprime)
__host__ __device__ constexpr int gt_inv_mod(int a, int m) {
  for (int x = 1; x < m; ++x)
    if ((long long)a * x % m == 1) return x;
  return 0;
}

template <int R1, int M>
struct GtCfg {
  static constexpr int N = R1 * M;
  static constexpr int T = M / 8;
  static constexpr int H = N / 2;
  static constexpr int U = gt_inv_mod(M % R1, R1);  // M^-1 mod R1
  static constexpr int V = gt_inv_mod(R1 % M, M);   // R1^-1 mod M
  static_assert(U > 0 && V > 0 && (M & (M - 1)) == 0 && M >= 64, "R1, M coprime; M = 2^k >= 64");
  static constexpr int ROW_NV = 256 / T;        // rows (teams) per row-pass CTA
  static constexpr int ROW_THREADS = ROW_NV * T;
  static constexpr int C = M <= 128 ? 16 : 8;  // columns per column-pass CTA
  static constexpr int COL_THREADS = C * T;
  static constexpr int PAD = fft_padded(M);     // one padded row sub-vector
  // input position of (n1, n2) and output position of (k1, k2)
  static __device__ __forceinline__ int in_pos(int n1, int n2) { return (M * n1 + R1 * n2) % N; }
  static __device__ __forceinline__ int out_pos(int k1, int k2) {
    return (k1 * M * U + k2 * R1 * V) % N;
  }
};

template <int R1>
__device__ __forceinline__ void bfly_small(float2* v) {
  static_assert(R1 == 3 || R1 == 5, "R1 must be 3 or 5");
  if constexpr (R1 == 3) bfly3(v);
  else bfly5(v);
}

// R1-point inverse DFTs across the sub-vectors, for each of the thread's 8 k2
__device__ __forceinline__ void gt_combine3(float2 (&x)[3][8]) {
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    float2 v[3] = {x[0][i], x[1][i], x[2][i]};
    bfly_small<3>(v);
    x[0][i] = v[0];
    x[1][i] = v[1];
    x[2][i] = v[2];
  }
}

// ------------------------------------------------------------------ rows
// Generate (noise x filter) or plain complex rows; ROW_NV rows per CTA.
template <int R1, int M>
__global__ void __launch_bounds__(GtCfg<R1, M>::ROW_THREADS)
k_rows_gt(const float2* __restrict__ tw, const float2* __restrict__ in, int gen, GenRowArgs ga,
          float2* __restrict__ work) {
  using G = GtCfg<R1, M>;
  constexpr int N = G::N, T = G::T, NV = G::ROW_NV, PAD = G::PAD, H = G::H;
  extern __shared__ float2 sm[];
  float2* stw = sm;                                  // M
  const int v = threadIdx.x / T, j = threadIdx.x % T;
  float2* team = sm + M + (size_t)v * 2 * R1 * PAD;  // two sets of R1 padded sub-vectors
  RowLayout sa[R1], sb[R1];
#pragma unroll
  for (int q = 0; q < R1; ++q) {
    sa[q] = RowLayout{team + q * PAD};
    sb[q] = RowLayout{team + (R1 + q) * PAD};
  }
  load_stage_tw<M>(stw, tw, R1);  // exp(2 pi i k / M) = tw_N[R1 k]
  const int kx = blockIdx.x * NV + v;
  const int img = blockIdx.y;
  if (gen) gen_coef_pair(ga, img);
  const bool ok = kx < N;
  float2 x[R1][8];
#pragma unroll
  for (int n1 = 0; n1 < R1; ++n1) {
    if (ok && gen && !ga.noise) {
      const uint64_t row = (uint64_t)(ga.img0 + img) * N + kx;
      const uint64_t pol = l2_evict_last();  // the filter is re-read by every image
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int na = G::in_pos(n1, j + T * i);  // its partner is na + N/2 (mod N)
        const int nb = na < H ? na + H : na - H;
        float2 lo, hi;
        philox_cnormal2(ga.seed, row * H + (na < H ? na : nb), ga.call, kDomainScreen, lo, hi);
        const float2 za = na < H ? lo : hi, zb = na < H ? hi : lo;
        const float a0 = ld_keep(ga.amplitude + (size_t)kx * N + na, pol);
        const float a1 = ld_keep(ga.amplitude + (size_t)kx * N + nb, pol);
        x[n1][i] = make_float2(za.x * a0, za.y * a0);
        x[n1][i + 4] = make_float2(zb.x * a1, zb.y * a1);
      }
    } else {
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int n = G::in_pos(n1, j + T * i);
        float2 val = make_float2(0.f, 0.f);
        if (ok) {
          if (gen) {
            const size_t e = ((size_t)(ga.img0 + img) * N + kx) * N + n;
            const size_t plane = (size_t)ga.n_fft * N * N;
            const float amp = ga.amplitude[(size_t)kx * N + n];
            val = make_float2(ga.noise[e] * amp, ga.noise[plane + e] * amp);
          } else {
            val = in[((size_t)img * N + kx) * N + n];
          }
        }
        x[n1][i] = val;
      }
    }
  }
  __syncthreads();  // twiddles
  reg_fft_multi<M, R1>(x, j, stw, sa, sb);
  gt_combine3(x);
  // outputs through the set the last exchange did not read (its barrier
  // ordered every earlier read of it), then coalesced stores
  constexpr bool last_in_a = (Pow2Plan<M>::stages - 1) % 2 == 1;  // exchanges alternate a, b, a, ...
  float2* rowbuf = team + (last_in_a ? R1 * PAD : 0);
#pragma unroll
  for (int k1 = 0; k1 < R1; ++k1)
#pragma unroll
    for (int i = 0; i < 8; ++i) rowbuf[G::out_pos(k1, j + T * i)] = x[k1][i];
  __syncthreads();
  if (ok) {
#pragma unroll
    for (int e = j; e < N; e += T) work[((size_t)img * N + kx) * N + e] = rowbuf[e];
  }
}

// ------------------------------------------------------------------ columns
// The paired real epilogue of k_pair_cols_reg (subharmonic low-order screens,
// mean, crop, scale) on the Good-Thomas column transform; C columns per CTA.
template <int R1, int M>
__global__ void __launch_bounds__(GtCfg<R1, M>::COL_THREADS)
k_pair_cols_gt(const float2* __restrict__ tw, const float2* __restrict__ work, int pair0,
               PairStore st) {
  using G = GtCfg<R1, M>;
  constexpr int N = G::N, T = G::T, C = G::C;
  extern __shared__ float2 sm[];
  float2* stw = sm;                       // M
  float2* buf = sm + M;                   // 2 R1 sub-vectors of M x C, column-interleaved
  float2* mtab = buf + 2 * R1 * M * C;    // (2, 3P, C), then U/W (P, C) float4, staged basis
  const int c = threadIdx.x % C, j = threadIdx.x / C;
  ColLayout<C> sa[R1], sb[R1];
#pragma unroll
  for (int q = 0; q < R1; ++q) {
    sa[q] = ColLayout<C>{buf + (size_t)q * M * C + c};
    sb[q] = ColLayout<C>{buf + (size_t)(R1 + q) * M * C + c};
  }
  load_stage_tw<M>(stw, tw, R1);
  const int y = blockIdx.x * C + c;
  const int pl = blockIdx.y;
  const int pair = pair0 + pl;
  const bool ok = y < N;
  const int img_re = pair * st.re_mul + st.re_add;
  const int img_im = pair * st.im_mul + st.im_add;
  const bool do_re = img_re < st.count, do_im = img_im < st.count;
  const int row_re = pl * st.crow_mul + st.crow_re, row_im = pl * st.crow_mul + st.crow_im;
  const int P = st.P;
  for (int i = threadIdx.x; i < 2 * 3 * P * C; i += blockDim.x) {
    const int cc = i % C;
    const int pi = (i / C) % (3 * P);
    const int o = i / (C * 3 * P);
    const bool take = o == 0 ? do_re : do_im;
    const int row = o == 0 ? row_re : row_im;
    const int yy = blockIdx.x * C + cc;
    float2 m = make_float2(0.f, 0.f);
    if (take && yy < N) {
      const int p = pi / 3, ii = pi % 3;
      const float2* cf = st.coef + ((size_t)row * P + p) * 9 + ii * 3;
#pragma unroll
      for (int jj = 0; jj < 3; ++jj) m = cfma(cf[jj], st.basis[((size_t)p * 3 + jj) * N + yy], m);
    }
    mtab[i] = m;
  }
  float2 x[R1][8];
#pragma unroll
  for (int n1 = 0; n1 < R1; ++n1)
#pragma unroll
    for (int i = 0; i < 8; ++i)
      x[n1][i] = ok ? __ldcs(work + ((size_t)pl * N + G::in_pos(n1, j + T * i)) * N + y)
                    : make_float2(0.f, 0.f);
  __syncthreads();
  float4* utab = (float4*)(mtab + 2 * 3 * P * C);  // even offset: M C and 6 P C are even
  float2* sbasis = mtab + 8 * (P > 0 ? P : 1) * C;
  const bool sb_ok = st.sym && P * N <= kColBasisMax;
  float k0 = 0.f, k1 = 0.f;
  if (st.sym) {
    for (int p = 0; p < P; ++p) {
      k0 += mtab[(0 * 3 * P + 3 * p + 1) * C + c].x;
      k1 += mtab[(1 * 3 * P + 3 * p + 1) * C + c].x;
    }
    if (P > 0 && do_re) k0 -= st.mean[row_re];
    if (P > 0 && do_im) k1 -= st.mean[row_im];
    for (int i = threadIdx.x; i < P * C; i += blockDim.x) {
      const int p = i / C, cc = i % C;
      const float2 m00 = mtab[(0 * 3 * P + 3 * p) * C + cc], m02 = mtab[(0 * 3 * P + 3 * p + 2) * C + cc];
      const float2 m10 = mtab[(1 * 3 * P + 3 * p) * C + cc], m12 = mtab[(1 * 3 * P + 3 * p + 2) * C + cc];
      utab[i] = make_float4(m00.x + m02.x, m02.y - m00.y, m10.x + m12.x, m12.y - m10.y);
    }
    if (sb_ok)
      for (int i = threadIdx.x; i < P * N; i += blockDim.x)
        sbasis[i] = __ldg(st.basis + (size_t)(3 * (i / N)) * N + (i % N));
  }
  __syncthreads();
  reg_fft_multi<M, R1>(x, j, stw, sa, sb);
  gt_combine3(x);
  if (!ok) return;
  const int yo = y - st.crop;
  if (yo < 0 || yo >= st.n_out) return;
  const float mre = (P > 0 && do_re) ? st.mean[row_re] : 0.f;
  const float mim = (P > 0 && do_im) ? st.mean[row_im] : 0.f;
  const float sre = img_scale_of(st, img_re), sim = img_scale_of(st, img_im);
  const size_t plane = (size_t)st.n_out * st.n_out;
  float* ore = st.out + (size_t)(do_re ? img_re : 0) * plane + yo;
  float* oim = st.out + (size_t)(do_im ? img_im : 0) * plane + yo;
#pragma unroll
  for (int k1i = 0; k1i < R1; ++k1i)
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int xr = G::out_pos(k1i, j + T * i);
      const int xo = xr - st.crop;
      if (xo < 0 || xo >= st.n_out) continue;
      float lre, lim;
      if (st.sym) {
        lre = k0;
        lim = k1;
        for (int p = 0; p < P; ++p) {
          const float2 b = sb_ok ? sbasis[p * N + xr] : __ldg(st.basis + (size_t)(3 * p) * N + xr);
          const float4 u = utab[p * C + c];
          lre = fmaf(b.x, u.x, fmaf(b.y, u.y, lre));
          lim = fmaf(b.x, u.z, fmaf(b.y, u.w, lim));
        }
      } else {
        lre = -mre;
        lim = -mim;
        for (int pi = 0; pi < 3 * P; ++pi) {
          const float2 b = st.basis[(size_t)pi * N + xr];
          const float2 m0 = mtab[(0 * 3 * P + pi) * C + c];
          const float2 m1 = mtab[(1 * 3 * P + pi) * C + c];
          lre = fmaf(b.x, m0.x, fmaf(-b.y, m0.y, lre));
          lim = fmaf(b.x, m1.x, fmaf(-b.y, m1.y, lim));
        }
      }
      const size_t o = (size_t)xo * st.n_out;
      if (st.accumulate) {
        if (do_re) ore[o] += sre * (x[k1i][i].x + lre);
        if (do_im) oim[o] += sim * (x[k1i][i].y + lim);
      } else {
        if (do_re) __stcs(ore + o, sre * (x[k1i][i].x + lre));
        if (do_im) __stcs(oim + o, sim * (x[k1i][i].y + lim));
      }
    }
}
