// Power-of-two fast path of the spectral passes, included by spectral.cu
// inside namespace pt after the shared argument structs: the register FFT of
// fft_reg.cuh with bank-conflict-free swizzled layouts, and the frame
// synthesis with packed float32 pairs (fma.rn.f32x2 / mul / add on two
// layers at once).
#pragma once

template <int N>
struct RegCfg {
  static constexpr int T = N / 8;
  static constexpr int NV0 = (512 / T) < 1 ? 1 : (512 / T);
  static constexpr int NV = NV0 < N ? NV0 : N;  // transforms (rows) per CTA
  static constexpr int C = NV;                  // columns per CTA
  static constexpr int THREADS = NV * T;
};

// The paired column pass (generate / frames epilogue): 16 columns per CTA at
// N = 512 and 8 at N = 1024 (1024 threads: each CTA's twiddle and basis
// staging serves more columns, and a warp's output stores cover whole
// sectors); RegCfg's columns otherwise.
template <int N>
struct PairColCfg {
  static constexpr int C = N == 1024 ? 8 : (N == 512 ? 16 : RegCfg<N>::C);
  static constexpr int THREADS = C * RegCfg<N>::T;
};

__device__ __forceinline__ void load_tw(float2* stw, const float2* tw, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) stw[i] = tw[i];
}

// 64-bit read-only load with an L2 cache policy (createpolicy)
__device__ __forceinline__ float2 ld_evict_last(const float2* p, uint64_t pol) {
  float2 v;
  asm("ld.global.nc.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;"
               : "=f"(v.x), "=f"(v.y)
               : "l"(p), "l"(pol));
  return v;
}

// ------------------------------------------------------------------ packed f32x2
typedef unsigned long long f2x;
__device__ __forceinline__ f2x pk2(float lo, float hi) {
  f2x r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ void upk2(f2x v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f2x fma2(f2x a, f2x b, f2x c) {
  f2x d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ f2x mul2(f2x a, f2x b) {
  f2x d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
// both lanes negated (sign bits flipped)
__device__ __forceinline__ f2x neg2(f2x a) { return a ^ 0x8000000080000000ull; }
__device__ __forceinline__ f2x add2(f2x a, f2x b) {
  f2x d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}

// ------------------------------------------------------------------ rows
// plain complex input (pt_ifft2) or generate's coloured noise
template <int N>
__global__ void __launch_bounds__(RegCfg<N>::THREADS)
k_rows_reg(const float2* __restrict__ tw, const float2* __restrict__ in, int gen, GenRowArgs ga,
           float2* __restrict__ work) {
  constexpr int T = RegCfg<N>::T, NV = RegCfg<N>::NV;
  extern __shared__ float2 sm[];
  float2* stw = sm;
  const int v = threadIdx.x / T, j = threadIdx.x % T;
  const RowLayout s{sm + N + v * fft_padded(N)};
  const RowLayout s2{sm + N + (NV + v) * fft_padded(N)};  // second exchange vector
  // a column pass launched as a programmatic dependent may start its
  // prologue once every CTA of this grid is running (it waits for this
  // grid's completion before it reads any result)
  asm volatile("griddepcontrol.launch_dependents;");
  load_stage_tw<N>(stw, tw);
  const int kx = blockIdx.x * NV + v;
  const int img = blockIdx.y;
  if (gen) gen_coef_pair(ga, img);
  const bool ok = kx < N;
  float2 x[8];
  if (ok && gen && !ga.noise) {
    // one Philox call per element pair (ky, ky + N/2): elements i and i + 4
    const uint64_t row = (uint64_t)(ga.img0 + img) * N + kx;
    const uint64_t pol = l2_evict_last();  // the filter is re-read by every image
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      float2 lo, hi;
      philox_cnormal2(ga.seed, row * (N / 2) + j + T * i, ga.call, kDomainScreen, lo, hi);
      const float a0 = ld_keep(ga.amplitude + (size_t)kx * N + j + T * i, pol);
      const float a1 = ld_keep(ga.amplitude + (size_t)kx * N + j + T * (i + 4), pol);
      x[i] = make_float2(lo.x * a0, lo.y * a0);
      x[i + 4] = make_float2(hi.x * a1, hi.y * a1);
    }
  } else {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int ky = j + T * i;
      float2 val = make_float2(0.f, 0.f);
      if (ok) {
        if (gen) {
          const size_t e = ((size_t)(ga.img0 + img) * N + kx) * N + ky;
          const size_t plane = (size_t)ga.n_fft * N * N;
          const float amp = ga.amplitude[(size_t)kx * N + ky];
          val = make_float2(ga.noise[e] * amp, ga.noise[plane + e] * amp);
        } else {
          val = in[((size_t)img * N + kx) * N + ky];
        }
      }
      x[i] = val;
    }
  }
  __syncthreads();  // twiddles loaded
  reg_fft_db<N>(x, j, stw, s, s2);
  if (ok) {
#pragma unroll
    for (int i = 0; i < 8; ++i) work[((size_t)img * N + kx) * N + j + T * i] = x[i];
  }
}

// ------------------------------------------------------------------ columns
template <int N>
__global__ void __launch_bounds__(RegCfg<N>::THREADS)
k_plain_cols_reg(const float2* __restrict__ tw, const float2* __restrict__ work,
                 float2* __restrict__ out) {
  constexpr int T = RegCfg<N>::T, C = RegCfg<N>::C;
  extern __shared__ float2 sm[];
  float2* stw = sm;
  const int c = threadIdx.x % C, j = threadIdx.x / C;
  const ColLayout<C> s{sm + N + c};
  const ColLayout<C> s2{sm + N + N * C + c};  // second exchange buffer
  load_stage_tw<N>(stw, tw);
  const int y = blockIdx.x * C + c;
  const int img = blockIdx.y;
  const bool ok = y < N;
  float2 x[8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
    x[i] = ok ? work[((size_t)img * N + j + T * i) * N + y] : make_float2(0.f, 0.f);
  __syncthreads();
  reg_fft_db<N>(x, j, stw, s, s2);
  if (ok) {
#pragma unroll
    for (int i = 0; i < 8; ++i) out[((size_t)img * N + j + T * i) * N + y] = x[i];
  }
}

// Columns with the paired real epilogue (generate and frames). With the
// reference's symmetric subharmonic frequencies {-a, 0, +a} the bases obey
// b1 = 1 and b2 = conj(b0), so the low-order screen of one output is
//   K + sum_p (Re b0_p(x) U_p + Im b0_p(x) W_p),
//   K = sum_p Re m1_p - mean, U_p = Re(m0_p + m2_p), W_p = Im(m2_p - m0_p)
// with m_pi(y) = sum_j coef_pij b_pj(y): 2P FMAs per element and output.
template <int N>
__global__ void __launch_bounds__(PairColCfg<N>::THREADS)
k_pair_cols_reg(const float2* __restrict__ tw, const float2* __restrict__ work, int pair0,
                PairStore st) {
  constexpr int T = RegCfg<N>::T, C = PairColCfg<N>::C;
  extern __shared__ float2 sm[];
  float2* stw = sm;
  float2* buf = sm + N;             // 2 x N * C, column-interleaved exchange buffers
  float2* mtab = buf + 2 * N * C;   // (2, 3P, C) or (2, P, C) (U, W) + (2, C) (K, 0)
  const int c = threadIdx.x % C, j = threadIdx.x / C;
  const ColLayout<C> s{buf + c};
  const ColLayout<C> s2{buf + N * C + c};
  load_stage_tw<N>(stw, tw);
  // launched as a programmatic dependent of the row pass: everything below
  // reads the row pass's results (a no-op in an ordinary launch)
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const int y = blockIdx.x * C + c;
  const int pl = blockIdx.y;
  const int pair = pair0 + pl;
  const bool ok = y < N;
  const int img_re = pair * st.re_mul + st.re_add;
  const int img_im = pair * st.im_mul + st.im_add;
  const bool do_re = img_re < st.count, do_im = img_im < st.count;
  const int row_re = pl * st.crow_mul + st.crow_re, row_im = pl * st.crow_mul + st.crow_im;
  const int P = st.P;
  // m[o][p*3+i][c] = sum_j coef[o][p][i][j] basis[p][j][y]
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
  float2 x[8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
    x[i] = ok ? __ldcs(work + ((size_t)pl * N + j + T * i) * N + y) : make_float2(0.f, 0.f);
  __syncthreads();
  // per-column symmetric-basis constants: K (this thread's registers) and,
  // per level, (U_re, W_re, U_im, W_im) in a shared float4 table read once per
  // output element; the first basis row of each level is staged in shared
  // memory too when it fits (kColBasisMax float2)
  float4* utab = (float4*)(mtab + 2 * 3 * P * C);
  float2* sbasis = mtab + 8 * (P > 0 ? P : 1) * C;
  const bool sb = st.sym && P * N <= kColBasisMax;
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
    if (sb)
      for (int i = threadIdx.x; i < P * N; i += blockDim.x)
        sbasis[i] = __ldg(st.basis + (size_t)(3 * (i / N)) * N + (i % N));
  }
  __syncthreads();
  reg_fft_db<N>(x, j, stw, s, s2);
  if (!ok) return;
  const int yo = y - st.crop;
  if (yo < 0 || yo >= st.n_out) return;
  // the low-order screens of this column, level by level into the
  // transform's registers (x[i].x: screen img_re, x[i].y: screen img_im)
  if (st.sym) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      x[i].x += k0;
      x[i].y += k1;
    }
    if (sb) {
      for (int p = 0; p < P; ++p) {
        const float4 u = utab[p * C + c];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const float2 b = sbasis[p * N + j + T * i];
          x[i].x = fmaf(b.x, u.x, fmaf(b.y, u.y, x[i].x));
          x[i].y = fmaf(b.x, u.z, fmaf(b.y, u.w, x[i].y));
        }
      }
    } else {
      for (int p = 0; p < P; ++p) {
        const float4 u = utab[p * C + c];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const float2 b = __ldg(st.basis + (size_t)(3 * p) * N + j + T * i);
          x[i].x = fmaf(b.x, u.x, fmaf(b.y, u.y, x[i].x));
          x[i].y = fmaf(b.x, u.z, fmaf(b.y, u.w, x[i].y));
        }
      }
    }
  } else {
    const float mre = (P > 0 && do_re) ? st.mean[row_re] : 0.f;
    const float mim = (P > 0 && do_im) ? st.mean[row_im] : 0.f;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      x[i].x -= mre;
      x[i].y -= mim;
    }
    for (int pi = 0; pi < 3 * P; ++pi) {
      const float2 m0 = mtab[(0 * 3 * P + pi) * C + c];
      const float2 m1 = mtab[(1 * 3 * P + pi) * C + c];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const float2 b = st.basis[(size_t)pi * N + j + T * i];
        x[i].x = fmaf(b.x, m0.x, fmaf(-b.y, m0.y, x[i].x));
        x[i].y = fmaf(b.x, m1.x, fmaf(-b.y, m1.y, x[i].y));
      }
    }
  }
  const size_t plane = (size_t)st.n_out * st.n_out;
  const float sre = img_scale_of(st, img_re), sim = img_scale_of(st, img_im);
  float* ore = st.out + (size_t)(do_re ? img_re : 0) * plane + yo;
  float* oim = st.out + (size_t)(do_im ? img_im : 0) * plane + yo;
  const bool full = st.crop == 0 && st.n_out == N;  // every row of the column is kept
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int xo = j + T * i - st.crop;
    if (!full && (xo < 0 || xo >= st.n_out)) continue;
    const size_t o = (size_t)xo * st.n_out;
    if (st.accumulate) {
      if (do_re) ore[o] += sre * x[i].x;
      if (do_im) oim[o] += sim * x[i].y;
    } else {
      if (do_re) __stcs(ore + o, sre * x[i].x);
      if (do_im) __stcs(oim + o, sim * x[i].y);
    }
  }
}

// ------------------------------------------------------------------ uniform frames
// Fused synthesis + row transform. CTA = the row pair {kx, N - kx} of one
// anchor block of frames. Threads first own columns (E each) and advance the
// layer recurrence two layers per packed register pair, writing NV rows (NV/2
// frame pairs, two mirrored rows each) into shared memory; then NV teams
// transform those rows.
// Separable anchor phasors Q(kx, ky) = Px(kx) Py(ky) per layer: px0/py0
// (n_blocks, L, N) at each anchor block's first frame, rx/ry (L, N) per-frame
// ratios; filled by k_uniform_prep from the exact fixed-point phases.
struct UniformTables {
  const float2* px0;
  const float2* py0;
  const float2* rx;
  const float2* ry;
};

template <int LM, int N>
__global__ void __launch_bounds__(N < 512 ? N : 512)
k_frame_rows_uniform_reg(const float2* __restrict__ tw, const float2* __restrict__ spectra,
                         int L, int F, UniformTables ut, const float2* __restrict__ hn,
                         float2* __restrict__ work) {
  constexpr int THREADS = N < 512 ? N : 512;
  constexpr int E = N / THREADS;  // columns per thread
  constexpr int T = N / 8;
  constexpr int NV = THREADS / T;  // pair rows per batch
  constexpr int LP = (LM + 1) / 2;  // packed layer pairs
  extern __shared__ float2 sm[];
  float2* stw = sm;
  float2* rows = sm + N;  // NV * fft_padded(N), then NV exchange vectors
  // exact Hermitian parts at (kx, N/2) of this anchor block's frames, read
  // once here instead of by one thread inside the pair loop (which stalled
  // every batch's barrier on a global load)
  __shared__ float2 hcol[kAnchor];
  // the column pass after it is a programmatic dependent (it waits for this
  // grid's completion before reading the rows)
  asm volatile("griddepcontrol.launch_dependents;");
  load_stage_tw<N>(stw, tw);
  const int kx = blockIdx.x;
  const int fbeg = blockIdx.y * kAnchor;
  const int nkx = (N - kx) & (N - 1);
  const int nfr = min(kAnchor, F - fbeg);
  // row N/2 is the Nyquist row: every element comes from hn, no recurrence
  const bool nyq_row = kx == N / 2;
  // the layer spectra are re-read by every chunk: keep them in L2
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
  if (threadIdx.x < nfr) hcol[threadIdx.x] = hn[(size_t)(fbeg + threadIdx.x) * 2 * N + N + kx];
  // packed state: lanes (layer 2q, layer 2q+1). With one column per thread
  // -Ry is kept beside Ry so the complex step needs no separate negation
  // (two columns per thread would spill it).
  constexpr bool kNegR = E == 1;
  f2x Ax[E][LP], Ay[E][LP], Rx[E][LP], Ry[E][LP], NRy[kNegR ? E : 1][kNegR ? LP : 1];
#pragma unroll
  for (int e = 0; e < E; ++e) {
    const int ky = threadIdx.x + e * THREADS;
    const int nky = (N - ky) & (N - 1);
#pragma unroll
    for (int q = 0; q < LP; ++q) {
      float ax[2], ay[2], rx[2], ry[2];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int l = 2 * q + h;
        ax[h] = ay[h] = ry[h] = 0.f;
        rx[h] = 1.f;
        if (l < LM && l < L) {
          const float2 sa = ld_evict_last(spectra + ((size_t)l * N + kx) * N + ky, pol);
          const float2 sb = ld_evict_last(spectra + ((size_t)l * N + nkx) * N + nky, pol);
          const float2 sh = make_float2(0.5f * (sa.x + sb.x), 0.5f * (sa.y - sb.y));
          const size_t bl = (size_t)blockIdx.y * L + l;
          const float2 a = cmul(cmul(sh, ut.px0[bl * N + kx]), ut.py0[bl * N + ky]);
          const float2 r = cmul(ut.rx[(size_t)l * N + kx], ut.ry[(size_t)l * N + ky]);
          ax[h] = a.x;
          ay[h] = a.y;
          rx[h] = r.x;
          ry[h] = r.y;
        }
      }
      Ax[e][q] = pk2(ax[0], ax[1]);
      Ay[e][q] = pk2(ay[0], ay[1]);
      Rx[e][q] = pk2(rx[0], rx[1]);
      Ry[e][q] = pk2(ry[0], ry[1]);
      if constexpr (kNegR) NRy[e][q] = pk2(-ry[0], -ry[1]);
    }
  }
  // Hermitian symmetry H(-k) = conj H(k): this CTA synthesises row kx only and
  // also emits the mirrored row N - kx (columns reversed), so the recurrence
  // runs on half of the spectrum. Rows 0 and N/2 are their own mirrors.
  const bool self = (kx == 0) || nyq_row;
  constexpr int PB = NV / 2;  // frame pairs per transform batch (two rows each)
  const int npairs = (nfr + 1) / 2;
  const int v = threadIdx.x / T, j = threadIdx.x % T;
  __syncthreads();  // hcol
  for (int pb = 0; pb < npairs; pb += PB) {
    const int np = min(PB, npairs - pb);
    if (nyq_row) {
      // loads of PH pairs in flight together, then their stores
      constexpr int PH = E == 1 ? PB : 1;
      for (int p0 = 0; p0 < np; p0 += PH) {
        float2 hv[PH][2][E];
#pragma unroll
        for (int q = 0; q < PH; ++q) {
          const int p = p0 + q;
          const int fa = fbeg + 2 * (pb + p);
#pragma unroll
          for (int e = 0; e < E; ++e) {
            const int ky = threadIdx.x + e * THREADS;
            hv[q][0][e] = p < np ? hn[(size_t)fa * 2 * N + ky] : make_float2(0.f, 0.f);
            hv[q][1][e] = p < np && fa + 1 < fbeg + nfr ? hn[(size_t)(fa + 1) * 2 * N + ky]
                                                        : make_float2(0.f, 0.f);
          }
        }
#pragma unroll
        for (int q = 0; q < PH; ++q) {
          const int p = p0 + q;
          if (p >= np) break;
#pragma unroll
          for (int e = 0; e < E; ++e) {
            const int ky = threadIdx.x + e * THREADS;
            const RowLayout ra{rows + (2 * p) * fft_padded(N)};
            ra[ky] = make_float2(hv[q][0][e].x - hv[q][1][e].y, hv[q][0][e].y + hv[q][1][e].x);
          }
        }
      }
    }
    for (int p = 0; p < (nyq_row ? 0 : np); ++p) {
      const bool two = 2 * (pb + p) + 1 < nfr;
#pragma unroll
      for (int e = 0; e < E; ++e) {
        float2 h[2];
#pragma unroll
        for (int fr = 0; fr < 2; ++fr) {
          f2x hxa = 0ull, hya = 0ull, hxb = 0ull, hyb = 0ull;
          if (fr == 0 || two) {
#pragma unroll
            for (int q = 0; q < LP; ++q) {
              if (q & 1) {
                hxb = add2(hxb, Ax[e][q]);
                hyb = add2(hyb, Ay[e][q]);
              } else {
                hxa = add2(hxa, Ax[e][q]);
                hya = add2(hya, Ay[e][q]);
              }
              f2x nx;
              if constexpr (kNegR) nx = fma2(Ax[e][q], Rx[e][q], mul2(Ay[e][q], NRy[e][q]));
              else nx = fma2(Ax[e][q], Rx[e][q], neg2(mul2(Ay[e][q], Ry[e][q])));
              const f2x ny = fma2(Ax[e][q], Ry[e][q], mul2(Ay[e][q], Rx[e][q]));
              Ax[e][q] = nx;
              Ay[e][q] = ny;
            }
          }
          float a0, a1, b0, b1;
          upk2(add2(hxa, hxb), a0, a1);
          upk2(add2(hya, hyb), b0, b1);
          h[fr] = make_float2(a0 + a1, b0 + b1);
        }
        const int ky = threadIdx.x + e * THREADS;
        if (ky == N / 2) {
          h[0] = hcol[2 * (pb + p)];
          h[1] = two ? hcol[2 * (pb + p) + 1] : make_float2(0.f, 0.f);
        }
        const RowLayout ra{rows + (2 * p) * fft_padded(N)};
        ra[ky] = make_float2(h[0].x - h[1].y, h[0].y + h[1].x);
        if (!self) {
          // Y(-k) = conj H0(k) + i conj H1(k)
          const RowLayout rb{rows + (2 * p + 1) * fft_padded(N)};
          rb[(N - ky) & (N - 1)] = make_float2(h[0].x + h[1].y, h[1].x - h[0].y);
        }
      }
    }
    __syncthreads();
    const int pv = v >> 1, half = v & 1;  // team v: pair pv, row kx (0) or N - kx (1)
    const bool active = pv < np && (half == 0 || !self);
    float2 x[8];
    const RowLayout s{rows + v * fft_padded(N)};
    const RowLayout s2{rows + (NV + v) * fft_padded(N)};
    // the team's own row from here on: team barriers, not CTA barriers. The
    // first exchange goes to s2 (last read before this batch's first barrier),
    // so the gather from s needs no barrier of its own.
    const TeamSync team{1 + v, T};
    if (active) reg_gather8<N>(x, j, s);
    reg_fft_db<N>(x, j, stw, s2, s, team);
    if (active) {
      const int pair = fbeg / 2 + pb + pv;
      const int row = half ? nkx : kx;
#pragma unroll
      for (int i = 0; i < 8; ++i) work[((size_t)pair * N + row) * N + j + T * i] = x[i];
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------ uniform prep
// Everything the uniform frame kernels need besides the spectra, in one launch
// (block ranges select the role):
//   tables  — separable anchor/ratio phasors (as k_uniform_tables);
//   nyquist — exact Hermitian parts on the Nyquist cross, by the same
//             geometric recurrence from an exact anchor every kNyqGroup
//             frames (one thread per cross element and frame group);
//   coef    — per frame, shifted subharmonic coefficients summed over layers
//             and their grid mean (as k_frame_coef), with the shifts
//             s0 + f delta formed in FP64.
constexpr int kNyqGroup = 4;  // frames per Nyquist-cross thread (one exact anchor each)

struct UniformPrep {
  UniformParams up;
  double s0x[kMaxUniformLayers], s0y[kMaxUniformLayers];
  double dsx[kMaxUniformLayers], dsy[kMaxUniformLayers];
  const float2* spectra;
  const float2* sh_coef;  // (P, L, 3, 3)
  const double* sh_freq;  // (P, 3)
  const double* beta;     // (P, 3, 2)
  float2* px0;
  float2* py0;
  float2* rx;
  float2* ry;
  float2* hn;    // (F, 2N)
  float2* coef;  // (F, P, 9)
  float* mean;   // (F)
  int N, L, P, F, nb;
  int blocks_tab, blocks_nyq;
};

__global__ void __launch_bounds__(256) k_uniform_prep(UniformPrep a) {
  const int N = a.N, L = a.L;
  int blk = blockIdx.x;
  if (blk < a.blocks_tab) {  // ---- tables
    const int idx = blk * blockDim.x + threadIdx.x;
    if (idx >= (a.nb + 1) * L * N) return;
    const int k = idx % N, bl = idx / N;
    const int b = bl / L, l = bl % L;
    const uint64_t kk = (uint64_t)(int64_t)signed_freq(k, N);
    if (b < a.nb) {
      const uint64_t f0 = (uint64_t)b * kAnchor;
      a.px0[(size_t)bl * N + k] = phasor_from_fixed(kk * (a.up.ux0[l] + f0 * a.up.dux[l]));
      a.py0[(size_t)bl * N + k] = phasor_from_fixed(kk * (a.up.uy0[l] + f0 * a.up.duy[l]));
    } else {
      a.rx[(size_t)l * N + k] = phasor_from_fixed(kk * a.up.dux[l]);
      a.ry[(size_t)l * N + k] = phasor_from_fixed(kk * a.up.duy[l]);
    }
    return;
  }
  blk -= a.blocks_tab;
  if (blk < a.blocks_nyq) {  // ---- Nyquist cross, kNyqGroup frames per thread
    const int idx = blk * blockDim.x + threadIdx.x;
    const int groups = (a.F + kNyqGroup - 1) / kNyqGroup;
    if (idx >= 2 * N * groups) return;
    const int e = idx % (2 * N), gi = idx / (2 * N);
    const int kx = e < N ? N / 2 : e - N;
    const int ky = e < N ? e : N / 2;
    const int nkx = (N - kx) % N, nky = (N - ky) % N;
    const int ka = signed_freq(kx, N), kb = signed_freq(ky, N);
    const int na = signed_freq(nkx, N), nbf = signed_freq(nky, N);
    const int fbeg = gi * kNyqGroup;
    const int nfr = min(kNyqGroup, a.F - fbeg);
    float2 h[kNyqGroup];
#pragma unroll
    for (int f = 0; f < kNyqGroup; ++f) h[f] = make_float2(0.f, 0.f);
    // issue every layer's loads before any arithmetic (the loop below is a
    // dependent chain; serial loads would dominate this short kernel)
    float2 s1[kMaxUniformLayers], s2[kMaxUniformLayers];
#pragma unroll
    for (int l = 0; l < kMaxUniformLayers; ++l) {
      if (l < L) {
        s1[l] = a.spectra[((size_t)l * N + kx) * N + ky];
        s2[l] = a.spectra[((size_t)l * N + nkx) * N + nky];
      }
    }
#pragma unroll
    for (int l = 0; l < kMaxUniformLayers; ++l) {
      if (l >= L) break;
      const uint64_t ux = a.up.ux0[l] + (uint64_t)fbeg * a.up.dux[l];
      const uint64_t uy = a.up.uy0[l] + (uint64_t)fbeg * a.up.duy[l];
      float2 x1 = cmul(s1[l], phasor2(ka, kb, ux, uy));
      float2 x2 = cmul(s2[l], phasor2(na, nbf, ux, uy));
      const float2 r1 = phasor2(ka, kb, a.up.dux[l], a.up.duy[l]);
      const float2 r2 = phasor2(na, nbf, a.up.dux[l], a.up.duy[l]);
#pragma unroll
      for (int f = 0; f < kNyqGroup; ++f) {
        h[f].x += 0.5f * (x1.x + x2.x);
        h[f].y += 0.5f * (x1.y - x2.y);
        x1 = cmul(x1, r1);
        x2 = cmul(x2, r2);
      }
    }
#pragma unroll
    for (int f = 0; f < kNyqGroup; ++f)
      if (f < nfr) a.hn[(size_t)(fbeg + f) * 2 * N + e] = h[f];
    return;
  }
  blk -= a.blocks_nyq;
  // ---- subharmonic coefficients of frame blk
  __shared__ double part[8];
  const int f = blk;
  if (f >= a.F) return;
  const int t = threadIdx.x;
  double term = 0.0;
  if (t < a.P * 9) {
    const int p = t / 9, ij = t % 9, i = ij / 3, k = ij % 3;
    const double fi = a.sh_freq[p * 3 + i], fk = a.sh_freq[p * 3 + k];
    float2 acc = make_float2(0.f, 0.f);
    float2 cf[kMaxUniformLayers];
#pragma unroll
    for (int l = 0; l < kMaxUniformLayers; ++l)
      if (l < L) cf[l] = a.sh_coef[(((size_t)p * L + l) * 3 + i) * 3 + k];
#pragma unroll
    for (int l = 0; l < kMaxUniformLayers; ++l) {
      if (l >= L) break;
      const double sx = a.s0x[l] + (double)f * a.dsx[l];
      const double sy = a.s0y[l] + (double)f * a.dsy[l];
      double ph = fi * sx + fk * sy;
      ph -= floor(ph);
      float sn, cs;
      sincospif(2.0f * (float)ph, &sn, &cs);
      acc = cfma(cf[l], make_float2(cs, sn), acc);
    }
    a.coef[((size_t)f * a.P + p) * 9 + ij] = acc;
    const double bir = a.beta[(p * 3 + i) * 2], bii = a.beta[(p * 3 + i) * 2 + 1];
    const double bkr = a.beta[(p * 3 + k) * 2], bki = a.beta[(p * 3 + k) * 2 + 1];
    const double br = bir * bkr - bii * bki, bi = bir * bki + bii * bkr;
    term = (double)acc.x * br - (double)acc.y * bi;
  }
  for (int o = 16; o > 0; o >>= 1) term += __shfl_down_sync(0xffffffffu, term, o);
  if ((t & 31) == 0) part[t >> 5] = term;
  __syncthreads();
  if (t == 0) {
    double m = 0.0;
    for (int w = 0; w < (int)(blockDim.x + 31) / 32; ++w) m += part[w];
    a.mean[f] = (float)m;
  }
}
