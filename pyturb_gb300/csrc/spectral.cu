// Spectral synthesis on the GB300: PhaseScreen.generate, the frozen-flow
// frame readout of the spectral engine, per-layer LGS screens, the LGS cone
// zoom and spectral boiling.
//
// A 2-D inverse transform is two shared-memory passes:
//   pass 1 (rows, axis 1): a producer writes one complex row into shared
//     memory (coloured noise, or the phasor-weighted layer sum), the row is
//     transformed and written to the workspace;
//   pass 2 (columns, axis 0): tiles of C columns are transformed and the
//     epilogue writes the real/imaginary parts as two real screens with the
//     subharmonic low-frequency sum added, cropped and scaled.
// Two real outputs share one complex transform: generate() uses the
// reference's own Re/Im pairing, frames are paired through their
// Hermitian parts, H = (X(k) + conj X(-k)) / 2, so Re ifft2(X1) + i Re
// ifft2(X2) = ifft2(H1 + i H2).
#include <cuda.h>  // CUtensorMap (types only; the encoder comes from the runtime's entry point)
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "fft.cuh"
#include "fft_reg.cuh"

namespace pt {
uint64_t* launch_counter();
}

struct pt_grid {
  int ns;
  double dx;
  int P;
  pt::FftDesc desc;
  float2* tw;       // (ns) exp(+2 pi i k / ns)
  float2* basis;    // (P, 3, ns) exp(2 pi i f_p (x - ns/2) dx)
  double* sh_freq;  // (P, 3)
  double* beta;     // (P, 3, 2) grid mean of each basis row
  int sym;          // every level's frequencies are {-a, 0, +a}
  int cols_variant; // power-of-two column pass: 0 register-fed, 1 TMA-fed
  float2* blu;      // Bluestein tables of desc (chirp, bhat, twM), or NULL
};

namespace pt {

constexpr int kMaxLevels = 16;
constexpr int kThreads = 256;
// Largest P * ns (float2) of first basis rows the column kernels stage in
// shared memory for the subharmonic epilogue.
constexpr int kColBasisMax = 4096;

static inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Number of complex ns x ns images one internal pass batches.
static inline int image_chunk(int ns) {
  size_t per = (size_t)ns * ns * sizeof(float2);
  size_t c = (size_t)(64u << 20) / per;
  return (int)std::max<size_t>(1, std::min<size_t>(32, c));
}
// Transforms per chunk of generate / ifft2: up to 256 as long as the row-pass
// intermediate of a chunk stays within 64 MB (L2-resident between the passes),
// so small screens run as a few large launches.
static inline int gen_chunk(int ns) {
  size_t per = (size_t)ns * ns * sizeof(float2);
  size_t c = (size_t)(64u << 20) / per;
  return (int)std::max<size_t>(1, std::min<size_t>(256, c));
}
// Rows per CTA of the shared-memory row pass: about 2048 elements, so every
// stage gives most of the 256 threads a butterfly.
// rows / columns a CTA of the shared-memory passes transforms, from the
// buffer length (fft_buf_len: M for a Bluestein grid)
static inline int rows_per_cta(int nb) { return std::max(1, std::min(16, 2048 / nb)); }
static inline int cols_per_cta(int nb) { return std::max(1, std::min(16, 4096 / nb)); }

static inline void count_launch(int k = 1) {
  __atomic_add_fetch(launch_counter(), (uint64_t)k, __ATOMIC_RELAXED);
}

// fftfreq index: k for k < (n+1)/2, else k - n
__device__ __forceinline__ int signed_freq(int k, int n) { return k < (n + 1) / 2 ? k : k - n; }

// ---------------------------------------------------------------- workspace
struct SpecWork {
  float2* img;     // (chunk, ns, ns)
  float2* coef;    // (2 chunk, P, 9)
  float* mean;     // (2 chunk)
  float2* px;      // (2 chunk, J, ns)
  float2* py;      // (2 chunk, J, ns)
  float2* hn;      // (2 chunk, 2 ns) Hermitian parts on the Nyquist cross
  size_t bytes;
};

static SpecWork carve(const pt_grid* g, int L, void* base) {
  const int ns = g->ns, ch = image_chunk(ns), gch = gen_chunk(ns), P = std::max(1, g->P);
  const int F = 2 * ch;
  const int J = std::max(1, L);
  size_t off = 0;
  SpecWork w{};
  char* b = (char*)base;
  auto take = [&](size_t bytes) {
    char* p = b ? b + off : nullptr;
    off += align256(bytes);
    return p;
  };
  w.img = (float2*)take((size_t)std::max(ch, gch) * ns * ns * sizeof(float2));
  w.coef = (float2*)take((size_t)2 * std::max(ch, gch) * P * 9 * sizeof(float2));
  w.mean = (float*)take((size_t)2 * std::max(ch, gch) * sizeof(float));
  w.px = (float2*)take((size_t)F * J * ns * sizeof(float2));
  w.py = (float2*)take((size_t)F * J * ns * sizeof(float2));
  w.hn = (float2*)take((size_t)F * 2 * ns * sizeof(float2));
  w.bytes = off;
  return w;
}

// ================================================================ pass 1 producers
// Generate: X[kx, ky] = (n0 + i n1) * amplitude[kx, ky]
struct GenRowArgs {
  const float* amplitude;
  const float* noise;  // (2, n_fft, ns, ns) or null
  int n_fft;
  int img0;            // first FFT index of this chunk
  uint64_t seed, call;
  // subharmonic coefficients of the chunk's screens (P = 0: none), made by
  // warps 0 and 1 of each pair's first row CTA
  const float* sh_amp;    // (P, 9)
  const float* sh_noise;  // (P, 2, count, 3, 3) or null
  const double* beta;     // (P, 3, 2) grid means of the basis rows
  float2* coef;           // (2 ch, P, 9)
  float* mean;            // (2 ch)
  int count, ch, P;
};

// coef[slot][p][ij] = (n0 + i n1) * sh_amp[p][ij] of screen gc and
// mean[slot] = Re sum_p,ij coef beta_i beta_j: one warp, a lane per (level,
// 3x3 cell), the mean reduced by shuffles.
__device__ __forceinline__ void gen_coef_warp(const GenRowArgs& a, int gc, int slot, int lane) {
  double mr = 0.0;
  for (int q = lane; q < a.P * 9; q += 32) {
    const int p = q / 9, ij = q - 9 * p;
    float2 z;
    if (a.sh_noise) {
      // layout (P, 2, count, 3, 3)
      const size_t base = (size_t)p * 2 * a.count * 9;
      z = make_float2(a.sh_noise[base + (size_t)gc * 9 + ij],
                      a.sh_noise[base + (size_t)a.count * 9 + (size_t)gc * 9 + ij]);
    } else {
      z = philox_cnormal(a.seed, ((uint64_t)gc * kMaxLevels + p) * 9 + ij, a.call, kDomainSub);
    }
    const float amp = a.sh_amp[q];
    const float2 cf = make_float2(z.x * amp, z.y * amp);
    a.coef[(size_t)slot * a.P * 9 + q] = cf;
    const int i = ij / 3, j = ij % 3;
    const double bir = a.beta[(p * 3 + i) * 2], bii = a.beta[(p * 3 + i) * 2 + 1];
    const double bjr = a.beta[(p * 3 + j) * 2], bji = a.beta[(p * 3 + j) * 2 + 1];
    const double br = bir * bjr - bii * bji, bi = bir * bji + bii * bjr;
    mr += (double)cf.x * br - (double)cf.y * bi;
  }
  for (int o = 16; o > 0; o >>= 1) mr += __shfl_xor_sync(0xffffffffu, mr, o);
  if (lane == 0) a.mean[slot] = (float)mr;
}

// In the first row CTA (blockIdx.x == 0) of transform pair `img` of the
// chunk, warp 0 makes the coefficients of its real-part screen b0 + img
// (slot img) and warp 1 those of its imaginary-part screen n_fft + b0 + img
// (slot ch + img), when they exist. No barrier is involved.
__device__ __forceinline__ void gen_coef_pair(const GenRowArgs& a, int img) {
  if (a.P <= 0 || blockIdx.x != 0 || threadIdx.x >= 64) return;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gc = (w == 0 ? 0 : a.n_fft) + a.img0 + img;
  if (gc >= a.count) return;  // warp-uniform
  gen_coef_warp(a, gc, w == 0 ? img : a.ch + img, lane);
}

// Plain complex rows (pt_ifft2) and generate rows share this kernel: `gen`
// selects the producer. rpc rows per CTA, one transform per row.
__global__ void __launch_bounds__(kThreads)
k_rows(FftDesc d, const float2* __restrict__ tw, int rpc, const float2* __restrict__ in,
       int gen, GenRowArgs ga, float2* __restrict__ work) {
  extern __shared__ float2 sm[];
  const int ns = d.n;
  const int row0 = blockIdx.x * rpc;
  const int img = blockIdx.y;  // image within this chunk
  if (gen) gen_coef_pair(ga, img);
  const int vs = fft_buf_len(d) + 1;
  float2* bufA = sm;
  float2* bufB = sm + rpc * vs;
  float2* stw = sm + 2 * rpc * vs;
  for (int i = threadIdx.x; i < ns; i += blockDim.x) stw[i] = tw[i];
  for (int i = threadIdx.x; i < rpc * ns; i += blockDim.x) {
    const int r = i / ns, ky = i % ns;
    const int kx = row0 + r;
    float2 v = make_float2(0.f, 0.f);
    if (kx < ns) {
      if (gen) {
        const size_t e = ((size_t)(ga.img0 + img) * ns + kx) * ns + ky;
        float2 z;
        if (ga.noise) {
          const size_t plane = (size_t)ga.n_fft * ns * ns;
          z = make_float2(ga.noise[e], ga.noise[plane + e]);
        } else {
          z = screen_normal(ga.seed, (uint64_t)(ga.img0 + img) * ns + kx, ky, ns, ga.call);
        }
        const float amp = ga.amplitude[(size_t)kx * ns + ky];
        v = make_float2(z.x * amp, z.y * amp);
      } else {
        v = in[((size_t)img * ns + kx) * ns + ky];
      }
    }
    bufA[r * vs + ky] = v;
  }
  __syncthreads();
  float2* res = fft_smem(bufA, bufB, d, stw, rpc, vs, 1, false);
  for (int i = threadIdx.x; i < rpc * ns; i += blockDim.x) {
    const int r = i / ns, ky = i % ns;
    const int kx = row0 + r;
    if (kx < ns) work[((size_t)img * ns + kx) * ns + ky] = res[r * vs + ky];
  }
}

// Frames: CTA = (row pair {kx, ns-kx}, frame pair). Each frame's row is the
// phasor-weighted layer sum X_f[kx, ky] = sum_j S_l[kx,ky] Px[f,j,kx] Py[f,j,ky]
// (l = j, or l = the frame's own layer in per-layer mode); the pair is then
// folded through its Hermitian parts into one complex row per kx.
struct FrameRowArgs {
  const float2* spectra;  // (L, ns, ns)
  const float2* px;       // (F, J, ns) for this chunk
  const float2* py;       // (F, J, ns)
  int J, F;               // J = terms per frame (L, or 1 per-layer); F frames in chunk
  int frame0;             // global index of the chunk's first frame (per-layer: its layer)
  int per_layer;
};

__global__ void __launch_bounds__(kThreads)
k_frame_rows(FftDesc d, const float2* __restrict__ tw, FrameRowArgs a, float2* __restrict__ work) {
  extern __shared__ float2 sm[];
  const int ns = d.n;
  const int rp = blockIdx.x;  // 0 .. ns/2
  const int pair = blockIdx.y;
  const int kxa = rp, kxb = (ns - rp) % ns;
  const int nrows = (kxa == kxb) ? 1 : 2;
  const int vs = fft_buf_len(d) + 1;
  // X rows: [frame 0 row a, frame 0 row b, frame 1 row a, frame 1 row b]
  float2* X = sm;                // 4 * vs
  float2* bufA = sm + 4 * vs;    // 2 * vs
  float2* bufB = bufA + 2 * vs;  // 2 * vs
  float2* stw = bufB + 2 * vs;   // ns
  for (int i = threadIdx.x; i < ns; i += blockDim.x) stw[i] = tw[i];
  const int f0 = 2 * pair, f1 = 2 * pair + 1;
  const bool has1 = f1 < a.F;
  for (int i = threadIdx.x; i < nrows * ns; i += blockDim.x) {
    const int r = i / ns, ky = i % ns;
    const int kx = r == 0 ? kxa : kxb;
    float2 acc0 = make_float2(0.f, 0.f), acc1 = make_float2(0.f, 0.f);
    for (int j = 0; j < a.J; ++j) {
      const int l0 = a.per_layer ? (a.frame0 + f0) : j;
      const float2 s0 = a.spectra[((size_t)l0 * ns + kx) * ns + ky];
      const size_t t0 = ((size_t)f0 * a.J + j) * ns;
      acc0 = cfma(s0, cmul(a.px[t0 + kx], a.py[t0 + ky]), acc0);
      if (has1) {
        const float2 s1 =
            a.per_layer ? a.spectra[((size_t)(a.frame0 + f1) * ns + kx) * ns + ky] : s0;
        const size_t t1 = ((size_t)f1 * a.J + j) * ns;
        acc1 = cfma(s1, cmul(a.px[t1 + kx], a.py[t1 + ky]), acc1);
      }
    }
    X[(0 * 2 + r) * vs + ky] = acc0;
    X[(1 * 2 + r) * vs + ky] = acc1;
  }
  __syncthreads();
  // Y[kx] = H0[kx] + i H1[kx], H_f[kx,ky] = (X_f[kx,ky] + conj X_f[-kx,-ky]) / 2
  for (int i = threadIdx.x; i < nrows * ns; i += blockDim.x) {
    const int r = i / ns, ky = i % ns;
    const int ro = (nrows == 1) ? 0 : 1 - r;  // row holding -kx
    const int kyn = (ns - ky) % ns;
    const float2 a0 = X[(0 * 2 + r) * vs + ky], b0 = X[(0 * 2 + ro) * vs + kyn];
    const float2 a1 = X[(1 * 2 + r) * vs + ky], b1 = X[(1 * 2 + ro) * vs + kyn];
    const float2 h0 = make_float2(0.5f * (a0.x + b0.x), 0.5f * (a0.y - b0.y));
    const float2 h1 = make_float2(0.5f * (a1.x + b1.x), 0.5f * (a1.y - b1.y));
    bufA[r * vs + ky] = make_float2(h0.x - h1.y, h0.y + h1.x);
  }
  __syncthreads();
  float2* res = fft_smem(bufA, bufB, d, stw, nrows, vs, 1, false);
  for (int i = threadIdx.x; i < nrows * ns; i += blockDim.x) {
    const int r = i / ns, ky = i % ns;
    const int kx = r == 0 ? kxa : kxb;
    work[((size_t)pair * ns + kx) * ns + ky] = res[r * vs + ky];
  }
}

// Uniformly spaced frames (shift of frame f, layer l = s0_l + f delta_l):
// only the Hermitian part Sh_l = (S_l(k) + conj S_l(-k)) / 2 of each layer
// contributes to a real frame, and its phasor is a geometric sequence in f,
//   H_f(k) = sum_l Sh_l(k) Q_l(k) R_l(k)^f,
// so each thread keeps A_l = Sh_l Q_l R_l^f and R_l in registers and advances
// a frame with one complex multiply-add per layer — no phasor tables. Anchors
// (exact 64-bit fixed-point phases, u0 + f du mod 1) are re-taken every
// kAnchor frames, bounding the float32 drift of the recurrence.
// CTA = one row kx x kFramesPerCta frames; thread = one column ky; frame
// pairs are packed as Y = H_f0 + i H_f1 and kPairsPerFft rows are transformed
// together.
constexpr int kMaxUniformLayers = 16;
constexpr int kAnchor = 64;
constexpr int kPairsPerFft = 4;

struct UniformParams {
  uint64_t ux0[kMaxUniformLayers], uy0[kMaxUniformLayers];  // frac(s0 df) of frame 0
  uint64_t dux[kMaxUniformLayers], duy[kMaxUniformLayers];  // frac(delta df) per frame
};

__device__ __forceinline__ float2 phasor2(int kxs, int kys, uint64_t ux, uint64_t uy) {
  return phasor_from_fixed((uint64_t)(int64_t)kxs * ux + (uint64_t)(int64_t)kys * uy);
}

// The phasor of the Nyquist index ns/2 is exp(-i pi ns u) on both k and -k
// (fftfreq gives -ns/2 for it), so Q(-k) = conj Q(k) fails on the Nyquist
// row and column and the shortcut through Sh does not hold there. This kernel
// forms H_f(k) = (X_f(k) + conj X_f(-k)) / 2 exactly on that cross (element e:
// e < ns is (ns/2, e), else (e - ns, ns/2)) for every frame of the chunk.
__global__ void k_nyquist_h(int ns, const float2* __restrict__ spectra, int L, int F,
                            UniformParams up, float2* __restrict__ hn) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int f = blockIdx.y;
  if (e >= 2 * ns || f >= F) return;
  const int kx = e < ns ? ns / 2 : e - ns;
  const int ky = e < ns ? e : ns / 2;
  const int nkx = (ns - kx) % ns, nky = (ns - ky) % ns;
  const int a = signed_freq(kx, ns), b = signed_freq(ky, ns);
  const int na = signed_freq(nkx, ns), nb = signed_freq(nky, ns);
  float2 h = make_float2(0.f, 0.f);
  for (int l = 0; l < L; ++l) {
    const uint64_t ux = up.ux0[l] + (uint64_t)f * up.dux[l];
    const uint64_t uy = up.uy0[l] + (uint64_t)f * up.duy[l];
    const float2 x = cmul(spectra[((size_t)l * ns + kx) * ns + ky], phasor2(a, b, ux, uy));
    const float2 y = cmul(spectra[((size_t)l * ns + nkx) * ns + nky], phasor2(na, nb, ux, uy));
    h = cadd(h, make_float2(0.5f * (x.x + y.x), 0.5f * (x.y - y.y)));
  }
  hn[(size_t)f * 2 * ns + e] = h;
}

template <int LM, int E>
__global__ void __launch_bounds__(512)
k_frame_rows_uniform(FftDesc d, const float2* __restrict__ tw,
                     const float2* __restrict__ spectra, int L, int F, UniformParams up,
                     const float2* __restrict__ hn, float2* __restrict__ work) {
  extern __shared__ float2 sm[];
  const int ns = d.n;
  const int kx = blockIdx.x;
  const int fbeg = blockIdx.y * kAnchor;  // this CTA's frames [fbeg, fbeg + kAnchor)
  const int vs = fft_buf_len(d) + 1;
  float2* bufA = sm;
  float2* bufB = sm + kPairsPerFft * vs;
  float2* stw = sm + 2 * kPairsPerFft * vs;
  for (int i = threadIdx.x; i < ns; i += blockDim.x) stw[i] = tw[i];
  const int kxs = signed_freq(kx, ns), nkx = (ns - kx) % ns;
  float2 A[E][LM], R[E][LM];
#pragma unroll
  for (int e = 0; e < E; ++e) {
    const int ky = threadIdx.x + e * blockDim.x;
    const bool live = ky < ns;
    const int kys = live ? signed_freq(ky, ns) : 0, nky = live ? (ns - ky) % ns : 0;
#pragma unroll
    for (int l = 0; l < LM; ++l) {
      A[e][l] = make_float2(0.f, 0.f);
      R[e][l] = make_float2(1.f, 0.f);
      if (l < L && live) {
        const float2 s = spectra[((size_t)l * ns + kx) * ns + ky];
        const float2 t = spectra[((size_t)l * ns + nkx) * ns + nky];
        const float2 sh = make_float2(0.5f * (s.x + t.x), 0.5f * (s.y - t.y));
        A[e][l] = cmul(sh, phasor2(kxs, kys, up.ux0[l] + (uint64_t)fbeg * up.dux[l],
                                   up.uy0[l] + (uint64_t)fbeg * up.duy[l]));
        R[e][l] = phasor2(kxs, kys, up.dux[l], up.duy[l]);
      }
    }
  }
  const int nfr = min(kAnchor, F - fbeg);
  const int npairs = (nfr + 1) / 2;
  for (int pb = 0; pb < npairs; pb += kPairsPerFft) {
    const int np = min(kPairsPerFft, npairs - pb);
    for (int p = 0; p < np; ++p) {
      const bool two = 2 * (pb + p) + 1 < nfr;
#pragma unroll
      for (int e = 0; e < E; ++e) {
        float2 h0a = make_float2(0.f, 0.f), h0b = h0a, h1a = h0a, h1b = h0a;
#pragma unroll
        for (int l = 0; l < LM; ++l) {
          if (l & 1) h0b = cadd(h0b, A[e][l]);
          else h0a = cadd(h0a, A[e][l]);
          A[e][l] = cmul(A[e][l], R[e][l]);
        }
        if (two) {
#pragma unroll
          for (int l = 0; l < LM; ++l) {
            if (l & 1) h1b = cadd(h1b, A[e][l]);
            else h1a = cadd(h1a, A[e][l]);
            A[e][l] = cmul(A[e][l], R[e][l]);
          }
        }
        float2 h0 = cadd(h0a, h0b), h1 = cadd(h1a, h1b);
        const int ky = threadIdx.x + e * blockDim.x;
        const bool even = (ns & 1) == 0;
        if (even && (kx == ns / 2 || ky == ns / 2) && ky < ns) {
          const int el = kx == ns / 2 ? ky : ns + kx;
          const int fa = fbeg + 2 * (pb + p);
          h0 = hn[(size_t)fa * 2 * ns + el];
          h1 = two ? hn[(size_t)(fa + 1) * 2 * ns + el] : make_float2(0.f, 0.f);
        }
        if (ky < ns) bufA[p * vs + ky] = make_float2(h0.x - h1.y, h0.y + h1.x);
      }
    }
    __syncthreads();
    float2* res = fft_smem(bufA, bufB, d, stw, np, vs, 1, false);
    for (int i = threadIdx.x; i < np * ns; i += blockDim.x) {
      const int p = i / ns, c = i % ns;
      const int pair = fbeg / 2 + pb + p;
      work[((size_t)pair * ns + kx) * ns + c] = res[p * vs + c];
    }
    __syncthreads();
  }
}

// ================================================================ pass 2
// Column transform of a tile of C columns plus the paired real epilogue:
// Re -> output image (pair*re_mul + re_add), Im -> (pair*im_mul + im_add),
// each plus its subharmonic sum (coefficient row pl*crow_mul + crow_add_*)
// minus that sum's grid mean, cropped and scaled.
struct PairStore {
  float* out;
  int n_out, crop;
  float scale;
  int accumulate;
  int count;  // valid output images (global)
  int re_mul, re_add, im_mul, im_add;
  int crow_mul, crow_re, crow_im;
  const float2* coef;   // (rows, P, 9)
  const float* mean;    // (rows)
  const float2* basis;  // (P, 3, ns)
  int P;
  int sym;  // symmetric subharmonic frequencies (see k_pair_cols_reg)
  const float* img_scale;  // per output image factor on top of `scale` (NULL: none)
};

__device__ __forceinline__ float img_scale_of(const PairStore& st, int img) {
  return st.img_scale ? st.scale * __ldg(st.img_scale + img) : st.scale;
}

__global__ void __launch_bounds__(kThreads)
k_pair_cols(FftDesc d, const float2* __restrict__ tw, const float2* __restrict__ work, int C,
            int pair0, PairStore st) {
  extern __shared__ float2 sm[];
  const int ns = d.n;
  const int y0 = blockIdx.x * C;
  const int pl = blockIdx.y;  // pair within chunk
  const int pair = pair0 + pl;
  const int nb = fft_buf_len(d);
  float2* bufA = sm;
  float2* bufB = sm + nb * C;
  float2* stw = bufB + nb * C;
  // column tables from an even float2 offset: utab below is read as float4
  float2* mtab = stw + ((ns + 1) & ~1);  // (2, 3P, C)
  for (int i = threadIdx.x; i < ns; i += blockDim.x) stw[i] = tw[i];
  for (int i = threadIdx.x; i < ns * C; i += blockDim.x) {
    const int x = i / C, c = i % C;
    const int y = y0 + c;
    bufA[i] = y < ns ? __ldcs(work + ((size_t)pl * ns + x) * ns + y) : make_float2(0.f, 0.f);
  }
  const int img_re = pair * st.re_mul + st.re_add;
  const int img_im = pair * st.im_mul + st.im_add;
  const bool do_re = img_re < st.count, do_im = img_im < st.count;
  const int row_re = pl * st.crow_mul + st.crow_re, row_im = pl * st.crow_mul + st.crow_im;
  const int P = st.P;
  // m[o][p*3+i][c] = sum_j coef[o][p][i][j] basis[p][j][y]
  for (int i = threadIdx.x; i < 2 * 3 * P * C; i += blockDim.x) {
    const int c = i % C;
    const int pi = (i / C) % (3 * P);
    const int o = i / (C * 3 * P);
    const bool ok = o == 0 ? do_re : do_im;
    const int row = o == 0 ? row_re : row_im;
    const int y = y0 + c;
    float2 m = make_float2(0.f, 0.f);
    if (ok && y < ns) {
      const int p = pi / 3, ii = pi % 3;
      const float2* cf = st.coef + ((size_t)row * P + p) * 9 + ii * 3;
#pragma unroll
      for (int j = 0; j < 3; ++j) m = cfma(cf[j], st.basis[((size_t)p * 3 + j) * ns + y], m);
    }
    mtab[i] = m;
  }
  __syncthreads();
  // symmetric bases (b1 = 1, b2 = conj b0): per column K = sum_p m[p][1].x
  // minus the mean, per (level, column) (U_re, W_re, U_im, W_im), and the
  // first basis row of each level staged when it fits, as in the register
  // column pass; the transform's barriers order these writes before the reads
  float4* utab = (float4*)(mtab + 2 * 3 * P * C);   // P * C
  float2* ktab = mtab + 8 * (P > 0 ? P : 1) * C;     // C: (K_re, K_im)
  float2* sbasis = ktab + C;                         // P * ns
  const bool sb = st.sym && P * ns <= kColBasisMax;
  if (st.sym) {
    for (int i = threadIdx.x; i < P * C; i += blockDim.x) {
      const int p = i / C, c = i % C;
      const float2 m00 = mtab[(0 * 3 * P + 3 * p) * C + c], m02 = mtab[(0 * 3 * P + 3 * p + 2) * C + c];
      const float2 m10 = mtab[(1 * 3 * P + 3 * p) * C + c], m12 = mtab[(1 * 3 * P + 3 * p + 2) * C + c];
      utab[i] = make_float4(m00.x + m02.x, m02.y - m00.y, m10.x + m12.x, m12.y - m10.y);
    }
    for (int c = threadIdx.x; c < C; c += blockDim.x) {
      float k0 = 0.f, k1 = 0.f;
      for (int p = 0; p < P; ++p) {
        k0 += mtab[(0 * 3 * P + 3 * p + 1) * C + c].x;
        k1 += mtab[(1 * 3 * P + 3 * p + 1) * C + c].x;
      }
      if (P > 0 && do_re) k0 -= st.mean[row_re];
      if (P > 0 && do_im) k1 -= st.mean[row_im];
      ktab[c] = make_float2(k0, k1);
    }
    if (sb)
      for (int i = threadIdx.x; i < P * ns; i += blockDim.x)
        sbasis[i] = __ldg(st.basis + (size_t)(3 * (i / ns)) * ns + (i % ns));
  }
  float2* res = fft_smem(bufA, bufB, d, stw, C, 1, C, true);
  const float mre = (P > 0 && do_re) ? st.mean[row_re] : 0.f;
  const float mim = (P > 0 && do_im) ? st.mean[row_im] : 0.f;
  const float sre = img_scale_of(st, img_re), sim = img_scale_of(st, img_im);
  const size_t plane = (size_t)st.n_out * st.n_out;
  for (int i = threadIdx.x; i < ns * C; i += blockDim.x) {
    const int x = i / C, c = i % C;
    const int y = y0 + c;
    if (y >= ns) continue;
    const int xo = x - st.crop, yo = y - st.crop;
    if (xo < 0 || yo < 0 || xo >= st.n_out || yo >= st.n_out) continue;
    const float2 v = res[i];
    float lre, lim;
    if (st.sym) {
      const float2 k = ktab[c];
      lre = k.x;
      lim = k.y;
      for (int p = 0; p < P; ++p) {
        const float2 b = sb ? sbasis[p * ns + x] : __ldg(st.basis + (size_t)(3 * p) * ns + x);
        const float4 u = utab[p * C + c];
        lre = fmaf(b.x, u.x, fmaf(b.y, u.y, lre));
        lim = fmaf(b.x, u.z, fmaf(b.y, u.w, lim));
      }
    } else {
      lre = -mre;
      lim = -mim;
      for (int pi = 0; pi < 3 * P; ++pi) {
        const float2 b = st.basis[(size_t)pi * ns + x];
        const float2 m0 = mtab[(0 * 3 * P + pi) * C + c];
        const float2 m1 = mtab[(1 * 3 * P + pi) * C + c];
        lre = fmaf(b.x, m0.x, fmaf(-b.y, m0.y, lre));
        lim = fmaf(b.x, m1.x, fmaf(-b.y, m1.y, lim));
      }
    }
    const size_t o = (size_t)xo * st.n_out + yo;
    if (st.accumulate) {
      if (do_re) st.out[(size_t)img_re * plane + o] += sre * (v.x + lre);
      if (do_im) st.out[(size_t)img_im * plane + o] += sim * (v.y + lim);
    } else {
      if (do_re) __stcs(st.out + (size_t)img_re * plane + o, sre * (v.x + lre));
      if (do_im) __stcs(st.out + (size_t)img_im * plane + o, sim * (v.y + lim));
    }
  }
}

// plain complex column pass (pt_ifft2)
__global__ void __launch_bounds__(kThreads)
k_plain_cols(FftDesc d, const float2* __restrict__ tw, const float2* __restrict__ work, int C,
             float2* __restrict__ out) {
  extern __shared__ float2 sm[];
  const int ns = d.n;
  const int y0 = blockIdx.x * C;
  const int img = blockIdx.y;
  const int nb = fft_buf_len(d);
  float2* bufA = sm;
  float2* bufB = sm + nb * C;
  float2* stw = bufB + nb * C;
  for (int i = threadIdx.x; i < ns; i += blockDim.x) stw[i] = tw[i];
  for (int i = threadIdx.x; i < ns * C; i += blockDim.x) {
    const int x = i / C, c = i % C;
    const int y = y0 + c;
    bufA[i] = y < ns ? work[((size_t)img * ns + x) * ns + y] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  float2* res = fft_smem(bufA, bufB, d, stw, C, 1, C, true);
  for (int i = threadIdx.x; i < ns * C; i += blockDim.x) {
    const int x = i / C, c = i % C;
    const int y = y0 + c;
    if (y < ns) out[((size_t)img * ns + x) * ns + y] = res[i];
  }
}

// frames: per frame f of a chunk, shifted-and-summed subharmonic
// coefficients (FP64 phases), their grid mean, and the main-grid phasor tables.
// Displacements travel to the device inside the launch parameters (no
// pageable copy, hence no stream synchronisation on the frame path).
constexpr int kShiftDoubles = 1792;
struct ShiftParams {
  double v[kShiftDoubles];  // (nf, J, 2) for frames [fbeg, fbeg + nf) of the chunk
};

struct FramePrepArgs {
  const float2* sh_coef;  // (P, L, 3, 3)
  const double* sh_freq;  // (P, 3)
  const double* beta;     // (P, 3, 2)
  float2* coef;           // (F, P, 9)
  float* mean;            // (F)
  float2* px;             // (F, J, ns)
  float2* py;
  int F, L, J, P, ns, per_layer, frame0;
  double df;
};

// One CTA per frame, one thread per (level, 3x3 cell): the per-layer phases
// f_p . s are FP64 products reduced mod 1 (so the error does not grow with the
// travel), the phasors and the layer sum are float32 (the reference's own
// complex64 path), and the CTA reduces the grid mean of the low-order screen.
__global__ void k_frame_coef(FramePrepArgs a, ShiftParams sp, int fbeg, int nf) {
  __shared__ double part[32];
  const int fl = blockIdx.x;
  if (fl >= nf) return;
  const int f = fbeg + fl;
  const int t = threadIdx.x;
  double term = 0.0;
  if (t < a.P * 9) {
    const int p = t / 9, ij = t % 9, i = ij / 3, k = ij % 3;
    const double fi = a.sh_freq[p * 3 + i], fk = a.sh_freq[p * 3 + k];
    float2 acc = make_float2(0.f, 0.f);
    for (int j = 0; j < a.J; ++j) {
      const int l = a.per_layer ? a.frame0 + f : j;
      const double sx = sp.v[(fl * a.J + j) * 2];
      const double sy = sp.v[(fl * a.J + j) * 2 + 1];
      double ph = fi * sx + fk * sy;
      ph -= floor(ph);
      float sn, cs;
      sincospif(2.0f * (float)ph, &sn, &cs);
      const float2 c = a.sh_coef[(((size_t)p * a.L + l) * 3 + i) * 3 + k];
      acc = cfma(c, make_float2(cs, sn), acc);
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

// px[f][j][k] = exp(2 pi i f_k sx[f][j]), f_k = k' df, phase wrapped exactly
// in 64-bit fixed point.
__global__ void k_frame_phasors(FramePrepArgs a, ShiftParams sp, int fbeg) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int fjl = blockIdx.y;  // (frame - fbeg) * J + j
  if (k >= a.ns) return;
  const double sx = sp.v[fjl * 2];
  const double sy = sp.v[fjl * 2 + 1];
  const size_t fj = (size_t)fbeg * a.J + fjl;
  const uint64_t ux = phase_fixed(sx * a.df), uy = phase_fixed(sy * a.df);
  const uint64_t kk = (uint64_t)(int64_t)signed_freq(k, a.ns);
  a.px[fj * a.ns + k] = phasor_from_fixed(kk * ux);
  a.py[fj * a.ns + k] = phasor_from_fixed(kk * uy);
}

// ================================================================ layers / boiling
struct SeedTable {
  uint64_t s[64];
};

__global__ void k_fill_spectra(int ns, const float* __restrict__ amplitude,
                               const float* __restrict__ noise, SeedTable seeds,
                               float2* __restrict__ spectra) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t plane = (size_t)ns * ns;
  const int l = blockIdx.y;
  if (e >= plane) return;
  float2 z;
  if (noise) {
    const float* nl = noise + (size_t)l * 2 * plane;
    z = make_float2(nl[e], nl[plane + e]);
  } else {
    z = philox_cnormal(seeds.s[l], e, 0, kDomainLayer);
  }
  const float amp = amplitude[(size_t)l * plane + e];
  spectra[(size_t)l * plane + e] = make_float2(z.x * amp, z.y * amp);
}

__global__ void k_fill_sh(int L, int P, const float* __restrict__ sh_amp,
                          const float* __restrict__ sh_noise, SeedTable seeds,
                          float2* __restrict__ sh_coef) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P * L * 9) return;
  const int ij = i % 9, l = (i / 9) % L, p = i / (9 * L);
  float2 z;
  if (sh_noise) {
    // (L, P, 2, 3, 3)
    const float* b = sh_noise + ((size_t)l * P + p) * 18;
    z = make_float2(b[ij], b[9 + ij]);
  } else {
    z = philox_cnormal(seeds.s[l], (uint64_t)p * 9 + ij, 0, kDomainLayerSub);
  }
  const float amp = sh_amp[i];
  sh_coef[i] = make_float2(z.x * amp, z.y * amp);
}

__global__ void k_boil(size_t n_el, float2* __restrict__ s, const float* __restrict__ amplitude,
                       const float* __restrict__ tau, float dt, const float* __restrict__ noise,
                       uint64_t seed, uint64_t call, uint64_t idx_base) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_el) return;
  const float a = expf(-dt / tau[e]);
  const float b = sqrtf(fmaxf(1.0f - a * a, 0.0f));
  const float2 z = noise ? make_float2(noise[e], noise[n_el + e])
                         : philox_cnormal(seed, idx_base + e, call, kDomainBoil);
  const float amp = amplitude[e];
  const float2 v = s[e];
  s[e] = make_float2(fmaf(a, v.x, b * (z.x * amp)), fmaf(a, v.y, b * (z.y * amp)));
}

// ================================================================ LGS zoom
__global__ void k_lgs_zoom(int L, int ns, int n, int T, const int32_t* __restrict__ idx,
                           const float* __restrict__ w, const float* __restrict__ screens,
                           float scale, float* __restrict__ out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y;
  if (j >= n) return;
  float acc = 0.f;
  for (int l = 0; l < L; ++l) {
    const float* s = screens + (size_t)l * ns * ns;
    const int32_t* il = idx + (size_t)l * T * n;
    const float* wl = w + (size_t)l * T * n;
    float v = 0.f;
    for (int a = 0; a < T; ++a) {
      const float* row = s + (size_t)il[a * n + i] * ns;
      float rs = 0.f;
      for (int b = 0; b < T; ++b) rs = fmaf(wl[b * n + j], row[il[b * n + j]], rs);
      v = fmaf(wl[a * n + i], rs, v);
    }
    acc += v;
  }
  out[(size_t)i * n + j] = scale * acc;
}

#include "frames_fast.cuh"  // power-of-two fast path kernels
#include "cols_tma.cuh"     // TMA-fed column pass
#include "gt_fast.cuh"       // register transforms of length 3 * 2^k (Good-Thomas)

// ================================================================ host helpers
// shared memory of the generic passes: nb = fft_buf_len of the grid's
// transform (exchange buffers), ns twiddles
static size_t rows_smem(int ns, int nb, int rpc) {
  return (size_t)(2 * rpc * (nb + 1) + ns) * sizeof(float2);
}
static size_t frame_rows_smem(int ns, int nb) {
  return (size_t)(8 * (nb + 1) + ns) * sizeof(float2);
}
static size_t cols_smem(int ns, int nb, int C, int P) {
  // exchange buffers, twiddles, (m, U/W, K) column tables, staged basis rows
  return (size_t)(2 * nb * C + ((ns + 1) & ~1) + 8 * std::max(P, 1) * C + C +
                  (P * ns <= kColBasisMax ? P * ns : 0)) *
         sizeof(float2);
}

// The grid's transform for the frame passes: the Bluestein form only when
// its buffers fit (the frame row kernels hold eight and 2 x kPairsPerFft
// rows); otherwise the direct-sum stages.
static FftDesc frame_desc(const pt_grid* g) {
  FftDesc d = g->desc;
  const int ns = g->ns;
  if (d.M > 0) {
    const size_t cap = 220 * 1024;
    if (frame_rows_smem(ns, d.M) > cap ||
        (size_t)(2 * kPairsPerFft * (d.M + 1) + ns) * sizeof(float2) > cap ||
        cols_smem(ns, d.M, cols_per_cta(d.M), g->P) > cap)
      d.M = 0;
  }
  return d;
}

template <class K>
static int set_smem(K kernel, size_t bytes, const char* name) {
  if (bytes > 227 * 1024)
    return fail(PT_ERR_UNSUPPORTED, std::string(name) + ": grid too large for shared memory");
  if (bytes > 48 * 1024) {
    cudaError_t e =
        cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) return check_cuda(e, name);
  }
  // prefer the largest shared-memory carveout so several CTAs fit per SM
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                       (int)cudaSharedmemCarveoutMaxShared);
  if (e != cudaSuccess) return check_cuda(e, name);
  return PT_OK;
}

static int check_grid(const pt_grid* g, const char* who) {
  if (!g) return fail(PT_ERR_ARG, std::string(who) + ": grid is NULL");
  return PT_OK;
}

// 64-bit binary fraction of frac(x), host side (matches phase_fixed on the device).
static uint64_t host_fixed(double x) {
  double f = x - std::floor(x);
  double v = std::ldexp(f, 64);
  if (!(v < 18446744073709551615.0)) return ~0ull;
  return (uint64_t)v;
}

// Frames [f0, f0 + nf) of a layer-sum request are equally spaced in shift
// (s_f = s_0 + f delta for every layer, to 1e-9 m + 1e-12 relative), on a grid
// the register-recurrence kernel handles (ns <= 1024, L <= 16).
static bool uniform_ok(const double* sx, const double* sy, int per_layer, int L, int f0, int nf,
                       int ns) {
  if (per_layer || nf < 2 || L > kMaxUniformLayers || ns > 1024) return false;
  for (int l = 0; l < L; ++l) {
    const double* v[2] = {sx, sy};
    for (const double* a : v) {
      const double s0 = a[(size_t)f0 * L + l];
      const double d = (a[(size_t)(f0 + nf - 1) * L + l] - s0) / (nf - 1);
      for (int f = 1; f < nf; ++f) {
        const double sf = a[(size_t)(f0 + f) * L + l];
        if (std::fabs(sf - (s0 + f * d)) > 1e-9 + 1e-12 * std::fabs(sf)) return false;
      }
    }
  }
  return true;
}

template <int LM>
static int launch_uniform_t(const pt_grid* g, const float2* spectra, int L, int nf,
                            const UniformParams& up, float2* hn, float2* ptab, float2* img,
                            cudaStream_t s) {
  const int ns = g->ns;
  if ((ns & 1) == 0) {
    k_nyquist_h<<<dim3((2 * ns + 127) / 128, nf), 128, 0, s>>>(ns, spectra, L, nf, up, hn);
    count_launch();
  }
  const dim3 grid(ns, (nf + kAnchor - 1) / kAnchor);
  ProfScope ps("k_frame_rows_uniform", s);
  (void)ptab;  // the power-of-two sizes 256/512/1024 take launch_uniform_reg_chunk instead
  const FftDesc fd = frame_desc(g);
  const size_t smem = (size_t)(2 * kPairsPerFft * (fft_buf_len(fd) + 1) + ns) * sizeof(float2);
  if (ns <= 512) {
    if (int rc = set_smem(k_frame_rows_uniform<LM, 1>, smem, "k_frame_rows_uniform")) return rc;
    k_frame_rows_uniform<LM, 1><<<grid, ns, smem, s>>>(fd, g->tw, spectra, L, nf, up, hn,
                                                       img);
  } else {
    if (int rc = set_smem(k_frame_rows_uniform<LM, 2>, smem, "k_frame_rows_uniform")) return rc;
    k_frame_rows_uniform<LM, 2><<<grid, (ns + 1) / 2, smem, s>>>(fd, g->tw, spectra, L, nf,
                                                                up, hn, img);
  }
  return PT_OK;
}

static int launch_uniform_rows(const pt_grid* g, const float2* spectra, int L, const double* sx,
                               const double* sy, int f0, int nf, float2* hn, float2* ptab,
                               float2* img, cudaStream_t s) {
  const double df = 1.0 / (g->ns * g->dx);
  UniformParams up{};
  for (int l = 0; l < L; ++l) {
    const double x0 = sx[(size_t)f0 * L + l], y0 = sy[(size_t)f0 * L + l];
    const double dx = (sx[(size_t)(f0 + nf - 1) * L + l] - x0) / (nf - 1);
    const double dy = (sy[(size_t)(f0 + nf - 1) * L + l] - y0) / (nf - 1);
    up.ux0[l] = host_fixed(x0 * df);
    up.uy0[l] = host_fixed(y0 * df);
    up.dux[l] = host_fixed(dx * df);
    up.duy[l] = host_fixed(dy * df);
  }
  if (L <= 1) return launch_uniform_t<1>(g, spectra, L, nf, up, hn, ptab, img, s);
  if (L <= 2) return launch_uniform_t<2>(g, spectra, L, nf, up, hn, ptab, img, s);
  if (L <= 3) return launch_uniform_t<3>(g, spectra, L, nf, up, hn, ptab, img, s);
  if (L <= 4) return launch_uniform_t<4>(g, spectra, L, nf, up, hn, ptab, img, s);
  if (L <= 6) return launch_uniform_t<6>(g, spectra, L, nf, up, hn, ptab, img, s);
  if (L <= 9) return launch_uniform_t<9>(g, spectra, L, nf, up, hn, ptab, img, s);
  if (L <= 12) return launch_uniform_t<12>(g, spectra, L, nf, up, hn, ptab, img, s);
  return launch_uniform_t<16>(g, spectra, L, nf, up, hn, ptab, img, s);
}

// ---- uniform frames on the 256/512/1024 register path: one prep launch + rows
template <int LM>
static int uniform_reg_rows_t(const pt_grid* g, const float2* spectra, int L, int nf,
                              const UniformTables& ut, const float2* hn, float2* img,
                              cudaStream_t s) {
  const int ns = g->ns;
  const dim3 pgrid(ns / 2 + 1, (nf + kAnchor - 1) / kAnchor);  // row pairs {kx, ns - kx}
  auto go = [&](auto kern, int threads, int nv) -> int {
    const size_t smem = (size_t)(ns + 2 * nv * fft_padded(ns)) * sizeof(float2);
    if (int rc = set_smem(kern, smem, "k_frame_rows_uniform_reg")) return rc;
    ProfScope ps("k_frame_rows_uniform", s);
    kern<<<pgrid, threads, smem, s>>>(g->tw, spectra, L, nf, ut, hn, img);
    return PT_OK;
  };
  if (ns == 256) return go(k_frame_rows_uniform_reg<LM, 256>, 256, 8);
  if (ns == 512) return go(k_frame_rows_uniform_reg<LM, 512>, 512, 8);
  return go(k_frame_rows_uniform_reg<LM, 1024>, 512, 4);
}

static int launch_uniform_reg_chunk(const pt_grid* g, const float2* spectra, const float2* sh_coef,
                                    int L, const double* sx, const double* sy, int f0, int nf,
                                    const SpecWork& w, cudaStream_t s) {
  const int ns = g->ns;
  const double df = 1.0 / (ns * g->dx);
  UniformPrep a{};
  for (int l = 0; l < L; ++l) {
    const double x0 = sx[(size_t)f0 * L + l], y0 = sy[(size_t)f0 * L + l];
    const double dx = (sx[(size_t)(f0 + nf - 1) * L + l] - x0) / (nf - 1);
    const double dy = (sy[(size_t)(f0 + nf - 1) * L + l] - y0) / (nf - 1);
    a.up.ux0[l] = host_fixed(x0 * df);
    a.up.uy0[l] = host_fixed(y0 * df);
    a.up.dux[l] = host_fixed(dx * df);
    a.up.duy[l] = host_fixed(dy * df);
    a.s0x[l] = x0;
    a.s0y[l] = y0;
    a.dsx[l] = dx;
    a.dsy[l] = dy;
  }
  const int nb = (nf + kAnchor - 1) / kAnchor;
  float2* ptab = w.px;
  a.px0 = ptab;
  a.py0 = ptab + (size_t)nb * L * ns;
  a.rx = ptab + (size_t)2 * nb * L * ns;
  a.ry = ptab + (size_t)(2 * nb + 1) * L * ns;
  a.spectra = spectra;
  a.sh_coef = sh_coef;
  a.sh_freq = g->sh_freq;
  a.beta = g->beta;
  a.hn = w.hn;
  a.coef = w.coef;
  a.mean = w.mean;
  a.N = ns;
  a.L = L;
  a.P = g->P;
  a.F = nf;
  a.nb = nb;
  a.blocks_tab = ((nb + 1) * L * ns + 255) / 256;
  a.blocks_nyq = (2 * ns * ((nf + kNyqGroup - 1) / kNyqGroup) + 255) / 256;
  {
    ProfScope ps("k_uniform_prep", s);
    k_uniform_prep<<<a.blocks_tab + a.blocks_nyq + nf, 256, 0, s>>>(a);
  }
  count_launch();
  const UniformTables ut{a.px0, a.py0, a.rx, a.ry};
  if (L <= 1) return uniform_reg_rows_t<1>(g, spectra, L, nf, ut, w.hn, w.img, s);
  if (L <= 2) return uniform_reg_rows_t<2>(g, spectra, L, nf, ut, w.hn, w.img, s);
  if (L <= 3) return uniform_reg_rows_t<3>(g, spectra, L, nf, ut, w.hn, w.img, s);
  if (L <= 4) return uniform_reg_rows_t<4>(g, spectra, L, nf, ut, w.hn, w.img, s);
  if (L <= 6) return uniform_reg_rows_t<6>(g, spectra, L, nf, ut, w.hn, w.img, s);
  if (L <= 9) return uniform_reg_rows_t<9>(g, spectra, L, nf, ut, w.hn, w.img, s);
  if (L <= 12) return uniform_reg_rows_t<12>(g, spectra, L, nf, ut, w.hn, w.img, s);
  return uniform_reg_rows_t<16>(g, spectra, L, nf, ut, w.hn, w.img, s);
}

// ---- power-of-two dispatch (runtime ns -> template N)
static bool pow2_fast(int ns) { return ns >= 8 && ns <= 4096 && (ns & (ns - 1)) == 0; }

#define PT_POW2_CASES(X) X(8) X(16) X(32) X(64) X(128) X(256) X(512) X(1024) X(2048) X(4096)

template <int N>
static int rows_reg_t(const pt_grid* g, const float2* in, int gen, const GenRowArgs& ga, int nimg,
                      float2* work, cudaStream_t s) {
  using Cfg = RegCfg<N>;
  const size_t smem = (size_t)(N + 2 * Cfg::NV * fft_padded(N)) * sizeof(float2);
  if (int rc = set_smem(k_rows_reg<N>, smem, "k_rows_reg")) return rc;
  ProfScope ps("k_rows", s);
  k_rows_reg<N><<<dim3((N + Cfg::NV - 1) / Cfg::NV, nimg), Cfg::THREADS, smem, s>>>(g->tw, in, gen,
                                                                                   ga, work);
  return PT_OK;
}

static int rows_reg(const pt_grid* g, const float2* in, int gen, const GenRowArgs& ga, int nimg,
                    float2* work, cudaStream_t s) {
  switch (g->ns) {
#define PT_CASE(n) \
  case n: return rows_reg_t<n>(g, in, gen, ga, nimg, work, s);
    PT_POW2_CASES(PT_CASE)
#undef PT_CASE
  }
  return fail(PT_ERR_UNSUPPORTED, "rows_reg: not a power of two");
}

template <int N>
static int plain_cols_reg_t(const pt_grid* g, const float2* work, int nimg, float2* out,
                            cudaStream_t s) {
  using Cfg = RegCfg<N>;
  const size_t smem = (size_t)(N + 2 * Cfg::C * N) * sizeof(float2);
  if (int rc = set_smem(k_plain_cols_reg<N>, smem, "k_plain_cols_reg")) return rc;
  ProfScope ps("k_plain_cols", s);
  k_plain_cols_reg<N><<<dim3((N + Cfg::C - 1) / Cfg::C, nimg), Cfg::THREADS, smem, s>>>(g->tw, work,
                                                                                        out);
  return PT_OK;
}

static int plain_cols_reg(const pt_grid* g, const float2* work, int nimg, float2* out,
                          cudaStream_t s) {
  switch (g->ns) {
#define PT_CASE(n) \
  case n: return plain_cols_reg_t<n>(g, work, nimg, out, s);
    PT_POW2_CASES(PT_CASE)
#undef PT_CASE
  }
  return fail(PT_ERR_UNSUPPORTED, "plain_cols_reg: not a power of two");
}

template <int N>
static int pair_cols_reg_t(const pt_grid* g, const float2* work, int npair, int pair0,
                           const PairStore& st, cudaStream_t s) {
  using Cfg = PairColCfg<N>;
  const int P = g->P;
  const size_t smem = (size_t)(N + 2 * Cfg::C * N + (2 * 3 + 2) * std::max(P, 1) * Cfg::C +
                               (P * N <= kColBasisMax ? P * N : 0)) *
                      sizeof(float2);
  if (int rc = set_smem(k_pair_cols_reg<N>, smem, "k_pair_cols_reg")) return rc;
  ProfScope ps("k_pair_cols", s);
  // a programmatic dependent of the row pass before it on the stream: its
  // CTAs stage their twiddles while the row pass's last wave runs, then wait
  // (griddepcontrol.wait) for the row pass to complete
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((N + Cfg::C - 1) / Cfg::C, npair);
  cfg.blockDim = dim3(Cfg::THREADS);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return check_cuda(cudaLaunchKernelEx(&cfg, k_pair_cols_reg<N>, g->tw, work, pair0, st),
                    "k_pair_cols_reg");
}

// ---- TMA-fed column pass (N = 256, 512, 1024)
typedef CUresult (*TensorMapEncodeFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                      const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                      const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                      CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static TensorMapEncodeFn tensor_map_encoder() {
  static std::once_flag once;
  static TensorMapEncodeFn fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<TensorMapEncodeFn>(p);
  });
  return fn;
}

template <int N>
static int pair_cols_tma_t(const pt_grid* g, const float2* work, int npair, int pair0,
                           const PairStore& st, cudaStream_t s) {
  using Cfg = TmaCfg<N>;
  TensorMapEncodeFn enc = tensor_map_encoder();
  if (!enc) return fail(PT_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled unavailable");
  // 2-D view of the (npair, N, N) complex workspace: x = column (inner), y = pair * N + row
  CUtensorMap map;
  const cuuint64_t dims[2] = {(cuuint64_t)N, (cuuint64_t)npair * N};
  const cuuint64_t strides[1] = {(cuuint64_t)N * sizeof(float2)};
  const cuuint32_t box[2] = {(cuuint32_t)Cfg::C, (cuuint32_t)Cfg::BOXR};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = enc(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, (void*)work, dims, strides, box,
                         estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(PT_ERR_CUDA, "cuTensorMapEncodeTiled failed");
  const int P1 = std::max(g->P, 1);
  const size_t smem =
      (size_t)(3 * N * Cfg::C + N + 2 * 3 * P1 * Cfg::C) * sizeof(float2) + 2 * sizeof(uint64_t);
  if (int rc = set_smem(k_pair_cols_tma<N>, smem, "k_pair_cols_tma")) return rc;
  const int xb = N / Cfg::C;
  const int groups = std::max(1, std::min(npair, (2 * 152 + xb - 1) / xb));
  ProfScope ps("k_pair_cols", s);
  k_pair_cols_tma<N><<<dim3(xb, groups), RegCfg<N>::THREADS, smem, s>>>(map, g->tw, npair, pair0,
                                                                        st);
  return PT_OK;
}

// The TMA-fed column pass is selected with PYTURB_GB300_COLS=tma (N = 256, 512,
// 1024). Measured on the GB300 it trails the one-CTA-per-tile register pass,
// whose 2048 short CTAs keep more loads in flight, so the latter is the default.
// default column-pass variant of new grids (PYTURB_GB300_COLS=tma selects TMA)
static int default_cols_variant() {
  static const int v = [] {
    const char* e = std::getenv("PYTURB_GB300_COLS");
    return (e && std::string(e) == "tma") ? 1 : 0;
  }();
  return v;
}

// ---- Good-Thomas register path: ns = 3 M, M = 64 .. 512
static int gt_m(int ns) {
  if (ns % 3 != 0) return 0;
  const int m = ns / 3;
  return (m >= 64 && m <= 512 && (m & (m - 1)) == 0) ? m : 0;
}

template <int M>
static int rows_gt_t(const pt_grid* g, const float2* in, int gen, const GenRowArgs& ga, int nimg,
                     float2* work, cudaStream_t s) {
  using G = GtCfg<3, M>;
  const size_t smem = (size_t)(M + G::ROW_NV * 2 * 3 * G::PAD) * sizeof(float2);
  if (int rc = set_smem(k_rows_gt<3, M>, smem, "k_rows_gt")) return rc;
  ProfScope ps("k_rows", s);
  k_rows_gt<3, M><<<dim3((G::N + G::ROW_NV - 1) / G::ROW_NV, nimg), G::ROW_THREADS, smem, s>>>(
      g->tw, in, gen, ga, work);
  return PT_OK;
}

template <int M>
static int pair_cols_gt_t(const pt_grid* g, const float2* work, int npair, int pair0,
                          const PairStore& st, cudaStream_t s) {
  using G = GtCfg<3, M>;
  const int P = g->P;
  const size_t smem = (size_t)(M + 2 * 3 * M * G::C + 8 * std::max(P, 1) * G::C +
                               (P * G::N <= kColBasisMax ? P * G::N : 0)) *
                      sizeof(float2);
  if (int rc = set_smem(k_pair_cols_gt<3, M>, smem, "k_pair_cols_gt")) return rc;
  ProfScope ps("k_pair_cols", s);
  k_pair_cols_gt<3, M><<<dim3((G::N + G::C - 1) / G::C, npair), G::COL_THREADS, smem, s>>>(
      g->tw, work, pair0, st);
  return PT_OK;
}

static int rows_gt(const pt_grid* g, const float2* in, int gen, const GenRowArgs& ga, int nimg,
                   float2* work, cudaStream_t s) {
  switch (gt_m(g->ns)) {
    case 64: return rows_gt_t<64>(g, in, gen, ga, nimg, work, s);
    case 128: return rows_gt_t<128>(g, in, gen, ga, nimg, work, s);
    case 256: return rows_gt_t<256>(g, in, gen, ga, nimg, work, s);
    case 512: return rows_gt_t<512>(g, in, gen, ga, nimg, work, s);
  }
  return fail(PT_ERR_UNSUPPORTED, "rows_gt: not 3 x 2^k");
}

static int pair_cols_gt(const pt_grid* g, const float2* work, int npair, int pair0,
                        const PairStore& st, cudaStream_t s) {
  switch (gt_m(g->ns)) {
    case 64: return pair_cols_gt_t<64>(g, work, npair, pair0, st, s);
    case 128: return pair_cols_gt_t<128>(g, work, npair, pair0, st, s);
    case 256: return pair_cols_gt_t<256>(g, work, npair, pair0, st, s);
    case 512: return pair_cols_gt_t<512>(g, work, npair, pair0, st, s);
  }
  return fail(PT_ERR_UNSUPPORTED, "pair_cols_gt: not 3 x 2^k");
}

static int pair_cols_reg(const pt_grid* g, const float2* work, int npair, int pair0,
                         const PairStore& st, cudaStream_t s) {
  if (g->cols_variant == 1) {
    if (g->ns == 256) return pair_cols_tma_t<256>(g, work, npair, pair0, st, s);
    if (g->ns == 512) return pair_cols_tma_t<512>(g, work, npair, pair0, st, s);
    if (g->ns == 1024) return pair_cols_tma_t<1024>(g, work, npair, pair0, st, s);
  }
  switch (g->ns) {
#define PT_CASE(n) \
  case n: return pair_cols_reg_t<n>(g, work, npair, pair0, st, s);
    PT_POW2_CASES(PT_CASE)
#undef PT_CASE
  }
  return fail(PT_ERR_UNSUPPORTED, "pair_cols_reg: not a power of two");
}

}  // namespace pt

using namespace pt;

// Device error word set by bounded waits that ran out (0 = none).
namespace pt {
int tc_device_error(int* out, int clear);
int dft_device_error(int* out, int clear);
}

extern "C" int pt_device_error(int* out, int clear) {
  if (!out) return fail(PT_ERR_ARG, "pt_device_error: out is NULL");
  if (int rc = check_cuda(cudaDeviceSynchronize(), "pt_device_error: sync")) return rc;
  if (int rc = check_cuda(cudaMemcpyFromSymbol(out, g_pt_device_error, sizeof(int)),
                          "pt_device_error: read"))
    return rc;
  if (clear) {
    const int zero = 0;
    if (int rc = check_cuda(cudaMemcpyToSymbol(g_pt_device_error, &zero, sizeof(int)),
                            "pt_device_error: clear"))
      return rc;
  }
  int tcw = 0, dftw = 0;  // the tensor-core kernels' own error words (separate modules)
  if (int rc = tc_device_error(&tcw, clear)) return rc;
  if (int rc = dft_device_error(&dftw, clear)) return rc;
  *out |= tcw | dftw;
  return PT_OK;
}

extern "C" int pt_selftest_wait_timeout(long long limit, int* timed_out) {
  if (!timed_out || limit < 1 || limit > (1ll << 24))
    return fail(PT_ERR_ARG, "pt_selftest_wait_timeout: bad arguments");
  int* d = nullptr;
  if (int rc = check_cuda(cudaMalloc(&d, sizeof(int)), "pt_selftest_wait_timeout: cudaMalloc"))
    return rc;
  k_selftest_wait_timeout<<<1, 32>>>(limit, d);
  int rc = check_launch("pt_selftest_wait_timeout");
  if (!rc) rc = check_cuda(cudaMemcpy(timed_out, d, sizeof(int), cudaMemcpyDeviceToHost),
                           "pt_selftest_wait_timeout: read");
  cudaFree(d);
  return rc;
}

using namespace pt;

// ================================================================ C-ABI
// Lengths whose largest prime factor exceeds kBluesteinPrime take the
// Bluestein form (fft_bluestein) when its padded length M fits the passes'
// shared memory: the direct-sum stage costs O(p) per element for a prime p.
constexpr int kBluesteinPrime = 61;
constexpr int kBluesteinMaxM = 8192;

static int largest_prime_factor(int n) {
  int best = 1;
  for (int p = 2; (long long)p * p <= n; ++p)
    while (n % p == 0) {
      best = p;
      n /= p;
    }
  return n > 1 ? std::max(best, n) : best;
}

// In-place radix-2 transform of a power-of-two length, exp(+2 pi i j k / n), FP64.
static void host_fft_pow2(std::vector<double>& re, std::vector<double>& im) {
  const size_t n = re.size();
  for (size_t i = 1, j = 0; i < n; ++i) {
    size_t bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) {
      std::swap(re[i], re[j]);
      std::swap(im[i], im[j]);
    }
  }
  for (size_t len = 2; len <= n; len <<= 1) {
    const double a = 2.0 * M_PI / (double)len;
    for (size_t i = 0; i < n; i += len)
      for (size_t k = 0; k < len / 2; ++k) {
        const double c = std::cos(a * (double)k), sn = std::sin(a * (double)k);
        const size_t u = i + k, v = i + k + len / 2;
        const double tr = re[v] * c - im[v] * sn, ti = re[v] * sn + im[v] * c;
        re[v] = re[u] - tr;
        im[v] = im[u] - ti;
        re[u] += tr;
        im[u] += ti;
      }
  }
}

static int bluestein_plan(pt_grid* g) {
  const int n = g->ns;
  if (largest_prime_factor(n) <= kBluesteinPrime) return PT_OK;
  int M = 1;
  while (M < 2 * n - 1) M <<= 1;
  if (M > kBluesteinMaxM) return PT_OK;  // keeps the direct-sum stage
  const FftDesc dm = make_fft_desc(M);
  std::vector<float2> tab((size_t)n + 2 * M);
  std::vector<double> br(M, 0.0), bi(M, 0.0);
  for (int e = 0; e < n; ++e) {
    const long long q = (long long)e * e % (2LL * n);  // exact phase index
    const double a = M_PI * (double)q / (double)n;
    const double c = std::cos(a), sn = std::sin(a);
    tab[e] = make_float2((float)c, (float)sn);
    br[e] = c;
    bi[e] = -sn;
    if (e > 0) {
      br[M - e] = c;
      bi[M - e] = -sn;
    }
  }
  host_fft_pow2(br, bi);
  for (int k = 0; k < M; ++k) {
    tab[(size_t)n + k] = make_float2((float)br[k], (float)bi[k]);
    const double a = 2.0 * M_PI * (double)k / (double)M;
    tab[(size_t)n + M + k] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
  int rc = check_cuda(cudaMalloc(&g->blu, tab.size() * sizeof(float2)), "pt_grid_create: cudaMalloc");
  if (!rc)
    rc = check_cuda(cudaMemcpy(g->blu, tab.data(), tab.size() * sizeof(float2), cudaMemcpyHostToDevice),
                    "pt_grid_create: cudaMemcpy");
  if (rc) return rc;
  g->desc.M = M;
  g->desc.mstages = dm.nstages;
  for (int i = 0; i < dm.nstages; ++i) g->desc.mradix[i] = dm.radix[i];
  g->desc.chirp = g->blu;
  g->desc.bhat = g->blu + n;
  g->desc.twM = g->blu + n + M;
  return PT_OK;
}

extern "C" int pt_grid_create(pt_grid** out, int ns, double dx, int P, const double* sh_freq) {
  if (!out) return fail(PT_ERR_ARG, "pt_grid_create: out is NULL");
  *out = nullptr;
  if (ns < 2 || ns > 8192) return fail(PT_ERR_ARG, "pt_grid_create: ns must be in [2, 8192]");
  if (!(dx > 0) || !std::isfinite(dx))
    return fail(PT_ERR_ARG, "pt_grid_create: pixel_scale must be positive and finite");
  if (P < 0 || P > kMaxLevels) return fail(PT_ERR_ARG, "pt_grid_create: n_levels must be in [0, 16]");
  if (P > 0 && !sh_freq) return fail(PT_ERR_ARG, "pt_grid_create: sh_freq is NULL");
  pt_grid* g = new pt_grid{};
  g->ns = ns;
  g->dx = dx;
  g->P = P;
  g->cols_variant = default_cols_variant();
  g->desc = make_fft_desc(ns);
  if (g->desc.nstages >= kMaxStages) {
    delete g;
    return fail(PT_ERR_UNSUPPORTED, "pt_grid_create: too many FFT stages");
  }
  std::vector<float2> tw(ns);
  for (int k = 0; k < ns; ++k) {
    const double a = 2.0 * M_PI * (double)k / ns;
    tw[k] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
  const int Pm = std::max(P, 1);
  std::vector<float2> basis((size_t)Pm * 3 * ns, make_float2(0.f, 0.f));
  std::vector<double> beta((size_t)Pm * 3 * 2, 0.0);
  for (int p = 0; p < P; ++p)
    for (int i = 0; i < 3; ++i) {
      const double f = sh_freq[p * 3 + i];
      double br = 0, bi = 0;
      for (int x = 0; x < ns; ++x) {
        const double arg = 2.0 * M_PI * f * (((double)x - ns / 2.0) * dx);
        const double c = std::cos(arg), s = std::sin(arg);
        basis[((size_t)p * 3 + i) * ns + x] = make_float2((float)c, (float)s);
        br += c;
        bi += s;
      }
      beta[(p * 3 + i) * 2] = br / ns;
      beta[(p * 3 + i) * 2 + 1] = bi / ns;
    }
  std::vector<double> freq((size_t)Pm * 3, 0.0);
  for (int i = 0; i < P * 3; ++i) freq[i] = sh_freq[i];
  g->sym = 1;
  for (int p = 0; p < P; ++p)
    if (!(sh_freq[p * 3 + 1] == 0.0 && sh_freq[p * 3] == -sh_freq[p * 3 + 2])) g->sym = 0;
  int rc = check_cuda(cudaMalloc(&g->tw, ns * sizeof(float2)), "pt_grid_create: cudaMalloc");
  if (!rc) rc = check_cuda(cudaMalloc(&g->basis, basis.size() * sizeof(float2)), "pt_grid_create: cudaMalloc");
  if (!rc) rc = check_cuda(cudaMalloc(&g->sh_freq, freq.size() * sizeof(double)), "pt_grid_create: cudaMalloc");
  if (!rc) rc = check_cuda(cudaMalloc(&g->beta, beta.size() * sizeof(double)), "pt_grid_create: cudaMalloc");
  if (!rc) rc = check_cuda(cudaMemcpy(g->tw, tw.data(), ns * sizeof(float2), cudaMemcpyHostToDevice), "pt_grid_create: cudaMemcpy");
  if (!rc) rc = check_cuda(cudaMemcpy(g->basis, basis.data(), basis.size() * sizeof(float2), cudaMemcpyHostToDevice), "pt_grid_create: cudaMemcpy");
  if (!rc) rc = check_cuda(cudaMemcpy(g->sh_freq, freq.data(), freq.size() * sizeof(double), cudaMemcpyHostToDevice), "pt_grid_create: cudaMemcpy");
  if (!rc) rc = check_cuda(cudaMemcpy(g->beta, beta.data(), beta.size() * sizeof(double), cudaMemcpyHostToDevice), "pt_grid_create: cudaMemcpy");
  if (!rc) rc = bluestein_plan(g);
  if (rc) {
    pt_grid_destroy(g);
    return rc;
  }
  *out = g;
  return PT_OK;
}

extern "C" int pt_grid_radices(const pt_grid* g, int* n_stages, int* radices) {
  if (int rc = check_grid(g, "pt_grid_radices")) return rc;
  if (!n_stages || !radices) return fail(PT_ERR_ARG, "pt_grid_radices: NULL pointer");
  *n_stages = g->desc.nstages;
  for (int i = 0; i < g->desc.nstages; ++i) radices[i] = g->desc.radix[i];
  return PT_OK;
}

extern "C" int pt_grid_set_radices(pt_grid* g, int n_stages, const int* radices) {
  if (int rc = check_grid(g, "pt_grid_set_radices")) return rc;
  if (!radices || n_stages < 1 || n_stages >= kMaxStages)
    return fail(PT_ERR_ARG, "pt_grid_set_radices: n_stages must be in [1, 23]");
  long long prod = 1;
  for (int i = 0; i < n_stages; ++i) {
    if (radices[i] < 2) return fail(PT_ERR_ARG, "pt_grid_set_radices: every radix must be >= 2");
    prod *= radices[i];
    if (prod > g->ns) break;
  }
  if (prod != g->ns) return fail(PT_ERR_ARG, "pt_grid_set_radices: radices must multiply to ns");
  g->desc.nstages = n_stages;
  for (int i = 0; i < n_stages; ++i) g->desc.radix[i] = radices[i];
  return PT_OK;
}

extern "C" int pt_grid_set_cols_variant(pt_grid* g, int variant) {
  if (int rc = check_grid(g, "pt_grid_set_cols_variant")) return rc;
  if (variant != 0 && variant != 1)
    return fail(PT_ERR_ARG, "pt_grid_set_cols_variant: variant must be 0 (register) or 1 (TMA)");
  g->cols_variant = variant;
  return PT_OK;
}

extern "C" int pt_grid_destroy(pt_grid* g) {
  if (!g) return PT_OK;
  cudaFree(g->tw);
  cudaFree(g->basis);
  cudaFree(g->sh_freq);
  cudaFree(g->beta);
  cudaFree(g->blu);
  delete g;
  return PT_OK;
}

extern "C" size_t pt_grid_workspace_bytes(const pt_grid* g, int L) {
  if (!g) return 0;
  return carve(g, std::max(1, L), nullptr).bytes;
}

extern "C" int pt_ifft2(const pt_grid* g, const float* in, float* out, int batch, void* work,
                        size_t work_bytes, void* stream) {
  if (int rc = check_grid(g, "pt_ifft2")) return rc;
  if (!in || !out || batch < 0) return fail(PT_ERR_ARG, "pt_ifft2: bad arguments");
  SpecWork w = carve(g, 1, work);
  if (!work || work_bytes < w.bytes) return fail(PT_ERR_ARG, "pt_ifft2: workspace too small");
  cudaStream_t s = (cudaStream_t)stream;
  const int ns = g->ns, blen = fft_buf_len(g->desc), ch = gen_chunk(ns),
            rpc = rows_per_cta(blen), C = cols_per_cta(blen);
  const size_t rs = rows_smem(ns, blen, rpc), cs = cols_smem(ns, blen, C, 0);
  if (int rc = set_smem(k_rows, rs, "k_rows")) return rc;
  if (int rc = set_smem(k_plain_cols, cs, "k_plain_cols")) return rc;
  GenRowArgs none{};
  for (int b0 = 0; b0 < batch; b0 += ch) {
    const int nb = std::min(ch, batch - b0);
    const float2* src = (const float2*)in + (size_t)b0 * ns * ns;
    float2* dst = (float2*)out + (size_t)b0 * ns * ns;
    if (pow2_fast(ns)) {
      if (int rc = rows_reg(g, src, 0, none, nb, w.img, s)) return rc;
      if (int rc = plain_cols_reg(g, w.img, nb, dst, s)) return rc;
    } else {
      {
        ProfScope ps("k_rows", s);
        k_rows<<<dim3((ns + rpc - 1) / rpc, nb), kThreads, rs, s>>>(g->desc, g->tw, rpc, src, 0,
                                                                   none, w.img);
      }
      ProfScope ps("k_plain_cols", s);
      k_plain_cols<<<dim3((ns + C - 1) / C, nb), kThreads, cs, s>>>(g->desc, g->tw, w.img, C, dst);
    }
    count_launch(2);
    if (int rc = check_launch("pt_ifft2")) return rc;
  }
  return PT_OK;
}

static int generate_impl(const pt_grid* g, int count, const float* amplitude,
                         const float* sh_amp, const float* noise, const float* sh_noise,
                         uint64_t seed, uint64_t call, int crop, int n_out, float scale,
                         const float* screen_scale, int accumulate, float* out, void* work,
                         size_t work_bytes, void* stream) {
  if (int rc = check_grid(g, "pt_generate")) return rc;
  const int ns = g->ns, P = g->P;
  if (count < 1) return fail(PT_ERR_ARG, "pt_generate: count must be >= 1");
  if (!amplitude || !out) return fail(PT_ERR_ARG, "pt_generate: NULL amplitude or out");
  if (P > 0 && !sh_amp) return fail(PT_ERR_ARG, "pt_generate: sh_amp is NULL");
  if (crop < 0 || n_out < 1 || crop + n_out > ns)
    return fail(PT_ERR_ARG, "pt_generate: crop window outside the grid");
  SpecWork w = carve(g, 1, work);
  if (!work || work_bytes < w.bytes) return fail(PT_ERR_ARG, "pt_generate: workspace too small");
  cudaStream_t s = (cudaStream_t)stream;
  const int n_fft = (count + 1) / 2;
  const int blen = fft_buf_len(g->desc);
  const int ch = gen_chunk(ns), rpc = rows_per_cta(blen), C = cols_per_cta(blen);
  const size_t rs = rows_smem(ns, blen, rpc), cs = cols_smem(ns, blen, C, P);
  if (int rc = set_smem(k_rows, rs, "k_rows")) return rc;
  if (int rc = set_smem(k_pair_cols, cs, "k_pair_cols")) return rc;
  for (int b0 = 0; b0 < n_fft; b0 += ch) {
    const int nb = std::min(ch, n_fft - b0);
    GenRowArgs ga{amplitude, noise, n_fft, b0, seed, call, sh_amp, sh_noise, g->beta,
                  w.coef, w.mean, count, ch, P};
    if (pow2_fast(ns)) {
      if (int rc = rows_reg(g, nullptr, 1, ga, nb, w.img, s)) return rc;
    } else if (gt_m(ns)) {
      if (int rc = rows_gt(g, nullptr, 1, ga, nb, w.img, s)) return rc;
    } else {
      ProfScope ps("k_rows", s);
      k_rows<<<dim3((ns + rpc - 1) / rpc, nb), kThreads, rs, s>>>(g->desc, g->tw, rpc, nullptr, 1,
                                                                 ga, w.img);
    }
    count_launch();
    PairStore st{};
    st.out = out;
    st.n_out = n_out;
    st.crop = crop;
    st.scale = scale;
    st.accumulate = accumulate;
    st.count = count;
    st.re_mul = 1;
    st.re_add = 0;
    st.im_mul = 1;
    st.im_add = n_fft;
    st.crow_mul = 1;
    st.crow_re = 0;   // rows [0, ch): screens b0 + pl
    st.crow_im = ch;  // rows [ch, 2 ch): screens n_fft + b0 + pl
    st.coef = w.coef;
    st.mean = w.mean;
    st.basis = g->basis;
    st.P = P;
    st.sym = g->sym;
    st.img_scale = screen_scale;
    if (pow2_fast(ns)) {
      if (int rc = pair_cols_reg(g, w.img, nb, b0, st, s)) return rc;
    } else if (gt_m(ns)) {
      if (int rc = pair_cols_gt(g, w.img, nb, b0, st, s)) return rc;
    } else {
      ProfScope ps("k_pair_cols", s);
      k_pair_cols<<<dim3((ns + C - 1) / C, nb), kThreads, cs, s>>>(g->desc, g->tw, w.img, C, b0, st);
    }
    count_launch();
    if (int rc = check_launch("pt_generate")) return rc;
  }
  return PT_OK;
}

extern "C" int pt_generate(const pt_grid* g, int count, const float* amplitude,
                           const float* sh_amp, const float* noise, const float* sh_noise,
                           uint64_t seed, uint64_t call, int crop, int n_out, float scale,
                           int accumulate, float* out, void* work, size_t work_bytes,
                           void* stream) {
  return generate_impl(g, count, amplitude, sh_amp, noise, sh_noise, seed, call, crop, n_out,
                       scale, nullptr, accumulate, out, work, work_bytes, stream);
}

extern "C" int pt_generate_scaled(const pt_grid* g, int count, const float* amplitude,
                                  const float* sh_amp, uint64_t seed, uint64_t call, int crop,
                                  int n_out, float scale, const float* screen_scale, float* out,
                                  void* work, size_t work_bytes, void* stream) {
  if (!screen_scale) return fail(PT_ERR_ARG, "pt_generate_scaled: screen_scale is NULL");
  return generate_impl(g, count, amplitude, sh_amp, nullptr, nullptr, seed, call, crop, n_out,
                       scale, screen_scale, 0, out, work, work_bytes, stream);
}

extern "C" int pt_layers_fill(const pt_grid* g, int L, const float* amplitude,
                              const float* sh_amp, const float* noise, const float* sh_noise,
                              const uint64_t* seeds, float* spectra, float* sh_coef,
                              void* stream) {
  if (int rc = check_grid(g, "pt_layers_fill")) return rc;
  if (L < 1 || L > 64) return fail(PT_ERR_ARG, "pt_layers_fill: n_layers must be in [1, 64]");
  if (!amplitude || !spectra) return fail(PT_ERR_ARG, "pt_layers_fill: NULL amplitude or spectra");
  if (g->P > 0 && (!sh_amp || !sh_coef)) return fail(PT_ERR_ARG, "pt_layers_fill: NULL sh_amp or sh_coef");
  if ((!noise || (g->P > 0 && !sh_noise)) && !seeds)
    return fail(PT_ERR_ARG, "pt_layers_fill: seeds required when noise is not injected");
  SeedTable st{};
  for (int l = 0; l < L; ++l) st.s[l] = seeds ? seeds[l] : 0;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t plane = (size_t)g->ns * g->ns;
  k_fill_spectra<<<dim3((unsigned)((plane + 255) / 256), L), 256, 0, s>>>(
      g->ns, amplitude, noise, st, (float2*)spectra);
  count_launch();
  if (g->P > 0) {
    const int n = g->P * L * 9;
    k_fill_sh<<<(n + 127) / 128, 128, 0, s>>>(L, g->P, sh_amp, sh_noise, st, (float2*)sh_coef);
    count_launch();
  }
  return check_launch("pt_layers_fill");
}

extern "C" int pt_frames(const pt_grid* g, int L, const float* spectra, const float* sh_coef,
                         int F, const double* sx, const double* sy, int per_layer, int crop,
                         int n_out, float scale, float* out, void* work, size_t work_bytes,
                         void* stream) {
  if (int rc = check_grid(g, "pt_frames")) return rc;
  const int ns = g->ns, P = g->P;
  if (L < 1) return fail(PT_ERR_ARG, "pt_frames: n_layers must be >= 1");
  if (F < 1) return fail(PT_ERR_ARG, "pt_frames: n_frames must be >= 1");
  if (!spectra || !out || !sx || !sy) return fail(PT_ERR_ARG, "pt_frames: NULL pointer");
  if (P > 0 && !sh_coef) return fail(PT_ERR_ARG, "pt_frames: sh_coef is NULL");
  if (per_layer && F != L) return fail(PT_ERR_ARG, "pt_frames: per-layer mode needs n_frames == n_layers");
  if (per_layer && (crop != 0 || n_out != ns)) return fail(PT_ERR_ARG, "pt_frames: per-layer screens are uncropped");
  if (crop < 0 || n_out < 1 || crop + n_out > ns)
    return fail(PT_ERR_ARG, "pt_frames: crop window outside the grid");
  SpecWork w = carve(g, L, work);
  if (!work || work_bytes < w.bytes) return fail(PT_ERR_ARG, "pt_frames: workspace too small");
  cudaStream_t s = (cudaStream_t)stream;
  const FftDesc fd = frame_desc(g);
  const int blen = fft_buf_len(fd);
  const int ch = image_chunk(ns), C = cols_per_cta(blen);
  const int J = per_layer ? 1 : L;
  if (2 * J > kShiftDoubles) return fail(PT_ERR_UNSUPPORTED, "pt_frames: at most 896 layers");
  const size_t rs = frame_rows_smem(ns, blen), cs = cols_smem(ns, blen, C, P);
  if (int rc = set_smem(k_frame_rows, rs, "k_frame_rows")) return rc;
  if (int rc = set_smem(k_pair_cols, cs, "k_pair_cols")) return rc;
  const int fchunk = 2 * ch;
  const int fsub = std::max(1, kShiftDoubles / (2 * J));  // frames per parameter block
  for (int f0 = 0; f0 < F; f0 += fchunk) {
    const int nf = std::min(fchunk, F - f0);
    const int npair = (nf + 1) / 2;
    FramePrepArgs pa{};
    pa.sh_coef = (const float2*)sh_coef;
    pa.sh_freq = g->sh_freq;
    pa.beta = g->beta;
    pa.coef = w.coef;
    pa.mean = w.mean;
    pa.px = w.px;
    pa.py = w.py;
    pa.F = nf;
    pa.L = L;
    pa.J = J;
    pa.P = P;
    pa.ns = ns;
    pa.per_layer = per_layer;
    pa.frame0 = f0;
    pa.df = 1.0 / (ns * g->dx);
    const bool uni = uniform_ok(sx, sy, per_layer, L, f0, nf, ns);
    const bool uni_reg = uni && (ns == 256 || ns == 512 || ns == 1024);
    if (uni_reg) {
      // one prep launch (tables, Nyquist cross, subharmonics) + the fused rows kernel
      if (int rc = launch_uniform_reg_chunk(g, (const float2*)spectra, (const float2*)sh_coef, L,
                                            sx, sy, f0, nf, w, s))
        return rc;
    }
    for (int fb = 0; fb < nf && !uni_reg; fb += fsub) {
      const int nb = std::min(fsub, nf - fb);
      ShiftParams sp;
      for (int f = 0; f < nb; ++f)
        for (int j = 0; j < J; ++j) {
          const int gf = f0 + fb + f;
          const size_t src = per_layer ? (size_t)gf : (size_t)gf * L + j;
          sp.v[(f * J + j) * 2] = sx[src];
          sp.v[(f * J + j) * 2 + 1] = sy[src];
        }
      if (P > 0) {
        k_frame_coef<<<nb, 32 * ((P * 9 + 31) / 32), 0, s>>>(pa, sp, fb, nb);
        count_launch();
      }
      if (uni) continue;  // no phasor tables needed
      ProfScope ps("k_frame_phasors", s);
      k_frame_phasors<<<dim3((ns + 255) / 256, nb * J), 256, 0, s>>>(pa, sp, fb);
      count_launch();
    }
    if (uni_reg) {
      // rows done above
    } else if (uni) {
      if (int rc = launch_uniform_rows(g, (const float2*)spectra, L, sx, sy, f0, nf, w.hn, w.px,
                                       w.img, s))
        return rc;
    } else {
      FrameRowArgs fa{(const float2*)spectra, w.px, w.py, J, nf, f0, per_layer};
      ProfScope ps("k_frame_rows", s);
      k_frame_rows<<<dim3(ns / 2 + 1, npair), kThreads, rs, s>>>(fd, g->tw, fa, w.img);
    }
    count_launch();
    PairStore st{};
    st.out = out + (size_t)f0 * n_out * n_out;
    st.n_out = n_out;
    st.crop = crop;
    st.scale = scale;
    st.accumulate = 0;
    st.count = nf;
    st.re_mul = 2;
    st.re_add = 0;
    st.im_mul = 2;
    st.im_add = 1;
    st.crow_mul = 2;
    st.crow_re = 0;
    st.crow_im = 1;
    st.coef = w.coef;
    st.mean = w.mean;
    st.basis = g->basis;
    st.P = P;
    st.sym = g->sym;
    if (pow2_fast(ns)) {
      if (int rc = pair_cols_reg(g, w.img, npair, 0, st, s)) return rc;
    } else {
      ProfScope ps("k_pair_cols", s);
      k_pair_cols<<<dim3((ns + C - 1) / C, npair), kThreads, cs, s>>>(fd, g->tw, w.img, C, 0,
                                                                     st);
    }
    count_launch();
    if (int rc = check_launch("pt_frames")) return rc;
  }
  return PT_OK;
}

extern "C" int pt_lgs_zoom(int L, int ns, int n, int T, const int32_t* idx, const float* w,
                           const float* screens, float scale, float* out, void* stream) {
  if (L < 1 || ns < 1 || n < 1 || T < 1 || T > 6) return fail(PT_ERR_ARG, "pt_lgs_zoom: bad sizes");
  if (!idx || !w || !screens || !out) return fail(PT_ERR_ARG, "pt_lgs_zoom: NULL pointer");
  cudaStream_t s = (cudaStream_t)stream;
  k_lgs_zoom<<<dim3((n + 127) / 128, n), 128, 0, s>>>(L, ns, n, T, idx, w, screens, scale, out);
  count_launch();
  return check_launch("pt_lgs_zoom");
}

extern "C" int pt_boil_step(const pt_grid* g, int L, float* spectra, float* sh_coef,
                            const float* amplitude, const float* sh_amp, const float* main_tau,
                            const float* sh_tau, double dt, const float* noise,
                            const float* sh_noise, uint64_t seed, uint64_t call, void* stream) {
  if (int rc = check_grid(g, "pt_boil_step")) return rc;
  if (L < 1 || !spectra || !amplitude || !main_tau) return fail(PT_ERR_ARG, "pt_boil_step: bad arguments");
  if (g->P > 0 && (!sh_coef || !sh_amp || !sh_tau)) return fail(PT_ERR_ARG, "pt_boil_step: NULL subharmonic table");
  if (!(dt > 0)) return fail(PT_ERR_ARG, "pt_boil_step: dt must be positive");
  cudaStream_t s = (cudaStream_t)stream;
  const size_t n_main = (size_t)L * g->ns * g->ns;
  k_boil<<<(unsigned)((n_main + 255) / 256), 256, 0, s>>>(n_main, (float2*)spectra, amplitude,
                                                         main_tau, (float)dt, noise, seed, call, 0);
  count_launch();
  if (g->P > 0) {
    const size_t n_sh = (size_t)g->P * L * 9;
    k_boil<<<(unsigned)((n_sh + 127) / 128), 128, 0, s>>>(n_sh, (float2*)sh_coef, sh_amp, sh_tau,
                                                         (float)dt, sh_noise, seed, call,
                                                         1ull << 40);
    count_launch();
  }
  return check_launch("pt_boil_step");
}

// ================================================================ allocation-free inverse FFT
// pt_ifft2_noalloc serves callers that cannot call cudaMalloc: code running
// inside a host framework that owns all device memory, or a process that must
// not grow its footprint after start-up. Its scratch is not a caller
// workspace but a file-scope device array of fixed size, which every GPU that
// loads this library holds until the process exits. Host code cannot use the
// array's name as a device address, so every call resolves the addresses with
// cudaGetSymbolAddress on the current device (a device reset or a rebuilt
// primary context can move the arrays, so an address kept from an earlier
// call could be stale). While the stream is being captured the address from
// the last uncaptured call on that device is used instead; make one call on
// each device before any stream capture. All calls
// share the arrays and the last call's contents stay in them; the row pass
// overwrites every scratch element it later reads and the twiddle table is
// rewritten by each call, so nothing has to start at zero. Calls that
// overlap on the GPU (on different streams or threads) race on the arrays.
#include <mutex>

namespace pt {

constexpr size_t kNoAllocScratchBytes = size_t(8) << 20;  // one 1024^2 complex image
constexpr int kNoAllocMaxN = 1024;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];
static __device__ __align__(256) float2 g_noalloc_tw[kNoAllocMaxN];

struct NoAllocPtrs {
  void* scratch;
  void* tw;
};
constexpr int kNoAllocMaxDevices = 64;
static std::mutex g_noalloc_mu;
static NoAllocPtrs g_noalloc_ptrs[kNoAllocMaxDevices];
static bool g_noalloc_ready[kNoAllocMaxDevices];

static int noalloc_setup(cudaStream_t s, NoAllocPtrs* out) {
  int dev = 0;
  if (int rc = check_cuda(cudaGetDevice(&dev), "pt_ifft2_noalloc: cudaGetDevice")) return rc;
  if (dev < 0 || dev >= kNoAllocMaxDevices)
    return fail(PT_ERR_UNSUPPORTED, "pt_ifft2_noalloc: device index beyond 63");
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (int rc = check_cuda(cudaStreamIsCapturing(s, &cap), "pt_ifft2_noalloc: cudaStreamIsCapturing"))
    return rc;
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (cap == cudaStreamCaptureStatusNone || !g_noalloc_ready[dev]) {
    NoAllocPtrs p{};
    if (int rc = check_cuda(cudaGetSymbolAddress(&p.scratch, g_noalloc_scratch),
                            "pt_ifft2_noalloc: cudaGetSymbolAddress(scratch)"))
      return rc;
    if (int rc = check_cuda(cudaGetSymbolAddress(&p.tw, g_noalloc_tw),
                            "pt_ifft2_noalloc: cudaGetSymbolAddress(twiddles)"))
      return rc;
    g_noalloc_ptrs[dev] = p;
    g_noalloc_ready[dev] = true;
  }
  *out = g_noalloc_ptrs[dev];
  return PT_OK;
}

// exp(+2 pi i k / n) from the FP64 sincospi of the exact fraction k / n
__global__ void k_noalloc_twiddles(float2* tw, int n) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  double s, c;
  sincospi(2.0 * (double)k / (double)n, &s, &c);
  tw[k] = make_float2((float)c, (float)s);
}

}  // namespace pt

extern "C" int pt_ifft2_noalloc(int ns, const float* in, float* out, int batch, void* stream) {
  if (ns < 2 || ns > kNoAllocMaxN)
    return fail(PT_ERR_ARG, "pt_ifft2_noalloc: ns must be in [2, 1024] (fixed 8 MiB scratch)");
  if (!in || !out || batch < 0) return fail(PT_ERR_ARG, "pt_ifft2_noalloc: bad arguments");
  if (batch == 0) return PT_OK;
  NoAllocPtrs p{};
  cudaStream_t s = (cudaStream_t)stream;
  if (int rc = noalloc_setup(s, &p)) return rc;
  pt_grid g{};  // a stack view over the static arrays: nothing is allocated
  g.ns = ns;
  g.dx = 1.0;
  g.P = 0;
  g.desc = make_fft_desc(ns);
  g.tw = (float2*)p.tw;
  float2* scratch = (float2*)p.scratch;
  const size_t per = (size_t)ns * ns;
  // images per pass: what the scratch holds, and at most 65535 (grid y limit)
  const int chunk = (int)std::min<size_t>(
      65535, std::max<size_t>(1, kNoAllocScratchBytes / (per * sizeof(float2))));
  k_noalloc_twiddles<<<(ns + 127) / 128, 128, 0, s>>>(g.tw, ns);
  count_launch();
  const int rpc = rows_per_cta(ns), C = cols_per_cta(ns);  // no Bluestein form here
  const size_t rs = rows_smem(ns, ns, rpc), cs = cols_smem(ns, ns, C, 0);
  if (!pow2_fast(ns)) {
    if (int rc = set_smem(k_rows, rs, "k_rows")) return rc;
    if (int rc = set_smem(k_plain_cols, cs, "k_plain_cols")) return rc;
  }
  GenRowArgs none{};
  for (int b0 = 0; b0 < batch; b0 += chunk) {
    const int nb = std::min(chunk, batch - b0);
    const float2* src = (const float2*)in + (size_t)b0 * per;
    float2* dst = (float2*)out + (size_t)b0 * per;
    if (pow2_fast(ns)) {
      if (int rc = rows_reg(&g, src, 0, none, nb, scratch, s)) return rc;
      if (int rc = plain_cols_reg(&g, scratch, nb, dst, s)) return rc;
    } else {
      k_rows<<<dim3((ns + rpc - 1) / rpc, nb), kThreads, rs, s>>>(g.desc, g.tw, rpc, src, 0, none,
                                                                 scratch);
      k_plain_cols<<<dim3((ns + C - 1) / C, nb), kThreads, cs, s>>>(g.desc, g.tw, scratch, C, dst);
    }
    count_launch(2);
    if (int rc = check_launch("pt_ifft2_noalloc")) return rc;
  }
  return PT_OK;
}

// ------------------------------------------------------------------ translate
// Layer spectra and subharmonic coefficients moved by a displacement per
// layer, out = in * exp(2 pi i (f_x sx[l] + f_y sy[l])): the shift theorem of
// FourierFlowScreen.translate / Atmosphere._integrate (src/pyturb/flow.py:
// 96-129, src/pyturb/atmosphere.py:904-916) applied to the stored state, so
// that frames rendered from the result at displacement s equal frames of the
// original at sx[l] + s. Main-grid phases are exact 64-bit fixed point
// (k' frac(s df) mod 1, fftfreq signs); subharmonic phases are FP64 mod 1.
namespace pt {
constexpr int kMaxTranslateLayers = 64;
struct TranslateArgs {
  uint64_t ux[kMaxTranslateLayers], uy[kMaxTranslateLayers];
  double sx[kMaxTranslateLayers], sy[kMaxTranslateLayers];
};

__global__ void k_translate_spectra(int ns, int L, TranslateArgs a, const float2* __restrict__ in,
                                    float2* __restrict__ out) {
  const size_t npix = (size_t)ns * ns;
  const size_t total = npix * L;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int l = (int)(i / npix);
    const size_t k = i % npix;
    const int kx = (int)(k / ns), ky = (int)(k % ns);
    const int64_t sx = kx <= (ns - 1) / 2 ? kx : kx - ns;
    const int64_t sy = ky <= (ns - 1) / 2 ? ky : ky - ns;
    const uint64_t ph = (uint64_t)sx * a.ux[l] + (uint64_t)sy * a.uy[l];
    out[i] = cmul(in[i], phasor_from_fixed(ph));
  }
}

__global__ void k_translate_sh(int P, int L, TranslateArgs a, const double* __restrict__ sh_freq,
                               const float2* __restrict__ in, float2* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P * L * 9) return;
  const int ij = i % 9, l = (i / 9) % L, p = i / (9 * L);
  const double fi = sh_freq[p * 3 + ij / 3], fk = sh_freq[p * 3 + ij % 3];
  double ph = fi * a.sx[l] + fk * a.sy[l];
  ph -= floor(ph);
  float sn, cs;
  sincospif(2.0f * (float)ph, &sn, &cs);
  out[i] = cmul(in[i], make_float2(cs, sn));
}
}  // namespace pt

// ================================================================ adjoint: subharmonics
// The subharmonic sum of a frame is Re sum_pij C_pij (b_pi(x) b_pj(y) - mean)
// with b_pi(x) = exp(2 pi i f_pi (x - ns/2) dx) (the grid's basis rows). Its
// adjoint needs, per frame f of an upstream gradient g (F, n_out, n_out) on the
// crop window, the projections
//   out[f][((p*3 + i)*3 + j)*2 + {re, im}] = sum_{x,y} g_f(x, y) b_pi(crop + x) b_pj(crop + y)
//   out[f][18 P] = sum_{x,y} g_f(x, y)
// One CTA per frame; thread t owns columns y = t, t + 256, ...; one pass over
// g per level; float sums along x, double products and a fixed-order reduce.
__global__ void __launch_bounds__(256)
k_adj_sh(int ns, int P, int crop, int n_out, const float2* __restrict__ basis,
         const float* __restrict__ g, double* __restrict__ out) {
  __shared__ double red[8][19];
  const int f = blockIdx.x;
  const float* gf = g + (size_t)f * n_out * n_out;
  const size_t stride = (size_t)18 * P + 1;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int p = 0; p < P; ++p) {
    const float2* b0 = basis + (size_t)p * 3 * ns + crop;
    double acc[19];
#pragma unroll
    for (int q = 0; q < 19; ++q) acc[q] = 0.0;
    for (int y = threadIdx.x; y < n_out; y += blockDim.x) {
      float2 u[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
      float sum = 0.f;
      for (int x = 0; x < n_out; ++x) {
        const float v = gf[(size_t)x * n_out + y];
        sum += v;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const float2 b = __ldg(b0 + (size_t)i * ns + x);
          u[i].x = fmaf(b.x, v, u[i].x);
          u[i].y = fmaf(b.y, v, u[i].y);
        }
      }
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const float2 b = __ldg(b0 + (size_t)j * ns + y);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          acc[(i * 3 + j) * 2] += (double)u[i].x * b.x - (double)u[i].y * b.y;
          acc[(i * 3 + j) * 2 + 1] += (double)u[i].x * b.y + (double)u[i].y * b.x;
        }
      }
      acc[18] += sum;
    }
#pragma unroll
    for (int q = 0; q < 19; ++q) {
      double v = acc[q];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) red[warp][q] = v;
    }
    __syncthreads();
    if (threadIdx.x < 19) {
      const int q = threadIdx.x;
      double v = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += red[w][q];
      if (q < 18) out[f * stride + (size_t)p * 18 + q] = v;
      else if (p == 0) out[f * stride + (size_t)18 * P] = v;
    }
    __syncthreads();
  }
}

extern "C" int pt_synth_adj_sh(const pt_grid* g, int F, int crop, int n_out, const float* grad,
                               double* out, void* stream) {
  if (int rc = check_grid(g, "pt_synth_adj_sh")) return rc;
  if (g->P < 1) return fail(PT_ERR_ARG, "pt_synth_adj_sh: the grid has no subharmonic levels");
  if (F < 1 || n_out < 1 || crop < 0 || crop + n_out > g->ns)
    return fail(PT_ERR_ARG, "pt_synth_adj_sh: crop window outside the grid");
  if (!grad || !out) return fail(PT_ERR_ARG, "pt_synth_adj_sh: NULL pointer");
  cudaStream_t s = (cudaStream_t)stream;
  ProfScope ps("k_adj_sh", s);
  k_adj_sh<<<F, 256, 0, s>>>(g->ns, g->P, crop, n_out, g->basis, grad, out);
  count_launch();
  return check_launch("pt_synth_adj_sh");
}

extern "C" int pt_layers_translate(const pt_grid* g, int L, const float* spectra_in,
                                   const float* sh_in, const double* sx, const double* sy,
                                   float* spectra_out, float* sh_out, void* stream) {
  if (int rc = check_grid(g, "pt_layers_translate")) return rc;
  if (L < 1 || L > kMaxTranslateLayers)
    return fail(PT_ERR_ARG, "pt_layers_translate: n_layers must be in [1, 64]");
  if (!spectra_in || !spectra_out || !sx || !sy)
    return fail(PT_ERR_ARG, "pt_layers_translate: NULL pointer");
  if (g->P > 0 && (!sh_in || !sh_out))
    return fail(PT_ERR_ARG, "pt_layers_translate: subharmonic coefficients are NULL");
  TranslateArgs a{};
  const double df = 1.0 / (g->ns * g->dx);
  for (int l = 0; l < L; ++l) {
    if (!std::isfinite(sx[l]) || !std::isfinite(sy[l]))
      return fail(PT_ERR_ARG, "pt_layers_translate: displacement is not finite");
    a.ux[l] = host_fixed(sx[l] * df);
    a.uy[l] = host_fixed(sy[l] * df);
    a.sx[l] = sx[l];
    a.sy[l] = sy[l];
  }
  cudaStream_t s = (cudaStream_t)stream;
  const size_t total = (size_t)g->ns * g->ns * L;
  k_translate_spectra<<<(unsigned)std::min<size_t>((total + 255) / 256, 152 * 16), 256, 0, s>>>(
      g->ns, L, a, (const float2*)spectra_in, (float2*)spectra_out);
  count_launch();
  if (g->P > 0) {
    const int n = g->P * L * 9;
    k_translate_sh<<<(n + 127) / 128, 128, 0, s>>>(g->P, L, a, g->sh_freq,
                                                   (const float2*)sh_in, (float2*)sh_out);
    count_launch();
  }
  return check_launch("pt_layers_translate");
}

// ------------------------------------------------------------------ temporal PSD
// pyturb.analysis.temporal_psd (src/pyturb/analysis.py:183-208): each series
// (samples along the last axis) minus its mean, |DFT|^2 * 2 dt / T, averaged
// over the series. The DFT is the grid's mixed-radix transform of length
// ns = T (|X(f)|^2 of a real series is the same for either sign). CTA b sums
// the power of series b, b + G, ... in shared memory; a second kernel sums
// the G partials in a fixed order.
namespace pt {
__global__ void __launch_bounds__(kThreads)
k_psd_series(FftDesc d, const float2* __restrict__ tw, int count,
             const float* __restrict__ series, float* __restrict__ partial) {
  extern __shared__ float2 sm[];
  __shared__ double red[32];
  const int T = d.n, H = T / 2 + 1, nb = fft_buf_len(d);
  float2* bufA = sm;
  float2* bufB = sm + nb;
  float2* stw = sm + 2 * nb;
  float* acc = (float*)(stw + T);
  for (int i = threadIdx.x; i < T; i += blockDim.x) stw[i] = tw[i];
  for (int f = threadIdx.x; f < H; f += blockDim.x) acc[f] = 0.f;
  for (int s = blockIdx.x; s < count; s += gridDim.x) {
    const float* x = series + (size_t)s * T;
    double m = 0.0;
    for (int i = threadIdx.x; i < T; i += blockDim.x) m += x[i];
    for (int o = 16; o > 0; o >>= 1) m += __shfl_xor_sync(0xffffffffu, m, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    double tot = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
    const float mean = (float)(tot / T);
    for (int i = threadIdx.x; i < T; i += blockDim.x) bufA[i] = make_float2(x[i] - mean, 0.f);
    __syncthreads();
    const float2* res = fft_smem(bufA, bufB, d, stw, 1, nb, 1, false);
    __syncthreads();
    for (int f = threadIdx.x; f < H; f += blockDim.x) {
      const float2 v = res[f];
      acc[f] += v.x * v.x + v.y * v.y;
    }
    __syncthreads();
  }
  for (int f = threadIdx.x; f < H; f += blockDim.x) partial[(size_t)blockIdx.x * H + f] = acc[f];
}

__global__ void k_psd_reduce(int H, int G, double scale, const float* __restrict__ partial,
                             float* __restrict__ psd) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= H) return;
  double s = 0.0;
  for (int b = 0; b < G; ++b) s += partial[(size_t)b * H + f];
  psd[f] = (float)(s * scale);
}

static int psd_blocks(int count) { return std::max(1, std::min(count, 2 * 152)); }
}  // namespace pt

extern "C" size_t pt_temporal_psd_workspace_bytes(const pt_grid* g, int count) {
  if (!g || count < 1) return 0;
  return (size_t)psd_blocks(count) * (g->ns / 2 + 1) * sizeof(float);
}

extern "C" int pt_temporal_psd(const pt_grid* g, int count, const float* series, double dt,
                               float* psd, void* work, size_t work_bytes, void* stream) {
  if (int rc = check_grid(g, "pt_temporal_psd")) return rc;
  if (count < 1 || !(dt > 0)) return fail(PT_ERR_ARG, "pt_temporal_psd: bad count or dt");
  if (!series || !psd) return fail(PT_ERR_ARG, "pt_temporal_psd: NULL pointer");
  if (!work || work_bytes < pt_temporal_psd_workspace_bytes(g, count))
    return fail(PT_ERR_ARG, "pt_temporal_psd: workspace too small");
  const int T = g->ns, H = T / 2 + 1, G = psd_blocks(count);
  const size_t smem = (size_t)(2 * fft_buf_len(g->desc) + T) * sizeof(float2) +
                      (size_t)H * sizeof(float);
  if (smem > 220 * 1024) return fail(PT_ERR_UNSUPPORTED, "pt_temporal_psd: series longer than 8192");
  if (int rc = set_smem(k_psd_series, smem, "k_psd_series")) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  {
    ProfScope ps("k_psd_series", s);
    k_psd_series<<<G, kThreads, smem, s>>>(g->desc, g->tw, count, series, (float*)work);
  }
  k_psd_reduce<<<(H + 127) / 128, 128, 0, s>>>(H, G, 2.0 * dt / T / count, (const float*)work, psd);
  count_launch(2);
  return check_launch("pt_temporal_psd");
}
