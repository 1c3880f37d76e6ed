// Differentiable multi-layer readout: a forward gather and its two adjoints.
//
// Layer screens phi (B, L, S, S) are sampled at the pupil grid of each
// direction and frame and summed with per-layer weights:
//   out[b,t,d,i,j] = sum_l w_l * bilerp(phi[b,l], u_r(i), u_c(j)),
//   u_r(i) = pos0[t,d,l,0] + mag[d,l] * i,   u_c(j) = pos0[t,d,l,1] + mag[d,l] * j,
// with periodic wrap on the S x S screen. This is the cone zoom of
// Atmosphere._build_lgs_zoom / _lgs_zoom (src/pyturb/atmosphere.py:581-616,
// 1048-1090: pupil scaled about the screen centre by mag = 1 - h/H) with the
// frozen-flow + direction displacement of _integrate_lgs (atmosphere.py:
// 1012-1022) applied as a sub-pixel bilinear shift instead of a phase ramp.
//
// Positions are 32.32 fixed point (k_lr_fix), reduced modulo S, so all three
// kernels form bit-identical taps. The adjoints are deterministic: the
// parameter gradients are block reductions written per (band, image), and the
// screen gradient is a gather in which each CTA owns one screen tile and walks
// every (frame, direction) in a fixed order, using the separability of the
// axis-aligned bilinear map (column pass, then row pass).

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>

#include "common.cuh"

namespace pt {
uint64_t* launch_counter();
static inline void count_launch_r(int k = 1) {
  __atomic_add_fetch(launch_counter(), (uint64_t)k, __ATOMIC_RELAXED);
}

constexpr int kLrMaxLayers = 32;
constexpr int kLrMaxMag = 256;   // D * L entries of the magnification table
constexpr int kLrBand = 64;      // pupil rows per CTA (forward, parameter gradients)
constexpr int kLrTile = 64;      // screen tile width (screen gradient); height TR = 64 or 128
constexpr long long kLrOne = 1ll << 32;

struct LrMag {
  double m[kLrMaxMag];
};

// fix[(t*D + d)*L + l] = {p0r, p0c, m}: positions of pupil pixel (0, 0)
// reduced into [0, S) and the per-pixel step, in units of 2^-32 px.
__global__ void k_lr_fix(int T, int D, int L, int S, const double* __restrict__ pos0, LrMag mag,
                         long long* __restrict__ fix) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= T * D * L) return;
  const int l = k % L, d = (k / L) % D;
  const long long span = (long long)S * kLrOne;
  long long out[2];
#pragma unroll
  for (int a = 0; a < 2; ++a) {
    const double p = pos0[2 * k + a];
    const double x = p - floor(p / S) * (double)S;
    long long v = llrint(ldexp(x, 32));
    if (v < 0) v += span;
    if (v >= span) v -= span;
    out[a] = v;
  }
  fix[3 * k + 0] = out[0];
  fix[3 * k + 1] = out[1];
  fix[3 * k + 2] = llrint(ldexp(mag.m[d * L + l], 32));
}

// One axis tap: u = p0 + i*m (p0 in [0, S), m*(n-1) < S - 2, so u < 2S).
struct Tap {
  int a0, a1;
  float f;
};
__device__ __forceinline__ Tap lr_tap(long long p0, long long m, int i, int S) {
  const long long u = p0 + (long long)i * m;
  int i0 = (int)(u >> 32);
  if (i0 >= S) i0 -= S;
  Tap t;
  t.a0 = i0;
  t.a1 = (i0 + 1 == S) ? 0 : i0 + 1;
  t.f = (float)(uint32_t)(u & 0xffffffffll) * 2.3283064365386963e-10f;
  return t;
}

struct RowTab {
  int o0, o1;  // row offsets (row * S)
  float f;
};

// Forward: CTA = (band of kLrBand pupil rows, t*D + d, b); threads walk
// columns, layers, then rows of the band.
template <int LM>
__global__ void __launch_bounds__(256)
k_lr_forward(int L, int S, int T, int D, int n, const float* __restrict__ screens,
             const float* __restrict__ w, const long long* __restrict__ fix,
             float* __restrict__ out) {
  __shared__ RowTab rt[LM][kLrBand];
  const int band0 = blockIdx.x * kLrBand;
  const int td = blockIdx.y, b = blockIdx.z;
  const int rows = min(kLrBand, n - band0);
  const long long* fx = fix + (size_t)td * L * 3;
  for (int k = threadIdx.x; k < L * kLrBand; k += blockDim.x) {
    const int l = k / kLrBand, r = k % kLrBand;
    const Tap t = lr_tap(fx[3 * l], fx[3 * l + 2], band0 + r, S);
    rt[l][r] = RowTab{t.a0 * S, t.a1 * S, t.f};
  }
  __syncthreads();
  const float* scr = screens + (size_t)b * L * S * S;
  float* o = out + ((size_t)b * T * D + td) * n * n + (size_t)band0 * n;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    Tap c[LM];
#pragma unroll
    for (int l = 0; l < LM; ++l)
      if (l < L) c[l] = lr_tap(fx[3 * l + 1], fx[3 * l + 2], j, S);
    for (int r = 0; r < rows; ++r) {
      float acc = 0.f;
#pragma unroll
      for (int l = 0; l < LM; ++l) {
        if (l < L) {
          const float* sl = scr + (size_t)l * S * S;
          const RowTab q = rt[l][r];
          const float v00 = __ldg(sl + q.o0 + c[l].a0), v01 = __ldg(sl + q.o0 + c[l].a1);
          const float v10 = __ldg(sl + q.o1 + c[l].a0), v11 = __ldg(sl + q.o1 + c[l].a1);
          const float top = fmaf(c[l].f, v01 - v00, v00);
          const float bot = fmaf(c[l].f, v11 - v10, v10);
          acc = fmaf(__ldg(w + l), fmaf(q.f, bot - top, top), acc);
        }
      }
      o[(size_t)r * n + j] = acc;
    }
  }
}

// Parameter gradients: per (band, image) and layer, the sums over the band's
// pixels of g * val, g * w * d val / d u_r and g * w * d val / d u_c (the
// derivative of the bilinear cell the sample lies in). Layers go in groups of
// kLrGroup so that taps and accumulators stay in few registers; the band of g
// is re-read from L2 once per group.
constexpr int kLrGroup = 4;
__global__ void __launch_bounds__(256)
k_lr_grad_params(int L, int S, int T, int D, int n, const float* __restrict__ screens,
                 const float* __restrict__ w, const long long* __restrict__ fix,
                 const float* __restrict__ g, float* __restrict__ partial) {
  __shared__ RowTab rt[kLrMaxLayers][kLrBand];
  __shared__ float red[8][3 * kLrGroup];
  const int band0 = blockIdx.x * kLrBand;
  const int td = blockIdx.y, b = blockIdx.z;
  const int rows = min(kLrBand, n - band0);
  const long long* fx = fix + (size_t)td * L * 3;
  for (int k = threadIdx.x; k < L * kLrBand; k += blockDim.x) {
    const int l = k / kLrBand, r = k % kLrBand;
    const Tap t = lr_tap(fx[3 * l], fx[3 * l + 2], band0 + r, S);
    rt[l][r] = RowTab{t.a0 * S, t.a1 * S, t.f};
  }
  __syncthreads();
  const float* scr = screens + (size_t)b * L * S * S;
  const float* gi = g + ((size_t)b * T * D + td) * n * n + (size_t)band0 * n;
  const int nb = gridDim.x;
  float* pp = partial + (((size_t)b * T * D + td) * nb + blockIdx.x) * L * 3;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int l0 = 0; l0 < L; l0 += kLrGroup) {
    float sv[kLrGroup], sr[kLrGroup], sc[kLrGroup];
#pragma unroll
    for (int q = 0; q < kLrGroup; ++q) sv[q] = sr[q] = sc[q] = 0.f;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
      Tap c[kLrGroup];
#pragma unroll
      for (int q = 0; q < kLrGroup; ++q)
        if (l0 + q < L) c[q] = lr_tap(fx[3 * (l0 + q) + 1], fx[3 * (l0 + q) + 2], j, S);
      for (int r = 0; r < rows; ++r) {
        const float gv = gi[(size_t)r * n + j];
#pragma unroll
        for (int q = 0; q < kLrGroup; ++q) {
          if (l0 + q < L) {
            const float* sl = scr + (size_t)(l0 + q) * S * S;
            const RowTab t = rt[l0 + q][r];
            const float v00 = __ldg(sl + t.o0 + c[q].a0), v01 = __ldg(sl + t.o0 + c[q].a1);
            const float v10 = __ldg(sl + t.o1 + c[q].a0), v11 = __ldg(sl + t.o1 + c[q].a1);
            const float dtop = v01 - v00, dbot = v11 - v10;
            const float top = fmaf(c[q].f, dtop, v00);
            const float bot = fmaf(c[q].f, dbot, v10);
            sv[q] = fmaf(gv, fmaf(t.f, bot - top, top), sv[q]);
            sr[q] = fmaf(gv, bot - top, sr[q]);
            sc[q] = fmaf(gv, fmaf(t.f, dbot - dtop, dtop), sc[q]);
          }
        }
      }
    }
#pragma unroll
    for (int q = 0; q < kLrGroup; ++q) {
      float a = sv[q], r = sr[q], c = sc[q];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        r += __shfl_xor_sync(0xffffffffu, r, o);
        c += __shfl_xor_sync(0xffffffffu, c, o);
      }
      if (lane == 0) {
        red[warp][3 * q] = a;
        red[warp][3 * q + 1] = r;
        red[warp][3 * q + 2] = c;
      }
    }
    __syncthreads();
    if (threadIdx.x < 3 * kLrGroup) {
      const int k = threadIdx.x, l = l0 + k / 3;
      if (l < L) {
        float s = 0.f;
        for (int q = 0; q < 8; ++q) s += red[q][k];
        pp[3 * l + k % 3] = (k % 3 == 0) ? s : s * w[l];
      }
    }
    __syncthreads();
  }
}

// First pupil index x with p0 + x*m > a (m > 0): a float estimate (|x| < 2^17,
// so off by less than one) corrected with exact 64-bit products, so the result
// equals the integer floor form. FP32 keeps it off the slow FP64 pipe.
__device__ __forceinline__ long long first_above(long long a, long long p0, long long m,
                                                 float inv_m) {
  long long x = (long long)floorf((float)(a - p0) * inv_m) + 1;
  if (p0 + (x - 1) * m > a) --x;
  if (p0 + x * m <= a) ++x;
  return x;
}

// Screen gradient: CTA = (screen tile of TR rows x 64 columns, layer, b). For
// each (t, d) and each wrap image of the tile window, the pupil block that
// reaches the tile is staged in shared memory, spread along columns into the
// tile's columns, then along rows into the tile's pixels, accumulated in
// registers in a fixed order and written once (times w_l, or added). KM
// bounds the pupil samples whose bilinear footprint covers one screen pixel
// along one axis: ceil(2 / mag); ymaxR / ymaxC bound the block's rows /
// columns. With vec (n a multiple of 4 and g 16-byte aligned) the block is
// staged with 16-byte copies from the 4-float boundary at or below its first
// column (sh floats of lead-in); otherwise with 4-byte copies (sh = 0). The
// stage row stride is ystr = ymaxC + 4 rounded up to a multiple of 4.
template <int KM, int TR>
__global__ void __launch_bounds__(256)
k_lr_grad_screens(int L, int S, int T, int D, int n, int tiles_c, int ymaxR, int ymaxC, int ystr,
                  int vec, const float* __restrict__ w, const long long* __restrict__ fix,
                  const float* __restrict__ g, int accumulate, float* __restrict__ grad) {
  constexpr int NQ = TR / 4;                     // pixels a thread accumulates
  extern __shared__ float smx[];
  float* gsm = smx;                              // ymaxR * ystr (16-byte aligned rows)
  float* hsm = gsm + (size_t)ymaxR * ystr;       // ymaxR * kLrTile
  float* rw = hsm + (size_t)ymaxR * kLrTile;     // TR * KM row weights
  int* rk = (int*)(rw + TR * KM);                // TR * KM: clamped hsm offsets of the taps
  const int tile_c = blockIdx.x % tiles_c, tile_r = blockIdx.x / tiles_c;
  const int l = blockIdx.y, b = blockIdx.z;
  const int R0 = tile_r * TR, C0 = tile_c * kLrTile;
  const int TH = min(TR, S - R0), TW = min(kLrTile, S - C0);
  const int pc = threadIdx.x & (kLrTile - 1), pq = threadIdx.x >> 6;  // 4 row groups
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long span = (long long)S * kLrOne;
  float acc[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) acc[q] = 0.f;
  for (int td = 0; td < T * D; ++td) {
    const long long* fx = fix + ((size_t)td * L + l) * 3;
    const long long p0r = fx[0], p0c = fx[1], m = fx[2];
    const float inv_m = 1.0f / (float)m;
    const long long ur1 = p0r + (long long)(n - 1) * m, uc1 = p0c + (long long)(n - 1) * m;
    const float* gi = g + ((size_t)b * T * D + td) * n * n;
    for (int kr = 0; kr < 2; ++kr) {
      // u_r values reaching tile rows [R0, R0 + TH): the open window (R0 - 1, R0 + TH) + kr S
      const long long wr0 = (long long)(R0 - 1) * kLrOne + kr * span;
      const long long wr1 = (long long)(R0 + TH) * kLrOne + kr * span;
      if (!(wr0 < ur1 && wr1 > p0r)) continue;
      const int ylo = (int)max(0ll, first_above(wr0, p0r, m, inv_m));
      const int yhi = (int)min((long long)n, first_above(wr1 - 1, p0r, m, inv_m));  // exclusive
      const int ny = min(yhi - ylo, ymaxR);  // the min cannot bind: ymaxR bounds the window
      if (ny <= 0) continue;
      for (int kc = 0; kc < 2; ++kc) {
        const long long wc0 = (long long)(C0 - 1) * kLrOne + kc * span;
        const long long wc1 = (long long)(C0 + TW) * kLrOne + kc * span;
        if (!(wc0 < uc1 && wc1 > p0c)) continue;
        const int xlo = (int)max(0ll, first_above(wc0, p0c, m, inv_m));
        const int xhi = (int)min((long long)n, first_above(wc1 - 1, p0c, m, inv_m));
        const int nx = min(xhi - xlo, ymaxC);
        if (nx <= 0) continue;
        const int sh = vec ? (xlo & 3) : 0;  // lead-in floats before xlo in a stage row
        // this thread's column taps (registers) as stage-row offsets
        float cwt[KM];
        int ci[KM];
        {
          const long long pf = (long long)(C0 + pc) * kLrOne + kc * span;
          const long long xa = first_above(pf - kLrOne, p0c, m, inv_m);
#pragma unroll
          for (int k = 0; k < KM; ++k) {
            const long long x = xa + k;
            const long long dl = p0c + x * m - pf;
            const long long ad = dl < 0 ? -dl : dl;
            const bool in = pc < TW && ad < kLrOne && x >= xlo && x < xlo + nx;
            cwt[k] = in ? 1.f - (float)ad * 2.3283064365386963e-10f : 0.f;
            ci[k] = sh + min(max((int)(x - xlo), 0), nx - 1);
          }
        }
        // row taps of the tile (shared): weights and clamped hsm offsets
        if (threadIdx.x < TR) {
          const int p = threadIdx.x;
          const long long pf = (long long)(R0 + p) * kLrOne + kr * span;
          const long long ya = first_above(pf - kLrOne, p0r, m, inv_m);
#pragma unroll
          for (int k = 0; k < KM; ++k) {
            const long long y = ya + k;
            const long long dl = p0r + y * m - pf;
            const long long ad = dl < 0 ? -dl : dl;
            const bool in = p < TH && ad < kLrOne && y >= ylo && y < ylo + ny;
            rw[p * KM + k] = in ? 1.f - (float)ad * 2.3283064365386963e-10f : 0.f;
            rk[p * KM + k] = min(max((int)(y - ylo), 0), ny - 1) * kLrTile;
          }
        }
        // stage the pupil block with asynchronous copies (all of a thread's
        // copies in flight at once, one wait)
        if (vec) {
          const int nq = (sh + nx + 3) >> 2;  // 16-byte pieces a row; ends at or before n
          for (int e = threadIdx.x; e < ny * nq; e += blockDim.x) {
            const int yy = e / nq, xq = e - yy * nq;
            const float* src = gi + (size_t)(ylo + yy) * n + (xlo - sh) + 4 * xq;
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                             (uint32_t)__cvta_generic_to_shared(gsm + yy * ystr + 4 * xq)),
                         "l"(src)
                         : "memory");
          }
        } else {
          for (int yy = warp; yy < ny; yy += 8) {
            const float* src = gi + (size_t)(ylo + yy) * n + xlo;
            for (int xx = lane; xx < nx; xx += 32) {
              asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(
                               (uint32_t)__cvta_generic_to_shared(gsm + yy * ystr + xx)),
                           "l"(src + xx)
                           : "memory");
            }
          }
        }
        asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
        __syncthreads();
        // column pass: h[yy][pc] = sum_k cwt[k] g[yy][ci[k]]
        for (int yy = pq; yy < ny; yy += 4) {
          const float* row = gsm + yy * ystr;
          float h = 0.f;
#pragma unroll
          for (int k = 0; k < KM; ++k) h = fmaf(cwt[k], row[ci[k]], h);
          hsm[yy * kLrTile + pc] = h;
        }
        __syncthreads();
        // row pass into the thread's NQ pixels
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
          const int r = pq + 4 * q;
          float sacc = acc[q];
#pragma unroll
          for (int k = 0; k < KM; ++k) sacc = fmaf(rw[r * KM + k], hsm[rk[r * KM + k] + pc], sacc);
          acc[q] = sacc;
        }
        __syncthreads();
      }
    }
  }
  const float wl = w[l];
  float* gl = grad + ((size_t)b * L + l) * S * S;
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    const int r = pq + 4 * q;
    if (r < TH && pc < TW) {
      float* o = gl + (size_t)(R0 + r) * S + C0 + pc;
      *o = accumulate ? *o + wl * acc[q] : wl * acc[q];
    }
  }
}

// ----------------------------------------------------------------- host side
static int lr_check(const char* who, int B, int L, int S, int T, int D, int n, const double* mag) {
  if (B < 1 || L < 1 || S < 2 || T < 1 || D < 1 || n < 1)
    return fail(PT_ERR_ARG, std::string(who) + ": bad sizes");
  if (L > kLrMaxLayers) return fail(PT_ERR_UNSUPPORTED, std::string(who) + ": at most 32 layers");
  if (D * L > kLrMaxMag)
    return fail(PT_ERR_UNSUPPORTED, std::string(who) + ": at most 256 direction-layer pairs");
  if (S > (1 << 20) || n > (1 << 16))
    return fail(PT_ERR_UNSUPPORTED, std::string(who) + ": screen or pupil too large");
  if (!mag) return fail(PT_ERR_ARG, std::string(who) + ": NULL magnification table");
  for (int k = 0; k < D * L; ++k) {
    const double m = mag[k];
    if (!(m >= 0.25 && m <= 4.0))
      return fail(PT_ERR_ARG, std::string(who) + ": magnification must lie in [0.25, 4]");
    if (!(m * (n - 1) + 2.0 < S))
      return fail(PT_ERR_ARG, std::string(who) + ": the pupil footprint must be smaller than the screen");
  }
  return PT_OK;
}

}  // namespace pt

using namespace pt;

extern "C" int pt_lr_fix(int T, int D, int L, int S, int n, const double* pos0, const double* mag,
                         int64_t* fix, void* stream) {
  if (int rc = lr_check("pt_lr_fix", 1, L, S, T, D, n, mag)) return rc;
  if (!pos0 || !fix) return fail(PT_ERR_ARG, "pt_lr_fix: NULL pointer");
  LrMag M{};
  for (int k = 0; k < D * L; ++k) M.m[k] = mag[k];
  cudaStream_t s = (cudaStream_t)stream;
  const int cnt = T * D * L;
  k_lr_fix<<<(cnt + 255) / 256, 256, 0, s>>>(T, D, L, S, pos0, M, (long long*)fix);
  count_launch_r();
  return check_launch("pt_lr_fix");
}

extern "C" int pt_lr_forward(int B, int L, int S, int T, int D, int n, const double* mag,
                             const float* screens, const float* weights, const int64_t* fix,
                             float* out, void* stream) {
  if (int rc = lr_check("pt_lr_forward", B, L, S, T, D, n, mag)) return rc;
  if (!screens || !weights || !fix || !out) return fail(PT_ERR_ARG, "pt_lr_forward: NULL pointer");
  if ((long long)T * D > 65535 || B > 65535)
    return fail(PT_ERR_UNSUPPORTED, "pt_lr_forward: T*D and B must be <= 65535");
  cudaStream_t s = (cudaStream_t)stream;
  dim3 grid((n + kLrBand - 1) / kLrBand, T * D, B);
  const long long* fx = (const long long*)fix;
  ProfScope ps("k_lr_forward", s);
  if (L <= 4) k_lr_forward<4><<<grid, 256, 0, s>>>(L, S, T, D, n, screens, weights, fx, out);
  else if (L <= 8) k_lr_forward<8><<<grid, 256, 0, s>>>(L, S, T, D, n, screens, weights, fx, out);
  else if (L <= 12) k_lr_forward<12><<<grid, 256, 0, s>>>(L, S, T, D, n, screens, weights, fx, out);
  else if (L <= 16) k_lr_forward<16><<<grid, 256, 0, s>>>(L, S, T, D, n, screens, weights, fx, out);
  else k_lr_forward<32><<<grid, 256, 0, s>>>(L, S, T, D, n, screens, weights, fx, out);
  count_launch_r();
  return check_launch("pt_lr_forward");
}

extern "C" int pt_lr_grad_params(int B, int L, int S, int T, int D, int n, const double* mag,
                                 const float* screens, const float* weights, const int64_t* fix,
                                 const float* grad_out, float* partial, void* stream) {
  if (int rc = lr_check("pt_lr_grad_params", B, L, S, T, D, n, mag)) return rc;
  if (!screens || !weights || !fix || !grad_out || !partial)
    return fail(PT_ERR_ARG, "pt_lr_grad_params: NULL pointer");
  if ((long long)T * D > 65535 || B > 65535)
    return fail(PT_ERR_UNSUPPORTED, "pt_lr_grad_params: T*D and B must be <= 65535");
  cudaStream_t s = (cudaStream_t)stream;
  dim3 grid((n + kLrBand - 1) / kLrBand, T * D, B);
  const long long* fx = (const long long*)fix;
  ProfScope ps("k_lr_grad_params", s);
k_lr_grad_params<<<grid, 256, 0, s>>>(L, S, T, D, n, screens, weights, fx, grad_out, partial);
  count_launch_r();
  return check_launch("pt_lr_grad_params");
}

extern "C" size_t pt_lr_partial_count(int B, int L, int T, int D, int n) {
  if (B < 1 || L < 1 || T < 1 || D < 1 || n < 1) return 0;
  return (size_t)B * T * D * ((n + kLrBand - 1) / kLrBand) * L * 3;
}

extern "C" int pt_lr_grad_screens(int B, int L, int S, int T, int D, int n, const double* mag,
                                  const float* weights, const int64_t* fix, const float* grad_out,
                                  int accumulate, float* grad_screens, void* stream) {
  if (int rc = lr_check("pt_lr_grad_screens", B, L, S, T, D, n, mag)) return rc;
  if (!weights || !fix || !grad_out || !grad_screens)
    return fail(PT_ERR_ARG, "pt_lr_grad_screens: NULL pointer");
  double mmin = 4.0;
  for (int k = 0; k < D * L; ++k) mmin = std::min(mmin, mag[k]);
  // pupil samples reaching an open window of E + 1 screen pixels: at most
  // ceil((E + 1) / mag); taps per screen pixel and axis: ceil(2 / mag)
  const int km = (int)std::ceil(2.0 / mmin);
  if (km > 8) return fail(PT_ERR_UNSUPPORTED, "pt_lr_grad_screens: magnification too small");
  const int KM = km <= 2 ? 2 : km <= 3 ? 3 : km <= 4 ? 4 : 8;
  const int ymaxC = (int)std::ceil((kLrTile + 1) / mmin) + 1;
  const int ystr = ((ymaxC + 4) + 3) & ~3;
  const int vec = (n % 4 == 0) && ((uintptr_t)grad_out % 16 == 0);
  auto smem_for = [&](int TR, int ymaxR) {
    return sizeof(float) * ((size_t)ymaxR * ystr + (size_t)ymaxR * kLrTile + (size_t)TR * KM) +
           (size_t)TR * KM * sizeof(int);
  };
  // tiles 128 high when two CTAs still fit an SM (per-tile work amortises the
  // per-(t, d) window and tap set-up), else 64
  int TR = 128, ymaxR = (int)std::ceil((128 + 1) / mmin) + 1;
  if (smem_for(TR, ymaxR) > 110 * 1024) {
    TR = 64;
    ymaxR = ymaxC;
  }
  const size_t smem = smem_for(TR, ymaxR);
  if (smem > 200 * 1024) return fail(PT_ERR_UNSUPPORTED, "pt_lr_grad_screens: magnification too small");
  if (B > 65535) return fail(PT_ERR_UNSUPPORTED, "pt_lr_grad_screens: B must be <= 65535");
  cudaStream_t s = (cudaStream_t)stream;
  const int tiles_c = (S + kLrTile - 1) / kLrTile, tiles_r = (S + TR - 1) / TR;
  dim3 grid(tiles_r * tiles_c, L, B);
  const long long* fx = (const long long*)fix;
  ProfScope ps("k_lr_grad_screens", s);
#define PT_LR_GS(KMV, TRV)                                                                     \
  do {                                                                                         \
    static bool attr = false;                                                                  \
    if (!attr) {                                                                               \
      if (int rc = check_cuda(cudaFuncSetAttribute(k_lr_grad_screens<KMV, TRV>,                \
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                                   200 * 1024), "pt_lr_grad_screens"))        \
        return rc;                                                                             \
      attr = true;                                                                             \
    }                                                                                          \
    k_lr_grad_screens<KMV, TRV><<<grid, 256, smem, s>>>(L, S, T, D, n, tiles_c, ymaxR, ymaxC,  \
                                                        ystr, vec, weights, fx, grad_out,      \
                                                        accumulate, grad_screens);             \
  } while (0)
  if (TR == 128) {
    if (KM == 2) PT_LR_GS(2, 128);
    else if (KM == 3) PT_LR_GS(3, 128);
    else if (KM == 4) PT_LR_GS(4, 128);
    else PT_LR_GS(8, 128);
  } else {
    if (KM == 2) PT_LR_GS(2, 64);
    else if (KM == 3) PT_LR_GS(3, 64);
    else if (KM == 4) PT_LR_GS(4, 64);
    else PT_LR_GS(8, 64);
  }
#undef PT_LR_GS
  count_launch_r();
  return check_launch("pt_lr_grad_screens");
}
