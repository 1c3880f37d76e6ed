// Adjoint of the spectral frame synthesis (no counterpart in the reference,
// which has no gradients). The forward is pt_frames without subharmonics:
//   y_f = scale * crop( Re sum_k X_f(k) e^{2 pi i k.x / ns} ),
//   X_f = sum_l w_l S_l(k) Phi_lf(k),  Phi_lf = e^{2 pi i (fx sx[f,l] + fy sy[f,l])}
// (Atmosphere._integrate, src/pyturb/atmosphere.py:882-938; fx along axis 0,
// fftfreq(ns, dx) with index ns/2 at -ns/2 as in the reference). For a real
// loss with upstream gradient g_f,
//   dL/dX_f = scale * DFT(pad(g_f))  (unnormalised forward DFT),
// obtained from the inverse transform as conj(IDFT(conj(z))) on the pair
// z = g_2p + i g_2p+1, whose two frames separate by Hermitian parts. Then
//   dL/dS_l  = w_l sum_f G_f conj(Phi_lf)                      (conjugate ramp)
//   dL/dw_l  = sum_f sum_k Re(conj(G_f) S_l Phi_lf)
//   dL/dsx_fl = -2 pi w_l sum_k fx Im(conj(G_f) S_l Phi_lf)    (ramp derivative)
// Phases are 64-bit fixed point as in the forward, so the adjoint ramps are
// the forward's.

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>

#include "common.cuh"

namespace pt {
uint64_t* launch_counter();
static inline void count_launch_a(int k = 1) {
  __atomic_add_fetch(launch_counter(), (uint64_t)k, __ATOMIC_RELAXED);
}

__device__ __forceinline__ int signed_freq(int k, int ns) { return k <= (ns - 1) / 2 ? k : k - ns; }

// z[p] = scale * conj(g[2p] + i g[2p+1]) placed at (crop, crop) of an ns x ns image.
__global__ void k_adj_pack(int ns, int F, int crop, int n_out, float scale,
                           const float* __restrict__ g, float2* __restrict__ z) {
  const int p = blockIdx.y;
  const size_t npix = (size_t)ns * ns;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < npix;
       k += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(k / ns), c = (int)(k % ns);
    const int i = r - crop, j = c - crop;
    float a = 0.f, b = 0.f;
    if (i >= 0 && i < n_out && j >= 0 && j < n_out) {
      a = g[((size_t)(2 * p) * n_out + i) * n_out + j];
      if (2 * p + 1 < F) b = g[((size_t)(2 * p + 1) * n_out + i) * n_out + j];
    }
    z[(size_t)p * npix + k] = make_float2(scale * a, -scale * b);
  }
}

// ph[((l * F + f) * 2 + a) * ns + k] = exp(2 pi i ks(k) s_a[f, l] / (ns dx)), a = 0: sx, 1: sy.
__global__ void k_adj_phasors(int ns, double df, int L, int F, const double* __restrict__ sx,
                              const double* __restrict__ sy, float2* __restrict__ ph) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t total = (size_t)L * F * 2 * ns;
  if (idx >= total) return;
  const int k = (int)(idx % ns);
  const int a = (int)((idx / ns) % 2);
  const int lf = (int)(idx / (2 * (size_t)ns));
  const int l = lf / F, f = lf % F;
  const double s = (a == 0 ? sx : sy)[(size_t)f * L + l];
  const uint64_t u = phase_fixed(s * df);
  ph[idx] = phasor_from_fixed((uint64_t)(int64_t)signed_freq(k, ns) * u);
}

// The two frames' gradients G_a (frame 2p) and G_b (frame 2p+1) at k from the
// transformed pair Z = IDFT(conj z): D = conj(Z), G_a = (D(k) + conj D(-k))/2,
// G_b = (D(k) - conj D(-k)) / 2i.
__device__ __forceinline__ void split_pair(float2 zk, float2 zn, float2& ga, float2& gb) {
  const float2 dk = make_float2(zk.x, -zk.y);       // D(k)
  const float2 cdn = zn;                              // conj D(-k) = Z(-k)
  ga = make_float2(0.5f * (dk.x + cdn.x), 0.5f * (dk.y + cdn.y));
  const float2 d = make_float2(dk.x - cdn.x, dk.y - cdn.y);
  gb = make_float2(0.5f * d.y, -0.5f * d.x);         // d / 2i
}

// grad_S[l][k] (+)= w_l sum_f G_f(k) conj(Phi_lf(k)).
__global__ void k_adj_spectra(int ns, int L, int F, const float* __restrict__ w,
                              const float2* __restrict__ Z, const float2* __restrict__ ph,
                              int accumulate, float2* __restrict__ gs) {
  const size_t npix = (size_t)ns * ns;
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int l = blockIdx.y;
  if (k >= npix) return;
  const int kr = (int)(k / ns), kc = (int)(k % ns);
  const size_t nk = (size_t)((ns - kr) % ns) * ns + (ns - kc) % ns;
  const int P2 = (F + 1) / 2;
  float2 acc = make_float2(0.f, 0.f);
  for (int p = 0; p < P2; ++p) {
    float2 ga, gb;
    split_pair(Z[(size_t)p * npix + k], Z[(size_t)p * npix + nk], ga, gb);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int f = 2 * p + h;
      if (f >= F) break;
      const float2* pf = ph + ((size_t)l * F + f) * 2 * ns;
      const float2 phi = cmul(pf[kr], pf[ns + kc]);
      acc = cfma(h == 0 ? ga : gb, cconj(phi), acc);
    }
  }
  float2 v = cscale(acc, w[l]);
  if (accumulate) {
    const float2 o = gs[(size_t)l * npix + k];
    v = make_float2(o.x + v.x, o.y + v.y);
  }
  gs[(size_t)l * npix + k] = v;
}

// Per (layer, frame pair): [sum Re q, -2 pi w sum fx Im q, -2 pi w sum fy Im q]
// with q = conj(G_f) S_l Phi_lf, for both frames of the pair, in float64.
__global__ void __launch_bounds__(256)
k_adj_params(int ns, double df, int L, int F, const float* __restrict__ w,
             const float2* __restrict__ spectra, const float2* __restrict__ Z,
             const float2* __restrict__ ph, double* __restrict__ out) {
  __shared__ double red[8][6];
  const int l = blockIdx.x, p = blockIdx.y;
  const size_t npix = (size_t)ns * ns;
  const float2* S = spectra + (size_t)l * npix;
  const float2* Zp = Z + (size_t)p * npix;
  const bool two = 2 * p + 1 < F;
  const float2* p0 = ph + ((size_t)l * F + 2 * p) * 2 * ns;
  const float2* p1 = two ? p0 + 2 * ns : p0;
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (size_t k = threadIdx.x; k < npix; k += blockDim.x) {
    const int kr = (int)(k / ns), kc = (int)(k % ns);
    const size_t nk = (size_t)((ns - kr) % ns) * ns + (ns - kc) % ns;
    float2 ga, gb;
    split_pair(Zp[k], Zp[nk], ga, gb);
    const float2 s = S[k];
    const float fxr = (float)signed_freq(kr, ns), fyc = (float)signed_freq(kc, ns);
    const float2 q0 = cmul(cconj(ga), cmul(s, cmul(p0[kr], p0[ns + kc])));
    acc[0] += q0.x;
    acc[1] += fxr * q0.y;
    acc[2] += fyc * q0.y;
    if (two) {
      const float2 q1 = cmul(cconj(gb), cmul(s, cmul(p1[kr], p1[ns + kc])));
      acc[3] += q1.x;
      acc[4] += fxr * q1.y;
      acc[5] += fyc * q1.y;
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    double v = acc[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp][i] = v;
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    const int i = threadIdx.x;
    double v = 0.0;
    for (int q = 0; q < 8; ++q) v += red[q][i];
    const int h = i / 3, c = i % 3;
    const int f = 2 * p + h;
    if (f < F) {
      const double ramp = -2.0 * M_PI * df * (double)w[l];
      out[((size_t)l * F + f) * 3 + c] = c == 0 ? v : v * ramp;
    }
  }
}

}  // namespace pt

using namespace pt;

extern "C" int pt_synth_adj_pack(int ns, int F, int crop, int n_out, float scale, const float* g,
                                 float* z, void* stream) {
  if (ns < 2 || F < 1 || n_out < 1 || crop < 0 || crop + n_out > ns)
    return fail(PT_ERR_ARG, "pt_synth_adj_pack: bad sizes");
  if (!g || !z) return fail(PT_ERR_ARG, "pt_synth_adj_pack: NULL pointer");
  const int P2 = (F + 1) / 2;
  if (P2 > 65535) return fail(PT_ERR_UNSUPPORTED, "pt_synth_adj_pack: too many frames");
  cudaStream_t s = (cudaStream_t)stream;
  const size_t npix = (size_t)ns * ns;
  const int blocks = (int)std::min<size_t>((npix + 255) / 256, 4096);
  k_adj_pack<<<dim3(blocks, P2), 256, 0, s>>>(ns, F, crop, n_out, scale, g, (float2*)z);
  count_launch_a();
  return check_launch("pt_synth_adj_pack");
}

extern "C" int pt_synth_adj_phasors(int ns, double pixel_scale, int L, int F, const double* sx,
                                    const double* sy, float* ph, void* stream) {
  if (ns < 2 || L < 1 || F < 1 || !(pixel_scale > 0))
    return fail(PT_ERR_ARG, "pt_synth_adj_phasors: bad sizes");
  if (!sx || !sy || !ph) return fail(PT_ERR_ARG, "pt_synth_adj_phasors: NULL pointer");
  cudaStream_t s = (cudaStream_t)stream;
  const size_t total = (size_t)L * F * 2 * ns;
  k_adj_phasors<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(
      ns, 1.0 / (ns * pixel_scale), L, F, sx, sy, (float2*)ph);
  count_launch_a();
  return check_launch("pt_synth_adj_phasors");
}

extern "C" int pt_synth_adj_spectra(int ns, int L, int F, const float* w, const float* Z,
                                    const float* ph, int accumulate, float* grad_spectra,
                                    void* stream) {
  if (ns < 2 || L < 1 || F < 1) return fail(PT_ERR_ARG, "pt_synth_adj_spectra: bad sizes");
  if (!w || !Z || !ph || !grad_spectra) return fail(PT_ERR_ARG, "pt_synth_adj_spectra: NULL pointer");
  if (L > 65535) return fail(PT_ERR_UNSUPPORTED, "pt_synth_adj_spectra: too many layers");
  cudaStream_t s = (cudaStream_t)stream;
  const size_t npix = (size_t)ns * ns;
  ProfScope ps("k_adj_spectra", s);
  k_adj_spectra<<<dim3((unsigned)((npix + 255) / 256), L), 256, 0, s>>>(
      ns, L, F, w, (const float2*)Z, (const float2*)ph, accumulate, (float2*)grad_spectra);
  count_launch_a();
  return check_launch("pt_synth_adj_spectra");
}

extern "C" int pt_synth_adj_params(int ns, double pixel_scale, int L, int F, const float* w,
                                   const float* spectra, const float* Z, const float* ph,
                                   double* out, void* stream) {
  if (ns < 2 || L < 1 || F < 1 || !(pixel_scale > 0))
    return fail(PT_ERR_ARG, "pt_synth_adj_params: bad sizes");
  if (!w || !spectra || !Z || !ph || !out) return fail(PT_ERR_ARG, "pt_synth_adj_params: NULL pointer");
  const int P2 = (F + 1) / 2;
  if (P2 > 65535) return fail(PT_ERR_UNSUPPORTED, "pt_synth_adj_params: too many frames");
  cudaStream_t s = (cudaStream_t)stream;
  ProfScope ps("k_adj_params", s);
  k_adj_params<<<dim3(L, P2), 256, 0, s>>>(ns, 1.0 / (ns * pixel_scale), L, F, w,
                                           (const float2*)spectra, (const float2*)Z,
                                           (const float2*)ph, out);
  count_launch_a();
  return check_launch("pt_synth_adj_params");
}
