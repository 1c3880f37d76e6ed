// Shared-memory Stockham autosort FFT (mixed radix 8/4/2/3/5/7 plus a
// direct-sum stage for any larger prime factor), inverse sign, unnormalised:
//   X[k] = sum_j x[j] exp(+2 pi i j k / n)
// which is numpy.fft.ifft(x) * n. Every transform of a pass lives in shared
// memory; passes run along rows (contiguous) or along columns (tiles of C
// columns), so a 2-D transform is two passes over HBM/L2.
#pragma once

#include "common.cuh"

namespace pt {

constexpr int kMaxStages = 24;

struct FftDesc {
  int n;
  int nstages;
  int radix[kMaxStages];
  // Bluestein form (M > 0), for lengths with a large prime factor: the
  // length-n transform as a circular convolution of length M, a power of two
  // >= 2n - 1, on the radix-8/4/2 stages; buffers then hold M elements a
  // vector (fft_buf_len)
  int M;
  int mstages;
  int mradix[kMaxStages];
  const float2* chirp;  // (n) exp(+i pi (e^2 mod 2n) / n)
  const float2* bhat;   // (M) sum_m b[m] exp(+2 pi i m k / M), b the wrapped conj(chirp)
  const float2* twM;    // (M) exp(+2 pi i e / M)
};

// Elements a vector buffer of fft_smem must hold for this transform.
__host__ __device__ inline int fft_buf_len(const FftDesc& d) { return d.M > 0 ? d.M : d.n; }

// Factor n into the stage radices used by the Stockham passes. Radix 8
// first keeps the stage count low; leftover prime factors > 7 become a
// single direct-sum stage each.
inline FftDesc make_fft_desc(int n) {
  FftDesc d{};
  d.n = n;
  int m = n, s = 0;
  const int pref[] = {8, 4, 2, 3, 5, 7};
  for (int r : pref) {
    while (m % r == 0 && s < kMaxStages) {
      d.radix[s++] = r;
      m /= r;
    }
  }
  for (int p = 11; m > 1 && s < kMaxStages; p += 2) {
    while (m % p == 0 && s < kMaxStages) {
      d.radix[s++] = p;
      m /= p;
    }
    if ((long long)p * p > m && m > 1) {
      d.radix[s++] = m;
      m = 1;
    }
  }
  d.nstages = s;
  return d;
}

// ------------------------------------------------------------------ butterflies
// In-register radix-R inverse DFTs, v[q] <- sum_r v[r] exp(+2 pi i q r / R).
__device__ __forceinline__ void bfly2(float2* v) {
  float2 a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}

__device__ __forceinline__ void bfly4(float2* v) {
  float2 a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
  float2 b0 = cadd(v[1], v[3]), b1 = cmul_i(csub(v[1], v[3]));
  v[0] = cadd(a0, b0);
  v[2] = csub(a0, b0);
  v[1] = cadd(a1, b1);
  v[3] = csub(a1, b1);
}

__device__ __forceinline__ void bfly8(float2* v) {
  const float h = 0.70710678118654752440f;
  // radix-2 over pairs (r, r+4)
  float2 a[4], b[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    a[r] = cadd(v[r], v[r + 4]);
    b[r] = csub(v[r], v[r + 4]);
  }
  // twiddle b[r] by w8^r, w8 = exp(+i pi/4)
  b[1] = make_float2(h * (b[1].x - b[1].y), h * (b[1].x + b[1].y));
  b[2] = cmul_i(b[2]);
  b[3] = make_float2(-h * (b[3].x + b[3].y), h * (b[3].x - b[3].y));
  bfly4(a);
  bfly4(b);
  // outputs: even q from a, odd q from b
  v[0] = a[0];
  v[2] = a[1];
  v[4] = a[2];
  v[6] = a[3];
  v[1] = b[0];
  v[3] = b[1];
  v[5] = b[2];
  v[7] = b[3];
}

__device__ __forceinline__ void bfly3(float2* v) {
  const float c1 = -0.5f, s1 = 0.86602540378443864676f;  // exp(+2 pi i/3)
  float2 t = cadd(v[1], v[2]);
  float2 d = csub(v[1], v[2]);
  float2 m = make_float2(v[0].x + c1 * t.x, v[0].y + c1 * t.y);
  float2 r = make_float2(-s1 * d.y, s1 * d.x);  // i*s1*d
  v[0] = cadd(v[0], t);
  v[1] = cadd(m, r);
  v[2] = csub(m, r);
}

__device__ __forceinline__ void bfly5(float2* v) {
  const float c1 = 0.30901699437494742410f, c2 = -0.80901699437494742410f;
  const float s1 = 0.95105651629515357212f, s2 = 0.58778525229247312917f;
  float2 t1 = cadd(v[1], v[4]), d1 = csub(v[1], v[4]);
  float2 t2 = cadd(v[2], v[3]), d2 = csub(v[2], v[3]);
  float2 m1 = make_float2(v[0].x + c1 * t1.x + c2 * t2.x, v[0].y + c1 * t1.y + c2 * t2.y);
  float2 m2 = make_float2(v[0].x + c2 * t1.x + c1 * t2.x, v[0].y + c2 * t1.y + c1 * t2.y);
  // i*(s1 d1 + s2 d2) and i*(s2 d1 - s1 d2)
  float2 r1 = make_float2(-(s1 * d1.y + s2 * d2.y), s1 * d1.x + s2 * d2.x);
  float2 r2 = make_float2(-(s2 * d1.y - s1 * d2.y), s2 * d1.x - s1 * d2.x);
  v[0] = cadd(v[0], cadd(t1, t2));
  v[1] = cadd(m1, r1);
  v[4] = csub(m1, r1);
  v[2] = cadd(m2, r2);
  v[3] = csub(m2, r2);
}

// Generic small radix (7): direct sum with the transform's own twiddle table.
template <int R>
__device__ __forceinline__ void bfly_direct(float2* v, const float2* tw, int n) {
  float2 o[R];
  const int step = n / R;
#pragma unroll
  for (int q = 0; q < R; ++q) {
    float2 acc = v[0];
#pragma unroll
    for (int r = 1; r < R; ++r) acc = cfma(v[r], tw[((q * r) % R) * step], acc);
    o[q] = acc;
  }
#pragma unroll
  for (int q = 0; q < R; ++q) v[q] = o[q];
}

// q = t / d, r = t mod d for 0 <= t < 2^22 and 1 <= d <= 2^14, through the
// float reciprocal inv = 1/d: t * inv carries a relative error below 2^-23,
// so the truncated quotient is off by at most one, and one step corrects it
// (a runtime integer division costs several times the instructions).
__device__ __forceinline__ void divmod_f(int t, int d, float inv, int& q, int& r) {
  q = __float2int_rz(__int2float_rn(t) * inv);
  r = t - q * d;
  if (r < 0) {
    --q;
    r += d;
  } else if (r >= d) {
    ++q;
    r -= d;
  }
}

// One Stockham stage with a compile-time radix. Work items are (vector,
// butterfly) pairs; `vfast` selects whether consecutive threads walk the
// vector index (column tiles) or the butterfly index (rows).
template <int R>
__device__ __forceinline__ void stage_r(const float2* __restrict__ a, float2* __restrict__ b,
                                        const float2* __restrict__ tw, int n, int Ns, int nvec,
                                        int vs, int es, bool vfast) {
  const int nb = n / R;
  const int total = nb * nvec;
  const int twstep = n / (Ns * R);
  const float inv_split = 1.0f / (float)(vfast ? nvec : nb);
  const float inv_ns = 1.0f / (float)Ns;
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    int v, j;
    if (vfast) divmod_f(t, nvec, inv_split, j, v);
    else divmod_f(t, nb, inv_split, v, j);
    const float2* src = a + v * vs;
    float2* dst = b + v * vs;
    int jq, jm;
    divmod_f(j, Ns, inv_ns, jq, jm);
    float2 x[R];
#pragma unroll
    for (int r = 0; r < R; ++r) x[r] = src[(j + r * nb) * es];
    if (Ns > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) x[r] = cmul(x[r], tw[r * jm * twstep]);
    }
    if (R == 2) bfly2(x);
    else if (R == 4) bfly4(x);
    else if (R == 8) bfly8(x);
    else if (R == 3) bfly3(x);
    else if (R == 5) bfly5(x);
    else bfly_direct<R>(x, tw, n);
    const int idxD = jq * Ns * R + jm;
#pragma unroll
    for (int q = 0; q < R; ++q) dst[(idxD + q * Ns) * es] = x[q];
  }
}

// Direct-sum stage for a large prime radix: every output is its own
// R-term sum, so the work items are (vector, butterfly, output) triples.
__device__ __forceinline__ void stage_generic(const float2* __restrict__ a, float2* __restrict__ b,
                                              const float2* __restrict__ tw, int n, int R, int Ns,
                                              int nvec, int vs, int es) {
  const int nb = n / R;
  const long total = (long)nb * R * nvec;
  const int twstep = n / (Ns * R);
  for (long t = threadIdx.x; t < total; t += blockDim.x) {
    const int v = (int)(t % nvec);
    const long rest = t / nvec;
    const int q = (int)(rest % R);
    const int j = (int)(rest / R);
    const float2* src = a + v * vs;
    const int jm = j % Ns;
    // exponent of input r: r * (jm * twstep + q * n / R)  (mod n)
    const int base = jm * twstep + q * (n / R);
    float2 acc = make_float2(0.f, 0.f);
    int e = 0;
    for (int r = 0; r < R; ++r) {
      acc = cfma(src[(j + r * nb) * es], tw[e], acc);
      e += base;
      if (e >= n) e -= n;
    }
    const int idxD = (j / Ns) * Ns * R + jm;
    b[v * vs + (idxD + q * Ns) * es] = acc;
  }
}

// The Stockham stages of a length-n transform with the given radices.
__device__ inline float2* fft_stages(float2* a, float2* b, const int* radix, int nstages,
                                     const float2* tw, int n, int nvec, int vs, int es,
                                     bool vfast) {
  int Ns = 1;
  for (int s = 0; s < nstages; ++s) {
    const int R = radix[s];
    switch (R) {
      case 2: stage_r<2>(a, b, tw, n, Ns, nvec, vs, es, vfast); break;
      case 3: stage_r<3>(a, b, tw, n, Ns, nvec, vs, es, vfast); break;
      case 4: stage_r<4>(a, b, tw, n, Ns, nvec, vs, es, vfast); break;
      case 5: stage_r<5>(a, b, tw, n, Ns, nvec, vs, es, vfast); break;
      case 7: stage_r<7>(a, b, tw, n, Ns, nvec, vs, es, vfast); break;
      case 8: stage_r<8>(a, b, tw, n, Ns, nvec, vs, es, vfast); break;
      default: stage_generic(a, b, tw, n, R, Ns, nvec, vs, es); break;
    }
    __syncthreads();
    float2* t = a;
    a = b;
    b = t;
    Ns *= R;
  }
  return a;
}

// Bluestein: with w[e] = exp(+i pi e^2 / n) and n k = (n^2 + k^2 - (k - n)^2)/2,
//   X[k] = w[k] (a (*) b)[k],  a[e] = x[e] w[e] (e < n, zero up to M),
// b[m] = conj(w[m]) for |m| < n wrapped modulo M, and the circular
// convolution is (1/M) conj(F(conj(F(a) bhat))) with F the inverse-sign
// transform of length M and bhat = F(b) precomputed.
__device__ inline float2* fft_bluestein(float2* a, float2* b, const FftDesc& d, int nvec, int vs,
                                        int es, bool vfast) {
  const int n = d.n, M = d.M;
  for (int t = threadIdx.x; t < nvec * M; t += blockDim.x) {
    const int v = vfast ? t % nvec : t / M, e = vfast ? t / nvec : t % M;
    float2* p = a + v * vs + e * es;
    *p = e < n ? cmul(*p, __ldg(d.chirp + e)) : make_float2(0.f, 0.f);
  }
  __syncthreads();
  float2* x = fft_stages(a, b, d.mradix, d.mstages, d.twM, M, nvec, vs, es, vfast);
  float2* y = x == a ? b : a;
  for (int t = threadIdx.x; t < nvec * M; t += blockDim.x) {
    const int v = vfast ? t % nvec : t / M, e = vfast ? t / nvec : t % M;
    float2* p = x + v * vs + e * es;
    *p = cconj(cmul(*p, __ldg(d.bhat + e)));
  }
  __syncthreads();
  float2* z = fft_stages(x, y, d.mradix, d.mstages, d.twM, M, nvec, vs, es, vfast);
  const float inv = 1.0f / (float)M;
  for (int t = threadIdx.x; t < nvec * n; t += blockDim.x) {
    const int v = vfast ? t % nvec : t / n, e = vfast ? t / nvec : t % n;
    float2* p = z + v * vs + e * es;
    *p = cscale(cmul(__ldg(d.chirp + e), cconj(*p)), inv);
  }
  __syncthreads();
  return z;
}

// Run all stages on `nvec` vectors held in shared memory. Element e of vector
// v sits at buf[v * vs + e * es]; both buffers hold fft_buf_len(d) elements
// a vector. Returns the buffer holding the result (a or b). Ends with
// __syncthreads().
__device__ inline float2* fft_smem(float2* a, float2* b, const FftDesc& d, const float2* tw,
                                   int nvec, int vs, int es, bool vfast) {
  if (d.M > 0) return fft_bluestein(a, b, d, nvec, vs, es, vfast);
  return fft_stages(a, b, d.radix, d.nstages, tw, d.n, nvec, vs, es, vfast);
}

}  // namespace pt
