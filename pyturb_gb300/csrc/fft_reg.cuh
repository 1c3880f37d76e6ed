// Register-resident Stockham FFT for power-of-two sizes N in [8, 4096]
// (inverse sign, unnormalised, as fft.cuh).
//
// A transform is done by a team of T = N / 8 threads; thread j holds the
// eight elements at positions j + T i (i = 0..7) in registers. Every stage
// reads that same pattern, so a stage is: twiddle + radix-R butterflies in
// registers, then (except after the last stage) one exchange through shared
// memory to the Stockham destinations. All radices, strides and index
// arithmetic are compile-time constants.
//
// Shared layouts (a functor maps element p of the team's vector to a float2
// slot) are XOR swizzles, bijective because every key bit that is itself
// modified depends only on higher, unmodified bits, and chosen so that every
// gather and every stage's scatter is free of bank conflicts for 64-bit
// accesses (checked by enumerating each warp's addresses for N = 64..1024):
//   RowLayout: teams are consecutive threads of one vector, vector v at
//     base + v (N + 8), slot p ^ ((p >> 3) & 15);
//   ColLayout: C vectors interleaved, lane c of a warp on vector c, slot
//     (p ^ ((p >> 3) & 3)) C + c.
#pragma once

#include "fft.cuh"

namespace pt {

__host__ __device__ constexpr int fft_padded(int n) { return n + 8; }

struct RowLayout {
  float2* base;
  __device__ __forceinline__ float2& operator[](int p) const {
    return base[p ^ ((p >> 3) & 15)];
  }
};

template <int C>
struct ColLayout {
  float2* base;  // already offset by the lane's column c
  __device__ __forceinline__ float2& operator[](int p) const {
    return base[(p ^ ((p >> 3) & 3)) * C];
  }
};

// radix of stage s for N = 8^a * r (r in {1, 2, 4}): all 8s first, the
// remainder last
template <int N>
struct Pow2Plan {
  static constexpr int log2n = (N <= 1) ? 0 : 1 + Pow2Plan<N / 2>::log2n;
  static constexpr int n8 = log2n / 3;
  static constexpr int rem = log2n % 3;  // 0, 1 or 2
  static constexpr int stages = n8 + (rem ? 1 : 0);
  __host__ __device__ static constexpr int radix(int s) { return s < n8 ? 8 : (rem == 1 ? 2 : 4); }
};
template <>
struct Pow2Plan<1> {
  static constexpr int log2n = 0, n8 = 0, rem = 0, stages = 0;
  __host__ __device__ static constexpr int radix(int) { return 1; }
};

template <int N>
struct is_pow2_fft {
  static constexpr bool value = N >= 8 && N <= 4096 && (N & (N - 1)) == 0;
};

// Stage twiddles live in shared memory per stage, ordered [jm][r-1] with
// jm = b mod Ns: consecutive butterflies read at a stride of R-1 float2
// (7, 3 or 1), which is conflict-free per half-warp. Stage s starts at
// tw_offset(N, s); the stages after the first fill fewer than N slots.
template <int N>
__host__ __device__ constexpr int tw_offset(int s) {
  int off = 0, ns = 1;
  for (int k = 0; k < s; ++k) {
    const int r = Pow2Plan<N>::radix(k);
    if (k > 0) off += ns * (r - 1);
    ns *= r;
  }
  return off;
}

// Fill the per-stage tables from the N-entry table exp(+2 pi i k / N), or
// from a longer table exp(+2 pi i k / (stride N)) read at every stride-th
// entry.
template <int N>
__device__ __forceinline__ void load_stage_tw(float2* stw, const float2* __restrict__ tw,
                                              int stride = 1) {
  int ns = Pow2Plan<N>::radix(0);
  for (int s = 1; s < Pow2Plan<N>::stages; ++s) {
    const int r = Pow2Plan<N>::radix(s);
    const int twstep = N / (ns * r);
    const int off = tw_offset<N>(s);
    for (int i = threadIdx.x; i < ns * (r - 1); i += blockDim.x) {
      const int jm = i / (r - 1), q = i % (r - 1) + 1;
      stw[off + i] = tw[((q * jm * twstep) & (N - 1)) * stride];
    }
    ns *= r;
  }
}

// Twiddle, butterflies of one stage on the thread's registers (in place:
// output q of the butterfly in register slot i0 + (8/R) q). `tw` here is the
// per-stage table of load_stage_tw.
template <int N, int R, int Ns, int S>
__device__ __forceinline__ void reg_stage(float2 (&x)[8], int j, const float2* __restrict__ tw) {
  constexpr int T = N / 8;
  constexpr int B = 8 / R;                // butterflies per thread
  constexpr int off = tw_offset<N>(S);
#pragma unroll
  for (int i0 = 0; i0 < B; ++i0) {
    const int b = j + T * i0;  // butterfly index (< N / R)
    const int jm = b & (Ns - 1);
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = x[i0 + B * r];
    if (Ns > 1) {
      const float2* t = tw + off + jm * (R - 1);
#pragma unroll
      for (int r = 1; r < R; ++r) v[r] = cmul(v[r], t[r - 1]);
    }
    if (R == 8) bfly8(v);
    else if (R == 4) bfly4(v);
    else bfly2(v);
#pragma unroll
    for (int q = 0; q < R; ++q) x[i0 + B * q] = v[q];
  }
}

// Write the stage outputs to their Stockham destinations.
template <int N, int R, int Ns, class Lay>
__device__ __forceinline__ void reg_scatter(const float2 (&x)[8], int j, const Lay& s) {
  constexpr int T = N / 8;
  constexpr int B = 8 / R;
#pragma unroll
  for (int i0 = 0; i0 < B; ++i0) {
    const int b = j + T * i0;
    const int idxD = (b / Ns) * Ns * R + (b & (Ns - 1));
#pragma unroll
    for (int q = 0; q < R; ++q) s[idxD + q * Ns] = x[i0 + B * q];
  }
}

template <int N, class Lay>
__device__ __forceinline__ void reg_gather8(float2 (&x)[8], int j, const Lay& s) {
#pragma unroll
  for (int i = 0; i < 8; ++i) x[i] = s[j + (N / 8) * i];
}

// Barrier policies of the exchanges: the whole CTA, or only the team that
// owns the exchanged vector (a named barrier; the team is whole warps).
struct CtaSync {
  __device__ __forceinline__ void operator()() const { __syncthreads(); }
};
struct TeamSync {
  int id, threads;  // barrier 1..15, thread count (a multiple of 32)
  __device__ __forceinline__ void operator()() const {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(threads) : "memory");
  }
};

template <int N, int S, int Ns, class Lay, class Sync>
struct RegStages {
  // run stages S.. ; x holds the inputs of stage S at positions j + T i
  static __device__ __forceinline__ void run(float2 (&x)[8], int j, const float2* tw,
                                             const Lay& s, const Sync& sync) {
    constexpr int R = Pow2Plan<N>::radix(S);
    reg_stage<N, R, Ns, S>(x, j, tw);
    if constexpr (S + 1 < Pow2Plan<N>::stages) {
      reg_scatter<N, R, Ns>(x, j, s);
      sync();
      reg_gather8<N>(x, j, s);
      sync();
      RegStages<N, S + 1, Ns * R, Lay, Sync>::run(x, j, tw, s, sync);
    }
  }
};

// As RegStages, with the exchanges alternating between two scratch vectors a
// and b: stage s scatters into one and gathers from it after one barrier; the
// next stage scatters into the other, so every thread has passed this stage's
// gather (the next barrier) before the vector is written again. One barrier
// per exchange instead of two.
template <int N, int S, int Ns, class Lay, class Sync>
struct RegStages2 {
  static __device__ __forceinline__ void run(float2 (&x)[8], int j, const float2* tw,
                                             const Lay& a, const Lay& b, const Sync& sync) {
    constexpr int R = Pow2Plan<N>::radix(S);
    reg_stage<N, R, Ns, S>(x, j, tw);
    if constexpr (S + 1 < Pow2Plan<N>::stages) {
      reg_scatter<N, R, Ns>(x, j, a);
      sync();
      reg_gather8<N>(x, j, a);
      RegStages2<N, S + 1, Ns * R, Lay, Sync>::run(x, j, tw, b, a, sync);
    }
  }
};

// Full transform of the thread's team. x in: element j + T i of the input;
// x out: element j + T i of the output. `s` addresses this team's scratch
// vector through its layout; tw is the shared per-stage twiddle table filled
// by load_stage_tw<N>. Every thread the barrier policy covers must call this
// (CtaSync: the whole CTA; TeamSync: the team), and the caller must
// synchronise those threads between its own last read of `s` and this call.
template <int N, class Lay, class Sync = CtaSync>
__device__ __forceinline__ void reg_fft(float2 (&x)[8], int j, const float2* tw, const Lay& s,
                                        const Sync& sync = Sync{}) {
  RegStages<N, 0, 1, Lay, Sync>::run(x, j, tw, s, sync);
}

// NV transforms of the same team in lockstep (one barrier per exchange for
// all of them), each on its own pair of scratch vectors a[v], b[v] used
// alternately as in RegStages2.
template <int N, int S, int Ns, int NV, class Lay, class Sync>
struct RegStagesMulti {
  static __device__ __forceinline__ void run(float2 (&x)[NV][8], int j, const float2* tw,
                                             const Lay* a, const Lay* b, const Sync& sync) {
    constexpr int R = Pow2Plan<N>::radix(S);
#pragma unroll
    for (int v = 0; v < NV; ++v) reg_stage<N, R, Ns, S>(x[v], j, tw);
    if constexpr (S + 1 < Pow2Plan<N>::stages) {
#pragma unroll
      for (int v = 0; v < NV; ++v) reg_scatter<N, R, Ns>(x[v], j, a[v]);
      sync();
#pragma unroll
      for (int v = 0; v < NV; ++v) reg_gather8<N>(x[v], j, a[v]);
      RegStagesMulti<N, S + 1, Ns * R, NV, Lay, Sync>::run(x, j, tw, b, a, sync);
    }
  }
};

// The same transform on two scratch vectors (first exchange in a). The caller
// must synchronise the barrier's threads between its own last access of `a`
// and this call; its last access of `b` only has to precede the call (the
// first exchange's barrier orders it before b is written).
// NV transforms in lockstep; the scratch vector arrays a and b hold NV
// layouts each. Ordering contract as reg_fft_db, for every a[v] and b[v].
template <int N, int NV, class Lay, class Sync = CtaSync>
__device__ __forceinline__ void reg_fft_multi(float2 (&x)[NV][8], int j, const float2* tw,
                                              const Lay* a, const Lay* b,
                                              const Sync& sync = Sync{}) {
  RegStagesMulti<N, 0, 1, NV, Lay, Sync>::run(x, j, tw, a, b, sync);
}

template <int N, class Lay, class Sync = CtaSync>
__device__ __forceinline__ void reg_fft_db(float2 (&x)[8], int j, const float2* tw, const Lay& a,
                                           const Lay& b, const Sync& sync = Sync{}) {
  RegStages2<N, 0, 1, Lay, Sync>::run(x, j, tw, a, b, sync);
}

}  // namespace pt
