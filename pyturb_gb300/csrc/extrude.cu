// Assemat-Wilson extrusion and the fused multi-layer readout on the GB300.
//
// Ring buffers: screen s occupies buf[s] = (cap, W) floats; virtual row v of
// the screen lives in physical row v mod cap, so advancing the wind moves an
// index instead of compacting rows.
//
// Extrusion step: every screen needing a row this step contributes one
// column X_j = [stencil rows (m W values) ; bscale_j * beta_j (W values)] and
// the new rows are the "TN" product out[j][r] = sum_k M_g[r][k] X_j[k] with
// M_g = [A_g | B_unit_g] (W x (m+1) W). A split-K SIMT GEMM with a
// deterministic reduction writes them straight into the ring.
//
// Readout: one thread per pupil pixel; per layer the rotated, magnified,
// shifted sample position is formed in 64-bit fixed point (exact up to
// 2^-40 px whatever the travel), the 2/4/6 separable taps gather from the
// ring and the layers are summed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <vector>

#include <cuda_bf16.h>

#include "common.cuh"
#include "tc.cuh"

namespace pt {
uint64_t* launch_counter();
static inline void count_launch_e(int k = 1) {
  __atomic_add_fetch(launch_counter(), (uint64_t)k, __ATOMIC_RELAXED);
}

constexpr int kTM = 64;   // output rows per CTA
constexpr int kTJ = 32;   // jobs (columns) per CTA
constexpr int kTK = 32;   // K step
constexpr int kMaxSplit = 16;
// register-tiled extrusion GEMM: 128 rows x 16 TJ jobs per CTA, K steps of 16
constexpr int kGBM = 128;
constexpr int kGBK = 16;
constexpr int kMaxSplitTiled = 32;

struct GatherJob {
  int screen, head;
  float bscale;
  uint64_t key, row;
  long long noise_off;
};
// Jobs travel inside the launch parameters (no pageable copy, no sync).
constexpr int kJobsPerLaunch = 192;
struct JobParams {
  GatherJob j[kJobsPerLaunch];
};
// Ring destination (screen, physical row) of each job's new row: what the
// reduce needs, in a fifth of the launch parameters.
struct RingDst {
  int2 d[kJobsPerLaunch];
};
// Sparse stencil points (column, rows back from the new row), appended to the
// m full rows in the operand: X = [m rows ; sparse values ; bscale * beta].
struct SparseDev {
  int n;
  int depth[PT_MAX_SPARSE];
  int col[PT_MAX_SPARSE];
};
__device__ __forceinline__ int ring_back(int head, int d, int cap) {
  int p = head - d;
  return p < 0 ? p + cap : p;
}

// X[j] for job j = blockIdx.z: block row blockIdx.y < m copies stencil row y
// from the ring, row m holds bscale * beta, row m + 1 (only with sparse
// points) the sparse values; each thread makes two adjacent columns (one
// Philox call for both noise values).
//
// With `prev` set, the previous launch extruded the same screens one row
// earlier and its split-K slices (prev_nz of them) are still unreduced: row
// m - 1 here is that new row, summed in the order of k_extrude_reduce and
// written both into the ring and into X (no thread reads that ring row; the
// sparse points lie deeper than m rows).
//
// With `incr` (the increment form, never together with `prev`) stencil row
// r < m - 1 becomes row_r - row_{r+1}, the newest row stays as it is and a
// sparse value becomes s_p - r1[c_p]: the operand of an increment-form
// operator, whose product is added to r1 by the reduce.
__global__ void k_extrude_gather(int W, int m, int cap, float* __restrict__ buf,
                                 const JobParams jobs, int J, const SparseDev sp,
                                 const float* __restrict__ noise, float* __restrict__ X,
                                 const float* __restrict__ prev, int prev_nz, int incr) {
  const int j = blockIdx.z;
  if (j >= J) return;
  const GatherJob& jb = jobs.j[j];
  const int K = (m + 1) * W + sp.n;
  const int r = blockIdx.y;
  const int c = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
  if (r == m + 1) {  // sparse points
    const float* slab = buf + (size_t)jb.screen * cap * W;
    const float* r1 = slab + (size_t)ring_back(jb.head, 1, cap) * W;
    float* dst = X + (size_t)j * K + (size_t)m * W;
    for (int e = c; e < c + 2 && e < sp.n; ++e) {
      const float v = slab[(size_t)ring_back(jb.head, sp.depth[e], cap) * W + sp.col[e]];
      dst[e] = incr ? v - r1[sp.col[e]] : v;
    }
    return;
  }
  if (c >= W) return;
  const bool two = c + 1 < W;
  if (r < m) {
    float* dst = X + (size_t)j * K + (size_t)r * W + c;
    int phys = jb.head - m + r;
    if (phys < 0) phys += cap;
    float* src = buf + ((size_t)jb.screen * cap + phys) * W + c;
    if (incr && r < m - 1) {
      const float* nxt = buf + ((size_t)jb.screen * cap + (phys + 1 == cap ? 0 : phys + 1)) * W + c;
      dst[0] = src[0] - nxt[0];
      if (two) dst[1] = src[1] - nxt[1];
    } else if (prev && r == m - 1) {
      float s0 = 0.f, s1 = 0.f;
      for (int z = 0; z < prev_nz; ++z) {
        const float* pz = prev + ((size_t)z * J + j) * W + c;
        s0 += __ldcs(pz);
        if (two) s1 += __ldcs(pz + 1);
      }
      src[0] = s0;
      dst[0] = s0;
      if (two) {
        src[1] = s1;
        dst[1] = s1;
      }
    } else {
      dst[0] = src[0];
      if (two) dst[1] = src[1];
    }
    return;
  }
  float* dst = X + (size_t)j * K + (size_t)m * W + sp.n + c;
  if (noise) {
    dst[0] = jb.bscale * noise[jb.noise_off + c];
    if (two) dst[1] = jb.bscale * noise[jb.noise_off + c + 1];
  } else {
    const float2 p = philox_cnormal(jb.key, (uint64_t)(c >> 1), jb.row, kDomainExtrude);
    dst[0] = jb.bscale * p.x;
    if (two) dst[1] = jb.bscale * p.y;
  }
}

// The same operand for the tensor-core form: split into `terms` bf16 terms and
// stored as B tiles, tiles[(kc * terms + t) * NP * Kc * 2 + core(j, k % Kc)]
// (Kc = tc::kTcKc), zero for padding columns k >= K and rows j >= J. One
// thread makes the 8 consecutive K values of one job that form a 16-byte row
// of a core matrix; consecutive threads take consecutive K groups of the same
// job, so a warp reads one contiguous stretch of that job's ring rows.
__global__ void k_tc_gather(int W, int m, int cap, const float* __restrict__ buf,
                            const JobParams jobs, int J, const SparseDev sp, int NP, int nkc,
                            int terms, const float* __restrict__ noise,
                            uint8_t* __restrict__ tiles, int incr) {
  constexpr int Kc = tc::kTcKc;
  const int mW = m * W, Kn = mW + sp.n;  // the noise section starts at Kn
  const int K = Kn + W;
  const size_t tile = (size_t)NP * Kc * 2;
  const int groups = nkc * (Kc / 8);
  const size_t total = (size_t)groups * NP;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(t / groups);
    const int k0 = (int)(t % groups) * 8;
    float v[8];
    if (j < J) {
      const GatherJob& jb = jobs.j[j];
      const float* slab = buf + (size_t)jb.screen * cap * W;
      // stencil row and column of k0 once (valid while k < mW), advanced per value
      int r = k0 / W, c = k0 - r * W;
      const float* src = nullptr;
      auto row_src = [&](int rr) {
        int phys = jb.head - m + rr;
        if (phys < 0) phys += cap;
        return slab + (size_t)phys * W;
      };
      if (r < m) src = row_src(r);
      float2 pn = make_float2(0.f, 0.f);
      int pc = -2;  // noise column pair whose normals are in pn
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int k = k0 + q;
        float val = 0.f;
        if (k < mW) {
          val = src[c];
          if (incr && r < m - 1) val -= row_src(r + 1)[c];
          if (++c == W) {
            c = 0;
            ++r;
            if (r < m) src = row_src(r);
          }
        } else if (k < Kn) {
          const int e = k - mW;
          val = slab[(size_t)ring_back(jb.head, sp.depth[e], cap) * W + sp.col[e]];
          if (incr) val -= slab[(size_t)ring_back(jb.head, 1, cap) * W + sp.col[e]];
        } else if (k < K) {
          const int cn = k - Kn;
          if (noise) {
            val = jb.bscale * noise[jb.noise_off + cn];
          } else {
            if ((cn >> 1) != pc) {
              pn = philox_cnormal(jb.key, (uint64_t)(cn >> 1), jb.row, kDomainExtrude);
              pc = cn >> 1;
            }
            val = jb.bscale * ((cn & 1) ? pn.y : pn.x);
          }
        }
        v[q] = val;
      }
    } else {
#pragma unroll
      for (int q = 0; q < 8; ++q) v[q] = 0.f;
    }
    uint8_t* blk = tiles + (size_t)(k0 / Kc) * terms * tile + tc::core_offset(j, k0 % Kc, Kc);
    for (int tt = 0; tt < terms; ++tt) {
      uint32_t w4[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const __nv_bfloat16 h0 = __float2bfloat16_rn(v[2 * q]);
        const __nv_bfloat16 h1 = __float2bfloat16_rn(v[2 * q + 1]);
        w4[q] = (uint32_t)__bfloat16_as_ushort(h0) | ((uint32_t)__bfloat16_as_ushort(h1) << 16);
        v[2 * q] -= __bfloat162float(h0);
        v[2 * q + 1] -= __bfloat162float(h1);
      }
      *(uint4*)(blk + tt * tile) = make_uint4(w4[0], w4[1], w4[2], w4[3]);
    }
  }
}

// The stencil part of the FP32 form's operand, X[j][0, Kz), as one bf16
// term in the tensor-core B-tile layout (zero beyond Kz and J): the operand
// of the operator correction (A - (float)A) X, whose bf16 rounding is far
// below float32 resolution (the correction itself is ~2^-24 of the product).
__global__ void k_lo_operand(const float* __restrict__ X, int J, int K, int Kz, int NP, int nkc,
                             uint8_t* __restrict__ tiles) {
  constexpr int Kc = tc::kTcKc;
  const int groups = nkc * (Kc / 8);
  const size_t total = (size_t)groups * NP;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(t / groups);
    const int k0 = (int)(t % groups) * 8;
    uint32_t w4[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int ka = k0 + 2 * q, kb = ka + 1;
      const float a = (j < J && ka < Kz) ? X[(size_t)j * K + ka] : 0.f;
      const float b = (j < J && kb < Kz) ? X[(size_t)j * K + kb] : 0.f;
      w4[q] = (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(a)) |
              ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(b)) << 16);
    }
    uint8_t* blk = tiles + (size_t)(k0 / Kc) * NP * Kc * 2 + tc::core_offset(j, k0 % Kc, Kc);
    *(uint4*)blk = make_uint4(w4[0], w4[1], w4[2], w4[3]);
  }
}

// ---------------------------------------------------------------- low-order anchor
// The row recursion amplifies errors in the smooth, large-scale modes of a row
// (its extrapolation is marginally stable there), so float32 rounding in the
// product, random per step, still walks those modes away from the float64
// result over hundreds of rows. The anchor recomputes the first R DCT-II
// modes of every new row in double-float arithmetic (float32 pairs, Dekker /
// Knuth error-free products and sums) from the same operand,
//   d = U^T A z - U^T new + U^T B (bscale beta),
// and adds U d to the row: the smooth modes then follow the float64 operator
// while the rest stays float32. U^T A and U are given as (hi, lo) float32
// pairs; the noise term is small and enters in float32.
// packed float32 pairs (two modes per instruction)
typedef unsigned long long f2p;
__device__ __forceinline__ f2p pack2(float lo, float hi) {
  f2p r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ void unpack2(f2p v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f2p padd(f2p a, f2p b) {
  f2p d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2p psub(f2p a, f2p b) {
  f2p d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2p pmul(f2p a, f2p b) {
  f2p d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2p pfma(f2p a, f2p b, f2p c) {
  f2p d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
// (s, c) += a x for two modes at once: exact product a_hi x = h + e, the
// lo part a_lo x in float32, h added to s by an error-free two-sum. The
// caller passes nah = -a_hi, so the product comes out negated (nh = -h,
// exact) and no sign flip is needed per product: t = s - nh = s + h and
// h - bv = -(nh + bv) round identically.
__device__ __forceinline__ void pmac(f2p& s, f2p& c, f2p ah, f2p nah, f2p al, f2p x2) {
  const f2p nh = pmul(nah, x2);
  const f2p e = pfma(ah, x2, nh);
  const f2p t = psub(s, nh);
  const f2p bv = psub(t, s);
  c = padd(c, pfma(al, x2, e));
  c = padd(c, psub(psub(s, psub(t, bv)), padd(nh, bv)));
  s = t;
}

struct AnchorDev {
  const f2p* th;   // (G, Kt, R/2) hi parts of [U^T A | U^T B | -U]^T, mode pairs
  const f2p* tl;   // (G, Kt, R/2) lo parts
  const float* u;  // (R, W) U in float32 (the correction is tiny)
};

// s + h into (s, c): s the rounded sum, c collects the exact rounding error
// (the _rn intrinsics keep the compiler from contracting or reordering the
// error-free transformations)
__device__ __forceinline__ void two_sum_acc(float& s, float& c, float h) {
  const float t = __fadd_rn(s, h);
  const float bv = __fsub_rn(t, s);
  c += __fadd_rn(__fsub_rn(s, __fsub_rn(t, bv)), __fsub_rn(h, bv));
  s = t;
}

// The anchor's projections as one small double-float GEMM over the
// concatenated columns [stencil (Kz) | noise (W) | new row (W)]:
//   part[z][j][i] = sum over slice z of P'[i][k] x'_j[k],
//   P' = [U^T A | U^T B | -U],  x'_j = [X_j[0, Kz) | X_j[Kz, K) | new_j],
// so d = sum_z part is U^T A z + U^T B (bscale beta) - U^T new. The table
// P'^T is prepared once on the host as (hi, lo) float32 rows of R values per
// column k, the modes of a row stored in pairs (i, i + 16), so a chunk of 64
// columns is one contiguous copy. A CTA takes 16 jobs x all R modes over one
// K slice (each thread one job and R/16 modes), staging 64-column chunks of
// x' and P' in shared memory; part holds (s, c) double-float pairs.
template <int R>
__global__ void __launch_bounds__(256)
k_anchor_gemm(int W, int K, int Kz, int cap, int g, int J, int kslice, int incr,
              const RingDst dst, const float* __restrict__ X, const AnchorDev an,
              const float* __restrict__ buf, float2* __restrict__ part) {
  // 32-column chunks keep the static shared memory under 48 KB; the operand
  // is staged as (x, x) pairs, ready for the packed products
  constexpr int KC = 32, NP2 = R / 2, JT = 64, JPT = JT * NP2 / 256;
  __shared__ f2p xs[JT][KC + 1];
  __shared__ f2p phs[KC][NP2], pls[KC][NP2];
  const int tid = threadIdx.x;
  const int j0 = blockIdx.x * JT, z = blockIdx.y;
  const int Kt = K + (incr ? 2 : 1) * W;  // [operand | new row | r1 (increment form)]
  const int kb = z * kslice, ke = min(Kt, kb + kslice);
  const int p = tid % NP2, jt = (tid / NP2) * JPT;  // this thread: pair p, jobs jt .. jt + JPT - 1
  const f2p* th = an.th + (size_t)g * Kt * NP2;
  const f2p* tl = an.tl + (size_t)g * Kt * NP2;
  f2p s[JPT], c[JPT];
#pragma unroll
  for (int q = 0; q < JPT; ++q) s[q] = c[q] = 0ull;
  for (int k0 = kb; k0 < ke; k0 += KC) {
    for (int e = tid; e < JT * KC; e += 256) {
      const int jj = e / KC, kk = e % KC, k = k0 + kk, j = j0 + jj;
      float v = 0.f;
      if (j < J && k < ke) {
        const float* slab = buf + (size_t)dst.d[j].x * cap * W;
        v = k < K ? X[(size_t)j * K + k]
                  : (k < K + W ? slab[(size_t)dst.d[j].y * W + (k - K)]
                               : slab[(size_t)ring_back(dst.d[j].y, 1, cap) * W + (k - K - W)]);
      }
      xs[jj][kk] = pack2(v, v);
    }
    // the table rows k0 .. k0 + KC - 1 are contiguous: straight copies
    for (int e = tid; e < KC * NP2; e += 256) {
      const bool in = k0 + e / NP2 < ke;
      phs[e / NP2][e % NP2] = in ? th[(size_t)k0 * NP2 + e] : 0ull;
      pls[e / NP2][e % NP2] = in ? tl[(size_t)k0 * NP2 + e] : 0ull;
    }
    __syncthreads();
    const int kn = min(KC, ke - k0);
    for (int kk = 0; kk < kn; ++kk) {
      const f2p ah = phs[kk][p];
      const int k = k0 + kk;
      if (k >= Kz && k < K) {
        // noise columns: U^T B (bscale beta) is ~1% of the row and its
        // rounding random from row to row, so plain float32 suffices
#pragma unroll
        for (int q = 0; q < JPT; ++q) c[q] = pfma(ah, xs[jt + q][kk], c[q]);
      } else {
        const f2p al = pls[kk][p];
        const f2p nah = ah ^ 0x8000000080000000ull;
#pragma unroll
        for (int q = 0; q < JPT; ++q) pmac(s[q], c[q], ah, nah, al, xs[jt + q][kk]);
      }
    }
    __syncthreads();
  }
  // pair p = modes (i0, i0 + 16), i0 = (p & 15) + 32 (p >> 4)
  const int i0 = (p & 15) + 32 * (p >> 4);
#pragma unroll
  for (int q = 0; q < JPT; ++q) {
    const int j = j0 + jt + q;
    if (j >= J) break;
    float s0, s1, c0, c1;
    unpack2(s[q], s0, s1);
    unpack2(c[q], c0, c1);
    part[((size_t)z * J + j) * R + i0] = make_float2(s0, c0);
    part[((size_t)z * J + j) * R + i0 + 16] = make_float2(s1, c1);
  }
}

// new row += U d, d = sum over the slices of part (fixed order), one CTA per
// job: warp w reduces modes w, w + 8, ... (lanes over slices, then a fixed
// butterfly), then every thread corrects its pixels.
template <int R>
__global__ void __launch_bounds__(256)
k_anchor_apply(int W, int cap, int J, int nsplit, const RingDst dst,
               const float2* __restrict__ part, const float* __restrict__ u,
               float* __restrict__ buf) {
  __shared__ float ds[R];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int j = blockIdx.x;
  if (j >= J) return;
  for (int i = warp; i < R; i += 8) {
    float ss = 0.f, cc = 0.f;
    for (int z = lane; z < nsplit; z += 32) {
      const float2 q = part[((size_t)z * J + j) * R + i];
      cc = __fadd_rn(cc, q.y);
      two_sum_acc(ss, cc, q.x);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float so = __shfl_xor_sync(0xffffffffu, ss, o);
      const float co = __shfl_xor_sync(0xffffffffu, cc, o);
      // the same operands in the same order on both lanes of a pair
      const float a = (lane & o) ? so : ss, b = (lane & o) ? ss : so;
      float s2 = a, c2 = (lane & o) ? __fadd_rn(co, cc) : __fadd_rn(cc, co);
      two_sum_acc(s2, c2, b);
      ss = s2;
      cc = c2;
    }
    if (lane == 0) ds[i] = ss + cc;
  }
  __syncthreads();
  float* row = buf + ((size_t)dst.d[j].x * cap + dst.d[j].y) * W;
  for (int w = tid; w < W; w += 256) {
    float v = 0.f;
#pragma unroll
    for (int i = 0; i < R; ++i) v = fmaf(__ldg(u + (size_t)i * W + w), ds[i], v);
    row[w] += v;
  }
}

// partial[z][j][r] = sum_{k in slice z} M[r][k] X[j][k]
__global__ void __launch_bounds__(256)
k_extrude_gemm(int W, int K, int J, int kslice, const float* __restrict__ M,
               const float* __restrict__ X, float* __restrict__ partial) {
  __shared__ float sA[kTM][kTK + 1];
  __shared__ float sX[kTJ][kTK + 1];
  const int r0 = blockIdx.x * kTM;
  const int j0 = blockIdx.y * kTJ;
  const int kb = blockIdx.z * kslice;
  const int ke = min(K, kb + kslice);
  const int tid = threadIdx.x;
  const int tr = tid / 16;  // 16 row groups of 4
  const int tj = tid % 16;  // 16 job groups of 2
  float acc[4][2] = {};
  for (int k0 = kb; k0 < ke; k0 += kTK) {
    for (int i = tid; i < kTM * kTK; i += 256) {
      const int rr = i / kTK, kk = i % kTK;
      const int r = r0 + rr, k = k0 + kk;
      sA[rr][kk] = (r < W && k < ke) ? M[(size_t)r * K + k] : 0.f;
    }
    for (int i = tid; i < kTJ * kTK; i += 256) {
      const int jj = i / kTK, kk = i % kTK;
      const int j = j0 + jj, k = k0 + kk;
      sX[jj][kk] = (j < J && k < ke) ? X[(size_t)j * K + k] : 0.f;
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < kTK; ++kk) {
      float a[4], x[2];
#pragma unroll
      for (int u = 0; u < 4; ++u) a[u] = sA[tr * 4 + u][kk];
#pragma unroll
      for (int v = 0; v < 2; ++v) x[v] = sX[tj * 2 + v][kk];
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 2; ++v) acc[u][v] = fmaf(a[u], x[v], acc[u][v]);
    }
    __syncthreads();
  }
  float* pz = partial + (size_t)blockIdx.z * J * W;
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 2; ++v) {
      const int r = r0 + tr * 4 + u, j = j0 + tj * 2 + v;
      if (r < W && j < J) pz[(size_t)j * W + r] = acc[u][v];
    }
}

// The same partial products for the extrusion shapes (W ~ 10^3 rows, tens to
// hundreds of jobs, K = (m+1) W): 256 threads as 16 row lanes x 16 job lanes,
// thread (tm, tj) accumulating rows {4 tm + u, 64 + 4 tm + u} (u < 4) x jobs
// tj TJ + v (v < TJ) in registers: per K value two 128-bit shared loads of A
// and TJ broadcast loads of X feed 8 TJ FMAs. Both operands are row-major with
// an odd K (no 16-byte alignment), so each stage is read with coalesced
// scalar loads into registers while the previous stage is multiplied, then
// stored K-major into the other shared buffer.
template <int TJ>
__global__ void __launch_bounds__(256, TJ >= 9 ? 1 : 2)
k_extrude_gemm_tiled(int W, int K, int J, int kslice, const float* __restrict__ M,
                     const float* __restrict__ X, float* __restrict__ partial) {
  constexpr int BJ = 16 * TJ;
  constexpr int AP = kGBM + 4;  // padded K-major rows (16-byte aligned)
  constexpr int XP = BJ + 4;
  __shared__ __align__(16) float sA[2][kGBK][AP];
  __shared__ __align__(16) float sX[2][kGBK][XP];
  const int tid = threadIdx.x;
  const int tm = tid & 15, tj = tid >> 4;
  const int r0 = blockIdx.x * kGBM, j0 = blockIdx.y * BJ;
  const int kb = blockIdx.z * kslice, ke = min(K, kb + kslice);
  // staging map: K offset lk, rows / jobs lr + 16 i
  const int lk = tid & 15, lr = tid >> 4;
  const uint64_t pol = l2_evict_last();  // the operator is re-read every row step
  float ra[8], rx[TJ];
  auto load = [&](int k0) {
    const int k = k0 + lk;
    const bool kin = k < ke;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int r = r0 + lr + 16 * i;
      ra[i] = (kin && r < W) ? ld_keep(M + (size_t)r * K + k, pol) : 0.f;
    }
#pragma unroll
    for (int v = 0; v < TJ; ++v) {
      const int j = j0 + lr + 16 * v;
      rx[v] = (kin && j < J) ? __ldg(X + (size_t)j * K + k) : 0.f;
    }
  };
  auto store = [&](int b) {
#pragma unroll
    for (int i = 0; i < 8; ++i) sA[b][lk][lr + 16 * i] = ra[i];
#pragma unroll
    for (int v = 0; v < TJ; ++v) sX[b][lk][lr + 16 * v] = rx[v];
  };
  float acc[8][TJ];
#pragma unroll
  for (int u = 0; u < 8; ++u)
#pragma unroll
    for (int v = 0; v < TJ; ++v) acc[u][v] = 0.f;
  load(kb);
  store(0);
  __syncthreads();
  int b = 0;
  for (int k0 = kb; k0 < ke; k0 += kGBK) {
    const bool more = k0 + kGBK < ke;
    if (more) load(k0 + kGBK);
#pragma unroll
    for (int kk = 0; kk < kGBK; ++kk) {
      const float4 a0 = *(const float4*)&sA[b][kk][tm * 4];
      const float4 a1 = *(const float4*)&sA[b][kk][64 + tm * 4];
      const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      float x[TJ];
#pragma unroll
      for (int v = 0; v < TJ; ++v) x[v] = sX[b][kk][tj * TJ + v];
#pragma unroll
      for (int u = 0; u < 8; ++u)
#pragma unroll
        for (int v = 0; v < TJ; ++v) acc[u][v] = fmaf(a[u], x[v], acc[u][v]);
    }
    // the other buffer was last read before the previous barrier
    if (more) store(b ^ 1);
    __syncthreads();
    b ^= 1;
  }
  float* pz = partial + (size_t)blockIdx.z * J * W;
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    const int r = r0 + (u < 4 ? 4 * tm + u : 64 + 4 * tm + (u - 4));
#pragma unroll
    for (int v = 0; v < TJ; ++v) {
      const int j = j0 + tj * TJ + v;
      if (r < W && j < J) pz[(size_t)j * W + r] = acc[u][v];
    }
  }
}

// new row = sum of the split-K slices (+ the newest stencil row r1, ring
// row head - 1, in the increment form: the slices then hold a correction)
__global__ void k_extrude_reduce(int W, int J, int cap, int nsplit, const float* __restrict__ partial,
                                 const RingDst dst, float* __restrict__ buf, int incr) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (r >= W || j >= J) return;
  float s = 0.f;
  for (int z = 0; z < nsplit; ++z) s += __ldcs(partial + ((size_t)z * J + j) * W + r);
  float* slab = buf + (size_t)dst.d[j].x * cap * W;
  if (incr) s += slab[(size_t)ring_back(dst.d[j].y, 1, cap) * W + r];
  slab[(size_t)dst.d[j].y * W + r] = s;
}

// ---------------------------------------------------------------- readout
struct RLayer {
  int screen, row_max, anchor_phys;
  long long ca, sa, ra, rp;  // fixed-point (2^-40) constants
};
constexpr int kMaxReadoutLayers = 64;
struct RLayers {
  RLayer l[kMaxReadoutLayers];
};

constexpr int kFix = 40;

__device__ __forceinline__ void split_fixed(long long v, int& i, float& f) {
  i = (int)(v >> kFix);
  f = (float)(v & ((1ll << kFix) - 1)) * (1.0f / 1099511627776.0f);
}

__device__ __forceinline__ float sincpi_f(float x) {
  if (x == 0.f) return 1.f;
  return sinpif(x) / (3.14159265358979323846f * x);
}

template <int T>
__device__ __forceinline__ void taps(float t, float* w) {
  if (T == 2) {
    w[0] = 1.f - t;
    w[1] = t;
  } else if (T == 4) {
    const float t2 = t * t, t3 = t2 * t;
    w[0] = 0.5f * (-t + 2.f * t2 - t3);
    w[1] = 0.5f * (2.f - 5.f * t2 + 3.f * t3);
    w[2] = 0.5f * (t + 4.f * t2 - 3.f * t3);
    w[3] = 0.5f * (-t2 + t3);
  } else {
    float tot = 0.f;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const float x = t - (float)(k - 2);
      w[k] = sincpi_f(x) * sincpi_f(x * (1.0f / 3.0f));
      tot += w[k];
    }
    const float inv = 1.f / tot;
#pragma unroll
    for (int k = 0; k < 6; ++k) w[k] *= inv;
  }
}

template <int T>
__global__ void __launch_bounds__(256)
k_readout(int n, int W, int cap, int L, RLayers P, const float* __restrict__ buf, float scale,
          float* __restrict__ out) {
  const int y = blockIdx.x * blockDim.x + threadIdx.x;
  const int x = blockIdx.y;
  if (y >= n) return;
  const int off0 = (T == 2) ? 0 : (T == 4 ? -1 : -2);
  const long long kx = 2ll * x - (n - 1), ky = 2ll * y - (n - 1);
  float acc = 0.f;
  for (int l = 0; l < L; ++l) {
    const RLayer p = P.l[l];
    const long long rowf = kx * p.ca + ky * p.sa + p.ra;
    const long long colf = -kx * p.sa + ky * p.ca + p.rp;
    int r0, c0;
    float fr, fc;
    split_fixed(rowf, r0, fr);
    split_fixed(colf, c0, fc);
    float wr[T], wc[T];
    taps<T>(fr, wr);
    taps<T>(fc, wc);
    const float* slab = buf + (size_t)p.screen * cap * W;
    int cc[T];
#pragma unroll
    for (int b = 0; b < T; ++b) cc[b] = min(max(c0 + off0 + b, 0), W - 1);
    float val = 0.f;
#pragma unroll
    for (int a = 0; a < T; ++a) {
      int rr = min(max(r0 + off0 + a, 0), p.row_max);
      int phys = p.anchor_phys + rr;
      if (phys >= cap) phys -= cap;
      const float* row = slab + (size_t)phys * W;
      float rs = 0.f;
#pragma unroll
      for (int b = 0; b < T; ++b) rs = fmaf(wc[b], __ldg(row + cc[b]), rs);
      val = fmaf(wr[a], rs, val);
    }
    acc += val;
  }
  out[(size_t)x * n + y] = scale * acc;
}

template <int T>
__global__ void k_rows_sample(int n, int cap, int anchor_phys, int row_max, int i0, float t,
                              const float* __restrict__ buf, float* __restrict__ out) {
  const int y = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y;
  if (y >= n) return;
  const int off0 = (T == 2) ? 0 : (T == 4 ? -1 : -2);
  float w[T];
  taps<T>(t, w);
  float v = 0.f;
#pragma unroll
  for (int a = 0; a < T; ++a) {
    const int rr = min(max(i0 + i + off0 + a, 0), row_max);
    int phys = anchor_phys + rr;
    if (phys >= cap) phys -= cap;
    v = fmaf(w[a], buf[(size_t)phys * n + y], v);
  }
  out[(size_t)i * n + y] = v;
}

static inline size_t al256(size_t x) { return (x + 255) & ~size_t(255); }

// tensor-core launchers (extrude_tc.cu)
int tc_max_jobs(int terms);
size_t tc_operator_bytes(int W, int K, int G, int terms);
size_t tc_btile_bytes(int W, int K, int J, int terms);
size_t tc_partial_floats(int W, int K, int J, int terms);
int tc_prepare_launch(int W, int K, int G, const float* M, int terms, void* tiles, cudaStream_t s);
int tc_gemm_launch(int W, int K, int J, int terms, const uint8_t* At, const uint8_t* Bt,
                   float* partial, int* nz_out, cudaStream_t s);

// The sparse points of a stencil, checked against the ring and the width.
static int sparse_dev(const char* who, const pt_sparse_stencil* sp, int W, int m, int cap,
                      SparseDev& out) {
  out = SparseDev{};
  if (!sp) return PT_OK;
  if (sp->count < 0 || sp->count > PT_MAX_SPARSE)
    return fail(PT_ERR_ARG, std::string(who) + ": sparse count must be in [0, 64]");
  out.n = sp->count;
  for (int i = 0; i < sp->count; ++i) {
    if (sp->depth[i] <= m || (cap > 0 && sp->depth[i] >= cap) || sp->column[i] < 0 ||
        sp->column[i] >= W)
      return fail(PT_ERR_ARG, std::string(who) +
                                  ": sparse points need m < depth < cap and 0 <= column < W");
    out.depth[i] = sp->depth[i];
    out.col[i] = sp->column[i];
  }
  return PT_OK;
}

// Jobs per thread of the tiled GEMM and its split-K: one wave of resident
// CTAs, each slice at least 8 K steps long.
static int tiled_tj(int J) { return J <= 32 ? 2 : (J <= 64 ? 4 : 9); }
static int tiled_split(int W, int J, int K) {
  const int bj = 16 * tiled_tj(J);
  const int ctas = ((W + kGBM - 1) / kGBM) * ((J + bj - 1) / bj);
  const int per_sm = tiled_tj(J) >= 9 ? 1 : 2;  // resident CTAs (registers)
  int s = std::max(1, std::min(kMaxSplitTiled, per_sm * 152 / ctas));
  return std::max(1, std::min(s, K / (8 * kGBK)));
}
static void launch_gemm_tiled(int W, int K, int J, const float* M, const float* X, float* partial,
                              int* nz_out, cudaStream_t s) {
  const int tj = tiled_tj(J), bj = 16 * tj;
  const int nsplit = tiled_split(W, J, K);
  const int kslice = ((K + nsplit - 1) / nsplit + kGBK - 1) / kGBK * kGBK;
  const int nz = (K + kslice - 1) / kslice;
  const dim3 grid((W + kGBM - 1) / kGBM, (J + bj - 1) / bj, nz);
  ProfScope ps("k_extrude_gemm", s);
  if (tj == 2) k_extrude_gemm_tiled<2><<<grid, 256, 0, s>>>(W, K, J, kslice, M, X, partial);
  else if (tj == 4) k_extrude_gemm_tiled<4><<<grid, 256, 0, s>>>(W, K, J, kslice, M, X, partial);
  else k_extrude_gemm_tiled<9><<<grid, 256, 0, s>>>(W, K, J, kslice, M, X, partial);
  *nz_out = nz;
}

static int split_for(int W, int J, int K) {
  const int ctas = ((W + kTM - 1) / kTM) * ((J + kTJ - 1) / kTJ);
  int s = std::max(1, std::min(kMaxSplit, (2 * 152 + ctas - 1) / ctas));
  // keep each slice at least 4 K-steps long
  s = std::max(1, std::min(s, K / (4 * kTK)));
  return s;
}

}  // namespace pt

using namespace pt;

// FP32-form workspace: X (J, K) | correction B tiles | partials of the FP32
// GEMM (up to kMaxSplitTiled slices) followed by those of the correction.
// (the partials are followed by the anchor's (s, c) pairs: up to
// kAnchorSplit x J x 64 float2)
constexpr int kAnchorSplit = 192;
struct Fp32Work {
  size_t x, lo_tiles, partial, total;
  int lo_nz, max_nz;
};
static Fp32Work fp32_work(int W, int m, int n_sparse, int J) {
  Fp32Work w{};
  const int K = (m + 1) * W + n_sparse, Kz = m * W + n_sparse;
  w.x = al256((size_t)J * K * sizeof(float));
  w.lo_tiles = al256(tc_btile_bytes(W, Kz, J, 1));
  w.lo_nz = (int)(tc_partial_floats(W, Kz, J, 1) / ((size_t)J * W));
  w.max_nz = std::max(kMaxSplit, kMaxSplitTiled) + w.lo_nz;
  w.partial = al256((size_t)w.max_nz * J * W * sizeof(float)) +
              al256((size_t)kAnchorSplit * J * 64 * sizeof(float2));
  w.total = w.x + w.lo_tiles + w.partial;
  return w;
}

extern "C" size_t pt_extrude_workspace_bytes(int W, int m, int n_sparse, int max_jobs) {
  if (W < 1 || m < 1 || max_jobs < 1 || n_sparse < 0 || n_sparse > PT_MAX_SPARSE) return 0;
  return fp32_work(W, m, n_sparse, std::min(max_jobs, kJobsPerLaunch)).total;
}

// The operator of one form: FP32 [A | B] (SIMT GEMM) or its bf16 term tiles
// (tensor cores, `terms` = 2 or 3).
struct ExtrudeForm {
  int terms;               // 0: FP32
  const float* M;          // (G, W, K) FP32
  const uint8_t* tiles;    // tensor-core operator tiles
  const uint8_t* lo;       // FP32 form: 1-term tiles of A - (float)A, or NULL
  const pt_extrude_anchor* anchor;  // FP32 form: low-order anchor, or NULL
  int incr;                // the operator is in increment form
};

static int extrude_jobs(const char* who, const ExtrudeForm& form, int W, int m,
                        const pt_sparse_stencil* sparse, int cap, int G, float* buf, int n_jobs,
                        const pt_extrude_job* jobs, const float* noise, void* work,
                        size_t work_bytes, cudaStream_t s) {
  if (W < 1 || m < 1 || cap < m + 1 || G < 1) return fail(PT_ERR_ARG, std::string(who) + ": bad sizes");
  SparseDev sp;
  if (int rc = sparse_dev(who, sparse, W, m, cap, sp)) return rc;
  if ((form.terms == 0 && !form.M) || (form.terms != 0 && !form.tiles) || !buf ||
      (n_jobs > 0 && !jobs))
    return fail(PT_ERR_ARG, std::string(who) + ": NULL pointer");
  if (n_jobs == 0) return PT_OK;
  // group jobs by (step, group), validating order and ranges
  int max_j = 0;
  {
    int cur = 1, prev_step = jobs[0].step;
    for (int i = 0; i < n_jobs; ++i) {
      const pt_extrude_job& jb = jobs[i];
      if (jb.group < 0 || jb.group >= G)
        return fail(PT_ERR_ARG, std::string(who) + ": job group out of range");
      if (jb.head < 0 || jb.head >= cap)
        return fail(PT_ERR_ARG, std::string(who) + ": job head out of range");
      if (jb.screen < 0) return fail(PT_ERR_ARG, std::string(who) + ": negative screen index");
      if (i > 0) {
        if (jb.step < prev_step)
          return fail(PT_ERR_ARG, std::string(who) + ": jobs must be sorted by step");
        cur = (jb.step == prev_step) ? cur + 1 : 1;
      }
      prev_step = jb.step;
      max_j = std::max(max_j, cur);
    }
  }
  const size_t need = form.terms ? pt_extrude_tc_workspace_bytes(W, m, sp.n, max_j, form.terms)
                                 : pt_extrude_workspace_bytes(W, m, sp.n, max_j);
  if (!work || work_bytes < need) return fail(PT_ERR_ARG, std::string(who) + ": workspace too small");
  const int K = (m + 1) * W + sp.n, Kz = m * W + sp.n;
  const int per_launch = form.terms ? tc_max_jobs(form.terms) : kJobsPerLaunch;
  const int jcap = std::min(max_j, per_launch);
  // FP32: X (jcap, K), correction B tiles, partials; tensor cores: B tiles then partials
  const Fp32Work fw = fp32_work(W, m, sp.n, jcap);
  const size_t first = form.terms ? al256(tc_btile_bytes(W, K, jcap, form.terms))
                                  : fw.x + fw.lo_tiles;
  float* X = (float*)work;
  uint8_t* Bt = (uint8_t*)work;
  uint8_t* Blo = (uint8_t*)work + fw.x;
  float* partial = (float*)((char*)work + first);
  const size_t op_group = form.terms ? tc_operator_bytes(W, K, 1, form.terms) : 0;
  const size_t lo_group = tc_operator_bytes(W, Kz, 1, 1);
  std::vector<GatherJob> hj;
  // The split-K reduce of a launch is deferred: when the next FP32 launch
  // extrudes the same screens in the same order one row further, its gather
  // makes the pending rows (they are its newest stencil rows); otherwise, and
  // after the last launch, the reduce runs on its own.
  struct Pending {
    bool on = false;
    int J = 0, nz = 0;
    RingDst dst;
  } pend;
  auto flush = [&]() -> int {
    if (!pend.on) return PT_OK;
    {
      ProfScope ps("k_extrude_reduce", s);
      k_extrude_reduce<<<dim3((W + 255) / 256, pend.J), 256, 0, s>>>(W, pend.J, cap, pend.nz,
                                                                    partial, pend.dst, buf,
                                                                    form.incr);
    }
    count_launch_e(1);
    pend.on = false;
    return check_launch(who);
  };
  int i = 0;
  while (i < n_jobs) {
    int e = i;
    while (e < n_jobs && jobs[e].step == jobs[i].step) ++e;
    // within one step, one launch chain per group
    std::map<int, std::vector<int>> by_group;
    for (int q = i; q < e; ++q) by_group[jobs[q].group].push_back(q);
    for (auto& kv : by_group) {
      hj.clear();
      for (int q : kv.second) {
        const pt_extrude_job& jb = jobs[q];
        hj.push_back(GatherJob{jb.screen, jb.head, jb.bscale, jb.key, jb.row, (long long)jb.noise_off});
      }
      for (size_t b = 0; b < hj.size(); b += per_launch) {
        const int J = (int)std::min<size_t>(per_launch, hj.size() - b);
        JobParams jp;
        for (int q = 0; q < J; ++q) jp.j[q] = hj[b + q];
        RingDst dst;
        for (int q = 0; q < J; ++q) dst.d[q] = make_int2(jp.j[q].screen, jp.j[q].head);
        // FP32 only: the tensor-core gather's threads each make 8 consecutive
        // values, so summing the slices there costs more than the reduce
        // (with the anchor every new row is anchored before it is read)
        bool fuse = form.terms == 0 && !form.anchor && !form.incr && pend.on && pend.J == J;
        for (int q = 0; fuse && q < J; ++q)
          fuse = pend.dst.d[q].x == dst.d[q].x && (pend.dst.d[q].y + 1) % cap == dst.d[q].y;
        if (!fuse)
          if (int rc = flush()) return rc;
        const float* prev = fuse ? partial : nullptr;
        const int prev_nz = fuse ? pend.nz : 0;
        pend.on = false;
        int nz = 0;
        if (form.terms == 0) {
          {
            ProfScope ps("k_extrude_gather", s);
            k_extrude_gather<<<dim3((W + 511) / 512, m + 1 + (sp.n > 0), J), 256, 0, s>>>(
                W, m, cap, buf, jp, J, sp, noise, X, prev, prev_nz, form.incr);
          }
          const float* Mg = form.M + (size_t)kv.first * W * K;
          launch_gemm_tiled(W, K, J, Mg, X, partial, &nz, s);
          if (form.lo) {
            // + (A - (float)A) X on the tensor cores, into the slices after the
            // FP32 GEMM's: without it the float32 rounding of A is a bias that
            // the recursion accumulates row after row
            const int NP = std::max(16, (J + 15) / 16 * 16);
            const int nkc = (Kz + tc::kTcKc - 1) / tc::kTcKc;
            const size_t items = (size_t)nkc * (tc::kTcKc / 8) * NP;
            {
              ProfScope ps("k_lo_operand", s);
              k_lo_operand<<<(unsigned)std::min<size_t>((items + 255) / 256, 152 * 4), 256, 0,
                             s>>>(X, J, K, Kz, NP, nkc, Blo);
            }
            count_launch_e();
            int nz_lo = 0;
            if (int rc = tc_gemm_launch(W, Kz, J, 1, form.lo + (size_t)kv.first * lo_group, Blo,
                                        partial + (size_t)nz * J * W, &nz_lo, s))
              return rc;
            nz += nz_lo;
          }
        } else {
          const int NP = std::max(16, (J + 15) / 16 * 16);
          const int nkc = (K + tc::kTcKc - 1) / tc::kTcKc;
          const size_t items = (size_t)nkc * (tc::kTcKc / 8) * NP;
          {
            ProfScope ps("k_tc_gather", s);
            k_tc_gather<<<(unsigned)std::min<size_t>((items + 255) / 256, 152 * 8), 256, 0, s>>>(
                W, m, cap, buf, jp, J, sp, NP, nkc, form.terms, noise, Bt, form.incr);
          }
          if (int rc = tc_gemm_launch(W, K, J, form.terms, form.tiles + (size_t)kv.first * op_group,
                                      Bt, partial, &nz, s))
            return rc;
        }
        pend.on = true;
        pend.J = J;
        pend.nz = nz;
        pend.dst = dst;
        if (form.anchor) {
          if (int rc = flush()) return rc;
          const AnchorDev an{(const f2p*)form.anchor->t_hi, (const f2p*)form.anchor->t_lo,
                             form.anchor->u};
          const int R = form.anchor->modes, Kt = K + (form.incr ? 2 : 1) * W;
          const int jb = (J + 63) / 64;
          // about four CTAs per SM (a single wave of two left SMs idle in its
          // tail), slices of 32 or more columns
          const int nsplit = std::max(1, std::min(std::min(kAnchorSplit, (Kt + 31) / 32),
                                                  (4 * 152 + jb - 1) / jb));
          const int kslice = ((Kt + nsplit - 1) / nsplit + 31) / 32 * 32;
          const int nz_a = (Kt + kslice - 1) / kslice;
          float2* apart =
              (float2*)((char*)partial + al256((size_t)fw.max_nz * J * W * sizeof(float)));
          {
            ProfScope ps("k_anchor", s);
            if (R == 32) {
              k_anchor_gemm<32><<<dim3(jb, nz_a), 256, 0, s>>>(W, K, Kz, cap, kv.first, J,
                                                               kslice, form.incr, dst, X, an, buf,
                                                               apart);
              k_anchor_apply<32><<<J, 256, 0, s>>>(W, cap, J, nz_a, dst, apart, an.u, buf);
            } else {
              k_anchor_gemm<64><<<dim3(jb, nz_a), 256, 0, s>>>(W, K, Kz, cap, kv.first, J,
                                                               kslice, form.incr, dst, X, an, buf,
                                                               apart);
              k_anchor_apply<64><<<J, 256, 0, s>>>(W, cap, J, nz_a, dst, apart, an.u, buf);
            }
          }
          count_launch_e(2);
        }
        count_launch_e(form.terms ? 1 : 2);
        if (int rc = check_launch(who)) return rc;
      }
    }
    i = e;
  }
  return flush();
}

namespace pt {
__global__ void k_matmul_reduce(int R, int J, int nsplit, const float* __restrict__ partial,
                                float* __restrict__ out) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (r >= R || j >= J) return;
  float s = 0.f;
  for (int z = 0; z < nsplit; ++z) s += partial[((size_t)z * J + j) * R + r];
  out[(size_t)j * R + r] = s;
}
}  // namespace pt

namespace pt {
constexpr int kMaxBoilRows = 64;
struct RowScales {
  float v[kMaxBoilRows];
};
// out[r][c] = scale[r] * N(0, 1), Philox keyed by (key, r * cols + c, call).
__global__ void k_fill_normals(uint64_t key, uint64_t call, int rows, int cols, RowScales sc,
                               float* __restrict__ out) {
  const size_t total = (size_t)rows * cols;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; 2 * i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const float2 z = philox_cnormal(key, i, call, kDomainBoilSeed);
    const size_t e = 2 * i;
    out[e] = sc.v[e / cols] * z.x;
    if (e + 1 < total) out[e + 1] = sc.v[(e + 1) / cols] * z.y;
  }
}

// ring rows phys0, phys0 + 1, ... (mod cap) of one screen: buf = a buf + b fresh
__global__ void k_ring_blend(int W, int cap, float* __restrict__ screen, int phys0, int h, float a,
                             float b, const float* __restrict__ fresh) {
  const size_t total = (size_t)h * W;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / W), c = (int)(i % W);
    int p = phys0 + r;
    if (p >= cap) p -= cap;
    float* d = screen + (size_t)p * W + c;
    *d = fmaf(a, *d, b * fresh[i]);
  }
}
}  // namespace pt

extern "C" int pt_fill_normals(uint64_t key, uint64_t call, int rows, int cols,
                               const float* row_scale, float* out, void* stream) {
  if (rows < 1 || cols < 1 || rows > kMaxBoilRows)
    return fail(PT_ERR_ARG, "pt_fill_normals: rows must be in [1, 64], cols >= 1");
  if (!row_scale || !out) return fail(PT_ERR_ARG, "pt_fill_normals: NULL pointer");
  RowScales sc{};
  for (int r = 0; r < rows; ++r) sc.v[r] = row_scale[r];
  const size_t pairs = ((size_t)rows * cols + 1) / 2;
  cudaStream_t s = (cudaStream_t)stream;
  k_fill_normals<<<(unsigned)std::min<size_t>((pairs + 255) / 256, 1024), 256, 0, s>>>(
      key, call, rows, cols, sc, out);
  count_launch_e();
  return check_launch("pt_fill_normals");
}

extern "C" int pt_ring_blend(int W, int cap, float* screen, int phys0, int h, float a, float b,
                             const float* fresh, void* stream) {
  if (W < 1 || cap < 1 || h < 0 || h > cap || phys0 < 0 || phys0 >= cap)
    return fail(PT_ERR_ARG, "pt_ring_blend: bad sizes");
  if (!screen || (h > 0 && !fresh)) return fail(PT_ERR_ARG, "pt_ring_blend: NULL pointer");
  if (h == 0) return PT_OK;
  const size_t total = (size_t)h * W;
  cudaStream_t s = (cudaStream_t)stream;
  k_ring_blend<<<(unsigned)std::min<size_t>((total + 255) / 256, 4096), 256, 0, s>>>(
      W, cap, screen, phys0, h, a, b, fresh);
  count_launch_e();
  return check_launch("pt_ring_blend");
}

extern "C" size_t pt_matmul_nt_workspace_bytes(int R, int K, int J) {
  if (R < 1 || K < 1 || J < 1) return 0;
  return (size_t)kMaxSplit * J * R * sizeof(float);
}

extern "C" int pt_matmul_nt(int R, int K, int J, const float* M, const float* X, float* out,
                            void* work, size_t work_bytes, void* stream) {
  if (R < 1 || K < 1 || J < 1) return fail(PT_ERR_ARG, "pt_matmul_nt: bad sizes");
  if (!M || !X || !out) return fail(PT_ERR_ARG, "pt_matmul_nt: NULL pointer");
  if (!work || work_bytes < pt_matmul_nt_workspace_bytes(R, K, J))
    return fail(PT_ERR_ARG, "pt_matmul_nt: workspace too small");
  if ((J + kTJ - 1) / kTJ > 65535) return fail(PT_ERR_UNSUPPORTED, "pt_matmul_nt: J too large");
  cudaStream_t s = (cudaStream_t)stream;
  const int nsplit = split_for(R, J, K);
  const int kslice = ((K + nsplit - 1) / nsplit + kTK - 1) / kTK * kTK;
  const int nz = (K + kslice - 1) / kslice;
  float* partial = (float*)work;
  {
    ProfScope ps("k_extrude_gemm", s);
    k_extrude_gemm<<<dim3((R + kTM - 1) / kTM, (J + kTJ - 1) / kTJ, nz), 256, 0, s>>>(
        R, K, J, kslice, M, X, partial);
  }
  k_matmul_reduce<<<dim3((R + 255) / 256, J), 256, 0, s>>>(R, J, nz, partial, out);
  count_launch_e(2);
  return check_launch("pt_matmul_nt");
}

static int anchor_ok(const char* who, const pt_extrude_anchor* a) {
  if (!a) return PT_OK;
  if (a->modes != 32 && a->modes != 64)
    return fail(PT_ERR_ARG, std::string(who) + ": the anchor takes 32 or 64 modes");
  if (!a->t_hi || !a->t_lo || !a->u)
    return fail(PT_ERR_ARG, std::string(who) + ": anchor with a NULL table");
  if ((((uintptr_t)a->t_hi) | ((uintptr_t)a->t_lo)) & 7)
    return fail(PT_ERR_ARG, std::string(who) + ": anchor tables must be 8-byte aligned");
  return PT_OK;
}

extern "C" int pt_extrude_rows(int W, int m, const pt_sparse_stencil* sparse, int increments,
                               int cap, int G, const float* M, const void* lo_tiles,
                               const pt_extrude_anchor* anchor, float* buf, int n_jobs,
                               const pt_extrude_job* jobs, const float* noise, void* work,
                               size_t work_bytes, void* stream) {
  if (lo_tiles && ((uintptr_t)lo_tiles & 255) != 0)
    return fail(PT_ERR_ARG, "pt_extrude_rows: correction tiles must be 256-byte aligned");
  if (int rc = anchor_ok("pt_extrude_rows", anchor)) return rc;
  return extrude_jobs("pt_extrude_rows",
                      ExtrudeForm{0, M, nullptr, (const uint8_t*)lo_tiles, anchor, increments != 0},
                      W, m, sparse, cap, G, buf, n_jobs, jobs, noise, work, work_bytes,
                      (cudaStream_t)stream);
}

// Jobs of `counts[s]` row steps on every screen s, step-major (the order of
// the noise rows), advancing top[s].
static int batch_jobs(const char* who, int W, int cap, int S, const int32_t* group,
                      const float* bscale, const uint64_t* key, int64_t* top,
                      const int32_t* counts, std::vector<pt_extrude_job>& jobs) {
  if (S < 1 || !group || !bscale || !key || !top || !counts)
    return fail(PT_ERR_ARG, std::string(who) + ": bad screen arrays");
  int steps = 0;
  for (int s = 0; s < S; ++s) {
    if (counts[s] < 0 || top[s] < 0) return fail(PT_ERR_ARG, std::string(who) + ": negative count");
    steps = std::max(steps, (int)counts[s]);
  }
  jobs.clear();
  jobs.reserve((size_t)S * steps);
  int64_t noff = 0;
  for (int k = 0; k < steps; ++k)
    for (int s = 0; s < S; ++s) {
      if (k >= counts[s]) continue;
      pt_extrude_job j{};
      j.screen = s;
      j.group = group[s];
      j.head = (int32_t)(top[s] % cap);
      j.step = k;
      j.bscale = bscale[s];
      j.key = key[s];
      j.row = (uint64_t)top[s];
      j.noise_off = noff;
      noff += W;
      top[s] += 1;
      jobs.push_back(j);
    }
  return PT_OK;
}

extern "C" int pt_extrude_batch(int W, int m, const pt_sparse_stencil* sparse, int increments,
                                int cap, int n_groups, const float* M, const void* lo_tiles,
                                const pt_extrude_anchor* anchor, float* buf, int S,
                                const int32_t* group, const float* bscale, const uint64_t* key,
                                int64_t* top, const int32_t* counts, const float* noise,
                                void* work, size_t work_bytes, void* stream) {
  if (lo_tiles && ((uintptr_t)lo_tiles & 255) != 0)
    return fail(PT_ERR_ARG, "pt_extrude_batch: correction tiles must be 256-byte aligned");
  if (int rc = anchor_ok("pt_extrude_batch", anchor)) return rc;
  std::vector<pt_extrude_job> jobs;
  if (int rc = batch_jobs("pt_extrude_batch", W, cap, S, group, bscale, key, top, counts, jobs))
    return rc;
  return extrude_jobs("pt_extrude_batch",
                      ExtrudeForm{0, M, nullptr, (const uint8_t*)lo_tiles, anchor, increments != 0},
                      W, m, sparse, cap, n_groups, buf, (int)jobs.size(), jobs.data(), noise, work,
                      work_bytes, (cudaStream_t)stream);
}

extern "C" size_t pt_extrude_lo_bytes(int W, int m, int n_sparse, int n_groups) {
  if (W < 1 || m < 1 || n_groups < 1 || n_sparse < 0 || n_sparse > PT_MAX_SPARSE) return 0;
  return tc_operator_bytes(W, m * W + n_sparse, n_groups, 1);
}

extern "C" int pt_extrude_lo_prepare(int W, int m, int n_sparse, int n_groups, const float* Mlo,
                                     void* tiles, size_t tiles_bytes, void* stream) {
  if (W < 1 || m < 1 || n_groups < 1 || n_sparse < 0 || n_sparse > PT_MAX_SPARSE)
    return fail(PT_ERR_ARG, "pt_extrude_lo_prepare: bad sizes");
  if (!Mlo || !tiles) return fail(PT_ERR_ARG, "pt_extrude_lo_prepare: NULL pointer");
  const int Kz = m * W + n_sparse;
  if (tiles_bytes < tc_operator_bytes(W, Kz, n_groups, 1))
    return fail(PT_ERR_ARG, "pt_extrude_lo_prepare: tile buffer too small");
  if (((uintptr_t)tiles & 255) != 0)
    return fail(PT_ERR_ARG, "pt_extrude_lo_prepare: tiles must be 256-byte aligned");
  return tc_prepare_launch(W, Kz, n_groups, Mlo, 1, tiles, (cudaStream_t)stream);
}

static bool tc_sizes_ok(int W, int m, int n_sparse, int n, int terms) {
  return W >= 1 && m >= 1 && n >= 1 && n_sparse >= 0 && n_sparse <= PT_MAX_SPARSE &&
         (terms == 2 || terms == 3);
}

extern "C" size_t pt_extrude_tc_operator_bytes(int W, int m, int n_sparse, int n_groups,
                                               int terms) {
  if (!tc_sizes_ok(W, m, n_sparse, n_groups, terms)) return 0;
  return tc_operator_bytes(W, (m + 1) * W + n_sparse, n_groups, terms);
}

extern "C" int pt_extrude_tc_prepare(int W, int m, int n_sparse, int n_groups, const float* M,
                                     int terms, void* tiles, size_t tiles_bytes, void* stream) {
  if (W < 1 || m < 1 || n_groups < 1 || n_sparse < 0 || n_sparse > PT_MAX_SPARSE)
    return fail(PT_ERR_ARG, "pt_extrude_tc_prepare: bad sizes");
  if (terms != 2 && terms != 3) return fail(PT_ERR_ARG, "pt_extrude_tc_prepare: terms must be 2 or 3");
  if (!M || !tiles) return fail(PT_ERR_ARG, "pt_extrude_tc_prepare: NULL pointer");
  const int K = (m + 1) * W + n_sparse;
  if (tiles_bytes < tc_operator_bytes(W, K, n_groups, terms))
    return fail(PT_ERR_ARG, "pt_extrude_tc_prepare: tile buffer too small");
  if (((uintptr_t)tiles & 255) != 0)
    return fail(PT_ERR_ARG, "pt_extrude_tc_prepare: tiles must be 256-byte aligned");
  return tc_prepare_launch(W, K, n_groups, M, terms, tiles, (cudaStream_t)stream);
}

extern "C" size_t pt_extrude_tc_workspace_bytes(int W, int m, int n_sparse, int max_jobs,
                                                int terms) {
  if (!tc_sizes_ok(W, m, n_sparse, max_jobs, terms)) return 0;
  const int J = std::min(max_jobs, tc_max_jobs(terms));
  const int K = (m + 1) * W + n_sparse;
  return al256(tc_btile_bytes(W, K, J, terms)) + al256(tc_partial_floats(W, K, J, terms) * sizeof(float));
}

extern "C" int pt_extrude_batch_tc(int W, int m, const pt_sparse_stencil* sparse,
                                   int increments, int cap, int n_groups, const void* tiles,
                                   int terms, float* buf, int S,
                                   const int32_t* group, const float* bscale,
                                   const uint64_t* key, int64_t* top, const int32_t* counts,
                                   const float* noise, void* work, size_t work_bytes,
                                   void* stream) {
  if (terms != 2 && terms != 3) return fail(PT_ERR_ARG, "pt_extrude_batch_tc: terms must be 2 or 3");
  if (work && ((uintptr_t)work & 255) != 0)
    return fail(PT_ERR_ARG, "pt_extrude_batch_tc: workspace must be 256-byte aligned");
  if (tiles && ((uintptr_t)tiles & 255) != 0)
    return fail(PT_ERR_ARG, "pt_extrude_batch_tc: tiles must be 256-byte aligned");
  std::vector<pt_extrude_job> jobs;
  if (int rc = batch_jobs("pt_extrude_batch_tc", W, cap, S, group, bscale, key, top, counts, jobs))
    return rc;
  return extrude_jobs("pt_extrude_batch_tc",
                      ExtrudeForm{terms, nullptr, (const uint8_t*)tiles, nullptr, nullptr,
                                  increments != 0},
                      W,
                      m, sparse, cap, n_groups, buf, (int)jobs.size(), jobs.data(), noise, work,
                      work_bytes, (cudaStream_t)stream);
}

extern "C" int pt_readout(int n, int W, int cap, int interp, int L, const pt_readout_layer* layers,
                          const float* buf, float scale, float* out, void* stream) {
  if (n < 1 || W < 1 || cap < 1 || L < 1) return fail(PT_ERR_ARG, "pt_readout: bad sizes");
  if (L > kMaxReadoutLayers) return fail(PT_ERR_UNSUPPORTED, "pt_readout: at most 64 layers");
  if (n > 8192) return fail(PT_ERR_UNSUPPORTED, "pt_readout: n must be <= 8192");
  if (!layers || !buf || !out) return fail(PT_ERR_ARG, "pt_readout: NULL pointer");
  if (interp < 0 || interp > 2) return fail(PT_ERR_ARG, "pt_readout: interp must be 0, 1 or 2");
  RLayers P{};
  const double one = (double)(1ll << kFix);
  for (int l = 0; l < L; ++l) {
    const pt_readout_layer& q = layers[l];
    if (q.row_max < 0 || q.anchor_phys < 0 || q.anchor_phys >= cap || q.screen < 0)
      return fail(PT_ERR_ARG, "pt_readout: bad layer ring parameters");
    if (q.row_max >= cap) return fail(PT_ERR_ARG, "pt_readout: row_max beyond the ring");
    const double lim = 4.0e6;
    if (!(std::fabs(q.shift_along) < lim) || !(std::fabs(q.shift_perp) + W < lim) ||
        !(std::fabs(q.mag) <= 4.0))
      return fail(PT_ERR_ARG, "pt_readout: shift or magnification out of range");
    P.l[l].screen = q.screen;
    P.l[l].row_max = q.row_max;
    P.l[l].anchor_phys = q.anchor_phys;
    P.l[l].ca = std::llround(q.mag * q.cos_t * 0.5 * one);
    P.l[l].sa = std::llround(q.mag * q.sin_t * 0.5 * one);
    P.l[l].ra = std::llround(q.shift_along * one);
    P.l[l].rp = std::llround((W / 2.0 + q.shift_perp) * one);
  }
  cudaStream_t s = (cudaStream_t)stream;
  dim3 grid((n + 255) / 256, n);
  ProfScope ps("k_readout", s);
  if (interp == 0) k_readout<2><<<grid, 256, 0, s>>>(n, W, cap, L, P, buf, scale, out);
  else if (interp == 1) k_readout<4><<<grid, 256, 0, s>>>(n, W, cap, L, P, buf, scale, out);
  else k_readout<6><<<grid, 256, 0, s>>>(n, W, cap, L, P, buf, scale, out);
  count_launch_e();
  return check_launch("pt_readout");
}

extern "C" int pt_rows_sample(int n, int cap, int interp, int anchor_phys, int row_max,
                              double shift, const float* buf, float* out, void* stream) {
  if (n < 1 || cap < 1 || row_max < 0 || row_max >= cap || anchor_phys < 0 || anchor_phys >= cap)
    return fail(PT_ERR_ARG, "pt_rows_sample: bad sizes");
  if (!buf || !out) return fail(PT_ERR_ARG, "pt_rows_sample: NULL pointer");
  if (interp < 0 || interp > 2) return fail(PT_ERR_ARG, "pt_rows_sample: interp must be 0, 1 or 2");
  if (!(std::fabs(shift) < 1e9)) return fail(PT_ERR_ARG, "pt_rows_sample: shift out of range");
  const double fl = std::floor(shift);
  const int i0 = (int)fl;
  const float t = (float)(shift - fl);
  cudaStream_t s = (cudaStream_t)stream;
  dim3 grid((n + 255) / 256, n);
  if (interp == 0) k_rows_sample<2><<<grid, 256, 0, s>>>(n, cap, anchor_phys, row_max, i0, t, buf, out);
  else if (interp == 1) k_rows_sample<4><<<grid, 256, 0, s>>>(n, cap, anchor_phys, row_max, i0, t, buf, out);
  else k_rows_sample<6><<<grid, 256, 0, s>>>(n, cap, anchor_phys, row_max, i0, t, buf, out);
  count_launch_e();
  return check_launch("pt_rows_sample");
}
