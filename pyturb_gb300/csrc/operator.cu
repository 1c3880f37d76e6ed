// The Assemat-Wilson extrusion operator built on the GPU in FP64.
//
// Points: the stencil Z (m full rows of W pixels at y = 0..m-1, flattened
// row-major, then any sparse points (column, y = m - depth)) and the new row
// X (W pixels at y = m). Their joint von Karman covariance
//
//   C = [[C_zz, C_zx], [C_xz, C_xx]]   (N x N, N = Kz + W)
//
// has the lower Cholesky factor [[L, 0], [Y^T, Ls]] with L L^T = C_zz,
// Y = L^-1 C_zx and Ls Ls^T = C_xx - Y^T Y, the conditional covariance of
// the new row. So one factorisation of C gives
//   A = C_xz C_zz^-1 = Y^T L^-1     (one triangular solve, in place),
//   B = Ls                          (B B^T = C_xx - A C_zx, the same
//                                    product the reference forms with an
//                                    eigen square root,
//                                    src/pyturb/extrude.py:250-304),
//   S = L                           (S S^T = C_zz: boiling's seed factor,
//                                    src/pyturb/extrude.py:290-303).
// Every entry of C depends only on the integer offset (|dx|, |dy|) of two
// points, so the covariance is evaluated once per distinct offset into a
// table and the matrix is filled from it.
//
// The von Karman covariance (src/pyturb/infinite.py:88-117) is
//   C(r) = c_pref x^{5/6} K_{5/6}(x),  x = 2 pi r / L0,  C(0) = c_pref 2^{-1/6} Gamma(5/6),
// with K_nu evaluated from its integral representation
//   K_nu(x) = int_0^inf exp(-x cosh t) cosh(nu t) dt
// by the trapezoidal rule. The integrand is analytic in the strip
// |Im t| < pi/2, so the rule converges geometrically: the step
// h = min(1/4, 0.7/sqrt(x)) keeps the discretisation error below ~1e-16
// relative for every x (the second bound keeps the peak near t = 0 resolved
// for large x), and the sum stops once a term falls below 1e-18 of it.
//
// Factorisation: right-looking blocked Cholesky with 64-column panels
// (diagonal block in shared memory, the panel below by row-wise forward
// substitution, the trailing lower triangle by an FP64 tiled GEMM). A pivot
// of the stencil block at or below `tol` is a failure (reported, the column
// is zeroed so no NaN spreads); a pivot of the conditional block at or below
// `tol` zeroes its column (a semidefinite conditional covariance).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <string>
#include <vector>

#include "common.cuh"

namespace pt {
uint64_t* launch_counter();
static inline void count_launch_o(int k = 1) {
  __atomic_add_fetch(launch_counter(), (uint64_t)k, __ATOMIC_RELAXED);
}

constexpr int kNb = 64;  // panel width of the blocked factorisation

// ---------------------------------------------------------------- covariance table
__device__ double vk_core(double x, double nu) {
  // x^nu K_nu(x) for x > 0 (trapezoidal rule on the integral representation)
  if (x > 700.0) return 0.0;
  const double h = fmin(0.25, 0.7 / sqrt(x));
  double sum = 0.5 * exp(-x);
  for (int k = 1; k < 4096; ++k) {
    const double t = k * h;
    const double term = exp(-x * cosh(t)) * cosh(nu * t);
    sum += term;
    if (term < 1e-18 * sum) break;
  }
  return pow(x, nu) * h * sum;
}

// T[s][i] = C(dx * hypot(i, dys[s])) for i in [0, W), s in [0, nslot)
__global__ void k_aw_table(int W, int nslot, const int* __restrict__ dys, double dx, double L0,
                           double pref, double c0, double* __restrict__ T) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = blockIdx.y;
  if (i >= W || s >= nslot) return;
  const double dy = (double)dys[s];
  const double r = dx * sqrt((double)i * (double)i + dy * dy);
  const double x = 2.0 * 3.14159265358979323846 * r / L0;
  T[(size_t)s * W + i] = (x > 0.0) ? pref * vk_core(x, 5.0 / 6.0) : c0;
}

// C[p][q] = T[slot(|y_p - y_q|)][|x_p - x_q|], plus `jitter` on the stencil diagonal
__global__ void k_aw_fill(int N, int Kz, const int* __restrict__ px, const int* __restrict__ py,
                          const int* __restrict__ slot_of, int W, const double* __restrict__ T,
                          double jitter, double* __restrict__ C) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int p = blockIdx.y;
  if (q >= N || p >= N) return;
  const int ddx = abs(px[p] - px[q]);
  const int ddy = abs(py[p] - py[q]);
  double v = T[(size_t)slot_of[ddy] * W + ddx];
  if (p == q && p < Kz) v += jitter;
  C[(size_t)p * N + q] = v;
}

// ---------------------------------------------------------------- blocked Cholesky
// Factor the kb x kb diagonal block at (k, k) in shared memory.
__global__ void __launch_bounds__(256)
k_potrf_diag(double* __restrict__ a, int lda, int k, int kb, int strict_end, double tol,
             int* __restrict__ info) {
  __shared__ double s[kNb][kNb + 1];
  __shared__ double piv;
  const int tid = threadIdx.x;
  for (int idx = tid; idx < kNb * kNb; idx += blockDim.x) {
    const int i = idx / kNb, j = idx % kNb;
    s[i][j] = (i < kb && j <= i) ? a[(size_t)(k + i) * lda + k + j] : 0.0;
  }
  __syncthreads();
  for (int j = 0; j < kb; ++j) {
    if (tid == 0) {
      const double d = s[j][j];
      if (d > tol) {
        piv = sqrt(d);
      } else {
        piv = 0.0;
        if (k + j < strict_end) atomicCAS(info, 0, k + j + 1);
      }
      s[j][j] = piv;
    }
    __syncthreads();
    const double p = piv;
    for (int i = j + 1 + tid; i < kb; i += blockDim.x) s[i][j] = (p > 0.0) ? s[i][j] / p : 0.0;
    __syncthreads();
    const int rem = kb - j - 1;
    for (int idx = tid; idx < rem * rem; idx += blockDim.x) {
      const int ii = j + 1 + idx / rem, ll = j + 1 + idx % rem;
      if (ll <= ii) s[ii][ll] -= s[ii][j] * s[ll][j];
    }
    __syncthreads();
  }
  for (int idx = tid; idx < kb * kb; idx += blockDim.x) {
    const int i = idx / kb, j = idx % kb;
    a[(size_t)(k + i) * lda + k + j] = (j <= i) ? s[i][j] : 0.0;
  }
}

// Rows [r0, r1) of block column [k, k + kb): x L11^T = a_row (forward
// substitution; a zeroed pivot gives x_j = 0). One thread per row.
__global__ void __launch_bounds__(128)
k_trsm_panel(double* __restrict__ a, int lda, int k, int kb, int r0, int r1) {
  __shared__ double L[kNb][kNb + 1];
  for (int idx = threadIdx.x; idx < kNb * kNb; idx += blockDim.x) {
    const int i = idx / kNb, j = idx % kNb;
    L[i][j] = (i < kb && j < kb) ? a[(size_t)(k + i) * lda + k + j] : (i == j ? 1.0 : 0.0);
  }
  __syncthreads();
  const int r = r0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= r1) return;
  double* row = a + (size_t)r * lda + k;
  double x[kNb];
#pragma unroll
  for (int j = 0; j < kNb; ++j) {
    double v = (j < kb) ? row[j] : 0.0;
#pragma unroll
    for (int l = 0; l < j; ++l) v -= x[l] * L[j][l];
    const double d = L[j][j];
    x[j] = (d != 0.0) ? v / d : 0.0;
  }
#pragma unroll
  for (int j = 0; j < kNb; ++j)
    if (j < kb) row[j] = x[j];
}

// Rows [0, rows) of y (ld ldy), block column [k, k + kb): x L_JJ = y_row
// (backward substitution with the lower block L_JJ at (k, k) of l).
__global__ void __launch_bounds__(128)
k_trsm_back(double* __restrict__ y, int ldy, int rows, const double* __restrict__ l, int ldl, int k,
            int kb) {
  __shared__ double L[kNb][kNb + 1];
  for (int idx = threadIdx.x; idx < kNb * kNb; idx += blockDim.x) {
    const int i = idx / kNb, j = idx % kNb;
    L[i][j] = (i < kb && j < kb) ? l[(size_t)(k + i) * ldl + k + j] : (i == j ? 1.0 : 0.0);
  }
  __syncthreads();
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  double* row = y + (size_t)r * ldy + k;
  double x[kNb];
#pragma unroll
  for (int j = kNb - 1; j >= 0; --j) {
    double v = (j < kb) ? row[j] : 0.0;
#pragma unroll
    for (int q = j + 1; q < kNb; ++q) v -= x[q] * L[q][j];
    const double d = L[j][j];
    x[j] = (d != 0.0) ? v / d : 0.0;
  }
#pragma unroll
  for (int j = 0; j < kNb; ++j)
    if (j < kb) row[j] = x[j];
}

// C (M x N, ldc) = beta C + alpha A B^T (BT: B is N x K, ldb) or alpha A B
// (B is K x N, ldb); A is M x K (lda). 64 x 64 tiles, K steps of 16, each of
// 256 threads accumulating 4 x 4 outputs. With lower_only, tiles strictly
// above the diagonal are skipped (and elements above it are left alone).
template <bool BT>
__global__ void __launch_bounds__(256)
k_dgemm(int M, int N, int K, double alpha, const double* __restrict__ A, int lda,
        const double* __restrict__ B, int ldb, double beta, double* __restrict__ C, int ldc,
        int lower_only) {
  constexpr int T = 64, BK = 16;
  const int m0 = blockIdx.y * T, n0 = blockIdx.x * T;
  if (lower_only && n0 > m0 + T - 1) return;
  __shared__ double As[BK][T + 1];
  __shared__ double Bs[BK][T + 1];
  const int tid = threadIdx.x;
  const int tm = tid / 16, tn = tid % 16;
  double acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += BK) {
    for (int idx = tid; idx < T * BK; idx += 256) {
      const int r = idx / BK, kk = idx % BK;
      const int gm = m0 + r, gk = k0 + kk;
      As[kk][r] = (gm < M && gk < K) ? A[(size_t)gm * lda + gk] : 0.0;
    }
    if (BT) {
      for (int idx = tid; idx < T * BK; idx += 256) {
        const int r = idx / BK, kk = idx % BK;
        const int gn = n0 + r, gk = k0 + kk;
        Bs[kk][r] = (gn < N && gk < K) ? B[(size_t)gn * ldb + gk] : 0.0;
      }
    } else {
      for (int idx = tid; idx < T * BK; idx += 256) {
        const int kk = idx / T, c = idx % T;
        const int gn = n0 + c, gk = k0 + kk;
        Bs[kk][c] = (gn < N && gk < K) ? B[(size_t)gk * ldb + gn] : 0.0;
      }
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      double av[4], bv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) av[u] = As[kk][tm + 16 * u];
#pragma unroll
      for (int v = 0; v < 4; ++v) bv[v] = Bs[kk][tn + 16 * v];
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = fma(av[u], bv[v], acc[u][v]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int gm = m0 + tm + 16 * u, gn = n0 + tn + 16 * v;
      if (gm < M && gn < N && (!lower_only || gn <= gm)) {
        double* c = C + (size_t)gm * ldc + gn;
        *c = (beta == 0.0 ? 0.0 : beta * *c) + alpha * acc[u][v];
      }
    }
}

__global__ void k_zero_upper(double* __restrict__ a, int n) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y;
  if (i < n && j < n && j > i) a[(size_t)i * n + j] = 0.0;
}

// The increment form of A (in place, rows [Kz, N) x columns [0, Kz) of the
// joint matrix): with d_i = row_i - row_{i+1} (i < m - 1, rows oldest first)
// and r1 the newest stencil row, A z = S r1 + sum_i (sum_{j <= i} A_j) d_i
// + sum_p a_p (s_p - r1[c_p]) + sum_p a_p r1[c_p], S = sum_j A_j. The block
// of r1 holds S - I plus each sparse weight at its column: the caller adds
// r1 itself exactly, and the product only forms the small correction.
__global__ void k_aw_increments(int W, int m, int Kz, int N, int ns,
                                const int* __restrict__ sparse_col, double* __restrict__ J) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int r = blockIdx.y;
  if (c >= W || r >= W) return;
  double* a = J + (size_t)(Kz + r) * N;
  double acc = 0.0;
  for (int j = 0; j < m; ++j) {
    acc += a[(size_t)j * W + c];
    if (j < m - 1) a[(size_t)j * W + c] = acc;
  }
  double v = acc - (c == r ? 1.0 : 0.0);
  for (int q = 0; q < ns; ++q)
    if (sparse_col[q] == c) v += a[(size_t)m * W + q];
  a[(size_t)(m - 1) * W + c] = v;
}

// M (W, Kz + W) float32 = [A | B] from the factored joint matrix (ld N):
// A = rows [Kz, N), columns [0, Kz); B = rows [Kz, N), columns [Kz, N).
// Mlo (W, Kz) float32 = A - float(A): what the float32 stencil operator
// leaves out (its relative size is ~2^-24).
__global__ void k_pack_operator(int W, int Kz, int N, const double* __restrict__ J,
                                float* __restrict__ M, double* __restrict__ M64,
                                float* __restrict__ Mlo) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int r = blockIdx.y;
  if (c >= N || r >= W) return;
  const double v = J[(size_t)(Kz + r) * N + c];
  if (M) M[(size_t)r * N + c] = (float)v;
  if (M64) M64[(size_t)r * N + c] = v;
  if (Mlo && c < Kz) Mlo[(size_t)r * Kz + c] = (float)(v - (double)(float)v);
}

// S (Kz, Kz) float32 = the stencil factor L
__global__ void k_pack_seed(int Kz, int N, const double* __restrict__ J, float* __restrict__ S) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int r = blockIdx.y;
  if (c >= Kz || r >= Kz) return;
  S[(size_t)r * Kz + c] = (float)J[(size_t)r * N + c];
}

static inline size_t al256o(size_t x) { return (x + 255) & ~size_t(255); }

static int dgemm(bool bt, int M, int N, int K, double alpha, const double* A, int lda,
                 const double* B, int ldb, double beta, double* C, int ldc, bool lower,
                 cudaStream_t s) {
  if (M <= 0 || N <= 0) return PT_OK;
  const dim3 grid((N + 63) / 64, (M + 63) / 64);
  if (grid.y > 65535) return fail(PT_ERR_UNSUPPORTED, "pt_aw_build: matrix too large");
  if (bt)
    k_dgemm<true><<<grid, 256, 0, s>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, lower);
  else
    k_dgemm<false><<<grid, 256, 0, s>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, lower);
  count_launch_o();
  return PT_OK;
}

// Lower Cholesky of the n x n matrix a (ld n) in place.
static int potrf(double* a, int n, int strict_end, double tol, int* info, cudaStream_t s) {
  for (int k = 0; k < n; k += kNb) {
    const int kb = std::min(kNb, n - k);
    k_potrf_diag<<<1, 256, 0, s>>>(a, n, k, kb, strict_end, tol, info);
    const int r0 = k + kb, rows = n - r0;
    if (rows > 0) {
      k_trsm_panel<<<(rows + 127) / 128, 128, 0, s>>>(a, n, k, kb, r0, n);
      // trailing lower triangle: a[r0:, r0:] -= P P^T, P = a[r0:, k:k+kb]
      const double* P = a + (size_t)r0 * n + k;
      if (int rc = dgemm(true, rows, rows, kb, -1.0, P, n, P, n, 1.0, a + (size_t)r0 * n + r0, n,
                         true, s))
        return rc;
      count_launch_o(2);
    } else {
      count_launch_o(1);
    }
    if (int rc = check_launch("pt_aw_build: factorisation")) return rc;
  }
  return PT_OK;
}

}  // namespace pt

using namespace pt;

static int stencil_points(int W, int m, const pt_sparse_stencil* sp, std::vector<int>& px,
                          std::vector<int>& py, const char* who) {
  px.clear();
  py.clear();
  for (int y = 0; y < m; ++y)
    for (int x = 0; x < W; ++x) {
      px.push_back(x);
      py.push_back(y);
    }
  if (sp) {
    if (sp->count < 0 || sp->count > PT_MAX_SPARSE)
      return fail(PT_ERR_ARG, std::string(who) + ": sparse count must be in [0, 64]");
    for (int i = 0; i < sp->count; ++i) {
      if (sp->depth[i] <= m || sp->column[i] < 0 || sp->column[i] >= W)
        return fail(PT_ERR_ARG, std::string(who) +
                                    ": sparse points need depth > stencil rows and 0 <= column < W");
      px.push_back(sp->column[i]);
      py.push_back(m - sp->depth[i]);
    }
  }
  for (int x = 0; x < W; ++x) {  // the new row
    px.push_back(x);
    py.push_back(m);
  }
  return PT_OK;
}

// Distinct |dy| offsets of all point pairs: the covariance table's rows.
static void offset_slots(const std::vector<int>& py, std::vector<int>& dys,
                         std::vector<int>& slot_of) {
  int ymin = 0, ymax = 0;
  for (int y : py) {
    ymin = std::min(ymin, y);
    ymax = std::max(ymax, y);
  }
  const int dspan = ymax - ymin;
  std::vector<int> ys(py.begin(), py.end());
  std::sort(ys.begin(), ys.end());
  ys.erase(std::unique(ys.begin(), ys.end()), ys.end());
  std::vector<char> used(dspan + 1, 0);
  for (size_t a = 0; a < ys.size(); ++a)
    for (size_t b = a; b < ys.size(); ++b) used[ys[b] - ys[a]] = 1;
  dys.clear();
  slot_of.assign(dspan + 1, 0);
  for (int d = 0; d <= dspan; ++d)
    if (used[d]) {
      slot_of[d] = (int)dys.size();
      dys.push_back(d);
    }
}

struct AwLayout {
  int Kz, N, nslot, dspan;
  size_t off_pts, off_dys, off_slot, off_table, off_info, total;
};

static int aw_layout(int W, int m, const pt_sparse_stencil* sp, std::vector<int>& px,
                     std::vector<int>& py, std::vector<int>& dys, std::vector<int>& slot_of,
                     AwLayout& L, const char* who) {
  if (W < 1 || m < 1) return fail(PT_ERR_ARG, std::string(who) + ": bad sizes");
  if (int rc = stencil_points(W, m, sp, px, py, who)) return rc;
  offset_slots(py, dys, slot_of);
  L.Kz = m * W + (sp ? sp->count : 0);
  L.N = L.Kz + W;
  L.nslot = (int)dys.size();
  L.dspan = (int)slot_of.size() - 1;
  size_t o = al256o((size_t)L.N * L.N * sizeof(double));
  L.off_pts = o;
  o += al256o(2 * (size_t)L.N * sizeof(int));
  L.off_dys = o;
  o += al256o((size_t)L.nslot * sizeof(int));
  L.off_slot = o;
  o += al256o((size_t)(L.dspan + 1) * sizeof(int));
  L.off_table = o;
  o += al256o((size_t)L.nslot * W * sizeof(double));
  L.off_info = o;
  o += 256;
  L.total = o;
  return PT_OK;
}

extern "C" size_t pt_aw_workspace_bytes(int W, int m, const pt_sparse_stencil* sparse) {
  std::vector<int> px, py, dys, slot_of;
  AwLayout L{};
  if (aw_layout(W, m, sparse, px, py, dys, slot_of, L, "pt_aw_workspace_bytes")) return 0;
  return L.total;
}

extern "C" int pt_aw_build(int W, int m, const pt_sparse_stencil* sparse, double pixel_scale,
                           double L0, double jitter, int increments, float* M, double* M64,
                           float* Mlo, float* seed, double* sigma, void* work,
                           size_t work_bytes, void* stream) {
  const char* who = "pt_aw_build";
  if (!(pixel_scale > 0.0) || !(L0 > 0.0) || !std::isfinite(L0))
    return fail(PT_ERR_ARG, std::string(who) + ": pixel_scale and a finite L0 must be positive");
  if (!(jitter >= 0.0)) return fail(PT_ERR_ARG, std::string(who) + ": jitter must be >= 0");
  if ((!M && !M64) || !work) return fail(PT_ERR_ARG, std::string(who) + ": NULL pointer");
  std::vector<int> px, py, dys, slot_of;
  AwLayout lay{};
  if (int rc = aw_layout(W, m, sparse, px, py, dys, slot_of, lay, who)) return rc;
  const int Kz = lay.Kz, N = lay.N, nslot = lay.nslot, dspan = lay.dspan;
  if (work_bytes < lay.total) return fail(PT_ERR_ARG, std::string(who) + ": workspace too small");
  if (N > 46340) return fail(PT_ERR_UNSUPPORTED, std::string(who) + ": joint covariance too large");
  char* w = (char*)work;
  double* J = (double*)w;
  int* dpx = (int*)(w + lay.off_pts);
  int* dpy = dpx + N;
  int* ddys = (int*)(w + lay.off_dys);
  int* dslot = (int*)(w + lay.off_slot);
  double* T = (double*)(w + lay.off_table);
  int* info = (int*)(w + lay.off_info);
  cudaStream_t s = (cudaStream_t)stream;
  // von Karman prefactor at unit r0 and the r = 0 value
  const double pi = 3.14159265358979323846;
  const double pref = std::pow(L0, 5.0 / 3.0) * std::pow(2.0, -5.0 / 6.0) * std::tgamma(11.0 / 6.0) /
                      std::pow(pi, 8.0 / 3.0) *
                      std::pow(24.0 / 5.0 * std::tgamma(6.0 / 5.0), 5.0 / 6.0);
  const double c0 = pref * std::pow(2.0, -1.0 / 6.0) * std::tgamma(5.0 / 6.0);
  if (int rc = check_cuda(cudaMemcpyAsync(dpx, px.data(), N * sizeof(int), cudaMemcpyHostToDevice, s),
                          "pt_aw_build: upload"))
    return rc;
  if (int rc = check_cuda(cudaMemcpyAsync(dpy, py.data(), N * sizeof(int), cudaMemcpyHostToDevice, s),
                          "pt_aw_build: upload"))
    return rc;
  if (int rc = check_cuda(cudaMemcpyAsync(ddys, dys.data(), nslot * sizeof(int),
                                          cudaMemcpyHostToDevice, s),
                          "pt_aw_build: upload"))
    return rc;
  if (int rc = check_cuda(cudaMemcpyAsync(dslot, slot_of.data(), (dspan + 1) * sizeof(int),
                                          cudaMemcpyHostToDevice, s),
                          "pt_aw_build: upload"))
    return rc;
  if (int rc = check_cuda(cudaMemsetAsync(info, 0, sizeof(int), s), "pt_aw_build: memset"))
    return rc;
  k_aw_table<<<dim3((W + 127) / 128, nslot), 128, 0, s>>>(W, nslot, ddys, pixel_scale, L0, pref, c0, T);
  k_aw_fill<<<dim3((N + 255) / 256, N), 256, 0, s>>>(N, Kz, dpx, dpy, dslot, W, T, jitter * c0,
                                                     J);
  count_launch_o(2);
  if (int rc = check_launch("pt_aw_build: covariance")) return rc;
  if (int rc = potrf(J, N, Kz, 1e-13 * c0, info, s)) return rc;
  k_zero_upper<<<dim3((N + 255) / 256, N), 256, 0, s>>>(J, N);
  count_launch_o();
  // A = Y^T L^-1: block columns of the (W x Kz) lower-left block, last first
  double* Yt = J + (size_t)Kz * N;
  const int nblk = (Kz + kNb - 1) / kNb;
  for (int b = nblk - 1; b >= 0; --b) {
    const int k = b * kNb, kb = std::min(kNb, Kz - k);
    k_trsm_back<<<(W + 127) / 128, 128, 0, s>>>(Yt, N, W, J, N, k, kb);
    count_launch_o();
    if (k > 0)  // Yt[:, 0:k] -= A_J L[J, 0:k]
      if (int rc = dgemm(false, W, k, kb, -1.0, Yt + k, N, J + (size_t)k * N, N, 1.0, Yt, N, false,
                         s))
        return rc;
    if (int rc = check_launch("pt_aw_build: solve")) return rc;
  }
  if (sigma)  // the conditional covariance Ls Ls^T (W x W, FP64)
    if (int rc = dgemm(true, W, W, W, 1.0, Yt + Kz, N, Yt + Kz, N, 0.0, sigma, W, false, s))
      return rc;
  if (increments) {
    // the sparse columns sit in the point list: x of sparse point q is px[m W + q]
    k_aw_increments<<<dim3((W + 255) / 256, W), 256, 0, s>>>(W, m, Kz, N, Kz - m * W,
                                                             dpx + (size_t)m * W, J);
    count_launch_o();
  }
  k_pack_operator<<<dim3((N + 255) / 256, W), 256, 0, s>>>(W, Kz, N, J, M, M64, Mlo);
  count_launch_o();
  if (seed) {
    k_pack_seed<<<dim3((Kz + 255) / 256, Kz), 256, 0, s>>>(Kz, N, J, seed);
    count_launch_o();
  }
  if (int rc = check_launch("pt_aw_build: pack")) return rc;
  int h_info = 0;
  if (int rc = check_cuda(cudaMemcpyAsync(&h_info, info, sizeof(int), cudaMemcpyDeviceToHost, s),
                          "pt_aw_build: status"))
    return rc;
  if (int rc = check_cuda(cudaStreamSynchronize(s), "pt_aw_build: synchronize")) return rc;
  if (h_info != 0)
    return fail(PT_ERR_NUMERIC, std::string(who) +
                                    ": stencil covariance not positive definite at pivot " +
                                    std::to_string(h_info - 1));
  return PT_OK;
}
