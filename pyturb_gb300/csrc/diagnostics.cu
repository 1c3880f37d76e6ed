// Validation diagnostics on the device: the phase structure function of a
// stack of screens (pyturb.utils.structure_function, src/pyturb/utils.py:
// 159-201). Sums are deterministic: Kahan-compensated float per thread,
// float64 per block, then a fixed-order sum over blocks.

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "common.cuh"

namespace pt {
uint64_t* launch_counter();
static inline void count_launch_d(int k = 1) {
  __atomic_add_fetch(launch_counter(), (uint64_t)k, __ATOMIC_RELAXED);
}

constexpr int kSfRows = 32;  // image rows per block

struct Kahan {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    const float y = x - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
};

// partial[((sep - 1) * nb + b) * 2 + {0, 1}]: sums over block b's rows of the
// squared differences at separation sep along axis -2 (rows) and axis -1.
__global__ void __launch_bounds__(256)
k_structure(int count, int ny, int nx, const float* __restrict__ phase, double* __restrict__ partial) {
  __shared__ double red[8][2];
  const int sep = blockIdx.y + 1, b = blockIdx.x, nb = gridDim.x;
  const long long r0 = (long long)b * kSfRows;
  const long long r1 = min((long long)count * ny, r0 + kSfRows);
  Kahan kr, kc;
  for (long long r = r0; r < r1; ++r) {
    const int i = (int)(r % ny);
    const float* row = phase + r * nx;
    const bool down = i + sep < ny;
    for (int j = threadIdx.x; j < nx; j += blockDim.x) {
      const float v = row[j];
      if (down) {
        const float d = row[(size_t)sep * nx + j] - v;
        kr.add(d * d);
      }
      if (j + sep < nx) {
        const float d = row[j + sep] - v;
        kc.add(d * d);
      }
    }
  }
  double a = (double)kr.s - (double)kr.c, c = (double)kc.s - (double)kc.c;
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    red[warp][0] = a;
    red[warp][1] = c;
  }
  __syncthreads();
  if (threadIdx.x < 2) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w][threadIdx.x];
    partial[((size_t)(sep - 1) * nb + b) * 2 + threadIdx.x] = s;
  }
}

// D[sep - 1] = (rows / (count (ny - sep) nx) + cols / (count ny (nx - sep))) / 2
__global__ void k_structure_reduce(int count, int ny, int nx, int max_sep, int nb,
                                   const double* __restrict__ partial, double* __restrict__ D) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= max_sep) return;
  const int sep = s + 1;
  double a = 0.0, c = 0.0;
  for (int b = 0; b < nb; ++b) {
    a += partial[((size_t)s * nb + b) * 2];
    c += partial[((size_t)s * nb + b) * 2 + 1];
  }
  const double na = (double)count * (ny - sep) * nx, nc = (double)count * ny * (nx - sep);
  D[s] = 0.5 * ((na > 0 ? a / na : 0.0) + (nc > 0 ? c / nc : 0.0));
}

}  // namespace pt

using namespace pt;

extern "C" size_t pt_structure_workspace_bytes(int count, int ny, int nx, int max_sep) {
  if (count < 1 || ny < 2 || nx < 2 || max_sep < 1) return 0;
  const long long nb = ((long long)count * ny + kSfRows - 1) / kSfRows;
  return (size_t)nb * max_sep * 2 * sizeof(double);
}

extern "C" int pt_structure_function(int count, int ny, int nx, const float* phase, int max_sep,
                                     double* D, void* work, size_t work_bytes, void* stream) {
  if (count < 1 || ny < 2 || nx < 2) return fail(PT_ERR_ARG, "pt_structure_function: bad sizes");
  if (max_sep < 1 || max_sep >= std::min(ny, nx))
    return fail(PT_ERR_ARG, "pt_structure_function: max_separation must be in [1, n)");
  if (!phase || !D) return fail(PT_ERR_ARG, "pt_structure_function: NULL pointer");
  const size_t need = pt_structure_workspace_bytes(count, ny, nx, max_sep);
  if (!work || work_bytes < need) return fail(PT_ERR_ARG, "pt_structure_function: workspace too small");
  const long long nb = ((long long)count * ny + kSfRows - 1) / kSfRows;
  if (nb > 0x7fffffff || max_sep > 65535)
    return fail(PT_ERR_UNSUPPORTED, "pt_structure_function: stack too large");
  cudaStream_t s = (cudaStream_t)stream;
  double* partial = (double*)work;
  {
    ProfScope ps("k_structure", s);
    k_structure<<<dim3((unsigned)nb, max_sep), 256, 0, s>>>(count, ny, nx, phase, partial);
  }
  k_structure_reduce<<<(max_sep + 127) / 128, 128, 0, s>>>(count, ny, nx, max_sep, (int)nb,
                                                          partial, D);
  count_launch_d(2);
  return check_launch("pt_structure_function");
}
