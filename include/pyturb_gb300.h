/*
 * pyturb_gb300 — C-ABI of the GB300 (sm_103a) phase-screen hot path.
 *
 * Plain C types only: device buffers are raw pointers (float data, complex
 * values as interleaved (re, im) float pairs), streams are `void*`
 * (a cudaStream_t, NULL = the legacy default stream). Every entry point
 * returns a status code (PT_OK on success) and leaves a message readable
 * through pt_last_error() on failure. Hot-path calls never allocate: their
 * scratch lives in a caller-provided workspace whose size the matching
 * *_workspace_bytes() query returns. Arguments are validated before any
 * launch, so a bad call returns PT_ERR_ARG and touches no memory.
 *
 * Each entry point names the reference (jacotay7/pyturb) interface it
 * replaces as `path:line`.
 */
#ifndef PYTURB_GB300_H
#define PYTURB_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  PT_OK = 0,
  PT_ERR_ARG = 1,         /* invalid argument (sizes, NULL pointers, workspace too small) */
  PT_ERR_CUDA = 2,        /* a CUDA runtime call or kernel launch failed */
  PT_ERR_UNSUPPORTED = 3, /* valid request outside what this build implements */
  PT_ERR_NUMERIC = 4      /* a factorisation met a non-positive pivot (see the message) */
};

/* Library version (major*10000 + minor*100 + patch). */
int pt_version(void);

/* Message of the last failed call on this host thread ("" if none). */
const char* pt_last_error(void);

/* Number of kernels this library has launched since load (all threads). */
uint64_t pt_launch_count(void);

/* Per-kernel timing with CUDA events recorded on each launch's stream
 * (no reference counterpart: measurement support). pt_prof_enable(1)
 * starts recording, pt_prof_report() synchronises the device, writes one
 * line "kernel launches total_ms" per kernel into buf and clears the log. */
int pt_prof_enable(int on);
int pt_prof_report(char* buf, size_t len);

/* Failure detection (no reference counterpart). Kernels that wait on an
 * mbarrier (the TMA-fed column pass, the tensor-core extrusion products and
 * the tensor-core DFT) bound every wait; a wait that runs out sets bit 1 of a
 * device error word and the kernel finishes instead of hanging.
 * pt_device_error synchronises the device and reads (and, with clear != 0,
 * resets) those words, combined. pt_selftest_wait_timeout runs one wait that
 * nothing completes, with `limit` polls (1..2^24), and reports in *timed_out
 * whether it ran out as designed. */
int pt_device_error(int* out, int clear);
int pt_selftest_wait_timeout(long long limit, int* timed_out);

/* ------------------------------------------------------------------ grid plan
 * An ns x ns FFT grid with pixel_scale dx and n_levels subharmonic levels:
 * twiddles, the subharmonic sinusoid bases and their grid means. Mirrors the
 * geometry part of PhaseScreen._build_filters (src/pyturb/fourier.py:174-228).
 * sh_freq: (n_levels, 3) host FP64 subharmonic frequencies f_p = {-1,0,1} df/3^p.
 * Allocates its constant tables on the current device; not a hot-path call.
 * A length with a prime factor above 61 whose padded length (the power of two
 * >= 2 ns - 1) is at most 8192 gets a Bluestein form of its transforms.
 */
typedef struct pt_grid pt_grid;

int pt_grid_create(pt_grid** out, int ns, double pixel_scale, int n_levels,
                   const double* sh_freq);
int pt_grid_destroy(pt_grid* grid);

/* Tuning knobs of a grid (no reference counterpart; read and set by the
 * package's autotuner). pt_grid_radices reports the stage radices of the
 * mixed-radix transform (used for sizes other than powers of two up to
 * 4096); pt_grid_set_radices replaces them with any factorisation of ns into
 * n_stages radices >= 2 (n_stages <= 23; radices other than 2, 3, 4, 5, 7, 8
 * run as direct-sum stages). pt_grid_set_cols_variant picks the column pass
 * of power-of-two grids: 0 register-fed (default), 1 TMA-fed. Results do not
 * depend on either choice beyond float32 rounding. */
int pt_grid_radices(const pt_grid* grid, int* n_stages, int* radices);
int pt_grid_set_radices(pt_grid* grid, int n_stages, const int* radices);
int pt_grid_set_cols_variant(pt_grid* grid, int variant);

/* Workspace needed by pt_generate / pt_frames / pt_ifft2 on this grid
 * (largest over the three, for the chunk sizes the library uses). */
size_t pt_grid_workspace_bytes(const pt_grid* grid, int n_layers);

/* Unnormalised inverse 2-D DFT, numpy.fft.ifft2(x) * ns^2, of `batch`
 * complex ns x ns images (in and out may alias). The transform under
 * PhaseScreen.generate (src/pyturb/fourier.py:259) and
 * Atmosphere._integrate (src/pyturb/atmosphere.py:918). */
int pt_ifft2(const pt_grid* grid, const float* in, float* out, int batch, void* work,
             size_t work_bytes, void* stream);

/* Tensor-core form of pt_ifft2 for ns = 512 (the split-precision DFT form;
 * no reference counterpart beyond the transform it replaces,
 * src/pyturb/fourier.py:259 and src/pyturb/atmosphere.py:918): each 512-point
 * line is a four-step DFT (32 x 16) of two small matrix products on tcgen05,
 * operands of each power-of-two scaled line split into two fp16 terms with
 * fp32 accumulation, a row pass then a column pass. in and out may alias. Other sizes: PT_ERR_UNSUPPORTED. */
int pt_ifft2_tc(int ns, const float* in, float* out, int batch, void* stream);

/* Allocation-free variant of pt_ifft2 — no counterpart in the reference.
 * For callers that cannot call cudaMalloc (a host framework that owns all
 * device memory, or a process that must not grow its footprint after
 * start-up): no grid plan and no workspace. Its scratch is a fixed 8 MiB
 * file-scope device array (plus a 1024-entry twiddle table) that every GPU
 * loading this library holds until exit. ns must be in [2, 1024]; larger
 * grids are rejected with PT_ERR_ARG. Every uncaptured call resolves the
 * arrays' addresses (cudaGetSymbolAddress) on the current device; a call made
 * while its stream is captured reuses the address of the last uncaptured call
 * on that device, so make one call on each device before any stream capture.
 * All calls share the arrays, so calls that overlap on the GPU (different
 * streams or threads) race: serialise them, e.g. on one stream. Nothing in
 * the arrays has to start at zero. */
int pt_ifft2_noalloc(int ns, const float* in, float* out, int batch, void* stream);

/* PhaseScreen.generate(count) (src/pyturb/fourier.py:233-282): coloured
 * complex noise x amplitude -> inverse FFT -> real parts are screens
 * [0, n_fft), imaginary parts screens [n_fft, 2 n_fft) (n_fft = ceil(count/2))
 * -> plus the 3x3-per-level subharmonic sum minus its screen mean.
 *   amplitude (ns, ns)      device f32, sqrt(PSD) * df with DC zeroed
 *   sh_amp    (P, 3, 3)     device f32 (NULL when P = 0)
 *   noise     (2, n_fft, ns, ns) device f32 normals, or NULL: in-kernel
 *                           Philox4x32-10 keyed by (seed, call)
 *   sh_noise  (P, 2, count, 3, 3) device f32, or NULL (Philox)
 * Output (count, n_out, n_out): the crop window [crop, crop + n_out) of each
 * screen times `scale`, added to `out` when accumulate != 0 (the L0-group sum
 * of Atmosphere.sample, src/pyturb/atmosphere.py:1213-1219). */
int pt_generate(const pt_grid* grid, int count, const float* amplitude, const float* sh_amp,
                const float* noise, const float* sh_noise, uint64_t seed, uint64_t call,
                int crop, int n_out, float scale, int accumulate, float* out, void* work,
                size_t work_bytes, void* stream);

/* pt_generate with one extra factor per screen (Philox noise, no
 * accumulation): screen i is scaled by scale * screen_scale[i] (device f32,
 * count entries). The von Karman amplitude is proportional to r0^(-5/6), so
 * one unit-r0 grid serves every screen of a (size, L0) group of a ragged
 * Monte-Carlo ensemble with screen_scale = r0_i^(-5/6): the ensemble of
 * independent PhaseScreen(n_i, dx, r0_i, L0_i).generate() calls
 * (src/pyturb/fourier.py:233-282) in one call per group. */
int pt_generate_scaled(const pt_grid* grid, int count, const float* amplitude,
                       const float* sh_amp, uint64_t seed, uint64_t call, int crop, int n_out,
                       float scale, const float* screen_scale, float* out, void* work,
                       size_t work_bytes, void* stream);

/* FourierFlowScreen.reseed (src/pyturb/flow.py:71-94) for L layers at once:
 *   spectra[l] = (noise[l,0] + i noise[l,1]) * amplitude[l]   (L, ns, ns) complex
 *   sh_coef[p, l] = (sh_noise[l,p,0] + i sh_noise[l,p,1]) * sh_amp[p, l]  (P, L, 3, 3) complex
 * noise / sh_noise NULL draws Philox normals keyed by seeds[l] (host array). */
int pt_layers_fill(const pt_grid* grid, int n_layers, const float* amplitude,
                   const float* sh_amp, const float* noise, const float* sh_noise,
                   const uint64_t* seeds, float* spectra, float* sh_coef, void* stream);

/* Frozen-flow readout of the spectral engine. Frame f is
 *   Re ifft2( sum_l S_l . exp(2 pi i (f_x sx[f,l] + f_y sy[f,l])) ) * ns^2
 *   + Re(sum_p basis^T shifted_p basis) - mean, cropped, times scale,
 * i.e. Atmosphere._integrate (src/pyturb/atmosphere.py:882-938), one frame
 * per (t, direction) pair of Atmosphere._integrate_dirs (940-998) and
 * FourierFlowScreen.translate (src/pyturb/flow.py:96-129) for L = 1.
 *   spectra (L, ns, ns) complex, sh_coef (P, L, 3, 3) complex (device)
 *   sx, sy  (F, L) host FP64 displacements [m] along axes 0 and 1
 * per_layer != 0 gives Atmosphere._integrate_lgs's per-layer screens
 * (src/pyturb/atmosphere.py:1013-1040): F must equal L, sx / sy are (L)
 * and frame l is layer l alone at shift (sx[l], sy[l]), uncropped. */
int pt_frames(const pt_grid* grid, int n_layers, const float* spectra, const float* sh_coef,
              int n_frames, const double* sx, const double* sy, int per_layer, int crop,
              int n_out, float scale, float* out, void* work, size_t work_bytes, void* stream);

/* The shift theorem applied to the stored layer state
 * (FourierFlowScreen.translate, src/pyturb/flow.py:96-129; the phasors of
 * Atmosphere._integrate, src/pyturb/atmosphere.py:904-916): spectra_out[l] =
 * spectra_in[l] * exp(2 pi i (f_x sx[l] + f_y sy[l])) with the same exact
 * fixed-point phases as pt_frames, and likewise the (P, L, 3, 3)
 * subharmonic coefficients (NULL when P = 0). sx, sy: host FP64 (L) [m].
 * Frames rendered from the output at displacement s equal frames of the
 * input at sx + s, which lets a captured frame loop (a CUDA graph of
 * pt_frames calls with fixed relative displacements) be replayed at any
 * start time. n_layers <= 64; in and out may alias. */
int pt_layers_translate(const pt_grid* grid, int n_layers, const float* spectra_in,
                        const float* sh_in, const double* sx, const double* sy,
                        float* spectra_out, float* sh_out, void* stream);

/* Atmosphere._lgs_zoom (src/pyturb/atmosphere.py:1047-1090): separable
 * T-tap cone zoom of L (ns, ns) layer screens into one (n, n) pupil,
 * summed over layers, times scale. idx (L, T, n) int32, w (L, T, n) f32. */
int pt_lgs_zoom(int n_layers, int ns, int n, int n_taps, const int32_t* idx, const float* w,
                const float* screens, float scale, float* out, void* stream);

/* Atmosphere._boil_step (src/pyturb/atmosphere.py:1092-1126): per-mode AR(1)
 *   S <- a S + sqrt(1 - a^2) (n0 + i n1) amplitude,  a = exp(-dt / tau)
 * on the stacked spectra and subharmonic coefficients, in place.
 * main_tau (L, ns, ns) f32, sh_tau (P, L, 3, 3) f32, amplitude (L, ns, ns),
 * sh_amp (P, L, 3, 3). noise (2, L, ns, ns) / sh_noise (2, P, L, 3, 3)
 * device normals, or NULL for Philox keyed by (seed, call). */
int pt_boil_step(const pt_grid* grid, int n_layers, float* spectra, float* sh_coef,
                 const float* amplitude, const float* sh_amp, const float* main_tau,
                 const float* sh_tau, double dt, const float* noise, const float* sh_noise,
                 uint64_t seed, uint64_t call, void* stream);

/* ------------------------------------------------------------------ extrusion
 * Sparse points appended to the m full stencil rows: point i is column
 * column[i] of the row depth[i] rows behind the new row (m < depth < ring
 * capacity). No reference counterpart: the reference stencil is
 * `stencil_rows` full rows only (src/pyturb/extrude.py:272-275,
 * src/pyturb/infinite.py:244-248). NULL (or count 0) = rows only. */
#define PT_MAX_SPARSE 64
typedef struct {
  int32_t count;
  int32_t depth[PT_MAX_SPARSE];
  int32_t column[PT_MAX_SPARSE];
} pt_sparse_stencil;

/* The Assemat-Wilson operator in FP64 on the GPU, at unit r0: the joint
 * von Karman covariance of the stencil (m rows of W pixels, then the sparse
 * points) and the new row, one blocked Cholesky factorisation
 * [[L, 0], [Y^T, Ls]] of it, and A = Y^T L^-1. Replaces phase_covariance,
 * _spd_solve and build_extrusion (src/pyturb/infinite.py:54-117,
 * src/pyturb/extrude.py:250-304) and the seed factor
 * (src/pyturb/extrude.py:290-303). Outputs (device, each may be NULL but
 * not both M and M64):
 *   M (W, K) f32 and M64 (W, K) f64 = [A | Ls], K = (m+1) W + count
 *     (Ls Ls^T is the conditional covariance the reference factors with
 *     eigh; any factor gives the same statistics);
 *   Mlo (W, Kz) f32 = A - (float)A, the correction that keeps a float32
 *     recursion on the float64 operator (pt_extrude_lo_prepare), or NULL;
 *   seed (Kz, Kz) f32 = L (L L^T = C_zz, Kz = m W + count), or NULL;
 *   sigma (W, W) f64 = Ls Ls^T, or NULL.
 * With `increments` the stencil part is returned in increment form, the
 * operand of pt_extrude_* with increments set: the stencil rows become
 * differences d_i = row_i - row_{i+1} (oldest first) and the newest row r1,
 * the sparse values s_p - r1[c_p], and the r1 block holds S - I (S = the sum
 * of the row blocks) plus each sparse weight at its column, so that
 * new row = r1 + M . operand. The product then forms only a small correction
 * to r1, and its float32 rounding is small in proportion.
 * `jitter` adds jitter * C(0) to the stencil diagonal. A non-positive pivot
 * of the stencil block returns PT_ERR_NUMERIC; pivots of the conditional
 * block at or below 1e-13 C(0) zero their column. Synchronises `stream`. */
size_t pt_aw_workspace_bytes(int W, int m, const pt_sparse_stencil* sparse);
int pt_aw_build(int W, int m, const pt_sparse_stencil* sparse, double pixel_scale, double L0,
                double jitter, int increments, float* M, double* M64, float* Mlo, float* seed,
                double* sigma, void* work, size_t work_bytes, void* stream);

/* One Assemat-Wilson row step for a set of ring-buffer screens
 * (_ExtrudeLayer._extrude_one, src/pyturb/extrude.py:424-430;
 * InfinitePhaseScreen._extrude_one, src/pyturb/infinite.py:274-281):
 *   buf[s, head] = A_g . [buf[s, head-m .. head-1] ; sparse values]
 *                  + B_g . (bscale * beta)
 * with ring rows taken modulo cap. M holds [A_g | B_unit_g] row-major,
 * shape (G, W, K), K = (m+1) W + sparse count. Jobs are processed in `step`
 * order; the jobs of one step are independent (distinct screens). */
typedef struct {
  int32_t screen;     /* slab of buf: (screen, cap, W) */
  int32_t group;      /* which [A | B] matrix */
  int32_t head;       /* physical ring row receiving the new row */
  int32_t step;       /* sequential step index (non-decreasing over the job list) */
  float bscale;       /* r0^(-5/6) of the screen */
  int32_t pad;
  uint64_t key;       /* Philox key for beta when noise == NULL */
  uint64_t row;       /* virtual row index (Philox counter) */
  int64_t noise_off;  /* element offset of this row's W normals in `noise` */
} pt_extrude_job;

size_t pt_extrude_workspace_bytes(int W, int m, int n_sparse, int max_jobs_per_step);

/* The same steps for S screens given as arrays (host): screen s extrudes
 * counts[s] rows, its k-th at virtual row top[s] + k (ring row modulo cap,
 * Philox counter = virtual row, key key[s]), scaled by bscale[s], operator
 * group[s]; top[] is advanced in place. Injected noise, when given, holds W
 * normals per row in step-major order (step k of screen s before step k of
 * screen s+1, all step-k rows before step k+1). Replaces the per-row loop of
 * _ExtrudeLayer._ensure (src/pyturb/extrude.py:446-449) for all layers and
 * realisations at once. */
/* Low-order anchor of the float32 form (no reference counterpart). The row
 * recursion amplifies errors in the smooth modes of a row, so float32
 * rounding in the product walks them away from the float64 result over
 * hundreds of rows. With an anchor, each new row's projection on an
 * orthonormal basis U of `modes` (32 or 64) row vectors is recomputed in
 * double-float arithmetic and set: row += U (U^T A z + U^T B (bscale beta)
 * - U^T row). The package's U is the smoothest DCT-II modes
 * (U[i][w] = sqrt((2 - [i=0]) / W) cos(pi i (w + 1/2) / W)). Tables (device):
 * t_hi / t_lo (G, Kt, modes) f32, Kt = K + W (K + 2 W in the increment
 * form), hi + lo = the float64 value: row k holds column k of
 * [U^T A | U^T B_unit | -U (| U for r1)], its modes stored in
 * pairs (i, i + 16): 0, 16, 1, 17, ..., 15, 31 (then 32, 48, ..., 47, 63);
 * u (modes, W) f32 = U. 8-byte aligned. */
typedef struct {
  int32_t modes;
  int32_t pad;
  const float* t_hi;
  const float* t_lo;
  const float* u;
} pt_extrude_anchor;

/* `increments` (no reference counterpart): M is in the increment form of
 * pt_aw_build, the operand holds row differences and the new row is the
 * newest stencil row plus the product. The reference multiplies the rows
 * themselves; the increment form keeps the float32 product a small
 * correction, so its rounding no longer walks the row recursion away from
 * the float64 result over long runs. */
int pt_extrude_batch(int W, int m, const pt_sparse_stencil* sparse, int increments, int cap,
                     int n_groups, const float* M, const void* lo_tiles,
                     const pt_extrude_anchor* anchor, float* buf, int S, const int32_t* group,
                     const float* bscale, const uint64_t* key, int64_t* top,
                     const int32_t* counts, const float* noise, void* work, size_t work_bytes,
                     void* stream);

int pt_extrude_rows(int W, int m, const pt_sparse_stencil* sparse, int increments, int cap,
                    int n_groups, const float* M, const void* lo_tiles,
                    const pt_extrude_anchor* anchor, float* buf, int n_jobs,
                    const pt_extrude_job* jobs, const float* noise, void* work,
                    size_t work_bytes, void* stream);

/* Operator correction of the float32 form (no reference counterpart): the
 * reference's float32 path multiplies by float32(A), whose rounding is a
 * fixed bias that the row recursion accumulates (relative error ~1e-4 after
 * 500 rows at W = 1449). Passing `lo_tiles` to pt_extrude_batch /
 * pt_extrude_rows adds (A - (float)A) . stencil each step as one bf16
 * tensor-core product, which keeps the recursion on the float64 operator.
 * pt_extrude_lo_prepare converts the (G, W, Kz) Mlo of pt_aw_build into
 * those tiles (pt_extrude_lo_bytes bytes, 256-byte aligned). */
size_t pt_extrude_lo_bytes(int W, int m, int n_sparse, int n_groups);
int pt_extrude_lo_prepare(int W, int m, int n_sparse, int n_groups, const float* Mlo,
                          void* tiles, size_t tiles_bytes, void* stream);

/* Fused multi-layer rotated sub-pixel readout of the extrusion engine
 * (ExtrudedAtmosphere._integrate_fused_kernel / _integrate_looped,
 * src/pyturb/extrude.py:864-915, kernels 91-198): per pupil pixel and layer
 *   row = along + shift_along, col = perp + W/2 + shift_perp
 * with along/perp the pupil grid rotated onto the layer's wind axis and
 * scaled by the LGS magnification; rows clamp to [0, row_max], columns to
 * [0, W-1]; 2/4/6-tap separable weights; layers summed, times scale.
 * interp: 0 linear, 1 cubic (Catmull-Rom), 2 Lanczos-3. */
typedef struct {
  int32_t screen;       /* slab of buf */
  int32_t row_max;      /* last readable row, relative to anchor */
  int32_t anchor_phys;  /* physical ring row of relative row 0 */
  int32_t pad;
  double cos_t, sin_t;  /* wind axis */
  double mag;           /* LGS cone magnification (1 = none) */
  double shift_along;   /* travel + off_along - anchor (rows) */
  double shift_perp;    /* off_perp (columns) */
} pt_readout_layer;

int pt_readout(int n, int W, int cap, int interp, int n_layers, const pt_readout_layer* layers,
               const float* buf, float scale, float* out, void* stream);

/* InfinitePhaseScreen._sample (src/pyturb/infinite.py:308-341): row-only
 * interpolation of an (n, n) window of one ring-buffer screen at relative
 * row position shift (rows clamp to [0, row_max], ring rows modulo cap). */
int pt_rows_sample(int n, int cap, int interp, int anchor_phys, int row_max, double shift,
                   const float* buf, float* out, void* stream);

/* Extrusion boiling helpers (ExtrudedAtmosphere.boil_step,
 * src/pyturb/extrude.py:661-753). pt_fill_normals: out (rows, cols) device
 * f32 = row_scale[r] (host, rows <= 64) * Philox N(0, 1) keyed by (key, call):
 * the white noise under the seed rows S . white of the fresh windows.
 * pt_ring_blend: ring rows phys0, phys0 + 1, ... (mod cap) of one (cap, W)
 * screen become a * buf + b * fresh (fresh: (h, W) device f32), the AR(1)
 * blend buf[lo:hi] = a buf + b fresh on the modular ring. */
int pt_fill_normals(uint64_t key, uint64_t call, int rows, int cols, const float* row_scale,
                    float* out, void* stream);
int pt_ring_blend(int W, int cap, float* screen, int phys0, int h, float a, float b,
                  const float* fresh, void* stream);

/* ---- tensor-core form of the extrusion product --------------------------
 * The split-precision form of pt_extrude_batch (same arguments and ring
 * semantics, src/pyturb/extrude.py:424-456): the operator [A | B_unit] and
 * the per-step operand [stencil ; bscale * beta] are split into `terms`
 * bf16 terms (x = x_hi + x_lo (+ x_mid); 2 terms: 3 products, 3 terms: 6)
 * and multiplied by tcgen05 MMAs into an fp32 accumulator in tensor memory.
 * pt_extrude_tc_prepare converts the FP32 (G, W, K) operator M once
 * into `tiles` (pt_extrude_tc_operator_bytes bytes, 256-byte aligned); the
 * workspace of pt_extrude_batch_tc is pt_extrude_tc_workspace_bytes (for the
 * largest number of screens stepped at once), 256-byte aligned. No reference
 * counterpart beyond the product it replaces. */
size_t pt_extrude_tc_operator_bytes(int W, int m, int n_sparse, int n_groups, int terms);
int pt_extrude_tc_prepare(int W, int m, int n_sparse, int n_groups, const float* M, int terms,
                          void* tiles, size_t tiles_bytes, void* stream);
size_t pt_extrude_tc_workspace_bytes(int W, int m, int n_sparse, int max_jobs, int terms);
int pt_extrude_batch_tc(int W, int m, const pt_sparse_stencil* sparse, int increments, int cap,
                        int n_groups, const void* tiles, int terms, float* buf, int n_screens,
                        const int32_t* group, const float* bscale, const uint64_t* key,
                        int64_t* top, const int32_t* counts, const float* noise, void* work,
                        size_t work_bytes, void* stream);

/* ---- differentiable multi-layer readout --------------------------------
 * out[b,t,d,i,j] = sum_l w[l] * bilerp(screens[b,l], u_r, u_c) with
 * u_r = pos0[t,d,l,0] + mag[d,l] * i, u_c = pos0[t,d,l,1] + mag[d,l] * j,
 * periodic on the S x S screen. The geometry is the LGS cone zoom of
 * Atmosphere._build_lgs_zoom / _lgs_zoom (src/pyturb/atmosphere.py:581-616,
 * 1048-1090) with the displacement of _integrate_lgs (atmosphere.py:1012-1022)
 * applied as a bilinear shift. The reference has no adjoint: the gradient
 * entry points have no counterpart there.
 *
 * Layouts: screens (B, L, S, S) f32; w (L,) f32; pos0 (T, D, L, 2) f64
 * (device); mag (D, L) f64 (HOST, in [0.25, 4], mag*(n-1) + 2 < S);
 * out / grad_out (B, T, D, n, n) f32. fix is a device workspace of
 * 3*T*D*L int64 filled by pt_lr_fix: the positions in 32.32 fixed point, so
 * the forward and the adjoints form identical taps. */
int pt_lr_fix(int T, int D, int L, int S, int n, const double* pos0, const double* mag,
              int64_t* fix, void* stream);
int pt_lr_forward(int B, int L, int S, int T, int D, int n, const double* mag,
                  const float* screens, const float* w, const int64_t* fix, float* out,
                  void* stream);
/* Number of floats in the partial-sum buffer of pt_lr_grad_params:
 * (B, T*D, ceil(n/64), L, 3) = per (image, band of 64 rows, layer):
 * [sum g*val, w*sum g*dval/du_r, w*sum g*dval/du_c]. Summing over b, t, d and
 * bands gives dL/dw; summing over b and bands gives dL/dpos0. */
size_t pt_lr_partial_count(int B, int L, int T, int D, int n);
int pt_lr_grad_params(int B, int L, int S, int T, int D, int n, const double* mag,
                      const float* screens, const float* w, const int64_t* fix,
                      const float* grad_out, float* partial, void* stream);
/* dL/dscreens (B, L, S, S): the transpose of the gather, as a deterministic
 * gather over screen tiles (every element written once, no atomics); added
 * to grad_screens when accumulate != 0 (frames taken in chunks). */
int pt_lr_grad_screens(int B, int L, int S, int T, int D, int n, const double* mag,
                       const float* w, const int64_t* fix, const float* grad_out,
                       int accumulate, float* grad_screens, void* stream);

/* ---- validation diagnostics ---------------------------------------------
 * pyturb.utils.structure_function (src/pyturb/utils.py:159-201): for a stack
 * phase (count, ny, nx) f32 (device), D[s-1] = (<(phi[i+s,j] - phi[i,j])^2> +
 * <(phi[i,j+s] - phi[i,j])^2>) / 2 for s = 1..max_sep (< min(ny, nx)), each
 * mean over all valid pairs of the stack; D is a DEVICE f64 array. */
size_t pt_structure_workspace_bytes(int count, int ny, int nx, int max_sep);
int pt_structure_function(int count, int ny, int nx, const float* phase, int max_sep, double* D,
                          void* work, size_t work_bytes, void* stream);
/* out (J, R) = X (J, K) . M (R, K)^T, f32 device, row-major (the
 * least-squares Zernike projection of pyturb.analysis.zernike_decompose,
 * src/pyturb/analysis.py:129-162, with M the pseudo-inverse of the pupil
 * design matrix built on the host). Split-K with a fixed-order reduce. */
size_t pt_matmul_nt_workspace_bytes(int R, int K, int J);
int pt_matmul_nt(int R, int K, int J, const float* M, const float* X, float* out, void* work,
                 size_t work_bytes, void* stream);
/* pyturb.analysis.temporal_psd (src/pyturb/analysis.py:183-208) for `count`
 * series of length T = grid ns (device f32, samples contiguous): psd[f] for
 * f = 0..T/2 (device f32) = mean over series of |DFT(x - mean x)|^2 * 2 dt / T.
 * T <= 8192 (any factorisation). */
size_t pt_temporal_psd_workspace_bytes(const pt_grid* grid, int count);
int pt_temporal_psd(const pt_grid* grid, int count, const float* series, double dt, float* psd,
                    void* work, size_t work_bytes, void* stream);

/* ---- tensor cores (tcgen05) ---------------------------------------------
 * Self-test of the tcgen05 path, no counterpart in the reference: one tile
 * D (128 x N) = A (128 x K) * B (N x K)^T with bf16 A, B (row-major, device)
 * and fp32 D (row-major, device), through shared-memory descriptors, an fp32
 * TMEM accumulator and tcgen05.ld. N, K multiples of 16 in [16, 256].
 * Synchronises the stream; PT_ERR_CUDA if a bounded wait timed out. */
int pt_tc_probe(int N, int K, const uint16_t* A, const uint16_t* B, float* D, void* stream);

/* ---- adjoint of the spectral frame synthesis ---------------------------
 * No counterpart in the reference (it has no gradients). The forward is
 * pt_frames, with per-layer weights folded into the spectra and the
 * subharmonic coefficients: y_f = scale * crop(Re IDFT(sum_l w_l S_l Phi_lf)
 * + low_f), Phi_lf = exp(2 pi i (fx sx[f,l] + fy sy[f,l])) (Atmosphere.
 * _integrate, src/pyturb/atmosphere.py:882-938). Backward, for upstream g
 * (F, n_out, n_out), frames in any chunks (the spectra gradient accumulates):
 *  1. pt_synth_adj_pack: z (ceil(F/2), ns, ns) complex = scale * conj(g_2p +
 *     i g_2p+1) zero-padded at (crop, crop);
 *  2. pt_ifft2(grid, z, z, ceil(F/2), ...) in place (the forward DFT by
 *     conjugation);
 *  3. pt_synth_adj_phasors: ph (L, F, 2, ns) complex from DEVICE shifts
 *     sx, sy (F, L) f64 [m], the forward's fixed-point ramps;
 *  4. pt_synth_adj_spectra: dL/dS (L, ns, ns) complex (d/dRe + i d/dIm),
 *     added to grad_spectra when accumulate != 0;
 *  5. pt_synth_adj_params: out (L, F, 3) f64 = [dL/dw_l contribution of
 *     frame f, dL/dsx[f,l], dL/dsy[f,l]];
 *  6. with subharmonic levels (atmosphere.py:921-935): pt_synth_adj_sh: out
 *     (F, 18 P + 1) f64 = per frame the projections sum_xy g_f(x, y)
 *     b_pi(crop + x) b_pj(crop + y) (re, im; p, i, j row-major) on the grid's
 *     basis rows b_pi(x) = exp(2 pi i f_pi (x - ns/2) dx), then sum_xy g_f;
 *     the caller forms the level gradients from these (9 P values a frame). */
int pt_synth_adj_pack(int ns, int F, int crop, int n_out, float scale, const float* g, float* z,
                      void* stream);
int pt_synth_adj_phasors(int ns, double pixel_scale, int L, int F, const double* sx,
                         const double* sy, float* ph, void* stream);
int pt_synth_adj_spectra(int ns, int L, int F, const float* w, const float* Z, const float* ph,
                         int accumulate, float* grad_spectra, void* stream);
int pt_synth_adj_params(int ns, double pixel_scale, int L, int F, const float* w,
                        const float* spectra, const float* Z, const float* ph, double* out,
                        void* stream);
int pt_synth_adj_sh(const pt_grid* grid, int F, int crop, int n_out, const float* g, double* out,
                    void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PYTURB_GB300_H */
