/*
 * pmgb.h -- C ABI of the GB300 particle-mesh engine (libpmgb.so).
 *
 * The engine replaces the single-device hot path of JaxPM: CIC painting and
 * reading (jaxpm/painting.py), the Fourier-space force solver
 * (jaxpm/pm.py:12-58, jaxpm/kernels.py:41-115), the FFT wrappers
 * (jaxpm/distributed.py:37-42) and the FastPM leapfrog kick/drift
 * (jaxpm/ode.py:13-82).  Every reference citation below is relative to the
 * JaxPM project root.
 *
 * Conventions
 *  - All pointers are device pointers owned by the caller unless stated.
 *    Meshes are float32, C order [nx][ny][nz].  Particle arrays are float32
 *    [np][3] (the reference layout of positions, velocities and forces).
 *    Half spectra are interleaved complex64 [nx][ny][nz/2+1].
 *  - Calls are stream ordered: they enqueue work on `stream` and return
 *    without synchronising.  `stream` is a cudaStream_t (0 = legacy default).
 *  - Every call returns PMGB_OK or an error code; pmgb_last_error() gives a
 *    message for the last failing call made by the calling thread.
 *  - Scratch memory is passed in as (workspace, workspace_bytes); the
 *    matching *_workspace_size() query returns the bytes needed.  cuFFT
 *    plans are created on first use per (device, shape, batch) and cached
 *    for the life of the process behind a mutex.
 *  - Kernels never trap and never spin: every index is wrapped into the
 *    mesh, so any finite position is safe.
 */
#ifndef PMGB_H_
#define PMGB_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *pmgb_stream_t; /* identical to cudaStream_t */

enum pmgb_status {
  PMGB_OK = 0,
  PMGB_ERR_INVALID_ARGUMENT = 1, /* bad shape, null pointer, bad mode    */
  PMGB_ERR_WORKSPACE = 2,        /* workspace missing or too small       */
  PMGB_ERR_CUDA = 3,             /* CUDA runtime error (message has it)  */
  PMGB_ERR_CUFFT = 4,            /* cuFFT error                          */
  PMGB_ERR_UNSUPPORTED = 5       /* valid request this build cannot serve */
};

/* Paint algorithms for the absolute-position painters. */
enum pmgb_paint_mode {
  PMGB_PAINT_ATOMIC = 0,  /* one thread per particle, 8 global fp32 atomics  */
  PMGB_PAINT_BINNED = 1,  /* particle chunks binned into a shared-memory box,
                             coalesced flush; global atomics when a chunk's box
                             does not fit                                   */
  PMGB_PAINT_DETERMINISTIC = 2 /* fixed-point 64-bit integer accumulation:
                             bit-identical results run to run.  Signed 32.32
                             fixed point: each contribution is rounded to a
                             multiple of 2^-32, and a cell's sum must stay
                             below 2^31 in magnitude (larger sums wrap
                             silently)                                    */
};

/* ---- library ----------------------------------------------------------- */

/* Version of this ABI (major*10000 + minor*100 + patch). */
int pmgb_version(void);

/* Message for the last failing call on this thread ("" if none). */
const char *pmgb_last_error(void);

/* Number of kernels this library has launched in this process (library
 * kernels only: cuFFT's are not counted; launches recorded into a CUDA
 * graph count once, at capture). */
uint64_t pmgb_launch_count(void);

/* ---- CIC mass assignment: absolute positions --------------------------- */

/* Scratch bytes needed by pmgb_cic_paint_f32 for this mode and size. */
size_t pmgb_cic_paint_workspace_size(int nx, int ny, int nz, int64_t np,
                                     int mode);

/* mesh[c] (+)= sum_p weight_p * W(pos_p, c), W the CIC kernel, indices
 * wrapped periodically.  weight_p = weight_scale * (weights ? weights[p] : 1).
 * accumulate = 0 overwrites mesh (it is zeroed first), 1 adds to it.
 * Replaces _cic_paint_impl / cic_paint, jaxpm/painting.py:15-45 and :48-75
 * (any particle count; the reference wrapper requires np == nx*ny*nz). */
int pmgb_cic_paint_f32(float *mesh, int nx, int ny, int nz, const float *pos,
                       int64_t np, const float *weights, float weight_scale,
                       int mode, int accumulate, void *workspace,
                       size_t workspace_bytes, pmgb_stream_t stream);

/* The deterministic paint (PMGB_PAINT_DETERMINISTIC semantics, same result
 * bit for bit) without any allocation and without a workspace argument.
 * No counterpart in the reference: it exists for callers that cannot hand
 * out device memory, such as a custom-call handler that only receives the
 * buffers its framework's allocator made, or code that must not call
 * cudaMalloc while another runtime's pool owns the device memory.  The
 * fixed-point scratch (8 bytes per cell) is a static device array inside
 * libpmgb, so meshes are limited to 128^3 = 2097152 cells (larger ones are
 * rejected with PMGB_ERR_INVALID_ARGUMENT).  A CUDA context takes those
 * 16 MiB when it first uses this code (lazy module loading, the default
 * since CUDA 12.2: the first call), or when it is created under
 * CUDA_MODULE_LOADING=EAGER, and holds them until it is destroyed.  The
 * first call in a context (the device's primary context, or the caller's
 * own current context) looks the array's address up with
 * cudaGetSymbolAddress and caches it under the context's unique id: make
 * that first call before any stream capture.  Same fixed-point range as
 * PMGB_PAINT_DETERMINISTIC (|cell sum| < 2^31, resolution 2^-32).  The scratch is
 * cleared by every call, but all calls share it: calls that overlap on the
 * GPU (different streams, or different host threads on one device) race
 * and must be serialised by the caller. */
int pmgb_cic_paint_deterministic_noalloc_f32(float *mesh, int nx, int ny,
                                             int nz, const float *pos,
                                             int64_t np, const float *weights,
                                             float weight_scale,
                                             int accumulate,
                                             pmgb_stream_t stream);

/* out[p] = sum_c W(pos_p, c) * mesh[c].
 * Replaces _cic_read_impl / cic_read, jaxpm/painting.py:78-128. */
int pmgb_cic_read_f32(const float *mesh, int nx, int ny, int nz,
                      const float *pos, int64_t np, float *out,
                      pmgb_stream_t stream);

/* Three meshes at once: mesh3 + i*comp_stride is component i;
 * out3[p][i] = read(component i).  Replaces the three cic_read calls of
 * jaxpm/pm.py:54-56 (indices and weights computed once). */
int pmgb_cic_read3_f32(const float *mesh3, int64_t comp_stride, int nx,
                       int ny, int nz, const float *pos, int64_t np,
                       float *out3, pmgb_stream_t stream);

/* Neighbour cells and weights of every particle, in the reference's order
 * (jaxpm/painting.py:21-37): idx [np][8][3] int32 (wrapped), w [np][8]. */
int pmgb_cic_weights_f32(const float *pos, int64_t np, int nx, int ny, int nz,
                         int32_t *idx, float *w, pmgb_stream_t stream);

/* Adjoint of pmgb_cic_paint_f32: given the cotangent mesh g_mesh,
 * g_pos[p][d] = weight_p * sum_c dW/dx_d * g_mesh[c]   (if g_pos != NULL)
 * g_w[p]      = sum_c W * g_mesh[c]                      (if g_w != NULL). */
int pmgb_cic_paint_vjp_f32(const float *g_mesh, int nx, int ny, int nz,
                           const float *pos, int64_t np, const float *weights,
                           float weight_scale, float *g_pos, float *g_w,
                           pmgb_stream_t stream);

/* Adjoint of pmgb_cic_read_f32: g_mesh += paint of g_out (if g_mesh != NULL),
 * g_pos[p][d] = g_out[p] * sum_c dW/dx_d * mesh[c] (if g_pos != NULL). */
int pmgb_cic_read_vjp_f32(const float *mesh, int nx, int ny, int nz,
                          const float *pos, int64_t np, const float *g_out,
                          float *g_mesh, float *g_pos, pmgb_stream_t stream);

/* ---- CIC mass assignment: relative (lattice + displacement) ------------ */

/* mesh (+)= paint of particles at lattice point i plus disp[i]; disp is
 * [nx*ny*nz][3].  Replaces cic_paint_dx, jaxpm/painting.py:161-215, with the
 * enmesh arithmetic of jaxpm/painting_utils.py:28-96. */
int pmgb_cic_paint_dx_f32(float *mesh, int nx, int ny, int nz,
                          const float *disp, const float *weights,
                          float weight_scale, int accumulate,
                          pmgb_stream_t stream);

/* out[i] = read at lattice point i plus disp[i].
 * Replaces cic_read_dx, jaxpm/painting.py:218-260. */
int pmgb_cic_read_dx_f32(const float *mesh, int nx, int ny, int nz,
                         const float *disp, float *out, pmgb_stream_t stream);

/* Neighbours and weights of the relative mode, in its neighbour order
 * (jaxpm/painting_utils.py:43-45,84-96): idx [n][8][3], w [n][8]. */
int pmgb_enmesh_f32(const float *disp, int nx, int ny, int nz, int32_t *idx,
                    float *w, pmgb_stream_t stream);

/* ---- FFT (jaxpm/distributed.py:37-42) ---------------------------------- */

/* Forward real-to-complex 3-D FFT, unnormalised, of `batch` meshes
 * (in + b*nx*ny*nz -> out + b*nx*ny*(nz/2+1)).  Replaces fft3d of a real
 * field (the reference transforms C2C; the half spectrum is identical). */
int pmgb_fft_r2c_f32(const float *in, void *out, int nx, int ny, int nz,
                     int batch, pmgb_stream_t stream);

/* Inverse complex-to-real 3-D FFT of `batch` half spectra, scaled by
 * 1/(nx*ny*nz) when normalize != 0.  The input is overwritten.  Replaces
 * ifft3d(x) = pifft3d(x).real. */
int pmgb_fft_c2r_f32(void *in, float *out, int nx, int ny, int nz, int batch,
                     int normalize, pmgb_stream_t stream);

/* The library's own 3-D FFT (power-of-two nx in [8,1024], ny in [64,512],
 * nz in [16,512]): a y-z plane transform (cuFFT's batched 2-D transforms,
 * or under PMGB_FFT_OWN the library's cluster-of-CTAs kernels) and the
 * library's x-column transform, in-place radix-8 stages in shared memory.
 * Its half spectra
 * use padded rows: [nx][ny][pmgb_fft3_pitch(nz)] complex, modes
 * kz < nz/2+1 meaningful (the forward transform zeroes the padding).  The
 * composite force calls (pmgb_pm_forces_f32, the FastPM steps and their
 * adjoints) use it, fused with the k-space kernel, whenever the mesh shape
 * allows; otherwise cuFFT.  No reference counterpart: the reference's
 * fft3d (distributed.py:37-42) is XLA's FFT. */
int pmgb_fft3_supported(int nx, int ny, int nz);
int pmgb_fft3_pitch(int nz);

/* Forward R2C, unnormalised, of `batch` meshes (16-byte aligned input):
 * in + b*nx*ny*nz -> out + b*nx*ny*pitch. */
int pmgb_fft3_r2c_f32(const float *in, void *out, int nx, int ny, int nz,
                      int batch, pmgb_stream_t stream);

/* Inverse C2R, unnormalised, of `batch` padded half spectra (overwritten)
 * into 16-byte aligned meshes.  The imaginary parts of the kz = 0 and
 * kz = nz/2 modes are ignored. */
int pmgb_fft3_c2r_f32(void *in, float *out, int nx, int ny, int nz, int batch,
                      pmgb_stream_t stream);

/* FFT path of the composite calls (process-wide): PMGB_FFT_CUFFT (cuFFT
 * 3-D R2C, pmgb_kspace_forces_f32, batched C2R), PMGB_FFT_FUSED (default:
 * cuFFT's batched 2-D plane transforms around the library's x-direction
 * kernel that fuses the forward x transform, the k-space multiply and the
 * inverse x transforms) or PMGB_FFT_OWN (the library's plane kernels too).
 * The last two apply where pmgb_fft3_supported; other shapes use cuFFT. */
enum pmgb_fft_path { PMGB_FFT_CUFFT = 0, PMGB_FFT_FUSED = 1, PMGB_FFT_OWN = 2 };
int pmgb_set_fft_path(int path);
int pmgb_fft_path(void);

/* Launch choices of the tile-sorted run loop (process-wide, read at every
 * launch): the quarters of the tiles the gather deals to its CTAs
 * statically before the rest go to whichever CTA asks first (0 to 4;
 * default 3), and the CTAs per SM of the gather and of the re-sort (0, the
 * default: as many as fit; otherwise at most that many), and the priority
 * of the re-sort's stream (0, the default: the device's highest, so its
 * blocks go ahead of the next force evaluation's; 1: the default priority,
 * so they fill in beside it).  Set by the
 * autotuner (jaxpm_gb300/autotune.py), which times the candidates on the
 * caller's own workload.  No counterpart in the reference: XLA picks the
 * launch shapes of its scatter and gather (painting.py:43-44, :104-106). */
typedef struct {
  int gather_static_quarters;
  int gather_ctas_per_sm;
  int resort_ctas_per_sm;
  int resort_priority;
  int reserved[4];
} pmgb_tuning;
int pmgb_get_tuning(pmgb_tuning *out);
int pmgb_set_tuning(const pmgb_tuning *in);

/* Launch timing of pmgb_fpm_run_sorted_f32 (process-wide, off by default):
 * while enabled, each run records CUDA events on its streams around every
 * gather, every force evaluation and every re-sort of the permutation.
 * Once the run's stream has been synchronised, pmgb_run_timing returns the
 * last timed run's mean milliseconds per launch of each phase (the re-sort
 * over the steps but the last, whose full sort differs) and its step
 * count; any pointer may be NULL.  An error before any timed run, or while
 * the run is still in flight.  Runs hold a process-wide lock while timing
 * is on.  No counterpart in the reference (XLA's profiler). */
int pmgb_set_run_timing(int enable);
int pmgb_run_timing(double *gather_ms, double *forces_ms, double *resort_ms, int *steps);

/* ---- Fourier-space force kernel (jaxpm/pm.py:49-56) --------------------- */

/* The spectral part of pm_forces on a real density mesh (pm.py:30-56 from
 * delta to the three force meshes, before the read):
 * force3[i] = ifft3d(-grad_i * invlaplace * longrange * fft3d(mesh)),
 * [3][nx][ny][nz].  Through the library's FFT pipeline where
 * pmgb_fft3_supported and the pointers are 16-byte aligned, else cuFFT
 * R2C + pmgb_kspace_forces_f32 + C2R.  mesh is not modified. */
size_t pmgb_mesh_forces_workspace_size(int nx, int ny, int nz);
int pmgb_mesh_forces_f32(const float *mesh, float *force3, int nx, int ny,
                         int nz, float r_split, void *workspace,
                         size_t workspace_bytes, pmgb_stream_t stream);

/* Adjoint: g_mesh = sum_i (ifft3d K_i fft3d)^T g_force3[i]. */
/* The potential of the run loop, pot = IFFT(delta_k * invlaplace *
 * longrange) (pm.py:49-53) as a real mesh [nx][ny][nz], through the spectral
 * pipeline (PMGB_ERR_UNSUPPORTED outside its shapes).  The forces of
 * pmgb_mesh_forces_f32 are its order-1 gradient, the stencil
 * (8 (p[+1] - p[-1]) - (p[+2] - p[-2])) / 12 per axis, negated.  Workspace:
 * pmgb_mesh_forces_workspace_size. */
int pmgb_mesh_potential_f32(const float *mesh, float *pot, int nx, int ny,
                            int nz, float r_split, void *workspace,
                            size_t workspace_bytes, pmgb_stream_t stream);

int pmgb_mesh_forces_vjp_f32(const float *g_force3, float *g_mesh, int nx,
                             int ny, int nz, float r_split, void *workspace,
                             size_t workspace_bytes, pmgb_stream_t stream);

/* One pass from delta_k to the three force spectra:
 * force_k[i] = -grad_i(k) * invlaplace(k) * longrange(k) * delta_k * scale,
 * grad order 1 = i(8 sin w - sin 2w)/6 or order 0 = i k with the Nyquist
 * entry zeroed (jaxpm/kernels.py:41-66); invlaplace = -1/k^2, k=0 -> 0,
 * fd_laplace selects the sinc-corrected form (kernels.py:69-92); longrange =
 * exp(-k^2 r_split^2) or 1 (kernels.py:95-115).  force_k + i*comp_stride is
 * component i.  Pass scale = 1/(nx*ny*nz) to fold the inverse-FFT
 * normalisation in. */
int pmgb_kspace_forces_f32(const void *delta_k, void *force_k,
                           int64_t comp_stride, int nx, int ny, int nz,
                           float r_split, int grad_order, int fd_laplace,
                           float scale, pmgb_stream_t stream);

/* Adjoint of pmgb_kspace_forces_f32 on half spectra:
 * g_delta_k = sum_i conj(K_i(k)) * g_force_k[i] * scale. */
int pmgb_kspace_forces_vjp_f32(const void *g_force_k, int64_t comp_stride,
                               void *g_delta_k, int nx, int ny, int nz,
                               float r_split, int grad_order, int fd_laplace,
                               float scale, pmgb_stream_t stream);

/* One-multiply-per-kernel forms of the same operator (comparison baseline):
 * spec *= invlaplace(k)*scale; spec *= longrange(k); out = -grad_d(k)*in. */
int pmgb_kspace_invlaplace_f32(void *spec, int nx, int ny, int nz,
                               int fd_laplace, float scale,
                               pmgb_stream_t stream);
int pmgb_kspace_longrange_f32(void *spec, int nx, int ny, int nz,
                              float r_split, pmgb_stream_t stream);
int pmgb_kspace_gradient_f32(const void *in, void *out, int nx, int ny, int nz,
                             int direction, int grad_order,
                             pmgb_stream_t stream);

/* ---- FastPM step (jaxpm/ode.py:13-82) ----------------------------------- */

/* Fused gather + leapfrog update: F = read3(force meshes at pos),
 * vel += kick * F, pos += drift * vel (both in place).  If forces_out is
 * not NULL, F is also stored [np][3].  kick/drift are the host-computed
 * FastPM coefficients (growth-factor kick and drift of ode.py:20-80 times
 * the step, with 1.5*Omega_m folded into kick). */
int pmgb_read3_kick_drift_f32(const float *force3, int64_t comp_stride, int nx,
                              int ny, int nz, float *pos, float *vel,
                              int64_t np, float kick, float drift,
                              float *forces_out, pmgb_stream_t stream);

/* Separate kick (vel += kick*forces) and drift (pos += drift*vel) kernels
 * of the one-kernel-per-op form. */
int pmgb_kick_f32(float *vel, const float *forces, int64_t np, float kick,
                  pmgb_stream_t stream);
int pmgb_drift_f32(float *pos, const float *vel, int64_t np, float drift,
                   pmgb_stream_t stream);

/* ---- composite calls ---------------------------------------------------- */

/* Scratch bytes for pmgb_pm_forces_f32 / pmgb_fpm_step_f32 /
 * pmgb_pm_forces_vjp_f32 on this mesh and particle count. */
size_t pmgb_pm_workspace_size(int nx, int ny, int nz, int64_t np,
                              int paint_mode);

/* forces[p] = pm_forces(pos)[p] (jaxpm/pm.py:12-58 with
 * paint_absolute_pos=True): paint, R2C, fused k-space kernel, batched C2R,
 * read3. */
int pmgb_pm_forces_f32(const float *pos, int64_t np, int nx, int ny, int nz,
                       float r_split, int paint_mode, float *forces,
                       void *workspace, size_t workspace_bytes,
                       pmgb_stream_t stream);

/* One fused FastPM step on (pos, vel) in place: forces at pos, kick, drift
 * (jaxpm/ode.py:35-58 kick then :20-33 drift, forces of pm.py:12-58).
 * If force3_out is not NULL the three force meshes [3][nx][ny][nz] of this
 * step are copied there (for adjoints). */
int pmgb_fpm_step_f32(float *pos, float *vel, int64_t np, int nx, int ny,
                      int nz, float kick, float drift, float r_split,
                      int paint_mode, void *workspace, size_t workspace_bytes,
                      pmgb_stream_t stream);

/* The same step as one kernel per operation: global-atomic paint, R2C,
 * invlaplace, longrange, three gradient multiplies, three C2R, three
 * separate reads, kick, drift.  The comparison baseline. */
int pmgb_fpm_step_plain_f32(float *pos, float *vel, int64_t np, int nx,
                            int ny, int nz, float kick, float drift,
                            float r_split, void *workspace,
                            size_t workspace_bytes, pmgb_stream_t stream);

/* Vector-Jacobian product of pm_forces w.r.t. positions:
 * g_pos = (d forces / d pos)^T g_forces (overwritten).  Recomputes the
 * forward meshes, paints the cotangents, applies the adjoint k-space
 * operator and gathers both position terms in one pass. */
int pmgb_pm_forces_vjp_f32(const float *pos, int64_t np, int nx, int ny,
                           int nz, float r_split, int paint_mode,
                           const float *g_forces, float *g_pos,
                           void *workspace, size_t workspace_bytes,
                           pmgb_stream_t stream);

/* ---- tile-sorted particle state (the fused FastPM loop) ----------------- */
/* The fast loop keeps (pos, vel) physically ordered by the 8^3-cell mesh
 * tile that holds each particle (tiles in Morton order), with id[p] the
 * particle's index in the caller's order.  Forces, kicks and drifts are
 * per particle, so the order changes no result; pmgb_unpermute3_f32 returns
 * arrays to the caller's order. */

/* Scratch bytes of pmgb_tile_sort_f32 / pmgb_fpm_step_sorted_f32 (tile
 * counts, offsets and one rank per particle). */
size_t pmgb_tile_sort_workspace_size(int nx, int ny, int nz, int64_t np);

/* Counting sort by tile: (pos, vel, id) -> (pos_out, vel_out, id_out).
 * vel/vel_out may be NULL; id NULL means the identity (id_out[q] = index of
 * the particle now at q). */
int pmgb_tile_sort_f32(const float *pos, const float *vel, const uint32_t *id,
                       int64_t np, int nx, int ny, int nz, float *pos_out,
                       float *vel_out, uint32_t *id_out, void *workspace,
                       size_t workspace_bytes, pmgb_stream_t stream);

/* out[id[p]] = in[p] for [np][3] arrays (back to the caller's order). */
int pmgb_unpermute3_f32(const float *in, const uint32_t *id, int64_t np,
                        float *out, pmgb_stream_t stream);

/* out[p] = in[id[p]] for [np][3] arrays (caller's order -> tile order). */
int pmgb_permute3_f32(const float *in, const uint32_t *id, int64_t np,
                      float *out, pmgb_stream_t stream);

/* pmgb_tile_sort_f32 that also records dest[p], the slot particle p went
 * to: out[p] = sorted[dest[p]] (pmgb_gather3_f32) returns a sorted array to
 * the caller's order with coalesced writes, in any number of pieces. */
int pmgb_tile_sort_dest_f32(const float *pos, const float *vel,
                            const uint32_t *id, int64_t np, int nx, int ny,
                            int nz, float *pos_out, float *vel_out,
                            uint32_t *id_out, uint32_t *dest, void *workspace,
                            size_t workspace_bytes, pmgb_stream_t stream);

/* out[p] = in[idx[p]] for p < n, in an [n_in][3] array (entries of idx at
 * or past n_in are skipped); out must not overlap in.  With idx = dest + a
 * and out = caller_array + 3 a it fills rows a .. a+n-1 of the caller's
 * order: the pieces a run returns to the host as each one is ready.  No
 * counterpart in the reference (JAX arrays never leave their order). */
int pmgb_gather3_f32(const float *in, int64_t n_in, const uint32_t *idx,
                     int64_t n, float *out, pmgb_stream_t stream);

/* Failure check of the tile-staged kernels: waits for `stream`, reads the
 * three counters a tile kernel kept in `stats` and returns
 * PMGB_ERR_CUDA if [2] is set, i.e. a wait on a TMA transfer reached its
 * spin limit and the kernel abandoned its work (the results of every call
 * since the counters were zeroed are then invalid); PMGB_OK otherwise, and
 * for stats == NULL.  No counterpart in the reference: JAX raises on its own
 * errors; here a device-side failure is reported through these counters
 * instead of a trap, which would take down the context.  The Python engine
 * calls it after every run, reverse sweep and host-state run. */
int pmgb_check_stats(const uint32_t *stats, pmgb_stream_t stream);

/* Test of the bounded wait behind that check: one CTA arms an mbarrier for
 * 16 bytes, issues no copy and waits for at most spin_limit polls (1 to
 * 2^20); *status (a device word) becomes 1 when the wait ran out, 0 if it
 * completed.  Nothing is in flight, so the kernel ends at once and the
 * context stays usable.  No counterpart in the reference. */
int pmgb_test_wait_timeout(uint32_t spin_limit, uint32_t *status,
                           pmgb_stream_t stream);

/* Paint of tile-sorted particles (the sorted loop's paint; mesh overwritten):
 * one CTA per tile accumulates the tile plus a one-cell halo in shared
 * memory (exact fixed point with native 32-bit atomics) from the
 * particle range recorded in sort_workspace by the last pmgb_tile_sort_f32 /
 * pmgb_tile_scatter_f32, then adds the box to the mesh with one TMA bulk
 * reduce-add (tiles whose box wraps around the mesh use 16-byte atomics).
 * Same result as pmgb_cic_paint_f32 up to the order of the float sums.
 * stats (nullable, 3 counters): [0] particles found outside their tile
 * (stale ranges; painted with global atomics), [2] set if a wait on a TMA
 * transfer reached its spin limit (the work was abandoned). */
int pmgb_cic_paint_sorted_f32(float *mesh, int nx, int ny, int nz,
                              const float *pos, int64_t np,
                              void *sort_workspace,
                              size_t sort_workspace_bytes, uint32_t *stats,
                              pmgb_stream_t stream);

/* Tile-staged gather + kick + drift of tile-sorted particles (the sorted
 * loop's read): one CTA per tile stages the tile plus a one-cell halo of
 * the three force meshes in shared memory (TMA bulk tensor loads, the next
 * tile's box prefetched into a second buffer) and interpolates from there.
 * Same results as pmgb_read3_kick_drift_f32.  It also counts the new
 * positions per tile and records each particle's rank in its new tile in
 * sort_workspace, for pmgb_tile_scatter_f32.  stats (nullable, 3
 * counters): [1] particles found outside their tile, [2] set if a TMA wait
 * reached its spin limit. */
int pmgb_read3_kick_drift_binned_f32(const float *force3, int64_t comp_stride,
                                     int nx, int ny, int nz, float *pos,
                                     float *vel, int64_t np, float kick,
                                     float drift, void *sort_workspace,
                                     size_t sort_workspace_bytes,
                                     uint32_t *stats, pmgb_stream_t stream);

/* pmgb_read3_kick_drift_binned_f32 that also paints the new positions into
 * mesh_next (overwritten): the density of the next step.  Particles that
 * stay in their tile paint into the tile's box in shared memory, added to
 * the mesh with TMA reduces; those that left it paint with global atomics.
 * The next step then needs no separate paint pass.  Same density as
 * pmgb_cic_paint_sorted_f32 of the new positions up to the order of the
 * float sums.  stats: as pmgb_read3_kick_drift_binned_f32. */
int pmgb_read3_kick_drift_paint_binned_f32(const float *force3,
                                           int64_t comp_stride, int nx, int ny,
                                           int nz, float *pos, float *vel,
                                           int64_t np, float kick, float drift,
                                           float *mesh_next,
                                           void *sort_workspace,
                                           size_t sort_workspace_bytes,
                                           uint32_t *stats,
                                           pmgb_stream_t stream);

/* Exclusive scan of the tile counts left in sort_workspace by
 * pmgb_read3_kick_drift_binned_f32, then the scatter of (pos, vel, id) to
 * (pos_out, vel_out, id_out) in tile order; dest_out (nullable) receives
 * each particle's new index. */
int pmgb_tile_scatter_f32(const float *pos, const float *vel,
                          const uint32_t *id, int64_t np, int nx, int ny,
                          int nz, float *pos_out, float *vel_out,
                          uint32_t *id_out, uint32_t *dest_out,
                          void *sort_workspace, size_t sort_workspace_bytes,
                          pmgb_stream_t stream);

/* One FastPM step on tile-sorted particles (jaxpm/ode.py:35-58 kick and
 * :20-33 drift, forces of jaxpm/pm.py:12-58): shared-memory box paint,
 * R2C, fused k-space kernel, batched C2R, box-staged gather + kick + drift
 * that also counts the new positions per tile, scan, scatter.  Reads
 * (pos, vel, id) and writes the advanced state, sorted by the new
 * positions, to (pos_out, vel_out, id_out); pos and id are left unchanged
 * (the drifted positions pass through the workspace), vel holds the kicked
 * velocities in the old order on return.  `workspace` is sized by
 * pmgb_pm_workspace_size(..., PMGB_PAINT_BINNED), `sort_workspace` by
 * pmgb_tile_sort_workspace_size.  What the reverse step needs can be
 * recorded (each nullable): force3_out [3][nx][ny][nz] receives the force
 * meshes (computed there in place of the workspace), dest_out [np] each
 * particle's index after the step, offsets_out the tile ranges of the
 * order the step started from (pmgb_tile_key_count + 1 entries).  stats
 * (nullable, 3 counters the caller zeroes): see pmgb_cic_paint_sorted_f32
 * and pmgb_read3_kick_drift_binned_f32. */
int pmgb_fpm_step_sorted_f32(const float *pos, float *vel, const uint32_t *id,
                             float *pos_out, float *vel_out, uint32_t *id_out,
                             int64_t np, int nx, int ny, int nz, float kick,
                             float drift, float r_split, void *workspace,
                             size_t workspace_bytes, void *sort_workspace,
                             size_t sort_workspace_bytes, float *force3_out,
                             uint32_t *dest_out, uint32_t *offsets_out,
                             uint32_t *stats, pmgb_stream_t stream);

/* n_steps FastPM steps of tile-sorted particles (the time loop of
 * jaxpm/ode.py driven over a_i = a0 + i da): each step as
 * pmgb_fpm_step_sorted_f32, except that the density of every step after the
 * first is painted by the previous step's gather
 * (pmgb_read3_kick_drift_paint_binned_f32), so each step reads the
 * particles once, and that between steps the particles are not moved: each
 * gather reads its tiles' particles through a permutation and writes them
 * in the order it read them, so the re-sort only rebuilds the permutation
 * (8 bytes per particle); one full sort after the last step leaves the
 * state in tile order.  The sort_workspace must hold the tile ranges of
 * (pos_a, ...) (as left by pmgb_tile_sort_f32 or a previous step).  kick and
 * drift are HOST arrays of n_steps coefficients.  The state ping-pongs
 * between the a and b buffers: after the call it is in a when n_steps is
 * even, in b when odd. */
/* pmgb_read3_kick_drift_paint_binned_f32 with the forces derived from the
 * potential mesh (pmgb_mesh_potential_f32) in each tile's shared-memory box:
 * the gather of the run loop.  mesh_next may be NULL (no paint). */
int pmgb_read_potential_kick_drift_paint_binned_f32(const float *pot, int nx,
                                                    int ny, int nz, float *pos,
                                                    float *vel, int64_t np,
                                                    float kick, float drift,
                                                    float *mesh_next,
                                                    void *sort_workspace,
                                                    size_t sort_workspace_bytes,
                                                    uint32_t *stats,
                                                    pmgb_stream_t stream);

/* The run loop's gather in its permuted form: slot p of the tile ranges in
 * sort_workspace is the particle at index perm[p] of (pos, vel) (perm NULL:
 * index p), gathered from the potential as
 * pmgb_read_potential_kick_drift_paint_binned_f32 does, and written to index
 * p of (pos_out, vel_out); its new tile key goes to the sort workspace for
 * pmgb_tile_resort_index.  With perm the outputs are other buffers than the
 * inputs; without it they may be the inputs (an in-place update).  The
 * particles then never move between steps: only the permutation is
 * re-sorted, and the ids follow it there.  No counterpart of its own in the
 * reference: it is the reference's cic_read x3 + kick + drift + next
 * cic_paint (pm.py:54-56, ode.py:20-58, painting.py:15-45) in the order the
 * particles already lie. */
int pmgb_read_potential_kick_drift_paint_perm_f32(
    const float *pot, int nx, int ny, int nz, const float *pos, const float *vel,
    const uint32_t *perm, float *pos_out, float *vel_out, int64_t np, float kick,
    float drift, float *mesh_next, void *sort_workspace,
    size_t sort_workspace_bytes, uint32_t *stats, pmgb_stream_t stream);

/* The permuted loop's re-sort: the exclusive scan of the tile counts left by
 * the last permuted gather, then perm_new[d] = p for every slot p, d the
 * slot it claims in its new tile (from the keys the gather wrote).  With
 * perm_old (the permutation that gather read through) the ids follow:
 * id_out[p] = id_in[perm_old[p]].  8 bytes of traffic per particle (20
 * with the ids) instead of moving (pos, vel, id). */
int pmgb_tile_resort_index(int64_t np, int nx, int ny, int nz,
                           const uint32_t *perm_old, uint32_t *perm_new,
                           const uint32_t *id_in, uint32_t *id_out,
                           void *sort_workspace, size_t sort_workspace_bytes,
                           pmgb_stream_t stream);

/* out[p] = in[idx[p]] for np 32-bit words (the ids after a permuted
 * gather, before the run's final full sort). */
int pmgb_gather_u32(const uint32_t *in, const uint32_t *idx, int64_t np,
                    uint32_t *out, pmgb_stream_t stream);

/* The forward run of the reverse sweep, recording what each step's
 * pmgb_fpm_step_sorted_vjp_f32 needs, as one call with the run loop's
 * fusions (each later density painted by the previous gather, the sort
 * overlapped with the next forces).  xs: [n_steps][np][3], xs[0] holds the
 * initial positions in tile order (ranges in sort_workspace); step i writes
 * the positions it ends with into xs[i+1] (the last step into pos_out), its
 * force meshes into force3s[i] ([n_steps][3][nx][ny][nz]), the re-sort map
 * into dests[i] ([n_steps][np]) and the tile ranges it started from into
 * offsets[i] ([n_steps][keys+1]).  Velocities and ids ping-pong between the
 * a and b buffers (final state in b when n_steps is odd); kick and drift are
 * HOST arrays of n_steps coefficients. */
int pmgb_fpm_run_sorted_record_f32(float *xs, float *vel_a, uint32_t *id_a,
                                   float *vel_b, uint32_t *id_b, float *pos_out,
                                   int64_t np, int nx, int ny, int nz,
                                   int n_steps, const float *kick,
                                   const float *drift, float r_split,
                                   void *workspace, size_t workspace_bytes,
                                   void *sort_workspace,
                                   size_t sort_workspace_bytes, float *force3s,
                                   uint32_t *dests, uint32_t *offsets,
                                   uint32_t *stats, pmgb_stream_t stream);

/* The same recording run keeping each step's potential instead of its three
 * force meshes: potentials[i] ([n_steps][nx][ny][nz]) is step i's
 * potential, from which that step's gather (and its reverse step,
 * pmgb_fpm_step_sorted_vjp_pot_f32) derive the forces with the order-1
 * gradient stencil, as pmgb_fpm_run_sorted_f32 does.  A third of the
 * recorded mesh bytes.  PMGB_ERR_UNSUPPORTED outside the potential
 * pipeline's shapes (pmgb_fft3_supported). */
int pmgb_fpm_run_sorted_record_pot_f32(float *xs, float *vel_a, uint32_t *id_a,
                                       float *vel_b, uint32_t *id_b,
                                       float *pos_out, int64_t np, int nx,
                                       int ny, int nz, int n_steps,
                                       const float *kick, const float *drift,
                                       float r_split, void *workspace,
                                       size_t workspace_bytes,
                                       void *sort_workspace,
                                       size_t sort_workspace_bytes,
                                       float *potentials, uint32_t *dests,
                                       uint32_t *offsets, uint32_t *stats,
                                       pmgb_stream_t stream);

int pmgb_fpm_run_sorted_f32(float *pos_a, float *vel_a, uint32_t *id_a,
                            float *pos_b, float *vel_b, uint32_t *id_b,
                            int64_t np, int nx, int ny, int nz, int n_steps,
                            const float *kick, const float *drift,
                            float r_split, void *workspace,
                            size_t workspace_bytes, void *sort_workspace,
                            size_t sort_workspace_bytes, uint32_t *stats,
                            pmgb_stream_t stream);

/* Number of tile keys of a mesh (the sorted loop's tile ranges have one
 * more entry). */
int64_t pmgb_tile_key_count(int nx, int ny, int nz);

/* Reverse (vector-Jacobian) step of pmgb_fpm_step_sorted_f32, on the
 * quantities that step recorded: pos = the positions it started from (tile
 * order i), force3 its force meshes, dest where each particle went
 * (order i -> i+1; NULL = identity), tile_offsets the ranges of order i.
 * Given the cotangents (g_pos_in, g_vel_in) of its outputs (order i+1), it
 * writes those of its inputs (order i):
 *   u = g_vel[dest] + drift * g_pos[dest],   g_vel_out = u,
 *   g_pos_out = g_pos[dest] + (dF/dx)^T (kick * u),
 * the force Jacobian-transpose product being a tile-sorted paint of the
 * three cotangent components (block-scaled fixed point in shared memory,
 * TMA reduce), three R2C, the conjugate k-space multiply, one C2R, and a
 * TMA-staged gather of both position terms.  Adjoint of the kick
 * (ode.py:35-80), the drift (:20-33) and pm_forces (pm.py:12-58); the
 * reference differentiates these with JAX's autodiff. */
int pmgb_fpm_step_sorted_vjp_f32(const float *pos, const float *force3,
                                 const uint32_t *dest,
                                 const uint32_t *tile_offsets,
                                 const float *g_pos_in, const float *g_vel_in,
                                 float *g_pos_out, float *g_vel_out,
                                 int64_t np, int nx, int ny, int nz,
                                 float kick, float drift, float r_split,
                                 void *workspace, size_t workspace_bytes,
                                 uint32_t *stats, pmgb_stream_t stream);

/* The cotangents of a recorded sorted step's kick and drift coefficients
 * (for gradients with respect to the cosmology, on which they depend),
 * added to two device doubles: out[0] += <g_vel, F(pos)>, F the CIC read
 * of the step's force meshes (comp_stride apart) at the positions it started
 * from, g_vel the velocity cotangent pmgb_fpm_step_sorted_vjp_f32 returned
 * (both order i); out[1] += <g_pos_next[dest], pos_next[dest] - pos>, with
 * pos_next the positions the step ended with and g_pos_next their cotangents
 * (order i+1; dest NULL = identity), i.e. drift * <g_x', v'>.  The kick's
 * cotangent is out[0], the drift's out[1] / drift.  The reference gets them
 * from JAX's autodiff through ode.py:20-80. */
int pmgb_fpm_coef_cotangents_f32(const float *pos, const float *pos_next,
                                 const uint32_t *dest, const float *force3,
                                 int64_t comp_stride, int nx, int ny, int nz,
                                 const float *g_pos_next, const float *g_vel,
                                 int64_t np, double *out, pmgb_stream_t stream);

/* pmgb_fpm_step_sorted_vjp_f32 for a step recorded by
 * pmgb_fpm_run_sorted_record_pot_f32: `potential` is the potential the step
 * took its forces from; the reverse gather derives each tile's forces from
 * a TMA-staged potential box. */
int pmgb_fpm_step_sorted_vjp_pot_f32(const float *pos, const float *potential,
                                     const uint32_t *dest,
                                     const uint32_t *tile_offsets,
                                     const float *g_pos_in,
                                     const float *g_vel_in, float *g_pos_out,
                                     float *g_vel_out, int64_t np, int nx,
                                     int ny, int nz, float kick, float drift,
                                     float r_split, void *workspace,
                                     size_t workspace_bytes, uint32_t *stats,
                                     pmgb_stream_t stream);

/* ---- initial conditions (jaxpm/pm.py:61-144) ----------------------------- */

/* linear_field colouring (jaxpm/pm.py:134-143) on a half spectrum:
 * spec *= sqrt(interp(|k|, table_k, table_p) * nx*ny*nz / V) * scale with
 * |k| = sqrt(sum_i (w_i / box_i * n_i)^2), w_i = 2*pi*fftfreq(n_i), and
 * interp the clamped linear interpolation of jnp.interp.  table_k/table_p
 * are device float32 arrays of n_table entries, table_k increasing. */
int pmgb_linear_field_colour_f32(void *spec, int nx, int ny, int nz,
                                 float box_x, float box_y, float box_z,
                                 const float *table_k, const float *table_p,
                                 int n_table, float scale,
                                 pmgb_stream_t stream);

/* Scratch bytes for pmgb_lpt2_source_f32. */
size_t pmgb_lpt2_source_workspace_size(int nx, int ny, int nz);

/* Adjoint of the 2LPT source as a function of the real linear field ic
 * (R2C then pmgb_lpt2_source_f32): the cotangent g_delta2 of delta2 ->
 * g_ic.  The maps ic -> phi_ij are real convolutions with even kernels
 * (self-adjoint), so g_ic = sum_ij phi_ij-operator(d delta2/d phi_ij *
 * g_delta2).  Workspace: pmgb_lpt2_source_workspace_size bytes. */
int pmgb_lpt2_source_vjp_f32(const float *ic, const float *g_delta2,
                             float *g_ic, int nx, int ny, int nz,
                             void *workspace, size_t workspace_bytes,
                             pmgb_stream_t stream);

/* Second-order LPT source (jaxpm/pm.py:88-109): from the half spectrum
 * delta_k, delta2 = sum_{i<j} (phi_ii phi_jj - phi_ij^2) with
 * phi_ij = ifft3d(grad_i grad_j * invlaplace * delta_k). */
int pmgb_lpt2_source_f32(const void *delta_k, float *delta2, int nx, int ny,
                         int nz, void *workspace, size_t workspace_bytes,
                         pmgb_stream_t stream);

/* out = ca*a + cb*b over n floats (b may be NULL: out = ca*a): the LPT
 * combinations dx, p, f of jaxpm/pm.py:85-87 and :118-124. */
int pmgb_lpt_combine_f32(const float *a, const float *b, int64_t n, float ca,
                         float cb, float *out, pmgb_stream_t stream);

/* ---- power spectrum (jaxpm/utils.py:14-128) ------------------------------ */

/* Binned auto power of a half spectrum (the unnormalised R2C of a mesh):
 * for bin b (np.digitize of |k| against kedges[0..n_edges-1], b in
 * 0..n_edges), psum[b] = sum |X|^2/(nx*ny*nz), pcount[b] = number of modes,
 * ksum[b] = sum |k|, all over the full spectrum (modes with
 * 0 < kz < nz/2 count twice).  |k| uses box lengths (h/Mpc).  Output arrays
 * are device float64 [n_edges+1]; n_edges <= 2000. */
int pmgb_power_spectrum_f32(const void *spec, int nx, int ny, int nz,
                            double box_x, double box_y, double box_z,
                            const double *kedges, int n_edges, double *psum,
                            double *pcount, double *ksum,
                            pmgb_stream_t stream);

/* ---- batched simulations (jax.vmap over the step: README.md:29,
 *      tests/test_distributed_pm.py:335-409) ------------------------------ */

/* One simulation of a batch: its mesh and its particle count.  The batch's
 * particle arrays are the concatenation, in table order, of every
 * simulation's [np][3] array (positions in that simulation's cell units). */
typedef struct pmgb_sim {
  int32_t nx, ny, nz;
  int32_t reserved; /* 0 */
  int64_t np;
} pmgb_sim;

/* Workspace bytes of the batched calls for this table (0 if the table is
 * invalid).  Simulations of equal mesh shape share batched FFT plans. */
size_t pmgb_batch_workspace_size(const pmgb_sim *sims, int n_sims);

/* Prepares a 256-byte aligned workspace for this table: uploads the device
 * descriptor table (stream ordered) and creates the FFT plans and k-space
 * tables of every mesh shape, so that the batched steps below only launch
 * work (and can be captured in a CUDA graph).  Every batched call checks
 * that its workspace was prepared for the same table. */
int pmgb_batch_init(const pmgb_sim *sims, int n_sims, void *workspace,
                    size_t workspace_bytes, pmgb_stream_t stream);

/* Forgets the preparation of a workspace (before freeing it). */
int pmgb_batch_release(const void *workspace);

/* Totals of a table: particles and mesh cells. */
int pmgb_batch_counts(const pmgb_sim *sims, int n_sims, int64_t *np_total,
                      int64_t *cells_total);

/* Unit-mass CIC paint of every simulation (painting.py:15-45): `meshes` is
 * the table-ordered concatenation of every simulation's [nx][ny][nz] mesh
 * (cleared here). */
int pmgb_cic_paint_batched_f32(const pmgb_sim *sims, int n_sims, float *meshes,
                               const float *pos, void *workspace,
                               size_t workspace_bytes, pmgb_stream_t stream);

/* pm_forces (pm.py:12-58, r_split as there) of every simulation at its
 * particles: pos, forces [sum np][3]. */
int pmgb_pm_forces_batched_f32(const pmgb_sim *sims, int n_sims,
                               const float *pos, float *forces, float r_split,
                               void *workspace, size_t workspace_bytes,
                               pmgb_stream_t stream);

/* One FastPM step of every simulation (as pmgb_fpm_step_f32, ode.py:13-82):
 * vel += kick[s] F(pos); pos += drift[s] vel, with kick and drift DEVICE
 * arrays of n_sims coefficients (one cosmology per simulation).  pos_before
 * (optional, [sum np][3]) receives the positions before the step, the
 * record the reverse sweep needs. */
int pmgb_fpm_step_batched_f32(const pmgb_sim *sims, int n_sims, float *pos,
                              float *vel, const float *kick, const float *drift,
                              float r_split, float *pos_before, void *workspace,
                              size_t workspace_bytes, pmgb_stream_t stream);

/* Adjoint of pmgb_fpm_step_batched_f32 from the step's starting positions
 * `pos`: (g_pos, g_vel) hold the cotangents of the step's outputs and are
 * overwritten with those of its inputs:
 * u = g_vel + drift g_pos; g_pos += (dF/dx)^T (kick u); g_vel = u. */
int pmgb_fpm_step_batched_vjp_f32(const pmgb_sim *sims, int n_sims,
                                  const float *pos, float *g_pos, float *g_vel,
                                  const float *kick, const float *drift,
                                  float r_split, void *workspace,
                                  size_t workspace_bytes, pmgb_stream_t stream);

/* ---- snapshots (np.save of fields, notebooks/05-MultiHost_PM.py:151-177) - */

typedef struct pmgb_snapshot pmgb_snapshot; /* opaque */

/* The NumPy .npy (format 1.0) header of a C-order array of dtype `descr`
 * (e.g. "<f4", "<c8", "<u4") and `shape`: writes it to buf when cap is
 * large enough and returns its length in bytes (a multiple of 64; 0 for
 * invalid arguments).  Host only. */
size_t pmgb_npy_header(const char *descr, const int64_t *shape, int ndim,
                       char *buf, size_t cap);

/* Starts writing the device array `array` (C order, `itemsize` bytes per
 * element, dtype `descr`) to the .npy file `path` and returns at once.  The
 * array's state is taken in stream order: with `staging` (device memory of
 * at least the array's bytes) by a device-to-device copy on `stream`, so the
 * caller may overwrite the array right away; with staging NULL the caller
 * must not modify the array until pmgb_snapshot_wait returns.  A host thread
 * then copies the data through pinned memory on its own stream and writes
 * the file.  Every started snapshot must be joined with pmgb_snapshot_wait. */
int pmgb_snapshot_begin_npy(const char *path, const void *array,
                            const char *descr, int itemsize,
                            const int64_t *shape, int ndim, void *staging,
                            size_t staging_bytes, pmgb_stream_t stream,
                            pmgb_snapshot **snapshot);

/* Waits for the snapshot's file to be complete, releases it and returns its
 * status (file or CUDA errors of the writer thread). */
int pmgb_snapshot_wait(pmgb_snapshot *snapshot);

#ifdef __cplusplus
}
#endif

#endif /* PMGB_H_ */
