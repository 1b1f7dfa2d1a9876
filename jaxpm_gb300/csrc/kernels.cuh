// Internal host-side entry points shared between the translation units of
// libpmgb.  The exported C ABI (abi.cu) validates arguments and forwards here.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace pmgb {

// cic.cu
size_t paint_workspace_size(int nx, int ny, int nz, int64_t np, int mode);
int paint(float *mesh, int nx, int ny, int nz, const float *pos, int64_t np,
          const float *weights, float wscale, int mode, int accumulate,
          void *ws, size_t ws_bytes, cudaStream_t s);
int read(const float *mesh, int nx, int ny, int nz, const float *pos,
         int64_t np, float *out, cudaStream_t s);
int read3(const float *mesh3, int64_t cs, int nx, int ny, int nz,
          const float *pos, int64_t np, float *out, cudaStream_t s);
int cic_weights(const float *pos, int64_t np, int nx, int ny, int nz,
                int32_t *idx, float *w, cudaStream_t s);
int paint_vjp(const float *g_mesh, int nx, int ny, int nz, const float *pos,
              int64_t np, const float *weights, float wscale, float *g_pos,
              float *g_w, cudaStream_t s);
int read_vjp(const float *mesh, int nx, int ny, int nz, const float *pos,
             int64_t np, const float *g_out, float *g_mesh, float *g_pos,
             cudaStream_t s);
int paint_dx(float *mesh, int nx, int ny, int nz, const float *disp,
             const float *weights, float wscale, int accumulate,
             cudaStream_t s);
int read_dx(const float *mesh, int nx, int ny, int nz, const float *disp,
            float *out, cudaStream_t s);
int enmesh(const float *disp, int nx, int ny, int nz, int32_t *idx, float *w,
           cudaStream_t s);
int paint_fixed_into(unsigned long long *acc, float *mesh, int nx, int ny,
                     int nz, const float *pos, int64_t np,
                     const float *weights, float wscale, int accumulate,
                     cudaStream_t s);

// fft.cu
int fft_r2c(const float *in, void *out, int nx, int ny, int nz, int batch,
            cudaStream_t s);
int fft_c2r(void *in, float *out, int nx, int ny, int nz, int batch,
            cudaStream_t s);
int scale_inplace(float *x, int64_t n, float scale, cudaStream_t s);
// Creates (if needed) the cached 3-D plan of fft_r2c (r2c=1) or fft_c2r.
int fft_prepare(int nx, int ny, int nz, int batch, int r2c);
// batched 2-D (y, z) transforms of x-planes, spectra [plane][ny][pitch]
int fft_planes_r2c(const float *in, void *out, int nplanes, int ny, int nz,
                   int pitch, cudaStream_t s);
int fft_planes_c2r(void *in, float *out, int nplanes, int ny, int nz, int pitch,
                   cudaStream_t s);

// kspace.cu
int kspace_forces(const void *dk, void *fk, int64_t cs, int nx, int ny, int nz,
                  float r_split, int grad_order, int fd, float scale,
                  cudaStream_t s);
int kspace_forces_vjp(const void *gfk, int64_t cs, void *gdk, int nx, int ny,
                      int nz, float r_split, int grad_order, int fd,
                      float scale, cudaStream_t s);
int kspace_invlaplace(void *spec, int nx, int ny, int nz, int fd, float scale,
                      cudaStream_t s);
int kspace_longrange(void *spec, int nx, int ny, int nz, float r_split,
                     cudaStream_t s);
int kspace_gradient(const void *in, void *out, int nx, int ny, int nz, int dir,
                    int grad_order, cudaStream_t s);

// step.cu
size_t pm_workspace_size(int nx, int ny, int nz, int64_t np, int mode);
int pm_forces(const float *pos, int64_t np, int nx, int ny, int nz,
              float r_split, int mode, float *forces, void *ws, size_t bytes,
              cudaStream_t s);
int read3_kick_drift(const float *f3, int64_t cs, int nx, int ny, int nz,
                     float *pos, float *vel, int64_t np, float kick,
                     float drift, float *fout, cudaStream_t s);
int fpm_step(float *pos, float *vel, int64_t np, int nx, int ny, int nz,
             float kick, float drift, float r_split, int mode, void *ws,
             size_t bytes, cudaStream_t s);
int fpm_step_plain(float *pos, float *vel, int64_t np, int nx, int ny, int nz,
                   float kick, float drift, float r_split, void *ws,
                   size_t bytes, cudaStream_t s);
int kick(float *vel, const float *forces, int64_t np, float k, cudaStream_t s);
int drift(float *pos, const float *vel, int64_t np, float d, cudaStream_t s);
int pm_forces_vjp(const float *pos, int64_t np, int nx, int ny, int nz,
                  float r_split, int mode, const float *g, float *gpos,
                  void *ws, size_t bytes, cudaStream_t s);

// lpt.cu
int linear_field_colour(void *spec, int nx, int ny, int nz, float bx, float by,
                        float bz, const float *tk, const float *tp, int nt,
                        float scale, cudaStream_t s);
size_t lpt2_source_workspace_size(int nx, int ny, int nz);
// adjoint of R2C(ic) -> lpt2_source: g = delta2 cotangent -> g_ic (same workspace)
int lpt2_source_vjp(const float *ic, const float *g, float *g_ic, int nx, int ny, int nz, void *ws,
                    size_t bytes, cudaStream_t s);
int lpt2_source(const void *dk, float *delta2, int nx, int ny, int nz,
                void *ws, size_t bytes, cudaStream_t s);
int lpt_combine(const float *a, const float *b, int64_t n, float ca, float cb,
                float *out, cudaStream_t s);

// sorted.cu
int paint_box(float *mesh, int nx, int ny, int nz, const float *pos, int64_t np,
              const float *weights, float wscale, unsigned *stats, cudaStream_t s);
int64_t tile_key_count(int nx, int ny, int nz);
size_t sort_workspace_size(int nx, int ny, int nz, int64_t np);
// dest (nullable): dest[p] = the slot particle p went to.
int tile_sort(const float *pos, const float *vel, const unsigned *id, int64_t np,
              int nx, int ny, int nz, float *pos2, float *vel2, unsigned *id2,
              void *ws, size_t bytes, cudaStream_t s, unsigned *dest = nullptr);
int unpermute3(const float *in, const unsigned *id, int64_t np, float *out,
               cudaStream_t s);
int permute3(const float *in, const unsigned *id, int64_t np, float *out,
             cudaStream_t s);
// out[p] = in[idx[p]] for p < n, idx into an [n_in][3] array (entries >= n_in
// skipped).
int gather3(const float *in, int64_t n_in, const unsigned *idx, int64_t n,
            float *out, cudaStream_t s);
int paint_sorted(float *mesh, int nx, int ny, int nz, const float *pos,
                 int64_t np, void *sort_ws, size_t sort_bytes, unsigned *stats,
                 cudaStream_t s);
// the recording forward of the reverse sweep as one run (see sorted.cu)
int fpm_run_sorted_record(float *xs, float *vel_a, unsigned *id_a, float *vel_b, unsigned *id_b,
                          float *pos_out, int64_t np, int nx, int ny, int nz, int n_steps,
                          const float *kick, const float *drift, float r_split, void *mesh_ws,
                          size_t mesh_bytes, void *sort_ws, size_t sort_bytes, float *f3s,
                          unsigned *dests, unsigned *offs, unsigned *stats, cudaStream_t s,
                          bool pot = false);

// The gather's permuted mode (the run loop): particle slot p of the tile
// ranges is read from index perm[p] of (pos, vel) and written, with its new
// tile key, to slot p of (pos_out, vel_out, key_out), so the arrays never
// need moving between steps; only perm is re-sorted (and the ids follow in
// the re-sort).  perm == nullptr reads slot p itself (the arrays are in tile
// order).
struct PermIO {
  const unsigned *perm = nullptr;
  float *vel_out = nullptr;  // nullptr: the velocities are updated in place
  // nullptr: keys are not written; else np pairs (new tile key, rank among
  // the particles that stayed in their tile, ~0 for those that left)
  unsigned *key_out = nullptr;
  unsigned *stay_out = nullptr;  // with key_out: per tile, how many stayed
};

// Launch choices of the sorted loop that the autotuner sets (process-wide):
// the quarters of the tiles the gather deals statically (the rest from a
// counter), and the CTAs per SM of the gather and of the re-sort (0: as many
// as fit).
struct Tuning {
  int gather_static_quarters = 3;
  int gather_ctas_per_sm = 0;
  int resort_ctas_per_sm = 0;
  int resort_priority = 0;  // 0: the highest stream priority, 1: the default
};
Tuning tuning();
void set_tuning(const Tuning &t);

int rkd_sorted(const float *f3, int64_t cs, int nx, int ny, int nz,
               const float *pos, float *pos_out, float *vel, int64_t np,
               float kick, float drift, void *sort_ws, size_t sort_bytes,
               unsigned *stats, cudaStream_t s, float *mesh_next = nullptr,
               bool pot = false, const PermIO &io = PermIO());
// n_steps sorted steps with the paint of each next density fused into the
// gather; the state ping-pongs between the a and b buffers (in a after an
// even number of steps).  kick/drift: host arrays of n_steps.
// launch timing of fpm_run_sorted (off by default): per-launch mean
// milliseconds of the last timed run's gathers, force evaluations and
// re-sorts
int set_run_timing(bool on);
int run_timing(double *gather_ms, double *forces_ms, double *resort_ms, int *steps);
int fpm_run_sorted(float *pos_a, float *vel_a, unsigned *id_a, float *pos_b,
                   float *vel_b, unsigned *id_b, int64_t np, int nx, int ny,
                   int nz, int n_steps, const float *kick, const float *drift,
                   float r_split, void *mesh_ws, size_t mesh_bytes,
                   void *sort_ws, size_t sort_bytes, unsigned *stats,
                   cudaStream_t s);
// step.cu: density mesh -> force meshes inside the composite workspace's
// spectra (dk, fk) by the selected FFT path.
int mesh_forces(const float *mesh, int nx, int ny, int nz, float r_split,
                void *dk, void *fk, float *f3, cudaStream_t s);
// the permuted gather's outputs in the sort workspace (keys, stayer ranks,
// stayer counts)
void perm_scratch(void *sort_ws, int nx, int ny, int nz, int64_t np, PermIO *io);
int check_sort_workspace(void *ws, size_t bytes, int nx, int ny, int nz, int64_t np);
// scan of the tile counts, then perm from the keys in the rank array (the
// permuted run loop's re-sort)
// (perm_new[d] = p for the slot d particle p claims); with perm_old, also
// id_out[p] = id_in[perm_old[p]] (the ids follow the permuted gather)
int index_resort(int64_t np, int nx, int ny, int nz, const unsigned *perm_old,
                 unsigned *perm_new, const unsigned *id_in, unsigned *id_out, void *sort_ws,
                 size_t sort_bytes, cudaStream_t s);
// out[p] = in[idx[p]] for np 32-bit words
int gather_u32(const unsigned *in, const unsigned *idx, int64_t np, unsigned *out,
               cudaStream_t s);
int tile_scatter(const float *pos, const float *vel, const unsigned *id,
                 int64_t np, int nx, int ny, int nz, float *pos2, float *vel2,
                 unsigned *id2, unsigned *dest, void *sort_ws, size_t sort_bytes,
                 cudaStream_t s);
const unsigned *tile_offsets(void *sort_ws, int nx, int ny, int nz, int64_t np);
int fpm_step_sorted(const float *pos, float *vel, const unsigned *id, float *pos2,
                    float *vel2, unsigned *id2, int64_t np, int nx, int ny,
                    int nz, float kick, float drift, float r_split,
                    void *mesh_ws, size_t mesh_bytes, void *sort_ws,
                    size_t sort_bytes, float *force3_out, unsigned *dest_out,
                    unsigned *offsets_out, unsigned *stats, cudaStream_t s);
int fpm_step_sorted_vjp(const float *pos, const float *force3,
                        const unsigned *dest, const unsigned *offsets,
                        const float *gx_in, const float *gv_in, float *gx_out,
                        float *gv_out, int64_t np, int nx, int ny, int nz,
                        float kick, float drift, float r_split, void *mesh_ws,
                        size_t mesh_bytes, unsigned *stats, cudaStream_t s,
                        bool pot = false);
// The cotangents of one sorted step's coefficients, added to out[0..1]:
// out[0] += <g_vel, F(pos)> (F read from force3 at pos, order i), out[1] +=
// <g_pos_next[dest], pos_next[dest] - pos> (order i+1 pulled to order i).
int coef_cotangents(const float *pos, const float *pos_next, const unsigned *dest,
                    const float *force3, int64_t cs, int nx, int ny, int nz,
                    const float *g_pos_next, const float *g_vel, int64_t np, double *out,
                    cudaStream_t s);
// step.cu: paint of tile-sorted particles -> R2C -> k-space -> C2R inside the
// composite workspace; *f3 receives the three force meshes (f3_out when it
// is given, else the workspace's region).
int force_meshes_sorted(const float *pos, int64_t np, int nx, int ny, int nz,
                        float r_split, void *ws, size_t bytes, void *sort_ws,
                        size_t sort_bytes, unsigned *stats, float *f3_out,
                        float **f3, cudaStream_t s);
// step.cu: density mesh -> the three force meshes (the spectral part of
// pm_forces), with caller workspace (mesh_forces_workspace_size).
size_t mesh_forces_workspace_size(int nx, int ny, int nz);
int mesh_forces_ws(const float *mesh, float *f3, int nx, int ny, int nz,
                   float r_split, void *ws, size_t bytes, cudaStream_t s);
// density mesh -> the potential mesh of the run loop (spectral pipeline only)
int mesh_potential_ws(const float *mesh, float *pot, int nx, int ny, int nz, float r_split,
                      void *ws, size_t bytes, cudaStream_t s);
int mesh_forces_vjp_ws(const float *g3, float *rbar, int nx, int ny, int nz,
                       float r_split, void *ws, size_t bytes, cudaStream_t s);
// step.cu: the three force-mesh cotangents g3 -> the density cotangent
// rbar (spectral pipeline or cuFFT; dk/fk are the workspace's spectra).
int mesh_forces_vjp(const float *g3, int nx, int ny, int nz, float r_split,
                    void *dk, void *fk, float *rbar, cudaStream_t s);
// step.cu: the composite workspace's [np][3] particle scratch (nullptr and
// an error left when the workspace is too small).
float *pm_workspace_particles(void *ws, size_t bytes, int nx, int ny, int nz,
                              int64_t np);
// step.cu: the composite workspace's regions used by the sorted adjoint.
int pm_workspace_regions(void *ws, size_t bytes, int nx, int ny, int nz,
                         int64_t np, float **mesh, void **dk, void **fk,
                         float **f3, float **g3, unsigned **work);

// spectral.cu: hand-written three-pass FFT pipeline for power-of-two
// meshes (nx in [8,1024], ny in [64,512], nz in [16,512]).  Spectra use the
// layout [nx][ny][spectral_pitch(nz)] complex (kz < nz/2+1 meaningful).
bool spectral_supported(int nx, int ny, int nz);
// Process-wide choice of the composite calls' FFT path (the pmgb_fft_path
// values): 0 cuFFT 3-D, 1 cuFFT planes + fused x pass, 2 own planes + fused
// x pass (1 and 2 only where spectral_supported).  Returns the previous.
bool spectral_enabled();
int spectral_mode();
int set_spectral(int mode);
int spectral_pitch(int nz);
int spectral_r2c(const float *in, void *out, int nx, int ny, int nz, int batch,
                 cudaStream_t s);
int spectral_c2r(void *in, float *out, int nx, int ny, int nz, int batch,
                 cudaStream_t s);
// mesh -> spec (density spectrum, plane-transformed) -> fspec (3 components)
// -> f3 [3][nx][ny][nz]: the force meshes of kspace_forces + C2R.
int spectral_forces(const float *mesh, void *spec, void *fspec, float *f3,
                    int nx, int ny, int nz, float r_split, int order, int fd,
                    float scale, cudaStream_t s);
// The order-1 gradient as a real-space stencil over `batch` meshes:
// f3 [b][3][nx][ny][nz] = -D pot [b][nx][ny][nz], and its transpose
// out [b] = sum_c D_c g3 [b][c].
int stencil_forces(const float *pot, float *f3, int nx, int ny, int nz, int batch,
                   cudaStream_t s);
int stencil_adjoint(const float *g3, float *out, int nx, int ny, int nz, int batch,
                    cudaStream_t s);
// mesh -> spec -> pot [nx][ny][nz]: the potential whose order-1 stencil
// gradient gives the forces of spectral_forces (order 1, fd 0).
int spectral_potential(const float *mesh, void *spec, float *pot, int nx, int ny, int nz,
                       float r_split, float scale, cudaStream_t s);
// g3 [3][nx][ny][nz] -> spec3 -> dspec -> rbar: the adjoint of the above.
int spectral_forces_vjp(const float *g3, void *spec3, void *dspec, float *rbar,
                        int nx, int ny, int nz, float r_split, int order,
                        int fd, float scale, cudaStream_t s);

// pk.cu
int power_spectrum(const void *spec, int nx, int ny, int nz, double bx,
                   double by, double bz, const double *edges, int n_edges,
                   double *psum, double *pcount, double *ksum, cudaStream_t s);

// batched.cu
size_t batch_workspace_size(const pmgb_sim *t, int n);
int batch_init(const pmgb_sim *t, int n, void *ws, size_t bytes, cudaStream_t s);
int batch_release(const void *ws);
int batch_counts(const pmgb_sim *t, int n, int64_t *np_total, int64_t *cells_total);
int cic_paint_batched(const pmgb_sim *t, int n, float *meshes, const float *pos, void *ws,
                      size_t bytes, cudaStream_t s);
int pm_forces_batched(const pmgb_sim *t, int n, const float *pos, float *forces, float r_split,
                      void *ws, size_t bytes, cudaStream_t s);
int fpm_step_batched(const pmgb_sim *t, int n, float *pos, float *vel, const float *kick,
                     const float *drift, float r_split, float *pos_before, void *ws,
                     size_t bytes, cudaStream_t s);
int fpm_step_batched_vjp(const pmgb_sim *t, int n, const float *pos, float *gpos, float *gvel,
                         const float *kick, const float *drift, float r_split, void *ws,
                         size_t bytes, cudaStream_t s);

// snapshot.cu
struct Snapshot;
size_t npy_header(const char *descr, const int64_t *shape, int ndim, char *buf, size_t cap);
int snapshot_begin_npy(const char *path, const void *dev, const char *descr, int itemsize,
                       const int64_t *shape, int ndim, void *staging, size_t staging_bytes,
                       cudaStream_t s, Snapshot **out);
int snapshot_wait(Snapshot *snap);

}  // namespace pmgb
