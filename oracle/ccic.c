/* Cloud-in-cell paint and read, restated in C with OpenMP threads.
 *
 * TEST INFRASTRUCTURE ONLY: the same arithmetic as ``oracle/cic.py``
 * (absolute mode, ``jaxpm/painting.py:15-45`` paint and ``:78-106`` read),
 * written in C so that the oracle can run the 256^3 and 512^3 workloads in
 * minutes instead of hours.  Only ``oracle/cic.py`` loads it; the tests
 * check it against the NumPy statement bit for bit (reads, weights) and to
 * float64 rounding (paint sums).
 *
 * Float order follows the reference: ``floor``, ``floor + offset`` in the
 * working dtype, ``k = 1 - |x - c|`` per axis, ``w = (k0*k1)*k2``; the
 * neighbour index is the int32 cast of ``floor + offset`` reduced
 * floor-modulo the mesh size (``painting.py:24-37``).  The read sums
 * ``v_j * w_j`` in neighbour order in the working dtype (``:104-106``);
 * the paint accumulates ``double(weight * w_j)`` (the NumPy oracle's
 * float64 ``bincount``) with atomic adds, so only the order of float64
 * additions differs.  Build with ``-ffp-contract=off`` so that no product
 * and sum fuse into one rounding.
 */
#include <math.h>
#include <stdint.h>

static const int CONN[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1},
                               {1, 1, 0}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};

static inline int64_t fmod_i32(int32_t a, int32_t n) {
  int32_t r = a % n;
  return (int64_t)(r < 0 ? r + n : r);
}

#define DEFINE_CIC(T, FLOOR, FABS, SUFFIX)                                          \
  static inline void weights_##SUFFIX(const T *p, int nx, int ny, int nz,           \
                                      int64_t idx[8], T w[8]) {                     \
    T f[3] = {FLOOR(p[0]), FLOOR(p[1]), FLOOR(p[2])};                               \
    const int32_t n[3] = {nx, ny, nz};                                               \
    for (int j = 0; j < 8; ++j) {                                                    \
      T k[3];                                                                        \
      int64_t c[3];                                                                  \
      for (int d = 0; d < 3; ++d) {                                                  \
        T nc = f[d] + (T)CONN[j][d];                                                 \
        k[d] = (T)1 - FABS(p[d] - nc);                                               \
        c[d] = fmod_i32((int32_t)nc, n[d]);                                          \
      }                                                                              \
      w[j] = (k[0] * k[1]) * k[2];                                                   \
      idx[j] = (c[0] * ny + c[1]) * nz + c[2];                                       \
    }                                                                                \
  }                                                                                  \
                                                                                     \
  void oc_read_##SUFFIX(const T *mesh, int nx, int ny, int nz, const T *pos,         \
                        int64_t np, T *out) {                                        \
    _Pragma("omp parallel for schedule(static)")                                     \
    for (int64_t i = 0; i < np; ++i) {                                               \
      int64_t idx[8];                                                                \
      T w[8];                                                                        \
      weights_##SUFFIX(pos + 3 * i, nx, ny, nz, idx, w);                             \
      T acc = mesh[idx[0]] * w[0];                                                   \
      for (int j = 1; j < 8; ++j) acc = acc + mesh[idx[j]] * w[j];                   \
      out[i] = acc;                                                                  \
    }                                                                                \
  }                                                                                  \
                                                                                     \
  void oc_paint_##SUFFIX(double *acc, int nx, int ny, int nz, const T *pos,          \
                         int64_t np, const T *weights, T weight) {                   \
    _Pragma("omp parallel for schedule(static)")                                     \
    for (int64_t i = 0; i < np; ++i) {                                               \
      int64_t idx[8];                                                                \
      T w[8];                                                                        \
      weights_##SUFFIX(pos + 3 * i, nx, ny, nz, idx, w);                             \
      T s = weights ? weights[i] : weight;                                           \
      for (int j = 0; j < 8; ++j) {                                                  \
        double v = (double)(s * w[j]);                                               \
        _Pragma("omp atomic")                                                        \
        acc[idx[j]] += v;                                                            \
      }                                                                              \
    }                                                                                \
  }                                                                                  \
                                                                                     \
  /* out[i] = sum_j mesh[idx_j] * grad W_j(pos_i): the position gradient of    \
     the interpolated field (d(1 - |u|)/du = -1 for u >= 0, +1 below, the    \
     rule JAX applies to abs; floor has a zero derivative) */                \
  void oc_grad_##SUFFIX(const T *mesh, int nx, int ny, int nz, const T *pos,         \
                        int64_t np, T *out) {                                        \
    _Pragma("omp parallel for schedule(static)")                                     \
    for (int64_t i = 0; i < np; ++i) {                                               \
      const T *p = pos + 3 * i;                                                      \
      T f[3] = {FLOOR(p[0]), FLOOR(p[1]), FLOOR(p[2])};                              \
      const int32_t n[3] = {nx, ny, nz};                                             \
      T g0 = 0, g1 = 0, g2 = 0;                                                      \
      for (int j = 0; j < 8; ++j) {                                                  \
        T k[3], dk[3];                                                               \
        int64_t c[3];                                                                \
        for (int d = 0; d < 3; ++d) {                                                \
          T nc = f[d] + (T)CONN[j][d];                                               \
          T u = p[d] - nc;                                                           \
          k[d] = (T)1 - FABS(u);                                                     \
          dk[d] = u >= 0 ? (T)-1 : (T)1;                                             \
          c[d] = fmod_i32((int32_t)nc, n[d]);                                        \
        }                                                                            \
        T m = mesh[(c[0] * ny + c[1]) * nz + c[2]];                                  \
        g0 += ((m * dk[0]) * k[1]) * k[2];                                           \
        g1 += ((m * k[0]) * dk[1]) * k[2];                                           \
        g2 += ((m * k[0]) * k[1]) * dk[2];                                           \
      }                                                                              \
      out[3 * i] = g0;                                                               \
      out[3 * i + 1] = g1;                                                           \
      out[3 * i + 2] = g2;                                                           \
    }                                                                                \
  }                                                                                  \
                                                                                     \
  void oc_weights_##SUFFIX(const T *pos, int64_t np, int nx, int ny, int nz,         \
                           int64_t *idx, T *w) {                                     \
    _Pragma("omp parallel for schedule(static)")                                     \
    for (int64_t i = 0; i < np; ++i)                                                 \
      weights_##SUFFIX(pos + 3 * i, nx, ny, nz, idx + 8 * i, w + 8 * i);             \
  }

DEFINE_CIC(float, floorf, fabsf, f32)
DEFINE_CIC(double, floor, fabs, f64)

#ifdef _OPENMP
#include <omp.h>
int oc_threads(void) { return omp_get_max_threads(); }
#else
int oc_threads(void) { return 1; }
#endif
