/*
 * ORACLE — test infrastructure only (see oracle_impl.h).  Instantiates the CPU
 * restatement in float (_f32) and double (_f64).  Build: oracle/build.py
 * (gcc -O2 -ffp-contract=off -fopenmp -shared).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

/* Grid, options and camera, shared by both instantiations. */
typedef struct {
  const int32_t* links; /* [X,Y,Z] */
  const float* density; /* [N] */
  const float* sh;      /* [N, 3*basis_dim] */
  int64_t n_voxels;
  int size[3];
  int basis_dim;
  float offset[3], scaling[3];
  /* MSI background (bg_nlayers == 0: none): links [2*reso, reso], data [capacity, nlayers, 4] */
  const int32_t* bg_links;
  const float* bg_data;
  int bg_reso, bg_nlayers;
} oracle_grid_t;

typedef struct {
  float bg, step, sigma_thresh, stop_thresh, near_clip;
  int spheric, last_opaque;
  int bg_cpu; /* background semantics: 0 the CUDA kernels', 1 the pure-PyTorch path's */
} oracle_opt_t;

typedef struct {
  const float* c2w; /* row-major, 4 columns */
  float fx, fy, cx, cy;
  int width, height;
  float ndcx, ndcy;
} oracle_cam_t;

#define REAL float
#define SUFFIX _f32
#define FMA fmaf
#define SQRT sqrtf
#define EXP expf
#define FMAX fmaxf
#define FMIN fminf
#define CEIL ceilf
#define NEXTAFTER nextafterf
#define ASIN asinf
#define ATAN2 atan2f
#define FABS fabsf
#define OMX(y) (1.f - expf(y))
#include "oracle_impl.h"
#undef REAL
#undef SUFFIX
#undef FMA
#undef SQRT
#undef EXP
#undef FMAX
#undef FMIN
#undef CEIL
#undef NEXTAFTER
#undef ASIN
#undef ATAN2
#undef FABS
#undef OMX

#define REAL double
#define SUFFIX _f64
#define FMA fma
#define SQRT sqrt
#define EXP exp
#define FMAX fmax
#define FMIN fmin
#define CEIL ceil
#define NEXTAFTER nextafter
#define ASIN asin
#define ATAN2 atan2
#define FABS fabs
#define OMX(y) (-expm1(y))
#include "oracle_impl.h"

/* accel_dist_prop, svox2/csrc/misc_kernel.cu:108-181 (kernels) and 356-416 (host):
 * restated as the reference computes it.  Pass 1 (accel_dist_set_kernel): every voxel
 * with link >= 0 marks its ancestor at each level of a pyramid that halves the sides
 * (rounding up) while all sides are > 1.  Pass 2 (accel_dist_prop_kernel): every voxel
 * with link < 0 becomes -1 minus the number of unmarked ancestors met going up before
 * the first marked one.  Integer work: the result is exact. */
void oracle_accel_dist_prop(int32_t* links, const int size[3]) {
  int64_t req = 0, sx = size[0], sy = size[1], sz = size[2], v, n = (int64_t)size[0] * size[1] * size[2];
  uint8_t* tmp;
  while (sx > 1 && sy > 1 && sz > 1) {
    sx = (sx + 1) / 2;
    sy = (sy + 1) / 2;
    sz = (sz + 1) / 2;
    req += sx * sy * sz;
  }
  tmp = (uint8_t*)calloc(req > 0 ? (size_t)req : 1, 1);
  for (v = 0; v < n; ++v) {
    int64_t x = v / ((int64_t)size[1] * size[2]), y = (v / size[2]) % size[1], z = v % size[2];
    int64_t ax = size[0], ay = size[1], az = size[2];
    uint8_t* base = tmp;
    if (links[v] < 0) continue;
    while (ax > 1 && ay > 1 && az > 1) {
      x >>= 1;
      y >>= 1;
      z >>= 1;
      ax = (ax + 1) / 2;
      ay = (ay + 1) / 2;
      az = (az + 1) / 2;
      base[x * ay * az + y * az + z] = 1;
      base += ax * ay * az;
    }
  }
  for (v = 0; v < n; ++v) {
    int64_t x = v / ((int64_t)size[1] * size[2]), y = (v / size[2]) % size[1], z = v % size[2];
    int64_t ax = size[0], ay = size[1], az = size[2];
    const uint8_t* base = tmp;
    int32_t result = -1;
    if (links[v] >= 0) continue;
    while (ax > 1 && ay > 1 && az > 1) {
      x >>= 1;
      y >>= 1;
      z >>= 1;
      ax = (ax + 1) / 2;
      ay = (ay + 1) / 2;
      az = (az + 1) / 2;
      if (base[x * ay * az + y * az + z]) break;
      result -= 1;
      base += ax * ay * az;
    }
    links[v] = result;
  }
  free(tmp);
}

int oracle_abi_version(void) { return 1; }
