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
} oracle_grid_t;

typedef struct {
  float bg, step, sigma_thresh, stop_thresh, near_clip;
  int spheric, last_opaque;
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

#define REAL double
#define SUFFIX _f64
#define FMA fma
#define SQRT sqrt
#define EXP exp
#define FMAX fmax
#define FMIN fmin
#define CEIL ceil
#define NEXTAFTER nextafter
#include "oracle_impl.h"

int oracle_abi_version(void) { return 1; }
