/*
 * CPU restatement of the reference renderer's hot path — TEST INFRASTRUCTURE.
 *
 * This file is the ORACLE: it is only compiled into oracle/liboracle.so and is
 * only used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline and
 * reference arms, to check or to time against.  Nothing in the svox2_gb300
 * product links or calls it.
 *
 * It is included twice by svox2_oracle.c, with REAL = float (suffix _f32) and
 * REAL = double (suffix _f64).  The float instance performs the reference
 * kernels' IEEE operations in the reference's order (fmaf where the reference
 * calls fmaf, no other contraction: it is built with -ffp-contract=off); the
 * double instance is the same algorithm in double precision, the yardstick
 * for every error statement.  Each function names the reference code it
 * restates (paths inside the reference project).
 *
 * Sampling geometry is float in both instances: the ray's grid-space origin,
 * direction and world step, its bounds, every sample's t, cell and position
 * in the cell, and the skip distances.  Those decide WHICH samples are taken
 * (links-level parity is bit-exact by requirement), so the double instance
 * takes exactly the float instance's samples and evaluates every value along
 * them (densities, colours, weights, transmittance, gradients) in double.
 * Its per-entry errors then measure the arithmetic alone.  The one value test
 * that decides the sample set, the early stop, can be handed to it from a
 * float run (oracle_render's stop_in), so that it also stops where the float
 * run stopped.
 *
 * A sample's opacity 1 - exp(-x) is OMX(-x): the float instance subtracts, as
 * the reference does (for x below 2^-24 that is exactly 0), the double
 * instance uses -expm1(-x), the same quantity without the cancellation, so the
 * yardstick is exact to double precision for the thin media where the
 * subtraction is not.
 *
 * Two places where the reference's device code calls approximate hardware
 * functions are restated from their mathematical definition:
 *   - rnorm3df (svox2/csrc/include/cuda_util.cuh:87-92) -> 1/sqrt formed in double;
 *   - the stop test __expf(logT) < stop_thresh (render_lerp_kernel_cuvol.cu:103,
 *     370) -> logT < L with L the smallest REAL >= ln(stop_thresh), which is the
 *     same predicate in exact arithmetic.
 */

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define FN(name) CAT(name, SUFFIX)

/* sampling geometry of a ray: float in both instances (see above) */
typedef struct {
  float o[3], d[3];
  float world_step, tmin, tmax;
} FN(ray_t);

static REAL FN(lerp)(REAL a, REAL b, REAL w) { return FMA(w, b - a, a); }

static REAL FN(log_stop)(float stop) {
  if (!(stop > 0.f)) return (REAL)(-INFINITY);
  double L = log((double)stop);
  REAL f = (REAL)L;
  if ((double)f < L) f = NEXTAFTER(f, (REAL)INFINITY);
  while ((double)NEXTAFTER(f, (REAL)(-INFINITY)) >= L) f = NEXTAFTER(f, (REAL)(-INFINITY));
  return f;
}

/* calc_sh, svox2/csrc/include/render_util.cuh:332-363 (degree <= 2). */
static void FN(calc_sh)(int bd, const REAL dir[3], REAL out[9]) {
  const REAL C0 = (REAL)0.28209479177387814f, C1 = (REAL)0.4886025119029199f;
  const REAL C20 = (REAL)1.0925484305920792f, C21 = (REAL)-1.0925484305920792f,
             C22 = (REAL)0.31539156525252005f, C23 = (REAL)-1.0925484305920792f,
             C24 = (REAL)0.5462742152960396f;
  REAL x = dir[0], y = dir[1], z = dir[2];
  out[0] = C0;
  if (bd >= 4) {
    out[1] = -C1 * y;
    out[2] = C1 * z;
    out[3] = -C1 * x;
  }
  if (bd >= 9) {
    REAL xx = x * x, yy = y * y, zz = z * z, xy = x * y, yz = y * z, xz = x * z;
    out[4] = C20 * xy;
    out[5] = C21 * yz;
    out[6] = (REAL)((double)C22 * (2.0 * (double)zz - (double)xx - (double)yy));
    out[7] = C23 * xz;
    out[8] = C24 * (xx - yy);
  }
}

static REAL FN(rnorm3)(REAL x, REAL y, REAL z) {
  double s = (double)x * (double)x + (double)y * (double)y + (double)z * (double)z;
  return (REAL)(1.0 / sqrt(s));
}

static REAL FN(recip)(REAL d) { return (REAL)(1.0 / (double)d); }

/* float forms of the two above, for the sampling geometry */
static float FN(rnorm3g)(float x, float y, float z) {
  double s = (double)x * (double)x + (double)y * (double)y + (double)z * (double)z;
  return (float)(1.0 / sqrt(s));
}

static float FN(recipg)(float d) { return (float)(1.0 / (double)d); }

/* ConcentricSpheresIntersector, render_util.cuh:546-576, in float (the spheric clip). */
static int FN(sphere_hitg)(const float o[3], const float d[3], float r, float* out, int near) {
  float dd = (d[0] * d[0] + d[1] * d[1]) + d[2] * d[2];
  float od = (o[0] * d[0] + o[1] * d[1]) + o[2] * d[2];
  float oo = (o[0] * o[0] + o[1] * o[1]) + o[2] * o[2];
  float q2a = 2 * dd, qb = 2 * od;
  float f = qb * qb - (2 * q2a) * oo;
  float det = f + ((2 * q2a) * r) * r;
  if (det < 0) return 0;
  float sq = sqrtf(det);
  *out = near ? (-qb - sq) / q2a : (-qb + sq) / q2a;
  return 1;
}

/* ConcentricSpheresIntersector, render_util.cuh:546-576. */
static int FN(sphere_hit)(const REAL o[3], const REAL d[3], REAL r, REAL* out, int near) {
  REAL dd = (d[0] * d[0] + d[1] * d[1]) + d[2] * d[2];
  REAL od = (o[0] * d[0] + o[1] * d[1]) + o[2] * d[2];
  REAL oo = (o[0] * o[0] + o[1] * o[1]) + o[2] * o[2];
  REAL q2a = 2 * dd, qb = 2 * od;
  REAL f = qb * qb - (2 * q2a) * oo;
  REAL det = f + ((2 * q2a) * r) * r;
  if (det < 0) return 0;
  REAL sq = SQRT(det);
  *out = near ? (-qb - sq) / q2a : (-qb + sq) / q2a;
  return 1;
}

/* ray_find_bounds, render_util.cuh:578-628 (+ transform_coord, _get_delta_scale). */
static void FN(find_bounds)(FN(ray_t) * r, const float org[3], const float dir[3], const oracle_grid_t* g,
                            const oracle_opt_t* opt) {
  int i;
  for (i = 0; i < 3; ++i) {
    r->o[i] = fmaf(org[i], g->scaling[i], g->offset[i]);
    r->d[i] = dir[i] * g->scaling[i];
  }
  float ds = FN(rnorm3g)(r->d[0], r->d[1], r->d[2]);
  for (i = 0; i < 3; ++i) r->d[i] = r->d[i] * ds;
  r->world_step = ds * opt->step;
  if (opt->spheric) {
    float so[3], sd[3];
    for (i = 0; i < 3; ++i) {
      float s = 2.f / (float)g->size[i];
      so[i] = fmaf(r->o[i] + 0.5f, s, -1.f);
      sd[i] = r->d[i] * s;
    }
    if (!FN(sphere_hitg)(so, sd, 1.f, &r->tmax, 0) || !FN(sphere_hitg)(so, sd, 1.f - opt->near_clip, &r->tmin, 1)) {
      r->tmin = 1e-9f;
      r->tmax = 0;
    }
  } else {
    r->tmin = opt->near_clip / r->world_step * opt->step;
    r->tmax = 2e3f;
    for (i = 0; i < 3; ++i) {
      float inv = FN(recipg)(r->d[i]);
      float t1 = (-0.5f - r->o[i]) * inv;
      float t2 = (((float)g->size[i] - 0.5f) - r->o[i]) * inv;
      if (r->d[i] != 0) {
        r->tmin = fmaxf(r->tmin, fminf(t1, t2));
        r->tmax = fminf(r->tmax, fmaxf(t1, t2));
      }
    }
  }
}

/* compute_skip_dist, render_util.cuh:235-295 (pos_offset = 0). */
static float FN(skip_dist)(int32_t link, const int l[3], const float pos[3], const float d[3]) {
  uint32_t dist = (uint32_t)(-link), shift = dist - 1u;
  uint32_t side = (uint32_t)((float)(1u << shift) - 1.f);
  float tmin = 0, tmax = 1e9f;
  int i;
  for (i = 0; i < 3; ++i) {
    int ul = ((l[i] >> shift) << shift) - l[i];
    float inv = FN(recipg)(d[i]);
    float t1 = ((float)ul - pos[i]) * inv;
    float t2 = ((float)((uint32_t)ul + side) - pos[i]) * inv;
    if (d[i] != 0) {
      tmin = fmaxf(tmin, fminf(t1, t2));
      tmax = fminf(tmax, fmaxf(t1, t2));
    }
  }
  return tmin > 0 ? 0 : tmax;
}

/* cam2world_ray + world2ndc, render_util.cuh:504-544.  c2w row-major, 4 columns. */
static void FN(camera_ray)(int ix, int iy, const oracle_cam_t* cam, float dir[3], float org[3]) {
  float x = (((float)ix + 0.5f) - cam->cx) / cam->fx;
  float y = (((float)iy + 0.5f) - cam->cy) / cam->fy;
  float z = sqrtf((float)((double)(x * x + y * y) + 1.0));
  int r, i;
  x = x / z;
  y = y / z;
  z = 1.f / z;
  for (r = 0; r < 3; ++r) {
    dir[r] = (cam->c2w[4 * r] * x + cam->c2w[4 * r + 1] * y) + cam->c2w[4 * r + 2] * z;
    org[r] = cam->c2w[4 * r + 3];
  }
  if (cam->ndcx > 0.f) {
    float t = (1.f - org[2]) / dir[2];
    for (i = 0; i < 3; ++i) org[i] = fmaf(t, dir[i], org[i]);
    dir[0] = cam->ndcx * (dir[0] / dir[2] - org[0] / org[2]);
    dir[1] = cam->ndcy * (dir[1] / dir[2] - org[1] / org[2]);
    dir[2] = 2.f / org[2];
    org[0] = cam->ndcx * (org[0] / org[2]);
    org[1] = cam->ndcy * (org[1] / org[2]);
    org[2] = 1.f - 2.f / org[2];
    float rn = FN(rnorm3g)(dir[0], dir[1], dir[2]);
    for (i = 0; i < 3; ++i) dir[i] = dir[i] * rn;
  }
}

static void FN(atomic_add)(REAL* p, REAL v) {
#pragma omp atomic
  *p += v;
}

/* Per-sample state of the march, shared by the forward and backward loops (geometry: float). */
typedef struct {
  float pos[3];
  int l[3];
  const int32_t* lp;
  int64_t base;
} FN(sample_t);

static void FN(locate)(const oracle_grid_t* g, const FN(ray_t) * r, float t, FN(sample_t) * s) {
  const int64_t offy = g->size[2], offx = (int64_t)g->size[1] * g->size[2];
  int j;
  for (j = 0; j < 3; ++j) {
    float p = fmaf(t, r->d[j], r->o[j]);
    p = fminf(fmaxf(p, 0.f), (float)g->size[j] - 1.f);
    s->l[j] = (int)p;
    if (s->l[j] > g->size[j] - 2) s->l[j] = g->size[j] - 2;
    s->pos[j] = p - (float)s->l[j];
  }
  s->base = (int64_t)s->l[0] * offx + (int64_t)s->l[1] * offy + s->l[2];
  s->lp = g->links + s->base;
}

/* trilerp_cuvol_one, render_util.cuh:71-91: z, then y, then x. */
static REAL FN(trilerp)(const oracle_grid_t* g, const FN(sample_t) * s, const float* data, int stride, int idx) {
  const int64_t offy = g->size[2], offx = (int64_t)g->size[1] * g->size[2];
  const int64_t co[8] = {0, 1, offy, offy + 1, offx, offx + 1, offx + offy, offx + offy + 1};
  REAL v[8];
  int j;
  for (j = 0; j < 8; ++j) {
    int32_t lk = s->lp[co[j]];
    v[j] = lk >= 0 ? (REAL)data[(int64_t)lk * stride + idx] : 0;
  }
  const REAL p0 = (REAL)s->pos[0], p1 = (REAL)s->pos[1], p2 = (REAL)s->pos[2];
  REAL ix0 = FN(lerp)(FN(lerp)(v[0], v[1], p2), FN(lerp)(v[2], v[3], p2), p1);
  REAL ix1 = FN(lerp)(FN(lerp)(v[4], v[5], p2), FN(lerp)(v[6], v[7], p2), p1);
  return FN(lerp)(ix0, ix1, p0);
}

/* Largest |value| of channel idx over the 8 corners of the sample's cell: the scale of the
 * absolute rounding error of its trilinear interpolation. */
static REAL FN(corner_max)(const oracle_grid_t* g, const FN(sample_t) * s, const float* data, int stride, int idx) {
  const int64_t offy = g->size[2], offx = (int64_t)g->size[1] * g->size[2];
  const int64_t co[8] = {0, 1, offy, offy + 1, offx, offx + 1, offx + offy, offx + offy + 1};
  REAL m = 0;
  int j;
  for (j = 0; j < 8; ++j) {
    int32_t lk = s->lp[co[j]];
    if (lk >= 0) m = FMAX(m, FABS((REAL)data[(int64_t)lk * stride + idx]));
  }
  return m;
}

/* Colour sum per channel group, before the +0.5 offset. */
static void FN(sample_colour)(const oracle_grid_t* g, const FN(sample_t) * s, const REAL basis[9], REAL col[3]) {
  const int bd = g->basis_dim, C = 3 * bd;
  int c;
  col[0] = col[1] = col[2] = 0;
  for (c = 0; c < C; ++c) col[c / bd] += FN(trilerp)(g, s, g->sh, C, c) * basis[c % bd];
}

/* Early stop of a ray: stop_in < -1 takes the ray's own test (log T below the
 * threshold's log); stop_in == -1 never stops; stop_in = n >= 1 stops right after the
 * ray's n-th evaluated sample.  The last two replay a float run's stops (reported
 * through stop_out) in the double instance. */
static int FN(stops)(int stop_in, REAL lt, REAL log_stop, int n_done) {
  if (stop_in < -1) return lt < log_stop;
  return stop_in >= 0 && n_done >= stop_in;
}

/* trace_ray_cuvol, render_lerp_kernel_cuvol.cu:30-120.  Returns the colour and
 * the log transmittance the reference reports (-1e3 after an early stop).
 * *stop_out: the ray's evaluated-sample count at its early stop, or -1. */
static void FN(fwd_ray)(const oracle_grid_t* g, const oracle_opt_t* opt, const float org[3], const float dir[3],
                        REAL out[3], REAL* log_t, uint64_t* trace, uint64_t* n_eval, int stop_in, int* stop_out,
                        REAL* chain_out) {
  const REAL log_stop = FN(log_stop)(opt->stop_thresh);
  const float step = opt->step;
  REAL basis[9], dr[3] = {dir[0], dir[1], dir[2]}, outv[3] = {0, 0, 0}, lt = 0;
  float t, ws;
  FN(ray_t) r;
  uint64_t h = 1469598103934665603ull;
  int c, ne = 0;
  REAL chain = 1;
  if (stop_out) *stop_out = -1;
  if (chain_out) *chain_out = 1;
  FN(calc_sh)(g->basis_dim, dr, basis);
  FN(find_bounds)(&r, org, dir, g, opt);
  if (r.tmin > r.tmax) {
    for (c = 0; c < 3; ++c) out[c] = g->bg_nlayers == 0 ? (REAL)opt->bg : (REAL)0;
    *log_t = 0;
    if (trace) *trace = h;
    return;
  }
  t = r.tmin;
  ws = r.world_step;
  while (t <= r.tmax) {
    FN(sample_t) s;
    FN(locate)(g, &r, t, &s);
    if (s.lp[0] < -1) {
      float skip = FN(skip_dist)(s.lp[0], s.l, s.pos, r.d);
      if (skip >= step) {
        h = ((h ^ (uint64_t)s.base) * 1099511628211ull ^ 3ull) * 1099511628211ull;
        t = t + ceilf(skip / step) * step;
        continue;
      }
    }
    REAL sigma = FN(trilerp)(g, &s, g->density, 1, 0);
    if (opt->last_opaque && t + step > r.tmax) ws = 1e9f;
    const int ev = sigma > (REAL)opt->sigma_thresh;
    h = (h ^ (uint64_t)s.base) * 1099511628211ull;
    h = (h ^ (ev ? 1ull : 2ull)) * 1099511628211ull;
    if (ev) {
      REAL col[3];
      FN(sample_colour)(g, &s, basis, col);
      const REAL pcnt = (REAL)ws * sigma;
      const REAL w = EXP(lt) * OMX(-pcnt);
      lt = lt - pcnt;
      chain += FABS(lt);
      ++*n_eval;
      ++ne;
      for (c = 0; c < 3; ++c) outv[c] = outv[c] + w * FMAX(col[c] + (REAL)0.5, (REAL)0);
      if (FN(stops)(stop_in, lt, log_stop, ne)) {
        lt = (REAL)-1e3f;
        if (stop_out) *stop_out = ne;
        break;
      }
    }
    t = t + step;
  }
  /* with an MSI background the brightness term is added after it (cuvol.cu:111-113, 474) */
  for (c = 0; c < 3; ++c) out[c] = g->bg_nlayers == 0 ? outv[c] + EXP(lt) * (REAL)opt->bg : outv[c];
  *log_t = lt;
  if (trace) *trace = h;
  if (chain_out) *chain_out = chain;
}

/* trace_ray_cuvol_backward, render_lerp_kernel_cuvol.cu:227-383, forward order:
 * accum starts at dot(colour, gout) and loses each sample's contribution.  Reports the
 * accum left after the last sample (beta term taken out) and the log transmittance there,
 * which the MSI background's backward starts from (cuvol.cu:253-258, 374-383).
 * mag_density / mag_sh (optional) receive, per gradient entry, the scale against which
 * float arithmetic loses precision: the sum over its terms of |term| * F.  F = 1 + sum of
 * |log T| over the ray's samples so far bounds, in units of the float rounding unit, the
 * rounding error that the float chain of log T subtractions has built up by then: every
 * later weight and transmittance inherits it as a relative error.  The density term counts
 * its two parts separately: |tc T_after| * F, and the light behind the sample, bounded by
 * the ray's total light A = sum_c |gout_c colour_c| + |beta term|, with F + nmax (a sum of
 * up to nmax terms, the ray's most samples, in any order).  An SH term basis_k * X counts
 * |X| (Fw |basis_k| + e_k), with Fw = F + 4 max|corner density| / sigma: the float
 * trilinear interpolation lerp(a, b, w) = a + w (b - a) errs by a few rounding units of its
 * corner values, which is large against a small sigma (a sample just inside a face whose far
 * corners are empty), and the sample's weight inherits it; gerr_c (from oracle_render: the
 * relative error, in rounding units, of a float run's loss residual out - gt, large where the
 * colour nearly matches its target) multiplies every term of channel c; the float basis of k = 6 (C * (2 zz - xx - yy)) and k = 8
 * (C * (xx - yy)) is a difference of float squares of a unit direction, whose absolute
 * error is e_k = 2 |C| rounding units however small the difference; the other basis
 * functions are products, relative to their value.  An SH term whose colour channel sits on
 * the clamp (|colour + 0.5| <= 1e-5, within float reach of the kink) may be in or out of the
 * float sum: it counts 2^24 times, i.e. its whole size. */
static void FN(bwd_ray)(const oracle_grid_t* g, const oracle_opt_t* opt, const float org[3], const float dir[3],
                        const REAL color[3], REAL log_t_in, const REAL gout[3], REAL beta_loss, REAL sparsity,
                        REAL* grad_density, REAL* grad_sh, uint8_t* mask, REAL* accum_out, REAL* log_t_out,
                        int stop_in, REAL* mag_density, REAL* mag_sh, const REAL gerr[3]) {
  const int bd = g->basis_dim, C = 3 * bd;
  const int64_t offy = g->size[2], offx = (int64_t)g->size[1] * g->size[2];
  const int64_t co[8] = {0, 1, offy, offy + 1, offx, offx + 1, offx + offy, offx + offy + 1};
  const REAL log_stop = FN(log_stop)(opt->stop_thresh);
  const float step = opt->step;
  REAL basis[9], berr[9], dr[3] = {dir[0], dir[1], dir[2]}, lt = 0, accum, beta_term = 0, amag, fchain = 1, nmax;
  float t, ws;
  FN(ray_t) r;
  int c, j, ne = 0;
  FN(calc_sh)(bd, dr, basis);
  FN(find_bounds)(&r, org, dir, g, opt);
  /* the most samples the ray can take: the length of any sum over them */
  nmax = r.tmax >= r.tmin ? ((REAL)r.tmax - (REAL)r.tmin) / (REAL)step + (REAL)2 : (REAL)0;
  for (c = 0; c < 9; ++c) berr[c] = 0;
  if (bd >= 9) {
    berr[6] = (REAL)2 * (REAL)0.31539156525252005;
    berr[8] = (REAL)2 * (REAL)0.5462742152960396;
  }
  accum = FMA(color[0], gout[0], FMA(color[1], gout[1], color[2] * gout[2]));
  *accum_out = accum;
  *log_t_out = 0;
  if (r.tmin > r.tmax) return;
  if (beta_loss > 0) {
    const REAL tin = EXP(log_t_in);
    beta_term = (REAL)((double)beta_loss * (1.0 - (double)tin / ((double)((REAL)1 - tin) + 1e-3)));
    accum += beta_term;
  }
  amag = (FABS(color[0] * gout[0]) + FABS(color[1] * gout[1])) + FABS(color[2] * gout[2]) + FABS(beta_term);
  t = r.tmin;
  ws = r.world_step;
  while (t <= r.tmax) {
    FN(sample_t) s;
    FN(locate)(g, &r, t, &s);
    if (s.lp[0] < -1) {
      float skip = FN(skip_dist)(s.lp[0], s.l, s.pos, r.d);
      if (skip >= step) {
        t = t + ceilf(skip / step) * step;
        continue;
      }
    }
    REAL sigma = FN(trilerp)(g, &s, g->density, 1, 0);
    if (opt->last_opaque && t + step > r.tmax) ws = 1e9f;
    if (sigma > (REAL)opt->sigma_thresh) {
      REAL col[3], tot[3], in01[3], wts[8], gsp = 0;
      int kink[3];
      FN(sample_colour)(g, &s, basis, col);
      const REAL pcnt = (REAL)ws * sigma;
      const REAL w = EXP(lt) * OMX(-pcnt);
      lt = lt - pcnt;
      ++ne;
      for (c = 0; c < 3; ++c) {
        const REAL lc = col[c] + (REAL)0.5;
        const REAL tc = FMAX(lc, (REAL)0);
        in01[c] = (tc == lc) ? (REAL)1 : (REAL)0;
        kink[c] = FABS(lc) <= (REAL)1e-5;
        tot[c] = tc * gout[c];
      }
      const REAL tcs = (tot[0] + tot[2]) + tot[1];
      const REAL tn = EXP(lt);
      fchain += FABS(lt);
      const REAL fw = fchain + (REAL)4 * FN(corner_max)(g, &s, g->density, 1, 0) / sigma;
      accum = accum - w * tcs;
      REAL gsig = (REAL)ws * (tcs * tn - accum);
      if (sparsity > 0) {
        gsp = sparsity * ((REAL)4 * sigma / ((REAL)1 + (REAL)2 * (sigma * sigma)));
        gsig += gsp;
      }
      /* trilerp_backward_cuvol_one(_density), render_util.cuh:94-153 */
      {
        const REAL p0 = (REAL)s.pos[0], p1 = (REAL)s.pos[1], p2 = (REAL)s.pos[2];
        const REAL ay = (REAL)1 - p1, az = (REAL)1 - p2;
        REAL xo = (REAL)1 - p0;
        wts[0] = ay * az * xo;
        wts[1] = ay * p2 * xo;
        wts[2] = p1 * az * xo;
        wts[3] = p1 * p2 * xo;
        xo = p0;
        wts[4] = ay * az * xo;
        wts[5] = ay * p2 * xo;
        wts[6] = p1 * az * xo;
        wts[7] = p1 * p2 * xo;
      }
      for (j = 0; j < 8; ++j) {
        const int32_t lk = s.lp[co[j]];
        if (lk < 0) continue;
        if (grad_sh)
          for (c = 0; c < C; ++c)
            FN(atomic_add)(grad_sh + (int64_t)lk * C + c, wts[j] * (basis[c % bd] * (w * in01[c / bd] * gout[c / bd])));
        if (grad_density) FN(atomic_add)(grad_density + lk, wts[j] * gsig);
        if (mag_sh)
          for (c = 0; c < C; ++c)
            FN(atomic_add)(mag_sh + (int64_t)lk * C + c,
                           FABS(wts[j] * (w * gout[c / bd])) *
                               (kink[c / bd] ? (REAL)16777216 * FABS(basis[c % bd])
                                             : in01[c / bd] * ((fw + gerr[c / bd]) * FABS(basis[c % bd]) +
                                                                   berr[c % bd])));
        if (mag_density)
          FN(atomic_add)(mag_density + lk,
                         wts[j] * ((REAL)ws * (fchain * FABS(tcs * tn) + (fchain + nmax) * amag) +
                                   fchain * FABS(gsp)));
        if (mask) mask[lk] = 1;
      }
      if (FN(stops)(stop_in, lt, log_stop, ne)) break;
    }
    t = t + step;
  }
  *accum_out = accum - beta_term;
  *log_t_out = lt;
}

/* ---- MSI background.
 * CUDA semantics (opt->bg_cpu == 0): render_background_forward / _backward,
 * render_lerp_kernel_cuvol.cu:386-607, with ray_find_bounds_bg (render_util.cuh:630-676),
 * _unitvec2equirect (render_util.cuh:482-490), trilerp_bg_one / trilerp_backward_bg_one
 * (render_util.cuh:155-232).  Shell i of n = int(nlayers / step) + 2 has radius
 * n / (n - i - 0.5); the ray is sampled at its far intersection with the shell, and the
 * sample's optical depth is sigma * world_step * (1/r_prev - 1/r).
 * Pure-PyTorch semantics (opt->bg_cpu == 1, svox2/svox2.py:796-876): the sample sits at
 * the midpoint between consecutive far intersections and its optical depth is
 * sigma * world_step * (t - t_prev); there is no early stop.  This variant exists only to
 * pin the pieces both share against the reference's own outputs. */
typedef struct {
  REAL o[3], d[3], ws, inner;
  int n_steps;
} FN(bgray_t);

static void FN(bg_setup)(FN(bgray_t) * b, const REAL org[3], const REAL dir[3], const oracle_grid_t* g,
                         const oracle_opt_t* opt) {
  int i;
  REAL ds, inorm, c[3];
  for (i = 0; i < 3; ++i) {
    b->o[i] = FMA(org[i], (REAL)g->scaling[i], (REAL)g->offset[i]);
    b->d[i] = dir[i] * (REAL)g->scaling[i];
  }
  ds = FN(rnorm3)(b->d[0], b->d[1], b->d[2]);
  for (i = 0; i < 3; ++i) b->d[i] = b->d[i] * ds;
  for (i = 0; i < 3; ++i) {
    const REAL sc = (REAL)2 / (REAL)g->size[i];
    b->o[i] = FMA(b->o[i] + (REAL)0.5, sc, (REAL)-1);
    b->d[i] = b->d[i] * sc;
  }
  inorm = FN(rnorm3)(b->d[0], b->d[1], b->d[2]);
  b->ws = ds * inorm;
  for (i = 0; i < 3; ++i) b->d[i] = b->d[i] * inorm;
  /* _dist_ray_to_origin (cuda_util.cuh:112-119): |o x d| */
  c[0] = b->o[1] * b->d[2] - b->o[2] * b->d[1];
  c[1] = b->o[2] * b->d[0] - b->o[0] * b->d[2];
  c[2] = b->o[0] * b->d[1] - b->o[1] * b->d[0];
  b->inner = FMAX((REAL)sqrt((double)c[0] * c[0] + (double)c[1] * c[1] + (double)c[2] * c[2]) + (REAL)1e-3f,
                  (REAL)1);
  b->n_steps = (int)((float)g->bg_nlayers / opt->step) + 2;
}

static REAL FN(bg_fetch)(const oracle_grid_t* g, int64_t u, int l2, REAL p2, int ch) {
  const int32_t lk = g->bg_links[u];
  const float* p;
  if (lk < 0) return 0;
  p = g->bg_data + ((int64_t)lk * g->bg_nlayers + l2) * 4 + ch;
  return FN(lerp)((REAL)p[0], (REAL)p[4], p2);
}

/* trilerp_bg_one: layers first, then y (wrapping at reso), then x (wrapping at 2 reso). */
static REAL FN(bg_trilerp)(const oracle_grid_t* g, const int l[3], const REAL pos[3], int ch) {
  const int64_t reso = g->bg_reso;
  const int ny = l[1] < reso - 1 ? l[1] + 1 : 0, nx = l[0] < 2 * reso - 1 ? l[0] + 1 : 0;
  const REAL ix0 = FN(lerp)(FN(bg_fetch)(g, reso * l[0] + l[1], l[2], pos[2], ch),
                            FN(bg_fetch)(g, reso * l[0] + ny, l[2], pos[2], ch), pos[1]);
  const REAL ix1 = FN(lerp)(FN(bg_fetch)(g, reso * nx + l[1], l[2], pos[2], ch),
                            FN(bg_fetch)(g, reso * nx + ny, l[2], pos[2], ch), pos[1]);
  return FN(lerp)(ix0, ix1, pos[0]);
}

static void FN(bg_add)(const oracle_grid_t* g, int64_t u, int l2, REAL p2, const REAL v[4], REAL* grad,
                       uint8_t* mask) {
  const int32_t lk = g->bg_links[u];
  int64_t row;
  int ch;
  if (lk < 0) return;
  row = (int64_t)lk * g->bg_nlayers + l2;
  for (ch = 0; ch < 4; ++ch) {
    FN(atomic_add)(grad + row * 4 + ch, v[ch] * ((REAL)1 - p2));
    FN(atomic_add)(grad + (row + 1) * 4 + ch, v[ch] * p2);
  }
  if (mask) mask[row] = mask[row + 1] = 1;
}

/* trilerp_backward_bg_one for the three colour channels and sigma at once. */
static void FN(bg_scatter)(const oracle_grid_t* g, const int l[3], const REAL pos[3], const REAL gch[4],
                           REAL* grad, uint8_t* mask) {
  const int64_t reso = g->bg_reso;
  const int ny = l[1] < reso - 1 ? l[1] + 1 : 0, nx = l[0] < 2 * reso - 1 ? l[0] + 1 : 0;
  const REAL ay = (REAL)1 - pos[1];
  const int64_t u[4] = {reso * l[0] + l[1], reso * l[0] + ny, reso * nx + l[1], reso * nx + ny};
  const REAL wy[4] = {ay, pos[1], ay, pos[1]};
  const REAL wx[4] = {(REAL)1 - pos[0], (REAL)1 - pos[0], pos[0], pos[0]};
  int k, ch;
  for (k = 0; k < 4; ++k) {
    REAL v[4];
    for (ch = 0; ch < 4; ++ch) v[ch] = wy[k] * (wx[k] * gch[ch]);
    FN(bg_add)(g, u[k], l[2], pos[2], v, grad, mask);
  }
}

/* One ray's background.  gout NULL: forward, adds the background (and the brightness
 * term) to out.  Otherwise backward: accum is what the foreground left, gradients go to
 * grad_bg / mask_bg. */
static void FN(bg_ray)(const oracle_grid_t* g, const oracle_opt_t* opt, const REAL org[3], const REAL dir[3],
                       REAL lt, const REAL* gout, REAL accum, REAL sparsity, REAL out[3], REAL* grad_bg,
                       uint8_t* mask_bg, uint64_t* n_samples) {
  const REAL C0 = (REAL)0.28209479177387814f;
  const int nl = g->bg_nlayers, cpu = opt->bg_cpu;
  const REAL log_stop = cpu ? (REAL)(-INFINITY) : FN(log_stop)(opt->stop_thresh);
  const double inv_pi = 0.31830988618379067154;
  FN(bgray_t) b;
  REAL invr_last, t_last = 0, outv[3] = {0, 0, 0};
  int i, j, c;
  FN(bg_setup)(&b, org, dir, g, opt);
  invr_last = (REAL)1 / b.inner;
  if (cpu) FN(sphere_hit)(b.o, b.d, b.inner, &t_last, 0);
  for (i = 0; i < b.n_steps; ++i) {
    const REAL r = (REAL)((double)b.n_steps / ((double)(b.n_steps - i) - 0.5));
    REAL t, p[3], pos[3], invr, width, sigma;
    int l[3];
    if (r < b.inner || !FN(sphere_hit)(b.o, b.d, r, &t, 0)) continue;
    if (cpu) {
      const REAL tm = (t + t_last) * (REAL)0.5;
      for (j = 0; j < 3; ++j) p[j] = b.o[j] + tm * b.d[j];
    } else {
      for (j = 0; j < 3; ++j) p[j] = FMA(t, b.d[j], b.o[j]);
    }
    invr = FN(rnorm3)(p[0], p[1], p[2]);
    for (j = 0; j < 3; ++j) p[j] = p[j] * invr;
    {
      /* y clamped to [-1, 1]: a last-bit excess would make asin NaN */
      const REAL lat = ASIN(FMIN(FMAX(p[1], (REAL)-1), (REAL)1)), lon = ATAN2(p[0], p[2]);
      pos[0] = (REAL)((double)(g->bg_reso * 2) * (0.5 + (double)lon * 0.5 * inv_pi));
      pos[1] = (REAL)((double)g->bg_reso * (0.5 - (double)lat * inv_pi));
    }
    pos[2] = FMIN(FMAX(((REAL)1 - invr) * (REAL)nl - (REAL)0.5, (REAL)0), (REAL)(nl - 1));
    /* truncation toward zero, as the device's conversion; a NaN or negative coordinate is cell 0 */
    for (j = 0; j < 3; ++j) l[j] = pos[j] > 0 ? (int)pos[j] : 0;
    if (l[0] > 2 * g->bg_reso - 1) l[0] = 2 * g->bg_reso - 1;
    if (l[1] > g->bg_reso - 1) l[1] = g->bg_reso - 1;
    if (l[2] > nl - 2) l[2] = nl - 2;
    for (j = 0; j < 3; ++j) pos[j] = pos[j] - (REAL)l[j];
    sigma = FN(bg_trilerp)(g, l, pos, 3);
    width = cpu ? t - t_last : invr_last - invr;
    if (sigma > 0) {
      const REAL pcnt = cpu ? b.ws * sigma * width : width * b.ws * sigma;
      const REAL w = EXP(lt) * OMX(-pcnt);
      lt = lt - pcnt;
      if (n_samples) ++*n_samples;
      if (gout == NULL) {
        for (c = 0; c < 3; ++c) outv[c] = outv[c] + w * FMAX(FN(bg_trilerp)(g, l, pos, c) * C0 + (REAL)0.5, (REAL)0);
      } else {
        REAL tc = 0, gch[4];
        for (c = 0; c < 3; ++c) {
          const REAL col = FN(bg_trilerp)(g, l, pos, c) * C0 + (REAL)0.5;
          tc = tc + FMAX(col, (REAL)0) * gout[c];
          gch[c] = col > 0 ? C0 * w * gout[c] : (REAL)0;
        }
        accum = accum - w * tc;
        gch[3] = b.ws * width * (tc * EXP(lt) - accum);
        if (sparsity > 0) gch[3] += sparsity * ((REAL)4 * sigma / ((REAL)1 + (REAL)2 * (sigma * sigma)));
        if (grad_bg) FN(bg_scatter)(g, l, pos, gch, grad_bg, mask_bg);
      }
      if (lt < log_stop) break;
    }
    invr_last = invr;
    t_last = t;
  }
  if (gout == NULL)
    for (c = 0; c < 3; ++c) out[c] = out[c] + (outv[c] + EXP(lt) * (REAL)opt->bg);
}

/* msi_tv_grad_sparse, svox2/csrc/loss_kernel.cu:248-333 (host 606-641): TV of the MSI
 * over the listed cells (index = (x * reso + y) * nlayers + z), one term per channel,
 * with forward differences in x and y that wrap and in z that stop at the last layer;
 * scale (colour channels) and scale_last (the last channel) are divided by the cell count. */
void FN(oracle_msi_tv_grad)(const int32_t* links, int size0, int size1, const float* msi, int nl, int nc,
                            const int32_t* cells, int64_t ncells, float scale, float scale_last, REAL* grad,
                            uint8_t* mask) {
  const float s_col = scale / (float)ncells, s_last = scale_last / (float)ncells;
  int64_t q;
  for (q = 0; q < ncells * nc; ++q) {
    const int ch = (int)(q % nc), idx = cells[q / nc];
    const int z = idx % nl, tmp = idx / nl, y = tmp % size1, x = tmp / size1;
    const int nx = x == size0 - 1 ? 0 : x + 1, ny = y == size1 - 1 ? 0 : y + 1;
    const int32_t l00 = links[(int64_t)x * size1 + y], l01 = links[(int64_t)x * size1 + ny],
                  l10 = links[(int64_t)nx * size1 + y];
    const REAL v00 = l00 >= 0 ? (REAL)msi[((int64_t)l00 * nl + z) * nc + ch] : 0;
    const REAL vz = (l00 >= 0 && z + 1 < nl) ? (REAL)msi[((int64_t)l00 * nl + z + 1) * nc + ch]
                                             : (ch == nc - 1 ? (REAL)0 : v00);
    const REAL v01 = l01 >= 0 ? (REAL)msi[((int64_t)l01 * nl + z) * nc + ch] : 0;
    const REAL v10 = l10 >= 0 ? (REAL)msi[((int64_t)l10 * nl + z) * nc + ch] : 0;
    const REAL sc = (REAL)(ch == nc - 1 ? s_last : s_col);
    REAL dx = v10 - v00, dy = v01 - v00, dz = vz - v00;
    const REAL idelta = sc * (REAL)(1.0 / sqrt((double)(((REAL)1e-9f + dx * dx) + dy * dy) + (double)(dz * dz)));
    REAL sm;
    dx = dx * ((REAL)size0 * ((REAL)1 / (REAL)256));
    dy = dy * ((REAL)size1 * ((REAL)1 / (REAL)256));
    dz = dz * ((REAL)nl * ((REAL)1 / (REAL)256));
    sm = -(dx + dy + dz);
#define MSI_ADD(link, zz, val)                                              \
  if ((link) >= 0 && (val) != 0) {                                          \
    grad[((int64_t)(link) * nl + (zz)) * nc + ch] += (val) * idelta;        \
    if (mask) mask[(int64_t)(link) * nl + (zz)] = 1;                        \
  }
    MSI_ADD(l00, z, sm);
    if (z + 1 < nl) MSI_ADD(l00, z + 1, dz);
    MSI_ADD(l01, z, dy);
    MSI_ADD(l10, z, dx);
#undef MSI_ADD
  }
}

/* Batch over rays: volume_render_cuvol / _fused / _backward
 * (render_lerp_kernel_cuvol.cu:918-958, 1070-1152, 1010-1068).
 *   mode 0: forward, rgb_out written.
 *   mode 1: fused MSE: forward into rgb_out, gout = (rgb_out - rgb_gt) * 2/(3Q), backward.
 *   mode 2: backward with grad_out; rgb_out must hold the forward colour (color_cache).
 * stop_out (optional) receives each ray's early-stop count (-1: no early stop); stop_in
 * (optional) makes every ray stop where such a record says instead of by its own test.
 * mag_density / mag_sh (optional): the per-entry magnitudes of bwd_ray. */
void FN(oracle_render)(const oracle_grid_t* g, const oracle_opt_t* opt, const float* origins, const float* dirs,
                       int64_t Q, int mode, const float* rgb_gt, const float* grad_out, float beta_loss,
                       float sparsity, REAL* rgb_out, REAL* grad_density, REAL* grad_sh, uint8_t* mask,
                       REAL* grad_bg, uint8_t* mask_bg, uint64_t* trace, uint64_t* n_eval_total,
                       uint64_t* n_bg_total, int nthreads, int32_t* stop_out, const int32_t* stop_in,
                       REAL* mag_density, REAL* mag_sh) {
  int64_t q;
  uint64_t total = 0, total_bg = 0;
  const REAL norm = (REAL)2.f / (REAL)(float)(3 * Q);
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads) reduction(+ : total, total_bg)
  for (q = 0; q < Q; ++q) {
    float org[3], dir[3];
    REAL orgr[3], dirr[3], out[3], gout[3], gerr[3] = {0, 0, 0}, lt = 0, acc_b = 0, lt_b = 0, chain = 1;
    const int bg = g->bg_nlayers > 0;
    const int sin_ = stop_in ? stop_in[q] : -2;
    uint64_t ne = 0, nb = 0;
    int i, so = -1;
    for (i = 0; i < 3; ++i) {
      org[i] = origins[q * 3 + i];
      dir[i] = dirs[q * 3 + i];
      orgr[i] = (REAL)org[i];
      dirr[i] = (REAL)dir[i];
    }
    if (mode == 0 || mode == 1) {
      FN(fwd_ray)(g, opt, org, dir, out, &lt, trace ? trace + q : NULL, &ne, sin_, &so, &chain);
      /* render_background_kernel skips rays whose log transmittance is below -25 */
      if (bg && lt >= (REAL)-25) FN(bg_ray)(g, opt, orgr, dirr, lt, NULL, 0, 0, out, NULL, NULL, &nb);
      for (i = 0; i < 3; ++i) rgb_out[q * 3 + i] = out[i];
      if (stop_out) stop_out[q] = so;
    }
    if (mode == 1) {
      for (i = 0; i < 3; ++i) {
        const REAL res = out[i] - (REAL)rgb_gt[q * 3 + i];
        gout[i] = res * norm;
        /* the residual's relative error in a float run, in rounding units: the colour's
         * (chain + 16) units of |out|, over |out - gt| */
        gerr[i] = (chain + (REAL)16) * FABS(out[i]) / FMAX(FABS(res), (REAL)1e-30);
      }
      FN(bwd_ray)(g, opt, org, dir, out, lt, gout, (REAL)beta_loss / (REAL)Q, (REAL)sparsity, grad_density,
                  grad_sh, mask, &acc_b, &lt_b, sin_, mag_density, mag_sh, gerr);
      /* the fused path's background backward starts from the forward's log transmittance */
      if (bg && lt >= (REAL)-25)
        FN(bg_ray)(g, opt, orgr, dirr, lt, gout, acc_b, (REAL)sparsity, NULL, grad_bg, mask_bg, NULL);
    } else if (mode == 2) {
      for (i = 0; i < 3; ++i) {
        out[i] = rgb_out[q * 3 + i];
        gout[i] = (REAL)grad_out[q * 3 + i];
      }
      FN(bwd_ray)(g, opt, org, dir, out, 0, gout, 0, 0, grad_density, grad_sh, NULL, &acc_b, &lt_b, sin_,
                  mag_density, mag_sh, gerr);
      /* volume_render_cuvol_backward: from the backward pass's own log transmittance */
      if (bg && lt_b >= (REAL)-25)
        FN(bg_ray)(g, opt, orgr, dirr, lt_b, gout, acc_b, 0, NULL, grad_bg, NULL, NULL);
    }
    total += ne;
    total_bg += nb;
  }
  if (n_eval_total) *n_eval_total += total;
  if (n_bg_total) *n_bg_total += total_bg;
}

/* trace_ray_expected_term (render_lerp_kernel_cuvol.cu:122-176) and trace_ray_sigma_thresh
 * (178-225): the expected termination distance sum w * (t / step) * world_step, or
 * (threshold) the distance (t / step) * world_step of the first sample with sigma >
 * sigma_thresh.  Neither applies last_sample_opaque. */
static REAL FN(depth_ray)(const oracle_grid_t* g, const oracle_opt_t* opt, const float org[3], const float dir[3],
                          int threshold, float sigma_thresh) {
  const REAL log_stop = FN(log_stop)(opt->stop_thresh), step = (REAL)opt->step;
  REAL lt = 0, outv = 0;
  float t;
  FN(ray_t) r;
  FN(find_bounds)(&r, org, dir, g, opt);
  if (r.tmin > r.tmax) return 0;
  t = r.tmin;
  while (t <= r.tmax) {
    FN(sample_t) s;
    FN(locate)(g, &r, t, &s);
    if (s.lp[0] < -1) {
      float skip = FN(skip_dist)(s.lp[0], s.l, s.pos, r.d);
      if (skip >= opt->step) {
        t = t + ceilf(skip / opt->step) * opt->step;
        continue;
      }
    }
    {
      const REAL sigma = FN(trilerp)(g, &s, g->density, 1, 0);
      if (threshold) {
        if (sigma > (REAL)sigma_thresh) return ((REAL)t / step) * (REAL)r.world_step;
      } else if (sigma > (REAL)opt->sigma_thresh) {
        const REAL pcnt = (REAL)r.world_step * sigma;
        const REAL w = EXP(lt) * OMX(-pcnt);
        lt = lt - pcnt;
        outv = outv + w * ((REAL)t / step) * (REAL)r.world_step;
        if (lt < log_stop) break;
      }
    }
    t = t + opt->step;
  }
  return outv;
}

void FN(oracle_render_depth)(const oracle_grid_t* g, const oracle_opt_t* opt, const float* origins,
                             const float* dirs, int64_t Q, int threshold, float sigma_thresh, REAL* out,
                             int nthreads) {
  int64_t q;
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
  for (q = 0; q < Q; ++q) {
    float org[3], dir[3];
    int i;
    for (i = 0; i < 3; ++i) {
      org[i] = origins[q * 3 + i];
      dir[i] = dirs[q * 3 + i];
    }
    out[q] = FN(depth_ray)(g, opt, org, dir, threshold, sigma_thresh);
  }
}

/* grid_weight_render, svox2/csrc/misc_kernel.cu:183-334 (grid_trace_ray + kernel): every pixel
 * ray of the camera through the dense density grid data [X,Y,Z]; each sample with sigma > 1e-8
 * raises wmax at its cell's 8 corners to the sample's weight.  The bounds and samples follow
 * find_bounds / locate (the grid's transform, near clip 0). */
void FN(oracle_grid_weight_render)(const float* data, const int size[3], const oracle_cam_t* cam, float step_size,
                                   float stop_thresh, int last_opaque, const float offset[3],
                                   const float scaling[3], REAL* wmax) {
  oracle_grid_t g;
  oracle_opt_t opt;
  const REAL log_stop = FN(log_stop)(stop_thresh);
  const int64_t offy = size[2], offx = (int64_t)size[1] * size[2];
  const int64_t co[8] = {0, 1, offy, offy + 1, offx, offx + 1, offx + offy, offx + offy + 1};
  int64_t q, n = (int64_t)cam->width * cam->height;
  int i;
  g.links = NULL;
  g.density = data;
  g.sh = NULL;
  g.n_voxels = 0;
  g.basis_dim = 1;
  for (i = 0; i < 3; ++i) {
    g.size[i] = size[i];
    g.offset[i] = offset[i];
    g.scaling[i] = scaling[i];
  }
  opt.bg = 0.f;
  opt.step = step_size;
  opt.sigma_thresh = 0.f;
  opt.stop_thresh = stop_thresh;
  opt.near_clip = 0.f;
  opt.spheric = 0;
  opt.last_opaque = last_opaque;
  for (q = 0; q < n; ++q) {
    float org[3], dir[3], t;
    REAL ll = 0;
    FN(ray_t) r;
    FN(camera_ray)((int)(q % cam->width), (int)(q / cam->width), cam, dir, org);
    FN(find_bounds)(&r, org, dir, &g, &opt);
    if (r.tmin > r.tmax) continue;
    t = r.tmin;
    while (t <= r.tmax) {
      REAL pos[3], v[8], sigma;
      int l[3], j;
      int64_t idx;
      for (j = 0; j < 3; ++j) {
        float p = fmaf(t, r.d[j], r.o[j]);
        p = fminf(fmaxf(p, 0.f), (float)size[j] - 1.f);
        l[j] = (int)p;
        if (l[j] > size[j] - 2) l[j] = size[j] - 2;
        pos[j] = (REAL)(p - (float)l[j]);
      }
      idx = (int64_t)l[0] * offx + (int64_t)l[1] * offy + l[2];
      for (j = 0; j < 8; ++j) v[j] = (REAL)data[idx + co[j]];
      sigma = FN(lerp)(FN(lerp)(FN(lerp)(v[0], v[1], pos[2]), FN(lerp)(v[2], v[3], pos[2]), pos[1]),
                       FN(lerp)(FN(lerp)(v[4], v[5], pos[2]), FN(lerp)(v[6], v[7], pos[2]), pos[1]), pos[0]);
      if (last_opaque && t + step_size > r.tmax) {
        sigma = sigma + (REAL)1e9f;
        ll = 0;
      }
      if (sigma > (REAL)1e-8f) {
        const REAL la = -((REAL)r.world_step * sigma);
        const REAL w = EXP(ll) * OMX(la);
        ll = ll + la;
        for (j = 0; j < 8; ++j)
          if (w > wmax[idx + co[j]]) wmax[idx + co[j]] = w;
        if (ll < log_stop) break;
      }
      t = t + step_size;
    }
  }
}

/* volume_render_cuvol_image, render_lerp_kernel_cuvol.cu:960-1008 (+ kernel 650-690). */
void FN(oracle_render_image)(const oracle_grid_t* g, const oracle_opt_t* opt, const oracle_cam_t* cam, REAL* out,
                             uint64_t* trace, int nthreads) {
  int64_t q, n = (int64_t)cam->width * cam->height;
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
  for (q = 0; q < n; ++q) {
    float org[3], dir[3];
    REAL orgr[3], dirr[3], rgb[3], lt;
    uint64_t ne = 0;
    int i;
    FN(camera_ray)((int)(q % cam->width), (int)(q / cam->width), cam, dir, org);
    FN(fwd_ray)(g, opt, org, dir, rgb, &lt, trace ? trace + q : NULL, &ne, -2, NULL, NULL);
    for (i = 0; i < 3; ++i) {
      orgr[i] = (REAL)org[i];
      dirr[i] = (REAL)dir[i];
    }
    if (g->bg_nlayers > 0 && lt >= (REAL)-25)
      FN(bg_ray)(g, opt, orgr, dirr, lt, NULL, 0, 0, rgb, NULL, NULL, NULL);
    for (i = 0; i < 3; ++i) out[q * 3 + i] = rgb[i];
  }
}

/* sample_grid / sample_grid_backward, svox2/csrc/svox2_kernel.cu:10-176. */
void FN(oracle_sample)(const oracle_grid_t* g, const float* pts, int64_t P, int want_colors, REAL* out_d,
                       REAL* out_sh) {
  const int C = 3 * g->basis_dim;
  int64_t p;
  for (p = 0; p < P; ++p) {
    FN(sample_t) s;
    int j, c;
    const int64_t offy = g->size[2], offx = (int64_t)g->size[1] * g->size[2];
    for (j = 0; j < 3; ++j) {
      REAL v = FMA((REAL)pts[p * 3 + j], (REAL)g->scaling[j], (REAL)g->offset[j]);
      v = FMIN(FMAX(v, (REAL)0), (REAL)g->size[j] - (REAL)1);
      s.l[j] = (int)v;
      if (s.l[j] > g->size[j] - 2) s.l[j] = g->size[j] - 2;
      s.pos[j] = v - (REAL)s.l[j];
    }
    s.base = (int64_t)s.l[0] * offx + (int64_t)s.l[1] * offy + s.l[2];
    s.lp = g->links + s.base;
    out_d[p] = FN(trilerp)(g, &s, g->density, 1, 0);
    if (want_colors)
      for (c = 0; c < C; ++c) out_sh[p * C + c] = FN(trilerp)(g, &s, g->sh, C, c);
  }
}

void FN(oracle_sample_backward)(const oracle_grid_t* g, const float* pts, int64_t P, int want_colors,
                                const float* gd, const float* gsh, REAL* out_gd, REAL* out_gsh) {
  const int C = 3 * g->basis_dim;
  const int64_t offy = g->size[2], offx = (int64_t)g->size[1] * g->size[2];
  const int64_t co[8] = {0, 1, offy, offy + 1, offx, offx + 1, offx + offy, offx + offy + 1};
  int64_t p;
  for (p = 0; p < P; ++p) {
    REAL pos[3];
    int l[3], j, c;
    for (j = 0; j < 3; ++j) {
      REAL v = FMA((REAL)pts[p * 3 + j], (REAL)g->scaling[j], (REAL)g->offset[j]);
      v = FMIN(FMAX(v, (REAL)0), (REAL)g->size[j] - (REAL)1);
      l[j] = (int)v;
      if (l[j] > g->size[j] - 2) l[j] = g->size[j] - 2;
      pos[j] = v - (REAL)l[j];
    }
    const int32_t* lp = g->links + (int64_t)l[0] * offx + (int64_t)l[1] * offy + l[2];
    const REAL xb = pos[0], yb = pos[1], zb = pos[2];
    const REAL xa = 1 - xb, ya = 1 - yb, za = 1 - zb;
    for (j = 0; j < 8; ++j) {
      const int32_t lk = lp[co[j]];
      if (lk < 0) continue;
      const REAL x = (j & 4) ? xb : xa, y = (j & 2) ? yb : ya, z = (j & 1) ? zb : za;
      out_gd[lk] += (y * (x * (REAL)gd[p])) * z;
      if (want_colors)
        for (c = 0; c < C; ++c) out_gsh[(int64_t)lk * C + c] += (y * (x * (REAL)gsh[p * C + c])) * z;
    }
  }
}

/* tv_kernel, svox2/csrc/loss_kernel.cu:42-109 (host 483-515): the TV value, the mean over
 * cells of sqrt(1e-5 + |d * size/256|^2) summed over channels [start, end); a cell whose voxel
 * has link 0 is skipped with ignore_edge (the reference's early return), and a missing
 * neighbour reads 0 (or the voxel's own value with ignore_edge).  Summed in REAL. */
REAL FN(oracle_tv_value)(const int32_t* links, const int size[3], const float* data, int ncols, int start,
                         int end, int ignore_edge) {
  const int64_t offy = size[2], offx = (int64_t)size[1] * size[2];
  const REAL sx = (REAL)size[0] * (REAL)(1.f / 256.f), sy = (REAL)size[1] * (REAL)(1.f / 256.f),
             sz = (REAL)size[2] * (REAL)(1.f / 256.f);
  const int nl = (size[0] - 1) * (size[1] - 1) * (size[2] - 1);
  REAL sum = 0;
  int x, y, z, c;
  for (x = 0; x < size[0] - 1; ++x)
    for (y = 0; y < size[1] - 1; ++y)
      for (z = 0; z < size[2] - 1; ++z) {
        const int32_t* lp = links + x * offx + y * offy + z;
        const int32_t l000 = lp[0], l100 = lp[offx], l010 = lp[offy], l001 = lp[1];
        if (ignore_edge && l000 == 0) continue;
        for (c = start; c < end; ++c) {
          const REAL v000 = l000 >= 0 ? (REAL)data[(int64_t)l000 * ncols + c] : 0;
          const REAL nul = ignore_edge ? v000 : 0;
          const REAL v100 = l100 >= 0 ? (REAL)data[(int64_t)l100 * ncols + c] : nul;
          const REAL v010 = l010 >= 0 ? (REAL)data[(int64_t)l010 * ncols + c] : nul;
          const REAL v001 = l001 >= 0 ? (REAL)data[(int64_t)l001 * ncols + c] : nul;
          const REAL dx = (v100 - v000) * sx, dy = (v010 - v000) * sy, dz = (v001 - v000) * sz;
          sum = sum + SQRT((REAL)1e-5f + dx * dx + dy * dy + dz * dz);
        }
      }
  return sum * ((REAL)1 / (REAL)nl);
}

/* tv_grad_sparse_kernel, svox2/csrc/loss_kernel.cu:178-246 (host 558-604), and
 * tv_grad_kernel 111-176 (host 522-556) when cells == NULL. */
void FN(oracle_tv_grad)(const int32_t* links, const int size[3], const float* data, int64_t n_rows, int ncols,
                        const int32_t* cells, int64_t n_cells, int start, int end, float scale, int ignore_edge,
                        int ignore_last_z, REAL* grad, uint8_t* mask) {
  const int X = size[0], Y = size[1], Z = size[2];
  const int64_t offy = Z, offx = (int64_t)Y * Z;
  const REAL sx = (REAL)(X * (1.f / 256.f)), sy = (REAL)(Y * (1.f / 256.f)), sz = (REAL)(Z * (1.f / 256.f));
  const int dense = cells == NULL;
  const int64_t ncell = dense ? (int64_t)(X - 1) * (Y - 1) * (Z - 1) : n_cells;
  const REAL sc = (REAL)(scale / (float)(int)ncell);
  int64_t k;
  int idx;
  (void)n_rows;
  for (k = 0; k < ncell; ++k) {
    int x, y, z;
    if (dense) {
      z = (int)(k % (Z - 1));
      y = (int)((k / (Z - 1)) % (Y - 1));
      x = (int)(k / ((int64_t)(Z - 1) * (Y - 1)));
    } else {
      int xyz = cells[k];
      z = xyz % Z;
      y = (xyz / Z) % Y;
      x = (xyz / Z) / Y;
    }
    const int32_t* lp = links + x * offx + y * offy + z;
    const int32_t l000 = lp[0];
    if (ignore_edge && l000 == 0) continue;
    int32_t l001, l010, l100;
    if (dense) {
      l001 = lp[1];
      l010 = lp[offy];
      l100 = lp[offx];
    } else {
      l001 = (z + 1 < Z && (!ignore_last_z || z != Z - 2)) ? lp[1] : 0;
      l010 = y + 1 < Y ? lp[offy] : 0;
      l100 = x + 1 < X ? lp[offx] : 0;
      if (ignore_last_z && z == Z - 2) continue;
    }
    for (idx = start; idx < end; ++idx) {
      const REAL v000 = l000 >= 0 ? (REAL)data[(int64_t)l000 * ncols + idx] : 0;
      const REAL nul = ignore_edge ? v000 : 0;
      const REAL v001 = l001 >= 0 ? (REAL)data[(int64_t)l001 * ncols + idx] : nul;
      const REAL v010 = l010 >= 0 ? (REAL)data[(int64_t)l010 * ncols + idx] : nul;
      const REAL v100 = l100 >= 0 ? (REAL)data[(int64_t)l100 * ncols + idx] : nul;
      REAL dx = v100 - v000, dy = v010 - v000, dz = v001 - v000;
      const REAL idelta = sc / SQRT((REAL)1e-9f + dx * dx + dy * dy + dz * dz);
      dx = dx * sx;
      dy = dy * sy;
      dz = dz * sz;
      const REAL sm = -((dx + dy) + dz);
      if (dense) {
        if (dx != 0 && l100 >= 0) grad[(int64_t)l100 * ncols + idx] += dx * idelta;
        if (dy != 0 && l010 >= 0) grad[(int64_t)l010 * ncols + idx] += dy * idelta;
        if (dz != 0 && l001 >= 0) grad[(int64_t)l001 * ncols + idx] += dz * idelta;
        if (l000 >= 0) grad[(int64_t)l000 * ncols + idx] += sm * idelta;
      } else {
        const int32_t lks[4] = {l000, l001, l010, l100};
        const REAL vals[4] = {sm, dz, dy, dx};
        int q;
        for (q = 0; q < 4; ++q)
          if (lks[q] >= 0 && vals[q] != 0) {
            grad[(int64_t)lks[q] * ncols + idx] += vals[q] * idelta;
            if (mask) mask[lks[q]] = 1;
          }
      }
    }
  }
}

/* rmsprop_once / sgd_once, svox2/csrc/optim_kernel.cu:15-25, 97-103, over the
 * rows selected by kind (0 all, 1 none, 2 mask, 3 index list). */
void FN(oracle_optim)(int rmsprop, REAL* data, REAL* rms, REAL* grad, int64_t n_rows, int ncols, int kind,
                      const uint8_t* mask, const int64_t* index, int64_t n_index, float beta, float lr, float eps,
                      float minval, float lr_last) {
  int64_t k, nr = kind == 3 ? n_index : n_rows;
  int c;
  if (kind == 1) return;
  if (lr_last < 0.f) lr_last = lr;
  for (k = 0; k < nr; ++k) {
    const int64_t row = kind == 3 ? index[k] : k;
    if (kind == 2 && !mask[row]) continue;
    for (c = 0; c < ncols; ++c) {
      const int64_t off = row * ncols + c;
      const REAL l = (REAL)(c == ncols - 1 ? lr_last : lr);
      const REAL g = grad[off];
      if (rmsprop) {
        const REAL g2 = g * g;
        REAL r = rms[off];
        r = (r == 0) ? g2 : FMA((REAL)beta, r - g2, g2);
        rms[off] = r;
        data[off] = FMAX(data[off] - (l * g) / (SQRT(r) + (REAL)eps), (REAL)minval);
      } else {
        data[off] = data[off] - l * g;
      }
      grad[off] = 0;
    }
  }
}

#undef FN
#undef CAT
#undef CAT_
