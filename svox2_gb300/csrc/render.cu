// Ray march, fused MSE adjoint and image render for the `cuvol` backend.
//
// Replaces svox2/csrc/render_lerp_kernel_cuvol.cu (trace_ray_cuvol 30-120,
// trace_ray_cuvol_backward 227-383, kernels 611-773, host 918-1152) with one
// kernel template and three modes:
//   kFwd   volume_render_cuvol / volume_render_cuvol_image
//   kFused volume_render_cuvol_fused   (forward, MSE residual, adjoint)
//   kBwd   volume_render_cuvol_backward (forward, given dL/drgb, adjoint)
//
// Work decomposition (one warp per ray, persistent warps pulling rays from a
// counter):
//   * Prologue, lanes = samples.  32 consecutive samples of the ray at once:
//     each lane forms its sample's t (sequential float adds, as the reference
//     does), grid position, cell, the 8 corner links and the trilinear density.
//     Transmittance is then carried through the evaluated lanes in order with
//     one subtraction per sample, exactly the reference's sequence.
//   * Colour, lanes = (colour channel g, cell corner j), 3 x 8 = 24 lanes.
//     Because the SH basis is fixed for the ray, each corner's colour is
//     reduced to D[j][g] = sum_k basis_k * sh[link_j][g*bd + k] once per cell
//     the ray enters, and a sample's colour is sum_j w_j(pos) D[j][g] — three
//     numbers per corner instead of 27.  Corners shared with the previous cell
//     move between lanes by shuffle; only new corners are gathered, with the
//     27 coefficients of a voxel read by 27 consecutive lanes.
//   * Adjoint, reverse order.  The forward pass stores a checkpoint (t, log T,
//     sample index) per 32-sample segment that holds evaluated samples, and the
//     per-sample colours (up to the cache capacity).  The adjoint walks the
//     segments last to first, recomputes each segment's samples and
//     transmittance from its checkpoint, and accumulates the light-after-sample
//     term as a suffix sum, so no colour_cache dot product is subtracted down to
//     the cancellation floor.  The gradient of d(colour)/d(sh) factorises as
//     basis_k * B[j][g]; B is summed in registers over all samples that share a
//     corner and flushed with one coalesced 27-wide atomic add per corner when
//     the ray leaves it (the reference issues 8 x 27 atomics per sample).
#include "common.cuh"

#include <climits>
#include <cmath>
#include <mutex>

namespace svx {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kThreads = 128;
constexpr int kWarps = kThreads / 32;
constexpr int kNumCkpt = 64;   // stored segment checkpoints per ray before thinning
constexpr int kMaxStride = 64; // checkpoint thinning limit: 64*64 segments per ray
constexpr int kDefaultCap = 192;

enum Mode { kFwd = 0, kFused = 1, kBwd = 2 };

template <typename T> struct SvxDt;
template <> struct SvxDt<float> { static constexpr int v = SVX_F32; };
template <> struct SvxDt<__nv_bfloat16> { static constexpr int v = SVX_BF16; };
template <> struct SvxDt<__half> { static constexpr int v = SVX_F16; };

// SH constants, svox2/csrc/include/render_util.cuh:300-318 (float roundings of
// the published double values).
constexpr float kC0 = 0.28209479177387814f;
constexpr float kC1 = 0.4886025119029199f;
constexpr float kC2_0 = 1.0925484305920792f;
constexpr float kC2_1 = -1.0925484305920792f;
constexpr float kC2_2 = 0.31539156525252005f;
constexpr float kC2_3 = -1.0925484305920792f;
constexpr float kC2_4 = 0.5462742152960396f;

struct GridP {
  const float* density;
  const void* sh;
  const int32_t* links;
  int size[3];
  long long offx, offy;
  float offset[3], scaling[3];
};

struct OptP {
  float bg, step, sigma_thresh, log_stop, near_clip;
  int spheric, last_opaque;
};

struct IoP {
  const float* origins;
  const float* dirs;
  long long n_rays;
  const float* c2w;
  float fx, fy, cx, cy, ndcx, ndcy;
  int width;
  float* rgb_out;
  const float* rgb_gt;
  const float* grad_out;
  float* grad_density;
  float* grad_sh;
  uint8_t* mask;
  float norm;      // 2 / (3 Q) for the fused MSE residual
  float beta;      // beta_loss / Q
  float sparsity;
  unsigned long long* work;    // ray counter (zeroed by the host)
  unsigned long long* eval_count;
  unsigned long long* trace;
  int cap;         // colour cache capacity (samples per ray)
};

// ---------------------------------------------------------------- per-ray setup

struct RayGeo {
  float o[3], d[3];
  float world_step, tmin, tmax;
};

// calc_sh, svox2/csrc/include/render_util.cuh:332-363 (degree <= 2).  The
// (2 zz - xx - yy) term is evaluated in double as the reference's 2.0 literal makes it.
template <int BD>
__device__ __forceinline__ void calc_sh(const float dir[3], float out[9]) {
  out[0] = kC0;
  const float x = dir[0], y = dir[1], z = dir[2];
  if (BD >= 4) {
    out[1] = __fmul_rn(-kC1, y);
    out[2] = __fmul_rn(kC1, z);
    out[3] = __fmul_rn(-kC1, x);
  }
  if (BD >= 9) {
    const float xx = __fmul_rn(x, x), yy = __fmul_rn(y, y), zz = __fmul_rn(z, z);
    const float xy = __fmul_rn(x, y), yz = __fmul_rn(y, z), xz = __fmul_rn(x, z);
    out[4] = __fmul_rn(kC2_0, xy);
    out[5] = __fmul_rn(kC2_1, yz);
    out[6] = (float)__dmul_rn((double)kC2_2,
                              __dsub_rn(__dsub_rn(__dmul_rn(2.0, (double)zz), (double)xx), (double)yy));
    out[7] = __fmul_rn(kC2_3, xz);
    out[8] = __fmul_rn(kC2_4, __fsub_rn(xx, yy));
  }
}

// ConcentricSpheresIntersector, render_util.cuh:546-576.
struct Spheres {
  float q2a, qb, f;
  __device__ Spheres(const float o[3], const float d[3]) {
    const float dd = __fadd_rn(__fadd_rn(__fmul_rn(d[0], d[0]), __fmul_rn(d[1], d[1])), __fmul_rn(d[2], d[2]));
    const float od = __fadd_rn(__fadd_rn(__fmul_rn(o[0], d[0]), __fmul_rn(o[1], d[1])), __fmul_rn(o[2], d[2]));
    const float oo = __fadd_rn(__fadd_rn(__fmul_rn(o[0], o[0]), __fmul_rn(o[1], o[1])), __fmul_rn(o[2], o[2]));
    q2a = __fmul_rn(2.f, dd);
    qb = __fmul_rn(2.f, od);
    f = __fsub_rn(__fmul_rn(qb, qb), __fmul_rn(__fmul_rn(2.f, q2a), oo));
  }
  __device__ bool intersect(float r, float* out, bool near) const {
    const float det = __fadd_rn(f, __fmul_rn(__fmul_rn(__fmul_rn(2.f, q2a), r), r));
    if (det < 0.f) return false;
    const float sq = __fsqrt_rn(det);
    *out = near ? __fdiv_rn(__fsub_rn(-qb, sq), q2a) : __fdiv_rn(__fadd_rn(-qb, sq), q2a);
    return true;
  }
};

// ray_find_bounds, render_util.cuh:578-628 (+ transform_coord cuda_util.cuh:61-67,
// _get_delta_scale render_util.cuh:463-474).
__device__ __forceinline__ void find_bounds(RayGeo& r, const float org[3], const float dir[3],
                                            const GridP& g, const OptP& opt) {
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    r.o[i] = fmaf(org[i], g.scaling[i], g.offset[i]);
    r.d[i] = __fmul_rn(dir[i], g.scaling[i]);
  }
  const float ds = rnorm3_exact(r.d[0], r.d[1], r.d[2]);
#pragma unroll
  for (int i = 0; i < 3; ++i) r.d[i] = __fmul_rn(r.d[i], ds);
  r.world_step = __fmul_rn(ds, opt.step);
  if (opt.spheric) {
    float so[3], sd[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const float s = __fdiv_rn(2.f, (float)g.size[i]);
      so[i] = fmaf(__fadd_rn(r.o[i], 0.5f), s, -1.f);
      sd[i] = __fmul_rn(r.d[i], s);
    }
    Spheres csi(so, sd);
    if (!csi.intersect(1.f, &r.tmax, false) ||
        !csi.intersect(__fsub_rn(1.f, opt.near_clip), &r.tmin, true)) {
      r.tmin = 1e-9f;
      r.tmax = 0.f;
    }
  } else {
    r.tmin = __fmul_rn(__fdiv_rn(opt.near_clip, r.world_step), opt.step);
    r.tmax = 2e3f;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const float inv = __frcp_rn(r.d[i]);
      const float t1 = __fmul_rn(__fsub_rn(-0.5f, r.o[i]), inv);
      const float t2 = __fmul_rn(__fsub_rn(__fsub_rn((float)g.size[i], 0.5f), r.o[i]), inv);
      if (r.d[i] != 0.f) {
        r.tmin = fmaxf(r.tmin, fminf(t1, t2));
        r.tmax = fminf(r.tmax, fmaxf(t1, t2));
      }
    }
  }
}

// cam2world_ray + world2ndc, render_util.cuh:504-544.
__device__ __forceinline__ void camera_ray(int ix, int iy, const IoP& io, float dir[3], float org[3]) {
  float x = __fdiv_rn(__fsub_rn(__fadd_rn((float)ix, 0.5f), io.cx), io.fx);
  float y = __fdiv_rn(__fsub_rn(__fadd_rn((float)iy, 0.5f), io.cy), io.fy);
  const float z = __fsqrt_rn((float)__dadd_rn((double)__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), 1.0));
  x = __fdiv_rn(x, z);
  y = __fdiv_rn(y, z);
  const float zi = __frcp_rn(z);
  const float* m = io.c2w;
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    dir[r] = __fadd_rn(__fadd_rn(__fmul_rn(__ldg(m + 4 * r + 0), x), __fmul_rn(__ldg(m + 4 * r + 1), y)),
                       __fmul_rn(__ldg(m + 4 * r + 2), zi));
    org[r] = __ldg(m + 4 * r + 3);
  }
  if (io.ndcx > 0.f) {
    const float t = __fdiv_rn(__fsub_rn(1.f, org[2]), dir[2]);
#pragma unroll
    for (int i = 0; i < 3; ++i) org[i] = fmaf(t, dir[i], org[i]);
    dir[0] = __fmul_rn(io.ndcx, __fsub_rn(__fdiv_rn(dir[0], dir[2]), __fdiv_rn(org[0], org[2])));
    dir[1] = __fmul_rn(io.ndcy, __fsub_rn(__fdiv_rn(dir[1], dir[2]), __fdiv_rn(org[1], org[2])));
    dir[2] = __fdiv_rn(2.f, org[2]);
    org[0] = __fmul_rn(io.ndcx, __fdiv_rn(org[0], org[2]));
    org[1] = __fmul_rn(io.ndcy, __fdiv_rn(org[1], org[2]));
    org[2] = __fsub_rn(1.f, __fdiv_rn(2.f, org[2]));
    const float rn = rnorm3_exact(dir[0], dir[1], dir[2]);
#pragma unroll
    for (int i = 0; i < 3; ++i) dir[i] = __fmul_rn(dir[i], rn);
  }
}

// compute_skip_dist, render_util.cuh:235-295 (pos_offset = 0).
__device__ __forceinline__ float skip_dist(int32_t link, const int l[3], const float pos[3],
                                           const float d[3]) {
  const uint32_t dist = (uint32_t)(-link);
  const uint32_t shift = dist - 1u;
  const uint32_t side = (uint32_t)((float)(1u << shift) - 1.f);
  float tmin = 0.f, tmax = 1e9f;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const int ul = ((l[i] >> shift) << shift) - l[i];
    const float inv = __frcp_rn(d[i]);
    const float t1 = __fmul_rn(__fsub_rn((float)ul, pos[i]), inv);
    const float t2 = __fmul_rn(__fsub_rn((float)((uint32_t)ul + side), pos[i]), inv);
    if (d[i] != 0.f) {
      tmin = fmaxf(tmin, fminf(t1, t2));
      tmax = fminf(tmax, fmaxf(t1, t2));
    }
  }
  return tmin > 0.f ? 0.f : tmax;
}

// ---------------------------------------------------------------- shared memory

struct WarpSmem {
  int* links;      // [32][8] corner links of the staged samples
  float* tile;     // [8][C] coefficient tile for the corner gather
  float* ck_t;     // [kNumCkpt]
  float* ck_lt;    // [kNumCkpt]
  int* ck_idx;     // [kNumCkpt]
  float* tmp_t;    // [kMaxStride]
  float* tmp_lt;
  int* tmp_idx;
  float* col;      // [cap][3]
};

__host__ __device__ constexpr int warp_smem_floats(int C, int cap) {
  return (32 * 8 + 8 * C + 3 * kNumCkpt + 3 * kMaxStride + 3 * cap + 3) & ~3;
}

__device__ __forceinline__ WarpSmem carve(float* base, int C, int cap) {
  WarpSmem s;
  s.links = reinterpret_cast<int*>(base);
  s.tile = base + 32 * 8;
  s.ck_t = s.tile + 8 * C;
  s.ck_lt = s.ck_t + kNumCkpt;
  s.ck_idx = reinterpret_cast<int*>(s.ck_lt + kNumCkpt);
  s.tmp_t = reinterpret_cast<float*>(s.ck_idx + kNumCkpt);
  s.tmp_lt = s.tmp_t + kMaxStride;
  s.tmp_idx = reinterpret_cast<int*>(s.tmp_lt + kMaxStride);
  s.col = reinterpret_cast<float*>(s.tmp_idx + kMaxStride);
  return s;
}

// ---------------------------------------------------------------- prologue

// One 32-sample segment of the march, lanes = samples.
struct Seg {
  int n;            // lanes [0, n) are ordinary samples (in range, not skipped)
  unsigned evm;     // evaluated lanes (sigma > sigma_thresh), after the stop cut
  bool stopped;     // early termination inside this segment
  bool end;         // the march ends after this segment
  float t_next;     // t of the next segment
  float lt_end;     // log transmittance after the segment
  // per-lane (valid for lanes in evm)
  float pos[3];
  int l[3];
  float sigma, pcnt, ws, lt_before, lt_after;
};

__device__ __forceinline__ void march_segment(Seg& s, float t0, float lt0, const RayGeo& r,
                                              const GridP& g, const OptP& opt, int* slinks,
                                              unsigned long long* trace_h, int lane) {
  __syncwarp();  // every lane is done with the previous segment's staged links
  // Sample t: t0 + step added lane times, one rounding per add (trace_ray_cuvol's t += step).
  float tk = t0;
#pragma unroll
  for (int i = 0; i < 31; ++i)
    if (i < lane) tk = __fadd_rn(tk, opt.step);
  const bool valid = tk <= r.tmax;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    float p = fmaf(tk, r.d[j], r.o[j]);
    p = fminf(fmaxf(p, 0.f), (float)g.size[j] - 1.f);
    s.l[j] = min((int)p, g.size[j] - 2);
    s.pos[j] = __fsub_rn(p, (float)s.l[j]);
  }
  const long long base = (long long)s.l[0] * g.offx + (long long)s.l[1] * g.offy + s.l[2];
  const int32_t* lp = g.links + base;
  const int32_t lk0 = valid ? __ldg(lp) : -1;
  float skip = 0.f;
  if (valid && lk0 < -1) skip = skip_dist(lk0, s.l, s.pos, r.d);
  const bool is_skip = valid && skip >= opt.step;
  const unsigned cut = __ballot_sync(kFull, !valid || is_skip);
  s.n = cut ? __ffs(cut) - 1 : 32;
  const bool normal = lane < s.n;

  float sigma = 0.f;
  if (normal) {
    int lk[8];
    lk[0] = lk0;
    lk[1] = __ldg(lp + 1);
    lk[2] = __ldg(lp + g.offy);
    lk[3] = __ldg(lp + g.offy + 1);
    lk[4] = __ldg(lp + g.offx);
    lk[5] = __ldg(lp + g.offx + 1);
    lk[6] = __ldg(lp + g.offx + g.offy);
    lk[7] = __ldg(lp + g.offx + g.offy + 1);
    float v[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = lk[j] >= 0 ? __ldg(g.density + lk[j]) : 0.f;
    // trilerp_cuvol_one, render_util.cuh:71-91: z, then y, then x.
    const float ix0y0 = lerpf(v[0], v[1], s.pos[2]);
    const float ix0y1 = lerpf(v[2], v[3], s.pos[2]);
    const float ix0 = lerpf(ix0y0, ix0y1, s.pos[1]);
    const float ix1y0 = lerpf(v[4], v[5], s.pos[2]);
    const float ix1y1 = lerpf(v[6], v[7], s.pos[2]);
    const float ix1 = lerpf(ix1y0, ix1y1, s.pos[1]);
    sigma = lerpf(ix0, ix1, s.pos[0]);
    int4* dst = reinterpret_cast<int4*>(slinks + lane * 8);
    dst[0] = make_int4(lk[0], lk[1], lk[2], lk[3]);
    dst[1] = make_int4(lk[4], lk[5], lk[6], lk[7]);
  }
  s.sigma = sigma;
  // last_sample_opaque: the final sample gets an infinite world step (cuvol.cu:79-81).
  s.ws = (opt.last_opaque && __fadd_rn(tk, opt.step) > r.tmax) ? 1e9f : r.world_step;
  s.pcnt = __fmul_rn(s.ws, sigma);
  unsigned evm = __ballot_sync(kFull, normal && sigma > opt.sigma_thresh);

  // Transmittance, evaluated samples in order (cuvol.cu:96-106).  The stop test
  // exp(log T) < stop_thresh is taken as log T < log_stop, log_stop being the
  // smallest float >= ln(stop_thresh).
  float lt = lt0;
  s.lt_before = 0.f;
  s.lt_after = 0.f;
  s.stopped = false;
  unsigned m = evm;
  while (m) {
    const int i = __ffs(m) - 1;
    m &= m - 1;
    const float pc = __shfl_sync(kFull, s.pcnt, i);
    if (lane == i) s.lt_before = lt;
    lt = __fsub_rn(lt, pc);
    if (lane == i) s.lt_after = lt;
    if (lt < opt.log_stop) {
      s.stopped = true;
      s.n = i + 1;
      evm &= (i == 31) ? kFull : ((2u << i) - 1u);
      break;
    }
  }
  s.evm = evm;
  s.lt_end = lt;

  if (trace_h != nullptr) {
    // FNV-1a over (cell, evaluated) of the ordinary samples, then the cut reason.
    unsigned long long h = *trace_h;
    for (int i = 0; i < s.n; ++i) {
      const long long b = __shfl_sync(kFull, base, i);
      h = (h ^ (unsigned long long)b) * 1099511628211ull;
      h = (h ^ (((evm >> i) & 1u) ? 1ull : 2ull)) * 1099511628211ull;
    }
    if (!s.stopped && s.n < 32) {
      const long long b = __shfl_sync(kFull, base, s.n);
      const int sk = __shfl_sync(kFull, (int)is_skip, s.n);
      if (sk) h = ((h ^ (unsigned long long)b) * 1099511628211ull ^ 3ull) * 1099511628211ull;
    }
    *trace_h = h;
  }

  // Next segment start.
  if (s.stopped) {
    s.end = true;
    s.t_next = 0.f;
  } else if (s.n < 32) {
    const float tm = __shfl_sync(kFull, tk, s.n);
    const float sk = __shfl_sync(kFull, skip, s.n);
    const int was_skip = __shfl_sync(kFull, (int)is_skip, s.n);
    if (was_skip) {
      s.t_next = __fadd_rn(tm, __fmul_rn(ceilf(__fdiv_rn(sk, opt.step)), opt.step));
      // a march whose t no longer advances (t + step == t in float) ends here
      s.end = !(s.t_next <= r.tmax) || !(s.t_next > t0);
    } else {
      s.end = true;
      s.t_next = tm;
    }
  } else {
    s.t_next = __fadd_rn(__shfl_sync(kFull, tk, 31), opt.step);
    s.end = !(s.t_next <= r.tmax) || !(s.t_next > t0);
  }
}

// Weight of a sample: T * (1 - exp(-sigma * step)) (trace_ray_cuvol, cuvol.cu:92).  The
// factor is evaluated as -expm1(-x), the same quantity without the cancellation that
// 1 - exp(-x) suffers for the small x of thin media (x ~ 1e-4 loses 3-4 digits).
__device__ __forceinline__ float sample_weight(float lt_before, float pcnt) {
  return __fmul_rn(expf(lt_before), -expm1f(-pcnt));
}

// ---------------------------------------------------------------- corner cache

// Corner j of a cell sits at offset (j>>2, (j>>1)&1, j&1) — the reference's
// link order 0, 1, offy, offy+1, offx, ... (render_util.cuh:79-88).
// Lane L owns (group g = L>>3, corner j = L&7); group 3 (lanes 24-31) carries
// density-gradient accumulators.
__device__ __forceinline__ int corner_src(int j, int dx, int dy, int dz) {
  const int sx = (j >> 2) + dx, sy = ((j >> 1) & 1) + dy, sz = (j & 1) + dz;
  if ((unsigned)sx > 1u || (unsigned)sy > 1u || (unsigned)sz > 1u) return -1;
  return (sx << 2) | (sy << 1) | sz;
}

__device__ __forceinline__ float corner_weight(int j, float px, float py, float pz) {
  const float wx = (j & 4) ? px : __fsub_rn(1.f, px);
  const float wy = (j & 2) ? py : __fsub_rn(1.f, py);
  const float wz = (j & 1) ? pz : __fsub_rn(1.f, pz);
  return __fmul_rn(__fmul_rn(wy, wz), wx);
}

// Move D (lane-resident per-corner colour) from cell `from` to cell `to` and
// gather the corners that are new.  links_to: the 8 corner links of `to`
// (shared memory, broadcast reads).
template <int BD, typename ShT>
__device__ __forceinline__ float update_colour_corners(float D, bool have_from, const int from[3],
                                                       const int to[3], const int* links_to,
                                                       float* tile, const float basis[9],
                                                       const ShT* __restrict__ sh, int lane) {
  constexpr int C = 3 * BD;
  const int dx = to[0] - from[0], dy = to[1] - from[1], dz = to[2] - from[2];
  const bool near = have_from && abs(dx) <= 1 && abs(dy) <= 1 && abs(dz) <= 1;
  const int j = lane & 7, grp = lane >> 3;
  unsigned need = 0;
#pragma unroll
  for (int c = 0; c < 8; ++c)
    if (!near || corner_src(c, dx, dy, dz) < 0) need |= 1u << c;
  const int src = near ? corner_src(j, dx, dy, dz) : -1;
  const float moved = __shfl_sync(kFull, D, src >= 0 ? grp * 8 + src : lane);
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    if (need & (1u << c)) {
      const int lk = links_to[c];
      if (lane < C) tile[c * C + lane] = lk >= 0 ? ldg_f32(sh + (long long)lk * C + lane) : 0.f;
    }
  }
  __syncwarp();
  float out = moved;
  if (grp < 3 && ((need >> j) & 1u)) {
    const float* row = tile + j * C + grp * BD;
    float acc = 0.f;
#pragma unroll
    for (int k = 0; k < BD; ++k) acc = fmaf(basis[k], row[k], acc);
    out = acc;
  }
  __syncwarp();
  return out;
}

// Colour of one sample from lane-resident D: lanes of group g return colour g.
__device__ __forceinline__ float sample_colour(float D, float px, float py, float pz, int lane) {
  float v = (lane < 24) ? __fmul_rn(corner_weight(lane & 7, px, py, pz), D) : 0.f;
  v = __fadd_rn(v, __shfl_xor_sync(kFull, v, 1));
  v = __fadd_rn(v, __shfl_xor_sync(kFull, v, 2));
  v = __fadd_rn(v, __shfl_xor_sync(kFull, v, 4));
  return v;
}

// Gradient accumulators B (lane-resident, same layout as D) for the corners of
// the tracked cell; flush_corners atomically adds the retiring ones.
template <int BD>
__device__ __forceinline__ void flush_corners(unsigned retire, float B, int lk_lane, float my_basis,
                                              float* __restrict__ grad_sh, float* __restrict__ grad_density,
                                              uint8_t* __restrict__ mask, int lane) {
  constexpr int C = 3 * BD;
#pragma unroll 1
  for (int c = 0; c < 8; ++c) {
    if (!((retire >> c) & 1u)) continue;
    const int lk = __shfl_sync(kFull, lk_lane, c);
    const float b = __shfl_sync(kFull, B, (lane < C ? (lane / BD) : 0) * 8 + c);
    if (lk >= 0 && lane < C && b != 0.f && grad_sh != nullptr)
      atomicAdd(grad_sh + (long long)lk * C + lane, __fmul_rn(my_basis, b));
  }
  // density accumulators live in lanes 24..31 (corner = lane - 24)
  if (lane >= 24 && ((retire >> (lane - 24)) & 1u) && lk_lane >= 0) {
    if (grad_density != nullptr && B != 0.f) atomicAdd(grad_density + lk_lane, B);
    if (mask != nullptr) mask[lk_lane] = 1;
  }
}

// ---------------------------------------------------------------- kernel

template <int BD, typename ShT, int MODE, bool IMAGE>
__global__ void __launch_bounds__(kThreads) render_kernel(GridP g, OptP opt, IoP io) {
  constexpr int C = 3 * BD;
  extern __shared__ float4 smem4[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  float* wbase = reinterpret_cast<float*>(smem4) + (size_t)wib * warp_smem_floats(C, io.cap);
  const WarpSmem sm = carve(wbase, C, io.cap);
  const ShT* __restrict__ sh = reinterpret_cast<const ShT*>(g.sh);
  const int grp = lane >> 3, cj = lane & 7;

  unsigned long long evals = 0;
  unsigned long long next = 0;
  if (lane == 0) next = atomicAdd(io.work, 1ull);
  next = __shfl_sync(kFull, next, 0);

  while (next < (unsigned long long)io.n_rays) {
    const long long ray = (long long)next;
    if (lane == 0) next = atomicAdd(io.work, 1ull);  // prefetch the following ray
    // ---- ray setup (all lanes, redundantly)
    float org[3], dir[3];
    if (IMAGE) {
      camera_ray((int)(ray % io.width), (int)(ray / io.width), io, dir, org);
    } else {
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        org[i] = __ldg(io.origins + ray * 3 + i);
        dir[i] = __ldg(io.dirs + ray * 3 + i);
      }
    }
    float basis[9];
    calc_sh<BD>(dir, basis);
    float my_basis = 0.f;
#pragma unroll
    for (int k = 0; k < BD; ++k)
      if (lane % BD == k) my_basis = basis[k];
    RayGeo rg;
    find_bounds(rg, org, dir, g, opt);
    unsigned long long th = 1469598103934665603ull;
    unsigned long long* thp = io.trace != nullptr ? &th : nullptr;

    if (!(rg.tmin <= rg.tmax)) {
      // Ray misses the grid: background only, no gradient (cuvol.cu:42-48, 253-258).
      if (MODE != kBwd && lane < 3) io.rgb_out[ray * 3 + lane] = opt.bg;
      if (io.trace != nullptr && lane == 0) io.trace[ray] = th;
      next = __shfl_sync(kFull, next, 0);
      continue;
    }

    // ---- forward march
    float t = rg.tmin, lt = 0.f;
    float acc = 0.f;             // lanes of group g: colour g
    float D = 0.f;
    int cell[3] = {0, 0, 0};
    bool have_cell = false;
    int n_eval = 0, nck = 0, stride = 1, seg_since_ck = 0;
    bool stopped = false;
    while (t <= rg.tmax) {
      Seg s;
      march_segment(s, t, lt, rg, g, opt, sm.links, thp, lane);
      if (MODE != kFwd && s.evm) {
        // checkpoint the segment (thinned to every stride-th evaluated segment)
        if (seg_since_ck == 0) {
          if (nck == kNumCkpt && stride < kMaxStride) {
            // keep every other checkpoint, double the stride (kNumCkpt == 64: one per lane pair)
            const float a = sm.ck_t[2 * lane], b = sm.ck_lt[2 * lane];
            const int c = sm.ck_idx[2 * lane];
            __syncwarp();
            sm.ck_t[lane] = a;
            sm.ck_lt[lane] = b;
            sm.ck_idx[lane] = c;
            __syncwarp();
            nck = kNumCkpt / 2;
            stride *= 2;
          }
          if (nck < kNumCkpt) {  // always true within the host's samples-per-ray limit
            if (lane == 0) {
              sm.ck_t[nck] = t;
              sm.ck_lt[nck] = lt;
              sm.ck_idx[nck] = n_eval;
            }
            ++nck;
          }
        }
        seg_since_ck = (seg_since_ck + 1) % stride;
      }
      __syncwarp();
      const float w_lane = sample_weight(s.lt_before, s.pcnt);
      unsigned m = s.evm;
      while (m) {
        const int i = __ffs(m) - 1;
        m &= m - 1;
        const int to[3] = {__shfl_sync(kFull, s.l[0], i), __shfl_sync(kFull, s.l[1], i),
                           __shfl_sync(kFull, s.l[2], i)};
        const float px = __shfl_sync(kFull, s.pos[0], i);
        const float py = __shfl_sync(kFull, s.pos[1], i);
        const float pz = __shfl_sync(kFull, s.pos[2], i);
        const float wi = __shfl_sync(kFull, w_lane, i);
        if (!have_cell || to[0] != cell[0] || to[1] != cell[1] || to[2] != cell[2]) {
          D = update_colour_corners<BD, ShT>(D, have_cell, cell, to, sm.links + i * 8, sm.tile, basis,
                                             sh, lane);
          cell[0] = to[0];
          cell[1] = to[1];
          cell[2] = to[2];
          have_cell = true;
        }
        const float col = sample_colour(D, px, py, pz, lane);
        acc = fmaf(wi, fmaxf(__fadd_rn(col, 0.5f), 0.f), acc);
        if (MODE != kFwd && n_eval < io.cap && cj == 0 && grp < 3) sm.col[n_eval * 3 + grp] = col;
        ++n_eval;
      }
      lt = s.lt_end;
      if (s.stopped) {
        stopped = true;
        break;
      }
      if (s.end) break;
      t = s.t_next;
    }
    __syncwarp();
    evals += (unsigned long long)n_eval;
    const float lt_fwd = stopped ? -1e3f : lt;   // cuvol.cu:103-106
    const float out_c = fmaf(expf(lt_fwd), opt.bg, acc);
    if (MODE != kBwd && grp < 3 && cj == 0) io.rgb_out[ray * 3 + grp] = out_c;
    if (io.trace != nullptr && lane == 0) io.trace[ray] = th;

    if (MODE != kFwd) {
      // ---- adjoint seed
      float gout[3];
      if (MODE == kFused) {
        // residual of the MSE loss (cuvol.cu:735-741)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const float oc = __shfl_sync(kFull, out_c, c * 8);
          gout[c] = __fmul_rn(__fsub_rn(oc, __ldg(io.rgb_gt + ray * 3 + c)), io.norm);
        }
      } else {
#pragma unroll
        for (int c = 0; c < 3; ++c) gout[c] = __ldg(io.grad_out + ray * 3 + c);
      }
      const float gmine = grp < 3 ? gout[grp == 0 ? 0 : (grp == 1 ? 1 : 2)] : 0.f;
      // light that passes the last sample: background, plus the beta-loss term (cuvol.cu:259-264)
      float accum = __fmul_rn(__fmul_rn(expf(lt_fwd), opt.bg),
                              __fadd_rn(__fadd_rn(gout[0], gout[1]), gout[2]));
      if (MODE == kFused && io.beta > 0.f) {
        const float tin = expf(lt_fwd);
        const double f = 1.0 - (double)tin / __dadd_rn((double)__fsub_rn(1.f, tin), 1e-3);
        accum = __fadd_rn(accum, (float)((double)io.beta * f));
      }

      // ---- reverse pass over checkpointed segments
      float B = 0.f;               // lanes <24: colour gradient per (g, corner); 24..31: density
      int lk_lane = -1;            // link of corner (lane & 7) of the tracked cell
      int bcell[3] = {0, 0, 0};
      bool have_b = false;
      bool have_d = false;
      int dcell[3] = {0, 0, 0};
      for (int k = nck - 1; k >= 0; --k) {
        // regenerate the starts of the evaluated segments this checkpoint covers
        int cnt = 0;
        if (stride == 1) {
          if (lane == 0) {
            sm.tmp_t[0] = sm.ck_t[k];
            sm.tmp_lt[0] = sm.ck_lt[k];
            sm.tmp_idx[0] = sm.ck_idx[k];
          }
          cnt = 1;
          __syncwarp();
        } else {
          float tt = sm.ck_t[k], ll = sm.ck_lt[k];
          int ii = sm.ck_idx[k];
          const int want = stride;
          while (cnt < want) {
            Seg s;
            march_segment(s, tt, ll, rg, g, opt, sm.links, nullptr, lane);
            if (s.evm) {
              if (lane == 0) {
                sm.tmp_t[cnt] = tt;
                sm.tmp_lt[cnt] = ll;
                sm.tmp_idx[cnt] = ii;
              }
              ++cnt;
              ii += __popc(s.evm);
            }
            ll = s.lt_end;
            if (s.stopped || s.end) break;
            tt = s.t_next;
          }
          __syncwarp();
        }
        for (int b = cnt - 1; b >= 0; --b) {
          Seg s;
          const float t0 = sm.tmp_t[b], lt0 = sm.tmp_lt[b];
          const int idx0 = sm.tmp_idx[b];
          __syncwarp();
          march_segment(s, t0, lt0, rg, g, opt, sm.links, nullptr, lane);
          __syncwarp();
          const float w_lane = sample_weight(s.lt_before, s.pcnt);
          const float tn_lane = expf(s.lt_after);
          unsigned m = s.evm;
          int rank = __popc(m);
          while (m) {
            const int i = 31 - __clz(m);
            m &= ~(1u << i);
            --rank;
            const int idx = idx0 + rank;
            const int to[3] = {__shfl_sync(kFull, s.l[0], i), __shfl_sync(kFull, s.l[1], i),
                               __shfl_sync(kFull, s.l[2], i)};
            const float px = __shfl_sync(kFull, s.pos[0], i);
            const float py = __shfl_sync(kFull, s.pos[1], i);
            const float pz = __shfl_sync(kFull, s.pos[2], i);
            const float wi = __shfl_sync(kFull, w_lane, i);
            const float tni = __shfl_sync(kFull, tn_lane, i);
            const float wsi = __shfl_sync(kFull, s.ws, i);
            const float sgi = __shfl_sync(kFull, s.sigma, i);
            if (!have_b || to[0] != bcell[0] || to[1] != bcell[1] || to[2] != bcell[2]) {
              const int dx = to[0] - bcell[0], dy = to[1] - bcell[1], dz = to[2] - bcell[2];
              const bool near = have_b && abs(dx) <= 1 && abs(dy) <= 1 && abs(dz) <= 1;
              if (have_b) {
                unsigned retire = 0;
#pragma unroll
                for (int c = 0; c < 8; ++c)
                  if (!near || corner_src(c, -dx, -dy, -dz) < 0) retire |= 1u << c;
                flush_corners<BD>(retire, B, lk_lane, my_basis, io.grad_sh, io.grad_density, io.mask,
                                  lane);
              }
              const int src = near ? corner_src(cj, dx, dy, dz) : -1;
              const float moved = __shfl_sync(kFull, B, src >= 0 ? grp * 8 + src : lane);
              B = src >= 0 ? moved : 0.f;
              lk_lane = sm.links[i * 8 + cj];
              bcell[0] = to[0];
              bcell[1] = to[1];
              bcell[2] = to[2];
              have_b = true;
            }
            float col;
            if (idx < io.cap) {
              col = grp < 3 ? sm.col[idx * 3 + grp] : 0.f;
            } else {
              if (!have_d || to[0] != dcell[0] || to[1] != dcell[1] || to[2] != dcell[2]) {
                D = update_colour_corners<BD, ShT>(D, have_d, dcell, to, sm.links + i * 8, sm.tile,
                                                   basis, sh, lane);
                dcell[0] = to[0];
                dcell[1] = to[1];
                dcell[2] = to[2];
                have_d = true;
              }
              col = sample_colour(D, px, py, pz, lane);
            }
            // d(loss)/d(colour) pieces, trace_ray_cuvol_backward cuvol.cu:311-344
            const float sc = __fadd_rn(col, 0.5f);
            const float part = grp < 3 ? __fmul_rn(fmaxf(sc, 0.f), gmine) : 0.f;
            const float p0 = __shfl_sync(kFull, part, 0);
            const float p1 = __shfl_sync(kFull, part, 8);
            const float p2 = __shfl_sync(kFull, part, 16);
            const float tc = __fadd_rn(__fadd_rn(p0, p2), p1);
            float gsig = __fmul_rn(wsi, __fsub_rn(__fmul_rn(tc, tni), accum));
            if (io.sparsity > 0.f)
              gsig = fmaf(io.sparsity,
                          __fdiv_rn(__fmul_rn(4.f, sgi), __fadd_rn(1.f, __fmul_rn(2.f, __fmul_rn(sgi, sgi)))),
                          gsig);
            accum = fmaf(wi, tc, accum);
            const float wt = corner_weight(cj, px, py, pz);
            if (grp < 3) {
              const float a = (sc >= 0.f) ? __fmul_rn(wi, gmine) : 0.f;
              B = fmaf(wt, a, B);
            } else {
              B = fmaf(wt, gsig, B);
            }
          }
          __syncwarp();
        }
      }
      if (have_b)
        flush_corners<BD>(0xffu, B, lk_lane, my_basis, io.grad_sh, io.grad_density, io.mask, lane);
    }
    __syncwarp();
    next = __shfl_sync(kFull, next, 0);
  }
  if (io.eval_count != nullptr && lane == 0 && evals) atomicAdd(io.eval_count, evals);
}

// ---------------------------------------------------------------- host side

int g_cap = kDefaultCap;

template <int BD, typename ShT, int MODE, bool IMAGE>
int launch_t(const GridP& g, const OptP& opt, IoP io, long long n_rays, cudaStream_t st) {
  constexpr int C = 3 * BD;
  auto kern = render_kernel<BD, ShT, MODE, IMAGE>;
  const int cap = MODE == kFwd ? 0 : io.cap;
  io.cap = cap;
  const size_t smem = sizeof(float) * (size_t)warp_smem_floats(C, cap) * kWarps;
  static std::mutex mu;
  static int blocks_per_sm[2][1024];  // indexed by device, cap/4 (0 = unset)
  int dev = 0;
  SVX_CUDA_TRY(cudaGetDevice(&dev));
  int bps;
  {
    std::lock_guard<std::mutex> lk(mu);
    int& slot = blocks_per_sm[dev & 1][(cap / 4) & 1023];
    if (slot == 0) {
      SVX_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      int b = 0;
      SVX_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, kThreads, smem));
      slot = b > 0 ? b : 1;
    }
    bps = slot;
  }
  long long blocks = (long long)num_sms() * bps;
  const long long need = (n_rays + kWarps - 1) / kWarps;
  if (blocks > need) blocks = need;
  if (blocks < 1) blocks = 1;
  SVX_CUDA_TRY(cudaMemsetAsync(io.work, 0, sizeof(unsigned long long), st));
  kern<<<(unsigned)blocks, kThreads, smem, st>>>(g, opt, io);
  SVX_LAUNCH_CHECK("render_kernel");
  return SVX_OK;
}

template <int MODE, bool IMAGE>
int dispatch(const svx_grid_t* grid, const GridP& g, const OptP& opt, const IoP& io, long long n,
             cudaStream_t st) {
  const int bd = grid->basis_dim;
  const int dt = grid->sh_dtype;
#define SVX_CASE(BDV, T)                                   \
  if (bd == BDV && dt == SvxDt<T>::v) return launch_t<BDV, T, MODE, IMAGE>(g, opt, io, n, st);
  SVX_CASE(9, float) SVX_CASE(9, __nv_bfloat16) SVX_CASE(9, __half)
  SVX_CASE(4, float) SVX_CASE(4, __nv_bfloat16) SVX_CASE(4, __half)
  SVX_CASE(1, float) SVX_CASE(1, __nv_bfloat16) SVX_CASE(1, __half)
#undef SVX_CASE
  set_error("unsupported basis_dim %d / sh dtype %d", bd, dt);
  return SVX_ERR_UNSUPPORTED;
}

}  // namespace

// Validation shared by the render entry points (SparseGridSpec::check,
// data_spec.hpp:32-51, plus what the kernels assume).
int check_grid(const svx_grid_t* grid) {
  SVX_REQUIRE(grid != nullptr, SVX_ERR_INVALID, "grid is null");
  SVX_REQUIRE(grid->links != nullptr && grid->density_data != nullptr && grid->sh_data != nullptr,
              SVX_ERR_INVALID, "grid tables must be non-null device pointers");
  for (int i = 0; i < 3; ++i)
    SVX_REQUIRE(grid->size[i] >= 2, SVX_ERR_INVALID, "grid size[%d] = %d, each side must be >= 2", i,
                grid->size[i]);
  SVX_REQUIRE(grid->basis_type == SVX_BASIS_SH, SVX_ERR_UNSUPPORTED,
              "basis_type %d: only SH (1) is built", grid->basis_type);
  SVX_REQUIRE(grid->basis_dim == 1 || grid->basis_dim == 4 || grid->basis_dim == 9, SVX_ERR_UNSUPPORTED,
              "basis_dim %d: SH of degree <= 2 (1, 4 or 9) is built", grid->basis_dim);
  SVX_REQUIRE(grid->sh_data_dim == 3 * grid->basis_dim, SVX_ERR_INVALID,
              "sh_data_dim %d != 3 * basis_dim %d", grid->sh_data_dim, grid->basis_dim);
  SVX_REQUIRE(grid->background_nlayers == 0, SVX_ERR_UNSUPPORTED,
              "MSI background (background_nlayers = %d) is not built", grid->background_nlayers);
  SVX_REQUIRE(grid->sh_dtype == SVX_F32 || grid->sh_dtype == SVX_BF16 || grid->sh_dtype == SVX_F16,
              SVX_ERR_INVALID, "sh_dtype %d unknown", grid->sh_dtype);
  SVX_REQUIRE(grid->n_voxels >= 0 && grid->n_voxels < (1ll << 31), SVX_ERR_TOO_LARGE,
              "n_voxels %lld must fit int32 links", (long long)grid->n_voxels);
  return SVX_OK;
}

static GridP make_grid(const svx_grid_t* grid) {
  GridP g;
  g.density = grid->density_data;
  g.sh = grid->sh_data;
  g.links = grid->links;
  for (int i = 0; i < 3; ++i) {
    g.size[i] = grid->size[i];
    g.offset[i] = grid->offset[i];
    g.scaling[i] = grid->scaling[i];
  }
  g.offy = grid->size[2];
  g.offx = (long long)grid->size[1] * grid->size[2];
  return g;
}

// Smallest float >= ln(x), so that (float l) < it  <=>  exp(l) < x exactly.
static float log_stop_threshold(float x) {
  if (!(x > 0.f)) return -INFINITY;
  const double L = std::log((double)x);
  float f = (float)L;
  if ((double)f < L) f = std::nextafter(f, INFINITY);
  // (double)f >= L; step down while the next lower float still is >= L
  while ((double)std::nextafter(f, -INFINITY) >= L) f = std::nextafter(f, -INFINITY);
  return f;
}

static int make_opt(const svx_render_opts_t* o, OptP* p) {
  SVX_REQUIRE(o != nullptr, SVX_ERR_INVALID, "render options are null");
  SVX_REQUIRE(o->step_size > 0.f, SVX_ERR_INVALID, "step_size must be > 0 (got %g)", (double)o->step_size);
  p->bg = o->background_brightness;
  p->step = o->step_size;
  p->sigma_thresh = o->sigma_thresh;
  p->log_stop = log_stop_threshold(o->stop_thresh);
  p->near_clip = o->near_clip;
  p->spheric = o->use_spheric_clip != 0;
  p->last_opaque = o->last_sample_opaque != 0;
  return SVX_OK;
}

// Scratch: the ray counter.  Stream-ordered allocation, released after the launch.
struct Scratch {
  unsigned long long* p = nullptr;
  cudaStream_t st;
  explicit Scratch(cudaStream_t s) : st(s) {}
  int alloc() {
    SVX_CUDA_TRY(cudaMallocAsync((void**)&p, 256, st));
    return SVX_OK;
  }
  ~Scratch() {
    if (p) cudaFreeAsync(p, st);
  }
};

template <int MODE>
static int render_rays(const svx_grid_t* grid, const svx_rays_t* rays, const svx_render_opts_t* opt,
                       IoP io, const svx_render_stats_t* stats, void* stream) {
  clear_error();
  int rc = check_grid(grid);
  if (rc) return rc;
  SVX_REQUIRE(rays != nullptr, SVX_ERR_INVALID, "rays are null");
  SVX_REQUIRE(rays->n_rays >= 0, SVX_ERR_INVALID, "n_rays < 0");
  if (rays->n_rays == 0) return SVX_OK;
  SVX_REQUIRE(rays->origins && rays->dirs, SVX_ERR_INVALID, "ray tables must be non-null");
  OptP o;
  rc = make_opt(opt, &o);
  if (rc) return rc;
  const GridP g = make_grid(grid);
  if (MODE != kFwd) {
    // every ray's samples must fit the adjoint's checkpoints (kNumCkpt x kMaxStride segments)
    const double diag = std::sqrt((double)g.size[0] * g.size[0] + (double)g.size[1] * g.size[1] +
                                  (double)g.size[2] * g.size[2]);
    const double max_samples = diag / (double)o.step + 2.0;
    SVX_REQUIRE(max_samples <= (double)kNumCkpt * kMaxStride, SVX_ERR_TOO_LARGE,
                "up to %.0f samples per ray (grid diagonal / step_size); the adjoint supports %d",
                max_samples, kNumCkpt * kMaxStride);
  }
  io.origins = rays->origins;
  io.dirs = rays->dirs;
  io.n_rays = rays->n_rays;
  io.eval_count = stats ? reinterpret_cast<unsigned long long*>(stats->eval_samples) : nullptr;
  io.trace = stats ? reinterpret_cast<unsigned long long*>(stats->ray_trace) : nullptr;
  io.cap = g_cap;
  cudaStream_t st = as_stream(stream);
  Scratch scr(st);
  rc = scr.alloc();
  if (rc) return rc;
  io.work = scr.p;
  return dispatch<MODE, false>(grid, g, o, io, rays->n_rays, st);
}

}  // namespace svx

using namespace svx;

extern "C" int svx_volume_render_cuvol(const svx_grid_t* grid, const svx_rays_t* rays,
                                       const svx_render_opts_t* opt, float* rgb_out,
                                       const svx_render_stats_t* stats, void* stream) {
  SVX_REQUIRE(rgb_out != nullptr || (rays && rays->n_rays == 0), SVX_ERR_INVALID, "rgb_out is null");
  IoP io{};
  io.rgb_out = rgb_out;
  return render_rays<kFwd>(grid, rays, opt, io, stats, stream);
}

extern "C" int svx_volume_render_cuvol_fused(const svx_grid_t* grid, const svx_rays_t* rays,
                                             const svx_render_opts_t* opt, const float* rgb_gt,
                                             float beta_loss, float sparsity_loss, float* rgb_out,
                                             const svx_grid_grads_t* grads,
                                             const svx_render_stats_t* stats, void* stream) {
  SVX_REQUIRE(rays != nullptr, SVX_ERR_INVALID, "rays are null");
  SVX_REQUIRE(grads != nullptr, SVX_ERR_INVALID, "grads are null");
  SVX_REQUIRE(rays->n_rays == 0 || (rgb_gt && rgb_out), SVX_ERR_INVALID, "rgb_gt / rgb_out are null");
  IoP io{};
  io.rgb_out = rgb_out;
  io.rgb_gt = rgb_gt;
  io.grad_density = grads->grad_density_out;
  io.grad_sh = grads->grad_sh_out;
  io.mask = grads->mask_out;
  io.norm = rays->n_rays > 0 ? 2.f / (float)(3 * (long long)rays->n_rays) : 0.f;
  io.beta = rays->n_rays > 0 ? beta_loss / (float)rays->n_rays : 0.f;
  io.sparsity = sparsity_loss;
  return render_rays<kFused>(grid, rays, opt, io, stats, stream);
}

extern "C" int svx_volume_render_cuvol_backward(const svx_grid_t* grid, const svx_rays_t* rays,
                                                const svx_render_opts_t* opt, const float* grad_out,
                                                const float* color_cache, const svx_grid_grads_t* grads,
                                                const svx_render_stats_t* stats, void* stream) {
  (void)color_cache;
  SVX_REQUIRE(rays != nullptr, SVX_ERR_INVALID, "rays are null");
  SVX_REQUIRE(grads != nullptr, SVX_ERR_INVALID, "grads are null");
  SVX_REQUIRE(rays->n_rays == 0 || grad_out, SVX_ERR_INVALID, "grad_out is null");
  IoP io{};
  io.grad_out = grad_out;
  io.grad_density = grads->grad_density_out;
  io.grad_sh = grads->grad_sh_out;
  io.mask = grads->mask_out;
  return render_rays<kBwd>(grid, rays, opt, io, stats, stream);
}

extern "C" int svx_volume_render_cuvol_image(const svx_grid_t* grid, const svx_camera_t* cam,
                                             const svx_render_opts_t* opt, float* rgb_out,
                                             const svx_render_stats_t* stats, void* stream) {
  clear_error();
  int rc = check_grid(grid);
  if (rc) return rc;
  SVX_REQUIRE(cam != nullptr, SVX_ERR_INVALID, "camera is null");
  SVX_REQUIRE(cam->width >= 0 && cam->height >= 0, SVX_ERR_INVALID, "negative image size");
  SVX_REQUIRE(cam->c2w_rows == 3 || cam->c2w_rows == 4, SVX_ERR_INVALID, "c2w must have 3 or 4 rows");
  const long long n = (long long)cam->width * cam->height;
  if (n == 0) return SVX_OK;
  SVX_REQUIRE(cam->c2w != nullptr && rgb_out != nullptr, SVX_ERR_INVALID, "c2w / rgb_out are null");
  OptP o;
  rc = make_opt(opt, &o);
  if (rc) return rc;
  const GridP g = make_grid(grid);
  IoP io{};
  io.c2w = cam->c2w;
  io.fx = cam->fx;
  io.fy = cam->fy;
  io.cx = cam->cx;
  io.cy = cam->cy;
  io.ndcx = cam->ndc_coeffx;
  io.ndcy = cam->ndc_coeffy;
  io.width = cam->width;
  io.n_rays = n;
  io.rgb_out = rgb_out;
  io.eval_count = stats ? reinterpret_cast<unsigned long long*>(stats->eval_samples) : nullptr;
  io.trace = stats ? reinterpret_cast<unsigned long long*>(stats->ray_trace) : nullptr;
  io.cap = 0;
  cudaStream_t st = as_stream(stream);
  Scratch scr(st);
  rc = scr.alloc();
  if (rc) return rc;
  io.work = scr.p;
  return dispatch<kFwd, true>(grid, g, o, io, n, st);
}

extern "C" int svx_color_cache_capacity(void) { return svx::g_cap; }

// ---------------------------------------------------------------- no-allocation entry point
//
// Some callers cannot allocate device memory while they run: code that
// executes inside another framework's stream callbacks or replayed work,
// embedded and real-time hosts that plan all device memory before they start,
// and processes where a foreign allocator owns the device heap, so that a
// cudaMalloc (or a stream-ordered allocation) would fail or compete with it.
// svx_volume_render_cuvol_fused_noalloc serves them: it is the fused render
// above with its one piece of scratch — the persistent warps' ray counter —
// taken from the file-scope array below instead of an allocation.
//
// The array is kStaticScratchWords 64-bit words (256 bytes).  Every GPU that
// loads this library holds one copy of it until the process exits.  A call
// needs one word; the entry rejects any request for more scratch than the
// array holds.  All calls share the array and it keeps the last call's
// contents: each call clears the counter on its stream before the kernel
// starts, so calls that overlap on the GPU (on different streams, or from
// different host threads) race on the counter and must be serialised by the
// caller.
constexpr int kStaticScratchWords = 32;
static __device__ __align__(256) unsigned long long g_static_scratch[kStaticScratchWords];

// Device address of g_static_scratch on the current device, looked up once
// per device (with that device current) and cached.  In host code the
// symbol's name is only a host-side stand-in; the kernel must be given the
// address cudaGetSymbolAddress returns.
static int static_scratch_address(unsigned long long** out) {
  static std::mutex mu;
  static unsigned long long* addr[64] = {nullptr};
  int dev = 0;
  SVX_CUDA_TRY(cudaGetDevice(&dev));
  SVX_REQUIRE(dev >= 0 && dev < 64, SVX_ERR_UNSUPPORTED, "device index %d: at most 64 devices", dev);
  std::lock_guard<std::mutex> lk(mu);
  if (addr[dev] == nullptr) {
    void* p = nullptr;
    SVX_CUDA_TRY(cudaGetSymbolAddress(&p, g_static_scratch));
    addr[dev] = reinterpret_cast<unsigned long long*>(p);
  }
  *out = addr[dev];
  return SVX_OK;
}

extern "C" int svx_volume_render_cuvol_fused_noalloc(const svx_grid_t* grid, const svx_rays_t* rays,
                                                     const svx_render_opts_t* opt, const float* rgb_gt,
                                                     float beta_loss, float sparsity_loss, float* rgb_out,
                                                     const svx_grid_grads_t* grads,
                                                     const svx_render_stats_t* stats, void* stream) {
  clear_error();
  SVX_REQUIRE(rays != nullptr, SVX_ERR_INVALID, "rays are null");
  SVX_REQUIRE(grads != nullptr, SVX_ERR_INVALID, "grads are null");
  SVX_REQUIRE(rays->n_rays == 0 || (rgb_gt && rgb_out), SVX_ERR_INVALID, "rgb_gt / rgb_out are null");
  int rc = check_grid(grid);
  if (rc) return rc;
  SVX_REQUIRE(rays->n_rays >= 0, SVX_ERR_INVALID, "n_rays < 0");
  if (rays->n_rays == 0) return SVX_OK;
  SVX_REQUIRE(rays->origins && rays->dirs, SVX_ERR_INVALID, "ray tables must be non-null");
  OptP o;
  rc = make_opt(opt, &o);
  if (rc) return rc;
  const GridP g = make_grid(grid);
  const double diag = std::sqrt((double)g.size[0] * g.size[0] + (double)g.size[1] * g.size[1] +
                                (double)g.size[2] * g.size[2]);
  const double max_samples = diag / (double)o.step + 2.0;
  SVX_REQUIRE(max_samples <= (double)kNumCkpt * kMaxStride, SVX_ERR_TOO_LARGE,
              "up to %.0f samples per ray (grid diagonal / step_size); the adjoint supports %d", max_samples,
              kNumCkpt * kMaxStride);
  const int need_words = 1;  // the ray counter
  SVX_REQUIRE(need_words <= kStaticScratchWords, SVX_ERR_TOO_LARGE,
              "needs %d words of static scratch, the array holds %d", need_words, kStaticScratchWords);
  unsigned long long* scratch = nullptr;
  rc = static_scratch_address(&scratch);
  if (rc) return rc;
  IoP io{};
  io.rgb_out = rgb_out;
  io.rgb_gt = rgb_gt;
  io.grad_density = grads->grad_density_out;
  io.grad_sh = grads->grad_sh_out;
  io.mask = grads->mask_out;
  io.norm = 2.f / (float)(3 * (long long)rays->n_rays);
  io.beta = beta_loss / (float)rays->n_rays;
  io.sparsity = sparsity_loss;
  io.origins = rays->origins;
  io.dirs = rays->dirs;
  io.n_rays = rays->n_rays;
  io.eval_count = stats ? reinterpret_cast<unsigned long long*>(stats->eval_samples) : nullptr;
  io.trace = stats ? reinterpret_cast<unsigned long long*>(stats->ray_trace) : nullptr;
  io.cap = g_cap;
  io.work = scratch;  // cleared on the stream by the launch, before the kernel
  return dispatch<kFused, false>(grid, g, o, io, rays->n_rays, as_stream(stream));
}
