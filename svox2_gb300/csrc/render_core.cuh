// Device side of the ray march: parameters, per-ray setup, the 32-sample segment march, cell
// runs and colours, the gradient flushes, and the render kernel template with its launcher.
// Shared by render.cu (grids without a background) and render_bg.cu (grids with the MSI
// background model), which compile their instantiations in parallel.
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
#pragma once
#include "common.cuh"

#include <climits>
#include <type_traits>
#include <cmath>
#include <map>
#include <mutex>
#include <utility>

namespace svx {
namespace rk {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kThreads = 128;
constexpr int kWarps = kThreads / 32;
constexpr int kNumCkpt = 64;   // stored segment checkpoints per ray before thinning
constexpr int kMaxStride = 64; // checkpoint thinning limit: 64*64 segments per ray
// samples per ray the adjoint's checkpoints cover: kNumCkpt checkpoints, each at most kMaxStride
// segments (of 32 samples) that hold evaluated samples apart
constexpr int kMaxAdjointSamples = kNumCkpt * kMaxStride * 32;
// shared-memory colour cache (launches without a global one): 48 entries of 16 bytes keep the
// adjoint instantiations at four blocks per SM
constexpr int kDefaultCap = 48;
constexpr int kGlobalCapMax = 4096;  // global colour cache: samples per ray, at most
constexpr int kAdjointBlocksPerSm = 4;  // __launch_bounds__ of the adjoint instantiations
constexpr long long kSortMinRays = 1 << 15;  // batches below this run in input order

enum Mode { kFwd = 0, kFused = 1, kBwd = 2, kFusedFwd = 3, kFusedRev = 4 };
// kFusedFwd / kFusedRev: the fused step (or the plain backward) as two kernels.  kFusedFwd runs
// the forward march and the adjoint's seed (the MSE residual, or the given grad_out; with the MSI
// background also the background's forward and adjoint) and writes, per ray, a record: the seed
// and, for every evaluated sample, its colour, the log transmittance before it, its t and sigma;
// kFusedRev runs the foreground's reverse pass from the records, without marching again.  Each
// kernel is about half of kFused's code and fits six blocks per SM.

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
  float* accum;    // optional padded gradient rows [n_voxels][accum_stride] (SH coefficients, density, 0s)
  int accum_stride;
  const int* order;            // optional processing order of the rays (a permutation)
  const svx_batch_grid_t* batch_grids;  // batch mode: per-grid descriptors (device)
  const int32_t* ray_grid;              // batch mode: grid of each ray (device)
  const long long* n_rays_dev;          // batch mode: ray count, read on the device
  unsigned long long* work;    // ray counter (zeroed by the host)
  unsigned long long* eval_count;
  unsigned long long* trace;
  int cap;         // colour cache (or, two-kernel step, record) capacity: samples per ray
  float* gcol;     // optional colour cache in global memory: one slice per resident warp (in the
                   // two-kernel step's forward, the MSI background's shells only)
  long long gcol_warps;  // slices in gcol (warps of the launch)
  int gcol_bg;     // background shells each slice also holds (4 float4 each, after the cap entries)
  float4* rec;     // kFusedFwd / kFusedRev: one record of rec_stride entries per ray position
  long long rec_stride;  // 2 + cap + cap / 2 (header, colour entries, (t, sigma) pairs)
  // kFusedFwd of a batch launch: rays with more evaluated samples than a record holds are listed
  // here (ray indices) for the one-kernel step; null where cap bounds every ray
  unsigned long long* ovf_count;
  int* ovf_list;
  // MSI background (grids that have one; render_kernel<..., BG = true>)
  const int32_t* bg_links;     // [2 reso, reso]
  const float* bg_data;        // [bg_cap, bg_nl, 4], rows 16-byte aligned
  long long bg_cap;
  int bg_reso, bg_nl;
  float* grad_bg;              // optional [bg_cap, bg_nl, 4]
  uint8_t* mask_bg;            // optional [bg_cap, bg_nl]
  unsigned long long* bg_eval_count;  // optional: += background samples
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
// Out of line with scalar arguments: only accelerated grids take this path, and keeping it out
// of the march's three inlined copies shortens the fused kernel.
static __device__ __noinline__ float skip_dist(int32_t link, int l0, int l1, int l2, float p0, float p1, float p2,
                                        float d0, float d1, float d2) {
  const int l[3] = {l0, l1, l2};
  const float pos[3] = {p0, p1, p2}, d[3] = {d0, d1, d2};
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

// Per-segment cell runs: consecutive evaluated samples in the same cell share
// one slot.  Slot 0 carries the previous segment's last cell (forward pass);
// slots 1..32 hold this segment's runs.
constexpr int kSlots = 33;
constexpr int kSlotStride = 33;  // floats per slot (odd: lanes reading different slots hit different banks)

// Floats per slot by mode: the forward kernels keep 24 colour values a slot (8 corners x 3
// groups), the adjoint 32 gradient sums (4 groups x 8 corners); both strides are odd, so lanes
// reading different slots hit different banks.  The forward kernels also carve no run-walk
// array.
__host__ __device__ constexpr int slot_stride(int mode) { return (mode == kFwd || mode == kFusedFwd) ? 25 : kSlotStride; }
__host__ __device__ constexpr bool has_walk(int mode) { return !(mode == kFwd || mode == kFusedFwd); }
// The adjoint modes that keep segment checkpoints in shared memory (the two-kernel step needs
// none: its reverse kernel reads every evaluated sample from the record).
__host__ __device__ constexpr bool ck_in_smem(int mode) { return mode == kFused || mode == kBwd; }

// Coefficient rows gathered per pass.  Rows are copied into shared memory with cp.async, all rows
// of a pass in flight at once (one memory round trip per pass, no registers held): 32 rows for
// the adjoint instantiations.  The forward ones at six blocks per SM take 12 FP32 rows (30 floats
// each) or 24 16-bit rows (14 words each): their blocks then fit the 196 KB shared-memory
// carve-out and leave 60 KB of the SM's 256 KB to L1, which holds the row copies and gathers in
// flight (FP32 forward 7% faster than with 23 rows and 28 KB of L1; the same 12-row layout
// padded into the 228 KB carve-out is 12% slower, with more memory-pipe stalls).  At five blocks
// per SM (the MSI background's and the batch launch's forward, five: true) 24 FP32 rows fit the
// same carve-out, and fewer passes per segment count for more with fewer warps to hide them.
// The reverse kernel of the two-kernel fused step gathers no rows (its colours are in the
// records): 0, and no row tables.
template <typename ShT, int MODE, bool five = false>
__host__ __device__ constexpr int tile_rows() {
  return (MODE == kFwd || MODE == kFusedFwd) ? (std::is_same<ShT, float>::value && !five ? 12 : 24)
         : MODE == kFusedRev                 ? 0
                                             : 32;
}

// 4-byte words a 16-bit row of C coefficients can span (it starts on a 2-byte boundary).
__host__ __device__ constexpr int row_words16(int C) { return C / 2 + 1; }
constexpr int kMaxRows = 8 * 32; // corner rows a segment can need

// Retiring corner rows the adjoint lists before a flush pass: 64, and 32 in the reverse kernel
// of the two-kernel step, whose shared memory then fits eight blocks per SM (27 KB a block).
// The forward kernels flush nothing.
__host__ __device__ constexpr int flush_cap(int mode) {
  return (mode == kFwd || mode == kFusedFwd) ? 0 : mode == kFusedRev ? 32 : 64;
}

// Floats between FP32 rows in the tile: C rounded up to an odd number of 8-byte words, so a lane
// reads its row as float2 words and the 16 lanes of each half-warp hit distinct banks (30 floats
// for SH9: 14 shared loads a row instead of 27).
__host__ __device__ constexpr int row_stride32(int C) { return (((C + 1) >> 1) | 1) << 1; }

// Floats a tile row takes for SH storage ShT.
template <typename ShT>
__host__ __device__ constexpr int tile_row_floats(int C) {
  return std::is_same<ShT, float>::value ? row_stride32(C) : row_words16(C);
}

// rs: floats a tile row takes; fc: the flush list's rows (4 sums and a link each), which reuse the
// tile.  A multiple of 4 floats: the corner links and optical depths carved after the tile are
// moved as int4 / float4 words.
__host__ __device__ constexpr int tile_floats(int rs, int rows, int fc) {
  return ((rows * rs > fc * 5 ? rows * rs : fc * 5) + 3) & ~3;
}

struct WarpSmem {
  int* links;        // [32][8] corner links of the staged samples
  float* slot;       // [kSlots][slot stride]: D[j*3+g] (colour pass) or B[g*8+j] (adjoint)
  float* tile;       // [rows][row stride] gathered coefficient rows (16-byte aligned); in the
                     // adjoint, the flush list
  int* rowlink;      // [kMaxRows] link of each row to gather
  short* rowdst;     // [kMaxRows] slot*8 + corner of each row
  int* run_lane;     // [kSlots] first lane of each run
  int* run_l;        // [kSlots][3] cell of each run
  unsigned char* run_need;  // [kSlots] colour pass: corners the run gathers (bit mask)
  signed char* run_delta;   // [kSlots] colour pass: index offset (-7..7) of a shared corner in the
                            // previous run
  int* run_walk;     // [kSlots] adjoint: each run's transition from the run after it (walk_info)
                     // (none in the forward kernels)
  float* pc;         // [32] forward kernels' march: the segment's optical depths (0 where not
                     // evaluated), right after links
  float* ck_t;       // [kNumCkpt]
  float* ck_lt;      // [kNumCkpt]
  int* ck_idx;       // [kNumCkpt]
  float* tmp_t;      // [kMaxStride]
  float* tmp_lt;
  int* tmp_idx;
  float* basis;      // [12] SH basis of the current ray
  float* col;        // [cap][4] colour cache entries (16-byte aligned)
};

// What a warp's slice of shared memory holds in one instantiation; the host sizes the slice and
// the kernel carves it from the same description.
struct SmemLayout {
  int rs;     // floats a tile row takes
  int rows;   // tile rows (0: no row tables)
  int fc;     // flush-list rows
  int ss;     // floats per slot
  int cap;    // colour-cache samples in shared memory
  bool ckpt;  // the reverse pass's checkpoint arrays (the one-kernel adjoint)
  bool walk;  // the run-walk array (adjoint)
  bool plan;  // run_need / run_delta (colour pass)
  bool pc;    // the optical depths of the forward kernels' march
};

template <typename ShT, int MODE, bool five>
__host__ __device__ constexpr SmemLayout smem_layout(int C, int cap) {
  return SmemLayout{tile_row_floats<ShT>(C), tile_rows<ShT, MODE, five>(), flush_cap(MODE), slot_stride(MODE), cap,
                    ck_in_smem(MODE), has_walk(MODE), MODE != kFusedRev, MODE == kFwd || MODE == kFusedFwd};
}

__host__ __device__ constexpr int warp_smem_floats(const SmemLayout& L) {
  return (tile_floats(L.rs, L.rows, L.fc) + 32 * 8 + (L.pc ? 32 : 0) + kSlots * L.ss +
          (L.rows > 0 ? kMaxRows + kMaxRows / 2 : 0) + kSlots * (L.walk ? 5 : 4) + (L.plan ? (2 * kSlots + 3) / 4 : 0) +
          (L.ckpt ? 3 * kNumCkpt + 3 * kMaxStride : 0) + 16 + 4 * L.cap + 3) & ~3;
}

__host__ __device__ __forceinline__ WarpSmem carve(float* base, const SmemLayout& L) {
  WarpSmem s;
  const int nrow = L.rows > 0 ? kMaxRows : 0;
  // the tile first: the warp's base is 16-byte aligned (warp_smem_floats is a multiple of 4)
  s.tile = base;
  s.links = reinterpret_cast<int*>(base + tile_floats(L.rs, L.rows, L.fc));
  s.pc = L.pc ? reinterpret_cast<float*>(s.links + 32 * 8) : nullptr;
  s.slot = reinterpret_cast<float*>(s.links + 32 * 8) + (L.pc ? 32 : 0);
  s.rowlink = reinterpret_cast<int*>(s.slot + kSlots * L.ss);
  s.rowdst = reinterpret_cast<short*>(s.rowlink + nrow);
  s.run_lane = s.rowlink + nrow + nrow / 2;
  s.run_l = s.run_lane + kSlots;
  s.run_walk = L.walk ? s.run_l + 3 * kSlots : nullptr;
  int* after = s.run_l + 3 * kSlots + (L.walk ? kSlots : 0);
  s.run_need = L.plan ? reinterpret_cast<unsigned char*>(after) : nullptr;
  s.run_delta = L.plan ? reinterpret_cast<signed char*>(after) + kSlots : nullptr;
  s.ck_t = reinterpret_cast<float*>(after + (L.plan ? (2 * kSlots + 3) / 4 : 0));
  s.ck_lt = s.ck_t + kNumCkpt;
  s.ck_idx = reinterpret_cast<int*>(s.ck_lt + kNumCkpt);
  s.tmp_t = reinterpret_cast<float*>(s.ck_idx + kNumCkpt);
  s.tmp_lt = s.tmp_t + kMaxStride;
  s.tmp_idx = reinterpret_cast<int*>(s.tmp_lt + kMaxStride);
  s.basis = L.ckpt ? reinterpret_cast<float*>(s.tmp_idx + kMaxStride) : s.ck_t;
  s.col = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(s.basis + 12) + 15) & ~(uintptr_t)15);
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
  long long base;   // linear index of the cell
  float t;          // the sample's t
  float sigma, pcnt, ws, lt_before, lt_after;
};

// SCAN (the forward-only instantiations): every lane forms its own log transmittance from the
// segment's optical depths, broadcast through shared memory (slinks + 256, the pc array), by the
// same subtractions in the same order as the serial chain (a sample that is not evaluated
// contributes 0, and x - 0 == x), so the values are identical; the lanes run the chain in
// parallel instead of one shuffle per evaluated sample.  The adjoint instantiations keep the
// serial chain: the scan's extra code slows the fused kernel, which waits on instruction fetch.
// replay (the adjoint, for a segment whose samples the colour cache holds): the log
// transmittance before each evaluated sample is the forward's, read from the cache entry of the
// sample (its index: idx0 plus the evaluated samples before it in the segment), and the
// forward's early stop is where its count of evaluated samples, n_total, ends; the serial chain
// of subtractions is not run again.  lt_after = lt_before - pcnt is the forward's same operation.
template <bool SCAN = false>
__device__ __forceinline__ void march_segment(Seg& s, float t0, float lt0, const RayGeo& r,
                                              const GridP& g, const OptP& opt, int* slinks,
                                              unsigned long long* trace_h, int lane,
                                              const float4* replay = nullptr, int idx0 = 0, int n_total = 0) {
  __syncwarp();  // every lane is done with the previous segment's staged links
  // Sample t: the reference adds step to t once per sample (trace_ray_cuvol's t += step).
  // Lane k's value of that chain equals the single-rounded t0 + k*step whenever every add
  // in the chain is exact; each lane checks its own link of the chain and the warp falls
  // back to the explicit sequence of adds if any is not.
  float tk = fmaf((float)lane, opt.step, t0);
  {
    const float prev = __shfl_up_sync(kFull, tk, 1);
    const bool ok = lane == 0 ? (tk == t0) : (__fadd_rn(prev, opt.step) == tk);
    if (!__all_sync(kFull, ok)) {
      tk = t0;
#pragma unroll 1
      for (int i = 0; i < lane; ++i) tk = __fadd_rn(tk, opt.step);  // rare: kept compact
    }
  }
  const bool valid = tk <= r.tmax;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    float p = fmaf(tk, r.d[j], r.o[j]);
    p = fminf(fmaxf(p, 0.f), (float)g.size[j] - 1.f);
    s.l[j] = min((int)p, g.size[j] - 2);
    s.pos[j] = __fsub_rn(p, (float)s.l[j]);
  }
  const long long base = (long long)s.l[0] * g.offx + (long long)s.l[1] * g.offy + s.l[2];
  s.base = base;
  const int32_t* lp = g.links + base;
  // all 8 corner links in one round trip (the cell is inside the grid for every lane)
  int lk[8];
  if (valid) {
    lk[0] = __ldg(lp);
    lk[1] = __ldg(lp + 1);
    lk[2] = __ldg(lp + g.offy);
    lk[3] = __ldg(lp + g.offy + 1);
    lk[4] = __ldg(lp + g.offx);
    lk[5] = __ldg(lp + g.offx + 1);
    lk[6] = __ldg(lp + g.offx + g.offy);
    lk[7] = __ldg(lp + g.offx + g.offy + 1);
  } else {
#pragma unroll
    for (int j = 0; j < 8; ++j) lk[j] = -1;
  }
  float skip = 0.f;
  if (valid && lk[0] < -1)
    skip = skip_dist(lk[0], s.l[0], s.l[1], s.l[2], s.pos[0], s.pos[1], s.pos[2], r.d[0], r.d[1], r.d[2]);
  const bool is_skip = valid && skip >= opt.step;
  const unsigned cut = __ballot_sync(kFull, !valid || is_skip);
  s.n = cut ? __ffs(cut) - 1 : 32;
  const bool normal = lane < s.n;

  float sigma = 0.f;
  if (normal) {
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
  s.t = tk;
  s.sigma = sigma;
  // last_sample_opaque: the final sample gets an infinite world step (cuvol.cu:79-81).
  s.ws = (opt.last_opaque && __fadd_rn(tk, opt.step) > r.tmax) ? 1e9f : r.world_step;
  s.pcnt = __fmul_rn(s.ws, sigma);
  unsigned evm = __ballot_sync(kFull, normal && sigma > opt.sigma_thresh);

  if (replay != nullptr) {
    const int idx = idx0 + __popc(evm & ((1u << lane) - 1u));
    const bool keep = ((evm >> lane) & 1u) && idx < n_total;
    const unsigned kept = __ballot_sync(kFull, keep);
    s.stopped = kept != evm;
    s.lt_before = keep ? replay[idx].w : 0.f;
    s.lt_after = keep ? __fsub_rn(s.lt_before, s.pcnt) : 0.f;
    s.evm = kept;
    s.n = kept ? 32 - __clz(kept) : 0;
    s.lt_end = 0.f;
    s.end = true;
    s.t_next = 0.f;
    return;
  }

  // Transmittance, evaluated samples in order (cuvol.cu:96-106).  The stop test
  // exp(log T) < stop_thresh is taken as log T < log_stop, log_stop being the
  // smallest float >= ln(stop_thresh).
  float lt = lt0;
  s.lt_before = 0.f;
  s.lt_after = 0.f;
  s.stopped = false;
  if (SCAN) {
    float* spc = reinterpret_cast<float*>(slinks + 32 * 8);
    const bool evl = (evm >> lane) & 1u;
    const float mine = evl ? s.pcnt : 0.f;
    spc[lane] = mine;
    __syncwarp();
    const float4* pc4 = reinterpret_cast<const float4*>(spc);
    float x = lt0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const float4 v = pc4[q];
      const int j = 4 * q;
      x = j + 0 < lane ? __fsub_rn(x, v.x) : x;
      x = j + 1 < lane ? __fsub_rn(x, v.y) : x;
      x = j + 2 < lane ? __fsub_rn(x, v.z) : x;
      x = j + 3 < lane ? __fsub_rn(x, v.w) : x;
    }
    __syncwarp();
    const float xa = __fsub_rn(x, mine);
    const unsigned sb = __ballot_sync(kFull, evl && xa < opt.log_stop);
    if (sb) {
      const int i = __ffs(sb) - 1;
      s.stopped = true;
      s.n = i + 1;
      evm &= (i == 31) ? kFull : ((2u << i) - 1u);
      lt = __shfl_sync(kFull, xa, i);
    } else if (evm) {
      lt = __shfl_sync(kFull, xa, 31 - __clz(evm));
    }
    if ((evm >> lane) & 1u) {
      s.lt_before = x;
      s.lt_after = xa;
    }
  } else {
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

// The reverse kernel of the two-kernel step reads its samples from the ray's record instead of
// marching again: evaluated samples c0 .. c0 + 31 (those below n_eval), each with the t and sigma
// and the log transmittance before it that the forward kernel stored.  From t it forms the grid
// position, cell and corner weights with the forward's operations, and loads the cell's corner
// links (for the gradient flush); sigma needs no density gathers.  Fills the fields of Seg the
// adjoint reads; evm holds the lanes with a sample.
__device__ __forceinline__ void record_chunk(Seg& s, const float4* ent, const float2* tsig, int c0, int n_eval,
                                             const RayGeo& r, const GridP& g, const OptP& opt, int* slinks,
                                             int lane) {
  __syncwarp();  // every lane is done with the previous chunk's staged links
  const int idx = c0 + lane;
  const bool valid = idx < n_eval;
  float tk = 0.f, sigma = 0.f, ltb = 0.f;
  if (valid) {
    const float2 a = tsig[idx];
    tk = a.x;
    sigma = a.y;
    ltb = ent[idx].w;
  }
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    float p = fmaf(tk, r.d[j], r.o[j]);
    p = fminf(fmaxf(p, 0.f), (float)g.size[j] - 1.f);
    s.l[j] = min((int)p, g.size[j] - 2);
    s.pos[j] = __fsub_rn(p, (float)s.l[j]);
  }
  const long long base = (long long)s.l[0] * g.offx + (long long)s.l[1] * g.offy + s.l[2];
  s.base = base;
  if (valid) {
    const int32_t* lp = g.links + base;
    int4* dst = reinterpret_cast<int4*>(slinks + lane * 8);
    dst[0] = make_int4(__ldg(lp), __ldg(lp + 1), __ldg(lp + g.offy), __ldg(lp + g.offy + 1));
    dst[1] = make_int4(__ldg(lp + g.offx), __ldg(lp + g.offx + 1), __ldg(lp + g.offx + g.offy),
                       __ldg(lp + g.offx + g.offy + 1));
  }
  s.t = tk;
  s.sigma = sigma;
  s.ws = (opt.last_opaque && __fadd_rn(tk, opt.step) > r.tmax) ? 1e9f : r.world_step;
  s.pcnt = __fmul_rn(s.ws, sigma);
  s.lt_before = ltb;
  s.lt_after = valid ? __fsub_rn(ltb, s.pcnt) : 0.f;
  s.evm = __ballot_sync(kFull, valid);
  s.n = __popc(s.evm);
  s.stopped = false;
  s.end = true;
  s.t_next = 0.f;
  s.lt_end = 0.f;
}

// Weight of a sample: T * (1 - exp(-sigma * step)) (trace_ray_cuvol, cuvol.cu:92).  The
// factor is evaluated as -expm1(-x), the same quantity without the cancellation that
// 1 - exp(-x) suffers for the small x of thin media (x ~ 1e-4 loses 3-4 digits).
__device__ __forceinline__ float sample_weight(float lt_before, float pcnt) {
  return __fmul_rn(expf(lt_before), -expm1f(-pcnt));
}

// ---------------------------------------------------------------- cell runs and corners

// Corner j of a cell sits at offset (j>>2, (j>>1)&1, j&1) — the reference's link
// order 0, 1, offy, offy+1, offx, ... (render_util.cuh:79-88).  When a ray moves
// from cell a to cell b = a + d with |d| <= 1 per axis, corner j of b is corner
// j + (4 dx + 2 dy + dz) of a unless it lies on a face that d moved across.
__device__ __forceinline__ unsigned new_corner_mask(int dx, int dy, int dz) {
  unsigned m = 0;
  if (dx > 0) m |= 0xF0u;   // corners with x = 1 of b are new
  if (dx < 0) m |= 0x0Fu;   // corners with x = 0
  if (dy > 0) m |= 0xCCu;
  if (dy < 0) m |= 0x33u;
  if (dz > 0) m |= 0xAAu;
  if (dz < 0) m |= 0x55u;
  return m;
}

// The 8 trilinear corner weights of a sample.
__device__ __forceinline__ void corner_weights(float px, float py, float pz, float w[8]) {
  const float ax = __fsub_rn(1.f, px), ay = __fsub_rn(1.f, py), az = __fsub_rn(1.f, pz);
  const float yz00 = __fmul_rn(ay, az), yz01 = __fmul_rn(ay, pz), yz10 = __fmul_rn(py, az),
              yz11 = __fmul_rn(py, pz);
  w[0] = __fmul_rn(yz00, ax);
  w[1] = __fmul_rn(yz01, ax);
  w[2] = __fmul_rn(yz10, ax);
  w[3] = __fmul_rn(yz11, ax);
  w[4] = __fmul_rn(yz00, px);
  w[5] = __fmul_rn(yz01, px);
  w[6] = __fmul_rn(yz10, px);
  w[7] = __fmul_rn(yz11, px);
}

// Split the segment's evaluated samples into runs of equal cells.  Returns the
// number of runs; *slot gets the lane's run slot (1..n, or 0 for samples that
// continue the carried cell when have_prev).  Writes run_lane / run_l.
__device__ __forceinline__ int segment_runs(const Seg& s, bool have_prev, long long prev_base,
                                            const WarpSmem& sm, int lane, int* slot) {
  const bool ev = (s.evm >> lane) & 1u;
  const unsigned below = s.evm & ((1u << lane) - 1u);
  const int p = below ? 31 - __clz(below) : 0;
  const long long pb = __shfl_sync(kFull, s.base, p);
  const bool start = ev && (below ? (s.base != pb) : (!have_prev || s.base != prev_base));
  const unsigned R = __ballot_sync(kFull, start);
  const unsigned upto = lane == 31 ? R : (R & ((2u << lane) - 1u));
  *slot = ev ? __popc(upto) : 0;
  if (start) {
    sm.run_lane[*slot] = lane;
    sm.run_l[*slot * 3 + 0] = s.l[0];
    sm.run_l[*slot * 3 + 1] = s.l[1];
    sm.run_l[*slot * 3 + 2] = s.l[2];
  }
  __syncwarp();
  return __popc(R);
}

// Per-corner colour of every run: slot[r][j*3+g] = sum_k basis_k sh[link_j][g*bd+k]
// for runs 1..nR.  Corners shared with the previous run (slot r-1; slot 0 is the
// carried cell when have_prev) are copied, the others gathered: 27 consecutive
// lanes read one voxel's coefficients, 30 lanes reduce 10 rows x 3 groups.
// 4-byte asynchronous copy global -> shared; src_bytes 0 writes a zero without reading.
__device__ __forceinline__ void cp_async4(float* dst, const float* src, int src_bytes) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(d), "l"(src), "r"(src_bytes) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

template <int BD, typename ShT, int TR, int SS>
__device__ __forceinline__ void run_colours(int nR, bool have_prev, const WarpSmem& sm, const float basis[9],
                                            const ShT* __restrict__ sh, int lane) {
  constexpr int C = 3 * BD;
  constexpr int RS = row_stride32(C);
  // lane r-1 plans run r
  unsigned need = 0;
  int delta = 0;
  const int r = lane + 1;
  if (r <= nR) {
    if (r == 1 && !have_prev) {
      need = 0xFFu;
    } else {
      const int dx = sm.run_l[r * 3 + 0] - sm.run_l[(r - 1) * 3 + 0];
      const int dy = sm.run_l[r * 3 + 1] - sm.run_l[(r - 1) * 3 + 1];
      const int dz = sm.run_l[r * 3 + 2] - sm.run_l[(r - 1) * 3 + 2];
      if (abs(dx) > 1 || abs(dy) > 1 || abs(dz) > 1) {
        need = 0xFFu;
      } else {
        need = new_corner_mask(dx, dy, dz);
        delta = 4 * dx + 2 * dy + dz;
      }
    }
    sm.run_need[r] = (unsigned char)need;
    sm.run_delta[r] = (signed char)delta;
  }
  // row table: exclusive prefix of the rows each run gathers
  const int cnt = __popc(need);
  int incl = cnt;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int y = __shfl_up_sync(kFull, incl, d);
    if (lane >= d) incl += y;
  }
  const int M = __shfl_sync(kFull, incl, 31);
  if (r <= nR) {
    int o = incl - cnt;
    const int* lk = sm.links + sm.run_lane[r] * 8;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      if ((need >> j) & 1u) {
        sm.rowlink[o] = lk[j];
        sm.rowdst[o] = (short)(r * 8 + j);
        ++o;
      }
    }
  }
  __syncwarp();
  // gather and reduce, TR rows per pass
  for (int m0 = 0; m0 < M; m0 += TR) {
    const int nrow = min(TR, M - m0);
    if constexpr (std::is_same<ShT, float>::value) {
      // every row of the pass in flight at once: lane k copies coefficient k of each row
      if (lane < C) {
        for (int u = 0; u < nrow; ++u) {
          const int lk = sm.rowlink[m0 + u];
          cp_async4(sm.tile + u * RS + lane, sh + (long long)(lk >= 0 ? lk : 0) * C + lane, lk >= 0 ? 4 : 0);
        }
        cp_async_wait_all();
      }
    } else {
      // 16-bit rows start on 2-byte boundaries: lane w copies the w-th aligned 4-byte word that
      // the row spans.  A row whose last coefficient is the low half of its word copies only
      // that half (2 bytes), so no word reaches past the row into memory the table may not own.
      // A row spans at most 16 words, so the two half-warps copy two rows per step.
      constexpr int W = row_words16(C);
      static_assert(W <= 16, "a 16-bit row must fit a half-warp");
      const int half = lane >> 4, wl = lane & 15;
      if (wl < W) {
        for (int u = half; u < nrow; u += 2) {
          const int lk = sm.rowlink[m0 + u];
          const uintptr_t rb = reinterpret_cast<uintptr_t>(sh + (long long)(lk >= 0 ? lk : 0) * C);
          const int par = (int)(rb >> 1) & 1;  // the row starts in the high half of a word
          const float* wp = reinterpret_cast<const float*>(rb & ~(uintptr_t)3);
          const int nw = (par + C + 1) >> 1;
          const int bytes = (lk < 0 || wl >= nw) ? 0 : ((wl == nw - 1 && ((par + C) & 1)) ? 2 : 4);
          cp_async4(sm.tile + u * W + wl, wp + (bytes ? wl : 0), bytes);
        }
        cp_async_wait_all();
      }
    }
    __syncwarp();
    if (lane < nrow) {
      const int dst = sm.rowdst[m0 + lane];
      float* out = sm.slot + (dst >> 3) * SS + (dst & 7) * 3;
      if constexpr (std::is_same<ShT, float>::value) {
        // the row as float4 words (RS / 4 shared loads instead of C)
        const float2* row4 = reinterpret_cast<const float2*>(sm.tile + lane * RS);
        float acc[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int w = 0; w < (C + 1) / 2; ++w) {
          const float2 v = row4[w];
          const float e[2] = {v.x, v.y};
#pragma unroll
          for (int i = 0; i < 2; ++i) {
            const int k = 2 * w + i;
            if (k < C) acc[k / BD] = fmaf(basis[k % BD], e[i], acc[k / BD]);
          }
        }
#pragma unroll
        for (int gg = 0; gg < 3; ++gg) out[gg] = acc[gg];
      } else {
        const int lk = sm.rowlink[m0 + lane];
        // the table starts on a 4-byte boundary, so a row's half-word parity is that of lk * C
        const unsigned short* row =
            reinterpret_cast<const unsigned short*>(sm.tile + lane * row_words16(C)) + ((lk & C) & 1);
#pragma unroll
        for (int gg = 0; gg < 3; ++gg) {
          float acc = 0.f;
#pragma unroll
          for (int k = 0; k < BD; ++k) acc = fmaf(basis[k], bits16_to_f32<ShT>(row[gg * BD + k]), acc);
          out[gg] = acc;
        }
      }
    }
    __syncwarp();
  }
  // Shared corners, two runs per step: each copy reads a slot that is already complete.  Run q
  // copies from run q - 1 (complete after the previous step); run q + 1 copies a corner that
  // run q shares from where run q got it: run q's own gathered row, or run q - 1.  Two runs a
  // step halve the chain of dependent shared-memory round trips; more runs a step cost more in
  // instructions than they save.
  const int cj = lane >> 2, cg = lane & 3;  // 24 lanes: corner cj, group cg (< 3)
  for (int q = 1; q <= nR; q += 2) {
    const int nd0 = sm.run_need[q], dl0 = sm.run_delta[q];
    const bool two = q + 1 <= nR;
    const int nd1 = two ? sm.run_need[q + 1] : 0xFF, dl1 = two ? sm.run_delta[q + 1] : 0;
    if (cg < 3) {
      if (!((nd0 >> cj) & 1))
        sm.slot[q * SS + cj * 3 + cg] = sm.slot[(q - 1) * SS + (cj + dl0) * 3 + cg];
      if (!((nd1 >> cj) & 1)) {
        const int j = cj + dl1;   // the corner's index in run q
        const int src = ((nd0 >> j) & 1) ? q * SS + j * 3 : (q - 1) * SS + (j + dl0) * 3;
        sm.slot[(q + 1) * SS + cj * 3 + cg] = sm.slot[src + cg];
      }
    }
    __syncwarp();
  }
}

// Colour (before the +0.5 offset) of the lane's sample from its run's corners.
template <int SS>
__device__ __forceinline__ void lane_colour(const WarpSmem& sm, int slot, const float w[8], float col[3]) {
  const float* d = sm.slot + slot * SS;
  float c0 = 0.f, c1 = 0.f, c2 = 0.f;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    c0 = fmaf(w[j], d[j * 3 + 0], c0);
    c1 = fmaf(w[j], d[j * 3 + 1], c1);
    c2 = fmaf(w[j], d[j * 3 + 2], c2);
  }
  col[0] = c0;
  col[1] = c1;
  col[2] = c2;
}

// The adjoint walks a segment's runs last to first, carrying per (group, corner) gradient sums B
// from one run to the one before it.  walk_info precomputes, for every run q in parallel (lane
// q - 1), the transition from the run walked before it (run q + 1, or for q = nR the carried cell
// of the later segment): bits 0-7 the corners of that run that q does not share (they retire),
// bits 8-15 the corners of q that are new, bits 16-20 the corner index shift 4 dx + 2 dy + dz
// (plus 16) of the shared ones, bit 21 set when the cell changes.  A run with no run before it
// in the walk retires nothing.
constexpr int kWalkTrans = 1 << 21;

__device__ __forceinline__ void walk_info(int nR, bool have_b, const int bcell[3], const WarpSmem& sm, int lane) {
  const int q = lane + 1;
  if (q <= nR) {
    const int c0 = sm.run_l[q * 3 + 0], c1 = sm.run_l[q * 3 + 1], c2 = sm.run_l[q * 3 + 2];
    const bool has_prev = q < nR || have_b;
    const int p0 = q < nR ? sm.run_l[(q + 1) * 3 + 0] : bcell[0];
    const int p1 = q < nR ? sm.run_l[(q + 1) * 3 + 1] : bcell[1];
    const int p2 = q < nR ? sm.run_l[(q + 1) * 3 + 2] : bcell[2];
    const int dx = c0 - p0, dy = c1 - p1, dz = c2 - p2;
    int info = 0;
    if (!has_prev || dx != 0 || dy != 0 || dz != 0) {
      const bool near = has_prev && abs(dx) <= 1 && abs(dy) <= 1 && abs(dz) <= 1;
      const unsigned retire = has_prev ? (near ? new_corner_mask(-dx, -dy, -dz) : 0xFFu) : 0u;
      const unsigned fresh = near ? new_corner_mask(dx, dy, dz) : 0xFFu;
      const int delta = near ? 4 * dx + 2 * dy + dz : 0;
      info = kWalkTrans | (int)retire | (int)(fresh << 8) | ((delta + 16) << 16);
    }
    sm.run_walk[q] = info;
  }
  __syncwarp();
}

// The adjoint lists retiring corners (their 4 accumulators and link) in shared
// memory and flushes the list in one pass: per corner row, lanes 0..C-1 add
// basis_k * B[group] to the row's C coefficients (one coalesced atomic add) and
// lane C adds the density gradient and marks the voxel.  Lane L holds B for
// (group L>>3, corner L&7); group 3 is the density.
__device__ __forceinline__ void list_retiring(unsigned retire, float B, int lk_lane, float* fl_val,
                                              int* fl_link, int F, int lane) {
  const int j = lane & 7, grp = lane >> 3;
  if ((retire >> j) & 1u) {
    const int o = F + __popc(retire & ((1u << j) - 1u));
    fl_val[o * 4 + grp] = B;
    if (grp == 0) fl_link[o] = lk_lane;
  }
}

// Vector flush into the padded rows: a padded row (SH coefficients 0..C-1, the density
// at C, then zeros) takes nvec = stride / 4 float4 atomic adds, ceil((C+1)/4) operations
// per corner row instead of C+1 scalar ones (the L2's atomic throughput is counted in
// operations).  The warp flushes 32 / nvec rows per pass: lane = row * nvec + q adds
// channels 4q..4q+3 of its row.  basis: the ray's SH basis in shared memory.
// Four-float atomic add whose result is not read (a reduction, no return value to wait for).
__device__ __forceinline__ void red_add_v4(float4* p, float a, float b, float c, float d) {
  asm volatile("red.relaxed.gpu.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(a), "f"(b), "f"(c), "f"(d)
               : "memory");
}

// The flushes are kept out of line: the fused kernel calls them from six places, and at
// this size its instruction fetch is part of what it waits on (out of line: 7% faster).
template <int BD>
__device__ __noinline__ void flush_list_vec(int F, const float* fl_val, const int* fl_link, const float* basis,
                                               float* __restrict__ accum, int stride, uint8_t* __restrict__ mask,
                                               int lane) {
  constexpr int C = 3 * BD;
  __syncwarp();
  const int nvec = stride >> 2;
  const int per = 32 / nvec;
  const int sub = lane / nvec, q = lane - sub * nvec;
  float coef[4];
  int grp[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const int c = 4 * q + e;
    coef[e] = c < C ? basis[c % BD] : 1.f;
    grp[e] = c < C ? c / BD : (c == C ? 3 : 4);
  }
  for (int f = sub; f - sub < F; f += per) {
    if (sub >= per || f >= F) continue;
    const int lk = fl_link[f];
    if (lk < 0) continue;
    float x[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) x[e] = grp[e] < 4 ? __fmul_rn(coef[e], fl_val[f * 4 + grp[e]]) : 0.f;
    if (x[0] != 0.f || x[1] != 0.f || x[2] != 0.f || x[3] != 0.f)
      red_add_v4(reinterpret_cast<float4*>(accum + (long long)lk * stride) + q, x[0], x[1], x[2], x[3]);
    if (q == 0 && mask != nullptr) mask[lk] = 1;
  }
  __syncwarp();
}

template <int BD>
__device__ __noinline__ void flush_list(int F, const float* fl_val, const int* fl_link, float my_basis,
                                           float* __restrict__ grad_sh, float* __restrict__ grad_density,
                                           uint8_t* __restrict__ mask, int lane) {
  constexpr int C = 3 * BD;
  __syncwarp();
  const int gsel = lane < C ? lane / BD : 3;
  for (int f = 0; f < F; ++f) {
    const int lk = fl_link[f];
    if (lk < 0) continue;
    const float b = fl_val[f * 4 + gsel];
    if (lane < C) {
      if (b != 0.f && grad_sh != nullptr) atomicAdd(grad_sh + (long long)lk * C + lane, __fmul_rn(my_basis, b));
    } else if (lane == C) {
      if (b != 0.f && grad_density != nullptr) atomicAdd(grad_density + lk, b);
      if (mask != nullptr) mask[lk] = 1;
    }
  }
  __syncwarp();
}

// Where a ray's gradients go: the call's buffers, or in a batch, its grid's.
struct GridOut {
  float* grad_density;
  float* grad_sh;
  uint8_t* mask;
  float* accum;
  int accum_stride;
  float norm, beta, sparsity;
};

__device__ __forceinline__ void load_batch_grid(const svx_batch_grid_t* bg, int gi, GridP& g, GridOut& go) {
  const svx_batch_grid_t& d = bg[gi];
  g.density = d.grid.density_data;
  g.sh = d.grid.sh_data;
  g.links = d.grid.links;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    g.size[i] = d.grid.size[i];
    g.offset[i] = d.grid.offset[i];
    g.scaling[i] = d.grid.scaling[i];
  }
  g.offy = d.grid.size[2];
  g.offx = (long long)d.grid.size[1] * d.grid.size[2];
  go.grad_density = d.grads.grad_density_out;
  go.grad_sh = d.grads.grad_sh_out;
  go.mask = d.grads.mask_out;
  go.accum = d.accum;
  go.accum_stride = d.accum_stride;
  go.norm = d.norm;
  go.beta = d.beta;
  go.sparsity = d.sparsity;
}

// ---------------------------------------------------------------- MSI background

// render_background_forward / _backward, render_lerp_kernel_cuvol.cu:386-607, for the light that
// leaves the grid: shell i of n = int(nlayers / step) + 2 has radius n / (n - i - 0.5) in the
// sphere that circumscribes the grid; the ray is sampled at its far intersection with each shell
// of radius >= max(|o x d| + 1e-3, 1), at equirectangular (x, y) and layer (1 - 1/r) nlayers - 0.5,
// and the sample's optical depth is sigma * world_step * (1/r_prev - 1/r).  Here the warp takes
// 32 shells at once, one per lane: every lane locates and gathers its sample (four wrapped
// (x, y) corners, two layers, the four channels in one 16-byte load each), then the
// transmittance is carried through the samples with sigma > 0 in shell order, one subtraction
// each as the reference does, and the early stop cuts the chunk where the reference breaks.
struct BgArgs {
  const int32_t* links;
  const float* data;
  float* grad;
  uint8_t* mask;
  long long cap;
  int reso, nl, n_steps;
  float brightness, log_stop;
  float o[3], d[3];       // ray in the unit-sphere frame, d unit length
  float ws, inner, invr0;  // world step per unit of 1/r, inner radius, 1 / inner
  float q2a, qb, f;        // ConcentricSpheresIntersector terms
};

// The background tables of a ray's grid: the launch's (IoP), or in a batch launch those of the
// ray's grid descriptor (nl == 0: the grid has none).
struct BgSrc {
  const int32_t* links;
  const float* data;
  float* grad;
  uint8_t* mask;
  long long cap;
  int reso, nl;
};

__device__ __forceinline__ void load_batch_bg(const svx_batch_grid_t* bgs, int gi, BgSrc& s) {
  const svx_batch_grid_t& d = bgs[gi];
  s.nl = d.grid.background_nlayers;
  s.links = d.grid.background_links;
  s.data = d.grid.background_data;
  s.cap = d.grid.background_capacity;
  s.reso = d.grid.background_reso;
  s.grad = d.grads.grad_background_out;
  s.mask = d.grads.mask_background_out;
}

// ray_find_bounds_bg, render_util.cuh:630-676 (transform_coord, _get_delta_scale, then the
// sphere frame), _dist_ray_to_origin (cuda_util.cuh:112-119).
__device__ __forceinline__ void bg_setup(BgArgs& b, const float org[3], const float dir[3], const GridP& g,
                                         const OptP& opt, const BgSrc& src) {
  b.links = src.links;
  b.data = src.data;
  b.grad = src.grad;
  b.mask = src.mask;
  b.cap = src.cap;
  b.reso = src.reso;
  b.nl = src.nl;
  b.n_steps = (int)__fdiv_rn((float)src.nl, opt.step) + 2;
  b.brightness = opt.bg;
  b.log_stop = opt.log_stop;
  float o[3], d[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    o[i] = fmaf(org[i], g.scaling[i], g.offset[i]);
    d[i] = __fmul_rn(dir[i], g.scaling[i]);
  }
  const float ds = rnorm3_exact(d[0], d[1], d[2]);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float sc = __fdiv_rn(2.f, (float)g.size[i]);
    o[i] = fmaf(__fadd_rn(o[i], 0.5f), sc, -1.f);
    d[i] = __fmul_rn(__fmul_rn(d[i], ds), sc);
  }
  const float inorm = rnorm3_exact(d[0], d[1], d[2]);
  b.ws = __fmul_rn(ds, inorm);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    b.o[i] = o[i];
    b.d[i] = __fmul_rn(d[i], inorm);
  }
  const float c0 = __fsub_rn(__fmul_rn(b.o[1], b.d[2]), __fmul_rn(b.o[2], b.d[1]));
  const float c1 = __fsub_rn(__fmul_rn(b.o[2], b.d[0]), __fmul_rn(b.o[0], b.d[2]));
  const float c2 = __fsub_rn(__fmul_rn(b.o[0], b.d[1]), __fmul_rn(b.o[1], b.d[0]));
  const double cc = __dadd_rn(__dadd_rn(__dmul_rn((double)c0, (double)c0), __dmul_rn((double)c1, (double)c1)),
                              __dmul_rn((double)c2, (double)c2));
  b.inner = fmaxf(__fadd_rn((float)__dsqrt_rn(cc), 1e-3f), 1.f);
  b.invr0 = __fdiv_rn(1.f, b.inner);
  const Spheres csi(b.o, b.d);
  b.q2a = csi.q2a;
  b.qb = csi.qb;
  b.f = csi.f;
}

// Sample of shell i: false when the shell is inside the inner radius or not hit.  Returns 1/r
// of the sample point, its (x, y, layer) cell and the fractional position in it.  The radius
// n / (n - i - 0.5) is one float division of exact operands (the reference divides in double
// and rounds to float, which differs only where the quotient sits on a float midpoint), and
// 1/|p| is rnorm3df, as the reference's _rnorm computes it.
__device__ __forceinline__ bool bg_sample(const BgArgs& b, int i, float& invr, int l[3], float pos[3]) {
  if (i >= b.n_steps) return false;
  const float r = __fdiv_rn((float)b.n_steps, __fsub_rn((float)(b.n_steps - i), 0.5f));
  if (r < b.inner) return false;
  const float det = __fadd_rn(b.f, __fmul_rn(__fmul_rn(__fmul_rn(2.f, b.q2a), r), r));
  if (det < 0.f) return false;
  const float t = __fdiv_rn(__fadd_rn(-b.qb, __fsqrt_rn(det)), b.q2a);
  float p[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) p[j] = fmaf(t, b.d[j], b.o[j]);
  invr = rnorm3df(p[0], p[1], p[2]);
#pragma unroll
  for (int j = 0; j < 3; ++j) p[j] = __fmul_rn(p[j], invr);
  // _unitvec2equirect, render_util.cuh:482-490 (its double constants make the arithmetic double).
  // y is clamped to [-1, 1] first: rounding can push a unit vector's component a last bit past 1,
  // where asinf is NaN (the reference would carry the NaN into the colour).
  constexpr double kInvPi = 0.31830988618379067154;
  const float lat = asinf(fminf(fmaxf(p[1], -1.f), 1.f)), lon = atan2f(p[0], p[2]);
  pos[0] = (float)__dmul_rn((double)(2 * b.reso), __dadd_rn(0.5, __dmul_rn(__dmul_rn((double)lon, 0.5), kInvPi)));
  pos[1] = (float)__dmul_rn((double)b.reso, __dsub_rn(0.5, __dmul_rn((double)lat, kInvPi)));
  pos[2] = fminf(fmaxf(__fsub_rn(__fmul_rn(__fsub_rn(1.f, invr), (float)b.nl), 0.5f), 0.f), (float)(b.nl - 1));
  l[0] = min((int)pos[0], 2 * b.reso - 1);
  l[1] = min((int)pos[1], b.reso - 1);
  l[2] = min((int)pos[2], b.nl - 2);
#pragma unroll
  for (int j = 0; j < 3; ++j) pos[j] = __fsub_rn(pos[j], (float)l[j]);
  return true;
}

// The four (x, y) corners of a sample's cell, wrapping in both: x at 2 reso, y at reso.
__device__ __forceinline__ void bg_corners(const BgArgs& b, const int l[3], long long u[4]) {
  const int ny = l[1] < b.reso - 1 ? l[1] + 1 : 0, nx = l[0] < 2 * b.reso - 1 ? l[0] + 1 : 0;
  u[0] = (long long)l[0] * b.reso + l[1];
  u[1] = (long long)l[0] * b.reso + ny;
  u[2] = (long long)nx * b.reso + l[1];
  u[3] = (long long)nx * b.reso + ny;
}

// trilerp_bg_one (render_util.cuh:155-189) of the four channels: layers, then y, then x.
// A link past the data's rows reads as empty, like a negative one.
__device__ __forceinline__ void bg_gather(const BgArgs& b, const int l[3], const float pos[3], float v[4],
                                          int lks[4]) {
  long long u[4];
  bg_corners(b, l, u);
  float c[4][4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int lk = __ldg(b.links + u[k]);
    lks[k] = lk;
    float4 lo = make_float4(0.f, 0.f, 0.f, 0.f), hi = lo;
    if (lk >= 0 && lk < b.cap) {
      const float4* q = reinterpret_cast<const float4*>(b.data) + (long long)lk * b.nl + l[2];
      lo = __ldg(q);
      hi = __ldg(q + 1);
    }
    c[k][0] = lerpf(lo.x, hi.x, pos[2]);
    c[k][1] = lerpf(lo.y, hi.y, pos[2]);
    c[k][2] = lerpf(lo.z, hi.z, pos[2]);
    c[k][3] = lerpf(lo.w, hi.w, pos[2]);
  }
#pragma unroll
  for (int ch = 0; ch < 4; ++ch)
    v[ch] = lerpf(lerpf(c[0][ch], c[1][ch], pos[1]), lerpf(c[2][ch], c[3][ch], pos[1]), pos[0]);
}

// One 32-shell chunk: locate and gather each lane's sample, pick 1/r of the previous hit shell,
// and carry the transmittance through the samples with sigma > 0.  On return em holds the
// lanes whose sample counts (before the stop), lt the log transmittance after the chunk.
struct BgChunk {
  bool valid;
  int l[3];
  int lk[4];        // the four (x, y) corners' links
  float pos[3], v[4];
  float width, pcnt, lt_before, lt_after;
  unsigned em;
  bool stopped;
};

// The reverse pass's copy of a chunk's samples: the forward stores, per shell, the sample's
// position in its cell and shell width, its four interpolated channels, its cell and its corner
// links (4 float4, 64 bytes), so the reverse pass reads them instead of intersecting, mapping and
// gathering the shell again.
__device__ __forceinline__ void bg_store(float4* e, const BgChunk& c) {
  e[0] = make_float4(c.pos[0], c.pos[1], c.pos[2], c.width);
  e[1] = make_float4(c.v[0], c.v[1], c.v[2], c.v[3]);
  e[2] = make_float4(__int_as_float(c.l[0]), __int_as_float(c.l[1]), __int_as_float(c.l[2]),
                     __int_as_float((int)c.valid));
  e[3] = make_float4(__int_as_float(c.lk[0]), __int_as_float(c.lk[1]), __int_as_float(c.lk[2]),
                     __int_as_float(c.lk[3]));
}

__device__ __forceinline__ void bg_load(const float4* e, BgChunk& c) {
  const float4 a = e[0], v = e[1], l = e[2], k = e[3];
  c.pos[0] = a.x;
  c.pos[1] = a.y;
  c.pos[2] = a.z;
  c.width = a.w;
  c.v[0] = v.x;
  c.v[1] = v.y;
  c.v[2] = v.z;
  c.v[3] = v.w;
  c.l[0] = __float_as_int(l.x);
  c.l[1] = __float_as_int(l.y);
  c.l[2] = __float_as_int(l.z);
  c.valid = __float_as_int(l.w) != 0;
  c.lk[0] = __float_as_int(k.x);
  c.lk[1] = __float_as_int(k.y);
  c.lk[2] = __float_as_int(k.z);
  c.lk[3] = __float_as_int(k.w);
}

// Locate and gather each lane's sample of the chunk and its shell width (1/r of the previous hit
// shell minus its own, render_background_forward's invr_last).
__device__ __forceinline__ void bg_locate(const BgArgs& b, int i0, int lane, float& invr_carry, BgChunk& c) {
  float invr = 0.f;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    c.l[j] = 0;
    c.pos[j] = 0.f;
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    c.v[j] = 0.f;
    c.lk[j] = -1;
  }
  c.valid = bg_sample(b, i0 + lane, invr, c.l, c.pos);
  if (c.valid) bg_gather(b, c.l, c.pos, c.v, c.lk);
  const unsigned vb = __ballot_sync(kFull, c.valid);
  const unsigned below = vb & ((1u << lane) - 1u);
  const float prev = __shfl_sync(kFull, invr, below ? 31 - __clz(below) : 0);
  const float invr_last = below ? prev : invr_carry;
  if (vb) invr_carry = __shfl_sync(kFull, invr, 31 - __clz(vb));
  c.width = __fsub_rn(invr_last, invr);
}

// Transmittance through the chunk's samples with sigma > 0, from lt (updated).
__device__ __forceinline__ void bg_transmit(const BgArgs& b, int lane, float& lt, BgChunk& c) {
  c.pcnt = __fmul_rn(__fmul_rn(c.width, b.ws), c.v[3]);
  unsigned em = __ballot_sync(kFull, c.valid && c.v[3] > 0.f);
  // Optical depth before and after each counted sample, as a prefix sum over the chunk.  The
  // reference subtracts the samples one by one; the sums differ from that sequence in the last
  // bits only.  The early stop cuts the chunk after the first counted sample whose
  // transmittance falls below the threshold, as the reference's break does.
  const bool mine = (em >> lane) & 1u;
  const float x = mine ? c.pcnt : 0.f;
  float incl = x;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const float y = __shfl_up_sync(kFull, incl, d);
    if (lane >= d) incl = __fadd_rn(incl, y);
  }
  float excl = __shfl_up_sync(kFull, incl, 1);
  if (lane == 0) excl = 0.f;
  c.lt_before = __fsub_rn(lt, excl);
  c.lt_after = __fsub_rn(lt, incl);
  const unsigned under = __ballot_sync(kFull, mine && c.lt_after < b.log_stop);
  c.stopped = under != 0u;
  if (c.stopped) {
    const int k = __ffs(under) - 1;
    em &= (k == 31) ? kFull : ((2u << k) - 1u);
    lt = __shfl_sync(kFull, c.lt_after, k);
  } else {
    lt = __shfl_sync(kFull, c.lt_after, 31);
  }
  c.em = em;
}

// Background colour from log transmittance lt, brightness term included (cuvol.cu:386-476);
// adds the number of samples that counted to *n_samples.
// cache (the adjoint, when its global cache has room for the ray's shells): one 4-float4 entry per
// shell for the reverse pass (bg_store).
__device__ __forceinline__ float3 bg_forward(const BgArgs& b, float lt, int lane, unsigned* n_samples,
                                             float4* cache) {
  float a0 = 0.f, a1 = 0.f, a2 = 0.f;
  float invr_carry = b.invr0;
  for (int i0 = 0; i0 < b.n_steps; i0 += 32) {
    BgChunk c;
    bg_locate(b, i0, lane, invr_carry, c);
    if (cache != nullptr && i0 + lane < b.n_steps) bg_store(cache + 4 * (i0 + lane), c);
    bg_transmit(b, lane, lt, c);
    *n_samples += __popc(c.em);
    if ((c.em >> lane) & 1u) {
      const float w = sample_weight(c.lt_before, c.pcnt);
      a0 = fmaf(w, fmaxf(__fadd_rn(__fmul_rn(c.v[0], kC0), 0.5f), 0.f), a0);
      a1 = fmaf(w, fmaxf(__fadd_rn(__fmul_rn(c.v[1], kC0), 0.5f), 0.f), a1);
      a2 = fmaf(w, fmaxf(__fadd_rn(__fmul_rn(c.v[2], kC0), 0.5f), 0.f), a2);
    }
    if (c.stopped) break;
  }
#pragma unroll
  for (int d = 16; d >= 1; d >>= 1) {
    a0 = __fadd_rn(a0, __shfl_xor_sync(kFull, a0, d));
    a1 = __fadd_rn(a1, __shfl_xor_sync(kFull, a1, d));
    a2 = __fadd_rn(a2, __shfl_xor_sync(kFull, a2, d));
  }
  const float tb = __fmul_rn(expf(lt), b.brightness);
  return make_float3(__fadd_rn(a0, tb), __fadd_rn(a1, tb), __fadd_rn(a2, tb));
}

// render_background_backward (cuvol.cu:478-607): accum is the part of dot(colour, dL/dcolour)
// the background carries; each sample's share w * dot(max(colour, 0), g) comes off it in shell
// order (a prefix sum over the chunk), and the gradients of the four channels of a corner-layer
// row go out as one vector atomic.
// cache: the forward's entries of this ray's shells (bg_forward), or nullptr to locate and gather
// them again.
__device__ __forceinline__ void bg_backward(const BgArgs& b, float lt, float g0, float g1, float g2, float accum,
                                            float sparsity, int lane, const float4* cache) {
  float invr_carry = b.invr0;
  for (int i0 = 0; i0 < b.n_steps; i0 += 32) {
    BgChunk c;
    if (cache != nullptr) {
      if (i0 + lane < b.n_steps) {
        bg_load(cache + 4 * (i0 + lane), c);
      } else {
        c.valid = false;
        c.width = 0.f;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          c.l[j] = 0;
          c.pos[j] = 0.f;
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          c.v[j] = 0.f;
          c.lk[j] = -1;
        }
      }
    } else {
      bg_locate(b, i0, lane, invr_carry, c);
    }
    bg_transmit(b, lane, lt, c);
    const bool on = (c.em >> lane) & 1u;
    const float col0 = __fadd_rn(__fmul_rn(c.v[0], kC0), 0.5f);
    const float col1 = __fadd_rn(__fmul_rn(c.v[1], kC0), 0.5f);
    const float col2 = __fadd_rn(__fmul_rn(c.v[2], kC0), 0.5f);
    const float tc = fmaf(fmaxf(col2, 0.f), g2, fmaf(fmaxf(col1, 0.f), g1, __fmul_rn(fmaxf(col0, 0.f), g0)));
    const float w = on ? sample_weight(c.lt_before, c.pcnt) : 0.f;
    const float x = __fmul_rn(w, tc);
    float incl = x;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const float y = __shfl_up_sync(kFull, incl, d);
      if (lane >= d) incl = __fadd_rn(incl, y);
    }
    const float acc_after = __fsub_rn(accum, incl);
    accum = __fsub_rn(accum, __shfl_sync(kFull, incl, 31));
    if (on && b.grad != nullptr) {
      float gs = __fmul_rn(__fmul_rn(b.ws, c.width), __fsub_rn(__fmul_rn(tc, expf(c.lt_after)), acc_after));
      if (sparsity > 0.f) {
        const float sg = c.v[3];
        gs = fmaf(sparsity, __fdiv_rn(__fmul_rn(4.f, sg), __fadd_rn(1.f, __fmul_rn(2.f, __fmul_rn(sg, sg)))), gs);
      }
      const float cw = __fmul_rn(kC0, w);
      const float gc0 = col0 > 0.f ? __fmul_rn(cw, g0) : 0.f;
      const float gc1 = col1 > 0.f ? __fmul_rn(cw, g1) : 0.f;
      const float gc2 = col2 > 0.f ? __fmul_rn(cw, g2) : 0.f;
      // trilerp_backward_bg_one (render_util.cuh:191-232), the four channels together
      const float ay = __fsub_rn(1.f, c.pos[1]), ax = __fsub_rn(1.f, c.pos[0]), az = __fsub_rn(1.f, c.pos[2]);
      const float wy[4] = {ay, c.pos[1], ay, c.pos[1]};
      const float wx[4] = {ax, ax, c.pos[0], c.pos[0]};
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int lk = c.lk[k];
        if (lk < 0 || lk >= b.cap) continue;
        const float wk = __fmul_rn(wy[k], wx[k]);
        const float e0 = __fmul_rn(wk, gc0), e1 = __fmul_rn(wk, gc1), e2 = __fmul_rn(wk, gc2),
                    e3 = __fmul_rn(wk, gs);
        const long long row = (long long)lk * b.nl + c.l[2];
        float4* q = reinterpret_cast<float4*>(b.grad) + row;
        red_add_v4(q, __fmul_rn(e0, az), __fmul_rn(e1, az), __fmul_rn(e2, az), __fmul_rn(e3, az));
        red_add_v4(q + 1, __fmul_rn(e0, c.pos[2]), __fmul_rn(e1, c.pos[2]), __fmul_rn(e2, c.pos[2]),
                   __fmul_rn(e3, c.pos[2]));
        if (b.mask != nullptr) {
          b.mask[row] = 1;
          b.mask[row + 1] = 1;
        }
      }
    }
    if (c.stopped) break;
  }
}

// ---------------------------------------------------------------- kernel

// The blocks per SM each mode is compiled for: six (80 registers) for the forward kernels, eight
// (64 registers, 84 bytes spilled; 1.2% faster than seven at 72 registers) for the two-kernel
// step's reverse, four (128 registers) for the one-kernel adjoint.  Those with the MSI background
// or of the batch launch keep five (96 registers): at 80 they spill, and the background's forward
// was 3% slower at six.
__host__ __device__ constexpr int blocks_per_sm_bound(int mode, bool multi, bool bg) {
  if (mode == kFwd || mode == kFusedFwd || mode == kFusedRev) return multi || bg ? 5 : mode == kFusedRev ? 8 : 6;
  return kAdjointBlocksPerSm;
}

template <int BD, typename ShT, int MODE, bool IMAGE, bool MULTI, bool BG = false>
// 128 registers and 13.8 KB of shared memory per warp (SH9) let four blocks (16 warps) of the
// one-kernel fused step share an SM; the march is latency-bound, so resident warps count for
// more than the registers a larger budget would save.  The forward kernels and the two-kernel
// step's reverse (no colour cache in shared memory; the forward keeps no checkpoints there, the
// reverse gathers no rows) fit the blocks blocks_per_sm_bound gives them.
__global__ void __launch_bounds__(kThreads, blocks_per_sm_bound(MODE, MULTI, BG)) render_kernel(GridP g0, OptP opt,
                                                                                         IoP io) {
  constexpr int C = 3 * BD;
  constexpr bool kSplit = MODE == kFusedFwd || MODE == kFusedRev;
  extern __shared__ float4 smem4[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  // The adjoint's per-sample colour cache: a slice of io.gcol (global memory, most of it held in
  // L2 between a ray's forward and reverse passes; sized by the host for the grid's longest ray),
  // the ray's record (two-kernel step), or, without either, cap samples in shared memory.
  // Samples past the capacity are gathered again.
  const int scap = (io.gcol != nullptr || kSplit) ? 0 : io.cap;  // samples in the shared-memory cache
  constexpr int TR = tile_rows<ShT, MODE, MULTI || BG>();
  constexpr int SS = slot_stride(MODE);
  constexpr int FC = flush_cap(MODE);
  const SmemLayout lay = smem_layout<ShT, MODE, MULTI || BG>(C, scap);
  float* wbase = reinterpret_cast<float*>(smem4) + (size_t)wib * warp_smem_floats(lay);
  const WarpSmem sm = carve(wbase, lay);
  const long long gslot = (long long)blockIdx.x * kWarps + wib;
  const bool gown = io.gcol != nullptr && gslot < io.gcol_warps;
  // one float4 per evaluated sample: its colour (before the +0.5 offset) and the log
  // transmittance before it
  // (in the two-kernel step the colours go to the ray's record and the slice holds only the
  // MSI background's shells)
  const long long slice = kSplit ? 4ll * io.gcol_bg : (long long)io.cap + 4ll * io.gcol_bg;
  float4* colc = gown ? reinterpret_cast<float4*>(io.gcol) + gslot * slice : reinterpret_cast<float4*>(sm.col);
  // the MSI background's shells, after the colour entries (the adjoint's global cache only)
  float4* bgc = gown && io.gcol_bg > 0 ? (kSplit ? colc : colc + io.cap) : nullptr;
  const int cap = (kSplit || io.gcol == nullptr || gown) ? io.cap : 0;
  const int grp = lane >> 3, cj = lane & 7;
  const long long n_rays = MULTI ? *io.n_rays_dev : io.n_rays;

  unsigned long long evals = 0;
  unsigned bg_evals = 0;   // background samples (grids with the MSI background)
  unsigned long long next = 0;
  if (lane == 0) next = atomicAdd(io.work, 1ull);
  next = __shfl_sync(kFull, next, 0);

  while (next < (unsigned long long)n_rays) {
    const long long pos = (long long)next;   // the ray's position in the processing order
    const long long ray = io.order != nullptr ? (long long)__ldg(io.order + pos) : pos;
    GridP g = g0;
    GridOut go{io.grad_density, io.grad_sh, io.mask, io.accum, io.accum_stride, io.norm, io.beta, io.sparsity};
    if (MULTI) load_batch_grid(io.batch_grids, __ldg(io.ray_grid + ray), g, go);
    BgSrc bsrc;
    if constexpr (BG) {
      if constexpr (MULTI) {
        load_batch_bg(io.batch_grids, __ldg(io.ray_grid + ray), bsrc);
      } else {
        bsrc = BgSrc{io.bg_links, io.bg_data, io.grad_bg, io.mask_bg, io.bg_cap, io.bg_reso, io.bg_nl};
      }
    }
    const ShT* __restrict__ sh = reinterpret_cast<const ShT*>(g.sh);
    if (lane == 0) next = atomicAdd(io.work, 1ull);  // prefetch the following ray
    // two-kernel fused step: the ray's record (by position): a header of 2 entries, the colour
    // entries (cap float4: colour, log transmittance before the sample), then cap float2 (t,
    // sigma) of the evaluated samples
    float4* rec = nullptr;
    float2* tsig_out = nullptr;
    if constexpr (kSplit) {
      rec = io.rec + pos * io.rec_stride;
      colc = rec + 2;
      tsig_out = reinterpret_cast<float2*>(rec + 2 + cap);
    }
    if constexpr (MODE == kFusedRev) {
      if (__float_as_int(rec[1].x) <= 0) {   // no evaluated sample, or a ray left to the one-kernel step
        next = __shfl_sync(kFull, next, 0);
        continue;
      }
    }
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
#pragma unroll
    for (int k = 0; k < BD; ++k)
      if (lane == k) sm.basis[k] = basis[k];
    RayGeo rg;
    find_bounds(rg, org, dir, g, opt);
    unsigned long long th = 1469598103934665603ull;
    unsigned long long* thp = io.trace != nullptr ? &th : nullptr;

    int n_eval = 0, nck = 0, stride = 1;
    float gout0 = 0.f, gout1 = 0.f, gout2 = 0.f;   // d(loss)/d(colour) of the ray
    float carry = 0.f;   // the adjoint's light behind the last sample
    if constexpr (MODE == kFusedRev) {
      // the forward kernel's record: the seed and the evaluated-sample count
      const float4 h0 = rec[0];
      gout0 = h0.x;
      gout1 = h0.y;
      gout2 = h0.z;
      carry = h0.w;
      n_eval = __float_as_int(rec[1].x);
    } else {
    if (!(rg.tmin <= rg.tmax)) {
      if constexpr (!BG) {
        // Ray misses the grid: background only, no gradient (cuvol.cu:42-48, 253-258).
        if (MODE != kBwd && io.rgb_out != nullptr && lane < 3) io.rgb_out[ray * 3 + lane] = opt.bg;
        if (io.trace != nullptr && lane == 0) io.trace[ray] = th;
        if constexpr (MODE == kFusedFwd) {
          if (lane == 0) rec[1] = make_float4(0.f, 0.f, 0.f, 0.f);   // no evaluated sample
        }
        next = __shfl_sync(kFull, next, 0);
        continue;
      }
      // With the MSI background the ray goes on with no foreground: the march below does not
      // run (t > tmax), and the background is rendered, and differentiated, from full
      // transmittance (cuvol.cu:42-48 writes 0, the background kernels add to it, 776-860).
    }

    // ---- forward march
    float t = rg.tmin, lt = 0.f;
    float acc0 = 0.f, acc1 = 0.f, acc2 = 0.f;   // this lane's samples' colour sum
    bool have_prev = false;
    long long prev_base = 0;
    int seg_since_ck = 0;
    bool stopped = false;
    while (t <= rg.tmax) {
      Seg s;
      march_segment<MODE == kFwd || MODE == kFusedFwd>(s, t, lt, rg, g, opt, sm.links, thp, lane);
      if (s.evm) {
        if (MODE != kFwd && MODE != kFusedFwd) {
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
        int slot;
        const int nR = segment_runs(s, have_prev, prev_base, sm, lane, &slot);
        run_colours<BD, ShT, TR, SS>(nR, have_prev, sm, basis, sh, lane);
        const bool ev = (s.evm >> lane) & 1u;
        if (ev) {
          float w8[8], col[3];
          corner_weights(s.pos[0], s.pos[1], s.pos[2], w8);
          lane_colour<SS>(sm, slot, w8, col);
          const float w = sample_weight(s.lt_before, s.pcnt);
          acc0 = fmaf(w, fmaxf(__fadd_rn(col[0], 0.5f), 0.f), acc0);
          acc1 = fmaf(w, fmaxf(__fadd_rn(col[1], 0.5f), 0.f), acc1);
          acc2 = fmaf(w, fmaxf(__fadd_rn(col[2], 0.5f), 0.f), acc2);
          if (MODE != kFwd) {
            const int idx = n_eval + __popc(s.evm & ((1u << lane) - 1u));
            if (idx < cap) {
              colc[idx] = make_float4(col[0], col[1], col[2], s.lt_before);
              if constexpr (MODE == kFusedFwd) tsig_out[idx] = make_float2(s.t, s.sigma);
            }
          }
        }
        // carry the last run to the next segment (after every lane has read the slots)
        const int last = 31 - __clz(s.evm);
        prev_base = __shfl_sync(kFull, s.base, last);
        __syncwarp();
        if (nR > 0) {
          if (lane < 24) sm.slot[(lane >> 3) + 3 * (lane & 7)] = sm.slot[nR * SS + (lane >> 3) + 3 * (lane & 7)];
          if (lane < 3) sm.run_l[lane] = sm.run_l[nR * 3 + lane];
        }
        have_prev = true;
        n_eval += __popc(s.evm);
        __syncwarp();
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
    // colour: this lane's partial sums, reduced over the warp
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) {
      acc0 = __fadd_rn(acc0, __shfl_xor_sync(kFull, acc0, d));
      acc1 = __fadd_rn(acc1, __shfl_xor_sync(kFull, acc1, d));
      acc2 = __fadd_rn(acc2, __shfl_xor_sync(kFull, acc2, d));
    }
    const float lt_fwd = stopped ? -1e3f : lt;   // cuvol.cu:103-106
    // light that passes the last sample: the brightness term, or the MSI background, which the
    // reference renders from the forward's log transmittance (-1e3 after an early stop) and, in
    // the plain backward, from the backward pass's own (cuvol.cu:1040-1066)
    float tb0, tb1, tb2;
    BgArgs bga;
    const float lt_bg = MODE == kBwd ? lt : lt_fwd;
    bool with_bg = false;
    if constexpr (BG) {
      with_bg = bsrc.nl > 0 && lt_bg >= -25.f;   // render_background_kernel's cut
      // a grid without a background (in a batch launch) keeps the brightness term
      tb0 = tb1 = tb2 = bsrc.nl > 0 ? 0.f : __fmul_rn(expf(lt_fwd), opt.bg);
      if (with_bg) {
        bg_setup(bga, org, dir, g, opt, bsrc);
        const float3 c = bg_forward(bga, lt_bg, lane, &bg_evals, bga.n_steps <= io.gcol_bg ? bgc : nullptr);
        tb0 = c.x;
        tb1 = c.y;
        tb2 = c.z;
      }
    } else {
      tb0 = tb1 = tb2 = __fmul_rn(expf(lt_fwd), opt.bg);
    }
    const float tb = tb0;
    const float out0 = __fadd_rn(acc0, tb0), out1 = __fadd_rn(acc1, tb1), out2 = __fadd_rn(acc2, tb2);
    if (MODE != kBwd && io.rgb_out != nullptr && lane == 0) {
      io.rgb_out[ray * 3 + 0] = out0;
      io.rgb_out[ray * 3 + 1] = out1;
      io.rgb_out[ray * 3 + 2] = out2;
    }
    if (io.trace != nullptr && lane == 0) io.trace[ray] = th;

    if (MODE != kFwd) {
      // ---- adjoint seed
      // kFusedFwd serves both the fused step (the residual) and the plain backward (given grad_out)
      if (MODE == kFused || (MODE == kFusedFwd && io.grad_out == nullptr)) {
        // residual of the MSE loss (cuvol.cu:735-741)
        gout0 = __fmul_rn(__fsub_rn(out0, __ldg(io.rgb_gt + ray * 3 + 0)), go.norm);
        gout1 = __fmul_rn(__fsub_rn(out1, __ldg(io.rgb_gt + ray * 3 + 1)), go.norm);
        gout2 = __fmul_rn(__fsub_rn(out2, __ldg(io.rgb_gt + ray * 3 + 2)), go.norm);
      } else {
        gout0 = __ldg(io.grad_out + ray * 3 + 0);
        gout1 = __ldg(io.grad_out + ray * 3 + 1);
        gout2 = __ldg(io.grad_out + ray * 3 + 2);
      }
      // light that passes the last sample: background, plus the beta-loss term (cuvol.cu:259-264)
      if constexpr (BG) {
        carry = fmaf(tb0, gout0, fmaf(tb1, gout1, __fmul_rn(tb2, gout2)));
        if (with_bg)
          bg_backward(bga, lt_bg, gout0, gout1, gout2, carry, go.sparsity, lane,
                      bga.n_steps <= io.gcol_bg ? bgc : nullptr);
      } else {
        carry = __fmul_rn(tb, __fadd_rn(__fadd_rn(gout0, gout1), gout2));
      }
      if ((MODE == kFused || MODE == kFusedFwd) && go.beta > 0.f) {
        const float tin = expf(lt_fwd);
        const double f = 1.0 - (double)tin / __dadd_rn((double)__fsub_rn(1.f, tin), 1e-3);
        carry = __fadd_rn(carry, (float)((double)go.beta * f));
      }
      if constexpr (MODE == kFusedFwd) {
        if (lane == 0) {   // the record's header
          rec[0] = make_float4(gout0, gout1, gout2, carry);
          if (n_eval > cap && io.ovf_list != nullptr) {
            // the record could not hold every sample: the one-kernel step redoes this ray
            rec[1] = make_float4(__int_as_float(-1), 0.f, 0.f, 0.f);
            io.ovf_list[atomicAdd(io.ovf_count, 1ull)] = (int)ray;
          } else {
            rec[1] = make_float4(__int_as_float(n_eval), 0.f, 0.f, 0.f);
          }
        }
      }
    }
    }   // the forward (all modes but kFusedRev)

    if constexpr (MODE == kFused || MODE == kBwd || MODE == kFusedRev) {
      // ---- reverse pass over checkpointed segments
      float B = 0.f;               // lanes <24: colour gradient per (g, corner); 24..31: density
      int lk_lane = -1;            // link of corner (lane & 7) of the tracked cell
      int bcell[3] = {0, 0, 0};
      bool have_b = false;
      // the adjoint of one segment's evaluated samples (s), whose cache entries start at idx0
      auto adjoint_segment = [&](Seg& s, int idx0) {
        int slot;
        const int nR = segment_runs(s, false, 0, sm, lane, &slot);
        const bool ev = (s.evm >> lane) & 1u;
        const int rank = __popc(s.evm & ((1u << lane) - 1u));
        float col[3] = {0.f, 0.f, 0.f};
        float w8[8];
        corner_weights(s.pos[0], s.pos[1], s.pos[2], w8);
        if (kSplit || idx0 + __popc(s.evm) <= cap) {
          if (ev) {
            const float4 e = colc[idx0 + rank];
            col[0] = e.x;
            col[1] = e.y;
            col[2] = e.z;
          }
        } else {
          // colours past the cache: gather again (the two-kernel step's records hold them all)
          if constexpr (TR > 0) {
            run_colours<BD, ShT, TR, SS>(nR, false, sm, basis, sh, lane);
            if (ev) lane_colour<SS>(sm, slot, w8, col);
          }
        }
        // d(loss)/d(colour) pieces, trace_ray_cuvol_backward cuvol.cu:311-344
        const float w = ev ? sample_weight(s.lt_before, s.pcnt) : 0.f;
        const float tn = expf(s.lt_after);
        const float sc0 = __fadd_rn(col[0], 0.5f), sc1 = __fadd_rn(col[1], 0.5f), sc2 = __fadd_rn(col[2], 0.5f);
        const float tc = __fadd_rn(__fadd_rn(__fmul_rn(fmaxf(sc0, 0.f), gout0), __fmul_rn(fmaxf(sc2, 0.f), gout2)),
                                   __fmul_rn(fmaxf(sc1, 0.f), gout1));
        // light after each sample = carry + suffix sum of w * tc over the later samples
        const float v = ev ? __fmul_rn(w, tc) : 0.f;
        float incl = v;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          const float y = __shfl_down_sync(kFull, incl, d);
          if (lane + d < 32) incl = __fadd_rn(incl, y);
        }
        float excl = __shfl_down_sync(kFull, incl, 1);
        if (lane == 31) excl = 0.f;
        const float after = __fadd_rn(carry, excl);
        float gsig = __fmul_rn(s.ws, __fsub_rn(__fmul_rn(tc, tn), after));
        if (go.sparsity > 0.f) {
          const float sg = s.sigma;
          gsig = fmaf(go.sparsity, __fdiv_rn(__fmul_rn(4.f, sg), __fadd_rn(1.f, __fmul_rn(2.f, __fmul_rn(sg, sg)))),
                      gsig);
        }
        carry = __fadd_rn(carry, __shfl_sync(kFull, incl, 0));
        const float a0 = sc0 >= 0.f ? __fmul_rn(w, gout0) : 0.f;
        const float a1 = sc1 >= 0.f ? __fmul_rn(w, gout1) : 0.f;
        const float a2 = sc2 >= 0.f ? __fmul_rn(w, gout2) : 0.f;
        // accumulate per run: slot[r][g*8 + j] (g = 3: density)
        __syncwarp();  // colours read from the slots (re-gather path) are consumed
        for (int q = lane; q < (nR + 1) * SS; q += 32) sm.slot[q] = 0.f;
        __syncwarp();
        if (ev) {
          float* d = sm.slot + slot * SS;
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            atomicAdd(d + 0 * 8 + j, __fmul_rn(w8[j], a0));
            atomicAdd(d + 1 * 8 + j, __fmul_rn(w8[j], a1));
            atomicAdd(d + 2 * 8 + j, __fmul_rn(w8[j], a2));
            atomicAdd(d + 3 * 8 + j, __fmul_rn(w8[j], gsig));
          }
        }
        __syncwarp();
        // walk the runs last to first: merge shared corners, list the others, flush the list
        float* fl_val = sm.tile;
        int* fl_link = reinterpret_cast<int*>(sm.tile + FC * 4);
        int F = 0;
        walk_info(nR, have_b, bcell, sm, lane);
        for (int q = nR; q >= 1; --q) {
          const int info = sm.run_walk[q];
          if (info & kWalkTrans) {
            // old corners not shared with the new cell (those on the faces it moved across) retire
            const unsigned retire = (unsigned)info & 0xFFu;
            if (retire) {
              if (F + 8 > FC) {
                if (go.accum != nullptr)
                  flush_list_vec<BD>(F, fl_val, fl_link, sm.basis, go.accum, go.accum_stride, go.mask, lane);
                else
                  flush_list<BD>(F, fl_val, fl_link, my_basis, go.grad_sh, go.grad_density, go.mask, lane);
                F = 0;
              }
              list_retiring(retire, B, lk_lane, fl_val, fl_link, F, lane);
              F += __popc(retire);
            }
            const bool fresh = (info >> (8 + cj)) & 1;
            const int delta = ((info >> 16) & 31) - 16;
            const float moved = __shfl_sync(kFull, B, fresh ? lane : lane + delta);
            B = fresh ? 0.f : moved;
            lk_lane = sm.links[sm.run_lane[q] * 8 + cj];
          }
          B = __fadd_rn(B, sm.slot[q * SS + lane]);
        }
        if (nR > 0) {
          bcell[0] = sm.run_l[3];
          bcell[1] = sm.run_l[4];
          bcell[2] = sm.run_l[5];
          have_b = true;
        }
        if (go.accum != nullptr)
          flush_list_vec<BD>(F, fl_val, fl_link, sm.basis, go.accum, go.accum_stride, go.mask, lane);
        else
          flush_list<BD>(F, fl_val, fl_link, my_basis, go.grad_sh, go.grad_density, go.mask, lane);
      };
      if constexpr (MODE == kFusedRev) {
        // the ray's evaluated samples, last chunk of 32 first, from the record
        const float4* ent = rec + 2;
        const float2* tsig = reinterpret_cast<const float2*>(rec + 2 + cap);
        for (int c0 = ((n_eval - 1) >> 5) << 5; c0 >= 0; c0 -= 32) {
          Seg s;
          record_chunk(s, ent, tsig, c0, n_eval, rg, g, opt, sm.links, lane);
          adjoint_segment(s, c0);
        }
      } else {
        for (int k = nck - 1; k >= 0; --k) {
          // starts of the evaluated segments this checkpoint covers
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
            while (cnt < stride) {
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
            // segments the colour cache holds replay the forward's transmittance
            const bool cached = idx0 + 32 <= cap;
            march_segment(s, t0, lt0, rg, g, opt, sm.links, nullptr, lane, cached ? colc : nullptr, idx0, n_eval);
            __syncwarp();
            adjoint_segment(s, idx0);
          }
        }
      }
      if (have_b) {
        float* fl_val = sm.tile;
        int* fl_link = reinterpret_cast<int*>(sm.tile + FC * 4);
        list_retiring(0xFFu, B, lk_lane, fl_val, fl_link, 0, lane);
        if (go.accum != nullptr)
          flush_list_vec<BD>(8, fl_val, fl_link, sm.basis, go.accum, go.accum_stride, go.mask, lane);
        else
          flush_list<BD>(8, fl_val, fl_link, my_basis, go.grad_sh, go.grad_density, go.mask, lane);
      }
    }
    __syncwarp();
    next = __shfl_sync(kFull, next, 0);
  }
  if (io.eval_count != nullptr && lane == 0 && evals) atomicAdd(io.eval_count, evals);
  if constexpr (BG) {
    if (io.bg_eval_count != nullptr && lane == 0 && bg_evals)
      atomicAdd(io.bg_eval_count, (unsigned long long)bg_evals);
  }
}

// colour cache capacity (samples per ray) of the adjoint; defined in render.cu
extern int g_cap;

template <int BD, typename ShT, int MODE, bool IMAGE, bool MULTI, bool BG = false>
int launch_t(const GridP& g, const OptP& opt, IoP io, long long n_rays, cudaStream_t st) {
  constexpr int C = 3 * BD;
  auto kern = render_kernel<BD, ShT, MODE, IMAGE, MULTI, BG>;
  const int cap = MODE == kFwd ? 0 : io.cap;
  io.cap = cap;
  if (MODE == kFwd) io.gcol = nullptr;
  const size_t smem =
      sizeof(float) *
      (size_t)warp_smem_floats(
          smem_layout<ShT, MODE, MULTI || BG>(C, (io.gcol != nullptr || MODE == kFusedFwd || MODE == kFusedRev) ? 0 : cap)) *
      kWarps;
  // The function's dynamic shared-memory limit is one attribute per device for every
  // configuration (colour cache in shared or global memory, its capacity), so it is only ever
  // raised, to the largest configuration launched so far; the occupancy each configuration
  // allows is looked up once per (device, configuration).
  static std::mutex mu;
  static std::map<std::pair<int, int>, int> blocks_per_sm;
  static std::map<int, size_t> smem_limit;
  int dev = 0;
  SVX_CUDA_TRY(cudaGetDevice(&dev));
  int bps;
  {
    std::lock_guard<std::mutex> lk(mu);
    size_t& lim = smem_limit[dev];
    if (smem > lim) {
      SVX_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      lim = smem;
    }
    int& slot = blocks_per_sm[std::make_pair(dev, io.gcol != nullptr ? -1 : cap)];
    if (slot == 0) {
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

template <int MODE, bool IMAGE, bool MULTI = false, bool BG = false>
int dispatch_bd(int bd, int dt, const GridP& g, const OptP& opt, const IoP& io, long long n, cudaStream_t st) {
#define SVX_CASE(BDV, T)                                   \
  if (bd == BDV && dt == SvxDt<T>::v) return launch_t<BDV, T, MODE, IMAGE, MULTI, BG>(g, opt, io, n, st);
  SVX_CASE(9, float) SVX_CASE(9, __nv_bfloat16) SVX_CASE(9, __half)
  SVX_CASE(4, float) SVX_CASE(4, __nv_bfloat16) SVX_CASE(4, __half)
  SVX_CASE(1, float) SVX_CASE(1, __nv_bfloat16) SVX_CASE(1, __half)
#undef SVX_CASE
  set_error("unsupported basis_dim %d / sh dtype %d", bd, dt);
  return SVX_ERR_UNSUPPORTED;
}

// Launches the render kernel of a grid with the MSI background (render_bg.cu).
int dispatch_bg(int mode, bool image, int bd, int dt, const GridP& g, const OptP& opt, const IoP& io,
                long long n, cudaStream_t st);
// Launches the forward kernel of the two-kernel fused step (SH9) for a grid with the MSI
// background (render_bg.cu); its reverse kernel is the one without the background.
int launch_bg_split_fwd(int dt, const GridP& g, const OptP& opt, const IoP& io, long long n, cudaStream_t st);
// Launches the batch kernel (SH9) whose grids may have an MSI background (render_bg.cu).
int dispatch_bg_batch(int mode, int dt, const GridP& g, const OptP& opt, const IoP& io, long long n,
                      cudaStream_t st);

}  // namespace rk
}  // namespace svx
