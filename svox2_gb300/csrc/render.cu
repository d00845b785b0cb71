// Ray march, fused MSE adjoint and image render for the `cuvol` backend: host side,
// and the instantiations for grids without the MSI background (render_bg.cu holds those
// with it).  The kernel template itself is in render_core.cuh.
//
// Replaces svox2/csrc/render_lerp_kernel_cuvol.cu (trace_ray_cuvol 30-120,
// trace_ray_cuvol_backward 227-383, kernels 611-773, host 918-1152) with one
// kernel template and three modes:
//   kFwd   volume_render_cuvol / volume_render_cuvol_image
//   kFused volume_render_cuvol_fused   (forward, MSE residual, adjoint)
//   kBwd   volume_render_cuvol_backward (forward, given dL/drgb, adjoint)
// plus the depth renders (depth_kernel), grid_weight_render (grid_weight_kernel), the
// coherence ray order and the accumulation-row flush.

#include "render_core.cuh"

#include <cub/cub.cuh>

#include <climits>
#include <cmath>
#include <cstdlib>
#include <map>
#include <mutex>
#include <utility>

namespace svx {
namespace rk {
int g_cap = kDefaultCap;
}  // namespace rk

using namespace rk;

namespace {


// ---------------------------------------------------------------- depth renders

// volume_render_expected_term / volume_render_sigma_thresh (trace_ray_expected_term and
// trace_ray_sigma_thresh, render_lerp_kernel_cuvol.cu:122-225): the ray's expected
// termination distance, sum over evaluated samples of w * (t / step) * world_step, or
// (THRESH) the distance of its first sample with sigma > thr.  Distances are along the
// ray in world units.  One warp per ray, with the forward march's sampling and stop
// rules; last_sample_opaque does not apply here, as in the reference.
template <bool THRESH>
__global__ void __launch_bounds__(kThreads) depth_kernel(GridP g, OptP opt, IoP io, float thr, float* __restrict__ out) {
  __shared__ int slinks[kWarps][32 * 8];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  OptP o = opt;
  o.last_opaque = 0;
  if (THRESH) {  // evaluated = sigma > thr, and no transmittance stop
    o.sigma_thresh = thr;
    o.log_stop = -INFINITY;
  }
  unsigned long long next = 0;
  if (lane == 0) next = atomicAdd(io.work, 1ull);
  next = __shfl_sync(kFull, next, 0);
  while (next < (unsigned long long)io.n_rays) {
    const long long ray = (long long)next;
    if (lane == 0) next = atomicAdd(io.work, 1ull);
    float org[3], dir[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      org[i] = __ldg(io.origins + ray * 3 + i);
      dir[i] = __ldg(io.dirs + ray * 3 + i);
    }
    RayGeo rg;
    find_bounds(rg, org, dir, g, o);
    float acc = 0.f;
    if (rg.tmin <= rg.tmax) {
      float t = rg.tmin, lt = 0.f;
      while (t <= rg.tmax) {
        Seg s;
        march_segment(s, t, lt, rg, g, o, slinks[wib], nullptr, lane);
        if (THRESH) {
          if (s.evm) {
            const float tf = __shfl_sync(kFull, s.t, __ffs(s.evm) - 1);
            acc = lane == 0 ? __fmul_rn(__fdiv_rn(tf, o.step), rg.world_step) : 0.f;
            break;
          }
        } else if ((s.evm >> lane) & 1u) {
          const float w = sample_weight(s.lt_before, s.pcnt);
          acc = fmaf(__fmul_rn(w, __fdiv_rn(s.t, o.step)), rg.world_step, acc);
        }
        lt = s.lt_end;
        if (s.stopped || s.end) break;
        t = s.t_next;
      }
    }
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) acc = __fadd_rn(acc, __shfl_xor_sync(kFull, acc, d));
    if (lane == 0) out[ray] = acc;
    next = __shfl_sync(kFull, next, 0);
  }
}

// ---------------------------------------------------------------- grid weight render

// grid_weight_render (misc_kernel.cu:183-334): every pixel ray of a camera is marched through
// a dense density grid data [X,Y,Z] (the resampled densities); each sample with sigma > 1e-8
// raises grid_weight at its cell's 8 corners to the sample's weight, so grid_weight ends as
// the largest weight any ray gave a voxel.  Weights are >= 0, so the maximum is taken on the
// float bit patterns as integers.  One thread per pixel: the grids are small and the pass
// runs once per camera during resampling.
__global__ void __launch_bounds__(256) grid_weight_kernel(GridP g, OptP opt, IoP io, long long n_pix,
                                                          const float* __restrict__ data,
                                                          float* __restrict__ wmax) {
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n_pix;
       q += (long long)gridDim.x * blockDim.x) {
    float org[3], dir[3];
    camera_ray((int)(q % io.width), (int)(q / io.width), io, dir, org);
    RayGeo r;
    find_bounds(r, org, dir, g, opt);
    if (!(r.tmin <= r.tmax)) continue;
    const long long co[8] = {0, 1, g.offy, g.offy + 1, g.offx, g.offx + 1, g.offx + g.offy, g.offx + g.offy + 1};
    float ll = 0.f, t = r.tmin;
    while (t <= r.tmax) {
      int l[3];
      float pos[3];
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        float p = fmaf(t, r.d[j], r.o[j]);
        p = fminf(fmaxf(p, 0.f), (float)g.size[j] - 1.f);
        l[j] = min((int)p, g.size[j] - 2);
        pos[j] = __fsub_rn(p, (float)l[j]);
      }
      const long long idx = (long long)l[0] * g.offx + (long long)l[1] * g.offy + l[2];
      float v[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) v[j] = __ldg(data + idx + co[j]);
      float sigma = lerpf(lerpf(lerpf(v[0], v[1], pos[2]), lerpf(v[2], v[3], pos[2]), pos[1]),
                          lerpf(lerpf(v[4], v[5], pos[2]), lerpf(v[6], v[7], pos[2]), pos[1]), pos[0]);
      if (opt.last_opaque && __fadd_rn(t, opt.step) > r.tmax) {
        sigma = __fadd_rn(sigma, 1e9f);
        ll = 0.f;
      }
      if (sigma > 1e-8f) {
        const float la = -__fmul_rn(r.world_step, sigma);
        const float w = __fmul_rn(expf(ll), -expm1f(la));
        ll = __fadd_rn(ll, la);
        const int wi = __float_as_int(w);
#pragma unroll
        for (int j = 0; j < 8; ++j) atomicMax(reinterpret_cast<int*>(wmax + idx + co[j]), wi);
        if (ll < opt.log_stop) break;
      }
      t = __fadd_rn(t, opt.step);
    }
  }
}

// ---------------------------------------------------------------- ray order

// Coherence key of a ray: 4 bits of direction (2 x 2 bits of its octahedral map)
// above the 24-bit Morton code of the midpoint of its chord through the grid.
// Rays with equal keys run nearly parallel through the same region, so warps that
// run them at the same time share cached corner rows and gradient lines.  Rays
// that miss the grid sort last.
__device__ __forceinline__ unsigned spread_bits3(unsigned v) {
  v &= 0xFFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

__global__ void __launch_bounds__(256) ray_keys_kernel(GridP g, OptP opt, const float* __restrict__ origins,
                                                       const float* __restrict__ dirs, long long n,
                                                       unsigned* __restrict__ keys, int* __restrict__ vals,
                                                       int base) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    float org[3], dir[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      org[j] = __ldg(origins + i * 3 + j);
      dir[j] = __ldg(dirs + i * 3 + j);
    }
    RayGeo r;
    find_bounds(r, org, dir, g, opt);
    unsigned key = 0xFFFFFFFFu;
    if (r.tmin <= r.tmax) {
      const float tm = 0.5f * (r.tmin + r.tmax);
      unsigned m = 0;
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const float p = fminf(fmaxf(fmaf(tm, r.d[j], r.o[j]) / (float)g.size[j], 0.f), 0.999f);
        m |= spread_bits3((unsigned)(p * 256.f)) << (2 - j);
      }
      const float s = fabsf(r.d[0]) + fabsf(r.d[1]) + fabsf(r.d[2]);
      float u = r.d[0] / s, v = r.d[1] / s;
      if (r.d[2] < 0.f) {
        const float uu = (1.f - fabsf(v)) * (u >= 0.f ? 1.f : -1.f);
        v = (1.f - fabsf(u)) * (v >= 0.f ? 1.f : -1.f);
        u = uu;
      }
      const unsigned qu = min((unsigned)((u + 1.f) * 2.f), 3u), qv = min((unsigned)((v + 1.f) * 2.f), 3u);
      key = ((qu << 2 | qv) << 24) | m;
    }
    keys[i] = key;
    vals[i] = base + (int)i;
  }
}

// ---------------------------------------------------------------- host side

// grad_sh[v, c] += accum[v, c], grad_density[v] += accum[v, C] for rows with any
// non-zero entry (untouched rows keep their exact values).
__global__ void __launch_bounds__(256) add_accum_kernel(const float* __restrict__ accum, int stride, int C,
                                                        long long n, float* __restrict__ grad_sh,
                                                        float* __restrict__ grad_density) {
  const int lane = threadIdx.x & 31;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long v = warp; v < n; v += nwarps) {
    const float x = lane < stride ? accum[v * stride + lane] : 0.f;
    if (__ballot_sync(0xffffffffu, x != 0.f) == 0u) continue;
    if (lane < C && grad_sh != nullptr) grad_sh[v * C + lane] += x;
    if (lane == C && grad_density != nullptr) grad_density[v] += x;
  }
}

// Grids with the MSI background run the kernel instantiations of render_bg.cu.
template <int MODE, bool IMAGE>
int dispatch(const svx_grid_t* grid, const GridP& g, const OptP& opt, const IoP& io, long long n,
             cudaStream_t st) {
  if (grid->background_nlayers > 0) return dispatch_bg(MODE, IMAGE, grid->basis_dim, grid->sh_dtype, g, opt, io, n, st);
  return dispatch_bd<MODE, IMAGE, false>(grid->basis_dim, grid->sh_dtype, g, opt, io, n, st);
}

// The MSI background's tables (svx_grid_t, checked by check_grid) and gradients: the vector
// atomics of the gradient scatter need 16-byte rows, and the shell count must fit an int.
int set_background(IoP& io, const svx_grid_t* grid, const OptP& o, const svx_grid_grads_t* grads) {
  if (grid->background_nlayers <= 0) return SVX_OK;
  SVX_REQUIRE((double)grid->background_nlayers / (double)o.step + 2.0 < (double)(1 << 30), SVX_ERR_TOO_LARGE,
              "background_nlayers / step_size = %g shells per ray is too many",
              (double)grid->background_nlayers / (double)o.step);
  if (grads != nullptr)
    SVX_REQUIRE((reinterpret_cast<uintptr_t>(grads->grad_background_out) & 15u) == 0, SVX_ERR_INVALID,
                "grad_background_out must be 16-byte aligned");
  io.bg_links = grid->background_links;
  io.bg_data = grid->background_data;
  io.bg_cap = grid->background_capacity;
  io.bg_reso = grid->background_reso;
  io.bg_nl = grid->background_nlayers;
  if (grads != nullptr) {
    io.grad_bg = grads->grad_background_out;
    io.mask_bg = grads->mask_background_out;
  }
  return SVX_OK;
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
  SVX_REQUIRE(grid->background_nlayers == 0 || grid->background_nlayers >= 2, SVX_ERR_INVALID,
              "background_nlayers = %d: 0, or at least 2 MSI layers", grid->background_nlayers);
  if (grid->background_nlayers > 0) {
    SVX_REQUIRE(grid->background_links != nullptr && grid->background_data != nullptr, SVX_ERR_INVALID,
                "background tables must be non-null device pointers");
    SVX_REQUIRE(grid->background_reso >= 1, SVX_ERR_INVALID, "background_reso = %d must be >= 1",
                grid->background_reso);
    SVX_REQUIRE(grid->background_capacity >= 0, SVX_ERR_INVALID, "background_capacity < 0");
    SVX_REQUIRE((reinterpret_cast<uintptr_t>(grid->background_data) & 15u) == 0, SVX_ERR_INVALID,
                "background_data must be 16-byte aligned");
    SVX_REQUIRE((long long)2 * grid->background_reso * grid->background_reso < (1ll << 31), SVX_ERR_TOO_LARGE,
                "background_links must have fewer than 2^31 entries");
  }
  SVX_REQUIRE(grid->sh_dtype == SVX_F32 || grid->sh_dtype == SVX_BF16 || grid->sh_dtype == SVX_F16,
              SVX_ERR_INVALID, "sh_dtype %d unknown", grid->sh_dtype);
  // the ray march copies SH rows into shared memory in aligned 4-byte words
  SVX_REQUIRE((reinterpret_cast<uintptr_t>(grid->sh_data) & 3u) == 0, SVX_ERR_INVALID,
              "sh_data must be 4-byte aligned (a 16-bit table must not start at an odd element)");
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

// Per-call scratch: stream-ordered allocations released after the launches.  The
// device's default memory pool keeps freed blocks (release threshold raised once per
// device), so steady-state calls do not go back to the driver.
struct Scratch {
  void* p[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  cudaStream_t st;
  explicit Scratch(cudaStream_t s) : st(s) {}
  int alloc(int i, size_t bytes) {
    const int rc = tune_pool();
    if (rc) return rc;
    SVX_CUDA_TRY(cudaMallocAsync(&p[i], bytes, st));
    return SVX_OK;
  }
  // As alloc, but a pool that cannot supply the bytes is not an error: returns -1, with the CUDA
  // error state cleared, so the caller can take a path that needs less memory.
  int try_alloc(int i, size_t bytes) {
    const int rc = tune_pool();
    if (rc) return rc;
    const cudaError_t e = cudaMallocAsync(&p[i], bytes, st);
    if (e == cudaErrorMemoryAllocation) {
      (void)cudaGetLastError();
      p[i] = nullptr;
      return -1;
    }
    SVX_CUDA_TRY(e);
    return SVX_OK;
  }
  static int tune_pool() {
    static std::mutex mu;
    static bool tuned[64] = {false};
    int dev = 0;
    SVX_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    if (dev >= 0 && dev < 64 && !tuned[dev]) {
      cudaMemPool_t pool;
      SVX_CUDA_TRY(cudaDeviceGetDefaultMemPool(&pool, dev));
      uint64_t thr = ~0ull;
      SVX_CUDA_TRY(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
      tuned[dev] = true;
    }
    return SVX_OK;
  }
  ~Scratch() {
    for (void* q : p)
      if (q) cudaFreeAsync(q, st);
  }
};

// Sorts rays [0, n) by coherence key (ray_keys_kernel) and returns the permutation, offset by
// base, in *order: written to out when it is non-null, else to scratch slot `slot` of scr.
static int coherence_sort(const GridP& g, const OptP& o, const float* origins, const float* dirs, long long n,
                          int base, int* out, Scratch& scr, int slot, int** order) {
  SVX_REQUIRE(n < (1ll << 31) && (long long)base + n <= (1ll << 31), SVX_ERR_TOO_LARGE,
              "%lld rays starting at index %d exceed the int32 order", n, base);
  cudaStream_t st = scr.st;
  size_t tmp_bytes = 0;
  SVX_CUDA_TRY(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, (const unsigned*)nullptr, (unsigned*)nullptr,
                                               (const int*)nullptr, (int*)nullptr, (int)n, 0, 32, st));
  const size_t part = ((size_t)n * 4 + 255) & ~(size_t)255;
  const size_t off_keys2 = part, off_vals = 2 * part, off_vals2 = 3 * part, off_tmp = 4 * part;
  int rc = scr.alloc(slot, off_tmp + tmp_bytes);
  if (rc) return rc;
  char* buf = reinterpret_cast<char*>(scr.p[slot]);
  unsigned* k_in = reinterpret_cast<unsigned*>(buf);
  unsigned* k_out = reinterpret_cast<unsigned*>(buf + off_keys2);
  int* v_in = reinterpret_cast<int*>(buf + off_vals);
  int* v_out = out != nullptr ? out : reinterpret_cast<int*>(buf + off_vals2);
  long long blocks = (n + 255) / 256;
  if (blocks > (long long)num_sms() * 16) blocks = (long long)num_sms() * 16;
  ray_keys_kernel<<<(unsigned)blocks, 256, 0, st>>>(g, o, origins, dirs, n, k_in, v_in, base);
  SVX_LAUNCH_CHECK("ray_keys_kernel");
  SVX_CUDA_TRY(cub::DeviceRadixSort::SortPairs(buf + off_tmp, tmp_bytes, k_in, k_out, v_in, v_out, (int)n, 0, 32,
                                               st));
  *order = v_out;
  return SVX_OK;
}

static int launch_add_accum(const float* accum, int stride, int C, long long n_voxels, float* grad_sh,
                            float* grad_density, cudaStream_t st) {
  if (n_voxels <= 0 || (grad_sh == nullptr && grad_density == nullptr)) return SVX_OK;
  long long blocks = (n_voxels + 7) / 8;
  const long long cap = (long long)num_sms() * 32;
  if (blocks > cap) blocks = cap;
  add_accum_kernel<<<(unsigned)blocks, 256, 0, st>>>(accum, stride, C, n_voxels, grad_sh, grad_density);
  SVX_LAUNCH_CHECK("add_accum_kernel");
  return SVX_OK;
}

// Records the caller's march_start / march_stop event (if any) on the stream.
static int mark(const svx_render_stats_t* stats, bool stop, cudaStream_t st) {
  if (stats == nullptr) return SVX_OK;
  void* ev = stop ? stats->march_stop : stats->march_start;
  if (ev != nullptr) SVX_CUDA_TRY(cudaEventRecord(reinterpret_cast<cudaEvent_t>(ev), st));
  return SVX_OK;
}

// The fused step of an SH9 grid runs as two kernels, the forward (kFusedFwd) and the reverse
// (kFusedRev), with a record per ray between them: 2 + cap float4 entries and cap float2 ones
// (cap = the grid's longest ray in samples, rounded up to 32; 21.5 KB a ray at the 256^3
// workload).  The records of a call
// take at most this many bytes (default 24 GiB: a million rays of the 256^3 workload in one
// chunk); larger calls run in chunks of rays, each chunk both kernels.  SVX_FUSED_SPLIT_BYTES sets
// the budget (0: always the one-kernel fused step).
static long long split_budget_bytes() {
  const char* e = std::getenv("SVX_FUSED_SPLIT_BYTES");
  if (e != nullptr && *e != '\0') return std::atoll(e);
  return 24ll << 30;
}

template <int MODE>
static int launch_sh9(int dt, const GridP& g, const OptP& o, const IoP& io, long long n, cudaStream_t st) {
  switch (dt) {
    case SVX_F32: return launch_t<9, float, MODE, false, false>(g, o, io, n, st);
    case SVX_BF16: return launch_t<9, __nv_bfloat16, MODE, false, false>(g, o, io, n, st);
    case SVX_F16: return launch_t<9, __half, MODE, false, false>(g, o, io, n, st);
  }
  set_error("sh_dtype %d unknown", dt);
  return SVX_ERR_INVALID;
}

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
  double max_samples = 0.0;
  if (MODE != kFwd) {
    // every ray's samples must fit the adjoint's checkpoints (kNumCkpt x kMaxStride segments)
    const double diag = std::sqrt((double)g.size[0] * g.size[0] + (double)g.size[1] * g.size[1] +
                                  (double)g.size[2] * g.size[2]);
    max_samples = diag / (double)o.step + 2.0;
    SVX_REQUIRE(max_samples <= (double)kMaxAdjointSamples, SVX_ERR_TOO_LARGE,
                "up to %.0f samples per ray (grid diagonal / step_size); the adjoint supports %d",
                max_samples, kMaxAdjointSamples);
  }
  io.origins = rays->origins;
  io.dirs = rays->dirs;
  io.n_rays = rays->n_rays;
  io.eval_count = stats ? reinterpret_cast<unsigned long long*>(stats->eval_samples) : nullptr;
  io.trace = stats ? reinterpret_cast<unsigned long long*>(stats->ray_trace) : nullptr;
  io.bg_eval_count = stats ? reinterpret_cast<unsigned long long*>(stats->background_samples) : nullptr;
  io.cap = g_cap;
  rc = set_background(io, grid, o, nullptr);
  if (rc) return rc;
  if (grid->background_nlayers > 0 && io.grad_bg != nullptr)
    SVX_REQUIRE((reinterpret_cast<uintptr_t>(io.grad_bg) & 15u) == 0, SVX_ERR_INVALID,
                "grad_background_out must be 16-byte aligned");
  cudaStream_t st = as_stream(stream);
  Scratch scr(st);
  rc = scr.alloc(0, 256);
  if (rc) return rc;
  io.work = reinterpret_cast<unsigned long long*>(scr.p[0]);
  // the two-kernel form of the fused step and of the plain backward (the latter without the MSI
  // background, whose adjoint there starts from the backward pass's own transmittance): every
  // sample's colour fits the record, and the rays of a chunk are a range of the coherence order
  // (or all of them)
  long long split_chunk = 0, rec_stride = 0;
  if (grid->basis_dim == 9 && (MODE == kFused || (MODE == kBwd && grid->background_nlayers == 0))) {
    const double want = std::ceil(max_samples / 32.0) * 32.0;
    rec_stride = 2 + (long long)want + (long long)want / 2;
    const long long budget = split_budget_bytes();
    const long long chunk = budget / (rec_stride * (long long)sizeof(float4));
    const bool sorted = rays->n_rays >= kSortMinRays && rays->n_rays < (1ll << 31);
    if (want <= (double)kGlobalCapMax && chunk >= 1 && (sorted || chunk >= rays->n_rays))
      split_chunk = std::min<long long>(chunk, rays->n_rays);
    if (split_chunk > 0) {
      // the records; a device that cannot hold them runs the one-kernel step instead
      rc = scr.try_alloc(4, sizeof(float4) * (size_t)rec_stride * (size_t)split_chunk);
      if (rc == -1) {
        split_chunk = 0;
        rc = SVX_OK;
      }
      if (rc) return rc;
    }
  }
  if (split_chunk > 0 && grid->background_nlayers > 0) {
    // the forward kernel's MSI background passes keep their shells in a per-warp slice, as in
    // the one-kernel step (int(nlayers / step) + 2 shells, 4 float4 each)
    io.gcol_warps = (long long)num_sms() * blocks_per_sm_bound(kFusedFwd, false, true) * kWarps;
    io.gcol_bg = (int)((float)grid->background_nlayers / o.step) + 2;
    rc = scr.alloc(3, sizeof(float4) * 4 * (size_t)io.gcol_bg * (size_t)io.gcol_warps);
    if (rc) return rc;
    io.gcol = reinterpret_cast<float*>(scr.p[3]);
  }
  if (MODE != kFwd && split_chunk == 0) {
    // The adjoint's colour cache: one slice per resident warp of the launch (the adjoint
    // instantiations are bounded to kAdjointBlocksPerSm blocks per SM), as long as the grid's
    // longest ray up to kGlobalCapMax samples, 16 bytes per sample.  At the 256^3 workload that
    // is 896 samples, about 35 MB in all, much of it held in L2 between a ray's forward and
    // reverse passes.
    const double want = std::ceil(max_samples / 32.0) * 32.0;
    io.cap = (int)std::min(want, (double)kGlobalCapMax);
    io.gcol_warps = (long long)num_sms() * kAdjointBlocksPerSm * kWarps;
    // with the MSI background, each slice also holds the ray's background shells (4 float4 each):
    // int(nlayers / step) + 2 of them, as the kernel counts them
    io.gcol_bg = grid->background_nlayers > 0 ? (int)((float)grid->background_nlayers / o.step) + 2 : 0;
    rc = scr.alloc(3, sizeof(float4) * (size_t)(io.cap + 4 * io.gcol_bg) * (size_t)io.gcol_warps);
    if (rc) return rc;
    io.gcol = reinterpret_cast<float*>(scr.p[3]);
  }
  const bool grads = MODE != kFwd && (io.grad_sh != nullptr || io.grad_density != nullptr);
  const int C = grid->sh_data_dim;
  const int stride = (C + 1 + 3) & ~3;
  // large batches accumulate into gradient rows padded to 16 bytes with vector atomics, added
  // once at the end; small ones add straight into the gradients with scalar atomics (clearing
  // and adding a table the size of the grid would cost more than the atomics it saves)
  const bool table = grads && rays->n_rays >= kSortMinRays;
  if (table) {
    const size_t bytes = sizeof(float) * (size_t)stride * (size_t)grid->n_voxels;
    rc = scr.alloc(1, bytes > 0 ? bytes : 16);
    if (rc) return rc;
    SVX_CUDA_TRY(cudaMemsetAsync(scr.p[1], 0, bytes, st));
    io.accum = reinterpret_cast<float*>(scr.p[1]);
    io.accum_stride = stride;
  }
  if (rays->n_rays >= kSortMinRays && rays->n_rays < (1ll << 31)) {
    // process the rays in coherence-key order
    int* order = nullptr;
    rc = coherence_sort(g, o, rays->origins, rays->dirs, rays->n_rays, 0, nullptr, scr, 2, &order);
    if (rc) return rc;
    io.order = order;
  }
  rc = mark(stats, false, st);
  if (rc) return rc;
  if (split_chunk > 0) {
    io.cap = (int)((rec_stride - 2) / 3 * 2);
    io.rec_stride = rec_stride;
    io.rec = reinterpret_cast<float4*>(scr.p[4]);
    for (long long c0 = 0; c0 < rays->n_rays; c0 += split_chunk) {
      IoP ioc = io;
      ioc.n_rays = std::min(split_chunk, rays->n_rays - c0);
      if (io.order != nullptr) ioc.order = io.order + c0;
      rc = grid->background_nlayers > 0 ? launch_bg_split_fwd(grid->sh_dtype, g, o, ioc, ioc.n_rays, st)
                                        : launch_sh9<kFusedFwd>(grid->sh_dtype, g, o, ioc, ioc.n_rays, st);
      if (rc) return rc;
      rc = launch_sh9<kFusedRev>(grid->sh_dtype, g, o, ioc, ioc.n_rays, st);
      if (rc) return rc;
    }
  } else {
    rc = dispatch<MODE, false>(grid, g, o, io, rays->n_rays, st);
    if (rc) return rc;
  }
  rc = mark(stats, true, st);
  if (rc) return rc;
  if (table) return launch_add_accum(io.accum, stride, C, grid->n_voxels, io.grad_sh, io.grad_density, st);
  return SVX_OK;
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
  io.grad_bg = grads->grad_background_out;
  io.mask_bg = grads->mask_background_out;
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
  io.grad_bg = grads->grad_background_out;
  io.mask_bg = grads->mask_background_out;
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
  io.bg_eval_count = stats ? reinterpret_cast<unsigned long long*>(stats->background_samples) : nullptr;
  io.cap = 0;
  rc = set_background(io, grid, o, nullptr);
  if (rc) return rc;
  cudaStream_t st = as_stream(stream);
  Scratch scr(st);
  rc = scr.alloc(0, 256);
  if (rc) return rc;
  io.work = reinterpret_cast<unsigned long long*>(scr.p[0]);
  rc = mark(stats, false, st);
  if (rc) return rc;
  rc = dispatch<kFwd, true>(grid, g, o, io, n, st);
  if (rc) return rc;
  return mark(stats, true, st);
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
// needs kNoallocWords of it whatever its size (the counter does not grow with
// the rays or the grid), which the static_assert below holds to the array.
// All calls share the array and it keeps the last call's contents: each call
// clears the counter on its stream before the kernel starts, so calls that
// overlap on the GPU (on different streams, or from different host threads)
// race on the counter and must be serialised by the caller.
constexpr int kStaticScratchWords = 32;
constexpr int kNoallocWords = 1;  // the ray counter
static_assert(kNoallocWords <= kStaticScratchWords, "the allocation-free render's scratch must fit the array");
static __device__ __align__(256) unsigned long long g_static_scratch[kStaticScratchWords];

// Device address of g_static_scratch on the current device, looked up with
// that device current and cached per device.  In host code the symbol's name
// is only a host-side stand-in; the kernel must be given the address
// cudaGetSymbolAddress returns.  The address belongs to the context that was
// current when it was looked up (the runtime's primary context of the
// device): a cached address is checked against the current context with
// cudaPointerGetAttributes on every call and looked up again when that no
// longer reports it as this device's memory (after cudaDeviceReset, or under
// another context).
static int static_scratch_address(unsigned long long** out) {
  static std::mutex mu;
  static unsigned long long* addr[64] = {nullptr};
  int dev = 0;
  SVX_CUDA_TRY(cudaGetDevice(&dev));
  SVX_REQUIRE(dev >= 0 && dev < 64, SVX_ERR_UNSUPPORTED, "device index %d: at most 64 devices", dev);
  std::lock_guard<std::mutex> lk(mu);
  if (addr[dev] != nullptr) {
    cudaPointerAttributes at{};
    const cudaError_t e = cudaPointerGetAttributes(&at, addr[dev]);
    if (e != cudaSuccess) (void)cudaGetLastError();  // a failed query must not reach the launch check
    if (e != cudaSuccess || at.type != cudaMemoryTypeDevice || at.device != dev) addr[dev] = nullptr;
  }
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
  SVX_REQUIRE(max_samples <= (double)kMaxAdjointSamples, SVX_ERR_TOO_LARGE,
              "up to %.0f samples per ray (grid diagonal / step_size); the adjoint supports %d", max_samples,
              kMaxAdjointSamples);
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
  io.bg_eval_count = stats ? reinterpret_cast<unsigned long long*>(stats->background_samples) : nullptr;
  io.cap = g_cap;
  rc = set_background(io, grid, o, grads);
  if (rc) return rc;
  io.work = scratch;  // cleared on the stream by the launch, before the kernel
  cudaStream_t st = as_stream(stream);
  rc = mark(stats, false, st);
  if (rc) return rc;
  rc = dispatch<kFused, false>(grid, g, o, io, rays->n_rays, st);
  if (rc) return rc;
  return mark(stats, true, st);
}

// ---------------------------------------------------------------- serving batches

__global__ void __launch_bounds__(256) camera_rays_kernel(IoP io, long long n, float* __restrict__ origins,
                                                          float* __restrict__ dirs) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    float org[3], dir[3];
    camera_ray((int)(i % io.width), (int)(i / io.width), io, dir, org);
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      origins[i * 3 + j] = org[j];
      dirs[i * 3 + j] = dir[j];
    }
  }
}

extern "C" int svx_camera_rays(const svx_camera_t* cam, float* origins, float* dirs, void* stream) {
  clear_error();
  SVX_REQUIRE(cam != nullptr, SVX_ERR_INVALID, "camera is null");
  SVX_REQUIRE(cam->width >= 0 && cam->height >= 0, SVX_ERR_INVALID, "negative image size");
  SVX_REQUIRE(cam->c2w_rows == 3 || cam->c2w_rows == 4, SVX_ERR_INVALID, "c2w must have 3 or 4 rows");
  const long long n = (long long)cam->width * cam->height;
  if (n == 0) return SVX_OK;
  SVX_REQUIRE(cam->c2w && origins && dirs, SVX_ERR_INVALID, "c2w / origins / dirs are null");
  IoP io{};
  io.c2w = cam->c2w;
  io.fx = cam->fx;
  io.fy = cam->fy;
  io.cx = cam->cx;
  io.cy = cam->cy;
  io.ndcx = cam->ndc_coeffx;
  io.ndcy = cam->ndc_coeffy;
  io.width = cam->width;
  long long blocks = (n + 255) / 256;
  if (blocks > (long long)num_sms() * 16) blocks = (long long)num_sms() * 16;
  camera_rays_kernel<<<(unsigned)blocks, 256, 0, as_stream(stream)>>>(io, n, origins, dirs);
  SVX_LAUNCH_CHECK("camera_rays_kernel");
  return SVX_OK;
}

// The batch launch's kernels (SH9, multi-grid) by SH storage type.
template <int MODE>
static int launch_batch(int dt, const GridP& g, const OptP& o, const IoP& io, long long n, cudaStream_t st) {
  switch (dt) {
    case SVX_F32: return launch_t<9, float, MODE, false, true>(g, o, io, n, st);
    case SVX_BF16: return launch_t<9, __nv_bfloat16, MODE, false, true>(g, o, io, n, st);
    case SVX_F16: return launch_t<9, __half, MODE, false, true>(g, o, io, n, st);
  }
  set_error("sh_dtype %d unknown", dt);
  return SVX_ERR_INVALID;
}

// Bytes before the records in a batch launch's record buffer: the overflow counter (16 bytes) and
// the overflow list (an int32 per ray), rounded up to 16.
static long long batch_record_head(long long max_rays) { return 16 + ((4 * max_rays + 15) & ~15ll); }

extern "C" int svx_render_batch(int32_t mode, const svx_batch_grid_t* grids, int32_t basis_dim, int32_t sh_dtype,
                                int32_t with_background, const float* origins, const float* dirs, const int32_t* ray_grid,
                                const int32_t* order, const int64_t* n_rays_dev, int64_t max_rays,
                                const svx_render_opts_t* opt, const float* rgb_gt, float* rgb_out, uint64_t* work,
                                float* colour_cache, int64_t colour_cache_bytes, void* stream) {
  clear_error();
  SVX_REQUIRE(mode == 0 || mode == 1, SVX_ERR_INVALID, "mode %d: 0 (render) or 1 (fused)", mode);
  SVX_REQUIRE(basis_dim == 9, SVX_ERR_UNSUPPORTED, "batched launches are built for basis_dim 9");
  SVX_REQUIRE(max_rays >= 0, SVX_ERR_INVALID, "max_rays < 0");
  if (max_rays == 0) return SVX_OK;
  SVX_REQUIRE(grids && origins && dirs && ray_grid && n_rays_dev && rgb_out && work, SVX_ERR_INVALID,
              "null batch buffer");
  SVX_REQUIRE(mode == 0 || rgb_gt != nullptr, SVX_ERR_INVALID, "rgb_gt is null");
  OptP o;
  int rc = make_opt(opt, &o);
  if (rc) return rc;
  IoP io{};
  io.origins = origins;
  io.dirs = dirs;
  io.n_rays = max_rays;
  io.rgb_out = rgb_out;
  io.rgb_gt = rgb_gt;
  io.batch_grids = grids;
  io.ray_grid = ray_grid;
  io.order = order;
  io.n_rays_dev = reinterpret_cast<const long long*>(n_rays_dev);
  io.work = reinterpret_cast<unsigned long long*>(work);
  io.cap = g_cap;
  GridP g{};  // per-ray grids come from the descriptors
  cudaStream_t st = as_stream(stream);
  if (mode == 1 && colour_cache != nullptr) {
    SVX_REQUIRE((reinterpret_cast<uintptr_t>(colour_cache) & 15u) == 0, SVX_ERR_INVALID,
                "colour_cache must be 16-byte aligned");
  }
  if (mode == 1 && colour_cache != nullptr && !with_background) {
    // the two-kernel step when the buffer holds a record of at least 64 samples for each of
    // max_rays rays (svx_batch_record_bytes): the overflow counter and list, then the records
    const long long head = batch_record_head(max_rays);
    const long long per = colour_cache_bytes > head ? (colour_cache_bytes - head) / max_rays / 16 : 0;
    const long long cap = std::min<long long>(per > 2 ? ((per - 2) * 2 / 3) & ~31ll : 0, kGlobalCapMax);
    if (cap >= 64) {
      char* base = reinterpret_cast<char*>(colour_cache);
      io.ovf_count = reinterpret_cast<unsigned long long*>(base);
      io.ovf_list = reinterpret_cast<int*>(base + 16);
      io.rec = reinterpret_cast<float4*>(base + head);
      io.rec_stride = 2 + cap + cap / 2;
      io.cap = (int)cap;
      SVX_CUDA_TRY(cudaMemsetAsync(io.ovf_count, 0, sizeof(unsigned long long), st));
      int rc2 = launch_batch<kFusedFwd>(sh_dtype, g, o, io, max_rays, st);
      if (rc2) return rc2;
      rc2 = launch_batch<kFusedRev>(sh_dtype, g, o, io, max_rays, st);
      if (rc2) return rc2;
      // the rays whose samples did not fit their record, in the one-kernel step
      IoP iov = io;
      iov.order = io.ovf_list;
      iov.n_rays_dev = reinterpret_cast<const long long*>(io.ovf_count);
      iov.rec = nullptr;
      iov.ovf_count = nullptr;
      iov.ovf_list = nullptr;
      iov.cap = g_cap;
      return launch_batch<kFused>(sh_dtype, g, o, iov, max_rays, st);
    }
  }
  if (mode == 1 && colour_cache != nullptr) {
    const long long warps = (long long)num_sms() * kAdjointBlocksPerSm * kWarps;
    const long long cap = colour_cache_bytes / (long long)sizeof(float4) / warps;
    if (cap >= 32) {
      io.gcol = colour_cache;
      io.gcol_warps = warps;
      io.cap = (int)std::min<long long>(cap, kGlobalCapMax);
    }
  }
  if (with_background) return dispatch_bg_batch(mode == 0 ? kFwd : kFused, sh_dtype, g, o, io, max_rays, st);
  return mode == 0 ? launch_batch<kFwd>(sh_dtype, g, o, io, max_rays, st)
                   : launch_batch<kFused>(sh_dtype, g, o, io, max_rays, st);
}

extern "C" int64_t svx_batch_record_bytes(int64_t max_rays, int32_t samples_per_ray) {
  if (max_rays <= 0 || samples_per_ray <= 0) return 0;
  const long long cap = std::min<long long>(((long long)samples_per_ray + 31) & ~31ll, kGlobalCapMax);
  return batch_record_head(max_rays) + max_rays * (2 + cap + cap / 2) * 16;
}

extern "C" int64_t svx_batch_colour_cache_bytes(int32_t samples_per_ray) {
  if (samples_per_ray <= 0) return 0;
  return (int64_t)num_sms() * kAdjointBlocksPerSm * kWarps * (int64_t)samples_per_ray * (int64_t)sizeof(float4);
}

extern "C" int svx_ray_order(const svx_grid_t* grid, const svx_rays_t* rays, const svx_render_opts_t* opt,
                             int32_t index_base, int32_t* order_out, void* stream) {
  clear_error();
  int rc = check_grid(grid);
  if (rc) return rc;
  SVX_REQUIRE(rays != nullptr, SVX_ERR_INVALID, "rays are null");
  SVX_REQUIRE(rays->n_rays >= 0, SVX_ERR_INVALID, "n_rays < 0");
  SVX_REQUIRE(index_base >= 0, SVX_ERR_INVALID, "index_base < 0");
  if (rays->n_rays == 0) return SVX_OK;
  SVX_REQUIRE(rays->origins && rays->dirs && order_out, SVX_ERR_INVALID, "origins / dirs / order_out are null");
  OptP o;
  rc = make_opt(opt, &o);
  if (rc) return rc;
  const GridP g = make_grid(grid);
  Scratch scr(as_stream(stream));
  int* order = nullptr;
  return coherence_sort(g, o, rays->origins, rays->dirs, rays->n_rays, index_base, order_out, scr, 0, &order);
}

extern "C" int svx_add_accum(const float* accum, int32_t stride, int32_t sh_data_dim, int64_t n_voxels,
                             float* grad_sh, float* grad_density, void* stream) {
  clear_error();
  SVX_REQUIRE(n_voxels >= 0, SVX_ERR_INVALID, "n_voxels < 0");
  SVX_REQUIRE(sh_data_dim >= 0 && sh_data_dim + 1 <= stride && stride <= 32 && stride % 4 == 0, SVX_ERR_INVALID,
              "stride %d must be a multiple of 4 in [sh_data_dim + 1, 32] (sh_data_dim %d)", stride, sh_data_dim);
  SVX_REQUIRE(n_voxels == 0 || accum != nullptr, SVX_ERR_INVALID, "accum is null");
  return launch_add_accum(accum, stride, sh_data_dim, n_voxels, grad_sh, grad_density, as_stream(stream));
}

// volume_render_expected_term / volume_render_sigma_thresh host side
// (render_lerp_kernel_cuvol.cu:1154-1195).
static int render_depth(const svx_grid_t* grid, const svx_rays_t* rays, const svx_render_opts_t* opt, bool thresh,
                        float thr, float* out, void* stream) {
  clear_error();
  int rc = check_grid(grid);
  if (rc) return rc;
  SVX_REQUIRE(rays != nullptr, SVX_ERR_INVALID, "rays are null");
  SVX_REQUIRE(rays->n_rays >= 0, SVX_ERR_INVALID, "n_rays < 0");
  if (rays->n_rays == 0) return SVX_OK;
  SVX_REQUIRE(rays->origins && rays->dirs && out, SVX_ERR_INVALID, "origins / dirs / out are null");
  OptP o;
  rc = make_opt(opt, &o);
  if (rc) return rc;
  const GridP g = make_grid(grid);
  IoP io{};
  io.origins = rays->origins;
  io.dirs = rays->dirs;
  io.n_rays = rays->n_rays;
  cudaStream_t st = as_stream(stream);
  Scratch scr(st);
  rc = scr.alloc(0, 256);
  if (rc) return rc;
  io.work = reinterpret_cast<unsigned long long*>(scr.p[0]);
  SVX_CUDA_TRY(cudaMemsetAsync(io.work, 0, sizeof(unsigned long long), st));
  long long blocks = (long long)num_sms() * 8;
  const long long need = (rays->n_rays + kWarps - 1) / kWarps;
  if (blocks > need) blocks = need;
  if (thresh)
    depth_kernel<true><<<(unsigned)blocks, kThreads, 0, st>>>(g, o, io, thr, out);
  else
    depth_kernel<false><<<(unsigned)blocks, kThreads, 0, st>>>(g, o, io, thr, out);
  SVX_LAUNCH_CHECK("depth_kernel");
  return SVX_OK;
}

extern "C" int svx_volume_render_expected_term(const svx_grid_t* grid, const svx_rays_t* rays,
                                               const svx_render_opts_t* opt, float* out, void* stream) {
  return render_depth(grid, rays, opt, false, 0.f, out, stream);
}

extern "C" int svx_volume_render_sigma_thresh(const svx_grid_t* grid, const svx_rays_t* rays,
                                              const svx_render_opts_t* opt, float sigma_thresh, float* out,
                                              void* stream) {
  return render_depth(grid, rays, opt, true, sigma_thresh, out, stream);
}

extern "C" int svx_grid_weight_render(const float* data, const int32_t size[3], const svx_camera_t* cam,
                                      float step_size, float stop_thresh, int32_t last_sample_opaque,
                                      const float offset[3], const float scaling[3], float* grid_weight,
                                      void* stream) {
  clear_error();
  SVX_REQUIRE(size != nullptr && cam != nullptr && offset != nullptr && scaling != nullptr, SVX_ERR_INVALID,
              "size / camera / offset / scaling is null");
  for (int i = 0; i < 3; ++i)
    SVX_REQUIRE(size[i] >= 2, SVX_ERR_INVALID, "grid size[%d] = %d, each side must be >= 2", i, size[i]);
  SVX_REQUIRE(cam->width >= 0 && cam->height >= 0, SVX_ERR_INVALID, "negative image size");
  SVX_REQUIRE(cam->c2w_rows == 3 || cam->c2w_rows == 4, SVX_ERR_INVALID, "c2w must have 3 or 4 rows");
  const long long n = (long long)cam->width * cam->height;
  if (n == 0) return SVX_OK;
  SVX_REQUIRE(data && grid_weight && cam->c2w, SVX_ERR_INVALID, "data / grid_weight / c2w is null");
  svx_render_opts_t ro{};
  ro.step_size = step_size;
  ro.stop_thresh = stop_thresh;
  ro.last_sample_opaque = last_sample_opaque;
  OptP o;
  int rc = make_opt(&ro, &o);
  if (rc) return rc;
  GridP g{};
  for (int i = 0; i < 3; ++i) {
    g.size[i] = size[i];
    g.offset[i] = offset[i];
    g.scaling[i] = scaling[i];
  }
  g.offy = size[2];
  g.offx = (long long)size[1] * size[2];
  IoP io{};
  io.c2w = cam->c2w;
  io.fx = cam->fx;
  io.fy = cam->fy;
  io.cx = cam->cx;
  io.cy = cam->cy;
  io.ndcx = cam->ndc_coeffx;
  io.ndcy = cam->ndc_coeffy;
  io.width = cam->width;
  long long blocks = (n + 255) / 256;
  if (blocks > (long long)num_sms() * 16) blocks = (long long)num_sms() * 16;
  grid_weight_kernel<<<(unsigned)blocks, 256, 0, as_stream(stream)>>>(g, o, io, n, data, grid_weight);
  SVX_LAUNCH_CHECK("grid_weight_kernel");
  return SVX_OK;
}
