// Trilinear sampling of the grid at points and its adjoint.
//
// Replaces svox2/csrc/svox2_kernel.cu (sample_grid_sh_kernel 10-46,
// sample_grid_density_kernel 48-78, backward kernels 81-176, host 181-267).
// The reference launched density and SH kernels on two freshly created streams
// per call and synchronised them; here both run as one kernel on the caller's
// stream with no host synchronisation.  One warp handles one point: lane 0..C-1
// owns an SH channel (coalesced 27-wide row reads and atomic adds), and the
// density is interpolated by every lane from the same 8 links.
#include "common.cuh"

namespace svx {
namespace {

constexpr unsigned kFull = 0xffffffffu;

struct SampleGrid {
  const float* density;
  const void* sh;
  const int32_t* links;
  int size[3];
  long long offx, offy;
  float offset[3], scaling[3];
  int C;
};

// Point -> cell and fractional position, svox2_kernel.cu:20-28 (transform_coord + clamp).
__device__ __forceinline__ long long locate(const SampleGrid& g, const float* pt, float p[3]) {
  int l[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    float v = fmaf(__ldg(pt + i), g.scaling[i], g.offset[i]);
    v = fminf(fmaxf(v, 0.f), (float)g.size[i] - 1.f);
    l[i] = min((int)v, g.size[i] - 2);
    p[i] = __fsub_rn(v, (float)l[i]);
  }
  return (long long)l[0] * g.offx + (long long)l[1] * g.offy + l[2];
}

template <typename ShT>
__global__ void __launch_bounds__(256) sample_fwd_kernel(SampleGrid g, const float* __restrict__ pts,
                                                         long long n, int want_colors,
                                                         float* __restrict__ out_d,
                                                         float* __restrict__ out_sh) {
  const int lane = threadIdx.x & 31;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  const ShT* __restrict__ sh = reinterpret_cast<const ShT*>(g.sh);
  for (long long pid = warp; pid < n; pid += nwarps) {
    float p[3];
    const int32_t* lp = g.links + locate(g, pts + pid * 3, p);
    const long long o[8] = {0, 1, g.offy, g.offy + 1, g.offx, g.offx + 1, g.offx + g.offy,
                            g.offx + g.offy + 1};
    int lk[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) lk[j] = __ldg(lp + o[j]);
    // density (lane 0 writes); lerp order of trilerp_cuvol_one (render_util.cuh:71-91)
    {
      float v[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) v[j] = lk[j] >= 0 ? __ldg(g.density + lk[j]) : 0.f;
      const float a = lerpf(lerpf(v[0], v[1], p[2]), lerpf(v[2], v[3], p[2]), p[1]);
      const float b = lerpf(lerpf(v[4], v[5], p[2]), lerpf(v[6], v[7], p[2]), p[1]);
      if (lane == 0) out_d[pid] = lerpf(a, b, p[0]);
    }
    if (want_colors) {
      for (int c = lane; c < g.C; c += 32) {
        float v[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) v[j] = lk[j] >= 0 ? ldg_f32(sh + (long long)lk[j] * g.C + c) : 0.f;
        const float a = lerpf(lerpf(v[0], v[1], p[2]), lerpf(v[2], v[3], p[2]), p[1]);
        const float b = lerpf(lerpf(v[4], v[5], p[2]), lerpf(v[6], v[7], p[2]), p[1]);
        out_sh[pid * g.C + c] = lerpf(a, b, p[0]);
      }
    }
  }
}

// Adjoint: weights as sample_grid_sh_backward_kernel (svox2_kernel.cu:106-121).
__global__ void __launch_bounds__(256) sample_bwd_kernel(SampleGrid g, const float* __restrict__ pts,
                                                         long long n, int want_colors,
                                                         const float* __restrict__ gd,
                                                         const float* __restrict__ gsh,
                                                         float* __restrict__ out_gd,
                                                         float* __restrict__ out_gsh) {
  const int lane = threadIdx.x & 31;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long pid = warp; pid < n; pid += nwarps) {
    float p[3];
    const int32_t* lp = g.links + locate(g, pts + pid * 3, p);
    const long long o[8] = {0, 1, g.offy, g.offy + 1, g.offx, g.offx + 1, g.offx + g.offy,
                            g.offx + g.offy + 1};
    int lk[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) lk[j] = __ldg(lp + o[j]);
    const float xb = p[0], yb = p[1], zb = p[2];
    const float xa = __fsub_rn(1.f, xb), ya = __fsub_rn(1.f, yb), za = __fsub_rn(1.f, zb);
    // per-corner weight with the reference's product order: ((x * go) * y) * z
    auto corner = [&](float go, int j) {
      const float x = (j & 4) ? xb : xa, y = (j & 2) ? yb : ya, z = (j & 1) ? zb : za;
      return __fmul_rn(__fmul_rn(y, __fmul_rn(x, go)), z);
    };
    if (lane < 8) {
      const float go = __ldg(gd + pid);
      int lkj = lk[0];
#pragma unroll
      for (int j = 1; j < 8; ++j)
        if (lane == j) lkj = lk[j];
      if (lkj >= 0) atomicAdd(out_gd + lkj, corner(go, lane));
    }
    if (want_colors) {
      for (int c = lane; c < g.C; c += 32) {
        const float go = __ldg(gsh + pid * g.C + c);
#pragma unroll
        for (int j = 0; j < 8; ++j)
          if (lk[j] >= 0) atomicAdd(out_gsh + (long long)lk[j] * g.C + c, corner(go, j));
      }
    }
  }
}

int make_sample_grid(const svx_grid_t* grid, SampleGrid* g) {
  SVX_REQUIRE(grid != nullptr, SVX_ERR_INVALID, "grid is null");
  SVX_REQUIRE(grid->links && grid->density_data, SVX_ERR_INVALID, "grid tables are null");
  for (int i = 0; i < 3; ++i)
    SVX_REQUIRE(grid->size[i] >= 2, SVX_ERR_INVALID, "grid size[%d] = %d must be >= 2", i, grid->size[i]);
  SVX_REQUIRE(grid->sh_data_dim >= 1 && grid->sh_data_dim <= 96, SVX_ERR_INVALID,
              "sh_data_dim %d out of range", grid->sh_data_dim);
  SVX_REQUIRE(grid->sh_dtype == SVX_F32 || grid->sh_dtype == SVX_BF16 || grid->sh_dtype == SVX_F16,
              SVX_ERR_INVALID, "sh_dtype %d unknown", grid->sh_dtype);
  g->density = grid->density_data;
  g->sh = grid->sh_data;
  g->links = grid->links;
  for (int i = 0; i < 3; ++i) {
    g->size[i] = grid->size[i];
    g->offset[i] = grid->offset[i];
    g->scaling[i] = grid->scaling[i];
  }
  g->offy = grid->size[2];
  g->offx = (long long)grid->size[1] * grid->size[2];
  g->C = grid->sh_data_dim;
  return SVX_OK;
}

unsigned blocks_for(long long n_points) {
  long long b = (n_points + 7) / 8;  // 8 warps of 32 per 256-thread block
  const long long cap = (long long)num_sms() * 16;
  if (b > cap) b = cap;
  return (unsigned)(b < 1 ? 1 : b);
}

}  // namespace
}  // namespace svx

using namespace svx;

extern "C" int svx_sample_grid(const svx_grid_t* grid, const float* points, int64_t n_points,
                               int32_t want_colors, float* out_density, float* out_sh, void* stream) {
  clear_error();
  SampleGrid g;
  int rc = make_sample_grid(grid, &g);
  if (rc) return rc;
  SVX_REQUIRE(n_points >= 0, SVX_ERR_INVALID, "n_points < 0");
  if (n_points == 0) return SVX_OK;
  SVX_REQUIRE(points && out_density, SVX_ERR_INVALID, "points / out_density are null");
  SVX_REQUIRE(!want_colors || (out_sh && grid->sh_data), SVX_ERR_INVALID, "out_sh / sh_data are null");
  cudaStream_t st = as_stream(stream);
  const unsigned blocks = blocks_for(n_points);
  switch (grid->sh_dtype) {
    case SVX_F32:
      sample_fwd_kernel<float><<<blocks, 256, 0, st>>>(g, points, n_points, want_colors, out_density, out_sh);
      break;
    case SVX_BF16:
      sample_fwd_kernel<__nv_bfloat16><<<blocks, 256, 0, st>>>(g, points, n_points, want_colors, out_density,
                                                               out_sh);
      break;
    default:
      sample_fwd_kernel<__half><<<blocks, 256, 0, st>>>(g, points, n_points, want_colors, out_density, out_sh);
  }
  SVX_LAUNCH_CHECK("sample_fwd_kernel");
  return SVX_OK;
}

extern "C" int svx_sample_grid_backward(const svx_grid_t* grid, const float* points, int64_t n_points,
                                        const float* grad_out_density, const float* grad_out_sh,
                                        float* grad_density_out, float* grad_sh_out, int32_t want_colors,
                                        void* stream) {
  clear_error();
  SampleGrid g;
  int rc = make_sample_grid(grid, &g);
  if (rc) return rc;
  SVX_REQUIRE(n_points >= 0, SVX_ERR_INVALID, "n_points < 0");
  if (n_points == 0) return SVX_OK;
  SVX_REQUIRE(points && grad_out_density && grad_density_out, SVX_ERR_INVALID,
              "points / grad_out_density / grad_density_out are null");
  SVX_REQUIRE(!want_colors || (grad_out_sh && grad_sh_out), SVX_ERR_INVALID,
              "grad_out_sh / grad_sh_out are null");
  cudaStream_t st = as_stream(stream);
  sample_bwd_kernel<<<blocks_for(n_points), 256, 0, st>>>(g, points, n_points, want_colors, grad_out_density,
                                                          grad_out_sh, grad_density_out, grad_sh_out);
  SVX_LAUNCH_CHECK("sample_bwd_kernel");
  return SVX_OK;
}
