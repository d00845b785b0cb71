// Total variation on the voxel grid: its value and its gradients.
//
// Replaces svox2/csrc/loss_kernel.cu: tv_kernel 42-109 (the value), tv_grad_kernel 111-176 (dense over all
// cells), tv_grad_sparse_kernel 178-246 (a list of cells, the training
// default) and msi_tv_grad_sparse_kernel 248-333 (the MSI background), with
// their host launchers 483-641.  One thread per (cell, channel),
// channels innermost so that a warp reads consecutive coefficients of the same
// voxel rows.  The reference's edge conventions are kept exactly:
//   * sparse: a neighbour outside the grid reads link 0 (voxel 0), not -1;
//   * ignore_edge && link(cell) == 0 skips the cell;
//   * ignore_last_z skips cells with z == size2 - 2 (and reads no +z neighbour there);
//   * the finite differences are normalised with rsqrt of the UNSCALED squared
//     gradient, then scaled by size/256 per axis; scale is divided by the
//     number of cells.
#include "common.cuh"

namespace svx {
namespace {

struct TvArgs {
  const int32_t* links;
  int X, Y, Z;
  const void* data;
  long long ncols;
  int start, nch;
  float scale;  // already divided by the number of cells
  int ignore_edge, ignore_last_z;
  float* grad;
  uint8_t* mask;
};

template <typename T>
__device__ __forceinline__ float rd(const TvArgs& a, int lnk, int idx) {
  return to_f32<T>(reinterpret_cast<const T*>(a.data)[(long long)lnk * a.ncols + idx]);
}

__device__ __forceinline__ float inv_norm(float dx, float dy, float dz, float scale) {
  return __fmul_rn(scale, rsqrtf(fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, 1e-9f)))));
}

template <typename T>
__global__ void __launch_bounds__(256) tv_sparse_kernel(TvArgs a, const int32_t* __restrict__ cells,
                                                        long long n) {
  const long long total = n * a.nch;
  const float sx = a.X * (1.f / 256.f), sy = a.Y * (1.f / 256.f), sz = a.Z * (1.f / 256.f);
  for (long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x; tid < total;
       tid += (long long)gridDim.x * blockDim.x) {
    const int idx = (int)(tid % a.nch) + a.start;
    const int xyz = __ldg(cells + tid / a.nch);
    if ((unsigned)xyz >= (unsigned)(a.X * a.Y * a.Z)) continue;  // cell index outside the grid
    const int z = xyz % a.Z, xy = xyz / a.Z;
    const int y = xy % a.Y, x = xy / a.Y;
    const long long offy = a.Z, offx = (long long)a.Y * a.Z;
    const int32_t* lp = a.links + x * offx + y * offy + z;
    const int l000 = __ldg(lp);
    if (a.ignore_edge && l000 == 0) continue;
    const int l001 = (z + 1 < a.Z && (!a.ignore_last_z || z != a.Z - 2)) ? __ldg(lp + 1) : 0;
    const int l010 = (y + 1 < a.Y) ? __ldg(lp + offy) : 0;
    const int l100 = (x + 1 < a.X) ? __ldg(lp + offx) : 0;
    if (a.ignore_last_z && z == a.Z - 2) continue;
    const float v000 = l000 >= 0 ? rd<T>(a, l000, idx) : 0.f;
    const float nul = a.ignore_edge ? v000 : 0.f;
    const float v001 = l001 >= 0 ? rd<T>(a, l001, idx) : nul;
    const float v010 = l010 >= 0 ? rd<T>(a, l010, idx) : nul;
    const float v100 = l100 >= 0 ? rd<T>(a, l100, idx) : nul;
    float dx = __fsub_rn(v100, v000), dy = __fsub_rn(v010, v000), dz = __fsub_rn(v001, v000);
    const float idelta = inv_norm(dx, dy, dz, a.scale);
    dx = __fmul_rn(dx, sx);
    dy = __fmul_rn(dy, sy);
    dz = __fmul_rn(dz, sz);
    const float sm = -__fadd_rn(__fadd_rn(dx, dy), dz);
    auto add = [&](int lnk, float v) {
      if (lnk >= 0 && v != 0.f) {
        atomicAdd(a.grad + (long long)lnk * a.ncols + idx, __fmul_rn(v, idelta));
        if (a.mask != nullptr) a.mask[lnk] = 1;
      }
    };
    add(l000, sm);
    add(l001, dz);
    add(l010, dy);
    add(l100, dx);
  }
}

template <typename T>
__global__ void __launch_bounds__(256) tv_dense_kernel(TvArgs a) {
  const long long ncell = (long long)(a.X - 1) * (a.Y - 1) * (a.Z - 1);
  const long long total = ncell * a.nch;
  const float sx = a.X * (1.f / 256.f), sy = a.Y * (1.f / 256.f), sz = a.Z * (1.f / 256.f);
  for (long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x; tid < total;
       tid += (long long)gridDim.x * blockDim.x) {
    const int idx = (int)(tid % a.nch) + a.start;
    const long long xyz = tid / a.nch;
    const int z = (int)(xyz % (a.Z - 1));
    const long long xy = xyz / (a.Z - 1);
    const int y = (int)(xy % (a.Y - 1)), x = (int)(xy / (a.Y - 1));
    const long long offy = a.Z, offx = (long long)a.Y * a.Z;
    const int32_t* lp = a.links + x * offx + y * offy + z;
    const int l000 = __ldg(lp);
    if (a.ignore_edge && l000 == 0) continue;
    const int l100 = __ldg(lp + offx), l010 = __ldg(lp + offy), l001 = __ldg(lp + 1);
    const float v000 = l000 >= 0 ? rd<T>(a, l000, idx) : 0.f;
    const float v100 = l100 >= 0 ? rd<T>(a, l100, idx) : (a.ignore_edge ? v000 : 0.f);
    const float v010 = l010 >= 0 ? rd<T>(a, l010, idx) : (a.ignore_edge ? v000 : 0.f);
    const float v001 = l001 >= 0 ? rd<T>(a, l001, idx) : (a.ignore_edge ? v000 : 0.f);
    float dx = __fsub_rn(v100, v000), dy = __fsub_rn(v010, v000), dz = __fsub_rn(v001, v000);
    const float idelta = inv_norm(dx, dy, dz, a.scale);
    dx = __fmul_rn(dx, sx);
    dy = __fmul_rn(dy, sy);
    dz = __fmul_rn(dz, sz);
    float* g = a.grad;
    if (dx != 0.f && l100 >= 0) atomicAdd(g + (long long)l100 * a.ncols + idx, __fmul_rn(dx, idelta));
    if (dy != 0.f && l010 >= 0) atomicAdd(g + (long long)l010 * a.ncols + idx, __fmul_rn(dy, idelta));
    if (dz != 0.f && l001 >= 0) atomicAdd(g + (long long)l001 * a.ncols + idx, __fmul_rn(dz, idelta));
    if (l000 >= 0)
      atomicAdd(g + (long long)l000 * a.ncols + idx,
                __fmul_rn(-__fadd_rn(__fadd_rn(dx, dy), dz), idelta));
  }
}

// The TV value (tv_kernel, loss_kernel.cu:42-109): the mean over cells of
// sqrt(1e-5 + |d ⊙ size/256|^2), summed over channels, d the forward differences of
// the cell's voxel to its +x/+y/+z neighbours (missing neighbour: 0, or the voxel's own
// value with ignore_edge; a cell whose voxel has link 0 is skipped with ignore_edge).
// Each block sums its terms in shared memory and adds the block's sum with one atomic;
// out (a device float, zeroed by the host) receives sum * scale.
template <typename T>
__global__ void __launch_bounds__(256) tv_value_kernel(TvArgs a, float* __restrict__ out) {
  __shared__ float part[8];
  const long long ncell = (long long)(a.X - 1) * (a.Y - 1) * (a.Z - 1);
  const long long total = ncell * a.nch;
  const float sx = a.X * (1.f / 256.f), sy = a.Y * (1.f / 256.f), sz = a.Z * (1.f / 256.f);
  float acc = 0.f;
  for (long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x; tid < total;
       tid += (long long)gridDim.x * blockDim.x) {
    const int idx = (int)(tid % a.nch) + a.start;
    const long long xyz = tid / a.nch;
    const int z = (int)(xyz % (a.Z - 1));
    const long long xy = xyz / (a.Z - 1);
    const int y = (int)(xy % (a.Y - 1)), x = (int)(xy / (a.Y - 1));
    const long long offy = a.Z, offx = (long long)a.Y * a.Z;
    const int32_t* lp = a.links + x * offx + y * offy + z;
    const int l000 = __ldg(lp);
    if (a.ignore_edge && l000 == 0) continue;
    const int l100 = __ldg(lp + offx), l010 = __ldg(lp + offy), l001 = __ldg(lp + 1);
    const float v000 = l000 >= 0 ? rd<T>(a, l000, idx) : 0.f;
    const float nul = a.ignore_edge ? v000 : 0.f;
    const float v100 = l100 >= 0 ? rd<T>(a, l100, idx) : nul;
    const float v010 = l010 >= 0 ? rd<T>(a, l010, idx) : nul;
    const float v001 = l001 >= 0 ? rd<T>(a, l001, idx) : nul;
    const float dx = __fmul_rn(__fsub_rn(v100, v000), sx);
    const float dy = __fmul_rn(__fsub_rn(v010, v000), sy);
    const float dz = __fmul_rn(__fsub_rn(v001, v000), sz);
    acc = __fadd_rn(acc, sqrtf(fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, 1e-5f)))));
  }
#pragma unroll
  for (int d = 16; d >= 1; d >>= 1) acc = __fadd_rn(acc, __shfl_xor_sync(0xffffffffu, acc, d));
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    float b = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) b = __fadd_rn(b, part[w]);
    atomicAdd(out, __fmul_rn(b, a.scale));
  }
}

int make_tv(const int32_t* links, const int32_t size[3], const svx_table_t* data, int start, int end,
            float* grad, TvArgs* a) {
  SVX_REQUIRE(links && size && data && data->data && grad, SVX_ERR_INVALID, "null argument");
  for (int i = 0; i < 3; ++i)
    SVX_REQUIRE(size[i] >= 2, SVX_ERR_INVALID, "links size[%d] = %d must be >= 2", i, size[i]);
  SVX_REQUIRE(data->n_cols >= 1, SVX_ERR_INVALID, "data has %d columns", data->n_cols);
  SVX_REQUIRE(0 <= start && start < end && end <= data->n_cols, SVX_ERR_INVALID,
              "channel range [%d, %d) outside [0, %d)", start, end, data->n_cols);
  SVX_REQUIRE(data->dtype == SVX_F32 || data->dtype == SVX_BF16 || data->dtype == SVX_F16, SVX_ERR_INVALID,
              "data dtype %d unknown", data->dtype);
  a->links = links;
  a->X = size[0];
  a->Y = size[1];
  a->Z = size[2];
  a->data = data->data;
  a->ncols = data->n_cols;
  a->start = start;
  a->nch = end - start;
  a->grad = grad;
  a->mask = nullptr;
  return SVX_OK;
}

unsigned grid_for(long long total) {
  long long b = (total + 255) / 256;
  const long long cap = (long long)num_sms() * 32;
  if (b > cap) b = cap;
  return (unsigned)(b < 1 ? 1 : b);
}

// msi_tv_grad_sparse_kernel, loss_kernel.cu:248-333: TV of the MSI background, one thread per
// (listed cell, channel), channels innermost.  x (2 reso columns) and y (reso rows) wrap; z
// stops at the last layer, where the colour channels compare with themselves and sigma with 0.
struct MsiArgs {
  const int32_t* links;
  int X, Y;  // 2 reso, reso
  const float* msi;
  long long capacity;  // rows of msi
  int nl, nc;
  float scale, scale_last;  // already divided by the number of cells
  float* grad;
  uint8_t* mask;
};

__global__ void __launch_bounds__(256) msi_tv_kernel(MsiArgs a, const int32_t* __restrict__ cells, long long n) {
  const long long total = n * a.nc;
  const long long n_cells_all = (long long)a.X * a.Y * a.nl;
  const float sx = a.X * (1.f / 256.f), sy = a.Y * (1.f / 256.f), sz = a.nl * (1.f / 256.f);
  for (long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x; tid < total;
       tid += (long long)gridDim.x * blockDim.x) {
    const int ch = (int)(tid % a.nc);
    const int idx = __ldg(cells + tid / a.nc);
    if (idx < 0 || idx >= n_cells_all) continue;  // cell index outside the MSI
    const int z = idx % a.nl, xy = idx / a.nl;
    const int y = xy % a.Y, x = xy / a.Y;
    const int nx = x == a.X - 1 ? 0 : x + 1, ny = y == a.Y - 1 ? 0 : y + 1;
    // a link past the data's rows reads as empty, like a negative one
    auto link = [&](int xx, int yy) {
      const int l = __ldg(a.links + (long long)xx * a.Y + yy);
      return l < a.capacity ? l : -1;
    };
    const int l00 = link(x, y), l01 = link(x, ny), l10 = link(nx, y);
    const bool last = ch == a.nc - 1;
    auto at = [&](int lnk, int zz) { return __ldg(a.msi + ((long long)lnk * a.nl + zz) * a.nc + ch); };
    const float v00 = l00 >= 0 ? at(l00, z) : 0.f;
    const float vz = (l00 >= 0 && z + 1 < a.nl) ? at(l00, z + 1) : (last ? 0.f : v00);
    const float v01 = l01 >= 0 ? at(l01, z) : 0.f;
    const float v10 = l10 >= 0 ? at(l10, z) : 0.f;
    float dx = __fsub_rn(v10, v00), dy = __fsub_rn(v01, v00), dz = __fsub_rn(vz, v00);
    const float idelta =
        __fmul_rn(last ? a.scale_last : a.scale, rsqrtf(fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, 1e-9f)))));
    dx = __fmul_rn(dx, sx);
    dy = __fmul_rn(dy, sy);
    dz = __fmul_rn(dz, sz);
    const float sm = -__fadd_rn(__fadd_rn(dx, dy), dz);
    auto add = [&](int lnk, int zz, float v) {
      if (lnk >= 0 && v != 0.f) {
        atomicAdd(a.grad + ((long long)lnk * a.nl + zz) * a.nc + ch, __fmul_rn(v, idelta));
        if (a.mask != nullptr) a.mask[(long long)lnk * a.nl + zz] = 1;
      }
    };
    add(l00, z, sm);
    if (z + 1 < a.nl) add(l00, z + 1, dz);
    add(l01, z, dy);
    add(l10, z, dx);
  }
}

}  // namespace
}  // namespace svx

using namespace svx;

extern "C" int svx_tv_grad(const int32_t* links, const int32_t size[3], const svx_table_t* data,
                           int32_t start_dim, int32_t end_dim, float scale, int32_t use_logalpha,
                           float logalpha_delta, int32_t ignore_edge, float ndc_coeffx, float ndc_coeffy,
                           float* grad, void* stream) {
  (void)use_logalpha;
  (void)logalpha_delta;
  (void)ndc_coeffx;
  (void)ndc_coeffy;
  clear_error();
  TvArgs a;
  int rc = make_tv(links, size, data, start_dim, end_dim, grad, &a);
  if (rc) return rc;
  const long long ncell = (long long)(a.X - 1) * (a.Y - 1) * (a.Z - 1);
  // the reference divides by the cell count held in an int (loss_kernel.cu:539)
  a.scale = scale / (float)(int)ncell;
  a.ignore_edge = ignore_edge != 0;
  a.ignore_last_z = 0;
  cudaStream_t st = as_stream(stream);
  const unsigned blocks = grid_for(ncell * a.nch);
  switch (data->dtype) {
    case SVX_F32: tv_dense_kernel<float><<<blocks, 256, 0, st>>>(a); break;
    case SVX_BF16: tv_dense_kernel<__nv_bfloat16><<<blocks, 256, 0, st>>>(a); break;
    default: tv_dense_kernel<__half><<<blocks, 256, 0, st>>>(a);
  }
  SVX_LAUNCH_CHECK("tv_dense_kernel");
  return SVX_OK;
}

extern "C" int svx_tv_grad_sparse(const int32_t* links, const int32_t size[3], const svx_table_t* data,
                                  const int32_t* rand_cells, int64_t n_cells, uint8_t* mask_out,
                                  int32_t start_dim, int32_t end_dim, float scale, int32_t use_logalpha,
                                  float logalpha_delta, int32_t ignore_edge, int32_t ignore_last_z,
                                  float ndc_coeffx, float ndc_coeffy, float* grad, void* stream) {
  (void)use_logalpha;
  (void)logalpha_delta;
  (void)ndc_coeffx;
  (void)ndc_coeffy;
  clear_error();
  TvArgs a;
  int rc = make_tv(links, size, data, start_dim, end_dim, grad, &a);
  if (rc) return rc;
  SVX_REQUIRE(n_cells >= 0, SVX_ERR_INVALID, "n_cells < 0");
  if (n_cells == 0) return SVX_OK;
  SVX_REQUIRE(rand_cells != nullptr, SVX_ERR_INVALID, "rand_cells is null");
  a.scale = scale / (float)(int)n_cells;
  a.ignore_edge = ignore_edge != 0;
  a.ignore_last_z = ignore_last_z != 0;
  a.mask = mask_out;
  cudaStream_t st = as_stream(stream);
  const unsigned blocks = grid_for(n_cells * a.nch);
  switch (data->dtype) {
    case SVX_F32: tv_sparse_kernel<float><<<blocks, 256, 0, st>>>(a, rand_cells, n_cells); break;
    case SVX_BF16: tv_sparse_kernel<__nv_bfloat16><<<blocks, 256, 0, st>>>(a, rand_cells, n_cells); break;
    default: tv_sparse_kernel<__half><<<blocks, 256, 0, st>>>(a, rand_cells, n_cells);
  }
  SVX_LAUNCH_CHECK("tv_sparse_kernel");
  return SVX_OK;
}

extern "C" int svx_tv(const int32_t* links, const int32_t size[3], const svx_table_t* data, int32_t start_dim,
                      int32_t end_dim, int32_t use_logalpha, float logalpha_delta, int32_t ignore_edge,
                      float ndc_coeffx, float ndc_coeffy, float* out, void* stream) {
  (void)logalpha_delta;
  (void)ndc_coeffx;
  (void)ndc_coeffy;
  clear_error();
  SVX_REQUIRE(!use_logalpha, SVX_ERR_UNSUPPORTED, "use_logalpha is no longer supported (as in the reference)");
  SVX_REQUIRE(out != nullptr, SVX_ERR_INVALID, "out is null");
  TvArgs a;
  int rc = make_tv(links, size, data, start_dim, end_dim, out, &a);
  if (rc) return rc;
  const long long ncell = (long long)(a.X - 1) * (a.Y - 1) * (a.Z - 1);
  a.scale = 1.f / (float)(int)ncell;
  a.ignore_edge = ignore_edge != 0;
  a.ignore_last_z = 0;
  cudaStream_t st = as_stream(stream);
  SVX_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(float), st));
  const unsigned blocks = grid_for(ncell * a.nch);
  switch (data->dtype) {
    case SVX_F32: tv_value_kernel<float><<<blocks, 256, 0, st>>>(a, out); break;
    case SVX_BF16: tv_value_kernel<__nv_bfloat16><<<blocks, 256, 0, st>>>(a, out); break;
    default: tv_value_kernel<__half><<<blocks, 256, 0, st>>>(a, out);
  }
  SVX_LAUNCH_CHECK("tv_value_kernel");
  return SVX_OK;
}

extern "C" int svx_msi_tv_grad_sparse(const int32_t* links, int32_t reso, const float* msi, int64_t capacity,
                                      int32_t nlayers, int32_t n_channels, const int32_t* rand_cells,
                                      int64_t n_cells, uint8_t* mask_out, float scale, float scale_last,
                                      float* grad, void* stream) {
  clear_error();
  SVX_REQUIRE(links && msi && grad, SVX_ERR_INVALID, "null argument");
  SVX_REQUIRE(reso >= 1, SVX_ERR_INVALID, "reso = %d must be >= 1", reso);
  SVX_REQUIRE(nlayers >= 1 && n_channels >= 1, SVX_ERR_INVALID, "nlayers = %d, n_channels = %d must be >= 1",
              nlayers, n_channels);
  SVX_REQUIRE(capacity >= 0, SVX_ERR_INVALID, "capacity < 0");
  SVX_REQUIRE((long long)2 * reso * reso * nlayers < (1ll << 31), SVX_ERR_TOO_LARGE,
              "the MSI's cell count must fit int32 cell indices");
  SVX_REQUIRE(n_cells >= 0, SVX_ERR_INVALID, "n_cells < 0");
  if (n_cells == 0) return SVX_OK;
  SVX_REQUIRE(rand_cells != nullptr, SVX_ERR_INVALID, "rand_cells is null");
  MsiArgs a;
  a.links = links;
  a.X = 2 * reso;
  a.Y = reso;
  a.msi = msi;
  a.capacity = capacity;
  a.nl = nlayers;
  a.nc = n_channels;
  a.scale = scale / (float)(int)n_cells;
  a.scale_last = scale_last / (float)(int)n_cells;
  a.grad = grad;
  a.mask = mask_out;
  cudaStream_t st = as_stream(stream);
  msi_tv_kernel<<<grid_for(n_cells * n_channels), 256, 0, st>>>(a, rand_cells, n_cells);
  SVX_LAUNCH_CHECK("msi_tv_kernel");
  return SVX_OK;
}
