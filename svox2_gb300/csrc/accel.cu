// Grid editing kernels of svox2/csrc/misc_kernel.cu: empty-space skip levels
// (accel_dist_prop) and 3-D mask dilation (dilate).
//
// Empty-space skip levels of a links table: accel_dist_prop
// (svox2/csrc/misc_kernel.cu:108-181 kernels, 356-416 host; SparseGrid.accelerate,
// svox2/svox2.py:1487-1494).
//
// Every voxel whose link is negative gets -(1 + e), where e counts the consecutive
// levels of a 2x occupancy pyramid, starting at the level above the voxel, whose
// ancestor cell holds no voxel with link >= 0.  The ray march reads such a link as
// "the enclosing 2^e-voxel block is empty" and jumps over it (compute_skip_dist).
// The pyramid halves each side with rounding up while every side of the previous
// level is > 1, so a 256^3 grid has 8 levels and a 20 x 28 x 36 grid 5.
//
// The reference marks every ancestor of every occupied voxel from that voxel's thread.
// Here the pyramid is built one level at a time (one thread per cell of the level
// below), then one thread per voxel walks up from its parent until an occupied cell.
#include "common.cuh"

namespace svx {
namespace {

constexpr int kMaxLevels = 32;

struct Pyramid {
  int n;                       // levels
  int sx[kMaxLevels], sy[kMaxLevels], sz[kMaxLevels];
  long long off[kMaxLevels];   // byte offset of each level in the occupancy buffer
  long long total;
};

Pyramid make_pyramid(int X, int Y, int Z) {
  Pyramid p{};
  long long off = 0;
  while (X > 1 && Y > 1 && Z > 1 && p.n < kMaxLevels) {
    X = (X + 1) / 2;
    Y = (Y + 1) / 2;
    Z = (Z + 1) / 2;
    p.sx[p.n] = X;
    p.sy[p.n] = Y;
    p.sz[p.n] = Z;
    p.off[p.n] = off;
    off += (long long)X * Y * Z;
    ++p.n;
  }
  p.total = off;
  return p;
}

// Level 0 of the pyramid from the voxels: cell (x>>1, y>>1, z>>1) is occupied if any of
// its voxels has a link >= 0.
__global__ void __launch_bounds__(256) mark_voxels_kernel(const int32_t* __restrict__ links, int X, int Y, int Z,
                                                          uint8_t* __restrict__ lvl, int sy, int sz) {
  const long long n = (long long)X * Y * Z;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (long long)gridDim.x * blockDim.x) {
    if (__ldg(links + v) < 0) continue;
    const int z = (int)(v % Z), y = (int)((v / Z) % Y), x = (int)(v / ((long long)Y * Z));
    const long long c = ((long long)(x >> 1) * sy + (y >> 1)) * sz + (z >> 1);
    if (!lvl[c]) lvl[c] = 1;  // every writer stores the same value
  }
}

// Level k+1 from level k.
__global__ void __launch_bounds__(256) mark_level_kernel(const uint8_t* __restrict__ below, int X, int Y, int Z,
                                                         uint8_t* __restrict__ above, int sy, int sz) {
  const long long n = (long long)X * Y * Z;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (long long)gridDim.x * blockDim.x) {
    if (!below[v]) continue;
    const int z = (int)(v % Z), y = (int)((v / Z) % Y), x = (int)(v / ((long long)Y * Z));
    const long long c = ((long long)(x >> 1) * sy + (y >> 1)) * sz + (z >> 1);
    if (!above[c]) above[c] = 1;
  }
}

__global__ void __launch_bounds__(256) skip_levels_kernel(int32_t* __restrict__ links, int X, int Y, int Z,
                                                          const uint8_t* __restrict__ occ, Pyramid p) {
  const long long n = (long long)X * Y * Z;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (long long)gridDim.x * blockDim.x) {
    if (links[v] >= 0) continue;
    int z = (int)(v % Z), y = (int)((v / Z) % Y), x = (int)(v / ((long long)Y * Z));
    int32_t result = -1;
    for (int k = 0; k < p.n; ++k) {
      x >>= 1;
      y >>= 1;
      z >>= 1;
      if (occ[p.off[k] + ((long long)x * p.sy[k] + y) * p.sz[k] + z]) break;
      --result;
    }
    links[v] = result;
  }
}

// dilate, misc_kernel.cu:20-48: out[v] = OR of grid over the 3x3x3 block around v, the block
// clamped at the grid's faces.
__global__ void __launch_bounds__(256) dilate_kernel(const uint8_t* __restrict__ in, int X, int Y, int Z,
                                                     uint8_t* __restrict__ out) {
  const long long n = (long long)X * Y * Z;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (long long)gridDim.x * blockDim.x) {
    const int z = (int)(v % Z), y = (int)((v / Z) % Y), x = (int)(v / ((long long)Y * Z));
    uint8_t acc = 0;
    for (int a = max(x - 1, 0); a <= min(x + 1, X - 1); ++a)
      for (int b = max(y - 1, 0); b <= min(y + 1, Y - 1); ++b) {
        const uint8_t* row = in + ((long long)a * Y + b) * Z;
        for (int c = max(z - 1, 0); c <= min(z + 1, Z - 1); ++c) acc |= row[c];
      }
    out[v] = acc ? 1 : 0;
  }
}

unsigned grid_blocks(long long n) {
  long long b = (n + 255) / 256;
  const long long cap = (long long)num_sms() * 32;
  if (b > cap) b = cap;
  return (unsigned)(b > 0 ? b : 1);
}

}  // namespace
}  // namespace svx

using namespace svx;

extern "C" int svx_accel_dist_prop(int32_t* links, const int32_t size[3], void* stream) {
  clear_error();
  SVX_REQUIRE(size != nullptr, SVX_ERR_INVALID, "size is null");
  const int X = size[0], Y = size[1], Z = size[2];
  SVX_REQUIRE(X >= 0 && Y >= 0 && Z >= 0, SVX_ERR_INVALID, "negative grid size");
  const long long n = (long long)X * Y * Z;
  if (n == 0) return SVX_OK;
  SVX_REQUIRE(links != nullptr, SVX_ERR_INVALID, "links is null");
  SVX_REQUIRE(n < (1ll << 40), SVX_ERR_TOO_LARGE, "grid of %lld voxels", n);
  const Pyramid p = make_pyramid(X, Y, Z);
  cudaStream_t st = as_stream(stream);
  uint8_t* occ = nullptr;
  if (p.total > 0) {
    SVX_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&occ), (size_t)p.total, st));
    cudaError_t e = cudaMemsetAsync(occ, 0, (size_t)p.total, st);
    if (e == cudaSuccess) {
      mark_voxels_kernel<<<grid_blocks(n), 256, 0, st>>>(links, X, Y, Z, occ + p.off[0], p.sy[0], p.sz[0]);
      e = cudaGetLastError();
    }
    for (int k = 0; e == cudaSuccess && k + 1 < p.n; ++k) {
      const long long m = (long long)p.sx[k] * p.sy[k] * p.sz[k];
      mark_level_kernel<<<grid_blocks(m), 256, 0, st>>>(occ + p.off[k], p.sx[k], p.sy[k], p.sz[k],
                                                         occ + p.off[k + 1], p.sy[k + 1], p.sz[k + 1]);
      e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
      cudaFreeAsync(occ, st);
      set_error("accel_dist_prop pyramid: %s", cudaGetErrorString(e));
      return SVX_ERR_CUDA;
    }
  }
  skip_levels_kernel<<<grid_blocks(n), 256, 0, st>>>(links, X, Y, Z, occ, p);
  const cudaError_t e = cudaGetLastError();
  if (occ != nullptr) cudaFreeAsync(occ, st);
  if (e != cudaSuccess) {
    set_error("launch of skip_levels_kernel failed: %s", cudaGetErrorString(e));
    return SVX_ERR_CUDA;
  }
  return SVX_OK;
}

extern "C" int svx_dilate(const uint8_t* grid, uint8_t* out, const int32_t size[3], void* stream) {
  clear_error();
  SVX_REQUIRE(size != nullptr, SVX_ERR_INVALID, "size is null");
  const int X = size[0], Y = size[1], Z = size[2];
  SVX_REQUIRE(X >= 0 && Y >= 0 && Z >= 0, SVX_ERR_INVALID, "negative grid size");
  const long long n = (long long)X * Y * Z;
  if (n == 0) return SVX_OK;
  SVX_REQUIRE(grid != nullptr && out != nullptr, SVX_ERR_INVALID, "grid / out is null");
  SVX_REQUIRE(grid != out, SVX_ERR_INVALID, "dilate cannot run in place");
  dilate_kernel<<<grid_blocks(n), 256, 0, as_stream(stream)>>>(grid, X, Y, Z, out);
  SVX_LAUNCH_CHECK("dilate_kernel");
  return SVX_OK;
}
