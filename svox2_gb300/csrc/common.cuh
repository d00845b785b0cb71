// Shared device helpers and host error plumbing for the svox2_gb300 kernels.
//
// Arithmetic that decides WHICH samples a ray takes (ray bounds, sample
// positions, cell indices, the sigma threshold, the skip distance) is written
// with explicit round-to-nearest intrinsics so that nvcc cannot contract it
// into FMAs the reference source does not spell out.  The CPU restatement in
// oracle/ performs the same IEEE operations in the same order, so the two
// agree bit for bit on every sample's cell and links.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>
#include <string>

#include "../../include/svox2_gb300.h"

namespace svx {

// ---------------------------------------------------------------- errors

// Thread-local message of the last failed call (svx_last_error()).
void set_error(const char* fmt, ...);
void clear_error();

#define SVX_REQUIRE(cond, code, ...)      \
  do {                                    \
    if (!(cond)) {                        \
      ::svx::set_error(__VA_ARGS__);      \
      return (code);                      \
    }                                     \
  } while (0)

#define SVX_CUDA_TRY(expr)                                                   \
  do {                                                                       \
    cudaError_t _e = (expr);                                                 \
    if (_e != cudaSuccess) {                                                 \
      ::svx::set_error("%s: %s (%s)", #expr, cudaGetErrorName(_e),           \
                       cudaGetErrorString(_e));                              \
      return SVX_ERR_CUDA;                                                   \
    }                                                                        \
  } while (0)

// Launch check: the launch configuration error, if any.
#define SVX_LAUNCH_CHECK(what)                                               \
  do {                                                                       \
    cudaError_t _e = cudaGetLastError();                                     \
    if (_e != cudaSuccess) {                                                 \
      ::svx::set_error("launch of %s failed: %s (%s)", what,                 \
                       cudaGetErrorName(_e), cudaGetErrorString(_e));        \
      return SVX_ERR_CUDA;                                                   \
    }                                                                        \
  } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Number of SMs of the current device (cached per device).
int num_sms();

// ---------------------------------------------------------------- loads

template <typename T> __device__ __forceinline__ float to_f32(T v);
template <> __device__ __forceinline__ float to_f32<float>(float v) { return v; }
template <> __device__ __forceinline__ float to_f32<__nv_bfloat16>(__nv_bfloat16 v) {
  return __bfloat162float(v);
}
template <> __device__ __forceinline__ float to_f32<__half>(__half v) { return __half2float(v); }

// A 16-bit table entry from its raw bits: bfloat16 is the top half of a float (a shift, no
// conversion instruction); float16 goes through the hardware conversion.
template <typename T> __device__ __forceinline__ float bits16_to_f32(unsigned short b);
template <> __device__ __forceinline__ float bits16_to_f32<__nv_bfloat16>(unsigned short b) {
  return __uint_as_float((unsigned)b << 16);
}
template <> __device__ __forceinline__ float bits16_to_f32<__half>(unsigned short b) {
  return __half2float(__ushort_as_half(b));
}

template <typename T> __device__ __forceinline__ T from_f32(float v);
template <> __device__ __forceinline__ float from_f32<float>(float v) { return v; }
template <> __device__ __forceinline__ __nv_bfloat16 from_f32<__nv_bfloat16>(float v) {
  return __float2bfloat16_rn(v);
}
template <> __device__ __forceinline__ __half from_f32<__half>(float v) { return __float2half_rn(v); }

// Read-only cached load of a grid table element.
template <typename T> __device__ __forceinline__ float ldg_f32(const T* p) { return to_f32<T>(__ldg(p)); }

// ---------------------------------------------------------------- math

// (1-w) a + w b as fmaf(w, b - a, a) — lerp, svox2/csrc/include/cuda_util.cuh:72-75.
__device__ __forceinline__ float lerpf(float a, float b, float w) {
  return fmaf(w, __fsub_rn(b, a), a);
}

// 1 / |v| for the direction rescale (_get_delta_scale,
// svox2/csrc/include/render_util.cuh:463-474).  The reference calls rnorm3df;
// this library forms the norm from exact double products and rounds once more to
// float, which any IEEE host reproduces exactly.
__device__ __forceinline__ float rnorm3_exact(float x, float y, float z) {
  double s = __dadd_rn(__dadd_rn(__dmul_rn((double)x, (double)x), __dmul_rn((double)y, (double)y)),
                       __dmul_rn((double)z, (double)z));
  return (float)__ddiv_rn(1.0, __dsqrt_rn(s));
}

}  // namespace svx
