// RMSprop and SGD steps on the grid tables.
//
// Replaces svox2/csrc/optim_kernel.cu (rmsprop_once 15-25, six kernels 27-147,
// host 154-267).  The update of one element is the reference's:
//   rms  = rms == 0 ? g^2 : lerp(g^2, rms, beta)      (fmaf(beta, rms - g^2, g^2))
//   data = max(data - lr * g / (sqrt(rms) + eps), minval)
//   g    = 0
// with lr_last for the last column, written with explicit round-to-nearest
// operations so the result is bit-identical to the CPU restatement.  The
// kernels are streaming (one element per thread, grid-stride): the dense and
// mask forms read the whole table, the mask form skips rows whose mask is 0
// after one byte read, the list form visits only the listed rows.  Data may be
// stored f32, bf16 or f16; rms and grad are f32.
#include "common.cuh"

namespace svx {
namespace {

struct OptArgs {
  void* data;
  float* rms;
  float* grad;
  long long n_rows;
  int n_cols;
  float beta, lr, eps, minval, lr_last;
};

template <typename T, bool RMS>
__device__ __forceinline__ void step_one(const OptArgs& a, long long off, int col) {
  T* d = reinterpret_cast<T*>(a.data) + off;
  const float lr = (col == a.n_cols - 1) ? a.lr_last : a.lr;
  const float g = a.grad[off];
  float v = to_f32<T>(*d);
  if (RMS) {
    const float g2 = __fmul_rn(g, g);
    float r = a.rms[off];
    r = (r == 0.f) ? g2 : fmaf(a.beta, __fsub_rn(r, g2), g2);
    a.rms[off] = r;
    v = fmaxf(__fsub_rn(v, __fdiv_rn(__fmul_rn(lr, g), __fadd_rn(__fsqrt_rn(r), a.eps))), a.minval);
  } else {
    v = __fsub_rn(v, __fmul_rn(lr, g));
  }
  *d = from_f32<T>(v);
  a.grad[off] = 0.f;
}

template <typename T, bool RMS>
__global__ void __launch_bounds__(256) step_all_kernel(OptArgs a) {
  const long long total = a.n_rows * a.n_cols;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x)
    step_one<T, RMS>(a, e, (int)(e % a.n_cols));
}

template <typename T, bool RMS>
__global__ void __launch_bounds__(256) step_mask_kernel(OptArgs a, const uint8_t* __restrict__ mask) {
  const long long total = a.n_rows * a.n_cols;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long row = e / a.n_cols;
    if (__ldg(mask + row) == 0) continue;
    step_one<T, RMS>(a, e, (int)(e - row * a.n_cols));
  }
}

template <typename T, bool RMS>
__global__ void __launch_bounds__(256) step_list_kernel(OptArgs a, const int64_t* __restrict__ idx,
                                                        long long n) {
  const long long total = n * a.n_cols;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long k = e / a.n_cols;
    const int col = (int)(e - k * a.n_cols);
    const long long row = __ldg(idx + k);
    if (row < 0 || row >= a.n_rows) continue;  // index outside the table
    step_one<T, RMS>(a, row * a.n_cols + col, col);
  }
}

unsigned grid_for(long long total) {
  long long b = (total + 255) / 256;
  const long long cap = (long long)num_sms() * 32;
  if (b > cap) b = cap;
  return (unsigned)(b < 1 ? 1 : b);
}

template <typename T, bool RMS>
int run(const OptArgs& a, int kind, const void* indexer, long long n_index, cudaStream_t st) {
  switch (kind) {
    case SVX_INDEX_ALL:
      step_all_kernel<T, RMS><<<grid_for(a.n_rows * a.n_cols), 256, 0, st>>>(a);
      break;
    case SVX_INDEX_MASK:
      step_mask_kernel<T, RMS><<<grid_for(a.n_rows * a.n_cols), 256, 0, st>>>(
          a, reinterpret_cast<const uint8_t*>(indexer));
      break;
    case SVX_INDEX_LIST:
      step_list_kernel<T, RMS><<<grid_for(n_index * a.n_cols), 256, 0, st>>>(
          a, reinterpret_cast<const int64_t*>(indexer), n_index);
      break;
    default:
      return SVX_OK;
  }
  SVX_LAUNCH_CHECK("optimizer step kernel");
  return SVX_OK;
}

template <bool RMS>
int optim_entry(void* data, int dtype, float* rms, float* grad, long long n_rows, int n_cols, int kind,
                const void* indexer, long long n_index, float beta, float lr, float eps, float minval,
                float lr_last, void* stream) {
  clear_error();
  SVX_REQUIRE(kind >= SVX_INDEX_ALL && kind <= SVX_INDEX_LIST, SVX_ERR_INVALID, "indexer kind %d unknown",
              kind);
  SVX_REQUIRE(n_rows >= 0 && n_cols >= 1, SVX_ERR_INVALID, "table shape [%lld, %d] invalid", n_rows, n_cols);
  if (kind == SVX_INDEX_NONE || n_rows == 0) return SVX_OK;
  if (kind == SVX_INDEX_LIST && n_index == 0) return SVX_OK;
  SVX_REQUIRE(data && grad && (!RMS || rms), SVX_ERR_INVALID, "data / rms / grad are null");
  SVX_REQUIRE(kind == SVX_INDEX_ALL || indexer, SVX_ERR_INVALID, "indexer is null");
  SVX_REQUIRE(n_index >= 0, SVX_ERR_INVALID, "n_index < 0");
  OptArgs a{data, rms, grad, n_rows, n_cols, beta, lr, eps, minval, lr_last < 0.f ? lr : lr_last};
  cudaStream_t st = as_stream(stream);
  switch (dtype) {
    case SVX_F32: return run<float, RMS>(a, kind, indexer, n_index, st);
    case SVX_BF16: return run<__nv_bfloat16, RMS>(a, kind, indexer, n_index, st);
    case SVX_F16: return run<__half, RMS>(a, kind, indexer, n_index, st);
  }
  set_error("data dtype %d unknown", dtype);
  return SVX_ERR_INVALID;
}

}  // namespace
}  // namespace svx

extern "C" int svx_rmsprop_step(void* data, int32_t data_dtype, float* rms, float* grad, int64_t n_rows,
                                int32_t n_cols, int32_t indexer_kind, const void* indexer, int64_t n_index,
                                float beta, float lr, float epsilon, float minval, float lr_last,
                                void* stream) {
  return svx::optim_entry<true>(data, data_dtype, rms, grad, n_rows, n_cols, indexer_kind, indexer, n_index,
                                beta, lr, epsilon, minval, lr_last, stream);
}

extern "C" int svx_sgd_step(void* data, int32_t data_dtype, float* grad, int64_t n_rows, int32_t n_cols,
                            int32_t indexer_kind, const void* indexer, int64_t n_index, float lr,
                            float lr_last, void* stream) {
  return svx::optim_entry<false>(data, data_dtype, nullptr, grad, n_rows, n_cols, indexer_kind, indexer,
                                 n_index, 0.f, lr, 0.f, 0.f, lr_last, stream);
}
