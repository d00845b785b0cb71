// Library-wide host plumbing: error messages, device properties, ABI version.
#include "common.cuh"

#include <cstdarg>
#include <cstdio>
#include <mutex>

namespace svx {

static thread_local char g_err[512] = {0};

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

void clear_error() { g_err[0] = 0; }

int num_sms() {
  static std::mutex mu;
  static int cache[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  std::lock_guard<std::mutex> lk(mu);
  int& v = cache[dev & 63];
  if (v == 0) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 1;
    v = n;
  }
  return v;
}

}  // namespace svx

extern "C" const char* svx_last_error(void) { return svx::g_err; }

extern "C" int svx_abi_version(void) { return SVX_ABI_VERSION; }
