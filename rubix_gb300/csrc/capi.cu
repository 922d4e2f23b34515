// Error state and small process-wide helpers of the C ABI.
#include "common.cuh"

#include <mutex>

namespace rubix {

static thread_local char g_last_error[1024] = {0};

int set_error(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return code;
}

void clear_error() { g_last_error[0] = 0; }

int sm_count() {
  static std::mutex mu;
  static int cached[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
  std::lock_guard<std::mutex> lock(mu);
  if (cached[dev] == 0) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
      n = 1;
    cached[dev] = n;
  }
  return cached[dev];
}

}  // namespace rubix

extern "C" int rubix_abi_version(void) { return RUBIX_ABI_VERSION; }

extern "C" const char* rubix_last_error(void) { return rubix::g_last_error; }
