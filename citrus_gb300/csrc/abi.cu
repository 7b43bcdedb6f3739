// Status plumbing of the C ABI: the per-thread error message, launch checks and device queries.
#include <stdarg.h>

#include <atomic>
#include <mutex>
#include <vector>

#include "common.cuh"

namespace citrus {

static thread_local char g_last_error[1024] = "";

int set_error(int code, const char* fmt, ...) {
  va_list args;
  va_start(args, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, args);
  va_end(args);
  return code;
}

int launch_status(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(CITRUS_ELAUNCH, "%s: %s", what, cudaGetErrorString(e));
  return CITRUS_OK;
}

static std::atomic<long long> g_launches{0};

void note_launches(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

int num_sms() {
  static std::mutex mutex;
  static std::vector<int> cache;
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess) return 1;
  std::lock_guard<std::mutex> lock(mutex);
  if ((int)cache.size() <= device) cache.resize(device + 1, 0);
  if (cache[device] == 0) {
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device);
    cache[device] = n > 0 ? n : 1;
  }
  return cache[device];
}

}  // namespace citrus

extern "C" int citrus_abi_version(void) { return CITRUS_GB300_ABI_VERSION; }

extern "C" const char* citrus_last_error_string(void) { return citrus::g_last_error; }

extern "C" int64_t citrus_launch_count(void) { return (int64_t)citrus::g_launches.load(std::memory_order_relaxed); }
