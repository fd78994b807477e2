// Error reporting, device properties and the launch counter of the C ABI.
#include "pe_common.cuh"

#include <atomic>
#include <mutex>

namespace pe {

namespace {
thread_local char g_message[512] = "";
std::atomic<long long> g_launches{0};
std::mutex g_sm_mutex;
int g_sm_counts[64] = {0};
}  // namespace

void set_error(const char* fmt, ...) {
  va_list args;
  va_start(args, fmt);
  vsnprintf(g_message, sizeof(g_message), fmt, args);
  va_end(args);
}

int current_device() {
  int device = 0;
  cudaGetDevice(&device);
  return device;
}

int sm_count() {
  int device = current_device();
  if (device < 0 || device >= 64) device = 0;
  std::lock_guard<std::mutex> lock(g_sm_mutex);
  if (g_sm_counts[device] == 0) {
    int count = 0;
    if (cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || count <= 0)
      count = 1;
    g_sm_counts[device] = count;
  }
  return g_sm_counts[device];
}

void count_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

}  // namespace pe

// Text of the last failure on the calling host thread ("" if none).
PE_API const char* pe_last_error(void) { return pe::g_message; }

// Number of kernels this library has launched since load (or the last reset).
PE_API long long pe_launch_count(void) { return pe::g_launches.load(); }
PE_API void pe_reset_launch_count(void) { pe::g_launches.store(0); }

// ABI version: bump on any signature change.
PE_API int pe_abi_version(void) { return 1; }
