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
PE_API int pe_abi_version(void) { return 2; }

namespace pe {
namespace {

// One thread waits on an mbarrier of its own with the bounded wait the pipelined kernels use; with
// `complete` it arrives first (the phase completes), else nothing ever arrives and the wait gives up
// after `limit` clock cycles. Bit 30 of *error reports the timeout. No asynchronous copy or tensor
// memory is involved, so the CTA simply returns.
__global__ void wait_selftest_kernel(long long limit, int complete, int* error) {
  __shared__ uint64_t bar;
  if (threadIdx.x != 0) return;
  mbar_init(&bar, 1);
  mbar_fence_init();
  if (complete) mbar_arrive(&bar);
  if (!mbar_wait(&bar, 0, limit)) atomicOr(error, 1 << 30);
}

}  // namespace
}  // namespace pe

// Diagnostics (no reference counterpart): exercises the bounded mbarrier wait on the device.
// *error is zeroed, then bit 30 is set when the wait timed out; limit_cycles in [1, 2^32].
PE_API int pe_wait_selftest(int64_t limit_cycles, int complete, int32_t* error, cudaStream_t stream) {
  PE_REQUIRE(limit_cycles >= 1 && limit_cycles <= (int64_t)1 << 32, "limit_cycles must be in [1, 2^32]");
  PE_CUDA(cudaMemsetAsync(error, 0, sizeof(int32_t), stream));
  pe::wait_selftest_kernel<<<1, 32, 0, stream>>>((long long)limit_cycles, complete, error);
  PE_LAUNCHED("wait_selftest");
  pe::count_launch();
  return pe::kOk;
}
