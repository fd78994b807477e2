// Shared helpers for the sm_103a kernels behind the pe_gb300 C ABI.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <cstdarg>
#include <climits>
#include <algorithm>

#include "pe_gb300.h"

#define PE_API extern "C" __attribute__((visibility("default")))

namespace pe {

using u64 = unsigned long long;
using u32 = unsigned int;

// Status codes shared by every entry point. Positive values are validation
// bitmasks with the reference's bit meanings (1: unknown ID / slot outside
// capacity, 2: bad class or slot 0 not void, 4: area/metadata mismatch).
enum Status : int {
  kOk = 0,
  kBadArgument = -1,
  kCudaError = -2,
  kWorkspaceTooSmall = -3,
  kUnsupported = -4,
};

void set_error(const char* fmt, ...);

#define PE_REQUIRE(cond, ...)                  \
  do {                                         \
    if (!(cond)) {                             \
      ::pe::set_error(__VA_ARGS__);            \
      return ::pe::kBadArgument;               \
    }                                          \
  } while (0)

#define PE_CUDA(call)                                                     \
  do {                                                                    \
    cudaError_t _e = (call);                                              \
    if (_e != cudaSuccess) {                                              \
      ::pe::set_error("%s failed: %s", #call, cudaGetErrorString(_e));    \
      return ::pe::kCudaError;                                            \
    }                                                                     \
  } while (0)

#define PE_LAUNCHED(name)                                                        \
  do {                                                                           \
    cudaError_t _e = cudaGetLastError();                                         \
    if (_e != cudaSuccess) {                                                     \
      ::pe::set_error("launch of %s failed: %s", name, cudaGetErrorString(_e));  \
      return ::pe::kCudaError;                                                   \
    }                                                                            \
  } while (0)

int sm_count();            // SMs of the current device (cached per device)
int current_device();
void count_launch(int n = 1);  // launch counter exposed through pe_launch_count()

__host__ __device__ inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }
__host__ __device__ inline int64_t round_up(int64_t a, int64_t b) { return ceil_div(a, b) * b; }

// ---- device helpers --------------------------------------------------------

// Warp-aggregated add: lanes holding the same key combine their values and
// one leader issues the atomic. Every lane of `active` must call it.
__device__ __forceinline__ void warp_add_shared(u32* bins, u32 active, u32 key, u32 value) {
  u32 peers = __match_any_sync(active, key);
  u32 total = __reduce_add_sync(peers, value);
  if ((threadIdx.x & 31) == (u32)(__ffs(peers) - 1)) atomicAdd(bins + key, total);
}

__device__ __forceinline__ void warp_add_global(u64* bins, u32 active, u64 key, u32 value) {
  u32 peers = __match_any_sync(active, key);
  u32 total = __reduce_add_sync(peers, value);
  if ((threadIdx.x & 31) == (u32)(__ffs(peers) - 1)) atomicAdd(bins + key, (u64)total);
}

// Slot of a map value. Without tables a value is its own slot when inside
// [0, S). With tables (sorted original IDs `ids[0..S)`, ids[0] = 0 for void)
// the slot comes from a binary search over ids[1..S), as the reference's
// lookup does (histogram_kernel.cu:25-38). Returns -1 when invalid.
__device__ __forceinline__ int resolve_slot(int64_t key, const int64_t* ids, const int* slots, int S) {
  if (ids == nullptr) return (key >= 0 && key < S) ? (int)key : -1;
  if (key == 0) return 0;
  if (key < 0 || key == INT64_MAX) return -1;
  int lo = 1, hi = S;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (ids[mid] < key) lo = mid + 1; else hi = mid;
  }
  if (lo == S || ids[lo] != key) return -1;
  int slot = slots[lo];
  return (slot > 0 && slot < S) ? slot : -1;
}

// ---- asynchronous copies and mbarriers (sm_90+ PTX) ------------------------

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Make barrier initialisation visible to the async proxy before first use.
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// Wait for the phase of `bar` with the given parity; false after ~`limit`
// SM clock cycles (the caller then reports a timeout instead of hanging).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long limit) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long start = clock64();
  while (!mbar_try_wait(bar, parity))
    if (clock64() - start > limit) return false;
  return true;
}

// Bulk (non-tensor) copy global -> shared, completing `bytes` on `bar`.
// Both addresses 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// Hint: bring [src, src + bytes) into L2 (16-byte aligned, multiple of 16).
__device__ __forceinline__ void bulk_prefetch_l2(const void* src, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

// Barrier among the first `threads` threads of the CTA (named barrier `id`).
__device__ __forceinline__ void named_sync(int id, int threads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(threads) : "memory");
}

// Bytes [o, o + 16) of the 32-byte string lo|hi (little-endian words), o in [0, 16): shifts by 8, 4
// and 0-3 bytes as selects and funnel shifts, with no branches (o may differ between lanes).
__device__ __forceinline__ uint4 realign16(uint4 lo, uint4 hi, int o) {
  uint32_t u0 = lo.x, u1 = lo.y, u2 = lo.z, u3 = lo.w, u4 = hi.x, u5 = hi.y, u6 = hi.z, u7 = hi.w;
  const bool b8 = o & 8, b4 = o & 4;
  u0 = b8 ? u2 : u0; u1 = b8 ? u3 : u1; u2 = b8 ? u4 : u2; u3 = b8 ? u5 : u3; u4 = b8 ? u6 : u4; u5 = b8 ? u7 : u5;
  u0 = b4 ? u1 : u0; u1 = b4 ? u2 : u1; u2 = b4 ? u3 : u2; u3 = b4 ? u4 : u3; u4 = b4 ? u5 : u4;
  const int sh = (o & 3) * 8;
  return make_uint4(__funnelshift_r(u0, u1, sh), __funnelshift_r(u1, u2, sh), __funnelshift_r(u2, u3, sh),
                    __funnelshift_r(u3, u4, sh));
}

}  // namespace pe
