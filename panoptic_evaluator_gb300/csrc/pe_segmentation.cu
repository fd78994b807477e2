// Batched segmentation evaluation over a device table of image descriptors.
//
// Images may differ in size and in segment / detection counts. One update of
// SegmentationEvaluator (combined PQ + mIoU + mask AP with a shared target) is
//   1. seg_sort       per image, stable descending score order of detections;
//                     sorted scores/classes are written straight into the
//                     caller's record store.
//   2. seg_pass       ONE pass over the pixels: target+prediction slot maps
//                     (16-byte loads) feed the privatised G x P pair histogram
//                     and the same target slots bin every detection mask
//                     (16-byte loads of 0/1 bytes, popcount per 16 pixels,
//                     warp-uniform skip of empty rows). Persistent CTAs walk
//                     contiguous runs of 8192-pixel chunks and flush their
//                     shared-memory bins only when the image changes.
//   3. seg_score      per image: areas and validation, then (gated on the
//                     device error word) PQ/confusion accumulation and the
//                     detection areas / thing-class targets for matching.
//   4. match          batched COCO greedy matching (pe_instance.cu), gated too.
// InstanceEvaluator's mask-vs-mask IoU path uses the same table with
// inst_overlap (bit-packed AND + popcount over chunks, order indirection).
#include "pe_common.cuh"
#include "pe_score.cuh"
#include "pe_bins.cuh"
#include "pe_desc.cuh"

#include <cfloat>
#include <map>
#include <mutex>

namespace pe {

int launch_match_gated(const void* pairs, bool pairs_u32, const int64_t* pair_off, const int64_t* d_off,
                       const int64_t* g_off, int64_t B, const int* pc, const double* pa, const int* gc,
                       const double* ga, const uint8_t* crowd, const double* areas, int C, int g_max, int8_t* flags,
                       int64_t chain_stride, int64_t det_stride, int* ranks, int64_t* counts, const int* gate,
                       const uint32_t* class_bits, cudaStream_t stream);

namespace {

constexpr int kPassThreads = 512;
constexpr int kPassPixels = 16;
constexpr int kChunk = kPassThreads * kPassPixels;  // 8192 pixels
constexpr int kSortCap = 4096;
constexpr int kScoreThreads = 512;  // 16 warps per image (0.062 ms for 256 images; 0.082 with 8 warps, 0.066 with 32)
constexpr size_t kScoreStageBytes = 100 * 1024;  // largest G x P histogram staged in shared memory

__device__ __forceinline__ bool score_before(double sa, int ia, double sb, int ib) {
  return sa > sb || (sa == sb && ia < ib);
}

__device__ void bitonic(double* key, int* idx, int n, int padded) {
  for (int i = n + threadIdx.x; i < padded; i += blockDim.x) {
    key[i] = -__longlong_as_double(0x7ff0000000000000ll);
    idx[i] = INT_MAX;
  }
  __syncthreads();
  for (int size = 2; size <= padded; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int i = threadIdx.x; i < padded; i += blockDim.x) {
        const int j = i ^ stride;
        if (j > i) {
          const bool ascending = (i & size) == 0;
          const double ki = key[i], kj = key[j];
          const int ii = idx[i], ij = idx[j];
          if (ascending ? score_before(kj, ij, ki, ii) : score_before(ki, ii, kj, ij)) {
            key[i] = kj; key[j] = ki; idx[i] = ij; idx[j] = ii;
          }
        }
      }
      __syncthreads();
    }
  }
}

// 1. Per-image stable descending score order.
__global__ void __launch_bounds__(256)
seg_sort_kernel(const int64_t* __restrict__ descs, const double* __restrict__ scores, const int* __restrict__ classes,
                int64_t* __restrict__ order, double* __restrict__ sorted_scores, int* __restrict__ sorted_classes,
                double* __restrict__ ws_key, int* __restrict__ ws_idx) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int64_t* d = desc_of(descs, blockIdx.x);
  const int D = (int)d[kD];
  const int64_t base = d[kDetBegin];
  if (D == 0) return;
  int padded = 1;
  while (padded < D) padded <<= 1;
  const bool in_smem = padded <= kSortCap;
  double* key = in_smem ? reinterpret_cast<double*>(smem_raw) : ws_key + 2 * base;
  int* idx = in_smem ? reinterpret_cast<int*>(smem_raw + sizeof(double) * kSortCap) : ws_idx + 2 * base;
  for (int i = threadIdx.x; i < D; i += blockDim.x) {
    key[i] = scores[base + i];
    idx[i] = i;
  }
  __syncthreads();
  bitonic(key, idx, D, padded);
  for (int r = threadIdx.x; r < D; r += blockDim.x) {
    const int i = idx[r];
    order[base + r] = i;
    sorted_scores[base + r] = key[r];
    sorted_classes[base + r] = classes[base + i];
  }
}

// Tunables of the fused pass (compile-time): masks per look-ahead group, and
// whether the first group is requested before the slot maps are consumed.
#ifndef PE_PASS_GROUP
#define PE_PASS_GROUP 4
#endif
#ifndef PE_PASS_PRELOAD
#define PE_PASS_PRELOAD 1
#endif
#ifndef PE_PASS_MIN_BLOCKS
#define PE_PASS_MIN_BLOCKS 1
#endif
constexpr int kGroup = PE_PASS_GROUP;

// 2. The fused pixel pass: one read of both slot maps and every detection mask.
__global__ void __launch_bounds__(kPassThreads, PE_PASS_MIN_BLOCKS)
seg_pass_kernel(const int64_t* __restrict__ descs, int64_t B, int64_t total_chunks, int64_t chunks_per_cta,
                const int64_t* __restrict__ bounds,
                const int64_t* __restrict__ order, u32* __restrict__ pairs, u32* __restrict__ dpairs,
                int* __restrict__ error) {
  // Contiguous chunk range of this CTA: host-balanced bounds, or an even split.
  const int64_t c_begin = bounds ? bounds[blockIdx.x] : (int64_t)blockIdx.x * chunks_per_cta;
  const int64_t c_end = bounds ? min(bounds[blockIdx.x + 1], total_chunks) : min(c_begin + chunks_per_cta, total_chunks);
  if (c_begin >= c_end) return;
  int64_t b = image_of_chunk(descs, B, c_begin);
  bool bad = false;
  const int lane = threadIdx.x & 31;
  int64_t chunk = c_begin;
  while (chunk < c_end) {
    const int64_t* d = desc_of(descs, b);
    const int64_t first = d[kChunkBegin];
    const int64_t pixels = d[kPixels];
    const int64_t last = first + ceil_div(pixels, kChunk);  // exclusive
    if (chunk >= last) { ++b; continue; }
    const int G = (int)d[kG], P = (int)d[kP], D = (int)d[kD];
    const int* target = reinterpret_cast<const int*>(d[kTarget]);
    const int* pred = reinterpret_cast<const int*>(d[kPred]);
    const uint8_t* masks = reinterpret_cast<const uint8_t*>(d[kMasks]);
    const int64_t stride = d[kMaskStride];
    const int64_t* ord = order + d[kDetBegin];
    const bool vec_maps = d[kFlags] & 1, vec_masks = d[kFlags] & 2;
    const ImageOut out{pairs + d[kPairBegin], dpairs + d[kDPairBegin], (u32)(G * P)};
    const int64_t stop = min(last, c_end);
    for (; chunk < stop; ++chunk) {
      const int64_t x = (chunk - first) * kChunk + (int64_t)threadIdx.x * kPassPixels;
      const int64_t xm = x < pixels ? x : pixels;
      uint4 cur[kGroup], nxt[kGroup];
      if (PE_PASS_PRELOAD) {  // first group of masks in flight before the slot maps are consumed
#pragma unroll
        for (int k = 0; k < kGroup; ++k)
          cur[k] = k < D ? load16_stream(masks + ord[k] * stride, xm, pixels, vec_masks) : make_uint4(0, 0, 0, 0);
      }
      int t[16];
      {
        int p[16];
        load16_maps(target, x, pixels, vec_maps, t);
        if (pred) load16_maps(pred, x, pixels, vec_maps, p);
        u32 run_key = kEmpty, run_count = 0;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          if (x + j >= pixels) continue;
          const bool tv = t[j] >= 0 && t[j] < G;
          const bool pv = !pred || (p[j] >= 0 && p[j] < P);
          if (!tv || !pv) { bad = true; continue; }
          if (pred) {
            const u32 key = (u32)(t[j] * P + p[j]);
            if (key != run_key) {
              if (run_count) global_add(out, run_key, run_count);
              run_key = key;
              run_count = 0;
            }
            ++run_count;
          }
        }
        if (pred) {
          const u32 peers = __match_any_sync(0xffffffffu, run_key);
          const u32 total = __reduce_add_sync(peers, run_count);
          if (lane == (int)(__ffs(peers) - 1) && total) global_add(out, run_key, total);
        }
      }
      if (!PE_PASS_PRELOAD) {
#pragma unroll
        for (int k = 0; k < kGroup; ++k)
          cur[k] = k < D ? load16_stream(masks + ord[k] * stride, xm, pixels, vec_masks) : make_uint4(0, 0, 0, 0);
      }
      const LaneSlots ls = lane_slots(t, x, pixels, G);
      // Detections: groups of kGroup masks with one group of look-ahead; one
      // warp-wide OR tells which masks of the group have any pixel here.
      for (int r0 = 0; r0 < D; r0 += kGroup) {
#pragma unroll
        for (int k = 0; k < kGroup; ++k) {
          const int r = r0 + kGroup + k;
          nxt[k] = r < D ? load16_stream(masks + ord[r] * stride, xm, pixels, vec_masks) : make_uint4(0, 0, 0, 0);
        }
        u32 bits = 0;
#pragma unroll
        for (int k = 0; k < kGroup; ++k) bits |= (u32)((cur[k].x | cur[k].y | cur[k].z | cur[k].w) != 0) << k;
        const u32 warp_bits = __reduce_or_sync(0xffffffffu, bits);
#pragma unroll
        for (int k = 0; k < kGroup; ++k)
          if ((warp_bits >> k) & 1u) bin_detection(out, ls, t, cur[k], r0 + k, G, lane);  // uniform across the warp
#pragma unroll
        for (int k = 0; k < kGroup; ++k) cur[k] = nxt[k];
      }
    }
    ++b;
  }
  if (bad && error) atomicOr(error, 1);
}

// 2b. The fused pass as a bulk-copy pipeline. ANY_ALIGN = false: every mask
// row starts on a 16-byte boundary (e.g. a ragged.SegmentationImages arena);
// true: rows at any byte offset, the producer copies the aligned 16-byte words
// covering each row segment and the consumers re-align them by the row's offset.
// Warp 8 is the producer: one lane takes 8192-pixel chunks, publishes each
// 4096-pixel half (image, first pixel) in a small queue of kHalfRing entries,
// prefetches its slot maps into L2 and streams its 4096-byte mask-row segments
// into a ring of kRing shared-memory slots with cp.async.bulk, completing on
// per-slot "full" mbarriers. Chunks come from a global counter (`schedule`,
// one atomicAdd per chunk), so CTAs that run faster take more of them, or,
// without a counter, from a contiguous range per CTA. Warps 0-7 consume: they
// take the next half from the queue, read the target/prediction slots of their
// 16 pixels with plain loads (kept in registers), then take each mask segment
// from the ring, bin it exactly as the register path does and release the slot
// on its "empty" mbarrier. All counts are integer atomics, so the result does
// not depend on which CTA took which chunk. Every wait is bounded by kWaitLimit
// clock cycles; a timeout sets bit 30 of *error, the producer waits for its
// copies in flight, and all roles return.
constexpr int kBulkConsumers = 256;
constexpr int kBulkThreads = kBulkConsumers + 32;
constexpr int kHalf = kBulkConsumers * kPassPixels;  // 4096 pixels per step
constexpr int kStageMasks = 4;  // mask-row segments per ring stage (one barrier each)
constexpr int kRing = 4;        // stages in flight per CTA
constexpr int kHalfRing = 4;    // published halves in flight per CTA
constexpr long long kWaitLimit = 4000000000ll;  // about two seconds of SM clock
constexpr int kTimeoutBit = 1 << 30;

struct BulkShared {
  unsigned char ring[kRing][kStageMasks][kHalf + 16];  // the aligned words covering each row segment
  unsigned char shift[kRing][kStageMasks];             // each row's start offset mod 16
  int64_t half_x0[kHalfRing];     // first pixel of the half
  int64_t half_image[kHalfRing];  // image index; -1 ends the CTA's work
  uint64_t full[kRing];
  uint64_t empty[kRing];
  uint64_t half_full[kHalfRing];
  uint64_t half_empty[kHalfRing];
  int abort;
};

template <bool ANY_ALIGN>
__global__ void __launch_bounds__(kBulkThreads, 2)
seg_pass_bulk_kernel(const int64_t* __restrict__ descs, int64_t B, int64_t total_chunks, int64_t chunks_per_cta,
                     const int64_t* __restrict__ bounds, unsigned long long* __restrict__ schedule, int grab,
                     const int64_t* __restrict__ order, u32* __restrict__ pairs, u32* __restrict__ dpairs,
                     int* __restrict__ error) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  BulkShared& sm = *reinterpret_cast<BulkShared*>(smem_raw);
  // Without a counter: a contiguous chunk range per CTA (host-balanced bounds, or an even split).
  const int64_t c_begin = bounds ? bounds[blockIdx.x] : (int64_t)blockIdx.x * chunks_per_cta;
  const int64_t c_end = bounds ? min(bounds[blockIdx.x + 1], total_chunks) : min(c_begin + chunks_per_cta, total_chunks);
  if (!schedule && c_begin >= c_end) return;
  if (threadIdx.x == 0) {
    for (int i = 0; i < kRing; ++i) {
      mbar_init(&sm.full[i], 1);
      mbar_init(&sm.empty[i], kBulkConsumers / 32);
    }
    for (int i = 0; i < kHalfRing; ++i) {
      mbar_init(&sm.half_full[i], 1);
      mbar_init(&sm.half_empty[i], kBulkConsumers / 32);
    }
    sm.abort = 0;
    mbar_fence_init();
  }
  __syncthreads();
  volatile int* abort = &sm.abort;

  if (threadIdx.x >= kBulkConsumers) {
    // ---- producer --------------------------------------------------------
    if (threadIdx.x != kBulkConsumers) return;
    int64_t seq = 0, halves = 0, next = c_begin;
    int64_t grabbed = 0, grab_end = 0;  // with a counter: the current grab of `grab` consecutive chunks
    bool ok = true;
    // Publish the next half (image -1: no more work); false when the wait for a free entry fails.
    auto publish = [&](int64_t image, int64_t x0) {
      const int h = (int)(halves % kHalfRing);
      const int64_t use = halves / kHalfRing;
      if ((use > 0 && !mbar_wait(&sm.half_empty[h], (uint32_t)((use - 1) & 1), kWaitLimit)) || *abort) return false;
      sm.half_x0[h] = x0;
      sm.half_image[h] = image;
      mbar_arrive(&sm.half_full[h]);  // release: the entry is visible to consumers that see the phase
      ++halves;
      return true;
    };
    while (ok) {
      int64_t chunk;
      if (schedule) {
        if (grabbed == grab_end) {
          grabbed = (int64_t)atomicAdd(schedule, (unsigned long long)grab);
          grab_end = min(grabbed + grab, total_chunks);
        }
        chunk = grabbed < grab_end ? grabbed++ : total_chunks;
      } else {
        chunk = next < c_end ? next++ : total_chunks;
      }
      if (chunk >= total_chunks) break;
      const int64_t b = image_of_chunk(descs, B, chunk);
      const int64_t* d = desc_of(descs, b);
      const int64_t first = d[kChunkBegin], pixels = d[kPixels];
      const int D = (int)d[kD];
      const int* target = reinterpret_cast<const int*>(d[kTarget]);
      const int* pred = reinterpret_cast<const int*>(d[kPred]);
      const uint8_t* masks = reinterpret_cast<const uint8_t*>(d[kMasks]);
      const int64_t stride = d[kMaskStride];
      const int64_t* ord = order + d[kDetBegin];
      const bool vec_maps = d[kFlags] & 1;
      for (int half = 0; half < kChunk / kHalf && ok; ++half) {
        const int64_t x0 = (chunk - first) * kChunk + (int64_t)half * kHalf;
        if (x0 >= pixels) break;
        if (!publish(b, x0)) {
          ok = false;
          break;
        }
        const int64_t len = min((int64_t)kHalf, pixels - x0);
        const uint32_t map_bytes = (uint32_t)((len * 4) & ~15ll);
        if (vec_maps && map_bytes) {
          bulk_prefetch_l2(target + x0, map_bytes);
          if (pred) bulk_prefetch_l2(pred + x0, map_bytes);
        }
        for (int r0 = 0; r0 < D; r0 += kStageMasks) {
          const int slot = (int)(seq % kRing);
          const int64_t use = seq / kRing;
          if ((use > 0 && !mbar_wait(&sm.empty[slot], (uint32_t)((use - 1) & 1), kWaitLimit)) || *abort) {
            ok = false;
            break;
          }
          const int n = min(kStageMasks, D - r0);
          // Rows may start at any byte: copy the aligned words from the one holding pixel x0 to the
          // one holding the segment's last byte; the consumers re-align by the row's offset.
          if constexpr (ANY_ALIGN) {
            const uint8_t* rows[kStageMasks];
            uint32_t total = 0;
            for (int k = 0; k < n; ++k) {
              rows[k] = masks + ord[r0 + k] * stride + x0;
              const int o = (int)(reinterpret_cast<uintptr_t>(rows[k]) & 15);
              sm.shift[slot][k] = (unsigned char)o;
              total += (uint32_t)round_up(len + o, 16);
            }
            mbar_arrive_expect_tx(&sm.full[slot], total);  // release: the offsets are visible with the phase
            for (int k = 0; k < n; ++k) {
              const int o = sm.shift[slot][k];
              bulk_copy_g2s(sm.ring[slot][k], rows[k] - o, (uint32_t)round_up(len + o, 16), &sm.full[slot]);
            }
          } else {  // every row starts on a 16-byte boundary
            const uint32_t bytes = (uint32_t)round_up(len, 16);
            mbar_arrive_expect_tx(&sm.full[slot], bytes * (uint32_t)n);
            for (int k = 0; k < n; ++k)
              bulk_copy_g2s(sm.ring[slot][k], masks + ord[r0 + k] * stride + x0, bytes, &sm.full[slot]);
          }
          ++seq;
        }
      }
    }
    if (ok) ok = publish(-1, 0);
    if (!ok) {
      *abort = 1;
      atomicOr(error, kTimeoutBit);
    }
    // Wait for the copies still in flight into this CTA's shared memory.
    for (int64_t q = seq > kRing ? seq - kRing : 0; q < seq; ++q)
      mbar_wait(&sm.full[q % kRing], (uint32_t)((q / kRing) & 1), kWaitLimit);
    return;
  }

  // ---- consumers ---------------------------------------------------------
  const int ctid = threadIdx.x, lane = ctid & 31;
  int64_t seq = 0, halves = 0;
  bool ok = true, bad = false;
  while (ok) {
    const int h = (int)(halves % kHalfRing);
    const bool ready = mbar_wait(&sm.half_full[h], (uint32_t)((halves / kHalfRing) & 1), kWaitLimit);
    if (!__all_sync(0xffffffffu, ready && !*abort)) {
      ok = false;
      break;
    }
    const int64_t b = sm.half_image[h], x0 = sm.half_x0[h];
    __syncwarp();
    if (lane == 0) mbar_arrive(&sm.half_empty[h]);
    ++halves;
    if (b < 0) break;
    const int64_t* d = desc_of(descs, b);
    const int64_t pixels = d[kPixels];
    const int G = (int)d[kG], P = (int)d[kP], D = (int)d[kD];
    const int* target = reinterpret_cast<const int*>(d[kTarget]);
    const int* pred = reinterpret_cast<const int*>(d[kPred]);
    const bool vec_maps = d[kFlags] & 1;
    const ImageOut out{pairs + d[kPairBegin], dpairs + d[kDPairBegin], (u32)(G * P)};
    const int64_t len = min((int64_t)kHalf, pixels - x0);
    const int64_t x = x0 + (int64_t)ctid * kPassPixels;
    int t[16];
    {
      int p[16];
      load16_maps(target, x, pixels, vec_maps, t);
      if (pred) load16_maps(pred, x, pixels, vec_maps, p);
      u32 run_key = kEmpty, run_count = 0;
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        if (x + j >= pixels) continue;
        const bool tv = t[j] >= 0 && t[j] < G;
        const bool pv = !pred || (p[j] >= 0 && p[j] < P);
        if (!tv || !pv) { bad = true; continue; }
        if (pred) {
          const u32 key = (u32)(t[j] * P + p[j]);
          if (key != run_key) {
            if (run_count) global_add(out, run_key, run_count);
            run_key = key;
            run_count = 0;
          }
          ++run_count;
        }
      }
      if (pred) {
        const u32 peers = __match_any_sync(0xffffffffu, run_key);
        const u32 total = __reduce_add_sync(peers, run_count);
        if (lane == (int)(__ffs(peers) - 1) && total) global_add(out, run_key, total);
      }
    }
    const bool in_range = x < x0 + len;
    const LaneSlots ls = lane_slots(t, x, pixels, G);
    for (int r0 = 0; r0 < D; r0 += kStageMasks) {
      const int slot = (int)(seq % kRing);
      const bool got = mbar_wait(&sm.full[slot], (uint32_t)((seq / kRing) & 1), kWaitLimit);
      if (!__all_sync(0xffffffffu, got && !*abort)) {  // warp-uniform decision
        ok = false;
        break;
      }
      const int n = min(kStageMasks, D - r0);
      uint4 w[kStageMasks];
      u32 bits = 0;
#pragma unroll
      for (int k = 0; k < kStageMasks; ++k) {
        w[k] = make_uint4(0, 0, 0, 0);
        if (in_range && k < n) {
          const uint4* words = reinterpret_cast<const uint4*>(&sm.ring[slot][k][ctid * kPassPixels]);
          if constexpr (ANY_ALIGN) {
            const int o = sm.shift[slot][k];  // the same for the whole warp
            w[k] = o ? realign16(words[0], words[1], o) : words[0];
          } else {
            w[k] = words[0];
          }
        }
        bits |= (u32)((w[k].x | w[k].y | w[k].z | w[k].w) != 0) << k;
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&sm.empty[slot]);
      ++seq;
      const u32 warp_bits = __reduce_or_sync(0xffffffffu, bits);
      if (!warp_bits) continue;
#pragma unroll
      for (int k = 0; k < kStageMasks; ++k)
        if ((warp_bits >> k) & 1u) bin_detection(out, ls, t, w[k], r0 + k, G, lane);  // uniform across the warp
    }
  }
  if (!ok) {
    *abort = 1;
    if (lane == 0) atomicOr(error, kTimeoutBit);
  }
  if (bad && error) atomicOr(error, 1);
}

// 3. Per-image scoring. mode bit 1: areas + validation, bit 2: accumulate
// (gated by *error when bit 4 is set).
__global__ void __launch_bounds__(kScoreThreads)
seg_score_kernel(const int64_t* __restrict__ descs, const u32* __restrict__ pairs, const u32* __restrict__ dpairs,
                 const int* __restrict__ gc, const int* __restrict__ pc, const uint8_t* __restrict__ crowd,
                 u64* __restrict__ areas, int* __restrict__ matched, ScoreOut out, int C,
                 const uint8_t* __restrict__ isthing, const int* __restrict__ det_classes,
                 const double* __restrict__ det_scores, double* __restrict__ det_pa, double* __restrict__ slot_ga,
                 int* __restrict__ slot_class, const double* __restrict__ ann_in, double* __restrict__ ann_out,
                 int mode, int validate, int reward, int stage_pairs, int hist_off, u32* __restrict__ class_bits,
                 int* __restrict__ error) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  if ((mode & 4) && *reinterpret_cast<volatile int*>(error)) return;
  const int64_t* d = desc_of(descs, blockIdx.x);
  const int G = (int)d[kG], P = (int)d[kP], D = (int)d[kD];
  const int64_t sb = d[kSlotBegin], pb = d[kPSlotBegin], db = d[kDetBegin];
  const u32* pan = pairs + d[kPairBegin];
  // The image's G x P histogram in shared memory when it fits (coalesced once; every later pass reads it
  // there), else read in place.
  const bool staged = P > 0 && (int64_t)G * P <= stage_pairs;
  if (staged) {
    u32* hs = reinterpret_cast<u32*>(smem_raw + hist_off);
    stage_counts(hs, pan, G * P);
    __syncthreads();
    pan = hs;
  }
  const u32* det = dpairs + d[kDPairBegin];
  gc += sb; crowd += sb; matched += sb;
  pc += pb;
  u64* ar = areas + sb + pb;  // per image G + P entries at offset (slot_begin + pslot_begin)
  if (mode & 1) {
    int err = 0;
    if (P > 0)
      err = reward ? score_areas<u32, true>(pan, gc, pc, crowd, ar, G, P, C, validate)
                   : score_areas<u32, false>(pan, gc, pc, crowd, ar, G, P, C, validate);
    // Detection areas (full mask area: every slot, including void and stuff): a warp sums the rows
    // of kAreaRows detections at once with coalesced loads, so their L2 round trips overlap.
    constexpr int kAreaRows = 4;
    const int lane = threadIdx.x & 31, warps = blockDim.x >> 5;
    for (int r0 = threadIdx.x >> 5; r0 < D; r0 += kAreaRows * warps) {
      u64 sum[kAreaRows];
#pragma unroll
      for (int j = 0; j < kAreaRows; ++j) sum[j] = 0;
      for (int s = lane; s < G; s += 32) {
#pragma unroll
        for (int j = 0; j < kAreaRows; ++j) {
          const int r = r0 + j * warps;
          if (r < D) sum[j] += det[(int64_t)r * G + s];
        }
      }
#pragma unroll
      for (int j = 0; j < kAreaRows; ++j) {
        const int r = r0 + j * warps;
#pragma unroll
        for (int off = 16; off; off >>= 1) sum[j] += __shfl_xor_sync(0xffffffffu, sum[j], off);
        if (lane || r >= D) continue;
        det_pa[db + r] = (double)sum[j];
        if (validate) {
          const int c = det_classes[db + r];
          if (c < 0 || c >= C || !isthing[c]) err |= 8;
          if (sum[j] == 0) err |= 16;
          const double sc = det_scores[db + r];
          if (!(sc == sc) || sc == __longlong_as_double(0x7ff0000000000000ll) ||
              sc == -__longlong_as_double(0x7ff0000000000000ll))
            err |= 32;
        }
      }
    }
    if (validate && ann_in) {
      for (int s = threadIdx.x; s < G; s += blockDim.x) {
        const double v = ann_in[sb + s];
        if (!(v >= 0.0) || v == __longlong_as_double(0x7ff0000000000000ll)) err |= 64;
      }
    }
    if (err) atomicOr(error, err);
    __syncthreads();
  }
  if (!(mode & 2)) return;
  if (reward) {  // per-image rows [B][C], no confusion (evaluator.py:497-538)
    const int64_t o = (int64_t)blockIdx.x * C;
    ScoreOut row{out.tp + o, out.fp + o, out.fn + o, out.iou_sum + o, nullptr};
    if (staged) score_accumulate_warps<true>(pan, gc, pc, crowd, ar, matched, G, P, C, row, smem_raw);
    else if (P > 0) score_accumulate<u32, true>(pan, gc, pc, crowd, ar, matched, G, P, C, row, smem_raw);
    return;
  }
  if (staged) score_accumulate_warps<false>(pan, gc, pc, crowd, ar, matched, G, P, C, out, smem_raw);
  else if (P > 0) score_accumulate<u32, false>(pan, gc, pc, crowd, ar, matched, G, P, C, out, smem_raw);
  // Classes present in the image for the matching (per-image bits): thing targets, and detections
  // (a class outside [0, C) marks class 0, whose matching warp handles such detections).
  u32* bits = class_bits ? class_bits + (int64_t)blockIdx.x * ((C + 31) / 32) : nullptr;
  if (bits) {
    for (int w = threadIdx.x; w < (C + 31) / 32; w += blockDim.x) bits[w] = 0;
    __syncthreads();
    for (int r = threadIdx.x; r < D; r += blockDim.x) {
      const int c = det_classes[db + r];
      const int k = c >= 0 && c < C ? c : 0;
      atomicOr(bits + (k >> 5), 1u << (k & 31));
    }
  }
  // Targets for matching: thing classes only, pixel areas, annotation areas.
  for (int s = threadIdx.x; s < G; s += blockDim.x) {
    const int c = gc[s];
    const int clamped = c < 0 ? 0 : (c >= C ? C - 1 : c);
    slot_class[sb + s] = (c >= 0 && isthing[clamped]) ? c : -1;
    if (bits && c >= 0 && c < C && isthing[c]) atomicOr(bits + (c >> 5), 1u << (c & 31));
    const double area = (double)ar[s];
    slot_ga[sb + s] = area;
    ann_out[sb + s] = ann_in ? ann_in[sb + s] : area;
  }
}

// Mask-vs-mask overlaps for InstanceEvaluator (pixel chunks of 4096).
constexpr int kOvThreads = 256;
constexpr int kOvWords = 128;

__device__ __forceinline__ uint32_t pack4(uint32_t w) { return (((w & 0x01010101u) * 0x08040201u) >> 24) & 0xfu; }

__global__ void __launch_bounds__(kOvThreads)
inst_overlap_kernel(const int64_t* __restrict__ descs, int64_t B, const int64_t* __restrict__ order,
                    const int* __restrict__ pc, const int* __restrict__ gc, u32* __restrict__ inter,
                    u64* __restrict__ pa, u64* __restrict__ ga) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int64_t b = image_of_chunk(descs, B, blockIdx.x);
  const int64_t* d = desc_of(descs, b);
  const int D = (int)d[kD], G = (int)d[kG];
  const int64_t pixels = d[kPixels], stride = d[kMaskStride];
  const uint8_t* pm = reinterpret_cast<const uint8_t*>(d[kMasks]);
  const uint8_t* gm = reinterpret_cast<const uint8_t*>(d[kTarget]);
  const bool vec = d[kFlags] & 2;
  const int64_t db = d[kDetBegin], gb = d[kSlotBegin];
  const int64_t x0 = (blockIdx.x - d[kChunkBegin]) * (int64_t)kOvWords * 32;
  const int rows = D + G;
  uint32_t* bits = reinterpret_cast<uint32_t*>(smem_raw);
  int2* range = reinterpret_cast<int2*>(bits + (int64_t)rows * kOvWords);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int r = warp; r < rows; r += kOvThreads / 32) {
    const uint8_t* row = r < D ? pm + order[db + r] * stride : gm + (int64_t)(r - D) * stride;
    int first = kOvWords, last = -1, ones = 0;
    for (int k = lane; k < kOvWords; k += 32) {
      const int64_t x = x0 + (int64_t)k * 32;
      uint32_t word = 0;
      if (x < pixels) {
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const uint4 w = load16_mask(row, x + 16 * q, pixels, vec);
          word |= (pack4(w.x) | pack4(w.y) << 4 | pack4(w.z) << 8 | pack4(w.w) << 12) << (16 * q);
        }
      }
      bits[(int64_t)r * kOvWords + k] = word;
      ones += __popc(word);
      if (word) { first = min(first, k); last = max(last, k); }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      first = min(first, __shfl_xor_sync(0xffffffffu, first, o));
      last = max(last, __shfl_xor_sync(0xffffffffu, last, o));
      ones += __shfl_xor_sync(0xffffffffu, ones, o);
    }
    if (lane == 0) {
      range[r] = make_int2(first, last);
      if (ones) atomicAdd(r < D ? pa + db + r : ga + gb + (r - D), (u64)ones);
    }
  }
  __syncthreads();
  u32* out = inter + d[kDPairBegin];
  for (int pair = threadIdx.x; pair < D * G; pair += blockDim.x) {
    const int i = pair / G, g = pair % G;
    if (pc[db + i] != gc[gb + g]) continue;
    const int2 rd = range[i], rg = range[D + g];
    const int lo = max(rd.x, rg.x), hi = min(rd.y, rg.y);
    if (lo > hi) continue;
    const uint32_t* a = bits + (int64_t)i * kOvWords;
    const uint32_t* c = bits + (int64_t)(D + g) * kOvWords;
    u32 count = 0;
    for (int k = lo; k <= hi; ++k) count += __popc(a[k] & c[k]);
    if (count) atomicAdd(out + pair, count);
  }
}

// Instance prep: pixel areas to double, validation of classes/scores/areas.
// Per-image metadata of an instance update gathered into flat arrays at each image's detection / slot
// offsets (one launch instead of a host-side concatenation per field). fields: one row of
// kGatherFields int64 per image: device pointers of its prediction classes, scores, target classes,
// crowd flags and annotation areas (0: absent), then element sizes (bit 0: prediction classes int64,
// bit 1: scores float64, bit 2: target classes int64, bit 4: areas float64; else int32 / float32).
constexpr int kGatherFields = 6;

__global__ void __launch_bounds__(128)
inst_gather_kernel(const int64_t* __restrict__ descs, const int64_t* __restrict__ fields, int* __restrict__ pc,
                   double* __restrict__ scores, int* __restrict__ gc, uint8_t* __restrict__ crowd,
                   double* __restrict__ areas) {
  const int64_t* d = desc_of(descs, blockIdx.x);
  const int64_t* f = fields + (int64_t)blockIdx.x * kGatherFields;
  const int D = (int)d[kD], G = (int)d[kG];
  const int64_t db = d[kDetBegin], sb = d[kSlotBegin], bits = f[5];
  for (int i = threadIdx.x; i < D; i += blockDim.x) {
    pc[db + i] = (bits & 1) ? (int)reinterpret_cast<const int64_t*>(f[0])[i] : reinterpret_cast<const int*>(f[0])[i];
    scores[db + i] = (bits & 2) ? reinterpret_cast<const double*>(f[1])[i]
                                : (double)reinterpret_cast<const float*>(f[1])[i];
  }
  for (int g = threadIdx.x; g < G; g += blockDim.x) {
    gc[sb + g] = (bits & 4) ? (int)reinterpret_cast<const int64_t*>(f[2])[g] : reinterpret_cast<const int*>(f[2])[g];
    crowd[sb + g] = f[3] ? reinterpret_cast<const uint8_t*>(f[3])[g] : 0;
    if (areas && f[4])
      areas[sb + g] = (bits & 16) ? reinterpret_cast<const double*>(f[4])[g]
                                  : (double)reinterpret_cast<const float*>(f[4])[g];
  }
}

__global__ void inst_prepare_kernel(const int64_t* __restrict__ descs, const u64* __restrict__ pa_count,
                                    const u64* __restrict__ ga_count, double* __restrict__ pa, double* __restrict__ ga,
                                    const int* __restrict__ pc, const int* __restrict__ gc,
                                    const double* __restrict__ scores, const double* __restrict__ ann_in,
                                    double* __restrict__ ann_out, int C, int validate, u32* __restrict__ class_bits,
                                    int* __restrict__ error) {
  const int64_t* d = desc_of(descs, blockIdx.x);
  const int D = (int)d[kD], G = (int)d[kG];
  const int64_t db = d[kDetBegin], gb = d[kSlotBegin];
  // Classes present in the image for the matching (a detection class outside [0, C) marks class 0).
  u32* bits = class_bits ? class_bits + (int64_t)blockIdx.x * ((C + 31) / 32) : nullptr;
  if (bits) {
    for (int w = threadIdx.x; w < (C + 31) / 32; w += blockDim.x) bits[w] = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < D; i += blockDim.x) {
      const int c = pc[db + i];
      const int k = c >= 0 && c < C ? c : 0;
      atomicOr(bits + (k >> 5), 1u << (k & 31));
    }
    for (int g = threadIdx.x; g < G; g += blockDim.x) {
      const int c = gc[gb + g];
      if (c >= 0 && c < C) atomicOr(bits + (c >> 5), 1u << (c & 31));
    }
  }
  int err = 0;
  const double inf = __longlong_as_double(0x7ff0000000000000ll);
  for (int i = threadIdx.x; i < D; i += blockDim.x) {
    pa[db + i] = (double)pa_count[db + i];
    if (validate) {
      if (pc[db + i] < 0 || pc[db + i] >= C) err |= 8;
      if (pa_count[db + i] == 0) err |= 16;
      const double s = scores[db + i];
      if (!(s == s) || s == inf || s == -inf) err |= 32;
    }
  }
  for (int g = threadIdx.x; g < G; g += blockDim.x) {
    const double area = (double)ga_count[gb + g];
    ga[gb + g] = area;
    ann_out[gb + g] = ann_in ? ann_in[gb + g] : area;
    if (validate) {
      if (gc[gb + g] < 0 || gc[gb + g] >= C) err |= 8;
      if (ga_count[gb + g] == 0) err |= 16;
      if (ann_in) {
        const double v = ann_in[gb + g];
        if (!(v >= 0.0) || v == inf) err |= 64;
      }
    }
  }
  if (err) atomicOr(error, err);
}

}  // namespace
}  // namespace pe

using namespace pe;

PE_API int pe_desc_fields(void) { return kDescFields; }

// Workspace for pe_seg_sort: key/index scratch for images with more than 4096 detections.
PE_API int64_t pe_seg_sort_workspace(int64_t total_detections) {
  return (int64_t)2 * round_up(total_detections + 1, 64) * (int64_t)(sizeof(double) + sizeof(int)) + 256;
}

// Stable descending score order per image (instance.py:139-141). order[det_begin + r]
// is the image-local index of the r-th best detection; sorted scores/classes
// go to the given outputs at det_begin + r.
PE_API int pe_seg_sort(const int64_t* descs, int64_t B, const double* scores, const int32_t* classes,
                       int64_t total_detections, int64_t* order, double* sorted_scores, int32_t* sorted_classes,
                       void* workspace, int64_t workspace_bytes, cudaStream_t stream) {
  PE_REQUIRE(B >= 0 && total_detections >= 0, "invalid batch");
  PE_REQUIRE(workspace_bytes >= pe_seg_sort_workspace(total_detections), "sort workspace too small");
  if (B == 0 || total_detections == 0) return kOk;
  const int64_t entries = 2 * round_up(total_detections + 1, 64);
  double* ws_key = static_cast<double*>(workspace);
  int* ws_idx = reinterpret_cast<int*>(ws_key + entries);
  const size_t smem = (sizeof(double) + sizeof(int)) * kSortCap;
  PE_CUDA(cudaFuncSetAttribute(seg_sort_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  seg_sort_kernel<<<(unsigned)B, 256, smem, stream>>>(descs, scores, classes, order, sorted_scores, sorted_classes,
                                                      ws_key, ws_idx);
  PE_LAUNCHED("seg_sort");
  count_launch();
  return kOk;
}

// The fused pixel pass. pairs (u32, sum of G*P) and dpairs (u32, sum of D*G)
// are zeroed here. pan_cap / det_cap: the largest per-image G*P and D*G.
// schedule (bulk form only, optional): one device u64, zeroed here, from which
// CTAs take chunks dynamically (cta_bounds is then unused).
// Launch choices of the batched pass with a chunk counter, per bucket floor(log2(total chunks)): chunks a
// producer takes per counter grab (1, 2 or 4) and CTAs per SM (1 or 2). Without an entry: 1 and 2.
namespace {
struct PassChoice {
  int grab = 1;
  int per_sm = 2;
};
std::mutex g_pass_mutex;
std::map<int, PassChoice> g_pass_tuning;

int log2_floor(int64_t v) { return v > 0 ? 63 - __builtin_clzll((unsigned long long)v) : -1; }

PassChoice pass_choice(int64_t chunks) {
  std::lock_guard<std::mutex> lock(g_pass_mutex);
  const auto it = g_pass_tuning.find(log2_floor(chunks));
  return it == g_pass_tuning.end() ? PassChoice{} : it->second;
}
}  // namespace

PE_API int pe_tune_pass(int64_t chunks, int grab, int ctas_per_sm) {
  PE_REQUIRE(chunks > 0, "chunks must be positive");
  std::lock_guard<std::mutex> lock(g_pass_mutex);
  if (grab < 0) {
    g_pass_tuning.erase(log2_floor(chunks));
    return kOk;
  }
  PE_REQUIRE(grab == 1 || grab == 2 || grab == 4, "grab must be 1, 2 or 4 chunks");
  PE_REQUIRE(ctas_per_sm == 1 || ctas_per_sm == 2, "ctas_per_sm must be 1 or 2");
  g_pass_tuning[log2_floor(chunks)] = PassChoice{grab, ctas_per_sm};
  return kOk;
}

PE_API int pe_pass_choice(int64_t chunks, int32_t* grab, int32_t* ctas_per_sm) {
  PE_REQUIRE(chunks > 0 && grab && ctas_per_sm, "invalid query");
  const PassChoice c = pass_choice(chunks);
  *grab = c.grab;
  *ctas_per_sm = c.per_sm;
  return kOk;
}

PE_API int pe_seg_pass(const int64_t* descs, int64_t B, int64_t total_chunks, const int64_t* order, uint32_t* pairs,
                       int64_t pairs_len, uint32_t* dpairs, int64_t dpairs_len, int64_t pan_cap, int64_t det_cap,
                       int bulk, const int64_t* cta_bounds, int64_t ctas, uint64_t* schedule, int32_t* error,
                       cudaStream_t stream) {
  PE_REQUIRE(B >= 0 && total_chunks >= 0 && pairs_len >= 0 && dpairs_len >= 0, "invalid batch");
  // Keys of one image are G*P + D*G < 2^32 - 1 (pan_cap, det_cap: largest per-image G*P and D*G).
  PE_REQUIRE(pan_cap >= 0 && det_cap >= 0 && pan_cap + det_cap < (int64_t)UINT32_MAX, "histogram too large");
  if (pairs_len) PE_CUDA(cudaMemsetAsync(pairs, 0, sizeof(uint32_t) * pairs_len, stream));
  if (dpairs_len) PE_CUDA(cudaMemsetAsync(dpairs, 0, sizeof(uint32_t) * dpairs_len, stream));
  if (B == 0 || total_chunks == 0) return kOk;
  PE_REQUIRE(!cta_bounds || (ctas > 0 && ctas <= INT_MAX), "invalid CTA count");
  if (bulk) {
    const PassChoice choice = pass_choice(total_chunks);
    const int64_t max_ctas = (int64_t)sm_count() * 2;
    const int64_t per_cta = ceil_div(total_chunks, std::min(total_chunks, max_ctas));
    int64_t grid = cta_bounds ? ctas : ceil_div(total_chunks, per_cta);
    if (schedule) {  // chunks taken from the counter, `grab` at a time, by the chosen CTAs per SM
      PE_CUDA(cudaMemsetAsync(schedule, 0, sizeof(uint64_t), stream));
      grid = std::min(ceil_div(total_chunks, choice.grab), (int64_t)sm_count() * choice.per_sm);
      cta_bounds = nullptr;
    }
    const size_t smem = sizeof(BulkShared) + 128;
    auto kernel = bulk == 2 ? seg_pass_bulk_kernel<true> : seg_pass_bulk_kernel<false>;
    PE_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kernel<<<(unsigned)grid, kBulkThreads, smem, stream>>>(
        descs, B, total_chunks, per_cta, cta_bounds, reinterpret_cast<unsigned long long*>(schedule), choice.grab,
        order, pairs, dpairs, error);
    PE_LAUNCHED("seg_pass_bulk");
    count_launch();
    return kOk;
  }
  const int64_t max_ctas = (int64_t)sm_count() * PE_PASS_MIN_BLOCKS;
  const int64_t per_cta = ceil_div(total_chunks, std::min(total_chunks, max_ctas));
  const int64_t grid = cta_bounds ? ctas : ceil_div(total_chunks, per_cta);
  seg_pass_kernel<<<(unsigned)grid, kPassThreads, 0, stream>>>(descs, B, total_chunks, per_cta, cta_bounds, order,
                                                               pairs, dpairs, error);
  PE_LAUNCHED("seg_pass");
  count_launch();
  return kOk;
}

// Per-image scoring of the fused pass (see seg_score_kernel). areas: sum of
// (G+P) u64 at slot_begin + pslot_begin; matched: sum of G ints. state: dataset
// tp/fp/fn/iou_sum [C], confusion [C, C+1]. Validation bits: 1/2/4 panoptic,
// 8 detection class not a thing, 16 empty detection, 32 non-finite score,
// 64 invalid annotation area. Accumulation is skipped when any bit is set.
PE_API int pe_seg_score(const int64_t* descs, int64_t B, int64_t max_p, int64_t max_pairs, const uint32_t* pairs,
                        const uint32_t* dpairs,
                        const int32_t* gc, const int32_t* pc, const uint8_t* crowd, int64_t* areas, int32_t* matched,
                        int64_t* tp, int64_t* fp, int64_t* fn, double* iou_sum, int64_t* confusion, int64_t C,
                        const uint8_t* isthing, const int32_t* det_classes, const double* det_scores, double* det_pa,
                        double* slot_ga, int32_t* slot_class, const double* ann_in, double* ann_out, int validate,
                        int reward, uint32_t* class_bits, int32_t* error, cudaStream_t stream) {
  PE_REQUIRE(B >= 0 && C > 0 && C < INT_MAX, "invalid batch");
  u32* bits = reward ? nullptr : reinterpret_cast<u32*>(class_bits);
  if (B == 0) return kOk;
  const size_t base = (score_staging_bytes(std::max<int64_t>(max_p, 1)) + 15) & ~size_t{15};
  PE_REQUIRE(base <= 200 * 1024, "too many prediction slots (P=%lld)", (long long)max_p);
  // Stage histograms up to kScoreStageBytes (two CTAs still fit an SM); larger images read theirs in place.
  const int stage = max_pairs > 0 && (size_t)max_pairs * 4 <= kScoreStageBytes ? (int)max_pairs : 0;
  const size_t smem = base + 4 * (size_t)stage;
  if (smem > 48 * 1024)
    PE_CUDA(cudaFuncSetAttribute(seg_score_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  ScoreOut out{reinterpret_cast<u64*>(tp), reinterpret_cast<u64*>(fp), reinterpret_cast<u64*>(fn), iou_sum,
               reinterpret_cast<u64*>(confusion)};
  auto* ua = reinterpret_cast<u64*>(areas);
  if (validate) {
    seg_score_kernel<<<(unsigned)B, kScoreThreads, smem, stream>>>(descs, pairs, dpairs, gc, pc, crowd, ua, matched,
                                                                   out, (int)C, isthing, det_classes, det_scores,
                                                                   det_pa, slot_ga, slot_class, ann_in, ann_out, 1, 1,
                                                                   reward, stage, (int)base, nullptr, error);
    PE_LAUNCHED("seg_score(areas)");
    seg_score_kernel<<<(unsigned)B, kScoreThreads, smem, stream>>>(descs, pairs, dpairs, gc, pc, crowd, ua, matched,
                                                                   out, (int)C, isthing, det_classes, det_scores,
                                                                   det_pa, slot_ga, slot_class, ann_in, ann_out, 2 | 4,
                                                                   1, reward, stage, (int)base, bits, error);
    PE_LAUNCHED("seg_score(accumulate)");
    count_launch(2);
    return kOk;
  }
  seg_score_kernel<<<(unsigned)B, kScoreThreads, smem, stream>>>(descs, pairs, dpairs, gc, pc, crowd, ua, matched, out,
                                                                 (int)C, isthing, det_classes, det_scores, det_pa,
                                                                 slot_ga, slot_class, ann_in, ann_out, 1 | 2, 0,
                                                                 reward, stage, (int)base, bits, error);
  PE_LAUNCHED("seg_score");
  count_launch();
  return kOk;
}

// Batched greedy matching over the descriptor table, gated on *gate (skipped
// when nonzero). pairs_u32: D x G intersections per image at dpair_begin.
// Offsets are read from device arrays d_off [B+1], g_off [B+1], pair_off [B].
PE_API int pe_seg_match(const uint32_t* pairs, const int64_t* pair_off, const int64_t* d_off, const int64_t* g_off,
                        int64_t B, const int32_t* pc, const double* pa, const int32_t* gc, const double* ga,
                        const uint8_t* crowd, const double* areas, int64_t C, int64_t g_max, int8_t* flags,
                        int64_t chain_stride, int64_t det_stride, int32_t* ranks, int64_t* counts,
                        const int32_t* gate, const uint32_t* class_bits, cudaStream_t stream) {
  PE_REQUIRE(B >= 0 && C > 0 && C <= INT_MAX / 120 && g_max >= 0 && g_max < INT_MAX, "invalid batch");
  return launch_match_gated(pairs, true, pair_off, d_off, g_off, B, pc, pa, gc, ga, crowd, areas, (int)C,
                            (int)std::max<int64_t>(g_max, 1), flags, chain_stride, det_stride, ranks, counts, gate,
                            class_bits, stream);
}

// Mask-vs-mask overlaps and pixel areas for InstanceEvaluator over the
// descriptor table (kTarget = gt masks, kMasks = prediction masks, rows
// kMaskStride bytes apart, kChunkBegin in 4096-pixel chunks). inter (u32,
// sum of D*G) and the area counters pa (sum of D), ga (sum of G) are zeroed here.
PE_API int pe_inst_overlap(const int64_t* descs, int64_t B, int64_t total_chunks, int64_t max_rows,
                           const int64_t* order, const int32_t* pc, const int32_t* gc, uint32_t* inter,
                           int64_t inter_len, uint64_t* pa, int64_t pa_len, uint64_t* ga, int64_t ga_len,
                           cudaStream_t stream) {
  PE_REQUIRE(B >= 0 && total_chunks >= 0, "invalid batch");
  if (inter_len) PE_CUDA(cudaMemsetAsync(inter, 0, sizeof(uint32_t) * inter_len, stream));
  if (pa_len) PE_CUDA(cudaMemsetAsync(pa, 0, sizeof(uint64_t) * pa_len, stream));
  if (ga_len) PE_CUDA(cudaMemsetAsync(ga, 0, sizeof(uint64_t) * ga_len, stream));
  if (B == 0 || total_chunks == 0) return kOk;
  const size_t smem = (size_t)std::max<int64_t>(max_rows, 1) * (kOvWords * sizeof(uint32_t) + sizeof(int2));
  PE_REQUIRE(smem <= 220 * 1024, "too many masks per image for the overlap kernel (%lld)", (long long)max_rows);
  if (smem > 48 * 1024)
    PE_CUDA(cudaFuncSetAttribute(inst_overlap_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  inst_overlap_kernel<<<(unsigned)total_chunks, kOvThreads, smem, stream>>>(descs, B, order, pc, gc, inter,
                                                                            reinterpret_cast<u64*>(pa),
                                                                            reinterpret_cast<u64*>(ga));
  PE_LAUNCHED("inst_overlap");
  count_launch();
  return kOk;
}

// Pixel areas to FP64, annotation areas (given or pixel) and validation
// bits 8 (class), 16 (empty mask), 32 (score), 64 (annotation area).
// Flat instance metadata from per-image tensors (see inst_gather_kernel): pc [sum D] int32, scores
// [sum D] float64, gc / crowd / areas [sum G] (int32, uint8, float64; areas may be NULL).
PE_API int pe_inst_gather(const int64_t* descs, const int64_t* fields, int64_t B, int32_t* pc, double* scores,
                          int32_t* gc, uint8_t* crowd, double* areas, cudaStream_t stream) {
  PE_REQUIRE(B >= 0 && B <= INT_MAX, "invalid batch");
  if (B == 0) return kOk;
  inst_gather_kernel<<<(unsigned)B, 128, 0, stream>>>(descs, fields, pc, scores, gc, crowd, areas);
  PE_LAUNCHED("inst_gather");
  count_launch();
  return kOk;
}

PE_API int pe_inst_prepare(const int64_t* descs, int64_t B, const uint64_t* pa_count, const uint64_t* ga_count,
                           double* pa, double* ga, const int32_t* pc, const int32_t* gc, const double* scores,
                           const double* ann_in, double* ann_out, int64_t C, int validate, uint32_t* class_bits,
                           int32_t* error, cudaStream_t stream) {
  PE_REQUIRE(B >= 0 && C > 0 && C < INT_MAX, "invalid batch");
  if (B == 0) return kOk;
  inst_prepare_kernel<<<(unsigned)B, 128, 0, stream>>>(descs, reinterpret_cast<const u64*>(pa_count),
                                                      reinterpret_cast<const u64*>(ga_count), pa, ga, pc, gc, scores,
                                                      ann_in, ann_out, (int)C, validate,
                                                      reinterpret_cast<u32*>(class_bits), error);
  PE_LAUNCHED("inst_prepare");
  count_launch();
  return kOk;
}
