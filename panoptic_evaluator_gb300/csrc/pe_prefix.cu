// Generation-order prefix evaluation (segmentation_prefixes) for many images.
//
// The reference draws masks one launch at a time and scores each step with a
// single CTA (prefix_kernel.cu:142-199: 2N+1 launches per image). Here every
// batch is six launches, whatever the number of images or masks:
//   1. prefix_pass   one read of the target map and of every mask byte. Each
//                    lane tracks the visible owner of its 16 pixels (the last
//                    mask drawn over them) and, at every requested checkpoint,
//                    emits the owner transitions since the previous checkpoint
//                    into per-checkpoint delta histograms [Q][G][N+1]. The same
//                    pass counts target areas and the raw mask x slot
//                    intersections used by instance matching.
//   2. prefix_scan   running sums over checkpoints turn deltas into the canvas
//                    pair histograms (column 0 starts with the target areas).
//   3. prefix_score  one CTA per (image, checkpoint): canvas PQ / confusion with
//                    active labels (segments with visible pixels), shared with
//                    the panoptic evaluator's scoring code.
//   4. prefix_match  one CTA per image, one warp per IoU threshold: greedy
//                    generation-order matching (prefix.py:106-118), snapshots
//                    of TP/FP/FN at the checkpoints; prefix_ratio then turns
//                    them into precision / recall over the whole grid.
//   5. pe_compute    per-checkpoint PQ/SQ/RQ/IoU summaries.
#include "pe_common.cuh"
#include "pe_score.cuh"
#include "pe_bins.cuh"

namespace pe {
namespace {

// Descriptor fields (int64 each).
enum : int {
  kPTarget = 0,   // int32 target slot map
  kPMasks,        // uint8 0/1 masks in generation order, rows kPStride bytes apart
  kPPixels,
  kPStride,
  kPChunkBegin,   // first 4096-pixel chunk of this image
  kPN,            // masks
  kPG,            // target slots
  kPDetBegin,     // offset into flat per-mask arrays (classes) and raw rows / N
  kPSlotBegin,    // offset into flat per-slot arrays (gc, crowd, ga)
  kPQBegin,       // first output row (checkpoint) of this image
  kPQ,            // checkpoints of this image
  kPPairBegin,    // offset of this image's [Q][G][N+1] histograms
  kPRawBegin,     // offset of this image's [N][G] raw intersections
  kPFlags,        // bit 0: target map 16-byte vectorisable, bit 1: mask rows 16-byte vectorisable
  kPStepBegin,    // offset of this image's step table (N+1 entries: checkpoint index or -1)
  kPCountBegin,   // offset of this image's [T][C][2] matching counters
  kPFields
};

constexpr int kPxThreads = 256;
constexpr int kPxChunk = kPxThreads * 16;
constexpr int kPxWindow = 4;  // masks whose 16-byte words each lane loads before processing them

__device__ __forceinline__ const int64_t* pdesc(const int64_t* descs, int64_t b) { return descs + b * kPFields; }

__device__ __forceinline__ int64_t find_image(const int64_t* descs, int64_t B, int field, int64_t value) {
  int64_t lo = 0, hi = B - 1;
  while (lo < hi) {
    const int64_t mid = (lo + hi + 1) >> 1;
    if (descs[mid * kPFields + field] <= value) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Target areas of one lane's 16 pixels, run-combined per lane and warp-aggregated; false on a slot
// outside [0, G).
__device__ __forceinline__ bool count_target(const int (&t)[16], int64_t x, int64_t pixels, int G, u32* ga_img,
                                             int lane) {
  bool bad = false;
  u32 key = kEmpty, n = 0;
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    if (x + j >= pixels) continue;
    if (t[j] < 0 || t[j] >= G) { bad = true; continue; }
    if ((u32)t[j] != key) {
      if (n) atomicAdd(ga_img + key, n);
      key = (u32)t[j];
      n = 0;
    }
    ++n;
  }
  const u32 peers = __match_any_sync(0xffffffffu, key);
  const u32 total = __reduce_add_sync(peers, n);
  if (lane == (int)(__ffs(peers) - 1) && total) atomicAdd(ga_img + key, total);
  return bad;
}

// Visible owner (1-based mask index, 0 = none) of one lane's 16 pixels, now and at the previous
// checkpoint: one byte per pixel when every image of the batch has at most 255 masks (kBytes), else
// 16 bits per pixel. Drawing a mask is a byte (or half-word) select per register, so its cost does not
// depend on how many of the 16 pixels it covers. Pixels outside the image or on an invalid slot are
// drawn too and skipped when transitions are emitted.
template <bool kBytes>
struct Owners {
  static constexpr int kWords = kBytes ? 4 : 8;
  u32 now[kWords], prev[kWords];
  __device__ __forceinline__ void clear() {
#pragma unroll
    for (int k = 0; k < kWords; ++k) now[k] = prev[k] = 0;
  }
  // lsb: the lane's 16 mask bytes reduced to 0/1; covered pixels take owner `value`.
  __device__ __forceinline__ void draw(const u32 (&lsb)[4], u32 value) {
    if constexpr (kBytes) {
      const u32 fill = value * 0x01010101u;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const u32 m = lsb[k] * 0xffu;  // 0x00 / 0xff per byte (no carries: bytes are 0 or 1)
        now[k] = (now[k] & ~m) | (fill & m);
      }
    } else {
      const u32 fill = value * 0x00010001u;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const u32 lo = __byte_perm(lsb[k], 0u, 0x4140) * 0xffffu, hi = __byte_perm(lsb[k], 0u, 0x4342) * 0xffffu;
        now[2 * k] = (now[2 * k] & ~lo) | (fill & lo);
        now[2 * k + 1] = (now[2 * k + 1] & ~hi) | (fill & hi);
      }
    }
  }
  __device__ __forceinline__ static int at(const u32 (&v)[kWords], int j) {
    if constexpr (kBytes) return (int)((v[j >> 2] >> (8 * (j & 3))) & 0xffu);
    else return (int)((v[j >> 1] >> (16 * (j & 1))) & 0xffffu);
  }
  __device__ __forceinline__ bool changed() const {
    u32 d = 0;
#pragma unroll
    for (int k = 0; k < kWords; ++k) d |= now[k] ^ prev[k];
    return d != 0;
  }
};

// True when some lane of the warp may hold a covered pixel in these staged words (a superset test on
// the raw words, before they are re-aligned). Warp-uniform.
__device__ __forceinline__ bool warp_may_cover(uint4 a, uint4 b, bool two) {
  u32 any = a.x | a.y | a.z | a.w;
  if (two) any |= b.x | b.y | b.z | b.w;
  return __any_sync(0xffffffffu, (any & 0x01010101u) != 0);
}

// Draw mask i (its 16 bytes for this lane in w) over the lane's pixels: the raw mask x slot
// intersections raw_row[slot] and the new owners. Called by every lane of the warp.
template <bool kBytes>
__device__ __forceinline__ void draw_mask(int i, uint4 w, const int (&t)[16], const LaneSlots& ls,
                                          const LanePeers& lp, u32 valid, u32* raw_row, Owners<kBytes>& s) {
  const u32 lsb[4] = {w.x & 0x01010101u, w.y & 0x01010101u, w.z & 0x01010101u, w.w & 0x01010101u};
  const auto pack4 = [](u32 v) { return (v * 0x01020408u) >> 24; };
  const u32 m = (pack4(lsb[0]) | pack4(lsb[1]) << 4 | pack4(lsb[2]) << 8 | pack4(lsb[3]) << 12) & valid;
  const u32 c1 = __popc(m & ls.e1), c2 = __popc(m & ls.e2);
  const u32 t1 = __reduce_add_sync(lp.peers1, c1);
  const u32 t2 = __reduce_add_sync(lp.peers2, c2);
  if (lp.lead1 && t1) atomicAdd(raw_row + ls.s1, t1);
  if (lp.lead2 && t2) atomicAdd(raw_row + ls.s2, t2);
  const u32 mid = m & ls.emid;  // a third slot inside 16 pixels: rare
  if (mid) {
#pragma unroll
    for (int j = 0; j < 16; ++j)
      if ((mid >> j) & 1u) atomicAdd(raw_row + t[j], 1u);
  }
  s.draw(lsb, (u32)(i + 1));
}

// At a requested checkpoint: the owner transitions of the lane's valid pixels since the previous
// checkpoint into that checkpoint's delta histogram dq [G][N + 1] (run-combined), then the owners
// become the previous ones. Called by every lane when any lane of the warp changed.
// Bytes of four words that differ from the byte before them (byte j against byte j - 1 across the words;
// byte 0 against `before`), as 16 bits.
__device__ __forceinline__ u32 byte_changes(const u32 (&v)[4]) {
  u32 bits = 0, carry = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    u32 x = v[k] ^ ((v[k] << 8) | carry);
    carry = v[k] >> 24;
    x |= x >> 4;
    x |= x >> 2;
    x |= x >> 1;
    bits |= (((x & 0x01010101u) * 0x01020408u) >> 24) << (4 * k);
  }
  return bits;
}

// Bytes where two sets of four words differ, as 16 bits.
__device__ __forceinline__ u32 byte_differs(const u32 (&a)[4], const u32 (&b)[4]) {
  u32 bits = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    u32 x = a[k] ^ b[k];
    x |= x >> 4;
    x |= x >> 2;
    x |= x >> 1;
    bits |= (((x & 0x01010101u) * 0x01020408u) >> 24) << (4 * k);
  }
  return bits;
}

// Byte j of four words (j uniform or not: three selects, no local memory).
__device__ __forceinline__ int byte_at(const u32 (&v)[4], int j) {
  const int k = j >> 2;
  const u32 w = k == 0 ? v[0] : (k == 1 ? v[1] : (k == 2 ? v[2] : v[3]));
  return (int)((w >> (8 * (j & 3))) & 0xffu);
}

// Byte-owner transitions of a lane, run by run rather than pixel by pixel: the changed valid pixels
// (cv) split into runs wherever the slot (gchg, fixed for the chunk), the old owner or the new owner
// changes from one pixel to the next; a lane usually has one to three runs. The first run is summed
// over the warp's lanes that share it, later runs go to memory directly.
__device__ __forceinline__ void emit_transitions_bytes(const int (&t)[16], const LaneSlots& ls, u32 valid, u32 gchg,
                                                       int* dq, int N, Owners<true>& s) {
  const u32 cv = byte_differs(s.now, s.prev) & valid;
  const u32 kchg = gchg | byte_changes(s.now) | byte_changes(s.prev) | 1u;
  u32 starts = cv & (~(cv << 1) | kchg);
  int fg = -1, fo = 0, fn = 0, fcnt = 0;
  while (starts) {
    const int j = __ffs(starts) - 1;
    starts &= starts - 1;
    const int end = starts ? __ffs(starts) - 1 : 16;
    const int cnt = __popc(cv & ((end == 16 ? 0xffffu : (1u << end) - 1u) & ~((1u << j) - 1u)));
    int g;
    if ((ls.e1 >> j) & 1u) {
      g = ls.s1;
    } else if ((ls.e2 >> j) & 1u) {
      g = ls.s2;
    } else {  // a third slot inside the lane: rare
      g = t[0];
#pragma unroll
      for (int k = 1; k < 16; ++k) g = k == j ? t[k] : g;
    }
    const int o = byte_at(s.prev, j), n = byte_at(s.now, j);
    if (fcnt == 0) {
      fg = g; fo = o; fn = n; fcnt = cnt;
    } else {
      atomicAdd(dq + (int64_t)g * (N + 1) + o, -cnt);
      atomicAdd(dq + (int64_t)g * (N + 1) + n, cnt);
    }
  }
  const unsigned long long key =
      fcnt ? ((unsigned long long)(u32)fg << 32) | ((unsigned long long)fo << 16) | (unsigned long long)fn : ~0ull;
  const u32 peers = __match_any_sync(0xffffffffu, key);
  const int total = (int)__reduce_add_sync(peers, (u32)fcnt);
  if (fcnt && (threadIdx.x & 31) == (int)(__ffs(peers) - 1)) {
    atomicAdd(dq + (int64_t)fg * (N + 1) + fo, -total);
    atomicAdd(dq + (int64_t)fg * (N + 1) + fn, total);
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) s.prev[k] = s.now[k];
}

// Slot changes between neighbouring pixels of a lane (bit j: pixel j's slot differs from pixel j - 1's).
__device__ __forceinline__ u32 slot_changes(const int (&t)[16]) {
  u32 bits = 1u;
#pragma unroll
  for (int j = 1; j < 16; ++j) bits |= (u32)(t[j] != t[j - 1]) << j;
  return bits;
}

// Transitions at a checkpoint: the run form for byte owners, the pixel loop for 16-bit owners.
template <bool kBytes>
__device__ __forceinline__ void emit_at_checkpoint(const int (&t)[16], const LaneSlots& ls, u32 valid, u32 gchg,
                                                   int* dq, int N, Owners<kBytes>& s);

// Each lane's first run of equal (slot, old owner, new owner) is summed over the lanes of the warp that
// share it (one pair of atomics per distinct run instead of one per lane: inside a large region every
// lane has the same transition); later runs, at region borders, go to memory directly.
template <bool kBytes>
__device__ __forceinline__ void emit_transitions(const int (&t)[16], u32 valid, int* dq, int N, Owners<kBytes>& s) {
  int rg = -1, ro = -1, rn = -1, cnt = 0;
  int fg = -1, fo = 0, fn = 0, fcnt = 0;  // the lane's first run
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    const int o = Owners<kBytes>::at(s.prev, j), n = Owners<kBytes>::at(s.now, j);
    if (!((valid >> j) & 1u) || o == n) continue;
    const int g = t[j];
    if (g == rg && o == ro && n == rn) {
      ++cnt;
    } else {
      if (cnt) {
        if (fcnt == 0) {
          fg = rg; fo = ro; fn = rn; fcnt = cnt;
        } else {
          atomicAdd(dq + (int64_t)rg * (N + 1) + ro, -cnt);
          atomicAdd(dq + (int64_t)rg * (N + 1) + rn, cnt);
        }
      }
      rg = g; ro = o; rn = n; cnt = 1;
    }
  }
  if (cnt) {
    if (fcnt == 0) {
      fg = rg; fo = ro; fn = rn; fcnt = cnt;
    } else {
      atomicAdd(dq + (int64_t)rg * (N + 1) + ro, -cnt);
      atomicAdd(dq + (int64_t)rg * (N + 1) + rn, cnt);
    }
  }
  // Owners are below 65536 (N < 65535), so (slot, old, new) packs into 64 bits.
  const unsigned long long key =
      fcnt ? ((unsigned long long)(u32)fg << 32) | ((unsigned long long)fo << 16) | (unsigned long long)fn : ~0ull;
  const u32 peers = __match_any_sync(0xffffffffu, key);
  const int total = (int)__reduce_add_sync(peers, (u32)fcnt);
  if (fcnt && (threadIdx.x & 31) == (int)(__ffs(peers) - 1)) {
    atomicAdd(dq + (int64_t)fg * (N + 1) + fo, -total);
    atomicAdd(dq + (int64_t)fg * (N + 1) + fn, total);
  }
#pragma unroll
  for (int k = 0; k < Owners<kBytes>::kWords; ++k) s.prev[k] = s.now[k];
}

template <>
__device__ __forceinline__ void emit_at_checkpoint<true>(const int (&t)[16], const LaneSlots& ls, u32 valid, u32 gchg,
                                                         int* dq, int N, Owners<true>& s) {
  emit_transitions_bytes(t, ls, valid, gchg, dq, N, s);
}

template <>
__device__ __forceinline__ void emit_at_checkpoint<false>(const int (&t)[16], const LaneSlots&, u32 valid, u32,
                                                          int* dq, int N, Owners<false>& s) {
  emit_transitions<false>(t, valid, dq, N, s);
}

// One CTA per 4096-pixel chunk, masks read with plain loads (rows at any alignment).
template <bool kBytes>
__global__ void __launch_bounds__(kPxThreads, 2)
prefix_pass_kernel(const int64_t* __restrict__ descs, int64_t B, const int* __restrict__ step_q, u32* __restrict__ ga,
                   u32* __restrict__ raw, int* __restrict__ delta, int* __restrict__ error) {
  const int64_t b = find_image(descs, B, kPChunkBegin, blockIdx.x);
  const int64_t* d = pdesc(descs, b);
  const int64_t pixels = d[kPPixels];
  const int64_t x = (blockIdx.x - d[kPChunkBegin]) * (int64_t)kPxChunk + (int64_t)threadIdx.x * 16;
  const int N = (int)d[kPN], G = (int)d[kPG];
  const int* target = reinterpret_cast<const int*>(d[kPTarget]);
  const uint8_t* masks = reinterpret_cast<const uint8_t*>(d[kPMasks]);
  const int64_t stride = d[kPStride];
  const bool vec_map = d[kPFlags] & 1, vec_masks = d[kPFlags] & 2;
  const int* steps = step_q + d[kPStepBegin];
  int* delta_img = delta + d[kPPairBegin];
  u32* raw_img = raw + d[kPRawBegin];
  const int64_t plane = (int64_t)G * (N + 1);
  const int lane = threadIdx.x & 31;

  int t[16];
  load16_maps(target, x, pixels, vec_map, t);
  const bool bad = count_target(t, x, pixels, G, ga + d[kPSlotBegin], lane);
  const LaneSlots ls = lane_slots(t, x, pixels, G);
  const LanePeers lp = lane_peers(ls, lane);
  const u32 valid = ls.e1 | ls.e2 | ls.emid;
  const u32 gchg = slot_changes(t);
  Owners<kBytes> s;
  s.clear();
  const int64_t xm = x < pixels ? x : pixels;
  uint4 window[kPxWindow];
  for (int i = 0; i < N; ++i) {
    if (i % kPxWindow == 0) {  // the next kPxWindow masks' words are all in flight before any is used
#pragma unroll
      for (int k = 0; k < kPxWindow; ++k)
        window[k] = i + k < N ? load16_mask(masks + (int64_t)(i + k) * stride, xm, pixels, vec_masks)
                              : make_uint4(0, 0, 0, 0);
    }
    uint4 w = window[0];
#pragma unroll
    for (int k = 1; k < kPxWindow; ++k)
      if (i % kPxWindow == k) w = window[k];
    if (warp_may_cover(w, w, false)) draw_mask<kBytes>(i, w, t, ls, lp, valid, raw_img + (int64_t)i * G, s);
    const int q = steps[i + 1];  // uniform across the CTA
    if (q >= 0 && __any_sync(0xffffffffu, s.changed()))
      emit_at_checkpoint<kBytes>(t, ls, valid, gchg, delta_img + q * plane, N, s);
  }
  if (bad) atomicOr(error, 1);
}

// Persistent form: a producer warp streams every mask's segment of the current 4096-pixel chunk into a
// shared-memory ring with cp.async.bulk (one copy per mask row and chunk: the 16-byte-aligned words
// covering the segment, since rows may start at any byte; completion on the stage's mbarrier) while
// 8 consumer warps draw the masks in order from shared memory, re-aligning each lane's 16 bytes from
// two staged words when the row is not aligned (the offset is per row, uniform across a warp). Each
// wait is bounded; a timeout sets bit 30 of *error, the producer waits (bounded) for its copies in
// flight, and every role returns.
constexpr int kPbConsumers = kPxThreads;
constexpr int kPbThreads = kPbConsumers + 32;
constexpr int kPbStage = 4;  // mask rows per ring stage
constexpr int kPbRing = 6;   // stages in flight per CTA
constexpr long long kPbWaitLimit = 4000000000ll;  // about two seconds of SM clock
constexpr int kPbTimeoutBit = 1 << 30;

constexpr int kPbSlot = kPxChunk + 16;  // staged bytes per mask row and chunk (aligned words covering it)

constexpr int kPbChunkRing = 4;  // published chunks in flight per CTA

struct PrefixShared {
  unsigned char ring[kPbRing][kPbStage][kPbSlot];
  int64_t chunk[kPbChunkRing];  // chunk published to the consumers; -1 ends the CTA's work
  uint64_t full[kPbRing];
  uint64_t empty[kPbRing];
  uint64_t chunk_full[kPbChunkRing];
  uint64_t chunk_empty[kPbChunkRing];
  int abort;
};

template <bool kBytes>
__global__ void __launch_bounds__(kPbThreads, 2)
prefix_pass_bulk_kernel(const int64_t* __restrict__ descs, int64_t B, int64_t total_chunks,
                        unsigned long long* __restrict__ schedule, const int* __restrict__ step_q,
                        u32* __restrict__ ga, u32* __restrict__ raw, int* __restrict__ delta,
                        int* __restrict__ error) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  PrefixShared& sm = *reinterpret_cast<PrefixShared*>(smem_raw);
  // Without a counter: contiguous chunk ranges whose sizes differ by at most one chunk.
  const int64_t c_begin = (int64_t)blockIdx.x * total_chunks / gridDim.x;
  const int64_t c_end = (int64_t)(blockIdx.x + 1) * total_chunks / gridDim.x;
  if (!schedule && c_begin >= c_end) return;
  if (threadIdx.x == 0) {
    for (int i = 0; i < kPbRing; ++i) {
      mbar_init(&sm.full[i], 1);
      mbar_init(&sm.empty[i], kPbConsumers / 32);
    }
    for (int i = 0; i < kPbChunkRing; ++i) {
      mbar_init(&sm.chunk_full[i], 1);
      mbar_init(&sm.chunk_empty[i], kPbConsumers / 32);
    }
    sm.abort = 0;
    mbar_fence_init();
  }
  __syncthreads();
  volatile int* abort = &sm.abort;

  if (threadIdx.x >= kPbConsumers) {
    // ---- producer ----------------------------------------------------------
    if (threadIdx.x != kPbConsumers) return;
    int64_t seq = 0, published = 0, next = c_begin;
    bool ok = true;
    // Publish a chunk to the consumers (-1: no more work); false when the wait for a free entry fails.
    auto publish = [&](int64_t chunk) {
      const int e = (int)(published % kPbChunkRing);
      const int64_t use = published / kPbChunkRing;
      if ((use > 0 && !mbar_wait(&sm.chunk_empty[e], (uint32_t)((use - 1) & 1), kPbWaitLimit)) || *abort)
        return false;
      sm.chunk[e] = chunk;
      mbar_arrive(&sm.chunk_full[e]);  // release: the entry is visible to consumers that see the phase
      ++published;
      return true;
    };
    while (ok) {
      const int64_t chunk = schedule ? (int64_t)atomicAdd(schedule, 1ull) : (next < c_end ? next++ : total_chunks);
      if (chunk >= total_chunks) break;
      if (!publish(chunk)) {
        ok = false;
        break;
      }
      const int64_t* d = pdesc(descs, find_image(descs, B, kPChunkBegin, chunk));
      const int64_t pixels = d[kPPixels];
      const int64_t x0 = (chunk - d[kPChunkBegin]) * (int64_t)kPxChunk;
      const int64_t len = min((int64_t)kPxChunk, pixels - x0);
      const int N = (int)d[kPN];
      const uint8_t* masks = reinterpret_cast<const uint8_t*>(d[kPMasks]);
      const int64_t stride = d[kPStride];
      const int* target = reinterpret_cast<const int*>(d[kPTarget]);
      const uint32_t map_bytes = (uint32_t)((len * 4) & ~15ll);
      if ((d[kPFlags] & 1) && map_bytes) bulk_prefetch_l2(target + x0, map_bytes);
      for (int r0 = 0; r0 < N; r0 += kPbStage) {
        const int slot = (int)(seq % kPbRing);
        const int64_t use = seq / kPbRing;
        if ((use > 0 && !mbar_wait(&sm.empty[slot], (uint32_t)((use - 1) & 1), kPbWaitLimit)) || *abort) {
          ok = false;
          break;
        }
        const int n = min(kPbStage, N - r0);
        uint32_t sizes[kPbStage], total = 0;
#pragma unroll
        for (int k = 0; k < kPbStage; ++k) {
          // Aligned words from the one holding pixel x0 to the one holding the segment's last byte.
          const int o = (int)(reinterpret_cast<uintptr_t>(masks + (int64_t)(r0 + k) * stride) & 15);
          sizes[k] = k < n ? (uint32_t)round_up(len + o, 16) : 0u;
          total += sizes[k];
        }
        mbar_arrive_expect_tx(&sm.full[slot], total);
        for (int k = 0; k < n; ++k) {
          const uint8_t* row = masks + (int64_t)(r0 + k) * stride;
          const int o = (int)(reinterpret_cast<uintptr_t>(row) & 15);
          bulk_copy_g2s(sm.ring[slot][k], row + x0 - o, sizes[k], &sm.full[slot]);
        }
        ++seq;
      }
    }
    if (ok) ok = publish(-1);
    if (!ok) {
      *abort = 1;
      atomicOr(error, kPbTimeoutBit);
    }
    for (int64_t q = seq > kPbRing ? seq - kPbRing : 0; q < seq; ++q)  // copies still in flight land first
      mbar_wait(&sm.full[q % kPbRing], (uint32_t)((q / kPbRing) & 1), kPbWaitLimit);
    return;
  }

  // ---- consumers -----------------------------------------------------------
  const int lane = threadIdx.x & 31;
  int64_t seq = 0, taken = 0;
  bool ok = true, bad = false;
  while (ok) {
    const int e = (int)(taken % kPbChunkRing);
    const bool ready = mbar_wait(&sm.chunk_full[e], (uint32_t)((taken / kPbChunkRing) & 1), kPbWaitLimit);
    if (!__all_sync(0xffffffffu, ready && !*abort)) {
      ok = false;
      break;
    }
    const int64_t chunk = sm.chunk[e];
    __syncwarp();
    if (lane == 0) mbar_arrive(&sm.chunk_empty[e]);
    ++taken;
    if (chunk < 0) break;
    const int64_t* d = pdesc(descs, find_image(descs, B, kPChunkBegin, chunk));
    const int64_t pixels = d[kPPixels];
    const int64_t x0 = (chunk - d[kPChunkBegin]) * (int64_t)kPxChunk;
    const int64_t x = x0 + (int64_t)threadIdx.x * 16;
    const int N = (int)d[kPN], G = (int)d[kPG];
    const int* steps = step_q + d[kPStepBegin];
    const int64_t plane = (int64_t)G * (N + 1);
    const uint8_t* masks = reinterpret_cast<const uint8_t*>(d[kPMasks]);
    const int64_t stride = d[kPStride];
    int* delta_img = delta + d[kPPairBegin];
    u32* raw_img = raw + d[kPRawBegin];
    int t[16];
    load16_maps(reinterpret_cast<const int*>(d[kPTarget]), x, pixels, d[kPFlags] & 1, t);
    bad |= count_target(t, x, pixels, G, ga + d[kPSlotBegin], lane);
    const LaneSlots ls = lane_slots(t, x, pixels, G);
    const LanePeers lp = lane_peers(ls, lane);
    const u32 valid = ls.e1 | ls.e2 | ls.emid;  // pixels past the image end are not valid: stale bytes ignored
    const u32 gchg = slot_changes(t);
    Owners<kBytes> s;
    s.clear();
    for (int r0 = 0; r0 < N; r0 += kPbStage) {
      const int slot = (int)(seq % kPbRing);
      const bool got = mbar_wait(&sm.full[slot], (uint32_t)((seq / kPbRing) & 1), kPbWaitLimit);
      if (!__all_sync(0xffffffffu, got && !*abort)) {  // warp-uniform decision
        ok = false;
        break;
      }
      const int n = min(kPbStage, N - r0);
      // One mask at a time, not unrolled: the drawing code is large and unrolled copies of it missed
      // the instruction cache. The next mask's staged words and checkpoint index are loaded before the
      // current mask is drawn, so their latency overlaps the drawing. Row offsets advance by the row
      // stride mod 16 (the same for the whole warp).
      int o = (int)(reinterpret_cast<uintptr_t>(masks + (int64_t)r0 * stride) & 15);
      const int o_step = (int)(stride & 15);
      const uint4* words = reinterpret_cast<const uint4*>(&sm.ring[slot][0][threadIdx.x * 16]);
      uint4 a = words[0];
      uint4 b = o ? words[1] : a;
      int q = steps[r0 + 1];
#pragma unroll 1
      for (int k = 0; k < n; ++k) {
        const int i = r0 + k;
        const int o_next = (o + o_step) & 15;
        uint4 a_next = a, b_next = b;
        int q_next = -1;
        if (k + 1 < n) {
          const uint4* next = reinterpret_cast<const uint4*>(&sm.ring[slot][k + 1][threadIdx.x * 16]);
          a_next = next[0];
          b_next = o_next ? next[1] : a_next;
          q_next = steps[i + 2];
        }
        if (warp_may_cover(a, b, o != 0))
          draw_mask<kBytes>(i, o ? realign16(a, b, o) : a, t, ls, lp, valid, raw_img + (int64_t)i * G, s);
        if (q >= 0 && __any_sync(0xffffffffu, s.changed()))  // q: uniform across the CTA
          emit_at_checkpoint<kBytes>(t, ls, valid, gchg, delta_img + q * plane, N, s);
        a = a_next;
        b = b_next;
        q = q_next;
        o = o_next;
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&sm.empty[slot]);
      ++seq;
    }
  }
  if (!ok) {
    *abort = 1;
    if (lane == 0) atomicOr(error, kPbTimeoutBit);
  }
  if (bad) atomicOr(error, 1);
}

// Running sums over checkpoints: delta[q] -> pairs[q] in place.
__global__ void prefix_scan_kernel(const int64_t* __restrict__ descs, const u32* __restrict__ ga,
                                   int* __restrict__ delta) {
  const int64_t* d = pdesc(descs, blockIdx.y);
  const int N = (int)d[kPN], G = (int)d[kPG], Q = (int)d[kPQ];
  const int64_t plane = (int64_t)G * (N + 1);
  const int64_t cell = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= plane) return;
  int* base = delta + d[kPPairBegin] + cell;
  const int g = (int)(cell / (N + 1)), j = (int)(cell % (N + 1));
  int v = j == 0 ? (int)ga[d[kPSlotBegin] + g] : 0;
  for (int q = 0; q < Q; ++q) {
    v += base[(int64_t)q * plane];
    base[(int64_t)q * plane] = v;
  }
}

// Canvas PQ of one (image, checkpoint) row. With stage_pairs > 0 the row's G x (N+1) histogram is
// copied to shared memory first (it fits when G x (N+1) <= stage_pairs) and scored one warp per mask.
constexpr int kPrefixScoreThreads = 512;
__global__ void __launch_bounds__(kPrefixScoreThreads)
prefix_score_kernel(const int64_t* __restrict__ descs, int64_t B, const int* __restrict__ pairs,
                    const int* __restrict__ classes, const int* __restrict__ gc, const uint8_t* __restrict__ crowd,
                    int C, int64_t* __restrict__ tp, int64_t* __restrict__ fp, int64_t* __restrict__ fn,
                    double* __restrict__ sums, int64_t* __restrict__ confusion, int stage_pairs, int hist_off) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int64_t row = blockIdx.x;
  const int64_t b = find_image(descs, B, kPQBegin, row);
  const int64_t* d = pdesc(descs, b);
  const int N = (int)d[kPN], G = (int)d[kPG], P = N + 1;
  const int q = (int)(row - d[kPQBegin]);
  const u32* pq = reinterpret_cast<const u32*>(pairs + d[kPPairBegin] + (int64_t)q * G * P);
  gc += d[kPSlotBegin];
  crowd += d[kPSlotBegin];
  classes += d[kPDetBegin];
  u64* areas = reinterpret_cast<u64*>(smem_raw);
  int* matched = reinterpret_cast<int*>(areas + G + P);
  int* labels = matched + G;
  unsigned char* staging = reinterpret_cast<unsigned char*>(labels + P);
  staging += (16 - reinterpret_cast<uintptr_t>(staging) % 16) % 16;
  const bool staged = (int64_t)G * P <= stage_pairs;
  if (staged) {
    u32* hs = reinterpret_cast<u32*>(smem_raw + hist_off);
    stage_counts(hs, pq, G * P);
    __syncthreads();
    pq = hs;
  }
  score_areas<u32, false>(pq, gc, labels, crowd, areas, G, P, C, false);
  __syncthreads();
  // Active labels: a mask's class while it has visible pixels (prefix.py:82).
  for (int p = threadIdx.x; p < P; p += blockDim.x) labels[p] = (p > 0 && areas[G + p] > 0) ? classes[p - 1] : -1;
  __syncthreads();
  ScoreOut out{reinterpret_cast<u64*>(tp + row * C), reinterpret_cast<u64*>(fp + row * C),
               reinterpret_cast<u64*>(fn + row * C), sums + row * C,
               reinterpret_cast<u64*>(confusion + row * C * (int64_t)(C + 1))};
  if (staged) score_accumulate_warps<false>(pq, gc, labels, crowd, areas, matched, G, P, C, out, staging);
  else score_accumulate<u32, false>(pq, gc, labels, crowd, areas, matched, G, P, C, out, staging);
}

// Greedy generation-order matching (prefix.py:106-118) and the validation of one image's metadata: one
// CTA per image. Phase 1 (all threads): each mask's area on valid slots and, for thing masks, its IoU
// with every target slot of its class, staged in shared memory (kStaged) or left to phase 2. Phase 2:
// one warp per IoU threshold walks the masks in generation order; its lanes split the candidate slots
// and a warp arg-max (largest IoU, first slot on ties) picks the match, so the chain has no block
// barrier; at every checkpoint the warp writes its threshold's snapshot. Error bits: 2 empty prediction
// mask, 4 bad target class / slot 0 not void, 8 target areas vs metadata, 16 bad prediction class.
constexpr int kPrefixMatchThreads = 512;  // 16 warps: every IoU threshold's chain has its own warp
constexpr int kSerialCandidates = 8;      // candidate slots a single lane scans in the chain
template <bool kStaged>
__global__ void __launch_bounds__(kPrefixMatchThreads)
prefix_match_kernel(const int64_t* __restrict__ descs, const u32* __restrict__ ga, const u32* __restrict__ raw,
                    const int* __restrict__ classes, const int* __restrict__ gc, const uint8_t* __restrict__ crowd,
                    const uint8_t* __restrict__ isthing, const double* __restrict__ thresholds, int T, int C,
                    const int* __restrict__ step_q, int64_t* __restrict__ itp, int64_t* __restrict__ ifp,
                    int64_t* __restrict__ ifn, double* __restrict__ precision, double* __restrict__ recall,
                    int validate, int* __restrict__ error) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int64_t* d = pdesc(descs, blockIdx.x);
  const int N = (int)d[kPN], G = (int)d[kPG];
  const int64_t qb = d[kPQBegin];
  const int* steps = step_q + d[kPStepBegin];
  ga += d[kPSlotBegin];
  gc += d[kPSlotBegin];
  crowd += d[kPSlotBegin];
  classes += d[kPDetBegin];
  raw += d[kPRawBegin];
  const int words = (G + 31) / 32;
  u64* areas = reinterpret_cast<u64*>(smem_raw);                   // N mask areas on valid slots
  long long* iou_all = reinterpret_cast<long long*>(areas + N);    // candidate IoU bit patterns (kStaged)
  int* ints = reinterpret_cast<int*>(iou_all + (kStaged ? (int64_t)N * G : 0));
  int* positives = ints;                                           // C
  int* by_class = positives + C;                                   // G slots ordered by class
  int* class_start = by_class + G;                                 // C + 1
  int* cand_off = class_start + C + 1;                             // N + 1
  int* tp_s = cand_off + N + 1;                                    // T x C
  int* fp_s = tp_s + T * C;                                        // T x C
  int* thing_class = fp_s + T * C;                                 // N: the mask's class if a thing, else -1
  int* step_s = thing_class + N;                                   // N + 1: checkpoint index of prefix k or -1
  u32* used = reinterpret_cast<u32*>(step_s + N + 1);              // T x words
  int* gc_s = reinterpret_cast<int*>(used + T * words);            // G: slot classes
  uint8_t* crowd_s = reinterpret_cast<uint8_t*>(gc_s + G);         // G
  __shared__ int s_err;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, warps = (int)(blockDim.x >> 5);
  if (tid == 0) s_err = 0;
  for (int c = tid; c < C; c += blockDim.x) positives[c] = 0;
  for (int k = tid; k <= C; k += blockDim.x) class_start[k] = 0;
  for (int k = tid; k < T * C; k += blockDim.x) tp_s[k] = fp_s[k] = 0;
  for (int k = tid; k < T * words; k += blockDim.x) used[k] = 0;
  // Everything the sequential chain reads per mask or slot is staged here, off its critical path.
  for (int k = tid; k <= N; k += blockDim.x) step_s[k] = steps[k];
  for (int g = tid; g < G; g += blockDim.x) {
    crowd_s[g] = crowd[g];
    gc_s[g] = gc[g];
  }
  for (int i = tid; i < N; i += blockDim.x) {
    const int c = classes[i];
    thing_class[i] = (c >= 0 && c < C && isthing[c]) ? c : -1;
  }
  __syncthreads();
  int err = 0;
  for (int g = tid; g < G; g += blockDim.x) {
    const int c = gc[g];
    if (c >= 0 && c < C) {
      atomicAdd(class_start + c + 1, 1);
      if (isthing[c] && !crowd[g]) atomicAdd(positives + c, 1);
    }
    if (validate) {
      if (c < -1 || c >= C || (g == 0 && (c != -1 || crowd[g]))) err |= 4;
      if (g > 0 && ((ga[g] > 0) != (c >= 0))) err |= 8;
    }
  }
  // Mask areas (one warp per mask).
  for (int i = warp; i < N; i += warps) {
    u64 area = 0;
    for (int g = lane; g < G; g += 32) area += raw[(int64_t)i * G + g];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) area += __shfl_xor_sync(0xffffffffu, area, off);
    if (lane == 0) {
      areas[i] = area;
      const int c = classes[i];
      if (validate && (c < 0 || c >= C)) err |= 16;
      if (validate && area == 0) err |= 2;
    }
  }
  if (err) atomicOr(&s_err, err);
  __syncthreads();
  if (warp == 0) {
    // Exclusive scan of the class sizes (C + 1 entries; entry c + 1 holds class c's size), then of the
    // thing masks' candidate counts.
    int carry = 0;
    for (int base = 0; base <= C; base += 32) {
      const int k = base + lane;
      int v = k <= C ? class_start[k] : 0;
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, v, off);
        if (lane >= off) v += u;
      }
      if (k <= C) class_start[k] = v + carry;
      carry += __shfl_sync(0xffffffffu, v, 31);
    }
    __syncwarp();
    carry = 0;
    for (int base = 0; base < N; base += 32) {
      const int i = base + lane;
      const int c = i < N ? classes[i] : -1;
      const int n = (c >= 0 && c < C && isthing[c]) ? class_start[c + 1] - class_start[c] : 0;
      int v = n;
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, v, off);
        if (lane >= off) v += u;
      }
      if (i < N) cand_off[i] = carry + v - n;
      carry += __shfl_sync(0xffffffffu, v, 31);
    }
  }
  __syncthreads();
  // Slots grouped by class, in slot order within a class (stable).
  for (int g = tid; g < G; g += blockDim.x) {
    const int c = gc[g];
    if (c < 0 || c >= C) continue;
    int rank = 0;
    for (int h = 0; h < g; ++h) rank += gc_s[h] == c;
    by_class[class_start[c] + rank] = g;
  }
  __syncthreads();
  // Same-class IoUs of every thing mask: inter / union, crowd slots against the mask area.
  auto iou_of = [&](int i, int g) -> long long {
    const u64 inter = raw[(int64_t)i * G + g];
    const u64 uni = crowd_s[g] ? areas[i] : areas[i] + ga[g] - inter;
    return __double_as_longlong((double)inter / (double)(uni > 1 ? uni : 1));
  };
  if constexpr (kStaged) {
    for (int i = warp; i < N; i += warps) {
      const int c = classes[i];
      if (c < 0 || c >= C || !isthing[c]) continue;
      const int s0 = class_start[c], s1 = class_start[c + 1];
      for (int k = s0 + lane; k < s1; k += 32) iou_all[cand_off[i] + k - s0] = iou_of(i, by_class[k]);
    }
    __syncthreads();
  }
  // Phase 2: one warp per threshold.
  for (int t = warp; t < T; t += warps) {
    const long long thr = __double_as_longlong(thresholds[t]);
    int* tpc = tp_s + t * C;
    int* fpc = fp_s + t * C;
    u32* taken = used + t * words;
    // Counts only: precision and recall of every row are computed afterwards by prefix_ratio_kernel over
    // the whole grid, so no FP64 division sits in this sequential chain.
    auto snapshot = [&](int q) {
      __syncwarp();
      const int64_t row = qb + q;
      for (int c = lane; c < C; c += 32) {
        const int64_t a = tpc[c], f = fpc[c], n = positives[c];
        const int64_t o = (row * T + t) * C + c;
        itp[o] = a;
        ifp[o] = f;
        ifn[o] = n - a;
      }
    };
    if (step_s[0] >= 0) snapshot(step_s[0]);
    for (int i = 0; i < N; ++i) {
      const int c = thing_class[i];
      if (c >= 0 && class_start[c + 1] - class_start[c] <= kSerialCandidates) {
        // Few candidate slots (the usual case): lane 0 scans them in slot order, keeping the first of the
        // largest IoUs, the same pick as the warp arg-max below without its shuffles.
        if (lane == 0) {
          const int s0 = class_start[c], s1 = class_start[c + 1];
          long long best_iou = -1;
          int best_k = INT_MAX;
          bool ignored = false;
          for (int k = s0; k < s1; ++k) {
            const int g = by_class[k];
            const long long iou = kStaged ? iou_all[cand_off[i] + k - s0] : iou_of(i, g);
            if (iou < thr) continue;
            if (crowd_s[g]) {
              ignored = true;
            } else if (!((taken[g >> 5] >> (g & 31)) & 1u) && iou > best_iou) {
              best_iou = iou;
              best_k = k;
            }
          }
          if (best_k != INT_MAX) {
            const int g = by_class[best_k];
            taken[g >> 5] |= 1u << (g & 31);
            ++tpc[c];
          } else if (!ignored) {
            ++fpc[c];
          }
        }
        __syncwarp();
      } else if (c >= 0) {
        const int s0 = class_start[c], s1 = class_start[c + 1];
        long long best_iou = -1;
        int best_k = INT_MAX;
        bool ignored = false;
        for (int k = s0 + lane; k < s1; k += 32) {
          const int g = by_class[k];
          const long long iou = kStaged ? iou_all[cand_off[i] + k - s0] : iou_of(i, g);
          if (iou < thr) continue;
          if (crowd_s[g]) {
            ignored = true;
          } else if (!((taken[g >> 5] >> (g & 31)) & 1u) && iou > best_iou) {
            best_iou = iou;  // each lane scans increasing k: strictly greater keeps the first slot
            best_k = k;
          }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
          const long long other_iou = __shfl_xor_sync(0xffffffffu, best_iou, off);
          const int other_k = __shfl_xor_sync(0xffffffffu, best_k, off);
          if (other_iou > best_iou || (other_iou == best_iou && other_k < best_k)) {
            best_iou = other_iou;
            best_k = other_k;
          }
        }
        ignored = __any_sync(0xffffffffu, ignored);
        if (lane == 0) {
          if (best_k != INT_MAX) {
            const int g = by_class[best_k];
            taken[g >> 5] |= 1u << (g & 31);
            ++tpc[c];
          } else if (!ignored) {
            ++fpc[c];
          }
        }
        __syncwarp();
      }
      const int q = step_s[i + 1];
      if (q >= 0) snapshot(q);
    }
  }
  __syncthreads();
  if (tid == 0 && s_err) atomicOr(error, s_err);
}

// Precision tp / max(tp + fp, 1) and recall tp / max(positives, 1) of every (row, threshold, class) from
// the matching counts (positives = tp + fn), grid-stride over all rows of the batch (prefix.py:106-118).
__global__ void prefix_ratio_kernel(const int64_t* __restrict__ itp, const int64_t* __restrict__ ifp,
                                    const int64_t* __restrict__ ifn, int64_t entries, double* __restrict__ precision,
                                    double* __restrict__ recall) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < entries; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = itp[e], f = ifp[e], n = a + ifn[e];
    precision[e] = (double)a / (double)(a + f > 1 ? a + f : 1);
    recall[e] = (double)a / (double)(n > 1 ? n : 1);
  }
}

}  // namespace
}  // namespace pe

using namespace pe;

PE_API int pe_prefix_desc_fields(void) { return kPFields; }

// Batched segmentation_prefixes (prefix.py:12-122; replaces the `prefix` op,
// prefix_kernel.cu:142-199, for any number of images). Inputs: descriptor
// table (pe_prefix_desc_fields() int64 per image), step table (per image N+1
// ints: checkpoint index of prefix k or -1), classes (sum N int32), gc and
// crowd (sum G), isthing [C], thresholds [T] f64. Workspace (zeroed here):
// ga (sum G u32), raw (sum N*G u32), pairs (sum Q*G*(N+1) int32), counters
// (B*T*C*2 int32). Outputs per checkpoint row (R = sum Q), zeroed here where
// accumulated: tp/fp/fn int64 [R,C], sums f64 [R,C], confusion int64
// [R,C,C+1], itp/ifp/ifn int64 [R,T,C], precision/recall f64 [R,T,C]; then
// per_class [R,4,C], summaries [R,3,3], counts [R,3], miou [R] (pe_compute).
// Validation bits in *error: 1 unknown target slot, 2 empty prediction mask,
// 4 bad target class, 8 target areas vs metadata, 16 bad prediction class.
PE_API int pe_prefix(const int64_t* descs, int64_t B, int64_t total_chunks, int64_t total_rows, int64_t max_g,
                     int64_t max_p, int64_t max_cells, const int32_t* step_q, const int32_t* classes,
                     const int32_t* gc, const uint8_t* crowd, const uint8_t* isthing, const double* thresholds,
                     int64_t T, int64_t C, uint32_t* ga, int64_t ga_len, uint32_t* raw, int64_t raw_len,
                     int32_t* pairs, int64_t pairs_len, int32_t* counters, int64_t counters_len, int64_t* tp,
                     int64_t* fp, int64_t* fn, double* sums, int64_t* confusion, int64_t* itp, int64_t* ifp,
                     int64_t* ifn, double* precision, double* recall, double* per_class, double* summaries,
                     int64_t* counts, double* miou, int validate, int bulk, uint64_t* schedule, int32_t* error,
                     cudaStream_t stream) {
  PE_REQUIRE(B >= 0 && total_rows >= 0 && C > 0 && C < INT_MAX && T > 0 && T <= 1024 && max_g >= 0 &&
                 max_p >= 1 && max_p < 65536,
             "invalid prefix batch (T must be 1..1024, masks per image < 65535)");
  PE_CUDA(cudaMemsetAsync(error, 0, sizeof(int32_t), stream));
  if (B == 0) return kOk;
  if (ga_len) PE_CUDA(cudaMemsetAsync(ga, 0, 4 * ga_len, stream));
  if (raw_len) PE_CUDA(cudaMemsetAsync(raw, 0, 4 * raw_len, stream));
  if (pairs_len) PE_CUDA(cudaMemsetAsync(pairs, 0, 4 * pairs_len, stream));
  if (counters_len) PE_CUDA(cudaMemsetAsync(counters, 0, 4 * counters_len, stream));
  if (total_rows) {
    PE_CUDA(cudaMemsetAsync(tp, 0, 8 * total_rows * C, stream));
    PE_CUDA(cudaMemsetAsync(fp, 0, 8 * total_rows * C, stream));
    PE_CUDA(cudaMemsetAsync(fn, 0, 8 * total_rows * C, stream));
    PE_CUDA(cudaMemsetAsync(sums, 0, 8 * total_rows * C, stream));
    PE_CUDA(cudaMemsetAsync(confusion, 0, 8 * total_rows * C * (C + 1), stream));
  }
  if (total_chunks) {
    if (bulk) {
      const int64_t grid = std::min(total_chunks, (int64_t)sm_count() * 2);  // two CTAs per SM
      if (schedule) PE_CUDA(cudaMemsetAsync(schedule, 0, sizeof(uint64_t), stream));
      const size_t smem = sizeof(PrefixShared);
      // Owners fit in a byte per pixel when no image has more than 255 masks.
      auto kernel = max_p <= 256 ? prefix_pass_bulk_kernel<true> : prefix_pass_bulk_kernel<false>;
      PE_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      kernel<<<(unsigned)grid, kPbThreads, smem, stream>>>(descs, B, total_chunks,
                                                          reinterpret_cast<unsigned long long*>(schedule), step_q, ga,
                                                          raw, pairs, error);
    } else {
      auto kernel = max_p <= 256 ? prefix_pass_kernel<true> : prefix_pass_kernel<false>;
      kernel<<<(unsigned)total_chunks, kPxThreads, 0, stream>>>(descs, B, step_q, ga, raw, pairs, error);
    }
    PE_LAUNCHED("prefix_pass");
    count_launch();
  }
  if (max_cells > 0) {
    prefix_scan_kernel<<<dim3((unsigned)ceil_div(max_cells, 256), (unsigned)B), 256, 0, stream>>>(descs, ga, pairs);
    PE_LAUNCHED("prefix_scan");
    count_launch();
  }
  if (total_rows) {
    const size_t base =
        (sizeof(u64) * (max_g + max_p) + sizeof(int) * (max_g + max_p) + score_staging_bytes(max_p) + 32 + 15) &
        ~size_t{15};
    PE_REQUIRE(base <= 200 * 1024, "prefix histogram too large for scoring (G=%lld, N+1=%lld)", (long long)max_g,
               (long long)max_p);
    // Stage each row's histogram when the largest fits 100 KB (two CTAs per SM); else read in place.
    const int64_t cells = std::max<int64_t>(max_g, 1) * std::max<int64_t>(max_p, 1);
    const int stage = cells * 4 <= 100 * 1024 ? (int)cells : 0;
    const size_t smem = base + 4 * (size_t)stage;
    if (smem > 48 * 1024)
      PE_CUDA(cudaFuncSetAttribute(prefix_score_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    prefix_score_kernel<<<(unsigned)total_rows, kPrefixScoreThreads, smem, stream>>>(
        descs, B, pairs, classes, gc, crowd, (int)C, tp, fp, fn, sums, confusion, stage, (int)base);
    PE_LAUNCHED("prefix_score");
    count_launch();
  }
  {
    const int64_t words = ceil_div(std::max<int64_t>(max_g, 1), 32);
    const int64_t n = max_p - 1;  // masks per image at most
    const size_t base = sizeof(u64) * n + sizeof(int) * (C + max_g + C + 1 + n + 1 + 2 * T * C + n + n + 1) +
                        sizeof(u32) * T * words + sizeof(int) * max_g + max_g + 16;
    const size_t staged = sizeof(long long) * n * std::max<int64_t>(max_g, 1);
    // Same-class IoUs staged in shared memory when every mask x slot pair fits, else computed in the chain.
    const bool stage = base + staged <= 160 * 1024;
    const size_t smem = base + (stage ? staged : 0);
    PE_REQUIRE(smem <= 200 * 1024, "prefix matching state too large (G=%lld, T=%lld, C=%lld)", (long long)max_g,
               (long long)T, (long long)C);
    auto kernel = stage ? prefix_match_kernel<true> : prefix_match_kernel<false>;
    if (smem > 48 * 1024) PE_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kernel<<<(unsigned)B, kPrefixMatchThreads, smem, stream>>>(descs, ga, raw, classes, gc, crowd, isthing, thresholds,
                                                               (int)T, (int)C,
                                               step_q, itp, ifp, ifn, precision, recall, validate, error);
    PE_LAUNCHED("prefix_match");
    count_launch();
  }
  if (total_rows) {
    const int64_t entries = total_rows * T * C;
    const int64_t blocks = std::min<int64_t>(ceil_div(entries, 256), (int64_t)sm_count() * 4);
    prefix_ratio_kernel<<<(unsigned)blocks, 256, 0, stream>>>(itp, ifp, ifn, entries, precision, recall);
    PE_LAUNCHED("prefix_ratio");
    count_launch();
  }
  if (total_rows) {
    const int status = pe_compute(tp, fp, fn, sums, confusion, isthing, total_rows, C, per_class, summaries, counts,
                                  miou, nullptr, nullptr, nullptr, nullptr, nullptr, stream);
    if (status != kOk) return status;
  }
  if (validate) {
    int code = 0;
    PE_CUDA(cudaMemcpyAsync(&code, error, sizeof(int), cudaMemcpyDeviceToHost, stream));
    PE_CUDA(cudaStreamSynchronize(stream));
    return code;
  }
  return kOk;
}
