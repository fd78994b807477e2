// Panoptic quality, semantic confusion and per-image reward statistics.
//
// One update is three stream-ordered kernels with no host round trip:
//   1. pair_histogram: one pass over the gt/pred segment maps. Each CTA owns a
//      contiguous run of 4096-pixel tiles, keeps a privatised G x P uint32
//      histogram in shared memory (global atomics when it does not fit), reads
//      the int32 maps with 16-byte vector loads, combines equal keys of a
//      thread's 8 pixels in registers and aggregates the last run across the
//      warp (__match_any_sync + __reduce_add_sync) before the shared atomic.
//   2. score (areas + validation): row/column sums of the histogram and the
//      reference's value checks, written to the caller's `areas` scratch.
//   3. score (accumulate): per prediction column the confusion contribution,
//      the integer `inter > union / 2` match test, the FP64 IoU, the
//      last-same-class-crowd ignore rule and FP/FN. Gated on the device by the
//      error word, so a failed validation never changes the totals.
// The confusion matrix is derived from the same histogram (no second pixel
// pass). Per-image class sums are reduced in a fixed order.
#include "pe_common.cuh"
#include "pe_score.cuh"

#include <cuda.h>

#include <map>
#include <mutex>

namespace pe {
namespace {

constexpr int kHistThreads = 512;
constexpr int kPixelsPerThread = 8;
constexpr int kTilePixels = kHistThreads * kPixelsPerThread;
constexpr int kScoreThreads = 256;
constexpr int kComputeThreads = 1024;
constexpr int kMaxSmemBins = 50 * 1024;  // 200 KB of uint32 bins

template <typename T>
__device__ __forceinline__ void load8(const T* __restrict__ p, int64_t x, int64_t v[8]);

template <>
__device__ __forceinline__ void load8<int>(const int* __restrict__ p, int64_t x, int64_t v[8]) {
  int4 a = __ldg(reinterpret_cast<const int4*>(p + x));
  int4 b = __ldg(reinterpret_cast<const int4*>(p + x + 4));
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
  v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}

template <>
__device__ __forceinline__ void load8<int64_t>(const int64_t* __restrict__ p, int64_t x, int64_t v[8]) {
  const longlong2* q = reinterpret_cast<const longlong2*>(p + x);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    longlong2 w = __ldg(q + i);
    v[2 * i] = w.x;
    v[2 * i + 1] = w.y;
  }
}

// Per-thread run of equal keys; the last run is warp-aggregated.
struct Run {
  u64 key = ~0ull;
  u32 count = 0;
};

template <bool SMEM>
__device__ __forceinline__ void emit(Run& run, u64 key, u32* bins, u64* pairs) {
  if (key != run.key) {
    if (run.count) {
      if (SMEM) atomicAdd(bins + run.key, run.count);
      else atomicAdd(pairs + run.key, (u64)run.count);
    }
    run.key = key;
    run.count = 0;
  }
  ++run.count;
}

template <typename GT, typename PR, bool SMEM, bool VEC>
__global__ void __launch_bounds__(kHistThreads)
pair_histogram(const GT* __restrict__ gt, const PR* __restrict__ pred, int64_t pixels, int64_t B,
               int G, int P, int64_t tiles_per_image, int64_t tiles_per_cta,
               const int64_t* __restrict__ gt_ids, const int* __restrict__ gt_slots,
               const int64_t* __restrict__ pred_ids, const int* __restrict__ pred_slots,
               u64* __restrict__ pairs, int* __restrict__ error) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  u32* bins = reinterpret_cast<u32*>(smem_raw);
  const int bins_count = G * P;
  const int64_t total_tiles = B * tiles_per_image;
  const int64_t t_begin = (int64_t)blockIdx.x * tiles_per_cta;
  const int64_t t_end = min(t_begin + tiles_per_cta, total_tiles);
  bool bad = false;
  int64_t current = -1;

  auto flush = [&](int64_t image) {
    __syncthreads();
    u64* out = pairs + image * (int64_t)bins_count;
    for (int k = threadIdx.x; k < bins_count; k += blockDim.x) {
      u32 v = bins[k];
      if (v) atomicAdd(out + k, (u64)v);
    }
  };

  for (int64_t t = t_begin; t < t_end; ++t) {
    const int64_t b = t / tiles_per_image;
    if (SMEM && b != current) {
      if (current >= 0) flush(current);
      __syncthreads();
      uint4 zero = make_uint4(0, 0, 0, 0);
      for (int k = threadIdx.x * 4; k + 3 < bins_count; k += blockDim.x * 4)
        *reinterpret_cast<uint4*>(bins + k) = zero;
      for (int k = (bins_count & ~3) + threadIdx.x; k < bins_count; k += blockDim.x) bins[k] = 0;
      __syncthreads();
    }
    current = b;
    const int64_t x0 = (t % tiles_per_image) * kTilePixels;
    const int64_t end = min(x0 + (int64_t)kTilePixels, pixels);
    const int64_t x = x0 + (int64_t)threadIdx.x * kPixelsPerThread;
    const GT* g_img = gt + b * pixels;
    const PR* p_img = pred + b * pixels;
    const int64_t* gi = gt_ids ? gt_ids + b * G : nullptr;
    const int* gs = gt_ids ? gt_slots + b * G : nullptr;
    const int64_t* pi = pred_ids ? pred_ids + b * P : nullptr;
    const int* ps = pred_ids ? pred_slots + b * P : nullptr;
    const u64 base = SMEM ? 0 : (u64)b * (u64)bins_count;

    int64_t gv[kPixelsPerThread], pv[kPixelsPerThread];
    int n = 0;
    if (x < end) {
      if (VEC && x + kPixelsPerThread <= end) {
        load8<GT>(g_img, x, gv);
        load8<PR>(p_img, x, pv);
        n = kPixelsPerThread;
      } else {
        n = (int)min((int64_t)kPixelsPerThread, end - x);
#pragma unroll
        for (int j = 0; j < kPixelsPerThread; ++j)
          if (j < n) { gv[j] = (int64_t)g_img[x + j]; pv[j] = (int64_t)p_img[x + j]; }
      }
    }
    Run run;
    int64_t last_graw = INT64_MIN, last_praw = INT64_MIN;
    int last_g = -1, last_p = -1;
#pragma unroll
    for (int j = 0; j < kPixelsPerThread; ++j) {
      if (j < n) {
        if (gv[j] != last_graw) { last_graw = gv[j]; last_g = resolve_slot(gv[j], gi, gs, G); }
        if (pv[j] != last_praw) { last_praw = pv[j]; last_p = resolve_slot(pv[j], pi, ps, P); }
        if (last_g >= 0 && last_p >= 0)
          emit<SMEM>(run, base + (u64)last_g * P + last_p, bins, pairs);
        else
          bad = true;
      }
    }
    // Last run of every lane: combine equal keys across the warp.
    const u32 peers = __match_any_sync(0xffffffffu, run.key);
    const u32 total = __reduce_add_sync(peers, run.count);
    if ((threadIdx.x & 31) == (u32)(__ffs(peers) - 1) && total) {
      if (SMEM) atomicAdd(bins + run.key, total);
      else atomicAdd(pairs + run.key, (u64)total);
    }
  }
  if (SMEM && current >= 0) flush(current);
  if (bad && error) atomicOr(error, 1);
}

// flags: 1 = areas, 2 = validate (needs areas), 4 = accumulate, 8 = gate on *error.
template <bool REWARD>
__global__ void __launch_bounds__(1024)
score(const u64* __restrict__ pairs, const int* __restrict__ gc, const int* __restrict__ pc,
      const uint8_t* __restrict__ crowd, u64* __restrict__ areas, int* __restrict__ matched,
      u64* __restrict__ tp, u64* __restrict__ fp, u64* __restrict__ fn, double* __restrict__ iou_sum,
      u64* __restrict__ confusion, int G, int P, int C, int flags, int* __restrict__ error) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int64_t b = blockIdx.x;
  if ((flags & 8) && *reinterpret_cast<volatile int*>(error)) return;
  pairs += b * (int64_t)G * P;
  gc += b * G;
  pc += b * P;
  crowd += b * G;
  areas += b * (int64_t)(G + P);
  matched += b * G;
  const int64_t o = REWARD ? b * C : 0;
  if (flags & 1) {
    const int err = score_areas<u64, REWARD>(pairs, gc, pc, crowd, areas, G, P, C, (flags & 2) != 0);
    if (err) atomicOr(error, err);
    __syncthreads();
  }
  if (!(flags & 4)) return;
  ScoreOut out{tp + o, fp + o, fn + o, iou_sum + o, REWARD ? nullptr : confusion};
  score_accumulate<u64, REWARD>(pairs, gc, pc, crowd, areas, matched, G, P, C, out, smem_raw);
}

__global__ void pack_slots_kernel(const void* maps, int is64, int64_t pixels, int64_t total,
                                  const int64_t* __restrict__ ids, const int* __restrict__ slots, int S,
                                  int* __restrict__ out, int* __restrict__ error) {
  bool bad = false;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i / pixels;
    const int64_t key = is64 ? reinterpret_cast<const int64_t*>(maps)[i]
                             : (int64_t)reinterpret_cast<const int*>(maps)[i];
    const int slot = resolve_slot(key, ids + b * S, slots + b * S, S);
    out[i] = slot >= 0 ? slot : 0;
    bad |= slot < 0;
  }
  if (bad) atomicOr(error, 1);
}

// COCO panoptic PNG pixels (RGB8, as decoded from the file) -> segment IDs
// R + 256 G + 65536 B (the reference's README input rule), then through the
// image's sorted lookup table (staged in shared memory) to a compact slot,
// or written as the ID itself when there is no table. One image per grid row,
// 16 pixels per thread: 48 bytes in, 64 bytes out; consecutive equal IDs reuse
// the previous lookup.
constexpr int kRgbThreads = 256;
constexpr int kRgbPixels = 16;

__global__ void __launch_bounds__(kRgbThreads)
rgb_slots_kernel(const uint8_t* __restrict__ rgb, int64_t pixels, const int64_t* __restrict__ ids,
                 const int* __restrict__ slots, int S, int vec, int* __restrict__ out, int* __restrict__ error) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  int64_t* s_ids = reinterpret_cast<int64_t*>(smem_raw);
  int* s_slots = reinterpret_cast<int*>(s_ids + S);
  const int64_t b = blockIdx.y;
  if (ids) {
    for (int i = threadIdx.x; i < S; i += blockDim.x) {
      s_ids[i] = ids[b * S + i];
      s_slots[i] = slots[b * S + i];
    }
    __syncthreads();
  }
  const uint8_t* src = rgb + b * pixels * 3;
  int* dst = out + b * pixels;
  bool bad = false;
  int64_t last_key = -1;
  int last_slot = 0;
  for (int64_t x = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * kRgbPixels; x < pixels;
       x += (int64_t)gridDim.x * blockDim.x * kRgbPixels) {
    uint32_t w[12];
    const bool full = x + kRgbPixels <= pixels;
    if (vec && full) {
      const uint4* q = reinterpret_cast<const uint4*>(src + x * 3);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const uint4 v = __ldcs(q + k);
        w[4 * k] = v.x; w[4 * k + 1] = v.y; w[4 * k + 2] = v.z; w[4 * k + 3] = v.w;
      }
    } else {
#pragma unroll
      for (int k = 0; k < 12; ++k) w[k] = 0;
#pragma unroll
      for (int k = 0; k < 3 * kRgbPixels; ++k)
        if (x * 3 + k < pixels * 3) w[k >> 2] |= (uint32_t)src[x * 3 + k] << (8 * (k & 3));
    }
    int v[kRgbPixels];
#pragma unroll
    for (int j = 0; j < kRgbPixels; ++j) {
      const uint32_t r = (w[(3 * j) >> 2] >> (8 * ((3 * j) & 3))) & 0xffu;
      const uint32_t g = (w[(3 * j + 1) >> 2] >> (8 * ((3 * j + 1) & 3))) & 0xffu;
      const uint32_t bl = (w[(3 * j + 2) >> 2] >> (8 * ((3 * j + 2) & 3))) & 0xffu;
      const int64_t key = (int64_t)(r | (g << 8) | (bl << 16));
      if (!ids) {
        v[j] = (int)key;
        continue;
      }
      if (key != last_key) {
        last_key = key;
        last_slot = resolve_slot(key, s_ids, s_slots, S);
      }
      const bool inside = x + j < pixels;
      bad |= inside && last_slot < 0;
      v[j] = last_slot >= 0 ? last_slot : 0;
    }
    if (vec && full) {
      int4* o = reinterpret_cast<int4*>(dst + x);
#pragma unroll
      for (int k = 0; k < 4; ++k) o[k] = make_int4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
    } else {
#pragma unroll
      for (int j = 0; j < kRgbPixels; ++j)
        if (x + j < pixels) dst[x + j] = v[j];
    }
  }
  if (bad) atomicOr(error, 1);
}

// Per-class PQ/SQ/RQ and semantic IoU, group means and mIoU for K rows of
// statistics, plus independent copies of the inputs (compute_kernel.cu:9-63).
// One CTA per row. The confusion matrix is read once, row-major and coalesced:
// warp w takes rows w, w + 32, ..., reduces each row with shuffles and keeps
// column partials in registers, added into shared column sums at the end of a
// 256-column tile. FP64 runs only where a value is produced: one class per
// thread for the per-class ratios, then one warp per summed quantity (fixed
// order: lane-strided classes, then a butterfly), so no warp issues FP64 adds
// of zeros (GB300's FP64 pipe runs at 1/64 of the FP32 rate).
constexpr int kComputeTile = 256;  // confusion columns per register tile (8 per lane)

__global__ void __launch_bounds__(kComputeThreads)
compute_kernel(const int64_t* __restrict__ tp, const int64_t* __restrict__ fp, const int64_t* __restrict__ fn,
               const double* __restrict__ sums, const int64_t* __restrict__ confusion,
               const bool* __restrict__ things, double* per_class, double* summaries, int64_t* counts,
               double* miou, int64_t* out_tp, int64_t* out_fp, int64_t* out_fn, double* out_sums,
               int64_t* out_confusion, int C) {
  const int64_t k = blockIdx.x;
  tp += k * C; fp += k * C; fn += k * C; sums += k * C;
  confusion += k * C * (int64_t)(C + 1);
  per_class += k * 4 * C;
  summaries += k * 9;
  counts += k * 3;
  if (out_tp) {
    out_tp += k * C; out_fp += k * C; out_fn += k * C; out_sums += k * C;
    out_confusion += k * C * (int64_t)(C + 1);
  }
  extern __shared__ __align__(16) unsigned char smem_raw[];
  int64_t* row_sum = reinterpret_cast<int64_t*>(smem_raw);  // C confusion row sums
  int64_t* col_sum = row_sum + C;                            // C column sums
  double* value = reinterpret_cast<double*>(col_sum + C);    // [4][C]: pq, sq, rq, iou (NaN: no pixels)
  int* group = reinterpret_cast<int*>(value + 4 * C);        // C: 0 inactive, 1 thing, 2 stuff (active)
  __shared__ double total[10];
  __shared__ int n_group[3], n_iou;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5, warps = blockDim.x >> 5;
  for (int c = t; c < C; c += blockDim.x) row_sum[c] = col_sum[c] = 0;
  if (t < 3) n_group[t] = 0;
  if (t == 0) n_iou = 0;
  // Snapshot copies (independent of everything below): 16-byte words when aligned.
  if (out_tp) {
    for (int c = t; c < C; c += blockDim.x) {
      out_tp[c] = tp[c]; out_fp[c] = fp[c]; out_fn[c] = fn[c]; out_sums[c] = sums[c];
    }
    const int64_t n = (int64_t)C * (C + 1);
    if (((reinterpret_cast<uintptr_t>(confusion) | reinterpret_cast<uintptr_t>(out_confusion)) & 15) == 0) {
      const int4* src = reinterpret_cast<const int4*>(confusion);
      int4* dst = reinterpret_cast<int4*>(out_confusion);
      for (int64_t i = t; i < n / 2; i += blockDim.x) dst[i] = src[i];
      if (t == 0 && (n & 1)) out_confusion[n - 1] = confusion[n - 1];
    } else {
      for (int64_t i = t; i < n; i += blockDim.x) out_confusion[i] = confusion[i];
    }
  }
  __syncthreads();
  // Row and column sums in one coalesced pass over the confusion rows.
  for (int t0 = 0; t0 <= C; t0 += kComputeTile) {
    int64_t acc[kComputeTile / 32];
#pragma unroll
    for (int i = 0; i < kComputeTile / 32; ++i) acc[i] = 0;
    for (int r = warp; r < C; r += warps) {
      const int64_t* row = confusion + (int64_t)r * (C + 1);
      int64_t part = 0;
#pragma unroll
      for (int i = 0; i < kComputeTile / 32; ++i) {
        const int j = t0 + lane + 32 * i;
        if (j <= C) {
          const int64_t v = row[j];
          part += v;
          if (j < C) acc[i] += v;
        }
      }
#pragma unroll
      for (int o = 16; o; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
      if (lane == 0) row_sum[r] += part;  // row r belongs to this warp alone
    }
#pragma unroll
    for (int i = 0; i < kComputeTile / 32; ++i) {
      const int j = t0 + lane + 32 * i;
      if (j < C && acc[i]) atomicAdd(reinterpret_cast<unsigned long long*>(col_sum + j), (unsigned long long)acc[i]);
    }
  }
  __syncthreads();
  // Per-class ratios, one class per thread.
  for (int c = t; c < C; c += blockDim.x) {
    const int64_t a = tp[c], f = fp[c], n = fn[c];
    const double s = sums[c];
    const double denom = (double)a + 0.5 * ((double)f + (double)n);
    const double pq = denom > 0 ? s / denom : 0.0;
    const double sq = a ? s / (double)a : 0.0;
    const double rq = denom > 0 ? (double)a / denom : 0.0;
    const int64_t diag = confusion[(int64_t)c * (C + 1) + c];
    const int64_t uni = row_sum[c] + col_sum[c] - diag;
    const double iou = uni ? (double)diag / (double)uni : __longlong_as_double(0x7ff8000000000000ll);
    per_class[c] = pq;
    per_class[C + c] = sq;
    per_class[2 * C + c] = rq;
    per_class[3 * C + c] = iou;
    value[c] = pq;
    value[C + c] = sq;
    value[2 * C + c] = rq;
    value[3 * C + c] = iou;
    const int g = denom > 0 ? (things[c] ? 1 : 2) : 0;
    group[c] = g;
    if (g) { atomicAdd(&n_group[0], 1); atomicAdd(&n_group[g], 1); }
    if (uni) atomicAdd(&n_iou, 1);
  }
  __syncthreads();
  // Ten sums, one warp each: quantity q = 3 * scope + metric (scope 0 all, 1 things, 2 stuff), q = 9 IoU.
  for (int q = warp; q < 10; q += warps) {
    const int metric = q < 9 ? q % 3 : 3, scope = q < 9 ? q / 3 : 0;
    double part = 0.0;
    for (int c = lane; c < C; c += 32) {
      const bool in = q < 9 ? (group[c] != 0 && (scope == 0 || group[c] == scope)) : !isnan(value[3 * C + c]);
      if (in) part += value[metric * C + c];
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if (lane == 0) total[q] = part;
  }
  __syncthreads();
  if (t < 9) {
    const int scope = t / 3;
    const int n = n_group[scope];
    summaries[t] = n ? total[t] / (double)n : 0.0;
  }
  if (t < 3) counts[t] = n_group[t];
  if (t == 0) miou[k] = n_iou ? total[9] / (double)n_iou : 0.0;
}

// Launch choices of the per-call update, set by the host's tuner per bucket of
// (floor(log2(G * P)), floor(log2(pixels per image))): histogram bins in shared memory or in
// global memory, histogram CTAs per SM, and threads of each image's scoring CTA. Without an entry
// the built-in rule applies: shared bins whenever they fit, up to 4 CTAs per SM as their shared
// memory allows, 256 scoring threads.
struct UpdateChoice {
  int smem;           // 1: shared-memory bins, 0: global bins
  int per_sm;         // histogram CTAs per SM
  int score_threads;  // threads of the per-image scoring CTA (256, 512 or 1024)
};
std::mutex g_tune_mutex;
std::map<std::pair<int, int>, UpdateChoice> g_update_tuning;

int log2_bucket(int64_t v) { return v > 0 ? 63 - __builtin_clzll((unsigned long long)v) : -1; }

// CTAs of kHistThreads threads one SM can hold (at most 4), and fewer when their bins fill shared memory.
int max_per_sm(bool smem, int64_t bins) {
  constexpr int kResident = 2048 / kHistThreads;
  if (!smem) return kResident;
  const size_t bytes = (size_t)round_up(bins, 4) * sizeof(u32);
  return (int)std::max<int64_t>(1, std::min<int64_t>(kResident, (220 * 1024) / (int64_t)std::max<size_t>(bytes, 1)));
}

UpdateChoice update_choice(int64_t bins, int64_t pixels) {
  const bool fits = bins <= kMaxSmemBins;
  UpdateChoice choice{fits ? 1 : 0, std::min(4, max_per_sm(fits, bins)), kScoreThreads};
  {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    const auto it = g_update_tuning.find({log2_bucket(bins), log2_bucket(pixels)});
    if (it != g_update_tuning.end()) choice = it->second;
  }
  choice.smem = choice.smem && fits;  // a tuned choice never exceeds what this launch can hold
  choice.per_sm = std::max(1, std::min(choice.per_sm, max_per_sm(choice.smem, bins)));
  if (choice.score_threads != 512 && choice.score_threads != 1024) choice.score_threads = kScoreThreads;
  return choice;
}

template <typename GT, typename PR>
int launch_histogram(const void* gt, const void* pred, int64_t B, int64_t pixels, int G, int P,
                     const int64_t* gi, const int* gs, const int64_t* pi, const int* ps, u64* pairs, int* error,
                     bool vec, cudaStream_t stream) {
  const int64_t bins = (int64_t)G * P;
  const UpdateChoice choice = update_choice(bins, pixels);
  const bool smem = choice.smem;
  const size_t smem_bytes = smem ? (size_t)round_up(bins, 4) * sizeof(u32) : 0;
  const int64_t tiles_per_image = ceil_div(pixels, kTilePixels);
  const int64_t total_tiles = B * tiles_per_image;
  const int per_sm = choice.per_sm;
  const int64_t max_ctas = (int64_t)sm_count() * per_sm;
  const int64_t tiles_per_cta = ceil_div(total_tiles, std::min<int64_t>(total_tiles, max_ctas));
  const int64_t grid = ceil_div(total_tiles, tiles_per_cta);
  auto* g = static_cast<const GT*>(gt);
  auto* p = static_cast<const PR*>(pred);
#define PE_HIST(SM, VC)                                                                                \
  do {                                                                                                 \
    auto kernel = pair_histogram<GT, PR, SM, VC>;                                                      \
    if (smem_bytes > 48 * 1024)                                                                        \
      PE_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes)); \
    kernel<<<(unsigned)grid, kHistThreads, smem_bytes, stream>>>(g, p, pixels, B, G, P, tiles_per_image, \
                                                                 tiles_per_cta, gi, gs, pi, ps, pairs, error); \
  } while (0)
  if (smem) {
    if (vec) PE_HIST(true, true); else PE_HIST(true, false);
  } else {
    if (vec) PE_HIST(false, true); else PE_HIST(false, false);
  }
#undef PE_HIST
  PE_LAUNCHED("pair_histogram");
  count_launch();
  return kOk;
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

}  // namespace
}  // namespace pe

using namespace pe;

// Drop-in for the reference's `update` op (bindings.cpp:29; histogram_kernel.cu:257-341).
PE_API int pe_update(const void* gt, int gt_is_int64, const void* pred, int pred_is_int64, int64_t B,
                     int64_t pixels, const int32_t* gc, const int32_t* pc, const uint8_t* crowd, int64_t G,
                     int64_t P, int64_t C, int64_t* pairs, int64_t* areas, int32_t* matched, int64_t* tp,
                     int64_t* fp, int64_t* fn, double* iou_sum, int64_t* confusion, const int64_t* gt_ids,
                     const int32_t* gt_slots, const int64_t* pred_ids, const int32_t* pred_slots, int32_t* error,
                     int validate, int reward, cudaStream_t stream) {
  PE_REQUIRE(B >= 0 && pixels >= 0, "negative batch or image size");
  PE_REQUIRE(C > 0 && C < INT_MAX && G > 0 && G < INT_MAX && P > 0 && P < INT_MAX, "invalid capacities");
  PE_REQUIRE(G * P < INT_MAX, "G x P histogram too large");
  PE_REQUIRE((gt_ids == nullptr) == (gt_slots == nullptr) && (pred_ids == nullptr) == (pred_slots == nullptr),
             "lookup IDs and slots must be supplied together");
  PE_REQUIRE(!validate || error, "validation needs an error word");
  PE_REQUIRE(reward || confusion, "confusion is required outside reward mode");
  if (B == 0) return kOk;
  PE_REQUIRE(gc && pc && crowd && pairs && areas && matched && tp && fp && fn && iou_sum, "null state pointer");
  const int64_t total = B * pixels;
  PE_CUDA(cudaMemsetAsync(pairs, 0, sizeof(int64_t) * B * G * P, stream));
  if (validate) PE_CUDA(cudaMemsetAsync(error, 0, sizeof(int32_t), stream));
  auto* upairs = reinterpret_cast<u64*>(pairs);
  int* err = validate ? error : nullptr;
  if (total > 0) {
    PE_REQUIRE(gt && pred, "null map pointer");
    const bool no_lookup = gt_ids == nullptr && pred_ids == nullptr;
    int status;
    if (!gt_is_int64 && !pred_is_int64) {
      const bool vec = no_lookup && pixels % 4 == 0 && aligned16(gt) && aligned16(pred);
      status = launch_histogram<int, int>(gt, pred, B, pixels, (int)G, (int)P, gt_ids, gt_slots, pred_ids,
                                          pred_slots, upairs, err, vec, stream);
    } else if (gt_is_int64 && pred_is_int64) {
      const bool vec = pixels % 2 == 0 && aligned16(gt) && aligned16(pred);
      status = launch_histogram<int64_t, int64_t>(gt, pred, B, pixels, (int)G, (int)P, gt_ids, gt_slots,
                                                  pred_ids, pred_slots, upairs, err, vec, stream);
    } else if (gt_is_int64) {
      status = launch_histogram<int64_t, int>(gt, pred, B, pixels, (int)G, (int)P, gt_ids, gt_slots, pred_ids,
                                              pred_slots, upairs, err, false, stream);
    } else {
      status = launch_histogram<int, int64_t>(gt, pred, B, pixels, (int)G, (int)P, gt_ids, gt_slots, pred_ids,
                                              pred_slots, upairs, err, false, stream);
    }
    if (status != kOk) return status;
  }
  const size_t smem = score_staging_bytes(P);
  PE_REQUIRE(smem <= 200 * 1024, "too many prediction slots for the scoring kernel (P=%lld)", (long long)P);
  auto kernel = reward ? score<true> : score<false>;
  const int score_threads = update_choice(G * P, pixels).score_threads;
  if (smem > 48 * 1024)
    PE_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  auto* ua = reinterpret_cast<u64*>(areas);
  auto* utp = reinterpret_cast<u64*>(tp);
  auto* ufp = reinterpret_cast<u64*>(fp);
  auto* ufn = reinterpret_cast<u64*>(fn);
  auto* uconf = reinterpret_cast<u64*>(confusion);
  auto* cr = crowd;
  if (validate) {
    kernel<<<(unsigned)B, score_threads, smem, stream>>>(upairs, gc, pc, cr, ua, matched, utp, ufp, ufn, iou_sum,
                                                         uconf, (int)G, (int)P, (int)C, 1 | 2, error);
    PE_LAUNCHED("score(areas)");
    kernel<<<(unsigned)B, score_threads, smem, stream>>>(upairs, gc, pc, cr, ua, matched, utp, ufp, ufn, iou_sum,
                                                         uconf, (int)G, (int)P, (int)C, 4 | 8, error);
    PE_LAUNCHED("score(accumulate)");
    count_launch(2);
    int code = 0;
    PE_CUDA(cudaMemcpyAsync(&code, error, sizeof(int), cudaMemcpyDeviceToHost, stream));
    PE_CUDA(cudaStreamSynchronize(stream));
    return code;
  }
  kernel<<<(unsigned)B, score_threads, smem, stream>>>(upairs, gc, pc, cr, ua, matched, utp, ufp, ufn, iou_sum,
                                                       uconf, (int)G, (int)P, (int)C, 1 | 4, nullptr);
  PE_LAUNCHED("score");
  count_launch();
  return kOk;
}

// Mean-class PQ per image from [B][C] reward statistics (evaluator.py:539-544),
// one warp per image, classes reduced in a fixed order; optionally adds the
// statistics into dataset totals [C].
__global__ void reward_pq_kernel(const int64_t* __restrict__ tp, const int64_t* __restrict__ fp,
                                 const int64_t* __restrict__ fn, const double* __restrict__ sums, int64_t B, int C,
                                 double* __restrict__ pq, int64_t* __restrict__ tot_tp, int64_t* __restrict__ tot_fp,
                                 int64_t* __restrict__ tot_fn, double* __restrict__ tot_sums) {
  const int64_t b = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (b >= B) return;
  const int64_t o = b * C;
  double total = 0.0;
  int active = 0;
  for (int c = lane; c < C; c += 32) {
    const int64_t a = tp[o + c], f = fp[o + c], n = fn[o + c];
    const double denom = (double)a + 0.5 * ((double)f + (double)n);
    if (denom > 0) {
      total += sums[o + c] / (denom > 1.0 ? denom : 1.0);
      ++active;
    }
    if (tot_tp && (a | f | n)) {
      atomicAdd(reinterpret_cast<u64*>(tot_tp) + c, (u64)a);
      atomicAdd(reinterpret_cast<u64*>(tot_fp) + c, (u64)f);
      atomicAdd(reinterpret_cast<u64*>(tot_fn) + c, (u64)n);
      atomicAdd(tot_sums + c, sums[o + c]);
    }
  }
#pragma unroll
  for (int s = 16; s; s >>= 1) {
    total += __shfl_xor_sync(0xffffffffu, total, s);
    active += __shfl_xor_sync(0xffffffffu, active, s);
  }
  if (lane == 0) pq[b] = total / (double)(active > 1 ? active : 1);
}

// Drop-in for the reference's `compute` / prefix compute (compute_kernel.cu:66-118).
// Rows k = 0..K-1 of tp/fp/fn/sums [K, C] and confusion [K, C, C+1]; output
// copies are skipped when out_tp is null.
PE_API int pe_compute(const int64_t* tp, const int64_t* fp, const int64_t* fn, const double* sums,
                      const int64_t* confusion, const uint8_t* things, int64_t K, int64_t C, double* per_class,
                      double* summaries, int64_t* counts, double* miou, int64_t* out_tp, int64_t* out_fp,
                      int64_t* out_fn, double* out_sums, int64_t* out_confusion, cudaStream_t stream) {
  PE_REQUIRE(C > 0 && C < INT_MAX && K >= 0 && K < INT_MAX, "invalid category or row count");
  if (K == 0) return kOk;
  const size_t smem = (sizeof(int64_t) * 2 + sizeof(double) * 4 + sizeof(int)) * (size_t)C;
  PE_REQUIRE(smem <= 200 * 1024, "too many categories for the compute kernel (C=%lld)", (long long)C);
  if (smem > 48 * 1024)
    PE_CUDA(cudaFuncSetAttribute(compute_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  compute_kernel<<<(unsigned)K, kComputeThreads, smem, stream>>>(tp, fp, fn, sums, confusion, reinterpret_cast<const bool*>(things),
                                                  per_class, summaries, counts, miou, out_tp, out_fp, out_fn,
                                                  out_sums, out_confusion, (int)C);
  PE_LAUNCHED("compute");
  count_launch();
  return kOk;
}

// Per-image mean-class PQ from [B][C] reward statistics into pq[B]; when
// tot_tp is not NULL the statistics are also added into dataset totals [C].
PE_API int pe_reward_pq(const int64_t* tp, const int64_t* fp, const int64_t* fn, const double* sums, int64_t B,
                        int64_t C, double* pq, int64_t* tot_tp, int64_t* tot_fp, int64_t* tot_fn, double* tot_sums,
                        cudaStream_t stream) {
  PE_REQUIRE(B >= 0 && C > 0 && C < INT_MAX, "invalid reward shapes");
  if (B == 0) return kOk;
  reward_pq_kernel<<<(unsigned)ceil_div(B, 8), 256, 0, stream>>>(tp, fp, fn, sums, B, (int)C, pq, tot_tp, tot_fp,
                                                                  tot_fn, tot_sums);
  PE_LAUNCHED("reward_pq");
  count_launch();
  return kOk;
}

// Drop-in for the reference's `pack` op (histogram_kernel.cu:343-366): original
// IDs -> compact slots; *error gets bit 1 for IDs absent from the tables.
PE_API int pe_pack(const void* maps, int maps_is_int64, int64_t B, int64_t pixels, const int64_t* ids,
                   const int32_t* slots, int64_t S, int32_t* out, int32_t* error, cudaStream_t stream) {
  PE_REQUIRE(B >= 0 && pixels >= 0 && S > 0 && S < INT_MAX, "invalid lookup shapes");
  PE_CUDA(cudaMemsetAsync(error, 0, sizeof(int32_t), stream));
  const int64_t total = B * pixels;
  if (total == 0) return kOk;
  const int64_t blocks = std::min<int64_t>(ceil_div(total, 256), (int64_t)sm_count() * 8);
  pack_slots_kernel<<<(unsigned)blocks, 256, 0, stream>>>(maps, maps_is_int64, pixels, total, ids, slots, (int)S,
                                                          out, error);
  PE_LAUNCHED("pack");
  count_launch();
  return kOk;
}

// COCO panoptic PNG pixels -> compact slots (or IDs). rgb: B x pixels x 3 uint8
// (R, G, B per pixel, the decoded PNG); ids / slots: sorted B x S lookup tables
// as for pe_pack, or both NULL to write the IDs R + 256 G + 65536 B instead.
// *error gets bit 1 for IDs absent from the tables.
PE_API int pe_pack_rgb(const uint8_t* rgb, int64_t B, int64_t pixels, const int64_t* ids, const int32_t* slots,
                       int64_t S, int32_t* out, int32_t* error, cudaStream_t stream) {
  PE_REQUIRE(B >= 0 && B <= 65535 && pixels >= 0, "invalid RGB batch (at most 65535 images per call)");
  PE_REQUIRE((ids == nullptr) == (slots == nullptr), "lookup IDs and slots go together");
  PE_REQUIRE(!ids || (S > 0 && S <= 16384), "lookup tables must have 1..16384 entries per image");
  if (error) PE_CUDA(cudaMemsetAsync(error, 0, sizeof(int32_t), stream));
  if (B == 0 || pixels == 0) return kOk;
  const size_t smem = ids ? (size_t)S * (sizeof(int64_t) + sizeof(int)) : 0;
  if (smem > 48 * 1024)
    PE_CUDA(cudaFuncSetAttribute(rgb_slots_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int vec = (reinterpret_cast<uintptr_t>(rgb) % 16 == 0) && (reinterpret_cast<uintptr_t>(out) % 16 == 0) &&
                  pixels % 16 == 0;
  const int64_t per_block = (int64_t)kRgbThreads * kRgbPixels;
  const int64_t want = std::max<int64_t>(1, (int64_t)sm_count() * 8 / std::max<int64_t>(B, 1));
  const int64_t gx = std::min<int64_t>(ceil_div(pixels, per_block), want);
  rgb_slots_kernel<<<dim3((unsigned)gx, (unsigned)B), kRgbThreads, smem, stream>>>(rgb, pixels, ids, slots, (int)S,
                                                                                    vec, out, error);
  PE_LAUNCHED("pack_rgb");
  count_launch();
  return kOk;
}

// ---- pe_update without caller-provided scratch ------------------------------
//
// Some host applications cannot call cudaMalloc: a process whose device memory
// is owned entirely by another runtime's allocator (a framework's caching
// allocator, or a serving engine that reserves all HBM at start-up), or a
// latency-critical loop where an allocation would synchronise the device.
// pe_update_noalloc serves them: it behaves like pe_update but takes its
// histogram, area and error scratch from one fixed array in this library's
// device memory, so the caller passes only inputs and outputs.
//
// The array below is 8 MiB and is held on every GPU that loads this library
// until the process exits. All calls share it: calls that overlap on the GPU
// (different streams, or different host threads) race on its contents.

namespace pe {
namespace {
constexpr size_t kNoAllocScratchBytes = size_t(8) << 20;
static __device__ __align__(256) unsigned char g_update_scratch[kNoAllocScratchBytes];

std::mutex g_scratch_mutex;
void* g_scratch_address[64] = {nullptr};
unsigned long long g_scratch_context[64] = {0};

// Unique ID of the calling thread's current CUDA context (0 when there is none
// or the CUDA driver does not say). cuCtxGetCurrent / cuCtxGetId are resolved once
// through the runtime, so the library does not link libcuda itself.
unsigned long long current_context_id() {
  using GetCurrent = CUresult (*)(CUcontext*);
  using GetId = CUresult (*)(CUcontext, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult found;
    void* fn = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &found) == cudaSuccess &&
        found == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrent>(fn);
    fn = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &found) == cudaSuccess &&
        found == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(fn);
  });
  CUcontext context = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&context) != CUDA_SUCCESS || context == nullptr ||
      get_id(context, &id) != CUDA_SUCCESS)
    return 0;
  return id;
}

// Device address of g_update_scratch on the current device. The host-side
// symbol is only a stand-in, never a device address. The address is looked up
// on a device's first call and again whenever the device's context is not the
// one it was looked up in (a cudaDeviceReset recreates the context and reloads
// this module, which moves the array).
int scratch_address(void** out) {
  const int device = current_device();
  if (device < 0 || device >= 64) {
    set_error("pe_update_noalloc: device %d outside the supported range", device);
    return kUnsupported;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  const unsigned long long context = current_context_id();
  if (g_scratch_address[device] == nullptr || context == 0 || context != g_scratch_context[device]) {
    void* ptr = nullptr;
    const cudaError_t status = cudaGetSymbolAddress(&ptr, g_update_scratch);
    if (status != cudaSuccess || ptr == nullptr) {
      set_error("pe_update_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(status));
      return kCudaError;
    }
    g_scratch_address[device] = ptr;
    g_scratch_context[device] = current_context_id();  // the lookup made the primary context current
  }
  *out = g_scratch_address[device];
  return kOk;
}
}  // namespace
}  // namespace pe

// Same arguments and results as pe_update minus pairs/areas/matched/error.
// Scratch needed: 8*B*G*P + 8*B*(G+P) + 4*B*G bytes (+ alignment) must fit in
// 8 MiB, otherwise -1 is returned and pe_last_error() names the sizes. The
// histogram scratch is cleared on the stream by every call (pe_update zeroes
// it); the area and match scratch are fully rewritten. The first call on each
// device (and the first after the device's context was recreated, as by
// cudaDeviceReset) looks up the scratch address (cudaGetSymbolAddress); make
// that first call before any stream capture on that device.
PE_API int pe_update_noalloc(const void* gt, int gt_is_int64, const void* pred, int pred_is_int64, int64_t B,
                             int64_t pixels, const int32_t* gc, const int32_t* pc, const uint8_t* crowd, int64_t G,
                             int64_t P, int64_t C, int64_t* tp, int64_t* fp, int64_t* fn, double* iou_sum,
                             int64_t* confusion, const int64_t* gt_ids, const int32_t* gt_slots,
                             const int64_t* pred_ids, const int32_t* pred_slots, int validate, int reward,
                             cudaStream_t stream) {
  PE_REQUIRE(B >= 0 && G > 0 && P > 0 && G < INT_MAX && P < INT_MAX, "invalid capacities");
  // Bound every factor before the byte counts below are formed, so none of them can wrap.
  PE_REQUIRE(B <= (int64_t)kNoAllocScratchBytes && G * P <= (int64_t)kNoAllocScratchBytes &&
                 B * G * P <= (int64_t)kNoAllocScratchBytes,
             "pe_update_noalloc: B=%lld G=%lld P=%lld exceeds the fixed scratch limit of %zu bytes "
             "(use pe_update with caller-provided scratch)",
             (long long)B, (long long)G, (long long)P, kNoAllocScratchBytes);
  const size_t pairs_bytes = (size_t)round_up(8 * B * G * P, 256);
  const size_t areas_bytes = (size_t)round_up(8 * B * (G + P), 256);
  const size_t matched_bytes = (size_t)round_up(4 * B * G, 256);
  const size_t need = pairs_bytes + areas_bytes + matched_bytes + 256;
  PE_REQUIRE(need <= kNoAllocScratchBytes,
             "pe_update_noalloc: B=%lld G=%lld P=%lld needs %zu bytes of scratch; the fixed limit is %zu bytes "
             "(use pe_update with caller-provided scratch)",
             (long long)B, (long long)G, (long long)P, need, kNoAllocScratchBytes);
  void* base = nullptr;
  const int status = scratch_address(&base);
  if (status != kOk) return status;
  unsigned char* bytes = static_cast<unsigned char*>(base);
  auto* pairs = reinterpret_cast<int64_t*>(bytes);
  auto* areas = reinterpret_cast<int64_t*>(bytes + pairs_bytes);
  auto* matched = reinterpret_cast<int32_t*>(bytes + pairs_bytes + areas_bytes);
  auto* error = reinterpret_cast<int32_t*>(bytes + pairs_bytes + areas_bytes + matched_bytes);
  return pe_update(gt, gt_is_int64, pred, pred_is_int64, B, pixels, gc, pc, crowd, G, P, C, pairs, areas, matched,
                   tp, fp, fn, iou_sum, confusion, gt_ids, gt_slots, pred_ids, pred_slots, error, validate, reward,
                   stream);
}

// Per-call update tuning (no reference counterpart; the reference reads PANOPTIC_HISTOGRAM and
// PANOPTIC_SCORING on every call, histogram_kernel.cu:240-246,309-310). Records, for the bucket of
// (floor(log2(bins)), floor(log2(pixels))), shared (1) or global (0) histogram bins, histogram CTAs
// per SM (1..4) and scoring threads per image (256, 512, 1024); smem < 0 removes the bucket's entry.
// pe_update_choice reports the choice a launch of that shape uses.
PE_API int pe_tune_update(int64_t bins, int64_t pixels, int smem, int ctas_per_sm, int score_threads) {
  PE_REQUIRE(bins > 0 && pixels > 0, "bins and pixels must be positive");
  const std::pair<int, int> key{log2_bucket(bins), log2_bucket(pixels)};
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  if (smem < 0) {
    g_update_tuning.erase(key);
    return kOk;
  }
  PE_REQUIRE(ctas_per_sm >= 1 && ctas_per_sm <= 4, "ctas_per_sm must be in 1..4");
  PE_REQUIRE(score_threads == 256 || score_threads == 512 || score_threads == 1024,
             "score_threads must be 256, 512 or 1024");
  g_update_tuning[key] = UpdateChoice{smem ? 1 : 0, ctas_per_sm, score_threads};
  return kOk;
}

PE_API int pe_update_choice(int64_t bins, int64_t pixels, int32_t* smem, int32_t* ctas_per_sm,
                            int32_t* score_threads) {
  PE_REQUIRE(bins > 0 && pixels > 0 && smem && ctas_per_sm && score_threads, "invalid query");
  const UpdateChoice choice = update_choice(bins, pixels);
  *smem = choice.smem;
  *ctas_per_sm = choice.per_sm;
  *score_threads = choice.score_threads;
  return kOk;
}
