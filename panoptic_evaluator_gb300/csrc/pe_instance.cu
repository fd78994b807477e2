// COCO mask AP/AR: detection x target-slot histograms, mask overlaps, greedy
// matching and 101-point precision/recall accumulation.
//
// Matching runs one warp per (image, class): the warp compacts the class's
// detections (score order, top 100 ranked) and ground truths (metadata
// order) with ballots, then each lane owns one of the 40 (area range x IoU
// threshold) chains and runs COCO's greedy scan for it. Per detection the warp
// first ballots, for each of the 10 thresholds, the targets whose IoU reaches
// it; a chain then visits only those candidates (bit masks of crowd and
// area-ignored targets remove the rest), in metadata order as the reference's
// scan does.
//
// Accumulation runs one CTA per class: it gathers the class's records in
// order (sorting them by descending score when they are not presorted), then
// each of 120 threads owns one (threshold, area, maxDets) chain. A chain puts
// the precision of every record into the bucket of its recall grid position
// and the interpolated curve is the suffix maximum of the buckets, which is
// the reference's searchsorted-on-envelope rule evaluated in one pass.
#include "pe_common.cuh"

#include <cfloat>

namespace pe {
namespace {

constexpr int kChains = 40;
constexpr int kMaxDets = 100;
constexpr int kMatchWarps = 8;

__device__ __forceinline__ void area_range(int a, double& lo, double& hi) {
  lo = a == 2 ? 1024.0 : (a == 3 ? 9216.0 : 0.0);
  hi = a == 1 ? 1024.0 : (a == 2 ? 9216.0 : 1e10);
}

__device__ __forceinline__ double iou_threshold(int t) {
  // instance.py:252 (0.8999999999999999 is the literal value, not 0.9).
  const double table[10] = {0.5, 0.55, 0.6, 0.65, 0.7, 0.75, 0.8, 0.85, 0.8999999999999999, 0.95};
  return table[t];
}

constexpr int kIouCap = 512;  // (detection, target) IoUs of one class staged up front when they fit

__host__ __device__ inline int iou_entries(int g_max) { return g_max > kIouCap ? g_max : kIouCap; }

// Shared memory of one matching warp for up to g_max targets per image: the class's IoU table (or
// one detection's row), its detections and targets, 40 chains' taken bits, target bit masks (crowd,
// ignored per area range, reaching each IoU threshold), per-target and per-detection flags.
__host__ __device__ inline size_t match_warp_bytes(int g_max) {
  const int words = (g_max + 31) / 32;
  const size_t bytes = sizeof(long long) * (size_t)iou_entries(g_max) + sizeof(int) * ((size_t)100 + g_max) +
                       sizeof(uint32_t) * (size_t)(40 + 15) * words + 2 * (size_t)g_max + 100;
  return (bytes + 15) / 16 * 16;
}

struct FlagLayout {
  int8_t* base;         // flags of image 0
  int64_t chain_stride;  // distance between chains
  int64_t det_stride;    // distance between detections
};

// ---- greedy matching ------------------------------------------------------

// The class of the n-th (0-based) set bit of row[0, words), or -1 when fewer
// bits are set; every lane of the warp gets the same answer.
__device__ __forceinline__ int nth_present_class(const u32* __restrict__ row, int words, int n, int lane) {
  for (int w0 = 0; w0 < words; w0 += 32) {
    const int w = w0 + lane;
    const u32 v = w < words ? row[w] : 0u;
    const int cnt = __popc(v);
    int incl = cnt;  // inclusive scan of the set bits over the lanes' words
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    if (n < total) {
      const int src = __ffs(__ballot_sync(0xffffffffu, incl > n)) - 1;  // the word holding bit n
      const int before = __shfl_sync(0xffffffffu, incl - cnt, src);
      u32 word = __shfl_sync(0xffffffffu, v, src);
      for (int k = n - before; k > 0; --k) word &= word - 1;  // drop the lower set bits
      return (w0 + src) * 32 + __ffs(word) - 1;
    }
    n -= total;
  }
  return -1;
}

template <typename Count>
__global__ void __launch_bounds__(kMatchWarps * 32, 4)  // four CTAs per SM, as shared memory allows at g_max 150
match_kernel(const Count* __restrict__ pairs, const int64_t* __restrict__ pair_off,
             const int64_t* __restrict__ d_off, const int64_t* __restrict__ g_off, int single_d, int single_g,
             const int* __restrict__ pc, const double* __restrict__ pa,
             const int* __restrict__ gc, const double* __restrict__ ga, const uint8_t* __restrict__ crowd,
             const double* __restrict__ areas, int C, int g_max, FlagLayout flags, int* __restrict__ ranks,
             int64_t* __restrict__ counts, const int* __restrict__ gate, int per_warp,
             const u32* __restrict__ class_bits, int batch) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  if (gate && *reinterpret_cast<const volatile int*>(gate)) return;  // validation failed upstream
  // Image b covers detections [d_off[b], d_off[b+1]) and targets [g_off[b], g_off[b+1]);
  // its D x G intersections start at pair_off[b]. Without offsets: one image.
  // One warp per (image, class) at a time: CTA k of an image covers warps x per_warp classes, warp w
  // taking entries c_base + w, c_base + w + warps, ... of the image's class list. Without per-image
  // class bits the list is every class and the CTAs go image by image. With them it is the classes
  // present in the image (about a third of them in COCO-like batches), so the busy warps fill CTAs
  // instead of sharing them with warps that have nothing to do, and the CTAs go class block by class
  // block (block 0 of every image first) so that the CTAs left without classes come last.
  const int warps = blockDim.x >> 5;
  const int class_blocks = (C + warps * per_warp - 1) / (warps * per_warp);
  const int b = class_bits ? (int)(blockIdx.x % (unsigned)batch) : (int)(blockIdx.x / class_blocks);
  const int block = class_bits ? (int)(blockIdx.x / (unsigned)batch) : (int)(blockIdx.x % class_blocks);
  const int c_base = block * warps * per_warp + (threadIdx.x >> 5);
  const int64_t d0 = d_off ? d_off[b] : 0, g0 = g_off ? g_off[b] : 0;
  const int D = d_off ? (int)(d_off[b + 1] - d0) : single_d;
  const int G = g_off ? (int)(g_off[b + 1] - g0) : single_g;
  const Count* P = pairs + (pair_off ? pair_off[b] : 0);
  pc += d0; pa += d0; ranks += d0;
  gc += g0; ga += g0; crowd += g0; areas += g0;
  int8_t* fbase = flags.base + d0 * flags.det_stride;
  const int bit_words = (C + 31) / 32;
  auto one_class = [&](const int c) {
  // Classes with neither detections nor targets in this image (per-image bits, when given) have no work.
  if (class_bits && !((class_bits[(int64_t)b * bit_words + (c >> 5)] >> (c & 31)) & 1u)) return;
  const int words = (g_max + 31) / 32;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned char* mine = smem_raw + (size_t)warp * match_warp_bytes(g_max);
  // IoUs as IEEE bit patterns: for non-negative doubles the int64 order is the
  // numeric order, so the chains compare integers only.
  long long* iou_s = reinterpret_cast<long long*>(mine);      // IoU table of the class, or the current row
  int* dets = reinterpret_cast<int*>(iou_s + iou_entries(g_max));
  int* gts = dets + kMaxDets;
  u32* used = reinterpret_cast<u32*>(gts + g_max);
  u32* crowd_m = used + kChains * words;  // bit j of word w: target 32 w + j is a crowd
  u32* ignore_m = crowd_m + words;        // [4][words]: ignored in area range a
  u32* reach_m = ignore_m + 4 * words;    // [10][words]: IoU with the current detection reaches threshold t
  unsigned char* crowd_s = reinterpret_cast<unsigned char*>(reach_m + 10 * words);
  unsigned char* ignore_s = crowd_s + g_max;                   // bit a: target ignored in area range a
  unsigned char* range_s = ignore_s + g_max;                   // bit a: detection area inside range a
  const u32 below = (1u << lane) - 1;
  {
    // Every detection's rank and flags are written by exactly one warp: the
    // warp of its class (beyond the 100-detection cap: rank 0, all flags -1),
    // or warp 0 of class block 0 for classes outside [0, C).
    // The class lists are read kScanBlocks blocks of 32 at a time, every lane's loads issued before the
    // ballots use them (one L2 round trip per group instead of one per block).
    constexpr int kScanBlocks = 4;
    int nd = 0;
    for (int group = 0; group < D; group += 32 * kScanBlocks) {
      int dcs[kScanBlocks];
#pragma unroll
      for (int u = 0; u < kScanBlocks; ++u) {
        const int d = group + 32 * u + lane;
        dcs[u] = d < D ? pc[d] : -1;
      }
#pragma unroll
      for (int u = 0; u < kScanBlocks; ++u) {
        const int base = group + 32 * u;
        if (base >= D) break;  // whole warp
        const int d = base + lane;
        const int dc = dcs[u];
        const bool sel = d < D && dc == c;
        const u32 ballot = __ballot_sync(0xffffffffu, sel);
        const bool stray = c == 0 && d < D && (dc < 0 || dc >= C);
        bool unranked = stray;
        if (sel) {
          const int rank = nd + __popc(ballot & below);
          if (rank < kMaxDets) {
            dets[rank] = d;
            ranks[d] = rank + 1;
          } else {
            unranked = true;
          }
        }
        if (unranked) {
          ranks[d] = 0;
          for (int k = 0; k < kChains; ++k) fbase[k * flags.chain_stride + (int64_t)d * flags.det_stride] = -1;
        }
        nd += __popc(ballot);
      }
    }
    nd = min(nd, kMaxDets);
    int ng = 0;
    int positive[4] = {0, 0, 0, 0};
    int gcs[kScanBlocks];
    for (int base = 0; base < G; base += 32) {
      const int u = (base >> 5) % kScanBlocks;
      if (u == 0) {
#pragma unroll
        for (int v = 0; v < kScanBlocks; ++v) {
          const int g = base + 32 * v + lane;
          gcs[v] = g < G ? gc[g] : -1;
        }
      }
      const int g = base + lane;
      int gcu = gcs[0];
#pragma unroll
      for (int v = 1; v < kScanBlocks; ++v) gcu = u == v ? gcs[v] : gcu;
      const bool sel = g < G && gcu == c;
      const u32 ballot = __ballot_sync(0xffffffffu, sel);
      if (sel) gts[ng + __popc(ballot & below)] = g;
      ng += __popc(ballot);
      const bool eligible = sel && !crowd[g];
      const double area = eligible ? areas[g] : 0.0;
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        double lo, hi;
        area_range(a, lo, hi);
        positive[a] += __popc(__ballot_sync(0xffffffffu, eligible && area >= lo && area <= hi));
      }
    }
    if (lane == 0 && ng)
      for (int a = 0; a < 4; ++a)
        if (positive[a]) atomicAdd(reinterpret_cast<u64*>(counts) + c * 4 + a, (u64)positive[a]);
    if (nd == 0) return;
    for (int k = lane; k < kChains * words; k += 32) used[k] = 0;
    // Per-target and per-detection range tests and every (detection, target)
    // IoU are evaluated once, lane-parallel (FP64 is slow on this part).
    // Targets' crowd / ignore bits and detections' area-range bits in one pass (their loads overlap).
    __syncwarp();  // gts / dets entries written by other lanes
    for (int j = lane; j < max(ng, nd); j += 32) {
      const int g = j < ng ? gts[j] : 0;
      const bool cr = j < ng && crowd[g] != 0;
      const double area = j < ng ? areas[g] : 0.0;
      const double dpa = j < nd ? pa[dets[j]] : 0.0;
      unsigned char ignore_bits = 0, range_bits = 0;
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        double lo, hi;
        area_range(a, lo, hi);
        ignore_bits |= (unsigned char)((cr || area < lo || area > hi) << a);
        range_bits |= (unsigned char)((lo <= dpa && dpa <= hi) << a);
      }
      if (j < ng) {
        crowd_s[j] = cr;
        ignore_s[j] = ignore_bits;
      }
      if (j < nd) range_s[j] = range_bits;
    }
    // Every (detection, target) IoU is computed once, lane-parallel, and read by all 40 chains
    // (FP64 division runs at 1/64 of the FP32 rate here): the whole table up front when it fits
    // kIouCap entries, else one detection's row at a time in score order.
    const bool staged = nd * ng <= kIouCap;
    // Entries e0 .. e0 + count of the row-major nd x ng table; each lane issues the loads of kFillLoads
    // entries before using them.
    constexpr int kFillLoads = 4;
    auto fill = [&](int e0, int count) {
      const int end = e0 + count;
      for (int e = e0 + lane; e < end; e += 32 * kFillLoads) {
        double inter[kFillLoads], pa_d[kFillLoads], ga_g[kFillLoads];
#pragma unroll
        for (int u = 0; u < kFillLoads; ++u) {
          const int eu = e + 32 * u;
          inter[u] = pa_d[u] = ga_g[u] = 0.0;
          if (eu < end) {
            const int i = eu / ng, j = eu - i * ng;
            const int d = dets[i], g = gts[j];
            inter[u] = (double)P[(int64_t)d * G + g];
            pa_d[u] = pa[d];
            ga_g[u] = ga[g];
          }
        }
#pragma unroll
        for (int u = 0; u < kFillLoads; ++u) {
          const int eu = e + 32 * u;
          if (eu >= end) break;
          const int j = eu - (eu / ng) * ng;
          const double uni = crowd_s[j] ? pa_d[u] : (pa_d[u] + ga_g[u]) - inter[u];
          iou_s[staged ? eu : j] = __double_as_longlong(inter[u] / fmax(uni, 1.0));
        }
      }
    };
    __syncwarp();  // crowd_s entries written by other lanes
    if (staged) fill(0, nd * ng);
    // Target masks of the class, one bit per target in metadata order.
    const int wc = (ng + 31) / 32;
    for (int w = 0; w < wc; ++w) {
      const int j = 32 * w + lane;
      const bool in = j < ng;
      const u32 crowd_bits = __ballot_sync(0xffffffffu, in && crowd_s[j]);
      if (lane == 0) crowd_m[w] = crowd_bits;
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        const u32 bits = __ballot_sync(0xffffffffu, in && ((ignore_s[j] >> a) & 1));
        if (lane == 0) ignore_m[a * words + w] = bits;
      }
    }
    __syncwarp();
    for (int i = 0; i < nd; ++i) {
      const int d = dets[i];
      if (!staged) {
        fill(i * ng, ng);
        __syncwarp();
      }
      const long long* row = staged ? iou_s + i * ng : iou_s;
      // Targets whose IoU with this detection reaches each threshold: a chain then visits only its
      // candidates (usually one or two) instead of every target of the class.
      for (int w = 0; w < wc; ++w) {
        const int j = 32 * w + lane;
        const long long iou = j < ng ? row[j] : -1ll;
#pragma unroll
        for (int t = 0; t < 10; ++t) {
          const u32 bits = __ballot_sync(0xffffffffu, iou >= __double_as_longlong(iou_threshold(t)));
          if (lane == 0) reach_m[t * words + w] = bits;
        }
      }
      __syncwarp();
      for (int chain = lane; chain < kChains; chain += 32) {
        const int a = chain / 10, t = chain % 10;
        const long long thr = __double_as_longlong(iou_threshold(t));
        u32* taken = used + chain * words;
        int best = -1;
        bool best_ignored = false;
        long long best_iou = thr;
        // Eligible ground truth first, then ignored, each in metadata order (a taken target is skipped
        // unless it is a crowd); a later entry with an equal IoU replaces the earlier one.
        for (int pass = 0; pass < 2 && best < 0; ++pass) {
          for (int w = 0; w < wc; ++w) {
            const u32 ig = ignore_m[a * words + w];
            u32 m = reach_m[t * words + w] & ~(taken[w] & ~crowd_m[w]) & (pass ? ig : ~ig);
            while (m) {
              const int j = 32 * w + __ffs(m) - 1;
              m &= m - 1;
              const long long iou = row[j];
              if (iou >= best_iou) {
                best = j;
                best_iou = iou;
                best_ignored = pass == 1;
              }
            }
          }
        }
        int8_t flag = -1;
        if (best >= 0) {
          taken[best >> 5] |= 1u << (best & 31);
          flag = best_ignored ? -1 : 1;
        } else if ((range_s[i] >> a) & 1) {
          flag = 0;
        }
        fbase[chain * flags.chain_stride + (int64_t)d * flags.det_stride] = flag;
      }
      __syncwarp();  // the threshold masks (and an unstaged row) are rewritten for the next detection
    }
  }
  };
  for (int k = 0; k < per_warp; ++k) {
    const int entry = c_base + k * warps;
    const int c = class_bits ? nth_present_class(class_bits + (int64_t)b * bit_words, bit_words, entry,
                                                 threadIdx.x & 31)
                             : entry;
    if (c < 0 || c >= C) break;  // whole warp: the list is exhausted
    one_class(c);
    __syncwarp();  // the warp's shared scratch is reused by its next class
  }
}

// ---- precision / recall accumulation -------------------------------------

constexpr int kAccThreads = 256;
constexpr int kSortCap = 1024;  // records of one class sorted and staged in shared memory, at most
constexpr int kAccParts = 2;    // CTAs sharing a class's chains at that cap (two fit on an SM)
constexpr int kSmallCap = 512;  // classes up to this many records: a smaller stage, more CTAs per class
constexpr int kSmallParts = 4;  // (256 records per class, 256 images: 0.096 ms against 0.114 at one cap)

__global__ void class_histogram_kernel(const int* __restrict__ classes, int64_t n, int C, int* __restrict__ hist) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int c = classes[i];
    if (c >= 0 && c < C) atomicAdd(hist + c, 1);
  }
}

// Exclusive scan of the class histogram into `cursor` (one CTA): cursor[c] is
// where class c's record indices start in the per-class list.
__global__ void __launch_bounds__(1024) class_offsets_kernel(const int* __restrict__ hist, int C, int* cursor) {
  __shared__ int s_warp[32];
  const int per = (C + blockDim.x - 1) / blockDim.x;
  const int c0 = min(C, (int)threadIdx.x * per), c1 = min(C, c0 + per);
  int local = 0;
  for (int c = c0; c < c1; ++c) local += hist[c];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int inclusive = local;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, inclusive, o);
    if (lane >= o) inclusive += v;
  }
  if (lane == 31) s_warp[warp] = inclusive;
  __syncthreads();
  if (warp == 0) {
    int w = lane < (int)(blockDim.x >> 5) ? s_warp[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += v;
    }
    s_warp[lane] = w;  // inclusive over warps
  }
  __syncthreads();
  int running = inclusive - local + (warp ? s_warp[warp - 1] : 0);
  for (int c = c0; c < c1; ++c) {
    cursor[c] = running;
    running += hist[c];
  }
}

// Record indices grouped by class (order inside a class is arbitrary: the
// accumulation sorts each class by score, then record index).
__global__ void class_scatter_kernel(const int* __restrict__ classes, int64_t n, int C, int* cursor,
                                     int* __restrict__ list) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int c = classes[i];
    if (c >= 0 && c < C) list[atomicAdd(cursor + c, 1)] = (int)i;
  }
}

// Sort key of a score: an unsigned integer that orders like the score descending (-0.0 taken as 0.0, so
// equal scores give equal keys), compared with integers instead of FP64 (GB300's FP64 pipe runs at 1/64
// of the FP32 rate). Ties sort by record index, which makes the sort stable.
__device__ __forceinline__ unsigned long long score_key(double score) {
  unsigned long long b = (unsigned long long)__double_as_longlong(score == 0.0 ? 0.0 : score);
  b = (b >> 63) ? ~b : (b | 0x8000000000000000ull);  // ascending in the score
  return ~b;                                           // descending
}

__device__ __forceinline__ bool before(unsigned long long ka, int ia, unsigned long long kb, int ib) {
  return ka < kb || (ka == kb && ia < ib);
}

// Bitonic sort of n <= cap (key, index) pairs, n padded to a power of two with
// sentinels that sort last. `global` arrays need a fence before each barrier.
template <bool kGlobal>
__device__ void bitonic_sort(unsigned long long* key, int* idx, int n, int padded) {
  for (int i = n + threadIdx.x; i < padded; i += blockDim.x) {
    key[i] = ~0ull;
    idx[i] = INT_MAX;
  }
  __syncthreads();
  for (int size = 2; size <= padded; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int i = threadIdx.x; i < padded; i += blockDim.x) {
        const int j = i ^ stride;
        if (j > i) {
          const bool ascending = (i & size) == 0;
          const unsigned long long ki = key[i], kj = key[j];
          const int ii = idx[i], ij = idx[j];
          const bool swap = ascending ? before(kj, ij, ki, ii) : before(ki, ii, kj, ij);
          if (swap) { key[i] = kj; key[j] = ki; idx[i] = ij; idx[j] = ii; }
        }
      }
      if constexpr (kGlobal) __threadfence_block();
      __syncthreads();
    }
  }
}

// One CTA per class. `scores` == nullptr means the records are already in
// global descending-score order. Records: classes[n], ranks[n] and flags at
// flags[chain * chain_stride + record * det_stride]. Classes with more than
// kSortCap records use per-class workspace regions instead of shared memory.
//
// Each of the 120 chains (threshold, area, maxDets) is handled by one warp at a
// time. Prefix counts of true and false positives over the score-ordered
// records come from ballots; the j-th true positive's cumulative false positives
// are kept per j. The precision envelope of the reference (the running maximum
// of precision from the end, instance.py:321) is a suffix maximum over j, taken
// with a warp scan; recall threshold r is first reached at the true positive
// j = tp_min[r], so precision[r] is the envelope at that j (instance.py:322-329).
// Runs of thresholds with the same envelope pair become segments, converted to
// FP64 once each with every lane converting a different segment. chain_stats
// [c][chain] receives the sum of the chain's 101 precision values and its recall
// (-1 when the class has no positives) for the summaries.
template <int kCap, int kParts>
__global__ void __launch_bounds__(kAccThreads)
accumulate_kernel(const int* __restrict__ list, const int* __restrict__ cursor, const int* __restrict__ ranks,
                  const int8_t* __restrict__ flags, int64_t chain_stride, int64_t det_stride,
                  const double* __restrict__ scores, const int64_t* __restrict__ positives,
                  const int* __restrict__ hist, unsigned long long* __restrict__ ws_key, int* __restrict__ ws_idx,
                  int C, long long* __restrict__ seg_ws, int* __restrict__ env_ws, double* __restrict__ precision,
                  double* __restrict__ recall, double* __restrict__ chain_stats, int above) {
  // The bitonic sort pads a class's records to the next power of two inside the kCap-entry stage.
  static_assert(kCap > 0 && (kCap & (kCap - 1)) == 0, "a stage cap must be a power of two");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int c = blockIdx.x / kParts, part = blockIdx.x % kParts;
  int64_t offset = 0;
  for (int k = 0; k < c; ++k) {
    const int h = hist[k];
    offset += h > kSortCap ? (int64_t)1 << (32 - __clz(h - 1)) : 0;
  }
  const int count = hist[c];
  // Classes of up to kCap records (more than `above`) are this launch's: the other launch takes the rest.
  if (count <= above || (kCap < kSortCap && count > kCap)) return;
  const bool staged = count <= kCap;
  // A staged class's chains are shared by kParts CTAs (each sorts and stages the class itself); a class
  // sorted in the workspace has one CTA, since the sort works in place there.
  const int parts = staged ? kParts : 1;
  if (part >= parts) return;
  int padded = 1;
  while (padded < max(count, 1)) padded <<= 1;
  unsigned long long* key = staged ? reinterpret_cast<unsigned long long*>(smem_raw) : ws_key + offset;
  int* idx = staged ? reinterpret_cast<int*>(smem_raw + sizeof(unsigned long long) * kCap) : ws_idx + offset;
  int* st_rank = reinterpret_cast<int*>(smem_raw + (sizeof(unsigned long long) + sizeof(int)) * kCap);
  int8_t* st_flags = reinterpret_cast<int8_t*>(st_rank + kCap);
  unsigned char* seg_lo = reinterpret_cast<unsigned char*>(st_flags + kChains * kCap);  // [120][101]
  // Per warp: cumulative false positives at the j-th true positive, then the envelope pair at j.
  unsigned short* env_s = reinterpret_cast<unsigned short*>(seg_lo + 120 * 101);  // [warps][2][kCap + 1]
  __shared__ int s_nseg[120], s_seg_off[121], s_hi[120];
  __shared__ double s_recall[120];
  for (int ch = threadIdx.x; ch < 120; ch += blockDim.x) s_nseg[ch] = 0;  // chains of the other parts stay empty
  // This class's record indices (from the per-class list), then sorted by (score desc, index asc); without
  // scores every key is equal and the sort restores record order.
  const int begin = cursor[c] - count;  // cursor[c] ends one past the class's segment after the scatter
  for (int k = threadIdx.x; k < count; k += blockDim.x) {
    const int i = list[begin + k];
    idx[k] = i;
    key[k] = score_key(scores ? scores[i] : 0.0);
  }
  __syncthreads();
  if (count > 1) {
    if (staged) bitonic_sort<false>(key, idx, count, padded);
    else bitonic_sort<true>(key, idx, count, padded);
  }
  __syncthreads();
  // Recall thresholds per area: tp_min[a][r] = the smallest true-positive count whose recall
  // fl(tp / npos) reaches fl(r * 0.01), found with a few exact FP64 checks around the estimate, so the
  // walk below compares integers (recall is monotone in tp).
  __shared__ int s_tpmin[4][101];
  for (int e = threadIdx.x; e < 4 * 101; e += blockDim.x) {
    const int a = e / 101, r = e % 101;
    const int64_t np = positives[c * 4 + a];
    int64_t t = 0;
    if (np > 0) {
      const double thr = (double)r * 0.01, den = (double)np;
      t = (int64_t)ceil(thr * den);
      t = t < 0 ? 0 : (t > np ? np : t);
      while (t > 0 && (double)(t - 1) / den >= thr) --t;
      while (t <= np && (double)t / den < thr) ++t;
    }
    s_tpmin[a][r] = (int)t;
  }
  if (staged) {  // ranks and the 40 flags of every record, in walk order
    for (int k = threadIdx.x; k < count; k += blockDim.x) st_rank[k] = ranks[idx[k]];
    if (chain_stride == 1 && det_stride == kChains && reinterpret_cast<uintptr_t>(flags) % 8 == 0) {
      // Record-major flags (the record store): one thread copies a record's 40 bytes as five 8-byte words.
      for (int k = threadIdx.x; k < count; k += blockDim.x) {
        const uint2* src = reinterpret_cast<const uint2*>(flags + (int64_t)idx[k] * kChains);
        uint2* dst = reinterpret_cast<uint2*>(st_flags + k * kChains);
        uint2 w[kChains / 8];
#pragma unroll
        for (int j = 0; j < kChains / 8; ++j) w[j] = src[j];
#pragma unroll
        for (int j = 0; j < kChains / 8; ++j) dst[j] = w[j];
      }
    } else {
      for (int e = threadIdx.x; e < count * kChains; e += blockDim.x) {
        const int k = e / kChains, ch = e % kChains;
        st_flags[e] = flags[ch * chain_stride + (int64_t)idx[k] * det_stride];
      }
    }
  }
  __syncthreads();
  // Phase A (integers only): one warp per chain builds the chain's envelope segments. Phase B: every
  // segment's FP64 value, the segments spread over all threads. Phase C: one warp per chain writes the
  // 101 precision values and sums them.
  long long* segs = seg_ws + (int64_t)c * 120 * 101;  // [chain][segment]: packed (tp, fp), then its value
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, warps = blockDim.x >> 5;
  const unsigned below = (1u << lane) - 1u;
  const int64_t prec_step = (int64_t)C * 12;  // distance between consecutive recall thresholds r
  // Envelope arrays of this warp: 16-bit in shared memory when the class is staged, else 32-bit in the
  // workspace (each class owns 2 * warps * (count + 1) ints there).
  unsigned short* fp16 = env_s + (int64_t)warp * 2 * (kCap + 1);
  unsigned short* t16 = fp16 + (kCap + 1);
  int* fp32 = env_ws + 2 * (int64_t)warps * ((int64_t)begin + c) + (int64_t)warp * 2 * (count + 1);
  int* t32 = fp32 + (count + 1);
  auto load_fp = [&](int j) -> unsigned { return staged ? fp16[j] : (unsigned)fp32[j]; };
  auto store_fp = [&](int j, unsigned v) { if (staged) fp16[j] = (unsigned short)v; else fp32[j] = (int)v; };
  auto load_t = [&](int j) -> unsigned { return staged ? t16[j] : (unsigned)t32[j]; };
  auto store_t = [&](int j, unsigned v) { if (staged) t16[j] = (unsigned short)v; else t32[j] = (int)v; };
  // Envelope order: (ct, cf) beats (bt, bf) when its precision ct / (ct + cf) is larger, or equal with
  // the incumbent at tp + fp = 1 (value 1 / (1 + eps) < 1.0) and the candidate not; (0, *) never wins.
  auto beats = [](unsigned ct, unsigned cf, unsigned bt, unsigned bf) {
    if (ct == 0) return false;
    if (bt == 0) return true;
    const int64_t lhs = (int64_t)ct * ((int64_t)bt + bf), rhs = (int64_t)bt * ((int64_t)ct + cf);
    return lhs > rhs || (lhs == rhs && bt + bf == 1 && ct + cf >= 2);
  };
  for (int ch = part + parts * warp; ch < 120; ch += parts * warps) {
    const int m = ch % 3, a = (ch / 3) % 4, t = ch / 12;
    const int64_t out_r = ((int64_t)t * C + c) * 4 + a;
    const int64_t npos = positives[c * 4 + a];
    double* prec = precision + ((((int64_t)t * 101) * C + c) * 4 + a) * 3 + m;
    double* stats = chain_stats ? chain_stats + ((int64_t)c * 120 + ch) * 2 : nullptr;
    int nseg = 0, hi = 0;
    if (!npos) {
      for (int r = lane; r <= 100; r += 32) prec[r * prec_step] = -1.0;
      if (lane == 0) {
        recall[out_r * 3 + m] = -1.0;
        if (stats) { stats[0] = -1.0; stats[1] = -1.0; }
      }
    } else {
      const int limit = m == 0 ? 1 : (m == 1 ? 10 : 100);
      const int chain = a * 10 + t;
      // Prefix counts over the records within maxDets: the j-th true positive's cumulative false
      // positives (those before it) go to fp[j].
      unsigned tp = 0, fp = 0, selected = 0;
      for (int base = 0; base < count; base += 32) {
        const int k = base + lane;
        int f = -1;
        bool sel = false;
        if (k < count) {
          const int rank = staged ? st_rank[k] : ranks[idx[k]];
          sel = rank >= 1 && rank <= limit;
          if (sel) f = staged ? st_flags[k * kChains + chain] : flags[chain * chain_stride + (int64_t)idx[k] * det_stride];
        }
        const unsigned bt = __ballot_sync(0xffffffffu, f == 1), bf = __ballot_sync(0xffffffffu, f == 0);
        const unsigned bs = __ballot_sync(0xffffffffu, sel);
        if (f == 1) store_fp(tp + __popc(bt & below) + 1, fp + __popc(bf & below));
        tp += __popc(bt);
        fp += __popc(bf);
        selected += __popc(bs);
      }
      if (!selected) {  // no detection within maxDets: zero curve (instance.py:315-318)
        for (int r = lane; r <= 100; r += 32) prec[r * prec_step] = 0.0;
        if (lane == 0) {
          recall[out_r * 3 + m] = 0.0;
          if (stats) { stats[0] = 0.0; stats[1] = 0.0; }
        }
      } else {
        if (lane == 0) s_recall[ch] = recall[out_r * 3 + m] = (double)tp / (double)npos;
        const int* tp_min = s_tpmin[a];
        int reached = 0;  // thresholds reached at the final recall (tp_min is nondecreasing in r)
        for (int r = lane; r <= 100; r += 32) reached += tp_min[r] <= (int)tp;
#pragma unroll
        for (int off = 16; off; off >>= 1) reached += __shfl_xor_sync(0xffffffffu, reached, off);
        hi = reached;
        for (int r = hi + lane; r <= 100; r += 32) prec[r * prec_step] = 0.0;  // thresholds never reached
        __syncwarp();
        // Suffix maximum of the envelope over j = tp, tp - 1, ..., 1 (lane 0 holds the largest j of a
        // chunk); the pair at j replaces fp[j] (its own entry, read first) and goes to t[j].
        unsigned ct = 0, cf = 0;  // the best pair of the chunks already scanned
        for (int top = (int)tp; top >= 1; top -= 32) {
          const int j = top - lane;
          unsigned vt = 0, vf = 0;
          if (j >= 1) { vt = (unsigned)j; vf = load_fp(j); }
#pragma unroll
          for (int off = 1; off < 32; off <<= 1) {
            const unsigned ot = __shfl_up_sync(0xffffffffu, vt, off), of = __shfl_up_sync(0xffffffffu, vf, off);
            if (lane >= off && beats(ot, of, vt, vf)) { vt = ot; vf = of; }
          }
          if (beats(ct, cf, vt, vf)) { vt = ct; vf = cf; }
          if (j >= 1) { store_t(j, vt); store_fp(j, vf); }
          ct = __shfl_sync(0xffffffffu, vt, 31);
          cf = __shfl_sync(0xffffffffu, vf, 31);
        }
        __syncwarp();
        // Threshold r < hi takes the envelope at j = tp_min[r] (thresholds reached with no true positive
        // take the envelope over all of them); runs of equal pairs are the chain's segments.
        unsigned char* lo_of = seg_lo + ch * 101;
        long long* pair_of = segs + ch * 101;
        int prev_t = -1, prev_f = -1;
        for (int r0 = 0; r0 < hi; r0 += 32) {
          const int r = r0 + lane;
          unsigned pt = 0, pf = 0;
          if (r < hi && tp > 0) {
            const int j = max(tp_min[r], 1);
            pt = load_t(j);
            pf = load_fp(j);
          }
          int lt = __shfl_up_sync(0xffffffffu, (int)pt, 1), lf = __shfl_up_sync(0xffffffffu, (int)pf, 1);
          if (lane == 0) { lt = prev_t; lf = prev_f; }
          const bool start = r < hi && ((int)pt != lt || (int)pf != lf);
          const unsigned starts = __ballot_sync(0xffffffffu, start);
          if (start) {
            const int sidx = nseg + __popc(starts & below);
            lo_of[sidx] = (unsigned char)r;
            pair_of[sidx] = (long long)(((unsigned long long)pt << 32) | pf);
          }
          nseg += __popc(starts);
          prev_t = __shfl_sync(0xffffffffu, (int)pt, 31);
          prev_f = __shfl_sync(0xffffffffu, (int)pf, 31);
        }
      }
    }
    if (lane == 0) {
      s_nseg[ch] = nseg;
      s_hi[ch] = hi;
    }
  }
  __syncthreads();
  if (threadIdx.x < 32) {  // segment offsets (exclusive scan over the 120 chains)
    int carry = 0;
    for (int base = 0; base < 120; base += 32) {
      const int ch = base + (int)threadIdx.x;
      const int v0 = ch < 120 ? s_nseg[ch] : 0;
      int v = v0;
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, v, off);
        if ((int)threadIdx.x >= off) v += u;
      }
      if (ch < 120) s_seg_off[ch] = carry + v - v0;
      carry += __shfl_sync(0xffffffffu, v, 31);
    }
    if (threadIdx.x == 0) s_seg_off[120] = carry;
  }
  __syncthreads();
  // Phase B: every segment's value, fl(tp / ((tp + fp) + eps)), the segments spread over all threads.
  const int total_segs = s_seg_off[120];
  for (int e = threadIdx.x; e < total_segs; e += blockDim.x) {
    int lo = 0, hi = 119;  // chain holding flat segment e
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (s_seg_off[mid] <= e) lo = mid; else hi = mid - 1;
    }
    long long* slot = segs + lo * 101 + (e - s_seg_off[lo]);
    const unsigned long long pair = (unsigned long long)*slot;
    const double bt = (double)(int64_t)(pair >> 32), bf = (double)(int64_t)(pair & 0xffffffffull);
    *slot = __double_as_longlong(bt / ((bt + bf) + DBL_EPSILON));
  }
  __syncthreads();
  // Phase C: each chain's precision values from its segments (segment s covers [lo_s, lo_{s+1}), the
  // last up to hi), and their sum for the summaries.
  for (int ch = part + parts * warp; ch < 120; ch += parts * warps) {
    const int nseg = s_nseg[ch];
    if (nseg == 0) continue;
    const int m = ch % 3, a = (ch / 3) % 4, t = ch / 12;
    double* prec = precision + ((((int64_t)t * 101) * C + c) * 4 + a) * 3 + m;
    const unsigned char* lo_of = seg_lo + ch * 101;
    const long long* val_of = segs + ch * 101;
    double psum = 0.0;
    for (int r = lane; r < s_hi[ch]; r += 32) {
      int lo = 0, hi = nseg - 1;  // the last segment starting at or before r
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (lo_of[mid] <= r) lo = mid; else hi = mid - 1;
      }
      const double v = __longlong_as_double(val_of[lo]);
      prec[r * prec_step] = v;
      psum += v;
    }
#pragma unroll
    for (int off = 16; off; off >>= 1) psum += __shfl_xor_sync(0xffffffffu, psum, off);
    if (lane == 0 && chain_stats) {
      double* stats = chain_stats + ((int64_t)c * 120 + ch) * 2;
      stats[0] = psum;
      stats[1] = s_recall[ch];
    }
  }
}

// The 12 summaries from per-chain statistics: CTA q reduces summary q over its
// (class, threshold) entries in a fixed order (thread-strided, each thread's
// loads issued together before any is used, then a butterfly per warp and the
// warps' partials in index order). One warp per summary walking the entries
// one dependent L2 load at a time took 26 us for 80 classes; the entries fit
// one load round per thread here.
constexpr int kSummarizeThreads = 256;
constexpr int kSummarizeLoads = 4;  // loads in flight per thread and round

__global__ void __launch_bounds__(kSummarizeThreads)
summarize_chains_kernel(const double* __restrict__ chain_stats, int C, double* __restrict__ out) {
  const int q = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // summary -> (uses precision sums?, area, maxDets index, single threshold or -1)
  const bool is_ap = q < 4 || q == 5 || q == 7;
  const int area = (q < 3 || q >= 9) ? 0 : (q <= 4 ? 1 : (q <= 6 ? 2 : 3));
  const int mi = q >= 9 ? q - 9 : 2;
  const int only_t = q == 1 ? 0 : (q == 2 ? 5 : -1);
  const int nt = only_t >= 0 ? 1 : 10;
  const int64_t n = (int64_t)nt * C;  // entry e: class e / nt, threshold e % nt (or only_t)
  const int field = is_ap ? 0 : 1;
  const long long weight = is_ap ? 101 : 1;
  double sum = 0.0;
  long long cnt = 0;
  for (int64_t e0 = tid; e0 < n; e0 += (int64_t)kSummarizeLoads * kSummarizeThreads) {
    double v[kSummarizeLoads];
#pragma unroll
    for (int j = 0; j < kSummarizeLoads; ++j) {
      const int64_t e = e0 + (int64_t)j * kSummarizeThreads;
      v[j] = -1.0;
      if (e < n) {
        const int64_t c = e / nt;
        const int t = only_t >= 0 ? only_t : (int)(e - c * nt);
        v[j] = chain_stats[(c * 120 + t * 12 + area * 3 + mi) * 2 + field];
      }
    }
#pragma unroll
    for (int j = 0; j < kSummarizeLoads; ++j) {
      if (v[j] >= 0.0) {
        sum += v[j];
        cnt += weight;
      }
    }
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    sum += __shfl_xor_sync(0xffffffffu, sum, o);
    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  }
  __shared__ double s_sum[kSummarizeThreads / 32];
  __shared__ long long s_cnt[kSummarizeThreads / 32];
  if (lane == 0) {
    s_sum[warp] = sum;
    s_cnt[warp] = cnt;
  }
  __syncthreads();
  if (tid == 0) {
    double total = 0.0;
    long long count = 0;
    for (int w = 0; w < kSummarizeThreads / 32; ++w) {
      total += s_sum[w];
      count += s_cnt[w];
    }
    out[q] = count ? total / (double)count : -1.0;
  }
}

// The 12 COCO summaries (instance.py:230-248): means of the entries >= 0.
__global__ void __launch_bounds__(256)
summarize_kernel(const double* __restrict__ precision, const double* __restrict__ recall, int C,
                 double* __restrict__ out) {
  // out: ap, ap50, ap75, ap_small, ar_small, ap_medium, ar_medium, ap_large, ar_large, ar1, ar10, ar100
  __shared__ double s_sum[256];
  __shared__ int s_cnt[256];
  {
    const int q = blockIdx.x;  // one CTA per summary
    double sum = 0.0;
    int cnt = 0;
    const bool is_precision = q < 3 || q == 3 || q == 5 || q == 7;
    if (is_precision) {
      const int area = q < 3 ? 0 : (q == 3 ? 1 : (q == 5 ? 2 : 3));
      const int t0 = q == 1 ? 0 : (q == 2 ? 5 : 0);
      const int t1 = q == 1 ? 1 : (q == 2 ? 6 : 10);
      const int64_t per_t = (int64_t)101 * C;
      const int64_t total = (t1 - t0) * per_t;
      for (int64_t e = threadIdx.x; e < total; e += blockDim.x) {
        const int64_t t = t0 + e / per_t, rc = e % per_t;  // rc = r * C + c
        const double v = precision[((t * 101 * C + rc) * 4 + area) * 3 + 2];
        if (v >= 0) { sum += v; ++cnt; }
      }
    } else {
      int area = 0, mi = 2;
      if (q == 4) area = 1;
      else if (q == 6) area = 2;
      else if (q == 8) area = 3;
      else mi = q - 9;  // ar1, ar10, ar100
      const int64_t total = (int64_t)10 * C;
      for (int64_t e = threadIdx.x; e < total; e += blockDim.x) {
        const double v = recall[(e * 4 + area) * 3 + mi];
        if (v >= 0) { sum += v; ++cnt; }
      }
    }
    s_sum[threadIdx.x] = sum;
    s_cnt[threadIdx.x] = cnt;
    __syncthreads();
    for (int s = 128; s; s >>= 1) {
      if ((int)threadIdx.x < s) {
        s_sum[threadIdx.x] += s_sum[threadIdx.x + s];
        s_cnt[threadIdx.x] += s_cnt[threadIdx.x + s];
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) out[q] = s_cnt[0] ? s_sum[0] / (double)s_cnt[0] : -1.0;
    __syncthreads();
  }
}

// ---- detection x target-slot histogram -----------------------------------

constexpr int kDetThreads = 512;
constexpr int kDetPixels = 16;                      // pixels per thread
constexpr int kDetChunk = kDetThreads * kDetPixels;  // pixels per CTA

__device__ __forceinline__ void load16(const uint8_t* p, int64_t x, int64_t end, int align, uint32_t w[4]) {
  if (align == 16 && x + 16 <= end) {
    const uint4 v = __ldg(reinterpret_cast<const uint4*>(p + x));
    w[0] = v.x; w[1] = v.y; w[2] = v.z; w[3] = v.w;
  } else if (align == 4 && x + 16 <= end) {
    const uint32_t* q = reinterpret_cast<const uint32_t*>(p + x);
    w[0] = __ldg(q); w[1] = __ldg(q + 1); w[2] = __ldg(q + 2); w[3] = __ldg(q + 3);
  } else {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      uint32_t v = 0;
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (x + 4 * k + j < end) v |= (uint32_t)(__ldg(p + x + 4 * k + j) != 0) << (8 * j);
      w[k] = v;
    }
  }
}

template <bool SMEM>
__global__ void __launch_bounds__(kDetThreads)
detection_histogram_kernel(const uint8_t* __restrict__ masks, int64_t pixels, int D, const int* __restrict__ target,
                           const int64_t* __restrict__ order, int S, int align, u64* __restrict__ pairs) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  u32* bins = reinterpret_cast<u32*>(smem_raw);
  const int bins_count = D * S;
  if (SMEM) {
    for (int k = threadIdx.x; k < bins_count; k += blockDim.x) bins[k] = 0;
    __syncthreads();
  }
  const int64_t x = (int64_t)blockIdx.x * kDetChunk + (int64_t)threadIdx.x * kDetPixels;
  int slot[kDetPixels];
  bool uniform = true;
#pragma unroll
  for (int j = 0; j < kDetPixels; ++j) {
    slot[j] = x + j < pixels ? target[x + j] : -1;
    if (slot[j] != slot[0]) uniform = false;
  }
  const bool valid0 = slot[0] >= 0 && slot[0] < S;
  for (int d = 0; d < D; ++d) {
    const uint8_t* mask = masks + order[d] * pixels;
    uint32_t w[4] = {0, 0, 0, 0};
    if (x < pixels) load16(mask, x, pixels, align, w);
    const bool any = (w[0] | w[1] | w[2] | w[3]) != 0;
    if (!__ballot_sync(0xffffffffu, any)) continue;
    // Lanes with one valid slot over their 16 pixels combine across the warp.
    const bool simple = any && uniform && valid0;
    const u32 count = simple ? (u32)(__popc(w[0]) + __popc(w[1]) + __popc(w[2]) + __popc(w[3])) : 0u;
    const u32 key = simple ? (u32)(d * S + slot[0]) : 0xffffffffu;
    const u32 peers = __match_any_sync(0xffffffffu, key);
    const u32 total = __reduce_add_sync(peers, count);
    if (simple && (threadIdx.x & 31) == (u32)(__ffs(peers) - 1)) {
      if (SMEM) atomicAdd(bins + key, total);
      else atomicAdd(pairs + key, (u64)total);
    }
    if (any && !simple) {
#pragma unroll
      for (int j = 0; j < kDetPixels; ++j) {
        const bool on = (w[j >> 2] >> (8 * (j & 3))) & 0xff;
        const int s = slot[j];
        if (on && s >= 0 && s < S) {
          if (SMEM) atomicAdd(bins + d * S + s, 1u);
          else atomicAdd(pairs + (int64_t)d * S + s, 1ull);
        }
      }
    }
  }
  if (SMEM) {
    __syncthreads();
    for (int k = threadIdx.x; k < bins_count; k += blockDim.x) {
      const u32 v = bins[k];
      if (v) atomicAdd(pairs + k, (u64)v);
    }
  }
}

// ---- mask x mask overlaps (bit-packed, sparse-aware) -----------------------

constexpr int kOvThreads = 256;
constexpr int kOvWords = 128;  // 32-bit words of packed pixels per CTA (4096 pixels)

// Pack 4 bytes holding 0/1 into 4 bits (any consistent bit order works for AND+popc).
__device__ __forceinline__ uint32_t pack4(uint32_t w) { return ((w & 0x01010101u) * 0x08040201u) >> 24 & 0xfu; }

__global__ void __launch_bounds__(kOvThreads)
mask_overlap_kernel(const uint8_t* __restrict__ pm, int D, const uint8_t* __restrict__ gm, int G, int64_t pixels,
                    int align, const int* __restrict__ pc, const int* __restrict__ gc, u64* __restrict__ inter) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int rows = D + G;
  uint32_t* bits = reinterpret_cast<uint32_t*>(smem_raw);            // rows x kOvWords
  int2* range = reinterpret_cast<int2*>(bits + (int64_t)rows * kOvWords);  // first/last nonzero word
  const int64_t x0 = (int64_t)blockIdx.x * kOvWords * 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // One warp packs one mask row of the chunk at a time: lane k packs word k + 32 i.
  for (int r = warp; r < rows; r += kOvThreads / 32) {
    const uint8_t* row = r < D ? pm + (int64_t)r * pixels : gm + (int64_t)(r - D) * pixels;
    int first = kOvWords, last = -1;
    for (int k = lane; k < kOvWords; k += 32) {
      const int64_t x = x0 + (int64_t)k * 32;
      uint32_t word = 0;
      if (x < pixels) {
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          uint32_t w[4];
          load16(row, x + 16 * q, pixels, align, w);
#pragma unroll
          for (int j = 0; j < 4; ++j) word |= pack4(w[j]) << (16 * q + 4 * j);
        }
      }
      bits[(int64_t)r * kOvWords + k] = word;
      if (word) { first = min(first, k); last = max(last, k); }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      first = min(first, __shfl_xor_sync(0xffffffffu, first, o));
      last = max(last, __shfl_xor_sync(0xffffffffu, last, o));
    }
    if (lane == 0) range[r] = make_int2(first, last);
  }
  __syncthreads();
  for (int pair = threadIdx.x; pair < D * G; pair += blockDim.x) {
    const int d = pair / G, g = pair % G;
    if (pc[d] != gc[g]) continue;
    const int2 rd = range[d], rg = range[D + g];
    const int lo = max(rd.x, rg.x), hi = min(rd.y, rg.y);
    if (lo > hi) continue;
    const uint32_t* a = bits + (int64_t)d * kOvWords;
    const uint32_t* b = bits + (int64_t)(D + g) * kOvWords;
    u32 count = 0;
    for (int k = lo; k <= hi; ++k) count += __popc(a[k] & b[k]);
    if (count) atomicAdd(inter + pair, (u64)count);
  }
}

int alignment_of(const void* p, int64_t pixels) {
  const uintptr_t a = reinterpret_cast<uintptr_t>(p);
  if ((a & 15) == 0 && pixels % 16 == 0) return 16;
  if ((a & 3) == 0 && pixels % 4 == 0) return 4;
  return 1;
}

}  // namespace

int launch_match(const void* pairs, bool pairs_u32, const int64_t* pair_off, const int64_t* d_off,
                 const int64_t* g_off, int single_d, int single_g, int64_t B, const int* pc, const double* pa,
                 const int* gc, const double* ga, const uint8_t* crowd, const double* areas, int C, int g_max,
                 int8_t* flags, int64_t chain_stride, int64_t det_stride, int* ranks, int64_t* counts,
                 cudaStream_t stream, const int* gate = nullptr, const uint32_t* class_bits = nullptr) {
  if (B == 0) return kOk;
  const size_t per_warp = match_warp_bytes(g_max);
  int warps = kMatchWarps;
  while (warps > 1 && per_warp * warps > 200 * 1024) warps >>= 1;
  if (per_warp * warps > 200 * 1024) {
    set_error("too many ground-truth slots per image for matching (G=%d)", g_max);
    return kUnsupported;
  }
  const size_t smem = per_warp * warps;
  const int classes_per_warp = 1;  // 2 or 4 measured the same on 256 images; one CTA per image 35 % slower
  const int64_t grid = B * ceil_div(C, warps * classes_per_warp);
  if (grid > INT_MAX) {
    set_error("too many (image, class) pairs for one matching launch (B=%lld, C=%d)", (long long)B, C);
    return kUnsupported;
  }
  FlagLayout layout{flags, chain_stride, det_stride};
  if (pairs_u32) {
    auto kernel = match_kernel<u32>;
    if (smem > 48 * 1024) PE_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kernel<<<(unsigned)grid, warps * 32, smem, stream>>>(static_cast<const u32*>(pairs), pair_off, d_off, g_off, single_d,
                                                      single_g, pc, pa, gc, ga, crowd, areas, C, g_max, layout, ranks,
                                                      counts, gate, classes_per_warp, class_bits, (int)B);
  } else {
    auto kernel = match_kernel<int64_t>;
    if (smem > 48 * 1024) PE_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kernel<<<(unsigned)grid, warps * 32, smem, stream>>>(static_cast<const int64_t*>(pairs), pair_off, d_off, g_off,
                                                      single_d, single_g, pc, pa, gc, ga, crowd, areas, C, g_max,
                                                      layout, ranks, counts, gate, classes_per_warp, class_bits, (int)B);
  }
  PE_LAUNCHED("match");
  count_launch();
  return kOk;
}

int launch_match_gated(const void* pairs, bool pairs_u32, const int64_t* pair_off, const int64_t* d_off,
                       const int64_t* g_off, int64_t B, const int* pc, const double* pa, const int* gc,
                       const double* ga, const uint8_t* crowd, const double* areas, int C, int g_max, int8_t* flags,
                       int64_t chain_stride, int64_t det_stride, int* ranks, int64_t* counts, const int* gate,
                       const uint32_t* class_bits, cudaStream_t stream) {
  return launch_match(pairs, pairs_u32, pair_off, d_off, g_off, 0, 0, B, pc, pa, gc, ga, crowd, areas, C, g_max,
                      flags, chain_stride, det_stride, ranks, counts, stream, gate, class_bits);
}

int64_t accumulate_workspace_bytes(int64_t n, int64_t C) {
  // Per-class overflow regions padded to powers of two (at most 2n entries), the per-class list (n), then
  // every class's envelope segments (120 chains x 101 of 8 bytes).
  return (int64_t)round_up(2 * n + 1, 64) * (int64_t)(sizeof(double) + sizeof(int)) +
         (int64_t)round_up(n + 1, 64) * (int64_t)sizeof(int) + C * 120 * 101 * (int64_t)sizeof(long long) +
         2 * (kAccThreads / 32) * (n + C) * (int64_t)sizeof(int);
}

int launch_accumulate(const int* classes, const int* ranks, const int8_t* flags, int64_t chain_stride,
                      int64_t det_stride, const double* scores, int64_t n, const int64_t* positives, int C,
                      void* workspace, int64_t workspace_bytes, int* hist, int* cursor, double* precision,
                      double* recall, double* chain_stats, double* summary, cudaStream_t stream) {
  const int64_t need = accumulate_workspace_bytes(n, C);
  if (workspace_bytes < need) {
    set_error("accumulate workspace too small: %lld < %lld bytes", (long long)workspace_bytes, (long long)need);
    return kWorkspaceTooSmall;
  }
  PE_CUDA(cudaMemsetAsync(hist, 0, sizeof(int) * C, stream));
  const int64_t entries = round_up(2 * n + 1, 64);
  auto* ws_key = static_cast<unsigned long long*>(workspace);
  int* ws_idx = reinterpret_cast<int*>(ws_key + entries);
  int* list = ws_idx + entries;
  long long* seg_ws = reinterpret_cast<long long*>(
      static_cast<char*>(workspace) + round_up(2 * n + 1, 64) * (int64_t)(sizeof(double) + sizeof(int)) +
      round_up(n + 1, 64) * (int64_t)sizeof(int));
  int* env_ws = reinterpret_cast<int*>(seg_ws + (int64_t)C * 120 * 101);
  if (n > 0) {
    const int64_t blocks = std::min<int64_t>(ceil_div(n, 256), (int64_t)sm_count() * 4);
    class_histogram_kernel<<<(unsigned)blocks, 256, 0, stream>>>(classes, n, C, hist);
    PE_LAUNCHED("class_histogram");
    class_offsets_kernel<<<1, 1024, 0, stream>>>(hist, C, cursor);
    PE_LAUNCHED("class_offsets");
    class_scatter_kernel<<<(unsigned)blocks, 256, 0, stream>>>(classes, n, C, cursor, list);
    PE_LAUNCHED("class_scatter");
    count_launch(3);
  }
  // Classes of up to kSmallCap records in a smaller stage with kSmallParts CTAs each; when some class
  // can be larger, a second launch takes those (staged up to kSortCap, else in the workspace).
  auto smem_for = [](int cap) {
    return (sizeof(unsigned long long) + 2 * sizeof(int) + kChains) * cap + 120 * 101 +
           sizeof(unsigned short) * 2 * (kAccThreads / 32) * (cap + 1);
  };
  auto small = accumulate_kernel<kSmallCap, kSmallParts>;
  PE_CUDA(cudaFuncSetAttribute(small, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_for(kSmallCap)));
  small<<<(unsigned)(C * kSmallParts), kAccThreads, smem_for(kSmallCap), stream>>>(
      list, cursor, ranks, flags, chain_stride, det_stride, scores, positives, hist, ws_key, ws_idx, C, seg_ws,
      env_ws, precision, recall, chain_stats, -1);
  PE_LAUNCHED("accumulate");
  count_launch();
  if (n > kSmallCap) {
    auto large = accumulate_kernel<kSortCap, kAccParts>;
    PE_CUDA(cudaFuncSetAttribute(large, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_for(kSortCap)));
    large<<<(unsigned)(C * kAccParts), kAccThreads, smem_for(kSortCap), stream>>>(
        list, cursor, ranks, flags, chain_stride, det_stride, scores, positives, hist, ws_key, ws_idx, C, seg_ws,
        env_ws, precision, recall, chain_stats, kSmallCap);
    PE_LAUNCHED("accumulate(large classes)");
    count_launch();
  }
  if (summary) {
    summarize_chains_kernel<<<12, kSummarizeThreads, 0, stream>>>(chain_stats, C, summary);
    PE_LAUNCHED("summarize_chains");
    count_launch();
  }
  return kOk;
}

int launch_summarize(const double* precision, const double* recall, int C, double* out, cudaStream_t stream) {
  summarize_kernel<<<12, 256, 0, stream>>>(precision, recall, C, out);
  PE_LAUNCHED("summarize");
  count_launch();
  return kOk;
}

}  // namespace pe

using namespace pe;

// Drop-in for `instance_histogram` (instance_kernel.cu:335-363): pairs[rank, s]
// counts the pixels of mask order[rank] on target slot s (all slots, including
// void and stuff, so row sums are full detection areas). pairs is zeroed here.
PE_API int pe_instance_histogram(const uint8_t* masks, int64_t D, int64_t pixels, const int32_t* target,
                                 const int64_t* order, int64_t S, int64_t* pairs, cudaStream_t stream) {
  PE_REQUIRE(D >= 0 && D < INT_MAX && pixels > 0 && S > 0 && S < INT_MAX && D * S < INT_MAX,
             "invalid shared ground-truth inputs");
  if (D == 0) return kOk;
  PE_CUDA(cudaMemsetAsync(pairs, 0, sizeof(int64_t) * D * S, stream));
  const int64_t bins = D * S;
  const bool smem = bins <= 48 * 1024;
  const size_t smem_bytes = smem ? sizeof(u32) * bins : 0;
  const int64_t grid = ceil_div(pixels, kDetChunk);
  const int align = alignment_of(masks, pixels);
  auto* out = reinterpret_cast<u64*>(pairs);
  if (smem) {
    if (smem_bytes > 48 * 1024)
      PE_CUDA(cudaFuncSetAttribute(detection_histogram_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)smem_bytes));
    detection_histogram_kernel<true><<<(unsigned)grid, kDetThreads, smem_bytes, stream>>>(
        masks, pixels, (int)D, target, order, (int)S, align, out);
  } else {
    detection_histogram_kernel<false><<<(unsigned)grid, kDetThreads, 0, stream>>>(masks, pixels, (int)D, target, order,
                                                                                  (int)S, align, out);
  }
  PE_LAUNCHED("detection_histogram");
  count_launch();
  return kOk;
}

// Drop-in for `instance_match_histogram` (instance_kernel.cu:365-381) and the
// matching half of `instance_update`: COCO greedy matching of D score-sorted
// detections against G targets from integer intersections pairs[D, G].
// Outputs flags [40, D] int8 (1 TP, 0 FP, -1 ignored / unmatched outside the
// area range), ranks [D] int32 (1..100 within class, 0 beyond), counts [C, 4]
// int64 positives (zeroed here).
PE_API int pe_instance_match(const int64_t* pairs, int64_t D, int64_t G, const int32_t* pc, const int32_t* gc,
                             const double* pa, const double* ga, const uint8_t* crowd, const double* areas,
                             int64_t C, int8_t* flags, int32_t* ranks, int64_t* counts, cudaStream_t stream) {
  PE_REQUIRE(D >= 0 && G >= 0 && D < INT_MAX && G < INT_MAX && D * G < INT_MAX, "too many instance pairs");
  PE_REQUIRE(C > 0 && C <= INT_MAX / 120, "invalid category count");
  PE_CUDA(cudaMemsetAsync(counts, 0, sizeof(int64_t) * C * 4, stream));
  if (D == 0 && G == 0) return kOk;
  return launch_match(pairs, false, nullptr, nullptr, nullptr, (int)D, (int)G, 1, pc, pa, gc, ga, crowd, areas,
                      (int)C, (int)std::max<int64_t>(G, 1), flags, D, 1, ranks, counts, stream);
}

// Intersections of every same-class (prediction, target) mask pair:
// inter[d, g] = |pm[d] & gm[g]| for pc[d] == gc[g], 0 otherwise. Part of
// `instance_update` (instance_kernel.cu:282-309). inter is zeroed here.
PE_API int pe_mask_overlap(const uint8_t* pm, int64_t D, const uint8_t* gm, int64_t G, int64_t pixels,
                           const int32_t* pc, const int32_t* gc, int64_t* inter, cudaStream_t stream) {
  PE_REQUIRE(D >= 0 && G >= 0 && pixels > 0 && D * G < INT_MAX, "invalid instance masks");
  if (D == 0 || G == 0) return kOk;
  PE_CUDA(cudaMemsetAsync(inter, 0, sizeof(int64_t) * D * G, stream));
  const size_t smem = (size_t)(D + G) * (kOvWords * sizeof(uint32_t) + sizeof(int2));
  PE_REQUIRE(smem <= 220 * 1024, "too many masks per image for the overlap kernel (D+G=%lld)", (long long)(D + G));
  const int align = std::min(alignment_of(pm, pixels), alignment_of(gm, pixels));
  if (smem > 48 * 1024)
    PE_CUDA(cudaFuncSetAttribute(mask_overlap_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t grid = ceil_div(pixels, (int64_t)kOvWords * 32);
  mask_overlap_kernel<<<(unsigned)grid, kOvThreads, smem, stream>>>(pm, (int)D, gm, (int)G, pixels, align, pc, gc,
                                                                     reinterpret_cast<u64*>(inter));
  PE_LAUNCHED("mask_overlap");
  count_launch();
  return kOk;
}

// Workspace bytes pe_instance_accumulate needs for n records and C classes.
PE_API int64_t pe_instance_accumulate_workspace(int64_t n, int64_t C) {
  return accumulate_workspace_bytes(n, C) + 2 * round_up(sizeof(int) * C, 64) + round_up(sizeof(double) * 240 * C, 64) +
         64;
}

// Drop-in for `instance_compute` (instance_kernel.cu:311-333) when scores is
// NULL (records already in global descending-score order, flags [40, n]), and
// the record-store accumulation of InstanceEvaluator.compute when scores is
// given (records in update order; sorted here by score, stably). Flags are
// read at flags[chain * chain_stride + record * det_stride].
// Outputs precision [10, 101, C, 4, 3] and recall [10, C, 4, 3] (fully written).
PE_API int pe_instance_accumulate(const int32_t* classes, const int32_t* ranks, const int8_t* flags,
                                  int64_t chain_stride, int64_t det_stride, const double* scores, int64_t n,
                                  const int64_t* positives, int64_t C, void* workspace, int64_t workspace_bytes,
                                  double* precision, double* recall, double* summary, cudaStream_t stream) {
  PE_REQUIRE(n >= 0 && n < INT_MAX && C > 0 && C <= INT_MAX / 120, "invalid instance state shapes");
  const int64_t ints = round_up(sizeof(int) * C, 64);
  const int64_t head = 2 * ints + round_up(sizeof(double) * 240 * C, 64);
  PE_REQUIRE(workspace_bytes >= head, "workspace too small");
  int* hist = static_cast<int*>(workspace);
  int* cursor = reinterpret_cast<int*>(static_cast<char*>(workspace) + ints);
  double* chain_stats = reinterpret_cast<double*>(static_cast<char*>(workspace) + 2 * ints);
  void* rest = static_cast<char*>(workspace) + head;
  return launch_accumulate(classes, ranks, flags, chain_stride, det_stride, scores, n, positives, (int)C, rest,
                           workspace_bytes - head, hist, cursor, precision, recall, chain_stats, summary, stream);
}

// The 12 AP/AR summaries (instance.py:230-248) into out[12]: ap, ap50, ap75,
// ap_small, ar_small, ap_medium, ar_medium, ap_large, ar_large, ar1, ar10, ar100.
PE_API int pe_instance_summarize(const double* precision, const double* recall, int64_t C, double* out,
                                 cudaStream_t stream) {
  PE_REQUIRE(C > 0 && C < INT_MAX / 120, "invalid category count");
  return launch_summarize(precision, recall, (int)C, out, stream);
}
