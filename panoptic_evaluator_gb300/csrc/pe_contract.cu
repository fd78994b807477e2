// Mask-vs-mask intersection counts for InstanceEvaluator on the tcgen05 tensor
// cores (sm_103a).
//
// inter[d][g] = sum_x pred[d][x] * gt[g][x] over 0/1 mask bytes is a dense
// (D x HW) by (HW x G) product, the contraction of the reference's
// pack_masks + overlap (instance_kernel.cu:10-39; CPU instance.py:255-264),
// which counts each pair with packed-word popcounts. Here each image is tiled
// into blocks of up to 127 detections x 63 targets (both in mask order). A CTA
// streams 128-pixel stages of those rows (one 128-byte swizzle atom of K)
// into shared memory in the canonical 128-byte-swizzled K-major layout. The
// mask bytes themselves are the operands: read as e4m3, 0x01 is the subnormal
// 2^-9 and 0x00 is zero, so each product is 2^-18 or 0. One thread issues
// tcgen05.mma kind::f8f6f4 (M = 128, N = 64, K = 32) into an fp32 accumulator
// in tensor memory. Row 127 of the A tile and row 63 of the B tile are
// constant ones, so the same product also yields the target areas (row 127)
// and the detection areas (column 63). The epilogue writes detection rows at
// their score rank (the inverse of pe_seg_sort's order).
//
// Exactness: each product is 0 or 2^-18 and an accumulator is read back
// (tcgen05.ld) at the end of every run of chunks of one block in a CTA, at
// most 2^22 pixels, so every fp32 partial sum is n * 2^-18 with n <= 2^22 <
// 2^24, held exactly whatever the accumulation order inside the tensor core;
// the epilogue scales by 2^18 to the integer count. They
// go to the global u32 / u64 counters with integer atomic adds, so results do
// not depend on how chunks are split across CTAs.
//
// Two ways into the operand stages:
//  - Images whose rows all start on 16-byte boundaries and that have a pair of
//    tensor maps (pe_contract_maps; descriptor flags bit 2) are loaded by TMA:
//    one 2-D tile load per operand and stage (127 x 128 and 63 x 128 bytes,
//    hardware 128-byte swizzle, zero fill past the last row and pixel) into an
//    eight-deep ring (the three operand slots and five slots carved from the
//    raw ring, idle once a CTA's staged blocks are done), issued by one thread.
//  - Other rows may start at any byte. Four copy warps stream, per stage and
//    row, the nine aligned 16-byte words covering the row's 128 bytes into a
//    five-deep raw ring with cp.async (completion on the stage's mbarrier);
//    words that start past the row end are not copied. Seven converter warps
//    take each row's bytes [o, o + 128) from the raw words (o = the row's start
//    offset mod 16; funnel shifts and selects; a lane turns five words into
//    four chunks, so shared-memory reads stay at 1.25x the bytes produced),
//    zero bytes past the row end and store them swizzled into a three-deep
//    operand ring.
// The host puts every TMA block after every staged block in chunk order, so a
// CTA switches kinds at most once (staged, then TMA). CTAs take contiguous
// chunk ranges of equal cost (rows x pixels).
//
// Roles per CTA (16 warps): warps 0-3 read the accumulator (TMEM lanes
// 32w..32w+31), warp 4 allocates TMEM and issues the MMAs, warps 5-8 copy,
// warps 9-15 convert (converter 0 also issues the TMA loads). Every mbarrier
// wait is bounded; a timeout sets bit 30 of *error (and bit 20 + the wait's
// site), every role leaves its loop, copies and TMA loads in flight land
// before the CTA exits, the MMA thread waits (bounded) for its MMAs to retire
// and TMEM is freed before the CTA exits.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cmath>
#include <type_traits>

#include "pe_common.cuh"
#include "pe_desc.cuh"

namespace pe {
namespace {

constexpr int kM = 128;                 // A rows: 127 detections + ones row
constexpr int kN = 64;                  // B rows: 63 targets + ones row
constexpr int kRowsA = kM - 1;
constexpr int kRowsB = kN - 1;
constexpr int kRows = kRowsA + kRowsB;  // mask rows of one block
constexpr int kAtom = 128;              // pixels of one stage: one 128-byte swizzle atom of K
constexpr int kMmaK = 32;               // K of one kind::f8f6f4 MMA (bytes)
constexpr int kInterval = 4096;         // pixels of one work chunk
constexpr int kSegmentChunks = 1024;    // chunks per accumulator read-back at most (2^22 pixels)
constexpr int kRawWords = kAtom / 16 + 1;  // aligned words covering 128 row bytes at any offset
constexpr int kRawRow = kRawWords * 16;
constexpr int kRawRing = 5;
constexpr int kRing = 3;
constexpr int kEpilogueWarps = 4;
constexpr int kMmaWarp = 4;
constexpr int kCopyWarps = 4;
constexpr int kConvertWarps = 7;
constexpr int kFirstCopyWarp = kMmaWarp + 1;
constexpr int kFirstConvertWarp = kFirstCopyWarp + kCopyWarps;
constexpr int kThreads = (kEpilogueWarps + 1 + kCopyWarps + kConvertWarps) * 32;
constexpr int kCopyRows = (kRows + kCopyWarps - 1) / kCopyWarps;        // rows per copy warp
constexpr int kCopyItems = (kCopyRows * kRawWords + 31) / 32;             // 16-byte copies per lane and stage
// A converter lane produces kConvertChunks adjacent 16-byte chunks of a row from kConvertChunks + 1 aligned
// raw words: shared-memory reads of 1.25x the output bytes, against 2x with one chunk per lane. The staged
// path is bound by shared-memory traffic, so this took it from 0.448 to 0.353 ms on 32 COCO-like images
// (two chunks per lane: 0.359).
constexpr int kConvertChunks = 4;
constexpr int kLanesPerRow = (kAtom / 16) / kConvertChunks;
constexpr int kConvertRowsPerWarp = 32 / kLanesPerRow;
constexpr int kConvertRowsPerRound = kConvertWarps * kConvertRowsPerWarp;
constexpr int kConvertRounds = (kRows + kConvertRowsPerRound - 1) / kConvertRowsPerRound;
constexpr int kTmemCols = 2 * kN;       // two accumulator buffers
constexpr int kTmaSlotBytes = (kM + kN) * kAtom;               // one TMA stage: A tile, then B tile
constexpr int kTmaExtra = 5;                                   // TMA slots carved from the raw ring
constexpr int kTmaRing = kRing + kTmaExtra;
constexpr uint32_t kTmaBytes = (uint32_t)(kRowsA + kRowsB) * kAtom;  // both tile loads of a stage
constexpr long long kWaitLimit = 4000000000ll;  // ~2 s at 2 GHz
constexpr int kTimeoutBit = 1 << 30;
constexpr int kOrderBit = 1 << 28;  // a CTA range has staged blocks after TMA blocks (the host orders them)
// Wait sites, recorded as bit (kSiteBit + site) beside kTimeoutBit when that wait times out.
enum : int { kSiteBit = 20, kAtAccEmpty = 0, kAtFull, kAtFullTma, kAtTmaSlot, kAtStageSlot, kAtAccFull, kAtRaw };
constexpr float kCountScale = 262144.0f;  // 2^18: one product of two mask bytes (e4m3 2^-9 each)

static_assert(kThreads == 512, "16 warps");
static_assert(kConvertRounds * kConvertRowsPerRound >= kRows, "converter rounds cover every row");
static_assert(kCopyItems <= 32, "copy items fit the live mask");
static_assert(kTmaExtra * kTmaSlotBytes <= kRawRing * kRows * kRawRow, "TMA slots fit the raw ring");
static_assert(kRowsA <= 4 * 32, "epilogue rows");

struct __align__(1024) ContractShared {
  uint8_t a[kRing][kM * kAtom];               // swizzled e4m3 operand tiles
  uint8_t b[kRing][kN * kAtom];
  uint8_t raw[kRawRing][kRows * kRawRow];     // aligned words of each row, in row order
  uint64_t full[kRing];  // staged operand stage: one arrival per converter warp
  uint64_t empty[kRing];
  uint64_t raw_full[kRawRing];
  uint64_t raw_empty[kRawRing];
  uint64_t tma_full[kTmaRing];  // TMA stage: one arrival carrying the stage's bytes
  uint64_t tma_empty[kTmaRing];
  uint64_t acc_full[2];
  uint64_t acc_empty[2];
  uint64_t done;
  int32_t rank[kEpilogueWarps][32];  // epilogue: score rank of each detection row of its block
  uint32_t tmem_base;
  int abort;
};
static_assert(sizeof(ContractShared) + 1024 <= 227 * 1024, "shared memory of one CTA");

// Block table row: image, first detection row, first target row, first chunk.
enum : int { kBlkImage = 0, kBlkM0, kBlkN0, kBlkChunk, kBlkFields };

// ---- tcgen05 / TMA / proxy helpers ------------------------------------------

__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t cols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(cols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t cols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mma_f8(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                       uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Arrive once on `bar` when every tcgen05 operation this thread issued so far has completed.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// 32 consecutive fp32 accumulator columns of this warp's 32 TMEM lanes (one row per thread).
__device__ __forceinline__ void tmem_load32(uint32_t taddr, uint32_t (&v)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
        "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]),
        "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
        "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr)
      : "memory");
}
__device__ __forceinline__ void tmem_wait_load() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 bytes apart.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// Instruction descriptor: kind::f8f6f4, A = B = e4m3, D = f32, both K-major, M = 128, N = 64.
constexpr uint32_t kIdesc = (1u << 4) | ((uint32_t)(kN >> 3) << 17) | ((uint32_t)(kM >> 4) << 24);

// 2-D TMA tile load (x = pixel, a multiple of 128; y = row) completing its bytes on `bar`.
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
      ::"r"(smem_u32(dst)), "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// Bounded wait that also gives up when another role has aborted; a timeout names its site.
__device__ __forceinline__ bool wait_bar(uint64_t* bar, uint32_t parity, volatile int* abort, int* error, int site) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long start = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (*abort) return false;
    if (clock64() - start > kWaitLimit) {
      *abort = 1;
      atomicOr(error, kTimeoutBit | (1 << (kSiteBit + site)));
      return false;
    }
  }
  return true;
}

// Position in a ring of N stages: the slot, the parity of its current use and whether it was used
// before (then its release must be awaited). Kept incrementally: no 64-bit division per stage.
template <int N>
struct Ring {
  int slot = 0;
  uint32_t phase = 0;
  bool reused = false;
  __device__ __forceinline__ void next() {
    if (++slot == N) {
      slot = 0;
      phase ^= 1u;
      reused = true;
    }
  }
};

// Operand tiles of TMA slot s: the staged operand slots first, then slots carved from the raw ring
// (1024-byte aligned: the raw ring starts 72 KB into the 1024-aligned shared block).
__device__ __forceinline__ uint8_t* tma_tile_a(ContractShared& sm, int s) {
  return s < kRing ? sm.a[s] : sm.raw[0] + (s - kRing) * kTmaSlotBytes;
}
__device__ __forceinline__ uint8_t* tma_tile_b(ContractShared& sm, int s) {
  return s < kRing ? sm.b[s] : sm.raw[0] + (s - kRing) * kTmaSlotBytes + kM * kAtom;
}

// Wait for the last phase of every barrier of a ring that has no further uses (so no phase can alias).
template <int N>
__device__ __forceinline__ bool drain(uint64_t* bars, const Ring<N>& r, volatile int* abort, int* error, int site) {
  for (int s = 0; s < N; ++s) {
    if (s < r.slot) {
      if (!wait_bar(&bars[s], r.phase, abort, error, site)) return false;
    } else if (r.reused) {
      if (!wait_bar(&bars[s], r.phase ^ 1u, abort, error, site)) return false;
    }
  }
  return true;
}

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
// Arrive once on `bar` (no pending-count increment) when this thread's earlier cp.async copies have landed.
__device__ __forceinline__ void cp_async_arrive(uint64_t* bar) {
  asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

__device__ __forceinline__ uint32_t keep_bytes(int keep) {
  return keep >= 4 ? 0xffffffffu : (keep <= 0 ? 0u : ((1u << (8 * keep)) - 1u));
}

// ---- work traversal (identical in every role) -----------------------------

struct Block {
  int64_t index = -1;
  int64_t first_chunk = 0, last_chunk = 0;  // [first, last)
  int64_t pixels = 0;
  bool tma = false;  // both operands come from the image's tensor maps
};

__device__ __forceinline__ int64_t block_of_chunk(const int64_t* blocks, int64_t n_blocks, int64_t chunk) {
  int64_t lo = 0, hi = n_blocks - 1;
  while (lo < hi) {
    const int64_t mid = (lo + hi + 1) >> 1;
    if (blocks[mid * kBlkFields + kBlkChunk] <= chunk) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Moves blk to the block holding `chunk`; true when this chunk starts a new accumulator segment
// (first chunk of the CTA, a block change, or kSegmentChunks chunks into the current segment).
__device__ __forceinline__ bool advance(Block& blk, int64_t& seg_start, const int64_t* descs, const int64_t* blocks,
                                        int64_t n_blocks, int64_t chunk, bool maps) {
  if (blk.index >= 0 && chunk < blk.last_chunk) {
    if (chunk - seg_start < kSegmentChunks) return false;
    seg_start = chunk;
    return true;
  }
  blk.index = blk.index < 0 ? block_of_chunk(blocks, n_blocks, chunk) : blk.index + 1;
  const int64_t* r = blocks + blk.index * kBlkFields;
  const int64_t* d = desc_of(descs, r[kBlkImage]);
  blk.pixels = d[kPixels];
  blk.tma = maps && (d[kFlags] & 4);
  blk.first_chunk = r[kBlkChunk];
  blk.last_chunk = blk.first_chunk + ceil_div(blk.pixels, kInterval);
  seg_start = chunk;
  return true;
}

// Segment ends after `chunk` (the CTA range ends, the block ends, or the segment is full).
__device__ __forceinline__ bool segment_ends(const Block& blk, int64_t seg_start, int64_t chunk, int64_t c_end) {
  return chunk + 1 >= c_end || chunk + 1 >= blk.last_chunk || chunk + 1 - seg_start >= kSegmentChunks;
}

__device__ __forceinline__ int stages_of(const Block& blk, int64_t chunk, int64_t* x_begin) {
  *x_begin = (chunk - blk.first_chunk) * kInterval;
  const int64_t len = min((int64_t)kInterval, blk.pixels - *x_begin);
  return (int)ceil_div(len, kAtom);
}

// Rows of one block: detections then targets (both in mask order), with their mask row pointers.
struct Rows {
  const uint8_t* pm;
  const uint8_t* gm;
  int64_t stride;
  int Dm, Gn;
  __device__ __forceinline__ const uint8_t* row(int r) const {
    return r < Dm ? pm + (int64_t)r * stride : gm + (int64_t)(r - Dm) * stride;
  }
};

__device__ __forceinline__ Rows rows_of(const int64_t* descs, const int64_t* blocks, int64_t index) {
  const int64_t* r = blocks + index * kBlkFields;
  const int64_t* d = desc_of(descs, r[kBlkImage]);
  const int64_t m0 = r[kBlkM0], n0 = r[kBlkN0];
  Rows rows;
  rows.stride = d[kMaskStride];
  rows.pm = reinterpret_cast<const uint8_t*>(d[kMasks]) + m0 * rows.stride;
  rows.gm = reinterpret_cast<const uint8_t*>(d[kTarget]) + n0 * rows.stride;
  rows.Dm = (int)min((int64_t)kRowsA, d[kD] - m0);
  rows.Gn = (int)min((int64_t)kRowsB, d[kG] - n0);
  return rows;
}

__global__ void __launch_bounds__(kThreads, 1)
inst_contract_kernel(const int64_t* __restrict__ descs, const int64_t* __restrict__ blocks, int64_t n_blocks,
                     int64_t total_chunks, int64_t chunks_per_cta, const int64_t* __restrict__ bounds,
                     const int64_t* __restrict__ order, u32* __restrict__ inter, u64* __restrict__ pa,
                     u64* __restrict__ ga, const CUtensorMap* __restrict__ maps, int* __restrict__ error) {
  extern __shared__ unsigned char smem_raw[];
  ContractShared& sm = *reinterpret_cast<ContractShared*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  const int64_t c_begin = bounds ? bounds[blockIdx.x] : (int64_t)blockIdx.x * chunks_per_cta;
  const int64_t c_end = bounds ? min(bounds[blockIdx.x + 1], total_chunks) : min(c_begin + chunks_per_cta, total_chunks);
  if (c_begin >= c_end) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool has_maps = maps != nullptr;

  // Constant ones rows (A row 127, B row 63) in every operand stage, barriers, TMEM.
  for (int i = threadIdx.x; i < kRing * (kAtom / 16); i += blockDim.x) {
    const int slot = i / (kAtom / 16), c = i % (kAtom / 16);
    const uint4 ones = make_uint4(0x01010101u, 0x01010101u, 0x01010101u, 0x01010101u);
    *reinterpret_cast<uint4*>(&sm.a[slot][kRowsA * kAtom + 16 * c]) = ones;
    *reinterpret_cast<uint4*>(&sm.b[slot][kRowsB * kAtom + 16 * c]) = ones;
  }
  if (threadIdx.x == 0) {
    for (int i = 0; i < kRing; ++i) {
      mbar_init(&sm.full[i], kConvertWarps);
      mbar_init(&sm.empty[i], 1);
    }
    for (int i = 0; i < kRawRing; ++i) {
      mbar_init(&sm.raw_full[i], kCopyWarps * 32);
      mbar_init(&sm.raw_empty[i], kConvertWarps);
    }
    for (int i = 0; i < kTmaRing; ++i) {
      mbar_init(&sm.tma_full[i], 1);
      mbar_init(&sm.tma_empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&sm.acc_full[i], 1);
      mbar_init(&sm.acc_empty[i], kEpilogueWarps);
    }
    mbar_init(&sm.done, 1);
    sm.abort = 0;
    mbar_fence_init();
  }
  fence_async_smem();
  if (warp == kMmaWarp) {
    tmem_alloc(&sm.tmem_base, kTmemCols);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = sm.tmem_base;
  volatile int* abort = &sm.abort;

  if (warp == kMmaWarp) {
    // ---- MMA issuer ----------------------------------------------------------
    if (lane == 0) {
      Block blk;
      int64_t seg_start = 0, segment = 0;
      Ring<kRing> ring;     // staged stages
      Ring<kTmaRing> tring;  // TMA stages
      bool ok = true, first = true;
      for (int64_t chunk = c_begin; chunk < c_end && ok; ++chunk) {
        const bool fresh = advance(blk, seg_start, descs, blocks, n_blocks, chunk, has_maps);
        const int buf = (int)(segment & 1);
        if (fresh) {
          if (segment >= 2 && !wait_bar(&sm.acc_empty[buf], (uint32_t)(((segment >> 1) - 1) & 1), abort, error, kAtAccEmpty)) {
            ok = false;
            break;
          }
          tc_fence_after();
          first = true;
        }
        int64_t x_begin;
        const int stages = stages_of(blk, chunk, &x_begin);
        const uint32_t d_tmem = tmem + (uint32_t)(buf * kN);
        for (int st = 0; st < stages; ++st) {
          const bool tma = blk.tma;
          const int slot = tma ? tring.slot : ring.slot;
          if (!wait_bar(tma ? &sm.tma_full[slot] : &sm.full[slot], tma ? tring.phase : ring.phase, abort, error,
                        tma ? kAtFullTma : kAtFull)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint64_t a_desc = sw128_desc(smem_u32(tma ? tma_tile_a(sm, slot) : sm.a[slot]));
          const uint64_t b_desc = sw128_desc(smem_u32(tma ? tma_tile_b(sm, slot) : sm.b[slot]));
#pragma unroll
          for (int k = 0; k < kAtom / kMmaK; ++k)
            mma_f8(d_tmem, a_desc + (uint64_t)(k * kMmaK / 16), b_desc + (uint64_t)(k * kMmaK / 16), kIdesc,
                   (first && k == 0) ? 0u : 1u);
          first = false;
          mma_commit(tma ? &sm.tma_empty[slot] : &sm.empty[slot]);  // the stage is free once its MMAs have read it
          if (tma) tring.next(); else ring.next();
        }
        if (!ok) break;
        if (segment_ends(blk, seg_start, chunk, c_end)) {
          mma_commit(&sm.acc_full[buf]);
          ++segment;
        }
      }
      // Every MMA issued so far retires before TMEM or shared memory is released.
      mma_commit(&sm.done);
      mbar_wait(&sm.done, 0, kWaitLimit);
    }
    __syncwarp();
  } else if (warp >= kFirstCopyWarp && warp < kFirstConvertWarp) {
    // ---- copy warps: aligned words of rows [c * kCopyRows, ...) -> raw ring ---
    // Lane item k = word (lane + 32 k) of the warp's rows, row-major: consecutive lanes copy
    // consecutive words of a row. Sources, bounds and destinations are set once per block.
    const int c = warp - kFirstCopyWarp;
    const int r0 = c * kCopyRows;
    const uint8_t* src[kCopyItems];  // the item's aligned word at x = 0
    int64_t room[kCopyItems];        // the word holds a row byte while x0 < room
    uint32_t dst[kCopyItems];        // byte offset in a raw stage
    uint32_t live = 0;               // bit k: item k exists in this block
    Block blk;
    int64_t seg_start = 0, cached = -1;
    Ring<kRawRing> ring;
    bool ok = true, seen_tma = false;
    for (int64_t chunk = c_begin; chunk < c_end && ok; ++chunk) {
      advance(blk, seg_start, descs, blocks, n_blocks, chunk, has_maps);
      if (blk.tma) {  // loaded by TMA into slots that include the raw ring
        seen_tma = true;
        continue;
      }
      if (seen_tma) break;  // staged after TMA: the converters report it
      if (blk.index != cached) {
        cached = blk.index;
        const Rows rows = rows_of(descs, blocks, blk.index);
        const int items = max(0, min(kCopyRows, rows.Dm + rows.Gn - r0)) * kRawWords;
        live = 0;
#pragma unroll
        for (int k = 0; k < kCopyItems; ++k) {
          const int i = lane + 32 * k;
          const int r = i / kRawWords, w = i - r * kRawWords;
          src[k] = nullptr;
          room[k] = 0;
          dst[k] = (uint32_t)((r0 + r) * kRawRow + 16 * w);
          if (i < items) {
            const uint8_t* p = rows.row(r0 + r);
            const int o = (int)(reinterpret_cast<uintptr_t>(p) & 15);
            src[k] = p - o + 16 * w;
            room[k] = blk.pixels + o - 16 * w;
            live |= 1u << k;
          }
        }
      }
      int64_t x_begin;
      const int stages = stages_of(blk, chunk, &x_begin);
      for (int st = 0; st < stages; ++st, ring.next()) {
        const int slot = ring.slot;
        const bool got = !ring.reused || wait_bar(&sm.raw_empty[slot], ring.phase ^ 1u, abort, error, kAtRaw);
        if (!__all_sync(0xffffffffu, got)) {
          ok = false;
          break;
        }
        const int64_t x0 = x_begin + (int64_t)st * kAtom;
        uint8_t* stage = sm.raw[slot];
#pragma unroll
        for (int k = 0; k < kCopyItems; ++k) {
          if (!((live >> k) & 1u)) continue;
          if (x0 < room[k]) cp_async16(stage + dst[k], src[k] + x0);  // words past the row end stay stale
        }
        cp_async_arrive(&sm.raw_full[slot]);
      }
    }
    cp_async_wait_all();  // no copy into shared memory outlives the CTA
  } else if (warp >= kFirstConvertWarp) {
    // ---- converters: raw words -> re-aligned, swizzled operand stages -----------
    // Lane = kLanesPerRow * q + h: row q of the warp's kConvertRowsPerWarp rows in a round, 16-byte chunks
    // c0 = h * kConvertChunks ... of the row's 128 bytes. Converter 0 also issues the TMA loads of TMA blocks.
    const int cw = warp - kFirstConvertWarp;
    const int q = lane / kLanesPerRow, c0 = (lane % kLanesPerRow) * kConvertChunks;
    Block blk;
    int64_t seg_start = 0, cached = -1;
    Ring<kRawRing> raw_ring;
    Ring<kRing> ring;
    Ring<kTmaRing> tring;  // converter 0 lane 0: TMA stages issued
    bool tma_started = false;
    uint32_t dst_row[kConvertRounds];  // this lane's tile row (bits 0-30), B tile (bit 31)
    int shift[kConvertRounds];
    bool valid[kConvertRounds];
    bool ok = true;
    for (int64_t chunk = c_begin; chunk < c_end && ok; ++chunk) {
      advance(blk, seg_start, descs, blocks, n_blocks, chunk, has_maps);
      int64_t x_begin;
      const int stages = stages_of(blk, chunk, &x_begin);
      if (blk.tma) {
        if (cw != 0) continue;
        if (!tma_started) {
          // The staged stages before are done: the MMA has read every staged operand stage and the
          // converters every raw stage (last phases, which cannot alias). Then the ones rows of the
          // slots carved from the raw ring.
          tma_started = true;
          bool got = true;
          if (lane == 0)
            got = drain(sm.empty, ring, abort, error, kAtStageSlot) && drain(sm.raw_empty, raw_ring, abort, error, kAtRaw);
          if (!__shfl_sync(0xffffffffu, (int)got, 0)) {
            ok = false;
            break;
          }
          const uint4 ones = make_uint4(0x01010101u, 0x01010101u, 0x01010101u, 0x01010101u);
          for (int i = lane; i < kTmaExtra * (kAtom / 16); i += 32) {
            const int s = kRing + i / (kAtom / 16), c16 = i % (kAtom / 16);
            *reinterpret_cast<uint4*>(tma_tile_a(sm, s) + kRowsA * kAtom + 16 * c16) = ones;
            *reinterpret_cast<uint4*>(tma_tile_b(sm, s) + kRowsB * kAtom + 16 * c16) = ones;
          }
          fence_async_smem();  // generic stores before the tensor core reads them
          __syncwarp();
        }
        bool got = true;
        if (lane == 0) {
          const int64_t* r = blocks + blk.index * kBlkFields;
          const CUtensorMap* m = maps + 2 * r[kBlkImage];
          for (int st = 0; st < stages; ++st, tring.next()) {
            const int slot = tring.slot;
            if (tring.reused && !wait_bar(&sm.tma_empty[slot], tring.phase ^ 1u, abort, error, kAtTmaSlot)) {
              got = false;
              break;
            }
            const int x = (int)(x_begin + (int64_t)st * kAtom);
            mbar_arrive_expect_tx(&sm.tma_full[slot], kTmaBytes);  // release: the ones rows above
            tma_load_2d(tma_tile_a(sm, slot), m, x, (int)r[kBlkM0], &sm.tma_full[slot]);
            tma_load_2d(tma_tile_b(sm, slot), m + 1, x, (int)r[kBlkN0], &sm.tma_full[slot]);
          }
        }
        if (!__shfl_sync(0xffffffffu, (int)got, 0)) ok = false;
        continue;
      }
      if (tma_started) {  // a staged block after a TMA block: the host orders them the other way
        if (lane == 0) atomicOr(error, kOrderBit);
        *abort = 1;
        ok = false;
        break;
      }
      if (blk.index != cached) {
        cached = blk.index;
        const Rows rows = rows_of(descs, blocks, blk.index);
#pragma unroll
        for (int k = 0; k < kConvertRounds; ++k) {
          const int row = cw * kConvertRowsPerWarp + q + kConvertRowsPerRound * k;
          valid[k] = row < rows.Dm + rows.Gn;
          shift[k] = valid[k] ? (int)(reinterpret_cast<uintptr_t>(rows.row(row)) & 15) : 0;
          const int t = row < rows.Dm ? row : row - rows.Dm;
          dst_row[k] = (uint32_t)t | (row < rows.Dm ? 0u : 0x80000000u);
        }
      }
      for (int st = 0; st < stages; ++st, raw_ring.next(), ring.next()) {
        const int rslot = raw_ring.slot, slot = ring.slot;
        bool got = wait_bar(&sm.raw_full[rslot], raw_ring.phase, abort, error, kAtRaw);
        got = got && (!ring.reused || wait_bar(&sm.empty[slot], ring.phase ^ 1u, abort, error, kAtStageSlot));
        if (!__all_sync(0xffffffffu, got)) {
          ok = false;
          break;
        }
        const int64_t x0 = x_begin + (int64_t)st * kAtom;
        const bool tail = blk.pixels - x0 < kAtom;  // the same for the whole CTA
        const int left = (int)min((int64_t)kAtom, blk.pixels - x0) - 16 * c0;  // row bytes from chunk c0 on
        const uint8_t* raw = sm.raw[rslot];
        uint8_t* tile_a = sm.a[slot];
        uint8_t* tile_b = sm.b[slot];
        // One round at a time (load, re-align, store): hoisting every load of the stage measured slower,
        // the register cap then limits the overlap. Separate loops for the tail: the mask costs selects.
        auto store = [&](auto masked) {
#pragma unroll
          for (int k = 0; k < kConvertRounds; ++k) {
            if (!valid[k]) continue;
            const int row = cw * kConvertRowsPerWarp + q + kConvertRowsPerRound * k;
            const uint4* words = reinterpret_cast<const uint4*>(raw + row * kRawRow) + c0;
            uint4 wv[kConvertChunks + 1];
#pragma unroll
            for (int j = 0; j <= kConvertChunks; ++j) wv[j] = words[j];
            const int t = (int)(dst_row[k] & 0x7fffffffu);
            uint8_t* tile = ((dst_row[k] & 0x80000000u) ? tile_b : tile_a) + t * kAtom;
#pragma unroll
            for (int j = 0; j < kConvertChunks; ++j) {
              uint4 v = realign16(wv[j], wv[j + 1], shift[k]);
              if constexpr (decltype(masked)::value) {  // bytes past the row end belong to the next row
                const int l = left - 16 * j;
                v.x &= keep_bytes(l);
                v.y &= keep_bytes(l - 4);
                v.z &= keep_bytes(l - 8);
                v.w &= keep_bytes(l - 12);
              }
              *reinterpret_cast<uint4*>(tile + (((c0 + j) ^ (t & 7)) << 4)) = v;
            }
          }
        };
        if (tail) store(std::true_type{}); else store(std::false_type{});
        fence_async_smem();
        __syncwarp();
        if (lane == 0) {
          mbar_arrive(&sm.raw_empty[rslot]);
          mbar_arrive(&sm.full[slot]);
        }
      }
    }
    if (cw == 0 && lane == 0 && tma_started)  // the last TMA load into every slot lands before the CTA exits
      for (int s = 0; s < kTmaRing; ++s) {
        if (s < tring.slot) mbar_wait(&sm.tma_full[s], tring.phase, kWaitLimit);
        else if (tring.reused) mbar_wait(&sm.tma_full[s], tring.phase ^ 1u, kWaitLimit);
      }
    __syncwarp();
  } else {
    // ---- epilogue: accumulator -> integer counts -> global counters ------------
    const int row = warp * 32 + lane;
    Block blk;
    int64_t seg_start = 0, segment = 0, ranked = -1;
    bool ok = true;
    for (int64_t chunk = c_begin; chunk < c_end && ok; ++chunk) {
      advance(blk, seg_start, descs, blocks, n_blocks, chunk, has_maps);
      if (!segment_ends(blk, seg_start, chunk, c_end)) continue;
      const int buf = (int)(segment & 1);
      const bool got = wait_bar(&sm.acc_full[buf], (uint32_t)((segment >> 1) & 1), abort, error, kAtAccFull);
      if (!__all_sync(0xffffffffu, got)) {
        ok = false;
        break;
      }
      tc_fence_after();
      uint32_t v0[32], v1[32];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(buf * kN);
      tmem_load32(taddr, v0);
      tmem_load32(taddr + 32, v1);
      tmem_wait_load();
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&sm.acc_empty[buf]);
      ++segment;
      const int64_t* r = blocks + blk.index * kBlkFields;
      const int64_t* d = desc_of(descs, r[kBlkImage]);
      const int m0 = (int)r[kBlkM0], n0 = (int)r[kBlkN0];
      const int G = (int)d[kG];
      const int D = (int)d[kD];
      const int Dm = min(kRowsA, D - m0), Gn = min(kRowsB, G - n0);
      if (ranked != blk.index) {
        // Score rank of this warp's detection rows m0 + 32 warp + lane: invert the image's score order.
        ranked = blk.index;
        const int64_t* ord = order + d[kDetBegin];
        const int lo = m0 + 32 * warp;
        __syncwarp();
        for (int i = lane; i < D; i += 32) {
          const int k = (int)ord[i] - lo;
          if (k >= 0 && k < 32) sm.rank[warp][k] = i;
        }
        __syncwarp();
      }
      if (row < Dm) {
        const int rank = sm.rank[warp][lane];
        u32* out = inter + d[kDPairBegin] + (int64_t)rank * G + n0;
#pragma unroll
        for (int col = 0; col < 32; ++col) {
          const u32 lo = (u32)__float2uint_rz(kCountScale * __uint_as_float(v0[col]));
          const u32 hi = (u32)__float2uint_rz(kCountScale * __uint_as_float(v1[col]));
          if (col < Gn && lo) atomicAdd(out + col, lo);
          if (col + 32 < Gn && hi) atomicAdd(out + col + 32, hi);
        }
        const u32 area = (u32)__float2uint_rz(kCountScale * __uint_as_float(v1[kRowsB - 32]));
        if (n0 == 0 && area) atomicAdd(pa + d[kDetBegin] + rank, (u64)area);
      }
      if (row == kRowsA && m0 == 0) {
#pragma unroll
        for (int col = 0; col < 32; ++col) {
          const u32 lo = (u32)__float2uint_rz(kCountScale * __uint_as_float(v0[col]));
          const u32 hi = (u32)__float2uint_rz(kCountScale * __uint_as_float(v1[col]));
          if (col < Gn && lo) atomicAdd(ga + d[kSlotBegin] + n0 + col, (u64)lo);
          if (col + 32 < Gn && hi) atomicAdd(ga + d[kSlotBegin] + n0 + col + 32, (u64)hi);
        }
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == kMmaWarp) {
    tc_fence_after();
    tmem_dealloc(tmem, kTmemCols);
  }
}

// cuTensorMapEncodeTiled from the CUDA driver API, looked up once.
PFN_cuTensorMapEncodeTiled_v12000 encode_tiled() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult found;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &found) !=
            cudaSuccess ||
        found != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }();
  return fn;
}

// One operand's map: rows x pixels bytes at `base`, `stride` bytes per row, boxes of box_rows x 128.
bool encode_rows(CUtensorMap* map, const void* base, int64_t pixels, int64_t rows, int64_t stride, int box_rows) {
  const cuuint64_t dims[2] = {(cuuint64_t)pixels, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)stride};
  const cuuint32_t box[2] = {(cuuint32_t)kAtom, (cuuint32_t)box_rows};
  const cuuint32_t elem[2] = {1, 1};
  return encode_tiled()(map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<void*>(base), dims, strides, box, elem,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace
}  // namespace pe

using namespace pe;

// Tensor maps for the contraction's TMA loads (host side, no GPU work). descs:
// the HOST copy of the instance descriptor table (B rows, before upload);
// maps: a host buffer of B x 2 x 128 bytes, 64-byte aligned. For every image
// whose mask rows start on 16-byte boundaries (flags bit 1) with detections,
// targets and pixels, writes the detection-mask map (box 127 rows x 128 bytes)
// and the target-mask map (63 x 128) and sets flags bit 2; other images keep
// bit 2 clear and are staged by the worker warps. Returns the number of images
// given maps, or a negative error code.
PE_API int pe_contract_maps(int64_t* descs, int64_t B, void* maps) {
  PE_REQUIRE(B >= 0 && (B == 0 || (descs && maps)), "invalid arguments");
  PE_REQUIRE((reinterpret_cast<uintptr_t>(maps) & 63) == 0, "tensor maps must be 64-byte aligned");
  if (!encode_tiled()) return 0;  // no driver entry point: every image is staged
  CUtensorMap* out = reinterpret_cast<CUtensorMap*>(maps);
  int given = 0;
  for (int64_t b = 0; b < B; ++b) {
    int64_t* d = descs + b * kDescFields;
    d[kFlags] &= ~int64_t{4};
    const int64_t pixels = d[kPixels], D = d[kD], G = d[kG], stride = d[kMaskStride];
    if (!(d[kFlags] & 2) || pixels <= 0 || D <= 0 || G <= 0 || stride % 16 || (d[kMasks] | d[kTarget]) % 16 ||
        pixels > stride || pixels > (int64_t{1} << 31) - kAtom || D > (int64_t{1} << 31) || G > (int64_t{1} << 31))
      continue;
    if (encode_rows(out + 2 * b, reinterpret_cast<const void*>(d[kMasks]), pixels, D, stride, kRowsA) &&
        encode_rows(out + 2 * b + 1, reinterpret_cast<const void*>(d[kTarget]), pixels, G, stride, kRowsB)) {
      d[kFlags] |= 4;
      ++given;
    }
  }
  return given;
}

// Block table and CTA chunk ranges of pe_inst_contract (host side, no GPU
// work). Image b has dets[b] detection masks, gts[b] target masks and
// pixels[b] pixels; tma (optional) marks the images loaded by TMA. Every image
// with pixels and masks is covered by 127 x 63 tiles (row-major over detection
// and target tiles) of ceil(pixels / 4096) chunks; staged images come first,
// TMA images after them, each group in image order, and chunks are numbered
// block after block. blocks receives the rows (image, first detection, first
// target, first chunk), at most blocks_cap of them; *total_chunks the chunk
// count. With ctas > 0, bounds (ctas + 1 entries) receives R + 1 chunk indices
// (R = min(ctas, total chunks), at least 1, in *ranges) that split the chunks
// into R contiguous ranges of about equal cost: a chunk costs its pixels x
// (the block's detection and target rows + 8), times tma_cost for TMA blocks.
// The split is found per block (a block's cost grows linearly over its
// chunks), so the planning costs O(blocks + R) whatever the pixel count.
// Returns the number of blocks, or a negative error code.
PE_API int64_t pe_contract_blocks(const int64_t* dets, const int64_t* gts, const int64_t* pixels, const uint8_t* tma,
                                  int64_t B, double tma_cost, int64_t ctas, int64_t* blocks, int64_t blocks_cap,
                                  int64_t* bounds, int64_t* total_chunks, int64_t* ranges) {
  PE_REQUIRE(B >= 0 && (B == 0 || (dets && gts && pixels)) && blocks_cap >= 0 && total_chunks && ranges,
             "invalid arguments");
  PE_REQUIRE(tma_cost > 0.0 && tma_cost < 1e6, "tma_cost must be positive");
  PE_REQUIRE(ctas <= 0 || bounds, "bounds required with ctas");
  int64_t n = 0, chunks = 0;
  for (int kind = 0; kind < 2; ++kind) {  // staged images, then TMA images
    for (int64_t b = 0; b < B; ++b) {
      if ((tma && tma[b]) != (kind == 1)) continue;
      const int64_t D = dets[b], G = gts[b], P = pixels[b];
      PE_REQUIRE(D >= 0 && G >= 0 && P >= 0, "negative size for image %lld", (long long)b);
      if (P == 0 || (D == 0 && G == 0)) continue;
      const int64_t m_tiles = std::max<int64_t>(ceil_div(D, kRowsA), 1);
      const int64_t n_tiles = std::max<int64_t>(ceil_div(G, kRowsB), 1);
      const int64_t per = ceil_div(P, kInterval);
      for (int64_t i = 0; i < m_tiles; ++i)
        for (int64_t j = 0; j < n_tiles; ++j, ++n, chunks += per) {
          if (n >= blocks_cap) continue;  // counted, reported below
          int64_t* r = blocks + n * kBlkFields;
          r[kBlkImage] = b;
          r[kBlkM0] = i * kRowsA;
          r[kBlkN0] = j * kRowsB;
          r[kBlkChunk] = chunks;
        }
    }
  }
  PE_REQUIRE(n <= blocks_cap, "block table needs %lld rows, %lld given", (long long)n, (long long)blocks_cap);
  *total_chunks = chunks;
  *ranges = 0;
  if (ctas <= 0) return n;
  const int64_t R = std::max<int64_t>(1, std::min(ctas, chunks));
  *ranges = R;
  bounds[0] = 0;
  bounds[R] = chunks;
  if (chunks == 0) return n;
  auto weight = [&](int64_t k) {
    const int64_t* r = blocks + k * kBlkFields;
    const int64_t b = r[kBlkImage];
    const int64_t rows = std::min<int64_t>(kRowsA, dets[b] - r[kBlkM0]) +
                         std::min<int64_t>(kRowsB, gts[b] - r[kBlkN0]) + 8;  // + fixed work per stage
    return (tma && tma[b] ? tma_cost : 1.0) * (double)rows;
  };
  double total = 0.0;
  for (int64_t k = 0; k < n; ++k) total += weight(k) * (double)pixels[blocks[k * kBlkFields + kBlkImage]];
  // Targets i x total / R in increasing order: walk the blocks once, keeping the cost at the end of block k.
  int64_t k = 0, prev = 0;
  double start = 0.0, w = weight(0);
  double end = w * (double)pixels[blocks[kBlkImage]];
  for (int64_t i = 1; i < R; ++i) {
    const double target = total * (double)i / (double)R;
    while (k + 1 < n && end < target) {
      ++k;
      start = end;
      w = weight(k);
      end = start + w * (double)pixels[blocks[k * kBlkFields + kBlkImage]];
    }
    // The first chunk of block k whose end reaches the target; the range boundary follows it.
    const int64_t* r = blocks + k * kBlkFields;
    const int64_t per = ceil_div(pixels[r[kBlkImage]], kInterval);
    int64_t j = (int64_t)std::ceil((target - start) / (w * (double)kInterval)) - 1;
    j = std::min(std::max<int64_t>(j, 0), per - 1);
    prev = std::max(prev, std::min(r[kBlkChunk] + j + 1, chunks));
    bounds[i] = prev;
  }
  return n;
}

// Detection x target intersection counts and both mask areas for the batched
// InstanceEvaluator, on the tensor cores. descs: instance descriptor table
// (kMasks = prediction masks, kTarget = target masks, kMaskStride bytes per
// row, kDetBegin / kSlotBegin / kDPairBegin offsets); blocks: n_blocks rows of
// (image, first detection, first target, first chunk) with 127 x 63 tiles and
// ceil(pixels / 4096) chunks each, ordered by first chunk; order: score order
// from pe_seg_sort. inter (u32, sum D*G, rows in score order), pa (u64, sum D,
// score order) and ga (u64, sum G) are zeroed here. maps (device memory, or
// NULL): pe_contract_maps' output for the same table; images with flags bit 2
// are then loaded by TMA. Drop-in for the reference's pack_masks + overlap
// (instance_kernel.cu:10-39).
PE_API int pe_inst_contract(const int64_t* descs, const int64_t* blocks, int64_t n_blocks, int64_t total_chunks,
                            const int64_t* cta_bounds, int64_t ctas, const int64_t* order, uint32_t* inter,
                            int64_t inter_len, uint64_t* pa, int64_t pa_len, uint64_t* ga, int64_t ga_len,
                            const void* maps, int32_t* error, cudaStream_t stream) {
  PE_REQUIRE(n_blocks >= 0 && total_chunks >= 0 && inter_len >= 0 && pa_len >= 0 && ga_len >= 0, "invalid batch");
  PE_REQUIRE(n_blocks > 0 || total_chunks == 0, "chunks without blocks");
  PE_REQUIRE((reinterpret_cast<uintptr_t>(maps) & 63) == 0, "tensor maps must be 64-byte aligned");
  if (inter_len) PE_CUDA(cudaMemsetAsync(inter, 0, sizeof(uint32_t) * inter_len, stream));
  if (pa_len) PE_CUDA(cudaMemsetAsync(pa, 0, sizeof(uint64_t) * pa_len, stream));
  if (ga_len) PE_CUDA(cudaMemsetAsync(ga, 0, sizeof(uint64_t) * ga_len, stream));
  if (total_chunks == 0) return kOk;
  PE_REQUIRE(!cta_bounds || (ctas > 0 && ctas <= INT_MAX), "invalid CTA count");
  const int64_t even = std::min<int64_t>(total_chunks, sm_count());
  const int64_t per_cta = ceil_div(total_chunks, even);
  const int64_t grid = cta_bounds ? ctas : ceil_div(total_chunks, per_cta);
  const size_t smem = sizeof(ContractShared) + 1024;
  PE_CUDA(cudaFuncSetAttribute(inst_contract_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  inst_contract_kernel<<<(unsigned)grid, kThreads, smem, stream>>>(
      descs, blocks, n_blocks, total_chunks, per_cta, cta_bounds, order, reinterpret_cast<u32*>(inter),
      reinterpret_cast<u64*>(pa), reinterpret_cast<u64*>(ga), reinterpret_cast<const CUtensorMap*>(maps), error);
  PE_LAUNCHED("inst_contract");
  count_launch();
  return kOk;
}
