// Mask-vs-mask intersection counts for InstanceEvaluator on the tcgen05 tensor
// cores (sm_103a).
//
// inter[d][g] = sum_x pred[d][x] * gt[g][x] over 0/1 mask bytes is a dense
// (D x HW) by (HW x G) product, the contraction of the reference's
// pack_masks + overlap (instance_kernel.cu:10-39; CPU instance.py:255-264),
// which counts each pair with packed-word popcounts. Here each image is tiled
// into blocks of up to 127 detections (in score order) x 63 targets. A CTA
// streams 256-pixel stages of those rows (two 128-byte swizzle atoms) into
// shared memory in the canonical 128-byte-swizzled K-major layout, as e4m3
// values (mask byte 1 -> 1.0, 0 -> 0.0), and one thread issues tcgen05.mma
// kind::f8f6f4 (M = 128, N = 64, K = 32) into an fp32 accumulator in tensor
// memory. Row 127 of the A tile and
// row 63 of the B tile are constant ones, so the same product also yields the
// target areas (row 127) and the detection areas (column 63).
//
// Exactness: every 4096 pixels the accumulator is read back (tcgen05.ld),
// converted to integers and added to 32-bit totals in shared memory, so no
// fp32 partial sum exceeds 4096 and each product is 0 or 1: the counts are
// exact integers whatever the accumulation order inside the tensor core.
// Totals go to the global u32 / u64 counters with atomic adds when the block
// changes, so results do not depend on how chunks are split across CTAs.
//
// Mask rows may start at any byte (row stride H*W): producer warps load
// aligned 16-byte words, re-align them with funnel shifts (the word that
// straddles two lanes comes from the neighbour by shuffle) and zero bytes past
// the row end. Every word they load holds at least one byte of the row. Each
// lane loads its word of both atoms of a stage before storing either, and CTAs
// take contiguous chunk ranges of equal cost (rows x pixels, set on the host).
//
// Roles per CTA (16 warps): warps 0-3 read the accumulator (TMEM lanes
// 32w..32w+31), warp 4 allocates TMEM and issues the MMAs, warps 5-15 fill the
// ring of shared-memory stages. Every mbarrier wait is bounded; a timeout sets
// bit 30 of *error, every role leaves its loop, the MMA thread waits (bounded)
// for its MMAs to retire and TMEM is freed before the CTA exits.
#include "pe_common.cuh"
#include "pe_desc.cuh"

namespace pe {
namespace {

constexpr int kM = 128;                 // A rows: 127 detections + ones row
constexpr int kN = 64;                  // B rows: 63 targets + ones row
constexpr int kRowsA = kM - 1;
constexpr int kRowsB = kN - 1;
constexpr int kAtom = 128;              // pixels of one 128-byte swizzle atom of K
constexpr int kAtoms = 2;               // atoms per stage
constexpr int kStagePixels = kAtom * kAtoms;
constexpr int kMmaK = 32;               // K of one kind::f8f6f4 MMA (bytes)
constexpr int kInterval = 4096;         // pixels per accumulator flush (one work chunk)
constexpr int kRing = 3;
constexpr int kEpilogueWarps = 4;
constexpr int kMmaWarp = 4;
constexpr int kProducerWarps = 11;
constexpr int kThreads = (kEpilogueWarps + 1 + kProducerWarps) * 32;
constexpr int kLaneBytes = 64;          // contiguous row bytes per producer lane and stage
constexpr int kLanesPerRow = kStagePixels / kLaneBytes;
constexpr int kRowsPerWarp = 32 / kLanesPerRow;
constexpr int kRowsPerRound = kProducerWarps * kRowsPerWarp;
constexpr int kRounds = (kRowsA + kRowsB + kRowsPerRound - 1) / kRowsPerRound;
constexpr int kTmemCols = 2 * kN;       // two accumulator buffers
constexpr long long kWaitLimit = 4000000000ll;  // ~2 s at 2 GHz
constexpr int kTimeoutBit = 1 << 30;
constexpr uint32_t kOne = 0x38u;        // e4m3 encoding of 1.0

static_assert(kRounds * kRowsPerRound >= kRowsA + kRowsB, "producer rounds cover every row");

struct __align__(1024) ContractShared {
  uint8_t a[kRing][kAtoms][kM * kAtom];
  uint8_t b[kRing][kAtoms][kN * kAtom];
  uint32_t totals[kN * kM];  // [column][row]
  uint64_t full[kRing];
  uint64_t empty[kRing];
  uint64_t acc_full[2];
  uint64_t acc_empty[2];
  uint64_t done;
  uint32_t tmem_base;
  int abort;
};

// Block table row: image, first detection row, first target row, first chunk.
enum : int { kBlkImage = 0, kBlkM0, kBlkN0, kBlkChunk, kBlkFields };

// ---- tcgen05 / proxy helpers ------------------------------------------------

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

// Bounded wait that also gives up when another role has aborted.
__device__ __forceinline__ bool wait_bar(uint64_t* bar, uint32_t parity, volatile int* abort, int* error) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long start = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (*abort) return false;
    if (clock64() - start > kWaitLimit) {
      *abort = 1;
      atomicOr(error, kTimeoutBit);
      return false;
    }
  }
  return true;
}

// ---- work traversal (identical in every role) -----------------------------

struct Block {
  int64_t index = -1;
  int64_t first_chunk = 0, last_chunk = 0;  // [first, last)
  int64_t pixels = 0;
};

__device__ __forceinline__ int64_t block_of_chunk(const int64_t* blocks, int64_t n_blocks, int64_t chunk) {
  int64_t lo = 0, hi = n_blocks - 1;
  while (lo < hi) {
    const int64_t mid = (lo + hi + 1) >> 1;
    if (blocks[mid * kBlkFields + kBlkChunk] <= chunk) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ void advance(Block& blk, const int64_t* descs, const int64_t* blocks, int64_t n_blocks,
                                        int64_t chunk) {
  if (blk.index >= 0 && chunk < blk.last_chunk) return;
  blk.index = blk.index < 0 ? block_of_chunk(blocks, n_blocks, chunk) : blk.index + 1;
  const int64_t* r = blocks + blk.index * kBlkFields;
  blk.pixels = desc_of(descs, r[kBlkImage])[kPixels];
  blk.first_chunk = r[kBlkChunk];
  blk.last_chunk = blk.first_chunk + ceil_div(blk.pixels, kInterval);
}

__device__ __forceinline__ int stages_of(const Block& blk, int64_t chunk, int64_t* x_begin) {
  *x_begin = (chunk - blk.first_chunk) * kInterval;
  const int64_t len = min((int64_t)kInterval, blk.pixels - *x_begin);
  return (int)ceil_div(len, kStagePixels);
}

// Bytes [o, o + 16) of the 32-byte string lo|hi (little-endian words), o in [0, 16): shifts by 8, 4
// and 0-3 bytes as selects and funnel shifts, with no branches (o differs between lanes).
__device__ __forceinline__ uint4 realign(uint4 lo, uint4 hi, int o) {
  uint32_t u0 = lo.x, u1 = lo.y, u2 = lo.z, u3 = lo.w, u4 = hi.x, u5 = hi.y, u6 = hi.z, u7 = hi.w;
  const bool b8 = o & 8, b4 = o & 4;
  u0 = b8 ? u2 : u0; u1 = b8 ? u3 : u1; u2 = b8 ? u4 : u2; u3 = b8 ? u5 : u3; u4 = b8 ? u6 : u4; u5 = b8 ? u7 : u5;
  u0 = b4 ? u1 : u0; u1 = b4 ? u2 : u1; u2 = b4 ? u3 : u2; u3 = b4 ? u4 : u3; u4 = b4 ? u5 : u4;
  const int sh = (o & 3) * 8;
  return make_uint4(__funnelshift_r(u0, u1, sh), __funnelshift_r(u1, u2, sh), __funnelshift_r(u2, u3, sh),
                    __funnelshift_r(u3, u4, sh));
}

__device__ __forceinline__ uint32_t keep_bytes(int keep) {
  return keep >= 4 ? 0xffffffffu : (keep <= 0 ? 0u : ((1u << (8 * keep)) - 1u));
}

__global__ void __launch_bounds__(kThreads, 1)
inst_contract_kernel(const int64_t* __restrict__ descs, const int64_t* __restrict__ blocks, int64_t n_blocks,
                     int64_t total_chunks, int64_t chunks_per_cta, const int64_t* __restrict__ bounds,
                     const int64_t* __restrict__ order, u32* __restrict__ inter, u64* __restrict__ pa,
                     u64* __restrict__ ga, int* __restrict__ error) {
  extern __shared__ unsigned char smem_raw[];
  ContractShared& sm = *reinterpret_cast<ContractShared*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  const int64_t c_begin = bounds ? bounds[blockIdx.x] : (int64_t)blockIdx.x * chunks_per_cta;
  const int64_t c_end = bounds ? min(bounds[blockIdx.x + 1], total_chunks) : min(c_begin + chunks_per_cta, total_chunks);
  if (c_begin >= c_end) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  // Constant ones rows (A row 127, B row 63) in every stage, zero totals, barriers, TMEM.
  for (int i = threadIdx.x; i < kRing * kAtoms * (kAtom / 16); i += blockDim.x) {
    const int slot = i / (kAtoms * (kAtom / 16)), h = (i / (kAtom / 16)) % kAtoms, c = i % (kAtom / 16);
    const uint4 ones = make_uint4(0x38383838u, 0x38383838u, 0x38383838u, 0x38383838u);
    *reinterpret_cast<uint4*>(&sm.a[slot][h][kRowsA * kAtom + 16 * c]) = ones;
    *reinterpret_cast<uint4*>(&sm.b[slot][h][kRowsB * kAtom + 16 * c]) = ones;
  }
  for (int i = threadIdx.x; i < kN * kM; i += blockDim.x) sm.totals[i] = 0;
  if (threadIdx.x == 0) {
    for (int i = 0; i < kRing; ++i) {
      mbar_init(&sm.full[i], kProducerWarps);
      mbar_init(&sm.empty[i], 1);
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
      int64_t seq = 0, interval = 0;
      bool ok = true;
      for (int64_t chunk = c_begin; chunk < c_end && ok; ++chunk) {
        advance(blk, descs, blocks, n_blocks, chunk);
        int64_t x_begin;
        const int stages = stages_of(blk, chunk, &x_begin);
        const int buf = (int)(interval & 1);
        if (interval >= 2 && !wait_bar(&sm.acc_empty[buf], (uint32_t)(((interval >> 1) - 1) & 1), abort, error)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t d_tmem = tmem + (uint32_t)(buf * kN);
        for (int st = 0; st < stages; ++st, ++seq) {
          const int slot = (int)(seq % kRing);
          if (!wait_bar(&sm.full[slot], (uint32_t)((seq / kRing) & 1), abort, error)) {
            ok = false;
            break;
          }
          tc_fence_after();
#pragma unroll
          for (int h = 0; h < kAtoms; ++h) {
            const uint64_t a_desc = sw128_desc(smem_u32(sm.a[slot][h]));
            const uint64_t b_desc = sw128_desc(smem_u32(sm.b[slot][h]));
#pragma unroll
            for (int k = 0; k < kAtom / kMmaK; ++k)
              mma_f8(d_tmem, a_desc + (uint64_t)(k * kMmaK / 16), b_desc + (uint64_t)(k * kMmaK / 16), kIdesc,
                     (st | h | k) != 0);
          }
          mma_commit(&sm.empty[slot]);  // the stage is free once these MMAs have read it
        }
        if (!ok) break;
        mma_commit(&sm.acc_full[buf]);
        ++interval;
      }
      // Every MMA issued so far retires before TMEM or shared memory is released.
      mma_commit(&sm.done);
      mbar_wait(&sm.done, 0, kWaitLimit);
    }
    __syncwarp();
  } else if (warp > kMmaWarp) {
    // ---- producers: mask rows -> swizzled e4m3 stages -------------------------
    // Lane = quarter * 8 + r: row r of the warp's 8 rows, bytes [64 * quarter, 64 * quarter + 64) of
    // the stage, i.e. chunks 4 * (quarter & 1) .. + 3 of atom quarter >> 1. The 8 lanes of a store
    // phase write one chunk column of 8 consecutive rows: 8 distinct swizzled positions, no conflicts.
    const int p = warp - kMmaWarp - 1;
    const int quarter = lane >> 3;
    const int atom = quarter >> 1;
    const int c0 = (quarter & 1) * 4;
    Block blk;
    int64_t cached = -1;
    const uint8_t* row_ptr[kRounds];
    uint32_t dst_off[kRounds];  // row offset in the atom (bits 0-23), row & 7 (bits 24-26), B tile (bit 31)
    int shift[kRounds];
    bool valid[kRounds];
    bool unaligned = false;
    int64_t pixels = 0;
    int64_t seq = 0;
    bool ok = true;
    for (int64_t chunk = c_begin; chunk < c_end && ok; ++chunk) {
      advance(blk, descs, blocks, n_blocks, chunk);
      if (blk.index != cached) {
        cached = blk.index;
        const int64_t* r = blocks + blk.index * kBlkFields;
        const int64_t* d = desc_of(descs, r[kBlkImage]);
        const int m0 = (int)r[kBlkM0], n0 = (int)r[kBlkN0];
        const int Dm = (int)min((int64_t)kRowsA, d[kD] - m0), Gn = (int)min((int64_t)kRowsB, d[kG] - n0);
        const uint8_t* pm = reinterpret_cast<const uint8_t*>(d[kMasks]);
        const uint8_t* gm = reinterpret_cast<const uint8_t*>(d[kTarget]);
        const int64_t stride = d[kMaskStride];
        pixels = d[kPixels];
        bool any = false;
#pragma unroll
        for (int k = 0; k < kRounds; ++k) {
          const int row = p * kRowsPerWarp + (lane & (kRowsPerWarp - 1)) + kRowsPerRound * k;
          valid[k] = row < Dm + Gn;
          row_ptr[k] = nullptr;
          shift[k] = 0;
          dst_off[k] = 0;
          if (row < Dm) {
            row_ptr[k] = pm + order[d[kDetBegin] + m0 + row] * stride;
            dst_off[k] = (uint32_t)(row * kAtom) | ((uint32_t)(row & 7) << 24);
          } else if (valid[k]) {
            const int rb = row - Dm;
            row_ptr[k] = gm + (int64_t)(n0 + rb) * stride;
            dst_off[k] = (uint32_t)(rb * kAtom) | ((uint32_t)(rb & 7) << 24) | 0x80000000u;
          }
          if (valid[k]) {
            shift[k] = (int)(reinterpret_cast<uintptr_t>(row_ptr[k]) & 15);
            any |= shift[k] != 0;
          }
        }
        unaligned = __any_sync(0xffffffffu, any);
      }
      int64_t x_begin;
      const int stages = stages_of(blk, chunk, &x_begin);
      for (int st = 0; st < stages; ++st, ++seq) {
        const int slot = (int)(seq % kRing);
        const int64_t use = seq / kRing;
        const int64_t x0 = x_begin + (int64_t)st * kStagePixels + (int64_t)quarter * kLaneBytes;
        // Aligned words w[k][i] at row bytes x0 + 16 i - shift; w16[k]: the word after the stage (last quarter).
        uint4 w[kRounds][4], w16[kRounds];
#pragma unroll
        for (int k = 0; k < kRounds; ++k) {
          const int o = shift[k];
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int64_t start = x0 + 16 * i - o;
            w[k][i] = valid[k] && start < pixels ? __ldg(reinterpret_cast<const uint4*>(row_ptr[k] + start))
                                                 : make_uint4(0, 0, 0, 0);
          }
          const int64_t tail = x0 + kLaneBytes - o;
          w16[k] = valid[k] && quarter == kLanesPerRow - 1 && o && tail < pixels
                       ? __ldg(reinterpret_cast<const uint4*>(row_ptr[k] + tail))
                       : make_uint4(0, 0, 0, 0);
        }
        // The loads are in flight while this waits for the ring slot to be released.
        if (use > 0 && !wait_bar(&sm.empty[slot], (uint32_t)((use - 1) & 1), abort, error)) {
          ok = false;
          break;
        }
        uint8_t* tile_a = sm.a[slot][atom];
        uint8_t* tile_b = sm.b[slot][atom];
#pragma unroll
        for (int k = 0; k < kRounds; ++k) {
          uint4 next = w16[k];
          if (unaligned) {
            // First word of the next quarter of the same row (8 lanes up); the last quarter keeps w16.
            const uint4 up = make_uint4(__shfl_down_sync(0xffffffffu, w[k][0].x, kRowsPerWarp),
                                        __shfl_down_sync(0xffffffffu, w[k][0].y, kRowsPerWarp),
                                        __shfl_down_sync(0xffffffffu, w[k][0].z, kRowsPerWarp),
                                        __shfl_down_sync(0xffffffffu, w[k][0].w, kRowsPerWarp));
            if (quarter < kLanesPerRow - 1) next = up;
          }
          if (!valid[k]) continue;
          const uint32_t off = dst_off[k];
          uint8_t* dst = ((off & 0x80000000u) ? tile_b : tile_a) + (off & 0x00ffffffu);
          const int swz = (int)((off >> 24) & 7);
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            uint4 v = realign(w[k][i], i < 3 ? w[k][i + 1] : next, shift[k]);
            const int64_t left = pixels - (x0 + 16 * i);  // row bytes at or after this chunk
            if (left < 16) {
              const int keep = (int)max((int64_t)0, left);
              v.x &= keep_bytes(keep);
              v.y &= keep_bytes(keep - 4);
              v.z &= keep_bytes(keep - 8);
              v.w &= keep_bytes(keep - 12);
            }
            v.x *= kOne; v.y *= kOne; v.z *= kOne; v.w *= kOne;  // bytes are 0/1: no carries
            *reinterpret_cast<uint4*>(dst + (((c0 + i) ^ swz) << 4)) = v;
          }
        }
        fence_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive(&sm.full[slot]);
      }
    }
  } else {
    // ---- epilogue: accumulator -> integer totals -> global counters ----------
    const int row = warp * 32 + lane;
    Block blk;
    int64_t current = -1, interval = 0;
    bool ok = true;
    auto flush = [&](int64_t index) {
      const int64_t* r = blocks + index * kBlkFields;
      const int64_t* d = desc_of(descs, r[kBlkImage]);
      const int m0 = (int)r[kBlkM0], n0 = (int)r[kBlkN0];
      const int G = (int)d[kG];
      const int Dm = (int)min((int64_t)kRowsA, d[kD] - m0), Gn = (int)min((int64_t)kRowsB, (int64_t)G - n0);
      if (row < Dm) {
        u32* out = inter + d[kDPairBegin] + (int64_t)(m0 + row) * G + n0;
        for (int g = 0; g < Gn; ++g) {
          const u32 v = sm.totals[g * kM + row];
          if (v) atomicAdd(out + g, v);
        }
        const u32 area = sm.totals[kRowsB * kM + row];
        if (n0 == 0 && area) atomicAdd(pa + d[kDetBegin] + m0 + row, (u64)area);
      }
      if (row == kRowsA && m0 == 0) {
        for (int g = 0; g < Gn; ++g) {
          const u32 v = sm.totals[g * kM + row];
          if (v) atomicAdd(ga + d[kSlotBegin] + n0 + g, (u64)v);
        }
      }
#pragma unroll 8
      for (int col = 0; col < kN; ++col) sm.totals[col * kM + row] = 0;
    };
    for (int64_t chunk = c_begin; chunk < c_end && ok; ++chunk) {
      advance(blk, descs, blocks, n_blocks, chunk);
      if (blk.index != current) {
        if (current >= 0) flush(current);
        current = blk.index;
      }
      const int buf = (int)(interval & 1);
      const bool got = wait_bar(&sm.acc_full[buf], (uint32_t)((interval >> 1) & 1), abort, error);
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
#pragma unroll
      for (int col = 0; col < 32; ++col) {
        sm.totals[col * kM + row] += (u32)__float2uint_rz(__uint_as_float(v0[col]));
        sm.totals[(col + 32) * kM + row] += (u32)__float2uint_rz(__uint_as_float(v1[col]));
      }
      ++interval;
    }
    if (ok && current >= 0) flush(current);
  }

  tc_fence_before();
  __syncthreads();
  if (warp == kMmaWarp) {
    tc_fence_after();
    tmem_dealloc(tmem, kTmemCols);
  }
}

}  // namespace
}  // namespace pe

using namespace pe;

// Detection x target intersection counts and both mask areas for the batched
// InstanceEvaluator, on the tensor cores. descs: instance descriptor table
// (kMasks = prediction masks, kTarget = target masks, kMaskStride bytes per
// row, kDetBegin / kSlotBegin / kDPairBegin offsets); blocks: n_blocks rows of
// (image, first detection, first target, first chunk) with 127 x 63 tiles and
// ceil(pixels / 4096) chunks each, ordered by first chunk; order: score order
// from pe_seg_sort. inter (u32, sum D*G, rows in score order), pa (u64, sum D)
// and ga (u64, sum G) are zeroed here. Drop-in for the reference's
// pack_masks + overlap (instance_kernel.cu:10-39).
PE_API int pe_inst_contract(const int64_t* descs, const int64_t* blocks, int64_t n_blocks, int64_t total_chunks,
                            const int64_t* cta_bounds, int64_t ctas, const int64_t* order, uint32_t* inter,
                            int64_t inter_len, uint64_t* pa, int64_t pa_len, uint64_t* ga, int64_t ga_len,
                            int32_t* error, cudaStream_t stream) {
  PE_REQUIRE(n_blocks >= 0 && total_chunks >= 0 && inter_len >= 0 && pa_len >= 0 && ga_len >= 0, "invalid batch");
  PE_REQUIRE(n_blocks > 0 || total_chunks == 0, "chunks without blocks");
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
  inst_contract_kernel<<<(unsigned)grid, kThreads, smem, stream>>>(descs, blocks, n_blocks, total_chunks, per_cta,
                                                                    cta_bounds, order, reinterpret_cast<u32*>(inter),
                                                                    reinterpret_cast<u64*>(pa),
                                                                    reinterpret_cast<u64*>(ga), error);
  PE_LAUNCHED("inst_contract");
  count_launch();
  return kOk;
}
