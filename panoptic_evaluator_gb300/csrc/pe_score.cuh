// Per-image PQ scoring from a G x P pair histogram, shared by the per-call
// update (pe_panoptic.cu) and the batched segmentation pipeline.
//
// Semantics follow the reference (histogram_kernel.cu:100-206; CPU
// evaluator.py:381-417): union = ga + pa - inter - void_overlap, a match iff
// same class, non-crowd target and inter > union / 2 (integer), IoU in FP64,
// the last same-class crowd target sets the ignored area, FP iff ignored
// <= pa / 2, FN for unmatched non-crowd targets. Class sums of one image are
// reduced in prediction order, so per-image results do not depend on timing.
#pragma once

#include "pe_common.cuh"

namespace pe {

struct ScoreOut {
  u64* tp;          // [C] (+ image offset applied by the caller in reward mode)
  u64* fp;
  u64* fn;
  double* iou_sum;
  u64* confusion;   // C x (C+1), or nullptr
};

// Row and column sums into areas[0..G) / areas[G..G+P), plus validation bits.
template <typename Count, bool REWARD>
__device__ int score_areas(const Count* __restrict__ pairs, const int* __restrict__ gc, const int* __restrict__ pc,
                           const uint8_t* __restrict__ crowd, u64* __restrict__ areas, int G, int P, int C,
                           bool validate) {
  int err = 0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
  for (int g = warp; g < G; g += warps) {
    u64 sum = 0;
    for (int p = lane; p < P; p += 32) sum += (u64)pairs[(int64_t)g * P + p];
#pragma unroll
    for (int o = 16; o; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if (lane == 0) {
      areas[g] = sum;
      if (validate) {
        const int c = gc[g];
        if (c < -1 || c >= C || (g == 0 && (c != -1 || crowd[g]))) err |= 2;
        if (g > 0 && ((sum > 0) != (c >= 0))) err |= 4;
      }
    }
  }
  for (int p = threadIdx.x; p < P; p += blockDim.x) {
    u64 sum = 0;
    for (int g = 0; g < G; ++g) sum += (u64)pairs[(int64_t)g * P + p];
    areas[G + p] = sum;
    if (validate) {
      const int c = pc[p];
      if (c < -1 || c >= C || (p == 0 && c != -1)) err |= 2;
      if (p > 0 && (REWARD ? (sum > 0 && c < 0) : ((sum > 0) != (c >= 0)))) err |= 4;
    }
  }
  return err;
}

// Accumulate one image. Needs areas from score_areas (after a barrier), a
// G-entry `matched` scratch, and shared staging of P * 13 bytes.
template <typename Count, bool REWARD>
__device__ void score_accumulate(const Count* __restrict__ pairs, const int* __restrict__ gc,
                                 const int* __restrict__ pc, const uint8_t* __restrict__ crowd,
                                 const u64* __restrict__ areas, int* __restrict__ matched, int G, int P, int C,
                                 ScoreOut out, unsigned char* staging) {
  for (int g = threadIdx.x; g < G; g += blockDim.x) matched[g] = 0;
  __syncthreads();
  double* s_sum = reinterpret_cast<double*>(staging);
  int* s_cls = reinterpret_cast<int*>(s_sum + P);
  unsigned char* s_kind = reinterpret_cast<unsigned char*>(s_cls + P);
  for (int p = threadIdx.x; p < P; p += blockDim.x) {
    const int prediction = pc[p];
    const bool vp = prediction >= 0 && prediction < C;
    const u64 void_overlap = (u64)pairs[p];
    const u64 pa = areas[G + p];
    u64 ignored = void_overlap;
    bool pm = false;
    double sum = 0.0;
    for (int g = 0; g < G; ++g) {
      const int target = gc[g];
      const u64 inter = (u64)pairs[(int64_t)g * P + p];
      const bool vt = target >= 0 && target < C;
      if (!REWARD && out.confusion && vt && inter && !crowd[g])
        atomicAdd(out.confusion + (int64_t)target * (C + 1) + (vp ? prediction : C), inter);
      if (!vt || !vp || target != prediction) continue;
      if (crowd[g]) {
        ignored = void_overlap + inter;  // the last same-class crowd segment wins
      } else if (inter) {
        const u64 uni = areas[g] + pa - inter - void_overlap;
        if (inter > uni / 2) {
          pm = true;
          sum += (double)inter / (double)uni;
          matched[g] = 1;
        }
      }
    }
    const bool counted = vp && (!REWARD || pa > 0);
    s_cls[p] = counted ? prediction : -1;
    // ignored <= pa / 2 (the reference's FP64 test) is exactly 2 * ignored <= pa for integer counts.
    s_kind[p] = pm ? 1 : ((2 * ignored <= pa) ? 2 : 0);
    s_sum[p] = sum;
  }
  __syncthreads();
  for (int c = threadIdx.x; c < C; c += blockDim.x) {
    u64 ntp = 0, nfp = 0;
    double total = 0.0;
    for (int p = 0; p < P; ++p) {
      if (s_cls[p] != c) continue;
      if (s_kind[p] == 1) {
        ++ntp;
        total += s_sum[p];
      } else if (s_kind[p] == 2) {
        ++nfp;
      }
    }
    if (ntp) {
      atomicAdd(out.tp + c, ntp);
      atomicAdd(out.iou_sum + c, total);
    }
    if (nfp) atomicAdd(out.fp + c, nfp);
  }
  for (int g = threadIdx.x; g < G; g += blockDim.x) {
    const int c = gc[g];
    if (c >= 0 && c < C && !crowd[g] && !matched[g]) atomicAdd(out.fn + c, 1ull);
  }
}

// score_accumulate over a histogram staged in shared memory `h`: one warp per
// prediction, lanes over targets. Targets are disjoint slots of one map, so at
// most one non-crowd target has inter > union / 2 with a prediction (two would
// need inter_1 + inter_2 > pa - void_overlap >= inter_1 + inter_2): the
// reference's per-prediction sum has one term, and the last same-class crowd
// target is the largest such index over the warp. Same results as
// score_accumulate.
template <bool REWARD>
__device__ void score_accumulate_warps(const u32* h, const int* __restrict__ gc, const int* __restrict__ pc,
                                       const uint8_t* __restrict__ crowd, const u64* __restrict__ areas,
                                       int* __restrict__ matched, int G, int P, int C, ScoreOut out,
                                       unsigned char* staging) {
  for (int g = threadIdx.x; g < G; g += blockDim.x) matched[g] = 0;
  __syncthreads();
  double* s_sum = reinterpret_cast<double*>(staging);
  int* s_cls = reinterpret_cast<int*>(s_sum + P);
  unsigned char* s_kind = reinterpret_cast<unsigned char*>(s_cls + P);
  const int lane = threadIdx.x & 31, warps = blockDim.x >> 5;
  for (int p = threadIdx.x >> 5; p < P; p += warps) {
    const int prediction = pc[p];
    const bool vp = prediction >= 0 && prediction < C;
    const u64 void_overlap = h[p];
    const u64 pa = areas[G + p];
    int last_crowd = -1, match = -1;
    double iou = 0.0;
    for (int g = lane; g < G; g += 32) {
      const int target = gc[g];
      const u64 inter = h[(int64_t)g * P + p];
      const bool vt = target >= 0 && target < C;
      if (!REWARD && out.confusion && vt && inter && !crowd[g])
        atomicAdd(out.confusion + (int64_t)target * (C + 1) + (vp ? prediction : C), inter);
      if (!vt || !vp || target != prediction) continue;
      if (crowd[g]) {
        last_crowd = g;
      } else if (inter) {
        const u64 uni = areas[g] + pa - inter - void_overlap;
        if (inter > uni / 2) {
          match = g;
          iou = (double)inter / (double)uni;
        }
      }
    }
    if (match >= 0) matched[match] = 1;
    last_crowd = __reduce_max_sync(0xffffffffu, last_crowd);
    const u32 matches = __ballot_sync(0xffffffffu, match >= 0);
    iou = __shfl_sync(0xffffffffu, iou, matches ? __ffs(matches) - 1 : 0);
    if (lane == 0) {
      const u64 ignored = last_crowd >= 0 ? void_overlap + h[(int64_t)last_crowd * P + p] : void_overlap;
      const bool counted = vp && (!REWARD || pa > 0);
      s_cls[p] = counted ? prediction : -1;
      s_kind[p] = matches ? 1 : ((2 * ignored <= pa) ? 2 : 0);
      s_sum[p] = matches ? 0.0 + iou : 0.0;
    }
  }
  __syncthreads();
  for (int c = threadIdx.x; c < C; c += blockDim.x) {
    u64 ntp = 0, nfp = 0;
    double total = 0.0;
    for (int p = 0; p < P; ++p) {
      if (s_cls[p] != c) continue;
      if (s_kind[p] == 1) {
        ++ntp;
        total += s_sum[p];
      } else if (s_kind[p] == 2) {
        ++nfp;
      }
    }
    if (ntp) {
      atomicAdd(out.tp + c, ntp);
      atomicAdd(out.iou_sum + c, total);
    }
    if (nfp) atomicAdd(out.fp + c, nfp);
  }
  for (int g = threadIdx.x; g < G; g += blockDim.x) {
    const int c = gc[g];
    if (c >= 0 && c < C && !crowd[g] && !matched[g]) atomicAdd(out.fn + c, 1ull);
  }
}

inline size_t score_staging_bytes(int64_t P) { return (size_t)P * (sizeof(double) + sizeof(int) + 1) + 16; }

// Copies n counts of one image's histogram (global, any 4-byte offset) into
// shared memory with every thread holding kStageLoads loads in flight: a copy
// of one load per thread and trip waits one L2 round trip per
// blockDim.x words. The caller synchronises the block afterwards.
constexpr int kStageLoads = 8;

__device__ __forceinline__ void stage_counts(u32* __restrict__ dst, const u32* __restrict__ src, int n) {
  for (int i0 = threadIdx.x; i0 < n; i0 += kStageLoads * blockDim.x) {
    u32 v[kStageLoads];
#pragma unroll
    for (int j = 0; j < kStageLoads; ++j) {
      const int i = i0 + j * (int)blockDim.x;
      v[j] = i < n ? src[i] : 0u;
    }
#pragma unroll
    for (int j = 0; j < kStageLoads; ++j) {
      const int i = i0 + j * (int)blockDim.x;
      if (i < n) dst[i] = v[j];
    }
  }
}

}  // namespace pe
