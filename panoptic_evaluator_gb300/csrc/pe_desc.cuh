// Per-image descriptor table shared by the batched kernels: kDescFields int64
// values per image, built on the host (panoptic_evaluator_gb300/_batch.py).
#pragma once

#include "pe_common.cuh"

namespace pe {

// Descriptor fields (int64 each, kDescFields per image).
enum DescField : int {
  kTarget = 0,    // segmentation: int32 target slot map; instance: gt masks (uint8)
  kPred,          // int32 prediction slot map (segmentation)
  kMasks,         // detection masks, uint8 0/1, rows `kMaskStride` bytes apart (unsorted order)
  kPixels,
  kMaskStride,
  kChunkBegin,    // first work chunk of this image
  kDetBegin,      // offset into flat per-detection arrays
  kSlotBegin,     // offset into flat per-target-slot arrays
  kPSlotBegin,    // offset into flat per-prediction-slot arrays
  kPairBegin,     // offset of this image's G x P pair histogram
  kDPairBegin,    // offset of this image's D x G detection histogram
  kD,
  kG,
  kP,
  kFlags,         // bit 0: slot maps 16-byte vectorisable; bit 1: masks 16-byte vectorisable
  kReserved,
  kDescFields
};

__device__ __forceinline__ const int64_t* desc_of(const int64_t* descs, int64_t b) { return descs + b * kDescFields; }

// Image owning chunk `chunk` (binary search over kChunkBegin).
__device__ __forceinline__ int64_t image_of_chunk(const int64_t* descs, int64_t B, int64_t chunk) {
  int64_t lo = 0, hi = B - 1;
  while (lo < hi) {
    const int64_t mid = (lo + hi + 1) >> 1;
    if (descs[mid * kDescFields + kChunkBegin] <= chunk) lo = mid; else hi = mid - 1;
  }
  return lo;
}

}  // namespace pe
