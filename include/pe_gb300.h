/*
 * pe_gb300: C ABI of the GB300 (sm_103a) panoptic / instance evaluation kernels.
 *
 * Every entry point takes raw device pointers, int64 sizes and a cudaStream_t,
 * launches its kernels on that stream and returns an int status:
 *     0   success
 *    >0   validation bitmask, with the reference's bit meanings
 *         (1: unknown segment ID or slot outside capacity,
 *          2: class outside [-1, C) or slot 0 not void,
 *          4: non-void slot pixels and active metadata disagree;
 *          prefix: 1 unknown target slot, 2 empty prediction mask)
 *    <0   argument error (-1), CUDA error (-2), workspace too small (-3),
 *         unsupported configuration (-4); pe_last_error() holds the text.
 * Boolean tensors are one byte per element (0 or 1). Counts that the
 * reference keeps as int64 are int64 here too. No entry point allocates
 * device memory: state, scratch and workspaces belong to the caller.
 * Calls that pass validate = 0 never block the host and may be captured in a
 * CUDA graph; validate = 1 reads the error word back and synchronises the
 * stream once, as the reference does.
 *
 * References below are to files of AndyBarcia/panoptic-evaluator.
 */
#ifndef PE_GB300_H
#define PE_GB300_H

#include <stdint.h>
#include <cuda_runtime_api.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- runtime ------------------------------------------------------------ */

/* Text of the last failure on the calling host thread. */
const char* pe_last_error(void);
/* Kernels launched by this library since load or the last reset. */
long long pe_launch_count(void);
void pe_reset_launch_count(void);
int pe_abi_version(void);

/* ---- panoptic quality / semantic confusion ------------------------------ */

/*
 * Replaces the `update` op: panoptic_evaluator/csrc/bindings.cpp:29-48,
 * update_cuda in panoptic_evaluator/csrc/histogram_kernel.cu:257-341.
 * gt/pred: B x pixels maps, int32 or int64 (flag *_is_int64), compact slots or
 * original IDs when the matching *_ids/*_slots tables (B x G / B x P, sorted
 * int64 IDs and int32 slots) are given. gc/pc: B x G / B x P int32 classes,
 * crowd: B x G bool. Scratch: pairs B x G x P int64 (histogram), areas
 * B x (G+P) int64 (row then column sums; valid after return), matched B x G
 * int32. State: tp/fp/fn int64 and iou_sum f64, [C] (dataset) or [B, C]
 * (reward = 1); confusion C x (C+1) int64 (dataset only, may be NULL for
 * reward). With validate, totals are left untouched when a bit is set.
 */
int pe_update(const void* gt, int gt_is_int64, const void* pred, int pred_is_int64, int64_t B,
              int64_t pixels, const int32_t* gc, const int32_t* pc, const uint8_t* crowd, int64_t G,
              int64_t P, int64_t C, int64_t* pairs, int64_t* areas, int32_t* matched, int64_t* tp,
              int64_t* fp, int64_t* fn, double* iou_sum, int64_t* confusion, const int64_t* gt_ids,
              const int32_t* gt_slots, const int64_t* pred_ids, const int32_t* pred_slots, int32_t* error,
              int validate, int reward, cudaStream_t stream);

/*
 * Replaces the `compute` op and compute_prefix_cuda:
 * panoptic_evaluator/csrc/compute_kernel.cu:66-118, bindings.cpp:49.
 * K rows of tp/fp/fn/sums [K, C] and confusion [K, C, C+1]; things [C] bool.
 * Outputs per_class [K, 4, C] (pq, sq, rq, iou), summaries [K, 3, 3]
 * (All/Things/Stuff x pq/sq/rq), counts [K, 3], miou [K], and copies of the
 * inputs in out_* (skipped when out_tp is NULL).
 */
int pe_compute(const int64_t* tp, const int64_t* fp, const int64_t* fn, const double* sums,
               const int64_t* confusion, const uint8_t* things, int64_t K, int64_t C, double* per_class,
               double* summaries, int64_t* counts, double* miou, int64_t* out_tp, int64_t* out_fp,
               int64_t* out_fn, double* out_sums, int64_t* out_confusion, cudaStream_t stream);

/*
 * Replaces the `pack` op: panoptic_evaluator/csrc/histogram_kernel.cu:343-366,
 * bindings.cpp:50. Original IDs -> compact int32 slots through sorted B x S
 * lookup tables; *error (device int) gets bit 1 for IDs absent from the tables.
 */
int pe_pack(const void* maps, int maps_is_int64, int64_t B, int64_t pixels, const int64_t* ids,
            const int32_t* slots, int64_t S, int32_t* out, int32_t* error, cudaStream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* PE_GB300_H */
