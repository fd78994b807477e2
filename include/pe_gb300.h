/*
 * pe_gb300: C ABI of the GB300 (sm_103a) panoptic / instance evaluation kernels.
 *
 * Every device entry point takes raw device pointers, int64 sizes and a
 * cudaStream_t, launches its kernels on that stream and returns an int status
 * (the host-side planning calls pe_contract_maps and pe_contract_blocks take
 * host arrays, launch nothing and return a count or a negative error; the
 * size queries return sizes):
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
/* Diagnostics, no reference counterpart: one thread waits on an mbarrier with the
 * bounded wait every pipelined kernel here uses (complete = 0: nothing arrives),
 * giving up after limit_cycles SM clock cycles (1..2^32); *error is zeroed, then
 * bit 30 is set on a timeout. Shows on the device that a wait that never
 * completes ends with an error status and leaves the context usable. */
int pe_wait_selftest(int64_t limit_cycles, int complete, int32_t* error, cudaStream_t stream);

/* ---- panoptic quality / semantic confusion ------------------------------ */

/* Tuning of the per-call update (no reference counterpart; the reference reads
 * PANOPTIC_HISTOGRAM and PANOPTIC_SCORING on every call,
 * panoptic_evaluator/csrc/histogram_kernel.cu:240-246,309-310). For the bucket
 * of (floor(log2(G * P)), floor(log2(pixels per image))) record shared (1) or
 * global (0) histogram bins, histogram CTAs per SM (1..4) and threads of the
 * per-image scoring CTA (256, 512, 1024); smem < 0 removes the entry (the
 * built-in rule applies again). A choice never exceeds what a launch can hold
 * (shared bins only when G * P fits). pe_update_choice reports the choice a
 * launch of that shape uses. */
int pe_tune_update(int64_t bins, int64_t pixels, int smem, int ctas_per_sm, int score_threads);
int pe_update_choice(int64_t bins, int64_t pixels, int32_t* smem, int32_t* ctas_per_sm, int32_t* score_threads);

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
 * Mean-class PQ per image from [B, C] reward statistics (the tail of
 * panoptic_quality, panoptic_evaluator/evaluator.py:539-544) into pq[B]. When
 * tot_tp is not NULL the statistics are also added into dataset totals [C]
 * (tot_tp/tot_fp/tot_fn int64, tot_sums f64).
 */
int pe_reward_pq(const int64_t* tp, const int64_t* fp, const int64_t* fn, const double* sums, int64_t B, int64_t C,
                 double* pq, int64_t* tot_tp, int64_t* tot_fp, int64_t* tot_fn, double* tot_sums, cudaStream_t stream);

/*
 * Replaces the `pack` op: panoptic_evaluator/csrc/histogram_kernel.cu:343-366,
 * bindings.cpp:50. Original IDs -> compact int32 slots through sorted B x S
 * lookup tables; *error (device int) gets bit 1 for IDs absent from the tables.
 */
int pe_pack(const void* maps, int maps_is_int64, int64_t B, int64_t pixels, const int64_t* ids,
            const int32_t* slots, int64_t S, int32_t* out, int32_t* error, cudaStream_t stream);

/*
 * COCO panoptic PNG pixels straight to compact slots: no counterpart op in the
 * reference, whose README (README.md:68) asks callers to decode RGB PNGs as
 * R + 256*G + 65536*B before PanopticBatch.from_coco (evaluator.py:33-106).
 * rgb is B x pixels x 3 uint8 (the decoded PNG, PNG decompression stays on the
 * host); with lookup tables (as for pe_pack) out gets int32 slots and *error
 * bit 1 for absent IDs, with ids = slots = NULL out gets the int32 IDs.
 */
int pe_pack_rgb(const uint8_t* rgb, int64_t B, int64_t pixels, const int64_t* ids, const int32_t* slots, int64_t S,
                int32_t* out, int32_t* error, cudaStream_t stream);

/*
 * pe_update without caller-provided scratch. No counterpart in the reference:
 * it exists for callers that cannot call cudaMalloc (device memory owned by
 * another runtime's allocator, or a loop where an allocation would
 * synchronise the device). Same arguments and results as pe_update minus
 * pairs/areas/matched/error; the scratch comes from one fixed 8 MiB array in
 * this library's device memory (held on every GPU that loads the library), so
 * 8*B*G*P + 8*B*(G+P) + 4*B*G bytes (+ alignment) must fit in 8 MiB or -1 is
 * returned. All calls share that array: calls that overlap on the GPU race.
 * The first call on each device (and the first after the device's context is
 * recreated, as by cudaDeviceReset) looks up the array's address; make it
 * before any stream capture on that device.
 */
int pe_update_noalloc(const void* gt, int gt_is_int64, const void* pred, int pred_is_int64, int64_t B,
                      int64_t pixels, const int32_t* gc, const int32_t* pc, const uint8_t* crowd, int64_t G,
                      int64_t P, int64_t C, int64_t* tp, int64_t* fp, int64_t* fn, double* iou_sum,
                      int64_t* confusion, const int64_t* gt_ids, const int32_t* gt_slots, const int64_t* pred_ids,
                      const int32_t* pred_slots, int validate, int reward, cudaStream_t stream);

/* ---- instance segmentation (COCO mask AP/AR) ----------------------------- */

/*
 * Replaces `instance_histogram`: panoptic_evaluator/csrc/instance_kernel.cu:335-363.
 * masks: D x pixels uint8 0/1, target: pixels int32 slot map, order: D int64
 * (row r of the output counts mask order[r]). pairs: D x S int64, zeroed here.
 */
int pe_instance_histogram(const uint8_t* masks, int64_t D, int64_t pixels, const int32_t* target,
                          const int64_t* order, int64_t S, int64_t* pairs, cudaStream_t stream);

/*
 * Replaces `instance_match_histogram` (instance_kernel.cu:365-381) and the
 * matching half of `instance_update` (instance_kernel.cu:153-174, 282-309):
 * COCO greedy matching (instance.py:267-297) of D score-sorted detections
 * against G targets from int64 intersections pairs[D, G]. Outputs flags
 * [40, D] int8, ranks [D] int32 (1..100 within class, 0 beyond the cap),
 * counts [C, 4] int64 positives (zeroed here).
 */
int pe_instance_match(const int64_t* pairs, int64_t D, int64_t G, const int32_t* pc, const int32_t* gc,
                      const double* pa, const double* ga, const uint8_t* crowd, const double* areas, int64_t C,
                      int8_t* flags, int32_t* ranks, int64_t* counts, cudaStream_t stream);

/*
 * Mask intersections of `instance_update` (pack_masks + overlap,
 * instance_kernel.cu:10-39): inter[d, g] = |pm[d] & gm[g]| when pc[d] ==
 * gc[g], else 0. pm: D x pixels, gm: G x pixels uint8 0/1. inter zeroed here.
 */
int pe_mask_overlap(const uint8_t* pm, int64_t D, const uint8_t* gm, int64_t G, int64_t pixels,
                    const int32_t* pc, const int32_t* gc, int64_t* inter, cudaStream_t stream);

/* Workspace bytes for pe_instance_accumulate over n records and C classes. */
int64_t pe_instance_accumulate_workspace(int64_t n, int64_t C);

/*
 * Replaces `instance_compute` (instance_kernel.cu:176-209, 311-333; CPU
 * instance.py:300-331) when scores == NULL: records already in global
 * descending-score order. With scores, records are in update order and are
 * sorted here per class (descending score, then record order), which is the
 * reference's global stable argsort (instance.py:209-215). flags are read at
 * flags[chain * chain_stride + record * det_stride]. Writes precision
 * [10, 101, C, 4, 3] and recall [10, C, 4, 3] in full (-1 where unavailable) and, when summary
 * is not NULL, the 12 summaries of pe_instance_summarize into summary[12].
 */
int pe_instance_accumulate(const int32_t* classes, const int32_t* ranks, const int8_t* flags, int64_t chain_stride,
                           int64_t det_stride, const double* scores, int64_t n, const int64_t* positives, int64_t C,
                           void* workspace, int64_t workspace_bytes, double* precision, double* recall,
                           double* summary, cudaStream_t stream);

/*
 * The 12 AP/AR summaries of instance.py:230-248 into out[12]: ap, ap50, ap75,
 * ap_small, ar_small, ap_medium, ar_medium, ap_large, ar_large, ar1, ar10, ar100.
 */
int pe_instance_summarize(const double* precision, const double* recall, int64_t C, double* out,
                          cudaStream_t stream);

/* ---- batched segmentation pipeline (descriptor table) -------------------- */
/*
 * These replace the per-image Python loops of combined.py:90-160 and
 * instance.py:188-202 with a fixed number of launches per batch. The table
 * holds pe_desc_fields() int64 per image: target map (or gt masks), prediction
 * map, detection masks, pixels, mask row stride, first work chunk, and the
 * offsets of the image in the flat per-detection / per-slot / per-pair arrays,
 * then D, G, P and alignment flags (see panoptic_evaluator_gb300/csrc/pe_segmentation.cu).
 */
int pe_desc_fields(void);
int64_t pe_seg_sort_workspace(int64_t total_detections);
int pe_seg_sort(const int64_t* descs, int64_t B, const double* scores, const int32_t* classes,
                int64_t total_detections, int64_t* order, double* sorted_scores, int32_t* sorted_classes,
                void* workspace, int64_t workspace_bytes, cudaStream_t stream);
/* bulk = 1 or 2 streams mask segments through a cp.async.bulk ring (a wait that times out sets bit 30
 * of *error): 1 when every mask row starts on a 16-byte boundary, 2 for rows at any byte offset (the
 * aligned words covering each segment are copied and re-aligned in the pass); 0 reads them with plain
 * loads.
 * cta_bounds (optional, ctas + 1 int64 chunk indices in device memory) gives each CTA a contiguous
 * chunk range, for example of equal bytes; NULL splits the chunks evenly (2 CTAs per SM when bulk).
 * schedule (bulk only, optional): one device uint64, zeroed here, from which the CTAs take chunks
 * dynamically (cta_bounds unused): by default 2 CTAs per SM taking one 8192-pixel chunk per grab, or
 * the choice recorded by pe_tune_pass for this batch size; results do not depend on which CTA took
 * which chunk. */
/* Tuning of the batched pass with a chunk counter (no reference counterpart: the reference has no
 * batched pass). For the bucket floor(log2(total_chunks)) record the chunks a producer takes per
 * counter grab (1, 2 or 4) and CTAs per SM (1 or 2); grab < 0 removes the entry. pe_pass_choice
 * reports the choice a launch of that size uses. */
int pe_tune_pass(int64_t chunks, int grab, int ctas_per_sm);
int pe_pass_choice(int64_t chunks, int32_t* grab, int32_t* ctas_per_sm);
int pe_seg_pass(const int64_t* descs, int64_t B, int64_t total_chunks, const int64_t* order, uint32_t* pairs,
                int64_t pairs_len, uint32_t* dpairs, int64_t dpairs_len, int64_t pan_cap, int64_t det_cap,
                int bulk, const int64_t* cta_bounds, int64_t ctas, uint64_t* schedule, int32_t* error,
                cudaStream_t stream);
/* max_p: largest P of the batch; max_pairs: largest G x P (each image's histogram is staged in shared
 * memory when the largest fits 100 KB, else read in place; the results are the same). class_bits
 * (optional, B x ceil(C / 32) u32): each image's classes with detections or thing targets, for
 * pe_seg_match (a detection class outside [0, C) marks class 0). */
int pe_seg_score(const int64_t* descs, int64_t B, int64_t max_p, int64_t max_pairs, const uint32_t* pairs,
                 const uint32_t* dpairs,
                 const int32_t* gc, const int32_t* pc, const uint8_t* crowd, int64_t* areas, int32_t* matched,
                 int64_t* tp, int64_t* fp, int64_t* fn, double* iou_sum, int64_t* confusion, int64_t C,
                 const uint8_t* isthing, const int32_t* det_classes, const double* det_scores, double* det_pa,
                 double* slot_ga, int32_t* slot_class, const double* ann_in, double* ann_out, int validate,
                 int reward, uint32_t* class_bits, int32_t* error, cudaStream_t stream);
/* class_bits (optional): pe_seg_score's per-image class bits; classes absent from an image are skipped. */
int pe_seg_match(const uint32_t* pairs, const int64_t* pair_off, const int64_t* d_off, const int64_t* g_off,
                 int64_t B, const int32_t* pc, const double* pa, const int32_t* gc, const double* ga,
                 const uint8_t* crowd, const double* areas, int64_t C, int64_t g_max, int8_t* flags,
                 int64_t chain_stride, int64_t det_stride, int32_t* ranks, int64_t* counts, const int32_t* gate,
                 const uint32_t* class_bits, cudaStream_t stream);
int pe_inst_overlap(const int64_t* descs, int64_t B, int64_t total_chunks, int64_t max_rows, const int64_t* order,
                    const int32_t* pc, const int32_t* gc, uint32_t* inter, int64_t inter_len, uint64_t* pa,
                    int64_t pa_len, uint64_t* ga, int64_t ga_len, cudaStream_t stream);
/*
 * Tensor-core form of the same counts (replaces pack_masks + overlap,
 * panoptic_evaluator/csrc/instance_kernel.cu:10-39): every detection x target
 * intersection, both mask areas, as a tcgen05 kind::f8f6f4 contraction over
 * the 0/1 mask bytes read as e4m3 (exact: fp32 sums of 2^-18 products read
 * back at most every 2^22 pixels). blocks holds
 * n_blocks rows of 4 int64 (image, first detection, first target, first chunk)
 * covering each image with 127 x 63 tiles (detections and targets in mask
 * order) of ceil(pixels / 4096) chunks, ordered by first chunk. inter rows and
 * pa follow the score order of pe_seg_sort (order). cta_bounds (optional,
 * ctas + 1 int64 chunk indices, device memory) gives each CTA a contiguous
 * chunk range; NULL splits chunks evenly over the SMs. maps (optional, device
 * memory, 64-byte aligned): pe_contract_maps' tensor maps for the same table;
 * images whose descriptor flags bit 2 is set are then loaded by TMA, the others
 * are staged and re-aligned by worker warps (same counts either way); in chunk
 * order every TMA block must follow every staged block (else bit 28 of *error
 * is set and the call stops). A wait that times out sets bit 30 of *error and
 * bit 20 + the wait's site (0-5).
 */
int pe_inst_contract(const int64_t* descs, const int64_t* blocks, int64_t n_blocks, int64_t total_chunks,
                     const int64_t* cta_bounds, int64_t ctas, const int64_t* order, uint32_t* inter,
                     int64_t inter_len, uint64_t* pa, int64_t pa_len, uint64_t* ga, int64_t ga_len, const void* maps,
                     int32_t* error, cudaStream_t stream);
/*
 * Host-side companion of pe_inst_contract (no GPU work): for each image of the
 * HOST descriptor table whose mask rows start on 16-byte boundaries (flags
 * bit 1), with detections and targets, encodes two CUtensorMap (detection
 * masks, box 127 x 128 bytes; target masks, box 63 x 128; 128-byte swizzle)
 * into maps (host, B x 256 bytes, 64-byte aligned) and sets flags bit 2.
 * Returns the number of images given maps.
 */
int pe_contract_maps(int64_t* descs, int64_t B, void* maps);
/*
 * Host-side planning of pe_inst_contract (no GPU work): the block table
 * (image, first detection, first target, first chunk) covering B images of
 * dets[b] / gts[b] masks and pixels[b] pixels with 127 x 63 tiles of
 * ceil(pixels / 4096) chunks, staged images first and images with tma[b] != 0
 * (optional) after them, at most blocks_cap rows; *total_chunks receives the
 * chunk count. With ctas > 0, bounds (ctas + 1 int64) receives R + 1 chunk
 * indices, R = max(1, min(ctas, chunks)) in *ranges, splitting the chunks into
 * contiguous ranges of about equal cost (pixels x (rows + 8), TMA blocks
 * weighted by tma_cost): pe_inst_contract's cta_bounds. Returns the number of
 * blocks (negative: error). Plans the work of the reference's per-image
 * instance_update loop (panoptic_evaluator/instance.py:187-201) for one launch.
 */
int64_t pe_contract_blocks(const int64_t* dets, const int64_t* gts, const int64_t* pixels, const uint8_t* tma,
                           int64_t B, double tma_cost, int64_t ctas, int64_t* blocks, int64_t blocks_cap,
                           int64_t* bounds, int64_t* total_chunks, int64_t* ranges);
/*
 * The per-image metadata of an instance update gathered into flat arrays (no reference counterpart:
 * replaces the host-side concatenations of instance.py:188-202). fields: B rows of 6 int64: device
 * pointers of each image's prediction classes, scores, target classes, crowd flags and annotation
 * areas (0: absent), then element-size bits (1: prediction classes int64, 2: scores float64, 4: target
 * classes int64, 16: areas float64; else int32 / float32). Outputs at each image's detection and slot
 * offsets of the descriptor table: pc, scores [sum D]; gc, crowd, areas [sum G] (areas may be NULL).
 */
int pe_inst_gather(const int64_t* descs, const int64_t* fields, int64_t B, int32_t* pc, double* scores,
                   int32_t* gc, uint8_t* crowd, double* areas, cudaStream_t stream);
/* class_bits (optional, B x ceil(C / 32) u32): each image's detection and target classes, for
 * pe_seg_match (a detection class outside [0, C) marks class 0). */
int pe_inst_prepare(const int64_t* descs, int64_t B, const uint64_t* pa_count, const uint64_t* ga_count, double* pa,
                    double* ga, const int32_t* pc, const int32_t* gc, const double* scores, const double* ann_in,
                    double* ann_out, int64_t C, int validate, uint32_t* class_bits, int32_t* error,
                    cudaStream_t stream);

/* ---- generation-order prefixes ------------------------------------------ */

/*
 * Replaces the `prefix` op (panoptic_evaluator/csrc/prefix_kernel.cu:142-199,
 * compute_prefix_cuda in compute_kernel.cu:98-118) and the per-image loop of
 * prefix.py:50-121, for any number of images in one call. The descriptor
 * table holds pe_prefix_desc_fields() int64 per image (target map, masks in
 * generation order, pixels, mask row stride, first 4096-pixel chunk, N, G,
 * offsets into the flat per-mask / per-slot / per-checkpoint / histogram /
 * counter arrays, alignment flags); step_q holds, per image, N+1 ints: the
 * checkpoint index of prefix k or -1. Workspaces: ga [sum G] u32, raw
 * [sum N*G] u32, pairs [sum Q*G*(N+1)] int32, all zeroed here; counters
 * [B*T*C*2] int32 is reserved (zeroed when given; NULL with counters_len 0
 * is accepted): the greedy matching keeps its counters in shared memory. Per checkpoint row (R = sum Q): tp/fp/fn [R,C] int64, sums
 * [R,C] f64, confusion [R,C,C+1] int64, itp/ifp/ifn [R,T,C] int64,
 * precision/recall [R,T,C] f64, per_class [R,4,C], summaries [R,3,3],
 * counts [R,3], miou [R]. With validate the call returns the error bits:
 * 1 unknown target slot, 2 empty prediction mask, 4 bad target class or slot
 * 0 not void, 8 target areas vs metadata, 16 bad prediction class.
 * bulk = 1 streams each mask's segment of every 4096-pixel chunk through a
 * cp.async.bulk ring (rows at any alignment; a wait that times out sets bit 30
 * of *error); 0 reads the masks with plain loads. schedule (bulk only,
 * optional): one device uint64, zeroed here, from which two CTAs per SM take
 * chunks dynamically; NULL gives each CTA a contiguous range.
 */
int pe_prefix_desc_fields(void);
int pe_prefix(const int64_t* descs, int64_t B, int64_t total_chunks, int64_t total_rows, int64_t max_g,
              int64_t max_p, int64_t max_cells, const int32_t* step_q, const int32_t* classes, const int32_t* gc,
              const uint8_t* crowd, const uint8_t* isthing, const double* thresholds, int64_t T, int64_t C,
              uint32_t* ga, int64_t ga_len, uint32_t* raw, int64_t raw_len, int32_t* pairs, int64_t pairs_len,
              int32_t* counters, int64_t counters_len, int64_t* tp, int64_t* fp, int64_t* fn, double* sums,
              int64_t* confusion, int64_t* itp, int64_t* ifp, int64_t* ifn, double* precision, double* recall,
              double* per_class, double* summaries, int64_t* counts, double* miou, int validate, int bulk,
              uint64_t* schedule, int32_t* error, cudaStream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* PE_GB300_H */
