/*
 * grand_engine.h -- batched, mixed-code decoding with device-resident codes.
 *
 * No upstream counterpart: upstream decodes one code per call with a serial
 * host loop over shots (grand_decoder.cu:885, 1199, 1466, 1762, 2073).  An
 * engine keeps any number of registered codes resident on the GPU and decodes
 * batches whose shots may use different codes in one persistent launch (its
 * warps classify shots, triage the hard ones and search the heaviest, work
 * stealing from each other), optionally replayed from a captured CUDA graph.  Results are identical to the five grand_decode_* calls on the
 * same shots.
 *
 * Shot records are int32 0/1 rows: the syndrome (n entries) or the error (m
 * entries) for CSS codes, as chosen at registration; the detectors followed by
 * the true logical flips (n + n_logicos entries) for DEM codes.
 */
#ifndef GRAND_ENGINE_H
#define GRAND_ENGINE_H

#include "grand_decoder.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct GrandEngine GrandEngine;

/* Variant selector for grand_engine_add_dem. */
#define GRAND_VARIANT_UNIFORM 0
#define GRAND_VARIANT_PROB    1
#define GRAND_VARIANT_ML      2

/* Create an engine on the current CUDA device. */
int grand_engine_create(GrandEngine **engine);
void grand_engine_destroy(GrandEngine *engine);

/* Register a CSS code.  probability_file == NULL selects the uniform search
 * (grand_decode_cc), otherwise the phase-ordered one (grand_decode_prob_cc).
 * records_are_errors != 0: records hold errors (m entries), else syndromes. */
int grand_engine_add_css(GrandEngine *engine, const int *Hx, const int *Hz, int n, int m,
                         char type_of_error, int records_are_errors,
                         const GrandDecoderConfig *config, const char *probability_file,
                         int *code_id);

/* Register a DEM code (grand_decode_cln / _prob_cln / _ML_cln semantics);
 * file is the phase-mask file (PROB) or the LLR file (ML), else NULL. */
int grand_engine_add_dem(GrandEngine *engine, const int *H_dem, const int *L_dem, int n, int m,
                         int n_logicos, const GrandDecoderConfig *config, int variant,
                         const char *file, int *code_id);

/* int32 entries per shot record of a registered code (or < 0). */
int grand_engine_record_len(GrandEngine *engine, int code_id);

/* On-device shot generation (no upstream counterpart; upstream draws shots in
 * Python).  Draws num_shots shots of code `code_id`: every error position (CSS:
 * qubit, DEM: mechanism) flips independently with probability d_p[j] (m FP32
 * values in device memory), and the code's records (grand_engine_record_len
 * ints per shot: errors or syndrome for CSS as registered, detectors then true
 * logical flips for DEM) are written to d_records, ready for
 * grand_engine_decode_device.  The draws come from Philox4x32-10 keyed by
 * `seed`; shot first_shot + i always gets the same draws, whatever the batch
 * split.  Asynchronous on `stream`. */
int grand_engine_sample(GrandEngine *engine, int code_id, const float *d_p,
                        unsigned long long seed, unsigned long long first_shot, int num_shots,
                        int *d_records, void *stream);

/* Decode num_shots records, concatenated in shot order, from host memory.
 * shot_code may be NULL when every shot uses code 0.  Synchronous. */
int grand_engine_decode(GrandEngine *engine, int num_shots, const int *shot_code,
                        const int *records, GrandDecoderResult *results,
                        const GrandDecodeOutputs *out);

/* Device-resident decode, asynchronous on `stream` (a cudaStream_t; NULL is
 * the legacy default stream).  All pointers are device pointers; d_offsets
 * (int64 record offsets) and d_shot_code may be NULL when every shot uses code
 * 0.  With use_graph != 0 the launch sequence is captured into a CUDA graph on
 * first use for this argument set and replayed afterwards.  Call
 * grand_engine_sync_status() to wait and read the completion status. */
int grand_engine_decode_device(GrandEngine *engine, int num_shots, const int *d_shot_code,
                               const long long *d_offsets, const int *d_records,
                               GrandDecoderResult *d_results, void *stream, int use_graph);

/* Wait for `stream` and return 0, or a GRAND_ERR_* code when the last device
 * decode on it hit a kernel limit (job table / scratch overflow, active set
 * beyond GRAND_MAX_TAM). */
int grand_engine_sync_status(GrandEngine *engine, void *stream);

/* The reference-style one-launch-per-call path: every shot is its own call
 * (host-to-device copy of its record, its decoding launch, a synchronous
 * read-back of its result), as upstream's GPU mode does per shot.
 * Kept for comparison with the batched path. */
int grand_engine_decode_plain(GrandEngine *engine, int num_shots, const int *shot_code,
                              const int *records, GrandDecoderResult *results);

/* Tuning knobs (also set by the GRAND_* environment variables):
 * light_log2: largest per-shot search (2^x candidates) finished by the warp
 * that triages the shot (larger ones become Jobs that every warp searches);
 * tile_k: prefixes per lane per search tile; search_ctas_per_sm: resident CTAs
 * per SM of the persistent decode kernel (0 = occupancy maximum). */
int grand_engine_set_tuning(GrandEngine *engine, int light_log2, int tile_k,
                            int search_ctas_per_sm);

/* Device times of the last non-graph device decode on `stream` (valid after
 * grand_engine_sync_status): *reset_ms the control-word reset before the
 * launch, *decode_ms the decode kernel. */
int grand_engine_kernel_times(GrandEngine *engine, void *stream, float *reset_ms,
                              float *decode_ms);

/* Work statistics of the last device decode on `stream` (after
 * grand_engine_sync_status): out[0] shots settled by classification (empty
 * syndromes, one-position weight-1 matches), out[1] shots that took the
 * per-shot path, out[2] Jobs published, out[3] search tiles of those Jobs,
 * out[4] scratch words staged for them.  With GRAND_PROFILE=1 in the
 * environment when the engine was created, out[5..8] are the warp-nanoseconds
 * the decode kernel's warps spent classifying, on the per-shot path, on search
 * tiles and waiting for work, out[9..12] when the last of each ended (ns after
 * the first warp started; -1: none), out[13] the number of work steps and
 * out[14..23] a finer split of the warp-nanoseconds: classification (records
 * read and syndromes formed, one-position test, results and queue), per-shot
 * path (record packed, flagged-check counts, planning and light search, Job
 * staging and publication, result written) and search (Job and block lookup
 * with staging, completed Jobs' results) and out[24..27] the Job publications
 * split into reservations, staging, the Job written and the steps that make it
 * searchable, out[28] when the last per-shot-path shot started, out[29] the
 * longest per-shot-path shot and out[30] the longest tile draw (ns); otherwise
 * those entries are 0 / -1.  `out` holds 31 entries. */
int grand_engine_launch_stats(GrandEngine *engine, void *stream, long long *out);

/* Times of the last host-buffer decode (grand_engine_decode / _decode_plain):
 * copies in, the control-word reset(s), the decode kernel(s) and copies out,
 * from CUDA events on the call's stream.  With zero-copy (records read and results
 * written in place over NVLink-C2C) the copy times are ~0 and the kernels'
 * times include reading host memory.  Any pointer may be NULL. */
int grand_engine_batch_times(GrandEngine *engine, float *h2d_ms, float *reset_ms,
                             float *decode_ms, float *d2h_ms);

/* Diagnostic: sustained 32-bit logic-op (lop3) issue rate of the current device
 * in ops/s, the ceiling of the search's integer roofline; < 0 on error. */
double grand_measure_int_peak(void);

/* Diagnostic: one line describing the current device as the library sees it
 * (SM count, resident CTAs per SM of the decode kernel, whether the GPU can read
 * pageable host memory directly).  Returns the length written or < 0. */
int grand_device_info(char *buf, int len);

#ifdef __cplusplus
}
#endif

#endif /* GRAND_ENGINE_H */
