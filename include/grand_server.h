/*
 * grand_server.h -- continuous-batching decode server on one GPU.
 *
 * No upstream counterpart: upstream decodes synchronously, one call at a time
 * (grand_decoder.cu:885, 1199, 1466, 1762, 2073).  A server owns a fixed set of
 * in-flight slots, each with its own CUDA stream and device workspace sized at
 * creation (admission by memory: the slots must fit the HBM budget and the free
 * device memory).  A dispatcher thread keeps forming micro-batches from the
 * requests waiting in arrival order -- shots of different codes mix freely, and
 * a request is admitted into a micro-batch while the batch's shots fit the slot
 * and the search scratch they are expected to stage (the scratch per shot of
 * the server's recent batches) fits 3/4 of the slot's arena --
 * and starts one on every free slot, so requests that arrive while others are on
 * the GPU join the next micro-batch and their work overlaps on the device with
 * the batches already running.  Results are identical to decoding each request
 * alone with grand_engine_decode.  Where the GPU can read pageable host memory
 * (NVLink-C2C on GB300), the decode kernel reads each request's records where
 * the caller keeps them, with no host or host-to-device copy of records; each
 * slot's persistent kernel takes 1/slots of the resident blocks, so the slots'
 * batches run on the GPU together.
 */
#ifndef GRAND_SERVER_H
#define GRAND_SERVER_H

#include "grand_engine.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct GrandServer GrandServer;

/* slots: micro-batches in flight at once; max_shots_per_batch: shots a slot
 * holds; hbm_budget_bytes: device memory the slots may use (0 = 1/4 of the free
 * memory).  Fewer slots than asked are created when the budget is smaller; the
 * call fails when not even one fits.  The engine's codes must be registered
 * before the server is created and the engine must outlive the server. */
int grand_server_create(GrandEngine *engine, int slots, int max_shots_per_batch,
                        size_t hbm_budget_bytes, GrandServer **server);
void grand_server_destroy(GrandServer *server);

/* Slots actually created and the device bytes they hold. */
int grand_server_info(GrandServer *server, int *slots, size_t *device_bytes);

/* Queue a request of num_shots records (concatenated, codes per shot as in
 * grand_engine_decode; shot_code NULL = code 0).  records, shot_code and
 * results are the caller's and must stay valid until the request completes;
 * num_shots <= max_shots_per_batch. */
int grand_server_submit(GrandServer *server, int num_shots, const int *shot_code,
                        const int *records, GrandDecoderResult *results,
                        unsigned long long *request_id);

/* Wait up to timeout_ms (< 0: forever) for a request.  Returns 0 when done (and
 * its submit-to-completion latency in *latency_ms if non-NULL), 1 on timeout, or
 * a GRAND_ERR_* code. */
int grand_server_wait(GrandServer *server, unsigned long long request_id, int timeout_ms,
                      double *latency_ms);

/* Replay a request trace: request i (num_shots[i] shots, records and shot codes
 * concatenated in request order) is submitted at arrival_s[i] seconds after the
 * start by a submitting thread, and results land in `results` (one per shot, in
 * order).  Returns after every request has completed, with per-request
 * latencies (ms) and the wall time from the first arrival to the last completion. */
int grand_server_replay(GrandServer *server, int num_requests, const double *arrival_s,
                        const int *num_shots, const int *shot_code, const int *records,
                        GrandDecoderResult *results, double *latency_ms, double *wall_s);

#ifdef __cplusplus
}
#endif

#endif /* GRAND_SERVER_H */
