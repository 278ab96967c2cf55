/*
 * grand_decoder.h -- C ABI of the GB300 GRAND decoder (libgranddecoder.so).
 *
 * GRAND (Guessing Random Additive Noise Decoding) over GF(2): for every shot the
 * decoder finds the lowest-ranked error pattern e of weight <= max_error_weight,
 * drawn from the shot's active positions, with H.e == s, and reports per-shot
 * statistics in GrandDecoderResult.
 *
 * Drop-in boundary.  The five grand_decode_* functions keep the names, argument
 * order, argument meaning, struct layouts and return codes of the upstream
 * library (CarolinaBoavida/Library_S_GRAND, grand_decoder.h:37-176), so an
 * existing ctypes caller (Examples/auxilary_functions.py:172-253) loads this
 * library unchanged.  Every search runs on the GPU (sm_103a kernels); there is
 * no CPU search path.  The search result is the one the upstream CPU search mode
 * returns (lowest rank in its enumeration order; minimum FP32 LLR cost with its
 * tie and pruning rules for the ML variant), whatever mode_of_search says;
 * mode_of_search, threshold_for_hybrid and max_size_active_positions keep their
 * upstream effect on which threshold iterations are searched and on the
 * hibrido / total_tested_combinations bookkeeping.
 *
 * All matrices are int32, row-major, with entries 0 or 1.  All buffers belong to
 * the caller.  Functions return 0 on success and a negative value on failure,
 * with a message on stderr.  Calls are reentrant: no state is shared between
 * calls except the immutable device binomial table and the code cache, which is
 * guarded by a mutex.
 */
#ifndef GRAND_DECODER_H
#define GRAND_DECODER_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Largest error weight the search enumerates (upstream grand_decoder.h:28). */
#define GRAND_MAX_W 6

/* Largest active-position set the GPU search accepts.  Upstream sizes its
 * binomial table for 300 (grand_decoder.cu:13) and reads past it above that. */
#define GRAND_MAX_TAM 2048

/* Error codes beyond the upstream -1. */
#define GRAND_ERR_INVALID   (-1) /* same cases as upstream (bad type, weight, file) */
#define GRAND_ERR_CUDA      (-2) /* a CUDA call failed; message on stderr            */
#define GRAND_ERR_LIMIT     (-3) /* a size is beyond what the kernels support        */
#define GRAND_ERR_CANCELLED (-4) /* a server request was cancelled                   */

/* Upstream grand_decoder.h:37-44 (24 bytes). */
typedef struct {
    int max_error_weight;          /* 1..7; searches weights 1..min(w, 6)           */
    int threads_per_block;         /* accepted for compatibility; tiles are chosen
                                      by the autotuner                              */
    int use_gpu_sum;               /* accepted for compatibility; column sums are
                                      always computed on the GPU                    */
    int max_size_active_positions; /* cap on the active set (see upstream quirks)   */
    int threshold_for_hybrid;      /* upstream CPU/GPU switch point (bookkeeping)   */
    int mode_of_search;            /* -1, 0 or 1 as upstream (bookkeeping + skips)  */
} GrandDecoderConfig;

/* Upstream grand_decoder.h:53-68 (72 bytes; u64 at offset 24, doubles at 40..64). */
typedef struct {
    int found;
    int found_weight;
    int original_weight;
    int degenerate;
    int is_equal;
    int tam;
    unsigned long long total_tested_combinations;
    int hibrido;
    int iteration;
    double time_sum_ms;
    double total_time_search_ms;
    double transfer_time_ms;
    double total_to_find_ms;
} GrandDecoderResult;

/* ---------------------------------------------------------------------------
 * The five upstream entry points.
 * ------------------------------------------------------------------------- */

/* Replaces upstream grand_decode_prob_cc (grand_decoder.h:92, grand_decoder.cu:790).
 * probability_file holds up to 20 lines "tam_upper o0 o1 o2 p0 p1 p2"; the line
 * whose tam_upper first covers the active-set size picks the phase order.  A file
 * with no such line is rejected (upstream reads before its mask array). */
int grand_decode_prob_cc(const int *Hx, const int *Hz, int n, int m, int *errors,
                         int *syndromes, int num_shots, const GrandDecoderConfig *config,
                         GrandDecoderResult *results, char type_of_error,
                         const char *probability_file);

/* Replaces upstream grand_decode_cc (grand_decoder.h:112, grand_decoder.cu:1117).
 * errors != NULL: errors (num_shots x m) are the true errors, the syndrome is
 * H.e and is_equal / degenerate are reported; errors == NULL: syndromes
 * (num_shots x n) are decoded.  type_of_error 'x'/'X' decodes with Hz, 'z'/'Z'
 * with Hx. */
int grand_decode_cc(const int *Hx, const int *Hz, int n, int m, int *errors, int *syndromes,
                    int num_shots, const GrandDecoderConfig *config,
                    GrandDecoderResult *results, char type_of_error);

/* Replaces upstream grand_decode_cln (grand_decoder.h:133, grand_decoder.cu:1399).
 * L_dem is m x n_logicos.  logicals (num_shots x n_logicos) is an INPUT: the
 * true observable flips; degenerate = 1 when the decoded flips equal them. */
int grand_decode_cln(int *H_dem, const int *L_dem, int n, int m, int n_logicos,
                     int *detectors, int *logicals, int num_shots,
                     const GrandDecoderConfig *config, GrandDecoderResult *results);

/* Replaces upstream grand_decode_prob_cln (grand_decoder.h:154, grand_decoder.cu:1672). */
int grand_decode_prob_cln(int *H_dem, const int *L_dem, int n, int m, int n_logicos,
                          int *detectors, int *logicals, int num_shots,
                          const GrandDecoderConfig *config, GrandDecoderResult *results,
                          const char *probability_file);

/* Replaces upstream grand_decode_ML_cln (grand_decoder.h:176, grand_decoder.cu:1996).
 * llr_file holds m FP32 values (one per mechanism).  Non-finite values are
 * rejected. */
int grand_decode_ML_cln(int *H_dem, const int *L_dem, int n, int m, int n_logicos,
                        int *detectors, int *logicals, int num_shots,
                        const GrandDecoderConfig *config, GrandDecoderResult *results,
                        const char *llr_file);

/* ---------------------------------------------------------------------------
 * Extensions (no upstream counterpart): the same five calls, also returning
 * what upstream computes but never hands back.
 * ------------------------------------------------------------------------- */

typedef struct {
    unsigned char *decoded_errors;   /* num_shots x m, 0/1, or NULL                   */
    unsigned char *decoded_logicals; /* num_shots x n_logicos, 0/1, or NULL (DEM)     */
    float *ml_cost;                  /* num_shots FP32 LLR cost of the winner, or NULL
                                        (ML only; 0 when nothing was found)           */
} GrandDecodeOutputs;

int grand_decode_prob_cc_ex(const int *Hx, const int *Hz, int n, int m, int *errors,
                            int *syndromes, int num_shots, const GrandDecoderConfig *config,
                            GrandDecoderResult *results, char type_of_error,
                            const char *probability_file, const GrandDecodeOutputs *out);
int grand_decode_cc_ex(const int *Hx, const int *Hz, int n, int m, int *errors, int *syndromes,
                       int num_shots, const GrandDecoderConfig *config,
                       GrandDecoderResult *results, char type_of_error,
                       const GrandDecodeOutputs *out);
int grand_decode_cln_ex(int *H_dem, const int *L_dem, int n, int m, int n_logicos,
                        int *detectors, int *logicals, int num_shots,
                        const GrandDecoderConfig *config, GrandDecoderResult *results,
                        const GrandDecodeOutputs *out);
int grand_decode_prob_cln_ex(int *H_dem, const int *L_dem, int n, int m, int n_logicos,
                             int *detectors, int *logicals, int num_shots,
                             const GrandDecoderConfig *config, GrandDecoderResult *results,
                             const char *probability_file, const GrandDecodeOutputs *out);
int grand_decode_ML_cln_ex(int *H_dem, const int *L_dem, int n, int m, int n_logicos,
                           int *detectors, int *logicals, int num_shots,
                           const GrandDecoderConfig *config, GrandDecoderResult *results,
                           const char *llr_file, const GrandDecodeOutputs *out);

/* No counterpart in the upstream library.  grand_decode_cc with syndrome input
 * for callers that may not allocate device memory while running (a real-time
 * decoding loop that reserved its memory at start-up, a process whose device
 * memory belongs to another framework's pool): it calls no cudaMalloc, cudaFree
 * or other allocating routine.  d_H (n x m int32, the matrix that decodes the
 * syndromes, i.e. Hz for X errors), d_syndromes (num_shots x n int32) and
 * d_results (num_shots records) are device pointers owned by the caller; the
 * deterministic result fields equal grand_decode_cc(Hx, Hz, n, m, NULL,
 * syndromes, ...) field for field, and the timing fields are per-shot GPU timer
 * values as with the other entry points.  Everything else lives in one fixed
 * file-scope device array of about 25 MiB, held by every GPU that loads it until
 * the process exits.  Limits: n <= 256, m <= 1024 (larger sizes return
 * GRAND_ERR_LIMIT with a message).  Shots run in chunks of 2048; hard shots of a
 * chunk share a 16 MiB search arena, and shots that find it full are re-run in
 * further rounds of the chunk with the arena emptied; a shot whose search data
 * alone exceeds the arena gets a zero result and the call returns
 * GRAND_ERR_LIMIT.  The call reads a status word back after each round, so it
 * synchronizes `stream` once per chunk.  The first call on a device does its
 * set-up (looks up the array's device address, fills its binomial table) and
 * synchronizes `stream`: make it before any stream capture.  Like the other
 * entry points, it keeps per-device state for the life of the process: after
 * cudaDeviceReset the process must be restarted before either is called again.
 * Every call reuses the same array, so calls that overlap on the GPU (other
 * threads, other streams) race; the call itself returns only when its work on
 * `stream` (a cudaStream_t, NULL for the legacy default stream) has finished. */
int grand_decode_cc_noalloc(const int *d_H, int n, int m, const int *d_syndromes, int num_shots,
                            const GrandDecoderConfig *config, GrandDecoderResult *d_results,
                            void *stream);

/* Library version string and last error message of the calling thread. */
/* ---------------------------------------------------------------------------
 * Bit-packed records (no upstream counterpart).  Upstream passes one int32 per
 * syndrome bit / error entry (Examples/auxilary_functions.py:262-274), 32x the
 * bytes the information needs; these entry points take each shot as LSB-first
 * uint32 words instead (bit i of word k is entry 32k + i; bits past the last
 * entry are ignored) and return the same results as the int32 calls.
 *
 * grand_decode_cc_packed: kind GRAND_PACKED_SYNDROMES gives ceil(n/32) syndrome
 * words per shot, GRAND_PACKED_ERRORS ceil(m/32) error words (then is_equal and
 * degeneracy are filled as with `errors`); probability_file NULL searches as
 * grand_decode_cc, otherwise as grand_decode_prob_cc with that phase-mask file.
 * grand_decode_cln_packed: ceil(n/32) detector words and ceil(n_logicos/32)
 * logical words per shot; variant 0, 1, 2 searches as grand_decode_cln,
 * grand_decode_prob_cln (file = phase masks) and grand_decode_ML_cln (file =
 * LLRs).  Other arguments and return codes as the int32 calls. */
#define GRAND_PACKED_SYNDROMES 0
#define GRAND_PACKED_ERRORS 1
int grand_decode_cc_packed(const int *Hx, const int *Hz, int n, int m, const unsigned int *records,
                           int kind, int num_shots, const GrandDecoderConfig *config,
                           GrandDecoderResult *results, char type_of_error,
                           const char *probability_file);
int grand_decode_cln_packed(const int *H_dem, const int *L_dem, int n, int m, int n_logicos,
                            const unsigned int *detectors, const unsigned int *logicals,
                            int num_shots, const GrandDecoderConfig *config,
                            GrandDecoderResult *results, int variant, const char *file);

/* Upstream's per-shot stdout line for one result record (no upstream function:
 * upstream prints it inline, grand_decoder.cu:1230-1238 and :1373-1380 for the CSS
 * functions with and without supplied errors, :1651-1653 for the DEM functions).
 * The decoders print these lines with GRAND_VERBOSE=1.  `shot` is the 1-based shot
 * number printed; returns the line length (as snprintf) or -1 for an unknown kind. */
#define GRAND_LINE_CSS_SYNDROMES 0
#define GRAND_LINE_CSS_ERRORS 1
#define GRAND_LINE_DEM 2
int grand_format_result(int kind, const GrandDecoderResult *result, int shot, char *buf,
                        int buf_len);

const char *grand_version(void);
const char *grand_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* GRAND_DECODER_H */
