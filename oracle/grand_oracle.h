/*
 * grand_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the upstream GRAND decoder's CPU search mode
 * (CarolinaBoavida/Library_S_GRAND, grand_decoder.cu), used as the parity
 * checker by tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline
 * leg.  The product library (libgranddecoder.so) never links, loads or calls it.
 *
 * Semantics: every searched threshold iteration is searched with the upstream
 * CPU algorithm (lowest rank in enumeration order; search_cpu_ml for the ML
 * variant).  The bookkeeping fields hibrido and total_tested_combinations follow
 * the branch upstream takes for the configured mode_of_search: the CPU-branch
 * count (candidates up to and including the winner) or the GPU-branch count
 * (the whole search space of every launched weight list).  With
 * mode_of_search == -1 this is exactly upstream's CPU mode.
 *
 * Parity pin: tests/test_oracle_pin.py checks every deterministic result field
 * against the upstream library compiled from source (oracle/_ref) and against the
 * committed golden fixtures in tests/golden/.
 */
#ifndef GRAND_ORACLE_H
#define GRAND_ORACLE_H

#include "../include/grand_decoder.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Family selectors for the generic drivers. */
#define ORACLE_UNIFORM 0
#define ORACLE_PROB    1
#define ORACLE_ML      2

/* CSS family: grand_decode_cc (variant ORACLE_UNIFORM) and grand_decode_prob_cc
 * (ORACLE_PROB).  decoded_errors: num_shots x m bytes or NULL. */
int oracle_decode_css(int variant, const int *Hx, const int *Hz, int n, int m,
                      const int *errors, const int *syndromes, int num_shots,
                      const GrandDecoderConfig *config, GrandDecoderResult *results,
                      char type_of_error, const char *probability_file,
                      unsigned char *decoded_errors);

/* DEM family: grand_decode_cln / grand_decode_prob_cln / grand_decode_ML_cln.
 * file is the phase-mask file (ORACLE_PROB) or the LLR file (ORACLE_ML).
 * decoded_errors: num_shots x m, decoded_logicals: num_shots x n_logicos,
 * ml_cost: num_shots (ML winner cost in FP32, the upstream summation order). */
int oracle_decode_dem(int variant, const int *H_dem, const int *L_dem, int n, int m,
                      int n_logicos, const int *detectors, const int *logicals,
                      int num_shots, const GrandDecoderConfig *config,
                      GrandDecoderResult *results, const char *file,
                      unsigned char *decoded_errors, unsigned char *decoded_logicals,
                      float *ml_cost);

/* FP64 cost of a decoded pattern: sum of double(llr[c]) over set positions, in
 * ascending position order (the independent FP64 check of the ML sums). */
double oracle_ml_cost_fp64(const float *llr, const unsigned char *pattern, int m);

/* Binomial C(n, k) as upstream nCr_cpu computes it (grand_decoder.cu:42-52). */
unsigned long long oracle_ncr(int n, int k);

/* Lexicographic unranking of a k-subset of [0, n) (grand_decoder.cu:264-280). */
void oracle_unrank(unsigned long long rank, int n, int k, int *out_combo);

#ifdef __cplusplus
}
#endif

#endif
