/*
 * grand_oracle.c -- TEST INFRASTRUCTURE ONLY (see grand_oracle.h).
 *
 * A plain-C restatement of the upstream CPU search mode of
 * CarolinaBoavida/Library_S_GRAND.  Each function names the upstream lines it
 * restates ("cu:N" = grand_decoder.cu line N).  The enumeration deliberately
 * keeps upstream's cost model -- every candidate index is mapped back to
 * (weight, rank) and unranked from scratch, and every candidate is checked row
 * by row on the int32 matrix -- so that timing this file measures the same
 * algorithm upstream runs.
 *
 * Deviations, all outside upstream's defined behaviour:
 *  - the binomial table covers n <= GRAND_MAX_TAM (upstream: 300, cu:13, and it
 *    reads past the table for larger active sets);
 *  - candidate counters are 64-bit (upstream counts CPU candidates in an int,
 *    cu:295,534,590, which wraps beyond 2^31 candidates per iteration);
 *  - a probability file without any mask line is rejected for the CSS family as
 *    it already is for the DEM family (upstream reads masks[-1], cu:761);
 *  - non-finite LLR values are rejected.
 */
#include "grand_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define N_TAB GRAND_MAX_TAM
#define MAX_MASKS 20 /* cu:11 */

typedef struct {
    int tam_upper;
    int order[3];
    float prob[3];
} PhaseMask; /* cu:15-19 */

static unsigned long long g_ncr[N_TAB + 1][GRAND_MAX_W + 1];
static int g_ncr_ready = 0;

unsigned long long oracle_ncr(int n, int k)
{
    /* cu:42-52: multiplicative binomial, exact at every step in u64. */
    if (k < 0 || k > n) return 0;
    if (k == 0 || k == n) return 1;
    unsigned long long r = 1;
    for (int i = 1; i <= k; ++i) r = r * (unsigned long long)(n - i + 1) / (unsigned long long)i;
    return r;
}

static void ncr_init(void)
{
    /* cu:54-63 (host half): table of C(n, k) for k <= GRAND_MAX_W. */
    if (g_ncr_ready) return;
    for (int n = 0; n <= N_TAB; ++n)
        for (int k = 0; k <= GRAND_MAX_W; ++k) g_ncr[n][k] = oracle_ncr(n, k);
    g_ncr_ready = 1;
}

static unsigned long long tab(int n, int k)
{
    if (n < 0 || k < 0 || k > GRAND_MAX_W || n > N_TAB) return 0;
    return g_ncr[n][k];
}

void oracle_unrank(unsigned long long rank, int n, int k, int *out_combo)
{
    /* cu:264-280: lexicographic order of ascending k-tuples.  Element i is the
     * smallest value whose block of completions (C(n-1-v, k-1-i) tuples) still
     * holds the remaining rank. */
    ncr_init();
    int v = 0;
    for (int i = 0; i < k; ++i) {
        int rest = k - 1 - i;
        unsigned long long block = tab(n - 1 - v, rest);
        while (rank >= block && (n - 1 - v) > rest) {
            rank -= block;
            ++v;
            block = tab(n - 1 - v, rest);
        }
        out_combo[i] = v++;
    }
}

/* cu:282-293: H.e == s checked row by row on int32 entries, first mismatch exits. */
static int syndrome_matches(const int *H, const int *s, const int *pos, const int *combo,
                            int w, int n_rows, int m_cols)
{
    for (int r = 0; r < n_rows; ++r) {
        int par = 0;
        for (int i = 0; i < w; ++i) par ^= H[(size_t)r * m_cols + pos[combo[i]]];
        if (par != s[r]) return 0;
    }
    return 1;
}

/* cu:495-504: ascending indices with a[i] >= threshold. */
static int positions_at_least(const int *a, int len, int *out, int threshold)
{
    int t = 0;
    for (int i = 0; i < len; ++i)
        if (a[i] >= threshold) out[t++] = i;
    return t;
}

/* Winner of one threshold iteration. */
typedef struct {
    int found;
    int weight;
    int pos[GRAND_MAX_W];   /* H column indices of the winner */
    float cost;             /* ML only */
    unsigned long long cpu_count; /* upstream CPU-branch candidate count */
    unsigned long long gpu_count; /* upstream GPU-branch candidate count */
} IterOutcome;

/* cu:534-588 (search_cpu_massively): candidate index t runs over the weights
 * 1..min(W,6) back to back; each t is mapped to (weight, rank) by walking the
 * weight blocks, unranked, and checked.  Count = t+1 at the first match. */
static void search_uniform(const int *H, const int *s, const int *pos, int tam, int n, int m,
                           int W, IterOutcome *o)
{
    if (W > GRAND_MAX_W) W = GRAND_MAX_W;
    unsigned long long total = 0;
    for (int w = 1; w <= W; ++w) total += tab(tam, w);
    o->gpu_count = total; /* cu:514-524 counts the same blocks for the GPU launch */
    o->cpu_count = 0;
    for (unsigned long long t = 0; t < total; ++t) {
        o->cpu_count++;
        int w_sel = -1;
        unsigned long long rank = 0, base = 0;
        for (int w = 1; w <= W; ++w) {
            unsigned long long blk = tab(tam, w);
            if (t < base + blk) { w_sel = w; rank = t - base; break; }
            base += blk;
        }
        if (w_sel < 0) continue;
        int combo[GRAND_MAX_W];
        oracle_unrank(rank, tam, w_sel, combo);
        if (syndrome_matches(H, s, pos, combo, w_sel, n, m)) {
            o->found = 1;
            o->weight = w_sel;
            for (int i = 0; i < w_sel; ++i) o->pos[i] = pos[combo[i]];
            return;
        }
    }
}

/* cu:764-786: phase 0 = weights 1..min(5, tam, GRAND_MAX_W); phase 1 = {6} when
 * tam >= 6; phase 2 would be {7}, which GRAND_MAX_W excludes; anything else = {}. */
static int phase_weights(int phase_id, int tam, int *ws)
{
    int len = 0;
    if (phase_id == 0) {
        for (int w = 1; w <= 5 && w <= tam && w <= GRAND_MAX_W; ++w) ws[len++] = w;
    } else if (phase_id == 1) {
        if (6 <= tam && 6 <= GRAND_MAX_W) ws[len++] = 6;
    } else if (phase_id == 2) {
        if (7 <= tam && 7 <= GRAND_MAX_W) ws[len++] = 7;
    }
    return len;
}

/* cu:754-762: first mask whose tam_upper covers tam, else the last one. */
static const PhaseMask *mask_for(int tam, const PhaseMask *masks, int n_masks)
{
    for (int i = 0; i < n_masks; ++i)
        if (tam <= masks[i].tam_upper) return &masks[i];
    return &masks[n_masks - 1];
}

/* cu:295-350 (search_cpu_weight / search_cpu_phase) and the per-phase loops of
 * cu:994-1032 (GPU branch) and cu:1038-1054 (CPU branch).  CPU count: every rank
 * tried, up to and including the winner; GPU count: the full size of every phase
 * launched, up to and including the phase that matched. */
static void search_prob(const int *H, const int *s, const int *pos, int tam, int n, int m,
                        const PhaseMask *pm, int num_phases, IterOutcome *o)
{
    o->cpu_count = 0;
    o->gpu_count = 0;
    for (int k = 0; k < num_phases; ++k) {
        int ws[GRAND_MAX_W];
        int len = phase_weights(pm->order[k], tam, ws);
        if (len == 0) continue;
        unsigned long long phase_total = 0;
        for (int i = 0; i < len; ++i) phase_total += oracle_ncr(tam, ws[i]);
        if (phase_total != 0) o->gpu_count += phase_total;
        for (int i = 0; i < len && !o->found; ++i) {
            int w = ws[i];
            if (w <= 0 || w > tam) continue;
            unsigned long long blk = tab(tam, w);
            for (unsigned long long rank = 0; rank < blk; ++rank) {
                o->cpu_count++;
                int combo[GRAND_MAX_W];
                oracle_unrank(rank, tam, w, combo);
                if (syndrome_matches(H, s, pos, combo, w, n, m)) {
                    o->found = 1;
                    o->weight = w;
                    for (int j = 0; j < w; ++j) o->pos[j] = pos[combo[j]];
                    break;
                }
            }
        }
        if (o->found) return;
    }
}

/* cu:590-666 (search_cpu_ml): active positions stably sorted by LLR ascending;
 * prefix[w] = FP32 sum of the w smallest LLRs; weight w is skipped (and the
 * loop ends) once a match exists and prefix[w] >= its cost; inside a weight
 * every rank is tried and a match replaces the best only when its FP32 cost,
 * summed in sorted order, is strictly smaller.  Count = every candidate tried. */
static void search_ml(const int *H, const int *s, const int *pos, int tam, int n, int m, int W,
                      const float *llr, IterOutcome *o)
{
    if (W > GRAND_MAX_W) W = GRAND_MAX_W;
    unsigned long long gpu_total = 0;
    for (int w = 1; w <= W; ++w) gpu_total += oracle_ncr(tam, w);
    o->gpu_count = gpu_total;
    o->cpu_count = 0;

    int *sp = (int *)malloc(sizeof(int) * (size_t)(tam > 0 ? tam : 1));
    for (int i = 0; i < tam; ++i) sp[i] = pos[i];
    for (int i = 1; i < tam; ++i) { /* stable insertion sort, cu:601-610 */
        int key = sp[i];
        float kl = llr[key];
        int j = i - 1;
        while (j >= 0 && llr[sp[j]] > kl) {
            sp[j + 1] = sp[j];
            --j;
        }
        sp[j + 1] = key;
    }
    int max_w = W < tam ? W : tam;
    float prefix[GRAND_MAX_W + 1];
    prefix[0] = 0.0f;
    for (int w = 1; w <= max_w; ++w) prefix[w] = prefix[w - 1] + llr[sp[w - 1]];

    int have = 0;
    float best = 0.0f;
    for (int w = 1; w <= max_w; ++w) {
        if (have && prefix[w] >= best) break;
        unsigned long long blk = tab(tam, w);
        for (unsigned long long rank = 0; rank < blk; ++rank) {
            o->cpu_count++;
            int combo[GRAND_MAX_W];
            oracle_unrank(rank, tam, w, combo);
            if (syndrome_matches(H, s, sp, combo, w, n, m)) {
                float c = 0.0f;
                for (int i = 0; i < w; ++i) c += llr[sp[combo[i]]];
                if (!have || c < best) {
                    have = 1;
                    best = c;
                    o->weight = w;
                    for (int i = 0; i < w; ++i) o->pos[i] = sp[combo[i]];
                }
            }
        }
    }
    free(sp);
    o->found = have;
    o->cost = have ? best : 0.0f;
}

/* cu:376-404: column weights, their maximum and whether all are equal. */
static void column_stats(const int *H, int n, int m, int *colw, int *max_soma, int *regular)
{
    *max_soma = 0;
    *regular = 1;
    for (int c = 0; c < m; ++c) {
        int sum = 0;
        for (int r = 0; r < n; ++r) sum += H[(size_t)r * m + c];
        colw[c] = sum;
        if (sum > *max_soma) *max_soma = sum;
    }
    for (int c = 1; c < m; ++c)
        if (colw[c] != colw[0]) { *regular = 0; break; }
}

/* cu:418-454: in-place reduced row echelon form over GF(2) (bit 0 of each entry). */
static int gf2_rref(int *A, int rows, int cols, int *piv)
{
    int r = 0;
    for (int c = 0; c < cols && r < rows; ++c) {
        int p = -1;
        for (int i = r; i < rows; ++i)
            if (A[(size_t)i * cols + c] & 1) { p = i; break; }
        if (p < 0) continue;
        if (p != r)
            for (int j = 0; j < cols; ++j) {
                int t = A[(size_t)r * cols + j];
                A[(size_t)r * cols + j] = A[(size_t)p * cols + j];
                A[(size_t)p * cols + j] = t;
            }
        for (int i = 0; i < rows; ++i) {
            if (i == r || !(A[(size_t)i * cols + c] & 1)) continue;
            for (int j = 0; j < cols; ++j) A[(size_t)i * cols + j] ^= A[(size_t)r * cols + j];
        }
        piv[r++] = c;
    }
    return r;
}

/* cu:456-474: is v in the row space of the reduced matrix?  v is consumed. */
static int in_rowspace(const int *R, int cols, const int *piv, int rank, int *v)
{
    for (int r = 0; r < rank; ++r) {
        int c = piv[r];
        if (v[c] & 1)
            for (int j = c; j < cols; ++j) v[j] ^= R[(size_t)r * cols + j];
    }
    for (int j = 0; j < cols; ++j)
        if (v[j] & 1) return 0;
    return 1;
}

/* cu:728-752: up to 20 records of "%d %d %d %d %f %f %f". */
static int read_masks(const char *path, PhaseMask *masks)
{
    FILE *f = path ? fopen(path, "r") : NULL;
    if (!f) {
        fprintf(stderr, "Error opening probability file: %s\n", path ? path : "(null)");
        return 0;
    }
    int count = 0;
    while (count < MAX_MASKS) {
        PhaseMask t;
        if (fscanf(f, "%d %d %d %d %f %f %f", &t.tam_upper, &t.order[0], &t.order[1],
                   &t.order[2], &t.prob[0], &t.prob[1], &t.prob[2]) != 7)
            break;
        masks[count++] = t;
    }
    fclose(f);
    return count;
}

/* cu:695-713: m values read with "%f". */
static int read_llr(const char *path, float *llr, int m)
{
    FILE *f = path ? fopen(path, "r") : NULL;
    if (!f) {
        fprintf(stderr, "Error opening LLR file: %s\n", path ? path : "(null)");
        return 0;
    }
    for (int i = 0; i < m; ++i) {
        if (fscanf(f, "%f", &llr[i]) != 1) {
            fprintf(stderr, "Error reading LLR file (expected %d values): %s\n", m, path);
            fclose(f);
            return 0;
        }
    }
    fclose(f);
    return 1;
}

/* Shared per-call state. */
typedef struct {
    int variant;
    const int *H;
    int n, m;
    int W;
    int num_phases;
    const PhaseMask *masks;
    int n_masks;
    const float *llr;
    const GrandDecoderConfig *cfg;
    int max_soma, regular;
    const int *colw;
    int dem; /* 1: apply the active-set cap quirk of cu:1550-1554 */
} Ctx;

typedef struct {
    int found, weight, iteration, tam, hibrido;
    unsigned long long tested;
    float cost;
} ShotOutcome;

/* The threshold-iteration driver shared by all five entry points:
 * cu:1243-1343 (cc), cu:928-1065 (prob_cc), cu:1501-1607 (cln),
 * cu:1795-1937 (prob_cln), cu:2106-2222 (ML).  e_est receives the winner. */
static void run_shot(const Ctx *x, const int *s, int *sum_cols, int *active, int *e_est,
                     ShotOutcome *so)
{
    const GrandDecoderConfig *cfg = x->cfg;
    int n = x->n, m = x->m;
    memset(so, 0, sizeof(*so));
    so->hibrido = -2;

    /* cu:352-374: column sums over the rows whose syndrome entry equals 1. */
    for (int c = 0; c < m; ++c) sum_cols[c] = 0;
    for (int r = 0; r < n; ++r) {
        if (s[r] != 1) continue;
        for (int c = 0; c < m; ++c) sum_cols[c] += x->H[(size_t)r * m + c];
    }
    /* cu:406-416: irregular matrices lift every non-empty column to max_soma. */
    if (!x->regular)
        for (int c = 0; c < m; ++c) sum_cols[c] = x->colw[c] == 0 ? 0 : sum_cols[c] + (x->max_soma - x->colw[c]);

    int it = 0, tam = 0, tam_old = 0;
    while (it < x->max_soma && it < 3) {
        int threshold = x->max_soma - it;
        ++it;
        tam = positions_at_least(sum_cols, m, active, threshold);
        if (x->dem) { /* cu:1550-1554: keep the previous size, truncating the new list */
            if (tam > cfg->max_size_active_positions) tam = tam_old;
            else tam_old = tam;
        }
        if (tam <= 0) continue;

        int gpu = (tam > cfg->threshold_for_hybrid && tam <= cfg->max_size_active_positions &&
                   cfg->mode_of_search == 1) || cfg->mode_of_search == 0;
        int cpu = !gpu && ((tam <= cfg->threshold_for_hybrid && cfg->mode_of_search == 1) ||
                           cfg->mode_of_search == -1);
        if (!gpu && !cpu) continue; /* cu:1296/1327: neither branch runs */

        IterOutcome o;
        memset(&o, 0, sizeof(o));
        if (x->variant == ORACLE_UNIFORM)
            search_uniform(x->H, s, active, tam, n, m, x->W, &o);
        else if (x->variant == ORACLE_PROB)
            search_prob(x->H, s, active, tam, n, m, mask_for(tam, x->masks, x->n_masks),
                        x->num_phases, &o);
        else
            search_ml(x->H, s, active, tam, n, m, x->W, x->llr, &o);

        if (gpu) {
            so->hibrido = so->hibrido == -1 ? 1 : 0;
            so->tested += o.gpu_count;
        } else {
            so->hibrido = -1;
            so->tested += o.cpu_count;
        }
        if (o.found) {
            so->found = 1;
            so->weight = o.weight;
            so->cost = o.cost;
            for (int i = 0; i < o.weight; ++i) e_est[o.pos[i]] = 1;
            break;
        }
    }
    so->iteration = it;
    so->tam = tam;
}

static void fill_result(GrandDecoderResult *r, const ShotOutcome *so, int found_weight,
                        int original_weight, int degenerate, int is_equal)
{
    memset(r, 0, sizeof(*r));
    r->found = so->found;
    r->found_weight = found_weight;
    r->original_weight = original_weight;
    r->degenerate = degenerate;
    r->is_equal = is_equal;
    r->tam = so->tam;
    r->total_tested_combinations = so->tested;
    r->hibrido = so->hibrido;
    r->iteration = so->iteration;
}

int oracle_decode_css(int variant, const int *Hx, const int *Hz, int n, int m,
                      const int *errors, const int *syndromes, int num_shots,
                      const GrandDecoderConfig *config, GrandDecoderResult *results,
                      char type_of_error, const char *probability_file,
                      unsigned char *decoded_errors)
{
    ncr_init();
    const int *H, *Hother;
    /* cu:833-846 / cu:1159-1172 */
    if (type_of_error == 'x' || type_of_error == 'X') { H = Hz; Hother = Hx; }
    else if (type_of_error == 'z' || type_of_error == 'Z') { H = Hx; Hother = Hz; }
    else {
        fprintf(stderr, "Invalid type_of_error: %c. Must be 'x' or 'z'.\n", type_of_error);
        return -1;
    }
    int W = config->max_error_weight;
    if (variant == ORACLE_UNIFORM && (W <= 0 || W > 7)) { /* cu:1174-1180 */
        fprintf(stderr, "Invalid max_error_weight: %d. Must be between 1 and 7.\n", W);
        return -1;
    }
    size_t nm = (size_t)n * m;
    int *colw = (int *)calloc((size_t)m + 1, sizeof(int));
    int *red = (int *)malloc(sizeof(int) * (nm + 1));
    int *piv = (int *)malloc(sizeof(int) * ((size_t)n + 1));
    PhaseMask masks[MAX_MASKS];
    int n_masks = 0, num_phases = 0, max_soma = 0, regular = 1;
    column_stats(H, n, m, colw, &max_soma, &regular);
    if (variant == ORACLE_PROB) n_masks = read_masks(probability_file, masks); /* cu:849 */
    memcpy(red, Hother, sizeof(int) * nm);
    int rank = gf2_rref(red, n, m, piv);
    if (variant == ORACLE_PROB) { /* cu:852-868 */
        if (W == 6) num_phases = 2;
        else if (W == 7) num_phases = 3;
        else if (W > 0 && W < 6) num_phases = 1;
        else {
            fprintf(stderr, "Invalid max_error_weight: %d. Must be 6 or 7.\n", W);
            free(colw); free(red); free(piv);
            return -1;
        }
        if (n_masks == 0) {
            fprintf(stderr, "No phase order masks read from: %s\n",
                    probability_file ? probability_file : "(null)");
            free(colw); free(red); free(piv);
            return -1;
        }
    }

    Ctx x = {variant, H, n, m, W, num_phases, masks, n_masks, NULL, config, max_soma, regular, colw, 0};
    int *s = (int *)malloc(sizeof(int) * ((size_t)n + 1));
    int *sum_cols = (int *)malloc(sizeof(int) * ((size_t)m + 1));
    int *active = (int *)malloc(sizeof(int) * ((size_t)m + 1));
    int *e_est = (int *)malloc(sizeof(int) * ((size_t)m + 1));
    int *delta = (int *)malloc(sizeof(int) * ((size_t)m + 1));

    for (int shot = 0; shot < num_shots; ++shot) {
        const int *e_real = NULL;
        int original_weight = 0;
        memset(e_est, 0, sizeof(int) * (size_t)m);
        if (errors) { /* cu:1211-1218 and cu:476-486 */
            e_real = errors + (size_t)shot * m;
            for (int c = 0; c < m; ++c) original_weight += e_real[c] >= 1;
            for (int r = 0; r < n; ++r) {
                int v = 0;
                for (int c = 0; c < m; ++c) v ^= H[(size_t)r * m + c] & e_real[c];
                s[r] = v;
            }
        } else {
            memcpy(s, syndromes + (size_t)shot * n, sizeof(int) * (size_t)n);
        }
        int ws = 0;
        for (int r = 0; r < n; ++r) ws += s[r] >= 1;

        ShotOutcome so;
        memset(&so, 0, sizeof(so));
        so.hibrido = -2;
        int found_weight = 0, degenerate = 0, is_equal = 0;
        if (ws > 0) { /* cu:1223-1241: an empty syndrome is reported unsearched */
            run_shot(&x, s, sum_cols, active, e_est, &so);
            if (so.found) { /* cu:1359-1366 */
                for (int c = 0; c < m; ++c) found_weight += e_est[c] >= 1;
                if (e_real) {
                    is_equal = 1;
                    for (int c = 0; c < m; ++c)
                        if (e_real[c] != e_est[c]) { is_equal = 0; break; }
                    for (int c = 0; c < m; ++c) delta[c] = e_real[c] ^ e_est[c];
                    degenerate = in_rowspace(red, m, piv, rank, delta);
                }
            }
        }
        fill_result(&results[shot], &so, found_weight, original_weight, degenerate, is_equal);
        if (decoded_errors)
            for (int c = 0; c < m; ++c) decoded_errors[(size_t)shot * m + c] = (unsigned char)e_est[c];
    }
    free(s); free(sum_cols); free(active); free(e_est); free(delta);
    free(colw); free(red); free(piv);
    return 0;
}

int oracle_decode_dem(int variant, const int *H_dem, const int *L_dem, int n, int m,
                      int n_logicos, const int *detectors, const int *logicals,
                      int num_shots, const GrandDecoderConfig *config,
                      GrandDecoderResult *results, const char *file,
                      unsigned char *decoded_errors, unsigned char *decoded_logicals,
                      float *ml_cost)
{
    ncr_init();
    int W = config->max_error_weight;
    if (W <= 0 || W > 7) { /* cu:1442-1448, cu:1714-1720, cu:2040-2046 */
        fprintf(stderr, "Invalid max_error_weight: %d. Must be between 1 and 7.\n", W);
        return -1;
    }
    float *llr = NULL;
    if (variant == ORACLE_ML) { /* cu:2048-2053 */
        llr = (float *)malloc(sizeof(float) * ((size_t)m + 1));
        if (!read_llr(file, llr, m)) { free(llr); return -1; }
        for (int i = 0; i < m; ++i)
            if (!isfinite(llr[i])) {
                fprintf(stderr, "Non-finite LLR value at position %d: %s\n", i, file);
                free(llr);
                return -1;
            }
    }
    int *colw = (int *)calloc((size_t)m + 1, sizeof(int));
    int max_soma = 0, regular = 1;
    column_stats(H_dem, n, m, colw, &max_soma, &regular);
    PhaseMask masks[MAX_MASKS];
    int n_masks = 0, num_phases = 0;
    if (variant == ORACLE_PROB) { /* cu:1723-1745 */
        n_masks = read_masks(file, masks);
        if (n_masks == 0) {
            fprintf(stderr, "No phase order masks read from: %s\n", file ? file : "(null)");
            free(colw);
            return -1;
        }
        num_phases = W == 6 ? 2 : (W == 7 ? 3 : 1);
    }

    Ctx x = {variant, H_dem, n, m, W, num_phases, masks, n_masks, llr, config, max_soma, regular, colw, 1};
    int *sum_cols = (int *)malloc(sizeof(int) * ((size_t)m + 1));
    int *active = (int *)malloc(sizeof(int) * ((size_t)m + 1));
    int *e_est = (int *)malloc(sizeof(int) * ((size_t)m + 1));
    int *lest = (int *)malloc(sizeof(int) * ((size_t)n_logicos + 1));

    for (int shot = 0; shot < num_shots; ++shot) {
        const int *s = detectors + (size_t)shot * n;
        const int *truth = logicals + (size_t)shot * n_logicos;
        memset(e_est, 0, sizeof(int) * (size_t)m);
        memset(lest, 0, sizeof(int) * (size_t)(n_logicos + 1));
        int ws = 0;
        for (int r = 0; r < n; ++r) ws += s[r] >= 1;

        ShotOutcome so;
        memset(&so, 0, sizeof(so));
        so.hibrido = -2;
        int found_weight = 0, degenerate = 0;
        if (ws > 0) { /* cu:1487-1499 */
            run_shot(&x, s, sum_cols, active, e_est, &so);
            if (so.found) { /* cu:1623-1644: decoded flips vs the supplied true flips */
                for (int c = 0; c < m; ++c) {
                    if (e_est[c] < 1) continue;
                    ++found_weight;
                    for (int j = 0; j < n_logicos; ++j) lest[j] ^= L_dem[(size_t)c * n_logicos + j];
                }
                degenerate = 1;
                for (int j = 0; j < n_logicos; ++j)
                    if ((lest[j] ^ truth[j]) == 1) degenerate = 0;
            }
        }
        fill_result(&results[shot], &so, found_weight, 0, degenerate, 0);
        if (decoded_errors)
            for (int c = 0; c < m; ++c) decoded_errors[(size_t)shot * m + c] = (unsigned char)e_est[c];
        if (decoded_logicals)
            for (int j = 0; j < n_logicos; ++j)
                decoded_logicals[(size_t)shot * n_logicos + j] = (unsigned char)lest[j];
        if (ml_cost) ml_cost[shot] = so.found ? so.cost : 0.0f;
    }
    free(sum_cols); free(active); free(e_est); free(lest); free(colw); free(llr);
    return 0;
}

double oracle_ml_cost_fp64(const float *llr, const unsigned char *pattern, int m)
{
    double acc = 0.0;
    for (int c = 0; c < m; ++c)
        if (pattern[c]) acc += (double)llr[c];
    return acc;
}
