// grand_capi.cpp -- the extern "C" entry points of libgranddecoder.so.
//
// Validation order, messages and return codes follow the upstream entry
// points (grand_decoder.cu:790-868, 1117-1180, 1399-1448, 1672-1745,
// 1996-2053); the work itself is one batched GPU launch per call.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>
#include <mutex>
#include <string>

#include <sys/stat.h>

#include "grand_host.h"

namespace grand {
const char *last_error();

struct Masks {
  int n = 0;
  int tam_upper[kMaxMasks];
  int order[kMaxMasks][3];
};

// Upstream read_phase_orders_from_file (grand_decoder.cu:728-752): up to 20
// records of "%d %d %d %d %f %f %f" read with the same scanf conversions.
Masks read_masks(const char *path) {
  Masks mk;
  FILE *f = path ? fopen(path, "r") : nullptr;
  if (!f) {
    fprintf(stderr, "Error opening probability file: %s\n", path ? path : "(null)");
    return mk;
  }
  while (mk.n < kMaxMasks) {
    int t, a, b, c;
    float p0, p1, p2;
    if (fscanf(f, "%d %d %d %d %f %f %f", &t, &a, &b, &c, &p0, &p1, &p2) != 7) break;
    mk.tam_upper[mk.n] = t;
    mk.order[mk.n][0] = a;
    mk.order[mk.n][1] = b;
    mk.order[mk.n][2] = c;
    ++mk.n;
  }
  fclose(f);
  return mk;
}

// The same, remembered per (path, modification time, size): callers decode batch
// after batch with the same mask file.
Masks read_masks_cached(const char *path) {
  static std::mutex mu;
  static std::string last_path;
  static long long last_mtime = -1, last_size = -1;
  static Masks last;
  struct stat st;
  if (!path || stat(path, &st) != 0) return read_masks(path);
  const long long mt = (long long)st.st_mtim.tv_sec * 1000000000LL + st.st_mtim.tv_nsec;
  std::lock_guard<std::mutex> lk(mu);
  if (last_path == path && last_mtime == mt && last_size == (long long)st.st_size) return last;
  Masks mk = read_masks(path);
  last_path = path;
  last_mtime = mt;
  last_size = (long long)st.st_size;
  last = mk;
  return mk;
}

// Upstream read_llr_from_file_ml (grand_decoder.cu:695-713), plus a finiteness check.
bool read_llr(const char *path, std::vector<float> &llr, int m) {
  FILE *f = path ? fopen(path, "r") : nullptr;
  if (!f) {
    fprintf(stderr, "Error opening LLR file: %s\n", path ? path : "(null)");
    return false;
  }
  llr.resize(m);
  for (int i = 0; i < m; ++i) {
    if (fscanf(f, "%f", &llr[i]) != 1) {
      fprintf(stderr, "Error reading LLR file (expected %d values): %s\n", m, path);
      fclose(f);
      return false;
    }
  }
  fclose(f);
  for (int i = 0; i < m; ++i)
    if (!isfinite(llr[i])) {
      fprintf(stderr, "Non-finite LLR value at position %d: %s\n", i, path);
      return false;
    }
  return true;
}

int num_phases_for(int W) {  // grand_decoder.cu:852-868
  if (W == 6) return 2;
  if (W == 7) return 3;
  if (W > 0 && W < 6) return 1;
  return 0;
}

bool read_llr_file(const char *path, std::vector<float> &llr, int m) { return read_llr(path, llr, m); }

// Phase masks for a registered code: the upstream checks, in upstream order.
int read_masks_into(const char *path, CallParams *p, int W) {
  Masks mk = read_masks_cached(path);
  p->num_phases = num_phases_for(W);
  if (p->num_phases == 0) {
    fprintf(stderr, "Invalid max_error_weight: %d. Must be 6 or 7.\n", W);
    return GRAND_ERR_INVALID;
  }
  if (mk.n == 0) {
    fprintf(stderr, "No phase order masks read from: %s\n", path ? path : "(null)");
    return GRAND_ERR_INVALID;
  }
  p->n_masks = mk.n;
  memcpy(p->mask_tam_upper, mk.tam_upper, sizeof(mk.tam_upper));
  memcpy(p->mask_order, mk.order, sizeof(mk.order));
  return 0;
}

namespace {

bool verbose() {
  static int v = [] {
    const char *s = getenv("GRAND_VERBOSE");
    return s && *s && *s != '0' ? 1 : 0;
  }();
  return v != 0;
}

void print_css(const GrandDecoderResult *res, int N, bool with_errors) {
  char line[512];
  for (int i = 0; i < N; ++i) {
    grand_format_result(with_errors ? GRAND_LINE_CSS_ERRORS : GRAND_LINE_CSS_SYNDROMES, &res[i],
                        i + 1, line, (int)sizeof(line));
    fputs(line, stdout);
  }
}

void print_dem(const GrandDecoderResult *res, int N) {
  char line[512];
  for (int i = 0; i < N; ++i) {
    grand_format_result(GRAND_LINE_DEM, &res[i], i + 1, line, (int)sizeof(line));
    fputs(line, stdout);
  }
}

struct WsGuard {
  Context *c;
  Workspace *w;
  ~WsGuard() { if (c && w) c->release(w); }
};

int decode_css(int variant, const int *Hx, const int *Hz, int n, int m, const int *errors,
               const int *syndromes, int num_shots, const GrandDecoderConfig *config,
               GrandDecoderResult *results, char type_of_error, const char *pfile,
               const GrandDecodeOutputs *out, bool packed = false) {
  const int *H, *Ho;
  if (type_of_error == 'x' || type_of_error == 'X') {
    H = Hz;
    Ho = Hx;
  } else if (type_of_error == 'z' || type_of_error == 'Z') {
    H = Hx;
    Ho = Hz;
  } else {
    fprintf(stderr, "Invalid type_of_error: %c. Must be 'x' or 'z'.\n", type_of_error);
    return GRAND_ERR_INVALID;
  }
  if (!config) {
    fprintf(stderr, "grand: config is NULL\n");
    return GRAND_ERR_INVALID;
  }
  const int W = config->max_error_weight;
  if (variant == kUniform && (W <= 0 || W > 7)) {
    fprintf(stderr, "Invalid max_error_weight: %d. Must be between 1 and 7.\n", W);
    return GRAND_ERR_INVALID;
  }
  Masks mk;
  CallParams p;
  p.variant = variant;
  if (variant == kProb) {
    mk = read_masks_cached(pfile);
    p.num_phases = num_phases_for(W);
    if (p.num_phases == 0) {
      fprintf(stderr, "Invalid max_error_weight: %d. Must be 6 or 7.\n", W);
      return GRAND_ERR_INVALID;
    }
    if (mk.n == 0) {
      fprintf(stderr, "No phase order masks read from: %s\n", pfile ? pfile : "(null)");
      return GRAND_ERR_INVALID;
    }
    p.n_masks = mk.n;
    memcpy(p.mask_tam_upper, mk.tam_upper, sizeof(mk.tam_upper));
    memcpy(p.mask_order, mk.order, sizeof(mk.order));
  }
  if (num_shots <= 0) return 0;
  if (!Hx || !Hz || !results || (!errors && !syndromes)) {
    fprintf(stderr, "grand: NULL matrix, result or shot buffer\n");
    return GRAND_ERR_INVALID;
  }
  if (n <= 0 || m <= 0 || n > kMaxRows || m > kMaxCols) {
    set_error("grand: matrix %d x %d outside the supported 1..%d rows, 1..%d columns", n, m,
              kMaxRows, kMaxCols);
    return GRAND_ERR_LIMIT;
  }
  int err = 0;
  Context *ctx = Context::get(&err);
  if (!ctx) return err;
  auto tab = ctx->tables(kCss, H, Ho, nullptr, n, m, 0, &err);
  if (!tab) return err;
  p.input_kind = errors ? kInErrors : kInSyndromes;
  p.W = W;
  p.mode = config->mode_of_search;
  p.thr = config->threshold_for_hybrid;
  p.cap = config->max_size_active_positions;
  WsGuard g{ctx, ctx->acquire()};
  if (!g.w) {
    set_error("grand: could not create a stream");
    return GRAND_ERR_CUDA;
  }
  BatchRequest req;
  req.num_shots = num_shots;
  req.codes.push_back(make_devcode(*tab, p));
  req.h_in = errors ? errors : syndromes;
  req.in_ints = (size_t)num_shots * (errors ? m : n);
  if (packed) {  // ceil(m/32) error words or ceil(n/32) syndrome words per shot
    const int words = errors ? (m + 31) / 32 : (n + 31) / 32;
    req.in_ints = (size_t)num_shots * words;
    req.codes[0].rec_len = words;
    req.codes[0].packed = 1;
  }
  req.h_results = results;
  req.h_dec_err = out ? out->decoded_errors : nullptr;
  req.dec_m = m;
  int rc = run_batch(ctx, g.w, req, nullptr);
  if (rc != 0 && rc != GRAND_ERR_LIMIT) return rc;
  if (verbose()) print_css(results, num_shots, errors != nullptr);
  return rc;
}

int decode_dem(int variant, const int *H, const int *L, int n, int m, int nl, const int *det,
               const int *logicals, int num_shots, const GrandDecoderConfig *config,
               GrandDecoderResult *results, const char *file, const GrandDecodeOutputs *out,
               bool packed = false) {
  if (!config) {
    fprintf(stderr, "grand: config is NULL\n");
    return GRAND_ERR_INVALID;
  }
  const int W = config->max_error_weight;
  if (W <= 0 || W > 7) {
    fprintf(stderr, "Invalid max_error_weight: %d. Must be between 1 and 7.\n", W);
    return GRAND_ERR_INVALID;
  }
  std::vector<float> llr;
  if (variant == kMl && !read_llr(file, llr, m)) return GRAND_ERR_INVALID;
  CallParams p;
  p.variant = variant;
  if (variant == kProb) {
    Masks mk = read_masks_cached(file);
    if (mk.n == 0) {
      fprintf(stderr, "No phase order masks read from: %s\n", file ? file : "(null)");
      return GRAND_ERR_INVALID;
    }
    p.num_phases = num_phases_for(W);
    p.n_masks = mk.n;
    memcpy(p.mask_tam_upper, mk.tam_upper, sizeof(mk.tam_upper));
    memcpy(p.mask_order, mk.order, sizeof(mk.order));
  }
  if (num_shots <= 0) return 0;
  if (!H || !results || !det || (nl > 0 && (!L || !logicals)) || nl < 0) {
    fprintf(stderr, "grand: NULL matrix, result or shot buffer\n");
    return GRAND_ERR_INVALID;
  }
  if (n <= 0 || m <= 0 || n > kMaxRows || m > kMaxCols || nl > kMaxLogicals) {
    set_error("grand: DEM %d x %d with %d logicals outside the supported limits", n, m, nl);
    return GRAND_ERR_LIMIT;
  }
  int err = 0;
  Context *ctx = Context::get(&err);
  if (!ctx) return err;
  auto tab = ctx->tables(kDem, H, nullptr, L, n, m, nl, &err);
  if (!tab) return err;
  WsGuard g{ctx, ctx->acquire()};
  if (!g.w) {
    set_error("grand: could not create a stream");
    return GRAND_ERR_CUDA;
  }
  if (variant == kMl) {
    cudaError_t e = ensure(&g.w->d_llr, &g.w->cap_llr, sizeof(float) * m);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(g.w->d_llr, llr.data(), sizeof(float) * m, cudaMemcpyHostToDevice,
                          g.w->stream);
    if (e != cudaSuccess) {
      set_error("grand: LLR upload failed (%s)", cudaGetErrorString(e));
      return GRAND_ERR_CUDA;
    }
    p.d_llr = (const float *)g.w->d_llr;
  }
  p.input_kind = kInDetectors;
  p.W = W;
  p.mode = config->mode_of_search;
  p.thr = config->threshold_for_hybrid;
  p.cap = config->max_size_active_positions;
  BatchRequest req;
  req.num_shots = num_shots;
  req.codes.push_back(make_devcode(*tab, p));
  req.h_in = det;
  req.in_ints = (size_t)num_shots * n;
  static const int zero = 0;
  req.h_in_log = nl > 0 ? logicals : &zero;
  req.in_log_ints = nl > 0 ? (size_t)num_shots * nl : 1;
  if (packed) {  // ceil(n/32) detector words and ceil(nl/32) logical words per shot
    req.in_ints = (size_t)num_shots * ((n + 31) / 32);
    req.in_log_ints = nl > 0 ? (size_t)num_shots * ((nl + 31) / 32) : 1;
    req.codes[0].rec_len = (n + 31) / 32;
    req.codes[0].packed = 1;
  }
  req.h_results = results;
  req.h_dec_err = out ? out->decoded_errors : nullptr;
  req.h_dec_log = out ? out->decoded_logicals : nullptr;
  req.h_cost = (out && variant == kMl) ? out->ml_cost : nullptr;
  req.dec_m = m;
  req.dec_nl = nl;
  int rc = run_batch(ctx, g.w, req, nullptr);
  if (rc != 0 && rc != GRAND_ERR_LIMIT) return rc;
  if (out && variant != kMl && out->ml_cost)
    for (int i = 0; i < num_shots; ++i) out->ml_cost[i] = 0.0f;
  if (verbose()) print_dem(results, num_shots);
  return rc;
}

}  // namespace
}  // namespace grand

using namespace grand;

extern "C" {

int grand_decode_prob_cc(const int *Hx, const int *Hz, int n, int m, int *errors, int *syndromes,
                         int num_shots, const GrandDecoderConfig *config,
                         GrandDecoderResult *results, char type_of_error,
                         const char *probability_file) {
  return decode_css(kProb, Hx, Hz, n, m, errors, syndromes, num_shots, config, results,
                    type_of_error, probability_file, nullptr);
}

int grand_decode_cc(const int *Hx, const int *Hz, int n, int m, int *errors, int *syndromes,
                    int num_shots, const GrandDecoderConfig *config, GrandDecoderResult *results,
                    char type_of_error) {
  return decode_css(kUniform, Hx, Hz, n, m, errors, syndromes, num_shots, config, results,
                    type_of_error, nullptr, nullptr);
}

int grand_decode_cln(int *H_dem, const int *L_dem, int n, int m, int n_logicos, int *detectors,
                     int *logicals, int num_shots, const GrandDecoderConfig *config,
                     GrandDecoderResult *results) {
  return decode_dem(kUniform, H_dem, L_dem, n, m, n_logicos, detectors, logicals, num_shots,
                    config, results, nullptr, nullptr);
}

int grand_decode_prob_cln(int *H_dem, const int *L_dem, int n, int m, int n_logicos,
                          int *detectors, int *logicals, int num_shots,
                          const GrandDecoderConfig *config, GrandDecoderResult *results,
                          const char *probability_file) {
  return decode_dem(kProb, H_dem, L_dem, n, m, n_logicos, detectors, logicals, num_shots, config,
                    results, probability_file, nullptr);
}

int grand_decode_ML_cln(int *H_dem, const int *L_dem, int n, int m, int n_logicos,
                        int *detectors, int *logicals, int num_shots,
                        const GrandDecoderConfig *config, GrandDecoderResult *results,
                        const char *llr_file) {
  return decode_dem(kMl, H_dem, L_dem, n, m, n_logicos, detectors, logicals, num_shots, config,
                    results, llr_file, nullptr);
}

int grand_decode_prob_cc_ex(const int *Hx, const int *Hz, int n, int m, int *errors,
                            int *syndromes, int num_shots, const GrandDecoderConfig *config,
                            GrandDecoderResult *results, char type_of_error,
                            const char *probability_file, const GrandDecodeOutputs *out) {
  return decode_css(kProb, Hx, Hz, n, m, errors, syndromes, num_shots, config, results,
                    type_of_error, probability_file, out);
}

int grand_decode_cc_ex(const int *Hx, const int *Hz, int n, int m, int *errors, int *syndromes,
                       int num_shots, const GrandDecoderConfig *config,
                       GrandDecoderResult *results, char type_of_error,
                       const GrandDecodeOutputs *out) {
  return decode_css(kUniform, Hx, Hz, n, m, errors, syndromes, num_shots, config, results,
                    type_of_error, nullptr, out);
}

int grand_decode_cln_ex(int *H_dem, const int *L_dem, int n, int m, int n_logicos,
                        int *detectors, int *logicals, int num_shots,
                        const GrandDecoderConfig *config, GrandDecoderResult *results,
                        const GrandDecodeOutputs *out) {
  return decode_dem(kUniform, H_dem, L_dem, n, m, n_logicos, detectors, logicals, num_shots,
                    config, results, nullptr, out);
}

int grand_decode_prob_cln_ex(int *H_dem, const int *L_dem, int n, int m, int n_logicos,
                             int *detectors, int *logicals, int num_shots,
                             const GrandDecoderConfig *config, GrandDecoderResult *results,
                             const char *probability_file, const GrandDecodeOutputs *out) {
  return decode_dem(kProb, H_dem, L_dem, n, m, n_logicos, detectors, logicals, num_shots, config,
                    results, probability_file, out);
}

int grand_decode_ML_cln_ex(int *H_dem, const int *L_dem, int n, int m, int n_logicos,
                           int *detectors, int *logicals, int num_shots,
                           const GrandDecoderConfig *config, GrandDecoderResult *results,
                           const char *llr_file, const GrandDecodeOutputs *out) {
  return decode_dem(kMl, H_dem, L_dem, n, m, n_logicos, detectors, logicals, num_shots, config,
                    results, llr_file, out);
}

int grand_decode_cc_packed(const int *Hx, const int *Hz, int n, int m, const unsigned int *records,
                           int kind, int num_shots, const GrandDecoderConfig *config,
                           GrandDecoderResult *results, char type_of_error,
                           const char *probability_file) {
  if (kind != GRAND_PACKED_SYNDROMES && kind != GRAND_PACKED_ERRORS) {
    fprintf(stderr, "grand: packed record kind %d is neither syndromes (0) nor errors (1)\n", kind);
    return GRAND_ERR_INVALID;
  }
  const int *rec = reinterpret_cast<const int *>(records);
  return decode_css(probability_file ? kProb : kUniform, Hx, Hz, n, m,
                    kind == GRAND_PACKED_ERRORS ? rec : nullptr,
                    kind == GRAND_PACKED_SYNDROMES ? rec : nullptr, num_shots, config, results,
                    type_of_error, probability_file, nullptr, true);
}

int grand_decode_cln_packed(const int *H_dem, const int *L_dem, int n, int m, int n_logicos,
                            const unsigned int *detectors, const unsigned int *logicals,
                            int num_shots, const GrandDecoderConfig *config,
                            GrandDecoderResult *results, int variant, const char *file) {
  if (variant < kUniform || variant > kMl) {
    fprintf(stderr, "grand: DEM variant %d is not uniform (0), prob (1) or ML (2)\n", variant);
    return GRAND_ERR_INVALID;
  }
  return decode_dem(variant, H_dem, L_dem, n, m, n_logicos, reinterpret_cast<const int *>(detectors),
                    reinterpret_cast<const int *>(logicals), num_shots, config, results, file,
                    nullptr, true);
}

// Upstream's per-shot stdout line (grand_decoder.cu:1230-1238 / 1373-1380 for the CSS
// functions with and without supplied errors, :1651-1653 for the DEM functions).
int grand_format_result(int kind, const GrandDecoderResult *r, int shot, char *buf, int buf_len) {
  if (!r || !buf || buf_len <= 0) return -1;
  if (kind == GRAND_LINE_CSS_ERRORS)
    return snprintf(buf, (size_t)buf_len,
                    "shot %d: found=%d, original_weight=%d, found_weight=%d, degenerate=%d, "
                    "is_equal=%d, iteration=%d, tam=%d, total_tested_combinations=%llu, hybrid=%d, "
                    "time_sum_ms=%.5f, total_time_search_ms=%.5f, transfer_time_ms=%.5f, "
                    "total_to_find_ms=%.5f\n",
                    shot, r->found, r->original_weight, r->found_weight, r->degenerate, r->is_equal,
                    r->iteration, r->tam, r->total_tested_combinations, r->hibrido, r->time_sum_ms,
                    r->total_time_search_ms, r->transfer_time_ms, r->total_to_find_ms);
  if (kind == GRAND_LINE_CSS_SYNDROMES)
    return snprintf(buf, (size_t)buf_len,
                    "shot %d: found=%d, found_weight=%d, iteration=%d, tam=%d, "
                    "total_tested_combinations=%llu, hybrid=%d, time_sum_ms=%.5f, "
                    "total_time_search_ms=%.5f, transfer_time_ms=%.5f, total_to_find_ms=%.5f\n",
                    shot, r->found, r->found_weight, r->iteration, r->tam,
                    r->total_tested_combinations, r->hibrido, r->time_sum_ms,
                    r->total_time_search_ms, r->transfer_time_ms, r->total_to_find_ms);
  if (kind == GRAND_LINE_DEM)
    return snprintf(buf, (size_t)buf_len,
                    "shot %d: found=%d, found_weight=%d, degenerate=%d, iteration=%d, tam=%d, "
                    "total_tested_combinations=%llu, hybrid=%d, time_sum_ms=%.5f, "
                    "total_time_search_ms=%.5f, transfer_time_ms=%.5f, total_to_find_ms=%.5f\n",
                    shot, r->found, r->found_weight, r->degenerate, r->iteration, r->tam,
                    r->total_tested_combinations, r->hibrido, r->time_sum_ms,
                    r->total_time_search_ms, r->transfer_time_ms, r->total_to_find_ms);
  return -1;
}

const char *grand_version(void) { return "grand-gb300 0.1 (sm_103a)"; }

const char *grand_last_error(void) { return grand::last_error(); }

}  // extern "C"
