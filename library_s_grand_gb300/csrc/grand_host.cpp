// grand_host.cpp -- device context, code tables, workspaces and the batch driver.
#include "grand_host.h"
#include "grand_solo.h"

#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>

namespace grand {

static thread_local char g_err[512];

void set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  fprintf(stderr, "%s\n", g_err);
}

const char *last_error() { return g_err; }

#define CK(call)                                                                    \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess) {                                                        \
      set_error("grand: CUDA error %s at %s:%d (%s)", cudaGetErrorString(e_), __FILE__, \
                __LINE__, #call);                                                   \
      return GRAND_ERR_CUDA;                                                        \
    }                                                                               \
  } while (0)

Tuning &tuning() {
  static Tuning t = [] {
    Tuning x;
    if (const char *s = getenv("GRAND_LIGHT_LOG2")) x.light_max_log2 = std::max(0, std::min(40, atoi(s)));
    if (const char *s = getenv("GRAND_TILE_K")) x.tile_k = std::max(1, std::min(64, atoi(s)));
    if (const char *s = getenv("GRAND_SEARCH_GRID_MULT")) x.search_grid_mult = std::max(0, atoi(s));
    if (const char *s = getenv("GRAND_ZERO_COPY")) x.zero_copy = atoi(s) != 0;
    if (const char *s = getenv("GRAND_FAST")) x.fast = atoi(s) != 0;
    if (const char *s = getenv("GRAND_PROFILE")) x.profile = atoi(s) != 0;
    return x;
  }();
  return t;
}

cudaError_t ensure(void **p, size_t *cap, size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (*p && *cap >= bytes) return cudaSuccess;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  size_t want = std::max(bytes, *cap + *cap / 2);
  cudaError_t e = cudaMalloc(p, want);
  if (e == cudaSuccess) *cap = want;
  else *p = nullptr;
  return e;
}

cudaError_t ensure_zeroed(void **p, size_t *cap, size_t bytes) {
  void *before = *p;
  cudaError_t e = ensure(p, cap, bytes);
  if (e == cudaSuccess && *p != before) e = cudaMemset(*p, 0, *cap);
  return e;
}

CodeTables::~CodeTables() {
  cudaFree(cols);
  cudaFree(colw);
  cudaFree(rref);
  cudaFree(pivrow);
  cudaFree(lcols);
  cudaFree(hcol);
  cudaFree(solo_keys);
  cudaFree(solo_cols);
}

Workspace::~Workspace() {
  void *bufs[] = {d_in, d_in2, d_res, d_dec, d_declog, d_cost, d_jobs, d_scratch, d_small,
                  d_deferred, d_map, d_codes, d_llr, d_off, d_shotcode};
  for (void *b : bufs) cudaFree(b);
  if (h_codes) cudaFreeHost(h_codes);
  if (h_status) cudaFreeHost(h_status);
  for (auto &e : ev) if (e) cudaEventDestroy(e);
  if (stream) cudaStreamDestroy(stream);
}

static int words_padded(int nw) {
  if (nw <= 2) return nw;
  if (nw <= 4) return 4;
  if (nw <= 8) return 8;
  return (nw + 3) & ~3;
}

// Binomials exactly as upstream's multiplicative nCr (grand_decoder.cu:42-52).
static unsigned long long ncr_host(int n, int k) {
  if (k < 0 || k > n) return 0;
  if (k == 0 || k == n) return 1;
  unsigned long long r = 1;
  for (int i = 1; i <= k; ++i) r = r * (unsigned long long)(n - i + 1) / (unsigned long long)i;
  return r;
}

Context *Context::get(int *err) {
  static std::mutex mu;
  static Context *ctxs[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_error("grand: no CUDA device available (%s)", cudaGetErrorString(e));
    *err = GRAND_ERR_CUDA;
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(mu);
  if (dev < 0 || dev >= 64) {
    *err = GRAND_ERR_CUDA;
    return nullptr;
  }
  if (ctxs[dev]) return ctxs[dev];
  cudaDeviceProp prop;
  e = cudaGetDeviceProperties(&prop, dev);
  if (e != cudaSuccess) {
    set_error("grand: cudaGetDeviceProperties failed (%s)", cudaGetErrorString(e));
    *err = GRAND_ERR_CUDA;
    return nullptr;
  }
  if (prop.major != 10 || prop.minor != 3) {
    set_error("grand: this library is built for sm_103a (GB300); device %d is sm_%d%d", dev,
              prop.major, prop.minor);
    *err = GRAND_ERR_CUDA;
    return nullptr;
  }
  Context *c = new Context();
  c->device = dev;
  c->sm_count = prop.multiProcessorCount;
  int pa = 0;
  cudaDeviceGetAttribute(&pa, cudaDevAttrPageableMemoryAccess, dev);
  c->pageable_access = pa;
  if (decode_occupancy(&c->decode_bps) != cudaSuccess || c->decode_bps < 1) c->decode_bps = 1;
  std::vector<unsigned long long> t((size_t)(kMaxTam + 1) * (kMaxW + 1));
  for (int n = 0; n <= kMaxTam; ++n)
    for (int k = 0; k <= kMaxW; ++k) t[(size_t)n * (kMaxW + 1) + k] = ncr_host(n, k);
  if (cudaMalloc(&c->d_ncr, t.size() * 8) != cudaSuccess ||
      cudaMemcpy(c->d_ncr, t.data(), t.size() * 8, cudaMemcpyHostToDevice) != cudaSuccess) {
    set_error("grand: could not upload the binomial table");
    *err = GRAND_ERR_CUDA;
    delete c;
    return nullptr;
  }
  ctxs[dev] = c;
  return c;
}

Workspace *Context::acquire() {
  {
    std::lock_guard<std::mutex> lk(mu_);
    if (!pool_.empty()) {
      Workspace *w = pool_.back();
      pool_.pop_back();
      return w;
    }
  }
  Workspace *w = new Workspace();
  if (cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete w;
    return nullptr;
  }
  for (auto &e : w->ev)
    if (cudaEventCreate(&e) != cudaSuccess) {
      delete w;
      return nullptr;
    }
  if (cudaHostAlloc(reinterpret_cast<void **>(&w->h_status), 256, cudaHostAllocDefault) !=
      cudaSuccess) {
    w->h_status = nullptr;
    delete w;
    return nullptr;
  }
  return w;
}

void Context::release(Workspace *w) {
  if (!w) return;
  std::lock_guard<std::mutex> lk(mu_);
  pool_.push_back(w);
}

// GF(2) reduced row echelon form of bit 0 of each entry (grand_decoder.cu:418-454).
static int rref_bits(std::vector<uint32_t> &rows, int n, int mw, int m, std::vector<int> &piv) {
  int r = 0;
  for (int c = 0; c < m && r < n; ++c) {
    const int q = c >> 5;
    const uint32_t bit = 1u << (c & 31);
    int p = -1;
    for (int i = r; i < n; ++i)
      if (rows[(size_t)i * mw + q] & bit) { p = i; break; }
    if (p < 0) continue;
    if (p != r)
      for (int j = 0; j < mw; ++j) std::swap(rows[(size_t)r * mw + j], rows[(size_t)p * mw + j]);
    for (int i = 0; i < n; ++i) {
      if (i == r || !(rows[(size_t)i * mw + q] & bit)) continue;
      for (int j = 0; j < mw; ++j) rows[(size_t)i * mw + j] ^= rows[(size_t)r * mw + j];
    }
    piv.push_back(c);
    ++r;
  }
  return r;
}

template <class T>
static cudaError_t upload(T **d, const std::vector<T> &h) {
  size_t bytes = std::max<size_t>(h.size() * sizeof(T), 16);
  cudaError_t e = cudaMalloc(d, bytes);
  if (e != cudaSuccess) return e;
  if (h.empty()) return cudaMemset(*d, 0, bytes);
  return cudaMemcpy(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
}

std::shared_ptr<CodeTables> Context::tables(int family, const int *H, const int *H_other,
                                            const int *L, int n, int m, int nl, int *err) {
  const size_t nm = (size_t)n * m;
  const int *second = family == kCss ? H_other : L;
  const size_t second_len = family == kCss ? nm : (size_t)m * nl;
  // Cache hit test: exact content comparison against the caller's arrays (no copy).
  auto same = [&](const CodeTables &c) {
    if (c.family != family || c.R != n || c.m != m || c.n_logicos != nl) return false;
    if (c.key.size() != 4 + nm + second_len) return false;
    if (memcmp(c.key.data() + 4, H, nm * sizeof(int)) != 0) return false;
    return second_len == 0 || memcmp(c.key.data() + 4 + nm, second, second_len * sizeof(int)) == 0;
  };
  {
    std::lock_guard<std::mutex> lk(mu_);
    for (size_t i = cache_.size(); i-- > 0;)
      if (same(*cache_[i])) {
        auto t = cache_[i];
        if (i + 1 != cache_.size()) {
          cache_.erase(cache_.begin() + i);
          cache_.push_back(t);
        }
        return t;
      }
  }
  std::vector<int> key;
  key.reserve(4 + nm + second_len);
  key.push_back(family);
  key.push_back(n);
  key.push_back(m);
  key.push_back(nl);
  key.insert(key.end(), H, H + nm);
  if (second_len) key.insert(key.end(), second, second + second_len);
  auto t = std::make_shared<CodeTables>();
  t->family = family;
  t->R = n;
  t->m = m;
  t->nw = (n + 31) / 32;
  t->nwp = words_padded(t->nw);
  t->mw = (m + 31) / 32;
  t->n_logicos = nl;
  t->nlw = (nl + 31) / 32;
  // columns packed LSB-first; statistics on the raw entries (grand_decoder.cu:376-404)
  std::vector<uint32_t> cols((size_t)m * t->nwp, 0u);
  std::vector<int> colw(m, 0);
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < m; ++c) {
      const int v = H[(size_t)r * m + c];
      colw[c] += v;
      if (v != 0) cols[(size_t)c * t->nwp + (r >> 5)] |= 1u << (r & 31);
    }
  t->max_soma = 0;
  for (int c = 0; c < m; ++c) t->max_soma = std::max(t->max_soma, colw[c]);
  t->regular = 1;
  for (int c = 1; c < m; ++c)
    if (colw[c] != colw[0]) { t->regular = 0; break; }
  std::vector<uint32_t> hcol(m, 0u);
  t->binary = 1;
  std::vector<int> lowrow(m, -1);  // lowest set row of each column
  for (int r = 0; r < n; ++r) {
    const uint32_t hr = row_hash(r);
    for (int c = 0; c < m; ++c) {
      const int v = H[(size_t)r * m + c];
      if (v != 0) {
        hcol[c] ^= hr;
        if (lowrow[c] < 0) lowrow[c] = r;
      }
      if (v != 0 && v != 1) t->binary = 0;
    }
  }
  // solo columns (nonzero, containing no other nonzero column) by sketch
  const SoloTable solo = build_solo_table(cols, t->nwp, t->nw, m, hcol);
  t->solo_mask = solo.mask;
  cudaError_t e = upload(&t->cols, cols);
  if (e == cudaSuccess) e = upload(&t->colw, colw);
  if (e == cudaSuccess) e = upload(&t->hcol, hcol);
  if (e == cudaSuccess) e = upload(&t->solo_keys, solo.keys);
  if (e == cudaSuccess) e = upload(&t->solo_cols, solo.cols);
  if (e == cudaSuccess && family == kCss) {
    std::vector<uint32_t> rows((size_t)n * t->mw, 0u);
    for (int r = 0; r < n; ++r)
      for (int c = 0; c < m; ++c)
        if (H_other[(size_t)r * m + c] & 1) rows[(size_t)r * t->mw + (c >> 5)] |= 1u << (c & 31);
    std::vector<int> piv;
    t->rank = rref_bits(rows, n, t->mw, m, piv);
    rows.resize((size_t)t->rank * t->mw);
    std::vector<int> pivrow(m, -1);
    for (int r = 0; r < t->rank; ++r) pivrow[piv[r]] = r;
    e = upload(&t->rref, rows);
    if (e == cudaSuccess) e = upload(&t->pivrow, pivrow);
  }
  if (e == cudaSuccess && family == kDem) {
    std::vector<uint32_t> lc((size_t)m * std::max(t->nlw, 1), 0u);
    for (int c = 0; c < m; ++c)
      for (int j = 0; j < nl; ++j)
        if (L[(size_t)c * nl + j] != 0) lc[(size_t)c * t->nlw + (j >> 5)] |= 1u << (j & 31);
    e = upload(&t->lcols, lc);
  }
  if (e != cudaSuccess) {
    set_error("grand: could not upload code tables (%s)", cudaGetErrorString(e));
    *err = GRAND_ERR_CUDA;
    return nullptr;
  }
  t->bytes = cols.size() * 4 + colw.size() * 4 + hcol.size() * 4 + key.size() * 4;
  t->key.swap(key);
  std::lock_guard<std::mutex> lk(mu_);
  cache_.push_back(t);
  cache_bytes_ += t->bytes;
  while (cache_.size() > 64 || (cache_bytes_ > (512u << 20) && cache_.size() > 1)) {
    cache_bytes_ -= cache_.front()->bytes;
    cache_.erase(cache_.begin());
  }
  return t;
}

DevCode make_devcode(const CodeTables &t, const CallParams &p) {
  DevCode d;
  memset(&d, 0, sizeof(d));
  d.R = t.R;
  d.m = t.m;
  d.nw = t.nw;
  d.nwp = t.nwp;
  d.mw = t.mw;
  d.max_soma = t.max_soma;
  d.regular = t.regular;
  d.family = t.family;
  d.variant = p.variant;
  d.input_kind = p.input_kind;
  d.W = p.W;
  d.Wc = std::min(p.W, (int)kMaxW);
  d.mode = p.mode;
  d.thr = p.thr;
  d.cap = p.cap;
  d.num_phases = p.num_phases;
  d.n_masks = p.n_masks;
  memcpy(d.mask_tam_upper, p.mask_tam_upper, sizeof(d.mask_tam_upper));
  memcpy(d.mask_order, p.mask_order, sizeof(d.mask_order));
  d.n_logicos = t.n_logicos;
  d.nlw = t.nlw;
  d.rank = t.rank;
  d.rec_len = p.rec_len ? p.rec_len : (p.input_kind == kInErrors ? t.m : t.R);
  d.packed = p.packed;
  d.cols = t.cols;
  d.colw = t.colw;
  d.rows = nullptr;
  d.rref = t.rref;
  d.pivrow = t.pivrow;
  d.lcols = t.lcols;
  d.llr = p.d_llr;
  d.hcol = t.hcol;
  d.binary = t.binary;
  d.solo_keys = t.solo_keys;
  d.solo_cols = t.solo_cols;
  d.solo_mask = t.solo_mask;
  return d;
}

int decode_blocks_per_sm(int occupancy_bps, const Tuning &tn) {
  const int occ = std::max(occupancy_bps, 1);
  return tn.search_grid_mult ? std::min(tn.search_grid_mult, occ) : occ;
}

cudaError_t launch_pipeline(const Context *ctx, const DevBatch &b, const Tuning &tn,
                            cudaStream_t s, cudaEvent_t mid) {
  cudaError_t e = cudaMemsetAsync(b.counters, 0, kCtlBytes, s);
  if (e != cudaSuccess) return e;
  if (mid) cudaEventRecord(mid, s);
  // persistent: as many blocks as are resident at once (fewer for a small batch,
  // whose shots and tiles would leave most warps idle)
  const int full = ctx->sm_count * decode_blocks_per_sm(ctx->decode_bps, tn);
  return launch_decode(b, full, s);
}

int run_batch(Context *ctx, Workspace *ws, const BatchRequest &req, BatchTiming *timing,
              const Tuning *tnp) {
  const int N = req.num_shots;
  if (N <= 0) return 0;
  cudaStream_t s = ws->stream;
  const Tuning &tn = tnp ? *tnp : tuning();
  const int ncodes = (int)req.codes.size();

  // Zero-copy: the GPU reads the caller's records and writes its results in
  // place, over NVLink-C2C, when the device can access pageable host memory.
  const bool zc = tn.zero_copy && ctx->pageable_access;
  if (!zc) {
    CK(ensure(&ws->d_in, &ws->cap_in, req.in_ints * sizeof(int)));
    if (req.h_in_log) CK(ensure(&ws->d_in2, &ws->cap_in2, req.in_log_ints * sizeof(int)));
    if (req.h_off) CK(ensure(&ws->d_off, &ws->cap_off, sizeof(long long) * N));
    if (req.h_shot_code) CK(ensure(&ws->d_shotcode, &ws->cap_shotcode, sizeof(int) * N));
    CK(ensure(&ws->d_res, &ws->cap_res, sizeof(GrandDecoderResult) * N));
    if (req.h_dec_err) CK(ensure(&ws->d_dec, &ws->cap_dec, (size_t)N * req.dec_m));
    if (req.h_dec_log) CK(ensure(&ws->d_declog, &ws->cap_declog, (size_t)N * std::max(req.dec_nl, 1)));
    if (req.h_cost) CK(ensure(&ws->d_cost, &ws->cap_cost, sizeof(float) * N));
  }
  const int max_jobs = std::min(N, 16384);
  CK(ensure_zeroed(&ws->d_jobs, &ws->cap_jobs, sizeof(Job) * max_jobs));
  const size_t scratch_words = 32ull << 20;
  CK(ensure(&ws->d_scratch, &ws->cap_scratch, scratch_words * 4));
  size_t small_cap = ws->d_small ? kCtlAllocBytes : 0;
  CK(ensure_zeroed(&ws->d_small, &small_cap, kCtlAllocBytes));
  CK(ensure_zeroed(&ws->d_deferred, &ws->cap_deferred, shot_buffer_bytes(N)));

  // Per-call host work is kept to the launches, one status read and one
  // synchronisation; events are recorded only when the caller asks for times,
  // and the DevCode array is uploaded only when it differs from the last one.
  const bool timed = timing != nullptr;
  const size_t code_bytes = sizeof(DevCode) * ncodes;
  void *codes_before = ws->d_codes;
  CK(ensure(&ws->d_codes, &ws->cap_codes, code_bytes));
  const bool send_codes = ws->d_codes != codes_before || ws->sent_codes.size() != code_bytes ||
                          memcmp(ws->sent_codes.data(), req.codes.data(), code_bytes) != 0;
  if (send_codes && ws->cap_hcodes < code_bytes) {
    // the previous copy from this buffer may still be in flight on this stream
    CK(cudaStreamSynchronize(s));
    if (ws->h_codes) cudaFreeHost(ws->h_codes);
    ws->h_codes = nullptr;
    ws->cap_hcodes = 0;
    CK(cudaHostAlloc(&ws->h_codes, std::max<size_t>(code_bytes, 4096), cudaHostAllocDefault));
    ws->cap_hcodes = std::max<size_t>(code_bytes, 4096);
  }
  if (timed) CK(cudaEventRecord(ws->ev[0], s));
  if (send_codes) {
    memcpy(ws->h_codes, req.codes.data(), code_bytes);  // stream is idle between calls
    CK(cudaMemcpyAsync(ws->d_codes, ws->h_codes, code_bytes, cudaMemcpyHostToDevice, s));
    ws->sent_codes.assign(reinterpret_cast<const unsigned char *>(req.codes.data()),
                          reinterpret_cast<const unsigned char *>(req.codes.data()) + code_bytes);
  }
  if (!zc) {
    CK(cudaMemcpyAsync(ws->d_in, req.h_in, req.in_ints * sizeof(int), cudaMemcpyHostToDevice, s));
    if (req.h_in_log)
      CK(cudaMemcpyAsync(ws->d_in2, req.h_in_log, req.in_log_ints * sizeof(int),
                         cudaMemcpyHostToDevice, s));
    if (req.h_off)
      CK(cudaMemcpyAsync(ws->d_off, req.h_off, sizeof(long long) * N, cudaMemcpyHostToDevice, s));
    if (req.h_shot_code)
      CK(cudaMemcpyAsync(ws->d_shotcode, req.h_shot_code, sizeof(int) * N,
                         cudaMemcpyHostToDevice, s));
  }
  if (timed) CK(cudaEventRecord(ws->ev[1], s));

  DevBatch b;
  memset(&b, 0, sizeof(b));
  b.num_codes = ncodes;
  b.codes = (const DevCode *)ws->d_codes;
  if (zc) {
    b.in = req.h_in;
    b.in_off = req.h_off;
    b.in_log = req.h_in_log;
    b.shot_code = req.h_shot_code;
    b.results = req.h_results;
    b.dec_err = req.h_dec_err;
    b.dec_log = req.h_dec_log;
    b.ml_cost = req.h_cost;
  } else {
    b.in = (const int *)ws->d_in;
    b.in_off = req.h_off ? (const long long *)ws->d_off : nullptr;
    b.in_log = req.h_in_log ? (const int *)ws->d_in2 : nullptr;
    b.shot_code = req.h_shot_code ? (const int *)ws->d_shotcode : nullptr;
    b.results = (GrandDecoderResult *)ws->d_res;
    b.dec_err = req.h_dec_err ? (unsigned char *)ws->d_dec : nullptr;
    b.dec_log = req.h_dec_log ? (unsigned char *)ws->d_declog : nullptr;
    b.ml_cost = req.h_cost ? (float *)ws->d_cost : nullptr;
  }
  b.ncr = ctx->d_ncr;
  b.jobs = (Job *)ws->d_jobs;
  b.max_jobs = max_jobs;
  b.counters = (unsigned long long *)ws->d_small;
  b.status = (unsigned *)((char *)ws->d_small + kStatusByteOffset);
  b.scratch = (uint32_t *)ws->d_scratch;
  b.scratch_words = scratch_words;
  b.deferred = (int *)ws->d_deferred;
  b.queue = shot_queue(ws->d_deferred, N);
  // records read in place from host memory: the per-shot path takes the bits the
  // chunk step kept instead of a second read over NVLink-C2C
  b.rec_cache = zc ? shot_rec_cache(ws->d_deferred, N) : nullptr;
  b.epoch = (unsigned *)((char *)ws->d_small + kCtlBytes);
  b.fast = tn.fast;
  b.profile = tn.profile;
  b.light_max_log2 = tn.light_max_log2;
  b.tile_k = tn.tile_k;
  for (const DevCode &c : req.codes) b.has_ml |= c.variant == kMl;

  std::vector<int> map;
  int todo = N;
  float tri_ms = 0, sea_ms = 0;
  int rounds = 0;
  unsigned status_all = 0;
  for (;;) {
    b.num_shots = todo;
    b.shot_map = rounds == 0 ? nullptr : (const int *)ws->d_map;
    if (timed) CK(cudaEventRecord(ws->ev[2], s));
    CK(launch_pipeline(ctx, b, tn, s, timed ? ws->ev[3] : nullptr));
    if (timed) CK(cudaEventRecord(ws->ev[4], s));
    CK(cudaMemcpyAsync(ws->h_status, b.status, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    const unsigned st = *ws->h_status;
    if (timed) {
      float a = 0, c = 0;
      cudaEventElapsedTime(&a, ws->ev[2], ws->ev[3]);
      cudaEventElapsedTime(&c, ws->ev[3], ws->ev[4]);
      tri_ms += a;
      sea_ms += c;
    }
    ++rounds;
    status_all |= st;
    if (!(st & (kStatusJobOverflow | kStatusScratchOverflow))) break;
    // Re-run the shots that did not fit the job table or scratch.
    std::vector<int> def(N);
    CK(cudaMemcpy(def.data(), ws->d_deferred, sizeof(int) * N, cudaMemcpyDeviceToHost));
    std::vector<int> prev = map;
    map.clear();
    if (rounds == 1) {
      for (int i = 0; i < N; ++i) if (def[i]) map.push_back(i);
    } else {
      for (int i : prev) if (def[i]) map.push_back(i);
    }
    if (map.empty() || rounds > 64) break;
    todo = (int)map.size();
    CK(ensure(&ws->d_map, &ws->cap_map, sizeof(int) * map.size()));
    CK(cudaMemcpyAsync(ws->d_map, map.data(), sizeof(int) * map.size(), cudaMemcpyHostToDevice, s));
  }

  if (timed) CK(cudaEventRecord(ws->ev[4], s));
  if (!zc) {
    CK(cudaMemcpyAsync(req.h_results, ws->d_res, sizeof(GrandDecoderResult) * N,
                       cudaMemcpyDeviceToHost, s));
    if (req.h_dec_err)
      CK(cudaMemcpyAsync(req.h_dec_err, ws->d_dec, (size_t)N * req.dec_m, cudaMemcpyDeviceToHost, s));
    if (req.h_dec_log && req.dec_nl > 0)
      CK(cudaMemcpyAsync(req.h_dec_log, ws->d_declog, (size_t)N * req.dec_nl,
                         cudaMemcpyDeviceToHost, s));
    if (req.h_cost)
      CK(cudaMemcpyAsync(req.h_cost, ws->d_cost, sizeof(float) * N, cudaMemcpyDeviceToHost, s));
  }
  if (timed) CK(cudaEventRecord(ws->ev[5], s));
  if (!zc || timed) CK(cudaStreamSynchronize(s));
  if (timing) {
    float h2d = 0, d2h = 0;
    cudaEventElapsedTime(&h2d, ws->ev[0], ws->ev[1]);
    cudaEventElapsedTime(&d2h, ws->ev[4], ws->ev[5]);
    timing->h2d_ms = h2d;
    timing->reset_ms = tri_ms;
    timing->decode_ms = sea_ms;
    timing->d2h_ms = d2h;
    timing->rounds = rounds;
  }
  if (status_all & kStatusTamLimit) {
    set_error("grand: an active-position set exceeded GRAND_MAX_TAM=%d; those shots are "
              "reported unsearched", kMaxTam);
    return GRAND_ERR_LIMIT;
  }
  if (status_all & kStatusCasLimit) {
    set_error("grand: internal ML reduction retry limit reached");
    return GRAND_ERR_CUDA;
  }
  return 0;
}

}  // namespace grand
