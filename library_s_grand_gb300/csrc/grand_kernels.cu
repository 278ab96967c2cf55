// grand_kernels.cu -- the two kernels of one decoding launch (sm_103a).
//
// triage_kernel (one warp per shot, grid-stride over the batch)
//   packs the shot's int32 record into bits, forms the syndrome, computes the
//   flagged-check count of every column (popc(col & s), upstream
//   grand_decoder.cu:67-81 / 352-374, with the irregular offset of :406-416),
//   the active sets of the <= 3 threshold iterations (:1284-1290, :495-504),
//   the upstream active-set cap and mode rules (:1296, :1327, :1550-1554), and
//   the weight blocks each searched iteration enumerates.  The iterations are
//   searched in upstream order by the same warp while each fits the light
//   budget; the first larger one and those after it become a Job for the
//   persistent search kernel.
//
// search_kernel (persistent, every warp an independent worker)
//   every warp repeatedly takes the next tiles (K colex prefixes per lane of
//   one weight block of one Job) from a global counter, stages the iteration's
//   active columns in its own shared-memory slice, evaluates them, publishes
//   the lowest matching global index (atomicMin) or the lowest {cost, rank}
//   key (128-bit CAS), and the warp that completes a Job's last tile writes its
//   result.  Tiles whose candidates all rank above an already-found match are
//   skipped.  No warp ever waits for another: there are no block barriers.
#include <cuda_runtime.h>

#include "grand_device.cuh"

namespace grand {

constexpr int kTriageWarps = 4;
constexpr int kLightTam = 96;
constexpr int kLightWords = kLightTam * 8;
constexpr int kSearchThreads = 256;
constexpr int kSearchWarps = kSearchThreads / 32;
constexpr int kWarpStage = 1280;  // staged active-column words per search warp
constexpr int kTilesPerFetch = 4;
constexpr int kRunKK = 8;       // prefixes per lane in a run tile (search kernel)
constexpr int kRunKKLight = 4;  // the same inside the triage warp's light search

struct alignas(16) WarpArea {
  uint32_t cols[kLightWords];
  float llr[kLightTam];
  int pos[kLightTam];
  int tmp[kLightTam];
  uint32_t sw[kMaxRows / 32];
  uint32_t eb[kMaxCols / 32];
  uint32_t am[kMaxIters][kMaxCols / 32];
  uint32_t delta[kMaxCols / 32];
  Job job;
};

// ---------------------------------------------------------------------------
// Planning: the threshold iterations and their weight blocks (lane 0 only).
// The planner is resumable: each call walks upstream's iteration loop
// (grand_decoder.cu:1284-1343) to the next iteration that is searched, appends
// it and its weight blocks to the Job and returns 1, or records the outcome
// fields of an exhausted loop and returns 0.  Shots usually resolve in their
// first searched iteration, so later iterations are only planned when needed.
// ---------------------------------------------------------------------------
struct PlanState {
  int i, tam, tam_old, passes;
  unsigned long long gbase;
};

__device__ int plan_next(const DevCode &cd, const unsigned long long *t, const int (&tam_raw)[3],
                         int L, int tile_k, Job &J, PlanState &P) {
  while (P.i < L) {
    const int i = P.i++;
    P.passes = i + 1;
    int tam = tam_raw[i];
    if (cd.family == kDem) {  // grand_decoder.cu:1550-1554
      if (tam > cd.cap) tam = P.tam_old;
      else P.tam_old = tam;
    }
    P.tam = tam;
    if (tam <= 0) continue;
    const bool gpu = (tam > cd.thr && tam <= cd.cap && cd.mode == 1) || cd.mode == 0;
    const bool cpu = !gpu && ((tam <= cd.thr && cd.mode == 1) || cd.mode == -1);
    if (!gpu && !cpu) continue;
    if (tam > kMaxTam) {
      J.failed = 1;
      continue;
    }
    IterInfo &I = J.it[J.n_it];
    I.it = i + 1;
    I.tam = tam;
    I.branch = gpu ? kBranchGpu : kBranchCpu;
    I.src = i;
    I.seg_lo = J.nseg;
    I.base = P.gbase;
    I.phase_end[0] = I.phase_end[1] = I.phase_end[2] = 0;
    unsigned long long tot = 0;
    int wl[kMaxSegsPerIter], ph[kMaxSegsPerIter], nwl = 0;
    if (cd.variant == kProb) {
      int mi = cd.n_masks - 1;  // grand_decoder.cu:754-762
      for (int q = 0; q < cd.n_masks; ++q)
        if (tam <= cd.mask_tam_upper[q]) { mi = q; break; }
      for (int k = 0; k < cd.num_phases; ++k) {  // grand_decoder.cu:764-786
        const int pid = cd.mask_order[mi][k];
        if (pid == 0) {
          for (int w = 1; w <= 5 && w <= tam && w <= kMaxW; ++w) { wl[nwl] = w; ph[nwl++] = k; }
        } else if (pid == 1) {
          if (6 <= tam && 6 <= kMaxW) { wl[nwl] = 6; ph[nwl++] = k; }
        }
      }
    } else {
      const int wmax = cd.Wc < tam ? cd.Wc : tam;
      for (int w = 1; w <= wmax; ++w) { wl[nwl] = w; ph[nwl++] = 0; }
    }
    unsigned seen = 0;
    for (int q = 0; q < nwl; ++q) {
      Seg &S = J.seg[J.nseg++];
      S.iter = J.n_it;
      S.w = wl[q];
      S.phase = ph[q];
      S.dup = (seen >> S.w) & 1u;
      seen |= 1u << S.w;
      S.count = ncr(t, tam, S.w);
      S.base = P.gbase + tot;
      S.nprefix = ncr(t, tam - 1, S.w - 1);
      S.runs = (S.w >= 3 && cd.nw <= 8) ? 1 : 0;
      S.cum = nullptr;
      S.K = S.runs ? kRunKK : (S.w <= 2 ? 1 : tile_k);
      // run-tile counts are built by the warp when a Job is published
      S.ntiles = S.runs ? 0ull : (S.nprefix + 32ull * S.K - 1) / (32ull * S.K);
      tot += S.count;
      if (cd.variant == kProb) I.phase_end[S.phase] = tot;
    }
    if (cd.variant == kProb)  // phases without weights keep the running total
      for (int k = 1; k < 3; ++k)
        if (I.phase_end[k] < I.phase_end[k - 1]) I.phase_end[k] = I.phase_end[k - 1];
    I.seg_hi = J.nseg;
    I.total = tot;
    P.gbase += tot;
    J.n_it++;
    return 1;
  }
  J.final_iteration = P.passes;
  J.final_tam = P.tam;
  return 0;
}

// ---------------------------------------------------------------------------
// Result writer shared by the light path and the search kernel (one warp).
// ---------------------------------------------------------------------------
struct Winner {
  int found;
  int ii;                   // index into J.it
  int seg;                  // index into J.seg
  unsigned long long rank;  // lexicographic rank inside the weight block
  unsigned long long count; // candidates the winning iteration reports
  float cost;
};

__device__ void finish_shot(const DevBatch &b, const DevCode &cd, const Job &J, int shot,
                            const Winner &wn, const uint32_t *ebits, uint32_t *delta) {
  const int lane = threadIdx.x & 31;
  int p[kMaxW];
  int w = 0;
  if (wn.found) {
    const Seg &S = J.seg[wn.seg];
    const IterInfo &I = J.it[wn.ii];
    w = S.w;
    int c[kMaxW];
    lex_unrank(b.ncr, wn.rank, I.tam, w, c);
#pragma unroll
    for (int i = 0; i < kMaxW; ++i) p[i] = (i < w) ? I.pos[c[i]] : -1;
  } else {
#pragma unroll
    for (int i = 0; i < kMaxW; ++i) p[i] = -1;
  }

  int degenerate = 0, is_equal = 0;
  if (wn.found && cd.family == kCss && cd.input_kind == kInErrors) {
    // is_equal: supplied error == decoded error (grand_decoder.cu:1362).
    bool eq = true;
    for (int q = lane; q < cd.mw; q += 32) {
      uint32_t e = 0;
#pragma unroll
      for (int i = 0; i < kMaxW; ++i)
        if (i < w && (p[i] >> 5) == q) e |= 1u << (p[i] & 31);
      uint32_t d = ebits[q] ^ e;
      delta[q] = d;
      eq = eq && d == 0u;
    }
    is_equal = __all_sync(kFull, eq) ? 1 : 0;
    __syncwarp();
    // degenerate: (e ^ e_est) in the row space of the other matrix
    // (grand_decoder.cu:456-474).  In reduced row echelon form the vector's own
    // bits at pivot columns decide alone which rows upstream adds, so the test
    // is delta == XOR of the rows pivoted on delta's set bits.
    uint32_t acc[4] = {0u, 0u, 0u, 0u};  // words lane, lane+32, lane+64, lane+96
    for (int q = 0; q < cd.mw; ++q) {
      uint32_t word = delta[q];
      while (word) {
        const int c = q * 32 + __ffs(word) - 1;
        word &= word - 1u;
        const int r = __ldg(cd.pivrow + c);
        if (r < 0) continue;
#pragma unroll
        for (int k = 0; k < 4; ++k)
          if (lane + 32 * k < cd.mw) acc[k] ^= __ldg(cd.rref + (size_t)r * cd.mw + lane + 32 * k);
      }
    }
    bool ok = true;
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (lane + 32 * k < cd.mw) ok = ok && acc[k] == delta[lane + 32 * k];
    degenerate = __all_sync(kFull, ok) ? 1 : 0;
  } else if (wn.found && cd.family == kDem) {
    // decoded logical flips vs the supplied true flips (grand_decoder.cu:1623-1644)
    bool eq = true;
    for (int q = lane; q < cd.nlw; q += 32) {
      uint32_t le = 0;
#pragma unroll
      for (int i = 0; i < kMaxW; ++i)
        if (i < w) le ^= __ldg(cd.lcols + (size_t)p[i] * cd.nlw + q);
      eq = eq && le == ebits[q];
      if (b.dec_log) {
        for (int j = 0; j < 32 && q * 32 + j < cd.n_logicos; ++j)
          b.dec_log[(size_t)shot * cd.n_logicos + q * 32 + j] = (unsigned char)((le >> j) & 1u);
      }
    }
    degenerate = __all_sync(kFull, eq) ? 1 : 0;
  } else if (cd.family == kDem && b.dec_log) {
    for (int j = lane; j < cd.n_logicos; j += 32) b.dec_log[(size_t)shot * cd.n_logicos + j] = 0;
  }

  if (b.dec_err) {
    for (int c = lane; c < cd.m; c += 32) {
      unsigned char v = 0;
#pragma unroll
      for (int i = 0; i < kMaxW; ++i)
        if (i < w && p[i] == c) v = 1;
      b.dec_err[(size_t)shot * cd.m + c] = v;
    }
  }

  if (lane == 0) {
    int h = -2;
    unsigned long long tested = 0;
    const int last = wn.found ? wn.ii : J.n_it - 1;
    for (int k = 0; k <= last; ++k) {
      h = (J.it[k].branch == kBranchGpu) ? (h == -1 ? 1 : 0) : -1;
      if (k < last || !wn.found) tested += J.it[k].total;
    }
    if (wn.found) tested += wn.count;
    GrandDecoderResult r;
    r.found = wn.found;
    r.found_weight = w;
    r.original_weight = J.original_weight;
    r.degenerate = degenerate;
    r.is_equal = is_equal;
    r.tam = wn.found ? J.it[wn.ii].tam : J.final_tam;
    r.total_tested_combinations = tested;
    r.hibrido = h;
    r.iteration = wn.found ? J.it[wn.ii].it : J.final_iteration;
    r.time_sum_ms = 0.0;
    r.total_time_search_ms = 0.0;
    r.transfer_time_ms = 0.0;
    r.total_to_find_ms = 0.0;
    b.results[shot] = r;
    if (b.ml_cost) b.ml_cost[shot] = wn.found ? wn.cost : 0.0f;
    if (J.failed) atomicOr(b.status, kStatusTamLimit);
  }
}

// Winner of a first-hit search from the lowest matching global index.
__device__ Winner winner_from_index(const Job &J, unsigned long long g, bool prob) {
  Winner wn;
  wn.found = 0;
  wn.ii = wn.seg = 0;
  wn.rank = wn.count = 0;
  wn.cost = 0.0f;
  if (g == kNone) return wn;
  for (int ii = 0; ii < J.n_it; ++ii) {
    const IterInfo &I = J.it[ii];
    if (g < I.base || g >= I.base + I.total) continue;
    for (int s = I.seg_lo; s < I.seg_hi; ++s) {
      const Seg &S = J.seg[s];
      if (S.dup || g < S.base || g >= S.base + S.count) continue;
      wn.found = 1;
      wn.ii = ii;
      wn.seg = s;
      wn.rank = g - S.base;
      if (I.branch == kBranchCpu) wn.count = g - I.base + 1ull;  // grand_decoder.cu:547-548
      else if (prob) wn.count = I.phase_end[S.phase];            // grand_decoder.cu:1006
      else wn.count = I.total;                                   // grand_decoder.cu:1303-1304
      return wn;
    }
  }
  return wn;
}

// ---------------------------------------------------------------------------
// Staging of one iteration's active set (positions, columns, LLRs).
// ---------------------------------------------------------------------------
__device__ void stage_iteration(const DevCode &cd, const uint32_t *am, int tam, int *pos,
                                int *tmp, uint32_t *cols, float *llr) {
  const int lane = threadIdx.x & 31;
  const bool ml = cd.variant == kMl;
  int *dst = ml ? tmp : pos;
  // ascending column indices of the first tam set bits (upstream extract_positions)
  int base = 0;
  for (int q = 0; q < cd.mw && base < tam; ++q) {
    const uint32_t word = am[q];
    const bool bit = (word >> lane) & 1u;
    const int idx = base + __popc(word & ((1u << lane) - 1u));
    if (bit && idx < tam) dst[idx] = q * 32 + lane;
    base += __popc(word);
  }
  __syncwarp();
  if (ml) {
    // stable sort by LLR ascending (upstream insertion sort, grand_decoder.cu:598-610)
    for (int i = lane; i < tam; i += 32) {
      const float key = __ldg(cd.llr + tmp[i]);
      int r = 0;
      for (int j = 0; j < tam; ++j) {
        const float kj = __ldg(cd.llr + tmp[j]);
        r += (kj < key) || (kj == key && j < i);
      }
      pos[r] = tmp[i];
    }
    __syncwarp();
  }
  const int nwp = cd.nwp;
  for (int idx = lane; idx < tam * nwp; idx += 32) {
    const int i = idx / nwp;
    cols[idx] = __ldg(cd.cols + (size_t)pos[i] * nwp + (idx - i * nwp));
  }
  if (ml)
    for (int i = lane; i < tam; i += 32) llr[i] = __ldg(cd.llr + pos[i]);
  __syncwarp();
}

// ---------------------------------------------------------------------------
// Evaluation dispatch on the column word count.
// ---------------------------------------------------------------------------
template <bool ML>
__device__ __forceinline__ void eval_dispatch(int nw, const SegView &sv,
                                              const unsigned long long *t, const uint32_t *sw,
                                              unsigned long long tile, LaneBest &lb) {
  switch (nw) {
    case 1: eval_tile<1, ML>(sv, t, sw, tile, lb); break;
    case 2: eval_tile<2, ML>(sv, t, sw, tile, lb); break;
    case 3: eval_tile<3, ML>(sv, t, sw, tile, lb); break;
    case 4: eval_tile<4, ML>(sv, t, sw, tile, lb); break;
    case 5: eval_tile<5, ML>(sv, t, sw, tile, lb); break;
    case 6: eval_tile<6, ML>(sv, t, sw, tile, lb); break;
    case 7: eval_tile<7, ML>(sv, t, sw, tile, lb); break;
    case 8: eval_tile<8, ML>(sv, t, sw, tile, lb); break;
    default: eval_tile<0, ML>(sv, t, sw, tile, lb); break;
  }
}

template <bool ML, int KK>
__device__ __forceinline__ void eval_run_dispatch(int nw, const SegView &sv,
                                                  const unsigned long long *t, const uint32_t *sw,
                                                  int c, unsigned long long r0, LaneBest &lb) {
  switch (nw) {
    case 1: eval_run_tile<1, KK, ML>(sv, t, sw, c, r0, lb); break;
    case 2: eval_run_tile<2, KK, ML>(sv, t, sw, c, r0, lb); break;
    case 3: eval_run_tile<3, KK, ML>(sv, t, sw, c, r0, lb); break;
    case 4: eval_run_tile<4, KK, ML>(sv, t, sw, c, r0, lb); break;
    case 5: eval_run_tile<5, KK, ML>(sv, t, sw, c, r0, lb); break;
    case 6: eval_run_tile<6, KK, ML>(sv, t, sw, c, r0, lb); break;
    case 7: eval_run_tile<7, KK, ML>(sv, t, sw, c, r0, lb); break;
    default: eval_run_tile<8, KK, ML>(sv, t, sw, c, r0, lb); break;
  }
}

// Every tile of one weight block, in order, by one warp (light path).
template <bool ML>
__device__ void eval_segment(const DevCode &cd, const SegView &sv, const Seg &S,
                             const unsigned long long *t, const uint32_t *sw, LaneBest &lb) {
  if (S.runs) {
    const unsigned long long per = 32ull * kRunKKLight;
    for (int c = S.w - 2; c <= sv.tam - 2; ++c) {
      const unsigned long long nt = run_tiles(t, c, S.w, kRunKKLight);
      for (unsigned long long q = 0; q < nt; ++q)
        eval_run_dispatch<ML, kRunKKLight>(cd.nw, sv, t, sw, c, q * per, lb);
    }
  } else {
    for (unsigned long long tile = 0; tile < S.ntiles; ++tile)
      eval_dispatch<ML>(cd.nw, sv, t, sw, tile, lb);
  }
}

// ---------------------------------------------------------------------------
// Kernel 1: triage + light search.
// ---------------------------------------------------------------------------
__device__ void light_search(const DevBatch &b, const DevCode &cd, Job &J, WarpArea &A, int ii,
                             Winner &wn) {
  const int lane = threadIdx.x & 31;
  const bool ml = cd.variant == kMl;
  IterInfo &I = J.it[ii];
  stage_iteration(cd, A.am[I.src], I.tam, A.pos, A.tmp, A.cols, A.llr);
  if (lane == 0) {
    I.pos = A.pos;
    I.cols = A.cols;
    I.llr = A.llr;
    if (ml) {
      float pf = 0.0f;
      I.prefix[0] = 0.0f;
      for (int w = 1; w <= kMaxW; ++w) {
        if (w <= I.tam) pf = __fadd_rn(pf, A.llr[w - 1]);
        I.prefix[w] = pf;
      }
    }
  }
  __syncwarp();
  if (!ml) {
    for (int s = I.seg_lo; s < I.seg_hi && !wn.found; ++s) {
      const Seg &S = J.seg[s];
      if (S.dup) continue;
      SegView sv{A.cols, A.llr, I.tam, S.w, S.K, cd.nwp, cd.nw, S.nprefix, S.base};
      LaneBest lb;
      lb.reset();
      eval_segment<false>(cd, sv, S, b.ncr, A.sw, lb);
      const unsigned long long g = warp_min_u64(lb.g);
      if (g != kNone) wn = winner_from_index(J, g, cd.variant == kProb);
    }
    return;
  }
  // upstream search_cpu_ml (grand_decoder.cu:620-656), one weight at a time
  uint32_t bo = 0xffffffffu;
  unsigned long long br = kNone, proc = 0;
  int bseg = -1;
  for (int s = I.seg_lo; s < I.seg_hi; ++s) {
    const Seg &S = J.seg[s];
    if (bseg >= 0 && I.prefix[S.w] >= key_cost(bo)) break;
    proc += S.count;
    SegView sv{A.cols, A.llr, I.tam, S.w, S.K, cd.nwp, cd.nw, S.nprefix, S.base};
    LaneBest lb;
    lb.reset();
    eval_segment<true>(cd, sv, S, b.ncr, A.sw, lb);
    uint32_t o = lb.o;
    unsigned long long r = lb.r;
    warp_min_key(o, r);
    if (o != 0xffffffffu && (bseg < 0 || o < bo)) {
      bo = o;
      br = r;
      bseg = s;
    }
  }
  if (bseg >= 0) {
    wn.found = 1;
    wn.ii = ii;
    wn.seg = bseg;
    wn.rank = br;
    wn.count = (I.branch == kBranchCpu) ? proc : I.total;
    wn.cost = key_cost(bo);
  }
}

__global__ void __launch_bounds__(kTriageWarps * 32) triage_kernel(DevBatch b) {
  __shared__ WarpArea areas[kTriageWarps];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  WarpArea &A = areas[wib];
  const int gw = blockIdx.x * kTriageWarps + wib;
  const int nwarps = gridDim.x * kTriageWarps;

  for (int slot = gw; slot < b.num_shots; slot += nwarps) {
    const int shot = b.shot_map ? b.shot_map[slot] : slot;
    const int ci = b.shot_code ? b.shot_code[shot] : 0;
    const DevCode &cd = b.codes[ci];
    const int *rec = b.in + (b.in_off ? b.in_off[shot] : (long long)shot * cd.rec_len);
    Job &J = A.job;

    // ---- pack the record ---------------------------------------------------
    uint32_t s_lane = 0;  // lane w holds syndrome word w
    int original_weight = 0;
    if (cd.input_kind == kInErrors) {
      for (int q = 0; q < cd.mw; ++q) {
        const int c = q * 32 + lane;
        const int v = c < cd.m ? rec[c] : 0;
        const uint32_t bits = __ballot_sync(kFull, v != 0);
        if (lane == 0) A.eb[q] = bits;
        original_weight += __popc(bits);
      }
      __syncwarp();
      // s = XOR of the columns of the supplied error (grand_decoder.cu:476-486)
      for (int q = 0; q < cd.mw; ++q) {
        uint32_t word = A.eb[q];
        while (word) {
          const int c = q * 32 + __ffs(word) - 1;
          word &= word - 1u;
          if (lane < cd.nw) s_lane ^= __ldg(cd.cols + (size_t)c * cd.nwp + lane);
        }
      }
    } else {
      for (int q = 0; q < cd.nw; ++q) {
        const int r = q * 32 + lane;
        const int v = r < cd.R ? rec[r] : 0;
        const uint32_t bits = __ballot_sync(kFull, v != 0);
        if (lane == q) s_lane = bits;
      }
      if (cd.family == kDem) {
        const int *lg = b.in_log ? b.in_log + (size_t)shot * cd.n_logicos : rec + cd.R;
        for (int q = 0; q < cd.nlw; ++q) {
          const int j = q * 32 + lane;
          const int v = j < cd.n_logicos ? lg[j] : 0;
          const uint32_t bits = __ballot_sync(kFull, v != 0);
          if (lane == 0) A.eb[q] = bits;
        }
      }
    }
    A.sw[lane] = (lane < cd.nw) ? s_lane : 0u;
    int ws = __popc(s_lane);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ws += __shfl_xor_sync(kFull, ws, o);
    __syncwarp();

    if (ws == 0) {  // grand_decoder.cu:1223-1241: nothing to search
      if (lane == 0) {
        GrandDecoderResult r = {};
        r.original_weight = original_weight;
        r.hibrido = -2;
        b.results[shot] = r;
        if (b.ml_cost) b.ml_cost[shot] = 0.0f;
      }
      if (b.dec_err)
        for (int c = lane; c < cd.m; c += 32) b.dec_err[(size_t)shot * cd.m + c] = 0;
      if (b.dec_log && cd.family == kDem)
        for (int j = lane; j < cd.n_logicos; j += 32) b.dec_log[(size_t)shot * cd.n_logicos + j] = 0;
      if (b.deferred && lane == 0) b.deferred[shot] = 0;
      __syncwarp();
      continue;
    }

    // ---- flagged-check counts and threshold masks ---------------------------
    const int L = cd.max_soma < kMaxIters ? cd.max_soma : kMaxIters;
    int tam_raw[3] = {0, 0, 0};
    for (int q = 0; q < cd.mw; ++q) {
      const int c = q * 32 + lane;
      int sum = 0;
      if (c < cd.m) {
        const uint32_t *col = cd.cols + (size_t)c * cd.nwp;
        for (int k = 0; k < cd.nw; ++k) sum += __popc(__ldg(col + k) & A.sw[k]);
        if (!cd.regular) {
          const int cw = __ldg(cd.colw + c);
          sum = cw == 0 ? 0 : sum + (cd.max_soma - cw);
        }
      }
#pragma unroll
      for (int i = 0; i < kMaxIters; ++i) {
        const uint32_t bits = __ballot_sync(kFull, c < cd.m && i < L && sum >= cd.max_soma - i);
        if (lane == 0) A.am[i][q] = bits;
        tam_raw[i] += __popc(bits);
      }
    }
    __shared__ PlanState plans[kTriageWarps];
    PlanState &P = plans[wib];
    if (lane == 0) {
      J.n_it = 0;
      J.nseg = 0;
      J.failed = 0;
      J.final_iteration = 0;
      J.final_tam = 0;
      P.i = 0;
      P.tam = 0;
      P.tam_old = 0;
      P.passes = 0;
      P.gbase = 0;
      J.shot = shot;
      J.code = ci;
      J.original_weight = original_weight;
      J.best = kNone;
      J.tiles_done = 0;
    }

    // ---- iterations in upstream order; the first one over the light budget
    //      and everything after it go to the search kernel ---------------------
    const bool ml = cd.variant == kMl;
    const unsigned long long budget = 1ull << b.light_max_log2;
    Winner wn;
    wn.found = 0;
    wn.ii = wn.seg = 0;
    wn.rank = wn.count = 0;
    wn.cost = 0.0f;
    int heavy_from = -1;
    for (;;) {
      int more = 0;
      if (lane == 0) more = plan_next(cd, b.ncr, tam_raw, L, b.tile_k, J, P);
      more = __shfl_sync(kFull, more, 0);
      __syncwarp();
      if (!more) break;
      const int ii = J.n_it - 1;
      const IterInfo &I = J.it[ii];
      if (I.total > budget || I.tam > kLightTam || I.tam * cd.nwp > kLightWords) {
        heavy_from = ii;
        if (lane == 0)
          while (plan_next(cd, b.ncr, tam_raw, L, b.tile_k, J, P)) {
          }
        __syncwarp();
        break;
      }
      light_search(b, cd, J, A, ii, wn);
      if (wn.found) break;
    }
    if (heavy_from < 0) {
      finish_shot(b, cd, J, shot, wn, A.eb, A.delta);
      if (b.deferred && lane == 0) b.deferred[shot] = 0;
      __syncwarp();
      continue;
    }

    // ---- heavy: publish a Job ------------------------------------------------
    unsigned long long words = 0;
    for (int ii = heavy_from; ii < J.n_it; ++ii) {
      const unsigned long long tm = (unsigned long long)J.it[ii].tam;
      words += (tm * cd.nwp + 3ull) & ~3ull;              // columns
      words += ((ml ? 2ull : 1ull) * tm + 3ull) & ~3ull;  // positions (+ sort buffer)
      if (ml) words += (tm + 3ull) & ~3ull;               // LLRs
    }
    for (int s = 0; s < J.nseg; ++s) {
      const Seg &S = J.seg[s];
      if (S.runs && !S.dup && S.iter >= heavy_from)
        words += (2ull * (unsigned long long)J.it[S.iter].tam + 3ull) & ~3ull;  // run-tile table
    }
    words += 128;  // supplied bits
    unsigned long long off = 0, jslot = 0, tbase = 0, ntl = 0;
    int ok = 1;
    if (lane == 0) {
      off = atomicAdd(&b.counters[2], words);
      if (off + words > b.scratch_words) {
        ok = 0;
        atomicOr(b.status, kStatusScratchOverflow);
      }
    }
    ok = __shfl_sync(kFull, ok, 0);
    if (!ok) {
      if (lane == 0 && b.deferred) b.deferred[shot] = 1;
      __syncwarp();
      continue;
    }
    off = __shfl_sync(kFull, off, 0);
    uint32_t *sp = b.scratch + off;
    for (int ii = heavy_from; ii < J.n_it; ++ii) {
      IterInfo &I = J.it[ii];
      const unsigned long long tm = (unsigned long long)I.tam;
      uint32_t *cols = sp;
      sp += (tm * cd.nwp + 3ull) & ~3ull;
      int *pos = reinterpret_cast<int *>(sp);
      int *tmp = pos + tm;
      sp += ((ml ? 2ull : 1ull) * tm + 3ull) & ~3ull;
      float *llr = nullptr;
      if (ml) {
        llr = reinterpret_cast<float *>(sp);
        sp += (tm + 3ull) & ~3ull;
      }
      stage_iteration(cd, A.am[I.src], I.tam, pos, tmp, cols, llr);
      if (lane == 0) {
        I.pos = pos;
        I.cols = cols;
        I.llr = llr;
        if (ml) {
          float pf = 0.0f;
          I.prefix[0] = 0.0f;
          for (int w = 1; w <= kMaxW; ++w) {
            if (w <= I.tam) pf = __fadd_rn(pf, llr[w - 1]);
            I.prefix[w] = pf;
          }
        }
      }
      __syncwarp();
    }
    // run-tile tables: cum[c] = run tiles before run c (warp prefix scan)
    for (int sgi = 0; sgi < J.nseg; ++sgi) {
      Seg &S = J.seg[sgi];
      if (!S.runs || S.dup || S.iter < heavy_from) continue;
      const int tam = J.it[S.iter].tam;
      unsigned long long *cum = reinterpret_cast<unsigned long long *>(sp);
      sp += (2ull * (unsigned long long)tam + 3ull) & ~3ull;
      unsigned long long carry = 0;
      for (int c0 = 0; c0 < tam; c0 += 32) {
        const int c = c0 + lane;
        const unsigned long long nt = (c <= tam - 2) ? run_tiles(b.ncr, c, S.w, kRunKK) : 0ull;
        unsigned long long incl = nt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const unsigned long long u = __shfl_up_sync(kFull, incl, o);
          if (lane >= o) incl += u;
        }
        if (c < tam) cum[c] = carry + incl - nt;
        carry += __shfl_sync(kFull, incl, 31);
      }
      if (lane == 0) {
        S.cum = cum;
        S.ntiles = carry;
      }
      __syncwarp();
    }
    if (lane == 0) {
      J.it_lo = heavy_from;
      for (int sgi = 0; sgi < J.nseg; ++sgi) {
        Seg &S = J.seg[sgi];
        S.njt = (S.dup || S.iter < heavy_from) ? 0ull : S.ntiles;
        S.tile_lo = ntl;
        ntl += S.njt;
      }
      const unsigned long long old = atomicAdd(&b.counters[0], (1ull << 40) | ntl);
      jslot = old >> 40;
      tbase = old & ((1ull << 40) - 1ull);
      if (jslot >= (unsigned long long)b.max_jobs) {
        ok = 0;
        atomicOr(b.status, kStatusJobOverflow);
      }
    }
    ok = __shfl_sync(kFull, ok, 0);
    if (!ok) {
      if (lane == 0 && b.deferred) b.deferred[shot] = 1;
      __syncwarp();
      continue;
    }
    jslot = __shfl_sync(kFull, jslot, 0);
    tbase = __shfl_sync(kFull, tbase, 0);
    ntl = __shfl_sync(kFull, ntl, 0);
    for (int q = lane; q < 128; q += 32) sp[q] = A.eb[q];
    J.sw[lane] = A.sw[lane];
    if (lane == 0) {
      J.ebits = sp;
      J.tile_base = tbase;
      J.ntiles = ntl;
      for (int i = 0; i < kMaxIters; ++i)
        for (int w = 0; w <= kMaxW; ++w) J.mlkey[i][w][0] = J.mlkey[i][w][1] = kNone;
    }
    __syncwarp();
    {
      const uint32_t *src = reinterpret_cast<const uint32_t *>(&J);
      uint32_t *dst = reinterpret_cast<uint32_t *>(b.jobs + jslot);
      for (int i = lane; i < (int)(sizeof(Job) / 4); i += 32) dst[i] = src[i];
    }
    if (lane == 0 && b.deferred) b.deferred[shot] = 0;
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// Kernel 2: persistent work-stealing search over the Jobs' tiles.
// ---------------------------------------------------------------------------
__device__ bool tile_skip(const Job &J, const Seg &S, const IterInfo &I, bool ml) {
  if (!ml) {
    const unsigned long long best = *reinterpret_cast<const volatile unsigned long long *>(&J.best);
    return S.base >= best;
  }
  for (int i = 0; i < S.iter; ++i)
    for (int w = 1; w <= kMaxW; ++w)
      if (*reinterpret_cast<const volatile unsigned long long *>(&J.mlkey[i][w][0]) != kNone)
        return true;
  for (int w = 1; w < S.w; ++w) {
    const unsigned long long o =
        *reinterpret_cast<const volatile unsigned long long *>(&J.mlkey[S.iter][w][0]);
    if (o != kNone && I.prefix[S.w] >= key_cost((uint32_t)o)) return true;
  }
  return false;
}

__device__ Winner winner_ml(const Job &J) {
  Winner wn;
  wn.found = 0;
  wn.ii = wn.seg = 0;
  wn.rank = wn.count = 0;
  wn.cost = 0.0f;
  for (int ii = J.it_lo; ii < J.n_it; ++ii) {
    const IterInfo &I = J.it[ii];
    uint32_t bo = 0xffffffffu;
    unsigned long long br = kNone, proc = 0;
    int bseg = -1;
    for (int s = I.seg_lo; s < I.seg_hi; ++s) {
      const Seg &S = J.seg[s];
      if (bseg >= 0 && I.prefix[S.w] >= key_cost(bo)) break;
      proc += S.count;
      const unsigned long long o = J.mlkey[ii][S.w][0];
      if (o != kNone && (bseg < 0 || (uint32_t)o < bo)) {
        bo = (uint32_t)o;
        br = J.mlkey[ii][S.w][1];
        bseg = s;
      }
    }
    if (bseg >= 0) {
      wn.found = 1;
      wn.ii = ii;
      wn.seg = bseg;
      wn.rank = br;
      wn.count = (I.branch == kBranchCpu) ? proc : I.total;
      wn.cost = key_cost(bo);
      return wn;
    }
  }
  return wn;
}

__global__ void __launch_bounds__(kSearchThreads, 3) search_kernel(DevBatch b) {
  __shared__ __align__(16) uint32_t s_stage[kSearchWarps][kWarpStage];
  __shared__ uint32_t s_sw[kSearchWarps][kMaxRows / 32];
  __shared__ uint32_t s_delta[kSearchWarps][kMaxCols / 32];

  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  uint32_t *stage = s_stage[warp];
  uint32_t *sw = s_sw[warp];
  const unsigned long long packed = *reinterpret_cast<volatile unsigned long long *>(b.counters);
  unsigned long long njobs = packed >> 40;
  unsigned long long total = packed & ((1ull << 40) - 1ull);
  if (njobs > (unsigned long long)b.max_jobs) {
    njobs = b.max_jobs;
    total = njobs ? b.jobs[njobs - 1].tile_base + b.jobs[njobs - 1].ntiles : 0ull;
  }
  int st_job = -1, st_it = -1;
  // per-warp caches of the last job / weight block / run looked up, and a
  // register copy of the current weight block's parameters
  int cj = -1, cs = -1, cc = -1;
  unsigned long long cj_lo = 0, cj_hi = 0, cs_lo = 0, cs_hi = 0, cc_lo = 0, cc_hi = 0;
  Job *Jp = nullptr;
  const DevCode *cdp = nullptr;
  SegView sv{};
  int s_runs = 0, s_iter = 0, s_ml = 0, s_prob = 0, s_nw = 0;
  const unsigned long long *s_cum = nullptr;

  for (;;) {
    unsigned long long t0 = 0;
    if (lane == 0) t0 = atomicAdd(&b.counters[1], (unsigned long long)kTilesPerFetch);
    t0 = __shfl_sync(kFull, t0, 0);
    if (t0 >= total) break;
    const unsigned long long t1 = (t0 + kTilesPerFetch < total) ? t0 + kTilesPerFetch : total;
    bool skip_known = false, skip = false;
    unsigned long long pending = 0;
    bool fenced = false;
    for (unsigned long long t = t0; t < t1; ++t) {
      if (cj < 0 || t < cj_lo || t >= cj_hi) {
        int lo = 0, hi = (int)njobs - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (b.jobs[mid].tile_base <= t) lo = mid;
          else hi = mid - 1;
        }
        cj = lo;
        Jp = &b.jobs[lo];
        cdp = &b.codes[Jp->code];
        cj_lo = Jp->tile_base;
        cj_hi = cj_lo + Jp->ntiles;
        cs = -1;
      }
      Job &J = *Jp;
      const unsigned long long lt = t - cj_lo;
      if (cs < 0 || lt < cs_lo || lt >= cs_hi) {
        int sg = 0;
        while (sg < J.nseg - 1 &&
               !(J.seg[sg].njt && lt >= J.seg[sg].tile_lo && lt < J.seg[sg].tile_lo + J.seg[sg].njt))
          ++sg;
        const Seg &S = J.seg[sg];
        const IterInfo &I = J.it[S.iter];
        cs = sg;
        cs_lo = S.tile_lo;
        cs_hi = cs_lo + S.njt;
        cc = -1;
        s_runs = S.runs;
        s_cum = S.cum;
        s_iter = S.iter;
        s_nw = cdp->nw;
        s_ml = cdp->variant == kMl;
        s_prob = cdp->variant == kProb;
        const bool staged = I.tam * cdp->nwp <= kWarpStage;
        sv = SegView{staged ? stage : I.cols, I.llr, I.tam, S.w, S.K, cdp->nwp, cdp->nw,
                     S.nprefix, S.base};
        if (st_job != cj || st_it != S.iter) {
          __syncwarp();
          if (staged) {
            const uint4 *src = reinterpret_cast<const uint4 *>(I.cols);
            uint4 *dst = reinterpret_cast<uint4 *>(stage);
            const int n4 = (I.tam * cdp->nwp + 3) / 4;
            for (int i = lane; i < n4; i += 32) dst[i] = src[i];
          }
          sw[lane] = J.sw[lane];
          __syncwarp();
          st_job = cj;
          st_it = S.iter;
        }
        skip_known = false;
      }
      if (!skip_known || s_ml) {
        skip = tile_skip(J, J.seg[cs], J.it[s_iter], s_ml);
        skip_known = true;
      }
      bool published = false;
      if (!skip) {
        LaneBest lb;
        lb.reset();
        const unsigned long long st = lt - cs_lo;
        if (s_runs) {
          if (cc < 0 || st < cc_lo || st >= cc_hi) {
            // run c holding segment tile st: largest c with cum[c] <= st
            int clo = 0, chi = sv.tam - 2;
            while (clo < chi) {
              const int mid = (clo + chi + 1) >> 1;
              if (s_cum[mid] <= st) clo = mid;
              else chi = mid - 1;
            }
            cc = clo;
            cc_lo = s_cum[clo];
            cc_hi = cc_lo + run_tiles(b.ncr, clo, sv.w, kRunKK);
          }
          const unsigned long long r0 = (st - cc_lo) * (32ull * kRunKK);
          if (s_ml) eval_run_dispatch<true, kRunKK>(s_nw, sv, b.ncr, sw, cc, r0, lb);
          else eval_run_dispatch<false, kRunKK>(s_nw, sv, b.ncr, sw, cc, r0, lb);
        } else {
          if (s_ml) eval_dispatch<true>(s_nw, sv, b.ncr, sw, st, lb);
          else eval_dispatch<false>(s_nw, sv, b.ncr, sw, st, lb);
        }
        if (!s_ml) {
          const unsigned long long g = warp_min_u64(lb.g);
          if (g != kNone) {
            published = true;
            skip_known = false;
            if (lane == 0) atomicMin(&J.best, g);
          }
        } else {
          uint32_t o = lb.o;
          unsigned long long r = lb.r;
          warp_min_key(o, r);
          if (o != 0xffffffffu) {
            published = true;
            if (lane == 0 && !atomic_min_key(J.mlkey[s_iter][sv.w], o, r))
              atomicOr(b.status, kStatusCasLimit);
          }
        }
      }
      // tiles of this fetch done for the current job: posted once per job per fetch
      pending += 1ull;
      fenced = fenced || published;
      const bool flush = (t + 1 == t1) || (t + 1 >= cj_hi);
      if (flush) {
        int last = 0;
        if (lane == 0) {
          if (fenced) __threadfence();  // order the published minima before the count
          last = (atomicAdd(&J.tiles_done, pending) + pending == J.ntiles) ? 1 : 0;
        }
        pending = 0;
        fenced = false;
        last = __shfl_sync(kFull, last, 0);
        if (last) {
          __threadfence();
          Winner wn;
          if (!s_ml)
            wn = winner_from_index(J, *reinterpret_cast<volatile unsigned long long *>(&J.best),
                                   s_prob != 0);
          else
            wn = winner_ml(J);
          finish_shot(b, *cdp, J, J.shot, wn, J.ebits, s_delta[warp]);
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Host-callable launchers.
// ---------------------------------------------------------------------------
cudaError_t launch_triage(const DevBatch &b, int grid, cudaStream_t s) {
  triage_kernel<<<grid, kTriageWarps * 32, 0, s>>>(b);
  return cudaGetLastError();
}

cudaError_t launch_search(const DevBatch &b, int grid, cudaStream_t s) {
  search_kernel<<<grid, kSearchThreads, 0, s>>>(b);
  return cudaGetLastError();
}

int triage_warps_per_block() { return kTriageWarps; }
int search_threads_per_block() { return kSearchThreads; }

cudaError_t occupancy(int *triage_blocks_per_sm, int *search_blocks_per_sm) {
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(triage_blocks_per_sm, triage_kernel,
                                                                kTriageWarps * 32, 0);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(search_blocks_per_sm, search_kernel,
                                                       kSearchThreads, 0);
}

}  // namespace grand
