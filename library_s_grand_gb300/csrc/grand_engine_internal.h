// grand_engine_internal.h -- the engine object shared by grand_engine.cpp and
// grand_server.cpp (not part of the C ABI).
#pragma once

#include <map>
#include <memory>
#include <mutex>
#include <tuple>
#include <vector>

#include "grand_engine.h"
#include "grand_host.h"

namespace grand {

// Job table, scratch and counters of one in-flight device decode.
struct EngineSlot {
  void *d_jobs = nullptr; size_t cap_jobs = 0;
  void *d_scratch = nullptr; size_t cap_scratch = 0;
  void *d_small = nullptr; size_t cap_small = 0;
  void *d_deferred = nullptr; size_t cap_deferred = 0;
  cudaEvent_t ev[3] = {};
  bool timed = false;
  ~EngineSlot() {
    for (auto &e : ev) if (e) cudaEventDestroy(e);
    cudaFree(d_jobs);
    cudaFree(d_scratch);
    cudaFree(d_small);
    cudaFree(d_deferred);
  }
};

struct GraphKey {
  int n;
  const void *a, *b, *c, *d;
  bool operator<(const GraphKey &o) const {
    return std::tie(n, a, b, c, d) < std::tie(o.n, o.a, o.b, o.c, o.d);
  }
};

}  // namespace grand

struct GrandEngine {
  grand::Context *ctx = nullptr;
  std::mutex mu;
  std::vector<grand::DevCode> codes;
  std::vector<std::shared_ptr<grand::CodeTables>> tabs;
  std::vector<float *> llr;
  std::vector<int> rec_len;
  void *d_codes = nullptr;
  size_t cap_codes = 0;
  bool dirty = true;
  grand::Tuning tn;
  std::map<const void *, grand::EngineSlot *> slots;  // per stream
  std::map<grand::GraphKey, cudaGraphExec_t> graphs;
  grand::BatchTiming last{};  // times of the last host-buffer decode
  ~GrandEngine() {
    for (auto &g : graphs) cudaGraphExecDestroy(g.second);
    for (auto &s : slots) delete s.second;
    for (float *p : llr) cudaFree(p);
    cudaFree(d_codes);
  }
};

namespace grand {

// Upload the engine's code descriptors when they changed (caller holds e->mu).
inline int upload_codes(GrandEngine *e) {
  if (!e->dirty) return 0;
  cudaError_t r = ensure(&e->d_codes, &e->cap_codes,
                         sizeof(DevCode) * (e->codes.empty() ? 1 : e->codes.size()));
  if (r == cudaSuccess && !e->codes.empty())
    r = cudaMemcpy(e->d_codes, e->codes.data(), sizeof(DevCode) * e->codes.size(),
                   cudaMemcpyHostToDevice);
  if (r != cudaSuccess) {
    set_error("grand: code table upload failed (%s)", cudaGetErrorString(r));
    return GRAND_ERR_CUDA;
  }
  e->dirty = false;
  return 0;
}

}  // namespace grand
