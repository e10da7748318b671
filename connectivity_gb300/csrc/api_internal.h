// Internal host-side declarations shared by api.cu and batch.cu: the
// layouts of the opaque handles and the run / allocation helpers.
#pragma once
#include <cstdint>
#include <vector>

#include "../../include/gbconn.h"
#include "gb_internal.cuh"

struct gb_ctx {
  int device = 0;
  // options per size class for runs given no options (gb_ctx_set_class_opts):
  // entry i covers graphs of at most cls_n[i] vertices, ascending
  std::vector<int64_t> cls_n;
  std::vector<gb_opts> cls_opts;
  cudaStream_t own = nullptr;
  cudaStream_t stream = nullptr;
  int grid = 0;                 // cooperative grid (all resident blocks)
  int32_t cap_n = -1;           // workspace capacity in vertices
  void* ws = nullptr;
  gb::Work w{};
  gb::Ctl* d_ctl = nullptr;
  gb::Ctl* h_ctl = nullptr;     // pinned
  int* d_sticky = nullptr;      // first error of any run since the last sync
  int* h_sticky = nullptr;      // pinned
  static constexpr int kRing = 64;
  cudaEvent_t ev[kRing][5] = {};  // events of the last kRing runs: [0] start, [1] after the
                                  // run kernel, [4] end (after the statistics pass)
  unsigned long long* d_tphase = nullptr;  // kRing x 4 device phase-boundary times
  unsigned long long* h_tphase = nullptr;  // pinned copy
  long long runs = 0;             // runs issued on this context
};

struct gb_graph {
  int device = 0;
  int32_t n = 0;
  int64_t m = 0;
  int symmetric = 0;
  int64_t* out_off = nullptr;
  int32_t* out_adj = nullptr;
  int64_t* in_off = nullptr;
  int32_t* in_adj = nullptr;
  int32_t* hint_out = nullptr;  // pull hints (null for the drop-in staging graph)
  int32_t* hint_in = nullptr;
  bool pooled = false;          // arrays from the stream-ordered pool
  cudaStream_t pool_stream = nullptr;
};


struct gb_batch;

namespace gb {
// Device allocation from cudaMalloc, or from the stream-ordered pool on
// stream s (pooled); the matching free.
cudaError_t dev_alloc(void** p, size_t bytes, bool pooled, cudaStream_t s);
void dev_free(void* p, bool pooled, cudaStream_t s);
// Records a CUDA failure for gb_last_error and maps it to a status.
gb_status cuda_fail(cudaError_t e, const char* where);
bool is_device_ptr(const void* p);
// Grows the context workspace to at least n vertices.
gb_status reserve_workspace(gb_ctx* c, int32_t n);
gb_status graph_alloc(gb_graph* g, bool with_in);
void graph_free(gb_graph* g);
gb_status graph_hints(gb_ctx* c, gb_graph* g);
gb_status validate_csr(gb_ctx* c, int32_t n, int64_t m, const int64_t* off, const int32_t* adj);
// The context's options for a graph (or union) of n vertices from its class
// table, or null when it has none.
const gb_opts* class_opts(const gb_ctx* c, int64_t n);
// One run over a graph; bv != null runs a batch union and returns labels
// local to each graph.
gb_status run_graph(gb_ctx* c, const gb_graph* g, RunKind kind, int32_t* labels,
                    const gb_opts* o, gb_stats* st, bool wait, const BatchView* bv);
// Graph from an edge list; pooled graphs take their arrays from the
// context stream's pool and free them on that stream.
gb_status graph_from_edges(gb_ctx* c, int32_t n, int64_t m, const int32_t* src,
                           const int32_t* dst, bool pooled, gb_graph** out);
// Batch from a concatenated global-id edge list (host or device).
gb_status batch_create(gb_ctx* c, int32_t count, const int64_t* vbase, int64_t m,
                       const int32_t* src, const int32_t* dst, bool check_edges, bool pooled,
                       gb_batch** out);
gb_status batch_run(gb_ctx* c, const gb_batch* b, RunKind kind, int32_t* labels,
                    const gb_opts* o, gb_stats* st, bool wait);
}  // namespace gb
