// Internal host-side declarations shared by api.cu and batch.cu: the
// layouts of the opaque handles and the run / allocation helpers.
#pragma once
#include <cstdint>

#include "../../include/gbconn.h"
#include "gb_internal.cuh"

struct gb_ctx {
  int device = 0;
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
  cudaEvent_t ev[kRing][5] = {};  // phase events of the last kRing runs
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
};


namespace gb {
// Records a CUDA failure for gb_last_error and maps it to a status.
gb_status cuda_fail(cudaError_t e, const char* where);
bool is_device_ptr(const void* p);
gb_status graph_alloc(gb_graph* g, bool with_in);
void graph_free(gb_graph* g);
gb_status graph_hints(gb_ctx* c, gb_graph* g);
gb_status validate_csr(gb_ctx* c, int32_t n, int64_t m, const int64_t* off, const int32_t* adj);
// One run over a graph; bv != null runs a batch union and returns labels
// local to each graph.
gb_status run_graph(gb_ctx* c, const gb_graph* g, RunKind kind, int32_t* labels,
                    const gb_opts* o, gb_stats* st, bool wait, const BatchView* bv);
}  // namespace gb
