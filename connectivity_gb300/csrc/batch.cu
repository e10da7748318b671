// Batched SCC / WCC: many independent graphs in one run.
//
// The reference has no batching; its per-graph equivalent is a loop of
// run_scc / run_cc calls (multistep/scc_main.cpp:210, cc_main.cpp:184).
// Here a batch is stored as one disjoint union -- graph g owns the vertices
// [vbase[g], vbase[g+1]) of one concatenated CSR with global ids -- and a
// run is the same three cooperative kernels as for one graph, advancing every
// graph at once: trim picks each graph's pivot (the reference rule, per
// graph), the reachability searches start from all pivots together (graphs
// share no edge, so each search stays inside its graph), the colour rounds
// run over the union, and the labels come back local to each graph.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/gbconn.h"
#include "api_internal.h"
#include "gb_internal.cuh"
#include "host_internal.h"

struct gb_batch {
  gb_graph* g = nullptr;        // the union
  int32_t count = 0;
  std::vector<int64_t> vbase;   // host copy, count + 1
  int64_t* d_vbase = nullptr;
  int32_t* d_gid = nullptr;
  unsigned long long* d_pkey = nullptr;
  int32_t* d_gmin = nullptr;
  int32_t* d_roots = nullptr;
  int32_t id_bits = 1;
  int32_t score_bits_scc = 0;   // bits of the largest out*in product
  int32_t score_bits_wcc = 0;   // bits of the largest total degree
  bool pooled = false;
  cudaStream_t pool_stream = nullptr;
};

namespace {

#define CKB(call, where)                                  \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return gb::cuda_fail(e_, where); \
  } while (0)

int bits_of(unsigned long long x) {
  int b = 0;
  while (b < 64 && (x >> b) != 0ull) ++b;
  return b;
}

void batch_free(gb_batch* b) {
  if (!b) return;
  if (b->g) {
    gb::graph_free(b->g);
    delete b->g;
    b->g = nullptr;
  }
  gb::dev_free(b->d_vbase, b->pooled, b->pool_stream);
  gb::dev_free(b->d_gid, b->pooled, b->pool_stream);
  gb::dev_free(b->d_pkey, b->pooled, b->pool_stream);
  gb::dev_free(b->d_gmin, b->pooled, b->pool_stream);
  gb::dev_free(b->d_roots, b->pooled, b->pool_stream);
  b->d_vbase = nullptr;
  b->d_gid = nullptr;
  b->d_pkey = nullptr;
  b->d_gmin = nullptr;
  b->d_roots = nullptr;
}

// Everything after the union's CSR exists: vertex -> graph map, per-graph
// scratch, and the pivot-key widths.
gb_status batch_finish(gb_ctx* c, gb_batch* b, const int32_t* d_src, const int32_t* d_dst,
                       bool check_edges) {
  const int32_t n = b->g->n;
  const int32_t count = b->count;
  const bool pl = b->pooled;
  cudaStream_t ps = b->pool_stream;
  CKB(gb::dev_alloc((void**)&b->d_vbase, (size_t)(count + 1) * 8, pl, ps), "batch allocation");
  CKB(cudaMemcpyAsync(b->d_vbase, b->vbase.data(), (size_t)(count + 1) * 8, cudaMemcpyHostToDevice,
                      c->stream),
      "batch upload");
  CKB(gb::dev_alloc((void**)&b->d_gid, (size_t)(n > 0 ? n : 1) * 4, pl, ps), "batch allocation");
  CKB(gb::dev_alloc((void**)&b->d_pkey, (size_t)(count > 0 ? count : 1) * 8, pl, ps), "batch allocation");
  CKB(gb::dev_alloc((void**)&b->d_gmin, (size_t)(count > 0 ? count : 1) * 4, pl, ps), "batch allocation");
  CKB(gb::dev_alloc((void**)&b->d_roots, (size_t)(count > 0 ? count : 1) * 4, pl, ps), "batch allocation");
  CKB(gb::batch_gid(n, b->d_vbase, count, b->d_gid, c->stream), "batch gid");
  if (check_edges && b->g->m > 0) {
    int bad = 0;
    CKB(gb::batch_check_within(d_src, d_dst, b->g->m, b->d_gid, c->stream, &bad), "batch check");
    if (bad) {
      gb_set_error("batch: %s", "an edge joins two graphs");
      return GB_ERR_INVALID;
    }
  }
  unsigned long long mo = 0, mi = 0;
  CKB(gb::max_degree(n, b->g->out_off, c->stream, &mo), "batch degrees");
  CKB(gb::max_degree(n, b->g->in_off, c->stream, &mi), "batch degrees");
  int ib = bits_of((unsigned long long)(n > 1 ? n - 1 : 1));
  b->id_bits = ib > 0 ? ib : 1;
  b->score_bits_scc = bits_of(mo * mi);
  b->score_bits_wcc = bits_of(mo + mi);
  return GB_OK;
}

gb_status batch_from_union(gb_ctx* c, int32_t count, const int64_t* vbase, int64_t m,
                           const int32_t* src, const int32_t* dst, bool check_edges,
                           bool pooled, gb_batch** out) {
  if (!c || !out || count < 1 || !vbase || m < 0 || (m > 0 && (!src || !dst))) {
    gb_set_error("batch: %s", "bad argument");
    return GB_ERR_INVALID;
  }
  *out = nullptr;
  if (vbase[0] != 0) return GB_ERR_INVALID;
  for (int32_t g = 0; g < count; ++g)
    if (vbase[g + 1] < vbase[g]) return GB_ERR_INVALID;
  if (vbase[count] > 0x7fffffffll) {
    gb_set_error("batch: %s", "more than 2^31-1 vertices in total");
    return GB_ERR_CAPACITY;
  }
  gb_batch* b = new (std::nothrow) gb_batch();
  if (!b) return GB_ERR_OOM;
  b->count = count;
  b->pooled = pooled;
  b->pool_stream = c->stream;
  b->vbase.assign(vbase, vbase + count + 1);
  gb_status s = gb::graph_from_edges(c, (int32_t)vbase[count], m, src, dst, pooled, &b->g);
  if (s == GB_OK) {
    // the checks need device copies of the edges; from_edges already
    // validated ids against n, so only the within-graph rule remains
    const int32_t *ds = src, *dd = dst;
    int32_t *ts = nullptr, *tt = nullptr;
    if (check_edges && m > 0 && !gb::is_device_ptr(src)) {
      if (gb::dev_alloc((void**)&ts, (size_t)m * 4, pooled, c->stream) != cudaSuccess ||
          gb::dev_alloc((void**)&tt, (size_t)m * 4, pooled, c->stream) != cudaSuccess ||
          cudaMemcpyAsync(ts, src, (size_t)m * 4, cudaMemcpyHostToDevice, c->stream) != cudaSuccess ||
          cudaMemcpyAsync(tt, dst, (size_t)m * 4, cudaMemcpyHostToDevice, c->stream) != cudaSuccess) {
        s = GB_ERR_OOM;
      }
      ds = ts;
      dd = tt;
    }
    if (s == GB_OK) s = batch_finish(c, b, ds, dd, check_edges);
    gb::dev_free(ts, pooled, c->stream);
    gb::dev_free(tt, pooled, c->stream);
  }
  if (s != GB_OK) {
    batch_free(b);
    delete b;
    return s;
  }
  *out = b;
  return GB_OK;
}

gb_status batch_run_impl(gb_ctx* c, const gb_batch* b, gb::RunKind kind, int32_t* labels,
                         const gb_opts* o, gb_stats* st, bool wait) {
  if (!b) return GB_ERR_INVALID;
  const int sb = kind == gb::kSCC ? b->score_bits_scc : b->score_bits_wcc;
  if (sb + b->id_bits > 63) {
    gb_set_error("batch: %s", "degrees too large to pack each graph's pivot key in 64 bits");
    return GB_ERR_UNSUPPORTED;
  }
  gb::BatchView bv{};
  bv.gid = b->d_gid;
  bv.vbase = b->d_vbase;
  bv.count = b->count;
  bv.id_bits = b->id_bits;
  bv.pkey = b->d_pkey;
  bv.gmin = b->d_gmin;
  bv.roots = b->d_roots;
  return gb::run_graph(c, b->g, kind, labels, o, st, wait, &bv);
}

}  // namespace

gb_status gb::batch_create(gb_ctx* c, int32_t count, const int64_t* vbase, int64_t m,
                           const int32_t* src, const int32_t* dst, bool check_edges, bool pooled,
                           gb_batch** out) {
  return batch_from_union(c, count, vbase, m, src, dst, check_edges, pooled, out);
}

gb_status gb::batch_run(gb_ctx* c, const gb_batch* b, RunKind kind, int32_t* labels,
                        const gb_opts* o, gb_stats* st, bool wait) {
  return batch_run_impl(c, b, kind, labels, o, st, wait);
}

extern "C" {

gb_status gb_batch_from_edges(gb_ctx* c, int32_t count, const int64_t* vbase, int64_t m,
                              const int32_t* src, const int32_t* dst, gb_batch** out) {
  return batch_from_union(c, count, vbase, m, src, dst, true, false, out);
}

gb_status gb_batch_rmat(gb_ctx* c, int32_t count, const int32_t* n, const int32_t* ef,
                        const uint64_t* seeds, double a, double bb, double cc, gb_batch** out) {
  if (!c || !out || count < 1 || !n || !ef || !seeds) return GB_ERR_INVALID;
  *out = nullptr;
  std::vector<int64_t> vb((size_t)count + 1, 0);
  for (int32_t g = 0; g < count; ++g) {
    if (n[g] < 1 || ef[g] < 1) return GB_ERR_INVALID;
    vb[g + 1] = vb[g] + n[g];
  }
  if (vb[count] > 0x7fffffffll) return GB_ERR_CAPACITY;
  CKB(cudaSetDevice(c->device), "cudaSetDevice");
  int id_bits = bits_of((unsigned long long)(vb[count] > 1 ? vb[count] - 1 : 1));
  int32_t *s = nullptr, *d = nullptr;
  int64_t m = 0;
  CKB(gb::batch_edges_device(count, n, ef, seeds, gb_rmat_thresholds(a, bb, cc), id_bits, vb.data(),
                             &s, &d, &m, c->stream),
      "batch R-MAT");
  gb_status st = batch_from_union(c, count, vb.data(), m, s, d, false, false, out);
  cudaFreeAsync(s, c->stream);
  cudaFreeAsync(d, c->stream);
  cudaStreamSynchronize(c->stream);
  return st;
}

gb_status gb_batch_info(const gb_batch* b, int32_t* count, int64_t* total_n, int64_t* total_m) {
  if (!b) return GB_ERR_INVALID;
  if (count) *count = b->count;
  if (total_n) *total_n = b->g->n;
  if (total_m) *total_m = b->g->m;
  return GB_OK;
}

gb_status gb_batch_vbase(const gb_batch* b, int64_t* vbase) {
  if (!b || !vbase) return GB_ERR_INVALID;
  std::memcpy(vbase, b->vbase.data(), b->vbase.size() * sizeof(int64_t));
  return GB_OK;
}

gb_status gb_batch_graph(const gb_batch* b, const gb_graph** g) {
  if (!b || !g) return GB_ERR_INVALID;
  *g = b->g;
  return GB_OK;
}

gb_status gb_batch_scc(gb_ctx* c, const gb_batch* b, int32_t* labels, const gb_opts* o,
                       gb_stats* st) {
  return batch_run_impl(c, b, gb::kSCC, labels, o, st, true);
}

gb_status gb_batch_wcc(gb_ctx* c, const gb_batch* b, int32_t* labels, const gb_opts* o,
                       gb_stats* st) {
  return batch_run_impl(c, b, gb::kWCC, labels, o, st, true);
}

gb_status gb_batch_scc_async(gb_ctx* c, const gb_batch* b, int32_t* labels_dev, const gb_opts* o) {
  return batch_run_impl(c, b, gb::kSCC, labels_dev, o, nullptr, false);
}

gb_status gb_batch_destroy(gb_batch* b) {
  if (!b) return GB_OK;
  if (b->g) cudaSetDevice(b->g->device);
  batch_free(b);
  delete b;
  return GB_OK;
}

}  // extern "C"
