// C ABI of libgbconn (include/gbconn.h): contexts, device graphs, runs and
// the reference-shaped drop-ins.  Host code only; the kernels live in
// kernels.cu and csr_build.cu.
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>

#include "../../include/gbconn.h"
#include "api_internal.h"
#include "gb_internal.cuh"
#include "host_internal.h"

namespace gb {

gb_status cuda_fail(cudaError_t e, const char* where) {
  char buf[256];
  std::snprintf(buf, sizeof(buf), "%s: %s", where, cudaGetErrorString(e));
  gb_set_error("%s", buf);
  if (e == cudaErrorMemoryAllocation) return GB_ERR_OOM;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return GB_ERR_NO_DEVICE;
  return GB_ERR_CUDA;
}
#define CK(call, where)                              \
  do {                                               \
    cudaError_t e_ = (call);                         \
    if (e_ != cudaSuccess) return cuda_fail(e_, where); \
  } while (0)

bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

}  // namespace gb

namespace {
using gb::cuda_fail;
using gb::is_device_ptr;

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Grows the context workspace to n vertices (never shrinks).
gb_status ensure_ws(gb_ctx* c, int32_t n) {
  if (n <= c->cap_n) return GB_OK;
  if (c->ws) {
    cudaStreamSynchronize(c->stream);
    cudaFree(c->ws);
    c->ws = nullptr;
    c->cap_n = -1;
  }
  const size_t nv = (size_t)(n > 0 ? n : 1) + 32;
  const size_t nw = nv / 32 + 2;
  const size_t arr = align256(nv * 4), bm = align256(nw * 4);
  const size_t G = (size_t)(c->grid > 0 ? c->grid : 1);
  const size_t total = 15 * arr + 4 * bm + align256(2 * G * 4) + align256(2 * G * 8);
  char* p = nullptr;
  CK(cudaMalloc(&p, total), "workspace allocation");
  c->ws = p;
  gb::Work& w = c->w;
  auto take = [&](size_t bytes) {
    char* r = p;
    p += bytes;
    return r;
  };
  w.label = (int32_t*)take(arr);
  w.colour = (int32_t*)take(arr);
  w.live_in = (int32_t*)take(arr);
  w.live_out = (int32_t*)take(arr);
  w.listA = (int32_t*)take(arr);
  w.listB = (int32_t*)take(arr);
  w.q = (int32_t*)take(arr);
  w.x0 = (int32_t*)take(arr);
  w.x1 = (int32_t*)take(arr);
  w.candA = (int32_t*)take(arr);
  w.candB = (int32_t*)take(arr);
  w.h0 = (int32_t*)take(arr);
  w.h1 = (int32_t*)take(arr);
  w.xa = (int32_t*)take(arr);
  w.xb = (int32_t*)take(arr);
  w.vbits = (uint32_t*)take(bm);
  w.fvis = (uint32_t*)take(bm);
  w.bvis = (uint32_t*)take(bm);
  w.done = (uint32_t*)take(bm);
  w.blk_i = (int32_t*)take(align256(2 * G * 4));
  w.blk_l = (long long*)take(align256(2 * G * 8));
  w.ctl = c->d_ctl;
  c->cap_n = n;
  return GB_OK;
}

void fill_params(const gb_opts* o, gb::RunParams& p) {
  gb_opts d;
  gb_opts_default(&d);
  if (!o) o = &d;
  p.trim_level = o->trim_level >= 2 ? 2 : (o->trim_level <= 0 ? 0 : 1);
  p.trim_pairs = o->trim_pairs ? 1 : 0;
  p.fwbw_rounds = o->fwbw_rounds > 1 ? o->fwbw_rounds : 1;
  p.canonical = o->canonical ? 1 : 0;
  p.pivot_hint = o->pivot;
  p.tune.t_block = o->t_block > 32 ? o->t_block : 32;
  p.tune.t_grid = o->t_grid > p.tune.t_block ? o->t_grid : p.tune.t_block + 1;
  p.tune.k_pull = o->k_pull > 0 ? o->k_pull : 1;
  p.tune.alpha = o->alpha > 0 ? o->alpha : 15.0f;
  p.tune.beta = o->beta > 0 ? o->beta : 25.0f;
  p.tune.max_steps = o->max_steps > 0 ? o->max_steps : (1 << 30);
  p.tune.expand_mode = o->expand_mode == 1 ? 1 : 0;
  p.colour_mode = o->colour_mode == 1 || o->colour_mode == 2 ? o->colour_mode : 0;
}

}  // namespace

namespace gb {

cudaError_t dev_alloc(void** p, size_t bytes, bool pooled, cudaStream_t s) {
  return pooled ? cudaMallocAsync(p, bytes, s) : cudaMalloc(p, bytes);
}

void dev_free(void* p, bool pooled, cudaStream_t s) {
  if (!p) return;
  if (pooled) cudaFreeAsync(p, s);
  else cudaFree(p);
}

// The hint arrays come from the stream-ordered pool whatever the graph's
// other arrays do.  On a graph that is not pooled they are freed once the
// whole device is idle, as cudaFree does for its other arrays.
void hint_free(gb_graph* g, int32_t*& p) {
  if (!p) return;
  if (g->pooled) {
    cudaFreeAsync(p, g->pool_stream);
  } else {
    cudaDeviceSynchronize();
    cudaFree(p);
  }
  p = nullptr;
}

gb_status graph_alloc(gb_graph* g, bool with_in) {
  const size_t offb = (size_t)(g->n + 1) * 8, adjb = (size_t)(g->m > 0 ? g->m : 1) * 4;
  cudaStream_t s = g->pool_stream;
  CK(dev_alloc((void**)&g->out_off, offb, g->pooled, s), "graph allocation");
  CK(dev_alloc((void**)&g->out_adj, adjb, g->pooled, s), "graph allocation");
  if (with_in) {
    CK(dev_alloc((void**)&g->in_off, offb, g->pooled, s), "graph allocation");
    CK(dev_alloc((void**)&g->in_adj, adjb, g->pooled, s), "graph allocation");
  }
  return GB_OK;
}

void graph_free(gb_graph* g) {
  if (!g) return;
  cudaStream_t s = g->pool_stream;
  dev_free(g->out_off, g->pooled, s);
  dev_free(g->out_adj, g->pooled, s);
  dev_free(g->in_off, g->pooled, s);
  dev_free(g->in_adj, g->pooled, s);
  hint_free(g, g->hint_out);
  hint_free(g, g->hint_in);
  g->out_off = g->in_off = nullptr;
  g->out_adj = g->in_adj = nullptr;
  g->hint_out = g->hint_in = nullptr;
}

// Builds the pull hints of a graph whose CSR is complete on the device
// (hint arrays from the pool: a rebuild maps no memory).
gb_status graph_hints(gb_ctx* c, gb_graph* g) {
  const size_t hb = (size_t)(g->n > 0 ? g->n : 1) * 4;
  if (!g->hint_out)
    CK(dev_alloc((void**)&g->hint_out, hb, true, c->stream), "hint allocation");
  if (!g->symmetric && !g->hint_in)
    CK(dev_alloc((void**)&g->hint_in, hb, true, c->stream), "hint allocation");
  CK(gb::build_hints(g->n, g->m, g->out_off, g->out_adj, g->in_off, g->in_adj, g->hint_out, g->hint_in,
                     c->stream),
     "hints");
  return GB_OK;
}
}  // namespace gb

namespace {
using gb::graph_alloc;
using gb::graph_free;
using gb::graph_hints;

// Phase times (ms) of the run in ring slot i: trim, reachability and colour
// from the device times the run kernel wrote at its phase boundaries, the
// tail (statistics pass) and the total from the run's events.  The ring copy
// must be current (the caller synchronised the stream).
gb_status run_phase_ms(gb_ctx* c, int i, double* ms) {
  const unsigned long long* t = c->h_tphase + 4 * i;
  for (int j = 0; j < 3; ++j) ms[j] = t[j + 1] > t[j] ? (double)(t[j + 1] - t[j]) / 1e6 : 0.0;
  cudaEvent_t* ev = c->ev[i];
  float tail = 0.f, tot = 0.f;
  CK(cudaEventElapsedTime(&tail, ev[1], ev[4]), "phase times");
  CK(cudaEventElapsedTime(&tot, ev[0], ev[4]), "phase times");
  ms[3] = tail;
  ms[4] = tot;
  return GB_OK;
}

gb_status copy_phase_ring(gb_ctx* c) {
  CK(cudaMemcpyAsync(c->h_tphase, c->d_tphase, sizeof(unsigned long long) * 4 * gb_ctx::kRing,
                     cudaMemcpyDeviceToHost, c->stream),
     "phase times");
  CK(cudaStreamSynchronize(c->stream), "phase times");
  return GB_OK;
}

gb_status finish_run(gb_ctx* c, const gb_graph* g, gb_stats* st) {
  CK(cudaStreamSynchronize(c->stream), "run");
  (void)g;
  const gb::Ctl& h = *c->h_ctl;
  if (st) {
    gb_status ps = copy_phase_ring(c);
    if (ps != GB_OK) return ps;
    std::memset(st, 0, sizeof(*st));
    double ms[5];
    if (run_phase_ms(c, (c->runs - 1) % gb_ctx::kRing, ms) == GB_OK) {
      st->ms_trim = ms[0];
      st->ms_reach = ms[1];
      st->ms_colour = ms[2];
      st->ms_canon = ms[3];
      st->ms_total = ms[4];
    }
    st->pivot = h.pivot;
    st->colour_rounds = h.ncolour_rounds;
    st->n_trim = h.ntrim;
    st->n_visit_fw = h.nvisit_fw;
    st->n_fwbw = h.nscc_fwbw;
    st->unassigned = h.unassigned;
    int64_t tv = 0, te = 0, tl = 0;
    for (int k = 0; k < 4; ++k) {
      tv += (int64_t)h.kst[k][0];
      te += (int64_t)h.kst[k][1];
      tl += (int64_t)h.kst[k][2];
    }
    st->vtx_reads = tv;
    st->edge_reads = te;
    st->list_rw = tl;
    const int64_t n = g->n, nb = (n + 7) / 8;
    auto kb = [&](int k) {
      return 16 * (int64_t)h.kst[k][0] + 4 * (int64_t)h.kst[k][1] + 4 * (int64_t)h.kst[k][2];
    };
    // trim: degrees (counted as offset records), labels, valid bitmap
    // written and re-read for the ordered list
    st->bytes_trim = kb(gb::kKTrim) + 4 * n + 2 * nb;
    // reach: per traversal the visited bitmap (read + write) and the allowed
    // bitmap (read); then labels of the found component and the valid
    // bitmap update
    const int64_t trav = (h.stat[gb::kStFwSteps] ? 1 : 0) + (h.stat[gb::kStBwSteps] ? 1 : 0);
    st->bytes_reach = kb(gb::kKReach) + trav * 3 * nb + 4 * (int64_t)h.nscc_fwbw + 2 * nb;
    // colour: every list entry also touches its colour (init + read)
    st->bytes_colour = kb(gb::kKColour) + 4 * (int64_t)h.kst[gb::kKColour][2];
    // final pass: one label read per vertex
    st->bytes_canon = 4 * n;
    st->m_visit_fw = (int64_t)h.mvis[0];
    st->m_visit_bw = (int64_t)h.mvis[1];
    st->pull_edges = (int64_t)h.pull_edges;
    st->fwbw_rounds = (h.pivot >= 0 ? 1 : 0) + (int64_t)h.nrounds;
    st->trim_steps = (int64_t)h.stat[gb::kStTrimSteps];
    st->fw_steps = (int64_t)h.stat[gb::kStFwSteps];
    st->bw_steps = (int64_t)h.stat[gb::kStBwSteps];
    st->pull_steps = (int64_t)h.stat[gb::kStPullSteps];
    st->colour_steps = (int64_t)h.stat[gb::kStColourSteps];
    st->mark_steps = (int64_t)h.stat[gb::kStMarkSteps];
    st->grid_blocks = c->grid;
    st->err_where = h.err_where;
  }
  *c->h_sticky = 0;
  cudaMemsetAsync(c->d_sticky, 0, 2 * sizeof(int), c->stream);
  if (h.err != 0) {
    char buf[128];
    std::snprintf(buf, sizeof(buf), "device error %d at site %d", h.err, h.err_where);
    gb_set_error("%s", buf);
    return (gb_status)h.err;
  }
  (void)g;
  return GB_OK;
}

// True when a run of g with options o takes the one-block path (small.cu).
// small_path 1 (automatic) takes it while the graph has at most
// kSmallAutoEdges edges: above that the one block's passes over the edges
// cost more than the cooperative grid's steps (measured on GB300, SCC:
// 101 against 215 us at 2,000 vertices and 25,000 edges, 173 against
// 220 us at 4,000 and 52,000, 233 against 222 us at 6,000 and 73,000);
// 2 takes it whenever the graph fits.
bool use_small(const gb_graph* g, const gb_opts* o) {
  if (g->n > gb::kSmallMaxN || g->m >= (1ll << 31)) return false;
  const int32_t mode = o ? o->small_path : 1;
  if (o && o->canonical == 0) return false;
  return mode >= 2 || (mode == 1 && g->m <= gb::kSmallAutoEdges);
}

// A graph of at most kSmallMaxN vertices: one thread block runs the whole
// pipeline (small.cu).  Same stream order, error latch and events as a run
// of the cooperative kernel; the statistics hold the times only.
gb_status run_small(gb_ctx* c, const gb_graph* g, gb::RunKind kind, int32_t* labels,
                    const gb_opts* o, gb_stats* st, bool wait) {
  const bool dev_labels = is_device_ptr(labels);
  if (!wait && !dev_labels) {
    gb_set_error("run: the asynchronous form needs device labels%s", "");
    return GB_ERR_INVALID;
  }
  gb_status s = ensure_ws(c, g->n);
  if (s != GB_OK) return s;
  int32_t* dl = dev_labels ? labels : c->w.label;
  cudaStream_t sm = c->stream;
  CK(cudaMemsetAsync(&c->d_ctl->err, 0, 2 * sizeof(int), sm), "memset");
  cudaEvent_t* ev = c->ev[c->runs % gb_ctx::kRing];
  CK(cudaMemsetAsync(c->d_tphase + 4 * (c->runs % gb_ctx::kRing), 0,
                     4 * sizeof(unsigned long long), sm),
     "memset");
  c->runs++;
  cudaEventRecord(ev[0], sm);
  gb::SmallDesc d{};
  d.n = g->n;
  d.m = g->m;
  d.out_off = g->out_off;
  d.out_adj = g->out_adj;
  d.in_off = g->symmetric ? nullptr : g->in_off;
  d.in_adj = g->symmetric ? nullptr : g->in_adj;
  d.labels = dl;
  const int32_t max_steps = o && o->max_steps > 0 ? o->max_steps : (1 << 30);
  CK(gb::launch_small(kind == gb::kSCC ? 0 : 1, d, nullptr, 1, g->n, max_steps, &c->d_ctl->err,
                      sm, o ? o->colour_mode : 2),
     "kernel launch");
  cudaEventRecord(ev[1], sm);
  cudaEventRecord(ev[4], sm);
  CK(gb::launch_latch(c->d_ctl, c->d_sticky, sm), "kernel launch");
  if (!dev_labels)
    CK(cudaMemcpyAsync(labels, dl, (size_t)g->n * 4, cudaMemcpyDeviceToHost, sm), "labels copy");
  CK(cudaMemcpyAsync(&c->h_ctl->err, &c->d_ctl->err, 2 * sizeof(int), cudaMemcpyDeviceToHost, sm),
     "status copy");
  if (!wait) return GB_OK;
  CK(cudaStreamSynchronize(sm), "run");
  if (st) {
    std::memset(st, 0, sizeof(*st));
    float tot = 0.f;
    if (cudaEventElapsedTime(&tot, ev[0], ev[4]) == cudaSuccess) st->ms_total = tot;
    st->pivot = -1;
    st->grid_blocks = 1;
    st->err_where = c->h_ctl->err_where;
  }
  *c->h_sticky = 0;
  cudaMemsetAsync(c->d_sticky, 0, 2 * sizeof(int), sm);
  const int err = c->h_ctl->err;
  if (err != 0) {
    gb_set_error("run: %s", err == gb::kErrIterLimit ? "a loop of the one-block path hit its step cap"
                                                     : "device error in the one-block path");
    return (gb_status)err;
  }
  return GB_OK;
}

// WCC of a device graph by sampled union-find (cc_sampled_device): the
// same bookkeeping as the one-block path (labels, events, status latch).
gb_status run_sampled_cc(gb_ctx* c, const gb_graph* g, int32_t* labels, gb_stats* st,
                         bool wait) {
  const bool dev_labels = is_device_ptr(labels);
  if (!wait && !dev_labels) {
    gb_set_error("run: the asynchronous form needs device labels%s", "");
    return GB_ERR_INVALID;
  }
  gb_status s = ensure_ws(c, g->n);
  if (s != GB_OK) return s;
  int32_t* dl = dev_labels ? labels : c->w.label;
  cudaStream_t sm = c->stream;
  CK(cudaMemsetAsync(&c->d_ctl->err, 0, 2 * sizeof(int), sm), "memset");
  cudaEvent_t* ev = c->ev[c->runs % gb_ctx::kRing];
  CK(cudaMemsetAsync(c->d_tphase + 4 * (c->runs % gb_ctx::kRing), 0,
                     4 * sizeof(unsigned long long), sm),
     "memset");
  c->runs++;
  cudaEventRecord(ev[0], sm);
  // (a checked device graph: the id flag, err_where, stays clear)
  CK(gb::cc_sampled_device(g->n, g->out_off, g->out_adj, g->symmetric ? nullptr : g->in_off,
                           g->symmetric ? nullptr : g->in_adj, dl, &c->d_ctl->err_where,
                           &c->d_ctl->err, sm),
     "kernel launch");
  cudaEventRecord(ev[1], sm);
  cudaEventRecord(ev[4], sm);
  CK(gb::launch_latch(c->d_ctl, c->d_sticky, sm), "kernel launch");
  if (!dev_labels)
    CK(cudaMemcpyAsync(labels, dl, (size_t)g->n * 4, cudaMemcpyDeviceToHost, sm), "labels copy");
  CK(cudaMemcpyAsync(&c->h_ctl->err, &c->d_ctl->err, 2 * sizeof(int), cudaMemcpyDeviceToHost, sm),
     "status copy");
  if (!wait) return GB_OK;
  CK(cudaStreamSynchronize(sm), "run");
  if (st) {
    std::memset(st, 0, sizeof(*st));
    float tot = 0.f;
    if (cudaEventElapsedTime(&tot, ev[0], ev[4]) == cudaSuccess) st->ms_total = tot;
    st->pivot = -1;
    st->err_where = c->h_ctl->err_where;
  }
  *c->h_sticky = 0;
  cudaMemsetAsync(c->d_sticky, 0, 2 * sizeof(int), sm);
  const int err = c->h_ctl->err;
  if (err != 0) {
    gb_set_error("run: %s", "a union-find link ran out of retries");
    return (gb_status)err;
  }
  return GB_OK;
}

gb_status run_graph_impl(gb_ctx* c, const gb_graph* g, gb::RunKind kind, int32_t* labels,
                         const gb_opts* o, gb_stats* st, bool wait, const gb::BatchView* bv) {
  if (!c || !g) {
    gb_set_error("run: null context or graph%s", "");
    return GB_ERR_INVALID;
  }
  if (g->n > 0 && !labels) {
    gb_set_error("run: null labels%s", "");
    return GB_ERR_INVALID;
  }
  if (g->device != c->device) {
    gb_set_error("run: graph and context are on different devices%s", "");
    return GB_ERR_INVALID;
  }
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  if (g->n == 0) return GB_OK;
  if (bv == nullptr && use_small(g, o)) return run_small(c, g, kind, labels, o, st, wait);
  if (bv == nullptr && kind == gb::kWCC && o && o->wcc_mode == 1)
    return run_sampled_cc(c, g, labels, st, wait);
  gb_status s = ensure_ws(c, g->n);
  if (s != GB_OK) return s;
  const bool dev_labels = is_device_ptr(labels);
  if (!wait && !dev_labels) {
    gb_set_error("run: the asynchronous form needs device labels%s", "");
    return GB_ERR_INVALID;
  }
  gb::Work w = c->w;
  w.n = g->n;
  w.nwords = (g->n + 31) / 32;
  w.m = g->m;
  if (dev_labels) w.label = labels;
  gb::RunParams p{};
  fill_params(o, p);
  p.count_unassigned = st != nullptr ? 1 : 0;
  int grid = c->grid;
  if (o && o->grid_blocks > 0 && o->grid_blocks < grid) grid = o->grid_blocks;
  gb::GraphView gv{};
  gv.n = g->n;
  gv.m = g->m;
  gv.out = {g->out_off, g->out_adj, g->hint_out};
  if (g->symmetric) {
    // a symmetric graph is its own reverse
    gv.in = kind == gb::kSCC ? gv.out : gb::Csr{nullptr, nullptr, nullptr};
  } else {
    gv.in = {g->in_off, g->in_adj, g->hint_in};
  }
  gv.batch = gb::BatchView{};
  cudaStream_t sm = c->stream;
  if (bv != nullptr) {
    gv.batch = *bv;
    CK(cudaMemsetAsync(bv->pkey, 0, (size_t)bv->count * 8, sm), "memset");
    CK(cudaMemsetAsync(bv->gmin, 0x7f, (size_t)bv->count * 4, sm), "memset");
  }
  // the reached and done bitmaps are adjacent in the workspace: one memset
  // clears all three
  CK(cudaMemsetAsync(c->d_ctl, 0, sizeof(gb::Ctl), sm), "memset");
  CK(cudaMemsetAsync(w.fvis, 0,
                     (size_t)((char*)(w.done + w.nwords) - (char*)w.fvis), sm),
     "memset");
  cudaEvent_t* ev = c->ev[c->runs % gb_ctx::kRing];
  w.tphase = c->d_tphase + 4 * (c->runs % gb_ctx::kRing);
  CK(cudaMemsetAsync(w.tphase, 0, 4 * sizeof(unsigned long long), sm), "memset");
  c->runs++;
  CK(gb::launch_run(gv, kind, p, w, grid, sm, ev), "kernel launch");
  CK(gb::launch_latch(c->d_ctl, c->d_sticky, sm), "kernel launch");
  if (bv != nullptr) CK(gb::launch_localize(w.label, g->n, bv->gid, bv->vbase, sm), "localize");
  if (!dev_labels)
    CK(cudaMemcpyAsync(labels, w.label, (size_t)g->n * 4, cudaMemcpyDeviceToHost, sm), "labels copy");
  CK(cudaMemcpyAsync(c->h_ctl, c->d_ctl, sizeof(gb::Ctl), cudaMemcpyDeviceToHost, sm), "status copy");
  if (!wait) return GB_OK;
  return finish_run(c, g, st);
}

}  // namespace

const gb_opts* gb::class_opts(const gb_ctx* c, int64_t n) {
  if (!c || c->cls_n.empty()) return nullptr;
  for (size_t i = 0; i < c->cls_n.size(); ++i)
    if (n <= c->cls_n[i]) return &c->cls_opts[i];
  return &c->cls_opts.back();
}

gb_status gb::run_graph(gb_ctx* c, const gb_graph* g, RunKind kind, int32_t* labels,
                        const gb_opts* o, gb_stats* st, bool wait, const BatchView* bv) {
  // a run given no options takes the context's options for its size class
  if (!o && c && g) o = class_opts(c, g->n);
  return run_graph_impl(c, g, kind, labels, o, st, wait, bv);
}

namespace {
using gb::validate_csr;

std::mutex g_default_mu;
gb_ctx* g_default_ctx = nullptr;
gb_graph* g_stage = nullptr;     // reused device buffers of the drop-ins
// gb_run_scc: share of the in-edges whose lists are derived on the device
// (the rest of in_array is copied beside the derivation)
std::atomic<double> g_dropin_share{0.8};
int64_t g_stage_m = -1;
int32_t g_stage_n = -1;

}  // namespace

extern "C" {

void gb_struct_sizes(int64_t sizes[3]) {
  if (!sizes) return;
  sizes[0] = (int64_t)sizeof(gb_opts);
  sizes[1] = (int64_t)sizeof(gb_stats);
  sizes[2] = (int64_t)sizeof(gb_server_stats);
}

void gb_opts_default(gb_opts* o) {
  if (!o) return;
  o->trim_level = 1;
  o->canonical = 1;
  o->pivot = -1;
  o->vert_cutoff = 10000;
  o->t_block = 512;
  o->t_grid = 32768;
  o->k_pull = 4;
  o->alpha = 15.0f;
  o->beta = 25.0f;
  o->max_steps = 1 << 30;
  o->grid_blocks = 0;
  o->trim_pairs = 0;
  o->fwbw_rounds = 1;
  o->expand_mode = 0;
  o->small_path = 1;
  o->colour_mode = 2;
  o->wcc_mode = 0;
}

gb_status gb_ctx_create(int device, gb_ctx** out) {
  if (!out) return GB_ERR_INVALID;
  *out = nullptr;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    cudaGetLastError();
    gb_set_error("gb_ctx_create: %s", e != cudaSuccess ? cudaGetErrorString(e) : "no device");
    return GB_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= count) return GB_ERR_INVALID;
  CK(cudaSetDevice(device), "cudaSetDevice");
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties");
  if (prop.major != 10 || prop.minor != 3 || !prop.cooperativeLaunch) {
    char buf[128];
    std::snprintf(buf, sizeof(buf), "device %d is sm_%d%d (needs sm_103 with cooperative launch)",
                  device, prop.major, prop.minor);
    gb_set_error("gb_ctx_create: %s", buf);
    return GB_ERR_UNSUPPORTED;
  }
  gb_ctx* c = new (std::nothrow) gb_ctx();
  if (!c) return GB_ERR_OOM;
  c->device = device;
  gb_status s = GB_OK;
  do {
    cudaError_t r;
    if ((r = cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking)) != cudaSuccess) { s = cuda_fail(r, "stream"); break; }
    c->stream = c->own;
    if ((r = cudaMalloc(&c->d_ctl, sizeof(gb::Ctl))) != cudaSuccess) { s = cuda_fail(r, "ctl"); break; }
    if ((r = cudaMallocHost(&c->h_ctl, sizeof(gb::Ctl))) != cudaSuccess) { s = cuda_fail(r, "ctl"); break; }
    if ((r = cudaMalloc(&c->d_sticky, 2 * sizeof(int))) != cudaSuccess) { s = cuda_fail(r, "sticky"); break; }
    const size_t pr = sizeof(unsigned long long) * 4 * gb_ctx::kRing;
    if ((r = cudaMalloc(&c->d_tphase, pr)) != cudaSuccess) { s = cuda_fail(r, "phase ring"); break; }
    if ((r = cudaMallocHost(&c->h_tphase, pr)) != cudaSuccess) { s = cuda_fail(r, "phase ring"); break; }
    cudaMemset(c->d_tphase, 0, pr);
    std::memset(c->h_tphase, 0, pr);
    if ((r = cudaMallocHost(&c->h_sticky, 2 * sizeof(int))) != cudaSuccess) { s = cuda_fail(r, "sticky"); break; }
    cudaMemset(c->d_sticky, 0, 2 * sizeof(int));
    std::memset(c->h_ctl, 0, sizeof(gb::Ctl));
    c->h_sticky[0] = c->h_sticky[1] = 0;
    for (int k = 0; k < gb_ctx::kRing && s == GB_OK; ++k)
      for (int i = 0; i < 5 && s == GB_OK; ++i)
        if ((r = cudaEventCreate(&c->ev[k][i])) != cudaSuccess) s = cuda_fail(r, "event");
    if (s != GB_OK) break;
    c->grid = gb::max_coop_grid(device);
    if (c->grid <= 0) { gb_set_error("gb_ctx_create: %s", "no cooperative occupancy"); s = GB_ERR_UNSUPPORTED; break; }
    // Scratch freed through the stream-ordered allocator stays reserved in
    // the device's pool, up to kPoolKeep, instead of going back to the
    // driver at every synchronise: per-call scratch (hint lists, union-find
    // parents, staged labels) is then not mapped afresh on every call.  A
    // larger threshold already set in the process is left as it is.
    constexpr uint64_t kPoolKeep = 4ull << 30;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
      uint64_t cur = 0;
      if (cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &cur) == cudaSuccess &&
          cur < kPoolKeep) {
        uint64_t keep = kPoolKeep;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
      }
    }
    cudaGetLastError();
  } while (0);
  if (s != GB_OK) {
    gb_ctx_destroy(c);
    return s;
  }
  *out = c;
  return GB_OK;
}

gb_status gb_ctx_destroy(gb_ctx* c) {
  if (!c) return GB_OK;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  cudaFree(c->ws);
  cudaFree(c->d_ctl);
  cudaFree(c->d_sticky);
  cudaFree(c->d_tphase);
  if (c->h_tphase) cudaFreeHost(c->h_tphase);
  if (c->h_ctl) cudaFreeHost(c->h_ctl);
  if (c->h_sticky) cudaFreeHost(c->h_sticky);
  for (auto& set : c->ev)
    for (auto& e : set)
      if (e) cudaEventDestroy(e);
  if (c->own) cudaStreamDestroy(c->own);
  delete c;
  return GB_OK;
}

gb_status gb_ctx_set_stream(gb_ctx* c, void* s) {
  if (!c) return GB_ERR_INVALID;
  c->stream = s ? (cudaStream_t)s : c->own;
  return GB_OK;
}

void* gb_ctx_stream(gb_ctx* c) { return c ? (void*)c->stream : nullptr; }

gb_status gb_ctx_sync(gb_ctx* c) {
  if (!c) return GB_ERR_INVALID;
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  CK(cudaMemcpyAsync(c->h_sticky, c->d_sticky, 2 * sizeof(int), cudaMemcpyDeviceToHost, c->stream), "sync");
  CK(cudaStreamSynchronize(c->stream), "sync");
  const int err = c->h_sticky[0], where = c->h_sticky[1];
  CK(cudaMemsetAsync(c->d_sticky, 0, 2 * sizeof(int), c->stream), "sync");
  if (err) {
    char buf[96];
    std::snprintf(buf, sizeof(buf), "device error %d at site %d", err, where);
    gb_set_error("%s", buf);
    return (gb_status)err;
  }
  return GB_OK;
}

gb_status gb_ctx_phase_times(gb_ctx* c, int32_t count, double* ms) {
  if (!c || !ms || count < 0 || count > gb_ctx::kRing || count > c->runs) return GB_ERR_INVALID;
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  gb_status s = copy_phase_ring(c);
  if (s != GB_OK) return s;
  for (int32_t i = 0; i < count; ++i) {
    s = run_phase_ms(c, (int)((c->runs - count + i) % gb_ctx::kRing), ms + 5 * i);
    if (s != GB_OK) return s;
  }
  return GB_OK;
}

int32_t gb_ctx_reach_trace(gb_ctx* c, int64_t* t_ns, int32_t* count, int32_t* mode, int32_t cap) {
  return gb_ctx_reach_trace2(c, t_ns, count, mode, nullptr, cap);
}

int32_t gb_ctx_block_times(gb_ctx* c, int64_t* t_ns, int32_t cap) {
  if (!c || !t_ns || cap < 0) return 0;
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return 0;
  const int k = cap < gb::kBlkTimes ? cap : gb::kBlkTimes;
  for (int i = 0; i < k; ++i) t_ns[i] = (int64_t)c->h_ctl->blk_t[i];
  return k;
}

int32_t gb_ctx_reach_trace2(gb_ctx* c, int64_t* t_ns, int32_t* count, int32_t* mode,
                            int64_t* extra, int32_t cap) {
  if (!c || cap < 0) return 0;
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return 0;
  const gb::Ctl& h = *c->h_ctl;
  const int total = h.ntrace;
  const int have = total < gb::kTrace ? total : gb::kTrace;
  const int k = have < cap ? have : cap;
  for (int i = 0; i < k; ++i) {
    const auto& e = h.trace[(total - k + i) % gb::kTrace];
    if (t_ns) t_ns[i] = (int64_t)e.t;
    if (count) count[i] = e.count;
    if (mode) mode[i] = e.mode;
    if (extra) {
      extra[3 * i] = e.t_mid ? (int64_t)(e.t_mid - e.t) : 0;
      extra[3 * i + 1] = e.nwarp;
      extra[3 * i + 2] = e.nblock;
    }
  }
  return k;
}

}  // extern "C"

gb_status gb::graph_from_edges(gb_ctx* c, int32_t n, int64_t m, const int32_t* src,
                               const int32_t* dst, bool pooled, gb_graph** out) {
  if (!c || !out || n < 0 || m < 0 || (m > 0 && (!src || !dst))) return GB_ERR_INVALID;
  *out = nullptr;
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  gb_graph* g = new (std::nothrow) gb_graph();
  if (!g) return GB_ERR_OOM;
  g->device = c->device;
  g->n = n;
  g->m = m;
  g->pooled = pooled;
  g->pool_stream = c->stream;
  gb_status s = graph_alloc(g, true);
  const int32_t *ds = src, *dd = dst;
  int32_t *ts = nullptr, *tt = nullptr;
  if (s == GB_OK && m > 0 && !is_device_ptr(src)) {
    cudaError_t e = gb::dev_alloc((void**)&ts, (size_t)m * 4, pooled, c->stream);
    if (e == cudaSuccess) e = gb::dev_alloc((void**)&tt, (size_t)m * 4, pooled, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ts, src, (size_t)m * 4, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(tt, dst, (size_t)m * 4, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) s = cuda_fail(e, "edge upload");
    ds = ts;
    dd = tt;
  }
  if (s == GB_OK) {
    bool ok = true;
    cudaError_t e = gb::build_csr(n, m, ds, dd, g->out_off, g->out_adj, g->in_off, g->in_adj, c->stream, &ok);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) s = cuda_fail(e, "CSR build");
    else if (!ok) {
      gb_set_error("gb_graph_from_edges: %s", "vertex id outside [0, n)");
      s = GB_ERR_INVALID;
    }
  }
  gb::dev_free(ts, pooled, c->stream);
  gb::dev_free(tt, pooled, c->stream);
  if (s == GB_OK) s = graph_hints(c, g);
  if (s != GB_OK) {
    graph_free(g);
    delete g;
    return s;
  }
  *out = g;
  return GB_OK;
}

extern "C" {

gb_status gb_graph_from_edges(gb_ctx* c, int32_t n, int64_t m, const int32_t* src,
                              const int32_t* dst, gb_graph** out) {
  return gb::graph_from_edges(c, n, m, src, dst, false, out);
}

// Validates CSR arrays already on the device: off[0] == 0, off[n] == m,
// offsets non-decreasing, ids in [0, n).
}  // extern "C"

gb_status gb::reserve_workspace(gb_ctx* c, int32_t n) { return ensure_ws(c, n); }

gb_status gb::validate_csr(gb_ctx* c, int32_t n, int64_t m, const int64_t* off,
                           const int32_t* adj) {
  int bad = 0;
  cudaError_t e = gb::check_csr(n, m, off, adj, c->stream, &bad);
  if (e != cudaSuccess) return cuda_fail(e, "CSR check");
  if (bad) {
    gb_set_error("CSR check: %s", "offsets not monotone from 0 to m, or an id outside [0, n)");
    return GB_ERR_INVALID;
  }
  return GB_OK;
}

extern "C" {

static gb_status upload(gb_ctx* c, void* dst, const void* src, size_t bytes) {
  if (bytes == 0) return GB_OK;
  CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, c->stream), "upload");
  return GB_OK;
}

gb_status gb_graph_from_csr(gb_ctx* c, int32_t n, int64_t m, const int64_t* out_off,
                            const int32_t* out_adj, const int64_t* in_off, const int32_t* in_adj,
                            gb_graph** out) {
  if (!c || !out || n < 0 || m < 0 || !out_off || (m > 0 && !out_adj)) return GB_ERR_INVALID;
  if (in_off == nullptr ? in_adj != nullptr : (m > 0 && in_adj == nullptr)) return GB_ERR_INVALID;
  *out = nullptr;
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  gb_graph* g = new (std::nothrow) gb_graph();
  if (!g) return GB_ERR_OOM;
  g->device = c->device;
  g->n = n;
  g->m = m;
  g->symmetric = in_off == nullptr;
  gb_status s = graph_alloc(g, !g->symmetric);
  if (s == GB_OK) s = upload(c, g->out_off, out_off, (size_t)(n + 1) * 8);
  if (s == GB_OK) s = upload(c, g->out_adj, out_adj, (size_t)m * 4);
  if (s == GB_OK && !g->symmetric) s = upload(c, g->in_off, in_off, (size_t)(n + 1) * 8);
  if (s == GB_OK && !g->symmetric) s = upload(c, g->in_adj, in_adj, (size_t)m * 4);
  if (s == GB_OK) s = validate_csr(c, n, m, g->out_off, g->out_adj);
  if (s == GB_OK && !g->symmetric) s = validate_csr(c, n, m, g->in_off, g->in_adj);
  if (s == GB_OK) s = graph_hints(c, g);
  if (s != GB_OK) {
    graph_free(g);
    delete g;
    return s;
  }
  *out = g;
  return GB_OK;
}

// Whether the current device reads pageable host memory through the host's
// page tables (Grace-class hosts), at the host link's rate; cached per
// device.
static bool pageable_readable() {
  static int cache[64] = {0};  // 0 unknown, 1 no, 2 yes
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return false;
  if (cache[dev] == 0) {
    int a = 0, b = 0;
    cudaDeviceGetAttribute(&a, cudaDevAttrPageableMemoryAccess, dev);
    cudaDeviceGetAttribute(&b, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev);
    cache[dev] = a && b ? 2 : 1;
  }
  return cache[dev] == 2;
}

// An address the device's kernels can read host memory at: pinned memory's
// device address (the same under unified addressing), pageable memory itself
// where the device reads it through the host's page tables; null otherwise
// (and for device memory).
static const void* host_view(const void* p) {
  if (!p) return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type == cudaMemoryTypeHost) return a.devicePointer;
  if (a.type == cudaMemoryTypeUnregistered && pageable_readable()) return p;
  return nullptr;
}

// Whether the host can read p (pageable, pinned or managed memory).
static bool host_readable(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return true;  // not known to the runtime: ordinary host memory
  }
  return a.type != cudaMemoryTypeDevice;
}

// Fills g (whose buffers hold at least n / m) from the reference's CSR layout.
// Host arrays the device can read (pinned, or pageable where the device
// reads it through the host's page tables) are read by the ingest kernels
// directly (one crossing of the host link, checked on the way); other
// memory is copied first.
// derive_share (directed graphs, m < 2^31): the in-lists holding the first
// derive_share of the in-edges (targets below the split vertex) are written
// on the device from the out-CSR while it is read, and the rest of in_array
// is copied by the same kernel (tiles of both interleaved), so the device's
// placement and the host link share the work; 0 copies in_array whole, 1
// (or in_array NULL) does not read it.  The derived lists are checked
// against idl.
static gb_status fill_csr32(gb_ctx* c, gb_graph* g, int32_t n, uint32_t m, const int32_t* out_array,
                            const uint32_t* odl, const int32_t* in_array, const uint32_t* idl,
                            double derive_share) {
  bool derive_in = !g->symmetric && m < (1u << 31) && (derive_share > 0.0 || !in_array);
  // the split is chosen on the host from idl: arrays in device memory are
  // derived whole
  if (!in_array || !host_readable(idl)) derive_share = 1.0;
  // split vertex: the first whose in-offset reaches the derived share
  int32_t t_split = n;
  int64_t e_split = m;
  if (derive_in && derive_share < 1.0 && n > 0 && m > 0) {
    const double goal = derive_share * (double)m;
    int32_t lo = 0, hi = n;
    while (lo < hi) {
      const int32_t mid = lo + (hi - lo) / 2;
      if ((double)idl[mid] >= goal) hi = mid;
      else lo = mid + 1;
    }
    t_split = lo;
    e_split = (int64_t)idl[lo] <= (int64_t)m ? (int64_t)idl[lo] : (int64_t)m;
  }
  const void* vo = host_view(odl);
  const void* va = m > 0 ? host_view(out_array) : odl;
  const void* vi = g->symmetric ? odl : host_view(idl);
  const void* vb = g->symmetric || m == 0 || (derive_in && e_split >= (int64_t)m) ? odl
                                                                                  : host_view(in_array);
  uint32_t* tmp = nullptr;
  if (!(vo && va && vi && vb)) {
    if (!derive_in) {
      CK(cudaMallocAsync(&tmp, (size_t)(n + 1) * 4, c->stream), "offset staging");
      gb_status s = upload(c, tmp, odl, (size_t)(n + 1) * 4);
      if (s == GB_OK) CK(gb::widen_offsets(tmp, g->out_off, (int64_t)n + 1, c->stream), "widen");
      if (s == GB_OK) s = upload(c, g->out_adj, out_array, (size_t)m * 4);
      if (s == GB_OK && !g->symmetric) {
        s = upload(c, tmp, idl, (size_t)(n + 1) * 4);
        if (s == GB_OK) CK(gb::widen_offsets(tmp, g->in_off, (int64_t)n + 1, c->stream), "widen");
        if (s == GB_OK) s = upload(c, g->in_adj, in_array, (size_t)m * 4);
      }
      cudaFreeAsync(tmp, c->stream);
      if (s == GB_OK) s = validate_csr(c, n, m, g->out_off, g->out_adj);
      if (s == GB_OK && !g->symmetric) s = validate_csr(c, n, m, g->in_off, g->in_adj);
      return s;
    }
    // staged on the device, then ingested from there (the out-lists in place)
    CK(cudaMallocAsync(&tmp, (size_t)(n + 1) * 8, c->stream), "offset staging");
    gb_status s = upload(c, tmp, odl, (size_t)(n + 1) * 4);
    if (s == GB_OK) s = upload(c, tmp + n + 1, idl, (size_t)(n + 1) * 4);
    if (s == GB_OK) s = upload(c, g->out_adj, out_array, (size_t)m * 4);
    if (s == GB_OK && e_split < (int64_t)m)
      s = upload(c, g->in_adj + e_split, in_array + e_split, (size_t)((int64_t)m - e_split) * 4);
    if (s != GB_OK) {
      cudaFreeAsync(tmp, c->stream);
      return s;
    }
    vo = tmp;
    vi = tmp + n + 1;
    va = g->out_adj;
  }
  int* d_bad = nullptr;
  cudaError_t e = cudaMallocAsync(&d_bad, sizeof(int), c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_bad, 0, sizeof(int), c->stream);
  // the in-lists from e_split on: copied inside the derivation kernel from
  // host memory it reads, or already staged (then checked here)
  const bool tail_in_kernel = tmp == nullptr && e_split < (int64_t)m;
  if (e == cudaSuccess && derive_in)
    e = gb::ingest_csr32_derive_in(n, m, (const uint32_t*)vo, (const int32_t*)va,
                                   (const uint32_t*)vi, g->out_off, g->out_adj, g->in_off,
                                   g->in_adj, t_split,
                                   tail_in_kernel ? (const int32_t*)vb : nullptr,
                                   tail_in_kernel ? e_split : (int64_t)m, d_bad, c->stream);
  if (e == cudaSuccess && derive_in && !tail_in_kernel && e_split < (int64_t)m)
    e = gb::check_ids_flag(n, g->in_adj + e_split, (int64_t)m - e_split, d_bad, c->stream);
  if (e == cudaSuccess && !derive_in)
    e = gb::ingest_csr32(n, m, (const uint32_t*)vo, (const int32_t*)va, g->out_off, g->out_adj,
                         d_bad, c->stream);
  if (e == cudaSuccess && !derive_in && !g->symmetric)
    e = gb::ingest_csr32(n, m, (const uint32_t*)vi, (const int32_t*)vb, g->in_off, g->in_adj,
                         d_bad, c->stream);
  int bad = 0;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (d_bad) cudaFreeAsync(d_bad, c->stream);
  if (tmp) cudaFreeAsync(tmp, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "ingest");
  if (bad) {
    gb_set_error("CSR check: %s",
                 derive_in ? "offsets not monotone from 0 to m, an id outside [0, n), or in-degrees "
                             "that do not match the out-CSR"
                           : "offsets not monotone from 0 to m, or an id outside [0, n)");
    return GB_ERR_INVALID;
  }
  return GB_OK;
}

gb_status gb_graph_from_csr32(gb_ctx* c, int32_t n, uint32_t m, const int32_t* out_array,
                              const uint32_t* odl, const int32_t* in_array, const uint32_t* idl,
                              gb_graph** out) {
  if (!c || !out || n < 0 || !odl || (m > 0 && !out_array) || (in_array && !idl))
    return GB_ERR_INVALID;
  // in-offsets without in-lists: the in-lists come from the out-CSR
  const bool derive = idl && !in_array;
  if (derive && m >= (1u << 31)) {
    gb_set_error("gb_graph_from_csr32: %s", "deriving the in-lists needs m < 2^31");
    return GB_ERR_INVALID;
  }
  *out = nullptr;
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  gb_graph* g = new (std::nothrow) gb_graph();
  if (!g) return GB_ERR_OOM;
  g->device = c->device;
  g->n = n;
  g->m = m;
  g->symmetric = idl == nullptr;
  gb_status s = graph_alloc(g, !g->symmetric);
  if (s == GB_OK) s = fill_csr32(c, g, n, m, out_array, odl, in_array, idl, derive ? 1.0 : 0.0);
  if (s == GB_OK) s = graph_hints(c, g);
  if (s != GB_OK) {
    graph_free(g);
    delete g;
    return s;
  }
  *out = g;
  return GB_OK;
}

gb_status gb_graph_rmat(gb_ctx* c, int32_t scale, int32_t ef, uint64_t seed, double a, double b,
                        double cc, gb_graph** out) {
  if (!c || !out || scale < 1 || scale > 30 || ef < 1) return GB_ERR_INVALID;
  *out = nullptr;
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  int32_t *s = nullptr, *d = nullptr;
  int64_t m = 0;
  CK(gb::rmat_edges_device((int32_t)(1 << scale), ef, seed, gb_rmat_thresholds(a, b, cc), &s, &d, &m,
                           c->stream),
     "R-MAT");
  gb_status st = gb_graph_from_edges(c, (int32_t)(1 << scale), m, s, d, out);
  cudaFreeAsync(s, c->stream);
  cudaFreeAsync(d, c->stream);
  cudaStreamSynchronize(c->stream);
  return st;
}

gb_status gb_graph_rmat_n(gb_ctx* c, int32_t n, int32_t ef, uint64_t seed, double a, double b,
                          double cc, gb_graph** out) {
  if (!c || !out || n < 1 || ef < 1) return GB_ERR_INVALID;
  *out = nullptr;
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  int32_t *s = nullptr, *d = nullptr;
  int64_t m = 0;
  CK(gb::rmat_edges_device(n, ef, seed, gb_rmat_thresholds(a, b, cc), &s, &d, &m, c->stream),
     "R-MAT");
  gb_status st = gb_graph_from_edges(c, n, m, s, d, out);
  cudaFreeAsync(s, c->stream);
  cudaFreeAsync(d, c->stream);
  cudaStreamSynchronize(c->stream);
  return st;
}

gb_status gb_graph_info(const gb_graph* g, int32_t* n, int64_t* m, int32_t* symmetric) {
  if (!g) return GB_ERR_INVALID;
  if (n) *n = g->n;
  if (m) *m = g->m;
  if (symmetric) *symmetric = g->symmetric;
  return GB_OK;
}

gb_status gb_graph_csr_to_host(const gb_graph* g, int64_t* out_off, int32_t* out_adj,
                               int64_t* in_off, int32_t* in_adj) {
  if (!g) return GB_ERR_INVALID;
  CK(cudaSetDevice(g->device), "cudaSetDevice");
  if (out_off) CK(cudaMemcpy(out_off, g->out_off, (size_t)(g->n + 1) * 8, cudaMemcpyDeviceToHost), "download");
  if (out_adj && g->m) CK(cudaMemcpy(out_adj, g->out_adj, (size_t)g->m * 4, cudaMemcpyDeviceToHost), "download");
  if (!g->symmetric) {
    if (in_off) CK(cudaMemcpy(in_off, g->in_off, (size_t)(g->n + 1) * 8, cudaMemcpyDeviceToHost), "download");
    if (in_adj && g->m) CK(cudaMemcpy(in_adj, g->in_adj, (size_t)g->m * 4, cudaMemcpyDeviceToHost), "download");
  }
  return GB_OK;
}

gb_status gb_graph_hints_to_host(const gb_graph* g, int32_t* hint_out, int32_t* hint_in) {
  if (!g || !g->hint_out) return GB_ERR_INVALID;
  CK(cudaSetDevice(g->device), "cudaSetDevice");
  if (hint_out && g->n)
    CK(cudaMemcpy(hint_out, g->hint_out, (size_t)g->n * 4, cudaMemcpyDeviceToHost), "download");
  if (hint_in && g->n && g->hint_in)
    CK(cudaMemcpy(hint_in, g->hint_in, (size_t)g->n * 4, cudaMemcpyDeviceToHost), "download");
  return GB_OK;
}

gb_status gb_graph_device_csr(const gb_graph* g, const int64_t** out_off, const int32_t** out_adj,
                              const int64_t** in_off, const int32_t** in_adj) {
  if (!g) return GB_ERR_INVALID;
  if (out_off) *out_off = g->out_off;
  if (out_adj) *out_adj = g->out_adj;
  if (in_off) *in_off = g->in_off;
  if (in_adj) *in_adj = g->in_adj;
  return GB_OK;
}

gb_status gb_graph_pivot(gb_ctx* c, const gb_graph* g, int32_t kind, int32_t* pivot, double* avg) {
  if (!c || !g || !pivot) return GB_ERR_INVALID;
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  const int64_t* in_off = g->symmetric ? (kind == 0 ? g->out_off : nullptr) : g->in_off;
  int32_t pv = -1;
  CK(gb::pivot_device(g->n, g->out_off, in_off, kind, c->stream, &pv), "pivot");
  *pivot = pv;
  if (avg) {
    double deg = (double)g->m;
    if (kind == 1 && !g->symmetric) deg *= 2.0;  // the mirrored graph has 2m arcs
    *avg = g->n ? deg / (double)g->n : 0.0;
  }
  return GB_OK;
}

gb_status gb_graph_destroy(gb_graph* g) {
  if (!g) return GB_OK;
  cudaSetDevice(g->device);
  graph_free(g);
  delete g;
  return GB_OK;
}

gb_status gb_graph_set_hints(gb_ctx* c, gb_graph* g, int32_t on) {
  if (!c || !g || (on != 0 && on != 1)) return GB_ERR_INVALID;
  if (c->device != g->device) {
    gb_set_error("gb_graph_set_hints: %s", "graph and context are on different devices");
    return GB_ERR_INVALID;
  }
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  // runs already queued on the context may still read the hints
  CK(cudaStreamSynchronize(c->stream), "gb_graph_set_hints");
  if (on) return graph_hints(c, g);
  gb::hint_free(g, g->hint_out);
  gb::hint_free(g, g->hint_in);
  return GB_OK;
}

gb_status gb_graph_has_hints(const gb_graph* g, int32_t* on) {
  if (!g || !on) return GB_ERR_INVALID;
  *on = g->hint_out != nullptr;
  return GB_OK;
}

gb_status gb_ctx_set_class_opts(gb_ctx* c, int32_t count, const int64_t* n_max,
                                const gb_opts* opts) {
  if (!c || count < 0 || (count > 0 && (!n_max || !opts))) return GB_ERR_INVALID;
  for (int32_t i = 1; i < count; ++i)
    if (n_max[i] <= n_max[i - 1]) {
      gb_set_error("gb_ctx_set_class_opts: %s", "class bounds must rise");
      return GB_ERR_INVALID;
    }
  c->cls_n.assign(n_max, n_max + count);
  c->cls_opts.assign(opts, opts + count);
  return GB_OK;
}

gb_status gb_scc(gb_ctx* c, const gb_graph* g, int32_t* labels, const gb_opts* o, gb_stats* st) {
  return gb::run_graph(c, g, gb::kSCC, labels, o, st, true, nullptr);
}
gb_status gb_wcc(gb_ctx* c, const gb_graph* g, int32_t* labels, const gb_opts* o, gb_stats* st) {
  return gb::run_graph(c, g, gb::kWCC, labels, o, st, true, nullptr);
}
gb_status gb_cc(gb_ctx* c, const gb_graph* g, int32_t* labels, const gb_opts* o, gb_stats* st) {
  return gb::run_graph(c, g, gb::kWCC, labels, o, st, true, nullptr);
}
}  // extern "C"

namespace {
// SCC / WCC of an edge list: small graphs take the one-block path straight
// from the edges (no CSR build by radix sort, one launch); others get a
// device graph that is built, run and freed.
gb_status run_edges(gb_ctx* c, gb::RunKind kind, int32_t n, int64_t m, const int32_t* src,
                    const int32_t* dst, int32_t* labels, const gb_opts* o) {
  if (!c || n < 0 || m < 0 || (m > 0 && (!src || !dst)) || (n > 0 && !labels)) {
    gb_set_error("run from edges: %s", "bad argument");
    return GB_ERR_INVALID;
  }
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  if (n == 0) return GB_OK;
  gb_opts d;
  gb_opts_default(&d);
  if (!o) o = gb::class_opts(c, n);
  if (!o) o = &d;
  if (n > gb::kSmallMaxN || m >= (1ll << 31) || !o->small_path || !o->canonical) {
    gb_graph* g = nullptr;
    gb_status s = gb_graph_from_edges(c, n, m, src, dst, &g);
    if (s != GB_OK) return s;
    s = gb::run_graph(c, g, kind, labels, o, nullptr, true, nullptr);
    gb_graph_destroy(g);
    return s;
  }
  cudaStream_t sm = c->stream;
  const bool dev_edges = m == 0 || is_device_ptr(src);
  const bool dev_labels = is_device_ptr(labels);
  // one stream-ordered allocation: the edges (from host memory), the SCC
  // CSR built by the block (2m ints) and the labels (for host labels)
  const size_t edge_b = dev_edges ? 0 : (size_t)m * 8;
  const size_t scr_b = kind == gb::kSCC ? (size_t)m * 8 : 0;
  const size_t lab_b = dev_labels ? 0 : (size_t)n * 4;
  char* buf = nullptr;
  if (edge_b + scr_b + lab_b > 0)
    CK(cudaMallocAsync((void**)&buf, edge_b + scr_b + lab_b, sm), "edge staging");
  gb::SmallDesc sd{};
  sd.n = n;
  sd.m = m;
  sd.src = src;
  sd.dst = dst;
  cudaError_t e = cudaSuccess;
  if (!dev_edges) {
    int32_t* ds = reinterpret_cast<int32_t*>(buf);
    e = cudaMemcpyAsync(ds, src, (size_t)m * 4, cudaMemcpyHostToDevice, sm);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(ds + m, dst, (size_t)m * 4, cudaMemcpyHostToDevice, sm);
    sd.src = ds;
    sd.dst = ds + m;
  }
  sd.adj_scratch = scr_b ? reinterpret_cast<int32_t*>(buf + edge_b) : nullptr;
  sd.labels = dev_labels ? labels : reinterpret_cast<int32_t*>(buf + edge_b + scr_b);
  const int32_t max_steps = o->max_steps > 0 ? o->max_steps : (1 << 30);
  if (e == cudaSuccess) e = cudaMemsetAsync(&c->d_ctl->err, 0, 2 * sizeof(int), sm);
  if (e == cudaSuccess)
    e = gb::launch_small(kind == gb::kSCC ? 0 : 1, sd, nullptr, 1, n, max_steps, &c->d_ctl->err,
                         sm, o->colour_mode);
  if (e == cudaSuccess && !dev_labels)
    e = cudaMemcpyAsync(labels, sd.labels, (size_t)n * 4, cudaMemcpyDeviceToHost, sm);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&c->h_ctl->err, &c->d_ctl->err, 2 * sizeof(int), cudaMemcpyDeviceToHost,
                        sm);
  if (buf) cudaFreeAsync(buf, sm);
  const cudaError_t e2 = cudaStreamSynchronize(sm);
  if (e == cudaSuccess) e = e2;
  if (e != cudaSuccess) return cuda_fail(e, "run from edges");
  const int err = c->h_ctl->err;
  if (err != 0) {
    gb_set_error("run from edges: %s", err == gb::kErrInvalid ? "vertex id outside [0, n)"
                                                              : "a loop hit its step cap");
    return (gb_status)err;
  }
  return GB_OK;
}
}  // namespace

extern "C" {

gb_status gb_scc_edges(gb_ctx* c, int32_t n, int64_t m, const int32_t* src, const int32_t* dst,
                       int32_t* labels, const gb_opts* o) {
  return run_edges(c, gb::kSCC, n, m, src, dst, labels, o);
}
gb_status gb_wcc_edges(gb_ctx* c, int32_t n, int64_t m, const int32_t* src, const int32_t* dst,
                       int32_t* labels, const gb_opts* o) {
  return run_edges(c, gb::kWCC, n, m, src, dst, labels, o);
}

gb_status gb_scc_async(gb_ctx* c, const gb_graph* g, int32_t* labels, const gb_opts* o) {
  return gb::run_graph(c, g, gb::kSCC, labels, o, nullptr, false, nullptr);
}
gb_status gb_wcc_async(gb_ctx* c, const gb_graph* g, int32_t* labels, const gb_opts* o) {
  return gb::run_graph(c, g, gb::kWCC, labels, o, nullptr, false, nullptr);
}

// Drop-ins with the reference's signatures: a library-owned context on
// device 0 and reusable device buffers for the graph.
static gb_status default_ctx(gb_ctx** c) {
  if (!g_default_ctx) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
      cudaGetLastError();
      dev = 0;
    }
    gb_status s = gb_ctx_create(dev, &g_default_ctx);
    if (s != GB_OK) return s;
  }
  *c = g_default_ctx;
  return GB_OK;
}

static gb_status stage_graph(gb_ctx* c, int32_t n, int64_t m, bool symmetric, gb_graph** out) {
  if (!g_stage || n > g_stage_n || m > g_stage_m || (g_stage->symmetric && !symmetric)) {
    if (g_stage) {
      graph_free(g_stage);
      delete g_stage;
      g_stage = nullptr;
    }
    g_stage = new (std::nothrow) gb_graph();
    if (!g_stage) return GB_ERR_OOM;
    g_stage->device = c->device;
    g_stage->n = n;
    g_stage->m = m;
    g_stage->symmetric = symmetric;
    gb_status s = graph_alloc(g_stage, !symmetric);
    if (s != GB_OK) {
      graph_free(g_stage);
      delete g_stage;
      g_stage = nullptr;
      return s;
    }
    g_stage_n = n;
    g_stage_m = m;
  }
  g_stage->n = n;
  g_stage->m = m;
  g_stage->symmetric = symmetric;
  *out = g_stage;
  return GB_OK;
}

gb_status gb_dropin_set_derive_share(double share) {
  if (!(share >= 0.0 && share <= 1.0)) return GB_ERR_INVALID;
  g_dropin_share.store(share);
  return GB_OK;
}

gb_status gb_run_scc(int n, unsigned m, const int* out_array, const int* in_array,
                     const unsigned* out_degree_list, const unsigned* in_degree_list, int* scc_maps,
                     int max_deg_vert, double avg_degree, int vert_cutoff) {
  (void)avg_degree;
  const double share = g_dropin_share.load();
  const bool derive = (share > 0.0 || !in_array) && m < (1u << 31);
  if (n < 0 || !out_degree_list || !in_degree_list || (m > 0 && (!out_array || (!derive && !in_array))) ||
      (n > 0 && !scc_maps))
    return GB_ERR_INVALID;
  std::lock_guard<std::mutex> lk(g_default_mu);
  gb_ctx* c;
  gb_status s = default_ctx(&c);
  if (s != GB_OK) return s;
  gb_graph* g;
  if ((s = stage_graph(c, n, m, false, &g)) != GB_OK) return s;
  s = fill_csr32(c, g, n, m, out_array, out_degree_list, in_array, in_degree_list,
                 derive ? share : 0.0);
  if (s != GB_OK) return s;
  gb_opts o;
  gb_opts_default(&o);
  o.pivot = max_deg_vert;
  o.vert_cutoff = vert_cutoff;
  return gb_scc(c, g, scc_maps, &o, nullptr);
}

gb_status gb_run_cc(int n, unsigned m, const int* out_array, const unsigned* out_degree_list,
                    int* cc_maps, int max_deg_vert, double avg_degree) {
  (void)avg_degree;
  if (n < 0 || !out_degree_list || (m > 0 && !out_array) || (n > 0 && !cc_maps)) return GB_ERR_INVALID;
  std::lock_guard<std::mutex> lk(g_default_mu);
  gb_ctx* c;
  gb_status s = default_ctx(&c);
  if (s != GB_OK) return s;
  // A CSR the device reads in place: sampled union-find straight from it,
  // which leaves most of the largest component's lists unread.
  const void* vo = host_view(out_degree_list);
  const void* va = m > 0 ? host_view(out_array) : out_degree_list;
  if (vo && va && n > 0 && m < 0xfffffff0u) {
    CK(cudaSetDevice(c->device), "cudaSetDevice");
    const bool dev_labels = is_device_ptr(cc_maps);
    char* buf = nullptr;
    const size_t lab_b = dev_labels ? 0 : (size_t)n * 4;
    CK(cudaMallocAsync((void**)&buf, lab_b + 16, c->stream), "labels");
    int* d_flags = reinterpret_cast<int*>(buf + lab_b);  // [0] bad CSR, [1] error
    int32_t* dl = dev_labels ? cc_maps : reinterpret_cast<int32_t*>(buf);
    int h_flags[2] = {0, 0};
    cudaError_t e = cudaMemsetAsync(d_flags, 0, 8, c->stream);
    if (e == cudaSuccess)
      e = gb::cc_sampled(n, m, (const uint32_t*)vo, (const int32_t*)va, dl, d_flags, d_flags + 1,
                         c->stream);
    if (e == cudaSuccess && !dev_labels)
      e = cudaMemcpyAsync(cc_maps, dl, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h_flags, d_flags, 8, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFreeAsync(buf, c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "gb_run_cc");
    if (h_flags[0]) {
      gb_set_error("CSR check: %s", "offsets not monotone from 0 to m, or an id outside [0, n)");
      return GB_ERR_INVALID;
    }
    if (h_flags[1]) {
      gb_set_error("gb_run_cc: %s", "a union-find link ran out of retries");
      return (gb_status)h_flags[1];
    }
    return GB_OK;
  }
  gb_graph* g;
  if ((s = stage_graph(c, n, m, true, &g)) != GB_OK) return s;
  s = fill_csr32(c, g, n, m, out_array, out_degree_list, nullptr, nullptr, 0.0);
  if (s != GB_OK) return s;
  gb_opts o;
  gb_opts_default(&o);
  o.pivot = max_deg_vert;
  return gb_wcc(c, g, cc_maps, &o, nullptr);
}

}  // extern "C"
