// Autotuner: picks the run's tunables for one graph (or one batch) by
// timing runs on the device.
//
// The tunables are the degree cutoffs of the push tiers (t_block: a block
// walks the vertex; t_grid: every block takes a slice), the in-edges a
// thread scans in a pull step before the candidate moves to a warp (k_pull),
// the direction-switch factors (alpha: push -> pull, beta: pull -> push),
// the number of resident blocks the cooperative kernel uses, the push
// scheme of the searches: the degree tiers (warp, block, grid slice) or the
// global edge balance of the Kokkos variant's "manhattan global" FW-BW
// (kokkos_scc/fwbw_manhattan_global.cpp:186-289), and for a graph of at
// most 6144 vertices the one-block path against the cooperative grid.  The search is
// coordinate descent from the defaults: each tunable in turn tries its
// candidate values with the others held, and a value is kept when it beats
// the best time so far by more than 2 %; two passes.  Every time is the
// minimum over `reps` device-timed runs (CUDA events on the context stream)
// after one warm-up run.  Results do not depend on the tunables: every
// setting gives the same labels.
//
// The reference has no autotuner; its switch constants are ALPHA / BETA
// (multistep/scc_main.cpp:64-65) and its thread queues are fixed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/gbconn.h"
#include "api_internal.h"
#include "host_internal.h"

namespace {

struct Param {
  int which;  // 0 t_block, 1 t_grid, 2 k_pull, 3 alpha, 4 beta, 5 grid_blocks (fraction),
              // 6 expand_mode, 7 small_path, 8 colour_mode
  std::vector<double> values;
};

void set_param(gb_opts& o, int which, double v, int grid) {
  switch (which) {
    case 0: o.t_block = (int32_t)v; break;
    case 1: o.t_grid = (int32_t)v; break;
    case 2: o.k_pull = (int32_t)v; break;
    case 3: o.alpha = (float)v; break;
    case 4: o.beta = (float)v; break;
    case 5: o.grid_blocks = v >= 1.0 ? 0 : std::max(1, (int)(grid * v)); break;
    case 6: o.expand_mode = (int32_t)v; break;
    case 7: o.small_path = (int32_t)v; break;
    case 8: o.colour_mode = (int32_t)v; break;
  }
}

double get_param(const gb_opts& o, int which, int grid) {
  switch (which) {
    case 0: return o.t_block;
    case 1: return o.t_grid;
    case 2: return o.k_pull;
    case 3: return o.alpha;
    case 4: return o.beta;
    case 6: return o.expand_mode;
    case 7: return o.small_path;
    case 8: return o.colour_mode;
    default: return o.grid_blocks <= 0 ? 1.0 : (double)o.grid_blocks / grid;
  }
}

// Runs `run(o)` (one asynchronous run on c's stream) reps times after one
// warm-up; the minimum device time in ms.
template <class Run>
gb_status time_runs(gb_ctx* c, const gb_opts& o, int reps, Run run, double* ms) {
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return GB_ERR_CUDA;
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return GB_ERR_CUDA;
  }
  gb_status s = run(o);
  if (s == GB_OK) s = gb_ctx_sync(c);
  double best = 1e30;
  for (int r = 0; r < reps && s == GB_OK; ++r) {
    cudaEventRecord(e0, c->stream);
    s = run(o);
    cudaEventRecord(e1, c->stream);
    if (s == GB_OK) s = gb_ctx_sync(c);
    float x = 0.f;
    if (s == GB_OK && cudaEventElapsedTime(&x, e0, e1) == cudaSuccess) best = std::min(best, (double)x);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms = best;
  return s;
}

template <class Run>
gb_status tune(gb_ctx* c, int reps, Run run, gb_opts* best, double* ms_out) {
  const std::vector<Param> params = {
      {7, {0, 1, 2}},  // the grid, automatic, one thread block (at most 6144 vertices)
      {0, {128, 512, 2048}},
      {1, {8192, 32768, 131072}},
      {2, {1, 2, 4}},
      {3, {5, 15, 50}},
      {4, {10, 25, 100}},
      {5, {0.5, 1.0}},
      {6, {0, 1}},
      {8, {0, 1, 2}},  // colour rounds, signature rounds, by residual size
  };
  gb_opts cur;
  gb_opts_default(&cur);
  double cur_ms = 0.0;
  gb_status s = time_runs(c, cur, reps, run, &cur_ms);
  const double default_ms = cur_ms;
  for (int pass = 0; pass < 2 && s == GB_OK; ++pass) {
    bool moved = false;
    for (const Param& p : params) {
      const double have = get_param(cur, p.which, c->grid);
      for (double v : p.values) {
        if (v == have || s != GB_OK) continue;
        gb_opts o = cur;
        set_param(o, p.which, v, c->grid);
        if (o.t_grid <= o.t_block) continue;
        double ms = 0.0;
        s = time_runs(c, o, reps, run, &ms);
        if (s == GB_OK && ms < cur_ms * 0.98) {
          cur = o;
          cur_ms = ms;
          moved = true;
        }
      }
    }
    if (!moved) break;
  }
  if (s == GB_OK) {
    *best = cur;
    if (ms_out) {
      ms_out[0] = cur_ms;
      ms_out[1] = default_ms;
    }
  }
  return s;
}

}  // namespace

extern "C" {

gb_status gb_tune(gb_ctx* c, const gb_graph* g, int32_t kind, int32_t reps, gb_opts* best,
                  double* ms) {
  if (!c || !g || !best || (kind != 0 && kind != 1) || reps < 1) return GB_ERR_INVALID;
  if (cudaSetDevice(c->device) != cudaSuccess) return GB_ERR_CUDA;
  int32_t* labels = nullptr;
  if (cudaMalloc(&labels, (size_t)(g->n > 0 ? g->n : 1) * 4) != cudaSuccess) return GB_ERR_OOM;
  auto run = [&](const gb_opts& o) {
    return kind == 0 ? gb_scc_async(c, g, labels, &o) : gb_wcc_async(c, g, labels, &o);
  };
  const gb_status s = tune(c, reps, run, best, ms);
  cudaFree(labels);
  return s;
}

gb_status gb_tune_batch(gb_ctx* c, const gb_batch* b, int32_t kind, int32_t reps, gb_opts* best,
                        double* ms) {
  if (!c || !b || !best || (kind != 0 && kind != 1) || reps < 1) return GB_ERR_INVALID;
  if (cudaSetDevice(c->device) != cudaSuccess) return GB_ERR_CUDA;
  int32_t cnt = 0;
  int64_t tn = 0, tm = 0;
  gb_status s = gb_batch_info(b, &cnt, &tn, &tm);
  if (s != GB_OK) return s;
  int32_t* labels = nullptr;
  if (cudaMalloc(&labels, (size_t)(tn > 0 ? tn : 1) * 4) != cudaSuccess) return GB_ERR_OOM;
  auto run = [&](const gb_opts& o) {
    return gb::batch_run(c, b, kind == 0 ? gb::kSCC : gb::kWCC, labels, &o, nullptr, false);
  };
  s = tune(c, reps, run, best, ms);
  cudaFree(labels);
  return s;
}

}  // extern "C"
