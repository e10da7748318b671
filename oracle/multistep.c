/*
 * oracle/multistep.c -- CPU restatement of the Multistep connectivity
 * pipeline (HPCGraphAnalysis/Connectivity, multistep/).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU path and the
 * timed CPU baseline ("port"); the product never links or calls it.  Only the
 * tests, the smoke check and the CPU-baseline leg of the benchmark load it.
 *
 * Parity is pinned two ways: (1) against the reference's own golden vector
 * (multistep/test.graph: SCC {0,1},{2}; CC one component), and (2) against
 * the unmodified reference compiled from its sources by oracle/build_ref.sh,
 * whose outputs on seeded graphs are committed as fixtures in tests/golden/.
 *
 * The phases follow the reference step by step (OpenMP threads with
 * per-thread staging queues, direction-optimising BFS with the same switch
 * rule and constants, max-colour propagation, serial Tarjan below the vertex
 * cutoff).  Differences, none of which change the component partition:
 *   - offsets are int64 (the reference uses 32-bit unsigned);
 *   - "visited" flags are claimed with an atomic exchange, so a vertex is
 *     queued at most once (the reference's plain stores can queue a vertex
 *     twice; scc_fwbw.cpp:97-100);
 *   - Tarjan is iterative instead of recursive (scc_serial.cpp:216-258);
 *   - cc's update_valid scans num_valid entries (cc_bfs.cpp:231 scans g.n
 *     entries of a num_valid-long list, an out-of-bounds read);
 *   - a graph whose every degree product is zero has no pivot: FW-BW is
 *     skipped instead of starting from an uninitialised vertex
 *     (scc_main.cpp:177-181, :334).
 * Labels are the reference's kind (trim: self; FW-BW: pivot; colour: colour
 * root; Tarjan: DFS root).  orc_canonicalize maps each to the component's
 * minimum vertex id, which is what every comparison uses.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#include <omp.h>

#define ORC_TQ 2048      /* per-thread queue, THREAD_QUEUE_SIZE scc_main.cpp:63 */
#define ORC_ALPHA 15.0   /* scc_main.cpp:64 */
#define ORC_BETA 25      /* scc_main.cpp:65 */

typedef struct orc_graph {
  int32_t n;
  int64_t m;
  const int64_t* out_off;
  const int32_t* out_adj;
  const int64_t* in_off;   /* NULL for the symmetric graph used by CC */
  const int32_t* in_adj;
} orc_graph;

typedef struct orc_times {
  double trim, fwbw, colour, serial, total;
  int64_t num_trim, num_fwbw, num_colour_sccs, num_serial_sccs;
  int32_t pivot, colour_rounds;
} orc_times;

static double now_s(void) { return omp_get_wtime(); }

/* ---- per-thread staging queue (the reference's thread_queue pattern,
 *      e.g. scc_trim.cpp:97-133) ---- */
typedef struct tq { int len; int32_t buf[ORC_TQ]; } tq;

static inline void tq_flush(tq* t, int32_t* dst, int64_t* shared_len) {
  if (t->len == 0) return;
  int64_t at = __atomic_fetch_add(shared_len, (int64_t)t->len, __ATOMIC_RELAXED);
  memcpy(dst + at, t->buf, (size_t)t->len * sizeof(int32_t));
  t->len = 0;
}
static inline void tq_push(tq* t, int32_t v, int32_t* dst, int64_t* shared_len) {
  t->buf[t->len++] = v;
  if (t->len == ORC_TQ) tq_flush(t, dst, shared_len);
}
static inline int claim8(uint8_t* f, int32_t v) {
  if (__atomic_load_n(&f[v], __ATOMIC_RELAXED)) return 0;
  return __atomic_exchange_n(&f[v], (uint8_t)1, __ATOMIC_RELAXED) == 0;
}
static inline int32_t ld32(const int32_t* p) { return __atomic_load_n(p, __ATOMIC_RELAXED); }
static inline void st32(int32_t* p, int32_t v) { __atomic_store_n(p, v, __ATOMIC_RELAXED); }
static inline uint8_t ld8(const uint8_t* p) { return __atomic_load_n(p, __ATOMIC_RELAXED); }
static inline void st8(uint8_t* p, uint8_t v) { __atomic_store_n(p, v, __ATOMIC_RELAXED); }

#define DEG(off, v) ((off)[(v) + 1] - (off)[(v)])

/* ------------------------------------------------------------------ */
/* CSR construction: stable counting sort, adjacency in input order.   */
/* create_csr, scc_main.cpp:127-191 (out side :150-156, in side :158-166) */
int orc_build_csr(int32_t n, int64_t m, const int32_t* src, const int32_t* dst,
                  int64_t* off, int32_t* adj) {
  if (n < 0 || m < 0) return 1;
  int64_t* cur = (int64_t*)calloc((size_t)n + 1, sizeof(int64_t));
  if (!cur) return 2;
  for (int64_t i = 0; i < m; ++i) {
    if (src[i] < 0 || src[i] >= n || dst[i] < 0 || dst[i] >= n) { free(cur); return 1; }
    cur[src[i] + 1]++;
  }
  off[0] = 0;
  for (int32_t v = 0; v < n; ++v) off[v + 1] = off[v] + cur[v + 1];
  memcpy(cur, off, (size_t)n * sizeof(int64_t));
  for (int64_t i = 0; i < m; ++i) adj[cur[src[i]]++] = dst[i];
  free(cur);
  return 0;
}

/* Pivot for SCC: lowest id maximising out_degree * in_degree, strictly
 * positive (scc_main.cpp:169-183).  Returns -1 when every product is 0. */
int32_t orc_pivot_scc(const orc_graph* g, double* avg_degree) {
  double best = 0.0, sum = 0.0;
  int32_t piv = -1;
  for (int32_t v = 0; v < g->n; ++v) {
    double d = (double)DEG(g->out_off, v) * (double)DEG(g->in_off, v);
    sum += (double)DEG(g->out_off, v);
    if (d > best) { best = d; piv = v; }
  }
  if (avg_degree) *avg_degree = g->n ? sum / (double)g->n : 0.0;
  return piv;
}

/* Pivot for CC: lowest id of maximum out-degree in the mirrored graph
 * (cc_main.cpp:148-160).  Returns -1 when the graph has no edge. */
int32_t orc_pivot_cc(const orc_graph* g, double* avg_degree) {
  int64_t best = 0;
  double sum = 0.0;
  int32_t piv = -1;
  for (int32_t v = 0; v < g->n; ++v) {
    int64_t d = DEG(g->out_off, v);
    sum += (double)d;
    if (d > best) { best = d; piv = v; }
  }
  if (avg_degree) *avg_degree = g->n ? sum / (double)g->n : 0.0;
  return piv;
}

/* ------------------------------------------------------------------ */
/* Trim.                                                               */

/* No trim (TRIM_LEVEL 0, scc_main.cpp:229-246): every vertex stays valid,
 * the valid list is 0..n-1 and every label starts at -1. */
static int64_t trim_none(const orc_graph* g, uint8_t* valid, int32_t* labels,
                         int32_t* list, int64_t* nlist) {
  for (int32_t v = 0; v < g->n; ++v) {
    valid[v] = 1;
    labels[v] = -1;
    list[v] = v;
  }
  *nlist = g->n;
  return 0;
}

/* One pass: in- or out-degree 0 in the original graph -> own component
 * (scc_trim, scc_trim.cpp:89-139).  Survivors go to list. */
static int64_t trim_once(const orc_graph* g, uint8_t* valid, int32_t* labels,
                         int32_t* list, int64_t* nlist) {
  int64_t len = 0;
#pragma omp parallel
  {
    tq* t = (tq*)malloc(sizeof(tq));
    t->len = 0;
#pragma omp for schedule(guided) nowait
    for (int32_t v = 0; v < g->n; ++v) {
      if (DEG(g->out_off, v) < 1 || DEG(g->in_off, v) < 1) {
        valid[v] = 0;
        labels[v] = v;
      } else {
        valid[v] = 1;
        labels[v] = -1;
        tq_push(t, v, list, &len);
      }
    }
    tq_flush(t, list, &len);
    free(t);
  }
  *nlist = len;
  return (int64_t)g->n - len;
}

/* Fixed point: a vertex with no valid out-neighbour or no valid in-neighbour
 * other than itself is removed, and the neighbours that may lose their last
 * edge are re-examined (scc_trim_complete, scc_trim.cpp:141-297).  The valid
 * list is rebuilt in id order afterwards (scc_main.cpp:258-259). */
static int64_t trim_fixed_point(const orc_graph* g, uint8_t* valid, int32_t* labels,
                                int32_t* list, int64_t* nlist) {
  int32_t n = g->n;
  int32_t* q = (int32_t*)malloc(((size_t)n + 1) * sizeof(int32_t));
  int32_t* qn = (int32_t*)malloc(((size_t)n + 1) * sizeof(int32_t));
  uint8_t* inq = (uint8_t*)calloc((size_t)n + 1, 1);
  int64_t qsize = n, nsize = 0, removed = 0;
  for (int32_t v = 0; v < n; ++v) { valid[v] = 1; labels[v] = -1; q[v] = v; }
  while (qsize) {
    nsize = 0;
#pragma omp parallel reduction(+ : removed)
    {
      tq* t = (tq*)malloc(sizeof(tq));
      t->len = 0;
#pragma omp for schedule(guided) nowait
      for (int64_t i = 0; i < qsize; ++i) {
        int32_t v = q[i];
        st8(&inq[v], 0);
        int has_out = 0, has_in = 0;
        for (int64_t e = g->out_off[v]; e < g->out_off[v + 1]; ++e) {
          int32_t w = g->out_adj[e];
          if (w != v && ld8(&valid[w])) { has_out = 1; break; }
        }
        for (int64_t e = g->in_off[v]; e < g->in_off[v + 1]; ++e) {
          int32_t u = g->in_adj[e];
          if (u != v && ld8(&valid[u])) { has_in = 1; break; }
        }
        if (has_out && has_in) continue;
        ++removed;
        st32(&labels[v], v);
        st8(&valid[v], 0);
        /* the side that still has valid neighbours may lose its last edge */
        const int64_t* off = has_in ? g->in_off : g->out_off;
        const int32_t* adj = has_in ? g->in_adj : g->out_adj;
        if (!has_in && !has_out) continue;
        for (int64_t e = off[v]; e < off[v + 1]; ++e) {
          int32_t u = adj[e];
          if (ld8(&valid[u]) && claim8(inq, u)) tq_push(t, u, qn, &nsize);
        }
      }
      tq_flush(t, qn, &nsize);
      free(t);
    }
    int32_t* tmp = q; q = qn; qn = tmp;
    qsize = nsize;
  }
  int64_t len = 0;
  for (int32_t v = 0; v < n; ++v) if (valid[v]) list[len++] = v;
  *nlist = len;
  free(q); free(qn); free(inq);
  return removed;
}

/* ------------------------------------------------------------------ */
/* Direction-optimising reachability from root.
 * Forward (scc_fwbw_fw, scc_fwbw.cpp:47-227): push over out-edges to allowed,
 * unreached vertices; pull: every candidate scans its in-edges for a reached
 * vertex and stops at the first.  Backward (scc_fwbw_bw, :230-409) is the same
 * with the two adjacencies swapped and "allowed" = forward-reached.  CC's BFS
 * (cc_bfs_search, cc_bfs.cpp:47-214) uses the symmetric out-edges for both.
 * The switch rule and its constants are the reference's (:168-195). */
static int64_t reach(int32_t n, const int64_t* push_off, const int32_t* push_adj,
                     const int64_t* pull_off, const int32_t* pull_adj,
                     const uint8_t* allow, uint8_t* reached,
                     const int32_t* cand, int64_t ncand, int32_t root,
                     double avg_degree) {
  int32_t* q = (int32_t*)malloc(((size_t)ncand + 2) * sizeof(int32_t));
  int32_t* qn = (int32_t*)malloc(((size_t)ncand + 2) * sizeof(int32_t));
  int64_t qsize = 0, nsize = 0, total = 0;
  int pull = 0, switched_back = 0;
  q[qsize++] = root;
  reached[root] = 1;
  while (qsize) {
    nsize = 0;
#pragma omp parallel
    {
      tq* t = (tq*)malloc(sizeof(tq));
      t->len = 0;
      if (!pull) {
#pragma omp for schedule(guided) nowait
        for (int64_t i = 0; i < qsize; ++i) {
          int32_t v = q[i];
          for (int64_t e = push_off[v]; e < push_off[v + 1]; ++e) {
            int32_t w = push_adj[e];
            if (allow[w] && claim8(reached, w)) tq_push(t, w, qn, &nsize);
          }
        }
      } else {
#pragma omp for schedule(guided) nowait
        for (int64_t i = 0; i < ncand; ++i) {
          int32_t v = cand[i];
          if (!allow[v] || ld8(&reached[v])) continue;
          for (int64_t e = pull_off[v]; e < pull_off[v + 1]; ++e) {
            if (ld8(&reached[pull_adj[e]])) {
              if (claim8(reached, v)) tq_push(t, v, qn, &nsize);
              break;
            }
          }
        }
      }
      tq_flush(t, qn, &nsize);
      free(t);
    }
    total += nsize;
    if (!switched_back && !pull) {
      double front = (double)nsize * avg_degree;
      double rest = (double)(n - total) * avg_degree;
      if (rest / ORC_ALPHA < front) pull = 1;
    } else if (!switched_back && (n / ORC_BETA) > nsize) {
      pull = 0;
      switched_back = 1;
    }
    int32_t* tmp = q; q = qn; qn = tmp;
    qsize = nsize;
  }
  free(q); free(qn);
  return total + 1;
}

/* Keep the still-valid vertices of list, in order (update_valid,
 * scc_fwbw.cpp:412-466 / scc_color.cpp:292-337 / cc_bfs.cpp:217-271).
 * Vertices flagged in hit get label and leave the valid set first. */
static void commit_compact(int32_t* list, int64_t* nlist, uint8_t* valid,
                           const uint8_t* hit, int32_t* labels, int32_t label) {
  int64_t k = 0, len = *nlist;
  int32_t* out = (int32_t*)malloc(((size_t)len + 1) * sizeof(int32_t));
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < len; ++i) {
    int32_t v = list[i];
    if (hit && hit[v]) { valid[v] = 0; labels[v] = label; }
  }
  for (int64_t i = 0; i < len; ++i) if (valid[list[i]]) out[k++] = list[i];
  memcpy(list, out, (size_t)k * sizeof(int32_t));
  *nlist = k;
  free(out);
}

/* ------------------------------------------------------------------ */
/* Max-colour propagation over out-edges of valid vertices, to a fixed
 * point (scc_color_propagate scc_color.cpp:47-163; cc_color_propagate
 * cc_color.cpp:47-175 writes straight into the labels).  A writer whose
 * store lost a race re-queues itself, so the fixed point is reached. */
static void colour_propagate(int32_t n, const int64_t* off, const int32_t* adj,
                             const uint8_t* valid, const int32_t* list, int64_t nlist,
                             int32_t* colour) {
  int32_t* q = (int32_t*)malloc(((size_t)n + 1) * sizeof(int32_t));
  int32_t* qn = (int32_t*)malloc(((size_t)n + 1) * sizeof(int32_t));
  uint8_t* inq = (uint8_t*)calloc((size_t)n + 1, 1);
  uint8_t* inqn = (uint8_t*)calloc((size_t)n + 1, 1);
  memcpy(q, list, (size_t)nlist * sizeof(int32_t));
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < nlist; ++i) colour[list[i]] = list[i];
  int64_t qsize = nlist, nsize;
  while (qsize) {
    nsize = 0;
#pragma omp parallel
    {
      tq* t = (tq*)malloc(sizeof(tq));
      t->len = 0;
#pragma omp for schedule(guided) nowait
      for (int64_t i = 0; i < qsize; ++i) {
        int32_t v = q[i];
        st8(&inq[v], 0);
        int32_t c = ld32(&colour[v]);
        int changed = 0;
        for (int64_t e = off[v]; e < off[v + 1]; ++e) {
          int32_t w = adj[e];
          if (valid[w] && c > ld32(&colour[w])) {
            st32(&colour[w], c);
            changed = 1;
            if (claim8(inqn, w)) tq_push(t, w, qn, &nsize);
          }
        }
        if (changed && claim8(inqn, v)) tq_push(t, v, qn, &nsize);
      }
      tq_flush(t, qn, &nsize);
      free(t);
    }
    int32_t* tmp = q; q = qn; qn = tmp;
    uint8_t* tb = inq; inq = inqn; inqn = tb;
    qsize = nsize;
  }
  free(q); free(qn); free(inq); free(inqn);
}

/* One colour round (scc_color loop body, scc_color.cpp:340-373):
 * propagate; every vertex whose colour is its own id is a root
 * (scc_color_get_roots :165-212); a backward search from the roots over
 * same-colour valid vertices collects each root's SCC (scc_color_find_sccs
 * :214-289); the valid list is compacted (update_valid :292-337). */
static int64_t colour_round(const orc_graph* g, uint8_t* valid, int32_t* list,
                            int64_t* nlist, int32_t* labels, int32_t* colour,
                            int32_t* q, int32_t* qn) {
  int64_t len = *nlist;
  colour_propagate(g->n, g->out_off, g->out_adj, valid, list, len, colour);
  int64_t nroots = 0;
#pragma omp parallel
  {
    tq* t = (tq*)malloc(sizeof(tq));
    t->len = 0;
#pragma omp for schedule(guided) nowait
    for (int64_t i = 0; i < len; ++i) {
      int32_t v = list[i];
      if (colour[v] == v) { valid[v] = 0; labels[v] = v; tq_push(t, v, q, &nroots); }
    }
    tq_flush(t, q, &nroots);
    free(t);
  }
  int64_t qsize = nroots, nsize;
  while (qsize) {
    nsize = 0;
#pragma omp parallel
    {
      tq* t = (tq*)malloc(sizeof(tq));
      t->len = 0;
#pragma omp for schedule(guided) nowait
      for (int64_t i = 0; i < qsize; ++i) {
        int32_t v = q[i];
        int32_t c = colour[v];
        for (int64_t e = g->in_off[v]; e < g->in_off[v + 1]; ++e) {
          int32_t u = g->in_adj[e];
          if (colour[u] == c && ld8(&valid[u]) &&
              __atomic_exchange_n(&valid[u], (uint8_t)0, __ATOMIC_RELAXED)) {
            labels[u] = c;
            tq_push(t, u, qn, &nsize);
          }
        }
      }
      tq_flush(t, qn, &nsize);
      free(t);
    }
    int32_t* tmp = q; q = qn; qn = tmp;
    qsize = nsize;
  }
  commit_compact(list, nlist, valid, NULL, labels, 0);
  return nroots;
}

/* Iterative Tarjan over the valid vertices, visited in list order
 * (tarjan::run_valid / scc_serial_valid, scc_serial.cpp:160-258).
 * Each SCC is labelled with the vertex its search entered first. */
static int64_t tarjan_valid(const orc_graph* g, const uint8_t* valid,
                            const int32_t* list, int64_t nlist, int32_t* labels) {
  int32_t n = g->n;
  int32_t* index = (int32_t*)malloc(((size_t)n + 1) * sizeof(int32_t));
  int32_t* low = (int32_t*)malloc(((size_t)n + 1) * sizeof(int32_t));
  uint8_t* on = (uint8_t*)calloc((size_t)n + 1, 1);
  int32_t* stk = (int32_t*)malloc(((size_t)nlist + 1) * sizeof(int32_t));
  int32_t* cs_v = (int32_t*)malloc(((size_t)nlist + 1) * sizeof(int32_t));
  int64_t* cs_e = (int64_t*)malloc(((size_t)nlist + 1) * sizeof(int64_t));
  for (int64_t i = 0; i < nlist; ++i) index[list[i]] = -1;
  int32_t next = 0;
  int64_t sp = 0, count = 0;
  for (int64_t s = 0; s < nlist; ++s) {
    int32_t root = list[s];
    if (index[root] != -1) continue;
    int64_t cp = 0;
    cs_v[cp] = root; cs_e[cp] = g->out_off[root]; ++cp;
    index[root] = low[root] = next++;
    stk[sp++] = root; on[root] = 1;
    while (cp) {
      int32_t v = cs_v[cp - 1];
      int64_t e = cs_e[cp - 1];
      if (e < g->out_off[v + 1]) {
        cs_e[cp - 1] = e + 1;
        int32_t w = g->out_adj[e];
        if (!valid[w]) continue;
        if (index[w] == -1) {
          index[w] = low[w] = next++;
          stk[sp++] = w; on[w] = 1;
          cs_v[cp] = w; cs_e[cp] = g->out_off[w]; ++cp;
        } else if (on[w] && index[w] < low[v]) {
          low[v] = index[w];
        }
        continue;
      }
      --cp;
      if (cp && low[v] < low[cs_v[cp - 1]]) low[cs_v[cp - 1]] = low[v];
      if (low[v] == index[v]) {
        int32_t w;
        do { w = stk[--sp]; on[w] = 0; labels[w] = v; } while (w != v);
        ++count;
      }
    }
  }
  free(index); free(low); free(on); free(stk); free(cs_v); free(cs_e);
  return count;
}

/* ------------------------------------------------------------------ */
/* run_scc (scc_main.cpp:210-317).  trim_level 0 = no trim, 1 = scc_trim
 * (the reference default, TRIM_LEVEL 1 at :61), 2 = scc_trim_complete
 * (the switch at :241-259). */
int orc_scc(const orc_graph* g, int32_t* labels, int32_t pivot, double avg_degree,
            int32_t vert_cutoff, int32_t trim_level, orc_times* tm) {
  int32_t n = g->n;
  double t0 = now_s(), t1;
  orc_times dummy;
  if (!tm) tm = &dummy;
  memset(tm, 0, sizeof(*tm));
  tm->pivot = pivot;
  if (n <= 0) return 0;
  uint8_t* valid = (uint8_t*)malloc((size_t)n);
  int32_t* list = (int32_t*)malloc((size_t)n * sizeof(int32_t));
  int64_t nlist = 0;
  if (!valid || !list) return 2;

  tm->num_trim = trim_level <= 0 ? trim_none(g, valid, labels, list, &nlist)
                 : trim_level >= 2 ? trim_fixed_point(g, valid, labels, list, &nlist)
                                   : trim_once(g, valid, labels, list, &nlist);
  t1 = now_s(); tm->trim = t1 - t0; t0 = t1;

  if (pivot >= 0 && pivot < n && valid[pivot]) {
    uint8_t* fw = (uint8_t*)calloc((size_t)n, 1);
    uint8_t* bw = (uint8_t*)calloc((size_t)n, 1);
    reach(n, g->out_off, g->out_adj, g->in_off, g->in_adj, valid, fw, list, nlist,
          pivot, avg_degree);
    reach(n, g->in_off, g->in_adj, g->out_off, g->out_adj, fw, bw, list, nlist,
          pivot, avg_degree);
    int64_t before = nlist;
    commit_compact(list, &nlist, valid, bw, labels, pivot);
    tm->num_fwbw = before - nlist;
    free(fw); free(bw);
  }
  t1 = now_s(); tm->fwbw = t1 - t0; t0 = t1;

  int32_t* colour = (int32_t*)malloc((size_t)n * sizeof(int32_t));
  int32_t* q = (int32_t*)malloc(((size_t)n + 1) * sizeof(int32_t));
  int32_t* qn = (int32_t*)malloc(((size_t)n + 1) * sizeof(int32_t));
  while (nlist > vert_cutoff) {
    tm->num_colour_sccs += colour_round(g, valid, list, &nlist, labels, colour, q, qn);
    tm->colour_rounds++;
  }
  free(colour); free(q); free(qn);
  t1 = now_s(); tm->colour = t1 - t0; t0 = t1;

  tm->num_serial_sccs = tarjan_valid(g, valid, list, nlist, labels);
  t1 = now_s(); tm->serial = t1 - t0;
  tm->total = tm->trim + tm->fwbw + tm->colour + tm->serial;
  free(valid); free(list);
  return 0;
}

/* run_cc (cc_main.cpp:184-245) on a symmetric (mirrored) out-CSR:
 * cc_trim (cc_trim.cpp:47-97), cc_bfs (cc_bfs.cpp:273-291), cc_color
 * (cc_color.cpp:197-214).  The colour step labels each remaining vertex
 * with the largest id of its component. */
int orc_cc(const orc_graph* g, int32_t* labels, int32_t pivot, double avg_degree,
           orc_times* tm) {
  int32_t n = g->n;
  double t0 = now_s(), t1;
  orc_times dummy;
  if (!tm) tm = &dummy;
  memset(tm, 0, sizeof(*tm));
  tm->pivot = pivot;
  if (n <= 0) return 0;
  uint8_t* valid = (uint8_t*)malloc((size_t)n);
  int32_t* list = (int32_t*)malloc((size_t)n * sizeof(int32_t));
  int64_t nlist = 0;
  {
    int64_t len = 0;
#pragma omp parallel
    {
      tq* t = (tq*)malloc(sizeof(tq));
      t->len = 0;
#pragma omp for nowait
      for (int32_t v = 0; v < n; ++v) {
        if (DEG(g->out_off, v) < 1) { valid[v] = 0; labels[v] = v; }
        else { valid[v] = 1; labels[v] = -1; tq_push(t, v, list, &len); }
      }
      tq_flush(t, list, &len);
      free(t);
    }
    nlist = len;
    tm->num_trim = n - len;
  }
  t1 = now_s(); tm->trim = t1 - t0; t0 = t1;
  if (pivot >= 0 && pivot < n && valid[pivot]) {
    uint8_t* hit = (uint8_t*)calloc((size_t)n, 1);
    reach(n, g->out_off, g->out_adj, g->out_off, g->out_adj, valid, hit, list, nlist,
          pivot, avg_degree);
    int64_t before = nlist;
    commit_compact(list, &nlist, valid, hit, labels, pivot);
    tm->num_fwbw = before - nlist;
    free(hit);
  }
  t1 = now_s(); tm->fwbw = t1 - t0; t0 = t1;
  colour_propagate(n, g->out_off, g->out_adj, valid, list, nlist, labels);
  t1 = now_s(); tm->colour = t1 - t0;
  tm->total = tm->trim + tm->fwbw + tm->colour;
  free(valid); free(list);
  return 0;
}

/* ------------------------------------------------------------------ */
/* Canonical form: every label becomes the minimum vertex id carrying it.
 * Unassigned (-1) stays -1. */
void orc_canonicalize(int32_t n, int32_t* labels) {
  int32_t* rep = (int32_t*)malloc(((size_t)n + 1) * sizeof(int32_t));
  for (int32_t v = 0; v < n; ++v) rep[v] = -1;
  for (int32_t v = 0; v < n; ++v) {
    int32_t l = labels[v];
    if (l >= 0 && l < n && rep[l] < 0) rep[l] = v;  /* ascending v: first is min */
  }
  for (int32_t v = 0; v < n; ++v) {
    int32_t l = labels[v];
    if (l >= 0 && l < n) labels[v] = rep[l];
  }
  free(rep);
}

/* Statistics of scc_verify (scc_verify.cpp:47-77) and cc_verify
 * (cc_verify.cpp:47-74): components, components larger than one, largest,
 * unassigned.  They do not depend on which member names a component. */
void orc_label_stats(int32_t n, const int32_t* labels, int64_t out[4]) {
  int32_t* cnt = (int32_t*)calloc((size_t)n + 1, sizeof(int32_t));
  int64_t comps = 0, nontriv = 0, maxc = 0, unassigned = 0;
  for (int32_t v = 0; v < n; ++v) {
    if (labels[v] >= 0 && labels[v] < n) cnt[labels[v]]++;
    else ++unassigned;
  }
  for (int32_t v = 0; v < n; ++v) {
    if (!cnt[v]) continue;
    ++comps;
    if (cnt[v] > 1) ++nontriv;
    if (cnt[v] > maxc) maxc = cnt[v];
  }
  out[0] = comps; out[1] = nontriv; out[2] = maxc; out[3] = unassigned;
  free(cnt);
}

/* Independent check: iterative Tarjan over the whole graph, serial. */
int orc_scc_tarjan(const orc_graph* g, int32_t* labels) {
  int32_t n = g->n;
  if (n <= 0) return 0;
  uint8_t* valid = (uint8_t*)malloc((size_t)n);
  int32_t* list = (int32_t*)malloc((size_t)n * sizeof(int32_t));
  memset(valid, 1, (size_t)n);
  for (int32_t v = 0; v < n; ++v) list[v] = v;
  tarjan_valid(g, valid, list, n, labels);
  free(valid); free(list);
  return 0;
}

int orc_num_threads(void) { return omp_get_max_threads(); }
void orc_set_threads(int t) { if (t > 0) omp_set_num_threads(t); }
