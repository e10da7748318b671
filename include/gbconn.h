/*
 * gbconn.h -- C ABI of libgbconn, a GB300 (sm_103a) implementation of the
 * Multistep connectivity pipeline (trim, forward/backward reachability from a
 * max in-degree x out-degree pivot, colour propagation, cleanup) for strongly,
 * weakly and plain connected components.
 *
 * It is a drop-in for the OpenMP Multistep code of HPCGraphAnalysis/
 * Connectivity (multistep/).  That code has no library API: its surface is
 * the two executables and the functions inside their translation units.  Each
 * entry point below names the reference function it replaces (path:line in
 * that project).
 *
 * Conventions
 *   - Every function returns a gb_status; nothing calls exit().  The reference
 *     has no error reporting (bad ids, missing files and zero-edge graphs are
 *     undefined behaviour there); here they are GB_ERR_INVALID / GB_ERR_IO.
 *   - Vertex ids are int32 in [0, n); edge counts and offsets are int64.
 *   - Label arrays hold n int32 and are owned by the caller.  They may be host
 *     or device (cudaMalloc) memory; the library detects which.
 *   - Labels come back in canonical form by default: every vertex is labelled
 *     with the smallest vertex id of its component.  The reference labels a
 *     component with whichever member the phase that found it used (trim: the
 *     vertex; FW-BW: the pivot; colour: the largest id; Tarjan: the DFS root,
 *     which depends on thread timing); the partition is the same, and the
 *     verify lines, which only count, are byte-identical.
 *   - A gb_ctx owns one CUDA stream and the device workspace; calls on one
 *     context are serialised by the caller, calls on different contexts may
 *     run concurrently.  No CPU fallback exists: without a usable GB300 the
 *     compute calls return GB_ERR_NO_DEVICE or GB_ERR_CUDA.
 */
#ifndef GBCONN_H
#define GBCONN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t gb_status;
#define GB_OK 0
#define GB_ERR_INVALID 1     /* bad argument: null pointer, negative size, id out of range */
#define GB_ERR_CUDA 2        /* a CUDA runtime call failed */
#define GB_ERR_OOM 3         /* a device or pinned allocation failed */
#define GB_ERR_TIMEOUT 4     /* a device-side wait or a kernel hit its time limit */
#define GB_ERR_ITER_LIMIT 5  /* a fixed-point loop hit its step cap */
#define GB_ERR_IO 6          /* a file could not be opened, read, parsed or written */
#define GB_ERR_NO_DEVICE 7   /* no CUDA device */
#define GB_ERR_UNSUPPORTED 8 /* device is not sm_103 or lacks cooperative launch */
#define GB_ERR_CAPACITY 9    /* a size exceeds a fixed maximum */

/* Human-readable name of a status, and the detail of the last failure on
 * the calling thread. */
const char* gb_status_string(gb_status s);
const char* gb_last_error(void);

typedef struct gb_ctx gb_ctx;     /* stream + device workspace */
typedef struct gb_graph gb_graph; /* device-resident out- and in-CSR */

/* Run options.  gb_opts_default fills the defaults noted per field. */
typedef struct gb_opts {
  int32_t trim_level;  /* 0: no trim (TRIM_LEVEL 0, multistep/scc_main.cpp:
                          241-246); 1: one pass (reference default,
                          TRIM_LEVEL 1 at scc_main.cpp:61, scc_trim.cpp:
                          89-139); 2: iterate to the fixed point
                          (scc_trim_complete, scc_trim.cpp:141-297).
                          Default 1. SCC only. */
  int32_t canonical;   /* 1: minimum-member labels (default); 0: labels as
                          the phases produce them */
  int32_t pivot;       /* -1 (default): the reference rule, lowest id of
                          maximum out*in (SCC) or degree (WCC); >= 0: that
                          vertex, if it survives trim */
  int32_t vert_cutoff; /* accepted for run_scc parity (scc_main.cpp:336);
                          the device colours every remaining vertex */
  int32_t t_block;     /* degree from which a block expands one vertex (512) */
  int32_t t_grid;      /* degree from which all blocks share one vertex (32768) */
  int32_t k_pull;      /* in-edges one thread scans in a pull step before the
                          candidate moves to a warp (1..4, default 4) */
  float alpha;         /* push -> pull when frontier edges * alpha > unvisited
                          edges (15, the reference's ALPHA scc_main.cpp:64) */
  float beta;          /* pull -> push when frontier * beta < candidates
                          (25, the reference's BETA scc_main.cpp:65) */
  int32_t max_steps;   /* cap on device steps per phase (1 << 30) */
  int32_t grid_blocks; /* 0: all resident blocks; else a smaller grid */
  int32_t trim_pairs;  /* 1: after the trim, remove size-2 SCCs (two vertices
                          that are each other's only in-neighbour, or only
                          out-neighbour, among the valid vertices), labelled
                          with the smaller id.  No reference counterpart;
                          default 0.  SCC only. */
  int32_t fwbw_rounds; /* FW-BW rounds before the colour rounds, each from a
                          new pivot chosen by the same rule among the
                          vertices still valid (1: the reference's single
                          round, scc_main.cpp:273-276, the default).  A round
                          is skipped once fewer than 4096 vertices are left.
                          Ignored by batches. */
  int32_t expand_mode; /* push steps of the searches: 0 (default) degree
                          tiers (warp / block / grid slice, t_block and
                          t_grid); 1 global edge balance: the frontier's
                          edges split evenly over all warps, the scheme of
                          the Kokkos variant's manhattan-global FW-BW
                          (kokkos_scc/fwbw_manhattan_global.cpp:186-289).
                          An autotuner candidate. */
  int32_t small_path;  /* graphs of at most 6144 vertices can run in one
                          thread block with all their per-vertex state in
                          shared memory (trim to the fixed point, FW-BW,
                          colour rounds; WCC by union-find), with no
                          cooperative grid.  1 (default): for a device graph
                          of at most 65536 edges, and for every such edge
                          list (gb_scc_edges, served requests); 2: whenever
                          the graph fits; 0: never.  Needs canonical = 1;
                          the statistics then hold the times only.  No
                          reference counterpart. */
  int32_t colour_mode; /* SCC after FW-BW: 0 the reference's colour rounds
                          (scc_color.cpp:340-373); 1 signature rounds: every
                          round propagates the smallest reaching id and the
                          smallest reached id inside classes of vertices
                          whose pair matched the round before, labels the
                          vertices whose two ids agree, and never follows an
                          edge between classes again; 2 (default) signature
                          rounds when at least 1048576 vertices are left after
                          FW-BW, else up to four colour rounds and signature
                          rounds for what they leave.  Same labels. */
  int32_t wcc_mode;    /* WCC / CC of a device graph: 0 (default) the
                          reference's phases (trim, BFS from the pivot,
                          colour propagation, cc_main.cpp:184-245); 1 sampled
                          union-find (every vertex links its first
                          neighbour per list, then only the vertices outside
                          the sampled largest component link the rest; the
                          published Afforest scheme), which gb_run_cc uses on
                          a CSR in host memory.  Same labels.  Batches and
                          graphs on the one-block path ignore it. */
} gb_opts;

void gb_opts_default(gb_opts* o);

/* sizeof(gb_opts), sizeof(gb_stats) and sizeof(gb_server_stats) as this
 * library was built, into sizes[0..2]: bindings that mirror the structs
 * (ctypes, cgo) check their layouts against it.  No device is needed. */
void gb_struct_sizes(int64_t sizes[3]);

/* Per-run results.  Times are in milliseconds: trim, reach and colour from
 * the device clock at the run kernel's phase boundaries; canon (the
 * statistics pass) and total from CUDA events on the context stream. */
typedef struct gb_stats {
  double ms_trim, ms_reach, ms_colour, ms_canon, ms_total;
  int32_t pivot;          /* FW-BW source, -1 if none */
  int32_t colour_rounds;
  int64_t n_trim;         /* vertices labelled by trim */
  int64_t n_visit_fw;     /* vertices reached forward from the pivot */
  int64_t n_fwbw;         /* vertices labelled by FW-BW */
  int64_t unassigned;     /* labels < 0 after the run (0 when correct) */
  int64_t vtx_reads;      /* vertex offset records read (8 B x 2 each) */
  int64_t edge_reads;     /* adjacency entries read (4 B each) */
  int64_t list_rw;        /* list entries read or written (4 B each) */
  /* algorithmic bytes moved by each kernel (trim, reach, colour, canon):
   * offset records x 16 + adjacency x 4 + list entries x 4 + the per-vertex
   * arrays and bitmaps each kernel must read or write once */
  int64_t bytes_trim, bytes_reach, bytes_colour, bytes_canon;
  int64_t trim_steps, fw_steps, bw_steps, pull_steps, colour_steps, mark_steps;
  int32_t grid_blocks;
  int32_t err_where;      /* device location code of a failure, 0 if none */
  /* push-direction edges of the vertices reached forward / backward (the
   * m_visited of a traversal) and adjacency entries scanned by pull steps */
  int64_t m_visit_fw, m_visit_bw, pull_edges;
  int64_t fwbw_rounds;    /* FW-BW rounds run (0 when there was no pivot) */
} gb_stats;

/* ---- contexts --------------------------------------------------------- */
/* A context owns a stream, its control block and event ring on `device`.
 * It raises the release threshold of the device's default memory pool
 * (cudaDeviceGetDefaultMemPool) to at least 4 GB, process-wide, so that
 * memory freed with cudaFreeAsync stays reserved for the next call instead
 * of going back to the driver at every synchronise; a larger threshold set
 * before is left as it is.  A host that wants its own threshold sets it
 * after creating its contexts. */
gb_status gb_ctx_create(int device, gb_ctx** ctx);
gb_status gb_ctx_destroy(gb_ctx* ctx);
/* Use an existing cudaStream_t (e.g. a framework's current stream) for all
 * work of this context; NULL restores the context's own stream. */
gb_status gb_ctx_set_stream(gb_ctx* ctx, void* cuda_stream);
void* gb_ctx_stream(gb_ctx* ctx);
/* Wait for all work queued on the context; returns the first device error
 * raised by any run since the last wait. */
gb_status gb_ctx_sync(gb_ctx* ctx);
/* Device times of the last `count` runs (count <= 64), oldest first, five
 * values per run in milliseconds: trim, reach, colour (device clock at the
 * run kernel's phase boundaries), the statistics pass, and the run's total
 * (CUDA events).  Waits for the context's stream.  Lets a caller time every
 * phase of a run of asynchronous calls. */
gb_status gb_ctx_phase_times(gb_ctx* ctx, int32_t count, double* ms);
/* Options per size class for the runs of this context that are given no
 * options (opts NULL in gb_scc, gb_wcc, the batch runs, gb_scc_edges, and the
 * merged runs of a server whose options were not set): entry i applies to a
 * graph (or batch union, or merged set) of at most n_max[i] vertices; the
 * last entry also covers larger ones.  n_max rises.  count 0 removes the
 * table.  A table comes from the autotuner run over seeded graphs of each
 * class (connectivity_gb300/tune.py writes one).  No reference counterpart:
 * the reference's switch constants are fixed (scc_main.cpp:64-65). */
gb_status gb_ctx_set_class_opts(gb_ctx* ctx, int32_t count, const int64_t* n_max,
                                const gb_opts* opts);
/* Diagnostic: the step trace of the context's last completed run (its last
 * 128 records), oldest first: device time (ns) at the start of each step,
 * the step's input count, and a mode.  Reachability steps: bit 0 pull step,
 * bit 1 heavy vertices pending, bit 2 backward search.  Colour steps: 8
 * colours reset, 9 propagation, 10 roots, 11 same-colour marking, 12
 * compaction; 15 end of a phase.  Trim: 16 start, 17 degree pass done, 18
 * list counted, 19 list written.  Writes up to cap entries and returns how
 * many were written (0 on error). */
int32_t gb_ctx_reach_trace(gb_ctx* ctx, int64_t* t_ns, int32_t* count, int32_t* mode, int32_t cap);
/* As gb_ctx_reach_trace, plus three values per step in extra (3 x cap):
 * for pull steps, ns from the step's start to the end of its thread tier,
 * and the lengths of its warp- and block-tier candidate lists. */
int32_t gb_ctx_reach_trace2(gb_ctx* ctx, int64_t* t_ns, int32_t* count, int32_t* mode,
                            int64_t* extra, int32_t cap);
/* Diagnostic: device time (ns) at which each block of the last completed run
 * finished the thread tier of its first pull step (0 for blocks that did
 * not run one).  Returns the number of entries written (<= 256). */
int32_t gb_ctx_block_times(gb_ctx* ctx, int64_t* t_ns, int32_t cap);

/* ---- graphs: create_csr (multistep/scc_main.cpp:127-191) --------------- */
/* Device CSR build from an edge list (host or device arrays, m entries
 * each): out- and in-CSR by stable radix sort on the device, adjacency in
 * input order within a vertex as in the reference's counting sort. */
gb_status gb_graph_from_edges(gb_ctx* ctx, int32_t n, int64_t m, const int32_t* src,
                              const int32_t* dst, gb_graph** g);
/* From CSR arrays (host or device).  in_off/in_adj may be NULL for a
 * symmetric graph (the mirrored CSR that cc builds, cc_main.cpp:123-165);
 * such a graph supports gb_wcc only. */
gb_status gb_graph_from_csr(gb_ctx* ctx, int32_t n, int64_t m, const int64_t* out_off,
                            const int32_t* out_adj, const int64_t* in_off,
                            const int32_t* in_adj, gb_graph** g);
/* From the reference's own CSR layout (graph struct, scc_main.cpp:75-86):
 * 32-bit unsigned offsets out_degree_list[n+1] / in_degree_list[n+1].
 * in_* may be NULL (symmetric graph of cc_main.cpp:72-79).  in_array NULL
 * with in_degree_list given (m < 2^31): the in-lists are written on the
 * device from the out-CSR while it is read (only the out-CSR and the
 * in-offsets cross the host link); their order within a vertex is then not
 * the caller's, and in-offsets that are not those of the out-CSR's
 * transpose give GB_ERR_INVALID. */
gb_status gb_graph_from_csr32(gb_ctx* ctx, int32_t n, uint32_t m, const int32_t* out_array,
                              const uint32_t* out_degree_list, const int32_t* in_array,
                              const uint32_t* in_degree_list, gb_graph** g);
/* From a graph file, parsed on the device (read_edge, scc_main.cpp:94-125,
 * replaced).  Text: the reference's format, "n m" then m lines "src dst"
 * (any blanks between tokens; tokens after the first 2m ignored).  Binary:
 * "GBEDGES1", int64 n, int64 m, m int32 sources, m int32 targets (little
 * endian; see gb_write_binary).  GB_ERR_IO: unreadable file, bad header or
 * too few edges; GB_ERR_INVALID: a token that is not an id in [0, n). */
gb_status gb_graph_from_file(gb_ctx* ctx, const char* path, gb_graph** g);
/* As gb_graph_from_file with the text tokenizer's byte chunk per thread
 * (0: default 256); small chunks exist to test tokens across chunks. */
gb_status gb_graph_from_file2(gb_ctx* ctx, const char* path, int32_t chunk, gb_graph** g);
/* Writes an edge list in the reference's text format ("n m" then "src dst"
 * lines), the input of read_edge. */
gb_status gb_write_text(const char* path, int32_t n, int64_t m, const int32_t* src,
                        const int32_t* dst);
/* Writes an edge list in the binary graph-file format. */
gb_status gb_write_binary(const char* path, int32_t n, int64_t m, const int32_t* src,
                          const int32_t* dst);
/* Seeded directed R-MAT graph built on the device: edge_factor << scale
 * edges drawn with probabilities (a, b, c, 1-a-b-c), self-loops and
 * duplicates removed.  Same edges as gb_rmat_edges_host. */
gb_status gb_graph_rmat(gb_ctx* ctx, int32_t scale, int32_t edge_factor, uint64_t seed, double a,
                        double b, double c, gb_graph** g);
/* R-MAT graph on any n: edge_factor * n candidate edges at scale
 * ceil(log2 n), ids >= n dropped (the batch rule).  Same edges as
 * gb_rmat_edges_host_n. */
gb_status gb_graph_rmat_n(gb_ctx* ctx, int32_t n, int32_t edge_factor, uint64_t seed, double a,
                          double b, double c, gb_graph** g);
gb_status gb_graph_info(const gb_graph* g, int32_t* n, int64_t* m, int32_t* symmetric);
/* Copies the CSR to host arrays (n+1 offsets, m entries; in_* ignored when
 * NULL). */
gb_status gb_graph_csr_to_host(const gb_graph* g, int64_t* out_off, int32_t* out_adj,
                               int64_t* in_off, int32_t* in_adj);
/* Device pointers of the CSR arrays (in_* NULL for a symmetric graph). */
gb_status gb_graph_device_csr(const gb_graph* g, const int64_t** out_off,
                              const int32_t** out_adj, const int64_t** in_off,
                              const int32_t** in_adj);
/* The reference's pivot and average degree: kind 0 = SCC rule
 * (scc_main.cpp:169-183), kind 1 = cc rule on the mirrored graph
 * (cc_main.cpp:148-160).  *pivot = -1 when no vertex qualifies. */
gb_status gb_graph_pivot(gb_ctx* ctx, const gb_graph* g, int32_t kind, int32_t* pivot,
                         double* avg_degree);
gb_status gb_graph_destroy(gb_graph* g);
/* Pull hints: per vertex and direction, the neighbour of largest total
 * degree, counted exactly below 32 and above it in eight steps per power of
 * two (first in adjacency order on ties), an index derived from the CSR
 * that lets a pull step settle most candidates with one lookup.  Every
 * gb_graph_from_* / gb_graph_rmat* call builds them (n int32 per direction);
 * on = 0 frees them and runs then scan in-edges only, on = 1 (re)builds
 * them.  Labels do not depend on them.  No reference counterpart: the
 * reference's create_csr (scc_main.cpp:127-191) computes the pivot and the
 * average degree only, and its pull step (scc_fwbw.cpp:116-149) scans
 * in-edges.  Waits for the context's queued work first. */
gb_status gb_graph_set_hints(gb_ctx* ctx, gb_graph* g, int32_t on);
gb_status gb_graph_has_hints(const gb_graph* g, int32_t* on);
/* Copies the hints to host arrays of n entries (hint_in ignored when NULL or
 * for a symmetric graph); GB_ERR_INVALID when the graph has none. */
gb_status gb_graph_hints_to_host(const gb_graph* g, int32_t* hint_out, int32_t* hint_in);

/* ---- runs ------------------------------------------------------------- */
/* run_scc (multistep/scc_main.cpp:210-317): trim, FW-BW from the pivot,
 * colour rounds until every vertex is labelled. */
gb_status gb_scc(gb_ctx* ctx, const gb_graph* g, int32_t* labels, const gb_opts* opts,
                 gb_stats* stats);
/* run_cc (multistep/cc_main.cpp:184-245) on the mirrored graph: weakly
 * connected components of a directed graph, or connected components of an
 * undirected graph given as a symmetric CSR or as an edge list with each
 * edge once (cc mirrors it, cc_main.cpp:102-118). */
gb_status gb_wcc(gb_ctx* ctx, const gb_graph* g, int32_t* labels, const gb_opts* opts,
                 gb_stats* stats);
gb_status gb_cc(gb_ctx* ctx, const gb_graph* g, int32_t* labels, const gb_opts* opts,
                gb_stats* stats);
/* From an edge list to labels in one call (read_edge's arrays, scc_main.cpp:
 * 94-125, straight into run_scc / run_cc, scc_main.cpp:210 and cc_main.cpp:
 * 184): src / dst hold m ids in [0, n) (host or device memory), labels n
 * entries (host or device).  A graph of at most 6144 vertices (small_path,
 * the default) runs in one thread block that builds its own CSR in shared
 * memory and scratch from the stream-ordered pool: one launch, no radix
 * sort.  Larger graphs are built as a device graph, run and freed.  Waits
 * for the result.  GB_ERR_INVALID: an id outside [0, n). */
gb_status gb_scc_edges(gb_ctx* ctx, int32_t n, int64_t m, const int32_t* src, const int32_t* dst,
                       int32_t* labels, const gb_opts* opts);
gb_status gb_wcc_edges(gb_ctx* ctx, int32_t n, int64_t m, const int32_t* src, const int32_t* dst,
                       int32_t* labels, const gb_opts* opts);
/* As gb_scc / gb_wcc but without waiting: labels must be device memory; the
 * status is collected by gb_ctx_sync. */
gb_status gb_scc_async(gb_ctx* ctx, const gb_graph* g, int32_t* labels_dev, const gb_opts* opts);
gb_status gb_wcc_async(gb_ctx* ctx, const gb_graph* g, int32_t* labels_dev, const gb_opts* opts);

/* SCC labels without any device allocation.  No counterpart in the
 * reference.  For callers that may not call cudaMalloc (code inside a
 * framework's memory pool, plug-ins whose host process has reserved or capped
 * device memory, loops that cannot take an allocation's latency or failure):
 * the run's scratch is a fixed static device array inside the library (about
 * 17 MB, held by every GPU that loads the library until exit).  The CSR
 * (out_off/in_off n+1 entries, out_adj/in_adj m entries) and labels (n
 * entries, canonical minimum member ids) are device memory owned by the
 * caller; the work goes on `stream` (NULL: the legacy default stream) and
 * the call returns after it completes.  At most 262144 vertices (more:
 * GB_ERR_CAPACITY, nothing queued).  The five arrays must be device memory
 * of the current device, and the CSR is checked on the device before the run
 * (off[0] = 0, off[n] = m, offsets non-decreasing, ids in [0, n)); a failure
 * of either is GB_ERR_INVALID and nothing runs on the arrays.  All calls
 * share the scratch: calls that overlap on the GPU race and must be
 * serialised.  The first call on a device sets that device up (symbol
 * address, kernel attributes); make it before any stream capture.  With
 * stream NULL the work goes on the legacy default stream, which waits for
 * and holds up the device's blocking streams: a caller whose other threads
 * capture CUDA graphs passes a non-blocking stream of its own. */
gb_status gb_scc_noalloc(int32_t n, int64_t m, const int64_t* out_off, const int32_t* out_adj,
                         const int64_t* in_off, const int32_t* in_adj, int32_t* labels,
                         void* stream);

/* ---- batches: many independent graphs per run ------------------------- */
/* No counterpart in the reference, whose equivalent is a loop of run_scc /
 * run_cc (multistep/scc_main.cpp:210, cc_main.cpp:184) per graph.  A batch
 * is one disjoint union: graph g owns vertices [vbase[g], vbase[g+1]) and its
 * edges use those global ids.  A run advances every graph in the same
 * kernels (each phase one cooperative launch), with each graph's pivot chosen
 * by the reference rule within the graph, and returns labels local to each
 * graph (its smallest member's local id), identical to running the graph
 * alone. */
typedef struct gb_batch gb_batch;
/* From a concatenated edge list (host or device, m entries, global ids);
 * vbase has count + 1 entries starting at 0.  An edge that joins two graphs
 * is rejected (GB_ERR_INVALID). */
gb_status gb_batch_from_edges(gb_ctx* ctx, int32_t count, const int64_t* vbase, int64_t m,
                              const int32_t* src, const int32_t* dst, gb_batch** b);
/* count seeded R-MAT graphs built on the device: graph g has n[g] vertices,
 * edge factor ef[g], seed seeds[g] (the gb_graph_rmat_n rule per graph). */
gb_status gb_batch_rmat(gb_ctx* ctx, int32_t count, const int32_t* n, const int32_t* ef,
                        const uint64_t* seeds, double a, double b, double c, gb_batch** batch);
gb_status gb_batch_info(const gb_batch* b, int32_t* count, int64_t* total_n, int64_t* total_m);
gb_status gb_batch_vbase(const gb_batch* b, int64_t* vbase);
/* The union as a graph (owned by the batch). */
gb_status gb_batch_graph(const gb_batch* b, const gb_graph** g);
/* labels: total_n entries (host or device), local ids per graph. */
gb_status gb_batch_scc(gb_ctx* ctx, const gb_batch* b, int32_t* labels, const gb_opts* opts,
                       gb_stats* stats);
gb_status gb_batch_wcc(gb_ctx* ctx, const gb_batch* b, int32_t* labels, const gb_opts* opts,
                       gb_stats* stats);
gb_status gb_batch_scc_async(gb_ctx* ctx, const gb_batch* b, int32_t* labels_dev,
                             const gb_opts* opts);
gb_status gb_batch_destroy(gb_batch* b);
/* Sharding a batch over devices (one context per device, each running the
 * union of its graphs; graphs are independent, so no data moves between
 * shards until the labels are gathered on the host).  cost[g] is graph g's
 * work (vertices + edges is a fair measure); shard_of[g] receives its shard
 * and load[s] (or NULL) each shard's total cost.  Largest cost first, each to
 * the least loaded shard: the heaviest shard is within one graph's cost of
 * the mean, and the plan is deterministic, so every rank of a job computes
 * the same one.  No reference counterpart (the reference runs graphs one
 * after another, multistep/scc_main.cpp:210). */
gb_status gb_shard_plan(int32_t count, const int64_t* cost, int32_t shards, int32_t* shard_of,
                        int64_t* load);

/* ---- autotuner ---------------------------------------------------------- */
/* No counterpart in the reference (its switch constants are fixed,
 * scc_main.cpp:64-65).  Picks the run's tunables for one graph or batch by
 * timing runs on the device: the push-tier degree cutoffs (t_block, t_grid),
 * the pull step's per-thread edge budget (k_pull), the direction-switch
 * factors (alpha, beta) and the number of resident blocks (grid_blocks).
 * Coordinate descent from gb_opts_default over a fixed candidate set, two
 * passes; each time is the minimum of `reps` device-timed runs after one
 * warm-up.  kind 0 = SCC, 1 = WCC.  ms (2 values, or NULL): the best time
 * and the defaults' time.  Labels do not depend on the tunables. */
gb_status gb_tune(gb_ctx* ctx, const gb_graph* g, int32_t kind, int32_t reps, gb_opts* best,
                  double* ms);
gb_status gb_tune_batch(gb_ctx* ctx, const gb_batch* b, int32_t kind, int32_t reps,
                        gb_opts* best, double* ms);

/* ---- serving: a request stream with continuous batching --------------- */
/* No counterpart in the reference, whose equivalent is one run_scc / run_cc
 * call per request (multistep/scc_main.cpp:210, cc_main.cpp:184).  A server
 * owns an engine thread over one context: it admits every request that has
 * arrived and fits the device-memory budget (at most max_graphs per merged
 * run), merges them into one SCC and one WCC batch, and delivers each
 * request's labels -- identical to the graph's own gb_scc / gb_wcc labels --
 * into the caller's host buffer.  The next requests' edges are copied to the
 * device while the current merged runs compute.  Graph state comes from the
 * stream-ordered device pool.  While a server runs, its context must not be
 * used by other calls. */
typedef struct gb_server gb_server;
typedef struct gb_server_stats {
  int64_t completed;   /* requests finished */
  int64_t batches;     /* merged runs (an SCC and a WCC part count as one) */
  double mean_batch;   /* requests per merged run */
  double p50_ms;       /* latency = completion - arrival */
  double p99_ms;
  double max_ms;
  double graphs_per_s; /* completed / (last completion - first arrival) */
} gb_server_stats;
/* budget_bytes <= 0: half the device's free memory at creation. */
gb_status gb_server_create(gb_ctx* ctx, int64_t budget_bytes, int32_t max_graphs,
                           gb_server** server);
/* Options of the merged runs (default gb_opts_default); before the start
 * only.  gb_tune_batch on a sample of the expected requests finds them. */
gb_status gb_server_set_opts(gb_server* server, const gb_opts* opts);
/* Starts the engine and the server clock (t = 0). */
gb_status gb_server_start(gb_server* server);
/* kind 0 = SCC, 1 = WCC.  src / dst / labels_out are host arrays that stay
 * valid until the request completes.  arrival_ns: arrival time on the server
 * clock; the engine does not admit the request before it (a negative value
 * means now).  GB_ERR_CAPACITY: the request alone exceeds the budget. */
gb_status gb_server_submit(gb_server* server, int32_t kind, int32_t n, int64_t m,
                           const int32_t* src, const int32_t* dst, int32_t* labels_out,
                           int64_t arrival_ns, int64_t* id);
/* Blocks until request id completes; its status and latency. */
gb_status gb_server_wait(gb_server* server, int64_t id, int64_t* latency_ns);
/* Blocks until every submitted request completes; the first error seen. */
gb_status gb_server_drain(gb_server* server);
gb_status gb_server_stats_get(gb_server* server, gb_server_stats* stats);
/* Finishes the requests in flight, stops the engine and frees everything. */
gb_status gb_server_destroy(gb_server* server);

/* ---- reference-shaped drop-ins (host buffers, reference layout) ------- */
/* How gb_run_scc gets the in-lists.  The in-CSR is the out-CSR transposed
 * (create_csr, scc_main.cpp:127-191, builds both), so half of its lists can
 * be written on the device from the out-lists while they are read, instead
 * of crossing the host link.  share = the fraction of the in-edges (those of
 * the lowest target ids) whose lists are derived so; the rest of in_array
 * is copied beside the derivation.  1: in_array is not read (it may be
 * NULL); 0: in_array is copied whole.  Default 0.8.  Derived lists are
 * checked against in_degree_list (GB_ERR_INVALID when it is not the
 * transpose's), and their order within a vertex is free; the labels are the
 * same for every share.  Graphs of m >= 2^31 copy. */
gb_status gb_dropin_set_derive_share(double share);
/* run_scc(graph& g, int*& scc_maps, int max_deg_vert, double avg_degree,
 * int vert_cutoff), multistep/scc_main.cpp:210-211, with the graph struct's
 * fields passed one by one and scc_maps owned by the caller (n ints).  Uses
 * a library-owned context on the calling thread's current CUDA device
 * (created at the first call) and keeps the graph's device buffers for reuse.  avg_degree is accepted for parity;
 * the direction switch uses exact edge counts. */
gb_status gb_run_scc(int n, unsigned m, const int* out_array, const int* in_array,
                     const unsigned* out_degree_list, const unsigned* in_degree_list,
                     int* scc_maps, int max_deg_vert, double avg_degree, int vert_cutoff);
/* run_cc(graph& g, int*& cc_maps, int max_deg_vert, double avg_degree),
 * multistep/cc_main.cpp:184-185, on the mirrored out-CSR of cc's graph
 * struct (cc_main.cpp:72-79). */
gb_status gb_run_cc(int n, unsigned m, const int* out_array, const unsigned* out_degree_list,
                    int* cc_maps, int max_deg_vert, double avg_degree);

/* ---- host utilities --------------------------------------------------- */
/* read_edge (scc_main.cpp:94-125): "n m" then m lines "src dst".  Returns
 * malloc'd arrays (free with gb_free_host).  Ids are checked against n.  cc's
 * reader mirrors the edges (cc_main.cpp:102-118); here mirroring is done by
 * gb_wcc itself, so one reader serves both. */
gb_status gb_read_edge(const char* path, int32_t* n, int64_t* m, int32_t** srcs, int32_t** dsts);
/* gb_read_edge with the body parsed in `pieces` pieces by OpenMP threads (0:
 * about 1 MB each, the choice gb_read_edge makes).  Every piece count gives
 * the same arrays and the same status as one piece. */
gb_status gb_read_edge_pieces(const char* path, int32_t pieces, int32_t* n, int64_t* m,
                              int32_t** srcs, int32_t** dsts);
void gb_free_host(void* p);
/* output_scc / output_cc (scc_main.cpp:193-202, cc_main.cpp:167-176): one
 * label per line. */
gb_status gb_output_labels(const char* path, int32_t n, const int32_t* labels);
/* scc_verify (multistep/scc_verify.cpp:47-77): writes the exact line
 * "Num SCCs: %d, Nontrivial: %d, Max SCC: %d, Unassigned %d\n" into line
 * (cap bytes) and the four numbers into stats (either may be NULL). */
gb_status gb_scc_verify(int32_t n, const int32_t* labels, char* line, size_t cap,
                        int64_t stats[4]);
/* cc_verify (multistep/cc_verify.cpp:47-74): "Num CCs: %d, Max CC: %d,
 * Unassigned %d\n"; stats = components, largest, unassigned. */
gb_status gb_cc_verify(int32_t n, const int32_t* labels, char* line, size_t cap,
                       int64_t stats[3]);
/* Host relabelling to the minimum member id. */
gb_status gb_canonicalize(int32_t n, int32_t* labels);
/* Seeded generators (host, deterministic across machines).
 * R-MAT: as gb_graph_rmat; the edge arrays (*src, *dst) are malloc'd and sorted by (src, dst). */
gb_status gb_rmat_edges_host(int32_t scale, int32_t edge_factor, uint64_t seed, double a,
                             double b, double c, int64_t* m, int32_t** src, int32_t** dst);
/* R-MAT on any n (the batch rule, see gb_graph_rmat_n). */
gb_status gb_rmat_edges_host_n(int32_t n, int32_t edge_factor, uint64_t seed, double a, double b,
                               double c, int64_t* m, int32_t** src, int32_t** dst);
/* side x side lattice, every lattice edge u->v, v->u, both or none with
 * probability 1/4 each, plus `extra` vertices hung off random lattice
 * vertices in chains of length 1..max_chain (half feeding in from an
 * in-degree-0 head, half draining to an out-degree-0 tail). */
gb_status gb_grid_edges_host(int32_t side, int32_t extra, int32_t max_chain, uint64_t seed,
                             int32_t* n, int64_t* m, int32_t** src, int32_t** dst);
/* Sizes of a batch of graphs: n_i = round(median * exp(sigma * z_i))
 * clipped to [n_min, n_max], z_i standard normal (sum of 12 uniforms - 6),
 * edge factor uniform in [ef_min, ef_max], per-graph seeds. */
gb_status gb_batch_sizes(int32_t count, uint64_t seed, double median, double sigma,
                         int32_t n_min, int32_t n_max, int32_t ef_min, int32_t ef_max,
                         int32_t* n_out, int32_t* ef_out, uint64_t* seed_out);

#ifdef __cplusplus
}
#endif
#endif /* GBCONN_H */
