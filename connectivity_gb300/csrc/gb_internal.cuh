// Internal declarations shared by the CUDA translation units of libgbconn:
// the device control block, tuning parameters, kernel argument structs and
// the host-side launchers.  Nothing here is part of the C ABI.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "gen_common.h"

namespace gb {

constexpr int kBlock = 1024;              // threads per block, cooperative kernels
constexpr int kMinBlocks = 1024 / kBlock; // resident blocks per SM (64 registers)
constexpr int kWarps = kBlock / 32;       // <= 32 (block scans use one warp)
constexpr int kBlkList = 128;             // per-block list of large vertices
constexpr unsigned kFull = 0xffffffffu;

// Error codes written by kernels; equal to the gb_status values of gbconn.h.
enum : int {
  kErrNone = 0,
  kErrInvalid = 1,     // an input id outside [0, n)
  kErrTimeout = 4,     // a grid barrier wait hit its time / spin limit
  kErrIterLimit = 5,   // a fixed-point loop hit its step cap
  kErrCapacity = 9,    // an append would overflow its array
};

struct Csr {
  const int64_t* off;   // n + 1 offsets
  const int32_t* adj;   // neighbour ids
  const int32_t* hint;  // per vertex, the neighbour of largest degree key
                        // (-1: none), or null
};

// Counters filled during one step and read by every block after the
// barrier that ends it.  Three slots rotate: step s reads slot s%3, appends
// into slot (s+1)%3 and clears slot (s+2)%3.
// The step counters take atomics from every warp of the grid, and the
// barrier word is polled by every block: each hot word sits in its own
// 128-byte line, so that no L2 slice serves two of them.
struct Slot {
  alignas(128) int32_t count;     // vertices appended to the step's output list
  alignas(128) int32_t cand;      // candidates kept by a pull step
  alignas(128) int32_t huge;      // heavy vertices deferred to the next step
  int32_t pad;
  unsigned long long edges;       // push-degree sum of the appended vertices
};

// Statistic slots (64-bit counters, summed over the whole run).
enum Stat : int {
  kStTrimSteps = 0,
  kStFwSteps,
  kStBwSteps,
  kStPullSteps,
  kStColourRounds,
  kStColourSteps,
  kStMarkSteps,
  kStNum = 16
};

struct Ctl {
  // grid barrier word: arrivals so far (low 32 bits, never reset within a
  // run), bit 63 = an error was raised
  alignas(128) unsigned long long bar;
  alignas(128) int err;
  int err_where;
  int step;               // step counter, continued by each kernel of a run
  int pad0;
  Slot ring[3][2];        // [step % 3][search]: the forward and backward searches of
                          // one step count separately
  int32_t pivot;          // FW-BW source (-1: none)
  int32_t nvalid;         // length of the current valid list
  int32_t nvisit_fw;      // vertices reached forward
  int32_t nscc_fwbw;      // vertices labelled by FW-BW
  int32_t ntrim;          // vertices labelled by trim
  int32_t ncolour_rounds;
  int32_t unassigned;
  int32_t ncolour;        // vertices labelled by the colour rounds
  int32_t nroots;         // batch: pivots in BatchView::roots
  int32_t rpivot;         // pivot of the FW-BW round after the first (-1: none)
  int32_t nrounds;        // FW-BW rounds after the first
  alignas(128) int32_t minv[2];       // smallest vertex reached forward / backward
  // pull steps, per search and per parity of the search's pull steps:
  alignas(128) int32_t lcount[2][2][2];  // warp- and block-tier list lengths
  alignas(128) long long pnext[2][2];    // next unclaimed candidate of the thread tier
  alignas(128) int32_t pad1;
  unsigned long long m_cand;   // push-degree sum of the valid list after trim
  unsigned long long stat[kStNum];
  // Algorithmic traffic per kernel (trim, reach, colour, canon): vertex
  // offset records read, adjacency entries read, list entries read/written.
  unsigned long long kst[4][3];
  // Per-step trace (last kTrace steps): device time at the start of the
  // step and the step's input count.  Reachability steps: mode bit 0 =
  // pull, bit 1 = heavy vertices pending, bit 2 = backward search.  Colour
  // steps: mode 8 = colours reset, 9 = propagation, 10 = roots,
  // 11 = same-colour marking, 12 = compaction; 15 = end of a kernel.
  // Trim: 16 = start, 17 = degree pass done, 18 = list counted, 19 = list
  // written.
  struct Trace {
    unsigned long long t;
    unsigned long long t_mid;   // pull steps: end of the thread tier
    int32_t count;
    int32_t mode;
    int32_t nwarp;              // pull steps: warp-tier candidates
    int32_t nblock;             // pull steps: block-tier candidates
  } trace[128];
  int32_t ntrace;
  int32_t pad2;
  // statistics runs: push-direction edges of the forward / backward reached
  // vertices, and adjacency entries scanned by pull steps
  unsigned long long mvis[2];
  unsigned long long pull_edges;
  // Diagnostic: device time at which each block finished the thread tier of
  // the first pull step of the run.
  unsigned long long blk_t[256];
};
constexpr int kTrace = 128;
constexpr int kBlkTimes = 256;

enum KernelId : int { kKTrim = 0, kKReach = 1, kKColour = 2, kKCanon = 3 };

struct Tune {
  int32_t t_block;        // degree from which a whole block expands a vertex
  int32_t t_grid;         // degree from which every block takes a slice
  int32_t k_pull;         // in-edges a thread scans before handing a pull
                          // candidate to a warp
  float alpha;            // push -> pull when m_f > m_u / alpha
  float beta;             // pull -> push when n_f < n_cand / beta
  int32_t max_steps;      // cap on barrier steps per kernel
  int32_t expand_mode;    // push steps of the searches: 0 degree tiers,
                          // 1 global edge balance
};

// Device workspace of one run (all arrays sized for n vertices).
struct Work {
  int32_t n;
  int32_t nwords;         // (n + 31) / 32
  int64_t m;
  int32_t* label;
  int32_t* colour;        // colours; canonicalisation reuses it
  int32_t* live_in;
  int32_t* live_out;
  uint32_t* vbits;        // valid (unassigned) vertices
  uint32_t* fvis;         // forward reached
  uint32_t* bvis;         // backward reached
  uint32_t* done;         // labelled in the current colour round
  int32_t* listA;         // valid list
  int32_t* listB;
  int32_t* q;             // traversal visit queue
  int32_t* x0;            // push frontiers
  int32_t* x1;
  int32_t* candA;         // pull candidate lists
  int32_t* candB;
  int32_t* h0;            // heavy-vertex lists
  int32_t* h1;
  int32_t* xa;            // backward search's pull tier lists when both
  int32_t* xb;            // searches run in the same steps
  int32_t* blk_i;         // per-block scratch (2 x grid size: counts, then pivot ids)
  unsigned long long* tphase;  // this run's 4 phase-boundary device times, or null
  long long* blk_l;       // per-block scratch (2 x grid size: pivot keys, then edge sums)
  Ctl* ctl;
};

// A batch of independent graphs stored as one disjoint union: graph g owns
// vertices [vbase[g], vbase[g+1]).  gid == null for a single graph.
struct BatchView {
  const int32_t* gid;          // vertex -> graph
  const int64_t* vbase;        // count + 1 entries
  int32_t count;
  int32_t id_bits;             // pivot keys: (score << id_bits) | (mask - v)
  unsigned long long* pkey;    // per graph pivot key (zeroed per run)
  int32_t* gmin;               // per graph smallest FW-BW member (INT_MAX per run)
  int32_t* roots;              // per run: the pivots of all graphs
};

// One graph (or a batch union) as the kernels see it.  `in` is null for a
// symmetric CSR.
struct GraphView {
  int32_t n;
  int64_t m;
  Csr out;
  Csr in;
  BatchView batch;
};

// Kind of run.
enum RunKind : int { kSCC = 0, kWCC = 1 };

struct RunParams {
  int32_t trim_level;     // 0: none, 1: one pass, 2: fixed point
  int32_t trim_pairs;     // 1: size-2 components leave with the trim
  int32_t fwbw_rounds;    // FW-BW rounds, each from a new pivot (>= 1)
  int32_t canonical;      // 1: relabel with the minimum member id
  int32_t pivot_hint;     // >= 0: use as FW-BW source if still valid
  int32_t count_unassigned;  // 1: a final pass counts labels outside [0, n)
  int32_t colour_mode;    // SCC: 0 colour rounds, 1 signature rounds, 2 the
                          // signature rounds from kSigMin residual vertices
  Tune tune;
};

// Host launchers (kernels.cu).  All enqueue on `stream`; none synchronise.
cudaError_t launch_run(const GraphView& g, RunKind kind, const RunParams& p,
                       const Work& w, int grid, cudaStream_t stream,
                       cudaEvent_t* ev /* 5 events or null */);
int max_coop_grid(int device);   // cooperative grid size for the run kernels
// The run with the optional features compiled in (kernels_options.cu;
// launch_run calls it for fwbw_rounds > 1 on a single graph or for
// expand_mode 1), and the blocks per SM of its kernels.
cudaError_t launch_run_options(const GraphView& g, RunKind kind, const RunParams& p,
                               const Work& w, int grid, cudaStream_t stream);
int run_options_blocks_per_sm();

// CSR construction (csr_build.cu).  build_csr sorts device edge arrays into
// out- and (if in_off != null) in-CSR; *ids_ok = false if an id is outside
// [0, n) (nothing is built then).  Synchronises the stream.
cudaError_t build_csr(int32_t n, int64_t m, const int32_t* d_src, const int32_t* d_dst,
                      int64_t* out_off, int32_t* out_adj, int64_t* in_off, int32_t* in_adj,
                      cudaStream_t s, bool* ids_ok);
// Sets *bad when off[0] != 0, off[n] != m, offsets decrease or an id is
// outside [0, n).  Synchronises the stream.
cudaError_t check_csr(int32_t n, int64_t m, const int64_t* off, const int32_t* adj,
                      cudaStream_t s, int* bad);
// As check_csr, without allocating: ORs 1 into *d_bad (device memory, left
// as it is when the CSR is good) and does not wait.
cudaError_t check_csr_flag(int32_t n, int64_t m, const int64_t* off, const int32_t* adj,
                           int* d_bad, cudaStream_t s);
// Reference pivot: kind 0 = lowest id maximising out*in (> 0), kind 1 =
// lowest id maximising out (+ in when in_off != null).  -1 when none.
// Synchronises the stream.
cudaError_t pivot_device(int32_t n, const int64_t* out_off, const int64_t* in_off, int kind,
                         cudaStream_t s, int32_t* pivot);
// Copies the first device error of a run into sticky[0..1] (code, site)
// unless an earlier one is already there.
cudaError_t launch_latch(Ctl* ctl, int* sticky, cudaStream_t s);

// Small graphs, one thread block per graph (small.cu).  A graph of at most
// kSmallMaxN vertices keeps its per-vertex state in shared memory.
constexpr int32_t kSmallMaxN = 6144;
// edges up to which a device graph takes the one-block path by default (an
// edge list always does: it saves the CSR build)
constexpr int64_t kSmallAutoEdges = 65536;
struct SmallDesc {
  int32_t n;
  int32_t id_base;          // subtracted from every adjacency entry (batch unions)
  int64_t m;
  // CSR form (out_off != null): n + 1 absolute offsets per side, adjacency
  // holding ids id_base .. id_base + n - 1; in_off null = symmetric graph
  const int64_t* out_off;
  const int32_t* out_adj;
  const int64_t* in_off;
  const int32_t* in_adj;
  // edge form (out_off == null): m local ids each; SCC builds its CSR into
  // adj_scratch (2m ints), WCC needs no scratch
  const int32_t* src;
  const int32_t* dst;
  int32_t* adj_scratch;
  int32_t* labels;          // n outputs: smallest member id per component
};
// Dynamic shared memory of a block for graphs of at most max_n vertices.
size_t small_smem_bytes(int32_t max_n);
// kind 0 = SCC, 1 = WCC.  One block per graph: `count` descriptors from
// `many` (device memory), or `one` when many is null (count 1).  A failure
// (an id outside [0, n) in edge form: kErrInvalid; a loop past max_steps:
// kErrIterLimit) is written to *err with atomicCAS from 0.  colour_mode as
// in gb_opts: 0 colour rounds to the end, 1 signature rounds, 2 four colour
// rounds and signature rounds for the rest.
cudaError_t launch_small(int kind, const SmallDesc& one, const SmallDesc* many, int count,
                         int32_t max_n, int32_t max_steps, int* err, cudaStream_t s,
                         int32_t colour_mode = 2);
cudaError_t widen_offsets(const uint32_t* in, int64_t* out, int64_t count, cudaStream_t s);
// Reference-layout CSR (32-bit offsets) from device-readable host memory into
// an int64-offset device CSR, checked on the way (*d_bad |= 1 on a bad CSR).
cudaError_t ingest_csr32(int32_t n, int64_t m, const uint32_t* h_off, const int32_t* h_adj,
                         int64_t* off, int32_t* adj, int* d_bad, cudaStream_t s);
// The same for a directed graph given its out-CSR and its in-offsets: the
// in-lists of the targets below t_split are written on the device while the
// out-lists are read (their order within a list is then not the input's);
// the in-list entries from tail0 on (those of the targets from t_split on)
// are copied from h_in_adj in the same kernel, checked against [0, n), when
// tail0 < m (tail0 == m: the caller fills them).  *d_bad |= 1 on a bad CSR
// or in-offsets that are not those of the out-CSR's transpose (below
// t_split).  The adjacency may be read from out_adj itself (already on the
// device).  m < 2^31, 0 <= t_split <= n.
cudaError_t ingest_csr32_derive_in(int32_t n, int64_t m, const uint32_t* h_out_off,
                                   const int32_t* h_out_adj, const uint32_t* h_in_off,
                                   int64_t* out_off, int32_t* out_adj, int64_t* in_off,
                                   int32_t* in_adj, int32_t t_split, const int32_t* h_in_adj,
                                   int64_t tail0, int* d_bad, cudaStream_t s);
// Connected components of a symmetric 32-bit CSR that the device reads in
// place (host memory it can read, or device memory), by sampled union-find
// that never reads the largest component's lists past their first entry
// (afforest.cu).  labels (device, n) get each component's smallest
// id.  *d_bad |= 1 on a bad CSR; *d_err = kErrIterLimit when a link ran out
// of retries.  m < 2^32 - 16.  Does not wait.
cudaError_t cc_sampled(int32_t n, int64_t m, const uint32_t* h_off, const int32_t* h_adj,
                       int32_t* labels, int* d_bad, int* d_err, cudaStream_t s);
// The same for a device graph: its symmetric CSR (in_off null) or the union
// of its out- and in-lists.
cudaError_t cc_sampled_device(int32_t n, const int64_t* out_off, const int32_t* out_adj,
                              const int64_t* in_off, const int32_t* in_adj, int32_t* labels,
                              int* d_bad, int* d_err, cudaStream_t s);
// *d_bad |= 1 when an id of adj[0, count) is outside [0, n).  Does not wait.
cudaError_t check_ids_flag(int32_t n, const int32_t* adj, int64_t count, int* d_bad,
                           cudaStream_t s);
// Batch labels: global ids -> ids local to each graph.
cudaError_t launch_localize(int32_t* labels, int32_t n, const int32_t* gid, const int64_t* vbase,
                            cudaStream_t s);
// Pull hints: for every vertex, its neighbour of largest degree key (the
// total degree, above 32 rounded down to eight steps per power of two) in
// each CSR of m entries (hint_in may be null when in_off is).  Synchronises
// the stream.
cudaError_t build_hints(int32_t n, int64_t m, const int64_t* out_off, const int32_t* out_adj,
                        const int64_t* in_off, const int32_t* in_adj, int32_t* hint_out,
                        int32_t* hint_in, cudaStream_t s);
// Seeded R-MAT edge list on the device for n vertices: edge_factor * n
// candidate edges at scale ceil(log2 n), ids >= n, self-loops and duplicates
// dropped, sorted by (src, dst); *d_src / *d_dst are cudaMallocAsync'd.
cudaError_t rmat_edges_device(int32_t n, int edge_factor, uint64_t seed, gb_rmat_thr thr,
                              int32_t** d_src, int32_t** d_dst, int64_t* m_out, cudaStream_t s);
// The same for a batch: graph g (h_n[g] vertices, h_ef[g], h_seeds[g]) gets
// global ids from h_vbase[g]; id_bits >= bits of the total vertex count.
cudaError_t batch_edges_device(int32_t count, const int32_t* h_n, const int32_t* h_ef,
                               const uint64_t* h_seeds, gb_rmat_thr thr, int id_bits,
                               const int64_t* h_vbase, int32_t** d_src, int32_t** d_dst,
                               int64_t* m_out, cudaStream_t s);
cudaError_t batch_gid(int32_t n, const int64_t* d_vbase, int32_t count, int32_t* gid,
                      cudaStream_t s);
// Sets *bad if an edge joins two graphs.  Synchronises the stream.
cudaError_t batch_check_within(const int32_t* src, const int32_t* dst, int64_t m,
                               const int32_t* gid, cudaStream_t s, int* bad);
// Largest degree of a CSR.  Synchronises the stream.
cudaError_t max_degree(int32_t n, const int64_t* off, cudaStream_t s, unsigned long long* out);

}  // namespace gb
