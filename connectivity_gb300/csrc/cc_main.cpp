// cc -- drop-in for the reference's `cc` executable
// (HPCGraphAnalysis/Connectivity multistep/cc_main.cpp:247-319).
//
//   cc <graph> [output file]
//
// The reference mirrors every edge it reads (cc_main.cpp:102-118), so on a
// directed edge list it computes weakly connected components and on an
// undirected list (each edge once) connected components.  Here the graph is
// kept as out- and in-CSR and the run walks their union, which is the same
// mirrored graph.  Stdout: "Multistep CC time: %9.6lf" (cc_main.cpp:301)
// then the cc_verify line; the optional file gets one label per line
// (output_cc :167-176).  The graph file is parsed and its CSR built on the
// GPU, outside the timed region; the timed region is the first device run,
// with the allocation of its workspace and the labels' copy back to host
// memory, as the reference times its first run_cc (cc_main.cpp:296-302) with
// the allocations inside it.  Labels are the canonical minimum member ids.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../include/gbconn.h"

static void print_usage(char** argv) {
  std::printf("Usage: %s [graph] [optional: output file]\n", argv[0]);
  std::exit(0);
}

static int fail(const char* what, gb_status s) {
  std::fprintf(stderr, "%s: %s (%s)\n", what, gb_status_string(s), gb_last_error());
  return 1;
}

int main(int argc, char** argv) {
  setbuf(stdout, NULL);
  if (argc < 2) print_usage(argv);
  gb_ctx* ctx = nullptr;
  gb_status s = gb_ctx_create(0, &ctx);
  if (s != GB_OK) return fail("gb_ctx_create", s);
  // read_edge + create_csr: the file is parsed and the CSR built on the device
  gb_graph* g = nullptr;
  if ((s = gb_graph_from_file(ctx, argv[1], &g)) != GB_OK) return fail("read_edge", s);
  int32_t n = 0;
  int64_t m = 0;
  int32_t sym = 0;
  if ((s = gb_graph_info(g, &n, &m, &sym)) != GB_OK) return fail("create_csr", s);
  std::vector<int32_t> maps((size_t)n + 1);
  gb_opts o;
  gb_opts_default(&o);
  const auto t0 = std::chrono::steady_clock::now();
  s = gb_wcc(ctx, g, maps.data(), &o, nullptr);
  const auto t1 = std::chrono::steady_clock::now();
  if (s != GB_OK) return fail("run_cc", s);
  std::printf("Multistep CC time: %9.6lf\n", std::chrono::duration<double>(t1 - t0).count());
  char line[256];
  gb_cc_verify(n, maps.data(), line, sizeof(line), nullptr);
  std::fputs(line, stdout);
  if (argc == 3 && (s = gb_output_labels(argv[2], n, maps.data())) != GB_OK)
    return fail("output_cc", s);
  gb_graph_destroy(g);
  gb_ctx_destroy(ctx);
  return 0;
}
