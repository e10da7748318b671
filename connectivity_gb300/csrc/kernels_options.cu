// Run kernels with the optional features compiled in (FW-BW rounds after the
// first, the edge-balanced push), in their own translation unit: the default
// run kernels in kernels.cu keep their code whether or not this variant
// exists.
#include "run_device.cuh"

namespace gb {

cudaError_t launch_run_options(const GraphView& g, RunKind kind, const RunParams& p, const Work& w,
                              int grid, cudaStream_t stream) {
  Args a{};
  a.g = g;
  a.p = p;
  a.w = w;
  a.kind = kind;
  return (kind == kSCC || g.in.off == nullptr) ? coop(k_run<1, true>, grid, a, stream)
                                               : coop(k_run<2, true>, grid, a, stream);
}

int run_options_blocks_per_sm() {
  const int a = run_blocks_per_sm(k_run<1, true>), b = run_blocks_per_sm(k_run<2, true>);
  return a < b ? a : b;
}

}  // namespace gb
