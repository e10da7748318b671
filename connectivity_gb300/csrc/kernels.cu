// Default run kernels (one FW-BW round), the statistics and batch-label
// kernels, and the host launchers.  The device code of a run is in
// run_device.cuh; the run kernels with the optional features compiled in
// are in kernels_options.cu.
#include "run_device.cuh"

namespace gb {
namespace {

// Counts labels outside [0, n) (0 after a complete run); enqueued when the
// caller asks for statistics.
__global__ void k_count_unassigned(Args A) {
  Work& w = A.w;
  const int32_t n = A.g.n;
  const GraphView& g = A.g;
  const bool scc = A.kind == kSCC;
  int un = 0;
  // push-direction degrees of the reached vertices: SCC forward = out,
  // backward = in; WCC forward = out + in
  unsigned long long mf = 0ull, mb = 0ull;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (long long)gridDim.x * blockDim.x) {
    const int32_t l = w.label[v];
    if (l < 0 || l >= n) ++un;
    const long long dout = g.out.off[v + 1] - g.out.off[v];
    const long long din = g.in.off != nullptr ? g.in.off[v + 1] - g.in.off[v] : 0;
    if ((w.fvis[v >> 5] >> (v & 31)) & 1u) mf += (unsigned long long)(scc ? dout : dout + din);
    if (scc && ((w.bvis[v >> 5] >> (v & 31)) & 1u)) mb += (unsigned long long)din;
  }
  for (int o = 16; o; o >>= 1) un += __shfl_xor_sync(kFull, un, o);
  mf = warp_sum64(mf);
  mb = warp_sum64(mb);
  if (lane_id() == 0) {
    if (un) atomicAdd(&w.ctl->unassigned, un);
    if (mf) atomicAdd(&w.ctl->mvis[0], mf);
    if (mb) atomicAdd(&w.ctl->mvis[1], mb);
  }
}

__global__ void k_localize(int32_t* labels, int32_t n, const int32_t* gid, const int64_t* vbase) {
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (long long)gridDim.x * blockDim.x) {
    const int32_t l = labels[v];
    if (l >= 0) labels[v] = (int32_t)(l - vbase[gid[v]]);
  }
}

}  // namespace

int max_coop_grid(int device) {
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 0;
  int best = run_options_blocks_per_sm();
  const int per[] = {run_blocks_per_sm(k_run<1, false>), run_blocks_per_sm(k_run<2, false>)};
  for (int k : per) best = k < best ? k : best;
  if (best < 1) return 0;
  return best * sms;
}

cudaError_t launch_localize(int32_t* labels, int32_t n, const int32_t* gid, const int64_t* vbase,
                            cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  long long blocks = ((long long)n + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  k_localize<<<(int)blocks, 256, 0, s>>>(labels, n, gid, vbase);
  return cudaGetLastError();
}

cudaError_t launch_run(const GraphView& g, RunKind kind, const RunParams& p, const Work& w,
                       int grid, cudaStream_t stream, cudaEvent_t* ev) {
  Args a{};
  a.g = g;
  a.p = p;
  a.w = w;
  a.kind = kind;
  cudaError_t e;
  if (ev) cudaEventRecord(ev[0], stream);
  // SCC and symmetric graphs walk one CSR per direction; WCC of a directed
  // graph walks the union of both
  if ((p.fwbw_rounds > 1 && g.batch.gid == nullptr) || p.tune.expand_mode != 0)
    e = launch_run_options(g, kind, p, w, grid, stream);
  else
    e = (kind == kSCC || g.in.off == nullptr) ? coop(k_run<1, false>, grid, a, stream)
                                              : coop(k_run<2, false>, grid, a, stream);
  if (e != cudaSuccess) return e;
  if (ev) cudaEventRecord(ev[1], stream);
  if (p.count_unassigned) {
    k_count_unassigned<<<grid, kBlock, 0, stream>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  if (ev) cudaEventRecord(ev[4], stream);
  return cudaSuccess;
}

}  // namespace gb
