// gb_scc_noalloc: the SCC run for callers that cannot allocate device memory.
//
// Some callers may not call cudaMalloc at all: code that runs inside a
// framework's memory pool and must not fragment it, code that runs while a
// CUDA graph is being captured or replayed on another thread, plug-ins whose
// host process has already reserved (or capped) all device memory, and
// real-time loops where an allocation's latency or failure is not acceptable.
// For them this file keeps the whole run's scratch -- labels work arrays,
// bitmaps, lists and the device control block -- in one file-scope device
// array of fixed size, so a call allocates nothing.  The caller passes the
// CSR (inputs) and the label array (output), both already in device memory.
//
// Limits and sharing:
//   - at most kNoAllocMaxVertices vertices; larger graphs are rejected with
//     GB_ERR_CAPACITY before any work is queued;
//   - the array is held by every GPU that loads the library, until exit
//     (about 17 MB);
//   - all calls share the array and it keeps the last call's contents; every
//     call clears what must start at zero.  Calls whose work overlaps on the
//     GPU (two streams, or two host threads) race on it: serialise them.
//   - the first call on a device sets that device up (cudaGetSymbolAddress of
//     the array, the kernels' shared-memory attribute and cooperative grid
//     size); make that first call before any stream capture.
//   - the CSR is checked on the device before the run (offsets from 0 to m,
//     non-decreasing; ids in [0, n)), with the check's flag in the same
//     array, and every pointer must be device memory of the current device:
//     a bad CSR or a host pointer is GB_ERR_INVALID, and nothing runs on it.
//   - with stream NULL (the legacy default stream) the call's work waits for,
//     and holds up, the blocking streams of the device; a caller whose other
//     threads capture CUDA graphs passes a non-blocking stream of its own.
#include <cstdint>
#include <cstdio>
#include <mutex>

#include "../../include/gbconn.h"
#include "gb_internal.cuh"
#include "host_internal.h"

namespace {

constexpr int32_t kNoAllocMaxVertices = 1 << 18;
constexpr int kNoAllocMaxGrid = 1024;   // cooperative grid bound (blocks)
constexpr int kMaxDevices = 64;

constexpr size_t al256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kArr = al256((size_t)(kNoAllocMaxVertices + 32) * 4);
constexpr size_t kWords = (size_t)(kNoAllocMaxVertices + 32) / 32 + 2;
constexpr size_t kBm = al256(kWords * 4);
constexpr size_t kCtl = al256(sizeof(gb::Ctl));
constexpr size_t kCheck = 256;  // the CSR check's flag
constexpr size_t kScratchBytes = kCtl + 15 * kArr + 4 * kBm + al256(2 * kNoAllocMaxGrid * 4) +
                                 al256(2 * kNoAllocMaxGrid * 8) + kCheck;

// The scratch.  Host code must not pass this name to a kernel: on the host
// it is a stand-in symbol, not a device address; its device address comes
// from cudaGetSymbolAddress at set-up.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

struct DeviceSetup {
  bool ready = false;
  unsigned char* scratch = nullptr;  // device address of g_noalloc_scratch
  int grid = 0;
};
DeviceSetup g_setup[kMaxDevices];
std::mutex g_setup_mu;

gb_status setup_device(int dev, DeviceSetup** out) {
  std::lock_guard<std::mutex> lk(g_setup_mu);
  DeviceSetup& d = g_setup[dev];
  if (!d.ready) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      gb_set_error("gb_scc_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
      return GB_ERR_CUDA;
    }
    const int grid = gb::max_coop_grid(dev);
    if (grid <= 0 || grid > kNoAllocMaxGrid) {
      gb_set_error("gb_scc_noalloc: %s", "no usable cooperative grid on this device");
      return GB_ERR_UNSUPPORTED;
    }
    d.scratch = static_cast<unsigned char*>(p);
    d.grid = grid;
    d.ready = true;
  }
  *out = &d;
  return GB_OK;
}

// Device memory of device dev (or managed memory): the only memory the run
// kernels may be given.
bool on_device(const void* p, int dev) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (a.type == cudaMemoryTypeManaged) return true;
  return a.type == cudaMemoryTypeDevice && a.device == dev;
}

}  // namespace

extern "C" gb_status gb_scc_noalloc(int32_t n, int64_t m, const int64_t* out_off,
                                    const int32_t* out_adj, const int64_t* in_off,
                                    const int32_t* in_adj, int32_t* labels, void* stream) {
  if (n < 0 || m < 0 || (n > 0 && (!out_off || !in_off || !labels)) ||
      (m > 0 && (!out_adj || !in_adj))) {
    gb_set_error("gb_scc_noalloc: %s", "bad argument");
    return GB_ERR_INVALID;
  }
  if (n > kNoAllocMaxVertices) {
    gb_set_error("gb_scc_noalloc: %s", "more vertices than the fixed scratch holds (262144)");
    return GB_ERR_CAPACITY;
  }
  if (n == 0) return GB_OK;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    gb_set_error("gb_scc_noalloc: %s", e != cudaSuccess ? cudaGetErrorString(e) : "device index");
    return e == cudaErrorNoDevice ? GB_ERR_NO_DEVICE : GB_ERR_CUDA;
  }
  if (!on_device(out_off, dev) || !on_device(in_off, dev) || !on_device(labels, dev) ||
      (m > 0 && (!on_device(out_adj, dev) || !on_device(in_adj, dev)))) {
    gb_set_error("gb_scc_noalloc: %s", "CSR and labels must be device memory of the current device");
    return GB_ERR_INVALID;
  }
  DeviceSetup* d = nullptr;
  gb_status st = setup_device(dev, &d);
  if (st != GB_OK) return st;

  // carve the scratch (same arrays as a context's workspace)
  unsigned char* p = d->scratch;
  gb::Ctl* ctl = reinterpret_cast<gb::Ctl*>(p);
  p += kCtl;
  gb::Work w{};
  auto take = [&](size_t bytes) {
    unsigned char* r = p;
    p += bytes;
    return r;
  };
  w.label = labels;  // the caller's output array
  take(kArr);        // (the workspace label slot stays unused here)
  w.colour = (int32_t*)take(kArr);
  w.live_in = (int32_t*)take(kArr);
  w.live_out = (int32_t*)take(kArr);
  w.listA = (int32_t*)take(kArr);
  w.listB = (int32_t*)take(kArr);
  w.q = (int32_t*)take(kArr);
  w.x0 = (int32_t*)take(kArr);
  w.x1 = (int32_t*)take(kArr);
  w.candA = (int32_t*)take(kArr);
  w.candB = (int32_t*)take(kArr);
  w.h0 = (int32_t*)take(kArr);
  w.h1 = (int32_t*)take(kArr);
  w.xa = (int32_t*)take(kArr);
  w.xb = (int32_t*)take(kArr);
  w.vbits = (uint32_t*)take(kBm);
  w.fvis = (uint32_t*)take(kBm);
  w.bvis = (uint32_t*)take(kBm);
  w.done = (uint32_t*)take(kBm);
  w.blk_i = (int32_t*)take(al256(2 * kNoAllocMaxGrid * 4));
  w.blk_l = (long long*)take(al256(2 * kNoAllocMaxGrid * 8));
  int* d_bad = (int*)take(kCheck);
  w.ctl = ctl;
  w.n = n;
  w.nwords = (n + 31) / 32;
  w.m = m;

  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // the caller's CSR is checked before any kernel indexes through it
  static thread_local int h_bad;
  h_bad = 0;
  if ((e = cudaMemsetAsync(d_bad, 0, sizeof(int), s)) != cudaSuccess ||
      (e = gb::check_csr_flag(n, m, out_off, out_adj, d_bad, s)) != cudaSuccess ||
      (e = gb::check_csr_flag(n, m, in_off, in_adj, d_bad, s)) != cudaSuccess ||
      (e = cudaMemcpyAsync(&h_bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, s)) !=
          cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess) {
    gb_set_error("gb_scc_noalloc: %s", cudaGetErrorString(e));
    return GB_ERR_CUDA;
  }
  if (h_bad != 0) {
    gb_set_error("gb_scc_noalloc: %s",
                 "CSR check failed: offsets not monotone from 0 to m, or an id outside [0, n)");
    return GB_ERR_INVALID;
  }
  // state that must start cleared (the array keeps the previous call's)
  if ((e = cudaMemsetAsync(ctl, 0, sizeof(gb::Ctl), s)) != cudaSuccess ||
      (e = cudaMemsetAsync(w.fvis, 0, (size_t)w.nwords * 4, s)) != cudaSuccess ||
      (e = cudaMemsetAsync(w.bvis, 0, (size_t)w.nwords * 4, s)) != cudaSuccess ||
      (e = cudaMemsetAsync(w.done, 0, (size_t)w.nwords * 4, s)) != cudaSuccess) {
    gb_set_error("gb_scc_noalloc: %s", cudaGetErrorString(e));
    return GB_ERR_CUDA;
  }
  gb::GraphView gv{};
  gv.n = n;
  gv.m = m;
  gv.out = {out_off, out_adj, nullptr};
  gv.in = {in_off, in_adj, nullptr};
  gb_opts o;
  gb_opts_default(&o);
  gb::RunParams prm{};
  prm.trim_level = o.trim_level;
  prm.fwbw_rounds = 1;
  prm.canonical = 1;
  prm.pivot_hint = -1;
  prm.count_unassigned = 0;
  prm.tune.t_block = o.t_block;
  prm.tune.t_grid = o.t_grid;
  prm.tune.k_pull = o.k_pull;
  prm.tune.alpha = o.alpha;
  prm.tune.beta = o.beta;
  prm.tune.max_steps = o.max_steps;
  if ((e = gb::launch_run(gv, gb::kSCC, prm, w, d->grid, s, nullptr)) != cudaSuccess) {
    gb_set_error("gb_scc_noalloc: %s", cudaGetErrorString(e));
    return GB_ERR_CUDA;
  }
  // the device-side status of this call (a bounded wait or a capacity check)
  static thread_local int h_err[2];
  if ((e = cudaMemcpyAsync(h_err, &ctl->err, 2 * sizeof(int), cudaMemcpyDeviceToHost, s)) !=
          cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess) {
    gb_set_error("gb_scc_noalloc: %s", cudaGetErrorString(e));
    return GB_ERR_CUDA;
  }
  if (h_err[0] != 0) {
    char buf[64];
    std::snprintf(buf, sizeof(buf), "device error %d at site %d", h_err[0], h_err[1]);
    gb_set_error("gb_scc_noalloc: %s", buf);
    return (gb_status)h_err[0];
  }
  return GB_OK;
}
