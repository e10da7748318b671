// Graph files read on the device.
//
// Text: the reference's edge-list format (read_edge, multistep/
// scc_main.cpp:94-125): "n m", then m lines "src dst".  The host reads the
// header and streams the file body to the device through two pinned staging
// buffers; the device splits the body into tokens (maximal runs of
// non-blank bytes), numbers them with a scan over fixed byte chunks, and
// parses token k into edge k / 2 (k even: source, odd: target).  Tokens after
// the first 2m are ignored, as the reference stops after m lines; a token
// that is not a decimal integer in [0, n), or too few tokens, is an error.
//
// Binary: "GBEDGES1", int64 n, int64 m (little endian), m int32 sources,
// m int32 targets.  The arrays are streamed to the device the same way.
//
// Either way the edges end on the device and the CSR is built there
// (gb::graph_from_edges).
#include <cub/cub.cuh>

#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/gbconn.h"
#include "api_internal.h"
#include "gb_internal.cuh"
#include "host_internal.h"

namespace {

constexpr char kMagic[8] = {'G', 'B', 'E', 'D', 'G', 'E', 'S', '1'};
constexpr size_t kStageBytes = 64u << 20;  // per pinned staging buffer

__device__ __forceinline__ bool is_blank(unsigned char ch) {
  return ch == ' ' || ch == '\t' || ch == '\r' || ch == '\n';
}

// Tokens starting in each chunk of `chunk` bytes.
__global__ void k_tok_count(const unsigned char* __restrict__ t, int64_t len, int64_t nchunks,
                            int chunk, int64_t* __restrict__ cnt) {
  for (int64_t ci = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; ci < nchunks;
       ci += (int64_t)gridDim.x * blockDim.x) {
    const int64_t lo = ci * chunk, hi = lo + chunk < len ? lo + chunk : len;
    bool prev_blank = lo == 0 ? true : is_blank(__ldg(t + lo - 1));
    int64_t c = 0;
    for (int64_t i = lo; i < hi; ++i) {
      const bool b = is_blank(__ldg(t + i));
      c += (!b && prev_blank) ? 1 : 0;
      prev_blank = b;
    }
    cnt[ci] = c;
  }
}

// Parses the tokens starting in each chunk (first[ci]: rank of the chunk's
// first token).  bad |= 1: a token that is not an integer in [0, n).
__global__ void k_tok_parse(const unsigned char* __restrict__ t, int64_t len, int64_t nchunks,
                            int chunk, const int64_t* __restrict__ first, int64_t m, int32_t n,
                            int32_t* __restrict__ src, int32_t* __restrict__ dst, int* bad) {
  for (int64_t ci = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; ci < nchunks;
       ci += (int64_t)gridDim.x * blockDim.x) {
    int64_t k = first[ci];
    if (k >= 2 * m) continue;
    const int64_t lo = ci * chunk, hi = lo + chunk < len ? lo + chunk : len;
    bool prev_blank = lo == 0 ? true : is_blank(__ldg(t + lo - 1));
    for (int64_t i = lo; i < hi && k < 2 * m; ++i) {
      const unsigned char ch0 = __ldg(t + i);
      const bool b = is_blank(ch0);
      if (!b && prev_blank) {
        // the token may run past the chunk
        int64_t j = i;
        bool neg = false, ok = true, any = false;
        if (ch0 == '+' || ch0 == '-') {
          neg = ch0 == '-';
          ++j;
        }
        long long v = 0;
        for (; j < len; ++j) {
          const unsigned char ch = __ldg(t + j);
          if (is_blank(ch)) break;
          if (ch < '0' || ch > '9') {
            ok = false;
            break;
          }
          any = true;
          if (v <= (long long)n) v = v * 10 + (ch - '0');
        }
        if (!ok || !any || (neg && v != 0) || v >= n) atomicOr(bad, 1);
        (k & 1 ? dst : src)[k >> 1] = (int32_t)(v < n ? v : 0);
        ++k;
      }
      prev_blank = b;
    }
  }
}

#define CKI(call, where)                                   \
  do {                                                     \
    cudaError_t e_ = (call);                               \
    if (e_ != cudaSuccess) return gb::cuda_fail(e_, where); \
  } while (0)

int grid_of(int64_t work) {
  int64_t g = (work + 255) / 256;
  if (g > 152 * 16) g = 152 * 16;
  return (int)(g < 1 ? 1 : g);
}

// Streams `bytes` bytes of f to dev through two pinned buffers (the copy of
// one overlaps the read of the next).
gb_status stream_to_device(gb_ctx* c, FILE* f, unsigned char* dev, int64_t bytes,
                           const char* path) {
  if (bytes <= 0) return GB_OK;
  unsigned char* stage[2] = {nullptr, nullptr};
  cudaEvent_t done[2] = {nullptr, nullptr};
  gb_status s = GB_OK;
  const size_t sb = (size_t)(bytes < (int64_t)kStageBytes ? bytes : (int64_t)kStageBytes);
  for (int i = 0; i < 2 && s == GB_OK; ++i) {
    if (cudaMallocHost(&stage[i], sb) != cudaSuccess ||
        cudaEventCreateWithFlags(&done[i], cudaEventDisableTiming) != cudaSuccess)
      s = GB_ERR_OOM;
  }
  int64_t off = 0;
  for (int i = 0; s == GB_OK && off < bytes; i ^= 1) {
    const size_t want = (size_t)(bytes - off < (int64_t)sb ? bytes - off : (int64_t)sb);
    if (cudaEventSynchronize(done[i]) != cudaSuccess) { s = GB_ERR_CUDA; break; }
    if (std::fread(stage[i], 1, want, f) != want) {
      gb_set_error("graph file: short read of %s", path);
      s = GB_ERR_IO;
      break;
    }
    if (cudaMemcpyAsync(dev + off, stage[i], want, cudaMemcpyHostToDevice, c->stream) !=
            cudaSuccess ||
        cudaEventRecord(done[i], c->stream) != cudaSuccess) {
      s = GB_ERR_CUDA;
      break;
    }
    off += (int64_t)want;
  }
  cudaStreamSynchronize(c->stream);
  for (int i = 0; i < 2; ++i) {
    if (stage[i]) cudaFreeHost(stage[i]);
    if (done[i]) cudaEventDestroy(done[i]);
  }
  return s;
}

// Reads one decimal integer from the file's header bytes.
bool header_int(const std::vector<char>& h, size_t& p, long long& out) {
  while (p < h.size() && (h[p] == ' ' || h[p] == '\t' || h[p] == '\r' || h[p] == '\n')) ++p;
  if (p >= h.size() || h[p] < '0' || h[p] > '9') return false;
  long long v = 0;
  while (p < h.size() && h[p] >= '0' && h[p] <= '9') {
    v = v * 10 + (h[p] - '0');
    if (v > (1ll << 40)) return false;
    ++p;
  }
  out = v;
  return true;
}

gb_status from_text(gb_ctx* c, FILE* f, const char* path, int64_t size, int chunk,
                    gb_graph** out) {
  // header: the first two tokens
  std::vector<char> h((size_t)(size < 256 ? size : 256));
  if (!h.empty() && std::fread(h.data(), 1, h.size(), f) != h.size()) {
    gb_set_error("graph file: short read of %s", path);
    return GB_ERR_IO;
  }
  size_t p = 0;
  long long nn = 0, mm = 0;
  if (!header_int(h, p, nn) || !header_int(h, p, mm) || nn > 0x7fffffffll ||
      (p < h.size() && !(h[p] == ' ' || h[p] == '\t' || h[p] == '\r' || h[p] == '\n'))) {
    gb_set_error("graph file: bad header in %s", path);
    return GB_ERR_IO;
  }
  const int32_t n = (int32_t)nn;
  const int64_t m = mm;
  const int64_t body = size - (int64_t)p;
  std::fseek(f, (long)p, SEEK_SET);
  cudaStream_t s = c->stream;
  unsigned char* text = nullptr;
  int64_t* cnt = nullptr;
  int64_t* first = nullptr;
  int32_t *src = nullptr, *dst = nullptr;
  int* bad = nullptr;
  void* tmp = nullptr;
  size_t tmp_bytes = 0;
  const int64_t nchunks = (body + chunk - 1) / chunk;
  gb_status st = GB_OK;
  auto cleanup = [&]() {
    cudaFreeAsync(text, s);
    cudaFreeAsync(cnt, s);
    cudaFreeAsync(first, s);
    cudaFreeAsync(src, s);
    cudaFreeAsync(dst, s);
    cudaFreeAsync(bad, s);
    cudaFreeAsync(tmp, s);
    cudaStreamSynchronize(s);
  };
  if (cudaMallocAsync(&text, (size_t)(body > 0 ? body : 1), s) != cudaSuccess ||
      cudaMallocAsync(&cnt, (size_t)(nchunks + 1) * 8, s) != cudaSuccess ||
      cudaMallocAsync(&first, (size_t)(nchunks + 1) * 8, s) != cudaSuccess ||
      cudaMallocAsync(&src, (size_t)(m > 0 ? m : 1) * 4, s) != cudaSuccess ||
      cudaMallocAsync(&dst, (size_t)(m > 0 ? m : 1) * 4, s) != cudaSuccess ||
      cudaMallocAsync(&bad, sizeof(int), s) != cudaSuccess) {
    cleanup();
    gb_set_error("graph file: %s", "out of device memory");
    return GB_ERR_OOM;
  }
  st = stream_to_device(c, f, text, body, path);
  if (st != GB_OK) {
    cleanup();
    return st;
  }
  int64_t ntok = 0;
  int hbad = 0;
  if (nchunks > 0) {
    cudaMemsetAsync(cnt + nchunks, 0, 8, s);
    k_tok_count<<<grid_of(nchunks), 256, 0, s>>>(text, body, nchunks, chunk, cnt);
    cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, cnt, first, nchunks + 1, s);
    if (cudaMallocAsync(&tmp, tmp_bytes ? tmp_bytes : 16, s) != cudaSuccess) {
      cleanup();
      return GB_ERR_OOM;
    }
    cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, cnt, first, nchunks + 1, s);
    cudaMemsetAsync(bad, 0, sizeof(int), s);
    k_tok_parse<<<grid_of(nchunks), 256, 0, s>>>(text, body, nchunks, chunk, first, m, n, src,
                                                  dst, bad);
    cudaMemcpyAsync(&ntok, first + nchunks, 8, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, s);
  }
  const cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess || cudaGetLastError() != cudaSuccess) {
    cleanup();
    return gb::cuda_fail(e != cudaSuccess ? e : cudaErrorUnknown, "graph file parse");
  }
  if (ntok < 2 * m) {
    cleanup();
    gb_set_error("graph file: fewer edges than the header says in %s", path);
    return GB_ERR_IO;
  }
  if (hbad) {
    cleanup();
    gb_set_error("graph file: a token that is not a vertex id in [0, n) in %s", path);
    return GB_ERR_INVALID;
  }
  cudaFreeAsync(text, s);
  text = nullptr;
  st = gb::graph_from_edges(c, n, m, src, dst, false, out);
  cleanup();
  return st;
}

gb_status from_binary(gb_ctx* c, FILE* f, const char* path, int64_t size, gb_graph** out) {
  int64_t hdr[2];
  if (std::fread(hdr, 8, 2, f) != 2 || hdr[0] < 0 || hdr[0] > 0x7fffffffll || hdr[1] < 0 ||
      size < 24 + 8 * hdr[1]) {
    gb_set_error("graph file: bad binary header in %s", path);
    return GB_ERR_IO;
  }
  const int32_t n = (int32_t)hdr[0];
  const int64_t m = hdr[1];
  cudaStream_t s = c->stream;
  int32_t *src = nullptr, *dst = nullptr;
  if (cudaMallocAsync(&src, (size_t)(m > 0 ? m : 1) * 4, s) != cudaSuccess ||
      cudaMallocAsync(&dst, (size_t)(m > 0 ? m : 1) * 4, s) != cudaSuccess) {
    cudaFreeAsync(src, s);
    cudaFreeAsync(dst, s);
    return GB_ERR_OOM;
  }
  gb_status st = stream_to_device(c, f, (unsigned char*)src, m * 4, path);
  if (st == GB_OK) st = stream_to_device(c, f, (unsigned char*)dst, m * 4, path);
  if (st == GB_OK) st = gb::graph_from_edges(c, n, m, src, dst, false, out);
  cudaFreeAsync(src, s);
  cudaFreeAsync(dst, s);
  cudaStreamSynchronize(s);
  return st;
}

}  // namespace

extern "C" {

gb_status gb_graph_from_file2(gb_ctx* c, const char* path, int32_t chunk, gb_graph** out) {
  if (!c || !path || !out || chunk < 0) {
    gb_set_error("graph file: %s", "bad argument");
    return GB_ERR_INVALID;
  }
  *out = nullptr;
  if (cudaSetDevice(c->device) != cudaSuccess) return GB_ERR_CUDA;
  FILE* f = std::fopen(path, "rb");
  if (!f) {
    gb_set_error("graph file: cannot open %s", path);
    return GB_ERR_IO;
  }
  std::fseek(f, 0, SEEK_END);
  const int64_t size = (int64_t)std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  char magic[8] = {0};
  const bool binary = size >= 24 && std::fread(magic, 1, 8, f) == 8 &&
                      std::memcmp(magic, kMagic, 8) == 0;
  gb_status st;
  if (binary) {
    st = from_binary(c, f, path, size, out);
  } else {
    std::fseek(f, 0, SEEK_SET);
    st = from_text(c, f, path, size, chunk > 0 ? chunk : 256, out);
  }
  std::fclose(f);
  return st;
}

gb_status gb_graph_from_file(gb_ctx* c, const char* path, gb_graph** out) {
  return gb_graph_from_file2(c, path, 0, out);
}

gb_status gb_write_binary(const char* path, int32_t n, int64_t m, const int32_t* src,
                          const int32_t* dst) {
  if (!path || n < 0 || m < 0 || (m > 0 && (!src || !dst))) return GB_ERR_INVALID;
  FILE* f = std::fopen(path, "wb");
  if (!f) {
    gb_set_error("gb_write_binary: cannot open %s", path);
    return GB_ERR_IO;
  }
  const int64_t hdr[2] = {n, m};
  const bool ok = std::fwrite(kMagic, 1, 8, f) == 8 && std::fwrite(hdr, 8, 2, f) == 2 &&
                  (m == 0 || (std::fwrite(src, 4, (size_t)m, f) == (size_t)m &&
                              std::fwrite(dst, 4, (size_t)m, f) == (size_t)m));
  if (std::fclose(f) != 0 || !ok) {
    gb_set_error("gb_write_binary: write failed for %s", path);
    return GB_ERR_IO;
  }
  return GB_OK;
}

}  // extern "C"
