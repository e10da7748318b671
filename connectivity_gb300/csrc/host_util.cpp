// Host-side parts of libgbconn: the edge-list reader and label writer, the
// verify statistics, host relabelling, status strings and the seeded
// synthetic-graph generators.  No CUDA here; these run without a GPU.
//
// This file is compiled with -ffp-contract=off: the batch-size generator
// uses only IEEE-754 +, -, *, / in a fixed order, so x86-64 and aarch64
// produce the same sizes.
#include <algorithm>
#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <fcntl.h>
#include <omp.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include "../../include/gbconn.h"
#include "gen_common.h"
#include "host_internal.h"

namespace {
thread_local std::string g_last_error;
}

void gb_set_error(const char* fmt, const char* detail) {
  char buf[512];
  std::snprintf(buf, sizeof(buf), fmt, detail ? detail : "");
  g_last_error = buf;
}

extern "C" const char* gb_last_error(void) { return g_last_error.c_str(); }

extern "C" const char* gb_status_string(gb_status s) {
  switch (s) {
    case GB_OK: return "ok";
    case GB_ERR_INVALID: return "invalid argument";
    case GB_ERR_CUDA: return "CUDA error";
    case GB_ERR_OOM: return "out of memory";
    case GB_ERR_TIMEOUT: return "device wait timed out";
    case GB_ERR_ITER_LIMIT: return "iteration limit reached";
    case GB_ERR_IO: return "I/O error";
    case GB_ERR_NO_DEVICE: return "no CUDA device";
    case GB_ERR_UNSUPPORTED: return "unsupported device";
    case GB_ERR_CAPACITY: return "capacity exceeded";
    default: return "unknown status";
  }
}

extern "C" void gb_free_host(void* p) { std::free(p); }

// ---------------------------------------------------------------------------
// Text edge list: "n m" on the first line, then m lines "src dst"
// (read_edge, multistep/scc_main.cpp:94-125).  The reference splits fields on
// a single space and converts with atoi; this parser accepts any run of
// blanks and checks every id against n.
// ---------------------------------------------------------------------------
namespace {
struct Cursor {
  const char* p;
  const char* end;
  bool skip_ws() {
    while (p < end && (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\n')) ++p;
    return p < end;
  }
  bool read_i64(long long& out) {
    if (!skip_ws()) return false;
    bool neg = false;
    if (*p == '-' || *p == '+') { neg = *p == '-'; ++p; }
    if (p >= end || *p < '0' || *p > '9') return false;
    long long v = 0;
    while (p < end && *p >= '0' && *p <= '9') {
      v = v * 10 + (*p - '0');
      if (v > (1ll << 62)) return false;
      ++p;
    }
    out = neg ? -v : v;
    return true;
  }
};
}  // namespace

// The body is parsed in pieces by OpenMP threads.  A piece starts at a
// blank, so it never splits a number, and every piece is read with the same
// cursor as a whole file would be.  Pass 1 counts the numbers each piece
// holds up to its end or its first unreadable byte; a prefix over the counts
// places each piece's numbers in the global sequence; pass 2 stores number
// k into edge k / 2 and notes the first edge with an id outside [0, n).
// The outcome is the sequential reader's: the first failure in edge order
// wins (an unreadable or missing number: GB_ERR_IO; an id out of range in an
// edge read whole: GB_ERR_INVALID), and numbers after the first 2m are
// ignored.
namespace {
struct Piece {
  const char* lo;
  const char* hi;
  long long count = 0;  // numbers read before hi or the failure
  bool failed = false;  // an unreadable byte before hi
  long long first = 0;  // global index of the piece's first number
};

long long read_body(const char* body, const char* end, long long nn, long long mm, int pieces,
                    int32_t* s, int32_t* d, long long* bad_edge) {
  // returns the count of numbers readable before the first failure (capped
  // at 2m); *bad_edge = first edge with an id out of range, or mm
  const long long len = (long long)(end - body);
  if (pieces <= 0) {
    const long long want = len / (1 << 20) + 1;  // about 1 MB per piece
    pieces = (int)std::min<long long>(want, 64LL * omp_get_max_threads());
  }
  if (pieces > len) pieces = (int)std::max<long long>(len, 1);
  auto blank = [](char ch) { return ch == ' ' || ch == '\t' || ch == '\r' || ch == '\n'; };
  std::vector<Piece> pc((size_t)pieces);
  for (int i = 0; i < pieces; ++i) {
    const char* lo = body + len * i / pieces;
    if (i > 0)
      while (lo < end && !blank(*lo)) ++lo;  // start at a blank (or the end)
    pc[(size_t)i].lo = lo;
  }
  for (int i = 0; i < pieces; ++i) pc[(size_t)i].hi = i + 1 < pieces ? pc[(size_t)i + 1].lo : end;
  for (int i = 0; i + 1 < pieces; ++i)  // a later start pushed past an earlier one
    if (pc[(size_t)i].hi < pc[(size_t)i].lo) pc[(size_t)i].hi = pc[(size_t)i].lo;
#pragma omp parallel for schedule(dynamic, 1)
  for (int i = 0; i < pieces; ++i) {
    Piece& q = pc[(size_t)i];
    Cursor c{q.lo, q.hi};
    long long v;
    while (c.skip_ws()) {
      if (!c.read_i64(v)) {
        q.failed = true;
        break;
      }
      ++q.count;
    }
  }
  long long avail = 0;  // numbers before the first failure
  bool stop = false;
  for (int i = 0; i < pieces; ++i) {
    Piece& q = pc[(size_t)i];
    if (stop) {  // after the first failure, or past 2m numbers: not stored
      q.count = 0;
      continue;
    }
    q.first = avail;
    avail += q.count;
    stop = q.failed || avail >= 2 * mm;
  }
  if (avail > 2 * mm) avail = 2 * mm;
  long long bad = mm;
#pragma omp parallel for schedule(dynamic, 1) reduction(min : bad)
  for (int i = 0; i < pieces; ++i) {
    Piece& q = pc[(size_t)i];
    if (q.count == 0 || q.first >= avail) continue;
    Cursor c{q.lo, q.hi};
    long long v = 0;
    for (long long k = q.first; k < avail && k < q.first + q.count; ++k) {
      c.read_i64(v);  // counted in pass 1: it reads
      const long long e = k >> 1;
      if (v < 0 || v >= nn) bad = std::min(bad, e);
      if (k & 1) d[e] = (int32_t)v;
      else s[e] = (int32_t)v;
    }
  }
  *bad_edge = bad;
  return avail;
}
}  // namespace

extern "C" gb_status gb_read_edge_pieces(const char* path, int32_t pieces, int32_t* n, int64_t* m,
                                         int32_t** srcs, int32_t** dsts) {
  if (!path || !n || !m || !srcs || !dsts) {
    gb_set_error("gb_read_edge: null argument%s", "");
    return GB_ERR_INVALID;
  }
  // the file is mapped, not copied (a multi-GB edge list is parsed in place)
  const int fd = ::open(path, O_RDONLY);
  if (fd < 0) {
    gb_set_error("gb_read_edge: cannot open %s", path);
    return GB_ERR_IO;
  }
  struct stat sb;
  if (::fstat(fd, &sb) != 0) {
    ::close(fd);
    gb_set_error("gb_read_edge: cannot stat %s", path);
    return GB_ERR_IO;
  }
  const size_t size = (size_t)(sb.st_size > 0 ? sb.st_size : 0);
  const char* base = "";
  void* map = nullptr;
  if (size > 0) {
    map = ::mmap(nullptr, size, PROT_READ, MAP_PRIVATE, fd, 0);
    if (map == MAP_FAILED) {
      ::close(fd);
      gb_set_error("gb_read_edge: cannot map %s", path);
      return GB_ERR_IO;
    }
    ::madvise(map, size, MADV_SEQUENTIAL);
    base = (const char*)map;
  }
  ::close(fd);
  struct Unmap {
    void* p;
    size_t n;
    ~Unmap() {
      if (p) ::munmap(p, n);
    }
  } unmap{map, size};
  Cursor c{base, base + size};
  long long nn, mm;
  if (!c.read_i64(nn) || !c.read_i64(mm) || nn < 0 || nn > 0x7fffffffll || mm < 0) {
    gb_set_error("gb_read_edge: bad header in %s", path);
    return GB_ERR_IO;
  }
  // every edge takes at least 4 bytes of the body (a blank, an id, a blank,
  // an id), so a header m above that cannot be met; checked before the
  // arrays are sized from it
  if (mm > (long long)((size_t)(base + size - c.p) / 4)) {
    gb_set_error("gb_read_edge: fewer edges than the header says in %s", path);
    return GB_ERR_IO;
  }
  int32_t* s = (int32_t*)std::malloc((size_t)(mm > 0 ? mm : 1) * sizeof(int32_t));
  int32_t* d = (int32_t*)std::malloc((size_t)(mm > 0 ? mm : 1) * sizeof(int32_t));
  if (!s || !d) {
    std::free(s);
    std::free(d);
    gb_set_error("gb_read_edge: out of host memory%s", "");
    return GB_ERR_OOM;
  }
  long long bad = mm;
  const long long avail = read_body(c.p, base + size, nn, mm, pieces, s, d, &bad);
  const long long whole = avail / 2;  // edges read whole before the first failure
  if (bad < whole) {
    std::free(s);
    std::free(d);
    gb_set_error("gb_read_edge: vertex id out of range in %s", path);
    return GB_ERR_INVALID;
  }
  if (avail < 2 * mm) {
    std::free(s);
    std::free(d);
    gb_set_error("gb_read_edge: fewer edges than the header says in %s", path);
    return GB_ERR_IO;
  }
  *n = (int32_t)nn;
  *m = mm;
  *srcs = s;
  *dsts = d;
  return GB_OK;
}

extern "C" gb_status gb_read_edge(const char* path, int32_t* n, int64_t* m, int32_t** srcs,
                                  int32_t** dsts) {
  return gb_read_edge_pieces(path, 0, n, m, srcs, dsts);
}

// The decimal digits of v at p; returns the end.
static char* put_u32(char* p, uint32_t v) {
  char tmp[12];
  int k = 0;
  do {
    tmp[k++] = (char)('0' + v % 10);
    v /= 10;
  } while (v);
  while (k) *p++ = tmp[--k];
  return p;
}

// One label per line ("%d\n", as output_scc writes them), formatted in
// 1 MB blocks of lines.
extern "C" gb_status gb_output_labels(const char* path, int32_t n, const int32_t* labels) {
  if (!path || (n > 0 && !labels) || n < 0) return GB_ERR_INVALID;
  FILE* f = std::fopen(path, "wb");
  if (!f) {
    gb_set_error("gb_output_labels: cannot open %s", path);
    return GB_ERR_IO;
  }
  constexpr size_t kBlock = 1 << 20;
  std::vector<char> out(kBlock + 16);
  char* p = out.data();
  bool ok = true;
  for (int32_t i = 0; i < n && ok; ++i) {
    const int32_t l = labels[i];
    if (l < 0) *p++ = '-';
    p = put_u32(p, l < 0 ? 0u - (uint32_t)l : (uint32_t)l);
    *p++ = '\n';
    if ((size_t)(p - out.data()) >= kBlock) {
      ok = std::fwrite(out.data(), 1, (size_t)(p - out.data()), f) == (size_t)(p - out.data());
      p = out.data();
    }
  }
  ok = ok && std::fwrite(out.data(), 1, (size_t)(p - out.data()), f) == (size_t)(p - out.data());
  ok = (std::fclose(f) == 0) && ok;
  return ok ? GB_OK : GB_ERR_IO;
}

// Edge list in the reference's text format ("n m", then "src dst" lines),
// the input of read_edge (scc_main.cpp:94-125).
extern "C" gb_status gb_write_text(const char* path, int32_t n, int64_t m, const int32_t* src,
                                   const int32_t* dst) {
  if (!path || n < 0 || m < 0 || (m > 0 && (!src || !dst))) return GB_ERR_INVALID;
  FILE* f = std::fopen(path, "wb");
  if (!f) {
    gb_set_error("gb_write_text: cannot open %s", path);
    return GB_ERR_IO;
  }
  std::vector<char> out(1 << 22);
  int len = std::snprintf(out.data(), out.size(), "%d %lld\n", n, (long long)m);
  char* p = out.data() + len;
  bool ok = true;
  for (int64_t i = 0; i < m && ok; ++i) {
    if (src[i] < 0 || dst[i] < 0) {
      ok = false;
      break;
    }
    p = put_u32(p, (uint32_t)src[i]);
    *p++ = ' ';
    p = put_u32(p, (uint32_t)dst[i]);
    *p++ = '\n';
    if ((size_t)(p - out.data()) > out.size() - 32) {
      ok = std::fwrite(out.data(), 1, (size_t)(p - out.data()), f) == (size_t)(p - out.data());
      p = out.data();
    }
  }
  if (ok) ok = std::fwrite(out.data(), 1, (size_t)(p - out.data()), f) == (size_t)(p - out.data());
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) gb_set_error("gb_write_text: write failed for %s", path);
  return ok ? GB_OK : GB_ERR_IO;
}

// ---------------------------------------------------------------------------
// Verify statistics (scc_verify.cpp:47-77, cc_verify.cpp:47-74): a label
// histogram; components, components with more than one vertex, the largest,
// and vertices without a label.
// ---------------------------------------------------------------------------
static void label_stats(int32_t n, const int32_t* labels, long long out[4]) {
  std::vector<int32_t> cnt((size_t)n + 1, 0);
  long long un = 0;
  for (int32_t i = 0; i < n; ++i) {
    int32_t l = labels[i];
    if (l >= 0 && l < n) cnt[l]++;
    else ++un;
  }
  long long comps = 0, nontriv = 0, mx = 0;
  for (int32_t i = 0; i < n; ++i) {
    if (!cnt[i]) continue;
    ++comps;
    if (cnt[i] > 1) ++nontriv;
    if (cnt[i] > mx) mx = cnt[i];
  }
  out[0] = comps;
  out[1] = nontriv;
  out[2] = mx;
  out[3] = un;
}

extern "C" gb_status gb_scc_verify(int32_t n, const int32_t* labels, char* line, size_t cap,
                                   int64_t stats[4]) {
  if (n < 0 || (n > 0 && !labels)) return GB_ERR_INVALID;
  long long s[4];
  label_stats(n, labels, s);
  if (line && cap) {
    std::snprintf(line, cap, "Num SCCs: %d, Nontrivial: %d, Max SCC: %d, Unassigned %d\n",
                  (int)s[0], (int)s[1], (int)s[2], (int)s[3]);
  }
  if (stats) for (int i = 0; i < 4; ++i) stats[i] = s[i];
  return GB_OK;
}

extern "C" gb_status gb_cc_verify(int32_t n, const int32_t* labels, char* line, size_t cap,
                                  int64_t stats[3]) {
  if (n < 0 || (n > 0 && !labels)) return GB_ERR_INVALID;
  long long s[4];
  label_stats(n, labels, s);
  if (line && cap) {
    std::snprintf(line, cap, "Num CCs: %d, Max CC: %d, Unassigned %d\n", (int)s[0], (int)s[2],
                  (int)s[3]);
  }
  if (stats) {
    stats[0] = s[0];
    stats[1] = s[2];
    stats[2] = s[3];
  }
  return GB_OK;
}

extern "C" gb_status gb_canonicalize(int32_t n, int32_t* labels) {
  if (n < 0 || (n > 0 && !labels)) return GB_ERR_INVALID;
  std::vector<int32_t> rep((size_t)n + 1, -1);
  for (int32_t v = 0; v < n; ++v) {
    int32_t l = labels[v];
    if (l >= 0 && l < n && rep[l] < 0) rep[l] = v;
  }
  for (int32_t v = 0; v < n; ++v) {
    int32_t l = labels[v];
    if (l >= 0 && l < n) labels[v] = rep[l];
  }
  return GB_OK;
}

// ---------------------------------------------------------------------------
// Generators
// ---------------------------------------------------------------------------
gb_rmat_thr gb_rmat_thresholds(double a, double b, double c) {
  auto fix = [](double x) -> uint32_t {
    if (x <= 0.0) return 0u;
    double v = x * 4294967296.0;
    if (v >= 4294967295.0) return 4294967295u;
    return (uint32_t)(v + 0.5);
  };
  gb_rmat_thr t;
  t.ta = fix(a);
  t.tab = fix(a + b);
  t.tabc = fix(a + b + c);
  return t;
}

// Parallel LSD radix sort of 64-bit keys on their low `bits` bits.
static void radix_sort_u64(std::vector<uint64_t>& keys, int bits) {
  const size_t n = keys.size();
  std::vector<uint64_t> tmp(n);
  const int R = 16, B = 1 << R;
  const int passes = (bits + R - 1) / R;
  int nt = omp_get_max_threads();
  std::vector<size_t> hist((size_t)nt * B);
  uint64_t* src = keys.data();
  uint64_t* dst = tmp.data();
  for (int p = 0; p < passes; ++p) {
    const int sh = p * R;
    std::fill(hist.begin(), hist.end(), 0);
#pragma omp parallel num_threads(nt)
    {
      const int t = omp_get_thread_num();
      const size_t lo = n * t / nt, hi = n * (t + 1) / nt;
      size_t* h = hist.data() + (size_t)t * B;
      for (size_t i = lo; i < hi; ++i) h[(src[i] >> sh) & (B - 1)]++;
    }
    size_t run = 0;
    for (int d = 0; d < B; ++d)
      for (int t = 0; t < nt; ++t) {
        size_t c = hist[(size_t)t * B + d];
        hist[(size_t)t * B + d] = run;
        run += c;
      }
#pragma omp parallel num_threads(nt)
    {
      const int t = omp_get_thread_num();
      const size_t lo = n * t / nt, hi = n * (t + 1) / nt;
      size_t* h = hist.data() + (size_t)t * B;
      for (size_t i = lo; i < hi; ++i) dst[h[(src[i] >> sh) & (B - 1)]++] = src[i];
    }
    std::swap(src, dst);
  }
  if (src != keys.data()) std::memcpy(keys.data(), src, n * sizeof(uint64_t));
}

// R-MAT graph on n vertices: edge_factor * n candidate edges drawn at scale
// ceil(log2 n); ids >= n, self-loops and duplicates dropped; sorted by
// (src, dst).  For n a power of two nothing is dropped but self-loops and
// duplicates.  The device generator follows the same rule.
static gb_status rmat_host(int32_t n, int32_t edge_factor, uint64_t seed, double a, double b,
                           double c, int64_t* m, int32_t** src, int32_t** dst) {
  if (n < 1 || edge_factor < 1 || !m || !src || !dst) return GB_ERR_INVALID;
  int scale = 1;
  while (scale < 31 && (1ll << scale) < (long long)n) ++scale;
  const long long m0 = (long long)edge_factor * n;
  const gb_rmat_thr thr = gb_rmat_thresholds(a, b, c);
  const uint64_t self = (1ull << (2 * scale)) - 1ull;  // marker of a dropped edge
  std::vector<uint64_t> keys((size_t)m0);
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < m0; ++i) {
    uint32_t s, d;
    gb_rmat_edge(seed, (uint64_t)i, scale, thr, &s, &d);
    keys[(size_t)i] = (s == d || s >= (uint32_t)n || d >= (uint32_t)n)
                          ? self
                          : (((uint64_t)s << scale) | d);
  }
  radix_sort_u64(keys, 2 * scale);
  size_t k = 0;
  for (size_t i = 0; i < keys.size(); ++i) {
    if (keys[i] == self) continue;
    if (k > 0 && keys[k - 1] == keys[i]) continue;
    keys[k++] = keys[i];
  }
  int32_t* s = (int32_t*)std::malloc((k ? k : 1) * sizeof(int32_t));
  int32_t* d = (int32_t*)std::malloc((k ? k : 1) * sizeof(int32_t));
  if (!s || !d) {
    std::free(s);
    std::free(d);
    return GB_ERR_OOM;
  }
  const uint64_t mask = (1ull << scale) - 1ull;
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < (long long)k; ++i) {
    s[i] = (int32_t)(keys[(size_t)i] >> scale);
    d[i] = (int32_t)(keys[(size_t)i] & mask);
  }
  *m = (int64_t)k;
  *src = s;
  *dst = d;
  return GB_OK;
}

extern "C" gb_status gb_rmat_edges_host(int32_t scale, int32_t edge_factor, uint64_t seed,
                                        double a, double b, double c, int64_t* m, int32_t** src,
                                        int32_t** dst) {
  if (scale < 1 || scale > 30) return GB_ERR_INVALID;
  return rmat_host((int32_t)(1 << scale), edge_factor, seed, a, b, c, m, src, dst);
}

extern "C" gb_status gb_rmat_edges_host_n(int32_t n, int32_t edge_factor, uint64_t seed, double a,
                                          double b, double c, int64_t* m, int32_t** src,
                                          int32_t** dst) {
  return rmat_host(n, edge_factor, seed, a, b, c, m, src, dst);
}

extern "C" gb_status gb_grid_edges_host(int32_t side, int32_t extra, int32_t max_chain,
                                        uint64_t seed, int32_t* n, int64_t* m, int32_t** src,
                                        int32_t** dst) {
  if (side < 1 || side > 40000 || extra < 0 || max_chain < 1 || !n || !m || !src || !dst)
    return GB_ERR_INVALID;
  const long long nl = (long long)side * side;
  if (nl + extra > 0x7fffffffll) return GB_ERR_INVALID;
  std::vector<int32_t> S, D;
  S.reserve((size_t)(nl * 2 + extra + 16));
  D.reserve((size_t)(nl * 2 + extra + 16));
  auto add = [&](long long u, long long v) {
    S.push_back((int32_t)u);
    D.push_back((int32_t)v);
  };
  for (long long r = 0; r < side; ++r) {
    for (long long cc = 0; cc < side; ++cc) {
      const long long u = r * side + cc;
      for (uint32_t axis = 0; axis < 2; ++axis) {
        if (axis == 0 && cc + 1 >= side) continue;
        if (axis == 1 && r + 1 >= side) continue;
        const long long v = axis == 0 ? u + 1 : u + side;
        switch (gb_grid_orient(seed, (uint64_t)u, axis)) {
          case 0: add(u, v); break;
          case 1: add(v, u); break;
          case 2: add(u, v); add(v, u); break;
          default: break;
        }
      }
    }
  }
  // chains of new vertices hung off random lattice vertices
  long long next = nl, left = extra, k = 0;
  const uint64_t cseed = seed ^ 0xC2B2AE3D27D4EB4Full;
  while (left > 0) {
    long long len = 1 + (long long)(gb_rand64(cseed, (uint64_t)k, 0) % (uint64_t)max_chain);
    if (len > left) len = left;
    const long long anchor = (long long)(gb_rand64(cseed, (uint64_t)k, 1) % (uint64_t)nl);
    const bool source_chain = (gb_rand64(cseed, (uint64_t)k, 2) & 1ull) == 0ull;
    if (source_chain) {  // head (in-degree 0) -> ... -> tail -> anchor
      for (long long j = 0; j + 1 < len; ++j) add(next + j, next + j + 1);
      add(next + len - 1, anchor);
    } else {  // anchor -> head -> ... -> tail (out-degree 0)
      add(anchor, next);
      for (long long j = 0; j + 1 < len; ++j) add(next + j, next + j + 1);
    }
    next += len;
    left -= len;
    ++k;
  }
  const size_t mm = S.size();
  int32_t* s = (int32_t*)std::malloc((mm ? mm : 1) * sizeof(int32_t));
  int32_t* d = (int32_t*)std::malloc((mm ? mm : 1) * sizeof(int32_t));
  if (!s || !d) {
    std::free(s);
    std::free(d);
    return GB_ERR_OOM;
  }
  std::memcpy(s, S.data(), mm * sizeof(int32_t));
  std::memcpy(d, D.data(), mm * sizeof(int32_t));
  *n = (int32_t)(nl + extra);
  *m = (int64_t)mm;
  *src = s;
  *dst = d;
  return GB_OK;
}

// exp(x) from range reduction x = k ln2 + r and a Taylor series in r, using
// only correctly rounded IEEE operations (no libm), so that every platform
// computes the same bits.
static double det_exp(double x) {
  const double ln2 = 0.6931471805599453;
  double kf = x / ln2;
  long long k = (long long)(kf < 0 ? kf - 0.5 : kf + 0.5);
  double r = x - (double)k * ln2;
  double term = 1.0, sum = 1.0;
  for (int i = 1; i < 30; ++i) {
    term = term * r / (double)i;
    sum = sum + term;
  }
  // scale by 2^k exactly
  while (k > 0) { sum *= 2.0; --k; }
  while (k < 0) { sum *= 0.5; ++k; }
  return sum;
}

extern "C" gb_status gb_batch_sizes(int32_t count, uint64_t seed, double median, double sigma,
                                    int32_t n_min, int32_t n_max, int32_t ef_min, int32_t ef_max,
                                    int32_t* n_out, int32_t* ef_out, uint64_t* seed_out) {
  if (count < 0 || n_min < 1 || n_max < n_min || ef_min < 1 || ef_max < ef_min || median <= 0 ||
      (count > 0 && (!n_out || !ef_out || !seed_out)))
    return GB_ERR_INVALID;
  for (int32_t i = 0; i < count; ++i) {
    double z = 0.0;
    for (int j = 0; j < 12; ++j) {
      const uint64_t r = gb_rand64(seed, (uint64_t)i, (uint64_t)j);
      z = z + (double)(r >> 11) * (1.0 / 9007199254740992.0);
    }
    z = z - 6.0;
    double x = median * det_exp(sigma * z);
    long long v = (long long)(x + 0.5);
    if (v < n_min) v = n_min;
    if (v > n_max) v = n_max;
    n_out[i] = (int32_t)v;
    const uint64_t r = gb_rand64(seed, (uint64_t)i, 100);
    ef_out[i] = ef_min + (int32_t)(r % (uint64_t)(ef_max - ef_min + 1));
    seed_out[i] = gb_mix64(seed ^ (0x5851F42D4C957F2Dull * (uint64_t)(i + 1)));
  }
  return GB_OK;
}

// ---------------------------------------------------------------------------
// Sharding a batch over devices
// ---------------------------------------------------------------------------
// Longest-processing-time-first: graphs in decreasing cost (ties: lower
// index first) each go to the shard with the least load so far (ties: lower
// shard).  The largest shard's load is at most the mean load plus the
// largest single cost.  Deterministic, so every rank of a job computes the
// same plan without communicating.
extern "C" gb_status gb_shard_plan(int32_t count, const int64_t* cost, int32_t shards,
                                   int32_t* shard_of, int64_t* load) {
  if (count < 0 || shards < 1 || (count > 0 && (!cost || !shard_of))) return GB_ERR_INVALID;
  for (int32_t i = 0; i < count; ++i)
    if (cost[i] < 0) return GB_ERR_INVALID;
  std::vector<int32_t> order((size_t)count);
  for (int32_t i = 0; i < count; ++i) order[(size_t)i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int32_t a, int32_t b) { return cost[a] > cost[b]; });
  std::vector<int64_t> acc((size_t)shards, 0);
  for (int32_t i : order) {
    int32_t best = 0;
    for (int32_t s = 1; s < shards; ++s)
      if (acc[(size_t)s] < acc[(size_t)best]) best = s;
    shard_of[i] = best;
    acc[(size_t)best] += cost[i];
  }
  if (load)
    for (int32_t s = 0; s < shards; ++s) load[s] = acc[(size_t)s];
  return GB_OK;
}
