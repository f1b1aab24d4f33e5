// graphio.cu -- graph files in the reference's formats, host side.
//
//   AdjacencyGraph text (gbbs/graph_io.cc:35-85): whitespace-separated tokens
//     "AdjacencyGraph", n, m, n offsets, m neighbour ids; offsets[n] = m.
//   binary CSR (gbbs/graph_io.cc:86-95 in a -DLONG build, .bazelrc:28): three
//     int64 words n, m and the file size, (n+1) uint64 offsets, m uint32 ids.
//
// Text is parsed by all host threads: the file is cut into chunks at
// whitespace, each chunk counts its tokens, a prefix over the counts gives
// every chunk its first token index, and the chunks then parse in parallel.
#include <algorithm>
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "internal.h"

namespace byo {

namespace {

constexpr char kHeader[] = "AdjacencyGraph";

bool is_space(char c) { return c == ' ' || c == '\n' || c == '\r' || c == '\t' || c == '\f' || c == '\v'; }

bool read_file(const char *path, std::vector<char> &buf) {
  FILE *f = std::fopen(path, "rb");
  if (!f) return false;
  bool ok = std::fseek(f, 0, SEEK_END) == 0;
  const long sz = ok ? std::ftell(f) : -1;
  ok = ok && sz >= 0 && std::fseek(f, 0, SEEK_SET) == 0;
  if (ok) {
    buf.resize((size_t)sz);
    ok = sz == 0 || std::fread(buf.data(), 1, (size_t)sz, f) == (size_t)sz;
  }
  std::fclose(f);
  return ok;
}

struct Chunk {
  size_t b = 0, e = 0;   // byte range, cut at whitespace
  uint64_t tokens = 0;   // tokens starting in the range
  uint64_t first = 0;    // index of its first token
  bool bad = false;      // a token that is not a decimal number
};

// Calls f(index, value) for every numeric token of [b, e), numbering from
// `first`; returns false on a non-numeric token.
template <typename F>
bool parse_range(const char *s, size_t b, size_t e, uint64_t first, F f) {
  size_t i = b;
  uint64_t k = first;
  while (i < e) {
    while (i < e && is_space(s[i])) i++;
    if (i >= e) break;
    uint64_t v = 0;
    size_t j = i;
    while (j < e && !is_space(s[j])) {
      const unsigned d = (unsigned)(unsigned char)s[j] - (unsigned)'0';
      if (d > 9 || v > (UINT64_MAX - d) / 10) return false;
      v = v * 10 + d;
      j++;
    }
    f(k++, v);
    i = j;
  }
  return true;
}

int parse_text(byo_ctx *ctx, const std::vector<char> &buf, uint64_t *n_out, uint64_t *m_out, uint64_t *offsets,
               uint32_t *nbrs) {
  const char *s = buf.data();
  const size_t len = buf.size();
  size_t i = 0;
  while (i < len && is_space(s[i])) i++;
  const size_t hl = sizeof(kHeader) - 1;
  if (len - i < hl || std::memcmp(s + i, kHeader, hl) != 0 || (i + hl < len && !is_space(s[i + hl])))
    return set_error(ctx, BYO_EINVAL, "graph file: missing AdjacencyGraph header");
  i += hl;
  uint64_t nm[2] = {0, 0};
  int got = 0;
  while (got < 2) {
    while (i < len && is_space(s[i])) i++;
    size_t j = i;
    while (j < len && !is_space(s[j])) j++;
    if (j == i) return set_error(ctx, BYO_EINVAL, "graph file: missing n or m");
    bool ok = parse_range(s, i, j, 0, [&](uint64_t, uint64_t v) { nm[got] = v; });
    if (!ok) return set_error(ctx, BYO_EINVAL, "graph file: n or m is not a number");
    got++;
    i = j;
  }
  const uint64_t n = nm[0], m = nm[1];
  if (n >= (1ull << 32) - 1) return set_error(ctx, BYO_EINVAL, "graph file: n does not fit 32-bit ids");
  *n_out = n;
  *m_out = m;
  if (!offsets) return BYO_OK;
  // chunks at whitespace boundaries
  unsigned nt = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
  const size_t body = len - i;
  if (body < (1u << 20)) nt = 1;
  std::vector<Chunk> ch(nt);
  size_t pos = i;
  for (unsigned t = 0; t < nt; t++) {
    size_t e = t + 1 == nt ? len : std::max(pos, i + body / nt * (t + 1));
    while (e < len && !is_space(s[e])) e++;
    ch[t].b = pos;
    ch[t].e = e;
    pos = e;
  }
  auto count = [&](Chunk &c) {
    bool in = false;
    for (size_t k = c.b; k < c.e; k++) {
      const bool sp = is_space(s[k]);
      if (!sp && !in) c.tokens++;
      in = !sp;
    }
  };
  {
    std::vector<std::thread> th;
    for (unsigned t = 1; t < nt; t++) th.emplace_back(count, std::ref(ch[t]));
    count(ch[0]);
    for (auto &x : th) x.join();
  }
  uint64_t total = 0;
  for (auto &c : ch) {
    c.first = total;
    total += c.tokens;
  }
  if (total < n + m) return set_error(ctx, BYO_EINVAL, "graph file: fewer than n + m numbers after the header");
  auto fill = [&](Chunk &c) {
    c.bad = !parse_range(s, c.b, c.e, c.first, [&](uint64_t k, uint64_t v) {
      if (k < n) offsets[k] = v;
      else if (k < n + m) nbrs[k - n] = v > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)v;
    });
  };
  {
    std::vector<std::thread> th;
    for (unsigned t = 1; t < nt; t++) th.emplace_back(fill, std::ref(ch[t]));
    fill(ch[0]);
    for (auto &x : th) x.join();
  }
  for (auto &c : ch)
    if (c.bad) return set_error(ctx, BYO_EINVAL, "graph file: a token is not a number");
  offsets[n] = m;
  return BYO_OK;
}

int parse_binary(byo_ctx *ctx, const char *path, uint64_t *n_out, uint64_t *m_out, uint64_t *offsets,
                 uint32_t *nbrs) {
  FILE *f = std::fopen(path, "rb");
  if (!f) return set_error(ctx, BYO_EINVAL, "graph file: cannot open");
  int64_t hdr[3];
  int rc = BYO_OK;
  if (std::fread(hdr, 8, 3, f) != 3 || hdr[0] < 0 || hdr[1] < 0)
    rc = set_error(ctx, BYO_EINVAL, "graph file: short binary header");
  else if ((uint64_t)hdr[0] >= (1ull << 32) - 1)
    rc = set_error(ctx, BYO_EINVAL, "graph file: n does not fit 32-bit ids");
  if (rc == BYO_OK) {
    *n_out = (uint64_t)hdr[0];
    *m_out = (uint64_t)hdr[1];
    if (offsets) {
      const uint64_t n = *n_out, m = *m_out;
      if (std::fread(offsets, 8, n + 1, f) != n + 1 || (m && std::fread(nbrs, 4, m, f) != m))
        rc = set_error(ctx, BYO_EINVAL, "graph file: binary body shorter than n and m say");
    }
  }
  std::fclose(f);
  return rc;
}

}  // namespace

int adj_read_host(byo_ctx *ctx, const char *path, int binary, uint64_t *n, uint64_t *m, uint64_t *offsets,
                  uint32_t *nbrs) {
  int rc;
  if (binary) {
    rc = parse_binary(ctx, path, n, m, offsets, nbrs);
  } else {
    std::vector<char> buf;
    if (!read_file(path, buf)) return set_error(ctx, BYO_EINVAL, "graph file: cannot read");
    rc = parse_text(ctx, buf, n, m, offsets, nbrs);
  }
  if (rc != BYO_OK || !offsets) return rc;
  // offsets from 0 to m, non-decreasing; ids below n
  if (offsets[0] != 0 || offsets[*n] != *m) return set_error(ctx, BYO_EINVAL, "graph file: offsets not 0 .. m");
  for (uint64_t i = 0; i < *n; i++)
    if (offsets[i + 1] < offsets[i]) return set_error(ctx, BYO_EINVAL, "graph file: offsets decrease");
  for (uint64_t j = 0; j < *m; j++)
    if (nbrs[j] >= *n) return set_error(ctx, BYO_EINVAL, "graph file: neighbour id >= n");
  return BYO_OK;
}

int adj_write_host(byo_ctx *ctx, const char *path, int binary, uint64_t n, uint64_t m, const uint64_t *offsets,
                   const uint32_t *nbrs) {
  FILE *f = std::fopen(path, "wb");
  if (!f) return set_error(ctx, BYO_EINVAL, "graph file: cannot create");
  bool ok = true;
  if (binary) {
    const int64_t hdr[3] = {(int64_t)n, (int64_t)m, (int64_t)(24 + 8 * (n + 1) + 4 * m)};
    ok = std::fwrite(hdr, 8, 3, f) == 3 && std::fwrite(offsets, 8, n + 1, f) == n + 1 &&
         (m == 0 || std::fwrite(nbrs, 4, m, f) == m);
  } else {
    // the dump of Graph::write_adj (gbbs/graph.h:3018-3044)
    std::string out;
    out.reserve(1 << 22);
    char tmp[32];
    auto put = [&](uint64_t v) {
      int k = 0;
      do {
        tmp[k++] = (char)('0' + v % 10);
        v /= 10;
      } while (v);
      while (k) out.push_back(tmp[--k]);
      out.push_back('\n');
      if (out.size() >= (1u << 22)) {
        ok = ok && std::fwrite(out.data(), 1, out.size(), f) == out.size();
        out.clear();
      }
    };
    out += kHeader;
    out.push_back('\n');
    put(n);
    put(m);
    for (uint64_t i = 0; i < n; i++) put(offsets[i]);
    for (uint64_t i = 0; i < m; i++) put(nbrs[i]);
    ok = ok && std::fwrite(out.data(), 1, out.size(), f) == out.size();
  }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? BYO_OK : set_error(ctx, BYO_EINVAL, "graph file: write failed");
}

}  // namespace byo
