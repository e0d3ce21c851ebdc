// Graph file ingest (host side): the two formats the reference's drivers
// read (internal/helpers.hpp:379-657), parsed into interleaved (row, col)
// pairs, and a loader that builds a device graph from them with the same
// batch insert the reference's drivers use (internal/test.hpp:427-450).
//
//  - Matrix Market (.mtx): "%%MatrixMarket matrix coordinate <field>
//    <symmetry>", field integer / real / pattern, symmetry symmetric or
//    general; '%' comment lines after the first line; then "rows cols m"
//    and m entries (2 tokens for pattern, 3 otherwise; values ignored).
//    Ids are one-based; every entry (a, b) yields (a-1, b-1) and (b-1, a-1)
//    in file order, as helpers.hpp:512-521 does.  Rows must equal cols.
//  - PBBS adjacency (.adj, .adj.shuf): "AdjacencyGraph" or
//    "WeightedAdjacencyGraph", n, m, n offsets, m targets (and m weights,
//    ignored); row i's targets in order, not symmetrised (helpers.hpp:588-602).
// Malformed input is an SST_EINVAL with a message (the reference exits).
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "graph.cuh"

namespace {

using sst::set_error_message;

bool ends_with(const std::string &s, const char *suf) {
  size_t k = strlen(suf);
  return s.size() >= k && s.compare(s.size() - k, k, suf) == 0;
}

bool read_file(const char *path, std::string *out) {
  FILE *f = fopen(path, "rb");
  if (!f) return false;
  std::string s;
  char buf[1 << 16];
  size_t k;
  while ((k = fread(buf, 1, sizeof(buf), f)) > 0) s.append(buf, k);
  fclose(f);
  *out = std::move(s);
  return true;
}

inline bool is_space(char c) {
  return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\f' || c == '\v';
}

// whitespace-separated tokens of s from position `from`
std::vector<std::pair<size_t, size_t>> tokens(const std::string &s, size_t from) {
  std::vector<std::pair<size_t, size_t>> t;
  size_t i = from, n = s.size();
  while (i < n) {
    while (i < n && (is_space(s[i]) || s[i] == 0)) i++;
    if (i >= n) break;
    size_t b = i;
    while (i < n && !is_space(s[i]) && s[i] != 0) i++;
    t.emplace_back(b, i - b);
  }
  return t;
}

bool tok_is(const std::string &s, std::pair<size_t, size_t> t, const char *w) {
  return t.second == strlen(w) && s.compare(t.first, t.second, w) == 0;
}

bool tok_u64(const std::string &s, std::pair<size_t, size_t> t, uint64_t *v) {
  if (t.second == 0 || t.second > 20) return false;
  uint64_t x = 0;
  for (size_t i = 0; i < t.second; i++) {
    char c = s[t.first + i];
    if (c < '0' || c > '9') return false;
    x = x * 10 + (uint64_t)(c - '0');
  }
  *v = x;
  return true;
}

sst_status parse_mtx(std::string &s, uint32_t *rows,
                     std::vector<uint32_t> *pairs) {
  // comment lines after the first line start with '%'
  size_t i = s.find('\n');
  if (i == std::string::npos) {
    set_error_message("bad mtx file: no line breaks");
    return SST_EINVAL;
  }
  i++;
  while (i < s.size() && s[i] == '%') {
    while (i < s.size() && s[i] != '\n') s[i++] = ' ';
    i++;
  }
  auto t = tokens(s, 0);
  if (t.size() < 8 || !tok_is(s, t[0], "%%MatrixMarket")) {
    set_error_message("bad mtx file: missing %%%%MatrixMarket header");
    return SST_EINVAL;
  }
  if (!tok_is(s, t[1], "matrix") || !tok_is(s, t[2], "coordinate")) {
    set_error_message("mtx: only 'matrix coordinate' files are read");
    return SST_EINVAL;
  }
  const bool pattern = tok_is(s, t[3], "pattern");
  if (!pattern && !tok_is(s, t[3], "integer") && !tok_is(s, t[3], "real")) {
    set_error_message("mtx: field must be integer, real or pattern");
    return SST_EINVAL;
  }
  if (!tok_is(s, t[4], "symmetric") && !tok_is(s, t[4], "general")) {
    set_error_message("mtx: only symmetric and general files are read");
    return SST_EINVAL;
  }
  uint64_t r = 0, c = 0, m = 0;
  if (!tok_u64(s, t[5], &r) || !tok_u64(s, t[6], &c) || !tok_u64(s, t[7], &m)) {
    set_error_message("mtx: bad size line");
    return SST_EINVAL;
  }
  const uint64_t per = pattern ? 2 : 3;
  if (t.size() - 8 != m * per) {
    set_error_message("mtx: %llu entry tokens for m = %llu",
                      (unsigned long long)(t.size() - 8), (unsigned long long)m);
    return SST_EINVAL;
  }
  if (r != c) {
    set_error_message("mtx: matrix is not square (%llu x %llu)",
                      (unsigned long long)r, (unsigned long long)c);
    return SST_EINVAL;
  }
  if (r >= 0xFFFFFFFFull) {
    set_error_message("mtx: too many rows for uint32 ids");
    return SST_EINVAL;
  }
  pairs->resize(4 * m);
  for (uint64_t k = 0; k < m; k++) {
    uint64_t a = 0, b = 0;
    if (!tok_u64(s, t[8 + k * per], &a) || !tok_u64(s, t[9 + k * per], &b) ||
        a == 0 || b == 0 || a > r || b > r) {
      set_error_message("mtx: bad entry %llu", (unsigned long long)k);
      return SST_EINVAL;
    }
    (*pairs)[4 * k] = (uint32_t)(a - 1);
    (*pairs)[4 * k + 1] = (uint32_t)(b - 1);
    (*pairs)[4 * k + 2] = (uint32_t)(b - 1);
    (*pairs)[4 * k + 3] = (uint32_t)(a - 1);
  }
  *rows = (uint32_t)r;
  return SST_OK;
}

sst_status parse_adj(const std::string &s, uint32_t *rows,
                     std::vector<uint32_t> *pairs) {
  auto t = tokens(s, 0);
  if (t.empty() || (!tok_is(s, t[0], "AdjacencyGraph") &&
                    !tok_is(s, t[0], "WeightedAdjacencyGraph"))) {
    set_error_message("bad adj file: missing AdjacencyGraph header");
    return SST_EINVAL;
  }
  uint64_t n = 0, m = 0;
  if (t.size() < 3 || !tok_u64(s, t[1], &n) || !tok_u64(s, t[2], &m) || n == 0 ||
      m == 0) {
    set_error_message("adj: no vertices or no edges");
    return SST_EINVAL;
  }
  const uint64_t len = t.size() - 1;
  if (len != n + m + 2 && len != n + 2 * m + 2) {
    set_error_message("adj: %llu numbers for n = %llu, m = %llu",
                      (unsigned long long)len, (unsigned long long)n,
                      (unsigned long long)m);
    return SST_EINVAL;
  }
  if (n >= 0xFFFFFFFFull) {
    set_error_message("adj: too many vertices for uint32 ids");
    return SST_EINVAL;
  }
  std::vector<uint64_t> off(n + 1);
  for (uint64_t i = 0; i < n; i++)
    if (!tok_u64(s, t[3 + i], &off[i])) {
      set_error_message("adj: bad offset %llu", (unsigned long long)i);
      return SST_EINVAL;
    }
  off[n] = m;
  pairs->resize(2 * m);
  for (uint64_t i = 0; i < n; i++) {
    if (off[i] > off[i + 1] || off[i + 1] > m) {
      set_error_message("adj: offsets not increasing at %llu", (unsigned long long)i);
      return SST_EINVAL;
    }
    for (uint64_t j = off[i]; j < off[i + 1]; j++) {
      uint64_t d = 0;
      if (!tok_u64(s, t[3 + n + j], &d) || d >= n) {
        set_error_message("adj: bad edge %llu", (unsigned long long)j);
        return SST_EINVAL;
      }
      (*pairs)[2 * j] = (uint32_t)i;
      (*pairs)[2 * j + 1] = (uint32_t)d;
    }
  }
  *rows = (uint32_t)n;
  return SST_OK;
}

sst_status read_pairs(const char *path, uint32_t *rows,
                      std::vector<uint32_t> *pairs) {
  if (!path || !rows) {
    set_error_message("null argument");
    return SST_EINVAL;
  }
  std::string p(path), s;
  const bool mtx = ends_with(p, ".mtx");
  if (!mtx && !ends_with(p, ".adj") && !ends_with(p, ".adj.shuf")) {
    set_error_message("unknown graph file format (.mtx, .adj, .adj.shuf): %s", path);
    return SST_EINVAL;
  }
  if (!read_file(path, &s)) {
    set_error_message("cannot read %s: %s", path, strerror(errno));
    return SST_EINVAL;
  }
  if (s.empty()) {
    set_error_message("%s is empty", path);
    return SST_EINVAL;
  }
  return mtx ? parse_mtx(s, rows, pairs) : parse_adj(s, rows, pairs);
}

}  // namespace

extern "C" {

sst_status sst_read_graph_file(const char *path, uint32_t *rows,
                               uint64_t *n_pairs, uint32_t **pairs) {
  if (!n_pairs || !pairs) {
    set_error_message("null argument");
    return SST_EINVAL;
  }
  *pairs = nullptr;
  *n_pairs = 0;
  std::vector<uint32_t> v;
  sst_status st = read_pairs(path, rows, &v);
  if (st != SST_OK) return st;
  uint32_t *out = static_cast<uint32_t *>(malloc(v.empty() ? 4 : v.size() * 4));
  if (!out) return SST_ENOMEM;
  if (!v.empty()) memcpy(out, v.data(), v.size() * 4);
  *pairs = out;
  *n_pairs = v.size() / 2;
  return SST_OK;
}

void sst_free(void *p) { free(p); }

sst_status sst_load_graph_file(const char *path, const sst_config *cfg,
                               sst_graph **out) {
  if (!out) {
    set_error_message("null output handle");
    return SST_EINVAL;
  }
  *out = nullptr;
  uint32_t rows = 0;
  std::vector<uint32_t> v;
  sst_status st = read_pairs(path, &rows, &v);
  if (st != SST_OK) return st;
  sst_graph *g = nullptr;
  st = sst_graph_create(rows, rows, cfg, &g);
  if (st != SST_OK) return st;
  uint64_t bad = 0;
  st = sst_insert_batch(g, v.data(), v.size() / 2, SST_HOST_PTR, &bad);
  if (st != SST_OK) {
    sst_graph_destroy(g);
    return st;
  }
  *out = g;
  return SST_OK;
}

}  // extern "C"
