// Host-side graph construction (libpsc_host.so): seeded generators, CSR and
// transpose building, symmetrisation and GBBS .bin I/O.  C++17 + OpenMP.
// Declared in include/psc_host.h.
#include <omp.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/psc_host.h"
#include "psc_hash.h"

struct psc_hgraph_s {
  uint64_t n = 0, m = 0;
  std::vector<uint64_t> off;
  std::vector<uint32_t> E;
  std::vector<uint64_t> in_off;
  std::vector<uint32_t> in_E;
  bool symmetric = false;
  bool has_transpose = false;
};

namespace {

thread_local std::string g_err;

void set_err(const std::string& s) { g_err = s; }

// Exclusive prefix sum in place over cnt[0..n], result cnt[n] = total.
void scan_inplace(std::vector<uint64_t>& a) {
  uint64_t s = 0;
  for (auto& x : a) {
    uint64_t t = x;
    x = s;
    s += t;
  }
}

// Builds a sorted, deduplicated CSR from per-source buckets produced by a
// counting sort of (src, dst) pairs.
psc_hgraph_t csr_from_pairs(uint64_t n, uint64_t m, const uint32_t* src, const uint32_t* dst,
                            bool drop_self) {
  auto* g = new psc_hgraph_s();
  g->n = n;
  std::vector<uint64_t> cnt(n + 1, 0);
  {
    std::vector<std::atomic<uint64_t>> acnt(n);
#pragma omp parallel for
    for (int64_t i = 0; i < (int64_t)n; i++) acnt[i].store(0, std::memory_order_relaxed);
#pragma omp parallel for
    for (int64_t e = 0; e < (int64_t)m; e++) {
      if (src[e] >= n || dst[e] >= n) continue;
      if (drop_self && src[e] == dst[e]) continue;
      acnt[src[e]].fetch_add(1, std::memory_order_relaxed);
    }
    for (uint64_t i = 0; i < n; i++) cnt[i] = acnt[i].load(std::memory_order_relaxed);
  }
  scan_inplace(cnt);
  uint64_t tot = cnt[n];
  std::vector<uint32_t> tmp(tot);
  {
    std::vector<std::atomic<uint64_t>> cur(n);
#pragma omp parallel for
    for (int64_t i = 0; i < (int64_t)n; i++) cur[i].store(cnt[i], std::memory_order_relaxed);
#pragma omp parallel for
    for (int64_t e = 0; e < (int64_t)m; e++) {
      if (src[e] >= n || dst[e] >= n) continue;
      if (drop_self && src[e] == dst[e]) continue;
      tmp[cur[src[e]].fetch_add(1, std::memory_order_relaxed)] = dst[e];
    }
  }
  // sort + unique each bucket, then compact
  std::vector<uint64_t> deg(n + 1, 0);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t u = 0; u < (int64_t)n; u++) {
    uint32_t* b = tmp.data() + cnt[u];
    uint32_t* e = tmp.data() + cnt[u + 1];
    std::sort(b, e);
    deg[u] = (uint64_t)(std::unique(b, e) - b);
  }
  g->off.assign(n + 1, 0);
  for (uint64_t u = 0; u < n; u++) g->off[u + 1] = g->off[u] + deg[u];
  g->m = g->off[n];
  g->E.resize(g->m);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t u = 0; u < (int64_t)n; u++)
    std::memcpy(g->E.data() + g->off[u], tmp.data() + cnt[u], deg[u] * sizeof(uint32_t));
  return g;
}

}  // namespace

extern "C" {

const char* psc_host_last_error(void) { return g_err.c_str(); }

psc_hgraph_t psc_hgraph_from_edges(uint64_t n, uint64_t m, const uint32_t* src,
                                   const uint32_t* dst, int drop_self) {
  if (n >= 0xFFFFFFFFull) {
    set_err("n must be below 2^32-1 (u32 vertex ids)");
    return nullptr;
  }
  return csr_from_pairs(n, m, src, dst, drop_self != 0);
}

psc_hgraph_t psc_hgraph_from_csr(uint64_t n, uint64_t m, const uint64_t* off, const uint32_t* E) {
  if (n >= 0xFFFFFFFFull) {
    set_err("n must be below 2^32-1 (u32 vertex ids)");
    return nullptr;
  }
  if (off[0] != 0 || off[n] != m) {
    set_err("offsets must start at 0 and end at m");
    return nullptr;
  }
  for (uint64_t i = 0; i < n; i++)
    if (off[i + 1] < off[i]) {
      set_err("offsets must be non-decreasing");
      return nullptr;
    }
  for (uint64_t j = 0; j < m; j++)
    if (E[j] >= n) {
      set_err("edge target out of range");
      return nullptr;
    }
  auto* g = new psc_hgraph_s();
  g->n = n;
  g->m = m;
  g->off.assign(off, off + n + 1);
  g->E.assign(E, E + m);
  return g;
}

psc_hgraph_t psc_hgraph_rmat(uint32_t log2n, uint64_t draws, double a, double b, double c,
                             uint64_t seed) {
  if (log2n == 0 || log2n > 31) {
    set_err("log2n must be in [1, 31]");
    return nullptr;
  }
  uint64_t n = 1ull << log2n;
  std::vector<uint32_t> src(draws), dst(draws);
  const double ab = a + b, abc = a + b + c;
#pragma omp parallel for schedule(static, 65536)
  for (int64_t e = 0; e < (int64_t)draws; e++) {
    uint32_t u = 0, v = 0;
    for (uint32_t l = 0; l < log2n; l++) {
      double r = psc::rng_unit(seed, (uint64_t)e * 64 + l);
      uint32_t bu = r >= ab ? 1u : 0u;
      uint32_t bv = (r >= a && r < ab) || r >= abc ? 1u : 0u;
      u = (u << 1) | bu;
      v = (v << 1) | bv;
    }
    src[e] = u;
    dst[e] = v;
  }
  return csr_from_pairs(n, draws, src.data(), dst.data(), true);
}

psc_hgraph_t psc_hgraph_knn(uint64_t npts, uint32_t k, uint64_t seed) {
  if (npts == 0 || npts >= 0xFFFFFFFFull) {
    set_err("npts must be in [1, 2^32-1)");
    return nullptr;
  }
  const uint64_t n = npts;
  std::vector<double> X(n), Y(n);
#pragma omp parallel for
  for (int64_t i = 0; i < (int64_t)n; i++) {
    X[i] = psc::rng_unit(seed, 2 * (uint64_t)i);
    Y[i] = psc::rng_unit(seed, 2 * (uint64_t)i + 1);
  }
  uint64_t G = (uint64_t)std::floor(std::sqrt((double)n / 2.0));
  if (G < 1) G = 1;
  const double h = 1.0 / (double)G;
  auto cell_of = [&](double x) {
    uint64_t c = (uint64_t)(x * (double)G);
    return c >= G ? G - 1 : c;
  };
  std::vector<uint64_t> cstart(G * G + 1, 0);
  std::vector<uint32_t> cell(n);
  for (uint64_t i = 0; i < n; i++) {
    uint32_t id = (uint32_t)(cell_of(Y[i]) * G + cell_of(X[i]));
    cell[i] = id;
    cstart[id + 1]++;
  }
  for (uint64_t c = 0; c < G * G; c++) cstart[c + 1] += cstart[c];
  std::vector<uint32_t> pts(n);
  {
    std::vector<uint64_t> cur(cstart.begin(), cstart.end() - 1);
    for (uint64_t i = 0; i < n; i++) pts[cur[cell[i]]++] = (uint32_t)i;
  }
  const uint32_t kk = (uint32_t)std::min<uint64_t>(k, n - 1);
  std::vector<uint32_t> nbr(n * (uint64_t)kk);
#pragma omp parallel
  {
    std::vector<std::pair<double, uint32_t>> best;
    best.reserve(kk + 1);
#pragma omp for schedule(dynamic, 4096)
    for (int64_t ii = 0; ii < (int64_t)n; ii++) {
      const uint32_t i = (uint32_t)ii;
      best.clear();
      const int64_t cx = (int64_t)cell_of(X[i]), cy = (int64_t)cell_of(Y[i]);
      auto consider = [&](uint32_t j) {
        if (j == i) return;
        double dx = X[j] - X[i], dy = Y[j] - Y[i];
        std::pair<double, uint32_t> c(dx * dx + dy * dy, j);
        if (best.size() < kk) {
          best.push_back(c);
          std::push_heap(best.begin(), best.end());
        } else if (c < best.front()) {
          std::pop_heap(best.begin(), best.end());
          best.back() = c;
          std::push_heap(best.begin(), best.end());
        }
      };
      for (int64_t r = 0;; r++) {
        for (int64_t dy = -r; dy <= r; dy++) {
          int64_t y = cy + dy;
          if (y < 0 || y >= (int64_t)G) continue;
          bool edge_row = (dy == -r || dy == r);
          for (int64_t dx = -r; dx <= r; dx += (edge_row ? 1 : 2 * r)) {
            int64_t x = cx + dx;
            if (x >= 0 && x < (int64_t)G) {
              uint64_t c = (uint64_t)y * G + (uint64_t)x;
              for (uint64_t p = cstart[c]; p < cstart[c + 1]; p++) consider(pts[p]);
            }
            if (r == 0) break;
          }
        }
        // every point in a ring beyond r lies at least r*h away
        bool done = best.size() == kk && best.front().first <= (double)(r * r) * h * h;
        if (done || r > (int64_t)G) break;
      }
      std::sort(best.begin(), best.end());
      for (uint32_t t = 0; t < kk; t++) nbr[(uint64_t)i * kk + t] = best[t].second;
    }
  }
  std::vector<uint32_t> src(n * (uint64_t)kk);
#pragma omp parallel for
  for (int64_t e = 0; e < (int64_t)(n * kk); e++) src[e] = (uint32_t)(e / kk);
  return csr_from_pairs(n, n * kk, src.data(), nbr.data(), true);
}

psc_hgraph_t psc_hgraph_grid(uint32_t rows, uint32_t cols, double p_bidir, uint64_t seed) {
  uint64_t n = (uint64_t)rows * cols;
  if (n == 0 || n >= 0xFFFFFFFFull) {
    set_err("rows*cols must be in [1, 2^32-1)");
    return nullptr;
  }
  const uint64_t nh = (uint64_t)rows * (cols ? cols - 1 : 0);
  // lattice edge e joins a < b; returns the directions present
  // bit0: a->b, bit1: b->a
  auto dirs = [&](uint64_t e) -> uint32_t {
    uint32_t coin = (uint32_t)(psc::rng64(seed, 2 * e) & 1);
    bool both = psc::rng_unit(seed, 2 * e + 1) < p_bidir;
    return both ? 3u : (coin ? 2u : 1u);
  };
  auto* g = new psc_hgraph_s();
  g->n = n;
  std::vector<uint64_t> deg(n + 1, 0);
  auto for_out = [&](uint64_t v, auto&& emit) {
    uint64_t r = v / cols, c = v % cols;
    // neighbours in increasing id order: up, left, right, down
    if (r > 0) {  // vertical edge (r-1,c)-(r,c): a = up, b = v
      uint64_t e = nh + (r - 1) * cols + c;
      if (dirs(e) & 2u) emit((uint32_t)(v - cols));
    }
    if (c > 0) {  // horizontal (r,c-1)-(r,c): a = left, b = v
      uint64_t e = r * (cols - 1) + (c - 1);
      if (dirs(e) & 2u) emit((uint32_t)(v - 1));
    }
    if (c + 1 < cols) {  // (r,c)-(r,c+1): a = v
      uint64_t e = r * (cols - 1) + c;
      if (dirs(e) & 1u) emit((uint32_t)(v + 1));
    }
    if (r + 1 < rows) {  // (r,c)-(r+1,c): a = v
      uint64_t e = nh + r * cols + c;
      if (dirs(e) & 1u) emit((uint32_t)(v + cols));
    }
  };
#pragma omp parallel for schedule(static, 4096)
  for (int64_t v = 0; v < (int64_t)n; v++) {
    uint64_t d = 0;
    for_out((uint64_t)v, [&](uint32_t) { d++; });
    deg[v] = d;
  }
  g->off.assign(n + 1, 0);
  for (uint64_t v = 0; v < n; v++) g->off[v + 1] = g->off[v] + deg[v];
  g->m = g->off[n];
  g->E.resize(g->m);
#pragma omp parallel for schedule(static, 4096)
  for (int64_t v = 0; v < (int64_t)n; v++) {
    uint64_t p = g->off[v];
    for_out((uint64_t)v, [&](uint32_t w) { g->E[p++] = w; });
  }
  return g;
}

int psc_hgraph_build_transpose(psc_hgraph_t g) {
  if (!g) return -1;
  if (g->has_transpose) return 0;
  const uint64_t n = g->n, m = g->m;
  g->in_off.assign(n + 1, 0);
  g->in_E.resize(m);
  {
    std::vector<std::atomic<uint64_t>> cnt(n);
#pragma omp parallel for
    for (int64_t i = 0; i < (int64_t)n; i++) cnt[i].store(0, std::memory_order_relaxed);
#pragma omp parallel for
    for (int64_t j = 0; j < (int64_t)m; j++) cnt[g->E[j]].fetch_add(1, std::memory_order_relaxed);
    for (uint64_t v = 0; v < n; v++) g->in_off[v + 1] = g->in_off[v] + cnt[v].load();
  }
  // Sources are visited in increasing order per thread-chunk, so a plain
  // atomic-cursor scatter leaves lists unordered; sort each in-list after.
  {
    std::vector<std::atomic<uint64_t>> cur(n);
#pragma omp parallel for
    for (int64_t v = 0; v < (int64_t)n; v++) cur[v].store(g->in_off[v], std::memory_order_relaxed);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t u = 0; u < (int64_t)n; u++)
      for (uint64_t j = g->off[u]; j < g->off[u + 1]; j++)
        g->in_E[cur[g->E[j]].fetch_add(1, std::memory_order_relaxed)] = (uint32_t)u;
  }
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t v = 0; v < (int64_t)n; v++)
    std::sort(g->in_E.begin() + g->in_off[v], g->in_E.begin() + g->in_off[v + 1]);
  g->has_transpose = true;
  return 0;
}

psc_hgraph_t psc_hgraph_symmetrize(psc_hgraph_t g) {
  if (!g) return nullptr;
  if (psc_hgraph_build_transpose(g) != 0) return nullptr;
  const uint64_t n = g->n;
  auto* s = new psc_hgraph_s();
  s->n = n;
  std::vector<uint64_t> deg(n + 1, 0);
  auto merge = [&](uint64_t u, auto&& emit) {
    uint64_t i = g->off[u], ie = g->off[u + 1], j = g->in_off[u], je = g->in_off[u + 1];
    int64_t last = -1;
    while (i < ie || j < je) {
      uint32_t x;
      if (j >= je || (i < ie && g->E[i] <= g->in_E[j]))
        x = g->E[i++];
      else
        x = g->in_E[j++];
      if ((int64_t)x != last && x != u) emit(x);
      last = x;
    }
  };
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t u = 0; u < (int64_t)n; u++) {
    uint64_t d = 0;
    merge((uint64_t)u, [&](uint32_t) { d++; });
    deg[u] = d;
  }
  s->off.assign(n + 1, 0);
  for (uint64_t u = 0; u < n; u++) s->off[u + 1] = s->off[u] + deg[u];
  s->m = s->off[n];
  s->E.resize(s->m);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t u = 0; u < (int64_t)n; u++) {
    uint64_t p = s->off[u];
    merge((uint64_t)u, [&](uint32_t x) { s->E[p++] = x; });
  }
  s->symmetric = true;
  s->in_off = s->off;
  s->in_E = s->E;
  s->has_transpose = true;
  return s;
}

static bool read_csr_block(FILE* f, psc_hgraph_s* g, bool second) {
  uint64_t hdr[3];
  if (fread(hdr, sizeof(uint64_t), 3, f) != 3) return false;
  uint64_t n = hdr[0], m = hdr[1];
  if (hdr[2] != (n + 1) * 8 + m * 4 + 3 * 8) return false;
  if (second && (n != g->n || m != g->m)) return false;
  auto& off = second ? g->in_off : g->off;
  auto& E = second ? g->in_E : g->E;
  g->n = n;
  g->m = m;
  off.resize(n + 1);
  E.resize(m);
  if (fread(off.data(), sizeof(uint64_t), n + 1, f) != n + 1) return false;
  if (m && fread(E.data(), sizeof(uint32_t), m, f) != m) return false;
  return true;
}

psc_hgraph_t psc_hgraph_read_bin(const char* path) {
  FILE* f = fopen(path, "rb");
  if (!f) {
    set_err(std::string("Cannot open file ") + path);
    return nullptr;
  }
  auto* g = new psc_hgraph_s();
  bool ok = read_csr_block(f, g, false);
  if (ok && fgetc(f) != EOF) ok = false;
  fclose(f);
  if (!ok) {
    delete g;
    set_err(std::string("Bad data in ") + path);
    return nullptr;
  }
  return g;
}

psc_hgraph_t psc_hgraph_read_adj(const char* path) {
  FILE* f = fopen(path, "rb");
  if (!f) {
    set_err(std::string("Cannot open file ") + path);
    return nullptr;
  }
  std::string text;
  {
    char buf[1 << 16];
    size_t k;
    while ((k = fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, k);
    fclose(f);
  }
  // whitespace-separated words (src/graph.hpp:88-105)
  std::vector<const char*> words;
  for (size_t i = 0; i < text.size();) {
    while (i < text.size() && (text[i] == ' ' || text[i] == '\n' || text[i] == '\r' ||
                               text[i] == '\t' || text[i] == 0))
      text[i++] = 0;
    if (i < text.size()) words.push_back(&text[i]);
    while (i < text.size() && !(text[i] == ' ' || text[i] == '\n' || text[i] == '\r' ||
                                text[i] == '\t' || text[i] == 0))
      i++;
  }
  if (words.size() < 3) {
    set_err(std::string("Bad data in ") + path);
    return nullptr;
  }
  uint64_t n = strtoull(words[1], nullptr, 10), m = strtoull(words[2], nullptr, 10);
  if (words.size() < 3 + n + m || n >= 0xFFFFFFFFull) {
    set_err(std::string("Bad data in ") + path);
    return nullptr;
  }
  auto* g = new psc_hgraph_s();
  g->n = n;
  g->m = m;
  g->off.resize(n + 1);
  g->E.resize(m);
  for (uint64_t i = 0; i < n; i++) g->off[i] = strtoull(words[3 + i], nullptr, 10);
  g->off[n] = m;
  for (uint64_t j = 0; j < m; j++) g->E[j] = (uint32_t)strtoull(words[3 + n + j], nullptr, 10);
  for (uint64_t i = 0; i < n; i++)
    if (g->off[i + 1] < g->off[i]) {
      delete g;
      set_err(std::string("Bad offsets in ") + path);
      return nullptr;
    }
  return g;
}

psc_hgraph_t psc_hgraph_read_large(const char* path) {
  FILE* f = fopen(path, "rb");
  if (!f) {
    set_err(std::string("Cannot open file ") + path);
    return nullptr;
  }
  auto* g = new psc_hgraph_s();
  bool ok = read_csr_block(f, g, false) && read_csr_block(f, g, true);
  if (ok && fgetc(f) != EOF) ok = false;
  fclose(f);
  if (!ok) {
    delete g;
    set_err(std::string("Bad data in ") + path);
    return nullptr;
  }
  g->has_transpose = true;
  return g;
}

int psc_hgraph_write_bin(psc_hgraph_t g, const char* path) {
  if (!g) return -1;
  FILE* f = fopen(path, "wb");
  if (!f) {
    set_err(std::string("Cannot open file ") + path);
    return -1;
  }
  uint64_t hdr[3] = {g->n, g->m, (g->n + 1) * 8 + g->m * 4 + 3 * 8};
  bool ok = fwrite(hdr, sizeof(uint64_t), 3, f) == 3 &&
            fwrite(g->off.data(), sizeof(uint64_t), g->n + 1, f) == g->n + 1 &&
            (g->m == 0 || fwrite(g->E.data(), sizeof(uint32_t), g->m, f) == g->m);
  ok = (fclose(f) == 0) && ok;
  if (!ok) set_err(std::string("Write failed: ") + path);
  return ok ? 0 : -1;
}

uint64_t psc_hgraph_n(psc_hgraph_t g) { return g ? g->n : 0; }
uint64_t psc_hgraph_m(psc_hgraph_t g) { return g ? g->m : 0; }
const uint64_t* psc_hgraph_off(psc_hgraph_t g) { return g ? g->off.data() : nullptr; }
const uint32_t* psc_hgraph_E(psc_hgraph_t g) { return g ? g->E.data() : nullptr; }
const uint64_t* psc_hgraph_in_off(psc_hgraph_t g) {
  return g && g->has_transpose ? g->in_off.data() : nullptr;
}
const uint32_t* psc_hgraph_in_E(psc_hgraph_t g) {
  return g && g->has_transpose ? g->in_E.data() : nullptr;
}
void psc_hgraph_free(psc_hgraph_t g) { delete g; }

psc_hgraph_t psc_hgraph_pack(const psc_hgraph_t* graphs, uint32_t count, uint64_t* vbase_out) {
  if (!graphs || count == 0 || !vbase_out) {
    set_err("pack needs at least one graph and a vbase array");
    return nullptr;
  }
  std::vector<uint64_t> vb(count + 1, 0), eb(count + 1, 0);
  bool sym = true;
  for (uint32_t k = 0; k < count; k++) {
    if (!graphs[k]) {
      set_err("pack: null graph");
      return nullptr;
    }
    vb[k + 1] = vb[k] + graphs[k]->n;
    eb[k + 1] = eb[k] + graphs[k]->m;
    sym = sym && graphs[k]->symmetric;
  }
  if (vb[count] >= 0xFFFFFFFFull) {
    set_err("pack: more than 2^32-2 vertices");
    return nullptr;
  }
  for (uint32_t k = 0; k < count; k++)
    if (psc_hgraph_build_transpose(graphs[k]) != 0) return nullptr;
  auto* p = new psc_hgraph_s();
  p->n = vb[count];
  p->m = eb[count];
  p->off.resize(p->n + 1);
  p->E.resize(p->m);
  p->in_off.resize(p->n + 1);
  p->in_E.resize(p->m);
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t k = 0; k < (int64_t)count; k++) {
    const psc_hgraph_s* g = graphs[k];
    const uint64_t v0 = vb[k], e0 = eb[k];
    for (uint64_t i = 0; i < g->n; i++) {
      p->off[v0 + i] = e0 + g->off[i];
      p->in_off[v0 + i] = e0 + g->in_off[i];
    }
    for (uint64_t j = 0; j < g->m; j++) {
      p->E[e0 + j] = (uint32_t)(v0 + g->E[j]);
      p->in_E[e0 + j] = (uint32_t)(v0 + g->in_E[j]);
    }
  }
  p->off[p->n] = p->m;
  p->in_off[p->n] = p->m;
  p->symmetric = sym;
  p->has_transpose = true;
  std::copy(vb.begin(), vb.end(), vbase_out);
  return p;
}

// The batch workload: member k is seeded by seed0 + k; its size exponent u is
// uniform in [log2_min, log2_max) (a log-uniform vertex count).  Even members
// are R-MAT graphs with 2^round(u) vertices, 16 draws per vertex and
// (a, b, c) = (0.57, 0.19, 0.19); odd members are 2D kNN graphs with
// floor(2^u) points and k = 5.
int psc_batch_member_spec(uint32_t k, uint64_t seed0, double log2_min, double log2_max,
                          uint32_t* kind, uint64_t* size) {
  if (!(log2_max >= log2_min) || log2_min < 1 || log2_max > 31) return -1;
  const uint64_t seed = seed0 + k;
  const double u = log2_min + (log2_max - log2_min) * psc::rng_unit(seed, 0);
  if (k % 2 == 0) {
    if (kind) *kind = 0;
    if (size) *size = (uint64_t)std::llround(u);  // log2 of the vertex count
  } else {
    if (kind) *kind = 1;
    if (size) *size = std::max<uint64_t>(6, (uint64_t)std::floor(std::exp2(u)));
  }
  return 0;
}

psc_hgraph_t psc_hgraph_batch_member(uint32_t k, uint64_t seed0, double log2_min, double log2_max) {
  uint32_t kind = 0;
  uint64_t size = 0;
  if (psc_batch_member_spec(k, seed0, log2_min, log2_max, &kind, &size) != 0) {
    set_err("batch member: log2 range must lie in [1, 31]");
    return nullptr;
  }
  psc_hgraph_t g = kind == 0 ? psc_hgraph_rmat((uint32_t)size, 16ull << size, 0.57, 0.19, 0.19, seed0 + k)
                             : psc_hgraph_knn(size, 5, seed0 + k);
  if (g && psc_hgraph_build_transpose(g) != 0) {
    delete g;
    return nullptr;
  }
  return g;
}

psc_hgraph_t psc_hgraph_batch(uint32_t count, uint64_t seed0, double log2_min, double log2_max,
                              uint64_t* vbase_out) {
  if (count == 0 || !vbase_out) {
    set_err("batch: count must be positive");
    return nullptr;
  }
  std::vector<psc_hgraph_t> members(count, nullptr);
  // members in parallel; each member's own parallel loops run on its thread
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t k = 0; k < (int64_t)count; k++)
    members[k] = psc_hgraph_batch_member((uint32_t)k, seed0, log2_min, log2_max);
  psc_hgraph_t p = nullptr;
  bool ok = true;
  for (auto m : members) ok = ok && m != nullptr;
  if (ok)
    p = psc_hgraph_pack(members.data(), count, vbase_out);
  else
    set_err("batch: a member could not be generated");
  for (auto m : members) delete m;
  return p;
}

void psc_random_permutation(uint64_t n, uint64_t seed, uint32_t* out) {
  psc::FeistelKey f = psc::feistel_key(n, seed);
#pragma omp parallel for schedule(static, 65536)
  for (int64_t i = 0; i < (int64_t)n; i++) out[i] = (uint32_t)psc::feistel(f, (uint64_t)i);
}

}  // extern "C"
