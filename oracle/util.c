/*
 * Oracle utilities — TEST INFRASTRUCTURE (see oracle.h).
 * Transpose, pivot order, sequential reach/BFS, iterative Tarjan and
 * partition canonicalisation.
 */
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#include "common.h"
#include "oracle.h"

void orc_vec_push(orc_vec* v, uint32_t x) {
  if (v->n == v->cap) {
    v->cap = v->cap ? v->cap * 2 : 1024;
    v->a = (uint32_t*)realloc(v->a, v->cap * sizeof(uint32_t));
  }
  v->a[v->n++] = x;
}

size_t orc_vec_gather(orc_vec* vs, int nt, uint32_t* out) {
  size_t* pre = (size_t*)malloc(sizeof(size_t) * (nt + 1));
  pre[0] = 0;
  for (int t = 0; t < nt; t++) pre[t + 1] = pre[t] + vs[t].n;
#pragma omp parallel for schedule(static, 1)
  for (int t = 0; t < nt; t++) {
    if (vs[t].n) memcpy(out + pre[t], vs[t].a, vs[t].n * sizeof(uint32_t));
    vs[t].n = 0;
  }
  size_t total = pre[nt];
  free(pre);
  return total;
}

void orc_vec_free(orc_vec* vs, int nt) {
  for (int t = 0; t < nt; t++) free(vs[t].a);
  free(vs);
}

uint64_t orc_perm_at(uint64_t i, uint64_t k, uint64_t seed) { return orc_perm(i, k, seed); }
uint32_t orc_hash32_at(uint32_t x) { return orc_hash32(x); }
uint64_t orc_hash64_at(uint64_t x) { return orc_hash64(x); }

/* src/graph.hpp:222-245: the reference sorts (target, source) pairs; a
 * counting sort by target that walks sources in increasing order gives the
 * same in-lists (sorted by source). */
void orc_transpose(uint64_t n, uint64_t m, const uint64_t* off, const uint32_t* E,
                   uint64_t* in_off, uint32_t* in_E) {
  memset(in_off, 0, sizeof(uint64_t) * (n + 1));
  for (uint64_t j = 0; j < m; j++) in_off[E[j] + 1]++;
  for (uint64_t v = 0; v < n; v++) in_off[v + 1] += in_off[v];
  uint64_t* cur = (uint64_t*)malloc(sizeof(uint64_t) * (n ? n : 1));
  memcpy(cur, in_off, sizeof(uint64_t) * n);
  for (uint64_t u = 0; u < n; u++)
    for (uint64_t j = off[u]; j < off[u + 1]; j++) in_E[cur[E[j]]++] = (uint32_t)u;
  free(cur);
}

/* src/scc.hpp:295-303: NON_ZEROS = vertices with in- and out-degree > 0, in
 * id order; P = NON_ZEROS permuted (Feistel bijection, see common.h). */
uint64_t orc_pivot_order(uint64_t n, const uint64_t* off, const uint64_t* in_off,
                         uint64_t seed, uint32_t* P, uint64_t* n_zeros) {
  uint32_t* nz = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1));
  uint64_t k = 0;
  for (uint64_t v = 0; v < n; v++)
    if (off[v + 1] != off[v] && in_off[v + 1] != in_off[v]) nz[k++] = (uint32_t)v;
#pragma omp parallel for
  for (uint64_t i = 0; i < k; i++) P[i] = nz[orc_perm(i, k, seed)];
  free(nz);
  if (n_zeros) *n_zeros = n - k;
  return k;
}

/* src/reach.hpp:57-74 */
void orc_reach_seq(uint64_t n, const uint64_t* off, const uint32_t* E, uint32_t src,
                   uint8_t* dst) {
  memset(dst, 0, n);
  uint32_t* q = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1));
  uint64_t h = 0, t = 0;
  q[t++] = src;
  dst[src] = 1;
  while (h < t) {
    uint32_t u = q[h++];
    for (uint64_t j = off[u]; j < off[u + 1]; j++) {
      uint32_t v = E[j];
      if (!dst[v]) {
        dst[v] = 1;
        q[t++] = v;
      }
    }
  }
  free(q);
}

/* src/bfs.hpp:59-76 */
void orc_bfs_seq(uint64_t n, const uint64_t* off, const uint32_t* E, uint32_t src,
                 uint32_t* dist) {
  for (uint64_t i = 0; i < n; i++) dist[i] = ORC_NMAX;
  uint32_t* q = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1));
  uint64_t h = 0, t = 0;
  q[t++] = src;
  dist[src] = 0;
  while (h < t) {
    uint32_t u = q[h++];
    for (uint64_t j = off[u]; j < off[u + 1]; j++) {
      uint32_t v = E[j];
      if (dist[v] == ORC_NMAX) {
        dist[v] = dist[u] + 1;
        q[t++] = v;
      }
    }
  }
  free(q);
}

/* baselines/tarjan_scc/tarjan_scc.hpp:39-76, with the recursion replaced by
 * an explicit frame stack; the low-link update after a child returns happens
 * when the child's frame is popped, so labels match the recursive order. */
uint32_t orc_tarjan(uint64_t n, const uint64_t* off, const uint32_t* E, uint32_t* scc) {
  uint32_t* low = (uint32_t*)calloc(n ? n : 1, sizeof(uint32_t));
  uint32_t* dfn = (uint32_t*)calloc(n ? n : 1, sizeof(uint32_t));
  uint64_t* ep = (uint64_t*)malloc(sizeof(uint64_t) * (n ? n : 1));
  uint32_t* cs = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1)); /* call stack */
  uint32_t* sk = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1)); /* tarjan stack */
  memset(scc, 0, sizeof(uint32_t) * n);
  uint64_t ncs = 0, nsk = 0;
  uint32_t idx = 0, cnt = 0;
  for (uint64_t s = 0; s < n; s++) {
    if (dfn[s]) continue;
    low[s] = dfn[s] = ++idx;
    sk[nsk++] = (uint32_t)s;
    ep[s] = off[s];
    cs[ncs++] = (uint32_t)s;
    while (ncs) {
      uint32_t u = cs[ncs - 1];
      if (ep[u] < off[u + 1]) {
        uint32_t v = E[ep[u]++];
        if (!dfn[v]) {
          low[v] = dfn[v] = ++idx;
          sk[nsk++] = v;
          ep[v] = off[v];
          cs[ncs++] = v;
        } else if (!scc[v]) {
          if (dfn[v] < low[u]) low[u] = dfn[v];
        }
      } else {
        if (low[u] == dfn[u]) {
          cnt++;
          for (;;) {
            uint32_t x = sk[--nsk];
            scc[x] = cnt;
            if (x == u) break;
          }
        }
        ncs--;
        if (ncs) {
          uint32_t p = cs[ncs - 1];
          if (low[u] < low[p]) low[p] = low[u];
        }
      }
    }
  }
  free(low);
  free(dfn);
  free(ep);
  free(cs);
  free(sk);
  return cnt;
}

/* Canonical form of a partition: each vertex gets the smallest vertex id of
 * its class.  Open-addressing map label -> first (= smallest) vertex. */
void orc_canon_u64(uint64_t n, const uint64_t* labels, uint32_t* out) {
  uint64_t cap = 1;
  while (cap < 2 * n + 2) cap <<= 1;
  uint64_t* key = (uint64_t*)malloc(sizeof(uint64_t) * cap);
  uint32_t* val = (uint32_t*)malloc(sizeof(uint32_t) * cap);
  uint8_t* used = (uint8_t*)calloc(cap, 1);
  for (uint64_t v = 0; v < n; v++) {
    uint64_t h = orc_hash64(labels[v]) & (cap - 1);
    while (used[h] && key[h] != labels[v]) h = (h + 1) & (cap - 1);
    if (!used[h]) {
      used[h] = 1;
      key[h] = labels[v];
      val[h] = (uint32_t)v;
    }
    out[v] = val[h];
  }
  free(key);
  free(val);
  free(used);
}

void orc_canon_u32(uint64_t n, const uint32_t* labels, uint32_t* out) {
  uint64_t* l64 = (uint64_t*)malloc(sizeof(uint64_t) * (n ? n : 1));
  for (uint64_t v = 0; v < n; v++) l64[v] = labels[v];
  orc_canon_u64(n, l64, out);
  free(l64);
}
