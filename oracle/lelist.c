/*
 * Oracle LE-lists — TEST INFRASTRUCTURE (see oracle.h).
 *
 * orc_lelist_seq restates the reference's sequential definition
 * (src/LeList.hpp:76-115): vertices in priority order run a BFS that only
 * records (target, priority, dist) when dist strictly improves on every
 * earlier priority.  orc_lelist_par restates the parallel algorithm
 * (src/LeList.hpp:127-328): a BFS from centers[0], then prefix-doubling
 * batches of multi-source BFS over (priority, vertex) pairs pruned by the
 * distances of earlier batches, a sort by (target, priority) and a filter to
 * strictly decreasing distances.  Output triples are (target, source vertex,
 * distance), u32 each, sorted by (target, priority).
 */
#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#include "common.h"
#include "oracle.h"

typedef struct {
  uint32_t t, p, d;
} trip;

typedef struct {
  trip* a;
  uint64_t n, cap;
} tvec;

static void tv_push(tvec* v, uint32_t t, uint32_t p, uint32_t d) {
  if (v->n == v->cap) {
    v->cap = v->cap ? v->cap * 2 : 4096;
    v->a = (trip*)realloc(v->a, v->cap * sizeof(trip));
  }
  v->a[v->n].t = t;
  v->a[v->n].p = p;
  v->a[v->n].d = d;
  v->n++;
}

/* Stable two-pass LSD counting sort by (t, p): p first, then t. */
static void sort_tp(trip* a, uint64_t len, uint64_t n) {
  trip* tmp = (trip*)malloc(sizeof(trip) * (len ? len : 1));
  uint64_t* cnt = (uint64_t*)calloc(n + 1, sizeof(uint64_t));
  for (int pass = 0; pass < 2; pass++) {
    memset(cnt, 0, sizeof(uint64_t) * (n + 1));
    for (uint64_t i = 0; i < len; i++) cnt[(pass ? a[i].t : a[i].p) + 1]++;
    for (uint64_t k = 0; k < n; k++) cnt[k + 1] += cnt[k];
    for (uint64_t i = 0; i < len; i++) tmp[cnt[pass ? a[i].t : a[i].p]++] = a[i];
    memcpy(a, tmp, sizeof(trip) * len);
  }
  free(cnt);
  free(tmp);
}

static int emit(const trip* a, uint64_t len, const uint32_t* perm, uint32_t* out, uint64_t cap,
                uint64_t* olen) {
  *olen = len;
  if (len > cap) return -1;
  for (uint64_t i = 0; i < len; i++) {
    out[3 * i] = a[i].t;
    out[3 * i + 1] = perm[a[i].p];
    out[3 * i + 2] = a[i].d;
  }
  return 0;
}

int orc_lelist_seq(uint64_t n, const uint64_t* off, const uint32_t* E, const uint32_t* perm,
                   uint32_t* out, uint64_t cap, uint64_t* len) {
  uint32_t* dist = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1));
  uint32_t* q = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1));
  for (uint64_t i = 0; i < n; i++) dist[i] = ORC_NMAX;
  tvec L = {0, 0, 0};
  for (uint64_t i = 0; i < n; i++) {
    uint64_t h = 0, t = 0;
    uint32_t c = perm[i];
    q[t++] = c;
    dist[c] = 0;
    tv_push(&L, c, (uint32_t)i, 0);
    while (h < t) {
      uint32_t u = q[h++];
      for (uint64_t j = off[u]; j < off[u + 1]; j++) {
        uint32_t w = E[j];
        if (dist[u] + 1 < dist[w]) {
          dist[w] = dist[u] + 1;
          tv_push(&L, w, (uint32_t)i, dist[w]);
          q[t++] = w;
        }
      }
    }
  }
  sort_tp(L.a, L.n, n);
  int rc = emit(L.a, L.n, perm, out, cap, len);
  free(L.a);
  free(dist);
  free(q);
  return rc;
}

/* (priority, vertex) pair set (src/resizable_set.hpp), open addressing on u64. */
typedef struct {
  uint64_t* s;
  uint64_t m;
} pset;

static void ps_make(pset* p, uint64_t need) {
  uint64_t m = 1024;
  while (m < 2 * need) m <<= 1;
  free(p->s);
  p->s = (uint64_t*)malloc(sizeof(uint64_t) * m);
  p->m = m;
#pragma omp parallel for
  for (uint64_t i = 0; i < m; i++) p->s[i] = ~(uint64_t)0;
}

static int ps_insert(pset* p, uint64_t kv) {
  uint64_t h = orc_hash64(kv) & (p->m - 1);
  for (;;) {
    uint64_t c = orc_load64(&p->s[h]);
    if (c == kv) return 0;
    if (c == ~(uint64_t)0) {
      if (orc_cas64(&p->s[h], c, kv)) return 1;
      if (orc_load64(&p->s[h]) == kv) return 0;
    }
    h = (h + 1) & (p->m - 1);
  }
}

typedef struct {
  uint64_t* a;
  uint64_t n, cap;
} pvec;

static void pv_push(pvec* v, uint64_t x) {
  if (v->n == v->cap) {
    v->cap = v->cap ? v->cap * 2 : 1024;
    v->a = (uint64_t*)realloc(v->a, v->cap * sizeof(uint64_t));
  }
  v->a[v->n++] = x;
}

int orc_lelist_par(uint64_t n, const uint64_t* off, const uint32_t* E, const uint32_t* perm,
                   double beta, uint32_t* out, uint64_t cap, uint64_t* len, int nthreads) {
  if (nthreads <= 0) nthreads = omp_get_max_threads();
  if (n == 0) {
    *len = 0;
    return 0;
  }
  uint32_t* dist = (uint32_t*)malloc(sizeof(uint32_t) * n);
  uint32_t* next_dist = (uint32_t*)malloc(sizeof(uint32_t) * n);
  tvec L = {0, 0, 0};
  /* first round: BFS from centers[0] (LeList.hpp:232-253) */
  orc_bfs_seq(n, off, E, perm[0], dist);
  for (uint64_t i = 0; i < n; i++) {
    next_dist[i] = dist[i];
    if (dist[i] != ORC_NMAX) tv_push(&L, (uint32_t)i, 0, dist[i]);
  }
  pvec* loc = (pvec*)calloc(nthreads, sizeof(pvec));
  uint64_t* front = NULL;
  uint64_t fcap = 0;
  pset set = {0, 0};
  uint64_t step = 1, finished = 1;
  uint64_t table_m = n >> 1;
  while (finished != n) { /* LeList.hpp:259-276 */
    step = (uint64_t)ceil((double)(uint32_t)step * beta);
    uint64_t end = finished + step < n ? finished + step : n;
    uint64_t start = finished, nf = end - start;
    /* multi_search, LeList.hpp:127-218 */
    if (table_m < nf) table_m = nf;
    ps_make(&set, table_m);
    if (fcap < nf) {
      fcap = nf;
      front = (uint64_t*)realloc(front, sizeof(uint64_t) * fcap);
    }
    for (uint64_t i = start; i < end; i++) {
      uint64_t pr = ((uint64_t)i << 32) | perm[i];
      front[i - start] = pr;
      ps_insert(&set, pr);
      next_dist[perm[i]] = 0;
      tv_push(&L, perm[i], (uint32_t)i, 0);
    }
    uint64_t sub_n = nf, ne = nf;
    uint32_t sub_round = 0;
    while (sub_n > 0) {
      sub_round++;
      /* grow the set so every possible insert fits (maybe_resize) */
      uint64_t sum = 0;
#pragma omp parallel for reduction(+ : sum) num_threads(nthreads)
      for (uint64_t i = 0; i < sub_n; i++) {
        uint32_t v = (uint32_t)front[i];
        sum += off[v + 1] - off[v];
      }
      if (2 * (ne + sum) > set.m) {
        pset ns = {0, 0};
        ps_make(&ns, ne + sum);
        for (uint64_t i = 0; i < set.m; i++)
          if (set.s[i] != ~(uint64_t)0) ps_insert(&ns, set.s[i]);
        free(set.s);
        set = ns;
      }
#pragma omp parallel num_threads(nthreads)
      {
        pvec* b = &loc[omp_get_thread_num()];
#pragma omp for schedule(dynamic, 64)
        for (uint64_t i = 0; i < sub_n; i++) {
          uint64_t lab = front[i] >> 32;
          uint32_t u = (uint32_t)front[i];
          for (uint64_t j = off[u]; j < off[u + 1]; j++) {
            uint32_t w = E[j];
            if (sub_round < dist[w]) {
              uint64_t com = (lab << 32) | w;
              if (ps_insert(&set, com)) {
                pv_push(b, com);
                if (orc_load32(&next_dist[w]) > sub_round)
                  __atomic_store_n(&next_dist[w], sub_round, __ATOMIC_RELAXED);
              }
            }
          }
        }
      }
      uint64_t tot = 0;
      for (int t = 0; t < nthreads; t++) tot += loc[t].n;
      if (fcap < tot) {
        fcap = tot;
        front = (uint64_t*)realloc(front, sizeof(uint64_t) * fcap);
      }
      uint64_t k = 0;
      for (int t = 0; t < nthreads; t++) {
        memcpy(front + k, loc[t].a, loc[t].n * sizeof(uint64_t));
        k += loc[t].n;
        loc[t].n = 0;
      }
      sub_n = tot;
      ne += tot;
      for (uint64_t i = 0; i < sub_n; i++)
        tv_push(&L, (uint32_t)front[i], (uint32_t)(front[i] >> 32), sub_round);
    }
    table_m = ne;
    memcpy(dist, next_dist, sizeof(uint32_t) * n);
    finished += nf;
    table_m = (uint64_t)ceil((double)table_m * beta);
  }
  /* sort by (target, priority) and keep strictly decreasing distances
   * (LeList.hpp:278-327) */
  sort_tp(L.a, L.n, n);
  uint64_t k = 0;
  for (uint64_t i = 0; i < L.n;) {
    uint64_t j;
    uint32_t tgt = L.a[i].t, best = L.a[i].d;
    L.a[k++] = L.a[i];
    for (j = i + 1; j < L.n && L.a[j].t == tgt; j++) {
      if (L.a[j].d < best) {
        best = L.a[j].d;
        L.a[k++] = L.a[j];
      }
    }
    i = j;
  }
  int rc = emit(L.a, k, perm, out, cap, len);
  for (int t = 0; t < nthreads; t++) free(loc[t].a);
  free(loc);
  free(front);
  free(set.s);
  free(L.a);
  free(dist);
  free(next_dist);
  return rc;
}
