/*
 * Oracle SCC — TEST INFRASTRUCTURE (see oracle.h).
 *
 * C11/OpenMP restatement of src/reach.hpp (REACH) and src/scc.hpp (SCC):
 * single-level trimming, first-pivot forward/backward reachability with the
 * push/pull switch and VGC local queues, prefix-doubling multi-search over a
 * (vertex, pivot) linear-probing multimap keyed by vertex, and the max-label
 * partition.  The hashbag frontier (src/hash_bag.h) is replaced by per-thread
 * vectors: only the frontier's vertex set matters to the result.
 */
#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#include "common.h"
#include "oracle.h"

/* Frontier vertices whose edge loop the reference runs as a nested
 * parallel_for are gathered and expanded edge-parallel in a second phase. */
#define ORC_HEAVY_DEG 4096

/* ------------------------------------------------------------------ */
/* REACH (src/reach.hpp:21-243)                                        */
/* ------------------------------------------------------------------ */
typedef struct {
  uint64_t n, m;
  const uint64_t *off, *in_off;
  const uint32_t *E, *in_E;
  uint32_t* front;
  uint8_t* dense_front;
  uint8_t* new_dense;
  uint64_t n_front, threshold, num_round;
  int sparse_pre;
  int nt;
  orc_vec* bag;
  uint32_t** lq; /* per-thread VGC queues */
  uint32_t tau;
} reach_t;

static void reach_sparse2dense(reach_t* r) { /* reach.hpp:76-79 */
  memset(r->dense_front, 0, r->n);
#pragma omp parallel for
  for (uint64_t i = 0; i < r->n_front; i++) r->dense_front[r->front[i]] = 1;
}

static void reach_dense2sparse(reach_t* r) { /* reach.hpp:81-84 */
  uint64_t k = 0;
  for (uint64_t v = 0; v < r->n; v++)
    if (r->dense_front[v]) r->front[k++] = (uint32_t)v;
}

static uint64_t reach_dense_sample(reach_t* r, uint32_t seed) { /* reach.hpp:192-206 */
  int count = 0;
  uint64_t out_edges = 0;
  uint32_t i = 0;
  while (count < 50) {
    i++;
    uint32_t idx = (uint32_t)(orc_hash32(seed + i) % r->n);
    if (r->dense_front[idx]) {
      count++;
      out_edges += r->off[idx + 1] - r->off[idx];
    }
  }
  return r->n_front * (out_edges / (uint64_t)count);
}

static int reach_judge(reach_t* r) { /* reach.hpp:86-112 */
  uint64_t front_out_edges = 0;
  int both = 0;
  if (!r->sparse_pre && r->n_front < (1u << 14)) {
    reach_dense2sparse(r);
    both = 1;
  }
  if (r->sparse_pre || both) {
    uint64_t s = 0;
#pragma omp parallel for reduction(+ : s)
    for (uint64_t i = 0; i < r->n_front; i++) {
      uint32_t u = r->front[i];
      s += r->off[u + 1] - r->off[u];
    }
    front_out_edges = s;
  } else {
    front_out_edges = reach_dense_sample(r, orc_hash32((uint32_t)r->num_round));
  }
  int sparse_now = (r->n_front + front_out_edges) < r->threshold;
  if (!both && r->sparse_pre != sparse_now) {
    if (!sparse_now)
      reach_sparse2dense(r);
    else
      reach_dense2sparse(r);
  }
  return sparse_now;
}

static uint64_t reach_sparse_update(reach_t* r, uint8_t* dst, int local) { /* reach.hpp:114-171 */
  const uint64_t* off = r->off;
  const uint32_t* E = r->E;
  uint64_t qsize = r->tau;
  orc_vec* heavy = (orc_vec*)calloc(r->nt, sizeof(orc_vec));
#pragma omp parallel num_threads(r->nt)
  {
    int tid = omp_get_thread_num();
    orc_vec* bag = &r->bag[tid];
    uint32_t* Q = r->lq[tid];
#pragma omp for schedule(dynamic, 64)
    for (uint64_t i = 0; i < r->n_front; i++) {
      uint32_t node = r->front[i];
      uint64_t cnt = 0;
      uint64_t deg_f = off[node + 1] - off[node];
      if (local && deg_f < qsize && deg_f > 0 && cnt < qsize) {
        uint64_t head = 0, tail = 0;
        Q[tail++] = node;
        while (head < tail && tail < qsize) {
          uint32_t u = Q[head++];
          uint64_t deg_u = off[u + 1] - off[u];
          if (deg_u > qsize) {
            orc_vec_push(bag, u);
            break;
          }
          for (uint64_t j = off[u]; j < off[u + 1]; j++) {
            uint32_t v = E[j];
            if (!orc_load8(&dst[v]) && orc_cas8(&dst[v], 0, 1)) {
              cnt++;
              if (tail < qsize && cnt < qsize)
                Q[tail++] = v;
              else
                orc_vec_push(bag, v);
            }
          }
        }
        for (uint64_t j = head; j < tail; j++) orc_vec_push(bag, Q[j]);
      } else if (deg_f > 0) {
        if (deg_f >= ORC_HEAVY_DEG) {
          orc_vec_push(&heavy[tid], node);
        } else {
          for (uint64_t j = off[node]; j < off[node + 1]; j++) {
            uint32_t v = E[j];
            if (!orc_load8(&dst[v]) && orc_cas8(&dst[v], 0, 1)) orc_vec_push(bag, v);
          }
        }
      }
    }
  }
  for (int t = 0; t < r->nt; t++) {
    for (size_t h = 0; h < heavy[t].n; h++) {
      uint32_t node = heavy[t].a[h];
#pragma omp parallel num_threads(r->nt)
      {
        orc_vec* bag = &r->bag[omp_get_thread_num()];
#pragma omp for schedule(static, 2048)
        for (uint64_t j = off[node]; j < off[node + 1]; j++) {
          uint32_t v = E[j];
          if (!orc_load8(&dst[v]) && orc_cas8(&dst[v], 0, 1)) orc_vec_push(bag, v);
        }
      }
    }
  }
  orc_vec_free(heavy, r->nt);
  return orc_vec_gather(r->bag, r->nt, r->front);
}

static uint64_t reach_dense_update(reach_t* r, uint8_t* dst) { /* reach.hpp:173-190 */
  uint64_t cnt = 0;
#pragma omp parallel for schedule(dynamic, 1024) reduction(+ : cnt) num_threads(r->nt)
  for (uint64_t i = 0; i < r->n; i++) {
    r->new_dense[i] = 0;
    if (!dst[i]) {
      for (uint64_t j = r->in_off[i]; j < r->in_off[i + 1]; j++) {
        if (r->dense_front[r->in_E[j]]) {
          dst[i] = 1;
          r->new_dense[i] = 1;
          cnt++;
          break;
        }
      }
    }
  }
  uint8_t* t = r->dense_front;
  r->dense_front = r->new_dense;
  r->new_dense = t;
  return cnt;
}

static void reach_init(reach_t* r, uint64_t n, uint64_t m, const uint64_t* off, const uint32_t* E,
                       const uint64_t* in_off, const uint32_t* in_E, uint32_t tau, int nt) {
  memset(r, 0, sizeof(*r));
  r->n = n;
  r->m = m;
  r->off = off;
  r->E = E;
  r->in_off = in_off;
  r->in_E = in_E;
  r->tau = tau;
  r->nt = nt;
  r->front = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1));
  r->dense_front = (uint8_t*)calloc(n ? n : 1, 1);
  r->new_dense = (uint8_t*)calloc(n ? n : 1, 1);
  r->threshold = m / 20;
  r->bag = (orc_vec*)calloc(nt, sizeof(orc_vec));
  r->lq = (uint32_t**)malloc(sizeof(uint32_t*) * nt);
  for (int t = 0; t < nt; t++) r->lq[t] = (uint32_t*)malloc(sizeof(uint32_t) * (tau + 1));
}

static void reach_free(reach_t* r) {
  free(r->front);
  free(r->dense_front);
  free(r->new_dense);
  orc_vec_free(r->bag, r->nt);
  for (int t = 0; t < r->nt; t++) free(r->lq[t]);
  free(r->lq);
}

/* reach.hpp:208-243 */
static int reach_run(reach_t* r, uint32_t src, uint8_t* dst, int local) {
  memset(dst, 0, r->n);
  r->front[0] = src;
  dst[src] = 1;
  r->n_front = 1;
  r->sparse_pre = 1;
  r->num_round = 0;
  while (r->n_front > 0) {
    r->num_round++;
    int sparse_now = reach_judge(r);
    if (sparse_now)
      r->n_front = reach_sparse_update(r, dst, local);
    else
      r->n_front = reach_dense_update(r, dst);
    r->sparse_pre = sparse_now;
  }
  return (int)r->num_round;
}

int orc_reach(uint64_t n, uint64_t m, const uint64_t* off, const uint32_t* E,
              const uint64_t* in_off, const uint32_t* in_E, uint32_t src, uint8_t* dst,
              int local, uint32_t tau, int nthreads) {
  if (nthreads <= 0) nthreads = omp_get_max_threads();
  reach_t r;
  reach_init(&r, n, m, off, E, in_off, in_E, tau, nthreads);
  int rounds = reach_run(&r, src, dst, local);
  reach_free(&r);
  return rounds;
}

/* ------------------------------------------------------------------ */
/* (vertex, pivot) multimap (src/resizable_table.h:99-313)              */
/* Entry packed as key<<32 | value; empty = (UINT_N_MAX, UINT_N_MAX).   */
/* ------------------------------------------------------------------ */
#define OT_EMPTY (~(uint64_t)0)

typedef struct {
  uint64_t* slot;
  uint64_t m, mask;
  int full;
  uint64_t ne;
} otable;

static void ot_clear(otable* t) {
#pragma omp parallel for
  for (uint64_t i = 0; i < t->m; i++) t->slot[i] = OT_EMPTY;
}

static void ot_make(otable* t, uint64_t m_req) { /* resizable_table.h:136-148 */
  uint64_t m = 1;
  while (m < m_req) m <<= 1;
  free(t->slot);
  t->m = m;
  t->mask = m - 1;
  t->slot = (uint64_t*)malloc(sizeof(uint64_t) * m);
  t->full = 0;
  t->ne = 0;
  ot_clear(t);
}

static void ot_double(otable* t) { ot_make(t, 2 * t->m); } /* :196-204 */

static inline uint64_t ot_first(const otable* t, uint32_t k) {
  return (uint64_t)orc_hash32(k) & t->mask;
}

/* :214-240 — gives up after 0.8m probes and raises table_full */
static int ot_insert(otable* t, uint32_t k, uint32_t v) {
  uint64_t kv = ((uint64_t)k << 32) | v;
  uint64_t h = ot_first(t, k);
  for (uint64_t count = 0; (double)count < 0.8 * (double)t->m; count++) {
    if (__atomic_load_n(&t->full, __ATOMIC_RELAXED)) return 0;
    uint64_t cur = orc_load64(&t->slot[h]);
    if ((uint32_t)(cur >> 32) == ORC_NMAX && orc_cas64(&t->slot[h], OT_EMPTY, kv)) {
      __atomic_fetch_add(&t->ne, 1, __ATOMIC_RELAXED);
      return 1;
    }
    if (orc_load64(&t->slot[h]) == kv) return 0;
    h = (h + 1) & t->mask;
  }
  __atomic_store_n(&t->full, 1, __ATOMIC_RELAXED);
  return 0;
}

/* :283-294 (bounded by m probes) */
static int ot_contains(const otable* t, uint32_t k, uint32_t v) {
  uint64_t kv = ((uint64_t)k << 32) | v;
  uint64_t h = ot_first(t, k);
  for (uint64_t c = 0; c < t->m; c++) {
    uint64_t cur = t->slot[h];
    if (cur == kv) return 1;
    if ((uint32_t)(cur >> 32) == ORC_NMAX) return 0;
    h = (h + 1) & t->mask;
  }
  return 0;
}

/* ------------------------------------------------------------------ */
/* SCC (src/scc.hpp:38-476)                                            */
/* ------------------------------------------------------------------ */
typedef struct {
  uint64_t n, m;
  const uint64_t *off, *in_off;
  const uint32_t *E, *in_E;
  uint64_t* labels;
  uint32_t* front;
  uint32_t* sub_front;
  uint8_t* bits;
  uint64_t n_front;
  uint64_t label_offset;
  uint32_t tau;
  int nt;
  orc_vec* bag;
  uint32_t** lq;
} scc_t;

/* scc.hpp:117-136: copy every pivot label of cur_node to ngb_node
 * (iter_kv walk, resizable_table.h:49-97). */
static int edge_map(otable* t, uint32_t cur, uint32_t ngb) {
  int changed = 0;
  uint64_t h = ot_first(t, cur);
  int found = 0;
  uint64_t e = 0;
  for (uint64_t i = 0; i < t->m; i++) { /* init() */
    e = orc_load64(&t->slot[h]);
    uint32_t key = (uint32_t)(e >> 32);
    if (key == ORC_NMAX) break;
    if (key == cur) {
      found = 1;
      break;
    }
    h = (h + 1) & t->mask;
  }
  if (!found) return 0;
  changed |= ot_insert(t, ngb, (uint32_t)e);
  if (t->full) return 0;
  uint64_t probes = 0;
  for (;;) { /* has_next() */
    h = (h + 1) & t->mask;
    found = 0;
    while (probes < t->m) {
      e = orc_load64(&t->slot[h]);
      uint32_t key = (uint32_t)(e >> 32);
      if (key == ORC_NMAX) break;
      if (key == cur) {
        found = 1;
        break;
      }
      h = (h + 1) & t->mask;
      probes++;
    }
    if (!found) break;
    changed |= ot_insert(t, ngb, (uint32_t)e);
    if (t->full) return 0;
  }
  return changed;
}

/* scc.hpp:144-254 */
static long multi_search(scc_t* s, otable* t, int forward, int local) {
  const uint64_t* off = forward ? s->off : s->in_off;
  const uint32_t* E = forward ? s->E : s->in_E;
  const uint64_t* labels = s->labels;
  uint64_t label_offset = s->label_offset;
#pragma omp parallel for num_threads(s->nt)
  for (uint64_t i = 0; i < s->n_front; i++) {
    ot_insert(t, s->front[i], (uint32_t)(label_offset + i));
    s->sub_front[i] = s->front[i];
  }
  uint64_t sub_n = s->n_front;
  long round = 0;
  uint64_t qsize = s->tau;
  int sub_round = 0;
  orc_vec* heavy = (orc_vec*)calloc(s->nt, sizeof(orc_vec));
  /* heavy entries carry (node, frontier index) pairs */
  while (sub_n > 0) {
    sub_round++;
    round++;
#pragma omp parallel for num_threads(s->nt)
    for (uint64_t i = 0; i < sub_n; i++) s->bits[s->sub_front[i]] = 0;
#pragma omp parallel num_threads(s->nt)
    {
      int tid = omp_get_thread_num();
      orc_vec* bag = &s->bag[tid];
      uint32_t* Q = s->lq[tid];
#pragma omp for schedule(dynamic, 16)
      for (uint64_t i = 0; i < sub_n; i++) {
        uint32_t node = s->sub_front[i];
        uint64_t degree = off[node + 1] - off[node];
        uint64_t cnt = 0;
        if (local && degree < qsize && cnt < qsize) {
          uint64_t head = 0, tail = 0;
          Q[tail++] = node;
          while (head < tail && cnt < qsize) {
            uint32_t u = Q[head];
            uint64_t deg = off[u + 1] - off[u];
            if (deg >= qsize) break;
            head++;
            for (uint64_t j = off[u]; j < off[u + 1]; j++) {
              uint32_t v = E[j];
              if (!(labels[v] & ORC_TOP_BIT) && labels[v] == labels[u]) {
                cnt++;
                int ok = (sub_round == 1 && local)
                             ? ot_insert(t, v, (uint32_t)(label_offset + i))
                             : edge_map(t, node, v);
                if (ok) {
                  if (cnt < qsize) {
                    Q[tail++] = v;
                  } else if (orc_cas8(&s->bits[v], 0, 1)) {
                    orc_vec_push(bag, v);
                  }
                }
              }
            }
          }
          for (uint64_t j = head; j < tail; j++) {
            uint32_t u = Q[j];
            if (orc_cas8(&s->bits[u], 0, 1)) orc_vec_push(bag, u);
          }
        } else if (degree > 0) {
          if (degree >= ORC_HEAVY_DEG) {
            orc_vec_push(&heavy[tid], node);
            orc_vec_push(&heavy[tid], (uint32_t)i);
          } else {
            for (uint64_t j = off[node]; j < off[node + 1]; j++) {
              uint32_t v = E[j];
              if (!(labels[v] & ORC_TOP_BIT) && labels[v] == labels[node]) {
                int ok = (sub_round == 1 && local)
                             ? ot_insert(t, v, (uint32_t)(label_offset + i))
                             : edge_map(t, node, v);
                if (ok && orc_cas8(&s->bits[v], 0, 1)) orc_vec_push(bag, v);
              }
            }
          }
        }
      }
    }
    for (int th = 0; th < s->nt; th++) {
      for (size_t h = 0; h + 1 < heavy[th].n; h += 2) {
        uint32_t node = heavy[th].a[h];
        uint32_t i = heavy[th].a[h + 1];
#pragma omp parallel num_threads(s->nt)
        {
          orc_vec* bag = &s->bag[omp_get_thread_num()];
#pragma omp for schedule(dynamic, 1024)
          for (uint64_t j = off[node]; j < off[node + 1]; j++) {
            uint32_t v = E[j];
            if (!(labels[v] & ORC_TOP_BIT) && labels[v] == labels[node]) {
              int ok = (sub_round == 1 && local)
                           ? ot_insert(t, v, (uint32_t)(label_offset + i))
                           : edge_map(t, node, v);
              if (ok && orc_cas8(&s->bits[v], 0, 1)) orc_vec_push(bag, v);
            }
          }
        }
      }
      heavy[th].n = 0;
    }
    if (t->full) {
      for (int th = 0; th < s->nt; th++) s->bag[th].n = 0;
      orc_vec_free(heavy, s->nt);
      return -1;
    }
    sub_n = orc_vec_gather(s->bag, s->nt, s->sub_front);
  }
  orc_vec_free(heavy, s->nt);
  return round;
}

/* scc.hpp:256-275 */
static long multi_search_safe(scc_t* s, otable* t, int forward, int local) {
  long round;
  for (;;) {
    round = multi_search(s, t, forward, local);
    if (round != -1) break;
    memset(s->bits, 0, s->n);
    ot_double(t);
  }
  return round;
}

int orc_scc(uint64_t n, uint64_t m, const uint64_t* off, const uint32_t* E,
            const uint64_t* in_off, const uint32_t* in_E, double beta, uint32_t tau,
            int local_reach, int local_scc, uint64_t seed, uint64_t* labels, int nthreads) {
  if (nthreads <= 0) nthreads = omp_get_max_threads();
  if (n == 0) return 0;
  scc_t s;
  memset(&s, 0, sizeof(s));
  s.n = n;
  s.m = m;
  s.off = off;
  s.E = E;
  s.in_off = in_off;
  s.in_E = in_E;
  s.labels = labels;
  s.tau = tau;
  s.nt = nthreads;
  s.front = (uint32_t*)malloc(sizeof(uint32_t) * n);
  s.sub_front = (uint32_t*)malloc(sizeof(uint32_t) * n);
  s.bits = (uint8_t*)calloc(n, 1);
  s.bag = (orc_vec*)calloc(nthreads, sizeof(orc_vec));
  s.lq = (uint32_t**)malloc(sizeof(uint32_t*) * nthreads);
  for (int t = 0; t < nthreads; t++) s.lq[t] = (uint32_t*)malloc(sizeof(uint32_t) * (tau + 1));

  /* init / trim: scc.hpp:288-305 */
  memset(labels, 0, sizeof(uint64_t) * n);
  uint32_t* P = (uint32_t*)malloc(sizeof(uint32_t) * n);
  uint64_t n_zeros = 0;
  uint64_t np = orc_pivot_order(n, off, in_off, seed, P, &n_zeros);
  {
    uint64_t i = 0;
    for (uint64_t v = 0; v < n; v++)
      if (off[v + 1] == off[v] || in_off[v + 1] == in_off[v]) {
        labels[v] = 1 + (i | ORC_TOP_BIT);
        i++;
      }
  }
  s.label_offset = n_zeros + 1;

  if (np > 0) {
    /* first pivot: scc.hpp:316-355 */
    uint8_t* d1 = (uint8_t*)malloc(n);
    uint8_t* d2 = (uint8_t*)malloc(n);
    reach_t r;
    reach_init(&r, n, m, off, E, in_off, in_E, tau, nthreads);
    reach_run(&r, P[0], d1, local_reach);
    /* swap_graph(): the backward search runs on the transpose */
    r.off = in_off;
    r.E = in_E;
    r.in_off = off;
    r.in_E = E;
    reach_run(&r, P[0], d2, local_reach);
    reach_free(&r);
    uint64_t label = s.label_offset;
#pragma omp parallel for num_threads(nthreads)
    for (uint64_t i = 0; i < np; i++) {
      uint32_t v = P[i];
      if (d1[v] && d2[v])
        labels[v] = label | ORC_TOP_BIT;
      else if (d1[v] || d2[v])
        labels[v] = label;
    }
    free(d1);
    free(d2);
    uint32_t* centers = (uint32_t*)malloc(sizeof(uint32_t) * np);
    uint64_t nc = 0;
    for (uint64_t i = 0; i < np; i++)
      if (!(labels[P[i]] & ORC_TOP_BIT)) centers[nc++] = P[i];
    s.label_offset++;

    /* prefix-doubling rounds: scc.hpp:365-473 */
    uint32_t step_size = 1, cur_offset = 0, finished = 0;
    uint32_t n_remaining = (uint32_t)nc;
    uint32_t in_table_ne = 1, out_table_ne = 1;
    otable tf, tb;
    memset(&tf, 0, sizeof(tf));
    memset(&tb, 0, sizeof(tb));
    while (finished != n_remaining) {
      uint32_t end = cur_offset + step_size < n_remaining ? cur_offset + step_size : n_remaining;
      uint32_t vs_size = end - cur_offset;
      finished += vs_size;
      step_size = (uint32_t)ceil(step_size * beta);
      uint64_t nf = 0;
      for (uint32_t i = 0; i < vs_size; i++) {
        uint32_t v = centers[cur_offset + i];
        if (!(labels[v] & ORC_TOP_BIT)) s.front[nf++] = v;
      }
      s.n_front = nf;
      cur_offset = end;
      if (nf == 0) continue;
      uint32_t a = (uint32_t)ceil(0.3 * n_remaining);
      if (a > 6000000u) a = 6000000u;
      uint64_t out_m = 2 * ((uint64_t)a > (uint64_t)beta * out_table_ne ? (uint64_t)a
                                                                         : (uint64_t)beta * out_table_ne);
      ot_make(&tf, out_m);
      multi_search_safe(&s, &tf, 1, local_scc);
      uint64_t in_m = 2 * ((uint64_t)a > (uint64_t)beta * in_table_ne ? (uint64_t)a
                                                                       : (uint64_t)beta * in_table_ne);
      ot_make(&tb, in_m);
      multi_search_safe(&s, &tb, 0, local_scc);
      s.label_offset += nf;

      otable* sm = (tf.m <= tb.m) ? &tf : &tb;
      otable* lg = (tf.m <= tb.m) ? &tb : &tf;
      /* scc.hpp:441-464 */
#pragma omp parallel for num_threads(nthreads) schedule(static, 4096)
      for (uint64_t i = 0; i < sm->m; i++) {
        uint64_t e = sm->slot[i];
        if ((uint32_t)(e >> 32) == ORC_NMAX) continue;
        uint32_t v = (uint32_t)(e >> 32);
        uint64_t l = (uint32_t)e;
        if (ot_contains(lg, v, (uint32_t)l))
          orc_write_max64(&labels[v], l | ORC_TOP_BIT);
        else
          orc_write_max64(&labels[v], l);
      }
#pragma omp parallel for num_threads(nthreads) schedule(static, 4096)
      for (uint64_t i = 0; i < lg->m; i++) {
        uint64_t e = lg->slot[i];
        if ((uint32_t)(e >> 32) == ORC_NMAX) continue;
        orc_write_max64(&labels[(uint32_t)(e >> 32)], (uint32_t)e);
      }
      out_table_ne = (uint32_t)tf.ne;
      in_table_ne = (uint32_t)tb.ne;
    }
    free(tf.slot);
    free(tb.slot);
    free(centers);
  }

  /* finalise: scc.hpp:475-476 */
#pragma omp parallel for num_threads(nthreads)
  for (uint64_t i = 0; i < n; i++) labels[i] = (labels[i] & ORC_VAL_MASK) - 1;

  free(P);
  free(s.front);
  free(s.sub_front);
  free(s.bits);
  orc_vec_free(s.bag, nthreads);
  for (int t = 0; t < nthreads; t++) free(s.lq[t]);
  free(s.lq);
  return 0;
}
