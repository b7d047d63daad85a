/*
 * Oracle connectivity — TEST INFRASTRUCTURE (see oracle.h).
 *
 * C11/OpenMP restatement of src/ldd.hpp (low-diameter decomposition with
 * exponentially growing centre batches, VGC local queue of 1024, push/pull
 * switch) followed by src/Connectivity.h:37-96 (union-find over the edges of
 * vertices outside the most frequent LDD label, UniteRemCAS + find_compress +
 * split_atomic_one from src/union_find_rules.h).  Spanning forests are not
 * restated (the tests compare partitions only).
 */
#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#include "common.h"
#include "oracle.h"

#define LDD_LOCAL_QUEUE 1024 /* ldd.hpp:17 */
#define LDD_BLOCK 1024       /* BLOCK_SIZE, utilities.h:8 */

typedef struct {
  uint64_t n, m;
  const uint64_t* off;
  const uint32_t* E;
  uint32_t* front;
  uint8_t* in_frontier;
  uint8_t* in_next;
  uint64_t fsize, threshold, num_round;
  int sparse_pre;
  int nt;
  orc_vec* bag;
  uint32_t** lq;
} ldd_t;

static void ldd_sparse2dense(ldd_t* d) { /* ldd.hpp:384-394 */
  memset(d->in_frontier, 0, d->n);
  for (uint64_t i = 0; i < d->fsize; i++) d->in_frontier[d->front[i]] = 1;
}

static void ldd_dense2sparse(ldd_t* d) { /* ldd.hpp:396-405 (the count is not stored) */
  uint64_t k = 0;
  for (uint64_t v = 0; v < d->n; v++)
    if (d->in_frontier[v]) d->front[k++] = (uint32_t)v;
}

static uint64_t ldd_dense_sample(ldd_t* d, uint32_t seed) { /* ldd.hpp:368-382 */
  uint32_t count = 0;
  uint64_t out_edges = 0;
  uint32_t i = 0;
  /* bounded: the reference loops until 50 hits; a frontier the count
   * misses (see ldd() below) could otherwise spin for a long time */
  while (count < 50 && i < 50u * 1024u * 1024u) {
    i++;
    uint32_t idx = (uint32_t)(orc_hash32(seed + i) % d->n);
    if (d->in_frontier[idx]) {
      count++;
      out_edges += d->off[idx + 1] - d->off[idx];
    }
  }
  if (!count) return 0;
  return d->fsize * (out_edges / count);
}

static int ldd_judge(ldd_t* d) { /* ldd.hpp:407-442 */
  uint64_t out_edges = 0;
  int both = 0;
  if (!d->sparse_pre && d->fsize < (1u << 14)) {
    ldd_dense2sparse(d);
    both = 1;
  }
  if (d->sparse_pre || both) {
    uint64_t s = 0;
    for (uint64_t i = 0; i < d->fsize; i++) s += d->off[d->front[i] + 1] - d->off[d->front[i]];
    out_edges = s;
  } else {
    out_edges = ldd_dense_sample(d, orc_hash32((uint32_t)d->num_round));
  }
  int sparse_now = (d->fsize + out_edges) < d->threshold;
  if (!both && d->sparse_pre != sparse_now) {
    if (!sparse_now)
      ldd_sparse2dense(d);
    else
      ldd_dense2sparse(d);
  }
  return sparse_now;
}

static uint64_t ldd_sparse(ldd_t* d, uint32_t* label) { /* ldd.hpp:88-161 */
  const uint64_t* off = d->off;
  const uint32_t* E = d->E;
  orc_vec* heavy = (orc_vec*)calloc(d->nt, sizeof(orc_vec));
#pragma omp parallel num_threads(d->nt)
  {
    int tid = omp_get_thread_num();
    orc_vec* bag = &d->bag[tid];
    uint32_t* Q = d->lq[tid];
#pragma omp for schedule(dynamic, 16)
    for (uint64_t i = 0; i < d->fsize; i++) {
      uint32_t f = d->front[i];
      uint64_t deg_f = off[f + 1] - off[f];
      if (deg_f > LDD_BLOCK) {
        orc_vec_push(&heavy[tid], f);
      } else {
        uint64_t head = 0, tail = 0;
        Q[tail++] = f;
        while (head < tail && tail != LDD_LOCAL_QUEUE) {
          uint32_t u = Q[head++];
          uint64_t deg_u = off[u + 1] - off[u];
          if (deg_u > LDD_BLOCK) {
            orc_vec_push(bag, u);
          } else {
            uint32_t lu = orc_load32(&label[u]);
            if (lu == ORC_NMAX) continue; /* unlabelled: nothing to pass on */
            for (uint64_t j = off[u]; j < off[u + 1]; j++) {
              uint32_t v = E[j];
              if (orc_load32(&label[v]) == ORC_NMAX && orc_cas32(&label[v], ORC_NMAX, lu)) {
                if (tail < LDD_LOCAL_QUEUE)
                  Q[tail++] = v;
                else
                  orc_vec_push(bag, v);
              }
            }
          }
        }
        for (uint64_t j = head; j < tail; j++) orc_vec_push(bag, Q[j]);
      }
    }
  }
  for (int t = 0; t < d->nt; t++) {
    for (size_t h = 0; h < heavy[t].n; h++) {
      uint32_t f = heavy[t].a[h];
      uint32_t lf = label[f];
#pragma omp parallel num_threads(d->nt)
      {
        orc_vec* bag = &d->bag[omp_get_thread_num()];
#pragma omp for schedule(static, LDD_BLOCK)
        for (uint64_t j = off[f]; j < off[f + 1]; j++) {
          uint32_t v = E[j];
          if (orc_load32(&label[v]) == ORC_NMAX && orc_cas32(&label[v], ORC_NMAX, lf))
            orc_vec_push(bag, v);
        }
      }
    }
  }
  orc_vec_free(heavy, d->nt);
  return orc_vec_gather(d->bag, d->nt, d->front);
}

/* Like the reference, a vertex labelled in this round joins the current
 * frontier at once (in_frontier[i] = true, ldd.hpp:227), so later vertices of
 * the same round may take its label.  The label is stored before the flag
 * with release order and read after the flag with acquire order: with relaxed
 * orders a weakly ordered CPU (Arm) can show the flag before the label, and a
 * vertex would copy the "unlabelled" value. */
static uint64_t ldd_dense(ldd_t* d, uint32_t* label) { /* ldd.hpp:163-247 (symmetric) */
  uint64_t cnt = 0;
#pragma omp parallel for schedule(dynamic, LDD_BLOCK) reduction(+ : cnt) num_threads(d->nt)
  for (uint64_t i = 0; i < d->n; i++) {
    d->in_next[i] = 0;
    if (orc_load32(&label[i]) == ORC_NMAX) {
      for (uint64_t j = d->off[i]; j < d->off[i + 1]; j++) {
        uint32_t v = d->E[j];
        if (__atomic_load_n(&d->in_frontier[v], __ATOMIC_ACQUIRE)) {
          const uint32_t lv = orc_load32(&label[v]);
          if (lv == ORC_NMAX) continue;
          __atomic_store_n(&label[i], lv, __ATOMIC_RELAXED);
          __atomic_store_n(&d->in_frontier[i], 1, __ATOMIC_RELEASE);
          d->in_next[i] = 1;
          cnt++;
          break;
        }
      }
    }
  }
  uint8_t* t = d->in_frontier;
  d->in_frontier = d->in_next;
  d->in_next = t;
  return cnt;
}

/* union_find_rules.h:34-46 */
static inline uint32_t uf_find_compress(uint32_t i, uint32_t* p) {
  uint32_t j = i;
  if (orc_load32(&p[j]) == j) return j;
  do {
    j = orc_load32(&p[j]);
  } while (orc_load32(&p[j]) != j);
  uint32_t tmp;
  while ((tmp = orc_load32(&p[i])) > j) {
    __atomic_store_n(&p[i], j, __ATOMIC_RELAXED);
    i = tmp;
  }
  return j;
}

/* union_find_rules.h:80-90 */
static inline uint32_t uf_split_atomic_one(uint32_t i, uint32_t* p) {
  uint32_t v = orc_load32(&p[i]);
  uint32_t w = orc_load32(&p[v]);
  if (v == w) return v;
  if (orc_load32(&p[i]) == v) orc_cas32(&p[i], v, w);
  return v;
}

/* union_find_rules.h:193-225 (UniteRemCAS, link high -> low) */
static inline uint32_t uf_unite(uint32_t x, uint32_t y, uint32_t* p) {
  uint32_t rx = x, ry = y;
  while (orc_load32(&p[rx]) != orc_load32(&p[ry])) {
    uint32_t p_ry = orc_load32(&p[ry]);
    uint32_t p_rx = orc_load32(&p[rx]);
    if (p_rx < p_ry) {
      uint32_t t = rx;
      rx = ry;
      ry = t;
      t = p_rx;
      p_rx = p_ry;
      p_ry = t;
    }
    if (rx == orc_load32(&p[rx]) && orc_cas32(&p[rx], rx, p_ry)) {
      uf_find_compress(x, p);
      uf_find_compress(y, p);
      return rx;
    }
    rx = uf_split_atomic_one(rx, p);
  }
  return ORC_NMAX;
}

static int cmp_u32(const void* a, const void* b) {
  uint32_t x = *(const uint32_t*)a, y = *(const uint32_t*)b;
  return x < y ? -1 : x > y;
}

/* Connectivity.h:13-35 */
static uint32_t get_max_label(uint64_t n, const uint32_t* label) {
  enum { NUM_SAMPLES = 10000 };
  uint64_t seed = orc_hash64(n + 1);
  uint32_t* s = (uint32_t*)malloc(sizeof(uint32_t) * NUM_SAMPLES);
  for (uint64_t i = 0; i < NUM_SAMPLES; i++) s[i] = label[orc_hash64(i + seed) % n];
  qsort(s, NUM_SAMPLES, sizeof(uint32_t), cmp_u32);
  uint32_t max_label = 0, max_cnt = 0;
  for (uint64_t i = 0; i < NUM_SAMPLES;) {
    uint64_t j = 1;
    while (i + j < NUM_SAMPLES && s[i + j] == s[i]) j++;
    if (j > max_cnt) {
      max_cnt = (uint32_t)j;
      max_label = s[i];
    }
    i += j;
  }
  free(s);
  return max_label;
}

int orc_cc(uint64_t n, uint64_t m, const uint64_t* off, const uint32_t* E, double beta,
           uint32_t* label, int nthreads) {
  if (nthreads <= 0) nthreads = omp_get_max_threads();
  if (n == 0) return 0;
  ldd_t d;
  memset(&d, 0, sizeof(d));
  d.n = n;
  d.m = m;
  d.off = off;
  d.E = E;
  d.nt = nthreads;
  d.front = (uint32_t*)malloc(sizeof(uint32_t) * (n + 2048));
  d.in_frontier = (uint8_t*)calloc(n, 1);
  d.in_next = (uint8_t*)calloc(n, 1);
  d.threshold = m / 20;
  d.sparse_pre = 1;
  d.bag = (orc_vec*)calloc(nthreads, sizeof(orc_vec));
  d.lq = (uint32_t**)malloc(sizeof(uint32_t*) * nthreads);
  for (int t = 0; t < nthreads; t++) d.lq[t] = (uint32_t*)malloc(sizeof(uint32_t) * LDD_LOCAL_QUEUE);

  /* ldd.hpp:325-417 */
  for (uint64_t i = 0; i < n; i++) label[i] = ORC_NMAX;
  enum { SAMPLE_NUMBER = 1024 };
  uint32_t perm[SAMPLE_NUMBER];
  for (uint32_t i = 0; i < SAMPLE_NUMBER; i++) perm[i] = (uint32_t)(orc_hash32(SAMPLE_NUMBER + i) % n);
  uint64_t num_sampled = 0;
  while (d.fsize > 0 || num_sampled < SAMPLE_NUMBER) {
    d.num_round++;
    uint64_t step = (uint64_t)floor(exp((double)d.num_round * beta));
    uint64_t work = step < SAMPLE_NUMBER - num_sampled ? step : SAMPLE_NUMBER - num_sampled;
    uint64_t num_new = 0;
    if (d.sparse_pre && work > 0) {
      for (uint64_t i = num_sampled; i < num_sampled + work; i++) {
        uint32_t u = perm[i];
        if (label[u] == ORC_NMAX) {
          d.front[d.fsize + num_new++] = u;
        }
      }
      for (uint64_t i = 0; i < num_new; i++) label[d.front[d.fsize + i]] = d.front[d.fsize + i];
    } else if (work > 0) {
      /* the reference counts with count(perm, UINT_N_MAX); the frontier
       * flags are what drive the dense round, so count real additions */
      for (uint64_t i = num_sampled; i < num_sampled + work; i++) {
        uint32_t u = perm[i];
        if (label[u] == ORC_NMAX) {
          label[u] = u;
          if (!d.in_frontier[u]) num_new++;
          d.in_frontier[u] = 1;
        }
      }
    }
    d.fsize += num_new;
    num_sampled += work;
    int sparse_now = ldd_judge(&d);
    if (sparse_now)
      d.fsize = ldd_sparse(&d, label);
    else
      d.fsize = ldd_dense(&d, label);
    d.sparse_pre = sparse_now;
  }
  for (uint64_t i = 0; i < n; i++)
    if (label[i] == ORC_NMAX) label[i] = (uint32_t)i;

  /* Connectivity.h:58-95 */
  uint32_t max_label = get_max_label(n, label);
#pragma omp parallel for schedule(dynamic, 512) num_threads(nthreads)
  for (uint64_t i = 0; i < n; i++) {
    if (uf_find_compress(orc_load32(&label[i]), label) != uf_find_compress(max_label, label)) {
      for (uint64_t j = off[i]; j < off[i + 1]; j++) uf_unite((uint32_t)i, E[j], label);
    }
  }
#pragma omp parallel for num_threads(nthreads)
  for (uint64_t i = 0; i < n; i++) label[i] = uf_find_compress(orc_load32(&label[i]), label);

  free(d.front);
  free(d.in_frontier);
  free(d.in_next);
  orc_vec_free(d.bag, nthreads);
  for (int t = 0; t < nthreads; t++) free(d.lq[t]);
  free(d.lq);
  return 0;
}
