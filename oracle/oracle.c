/*
 * oracle.c -- CPU restatement of BYO's hot path.  TEST INFRASTRUCTURE ONLY:
 * the checker for the CUDA path and the CPU baseline, never part of the
 * product.  See oracle.h for the contract and the reference citations.
 *
 * Build: gcc -O3 -fopenmp -ffp-contract=off -fPIC -shared (oracle/Makefile or
 * byo_gb300/build.py).  -ffp-contract=off keeps the FP64 PageRank and the
 * Chung-Lu table identical across x86 and aarch64.
 */
#include "oracle.h"

#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#define GAMMA64 0x9E3779B97F4A7C15ull

int orc_num_threads(void) { return omp_get_max_threads(); }
void orc_set_num_threads(int t) {
  if (t > 0) omp_set_num_threads(t);
}

static void *xmalloc(size_t bytes) {
  void *p = malloc(bytes ? bytes : 1);
  if (!p) abort();
  return p;
}

/* ------------------------------------------------------------------ generators */

uint64_t orc_mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static inline uint64_t draw(uint64_t key, uint64_t ctr) { return orc_mix64(key + ctr * GAMMA64); }

static uint32_t prob_to_u32(double p) {
  if (p <= 0.0) return 0;
  double s = p * 4294967296.0;
  if (s >= 4294967295.0) return 0xFFFFFFFFu;
  return (uint32_t)s;
}

void orc_rmat_thresholds(double a, double b, double c, uint32_t out[3]) {
  out[0] = prob_to_u32(a);
  out[1] = prob_to_u32(a + b);
  out[2] = prob_to_u32(a + b + c);
}

void orc_rmat_edges(uint64_t seed, uint32_t lg_n, uint64_t first, uint64_t count,
                    const uint32_t thr[3], uint32_t *src, uint32_t *dst) {
  const uint64_t key = orc_mix64(seed);
  const uint32_t ta = thr[0], tab = thr[1], tabc = thr[2];
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < (int64_t)count; k++) {
    uint64_t i = first + (uint64_t)k;
    uint32_t s = 0, d = 0;
    uint64_t w = 0;
    for (uint32_t l = 0; l < lg_n; l++) {
      if ((l & 1) == 0) w = draw(key, i * 32 + (l >> 1));
      uint32_t r = (l & 1) ? (uint32_t)(w >> 32) : (uint32_t)w;
      uint32_t bit = 1u << (lg_n - 1 - l);
      if (r < ta) {
      } else if (r < tab) {
        d |= bit;
      } else if (r < tabc) {
        s |= bit;
      } else {
        s |= bit;
        d |= bit;
      }
    }
    src[k] = s;
    dst[k] = d;
  }
}

void orc_uniform_pairs(uint64_t seed, uint64_t n, uint64_t first, uint64_t count, uint32_t *src,
                       uint32_t *dst) {
  const uint64_t key = orc_mix64(seed);
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < (int64_t)count; k++) {
    uint64_t w = draw(key, first + (uint64_t)k);
    src[k] = (uint32_t)(((w & 0xFFFFFFFFull) * n) >> 32);
    dst[k] = (uint32_t)(((w >> 32) * n) >> 32);
  }
}

uint64_t orc_grid_pairs(uint32_t rows, uint32_t cols, uint32_t *src, uint32_t *dst) {
  uint64_t k = 0;
  for (uint32_t r = 0; r < rows; r++) {
    for (uint32_t c = 0; c < cols; c++) {
      uint32_t v = r * cols + c;
      if (c + 1 < cols) {
        src[k] = v;
        dst[k] = v + 1;
        k++;
      }
      if (r + 1 < rows) {
        src[k] = v;
        dst[k] = v + cols;
        k++;
      }
    }
  }
  return k;
}

void orc_chung_lu_cdf(uint64_t n, double exponent, uint64_t *cdf) {
  /* sequential on purpose: the running sum order fixes the table bits */
  double alpha = 1.0 / (exponent - 1.0), total = 0.0;
  for (uint64_t i = 0; i < n; i++) total += pow((double)(i + 1), -alpha);
  double run = 0.0;
  const double scale = 9223372036854775808.0; /* 2^63 */
  for (uint64_t i = 0; i < n; i++) {
    run += pow((double)(i + 1), -alpha);
    double f = run / total * scale;
    cdf[i] = f >= scale ? (1ull << 63) : (uint64_t)f;
  }
  cdf[n - 1] = 1ull << 63;
}

static inline uint32_t cdf_pick(const uint64_t *cdf, uint64_t n, uint64_t x) {
  uint64_t lo = 0, hi = n - 1; /* first i with x < cdf[i]; cdf[n-1] = 2^63 > x */
  while (lo < hi) {
    uint64_t mid = (lo + hi) >> 1;
    if (x < cdf[mid])
      hi = mid;
    else
      lo = mid + 1;
  }
  return (uint32_t)lo;
}

void orc_chung_lu_pairs(uint64_t seed, uint64_t n, const uint64_t *cdf, uint64_t first,
                        uint64_t count, uint32_t *src, uint32_t *dst) {
  const uint64_t key = orc_mix64(seed);
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < (int64_t)count; k++) {
    uint64_t i = first + (uint64_t)k;
    src[k] = cdf_pick(cdf, n, draw(key, 2 * i) >> 1);
    dst[k] = cdf_pick(cdf, n, draw(key, 2 * i + 1) >> 1);
  }
}

/* ------------------------------------------------------------------ sorting */

/* LSD radix sort over the bytes that differ, 8 bits per pass, per-thread
 * histograms; stable, so the result is independent of the thread count. */
static void radix_sort_u64(uint64_t *keys, uint64_t count) {
  if (count < 2) return;
  uint64_t or_all = 0, and_all = ~0ull;
  for (uint64_t i = 0; i < count; i++) {
    or_all |= keys[i];
    and_all &= keys[i];
  }
  uint64_t diff = or_all ^ and_all;
  uint64_t *tmp = xmalloc(count * sizeof(uint64_t));
  int T = omp_get_max_threads();
  uint64_t *hist = xmalloc((size_t)T * 256 * sizeof(uint64_t));
  uint64_t *a = keys, *b = tmp;
  for (int shift = 0; shift < 64; shift += 8) {
    if (((diff >> shift) & 0xFF) == 0) continue;
    memset(hist, 0, (size_t)T * 256 * sizeof(uint64_t));
#pragma omp parallel num_threads(T)
    {
      int t = omp_get_thread_num(), nt = omp_get_num_threads();
      uint64_t lo = count * (uint64_t)t / (uint64_t)nt, hi = count * (uint64_t)(t + 1) / (uint64_t)nt;
      uint64_t *h = hist + (size_t)t * 256;
      for (uint64_t i = lo; i < hi; i++) h[(a[i] >> shift) & 0xFF]++;
#pragma omp barrier
#pragma omp single
      {
        uint64_t run = 0;
        for (int d = 0; d < 256; d++)
          for (int q = 0; q < nt; q++) {
            uint64_t c = hist[(size_t)q * 256 + d];
            hist[(size_t)q * 256 + d] = run;
            run += c;
          }
      }
      for (uint64_t i = lo; i < hi; i++) b[h[(a[i] >> shift) & 0xFF]++] = a[i];
    }
    uint64_t *s = a;
    a = b;
    b = s;
  }
  if (a != keys) memcpy(keys, a, count * sizeof(uint64_t));
  free(tmp);
  free(hist);
}

uint64_t orc_sort_unique_u64(uint64_t *keys, uint64_t count) {
  if (count == 0) return 0;
  radix_sort_u64(keys, count);
  uint64_t w = 1;
  for (uint64_t i = 1; i < count; i++)
    if (keys[i] != keys[w - 1]) keys[w++] = keys[i];
  return w;
}

uint64_t orc_build_csr(uint64_t n, const uint32_t *src, const uint32_t *dst, uint64_t count,
                       int symmetrise, int drop_self_loops, uint64_t *offsets, uint32_t *nbrs) {
  uint64_t total = symmetrise ? 2 * count : count;
  uint64_t *keys = xmalloc(total * sizeof(uint64_t));
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)count; i++) {
    keys[i] = ((uint64_t)src[i] << 32) | dst[i];
    if (symmetrise) keys[count + i] = ((uint64_t)dst[i] << 32) | src[i];
  }
  uint64_t u = orc_sort_unique_u64(keys, total);
  memset(offsets, 0, (n + 1) * sizeof(uint64_t));
  uint64_t m = 0;
  for (uint64_t i = 0; i < u; i++) {
    uint32_t s = (uint32_t)(keys[i] >> 32), d = (uint32_t)keys[i];
    if (drop_self_loops && s == d) continue;
    offsets[s + 1]++;
    nbrs[m++] = d;
  }
  for (uint64_t v = 0; v < n; v++) offsets[v + 1] += offsets[v];
  free(keys);
  return m;
}

/* ------------------------------------------------------------------ BFS */

typedef struct {
  uint32_t *a;
  uint64_t len, cap;
} vec32;

static inline void vec_push(vec32 *v, uint32_t x) {
  if (v->len == v->cap) {
    v->cap = v->cap ? 2 * v->cap : 1024;
    v->a = realloc(v->a, v->cap * sizeof(uint32_t));
    if (!v->a) abort();
  }
  v->a[v->len++] = x;
}

static inline int atomic_min_u64(uint64_t *p, uint64_t val, uint64_t *old_out) {
  uint64_t old = __atomic_load_n(p, __ATOMIC_RELAXED);
  while (val < old) {
    if (__atomic_compare_exchange_n(p, &old, val, 1, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
      *old_out = old;
      return 1;
    }
  }
  *old_out = old;
  return 0;
}

uint32_t orc_bfs(uint64_t n, const uint64_t *offsets, const uint32_t *nbrs, uint32_t src,
                 uint32_t *parent, uint32_t *level) {
  const uint64_t M = offsets[n];
  const uint64_t NONE64 = ~0ull;
  uint64_t *lp = xmalloc(n * sizeof(uint64_t));
#pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < (int64_t)n; v++) lp[v] = NONE64;
  lp[src] = src; /* level 0 */
  uint32_t *front = xmalloc(n * sizeof(uint32_t));
  uint64_t fsize = 1;
  front[0] = src;
  int fdense = 0; /* whether the current frontier came out of a dense round */
  uint8_t *inF = xmalloc(n);
  uint8_t *mark = xmalloc(n);
  memset(inF, 0, n);
  int T = omp_get_max_threads();
  vec32 *loc = calloc((size_t)T, sizeof(vec32));
  uint32_t r = 1;
  while (fsize > 0) {
    int dense;
    if (fdense && fsize > n / 10) {
      dense = 1; /* edge_map_data.h:263 */
    } else {
      uint64_t outdeg = 0;
#pragma omp parallel for reduction(+ : outdeg) schedule(static)
      for (int64_t i = 0; i < (int64_t)fsize; i++) outdeg += offsets[front[i] + 1] - offsets[front[i]];
      if (outdeg == 0) break;                 /* edge_map_data.h:290 */
      dense = (fsize + outdeg > M / 20);       /* :291 with threshold -1 => M/20 (:259) */
    }
    if (dense) {
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < (int64_t)fsize; i++) inF[front[i]] = 1;
#pragma omp parallel for schedule(dynamic, 256)
      for (int64_t v = 0; v < (int64_t)n; v++) {
        mark[v] = 0;
        if (lp[v] != NONE64) continue;
        for (uint64_t j = offsets[v]; j < offsets[v + 1]; j++) {
          uint32_t u = nbrs[j];
          if (inF[u]) { /* first frontier neighbour in sorted order = min id */
            lp[v] = ((uint64_t)r << 32) | u;
            mark[v] = 1;
            break;
          }
        }
      }
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < (int64_t)fsize; i++) inF[front[i]] = 0;
      uint64_t k = 0;
      for (uint64_t v = 0; v < n; v++)
        if (mark[v]) front[k++] = (uint32_t)v;
      fsize = k;
      fdense = 1;
    } else {
      const uint64_t lvl = (uint64_t)r << 32;
#pragma omp parallel num_threads(T)
      {
        vec32 *mine = &loc[omp_get_thread_num()];
        mine->len = 0;
#pragma omp for schedule(dynamic, 64)
        for (int64_t i = 0; i < (int64_t)fsize; i++) {
          uint32_t u = front[i];
          for (uint64_t j = offsets[u]; j < offsets[u + 1]; j++) {
            uint32_t v = nbrs[j];
            uint64_t cur = __atomic_load_n(&lp[v], __ATOMIC_RELAXED);
            if (cur < lvl) continue; /* reached in an earlier round */
            uint64_t old;
            if (atomic_min_u64(&lp[v], lvl | u, &old) && old == NONE64) vec_push(mine, v);
          }
        }
      }
      uint64_t k = 0;
      for (int t = 0; t < T; t++) {
        memcpy(front + k, loc[t].a, loc[t].len * sizeof(uint32_t));
        k += loc[t].len;
      }
      fsize = k;
      fdense = 0;
    }
    r++;
  }
#pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < (int64_t)n; v++) {
    uint64_t x = lp[v];
    parent[v] = x == NONE64 ? ORC_NONE : (uint32_t)x;
    if (level) level[v] = x == NONE64 ? ORC_NONE : (uint32_t)(x >> 32);
  }
  for (int t = 0; t < T; t++) free(loc[t].a);
  free(loc);
  free(lp);
  free(front);
  free(inF);
  free(mark);
  return r;
}

/* ------------------------------------------------------------------ connectivity */

/* find_compress (SimpleUnionAsync/Connectivity.h:32-47) */
static inline uint32_t find_compress(uint32_t i, uint32_t *parents) {
  uint32_t j = i;
  if (__atomic_load_n(&parents[j], __ATOMIC_RELAXED) == j) return j;
  do {
    j = __atomic_load_n(&parents[j], __ATOMIC_RELAXED);
  } while (__atomic_load_n(&parents[j], __ATOMIC_RELAXED) != j);
  uint32_t tmp;
  while ((tmp = __atomic_load_n(&parents[i], __ATOMIC_RELAXED)) > j) {
    __atomic_store_n(&parents[i], j, __ATOMIC_RELAXED);
    i = tmp;
  }
  return j;
}

/* unite_impl (Connectivity.h:49-65): CAS the larger root onto the smaller */
static inline void unite(uint32_t u, uint32_t v, uint32_t *parents) {
  for (;;) {
    u = find_compress(u, parents);
    v = find_compress(v, parents);
    if (u == v) break;
    if (u > v) {
      uint32_t e = u;
      if (__atomic_load_n(&parents[u], __ATOMIC_RELAXED) == u &&
          __atomic_compare_exchange_n(&parents[u], &e, v, 0, __ATOMIC_RELAXED, __ATOMIC_RELAXED))
        break;
    } else {
      uint32_t e = v;
      if (__atomic_load_n(&parents[v], __ATOMIC_RELAXED) == v &&
          __atomic_compare_exchange_n(&parents[v], &e, u, 0, __ATOMIC_RELAXED, __ATOMIC_RELAXED))
        break;
    }
  }
}

void orc_cc(uint64_t n, const uint64_t *offsets, const uint32_t *nbrs, uint32_t *label) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; i++) label[i] = (uint32_t)i;
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < (int64_t)n; i++)
    for (uint64_t j = offsets[i]; j < offsets[i + 1]; j++) unite((uint32_t)i, nbrs[j], label);
  /* finish(): SimpleUnionAsyncStruct::finish, Connectivity.h:113-116 */
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; i++) find_compress((uint32_t)i, label);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; i++) label[i] = __atomic_load_n(&label[label[i]], __ATOMIC_RELAXED);
}

void orc_bfs_cc(uint64_t n, const uint64_t *offsets, const uint32_t *nbrs, uint32_t *label) {
  /* BFSCC/Connectivity.h:57-88: sequential outer loop over vertices not yet
   * covered; each BFS labels its component with its source. */
  for (uint64_t v = 0; v < n; v++) label[v] = ORC_NONE;
  uint32_t *q = xmalloc(n * sizeof(uint32_t));
  for (uint64_t s = 0; s < n; s++) {
    if (label[s] != ORC_NONE) continue;
    uint64_t head = 0, tail = 0;
    q[tail++] = (uint32_t)s;
    label[s] = (uint32_t)s;
    while (head < tail) {
      uint32_t u = q[head++];
      for (uint64_t j = offsets[u]; j < offsets[u + 1]; j++) {
        uint32_t v = nbrs[j];
        if (label[v] == ORC_NONE) {
          label[v] = (uint32_t)s;
          q[tail++] = v;
        }
      }
    }
  }
  free(q);
}

/* ------------------------------------------------------------------ PageRank */

void orc_pagerank(uint64_t n, const uint64_t *offsets, const uint32_t *nbrs, double eps,
                  uint32_t max_iters, double *p_out, uint32_t *iters_out, double *l1_out) {
  const double damping = 0.85;
  const double added = (1 - damping) * (1 / (double)n);
  const double one_over_n = 1 / (double)n;
  double *p_curr = xmalloc(n * sizeof(double));
  double *p_next = xmalloc(n * sizeof(double));
  double *p_div = xmalloc(n * sizeof(double));
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; i++) {
    p_curr[i] = one_over_n;
    p_next[i] = 0;
    p_div[i] = one_over_n / (double)(offsets[i + 1] - offsets[i]); /* inf when deg 0, never read */
  }
  const int64_t CH = 4096;
  const int64_t nch = ((int64_t)n + CH - 1) / CH;
  double *part = xmalloc((size_t)(nch ? nch : 1) * sizeof(double));
  uint32_t iter = 0;
  double L1 = 0;
  double *last = NULL;
  while (iter++ < max_iters) {
    /* edgeMapReduce_dense with no_output (edge_map_reduce.h:469-484).  The
     * reference's apply_f (PageRank.h:153-160) rewrites p_div[u] inside the
     * same parallel loop whose map_f reads p_div, so its result depends on the
     * schedule; the restatement takes the Jacobi order that the commented-out
     * map_f (p_curr[s] / degrees[s], PageRank.h:151) spells out: every read in
     * an iteration sees the previous iteration's p_div. */
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t v = 0; v < (int64_t)n; v++) {
      double s = 0.0;
      for (uint64_t j = offsets[v]; j < offsets[v + 1]; j++) s += p_div[nbrs[j]];
      p_next[v] = damping * s + added;
    }
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < nch; c++) {
      double acc = 0.0;
      int64_t hi = (c + 1) * CH < (int64_t)n ? (c + 1) * CH : (int64_t)n;
      for (int64_t i = c * CH; i < hi; i++) {
        acc += fabs(p_curr[i] - p_next[i]);
        p_curr[i] = 0;
        p_div[i] = p_next[i] / (double)(offsets[i + 1] - offsets[i]);
      }
      part[c] = acc;
    }
    L1 = 0;
    for (int64_t c = 0; c < nch; c++) L1 += part[c];
    last = p_next;
    if (L1 < eps) break;
    double *t = p_curr;
    p_curr = p_next;
    p_next = t;
  }
  if (iter > max_iters) iter = max_iters;
  /* The reference returns p_next after its final swap, i.e. the zeroed
   * previous iterate whenever max_iters ends the loop (PageRank.h:181-192);
   * the restatement returns the last computed iterate in both cases. */
  memcpy(p_out, last ? last : p_curr, n * sizeof(double));
  if (iters_out) *iters_out = iter;
  if (l1_out) *l1_out = L1;
  free(part);
  free(p_curr);
  free(p_next);
  free(p_div);
}

/* ------------------------------------------------------------------ PageRank, delta variant */

void orc_pagerank_delta(uint64_t n, const uint64_t *offsets, const uint32_t *nbrs, double eps, double local_eps,
                        uint32_t max_iters, double *p, uint32_t *rounds_out, double *l1_out) {
  /* delta::PageRankDelta (PageRank.h:340-398).  nghSum[v] = sum of
   * delta_over_degree over v's neighbours in the frontier: the dense branch of
   * sparse_or_dense (PageRank.h:235-267, edgeMapReduce_dense over in-edges)
   * and the push branch (PR_Delta_F, PageRank.h:207-229) compute the same
   * sum; the restatement adds left to right over sorted neighbours. */
  const double damping = 0.85;
  const double one_over_n = 1 / (double)n;
  const double added = (1 - damping) * one_over_n;
  double *delta = xmalloc((n ? n : 1) * sizeof(double));
  double *dod = xmalloc((n ? n : 1) * sizeof(double));
  double *ngh = xmalloc((n ? n : 1) * sizeof(double));
  uint8_t *front = xmalloc(n ? n : 1);
  uint8_t *next = xmalloc(n ? n : 1);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; i++) {
    p[i] = 0.0;
    delta[i] = one_over_n;
    dod[i] = one_over_n / (double)(offsets[i + 1] - offsets[i]); /* inf when deg 0, never read */
    ngh[i] = 0.0;
    front[i] = 1;
  }
  uint32_t round = 0;
  double L1 = 0;
  while (round++ < max_iters) {
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t v = 0; v < (int64_t)n; v++) {
      double s = 0.0;
      for (uint64_t j = offsets[v]; j < offsets[v + 1]; j++)
        if (front[nbrs[j]]) s += dod[nbrs[j]];
      ngh[v] = s;
    }
    /* vertexFilter over all vertices: PR_Vertex_F_FirstRound (:271-290) in the
     * first round, PR_Vertex_F (:307-323) after */
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; i++) {
      const double deg = (double)(offsets[i + 1] - offsets[i]);
      if (round == 1) {
        const double pre_init = damping * ngh[i] + added;
        p[i] += pre_init;
        const double nd = pre_init - one_over_n;
        delta[i] = nd;
        dod[i] = nd / deg;
        next[i] = nd > local_eps * p[i];
      } else {
        const double nd = ngh[i] * damping;
        delta[i] = nd;
        dod[i] = nd / deg;
        if (fabs(nd) > local_eps * p[i]) {
          p[i] += nd;
          next[i] = 1;
        } else {
          next[i] = 0;
        }
      }
      ngh[i] = 0.0;
    }
    L1 = 0;
    for (uint64_t i = 0; i < n; i++) L1 += fabs(delta[i]);
    if (L1 < eps) break;
    uint8_t *t = front;
    front = next;
    next = t;
  }
  if (round > max_iters) round = max_iters;
  if (rounds_out) *rounds_out = round;
  if (l1_out) *l1_out = L1;
  free(delta);
  free(dod);
  free(ngh);
  free(front);
  free(next);
}

/* byte-PD (see oracle.h): byte_pd_amortized.cc:7-55 and
 * byte_pd_amortized.h:1100-1155 restated. */
static uint64_t varint_len(uint64_t v) { /* 7 bits per byte, at least 0 bytes for 0 */
  uint64_t k = 0;
  while (v) {
    k++;
    v >>= 7;
  }
  return k;
}

static uint64_t first_len(int64_t diff) {
  uint64_t a = (uint64_t)(diff < 0 ? -diff : diff);
  return 1 + varint_len(a >> 6);
}

static uint64_t vertex_bytes(const uint32_t *nb, uint64_t d, uint32_t src, uint32_t P) {
  if (!d) return 0;
  const uint64_t nbk = 1 + (d - 1) / P;
  uint64_t bytes = 4 + 4 * (nbk - 1) + 4 * nbk;
  for (uint64_t e = 0; e < d; e++)
    bytes += (e % P == 0) ? first_len((int64_t)nb[e] - (int64_t)src) : varint_len((uint64_t)(nb[e] - nb[e - 1]));
  return bytes;
}

uint64_t orc_bytepd_sizes(uint64_t n, const uint64_t *offsets, const uint32_t *nbrs, uint32_t P, uint64_t *sizes) {
  uint64_t total = 0;
#pragma omp parallel for schedule(dynamic, 1024) reduction(+ : total)
  for (int64_t v = 0; v < (int64_t)n; v++) {
    sizes[v] = vertex_bytes(nbrs + offsets[v], offsets[v + 1] - offsets[v], (uint32_t)v, P);
    total += sizes[v];
  }
  return total;
}

static void put_u32(unsigned char *p, uint32_t x) { memcpy(p, &x, 4); }
static uint32_t get_u32(const unsigned char *p) {
  uint32_t x;
  memcpy(&x, p, 4);
  return x;
}

static unsigned char *put_first(unsigned char *p, int64_t diff) {
  uint64_t a = (uint64_t)(diff < 0 ? -diff : diff);
  unsigned char b = (unsigned char)(a & 0x3f);
  if (diff < 0) b |= 0x40;
  a >>= 6;
  if (a) b |= 0x80;
  *p++ = b;
  while (a) {
    unsigned char c = (unsigned char)(a & 0x7f);
    a >>= 7;
    if (a) c |= 0x80;
    *p++ = c;
  }
  return p;
}

static unsigned char *put_diff(unsigned char *p, uint64_t a) {
  while (a) {
    unsigned char c = (unsigned char)(a & 0x7f);
    a >>= 7;
    if (a) c |= 0x80;
    *p++ = c;
  }
  return p;
}

void orc_bytepd_encode(uint64_t n, const uint64_t *offsets, const uint32_t *nbrs, uint32_t P,
                       const uint64_t *byte_offsets, unsigned char *bytes) {
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t v = 0; v < (int64_t)n; v++) {
    const uint64_t d = offsets[v + 1] - offsets[v];
    if (!d) continue;
    const uint32_t *nb = nbrs + offsets[v];
    unsigned char *base = bytes + byte_offsets[v];
    const uint64_t nbk = 1 + (d - 1) / P;
    put_u32(base, (uint32_t)d);
    unsigned char *p = base + 4 + 4 * (nbk - 1);
    for (uint64_t i = 0; i < nbk; i++) {
      if (i > 0) put_u32(base + 4 + 4 * (i - 1), (uint32_t)(p - base));
      put_u32(p, (uint32_t)(i * P));
      p += 4;
      const uint64_t e0 = i * P, e1 = e0 + P < d ? e0 + P : d;
      p = put_first(p, (int64_t)nb[e0] - (int64_t)v);
      for (uint64_t e = e0 + 1; e < e1; e++) p = put_diff(p, (uint64_t)(nb[e] - nb[e - 1]));
    }
  }
}

int orc_bytepd_decode(uint64_t n, const uint64_t *byte_offsets, const uint32_t *degrees, const unsigned char *bytes,
                      uint64_t nbytes, uint32_t P, uint64_t *offsets, uint32_t *nbrs) {
  offsets[0] = 0;
  for (uint64_t v = 0; v < n; v++) offsets[v + 1] = offsets[v] + degrees[v];
  int bad = 0;
#pragma omp parallel for schedule(dynamic, 1024) reduction(| : bad)
  for (int64_t v = 0; v < (int64_t)n; v++) {
    const uint64_t d = degrees[v];
    if (!d) continue;
    const unsigned char *base = bytes + byte_offsets[v], *end = bytes + byte_offsets[v + 1];
    if (byte_offsets[v + 1] > nbytes || base + 4 > end || get_u32(base) != d) {
      bad = 1;
      continue;
    }
    const uint64_t nbk = 1 + (d - 1) / P;
    uint32_t *out = nbrs + offsets[v];
    for (uint64_t i = 0; i < nbk && !bad; i++) {
      const unsigned char *p = i == 0 ? base + 4 + 4 * (nbk - 1) : base + get_u32(base + 4 + 4 * (i - 1));
      const uint64_t e0 = get_u32(p), e1 = i + 1 == nbk ? d : get_u32(base + get_u32(base + 4 + 4 * i));
      p += 4;
      int64_t last = 0;
      for (uint64_t e = e0; e < e1; e++) {
        uint64_t a = 0;
        int shift, neg = 0;
        if (p >= end) {
          bad = 1;
          break;
        }
        unsigned char b = *p++;
        if (e == e0) {
          a = b & 0x3f;
          neg = (b & 0x40) != 0;
          shift = 6;
        } else {
          a = b & 0x7f;
          shift = 7;
        }
        while ((b & 0x80) && p < end && shift < 64) {
          b = *p++;
          a |= (uint64_t)(b & 0x7f) << shift;
          shift += 7;
        }
        last = e == e0 ? (neg ? (int64_t)v - (int64_t)a : (int64_t)v + (int64_t)a) : last + (int64_t)a;
        out[e] = (uint32_t)last;
      }
    }
  }
  return bad ? -1 : 0;
}

/* Map.h:8-18 and RemoteRead/Map.h:21-33: a parallel_for over vertices, each
 * summing over its neighbours, combined by a Reducer_sum<size_t>. */
uint64_t orc_map_sum(uint64_t n, const uint64_t *offsets, const uint32_t *nbrs) {
  uint64_t total = 0;
#pragma omp parallel for schedule(dynamic, 1024) reduction(+ : total)
  for (int64_t i = 0; i < (int64_t)n; i++)
    for (uint64_t e = offsets[i]; e < offsets[i + 1]; e++) total += nbrs[e];
  return total;
}

static uint64_t remote_at(const unsigned char *r, uint32_t width, uint32_t v) {
  switch (width) {
    case 0: return (((const uint64_t *)r)[v >> 6] >> (v & 63)) & 1u;
    case 1: return r[v];
    case 2: return ((const uint16_t *)r)[v];
    case 4: return ((const uint32_t *)r)[v];
    default: return *(const uint64_t *)(r + (uint64_t)v * width);
  }
}

uint64_t orc_map_remote(uint64_t n, const uint64_t *offsets, const uint32_t *nbrs, const void *remote,
                        uint32_t width) {
  const unsigned char *r = (const unsigned char *)remote;
  uint64_t total = 0;
#pragma omp parallel for schedule(dynamic, 1024) reduction(+ : total)
  for (int64_t i = 0; i < (int64_t)n; i++)
    for (uint64_t e = offsets[i]; e < offsets[i + 1]; e++) total += remote_at(r, width, nbrs[e]);
  return total;
}

/* ------------------------------------------------------------------ triangles */

uint64_t orc_triangle_count(uint64_t n, const uint64_t *offsets, const uint32_t *nbrs) {
  /* rankNodes (Triangle.h:57-68): order by degree; ties by id */
  uint64_t *key = xmalloc((n ? n : 1) * sizeof(uint64_t));
#pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < (int64_t)n; v++) key[v] = ((offsets[v + 1] - offsets[v]) << 32) | (uint64_t)v;
  radix_sort_u64(key, n);
  uint32_t *rank = xmalloc((n ? n : 1) * sizeof(uint32_t));
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; i++) rank[(uint32_t)key[i]] = (uint32_t)i;
  free(key);
  /* filterGraph (gbbs/graph_mutation.h:15-81) keeping rank[u] < rank[v] */
  uint64_t *doff = xmalloc((n + 1) * sizeof(uint64_t));
  doff[0] = 0;
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t u = 0; u < (int64_t)n; u++) {
    uint64_t c = 0;
    for (uint64_t j = offsets[u]; j < offsets[u + 1]; j++) c += rank[u] < rank[nbrs[j]];
    doff[u + 1] = c;
  }
  for (uint64_t u = 0; u < n; u++) doff[u + 1] += doff[u];
  uint32_t *dn = xmalloc((doff[n] ? doff[n] : 1) * sizeof(uint32_t));
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t u = 0; u < (int64_t)n; u++) {
    uint64_t k = doff[u];
    for (uint64_t j = offsets[u]; j < offsets[u + 1]; j++)
      if (rank[u] < rank[nbrs[j]]) dn[k++] = nbrs[j];
  }
  /* CountDirectedBalanced (Triangle.h:99-150) with intersection::merge
   * (gbbs/intersect.h:111-134) */
  uint64_t total = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : total)
  for (int64_t u = 0; u < (int64_t)n; u++) {
    for (uint64_t j = doff[u]; j < doff[u + 1]; j++) {
      uint32_t v = dn[j];
      uint64_t a = doff[u], ae = doff[u + 1], b = doff[v], be = doff[v + 1];
      while (a < ae && b < be) {
        if (dn[a] == dn[b]) {
          total++;
          a++;
          b++;
        } else if (dn[a] < dn[b]) {
          a++;
        } else {
          b++;
        }
      }
    }
  }
  free(rank);
  free(doff);
  free(dn);
  return total;
}

/* ------------------------------------------------------------------ container model */

struct orc_store {
  uint64_t n, m;
  uint32_t **adj;
  uint32_t *deg, *cap;
};

orc_store *orc_store_create(uint64_t n, const uint64_t *offsets, const uint32_t *nbrs) {
  orc_store *s = xmalloc(sizeof(orc_store));
  s->n = n;
  s->m = offsets ? offsets[n] : 0;
  s->adj = xmalloc((n ? n : 1) * sizeof(uint32_t *));
  s->deg = xmalloc((n ? n : 1) * sizeof(uint32_t));
  s->cap = xmalloc((n ? n : 1) * sizeof(uint32_t));
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t v = 0; v < (int64_t)n; v++) {
    uint64_t d = offsets ? offsets[v + 1] - offsets[v] : 0;
    s->deg[v] = (uint32_t)d;
    s->cap[v] = (uint32_t)(d ? d : 0);
    s->adj[v] = d ? xmalloc(d * sizeof(uint32_t)) : NULL;
    if (d) memcpy(s->adj[v], nbrs + offsets[v], d * sizeof(uint32_t));
  }
  return s;
}

void orc_store_destroy(orc_store *s) {
  if (!s) return;
  for (uint64_t v = 0; v < s->n; v++) free(s->adj[v]);
  free(s->adj);
  free(s->deg);
  free(s->cap);
  free(s);
}

uint64_t orc_store_num_edges(const orc_store *s) { return s->m; }

/* group boundaries of a sorted key array by src (the high word) */
static uint64_t group_by_src(const uint64_t *k, uint64_t cnt, uint64_t **starts_out) {
  uint64_t *st = xmalloc((cnt + 1) * sizeof(uint64_t));
  uint64_t g = 0;
  for (uint64_t i = 0; i < cnt; i++)
    if (i == 0 || (k[i] >> 32) != (k[i - 1] >> 32)) st[g++] = i;
  st[g] = cnt;
  *starts_out = st;
  return g;
}

static uint64_t store_update(orc_store *s, const uint64_t *keys, uint64_t count, int insert) {
  if (count == 0) return 0;
  uint64_t *k = xmalloc(count * sizeof(uint64_t));
  memcpy(k, keys, count * sizeof(uint64_t));
  uint64_t u = orc_sort_unique_u64(k, count);
  uint64_t *st;
  uint64_t g = group_by_src(k, u, &st);
  uint64_t changed = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : changed)
  for (int64_t q = 0; q < (int64_t)g; q++) {
    uint32_t v = (uint32_t)(k[st[q]] >> 32);
    if (v >= s->n) continue;
    uint64_t bl = st[q + 1] - st[q];
    const uint64_t *b = k + st[q];
    uint32_t d = s->deg[v];
    uint32_t *a = s->adj[v];
    uint32_t *out = xmalloc(((uint64_t)d + bl) * sizeof(uint32_t));
    uint64_t i = 0, j = 0, o = 0;
    if (insert) {
      while (i < d || j < bl) {
        uint32_t bj = j < bl ? (uint32_t)b[j] : 0;
        if (j >= bl || (i < d && a[i] < bj)) {
          out[o++] = a[i++];
        } else if (i >= d || bj < a[i]) {
          out[o++] = bj;
          j++;
        } else {
          out[o++] = a[i++];
          j++;
        }
      }
      changed += o - d;
    } else {
      while (i < d) {
        while (j < bl && (uint32_t)b[j] < a[i]) j++;
        if (j < bl && (uint32_t)b[j] == a[i])
          i++;
        else
          out[o++] = a[i++];
      }
      changed += d - o;
    }
    free(s->adj[v]);
    s->adj[v] = out;
    s->deg[v] = (uint32_t)o;
    s->cap[v] = (uint32_t)(d + bl);
  }
  if (insert)
    s->m += changed;
  else
    s->m -= changed;
  free(st);
  free(k);
  return changed;
}

uint64_t orc_store_insert_batch(orc_store *s, const uint64_t *keys, uint64_t count) {
  return store_update(s, keys, count, 1);
}

uint64_t orc_store_remove_batch(orc_store *s, const uint64_t *keys, uint64_t count) {
  return store_update(s, keys, count, 0);
}

void orc_store_export_csr(const orc_store *s, uint64_t *offsets, uint32_t *nbrs) {
  offsets[0] = 0;
  for (uint64_t v = 0; v < s->n; v++) offsets[v + 1] = offsets[v] + s->deg[v];
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t v = 0; v < (int64_t)s->n; v++)
    if (s->deg[v]) memcpy(nbrs + offsets[v], s->adj[v], s->deg[v] * sizeof(uint32_t));
}
