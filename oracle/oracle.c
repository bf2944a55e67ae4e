/*
 * oracle.c -- CPU restatement of chapeiro/proteus's hash-join, group-by and
 * radix-cluster semantics.  TEST INFRASTRUCTURE ONLY: the oracle the CUDA
 * path's results are compared with, and the CPU baseline of the benchmark;
 * never part of the product.
 * Every function names the reference file:line it restates.
 */
#define _GNU_SOURCE
#include "oracle.h"

#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* Codes of gbjoin.h (kept numerically identical). */
enum { A_COUNT = 0, A_SUM = 1, A_MIN = 2, A_MAX = 3, A_OR = 4, A_AND = 5 };
enum {
  V_ONE = 0,
  V_BUILD = 1,
  V_PROBE = 2,
  V_PRODUCT = 3,
  V_BUILD_ROWID = 4,
  V_PROBE_ROWID = 5,
  V_ROWID_XOR = 6,
  V_BUILD_KEY = 7
};

/* expressions-hasher.cpp:39-58: sext to i64, xor-shift / multiply with the
 * murmur3 fmix32 constants, all in 64-bit arithmetic. */
uint64_t orc_hash_int32(int32_t key) {
  uint64_t h = (uint64_t)(int64_t)key;
  h ^= h >> 16;
  h *= 0x85ebca6bULL;
  h ^= h >> 13;
  h *= 0xc2b2ae35ULL;
  h ^= h >> 16;
  return h;
}

/* hashInt64 (expressions-hasher.cpp:66-84): the murmur3 64-bit finaliser. */
uint64_t orc_hash_int64(int64_t key) {
  uint64_t h = (uint64_t)key;
  h ^= h >> 33;
  h *= 0xff51afd7ed558ccdULL;
  h ^= h >> 33;
  h *= 0xc4ceb9fe1a85ec53ULL;
  h ^= h >> 33;
  return h;
}

/* gpu-partitioned-hash-join-chained-helpers.cpp:49-56 (32-bit wrap). */
uint32_t orc_hashd(int32_t key) {
  uint32_t h = (uint32_t)key;
  h ^= h >> 16;
  h *= 0x85ebca6bu;
  h ^= h >> 13;
  h *= 0xc2b2ae35u;
  h ^= h >> 16;
  return h;
}

static int auto_hash_bits(uint64_t n) {
  /* relbuilder.cpp:653-668: ceil(log2(maxBuildInputSize)) + 1 */
  int b = 0;
  while ((1ULL << b) < (n ? n : 1)) ++b;
  return b + 1;
}

static inline uint64_t bucket_of(int32_t key, int hash_bits) {
  /* hash-join-chained.cpp:233-239: URem 2^hash_bits */
  return orc_hash_int32(key) & ((1ULL << hash_bits) - 1);
}

/* ------------------------------------------------------------ hash join */

int orc_join_build(const int32_t *keys, const int32_t *payload, uint64_t n,
                   int32_t hash_bits, orc_chained_table *t) {
  if (!t || (n && !keys) || n > 0x7fffffffULL) return -1;
  if (hash_bits <= 0) hash_bits = auto_hash_bits(n);
  if (hash_bits > 32) return -1;
  uint64_t nb = 1ULL << hash_bits;
  t->head = (int32_t *)malloc(nb * sizeof(int32_t));
  t->next = (int32_t *)malloc((n ? n : 1) * sizeof(int32_t));
  if (!t->head || !t->next) return -1;
  memset(t->head, 0xff, nb * sizeof(int32_t)); /* open_build: memset -1 */
  t->key = keys;
  t->key64 = 0;
  t->payload = payload;
  t->n = n;
  t->hash_bits = hash_bits;
  /* generate_build (hash-join-chained.cpp:262-319):
   *   idx = cnt++; old = xchg(head[h], idx); packet[idx] = {old, key, ...} */
  for (uint64_t i = 0; i < n; ++i) {
    uint64_t h = bucket_of(keys[i], hash_bits);
    t->next[i] = t->head[h];
    t->head[h] = (int32_t)i;
  }
  return 0;
}

typedef struct {
  const int32_t *keys;
  orc_chained_table *t;
  uint64_t lo, hi;
  int32_t *cnt;
} build_mt_arg;

static void *build_mt_worker(void *p) {
  build_mt_arg *a = (build_mt_arg *)p;
  for (uint64_t k = a->lo; k < a->hi; ++k) {
    /* hash-join-chained-morsel.cpp:29-129: seq-cst atomic index + xchg */
    int32_t idx = __atomic_fetch_add(a->cnt, 1, __ATOMIC_SEQ_CST);
    (void)idx;
    uint64_t i = k; /* store each row at its own position (idx order only
                       affects chain order, not results) */
    uint64_t h = bucket_of(a->keys[i], a->t->hash_bits);
    int32_t old = __atomic_exchange_n(&a->t->head[h], (int32_t)i,
                                      __ATOMIC_SEQ_CST);
    a->t->next[i] = old;
  }
  return 0;
}

int orc_join_build_mt(const int32_t *keys, const int32_t *payload, uint64_t n,
                      int32_t hash_bits, int threads, orc_chained_table *t) {
  if (threads <= 1 || n < 65536)
    return orc_join_build(keys, payload, n, hash_bits, t);
  if (!t || !keys || n > 0x7fffffffULL) return -1;
  if (hash_bits <= 0) hash_bits = auto_hash_bits(n);
  if (hash_bits > 32) return -1;
  uint64_t nb = 1ULL << hash_bits;
  t->head = (int32_t *)malloc(nb * sizeof(int32_t));
  t->next = (int32_t *)malloc(n * sizeof(int32_t));
  if (!t->head || !t->next) return -1;
  memset(t->head, 0xff, nb * sizeof(int32_t));
  t->key = keys;
  t->key64 = 0;
  t->payload = payload;
  t->n = n;
  t->hash_bits = hash_bits;
  int32_t cnt = 0;
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * threads);
  build_mt_arg *args = (build_mt_arg *)malloc(sizeof(build_mt_arg) * threads);
  uint64_t chunk = (n + threads - 1) / threads;
  for (int i = 0; i < threads; ++i) {
    args[i].keys = keys;
    args[i].t = t;
    args[i].lo = i * chunk < n ? i * chunk : n;
    args[i].hi = (i + 1) * chunk < n ? (i + 1) * chunk : n;
    args[i].cnt = &cnt;
    pthread_create(&th[i], 0, build_mt_worker, &args[i]);
  }
  for (int i = 0; i < threads; ++i) pthread_join(th[i], 0);
  free(th);
  free(args);
  return 0;
}

void orc_join_free(orc_chained_table *t) {
  if (!t) return;
  free(t->head);
  free(t->next);
  t->head = t->next = 0;
}

typedef struct {
  int64_t v[8];
} acc8;

/* Identities: MIN/MAX of nothing as int64 extremes; the logical AND of
 * nothing is true (LogAndMonoid, gmonoids.cpp:286-290; its atomic form only
 * ever stores false, :292-321), the logical OR of nothing false. */
static void acc_init(acc8 *a, const int32_t *ops, int n_aggs) {
  for (int j = 0; j < n_aggs; ++j) {
    if (ops[j] == A_MIN)
      a->v[j] = INT64_MAX;
    else if (ops[j] == A_MAX)
      a->v[j] = INT64_MIN;
    else if (ops[j] == A_AND)
      a->v[j] = 1;
    else
      a->v[j] = 0;
  }
}

static inline int64_t operand_value(int operand, int64_t bkey, int64_t bval,
                                    int64_t pval, int64_t brow, int64_t prow) {
  switch (operand) {
    case V_ONE: return 1;
    case V_BUILD: return bval;
    case V_PROBE: return pval;
    case V_PRODUCT: return bval * pval;
    case V_BUILD_ROWID: return brow;
    case V_PROBE_ROWID: return prow;
    case V_ROWID_XOR: return brow ^ prow;
    case V_BUILD_KEY: return bkey;
    default: return 0;
  }
}

static inline void acc_update(acc8 *a, const int32_t *ops,
                              const int32_t *operands, int n_aggs,
                              int64_t bkey, int64_t bval, int64_t pval,
                              int64_t brow, int64_t prow) {
  for (int j = 0; j < n_aggs; ++j) {
    int64_t x = operand_value(operands[j], bkey, bval, pval, brow, prow);
    switch (ops[j]) {
      case A_COUNT: a->v[j] += 1; break;
      case A_SUM: a->v[j] += x; break;
      case A_MIN: if (x < a->v[j]) a->v[j] = x; break;
      case A_MAX: if (x > a->v[j]) a->v[j] = x; break;
      /* LogOrMonoid / LogAndMonoid (gmonoids.cpp:286-290, 363-376): the
       * operand is a truth value, any non-zero value is true */
      case A_OR: a->v[j] = a->v[j] | (x != 0); break;
      case A_AND: a->v[j] = a->v[j] & (x != 0); break;
    }
  }
}

static void acc_merge(acc8 *dst, const acc8 *src, const int32_t *ops,
                      int n_aggs) {
  for (int j = 0; j < n_aggs; ++j) {
    if (ops[j] == A_MIN) {
      if (src->v[j] < dst->v[j]) dst->v[j] = src->v[j];
    } else if (ops[j] == A_MAX) {
      if (src->v[j] > dst->v[j]) dst->v[j] = src->v[j];
    } else if (ops[j] == A_OR) {
      dst->v[j] |= src->v[j];
    } else if (ops[j] == A_AND) {
      dst->v[j] &= src->v[j];
    } else {
      dst->v[j] += src->v[j];
    }
  }
}

static int check_aggs(const int32_t *ops, const int32_t *operands, int n) {
  if (n < 0 || n > 8 || (n && (!ops || !operands))) return -1;
  for (int j = 0; j < n; ++j) {
    if (ops[j] < A_COUNT || ops[j] > A_AND) return -1;
    if (operands[j] < V_ONE || operands[j] > V_BUILD_KEY) return -1;
  }
  return 0;
}

typedef struct {
  const orc_chained_table *t;
  const int32_t *keys, *payload;
  uint64_t lo, hi;
  const int32_t *ops, *operands;
  int n_aggs;
  acc8 acc;
} probe_arg;

/* generate_probe (hash-join-chained.cpp:321-566): cur = head[h]; while
 * (cur != ~0) { load packet; cur = packet.next; if (key == probe key)
 * consume(parent) } -- the parent here is the fused aggregate. */
static void *probe_worker(void *p) {
  probe_arg *a = (probe_arg *)p;
  const orc_chained_table *t = a->t;
  for (uint64_t i = a->lo; i < a->hi; ++i) {
    int32_t k = a->keys[i];
    int64_t pv = a->payload ? a->payload[i] : 0;
    for (int32_t cur = t->head[bucket_of(k, t->hash_bits)]; cur != -1;
         cur = t->next[cur]) {
      if (t->key[cur] == k) {
        int64_t bv = t->payload ? t->payload[cur] : 0;
        acc_update(&a->acc, a->ops, a->operands, a->n_aggs, k, bv, pv, cur,
                   (int64_t)i);
      }
    }
  }
  return 0;
}

int orc_join_probe_agg(const orc_chained_table *t, const int32_t *keys,
                       const int32_t *payload, uint64_t n, const int32_t *ops,
                       const int32_t *operands, int32_t n_aggs, int64_t *out,
                       int threads) {
  if (!t || (n && !keys) || !out || check_aggs(ops, operands, n_aggs))
    return -1;
  if (threads < 1) threads = 1;
  if (n < 65536) threads = 1;
  probe_arg *args = (probe_arg *)calloc(threads, sizeof(probe_arg));
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * threads);
  uint64_t chunk = (n + threads - 1) / threads;
  for (int i = 0; i < threads; ++i) {
    probe_arg *a = &args[i];
    a->t = t;
    a->keys = keys;
    a->payload = payload;
    a->lo = i * chunk < n ? i * chunk : n;
    a->hi = (i + 1) * chunk < n ? (i + 1) * chunk : n;
    a->ops = ops;
    a->operands = operands;
    a->n_aggs = n_aggs;
    acc_init(&a->acc, ops, n_aggs);
    if (threads == 1)
      probe_worker(a);
    else
      pthread_create(&th[i], 0, probe_worker, a);
  }
  acc8 total;
  acc_init(&total, ops, n_aggs);
  for (int i = 0; i < threads; ++i) {
    if (threads > 1) pthread_join(th[i], 0);
    acc_merge(&total, &args[i].acc, ops, n_aggs);
  }
  for (int j = 0; j < n_aggs; ++j) out[j] = total.v[j];
  free(args);
  free(th);
  return 0;
}

int64_t orc_join_probe_pairs(const orc_chained_table *t, const int32_t *keys,
                             uint64_t n, int32_t *build_rows,
                             int32_t *probe_rows, uint64_t cap) {
  if (!t || (n && !keys)) return -1;
  int64_t m = 0;
  for (uint64_t i = 0; i < n; ++i) {
    int32_t k = keys[i];
    for (int32_t cur = t->head[bucket_of(k, t->hash_bits)]; cur != -1;
         cur = t->next[cur]) {
      if (t->key[cur] == k) {
        if ((uint64_t)m < cap) {
          if (build_rows) build_rows[m] = cur;
          if (probe_rows) probe_rows[m] = (int32_t)i;
        }
        ++m;
      }
    }
  }
  return m;
}

/* ------------------------------------------------ hash join, int64 keys */

static inline uint64_t bucket_of64(int64_t key, int hash_bits) {
  return orc_hash_int64(key) & ((1ULL << hash_bits) - 1);
}

/* generate_build (hash-join-chained.cpp:262-319) with an int64 key. */
int orc_join_build_i64(const int64_t *keys, const int32_t *payload, uint64_t n,
                       int32_t hash_bits, orc_chained_table *t) {
  if (!t || (n && !keys) || n > 0x7fffffffULL) return -1;
  if (hash_bits <= 0) hash_bits = auto_hash_bits(n);
  if (hash_bits > 32) return -1;
  uint64_t nb = 1ULL << hash_bits;
  t->head = (int32_t *)malloc(nb * sizeof(int32_t));
  t->next = (int32_t *)malloc((n ? n : 1) * sizeof(int32_t));
  if (!t->head || !t->next) return -1;
  memset(t->head, 0xff, nb * sizeof(int32_t));
  t->key = 0;
  t->key64 = keys;
  t->payload = payload;
  t->n = n;
  t->hash_bits = hash_bits;
  for (uint64_t i = 0; i < n; ++i) {
    uint64_t h = bucket_of64(keys[i], hash_bits);
    t->next[i] = t->head[h];
    t->head[h] = (int32_t)i;
  }
  return 0;
}

/* generate_probe (hash-join-chained.cpp:321-566) with an int64 key. */
int orc_join_probe_agg_i64(const orc_chained_table *t, const int64_t *keys,
                           const int32_t *payload, uint64_t n,
                           const int32_t *ops, const int32_t *operands,
                           int32_t n_aggs, int64_t *out) {
  if (!t || !t->key64 || (n && !keys) || !out || check_aggs(ops, operands, n_aggs))
    return -1;
  acc8 acc;
  acc_init(&acc, ops, n_aggs);
  for (uint64_t i = 0; i < n; ++i) {
    int64_t k = keys[i];
    int64_t pv = payload ? payload[i] : 0;
    for (int32_t cur = t->head[bucket_of64(k, t->hash_bits)]; cur != -1;
         cur = t->next[cur]) {
      if (t->key64[cur] == k) {
        int64_t bv = t->payload ? t->payload[cur] : 0;
        acc_update(&acc, ops, operands, n_aggs, k, bv, pv, cur, (int64_t)i);
      }
    }
  }
  for (int j = 0; j < n_aggs; ++j) out[j] = acc.v[j];
  return 0;
}

int64_t orc_join_probe_pairs_i64(const orc_chained_table *t,
                                 const int64_t *keys, uint64_t n,
                                 int32_t *build_rows, int32_t *probe_rows,
                                 uint64_t cap) {
  if (!t || !t->key64 || (n && !keys)) return -1;
  int64_t m = 0;
  for (uint64_t i = 0; i < n; ++i) {
    int64_t k = keys[i];
    for (int32_t cur = t->head[bucket_of64(k, t->hash_bits)]; cur != -1;
         cur = t->next[cur]) {
      if (t->key64[cur] == k) {
        if ((uint64_t)m < cap) {
          if (build_rows) build_rows[m] = cur;
          if (probe_rows) probe_rows[m] = (int32_t)i;
        }
        ++m;
      }
    }
  }
  return m;
}

/* ---------------------------------------------------------- radix cluster */

static inline uint32_t digit_of(int32_t key, uint32_t M, int R, int hashed) {
  /* radix-join.cpp:6 HASH_BIT_MODULO(K, MASK, NBITS) = ((K & MASK) >> NBITS) */
  uint32_t v = hashed ? orc_hashd(key) : (uint32_t)key;
  return (v & M) >> R;
}

/* radix_cluster_nopadding (radix-join.cpp:85-155): count per cluster, prefix
 * the cluster starts, then copy each tuple to dst[idx]++ in input order. */
void orc_radix_cluster(const int32_t *keys, const int32_t *payload,
                       uint64_t n, int32_t R, int32_t D, int32_t hashed,
                       int32_t *out_keys, int32_t *out_payload,
                       uint64_t *offsets) {
  const uint32_t M = (uint32_t)(((1ULL << D) - 1) << R);
  const uint64_t fan = 1ULL << D;
  uint64_t *cnt = (uint64_t *)calloc(fan + 1, sizeof(uint64_t));
  for (uint64_t i = 0; i < n; ++i) cnt[digit_of(keys[i], M, R, hashed)]++;
  uint64_t off = 0;
  for (uint64_t p = 0; p < fan; ++p) {
    uint64_t c = cnt[p];
    cnt[p] = off;
    if (offsets) offsets[p] = off;
    off += c;
  }
  if (offsets) offsets[fan] = off;
  for (uint64_t i = 0; i < n; ++i) {
    uint64_t d = cnt[digit_of(keys[i], M, R, hashed)]++;
    if (out_keys) out_keys[d] = keys[i];
    if (out_payload) out_payload[d] = payload ? payload[i] : (int32_t)i;
  }
  free(cnt);
}

#define ORC_RADIX_BITS 14 /* prj_params.h:16 NUM_RADIX_BITS */
#define ORC_PASSES 2      /* prj_params.h:21 NUM_PASSES */

static void two_pass_cluster(int32_t *k, uint64_t n) {
  int32_t *tmp = (int32_t *)malloc((n ? n : 1) * sizeof(int32_t));
  /* partitionHT (radix-join.cpp:253-266): pass 1 = bits [0,7), pass 2 =
   * bits [7,14); stable, so the result is ordered by the low 14 key bits */
  orc_radix_cluster(k, 0, n, 0, ORC_RADIX_BITS / ORC_PASSES, 0, tmp, 0, 0);
  orc_radix_cluster(tmp, 0, n, ORC_RADIX_BITS / ORC_PASSES,
                    ORC_RADIX_BITS - ORC_RADIX_BITS / ORC_PASSES, 0, k, 0, 0);
  free(tmp);
}

void orc_partition_ht_counts(const int32_t *keys, uint64_t n,
                             int32_t *counts) {
  /* radix-join.cpp:268-275: count_per_cluster[key & (2^14-1)]++ */
  memset(counts, 0, sizeof(int32_t) << ORC_RADIX_BITS);
  for (uint64_t i = 0; i < n; ++i)
    counts[(uint32_t)keys[i] & ((1u << ORC_RADIX_BITS) - 1)]++;
}

int64_t orc_rj_stepwise(const int32_t *keys_r, uint64_t nr,
                        const int32_t *keys_s, uint64_t ns) {
  int32_t *r = (int32_t *)malloc((nr ? nr : 1) * sizeof(int32_t));
  int32_t *s = (int32_t *)malloc((ns ? ns : 1) * sizeof(int32_t));
  memcpy(r, keys_r, nr * sizeof(int32_t));
  memcpy(s, keys_s, ns * sizeof(int32_t));
  /* radix-join.cpp:298-310 two passes on each side */
  two_pass_cluster(r, nr);
  two_pass_cluster(s, ns);
  int32_t *rc = (int32_t *)calloc(1u << ORC_RADIX_BITS, sizeof(int32_t));
  int32_t *sc = (int32_t *)calloc(1u << ORC_RADIX_BITS, sizeof(int32_t));
  orc_partition_ht_counts(r, nr, rc);
  orc_partition_ht_counts(s, ns, sc);
  int64_t result = 0;
  uint64_t ro = 0, so = 0;
  for (uint32_t c = 0; c < (1u << ORC_RADIX_BITS); ++c) {
    if (rc[c] > 0 && sc[c] > 0) {
      /* bucket_chaining_join_prepare (radix-join.cpp:196-215): N =
       * nextpow2(numR), MASK = (N-1) << 14, 1-based chains */
      uint32_t numR = (uint32_t)rc[c], N = 1;
      while (N < numR) N <<= 1;
      uint32_t mask = (N - 1) << ORC_RADIX_BITS;
      int32_t *bucket = (int32_t *)calloc(N, sizeof(int32_t));
      int32_t *next = (int32_t *)malloc(numR * sizeof(int32_t));
      const int32_t *rt = r + ro;
      for (uint32_t i = 0; i < numR;) {
        uint32_t idx = ((uint32_t)rt[i] & mask) >> ORC_RADIX_BITS;
        next[i] = bucket[idx];
        bucket[idx] = (int32_t)++i;
      }
      /* bucket_chaining_join_probe (radix-join.cpp:221-235) */
      const int32_t *st = s + so;
      for (int32_t j = 0; j < sc[c]; ++j) {
        uint32_t idx = ((uint32_t)st[j] & mask) >> ORC_RADIX_BITS;
        for (int32_t hit = bucket[idx]; hit > 0; hit = next[hit - 1])
          if (st[j] == rt[hit - 1]) ++result;
      }
      free(bucket);
      free(next);
    }
    ro += (uint64_t)rc[c];
    so += (uint64_t)sc[c];
  }
  free(rc);
  free(sc);
  free(r);
  free(s);
  return result;
}

/* ----------------------------------------- multi-threaded radix join (CPU) */

typedef struct {
  const int32_t *keys, *pay;
  uint64_t lo, hi;
  int bits;
  uint64_t *hist; /* [threads][P] */
  int tid;
  int32_t *out_k, *out_v;
  int carry_rowid;
} rpart_arg;

static void *rpart_count(void *p) {
  rpart_arg *a = (rpart_arg *)p;
  uint64_t P = 1ULL << a->bits, *h = a->hist + (uint64_t)a->tid * P;
  for (uint64_t i = a->lo; i < a->hi; ++i) h[orc_hashd(a->keys[i]) & (P - 1)]++;
  return 0;
}

static void *rpart_scatter(void *p) {
  rpart_arg *a = (rpart_arg *)p;
  uint64_t P = 1ULL << a->bits, *h = a->hist + (uint64_t)a->tid * P;
  for (uint64_t i = a->lo; i < a->hi; ++i) {
    uint64_t d = h[orc_hashd(a->keys[i]) & (P - 1)]++;
    a->out_k[d] = a->keys[i];
    a->out_v[d] = a->carry_rowid ? (int32_t)i : (a->pay ? a->pay[i] : 0);
  }
  return 0;
}

static void parallel_partition(const int32_t *keys, const int32_t *pay,
                               uint64_t n, int bits, int threads,
                               int carry_rowid, int32_t *out_k,
                               int32_t *out_v, uint64_t *offsets) {
  uint64_t P = 1ULL << bits;
  uint64_t *hist = (uint64_t *)calloc(P * threads, sizeof(uint64_t));
  rpart_arg *args = (rpart_arg *)calloc(threads, sizeof(rpart_arg));
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * threads);
  uint64_t chunk = (n + threads - 1) / threads;
  for (int t = 0; t < threads; ++t) {
    rpart_arg *a = &args[t];
    a->keys = keys;
    a->pay = pay;
    a->lo = t * chunk < n ? t * chunk : n;
    a->hi = (t + 1) * chunk < n ? (t + 1) * chunk : n;
    a->bits = bits;
    a->hist = hist;
    a->tid = t;
    a->out_k = out_k;
    a->out_v = out_v;
    a->carry_rowid = carry_rowid;
    pthread_create(&th[t], 0, rpart_count, a);
  }
  for (int t = 0; t < threads; ++t) pthread_join(th[t], 0);
  uint64_t off = 0;
  for (uint64_t p = 0; p < P; ++p) {
    offsets[p] = off;
    for (int t = 0; t < threads; ++t) {
      uint64_t c = hist[(uint64_t)t * P + p];
      hist[(uint64_t)t * P + p] = off;
      off += c;
    }
  }
  offsets[P] = off;
  for (int t = 0; t < threads; ++t)
    pthread_create(&th[t], 0, rpart_scatter, &args[t]);
  for (int t = 0; t < threads; ++t) pthread_join(th[t], 0);
  free(hist);
  free(args);
  free(th);
}

typedef struct {
  const int32_t *rk, *rv, *sk, *sv;
  const uint64_t *ro, *so;
  uint64_t P;
  int bits;
  volatile int64_t *next_part;
  const int32_t *ops, *operands;
  int n_aggs;
  /* rv / sv carry row positions; the minor keys and payloads are read
   * through them (orc_radix_join_agg_minor) */
  int by_rows;
  const int32_t *minor_r, *minor_s, *pay_r, *pay_s;
  acc8 acc;
} rjoin_arg;

static void *rjoin_worker(void *p) {
  rjoin_arg *a = (rjoin_arg *)p;
  uint32_t cap = 0;
  int32_t *bucket = 0, *next = 0;
  for (;;) {
    int64_t part = __atomic_fetch_add(a->next_part, 1, __ATOMIC_RELAXED);
    if ((uint64_t)part >= a->P) break;
    uint64_t r0 = a->ro[part], r1 = a->ro[part + 1];
    uint64_t s0 = a->so[part], s1 = a->so[part + 1];
    if (r0 == r1 || s0 == s1) continue;
    uint32_t numR = (uint32_t)(r1 - r0), N = 1;
    while (N < numR) N <<= 1;
    if (N > cap) {
      free(bucket);
      free(next);
      cap = N;
      bucket = (int32_t *)malloc(sizeof(int32_t) * cap);
      next = (int32_t *)malloc(sizeof(int32_t) * cap);
    }
    memset(bucket, 0, sizeof(int32_t) * N);
    /* bucket chaining on the hash bits above the partition bits */
    for (uint32_t i = 0; i < numR;) {
      uint32_t idx = (orc_hashd(a->rk[r0 + i]) >> a->bits) & (N - 1);
      next[i] = bucket[idx];
      bucket[idx] = (int32_t)++i;
    }
    for (uint64_t j = s0; j < s1; ++j) {
      int32_t k = a->sk[j];
      uint32_t idx = (orc_hashd(k) >> a->bits) & (N - 1);
      for (int32_t hit = bucket[idx]; hit > 0; hit = next[hit - 1]) {
        uint64_t r = r0 + (uint64_t)(hit - 1);
        if (a->rk[r] != k) continue;
        if (a->by_rows) {
          const int32_t br = a->rv[r], pr = a->sv[j];
          /* gpu-partitioned-hash-join-chained.cpp:1284-1333: after the key
           * compare, the build and probe minor keys must be equal too */
          if (a->minor_r && a->minor_r[br] != a->minor_s[pr]) continue;
          acc_update(&a->acc, a->ops, a->operands, a->n_aggs, k,
                     a->pay_r ? a->pay_r[br] : 0, a->pay_s ? a->pay_s[pr] : 0, br, pr);
        } else {
          acc_update(&a->acc, a->ops, a->operands, a->n_aggs, k, a->rv[r],
                     a->sv[j], a->rv[r], a->sv[j]);
        }
      }
    }
  }
  free(bucket);
  free(next);
  return 0;
}

static int side_carries_rowid(const int32_t *operands, int n, int build) {
  for (int j = 0; j < n; ++j) {
    int o = operands[j];
    if (o == V_ROWID_XOR) return 1;
    if (build && o == V_BUILD_ROWID) return 1;
    if (!build && o == V_PROBE_ROWID) return 1;
  }
  return 0;
}

static int radix_join_impl(const int32_t *keys_r, const int32_t *minor_r,
                           const int32_t *pay_r, uint64_t nr,
                           const int32_t *keys_s, const int32_t *minor_s,
                           const int32_t *pay_s, uint64_t ns, int32_t bits,
                           int by_rows, const int32_t *ops,
                           const int32_t *operands, int32_t n_aggs,
                           int64_t *out, int threads) {
  if (check_aggs(ops, operands, n_aggs) || !out) return -1;
  if (threads < 1) threads = 1;
  if (bits <= 0) {
    bits = 1;
    while (bits < 16 && (nr >> bits) > 2048) ++bits;
  }
  uint64_t P = 1ULL << bits;
  int32_t *rk = (int32_t *)malloc((nr + 1) * sizeof(int32_t));
  int32_t *rv = (int32_t *)malloc((nr + 1) * sizeof(int32_t));
  int32_t *sk = (int32_t *)malloc((ns + 1) * sizeof(int32_t));
  int32_t *sv = (int32_t *)malloc((ns + 1) * sizeof(int32_t));
  uint64_t *ro = (uint64_t *)malloc((P + 1) * sizeof(uint64_t));
  uint64_t *so = (uint64_t *)malloc((P + 1) * sizeof(uint64_t));
  /* the value carried through the partitions is the rowid when an
   * aggregate reads one, else the payload (operand_value then reads it as
   * "bval"/"pval" and as the rowid consistently). */
  int r_rowid = by_rows || side_carries_rowid(operands, n_aggs, 1);
  int s_rowid = by_rows || side_carries_rowid(operands, n_aggs, 0);
  parallel_partition(keys_r, pay_r, nr, bits, threads, r_rowid, rk, rv, ro);
  parallel_partition(keys_s, pay_s, ns, bits, threads, s_rowid, sk, sv, so);
  volatile int64_t next_part = 0;
  rjoin_arg *args = (rjoin_arg *)calloc(threads, sizeof(rjoin_arg));
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * threads);
  for (int t = 0; t < threads; ++t) {
    rjoin_arg *a = &args[t];
    a->rk = rk;
    a->rv = rv;
    a->sk = sk;
    a->sv = sv;
    a->ro = ro;
    a->so = so;
    a->P = P;
    a->bits = bits;
    a->next_part = &next_part;
    a->ops = ops;
    a->operands = operands;
    a->n_aggs = n_aggs;
    a->by_rows = by_rows;
    a->minor_r = minor_r;
    a->minor_s = minor_s;
    a->pay_r = pay_r;
    a->pay_s = pay_s;
    acc_init(&a->acc, ops, n_aggs);
    pthread_create(&th[t], 0, rjoin_worker, a);
  }
  acc8 total;
  acc_init(&total, ops, n_aggs);
  for (int t = 0; t < threads; ++t) {
    pthread_join(th[t], 0);
    acc_merge(&total, &args[t].acc, ops, n_aggs);
  }
  for (int j = 0; j < n_aggs; ++j) out[j] = total.v[j];
  free(args);
  free(th);
  free(rk);
  free(rv);
  free(sk);
  free(sv);
  free(ro);
  free(so);
  return 0;
}

int orc_radix_join_agg(const int32_t *keys_r, const int32_t *pay_r,
                       uint64_t nr, const int32_t *keys_s,
                       const int32_t *pay_s, uint64_t ns, int32_t bits,
                       const int32_t *ops, const int32_t *operands,
                       int32_t n_aggs, int64_t *out, int threads) {
  return radix_join_impl(keys_r, 0, pay_r, nr, keys_s, 0, pay_s, ns, bits, 0,
                         ops, operands, n_aggs, out, threads);
}

/* GpuPartitionedHashJoinChained with build_k_minor / probe_k_minor
 * (plan-parser.cpp:872-880; the check at
 * gpu-partitioned-hash-join-chained.cpp:1284-1333): a pair matches when the
 * keys are equal and the minor keys are equal.  Both sides carry their row
 * positions through the partitions; minor keys and payloads are read by
 * row.  minor_r / minor_s: both given, or both 0 (then this is the plain
 * partitioned join). */
int orc_radix_join_agg_minor(const int32_t *keys_r, const int32_t *minor_r,
                             const int32_t *pay_r, uint64_t nr,
                             const int32_t *keys_s, const int32_t *minor_s,
                             const int32_t *pay_s, uint64_t ns, int32_t bits,
                             const int32_t *ops, const int32_t *operands,
                             int32_t n_aggs, int64_t *out, int threads) {
  if (!minor_r != !minor_s) return -1;
  return radix_join_impl(keys_r, minor_r, pay_r, nr, keys_s, minor_s, pay_s, ns,
                         bits, 1, ops, operands, n_aggs, out, threads);
}

/* ------------------------------------------------------------ group-by */

typedef struct {
  int32_t key;
  int32_t next; /* packet 0 = {int32 next} */
  int64_t cnt, sum;
  int32_t mn, mx;
} orc_group;

typedef struct {
  int32_t *head;
  orc_group *e;
  uint64_t n, cap;
  int hash_bits;
} orc_gtable;

static int gtable_init(orc_gtable *g, int hash_bits, uint64_t cap) {
  g->hash_bits = hash_bits;
  g->head = (int32_t *)malloc(sizeof(int32_t) << hash_bits);
  g->cap = cap ? cap : 16;
  g->e = (orc_group *)malloc(sizeof(orc_group) * g->cap);
  g->n = 0;
  if (!g->head || !g->e) return -1;
  memset(g->head, 0xff, sizeof(int32_t) << hash_bits);
  return 0;
}

/* generate_build (hash-group-by-chained.cpp:267-633): walk the chain of
 * head[h]; on a key hit apply each monoid update; at the chain end append a
 * new entry initialised from the row (monoid create) and link it. */
static void gtable_grow_heads(orc_gtable *g) {
  /* placement only: chain order changes, results do not */
  int hb = g->hash_bits + 1;
  int32_t *head = (int32_t *)malloc(sizeof(int32_t) << hb);
  if (!head) return;
  memset(head, 0xff, sizeof(int32_t) << hb);
  for (uint64_t i = 0; i < g->n; ++i) {
    uint64_t h = bucket_of(g->e[i].key, hb);
    g->e[i].next = head[h];
    head[h] = (int32_t)i;
  }
  free(g->head);
  g->head = head;
  g->hash_bits = hb;
}

static int gtable_update(orc_gtable *g, int32_t key, int64_t cnt, int64_t sum,
                         int32_t mn, int32_t mx) {
  if (g->n >= (2ULL << g->hash_bits) && g->hash_bits < 28)
    gtable_grow_heads(g);
  uint64_t h = bucket_of(key, g->hash_bits);
  for (int32_t cur = g->head[h]; cur != -1; cur = g->e[cur].next) {
    orc_group *x = &g->e[cur];
    if (x->key == key) {
      x->cnt += cnt;
      x->sum += sum;
      if (mn < x->mn) x->mn = mn;
      if (mx > x->mx) x->mx = mx;
      return 0;
    }
  }
  if (g->n == g->cap) {
    g->cap *= 2;
    g->e = (orc_group *)realloc(g->e, sizeof(orc_group) * g->cap);
    if (!g->e) return -1;
  }
  orc_group *x = &g->e[g->n];
  x->key = key;
  x->cnt = cnt;
  x->sum = sum;
  x->mn = mn;
  x->mx = mx;
  x->next = g->head[h];
  g->head[h] = (int32_t)g->n;
  g->n++;
  return 0;
}

static int cmp_group(const void *a, const void *b) {
  int32_t x = ((const orc_group *)a)->key, y = ((const orc_group *)b)->key;
  return (x > y) - (x < y);
}

typedef struct {
  const int32_t *keys, *vals;
  const uint64_t *off;
  uint64_t p0, p1;
  orc_gtable g;
  int rc;
} gb_arg;

static void *gb_worker(void *p) {
  gb_arg *a = (gb_arg *)p;
  for (uint64_t part = a->p0; part < a->p1 && !a->rc; ++part)
    for (uint64_t i = a->off[part]; i < a->off[part + 1]; ++i)
      if (gtable_update(&a->g, a->keys[i], 1, a->vals[i], a->vals[i],
                        a->vals[i]))
        a->rc = -1;
  return 0;
}

int64_t orc_groupby(const int32_t *keys, const int32_t *values, uint64_t n,
                    int32_t hash_bits, int threads, int32_t *out_keys,
                    int64_t *out_count, int64_t *out_sum, int32_t *out_min,
                    int32_t *out_max, uint64_t cap) {
  if ((n && (!keys || !values))) return -1;
  if (threads < 1) threads = 1;
  if (n < 65536) threads = 1;
  orc_group *all = 0;
  uint64_t ng = 0;
  if (threads == 1) {
    orc_gtable g;
    int hb = hash_bits > 0 ? hash_bits : 10;
    if (gtable_init(&g, hb, 1024)) return -1;
    for (uint64_t i = 0; i < n; ++i)
      if (gtable_update(&g, keys[i], 1, values[i], values[i], values[i]))
        return -1;
    all = g.e;
    ng = g.n;
    free(g.head);
  } else {
    /* partition on fmix32 bits so each worker owns disjoint keys */
    int bits = 1;
    while ((1 << bits) < threads * 8) ++bits;
    uint64_t P = 1ULL << bits;
    int32_t *pk = (int32_t *)malloc(n * sizeof(int32_t));
    int32_t *pv = (int32_t *)malloc(n * sizeof(int32_t));
    uint64_t *off = (uint64_t *)malloc((P + 1) * sizeof(uint64_t));
    parallel_partition(keys, values, n, bits, threads, 0, pk, pv, off);
    gb_arg *args = (gb_arg *)calloc(threads, sizeof(gb_arg));
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * threads);
    uint64_t per = (P + threads - 1) / threads;
    int hb = hash_bits > 0 ? hash_bits : 16;
    for (int t = 0; t < threads; ++t) {
      gb_arg *a = &args[t];
      a->keys = pk;
      a->vals = pv;
      a->off = off;
      a->p0 = t * per < P ? t * per : P;
      a->p1 = (t + 1) * per < P ? (t + 1) * per : P;
      if (gtable_init(&a->g, hb, 1024)) return -1;
      pthread_create(&th[t], 0, gb_worker, a);
    }
    for (int t = 0; t < threads; ++t) {
      pthread_join(th[t], 0);
      if (args[t].rc) return -1;
      ng += args[t].g.n;
    }
    all = (orc_group *)malloc(sizeof(orc_group) * (ng ? ng : 1));
    uint64_t o = 0;
    for (int t = 0; t < threads; ++t) {
      memcpy(all + o, args[t].g.e, sizeof(orc_group) * args[t].g.n);
      o += args[t].g.n;
      free(args[t].g.e);
      free(args[t].g.head);
    }
    free(args);
    free(th);
    free(pk);
    free(pv);
    free(off);
  }
  qsort(all, ng, sizeof(orc_group), cmp_group);
  for (uint64_t i = 0; i < ng && i < cap; ++i) {
    if (out_keys) out_keys[i] = all[i].key;
    if (out_count) out_count[i] = all[i].cnt;
    if (out_sum) out_sum[i] = all[i].sum;
    if (out_min) out_min[i] = all[i].mn;
    if (out_max) out_max[i] = all[i].mx;
  }
  free(all);
  return (int64_t)ng;
}

void orc_reduce(const int32_t *col, const int32_t *rows, uint64_t n,
                const int32_t *ops, const int32_t *operands, int32_t n_aggs,
                int64_t *out) {
  acc8 a;
  acc_init(&a, ops, n_aggs);
  for (uint64_t i = 0; i < n; ++i) {
    int64_t r = rows ? rows[i] : (int64_t)i;
    int64_t v = col ? col[r] : 0;
    /* a column reduce reads the column as the "probe" value */
    acc_update(&a, ops, operands, n_aggs, (int32_t)v, v, v, r, r);
  }
  for (int j = 0; j < n_aggs; ++j) out[j] = a.v[j];
}

/* ------------------------------------------------------------ star join */
/* One star-join query as a chain of the reference's operators: Select on
 * each joined dimension (select.cpp:26-37); HashJoinChained with the
 * qualifying dimension rows as build side keyed by their primary key and
 * the fact's foreign key as probe key (hash-join-chained.cpp:262-566, via
 * orc_join_build); HashGroupByChained on the two group attributes with
 * COUNT and SUM((int64)price * quantity) (hash-group-by-chained.cpp:
 * 267-853; the int64 product is the plan's CastExpression,
 * expressions.hpp:1162).  Fact rows are split over threads, each with its
 * own group table; the tables are merged and sorted by (a, b). */

static int32_t star_attr(const orc_star_dim *d, int a, uint64_t i) {
  return d->attr_type[a] == 1 ? (int32_t)((const int8_t *)d->attr[a])[i]
                              : ((const int32_t *)d->attr[a])[i];
}

typedef struct {
  int32_t a, b, next;
  int64_t cnt, sum;
} star_group;

typedef struct {
  int32_t *head;
  star_group *e;
  uint64_t n, cap;
  int hb;
} star_gtable;

/* combineHashes (core/olap/lib/util/functions.cpp:397-400): boost-style
 * hash_combine of the two key hashes.  Placement only. */
static uint64_t star_pair_hash(int32_t a, int32_t b) {
  uint64_t h = orc_hash_int32(a);
  h ^= orc_hash_int32(b) + 0x9e3779b9ULL + (h << 6) + (h >> 2);
  return h;
}

static int star_gt_init(star_gtable *g) {
  g->hb = 12;
  g->head = (int32_t *)malloc(sizeof(int32_t) << g->hb);
  g->cap = 1024;
  g->e = (star_group *)malloc(sizeof(star_group) * g->cap);
  g->n = 0;
  if (!g->head || !g->e) return -1;
  memset(g->head, 0xff, sizeof(int32_t) << g->hb);
  return 0;
}

static void star_gt_free(star_gtable *g) {
  free(g->head);
  free(g->e);
}

static int star_gt_update(star_gtable *g, int32_t a, int32_t b, int64_t cnt, int64_t sum) {
  if (g->n >= (2ULL << g->hb) && g->hb < 24) {
    int hb = g->hb + 1;
    int32_t *head = (int32_t *)malloc(sizeof(int32_t) << hb);
    if (!head) return -1;
    memset(head, 0xff, sizeof(int32_t) << hb);
    for (uint64_t i = 0; i < g->n; ++i) {
      uint64_t h = star_pair_hash(g->e[i].a, g->e[i].b) & ((1ULL << hb) - 1);
      g->e[i].next = head[h];
      head[h] = (int32_t)i;
    }
    free(g->head);
    g->head = head;
    g->hb = hb;
  }
  uint64_t h = star_pair_hash(a, b) & ((1ULL << g->hb) - 1);
  for (int32_t cur = g->head[h]; cur != -1; cur = g->e[cur].next) {
    star_group *x = &g->e[cur];
    if (x->a == a && x->b == b) {
      x->cnt += cnt;
      x->sum += sum;
      return 0;
    }
  }
  if (g->n == g->cap) {
    g->cap *= 2;
    star_group *e = (star_group *)realloc(g->e, sizeof(star_group) * g->cap);
    if (!e) return -1;
    g->e = e;
  }
  star_group *x = &g->e[g->n];
  x->a = a;
  x->b = b;
  x->cnt = cnt;
  x->sum = sum;
  x->next = g->head[h];
  g->head[h] = (int32_t)g->n;
  g->n++;
  return 0;
}

static int star_cmp(const void *p, const void *q) {
  const star_group *x = (const star_group *)p, *y = (const star_group *)q;
  if (x->a != y->a) return (x->a > y->a) - (x->a < y->a);
  return (x->b > y->b) - (x->b < y->b);
}

typedef struct {
  const int32_t *const *fk;
  const int32_t *qty, *price;
  const orc_star_dim *dims;
  const orc_star_q *q;
  const orc_chained_table *ht; /* per dimension, joined ones only */
  int32_t n_dims;
  uint64_t lo, hi;
  star_gtable g;
  int rc;
} star_arg;

static void *star_worker(void *p) {
  star_arg *s = (star_arg *)p;
  const orc_star_q *q = s->q;
  for (uint64_t i = s->lo; i < s->hi && !s->rc; ++i) {
    int64_t row[4] = {-1, -1, -1, -1};
    int ok = 1;
    for (int d = 0; d < s->n_dims && ok; ++d) {
      if (!((q->join_mask >> d) & 1)) continue;
      const orc_chained_table *t = &s->ht[d];
      const int32_t k = s->fk[d][i];
      int64_t hit = -1;
      /* probe: walk head[h] chain, eq(key) (hash-join-chained.cpp:321-566) */
      for (int32_t cur = t->head[bucket_of(k, t->hash_bits)]; cur != -1; cur = t->next[cur])
        if (t->key[cur] == k) {
          hit = t->payload[cur];
          break; /* primary keys: at most one match */
        }
      if (hit < 0) ok = 0;
      row[d] = hit;
    }
    if (!ok) continue;
    const int32_t a = star_attr(&s->dims[q->group_dim[0]], q->group_attr[0], (uint64_t)row[q->group_dim[0]]);
    const int32_t b = star_attr(&s->dims[q->group_dim[1]], q->group_attr[1], (uint64_t)row[q->group_dim[1]]);
    if (star_gt_update(&s->g, a, b, 1, (int64_t)s->price[i] * (int64_t)s->qty[i])) s->rc = -1;
  }
  return 0;
}

int64_t orc_star_query(const int32_t *const *fk, int32_t n_dims, const int32_t *qty,
                       const int32_t *price, uint64_t n_fact, const orc_star_dim *dims,
                       const orc_star_q *q, int threads, int32_t *out_a, int32_t *out_b,
                       int64_t *out_count, int64_t *out_sum, uint64_t cap) {
  if (!dims || !q || n_dims < 1 || n_dims > 4 || (n_fact && (!fk || !qty || !price))) return -1;
  for (int k = 0; k < 2; ++k)
    if (q->group_dim[k] < 0 || q->group_dim[k] >= n_dims || !((q->join_mask >> q->group_dim[k]) & 1))
      return -1;
  if (threads < 1) threads = 1;
  if (n_fact < 65536) threads = 1;
  orc_chained_table ht[4];
  int32_t *bkeys[4] = {0, 0, 0, 0}, *brows[4] = {0, 0, 0, 0};
  memset(ht, 0, sizeof(ht));
  int64_t rc = 0;
  for (int d = 0; d < n_dims && !rc; ++d) {
    if (!((q->join_mask >> d) & 1)) continue;
    const orc_star_dim *dd = &dims[d];
    bkeys[d] = (int32_t *)malloc(sizeof(int32_t) * (dd->n ? dd->n : 1));
    brows[d] = (int32_t *)malloc(sizeof(int32_t) * (dd->n ? dd->n : 1));
    if (!bkeys[d] || !brows[d]) {
      rc = -1;
      break;
    }
    uint64_t m = 0;
    const int pa = q->pred_attr[d];
    for (uint64_t r = 0; r < dd->n; ++r) {
      if (pa >= 0) {
        const int32_t v = star_attr(dd, pa, r);
        if (v < q->pred_lo[d] || v > q->pred_hi[d]) continue; /* Select */
      }
      bkeys[d][m] = dd->keys ? dd->keys[r] : dd->key_base + (int32_t)r;
      brows[d][m] = (int32_t)r;
      ++m;
    }
    if (orc_join_build(bkeys[d], brows[d], m, 0, &ht[d])) rc = -1;
  }
  star_arg *args = (star_arg *)calloc((size_t)threads, sizeof(star_arg));
  pthread_t *th = (pthread_t *)calloc((size_t)threads, sizeof(pthread_t));
  if (!args || !th) rc = -1;
  for (int t = 0; t < threads && !rc; ++t) {
    args[t].fk = fk;
    args[t].qty = qty;
    args[t].price = price;
    args[t].dims = dims;
    args[t].q = q;
    args[t].ht = ht;
    args[t].n_dims = n_dims;
    args[t].lo = n_fact * (uint64_t)t / (uint64_t)threads;
    args[t].hi = n_fact * (uint64_t)(t + 1) / (uint64_t)threads;
    if (star_gt_init(&args[t].g)) rc = -1;
  }
  if (!rc) {
    for (int t = 1; t < threads; ++t) pthread_create(&th[t], 0, star_worker, &args[t]);
    star_worker(&args[0]);
    for (int t = 1; t < threads; ++t) pthread_join(th[t], 0);
    for (int t = 0; t < threads; ++t)
      if (args[t].rc) rc = -1;
  }
  if (!rc) {
    star_gtable *g = &args[0].g;
    for (int t = 1; t < threads && !rc; ++t)
      for (uint64_t i = 0; i < args[t].g.n; ++i)
        if (star_gt_update(g, args[t].g.e[i].a, args[t].g.e[i].b, args[t].g.e[i].cnt, args[t].g.e[i].sum)) {
          rc = -1;
          break;
        }
    if (!rc) {
      qsort(g->e, g->n, sizeof(star_group), star_cmp);
      for (uint64_t i = 0; i < g->n && i < cap; ++i) {
        if (out_a) out_a[i] = g->e[i].a;
        if (out_b) out_b[i] = g->e[i].b;
        if (out_count) out_count[i] = g->e[i].cnt;
        if (out_sum) out_sum[i] = g->e[i].sum;
      }
      rc = (int64_t)g->n;
    }
  }
  if (args)
    for (int t = 0; t < threads; ++t)
      if (args[t].g.head) star_gt_free(&args[t].g);
  free(args);
  free(th);
  for (int d = 0; d < 4; ++d) {
    if (ht[d].head) orc_join_free(&ht[d]);
    free(bkeys[d]);
    free(brows[d]);
  }
  return rc;
}

/* ------------------------------------------------- join -> group-by */
/* HashJoinChained (build keys with the group column as payload; every
 * build row inserted; a probe emits one binding per matching build row,
 * hash-join-chained.cpp:262-566) feeding HashGroupByChained on the build
 * row's group with COUNT and SUM/MIN/MAX of the probe value
 * (hash-group-by-chained.cpp:267-633).  Probe rows are split over threads,
 * each with its own group table; merged and sorted by group key. */
typedef struct {
  const orc_chained_table *t;
  const int32_t *pk, *pv;
  uint64_t lo, hi;
  orc_gtable g;
  int rc;
} jg_arg;

static void *jg_worker(void *p) {
  jg_arg *a = (jg_arg *)p;
  const orc_chained_table *t = a->t;
  for (uint64_t i = a->lo; i < a->hi && !a->rc; ++i) {
    const int32_t k = a->pk[i];
    for (int32_t cur = t->head[bucket_of(k, t->hash_bits)]; cur != -1; cur = t->next[cur])
      if (t->key[cur] == k && gtable_update(&a->g, t->payload[cur], 1, a->pv[i], a->pv[i], a->pv[i]))
        a->rc = -1;
  }
  return 0;
}

int64_t orc_join_groupby(const int32_t *bk, const int32_t *bg, uint64_t nb, const int32_t *pk,
                         const int32_t *pv, uint64_t np, int threads, int32_t *out_keys,
                         int64_t *out_count, int64_t *out_sum, int32_t *out_min, int32_t *out_max,
                         uint64_t cap) {
  if ((nb && (!bk || !bg)) || (np && (!pk || !pv))) return -1;
  if (threads < 1) threads = 1;
  if (np < 65536) threads = 1;
  orc_chained_table t;
  memset(&t, 0, sizeof(t));
  if (orc_join_build(bk, bg, nb, 0, &t)) return -1;
  jg_arg *args = (jg_arg *)calloc((size_t)threads, sizeof(jg_arg));
  pthread_t *th = (pthread_t *)calloc((size_t)threads, sizeof(pthread_t));
  int64_t rc = (args && th) ? 0 : -1;
  for (int i = 0; i < threads && !rc; ++i) {
    args[i].t = &t;
    args[i].pk = pk;
    args[i].pv = pv;
    args[i].lo = np * (uint64_t)i / (uint64_t)threads;
    args[i].hi = np * (uint64_t)(i + 1) / (uint64_t)threads;
    if (gtable_init(&args[i].g, 10, 1024)) rc = -1;
  }
  if (!rc) {
    for (int i = 1; i < threads; ++i) pthread_create(&th[i], 0, jg_worker, &args[i]);
    jg_worker(&args[0]);
    for (int i = 1; i < threads; ++i) pthread_join(th[i], 0);
    for (int i = 0; i < threads; ++i)
      if (args[i].rc) rc = -1;
  }
  if (!rc) {
    orc_gtable *g = &args[0].g;
    for (int i = 1; i < threads && !rc; ++i)
      for (uint64_t j = 0; j < args[i].g.n; ++j) {
        const orc_group *x = &args[i].g.e[j];
        if (gtable_update(g, x->key, x->cnt, x->sum, x->mn, x->mx)) {
          rc = -1;
          break;
        }
      }
    if (!rc) {
      qsort(g->e, g->n, sizeof(orc_group), cmp_group);
      for (uint64_t j = 0; j < g->n && j < cap; ++j) {
        if (out_keys) out_keys[j] = g->e[j].key;
        if (out_count) out_count[j] = g->e[j].cnt;
        if (out_sum) out_sum[j] = g->e[j].sum;
        if (out_min) out_min[j] = g->e[j].mn;
        if (out_max) out_max[j] = g->e[j].mx;
      }
      rc = (int64_t)g->n;
    }
  }
  if (args)
    for (int i = 0; i < threads; ++i) {
      free(args[i].g.head);
      free(args[i].g.e);
    }
  free(args);
  free(th);
  orc_join_free(&t);
  return rc;
}

/* ---------------------------------------------------------- bloom filter */
/* BloomFilterBuild / BloomFilterProbe (bloom-filter-build.cpp:28-59,
 * bloom-filter-probe.cpp:28-53): flags[key & (filter_size - 1)] set for every
 * build key (bloom-filter.cpp:65-95; the key itself is the position); the
 * probe keeps rows whose flag is set.  Returns the number of passing rows
 * and writes their positions in order (up to cap). */
int64_t orc_bloom_semijoin(const int32_t *build, uint64_t nb, const int32_t *probe, uint64_t np,
                           uint64_t filter_size, int32_t *rows, uint64_t cap) {
  if (!filter_size || (filter_size & (filter_size - 1))) return -1;
  unsigned char *flags = (unsigned char *)calloc(filter_size, 1);
  if (!flags) return -1;
  const uint32_t mask = (uint32_t)(filter_size - 1);
  for (uint64_t i = 0; i < nb; ++i) flags[(uint32_t)build[i] & mask] = 1;
  int64_t m = 0;
  for (uint64_t i = 0; i < np; ++i)
    if (flags[(uint32_t)probe[i] & mask]) {
      if ((uint64_t)m < cap && rows) rows[m] = (int32_t)i;
      ++m;
    }
  free(flags);
  return m;
}

/* ----------------------------------- radix clustering of int64-key tuples */
/* The aggregation twin of radix_cluster_nopadding (core/platform/lib/util/
 * radix/aggregations/radix-aggr.cpp:82-155): stable counting sort of
 * agg::tuple_t {int64 key; int64 payload} on digit
 * (key & (((1 << D) - 1) << R)) >> R of the 64-bit key. */
void orc_radix_cluster_i64(const int64_t *keys, const int64_t *payload, uint64_t n, int32_t R, int32_t D,
                           int64_t *out_keys, int64_t *out_payload, uint64_t *offsets) {
  const uint64_t M = ((1ULL << D) - 1) << R;
  const uint64_t parts = 1ULL << D;
  uint64_t *hist = (uint64_t *)calloc(parts + 1, sizeof(uint64_t));
  for (uint64_t i = 0; i < n; ++i) hist[(((uint64_t)keys[i]) & M) >> R]++;
  uint64_t acc = 0;
  for (uint64_t p = 0; p < parts; ++p) {
    const uint64_t c = hist[p];
    hist[p] = acc;
    if (offsets) offsets[p] = acc;
    acc += c;
  }
  if (offsets) offsets[parts] = acc;
  for (uint64_t i = 0; i < n; ++i) {
    const uint64_t d = (((uint64_t)keys[i]) & M) >> R;
    const uint64_t o = hist[d]++;
    out_keys[o] = keys[i];
    out_payload[o] = payload ? payload[i] : (int64_t)i;
  }
  free(hist);
}

/* partitionHT of the twin (radix-aggr.cpp:237-259): two passes (bits [0,7)
 * then [7,14)), then the number of tuples per cluster key & (2^14 - 1).
 * out_keys / out_payload get the clustered tuples (payload = row id). */
void orc_partition_ht_agg(const int64_t *keys, uint64_t n, int32_t *counts, int64_t *out_keys,
                          int64_t *out_payload) {
  int64_t *tk = (int64_t *)malloc((n ? n : 1) * sizeof(int64_t));
  int64_t *tp = (int64_t *)malloc((n ? n : 1) * sizeof(int64_t));
  orc_radix_cluster_i64(keys, 0, n, 0, ORC_RADIX_BITS / ORC_PASSES, tk, tp, 0);
  orc_radix_cluster_i64(tk, tp, n, ORC_RADIX_BITS / ORC_PASSES, ORC_RADIX_BITS - ORC_RADIX_BITS / ORC_PASSES,
                        out_keys, out_payload, 0);
  memset(counts, 0, sizeof(int32_t) << ORC_RADIX_BITS);
  for (uint64_t i = 0; i < n; ++i) counts[(uint64_t)out_keys[i] & ((1u << ORC_RADIX_BITS) - 1)]++;
  free(tk);
  free(tp);
}

/* Bucket chains over one cluster of int64-key tuples, as the twin's
 * bucket_chaining_agg_prepare (radix-agg: radix-aggr.cpp:181-204):
 * N = next power of two >= n, MASK = (N - 1) << 14, bucket index
 * (key & MASK) >> 14, chains 1-based through next[]. */
typedef struct {
  int *bucket, *next;
  uint64_t mask;
} orc_chain_ht;

static void orc_chain_prepare(const int64_t *keys, uint32_t n, orc_chain_ht *ht) {
  uint32_t N = 1;
  while (N < n) N <<= 1;
  ht->mask = (uint64_t)(N - 1) << ORC_RADIX_BITS;
  ht->next = (int *)malloc((n ? n : 1) * sizeof(int));
  ht->bucket = (int *)calloc(N, sizeof(int));
  for (uint32_t i = 0; i < n;) {
    const uint64_t idx = ((uint64_t)keys[i] & ht->mask) >> ORC_RADIX_BITS;
    ht->next[i] = ht->bucket[idx];
    ht->bucket[idx] = (int)++i;
  }
}

static void orc_chain_free(orc_chain_ht *ht) {
  free(ht->bucket);
  free(ht->next);
}

/* RJStepwise of the int64-key twin (radix-aggr.cpp:261-358): both sides
 * clustered by partitionHT, then per cluster present on both sides, the
 * bucket chains of R probed by every S tuple (bucket_chaining_agg_probe,
 * :206-223); returns the number of (R, S) pairs with equal keys. */
int64_t orc_join_count_i64(const int64_t *rk, uint64_t nr, const int64_t *sk, uint64_t ns) {
  const uint32_t C = 1u << ORC_RADIX_BITS;
  int32_t *rc = (int32_t *)malloc(C * sizeof(int32_t)), *sc = (int32_t *)malloc(C * sizeof(int32_t));
  int64_t *rkk = (int64_t *)malloc((nr ? nr : 1) * sizeof(int64_t)), *rp = (int64_t *)malloc((nr ? nr : 1) * sizeof(int64_t));
  int64_t *skk = (int64_t *)malloc((ns ? ns : 1) * sizeof(int64_t)), *sp = (int64_t *)malloc((ns ? ns : 1) * sizeof(int64_t));
  orc_partition_ht_agg(rk, nr, rc, rkk, rp);
  orc_partition_ht_agg(sk, ns, sc, skk, sp);
  int64_t result = 0;
  uint64_t r = 0, s = 0;
  for (uint32_t c = 0; c < C; ++c) {
    if (rc[c] > 0 && sc[c] > 0) {
      orc_chain_ht ht;
      orc_chain_prepare(rkk + r, (uint32_t)rc[c], &ht);
      for (int32_t j = 0; j < sc[c]; ++j) {
        const int64_t key = skk[s + j];
        const uint64_t idx = ((uint64_t)key & ht.mask) >> ORC_RADIX_BITS;
        for (int hit = ht.bucket[idx]; hit > 0; hit = ht.next[hit - 1])
          if (rkk[r + hit - 1] == key) result++;
      }
      orc_chain_free(&ht);
    }
    r += rc[c];
    s += sc[c];
  }
  free(rc);
  free(sc);
  free(rkk);
  free(rp);
  free(skk);
  free(sp);
  return result;
}

static int orc_cmp_i64_first(const void *a, const void *b) {
  const int64_t x = ((const int64_t *)a)[0], y = ((const int64_t *)b)[0];
  return x < y ? -1 : x > y;
}

/* RadixNest over int64-key tuples (radix-nest.cpp:326-700 with the twin's
 * partitionHT and bucket chains): tuples are clustered, each cluster gets
 * its bucket chains, and every tuple not yet marked starts a group, walks
 * its chain, folds every tuple of equal key into the group (COUNT, SUM with
 * int64 wrap-around, MIN, MAX of the value column) and marks it.  Groups are
 * returned sorted by key.  Returns the number of groups; with out_cap below
 * it only that many are written. */
int64_t orc_nest_i64(const int64_t *keys, const int64_t *vals, uint64_t n, int64_t *out_keys, int64_t *out_cnt,
                     int64_t *out_sum, int64_t *out_min, int64_t *out_max, uint64_t out_cap) {
  const uint32_t C = 1u << ORC_RADIX_BITS;
  int32_t *cnt = (int32_t *)malloc(C * sizeof(int32_t));
  int64_t *ck = (int64_t *)malloc((n ? n : 1) * sizeof(int64_t)), *crow = (int64_t *)malloc((n ? n : 1) * sizeof(int64_t));
  orc_partition_ht_agg(keys, n, cnt, ck, crow);
  /* groups as rows of {key, count, sum, min, max} */
  int64_t *g = (int64_t *)malloc((n ? n : 1) * 5 * sizeof(int64_t));
  uint64_t ng = 0, r = 0;
  unsigned char *marked = (unsigned char *)calloc(n ? n : 1, 1);
  for (uint32_t c = 0; c < C; ++c) {
    const uint32_t m = (uint32_t)cnt[c];
    if (m > 0) {
      orc_chain_ht ht;
      orc_chain_prepare(ck + r, m, &ht);
      for (uint32_t j = 0; j < m; ++j) {
        if (marked[r + j]) continue;
        const int64_t key = ck[r + j];
        uint64_t count = 0, sum = 0;
        int64_t mn = INT64_MAX, mx = INT64_MIN;
        const uint64_t idx = ((uint64_t)key & ht.mask) >> ORC_RADIX_BITS;
        for (int hit = ht.bucket[idx]; hit > 0; hit = ht.next[hit - 1]) {
          const uint64_t t = r + (uint64_t)(hit - 1);
          if (ck[t] != key) continue;
          const int64_t v = vals ? vals[crow[t]] : 0;
          count++;
          sum += (uint64_t)v;
          if (v < mn) mn = v;
          if (v > mx) mx = v;
          marked[t] = 1;
        }
        int64_t *o = g + 5 * ng++;
        o[0] = key;
        o[1] = (int64_t)count;
        o[2] = (int64_t)sum;
        o[3] = mn;
        o[4] = mx;
      }
      orc_chain_free(&ht);
    }
    r += m;
  }
  qsort(g, ng, 5 * sizeof(int64_t), orc_cmp_i64_first);
  for (uint64_t i = 0; i < ng && i < out_cap; ++i) {
    if (out_keys) out_keys[i] = g[5 * i];
    if (out_cnt) out_cnt[i] = g[5 * i + 1];
    if (out_sum) out_sum[i] = g[5 * i + 2];
    if (out_min) out_min[i] = g[5 * i + 3];
    if (out_max) out_max[i] = g[5 * i + 4];
  }
  free(cnt);
  free(ck);
  free(crow);
  free(g);
  free(marked);
  return (int64_t)ng;
}
