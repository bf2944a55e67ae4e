/*
 * oracle.h -- CPU restatement of chapeiro/proteus's join / group-by semantics.
 *
 * TEST INFRASTRUCTURE ONLY.  The CUDA path's results are compared with the
 * oracle's (bit-exact: every result is integer).  Only the test suite,
 * the smoke check and the benchmark's CPU-baseline leg may load it; the
 * product library never links or calls it.
 *
 * Parity pins: the oracle is checked against (1) the reference's own golden
 * outputs for its sailors / reserves / boats / lineitem fixtures and (2) the
 * match counts and cluster counts of the reference's RJStepwise / partitionHT
 * compiled from source (oracle/_ref), both committed under tests/golden/.
 */
#ifndef GBJ_ORACLE_H
#define GBJ_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Hash of an int32 key as the JIT'd operators compute it: sign-extend to 64
 * bits, murmur3 fmix32 constants in 64-bit arithmetic
 * (core/olap/lib/expressions/expressions-hasher.cpp:39-58). */
uint64_t orc_hash_int32(int32_t key);

/* murmur3 fmix32 in 32-bit arithmetic, the GPU partitioner's hashd
 * (core/olap/lib/operators/gpu/gpu-partitioned-hash-join-chained-helpers.cpp:
 * 49-56). */
uint32_t orc_hashd(int32_t key);

/* ---- chained hash join (core/olap/lib/operators/hash-join-chained.cpp) ---- */
typedef struct orc_chained_table {
  int32_t *head;          /* 2^hash_bits chain heads, -1 = empty             */
  int32_t *next;          /* per entry: previous head (packet field 0)       */
  const int32_t *key;     /* per entry key  (packet 0, offset 32)            */
  const int32_t *payload; /* per entry payload (further packets), may be 0   */
  uint64_t n;
  int32_t hash_bits;
  const int64_t *key64;   /* int64 keys (orc_join_build_i64), else 0     */
} orc_chained_table;

int orc_join_build(const int32_t *keys, const int32_t *payload, uint64_t n,
                   int32_t hash_bits, orc_chained_table *t);
/* Multi-worker build with atomic slot counter and atomic head exchange, as
 * HashJoinChainedMorsel (core/olap/lib/operators/hash-join-chained-morsel.cpp:
 * 29-129).  Same chains up to order. */
int orc_join_build_mt(const int32_t *keys, const int32_t *payload, uint64_t n,
                      int32_t hash_bits, int threads, orc_chained_table *t);
void orc_join_free(orc_chained_table *t);

/* Probe + fused aggregate; ops/operands use the gbj_agg_op / gbj_operand
 * codes of gbjoin.h.  Returns 0 or -1 on a bad argument. */
int orc_join_probe_agg(const orc_chained_table *t, const int32_t *keys,
                       const int32_t *payload, uint64_t n,
                       const int32_t *ops, const int32_t *operands,
                       int32_t n_aggs, int64_t *out, int threads);

/* Every match as (build row, probe row), probe order then chain order.
 * Returns the number of matches (pairs beyond cap are not written). */
int64_t orc_join_probe_pairs(const orc_chained_table *t, const int32_t *keys,
                             uint64_t n, int32_t *build_rows,
                             int32_t *probe_rows, uint64_t cap);

/* The same join over int64 keys, chains placed by the reference's int64
 * hash (expressions-hasher.cpp:66-84, murmur3's 64-bit finaliser). */
uint64_t orc_hash_int64(int64_t key);
int orc_join_build_i64(const int64_t *keys, const int32_t *payload, uint64_t n,
                       int32_t hash_bits, orc_chained_table *t);
int orc_join_probe_agg_i64(const orc_chained_table *t, const int64_t *keys,
                           const int32_t *payload, uint64_t n,
                           const int32_t *ops, const int32_t *operands,
                           int32_t n_aggs, int64_t *out);
int64_t orc_join_probe_pairs_i64(const orc_chained_table *t,
                                 const int64_t *keys, uint64_t n,
                                 int32_t *build_rows, int32_t *probe_rows,
                                 uint64_t cap);

/* ---- radix clustering (core/platform/lib/util/radix/joins/radix-join.cpp) */
/* Stable counting-sort cluster on digit = (f(key) & (((1<<D)-1)<<R)) >> R,
 * f = identity (hashed = 0, radix_cluster_nopadding :85-155) or fmix32
 * (hashed = 1).  payload may be 0 (row positions are carried). offsets gets
 * 2^D + 1 entries (may be 0). */
void orc_radix_cluster(const int32_t *keys, const int32_t *payload,
                       uint64_t n, int32_t R, int32_t D, int32_t hashed,
                       int32_t *out_keys, int32_t *out_payload,
                       uint64_t *offsets);

/* RJStepwise (radix-join.cpp:278-375): two-pass cluster on the low
 * NUM_RADIX_BITS=14 key bits (7 + 7), then per-cluster bucket-chaining
 * join; returns the match count. Single-threaded like the original. */
int64_t orc_rj_stepwise(const int32_t *keys_r, uint64_t nr,
                        const int32_t *keys_s, uint64_t ns);
/* partitionHT (radix-join.cpp:253-276): cluster counts of the 2^14 clusters
 * after the two passes (counts must hold 16384 ints). */
void orc_partition_ht_counts(const int32_t *keys, uint64_t n, int32_t *counts);

/* Multi-threaded radix join with fused aggregates: the CPU baseline for the
 * partitioned join (partition both sides on fmix32 bits, then a chained
 * table per partition, as bucket_chaining_join_prepare/probe, radix-join.cpp:
 * 177-235, but carrying payloads/rowids for the aggregate). */
int orc_radix_join_agg(const int32_t *keys_r, const int32_t *pay_r,
                       uint64_t nr, const int32_t *keys_s,
                       const int32_t *pay_s, uint64_t ns, int32_t bits,
                       const int32_t *ops, const int32_t *operands,
                       int32_t n_aggs, int64_t *out, int threads);
/* Composite-key form (build_k_minor / probe_k_minor of the reference's
 * partitioned join): a pair also needs equal minor keys; minor columns both
 * given or both 0.  Row ids and payloads are read by row position. */
int orc_radix_join_agg_minor(const int32_t *keys_r, const int32_t *minor_r,
                             const int32_t *pay_r, uint64_t nr,
                             const int32_t *keys_s, const int32_t *minor_s,
                             const int32_t *pay_s, uint64_t ns, int32_t bits,
                             const int32_t *ops, const int32_t *operands,
                             int32_t n_aggs, int64_t *out, int threads);

/* ---- chained hash group-by (core/olap/lib/operators/
 *      hash-group-by-chained.cpp:267-633 build, :638-853 emit scan) ---- */
/* One output row per distinct key: COUNT int64, SUM int64, MIN/MAX int32,
 * sorted by key (the reference compares unordered results after a sort,
 * core/olap/tests/olap-test-utils/lib/test-utils.cpp:71-85).  threads > 1
 * partitions the rows by hash first and aggregates partitions in parallel.
 * Returns the number of groups (only the first cap are written), or -1. */
int64_t orc_groupby(const int32_t *keys, const int32_t *values, uint64_t n,
                    int32_t hash_bits, int threads, int32_t *out_keys,
                    int64_t *out_count, int64_t *out_sum, int32_t *out_min,
                    int32_t *out_max, uint64_t cap);

/* Global aggregate over a column restricted to a row list (Reduce,
 * core/olap/lib/operators/reduce-opt.cpp:52-481). rows may be 0. */
void orc_reduce(const int32_t *col, const int32_t *rows, uint64_t n,
                const int32_t *ops, const int32_t *operands, int32_t n_aggs,
                int64_t *out);


/* ---- star-join query: Select -> HashJoinChained per joined dimension ->
 *      HashGroupByChained on two dimension attributes (compositions of the
 *      functions above; see oracle.c) ---- */
typedef struct orc_star_dim {
  uint64_t n;
  int32_t key_base; /* primary key of row 0; row i has key_base + i */
  int32_t n_attrs;
  const void *attr[4];
  int32_t attr_type[4]; /* 0 int32, 1 int8 */
  int32_t attr_min[4];  /* unused by the oracle (same layout as gbjoin.h) */
  int32_t attr_max[4];
  const int32_t *keys;  /* primary key of each row; 0: key_base + row    */
} orc_star_dim;

typedef struct orc_star_q {
  int32_t join_mask;
  int32_t pred_attr[4]; /* -1: no predicate */
  int32_t pred_lo[4];
  int32_t pred_hi[4];
  int32_t group_dim[2];
  int32_t group_attr[2];
} orc_star_q;

/* Groups (a, b, COUNT, SUM((int64)price * quantity)) sorted by (a, b);
 * returns the group count (only the first cap are written) or -1. */
int64_t orc_star_query(const int32_t *const *fk, int32_t n_dims,
                       const int32_t *qty, const int32_t *price,
                       uint64_t n_fact, const orc_star_dim *dims,
                       const orc_star_q *q, int threads, int32_t *out_a,
                       int32_t *out_b, int64_t *out_count, int64_t *out_sum,
                       uint64_t cap);


/* HashJoinChained (build payload = group column) feeding HashGroupByChained
 * on the matched build row's group: COUNT and SUM/MIN/MAX of the probe
 * value per group, sorted by group key.  Returns the group count (only the
 * first cap are written) or -1. */
int64_t orc_join_groupby(const int32_t *bk, const int32_t *bg, uint64_t nb,
                         const int32_t *pk, const int32_t *pv, uint64_t np,
                         int threads, int32_t *out_keys, int64_t *out_count,
                         int64_t *out_sum, int32_t *out_min, int32_t *out_max,
                         uint64_t cap);


/* Bloom-filter semi-join with the reference's single-position filter
 * (flags[key & (filter_size - 1)]): positions of passing probe rows. */
int64_t orc_bloom_semijoin(const int32_t *build, uint64_t nb, const int32_t *probe,
                           uint64_t np, uint64_t filter_size, int32_t *rows,
                           uint64_t cap);


/* Aggregation twins (core/platform/lib/util/radix/aggregations/radix-aggr.cpp):
 * stable radix cluster of {int64 key, int64 payload} tuples (payload 0 =
 * row ids) and partitionHT's two-pass cluster + counts on 2^14 clusters. */
void orc_radix_cluster_i64(const int64_t *keys, const int64_t *payload,
                           uint64_t n, int32_t R, int32_t D, int64_t *out_keys,
                           int64_t *out_payload, uint64_t *offsets);
void orc_partition_ht_agg(const int64_t *keys, uint64_t n, int32_t *counts,
                          int64_t *out_keys, int64_t *out_payload);

/* RJStepwise of the int64-key twin: number of (R, S) pairs with equal keys. */
int64_t orc_join_count_i64(const int64_t *rk, uint64_t nr, const int64_t *sk, uint64_t ns);

/* RadixNest over int64 keys: per distinct key COUNT, SUM (int64, wrapping),
 * MIN, MAX of vals (NULL: 0), sorted by key; returns the number of groups. */
int64_t orc_nest_i64(const int64_t *keys, const int64_t *vals, uint64_t n, int64_t *out_keys, int64_t *out_cnt,
                     int64_t *out_sum, int64_t *out_min, int64_t *out_max, uint64_t out_cap);

#ifdef __cplusplus
}
#endif
#endif
