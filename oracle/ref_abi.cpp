// extern "C" entry points over the reference's own radix-join helpers
// (core/platform/lib/util/radix/joins/radix-join.cpp) and their int64-key
// aggregation twins (core/platform/lib/util/radix/aggregations/
// radix-aggr.cpp), compiled from the
// reference sources in place by oracle/Makefile into oracle/_ref/.  TEST
// INFRASTRUCTURE ONLY: used to pin the oracle's restatement and to produce
// the committed golden counts under tests/golden/.
#include <platform/util/radix/aggregations/radix-aggr.hpp>
#include <platform/util/radix/joins/radix-join.hpp>

#include <cstdlib>
#include <cstring>

extern "C" {

// RJStepwise on int32 keys (payload = row position); returns the match count.
// R and S are copied into the reference's AoS joins::tuple_t layout first
// (core/platform/include/platform/util/radix/joins/types.h:22-44).
int64_t ref_rj_stepwise(const int32_t *keys_r, uint32_t nr,
                        const int32_t *keys_s, uint32_t ns) {
  joins::relation_t r, s;
  // RJStepwise clusters in place and reads RELATION_PADDING_JOIN slack.
  size_t pad = RELATION_PADDING_JOIN;
  r.tuples = (joins::tuple_t *)malloc(nr * sizeof(joins::tuple_t) + pad);
  s.tuples = (joins::tuple_t *)malloc(ns * sizeof(joins::tuple_t) + pad);
  r.num_tuples = nr;
  s.num_tuples = ns;
  for (uint32_t i = 0; i < nr; ++i) r.tuples[i] = {keys_r[i], (int64_t)i};
  for (uint32_t i = 0; i < ns; ++i) s.tuples[i] = {keys_s[i], (int64_t)i};
  int64_t m = RJStepwise(&r, &s);
  free(r.tuples);
  free(s.tuples);
  return m;
}

// partitionHT: two-pass cluster in place; returns the 2^NUM_RADIX_BITS
// cluster counts in `counts` and the clustered keys / payload row ids.
void ref_partition_ht(const int32_t *keys, uint32_t n, int32_t *counts,
                      int32_t *out_keys, int64_t *out_rows) {
  joins::tuple_t *t =
      (joins::tuple_t *)malloc(n * sizeof(joins::tuple_t) + 64);
  for (uint32_t i = 0; i < n; ++i) t[i] = {keys[i], (int64_t)i};
  int *c = partitionHT(n, t);
  memcpy(counts, c, sizeof(int) << NUM_RADIX_BITS);
  for (uint32_t i = 0; i < n; ++i) {
    if (out_keys) out_keys[i] = t[i].key;
    if (out_rows) out_rows[i] = t[i].payload;
  }
  free(c);
  free(t);
}

// partitionHT of the aggregation twin: agg::tuple_t {int64 key; int64
// payload} (core/platform/include/platform/util/radix/aggregations/types.h),
// clustered in place on the low NUM_RADIX_BITS key bits; counts per cluster.
void ref_partition_ht_agg(const int64_t *keys, uint32_t n, int32_t *counts, int64_t *out_keys,
                          int64_t *out_payload) {
  agg::tuple_t *t = (agg::tuple_t *)malloc(n * sizeof(agg::tuple_t) + 64);
  for (uint32_t i = 0; i < n; ++i) t[i] = {keys[i], (int64_t)i};
  int *c = partitionHT(n, t);
  memcpy(counts, c, sizeof(int) << NUM_RADIX_BITS);
  for (uint32_t i = 0; i < n; ++i) {
    if (out_keys) out_keys[i] = t[i].key;
    if (out_payload) out_payload[i] = t[i].payload;
  }
  free(c);
  free(t);
}

// RJStepwise of the aggregation twin (radix-aggr.cpp:261-358): int64 keys,
// payload = row position; returns the number of matching (R, S) pairs.
int64_t ref_rj_stepwise_agg(const int64_t *keys_r, uint32_t nr, const int64_t *keys_s, uint32_t ns) {
  agg::relation_t r, s;
  r.tuples = (agg::tuple_t *)malloc(nr * sizeof(agg::tuple_t) + RELATION_PADDING_AGG);
  s.tuples = (agg::tuple_t *)malloc(ns * sizeof(agg::tuple_t) + RELATION_PADDING_AGG);
  r.num_tuples = nr;
  s.num_tuples = ns;
  for (uint32_t i = 0; i < nr; ++i) r.tuples[i] = {keys_r[i], (int64_t)i};
  for (uint32_t i = 0; i < ns; ++i) s.tuples[i] = {keys_s[i], (int64_t)i};
  int64_t m = RJStepwise(&r, &s);
  free(r.tuples);
  free(s.tuples);
  return m;
}

}  // extern "C"

// Defined in radix-aggr.cpp:206-223,225-233 without a header declaration.
int64_t bucket_chaining_agg_probe(const agg::relation_t *const R, HT *ht, const agg::tuple_t *const s);
void bucket_chaining_agg_finish(HT *ht);

extern "C" {

// The reference's own chains give each query key's group size: the tuples
// are clustered with partitionHT, the cluster of query key q gets
// bucket_chaining_agg_prepare's chains, and bucket_chaining_agg_probe counts
// the tuples equal to q (what RadixNest folds into q's group).
void ref_nest_counts(const int64_t *keys, uint32_t n, const int64_t *query, uint32_t nq, int64_t *counts) {
  agg::tuple_t *t = (agg::tuple_t *)malloc(n * sizeof(agg::tuple_t) + RELATION_PADDING_AGG);
  for (uint32_t i = 0; i < n; ++i) t[i] = {keys[i], (int64_t)i};
  int *c = partitionHT(n, t);
  const uint32_t C = 1u << NUM_RADIX_BITS;
  uint32_t *start = (uint32_t *)malloc((C + 1) * sizeof(uint32_t));
  start[0] = 0;
  for (uint32_t i = 0; i < C; ++i) start[i + 1] = start[i] + (uint32_t)c[i];
  for (uint32_t j = 0; j < nq; ++j) {
    const uint32_t cl = (uint32_t)((uint64_t)query[j] & (C - 1));
    agg::relation_t rel;
    rel.tuples = t + start[cl];
    rel.num_tuples = (uint32_t)c[cl];
    counts[j] = 0;
    if (rel.num_tuples == 0) continue;
    HT ht;
    bucket_chaining_agg_prepare(rel.tuples, (int)rel.num_tuples, &ht);
    agg::tuple_t probe = {query[j], 0};
    counts[j] = bucket_chaining_agg_probe(&rel, &ht, &probe);
    bucket_chaining_agg_finish(&ht);
  }
  free(start);
  free(c);
  free(t);
}

int32_t ref_num_radix_bits() { return NUM_RADIX_BITS; }

}  // extern "C"
