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

int32_t ref_num_radix_bits() { return NUM_RADIX_BITS; }

}  // extern "C"
