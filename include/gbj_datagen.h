/*
 * gbj_datagen.h -- seeded synthetic inputs of the workload shapes
 * (libgbj_datagen.so, built from datagen/datagen.cpp).
 *
 * A library of its own, apart from libgbjoin.so, so that the benchmark's CPU
 * arm (the oracle timed alone) generates its inputs without loading the GPU
 * library.  Every value is a pure function of (seed, stream, row), so the
 * same columns come out on every host and for any thread count.  The entry
 * points return GBJ_OK, or GBJ_ERR_INVALID for a bad argument.
 *
 * The reference has no counterpart: its benchmarks read SSB / TPC-H files
 * (apps/benchmarks/olap/benchmark-ssb/ssb-fixture.hpp:62-69), which this
 * build does not ship; these generators give inputs of the shapes the
 * measured workloads name.
 */
#ifndef GBJ_DATAGEN_H
#define GBJ_DATAGEN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Deterministic, thread-parallel generators for the workload shapes; pure
 * functions of (seed, row), identical on every host.  threads <= 0 uses all
 * hardware threads. */
int gbj_gen_build_side(uint64_t seed, uint64_t n, int32_t *h_keys,
                       int32_t *h_payload, int threads);
int gbj_gen_probe_uniform(uint64_t seed, uint64_t n, uint64_t n_build,
                          int32_t *h_keys, int32_t *h_payload, int threads);
int gbj_gen_probe_zipf(uint64_t seed, uint64_t n, uint64_t n_build,
                       double theta, double hit_rate, int32_t *h_keys,
                       int32_t *h_payload, int threads);
int gbj_gen_groupby(uint64_t seed, uint64_t n, uint64_t cardinality,
                    double theta, int32_t *h_keys, int32_t *h_values,
                    int threads);
/* out[i] = lo + a uniform draw from {0 .. hi - lo} of column stream
 * `stream` (independent streams for independent columns). */
int gbj_gen_uniform_i32(uint64_t seed, uint64_t stream, uint64_t n,
                        int32_t lo, int32_t hi, int32_t *h_out, int threads);
/* One served join + group-by query (gbj_serve_query inputs): build keys a
 * seeded permutation of 1..n_build, build groups `cardinality` distinct
 * int32 values, probe keys hitting a uniform build key with probability
 * match_rate (else a key above every build key), probe values U[0, 1000). */
int gbj_gen_serve_query(uint64_t seed, uint64_t n_build, uint64_t n_probe,
                        double match_rate, uint64_t cardinality,
                        int32_t *h_build_keys, int32_t *h_build_group,
                        int32_t *h_probe_keys, int32_t *h_probe_vals,
                        int threads);
uint64_t gbj_gen_rand(uint64_t seed, uint64_t stream, uint64_t i);
uint64_t gbj_gen_perm(uint64_t seed, uint64_t stream, uint64_t n, uint64_t i);
uint64_t gbj_gen_zipf(uint64_t seed, uint64_t stream, uint64_t n, double theta,
                      uint64_t i);
double gbj_gen_det_log(double x);
double gbj_gen_det_exp(double x);

#ifdef __cplusplus
}
#endif

#endif /* GBJ_DATAGEN_H */
