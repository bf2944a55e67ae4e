/*
 * gbjoin.h -- C ABI of the GB300 relational hot path: radix partitioning,
 * hash-join build/probe and hash group-by aggregation.
 *
 * Plain C types only (pointers, sizes, int32/int64).  Column pointers named
 * d_* are device pointers that the caller owns; h_* are host pointers.  Every
 * call that takes a `stream` (a cudaStream_t passed as void*, NULL = the
 * context's own stream) is stream-ordered and returns without a device sync
 * unless its comment says otherwise.  Every entry point returns a gbj_status;
 * the text of the last error of a context is available from gbj_last_error().
 * No entry point aborts the process.
 *
 * Each declaration cites the interface of chapeiro/proteus it stands in for
 * (paths are relative to the proteus source tree).
 */
#ifndef GBJOIN_H
#define GBJOIN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */
/* Replaces gpu_run()/gpuAssert aborts (core/platform/include/platform/common/
 * gpu/gpu-common.hpp:93-110) and capacity asserts
 * (core/olap/lib/operators/gpu/gpu-hash-join-chained.cpp:60-69). */
typedef enum gbj_status {
  GBJ_OK = 0,
  GBJ_ERR_INVALID = 1,     /* bad argument (null pointer, size, enum)        */
  GBJ_ERR_OOM = 2,         /* device pool cannot hold the request            */
  GBJ_ERR_CAPACITY = 3,    /* a table or output buffer was too small         */
  GBJ_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up             */
  GBJ_ERR_CUDA = 5,        /* a CUDA runtime call failed                     */
  GBJ_ERR_UNSUPPORTED = 6, /* valid request the library does not implement  */
  GBJ_ERR_BUDGET = 7,      /* admission refused: HBM budget exhausted        */
  GBJ_ERR_CANCELLED = 8    /* request cancelled before it ran                */
} gbj_status;

typedef struct gbj_ctx gbj_ctx;     /* one device, one resident pool     */
typedef struct gbj_table gbj_table; /* a built join hash table           */

/* --------------------------------------------------------------- context */
/* Stands in for proteus::platform / MemoryManager::init + buffer_manager::init
 * (core/platform/include/platform/common/common.hpp:177-183,
 *  core/platform/include/platform/memory/memory-manager.hpp:152-154).
 * Reserves `pool_bytes` of device memory once (0 = 40% of free memory); all
 * scratch space of later calls comes from that resident pool. */
int gbj_ctx_create(int device, uint64_t pool_bytes, gbj_ctx **out);
int gbj_ctx_destroy(gbj_ctx *ctx);
const char *gbj_last_error(gbj_ctx *ctx);
/* Number of SMs and L2 bytes of the context's device (host query). */
int gbj_ctx_device_info(gbj_ctx *ctx, int *sm_count, uint64_t *l2_bytes,
                        uint64_t *smem_per_block_optin);
/* Synchronises `stream` and reports (and clears) any error a kernel latched
 * on the device (capacity overflow, bounded-wait timeout). */
int gbj_sync(gbj_ctx *ctx, void *stream);
/* Number of gbj kernels launched through this context so far. */
uint64_t gbj_kernel_launches(gbj_ctx *ctx);

/* Kernel timing, standing in for the reference's per-kernel cudaEvent
 * timers and time_block registry (core/olap/lib/operators/gpu/
 * gpu-partitioned-hash-join-chained.cpp:303-387, core/platform/include/
 * platform/util/timing.hpp:65-140).  While enabled, an event is recorded on
 * the launching stream after every kernel; a kernel's time is the interval
 * since the previous event on that stream.  Enabling or disabling clears the
 * totals.  gbj_profile_kernel / gbj_profile_dump synchronise the events. */
int gbj_profile_enable(gbj_ctx *ctx, int on);
int gbj_profile_kernel(gbj_ctx *ctx, const char *kernel, uint64_t *launches,
                       double *total_ms);
/* "name launches total_ms" lines, NUL-terminated. */
int gbj_profile_dump(gbj_ctx *ctx, char *buf, uint64_t buflen);

/* ---------------------------------------------------- resident device pool */
/* Replaces MemoryManager::mallocGpu/freeGpu and the buffer-manager block
 * pools (core/platform/lib/memory/memory-manager.cpp,
 * core/platform/lib/memory/buffer-manager.cu).  Allocation is host-side
 * bookkeeping over the block reserved at gbj_ctx_create; nothing calls
 * cudaMalloc after that. */
int gbj_pool_alloc(gbj_ctx *ctx, uint64_t bytes, void **d_ptr);
int gbj_pool_free(gbj_ctx *ctx, void *d_ptr);
int gbj_pool_stats(gbj_ctx *ctx, uint64_t *capacity, uint64_t *in_use,
                   uint64_t *peak);
/* Caps the bytes the pool hands out at `bytes` (0 = the whole pool): an
 * allocation past the cap fails with GBJ_ERR_OOM as if the pool were full.
 * The reference's MemoryManager has a fixed pool per device
 * (core/platform/lib/memory/memory-manager.cpp); this is the knob that
 * shrinks ours without re-creating the context, e.g. to leave room for other
 * users of the device or to exercise the out-of-memory paths. */
int gbj_ctx_set_pool_limit(gbj_ctx *ctx, uint64_t bytes);

/* ---------------------------------------------------- fused aggregations */
/* Aggregates computed on join matches, standing in for the parent Reduce
 * (core/olap/lib/operators/reduce-opt.cpp:52-481, gpu/gpu-reduce.cpp:155-198)
 * with gpu::Monoid update semantics (core/olap/lib/operators/gpu/
 * gmonoids.cpp:122-360).  SUM accumulates in int64, as the reference does
 * after a CastExpression (core/olap/include/olap/expressions/
 * expressions.hpp:1162).  OR and AND are the logical monoids of the
 * reference's GPU path (LogOrMonoid / LogAndMonoid, gmonoids.cpp:286-290,
 * 363-376, parsed from "or" / "and" at expression-parser.cpp:790-793): the
 * operand counts as true when it is not zero and the result is 0 or 1.  On
 * an empty input COUNT/SUM/OR give 0, AND gives 1, MIN gives INT64_MAX and
 * MAX gives INT64_MIN. */
typedef enum gbj_agg_op {
  GBJ_AGG_COUNT = 0,
  GBJ_AGG_SUM = 1,
  GBJ_AGG_MIN = 2,
  GBJ_AGG_MAX = 3,
  GBJ_AGG_OR = 4,
  GBJ_AGG_AND = 5
} gbj_agg_op;

/* Value a join aggregate reads for one matching (build row, probe row). */
typedef enum gbj_operand {
  GBJ_VAL_ONE = 0,         /* constant 1                                */
  GBJ_VAL_BUILD = 1,       /* build payload column                      */
  GBJ_VAL_PROBE = 2,       /* probe payload column                      */
  GBJ_VAL_PRODUCT = 3,     /* (int64)build payload * probe payload      */
  GBJ_VAL_BUILD_ROWID = 4, /* 0-based build row position                */
  GBJ_VAL_PROBE_ROWID = 5, /* 0-based probe row position                */
  GBJ_VAL_ROWID_XOR = 6,   /* build rowid XOR probe rowid               */
  GBJ_VAL_BUILD_KEY = 7    /* the join key                              */
} gbj_operand;

typedef struct gbj_agg {
  int32_t op;      /* gbj_agg_op  */
  int32_t operand; /* gbj_operand */
} gbj_agg;

#define GBJ_MAX_AGGS 8

/* ----------------------------------------------- chained hash join (plain) */
/* HashJoinChained / GpuHashJoinChained build side
 * (core/olap/lib/operators/hash-join-chained.cpp:262-319, open_build
 * core/olap/lib/operators/gpu/gpu-hash-join-chained.cpp:31-58).
 * Every build row is inserted (duplicate keys allowed).  `hash_bits` and
 * `max_build` are the plan's sizing fields; 0 lets the library size the
 * table from n.  A non-zero max_build smaller than n gives GBJ_ERR_CAPACITY
 * (the reference asserts).  d_payload may be NULL.  The table references
 * d_keys/d_payload: keep them alive until gbj_table_destroy. */
int gbj_join_build(gbj_ctx *ctx, const int32_t *d_keys,
                   const int32_t *d_payload, uint64_t n, int32_t hash_bits,
                   uint64_t max_build, void *stream, gbj_table **out);

/* Probe side with the parent's aggregate fused in
 * (core/olap/lib/operators/hash-join-chained.cpp:321-566 feeding
 *  gpu/gpu-reduce.cpp:155-198).  Writes n_aggs int64 results to d_out. */
int gbj_join_probe_agg(gbj_ctx *ctx, const gbj_table *table,
                       const int32_t *d_keys, const int32_t *d_payload,
                       uint64_t n, const gbj_agg *aggs, int32_t n_aggs,
                       int64_t *d_out, void *stream);

/* Probe side emitting every match as a (build row, probe row) pair, the
 * bindings HashJoinChained hands to its parent's consume().  Pairs are
 * written in no particular order.  The match count goes to *d_count; if it
 * exceeds `capacity` the pairs beyond it are dropped and gbj_sync reports
 * GBJ_ERR_CAPACITY.  d_probe_rows may be NULL to use 0..n-1 as probe row ids,
 * otherwise probe key i is reported as d_probe_rows[i]. */
int gbj_join_probe_pairs(gbj_ctx *ctx, const gbj_table *table,
                         const int32_t *d_keys, const int32_t *d_probe_rows,
                         uint64_t n, int32_t *d_build_rows,
                         int32_t *d_out_probe_rows, uint64_t capacity,
                         uint64_t *d_count, void *stream);

/* The same three calls over int64 keys: HashJoinChained with an int64 join
 * key, placed by the reference's int64 hash (the murmur3 64-bit finaliser,
 * core/olap/lib/expressions/expressions-hasher.cpp:66-84).  Payloads and
 * row ids stay int32; GBJ_VAL_BUILD_KEY gives the int64 key.  A table built
 * here is probed only by the _i64 probes (and the other way round): a
 * mismatch gives GBJ_ERR_INVALID. */
int gbj_join_build_i64(gbj_ctx *ctx, const int64_t *d_keys,
                       const int32_t *d_payload, uint64_t n, int32_t hash_bits,
                       uint64_t max_build, void *stream, gbj_table **out);
int gbj_join_probe_agg_i64(gbj_ctx *ctx, const gbj_table *table,
                           const int64_t *d_keys, const int32_t *d_payload,
                           uint64_t n, const gbj_agg *aggs, int32_t n_aggs,
                           int64_t *d_out, void *stream);
int gbj_join_probe_pairs_i64(gbj_ctx *ctx, const gbj_table *table,
                             const int64_t *d_keys, const int32_t *d_probe_rows,
                             uint64_t n, int32_t *d_build_rows,
                             int32_t *d_out_probe_rows, uint64_t capacity,
                             uint64_t *d_count, void *stream);

int gbj_table_destroy(gbj_ctx *ctx, gbj_table *table);
/* Number of slots of the table (host query). */
uint64_t gbj_table_slots(const gbj_table *table);

/* ------------------------------------------------------ radix partitioning */
/* HashPartitioner (core/olap/lib/operators/gpu/
 * gpu-partitioned-hash-join-chained.cpp:120-404, kernels in
 * gpu-partitioned-hash-join-chained-helpers.cpp:243-481) and
 * radix_cluster_nopadding / partitionHT (core/platform/lib/util/radix/joins/
 * radix-join.cpp:85-155,253-276).
 * digit = (f(key) >> shift) & (2^bits - 1) with f = identity
 * (GBJ_DIGIT_KEY, radix_cluster_nopadding) or the murmur3 32-bit finaliser
 * (GBJ_DIGIT_HASH, the GPU partitioner's hashd).  Partition p holds exactly
 * the tuples whose digit is p, contiguous and in partition order; inside a
 * partition the order is unspecified (as with the reference's GPU
 * HashPartitioner), so sorted per partition the result equals the
 * counting-sort cluster of radix_cluster_nopadding.
 * d_payload may be NULL: then the 0-based row position is carried instead.
 * d_offsets receives 2^bits + 1 partition start offsets.  bits in [1, 15],
 * shift + bits <= 32, n < 2^31.  No host synchronisation. */
typedef enum gbj_digit { GBJ_DIGIT_KEY = 0, GBJ_DIGIT_HASH = 1 } gbj_digit;

int gbj_partition(gbj_ctx *ctx, const int32_t *d_keys,
                  const int32_t *d_payload, uint64_t n, int32_t digit,
                  int32_t shift, int32_t bits, int32_t *d_out_keys,
                  int32_t *d_out_payload, uint64_t *d_offsets, void *stream);

/* ------------------------------------------------------ radix hash join */
/* GpuPartitionedHashJoinChained (core/olap/lib/operators/gpu/
 * gpu-partitioned-hash-join-chained.cpp:612-1586) and RJStepwise
 * (core/platform/lib/util/radix/joins/radix-join.cpp:278-375): partition
 * both sides on hash bits so each build partition's table fits on-chip,
 * then build and probe per partition with the aggregate fused in.  Each side
 * carries ONE 32-bit value into the partitions: its payload if an aggregate
 * reads GBJ_VAL_BUILD/PROBE/PRODUCT, its row position if one reads a rowid
 * operand; when one side needs both, both sides carry row positions and
 * matches read the payloads by row.  Work items are sized on the device, so
 * the call never synchronises with the host. */
/* Radix clustering of {int64 key, int64 payload} tuples: the aggregation
 * twins radix_cluster_nopadding / partitionHT of core/platform/lib/util/
 * radix/aggregations/radix-aggr.cpp:82-155,237-259 (agg::tuple_t, KEY_8B).
 * Digit = (key >> shift) & (2^bits - 1) of the 64-bit key; output
 * partition-major (unordered inside a partition), offsets 2^bits + 1;
 * d_payload NULL carries 0-based row ids.  partitionHT's clustering is two
 * calls (shift 0, bits 7; then per the reference, bits 7..13) or one call
 * with bits 14, which gives the same clusters and counts. */
int gbj_partition_i64(gbj_ctx *ctx, const int64_t *d_keys,
                      const int64_t *d_payload, uint64_t n, int32_t shift,
                      int32_t bits, int64_t *d_out_keys,
                      int64_t *d_out_payload, uint64_t *d_offsets,
                      void *stream);
/* RadixNest over int64 keys (Nest, core/olap/lib/operators/radix-nest.cpp:
 * 326-700, on the aggregation twin's clusters and bucket chains,
 * radix-aggr.cpp:163-259): one output row per distinct key with COUNT and,
 * for d_vals not NULL, SUM (int64, two's-complement wrap), MIN and MAX of
 * the value column (0 when d_vals is NULL).  Groups come out unordered;
 * *d_n_groups (device) gets their number even when it exceeds out_capacity
 * (then GBJ_ERR_CAPACITY at the next sync).  expected_groups sizes the
 * table (0: min(n, 2^24)); more distinct keys than the table holds also
 * give GBJ_ERR_CAPACITY. */
int gbj_nest_i64(gbj_ctx *ctx, const int64_t *d_keys, const int64_t *d_vals, uint64_t n,
                 uint64_t expected_groups, int64_t *d_out_keys, int64_t *d_out_count,
                 int64_t *d_out_sum, int64_t *d_out_min, int64_t *d_out_max,
                 uint64_t out_capacity, uint64_t *d_n_groups, void *stream);
/* RJStepwise of the aggregation twin (radix-aggr.cpp:261-358): the number of
 * (R, S) pairs with equal int64 keys into *d_count (device). */
int gbj_radix_join_count_i64(gbj_ctx *ctx, const int64_t *d_r_keys, uint64_t nr,
                             const int64_t *d_s_keys, uint64_t ns, int64_t *d_count,
                             void *stream);

/* Every field is honoured or the call fails with GBJ_ERR_UNSUPPORTED: bits
 * and log_parts in [0, 15]; passes 1 needs bits <= 8 and passes 2 bits >= 2
 * (with bits unset, a pinned pass count bounds the automatic choice); block
 * is 0 or the join kernel's 1024 threads. */
typedef struct gbj_radix_params {
  int32_t bits;       /* radix bits, 0 = autotuned                        */
  int32_t passes;     /* 1 or 2, 0 = one pass up to 8 bits, two above     */
  int32_t block;      /* threads per block of the join kernel, 0 = auto   */
  int32_t log_parts;  /* plan field log_parts (reference: 13), 0 = unset  */
} gbj_radix_params;

int gbj_radix_join_agg(gbj_ctx *ctx, const int32_t *d_build_keys,
                       const int32_t *d_build_payload, uint64_t n_build,
                       const int32_t *d_probe_keys,
                       const int32_t *d_probe_payload, uint64_t n_probe,
                       const gbj_radix_params *params, const gbj_agg *aggs,
                       int32_t n_aggs, int64_t *d_out, void *stream);

/* The partitioned join with a minor key: GpuPartitionedHashJoinChained built
 * with build_k_minor / probe_k_minor (core/olap/lib/plan/plan-parser.cpp:
 * 872-880), which after the key compare of a chain match also requires the
 * build and probe minor keys to be equal (core/olap/lib/operators/gpu/
 * gpu-partitioned-hash-join-chained.cpp:1284-1333).  Partitions are on the
 * (major) key's hash; both sides carry their row positions and a match reads
 * the minor keys and payloads by row, so any operand mix is allowed.  Both
 * minor columns are required (GBJ_ERR_INVALID otherwise). */
int gbj_radix_join_agg_minor(gbj_ctx *ctx, const int32_t *d_build_keys,
                             const int32_t *d_build_minor,
                             const int32_t *d_build_payload, uint64_t n_build,
                             const int32_t *d_probe_keys,
                             const int32_t *d_probe_minor,
                             const int32_t *d_probe_payload, uint64_t n_probe,
                             const gbj_radix_params *params,
                             const gbj_agg *aggs, int32_t n_aggs,
                             int64_t *d_out, void *stream);

/* ------------------------------------------------------ hash group-by */
/* GpuHashGroupByChained (core/olap/lib/operators/gpu/
 * gpu-hash-group-by-chained.cpp:77-556) with HashGroupByChained's emit scan
 * (core/olap/lib/operators/hash-group-by-chained.cpp:638-853).  One output
 * row per distinct key with COUNT (int64), SUM of the value (int64), MIN and
 * MAX (int32).  Groups come out in no particular order; *d_n_groups gets the
 * group count.  More groups than out_capacity gives GBJ_ERR_CAPACITY at
 * gbj_sync.  Any of the five output columns may be NULL. */
typedef struct gbj_groupby_params {
  int32_t hash_bits;        /* plan field, 0 = unset                     */
  int32_t strategy;         /* 0 auto, 1 on-chip + global table,
                               2 radix-partitioned                       */
  uint64_t max_input_size;  /* plan field maxInputSize, 0 = unset        */
  uint64_t expected_groups; /* cardinality hint, 0 = unknown             */
} gbj_groupby_params;

int gbj_groupby(gbj_ctx *ctx, const int32_t *d_keys, const int32_t *d_values,
                uint64_t n, const gbj_groupby_params *params,
                int32_t *d_out_keys, int64_t *d_out_count, int64_t *d_out_sum,
                int32_t *d_out_min, int32_t *d_out_max, uint64_t out_capacity,
                uint64_t *d_n_groups, void *stream);

/* gbj_groupby over int64 keys (a HashGroupByChained whose key expression is
 * int64, placed by the reference's int64 hash, expressions-hasher.cpp:
 * 66-84): one output row per distinct key with COUNT, SUM (int64) and MIN /
 * MAX (int32) of the int32 value column.  params as for gbj_groupby;
 * strategy 2 (radix-partitioned) is not offered for int64 keys and gives
 * GBJ_ERR_UNSUPPORTED.  The grouping engine is the one gbj_nest_i64 uses. */
int gbj_groupby_i64(gbj_ctx *ctx, const int64_t *d_keys, const int32_t *d_values,
                    uint64_t n, const gbj_groupby_params *params,
                    int64_t *d_out_keys, int64_t *d_out_count, int64_t *d_out_sum,
                    int32_t *d_out_min, int32_t *d_out_max, uint64_t out_capacity,
                    uint64_t *d_n_groups, void *stream);

/* ------------------------------------------------------------ bloom filter */
/* BloomFilterBuild / BloomFilterProbe (core/olap/lib/operators/bloom-filter/
 * bloom-filter-build.cpp:28-59, bloom-filter-probe.cpp:28-53): a filter of
 * filter_size (power of two) flags; a key's flag is at key & (filter_size-1)
 * (bloom-filter.cpp:65-95).  Build sets the flags of d_keys; probe writes the
 * positions of the rows whose flag is set (ascending) and their number --
 * exactly the rows the reference's probe passes to its parent.  Flags are
 * bits: filter_size / 8 bytes from the pool. */
typedef struct gbj_bloom gbj_bloom;

int gbj_bloom_build(gbj_ctx *ctx, const int32_t *d_keys, uint64_t n,
                    uint64_t filter_size, void *stream, gbj_bloom **out);
int gbj_bloom_probe(gbj_ctx *ctx, const gbj_bloom *filter,
                    const int32_t *d_keys, uint64_t n, int32_t *d_rows_out,
                    uint64_t *d_count, void *stream);
int gbj_bloom_destroy(gbj_ctx *ctx, gbj_bloom *filter);

/* ---------------------------------------------------------- hash rearrange */
/* HashRearrange / GpuHashRearrange (core/olap/lib/operators/
 * hash-rearrange.cpp:131-405, gpu/gpu-hash-rearrange.cpp:87-700): every row
 * goes to bucket hash(key) mod num_buckets, hash = the expression hasher's
 * 64-bit hash of an int32 (core/olap/lib/expressions/expressions-hasher.cpp:
 * 39-58), unsigned remainder -- the same bucket as the reference.  The
 * n_cols int32 columns (the key column among them) are written bucket-major
 * to d_out_cols; d_bucket_offsets gets num_buckets + 1 entries (bucket b is
 * rows [off[b], off[b+1])).  Rows keep no particular order inside a bucket,
 * as the reference's concurrent block appends do not. */
#define GBJ_REARRANGE_MAX_COLS 16

int gbj_hash_rearrange(gbj_ctx *ctx, const int32_t *const *d_cols,
                       int32_t n_cols, uint64_t n, int32_t key_col,
                       uint32_t num_buckets, int32_t *const *d_out_cols,
                       uint64_t *d_bucket_offsets, void *stream);

/* ------------------------------------------------------------------ sort */
/* ORDER BY one int32 column (the reference's GPU sort, core/olap/lib/
 * operators/gpu/gpu-sort.cpp, which calls thrust::sort from
 * core/platform/lib/util/sort/gpu/sort-util.cu:191-218): writes the n_cols
 * int32 columns to d_out_cols with rows ordered by column key_col, signed
 * ascending (descending != 0: descending); rows with equal keys keep their
 * input order. */
#define GBJ_SORT_MAX_COLS 16

int gbj_sort_by_key(gbj_ctx *ctx, const int32_t *const *d_cols, int32_t n_cols,
                    uint64_t n, int32_t key_col, int32_t descending,
                    int32_t *const *d_out_cols, void *stream);

/* ------------------------------------------------------ column helpers */
/* Global aggregate over one int32 column restricted to an optional row list
 * (Reduce, core/olap/lib/operators/reduce-opt.cpp:52-481).  d_rows may be
 * NULL for all rows 0..n-1. */
int gbj_reduce(gbj_ctx *ctx, const int32_t *d_col, const int32_t *d_rows,
               uint64_t n, const gbj_agg *aggs, int32_t n_aggs,
               int64_t *d_out, void *stream);

/* Gather d_out[i] = d_col[d_rows[i]] (late materialisation of a join side). */
int gbj_gather(gbj_ctx *ctx, const int32_t *d_col, const int32_t *d_rows,
               uint64_t n, int32_t *d_out, void *stream);

/* Select (core/olap/lib/operators/select.cpp:26-37) for the predicate forms
 * the workloads use: lo <= col <= hi (inclusive).  Writes the positions of
 * passing rows (ascending) to d_rows_out and their number to *d_count. */
int gbj_select_range(gbj_ctx *ctx, const int32_t *d_col, uint64_t n,
                     int32_t lo, int32_t hi, int32_t *d_rows_out,
                     uint64_t *d_count, void *stream);

/* ------------------------------------------------ batched star join */
/* Up to GBJ_STAR_MAX_QUERIES star-join queries over one fact table in one
 * pass.  Each query computes what a reference plan of
 *   select(dim predicate) -> hashjoin-chained(build dim.PK, probe fact.FK)
 *   for each joined dimension -> groupby(dimA.attr, dimB.attr;
 *   COUNT, SUM(int64 price * quantity))
 * computes with the operators of core/olap/lib/operators/select.cpp:26-37,
 * hash-join-chained.cpp:262-566 and hash-group-by-chained.cpp:267-853; the
 * reference runs such plans one query at a time (its SSB plans,
 * tests/inputs/plans/gpu-ssb/ *.json, have this shape).  Here every query of
 * a batch shares one read of the fact columns.
 *
 * A dimension's primary keys are dense (d_keys NULL: row i has key
 * key_base + i, and a fact foreign key outside [key_base, key_base + n)
 * matches nothing) or a column of distinct int32 values (d_keys, e.g. the
 * SSB date dimension's yyyymmdd keys), which the plan places in an
 * open-addressing table at creation; a duplicate primary key fails the
 * plan with GBJ_ERR_INVALID.  Group keys must come from
 * joined dimensions and their declared [attr_min, attr_max] domains must
 * multiply to at most GBJ_STAR_MAX_GROUPS groups; a value outside its
 * declared domain is reported as GBJ_ERR_INVALID at gbj_sync.
 *
 * Results of query q: rows [q * group_cap, q * group_cap + d_n_groups[q])
 * of the output columns, one per group with at least one row, sorted by
 * (key_a, key_b). */
#define GBJ_STAR_MAX_DIMS 4
#define GBJ_STAR_MAX_ATTRS 4
#define GBJ_STAR_MAX_QUERIES 64
#define GBJ_STAR_MAX_GROUPS 4096

typedef enum gbj_attr_type { GBJ_ATTR_I32 = 0, GBJ_ATTR_I8 = 1 } gbj_attr_type;

typedef struct gbj_star_dim {
  uint64_t n;                              /* rows (< 2^31)               */
  int32_t key_base;                        /* primary key of row 0        */
  int32_t n_attrs;
  const void *d_attr[GBJ_STAR_MAX_ATTRS];  /* int32 or int8 columns       */
  int32_t attr_type[GBJ_STAR_MAX_ATTRS];   /* gbj_attr_type               */
  int32_t attr_min[GBJ_STAR_MAX_ATTRS];    /* value domain (group keys)   */
  int32_t attr_max[GBJ_STAR_MAX_ATTRS];
  const int32_t *d_keys;                   /* primary keys, NULL = dense  */
} gbj_star_dim;

typedef struct gbj_star_fact {
  uint64_t n;
  int32_t n_dims;                          /* 1..GBJ_STAR_MAX_DIMS        */
  const int32_t *d_fk[GBJ_STAR_MAX_DIMS];  /* fk column d -> dimension d  */
  const int32_t *d_quantity;
  const int32_t *d_price;
} gbj_star_fact;

typedef struct gbj_star_query {
  int32_t join_mask;                       /* bit d: join dimension d     */
  int32_t pred_attr[GBJ_STAR_MAX_DIMS];    /* attribute filtered, -1 none */
  int32_t pred_lo[GBJ_STAR_MAX_DIMS];      /* lo <= attr <= hi            */
  int32_t pred_hi[GBJ_STAR_MAX_DIMS];
  int32_t group_dim[2];                    /* group key a, b: dimension   */
  int32_t group_attr[2];                   /*   and attribute             */
} gbj_star_query;

typedef struct gbj_star_out {
  int32_t *d_key_a;       /* [n_queries * group_cap] each                 */
  int32_t *d_key_b;
  int64_t *d_count;
  int64_t *d_sum;         /* SUM((int64)price * quantity)                 */
  uint64_t *d_n_groups;   /* [n_queries]                                  */
  uint64_t group_cap;
} gbj_star_out;

/* A plan holds a schema's per-batch device state (dimension masks, group
 * tables, the descriptor buffers) and the CUDA graphs of a batch.  The
 * columns stay caller-owned and must outlive the plan. */
typedef struct gbj_star_plan gbj_star_plan;

int gbj_star_plan_create(gbj_ctx *ctx, const gbj_star_fact *fact,
                         const gbj_star_dim *dims, gbj_star_plan **out);
/* Runs n_queries (1..GBJ_STAR_MAX_QUERIES) queries on `stream`.  use_graph:
 * the batch's copies and three kernels are captured into a CUDA graph on
 * first use and replayed afterwards (two graphs alternate so the host can
 * prepare the next batch while one runs).  Runs of one plan must be ordered
 * (one stream, or synchronised): they share the plan's device state. */
int gbj_star_run(gbj_star_plan *plan, const gbj_star_query *queries,
                 int32_t n_queries, const gbj_star_out *out,
                 int32_t use_graph, void *stream);
void gbj_star_plan_destroy(gbj_star_plan *plan);

/* ------------------------------------------------------- query serving */
/* A request loop for join + group-by queries over resident device columns:
 *   SELECT b.group, COUNT(*), SUM((int64)p.value)
 *   FROM build b JOIN probe p ON b.key = p.key GROUP BY b.group
 * with HashJoinChained semantics (every build row inserted, duplicates
 * allowed; core/olap/lib/operators/hash-join-chained.cpp:262-566) feeding
 * HashGroupByChained (hash-group-by-chained.cpp:267-853).
 *
 * It stands in for the reference's per-query execution path: operators that
 * allocate their tables through MemoryManager / buffer_manager at open() and
 * free them at close() (core/olap/lib/operators/gpu/
 * gpu-hash-join-chained.cpp:31-73, core/platform/lib/memory/
 * memory-manager.cpp), one query after another with a stream sync per GPU
 * operator.  Here the tables of admitted queries come from the context's
 * resident pool within an HBM budget; queries that arrive while others run
 * are admitted as soon as an in-flight slot and budget are free, and each
 * admitted group runs as one batch: five persistent kernels (clear, build,
 * probe + group-by, emit, finish) over the work items of all its queries,
 * captured once per slot as a CUDA graph and replayed.  Slots run on their
 * own streams, so batches overlap on the device.
 *
 * max_batch = 1, max_inflight = 1, use_graph = 0 is the plain form: one query
 * per launch sequence, each waited for before the next starts.
 *
 * Output groups come out in no particular order; *out_n_groups is written
 * when the query completes.  Output pointers may be device memory or mapped
 * pinned host memory. */
#define GBJ_SERVE_MAX_BATCH 64

typedef struct gbj_serve_query {
  const int32_t *d_build_keys;
  const int32_t *d_build_group;  /* group key of each build row        */
  uint64_t n_build;
  const int32_t *d_probe_keys;
  const int32_t *d_probe_vals;
  uint64_t n_probe;
  uint64_t expected_groups;      /* upper bound of distinct groups     */
  int32_t *out_group;
  int64_t *out_count;
  int64_t *out_sum;
  uint64_t *out_n_groups;
  uint64_t out_capacity;
  uint64_t table_id;             /* 0: build from d_build_keys/d_build_group
                                    per query; else a table registered with
                                    gbj_server_register_table (the build
                                    columns and n_build are then ignored) */
} gbj_serve_query;

typedef struct gbj_server_params {
  uint64_t hbm_budget;   /* pool bytes queries in flight may hold (0 = pool) */
  int32_t max_batch;     /* queries per batch, 1..GBJ_SERVE_MAX_BATCH        */
  int32_t max_inflight;  /* batches in flight (streams), 1..8                */
  int32_t use_graph;     /* replay each slot's batch from a CUDA graph       */
  int32_t large_slots;   /* slots reserved for large queries (0 = one class) */
  uint64_t small_rows;   /* a query with n_build + n_probe above this is
                            large (0 = 2^22); large queries queue apart,
                            run on low-priority streams with one work item
                            per CTA, so small batches on the high-priority
                            slots take SMs as the large batch's CTAs retire */
} gbj_server_params;

typedef struct gbj_server gbj_server;

int gbj_server_create(gbj_ctx *ctx, const gbj_server_params *params,
                      gbj_server **out);
/* Queues a query (non-blocking; the columns and outputs must stay valid
 * until it completes).  A query whose tables exceed the whole budget is
 * completed at once with GBJ_ERR_BUDGET. */
int gbj_server_submit(gbj_server *srv, const gbj_serve_query *q,
                      uint64_t *ticket);
/* Queues n queries under one lock (so the request loop sees them together);
 * tickets[i] gets query i's ticket.  All or none are queued. */
int gbj_server_submit_batch(gbj_server *srv, const gbj_serve_query *qs,
                            uint64_t n, uint64_t *tickets);
/* Waits up to timeout_s (< 0: forever) for a query; *status gets its
 * result status.  Returns GBJ_ERR_TIMEOUT if it is still running. */
int gbj_server_wait(gbj_server *srv, uint64_t ticket, double timeout_s,
                    int32_t *status);
/* Host-clock seconds (since the server started) at which the query was
 * submitted, launched and seen complete; -1 for a stage not reached. */
int gbj_server_times(gbj_server *srv, uint64_t ticket, double *submitted,
                     double *launched, double *completed);
/* Cancels a query that is still queued (not yet launched): it completes at
 * once with status GBJ_ERR_CANCELLED and *cancelled = 1.  A query already
 * launched or complete is left alone (*cancelled = 0).  The reference runs
 * one query at a time with nothing queued to cancel; this is the serving
 * loop's own control. */
int gbj_server_cancel(gbj_server *srv, uint64_t ticket, int32_t *cancelled);
/* paused != 0: the loop launches no new batches (batches in flight finish,
 * submissions queue up); 0 resumes.  gbj_server_destroy resumes first. */
int gbj_server_pause(gbj_server *srv, int32_t paused);
/* Number of automatic retries so far: a query (or a registered table) whose
 * distinct build groups outnumbered its expected_groups runs once more with
 * a group table sized for n_build groups, which cannot overflow; only a
 * query that still fails reports GBJ_ERR_CAPACITY. */
int gbj_server_retries(gbj_server *srv, uint64_t *retried);
/* Waits for every submitted query (a paused server must be resumed for its
 * queued queries to complete). */
int gbj_server_drain(gbj_server *srv);
/* Totals: queries completed, batches launched, peak budget bytes held. */
int gbj_server_stats(gbj_server *srv, uint64_t *completed, uint64_t *batches,
                     uint64_t *peak_bytes);
/* Device time of the completed batches, each from before its first
 * operation to after its last (milliseconds, summed; batches of different
 * in-flight slots may overlap, so with one slot in flight the sum is the
 * time the GPU spent on the server's work). */
int gbj_server_busy(gbj_server *srv, double *batch_ms);
/* Drains, stops the request loop and frees the server. */
int gbj_server_destroy(gbj_server *srv);
/* Builds the join table and group-key map of one build relation once and
 * keeps it resident in the pool, counted against the HBM budget, until
 * unregistered.  Queries that set table_id to *table_id skip the clear and
 * build phases and reset only their own group counters.  Builds
 * synchronously on the context's stream; the build columns may be freed on
 * return.  GBJ_ERR_BUDGET if it does not fit the budget. */
int gbj_server_register_table(gbj_server *srv, const int32_t *d_build_keys,
                              const int32_t *d_build_group, uint64_t n_build,
                              uint64_t expected_groups, uint64_t *table_id);
/* Drains the server, then frees the table.  No query naming it may be
 * submitted while this runs. */
int gbj_server_unregister_table(gbj_server *srv, uint64_t table_id);

/* -------------------------------------------------------------- autotuner */
/* Times candidate plans on the caller's inputs (one warm-up run, then the
 * fastest of two timed runs, CUDA events on `stream`) and caches the winner
 * in the context under the operation and the log2 sizes of its inputs.
 * Later calls of that shape that pass no explicit sizing use it:
 *   radix join     join kernel block size (512: two blocks per SM with
 *                  4608-tuple build chunks; 1024: one block, 9216) and,
 *                  for each, partition bits 1..15 (bits > 8 means two
 *                  passes) -- gbj_radix_join_agg with params NULL or zero
 *                  bits / block;
 *   plain join     table size 2^hash_bits (load factor 1/2, 1/4, 1/8) --
 *                  gbj_join_build with hash_bits 0;
 *   group-by       strategy 1, or strategy 2 with its partition bits --
 *                  gbj_groupby with strategy 0 and the same
 *                  expected_groups.
 * The reference sizes these by hand per plan (hash_bits, maxInputSize) and
 * fixes its radix bits at compile time (NUM_RADIX_BITS,
 * core/platform/lib/util/radix/joins/radix-join.cpp). */
int gbj_autotune_radix_join(gbj_ctx *ctx, const int32_t *d_build_keys,
                            const int32_t *d_build_payload, uint64_t n_build,
                            const int32_t *d_probe_keys,
                            const int32_t *d_probe_payload, uint64_t n_probe,
                            const gbj_agg *aggs, int32_t n_aggs,
                            int32_t *best_bits, double *best_ms, void *stream);
int gbj_autotune_join(gbj_ctx *ctx, const int32_t *d_build_keys,
                      const int32_t *d_build_payload, uint64_t n_build,
                      const int32_t *d_probe_keys,
                      const int32_t *d_probe_payload, uint64_t n_probe,
                      const gbj_agg *aggs, int32_t n_aggs,
                      int32_t *best_hash_bits, double *best_ms, void *stream);
int gbj_autotune_groupby(gbj_ctx *ctx, const int32_t *d_keys,
                         const int32_t *d_values, uint64_t n,
                         uint64_t expected_groups, int32_t *best_strategy,
                         int32_t *best_bits, double *best_ms, void *stream);
/* Cached decision for op "radixblock" (a = n_build, b = n_probe; the join
 * kernel's block size), "radix" / "radix512" (the partition bits used with
 * 1024 / 512 threads), "join" (a = n_build, b = 0) or "groupby" (a = n,
 * b = expected_groups; value = strategy << 8 | bits); -1 when none. */
int gbj_tune_lookup(gbj_ctx *ctx, const char *op, uint64_t a, uint64_t b,
                    int32_t *value);
int gbj_tune_clear(gbj_ctx *ctx);
/* Text file, one "op log2a log2b value" line per decision. */
int gbj_tune_save(gbj_ctx *ctx, const char *path);
int gbj_tune_load(gbj_ctx *ctx, const char *path);

/* ------------------------------------------------------------ plan façade */
/* Executes a JSON plan in the reference's plan format (operator names and
 * fields of core/olap/lib/plan/plan-parser.cpp; expressions of
 * core/olap/lib/plan/expression-parser.cpp) over int32 device columns named
 * in a catalog (relation name = the scan plugin's "name", attribute = the
 * projection's "attrName").  Supported operators: scan, select, project,
 * sort, hash-rearrange / hash-pack, hashjoin-chained,
 * partitioned-hashjoin-chained, join, groupby / hashgroupby-chained (one
 * int32 key) and reduce (the last two at the root, or under a root sort);
 * expressions recordProjection, int, int64, bool, cast, eq, lt, le, gt, ge,
 * and, multiply; accumulators sum, max, min.  Anything else gives
 * GBJ_ERR_UNSUPPORTED with a message naming it.  Sizing fields (hash_bits,
 * maxBuildInputSize, maxInputSize) are capacity hints.  Execution is
 * synchronous; results are int64 host columns (group-by rows sorted by key).
 * The catalog holds pointers only: columns stay caller-owned. */
typedef struct gbj_catalog gbj_catalog;
typedef struct gbj_result gbj_result;

int gbj_catalog_create(gbj_ctx *ctx, gbj_catalog **out);
int gbj_catalog_add_column(gbj_catalog *cat, const char *rel,
                           const char *attr, const int32_t *d_col, uint64_t n);
/* Loads the int32 columns (int, boolean, dictionary-coded string) of a
 * catalog.json in the reference's columnar file layout (tools/prepare_data.py:
 * one little-endian binary file per column at "<base_dir>/<path>.<attrName>")
 * into the context's pool and registers them as (path, attrName); relation
 * NULL loads every relation, else only the one whose key or path matches.
 * int64 / date / float columns are skipped.  The catalog owns these columns. */
int gbj_catalog_load(gbj_catalog *cat, const char *catalog_json,
                     const char *base_dir, const char *relation,
                     uint64_t *columns_loaded);
int gbj_catalog_destroy(gbj_catalog *cat);
/* Parses and checks a plan (operator names, required fields) without a GPU;
 * on failure err gets the message. */
int gbj_plan_validate(const char *plan_json, char *err, uint64_t err_len);
int gbj_plan_execute(gbj_catalog *cat, const char *plan_json,
                     gbj_result **out);
int gbj_result_shape(const gbj_result *r, int32_t *n_cols, uint64_t *n_rows);
const char *gbj_result_name(const gbj_result *r, int32_t col);
int gbj_result_column(const gbj_result *r, int32_t col, int64_t *h_out);
void gbj_result_destroy(gbj_result *r);

/* --------------------------------------- allocation-free join + aggregate */
/* This entry point has no counterpart in the reference.  It is for callers
 * that may not allocate device memory at the moment they call: a host engine
 * whose buffer manager has already reserved the device memory it is allowed
 * to use (the reference's buffer manager pre-reserves its GPU block pools at
 * start-up), a code path with a fixed memory budget checked at admission
 * time, or a latency-critical path where cudaMalloc's implicit device
 * synchronisation cannot be paid.  It needs no gbj_ctx and calls no
 * allocating routine (no cudaMalloc, cudaFree or library allocator).
 *
 * It builds the same table as gbj_join_build and probes it as
 * gbj_join_probe_agg does, with the same results, but the table lives in one
 * fixed array inside the library's device code: 16 MiB, enough for build
 * sides of up to GBJ_NOALLOC_MAX_BUILD rows.  Every GPU that loads the
 * library holds that array until the process exits.  A larger build side is
 * rejected with GBJ_ERR_CAPACITY and a message.
 *
 * Runs on `stream` (NULL = the legacy default stream) of the current device.
 * The first call on a device looks up the array's device address for that
 * device (cudaGetSymbolAddress); make that first call before any stream
 * capture.  After cudaDeviceReset the next call on that device looks the
 * address up again, in the new context.  All calls share the one array and it keeps the previous call's
 * contents: each call clears the part it uses first, and calls whose work
 * overlaps on the GPU (other streams, other host threads) race on the table,
 * so the caller must order them.  On failure the message is available from
 * gbj_last_error(NULL) on the calling thread. */
#define GBJ_NOALLOC_MAX_BUILD (1u << 20)

int gbj_join_agg_noalloc(const int32_t *d_build_keys,
                         const int32_t *d_build_payload, uint64_t n_build,
                         const int32_t *d_probe_keys,
                         const int32_t *d_probe_payload, uint64_t n_probe,
                         const gbj_agg *aggs, int32_t n_aggs, int64_t *d_out,
                         void *stream);

#ifdef __cplusplus
}
#endif

#endif /* GBJOIN_H */
