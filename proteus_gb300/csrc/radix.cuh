// Radix partitioning shared by the partitioned join and group-by.
#pragma once
#include "gbj_internal.cuh"

namespace gbj {

constexpr int kMaxPartBits = 15;

// Partitions n (key, value) tuples on digit = (f(key) >> shift) & (2^bits-1)
// into a contiguous, partition-major output.  vals == nullptr carries the
// row position.  Output either AoS (out_pairs != nullptr, int2 {key, val})
// or SoA (out_keys / out_vals).  offsets gets 2^bits + 1 entries.
// One histogram pass, then one tile pass per digit group; tuples keep no
// particular order inside a partition.  passes: 0 = one pass up to 8 bits,
// two above; 1 = one pass (bits <= 8); 2 = two passes (bits >= 2).
// hash_out (GBJ_DIGIT_HASH, AoS output only): each tuple leaves with
// fmix32(key) in place of the key, as the partitioned join consumes them.
int partition_tuples(gbj_ctx *ctx, const int32_t *keys, const int32_t *vals,
                     uint64_t n, int digit, int shift, int bits,
                     int2 *out_pairs, int32_t *out_keys, int32_t *out_vals,
                     uint64_t *offsets, cudaStream_t s, int passes = 0,
                     bool hash_out = false);

}  // namespace gbj
