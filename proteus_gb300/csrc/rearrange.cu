// Hash rearrange: every row goes to bucket hash(key) mod numOfBuckets and the
// columns come out bucket-major.
//
// Stands in for HashRearrange / GpuHashRearrange (core/olap/lib/operators/
// hash-rearrange.cpp:131-405, gpu/gpu-hash-rearrange.cpp:87-700), the
// router-side partitioner of "hash-pack" plans: the target bucket is the
// expression hasher's 64-bit hash of the key (expressions-hasher.cpp:39-58)
// with an unsigned remainder (expressions-generator.cpp:1215-1230), so every
// row lands in the same bucket as in the reference.  The reference appends
// rows to per-bucket 2 MiB blocks; here each bucket is one contiguous range
// (block boundaries follow from the offsets).
//
// GB300 design: one streaming kernel computes the bucket of every row; the
// tile-pass radix partitioner (radix.cu) sorts (bucket, row) pairs; one gather
// kernel then writes every column in bucket order (the row id is read once
// per output row for all columns).
#include <algorithm>

#include "gbj_internal.cuh"
#include "radix.cuh"

using namespace gbj;

namespace {

constexpr int kMaxCols = GBJ_REARRANGE_MAX_COLS;

// The expression hasher's int32 hash: sign-extend to 64 bits, then the
// murmur3 finaliser steps with its 32-bit constants in 64-bit arithmetic.
__device__ __forceinline__ uint64_t hash_int32_64(int32_t k) {
  uint64_t h = (uint64_t)(int64_t)k;
  h ^= h >> 16;
  h *= 0x85ebca6bull;
  h ^= h >> 13;
  h *= 0xc2b2ae35ull;
  h ^= h >> 16;
  return h;
}

__global__ void __launch_bounds__(256)
    k_bucket_ids(const int32_t *__restrict__ keys, uint64_t n, uint64_t buckets, int32_t *__restrict__ ids) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride)
    ids[i] = (int32_t)(hash_int32_64(__ldcs(keys + i)) % buckets);
}

struct Cols {
  const int32_t *in[kMaxCols];
  int32_t *out[kMaxCols];
  int32_t n;
};

__global__ void __launch_bounds__(256)
    k_gather_cols(const int2 *__restrict__ pairs, uint64_t n, Cols c) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    const uint32_t r = (uint32_t)__ldcs(&pairs[i].y);
#pragma unroll 4
    for (int j = 0; j < c.n; ++j) c.out[j][i] = __ldg(c.in[j] + r);
  }
}

// Digit of an int64 key: (key >> shift) & mask over the 64-bit key.
__global__ void __launch_bounds__(256)
    k_digits_i64(const int64_t *__restrict__ keys, uint64_t n, int shift, uint64_t mask, int32_t *__restrict__ ids) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride)
    ids[i] = (int32_t)(((uint64_t)__ldcs(keys + i) >> shift) & mask);
}

// Clustered {int64 key, int64 payload} tuples (payload null: row ids).
__global__ void __launch_bounds__(256)
    k_gather_i64(const int2 *__restrict__ pairs, uint64_t n, const int64_t *__restrict__ keys,
                 const int64_t *__restrict__ payload, int64_t *__restrict__ out_keys, int64_t *__restrict__ out_payload) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    const uint32_t r = (uint32_t)__ldcs(&pairs[i].y);
    out_keys[i] = __ldg(keys + r);
    out_payload[i] = payload ? __ldg(payload + r) : (int64_t)r;
  }
}

}  // namespace

// Radix clustering of 16-byte {int64 key, int64 payload} tuples, the
// aggregation twin of radix_cluster_nopadding / partitionHT
// (core/platform/lib/util/radix/aggregations/radix-aggr.cpp:82-155,237-259):
// one digit kernel, the tile-pass partitioner on (digit, row) pairs, one
// gather of the 16-byte tuples.
extern "C" int gbj_partition_i64(gbj_ctx *ctx, const int64_t *d_keys, const int64_t *d_payload, uint64_t n,
                                 int32_t shift, int32_t bits, int64_t *d_out_keys, int64_t *d_out_payload,
                                 uint64_t *d_offsets, void *stream) {
  if (!ctx) return GBJ_ERR_INVALID;
  if (bits < 1 || bits > kMaxPartBits || shift < 0 || shift > 63)
    return set_error(ctx, GBJ_ERR_INVALID, "partition_i64: bits must be 1..15, shift 0..63");
  if (n && (!d_keys || !d_out_keys || !d_out_payload)) return set_error(ctx, GBJ_ERR_INVALID, "partition_i64: null column");
  if (!d_offsets) return set_error(ctx, GBJ_ERR_INVALID, "partition_i64: null offsets");
  if (n >= (1ull << 31)) return set_error(ctx, GBJ_ERR_INVALID, "partition_i64: n >= 2^31");
  cudaStream_t s = pick_stream(ctx, stream);
  prof_mark(ctx, s);
  if (n == 0) {
    GBJ_CHECK_CUDA(ctx, cudaMemsetAsync(d_offsets, 0, sizeof(uint64_t) * ((1ull << bits) + 1), s));
    return GBJ_OK;
  }
  Scratch scratch(ctx, s);
  int32_t *ids;
  int2 *pairs;
  GBJ_TRY(scratch.get(n, &ids));
  GBJ_TRY(scratch.get(n, &pairs));
  const unsigned grid = (unsigned)std::min<uint64_t>((n + 255) / 256, (uint64_t)ctx->sm_count * 16);
  k_digits_i64<<<grid, 256, 0, s>>>(d_keys, n, shift, (1ull << bits) - 1, ids);
  GBJ_TRY(after_launch(ctx, "k_digits_i64", s));
  GBJ_TRY(partition_tuples(ctx, ids, nullptr, n, GBJ_DIGIT_KEY, 0, bits, pairs, nullptr, nullptr, d_offsets, s));
  k_gather_i64<<<grid, 256, 0, s>>>(pairs, n, d_keys, d_payload, d_out_keys, d_out_payload);
  return after_launch(ctx, "k_gather_i64", s);
}

extern "C" int gbj_hash_rearrange(gbj_ctx *ctx, const int32_t *const *d_cols, int32_t n_cols, uint64_t n,
                                  int32_t key_col, uint32_t num_buckets, int32_t *const *d_out_cols,
                                  uint64_t *d_bucket_offsets, void *stream) {
  if (!ctx) return GBJ_ERR_INVALID;
  if (n_cols < 1 || n_cols > kMaxCols || key_col < 0 || key_col >= n_cols || !d_cols || !d_out_cols)
    return set_error(ctx, GBJ_ERR_INVALID, "hash_rearrange: need 1..16 columns and a key column among them");
  if (num_buckets < 1 || num_buckets > (1u << kMaxPartBits))
    return set_error(ctx, GBJ_ERR_INVALID, "hash_rearrange: num_buckets must be 1..32768");
  if (!d_bucket_offsets) return set_error(ctx, GBJ_ERR_INVALID, "hash_rearrange: null offsets");
  if (n >= (1ull << 31)) return set_error(ctx, GBJ_ERR_INVALID, "hash_rearrange: n >= 2^31");
  for (int j = 0; j < n_cols; ++j)
    if (n && (!d_cols[j] || !d_out_cols[j])) return set_error(ctx, GBJ_ERR_INVALID, "hash_rearrange: null column");
  cudaStream_t s = pick_stream(ctx, stream);
  prof_mark(ctx, s);
  if (n == 0) {
    GBJ_CHECK_CUDA(ctx, cudaMemsetAsync(d_bucket_offsets, 0, sizeof(uint64_t) * (num_buckets + 1), s));
    return GBJ_OK;
  }
  const int bits = std::max(1, log2_ceil(num_buckets));
  Scratch scratch(ctx, s);
  int32_t *ids;
  int2 *pairs;
  uint64_t *off;
  GBJ_TRY(scratch.get(n, &ids));
  GBJ_TRY(scratch.get(n, &pairs));
  GBJ_TRY(scratch.get((1ull << bits) + 1, &off));
  const unsigned grid = (unsigned)std::min<uint64_t>((n + 255) / 256, (uint64_t)ctx->sm_count * 16);
  k_bucket_ids<<<grid, 256, 0, s>>>(d_cols[key_col], n, num_buckets, ids);
  GBJ_TRY(after_launch(ctx, "k_bucket_ids", s));
  // (bucket, row) pairs, bucket-major; buckets >= num_buckets stay empty
  GBJ_TRY(partition_tuples(ctx, ids, nullptr, n, GBJ_DIGIT_KEY, 0, bits, pairs, nullptr, nullptr, off, s));
  GBJ_CHECK_CUDA(ctx, cudaMemcpyAsync(d_bucket_offsets, off, sizeof(uint64_t) * (num_buckets + 1),
                                      cudaMemcpyDeviceToDevice, s));
  Cols c{};
  c.n = n_cols;
  for (int j = 0; j < n_cols; ++j) {
    c.in[j] = d_cols[j];
    c.out[j] = d_out_cols[j];
  }
  k_gather_cols<<<grid, 256, 0, s>>>(pairs, n, c);
  return after_launch(ctx, "k_gather_cols", s);
}
