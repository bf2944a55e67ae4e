// Bloom-filter semi-join pre-filter.
//
// Stands in for BloomFilterBuild / BloomFilterProbe (core/olap/lib/
// operators/bloom-filter/bloom-filter-build.cpp:28-59,
// bloom-filter-probe.cpp:28-53, position function bloom-filter.cpp:65-95):
// a filter of filterSize (a power of two) flags, the flag of a key at
// position key & (filterSize - 1) (the reference indexes the filter with the
// key itself, not a hash); the build side sets the flags of its keys, the
// probe side keeps the rows whose flag is set.  The reference stores one
// byte-sized flag per position; here the flags are bits (filterSize / 8
// bytes, e.g. 2 MiB for 2^24 positions: L2-resident), set with atomicOr and
// tested with one 32-bit load per probe row.  Which rows pass is exactly the
// reference's.
#include "compact.cuh"
#include "gbj_internal.cuh"

using namespace gbj;

struct gbj_bloom {
  uint32_t *bits = nullptr;  // pool block
  uint64_t size = 0;         // positions (power of two)
};

namespace {

__global__ void __launch_bounds__(256)
    k_bloom_build(const int32_t *__restrict__ keys, uint64_t n, uint32_t mask, uint32_t *__restrict__ bits) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    const uint32_t p = (uint32_t)__ldcs(keys + i) & mask;
    atomicOr(&bits[p >> 5], 1u << (p & 31));
  }
}

struct BloomPred {
  const int32_t *keys;
  const uint32_t *bits;
  uint32_t mask;
  __device__ __forceinline__ bool operator()(uint64_t i) const {
    const uint32_t p = (uint32_t)keys[i] & mask;
    return (__ldg(bits + (p >> 5)) >> (p & 31)) & 1u;
  }
};

}  // namespace

extern "C" int gbj_bloom_build(gbj_ctx *ctx, const int32_t *d_keys, uint64_t n, uint64_t filter_size,
                               void *stream, gbj_bloom **out) {
  if (!ctx || !out) return GBJ_ERR_INVALID;
  *out = nullptr;
  if (filter_size < 32 || filter_size > (1ull << 31) || (filter_size & (filter_size - 1)))
    return set_error(ctx, GBJ_ERR_INVALID, "bloom: filter_size must be a power of two in [32, 2^31]");
  if (n && !d_keys) return set_error(ctx, GBJ_ERR_INVALID, "bloom: null keys");
  cudaStream_t s = pick_stream(ctx, stream);
  prof_mark(ctx, s);
  auto f = new gbj_bloom();
  f->size = filter_size;
  const int rc = pool_alloc(ctx, filter_size / 8, s, reinterpret_cast<void **>(&f->bits));
  if (rc) {
    delete f;
    return rc;
  }
  GBJ_CHECK_CUDA(ctx, cudaMemsetAsync(f->bits, 0, filter_size / 8, s));
  if (n) {
    const unsigned grid = (unsigned)std::min<uint64_t>((n + 255) / 256, (uint64_t)ctx->sm_count * 16);
    k_bloom_build<<<grid, 256, 0, s>>>(d_keys, n, (uint32_t)(filter_size - 1), f->bits);
    const int r = after_launch(ctx, "k_bloom_build", s);
    if (r) {
      pool_release(ctx, f->bits, s);
      delete f;
      return r;
    }
  }
  *out = f;
  return GBJ_OK;
}

extern "C" int gbj_bloom_probe(gbj_ctx *ctx, const gbj_bloom *filter, const int32_t *d_keys, uint64_t n,
                               int32_t *d_rows_out, uint64_t *d_count, void *stream) {
  if (!ctx || !filter || !d_count || (n && (!d_keys || !d_rows_out))) return GBJ_ERR_INVALID;
  if (n >= (1ull << 31)) return set_error(ctx, GBJ_ERR_INVALID, "bloom: n >= 2^31");
  cudaStream_t s = pick_stream(ctx, stream);
  prof_mark(ctx, s);
  return compact_rows(ctx, BloomPred{d_keys, filter->bits, (uint32_t)(filter->size - 1)}, n, d_rows_out,
                      d_count, s);
}

extern "C" int gbj_bloom_destroy(gbj_ctx *ctx, gbj_bloom *filter) {
  if (!ctx || !filter) return GBJ_ERR_INVALID;
  pool_release(ctx, filter->bits, ctx->stream);
  delete filter;
  return GBJ_OK;
}
