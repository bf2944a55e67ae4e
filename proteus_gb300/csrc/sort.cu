// Sort rows by an int32 key (ORDER BY), e.g. a group-by's output.
//
// Stands in for the reference's GPU sort (core/olap/lib/operators/gpu/
// gpu-sort.cpp; core/platform/lib/util/sort/gpu/sort-util.cu:191-218 calls
// thrust::sort on packed tuples).  Here: a stable LSD radix sort of
// (order-preserving key, row id) pairs, four 8-bit passes, then one gather
// of every column in the sorted order -- ties keep their input order, so
// the result is deterministic.
//
// Each pass: a histogram per 2048-row tile (stored digit-major), one scan
// over the (digit, tile) counts, and a stable scatter in which a warp ranks
// its 32 consecutive rows among equal digits (the lanes with the same digit
// found with one ballot per digit bit -- __match_any_sync costs far more on
// this part) and the warps of a tile combine their counts in shared memory.
#include <algorithm>

#include "gbj_internal.cuh"
#include "scan.cuh"

using namespace gbj;

namespace {

constexpr int kSortTile = 2048;
constexpr int kSortThreads = 512;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kMaxCols = GBJ_SORT_MAX_COLS;

__global__ void __launch_bounds__(256)
    k_sort_init(const int32_t *__restrict__ keys, uint64_t n, uint32_t flip_mask, uint2 *__restrict__ out) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride)
    out[i] = make_uint2(((uint32_t)keys[i] ^ 0x80000000u) ^ flip_mask, (uint32_t)i);
}

__global__ void __launch_bounds__(256)
    k_sort_hist(const uint2 *__restrict__ in, uint64_t n, int shift, uint64_t ntiles, uint32_t *__restrict__ counts) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const uint64_t base = (uint64_t)blockIdx.x * kSortTile;
  for (int j = threadIdx.x; j < kSortTile; j += blockDim.x) {
    const uint64_t i = base + j;
    if (i < n) atomicAdd(&h[(in[i].x >> shift) & 0xffu], 1u);
  }
  __syncthreads();
  counts[(uint64_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];  // digit-major
}

__global__ void __launch_bounds__(kSortThreads)
    k_sort_scatter(const uint2 *__restrict__ in, uint64_t n, int shift, uint64_t ntiles,
                   const uint64_t *__restrict__ offsets, uint2 *__restrict__ out) {
  __shared__ uint32_t wcnt[kSortWarps][256];  // per warp: count, then exclusive prefix over warps
  __shared__ uint32_t ctot[256];              // per digit: rows of this chunk
  __shared__ uint64_t run[256];               // per digit: next output position of this tile
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  if (threadIdx.x < 256) run[threadIdx.x] = offsets[(uint64_t)threadIdx.x * ntiles + blockIdx.x];
  const uint64_t base = (uint64_t)blockIdx.x * kSortTile;
  for (int c0 = 0; c0 < kSortTile; c0 += kSortThreads) {  // chunks in row order: stable
    for (int d = lane; d < 256; d += 32) wcnt[warp][d] = 0;
    __syncthreads();
    const uint64_t i = base + c0 + threadIdx.x;
    const bool ok = i < n;
    const uint2 e = ok ? in[i] : make_uint2(0, 0);
    const uint32_t d = ok ? (e.x >> shift) & 0xffu : 256u;  // 256: no row
    // lanes with the same 9-bit value d (256 = no row): one ballot per bit
    unsigned peers = 0xffffffffu;
#pragma unroll
    for (int bit = 0; bit < 9; ++bit) {
      const bool set = (d >> bit) & 1u;
      const unsigned bal = __ballot_sync(0xffffffffu, set);
      peers &= set ? bal : ~bal;
    }
    const uint32_t rank = __popc(peers & lt);  // equal digits before this lane
    if (ok && rank == 0) wcnt[warp][d] = __popc(peers);
    __syncthreads();
    if (threadIdx.x < 256) {
      uint32_t acc = 0;
#pragma unroll
      for (int w = 0; w < kSortWarps; ++w) {
        const uint32_t c = wcnt[w][threadIdx.x];
        wcnt[w][threadIdx.x] = acc;
        acc += c;
      }
      ctot[threadIdx.x] = acc;
    }
    __syncthreads();
    if (ok) out[run[d] + wcnt[warp][d] + rank] = e;
    __syncthreads();
    if (threadIdx.x < 256) run[threadIdx.x] += ctot[threadIdx.x];
  }
}

struct Cols {
  const int32_t *in[kMaxCols];
  int32_t *out[kMaxCols];
  int32_t n;
};

__global__ void __launch_bounds__(256) k_sort_gather(const uint2 *__restrict__ sorted, uint64_t n, Cols c) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    const uint32_t r = sorted[i].y;
#pragma unroll 4
    for (int j = 0; j < c.n; ++j) c.out[j][i] = __ldg(c.in[j] + r);
  }
}

}  // namespace

extern "C" int gbj_sort_by_key(gbj_ctx *ctx, const int32_t *const *d_cols, int32_t n_cols, uint64_t n,
                               int32_t key_col, int32_t descending, int32_t *const *d_out_cols, void *stream) {
  if (!ctx) return GBJ_ERR_INVALID;
  if (n_cols < 1 || n_cols > kMaxCols || key_col < 0 || key_col >= n_cols || !d_cols || !d_out_cols)
    return set_error(ctx, GBJ_ERR_INVALID, "sort: need 1..16 columns and a key column among them");
  if (n >= (1ull << 31)) return set_error(ctx, GBJ_ERR_INVALID, "sort: n >= 2^31");
  for (int j = 0; j < n_cols; ++j)
    if (n && (!d_cols[j] || !d_out_cols[j])) return set_error(ctx, GBJ_ERR_INVALID, "sort: null column");
  cudaStream_t s = pick_stream(ctx, stream);
  prof_mark(ctx, s);
  if (n == 0) return GBJ_OK;
  const uint64_t ntiles = (n + kSortTile - 1) / kSortTile;
  Scratch scratch(ctx, s);
  uint2 *a, *b;
  uint32_t *counts;
  uint64_t *offs;
  GBJ_TRY(scratch.get(n, &a));
  GBJ_TRY(scratch.get(n, &b));
  GBJ_TRY(scratch.get(256 * ntiles, &counts));
  GBJ_TRY(scratch.get(256 * ntiles + 1, &offs));
  const unsigned grid = (unsigned)std::min<uint64_t>((n + 255) / 256, (uint64_t)ctx->sm_count * 16);
  k_sort_init<<<grid, 256, 0, s>>>(d_cols[key_col], n, descending ? 0xffffffffu : 0u, a);
  GBJ_TRY(after_launch(ctx, "k_sort_init", s));
  for (int pass = 0; pass < 4; ++pass) {
    const int shift = 8 * pass;
    k_sort_hist<<<(unsigned)ntiles, 256, 0, s>>>(a, n, shift, ntiles, counts);
    GBJ_TRY(after_launch(ctx, "k_sort_hist", s));
    GBJ_TRY(scan_u32_to_u64(ctx, counts, offs, 256 * ntiles, s));
    k_sort_scatter<<<(unsigned)ntiles, kSortThreads, 0, s>>>(a, n, shift, ntiles, offs, b);
    GBJ_TRY(after_launch(ctx, "k_sort_scatter", s));
    std::swap(a, b);
  }
  Cols c{};
  c.n = n_cols;
  for (int j = 0; j < n_cols; ++j) {
    c.in[j] = d_cols[j];
    c.out[j] = d_out_cols[j];
  }
  k_sort_gather<<<grid, 256, 0, s>>>(a, n, c);
  return after_launch(ctx, "k_sort_gather", s);
}
