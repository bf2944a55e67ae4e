// Ordered row compaction shared by the range select and the bloom-filter
// probe: the positions of rows that pass a predicate, ascending.  Tiles of
// kSelTile rows count their passing rows, a scan gives each tile its output
// offset, and a second pass writes the row ids in order (stable).
#pragma once
#include "gbj_internal.cuh"
#include "scan.cuh"

namespace gbj {

constexpr int kSelTile = 4096;  // rows per compaction tile (one block)

template <typename Pred>
__global__ void __launch_bounds__(1024) k_compact_count(Pred pred, uint64_t n, uint64_t *tile_counts) {
  __shared__ uint32_t c;
  if (threadIdx.x == 0) c = 0;
  __syncthreads();
  uint32_t mine = 0;
  const uint64_t base = (uint64_t)blockIdx.x * kSelTile;
  for (int j = threadIdx.x; j < kSelTile; j += blockDim.x) {
    const uint64_t i = base + j;
    if (i < n) mine += pred(i) ? 1u : 0u;
  }
  mine = __reduce_add_sync(0xffffffffu, mine);
  if ((threadIdx.x & 31) == 0) atomicAdd(&c, mine);
  __syncthreads();
  if (threadIdx.x == 0) tile_counts[blockIdx.x] = c;
}

template <typename Pred>
__global__ void __launch_bounds__(1024)
    k_compact_write(Pred pred, uint64_t n, const uint64_t *tile_off, int32_t *out) {
  __shared__ uint32_t warp_cnt[32];
  __shared__ uint64_t run;
  if (threadIdx.x == 0) run = tile_off[blockIdx.x];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint64_t base = (uint64_t)blockIdx.x * kSelTile;
  for (int j0 = 0; j0 < kSelTile; j0 += blockDim.x) {
    __syncthreads();
    const uint64_t i = base + j0 + threadIdx.x;
    const bool pass = i < n && pred(i);
    const uint32_t b = __ballot_sync(0xffffffffu, pass);
    if (lane == 0) warp_cnt[warp] = __popc(b);
    __syncthreads();
    uint64_t before = run;
    for (int w = 0; w < warp; ++w) before += warp_cnt[w];
    if (pass) out[before + __popc(b & ((1u << lane) - 1))] = (int32_t)i;
    __syncthreads();
    if (threadIdx.x == 0) {
      uint64_t t = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += warp_cnt[w];
      run += t;
    }
  }
}

__global__ void k_compact_total(const uint64_t *off, uint64_t ntiles, uint64_t *dst);

// Writes the passing row ids of [0, n) to d_rows_out (ascending) and their
// number to *d_count.  `name` labels the launches in the profile.
template <typename Pred>
int compact_rows(gbj_ctx *ctx, Pred pred, uint64_t n, int32_t *d_rows_out, uint64_t *d_count,
                 cudaStream_t s) {
  if (n == 0) {
    GBJ_CHECK_CUDA(ctx, cudaMemsetAsync(d_count, 0, sizeof(uint64_t), s));
    return GBJ_OK;
  }
  const uint64_t ntiles = (n + kSelTile - 1) / kSelTile;
  Scratch scratch(ctx, s);
  uint64_t *cnt;
  GBJ_TRY(scratch.get(ntiles + 1, &cnt));
  k_compact_count<<<(unsigned)ntiles, 1024, 0, s>>>(pred, n, cnt);
  GBJ_TRY(after_launch(ctx, "k_compact_count", s));
  GBJ_TRY(scan_u64(ctx, cnt, cnt, ntiles, s));
  k_compact_write<<<(unsigned)ntiles, 1024, 0, s>>>(pred, n, cnt, d_rows_out);
  GBJ_TRY(after_launch(ctx, "k_compact_write", s));
  k_compact_total<<<1, 1, 0, s>>>(cnt, ntiles, d_count);
  return after_launch(ctx, "k_compact_total", s);
}

}  // namespace gbj
