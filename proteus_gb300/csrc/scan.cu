// Multi-level exclusive scan: each 1024-thread block scans a tile of
// kTile = 4096 values (4 per thread) and writes its total; the totals are
// scanned recursively and added back.
#include "scan.cuh"

namespace gbj {
namespace {

constexpr int kThreads = 1024;
constexpr int kPer = 4;
constexpr uint64_t kTile = kThreads * kPer;

template <typename In>
__global__ void __launch_bounds__(kThreads)
    k_scan_tiles(const In *in, uint64_t *out, uint64_t n, uint64_t *tile_sums) {
  __shared__ uint64_t warp_tot[32];
  const uint64_t base = blockIdx.x * kTile + (uint64_t)threadIdx.x * kPer;
  uint64_t v[kPer];
  uint64_t local = 0;
#pragma unroll
  for (int j = 0; j < kPer; ++j) {
    v[j] = (base + j < n) ? (uint64_t)in[base + j] : 0;
    local += v[j];
  }
  // inclusive warp scan of thread totals
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint64_t x = local;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint64_t t = warp_tot[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint64_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    warp_tot[lane] = t;  // inclusive
  }
  __syncthreads();
  uint64_t excl = x - local + (warp ? warp_tot[warp - 1] : 0);
#pragma unroll
  for (int j = 0; j < kPer; ++j) {
    if (base + j < n) out[base + j] = excl;
    excl += v[j];
  }
  if (threadIdx.x == kThreads - 1) tile_sums[blockIdx.x] = excl;
}

__global__ void k_scan_add(uint64_t *out, uint64_t n, const uint64_t *tile_off) {
  const uint64_t i = blockIdx.x * kTile + threadIdx.x;
  const uint64_t add = tile_off[blockIdx.x];
#pragma unroll
  for (int j = 0; j < kPer; ++j) {
    uint64_t k = i + (uint64_t)j * kThreads;
    if (k < n) out[k] += add;
  }
}

__global__ void k_set_total(uint64_t *out, uint64_t n, const uint64_t *tile_off,
                            uint64_t ntiles) {
  out[n] = tile_off[ntiles];
}

template <typename In>
int scan_impl(gbj_ctx *ctx, const In *in, uint64_t *out, uint64_t n,
              cudaStream_t s) {
  if (n == 0) {
    GBJ_CHECK_CUDA(ctx, cudaMemsetAsync(out, 0, sizeof(uint64_t), s));
    return GBJ_OK;
  }
  const uint64_t ntiles = (n + kTile - 1) / kTile;
  Scratch scratch(ctx, s);
  uint64_t *sums;
  GBJ_TRY(scratch.get(ntiles + 1, &sums));
  k_scan_tiles<In><<<(unsigned)ntiles, kThreads, 0, s>>>(in, out, n, sums);
  GBJ_TRY(after_launch(ctx, "k_scan_tiles", s));
  if (ntiles == 1) {
    // single tile: its total is the grand total
    k_set_total<<<1, 1, 0, s>>>(out, n, sums, 0);
    return after_launch(ctx, "k_set_total", s);
  }
  // sums[0..ntiles) -> exclusive offsets in place, sums[ntiles] = total
  GBJ_TRY(scan_impl<uint64_t>(ctx, sums, sums, ntiles, s));
  k_scan_add<<<(unsigned)ntiles, kThreads, 0, s>>>(out, n, sums);
  GBJ_TRY(after_launch(ctx, "k_scan_add", s));
  k_set_total<<<1, 1, 0, s>>>(out, n, sums, ntiles);
  return after_launch(ctx, "k_set_total", s);
}

}  // namespace

int scan_u64(gbj_ctx *ctx, const uint64_t *in, uint64_t *out, uint64_t n,
             cudaStream_t s) {
  return scan_impl<uint64_t>(ctx, in, out, n, s);
}

int scan_u32_to_u64(gbj_ctx *ctx, const uint32_t *in, uint64_t *out,
                    uint64_t n, cudaStream_t s) {
  return scan_impl<uint32_t>(ctx, in, out, n, s);
}

}  // namespace gbj
