// Hash group-by with COUNT / SUM(int64) / MIN / MAX of one int32 value.
//
// Stands in for GpuHashGroupByChained (core/olap/lib/operators/gpu/
// gpu-hash-group-by-chained.cpp:77-556): the reference inserts every row
// into one global chained table with CAS on the chain heads and monoid
// atomics (gmonoids.cpp:122-360), then a scan pipeline emits entries whose
// next != self (hash-group-by-chained.cpp:638-853).
//
// GB300 design, two levels:
//  * level 1 -- a per-CTA open-addressing table in shared memory (4096
//    slots, SoA: key / count / sum / min / max) absorbs rows; for small
//    key domains a warp first merges equal keys with __match_any_sync and
//    redux.sync so one lane updates the table per distinct key;
//  * level 2 -- a global open-addressing table receives the level-1
//    contents at the end of each work item (and rows that find level 1
//    full), with integer atomics, so the result is exact in any order.
// High-cardinality inputs are first radix-partitioned on fmix32 bits so a
// partition's groups fit level 1; a work item that covers a whole
// partition then writes its groups straight to the output and never
// touches level 2.
//
// Stored forms (all-zero = empty / identity, so one memset initialises):
//   key' = key ^ 0x80000000 (0 is the empty slot; rows whose key is
//          INT32_MIN go to a dedicated accumulator instead),
//   max' = value ^ 0x80000000 and min' = ~(value ^ 0x80000000), both
//          combined with unsigned atomicMax.
#include <algorithm>

#include "gbj_internal.cuh"
#include "radix.cuh"
#include "scan.cuh"

using namespace gbj;

namespace {

constexpr int kThreads = 512;
constexpr int kSlots = 4096;  // level-1 slots per CTA
constexpr int kProbeL1 = 32;  // level-1 probe limit before spilling to L2
constexpr uint32_t kFlip = 0x80000000u;

struct GTable {
  uint32_t *key;  // key' (0 = empty)
  unsigned long long *cnt;
  unsigned long long *sum;
  uint32_t *mn;  // min'
  uint32_t *mx;  // max'
  uint64_t mask;
  // dedicated INT32_MIN group at index mask + 1 of cnt/sum/mn/mx
};

__device__ __forceinline__ uint32_t enc_max(int32_t v) { return (uint32_t)v ^ kFlip; }
__device__ __forceinline__ uint32_t enc_min(int32_t v) { return ~((uint32_t)v ^ kFlip); }
__device__ __forceinline__ int32_t dec_max(uint32_t u) { return (int32_t)(u ^ kFlip); }
__device__ __forceinline__ int32_t dec_min(uint32_t u) { return (int32_t)(~u ^ kFlip); }

// Finds or claims the global slot of `key` (key != INT32_MIN).
__device__ __forceinline__ int64_t g_slot(const GTable &g, int32_t key, uint32_t *status) {
  const uint32_t kk = (uint32_t)key ^ kFlip;
  uint64_t h = gbjd::fmix32((uint32_t)key) & g.mask;
  for (uint64_t step = 0; step <= g.mask; ++step) {
    uint32_t cur = *(volatile uint32_t *)&g.key[h];
    if (cur == kk) return (int64_t)h;
    if (cur == 0) {
      cur = atomicCAS(&g.key[h], 0u, kk);
      if (cur == 0 || cur == kk) return (int64_t)h;
    }
    h = (h + 1) & g.mask;
  }
  gbjd::latch(status, GBJ_DEV_CAPACITY);
  return -1;
}

__device__ __forceinline__ void g_update(const GTable &g, int64_t slot, uint32_t c,
                                         int64_t s, uint32_t mn_enc, uint32_t mx_enc) {
  if (slot < 0) return;
  atomicAdd(&g.cnt[slot], (unsigned long long)c);
  atomicAdd(&g.sum[slot], (unsigned long long)s);
  atomicMax(&g.mn[slot], mn_enc);
  atomicMax(&g.mx[slot], mx_enc);
}

__device__ __forceinline__ void g_row(const GTable &g, int32_t key, uint32_t c, int64_t s,
                                      uint32_t mn_enc, uint32_t mx_enc, uint32_t *status) {
  const int64_t slot = key == INT32_MIN ? (int64_t)(g.mask + 1) : g_slot(g, key, status);
  g_update(g, slot, c, s, mn_enc, mx_enc);
}

struct L1 {
  uint32_t *key;
  uint32_t *cnt;
  unsigned long long *sum;
  uint32_t *mn, *mx;
};

struct Out {
  int32_t *keys;
  int64_t *cnt, *sum;
  int32_t *mn, *mx;
  uint64_t cap;
  unsigned long long *n;
};

__device__ __forceinline__ void emit(const Out &o, uint64_t pos, int32_t key, uint64_t c,
                                     int64_t s, int32_t mn, int32_t mx, uint32_t *status) {
  if (pos >= o.cap) {
    gbjd::latch(status, GBJ_DEV_CAPACITY);
    return;
  }
  if (o.keys) o.keys[pos] = key;
  if (o.cnt) o.cnt[pos] = (int64_t)c;
  if (o.sum) o.sum[pos] = s;
  if (o.mn) o.mn[pos] = mn;
  if (o.mx) o.mx[pos] = mx;
}

// Aggregation kernel.  Work item i covers rows [item_lo(i), item_hi(i)) of
// either the raw SoA input or the partitioned AoS pairs.  kMatch enables the
// warp-level merge of equal keys.
template <bool kMatch, bool kPairs>
__global__ void __launch_bounds__(kThreads)
    k_groupby(const int32_t *__restrict__ keys, const int32_t *__restrict__ vals,
              const int2 *__restrict__ pairs, uint64_t n,
              // raw mode: items of w rows; partitioned mode: item_off over P
              uint64_t w, const uint64_t *__restrict__ poff,
              const uint64_t *__restrict__ item_off, uint32_t P, GTable g, Out o,
              unsigned long long *item_ctr, uint32_t *status) {
  extern __shared__ __align__(16) unsigned char smem[];
  L1 t;
  t.sum = reinterpret_cast<unsigned long long *>(smem);
  t.key = reinterpret_cast<uint32_t *>(t.sum + kSlots);
  t.cnt = t.key + kSlots;
  t.mn = t.cnt + kSlots;
  t.mx = t.mn + kSlots;
  __shared__ unsigned long long s_item;
  __shared__ int s_spill;
  __shared__ uint32_t s_warp[kThreads / 32];
  __shared__ unsigned long long s_base;
  const uint64_t total_items = kPairs ? item_off[P] : (n + w - 1) / w;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

  for (;;) {
    if (threadIdx.x == 0) {
      s_item = atomicAdd(item_ctr, 1ull);
      s_spill = 0;
    }
    for (int i = threadIdx.x; i < kSlots; i += kThreads) {
      t.key[i] = 0;
      t.cnt[i] = 0;
      t.sum[i] = 0;
      t.mn[i] = 0;
      t.mx[i] = 0;
    }
    __syncthreads();
    const uint64_t item = s_item;
    if (item >= total_items) break;
    uint64_t lo, hi;
    bool whole = false;
    if (kPairs) {
      uint32_t a = 0, b = P;
      while (b - a > 1) {
        const uint32_t mid = (a + b) >> 1;
        if (item_off[mid] <= item) a = mid; else b = mid;
      }
      const uint64_t p0 = poff[a], p1 = poff[a + 1];
      lo = p0 + (item - item_off[a]) * w;
      hi = lo + w < p1 ? lo + w : p1;
      whole = (p1 - p0) <= w;
    } else {
      lo = item * w;
      hi = lo + w < n ? lo + w : n;
    }
    // rows of this item; whole warps iterate together for __match_any_sync
    for (uint64_t base = lo; base < hi; base += kThreads) {
      const uint64_t i = base + threadIdx.x;
      const bool valid = i < hi;
      int32_t k = 0, v = 0;
      if (valid) {
        if (kPairs) {
          const int2 pv = __ldcs(pairs + i);
          k = pv.x;
          v = pv.y;
        } else {
          k = __ldcs(keys + i);
          v = __ldcs(vals + i);
        }
      }
      uint32_t c = 1;
      int64_t s = v;
      uint32_t mn_e = enc_min(v), mx_e = enc_max(v);
      bool leader = valid;
      if (kMatch) {
        const unsigned act = __ballot_sync(0xffffffffu, valid);
        if (valid) {
          const unsigned peers = __match_any_sync(act, k);
          leader = (__ffs(peers) - 1) == lane;
          c = __popc(peers);
          // exact 32-lane sum of int32 values: 16-bit halves
          const int32_t shi = (int32_t)__reduce_add_sync(peers, (unsigned)(v >> 16));
          const uint32_t slo = __reduce_add_sync(peers, (unsigned)v & 0xffffu);
          s = (int64_t)shi * 65536 + (int64_t)slo;
          mn_e = enc_min(__reduce_min_sync(peers, v));
          mx_e = enc_max(__reduce_max_sync(peers, v));
        }
      }
      if (leader) {
        if (k == INT32_MIN) {
          g_row(g, k, c, s, mn_e, mx_e, status);
          s_spill = 1;
        } else {
          const uint32_t kk = (uint32_t)k ^ kFlip;
          uint32_t h = gbjd::fmix32((uint32_t)k) & (kSlots - 1);
          int slot = -1;
          for (int step = 0; step < kProbeL1; ++step) {
            uint32_t cur = t.key[h];
            if (cur == 0) cur = atomicCAS(&t.key[h], 0u, kk);
            if (cur == 0 || cur == kk) {
              slot = (int)h;
              break;
            }
            h = (h + 1) & (kSlots - 1);
          }
          if (slot >= 0) {
            atomicAdd(&t.cnt[slot], c);
            atomicAdd(&t.sum[slot], (unsigned long long)s);
            atomicMax(&t.mn[slot], mn_e);
            atomicMax(&t.mx[slot], mx_e);
          } else {
            g_row(g, k, c, s, mn_e, mx_e, status);
            s_spill = 1;
          }
        }
      }
    }
    __syncthreads();
    if (kPairs && whole && !s_spill) {
      // final groups of a whole partition: compact straight to the output
      uint32_t mine = 0;
      for (int i = threadIdx.x; i < kSlots; i += kThreads) mine += t.key[i] != 0;
      mine = __reduce_add_sync(0xffffffffu, mine);
      if (lane == 0) s_warp[warp] = mine;
      __syncthreads();
      if (threadIdx.x == 0) {
        uint32_t tot = 0;
        for (int w2 = 0; w2 < kThreads / 32; ++w2) tot += s_warp[w2];
        s_base = tot ? atomicAdd(o.n, (unsigned long long)tot) : 0;
      }
      __syncthreads();
      // ordered write positions: slot ranges per warp, ballot inside
      uint64_t pos = s_base;
      for (int w2 = 0; w2 < warp; ++w2) pos += s_warp[w2];
      for (int i0 = warp * 32; i0 < kSlots; i0 += kThreads) {
        const int i = i0 + lane;
        const bool occ = t.key[i] != 0;
        const unsigned b = __ballot_sync(0xffffffffu, occ);
        if (occ)
          emit(o, pos + __popc(b & ((1u << lane) - 1)), (int32_t)(t.key[i] ^ kFlip), t.cnt[i],
               (int64_t)t.sum[i], dec_min(t.mn[i]), dec_max(t.mx[i]), status);
        pos += __popc(b);
      }
    } else {
      for (int i = threadIdx.x; i < kSlots; i += kThreads) {
        if (t.key[i] != 0) {
          const int32_t k = (int32_t)(t.key[i] ^ kFlip);
          g_update(g, g_slot(g, k, status), t.cnt[i], (int64_t)t.sum[i], t.mn[i], t.mx[i]);
        }
      }
    }
    __syncthreads();
  }
}

// Emits every occupied level-2 slot (and the INT32_MIN group).  The loop
// trip count is uniform per warp so the output reservation is one
// full-warp ballot + one atomic per warp.
__global__ void k_groupby_emit(GTable g, Out o, uint32_t *status) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t cap = g.mask + 1;
  const int lane = threadIdx.x & 31;
  for (uint64_t b0 = blockIdx.x * (uint64_t)blockDim.x; b0 <= cap; b0 += stride) {
    const uint64_t i = b0 + threadIdx.x;
    bool occ = false;
    int32_t key = INT32_MIN;
    if (i < cap) {
      occ = g.key[i] != 0;
      key = (int32_t)(g.key[i] ^ kFlip);
    } else if (i == cap) {
      occ = g.cnt[i] != 0;
    }
    const unsigned b = __ballot_sync(0xffffffffu, occ);
    unsigned long long base = 0;
    if (lane == 0 && b) base = atomicAdd(o.n, (unsigned long long)__popc(b));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (occ)
      emit(o, base + __popc(b & ((1u << lane) - 1)), key, g.cnt[i], (int64_t)g.sum[i],
           dec_min(g.mn[i]), dec_max(g.mx[i]), status);
  }
}

__global__ void k_groupby_items(const uint64_t *__restrict__ poff, uint32_t P, uint64_t w,
                                uint64_t *__restrict__ items) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  const uint64_t m = poff[p + 1] - poff[p];
  items[p] = (m + w - 1) / w;
}

__global__ void k_copy_count(const unsigned long long *src, uint64_t *dst) { *dst = *src; }

}  // namespace

extern "C" int gbj_groupby(gbj_ctx *ctx, const int32_t *d_keys, const int32_t *d_values,
                           uint64_t n, const gbj_groupby_params *params, int32_t *d_out_keys,
                           int64_t *d_out_count, int64_t *d_out_sum, int32_t *d_out_min,
                           int32_t *d_out_max, uint64_t out_capacity, uint64_t *d_n_groups,
                           void *stream) {
  if (!ctx || !d_n_groups) return GBJ_ERR_INVALID;
  if (n && (!d_keys || !d_values)) return set_error(ctx, GBJ_ERR_INVALID, "groupby: null column");
  if (n >= (1ULL << 31)) return set_error(ctx, GBJ_ERR_INVALID, "groupby: n >= 2^31");
  cudaStream_t s = pick_stream(ctx, stream);
  prof_mark(ctx, s);
  GBJ_CHECK_CUDA(ctx, cudaMemsetAsync(d_n_groups, 0, sizeof(uint64_t), s));
  if (n == 0) return GBJ_OK;

  // ---- plan ----
  uint64_t hint = 0;
  int strategy = 0;
  if (params) {
    hint = params->expected_groups ? params->expected_groups : params->max_input_size;
    strategy = params->strategy;
  }
  if (strategy < 0 || strategy > 2) return set_error(ctx, GBJ_ERR_INVALID, "groupby: bad strategy");
  const uint64_t groups_cap = std::max<uint64_t>(1024, hint ? std::min<uint64_t>(hint, n) : std::min<uint64_t>(n, 1ull << 24));
  if (strategy == 0) strategy = (hint && hint <= kSlots / 2) ? 1 : (hint ? 2 : 1);
  const bool match = hint && hint <= 256;

  Scratch scratch(ctx, s);
  // level-2 table: cap slots + 1 dedicated INT32_MIN group
  const uint64_t cap = next_pow2(2 * groups_cap);
  GTable g;
  char *gmem;
  const uint64_t gbytes = (cap + 1) * (4 + 8 + 8 + 4 + 4) + 64;
  GBJ_TRY(scratch.get(gbytes, &gmem));
  GBJ_CHECK_CUDA(ctx, cudaMemsetAsync(gmem, 0, gbytes, s));
  g.cnt = reinterpret_cast<unsigned long long *>(gmem);
  g.sum = g.cnt + (cap + 1);
  g.key = reinterpret_cast<uint32_t *>(g.sum + (cap + 1));
  g.mn = g.key + (cap + 1);
  g.mx = g.mn + (cap + 1);
  g.mask = cap - 1;
  Out o{d_out_keys, d_out_count, d_out_sum, d_out_min, d_out_max, out_capacity,
        reinterpret_cast<unsigned long long *>(d_n_groups)};
  unsigned long long *ctr;
  GBJ_TRY(scratch.get(1, &ctr));
  GBJ_CHECK_CUDA(ctx, cudaMemsetAsync(ctr, 0, sizeof(unsigned long long), s));

  const size_t smem = (size_t)kSlots * (8 + 4 + 4 + 4 + 4);
  auto launch = [&](auto kern, const int2 *pairs, uint64_t w, const uint64_t *poff,
                    const uint64_t *items, uint32_t P) -> int {
    GBJ_CHECK_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 1;
    GBJ_CHECK_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem));
    per_sm = std::max(per_sm, 1);
    kern<<<ctx->sm_count * per_sm, kThreads, smem, s>>>(d_keys, d_values, pairs, n, w, poff, items,
                                                        P, g, o, ctr, ctx->d_status);
    return after_launch(ctx, "k_groupby", s);
  };

  if (strategy == 1) {
    // raw input in items of w rows (enough to amortise the level-1 flush)
    const uint64_t w = std::max<uint64_t>(1u << 16, (n + ctx->sm_count * 4 - 1) / (ctx->sm_count * 4));
    if (match)
      GBJ_TRY(launch(k_groupby<true, false>, nullptr, w, nullptr, nullptr, 0));
    else
      GBJ_TRY(launch(k_groupby<false, false>, nullptr, w, nullptr, nullptr, 0));
  } else {
    // partition so each partition holds ~kSlots/4 groups
    int bits = 1;
    while (bits < kMaxPartBits && (groups_cap >> bits) > (uint64_t)kSlots / 4) ++bits;
    if (params && params->hash_bits > 0 && strategy == 2 && !hint) bits = std::min(params->hash_bits, kMaxPartBits);
    const uint32_t P = 1u << bits;
    int2 *pairs;
    uint64_t *poff, *items;
    GBJ_TRY(scratch.get(n, &pairs));
    GBJ_TRY(scratch.get(P + 1, &poff));
    GBJ_TRY(scratch.get(P + 1, &items));
    GBJ_TRY(partition_tuples(ctx, d_keys, d_values, n, GBJ_DIGIT_HASH, 0, bits, pairs, nullptr,
                             nullptr, poff, s));
    const uint64_t w = 1u << 17;
    k_groupby_items<<<(P + 255) / 256, 256, 0, s>>>(poff, P, w, items);
    GBJ_TRY(after_launch(ctx, "k_groupby_items", s));
    GBJ_TRY(scan_u64(ctx, items, items, P, s));
    GBJ_TRY(launch(k_groupby<false, true>, pairs, w, poff, items, P));
  }
  const uint64_t emit_threads = 256;
  const uint64_t emit_blocks = std::min<uint64_t>((cap + emit_threads) / emit_threads, (uint64_t)ctx->sm_count * 8);
  k_groupby_emit<<<(unsigned)emit_blocks, emit_threads, 0, s>>>(g, o, ctx->d_status);
  return after_launch(ctx, "k_groupby_emit", s);
}
