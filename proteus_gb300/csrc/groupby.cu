// Hash group-by with COUNT / SUM(int64) / MIN / MAX of one int32 value.
//
// Stands in for GpuHashGroupByChained (core/olap/lib/operators/gpu/
// gpu-hash-group-by-chained.cpp:77-556): the reference inserts every row
// into one global chained table with CAS on the chain heads and monoid
// atomics (gmonoids.cpp:122-360), then a scan pipeline emits entries whose
// next != self (hash-group-by-chained.cpp:638-853).
//
// GB300 design:
//  * level 1 lives in shared memory: for at most 64 groups each warp keeps a
//    private 128-slot table where count and biased sum share one 64-bit
//    atomic per row (flushed to level 2 every 4096 rows of the warp, which
//    bounds the packed fields); otherwise one table of up to 4096 slots per
//    CTA with count and sum atomics.  Min and max atomics are issued only
//    when the value improves the stored extreme, so they fade out as a
//    group fills;
//  * level 2 is a global open-addressing table that receives level 1 when a
//    CTA finishes (and rows that find level 1 full), with integer atomics,
//    so the result is exact in any order;
//  * high-cardinality inputs are first radix-partitioned on fmix32 bits so a
//    partition's groups fit level 1; a work item that covers a whole
//    partition writes its groups straight to the output.
//
// Stored forms (all-zero = empty / identity, so one memset initialises):
//   key' = key ^ 0x80000000 (0 is the empty slot; rows whose key is
//          INT32_MIN go to a dedicated level-2 accumulator instead),
//   max' = value ^ 0x80000000 and min' = ~(value ^ 0x80000000), both
//          combined with unsigned max.
#include <algorithm>

#include "gbj_internal.cuh"
#include "radix.cuh"
#include "scan.cuh"

using namespace gbj;

namespace {

constexpr int kThreads = 512;
constexpr int kWarps = kThreads / 32;
constexpr int kSlots = 4096;     // CTA level-1 table slots
constexpr int kPrivSlots = 128;  // per-warp level-1 table slots (<= 64 groups)
constexpr int kProbeL1 = 32;     // level-1 probe limit before spilling to level 2
constexpr uint32_t kFlip = 0x80000000u;
constexpr uint64_t kPrivMaxGroups = 64;

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

__device__ __forceinline__ void g_update(const GTable &g, int64_t slot, uint64_t c,
                                         int64_t s, uint32_t mn_enc, uint32_t mx_enc) {
  if (slot < 0) return;
  atomicAdd(&g.cnt[slot], (unsigned long long)c);
  atomicAdd(&g.sum[slot], (unsigned long long)s);
  atomicMax(&g.mn[slot], mn_enc);
  atomicMax(&g.mx[slot], mx_enc);
}

__device__ __forceinline__ void g_row(const GTable &g, int32_t key, uint64_t c, int64_t s,
                                      uint32_t mn_enc, uint32_t mx_enc, uint32_t *status) {
  const int64_t slot = key == INT32_MIN ? (int64_t)(g.mask + 1) : g_slot(g, key, status);
  g_update(g, slot, c, s, mn_enc, mx_enc);
}

// A level-1 table (CTA-shared or one warp's private table).
struct L1 {
  uint32_t *key;
  uint32_t *cnt;
  unsigned long long *sum;
  uint32_t *mn, *mx;
  uint32_t mask;   // slots - 1
  uint32_t shift;  // 32 - log2(slots): the home slot is the hash's top bits
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

// Level-1 slot of key' kk (claimed with CAS when new), or -1 when the probe
// limit is reached.  The home slot comes from the top bits of the hash: the
// partitioning digit is its low bits, so within a partition those are equal.
__device__ __forceinline__ int l1_slot(const L1 &t, int32_t k, uint32_t kk) {
  uint32_t h = gbjd::fmix32((uint32_t)k) >> t.shift;
  for (int step = 0; step < kProbeL1; ++step) {
    uint32_t cur = t.key[h];
    if (cur == 0) cur = atomicCAS(&t.key[h], 0u, kk);
    if (cur == 0 || cur == kk) return (int)h;
    h = (h + 1) & t.mask;
  }
  return -1;
}

// Packed per-warp accumulator: count in bits [44, 64), sum of the biased
// values (v + 2^31, each < 2^32) in bits [0, 44).  Exact while a slot sees at
// most 4096 rows between flushes (4096 * 2^32 = 2^44), which the per-warp
// flush every kPrivFlushRows rows guarantees.
constexpr int kPackShift = 44;
constexpr uint32_t kPrivFlushRows = 4096;
constexpr int kMergeMin = 5;

// Applies c rows of key k (sum s, extremes mn/mx) to a level-1 table.
// kPrivate: the table belongs to this warp, count and biased sum travel in
// one packed 64-bit atomic (in `sum`).  Otherwise: count and sum atomics.
// Min and max use an atomic only when the value improves the stored extreme.
template <bool kPrivate>
__device__ __forceinline__ void l1_apply(const L1 &t, const GTable &g, int32_t k, uint32_t c,
                                         int64_t s, int32_t mn, int32_t mx, bool &spill,
                                         uint32_t *status) {
  const uint32_t emn = enc_min(mn), emx = enc_max(mx);
  if (k == INT32_MIN) {
    g_row(g, k, c, s, emn, emx, status);
    spill = true;
    return;
  }
  const uint32_t kk = (uint32_t)k ^ kFlip;
  const int slot = l1_slot(t, k, kk);
  if (slot < 0) {
    g_row(g, k, c, s, emn, emx, status);
    spill = true;
    return;
  }
  if (kPrivate) {
    atomicAdd(&t.sum[slot], ((unsigned long long)c << kPackShift) +
                                (unsigned long long)(s + (int64_t)c * (int64_t)kFlip));
  } else {
    atomicAdd(&t.cnt[slot], c);
    atomicAdd(&t.sum[slot], (unsigned long long)s);
  }
  if (emn > t.mn[slot]) atomicMax(&t.mn[slot], emn);
  if (emx > t.mx[slot]) atomicMax(&t.mx[slot], emx);
}

// One row per lane (ok = lane holds a row); called by the whole warp.  When
// at least kMergeMin lanes share the key of the first active lane they are
// merged first with warp reductions (the sum as signed high and unsigned low
// 16-bit halves, exact in 32 bits for 32 lanes), so a hot key costs one set
// of atomics per warp instead of one per row.  A second merge round runs
// only when the first merged (skewed input); other inputs pay two ballots.
// Below the threshold the duplicate atomics are cheaper than the merge.
template <bool kPrivate>
__device__ __forceinline__ void warp_rows(const L1 &t, const GTable &g, int32_t k, int32_t v,
                                          bool ok, bool &spill, uint32_t *status) {
  const int lane = threadIdx.x & 31;
  unsigned act = __ballot_sync(0xffffffffu, ok);
#pragma unroll
  for (int round = 0; round < 2; ++round) {
    if (!act) return;
    const int lead = __ffs(act) - 1;
    const int32_t k0 = __shfl_sync(0xffffffffu, k, lead);
    const bool same = ok && k == k0;
    const unsigned m = __ballot_sync(0xffffffffu, same);
    if (__popc(m) < kMergeMin) break;
    const uint32_t lo = __reduce_add_sync(0xffffffffu, same ? ((uint32_t)v & 0xffffu) : 0u);
    const int32_t hi = (int32_t)__reduce_add_sync(0xffffffffu, same ? (uint32_t)(v >> 16) : 0u);
    const int32_t mn = __reduce_min_sync(0xffffffffu, same ? v : INT32_MAX);
    const int32_t mx = __reduce_max_sync(0xffffffffu, same ? v : INT32_MIN);
    if (lane == lead)
      l1_apply<kPrivate>(t, g, k0, (uint32_t)__popc(m), (int64_t)hi * 65536 + (int64_t)lo, mn, mx,
                         spill, status);
    ok = ok && !same;
    act &= ~m;
  }
  if (ok) l1_apply<kPrivate>(t, g, k, 1u, v, v, v, spill, status);
}

// Moves one slot of a level-1 table to level 2 (packed or plain form).
template <bool kPacked>
__device__ __forceinline__ void slot_to_l2(const GTable &g, uint32_t key, uint32_t cnt,
                                           unsigned long long sum, uint32_t mn, uint32_t mx,
                                           uint32_t *status) {
  uint64_t c = cnt;
  int64_t s = (int64_t)sum;
  if (kPacked) {
    c = sum >> kPackShift;
    s = (int64_t)(sum & ((1ull << kPackShift) - 1)) - (int64_t)c * (int64_t)kFlip;
  }
  if (c == 0) return;
  const int32_t k = (int32_t)(key ^ kFlip);
  g_update(g, g_slot(g, k, status), c, s, mn, mx);
}

// A warp flushes its private table to level 2 and resets the accumulators
// (keys stay claimed).
__device__ __forceinline__ void warp_flush(const L1 &t, const GTable &g, uint32_t *status) {
  __syncwarp();
  for (int i = threadIdx.x & 31; i <= (int)t.mask; i += 32) {
    if (t.key[i] != 0) {
      slot_to_l2<true>(g, t.key[i], 0, t.sum[i], t.mn[i], t.mx[i], status);
      t.sum[i] = 0;
      t.mn[i] = 0;
      t.mx[i] = 0;
    }
  }
  __syncwarp();
}

// Aggregation kernel.  Work item i covers rows [item_lo(i), item_hi(i)) of
// either the raw SoA input (items of w rows; level 1 persists across items
// and is flushed to level 2 when the CTA finishes) or the partitioned AoS
// pairs (one partition, or a w-row piece of one; level 1 is cleared per
// item and a whole partition is emitted directly).
template <bool kPrivate, bool kPairs>
__global__ void __launch_bounds__(kThreads)
    k_groupby(const int32_t *__restrict__ keys, const int32_t *__restrict__ vals,
              const int2 *__restrict__ pairs, uint64_t n, uint64_t w,
              const uint64_t *__restrict__ poff, const uint64_t *__restrict__ item_off, uint32_t P,
              uint32_t tslots, GTable g, Out o, unsigned long long *item_ctr, uint32_t *status) {
  static_assert(!(kPrivate && kPairs), "private tables are for raw input");
  extern __shared__ __align__(16) unsigned char smem[];
  // shared-table size: a power of two <= kSlots chosen by the host from the
  // expected groups per item; the arrays below are laid out for kSlots
  const int kTab = kPrivate ? kPrivSlots * kWarps : (int)tslots;
  constexpr int kLayout = kPrivate ? kPrivSlots * kWarps : kSlots;
  unsigned long long *sum_all = reinterpret_cast<unsigned long long *>(smem);
  uint32_t *key_all = reinterpret_cast<uint32_t *>(sum_all + kLayout);
  uint32_t *cnt_all = key_all + kLayout;
  uint32_t *mn_all = cnt_all + kLayout;
  uint32_t *mx_all = mn_all + kLayout;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  L1 t;
  if (kPrivate) {
    const int o0 = warp * kPrivSlots;
    t = L1{key_all + o0, cnt_all + o0, sum_all + o0, mn_all + o0, mx_all + o0, kPrivSlots - 1,
           32u - (uint32_t)__popc(kPrivSlots - 1)};
  } else {
    t = L1{key_all, cnt_all, sum_all, mn_all, mx_all, tslots - 1, 32u - (uint32_t)__popc(tslots - 1)};
  }
  __shared__ unsigned long long s_item;
  __shared__ int s_spill;
  __shared__ uint32_t s_warp[kWarps];
  __shared__ unsigned long long s_base;
  const uint64_t total_items = kPairs ? item_off[P] : (n + w - 1) / w;

  auto clear = [&]() {
    for (int i = threadIdx.x; i < kTab; i += kThreads) {
      key_all[i] = 0;
      cnt_all[i] = 0;
      sum_all[i] = 0;
      mn_all[i] = 0;
      mx_all[i] = 0;
    }
  };
  // level 1 -> level 2 (every occupied slot of the CTA's tables)
  auto flush = [&]() {
    for (int i = threadIdx.x; i < kTab; i += kThreads) {
      if (key_all[i] != 0)
        slot_to_l2<kPrivate>(g, key_all[i], cnt_all[i], sum_all[i], mn_all[i], mx_all[i], status);
    }
  };

  clear();
  uint32_t warp_rows_done = 0;  // rows this warp added since its last flush
  for (;;) {
    if (threadIdx.x == 0) {
      s_item = atomicAdd(item_ctr, 1ull);
      s_spill = 0;
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
    bool spill = false;
    // 4 rows per thread per round, loads issued together; whole warps run
    // every round (a private table is flushed every kPrivFlushRows rows of
    // its warp)
    for (uint64_t base = lo; base < hi; base += 4 * kThreads) {
      int32_t k[4], v[4];
      bool ok[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const uint64_t i = base + threadIdx.x + (uint64_t)u * kThreads;
        ok[u] = i < hi;
        if (ok[u]) {
          if (kPairs) {
            const int2 pv = __ldcs(pairs + i);
            k[u] = pv.x;
            v[u] = pv.y;
          } else {
            k[u] = __ldcs(keys + i);
            v[u] = __ldcs(vals + i);
          }
        } else {
          k[u] = 0;
          v[u] = 0;
        }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
        warp_rows<kPrivate>(t, g, k[u], v[u], ok[u], spill, status);
      if (kPrivate) {
        warp_rows_done += 4 * 32;
        if (warp_rows_done >= kPrivFlushRows) {
          warp_flush(t, g, status);
          warp_rows_done = 0;
        }
      }
    }
    if (spill) s_spill = 1;
    __syncthreads();
    if (kPairs) {
      if (whole && !s_spill) {
        // final groups of a whole partition: compact straight to the output
        uint32_t mine = 0;
        for (int i = threadIdx.x; i < kTab; i += kThreads) mine += key_all[i] != 0;
        mine = __reduce_add_sync(0xffffffffu, mine);
        if (lane == 0) s_warp[warp] = mine;
        __syncthreads();
        if (threadIdx.x == 0) {
          uint32_t tot = 0;
          for (int w2 = 0; w2 < kWarps; ++w2) tot += s_warp[w2];
          s_base = tot ? atomicAdd(o.n, (unsigned long long)tot) : 0;
        }
        __syncthreads();
        uint64_t pos = s_base;
        for (int w2 = 0; w2 < warp; ++w2) pos += s_warp[w2];
        for (int i0 = warp * 32; i0 < kTab; i0 += kThreads) {
          const int i = i0 + lane;
          const bool occ = key_all[i] != 0;
          const unsigned b = __ballot_sync(0xffffffffu, occ);
          if (occ)
            emit(o, pos + __popc(b & ((1u << lane) - 1)), (int32_t)(key_all[i] ^ kFlip), cnt_all[i],
                 (int64_t)sum_all[i], dec_min(mn_all[i]), dec_max(mx_all[i]), status);
          pos += __popc(b);
        }
      } else {
        flush();
      }
      __syncthreads();
      clear();
    }
    __syncthreads();
  }
  if (!kPairs) {
    __syncthreads();
    flush();
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

  // ---- plan: on-chip tables for small key domains, radix partitioning
  //      (so a partition's groups fit on chip) for large ones ----
  uint64_t hint = 0;
  int strategy = 0;
  if (params) {
    hint = params->expected_groups ? params->expected_groups : params->max_input_size;
    strategy = params->strategy;
  }
  if (strategy < 0 || strategy > 2) return set_error(ctx, GBJ_ERR_INVALID, "groupby: bad strategy");
  int32_t tuned_bits = 0;
  if (strategy == 0) {  // an autotuned plan for this (rows, groups) bucket, if any
    const int32_t tv = tuned_value(ctx, tune_key("groupby", n, hint));
    if (tv > 0) {
      strategy = tv >> 8;
      tuned_bits = tv & 0xff;
    }
  }
  const uint64_t groups_cap =
      std::max<uint64_t>(1024, hint ? std::min<uint64_t>(hint, n) : std::min<uint64_t>(n, 1ull << 24));
  if (strategy == 0) strategy = (hint && hint <= kSlots / 2) ? 1 : (hint ? 2 : 1);
  const bool priv = strategy == 1 && hint && hint <= kPrivMaxGroups;

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

  uint32_t tslots_arg = kSlots;
  auto launch = [&](auto kern, int tab, const int2 *pairs, uint64_t w, const uint64_t *poff,
                    const uint64_t *items, uint32_t P) -> int {
    const size_t smem = (size_t)tab * (8 + 4 + 4 + 4 + 4);
    GBJ_CHECK_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 1;
    GBJ_CHECK_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem));
    per_sm = std::max(per_sm, 1);
    kern<<<ctx->sm_count * per_sm, kThreads, smem, s>>>(d_keys, d_values, pairs, n, w, poff, items,
                                                        P, tslots_arg, g, o, ctr, ctx->d_status);
    return after_launch(ctx, "k_groupby", s);
  };

  if (strategy == 1) {
    // raw input in items of w rows; level 1 persists for the CTA's lifetime
    const uint64_t w = std::max<uint64_t>(1u << 16, (n + ctx->sm_count * 8 - 1) / (ctx->sm_count * 8));
    const uint64_t wq = (w + 3) / 4 * 4;
    if (priv) {
      GBJ_TRY(launch(k_groupby<true, false>, kPrivSlots * kWarps, nullptr, wq, nullptr, nullptr, 0));
    } else {
      tslots_arg = (uint32_t)std::min<uint64_t>(kSlots, std::max<uint64_t>(64, next_pow2(2 * groups_cap)));
      GBJ_TRY(launch(k_groupby<false, false>, kSlots, nullptr, wq, nullptr, nullptr, 0));
    }
  } else {
    // partition so each partition holds ~kSlots/4 groups; add bits (without
    // adding a partitioning pass) so partitions fit one work item of w rows
    // and are emitted directly
    const uint64_t w = 1u << 17;
    int bits = 1;
    while (bits < kMaxPartBits && (groups_cap >> bits) > (uint64_t)kSlots / 4) ++bits;
    const int free_bits = bits <= 8 ? 8 : kMaxPartBits;
    while (bits < free_bits && (n >> bits) > w / 2) ++bits;
    if (params && params->hash_bits > 0 && strategy == 2 && !hint)
      bits = std::min(params->hash_bits, kMaxPartBits);
    if (tuned_bits > 0) bits = std::min<int>(tuned_bits, kMaxPartBits);
    const uint32_t P = 1u << bits;
    tslots_arg = (uint32_t)std::min<uint64_t>(
        kSlots, std::max<uint64_t>(64, next_pow2(4 * ((groups_cap + P - 1) >> bits))));
    int2 *pairs;
    uint64_t *poff, *items;
    GBJ_TRY(scratch.get(n, &pairs));
    GBJ_TRY(scratch.get(P + 1, &poff));
    GBJ_TRY(scratch.get(P + 1, &items));
    GBJ_TRY(partition_tuples(ctx, d_keys, d_values, n, GBJ_DIGIT_HASH, 0, bits, pairs, nullptr,
                             nullptr, poff, s));
    k_groupby_items<<<(P + 255) / 256, 256, 0, s>>>(poff, P, w, items);
    GBJ_TRY(after_launch(ctx, "k_groupby_items", s));
    GBJ_TRY(scan_u64(ctx, items, items, P, s));
    GBJ_TRY(launch(k_groupby<false, true>, kSlots, pairs, w, poff, items, P));
  }
  const uint64_t emit_threads = 256;
  const uint64_t emit_blocks =
      std::min<uint64_t>((cap + emit_threads) / emit_threads, (uint64_t)ctx->sm_count * 8);
  k_groupby_emit<<<(unsigned)emit_blocks, emit_threads, 0, s>>>(g, o, ctx->d_status);
  return after_launch(ctx, "k_groupby_emit", s);
}
