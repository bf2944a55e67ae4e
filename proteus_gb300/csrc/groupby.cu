// Hash group-by with COUNT / SUM(int64) / MIN / MAX of one int32 value.
//
// Stands in for GpuHashGroupByChained (core/olap/lib/operators/gpu/
// gpu-hash-group-by-chained.cpp:77-556): the reference inserts every row
// into one global chained table with CAS on the chain heads and monoid
// atomics (gmonoids.cpp:122-360), then a scan pipeline emits entries whose
// next != self (hash-group-by-chained.cpp:638-853).
//
// GB300 design:
//  * level 1 is one open-addressing table of up to 4096 slots per CTA in
//    shared memory, updated with 32-bit atomics only (count, and the sum as
//    two 16-bit halves of the biased value, which stay exact while a slot
//    takes at most 65535 rows between flushes; hot slots move to level 2
//    before that).  Min and max atomics are issued only when the value
//    improves the stored extreme, so they fade out as a group fills;
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
constexpr int kSlots = 4096;     // level-1 table slots per CTA (at most)
constexpr int kProbeL1 = 32;     // level-1 probe limit before spilling to level 2
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

// Level 1: one table per CTA in shared memory, updated with 32-bit atomics
// only (64-bit shared atomics have no native form and cost a CAS loop).
// Structure of arrays, so that the atomics of a warp's 32 random slots
// spread over all 32 banks:
//   key[]  key' (0 = empty)
//   ext[]  {min', max'}: also the hints that decide whether a min/max
//          atomic is issued
//   cnt[]  rows
//   a[], b[]  with u = value + 2^31 (unsigned, < 2^32), a sums the low 16
//          bits of u and b the high 16 bits, so
//          SUM(value) = b * 2^16 + a - count * 2^31.
// a, b and cnt stay exact while a slot takes at most 65535 rows between
// flushes; the kernel tracks a CTA-wide bound on every slot's count and moves
// slots above kHot rows to level 2 before the bound could pass 65535.
// cnt, a and b have 2^rlog columns per slot, column = lane mod 2^rlog: a
// shared atomic costs a data-pipe pass per bank it hits twice, and with
// lane-indexed columns the lanes of a warp that land on slots in one bank
// fall on different banks (32 columns: never two lanes on one bank).  The
// host takes as many columns as shared memory allows; a slot's value is the
// sum of its columns.
__device__ __forceinline__ uint32_t s_ld(uint32_t a) {
  uint32_t r;
  asm("ld.shared.u32 %0, [%1];" : "=r"(r) : "r"(a));
  return r;
}
__device__ __forceinline__ uint2 s_ld2(uint32_t a) {
  uint2 r;
  asm("ld.shared.v2.u32 {%0, %1}, [%2];" : "=r"(r.x), "=r"(r.y) : "r"(a));
  return r;
}
__device__ __forceinline__ void s_st(uint32_t a, uint32_t v) {
  asm volatile("st.shared.u32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}
__device__ __forceinline__ void s_st2(uint32_t a, uint2 v) {
  asm volatile("st.shared.v2.u32 [%0], {%1, %2};" ::"r"(a), "r"(v.x), "r"(v.y) : "memory");
}

// The table's arrays by their shared-state-space addresses (32-bit).
struct L1 {
  uint32_t ext, key, cnt, a, b;
  uint32_t mask;   // slots - 1
  uint32_t shift;  // 32 - log2(slots): the home slot is the hash's top bits
  uint32_t rlog;   // log2 of the columns of cnt, a, b

  // Lays the arrays out from shared address `base` for `slots` slots.
  __device__ __forceinline__ void place(uint32_t base, uint32_t slots, uint32_t rlog_) {
    rlog = rlog_;
    ext = base;
    key = ext + 8u * slots;
    cnt = key + 4u * slots;
    a = cnt + (4u * slots << rlog);
    b = a + (4u * slots << rlog);
    mask = slots - 1;
    shift = 32u - (uint32_t)__popc(slots - 1);
  }
  // this lane's column of slot h (byte offset into cnt / a / b)
  __device__ __forceinline__ uint32_t col(uint32_t h) const {
    return ((h << rlog) + ((threadIdx.x & 31) & ((1u << rlog) - 1))) * 4u;
  }
  __device__ __forceinline__ uint32_t sum_cols(uint32_t arr, int i) const {
    uint32_t v = 0;
    for (uint32_t r = 0; r < (1u << rlog); ++r) v += s_ld(arr + (((uint32_t)i << rlog) + r) * 4u);
    return v;
  }
  // a slot as {key', min', max', count} and {a, b} (block-synchronised paths)
  __device__ __forceinline__ uint4 meta(int i) const {
    const uint2 e = s_ld2(ext + 8u * i);
    return make_uint4(s_ld(key + 4u * i), e.x, e.y, count(i));
  }
  __device__ __forceinline__ uint2 sums(int i) const { return make_uint2(sum_cols(a, i), sum_cols(b, i)); }
  __device__ __forceinline__ uint32_t count(int i) const { return sum_cols(cnt, i); }
  __device__ __forceinline__ void reset(int i, uint32_t k) const {
    s_st(key + 4u * i, k);
    s_st2(ext + 8u * i, make_uint2(0, 0));
    for (uint32_t r = 0; r < (1u << rlog); ++r) {
      const uint32_t o = (((uint32_t)i << rlog) + r) * 4u;
      s_st(cnt + o, 0);
      s_st(a + o, 0);
      s_st(b + o, 0);
    }
  }
};
// shared bytes per slot with 2^rlog accumulator columns
__host__ __device__ constexpr size_t slot_bytes(int rlog) { return 12 + ((size_t)12 << rlog); }
// Shared bytes the table may take per CTA (two CTAs per SM).
constexpr size_t kTableBudget = 96 * 1024;

constexpr uint32_t kChunk = 32768;        // rows per step between bound checks
constexpr uint32_t kCountLimit = 65535;   // rows a slot may take between flushes
constexpr uint32_t kHot = kCountLimit - kChunk;  // slots above go to level 2 at a check

// Shared-memory accesses of the level-1 table, in the shared state space
// explicitly (32-bit atomics only; a load of a slot may run ahead of an
// earlier row's atomics: it only decides the claim path, which re-checks with
// CAS, and whether a min/max atomic is worth issuing).
__device__ __forceinline__ uint32_t s_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ uint32_t s_ld_volatile(uint32_t a) {
  uint32_t r;
  asm volatile("ld.volatile.shared.u32 %0, [%1];" : "=r"(r) : "r"(a) : "memory");
  return r;
}
__device__ __forceinline__ void s_red_add(uint32_t a, uint32_t v) {
  asm volatile("red.shared.add.u32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}
// red.max issued only when v is above the loaded hint (predicated, no branch).
__device__ __forceinline__ void s_red_max_above(uint32_t a, uint32_t v, uint32_t hint) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.gt.u32 p, %1, %2;\n\t@p red.shared.max.u32 [%0], %1;\n\t}" ::"r"(a),
      "r"(v), "r"(hint)
      : "memory");
}
__device__ __forceinline__ uint32_t s_cas(uint32_t a, uint32_t cmp, uint32_t v) {
  uint32_t r;
  asm volatile("atom.shared.cas.b32 %0, [%1], %2, %3;" : "=r"(r) : "r"(a), "r"(cmp), "r"(v) : "memory");
  return r;
}

// Home slot: Fibonacci hashing, top bits.  Independent of the fmix32 low bits
// that pick a key's partition, so it also spreads the keys of one partition.
// The home is a bucket of two slots (an even slot and the next): one 8-byte
// load checks both, so a key displaced by one collision still takes the
// fast path.  Insertion claims the first empty slot from the bucket on.
__device__ __forceinline__ uint32_t l1_home(const L1 &t, int32_t k) {
  return (((uint32_t)k * 0x9E3779B1u) >> (t.shift + 1)) << 1;
}

__device__ __forceinline__ int64_t l1_sum(uint2 ab, uint32_t c) {
  return (int64_t)(((uint64_t)ab.y << 16) + ab.x) - (int64_t)c * (int64_t)kFlip;
}

// The slow path of a row whose key is not in its home slot: probes on,
// claiming an empty slot with CAS.  Returns the slot, or -1 after sending
// the row to level 2 (INT32_MIN keys, or no slot within kProbeL1 steps).
__device__ __forceinline__ int l1_find(const L1 &t, const GTable &g, int32_t k, int32_t v, uint32_t h,
                                    uint32_t *status) {
  const uint32_t u = (uint32_t)v ^ kFlip;
  if (k != INT32_MIN) {
    const uint32_t kk = (uint32_t)k ^ kFlip;
    const uint32_t base = t.key;
    for (int step = 0; step < kProbeL1; ++step) {
      const uint32_t a = base + h * 4u;
      uint32_t cur = s_ld_volatile(a);
      if (cur == 0) cur = s_cas(a, 0u, kk);
      if (cur == 0 || cur == kk) return (int)h;
      h = (h + 1) & t.mask;
    }
  }
  g_row(g, k, 1, v, ~u, u, status);
  return -1;
}

// One row into level 1; rows that go to level 2 set `spill`.
__device__ __forceinline__ void l1_row(const L1 &t, const GTable &g, int32_t k, int32_t v, bool &spill,
                                       uint32_t *status) {
  const uint32_t u = (uint32_t)v ^ kFlip;  // biased value = max' encoding; ~u = min'
  uint32_t h = l1_home(t, k);
  const uint32_t kk = (uint32_t)k ^ kFlip;
  uint2 pair = s_ld2(t.key + h * 4u);
  // INT32_MIN's key' is 0 (the empty mark), so it always takes the slow path
  bool found = k != INT32_MIN && (pair.x == kk || pair.y == kk);
  if (found) {
    h += pair.x != kk;
  } else if (k != INT32_MIN) {
    // the next bucket holds most keys displaced from their home
    const uint32_t h2 = (h + 2) & t.mask;
    pair = s_ld2(t.key + h2 * 4u);
    found = pair.x == kk || pair.y == kk;
    if (found) h = h2 + (pair.x != kk);
  }
  if (!found) {
    const int f = l1_find(t, g, k, v, h, status);
    if (f < 0) {
      spill = true;
      return;
    }
    h = (uint32_t)f;
  }
  const uint32_t ea = t.ext + h * 8u;
  const uint2 e = s_ld2(ea);
  const uint32_t c = t.col(h);
  s_red_add(t.cnt + c, 1u);
  s_red_add(t.a + c, u & 0xffffu);
  s_red_add(t.b + c, u >> 16);
  s_red_max_above(ea, ~u, e.x);
  s_red_max_above(ea + 4, u, e.y);
}

// Moves one level-1 slot to level 2.
__device__ __forceinline__ void slot_to_l2(const GTable &g, uint4 m, uint2 ab, uint32_t *status) {
  if (m.w == 0) return;
  const int32_t k = (int32_t)(m.x ^ kFlip);
  g_update(g, g_slot(g, k, status), m.w, l1_sum(ab, m.w), m.y, m.z);
}

// Block-wide helpers (every thread of the CTA calls them).
__device__ __forceinline__ void l1_clear(const L1 &t, int tab, uint32_t &s_bound) {
  for (int i = threadIdx.x; i < tab; i += kThreads) t.reset(i, 0);
  if (threadIdx.x == 0) s_bound = 0;
}

// level 1 -> level 2 (every occupied slot)
__device__ __forceinline__ void l1_flush(const L1 &t, int tab, const GTable &g, uint32_t *status) {
  for (int i = threadIdx.x; i < tab; i += kThreads) slot_to_l2(g, t.meta(i), t.sums(i), status);
}

// Before adding `rows` rows: if the bound on every slot's count could pass
// kCountLimit, move the hot slots to level 2 and recompute the bound.  Ends
// with s_bound updated by thread 0; the caller's next __syncthreads
// publishes it.
__device__ __forceinline__ void l1_make_room(const L1 &t, int tab, const GTable &g, uint32_t rows, bool &spill,
                                             uint32_t *status, uint32_t &s_bound, uint32_t *s_warp) {
  if (s_bound + rows <= kCountLimit) {
    __syncthreads();
    if (threadIdx.x == 0) s_bound += rows;
    return;
  }
  __syncthreads();
  uint32_t mx = 0;
  for (int i = threadIdx.x; i < tab; i += kThreads) {
    const uint4 m = t.meta(i);
    if (m.w > kHot) {
      slot_to_l2(g, m, t.sums(i), status);
      t.reset(i, m.x);
      spill = true;
    } else {
      mx = max(mx, m.w);
    }
  }
  mx = __reduce_max_sync(0xffffffffu, mx);
  if ((threadIdx.x & 31) == 0) s_warp[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t b = 0;
    for (int w2 = 0; w2 < kWarps; ++w2) b = max(b, s_warp[w2]);
    s_bound = b + rows;
  }
}

// Reads keys/values rows [i, i+4) with 16-byte loads.
__device__ __forceinline__ void load4(const int32_t *__restrict__ keys, const int32_t *__restrict__ vals,
                                      uint64_t i, int4 &k, int4 &v) {
  k = __ldcs(reinterpret_cast<const int4 *>(keys + i));
  v = __ldcs(reinterpret_cast<const int4 *>(vals + i));
}

// Aggregation kernel.  Work item i covers rows [item_lo(i), item_hi(i)) of
// either the raw SoA input (items of w rows; level 1 persists across items
// and is flushed to level 2 when the CTA finishes) or the partitioned AoS
// pairs (one partition, or a w-row piece of one; level 1 is cleared per
// item and a whole partition is emitted directly).  kVec: the raw columns
// are 16-byte aligned and read 4 rows per thread per load.
template <bool kPairs, bool kVec>
__global__ void __launch_bounds__(kThreads, 2)
    k_groupby(const int32_t *__restrict__ keys, const int32_t *__restrict__ vals,
              const int2 *__restrict__ pairs, uint64_t n, uint64_t w,
              const uint64_t *__restrict__ poff, const uint64_t *__restrict__ item_off, uint32_t P,
              uint32_t tslots, uint32_t rlog, GTable g, Out o, unsigned long long *item_ctr, uint32_t *status) {
  extern __shared__ __align__(16) unsigned char smem[];
  // shared-table size: a power of two <= kSlots chosen by the host from the
  // expected groups per item
  const int kTab = (int)tslots;
  L1 t;
  t.place(s_addr(smem), tslots, rlog);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __shared__ unsigned long long s_item;
  __shared__ int s_spill;
  __shared__ uint32_t s_warp[kWarps];
  __shared__ unsigned long long s_base;
  __shared__ uint32_t s_bound;  // >= every slot's count
  const uint64_t total_items = kPairs ? item_off[P] : (n + w - 1) / w;

  l1_clear(t, kTab, s_bound);
  for (;;) {
    __syncthreads();
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
    for (uint64_t c0 = lo; c0 < hi; c0 += kChunk) {
      const uint64_t c1 = c0 + kChunk < hi ? c0 + kChunk : hi;
      l1_make_room(t, kTab, g, (uint32_t)(c1 - c0), spill, status, s_bound, s_warp);
      __syncthreads();
      if (!kPairs && kVec) {
        // 4 rows per thread per step; the loads of the next two steps are
        // in flight while this step's rows are applied
        constexpr uint64_t kStep = 4 * kThreads;
        uint64_t i = c0 + 4 * (uint64_t)threadIdx.x;
        int4 ka = make_int4(0, 0, 0, 0), va = ka, kb = ka, vb = ka;
        if (i + 4 <= c1) load4(keys, vals, i, ka, va);
        if (i + kStep + 4 <= c1) load4(keys, vals, i + kStep, kb, vb);
        for (; i < c1; i += kStep) {
          const int4 kc = ka, vc = va;
          ka = kb;
          va = vb;
          const bool full = i + 4 <= c1;
          if (i + 2 * kStep + 4 <= c1) load4(keys, vals, i + 2 * kStep, kb, vb);
          if (full) {
            l1_row(t, g, kc.x, vc.x, spill, status);
            l1_row(t, g, kc.y, vc.y, spill, status);
            l1_row(t, g, kc.z, vc.z, spill, status);
            l1_row(t, g, kc.w, vc.w, spill, status);
          } else {
            for (uint64_t r = i; r < c1; ++r) l1_row(t, g, __ldcs(keys + r), __ldcs(vals + r), spill, status);
          }
        }
      } else {
        // 4 rows per thread per step (stride kThreads); the next step's
        // loads are issued before this step's rows are applied
        auto load = [&](uint64_t base, int2 (&r)[4]) {
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const uint64_t i = base + threadIdx.x + (uint64_t)u * kThreads;
            r[u] = make_int2(0, 0);
            if (i < c1) {
              if (kPairs) r[u] = __ldcs(pairs + i);
              else r[u] = make_int2(__ldcs(keys + i), __ldcs(vals + i));
            }
          }
        };
        int2 nx[4];
        load(c0, nx);
        for (uint64_t base = c0; base < c1; base += 4 * kThreads) {
          int2 cur[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) cur[u] = nx[u];
          if (base + 4 * kThreads < c1) load(base + 4 * kThreads, nx);
#pragma unroll
          for (int u = 0; u < 4; ++u)
            if (base + threadIdx.x + (uint64_t)u * kThreads < c1) l1_row(t, g, cur[u].x, cur[u].y, spill, status);
        }
      }
    }
    if (spill) s_spill = 1;
    __syncthreads();
    if (kPairs) {
      if (whole && !s_spill) {
        // final groups of a whole partition: compact straight to the output
        uint32_t mine = 0;
        for (int i = threadIdx.x; i < kTab; i += kThreads) mine += t.count(i) != 0;
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
          const uint4 m = i < kTab ? t.meta(i) : make_uint4(0, 0, 0, 0);
          const bool occ = m.w != 0;
          const unsigned b = __ballot_sync(0xffffffffu, occ);
          if (occ)
            emit(o, pos + __popc(b & ((1u << lane) - 1)), (int32_t)(m.x ^ kFlip), m.w, l1_sum(t.sums(i), m.w),
                 dec_min(m.y), dec_max(m.z), status);
          pos += __popc(b);
        }
      } else {
        l1_flush(t, kTab, g, status);
      }
      __syncthreads();
      l1_clear(t, kTab, s_bound);
    }
  }
  if (!kPairs) {
    __syncthreads();
    l1_flush(t, kTab, g, status);
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

  uint32_t tslots_arg = kSlots, rlog_arg = 0;
  // as many accumulator columns (up to 32) as the table budget allows
  auto pick_rlog = [&]() {
    rlog_arg = 0;
    while (rlog_arg < 5 && (size_t)tslots_arg * slot_bytes(rlog_arg + 1) <= kTableBudget) ++rlog_arg;
  };
  auto launch = [&](auto kern, int tab, const int2 *pairs, uint64_t w, const uint64_t *poff,
                    const uint64_t *items, uint32_t P) -> int {
    const size_t smem = (size_t)tab * slot_bytes(rlog_arg);
    GBJ_CHECK_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 1;
    GBJ_CHECK_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem));
    per_sm = std::max(per_sm, 1);
    kern<<<ctx->sm_count * per_sm, kThreads, smem, s>>>(d_keys, d_values, pairs, n, w, poff, items,
                                                        P, tslots_arg, rlog_arg, g, o, ctr, ctx->d_status);
    return after_launch(ctx, "k_groupby", s);
  };

  if (strategy == 1) {
    // raw input in items of w rows; level 1 persists for the CTA's lifetime
    const uint64_t w = std::max<uint64_t>(1u << 16, (n + ctx->sm_count * 8 - 1) / (ctx->sm_count * 8));
    const uint64_t wq = (w + 3) / 4 * 4;
    tslots_arg = (uint32_t)std::min<uint64_t>(kSlots, std::max<uint64_t>(64, next_pow2(16 * (hint ? hint : groups_cap))));
    pick_rlog();
    const bool aligned = (reinterpret_cast<uintptr_t>(d_keys) | reinterpret_cast<uintptr_t>(d_values)) % 16 == 0;
    if (aligned) GBJ_TRY(launch(k_groupby<false, true>, (int)tslots_arg, nullptr, wq, nullptr, nullptr, 0));
    else GBJ_TRY(launch(k_groupby<false, false>, (int)tslots_arg, nullptr, wq, nullptr, nullptr, 0));
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
    pick_rlog();
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
    GBJ_TRY(launch(k_groupby<true, false>, (int)tslots_arg, pairs, w, poff, items, P));
  }
  const uint64_t emit_threads = 256;
  const uint64_t emit_blocks =
      std::min<uint64_t>((cap + emit_threads) / emit_threads, (uint64_t)ctx->sm_count * 8);
  k_groupby_emit<<<(unsigned)emit_blocks, emit_threads, 0, s>>>(g, o, ctx->d_status);
  return after_launch(ctx, "k_groupby_emit", s);
}
