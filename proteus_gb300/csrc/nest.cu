// The int64-key twins of the radix path: RadixNest's grouping and the
// int64 RJStepwise match count.
//
// Stand in for Nest (RadixNest, core/olap/lib/operators/radix-nest.cpp:
// 326-700), which clusters {int64 key, int64 payload} tuples with the
// aggregation twin's partitionHT, builds bucket chains per cluster and folds
// every tuple of a key into that key's group (core/platform/lib/util/radix/
// aggregations/radix-aggr.cpp:163-259), and for the twin's RJStepwise
// (radix-aggr.cpp:261-358), which counts the (R, S) pairs with equal keys.
// The same grouping engine serves HashGroupByChained over int64 keys with
// int32 values (gbj_groupby_i64, hash-group-by-chained.cpp:267-853).
//
// GB300 design: for few groups an on-chip level per CTA (32-bit shared
// reductions only) in front of the global table; otherwise one global
// open-addressing table per call, 2^k slots of
// 64-bit keys (key ^ 2^63, so all-zero = empty; INT64_MIN, whose stored form
// is 0, has a dedicated slot), updated with native 64-bit global atomics
// (the table of up to ~2^22 groups stays in the 126 MB L2).  The nest keeps
// COUNT, SUM (two's-complement wrap, as int64 addition), and MIN / MAX in
// order-preserving unsigned encodings combined with atomicMax, issued only
// when the value improves the stored extreme.  The join count stores each
// R key's multiplicity and every S row adds the multiplicity of its key.
#include <algorithm>

#include "gbj_internal.cuh"

using namespace gbj;

namespace {

constexpr int kThreads = 256;
constexpr uint64_t kFlip64 = 0x8000000000000000ull;

__device__ __forceinline__ uint64_t fmix64(uint64_t k) {  // murmur3 64-bit finaliser
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ull;
  k ^= k >> 33;
  return k;
}

struct Table64 {
  unsigned long long *key;  // key ^ 2^63; 0 = empty
  unsigned long long *cnt;
  unsigned long long *sum;
  unsigned long long *mn;   // ~(value ^ 2^63), combined with max
  unsigned long long *mx;   // value ^ 2^63
  uint64_t mask;            // slots - 1; slot mask + 1 is INT64_MIN's
};

// Slot of key k (claimed when new), or -1 when the table is full.
__device__ __forceinline__ int64_t slot_of(const Table64 &t, int64_t k, uint32_t *status) {
  if (k == INT64_MIN) return (int64_t)(t.mask + 1);
  const unsigned long long kk = (unsigned long long)k ^ kFlip64;
  uint64_t h = fmix64((uint64_t)k) & t.mask;
  for (uint64_t step = 0; step <= t.mask; ++step) {
    unsigned long long cur = *(volatile unsigned long long *)&t.key[h];
    if (cur == kk) return (int64_t)h;
    if (cur == 0) {
      cur = atomicCAS(&t.key[h], 0ull, kk);
      if (cur == 0 || cur == kk) return (int64_t)h;
    }
    h = (h + 1) & t.mask;
  }
  gbjd::latch(status, GBJ_DEV_CAPACITY);
  return -1;
}

// Slot of key k when present, else -1 (read only).
__device__ __forceinline__ int64_t find(const Table64 &t, int64_t k) {
  if (k == INT64_MIN) return (int64_t)(t.mask + 1);
  const unsigned long long kk = (unsigned long long)k ^ kFlip64;
  uint64_t h = fmix64((uint64_t)k) & t.mask;
  for (uint64_t step = 0; step <= t.mask; ++step) {
    const unsigned long long cur = __ldg(&t.key[h]);
    if (cur == kk) return (int64_t)h;
    if (cur == 0) return -1;
    h = (h + 1) & t.mask;
  }
  return -1;
}

// One row (key k, value v when has_v) into the global table.
__device__ __forceinline__ void add_kv(const Table64 &t, int64_t k, int64_t v, bool has_v, uint32_t *status) {
  const int64_t s = slot_of(t, k, status);
  if (s < 0) return;
  atomicAdd(&t.cnt[s], 1ull);
  if (has_v) {
    atomicAdd(&t.sum[s], (unsigned long long)v);
    const unsigned long long emx = (unsigned long long)v ^ kFlip64, emn = ~emx;
    if (emn > *(volatile unsigned long long *)&t.mn[s]) atomicMax(&t.mn[s], emn);
    if (emx > *(volatile unsigned long long *)&t.mx[s]) atomicMax(&t.mx[s], emx);
  }
}

template <typename V>
__device__ __forceinline__ void add_row(const Table64 &t, int64_t k, const V *vals, uint64_t i,
                                        uint32_t *status) {
  add_kv(t, k, vals ? (int64_t)__ldcs(vals + i) : 0, vals != nullptr, status);
}

// Every row into its group (vals null: counts only); V is the value
// column's type (int64 for the nest, int32 for the int64-key group-by).
template <typename V>
__global__ void __launch_bounds__(kThreads)
    k_nest_build(const int64_t *__restrict__ keys, const V *__restrict__ vals, uint64_t n, Table64 t,
                 uint32_t *status) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride)
    add_row(t, __ldcs(keys + i), vals, i, status);
}

// ---------------------------------------------------------------------------
// On-chip level for few groups (expected groups <= kL1MaxGroups): one table
// per CTA in shared memory, updated with 32-bit reductions only (64-bit
// shared atomics have no native form): the count, and the value as four
// 16-bit chunk sums (SUM = sum of chunk_i << 16 i, modulo 2^64 like int64
// addition), exact while a slot takes at most kL1Limit rows between flushes.
// The CTA keeps a bound on every slot's count and moves slots above kL1Hot
// rows to the global table before the bound could pass kL1Limit.  Min and
// max keep 64-bit encodings whose (emulated) atomics are issued only when a
// value improves the stored extreme.  The global table is level 2.
constexpr int kL1Threads = 512;
constexpr int kL1Warps = kL1Threads / 32;
constexpr uint64_t kL1MaxGroups = 2048;
constexpr uint32_t kL1MaxSlots = 4096;
constexpr uint32_t kL1Chunk = 32768;                 // rows per item (one bound check each)
constexpr uint32_t kL1Limit = 65535;                 // rows a slot may take between flushes
constexpr uint32_t kL1Hot = kL1Limit - kL1Chunk;     // slots above go to level 2 at a check
constexpr int kL1Probe = 32;
// key and {min', max'} per slot; count and 4 chunk sums per slot and column
__host__ __device__ constexpr uint32_t l1_slot_bytes(uint32_t rlog) { return 24 + (20u << rlog); }
constexpr size_t kL1Budget = 200 * 1024;  // shared bytes of the one CTA per SM

__device__ __forceinline__ uint32_t s_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ unsigned long long s_ld64(uint32_t a) {
  unsigned long long r;
  asm volatile("ld.volatile.shared.u64 %0, [%1];" : "=l"(r) : "r"(a) : "memory");
  return r;
}
__device__ __forceinline__ uint32_t s_ld32(uint32_t a) {
  uint32_t r;
  asm volatile("ld.volatile.shared.u32 %0, [%1];" : "=r"(r) : "r"(a) : "memory");
  return r;
}
__device__ __forceinline__ ulonglong2 s_ld128(uint32_t a) {
  ulonglong2 r;
  asm volatile("ld.volatile.shared.v2.u64 {%0, %1}, [%2];" : "=l"(r.x), "=l"(r.y) : "r"(a) : "memory");
  return r;
}
__device__ __forceinline__ void s_st64(uint32_t a, unsigned long long v) {
  asm volatile("st.shared.u64 [%0], %1;" ::"r"(a), "l"(v) : "memory");
}
__device__ __forceinline__ void s_st32(uint32_t a, uint32_t v) {
  asm volatile("st.shared.u32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long s_cas64(uint32_t a, unsigned long long c, unsigned long long v) {
  unsigned long long r;
  asm volatile("atom.shared.cas.b64 %0, [%1], %2, %3;" : "=l"(r) : "r"(a), "l"(c), "l"(v) : "memory");
  return r;
}
__device__ __forceinline__ void s_red32(uint32_t a, uint32_t v) {
  asm volatile("red.shared.add.u32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}
__device__ __forceinline__ void s_redmax64(uint32_t a, unsigned long long v) {
  asm volatile("red.shared.max.u64 [%0], %1;" ::"r"(a), "l"(v) : "memory");
}

// The table's arrays by shared-state-space address.
// count and chunk sums have 2^rlog columns per slot, column = lane mod 2^rlog,
// so the reductions of a warp's lanes on one hot slot fall on different
// addresses and banks; a slot's value is the sum of its columns.
struct L1N {
  uint32_t key;  // u64 [T]: key ^ 2^63, 0 = empty
  uint32_t ext;  // u64 [2T]: {min', max'}
  uint32_t cnt;  // u32 [T << rlog]
  uint32_t sum;  // u32 [4 (T << rlog)]: the 4 chunk sums of column c at 16 c
  uint32_t mask, shift;  // T - 1, 64 - log2 T
  uint32_t rlog;
  __device__ __forceinline__ uint32_t col(uint32_t h) const {
    return (h << rlog) + ((threadIdx.x & 31) & ((1u << rlog) - 1));
  }
  __device__ __forceinline__ uint32_t count(uint32_t i) const {
    uint32_t c = 0;
    for (uint32_t r = 0; r < (1u << rlog); ++r) c += s_ld32(cnt + 4u * ((i << rlog) + r));
    return c;
  }
  __device__ __forceinline__ uint32_t chunk(uint32_t i, int j) const {
    uint32_t c = 0;
    for (uint32_t r = 0; r < (1u << rlog); ++r) c += s_ld32(sum + 16u * ((i << rlog) + r) + 4u * j);
    return c;
  }
  __device__ __forceinline__ void reset_acc(uint32_t i) const {
    for (uint32_t r = 0; r < (1u << rlog); ++r) {
      const uint32_t c = (i << rlog) + r;
      s_st32(cnt + 4u * c, 0);
      for (int j = 0; j < 4; ++j) s_st32(sum + 16u * c + 4u * j, 0);
    }
  }
};

__device__ __forceinline__ void l1n_row(const L1N &t, const Table64 &g, int64_t k, int64_t v, bool has_v,
                                        bool &spill, uint32_t *status) {
  if (k == INT64_MIN) {  // its stored form is the empty mark
    add_kv(g, k, v, has_v, status);
    spill = true;
    return;
  }
  const unsigned long long kk = (unsigned long long)k ^ kFlip64;
  uint32_t h = (uint32_t)(((uint64_t)k * 0x9E3779B97F4A7C15ull) >> t.shift);
  for (int step = 0;; ++step) {
    unsigned long long cur = s_ld64(t.key + 8u * h);
    if (cur == kk) break;
    if (cur == 0) {
      cur = s_cas64(t.key + 8u * h, 0ull, kk);
      if (cur == 0 || cur == kk) break;
    }
    if (step + 1 == kL1Probe) {
      add_kv(g, k, v, has_v, status);
      spill = true;
      return;
    }
    h = (h + 1) & t.mask;
  }
  const uint32_t c = t.col(h);
  s_red32(t.cnt + 4u * c, 1u);
  if (has_v) {
    const unsigned long long u = (unsigned long long)v;
    const uint32_t sa = t.sum + 16u * c;
    s_red32(sa, (uint32_t)(u & 0xffffu));
    s_red32(sa + 4, (uint32_t)((u >> 16) & 0xffffu));
    s_red32(sa + 8, (uint32_t)((u >> 32) & 0xffffu));
    s_red32(sa + 12, (uint32_t)(u >> 48));
    const unsigned long long emx = u ^ kFlip64, emn = ~emx;
    const ulonglong2 e = s_ld128(t.ext + 16u * h);
    if (emn > e.x) s_redmax64(t.ext + 16u * h, emn);
    if (emx > e.y) s_redmax64(t.ext + 16u * h + 8, emx);
  }
}

// Slot i of level 1 into the global table (and reset its accumulators).
__device__ __forceinline__ void l1n_flush_slot(const L1N &t, const Table64 &g, uint32_t i, bool has_v,
                                               uint32_t *status) {
  const uint32_t c = t.count(i);
  if (c == 0) return;
  const int64_t k = (int64_t)(s_ld64(t.key + 8u * i) ^ kFlip64);
  const int64_t s = slot_of(g, k, status);
  if (s >= 0) {
    atomicAdd(&g.cnt[s], (unsigned long long)c);
    if (has_v) {
      const unsigned long long sum = (unsigned long long)t.chunk(i, 0) + ((unsigned long long)t.chunk(i, 1) << 16) +
                                     ((unsigned long long)t.chunk(i, 2) << 32) +
                                     ((unsigned long long)t.chunk(i, 3) << 48);
      atomicAdd(&g.sum[s], sum);
      const ulonglong2 e = s_ld128(t.ext + 16u * i);
      if (e.x) atomicMax(&g.mn[s], e.x);
      if (e.y) atomicMax(&g.mx[s], e.y);
    }
  }
  t.reset_acc(i);
  s_st64(t.ext + 16u * i, 0);
  s_st64(t.ext + 16u * i + 8, 0);
}

// Raw int64 rows in items of kL1Chunk; level 1 persists for the CTA's
// lifetime and goes to the global table when the CTA finishes.
template <typename V>
__global__ void __launch_bounds__(kL1Threads, 1)
    k_nest_l1(const int64_t *__restrict__ keys, const V *__restrict__ vals, uint64_t n, uint32_t tslots,
              uint32_t rlog, Table64 g, unsigned long long *item_ctr, uint32_t *status) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ unsigned long long s_item;
  __shared__ uint32_t s_bound;
  __shared__ uint32_t s_warp[kL1Warps];
  const uint32_t T = tslots;
  const uint32_t base = s_addr(smem);
  L1N t{base, base + 8u * T, base + 24u * T, base + 24u * T + ((4u * T) << rlog),
        T - 1, 64u - (uint32_t)__popc(T - 1), rlog};
  const bool has_v = vals != nullptr;
  for (uint32_t i = threadIdx.x; i < T; i += kL1Threads) {
    s_st64(t.key + 8u * i, 0);
    s_st64(t.ext + 16u * i, 0);
    s_st64(t.ext + 16u * i + 8, 0);
    t.reset_acc(i);
  }
  if (threadIdx.x == 0) s_bound = 0;
  const uint64_t items = (n + kL1Chunk - 1) / kL1Chunk;
  bool spill = false;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_item = atomicAdd(item_ctr, 1ull);
    __syncthreads();
    const uint64_t item = s_item;
    if (item >= items) break;
    const uint64_t lo = item * kL1Chunk, hi = lo + kL1Chunk < n ? lo + kL1Chunk : n;
    const uint32_t rows = (uint32_t)(hi - lo);
    // room for this item's rows: every slot's count stays <= kL1Limit
    if (s_bound + rows > kL1Limit) {
      uint32_t mx = 0;
      for (uint32_t i = threadIdx.x; i < T; i += kL1Threads) {
        const uint32_t c = t.count(i);
        if (c > kL1Hot) l1n_flush_slot(t, g, i, has_v, status);
        else mx = max(mx, c);
      }
      mx = __reduce_max_sync(0xffffffffu, mx);
      if ((threadIdx.x & 31) == 0) s_warp[threadIdx.x >> 5] = mx;
      __syncthreads();
      if (threadIdx.x == 0) {
        uint32_t b = 0;
        for (int w2 = 0; w2 < kL1Warps; ++w2) b = max(b, s_warp[w2]);
        s_bound = b + rows;
      }
    } else {
      __syncthreads();
      if (threadIdx.x == 0) s_bound += rows;
    }
    __syncthreads();
    // 4 rows per thread per step (stride kL1Threads), the next step's loads
    // issued before this step's rows are applied
    int64_t nk[4], nv[4];
    auto load = [&](uint64_t b0) {
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const uint64_t i = b0 + threadIdx.x + (uint64_t)u * kL1Threads;
        nk[u] = i < hi ? __ldcs(keys + i) : 0;
        nv[u] = (i < hi && has_v) ? (int64_t)__ldcs(vals + i) : 0;
      }
    };
    load(lo);
    for (uint64_t b0 = lo; b0 < hi; b0 += 4 * kL1Threads) {
      int64_t ck[4], cv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        ck[u] = nk[u];
        cv[u] = nv[u];
      }
      if (b0 + 4 * kL1Threads < hi) load(b0 + 4 * kL1Threads);
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (b0 + threadIdx.x + (uint64_t)u * kL1Threads < hi) l1n_row(t, g, ck[u], cv[u], has_v, spill, status);
    }
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < T; i += kL1Threads) l1n_flush_slot(t, g, i, has_v, status);
}

// The occupied slots (and INT64_MIN's) to the output; one output
// reservation per warp.
template <typename M>
__global__ void __launch_bounds__(kThreads)
    k_nest_emit(Table64 t, bool with_vals, int64_t *__restrict__ ok, int64_t *__restrict__ oc,
                int64_t *__restrict__ os, M *__restrict__ omn, M *__restrict__ omx, uint64_t cap,
                unsigned long long *__restrict__ n_out, uint32_t *status) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t slots = t.mask + 2;
  const int lane = threadIdx.x & 31;
  for (uint64_t b0 = blockIdx.x * (uint64_t)blockDim.x; b0 < slots; b0 += stride) {
    const uint64_t i = b0 + threadIdx.x;
    bool occ = false;
    int64_t key = INT64_MIN;
    if (i <= t.mask) {
      occ = t.key[i] != 0;
      key = (int64_t)(t.key[i] ^ kFlip64);
    } else if (i == t.mask + 1) {
      occ = t.cnt[i] != 0;
    }
    const unsigned bal = __ballot_sync(0xffffffffu, occ);
    unsigned long long base = 0;
    if (lane == 0 && bal) base = atomicAdd(n_out, (unsigned long long)__popc(bal));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (!occ) continue;
    const uint64_t pos = base + __popc(bal & ((1u << lane) - 1));
    if (pos >= cap) {
      gbjd::latch(status, GBJ_DEV_CAPACITY);
      continue;
    }
    if (ok) ok[pos] = key;
    if (oc) oc[pos] = (int64_t)t.cnt[i];
    if (os) os[pos] = with_vals ? (int64_t)t.sum[i] : 0;
    if (omn) omn[pos] = with_vals ? (M)(int64_t)(~t.mn[i] ^ kFlip64) : 0;
    if (omx) omx[pos] = with_vals ? (M)(int64_t)(t.mx[i] ^ kFlip64) : 0;
  }
}

// S rows add the multiplicity of their key in R; one atomic per block.
__global__ void __launch_bounds__(kThreads)
    k_join_count_probe(const int64_t *__restrict__ keys, uint64_t n, Table64 t,
                       unsigned long long *__restrict__ out) {
  __shared__ unsigned long long red[kThreads / 32];
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  unsigned long long acc = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    const int64_t s = find(t, __ldcs(keys + i));
    if (s >= 0) acc += __ldg(&t.cnt[s]);
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long tot = 0;
    for (int w = 0; w < kThreads / 32; ++w) tot += red[w];
    if (tot) atomicAdd(out, tot);
  }
}

// Table64 with `slots` slots (+ the INT64_MIN slot), zeroed, from scratch.
int make_table(gbj_ctx *ctx, Scratch &scratch, uint64_t slots, bool with_vals, cudaStream_t s, Table64 *t) {
  const uint64_t cols = with_vals ? 5 : 2;
  unsigned long long *mem;
  GBJ_TRY(scratch.get(cols * (slots + 1), &mem));
  GBJ_CHECK_CUDA(ctx, cudaMemsetAsync(mem, 0, sizeof(unsigned long long) * cols * (slots + 1), s));
  t->key = mem;
  t->cnt = mem + (slots + 1);
  t->sum = with_vals ? mem + 2 * (slots + 1) : nullptr;
  t->mn = with_vals ? mem + 3 * (slots + 1) : nullptr;
  t->mx = with_vals ? mem + 4 * (slots + 1) : nullptr;
  t->mask = slots - 1;
  return GBJ_OK;
}

unsigned grid_for(gbj_ctx *ctx, uint64_t n) {
  return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((n + kThreads - 1) / kThreads,
                                                            (uint64_t)ctx->sm_count * 8));
}


// Grouping over int64 keys: the nest's (V = M = int64) and the int64-key
// group-by's (V = M = int32).  `groups` sizes the global table; an expected
// group count up to kL1MaxGroups (use_l1) puts the on-chip level in front.
template <typename V, typename M>
int nest_impl(gbj_ctx *ctx, const int64_t *d_keys, const V *d_vals, uint64_t n, uint64_t groups, bool use_l1,
              uint64_t expected_groups, int64_t *d_out_keys, int64_t *d_out_count, int64_t *d_out_sum,
              M *d_out_min, M *d_out_max, uint64_t out_capacity, uint64_t *d_n_groups, cudaStream_t s) {
  Scratch scratch(ctx, s);
  Table64 t;
  GBJ_TRY(make_table(ctx, scratch, next_pow2(2 * groups), d_vals != nullptr, s, &t));
  if (use_l1) {
    // few groups: the on-chip level first (tables at 8 x groups)
    const uint32_t tslots =
        (uint32_t)std::min<uint64_t>(kL1MaxSlots, std::max<uint64_t>(64, next_pow2(8 * expected_groups)));
    uint32_t rlog = 0;  // as many accumulator columns (<= 32) as the budget allows
    while (rlog < 5 && (size_t)tslots * l1_slot_bytes(rlog + 1) <= kL1Budget) ++rlog;
    const size_t smem = (size_t)tslots * l1_slot_bytes(rlog);
    unsigned long long *ctr;
    GBJ_TRY(scratch.get(1, &ctr));
    GBJ_CHECK_CUDA(ctx, cudaMemsetAsync(ctr, 0, sizeof(unsigned long long), s));
    auto kern = k_nest_l1<V>;
    GBJ_CHECK_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 1;
    GBJ_CHECK_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kL1Threads, smem));
    per_sm = std::max(per_sm, 1);
    kern<<<ctx->sm_count * per_sm, kL1Threads, smem, s>>>(d_keys, d_vals, n, tslots, rlog, t, ctr, ctx->d_status);
    GBJ_TRY(after_launch(ctx, "k_nest_l1", s));
  } else {
    k_nest_build<V><<<grid_for(ctx, n), kThreads, 0, s>>>(d_keys, d_vals, n, t, ctx->d_status);
    GBJ_TRY(after_launch(ctx, "k_nest_build", s));
  }
  k_nest_emit<M><<<grid_for(ctx, t.mask + 2), kThreads, 0, s>>>(
      t, d_vals != nullptr, d_out_keys, d_out_count, d_out_sum, d_out_min, d_out_max, out_capacity,
      reinterpret_cast<unsigned long long *>(d_n_groups), ctx->d_status);
  return after_launch(ctx, "k_nest_emit", s);
}

}  // namespace

extern "C" int gbj_nest_i64(gbj_ctx *ctx, const int64_t *d_keys, const int64_t *d_vals, uint64_t n,
                            uint64_t expected_groups, int64_t *d_out_keys, int64_t *d_out_count,
                            int64_t *d_out_sum, int64_t *d_out_min, int64_t *d_out_max, uint64_t out_capacity,
                            uint64_t *d_n_groups, void *stream) {
  if (!ctx) return GBJ_ERR_INVALID;
  if (!d_n_groups) return set_error(ctx, GBJ_ERR_INVALID, "nest_i64: null group count");
  if (n && !d_keys) return set_error(ctx, GBJ_ERR_INVALID, "nest_i64: null key column");
  if (n >= (1ull << 40)) return set_error(ctx, GBJ_ERR_INVALID, "nest_i64: n >= 2^40");
  cudaStream_t s = pick_stream(ctx, stream);
  prof_mark(ctx, s);
  GBJ_CHECK_CUDA(ctx, cudaMemsetAsync(d_n_groups, 0, sizeof(uint64_t), s));
  if (n == 0) return GBJ_OK;
  const uint64_t groups = std::max<uint64_t>(1024, expected_groups ? std::min(expected_groups, n)
                                                                   : std::min<uint64_t>(n, 1ull << 24));
  return nest_impl<int64_t, int64_t>(ctx, d_keys, d_vals, n, groups,
                                     expected_groups && expected_groups <= kL1MaxGroups, expected_groups,
                                     d_out_keys, d_out_count, d_out_sum, d_out_min, d_out_max, out_capacity,
                                     d_n_groups, s);
}

extern "C" int gbj_groupby_i64(gbj_ctx *ctx, const int64_t *d_keys, const int32_t *d_values, uint64_t n,
                               const gbj_groupby_params *params, int64_t *d_out_keys, int64_t *d_out_count,
                               int64_t *d_out_sum, int32_t *d_out_min, int32_t *d_out_max, uint64_t out_capacity,
                               uint64_t *d_n_groups, void *stream) {
  if (!ctx || !d_n_groups) return GBJ_ERR_INVALID;
  if (n && (!d_keys || !d_values)) return set_error(ctx, GBJ_ERR_INVALID, "groupby_i64: null column");
  if (n >= (1ULL << 31)) return set_error(ctx, GBJ_ERR_INVALID, "groupby_i64: n >= 2^31");
  uint64_t hint = 0;
  int32_t hash_bits = 0;
  int strategy = 0;
  if (params) {
    hint = params->expected_groups ? params->expected_groups : params->max_input_size;
    hash_bits = params->hash_bits;
    strategy = params->strategy;
  }
  if (hash_bits < 0 || hash_bits > 32) return set_error(ctx, GBJ_ERR_INVALID, "groupby_i64: bad hash_bits");
  if (strategy < 0 || strategy > 2) return set_error(ctx, GBJ_ERR_INVALID, "groupby_i64: bad strategy");
  if (strategy == 2)
    return set_error(ctx, GBJ_ERR_UNSUPPORTED, "groupby_i64: no radix-partitioned strategy for int64 keys");
  cudaStream_t s = pick_stream(ctx, stream);
  prof_mark(ctx, s);
  GBJ_CHECK_CUDA(ctx, cudaMemsetAsync(d_n_groups, 0, sizeof(uint64_t), s));
  if (n == 0) return GBJ_OK;
  uint64_t groups = std::max<uint64_t>(1024, hint ? std::min(hint, n) : std::min<uint64_t>(n, 1ull << 24));
  if (hash_bits) groups = std::max<uint64_t>(groups, (1ULL << hash_bits) / 2);  // the table holds 2^hash_bits slots
  return nest_impl<int32_t, int32_t>(ctx, d_keys, d_values, n, groups, hint && hint <= kL1MaxGroups, hint,
                                     d_out_keys, d_out_count, d_out_sum, d_out_min, d_out_max, out_capacity,
                                     d_n_groups, s);
}

extern "C" int gbj_radix_join_count_i64(gbj_ctx *ctx, const int64_t *d_r_keys, uint64_t nr,
                                        const int64_t *d_s_keys, uint64_t ns, int64_t *d_count, void *stream) {
  if (!ctx) return GBJ_ERR_INVALID;
  if (!d_count) return set_error(ctx, GBJ_ERR_INVALID, "join_count_i64: null output");
  if ((nr && !d_r_keys) || (ns && !d_s_keys)) return set_error(ctx, GBJ_ERR_INVALID, "join_count_i64: null key column");
  if (nr >= (1ull << 40) || ns >= (1ull << 40)) return set_error(ctx, GBJ_ERR_INVALID, "join_count_i64: n >= 2^40");
  cudaStream_t s = pick_stream(ctx, stream);
  prof_mark(ctx, s);
  GBJ_CHECK_CUDA(ctx, cudaMemsetAsync(d_count, 0, sizeof(int64_t), s));
  if (nr == 0 || ns == 0) return GBJ_OK;
  Scratch scratch(ctx, s);
  Table64 t;
  GBJ_TRY(make_table(ctx, scratch, next_pow2(std::max<uint64_t>(2 * nr, 1024)), false, s, &t));
  k_nest_build<int64_t><<<grid_for(ctx, nr), kThreads, 0, s>>>(d_r_keys, nullptr, nr, t, ctx->d_status);
  GBJ_TRY(after_launch(ctx, "k_nest_build", s));
  k_join_count_probe<<<grid_for(ctx, ns), kThreads, 0, s>>>(d_s_keys, ns, t,
                                                            reinterpret_cast<unsigned long long *>(d_count));
  return after_launch(ctx, "k_join_count_probe", s);
}
