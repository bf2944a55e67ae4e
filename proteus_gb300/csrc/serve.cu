// Query serving: a request loop that admits join + group-by queries by HBM
// budget and runs each admitted group as one batch of persistent kernels.
//
// Stands in for the reference's per-query GPU execution: HashJoinChained
// build/probe (core/olap/lib/operators/hash-join-chained.cpp:262-566,
// gpu/gpu-hash-join-chained.cpp:31-73) feeding HashGroupByChained
// (hash-group-by-chained.cpp:267-853), with tables allocated per query by
// MemoryManager / buffer_manager (core/platform/lib/memory/) and a stream
// sync after each GPU operator.
//
// GB300 design:
//  * a batch is five launches over the work items of all its queries:
//    clear (table + group table), build, probe + group-by, emit, finish.
//    Each kernel is a persistent grid that takes items from one atomic
//    counter; an item is a fixed-size chunk of one query's rows or slots,
//    so big and small queries share the SMs without per-query launches;
//  * the join table is open addressing with one 64-bit slot per build row
//    holding {key | group slot << 32} (load factor <= 0.5), and duplicate
//    build keys keep HashJoinChained's every-match semantics.  A slot whose
//    key half is INT32_MIN is empty; build rows with that key go to a side
//    list that probes of INT32_MIN walk;
//  * each build row's group is resolved to its group-table slot at build
//    time and stored in its join-table entry, so a probe match adds to a
//    known slot: in a shared-memory array indexed by slot (flushed once per
//    work item) when the group table has at most 2048 slots, else straight
//    to the global slot;
//  * each in-flight slot owns a stream, a pinned descriptor, device
//    counters and (with use_graph) a CUDA graph of the whole batch, so
//    replaying a batch costs one graph launch; slots overlap on the device;
//  * a dispatcher thread completes batches (event polling), releases their
//    tables to the resident pool and launches the next batch from the FIFO
//    as soon as a slot and budget are free (continuous batching).
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <thread>
#include <vector>

#include "gbj_internal.cuh"

using namespace gbj;

namespace {

constexpr int kMaxB = GBJ_SERVE_MAX_BATCH;
constexpr int kMaxSlots = 8;
// Work-item sizes per phase: a query is cut into about 8 items per SM,
// within these bounds, so a query running alone still spreads over the
// whole GPU and a big one does not hold a CTA for long.
constexpr uint64_t kChunkMin[4] = {1u << 12, 1u << 8, 1u << 11, 1u << 10};
constexpr uint64_t kChunkMax[4] = {1u << 16, 1u << 15, 1u << 16, 1u << 14};
constexpr int kThreads = 256;
constexpr int kProbeThreads = 512;
constexpr int kL1 = 2048;  // shared-memory group slots per probe CTA
constexpr uint32_t kFlip = 0x80000000u;
constexpr unsigned long long kEmptySlot = 0x80000000ull;  // key half INT32_MIN, group 0
// clear phase: join table, group keys, per-query group counters
enum : int32_t { kClearTable = 1, kClearKeys = 2, kClearCounts = 4 };

enum { kPhClear = 0, kPhBuild = 1, kPhProbe = 2, kPhEmit = 3, kPhases = 4 };

// One query of a batch as the kernels read it.
struct SQ {
  const int32_t *bk, *bg, *pk, *pv;
  uint64_t nb, np;
  unsigned long long *table;
  uint64_t tmask;  // join table slots - 1
  int32_t *side;   // groups of build rows whose key is INT32_MIN
  unsigned long long *side_n;  // its length (per batch slot, or kept with a resident table)
  int32_t use_l1;  // pre-aggregate in shared memory
  int32_t clear_mode;  // kClear* bits: what the clear phase resets
  uint32_t *gkey;  // group table: key' (0 empty); slot gmask + 1 = INT32_MIN
  unsigned long long *gcnt, *gsum;
  uint64_t gmask;
  int32_t *out_g;
  int64_t *out_c, *out_s;
  uint64_t *out_n;
  uint64_t out_cap;
  uint64_t item0[kPhases];  // first item of this query in each phase
  uint64_t chunk[kPhases];  // rows or slots per item in each phase
  uint64_t clear_t_items;   // clear items that cover the join table
};

struct SBatch {
  int32_t nq;
  int32_t pad;
  uint64_t items[kPhases];
  SQ q[kMaxB];
};

// Per-slot device state, zeroed at the start of every batch.
struct SlotDev {
  unsigned long long ctr[kPhases + 1];
  unsigned long long dcount[kMaxB];  // groups emitted per query
  unsigned long long side_n[kMaxB];  // side-list lengths
  uint32_t status[kMaxB];            // GBJ_DEV_* bits per query
};

// Item -> query of a phase (binary search over the batch's prefix sums).
__device__ __forceinline__ int item_query(const uint64_t *s_item0, int nq, uint64_t item) {
  int a = 0, b = nq;
  while (b - a > 1) {
    const int mid = (a + b) >> 1;
    if (s_item0[mid] <= item) a = mid; else b = mid;
  }
  return a;
}

// Shared prologue: loads the phase's item offsets into shared memory.
__device__ __forceinline__ int load_item0(const SBatch *__restrict__ d, int ph, uint64_t *s_item0) {
  const int nq = d->nq;
  for (int q = threadIdx.x; q < nq; q += blockDim.x) s_item0[q] = d->q[q].item0[ph];
  return nq;
}

// Next item for the CTA (thread 0 draws, everyone reads after the barrier).
__device__ __forceinline__ uint64_t next_item(unsigned long long *ctr, unsigned long long *s_it) {
  __syncthreads();
  if (threadIdx.x == 0) *s_it = atomicAdd(ctr, 1ull);
  __syncthreads();
  return *s_it;
}

__global__ void __launch_bounds__(kThreads) k_serve_clear(const SBatch *__restrict__ d, SlotDev *slot) {
  __shared__ uint64_t s_item0[kMaxB];
  __shared__ unsigned long long s_it;
  const int nq = load_item0(d, kPhClear, s_item0);
  const uint64_t total = d->items[kPhClear];
  for (;;) {
    const uint64_t it = next_item(&slot->ctr[kPhClear], &s_it);
    if (it >= total) break;
    const SQ q = d->q[item_query(s_item0, nq, it)];  // by value: registers, not reloads
    const uint64_t local = it - q.item0[kPhClear];
    if (local < q.clear_t_items) {
      const uint64_t lo = local * q.chunk[kPhClear], hi = min(lo + q.chunk[kPhClear], q.tmask + 1);
      for (uint64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) q.table[i] = kEmptySlot;
    } else {
      const uint64_t lo = (local - q.clear_t_items) * q.chunk[kPhClear];
      const uint64_t hi = min(lo + q.chunk[kPhClear], q.gmask + 2);
      for (uint64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        if (q.clear_mode & kClearKeys) q.gkey[i] = 0u;
        if (q.clear_mode & kClearCounts) {
          q.gcnt[i] = 0ull;
          q.gsum[i] = 0ull;
        }
      }
    }
  }
}

// Slot of group g in the query's group table, claimed when new; INT32_MIN
// has the dedicated slot gmask + 1.  Returns -1 when the table is full.
__device__ __forceinline__ int64_t g_claim(const SQ &q, int32_t g) {
  if (g == INT32_MIN) return (int64_t)(q.gmask + 1);
  const uint32_t kk = (uint32_t)g ^ kFlip;
  uint64_t h = gbjd::fmix32((uint32_t)g) & q.gmask;
  for (uint64_t step = 0; step <= q.gmask; ++step) {
    uint32_t cur = *(volatile uint32_t *)&q.gkey[h];
    if (cur == 0) cur = atomicCAS(&q.gkey[h], 0u, kk);
    if (cur == 0 || cur == kk) return (int64_t)h;
    h = (h + 1) & q.gmask;
  }
  return -1;
}

// Build: each row's group is resolved to its group-table slot here, once,
// and the join table stores {key | slot << 32}; a probe match then adds to
// a known slot with no further lookup.
// With a small group table (use_l1) each CTA mirrors it in shared memory:
// an entry of the mirror sits at the same index as in the global table, so
// a mirror hit gives the global slot and only misses go to L2 (few groups
// would otherwise make every build row load the same few L2 addresses).
__global__ void __launch_bounds__(kThreads) k_serve_build(const SBatch *__restrict__ d, SlotDev *slot) {
  __shared__ uint64_t s_item0[kMaxB];
  __shared__ unsigned long long s_it;
  __shared__ uint32_t s_gkey[kL1];
  const int nq = load_item0(d, kPhBuild, s_item0);
  const uint64_t total = d->items[kPhBuild];
  for (;;) {
    const uint64_t it = next_item(&slot->ctr[kPhBuild], &s_it);
    if (it >= total) break;
    const int qi = item_query(s_item0, nq, it);
    const SQ q = d->q[qi];  // by value: registers, not reloads after atomics
    const uint64_t lo = (it - q.item0[kPhBuild]) * q.chunk[kPhBuild], hi = min(lo + q.chunk[kPhBuild], q.nb);
    const bool mirror = q.use_l1 != 0;
    if (mirror) {
      for (uint64_t j = threadIdx.x; j <= q.gmask; j += blockDim.x) s_gkey[j] = 0;
      __syncthreads();
    }
    auto claim = [&](int32_t g) -> int64_t {
      if (mirror && g != INT32_MIN) {
        const uint32_t kk = (uint32_t)g ^ kFlip;
        uint64_t h = gbjd::fmix32((uint32_t)g) & q.gmask;
        for (uint64_t step = 0; step <= q.gmask; ++step) {
          const uint32_t cur = s_gkey[h];
          if (cur == kk) return (int64_t)h;
          if (cur == 0) break;
          h = (h + 1) & q.gmask;
        }
        const int64_t gs = g_claim(q, g);
        if (gs >= 0) s_gkey[gs] = kk;
        return gs;
      }
      return g_claim(q, g);
    };
    for (uint64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
      const int32_t k = __ldcs(q.bk + i);
      const int64_t gs = claim(__ldcs(q.bg + i));
      if (gs < 0) {  // more distinct groups than expected_groups allowed for
        gbjd::latch(&slot->status[qi], GBJ_DEV_GROUPS);
        continue;
      }
      if (k == INT32_MIN) {
        q.side[atomicAdd(q.side_n, 1ull)] = (int32_t)gs;
        continue;
      }
      const unsigned long long e = (unsigned long long)(uint32_t)k | ((unsigned long long)gs << 32);
      uint64_t h = gbjd::fmix32((uint32_t)k) & q.tmask;
      bool placed = false;
      for (uint64_t step = 0; step <= q.tmask; ++step) {
        if (atomicCAS(&q.table[h], kEmptySlot, e) == kEmptySlot) {
          placed = true;
          break;
        }
        h = (h + 1) & q.tmask;
      }
      if (!placed) gbjd::latch(&slot->status[qi], GBJ_DEV_CAPACITY);
    }
  }
}

// Probe + group-by.  With at most kL1 group slots the matches of an item
// accumulate in shared memory indexed by group slot and are flushed once
// per item; otherwise each match adds to the global group slot directly.
// The shared accumulators use 32-bit atomics only (64-bit shared atomics
// have no native form): a count, and the low / high 16 bits of the biased
// value v + 2^31 in l1_a / l1_b, exact for the first 65535 matches of a slot
// in an item; later matches (duplicate-heavy builds) add their value to the
// global 64-bit sum directly.
constexpr uint32_t kL1Exact = 65535;

__global__ void __launch_bounds__(kProbeThreads) k_serve_probe(const SBatch *__restrict__ d, SlotDev *slot) {
  __shared__ uint64_t s_item0[kMaxB];
  __shared__ unsigned long long s_it;
  __shared__ uint32_t l1_cnt[kL1];
  __shared__ uint32_t l1_a[kL1];
  __shared__ uint32_t l1_b[kL1];
  const int nq = load_item0(d, kPhProbe, s_item0);
  const uint64_t total = d->items[kPhProbe];
  for (int i = threadIdx.x; i < kL1; i += blockDim.x) {
    l1_cnt[i] = 0;
    l1_a[i] = 0;
    l1_b[i] = 0;
  }
  for (;;) {
    const uint64_t it = next_item(&slot->ctr[kPhProbe], &s_it);
    if (it >= total) break;
    const int qi = item_query(s_item0, nq, it);
    const SQ q = d->q[qi];  // by value: registers, not reloads after atomics
    const uint64_t lo = (it - q.item0[kPhProbe]) * q.chunk[kPhProbe], hi = min(lo + q.chunk[kPhProbe], q.np);
    const bool use_l1 = q.use_l1 != 0;
    const unsigned long long side_n = *q.side_n;
    auto add = [&](uint32_t gs, int32_t v) {
      if (use_l1) {
        if (atomicAdd(&l1_cnt[gs], 1u) < kL1Exact) {
          const uint32_t u = (uint32_t)v ^ kFlip;
          atomicAdd(&l1_a[gs], u & 0xffffu);
          atomicAdd(&l1_b[gs], u >> 16);
        } else {
          atomicAdd(&q.gsum[gs], (unsigned long long)(int64_t)v);
        }
      } else {
        atomicAdd(&q.gcnt[gs], 1ull);
        atomicAdd(&q.gsum[gs], (unsigned long long)(int64_t)v);
      }
    };
    for (uint64_t base = lo; base < hi; base += 4 * kProbeThreads) {
      int32_t k[4], v[4];
      uint64_t h[4];
      bool ok[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const uint64_t i = base + threadIdx.x + (uint64_t)u * kProbeThreads;
        ok[u] = i < hi;
        k[u] = ok[u] ? __ldcs(q.pk + i) : 0;
        v[u] = ok[u] ? __ldcs(q.pv + i) : 0;
        h[u] = gbjd::fmix32((uint32_t)k[u]) & q.tmask;
      }
      unsigned long long e[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) e[u] = ok[u] && k[u] != INT32_MIN ? __ldg(q.table + h[u]) : kEmptySlot;
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (ok[u] && k[u] == INT32_MIN)
          for (unsigned long long j = 0; j < side_n; ++j) add((uint32_t)q.side[j], v[u]);
        uint64_t hh = h[u];
        unsigned long long ee = e[u];
        for (uint64_t step = 0; (uint32_t)ee != kFlip && step <= q.tmask; ++step) {
          if ((uint32_t)ee == (uint32_t)k[u]) add((uint32_t)(ee >> 32), v[u]);
          hh = (hh + 1) & q.tmask;
          ee = __ldg(q.table + hh);
        }
      }
    }
    if (use_l1) {
      __syncthreads();
      for (uint64_t i = threadIdx.x; i <= q.gmask + 1; i += blockDim.x) {
        const uint32_t c = l1_cnt[i];
        if (c) {
          const uint64_t in_ab = c < kL1Exact ? c : kL1Exact;  // matches summed in a / b
          const int64_t sum = (int64_t)(((uint64_t)l1_b[i] << 16) + l1_a[i]) - (int64_t)in_ab * (int64_t)kFlip;
          atomicAdd(&q.gcnt[i], (unsigned long long)c);
          atomicAdd(&q.gsum[i], (unsigned long long)sum);
          l1_cnt[i] = 0;
          l1_a[i] = 0;
          l1_b[i] = 0;
        }
      }
    }
  }
}

__global__ void __launch_bounds__(kThreads) k_serve_emit(const SBatch *__restrict__ d, SlotDev *slot) {
  __shared__ uint64_t s_item0[kMaxB];
  __shared__ unsigned long long s_it;
  const int nq = load_item0(d, kPhEmit, s_item0);
  const uint64_t total = d->items[kPhEmit];
  const int lane = threadIdx.x & 31;
  for (;;) {
    const uint64_t it = next_item(&slot->ctr[kPhEmit], &s_it);
    if (it >= total) break;
    const int qi = item_query(s_item0, nq, it);
    const SQ q = d->q[qi];  // by value: registers, not reloads after atomics
    const uint64_t lo = (it - q.item0[kPhEmit]) * q.chunk[kPhEmit], hi = min(lo + q.chunk[kPhEmit], q.gmask + 2);
    for (uint64_t b0 = lo; b0 < hi; b0 += blockDim.x) {  // uniform trip count per warp
      const uint64_t i = b0 + threadIdx.x;
      bool occ = false;
      if (i < hi) occ = q.gcnt[i] != 0ull;  // groups with at least one match
      const unsigned b = __ballot_sync(0xffffffffu, occ);
      unsigned long long base = 0;
      if (lane == 0 && b) base = atomicAdd(&slot->dcount[qi], (unsigned long long)__popc(b));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (occ) {
        const uint64_t pos = base + __popc(b & ((1u << lane) - 1));
        if (pos < q.out_cap) {
          q.out_g[pos] = i <= q.gmask ? (int32_t)(q.gkey[i] ^ kFlip) : INT32_MIN;
          q.out_c[pos] = (int64_t)q.gcnt[i];
          q.out_s[pos] = (int64_t)q.gsum[i];
        } else {
          gbjd::latch(&slot->status[qi], GBJ_DEV_CAPACITY);
        }
      }
    }
  }
}

__global__ void k_serve_finish(const SBatch *__restrict__ d, SlotDev *slot) {
  for (int q = threadIdx.x; q < d->nq; q += blockDim.x) *d->q[q].out_n = slot->dcount[q];
}

struct QueryRec {
  gbj_serve_query q{};
  uint64_t bytes = 0;
  double t_sub = -1, t_launch = -1, t_done = -1;
  int32_t status = GBJ_OK;
  bool done = false;
  bool launched = false;
  int retries = 0;
  void *mem = nullptr;
};

struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t start = nullptr;  // before the batch's first operation (timing)
  cudaEvent_t done = nullptr;
  SBatch *h_desc = nullptr;    // pinned
  SBatch *d_desc = nullptr;    // pool
  SlotDev *d_slot = nullptr;   // pool
  uint32_t *h_status = nullptr;  // pinned [kMaxB]
  cudaGraphExec_t exec = nullptr;
  bool busy = false;
  bool large = false;  // serves the large-query queue
  std::vector<uint64_t> tickets;
  uint64_t bytes = 0;
  uint64_t items[kPhases] = {0, 0, 0, 0};
};

}  // namespace

// A registered build relation's join table, kept resident in the pool: the
// table, its group-key map (group slots) and the INT32_MIN side list.
struct ResTable {
  void *mem = nullptr;
  uint64_t bytes = 0;
  unsigned long long *table = nullptr;
  uint64_t tmask = 0;
  uint32_t *gkey = nullptr;
  uint64_t gmask = 0;
  int32_t *side = nullptr;
  unsigned long long *side_n = nullptr;
};

struct gbj_server {
  gbj_ctx *ctx = nullptr;
  std::map<uint64_t, ResTable> tables;
  uint64_t next_table = 1;
  gbj_server_params prm{};
  uint64_t budget = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<uint64_t> queue[2];  // [0] small (or all), [1] large
  std::vector<QueryRec> recs;  // index = ticket - 1
  Slot slots[kMaxSlots];
  int nslots = 0;
  uint64_t held = 0, peak = 0, completed = 0, batches = 0, retried = 0;
  double batch_ms = 0;  // device time of the completed batches, start to done
  bool stop = false;
  bool paused = false;  // gbj_server_pause: no new batches are launched
  std::thread th;
  std::chrono::steady_clock::time_point t0;
  int grid[kPhases] = {0, 0, 0, 0};

  double now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
};

namespace {

uint64_t table_slots(uint64_t nb) { return next_pow2(std::max<uint64_t>(2 * nb, 1024)); }
uint64_t group_slots(const gbj_serve_query &q) {
  uint64_t e = q.expected_groups ? q.expected_groups : std::min<uint64_t>(std::max<uint64_t>(q.n_build, 1), 1u << 20);
  return next_pow2(std::max<uint64_t>(2 * e, 64));
}
// Pool bytes of one query: join table + group table (+ its INT32_MIN slot)
// + side list; with a resident table only the group counters.
uint64_t query_bytes(const gbj_server *sv, const gbj_serve_query &q) {
  if (q.table_id) {
    const ResTable &t = sv->tables.at(q.table_id);
    return (t.gmask + 2) * 16 + 256;
  }
  const uint64_t gs = group_slots(q) + 1;
  return table_slots(q.n_build) * 8 + gs * (8 + 8 + 4) + q.n_build * 4 + 512;
}

// Work items of one query (clear, build, probe, emit) from its layout.
void size_items(gbj_ctx *ctx, SQ &q, uint64_t ts, uint64_t gs, uint64_t n_items[kPhases]) {
  const uint64_t clear_t = (q.clear_mode & kClearTable) ? ts : 0;
  const uint64_t work[kPhases] = {clear_t + gs + 1, q.nb, q.np, gs + 1};
  const uint64_t per = 8 * (uint64_t)ctx->sm_count;
  for (int ph = 0; ph < kPhases; ++ph)
    q.chunk[ph] = std::min(kChunkMax[ph], std::max(kChunkMin[ph], next_pow2((work[ph] + per - 1) / per)));
  auto div_up = [](uint64_t a, uint64_t b) { return (a + b - 1) / b; };
  q.clear_t_items = div_up(clear_t, q.chunk[kPhClear]);
  n_items[kPhClear] = q.clear_t_items + div_up(gs + 1, q.chunk[kPhClear]);
  n_items[kPhBuild] = div_up(q.nb, q.chunk[kPhBuild]);
  n_items[kPhProbe] = div_up(q.np, q.chunk[kPhProbe]);
  n_items[kPhEmit] = div_up(gs + 1, q.chunk[kPhEmit]);
}

int launched(gbj_ctx *ctx, const char *name, bool count) {
  if (count) ctx->launches.fetch_add(1, std::memory_order_relaxed);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(ctx, e, name);
  return GBJ_OK;
}

// The batch's work on the slot's stream (also what a graph captures;
// `persistent`: full persistent grids, as a captured graph needs).
int enqueue_batch(gbj_server *sv, Slot &sl, bool persistent) {
  const bool count = !persistent || !sv->prm.use_graph;
  gbj_ctx *ctx = sv->ctx;
  cudaStream_t s = sl.stream;
  GBJ_CHECK_CUDA(ctx, cudaMemcpyAsync(sl.d_desc, sl.h_desc, sizeof(SBatch), cudaMemcpyHostToDevice, s));
  GBJ_CHECK_CUDA(ctx, cudaMemsetAsync(sl.d_slot, 0, sizeof(SlotDev), s));
  // large slots: one CTA per work item, so the SMs free up item by item
  const uint64_t cap = sl.large ? (1ull << 24) : 0;
  auto g = [&](int ph) {
    if (persistent) return sv->grid[ph];
    const uint64_t lim = cap ? cap : (uint64_t)sv->grid[ph];
    return (int)std::max<uint64_t>(1, std::min<uint64_t>(sl.items[ph], lim));
  };
  k_serve_clear<<<g(kPhClear), kThreads, 0, s>>>(sl.d_desc, sl.d_slot);
  GBJ_TRY(launched(ctx, "k_serve_clear", count));
  k_serve_build<<<g(kPhBuild), kThreads, 0, s>>>(sl.d_desc, sl.d_slot);
  GBJ_TRY(launched(ctx, "k_serve_build", count));
  k_serve_probe<<<g(kPhProbe), kProbeThreads, 0, s>>>(sl.d_desc, sl.d_slot);
  GBJ_TRY(launched(ctx, "k_serve_probe", count));
  k_serve_emit<<<g(kPhEmit), kThreads, 0, s>>>(sl.d_desc, sl.d_slot);
  GBJ_TRY(launched(ctx, "k_serve_emit", count));
  k_serve_finish<<<1, kMaxB, 0, s>>>(sl.d_desc, sl.d_slot);
  GBJ_TRY(launched(ctx, "k_serve_finish", count));
  GBJ_CHECK_CUDA(ctx, cudaMemcpyAsync(sl.h_status, sl.d_slot->status, sizeof(uint32_t) * kMaxB,
                                      cudaMemcpyDeviceToHost, s));
  return GBJ_OK;
}

// Marks a query done and wakes its waiters.  Caller holds sv->mu.
void finish_query(gbj_server *sv, QueryRec &r, int32_t status, double t) {
  r.status = status;
  r.t_done = t;
  r.done = true;
  sv->completed++;
  sv->cv_done.notify_all();
}

uint64_t enqueue_rec(gbj_server *sv, uint64_t ticket);

// Completes the slot's batch (its event has fired).  Caller holds sv->mu.
// A query whose group table ran out of slots (expected_groups below its
// distinct build groups) is queued once more, sized for every build row
// being its own group, which cannot overflow; other failures complete it.
void complete_slot(gbj_server *sv, Slot &sl) {
  const double t = sv->now();
  float ms = 0;
  if (cudaEventElapsedTime(&ms, sl.start, sl.done) == cudaSuccess) sv->batch_ms += ms;
  else (void)cudaGetLastError();
  for (size_t i = 0; i < sl.tickets.size(); ++i) {
    QueryRec &r = sv->recs[sl.tickets[i] - 1];
    const uint32_t bits = sl.h_status[i];
    if (r.mem) pool_release(sv->ctx, r.mem, sl.stream);
    r.mem = nullptr;
    if (bits == GBJ_DEV_GROUPS && r.retries == 0 && !r.q.table_id &&
        r.q.expected_groups < std::max<uint64_t>(r.q.n_build, 1) && !sv->stop) {
      r.retries = 1;
      r.launched = false;
      r.q.expected_groups = std::max<uint64_t>(r.q.n_build, 1);
      r.bytes = query_bytes(sv, r.q);
      sv->retried++;
      enqueue_rec(sv, sl.tickets[i]);
      continue;
    }
    const int32_t st = bits & (GBJ_DEV_CAPACITY | GBJ_DEV_GROUPS) ? GBJ_ERR_CAPACITY
                       : bits & GBJ_DEV_TIMEOUT ? GBJ_ERR_TIMEOUT
                       : bits ? GBJ_ERR_INVALID : GBJ_OK;
    finish_query(sv, r, st, t);
  }
  sv->held -= sl.bytes;
  sl.bytes = 0;
  sl.tickets.clear();
  sl.busy = false;
}

// Forms and launches one batch on a free slot.  Returns true if it launched.
bool launch_batch(gbj_server *sv, Slot &sl) {
  gbj_ctx *ctx = sv->ctx;
  SBatch *b = sl.h_desc;
  std::vector<uint64_t> take;
  uint64_t bytes = 0;
  std::deque<uint64_t> &queue = sv->queue[sl.large ? 1 : 0];
  while (!queue.empty() && (int)take.size() < sv->prm.max_batch) {
    const uint64_t t = queue.front();
    QueryRec &r = sv->recs[t - 1];
    if (r.bytes > sv->budget) {  // can never be admitted
      queue.pop_front();
      finish_query(sv, r, GBJ_ERR_BUDGET, sv->now());
      continue;
    }
    if (sv->held + bytes + r.bytes > sv->budget) break;
    void *mem = nullptr;
    if (pool_alloc(ctx, r.bytes, sl.stream, &mem) != GBJ_OK) break;  // pool busy: retry later
    r.mem = mem;
    r.launched = true;
    take.push_back(t);
    bytes += r.bytes;
    queue.pop_front();
  }
  if (take.empty()) return false;
  std::memset(b, 0, sizeof(SBatch));
  b->nq = (int32_t)take.size();
  uint64_t items[kPhases] = {0, 0, 0, 0};
  for (size_t i = 0; i < take.size(); ++i) {
    QueryRec &r = sv->recs[take[i] - 1];
    const gbj_serve_query &u = r.q;
    SQ &q = b->q[i];
    char *p = static_cast<char *>(r.mem);
    uint64_t ts = 0, gs = 0;
    if (u.table_id) {  // resident table: only this query's group counters are fresh
      const ResTable &t = sv->tables.at(u.table_id);
      ts = t.tmask + 1;
      gs = t.gmask + 1;
      q.table = t.table;
      q.gkey = t.gkey;
      q.side = t.side;
      q.side_n = t.side_n;
      q.gcnt = reinterpret_cast<unsigned long long *>(p);
      q.gsum = q.gcnt + (gs + 1);
      q.nb = 0;
      q.clear_mode = kClearCounts;
    } else {
      ts = table_slots(u.n_build);
      gs = group_slots(u);
      q.table = reinterpret_cast<unsigned long long *>(p);
      q.gcnt = reinterpret_cast<unsigned long long *>(p + ts * 8);
      q.gsum = q.gcnt + (gs + 1);
      q.gkey = reinterpret_cast<uint32_t *>(q.gsum + (gs + 1));
      q.side = reinterpret_cast<int32_t *>(q.gkey + (gs + 1));
      q.side_n = &sl.d_slot->side_n[i];
      q.nb = u.n_build;
      q.clear_mode = kClearTable | kClearKeys | kClearCounts;
    }
    q.use_l1 = gs + 1 <= (uint64_t)kL1 ? 1 : 0;
    q.tmask = ts - 1;
    q.gmask = gs - 1;
    q.bk = u.d_build_keys;
    q.bg = u.d_build_group;
    q.pk = u.d_probe_keys;
    q.pv = u.d_probe_vals;
    q.np = u.n_probe;
    q.out_g = u.out_group;
    q.out_c = u.out_count;
    q.out_s = u.out_sum;
    q.out_n = u.out_n_groups;
    q.out_cap = u.out_capacity;
    uint64_t n_items[kPhases];
    size_items(ctx, q, ts, gs, n_items);
    for (int ph = 0; ph < kPhases; ++ph) {
      q.item0[ph] = items[ph];
      items[ph] += n_items[ph];
    }
    r.t_launch = sv->now();
  }
  for (int ph = 0; ph < kPhases; ++ph) {
    b->items[ph] = items[ph];
    sl.items[ph] = items[ph];
  }
  int rc = GBJ_OK;
  if (cudaEventRecord(sl.start, sl.stream) != cudaSuccess) rc = cuda_error(ctx, cudaGetLastError(), "cudaEventRecord");
  if (rc == GBJ_OK && sv->prm.use_graph && !sl.large) {
    if (!sl.exec) {
      cudaError_t e = cudaStreamBeginCapture(sl.stream, cudaStreamCaptureModeThreadLocal);
      if (e != cudaSuccess) rc = cuda_error(ctx, e, "cudaStreamBeginCapture");
      if (rc == GBJ_OK) {
        rc = enqueue_batch(sv, sl, true);
        cudaGraph_t graph = nullptr;
        e = cudaStreamEndCapture(sl.stream, &graph);
        if (rc == GBJ_OK && e != cudaSuccess) rc = cuda_error(ctx, e, "cudaStreamEndCapture");
        if (rc == GBJ_OK) {
          e = cudaGraphInstantiate(&sl.exec, graph, 0);
          if (e != cudaSuccess) {
            sl.exec = nullptr;
            rc = cuda_error(ctx, e, "cudaGraphInstantiate");
          }
        }
        if (graph) cudaGraphDestroy(graph);
      }
    }
    if (rc == GBJ_OK) {
      const cudaError_t e = cudaGraphLaunch(sl.exec, sl.stream);
      if (e != cudaSuccess) rc = cuda_error(ctx, e, "cudaGraphLaunch");
      // the launches were counted at capture; count the replay's kernels
      else ctx->launches.fetch_add(5, std::memory_order_relaxed);
    }
  } else if (rc == GBJ_OK) {
    rc = enqueue_batch(sv, sl, false);
  }
  if (rc == GBJ_OK) {
    const cudaError_t e = cudaEventRecord(sl.done, sl.stream);
    if (e != cudaSuccess) rc = cuda_error(ctx, e, "cudaEventRecord");
  }
  if (rc != GBJ_OK) {
    // nothing usable was enqueued: fail the batch's queries
    cudaStreamSynchronize(sl.stream);
    for (uint64_t t : take) {
      QueryRec &r = sv->recs[t - 1];
      if (r.mem) pool_release(ctx, r.mem, sl.stream);
      r.mem = nullptr;
      finish_query(sv, r, rc, sv->now());
    }
    sv->cv_done.notify_all();
    return false;
  }
  sl.tickets = std::move(take);
  sl.bytes = bytes;
  sl.busy = true;
  sv->held += bytes;
  sv->peak = std::max(sv->peak, sv->held);
  sv->batches++;
  return true;
}

void dispatcher(gbj_server *sv) {
  cudaSetDevice(sv->ctx->device);
  std::unique_lock<std::mutex> lk(sv->mu);
  for (;;) {
    bool progressed = false, busy = false;
    for (int i = 0; i < sv->nslots; ++i) {
      Slot &sl = sv->slots[i];
      if (sl.busy && cudaEventQuery(sl.done) == cudaSuccess) {
        complete_slot(sv, sl);
        progressed = true;
      }
    }
    if (progressed) sv->cv_done.notify_all();
    for (int i = 0; i < sv->nslots && !sv->paused; ++i) {
      Slot &sl = sv->slots[i];
      if (!sl.busy && !sv->queue[sl.large ? 1 : 0].empty() && launch_batch(sv, sl)) progressed = true;
    }
    for (int i = 0; i < sv->nslots; ++i) busy = busy || sv->slots[i].busy;
    const bool queued = !sv->queue[0].empty() || !sv->queue[1].empty();
    if (!busy && queued && !progressed && !sv->paused) {
      // nothing in flight and a head query still does not fit the pool
      std::deque<uint64_t> &qq = sv->queue[sv->queue[0].empty() ? 1 : 0];
      QueryRec &r = sv->recs[qq.front() - 1];
      qq.pop_front();
      finish_query(sv, r, GBJ_ERR_OOM, sv->now());
      sv->cv_done.notify_all();
      continue;
    }
    if (sv->stop && !queued && !busy) break;
    if (busy) {
      lk.unlock();
      std::this_thread::yield();
      lk.lock();
      continue;
    }
    sv->cv_work.wait(lk, [&] {
      return sv->stop || (!sv->paused && (!sv->queue[0].empty() || !sv->queue[1].empty()));
    });
  }
}

void free_slots(gbj_server *sv) {
  for (int i = 0; i < kMaxSlots; ++i) {
    Slot &sl = sv->slots[i];
    if (sl.exec) cudaGraphExecDestroy(sl.exec);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.start) cudaEventDestroy(sl.start);
    if (sl.h_desc) cudaFreeHost(sl.h_desc);
    if (sl.h_status) cudaFreeHost(sl.h_status);
    if (sl.d_desc) pool_release(sv->ctx, sl.d_desc, sl.stream);
    if (sl.d_slot) pool_release(sv->ctx, sl.d_slot, sl.stream);
    if (sl.stream) cudaStreamDestroy(sl.stream);
    sl = Slot();
  }
}

}  // namespace

extern "C" int gbj_server_create(gbj_ctx *ctx, const gbj_server_params *params, gbj_server **out) {
  if (!ctx || !out) return GBJ_ERR_INVALID;
  *out = nullptr;
  gbj_server_params prm{0, kMaxB, 2, 1, 0, 0};
  if (params) prm = *params;
  if (prm.small_rows == 0) prm.small_rows = 1ull << 22;
  if (prm.large_slots < 0 || prm.large_slots >= std::max(prm.max_inflight, 1))
    return set_error(ctx, GBJ_ERR_INVALID, "server: large_slots must leave at least one slot");
  if (prm.max_batch < 1 || prm.max_batch > kMaxB)
    return set_error(ctx, GBJ_ERR_INVALID, "server: max_batch must be 1..64");
  if (prm.max_inflight < 1 || prm.max_inflight > kMaxSlots)
    return set_error(ctx, GBJ_ERR_INVALID, "server: max_inflight must be 1..8");
  auto sv = new gbj_server();
  sv->ctx = ctx;
  sv->prm = prm;
  sv->budget = prm.hbm_budget ? prm.hbm_budget : ctx->pool.capacity;
  sv->nslots = prm.max_inflight;
  sv->t0 = std::chrono::steady_clock::now();
  auto fail = [&](int rc) {
    free_slots(sv);
    delete sv;
    return rc;
  };
  int prio_low = 0, prio_high = 0;  // numerically: greatest = lowest priority
  {
    const cudaError_t e = cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
    if (e != cudaSuccess) return fail(cuda_error(ctx, e, "cudaDeviceGetStreamPriorityRange"));
  }
  for (int i = 0; i < sv->nslots; ++i) {
    Slot &sl = sv->slots[i];
    sl.large = i >= sv->nslots - prm.large_slots;
    const int prio = prm.large_slots == 0 ? 0 : (sl.large ? prio_low : prio_high);
    cudaError_t e = cudaStreamCreateWithPriority(&sl.stream, cudaStreamNonBlocking, prio);
    if (e == cudaSuccess) e = cudaEventCreate(&sl.done);
    if (e == cudaSuccess) e = cudaEventCreate(&sl.start);
    if (e == cudaSuccess) e = cudaHostAlloc(reinterpret_cast<void **>(&sl.h_desc), sizeof(SBatch), cudaHostAllocDefault);
    if (e == cudaSuccess)
      e = cudaHostAlloc(reinterpret_cast<void **>(&sl.h_status), sizeof(uint32_t) * kMaxB, cudaHostAllocDefault);
    if (e != cudaSuccess) return fail(cuda_error(ctx, e, "server slot setup"));
    int rc = pool_alloc(ctx, sizeof(SBatch), sl.stream, reinterpret_cast<void **>(&sl.d_desc));
    if (rc == GBJ_OK) rc = pool_alloc(ctx, sizeof(SlotDev), sl.stream, reinterpret_cast<void **>(&sl.d_slot));
    if (rc != GBJ_OK) return fail(rc);
  }
  const void *kerns[kPhases] = {(const void *)k_serve_clear, (const void *)k_serve_build,
                                (const void *)k_serve_probe, (const void *)k_serve_emit};
  const int threads[kPhases] = {kThreads, kThreads, kProbeThreads, kThreads};
  for (int ph = 0; ph < kPhases; ++ph) {
    int per_sm = 1;
    const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kerns[ph], threads[ph], 0);
    if (e != cudaSuccess) return fail(cuda_error(ctx, e, "occupancy"));
    sv->grid[ph] = ctx->sm_count * std::max(per_sm, 1);
  }
  const cudaError_t e = cudaDeviceSynchronize();  // pool memory is ordered on the slot streams
  if (e != cudaSuccess) return fail(cuda_error(ctx, e, "cudaDeviceSynchronize"));
  sv->th = std::thread(dispatcher, sv);
  *out = sv;
  return GBJ_OK;
}

namespace {
int check_query(gbj_ctx *ctx, const gbj_serve_query *q) {
  if ((!q->table_id && q->n_build && (!q->d_build_keys || !q->d_build_group)) ||
      (q->n_probe && (!q->d_probe_keys || !q->d_probe_vals)))
    return set_error(ctx, GBJ_ERR_INVALID, "server: null input column");
  if (!q->out_group || !q->out_count || !q->out_sum || !q->out_n_groups || q->out_capacity == 0)
    return set_error(ctx, GBJ_ERR_INVALID, "server: null output or zero out_capacity");
  if (q->n_build >= (1ull << 31) || q->n_probe >= (1ull << 40))
    return set_error(ctx, GBJ_ERR_INVALID, "server: n_build must be < 2^31");
  return GBJ_OK;
}

// Puts a recorded query on its size class's queue.  Caller holds sv->mu.
uint64_t enqueue_rec(gbj_server *sv, uint64_t ticket) {
  const gbj_serve_query &q = sv->recs[ticket - 1].q;
  const uint64_t build_rows = q.table_id ? 0 : q.n_build;
  const bool large = sv->prm.large_slots > 0 && build_rows + q.n_probe > sv->prm.small_rows;
  sv->queue[large ? 1 : 0].push_back(ticket);
  return ticket;
}

// Queues one checked query.  Caller holds sv->mu.
uint64_t enqueue_query(gbj_server *sv, const gbj_serve_query *q, double t) {
  QueryRec r;
  r.q = *q;
  r.bytes = query_bytes(sv, *q);
  r.t_sub = t;
  sv->recs.push_back(r);
  return enqueue_rec(sv, sv->recs.size());
}
}  // namespace

extern "C" int gbj_server_submit(gbj_server *sv, const gbj_serve_query *q, uint64_t *ticket) {
  return gbj_server_submit_batch(sv, q, 1, ticket);
}

extern "C" int gbj_server_submit_batch(gbj_server *sv, const gbj_serve_query *qs, uint64_t n,
                                       uint64_t *tickets) {
  if (!sv || (n && (!qs || !tickets))) return GBJ_ERR_INVALID;
  for (uint64_t i = 0; i < n; ++i) GBJ_TRY(check_query(sv->ctx, &qs[i]));
  std::lock_guard<std::mutex> lk(sv->mu);
  if (sv->stop) return set_error(sv->ctx, GBJ_ERR_CANCELLED, "server: stopping");
  for (uint64_t i = 0; i < n; ++i)
    if (qs[i].table_id && !sv->tables.count(qs[i].table_id))
      return set_error(sv->ctx, GBJ_ERR_INVALID, "server: unknown table_id");
  const double t = sv->now();
  for (uint64_t i = 0; i < n; ++i) tickets[i] = enqueue_query(sv, &qs[i], t);
  sv->cv_work.notify_one();
  return GBJ_OK;
}

extern "C" int gbj_server_wait(gbj_server *sv, uint64_t ticket, double timeout_s, int32_t *status) {
  if (!sv) return GBJ_ERR_INVALID;
  std::unique_lock<std::mutex> lk(sv->mu);
  if (ticket == 0 || ticket > sv->recs.size()) return set_error(sv->ctx, GBJ_ERR_INVALID, "server: unknown ticket");
  auto ready = [&] { return sv->recs[ticket - 1].done; };
  if (timeout_s < 0) {
    sv->cv_done.wait(lk, ready);
  } else if (!sv->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), ready)) {
    return GBJ_ERR_TIMEOUT;
  }
  if (status) *status = sv->recs[ticket - 1].status;
  return GBJ_OK;
}

extern "C" int gbj_server_cancel(gbj_server *sv, uint64_t ticket, int32_t *cancelled) {
  if (!sv) return GBJ_ERR_INVALID;
  std::lock_guard<std::mutex> lk(sv->mu);
  if (ticket == 0 || ticket > sv->recs.size()) return set_error(sv->ctx, GBJ_ERR_INVALID, "server: unknown ticket");
  QueryRec &r = sv->recs[ticket - 1];
  bool hit = false;
  if (!r.done && !r.launched) {
    for (auto &qq : sv->queue) {
      auto it = std::find(qq.begin(), qq.end(), ticket);
      if (it != qq.end()) {
        qq.erase(it);
        hit = true;
        break;
      }
    }
    if (hit) finish_query(sv, r, GBJ_ERR_CANCELLED, sv->now());
  }
  if (cancelled) *cancelled = hit ? 1 : 0;
  return GBJ_OK;
}

extern "C" int gbj_server_pause(gbj_server *sv, int32_t paused) {
  if (!sv) return GBJ_ERR_INVALID;
  std::lock_guard<std::mutex> lk(sv->mu);
  sv->paused = paused != 0;
  sv->cv_work.notify_one();
  return GBJ_OK;
}

extern "C" int gbj_server_retries(gbj_server *sv, uint64_t *retried) {
  if (!sv || !retried) return GBJ_ERR_INVALID;
  std::lock_guard<std::mutex> lk(sv->mu);
  *retried = sv->retried;
  return GBJ_OK;
}

extern "C" int gbj_server_times(gbj_server *sv, uint64_t ticket, double *submitted, double *launched,
                                double *completed) {
  if (!sv) return GBJ_ERR_INVALID;
  std::lock_guard<std::mutex> lk(sv->mu);
  if (ticket == 0 || ticket > sv->recs.size()) return set_error(sv->ctx, GBJ_ERR_INVALID, "server: unknown ticket");
  const QueryRec &r = sv->recs[ticket - 1];
  if (submitted) *submitted = r.t_sub;
  if (launched) *launched = r.t_launch;
  if (completed) *completed = r.t_done;
  return GBJ_OK;
}

extern "C" int gbj_server_drain(gbj_server *sv) {
  if (!sv) return GBJ_ERR_INVALID;
  std::unique_lock<std::mutex> lk(sv->mu);
  sv->cv_done.wait(lk, [&] { return sv->completed == sv->recs.size(); });
  return GBJ_OK;
}

extern "C" int gbj_server_stats(gbj_server *sv, uint64_t *completed, uint64_t *batches, uint64_t *peak_bytes) {
  if (!sv) return GBJ_ERR_INVALID;
  std::lock_guard<std::mutex> lk(sv->mu);
  if (completed) *completed = sv->completed;
  if (batches) *batches = sv->batches;
  if (peak_bytes) *peak_bytes = sv->peak;
  return GBJ_OK;
}

extern "C" int gbj_server_busy(gbj_server *sv, double *batch_ms) {
  if (!sv || !batch_ms) return GBJ_ERR_INVALID;
  std::lock_guard<std::mutex> lk(sv->mu);
  *batch_ms = sv->batch_ms;
  return GBJ_OK;
}

extern "C" int gbj_server_destroy(gbj_server *sv) {
  if (!sv) return GBJ_ERR_INVALID;
  gbj_server_pause(sv, 0);  // queued queries run before the loop stops
  gbj_server_drain(sv);
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->stop = true;
  }
  sv->cv_work.notify_all();
  if (sv->th.joinable()) sv->th.join();
  for (int i = 0; i < sv->nslots; ++i) cudaStreamSynchronize(sv->slots[i].stream);
  free_slots(sv);
  // resident tables still registered go back to the pool
  for (auto &kv : sv->tables) pool_release(sv->ctx, kv.second.mem, sv->ctx->stream);
  sv->tables.clear();
  delete sv;
  return GBJ_OK;
}

// One registration attempt; *dev_status gets the build's device status bits.
static int register_table_once(gbj_server *sv, const int32_t *d_build_keys, const int32_t *d_build_group,
                               uint64_t n_build, uint64_t expected_groups, uint64_t *table_id,
                               uint32_t *dev_status) {
  if (!sv || !table_id) return GBJ_ERR_INVALID;
  gbj_ctx *ctx = sv->ctx;
  if (n_build && (!d_build_keys || !d_build_group))
    return set_error(ctx, GBJ_ERR_INVALID, "server: null build column");
  if (n_build >= (1ull << 31)) return set_error(ctx, GBJ_ERR_INVALID, "server: n_build must be < 2^31");
  gbj_serve_query tmp{};
  tmp.n_build = n_build;
  tmp.expected_groups = expected_groups;
  const uint64_t ts = table_slots(n_build), gs = group_slots(tmp);
  const uint64_t bytes = ts * 8 + 64 + (gs + 1) * 4 + n_build * 4 + 64;
  std::lock_guard<std::mutex> lk(sv->mu);
  if (sv->held + bytes > sv->budget) return set_error(ctx, GBJ_ERR_BUDGET, "server: table does not fit the budget");
  cudaStream_t s = ctx->stream;
  ResTable t;
  GBJ_TRY(pool_alloc(ctx, bytes, s, &t.mem));
  char *p = static_cast<char *>(t.mem);
  t.bytes = bytes;
  t.table = reinterpret_cast<unsigned long long *>(p);
  t.side_n = reinterpret_cast<unsigned long long *>(p + ts * 8);
  t.gkey = reinterpret_cast<uint32_t *>(p + ts * 8 + 64);
  t.side = reinterpret_cast<int32_t *>(t.gkey + (gs + 1));
  t.tmask = ts - 1;
  t.gmask = gs - 1;
  // build with the batch kernels: one query, clear (table + keys) and build
  SBatch *h = new SBatch();
  std::memset(h, 0, sizeof(SBatch));
  h->nq = 1;
  SQ &q = h->q[0];
  q.table = t.table;
  q.tmask = t.tmask;
  q.gkey = t.gkey;
  q.gmask = t.gmask;
  q.side = t.side;
  q.side_n = t.side_n;
  q.bk = d_build_keys;
  q.bg = d_build_group;
  q.nb = n_build;
  q.use_l1 = gs + 1 <= (uint64_t)kL1 ? 1 : 0;
  q.clear_mode = kClearTable | kClearKeys;
  uint64_t n_items[kPhases];
  size_items(ctx, q, ts, gs, n_items);
  h->items[kPhClear] = n_items[kPhClear];
  h->items[kPhBuild] = n_items[kPhBuild];
  SBatch *d_desc = nullptr;
  SlotDev *d_slot = nullptr;
  int rc = pool_alloc(ctx, sizeof(SBatch), s, reinterpret_cast<void **>(&d_desc));
  if (rc == GBJ_OK) rc = pool_alloc(ctx, sizeof(SlotDev), s, reinterpret_cast<void **>(&d_slot));
  uint32_t status = 0;
  if (rc == GBJ_OK) {
    cudaMemcpyAsync(d_desc, h, sizeof(SBatch), cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(d_slot, 0, sizeof(SlotDev), s);
    cudaMemsetAsync(t.side_n, 0, sizeof(unsigned long long), s);
    auto g = [&](int ph) {
      return (int)std::max<uint64_t>(1, std::min<uint64_t>(n_items[ph], (uint64_t)sv->grid[ph]));
    };
    k_serve_clear<<<g(kPhClear), kThreads, 0, s>>>(d_desc, d_slot);
    rc = launched(ctx, "k_serve_clear", true);
    if (rc == GBJ_OK) {
      k_serve_build<<<g(kPhBuild), kThreads, 0, s>>>(d_desc, d_slot);
      rc = launched(ctx, "k_serve_build", true);
    }
    if (rc == GBJ_OK) {
      const cudaError_t e = cudaMemcpyAsync(&status, d_slot->status, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
      const cudaError_t e2 = cudaStreamSynchronize(s);
      if (e != cudaSuccess || e2 != cudaSuccess) rc = cuda_error(ctx, e != cudaSuccess ? e : e2, "server: build");
    }
  }
  delete h;
  if (d_desc) pool_release(ctx, d_desc, s);
  if (d_slot) pool_release(ctx, d_slot, s);
  *dev_status = status;
  if (rc == GBJ_OK && status) rc = set_error(ctx, GBJ_ERR_CAPACITY, "server: table build overflowed");
  if (rc != GBJ_OK) {
    pool_release(ctx, t.mem, s);
    return rc;
  }
  *table_id = sv->next_table++;
  sv->tables[*table_id] = t;
  sv->held += bytes;
  sv->peak = std::max(sv->peak, sv->held);
  return GBJ_OK;
}

// A build whose groups outnumber expected_groups is built once more with a
// group table for every build row being its own group.
extern "C" int gbj_server_register_table(gbj_server *sv, const int32_t *d_build_keys,
                                         const int32_t *d_build_group, uint64_t n_build,
                                         uint64_t expected_groups, uint64_t *table_id) {
  uint32_t bits = 0;
  const int rc = register_table_once(sv, d_build_keys, d_build_group, n_build, expected_groups, table_id, &bits);
  if (rc == GBJ_ERR_CAPACITY && bits == GBJ_DEV_GROUPS && expected_groups < n_build) {
    {
      std::lock_guard<std::mutex> lk(sv->mu);
      sv->retried++;
    }
    return register_table_once(sv, d_build_keys, d_build_group, n_build, n_build, table_id, &bits);
  }
  return rc;
}

extern "C" int gbj_server_unregister_table(gbj_server *sv, uint64_t table_id) {
  if (!sv) return GBJ_ERR_INVALID;
  gbj_server_drain(sv);  // no query may still read it
  std::lock_guard<std::mutex> lk(sv->mu);
  auto it = sv->tables.find(table_id);
  if (it == sv->tables.end()) return set_error(sv->ctx, GBJ_ERR_INVALID, "server: unknown table_id");
  pool_release(sv->ctx, it->second.mem, sv->ctx->stream);
  sv->held -= it->second.bytes;
  sv->tables.erase(it);
  return GBJ_OK;
}
