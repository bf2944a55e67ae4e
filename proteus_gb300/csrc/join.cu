// Non-partitioned hash join: build, probe with fused aggregate, probe with
// pair materialisation; plus the column helpers (reduce, gather, select).
//
// Replaces the JIT'd build / probe loops of HashJoinChained and
// GpuHashJoinChained (core/olap/lib/operators/hash-join-chained.cpp:262-566,
// core/olap/lib/operators/gpu/gpu-hash-join-chained.cpp:31-73).  The
// reference chains entries behind a head array; here the table is an array
// of 32-byte buckets of four slots (keys, then payloads or rows + 1) sized
// to a power of two with load factor <= 1/2, so a probe is one L2 sector in
// the common case and the table for a 2^20-row build side (16 MiB) stays
// resident in the 129 MB L2 while the probe side streams from HBM.  The
// allocation-free entry point keeps a plain open-addressing array of 64-bit
// {key, row + 1} slots in a static device array.
// Semantics are the reference's: every build row is inserted (duplicates
// allowed) and a probe row meets every build row with an equal key.
#include <cooperative_groups.h>

#include "compact.cuh"
#include "gbj_internal.cuh"
#include "scan.cuh"

namespace cg = cooperative_groups;
using namespace gbj;

namespace {

constexpr int kThreads = 512;

__device__ __forceinline__ uint64_t make_slot(int32_t key, uint64_t row) {
  return ((row + 1) << 32) | (uint32_t)key;
}

// Build of the allocation-free entry point's table: 64-bit slots {key,
// row + 1}, 0 = empty, linear probing; meta[0] = 1 once a duplicate build key
// was seen (probes may then not stop at the first match).  The table has at
// least 2n slots, so every row finds one.
__global__ void __launch_bounds__(kThreads)
    k_join_build(const int32_t *__restrict__ keys, uint64_t n, uint64_t *__restrict__ slots, uint64_t mask,
                 uint32_t *__restrict__ meta) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  bool dup = false;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    const int32_t k = keys[i];
    const uint64_t entry = make_slot(k, i);
    uint64_t h = gbjd::fmix32((uint32_t)k) & mask;
    for (uint64_t probe = 0; probe <= mask; ++probe) {
      unsigned long long *w = reinterpret_cast<unsigned long long *>(slots) + h;
      uint64_t cur = *(volatile uint64_t *)w;
      if (cur == 0) {
        cur = atomicCAS(w, 0ull, (unsigned long long)entry);
        if (cur == 0) break;
      }
      dup |= ((int32_t)(uint32_t)cur == k);
      h = (h + 1) & mask;
    }
  }
  if (dup) meta[0] = 1;
}

enum : int { kAggGeneric = 0, kAggCountXor = 1, kAggCountProduct = 2 };

// Probe with fused aggregate over the allocation-free entry point's table.
// Eight probe keys per thread walk their slot chains in lockstep: every
// round checks the slot each still-open probe holds and issues the next
// slot loads of all of them together, so a warp waits for the longest chain
// once per round instead of once per probe and keeps up to eight L2
// requests per thread in flight.  kAgg selects a specialised accumulator
// for the two aggregate lists the workloads use.
template <bool kVec, int kAgg>
__global__ void __launch_bounds__(kThreads)
    k_join_probe_agg(const int32_t *__restrict__ keys, const int32_t *__restrict__ pay, uint64_t n,
                     const uint64_t *__restrict__ slots, uint64_t mask, const int32_t *__restrict__ bpay,
                     const uint32_t *__restrict__ meta, gbj::AggSpec spec, int64_t *out) {
  __shared__ int64_t red[32 * GBJ_MAX_AGGS];
  gbjd::Acc acc;
  acc.init(spec);
  int64_t a_cnt = 0, a_sum = 0;
  const bool unique = meta[0] == 0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  // a slot is {key (low word), row + 1 (high word)}; row + 1 == 0: empty
  auto skey = [](uint64_t e) { return (int32_t)(uint32_t)e; };
  auto srow1 = [](uint64_t e) { return (uint32_t)(e >> 32); };
  auto match = [&](int32_t k, int64_t pv, uint64_t prow, uint64_t e) {
    const uint32_t r = srow1(e) - 1;
    if (kAgg == kAggCountXor) {
      a_cnt += 1;
      a_sum += (int64_t)r ^ (int64_t)prow;
    } else {
      const int64_t bv = bpay ? (int64_t)__ldg(&bpay[r]) : 0;
      if (kAgg == kAggCountProduct) {
        a_cnt += 1;
        a_sum += bv * pv;
      } else {
        acc.update(spec, k, bv, pv, r, prow);
      }
    }
  };
  uint64_t done = 0;
  if (kVec) {
    const uint64_t n8 = n / 8;
    const int4 *k4 = reinterpret_cast<const int4 *>(keys);
    const int4 *p4 = reinterpret_cast<const int4 *>(pay);
    for (uint64_t q = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; q < n8; q += stride) {
      const int4 ka = __ldcs(k4 + 2 * q), kb = __ldcs(k4 + 2 * q + 1);
      int4 pa = make_int4(0, 0, 0, 0), pb = pa;
      if (pay) {
        pa = __ldcs(p4 + 2 * q);
        pb = __ldcs(p4 + 2 * q + 1);
      }
      const int32_t kk[8] = {ka.x, ka.y, ka.z, ka.w, kb.x, kb.y, kb.z, kb.w};
      const int32_t pp[8] = {pa.x, pa.y, pa.z, pa.w, pb.x, pb.y, pb.z, pb.w};
      // slot indices fit 32 bits: the table holds at most 2^21 slots
      const uint32_t m32 = (uint32_t)mask;
      uint32_t h[8];
      uint64_t e[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        h[j] = gbjd::fmix32((uint32_t)kk[j]) & m32;
        e[j] = __ldg(slots + h[j]);
      }
      uint32_t open = 0xffu;  // probes whose chain is not finished
      for (uint64_t step = 0; open && step <= mask; ++step) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          if (open >> j & 1u) {
            if (srow1(e[j]) == 0) {
              open &= ~(1u << j);
            } else if (skey(e[j]) == kk[j]) {
              match(kk[j], pp[j], q * 8 + j, e[j]);
              if (unique) open &= ~(1u << j);
            }
          }
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          if (open >> j & 1u) {
            h[j] = (h[j] + 1) & m32;
            e[j] = __ldg(slots + h[j]);
          }
        }
      }
    }
    done = n8 * 8;
  }
  // rows the vector loop did not cover (all of them without kVec)
  for (uint64_t i = done + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    const int32_t k = keys[i];
    const int64_t pv = pay ? pay[i] : 0;
    uint64_t h = gbjd::fmix32((uint32_t)k) & mask;
    for (uint64_t step = 0; step <= mask; ++step) {
      const uint64_t e = __ldg(slots + h);
      if (srow1(e) == 0) break;
      if (skey(e) == k) {
        match(k, pv, i, e);
        if (unique) break;
      }
      h = (h + 1) & mask;
    }
  }
  if (kAgg != kAggGeneric) {
    acc.v[0] = a_cnt;
    acc.v[1] = a_sum;
  }
  gbjd::block_flush(spec, acc, red, out);
}

// ------------------------------------------------ bucketed join table
// The table gbj_join_build makes: buckets of four slots, 32 bytes each --
// four keys then four values (the build payload, or row + 1 when the build
// side has none) -- so a probe reads one L2 sector per bucket and finds the
// key and its payload without a second, dependent load.  Keys are stored
// xor INT32_MIN, so the all-zero word of a cleared table marks an empty
// slot; build rows whose key is INT32_MIN (stored word 0) go to a side list
// instead.  A table with a payload keeps row + 1 of every slot in a
// parallel array of 16-byte bucket rows, read only when an aggregate or the
// pair output needs the build row.  A key sits in its home bucket (fmix32
// bits) or, when that bucket was full at insert time, in a later one; a
// probe stops at the first bucket with an empty slot.
// Probe shape: kJbGroup probes per thread at a time (a multiple of 4), and
// the CTAs per SM the specialised probe kernels are compiled for (512
// threads each).  Measured on GB300 for the plain join (2^20 build rows,
// 2^24 probes): 4 probes x 2 CTAs ahead of 8 x 2 (register spills), 8 x 1
// and 4 x 3.
#ifndef GBJ_JB_MIN_BLOCKS
#define GBJ_JB_MIN_BLOCKS 2
#endif
#ifndef GBJ_JB_GROUP
#define GBJ_JB_GROUP 4
#endif
constexpr int kJbGroup = GBJ_JB_GROUP;
struct __align__(32) JBucket {
  int4 k;  // key ^ INT32_MIN, 0 = empty
  int4 x;  // payload, or row + 1
};

// One bucket in a single 256-bit load (ld.global.nc.v8, sm_100 and later):
// one L2 request per bucket instead of two.
__device__ __forceinline__ JBucket ld_bucket(const JBucket *p) {
  JBucket r;
  asm("ld.global.nc.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=r"(r.k.x), "=r"(r.k.y), "=r"(r.k.z), "=r"(r.k.w), "=r"(r.x.x), "=r"(r.x.y), "=r"(r.x.z), "=r"(r.x.w)
      : "l"(p));
  return r;
}
constexpr int32_t kKeyFlip = INT32_MIN;

__device__ __forceinline__ int32_t lane4(const int4 &v, uint32_t i) {
  return i == 0 ? v.x : i == 1 ? v.y : i == 2 ? v.z : v.w;
}
__device__ __forceinline__ uint32_t hits4(const int4 &k, int32_t kf) {
  return (uint32_t)(k.x == kf) | ((uint32_t)(k.y == kf) << 1) | ((uint32_t)(k.z == kf) << 2) |
         ((uint32_t)(k.w == kf) << 3);
}
__device__ __forceinline__ bool room4(const int4 &k) { return (k.x == 0) | (k.y == 0) | (k.z == 0) | (k.w == 0); }

// meta[0]: a duplicate build key was seen; meta[1]: side-list length.  A
// row claims the first free slot of its home bucket, starting at a slot
// chosen by the top hash bits, then of the following buckets.
__global__ void __launch_bounds__(kThreads)
    k_jb_build(const int32_t *__restrict__ keys, const int32_t *__restrict__ payload, uint64_t n,
               JBucket *__restrict__ bk, int4 *__restrict__ rows, uint32_t bmask, uint32_t *__restrict__ meta,
               int32_t *__restrict__ side, uint32_t *status) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  bool dup = false;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    const int32_t key = keys[i];
    const int32_t pv = payload ? payload[i] : (int32_t)(i + 1);
    const int32_t kf = key ^ kKeyFlip;
    if (kf == 0) {  // INT32_MIN: the side list
      side[atomicAdd(&meta[1], 1u)] = (int32_t)i;
      continue;
    }
    const uint32_t h = gbjd::fmix32((uint32_t)key);
    uint32_t b = h & bmask;
    const uint32_t o = h >> 30;  // start slot (high bits, independent of the bucket for 2^30 buckets or fewer)
    bool placed = false;
    for (uint32_t step = 0; step <= bmask && !placed; ++step) {
      int32_t *kw = reinterpret_cast<int32_t *>(&bk[b].k);
#pragma unroll
      for (uint32_t j = 0; j < 4; ++j) {
        if (placed) break;
        const uint32_t sl = (o + j) & 3u;
        const int32_t old = atomicCAS(&kw[sl], 0, kf);
        if (old == 0) {
          reinterpret_cast<int32_t *>(&bk[b].x)[sl] = pv;
          if (rows) reinterpret_cast<int32_t *>(&rows[b])[sl] = (int32_t)(i + 1);
          placed = true;
        } else {
          dup |= old == kf;
        }
      }
      b = (b + 1) & bmask;
    }
    if (!placed) gbjd::latch(status, GBJ_DEV_CAPACITY);
  }
  if (dup) meta[0] = 1;
}

// Probe with fused aggregate over the bucketed table.  A probe visits its
// home bucket and folds every slot whose key matches into the aggregate
// without branching (a count of the matches and, for the specialised
// aggregate lists, a select-and-sum of their values); it moves on to the
// next bucket only when the bucket is full and either has no match or the
// build keys are not unique -- the rare case, taken out of line.  Each
// thread handles kJbGroup probes at a time: their bucket loads (one 256-bit
// load each) are issued together, and the next group's probe keys and
// payloads are loaded while they are in flight.  kPay: the values are build
// payloads and build rows come from the row array.
template <bool kVec, int kAgg, bool kPay>
__global__ void __launch_bounds__(kThreads, kAgg == kAggGeneric ? 1 : GBJ_JB_MIN_BLOCKS)
    k_jb_probe_agg(const int32_t *__restrict__ keys, const int32_t *__restrict__ pay, uint64_t n,
                   const JBucket *__restrict__ bk, const int4 *__restrict__ rows, uint32_t bmask,
                   const int32_t *__restrict__ bpay, const uint32_t *__restrict__ meta,
                   const int32_t *__restrict__ side, gbj::AggSpec spec, int64_t *out) {
  __shared__ int64_t red[32 * GBJ_MAX_AGGS];
  gbjd::Acc acc;  // the specialised accumulators fill it only at the end
  if (kAgg == kAggGeneric) acc.init(spec);
  int64_t a_cnt = 0, a_sum = 0;
  const bool unique = meta[0] == 0;
  const uint32_t nside = meta[1];
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  // does the generic aggregate list read build rows? (payload tables keep them apart)
  bool need_row = !kPay;
  if (kPay && kAgg == kAggGeneric)
    for (int j = 0; j < spec.n; ++j)
      need_row |= spec.operand[j] == GBJ_VAL_BUILD_ROWID || spec.operand[j] == GBJ_VAL_ROWID_XOR;
  // folds the matching slots of bucket b (contents e) into the aggregate;
  // returns the number of matches
  auto visit = [&](int32_t k, int32_t kf, int64_t pv, uint64_t prow, uint32_t b, const JBucket &e) -> uint32_t {
    const bool m0 = e.k.x == kf, m1 = e.k.y == kf, m2 = e.k.z == kf, m3 = e.k.w == kf;
    const uint32_t c = (uint32_t)m0 + (uint32_t)m1 + (uint32_t)m2 + (uint32_t)m3;
    if (kAgg == kAggCountProduct) {
      a_cnt += c;
      if (kPay)
        a_sum += ((int64_t)(m0 ? e.x.x : 0) + (m1 ? e.x.y : 0) + (int64_t)(m2 ? e.x.z : 0) + (m3 ? e.x.w : 0)) * pv;
    } else if (kAgg == kAggCountXor && !kPay) {
      a_cnt += c;
      const int64_t pr = (int64_t)prow;
      a_sum += (m0 ? ((int64_t)(e.x.x - 1) ^ pr) : 0) + (m1 ? ((int64_t)(e.x.y - 1) ^ pr) : 0) +
               (m2 ? ((int64_t)(e.x.z - 1) ^ pr) : 0) + (m3 ? ((int64_t)(e.x.w - 1) ^ pr) : 0);
    } else if (c) {
      const bool rows_needed = kAgg == kAggCountXor || need_row;
      const int4 rw = kPay && rows_needed ? __ldg(&rows[b]) : e.x;
      uint32_t hits = (uint32_t)m0 | ((uint32_t)m1 << 1) | ((uint32_t)m2 << 2) | ((uint32_t)m3 << 3);
      while (hits) {
        const uint32_t idx = __ffs(hits) - 1;
        const int64_t bv = kPay ? lane4(e.x, idx) : 0;
        const int64_t brow = (kPay && !rows_needed) ? 0 : lane4(rw, idx) - 1;
        if (kAgg == kAggCountXor) {
          a_cnt += 1;
          a_sum += brow ^ (int64_t)prow;
        } else {
          acc.update(spec, k, bv, pv, brow, prow);
        }
        hits &= hits - 1;
      }
    }
    return c;
  };
  // the buckets after a full home bucket (out of line, rare)
  auto walk = [&](int32_t k, int32_t kf, int64_t pv, uint64_t prow, uint32_t b, uint32_t matched) {
    for (uint32_t step = 1; step <= bmask; ++step) {
      b = (b + 1) & bmask;
      const JBucket e = ld_bucket(&bk[b]);
      matched += visit(k, kf, pv, prow, b, e);
      if (room4(e.k) || (unique && matched)) return;
    }
  };
  // a probe key INT32_MIN meets the side list
  auto side_probe = [&](int32_t k, int64_t pv, uint64_t prow) {
    for (uint32_t s = 0; s < nside; ++s) {
      const int32_t r = side[s];
      const int64_t bv = kPay ? (int64_t)bpay[r] : 0;
      if (kAgg == kAggCountProduct) {
        a_cnt += 1;
        a_sum += bv * pv;
      } else if (kAgg == kAggCountXor) {
        a_cnt += 1;
        a_sum += (int64_t)r ^ (int64_t)prow;
      } else {
        acc.update(spec, k, bv, pv, r, prow);
      }
      if (unique) break;
    }
  };
  auto finish = [&](int32_t k, int64_t pv, uint64_t prow, uint32_t b, const JBucket &e) {
    const int32_t kf = k ^ kKeyFlip;
    if (kf == 0) {
      side_probe(k, pv, prow);
      return;
    }
    const uint32_t c = visit(k, kf, pv, prow, b, e);
    if (!room4(e.k) && !(unique && c)) walk(k, kf, pv, prow, b, c);
  };
  uint64_t done = 0;
  if (kVec) {
    constexpr int G = kJbGroup;  // probes per thread at a time (a multiple of 4)
    const uint64_t ng = n / G;
    const int4 *k4 = reinterpret_cast<const int4 *>(keys);
    const int4 *p4 = reinterpret_cast<const int4 *>(pay);
    int4 nk[G / 4], np[G / 4];
    auto load_group = [&](uint64_t qq) {
#pragma unroll
      for (int v = 0; v < G / 4; ++v) {
        nk[v] = __ldcs(k4 + (G / 4) * qq + v);
        np[v] = pay ? __ldcs(p4 + (G / 4) * qq + v) : make_int4(0, 0, 0, 0);
      }
    };
    uint64_t q = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (q < ng) load_group(q);
    for (; q < ng; q += stride) {
      int32_t kk[G], pp[G];
#pragma unroll
      for (int v = 0; v < G / 4; ++v) {
        kk[4 * v] = nk[v].x, kk[4 * v + 1] = nk[v].y, kk[4 * v + 2] = nk[v].z, kk[4 * v + 3] = nk[v].w;
        pp[4 * v] = np[v].x, pp[4 * v + 1] = np[v].y, pp[4 * v + 2] = np[v].z, pp[4 * v + 3] = np[v].w;
      }
      uint32_t b[G];
      JBucket e[G];
#pragma unroll
      for (int j = 0; j < G; ++j) {
        b[j] = gbjd::fmix32((uint32_t)kk[j]) & bmask;
        e[j] = ld_bucket(&bk[b[j]]);
      }
      if (q + stride < ng) load_group(q + stride);
#pragma unroll
      for (int j = 0; j < G; ++j) finish(kk[j], pp[j], q * G + j, b[j], e[j]);
    }
    done = ng * G;
  }
  for (uint64_t i = done + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    const int32_t k = keys[i];
    const uint32_t b = gbjd::fmix32((uint32_t)k) & bmask;
    finish(k, pay ? pay[i] : 0, i, b, ld_bucket(&bk[b]));
  }
  if (kAgg != kAggGeneric) {
    acc.init(spec);
    acc.v[0] = a_cnt;
    acc.v[1] = a_sum;
  }
  gbjd::block_flush(spec, acc, red, out);
}

// Pair output over the bucketed table (warp-aggregated output reservations).
template <bool kPay>
__global__ void __launch_bounds__(kThreads)
    k_jb_probe_pairs(const int32_t *__restrict__ keys, const int32_t *__restrict__ prows, uint64_t n,
                     const JBucket *__restrict__ bk, const int4 *__restrict__ rows, uint32_t bmask,
                     const uint32_t *__restrict__ meta, const int32_t *__restrict__ side,
                     int32_t *__restrict__ out_b, int32_t *__restrict__ out_p, uint64_t cap,
                     unsigned long long *count, uint32_t *status) {
  const bool unique = meta[0] == 0;
  const uint32_t nside = meta[1];
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  auto emit = [&](int32_t br, int32_t pr) {
    cg::coalesced_group g = cg::coalesced_threads();
    unsigned long long base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(count, (unsigned long long)g.size());
    base = g.shfl(base, 0) + g.thread_rank();
    if (base < cap) {
      out_b[base] = br;
      out_p[base] = pr;
    } else {
      gbjd::latch(status, GBJ_DEV_CAPACITY);
    }
  };
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    const int32_t k = keys[i];
    const int32_t pr = prows ? prows[i] : (int32_t)i;
    const int32_t kf = k ^ kKeyFlip;
    if (kf == 0) {
      for (uint32_t s = 0; s < nside; ++s) {
        emit(side[s], pr);
        if (unique) break;
      }
      continue;
    }
    uint32_t b = gbjd::fmix32((uint32_t)k) & bmask;
    for (uint32_t step = 0; step <= bmask; ++step) {
      const JBucket e = ld_bucket(&bk[b]);
      uint32_t hits = hits4(e.k, kf);
      bool stop = room4(e.k);
      while (hits) {
        const uint32_t idx = __ffs(hits) - 1;
        emit(lane4(kPay ? __ldg(&rows[b]) : e.x, idx) - 1, pr);
        if (unique) {
          stop = true;
          break;
        }
        hits &= hits - 1;
      }
      if (stop) break;
      b = (b + 1) & bmask;
    }
  }
}

// ------------------------------------------------ int64-key table
// gbj_join_build_i64's table: 32-byte buckets of two slots -- two keys
// (xor 2^63, so zero marks an empty slot; INT64_MIN goes to the side list),
// their build payloads and their rows + 1 -- read with one 256-bit load.
// Placement is the reference's int64 hash, the murmur3 64-bit finaliser
// (core/olap/lib/expressions/expressions-hasher.cpp:66-84).
struct __align__(32) JBucket64 {
  unsigned long long k[2];
  int32_t x[2];  // build payload (0 without one)
  int32_t r[2];  // row + 1
};
constexpr unsigned long long kFlip64 = 0x8000000000000000ull;

__device__ __forceinline__ uint64_t fmix64(uint64_t k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ull;
  k ^= k >> 33;
  return k;
}

__device__ __forceinline__ JBucket64 ld_bucket64(const JBucket64 *p) {
  uint32_t w[8];
  asm("ld.global.nc.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=r"(w[0]), "=r"(w[1]), "=r"(w[2]), "=r"(w[3]), "=r"(w[4]), "=r"(w[5]), "=r"(w[6]), "=r"(w[7])
      : "l"(p));
  JBucket64 b;
  b.k[0] = ((unsigned long long)w[1] << 32) | w[0];
  b.k[1] = ((unsigned long long)w[3] << 32) | w[2];
  b.x[0] = (int32_t)w[4], b.x[1] = (int32_t)w[5];
  b.r[0] = (int32_t)w[6], b.r[1] = (int32_t)w[7];
  return b;
}

// meta[0]: a duplicate build key was seen; meta[1]: side-list length.
__global__ void __launch_bounds__(kThreads)
    k_jb64_build(const int64_t *__restrict__ keys, const int32_t *__restrict__ payload, uint64_t n,
                 JBucket64 *__restrict__ bk, uint64_t bmask, uint32_t *__restrict__ meta,
                 int32_t *__restrict__ side, uint32_t *status) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  bool dup = false;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    const int64_t key = keys[i];
    const int32_t pv = payload ? payload[i] : 0;
    const unsigned long long kf = (unsigned long long)key ^ kFlip64;
    if (kf == 0) {
      side[atomicAdd(&meta[1], 1u)] = (int32_t)i;
      continue;
    }
    const uint64_t h = fmix64((uint64_t)key);
    uint64_t b = h & bmask;
    const uint32_t o = (uint32_t)(h >> 63);
    bool placed = false;
    for (uint64_t step = 0; step <= bmask && !placed; ++step) {
#pragma unroll
      for (uint32_t j = 0; j < 2; ++j) {
        if (placed) break;
        const uint32_t sl = (o + j) & 1u;
        const unsigned long long old = atomicCAS(&bk[b].k[sl], 0ull, kf);
        if (old == 0) {
          bk[b].x[sl] = pv;
          bk[b].r[sl] = (int32_t)(i + 1);
          placed = true;
        } else {
          dup |= old == kf;
        }
      }
      b = (b + 1) & bmask;
    }
    if (!placed) gbjd::latch(status, GBJ_DEV_CAPACITY);
  }
  if (dup) meta[0] = 1;
}

// Probe with fused aggregate over the int64-key table: four probes per
// thread, their bucket loads issued together; a probe moves past its home
// bucket only when it is full and (for unique build keys) has no match.
__global__ void __launch_bounds__(kThreads)
    k_jb64_probe_agg(const int64_t *__restrict__ keys, const int32_t *__restrict__ pay, uint64_t n,
                     const JBucket64 *__restrict__ bk, uint64_t bmask, const int32_t *__restrict__ bpay,
                     const uint32_t *__restrict__ meta, const int32_t *__restrict__ side, gbj::AggSpec spec,
                     int64_t *out) {
  __shared__ int64_t red[32 * GBJ_MAX_AGGS];
  gbjd::Acc acc;
  acc.init(spec);
  const bool unique = meta[0] == 0;
  const uint32_t nside = meta[1];
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  auto visit = [&](int64_t k, unsigned long long kf, int64_t pv, uint64_t prow, const JBucket64 &e) -> uint32_t {
    uint32_t c = 0;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      if (e.k[j] == kf) {
        acc.update(spec, k, e.x[j], pv, (int64_t)e.r[j] - 1, (int64_t)prow);
        ++c;
      }
    }
    return c;
  };
  auto room = [](const JBucket64 &e) { return e.k[0] == 0 || e.k[1] == 0; };
  auto finish = [&](int64_t k, int64_t pv, uint64_t prow, uint64_t b, const JBucket64 &e0) {
    const unsigned long long kf = (unsigned long long)k ^ kFlip64;
    if (kf == 0) {  // INT64_MIN meets the side list
      for (uint32_t s = 0; s < nside; ++s) {
        const int32_t r = side[s];
        acc.update(spec, k, bpay ? (int64_t)bpay[r] : 0, pv, r, (int64_t)prow);
        if (unique) break;
      }
      return;
    }
    uint32_t matched = visit(k, kf, pv, prow, e0);
    if (room(e0) || (unique && matched)) return;
    for (uint64_t step = 1; step <= bmask; ++step) {
      b = (b + 1) & bmask;
      const JBucket64 e = ld_bucket64(&bk[b]);
      matched += visit(k, kf, pv, prow, e);
      if (room(e) || (unique && matched)) return;
    }
  };
  constexpr int G = 4;
  const uint64_t ng = n / G;
  for (uint64_t q = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; q < ng; q += stride) {
    int64_t kk[G];
    int64_t pp[G];
    uint64_t b[G];
    JBucket64 e[G];
#pragma unroll
    for (int j = 0; j < G; ++j) {
      kk[j] = __ldcs(keys + q * G + j);
      pp[j] = pay ? __ldcs(pay + q * G + j) : 0;
    }
#pragma unroll
    for (int j = 0; j < G; ++j) {
      b[j] = fmix64((uint64_t)kk[j]) & bmask;
      e[j] = ld_bucket64(&bk[b[j]]);
    }
#pragma unroll
    for (int j = 0; j < G; ++j) finish(kk[j], pp[j], q * G + j, b[j], e[j]);
  }
  for (uint64_t i = ng * G + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    const int64_t k = keys[i];
    const uint64_t b = fmix64((uint64_t)k) & bmask;
    finish(k, pay ? pay[i] : 0, i, b, ld_bucket64(&bk[b]));
  }
  gbjd::block_flush(spec, acc, red, out);
}

// Pair output over the int64-key table (warp-aggregated output reservations).
__global__ void __launch_bounds__(kThreads)
    k_jb64_probe_pairs(const int64_t *__restrict__ keys, const int32_t *__restrict__ prows, uint64_t n,
                       const JBucket64 *__restrict__ bk, uint64_t bmask, const uint32_t *__restrict__ meta,
                       const int32_t *__restrict__ side, int32_t *__restrict__ out_b,
                       int32_t *__restrict__ out_p, uint64_t cap, unsigned long long *count, uint32_t *status) {
  const bool unique = meta[0] == 0;
  const uint32_t nside = meta[1];
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  auto emit = [&](int32_t br, int32_t pr) {
    cg::coalesced_group g = cg::coalesced_threads();
    unsigned long long base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(count, (unsigned long long)g.size());
    base = g.shfl(base, 0) + g.thread_rank();
    if (base < cap) {
      out_b[base] = br;
      out_p[base] = pr;
    } else {
      gbjd::latch(status, GBJ_DEV_CAPACITY);
    }
  };
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    const int64_t k = keys[i];
    const int32_t pr = prows ? prows[i] : (int32_t)i;
    const unsigned long long kf = (unsigned long long)k ^ kFlip64;
    if (kf == 0) {
      for (uint32_t s = 0; s < nside; ++s) {
        emit(side[s], pr);
        if (unique) break;
      }
      continue;
    }
    uint64_t b = fmix64((uint64_t)k) & bmask;
    for (uint64_t step = 0; step <= bmask; ++step) {
      const JBucket64 e = ld_bucket64(&bk[b]);
      bool stop = e.k[0] == 0 || e.k[1] == 0;
      for (int j = 0; j < 2; ++j) {
        if (e.k[j] == kf) {
          emit(e.r[j] - 1, pr);
          if (unique) stop = true;
        }
      }
      if (stop) break;
      b = (b + 1) & bmask;
    }
  }
}

// Column reduce (Reduce over one column, optional row list).
__global__ void __launch_bounds__(kThreads)
    k_reduce(const int32_t *__restrict__ col, const int32_t *__restrict__ rows,
             uint64_t n, gbj::AggSpec spec, int64_t *out) {
  __shared__ int64_t red[32 * GBJ_MAX_AGGS];
  gbjd::Acc acc;
  acc.init(spec);
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    const int64_t r = rows ? rows[i] : (int64_t)i;
    const int64_t v = col ? col[r] : 0;
    acc.update(spec, (int32_t)v, v, v, r, r);
  }
  gbjd::block_flush(spec, acc, red, out);
}

__global__ void k_gather(const int32_t *__restrict__ col,
                         const int32_t *__restrict__ rows, uint64_t n,
                         int32_t *__restrict__ out) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride)
    out[i] = col[rows[i]];
}

// Range predicate of gbj_select_range (inclusive bounds).
struct RangePred {
  const int32_t *col;
  int32_t lo, hi;
  __device__ __forceinline__ bool operator()(uint64_t i) const {
    const int32_t v = col[i];
    return v >= lo && v <= hi;
  }
};

int grid_for_sms(int sm_count, uint64_t work, int threads, int per_sm = 4) {
  uint64_t blocks = (work + threads - 1) / threads;
  uint64_t cap = (uint64_t)sm_count * per_sm;
  if (blocks > cap) blocks = cap;
  if (blocks == 0) blocks = 1;
  return (int)blocks;
}

int grid_for(gbj_ctx *ctx, uint64_t work, int threads, int per_sm = 4) {
  return grid_for_sms(ctx->sm_count, work, threads, per_sm);
}

// Probe kernel of the allocation-free entry point: 16-byte loads when both
// probe columns are 16-byte aligned, a specialised accumulator for COUNT +
// SUM(product / xor).
void launch_probe(int sm_count, const int32_t *keys, const int32_t *pay, uint64_t n, const uint64_t *slots,
                  uint64_t mask, const int32_t *bpay, const uint32_t *meta, const gbj::AggSpec &spec,
                  int64_t *out, cudaStream_t s) {
  const bool vec = ((uintptr_t)keys % 16 == 0) && (!pay || (uintptr_t)pay % 16 == 0);
  const bool two = spec.n == 2 && spec.op[0] == GBJ_AGG_COUNT && spec.op[1] == GBJ_AGG_SUM;
  const int agg = two && spec.operand[1] == GBJ_VAL_ROWID_XOR ? kAggCountXor
                  : two && spec.operand[1] == GBJ_VAL_PRODUCT ? kAggCountProduct
                                                              : kAggGeneric;
  const int gv = grid_for_sms(sm_count, (n + 7) / 8, kThreads);
  const int gs = grid_for_sms(sm_count, n, kThreads);
#define GBJ_PROBE(V, A) \
  k_join_probe_agg<V, A><<<V ? gv : gs, kThreads, 0, s>>>(keys, pay, n, slots, mask, bpay, meta, spec, out)
  if (vec) {
    if (agg == kAggCountXor) GBJ_PROBE(true, kAggCountXor);
    else if (agg == kAggCountProduct) GBJ_PROBE(true, kAggCountProduct);
    else GBJ_PROBE(true, kAggGeneric);
  } else {
    if (agg == kAggCountXor) GBJ_PROBE(false, kAggCountXor);
    else if (agg == kAggCountProduct) GBJ_PROBE(false, kAggCountProduct);
    else GBJ_PROBE(false, kAggGeneric);
  }
#undef GBJ_PROBE
}

// Probe kernel over a bucketed table: 16-byte probe loads when both probe
// columns are aligned, the specialised accumulators, the table's layout.
template <bool kPay>
void launch_jb_probe_t(int sm_count, const gbj_table *t, const int32_t *keys, const int32_t *pay, uint64_t n,
                       const gbj::AggSpec &spec, int64_t *out, cudaStream_t s) {
  const bool vec = ((uintptr_t)keys % 16 == 0) && (!pay || (uintptr_t)pay % 16 == 0);
  const bool two = spec.n == 2 && spec.op[0] == GBJ_AGG_COUNT && spec.op[1] == GBJ_AGG_SUM;
  const int agg = two && spec.operand[1] == GBJ_VAL_ROWID_XOR ? kAggCountXor
                  : two && spec.operand[1] == GBJ_VAL_PRODUCT ? kAggCountProduct
                                                              : kAggGeneric;
  const JBucket *bk = static_cast<const JBucket *>(t->slots);
  const uint32_t bmask = (uint32_t)((t->mask + 1) / 4 - 1);
  const int gv = grid_for_sms(sm_count, (n + kJbGroup - 1) / kJbGroup, kThreads, 2);
  const int gs = grid_for_sms(sm_count, n, kThreads);
#define GBJ_JB_PROBE(V, A)                                                                               \
  k_jb_probe_agg<V, A, kPay><<<V ? gv : gs, kThreads, 0, s>>>(keys, pay, n, bk, t->rows, bmask, t->payload, \
                                                              t->meta, t->side, spec, out)
  if (vec) {
    if (agg == kAggCountXor) GBJ_JB_PROBE(true, kAggCountXor);
    else if (agg == kAggCountProduct) GBJ_JB_PROBE(true, kAggCountProduct);
    else GBJ_JB_PROBE(true, kAggGeneric);
  } else {
    if (agg == kAggCountXor) GBJ_JB_PROBE(false, kAggCountXor);
    else if (agg == kAggCountProduct) GBJ_JB_PROBE(false, kAggCountProduct);
    else GBJ_JB_PROBE(false, kAggGeneric);
  }
#undef GBJ_JB_PROBE
}

void launch_jb_probe(int sm_count, const gbj_table *t, const int32_t *keys, const int32_t *pay, uint64_t n,
                     const gbj::AggSpec &spec, int64_t *out, cudaStream_t s) {
  if (t->rows) launch_jb_probe_t<true>(sm_count, t, keys, pay, n, spec, out, s);
  else launch_jb_probe_t<false>(sm_count, t, keys, pay, n, spec, out, s);
}

// ------------------------------------------------ allocation-free variant
// Hash table of gbj_join_agg_noalloc: a fixed array in the module's device
// memory, so that entry point never allocates.  Slots for build sides of up
// to GBJ_NOALLOC_MAX_BUILD rows at load factor 1/2, then 32 words of table
// metadata (the duplicate-key flag).  The table always has at least 2n
// slots, so its build cannot run out of room and needs no status word.
constexpr uint64_t kNoAllocSlots = 2ull * GBJ_NOALLOC_MAX_BUILD;
static __device__ __align__(256) uint64_t g_noalloc_scratch[kNoAllocSlots + 32];

__global__ void k_noalloc_init_out(gbj::AggSpec s, int64_t *out) {
  const int j = threadIdx.x;
  if (j < s.n) out[j] = gbjd::agg_identity(s.op[j]);
}

// Per-device set-up of the allocation-free entry point: the device address
// of g_noalloc_scratch (host code cannot use the symbol itself) and the SM
// count, looked up once per device and CUDA context with that device current.
// The context is part of the key because cudaDeviceReset ends the context
// that address belongs to; the next call then looks it up again.
struct NoAllocDevice {
  uint64_t *scratch = nullptr;
  int sm_count = 0;
};
std::mutex g_noalloc_mu;
std::map<std::pair<int, unsigned long long>, NoAllocDevice> g_noalloc_devices;

// Unique id of the calling thread's current CUDA context (0 when there is
// none yet), through the driver entry points the runtime hands out, so the
// library needs no link against the driver library.
unsigned long long current_context_id() {
  typedef int (*GetCurrent)(void **);
  typedef int (*GetId)(void *, unsigned long long *);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrent>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(f);
    (void)cudaGetLastError();
  });
  void *c = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&c) != 0 || !c || get_id(c, &id) != 0) return 0;
  return id;
}
thread_local std::string g_noalloc_error;

int noalloc_fail(int code, const char *msg) {
  g_noalloc_error = msg;
  return code;
}

}  // namespace

namespace gbj {
const char *noalloc_error_text_impl() { return g_noalloc_error.c_str(); }
}  // namespace gbj

extern "C" {

int gbj_join_build(gbj_ctx *ctx, const int32_t *d_keys,
                   const int32_t *d_payload, uint64_t n, int32_t hash_bits,
                   uint64_t max_build, void *stream, gbj_table **out) {
  if (!ctx || !out) return GBJ_ERR_INVALID;
  *out = nullptr;
  if (n && !d_keys) return set_error(ctx, GBJ_ERR_INVALID, "join_build: null keys");
  if (n >= (1ULL << 31)) return set_error(ctx, GBJ_ERR_INVALID, "join_build: n >= 2^31");
  if (hash_bits < 0 || hash_bits > 31)
    return set_error(ctx, GBJ_ERR_INVALID, "join_build: hash_bits out of range");
  if (max_build && n > max_build)
    return set_error(ctx, GBJ_ERR_CAPACITY,
                     "Build input size exceeded given parameter (maxBuildInputSize)");
  cudaStream_t s = pick_stream(ctx, stream);
  prof_mark(ctx, s);
  uint64_t slots = next_pow2(2 * (n ? n : 1));
  if (!hash_bits) {  // an autotuned table size for build sides of this size, if any
    const int32_t tb = tuned_value(ctx, tune_key("join", n, 0));
    if (tb > 0) hash_bits = tb;
  }
  if (hash_bits && (1ULL << hash_bits) > slots) slots = 1ULL << hash_bits;
  if (slots < 64) slots = 64;
  if (slots > (1ULL << 32)) return set_error(ctx, GBJ_ERR_INVALID, "join_build: table above 2^32 slots");
  const uint64_t nbk = slots / 4;
  const bool with_pay = d_payload != nullptr;
  // buckets | rows (payload tables) | metadata | INT32_MIN side list
  const uint64_t b_bytes = nbk * sizeof(JBucket), r_bytes = with_pay ? nbk * sizeof(int4) : 0;
  const uint64_t clear_bytes = b_bytes + r_bytes + 256;
  gbj_table *t = new gbj_table();
  void *mem = nullptr;
  int rc = pool_alloc(ctx, clear_bytes + (n + 4) * sizeof(int32_t), s, &mem);
  if (rc) {
    delete t;
    return rc;
  }
  char *base = static_cast<char *>(mem);
  t->slots = mem;
  t->rows = with_pay ? reinterpret_cast<int4 *>(base + b_bytes) : nullptr;
  t->meta = reinterpret_cast<uint32_t *>(base + b_bytes + r_bytes);
  t->side = reinterpret_cast<int32_t *>(base + clear_bytes);
  t->mask = slots - 1;
  t->keys = d_keys;
  t->payload = d_payload;
  t->n = n;
  cudaError_t e = cudaMemsetAsync(mem, 0, clear_bytes, s);
  if (e != cudaSuccess) {
    pool_release(ctx, mem, s);
    delete t;
    return cuda_error(ctx, e, "cudaMemsetAsync(table)");
  }
  if (n) {
    k_jb_build<<<grid_for(ctx, n, kThreads), kThreads, 0, s>>>(d_keys, d_payload, n,
                                                                reinterpret_cast<JBucket *>(mem), t->rows,
                                                                (uint32_t)(nbk - 1), t->meta, t->side,
                                                                ctx->d_status);
    rc = after_launch(ctx, "k_jb_build", s);
    if (rc) {
      pool_release(ctx, mem, s);
      delete t;
      return rc;
    }
  }
  *out = t;
  return GBJ_OK;
}

int gbj_table_destroy(gbj_ctx *ctx, gbj_table *table) {
  if (!ctx || !table) return GBJ_ERR_INVALID;
  int rc = pool_release(ctx, table->slots, ctx->stream);
  delete table;
  return rc;
}

uint64_t gbj_table_slots(const gbj_table *table) { return table ? table->mask + 1 : 0; }

int gbj_join_probe_agg(gbj_ctx *ctx, const gbj_table *t, const int32_t *d_keys,
                       const int32_t *d_payload, uint64_t n, const gbj_agg *aggs,
                       int32_t n_aggs, int64_t *d_out, void *stream) {
  if (!ctx || !t || !d_out) return GBJ_ERR_INVALID;
  if (t->i64) return set_error(ctx, GBJ_ERR_INVALID, "join_probe: the table has int64 keys (use the _i64 probe)");
  if (n && !d_keys) return set_error(ctx, GBJ_ERR_INVALID, "join_probe: null keys");
  GBJ_TRY(validate_aggs(ctx, aggs, n_aggs));
  AggSpec spec = make_spec(aggs, n_aggs);
  for (int j = 0; j < n_aggs; ++j) {
    int o = spec.operand[j];
    if ((o == GBJ_VAL_BUILD || o == GBJ_VAL_PRODUCT) && !t->payload && t->n)
      return set_error(ctx, GBJ_ERR_INVALID, "aggregate reads the build payload, table has none");
    if ((o == GBJ_VAL_PROBE || o == GBJ_VAL_PRODUCT) && !d_payload && n)
      return set_error(ctx, GBJ_ERR_INVALID, "aggregate reads the probe payload, none given");
  }
  cudaStream_t s = pick_stream(ctx, stream);
  prof_mark(ctx, s);
  GBJ_TRY(init_agg_out(ctx, spec, d_out, s));
  if (n == 0) return GBJ_OK;
  launch_jb_probe(ctx->sm_count, t, d_keys, d_payload, n, spec, d_out, s);
  return after_launch(ctx, "k_jb_probe_agg", s);
}

int gbj_join_probe_pairs(gbj_ctx *ctx, const gbj_table *t, const int32_t *d_keys,
                         const int32_t *d_probe_rows, uint64_t n,
                         int32_t *d_build_rows, int32_t *d_out_probe_rows,
                         uint64_t capacity, uint64_t *d_count, void *stream) {
  if (!ctx || !t || !d_count || !d_build_rows || !d_out_probe_rows)
    return GBJ_ERR_INVALID;
  if (t->i64) return set_error(ctx, GBJ_ERR_INVALID, "join_probe: the table has int64 keys (use the _i64 probe)");
  if (n && !d_keys) return set_error(ctx, GBJ_ERR_INVALID, "join_probe: null keys");
  cudaStream_t s = pick_stream(ctx, stream);
  prof_mark(ctx, s);
  GBJ_CHECK_CUDA(ctx, cudaMemsetAsync(d_count, 0, sizeof(uint64_t), s));
  if (n == 0) return GBJ_OK;
  const JBucket *bk = static_cast<const JBucket *>(t->slots);
  const uint32_t bmask = (uint32_t)((t->mask + 1) / 4 - 1);
  if (t->rows)
    k_jb_probe_pairs<true><<<grid_for(ctx, n, kThreads), kThreads, 0, s>>>(
        d_keys, d_probe_rows, n, bk, t->rows, bmask, t->meta, t->side, d_build_rows, d_out_probe_rows, capacity,
        (unsigned long long *)d_count, ctx->d_status);
  else
    k_jb_probe_pairs<false><<<grid_for(ctx, n, kThreads), kThreads, 0, s>>>(
        d_keys, d_probe_rows, n, bk, nullptr, bmask, t->meta, t->side, d_build_rows, d_out_probe_rows, capacity,
        (unsigned long long *)d_count, ctx->d_status);
  return after_launch(ctx, "k_jb_probe_pairs", s);
}

int gbj_join_build_i64(gbj_ctx *ctx, const int64_t *d_keys, const int32_t *d_payload, uint64_t n,
                       int32_t hash_bits, uint64_t max_build, void *stream, gbj_table **out) {
  if (!ctx || !out) return GBJ_ERR_INVALID;
  *out = nullptr;
  if (n && !d_keys) return set_error(ctx, GBJ_ERR_INVALID, "join_build: null keys");
  if (n >= (1ULL << 31)) return set_error(ctx, GBJ_ERR_INVALID, "join_build: n >= 2^31");
  if (hash_bits < 0 || hash_bits > 32)
    return set_error(ctx, GBJ_ERR_INVALID, "join_build: hash_bits out of range");
  if (max_build && n > max_build)
    return set_error(ctx, GBJ_ERR_CAPACITY, "Build input size exceeded given parameter (maxBuildInputSize)");
  cudaStream_t s = pick_stream(ctx, stream);
  prof_mark(ctx, s);
  uint64_t slots = next_pow2(2 * (n ? n : 1));
  if (hash_bits && (1ULL << hash_bits) > slots) slots = 1ULL << hash_bits;
  if (slots < 64) slots = 64;
  const uint64_t nbk = slots / 2;
  const uint64_t clear_bytes = nbk * sizeof(JBucket64) + 256;
  gbj_table *t = new gbj_table();
  void *mem = nullptr;
  int rc = pool_alloc(ctx, clear_bytes + (n + 4) * sizeof(int32_t), s, &mem);
  if (rc) {
    delete t;
    return rc;
  }
  char *base = static_cast<char *>(mem);
  t->slots = mem;
  t->meta = reinterpret_cast<uint32_t *>(base + nbk * sizeof(JBucket64));
  t->side = reinterpret_cast<int32_t *>(base + clear_bytes);
  t->mask = slots - 1;
  t->payload = d_payload;
  t->n = n;
  t->i64 = true;
  cudaError_t e = cudaMemsetAsync(mem, 0, clear_bytes, s);
  if (e != cudaSuccess) {
    pool_release(ctx, mem, s);
    delete t;
    return cuda_error(ctx, e, "cudaMemsetAsync(table)");
  }
  if (n) {
    k_jb64_build<<<grid_for(ctx, n, kThreads), kThreads, 0, s>>>(d_keys, d_payload, n,
                                                                  reinterpret_cast<JBucket64 *>(mem), nbk - 1,
                                                                  t->meta, t->side, ctx->d_status);
    rc = after_launch(ctx, "k_jb64_build", s);
    if (rc) {
      pool_release(ctx, mem, s);
      delete t;
      return rc;
    }
  }
  *out = t;
  return GBJ_OK;
}

int gbj_join_probe_agg_i64(gbj_ctx *ctx, const gbj_table *t, const int64_t *d_keys, const int32_t *d_payload,
                           uint64_t n, const gbj_agg *aggs, int32_t n_aggs, int64_t *d_out, void *stream) {
  if (!ctx || !t || !d_out) return GBJ_ERR_INVALID;
  if (!t->i64) return set_error(ctx, GBJ_ERR_INVALID, "join_probe_i64: the table has int32 keys");
  if (n && !d_keys) return set_error(ctx, GBJ_ERR_INVALID, "join_probe: null keys");
  GBJ_TRY(validate_aggs(ctx, aggs, n_aggs));
  AggSpec spec = make_spec(aggs, n_aggs);
  for (int j = 0; j < n_aggs; ++j) {
    int o = spec.operand[j];
    if ((o == GBJ_VAL_BUILD || o == GBJ_VAL_PRODUCT) && !t->payload && t->n)
      return set_error(ctx, GBJ_ERR_INVALID, "aggregate reads the build payload, table has none");
    if ((o == GBJ_VAL_PROBE || o == GBJ_VAL_PRODUCT) && !d_payload && n)
      return set_error(ctx, GBJ_ERR_INVALID, "aggregate reads the probe payload, none given");
  }
  cudaStream_t s = pick_stream(ctx, stream);
  prof_mark(ctx, s);
  GBJ_TRY(init_agg_out(ctx, spec, d_out, s));
  if (n == 0) return GBJ_OK;
  k_jb64_probe_agg<<<grid_for(ctx, (n + 3) / 4, kThreads, 2), kThreads, 0, s>>>(
      d_keys, d_payload, n, static_cast<const JBucket64 *>(t->slots), (t->mask + 1) / 2 - 1, t->payload, t->meta,
      t->side, spec, d_out);
  return after_launch(ctx, "k_jb64_probe_agg", s);
}

int gbj_join_probe_pairs_i64(gbj_ctx *ctx, const gbj_table *t, const int64_t *d_keys,
                             const int32_t *d_probe_rows, uint64_t n, int32_t *d_build_rows,
                             int32_t *d_out_probe_rows, uint64_t capacity, uint64_t *d_count, void *stream) {
  if (!ctx || !t || !d_count || !d_build_rows || !d_out_probe_rows) return GBJ_ERR_INVALID;
  if (!t->i64) return set_error(ctx, GBJ_ERR_INVALID, "join_probe_i64: the table has int32 keys");
  if (n && !d_keys) return set_error(ctx, GBJ_ERR_INVALID, "join_probe: null keys");
  cudaStream_t s = pick_stream(ctx, stream);
  prof_mark(ctx, s);
  GBJ_CHECK_CUDA(ctx, cudaMemsetAsync(d_count, 0, sizeof(uint64_t), s));
  if (n == 0) return GBJ_OK;
  k_jb64_probe_pairs<<<grid_for(ctx, n, kThreads), kThreads, 0, s>>>(
      d_keys, d_probe_rows, n, static_cast<const JBucket64 *>(t->slots), (t->mask + 1) / 2 - 1, t->meta, t->side,
      d_build_rows, d_out_probe_rows, capacity, (unsigned long long *)d_count, ctx->d_status);
  return after_launch(ctx, "k_jb64_probe_pairs", s);
}

int gbj_reduce(gbj_ctx *ctx, const int32_t *d_col, const int32_t *d_rows,
               uint64_t n, const gbj_agg *aggs, int32_t n_aggs, int64_t *d_out,
               void *stream) {
  if (!ctx || !d_out) return GBJ_ERR_INVALID;
  GBJ_TRY(validate_aggs(ctx, aggs, n_aggs));
  AggSpec spec = make_spec(aggs, n_aggs);
  for (int j = 0; j < n_aggs; ++j)
    if (spec.operand[j] != GBJ_VAL_ONE && !d_col)
      return set_error(ctx, GBJ_ERR_INVALID, "reduce: aggregate reads a null column");
  cudaStream_t s = pick_stream(ctx, stream);
  prof_mark(ctx, s);
  GBJ_TRY(init_agg_out(ctx, spec, d_out, s));
  if (n == 0) return GBJ_OK;
  k_reduce<<<grid_for(ctx, n, kThreads), kThreads, 0, s>>>(d_col, d_rows, n, spec, d_out);
  return after_launch(ctx, "k_reduce", s);
}

int gbj_gather(gbj_ctx *ctx, const int32_t *d_col, const int32_t *d_rows,
               uint64_t n, int32_t *d_out, void *stream) {
  if (!ctx || (n && (!d_col || !d_rows || !d_out))) return GBJ_ERR_INVALID;
  if (n == 0) return GBJ_OK;
  cudaStream_t s = pick_stream(ctx, stream);
  prof_mark(ctx, s);
  k_gather<<<grid_for(ctx, n, 256, 8), 256, 0, s>>>(d_col, d_rows, n, d_out);
  return after_launch(ctx, "k_gather", s);
}

int gbj_select_range(gbj_ctx *ctx, const int32_t *d_col, uint64_t n, int32_t lo,
                     int32_t hi, int32_t *d_rows_out, uint64_t *d_count,
                     void *stream) {
  if (!ctx || !d_count || (n && (!d_col || !d_rows_out))) return GBJ_ERR_INVALID;
  if (n >= (1ULL << 31)) return set_error(ctx, GBJ_ERR_INVALID, "select: n >= 2^31");
  cudaStream_t s = pick_stream(ctx, stream);
  prof_mark(ctx, s);
  if (n == 0) {
    GBJ_CHECK_CUDA(ctx, cudaMemsetAsync(d_count, 0, sizeof(uint64_t), s));
    return GBJ_OK;
  }
  return compact_rows(ctx, RangePred{d_col, lo, hi}, n, d_rows_out, d_count, s);
}

int gbj_join_agg_noalloc(const int32_t *d_build_keys, const int32_t *d_build_payload,
                         uint64_t n_build, const int32_t *d_probe_keys,
                         const int32_t *d_probe_payload, uint64_t n_probe, const gbj_agg *aggs,
                         int32_t n_aggs, int64_t *d_out, void *stream) {
  g_noalloc_error.clear();
  if (!d_out || !aggs || n_aggs < 1 || n_aggs > GBJ_MAX_AGGS)
    return noalloc_fail(GBJ_ERR_INVALID, "join_agg_noalloc: null output or bad aggregate count");
  if ((n_build && !d_build_keys) || (n_probe && !d_probe_keys))
    return noalloc_fail(GBJ_ERR_INVALID, "join_agg_noalloc: null key column");
  if (n_build > GBJ_NOALLOC_MAX_BUILD)
    return noalloc_fail(GBJ_ERR_CAPACITY,
                        "join_agg_noalloc: build side larger than GBJ_NOALLOC_MAX_BUILD "
                        "(1048576 rows); use gbj_join_build / gbj_join_probe_agg instead");
  if (n_probe >= (1ULL << 32))
    return noalloc_fail(GBJ_ERR_INVALID, "join_agg_noalloc: probe side must have < 2^32 rows");
  for (int j = 0; j < n_aggs; ++j) {
    if (aggs[j].op < GBJ_AGG_COUNT || aggs[j].op > GBJ_AGG_AND || aggs[j].operand < GBJ_VAL_ONE ||
        aggs[j].operand > GBJ_VAL_BUILD_KEY)
      return noalloc_fail(GBJ_ERR_INVALID, "join_agg_noalloc: bad aggregate");
    const int o = aggs[j].operand;
    if ((o == GBJ_VAL_BUILD || o == GBJ_VAL_PRODUCT) && !d_build_payload && n_build)
      return noalloc_fail(GBJ_ERR_INVALID, "join_agg_noalloc: aggregate reads a null build payload");
    if ((o == GBJ_VAL_PROBE || o == GBJ_VAL_PRODUCT) && !d_probe_payload && n_probe)
      return noalloc_fail(GBJ_ERR_INVALID, "join_agg_noalloc: aggregate reads a null probe payload");
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    (void)cudaGetLastError();
    return noalloc_fail(GBJ_ERR_CUDA, "join_agg_noalloc: no current CUDA device");
  }
  NoAllocDevice d;
  {
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    auto it = g_noalloc_devices.find({dev, current_context_id()});
    if (it == g_noalloc_devices.end()) {
      // first call on this device in this context: resolve the array's
      // device address (this also makes the runtime's context current)
      void *ptr = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
      if (e != cudaSuccess || !ptr) {
        (void)cudaGetLastError();
        return noalloc_fail(GBJ_ERR_CUDA, "join_agg_noalloc: cudaGetSymbolAddress failed");
      }
      NoAllocDevice nd;
      nd.scratch = static_cast<uint64_t *>(ptr);
      if (cudaDeviceGetAttribute(&nd.sm_count, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        (void)cudaGetLastError();
        return noalloc_fail(GBJ_ERR_CUDA, "join_agg_noalloc: device query failed");
      }
      it = g_noalloc_devices.insert_or_assign({dev, current_context_id()}, nd).first;
    }
    d = it->second;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  AggSpec spec = make_spec(aggs, n_aggs);
  uint64_t slots = next_pow2(2 * (n_build ? n_build : 1));
  if (slots < 64) slots = 64;
  uint64_t *table = d.scratch;
  uint32_t *meta = reinterpret_cast<uint32_t *>(d.scratch + kNoAllocSlots);
  // the array keeps the previous call's table: clear the part this call uses
  if (cudaMemsetAsync(table, 0, slots * sizeof(uint64_t), s) != cudaSuccess ||
      cudaMemsetAsync(meta, 0, sizeof(uint32_t), s) != cudaSuccess) {
    (void)cudaGetLastError();
    return noalloc_fail(GBJ_ERR_CUDA, "join_agg_noalloc: cudaMemsetAsync failed");
  }
  k_noalloc_init_out<<<1, 32, 0, s>>>(spec, d_out);
  if (n_build)
    k_join_build<<<grid_for_sms(d.sm_count, n_build, kThreads), kThreads, 0, s>>>(d_build_keys, n_build, table,
                                                                                   slots - 1, meta);
  if (n_probe)
    launch_probe(d.sm_count, d_probe_keys, d_probe_payload, n_probe, table, slots - 1,
                 d_build_payload, meta, spec, d_out, s);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return noalloc_fail(GBJ_ERR_CUDA, cudaGetErrorString(e));
  return GBJ_OK;
}

}  // extern "C"

// Shared by every ordered compaction (compact.cuh): the total row count.
__global__ void gbj::k_compact_total(const uint64_t *off, uint64_t ntiles, uint64_t *dst) {
  *dst = off[ntiles];
}
