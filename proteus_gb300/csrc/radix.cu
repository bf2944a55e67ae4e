// Radix partitioning and the partitioned (radix) hash join.
//
// Stands in for the GPU radix join of the reference: HashPartitioner +
// build_partitions (core/olap/lib/operators/gpu/
// gpu-partitioned-hash-join-chained.cpp:249-404,
// gpu-partitioned-hash-join-chained-helpers.cpp:243-481) followed by the
// per-partition shared-memory build/probe loop of
// GpuPartitionedHashJoinChained (gpu-partitioned-hash-join-chained.cpp:
// 612-1586), and for the CPU RJStepwise / partitionHT path
// (core/platform/lib/util/radix/joins/radix-join.cpp:253-375).  Like the
// reference's GPU partitioner it uses two passes for wide fan-outs (there
// 7 + 6 bits); each pass here is a tile sort rather than bucket chains.
//
// GB300 layout:
//  * a histogram kernel counts the final partition ids (<= 2^15) once;
//  * each pass (<= 8 digit bits) sorts 4096-tuple tiles by digit in shared
//    memory (one histogram row per warp gives every tuple its rank), takes
//    one output range per digit with a single global atomic, and writes the
//    tile digit-run by digit-run, so stores are coalesced and at most 256
//    output regions are open per pass (the first pass of a 2^14 fan-out
//    writes 128 regions; the second writes inside one 32 MB bucket).  The
//    pass is software-pipelined: a CTA issues the next tile's loads as soon
//    as the current tile sits in shared memory, and the output-range atomic
//    is in flight while the tile is scattered on chip;
//  * radix bits are chosen so the largest build partition fits an on-chip
//    table of kRMax tuples (the bench's 2^27-row side: 16384 partitions of
//    8192 +- 90 tuples);
//  * the join kernel is persistent: CTAs pull work items (partition, build
//    chunk, probe chunk) from an atomic counter, so a skewed probe partition
//    (Zipf keys) is spread over many SMs.  The on-chip table stores keys and
//    values in two arrays; a probe reads four keys per 16-byte shared load
//    and resolves match / empty with bit masks, so nearly every probe is one
//    load.  The partition that INT32_MIN (the empty marker) hashes to uses
//    an index table instead.
#include <algorithm>
#include <cmath>

#include "gbj_internal.cuh"
#include "radix.cuh"
#include "scan.cuh"
#include "tma.cuh"

using namespace gbj;

namespace {

// Tile shapes of the partition passes: 0 = 2048 tuples x 256 threads (4
// CTAs per SM), for passes of up to 7 digit bits with 8-byte pair output;
// 1 = 4096 x 512 (2 CTAs per SM), for 8-bit passes and 4-byte column
// output, whose digit runs would be too short in a smaller tile.  Measured
// on GB300 (radix join, R 2^27, S 2^29, 14 bits; ms of tile passes per 60
// launches): 2048 x 256 66.0, 3072 x 256 68.1, 4096 x 512 70.1, 4096 x 256
// 80.7, 2048 x 512 85.0, 4096 x 1024 95.6, 1024 x 256 102.4; the group-by's
// 8-bit column passes ran 60 % longer with the small tile.
template <int kSh>
struct TileShape {
  static constexpr int tile = kSh == 0 ? 2048 : 4096;
  static constexpr int threads = kSh == 0 ? 256 : 512;  // >= 256: one thread per digit in the scans
  static constexpr int per = tile / threads;            // tuples per thread
  static constexpr int warps = threads / 32;
  static constexpr int ctas = 1024 / threads;  // CTAs per SM (64 registers per thread)
};
constexpr int kMaxDigits = 256;      // <= 8 digit bits per pass
#ifndef GBJ_TILE_TMA
#define GBJ_TILE_TMA 0
#endif
// Tile passes load through bulk copies when set.  Measured on GB300 (radix
// join, R 2^27, S 2^29, 14 bits): 77.3 ms of tile passes per 60 launches with
// bulk copies against 70.0 ms through registers -- the copies add a shared
// read of every tuple to a kernel bound by its shared-memory pipe, and the
// pair passes have only one 32 KB stage -- so registers are the default.
constexpr bool kTileTma = GBJ_TILE_TMA;
constexpr int32_t kEmpty = INT32_MIN;

// Digit functions: of the key itself (GBJ_DIGIT_KEY), of fmix32(key)
// (GBJ_DIGIT_HASH), or of a tuple word that already holds fmix32(key)
// (kDigitPre: the partitioned join's tuples).
constexpr int kDigitPre = 2;

template <int kDigit>
__device__ __forceinline__ uint32_t digit_of(int32_t key, int shift, uint32_t mask) {
  const uint32_t v = kDigit == GBJ_DIGIT_HASH ? gbjd::fmix32((uint32_t)key) : (uint32_t)key;
  return (v >> shift) & mask;
}

// Global histogram of partition ids (shared-memory counts, one global
// atomic per non-empty bin and CTA).
template <int kDigit>
__global__ void __launch_bounds__(1024)
    k_pid_hist(const int32_t *__restrict__ keys, uint64_t n, int shift, uint32_t pmask,
               uint32_t *__restrict__ ghist) {
  extern __shared__ uint32_t sh[];
  const uint32_t P = pmask + 1;
  for (uint32_t p = threadIdx.x; p < P; p += blockDim.x) sh[p] = 0;
  __syncthreads();
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  uint64_t done = 0;
  if ((reinterpret_cast<uintptr_t>(keys) & 15) == 0) {
    // 16-byte loads, four in flight per thread (16 keys)
    const int4 *k4 = reinterpret_cast<const int4 *>(keys);
    const uint64_t n4 = n / 4;
    uint64_t i = tid;
    for (; i + 3 * stride < n4; i += 4 * stride) {
      int4 k[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) k[u] = __ldcs(k4 + i + u * stride);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        atomicAdd(&sh[digit_of<kDigit>(k[u].x, shift, pmask)], 1u);
        atomicAdd(&sh[digit_of<kDigit>(k[u].y, shift, pmask)], 1u);
        atomicAdd(&sh[digit_of<kDigit>(k[u].z, shift, pmask)], 1u);
        atomicAdd(&sh[digit_of<kDigit>(k[u].w, shift, pmask)], 1u);
      }
    }
    for (; i < n4; i += stride) {
      const int4 k = __ldcs(k4 + i);
      atomicAdd(&sh[digit_of<kDigit>(k.x, shift, pmask)], 1u);
      atomicAdd(&sh[digit_of<kDigit>(k.y, shift, pmask)], 1u);
      atomicAdd(&sh[digit_of<kDigit>(k.z, shift, pmask)], 1u);
      atomicAdd(&sh[digit_of<kDigit>(k.w, shift, pmask)], 1u);
    }
    done = n4 * 4;
  }
  for (uint64_t i = done + tid; i < n; i += stride)
    atomicAdd(&sh[digit_of<kDigit>(__ldg(keys + i), shift, pmask)], 1u);
  __syncthreads();
  for (uint32_t p = threadIdx.x; p < P; p += blockDim.x)
    if (sh[p]) atomicAdd(&ghist[p], sh[p]);
}

template <int kSh>
struct TileSmem {
  uint32_t whist[TileShape<kSh>::warps][kMaxDigits];  // per-warp digit counts, then each warp's run start
  int2 sorted[TileShape<kSh>::tile];
  uint32_t gdelta[kMaxDigits];  // output position of sorted[i] = gdelta[digit] + i
  uint32_t wsum[8];
};

// One partition pass.  Tiles of kTile tuples: contiguous from the SoA input
// (kPairsIn = false), or, for a second pass, kTile-tuple pieces of each
// parent bucket of the AoS input (tile_off = prefix of tiles per bucket).
// digit = (f(key) >> dshift) & dmask; the output cursor of (bucket b,
// digit d) is cursor[b * (dmask + 1) + d].  kHashLoad: the SoA keys are
// replaced by fmix32(key) as they are loaded (the tuples then carry the
// hash and kDigit is kDigitPre).  Row positions are below 2^31, so tile
// arithmetic is 32-bit.
//
// kTma: the input tiles arrive by bulk copies (cp.async.bulk) into a 32 KB
// shared-memory ring behind TileSmem -- two 16 KB stages (key columns
// without values: two tiles ahead) or one 32 KB stage (pairs, or keys and
// values: one tile ahead) -- instead of through registers.  A copy covers
// the 16-byte aligned middle of the tile; the (at most three) tuples either
// side of it are loaded directly.  Input columns must be 16-byte aligned.
template <int kDigit, bool kPairsIn, bool kAoSOut, bool kHashLoad, bool kTma, int kSh>
__global__ void __launch_bounds__(TileShape<kSh>::threads, TileShape<kSh>::ctas)
    k_tile_pass(const int32_t *__restrict__ keys, const int32_t *__restrict__ vals,
                const int2 *__restrict__ pin, uint32_t n, int dshift, uint32_t dmask,
                const uint64_t *__restrict__ bucket_off, const uint64_t *__restrict__ tile_off,
                uint32_t nb, uint32_t *__restrict__ cursor, int2 *__restrict__ out_pairs,
                int32_t *__restrict__ out_k, int32_t *__restrict__ out_v, uint32_t *status) {
  constexpr int kTile = TileShape<kSh>::tile, kTileThreads = TileShape<kSh>::threads;
  constexpr int kTilePer = TileShape<kSh>::per, kTileWarps = TileShape<kSh>::warps;
  constexpr uint32_t kRingBytes = kTile * 8;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TileSmem<kSh> &S = *reinterpret_cast<TileSmem<kSh> *>(smem_raw);
  unsigned char *ring = smem_raw + sizeof(TileSmem<kSh>);
  uint64_t *bars = reinterpret_cast<uint64_t *>(ring + kRingBytes);
  const uint32_t stage_bytes = (kPairsIn || vals) ? kRingBytes : kRingBytes / 2;
  const uint32_t nst = kRingBytes / stage_bytes;  // stages: 1 or 2
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t ndig = dmask + 1;
  const uint32_t ntiles = kPairsIn ? (uint32_t)tile_off[nb] : (n + kTile - 1) / kTile;
  // tile t -> its rows [lo, hi) and bucket b
  auto tile_range = [&](uint32_t t, uint32_t &lo, uint32_t &hi, uint32_t &b) {
    b = 0;
    if (kPairsIn) {
      uint32_t a = 0, z = nb;  // tile_off[a] <= t < tile_off[z]
      while (z - a > 1) {
        const uint32_t mid = (a + z) >> 1;
        if (tile_off[mid] <= t) a = mid; else z = mid;
      }
      b = a;
      const uint32_t bend = (uint32_t)bucket_off[b + 1];
      lo = (uint32_t)bucket_off[b] + (t - (uint32_t)tile_off[b]) * kTile;
      hi = lo + kTile < bend ? lo + kTile : bend;
    } else {
      lo = t * kTile;
      hi = lo + kTile < n ? lo + kTile : n;
    }
  };
  int2 tup[kTilePer];
  auto load_tile = [&](uint32_t lo, uint32_t hi) {
#pragma unroll
    for (int j = 0; j < kTilePer; ++j) {
      const uint32_t i = lo + tid + j * kTileThreads;
      if (i < hi) {
        if (kPairsIn) {
          tup[j] = __ldcs(pin + i);
        } else {
          // (kHashLoad: hashed when the tile is consumed, so this prefetch
          // stays in flight through the previous tile's write phase)
          tup[j].x = __ldcs(keys + i);
          tup[j].y = vals ? __ldcs(vals + i) : (int32_t)i;
        }
      }
    }
  };
  // kTma: the bulk-copied range [a, e) of the tile [lo, hi)
  auto tma_range = [&](uint32_t l, uint32_t h, uint32_t &a, uint32_t &e) {
    if (kPairsIn) {  // 8-byte tuples: even positions are 16-byte aligned
      a = (l + 1) & ~1u;
      e = h & ~1u;
    } else {  // 4-byte columns: tiles start at multiples of kTile
      a = l;
      e = l + ((h - l) & ~3u);
    }
    if (e < a) e = a;
  };
  auto issue = [&](uint32_t tt, uint32_t st) {
    uint32_t l, h, bb, a, e;
    tile_range(tt, l, h, bb);
    tma_range(l, h, a, e);
    unsigned char *dst = ring + st * stage_bytes;
    const uint32_t cols = kPairsIn ? 2 : (vals ? 2 : 1);
    gbjd::mbar_arrive_expect_tx(&bars[st], (e - a) * 4 * cols);
    if (e > a) {
      if (kPairsIn) {
        gbjd::bulk_load(dst, pin + a, (e - a) * 8, &bars[st]);
      } else {
        gbjd::bulk_load(dst, keys + a, (e - a) * 4, &bars[st]);
        if (vals) gbjd::bulk_load(dst + kTile * 4, vals + a, (e - a) * 4, &bars[st]);
      }
    }
  };
  auto read_tile = [&](uint32_t l, uint32_t h, uint32_t st) {
    uint32_t a, e;
    tma_range(l, h, a, e);
    const unsigned char *src = ring + st * stage_bytes;
#pragma unroll
    for (int j = 0; j < kTilePer; ++j) {
      const uint32_t i = l + tid + j * kTileThreads;
      if (i < h) {
        if (i >= a && i < e) {
          if (kPairsIn) {
            tup[j] = reinterpret_cast<const int2 *>(src)[i - a];
          } else {
            tup[j].x = reinterpret_cast<const int32_t *>(src)[i - a];
            tup[j].y = vals ? reinterpret_cast<const int32_t *>(src + kTile * 4)[i - a] : (int32_t)i;
          }
        } else if (kPairsIn) {
          tup[j] = __ldcs(pin + i);
        } else {
          tup[j].x = __ldcs(keys + i);
          tup[j].y = vals ? __ldcs(vals + i) : (int32_t)i;
        }
      }
    }
  };
  uint32_t t = blockIdx.x, lo = 0, hi = 0;
  uint32_t b = 0, it = 0;
  if (kTma) {
    if (tid == 0) {
      gbjd::mbar_init(&bars[0], 1);
      gbjd::mbar_init(&bars[1], 1);
      gbjd::mbar_init_fence();
    }
    __syncthreads();
    if (tid == 0)
      for (uint32_t k = 0; k < nst; ++k)
        if (t + k * gridDim.x < ntiles) issue(t + k * gridDim.x, k);
  } else if (t < ntiles) {
    tile_range(t, lo, hi, b);
    load_tile(lo, hi);
  }
  // Software pipeline: the next tile's loads are issued once this tile's
  // tuples sit in shared memory, so their DRAM latency overlaps the write
  // phase; the cursor atomic's L2 round trip overlaps the shared scatter.
  for (; t < ntiles; t += gridDim.x, ++it) {
    if (kTma) {
      tile_range(t, lo, hi, b);
      const uint32_t st = it % nst;
      const bool ok = gbjd::mbar_wait(&bars[st], (it / nst) & 1, kSpinLimit);
      if (__syncthreads_or(!ok)) {
        // a copy did not complete: report, wait (bounded) for the other
        // stage's copy, and stop
        if (tid == 0) {
          gbjd::latch(status, GBJ_DEV_TIMEOUT);
          if (nst == 2 && t + gridDim.x < ntiles)
            gbjd::mbar_wait(&bars[(it + 1) % nst], ((it + 1) / nst) & 1, kSpinLimit);
        }
        return;
      }
      read_tile(lo, hi, st);
    }
    for (uint32_t d = lane; d < ndig; d += 32) S.whist[warp][d] = 0;
    __syncwarp();
    const uint32_t cnt = hi - lo;
    uint32_t dg[kTilePer], rk[kTilePer];
#pragma unroll
    for (int j = 0; j < kTilePer; ++j) {
      if (kHashLoad) tup[j].x = (int32_t)gbjd::fmix32((uint32_t)tup[j].x);
      if (tid + j * kTileThreads < cnt) {
        dg[j] = digit_of<kDigit>(tup[j].x, dshift, dmask);
        rk[j] = atomicAdd(&S.whist[warp][dg[j]], 1u);
      }
    }
    __syncthreads();
    // kTma: every thread has read this stage; refill it two tiles ahead
    if (kTma && tid == 0 && t + nst * gridDim.x < ntiles) issue(t + nst * gridDim.x, it % nst);
    // per digit: the tile total (the per-warp starts follow the digit scan)
    uint32_t tot = 0;
    if ((uint32_t)tid < ndig) {
#pragma unroll
      for (int w = 0; w < kTileWarps; ++w) tot += S.whist[w][tid];
    }
    // this tile's run of each digit in the output (consumed after the scatter)
    uint32_t gpos = 0;
    if ((uint32_t)tid < ndig && tot) gpos = atomicAdd(&cursor[(uint64_t)b * ndig + tid], tot);
    // exclusive scan of the digit totals (ndig <= 256: warps 0..7)
    uint32_t incl = 0;
    if (tid < kMaxDigits) {
      incl = tot;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      if (lane == 31) S.wsum[warp] = incl;
    }
    __syncthreads();
    uint32_t my_start = 0;
    if ((uint32_t)tid < ndig) {
      uint32_t add = 0;
      for (int w = 0; w < warp; ++w) add += S.wsum[w];
      my_start = add + incl - tot;
      // absolute start of each warp's run of this digit in the tile
      uint32_t run = my_start;
#pragma unroll
      for (int w = 0; w < kTileWarps; ++w) {
        const uint32_t c = S.whist[w][tid];
        S.whist[w][tid] = run;
        run += c;
      }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kTilePer; ++j) {
      if (tid + j * kTileThreads < cnt) {
        const uint32_t pos = S.whist[warp][dg[j]] + rk[j];
        S.sorted[pos] = tup[j];
      }
    }
    // written after the scatter, so the cursor atomic's round trip overlaps it
    // (modulo 2^32: gdelta + i is the output position)
    if ((uint32_t)tid < ndig) S.gdelta[tid] = gpos - my_start;
    const uint32_t tn = t + gridDim.x;
    if (!kTma && tn < ntiles) {
      tile_range(tn, lo, hi, b);
      load_tile(lo, hi);
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kTilePer; ++j) {
      const uint32_t i = tid + j * kTileThreads;
      if (i < cnt) {
        // the digit again from the key: cheaper than storing it beside the
        // tuple at the scatter (a bank-conflicting shared store) and loading it
        const int2 v = S.sorted[i];
        const uint32_t g = S.gdelta[digit_of<kDigit>(v.x, dshift, dmask)] + i;
        if (kAoSOut) {
          out_pairs[g] = v;
        } else {
          out_k[g] = v.x;
          out_v[g] = v.y;
        }
      }
    }
    __syncthreads();
  }
}

// cursor2[p] = off[p]; for a two-pass partition also the pass-1 bucket
// starts cursor1[b] = bucket_off[b] = off[b << bits2] (bucket_off[B1] = n).
__global__ void k_cursors(const uint64_t *__restrict__ off, uint32_t P, int bits2,
                          uint32_t *__restrict__ cursor1, uint32_t *__restrict__ cursor2,
                          uint64_t *__restrict__ bucket_off) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < P) {
    cursor2[p] = (uint32_t)off[p];
    if (cursor1 && (p & ((1u << bits2) - 1)) == 0) {
      cursor1[p >> bits2] = (uint32_t)off[p];
      bucket_off[p >> bits2] = off[p];
    }
  }
  if (cursor1 && p == 0) bucket_off[P >> bits2] = off[P];
}

// Tiles of `tile` tuples per pass-1 bucket (the second pass's tile shape).
__global__ void k_bucket_tiles(const uint64_t *__restrict__ bucket_off, uint32_t nb, uint32_t tile,
                               uint64_t *__restrict__ tiles) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < nb) tiles[b] = (bucket_off[b + 1] - bucket_off[b] + tile - 1) / tile;
}

// ---------------------------------------------------------------- join

// Work items per partition: ceil(|R_p| / rmax) build chunks times
// ceil(|S_p| / w) probe chunks (zero when either side is empty).
__global__ void k_join_items(const uint64_t *__restrict__ ro, const uint64_t *__restrict__ so,
                             uint32_t P, uint32_t rmax, uint64_t w, uint64_t *__restrict__ items) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  const uint64_t nr = ro[p + 1] - ro[p], ns = so[p + 1] - so[p];
  items[p] = (nr && ns) ? ((nr + rmax - 1) / rmax) * ((ns + w - 1) / w) : 0;
}

// Partition of work item `item`: largest p with item_off[p] <= item, where
// item_off[0] = 0 <= item < item_off[P] = total.  Starts from the
// proportional guess and gallops, so the common case (about one item per
// partition) costs two or three dependent loads.
__device__ __forceinline__ uint32_t item_partition(const uint64_t *__restrict__ off, uint32_t P,
                                                   uint64_t total, uint64_t item) {
  uint32_t lo = (uint32_t)((item * (uint64_t)P) / total);
  if (lo >= P) lo = P - 1;
  uint32_t hi;
  if (off[lo] <= item) {
    uint32_t step = 1;
    hi = lo + 1;
    while (hi < P && off[hi] <= item) {
      lo = hi;
      step <<= 1;
      hi = lo + step < P ? lo + step : P;
    }
  } else {
    uint32_t step = 1;
    hi = lo;
    for (;;) {  // off[hi] > item; off[0] = 0 <= item ends the walk
      lo = hi > step ? hi - step : 0;
      if (off[lo] <= item) break;
      hi = lo;
      step <<= 1;
    }
  }
  while (hi - lo > 1) {  // off[lo] <= item < off[hi]
    const uint32_t mid = (lo + hi) >> 1;
    if (off[mid] <= item) lo = mid; else hi = mid;
  }
  return lo;
}

// kAggRows: both sides carry row positions; a match first compares the
// minor keys (when given), then reads the payloads by row.
enum : int { kAggGeneric = 0, kAggCountXor = 1, kAggCountProduct = 2, kAggRows = 3 };

// Columns a kAggRows match reads by row position (any may be null; the
// minor-key columns are both set or both null).
struct RowCols {
  const int32_t *bmin, *pmin, *bpay, *ppay;
};

// The join works on hashed tuples: the first word of every partitioned
// tuple is h = fmix32(key), which is a bijection of the 32-bit keys, so
// h equality is key equality and the key itself is fmix32_inv(h) when an
// aggregate reads it.  The partition id is the low `bits` bits of h; the
// on-chip table places h by its high bits (independent of the partition).
//
// Table: 4-slot buckets; bucket b = slots [4b, 4b + 4).  An insert tries
// the four slots of its home bucket, then the next bucket; a probe reads a
// whole bucket with one 16-byte shared load and stops at a bucket with an
// empty slot (slots only fill during the build, so a key was never placed
// past a bucket that still has room).
__device__ __forceinline__ uint32_t home_bucket(uint32_t h, uint32_t nb) { return __umulhi(h, nb); }

template <int kAgg>
__device__ __forceinline__ void join_match(const gbj::AggSpec &spec, const RowCols &rc, gbjd::Acc &acc,
                                           int64_t &a_cnt, int64_t &a_sum, uint32_t h, int32_t bv,
                                           int32_t pv) {
  if (kAgg == kAggCountXor) {
    // row ids are non-negative: their xor is a zero-extended 32-bit value
    a_cnt += 1;
    a_sum += (uint32_t)(bv ^ pv);
  } else if (kAgg == kAggCountProduct) {
    a_cnt += 1;
    a_sum += (int64_t)bv * (int64_t)pv;
  } else if (kAgg == kAggRows) {
    // the minor-key check of the reference's partitioned join
    // (gpu-partitioned-hash-join-chained.cpp:1284-1333)
    if (rc.bmin && __ldg(rc.bmin + bv) != __ldg(rc.pmin + pv)) return;
    const int64_t b = rc.bpay ? __ldg(rc.bpay + bv) : 0;
    const int64_t p = rc.ppay ? __ldg(rc.ppay + pv) : 0;
    acc.update(spec, (int32_t)gbjd::fmix32_inv(h), b, p, bv, pv);
  } else {
    acc.update(spec, (int32_t)gbjd::fmix32_inv(h), bv, pv, bv, pv);
  }
}

// One work item's extent, computed by thread 0 and shared with the block.
struct JoinItem {
  unsigned long long rb, sb;  // first build / probe tuple (global index)
  uint32_t m, ns;             // build chunk size, probe chunk size
  uint32_t part;
  int valid;
};

// Persistent partition join.  Dynamic shared memory holds, for the current
// build chunk of m tuples (nb = ceil(2m / 4) buckets rounded up to 16):
//   keys[4 nb] + values[4 nb]            (every partition but one), or
//   pairs[kRMax] + index[4 nb] (16-bit) (the partition whose tuples may hash
//                                         to the empty marker),
// followed by the per-warp probe queues.  kCtas blocks share an SM, so one
// block's clear / build / barriers overlap another's probes.
template <int kRMax, int kThreads, int kCtas, int kAgg>
__global__ void __launch_bounds__(kThreads, kCtas)
    k_radix_join(const int2 *__restrict__ R, const uint64_t *__restrict__ ro,
                 const int2 *__restrict__ S, const uint64_t *__restrict__ so,
                 const uint64_t *__restrict__ item_off, uint32_t P, uint32_t w,
                 uint32_t sentinel_part, gbj::AggSpec spec, RowCols rc, int64_t *out,
                 unsigned long long *item_ctr) {
  static_assert(2 * kRMax + 64 <= 65535, "16-bit index entries");
  constexpr uint32_t kCapMax = 2 * kRMax + 64;
  extern __shared__ __align__(16) unsigned char smem[];
  int32_t *tkey = reinterpret_cast<int32_t *>(smem);
  int32_t *tval = tkey + kCapMax;
  int2 *rp = reinterpret_cast<int2 *>(smem);
  unsigned short *tab = reinterpret_cast<unsigned short *>(rp + kRMax);
  // unresolved probes of one round, 128 per warp: {h, probe value, next bucket, -}
  int4 *queue = reinterpret_cast<int4 *>(tval + kCapMax);
  __shared__ int64_t red[32 * GBJ_MAX_AGGS];
  __shared__ JoinItem s_it;
  __shared__ int s_dup;
  gbjd::Acc acc;  // the specialised accumulators fill it only at the end
  if (kAgg != kAggCountXor && kAgg != kAggCountProduct) acc.init(spec);
  int64_t a_cnt = 0, a_sum = 0;
  const unsigned long long total = item_off[P];
  // thread 0: claims the next item and resolves its extent
  auto fetch = [&]() {
    const unsigned long long item = atomicAdd(item_ctr, 1ull);
    s_it.valid = item < total;
    if (item < total) {
      const uint32_t p = item_partition(item_off, P, total, item);
      const uint64_t r0 = ro[p], r1 = ro[p + 1], s0 = so[p], s1 = so[p + 1];
      const uint64_t nrc = (r1 - r0 + kRMax - 1) / kRMax;
      const uint64_t local = item - item_off[p];
      const uint64_t rb = r0 + (local % nrc) * kRMax, sb = s0 + (local / nrc) * w;
      s_it.rb = rb;
      s_it.m = (uint32_t)((rb + kRMax < r1 ? rb + kRMax : r1) - rb);
      s_it.sb = sb;
      s_it.ns = (uint32_t)((sb + w < s1 ? sb + w : s1) - sb);
      s_it.part = p;
    }
  };
  if (threadIdx.x == 0) fetch();
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  int4 *wq = queue + (threadIdx.x >> 5) * (4 * 32);
  for (;;) {
    if (!s_it.valid) break;
    const int2 *Rp = R + s_it.rb;
    const int2 *Sp = S + s_it.sb;
    const uint32_t m = s_it.m, ns = s_it.ns;
    const bool fast = s_it.part != sentinel_part;
    const uint32_t nb = ((2 * m + 3) / 4 + 15) & ~15u;  // buckets
    const uint32_t cap = 4 * nb;
    if (threadIdx.x == 0) s_dup = 0;
    if (fast) {
      // ---- keys + values table of 4-slot buckets ----
      int4 *tk4 = reinterpret_cast<int4 *>(tkey);
      for (uint32_t i = threadIdx.x; i < nb; i += kThreads) tk4[i] = make_int4(kEmpty, kEmpty, kEmpty, kEmpty);
      __syncthreads();
      bool dup = false;
      // An insert CASes the slots of its home bucket, starting at a slot
      // chosen by hash bits and wrapping within the bucket, then passes to
      // the next bucket.  No read of the bucket first: a CAS is as cheap as
      // a shared load and returns the slot's key, which also reveals a
      // duplicate (equal keys try slots in the same order, so a later one
      // meets the earlier one before any empty slot).
      auto insert = [&](int2 t) {
        uint32_t b = home_bucket((uint32_t)t.x, nb);
        const uint32_t o = ((uint32_t)t.x >> 16) & 3u;
        for (uint32_t step = 0; step < nb; ++step) {
#pragma unroll
          for (uint32_t j = 0; j < 4; ++j) {
            const uint32_t sl = 4 * b + ((o + j) & 3u);
            const int32_t old = atomicCAS(&tkey[sl], kEmpty, t.x);
            if (old == kEmpty) {
              tval[sl] = t.y;
              return;
            }
            dup |= old == t.x;
          }
          b = b + 1 == nb ? 0 : b + 1;
        }
      };
      // the whole chunk's loads in flight at once (8 per thread per round)
      for (uint32_t i0 = threadIdx.x; i0 < m; i0 += 8 * kThreads) {
        int2 t[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const uint32_t i = i0 + u * kThreads;
          if (i < m) t[u] = __ldcs(Rp + i);
        }
#pragma unroll
        for (int u = 0; u < 8; ++u)
          if (i0 + u * kThreads < m) insert(t[u]);
      }
      if (dup) s_dup = 1;
    } else {
      // ---- pairs + 16-bit index table (any hash value allowed) ----
      uint32_t *tab32 = reinterpret_cast<uint32_t *>(tab);
      for (uint32_t i = threadIdx.x; i < cap / 2; i += kThreads) tab32[i] = 0;
      for (uint32_t i = threadIdx.x; i < m; i += kThreads) rp[i] = Rp[i];
      __syncthreads();
      bool dup = false;
      for (uint32_t i = threadIdx.x; i < m; i += kThreads) {
        const int32_t k = rp[i].x;
        uint32_t hh = __umulhi((uint32_t)k, cap);
        for (uint32_t step = 0; step < cap; ++step) {
          const unsigned short old = atomicCAS(&tab[hh], (unsigned short)0, (unsigned short)(i + 1));
          if (old == 0) break;
          dup |= (rp[old - 1].x == k);
          if (++hh == cap) hh = 0;
        }
      }
      if (dup) s_dup = 1;
    }
    __syncthreads();
    const bool unique = s_dup == 0;
    // next item: fetched now, consumed after the closing barrier (every
    // thread has read this item's extent above)
    if (threadIdx.x == 0) fetch();
    if (fast) {
      const int4 *tk4 = reinterpret_cast<const int4 *>(tkey);
      // One bucket, general form (duplicate build keys, queued probes):
      // every match; true when the probe is done.
      auto bucket = [&](uint32_t h, int32_t v, uint32_t b) -> bool {
        const int4 kk = tk4[b];
        const int32_t k = (int32_t)h;
        uint32_t hits = (kk.x == k) | ((kk.y == k) << 1) | ((kk.z == k) << 2) | ((kk.w == k) << 3);
        const bool room = (kk.x == kEmpty) | (kk.y == kEmpty) | (kk.z == kEmpty) | (kk.w == kEmpty);
        while (hits) {
          join_match<kAgg>(spec, rc, acc, a_cnt, a_sum, h, tval[4 * b + __ffs(hits) - 1], v);
          if (unique) return true;
          hits &= hits - 1;
        }
        return room;
      };
      // Probe rounds of 4 tuples per thread: every probe checks its home
      // bucket; the few that must continue go to the warp's own queue, which
      // the warp's lanes then drain together.  The next round's tuples are
      // loaded while this round is probed.  With unique build keys a home
      // bucket resolves a probe without a loop: at most one slot matches.
      int2 nxt[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const uint32_t j = threadIdx.x + u * kThreads;
        nxt[u] = j < ns ? __ldcs(Sp + j) : make_int2(0, 0);
      }
      for (uint32_t j0 = 0; j0 < ns; j0 += 4 * kThreads) {
        int2 t[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          t[u] = nxt[u];
          const uint32_t j = j0 + 4 * kThreads + threadIdx.x + u * kThreads;
          nxt[u] = j < ns ? __ldcs(Sp + j) : make_int2(0, 0);
        }
        uint32_t qn = 0;  // warp-uniform queue length
        if (unique && kAgg != kAggGeneric && kAgg != kAggRows) {
          uint32_t more = 0;  // bit u: tuple u must go on past its home bucket
          // the specialised aggregates: the match folded in without a
          // branch (at most one slot matches; the value load is issued
          // whether or not it did), and the queue touched only when some
          // lane of the warp must go on
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const bool valid = j0 + threadIdx.x + u * kThreads < ns;
            const uint32_t b = home_bucket((uint32_t)t[u].x, nb);
            const int4 kk = tk4[b];
            const int32_t k = t[u].x;
            const bool e0 = kk.x == k, e1 = kk.y == k, e2 = kk.z == k, e3 = kk.w == k;
            const bool room = (kk.x == kEmpty) | (kk.y == kEmpty) | (kk.z == kEmpty) | (kk.w == kEmpty);
            const bool found = valid & (e0 | e1 | e2 | e3);
            const int32_t bv = tval[4 * b + (e0 ? 0 : e1 ? 1 : e2 ? 2 : 3)];
            a_cnt += found;
            if (kAgg == kAggCountXor) a_sum += found ? (uint32_t)(bv ^ t[u].y) : 0u;
            else a_sum += found ? (int64_t)bv * (int64_t)t[u].y : 0;
            more |= (uint32_t)(valid & !found & !room) << u;
          }
          if (__any_sync(0xffffffffu, more != 0)) {
#pragma unroll
            for (int u = 0; u < 4; ++u) {
              const bool mo = (more >> u) & 1u;
              const unsigned bal = __ballot_sync(0xffffffffu, mo);
              if (mo) {
                const uint32_t b = home_bucket((uint32_t)t[u].x, nb);
                wq[qn + __popc(bal & lt)] = make_int4(t[u].x, t[u].y, (int)(b + 1 == nb ? 0 : b + 1), 0);
              }
              qn += __popc(bal);
            }
          }
        } else {
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const bool valid = j0 + threadIdx.x + u * kThreads < ns;
            const uint32_t h = (uint32_t)t[u].x;
            const uint32_t b = home_bucket(h, nb);
            bool mo;
            if (unique) {
              const int4 kk = tk4[b];
              const bool e0 = kk.x == t[u].x, e1 = kk.y == t[u].x, e2 = kk.z == t[u].x, e3 = kk.w == t[u].x;
              const bool room = (kk.x == kEmpty) | (kk.y == kEmpty) | (kk.z == kEmpty) | (kk.w == kEmpty);
              const bool found = valid & (e0 | e1 | e2 | e3);
              if (found) {
                const uint32_t idx = e0 ? 0 : e1 ? 1 : e2 ? 2 : 3;
                join_match<kAgg>(spec, rc, acc, a_cnt, a_sum, h, tval[4 * b + idx], t[u].y);
              }
              mo = valid & !found & !room;
            } else {
              mo = valid && !bucket(h, t[u].y, b);
            }
            const unsigned bal = __ballot_sync(0xffffffffu, mo);
            if (mo) wq[qn + __popc(bal & lt)] = make_int4(t[u].x, t[u].y, (int)(b + 1 == nb ? 0 : b + 1), 0);
            qn += __popc(bal);
          }
        }
        if (qn) {
          __syncwarp();
          for (uint32_t i = lane; i < qn; i += 32) {
            const int4 e = wq[i];
            uint32_t b = (uint32_t)e.z;
            for (uint32_t step = 1; step < nb; ++step) {
              if (bucket((uint32_t)e.x, e.y, b)) break;
              b = b + 1 == nb ? 0 : b + 1;
            }
          }
          __syncwarp();
        }
      }
    } else {
      // index table: plain linear probing, one slot per step
      for (uint32_t j0 = threadIdx.x; j0 < ns; j0 += 4 * kThreads) {
        int2 t[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const uint32_t j = j0 + u * kThreads;
          t[u] = j < ns ? __ldcs(Sp + j) : make_int2(0, 0);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          if (j0 + u * kThreads >= ns) continue;
          const int32_t k = t[u].x;
          uint32_t hh = __umulhi((uint32_t)k, cap);
          for (uint32_t step = 0; step < cap; ++step) {
            const unsigned short idx = tab[hh];
            if (idx == 0) break;
            const int2 bt = rp[idx - 1];
            if (bt.x == k) {
              join_match<kAgg>(spec, rc, acc, a_cnt, a_sum, (uint32_t)k, bt.y, t[u].y);
              if (unique) break;
            }
            if (++hh == cap) hh = 0;
          }
        }
      }
    }
    __syncthreads();
  }
  if (kAgg == kAggCountXor || kAgg == kAggCountProduct) {
    acc.init(spec);
    acc.v[0] = a_cnt;
    acc.v[1] = a_sum;
  }
  gbjd::block_flush(spec, acc, red, out);
}

// keys + values table (>= pairs + 16-bit index) and the probe queue of one
// round (4 probes per thread).
template <int kRMax, int kThreads>
constexpr size_t join_smem() {
  return (size_t)2 * (2 * kRMax + 64) * sizeof(int32_t) + (size_t)4 * kThreads * sizeof(int4);
}

template <int kRMax, int kThreads, int kCtas, int kAgg>
int launch_join(gbj_ctx *ctx, const int2 *R, const uint64_t *ro, const int2 *S,
                const uint64_t *so, const uint64_t *item_off, uint32_t P,
                uint32_t w, uint32_t sentinel_part, const AggSpec &spec, const RowCols &rc,
                int64_t *out, unsigned long long *ctr, cudaStream_t s) {
  const size_t smem = join_smem<kRMax, kThreads>();
  auto kern = k_radix_join<kRMax, kThreads, kCtas, kAgg>;
  GBJ_CHECK_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem));
  int per_sm = 0;
  GBJ_CHECK_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem));
  if (per_sm < 1) return set_error(ctx, GBJ_ERR_CUDA, "k_radix_join: no resident block fits");
  kern<<<ctx->sm_count * per_sm, kThreads, smem, s>>>(R, ro, S, so, item_off, P, w,
                                                     sentinel_part, spec, rc, out, ctr);
  return after_launch(ctx, "k_radix_join", s);
}

// The two join kernel shapes: 1024 threads with build chunks of 9216 tuples
// (one block per SM), or 512 threads with chunks of 4608 (two blocks per
// SM; partitions then need one more radix bit).
struct JoinShape {
  int threads, rmax;
};
constexpr JoinShape kJoinWide{1024, 9216};
constexpr JoinShape kJoinPair{512, 4608};

template <int kRMax, int kThreads, int kCtas>
int launch_join_agg(gbj_ctx *ctx, bool by_rows, const AggSpec &spec, const int2 *R, const uint64_t *ro,
                    const int2 *S, const uint64_t *so, const uint64_t *items, uint32_t P, uint32_t w,
                    uint32_t sentinel_part, const RowCols &rc, int64_t *d_out, unsigned long long *ctr,
                    cudaStream_t s) {
  if (by_rows)
    return launch_join<kRMax, kThreads, kCtas, kAggRows>(ctx, R, ro, S, so, items, P, w, sentinel_part, spec, rc,
                                                         d_out, ctr, s);
  const bool two = spec.n == 2 && spec.op[0] == GBJ_AGG_COUNT && spec.op[1] == GBJ_AGG_SUM;
  if (two && spec.operand[1] == GBJ_VAL_ROWID_XOR)
    return launch_join<kRMax, kThreads, kCtas, kAggCountXor>(ctx, R, ro, S, so, items, P, w, sentinel_part, spec,
                                                             rc, d_out, ctr, s);
  if (two && spec.operand[1] == GBJ_VAL_PRODUCT)
    return launch_join<kRMax, kThreads, kCtas, kAggCountProduct>(ctx, R, ro, S, so, items, P, w, sentinel_part,
                                                                 spec, rc, d_out, ctr, s);
  return launch_join<kRMax, kThreads, kCtas, kAggGeneric>(ctx, R, ro, S, so, items, P, w, sentinel_part, spec, rc,
                                                          d_out, ctr, s);
}

// The tile shape of a pass with `ndig` digits and pair (AoS) or column output.
int tile_shape_for(uint32_t ndig, bool aos) { return ndig <= 128 && aos ? 0 : 1; }

template <int kDigit, bool kPairsIn, bool kAoSOut, bool kHashLoad, int kSh>
int launch_tile_pass_sh(gbj_ctx *ctx, const int32_t *keys, const int32_t *vals, const int2 *pin,
                        uint64_t n, int dshift, uint32_t dmask, const uint64_t *bucket_off,
                        const uint64_t *tile_off, uint32_t nb, uint32_t *cursor, int2 *op, int32_t *ok,
                        int32_t *ov, cudaStream_t s) {
  using TS = TileShape<kSh>;
  // bulk-copy loads when the input columns are 16-byte aligned
  auto al16 = [](const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; };
  const bool tma = kTileTma && (kPairsIn ? al16(pin) : (al16(keys) && (!vals || al16(vals))));
  auto kern = tma ? k_tile_pass<kDigit, kPairsIn, kAoSOut, kHashLoad, true, kSh>
                  : k_tile_pass<kDigit, kPairsIn, kAoSOut, kHashLoad, false, kSh>;
  const size_t smem = sizeof(TileSmem<kSh>) + (tma ? (size_t)TS::tile * 8 + 16 : 0);
  GBJ_CHECK_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  GBJ_CHECK_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, TS::threads, smem));
  if (per_sm < 1) per_sm = 1;
  const uint64_t tiles_hint = (n + TS::tile - 1) / TS::tile + nb;
  const uint64_t grid = std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)ctx->sm_count * per_sm, tiles_hint));
  kern<<<(unsigned)grid, TS::threads, smem, s>>>(keys, vals, pin, (uint32_t)n, dshift, dmask, bucket_off, tile_off,
                                                 nb, cursor, op, ok, ov, ctx->d_status);
  return after_launch(ctx, "k_tile_pass", s);
}

template <int kDigit, bool kPairsIn, bool kAoSOut, bool kHashLoad>
int launch_tile_pass(gbj_ctx *ctx, const int32_t *keys, const int32_t *vals, const int2 *pin,
                     uint64_t n, int dshift, uint32_t dmask, const uint64_t *bucket_off,
                     const uint64_t *tile_off, uint32_t nb, uint32_t *cursor, int2 *op, int32_t *ok,
                     int32_t *ov, cudaStream_t s) {
  if (tile_shape_for(dmask + 1, kAoSOut) == 0)
    return launch_tile_pass_sh<kDigit, kPairsIn, kAoSOut, kHashLoad, 0>(ctx, keys, vals, pin, n, dshift, dmask,
                                                                       bucket_off, tile_off, nb, cursor, op, ok,
                                                                       ov, s);
  return launch_tile_pass_sh<kDigit, kPairsIn, kAoSOut, kHashLoad, 1>(ctx, keys, vals, pin, n, dshift, dmask,
                                                                     bucket_off, tile_off, nb, cursor, op, ok, ov,
                                                                     s);
}

// kHashOut: the tuples leave with fmix32(key) in place of the key (the
// partitioned join's layout; AoS output only), and the passes take their
// digits from that word.
template <int kDigit, bool kHashOut>
int partition_impl(gbj_ctx *ctx, const int32_t *keys, const int32_t *vals, uint64_t n, int shift,
                   int bits, int2 *out_pairs, int32_t *out_keys, int32_t *out_vals,
                   uint64_t *offsets, cudaStream_t s, int passes) {
  if ((passes == 1 && bits > 8) || (passes == 2 && bits < 2) || passes < 0 || passes > 2)
    return set_error(ctx, GBJ_ERR_UNSUPPORTED,
                     "partition: one pass takes at most 8 radix bits, two passes at least 2");
  if (n >= (1ull << 31)) return set_error(ctx, GBJ_ERR_INVALID, "partition: n >= 2^31");
  if (kHashOut && !out_pairs) return set_error(ctx, GBJ_ERR_INVALID, "partition: hashed tuples are AoS only");
  // digit function of the tile passes: of the loaded key, or of the hash word
  constexpr int kPass = kHashOut ? kDigitPre : kDigit;
  const uint32_t P = 1u << bits, pmask = P - 1;
  Scratch scratch(ctx, s);
  uint32_t *hist, *cursor2;
  uint64_t *off;
  GBJ_TRY(scratch.get(P + 1, &hist));
  GBJ_TRY(scratch.get(P + 1, &cursor2));
  GBJ_TRY(scratch.get(P + 1, &off));
  GBJ_CHECK_CUDA(ctx, cudaMemsetAsync(hist, 0, sizeof(uint32_t) * P, s));
  {
    const size_t smem = (size_t)P * sizeof(uint32_t);
    GBJ_CHECK_CUDA(ctx, cudaFuncSetAttribute(k_pid_hist<kDigit>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 1;
    GBJ_CHECK_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pid_hist<kDigit>, 1024, smem));
    const uint64_t grid = std::max<uint64_t>(
        1, std::min<uint64_t>((uint64_t)ctx->sm_count * std::max(per_sm, 1), (n + 16383) / 16384));
    k_pid_hist<kDigit><<<(unsigned)grid, 1024, smem, s>>>(keys, n, shift, pmask, hist);
    GBJ_TRY(after_launch(ctx, "k_pid_hist", s));
  }
  GBJ_TRY(scan_u32_to_u64(ctx, hist, off, P, s));
  if (passes == 1 || (passes == 0 && bits <= 8)) {
    k_cursors<<<(P + 255) / 256, 256, 0, s>>>(off, P, 0, nullptr, cursor2, nullptr);
    GBJ_TRY(after_launch(ctx, "k_cursors", s));
    if (out_pairs)
      GBJ_TRY((launch_tile_pass<kPass, false, true, kHashOut>(ctx, keys, vals, nullptr, n, shift, pmask, nullptr,
                                                              nullptr, 1, cursor2, out_pairs, nullptr, nullptr, s)));
    else
      GBJ_TRY((launch_tile_pass<kPass, false, false, false>(ctx, keys, vals, nullptr, n, shift, pmask, nullptr,
                                                            nullptr, 1, cursor2, nullptr, out_keys, out_vals, s)));
  } else {
    const int bits2 = bits / 2, bits1 = bits - bits2;
    const uint32_t B1 = 1u << bits1;
    uint32_t *cursor1;
    uint64_t *bucket_off, *tiles;
    int2 *tmp;
    GBJ_TRY(scratch.get(B1 + 1, &cursor1));
    GBJ_TRY(scratch.get(B1 + 1, &bucket_off));
    GBJ_TRY(scratch.get(B1 + 1, &tiles));
    GBJ_TRY(scratch.get(n + 1, &tmp));
    k_cursors<<<(P + 255) / 256, 256, 0, s>>>(off, P, bits2, cursor1, cursor2, bucket_off);
    GBJ_TRY(after_launch(ctx, "k_cursors", s));
    GBJ_TRY((launch_tile_pass<kPass, false, true, kHashOut>(ctx, keys, vals, nullptr, n, shift + bits2, B1 - 1,
                                                            nullptr, nullptr, 1, cursor1, tmp, nullptr, nullptr,
                                                            s)));
    const uint32_t m2 = (1u << bits2) - 1;
    const uint32_t tile2 = tile_shape_for(m2 + 1, out_pairs != nullptr) == 0 ? TileShape<0>::tile
                                                                            : TileShape<1>::tile;
    k_bucket_tiles<<<(B1 + 255) / 256, 256, 0, s>>>(bucket_off, B1, tile2, tiles);
    GBJ_TRY(after_launch(ctx, "k_bucket_tiles", s));
    GBJ_TRY(scan_u64(ctx, tiles, tiles, B1, s));
    if (out_pairs)
      GBJ_TRY((launch_tile_pass<kPass, true, true, false>(ctx, nullptr, nullptr, tmp, n, shift, m2, bucket_off,
                                                          tiles, B1, cursor2, out_pairs, nullptr, nullptr, s)));
    else
      GBJ_TRY((launch_tile_pass<kPass, true, false, false>(ctx, nullptr, nullptr, tmp, n, shift, m2, bucket_off,
                                                           tiles, B1, cursor2, nullptr, out_keys, out_vals, s)));
  }
  if (offsets) GBJ_CHECK_CUDA(ctx, cudaMemcpyAsync(offsets, off, sizeof(uint64_t) * (P + 1),
                                                   cudaMemcpyDeviceToDevice, s));
  return GBJ_OK;
}

}  // namespace

namespace gbj {

int partition_tuples(gbj_ctx *ctx, const int32_t *keys, const int32_t *vals, uint64_t n,
                     int digit, int shift, int bits, int2 *out_pairs, int32_t *out_keys,
                     int32_t *out_vals, uint64_t *offsets, cudaStream_t s, int passes, bool hash_out) {
  if (hash_out) {
    if (digit != GBJ_DIGIT_HASH) return set_error(ctx, GBJ_ERR_INVALID, "partition: hashed tuples need hash digits");
    return partition_impl<GBJ_DIGIT_HASH, true>(ctx, keys, vals, n, shift, bits, out_pairs, out_keys, out_vals,
                                                offsets, s, passes);
  }
  if (digit == GBJ_DIGIT_HASH)
    return partition_impl<GBJ_DIGIT_HASH, false>(ctx, keys, vals, n, shift, bits, out_pairs, out_keys,
                                                 out_vals, offsets, s, passes);
  return partition_impl<GBJ_DIGIT_KEY, false>(ctx, keys, vals, n, shift, bits, out_pairs, out_keys,
                                              out_vals, offsets, s, passes);
}

}  // namespace gbj

extern "C" {

int gbj_partition(gbj_ctx *ctx, const int32_t *d_keys, const int32_t *d_payload, uint64_t n,
                  int32_t digit, int32_t shift, int32_t bits, int32_t *d_out_keys,
                  int32_t *d_out_payload, uint64_t *d_offsets, void *stream) {
  if (!ctx) return GBJ_ERR_INVALID;
  if (digit != GBJ_DIGIT_KEY && digit != GBJ_DIGIT_HASH)
    return set_error(ctx, GBJ_ERR_INVALID, "partition: bad digit function");
  if (bits < 1 || bits > kMaxPartBits || shift < 0 || shift + bits > 32)
    return set_error(ctx, GBJ_ERR_INVALID, "partition: bits must be in [1, 15], shift+bits <= 32");
  if (n >= (1ULL << 31)) return set_error(ctx, GBJ_ERR_INVALID, "partition: n >= 2^31");
  if (n && (!d_keys || !d_out_keys || !d_out_payload))
    return set_error(ctx, GBJ_ERR_INVALID, "partition: null column");
  cudaStream_t s = pick_stream(ctx, stream);
  prof_mark(ctx, s);
  if (n == 0) {
    if (d_offsets)
      GBJ_CHECK_CUDA(ctx, cudaMemsetAsync(d_offsets, 0, sizeof(uint64_t) * ((1ull << bits) + 1), s));
    return GBJ_OK;
  }
  return partition_tuples(ctx, d_keys, d_payload, n, digit, shift, bits, nullptr, d_out_keys,
                          d_out_payload, d_offsets, s);
}

}  // extern "C"

// Shared body of gbj_radix_join_agg and gbj_radix_join_agg_minor.
static int radix_join_impl(gbj_ctx *ctx, const int32_t *d_build_keys, const int32_t *d_build_minor,
                           const int32_t *d_build_payload, uint64_t n_build,
                           const int32_t *d_probe_keys, const int32_t *d_probe_minor,
                           const int32_t *d_probe_payload, uint64_t n_probe,
                           const gbj_radix_params *params, const gbj_agg *aggs, int32_t n_aggs,
                           int64_t *d_out, void *stream) {
  if (!ctx || !d_out) return GBJ_ERR_INVALID;
  GBJ_TRY(validate_aggs(ctx, aggs, n_aggs));
  if (n_build >= (1ULL << 31) || n_probe >= (1ULL << 31))
    return set_error(ctx, GBJ_ERR_INVALID, "radix_join: inputs must have < 2^31 rows");
  if ((n_build && !d_build_keys) || (n_probe && !d_probe_keys))
    return set_error(ctx, GBJ_ERR_INVALID, "radix_join: null key column");
  const bool minor = d_build_minor || d_probe_minor;
  if (minor && ((n_build && !d_build_minor) || (n_probe && !d_probe_minor)))
    return set_error(ctx, GBJ_ERR_INVALID,
                     "radix_join: a minor key needs both sides (build_k_minor and probe_k_minor)");
  // Every field of the parameters is honoured or refused.
  if (params) {
    if (params->bits < 0 || params->bits > kMaxPartBits || params->log_parts < 0 ||
        params->log_parts > kMaxPartBits)
      return set_error(ctx, GBJ_ERR_UNSUPPORTED, "radix_join: radix bits must be in [0, 15]");
    if (params->passes < 0 || params->passes > 2)
      return set_error(ctx, GBJ_ERR_UNSUPPORTED, "radix_join: passes must be 0 (auto), 1 or 2");
    if (params->block != 0 && params->block != kJoinWide.threads && params->block != kJoinPair.threads)
      return set_error(ctx, GBJ_ERR_UNSUPPORTED,
                       "radix_join: the join kernel runs 512 or 1024 threads per block (block 0, 512 or 1024)");
  }
  AggSpec spec = make_spec(aggs, n_aggs);
  // Which value each side carries into the partitions.
  bool b_row = false, b_pay = false, p_row = false, p_pay = false;
  for (int j = 0; j < n_aggs; ++j) {
    switch (spec.operand[j]) {
      case GBJ_VAL_BUILD: b_pay = true; break;
      case GBJ_VAL_PROBE: p_pay = true; break;
      case GBJ_VAL_PRODUCT: b_pay = p_pay = true; break;
      case GBJ_VAL_BUILD_ROWID: b_row = true; break;
      case GBJ_VAL_PROBE_ROWID: p_row = true; break;
      case GBJ_VAL_ROWID_XOR: b_row = p_row = true; break;
      default: break;
    }
  }
  if ((b_pay && !d_build_payload && n_build) || (p_pay && !d_probe_payload && n_probe))
    return set_error(ctx, GBJ_ERR_INVALID, "radix_join: aggregate reads a missing payload");
  // Row mode: both sides carry row positions and a match reads the minor
  // keys and payloads by row (a composite key, or one side needing both its
  // payload and its row id).
  const bool by_rows = minor || (b_row && b_pay) || (p_row && p_pay);
  cudaStream_t s = pick_stream(ctx, stream);
  prof_mark(ctx, s);
  GBJ_TRY(init_agg_out(ctx, spec, d_out, s));
  if (n_build == 0 || n_probe == 0) return GBJ_OK;

  // ---- plan: fewest radix bits whose largest expected build partition
  //      (mean + 5 sd) fits the on-chip table; explicit params override ----
  const int passes = params ? params->passes : 0;
  // join kernel shape: the caller's block size, else an autotuned one, else
  // two 512-thread blocks per SM
  int block = params ? params->block : 0;
  if (!block) {
    const int32_t tb = tuned_value(ctx, tune_key("radixblock", n_build, n_probe));
    block = tb > 0 ? tb : kJoinPair.threads;
  }
  const JoinShape shape = block == kJoinWide.threads ? kJoinWide : kJoinPair;
  const uint32_t kRMax = (uint32_t)shape.rmax;
  int bits = 1;
  while (bits < kMaxPartBits) {
    const double mean = (double)n_build / (double)(1u << bits);
    if (mean + 5.0 * std::sqrt(mean) <= (double)kRMax) break;
    ++bits;
  }
  const bool explicit_bits = params && (params->log_parts > 0 || params->bits > 0);
  if (!explicit_bits) {  // an autotuned choice for this size bucket, if any
    const int32_t tb = tuned_value(ctx, tune_key(shape.threads == kJoinWide.threads ? "radix" : "radix512",
                                                 n_build, n_probe));
    if (tb > 0) bits = std::min<int>(tb, kMaxPartBits);
    // a pinned pass count bounds the automatic choice
    if (passes == 1) bits = std::min(bits, 8);
    if (passes == 2) bits = std::max(bits, 2);
  }
  if (params && params->log_parts > 0) bits = params->log_parts;
  if (params && params->bits > 0) bits = params->bits;
  if ((passes == 1 && bits > 8) || (passes == 2 && bits < 2))
    return set_error(ctx, GBJ_ERR_UNSUPPORTED,
                     "radix_join: one pass takes at most 8 radix bits, two passes at least 2");
  const uint32_t P = 1u << bits;
  const uint64_t w = 1u << 17;  // probe tuples per work item
  // tuples carry fmix32(key); the partition of the hash equal to the empty
  // marker takes the index-table path
  const uint32_t sentinel_part = (uint32_t)kEmpty & (P - 1);

  Scratch scratch(ctx, s);
  int2 *R, *S;
  uint64_t *ro, *so, *items;
  unsigned long long *ctr;
  GBJ_TRY(scratch.get(n_build + 2, &R));
  GBJ_TRY(scratch.get(n_probe + 2, &S));
  GBJ_TRY(scratch.get(P + 1, &ro));
  GBJ_TRY(scratch.get(P + 1, &so));
  GBJ_TRY(scratch.get(P + 1, &items));
  GBJ_TRY(scratch.get(1, &ctr));
  GBJ_TRY(partition_tuples(ctx, d_build_keys, b_pay && !by_rows ? d_build_payload : nullptr, n_build,
                           GBJ_DIGIT_HASH, 0, bits, R, nullptr, nullptr, ro, s, passes, true));
  GBJ_TRY(partition_tuples(ctx, d_probe_keys, p_pay && !by_rows ? d_probe_payload : nullptr, n_probe,
                           GBJ_DIGIT_HASH, 0, bits, S, nullptr, nullptr, so, s, passes, true));
  k_join_items<<<(P + 255) / 256, 256, 0, s>>>(ro, so, P, kRMax, w, items);
  GBJ_TRY(after_launch(ctx, "k_join_items", s));
  GBJ_TRY(scan_u64(ctx, items, items, P, s));
  GBJ_CHECK_CUDA(ctx, cudaMemsetAsync(ctr, 0, sizeof(unsigned long long), s));
  const RowCols rc{minor ? d_build_minor : nullptr, minor ? d_probe_minor : nullptr,
                   b_pay ? d_build_payload : nullptr, p_pay ? d_probe_payload : nullptr};
  if (shape.threads == kJoinWide.threads)
    return launch_join_agg<kJoinWide.rmax, kJoinWide.threads, 1>(ctx, by_rows, spec, R, ro, S, so, items, P, w,
                                                                 sentinel_part, rc, d_out, ctr, s);
  return launch_join_agg<kJoinPair.rmax, kJoinPair.threads, 2>(ctx, by_rows, spec, R, ro, S, so, items, P, w,
                                                               sentinel_part, rc, d_out, ctr, s);
}

extern "C" {

int gbj_radix_join_agg(gbj_ctx *ctx, const int32_t *d_build_keys,
                       const int32_t *d_build_payload, uint64_t n_build,
                       const int32_t *d_probe_keys, const int32_t *d_probe_payload,
                       uint64_t n_probe, const gbj_radix_params *params, const gbj_agg *aggs,
                       int32_t n_aggs, int64_t *d_out, void *stream) {
  return radix_join_impl(ctx, d_build_keys, nullptr, d_build_payload, n_build, d_probe_keys, nullptr,
                         d_probe_payload, n_probe, params, aggs, n_aggs, d_out, stream);
}

int gbj_radix_join_agg_minor(gbj_ctx *ctx, const int32_t *d_build_keys,
                             const int32_t *d_build_minor, const int32_t *d_build_payload,
                             uint64_t n_build, const int32_t *d_probe_keys,
                             const int32_t *d_probe_minor, const int32_t *d_probe_payload,
                             uint64_t n_probe, const gbj_radix_params *params,
                             const gbj_agg *aggs, int32_t n_aggs, int64_t *d_out,
                             void *stream) {
  if (ctx && ((n_build && !d_build_minor) || (n_probe && !d_probe_minor)))
    return set_error(ctx, GBJ_ERR_INVALID, "radix_join_minor: both minor-key columns are required");
  return radix_join_impl(ctx, d_build_keys, d_build_minor, d_build_payload, n_build, d_probe_keys,
                         d_probe_minor, d_probe_payload, n_probe, params, aggs, n_aggs, d_out, stream);
}

}  // extern "C"
