// Radix partitioning and the partitioned (radix) hash join.
//
// Stands in for the GPU radix join of the reference: HashPartitioner +
// build_partitions (core/olap/lib/operators/gpu/
// gpu-partitioned-hash-join-chained.cpp:249-404,
// gpu-partitioned-hash-join-chained-helpers.cpp:243-481) followed by the
// per-partition shared-memory build/probe loop of
// GpuPartitionedHashJoinChained (gpu-partitioned-hash-join-chained.cpp:
// 612-1586), and for the CPU RJStepwise / partitionHT path
// (core/platform/lib/util/radix/joins/radix-join.cpp:253-375).
//
// GB300 layout:
//  * one partitioning pass of up to 15 bits of fmix32(key): a count kernel
//    builds one shared-memory histogram per CTA segment, a scan turns the
//    [partition][cta] counts into write cursors, and a scatter kernel
//    re-reads its segment and writes (key, value) pairs with shared-memory
//    cursors -- no global atomics, one read of the input per pass, 8 B per
//    tuple written;
//  * radix bits chosen so an average build partition holds about half of
//    an on-chip table (kRMax tuples), so build partitions never leave
//    shared memory;
//  * the join kernel is persistent: CTAs pull work items (partition,
//    build chunk, probe chunk) from an atomic counter, so one skewed probe
//    partition (Zipf keys) is spread over many SMs.
#include <algorithm>

#include "gbj_internal.cuh"
#include "radix.cuh"
#include "scan.cuh"

using namespace gbj;

namespace {

constexpr int kPartThreads = 1024;

template <int kDigit>
__device__ __forceinline__ uint32_t digit_of(int32_t key, int shift, uint32_t pmask) {
  const uint32_t v = kDigit == GBJ_DIGIT_HASH ? gbjd::fmix32((uint32_t)key) : (uint32_t)key;
  return (v >> shift) & pmask;
}

// Count pass: CTA c histograms segment [c*seg, (c+1)*seg) into shared
// memory and stores it column c of hist[P][G].
template <int kDigit>
__global__ void __launch_bounds__(kPartThreads)
    k_part_count(const int32_t *__restrict__ keys, uint64_t n, int shift,
                 uint32_t pmask, uint64_t seg, uint32_t *__restrict__ hist) {
  extern __shared__ uint32_t sh[];
  const uint32_t P = pmask + 1;
  for (uint32_t p = threadIdx.x; p < P; p += blockDim.x) sh[p] = 0;
  __syncthreads();
  const uint64_t lo = blockIdx.x * seg;
  const uint64_t hi = lo + seg < n ? lo + seg : n;
  if (lo < hi) {
    const uint64_t qlo = lo / 4, qhi = hi / 4;  // seg % 4 == 0
    const int4 *k4 = reinterpret_cast<const int4 *>(keys);
    for (uint64_t q = qlo + threadIdx.x; q < qhi; q += blockDim.x) {
      const int4 k = __ldcs(k4 + q);
      atomicAdd(&sh[digit_of<kDigit>(k.x, shift, pmask)], 1u);
      atomicAdd(&sh[digit_of<kDigit>(k.y, shift, pmask)], 1u);
      atomicAdd(&sh[digit_of<kDigit>(k.z, shift, pmask)], 1u);
      atomicAdd(&sh[digit_of<kDigit>(k.w, shift, pmask)], 1u);
    }
    for (uint64_t i = qhi * 4 + threadIdx.x; i < hi; i += blockDim.x)
      atomicAdd(&sh[digit_of<kDigit>(keys[i], shift, pmask)], 1u);
  }
  __syncthreads();
  const uint32_t G = gridDim.x;
  for (uint32_t p = threadIdx.x; p < P; p += blockDim.x) hist[(uint64_t)p * G + blockIdx.x] = sh[p];
}

// Scatter pass: same segments; cursors start at the scanned offsets.
template <int kDigit, bool kAoS>
__global__ void __launch_bounds__(kPartThreads)
    k_part_scatter(const int32_t *__restrict__ keys, const int32_t *__restrict__ vals,
                   uint64_t n, int shift, uint32_t pmask, uint64_t seg,
                   const uint64_t *__restrict__ base, int2 *__restrict__ out_pairs,
                   int32_t *__restrict__ out_k, int32_t *__restrict__ out_v) {
  extern __shared__ uint32_t cur[];
  const uint32_t P = pmask + 1, G = gridDim.x;
  for (uint32_t p = threadIdx.x; p < P; p += blockDim.x)
    cur[p] = (uint32_t)base[(uint64_t)p * G + blockIdx.x];
  __syncthreads();
  const uint64_t lo = blockIdx.x * seg;
  const uint64_t hi = lo + seg < n ? lo + seg : n;
  auto put = [&](int32_t k, int32_t v) {
    const uint32_t pos = atomicAdd(&cur[digit_of<kDigit>(k, shift, pmask)], 1u);
    if (kAoS) {
      out_pairs[pos] = make_int2(k, v);
    } else {
      out_k[pos] = k;
      out_v[pos] = v;
    }
  };
  if (lo < hi) {
    const uint64_t qlo = lo / 4, qhi = hi / 4;
    const int4 *k4 = reinterpret_cast<const int4 *>(keys);
    const int4 *v4 = reinterpret_cast<const int4 *>(vals);
    for (uint64_t q = qlo + threadIdx.x; q < qhi; q += blockDim.x) {
      const int4 k = __ldcs(k4 + q);
      int4 v;
      if (vals) {
        v = __ldcs(v4 + q);
      } else {
        const int32_t r = (int32_t)(q * 4);
        v = make_int4(r, r + 1, r + 2, r + 3);
      }
      put(k.x, v.x);
      put(k.y, v.y);
      put(k.z, v.z);
      put(k.w, v.w);
    }
    for (uint64_t i = qhi * 4 + threadIdx.x; i < hi; i += blockDim.x)
      put(keys[i], vals ? vals[i] : (int32_t)i);
  }
}

__global__ void k_part_offsets(const uint64_t *__restrict__ base, uint32_t P, uint32_t G,
                               uint64_t n, uint64_t *__restrict__ offsets) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < P) offsets[p] = base[(uint64_t)p * G];
  if (p == 0) offsets[P] = n;
}

// Scalar count/scatter for inputs whose pointers are not 16-byte aligned:
// copy into aligned scratch first (one extra pass, only for odd callers).
__global__ void k_copy_i32(const int32_t *__restrict__ in, int32_t *__restrict__ out, uint64_t n) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride) out[i] = in[i];
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

// Persistent partition join.  Shared memory: build keys and values of one
// build chunk (kRMax each) and an open-addressing index of 16-bit
// (position + 1) entries, 2 * kRMax slots, probed with the fmix32 bits
// above the partition bits.
template <int kRMax, int kThreads>
__global__ void __launch_bounds__(kThreads)
    k_radix_join(const int2 *__restrict__ R, const uint64_t *__restrict__ ro,
                 const int2 *__restrict__ S, const uint64_t *__restrict__ so,
                 const uint64_t *__restrict__ item_off, uint32_t P, int bits, uint64_t w,
                 gbj::AggSpec spec, int64_t *out, unsigned long long *item_ctr) {
  extern __shared__ __align__(16) unsigned char smem[];
  int32_t *rk = reinterpret_cast<int32_t *>(smem);
  int32_t *rv = rk + kRMax;
  unsigned short *tab = reinterpret_cast<unsigned short *>(rv + kRMax);
  __shared__ int64_t red[32 * GBJ_MAX_AGGS];
  __shared__ unsigned long long s_item;
  __shared__ int s_dup;
  gbjd::Acc acc;
  acc.init(spec);
  const uint64_t total = item_off[P];
  for (;;) {
    if (threadIdx.x == 0) {
      s_item = atomicAdd(item_ctr, 1ull);
      s_dup = 0;
    }
    __syncthreads();
    const uint64_t item = s_item;
    if (item >= total) break;
    uint32_t lo = 0, hi = P;  // item_off[lo] <= item < item_off[hi]
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (item_off[mid] <= item) lo = mid; else hi = mid;
    }
    const uint32_t p = lo;
    const uint64_t r0 = ro[p], r1 = ro[p + 1], s0 = so[p], s1 = so[p + 1];
    const uint64_t nrc = (r1 - r0 + kRMax - 1) / kRMax;
    const uint64_t local = item - item_off[p];
    const uint64_t rb = r0 + (local % nrc) * kRMax;
    const uint64_t re = rb + kRMax < r1 ? rb + kRMax : r1;
    const uint64_t sb = s0 + (local / nrc) * w;
    const uint64_t se = sb + w < s1 ? sb + w : s1;
    const int m = (int)(re - rb);
    int cap = 64;
    while (cap < 2 * m) cap <<= 1;
    const uint32_t cmask = cap - 1;
    uint32_t *tab32 = reinterpret_cast<uint32_t *>(tab);
    for (int i = threadIdx.x; i < cap / 2; i += kThreads) tab32[i] = 0;
    for (int i = threadIdx.x; i < m; i += kThreads) {
      const int2 t = R[rb + i];
      rk[i] = t.x;
      rv[i] = t.y;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < m; i += kThreads) {
      const int32_t k = rk[i];
      uint32_t h = (gbjd::fmix32((uint32_t)k) >> bits) & cmask;
      bool dup = false;
      for (int step = 0; step < cap; ++step) {
        const unsigned short old = atomicCAS(&tab[h], (unsigned short)0, (unsigned short)(i + 1));
        if (old == 0) break;
        dup |= (rk[old - 1] == k);
        h = (h + 1) & cmask;
      }
      if (dup) s_dup = 1;
    }
    __syncthreads();
    const bool unique = s_dup == 0;
    // probe: 4 independent tuples per thread per round for memory-level
    // parallelism on the streamed probe chunk
    for (uint64_t j0 = sb + threadIdx.x; j0 < se; j0 += 4 * kThreads) {
      int2 t[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const uint64_t j = j0 + (uint64_t)u * kThreads;
        t[u] = j < se ? __ldcs(S + j) : make_int2(0, 0);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (j0 + (uint64_t)u * kThreads >= se) continue;
        const int32_t k = t[u].x;
        uint32_t h = (gbjd::fmix32((uint32_t)k) >> bits) & cmask;
        for (int step = 0; step < cap; ++step) {
          const unsigned short idx = tab[h];
          if (idx == 0) break;
          if (rk[idx - 1] == k) {
            const int64_t bv = rv[idx - 1];
            acc.update(spec, k, bv, t[u].y, bv, t[u].y);
            if (unique) break;
          }
          h = (h + 1) & cmask;
        }
      }
    }
    __syncthreads();
  }
  gbjd::block_flush(spec, acc, red, out);
}

struct JoinCfg {
  int rmax;
  int threads;
};

template <int kRMax, int kThreads>
int launch_join(gbj_ctx *ctx, const int2 *R, const uint64_t *ro, const int2 *S,
                const uint64_t *so, const uint64_t *item_off, uint32_t P, int bits,
                uint64_t w, const AggSpec &spec, int64_t *out, unsigned long long *ctr,
                cudaStream_t s) {
  const size_t smem = (size_t)kRMax * 8 + (size_t)kRMax * 2 * 2;
  auto kern = k_radix_join<kRMax, kThreads>;
  GBJ_CHECK_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem));
  int per_sm = 0;
  GBJ_CHECK_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem));
  if (per_sm < 1) per_sm = 1;
  kern<<<ctx->sm_count * per_sm, kThreads, smem, s>>>(R, ro, S, so, item_off, P, bits, w, spec,
                                                     out, ctr);
  return after_launch(ctx, "k_radix_join", s);
}

int part_grid(gbj_ctx *ctx, uint64_t n, uint64_t *seg) {
  // One CTA per SM (the shared histogram / cursors take up to 128 KB);
  // segments are multiples of 4 tuples for the int4 loads.
  uint64_t G = (uint64_t)ctx->sm_count;
  if (n < (1u << 16)) G = 1;
  else if (n < (1u << 22)) G = std::max<uint64_t>(1, std::min<uint64_t>(G, n >> 14));
  uint64_t sg = (n + G - 1) / G;
  sg = (sg + 3) / 4 * 4;
  if (sg == 0) sg = 4;
  G = (n + sg - 1) / sg;
  if (G == 0) G = 1;
  *seg = sg;
  return (int)G;
}

}  // namespace

namespace gbj {

int partition_tuples(gbj_ctx *ctx, const int32_t *keys, const int32_t *vals, uint64_t n,
                     int digit, int shift, int bits, int2 *out_pairs, int32_t *out_keys,
                     int32_t *out_vals, uint64_t *offsets, cudaStream_t s) {
  const uint32_t P = 1u << bits, pmask = P - 1;
  Scratch scratch(ctx, s);
  // int4 loads need 16-byte aligned inputs; realign odd callers once.
  if ((uintptr_t)keys % 16 || (vals && (uintptr_t)vals % 16)) {
    int32_t *k2, *v2 = nullptr;
    GBJ_TRY(scratch.get(n, &k2));
    k_copy_i32<<<ctx->sm_count * 4, 256, 0, s>>>(keys, k2, n);
    GBJ_TRY(after_launch(ctx, "k_copy_i32", s));
    if (vals) {
      GBJ_TRY(scratch.get(n, &v2));
      k_copy_i32<<<ctx->sm_count * 4, 256, 0, s>>>(vals, v2, n);
      GBJ_TRY(after_launch(ctx, "k_copy_i32", s));
    }
    keys = k2;
    vals = v2;
  }
  uint64_t seg;
  const int G = part_grid(ctx, n, &seg);
  uint32_t *hist;
  uint64_t *base;
  GBJ_TRY(scratch.get((uint64_t)P * G, &hist));
  GBJ_TRY(scratch.get((uint64_t)P * G + 1, &base));
  const size_t smem = (size_t)P * sizeof(uint32_t);
  if (digit == GBJ_DIGIT_HASH) {
    GBJ_CHECK_CUDA(ctx, cudaFuncSetAttribute(k_part_count<GBJ_DIGIT_HASH>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_part_count<GBJ_DIGIT_HASH><<<G, kPartThreads, smem, s>>>(keys, n, shift, pmask, seg, hist);
  } else {
    GBJ_CHECK_CUDA(ctx, cudaFuncSetAttribute(k_part_count<GBJ_DIGIT_KEY>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_part_count<GBJ_DIGIT_KEY><<<G, kPartThreads, smem, s>>>(keys, n, shift, pmask, seg, hist);
  }
  GBJ_TRY(after_launch(ctx, "k_part_count", s));
  GBJ_TRY(scan_u32_to_u64(ctx, hist, base, (uint64_t)P * G, s));
#define GBJ_SCATTER(D, A)                                                                     \
  do {                                                                                        \
    GBJ_CHECK_CUDA(ctx, cudaFuncSetAttribute(k_part_scatter<D, A>,                            \
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,     \
                                             (int)smem));                                     \
    k_part_scatter<D, A><<<G, kPartThreads, smem, s>>>(keys, vals, n, shift, pmask, seg, base, \
                                                       out_pairs, out_keys, out_vals);       \
  } while (0)
  if (digit == GBJ_DIGIT_HASH) {
    if (out_pairs) GBJ_SCATTER(GBJ_DIGIT_HASH, true); else GBJ_SCATTER(GBJ_DIGIT_HASH, false);
  } else {
    if (out_pairs) GBJ_SCATTER(GBJ_DIGIT_KEY, true); else GBJ_SCATTER(GBJ_DIGIT_KEY, false);
  }
#undef GBJ_SCATTER
  GBJ_TRY(after_launch(ctx, "k_part_scatter", s));
  if (offsets) {
    k_part_offsets<<<(P + 256) / 256, 256, 0, s>>>(base, P, G, n, offsets);
    GBJ_TRY(after_launch(ctx, "k_part_offsets", s));
  }
  return GBJ_OK;
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

int gbj_radix_join_agg(gbj_ctx *ctx, const int32_t *d_build_keys,
                       const int32_t *d_build_payload, uint64_t n_build,
                       const int32_t *d_probe_keys, const int32_t *d_probe_payload,
                       uint64_t n_probe, const gbj_radix_params *params, const gbj_agg *aggs,
                       int32_t n_aggs, int64_t *d_out, void *stream) {
  if (!ctx || !d_out) return GBJ_ERR_INVALID;
  GBJ_TRY(validate_aggs(ctx, aggs, n_aggs));
  if (n_build >= (1ULL << 31) || n_probe >= (1ULL << 31))
    return set_error(ctx, GBJ_ERR_INVALID, "radix_join: inputs must have < 2^31 rows");
  if ((n_build && !d_build_keys) || (n_probe && !d_probe_keys))
    return set_error(ctx, GBJ_ERR_INVALID, "radix_join: null key column");
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
  if ((b_row && b_pay) || (p_row && p_pay))
    return set_error(ctx, GBJ_ERR_UNSUPPORTED,
                     "radix_join: one side cannot carry both its payload and its row id");
  if ((b_pay && !d_build_payload && n_build) || (p_pay && !d_probe_payload && n_probe))
    return set_error(ctx, GBJ_ERR_INVALID, "radix_join: aggregate reads a missing payload");
  cudaStream_t s = pick_stream(ctx, stream);
  prof_mark(ctx, s);
  GBJ_TRY(init_agg_out(ctx, spec, d_out, s));
  if (n_build == 0 || n_probe == 0) return GBJ_OK;

  // ---- plan (autotuned defaults; explicit params override) ----
  constexpr int kRMax = 8192;
  int bits = 1;
  while (bits < kMaxPartBits && (n_build >> bits) > (uint64_t)kRMax / 2) ++bits;
  if (params && params->log_parts > 0) bits = std::min(params->log_parts, kMaxPartBits);
  if (params && params->bits > 0) bits = std::min(params->bits, kMaxPartBits);
  if (params && params->passes > 1)
    return set_error(ctx, GBJ_ERR_UNSUPPORTED, "radix_join: only single-pass partitioning");
  const uint32_t P = 1u << bits;
  const uint64_t w = 1u << 16;  // probe tuples per work item

  Scratch scratch(ctx, s);
  int2 *R, *S;
  uint64_t *ro, *so, *items;
  unsigned long long *ctr;
  GBJ_TRY(scratch.get(n_build, &R));
  GBJ_TRY(scratch.get(n_probe, &S));
  GBJ_TRY(scratch.get(P + 1, &ro));
  GBJ_TRY(scratch.get(P + 1, &so));
  GBJ_TRY(scratch.get(P + 1, &items));
  GBJ_TRY(scratch.get(1, &ctr));
  GBJ_TRY(partition_tuples(ctx, d_build_keys, b_pay ? d_build_payload : nullptr, n_build,
                           GBJ_DIGIT_HASH, 0, bits, R, nullptr, nullptr, ro, s));
  GBJ_TRY(partition_tuples(ctx, d_probe_keys, p_pay ? d_probe_payload : nullptr, n_probe,
                           GBJ_DIGIT_HASH, 0, bits, S, nullptr, nullptr, so, s));
  k_join_items<<<(P + 255) / 256, 256, 0, s>>>(ro, so, P, kRMax, w, items);
  GBJ_TRY(after_launch(ctx, "k_join_items", s));
  GBJ_TRY(scan_u64(ctx, items, items, P, s));
  GBJ_CHECK_CUDA(ctx, cudaMemsetAsync(ctr, 0, sizeof(unsigned long long), s));
  return launch_join<kRMax, 512>(ctx, R, ro, S, so, items, P, bits, w, spec, d_out, ctr, s);
}

}  // extern "C"
