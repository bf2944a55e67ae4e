// Batched star join: many select -> join x k -> group-by queries over one
// fact table, sharing one read of the fact columns.
//
// Each query is what a reference plan of Select (core/olap/lib/operators/
// select.cpp:26-37), HashJoinChained per dimension (hash-join-chained.cpp:
// 262-566, build = qualifying dimension rows keyed by their primary key,
// probe = the fact's foreign key) and HashGroupByChained on two dimension
// attributes (hash-group-by-chained.cpp:267-853) computes.  The reference
// runs one such plan per query.
//
// GB300 design (one batch = three kernels, captured once in a CUDA graph):
//  * k_star_mask: one pass over every dimension row evaluates all queries'
//    predicates and stores a 64-bit mask (bit q: query q keeps the row, or
//    does not join this dimension).  Dense primary keys make the join a
//    direct index, so the "hash table" of a dimension is this mask array
//    (8 B per row, ~19 MB for the workload's four dimensions: L2-resident).
//    A dimension with explicit keys (yyyymmdd dates) gets an open-addressing
//    table at plan creation -- slot keys, the row of each slot and the slot
//    of each row -- and its masks are stored per slot, so a lookup probes
//    the slot keys and reads the mask beside the match.
//  * k_star_fact: a persistent grid streams the fact columns with 128-bit
//    loads (4 rows per thread), gathers the masks of the row's foreign keys
//    most-selective dimension first, and stops at the first zero AND; the
//    surviving bits are (row, query) matches that add COUNT and
//    SUM(price * quantity) into dense per-query group arrays.
//  * k_star_emit: one CTA per query compacts the non-empty groups in key
//    order.
#include <algorithm>
#include <cstring>

#include "gbj_internal.cuh"

using namespace gbj;

namespace {

constexpr int kMaxDims = GBJ_STAR_MAX_DIMS;
constexpr int kMaxAttrs = GBJ_STAR_MAX_ATTRS;
constexpr int kMaxQ = GBJ_STAR_MAX_QUERIES;
constexpr int kMaxGroups = GBJ_STAR_MAX_GROUPS;
constexpr int kFactThreads = 256;
constexpr int kEmitThreads = 1024;
constexpr uint32_t kSmemMaskRows = 4096;  // dimensions up to this size: mask in shared memory
constexpr uint32_t kSmemMaskMax = 6144;   // total mask rows staged in shared memory
static_assert(kMaxGroups == 4 * kEmitThreads, "emit covers 4 groups per thread");

struct DimDev {
  const void *attr[kMaxAttrs];
  int32_t type[kMaxAttrs];
  int32_t n_attrs;
  uint32_t n;
  int32_t base;
  uint64_t row0;   // first row of this dimension in the concatenated mask pass
  uint64_t *mask;  // [n] (dense keys) or [ents] (explicit keys)
  int32_t smem_off;  // offset of the mask copy in the fact kernel's shared memory, -1 none
  // Explicit keys: kind 1, a range index over [kmin, kmin + 32 * aux_words / 2)
  // -- aux holds one {bitmap word, keys before it} pair per 32 values, and a
  // key's entry is its rank among the keys; kind 2, a hash table -- aux holds
  // the slot keys of `slots` slots (home slot fmix32(key) scaled to [0,
  // slots)), empty slots hold `empty` (a value no key has).  Masks are per
  // entry; ent_row[entry] and row_ent[row] link entries and rows.
  int32_t kind;  // 0 dense keys
  const int32_t *aux;
  uint32_t aux_words;  // 4-byte words of aux
  const int32_t *ent_row;
  const int32_t *row_ent;
  uint32_t ents;
  uint32_t slots;
  int32_t empty;
  int32_t kmin;
  int32_t smem_koff;  // offset of aux in the fact kernel's shared aux copy, -1 none
};

struct Dims {
  DimDev d[kMaxDims];
  int32_t nd;
  int32_t late;  // dimension whose mask is gathered only for rows still alive, -1 none
  uint64_t total_rows;
};

struct FactDev {
  const int32_t *fk[kMaxDims];
  const int32_t *qty, *price;
  uint64_t n;
};

// One query as the kernels read it (built on the host, uploaded per batch).
struct QDev {
  uint32_t join_mask;
  int32_t pred_attr[kMaxDims];
  int32_t lo[kMaxDims], hi[kMaxDims];
  int32_t gd[2], ga[2];
  int32_t gmin[2];
  uint32_t gspan[2];
  int32_t *out_a, *out_b;
  int64_t *out_cnt, *out_sum;
  uint64_t *out_n;
};

struct Desc {
  int32_t nq;
  int32_t pad;
  uint64_t cap;  // output rows per query
  QDev q[kMaxQ];
};

__device__ __forceinline__ int32_t attr_at(const DimDev &d, int a, uint32_t i) {
  return d.type[a] == GBJ_ATTR_I8 ? (int32_t)(static_cast<const int8_t *>(d.attr[a]))[i]
                                  : (static_cast<const int32_t *>(d.attr[a]))[i];
}

// Predicate masks of every dimension row.
__global__ void __launch_bounds__(256) k_star_mask(const Desc *__restrict__ desc, Dims dims) {
  __shared__ uint32_t s_join[kMaxQ];
  __shared__ int32_t s_pa[kMaxQ][kMaxDims], s_lo[kMaxQ][kMaxDims], s_hi[kMaxQ][kMaxDims];
  const int nq = desc->nq;
  for (int q = threadIdx.x; q < nq; q += blockDim.x) {
    s_join[q] = desc->q[q].join_mask;
    for (int d = 0; d < kMaxDims; ++d) {
      s_pa[q][d] = desc->q[q].pred_attr[d];
      s_lo[q][d] = desc->q[q].lo[d];
      s_hi[q][d] = desc->q[q].hi[d];
    }
  }
  __syncthreads();
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g < dims.total_rows;
       g += stride) {
    int d = 0;
#pragma unroll
    for (int j = 1; j < kMaxDims; ++j)
      if (j < dims.nd && g >= dims.d[j].row0) d = j;
    const DimDev &dd = dims.d[d];
    const uint32_t r = (uint32_t)(g - dd.row0);
    int32_t v0 = 0, v1 = 0, v2 = 0, v3 = 0;
    if (dd.n_attrs > 0) v0 = attr_at(dd, 0, r);
    if (dd.n_attrs > 1) v1 = attr_at(dd, 1, r);
    if (dd.n_attrs > 2) v2 = attr_at(dd, 2, r);
    if (dd.n_attrs > 3) v3 = attr_at(dd, 3, r);
    uint64_t m = 0;
    for (int q = 0; q < nq; ++q) {
      const int pa = s_pa[q][d];
      int32_t x = pa == 1 ? v1 : v0;
      x = pa == 2 ? v2 : x;
      x = pa == 3 ? v3 : x;
      const bool keep = !((s_join[q] >> d) & 1u) || pa < 0 || (x >= s_lo[q][d] && x <= s_hi[q][d]);
      m |= (uint64_t)keep << q;
    }
    dd.mask[dd.kind ? (uint32_t)dd.row_ent[r] : r] = m;
  }
}

// Entry of key k in a dimension with explicit keys (aux from shared or
// global memory), -1 when absent.
__device__ __forceinline__ int32_t keyed_ent(const DimDev &dd, const int32_t *aux, int32_t k) {
  if (dd.kind == 1) {
    const int64_t idx = (int64_t)k - dd.kmin;
    if (idx < 0 || idx >= (int64_t)dd.aux_words * 16) return -1;
    const uint2 e = reinterpret_cast<const uint2 *>(aux)[idx >> 5];
    const uint32_t b = (uint32_t)idx & 31u;
    if (!((e.x >> b) & 1u)) return -1;
    return (int32_t)(e.y + __popc(e.x & ((1u << b) - 1u)));
  }
  if (k == dd.empty) return -1;  // no key has the empty-slot value
  uint32_t h = __umulhi(gbjd::fmix32((uint32_t)k), dd.slots);
  for (uint32_t step = 0; step < dd.slots; ++step) {
    const int32_t x = aux[h];
    if (x == k) return (int32_t)h;
    if (x == dd.empty) return -1;
    h = h + 1 == dd.slots ? 0 : h + 1;
  }
  return -1;
}

// Row of key k (-1 when absent): dense or explicit keys (aux from shared
// memory when staged there).
__device__ __forceinline__ int64_t dim_row(const DimDev &dd, const int32_t *s_aux, int32_t k) {
  if (dd.kind) {
    const int32_t e = keyed_ent(dd, dd.smem_off >= 0 ? s_aux + dd.smem_koff : dd.aux, k);
    return e < 0 ? -1 : __ldg(dd.ent_row + e);
  }
  const uint32_t idx = (uint32_t)(k - dd.base);
  return idx < dd.n ? (int64_t)idx : -1;
}

struct GroupSpec {
  int32_t gd[2], ga[2], gmin[2];
  uint32_t gspan[2];
};

// The (row, query) matches of one fact row: COUNT and SUM(price * quantity)
// into the query's dense group arrays.
template <bool kKeyed>
__device__ __forceinline__ void star_matches(const Dims &dims, const int32_t *s_keys, uint64_t m,
                                             const GroupSpec *sg,
                                             const int32_t (&fk)[kMaxDims], int32_t qty,
                                             int32_t price, unsigned long long *__restrict__ gcnt,
                                             unsigned long long *__restrict__ gsum,
                                             uint32_t *status) {
  const unsigned long long val = (unsigned long long)((int64_t)price * (int64_t)qty);
  // the row of the last hashed dimension looked up (the fact row's key of a
  // dimension is the same for every query)
  int hd = -1;
  uint32_t hrow = 0;
  while (m) {
    const int q = __ffsll((long long)m) - 1;
    m &= m - 1;
    const GroupSpec &gs = sg[q];
    int32_t key[2];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const int d = gs.gd[s];
      const int32_t k = d == 0 ? fk[0] : d == 1 ? fk[1] : d == 2 ? fk[2] : fk[3];
      const DimDev &dd = dims.d[d];
      // a joined dimension passed the row, so its key is present
      uint32_t row;
      if (kKeyed && dd.kind) {
        if (hd != d) {
          hrow = (uint32_t)dim_row(dd, s_keys, k);
          hd = d;
        }
        row = hrow;
      } else {
        row = (uint32_t)(k - dd.base);
      }
      key[s] = attr_at(dd, gs.ga[s], row);
    }
    const uint32_t a = (uint32_t)(key[0] - gs.gmin[0]), b = (uint32_t)(key[1] - gs.gmin[1]);
    if (a >= gs.gspan[0] || b >= gs.gspan[1]) {
      gbjd::latch(status, GBJ_DEV_INVALID);
      continue;
    }
    const uint64_t gi = (uint64_t)q * kMaxGroups + a * gs.gspan[1] + b;
    atomicAdd(&gcnt[gi], 1ull);
    atomicAdd(&gsum[gi], val);
  }
}

// Mask of dimension d for foreign key k: from shared memory for small
// dimensions, else an L2 gather; keys outside the dimension pass only the
// queries that do not join it.
__device__ __forceinline__ uint64_t keyed_mask(const DimDev &dd, const uint64_t *s_mask, const int32_t *s_aux,
                                              int32_t k, uint64_t nojoin) {
  const bool sm = dd.smem_off >= 0;
  const int32_t e = keyed_ent(dd, sm ? s_aux + dd.smem_koff : dd.aux, k);
  if (e < 0) return nojoin;
  return sm ? s_mask[dd.smem_off + e] : __ldg(dd.mask + e);
}

template <bool kKeyed>
__device__ __forceinline__ uint64_t dim_mask(const DimDev &dd, const uint64_t *s_mask, const int32_t *s_keys,
                                             int32_t k, uint64_t nojoin) {
  if (kKeyed && dd.kind) return keyed_mask(dd, s_mask, s_keys, k, nojoin);
  const uint32_t idx = (uint32_t)(k - dd.base);
  if (idx >= dd.n) return nojoin;
  return dd.smem_off >= 0 ? s_mask[dd.smem_off + idx] : __ldg(dd.mask + idx);
}

// Fact scan.  Each thread takes 4 rows per round (one 128-bit load per
// column) and issues every mask lookup of the 4 rows before combining them,
// so a thread keeps up to 16 independent gathers in flight instead of
// walking dimensions one dependent load at a time.
template <bool kVec, bool kKeyed>
__global__ void __launch_bounds__(kFactThreads)
    k_star_fact(const Desc *__restrict__ desc, FactDev f, Dims dims, uint32_t smem_masks,
                unsigned long long *__restrict__ gcnt, unsigned long long *__restrict__ gsum,
                uint32_t *status) {
  extern __shared__ uint64_t s_mask[];  // masks of the small dimensions, then slot keys of hashed ones
  int32_t *s_keys = reinterpret_cast<int32_t *>(s_mask + smem_masks);
  __shared__ GroupSpec sg[kMaxQ];
  __shared__ uint64_t s_nojoin[kMaxDims];
  const int nq = desc->nq;
  for (int q = threadIdx.x; q < nq; q += blockDim.x) {
    const QDev &qd = desc->q[q];
    for (int s = 0; s < 2; ++s) {
      sg[q].gd[s] = qd.gd[s];
      sg[q].ga[s] = qd.ga[s];
      sg[q].gmin[s] = qd.gmin[s];
      sg[q].gspan[s] = qd.gspan[s];
    }
  }
  if (threadIdx.x < kMaxDims) {
    // queries that do not join dimension d pass it whatever the key
    uint64_t nj = 0;
    for (int q = 0; q < nq; ++q) nj |= (uint64_t)(((desc->q[q].join_mask >> threadIdx.x) & 1u) == 0) << q;
    s_nojoin[threadIdx.x] = nj;
  }
#pragma unroll
  for (int d = 0; d < kMaxDims; ++d) {
    if (d < dims.nd && dims.d[d].smem_off >= 0) {
      const DimDev &dd = dims.d[d];
      const uint32_t cnt = kKeyed && dd.kind ? dd.ents : dd.n;
      for (uint32_t i = threadIdx.x; i < cnt; i += blockDim.x) s_mask[dd.smem_off + i] = dd.mask[i];
      if (kKeyed && dd.kind)
        for (uint32_t i = threadIdx.x; i < dd.aux_words; i += blockDim.x) s_keys[dd.smem_koff + i] = dd.aux[i];
    }
  }
  __syncthreads();
  uint64_t nojoin[kMaxDims];
#pragma unroll
  for (int d = 0; d < kMaxDims; ++d) nojoin[d] = s_nojoin[d];
  const uint64_t active = nq >= 64 ? ~0ull : ((1ull << nq) - 1);
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  uint64_t done = 0;
  if (kVec) {
    const uint64_t n4 = f.n / 4;
    for (uint64_t i = tid; i < n4; i += stride) {
      int4 k4[kMaxDims];
#pragma unroll
      for (int d = 0; d < kMaxDims; ++d)
        k4[d] = d < dims.nd ? __ldcs(reinterpret_cast<const int4 *>(f.fk[d]) + i) : make_int4(0, 0, 0, 0);
      const int4 q4 = __ldcs(reinterpret_cast<const int4 *>(f.qty) + i);
      const int4 p4 = __ldcs(reinterpret_cast<const int4 *>(f.price) + i);
      uint64_t m[4] = {active, active, active, active};
#pragma unroll
      for (int d = 0; d < kMaxDims; ++d) {
        if (d < dims.nd && d != dims.late && (!kKeyed || dims.d[d].kind != 2)) {
          m[0] &= dim_mask<kKeyed>(dims.d[d], s_mask, s_keys, k4[d].x, nojoin[d]);
          m[1] &= dim_mask<kKeyed>(dims.d[d], s_mask, s_keys, k4[d].y, nojoin[d]);
          m[2] &= dim_mask<kKeyed>(dims.d[d], s_mask, s_keys, k4[d].z, nojoin[d]);
          m[3] &= dim_mask<kKeyed>(dims.d[d], s_mask, s_keys, k4[d].w, nojoin[d]);
        }
      }
      // hash-table dimensions (a probe loop each), then the largest gathered
      // dimension, only for rows some query still passes (most rows have
      // failed every query by then).  The hash probes run in a loop over the
      // four rows that is not unrolled, so the kernel carries one copy.
#pragma unroll
      for (int d = 0; d < kMaxDims; ++d) {
        if (kKeyed && d < dims.nd && dims.d[d].kind == 2) {
#pragma unroll 1
          for (int r = 0; r < 4; ++r) {
            const uint64_t mr = r == 0 ? m[0] : r == 1 ? m[1] : r == 2 ? m[2] : m[3];
            if (!mr) continue;
            const int32_t k = r == 0 ? k4[d].x : r == 1 ? k4[d].y : r == 2 ? k4[d].z : k4[d].w;
            const uint64_t v = mr & keyed_mask(dims.d[d], s_mask, s_keys, k, nojoin[d]);
            m[0] = r == 0 ? v : m[0];
            m[1] = r == 1 ? v : m[1];
            m[2] = r == 2 ? v : m[2];
            m[3] = r == 3 ? v : m[3];
          }
        }
      }
#pragma unroll
      for (int d = 0; d < kMaxDims; ++d) {
        if (d < dims.nd && d == dims.late && (!kKeyed || !dims.d[d].kind)) {
          if (m[0]) m[0] &= dim_mask<kKeyed>(dims.d[d], s_mask, s_keys, k4[d].x, nojoin[d]);
          if (m[1]) m[1] &= dim_mask<kKeyed>(dims.d[d], s_mask, s_keys, k4[d].y, nojoin[d]);
          if (m[2]) m[2] &= dim_mask<kKeyed>(dims.d[d], s_mask, s_keys, k4[d].z, nojoin[d]);
          if (m[3]) m[3] &= dim_mask<kKeyed>(dims.d[d], s_mask, s_keys, k4[d].w, nojoin[d]);
        }
      }
      if (m[0]) {
        const int32_t fk[kMaxDims] = {k4[0].x, k4[1].x, k4[2].x, k4[3].x};
        star_matches<kKeyed>(dims, s_keys, m[0], sg, fk, q4.x, p4.x, gcnt, gsum, status);
      }
      if (m[1]) {
        const int32_t fk[kMaxDims] = {k4[0].y, k4[1].y, k4[2].y, k4[3].y};
        star_matches<kKeyed>(dims, s_keys, m[1], sg, fk, q4.y, p4.y, gcnt, gsum, status);
      }
      if (m[2]) {
        const int32_t fk[kMaxDims] = {k4[0].z, k4[1].z, k4[2].z, k4[3].z};
        star_matches<kKeyed>(dims, s_keys, m[2], sg, fk, q4.z, p4.z, gcnt, gsum, status);
      }
      if (m[3]) {
        const int32_t fk[kMaxDims] = {k4[0].w, k4[1].w, k4[2].w, k4[3].w};
        star_matches<kKeyed>(dims, s_keys, m[3], sg, fk, q4.w, p4.w, gcnt, gsum, status);
      }
    }
    done = n4 * 4;
  }
  for (uint64_t r = done + tid; r < f.n; r += stride) {
    int32_t fk[kMaxDims];
    uint64_t m = active;
#pragma unroll
    for (int d = 0; d < kMaxDims; ++d) {
      fk[d] = d < dims.nd ? f.fk[d][r] : 0;
      if (d < dims.nd) m &= dim_mask<kKeyed>(dims.d[d], s_mask, s_keys, fk[d], nojoin[d]);
    }
    if (m) star_matches<kKeyed>(dims, s_keys, m, sg, fk, f.qty[r], f.price[r], gcnt, gsum, status);
  }
}

// One CTA per query: the non-empty groups in (key_a, key_b) order.
__global__ void __launch_bounds__(kEmitThreads)
    k_star_emit(const Desc *__restrict__ desc, const unsigned long long *__restrict__ gcnt,
                const unsigned long long *__restrict__ gsum, uint32_t *status) {
  __shared__ uint32_t s_warp[kEmitThreads / 32];
  const int q = blockIdx.x;
  if (q >= desc->nq) return;
  const QDev &qd = desc->q[q];
  const uint32_t groups = qd.gspan[0] * qd.gspan[1];
  const unsigned long long *cnt = gcnt + (uint64_t)q * kMaxGroups;
  const unsigned long long *sum = gsum + (uint64_t)q * kMaxGroups;
  const uint32_t g0 = threadIdx.x * 4;
  unsigned long long c[4];
  uint32_t mine = 0;
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    c[u] = g0 + u < groups ? cnt[g0 + u] : 0;
    mine += c[u] != 0;
  }
  // exclusive scan of `mine` over the CTA
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = mine;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = s_warp[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    s_warp[lane] = w;  // inclusive over warps
  }
  __syncthreads();
  uint64_t pos = (warp ? s_warp[warp - 1] : 0) + incl - mine;
  const uint64_t total = s_warp[kEmitThreads / 32 - 1];
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    if (c[u] == 0) continue;
    if (pos >= desc->cap) {
      gbjd::latch(status, GBJ_DEV_CAPACITY);
      break;
    }
    const uint32_t gi = g0 + u;
    qd.out_a[pos] = qd.gmin[0] + (int32_t)(gi / qd.gspan[1]);
    qd.out_b[pos] = qd.gmin[1] + (int32_t)(gi % qd.gspan[1]);
    qd.out_cnt[pos] = (int64_t)c[u];
    qd.out_sum[pos] = (int64_t)sum[gi];
    ++pos;
  }
  if (threadIdx.x == 0) *qd.out_n = total;
}

// Smallest and largest key of a hashed dimension (mm = {INT32_MAX, INT32_MIN}
// on entry).
__global__ void k_star_key_range(const int32_t *__restrict__ keys, uint64_t n, int32_t *mm) {
  int32_t lo = INT32_MAX, hi = INT32_MIN;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    lo = min(lo, keys[i]);
    hi = max(hi, keys[i]);
  }
  lo = __reduce_min_sync(0xffffffffu, lo);
  hi = __reduce_max_sync(0xffffffffu, hi);
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&mm[0], lo);
    atomicMax(&mm[1], hi);
  }
}

__global__ void k_star_fill(int32_t *__restrict__ a, uint64_t n, int32_t v) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    a[i] = v;
}

// Places every row of a hashed dimension (linear probing from fmix32(key));
// a key met twice latches GBJ_DEV_INVALID.
__global__ void k_star_hash_build(const int32_t *__restrict__ keys, uint32_t n, int32_t *__restrict__ hkeys,
                                  uint32_t slots, int32_t empty, int32_t *__restrict__ ent_row,
                                  int32_t *__restrict__ row_ent, uint32_t *status) {
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    const int32_t k = keys[r];
    uint32_t h = __umulhi(gbjd::fmix32((uint32_t)k), slots);
    bool placed = false;
    for (uint32_t step = 0; step < slots; ++step) {
      const int32_t old = atomicCAS(&hkeys[h], empty, k);
      if (old == empty) {
        ent_row[h] = (int32_t)r;
        row_ent[r] = (int32_t)h;
        placed = true;
        break;
      }
      if (old == k) {
        gbjd::latch(status, GBJ_DEV_INVALID);
        placed = true;
        break;
      }
      h = h + 1 == slots ? 0 : h + 1;
    }
    if (!placed) gbjd::latch(status, GBJ_DEV_CAPACITY);
  }
}

// Range index, step 1: the bitmap (aux[2 w] = bits of values 32 w ..
// 32 w + 31 above kmin); a key met twice latches GBJ_DEV_INVALID.
__global__ void k_star_range_bits(const int32_t *__restrict__ keys, uint32_t n, int32_t kmin,
                                  uint32_t *__restrict__ aux, uint32_t *status) {
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    const uint32_t idx = (uint32_t)((int64_t)keys[r] - kmin);
    const uint32_t bit = 1u << (idx & 31u);
    if (atomicOr(&aux[2 * (idx >> 5)], bit) & bit) gbjd::latch(status, GBJ_DEV_INVALID);
  }
}

// Step 2 (one CTA of 1024 threads): aux[2 w + 1] = keys in words before w.
__global__ void __launch_bounds__(1024) k_star_range_rank(uint32_t *__restrict__ aux, uint32_t words) {
  __shared__ uint32_t s_warp[32];
  const uint32_t chunk = (words + 1023) / 1024;
  const uint32_t lo = min(words, threadIdx.x * chunk), hi = min(words, lo + chunk);
  uint32_t mine = 0;
  for (uint32_t w = lo; w < hi; ++w) mine += __popc(aux[2 * w]);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = mine;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t v = s_warp[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += y;
    }
    s_warp[lane] = v;
  }
  __syncthreads();
  uint32_t run = (warp ? s_warp[warp - 1] : 0) + incl - mine;
  for (uint32_t w = lo; w < hi; ++w) {
    aux[2 * w + 1] = run;
    run += __popc(aux[2 * w]);
  }
}

// Step 3: entries (ranks) of the rows, both ways.
__global__ void k_star_range_ent(const int32_t *__restrict__ keys, uint32_t n, int32_t kmin,
                                 const uint32_t *__restrict__ aux, int32_t *__restrict__ ent_row,
                                 int32_t *__restrict__ row_ent) {
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    const uint32_t idx = (uint32_t)((int64_t)keys[r] - kmin);
    const uint32_t w = idx >> 5, b = idx & 31u;
    const int32_t e = (int32_t)(aux[2 * w + 1] + __popc(aux[2 * w] & ((1u << b) - 1u)));
    ent_row[e] = (int32_t)r;
    row_ent[r] = e;
  }
}

}  // namespace

struct gbj_star_plan {
  gbj_ctx *ctx = nullptr;
  FactDev fact{};
  Dims dims{};
  gbj_star_dim host_dims[kMaxDims]{};
  bool vec = false;
  uint64_t *masks = nullptr;
  int32_t *hash_mem = nullptr;  // slot keys, slot rows and row slots of hashed dimensions
  size_t fact_smem = 0;
  uint32_t smem_masks = 0;      // 8-byte masks staged in shared memory (index words follow)
  bool keyed = false;           // some dimension has explicit keys
  unsigned long long *gcnt = nullptr, *gsum = nullptr;
  Desc *d_desc = nullptr;
  Desc *h_desc[2] = {nullptr, nullptr};  // pinned
  cudaEvent_t done[2] = {nullptr, nullptr};
  bool used[2] = {false, false};
  cudaGraphExec_t exec[2] = {nullptr, nullptr};
  cudaStream_t cap_stream = nullptr;
  int slot = 0;
  int fact_grid = 0;
};

namespace {

int star_validate(gbj_star_plan *p, const gbj_star_query *qs, int32_t nq, const gbj_star_out *out) {
  gbj_ctx *ctx = p->ctx;
  if (!qs || nq < 1 || nq > kMaxQ) return set_error(ctx, GBJ_ERR_INVALID, "star: n_queries must be 1..64");
  if (!out || !out->d_key_a || !out->d_key_b || !out->d_count || !out->d_sum || !out->d_n_groups ||
      out->group_cap == 0)
    return set_error(ctx, GBJ_ERR_INVALID, "star: null output or zero group_cap");
  const int nd = p->dims.nd;
  for (int q = 0; q < nq; ++q) {
    const gbj_star_query &s = qs[q];
    if (s.join_mask <= 0 || (s.join_mask >> nd) != 0)
      return set_error(ctx, GBJ_ERR_INVALID, "star: query " + std::to_string(q) + ": bad join_mask");
    for (int d = 0; d < nd; ++d) {
      if (!((s.join_mask >> d) & 1)) continue;
      if (s.pred_attr[d] >= p->host_dims[d].n_attrs || s.pred_attr[d] < -1)
        return set_error(ctx, GBJ_ERR_INVALID, "star: query " + std::to_string(q) + ": bad pred_attr");
    }
    uint64_t groups = 1;
    for (int k = 0; k < 2; ++k) {
      const int d = s.group_dim[k], a = s.group_attr[k];
      if (d < 0 || d >= nd || !((s.join_mask >> d) & 1) || a < 0 || a >= p->host_dims[d].n_attrs)
        return set_error(ctx, GBJ_ERR_INVALID,
                         "star: query " + std::to_string(q) + ": group key must be an attribute of a joined dimension");
      const int64_t span = (int64_t)p->host_dims[d].attr_max[a] - p->host_dims[d].attr_min[a] + 1;
      if (span < 1) return set_error(ctx, GBJ_ERR_INVALID, "star: empty attribute domain");
      groups *= (uint64_t)span;
    }
    if (groups > (uint64_t)kMaxGroups)
      return set_error(ctx, GBJ_ERR_INVALID,
                       "star: query " + std::to_string(q) + ": group domain exceeds GBJ_STAR_MAX_GROUPS");
  }
  return GBJ_OK;
}

void star_fill_desc(const gbj_star_plan *p, const gbj_star_query *qs, int32_t nq,
                    const gbj_star_out *out, Desc *h) {
  std::memset(h, 0, sizeof(Desc));
  h->nq = nq;
  h->cap = out->group_cap;
  for (int q = 0; q < nq; ++q) {
    const gbj_star_query &s = qs[q];
    QDev &d = h->q[q];
    d.join_mask = (uint32_t)s.join_mask;
    for (int k = 0; k < kMaxDims; ++k) {
      const bool joined = k < p->dims.nd && ((s.join_mask >> k) & 1);
      d.pred_attr[k] = joined ? s.pred_attr[k] : -1;
      d.lo[k] = s.pred_lo[k];
      d.hi[k] = s.pred_hi[k];
    }
    for (int k = 0; k < 2; ++k) {
      const gbj_star_dim &hd = p->host_dims[s.group_dim[k]];
      d.gd[k] = s.group_dim[k];
      d.ga[k] = s.group_attr[k];
      d.gmin[k] = hd.attr_min[s.group_attr[k]];
      d.gspan[k] = (uint32_t)((int64_t)hd.attr_max[s.group_attr[k]] - hd.attr_min[s.group_attr[k]] + 1);
    }
    const uint64_t off = (uint64_t)q * out->group_cap;
    d.out_a = out->d_key_a + off;
    d.out_b = out->d_key_b + off;
    d.out_cnt = out->d_count + off;
    d.out_sum = out->d_sum + off;
    d.out_n = out->d_n_groups + q;
  }
}

// Kernel-launch bookkeeping that is legal inside stream capture (no events).
int star_launched(gbj_ctx *ctx, const char *name, cudaStream_t s, bool capturing) {
  if (!capturing) return after_launch(ctx, name, s);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(ctx, e, name);
  return GBJ_OK;
}

// The batch's work on `s`: descriptor upload, resets, three kernels.
int star_enqueue(gbj_star_plan *p, int slot, cudaStream_t s, bool capturing) {
  gbj_ctx *ctx = p->ctx;
  GBJ_CHECK_CUDA(ctx, cudaMemcpyAsync(p->d_desc, p->h_desc[slot], sizeof(Desc), cudaMemcpyHostToDevice, s));
  GBJ_CHECK_CUDA(ctx, cudaMemsetAsync(p->gcnt, 0, sizeof(unsigned long long) * kMaxQ * kMaxGroups * 2, s));
  const uint64_t rows = p->dims.total_rows;
  const unsigned mask_grid = (unsigned)std::max<uint64_t>(
      1, std::min<uint64_t>((rows + 255) / 256, (uint64_t)ctx->sm_count * 8));
  k_star_mask<<<mask_grid, 256, 0, s>>>(p->d_desc, p->dims);
  GBJ_TRY(star_launched(ctx, "k_star_mask", s, capturing));
  auto fact = p->vec ? (p->keyed ? k_star_fact<true, true> : k_star_fact<true, false>)
                     : (p->keyed ? k_star_fact<false, true> : k_star_fact<false, false>);
  fact<<<p->fact_grid, kFactThreads, p->fact_smem, s>>>(p->d_desc, p->fact, p->dims, p->smem_masks, p->gcnt,
                                                        p->gsum, ctx->d_status);
  GBJ_TRY(star_launched(ctx, "k_star_fact", s, capturing));
  k_star_emit<<<kMaxQ, kEmitThreads, 0, s>>>(p->d_desc, p->gcnt, p->gsum, ctx->d_status);
  return star_launched(ctx, "k_star_emit", s, capturing);
}

}  // namespace

extern "C" int gbj_star_plan_create(gbj_ctx *ctx, const gbj_star_fact *fact,
                                    const gbj_star_dim *dims, gbj_star_plan **out) {
  if (!ctx || !out) return GBJ_ERR_INVALID;
  *out = nullptr;
  if (!fact || !dims) return set_error(ctx, GBJ_ERR_INVALID, "star: null fact or dims");
  if (fact->n_dims < 1 || fact->n_dims > kMaxDims)
    return set_error(ctx, GBJ_ERR_INVALID, "star: n_dims must be 1..4");
  if (fact->n && (!fact->d_quantity || !fact->d_price))
    return set_error(ctx, GBJ_ERR_INVALID, "star: null quantity or price column");
  auto p = new gbj_star_plan();
  p->ctx = ctx;
  p->fact.n = fact->n;
  p->fact.qty = fact->d_quantity;
  p->fact.price = fact->d_price;
  bool aligned = (reinterpret_cast<uintptr_t>(fact->d_quantity) % 16 == 0) &&
                 (reinterpret_cast<uintptr_t>(fact->d_price) % 16 == 0);
  p->dims.nd = fact->n_dims;
  uint64_t rows = 0, masks_total = 0, mask_slots[kMaxDims] = {0, 0, 0, 0};
  auto fail = [&](int rc) {
    gbj_star_plan_destroy(p);
    return rc;
  };
  for (int d = 0; d < fact->n_dims; ++d) {
    const gbj_star_dim &hd = dims[d];
    if (fact->n && !fact->d_fk[d]) return fail(set_error(ctx, GBJ_ERR_INVALID, "star: null fk column"));
    if (hd.n == 0 || hd.n >= (1ull << 31) || hd.n_attrs < 0 || hd.n_attrs > kMaxAttrs)
      return fail(set_error(ctx, GBJ_ERR_INVALID, "star: dimension size or attribute count out of range"));
    for (int a = 0; a < hd.n_attrs; ++a) {
      if (!hd.d_attr[a] || (hd.attr_type[a] != GBJ_ATTR_I32 && hd.attr_type[a] != GBJ_ATTR_I8))
        return fail(set_error(ctx, GBJ_ERR_INVALID, "star: bad dimension attribute"));
    }
    p->host_dims[d] = hd;
    p->fact.fk[d] = fact->d_fk[d];
    aligned = aligned && reinterpret_cast<uintptr_t>(fact->d_fk[d]) % 16 == 0;
    DimDev &dd = p->dims.d[d];
    for (int a = 0; a < kMaxAttrs; ++a) {
      dd.attr[a] = a < hd.n_attrs ? hd.d_attr[a] : nullptr;
      dd.type[a] = a < hd.n_attrs ? hd.attr_type[a] : GBJ_ATTR_I32;
    }
    dd.n_attrs = hd.n_attrs;
    dd.n = (uint32_t)hd.n;
    dd.base = hd.key_base;
    dd.row0 = rows;
    rows += hd.n;
    dd.smem_off = dd.smem_koff = -1;
    dd.kind = 0;
    dd.aux = nullptr;
  }
  p->dims.total_rows = rows;
  cudaStream_t s = ctx->stream;
  int rc = GBJ_OK;
  // explicit keys: the key range picks the index -- a range index when the
  // keys fill at least 1/64 of their range (dates: 2,557 of 61,131 values),
  // else a hash table at load factor <= 3/4 (slots a multiple of 32) -- and
  // gives the hash table's empty-slot value
  int32_t *mm = nullptr;
  for (int d = 0; d < fact->n_dims; ++d) {
    const gbj_star_dim &hd = dims[d];
    if (!hd.d_keys) {
      mask_slots[d] = hd.n;
      masks_total += hd.n;
      continue;
    }
    if (!mm) {
      rc = pool_alloc(ctx, 4 * sizeof(int32_t), s, reinterpret_cast<void **>(&mm));
      if (rc) return fail(rc);
    }
    const int32_t init[2] = {INT32_MAX, INT32_MIN};
    int32_t got[2];
    cudaError_t e = cudaMemcpyAsync(mm, init, sizeof(init), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return fail(cuda_error(ctx, e, "star: key range"));
    const unsigned g = (unsigned)std::min<uint64_t>((hd.n + 255) / 256, (uint64_t)ctx->sm_count * 4);
    k_star_key_range<<<g, 256, 0, s>>>(hd.d_keys, hd.n, mm);
    rc = after_launch(ctx, "k_star_key_range", s);
    if (rc) return fail(rc);
    e = cudaMemcpyAsync(got, mm, sizeof(got), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(cuda_error(ctx, e, "star: key range"));
    DimDev &dd = p->dims.d[d];
    const int64_t range = (int64_t)got[1] - got[0] + 1;
    dd.kmin = got[0];
    if (range <= 64 * (int64_t)hd.n && range <= (1ll << 26)) {
      dd.kind = 1;
      dd.aux_words = (uint32_t)(2 * ((range + 31) / 32));
      dd.ents = (uint32_t)hd.n;
    } else {
      if (got[0] != INT32_MIN) dd.empty = got[0] - 1;
      else if (got[1] != INT32_MAX) dd.empty = got[1] + 1;
      else return fail(set_error(ctx, GBJ_ERR_UNSUPPORTED, "star: dimension keys span the whole int32 range"));
      dd.kind = 2;
      dd.slots = (uint32_t)std::max<uint64_t>(64, ((4 * hd.n + 2) / 3 + 31) / 32 * 32);
      dd.aux_words = dd.slots;
      dd.ents = dd.slots;
    }
    mask_slots[d] = dd.ents;
    masks_total += dd.ents;
    p->keyed = true;
  }
  if (mm) pool_release(ctx, mm, s);
  // small dimensions' masks (and index words) go to the fact kernel's shared
  // memory, within kSmemMaskMax * 8 bytes
  {
    uint64_t mask_units = 0, key_units = 0;
    for (int d = 0; d < fact->n_dims; ++d) {
      DimDev &dd = p->dims.d[d];
      const uint64_t m = mask_slots[d];
      const uint64_t ku = dd.kind ? ((key_units + 1) & ~1ull) + dd.aux_words : key_units;  // range pairs 8-aligned
      if (m > kSmemMaskRows) continue;
      if ((mask_units + m) * 8 + ku * 4 > (uint64_t)kSmemMaskMax * 8) continue;
      dd.smem_off = (int32_t)mask_units;
      mask_units += m;
      if (dd.kind) {
        dd.smem_koff = (int32_t)(ku - dd.aux_words);
        key_units = ku;
      }
    }
    p->smem_masks = (uint32_t)mask_units;
    p->fact_smem = mask_units * 8 + key_units * 4;
  }
  // the late dimension: the largest one gathered from L2, when another
  // gathered dimension is checked before it
  p->dims.late = -1;
  {
    int gathered = 0, big = -1;
    for (int d = 0; d < fact->n_dims; ++d) {
      if (p->dims.d[d].smem_off >= 0 || p->dims.d[d].kind) continue;
      ++gathered;
      if (big < 0 || p->dims.d[d].n > p->dims.d[big].n) big = d;
    }
    if (gathered >= 2) p->dims.late = big;
  }
  p->vec = aligned;
  rc = pool_alloc(ctx, masks_total * sizeof(uint64_t) + 16, s, reinterpret_cast<void **>(&p->masks));
  if (rc) return fail(rc);
  {
    uint64_t off = 0;
    for (int d = 0; d < fact->n_dims; ++d) {
      p->dims.d[d].mask = p->masks + off;
      off += mask_slots[d];
    }
  }
  // the indexes of explicit keys: aux words, entry rows, row entries
  uint64_t words = 0;
  for (int d = 0; d < fact->n_dims; ++d)
    if (p->dims.d[d].kind)
      words += ((((uint64_t)p->dims.d[d].aux_words + 1) / 2 * 2 + p->dims.d[d].ents + dims[d].n) + 1) / 2 * 2;
  if (words) {
    rc = pool_alloc(ctx, words * sizeof(int32_t) + 16, s, reinterpret_cast<void **>(&p->hash_mem));
    if (rc) return fail(rc);
    uint64_t off = 0;
    for (int d = 0; d < fact->n_dims; ++d) {
      const gbj_star_dim &hd = dims[d];
      DimDev &dd = p->dims.d[d];
      if (!dd.kind) continue;
      int32_t *aux = p->hash_mem + off;  // 8-byte aligned: every block is an even number of words
      int32_t *erow = aux + (dd.aux_words + 1) / 2 * 2, *rent = erow + dd.ents;
      off += (dd.aux_words + 1) / 2 * 2 + dd.ents + hd.n;
      if (off % 2) ++off;
      const unsigned g = (unsigned)std::min<uint64_t>((hd.n + 255) / 256, (uint64_t)ctx->sm_count * 4);
      if (dd.kind == 1) {
        GBJ_CHECK_CUDA(ctx, cudaMemsetAsync(aux, 0, sizeof(int32_t) * dd.aux_words, s));
        k_star_range_bits<<<g, 256, 0, s>>>(hd.d_keys, (uint32_t)hd.n, dd.kmin, reinterpret_cast<uint32_t *>(aux),
                                            ctx->d_status);
        rc = after_launch(ctx, "k_star_range_bits", s);
        if (rc) return fail(rc);
        k_star_range_rank<<<1, 1024, 0, s>>>(reinterpret_cast<uint32_t *>(aux), dd.aux_words / 2);
        rc = after_launch(ctx, "k_star_range_rank", s);
        if (rc) return fail(rc);
        k_star_range_ent<<<g, 256, 0, s>>>(hd.d_keys, (uint32_t)hd.n, dd.kmin,
                                           reinterpret_cast<const uint32_t *>(aux), erow, rent);
        rc = after_launch(ctx, "k_star_range_ent", s);
        if (rc) return fail(rc);
      } else {
        k_star_fill<<<(unsigned)std::min<uint64_t>((dd.slots + 255) / 256, 4096), 256, 0, s>>>(aux, dd.slots,
                                                                                               dd.empty);
        rc = after_launch(ctx, "k_star_fill", s);
        if (rc) return fail(rc);
        k_star_hash_build<<<g, 256, 0, s>>>(hd.d_keys, (uint32_t)hd.n, aux, dd.slots, dd.empty, erow, rent,
                                            ctx->d_status);
        rc = after_launch(ctx, "k_star_hash_build", s);
        if (rc) return fail(rc);
      }
      dd.aux = aux;
      dd.ent_row = erow;
      dd.row_ent = rent;
    }
    // a duplicate primary key fails the plan
    const int src = gbj_sync(ctx, s);
    if (src != GBJ_OK) {
      if (src == GBJ_ERR_INVALID) set_error(ctx, GBJ_ERR_INVALID, "star: duplicate primary key in a dimension");
      return fail(src);
    }
  }
  rc = pool_alloc(ctx, sizeof(unsigned long long) * kMaxQ * kMaxGroups * 2, s,
                  reinterpret_cast<void **>(&p->gcnt));
  if (rc) return fail(rc);
  p->gsum = p->gcnt + (uint64_t)kMaxQ * kMaxGroups;
  rc = pool_alloc(ctx, sizeof(Desc), s, reinterpret_cast<void **>(&p->d_desc));
  if (rc) return fail(rc);
  for (int i = 0; i < 2; ++i) {
    cudaError_t e = cudaHostAlloc(reinterpret_cast<void **>(&p->h_desc[i]), sizeof(Desc), cudaHostAllocDefault);
    if (e != cudaSuccess) return fail(cuda_error(ctx, e, "cudaHostAlloc(star descriptors)"));
    e = cudaEventCreateWithFlags(&p->done[i], cudaEventDisableTiming);
    if (e != cudaSuccess) return fail(cuda_error(ctx, e, "cudaEventCreate"));
  }
  cudaError_t e = cudaStreamCreateWithFlags(&p->cap_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return fail(cuda_error(ctx, e, "cudaStreamCreate"));
  // static plus dynamic shared memory may pass 48 KB: opt in
  for (auto kern : {k_star_fact<true, false>, k_star_fact<false, false>, k_star_fact<true, true>,
                    k_star_fact<false, true>}) {
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p->fact_smem);
    if (e != cudaSuccess) return fail(cuda_error(ctx, e, "star: shared memory attribute"));
  }
  int per_sm = 1;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, p->keyed ? k_star_fact<true, true> : k_star_fact<true, false>,
                                                    kFactThreads, p->fact_smem);
  if (e != cudaSuccess) return fail(cuda_error(ctx, e, "occupancy"));
  p->fact_grid = ctx->sm_count * std::max(per_sm, 1);
  // the allocations above are stream-ordered on the context stream
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(cuda_error(ctx, e, "cudaStreamSynchronize"));
  *out = p;
  return GBJ_OK;
}

extern "C" int gbj_star_run(gbj_star_plan *p, const gbj_star_query *queries, int32_t n_queries,
                            const gbj_star_out *out, int32_t use_graph, void *stream) {
  if (!p) return GBJ_ERR_INVALID;
  gbj_ctx *ctx = p->ctx;
  GBJ_TRY(star_validate(p, queries, n_queries, out));
  cudaStream_t s = pick_stream(ctx, stream);
  const int slot = p->slot;
  // the slot's previous batch must have consumed its pinned descriptor
  if (p->used[slot]) GBJ_CHECK_CUDA(ctx, cudaEventSynchronize(p->done[slot]));
  star_fill_desc(p, queries, n_queries, out, p->h_desc[slot]);
  prof_mark(ctx, s);
  if (use_graph) {
    if (!p->exec[slot]) {
      GBJ_CHECK_CUDA(ctx, cudaStreamBeginCapture(p->cap_stream, cudaStreamCaptureModeThreadLocal));
      const int rc = star_enqueue(p, slot, p->cap_stream, true);
      cudaGraph_t graph = nullptr;
      const cudaError_t e = cudaStreamEndCapture(p->cap_stream, &graph);
      if (rc != GBJ_OK) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
      }
      if (e != cudaSuccess) return cuda_error(ctx, e, "cudaStreamEndCapture");
      const cudaError_t e2 = cudaGraphInstantiate(&p->exec[slot], graph, 0);
      cudaGraphDestroy(graph);
      if (e2 != cudaSuccess) {
        p->exec[slot] = nullptr;
        return cuda_error(ctx, e2, "cudaGraphInstantiate");
      }
    }
    GBJ_CHECK_CUDA(ctx, cudaGraphLaunch(p->exec[slot], s));
    // three kernels per replay; the profile shows the replay as one entry
    ctx->launches += 2;
    GBJ_TRY(after_launch(ctx, "star_graph", s));
  } else {
    GBJ_TRY(star_enqueue(p, slot, s, false));
  }
  GBJ_CHECK_CUDA(ctx, cudaEventRecord(p->done[slot], s));
  p->used[slot] = true;
  p->slot ^= 1;
  return GBJ_OK;
}

extern "C" void gbj_star_plan_destroy(gbj_star_plan *p) {
  if (!p) return;
  gbj_ctx *ctx = p->ctx;
  for (int i = 0; i < 2; ++i) {
    if (p->done[i]) {
      cudaEventSynchronize(p->done[i]);
      cudaEventDestroy(p->done[i]);
    }
    if (p->exec[i]) cudaGraphExecDestroy(p->exec[i]);
    if (p->h_desc[i]) cudaFreeHost(p->h_desc[i]);
  }
  if (p->cap_stream) cudaStreamDestroy(p->cap_stream);
  if (p->masks) pool_release(ctx, p->masks, ctx->stream);
  if (p->hash_mem) pool_release(ctx, p->hash_mem, ctx->stream);
  if (p->gcnt) pool_release(ctx, p->gcnt, ctx->stream);
  if (p->d_desc) pool_release(ctx, p->d_desc, ctx->stream);
  delete p;
}
