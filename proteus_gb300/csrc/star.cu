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
  uint64_t *mask;  // [n]
  int32_t smem_off;  // offset of the mask copy in the fact kernel's shared memory, -1 none
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
    dd.mask[r] = m;
  }
}

struct GroupSpec {
  int32_t gd[2], ga[2], gmin[2];
  uint32_t gspan[2];
};

// The (row, query) matches of one fact row: COUNT and SUM(price * quantity)
// into the query's dense group arrays.
__device__ __forceinline__ void star_matches(const Dims &dims, uint64_t m, const GroupSpec *sg,
                                             const int32_t (&fk)[kMaxDims], int32_t qty,
                                             int32_t price, unsigned long long *__restrict__ gcnt,
                                             unsigned long long *__restrict__ gsum,
                                             uint32_t *status) {
  const unsigned long long val = (unsigned long long)((int64_t)price * (int64_t)qty);
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
      key[s] = attr_at(dd, gs.ga[s], (uint32_t)(k - dd.base));
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
__device__ __forceinline__ uint64_t dim_mask(const DimDev &dd, const uint64_t *s_mask, int32_t k,
                                             uint64_t nojoin) {
  const uint32_t idx = (uint32_t)(k - dd.base);
  if (idx >= dd.n) return nojoin;
  return dd.smem_off >= 0 ? s_mask[dd.smem_off + idx] : __ldg(dd.mask + idx);
}

// Fact scan.  Each thread takes 4 rows per round (one 128-bit load per
// column) and issues every mask lookup of the 4 rows before combining them,
// so a thread keeps up to 16 independent gathers in flight instead of
// walking dimensions one dependent load at a time.
template <bool kVec>
__global__ void __launch_bounds__(kFactThreads)
    k_star_fact(const Desc *__restrict__ desc, FactDev f, Dims dims,
                unsigned long long *__restrict__ gcnt, unsigned long long *__restrict__ gsum,
                uint32_t *status) {
  extern __shared__ uint64_t s_mask[];  // masks of the small dimensions
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
    if (d < dims.nd && dims.d[d].smem_off >= 0)
      for (uint32_t i = threadIdx.x; i < dims.d[d].n; i += blockDim.x)
        s_mask[dims.d[d].smem_off + i] = dims.d[d].mask[i];
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
        if (d < dims.nd && d != dims.late) {
          m[0] &= dim_mask(dims.d[d], s_mask, k4[d].x, nojoin[d]);
          m[1] &= dim_mask(dims.d[d], s_mask, k4[d].y, nojoin[d]);
          m[2] &= dim_mask(dims.d[d], s_mask, k4[d].z, nojoin[d]);
          m[3] &= dim_mask(dims.d[d], s_mask, k4[d].w, nojoin[d]);
        }
      }
      // the largest gathered dimension last, only for rows some query still
      // passes (most rows have failed every query by then)
#pragma unroll
      for (int d = 0; d < kMaxDims; ++d) {
        if (d < dims.nd && d == dims.late) {
          if (m[0]) m[0] &= dim_mask(dims.d[d], s_mask, k4[d].x, nojoin[d]);
          if (m[1]) m[1] &= dim_mask(dims.d[d], s_mask, k4[d].y, nojoin[d]);
          if (m[2]) m[2] &= dim_mask(dims.d[d], s_mask, k4[d].z, nojoin[d]);
          if (m[3]) m[3] &= dim_mask(dims.d[d], s_mask, k4[d].w, nojoin[d]);
        }
      }
      if (m[0]) {
        const int32_t fk[kMaxDims] = {k4[0].x, k4[1].x, k4[2].x, k4[3].x};
        star_matches(dims, m[0], sg, fk, q4.x, p4.x, gcnt, gsum, status);
      }
      if (m[1]) {
        const int32_t fk[kMaxDims] = {k4[0].y, k4[1].y, k4[2].y, k4[3].y};
        star_matches(dims, m[1], sg, fk, q4.y, p4.y, gcnt, gsum, status);
      }
      if (m[2]) {
        const int32_t fk[kMaxDims] = {k4[0].z, k4[1].z, k4[2].z, k4[3].z};
        star_matches(dims, m[2], sg, fk, q4.z, p4.z, gcnt, gsum, status);
      }
      if (m[3]) {
        const int32_t fk[kMaxDims] = {k4[0].w, k4[1].w, k4[2].w, k4[3].w};
        star_matches(dims, m[3], sg, fk, q4.w, p4.w, gcnt, gsum, status);
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
      if (d < dims.nd) m &= dim_mask(dims.d[d], s_mask, fk[d], nojoin[d]);
    }
    if (m) star_matches(dims, m, sg, fk, f.qty[r], f.price[r], gcnt, gsum, status);
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

}  // namespace

struct gbj_star_plan {
  gbj_ctx *ctx = nullptr;
  FactDev fact{};
  Dims dims{};
  gbj_star_dim host_dims[kMaxDims]{};
  bool vec = false;
  uint64_t *masks = nullptr;
  size_t fact_smem = 0;
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
  if (p->vec)
    k_star_fact<true><<<p->fact_grid, kFactThreads, p->fact_smem, s>>>(p->d_desc, p->fact, p->dims,
                                                                       p->gcnt, p->gsum, ctx->d_status);
  else
    k_star_fact<false><<<p->fact_grid, kFactThreads, p->fact_smem, s>>>(p->d_desc, p->fact, p->dims,
                                                                        p->gcnt, p->gsum, ctx->d_status);
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
  uint64_t rows = 0;
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
    dd.smem_off = -1;
    if (hd.n <= kSmemMaskRows && p->fact_smem / sizeof(uint64_t) + hd.n <= kSmemMaskMax) {
      dd.smem_off = (int32_t)(p->fact_smem / sizeof(uint64_t));
      p->fact_smem += hd.n * sizeof(uint64_t);
    }
  }
  p->dims.total_rows = rows;
  // the late dimension: the largest one gathered from L2, when another
  // gathered dimension is checked before it
  p->dims.late = -1;
  {
    int gathered = 0, big = -1;
    for (int d = 0; d < fact->n_dims; ++d) {
      if (p->dims.d[d].smem_off >= 0) continue;
      ++gathered;
      if (big < 0 || p->dims.d[d].n > p->dims.d[big].n) big = d;
    }
    if (gathered >= 2) p->dims.late = big;
  }
  p->vec = aligned;
  cudaStream_t s = ctx->stream;
  int rc = pool_alloc(ctx, rows * sizeof(uint64_t) + 16, s, reinterpret_cast<void **>(&p->masks));
  if (rc) return fail(rc);
  for (int d = 0; d < fact->n_dims; ++d) p->dims.d[d].mask = p->masks + p->dims.d[d].row0;
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
  int per_sm = 1;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_star_fact<true>, kFactThreads, p->fact_smem);
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
  if (p->gcnt) pool_release(ctx, p->gcnt, ctx->stream);
  if (p->d_desc) pool_release(ctx, p->d_desc, ctx->stream);
  delete p;
}
