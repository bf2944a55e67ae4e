// Internal definitions shared by the gbjoin translation units.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <map>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "gbjoin.h"

// ----------------------------------------------------------------- status
// Device-side error bits latched into the context's status word; gbj_sync
// maps the first one to a gbj_status.
enum : uint32_t {
  GBJ_DEV_CAPACITY = 1u << 0,  // a table / output buffer overflowed
  GBJ_DEV_TIMEOUT = 1u << 1,   // a bounded spin gave up
  GBJ_DEV_INVALID = 1u << 2,   // a device-side consistency check failed
  GBJ_DEV_GROUPS = 1u << 3,    // a served query's group table was full
};

// Upper bound on the iterations of any device-side spin (bounded waits).
constexpr uint32_t kSpinLimit = 1u << 22;

struct Pool {
  // Best-fit allocator over one cudaMalloc'd block.  Freed blocks stay
  // "deferred" behind a CUDA event until the stream that used them has
  // passed that point; a request on the same stream may reuse them at once
  // (stream order), a request on another stream reclaims them once the
  // event has completed (or waits on it when nothing else fits).
  char *base = nullptr;
  uint64_t capacity = 0, in_use = 0, peak = 0;
  uint64_t limit = 0;  // gbj_ctx_set_pool_limit: most bytes handed out (0 = capacity)
  std::map<uint64_t, uint64_t> free_by_off;  // offset -> size
  std::unordered_map<uint64_t, uint64_t> used;  // offset -> size
  struct Deferred {
    uint64_t off, size;
    cudaStream_t stream;
    cudaEvent_t ev;
  };
  std::vector<Deferred> deferred;
};

struct gbj_ctx {
  int device = 0;
  int sm_count = 0;
  uint64_t l2_bytes = 0;
  uint64_t smem_optin = 0;
  cudaStream_t stream = nullptr;
  uint32_t *d_status = nullptr;  // [0] error bits, [1] detail
  Pool pool;
  std::mutex mu;
  std::string last_error;
  std::atomic<uint64_t> launches{0};
  // kernel timing (gbj_profile_*): one event after every launch; a kernel's
  // time is the interval since the previous event on its stream.
  bool prof_on = false;
  struct ProfRec {
    const char *name;
    cudaEvent_t a, b;
  };
  std::vector<ProfRec> prof_pending;
  std::vector<cudaEvent_t> prof_events;
  std::unordered_map<cudaStream_t, cudaEvent_t> prof_last;
  std::map<std::string, std::pair<uint64_t, double>> prof_totals;
  // autotuner decisions: "<op> <log2 size> <log2 size>" -> chosen value
  std::map<std::string, int32_t> tuned;
};

struct gbj_table {
  // 32-byte buckets of four slots (keys, then payloads or rows + 1), the
  // rows of a payload table, the metadata words and the INT32_MIN side
  // list, in one pool block starting at `slots`.
  void *slots = nullptr;
  int4 *rows = nullptr;
  uint32_t *meta = nullptr;
  int32_t *side = nullptr;
  uint64_t mask = 0;          // slots - 1 (4 slots per bucket)
  const int32_t *keys = nullptr;
  const int32_t *payload = nullptr;
  uint64_t n = 0;
  bool i64 = false;  // int64 keys (gbj_join_build_i64): 2-slot buckets
};

// ------------------------------------------------------------ host helpers
namespace gbj {

int set_error(gbj_ctx *ctx, int code, const std::string &msg);
int cuda_error(gbj_ctx *ctx, cudaError_t e, const char *what);
cudaStream_t pick_stream(gbj_ctx *ctx, void *stream);
int pool_alloc(gbj_ctx *ctx, uint64_t bytes, cudaStream_t s, void **out);
// Releases after the work already enqueued on `s` (records an event).
int pool_release(gbj_ctx *ctx, void *p, cudaStream_t s);

// Scratch allocations owned by one entry-point call; released (deferred on
// the call's stream) when the scope ends.
class Scratch {
 public:
  Scratch(gbj_ctx *ctx, cudaStream_t s) : ctx_(ctx), s_(s) {}
  ~Scratch() {
    for (void *p : ptrs_) pool_release(ctx_, p, s_);
  }
  template <typename T>
  int get(uint64_t count, T **out) {
    void *p = nullptr;
    int rc = pool_alloc(ctx_, count * sizeof(T) + 16, s_, &p);
    if (rc) return rc;
    ptrs_.push_back(p);
    *out = static_cast<T *>(p);
    return GBJ_OK;
  }

 private:
  gbj_ctx *ctx_;
  cudaStream_t s_;
  std::vector<void *> ptrs_;
};

inline uint64_t next_pow2(uint64_t v) {
  uint64_t p = 1;
  while (p < v) p <<= 1;
  return p;
}
inline int log2_ceil(uint64_t v) {
  int b = 0;
  while ((1ULL << b) < v) ++b;
  return b;
}

// Text of the last failure of gbj_join_agg_noalloc on the calling thread.
const char *noalloc_error_text_impl();

// Counts a kernel launch, records its timing event when profiling is on,
// and turns a launch error into a status.
int after_launch(gbj_ctx *ctx, const char *name, cudaStream_t s);
// Marks the start of an entry point's work on `s` (profiling only).
void prof_mark(gbj_ctx *ctx, cudaStream_t s);

int validate_aggs(gbj_ctx *ctx, const gbj_agg *aggs, int32_t n_aggs);

// Autotuner cache (keys built by tune_key; -1 = no decision yet).
std::string tune_key(const char *op, uint64_t a, uint64_t b);
int32_t tuned_value(gbj_ctx *ctx, const std::string &key);

// Kernel-side aggregate description (passed by value).
struct AggSpec {
  int32_t n;
  int32_t op[GBJ_MAX_AGGS];
  int32_t operand[GBJ_MAX_AGGS];
};
AggSpec make_spec(const gbj_agg *aggs, int32_t n_aggs);

// Initialises d_out[j] to the identity of aggregate j (stream-ordered).
int init_agg_out(gbj_ctx *ctx, const AggSpec &spec, int64_t *d_out,
                 cudaStream_t s);

}  // namespace gbj

// ---------------------------------------------------------- device helpers
namespace gbjd {

// murmur3 fmix32 (32-bit), the placement hash of every table and partition.
__host__ __device__ __forceinline__ uint32_t fmix32(uint32_t h) {
  h ^= h >> 16;
  h *= 0x85ebca6bu;
  h ^= h >> 13;
  h *= 0xc2b2ae35u;
  h ^= h >> 16;
  return h;
}

// Inverse of fmix32 (each step of the finaliser is invertible modulo 2^32:
// x ^= x >> 16 is its own inverse, x ^= x >> 13 is undone by
// x ^= (x >> 13) ^ (x >> 26), and the odd multipliers have the modular
// inverses 0xa5cb9243 = 0x85ebca6b^-1 and 0x7ed1b41d = 0xc2b2ae35^-1).
// Partitioned join tuples carry fmix32(key); this recovers the key.
__host__ __device__ __forceinline__ uint32_t fmix32_inv(uint32_t h) {
  h ^= h >> 16;
  h *= 0x7ed1b41du;
  h ^= (h >> 13) ^ (h >> 26);
  h *= 0xa5cb9243u;
  h ^= h >> 16;
  return h;
}

__device__ __forceinline__ void latch(uint32_t *status, uint32_t bit) {
  atomicOr(status, bit);
}

__device__ __forceinline__ int64_t operand_value(int operand, int64_t key,
                                                 int64_t bval, int64_t pval,
                                                 int64_t brow, int64_t prow) {
  switch (operand) {
    case GBJ_VAL_ONE: return 1;
    case GBJ_VAL_BUILD: return bval;
    case GBJ_VAL_PROBE: return pval;
    case GBJ_VAL_PRODUCT: return bval * pval;
    case GBJ_VAL_BUILD_ROWID: return brow;
    case GBJ_VAL_PROBE_ROWID: return prow;
    case GBJ_VAL_ROWID_XOR: return brow ^ prow;
    case GBJ_VAL_BUILD_KEY: return key;
    default: return 0;
  }
}

// Identity of each aggregate: 0 for COUNT / SUM / OR, the int64 extremes for
// MIN / MAX, true (1) for AND.
__device__ __forceinline__ int64_t agg_identity(int op) {
  return op == GBJ_AGG_MIN ? INT64_MAX
                           : (op == GBJ_AGG_MAX ? INT64_MIN : (op == GBJ_AGG_AND ? 1 : 0));
}

struct Acc {
  int64_t v[GBJ_MAX_AGGS];
  __device__ __forceinline__ void init(const gbj::AggSpec &s) {
#pragma unroll
    for (int j = 0; j < GBJ_MAX_AGGS; ++j) v[j] = j < s.n ? agg_identity(s.op[j]) : 0;
  }
  // Branch-free: operand and op are selected with predicated moves, so a
  // match costs a few instructions per aggregate and no jump tables.
  __device__ __forceinline__ void update(const gbj::AggSpec &s, int64_t key,
                                         int64_t bval, int64_t pval,
                                         int64_t brow, int64_t prow) {
    const int64_t prod = bval * pval, xr = brow ^ prow;
#pragma unroll
    for (int j = 0; j < GBJ_MAX_AGGS; ++j) {
      if (j < s.n) {
        const int o = s.operand[j];
        int64_t x = o == GBJ_VAL_BUILD ? bval : 1;
        x = o == GBJ_VAL_PROBE ? pval : x;
        x = o == GBJ_VAL_PRODUCT ? prod : x;
        x = o == GBJ_VAL_BUILD_ROWID ? brow : x;
        x = o == GBJ_VAL_PROBE_ROWID ? prow : x;
        x = o == GBJ_VAL_ROWID_XOR ? xr : x;
        x = o == GBJ_VAL_BUILD_KEY ? (int64_t)key : x;
        const int op = s.op[j];
        const int64_t add = v[j] + (op == GBJ_AGG_COUNT ? 1 : x);
        const int64_t mm = op == GBJ_AGG_MIN ? (x < v[j] ? x : v[j]) : (x > v[j] ? x : v[j]);
        // OR / AND are logical: the operand is true when it is not zero
        const int64_t tv = (int64_t)(x != 0);
        const int64_t lg = op == GBJ_AGG_OR ? (v[j] | tv) : (v[j] & tv);
        v[j] = op <= GBJ_AGG_SUM ? add : (op <= GBJ_AGG_MAX ? mm : lg);
      }
    }
  }
};

__device__ __forceinline__ int64_t combine(int op, int64_t a, int64_t b) {
  if (op == GBJ_AGG_MIN) return a < b ? a : b;
  if (op == GBJ_AGG_MAX) return a > b ? a : b;
  if (op == GBJ_AGG_OR) return a | b;
  if (op == GBJ_AGG_AND) return a & b;
  return a + b;
}

// Block-wide reduction of the accumulators; thread 0 applies one atomic per
// aggregate to d_out.  `red` must hold 32 * GBJ_MAX_AGGS int64 of shared
// memory.  Must be called by all threads of the block.
__device__ __forceinline__ void block_flush(const gbj::AggSpec &s, Acc &a,
                                            int64_t *red, int64_t *d_out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int j = 0; j < GBJ_MAX_AGGS; ++j) {
    if (j < s.n) {
      int64_t x = a.v[j];
      for (int o = 16; o > 0; o >>= 1)
        x = combine(s.op[j], x, __shfl_xor_sync(0xffffffffu, x, o));
      if (lane == 0) red[warp * GBJ_MAX_AGGS + j] = x;
    }
  }
  __syncthreads();
  if (threadIdx.x < GBJ_MAX_AGGS && (int)threadIdx.x < s.n) {
    const int j = threadIdx.x;
    int64_t x = agg_identity(s.op[j]);
    for (int w = 0; w < nwarps; ++w) x = combine(s.op[j], x, red[w * GBJ_MAX_AGGS + j]);
    if (s.op[j] == GBJ_AGG_MIN) {
      if (x != INT64_MAX) atomicMin((long long *)&d_out[j], (long long)x);
    } else if (s.op[j] == GBJ_AGG_MAX) {
      if (x != INT64_MIN) atomicMax((long long *)&d_out[j], (long long)x);
    } else if (s.op[j] == GBJ_AGG_OR) {
      if (x) atomicOr((unsigned long long *)&d_out[j], 1ull);
    } else if (s.op[j] == GBJ_AGG_AND) {
      if (!x) atomicAnd((unsigned long long *)&d_out[j], 0ull);
    } else {
      atomicAdd((unsigned long long *)&d_out[j], (unsigned long long)x);
    }
  }
}

}  // namespace gbjd

#define GBJ_CHECK_CUDA(ctx, expr)                         \
  do {                                                    \
    cudaError_t _e = (expr);                              \
    if (_e != cudaSuccess) return gbj::cuda_error(ctx, _e, #expr); \
  } while (0)

#define GBJ_TRY(expr)          \
  do {                         \
    int _rc = (expr);          \
    if (_rc != GBJ_OK) return _rc; \
  } while (0)
