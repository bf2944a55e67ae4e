// Context, resident device pool, status reporting.
//
// The pool replaces the reference's MemoryManager slab allocators and the
// buffer-manager's 2 MiB block pools (core/platform/lib/memory/
// memory-manager.cpp, buffer-manager.cu): one cudaMalloc at context creation,
// then host-side best-fit bookkeeping.  Scratch of every entry point comes
// from it, so steady-state calls never allocate device memory.
#include <cstdio>
#include <cstring>

#include "gbj_internal.cuh"

namespace gbj {

int set_error(gbj_ctx *ctx, int code, const std::string &msg) {
  if (ctx) ctx->last_error = msg;
  return code;
}

int cuda_error(gbj_ctx *ctx, cudaError_t e, const char *what) {
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  return set_error(ctx, e == cudaErrorMemoryAllocation ? GBJ_ERR_OOM : GBJ_ERR_CUDA, m);
}

cudaStream_t pick_stream(gbj_ctx *ctx, void *stream) {
  return stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
}

static cudaEvent_t prof_event(gbj_ctx *ctx, cudaStream_t s) {
  cudaEvent_t ev;
  if (cudaEventCreate(&ev) != cudaSuccess) return nullptr;
  if (cudaEventRecord(ev, s) != cudaSuccess) {
    cudaEventDestroy(ev);
    return nullptr;
  }
  ctx->prof_events.push_back(ev);
  return ev;
}

void prof_mark(gbj_ctx *ctx, cudaStream_t s) {
  if (!ctx->prof_on) return;
  std::lock_guard<std::mutex> g(ctx->mu);
  cudaEvent_t ev = prof_event(ctx, s);
  if (ev) ctx->prof_last[s] = ev;
}

int after_launch(gbj_ctx *ctx, const char *name, cudaStream_t s) {
  ctx->launches.fetch_add(1, std::memory_order_relaxed);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(ctx, e, name);
  if (ctx->prof_on) {
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaEvent_t b = prof_event(ctx, s);
    auto it = ctx->prof_last.find(s);
    if (b && it != ctx->prof_last.end()) ctx->prof_pending.push_back({name, it->second, b});
    if (b) ctx->prof_last[s] = b;
  }
  return GBJ_OK;
}

// Folds completed timing records into the per-kernel totals (syncs them).
static void prof_collect(gbj_ctx *ctx) {
  for (auto &r : ctx->prof_pending) {
    float ms = 0.f;
    if (cudaEventSynchronize(r.b) == cudaSuccess && cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
      auto &t = ctx->prof_totals[r.name];
      t.first += 1;
      t.second += ms;
    } else {
      (void)cudaGetLastError();
    }
  }
  ctx->prof_pending.clear();
  for (auto ev : ctx->prof_events) cudaEventDestroy(ev);
  ctx->prof_events.clear();
  ctx->prof_last.clear();
}

static constexpr uint64_t kAlign = 256;

static void pool_insert_free(Pool &p, uint64_t off, uint64_t size) {
  auto it = p.free_by_off.lower_bound(off);
  if (it != p.free_by_off.end() && off + size == it->first) {
    size += it->second;
    it = p.free_by_off.erase(it);
  }
  if (it != p.free_by_off.begin()) {
    auto prev = std::prev(it);
    if (prev->first + prev->second == off) {
      prev->second += size;
      return;
    }
  }
  p.free_by_off.emplace(off, size);
}

// Moves deferred blocks whose work is done (or that belong to `s`) back to
// the free map.  `wait` blocks on pending events of other streams.
static void pool_reclaim(Pool &p, cudaStream_t s, bool wait) {
  std::vector<Pool::Deferred> keep;
  for (auto &d : p.deferred) {
    bool ok = (d.stream == s);
    if (!ok) {
      cudaError_t q = wait ? cudaEventSynchronize(d.ev) : cudaEventQuery(d.ev);
      ok = (q == cudaSuccess);
      if (q != cudaSuccess && q != cudaErrorNotReady) (void)cudaGetLastError();
    }
    if (ok) {
      // Same-stream reuse is ordered after the recorded point; the event
      // is no longer needed either way.
      cudaEventDestroy(d.ev);
      pool_insert_free(p, d.off, d.size);
    } else {
      keep.push_back(d);
    }
  }
  p.deferred.swap(keep);
}

static bool pool_take(Pool &p, uint64_t size, uint64_t *off) {
  auto best = p.free_by_off.end();
  for (auto it = p.free_by_off.begin(); it != p.free_by_off.end(); ++it)
    if (it->second >= size && (best == p.free_by_off.end() || it->second < best->second))
      best = it;
  if (best == p.free_by_off.end()) return false;
  *off = best->first;
  uint64_t rest = best->second - size;
  uint64_t roff = best->first + size;
  p.free_by_off.erase(best);
  if (rest) p.free_by_off.emplace(roff, rest);
  return true;
}

int pool_alloc(gbj_ctx *ctx, uint64_t bytes, cudaStream_t s, void **out) {
  if (!out) return set_error(ctx, GBJ_ERR_INVALID, "pool_alloc: null out");
  std::lock_guard<std::mutex> g(ctx->mu);
  Pool &p = ctx->pool;
  uint64_t size = (bytes + kAlign - 1) / kAlign * kAlign;
  if (size == 0) size = kAlign;
  uint64_t off;
  if (p.limit && p.in_use + size > p.limit)
    return set_error(ctx, GBJ_ERR_OOM,
                     "device pool limit reached: requested " + std::to_string(bytes) + " B, in use " +
                         std::to_string(p.in_use) + " of the " + std::to_string(p.limit) + " B limit");
  pool_reclaim(p, s, false);
  if (!pool_take(p, size, &off)) {
    pool_reclaim(p, s, true);
    if (!pool_take(p, size, &off))
      return set_error(ctx, GBJ_ERR_OOM,
                       "device pool exhausted: requested " + std::to_string(bytes) +
                           " B, in use " + std::to_string(p.in_use) + " of " +
                           std::to_string(p.capacity) + " B");
  }
  p.used[off] = size;
  p.in_use += size;
  if (p.in_use > p.peak) p.peak = p.in_use;
  *out = p.base + off;
  return GBJ_OK;
}

int pool_release(gbj_ctx *ctx, void *ptr, cudaStream_t s) {
  if (!ptr) return GBJ_OK;
  std::lock_guard<std::mutex> g(ctx->mu);
  Pool &p = ctx->pool;
  uint64_t off = (uint64_t)((char *)ptr - p.base);
  auto it = p.used.find(off);
  if ((char *)ptr < p.base || it == p.used.end())
    return set_error(ctx, GBJ_ERR_INVALID, "pool_free: pointer not from this pool");
  uint64_t size = it->second;
  p.used.erase(it);
  p.in_use -= size;
  cudaEvent_t ev;
  if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventRecord(ev, s) != cudaSuccess) {
    // Capturing streams cannot be queried: fall back to a full sync.
    (void)cudaGetLastError();
    cudaStreamSynchronize(s);
    (void)cudaGetLastError();
    pool_insert_free(p, off, size);
    return GBJ_OK;
  }
  p.deferred.push_back({off, size, s, ev});
  return GBJ_OK;
}

AggSpec make_spec(const gbj_agg *aggs, int32_t n_aggs) {
  AggSpec s;
  memset(&s, 0, sizeof(s));
  s.n = n_aggs;
  for (int j = 0; j < n_aggs; ++j) {
    s.op[j] = aggs[j].op;
    s.operand[j] = aggs[j].operand;
  }
  return s;
}

int validate_aggs(gbj_ctx *ctx, const gbj_agg *aggs, int32_t n_aggs) {
  if (n_aggs < 1 || n_aggs > GBJ_MAX_AGGS || !aggs)
    return set_error(ctx, GBJ_ERR_INVALID, "n_aggs must be in [1, 8]");
  for (int j = 0; j < n_aggs; ++j) {
    if (aggs[j].op < GBJ_AGG_COUNT || aggs[j].op > GBJ_AGG_AND)
      return set_error(ctx, GBJ_ERR_INVALID, "bad aggregate op");
    if (aggs[j].operand < GBJ_VAL_ONE || aggs[j].operand > GBJ_VAL_BUILD_KEY)
      return set_error(ctx, GBJ_ERR_INVALID, "bad aggregate operand");
  }
  return GBJ_OK;
}

__global__ void k_init_agg_out(AggSpec s, int64_t *out) {
  int j = threadIdx.x;
  if (j < s.n) out[j] = gbjd::agg_identity(s.op[j]);
}

int init_agg_out(gbj_ctx *ctx, const AggSpec &spec, int64_t *d_out,
                 cudaStream_t s) {
  k_init_agg_out<<<1, 32, 0, s>>>(spec, d_out);
  return after_launch(ctx, "k_init_agg_out", s);
}

}  // namespace gbj

using namespace gbj;

extern "C" {

int gbj_ctx_create(int device, uint64_t pool_bytes, gbj_ctx **out) {
  if (!out) return GBJ_ERR_INVALID;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    (void)cudaGetLastError();
    return GBJ_ERR_CUDA;
  }
  if (device < 0 || device >= ndev) return GBJ_ERR_INVALID;
  if (cudaSetDevice(device) != cudaSuccess) return GBJ_ERR_CUDA;
  gbj_ctx *ctx = new gbj_ctx();
  ctx->device = device;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) {
    delete ctx;
    return GBJ_ERR_CUDA;
  }
  ctx->sm_count = prop.multiProcessorCount;
  ctx->l2_bytes = prop.l2CacheSize;
  ctx->smem_optin = prop.sharedMemPerBlockOptin;
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete ctx;
    return GBJ_ERR_CUDA;
  }
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  if (pool_bytes == 0) pool_bytes = (uint64_t)(free_b * 0.4);
  pool_bytes = (pool_bytes + kAlign - 1) / kAlign * kAlign;
  if (cudaMalloc((void **)&ctx->pool.base, pool_bytes) != cudaSuccess) {
    (void)cudaGetLastError();
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return GBJ_ERR_OOM;
  }
  ctx->pool.capacity = pool_bytes;
  ctx->pool.free_by_off.emplace(0, pool_bytes);
  void *st = nullptr;
  if (pool_alloc(ctx, 2 * sizeof(uint32_t), ctx->stream, &st) != GBJ_OK) {
    cudaFree(ctx->pool.base);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return GBJ_ERR_OOM;
  }
  ctx->d_status = (uint32_t *)st;
  cudaMemsetAsync(ctx->d_status, 0, 2 * sizeof(uint32_t), ctx->stream);
  cudaStreamSynchronize(ctx->stream);
  *out = ctx;
  return GBJ_OK;
}

int gbj_ctx_destroy(gbj_ctx *ctx) {
  if (!ctx) return GBJ_ERR_INVALID;
  cudaSetDevice(ctx->device);
  cudaDeviceSynchronize();
  prof_collect(ctx);
  for (auto &d : ctx->pool.deferred) cudaEventDestroy(d.ev);
  cudaFree(ctx->pool.base);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return GBJ_OK;
}

const char *gbj_last_error(gbj_ctx *ctx) {
  return ctx ? ctx->last_error.c_str() : noalloc_error_text_impl();
}

int gbj_ctx_device_info(gbj_ctx *ctx, int *sm_count, uint64_t *l2_bytes,
                        uint64_t *smem_per_block_optin) {
  if (!ctx) return GBJ_ERR_INVALID;
  if (sm_count) *sm_count = ctx->sm_count;
  if (l2_bytes) *l2_bytes = ctx->l2_bytes;
  if (smem_per_block_optin) *smem_per_block_optin = ctx->smem_optin;
  return GBJ_OK;
}

int gbj_sync(gbj_ctx *ctx, void *stream) {
  if (!ctx) return GBJ_ERR_INVALID;
  cudaStream_t s = pick_stream(ctx, stream);
  prof_mark(ctx, s);
  GBJ_CHECK_CUDA(ctx, cudaStreamSynchronize(s));
  uint32_t st[2] = {0, 0};
  GBJ_CHECK_CUDA(ctx, cudaMemcpyAsync(st, ctx->d_status, sizeof(st),
                                      cudaMemcpyDeviceToHost, s));
  GBJ_CHECK_CUDA(ctx, cudaStreamSynchronize(s));
  if (st[0]) {
    GBJ_CHECK_CUDA(ctx, cudaMemsetAsync(ctx->d_status, 0, sizeof(st), s));
    GBJ_CHECK_CUDA(ctx, cudaStreamSynchronize(s));
    if (st[0] & GBJ_DEV_CAPACITY)
      return set_error(ctx, GBJ_ERR_CAPACITY,
                       "device: table or output capacity exceeded");
    if (st[0] & GBJ_DEV_TIMEOUT)
      return set_error(ctx, GBJ_ERR_TIMEOUT, "device: bounded wait expired");
    return set_error(ctx, GBJ_ERR_INVALID, "device: consistency check failed");
  }
  return GBJ_OK;
}

uint64_t gbj_kernel_launches(gbj_ctx *ctx) {
  return ctx ? ctx->launches.load() : 0;
}

int gbj_profile_enable(gbj_ctx *ctx, int on) {
  if (!ctx) return GBJ_ERR_INVALID;
  std::lock_guard<std::mutex> g(ctx->mu);
  prof_collect(ctx);
  ctx->prof_totals.clear();
  ctx->prof_on = on != 0;
  return GBJ_OK;
}

int gbj_profile_kernel(gbj_ctx *ctx, const char *kernel, uint64_t *launches,
                       double *total_ms) {
  if (!ctx || !kernel) return GBJ_ERR_INVALID;
  std::lock_guard<std::mutex> g(ctx->mu);
  prof_collect(ctx);
  auto it = ctx->prof_totals.find(kernel);
  if (launches) *launches = it == ctx->prof_totals.end() ? 0 : it->second.first;
  if (total_ms) *total_ms = it == ctx->prof_totals.end() ? 0.0 : it->second.second;
  return GBJ_OK;
}

int gbj_profile_dump(gbj_ctx *ctx, char *buf, uint64_t buflen) {
  if (!ctx || !buf || buflen == 0) return GBJ_ERR_INVALID;
  std::lock_guard<std::mutex> g(ctx->mu);
  prof_collect(ctx);
  std::string out;
  for (auto &kv : ctx->prof_totals) {
    char line[256];
    snprintf(line, sizeof(line), "%s %llu %.6f\n", kv.first.c_str(),
             (unsigned long long)kv.second.first, kv.second.second);
    out += line;
  }
  if (out.size() + 1 > buflen) return GBJ_ERR_CAPACITY;
  memcpy(buf, out.c_str(), out.size() + 1);
  return GBJ_OK;
}

int gbj_pool_alloc(gbj_ctx *ctx, uint64_t bytes, void **d_ptr) {
  if (!ctx || !d_ptr) return GBJ_ERR_INVALID;
  return pool_alloc(ctx, bytes, ctx->stream, d_ptr);
}

int gbj_pool_free(gbj_ctx *ctx, void *d_ptr) {
  if (!ctx) return GBJ_ERR_INVALID;
  return pool_release(ctx, d_ptr, ctx->stream);
}

int gbj_ctx_set_pool_limit(gbj_ctx *ctx, uint64_t bytes) {
  if (!ctx) return GBJ_ERR_INVALID;
  std::lock_guard<std::mutex> g(ctx->mu);
  ctx->pool.limit = bytes;
  return GBJ_OK;
}

int gbj_pool_stats(gbj_ctx *ctx, uint64_t *capacity, uint64_t *in_use,
                   uint64_t *peak) {
  if (!ctx) return GBJ_ERR_INVALID;
  std::lock_guard<std::mutex> g(ctx->mu);
  if (capacity) *capacity = ctx->pool.capacity;
  if (in_use) *in_use = ctx->pool.in_use;
  if (peak) *peak = ctx->pool.peak;
  return GBJ_OK;
}

}  // extern "C"
