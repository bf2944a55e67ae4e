// Autotuner: times candidate plans of the radix join (join kernel block size
// and partition bits, which also fix one or two partitioning passes), the
// plain join (hash-table
// size, i.e. load factor) and the group-by (strategy and partition bits) on
// the caller's own inputs, and caches the fastest per size bucket in the
// context.  Entry points called without explicit sizing read the cache
// (the key is the operation and the log2 sizes of its inputs), so one tuning
// call decides every later call of that shape.
//
// The reference sizes these by hand in each plan (hash_bits,
// maxBuildInputSize, maxInputSize: core/olap/lib/plan/plan-parser.cpp,
// relbuilder.cpp:653-668) and fixes its radix bits at compile time
// (NUM_RADIX_BITS, core/platform/lib/util/radix/joins/radix-join.cpp).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <functional>
#include <sstream>
#include <vector>

#include "gbj_internal.cuh"

using namespace gbj;

std::string gbj::tune_key(const char *op, uint64_t a, uint64_t b) {
  return std::string(op) + " " + std::to_string(log2_ceil(std::max<uint64_t>(a, 1))) + " " +
         std::to_string(log2_ceil(std::max<uint64_t>(b, 1)));
}

int32_t gbj::tuned_value(gbj_ctx *ctx, const std::string &key) {
  std::lock_guard<std::mutex> g(ctx->mu);
  auto it = ctx->tuned.find(key);
  return it == ctx->tuned.end() ? -1 : it->second;
}

namespace {

void set_tuned(gbj_ctx *ctx, const std::string &key, int32_t v) {
  std::lock_guard<std::mutex> g(ctx->mu);
  if (v < 0) ctx->tuned.erase(key);
  else ctx->tuned[key] = v;
}

// Runs fn once to warm up, then `reps` times; *ms = the fastest run (CUDA
// events on s).  A failing candidate reports its status.
int time_candidate(gbj_ctx *ctx, cudaStream_t s, const std::function<int()> &fn, int reps, double *ms) {
  GBJ_TRY(fn());
  GBJ_TRY(gbj_sync(ctx, s));
  cudaEvent_t a, b;
  GBJ_CHECK_CUDA(ctx, cudaEventCreate(&a));
  GBJ_CHECK_CUDA(ctx, cudaEventCreate(&b));
  double best = 1e30;
  int rc = GBJ_OK;
  for (int r = 0; r < reps && rc == GBJ_OK; ++r) {
    cudaEventRecord(a, s);
    rc = fn();
    cudaEventRecord(b, s);
    if (rc == GBJ_OK) rc = gbj_sync(ctx, s);
    float t = 0;
    if (rc == GBJ_OK && cudaEventElapsedTime(&t, a, b) == cudaSuccess) best = std::min(best, (double)t);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *ms = best;
  return rc;
}

// Tries each candidate value under `key` and keeps the fastest.
int tune(gbj_ctx *ctx, cudaStream_t s, const std::string &key, const std::vector<int32_t> &cands,
         const std::function<int()> &fn, int32_t *best_out, double *best_ms) {
  const int32_t prev = tuned_value(ctx, key);
  int32_t best = -1;
  double best_t = 1e30;
  for (int32_t c : cands) {
    set_tuned(ctx, key, c);
    double t = 0;
    const int rc = time_candidate(ctx, s, fn, 2, &t);
    if (rc != GBJ_OK) {
      set_tuned(ctx, key, prev);
      return rc;
    }
    if (t < best_t) best_t = t, best = c;
  }
  set_tuned(ctx, key, best);
  if (best_out) *best_out = best;
  if (best_ms) *best_ms = best_t;
  return GBJ_OK;
}

}  // namespace

extern "C" int gbj_autotune_radix_join(gbj_ctx *ctx, const int32_t *d_build_keys, const int32_t *d_build_payload,
                                       uint64_t n_build, const int32_t *d_probe_keys,
                                       const int32_t *d_probe_payload, uint64_t n_probe, const gbj_agg *aggs,
                                       int32_t n_aggs, int32_t *best_bits, double *best_ms, void *stream) {
  if (!ctx) return GBJ_ERR_INVALID;
  if (n_build == 0 || n_probe == 0) return set_error(ctx, GBJ_ERR_INVALID, "autotune: empty input");
  cudaStream_t s = pick_stream(ctx, stream);
  int64_t *out = nullptr;
  GBJ_TRY(pool_alloc(ctx, GBJ_MAX_AGGS * sizeof(int64_t), s, reinterpret_cast<void **>(&out)));
  // both join kernel shapes (512 threads, two blocks per SM, chunks of 4608
  // build tuples; 1024 threads, one block, chunks of 9216), each with the
  // radix bits around its default: fewest bits whose mean partition fits
  const std::string kblock = tune_key("radixblock", n_build, n_probe);
  const int32_t prev_block = tuned_value(ctx, kblock);
  int rc = GBJ_OK;
  int32_t best_block = -1, best_b = -1;
  double best_t = 1e30;
  for (const int32_t block : {512, 1024}) {
    const double rmax = block == 1024 ? 9216.0 : 4608.0;
    int d = 1;
    while (d < 15 && (double)n_build / (double)(1u << d) > rmax) ++d;
    std::vector<int32_t> cands;
    for (int b = std::max(1, d - 2); b <= std::min(15, d + 2); ++b) cands.push_back(b);
    set_tuned(ctx, kblock, block);
    int32_t bits = -1;
    double t = 0;
    rc = tune(ctx, s, tune_key(block == 1024 ? "radix" : "radix512", n_build, n_probe), cands, [&] {
      return gbj_radix_join_agg(ctx, d_build_keys, d_build_payload, n_build, d_probe_keys, d_probe_payload,
                                n_probe, nullptr, aggs, n_aggs, out, s);
    }, &bits, &t);
    if (rc != GBJ_OK) break;
    if (t < best_t) best_t = t, best_block = block, best_b = bits;
  }
  pool_release(ctx, out, s);
  if (rc != GBJ_OK) {
    set_tuned(ctx, kblock, prev_block);
    return rc;
  }
  set_tuned(ctx, kblock, best_block);
  if (best_bits) *best_bits = best_b;
  if (best_ms) *best_ms = best_t;
  return GBJ_OK;
}

extern "C" int gbj_autotune_join(gbj_ctx *ctx, const int32_t *d_build_keys, const int32_t *d_build_payload,
                                 uint64_t n_build, const int32_t *d_probe_keys, const int32_t *d_probe_payload,
                                 uint64_t n_probe, const gbj_agg *aggs, int32_t n_aggs, int32_t *best_hash_bits,
                                 double *best_ms, void *stream) {
  if (!ctx) return GBJ_ERR_INVALID;
  if (n_build == 0) return set_error(ctx, GBJ_ERR_INVALID, "autotune: empty build side");
  cudaStream_t s = pick_stream(ctx, stream);
  const int b0 = log2_ceil(next_pow2(2 * n_build));
  std::vector<int32_t> cands;  // load factor 1/2, 1/4, 1/8
  for (int b = b0; b <= std::min(31, b0 + 2); ++b) cands.push_back(std::max(b, 6));
  int64_t *out = nullptr;
  GBJ_TRY(pool_alloc(ctx, GBJ_MAX_AGGS * sizeof(int64_t), s, reinterpret_cast<void **>(&out)));
  const int rc = tune(ctx, s, tune_key("join", n_build, 0), cands, [&] {
    gbj_table *t = nullptr;
    GBJ_TRY(gbj_join_build(ctx, d_build_keys, d_build_payload, n_build, 0, 0, s, &t));
    const int r = gbj_join_probe_agg(ctx, t, d_probe_keys, d_probe_payload, n_probe, aggs, n_aggs, out, s);
    gbj_table_destroy(ctx, t);
    return r;
  }, best_hash_bits, best_ms);
  pool_release(ctx, out, s);
  return rc;
}

extern "C" int gbj_autotune_groupby(gbj_ctx *ctx, const int32_t *d_keys, const int32_t *d_values, uint64_t n,
                                    uint64_t expected_groups, int32_t *best_strategy, int32_t *best_bits,
                                    double *best_ms, void *stream) {
  if (!ctx) return GBJ_ERR_INVALID;
  if (n == 0 || expected_groups == 0)
    return set_error(ctx, GBJ_ERR_INVALID, "autotune: empty input or unknown group count");
  cudaStream_t s = pick_stream(ctx, stream);
  // strategy 1 (on-chip + global table) and strategy 2 around its default bits
  const uint64_t groups_cap = std::max<uint64_t>(1024, std::min<uint64_t>(expected_groups, n));
  int d = 1;
  while (d < 15 && (groups_cap >> d) > 1024) ++d;
  std::vector<int32_t> cands = {(1 << 8) | 0};
  for (int b = std::max(1, d - 1); b <= std::min(15, d + 2); ++b) cands.push_back((2 << 8) | b);
  const uint64_t cap = std::min<uint64_t>(n, expected_groups) + 16;
  char *mem = nullptr;
  const uint64_t bytes = cap * (4 + 8 + 8 + 4 + 4) + 64;
  GBJ_TRY(pool_alloc(ctx, bytes, s, reinterpret_cast<void **>(&mem)));
  int64_t *oc = reinterpret_cast<int64_t *>(mem);
  int64_t *os = oc + cap;
  int32_t *ok = reinterpret_cast<int32_t *>(os + cap);
  int32_t *omn = ok + cap, *omx = omn + cap;
  uint64_t *ng = reinterpret_cast<uint64_t *>(omx + cap + 1);
  ng = reinterpret_cast<uint64_t *>((reinterpret_cast<uintptr_t>(ng) + 7) & ~uintptr_t(7));
  gbj_groupby_params prm{0, 0, 0, expected_groups};
  int32_t best = -1;
  const int rc = tune(ctx, s, tune_key("groupby", n, expected_groups), cands, [&] {
    return gbj_groupby(ctx, d_keys, d_values, n, &prm, ok, oc, os, omn, omx, cap, ng, s);
  }, &best, best_ms);
  pool_release(ctx, mem, s);
  if (rc == GBJ_OK) {
    if (best_strategy) *best_strategy = best >> 8;
    if (best_bits) *best_bits = best & 0xff;
  }
  return rc;
}

extern "C" int gbj_tune_lookup(gbj_ctx *ctx, const char *op, uint64_t a, uint64_t b, int32_t *value) {
  if (!ctx || !op || !value) return GBJ_ERR_INVALID;
  *value = tuned_value(ctx, tune_key(op, a, b));
  return GBJ_OK;
}

extern "C" int gbj_tune_clear(gbj_ctx *ctx) {
  if (!ctx) return GBJ_ERR_INVALID;
  std::lock_guard<std::mutex> g(ctx->mu);
  ctx->tuned.clear();
  return GBJ_OK;
}

extern "C" int gbj_tune_save(gbj_ctx *ctx, const char *path) {
  if (!ctx || !path) return GBJ_ERR_INVALID;
  std::ofstream f(path);
  if (!f) return set_error(ctx, GBJ_ERR_INVALID, std::string("tune: cannot write ") + path);
  std::lock_guard<std::mutex> g(ctx->mu);
  for (const auto &kv : ctx->tuned) f << kv.first << " " << kv.second << "\n";
  return f ? GBJ_OK : GBJ_ERR_INVALID;
}

extern "C" int gbj_tune_load(gbj_ctx *ctx, const char *path) {
  if (!ctx || !path) return GBJ_ERR_INVALID;
  std::ifstream f(path);
  if (!f) return set_error(ctx, GBJ_ERR_INVALID, std::string("tune: cannot read ") + path);
  std::string line;
  std::map<std::string, int32_t> got;
  while (std::getline(f, line)) {
    if (line.empty()) continue;
    std::istringstream ls(line);
    std::string op, a, b;
    int32_t v;
    if (!(ls >> op >> a >> b >> v)) return set_error(ctx, GBJ_ERR_INVALID, "tune: malformed line: " + line);
    got[op + " " + a + " " + b] = v;
  }
  std::lock_guard<std::mutex> g(ctx->mu);
  for (const auto &kv : got) ctx->tuned[kv.first] = kv.second;
  return GBJ_OK;
}
