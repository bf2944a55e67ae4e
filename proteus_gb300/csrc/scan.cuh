// Device-wide exclusive prefix sum over uint64 counters (multi-level,
// stream-ordered).  Used for partition offsets and compaction.
#pragma once
#include "gbj_internal.cuh"

namespace gbj {

// out[i] = sum(in[0..i)); out[n] = total (out must hold n + 1 entries).
// `in` and `out` may alias.  Uses pool scratch for the block sums.
int scan_u64(gbj_ctx *ctx, const uint64_t *in, uint64_t *out, uint64_t n,
             cudaStream_t s);
// Same for uint32 inputs widened to uint64 outputs.
int scan_u32_to_u64(gbj_ctx *ctx, const uint32_t *in, uint64_t *out,
                    uint64_t n, cudaStream_t s);

}  // namespace gbj
