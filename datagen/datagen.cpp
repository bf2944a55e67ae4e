// Seeded synthetic column generator for the join / group-by workloads.
//
// Every value is a pure function of (seed, stream, row index), so columns can
// be generated in parallel, in any order, on any machine, and regenerated
// bit-identically.  Floating point appears only inside the Zipf sampler, which
// uses deterministic log/exp written here with + - * / and sqrt only (compiled
// with -ffp-contract=off), so x86-64 and aarch64 hosts produce the same bytes.
//
// Workload shapes (keys 1-based where the workload says so):
//   join-plain : R keys = permutation of 1..nR, payload U[0,1000);
//                S keys = U{1..nR}, payload U[0,1000).
//   join-radix : R keys = permutation of 1..nR; S rows hit R with prob 1/2;
//                hit keys = R key of a Zipf(theta) rank through a seeded
//                permutation, misses = U{nR+1..2nR}.
//   groupby    : key = bijection32(g), g = U{0..C-1} or Zipf(theta) rank - 1,
//                value = U[-2^20, 2^20).
#include "gbj_datagen.h"
#include "gbjoin.h"

#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace {

// SplitMix64 finaliser (Steele, Lea, Flood 2014).
inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

inline uint64_t stream_key(uint64_t seed, uint64_t stream) {
  return mix64(mix64(seed) ^ (stream * 0xD1B54A32D192ED03ULL));
}

// Counter-based 64-bit draw number i of a stream.
inline uint64_t draw(uint64_t key, uint64_t i) {
  return mix64(key ^ (i * 0x9E3779B97F4A7C15ULL));
}

// Uniform integer in [0, range) by 128-bit multiply-high (Lemire); the
// residual bias is below 2^-32 for every range used here.
inline uint64_t below(uint64_t r64, uint64_t range) {
  return (uint64_t)(((unsigned __int128)r64 * range) >> 64);
}

// Uniform double in [0, 1) from the top 53 bits.
inline double unit(uint64_t r64) { return (double)(r64 >> 11) * 0x1.0p-53; }

// ---------------------------------------------------------------------------
// Seeded bijection on [0, n): a 4-round mixing permutation on the enclosing
// power of two (odd multiply, add, xorshift -- each invertible mod 2^k), with
// cycle walking for n that is not a power of two.
struct Perm {
  uint64_t n = 1, mask = 0;
  int k = 0;
  uint64_t mul[4], add[4];
  int sh[4];
  Perm() = default;
  Perm(uint64_t n_, uint64_t key) : n(n_ ? n_ : 1) {
    k = 0;
    while ((1ULL << k) < n) ++k;
    mask = (k == 64) ? ~0ULL : ((1ULL << k) - 1);
    for (int r = 0; r < 4; ++r) {
      mul[r] = (draw(key, 2 * r) | 1ULL) & mask;
      if (mul[r] == 0) mul[r] = 1;
      add[r] = draw(key, 2 * r + 1) & mask;
      sh[r] = k / 2 + 1;
    }
  }
  inline uint64_t round_trip(uint64_t x) const {
    for (int r = 0; r < 4; ++r) {
      x = (x * mul[r]) & mask;
      x = (x + add[r]) & mask;
      if (sh[r] < k) x ^= x >> sh[r];
    }
    return x;
  }
  inline uint64_t operator()(uint64_t x) const {
    if (k == 0) return 0;
    uint64_t y = round_trip(x);
    while (y >= n) y = round_trip(y);
    return y;
  }
};

// Bijection on all 32-bit values (group keys spread over the int32 domain).
inline uint32_t perm32(uint32_t x, uint64_t key) {
  uint32_t a = (uint32_t)(key | 1u), b = (uint32_t)(key >> 32);
  uint32_t c = (uint32_t)(mix64(key) | 1u);
  x = x * a + b;
  x ^= x >> 16;
  x = x * c;
  x ^= x >> 13;
  x = x * a + (b ^ 0x5bd1e995u);
  x ^= x >> 15;
  return x;
}

// ---------------------------------------------------------------------------
// Deterministic elementary functions (basic IEEE operations only).
const double kLn2Hi = 6.93147180369123816490e-01;
const double kLn2Lo = 1.90821492927058770002e-10;
const double kLn2 = 0.69314718055994530942;

double det_exp(double x) {
  if (x > 709.0) return INFINITY;
  if (x < -745.0) return 0.0;
  double kd = x / kLn2;
  long k = (long)(kd < 0 ? kd - 0.5 : kd + 0.5);
  double r = (x - (double)k * kLn2Hi) - (double)k * kLn2Lo;  // |r| <= ~0.347
  // Taylor series to degree 16 (truncation error < 1e-17 relative).
  double term = 1.0, sum = 1.0;
  for (int i = 1; i <= 16; ++i) {
    term = term * r / (double)i;
    sum = sum + term;
  }
  return std::ldexp(sum, (int)k);
}

double det_log(double x) {
  if (!(x > 0.0)) return -INFINITY;
  int e;
  double m = std::frexp(x, &e);  // x = m * 2^e, m in [0.5, 1)
  if (m < 0.70710678118654752440) {
    m = m * 2.0;
    e -= 1;
  }
  // log(m) = 2 atanh(t), t = (m-1)/(m+1), |t| <= 0.1716
  double t = (m - 1.0) / (m + 1.0);
  double t2 = t * t, p = t, sum = t;
  for (int i = 3; i <= 41; i += 2) {
    p = p * t2;
    sum = sum + p / (double)i;
  }
  return 2.0 * sum + (double)e * kLn2;
}

// Zipf(theta) over ranks 1..N by rejection-inversion (W. Hoermann and
// G. Derflinger, "Rejection-inversion to generate variates from monotone
// discrete distributions", ACM TOMACS 6(3), 1996).  h(x) = x^-theta,
// H is an antiderivative of h, Hinv its inverse.
struct Zipf {
  double theta = 1.0, N = 1.0;
  double hx1 = 0, hN = 0, s = 0;
  Zipf() = default;
  Zipf(uint64_t n, double th) : theta(th), N((double)n) {
    hx1 = H(1.5) - 1.0;
    hN = H(N + 0.5);
    s = 2.0 - Hinv(H(2.5) - h(2.0));
  }
  double h(double x) const {
    if (theta == 1.0) return 1.0 / x;
    if (theta == 0.5) return 1.0 / std::sqrt(x);
    return det_exp(-theta * det_log(x));
  }
  double H(double x) const {
    if (theta == 1.0) return det_log(x);
    if (theta == 0.5) return 2.0 * (std::sqrt(x) - 1.0);
    return (det_exp((1.0 - theta) * det_log(x)) - 1.0) / (1.0 - theta);
  }
  double Hinv(double y) const {
    if (theta == 1.0) return det_exp(y);
    if (theta == 0.5) {
      double b = 1.0 + 0.5 * y;
      return b * b;
    }
    return det_exp(det_log(1.0 + (1.0 - theta) * y) / (1.0 - theta));
  }
  // rank in [1, N]; `key`/`i` select an independent uniform stream.
  uint64_t sample(uint64_t key, uint64_t i) const {
    for (uint64_t attempt = 0;; ++attempt) {
      double u01 = unit(draw(key, i * 64 + (attempt & 63) + (attempt >> 6) * 0x100000001ULL));
      double u = hN + u01 * (hx1 - hN);
      double x = Hinv(u);
      double kd = std::floor(x + 0.5);
      if (kd < 1.0) kd = 1.0;
      if (kd > N) kd = N;
      if (kd - x <= s || u >= H(kd + 0.5) - h(kd)) return (uint64_t)kd;
      if (attempt > 4096) return (uint64_t)kd;  // never reached in practice
    }
  }
};

enum Stream : uint64_t {
  kRKeyPerm = 1,
  kRPayload = 2,
  kSKey = 3,
  kSPayload = 4,
  kSHit = 5,
  kSZipf = 6,
  kRankPerm = 7,
  kSMiss = 8,
  kGKey = 9,
  kGVal = 10,
  kGPerm = 11,
  kGZipf = 12,
  kQKey = 13,
  kQGroup = 14,
  kQHit = 15,
  kQProbe = 16,
  kQVal = 17,
};

template <typename F>
void parallel_rows(uint64_t n, int threads, F f) {
  if (threads <= 0) threads = (int)std::thread::hardware_concurrency();
  if (threads <= 0) threads = 1;
  if (n < (1u << 16)) threads = 1;
  std::vector<std::thread> pool;
  uint64_t chunk = (n + threads - 1) / threads;
  for (int t = 0; t < threads; ++t) {
    uint64_t lo = t * chunk, hi = lo + chunk < n ? lo + chunk : n;
    if (lo >= hi) break;
    pool.emplace_back([=] { f(lo, hi); });
  }
  for (auto &th : pool) th.join();
}

}  // namespace

extern "C" {

uint64_t gbj_gen_rand(uint64_t seed, uint64_t stream, uint64_t i) {
  return draw(stream_key(seed, stream), i);
}

uint64_t gbj_gen_perm(uint64_t seed, uint64_t stream, uint64_t n, uint64_t i) {
  Perm p(n, stream_key(seed, stream));
  return p(i);
}

uint64_t gbj_gen_zipf(uint64_t seed, uint64_t stream, uint64_t n, double theta,
                      uint64_t i) {
  Zipf z(n, theta);
  return z.sample(stream_key(seed, stream), i);
}

double gbj_gen_det_log(double x) { return det_log(x); }
double gbj_gen_det_exp(double x) { return det_exp(x); }

int gbj_gen_build_side(uint64_t seed, uint64_t n, int32_t *keys,
                       int32_t *payload, int threads) {
  if (!keys && !payload) return GBJ_ERR_INVALID;
  if (n > (1ULL << 31)) return GBJ_ERR_INVALID;
  Perm perm(n, stream_key(seed, kRKeyPerm));
  uint64_t kp = stream_key(seed, kRPayload);
  parallel_rows(n, threads, [&](uint64_t lo, uint64_t hi) {
    for (uint64_t i = lo; i < hi; ++i) {
      if (keys) keys[i] = (int32_t)(1 + perm(i));
      if (payload) payload[i] = (int32_t)below(draw(kp, i), 1000);
    }
  });
  return GBJ_OK;
}

int gbj_gen_probe_uniform(uint64_t seed, uint64_t n, uint64_t n_build,
                          int32_t *keys, int32_t *payload, int threads) {
  if (n_build == 0 || n_build > (1ULL << 31)) return GBJ_ERR_INVALID;
  uint64_t kk = stream_key(seed, kSKey), kp = stream_key(seed, kSPayload);
  parallel_rows(n, threads, [&](uint64_t lo, uint64_t hi) {
    for (uint64_t i = lo; i < hi; ++i) {
      if (keys) keys[i] = (int32_t)(1 + below(draw(kk, i), n_build));
      if (payload) payload[i] = (int32_t)below(draw(kp, i), 1000);
    }
  });
  return GBJ_OK;
}

int gbj_gen_probe_zipf(uint64_t seed, uint64_t n, uint64_t n_build,
                       double theta, double hit_rate, int32_t *keys,
                       int32_t *payload, int threads) {
  if (n_build == 0 || n_build > (1ULL << 30)) return GBJ_ERR_INVALID;
  if (theta < 0.0 || hit_rate < 0.0 || hit_rate > 1.0) return GBJ_ERR_INVALID;
  uint64_t kh = stream_key(seed, kSHit), kz = stream_key(seed, kSZipf);
  uint64_t km = stream_key(seed, kSMiss), kp = stream_key(seed, kSPayload);
  Perm rank_perm(n_build, stream_key(seed, kRankPerm));
  Zipf zipf(n_build, theta > 0.0 ? theta : 1.0);
  uint64_t hit_threshold =
      hit_rate >= 1.0 ? ~0ULL : (uint64_t)(hit_rate * 18446744073709551616.0);
  parallel_rows(n, threads, [&](uint64_t lo, uint64_t hi) {
    for (uint64_t i = lo; i < hi; ++i) {
      if (keys) {
        bool hit = hit_rate >= 1.0 || draw(kh, i) < hit_threshold;
        if (hit) {
          uint64_t rank = theta > 0.0 ? zipf.sample(kz, i)
                                      : 1 + below(draw(kz, i), n_build);
          keys[i] = (int32_t)(1 + rank_perm(rank - 1));
        } else {
          keys[i] = (int32_t)(n_build + 1 + below(draw(km, i), n_build));
        }
      }
      if (payload) payload[i] = (int32_t)below(draw(kp, i), 1000);
    }
  });
  return GBJ_OK;
}

int gbj_gen_groupby(uint64_t seed, uint64_t n, uint64_t cardinality,
                    double theta, int32_t *keys, int32_t *values, int threads) {
  if (cardinality == 0 || cardinality > (1ULL << 32)) return GBJ_ERR_INVALID;
  uint64_t kg = stream_key(seed, kGKey), kv = stream_key(seed, kGVal);
  uint64_t kperm = stream_key(seed, kGPerm), kz = stream_key(seed, kGZipf);
  Perm gperm(cardinality, stream_key(seed, kRankPerm));
  Zipf zipf(cardinality, theta > 0.0 ? theta : 1.0);
  parallel_rows(n, threads, [&](uint64_t lo, uint64_t hi) {
    for (uint64_t i = lo; i < hi; ++i) {
      if (keys) {
        uint64_t g = theta > 0.0 ? gperm(zipf.sample(kz, i) - 1)
                                 : below(draw(kg, i), cardinality);
        keys[i] = (int32_t)perm32((uint32_t)g, kperm);
      }
      if (values)
        values[i] = (int32_t)((int64_t)below(draw(kv, i), 1u << 21) - (1 << 20));
    }
  });
  return GBJ_OK;
}

// out[i] = lo + uniform{0 .. hi - lo}, from column stream `stream`.
int gbj_gen_uniform_i32(uint64_t seed, uint64_t stream, uint64_t n, int32_t lo, int32_t hi,
                        int32_t *out, int threads) {
  if (hi < lo || (n && !out)) return GBJ_ERR_INVALID;
  const uint64_t key = stream_key(seed, stream);
  const uint64_t range = (uint64_t)((int64_t)hi - lo) + 1;
  parallel_rows(n, threads, [&](uint64_t a, uint64_t b) {
    for (uint64_t i = a; i < b; ++i) out[i] = (int32_t)((int64_t)lo + (int64_t)below(draw(key, i), range));
  });
  return GBJ_OK;
}

// One served join + group-by query: build keys = a seeded permutation of
// 1..n_build, build group uniform over [0, cardinality) spread over int32 by
// perm32; probe key = a uniform build key with probability match_rate, else
// a key above every build key; probe value U[0, 1000).
int gbj_gen_serve_query(uint64_t seed, uint64_t n_build, uint64_t n_probe, double match_rate,
                        uint64_t cardinality, int32_t *bk, int32_t *bg, int32_t *pk, int32_t *pv,
                        int threads) {
  if (n_build >= (1ULL << 30) || cardinality == 0 || match_rate < 0.0 || match_rate > 1.0)
    return GBJ_ERR_INVALID;
  Perm perm(n_build, stream_key(seed, kQKey));
  const uint64_t kgrp = stream_key(seed, kQGroup), khit = stream_key(seed, kQHit);
  const uint64_t kprobe = stream_key(seed, kQProbe), kval = stream_key(seed, kQVal);
  const uint64_t kgperm = stream_key(seed, kGPerm);
  parallel_rows(n_build, threads, [&](uint64_t lo, uint64_t hi) {
    for (uint64_t i = lo; i < hi; ++i) {
      if (bk) bk[i] = (int32_t)(1 + perm(i));
      if (bg) bg[i] = (int32_t)perm32((uint32_t)below(draw(kgrp, i), cardinality), kgperm);
    }
  });
  parallel_rows(n_probe, threads, [&](uint64_t lo, uint64_t hi) {
    for (uint64_t j = lo; j < hi; ++j) {
      if (pk) {
        const bool hit = n_build && unit(draw(khit, j)) < match_rate;
        const uint64_t r = draw(kprobe, j);
        pk[j] = hit ? (int32_t)(1 + below(r, n_build)) : (int32_t)(n_build + 1 + below(r, 1ULL << 30));
      }
      if (pv) pv[j] = (int32_t)below(draw(kval, j), 1000);
    }
  });
  return GBJ_OK;
}

}  // extern "C"
