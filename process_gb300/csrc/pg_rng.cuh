// Counter-based randomness and the integer/FP64 samplers of the placement and
// sequencing kernels.
//
// Every random decision of the hot path is a pure function of
// (seed, stream tag, object id, draw index), computed with Philox4x32-10
// (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3",
// SC'11). The CPU replay in oracle/ restates the same functions, so device and
// host results agree bit for bit. The reference draws from one sequential
// std::mt19937_64 stream (src/mutation_engine.hpp:50); a counter-based generator
// is what lets every edge, mutation and read draw independently.
//
// Floating-point samplers use only IEEE-754 +, -, *, / and explicit fma on
// doubles; this file is compiled with --fmad=false so the compiler does not
// contract anything, and log is computed by our own routine (below), never by
// the CUDA math library.
#pragma once
#include "pg_kernels.h"
#include <cstdint>

namespace pg {

// ---------------------------------------------------------------- Philox4x32-10
struct U4 { uint32_t x, y, z, w; };

__device__ __forceinline__ U4 philox(uint32_t k0, uint32_t k1,
                                     uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3) {
#pragma unroll
  for (int i = 0; i < 10; ++i) {
    const uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
    const uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
    const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
  return {c0, c1, c2, c3};
}

// The round keys of one key, computed on the host: a kernel that takes them
// as a parameter reads them as constant operands instead of stepping the
// key schedule per block (the same words as philox()).
struct RoundKeys { uint32_t k0[10], k1[10]; };

__host__ __device__ inline RoundKeys round_keys(uint32_t k0, uint32_t k1) {
  RoundKeys r;
  for (int i = 0; i < 10; ++i) { r.k0[i] = k0; r.k1[i] = k1; k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
  return r;
}

__device__ __forceinline__ U4 philox(const RoundKeys& rk, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3) {
#pragma unroll
  for (int i = 0; i < 10; ++i) {
    const uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
    const uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
    const uint32_t n0 = hi1 ^ c1 ^ rk.k0[i], n2 = hi0 ^ c3 ^ rk.k1[i];
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
  }
  return {c0, c1, c2, c3};
}

// Stream tags (counter word c3). One tag per kind of decision keeps the
// streams of different decisions disjoint for the same object id.
enum : uint32_t {
  TAG_EDGE_SNV = 1, TAG_EDGE_INDEL = 2, TAG_EDGE_CNA = 3,
  TAG_SNV = 4, TAG_INDEL = 5, TAG_DRIVER = 6,
  TAG_TILE_SPLIT = 7, TAG_PAIR = 8,
  TAG_GENOME = 11, TAG_CNA = 12
};


// uniform index in [0, n) from one 32-bit word (floor(u * n / 2^32))
__device__ __forceinline__ uint32_t uniform_index32(uint32_t u, uint32_t n) {
  return __umulhi(u, n);
}
// uniform index in [0, n) from a 64-bit word (floor(u64 * n / 2^64))
__device__ __forceinline__ uint64_t uniform_index64(uint32_t hi, uint32_t lo, uint64_t n) {
  return __umul64hi((uint64_t(hi) << 32) | lo, n);
}
// double in (0, 1) from two 32-bit words: (floor(u64 / 2^11) + 0.5) * 2^-53
__device__ __forceinline__ double u01_open(uint32_t hi, uint32_t lo) {
  const uint64_t u = ((uint64_t(hi) << 32) | lo) >> 11;
  return (double(u) + 0.5) * 0x1p-53;
}

// ---------------------------------------------------------------- FP64 math
// Natural log for finite positive normal doubles.  Method: x = m * 2^e with
// m in [sqrt(1/2), sqrt(2)); log(m) = 2*atanh(s), s = (m-1)/(m+1), summed as
// the odd power series of atanh (|s| <= 0.1716, 11 terms reach 2^-53).
// Reference: J.-M. Muller, "Elementary Functions", ch. 5 (series methods).
__device__ __forceinline__ double pg_log(double x) {
  int64_t bits = __double_as_longlong(x);
  int e = int((bits >> 52) & 0x7ff) - 1022;               // x = m * 2^e, m in [0.5, 1)
  double m = __longlong_as_double((bits & 0x000fffffffffffffLL) | 0x3fe0000000000000LL);
  if (m < 0.70710678118654752440) { m = m * 2.0; e = e - 1; }
  const double f = m - 1.0;
  const double s = f / (2.0 + f);
  const double s2 = s * s;
  double p = 1.0 / 23.0;
  p = fma(p, s2, 1.0 / 21.0); p = fma(p, s2, 1.0 / 19.0); p = fma(p, s2, 1.0 / 17.0);
  p = fma(p, s2, 1.0 / 15.0); p = fma(p, s2, 1.0 / 13.0); p = fma(p, s2, 1.0 / 11.0);
  p = fma(p, s2, 1.0 / 9.0);  p = fma(p, s2, 1.0 / 7.0);  p = fma(p, s2, 1.0 / 5.0);
  p = fma(p, s2, 1.0 / 3.0);
  const double logm = fma(2.0 * s * s2, p, 2.0 * s);
  const double de = double(e);
  // ln2 split (Cody-Waite): hi has 32 trailing zero bits so de*hi is exact
  return fma(de, 6.93147180369123816490e-01, fma(de, 1.90821492927058770002e-10, logm));
}

// exp for x in [-700, 700]. Method: x = k*ln2 + r, |r| <= ln2/2 (Cody-Waite
// reduction), exp(r) by its Taylor polynomial to degree 13, scaled by 2^k.
__device__ __forceinline__ double pg_exp(double x) {
  const double kd = floor(x * 1.44269504088896338700 + 0.5);
  double r = fma(-kd, 6.93147180369123816490e-01, x);
  r = fma(-kd, 1.90821492927058770002e-10, r);
  double p = 1.0 / 6227020800.0;                              // 1/13!
  p = fma(p, r, 1.0 / 479001600.0); p = fma(p, r, 1.0 / 39916800.0);
  p = fma(p, r, 1.0 / 3628800.0);   p = fma(p, r, 1.0 / 362880.0);
  p = fma(p, r, 1.0 / 40320.0);     p = fma(p, r, 1.0 / 5040.0);
  p = fma(p, r, 1.0 / 720.0);       p = fma(p, r, 1.0 / 120.0);
  p = fma(p, r, 1.0 / 24.0);        p = fma(p, r, 1.0 / 6.0);
  p = fma(p, r, 0.5);               p = fma(p, r, 1.0);
  p = fma(p, r, 1.0);
  const int k = int(kd);
  const double scale = __longlong_as_double(int64_t(k + 1023) << 52);
  return p * scale;
}

__device__ __forceinline__ double pg_factorial_small(int k) {   // k <= 20, exact in double
  double f = 1.0;
  for (int i = 2; i <= k; ++i) f = f * double(i);
  return f;
}

// log(k!) : exact factorial's log for k < 10, Stirling series for k >= 10
// (error of the truncated series below 1e-13 there).
__device__ __forceinline__ double pg_log_factorial(double k) {
  if (k < 10.0) return pg_log(pg_factorial_small(int(k)));
  const double x = k + 1.0;
  const double ix = 1.0 / x, ix2 = ix * ix;
  double series = -1.0 / 1680.0;
  series = fma(series, ix2, 1.0 / 1260.0);
  series = fma(series, ix2, -1.0 / 360.0);
  series = fma(series, ix2, 1.0 / 12.0);
  return (x - 0.5) * pg_log(x) - x + 0.91893853320467274178 + series * ix;
}

// Stirling-series tail log(k!) - [(k+1/2) log(k+1) - (k+1) + log(2 pi)/2],
// used by the binomial sampler (Hormann 1993, BTRS).
__device__ __forceinline__ double pg_stirling_tail(double k) {
  if (k <= 9.0) {
    return pg_log(pg_factorial_small(int(k))) -
           ((k + 0.5) * pg_log(k + 1.0) - (k + 1.0) + 0.91893853320467274178);
  }
  const double kp1 = k + 1.0;
  const double kp1sq = kp1 * kp1;
  return (1.0 / 12.0 - (1.0 / 360.0 - 1.0 / 1260.0 / kp1sq) / kp1sq) / kp1;
}

// ---------------------------------------------------------------- samplers
// A draw source: successive Philox blocks for one (key, c0..c2, tag) object;
// block j uses counter word c2' = c2 + (j << 20) ... kept simple: block index in
// the upper byte of the tag word.
struct Stream {
  Key key; uint32_t c0, c1, c2, tag; uint32_t block;
  __device__ __forceinline__ U4 next() {
    U4 r = philox(key.k0, key.k1, c0, c1, c2, tag | (block << 8));
    ++block;
    return r;
  }
};

// Poisson(lambda).  lambda < 10: sequential inversion (one uniform).
// lambda >= 10: PTRS, transformed rejection with squeeze (W. Hormann, "The
// transformed rejection method for generating Poisson random variables",
// Insurance: Mathematics and Economics 12, 1993).  Each attempt consumes one
// Philox block (U from words x,y; V from z,w).  At most 64 attempts; the
// acceptance rate is above 0.9, so the cap is never reached in practice, and
// the fallback (the mode) is documented.
__device__ __forceinline__ uint64_t poisson(Stream& st, double lambda) {
  if (!(lambda > 0.0)) return 0;
  if (lambda < 10.0) {
    const U4 r = st.next();
    const double u = u01_open(r.x, r.y);
    double p = pg_exp(-lambda);
    double F = p;
    uint64_t k = 0;
    while (u > F && k < 200) { k = k + 1; p = p * lambda / double(k); F = F + p; }
    return k;
  }
  const double slam = sqrt(lambda);
  const double loglam = pg_log(lambda);
  const double b = 0.931 + 2.53 * slam;
  const double a = -0.059 + 0.02483 * b;
  const double invalpha = 1.1239 + 1.1328 / (b - 3.4);
  const double vr = 0.9277 - 3.6224 / (b - 2.0);
  for (int it = 0; it < 64; ++it) {
    const U4 r = st.next();
    const double U = u01_open(r.x, r.y) - 0.5;
    const double V = u01_open(r.z, r.w);
    const double us = 0.5 - fabs(U);
    const double kd = floor((2.0 * a / us + b) * U + lambda + 0.43);
    if (us >= 0.07 && V <= vr) return uint64_t(kd);
    if (kd < 0.0 || (us < 0.013 && V > us)) continue;
    const double lhs = pg_log(V) + pg_log(invalpha) - pg_log(a / (us * us) + b);
    const double rhs = -lambda + kd * loglam - pg_log_factorial(kd);
    if (lhs <= rhs) return uint64_t(kd);
  }
  return uint64_t(floor(lambda));
}

// Binomial(n, p).  n*min(p,1-p) < 10: inversion (BINV, Kachitvichyanukul and
// Schmeiser, CACM 31, 1988).  Otherwise BTRS (Hormann, "The generation of
// binomial random variates", J. Stat. Comput. Simul. 46, 1993).
__device__ __forceinline__ uint64_t binomial(Stream& st, uint64_t n, double p) {
  if (n == 0 || !(p > 0.0)) return 0;
  if (!(p < 1.0)) return n;
  const bool flip = p > 0.5;
  const double pp = flip ? 1.0 - p : p;
  const double q = 1.0 - pp;
  const double nd = double(n);
  uint64_t k;
  if (nd * pp < 10.0) {
    const U4 r = st.next();
    double u = u01_open(r.x, r.y);
    const double s = pp / q;
    const double aa = (nd + 1.0) * s;
    double rr = pg_exp(nd * pg_log(q));
    k = 0;
    // rr > 0: once the pmf underflows the remaining mass is below rounding
    while (u > rr && k < n && rr > 0.0) { u = u - rr; k = k + 1; rr = rr * (aa / double(k) - s); }
  } else {
    const double spq = sqrt(nd * pp * q);
    const double b = 1.15 + 2.53 * spq;
    const double a = -0.0873 + 0.0248 * b + 0.01 * pp;
    const double c = nd * pp + 0.5;
    const double vr = 0.92 - 4.2 / b;
    const double alpha = (2.83 + 5.1 / b) * spq;
    const double lpq = pg_log(pp / q);
    const double m = floor((nd + 1.0) * pp);
    const double h = pg_stirling_tail(m) + pg_stirling_tail(nd - m);
    k = uint64_t(floor(c));  // fallback: about the mean
    for (int it = 0; it < 64; ++it) {
      const U4 r = st.next();
      const double U = u01_open(r.x, r.y) - 0.5;
      double V = u01_open(r.z, r.w);
      const double us = 0.5 - fabs(U);
      const double kd = floor((2.0 * a / us + b) * U + c);
      if (kd < 0.0 || kd > nd) continue;
      if (us >= 0.07 && V <= vr) { k = uint64_t(kd); break; }
      V = pg_log(V * alpha / (a / (us * us) + b));
      const double ub = (m + 0.5) * pg_log((m + 1.0) / (nd - m + 1.0)) +
                        (nd + 1.0) * pg_log((nd - m + 1.0) / (nd - kd + 1.0)) +
                        (kd + 0.5) * pg_log((nd - kd + 1.0) / (kd + 1.0)) +
                        (kd - m) * lpq + h - pg_stirling_tail(kd) - pg_stirling_tail(nd - kd);
      if (V <= ub) { k = uint64_t(kd); break; }
    }
  }
  return flip ? n - k : k;
}

// The first attempt of binomial(st, n, p) alone: true, with k its result,
// when binomial decides within that attempt without BTRS's exact test (the
// trivial cases and the squeeze); false when it needs more (BINV, or an
// attempt past the squeeze).  The expressions are binomial's, in its order,
// so a true answer equals binomial's result; Stream is taken by value.
__device__ __forceinline__ bool binomial_first(Stream st, uint64_t n, double p, uint64_t& k) {
  if (n == 0 || !(p > 0.0)) { k = 0; return true; }
  if (!(p < 1.0)) { k = n; return true; }
  const bool flip = p > 0.5;
  const double pp = flip ? 1.0 - p : p;
  const double q = 1.0 - pp;
  const double nd = double(n);
  if (nd * pp < 10.0) return false;
  const double spq = sqrt(nd * pp * q);
  const double b = 1.15 + 2.53 * spq;
  const double a = -0.0873 + 0.0248 * b + 0.01 * pp;
  const double c = nd * pp + 0.5;
  const double vr = 0.92 - 4.2 / b;
  const U4 r = st.next();
  const double U = u01_open(r.x, r.y) - 0.5;
  const double V = u01_open(r.z, r.w);
  const double us = 0.5 - fabs(U);
  const double kd = floor((2.0 * a / us + b) * U + c);
  if (kd < 0.0 || kd > nd) return false;
  if (!(us >= 0.07 && V <= vr)) return false;
  k = flip ? n - uint64_t(kd) : uint64_t(kd);
  return true;
}

// Inverse-CDF lookup with integer thresholds: thr[k] = floor(CDF(k) * 2^31)
// (the last class with positive mass holds 2^31); returns the first k with
// thr[k] > u/2, so zero-mass classes are never returned.
__device__ __forceinline__ uint32_t cdf_lookup(const uint32_t* thr, uint32_t n, uint32_t u) {
  const uint32_t v = u >> 1;
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (thr[mid] <= v) lo = mid + 1; else hi = mid;
  }
  return lo < n ? lo : n - 1;
}

}  // namespace pg
