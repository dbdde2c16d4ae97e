// ORACLE — test infrastructure only.  Nothing in the product links, imports or
// executes this file; tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline / reference arm load it as a checker.
//
// A plain sequential CPU restatement of the path ProCESS hands to RACES:
//   MutationEngine::place_mutations   src/mutation_engine.cpp:1085-1113 (call :1097-1101)
//   simulate_seq -> ReadSimulator     src/seq_simulation.cpp:517-601 (call :371,:413,:423)
//   ContextIndex / RSIndex builds     src/mutation_engine.cpp:211-275, 289-359
//   insert-size model get_bin_dist    src/seq_simulation.cpp:431-451
// The arithmetic lives in RACES (albertocasagrande/RACES @ 1142937,
// configure:9-13), which is absent here and cannot be fetched; the reference
// ships no tests or golden vectors for this path (its vignettes disclaim
// cross-compiler reproducibility, vignettes/sequencing.Rmd:27-34).
// PARITY UNPINNED: this restatement follows ProCESS's call sites and data
// contracts plus the documented model; it is not checked against RACES output.
//
// Two flavours:
//   flavour 0  "replay": the same counter-based Philox4x32-10 draws as the GPU
//              kernels, with the index, placement and read loops written
//              sequentially (explicit position lists, parent-walk ancestry
//              tests, a plain per-read loop) -> bit-exact comparison.
//   flavour 1  "reference engine": std::mt19937_64 (the engine type of
//              src/mutation_engine.hpp:50) with std::poisson_distribution,
//              std::discrete_distribution, std::uniform_int_distribution and
//              std::binomial_distribution (the reference's own insert-size
//              distribution, src/seq_simulation.cpp:431-451) drawn in
//              sequence -> distributional comparison and the CPU baseline.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <functional>
#include <map>
#include <memory>
#include <random>
#include <set>
#include <stdexcept>
#include <string>
#include <thread>
#include <unordered_set>
#include <unordered_map>
#include <vector>

namespace orc {

// ------------------------------------------------------------ Philox4x32-10
struct W4 { uint32_t v[4]; };

static inline uint32_t mulhi32(uint32_t a, uint32_t b) { return uint32_t((uint64_t(a) * b) >> 32); }

W4 philox(uint32_t k0, uint32_t k1, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3) {
  for (int round = 0; round < 10; ++round) {
    const uint64_t p0 = uint64_t(0xD2511F53u) * c0;
    const uint64_t p1 = uint64_t(0xCD9E8D57u) * c2;
    const uint32_t x0 = uint32_t(p1 >> 32) ^ c1 ^ k0;
    const uint32_t x1 = uint32_t(p1);
    const uint32_t x2 = uint32_t(p0 >> 32) ^ c3 ^ k1;
    const uint32_t x3 = uint32_t(p0);
    c0 = x0; c1 = x1; c2 = x2; c3 = x3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return {{c0, c1, c2, c3}};
}

enum : uint32_t {
  TAG_EDGE_SNV = 1, TAG_EDGE_INDEL = 2, TAG_EDGE_CNA = 3, TAG_SNV = 4, TAG_INDEL = 5, TAG_DRIVER = 6,
  TAG_TILE_SPLIT = 7, TAG_PAIR = 8, TAG_GENOME = 11, TAG_CNA = 12
};

static inline uint64_t index64(uint32_t hi, uint32_t lo, uint64_t n) {
  const unsigned __int128 u = (unsigned __int128)((uint64_t(hi) << 32) | lo) * n;
  return uint64_t(u >> 64);
}
static inline double open01(uint32_t hi, uint32_t lo) {
  const uint64_t u = ((uint64_t(hi) << 32) | lo) >> 11;
  return (double(u) + 0.5) * 0x1p-53;
}

// ------------------------------------------------------------ FP64 math
// log via the atanh series of s = (m-1)/(m+1), m in [sqrt(1/2), sqrt(2))
double my_log(double x) {
  int64_t bits;
  std::memcpy(&bits, &x, 8);
  int e = int((bits >> 52) & 0x7ff) - 1022;
  int64_t mb = (bits & 0x000fffffffffffffLL) | 0x3fe0000000000000LL;
  double m;
  std::memcpy(&m, &mb, 8);
  if (m < 0.70710678118654752440) { m = m * 2.0; e = e - 1; }
  const double f = m - 1.0;
  const double s = f / (2.0 + f);
  const double s2 = s * s;
  double p = 1.0 / 23.0;
  const double inv[10] = {1.0 / 21.0, 1.0 / 19.0, 1.0 / 17.0, 1.0 / 15.0, 1.0 / 13.0,
                          1.0 / 11.0, 1.0 / 9.0, 1.0 / 7.0, 1.0 / 5.0, 1.0 / 3.0};
  for (double c : inv) p = std::fma(p, s2, c);
  const double logm = std::fma(2.0 * s * s2, p, 2.0 * s);
  const double de = double(e);
  return std::fma(de, 6.93147180369123816490e-01, std::fma(de, 1.90821492927058770002e-10, logm));
}

// exp by Cody-Waite reduction and the degree-13 Taylor polynomial
double my_exp(double x) {
  const double kd = std::floor(x * 1.44269504088896338700 + 0.5);
  double r = std::fma(-kd, 6.93147180369123816490e-01, x);
  r = std::fma(-kd, 1.90821492927058770002e-10, r);
  const double c[14] = {1.0 / 6227020800.0, 1.0 / 479001600.0, 1.0 / 39916800.0, 1.0 / 3628800.0,
                        1.0 / 362880.0, 1.0 / 40320.0, 1.0 / 5040.0, 1.0 / 720.0, 1.0 / 120.0,
                        1.0 / 24.0, 1.0 / 6.0, 0.5, 1.0, 1.0};
  double p = c[0];
  for (int i = 1; i < 14; ++i) p = std::fma(p, r, c[i]);
  const int k = int(kd);
  const int64_t sb = int64_t(k + 1023) << 52;
  double scale;
  std::memcpy(&scale, &sb, 8);
  return p * scale;
}

double fact_small(int k) { double f = 1.0; for (int i = 2; i <= k; ++i) f = f * double(i); return f; }

double log_factorial(double k) {
  if (k < 10.0) return my_log(fact_small(int(k)));
  const double x = k + 1.0;
  const double ix = 1.0 / x, ix2 = ix * ix;
  double series = -1.0 / 1680.0;
  series = std::fma(series, ix2, 1.0 / 1260.0);
  series = std::fma(series, ix2, -1.0 / 360.0);
  series = std::fma(series, ix2, 1.0 / 12.0);
  return (x - 0.5) * my_log(x) - x + 0.91893853320467274178 + series * ix;
}

double stirling_tail(double k) {
  if (k <= 9.0) {
    return my_log(fact_small(int(k))) - ((k + 0.5) * my_log(k + 1.0) - (k + 1.0) + 0.91893853320467274178);
  }
  const double kp1 = k + 1.0;
  const double kp1sq = kp1 * kp1;
  return (1.0 / 12.0 - (1.0 / 360.0 - 1.0 / 1260.0 / kp1sq) / kp1sq) / kp1;
}

struct Stream {
  uint32_t k0, k1, c0, c1, c2, tag, block;
  W4 next() { W4 r = philox(k0, k1, c0, c1, c2, tag | (block << 8)); ++block; return r; }
};
static Stream stream(uint64_t seed, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t tag) {
  return {uint32_t(seed), uint32_t(seed >> 32), c0, c1, c2, tag, 0};
}

// Poisson: inversion below 10, PTRS (Hormann 1993) above
uint64_t poisson(Stream& st, double lambda) {
  if (!(lambda > 0.0)) return 0;
  if (lambda < 10.0) {
    const W4 r = st.next();
    const double u = open01(r.v[0], r.v[1]);
    double p = my_exp(-lambda), F = p;
    uint64_t k = 0;
    while (u > F && k < 200) { k = k + 1; p = p * lambda / double(k); F = F + p; }
    return k;
  }
  const double slam = std::sqrt(lambda), loglam = my_log(lambda);
  const double b = 0.931 + 2.53 * slam;
  const double a = -0.059 + 0.02483 * b;
  const double invalpha = 1.1239 + 1.1328 / (b - 3.4);
  const double vr = 0.9277 - 3.6224 / (b - 2.0);
  for (int it = 0; it < 64; ++it) {
    const W4 r = st.next();
    const double U = open01(r.v[0], r.v[1]) - 0.5;
    const double V = open01(r.v[2], r.v[3]);
    const double us = 0.5 - std::fabs(U);
    const double kd = std::floor((2.0 * a / us + b) * U + lambda + 0.43);
    if (us >= 0.07 && V <= vr) return uint64_t(kd);
    if (kd < 0.0 || (us < 0.013 && V > us)) continue;
    const double lhs = my_log(V) + my_log(invalpha) - my_log(a / (us * us) + b);
    const double rhs = -lambda + kd * loglam - log_factorial(kd);
    if (lhs <= rhs) return uint64_t(kd);
  }
  return uint64_t(std::floor(lambda));
}

// Binomial: BINV below n*p = 10, BTRS (Hormann 1993) above
uint64_t binomial(Stream& st, uint64_t n, double p) {
  if (n == 0 || !(p > 0.0)) return 0;
  if (!(p < 1.0)) return n;
  const bool flip = p > 0.5;
  const double pp = flip ? 1.0 - p : p;
  const double q = 1.0 - pp;
  const double nd = double(n);
  uint64_t k;
  if (nd * pp < 10.0) {
    const W4 r = st.next();
    double u = open01(r.v[0], r.v[1]);
    const double s = pp / q;
    const double aa = (nd + 1.0) * s;
    double rr = my_exp(nd * my_log(q));
    k = 0;
    while (u > rr && k < n && rr > 0.0) { u = u - rr; k = k + 1; rr = rr * (aa / double(k) - s); }
  } else {
    const double spq = std::sqrt(nd * pp * q);
    const double b = 1.15 + 2.53 * spq;
    const double a = -0.0873 + 0.0248 * b + 0.01 * pp;
    const double c = nd * pp + 0.5;
    const double vr = 0.92 - 4.2 / b;
    const double alpha = (2.83 + 5.1 / b) * spq;
    const double lpq = my_log(pp / q);
    const double m = std::floor((nd + 1.0) * pp);
    const double h = stirling_tail(m) + stirling_tail(nd - m);
    k = uint64_t(std::floor(c));
    for (int it = 0; it < 64; ++it) {
      const W4 r = st.next();
      const double U = open01(r.v[0], r.v[1]) - 0.5;
      double V = open01(r.v[2], r.v[3]);
      const double us = 0.5 - std::fabs(U);
      const double kd = std::floor((2.0 * a / us + b) * U + c);
      if (kd < 0.0 || kd > nd) continue;
      if (us >= 0.07 && V <= vr) { k = uint64_t(kd); break; }
      V = my_log(V * alpha / (a / (us * us) + b));
      const double ub = (m + 0.5) * my_log((m + 1.0) / (nd - m + 1.0)) +
                        (nd + 1.0) * my_log((nd - m + 1.0) / (nd - kd + 1.0)) +
                        (kd + 0.5) * my_log((nd - kd + 1.0) / (kd + 1.0)) +
                        (kd - m) * lpq + h - stirling_tail(kd) - stirling_tail(nd - kd);
      if (V <= ub) { k = uint64_t(kd); break; }
    }
  }
  return flip ? n - k : k;
}

// thresholds floor(CDF * 2^31), last positive-mass class 2^31
std::vector<uint32_t> thresholds(const std::vector<double>& w) {
  std::vector<uint32_t> thr(w.size(), 0);
  double tot = 0;
  for (double x : w) tot += x;
  if (!(tot > 0)) return thr;
  size_t last = 0;
  for (size_t i = 0; i < w.size(); ++i) if (w[i] > 0) last = i;
  double c = 0;
  for (size_t i = 0; i < w.size(); ++i) {
    c += w[i];
    double t = std::floor(c / tot * 2147483648.0);
    if (t > 2147483648.0) t = 2147483648.0;
    thr[i] = (i >= last) ? 2147483648u : uint32_t(t);
  }
  return thr;
}
uint32_t lookup(const uint32_t* thr, uint32_t n, uint32_t u) {
  const uint32_t v = u >> 1;
  for (uint32_t k = 0; k < n; ++k) if (thr[k] > v) return k;   // linear scan: same answer as a bisection
  return n - 1;
}

// ------------------------------------------------------------ genome and classes
int context_of(int x, int y, int z) {
  if (y == 1 || y == 3) return (y == 3 ? 16 : 0) + x * 4 + z;
  const int cy = 3 - y, cx = 3 - z, cz = 3 - x;
  return (cy == 3 ? 16 : 0) + cx * 4 + cz;
}
int sbs_ctx(int cls) { return (cls >= 48 ? 16 : 0) + (cls & 15); }
int sbs_alt(int cls) { const int a[6] = {0, 2, 3, 0, 1, 2}; return a[cls >> 4]; }

struct Genome {
  std::vector<uint8_t> b;            // codes
  std::vector<uint32_t> off;         // n_chr + 1
  uint32_t chr_of(uint32_t p) const {
    return uint32_t(std::upper_bound(off.begin(), off.end(), p) - off.begin()) - 1;
  }
};

// ID83 classes of position p (see the product's index for the table)
void id_classes(const Genome& g, uint32_t p, int out[16]) {
  for (int f = 0; f < 16; ++f) out[f] = -1;
  const uint32_t c = g.chr_of(p);
  const uint32_t cs = g.off[c], ce = g.off[c + 1];
  if (p <= cs || p >= ce) return;
  auto get = [&](int64_t q) -> int { return (q >= int64_t(cs) && q < int64_t(ce)) ? g.b[q] : 4; };
  const int b = get(p), prev = get(int64_t(p) - 1);
  if (b == 4 || prev == 4) return;     // the site or its anchor is unknown (N)
  int h = 1;
  while (h < 6 && get(int64_t(p) + h) == b) ++h;
  const bool runstart = prev != b;
  const bool pyrT = (b == 3 || b == 0);
  if (runstart) {
    out[0] = (pyrT ? 6 : 0) + h - 1;
    out[1] = 12 + (pyrT ? 6 : 0) + std::min(h, 5);
    for (int l = 2; l <= 5; ++l) out[12 + l - 2] = 48 + (l - 2) * 6;
  }
  if (b != 1 && b != 2 && prev != 1 && prev != 2) out[2] = 12;
  if (b != 0 && b != 3 && prev != 0 && prev != 3) out[3] = 18;
  const int mh_off[4] = {0, 1, 3, 6};
  for (int l = 2; l <= 5; ++l) {
    bool valid = true;
    for (int i = 0; i < l; ++i) valid = valid && get(int64_t(p) + i) != 4;
    if (!valid) continue;
    if (int64_t(p) >= int64_t(cs) + l) {
      bool same = true;
      for (int i = 0; i < l; ++i) same = same && get(int64_t(p) - l + i) == get(int64_t(p) + i);
      if (same) continue;
    }
    int r = 1;
    while (r < 6) {
      bool same = true;
      for (int i = 0; i < l; ++i) same = same && get(int64_t(p) + r * l + i) == get(int64_t(p) + i);
      if (!same) break;
      ++r;
    }
    if (r >= 2) {
      out[4 + l - 2] = 24 + (l - 2) * 6 + std::min(r - 1, 5);
    } else {
      int m = 0;
      while (m < l && get(int64_t(p) + l + m) == get(int64_t(p) + m)) ++m;
      out[4 + l - 2] = (m == 0) ? 24 + (l - 2) * 6 : 72 + mh_off[l - 2] + m - 1;
    }
    out[8 + l - 2] = 48 + (l - 2) * 6 + std::min(r, 5);
  }
}

// ------------------------------------------------------------ engine
struct Species { double snv = 0, indel = 0, cna = 0; std::vector<double> snv_e, indel_e; uint32_t mutant = 0; bool has = false; };
struct Driver { uint32_t chr, pos; std::string ref, alt; int32_t allele; };
struct Cna { bool amp; uint32_t chr, begin, len; int32_t allele, src; };   // 1-based begin
struct DriverEvent { int kind; Driver sid; Cna cna; };                      // 0 SID, 1 CNA, 2 WGD

struct Engine {
  Genome g;
  uint32_t context_sampling = 100, max_rep = 500000;
  std::vector<std::vector<uint32_t>> ctx, id;     // stored position lists
  std::vector<uint64_t> ctx_total, id_total;
  uint32_t n_sig[2] = {0, 0};
  std::vector<double> sigs[2];
  std::map<double, std::vector<double>> expo[2];
  std::map<uint32_t, Species> species;
  std::map<uint32_t, std::vector<DriverEvent>> drivers;
  std::vector<Cna> cands;                 // passenger CNA candidates
  bool infinite_sites = true;
  bool avoid_losses = true;
  std::vector<uint8_t> avoid;             // positions the SBS context index leaves out (empty: none)
};

// ContextIndex::build_index(ref, regions_to_avoid, sampling) and
// RSIndex::build_index (src/mutation_engine.cpp:260, 344): every position
// with its trinucleotide context (not inside a region to avoid) and its ID
// classes, then 1 in `context_sampling` / enough to keep at most max_rep per
// class, in position order
void build_index(Engine& e) {
  const uint64_t G = e.g.b.size();
  std::vector<std::vector<uint32_t>> all_ctx(32), all_id(83);
  for (uint64_t p = 0; p < G; ++p) {
    const uint32_t c = e.g.chr_of(uint32_t(p));
    const uint32_t cs = e.g.off[c], ce = e.g.off[c + 1];
    // a context with an unknown base (code 4, N) is not indexed
    const bool avoided = !e.avoid.empty() && e.avoid[p];
    if (!avoided && p > cs && p + 1 < ce && e.g.b[p - 1] < 4 && e.g.b[p] < 4 && e.g.b[p + 1] < 4)
      all_ctx[context_of(e.g.b[p - 1], e.g.b[p], e.g.b[p + 1])].push_back(uint32_t(p));
    int cl[16];
    id_classes(e.g, uint32_t(p), cl);
    for (int f = 0; f < 16; ++f) if (cl[f] >= 0) all_id[cl[f]].push_back(uint32_t(p));
  }
  e.ctx.assign(32, {}); e.id.assign(83, {});
  e.ctx_total.assign(32, 0); e.id_total.assign(83, 0);
  for (int k = 0; k < 32; ++k) {
    e.ctx_total[k] = all_ctx[k].size();
    for (size_t r = 0; r < all_ctx[k].size(); r += e.context_sampling) e.ctx[k].push_back(all_ctx[k][r]);
  }
  for (int k = 0; k < 83; ++k) {
    e.id_total[k] = all_id[k].size();
    const uint64_t sd = std::max<uint64_t>(1, (all_id[k].size() + e.max_rep - 1) / e.max_rep);
    for (size_t r = 0; r < all_id[k].size(); r += sd) e.id[k].push_back(all_id[k][r]);
  }
}

struct Forest {
  uint32_t n, n_samples;
  std::vector<int32_t> parent, sample;
  std::vector<double> birth;
  std::vector<uint32_t> species, divisions;
  std::vector<std::vector<uint32_t>> leaves;    // per sample, node ids in increasing order
  std::vector<uint8_t> is_leaf;
};

// ---- copy-number state.  A cell's genome maps every allele instance it
// holds to the sorted, disjoint intervals [b, e) (absolute positions) the
// instance still covers.  Instances 0 and 1 are the germline alleles; every
// amplification or WGD copy creates the next instance id, in the order the
// events are applied (nodes in index order, each node's events in order).
using Ivl = std::vector<std::pair<uint32_t, uint32_t>>;
using CellGenome = std::map<uint32_t, Ivl>;

bool ivl_has(const Ivl& v, uint32_t p) {
  auto it = std::upper_bound(v.begin(), v.end(), std::make_pair(p, 0xffffffffu));
  return it != v.begin() && std::prev(it)->first <= p && p < std::prev(it)->second;
}
Ivl ivl_minus(const Ivl& v, uint32_t b, uint32_t e) {
  Ivl out;
  for (auto [x, y] : v) {
    if (y <= b || x >= e) { out.push_back({x, y}); continue; }
    if (x < b) out.push_back({x, b});
    if (y > e) out.push_back({e, y});
  }
  return out;
}
Ivl ivl_within(const Ivl& v, uint32_t b, uint32_t e) {
  Ivl out;
  for (auto [x, y] : v) if (y > b && x < e) out.push_back({std::max(x, b), std::min(y, e)});
  return out;
}
// instances covering p, ascending
std::vector<uint32_t> covering(const CellGenome& g, uint32_t p) {
  std::vector<uint32_t> out;
  for (const auto& [inst, v] : g) if (ivl_has(v, p)) out.push_back(inst);
  return out;
}
uint64_t genome_size(const CellGenome& g) {
  uint64_t n = 0;
  for (const auto& kv : g) for (auto [x, y] : kv.second) n += y - x;
  return n;
}
// largest number of instances covering one position
uint32_t max_copies(const CellGenome& g) {
  std::vector<std::pair<uint32_t, int>> ev;
  for (const auto& kv : g) for (auto [x, y] : kv.second) { ev.push_back({x, 1}); ev.push_back({y, -1}); }
  std::sort(ev.begin(), ev.end());   // at equal positions ends (-1) come first
  int cur = 0, best = 0;
  for (auto [p, d] : ev) { cur += d; best = std::max(best, cur); }
  return uint32_t(best);
}

// Positions of a genome grouped into maximal runs covered by the same
// (ascending) instance list, for O(log) lookups
struct ClassIndex {
  std::vector<uint32_t> b, e;
  std::vector<std::vector<uint32_t>> insts;
};
ClassIndex class_index(const CellGenome& g) {
  std::vector<uint32_t> cuts;
  for (const auto& kv : g) for (auto [x, y] : kv.second) { cuts.push_back(x); cuts.push_back(y); }
  std::sort(cuts.begin(), cuts.end());
  cuts.erase(std::unique(cuts.begin(), cuts.end()), cuts.end());
  ClassIndex ix;
  for (size_t i = 0; i + 1 < cuts.size(); ++i) {
    auto cov = covering(g, cuts[i]);
    if (cov.empty()) continue;
    if (!ix.b.empty() && ix.e.back() == cuts[i] && ix.insts.back() == cov) { ix.e.back() = cuts[i + 1]; continue; }
    ix.b.push_back(cuts[i]); ix.e.push_back(cuts[i + 1]); ix.insts.push_back(std::move(cov));
  }
  return ix;
}
const std::vector<uint32_t>& covering(const ClassIndex& ix, uint32_t p) {
  static const std::vector<uint32_t> none;
  auto it = std::upper_bound(ix.b.begin(), ix.b.end(), p);
  if (it == ix.b.begin()) return none;
  const size_t i = size_t(it - ix.b.begin()) - 1;
  return p < ix.e[i] ? ix.insts[i] : none;
}

struct Placed;
void build_atoms(Placed& pl, uint32_t G);

// a copy made on edge `edge` by its event `event` (instance `made` from `from`)
struct CopyRec { uint32_t edge, event, made, from; };

struct CnaRec { uint32_t node; uint8_t type; uint32_t chr, begin, end, allele, src; uint8_t driver; };

struct Placed {
  std::vector<uint32_t> locus, edge, aux;
  std::vector<uint8_t> cls, sig, kind, nature;
  std::vector<uint16_t> allele;
  std::vector<int32_t> order;      // position among the edge's events: driver index, -1 preneoplastic,
                                   // INT32_MAX passengers (after every event of the edge)
  const Forest* forest = nullptr;
  const Engine* eng = nullptr;
  Forest forest_copy;
  std::vector<CellGenome> classes{1};   // genotype classes, class 0 = germline
  std::vector<ClassIndex> index;        // per class
  // atoms: the coarsest partition of the genome into intervals on which
  // every class's covering instances are constant, with those instances
  std::vector<uint32_t> atom_start;
  std::vector<std::vector<std::vector<uint32_t>>> atom_cov;   // [atom][class]
  std::vector<uint32_t> node_class;     // per node (+ the preneoplastic edge: class 0)
  std::vector<CopyRec> copies;
  std::vector<CnaRec> cnas;
  uint32_t n_inst = 2, cn_max = 2;
  bool has_cna = false;
};

void build_atoms(Placed& pl, uint32_t G) {
  std::vector<uint32_t> cuts{0u, G};
  for (const auto& g : pl.classes)
    for (const auto& kv : g) for (auto [x, y] : kv.second) { cuts.push_back(x); cuts.push_back(y); }
  std::sort(cuts.begin(), cuts.end());
  cuts.erase(std::unique(cuts.begin(), cuts.end()), cuts.end());
  pl.atom_start.clear(); pl.atom_cov.clear();
  for (size_t i = 0; i + 1 < cuts.size(); ++i) {
    std::vector<std::vector<uint32_t>> tuple;
    for (const auto& ix : pl.index) tuple.push_back(covering(ix, cuts[i]));
    if (!pl.atom_cov.empty() && pl.atom_cov.back() == tuple) continue;
    pl.atom_start.push_back(cuts[i]);
    pl.atom_cov.push_back(std::move(tuple));
  }
}

struct Tables {
  std::vector<double> times;
  uint32_t E = 1, S = 0;
  std::vector<double> snv_rate, id_rate;
  std::vector<std::vector<double>> sig_w[2];       // masked class weights per signature
  std::vector<std::vector<double>> expo_w[2];      // rows 0..E-1, row E preneoplastic
  std::vector<uint32_t> sig_cdf[2], expo_cdf[2];
  uint32_t ns[2] = {1, 1};
};

Tables make_tables(const Engine& e, const Forest& f, uint32_t n_pre_snv, uint32_t pre_sbs, uint32_t n_pre_id,
                   uint32_t pre_id) {
  Tables t;
  for (int ty = 0; ty < 2; ++ty) for (auto& kv : e.expo[ty]) t.times.push_back(kv.first);
  std::sort(t.times.begin(), t.times.end());
  t.times.erase(std::unique(t.times.begin(), t.times.end()), t.times.end());
  if (t.times.empty()) t.times.push_back(0.0);
  t.E = uint32_t(t.times.size());
  for (uint32_t v = 0; v < f.n; ++v) t.S = std::max(t.S, f.species[v] + 1);
  t.snv_rate.assign(uint64_t(t.S) * t.E, 0.0);
  t.id_rate.assign(uint64_t(t.S) * t.E, 0.0);
  for (uint32_t s = 0; s < t.S; ++s) {
    auto it = e.species.find(s);
    if (it == e.species.end()) continue;
    for (uint32_t ep = 0; ep < t.E; ++ep) {
      double rs = it->second.snv, ri = it->second.indel;
      if (!it->second.snv_e.empty()) { rs = it->second.snv_e[ep]; ri = it->second.indel_e[ep]; }
      t.snv_rate[uint64_t(s) * t.E + ep] = rs;
      t.id_rate[uint64_t(s) * t.E + ep] = ri;
    }
  }
  for (int ty = 0; ty < 2; ++ty) {
    const uint32_t NC = ty == 0 ? 96 : 83;
    t.ns[ty] = std::max<uint32_t>(e.n_sig[ty], 1);
    t.sig_w[ty].assign(t.ns[ty], std::vector<double>(NC, 0.0));
    t.sig_cdf[ty].assign(uint64_t(t.ns[ty]) * NC, 0);
    for (uint32_t s = 0; s < e.n_sig[ty]; ++s) {
      for (uint32_t k = 0; k < NC; ++k) {
        const size_t len = ty == 0 ? e.ctx[sbs_ctx(int(k))].size() : e.id[k].size();
        t.sig_w[ty][s][k] = len > 0 ? e.sigs[ty][uint64_t(s) * NC + k] : 0.0;
      }
      auto thr = thresholds(t.sig_w[ty][s]);
      std::copy(thr.begin(), thr.end(), t.sig_cdf[ty].begin() + uint64_t(s) * NC);
    }
    t.expo_w[ty].assign(t.E + 1, std::vector<double>(t.ns[ty], 0.0));
    t.expo_cdf[ty].assign(uint64_t(t.E + 1) * t.ns[ty], 0);
    for (uint32_t ep = 0; ep < t.E; ++ep) {
      if (!e.expo[ty].empty()) {
        auto it = e.expo[ty].upper_bound(t.times[ep]);
        t.expo_w[ty][ep] = (it == e.expo[ty].begin()) ? it->second : std::prev(it)->second;
      }
      auto thr = thresholds(t.expo_w[ty][ep]);
      std::copy(thr.begin(), thr.end(), t.expo_cdf[ty].begin() + uint64_t(ep) * t.ns[ty]);
    }
    const uint32_t n_pre = ty == 0 ? n_pre_snv : n_pre_id;
    const uint32_t ps = ty == 0 ? pre_sbs : pre_id;
    if (n_pre > 0) {
      t.expo_w[ty][t.E][ps] = 1.0;
      auto thr = thresholds(t.expo_w[ty][t.E]);
      std::copy(thr.begin(), thr.end(), t.expo_cdf[ty].begin() + uint64_t(t.E) * t.ns[ty]);
    }
  }
  return t;
}

uint32_t code(char c) {
  switch (c) { case 'A': return 0; case 'C': return 1; case 'G': return 2; case 'T': return 3; }
  return 0;
}

struct DriverRec { uint32_t locus, edge, aux, allele; int32_t order; uint8_t kind; };

// locus and descriptor of a driver SNV/indel (allele left to the caller)
DriverRec driver_site(const Engine& e, const Driver& d, uint32_t edge) {
  DriverRec r{};
  r.edge = edge;
  r.locus = e.g.off[d.chr] + d.pos - 1;
  if (d.ref.size() == 1 && d.alt.size() == 1) { r.kind = 0; r.aux = code(d.alt[0]); }
  else {
    r.kind = 1;
    if (d.alt.size() > 1) {
      uint32_t bases = 0;
      for (size_t k = 1; k < d.alt.size(); ++k) bases |= code(d.alt[k]) << (2 * (k - 1));
      r.aux = 1u | (uint32_t(d.alt.size() - 1) << 1) | (bases << 8);
    } else {
      r.aux = uint32_t(d.ref.size() - 1) << 1;
    }
  }
  return r;
}

uint32_t mutant_of(const Engine& e, const Forest& f, uint32_t node) {
  auto it = e.species.find(f.species[node]);
  return it == e.species.end() ? 0u : it->second.mutant;
}
// the driver list applied on edge v: the mutant's, on the first edge of its clone
const std::vector<DriverEvent>* drivers_of(const Engine& e, const Forest& f, uint32_t v) {
  const uint32_t m = mutant_of(e, f, v);
  if (f.parent[v] >= 0 && mutant_of(e, f, uint32_t(f.parent[v])) == m) return nullptr;
  auto it = e.drivers.find(m);
  return it == e.drivers.end() ? nullptr : &it->second;
}


// Applies every node's driver list (SNVs/indels, CNAs, WGD in declaration
// order; src/mutation_engine.cpp:789-862, vignettes/mutations.Rmd:159-177)
// and then its passenger CNAs (candidates of src/mutation_engine.cpp:441-487
// at the species' CNA rate; with avoid_homozygous_losses a passenger deletion
// never removes the last allele of a region, :1356) to the genome inherited
// from the parent.  Fills the genotype classes, copies and CNA records of
// `pl` and returns the driver SNVs/indels in node then event order.
// The random choices of the event replay.  PhiloxDraws uses the keyed
// counters of the GPU path; MtDraws draws them in sequence from the
// std::mt19937_64 engine of the reference-engine flavour.
struct PhiloxDraws {
  uint64_t seed;
  uint32_t k0() const { return uint32_t(seed); }
  uint32_t k1() const { return uint32_t(seed >> 32); }
  uint64_t pcna_count(uint32_t v, double lambda) {
    Stream st = stream(seed, 0, v, 0, TAG_EDGE_CNA);
    return poisson(st, lambda);
  }
  uint32_t pcna_cand(uint32_t v, uint32_t k, uint32_t n) { return mulhi32(philox(k0(), k1(), k, v, 0, TAG_CNA).v[0], n); }
  uint32_t pcna_ord(uint32_t v, uint32_t k, uint32_t n) { return mulhi32(philox(k0(), k1(), k, v, 0, TAG_CNA).v[1], n); }
  uint32_t cna_ord(uint32_t v, uint32_t j, uint32_t n) { return mulhi32(philox(k0(), k1(), j, v, 1, TAG_CNA).v[1], n); }
  uint32_t sid_ord(uint32_t idx, uint32_t v, uint32_t n) { return mulhi32(philox(k0(), k1(), idx, v, 0, TAG_DRIVER).v[0], n); }
};
struct MtDraws {
  std::mt19937_64& rng;
  uint64_t pcna_count(uint32_t, double lambda) {
    return lambda > 0 ? std::poisson_distribution<uint64_t>(lambda)(rng) : 0;
  }
  uint32_t pick(uint32_t n) { return std::uniform_int_distribution<uint32_t>(0, n - 1)(rng); }
  uint32_t pcna_cand(uint32_t, uint32_t, uint32_t n) { return pick(n); }
  uint32_t pcna_ord(uint32_t, uint32_t, uint32_t n) { return pick(n); }
  uint32_t cna_ord(uint32_t, uint32_t, uint32_t n) { return pick(n); }
  uint32_t sid_ord(uint32_t, uint32_t, uint32_t n) { return pick(n); }
};

template <class Draws>
std::vector<DriverRec> replay_events(const Engine& e, const Forest& f, Draws& draws, Placed& pl) {
  const uint32_t N = f.n;
  const uint32_t n_chr = uint32_t(e.g.off.size() - 1);
  CellGenome germ;
  for (uint32_t c = 0; c < n_chr; ++c)
    if (e.g.off[c] < e.g.off[c + 1])
      for (uint32_t a = 0; a < 2; ++a) germ[a].push_back({e.g.off[c], e.g.off[c + 1]});
  pl.classes.assign(1, germ);
  pl.node_class.assign(N + 1, 0);
  pl.copies.clear(); pl.cnas.clear();
  uint32_t n_inst = 2, n_sid = 0;
  // passenger CNA counts: Poisson(rate * germline allelic size * divisions)
  std::vector<uint64_t> n_pcna(N, 0);
  if (!e.cands.empty()) {
    const double germline = 2.0 * double(e.g.b.size());
    for (uint32_t v = 0; v < N; ++v) {
      auto it = e.species.find(f.species[v]);
      const double rate = it == e.species.end() ? 0.0 : it->second.cna;
      n_pcna[v] = draws.pcna_count(v, rate * germline * double(f.divisions[v]));
    }
  }
  std::vector<DriverRec> drv;
  for (uint32_t v = 0; v < N; ++v) {
    const uint32_t base = f.parent[v] >= 0 ? pl.node_class[f.parent[v]] : 0u;
    CellGenome g = pl.classes[base];
    bool changed = false;
    const auto* list = drivers_of(e, f, v);
    const uint32_t nd = list ? uint32_t(list->size()) : 0u;
    if (uint64_t(nd) + n_pcna[v] > 0x7ffd) throw std::runtime_error("too many driver and CNA events on one edge");
    // ord(n): ordinal among the n covering instances when the event names none
    auto cna = [&](const Cna& c, uint32_t event, auto ord_of, bool passenger) {
      const uint32_t b = e.g.off[c.chr] + c.begin - 1;
      const uint32_t end = uint32_t(std::min<uint64_t>(uint64_t(b) + c.len, e.g.off[c.chr + 1]));
      if (b >= end) return;
      const auto cov = covering(g, b);
      if (cov.empty()) return;
      const uint32_t last = c.begin + (end - b) - 1;
      if (c.amp) {
        const uint32_t ord = c.src >= 0 ? uint32_t(c.src) : ord_of(uint32_t(cov.size()));
        if (ord >= cov.size()) throw std::runtime_error("CNA source allele does not cover the region");
        const uint32_t x = cov[ord], made = n_inst++;
        g[made] = ivl_within(g[x], b, end);
        pl.copies.push_back({v, event, made, x});
        pl.cnas.push_back({v, 1, c.chr, c.begin, last, made, x, uint8_t(passenger ? 0 : 1)});
      } else {
        if (passenger && e.avoid_losses && cov.size() <= 1) return;
        const uint32_t ord = c.allele >= 0 ? uint32_t(c.allele) : ord_of(uint32_t(cov.size()));
        if (ord >= cov.size()) throw std::runtime_error("CNA allele does not cover the region");
        const uint32_t x = cov[ord];
        g[x] = ivl_minus(g[x], b, end);
        if (g[x].empty()) g.erase(x);
        pl.cnas.push_back({v, 0, c.chr, c.begin, last, x, x, uint8_t(passenger ? 0 : 1)});
      }
      changed = true;
    };
    for (uint32_t j = 0; j < nd; ++j) {
      const DriverEvent& de = (*list)[j];
      if (de.kind == 0) {
        DriverRec r = driver_site(e, de.sid, v);
        const auto cov = covering(g, r.locus);
        if (cov.empty()) throw std::runtime_error("a driver mutation lies where the cell has no allele left");
        uint32_t ord;
        if (de.sid.allele >= 0) {
          ord = uint32_t(de.sid.allele);
          if (ord >= cov.size()) throw std::runtime_error("driver allele does not exist there");
        } else {
          ord = draws.sid_ord(n_sid, v, uint32_t(cov.size()));
        }
        r.allele = cov[ord];
        r.order = int32_t(j);
        drv.push_back(r);
        ++n_sid;
      } else if (de.kind == 1) {
        cna(de.cna, j, [&](uint32_t n) { return draws.cna_ord(v, j, n); }, false);
      } else {
        std::vector<uint32_t> present;
        for (const auto& kv : g) present.push_back(kv.first);
        for (uint32_t x : present) {
          const uint32_t made = n_inst++;
          g[made] = g[x];
          pl.copies.push_back({v, j, made, x});
        }
        pl.cnas.push_back({v, 2, 0, 0, 0, 0, 0, 1});
        changed = true;
      }
    }
    for (uint64_t k = 0; k < n_pcna[v]; ++k) {
      const uint32_t kk = uint32_t(k);
      cna(e.cands[draws.pcna_cand(v, kk, uint32_t(e.cands.size()))], nd + kk,
          [&](uint32_t n) { return draws.pcna_ord(v, kk, n); }, true);
    }
    if (changed) { pl.classes.push_back(std::move(g)); pl.node_class[v] = uint32_t(pl.classes.size() - 1); }
    else pl.node_class[v] = base;
  }
  if (n_inst >= 0xffff) throw std::runtime_error("too many allele instances");
  pl.n_inst = n_inst;
  pl.has_cna = pl.classes.size() > 1 || n_inst > 2;
  pl.cn_max = 2;
  for (const auto& g : pl.classes) pl.cn_max = std::max(pl.cn_max, max_copies(g));
  pl.index.clear();
  for (const auto& g : pl.classes) pl.index.push_back(class_index(g));
  build_atoms(pl, uint32_t(e.g.b.size()));
  return drv;
}


// number of divisions of edge v per epoch
std::vector<uint32_t> divisions_per_epoch(const Forest& f, const Tables& t, uint32_t v) {
  std::vector<uint32_t> nd(t.E, 0);
  const double tv = f.birth[v];
  const double tu = f.parent[v] >= 0 ? f.birth[f.parent[v]] : tv;
  const uint32_t d = f.divisions[v];
  for (uint32_t j = 0; j < d; ++j) {
    const double tj = tu + (tv - tu) * (double(j + 1) / double(d));
    uint32_t ep = 0;
    while (ep + 1 < t.E && t.times[ep + 1] <= tj) ++ep;
    nd[ep] += 1;
  }
  return nd;
}

// indel descriptor of class cls at position p (random bits w)
uint32_t indel_aux(const Engine& e, uint32_t cls, uint32_t p, uint32_t w) {
  uint32_t ins = 0, l = 1, bases = 0;
  if (cls < 12) { ins = 0; l = 1; }
  else if (cls < 24) {
    ins = 1; l = 1;
    if ((cls - 12) % 6 >= 1) bases = e.g.b[p];
    else bases = (cls < 18) ? ((w & 1u) ? 2u : 1u) : ((w & 1u) ? 0u : 3u);
  } else if (cls < 48) { l = (cls - 24) / 6 + 2; }
  else if (cls < 72) {
    ins = 1; l = (cls - 48) / 6 + 2;
    if ((cls - 48) % 6 >= 1) { for (uint32_t k = 0; k < l; ++k) bases |= uint32_t(e.g.b[p + k]) << (2 * k); }
    else bases = w & ((1u << (2 * l)) - 1u);
  } else {
    l = cls == 72 ? 2 : (cls < 75 ? 3 : (cls < 78 ? 4 : 5));
  }
  return ins | (l << 1) | (bases << 8);
}

// ---- flavour 0: Philox replay
constexpr uint32_t LOCUS_NONE = 0xffffffffu;   // drawn where the cell has no allele left

void place_replay(const Engine& e, const Forest& f, uint32_t n_pre_snv, uint32_t pre_sbs, uint32_t n_pre_id,
                  uint32_t pre_id, uint64_t seed, Placed& out) {
  const Tables t = make_tables(e, f, n_pre_snv, pre_sbs, n_pre_id, pre_id);
  const uint32_t N = f.n, E = t.E;
  PhiloxDraws draws{seed};
  const auto drv = replay_events(e, f, draws, out);
  std::vector<double> class_size(out.classes.size());
  for (size_t c = 0; c < class_size.size(); ++c) class_size[c] = double(genome_size(out.classes[c]));
  std::vector<uint32_t> cnt_snv(uint64_t(N + 1) * E, 0), cnt_id(uint64_t(N + 1) * E, 0);
  for (uint32_t v = 0; v < N; ++v) {
    const auto nd = divisions_per_epoch(f, t, v);
    const uint32_t sp = f.species[v];
    const double A = class_size[out.node_class[v]];   // allelic size of the edge's genome
    for (uint32_t ep = 0; ep < E; ++ep) {
      const double ls = t.snv_rate[uint64_t(sp) * E + ep] * A * double(nd[ep]);
      const double li = t.id_rate[uint64_t(sp) * E + ep] * A * double(nd[ep]);
      Stream s1 = stream(seed, ep, v, 0, TAG_EDGE_SNV), s2 = stream(seed, ep, v, 0, TAG_EDGE_INDEL);
      cnt_snv[uint64_t(v) * E + ep] = uint32_t(poisson(s1, ls));
      cnt_id[uint64_t(v) * E + ep] = uint32_t(poisson(s2, li));
    }
  }
  cnt_snv[uint64_t(N) * E] = n_pre_snv;
  cnt_id[uint64_t(N) * E] = n_pre_id;
  // slots: all SNVs (edge-major, epoch, draw), then all indels, then drivers
  struct Slot { uint32_t edge, epoch, m; bool indel; };
  std::vector<Slot> slots;
  for (int ty = 0; ty < 2; ++ty) {
    const auto& cnt = ty == 0 ? cnt_snv : cnt_id;
    for (uint32_t v = 0; v <= N; ++v)
      for (uint32_t ep = 0; ep < E; ++ep)
        for (uint32_t m = 0; m < cnt[uint64_t(v) * E + ep]; ++m) slots.push_back({v, ep, m, ty == 1});
  }
  const size_t n_pass = slots.size(), n_all = n_pass + drv.size();
  std::vector<uint32_t> locus(n_all), aux(n_all), edge(n_all), attempt(n_all, 0);
  std::vector<uint8_t> cls(n_all), sig(n_all), kind(n_all), nature(n_all);
  std::vector<uint16_t> allele(n_all);
  std::vector<int32_t> order(n_all);
  auto draw_pos = [&](size_t i) {
    const Slot& sl = slots[i];
    Stream st = stream(seed, sl.m, sl.edge, sl.epoch, sl.indel ? TAG_INDEL : TAG_SNV);
    st.block = 1 + attempt[i];
    const W4 r = st.next();
    if (attempt[i] >= 4) {   // class redrawn from the same signature after 4 collisions
      const int ty = sl.indel ? 1 : 0;
      const uint32_t NC = ty == 0 ? 96 : 83;
      cls[i] = uint8_t(lookup(&t.sig_cdf[ty][uint64_t(sig[i]) * NC], NC, r.v[3]));
    }
    const std::vector<uint32_t>& list = sl.indel ? e.id[cls[i]] : e.ctx[sbs_ctx(cls[i])];
    const uint32_t p = list[index64(r.v[0], r.v[1], list.size())];
    const uint32_t loc = sl.indel ? p - 1 : p;
    const auto& cov = covering(out.index[out.node_class[sl.edge]], loc);
    if (cov.empty()) { locus[i] = LOCUS_NONE; return; }
    allele[i] = uint16_t(cov[mulhi32(r.v[2], uint32_t(cov.size()))]);
    locus[i] = loc;
    if (!sl.indel) {
      const int ref = e.g.b[p];
      const int ap = sbs_alt(cls[i]);
      aux[i] = uint32_t((ref == 1 || ref == 3) ? ap : 3 - ap);
    } else {
      aux[i] = indel_aux(e, cls[i], p, r.v[3]);
    }
  };
  for (size_t i = 0; i < n_pass; ++i) {
    const Slot& sl = slots[i];
    const int ty = sl.indel ? 1 : 0;
    const uint32_t NC = ty == 0 ? 96 : 83;
    Stream st = stream(seed, sl.m, sl.edge, sl.epoch, sl.indel ? TAG_INDEL : TAG_SNV);
    const W4 r = st.next();
    const uint32_t row = sl.edge == N ? E : sl.epoch;
    const uint32_t s = lookup(&t.expo_cdf[ty][uint64_t(row) * t.ns[ty]], t.ns[ty], r.v[0]);
    const uint32_t k = lookup(&t.sig_cdf[ty][uint64_t(s) * NC], NC, r.v[1]);
    sig[i] = uint8_t(s); cls[i] = uint8_t(k); edge[i] = sl.edge;
    kind[i] = sl.indel ? 1 : 0;
    nature[i] = sl.edge == N ? 2 : 0;
    order[i] = sl.edge == N ? -1 : INT32_MAX;
    draw_pos(i);
  }
  for (size_t d = 0; d < drv.size(); ++d) {
    const size_t i = n_pass + d;
    locus[i] = drv[d].locus; edge[i] = drv[d].edge; aux[i] = drv[d].aux; kind[i] = drv[d].kind;
    cls[i] = 0xff; sig[i] = 0xff; nature[i] = 1;
    allele[i] = uint16_t(drv[d].allele);
    order[i] = drv[d].order;
  }
  // redraw rounds: colliding loci under infinite sites (lowest slot wins), and
  // loci drawn where the edge's genome has no allele left
  if ((e.infinite_sites || out.has_cna) && n_pass > 0) {
    std::unordered_set<uint32_t> accepted;
    if (e.infinite_sites) for (size_t d = 0; d < drv.size(); ++d) accepted.insert(drv[d].locus);
    std::vector<size_t> pending(n_pass);
    for (size_t i = 0; i < n_pass; ++i) pending[i] = i;
    int round = 0;
    while (!pending.empty()) {
      if (round >= 256) throw std::runtime_error("no free locus left for some mutations");
      std::vector<size_t> next;
      if (e.infinite_sites) {
        std::unordered_map<uint32_t, size_t> best;
        std::vector<uint8_t> lost(pending.size(), 0);
        for (size_t q = 0; q < pending.size(); ++q) {
          const size_t i = pending[q];
          if (locus[i] == LOCUS_NONE || accepted.count(locus[i])) { lost[q] = 1; continue; }
          auto it = best.find(locus[i]);
          if (it == best.end() || i < it->second) best[locus[i]] = i;
        }
        for (size_t q = 0; q < pending.size(); ++q) {
          const size_t i = pending[q];
          if (!lost[q] && best[locus[i]] == i) accepted.insert(locus[i]);
          else next.push_back(i);
        }
      } else {
        for (size_t i : pending) if (locus[i] == LOCUS_NONE) next.push_back(i);
      }
      for (size_t i : next) { attempt[i] += 1; draw_pos(i); }
      pending.swap(next);
      ++round;
    }
  }
  std::vector<size_t> ord(n_all);
  for (size_t i = 0; i < n_all; ++i) ord[i] = i;
  std::sort(ord.begin(), ord.end(), [&](size_t a, size_t b) {
    return locus[a] != locus[b] ? locus[a] < locus[b] : a < b;
  });
  auto perm = [&](auto& v) { auto c = v; for (size_t i = 0; i < n_all; ++i) v[i] = c[ord[i]]; };
  perm(locus); perm(edge); perm(aux); perm(cls); perm(sig); perm(allele); perm(kind); perm(nature); perm(order);
  out.locus = locus; out.edge = edge; out.aux = aux; out.cls = cls; out.sig = sig;
  out.allele = allele; out.kind = kind; out.nature = nature; out.order = order;
}

// ---- flavour 1: sequential std::mt19937_64 engine
void place_mt(const Engine& e, const Forest& f, uint32_t n_pre_snv, uint32_t pre_sbs, uint32_t n_pre_id,
              uint32_t pre_id, uint64_t seed, Placed& out) {
  const Tables t = make_tables(e, f, n_pre_snv, pre_sbs, n_pre_id, pre_id);
  std::mt19937_64 rng(seed);
  const uint32_t N = f.n, E = t.E;
  std::unordered_set<uint32_t> used;
  MtDraws draws{rng};
  const auto drv = replay_events(e, f, draws, out);   // drivers carry their alleles
  std::vector<double> class_size(out.classes.size());
  for (size_t c = 0; c < class_size.size(); ++c) class_size[c] = double(genome_size(out.classes[c]));
  auto push = [&](uint32_t loc, uint32_t ed, uint32_t ax, int c, int s, int al, int k, int nat, int32_t o) {
    out.locus.push_back(loc); out.edge.push_back(ed); out.aux.push_back(ax); out.cls.push_back(uint8_t(c));
    out.sig.push_back(uint8_t(s)); out.allele.push_back(uint16_t(al)); out.kind.push_back(uint8_t(k));
    out.nature.push_back(uint8_t(nat)); out.order.push_back(o);
  };
  for (const auto& d : drv) {
    used.insert(d.locus);
    push(d.locus, d.edge, d.aux, 0xff, 0xff, int(d.allele), d.kind, 1, d.order);
  }
  auto place_one = [&](uint32_t v, uint32_t row, int ty) {
    const uint32_t NC = ty == 0 ? 96 : 83;
    std::discrete_distribution<uint32_t> ds(t.expo_w[ty][row].begin(), t.expo_w[ty][row].end());
    const uint32_t s = ds(rng);
    std::discrete_distribution<uint32_t> dc(t.sig_w[ty][s].begin(), t.sig_w[ty][s].end());
    uint32_t k = dc(rng);
    (void)NC;
    uint32_t p = 0, loc = 0;
    const ClassIndex& ix = out.index[out.node_class[v]];
    const std::vector<uint32_t>* cov = nullptr;
    for (int tries = 0;; ++tries) {
      if (tries >= 100000) throw std::runtime_error("no free locus left for some mutations");
      if (tries >= 16) k = dc(rng);   // class redrawn after 16 collisions
      const std::vector<uint32_t>& list = ty == 1 ? e.id[k] : e.ctx[sbs_ctx(int(k))];
      std::uniform_int_distribution<uint64_t> dp(0, list.size() - 1);
      p = list[dp(rng)];
      loc = ty == 0 ? p : p - 1;
      cov = &covering(ix, loc);        // no allele left there: draw again
      if (!cov->empty() && (!e.infinite_sites || !used.count(loc))) break;
    }
    if (e.infinite_sites) used.insert(loc);
    const int al = int((*cov)[std::uniform_int_distribution<size_t>(0, cov->size() - 1)(rng)]);
    uint32_t ax;
    if (ty == 0) { const int ref = e.g.b[p]; const int ap = sbs_alt(int(k)); ax = uint32_t((ref == 1 || ref == 3) ? ap : 3 - ap); }
    else ax = indel_aux(e, k, p, uint32_t(rng()));
    push(loc, v, ax, int(k), int(s), al, ty, v == N ? 2 : 0, v == N ? -1 : INT32_MAX);
  };
  for (uint32_t m = 0; m < n_pre_snv; ++m) place_one(N, E, 0);
  for (uint32_t m = 0; m < n_pre_id; ++m) place_one(N, E, 1);
  for (uint32_t v = 0; v < N; ++v) {
    const auto nd = divisions_per_epoch(f, t, v);
    const uint32_t sp = f.species[v];
    for (uint32_t ep = 0; ep < E; ++ep) {
      const double A = class_size[out.node_class[v]];
      const double ls = t.snv_rate[uint64_t(sp) * E + ep] * A * double(nd[ep]);
      const double li = t.id_rate[uint64_t(sp) * E + ep] * A * double(nd[ep]);
      const uint64_t ns = ls > 0 ? std::poisson_distribution<uint64_t>(ls)(rng) : 0;
      const uint64_t ni = li > 0 ? std::poisson_distribution<uint64_t>(li)(rng) : 0;
      for (uint64_t m = 0; m < ns; ++m) place_one(v, ep, 0);
      for (uint64_t m = 0; m < ni; ++m) place_one(v, ep, 1);
    }
  }
  const size_t n = out.locus.size();
  std::vector<size_t> order(n);
  for (size_t i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return out.locus[a] < out.locus[b]; });
  auto perm = [&](auto& v) { auto c = v; for (size_t i = 0; i < n; ++i) v[i] = c[order[i]]; };
  perm(out.locus); perm(out.edge); perm(out.aux); perm(out.cls); perm(out.sig); perm(out.allele);
  perm(out.kind); perm(out.nature); perm(out.order);
}

// ------------------------------------------------------------ sequencing
struct SeqCfg {  // same layout as pg_seq_cfg
  double coverage;
  uint32_t read_size, insert_size_mean, insert_size_stddev;
  int insert_model;
  double error_rate, purity;
  int with_normal_sample, preneoplastic_in_normal, normal_only;
  uint32_t n_chr_sel;
  const uint32_t* chr_sel;
  uint32_t tile_size;
};

struct SeqOut { uint32_t n_samples = 0; std::vector<uint32_t> alt, depth; uint64_t n_reads = 0; };

// insert-size pmf table (min insert, weights): the reference's binomial
// model (src/seq_simulation.cpp:431-451) or a discretised normal, tails
// below 1e-13 dropped, inserts shorter than a read folded onto the read size
void insert_weights(const SeqCfg& c, uint32_t R, uint32_t& k0, std::vector<double>& w) {
  const double mean = c.insert_size_mean, sd = c.insert_size_stddev;
  w.clear();
  k0 = 0;
  if (c.insert_model == 0) {
    const double q = double(c.insert_size_stddev) * double(c.insert_size_stddev) / mean;
    const double p = 1 - q;
    if (p <= 0) throw std::runtime_error("insert size mean below its variance");
    const uint32_t t = uint32_t(mean / p);
    const double lp = std::log(p), lq = q > 0 ? std::log(q) : -INFINITY;
    std::vector<double> pmf(t + 1);
    for (uint32_t k = 0; k <= t; ++k) {
      if (q <= 0) { pmf[k] = (k == t) ? 1.0 : 0.0; continue; }
      pmf[k] = std::exp(std::lgamma(t + 1.0) - std::lgamma(k + 1.0) - std::lgamma(double(t - k) + 1.0) + k * lp +
                        double(t - k) * lq);
    }
    uint32_t lo = 0, hi = t;
    double cum = 0;
    while (lo < t && cum + pmf[lo] < 1e-13) { cum += pmf[lo]; ++lo; }
    cum = 0;
    while (hi > lo && cum + pmf[hi] < 1e-13) { cum += pmf[hi]; --hi; }
    k0 = lo;
    w.assign(pmf.begin() + lo, pmf.begin() + hi + 1);
  } else {
    const double a = std::max(1.0, std::floor(mean - 10 * sd)), b = std::ceil(mean + 10 * sd);
    k0 = uint32_t(a);
    for (double k = a; k <= b; k += 1) {
      const double z0 = (k - 0.5 - mean) / (sd * std::sqrt(2.0)), z1 = (k + 0.5 - mean) / (sd * std::sqrt(2.0));
      w.push_back(0.5 * (std::erfc(z0) - std::erfc(z1)));
    }
  }
  if (k0 < R) {
    const uint32_t drop = std::min<uint32_t>(R - k0, uint32_t(w.size()) - 1);
    double mass = 0;
    for (uint32_t i = 0; i < drop; ++i) mass += w[i];
    w.erase(w.begin(), w.begin() + drop);
    w[0] += mass;
    k0 += drop;
    if (k0 < R) k0 = R;
  }
}

// does the read from `cell` (node id, or -1 for a normal cell) carry mutation i?
struct Carrier {
  const Forest& f;
  bool pre_in_normal;
  bool ancestor_or_self(uint32_t e, int64_t cell) const {
    if (e == f.n) return cell >= 0 || pre_in_normal;   // preneoplastic edge
    if (e == f.n + 1) return true;                     // germline
    if (cell < 0) return false;
    int64_t v = cell;
    while (v >= 0) { if (uint32_t(v) == e) return true; v = f.parent[v]; }
    return false;
  }
};

struct SampleDesc { std::vector<uint32_t> leaves; uint32_t normal_thr; bool all_normal; };

struct SeqSetup {
  std::vector<uint32_t> chrs;
  std::vector<SampleDesc> samples;
  uint32_t R, ins_min, err_thr;
  bool paired;
  std::vector<double> ins_w;
  std::vector<uint32_t> ins_thr;
};

SeqSetup seq_setup(const Placed& pl, const SeqCfg& c) {
  const Engine& e = *pl.eng;
  const Forest& f = *pl.forest;
  SeqSetup s;
  s.R = c.read_size;
  s.paired = c.insert_size_mean > 0;
  s.ins_min = s.R;
  s.ins_w = {1.0};
  if (s.paired) insert_weights(c, s.R, s.ins_min, s.ins_w);
  s.ins_thr = thresholds(s.ins_w);
  if (c.n_chr_sel) { s.chrs.assign(c.chr_sel, c.chr_sel + c.n_chr_sel); std::sort(s.chrs.begin(), s.chrs.end()); s.chrs.erase(std::unique(s.chrs.begin(), s.chrs.end()), s.chrs.end()); }
  else for (uint32_t i = 0; i + 1 < e.g.off.size(); ++i) s.chrs.push_back(i);
  double nthr = std::floor((1.0 - c.purity) * 4294967296.0);
  if (nthr > 4294967295.0) nthr = 4294967295.0;
  if (!c.normal_only) {
    for (uint32_t smp = 0; smp < f.n_samples; ++smp) {
      SampleDesc d;
      d.leaves = f.leaves[smp];
      if (d.leaves.empty()) throw std::runtime_error("sample without sampled cells");
      d.normal_thr = c.purity >= 1 ? 0u : uint32_t(nthr);
      d.all_normal = c.purity <= 0;
      s.samples.push_back(d);
    }
  }
  if (c.normal_only || c.with_normal_sample) s.samples.push_back({{}, 0u, true});
  double et = std::floor(c.error_rate * 4294967296.0);
  s.err_thr = et >= 4294967295.0 ? 0xffffffffu : uint32_t(et);
  return s;
}

// error words (the read kernel's mate_word / err_word in pg_seq.cu): a
// mate's word is the fragment's error word (the XOR of the four words of its
// Philox block) for mate 0 and w * 0x85EBCA6B + 0x27D4EB2F for mate 1; the
// visit of a mate to `locus` hashes it with the locus by one odd multiply.
// A word below the error threshold thr is a substitution error; the
// erroneous base is the first, second or third of the other bases as the
// word lies in [0, thr/3), [thr/3, 2thr/3) or [2thr/3, thr) (integer thirds)
uint32_t mate_word(uint32_t w, uint32_t mate) { return mate ? w * 0x85EBCA6Bu + 0x27D4EB2Fu : w; }

uint32_t error_word(uint32_t w, uint32_t locus, uint32_t mate) {
  return (mate_word(w, mate) ^ (locus * 0x9E3779B1u)) * 0xC2B2AE35u;
}

uint32_t error_third(uint32_t e, uint32_t thr) {
  const uint32_t t1 = thr / 3u, t2 = uint32_t(uint64_t(thr) * 2u / 3u);
  return e < t1 ? 0u : (e < t2 ? 1u : 2u);
}

// Allele instances carrying mutation i: its own instance and every copy made
// from a carrier after the mutation (later on its edge, or on an edge below
// it; preneoplastic mutations precede every copy).  Copies are visited in the
// order they were made, so a copy's source is settled before it.
std::vector<std::vector<uint32_t>> carrier_sets(const Placed& pl) {
  const Forest& f = *pl.forest;
  const size_t M = pl.locus.size();
  std::vector<std::vector<uint32_t>> out(M);
  auto below = [&](uint32_t u, uint32_t e) {
    for (int32_t x = f.parent[u]; x >= 0; x = f.parent[x]) if (uint32_t(x) == e) return true;
    return false;
  };
  for (size_t i = 0; i < M; ++i) {
    std::vector<uint32_t>& c = out[i];
    c.push_back(pl.allele[i]);
    const uint32_t ei = pl.edge[i];
    for (const CopyRec& cp : pl.copies) {
      if (std::find(c.begin(), c.end(), cp.from) == c.end()) continue;
      const bool after = ei >= f.n || (cp.edge == ei && int64_t(cp.event) > int64_t(pl.order[i])) ||
                         below(cp.edge, ei);
      if (after) c.push_back(cp.made);
    }
  }
  return out;
}

void count_mate(const Placed& pl, const Carrier& car, const std::vector<std::vector<uint32_t>>& carriers,
                uint32_t a, uint32_t R, int64_t cell, uint32_t allele, uint32_t err_thr, uint32_t mate, uint32_t w,
                uint32_t* alt, uint32_t* dep) {
  auto it = std::lower_bound(pl.locus.begin(), pl.locus.end(), a);
  for (size_t i = size_t(it - pl.locus.begin()); i < pl.locus.size() && pl.locus[i] < a + R; ++i) {
    const auto& cs = carriers[i];
    const bool carried = car.ancestor_or_self(pl.edge[i], cell) && std::find(cs.begin(), cs.end(), allele) != cs.end();
    bool obs;
    if (pl.kind[i] == 1) obs = carried;
    else {
      const uint32_t e = error_word(w, pl.locus[i], mate);
      const bool err = e < err_thr;
      obs = carried ? !err : (err && error_third(e, err_thr) == 0);   // the erroneous base is one of three
    }
    dep[i] += 1;
    if (obs) alt[i] += 1;
  }
}

// copies of genome g summed over positions [a, b), and the largest copy
// number there
void copies_in(const CellGenome& g, uint32_t a, uint32_t b, uint64_t& sum, uint32_t& mx) {
  std::vector<std::pair<uint32_t, int>> ev;
  sum = 0;
  for (const auto& kv : g)
    for (auto [x, y] : kv.second) {
      const uint32_t lo = std::max(x, a), hi = std::min(y, b);
      if (lo >= hi) continue;
      sum += hi - lo;
      ev.push_back({lo, 1});
      ev.push_back({hi, -1});
    }
  std::sort(ev.begin(), ev.end());
  int cur = 0, best = 0;
  for (auto [p, d] : ev) { cur += d; best = std::max(best, cur); }
  mx = uint32_t(best);
}

// ---- flavour 0: replay of the tiled read generation
// called once per fragment of the replay, in draw order: sample, chromosome,
// dropped (no DNA under the draw), mate starts, cell (node id, -1 normal),
// allele instance and the fragment's error word
using FragmentVisitor = std::function<void(uint32_t smp, uint32_t ci, bool dropped, uint32_t p0, uint32_t p1,
                                           int64_t cell, uint32_t allele, uint32_t fw)>;

void seq_replay(const Placed& pl, const SeqCfg& c, uint64_t seed, SeqOut& out, const FragmentVisitor* visit = nullptr) {
  const Engine& e = *pl.eng;
  const Forest& f = *pl.forest;
  const SeqSetup s = seq_setup(pl, c);
  const uint32_t T = c.tile_size;
  if (T == 0) throw std::runtime_error("the replay needs an explicit tile size");
  const size_t M = pl.locus.size();
  out.n_samples = uint32_t(s.samples.size());
  out.alt.assign(out.n_samples * M, 0);
  out.depth.assign(out.n_samples * M, 0);
  Carrier car{f, c.preneoplastic_in_normal != 0};
  const auto carriers = carrier_sets(pl);
  const double mates = s.paired ? 2.0 : 1.0;
  const uint32_t k0 = uint32_t(seed), k1 = uint32_t(seed >> 32);
  // With copy-number events, (start, cell, instance) follows the DNA of the
  // sample's cells: a cell is normal with probability wn (normal_thr / 2^32,
  // 1 for the normal sample), else one of the nl leaves.  Options: the
  // normal cells (class 0), then the leaf classes ascending, each with its
  // leaves in node order.  Over atom a an option weighs wn * copies(a, 0) or
  // (1 - wn) / nl * (n_c * copies(a, c)); a stretch of starts weighs
  // wn * I0 + (1 - wn) / nl * S with the integer copy sums I0 and S.
  struct Opt { uint32_t cls; std::vector<uint32_t> leaves; };
  struct SampleCn {
    double wn, wt;
    uint64_t nl;
    std::vector<Opt> opts;
    std::vector<std::vector<uint32_t>> opt_thr;    // per atom
    std::vector<uint64_t> icnt0, S;                 // per atom
    double mass(uint64_t i0, uint64_t sum) const {
      double m = wn * double(i0);
      if (nl > 0) m = m + (wt / double(nl)) * double(sum);
      return m;
    }
  };
  std::vector<SampleCn> scn(s.samples.size());
  if (pl.has_cna) {
    const size_t NA = pl.atom_start.size();
    for (size_t smp = 0; smp < s.samples.size(); ++smp) {
      const SampleDesc& sd = s.samples[smp];
      SampleCn& q = scn[smp];
      q.wn = sd.all_normal ? 1.0 : double(sd.normal_thr) * (1.0 / 4294967296.0);
      q.wt = 1.0 - q.wn;
      q.opts.push_back({0u, {}});
      std::map<uint32_t, std::vector<uint32_t>> by_class;
      if (q.wt > 0) for (uint32_t leaf : sd.leaves) by_class[pl.node_class[leaf]].push_back(leaf);
      q.nl = 0;
      for (auto& kv : by_class) { q.nl += kv.second.size(); q.opts.push_back({kv.first, kv.second}); }
      q.icnt0.assign(NA, 0); q.S.assign(NA, 0);
      for (size_t a = 0; a < NA; ++a) {
        const auto& cov = pl.atom_cov[a];
        std::vector<double> w{q.wn * double(cov[0].size())};
        for (size_t o = 1; o < q.opts.size(); ++o) {
          const uint64_t n = q.opts[o].leaves.size(), x = n * cov[q.opts[o].cls].size();
          w.push_back((q.wt / double(q.nl)) * double(x));
          q.S[a] += x;
        }
        q.icnt0[a] = cov[0].size();
        q.opt_thr.push_back(thresholds(w));
      }
    }
  }
  uint32_t tile_base = 0;   // global tile index of the chromosome's first tile
  for (uint32_t ci : s.chrs) {
    const uint32_t L = e.g.off[ci + 1] - e.g.off[ci];
    if (L < s.R) continue;
    const uint32_t S = L - s.R + 1, nt = (S + T - 1) / T;
    const uint64_t pairs = uint64_t(std::floor(c.coverage * double(L) / (double(s.R) * mates)));
    const uint32_t ce = e.g.off[ci + 1];
    for (uint32_t smp = 0; smp < out.n_samples; ++smp) {
      const SampleDesc& sd = s.samples[smp];
      // with copy-number events: the parts of each tile (one per atom it
      // meets), the part thresholds and the tile masses of this sample
      struct Part { uint32_t start, len, atom; };
      std::vector<std::vector<Part>> parts(nt);
      std::vector<std::vector<uint32_t>> part_thr(nt);
      // the mass before each tile is the mass of the exact integer copy sums
      // before it
      std::vector<double> cum(nt, 0.0);
      double tot = 0.0;
      uint64_t cum_i0 = 0, cum_s = 0;
      if (pl.has_cna) {
        const SampleCn& q = scn[smp];
        const auto& as = pl.atom_start;
        for (uint32_t k = 0; k < nt; ++k) {
          const uint32_t a = e.g.off[ci] + k * T, b = a + std::min<uint32_t>(T, S - k * T);
          size_t x = size_t(std::upper_bound(as.begin(), as.end(), a) - as.begin()) - 1;
          uint64_t i0 = 0, sum = 0;
          std::vector<double> pw;
          for (; x < as.size() && as[x] < b; ++x) {
            const uint32_t lo = std::max(a, as[x]);
            const uint32_t hi = std::min<uint32_t>(b, x + 1 < as.size() ? as[x + 1] : uint32_t(e.g.b.size()));
            parts[k].push_back({lo, hi - lo, uint32_t(x)});
            const uint64_t len = hi - lo;
            i0 += len * q.icnt0[x];
            sum += len * q.S[x];
            pw.push_back(q.mass(len * q.icnt0[x], len * q.S[x]));
          }
          if (pw.size() > 1) part_thr[k] = thresholds(pw);
          cum[k] = q.mass(cum_i0, cum_s);
          cum_i0 += i0;
          cum_s += sum;
        }
        tot = q.mass(cum_i0, cum_s);
      }
      // multinomial split by a binary tree over the padded tile range
      // [0, 2^D): node h covering [lo, lo+size) sends Binomial(n, w_left/w)
      // fragments to its left half (w = start positions of covered tiles, or
      // their mass)
      uint32_t D = 0;
      while ((uint64_t(1) << D) < nt) ++D;
      auto wts = [&](uint64_t a, uint64_t b) {
        return std::min<uint64_t>(b * T, S) - std::min<uint64_t>(a * T, S);
      };
      auto mass_at = [&](uint64_t a) { return a < nt ? cum[a] : tot; };
      std::vector<uint64_t> tile_pairs(nt, 0);
      struct Node { uint64_t lo, size; uint32_t id; uint64_t n; };
      std::vector<Node> stack{{0, uint64_t(1) << D, 1, pairs}};
      while (!stack.empty()) {
        Node nd = stack.back(); stack.pop_back();
        if (nd.size == 1) { if (nd.lo < nt) tile_pairs[nd.lo] = nd.n; continue; }
        const uint64_t half = nd.size / 2, mid = nd.lo + half;
        uint64_t nl = 0;
        if (!pl.has_cna) {
          const uint64_t wt = wts(nd.lo, nd.lo + nd.size);
          if (nd.n > 0 && wt > 0) {
            const double p = double(wts(nd.lo, mid)) / double(wt);
            Stream st = stream(seed, nd.id, ci, smp, TAG_TILE_SPLIT);
            nl = binomial(st, nd.n, p);
          }
        } else {
          const double lo_m = mass_at(nd.lo), wt = mass_at(nd.lo + nd.size) - lo_m;
          if (nd.n > 0 && wt > 0) {
            const double p = (mass_at(mid) - lo_m) / wt;
            Stream st = stream(seed, nd.id, ci, smp, TAG_TILE_SPLIT);
            nl = binomial(st, nd.n, p);
          }
        }
        stack.push_back({nd.lo, half, 2 * nd.id, nl});
        stack.push_back({mid, half, 2 * nd.id + 1, nd.n - nl});
      }
      uint32_t* alt = out.alt.data() + uint64_t(smp) * M;
      uint32_t* dep = out.depth.data() + uint64_t(smp) * M;
      for (uint32_t k = 0; k < nt; ++k) {
        const uint32_t t = tile_base + k;
        const uint32_t start = e.g.off[ci] + k * T, len = std::min<uint32_t>(T, S - k * T);
        for (uint32_t j = 0; j < tile_pairs[k]; ++j) {
          out.n_reads += s.paired ? 2 : 1;
          // start, cell and allele instance: one Philox block per fragment
          // (x start / part, y cell / option, z insert, w instance then
          // leaf from the fraction the instance draw leaves)
          const W4 r = philox(k0, k1, j, t, smp, TAG_PAIR);
          uint32_t p0, allele;
          int64_t cell;
          if (!pl.has_cna) {
            p0 = start + mulhi32(r.v[0], len);
            const bool normal = sd.all_normal || r.v[1] < sd.normal_thr;
            allele = mulhi32(r.v[3], 2);
            cell = normal ? -1 : int64_t(sd.leaves[mulhi32(r.v[3] * 2u, uint32_t(sd.leaves.size()))]);
          } else {
            // part (when the tile meets several atoms) and start in the part
            // from word x: the start from the word's place in the part's
            // threshold interval; option from y; instance, then leaf, from w
            const SampleCn& q = scn[smp];
            const auto& pk = parts[k];
            size_t pi = 0;
            if (pk.size() > 1) {
              pi = lookup(part_thr[k].data(), uint32_t(pk.size()), r.v[0]);
              const uint64_t lo = pi ? part_thr[k][pi - 1] : 0u, hi = part_thr[k][pi];
              p0 = pk[pi].start + uint32_t((uint64_t((r.v[0] >> 1) - lo) * pk[pi].len) / (hi - lo));
            } else {
              p0 = pk[0].start + mulhi32(r.v[0], pk[0].len);
            }
            const Part& pt = pk[pi];
            const uint32_t o = lookup(q.opt_thr[pt.atom].data(), uint32_t(q.opts.size()), r.v[1]);
            const Opt& op = q.opts[o];
            const auto& cov = pl.atom_cov[pt.atom][op.cls];
            if (cov.empty()) {             // an option without DNA here is never drawn
              if (visit) (*visit)(smp, ci, true, p0, p0, -1, 0, 0);
              continue;
            }
            const uint32_t n_cov = uint32_t(cov.size());
            allele = cov[mulhi32(r.v[3], n_cov)];
            cell = op.leaves.empty() ? -1
                                     : int64_t(op.leaves[mulhi32(r.v[3] * n_cov, uint32_t(op.leaves.size()))]);
          }
          const uint32_t fw = r.v[0] ^ r.v[1] ^ r.v[2] ^ r.v[3];
          count_mate(pl, car, carriers, p0, s.R, cell, allele, s.err_thr, 0, fw, alt, dep);
          uint32_t p1 = p0;
          if (s.paired) {
            const uint32_t ins = s.ins_min + lookup(s.ins_thr.data(), uint32_t(s.ins_thr.size()), r.v[2]);
            p1 = p0 + ins - s.R;
            if (p1 > ce - s.R) p1 = ce - s.R;
            count_mate(pl, car, carriers, p1, s.R, cell, allele, s.err_thr, 1, fw, alt, dep);
          }
          if (visit) (*visit)(smp, ci, false, p0, p1, cell, allele, fw);
        }
      }
    }
    tile_base += nt;
  }
}

// ---- SAM reads of the replay (simulate_seq with write_SAM, the reads of
// src/seq_simulation.cpp:540-564).  A mate starting at reference position p
// shows, position by position, the reference base, or the alt base of an SNV
// its allele carries (the first such record at the position), or a
// substitution where the visit's error word is below the error threshold:
// one of the three other bases, chosen by error_third among them in the order
// (counterpart allele first at an SNV site -- the alt base when the read
// shows the reference, the reference base when it shows the alt --, then
// the rest ascending).  Unknown reference bases read N.  After the anchor of
// an indel its allele carries (the first such record), an insertion adds its
// bases (each with its own error word: the fragment word mixed with the
// base's rank) and a deletion skips its bases; indels anchored before p are
// not applied, and none once the CIGAR would pass 16 operations.  The read
// stops after R bases or at the chromosome end.
struct OracleRead { std::vector<std::pair<char, uint32_t>> cigar; std::string seq; };

uint32_t other_base(uint32_t tb, int first, uint32_t k) {
  std::vector<uint32_t> o;
  if (first >= 0 && uint32_t(first) != tb) o.push_back(uint32_t(first));
  for (uint32_t x = 0; x < 4; ++x)
    if (x != tb && (o.empty() || x != o[0])) o.push_back(x);
  return o[k];
}

OracleRead oracle_read(const Placed& pl, const Carrier& car, const std::vector<std::vector<uint32_t>>& carriers,
                       const std::vector<uint32_t>& aux, uint32_t p, uint32_t ce, int64_t cell, uint32_t allele,
                       uint32_t fw, uint32_t mate, uint32_t R, uint32_t err_thr) {
  const Genome& g = pl.eng->g;
  const char* ACGT = "ACGT";
  const size_t kMaxCigar = 16;
  OracleRead out;
  auto push = [&](char op, uint32_t len) {
    if (!out.cigar.empty() && out.cigar.back().first == op) { out.cigar.back().second += len; return; }
    if (out.cigar.size() < kMaxCigar) out.cigar.push_back({op, len});
  };
  auto is_carried = [&](size_t i) {
    const auto& cs = carriers[i];
    return car.ancestor_or_self(pl.edge[i], cell) && std::find(cs.begin(), cs.end(), allele) != cs.end();
  };
  bool indels_open = true;
  uint32_t q = p;
  while (out.seq.size() < R && q < ce) {
    const uint32_t b = g.b[q];
    bool site = false, carried_snv = false, has_indel = false;
    uint32_t alt = 0, indel = 0;
    auto it = std::lower_bound(pl.locus.begin(), pl.locus.end(), q);
    for (size_t i = size_t(it - pl.locus.begin()); i < pl.locus.size() && pl.locus[i] == q; ++i) {
      if (pl.kind[i] == 0) {
        if (!site) { site = true; alt = aux[i] & 3u; }
        if (!carried_snv && is_carried(i)) { carried_snv = true; alt = aux[i] & 3u; }
      } else if (!has_indel && is_carried(i)) {
        has_indel = true;
        indel = aux[i];
      }
    }
    uint32_t tb = carried_snv ? alt : b;
    const uint32_t ew = error_word(fw, q, mate);
    if (ew < err_thr) tb = other_base(tb, site ? int(carried_snv ? b : alt) : -1, error_third(ew, err_thr));
    out.seq.push_back(b > 3 ? 'N' : ACGT[tb]);
    push('M', 1);
    ++q;
    if (has_indel && indels_open && out.cigar.size() < kMaxCigar - 2) {
      const uint32_t l = (indel >> 1) & 7u;
      if (indel & 1u) {
        for (uint32_t k = 0; k < l && out.seq.size() < R; ++k) {
          uint32_t ib = (indel >> (8 + 2 * k)) & 3u;
          const uint32_t ei = error_word(mate_word(fw, mate) ^ (0x9E3779B1u * (k + 1)), q - 1, 0);
          if (ei < err_thr) ib = other_base(ib, -1, error_third(ei, err_thr));
          out.seq.push_back(ACGT[ib]);
          push('I', 1);
        }
      } else if (out.seq.size() < R) {
        push('D', l);
        q += l;
      }
    } else if (has_indel) {
      indels_open = false;
    }
  }
  return out;
}

// ---- flavour 1: sequential reads, std::mt19937_64 and std:: distributions.
// `fraction` < 1 simulates that fraction of each chromosome's fragments (a
// bounded sample for the timed CPU baseline); `threads` splits the samples
// and chromosomes over host threads, each with its own engine.
void seq_mt(const Placed& pl, const SeqCfg& c, uint64_t seed, double fraction, int threads, SeqOut& out) {
  const Engine& e = *pl.eng;
  const Forest& f = *pl.forest;
  const SeqSetup s = seq_setup(pl, c);
  const size_t M = pl.locus.size();
  out.n_samples = uint32_t(s.samples.size());
  out.alt.assign(out.n_samples * M, 0);
  out.depth.assign(out.n_samples * M, 0);
  Carrier car{f, c.preneoplastic_in_normal != 0};
  const auto carriers = carrier_sets(pl);
  const double mates = s.paired ? 2.0 : 1.0;
  // insert distribution of the reference: std::binomial_distribution(t, p)
  uint32_t bin_t = 0;
  double bin_p = 1.0;
  if (s.paired && c.insert_model == 0) {
    const double q = double(c.insert_size_stddev) * double(c.insert_size_stddev) / double(c.insert_size_mean);
    bin_p = 1 - q;
    bin_t = uint32_t(double(c.insert_size_mean) / bin_p);
  }
  struct Job { uint32_t smp, chr; };
  std::vector<Job> jobs;
  for (uint32_t smp = 0; smp < out.n_samples; ++smp) for (uint32_t ci : s.chrs) jobs.push_back({smp, ci});
  std::atomic<size_t> next{0};
  std::atomic<uint64_t> reads{0};
  const int nth = std::max(1, threads);
  std::vector<std::vector<uint32_t>> alt_t(nth, std::vector<uint32_t>(out.n_samples * M, 0)),
      dep_t(nth, std::vector<uint32_t>(out.n_samples * M, 0));
  auto worker = [&](int w) {
    for (size_t ji = next.fetch_add(1); ji < jobs.size(); ji = next.fetch_add(1)) {
      const Job jb = jobs[ji];
      std::mt19937_64 rng(seed ^ (0x9E3779B97F4A7C15ull * (ji + 1)));
      const SampleDesc& sd = s.samples[jb.smp];
      const uint32_t L = e.g.off[jb.chr + 1] - e.g.off[jb.chr];
      if (L < s.R) continue;
      const uint32_t cs = e.g.off[jb.chr], ce = e.g.off[jb.chr + 1];
      const uint64_t pairs = uint64_t(std::floor(c.coverage * double(L) / (double(s.R) * mates) * fraction));
      std::uniform_int_distribution<uint32_t> dstart(0, L - s.R);
      std::uniform_real_distribution<double> dunit(0.0, 1.0);
      std::uniform_int_distribution<uint32_t> dleaf(0, sd.leaves.empty() ? 0 : uint32_t(sd.leaves.size()) - 1);
      // copy slots: the largest copy number on the chromosome in any class
      uint32_t cn_chr = 1;
      if (pl.has_cna)
        for (const auto& g : pl.classes) {
          uint64_t unused = 0;
          uint32_t m = 0;
          copies_in(g, cs, ce, unused, m);
          cn_chr = std::max(cn_chr, m);
        }
      std::uniform_int_distribution<uint32_t> dallele(0, 1), dbase(0, 2), dslot(0, cn_chr - 1);
      std::binomial_distribution<uint32_t> dbin(bin_t, bin_p);
      std::normal_distribution<double> dnorm(double(c.insert_size_mean), double(c.insert_size_stddev));
      std::bernoulli_distribution derr(c.error_rate);
      uint32_t* alt = alt_t[w].data() + uint64_t(jb.smp) * M;
      uint32_t* dep = dep_t[w].data() + uint64_t(jb.smp) * M;
      for (uint64_t j = 0; j < pairs; ++j) {
        // (start, cell, allele instance) uniform over the DNA of the mixture:
        // with copy-number events by rejection over the whole chromosome
        // (copy slot u < cn_chr kept when the cell has more than u instances
        // at the start)
        uint32_t p0 = 0, allele = 0;
        int64_t cell = -1;
        bool found = false;
        for (uint32_t att = 0; att < (1u << 20) && !found; ++att) {
          p0 = cs + dstart(rng);
          const bool normal = sd.all_normal || dunit(rng) < 1.0 - c.purity;
          cell = normal ? -1 : int64_t(sd.leaves[dleaf(rng)]);
          if (!pl.has_cna) { allele = dallele(rng); found = true; break; }
          const uint32_t u = dslot(rng);
          const auto& cov = covering(pl.index[cell < 0 ? 0u : pl.node_class[cell]], p0);
          if (u < cov.size()) { allele = cov[u]; found = true; }
        }
        if (!found) continue;
        auto mate = [&](uint32_t a) {
          auto it = std::lower_bound(pl.locus.begin(), pl.locus.end(), a);
          for (size_t i = size_t(it - pl.locus.begin()); i < M && pl.locus[i] < a + s.R; ++i) {
            const auto& cs_i = carriers[i];
            const bool carried = car.ancestor_or_self(pl.edge[i], cell) &&
                                 std::find(cs_i.begin(), cs_i.end(), allele) != cs_i.end();
            bool obs;
            if (pl.kind[i] == 1) obs = carried;
            else {
              const bool err = c.error_rate > 0 && derr(rng);
              obs = carried ? !err : (err && dbase(rng) == 0);
            }
            dep[i] += 1;
            if (obs) alt[i] += 1;
          }
        };
        mate(p0);
        if (s.paired) {
          int64_t ins = c.insert_model == 0 ? int64_t(dbin(rng)) : int64_t(std::llround(dnorm(rng)));
          if (ins < int64_t(s.R)) ins = s.R;
          uint64_t p1 = uint64_t(p0) + uint64_t(ins) - s.R;
          if (p1 > ce - s.R) p1 = ce - s.R;
          mate(uint32_t(p1));
        }
      }
      reads += pairs * (s.paired ? 2 : 1);
    }
  };
  std::vector<std::thread> pool;
  for (int w = 1; w < nth; ++w) pool.emplace_back(worker, w);
  worker(0);
  for (auto& th : pool) th.join();
  for (int w = 0; w < nth; ++w)
    for (size_t i = 0; i < out.alt.size(); ++i) { out.alt[i] += alt_t[w][i]; out.depth[i] += dep_t[w][i]; }
  out.n_reads = reads;
}

}  // namespace orc

// ====================================================================== C-ABI for the tests
using namespace orc;

thread_local std::string orc_err;

extern "C" {

const char* orc_last_error() { return orc_err.c_str(); }

void orc_philox(uint32_t k0, uint32_t k1, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t* out) {
  const W4 r = philox(k0, k1, c0, c1, c2, c3);
  for (int i = 0; i < 4; ++i) out[i] = r.v[i];
}
double orc_log(double x) { return my_log(x); }
double orc_exp(double x) { return my_exp(x); }
double orc_log_factorial(double k) { return log_factorial(k); }
uint64_t orc_poisson(uint64_t seed, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t tag, double lambda) {
  Stream st = stream(seed, c0, c1, c2, tag);
  return poisson(st, lambda);
}
uint64_t orc_binomial(uint64_t seed, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t tag, uint64_t n, double p) {
  Stream st = stream(seed, c0, c1, c2, tag);
  return binomial(st, n, p);
}

void orc_genome_synth(uint64_t G, uint64_t seed, double gc, uint8_t* out) {
  double tt = gc * 4294967296.0;
  const uint32_t thr = tt >= 4294967295.0 ? 0xffffffffu : uint32_t(tt);
  for (uint64_t blk = 0; blk * 4 < G; ++blk) {
    const W4 r = philox(uint32_t(seed), uint32_t(seed >> 32), uint32_t(blk), uint32_t(blk >> 32), 0, TAG_GENOME);
    for (int j = 0; j < 4; ++j) {
      const uint64_t i = blk * 4 + j;
      if (i >= G) break;
      const uint32_t u = r.v[j];
      out[i] = uint8_t((u < thr) ? (1u + (u & 1u)) : ((u & 1u) ? 3u : 0u));
    }
  }
}

void* orc_engine_create(uint32_t n_chr, const uint32_t* chr_len, const uint8_t* bases, uint64_t seed, double gc,
                        uint32_t context_sampling, uint32_t max_rep) {
  try {
    auto e = new Engine();
    e->g.off.assign(n_chr + 1, 0);
    uint64_t G = 0;
    for (uint32_t c = 0; c < n_chr; ++c) { e->g.off[c] = uint32_t(G); G += chr_len[c]; }
    e->g.off[n_chr] = uint32_t(G);
    e->g.b.resize(G);
    if (bases) {   // codes above 3 (N and the other ambiguity codes) are unknown: 4
      for (uint64_t i = 0; i < G; ++i) e->g.b[i] = bases[i] > 3 ? uint8_t(4) : bases[i];
    }
    else orc_genome_synth(G, seed, gc, e->g.b.data());
    e->context_sampling = context_sampling;
    e->max_rep = max_rep;
    build_index(*e);
    return e;
  } catch (const std::exception& ex) { orc_err = ex.what(); return nullptr; }
}
void orc_engine_destroy(void* e) { delete static_cast<Engine*>(e); }
// regions to avoid (chromosome index, 1-based begin, length), then the
// indices again
void orc_engine_set_avoid(void* ep, uint32_t n, const uint32_t* chr, const uint32_t* begin, const uint32_t* len) {
  Engine& e = *static_cast<Engine*>(ep);
  e.avoid.assign(e.g.b.size(), 0);
  for (uint32_t i = 0; i < n; ++i)
    for (uint32_t q = 0; q < len[i]; ++q) e.avoid[e.g.off[chr[i]] + begin[i] - 1 + q] = 1;
  build_index(e);
}

void orc_engine_index_info(void* ep, uint64_t* ctx_total, uint64_t* id_total, uint32_t* ctx_len, uint32_t* id_len) {
  auto* e = static_cast<Engine*>(ep);
  for (int k = 0; k < 32; ++k) { ctx_total[k] = e->ctx_total[k]; ctx_len[k] = uint32_t(e->ctx[k].size()); }
  for (int k = 0; k < 83; ++k) { id_total[k] = e->id_total[k]; id_len[k] = uint32_t(e->id[k].size()); }
}
void orc_engine_read_index(void* ep, int which, uint32_t cls, uint32_t* out) {
  auto* e = static_cast<Engine*>(ep);
  const auto& v = which == 0 ? e->ctx[cls] : e->id[cls];
  std::copy(v.begin(), v.end(), out);
}
void orc_engine_read_genome(void* ep, uint8_t* out) {
  auto* e = static_cast<Engine*>(ep);
  std::copy(e->g.b.begin(), e->g.b.end(), out);
}
void orc_engine_set_signatures(void* ep, int type, uint32_t n, const double* probs) {
  auto* e = static_cast<Engine*>(ep);
  const uint32_t NC = type == 0 ? 96 : 83;
  e->n_sig[type] = n;
  e->sigs[type].assign(probs, probs + uint64_t(n) * NC);
  e->expo[type].clear();
}
void orc_engine_add_exposure(void* ep, int type, double time, const double* coeffs) {
  auto* e = static_cast<Engine*>(ep);
  e->expo[type][time] = std::vector<double>(coeffs, coeffs + e->n_sig[type]);
}
void orc_engine_set_species_rates(void* ep, uint32_t sp, double snv, double indel, double cna) {
  auto& s = static_cast<Engine*>(ep)->species[sp];
  s.snv = snv; s.indel = indel; s.cna = cna; s.has = true;
}
void orc_engine_set_species_epoch_rates(void* ep, uint32_t sp, uint32_t n, const double* snv, const double* indel) {
  auto& s = static_cast<Engine*>(ep)->species[sp];
  s.snv_e.assign(snv, snv + n); s.indel_e.assign(indel, indel + n); s.has = true;
}
void orc_engine_set_species_mutant(void* ep, uint32_t sp, uint32_t mutant) {
  static_cast<Engine*>(ep)->species[sp].mutant = mutant;
}
void orc_engine_add_driver_sid(void* ep, uint32_t mutant, uint32_t chr, uint32_t pos, const char* ref, const char* alt,
                               int32_t allele) {
  DriverEvent d{};
  d.kind = 0;
  d.sid = {chr, pos, ref, alt, allele};
  static_cast<Engine*>(ep)->drivers[mutant].push_back(d);
}
void orc_engine_add_driver_cna(void* ep, uint32_t mutant, int amp, uint32_t chr, uint32_t begin, uint32_t len,
                               int32_t allele, int32_t src) {
  DriverEvent d{};
  d.kind = 1;
  d.cna = {amp != 0, chr, begin, len, allele, src};
  static_cast<Engine*>(ep)->drivers[mutant].push_back(d);
}
void orc_engine_add_driver_wgd(void* ep, uint32_t mutant) {
  DriverEvent d{};
  d.kind = 2;
  static_cast<Engine*>(ep)->drivers[mutant].push_back(d);
}
void orc_engine_add_passenger_cna(void* ep, uint32_t chr, uint32_t begin, uint32_t len, int amp) {
  static_cast<Engine*>(ep)->cands.push_back({amp != 0, chr, begin, len, -1, -1});
}
void orc_engine_set_avoid_homozygous_losses(void* ep, int on) { static_cast<Engine*>(ep)->avoid_losses = on != 0; }
void orc_engine_set_infinite_sites(void* ep, int on) { static_cast<Engine*>(ep)->infinite_sites = on != 0; }

void* orc_place(void* ep, uint32_t n, const int32_t* parent, const double* birth, const uint32_t* species,
                const int32_t* sample, const uint32_t* divisions, uint32_t n_samples, uint32_t n_pre_snv,
                uint32_t pre_sbs, uint32_t n_pre_id, uint32_t pre_id, uint64_t seed, int flavour) {
  try {
    auto* e = static_cast<Engine*>(ep);
    auto* p = new Placed();
    Forest& f = p->forest_copy;
    f.n = n; f.n_samples = n_samples;
    f.parent.assign(parent, parent + n); f.birth.assign(birth, birth + n);
    f.species.assign(species, species + n); f.sample.assign(sample, sample + n);
    f.divisions.assign(n, 1);
    if (divisions) f.divisions.assign(divisions, divisions + n);
    f.is_leaf.assign(n, 1);
    for (uint32_t v = 0; v < n; ++v) if (f.parent[v] >= 0) f.is_leaf[f.parent[v]] = 0;
    f.leaves.assign(n_samples, {});
    for (uint32_t v = 0; v < n; ++v) if (f.is_leaf[v] && f.sample[v] >= 0) f.leaves[f.sample[v]].push_back(v);
    p->forest = &f;
    p->eng = e;
    if (flavour == 0) place_replay(*e, f, n_pre_snv, pre_sbs, n_pre_id, pre_id, seed, *p);
    else place_mt(*e, f, n_pre_snv, pre_sbs, n_pre_id, pre_id, seed, *p);
    return p;
  } catch (const std::exception& ex) { orc_err = ex.what(); return nullptr; }
}
void orc_placed_destroy(void* p) { delete static_cast<Placed*>(p); }
uint64_t orc_placed_count(void* pp) { return static_cast<Placed*>(pp)->locus.size(); }
void orc_placed_copy(void* pp, uint32_t* locus, uint32_t* edge, uint32_t* aux, uint8_t* cls, uint8_t* sig,
                     uint16_t* allele, uint8_t* kind, uint8_t* nature) {
  auto* p = static_cast<Placed*>(pp);
  const size_t n = p->locus.size();
  if (locus) std::copy(p->locus.begin(), p->locus.end(), locus);
  if (edge) std::copy(p->edge.begin(), p->edge.end(), edge);
  if (aux) std::copy(p->aux.begin(), p->aux.end(), aux);
  if (cls) std::copy(p->cls.begin(), p->cls.end(), cls);
  if (sig) std::copy(p->sig.begin(), p->sig.end(), sig);
  if (allele) std::copy(p->allele.begin(), p->allele.end(), allele);
  if (kind) std::copy(p->kind.begin(), p->kind.end(), kind);
  if (nature) std::copy(p->nature.begin(), p->nature.end(), nature);
  (void)n;
}
// Replace the placed mutations of a table without copy-number events (used
// to sequence the same table the GPU placed)
int orc_placed_set(void* pp, uint64_t n, const uint32_t* locus, const uint32_t* edge, const uint16_t* allele,
                   const uint8_t* kind) {
  auto* p = static_cast<Placed*>(pp);
  if (p->has_cna) { orc_err = "orc_placed_set: the table has copy-number events"; return 1; }
  p->locus.assign(locus, locus + n); p->edge.assign(edge, edge + n);
  p->allele.assign(allele, allele + n); p->kind.assign(kind, kind + n);
  p->aux.assign(n, 0); p->cls.assign(n, 0); p->sig.assign(n, 0); p->nature.assign(n, 0);
  p->order.assign(n, 0);
  for (uint64_t i = 0; i < n; ++i) p->order[i] = edge[i] >= p->forest->n ? -1 : INT32_MAX;
  return 0;
}
uint64_t orc_placed_cna_count(void* pp) { return static_cast<Placed*>(pp)->cnas.size(); }
void orc_placed_cna_copy(void* pp, uint32_t* node, uint8_t* type, uint32_t* chr, uint32_t* begin, uint32_t* end,
                         uint32_t* allele, uint32_t* src, uint8_t* driver) {
  const auto& c = static_cast<Placed*>(pp)->cnas;
  for (size_t i = 0; i < c.size(); ++i) {
    node[i] = c[i].node; type[i] = c[i].type; chr[i] = c[i].chr; begin[i] = c[i].begin; end[i] = c[i].end;
    allele[i] = c[i].allele; src[i] = c[i].src; driver[i] = c[i].driver;
  }
}
// pieces (instance, [b, e)) of class c, and the germline allele of every instance
uint64_t orc_placed_class_pieces(void* pp, uint32_t c, uint32_t* inst, uint32_t* b, uint32_t* e) {
  auto* p = static_cast<Placed*>(pp);
  uint64_t n = 0;
  for (const auto& kv : p->classes[c])
    for (auto [x, y] : kv.second) {
      if (inst) { inst[n] = kv.first; b[n] = x; e[n] = y; }
      ++n;
    }
  return n;
}
// carrier instances of every placed mutation (carrier_sets): off has M + 1
// entries; returns the total (list may be NULL to size it)
uint64_t orc_placed_carriers(void* pp, uint32_t* off, uint32_t* list) {
  auto* p = static_cast<Placed*>(pp);
  const auto cs = carrier_sets(*p);
  uint64_t n = 0;
  for (size_t i = 0; i < cs.size(); ++i) {
    if (off) off[i] = uint32_t(n);
    for (uint32_t y : cs[i]) { if (list) list[n] = y; ++n; }
  }
  if (off) off[cs.size()] = uint32_t(n);
  return n;
}
uint32_t orc_placed_inst_roots(void* pp, uint8_t* root) {
  auto* p = static_cast<Placed*>(pp);
  std::vector<uint32_t> from(p->n_inst);
  for (uint32_t y = 0; y < p->n_inst; ++y) from[y] = y;
  for (const CopyRec& c : p->copies) from[c.made] = c.from;
  for (uint32_t y = 0; y < p->n_inst && root; ++y) {
    uint32_t r = y;
    while (from[r] != r) r = from[r];
    root[y] = uint8_t(r);
  }
  return p->n_inst;
}
// node classes (n nodes), number of classes, largest copy number
void orc_placed_node_classes(void* pp, uint32_t* node_class, uint32_t* n_classes, uint32_t* cn_max) {
  auto* p = static_cast<Placed*>(pp);
  if (node_class) std::copy(p->node_class.begin(), p->node_class.begin() + p->forest->n, node_class);
  if (n_classes) *n_classes = uint32_t(p->classes.size());
  if (cn_max) *cn_max = p->cn_max;
}

void* orc_seq(void* pp, const void* cfg, uint64_t seed, int flavour, double fraction, int threads) {
  try {
    auto* p = static_cast<Placed*>(pp);
    const SeqCfg& c = *static_cast<const SeqCfg*>(cfg);
    auto* o = new SeqOut();
    if (flavour == 0) seq_replay(*p, c, seed, *o);
    else seq_mt(*p, c, seed, fraction, threads, *o);
    return o;
  } catch (const std::exception& ex) { orc_err = ex.what(); return nullptr; }
}
// the replay's SAM reads as text, one line per read in the order of the
// SAM files (per chromosome and sample: tiles, fragments, mates): sample,
// chromosome index, FLAG, POS, CIGAR, mate POS, TLEN, SEQ (1-based positions
// within the chromosome; "*" fields for a read without DNA)
int orc_sam(void* pp, const void* cfg, uint64_t seed, const char* path) {
  try {
    const Placed& pl = *static_cast<Placed*>(pp);
    const SeqCfg& c = *static_cast<const SeqCfg*>(cfg);
    const Engine& e = *pl.eng;
    const SeqSetup s = seq_setup(pl, c);
    Carrier car{*pl.forest, c.preneoplastic_in_normal != 0};
    const auto carriers = carrier_sets(pl);
    std::ofstream f(path);
    if (!f) throw std::runtime_error("cannot write the expected reads");
    const uint32_t R = s.R;
    FragmentVisitor v = [&](uint32_t smp, uint32_t ci, bool dropped, uint32_t p0, uint32_t p1, int64_t cell,
                            uint32_t allele, uint32_t fw) {
      const uint32_t off = e.g.off[ci], ce = e.g.off[ci + 1];
      for (uint32_t m = 0; m < (s.paired ? 2u : 1u); ++m) {
        f << smp << '\t' << ci << '\t';
        if (dropped) { f << "4\t*\t*\t*\t*\t*\n"; continue; }
        const uint32_t p = m ? p1 : p0;
        const OracleRead rd = oracle_read(pl, car, carriers, pl.aux, p, ce, cell, allele, fw, m, R, s.err_thr);
        const uint32_t flag = s.paired ? (0x1u | 0x2u | (m ? (0x80u | 0x10u) : (0x40u | 0x20u))) : 0u;
        f << flag << '\t' << (p - off + 1) << '\t';
        for (const auto& [op, len] : rd.cigar) f << len << op;
        if (rd.cigar.empty()) f << '*';
        if (s.paired) {
          const int64_t span = int64_t(p1) + R - p0;
          f << '\t' << ((m ? p0 : p1) - off + 1) << '\t' << (m ? -span : span);
        } else {
          f << "\t0\t0";
        }
        f << '\t' << rd.seq << '\n';
      }
    };
    SeqOut out;
    seq_replay(pl, c, seed, out, &v);
    return 0;
  } catch (const std::exception& ex) { orc_err = ex.what(); return 1; }
}

void orc_seq_destroy(void* o) { delete static_cast<SeqOut*>(o); }
uint32_t orc_seq_samples(void* o) { return static_cast<SeqOut*>(o)->n_samples; }
uint64_t orc_seq_reads(void* o) { return static_cast<SeqOut*>(o)->n_reads; }
void orc_seq_copy(void* op, int32_t* alt, int32_t* depth) {
  auto* o = static_cast<SeqOut*>(op);
  for (size_t i = 0; i < o->alt.size(); ++i) { alt[i] = int32_t(o->alt[i]); depth[i] = int32_t(o->depth[i]); }
}

}  // extern "C"
