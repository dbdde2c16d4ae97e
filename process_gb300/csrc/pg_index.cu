// Genome storage and the two site indices the placement kernels draw from.
//
// Reference behaviour (ProCESS wrapper, RACES internals absent):
//   * ContextIndex<uint32_t>::build_index(ref, regions_to_avoid, context_sampling)
//     (src/mutation_engine.cpp:211-275, call :260): positions of the reference
//     grouped by pyrimidine-centred trinucleotide context, one kept in every
//     `context_sampling` occurrences (default 100, src/mutations.cpp:945-949).
//   * RSIndex::build_index(ref, max_motif_size, max_repetition_storage)
//     (src/mutation_engine.cpp:289-359, call :344): positions of repeated
//     sequences per ID class, at most `max_repetition_storage` per class.
//
// Here both are position lists in HBM, u32 absolute positions sorted
// ascending within each class, built in two streaming passes over the 2-bit
// genome: (1) per 4096-base unit, per class counts; (2) after a scan over
// the units, every warp walks its unit again and writes the positions whose
// rank within their class is a multiple of the class stride.  Positions are
// classified 32 at a time per lane as bit masks (one per class), counted
// with popcounts and warp reductions and numbered by a lane prefix sum, so
// the lists come out in position order without any sort.
#include <mutex>

#include "pg_common.cuh"
#include "pg_rng.cuh"
#include "pg_scan.cuh"
#include "pg_kernels.h"

namespace pg {


// ------------------------------------------------------------ genome fill
__global__ void k_genome_synth(uint32_t* __restrict__ words, uint64_t G, uint64_t nwords,
                               Key key, uint32_t gc_thr) {
  const uint64_t w = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (w >= nwords) return;
  uint32_t out = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const uint64_t blk = w * 4 + q;               // Philox block = 4 bases
    const U4 r = philox(key.k0, key.k1, uint32_t(blk), uint32_t(blk >> 32), 0u, TAG_GENOME);
    const uint32_t rw[4] = {r.x, r.y, r.z, r.w};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const uint64_t i = blk * 4 + j;
      if (i < G) {
        const uint32_t u = rw[j];
        // GC with probability gc_thr/2^32, then C/G or A/T by the low bit
        const uint32_t b = (u < gc_thr) ? (1u + (u & 1u)) : ((u & 1u) ? 3u : 0u);
        out |= b << (2 * (q * 4 + j));
      }
    }
  }
  words[w] = out;
}

__global__ void k_genome_pack(uint32_t* __restrict__ words, const uint8_t* __restrict__ codes,
                              uint64_t G, uint64_t nwords) {
  const uint64_t w = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (w >= nwords) return;
  uint32_t out = 0;
  for (int j = 0; j < 16; ++j) {
    const uint64_t i = w * 16 + j;
    if (i < G) out |= uint32_t(codes[i] & 3u) << (2 * j);
  }
  words[w] = out;
}

// unknown bases (N) are bits of nmask (NULL: none), one bit per position
__device__ __forceinline__ bool base_unknown(const uint32_t* __restrict__ nmask, uint64_t q) {
  return nmask && ((__ldg(nmask + (q >> 5)) >> (q & 31u)) & 1u);
}

// ------------------------------------------------------------ class families
// Both indices classify every position of the genome from the bases around
// it.  A lane classifies 32 consecutive positions at once with bit masks
// (bit i for position base + i): the bases as two bit planes (the low and
// the high bit of the 2-bit code), a validity plane (known bases of the
// position's chromosome), and from these one mask per class.  Features are
// computed on 64-bit windows (bit j = position q0 + j, q0 = base - 16 or
// base) whose bits 16..31 are the window's 16 positions; classes are
// bitwise functions of the features, so the two windows' features are
// packed side by side into 32-bit position masks first.
struct Planes {
  uint64_t p0, p1;   // low and high bit of each base
  uint64_t v;        // known base inside the position's chromosome
};

__device__ __forceinline__ uint64_t eq_shift(const Planes& w, int s) {   // base(j) == base(j + s), both valid
  return w.v & (w.v >> s) & ~((w.p0 ^ (w.p0 >> s)) | (w.p1 ^ (w.p1 >> s)));
}

__device__ __forceinline__ uint32_t pos16(uint64_t x) { return uint32_t(x >> 16) & 0xFFFFu; }

// SBS: one family, the pyrimidine-centred trinucleotide context of p (p - 1,
// p and p + 1 known and in p's chromosome; p not in a region to avoid).
// Context s*16 + a*4 + c: a forward-strand centre C (s 0) or T (s 1) with
// 5' base a and 3' base c, or a reverse-strand centre G (s 0) or A (s 1)
// whose complemented flanks read a, c on the pyrimidine strand.
struct SbsFamilies {
  static constexpr int NC = N_CTX;
  static constexpr int NF = 7;
  static constexpr bool AVOIDABLE = true;    // positions of the regions to avoid are not indexed
  // features: 0 indexable; 1, 2 planes of p - 1; 3, 4 of p; 5, 6 of p + 1
  __device__ static void features(const Planes& w, uint64_t avoid, uint32_t* f, uint32_t keep, int sh) {
    f[0] |= (pos16(w.v & (w.v << 1) & (w.v >> 1) & ~avoid) << sh) & keep;
    f[1] |= (pos16(w.p0 << 1) << sh) & keep;
    f[2] |= (pos16(w.p1 << 1) << sh) & keep;
    f[3] |= (pos16(w.p0) << sh) & keep;
    f[4] |= (pos16(w.p1) << sh) & keep;
    f[5] |= (pos16(w.p0 >> 1) << sh) & keep;
    f[6] |= (pos16(w.p1 >> 1) << sh) & keep;
  }
  template <class Sink>
  __device__ static void classes(const uint32_t* f, Sink sink) {
    const uint32_t ok = f[0];
    // forward centre C (s 0), T (s 1); reverse centre G (-> C), A (-> T)
    auto cen = [&](int s) { return s ? (f[3] & f[4]) : (f[3] & ~f[4]); };
    auto rev = [&](int s) { return s ? (~f[3] & ~f[4]) : (~f[3] & f[4]); };
    // base at p - 1 (x) / p + 1 (z) equal to b
    auto ex = [&](int b) { return ((b & 1) ? f[1] : ~f[1]) & ((b & 2) ? f[2] : ~f[2]); };
    auto ez = [&](int b) { return ((b & 1) ? f[5] : ~f[5]) & ((b & 2) ? f[6] : ~f[6]); };
#pragma unroll
    for (int s = 0; s < 2; ++s)
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int c = 0; c < 4; ++c)
          sink(s * 16 + a * 4 + c, ok & ((cen(s) & ex(a) & ez(c)) | (rev(s) & ez(3 - a) & ex(3 - c))));
  }
};

// ID83 (COSMIC order).  A position p (the first deleted base, or the base
// before which bases are inserted; p-1 is the anchor, and both are known)
// belongs to at most one class per family:
//   F0  1-bp deletion at a homopolymer run start, run length h 1..6+  (0-11)
//   F1  1-bp insertion at a run start, run length 1..5+               (12-23, idx 1-5)
//   F2  1-bp C/G insertion with no adjacent C/G                       (12)
//   F3  1-bp T/A insertion with no adjacent T/A                       (18)
//   F4-7  l=2..5 deletion of the unit starting a repeat tract: repeat
//         count r>=2 -> 24+(l-2)*6+min(r-1,5); r==1 -> microhomology
//         m = common prefix of the unit and the following l bases:
//         m==0 -> 24+(l-2)*6, else 72+off(l)+m-1
//   F8-11 l=2..5 insertion of one more unit at a tract start, r>=1   (48+(l-2)*6+min(r,5))
//   F12-15 l=2..5 insertion of l random bases at a run start          (48+(l-2)*6)
// The l-families need p..p+l-1 known and p not inside a tract (the l bases
// before p differ from the unit).  With E_l(q) = base(q) == base(q + l),
// both known: the run length from p is h >= k+1 iff E_1 holds at p..p+k-1;
// the repeat count r >= k+1 iff E_l holds at p..p+kl-1 (capped at 6); the
// microhomology m >= j iff E_l holds at p..p+j-1; "inside a tract" iff E_l
// holds at p-l..p-1.
struct IdFamilies {
  static constexpr int NC = N_ID;
  static constexpr int NF = 43;
  static constexpr bool AVOIDABLE = false;
  // features: 0 p and p-1 known; 1 run start; 2, 3 base of p / p-1 is A or T;
  // 4..8 h >= 2..6; then per l = 2..5: the family applies, r >= 2..6, m >= 1..l-1
  __device__ static void features(const Planes& w, uint64_t, uint32_t* f, uint32_t keep, int sh) {
    auto put = [&](int x, uint64_t m) { f[x] |= (pos16(m) << sh) & keep; };
    const uint64_t v = w.v, e1 = eq_shift(w, 1), bv = v & (v << 1), pt = ~(w.p0 ^ w.p1);
    put(0, bv);
    put(1, bv & ~(e1 << 1));
    put(2, pt);
    put(3, pt << 1);
    uint64_t h = e1;
    put(4, h);
#pragma unroll
    for (int k = 1; k <= 4; ++k) { h &= e1 >> k; put(4 + k, h); }
    int o = 9;
#pragma unroll
    for (int l = 2; l <= 5; ++l) {
      const uint64_t el = eq_shift(w, l);
      uint64_t vl = v, u = el, sb = el << 1;
#pragma unroll
      for (int i = 1; i < l; ++i) { vl &= v >> i; u &= el >> i; sb &= el << (i + 1); }
      put(o, bv & vl & ~sb);
      uint64_t r = u;
      put(o + 1, r);
#pragma unroll
      for (int q = 2; q <= 5; ++q) { r &= u >> ((q - 1) * l); put(o + q, r); }
      uint64_t m = el;
      put(o + 6, m);
#pragma unroll
      for (int j = 2; j < l; ++j) { m &= el >> (j - 1); put(o + 5 + j, m); }
      o += 5 + l;
    }
  }
  template <class Sink>
  __device__ static void classes(const uint32_t* f, Sink sink) {
    const uint32_t bv = f[0], rs = f[1], pt = f[2], ptp = f[3];
    const uint32_t hx[7] = {0u, ~f[4], f[4] & ~f[5], f[5] & ~f[6], f[6] & ~f[7], f[7] & ~f[8], f[8]};  // h exactly
#pragma unroll
    for (int c = 0; c < 12; ++c) sink(c, rs & (c >= 6 ? pt : ~pt) & hx[c % 6 + 1]);
#pragma unroll
    for (int py = 0; py < 2; ++py)
#pragma unroll
      for (int j = 1; j <= 5; ++j) sink(12 + py * 6 + j, rs & (py ? pt : ~pt) & (j < 5 ? hx[j] : f[7]));
    sink(12, bv & pt & ptp);
    sink(18, bv & ~pt & ~ptp);
    sink(48, rs); sink(54, rs); sink(60, rs); sink(66, rs);
    constexpr int mh_off[4] = {0, 1, 3, 6};
    int o = 9;
#pragma unroll
    for (int l = 2; l <= 5; ++l) {
      const uint32_t val = f[o], r2 = f[o + 1], r3 = f[o + 2], r4 = f[o + 3], r5 = f[o + 4], r6 = f[o + 5];
      const int b4 = 24 + (l - 2) * 6, b8 = 48 + (l - 2) * 6;
      const uint32_t x2 = val & r2 & ~r3, x3 = val & r3 & ~r4, x4 = val & r4 & ~r5, nr = val & ~r2;
      sink(b4 + 1, x2); sink(b4 + 2, x3); sink(b4 + 3, x4); sink(b4 + 4, val & r5 & ~r6); sink(b4 + 5, val & r6);
      sink(b4, nr & ~f[o + 6]);
#pragma unroll
      for (int j = 1; j < l; ++j) sink(72 + mh_off[l - 2] + j - 1, nr & f[o + 5 + j] & (j + 1 < l ? ~f[o + 6 + j] : ~0u));
      sink(b8 + 1, nr); sink(b8 + 2, x2); sink(b8 + 3, x3); sink(b8 + 4, x4); sink(b8 + 5, val & r5);
      o += 5 + l;
    }
  }
};

// ------------------------------------------------------------ index scans
// A lane takes 32 positions per round, a warp 32 lanes (1024 positions) per
// round and IX_ROUNDS rounds per unit; the count pass writes one count per
// (class, unit), and the emit pass, after a scan of that table over the
// units, numbers each class's positions in order: units in order, within a
// unit the rounds, within a round the lanes, within a lane the positions.
// Position p is written to its class's list when its number is a multiple
// of the class stride.
constexpr uint32_t IX_LANE_POS = 32;
constexpr uint32_t IX_ROUNDS = 4;
constexpr uint32_t IX_UNIT = 32 * IX_LANE_POS * IX_ROUNDS;   // 4096 positions
constexpr int IX_WARPS = 8;

// bit index of the n-th (from 0) set bit of m, n < popc(m): halving steps
// on popcounts, without a data-dependent loop
__device__ __forceinline__ uint32_t nth_set_bit(uint32_t m, uint32_t n) {
  uint32_t pos = 0;
#pragma unroll
  for (uint32_t w = 16; w >= 1; w >>= 1) {
    const uint32_t c = __popc(m & ((1u << w) - 1u));
    const bool up = n >= c;
    n = up ? n - c : n;
    pos = up ? pos + w : pos;
    m = up ? m >> w : m;
  }
  return pos;
}

// even bits of x to the low half, odd bits to the high half (an inverse
// perfect shuffle in four swap steps)
__device__ __forceinline__ uint32_t unshuffle32(uint32_t x) {
  uint32_t t = (x ^ (x >> 1)) & 0x22222222u; x ^= t ^ (t << 1);
  t = (x ^ (x >> 2)) & 0x0C0C0C0Cu; x ^= t ^ (t << 2);
  t = (x ^ (x >> 4)) & 0x00F000F0u; x ^= t ^ (t << 4);
  t = (x ^ (x >> 8)) & 0x0000FF00u; x ^= t ^ (t << 8);
  return x;
}

// bits [lo, hi) of a 64-bit window, clamped to the window
__device__ __forceinline__ uint64_t range_bits(int64_t lo, int64_t hi) {
  lo = lo < 0 ? 0 : lo;
  hi = hi > 64 ? 64 : hi;
  if (hi <= lo) return 0;
  const uint64_t top = hi >= 64 ? ~0ull : ((1ull << hi) - 1ull);
  return top & ~((1ull << lo) - 1ull);
}

// unknown base (N) masks and the like: 1 bit per position, bit q % 32 of word q / 32
__device__ __forceinline__ uint32_t mask_word(const uint32_t* __restrict__ m, int64_t wi, uint64_t nw) {
  return (m && wi >= 0 && uint64_t(wi) < nw) ? __ldg(m + wi) : 0u;
}

// warps per block: the emit pass keeps per warp the round's lane masks of
// the classes that write (shared memory), so its blocks are smaller
__host__ __device__ constexpr int ix_warps(int mode) { return mode == 0 ? IX_WARPS : IX_WARPS / 2; }

template <class F, int MODE>
__global__ void __launch_bounds__(32 * ix_warps(MODE)) k_index_scan(const uint32_t* __restrict__ g,
                                                                   const uint32_t* __restrict__ nmask,
                                                                   const uint32_t* __restrict__ amask, uint64_t G,
                                                                   const uint32_t* __restrict__ chr_off, int n_chr,
                                                                   uint32_t n_units, uint32_t* __restrict__ cnt,
                                                                   const uint32_t* __restrict__ stride,
                                                                   const uint64_t* __restrict__ list_off,
                                                                   const uint32_t* __restrict__ list_len,
                                                                   uint32_t* __restrict__ lists) {
  constexpr int NS = (F::NC + 31) / 32;
  constexpr uint32_t FULL = 0xffffffffu;
  constexpr int W = ix_warps(MODE);
  static_assert(MODE != 2 || F::NC == 32, "the every-position emit is for the 32 SBS contexts");
  constexpr int SN = MODE >= 1 ? F::NC : 1;
  constexpr int QW = MODE == 1 ? W : 1, QN = MODE == 1 ? F::NC : 1;
  constexpr int PW = MODE == 2 ? W : 1, PN = MODE == 2 ? 32 : 1, PB = MODE == 2 ? 32 * IX_LANE_POS : 1;
  __shared__ uint32_t s_stride[SN], s_len[SN];
  __shared__ uint64_t s_off[SN];
  // MODE 1, per warp: the classes of the round with a position to write
  // (class | hits << 8) and their lane masks; per class the hits before its
  // next written position and that position's index in the class list
  __shared__ uint32_t s_qk[QW][QN], s_qmask[QW][QN][32];
  __shared__ uint32_t s_dist[QW][QN], s_kidx[QW][QN];
  // MODE 2 (every position written), per warp: the round's positions grouped
  // by class (class runs in class order, in position order within a run), per
  // class and lane the lane's next slot in the run, per class the run's start,
  // its first list index and the next round's
  __shared__ uint32_t s_ppos[PW][PN][32], s_pbuf[PW][PB];
  __shared__ uint8_t s_pcls[PW][PB];
  __shared__ uint32_t s_prun[PW][PN], s_plist[PW][PN], s_pnext[PW][PN];
  if (MODE >= 1) {
    for (int k = threadIdx.x; k < F::NC; k += blockDim.x) {
      s_stride[k] = stride[k];
      s_len[k] = list_len[k];
      s_off[k] = list_off[k];
    }
    __syncthreads();
  }
  const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint32_t unit = blockIdx.x * W + w;
  if (unit >= n_units) return;
  // MODE 0: per class k the count, held by lane k % 32 in slot k / 32
  uint32_t run[NS];
#pragma unroll
  for (int s = 0; s < NS; ++s) run[s] = 0;
  if (MODE == 1) {
    for (uint32_t k = lane; k < uint32_t(F::NC); k += 32) {
      const uint32_t r0 = cnt[uint64_t(k) * n_units + unit], sd = s_stride[k];
      const uint32_t q = r0 / sd, rem = r0 - q * sd;
      s_dist[MODE == 1 ? w : 0][k] = rem ? sd - rem : 0u;
      s_kidx[MODE == 1 ? w : 0][k] = q + (rem ? 1u : 0u);
    }
    __syncwarp();
  }
  const uint32_t qw = MODE == 1 ? w : 0, pw = MODE == 2 ? w : 0;
  if (MODE == 2) {
    s_pnext[pw][lane] = cnt[uint64_t(lane) * n_units + unit];
    __syncwarp();
  }
  const uint64_t n_gw = (G + 15) / 16, n_mw = (G + 31) / 32;
  for (uint32_t round = 0; round < IX_ROUNDS; ++round) {
    const uint64_t wbase = uint64_t(unit) * IX_UNIT + uint64_t(round) * (32 * IX_LANE_POS);
    if (wbase >= G) break;
    const uint64_t base = wbase + uint64_t(lane) * IX_LANE_POS;
    uint32_t f[F::NF];
#pragma unroll
    for (int x = 0; x < F::NF; ++x) f[x] = 0;
    if (base < G) {
      // bases [base - 16, base + 64) as bit planes, 16 positions per half word
      uint32_t lo[5], hi[5];
#pragma unroll
      for (int i = 0; i < 5; ++i) {
        const int64_t wi = int64_t(base >> 4) - 1 + i;
        const uint32_t u = unshuffle32((wi >= 0 && uint64_t(wi) < n_gw) ? __ldg(g + wi) : 0u);
        lo[i] = u & 0xFFFFu;
        hi[i] = u >> 16;
      }
      uint32_t nw[3], aw[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const int64_t wi = int64_t(base >> 5) - 1 + i;
        nw[i] = mask_word(nmask, wi, n_mw);
        aw[i] = F::AVOIDABLE ? mask_word(amask, wi, n_mw) : 0u;
      }
      // chromosome of base: the largest c with chr_off[c] <= base
      int c = 0;
      {
        int lo_c = 0, hi_c = n_chr;
        while (hi_c - lo_c > 1) {
          const int mid = (lo_c + hi_c) >> 1;
          if (__ldg(chr_off + mid) <= base) lo_c = mid; else hi_c = mid;
        }
        c = lo_c;
      }
      // one segment per chromosome that holds some of the lane's positions
      for (; c < n_chr; ++c) {
        const uint64_t cs = __ldg(chr_off + c), ce = __ldg(chr_off + c + 1);
        if (cs >= base + IX_LANE_POS) break;
        if (ce <= base) continue;
        const uint32_t keep = uint32_t(range_bits(int64_t(cs) - int64_t(base), int64_t(ce) - int64_t(base)));
#pragma unroll
        for (int half = 0; half < 2; ++half) {
          const int64_t q0 = int64_t(base) - 16 + 16 * half;
          Planes wd;
          wd.p0 = uint64_t(lo[half]) | (uint64_t(lo[half + 1]) << 16) | (uint64_t(lo[half + 2]) << 32) |
                  (uint64_t(lo[half + 3]) << 48);
          wd.p1 = uint64_t(hi[half]) | (uint64_t(hi[half + 1]) << 16) | (uint64_t(hi[half + 2]) << 32) |
                  (uint64_t(hi[half + 3]) << 48);
          const uint64_t nm = half == 0 ? (uint64_t(nw[0] >> 16) | (uint64_t(nw[1]) << 16) | (uint64_t(nw[2]) << 48))
                                        : (uint64_t(nw[1]) | (uint64_t(nw[2]) << 32));
          const uint64_t am = half == 0 ? (uint64_t(aw[0] >> 16) | (uint64_t(aw[1]) << 16) | (uint64_t(aw[2]) << 48))
                                        : (uint64_t(aw[1]) | (uint64_t(aw[2]) << 32));
          wd.v = ~nm & range_bits(int64_t(cs) - q0, int64_t(ce) - q0);
          F::features(wd, am, f, keep, 16 * half);
        }
      }
    }
    uint32_t nq = 0, tk = 0;
    F::classes(f, [&](int k, uint32_t m) {
      if constexpr (MODE == 2) {
        // the lane's first slot in the class's run, and the run's length (held by lane k)
        const uint32_t c = __popc(m);
        uint32_t incl = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t y = __shfl_up_sync(FULL, incl, o);
          if (lane >= uint32_t(o)) incl += y;
        }
        s_ppos[pw][k][lane] = incl - c;
        const uint32_t t = __shfl_sync(FULL, incl, 31);
        if (lane == uint32_t(k)) tk = t;
        return;
      }
      const uint32_t t = __reduce_add_sync(FULL, uint32_t(__popc(m)));
      if constexpr (MODE == 0) {
        if (lane == (uint32_t(k) & 31u)) run[k >> 5] += t;
      } else {
        if (t == 0) return;
        const uint32_t d = s_dist[qw][k];                   // hits before the next written one
        if (t <= d) {
          if (lane == 0) s_dist[qw][k] = d - t;
          return;
        }
        s_qmask[qw][nq][lane] = m;
        if (lane == 0) s_qk[qw][nq] = uint32_t(k) | (t << 8);
        ++nq;
      }
    });
    if constexpr (MODE == 2) {
      // class runs in class order: lane k holds class k's run length tk
      uint32_t incl = tk;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(FULL, incl, o);
        if (lane >= uint32_t(o)) incl += y;
      }
      const uint32_t tot = __shfl_sync(FULL, incl, 31);
      s_prun[pw][lane] = incl - tk;
      s_plist[pw][lane] = s_pnext[pw][lane];
      s_pnext[pw][lane] += tk;
      __syncwarp();
      // each lane's positions into their class runs, in position order
      const uint32_t ok = f[0];
#pragma unroll 4
      for (uint32_t i = 0; i < IX_LANE_POS; ++i) {
        if ((ok >> i) & 1u) {
          const uint32_t x = ((f[1] >> i) & 1u) | (((f[2] >> i) & 1u) << 1);
          const uint32_t y0 = (f[3] >> i) & 1u, y1 = (f[4] >> i) & 1u;
          const uint32_t z = ((f[5] >> i) & 1u) | (((f[6] >> i) & 1u) << 1);
          // the context as SbsFamilies::classes numbers it
          const uint32_t k = y0 ? ((y1 << 4) | (x << 2) | z) : (((y1 ^ 1u) << 4) | ((3u - z) << 2) | (3u - x));
          const uint32_t slot = s_prun[pw][k] + s_ppos[pw][k][lane]++;
          s_pbuf[pw][slot] = uint32_t(base) + i;
          s_pcls[pw][slot] = uint8_t(k);
        }
      }
      __syncwarp();
      // the runs to the class lists, consecutive lanes to consecutive entries
      for (uint32_t e = lane; e < tot; e += 32) {
        const uint32_t k = s_pcls[pw][e];
        const uint32_t idx = s_plist[pw][k] + (e - s_prun[pw][k]);
        if (idx < s_len[k]) lists[s_off[k] + idx] = s_pbuf[pw][e];
      }
      __syncwarp();
    }
    if constexpr (MODE == 1) {
      __syncwarp();
      // the classes that write a position this round (one copy of the code)
      for (uint32_t qi = 0; qi < nq; ++qi) {
        const uint32_t qk = s_qk[qw][qi], k = qk & 0xffu, t = qk >> 8;
        const uint32_t m = s_qmask[qw][qi][lane], c = __popc(m);
        const uint32_t d = s_dist[qw][k], ki = s_kidx[qw][k], sd = s_stride[k];
        // hit numbers and their gaps within a round are below 1024 (32 lanes
        // x 32 positions): every quotient below is of a number < 1024
        uint32_t incl = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t y = __shfl_up_sync(FULL, incl, o);
          if (lane >= uint32_t(o)) incl += y;
        }
        const uint32_t ex = incl - c;                          // the lane's hits are numbered ex .. ex + c - 1
        uint32_t hit = d, idx = ki;                            // the lane's first written hit and its index
        if (ex > d) {
          const uint32_t gap = ex - d;
          const uint32_t q = gap <= sd ? 1u : (gap + sd - 1u) / sd;
          idx = ki + q;
          hit = (uint64_t(d) + uint64_t(q) * sd >= uint64_t(ex) + c) ? ex + c : d + q * sd;
        }
        if (hit < ex + c) {
          // the lane's written hits have ranks r, r + sd, ... (< c) among its set bits
          const uint32_t len = s_len[k];
          const uint64_t off = s_off[k];
          for (uint32_t r = hit - ex;; r += sd, ++idx) {
            if (idx < len) lists[off + idx] = uint32_t(base + nth_set_bit(m, r));
            if (sd >= c - r) break;
          }
        }
        if (lane == 0) {
          const uint32_t span = t - 1u - d;                    // hits after the first written one
          const uint32_t nk = (span < sd ? 0u : span / sd) + 1u;   // written this round
          s_dist[qw][k] = uint32_t(uint64_t(d) + uint64_t(nk) * sd - t);
          s_kidx[qw][k] = ki + nk;
        }
        __syncwarp();
      }
    }
  }
  if (MODE == 0) {
#pragma unroll
    for (int s = 0; s < NS; ++s) {
      const uint32_t k = s * 32 + lane;
      if (k < uint32_t(F::NC)) cnt[uint64_t(k) * n_units + unit] = run[s];
    }
  }
}

// ------------------------------------------------------------ host side
void genome_synth(uint32_t* words, uint64_t G, uint64_t seed, double gc, cudaStream_t st) {
  const uint64_t nwords = (G + 15) / 16;
  double t = gc * 4294967296.0;
  uint32_t thr = t >= 4294967295.0 ? 0xffffffffu : uint32_t(t);
  k_genome_synth<<<unsigned((nwords + 255) / 256), 256, 0, st>>>(words, G, nwords, make_key(seed), thr); note_launch();
}

void genome_pack(uint32_t* words, const uint8_t* codes, uint64_t G, cudaStream_t st) {
  const uint64_t nwords = (G + 15) / 16;
  k_genome_pack<<<unsigned((nwords + 255) / 256), 256, 0, st>>>(words, codes, G, nwords); note_launch();
}

uint32_t index_num_tiles(uint64_t G) { return uint32_t((G + IX_UNIT - 1) / IX_UNIT); }

template <class F>
static void index_count_t(const uint32_t* g, const uint32_t* nmask, const uint32_t* amask, uint64_t G,
                          const uint32_t* chr_off, int n_chr, uint32_t* cnt, uint32_t* part, uint32_t* totals,
                          cudaStream_t st) {
  const uint32_t ntiles = index_num_tiles(G);
  k_index_scan<F, 0><<<(ntiles + IX_WARPS - 1) / IX_WARPS, 256, 0, st>>>(g, nmask, amask, G, chr_off, n_chr, ntiles,
                                                                        cnt, nullptr, nullptr, nullptr, nullptr);
  note_launch();
  scan_rows<uint32_t>(cnt, cnt, ntiles, F::NC, part, totals, st);
}

template <class F>
static void index_emit_t(const uint32_t* g, const uint32_t* nmask, const uint32_t* amask, uint64_t G,
                         const uint32_t* chr_off, int n_chr, const uint32_t* cnt_scanned, const uint32_t* stride,
                         const uint64_t* list_off, const uint32_t* list_len, uint32_t* lists, bool every,
                         cudaStream_t st) {
  const uint32_t ntiles = index_num_tiles(G);
  bool done = false;
  if constexpr (F::NC == N_CTX) {
    if (every) {   // stride 1 for every context: each indexed position is written
      k_index_scan<F, 2><<<(ntiles + ix_warps(2) - 1) / ix_warps(2), 32 * ix_warps(2), 0, st>>>(
          g, nmask, amask, G, chr_off, n_chr, ntiles, const_cast<uint32_t*>(cnt_scanned), stride, list_off, list_len,
          lists);
      done = true;
    }
  }
  if (!done) {
    k_index_scan<F, 1><<<(ntiles + ix_warps(1) - 1) / ix_warps(1), 32 * ix_warps(1), 0, st>>>(
        g, nmask, amask, G, chr_off, n_chr, ntiles, const_cast<uint32_t*>(cnt_scanned), stride, list_off, list_len,
        lists);
  }
  note_launch();
}

void index_count(int which, const uint32_t* g, const uint32_t* nmask, const uint32_t* amask, uint64_t G,
                 const uint32_t* chr_off, int n_chr, uint32_t* cnt, uint32_t* part, uint32_t* totals, cudaStream_t st) {
  if (which == 0) index_count_t<SbsFamilies>(g, nmask, amask, G, chr_off, n_chr, cnt, part, totals, st);
  else index_count_t<IdFamilies>(g, nmask, nullptr, G, chr_off, n_chr, cnt, part, totals, st);
}

void index_emit(int which, const uint32_t* g, const uint32_t* nmask, const uint32_t* amask, uint64_t G,
                const uint32_t* chr_off, int n_chr, const uint32_t* cnt_scanned, const uint32_t* stride,
                const uint64_t* list_off, const uint32_t* list_len, uint32_t* lists, bool every, cudaStream_t st) {
  if (which == 0)
    index_emit_t<SbsFamilies>(g, nmask, amask, G, chr_off, n_chr, cnt_scanned, stride, list_off, list_len, lists,
                              every, st);
  else
    index_emit_t<IdFamilies>(g, nmask, nullptr, G, chr_off, n_chr, cnt_scanned, stride, list_off, list_len, lists,
                             every, st);
}

// the positions of the regions to avoid as bits of mask ((G + 31) / 32 words,
// zeroed by the caller)
__global__ void k_avoid_mask(const uint32_t* __restrict__ pos, uint64_t n, uint32_t* __restrict__ mask) {
  const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) atomicOr(mask + (pos[i] >> 5), 1u << (pos[i] & 31u));
}

void genome_avoid_mask(const uint32_t* pos, uint64_t n, uint32_t* mask, cudaStream_t st) {
  if (n) { k_avoid_mask<<<unsigned((n + 255) / 256), 256, 0, st>>>(pos, n, mask); note_launch(); }
}

int index_num_classes(int which) { return which == 0 ? SbsFamilies::NC : IdFamilies::NC; }

// ------------------------------------------------------------ allocation-free class counts
// The count pass above writes one count per (class, unit) into a table the
// engine allocates.  This variant keeps that table in a fixed array of the
// library's own device memory, so that a caller who may not allocate device
// memory can still count the classes of a genome it holds.  Genomes up to
// NOALLOC_MAX_BASES (8 Mbp, 2048 units) are accepted; the array (2.7 MB,
// NOALLOC_MAX_TILES entries per class) stays on every GPU that loads the
// library until the process ends.
static __device__ __align__(256) uint32_t g_noalloc_tile_counts[N_ID * NOALLOC_MAX_TILES];

// per-class sum of the tile counts (one block per class)
__global__ void k_class_totals(const uint32_t* __restrict__ cnt, uint32_t ntiles, uint64_t* __restrict__ totals) {
  __shared__ uint64_t s_part[8];
  const uint32_t k = blockIdx.x;
  uint64_t acc = 0;
  for (uint32_t t = threadIdx.x; t < ntiles; t += blockDim.x) acc += cnt[uint64_t(k) * ntiles + t];
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint64_t tot = 0;
    for (int w = 0; w < 8; ++w) tot += s_part[w];
    totals[k] = tot;
  }
}

// device address of g_noalloc_tile_counts per device (host code cannot use
// the symbol itself: on the host it names a stand-in, not device memory).
// The address is looked up once per device and kept; a cudaDeviceReset
// invalidates it, so the entry point is not for use after a device reset.
static std::mutex g_noalloc_mu;
static uint32_t* g_noalloc_addr[64] = {};

const char* index_counts_noalloc(int which, const uint32_t* g, uint64_t G, const uint32_t* chr_off, int n_chr,
                                 uint64_t* totals, cudaStream_t st) {
  constexpr uint64_t NOALLOC_MAX_BASES = uint64_t(NOALLOC_MAX_TILES) * 1024;
  static_assert(NOALLOC_MAX_BASES / IX_UNIT <= NOALLOC_MAX_TILES, "count array too small");
  if (G == 0 || G > NOALLOC_MAX_BASES) return "genome length must be in [1, 8388608] bases";
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return "no current CUDA device";
  uint32_t* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_tile_counts) != cudaSuccess || p == nullptr) {
        cudaGetLastError();
        return "cudaGetSymbolAddress failed for the library's count array";
      }
      g_noalloc_addr[dev] = static_cast<uint32_t*>(p);
    }
    scratch = g_noalloc_addr[dev];
  }
  const uint32_t ntiles = index_num_tiles(G);
  const int nc = index_num_classes(which);
  // an error left pending by earlier work on this thread is not this call's:
  // report it as such and leave it pending for its owner, launching nothing
  if (cudaPeekAtLastError() != cudaSuccess) return "a CUDA error from earlier work is pending; nothing was launched";
  // every (class, unit) entry is written by the count pass: nothing to clear
  const uint32_t blocks = (ntiles + IX_WARPS - 1) / IX_WARPS;
  if (which == 0)
    k_index_scan<SbsFamilies, 0><<<blocks, 256, 0, st>>>(g, nullptr, nullptr, G, chr_off, n_chr, ntiles, scratch,
                                                         nullptr, nullptr, nullptr, nullptr);
  else
    k_index_scan<IdFamilies, 0><<<blocks, 256, 0, st>>>(g, nullptr, nullptr, G, chr_off, n_chr, ntiles, scratch,
                                                        nullptr, nullptr, nullptr, nullptr);
  k_class_totals<<<nc, 256, 0, st>>>(scratch, ntiles, totals);
  note_launch(2);
  if (cudaGetLastError() != cudaSuccess) return "launch of the count kernels failed";
  return nullptr;
}

}  // namespace pg

namespace pg {

__global__ void k_gather_bases(const uint32_t* __restrict__ g, const uint32_t* __restrict__ nmask,
                               const uint32_t* __restrict__ pos, uint64_t n, uint64_t G, uint8_t* __restrict__ out) {
  const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n)
    out[i] = pos[i] < G && !base_unknown(nmask, pos[i]) ? uint8_t(base_at(g, pos[i])) : uint8_t(BASE_INVALID);
}

void genome_gather(const uint32_t* g, const uint32_t* nmask, uint64_t G, const uint32_t* pos, uint64_t n,
                   uint8_t* out, cudaStream_t st) {
  if (n) { k_gather_bases<<<unsigned((n + 255) / 256), 256, 0, st>>>(g, nmask, pos, n, G, out); note_launch(); }
}

// SID strings of placed mutations (the ref and alt columns of the result data
// frames): up to 8 characters each, 4 bits per character (A 1, C 2, G 3, N 4,
// T 5, the characters' alphabetical order; 0 ends the string), the first in
// the highest nibble, so that codes compare as the strings do.  An SNV is
// (reference base, alt base); an insertion (anchor, anchor + inserted bases);
// a deletion (anchor + deleted bases, anchor).
__device__ __forceinline__ uint32_t sid_char(const uint32_t* __restrict__ g, const uint32_t* __restrict__ nmask,
                                             uint64_t G, uint64_t p) {
  if (p >= G) p = G - 1;
  if (base_unknown(nmask, p)) return 4u;
  const uint32_t b = base_at(g, uint32_t(p));
  return b == 3u ? 5u : b + 1u;
}

__global__ void k_row_info(const uint32_t* __restrict__ locus, const uint32_t* __restrict__ aux,
                           const uint8_t* __restrict__ kind, const uint8_t* __restrict__ sig,
                           const uint8_t* __restrict__ nature, const uint32_t* __restrict__ rows, uint64_t n,
                           const uint32_t* __restrict__ g, const uint32_t* __restrict__ nmask, uint64_t G,
                           uint4* __restrict__ out) {
  const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t m = rows ? rows[i] : i;
  const uint32_t L = locus[m], a = aux[m], k = kind[m];
  const uint32_t anchor = sid_char(g, nmask, G, L) << 28;
  uint32_t ref = anchor, alt = anchor;
  if (k == 0) {
    const uint32_t b = a & 3u;
    alt = (b == 3u ? 5u : b + 1u) << 28;
  } else {
    const uint32_t l = (a >> 1) & 7u;
    for (uint32_t q = 0; q < l; ++q) {
      if (a & 1u) {
        const uint32_t b = (a >> (8 + 2 * q)) & 3u;
        alt |= (b == 3u ? 5u : b + 1u) << (24 - 4 * q);
      } else {
        ref |= sid_char(g, nmask, G, uint64_t(L) + 1 + q) << (24 - 4 * q);
      }
    }
  }
  out[i] = make_uint4(L, ref, alt, k | (uint32_t(sig[m]) << 8) | (uint32_t(nature[m]) << 16));
}

void row_info(const uint32_t* locus, const uint32_t* aux, const uint8_t* kind, const uint8_t* sig,
              const uint8_t* nature, const uint32_t* rows, uint64_t n, const uint32_t* g, const uint32_t* nmask,
              uint64_t G, uint4* out, cudaStream_t st) {
  if (n) {
    k_row_info<<<unsigned((n + 255) / 256), 256, 0, st>>>(locus, aux, kind, sig, nature, rows, n, g, nmask, G, out);
    note_launch();
  }
}

// the unknown bases (codes > 3) of an uploaded genome as one bit per position,
// and whether there is any
__global__ void k_genome_nmask(const uint8_t* __restrict__ codes, uint64_t G, uint64_t nwords,
                               uint32_t* __restrict__ mask, uint32_t* __restrict__ any) {
  const uint64_t w = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (w >= nwords) return;
  uint32_t m = 0;
  for (int j = 0; j < 32; ++j) {
    const uint64_t i = w * 32 + j;
    if (i < G && codes[i] > 3u) m |= 1u << j;
  }
  mask[w] = m;
  if (m) atomicOr(any, 1u);
}

void genome_nmask(const uint8_t* codes, uint64_t G, uint32_t* mask, uint32_t* any, cudaStream_t st) {
  const uint64_t nwords = (G + 31) / 32;
  if (nwords) { k_genome_nmask<<<unsigned((nwords + 255) / 256), 256, 0, st>>>(codes, G, nwords, mask, any); note_launch(); }
}

}  // namespace pg
