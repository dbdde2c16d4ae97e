// Bulk sequencing simulation: read placement, error model and per-mutation
// alt/depth counting.
//
// Reference call site: simulate_seq (src/seq_simulation.cpp:517-601) ->
// RACES ReadSimulator<>::operator()(sequencer, mutations_list, chr_ids,
// coverage, normal_sample, purity, ...) (:371, :413, :423; RACES absent).
// The counts produced here are what the reference flattens into
// `<sample>.occurrences` and `<sample>.coverage` (src/seq_simulation.cpp:92-140).
//
// Model:
//   * per (sample, chromosome) the number of fragments is
//     floor(coverage * L / (read_len * mates)); fragment starts are i.i.d.
//     uniform over the L - read_len + 1 positions.  Starts are generated tile
//     by tile: a binary tree of binomial draws splits the fragment count over
//     the tiles (an exact multinomial), then each tile draws its starts.
//   * a fragment comes from a normal cell with the purity-derived probability,
//     otherwise from a uniformly chosen sampled leaf; the allele is uniform.
//   * paired reads: insert size from a CDF table (the reference's binomial
//     model, src/seq_simulation.cpp:431-451, or a discretised normal); the
//     second mate starts at min(start + insert - read_len, chr_end - read_len).
//   * a read covering a mutation locus adds 1 to its depth; it adds 1 to alt
//     when it carries the mutation (edge is an ancestor of the cell, same
//     allele) and the base is not hit by a substitution error, or when it
//     does not carry it and an error turns the reference into that alt base.
//     The error word of a (mate, locus) visit is a multiplicative hash of the
//     mate's word (from the XOR of the fragment's Philox block) and the
//     locus; an error happens when it is below err_thr, and the erroneous
//     base is one of the three others by the third of [0, err_thr) the word
//     falls in, the first third being the alt base.
//     Indels are not affected by substitution errors.
//
// Kernel layout (one CTA per (tile, sample); fragments in batches):
//   phase A  every thread generates fragments (one Philox block each) and
//            writes its two mates to shared memory; mates are bucketed by
//            start position (16 bp buckets, counting sort);
//   phase B  work items (mutation record, start bucket) scan the mates of one
//            bucket that may cover the record and count depth and alt in
//            registers, one shared-memory atomic per item.
// Both phases keep every lane busy whatever the number of mutations a read
// covers.  Windows with more records than shared memory holds run a per-read
// loop on the global arrays instead.
#include <type_traits>

#include "pg_common.cuh"
#include "pg_rng.cuh"
#include "pg_kernels.h"
#include "pg_scan.cuh"

namespace pg {

constexpr int SEQ_THREADS = 256;
constexpr uint32_t SEQ_CAP = 512;        // mutation records staged per CTA
constexpr uint32_t SEQ_MCAP = 2 * SEQ_FRAGS_PER_BATCH;   // mates per batch
constexpr uint32_t SEQ_BW = 16;          // start bucket width (bp)
constexpr uint32_t SEQ_NBK = 1024;       // start buckets per window (window <= 16 kbp)
constexpr uint32_t SEQ_INS_CAP = 1024;   // insert-size CDF entries staged in shared memory
constexpr uint32_t SEQ_GUIDE = 256;      // guide table of the insert-size CDF

__global__ void k_seq_records(PlaceOut s, uint32_t n, const uint32_t* __restrict__ edge_tin,
                              const uint32_t* __restrict__ edge_tout, SeqRec* __restrict__ recs) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t e = s.edge[i];
  SeqRec r;
  r.locus = s.locus[i];
  r.tin = edge_tin[e];
  r.tout = edge_tout[e];
  r.info = uint32_t(s.allele[i]) | ((uint32_t(s.seq[i]) & 0x7fffu) << 16) | (uint32_t(s.kind[i]) << 31);
  recs[i] = r;
}

__device__ __forceinline__ uint32_t lower_bound_rec(const SeqRec* __restrict__ recs, uint32_t n, uint32_t key) {
  uint32_t lo = 0, hi = n;
  while (lo < hi) { const uint32_t mid = (lo + hi) >> 1; if (recs[mid].locus < key) lo = mid + 1; else hi = mid; }
  return lo;
}

// record range [lo, hi) of every tile's window [start, start + len - 1 + span)
__global__ void k_tile_ranges(const SeqRec* __restrict__ recs, uint32_t n_recs, const uint32_t* __restrict__ start,
                              const uint32_t* __restrict__ len, uint32_t n_tiles, uint32_t span,
                              uint32_t* __restrict__ rlo, uint32_t* __restrict__ rhi) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_tiles) return;
  rlo[t] = lower_bound_rec(recs, n_recs, start[t]);
  rhi[t] = lower_bound_rec(recs, n_recs, start[t] + len[t] - 1 + span);
}

// Multinomial split of a chromosome's fragments over its n tiles: a binary
// tree over the padded range [0, 2^D) of tiles (D = ceil(log2 n)); the node
// with heap id h at depth d covers tiles [i 2^(D-d), (i+1) 2^(D-d)) and sends
// Binomial(count, w_left / w_node) fragments to its left half, w being the
// number of start positions of the covered tiles or, with copy-number
// events, their DNA mass in the sample (so that fragments are proportional
// to copy number across tiles; the rejection draw of the start makes them so
// within a tile).  Every node's draw uses Philox counter
// (h, chromosome, sample, TAG_TILE_SPLIT).
struct TileSplit {
  uint64_t S;            // start positions of the chromosome
  uint32_t T;            // tile size
  uint32_t nt;           // tiles of the chromosome
  const double* cum;     // mass before each tile (NULL: weigh start positions)
  double tot;            // mass of the chromosome
  __device__ __forceinline__ uint64_t w(uint64_t a, uint64_t b) const {   // start positions of tiles [a, b)
    const uint64_t x = a * T < S ? a * T : S, y = b * T < S ? b * T : S;
    return y - x;
  }
  __device__ __forceinline__ double c(uint64_t a) const { return a < nt ? cum[a] : tot; }
  // the left child's share of the node [lo, hi) (0 when the node has no mass)
  __device__ __forceinline__ double share(uint64_t n, uint64_t lo, uint64_t mid, uint64_t hi) const {
    if (cum == nullptr) {
      const uint64_t wt = w(lo, hi);
      if (n == 0 || wt == 0) return 0.0;
      return double(w(lo, mid)) / double(wt);
    }
    const double base = c(lo), wt = c(hi) - base;
    if (n == 0 || !(wt > 0.0)) return 0.0;
    return (c(mid) - base) / wt;
  }
  __device__ __forceinline__ uint64_t left(Key key, uint32_t h, uint32_t chr, uint32_t s, uint64_t n, uint64_t lo,
                                           uint64_t mid, uint64_t hi) const {
    const double p = share(n, lo, mid, hi);
    if (!(p > 0.0)) return 0;
    Stream st{key, h, chr, s, TAG_TILE_SPLIT, 0u};
    return binomial(st, n, p);
  }
  // left() when its draw settles in the first attempt (false: call left())
  __device__ __forceinline__ bool left_first(Key key, uint32_t h, uint32_t chr, uint32_t s, uint64_t n, uint64_t lo,
                                             uint64_t mid, uint64_t hi, uint64_t& nl) const {
    const double p = share(n, lo, mid, hi);
    if (!(p > 0.0)) { nl = 0; return true; }
    return binomial_first(Stream{key, h, chr, s, TAG_TILE_SPLIT, 0u}, n, p, nl);
  }
};

constexpr uint32_t SPLIT_BLOCK_LOG = 6;   // 64 tiles per thread

// one thread per (sample, block of 64 tiles): walk from the root to the
// block's node, then draw the block's 63 internal splits top-down
__device__ __forceinline__ void tile_counts_one(uint32_t s, uint32_t bi, const uint32_t* __restrict__ blk_slot,
                                                const uint32_t* __restrict__ blk_index,
                                                const uint32_t* __restrict__ chr_first_tile,
                                                const uint32_t* __restrict__ chr_ntiles,
                                                const uint32_t* __restrict__ chr_depth,
                                                const uint32_t* __restrict__ chr_nstarts,
                                                const uint32_t* __restrict__ chr_id,
                                                const uint64_t* __restrict__ chr_pairs, uint32_t T, uint32_t n_tiles,
                                                const double* __restrict__ mass_cum,
                                                const double* __restrict__ mass_tot, uint32_t n_slots, Key key,
                                                uint32_t* __restrict__ pair_cnt) {
  const uint32_t slot = blk_slot[bi], b = blk_index[bi];
  const uint32_t D = chr_depth[slot], chr = chr_id[slot], nt = chr_ntiles[slot];
  const uint32_t base = chr_first_tile[slot];
  const TileSplit sp{chr_nstarts[slot], T, nt, mass_cum ? mass_cum + uint64_t(s) * n_tiles + base : nullptr,
                     mass_cum ? mass_tot[uint64_t(s) * n_slots + slot] : 0.0};
  const uint32_t Db = D < SPLIT_BLOCK_LOG ? D : SPLIT_BLOCK_LOG;   // depth of the block's subtree
  // root -> block node
  uint64_t n = chr_pairs[slot], lo = 0, size = uint64_t(1) << D;
  uint32_t h = 1;
  for (uint32_t d = 0; d < D - Db; ++d) {
    const uint64_t half = size >> 1, mid = lo + half;
    const uint64_t nl = sp.left(key, h, chr, s, n, lo, mid, lo + size);
    const bool right = (uint64_t(b) << Db) >= mid;   // the block lies in the right half
    if (right) { n -= nl; lo = mid; h = 2 * h + 1; } else { n = nl; h = 2 * h; }
    size = half;
  }
  // the block's subtree, breadth first (relative heap ids 1 .. 2^Db - 1)
  uint32_t c[2 << SPLIT_BLOCK_LOG];
  c[1] = uint32_t(n);
  const uint32_t nint = (1u << Db) - 1;
  for (uint32_t r = 1; r <= nint; ++r) {
    const uint32_t level = 31 - __clz(r);
    const uint64_t nsz = uint64_t(1) << (Db - level);
    const uint64_t nlo = lo + uint64_t(r - (1u << level)) * nsz;
    const uint32_t gh = (h << level) + (r - (1u << level));
    const uint64_t nl = sp.left(key, gh, chr, s, c[r], nlo, nlo + (nsz >> 1), nlo + nsz);
    c[2 * r] = uint32_t(nl);
    c[2 * r + 1] = c[r] - uint32_t(nl);
  }
  for (uint32_t r = 0; r < (1u << Db); ++r) {
    const uint64_t tile = lo + r;
    if (tile < nt) pair_cnt[uint64_t(s) * n_tiles + base + tile] = c[(1u << Db) + r];
  }
}

// Level-synchronous form of the same tree (the plain path): one launch per
// level, one thread per (sample, chromosome, node of the level) whose range
// meets the chromosome's tiles; node counts live in a per-(sample,
// chromosome) heap in global memory.  Every node draws with its own heap id,
// as in tile_counts_one, so the counts are the same.  A node whose draw
// settles in BTRS's first attempt (most do) is written at once; the others
// queue in shared memory and are drawn in full by consecutive threads, so
// that the exact test's logarithms run on dense warps.
constexpr uint32_t SPLIT_THREADS = 128;
__global__ void __launch_bounds__(SPLIT_THREADS) k_tile_split_level(
    uint32_t level, uint32_t n_slots, const uint32_t* __restrict__ chr_first_tile,
    const uint32_t* __restrict__ chr_ntiles, const uint32_t* __restrict__ chr_depth,
    const uint32_t* __restrict__ chr_nstarts, const uint32_t* __restrict__ chr_id,
    const uint64_t* __restrict__ chr_pairs, const uint64_t* __restrict__ heap_base, uint64_t heap_total, uint32_t T,
    uint32_t n_tiles, const double* __restrict__ mass_cum, const double* __restrict__ mass_tot, Key key,
    uint32_t* __restrict__ heap, uint32_t* __restrict__ pair_cnt) {
  __shared__ uint32_t s_q[SPLIT_THREADS];
  __shared__ uint32_t s_nq;
  const uint32_t s = blockIdx.z, slot = blockIdx.y;
  const uint32_t D = chr_depth[slot], nt = chr_ntiles[slot], first = chr_first_tile[slot];
  uint32_t* cnt = pair_cnt + uint64_t(s) * n_tiles + first;
  if (D == 0) {   // one tile: it takes every pair
    if (level == 0 && blockIdx.x == 0 && threadIdx.x == 0) cnt[0] = uint32_t(chr_pairs[slot]);
    return;
  }
  // whole blocks past the level's nodes leave together
  if (level >= D || uint64_t(blockIdx.x) * SPLIT_THREADS >= (uint64_t(1) << level)) return;
  if (threadIdx.x == 0) s_nq = 0;
  __syncthreads();
  const TileSplit sp{chr_nstarts[slot], T, nt, mass_cum ? mass_cum + uint64_t(s) * n_tiles + first : nullptr,
                     mass_cum ? mass_tot[uint64_t(s) * n_slots + slot] : 0.0};
  uint32_t* hp = heap + uint64_t(s) * heap_total + heap_base[slot];
  const uint64_t size = uint64_t(1) << (D - level);
  const uint32_t chr = chr_id[slot];
  // node of thread x of the block: its index in the level (valid when its
  // range meets the tiles), heap id, pair count
  auto node = [&](uint32_t x, uint64_t& i, uint32_t& h, uint64_t& n) {
    i = uint64_t(blockIdx.x) * SPLIT_THREADS + x;
    if (i >= (uint64_t(1) << level) || i * size >= nt) return false;
    h = uint32_t((uint64_t(1) << level) + i);
    n = level == 0 ? chr_pairs[slot] : hp[h];
    return true;
  };
  auto put = [&](uint64_t i, uint32_t h, uint64_t n, uint64_t nl) {
    const uint64_t lo = i * size;
    if (level + 1 == D) {   // the children are tiles lo and lo + 1
      cnt[lo] = uint32_t(nl);
      if (lo + 1 < nt) cnt[lo + 1] = uint32_t(n - nl);
    } else {
      hp[2 * h] = uint32_t(nl);
      hp[2 * h + 1] = uint32_t(n - nl);
    }
  };
  uint64_t i, n;
  uint32_t h;
  if (node(threadIdx.x, i, h, n)) {
    const uint64_t lo = i * size;
    uint64_t nl;
    if (sp.left_first(key, h, chr, s, n, lo, lo + (size >> 1), lo + size, nl)) put(i, h, n, nl);
    else s_q[atomicAdd(&s_nq, 1u)] = threadIdx.x;
  }
  __syncthreads();
  if (threadIdx.x < s_nq && node(s_q[threadIdx.x], i, h, n)) {
    const uint64_t lo = i * size;
    put(i, h, n, sp.left(key, h, chr, s, n, lo, lo + (size >> 1), lo + size));
  }
}

// Error words.  A mate's word: the fragment's error word for mate 0, an
// odd affine map of it for mate 1.  The visit of a mate (word wm) to locus:
// a multiplicative hash (uniform, as wm is), compared with err_thr for the
// substitution error and with its thirds err_t1, err_t2 for the erroneous
// base.
__device__ __forceinline__ uint32_t mate_word(uint32_t w, uint32_t mate) {
  return mate ? w * 0x85EBCA6Bu + 0x27D4EB2Fu : w;
}
__device__ __forceinline__ uint32_t err_word(uint32_t wm, uint32_t locus) {
  return (wm ^ (locus * 0x9E3779B1u)) * 0xC2B2AE35u;
}
// which of the three other bases an error word below err_thr picks
__device__ __forceinline__ uint32_t err_third(const SeqParams& prm, uint32_t e) {
  return e < prm.err_t1 ? 0u : (e < prm.err_t2 ? 1u : 2u);
}

// does allele instance y of the read's cell carry the mutation placed on
// instance x with order key key_m (tin of its edge << 16 | order on the edge)?
// y carries it when y is x, or when y descends from x through copies made
// after the mutation (a copy's key exceeds the mutation's: both lie on the
// cell's root path, where tin grows with depth)
__device__ __forceinline__ bool inst_carries(const SeqParams& prm, uint32_t y, uint32_t x, uint64_t key_m) {
  if (y == x) return true;
  if (!prm.has_cna) return false;
  for (uint32_t q = __ldg(prm.chain_off + y), e = __ldg(prm.chain_off + y + 1); q < e; ++q)
    if (__ldg(prm.chain_anc + q) == x) return __ldg(prm.chain_key + q) > key_m;
  return false;
}

// did the visit of a mate (word wm) observe the alt base?
__device__ __forceinline__ bool observed(const SeqParams& prm, uint32_t tin, uint32_t tout, uint32_t info,
                                         uint32_t cell, uint32_t inst, uint32_t wm, uint32_t locus) {
  // the cell is in the edge's subtree when tin <= cell < tout (one unsigned compare)
  // branch-free but for the lineage walk of a copied instance: the error
  // word is computed for indels too, and the caller evaluates every
  // candidate mate (covering or not), so that a warp does not diverge.
  // A copy has a larger instance number than its source, and instances 0
  // and 1 have no source: the walk is needed only when inst > max(x, 1).
  const bool sub = cell - tin < tout - tin;
  const uint32_t x = info & 0xffffu;
  bool carried = sub && inst == x;
  if (sub && inst > max(x, 1u) && prm.has_cna)
    carried = inst_carries(prm, inst, x, (uint64_t(tin) << 16) | ((info >> 16) & 0x7fffu));
  const uint32_t e = err_word(wm, locus);
  const bool snv = carried ? e >= prm.err_thr : e < prm.err_t1;
  return (info >> 31) ? carried : snv;
}

// One fragment's draws: mate starts, source cell, allele instance and its
// error word, all from ONE Philox4x32-10 block r (counter (j, t, s, TAG_PAIR)):
//   r.x  the start: uniform in the tile; with copy-number events, when the
//        tile meets several atoms, the part by its mass (31-bit thresholds)
//        and the start uniform in the part from the word's residual within
//        the part's threshold interval (exact integer arithmetic)
//   r.y  the cell: normal when below normal_thr, else a sampled leaf; with
//        copy-number events the cell option (normal cells or a leaf class)
//        by its copies in the part's atom
//   r.z  the insert size (31-bit thresholds of its CDF)
//   r.w  the allele instance, uniform among the n covering ones
//        (floor(r.w n / 2^32)), then the leaf, uniform in its class, from the
//        fraction that draw leaves (the low word of r.w n): the two indices
//        use disjoint information of the word
//   r.x ^ r.y ^ r.z ^ r.w  the fragment's error word
// Without copy-number events the instance is allele 0 or 1 and the leaf is
// uniform over the sample's leaves.
struct Fragment {
  uint32_t p0, p1, cell, inst, w;
};

// The copy-number draw tables of one (tile, sample) staged in shared memory:
// the tile's parts with their thresholds and, per part, the option
// thresholds of its atom and each option's covering instances there.
constexpr uint32_t SEQ_CN_PARTS = 4, SEQ_CN_OPTS = 8;
struct CnCache {
  uint32_t pstart[SEQ_CN_PARTS], plen[SEQ_CN_PARTS], pthr[SEQ_CN_PARTS];
  uint32_t othr[SEQ_CN_PARTS][SEQ_CN_OPTS], oioff[SEQ_CN_PARTS][SEQ_CN_OPTS], oicnt[SEQ_CN_PARTS][SEQ_CN_OPTS];
  uint32_t onl[SEQ_CN_OPTS], oloff[SEQ_CN_OPTS];
  uint32_t n_parts, n_opt;
};

__device__ __forceinline__ void fill_cn_cache(CnCache& c, const SeqParams& prm, const SeqSample& sm, uint32_t t,
                                              uint32_t s, uint32_t tid) {
  const uint32_t pb = prm.part_off[t], pn = prm.part_off[t + 1] - pb, no = sm.n_opt;
  if (tid == 0) { c.n_parts = pn; c.n_opt = no; }
  if (tid < pn) {
    c.pstart[tid] = prm.part_start[pb + tid];
    c.plen[tid] = prm.part_len[pb + tid];
    c.pthr[tid] = prm.part_cdf[uint64_t(s) * prm.n_parts + pb + tid];
  }
  if (tid < no) { c.onl[tid] = prm.opt_nleaf[sm.opt_off + tid]; c.oloff[tid] = prm.opt_leaf_off[sm.opt_off + tid]; }
  if (tid < pn * no) {
    const uint32_t p = tid / no, o = tid % no;
    const uint32_t atom = prm.part_atom[pb + p];
    c.othr[p][o] = prm.opt_cdf[sm.opt_cdf_off + atom * no + o];
    const uint32_t ai = atom * prm.n_classes + prm.opt_class[sm.opt_off + o];
    c.oioff[p][o] = prm.atom_ioff[ai];
    c.oicnt[p][o] = prm.atom_icnt[ai];
  }
}

// cdf_lookup for tables of at most NMAX (a power of two) thresholds: the
// count of thresholds <= u >> 1 by binary lifting, without a data-dependent
// loop (the same index as cdf_lookup for sorted thresholds)
template <uint32_t NMAX>
__device__ __forceinline__ uint32_t cdf_lookup_small(const uint32_t* thr, uint32_t n, uint32_t u) {
  const uint32_t v = u >> 1;
  uint32_t lo = 0;
#pragma unroll
  for (uint32_t step = NMAX; step >= 1; step >>= 1)
    if (lo + step <= n && thr[lo + step - 1] <= v) lo += step;
  return lo < n ? lo : n - 1;
}

// start offset in a part of length plen from the word u that selected the
// part, whose 31-bit value lies in the part's threshold interval [lo, hi)
__device__ __forceinline__ uint32_t part_offset(uint32_t u, uint32_t lo, uint32_t hi, uint32_t plen) {
  return uint32_t((uint64_t((u >> 1) - lo) * plen) / uint64_t(hi - lo));
}

// CN selects the copy-number path at compile time (0: no copy-number
// events, 1: the tile's tables in shared memory, 2: the tables in global
// memory) or, -1, at run time from prm.has_cna and cc.
// (KeyT: Key, or the precomputed RoundKeys of the same key)
__device__ __forceinline__ U4 pair_block(const Key& key, uint32_t j, uint32_t t, uint32_t s) {
  return philox(key.k0, key.k1, j, t, s, TAG_PAIR);
}
__device__ __forceinline__ U4 pair_block(const RoundKeys& rk, uint32_t j, uint32_t t, uint32_t s) {
  return philox(rk, j, t, s, TAG_PAIR);
}

template <bool INS_SMEM, int CN = -1, class KeyT>
__device__ __forceinline__ Fragment make_fragment(const KeyT& key, uint32_t j, uint32_t t, uint32_t s, uint32_t start,
                                                  uint32_t len, uint32_t ce, const SeqSample& sm,
                                                  const uint32_t* __restrict__ leaf_tin, const SeqParams& prm,
                                                  const uint32_t* ins, const uint16_t* guide,
                                                  const CnCache* cc = nullptr) {
  const U4 r = pair_block(key, j, t, s);
  Fragment f;
  const uint32_t R = prm.read_len;
  const int path = CN >= 0 ? CN : (!prm.has_cna ? 0 : (cc ? 1 : 2));
  if (path == 0) {
    f.p0 = start + __umulhi(r.x, len);
    const bool normal = sm.all_normal || r.y < sm.normal_thr;
    f.inst = __umulhi(r.w, prm.n_alleles);
    f.cell = normal ? prm.normal_tin
                    : __ldg(leaf_tin + sm.leaf_off + __umulhi(r.w * prm.n_alleles, sm.n_leaves));
  } else if (path == 1) {
    uint32_t part = 0;
    if (cc->n_parts > 1) {
      part = cdf_lookup_small<SEQ_CN_PARTS>(cc->pthr, cc->n_parts, r.x);
      f.p0 = cc->pstart[part] + part_offset(r.x, part ? cc->pthr[part - 1] : 0u, cc->pthr[part], cc->plen[part]);
    } else {
      f.p0 = cc->pstart[0] + __umulhi(r.x, cc->plen[0]);
    }
    const uint32_t o = cdf_lookup_small<SEQ_CN_OPTS>(cc->othr[part], cc->n_opt, r.y);
    const uint32_t nl = cc->onl[o], icnt = cc->oicnt[part][o];
    f.inst = icnt ? uint32_t(__ldg(prm.gc.inst_list + cc->oioff[part][o] + __umulhi(r.w, icnt))) : 0xffffu;
    f.cell = nl ? __ldg(prm.cls_leaf_tin + cc->oloff[o] + __umulhi(r.w * icnt, nl)) : prm.normal_tin;
  } else {
    const uint32_t pb = __ldg(prm.part_off + t), pn = __ldg(prm.part_off + t + 1) - pb;
    uint32_t part = pb;
    if (pn > 1) {
      const uint32_t* thr = prm.part_cdf + uint64_t(s) * prm.n_parts + pb;
      const uint32_t k = cdf_lookup(thr, pn, r.x);
      part = pb + k;
      f.p0 = __ldg(prm.part_start + part) +
             part_offset(r.x, k ? __ldg(thr + k - 1) : 0u, __ldg(thr + k), __ldg(prm.part_len + part));
    } else {
      f.p0 = __ldg(prm.part_start + part) + __umulhi(r.x, __ldg(prm.part_len + part));
    }
    const uint32_t atom = __ldg(prm.part_atom + part);
    const uint32_t o = sm.opt_off + cdf_lookup(prm.opt_cdf + sm.opt_cdf_off + atom * sm.n_opt, sm.n_opt, r.y);
    const uint32_t nl = __ldg(prm.opt_nleaf + o);
    const uint32_t ai = atom * prm.n_classes + __ldg(prm.opt_class + o);
    const uint32_t icnt = __ldg(prm.atom_icnt + ai);
    f.inst = icnt ? uint32_t(__ldg(prm.gc.inst_list + __ldg(prm.atom_ioff + ai) + __umulhi(r.w, icnt))) : 0xffffu;
    f.cell = nl ? __ldg(prm.cls_leaf_tin + __ldg(prm.opt_leaf_off + o) + __umulhi(r.w * icnt, nl)) : prm.normal_tin;
  }
  f.w = r.x ^ r.y ^ r.z ^ r.w;
  f.p1 = f.p0;
  if (prm.paired) {
    uint32_t k;
    if (INS_SMEM) {
      const uint32_t v = r.z >> 1;
      k = guide[v >> 23];
      while (k + 1 < prm.n_ins && ins[k] <= v) ++k;
    } else {
      k = cdf_lookup(prm.ins_cdf, prm.n_ins, r.z);
    }
    uint32_t p1 = f.p0 + prm.ins_min + k - R;
    if (p1 > ce - R) p1 = ce - R;
    f.p1 = p1;
  }
  return f;
}

// shared memory of one read CTA
struct ReadSmem {
  uint32_t s_locus[SEQ_CAP], s_tin[SEQ_CAP], s_tout[SEQ_CAP], s_info[SEQ_CAP];
  uint32_t s_alt[SEQ_CAP], s_dep[SEQ_CAP];
  // mates of the batch in start-bucket order
  uint32_t s_mpi[SEQ_MCAP];      // start offset in the window | allele instance << 16 (a dropped
                                 //   fragment: offset 0xffff, instance 0xffff)
  uint2 s_mcw[SEQ_MCAP];         // source cell (Euler index), the mate's error word
  uint32_t s_boff[SEQ_NBK + 4];  // bucket counts, then offsets
  uint32_t s_ins[SEQ_INS_CAP];
  uint16_t s_guide[SEQ_GUIDE];
  uint16_t s_wstart[SEQ_CAP];    // first candidate mate (sorted position) of each record
  uint32_t s_wpre[SEQ_CAP];      // prefix of the records' candidate counts
  uint32_t s_scan[8];
  uint32_t s_wtot;
  CnCache s_cn;
};

// One work item: the n_pairs fragments of tile t (window [start, ...),
// records [lo, lo + nw) of g_recs) for sample s, counted into the rows
// g_alt_row / g_dep_row (indexed by record).  Called by every thread of the
// CTA with the same arguments.
template <class KeyT>
__device__ __forceinline__ void read_tile(ReadSmem& sh, const SeqRec* __restrict__ g_recs, uint32_t t, uint32_t s,
                                          uint32_t n_pairs, uint32_t lo, uint32_t nw, uint32_t start, uint32_t len,
                                          uint32_t ce, const SeqSample& sm, const uint32_t* __restrict__ leaf_tin,
                                          const SeqParams& prm, const KeyT& key, uint32_t* __restrict__ g_alt_row,
                                          uint32_t* __restrict__ g_dep_row) {
  auto& s_locus = sh.s_locus; auto& s_tin = sh.s_tin; auto& s_tout = sh.s_tout; auto& s_info = sh.s_info;
  auto& s_alt = sh.s_alt; auto& s_dep = sh.s_dep;
  auto& s_mpi = sh.s_mpi; auto& s_mcw = sh.s_mcw;
  auto& s_boff = sh.s_boff; auto& s_ins = sh.s_ins; auto& s_guide = sh.s_guide;
  auto& s_wstart = sh.s_wstart; auto& s_wpre = sh.s_wpre; auto& s_scan = sh.s_scan;
  uint32_t& s_wtot = sh.s_wtot;
  CnCache& s_cn = sh.s_cn;
  const uint32_t tid = threadIdx.x;
  if (nw == 0 || n_pairs == 0) return;       // nothing to count in this window
  const uint32_t R = prm.read_len;
  const uint32_t wlen = len - 1 + prm.span;   // the window is [start, start + wlen)
  const uint32_t nbk = (wlen + SEQ_BW - 1) / SEQ_BW;
  uint32_t* galt = g_alt_row + lo;
  uint32_t* gdep = g_dep_row + lo;
  const SeqRec* grec = g_recs + lo;
  const bool ins_smem = prm.paired && prm.n_ins <= SEQ_INS_CAP;

  if (nw > SEQ_CAP || nbk > SEQ_NBK || wlen >= 32768u) {
    // dense or long window: per-read loop over the global records
    for (uint32_t j = tid; j < n_pairs; j += SEQ_THREADS) {
      const Fragment f = make_fragment<false>(key, j, t, s, start, len, ce, sm, leaf_tin, prm, nullptr, nullptr);
      if (f.inst == 0xffffu) continue;   // dropped: no covering instance
      for (uint32_t mate = 0; mate < (prm.paired ? 2u : 1u); ++mate) {
        const uint32_t a = mate ? f.p1 : f.p0;
        for (uint32_t i = lower_bound_rec(grec, nw, a); i < nw; ++i) {
          const SeqRec r = grec[i];
          if (r.locus >= a + R) break;
          atomicAdd(gdep + i, 1u);
          if (observed(prm, r.tin, r.tout, r.info, f.cell, f.inst, mate_word(f.w, mate), r.locus))
            atomicAdd(galt + i, 1u);
        }
      }
    }
    return;
  }

  for (uint32_t i = tid; i < nw; i += SEQ_THREADS) {
    const SeqRec r = grec[i];
    s_locus[i] = r.locus; s_tin[i] = r.tin; s_tout[i] = r.tout; s_info[i] = r.info;
    s_alt[i] = 0; s_dep[i] = 0;
  }
  if (ins_smem) {
    for (uint32_t i = tid; i < prm.n_ins; i += SEQ_THREADS) s_ins[i] = prm.ins_cdf[i];
    for (uint32_t g = tid; g < SEQ_GUIDE; g += SEQ_THREADS) s_guide[g] = prm.ins_guide[g];
  }
  // copy-number draws from shared memory when the tile's tables fit
  // (the first barrier of the batch loop publishes them)
  const bool cn_smem = prm.has_cna && prm.part_off[t + 1] - prm.part_off[t] <= SEQ_CN_PARTS &&
                       sm.n_opt <= SEQ_CN_OPTS;
  if (cn_smem) fill_cn_cache(s_cn, prm, sm, t, s, tid);
  const CnCache* cc = cn_smem ? &s_cn : nullptr;

  const uint32_t per_batch = SEQ_MCAP / 2;

  constexpr uint32_t FPT = SEQ_MCAP / 2 / SEQ_THREADS;   // fragments per thread and batch
  for (uint32_t b0 = 0; b0 < n_pairs; b0 += per_batch) {
    const uint32_t nb_pairs = min(per_batch, n_pairs - b0);
    for (uint32_t b = tid; b <= nbk; b += SEQ_THREADS) s_boff[b] = 0;
    __syncthreads();
    // phase A: fragments stay in registers (mate offsets, both < 2^15, and
    // bucket ranks, both < 2^16, packed in pairs); each mate takes its rank
    // within its start bucket from the histogram's atomic
    uint32_t o01[FPT], ca[FPT], fi[FPT], fw[FPT], rk01[FPT];
    // one instance of the draw code per (copy-number path, insert table)
    // pair, chosen once per tile: the unrolled loop holds only that path
    auto gen = [&](auto cn, auto ins_tag) {
#pragma unroll
      for (uint32_t q = 0; q < FPT; ++q) {
        const uint32_t k = tid + q * SEQ_THREADS;
        if (k < nb_pairs) {
          const Fragment f = make_fragment<decltype(ins_tag)::value, decltype(cn)::value>(
              key, b0 + k, t, s, start, len, ce, sm, leaf_tin, prm, ins_smem ? s_ins : nullptr,
              ins_smem ? s_guide : nullptr, cc);
          ca[q] = f.cell;
          fi[q] = f.inst;
          fw[q] = f.w;
          const uint32_t o0 = f.p0 - start;
          uint32_t rk = atomicAdd(s_boff + o0 / SEQ_BW, 1u);
          uint32_t o1 = 0;
          if (prm.paired) {
            o1 = f.p1 - start;
            rk |= atomicAdd(s_boff + o1 / SEQ_BW, 1u) << 16;
          }
          o01[q] = o0 | (o1 << 16);
          rk01[q] = rk;
        }
      }
    };
    using T0 = std::integral_constant<int, 0>;
    using T1 = std::integral_constant<int, 1>;
    using T2 = std::integral_constant<int, 2>;
    using YES = std::true_type;
    using NO = std::false_type;
    if (!prm.has_cna) { if (ins_smem) gen(T0{}, YES{}); else gen(T0{}, NO{}); }
    else if (cc) { if (ins_smem) gen(T1{}, YES{}); else gen(T1{}, NO{}); }
    else { if (ins_smem) gen(T2{}, YES{}); else gen(T2{}, NO{}); }
    __syncthreads();
    // bucket offsets (exclusive scan of at most 1024 counts)
    {
      uint32_t v[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) { const uint32_t b = tid * 4 + q; v[q] = b < nbk ? s_boff[b] : 0u; }
      const uint32_t tot = block_excl_scan4(v, s_scan);
#pragma unroll
      for (int q = 0; q < 4; ++q) { const uint32_t b = tid * 4 + q; if (b < nbk) s_boff[b] = v[q]; }
      if (tid == 0) s_boff[nbk] = tot;
    }
    __syncthreads();
    // scatter the mates in start-bucket order
#pragma unroll
    for (uint32_t q = 0; q < FPT; ++q) {
      const uint32_t k = tid + q * SEQ_THREADS;
      if (k < nb_pairs) {
        const uint32_t o0 = o01[q] & 0xffffu, o1 = o01[q] >> 16;
        const uint32_t x0 = s_boff[o0 / SEQ_BW] + (rk01[q] & 0xffffu);
        // a dropped fragment's mates carry the start offset 0xffff: past every locus
        const uint32_t oo0 = fi[q] == 0xffffu ? 0xffffu : o0, oo1 = fi[q] == 0xffffu ? 0xffffu : o1;
        s_mpi[x0] = oo0 | (fi[q] << 16); s_mcw[x0] = make_uint2(ca[q], fw[q]);
        if (prm.paired) {
          const uint32_t x1 = s_boff[o1 / SEQ_BW] + (rk01[q] >> 16);
          s_mpi[x1] = oo1 | (fi[q] << 16); s_mcw[x1] = make_uint2(ca[q], mate_word(fw[q], 1u));
        }
      }
    }
    __syncthreads();
    // phase B: a record's candidate mates (those starting in the buckets of
    // [L-R+1, L]) are one contiguous run of the bucket-sorted mates; the runs
    // of all records are concatenated and split evenly over the threads
    {
      uint32_t v[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const uint32_t i = tid * 4 + q;
        uint32_t cnt = 0;
        if (i < nw) {
          const uint32_t off = s_locus[i] - start;
          const uint32_t blo = (off + 1 >= R ? off + 1 - R : 0u) / SEQ_BW;
          const uint32_t bhi = min(off / SEQ_BW, nbk - 1);
          s_wstart[i] = uint16_t(s_boff[blo]);
          cnt = s_boff[bhi + 1] - s_boff[blo];
        }
        v[q] = cnt;
      }
      const uint32_t tot = block_excl_scan4(v, s_scan);
#pragma unroll
      for (int q = 0; q < 4; ++q) { const uint32_t i = tid * 4 + q; if (i < SEQ_CAP) s_wpre[i] = v[q]; }
      if (tid == 0) s_wtot = tot;
    }
    __syncthreads();
    {
      const uint32_t W = s_wtot;
      const uint32_t k0 = uint32_t(uint64_t(W) * tid / SEQ_THREADS);
      const uint32_t k1 = uint32_t(uint64_t(W) * (tid + 1) / SEQ_THREADS);
      if (k0 < k1) {
        uint32_t i = 0, hi = nw;                              // record holding work item k0
        while (hi - i > 1) { const uint32_t mid = (i + hi) >> 1; if (s_wpre[mid] <= k0) i = mid; else hi = mid; }
        uint32_t next = i + 1 < nw ? s_wpre[i + 1] : W;
        uint32_t L = s_locus[i], off = L - start, tin = s_tin[i], tout = s_tout[i], info = s_info[i];
        uint32_t base = s_wstart[i] - s_wpre[i];
        uint32_t dep = 0, alt = 0;
        for (uint32_t k = k0; k < k1;) {
          while (k >= next) {                                 // the run of the next record starts
            if (dep) { atomicAdd(s_dep + i, dep); if (alt) atomicAdd(s_alt + i, alt); }
            dep = 0; alt = 0;
            ++i;
            next = i + 1 < nw ? s_wpre[i + 1] : W;
            L = s_locus[i]; off = L - start; tin = s_tin[i]; tout = s_tout[i]; info = s_info[i];
            base = s_wstart[i] - s_wpre[i];
          }
          // two visits of the same record at a time when the run allows it
          const uint32_t nv = (k + 1 < next && k + 1 < k1) ? 2u : 1u;
          const uint32_t x = base + k, x1 = nv == 2u ? x + 1u : x;
          const uint32_t pi = s_mpi[x], pj = s_mpi[x1];
          const uint2 cw = s_mcw[x], cv = s_mcw[x1];
          // the mate covers L when its start o is in (L - R, L] (unsigned: o > off wraps)
          const bool cov = off - (pi & 0xffffu) < R;
          const bool cov1 = nv == 2u && off - (pj & 0xffffu) < R;
          const bool ob = observed(prm, tin, tout, info, cw.x, pi >> 16, cw.y, L);
          const bool ob1 = observed(prm, tin, tout, info, cv.x, pj >> 16, cv.y, L);
          dep += (cov ? 1u : 0u) + (cov1 ? 1u : 0u);
          alt += ((cov & ob) ? 1u : 0u) + ((cov1 & ob1) ? 1u : 0u);
          k += nv;
        }
        if (dep) { atomicAdd(s_dep + i, dep); if (alt) atomicAdd(s_alt + i, alt); }
      }
    }
    __syncthreads();
  }
  for (uint32_t i = tid; i < nw; i += SEQ_THREADS) {
    const uint32_t d = s_dep[i];
    if (d) {
      atomicAdd(gdep + i, d);
      const uint32_t a = s_alt[i];
      if (a) atomicAdd(galt + i, a);
    }
  }
}


__global__ void __launch_bounds__(SEQ_THREADS, 4) k_reads(const SeqRec* __restrict__ g_recs, SeqTiles tiles,
                                                          const uint32_t* __restrict__ pair_cnt,
                                                          const SeqSample* __restrict__ samples,
                                                          const uint32_t* __restrict__ leaf_tin, SeqParams prm,
                                                          RoundKeys key, uint64_t n_recs, uint32_t* __restrict__ g_alt,
                                                          uint32_t* __restrict__ g_dep) {
  __shared__ ReadSmem sh;
  const uint32_t t = blockIdx.x, s = blockIdx.y;
  const uint32_t lo = tiles.rec_lo[t];
  const SeqSample sm = samples[s];
  read_tile(sh, g_recs, t, s, pair_cnt[uint64_t(s) * tiles.n_tiles + t], lo, tiles.rec_hi[t] - lo, tiles.start[t],
            tiles.len[t], tiles.chr_end[t], sm, leaf_tin, prm, key, g_alt + uint64_t(s) * n_recs,
            g_dep + uint64_t(s) * n_recs);
}

static inline unsigned nblk(uint64_t n, int b = 256) { return unsigned((n + b - 1) / b); }

// ------------------------------------------------------------ SAM reads
// The bases of one mate starting at reference position p: the reference with
// the carried SNVs (alt base) and indels (inserted bases; skipped deleted
// bases, anchored at the base before them), and a substitution wherever the
// visit's error word is below the threshold.  A substitution picks one of the
// three other bases by the third of [0, err_thr) its word falls in; at an SNV
// site the first of them is the
// counterpart allele (the alt base when the read shows the reference, the
// reference when it shows the alt), so that the bases agree with the alt
// counts of the read kernel.  Inserted bases draw their errors from the word
// mixed with their rank.  Indels anchored before p are not applied.
__device__ void build_read(const SeqParams& prm, const uint32_t* __restrict__ genome, const SeqRec* __restrict__ recs,
                           uint32_t n_recs, const uint32_t* __restrict__ aux, uint32_t p, uint32_t ce, uint32_t cell,
                           uint32_t inst, uint32_t w, uint32_t mate, SamRead& out, char* __restrict__ seq) {
  const char* ACGT = "ACGT";
  const uint32_t R = prm.read_len;
  const uint32_t wm = mate_word(w, mate);
  uint32_t i = lower_bound_rec(recs, n_recs, p);
  uint32_t q = p, n = 0, nc = 0;
  auto push = [&](uint32_t op, uint32_t len) {
    if (nc > 0 && (out.cigar[nc - 1] & 15u) == op) { out.cigar[nc - 1] += len << 4; return; }
    if (nc < SAM_MAX_CIGAR) out.cigar[nc++] = (len << 4) | op;
  };
  auto others = [](uint32_t tb, int first, uint32_t k) {   // k-th base other than tb (first: preferred one)
    uint32_t o[3] = {0, 0, 0}, m = 0;
    if (first >= 0 && uint32_t(first) != tb) o[m++] = uint32_t(first);
    for (uint32_t x = 0; x < 4 && m < 3; ++x) if (x != tb && (m == 0 || x != o[0])) o[m++] = x;
    return o[k];
  };
  bool indels_open = true;
  while (n < R && q < ce) {
    const uint32_t b = base_at(genome, q);
    while (i < n_recs && recs[i].locus < q) ++i;
    bool site = false, carried_snv = false;
    uint32_t alt = 0, indel = 0;
    bool has_indel = false;
    for (uint32_t k = i; k < n_recs && recs[k].locus == q; ++k) {
      const SeqRec r = recs[k];
      const bool carried = (r.tin <= cell) && (cell < r.tout) &&
                           inst_carries(prm, inst, r.info & 0xffffu, (uint64_t(r.tin) << 16) | ((r.info >> 16) & 0x7fffu));
      if (!(r.info >> 31)) {
        if (!site) { site = true; alt = aux[k] & 3u; }
        if (carried && !carried_snv) { carried_snv = true; alt = aux[k] & 3u; }
      } else if (carried && !has_indel) {
        has_indel = true;
        indel = aux[k];
      }
    }
    uint32_t tb = carried_snv ? alt : b;
    const uint32_t e = err_word(wm, q);
    if (e < prm.err_thr) tb = others(tb, site ? int(carried_snv ? b : alt) : -1, err_third(prm, e));
    // an unknown reference base (N) reads as N
    const bool unknown = prm.nmask && ((__ldg(prm.nmask + (q >> 5)) >> (q & 31u)) & 1u);
    seq[n++] = unknown ? 'N' : ACGT[tb];
    push(0u, 1u);
    ++q;
    if (has_indel && indels_open && nc < SAM_MAX_CIGAR - 2) {
      const uint32_t l = (indel >> 1) & 7u;
      if (indel & 1u) {
        for (uint32_t k = 0; k < l && n < R; ++k) {
          uint32_t ib = (indel >> (8 + 2 * k)) & 3u;
          const uint32_t ei = err_word(wm ^ (0x9E3779B1u * (k + 1)), q - 1);
          if (ei < prm.err_thr) ib = others(ib, -1, err_third(prm, ei));
          seq[n++] = ACGT[ib];
          push(1u, 1u);
        }
      } else if (n < R) {
        push(2u, l);
        q += l;
      }
    } else if (has_indel) {
      indels_open = false;       // the CIGAR is full: later indels are not applied
    }
  }
  out.pos = p;
  out.n_cigar = uint16_t(nc);
  out.seq_len = n;
}

__global__ void k_sam_reads(const SeqRec* __restrict__ recs, uint32_t n_recs, const uint32_t* __restrict__ aux,
                            const uint32_t* __restrict__ genome, SeqTiles tiles, uint32_t t0, uint32_t n_chunk,
                            const uint32_t* __restrict__ pair_cnt, const SeqSample* __restrict__ samples,
                            const uint32_t* __restrict__ leaf_tin, SeqParams prm, Key key,
                            const uint64_t* __restrict__ out_off, SamRead* __restrict__ out, char* __restrict__ seq,
                            uint32_t max_len) {
  const uint32_t k = blockIdx.x, s = blockIdx.y, t = t0 + k;
  const uint32_t n_pairs = pair_cnt[uint64_t(s) * tiles.n_tiles + t];
  const uint32_t start = tiles.start[t], len = tiles.len[t], ce = tiles.chr_end[t];
  const SeqSample sm = samples[s];
  const uint64_t base = out_off[uint64_t(s) * n_chunk + k];
  const uint32_t mates = prm.paired ? 2u : 1u;
  for (uint32_t j = threadIdx.x; j < n_pairs; j += blockDim.x) {
    const Fragment f = make_fragment<false>(key, j, t, s, start, len, ce, sm, leaf_tin, prm, nullptr, nullptr);
    for (uint32_t m = 0; m < mates; ++m) {
      const uint64_t r = (base + j) * mates + m;
      SamRead& o = out[r];
      char* sq = seq + r * max_len;
      if (f.inst == 0xffffu) { o.pos = f.p0; o.mate_pos = f.p0; o.tlen = 0; o.flag = 4; o.n_cigar = 0; o.seq_len = 0; continue; }
      const uint32_t p = m ? f.p1 : f.p0;
      build_read(prm, genome, recs, n_recs, aux, p, ce, f.cell, f.inst, f.w, m, o, sq);
      if (prm.paired) {
        o.mate_pos = m ? f.p0 : f.p1;
        const int32_t span = int32_t(f.p1 + prm.read_len - f.p0);
        o.tlen = m ? -span : span;
        o.flag = uint16_t(0x1 | 0x2 | (m ? (0x80 | 0x10) : (0x40 | 0x20)));
      } else {
        o.mate_pos = 0; o.tlen = 0; o.flag = 0;
      }
    }
  }
}

void seq_sam_reads(const SeqRec* recs, uint32_t n_recs, const uint32_t* aux, const uint32_t* genome,
                   const SeqTiles& tiles, uint32_t t0, uint32_t n_chunk, const uint32_t* pair_cnt,
                   const SeqSample* samples, uint32_t n_samples, const uint32_t* leaf_tin, const SeqParams& prm,
                   uint64_t seed, const uint64_t* out_off, SamRead* out, char* seq, uint32_t max_len,
                   cudaStream_t st) {
  if (n_chunk == 0 || n_samples == 0) return;
  dim3 grid(n_chunk, n_samples);
  k_sam_reads<<<grid, 128, 0, st>>>(recs, n_recs, aux, genome, tiles, t0, n_chunk, pair_cnt, samples, leaf_tin, prm,
                                    make_key(seed), out_off, out, seq, max_len);
  note_launch();
}

// ------------------------------------------------------------ batched sequencing
__device__ __forceinline__ uint32_t batch_index(const uint32_t* __restrict__ off, uint32_t n, uint32_t x) {
  uint32_t lo = 0, hi = n;          // largest i < n with off[i] <= x
  while (hi - lo > 1) { const uint32_t mid = (lo + hi) >> 1; if (off[mid] <= x) lo = mid; else hi = mid; }
  return lo;
}

__global__ void k_seq_records_b(PlaceOut s, const uint16_t* __restrict__ inst_sorted, const uint32_t* __restrict__ n_dev,
                                uint32_t cap, SeqBatch b, SeqRec* __restrict__ recs) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cap || i >= *n_dev) return;
  const uint32_t e = b.inst[inst_sorted[i]].etin_off + s.edge[i];
  SeqRec r;
  r.locus = s.locus[i];
  r.tin = b.etin[e];
  r.tout = b.etout[e];
  r.info = uint32_t(s.allele[i]) | ((uint32_t(s.seq[i]) & 0x7fffu) << 16) | (uint32_t(s.kind[i]) << 31);
  recs[i] = r;
}

__global__ void k_tile_ranges_b(SeqBatch b, const SeqRec* __restrict__ recs) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= b.n_tiles_all) return;
  const uint32_t i = b.tile_inst[t];
  const uint32_t r0 = b.rec_off[i], nr = b.rec_off[i + 1] - r0;
  const uint32_t start = b.tile_start[t];
  b.rec_lo[t] = lower_bound_rec(recs + r0, nr, start);
  b.rec_hi[t] = lower_bound_rec(recs + r0, nr, start + b.tile_len[t] - 1 + b.inst[i].prm.span);
}

__global__ void k_tile_counts_b(SeqBatch b) {
  const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= b.n_cnt) return;
  const uint32_t i = batch_index(b.cnt_off, b.n_inst, gid);
  const SeqInst& in = b.inst[i];
  const uint32_t local = gid - b.cnt_off[i];
  tile_counts_one(local / in.n_blocks, local % in.n_blocks, b.blk_slot + in.blk_off, b.blk_index + in.blk_off,
                  b.c_first + in.slot_off, b.c_ntiles + in.slot_off, b.c_depth + in.slot_off,
                  b.c_nstarts + in.slot_off, b.c_id + in.slot_off, b.c_pairs + in.slot_off, in.T, in.n_tiles,
                  nullptr, nullptr, 0, b.keys[i], b.pair_cnt + in.pair_off);
}

// Persistent read kernel of a batch: each CTA takes work items from a global
// counter until none is left; an item is one (instance, sample, tile).
static_assert(sizeof(SeqParams) % 4 == 0 && sizeof(SeqParams) / 4 <= SEQ_THREADS, "SeqParams staging");

__global__ void __launch_bounds__(SEQ_THREADS, 4) k_reads_batch(SeqBatch b, const SeqRec* __restrict__ g_recs) {
  __shared__ ReadSmem sh;
  __shared__ SeqParams s_prm;        // the item's instance parameters, staged once per instance change
  __shared__ SeqSample s_sm;
  __shared__ Key s_key;
  __shared__ uint32_t s_item, s_inst, s_t, s_s, s_pairs, s_lo, s_nw, s_start, s_len, s_ce;
  __shared__ const SeqRec* s_recs;
  __shared__ uint64_t s_row;
  uint32_t cur = 0xffffffffu;        // instance whose parameters s_prm holds
  for (;;) {
    if (threadIdx.x == 0) {
      // decode the next work item once for the CTA
      const uint32_t item = atomicAdd(b.counter, 1u);
      s_item = item;
      if (item < b.n_items) {
        const uint32_t i = batch_index(b.item_off, b.n_inst, item);
        const SeqInst& in = b.inst[i];
        const uint32_t local = item - b.item_off[i];
        const uint32_t s = local / in.n_tiles, t = local % in.n_tiles, gt = in.tile_off + t;
        s_inst = i; s_t = t; s_s = s;
        s_lo = b.rec_lo[gt]; s_nw = b.rec_hi[gt] - s_lo;
        s_pairs = b.pair_cnt[in.pair_off + uint64_t(s) * in.n_tiles + t];
        s_start = b.tile_start[gt]; s_len = b.tile_len[gt]; s_ce = b.tile_end[gt];
        s_sm = b.samples[in.sample_off + s];
        s_key = b.keys[i];
        s_recs = g_recs + b.rec_off[i];
        s_row = in.count_off + uint64_t(s) * in.count_stride;
      }
    }
    __syncthreads();
    if (s_item >= b.n_items) return;
    const uint32_t i = s_inst;
    if (i != cur) {                  // block-uniform
      if (threadIdx.x < sizeof(SeqParams) / 4)
        reinterpret_cast<uint32_t*>(&s_prm)[threadIdx.x] =
            reinterpret_cast<const uint32_t*>(&b.inst[i].prm)[threadIdx.x];
      cur = i;
      __syncthreads();
    }
    read_tile(sh, s_recs, s_t, s_s, s_pairs, s_lo, s_nw, s_start, s_len, s_ce, s_sm, b.leaf_tin, s_prm, s_key,
              b.alt + s_row, b.depth + s_row);
    __syncthreads();
  }
}



__global__ void k_make_tiles(uint32_t n_slots, const uint32_t* __restrict__ c_first,
                             const uint32_t* __restrict__ c_ntiles, const uint32_t* __restrict__ c_start,
                             const uint32_t* __restrict__ c_nstarts, const uint32_t* __restrict__ c_end, uint32_t T,
                             uint32_t n_tiles, uint32_t* __restrict__ start, uint32_t* __restrict__ len,
                             uint32_t* __restrict__ end) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_tiles) return;
  uint32_t lo = 0, hi = n_slots;          // last slot whose first tile is <= t
  while (hi - lo > 1) { const uint32_t mid = (lo + hi) >> 1; if (c_first[mid] <= t) lo = mid; else hi = mid; }
  const uint32_t k = t - c_first[lo];
  start[t] = c_start[lo] + k * T;
  len[t] = min(T, c_nstarts[lo] - k * T);
  end[t] = c_end[lo];
  (void)c_ntiles;
}

// last atom starting at or before position a
__device__ __forceinline__ uint32_t atom_of(const uint32_t* __restrict__ atom_start, uint32_t n_atoms, uint32_t a) {
  uint32_t lo = 0, hi = n_atoms;
  while (hi - lo > 1) { const uint32_t mid = (lo + hi) >> 1; if (atom_start[mid] <= a) lo = mid; else hi = mid; }
  return lo;
}

__global__ void k_part_counts(uint32_t n_tiles, const uint32_t* __restrict__ tile_start,
                              const uint32_t* __restrict__ tile_len, const uint32_t* __restrict__ atom_start,
                              uint32_t n_atoms, uint32_t* __restrict__ cnt) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_tiles) return;
  const uint32_t a = tile_start[t], b = a + tile_len[t];
  uint32_t x = atom_of(atom_start, n_atoms, a), n = 0;
  for (; x < n_atoms && atom_start[x] < b; ++x) ++n;
  cnt[t] = n;
}

__global__ void k_part_emit(uint32_t n_tiles, const uint32_t* __restrict__ tile_start,
                            const uint32_t* __restrict__ tile_len, const uint32_t* __restrict__ atom_start,
                            uint32_t n_atoms, uint32_t genome_len, const uint32_t* __restrict__ part_off,
                            uint32_t* __restrict__ part_start, uint32_t* __restrict__ part_len,
                            uint32_t* __restrict__ part_atom) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_tiles) return;
  const uint32_t a = tile_start[t], b = a + tile_len[t];
  uint32_t q = part_off[t];
  for (uint32_t x = atom_of(atom_start, n_atoms, a); x < n_atoms && atom_start[x] < b; ++x, ++q) {
    const uint32_t lo = max(a, atom_start[x]);
    const uint32_t hi = min(b, x + 1 < n_atoms ? atom_start[x + 1] : genome_len);
    part_start[q] = lo; part_len[q] = hi - lo; part_atom[q] = x;
  }
}

// mass of one stretch of starts with integer copy sums (i0, sum)
__device__ __forceinline__ double stretch_mass(double wn, double wt, uint64_t nl, uint64_t i0, uint64_t sum) {
  double m = wn * double(i0);
  if (nl > 0) m = m + (wt / double(nl)) * double(sum);
  return m;
}

// one thread per (sample, tile): the tile's mass and, for tiles of several
// parts, the thresholds floor(CDF * 2^31) of the part draw with the last
// part of positive mass at 2^31 (the host's cdf_thresholds)
__global__ void k_tile_mass(uint32_t n_samples, uint32_t n_tiles, const uint32_t* __restrict__ part_off,
                            const uint32_t* __restrict__ part_len, const uint32_t* __restrict__ part_atom,
                            uint32_t n_atoms, const double* __restrict__ wn_s, const double* __restrict__ wt_s,
                            const uint64_t* __restrict__ nl_s, const uint64_t* __restrict__ icnt0,
                            const uint64_t* __restrict__ copy_sum, uint32_t n_parts, uint64_t* __restrict__ tile_i0,
                            uint64_t* __restrict__ tile_s, uint32_t* __restrict__ part_cdf) {
  const uint64_t gid = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (gid >= uint64_t(n_samples) * n_tiles) return;
  const uint32_t s = uint32_t(gid / n_tiles), t = uint32_t(gid % n_tiles);
  const double wn = wn_s[s], wt = wt_s[s];
  const uint64_t nl = nl_s[s];
  const uint64_t* i0a = icnt0 + uint64_t(s) * n_atoms;
  const uint64_t* sa = copy_sum + uint64_t(s) * n_atoms;
  const uint32_t pb = part_off[t], pe = part_off[t + 1];
  uint64_t i0 = 0, sum = 0;
  for (uint32_t q = pb; q < pe; ++q) {
    const uint64_t len = part_len[q], x = part_atom[q];
    i0 += len * i0a[x];
    sum += len * sa[x];
  }
  if (pe - pb > 1) {
    double tot = 0.0;
    uint32_t last = pb;
    for (uint32_t q = pb; q < pe; ++q) {
      const uint64_t len = part_len[q], x = part_atom[q];
      const double w = stretch_mass(wn, wt, nl, len * i0a[x], len * sa[x]);
      tot += w;
      if (w > 0) last = q;
    }
    uint32_t* thr = part_cdf + uint64_t(s) * n_parts;
    double c = 0.0;
    for (uint32_t q = pb; q < pe; ++q) {
      const uint64_t len = part_len[q], x = part_atom[q];
      c += stretch_mass(wn, wt, nl, len * i0a[x], len * sa[x]);
      if (!(tot > 0)) { thr[q] = 0u; continue; }
      double v = floor(c / tot * 2147483648.0);
      if (v > 2147483648.0) v = 2147483648.0;
      thr[q] = (q >= last) ? 2147483648u : uint32_t(v);
    }
  }
  tile_i0[gid] = i0;
  tile_s[gid] = sum;
}

// one CTA per (sample, chromosome slot): the integer copy sums before each
// tile by an exclusive block scan (exact, so independent of the order of
// the additions), and the mass before each tile as the mass of those sums
constexpr uint32_t MASS_PER_THREAD = 4;
__global__ void __launch_bounds__(256) k_mass_prefix(uint32_t n_slots, const uint32_t* __restrict__ c_first,
                                                     const uint32_t* __restrict__ c_ntiles, uint32_t n_tiles,
                                                     const double* __restrict__ wn_s, const double* __restrict__ wt_s,
                                                     const uint64_t* __restrict__ nl_s,
                                                     const uint64_t* __restrict__ tile_i0,
                                                     const uint64_t* __restrict__ tile_s,
                                                     double* __restrict__ mass_cum, double* __restrict__ mass_tot) {
  __shared__ uint64_t w_i0[8], w_s[8];
  __shared__ uint64_t carry_i0, carry_s;
  const uint32_t s = blockIdx.x / n_slots, slot = blockIdx.x % n_slots;
  const uint32_t first = c_first[slot], nt = c_ntiles[slot];
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const double wn = wn_s[s], wt = wt_s[s];
  const uint64_t nl = nl_s[s];
  const uint64_t base = uint64_t(s) * n_tiles + first;
  if (threadIdx.x == 0) { carry_i0 = 0; carry_s = 0; }
  __syncthreads();
  constexpr uint32_t CH = 256 * MASS_PER_THREAD;
  for (uint32_t c0 = 0; c0 < nt; c0 += CH) {
    uint64_t a[MASS_PER_THREAD], b[MASS_PER_THREAD], ta = 0, tb = 0;
#pragma unroll
    for (uint32_t q = 0; q < MASS_PER_THREAD; ++q) {
      const uint32_t t = c0 + threadIdx.x * MASS_PER_THREAD + q;
      a[q] = t < nt ? tile_i0[base + t] : 0;
      b[q] = t < nt ? tile_s[base + t] : 0;
      ta += a[q];
      tb += b[q];
    }
    // exclusive scan of the threads' sums: warp, then warps
    uint64_t ia = ta, ib = tb;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint64_t xa = __shfl_up_sync(0xffffffffu, ia, o), xb = __shfl_up_sync(0xffffffffu, ib, o);
      if (lane >= uint32_t(o)) { ia += xa; ib += xb; }
    }
    if (lane == 31) { w_i0[warp] = ia; w_s[warp] = ib; }
    __syncthreads();
    uint64_t pa = carry_i0, pb = carry_s;
    for (uint32_t w = 0; w < warp; ++w) { pa += w_i0[w]; pb += w_s[w]; }
    pa += ia - ta;
    pb += ib - tb;
#pragma unroll
    for (uint32_t q = 0; q < MASS_PER_THREAD; ++q) {
      const uint32_t t = c0 + threadIdx.x * MASS_PER_THREAD + q;
      if (t < nt) mass_cum[base + t] = stretch_mass(wn, wt, nl, pa, pb);
      pa += a[q];
      pb += b[q];
    }
    __syncthreads();
    if (threadIdx.x == 255) { carry_i0 = pa; carry_s = pb; }
    __syncthreads();
  }
  if (threadIdx.x == 0) mass_tot[uint64_t(s) * n_slots + slot] = stretch_mass(wn, wt, nl, carry_i0, carry_s);
}

void seq_tile_parts(uint32_t n_tiles, const uint32_t* tile_start, const uint32_t* tile_len,
                    const uint32_t* atom_start, uint32_t n_atoms, uint32_t genome_len, uint32_t* part_off,
                    uint32_t* scan_part, uint32_t* part_start, uint32_t* part_len, uint32_t* part_atom,
                    cudaStream_t st) {
  if (!n_tiles) return;
  k_part_counts<<<nblk(n_tiles), 256, 0, st>>>(n_tiles, tile_start, tile_len, atom_start, n_atoms, part_off);
  note_launch();
  scan_rows<uint32_t>(part_off, part_off, n_tiles, 1, scan_part, part_off + n_tiles, st);
  k_part_emit<<<nblk(n_tiles), 256, 0, st>>>(n_tiles, tile_start, tile_len, atom_start, n_atoms, genome_len,
                                             part_off, part_start, part_len, part_atom);
  note_launch();
}

void seq_tile_mass(uint32_t n_samples, uint32_t n_slots, const uint32_t* c_first, const uint32_t* c_ntiles,
                   const uint32_t* part_off, const uint32_t* part_len, const uint32_t* part_atom, uint32_t n_atoms,
                   const double* wn, const double* wt, const uint64_t* nl, const uint64_t* icnt0,
                   const uint64_t* copy_sum, uint32_t n_tiles, uint32_t n_parts, uint64_t* tile_sums,
                   double* mass_cum, double* mass_tot, uint32_t* part_cdf, cudaStream_t st) {
  const uint64_t n = uint64_t(n_samples) * n_tiles;
  if (!n) return;
  k_tile_mass<<<nblk(n), 256, 0, st>>>(n_samples, n_tiles, part_off, part_len, part_atom, n_atoms, wn, wt, nl, icnt0,
                                       copy_sum, n_parts, tile_sums, tile_sums + n, part_cdf);
  k_mass_prefix<<<n_samples * n_slots, 256, 0, st>>>(n_slots, c_first, c_ntiles, n_tiles, wn, wt, nl, tile_sums,
                                                     tile_sums + n, mass_cum, mass_tot);
  note_launch(2);
}

void seq_make_tiles(uint32_t n_slots, const uint32_t* c_first, const uint32_t* c_ntiles, const uint32_t* c_start,
                    const uint32_t* c_nstarts, const uint32_t* c_end, uint32_t T, uint32_t n_tiles, uint32_t* start,
                    uint32_t* len, uint32_t* end, cudaStream_t st) {
  if (n_tiles) { k_make_tiles<<<nblk(n_tiles), 256, 0, st>>>(n_slots, c_first, c_ntiles, c_start, c_nstarts, c_end, T,
                                                             n_tiles, start, len, end); note_launch(); }
}

void seq_build_records(const PlaceOut& sorted, uint32_t n, const uint32_t* edge_tin, const uint32_t* edge_tout,
                       SeqRec* recs, cudaStream_t st) {
  if (n) { k_seq_records<<<nblk(n), 256, 0, st>>>(sorted, n, edge_tin, edge_tout, recs); note_launch(); }
}

void seq_tile_ranges(const SeqRec* recs, uint32_t n_recs, const uint32_t* start, const uint32_t* len,
                     uint32_t n_tiles, uint32_t span, uint32_t* rlo, uint32_t* rhi, cudaStream_t st) {
  if (n_tiles) { k_tile_ranges<<<nblk(n_tiles), 256, 0, st>>>(recs, n_recs, start, len, n_tiles, span, rlo, rhi); note_launch(); }
}

void seq_tile_counts(uint32_t n_samples, uint32_t n_slots, uint32_t max_depth, const uint32_t* chr_first_tile,
                     const uint32_t* chr_ntiles, const uint32_t* chr_depth, const uint32_t* chr_nstarts,
                     const uint32_t* chr_id, const uint64_t* chr_pairs, const uint64_t* heap_base,
                     uint64_t heap_total, uint32_t* heap, uint32_t tile_size, uint32_t n_tiles,
                     const double* mass_cum, const double* mass_tot, uint64_t seed, uint32_t* pair_cnt,
                     cudaStream_t st) {
  if (n_samples == 0 || n_slots == 0) return;
  const Key key = make_key(seed);
  for (uint32_t level = 0; level < std::max<uint32_t>(max_depth, 1); ++level) {
    const dim3 grid(nblk(uint64_t(1) << level, SPLIT_THREADS), n_slots, n_samples);
    k_tile_split_level<<<grid, SPLIT_THREADS, 0, st>>>(level, n_slots, chr_first_tile, chr_ntiles, chr_depth, chr_nstarts,
                                             chr_id, chr_pairs, heap_base, heap_total, tile_size, n_tiles, mass_cum,
                                             mass_tot, key, heap, pair_cnt);
    note_launch();
  }
}

// ------------------------------------------------------------ observed rows
// The rows of the result a caller reads by default: mutations with an alt
// read in some sample (src/seq_simulation.cpp:52-90 keeps those unless
// include_non_sequenced_mutations).  Flags, their exclusive scan, then the
// compact [sample][row] tables and the rows' mutation indices.
__global__ void k_active_flags(const uint32_t* __restrict__ alt, uint32_t n_samples, uint64_t M,
                               uint32_t* __restrict__ flag) {
  const uint64_t m = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (m >= M) return;
  uint32_t any = 0;
  for (uint32_t s = 0; s < n_samples; ++s) any |= alt[uint64_t(s) * M + m];
  flag[m] = any ? 1u : 0u;
}

__global__ void k_active_gather(const uint32_t* __restrict__ alt, const uint32_t* __restrict__ depth,
                                uint32_t n_samples, uint64_t M, const uint32_t* __restrict__ pos, uint32_t n_active,
                                uint32_t* __restrict__ index, uint32_t* __restrict__ a_out,
                                uint32_t* __restrict__ d_out) {
  const uint64_t m = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (m >= M) return;
  const uint32_t p = pos[m];
  if ((m + 1 < M ? pos[m + 1] : n_active) == p) return;   // not observed
  index[p] = uint32_t(m);
  for (uint32_t s = 0; s < n_samples; ++s) {
    a_out[uint64_t(s) * n_active + p] = alt[uint64_t(s) * M + m];
    d_out[uint64_t(s) * n_active + p] = depth[uint64_t(s) * M + m];
  }
}

void seq_active_flags(const uint32_t* alt, uint32_t n_samples, uint64_t M, uint32_t* flag, cudaStream_t st) {
  if (M) { k_active_flags<<<nblk(M), 256, 0, st>>>(alt, n_samples, M, flag); note_launch(); }
}

void seq_active_gather(const uint32_t* alt, const uint32_t* depth, uint32_t n_samples, uint64_t M, const uint32_t* pos,
                       uint32_t n_active, uint32_t* index, uint32_t* a_out, uint32_t* d_out, cudaStream_t st) {
  if (M && n_active) {
    k_active_gather<<<nblk(M), 256, 0, st>>>(alt, depth, n_samples, M, pos, n_active, index, a_out, d_out);
    note_launch();
  }
}

void seq_reads(const SeqRec* recs, uint32_t n_recs, const SeqTiles& tiles, const uint32_t* pair_cnt,
               const SeqSample* samples, uint32_t n_samples, const uint32_t* leaf_tin, const SeqParams& prm,
               uint64_t seed, uint32_t* alt, uint32_t* depth, cudaStream_t st) {
  if (tiles.n_tiles == 0 || n_samples == 0 || n_recs == 0) return;
  dim3 grid(tiles.n_tiles, n_samples);
  const Key k = make_key(seed);
  k_reads<<<grid, SEQ_THREADS, 0, st>>>(recs, tiles, pair_cnt, samples, leaf_tin, prm, round_keys(k.k0, k.k1), n_recs,
                                         alt, depth); note_launch();
}

void seq_batch_records(const PlaceOut& sorted, const uint16_t* inst_sorted, const uint32_t* n_dev, uint32_t cap,
                       const SeqBatch& b, SeqRec* recs, cudaStream_t st) {
  if (cap) { k_seq_records_b<<<nblk(cap), 256, 0, st>>>(sorted, inst_sorted, n_dev, cap, b, recs); note_launch(); }
}

int seq_reads_batch_occupancy() {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_reads_batch, SEQ_THREADS, 0) != cudaSuccess) return 1;
  return n;
}

void seq_batch_reads(const SeqBatch& b, const SeqRec* recs, uint32_t grid, cudaStream_t st) {
  if (b.n_cnt) { k_tile_counts_b<<<nblk(b.n_cnt, 64), 64, 0, st>>>(b); note_launch(); }
  if (b.n_tiles_all) { k_tile_ranges_b<<<nblk(b.n_tiles_all), 256, 0, st>>>(b, recs); note_launch(); }
  cudaMemsetAsync(b.counter, 0, sizeof(uint32_t), st);
  if (b.n_items) { k_reads_batch<<<grid, SEQ_THREADS, 0, st>>>(b, recs); note_launch(); }
}
}  // namespace pg
