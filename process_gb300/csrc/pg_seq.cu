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
//     does not carry it and an error turns the reference into that alt base
//     (probability err/3).  Indels are not affected by substitution errors.
//
// Kernel layout: one CTA per (tile, sample).  The CTA stages the sorted
// mutation records of its window [tile start, tile end + span) in shared
// memory, keeps alt/depth counters there (block-private bins, shared-memory
// atomics), and flushes them to HBM once.  Windows larger than the shared
// capacity run the same loop on the global arrays.
#include "pg_common.cuh"
#include "pg_rng.cuh"
#include "pg_kernels.h"

namespace pg {

constexpr int SEQ_THREADS = 256;
constexpr uint32_t SEQ_CAP = 1024;   // mutation records staged per CTA

__global__ void k_seq_records(PlaceOut s, uint32_t n, const uint32_t* __restrict__ edge_tin,
                              const uint32_t* __restrict__ edge_tout, SeqRec* __restrict__ recs) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t e = s.edge[i];
  SeqRec r;
  r.locus = s.locus[i];
  r.tin = edge_tin[e];
  r.tout = edge_tout[e];
  r.info = uint32_t(s.allele[i]) | (uint32_t(s.kind[i]) << 8);
  recs[i] = r;
}

__global__ void k_tile_counts(uint32_t n_samples, uint32_t n_tiles, const uint32_t* __restrict__ tile_slot,
                              const uint32_t* __restrict__ tile_idx, const uint32_t* __restrict__ chr_ntiles,
                              const uint32_t* __restrict__ chr_nstarts, const uint32_t* __restrict__ chr_id,
                              const uint64_t* __restrict__ chr_pairs, uint32_t T, Key key,
                              uint32_t* __restrict__ pair_cnt) {
  const uint64_t gid = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (gid >= uint64_t(n_tiles) * n_samples) return;
  const uint32_t s = uint32_t(gid / n_tiles), t = uint32_t(gid % n_tiles);
  const uint32_t slot = tile_slot[t], idx = tile_idx[t];
  const uint64_t S = chr_nstarts[slot];
  uint64_t n = chr_pairs[slot];
  uint32_t lo = 0, hi = chr_ntiles[slot], node = 1;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    const uint64_t a = uint64_t(lo) * T;
    const uint64_t bm = uint64_t(mid) * T < S ? uint64_t(mid) * T : S;
    const uint64_t bh = uint64_t(hi) * T < S ? uint64_t(hi) * T : S;
    const double p = double(bm - a) / double(bh - a);
    Stream st{key, node, chr_id[slot], s, TAG_TILE_SPLIT, 0u};
    const uint64_t nl = binomial(st, n, p);
    if (idx < mid) { n = nl; hi = mid; node = 2 * node; }
    else { n = n - nl; lo = mid; node = 2 * node + 1; }
  }
  pair_cnt[gid] = uint32_t(n);
}

template <bool SMEM>
__device__ __forceinline__ void visit_mate(const SeqRec* __restrict__ recs, uint32_t nw, uint32_t* alt, uint32_t* dep,
                                           uint32_t a, uint32_t R, uint32_t cell, uint32_t allele,
                                           uint32_t err_thr, Key key, uint32_t j, uint32_t t, uint32_t s,
                                           uint32_t& q, U4& eblk) {
  // first record with locus >= a
  uint32_t lo = 0, hi = nw;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (recs[mid].locus < a) lo = mid + 1; else hi = mid;
  }
  for (uint32_t i = lo; i < nw; ++i) {
    const SeqRec r = recs[i];
    if (r.locus >= a + R) break;
    const bool carried = (r.tin <= cell) && (cell < r.tout) && ((r.info & 0xffu) == allele);
    bool obs;
    if ((r.info >> 8) & 1u) {
      obs = carried;
    } else {
      if ((q & 1u) == 0) eblk = philox(key.k0, key.k1, j, t, s, TAG_ERR | ((q >> 1) << 8));
      const uint32_t ew = (q & 1u) ? eblk.z : eblk.x;
      const uint32_t bw = (q & 1u) ? eblk.w : eblk.y;
      ++q;
      const bool err = ew < err_thr;
      obs = carried ? !err : (err && __umulhi(bw, 3u) == 0u);
    }
    atomicAdd(dep + i, 1u);
    if (obs) atomicAdd(alt + i, 1u);
  }
}

__global__ void __launch_bounds__(SEQ_THREADS) k_reads(const SeqRec* __restrict__ g_recs, uint32_t n_recs,
                                                       SeqTiles tiles, const uint32_t* __restrict__ pair_cnt,
                                                       const SeqSample* __restrict__ samples,
                                                       const uint32_t* __restrict__ leaf_tin, SeqParams prm,
                                                       Key key, uint32_t* __restrict__ g_alt,
                                                       uint32_t* __restrict__ g_dep) {
  __shared__ SeqRec s_rec[SEQ_CAP];
  __shared__ uint32_t s_alt[SEQ_CAP], s_dep[SEQ_CAP];
  __shared__ uint32_t s_lo, s_hi;
  const uint32_t t = blockIdx.x, s = blockIdx.y;
  const uint32_t n_pairs = pair_cnt[uint64_t(s) * tiles.n_tiles + t];
  const uint32_t start = tiles.start[t], len = tiles.len[t], ce = tiles.chr_end[t];
  const uint32_t R = prm.read_len;
  if (threadIdx.x < 2) {
    const uint32_t key_pos = threadIdx.x == 0 ? start : start + len - 1 + prm.span;
    uint32_t lo = 0, hi = n_recs;
    while (lo < hi) { const uint32_t mid = (lo + hi) >> 1; if (g_recs[mid].locus < key_pos) lo = mid + 1; else hi = mid; }
    if (threadIdx.x == 0) s_lo = lo; else s_hi = lo;
  }
  __syncthreads();
  const uint32_t lo = s_lo, nw = s_hi - s_lo;
  if (nw == 0 || n_pairs == 0) return;       // nothing to count in this window
  const bool smem = nw <= SEQ_CAP;
  if (smem) {
    for (uint32_t i = threadIdx.x; i < nw; i += SEQ_THREADS) { s_rec[i] = g_recs[lo + i]; s_alt[i] = 0; s_dep[i] = 0; }
  }
  __syncthreads();
  const SeqSample sm = samples[s];
  const uint64_t M = n_recs;
  uint32_t* galt = g_alt + uint64_t(s) * M + lo;
  uint32_t* gdep = g_dep + uint64_t(s) * M + lo;
  for (uint32_t j = threadIdx.x; j < n_pairs; j += SEQ_THREADS) {
    const U4 r = philox(key.k0, key.k1, j, t, s, TAG_PAIR);
    const uint32_t p0 = start + __umulhi(r.x, len);
    const bool normal = sm.all_normal || r.y < sm.normal_thr;
    const uint32_t cell = normal ? prm.normal_tin : __ldg(leaf_tin + sm.leaf_off + __umulhi(r.z, sm.n_leaves));
    const uint32_t allele = __umulhi(r.w, prm.n_alleles);
    uint32_t q = 0;
    U4 eblk{0, 0, 0, 0};
    if (smem) visit_mate<true>(s_rec, nw, s_alt, s_dep, p0, R, cell, allele, prm.err_thr, key, j, t, s, q, eblk);
    else visit_mate<false>(g_recs + lo, nw, galt, gdep, p0, R, cell, allele, prm.err_thr, key, j, t, s, q, eblk);
    if (prm.paired) {
      const U4 r2 = philox(key.k0, key.k1, j, t, s, TAG_PAIR2);
      const uint32_t ins = prm.ins_min + cdf_lookup(prm.ins_cdf, prm.n_ins, r2.x);
      uint32_t p1 = p0 + ins - R;
      if (p1 > ce - R) p1 = ce - R;
      if (smem) visit_mate<true>(s_rec, nw, s_alt, s_dep, p1, R, cell, allele, prm.err_thr, key, j, t, s, q, eblk);
      else visit_mate<false>(g_recs + lo, nw, galt, gdep, p1, R, cell, allele, prm.err_thr, key, j, t, s, q, eblk);
    }
  }
  if (smem) {
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < nw; i += SEQ_THREADS) {
      const uint32_t d = s_dep[i];
      if (d) {
        atomicAdd(gdep + i, d);
        const uint32_t a = s_alt[i];
        if (a) atomicAdd(galt + i, a);
      }
    }
  }
}

static inline unsigned nblk(uint64_t n, int b = 256) { return unsigned((n + b - 1) / b); }

void seq_build_records(const PlaceOut& sorted, uint32_t n, const uint32_t* edge_tin, const uint32_t* edge_tout,
                       SeqRec* recs, cudaStream_t st) {
  if (n) { k_seq_records<<<nblk(n), 256, 0, st>>>(sorted, n, edge_tin, edge_tout, recs); note_launch(); }
}

void seq_tile_counts(uint32_t n_samples, uint32_t n_tiles, const uint32_t* tile_chr_slot,
                     const uint32_t* tile_idx_in_chr, const uint32_t* chr_ntiles, const uint32_t* chr_nstarts,
                     const uint32_t* chr_id, const uint64_t* chr_pairs, uint32_t tile_size, uint64_t seed,
                     uint32_t* pair_cnt, cudaStream_t st) {
  const uint64_t n = uint64_t(n_samples) * n_tiles;
  if (n) { k_tile_counts<<<nblk(n, 128), 128, 0, st>>>(n_samples, n_tiles, tile_chr_slot, tile_idx_in_chr, chr_ntiles,
                                                     chr_nstarts, chr_id, chr_pairs, tile_size, make_key(seed),
                                                     pair_cnt); note_launch(); }
}

void seq_reads(const SeqRec* recs, uint32_t n_recs, const SeqTiles& tiles, const uint32_t* pair_cnt,
               const SeqSample* samples, uint32_t n_samples, const uint32_t* leaf_tin, const SeqParams& prm,
               uint64_t seed, uint32_t* alt, uint32_t* depth, cudaStream_t st) {
  if (tiles.n_tiles == 0 || n_samples == 0 || n_recs == 0) return;
  dim3 grid(tiles.n_tiles, n_samples);
  k_reads<<<grid, SEQ_THREADS, 0, st>>>(recs, n_recs, tiles, pair_cnt, samples, leaf_tin, prm, make_key(seed), alt,
                                         depth); note_launch();
}

}  // namespace pg
