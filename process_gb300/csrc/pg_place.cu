// Mutation placement on a samples forest.
//
// Reference call site: MutationEngine::place_mutations
// (src/mutation_engine.cpp:1085-1113) -> RACES
// MutationEngine<uint32_t, std::mt19937_64>::place_mutations (absent; model
// restated here and in oracle/).
//
// Model (one draw function per decision, all keyed Philox):
//   * edge v of the forest carries divisions d_v >= 1; division j happens at
//     t = t_parent + (t_v - t_parent) * (j+1)/d_v (roots: t_v), and belongs to
//     the exposure epoch whose start time is the last one <= t.
//   * passenger SNVs (indels) on (v, epoch e):
//       Poisson(rate[species_v][e] * allelic_size * divisions_in_e)
//     (per-species passenger rates: src/mutation_engine.cpp:864-1083; timed
//     exposures: :734-739).  The preneoplastic edge (index N) carries exactly
//     the requested numbers, drawn from the named signature
//     (src/mutation_engine.hpp:160-206).
//   * each mutation draws its signature from the epoch exposure, its class
//     from the signature, a position uniformly from the class's position list,
//     and an allele uniformly among the cell's alleles.
//   * infinite sites (src/mutation_engine.hpp:148-156): loci are unique over
//     the forest; colliding mutations keep their class and redraw the
//     position (attempt a uses Philox block 1+a), the lowest slot index wins
//     a contested locus, rounds repeat until no collision is left.  From
//     attempt RECLASS_ATTEMPTS on, the class is redrawn too (same signature),
//     so a class whose positions are all taken cannot stall the rounds.
#include <algorithm>

#include "pg_common.cuh"
#include "pg_rng.cuh"
#include "pg_scan.cuh"
#include "pg_kernels.h"

namespace pg {

constexpr uint32_t RECLASS_ATTEMPTS = 4;

// ------------------------------------------------------------ per-edge counts
// counts of edge v (v == n_nodes: the preneoplastic edge) into
// cnt_*[v * n_epochs + e]
__device__ __forceinline__ void edge_counts_one(const PlaceTables& t, uint32_t v, Key key, uint32_t* __restrict__ cnt_snv,
                                                uint32_t* __restrict__ cnt_id, uint32_t n_pre_snv,
                                                uint32_t n_pre_id) {
  const uint32_t N = t.n_nodes, E = t.n_epochs;
  if (v == N) {  // preneoplastic edge
    for (uint32_t e = 0; e < E; ++e) {
      cnt_snv[uint64_t(v) * E + e] = e == 0 ? n_pre_snv : 0u;
      cnt_id[uint64_t(v) * E + e] = e == 0 ? n_pre_id : 0u;
    }
    return;
  }
  const double tv = t.birth[v];
  const int par = t.parent[v];
  const double tu = par >= 0 ? t.birth[par] : tv;
  const uint32_t d = t.divisions[v];
  const uint32_t sp = t.species[v];
  uint32_t ndiv[MAX_EPOCHS];
  for (uint32_t e = 0; e < E; ++e) ndiv[e] = 0;
  for (uint32_t j = 0; j < d; ++j) {
    const double tj = tu + (tv - tu) * (double(j + 1) / double(d));
    uint32_t e = 0;
    while (e + 1 < E && t.epoch_start[e + 1] <= tj) ++e;
    ndiv[e] += 1;
  }
  const double A = t.node_size[v];   // allelic size of the edge's genome
  for (uint32_t e = 0; e < E; ++e) {
    const double lam_s = t.snv_rate[sp * E + e] * A * double(ndiv[e]);
    const double lam_i = t.indel_rate[sp * E + e] * A * double(ndiv[e]);
    Stream s1{key, e, v, 0u, TAG_EDGE_SNV, 0u};
    Stream s2{key, e, v, 0u, TAG_EDGE_INDEL, 0u};
    cnt_snv[uint64_t(v) * E + e] = uint32_t(poisson(s1, lam_s));
    cnt_id[uint64_t(v) * E + e] = uint32_t(poisson(s2, lam_i));
  }
}

__global__ void k_edge_counts(PlaceTables t, uint32_t* __restrict__ cnt_snv, uint32_t* __restrict__ cnt_id,
                              Key key, uint32_t n_pre_snv, uint32_t n_pre_id) {
  const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v > t.n_nodes) return;
  edge_counts_one(t, v, key, cnt_snv, cnt_id, n_pre_snv, n_pre_id);
}

// passenger CNA events per edge: Poisson(rate_cna[species] * 2G * divisions);
// the germline size is used so that the counts do not depend on the copy
// number the events themselves create
__global__ void k_cna_counts(PlaceTables t, uint32_t* __restrict__ cnt_cna, Key key, double germline_size) {
  const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= t.n_nodes) return;
  const double lam = t.cna_rate[t.species[v]] * germline_size * double(t.divisions[v]);
  Stream st{key, 0u, v, 0u, TAG_EDGE_CNA, 0u};
  cnt_cna[v] = uint32_t(poisson(st, lam));
}

// ------------------------------------------------------------ placement
__device__ __forceinline__ uint32_t find_cell(const uint32_t* __restrict__ off, uint32_t ncell, uint32_t i) {
  // largest q with off[q] <= i (off is the exclusive scan of the counts)
  uint32_t lo = 0, hi = ncell;
  while (hi - lo > 1) { const uint32_t mid = (lo + hi) >> 1; if (off[mid] <= i) lo = mid; else hi = mid; }
  return lo;
}

// Placement of slot i (first placement when redraw==0: class and position;
// redraw: position only, with attempt+1).  kind 0 = SNV slots [0, n_snv),
// kind 1 = indel slots [n_snv, n_snv+n_id).
// Mutation m of (edge v, epoch e), SNV or indel, written at `slot` of o.
__device__ __forceinline__ void place_one(const PlaceTables& t, const PlaceOut& o, Key key, uint32_t slot, bool is_id,
                                          uint32_t v, uint32_t e, uint32_t m, int redraw,
                                          uint32_t* __restrict__ err) {
  Stream st{key, m, v, e, is_id ? TAG_INDEL : TAG_SNV, 0u};
  uint32_t cls, sig;
  if (!redraw) {
    const U4 r = st.next();
    const uint32_t row = (v == t.n_nodes) ? t.n_epochs : e;
    if (!is_id) {
      sig = cdf_lookup(t.sbs_expo_cdf + row * t.n_sbs_sigs, t.n_sbs_sigs, r.x);
      cls = cdf_lookup(t.sbs_sig_cdf + sig * N_SBS, N_SBS, r.y);
    } else {
      sig = cdf_lookup(t.id_expo_cdf + row * t.n_id_sigs, t.n_id_sigs, r.x);
      cls = cdf_lookup(t.id_sig_cdf + sig * N_ID, N_ID, r.y);
    }
    o.cls[slot] = uint8_t(cls);
    o.sig[slot] = uint8_t(sig);
    o.edge[slot] = v;
    o.nature[slot] = (v == t.n_nodes) ? NATURE_PRENEOPLASTIC : NATURE_PASSENGER;
    o.kind[slot] = is_id ? KIND_INDEL : KIND_SNV;
    o.seq[slot] = (v == t.n_nodes) ? SEQ_PRENEOPLASTIC : SEQ_PASSENGER;
    o.attempt[slot] = 0;
  } else {
    cls = o.cls[slot];
    o.attempt[slot] += 1;
  }
  const uint32_t attempt = o.attempt[slot];
  st.block = 1u + attempt;
  const U4 r = st.next();
  if (attempt >= RECLASS_ATTEMPTS) {
    // the class keeps colliding (its free positions may be exhausted): redraw
    // the class from the same signature with word w
    sig = o.sig[slot];
    cls = is_id ? cdf_lookup(t.id_sig_cdf + sig * N_ID, N_ID, r.w) : cdf_lookup(t.sbs_sig_cdf + sig * N_SBS, N_SBS, r.w);
    o.cls[slot] = uint8_t(cls);
  }
  const uint32_t list = is_id ? cls : uint32_t(sbs_class_context(int(cls)));
  const uint32_t len = is_id ? t.id_len[list] : t.ctx_len[list];
  if (len == 0) { atomicOr(err, ERR_EMPTY_CLASS); o.locus[slot] = 0; return; }
  const uint64_t j = uniform_index64(r.x, r.y, len);
  const uint32_t p = is_id ? t.id_lists[t.id_off[list] + j] : t.ctx_lists[t.ctx_off[list] + j];
  // the allele: uniform among the instances of the edge's genome covering the locus
  {
    const uint32_t loc = is_id ? p - 1 : p;
    uint32_t ioff = 0;
    const uint32_t n = covering(t.gc, t.gc.node_class[v], loc, &ioff);
    if (n == 0) { o.locus[slot] = LOCUS_INVALID; return; }   // deleted here: redrawn next round
    o.allele[slot] = t.gc.inst_list[ioff + uniform_index32(r.z, n)];
  }
  if (!is_id) {
    const uint32_t ref = base_at(t.genome, p);
    const uint32_t alt_pyr = sbs_class_alt(int(cls));
    const bool fwd = (ref == 1u || ref == 3u);
    o.locus[slot] = p;
    o.aux[slot] = fwd ? alt_pyr : 3u - alt_pyr;
  } else {
    // indel descriptor: bit0 insertion, bits1-3 length, bits 8.. inserted bases (2 bits each)
    uint32_t ins = 0, l = 1, bases = 0;
    if (cls < 12) { ins = 0; l = 1; }
    else if (cls < 24) {
      ins = 1; l = 1;
      const uint32_t idx = (cls - 12) % 6;
      if (idx >= 1) bases = base_at(t.genome, p);
      else bases = (cls < 18) ? ((r.w & 1u) ? 2u : 1u) : ((r.w & 1u) ? 0u : 3u);
    } else if (cls < 48) { ins = 0; l = (cls - 24) / 6 + 2; }
    else if (cls < 72) {
      ins = 1; l = (cls - 48) / 6 + 2;
      if ((cls - 48) % 6 >= 1) { for (uint32_t k = 0; k < l; ++k) bases |= base_at(t.genome, p + k) << (2 * k); }
      else bases = r.w & ((1u << (2 * l)) - 1u);
    } else {
      ins = 0; l = cls == 72 ? 2 : (cls < 75 ? 3 : (cls < 78 ? 4 : 5));
    }
    o.locus[slot] = p - 1;                       // anchor base
    o.aux[slot] = ins | (l << 1) | (bases << 8);
  }
}

// slot -> its (edge, epoch) cell and index there, then place_one
__device__ __forceinline__ void place_slot(const PlaceTables& t, const PlaceOut& o, Key key,
                                           const uint32_t* __restrict__ off_snv, const uint32_t* __restrict__ off_id,
                                           uint32_t n_snv, uint32_t slot, int redraw, uint32_t* __restrict__ err) {
  const bool is_id = slot >= n_snv;
  const uint32_t i = is_id ? slot - n_snv : slot;
  const uint32_t ncell = (t.n_nodes + 1) * t.n_epochs;
  const uint32_t* off = is_id ? off_id : off_snv;
  const uint32_t q = find_cell(off, ncell, i);
  place_one(t, o, key, slot, is_id, q / t.n_epochs, q % t.n_epochs, i - off[q], redraw, err);
}

__global__ void k_place(PlaceTables t, PlaceOut o, Key key, const uint32_t* __restrict__ off_snv,
                        const uint32_t* __restrict__ off_id, uint32_t n_snv, uint32_t n_id,
                        const uint32_t* __restrict__ pending, uint32_t n_pending,
                        const uint32_t* __restrict__ n_dev, int redraw, uint32_t* __restrict__ err) {
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= (n_dev ? *n_dev : n_pending)) return;
  place_slot(t, o, key, off_snv, off_id, n_snv, pending ? pending[tid] : tid, redraw, err);
}

// ------------------------------------------------------------ hash sets
__device__ __forceinline__ uint32_t hash32(uint32_t k) {
  k ^= k >> 16; k *= 0x7feb352du; k ^= k >> 15; k *= 0x846ca68bu; k ^= k >> 16;
  return k;
}
constexpr uint32_t EMPTY = 0xffffffffu;

__device__ __forceinline__ bool hset_contains(const uint32_t* __restrict__ keys, uint32_t mask, uint32_t k) {
  uint32_t h = hash32(k) & mask;
  for (uint32_t probe = 0; probe <= mask; ++probe) {
    const uint32_t x = keys[h];
    if (x == k) return true;
    if (x == EMPTY) return false;
    h = (h + 1) & mask;
  }
  return false;
}

// returns the slot index of key k, inserting it when absent
__device__ __forceinline__ uint32_t hset_insert(uint32_t* __restrict__ keys, uint32_t mask, uint32_t k) {
  uint32_t h = hash32(k) & mask;
  for (uint32_t probe = 0; probe <= mask; ++probe) {
    const uint32_t prev = atomicCAS(keys + h, EMPTY, k);
    if (prev == EMPTY || prev == k) return h;
    h = (h + 1) & mask;
  }
  return EMPTY;
}


// The first infinite-sites round over every slot, against one table of all
// its candidates: an entry is (locus << 32 | code), code 0 for a driver's
// locus and slot + 1 for a passenger's, and a locus keeps the smallest code.
// A passenger wins its locus when the entry holds its own code, i.e. when no
// driver and no smaller slot drew it: the rule of the later rounds (the
// smallest pending slot wins a free locus).  The table then holds exactly
// the taken loci (drivers and the round's winners), so the later rounds test
// it instead of inserting the winners into the accepted set.
// The losers are marked while inserting: a slot that finds a smaller code
// at its locus marks itself, one that replaces a larger code marks that
// code's slot, so every code but the final holder of each locus is marked.
constexpr unsigned long long FIRST_EMPTY = ~0ull;

__device__ __forceinline__ void first_insert(unsigned long long* __restrict__ tab, uint32_t mask, uint32_t k,
                                             uint32_t code, uint8_t* __restrict__ lost, uint32_t* __restrict__ err) {
  const unsigned long long mine = (static_cast<unsigned long long>(k) << 32) | code;
  uint32_t h = hash32(k) & mask;
  for (uint32_t probe = 0; probe <= mask; ++probe) {
    // the table is mostly empty: try the swap first (one round trip)
    const unsigned long long x = atomicCAS(tab + h, FIRST_EMPTY, mine);
    if (x == FIRST_EMPTY) return;
    if (uint32_t(x >> 32) == k) {
      unsigned long long old = x;
      if (x > mine) old = atomicMin(tab + h, mine);
      if (old < mine) {
        if (code) lost[code - 1] = 1;                     // a smaller code holds the locus
      } else if (old > mine) {
        const uint32_t oc = uint32_t(old);                // replaced: that code's slot loses
        if (oc) lost[oc - 1] = 1;
      }
      return;
    }
    h = (h + 1) & mask;
  }
  atomicOr(err, ERR_CAPACITY);
}

// the entry of locus k, or FIRST_EMPTY
__device__ __forceinline__ unsigned long long first_find(const unsigned long long* __restrict__ tab, uint32_t mask,
                                                         uint32_t k) {
  uint32_t h = hash32(k) & mask;
  for (uint32_t probe = 0; probe <= mask; ++probe) {
    const unsigned long long x = tab[h];
    if (x == FIRST_EMPTY || uint32_t(x >> 32) == k) return x;
    h = (h + 1) & mask;
  }
  return FIRST_EMPTY;
}

// lost: n flags, zeroed by the caller
__global__ void k_first_insert(const uint32_t* __restrict__ locus, uint32_t n, const uint32_t* __restrict__ drv_locus,
                               uint32_t n_drv, unsigned long long* __restrict__ tab, uint32_t mask,
                               uint8_t* __restrict__ lost, uint32_t* __restrict__ err) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n_drv) first_insert(tab, mask, drv_locus[i], 0u, lost, err);
  if (i >= n) return;
  const uint32_t k = locus[i];
  if (k == LOCUS_INVALID) lost[i] = 1;                   // no allele at the drawn position
  else first_insert(tab, mask, k, i + 1, lost, err);
}

// the marked slots, in no particular order (warp-aggregated appends)
// (one append per block of 256 slots)
__global__ void __launch_bounds__(256) k_first_collect(const uint8_t* __restrict__ lost, uint32_t n,
                                                       uint32_t* __restrict__ next, uint32_t* __restrict__ n_next) {
  __shared__ uint32_t s_cnt[8], s_base;
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const bool mine = i < n && lost[i];
  const uint32_t ballot = __ballot_sync(0xffffffffu, mine);
  if (lane == 0) s_cnt[warp] = __popc(ballot);
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t tot = 0;
    for (int w = 0; w < 8; ++w) { const uint32_t c = s_cnt[w]; s_cnt[w] = tot; tot += c; }
    s_base = tot ? atomicAdd(n_next, tot) : 0u;
  }
  __syncthreads();
  if (mine) next[s_base + s_cnt[warp] + __popc(ballot & ((1u << lane) - 1u))] = i;
}

// The first draw of every slot with its insertion into the first round's
// table fused in (infinite sites): the insertion's atomics overlap the
// draws' gathers.  The drivers go in afterwards (k_first_insert with no
// passenger slots); the table's final state and the marks do not depend on
// the order of the insertions.  tab (all ones) and lost (zeros) are set by
// the caller.
__global__ void k_place_first(PlaceTables t, PlaceOut o, Key key, const uint32_t* __restrict__ off_snv,
                              const uint32_t* __restrict__ off_id, uint32_t n_snv, uint32_t n_slots,
                              unsigned long long* __restrict__ tab, uint32_t mask, uint8_t* __restrict__ lost,
                              uint32_t* __restrict__ err) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_slots) return;
  place_slot(t, o, key, off_snv, off_id, n_snv, i, 0, err);
  const uint32_t k = o.locus[i];
  if (k == LOCUS_INVALID) lost[i] = 1;                   // no allele at the drawn position
  else first_insert(tab, mask, k, i + 1, lost, err);
}

// ------------------------------------------------------------ redraw rounds in one launch
// After the first round, every later round (candidates, winners, redraws of
// the losers) runs inside one cooperative launch, the phases separated by a
// grid barrier, so the host waits once for all rounds.  A round: pending
// slots whose locus is free enter a candidate table (hkeys: loci accepted in
// the later rounds; first: the first round's table), the smallest slot of
// each locus wins and joins hkeys, the others (and slots without an allele
// at their locus) are redrawn with their next attempt.
// A barrier wait gives up after TAIL_SPIN_LIMIT polls (status bit 2); every
// block then leaves at its next barrier, which also gives up.
constexpr uint32_t TAIL_SPIN_LIMIT = 1u << 22;
constexpr uint32_t TAIL_SOLO = 2048;   // pending slots below which one block runs the rounds

__device__ __forceinline__ bool grid_barrier(TailCtl* __restrict__ c, uint32_t& gen) {
  __shared__ uint32_t s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    s_ok = 1u;
    const uint32_t g = gen;
    __threadfence();
    if (atomicAdd(&c->bar_count, 1u) == gridDim.x - 1) {
      atomicExch(&c->bar_count, 0u);
      __threadfence();
      atomicExch(&c->bar_gen, g + 1u);
    } else {
      uint32_t polls = 0;
      while (*reinterpret_cast<volatile uint32_t*>(&c->bar_gen) == g) {
        if (++polls > TAIL_SPIN_LIMIT) { s_ok = 0u; atomicOr(&c->status, TAIL_BARRIER_TIMEOUT); break; }
        __nanosleep(128);
      }
    }
    __threadfence();
    gen = g + 1u;
  }
  __syncthreads();
  return s_ok != 0u;
}

__device__ __forceinline__ uint32_t ctl_load(const uint32_t* p) { return *reinterpret_cast<const volatile uint32_t*>(p); }

__global__ void __launch_bounds__(256) k_sites_tail(PlaceTables t, PlaceOut o, Key key,
                                                    const uint32_t* __restrict__ off_snv,
                                                    const uint32_t* __restrict__ off_id, uint32_t n_snv,
                                                    TailArgs a, TailCtl* __restrict__ ctl, uint32_t* __restrict__ err) {
  uint32_t gen = 0;
  uint32_t nthr = gridDim.x * blockDim.x, tid = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t cur = 0;
  bool ident = a.identity_first != 0;
  // once few slots are pending, block 0 runs the remaining rounds alone
  // (block barriers instead of grid barriers)
  bool solo = gridDim.x == 1;
  auto sync = [&]() -> bool {
    if (solo) { __syncthreads(); return true; }
    return grid_barrier(ctl, gen);
  };
  if (a.redraw_first) {   // list 0 holds the first round's losers: redraw them
    const uint32_t n = ctl_load(&ctl->count[0]);
    for (uint32_t i = tid; i < n; i += nthr) place_slot(t, o, key, off_snv, off_id, n_snv, a.list[0][i], 1, err);
    if (!grid_barrier(ctl, gen)) return;
  }
  for (uint32_t round = a.round0;; ++round) {
    const uint32_t n = ctl_load(cur ? &ctl->count[1] : &ctl->count[0]);
    if (n == 0) break;
    if (!solo && n <= TAIL_SOLO) {   // every block reads the same count after the barrier
      if (blockIdx.x != 0) return;
      solo = true;
      nthr = blockDim.x;
      tid = threadIdx.x;
    }
    if (round >= TAIL_MAX_ROUND) {
      if (tid == 0) atomicOr(&ctl->status, TAIL_ROUNDS_EXHAUSTED);
      break;
    }
    const uint32_t* pend = cur ? a.list[1] : a.list[0];
    uint32_t* next = cur ? a.list[0] : a.list[1];
    uint32_t* n_next = cur ? &ctl->count[0] : &ctl->count[1];
    if (a.unique) {
      for (uint32_t i = tid; i < n; i += nthr) {
        const uint32_t slot = ident ? i : pend[i];
        const uint32_t k = o.locus[slot];
        uint32_t h = EMPTY;
        if (!(k == LOCUS_INVALID || hset_contains(a.hkeys, a.hmask, k) ||
              (a.first && first_find(a.first, a.fmask, k) != FIRST_EMPTY))) {
          h = hset_insert(a.ckeys, a.cmask, k);
          if (h == EMPTY) atomicOr(err, ERR_CAPACITY);
          else atomicMin(a.cvals + h, slot);
        }
        a.hpos[i] = h;
      }
      if (!sync()) return;
      for (uint32_t i = tid; i < n; i += nthr) {
        const uint32_t slot = ident ? i : pend[i];
        const uint32_t h = a.hpos[i];
        if (h != EMPTY && a.cvals[h] == slot) {
          if (hset_insert(a.hkeys, a.hmask, o.locus[slot]) == EMPTY) atomicOr(err, ERR_CAPACITY);
        } else {
          next[atomicAdd(n_next, 1u)] = slot;
        }
      }
    } else {
      for (uint32_t i = tid; i < n; i += nthr) {
        const uint32_t slot = ident ? i : pend[i];
        if (o.locus[slot] == LOCUS_INVALID) next[atomicAdd(n_next, 1u)] = slot;
      }
    }
    if (!sync()) return;
    // redraw the losers; clear the candidate entries of this round
    const uint32_t nn = ctl_load(n_next);
    for (uint32_t i = tid; i < nn; i += nthr) place_slot(t, o, key, off_snv, off_id, n_snv, next[i], 1, err);
    if (a.unique)
      for (uint32_t i = tid; i < n; i += nthr) {
        const uint32_t h = a.hpos[i];
        if (h != EMPTY) { a.ckeys[h] = EMPTY; a.cvals[h] = EMPTY; }
      }
    if (tid == 0) { ctl->count[cur] = 0u; ctl->rounds = round + 1u; }
    if (!sync()) return;
    cur ^= 1u;
    ident = false;
  }
}

// ------------------------------------------------------------ drivers
// Driver SIDs are applied on the first edge of their mutant, in application
// order with the mutant's CNAs and WGDs; their instance and order on the edge
// come from the host, which replays those events.
__global__ void k_drivers(PlaceOut o, const DriverRec* __restrict__ drv, uint32_t n_drv, uint32_t base_slot) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_drv) return;
  const DriverRec d = drv[i];
  const uint32_t slot = base_slot + i;
  o.locus[slot] = d.locus;
  o.edge[slot] = d.edge;
  o.kind[slot] = d.kind;
  o.cls[slot] = 0xff;
  o.sig[slot] = 0xff;
  o.aux[slot] = d.aux;
  o.nature[slot] = NATURE_DRIVER;
  o.attempt[slot] = 0;
  o.allele[slot] = uint16_t(d.allele);
  o.seq[slot] = uint16_t(d.seq);
}

// ------------------------------------------------------------ locus sort
constexpr int BUCKET_SHIFT = 10;

__global__ void k_bucket_count(const uint32_t* __restrict__ locus, uint32_t n, uint32_t* __restrict__ bcnt) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) atomicAdd(bcnt + (locus[i] >> BUCKET_SHIFT), 1u);
}
// Bucket sort on 64-bit keys (locus << 32 | slot) written by the scatter:
// the in-bucket insertion sort reads its bucket's keys contiguously, and
// ties of a locus fall in slot order.
__global__ void k_bucket_scatter_keys(const uint32_t* __restrict__ locus, uint32_t n, const uint32_t* __restrict__ boff,
                                      uint32_t* __restrict__ bfill, unsigned long long* __restrict__ keys) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t k = locus[i], b = k >> BUCKET_SHIFT;
  keys[boff[b] + atomicAdd(bfill + b, 1u)] = (static_cast<unsigned long long>(k) << 32) | i;
}
// One block per 256 consecutive buckets: their keys (one contiguous range)
// are staged in shared memory, each thread insertion-sorts one bucket there,
// and the block writes the order coalesced.  A range larger than the stage
// is sorted in place in global memory instead.
constexpr uint32_t SORT_BUCKETS = 256, SORT_STAGE = 5120;   // 40 KB of keys

__global__ void __launch_bounds__(SORT_BUCKETS) k_bucket_sort_keys(const uint32_t* __restrict__ boff, uint32_t nb,
                                                                   uint32_t n, unsigned long long* __restrict__ keys,
                                                                   uint32_t* __restrict__ order) {
  __shared__ unsigned long long s_keys[SORT_STAGE];
  const uint32_t b0 = blockIdx.x * SORT_BUCKETS, b1 = min(b0 + SORT_BUCKETS, nb), b = b0 + threadIdx.x;
  const uint32_t k0 = boff[b0], k1 = b1 < nb ? boff[b1] : n;
  auto isort = [](unsigned long long* a, uint32_t lo, uint32_t hi) {
    for (uint32_t i = lo + 1; i < hi; ++i) {
      const unsigned long long kx = a[i];
      uint32_t j = i;
      while (j > lo) {
        const unsigned long long ky = a[j - 1];
        if (ky <= kx) break;
        a[j] = ky;
        --j;
      }
      a[j] = kx;
    }
  };
  if (k1 - k0 <= SORT_STAGE) {
    for (uint32_t i = k0 + threadIdx.x; i < k1; i += SORT_BUCKETS) s_keys[i - k0] = keys[i];
    __syncthreads();
    if (b < b1) isort(s_keys, boff[b] - k0, (b + 1 < nb ? boff[b + 1] : n) - k0);
    __syncthreads();
    for (uint32_t i = k0 + threadIdx.x; i < k1; i += SORT_BUCKETS) order[i] = uint32_t(s_keys[i - k0]);
  } else {
    if (b >= b1) return;
    const uint32_t lo = boff[b], hi = (b + 1 < nb) ? boff[b + 1] : n;
    isort(keys, lo, hi);
    for (uint32_t i = lo; i < hi; ++i) order[i] = uint32_t(keys[i]);
  }
}

// The gather of the sorted columns through 32-byte records: every slot's
// columns packed by a coalesced pass, so the gather reads one 32-byte sector
// per mutation instead of one per column.
// (inst: the batched form's instance of each slot, carried along; may be NULL)
__global__ void k_pack_records(PlaceOut o, const uint16_t* __restrict__ inst, uint32_t n, uint4* __restrict__ rec) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  rec[2 * uint64_t(i)] = make_uint4(o.locus[i], o.edge[i], o.aux[i], o.attempt[i]);
  rec[2 * uint64_t(i) + 1] = make_uint4(uint32_t(o.allele[i]) | (uint32_t(o.seq[i]) << 16),
                                        uint32_t(o.cls[i]) | (uint32_t(o.sig[i]) << 8) | (uint32_t(o.kind[i]) << 16) |
                                            (uint32_t(o.nature[i]) << 24),
                                        inst ? uint32_t(inst[i]) : 0u, 0u);
}

__global__ void k_gather_records(const uint4* __restrict__ rec, const uint32_t* __restrict__ order, uint32_t n,
                                 PlaceOut s, uint16_t* __restrict__ inst_sorted) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t x = order[i];
  const uint4 a = rec[2 * x], b = rec[2 * x + 1];
  s.locus[i] = a.x; s.edge[i] = a.y; s.aux[i] = a.z; s.attempt[i] = a.w;
  s.allele[i] = uint16_t(b.x); s.seq[i] = uint16_t(b.x >> 16);
  s.cls[i] = uint8_t(b.y); s.sig[i] = uint8_t(b.y >> 8); s.kind[i] = uint8_t(b.y >> 16); s.nature[i] = uint8_t(b.y >> 24);
  if (inst_sorted) inst_sorted[i] = uint16_t(b.z);
}

// ------------------------------------------------------------ batched placement
// A batch places the forests of many instances on one genome in single
// launches.  Cells (edge, epoch) of instance i occupy [cell_off[i],
// cell_off[i+1]) of the count arrays; the global slot space is every SNV of
// every instance (cells in order) followed by every indel, so the slots of
// one instance keep their relative order and every per-instance decision
// (Philox counters, lowest-slot wins, ties of the sort) is that of the plain
// path for the instance alone.
__device__ __forceinline__ uint32_t upper_index(const uint32_t* __restrict__ off, uint32_t n, uint32_t x) {
  // largest i < n with off[i] <= x
  uint32_t lo = 0, hi = n;
  while (hi - lo > 1) { const uint32_t mid = (lo + hi) >> 1; if (off[mid] <= x) lo = mid; else hi = mid; }
  return lo;
}

__global__ void k_edge_counts_b(const PlaceTables* __restrict__ tabs, uint32_t n_inst,
                                const uint32_t* __restrict__ node_off, const uint32_t* __restrict__ cell_off,
                                const Key* __restrict__ keys, const uint32_t* __restrict__ pre_snv,
                                const uint32_t* __restrict__ pre_id, uint32_t* __restrict__ cnt_snv,
                                uint32_t* __restrict__ cnt_id) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= node_off[n_inst]) return;
  const uint32_t i = upper_index(node_off, n_inst, g);
  const PlaceTables& t = tabs[i];
  edge_counts_one(t, g - node_off[i], keys[i], cnt_snv + cell_off[i], cnt_id + cell_off[i], pre_snv[i], pre_id[i]);
}

__device__ __forceinline__ void place_slot_b(const PlaceTables* __restrict__ tabs, uint32_t n_inst,
                                             const uint32_t* __restrict__ cell_off, const Key* __restrict__ keys,
                                             const PlaceOut& o, uint16_t* __restrict__ inst_of,
                                             const uint32_t* __restrict__ off_snv, const uint32_t* __restrict__ off_id,
                                             uint32_t n_snv, uint32_t slot, int redraw, uint32_t* __restrict__ err) {
  const bool is_id = slot >= n_snv;
  const uint32_t j = is_id ? slot - n_snv : slot;
  const uint32_t n_cells = cell_off[n_inst];
  const uint32_t* off = is_id ? off_id : off_snv;
  const uint32_t q = find_cell(off, n_cells, j);        // global cell
  const uint32_t i = upper_index(cell_off, n_inst, q);
  const PlaceTables& t = tabs[i];
  const uint32_t lq = q - cell_off[i];
  if (!redraw) inst_of[slot] = uint16_t(i);
  place_one(t, o, keys[i], slot, is_id, lq / t.n_epochs, lq % t.n_epochs, j - off[q], redraw, err);
}

__global__ void k_place_b(const PlaceTables* __restrict__ tabs, uint32_t n_inst, const uint32_t* __restrict__ cell_off,
                          const Key* __restrict__ keys, PlaceOut o, uint16_t* __restrict__ inst_of,
                          const uint32_t* __restrict__ off_snv, const uint32_t* __restrict__ off_id, uint32_t n_snv,
                          const uint32_t* __restrict__ pending, uint32_t n_pending,
                          const uint32_t* __restrict__ n_dev, int redraw, uint32_t* __restrict__ err) {
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= (n_dev ? *n_dev : n_pending)) return;
  place_slot_b(tabs, n_inst, cell_off, keys, o, inst_of, off_snv, off_id, n_snv, pending ? pending[tid] : tid, redraw,
               err);
}

// infinite-sites rounds of a batch: loci are unique per instance, so the
// hash keys are (instance << 32 | locus)
__device__ __forceinline__ uint64_t hash64(uint64_t k) {
  k ^= k >> 33; k *= 0xff51afd7ed558ccdull; k ^= k >> 33; k *= 0xc4ceb9fe1a85ec53ull; k ^= k >> 33;
  return k;
}
constexpr uint64_t EMPTY64 = ~0ull;
__device__ __forceinline__ bool hset64_contains(const uint64_t* __restrict__ keys, uint64_t mask, uint64_t k) {
  uint64_t h = hash64(k) & mask;
  for (uint64_t probe = 0; probe <= mask; ++probe) {
    const uint64_t x = keys[h];
    if (x == k) return true;
    if (x == EMPTY64) return false;
    h = (h + 1) & mask;
  }
  return false;
}
__device__ __forceinline__ uint64_t hset64_insert(unsigned long long* __restrict__ keys, uint64_t mask, uint64_t k) {
  uint64_t h = hash64(k) & mask;
  for (uint64_t probe = 0; probe <= mask; ++probe) {
    const unsigned long long prev = atomicCAS(keys + h, (unsigned long long)EMPTY64, (unsigned long long)k);
    if (prev == EMPTY64 || prev == k) return h;
    h = (h + 1) & mask;
  }
  return EMPTY64;
}

__global__ void k_cand_insert_b(const uint32_t* __restrict__ locus, const uint16_t* __restrict__ inst_of,
                                const uint32_t* __restrict__ pending, uint32_t n, const uint32_t* __restrict__ n_dev,
                                const uint64_t* __restrict__ hkeys, uint64_t hmask,
                                const uint64_t* __restrict__ fkeys, uint64_t fmask,
                                unsigned long long* __restrict__ ckeys, uint32_t* __restrict__ cvals, uint64_t cmask,
                                uint8_t* __restrict__ lost, uint32_t* __restrict__ err) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (n_dev ? *n_dev : n)) return;
  const uint32_t slot = pending ? pending[i] : i;
  const uint32_t l = locus[slot];
  const uint64_t k = (uint64_t(inst_of[slot]) << 32) | l;
  if (l == LOCUS_INVALID || (hkeys && hset64_contains(hkeys, hmask, k)) ||
      (fkeys && hset64_contains(fkeys, fmask, k))) {
    lost[i] = 1;
    return;
  }
  lost[i] = 0;
  const uint64_t h = hset64_insert(ckeys, cmask, k);
  if (h == EMPTY64) { atomicOr(err, ERR_CAPACITY); return; }
  atomicMin(cvals + h, slot);
}

__global__ void k_cand_resolve_b(const uint32_t* __restrict__ locus, const uint16_t* __restrict__ inst_of,
                                 const uint32_t* __restrict__ pending, uint32_t n, const uint32_t* __restrict__ n_dev,
                                 unsigned long long* __restrict__ hkeys, uint64_t hmask,
                                 const uint64_t* __restrict__ ckeys, const uint32_t* __restrict__ cvals,
                                 uint64_t cmask, const uint8_t* __restrict__ lost, uint32_t* __restrict__ next,
                                 uint32_t* __restrict__ n_next, uint32_t* __restrict__ err) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (n_dev ? *n_dev : n)) return;
  const uint32_t slot = pending ? pending[i] : i;
  const uint64_t k = (uint64_t(inst_of[slot]) << 32) | locus[slot];
  bool win = false;
  if (!lost[i]) {
    uint64_t h = hash64(k) & cmask;
    for (uint64_t probe = 0; probe <= cmask; ++probe) {
      const uint64_t x = ckeys[h];
      if (x == k) { win = cvals[h] == slot; break; }
      if (x == EMPTY64) break;
      h = (h + 1) & cmask;
    }
  }
  if (win) {
    if (hkeys && hset64_insert(hkeys, hmask, k) == EMPTY64) atomicOr(err, ERR_CAPACITY);
  } else {
    next[atomicAdd(n_next, 1u)] = slot;
  }
}

// The later rounds of a batch in one cooperative launch: k_sites_tail's
// rounds with (instance << 32 | locus) keys.
__global__ void __launch_bounds__(256) k_sites_tail_b(const PlaceTables* __restrict__ tabs, uint32_t n_inst,
                                                      const uint32_t* __restrict__ cell_off,
                                                      const Key* __restrict__ keys, PlaceOut o,
                                                      uint16_t* __restrict__ inst_of,
                                                      const uint32_t* __restrict__ off_snv,
                                                      const uint32_t* __restrict__ off_id, uint32_t n_snv,
                                                      TailArgsB a, TailCtl* __restrict__ ctl,
                                                      uint32_t* __restrict__ err) {
  uint32_t gen = 0;
  uint32_t nthr = gridDim.x * blockDim.x, tid = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t cur = 0;
  bool solo = gridDim.x == 1;   // as k_sites_tail: block 0 alone once few slots are pending
  auto sync = [&]() -> bool {
    if (solo) { __syncthreads(); return true; }
    return grid_barrier(ctl, gen);
  };
  {   // list 0 holds the first round's losers: redraw them
    const uint32_t n = ctl_load(&ctl->count[0]);
    for (uint32_t i = tid; i < n; i += nthr)
      place_slot_b(tabs, n_inst, cell_off, keys, o, inst_of, off_snv, off_id, n_snv, a.list[0][i], 1, err);
    if (!grid_barrier(ctl, gen)) return;
  }
  for (uint32_t round = 1;; ++round) {
    const uint32_t n = ctl_load(cur ? &ctl->count[1] : &ctl->count[0]);
    if (n == 0) break;
    if (!solo && n <= TAIL_SOLO) {
      if (blockIdx.x != 0) return;
      solo = true;
      nthr = blockDim.x;
      tid = threadIdx.x;
    }
    if (round >= TAIL_MAX_ROUND) {
      if (tid == 0) atomicOr(&ctl->status, TAIL_ROUNDS_EXHAUSTED);
      break;
    }
    const uint32_t* pend = cur ? a.list[1] : a.list[0];
    uint32_t* next = cur ? a.list[0] : a.list[1];
    uint32_t* n_next = cur ? &ctl->count[0] : &ctl->count[1];
    for (uint32_t i = tid; i < n; i += nthr) {
      const uint32_t slot = pend[i];
      const uint32_t l = o.locus[slot];
      const uint64_t k = (uint64_t(inst_of[slot]) << 32) | l;
      uint64_t h = EMPTY64;
      if (!(l == LOCUS_INVALID || hset64_contains(reinterpret_cast<const uint64_t*>(a.hkeys), a.hmask, k) ||
            hset64_contains(a.fkeys, a.fmask, k))) {
        h = hset64_insert(a.ckeys, a.cmask, k);
        if (h == EMPTY64) atomicOr(err, ERR_CAPACITY);
        else atomicMin(a.cvals + h, slot);
      }
      a.hpos[i] = h;
    }
    if (!sync()) return;
    for (uint32_t i = tid; i < n; i += nthr) {
      const uint32_t slot = pend[i];
      const uint64_t h = a.hpos[i];
      if (h != EMPTY64 && a.cvals[h] == slot) {
        if (hset64_insert(a.hkeys, a.hmask, (uint64_t(inst_of[slot]) << 32) | o.locus[slot]) == EMPTY64)
          atomicOr(err, ERR_CAPACITY);
      } else {
        next[atomicAdd(n_next, 1u)] = slot;
      }
    }
    if (!sync()) return;
    const uint32_t nn = ctl_load(n_next);
    for (uint32_t i = tid; i < nn; i += nthr)
      place_slot_b(tabs, n_inst, cell_off, keys, o, inst_of, off_snv, off_id, n_snv, next[i], 1, err);
    for (uint32_t i = tid; i < n; i += nthr) {
      const uint64_t h = a.hpos[i];
      if (h != EMPTY64) { a.ckeys[h] = EMPTY64; a.cvals[h] = EMPTY; }
    }
    if (tid == 0) { ctl->count[cur] = 0u; ctl->rounds = round + 1u; }
    if (!sync()) return;
    cur ^= 1u;
  }
}

// sort of a batch by (instance, locus): bucket = instance * nb + locus >> 10
__global__ void k_bucket_count_b(const uint32_t* __restrict__ locus, const uint16_t* __restrict__ inst_of, uint32_t n,
                                 uint32_t nb, uint32_t* __restrict__ bcnt) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) atomicAdd(bcnt + uint64_t(inst_of[i]) * nb + (locus[i] >> BUCKET_SHIFT), 1u);
}
__global__ void k_bucket_scatter_b(const uint32_t* __restrict__ locus, const uint16_t* __restrict__ inst_of,
                                   uint32_t n, uint32_t nb, const uint32_t* __restrict__ boff,
                                   uint32_t* __restrict__ bfill, unsigned long long* __restrict__ keys) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t k = locus[i];
  const uint64_t b = uint64_t(inst_of[i]) * nb + (k >> BUCKET_SHIFT);
  keys[boff[b] + atomicAdd(bfill + b, 1u)] = (static_cast<unsigned long long>(k) << 32) | i;
}

// ------------------------------------------------------------ host launchers
static inline unsigned nblk(uint64_t n, int b = 256) { return unsigned((n + b - 1) / b); }

void place_cna_counts(const PlaceTables& t, uint32_t* cnt_cna, uint64_t seed, double germline_size, cudaStream_t st) {
  if (t.n_nodes) { k_cna_counts<<<nblk(t.n_nodes, 128), 128, 0, st>>>(t, cnt_cna, make_key(seed), germline_size); note_launch(); }
}

void place_edge_counts(const PlaceTables& t, uint32_t* cnt_snv, uint32_t* cnt_id, uint64_t seed,
                       uint32_t n_pre_snv, uint32_t n_pre_id, cudaStream_t st) {
  k_edge_counts<<<nblk(t.n_nodes + 1, 128), 128, 0, st>>>(t, cnt_snv, cnt_id, make_key(seed), n_pre_snv, n_pre_id); note_launch();
}

void place_mutations_launch(const PlaceTables& t, const PlaceOut& o, uint64_t seed, const uint32_t* off_snv,
                            const uint32_t* off_id, uint32_t n_snv, uint32_t n_id, const uint32_t* pending,
                            uint32_t n_pending, int redraw, uint32_t* err, cudaStream_t st, const uint32_t* n_dev) {
  if (n_pending == 0) return;
  k_place<<<nblk(n_pending), 256, 0, st>>>(t, o, make_key(seed), off_snv, off_id, n_snv, n_id, pending, n_pending,
                                           n_dev, redraw, err); note_launch();
}

void place_drivers(const PlaceOut& o, const DriverRec* drv, uint32_t n_drv, uint32_t base_slot, cudaStream_t st) {
  if (n_drv == 0) return;
  k_drivers<<<nblk(n_drv), 256, 0, st>>>(o, drv, n_drv, base_slot); note_launch();
}

void place_first_round(const PlaceTables& t, const PlaceOut& o, uint64_t seed, const uint32_t* off_snv,
                       const uint32_t* off_id, uint32_t n_snv, uint32_t n_slots, unsigned long long* first,
                       uint32_t fmask, uint8_t* lost, uint32_t* err, cudaStream_t st) {
  if (n_slots == 0) return;
  cudaMemsetAsync(lost, 0, n_slots, st);
  k_place_first<<<nblk(n_slots), 256, 0, st>>>(t, o, make_key(seed), off_snv, off_id, n_snv, n_slots, first, fmask,
                                               lost, err);
  note_launch();
}

void sites_first_finish(const uint32_t* drv_locus, uint32_t n_drv, unsigned long long* first, uint32_t fmask,
                        uint8_t* lost, uint32_t n_slots, uint32_t* next, uint32_t* n_next, uint32_t* err,
                        cudaStream_t st) {
  if (n_drv) {
    k_first_insert<<<nblk(n_drv), 256, 0, st>>>(nullptr, 0, drv_locus, n_drv, first, fmask, lost, err);
    note_launch();
  }
  if (n_slots) { k_first_collect<<<nblk(n_slots), 256, 0, st>>>(lost, n_slots, next, n_next); note_launch(); }
}

const char* sites_tail(const PlaceTables& t, const PlaceOut& o, uint64_t seed, const uint32_t* off_snv,
                       const uint32_t* off_id, uint32_t n_snv, const TailArgs& a, uint32_t n0, TailCtl* ctl,
                       uint32_t* err, cudaStream_t st) {
  if (n0 == 0) return nullptr;
  int dev = 0, n_sm = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sites_tail, 256, 0) != cudaSuccess || per_sm < 1)
    return "cannot size the cooperative launch of the redraw rounds";
  const uint64_t want = std::max<uint64_t>(1, (uint64_t(n0) + 255) / 256);
  const unsigned grid = unsigned(std::min<uint64_t>(want, uint64_t(n_sm) * uint64_t(per_sm)));
  Key key = make_key(seed);
  PlaceTables tt = t;
  PlaceOut oo = o;
  TailArgs aa = a;
  void* args[] = {&tt, &oo, &key, const_cast<uint32_t**>(&off_snv), const_cast<uint32_t**>(&off_id), &n_snv, &aa,
                  &ctl, &err};
  if (cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(k_sites_tail), dim3(grid), dim3(256), args, 0, st) !=
      cudaSuccess)
    return "cooperative launch of the redraw rounds failed";
  note_launch();
  return nullptr;
}

const char* sites_tail_batch(const PlaceTables* tabs, uint32_t n_inst, const uint32_t* cell_off, const Key* keys,
                             const PlaceOut& o, uint16_t* inst_of, const uint32_t* off_snv, const uint32_t* off_id,
                             uint32_t n_snv, const TailArgsB& a, uint32_t n0, TailCtl* ctl, uint32_t* err,
                             cudaStream_t st) {
  if (n0 == 0) return nullptr;
  int dev = 0, n_sm = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sites_tail_b, 256, 0) != cudaSuccess || per_sm < 1)
    return "cannot size the cooperative launch of the redraw rounds";
  const uint64_t want = std::max<uint64_t>(1, (uint64_t(n0) + 255) / 256);
  const unsigned grid = unsigned(std::min<uint64_t>(want, uint64_t(n_sm) * uint64_t(per_sm)));
  PlaceOut oo = o;
  TailArgsB aa = a;
  void* args[] = {&tabs, &n_inst, &cell_off, &keys, &oo, &inst_of, &off_snv, &off_id, &n_snv, &aa, &ctl, &err};
  if (cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(k_sites_tail_b), dim3(grid), dim3(256), args, 0, st) !=
      cudaSuccess)
    return "cooperative launch of the redraw rounds failed";
  note_launch();
  return nullptr;
}

void sort_by_locus(const PlaceOut& o, uint32_t n, uint64_t G, uint32_t* bcnt, uint32_t* bfill, uint32_t* part,
                   uint32_t* order, const PlaceOut& sorted, unsigned long long* keys, uint4* recs,
                   cudaStream_t st) {
  const uint32_t nb = uint32_t((G >> BUCKET_SHIFT) + 1);
  cudaMemsetAsync(bcnt, 0, sizeof(uint32_t) * nb, st);
  cudaMemsetAsync(bfill, 0, sizeof(uint32_t) * nb, st);
  if (n == 0) return;
  k_bucket_count<<<nblk(n), 256, 0, st>>>(o.locus, n, bcnt); note_launch();
  scan_rows<uint32_t>(bcnt, bcnt, nb, 1, part, nullptr, st);
  k_bucket_scatter_keys<<<nblk(n), 256, 0, st>>>(o.locus, n, bcnt, bfill, keys); note_launch();
  k_bucket_sort_keys<<<nblk(nb, SORT_BUCKETS), SORT_BUCKETS, 0, st>>>(bcnt, nb, n, keys, order); note_launch();
  k_pack_records<<<nblk(n), 256, 0, st>>>(o, nullptr, n, recs); note_launch();
  k_gather_records<<<nblk(n), 256, 0, st>>>(recs, order, n, sorted, nullptr); note_launch();
}

uint32_t sort_num_buckets(uint64_t G) { return uint32_t((G >> BUCKET_SHIFT) + 1); }

void place_edge_counts_batch(const PlaceTables* tabs, uint32_t n_inst, const uint32_t* node_off, uint32_t n_nodes_all,
                             const uint32_t* cell_off, const Key* keys, const uint32_t* pre_snv, const uint32_t* pre_id,
                             uint32_t* cnt_snv, uint32_t* cnt_id, cudaStream_t st) {
  if (n_nodes_all) { k_edge_counts_b<<<nblk(n_nodes_all, 128), 128, 0, st>>>(tabs, n_inst, node_off, cell_off, keys,
                                                                          pre_snv, pre_id, cnt_snv, cnt_id); note_launch(); }
}

void place_mutations_batch(const PlaceTables* tabs, uint32_t n_inst, const uint32_t* cell_off, const Key* keys,
                           const PlaceOut& o, uint16_t* inst_of, const uint32_t* off_snv, const uint32_t* off_id,
                           uint32_t n_snv, const uint32_t* pending, uint32_t n_pending, int redraw, uint32_t* err,
                           cudaStream_t st, const uint32_t* n_dev) {
  if (n_pending == 0) return;
  k_place_b<<<nblk(n_pending), 256, 0, st>>>(tabs, n_inst, cell_off, keys, o, inst_of, off_snv, off_id, n_snv, pending,
                                             n_pending, n_dev, redraw, err); note_launch();
}

void sites_round_batch(const uint32_t* locus, const uint16_t* inst_of, const uint32_t* pending, uint32_t n,
                       uint64_t* hkeys, uint64_t hmask, uint64_t* ckeys, uint32_t* cvals, uint64_t cmask,
                       uint8_t* lost, uint32_t* next, uint32_t* n_next, uint32_t* err, cudaStream_t st,
                       const uint32_t* n_dev, const uint64_t* fkeys, uint64_t fmask) {
  if (n == 0) return;
  k_cand_insert_b<<<nblk(n), 256, 0, st>>>(locus, inst_of, pending, n, n_dev, hkeys, hmask, fkeys, fmask,
                                           reinterpret_cast<unsigned long long*>(ckeys), cvals, cmask, lost, err);
  k_cand_resolve_b<<<nblk(n), 256, 0, st>>>(locus, inst_of, pending, n, n_dev,
                                            reinterpret_cast<unsigned long long*>(hkeys), hmask, ckeys, cvals, cmask,
                                            lost, next, n_next, err);
  note_launch(2);
}

void sort_batch(const PlaceOut& o, const uint16_t* inst_of, uint32_t n, uint32_t n_inst, uint64_t G, uint32_t* bcnt,
                uint32_t* bfill, uint32_t* part, uint32_t* order, const PlaceOut& sorted, uint16_t* inst_sorted,
                unsigned long long* keys, uint4* recs, cudaStream_t st) {
  const uint32_t nb = uint32_t((G >> BUCKET_SHIFT) + 1);
  const uint64_t nbt = uint64_t(nb) * n_inst;
  cudaMemsetAsync(bcnt, 0, sizeof(uint32_t) * (nbt + 1), st);
  cudaMemsetAsync(bfill, 0, sizeof(uint32_t) * nbt, st);
  if (n == 0) return;
  k_bucket_count_b<<<nblk(n), 256, 0, st>>>(o.locus, inst_of, n, nb, bcnt); note_launch();
  scan_rows<uint32_t>(bcnt, bcnt, nbt, 1, part, bcnt + nbt, st);
  k_bucket_scatter_b<<<nblk(n), 256, 0, st>>>(o.locus, inst_of, n, nb, bcnt, bfill, keys); note_launch();
  k_bucket_sort_keys<<<nblk(nbt, SORT_BUCKETS), SORT_BUCKETS, 0, st>>>(bcnt, uint32_t(nbt), n, keys, order);
  note_launch();
  k_pack_records<<<nblk(n), 256, 0, st>>>(o, inst_of, n, recs); note_launch();
  k_gather_records<<<nblk(n), 256, 0, st>>>(recs, order, n, sorted, inst_sorted); note_launch();
}

}  // namespace pg
