// Host-callable launchers of the device kernels and the plain-pointer
// structures they take.  Everything here is internal to the library; the
// public boundary is include/process_gb300.h.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace pg {

// Philox key of a call (the seed's two words)
struct Key { uint32_t k0, k1; };
__host__ __device__ inline Key make_key(uint64_t seed) {
  return {uint32_t(seed), uint32_t(seed >> 32)};
}

constexpr uint32_t MAX_EPOCHS = 16;

// Counts kernel launches of this library (read with pg_launch_count).
void note_launch(uint32_t n = 1);

// ---------------------------------------------------------------- index
void genome_synth(uint32_t* words, uint64_t G, uint64_t seed, double gc, cudaStream_t st);
void genome_pack(uint32_t* words, const uint8_t* codes, uint64_t G, cudaStream_t st);
// unknown bases (codes > 3, e.g. N) as one bit per position ((G + 31) / 32
// words); *any (zeroed by the caller) becomes 1 when there is one.  A NULL
// mask below means a genome without unknown bases.
void genome_nmask(const uint8_t* codes, uint64_t G, uint32_t* mask, uint32_t* any, cudaStream_t st);
uint32_t index_num_tiles(uint64_t G);
// bases at pos (BASE_INVALID for positions outside the genome or unknown)
void genome_gather(const uint32_t* g, const uint32_t* nmask, uint64_t G, const uint32_t* pos, uint64_t n,
                   uint8_t* out, cudaStream_t st);
// per placed mutation rows[i] (all rows when NULL): {locus, ref code, alt
// code, kind | signature << 8 | nature << 16}; the codes hold up to 8
// characters of "ACGNT" coded 1..5, 4 bits each, the first character highest
void row_info(const uint32_t* locus, const uint32_t* aux, const uint8_t* kind, const uint8_t* sig,
              const uint8_t* nature, const uint32_t* rows, uint64_t n, const uint32_t* g, const uint32_t* nmask,
              uint64_t G, uint4* out, cudaStream_t st);
int index_num_classes(int which);  // 0 = SBS contexts (32), 1 = ID classes (83)
// allocation-free per-class totals over a caller-held genome (see pg_index.cu);
// returns nullptr on success, else a message
constexpr uint32_t NOALLOC_MAX_TILES = 8192;
const char* index_counts_noalloc(int which, const uint32_t* g, uint64_t G, const uint32_t* chr_off, int n_chr,
                                 uint64_t* totals, cudaStream_t st);
// contexts and repeat sites that touch an unknown base are not indexed; the
// SBS contexts (which 0) also skip the positions set in amask (regions to
// avoid; NULL: none)
void index_count(int which, const uint32_t* g, const uint32_t* nmask, const uint32_t* amask, uint64_t G,
                 const uint32_t* chr_off, int n_chr, uint32_t* cnt, uint32_t* part, uint32_t* totals, cudaStream_t st);
void genome_avoid_mask(const uint32_t* pos, uint64_t n, uint32_t* mask, cudaStream_t st);
// every: all strides are 1 (each indexed position is written)
void index_emit(int which, const uint32_t* g, const uint32_t* nmask, const uint32_t* amask, uint64_t G,
                const uint32_t* chr_off, int n_chr, const uint32_t* cnt_scanned, const uint32_t* stride,
                const uint64_t* list_off, const uint32_t* list_len, uint32_t* lists, bool every, cudaStream_t st);

// ---------------------------------------------------------------- genome classes
// Copy-number events are rare, so the cells of a forest fall into few
// genotype classes: the genome below each CNA/WGD event edge.  A class is a
// list of segments (absolute [start, end), ascending) with the sorted ids of
// the allele instances covering each segment.  Class 0 is the germline:
// instances 0 and 1 over every chromosome.
struct GenomeClasses {
  uint32_t n_classes;
  const uint32_t* node_class;   // class of each edge's genome after its own events (n_nodes + 1 entries)
  const uint32_t* seg_off;      // n_classes + 1
  const uint32_t* seg_start;
  const uint32_t* seg_end;
  const uint32_t* seg_ioff;     // covering instances: inst_list[seg_ioff, seg_ioff + seg_icnt)
  const uint32_t* seg_icnt;
  const uint16_t* inst_list;
};

// ---------------------------------------------------------------- placement
struct PlaceTables {
  // forest (device)
  uint32_t n_nodes;
  const int32_t* parent;
  const double* birth;
  const uint32_t* species;
  const uint32_t* divisions;
  // epochs and rates (device); rates are [species][epoch]
  uint32_t n_epochs;
  const double* epoch_start;
  const double* snv_rate;
  const double* indel_rate;
  const double* cna_rate;       // per species (passenger CNAs per base per division)
  const double* node_size;      // allelic size of each edge's genome (n_nodes + 1 entries)
  GenomeClasses gc;
  // signatures: exposure CDFs [(n_epochs+1) rows][n_sigs], class CDFs [n_sigs][classes]
  uint32_t n_sbs_sigs, n_id_sigs;
  const uint32_t* sbs_expo_cdf;
  const uint32_t* sbs_sig_cdf;
  const uint32_t* id_expo_cdf;
  const uint32_t* id_sig_cdf;
  // indices
  const uint32_t* genome;
  const uint64_t* ctx_off; const uint32_t* ctx_len; const uint32_t* ctx_lists;
  const uint64_t* id_off; const uint32_t* id_len; const uint32_t* id_lists;
};

// SoA of placed mutations (device)
struct PlaceOut {
  uint32_t* locus;    // absolute position (SNV) or anchor position (indel)
  uint32_t* edge;     // node index; n_nodes = preneoplastic edge
  uint32_t* aux;      // SNV: alt base; indel: descriptor
  uint8_t* cls;       // SBS96 / ID83 class, 0xff for drivers
  uint8_t* sig;       // signature index (cause), 0xff for drivers
  uint16_t* allele;   // allele instance
  uint16_t* seq;      // order on the edge: driver event index, 0x7fff passengers, 0 preneoplastic
  uint8_t* kind;
  uint8_t* nature;
  uint32_t* attempt;
};

struct DriverRec {
  uint32_t locus, edge, aux, allele, seq;   // allele: the instance, chosen on the host
  uint8_t kind, pad[3];
};

void place_cna_counts(const PlaceTables& t, uint32_t* cnt_cna, uint64_t seed, double germline_size, cudaStream_t st);
void place_edge_counts(const PlaceTables& t, uint32_t* cnt_snv, uint32_t* cnt_id, uint64_t seed,
                       uint32_t n_pre_snv, uint32_t n_pre_id, cudaStream_t st);
// n_dev (optional): the number of pending slots in device memory (<= n_pending,
// which sizes the grid); the redraw rounds run without reading it on the host
void place_mutations_launch(const PlaceTables& t, const PlaceOut& o, uint64_t seed, const uint32_t* off_snv,
                            const uint32_t* off_id, uint32_t n_snv, uint32_t n_id, const uint32_t* pending,
                            uint32_t n_pending, int redraw, uint32_t* err, cudaStream_t st,
                            const uint32_t* n_dev = nullptr);
void place_drivers(const PlaceOut& o, const DriverRec* drv, uint32_t n_drv, uint32_t base_slot, cudaStream_t st);
// the first draw of slots [0, n_slots) fused with their insertion into the
// first round's table `first` (fmask + 1 entries, all ones on entry; lost:
// n_slots bytes of scratch); then sites_first_finish inserts the drivers'
// loci and lists the losing slots in next
void place_first_round(const PlaceTables& t, const PlaceOut& o, uint64_t seed, const uint32_t* off_snv,
                       const uint32_t* off_id, uint32_t n_snv, uint32_t n_slots, unsigned long long* first,
                       uint32_t fmask, uint8_t* lost, uint32_t* err, cudaStream_t st);
void sites_first_finish(const uint32_t* drv_locus, uint32_t n_drv, unsigned long long* first, uint32_t fmask,
                        uint8_t* lost, uint32_t n_slots, uint32_t* next, uint32_t* n_next, uint32_t* err,
                        cudaStream_t st);
// All redraw rounds after the first in one cooperative launch (k_sites_tail).
// list[0] holds the n0 pending slots (identity_first: slots 0 .. n0 - 1, no
// list); redraw_first: they are redrawn before the first round.  unique:
// infinite sites (hkeys accepted set, ckeys/cvals candidate table, all
// EMPTY on entry, capacities powers of two >= 2 n0; hpos n0 entries; first:
// the first round's table or NULL); else only loci without an allele are
// redrawn.  ctl (zeroed, count[0] = n0) reports the rounds and the status.
constexpr uint32_t TAIL_MAX_ROUND = 256;
enum : uint32_t { TAIL_ROUNDS_EXHAUSTED = 1u, TAIL_BARRIER_TIMEOUT = 2u };
struct TailCtl {
  uint32_t count[2];     // pending slots of the two lists
  uint32_t bar_count, bar_gen;
  uint32_t status;
  uint32_t rounds;       // the round counter after the last round run
};
struct TailArgs {
  uint32_t* list[2];
  int identity_first, redraw_first, unique;
  uint32_t round0;
  uint32_t* hkeys; uint32_t hmask;
  uint32_t* ckeys; uint32_t* cvals; uint32_t cmask;
  uint32_t* hpos;
  const unsigned long long* first; uint32_t fmask;
};
// the batched form: keys (instance << 32 | locus); list 0 holds the first
// round's losers, redrawn first; fkeys: the first round's table
struct TailArgsB {
  uint32_t* list[2];
  unsigned long long* hkeys; uint64_t hmask;
  unsigned long long* ckeys; uint32_t* cvals; uint64_t cmask;
  uint64_t* hpos;
  const uint64_t* fkeys; uint64_t fmask;
};
// returns nullptr, or a message when the launch could not be made
const char* sites_tail(const PlaceTables& t, const PlaceOut& o, uint64_t seed, const uint32_t* off_snv,
                       const uint32_t* off_id, uint32_t n_snv, const TailArgs& a, uint32_t n0, TailCtl* ctl,
                       uint32_t* err, cudaStream_t st);
uint32_t sort_num_buckets(uint64_t G);
// sort by (locus, slot) into `sorted`; keys: n 64-bit keys, recs: 2n
// 16-byte words (the 32-byte records of the gather)
void sort_by_locus(const PlaceOut& o, uint32_t n, uint64_t G, uint32_t* bcnt, uint32_t* bfill, uint32_t* part,
                   uint32_t* order, const PlaceOut& sorted, unsigned long long* keys, uint4* recs,
                   cudaStream_t st);

// ---------------------------------------------------------------- sequencing
struct SeqRec {            // 16 B, one per placed mutation, sorted by locus
  uint32_t locus;
  uint32_t tin, tout;      // Euler interval of the edge that carries it
  uint32_t info;           // instance | (order on the edge & 0x7fff) << 16 | kind << 31
};

// fragments the read kernel handles per shared-memory batch (5 per thread);
// tiles are sized so that their fragment count rarely exceeds one batch
constexpr uint32_t SEQ_FRAGS_PER_BATCH = 1280;

struct SeqTiles {
  uint32_t n_tiles;        // over all selected chromosomes
  const uint32_t* start;   // first start position of the tile (absolute)
  const uint32_t* len;     // number of start positions in the tile
  const uint32_t* chr_end; // absolute end of the tile's chromosome
  const uint32_t* rec_lo;  // records of the tile's window [start, start + len - 1 + span)
  const uint32_t* rec_hi;
};

struct SeqSample {
  uint32_t n_leaves;
  uint32_t leaf_off;       // into leaf_tin
  uint32_t normal_thr;     // read from a normal cell iff u < normal_thr
  uint32_t all_normal;     // the normal sample: every read from a normal cell
  // with copy-number events: the sample's cell options (option 0 its normal
  // cells, then the genotype classes of its leaves, ascending) and, per atom,
  // the thresholds of the option draw (rows of n_opt at opt_cdf_off)
  uint32_t opt_off, n_opt, opt_cdf_off;
};

// The thresholds that split a substitution error's word range [0, thr) into
// the three other bases: [0, t1), [t1, t2), [t2, thr).
inline void err_thirds(uint32_t thr, uint32_t& t1, uint32_t& t2) {
  t1 = thr / 3u;
  t2 = uint32_t(uint64_t(thr) * 2u / 3u);
}

struct SeqParams {
  uint32_t read_len;
  uint32_t paired;
  uint32_t span;           // max fragment span past the start (read_len or max insert)
  uint32_t ins_min, n_ins; // insert size = ins_min + index in the CDF table
  const uint32_t* ins_cdf;
  const uint16_t* ins_guide; // 256 entries: first index whose threshold exceeds g * 2^23
  uint32_t err_thr;        // substitution error iff u < err_thr
  uint32_t err_t1, err_t2; // the erroneous base: the first of the three others iff u < err_t1,
                           //   the second iff err_t1 <= u < err_t2, else the third
  uint32_t normal_tin;     // Euler index of normal cells
  uint32_t n_alleles;
  // copy-number state (has_cna == 0: every cell has instances 0 and 1 everywhere)
  uint32_t has_cna;
  GenomeClasses gc;
  const uint32_t* chain_off;  // instance lineage: for instance y, ancestors chain_anc[chain_off[y]..]
  const uint16_t* chain_anc;  //   with the order key (tin << 16 | seq + 1) of the copy that led towards y
  const uint64_t* chain_key;
  // Atoms: the coarsest partition of the genome into intervals on which every
  // class's covering instances are constant.  A tile's start range is cut
  // into parts, one per atom it meets.
  uint32_t n_classes;         // row length of atom_ioff / atom_icnt
  const uint32_t* atom_ioff;  // [atom * n_classes + class]: first covering instance in gc.inst_list
  const uint32_t* atom_icnt;  //   and their number (0: the class has no allele there)
  const uint32_t* part_off;   // parts of tile t: [part_off[t], part_off[t + 1])
  const uint32_t* part_start; // absolute first start position of the part
  const uint32_t* part_len;
  const uint32_t* part_atom;
  const uint32_t* part_cdf;   // [sample * n_parts + part]: thresholds of the part draw within its tile
  uint32_t n_parts;
  const uint32_t* opt_class;  // per cell option: genotype class
  const uint32_t* opt_leaf_off;   // its leaves in cls_leaf_tin
  const uint32_t* opt_nleaf;      // 0: the normal cells
  const uint32_t* cls_leaf_tin;   // every sample's leaves grouped by class (Euler indices)
  const uint32_t* opt_cdf;        // option thresholds (see SeqSample)
  const uint32_t* nmask;          // unknown reference bases (N), one bit each, or NULL (SAM output)
};

// tile t of chromosome slot c (c_first[c] <= t < c_first[c] + c_ntiles[c],
// k = t - c_first[c]) covers the starts [c_start + k T, + min(T, S - k T))
void seq_make_tiles(uint32_t n_slots, const uint32_t* c_first, const uint32_t* c_ntiles, const uint32_t* c_start,
                    const uint32_t* c_nstarts, const uint32_t* c_end, uint32_t T, uint32_t n_tiles, uint32_t* start,
                    uint32_t* len, uint32_t* end, cudaStream_t st);
// Copy-number tables of a sequencing call.  Parts: tile t's start range cut
// at atom boundaries, at part_off[t] .. part_off[t + 1] (part_off holds
// n_tiles + 1 entries; `part` is scan scratch of scan_part_elems(n_tiles, 1)).
void seq_tile_parts(uint32_t n_tiles, const uint32_t* tile_start, const uint32_t* tile_len,
                    const uint32_t* atom_start, uint32_t n_atoms, uint32_t genome_len, uint32_t* part_off,
                    uint32_t* scan_part, uint32_t* part_start, uint32_t* part_len, uint32_t* part_atom,
                    cudaStream_t st);
// Per (sample, tile) its integer copy sums (I0, S) (scratch tile_sums,
// 2 * n_samples * n_tiles) and, for tiles of several parts, the thresholds
// of the part draw (part_cdf[s * n_parts + part]); then per (sample,
// chromosome slot) the mass before each tile (mass_cum[s * n_tiles + t]) and
// the slot's total (mass_tot[s * n_slots + slot]), each the mass of the
// exact integer sums before it.  A stretch with integer copy sums (I0, S)
// weighs wn * I0 + (wt / nl) * S (the second term when nl > 0);
// icnt0 / copy_sum are per (sample, atom).
void seq_tile_mass(uint32_t n_samples, uint32_t n_slots, const uint32_t* c_first, const uint32_t* c_ntiles,
                   const uint32_t* part_off, const uint32_t* part_len, const uint32_t* part_atom, uint32_t n_atoms,
                   const double* wn, const double* wt, const uint64_t* nl, const uint64_t* icnt0,
                   const uint64_t* copy_sum, uint32_t n_tiles, uint32_t n_parts, uint64_t* tile_sums,
                   double* mass_cum, double* mass_tot, uint32_t* part_cdf, cudaStream_t st);
// ---------------------------------------------------------------- SAM records
// One aligned read as the SAM writer needs it; the host formats the text.
constexpr uint32_t SAM_MAX_CIGAR = 16;
struct SamRead {
  uint32_t pos;             // absolute first aligned reference position
  uint32_t mate_pos;        // absolute first position of the mate (paired reads)
  int32_t tlen;             // signed template length (0 for single-end reads)
  uint16_t flag;            // SAM FLAG
  uint16_t n_cigar;
  uint32_t seq_len;
  uint32_t cigar[SAM_MAX_CIGAR];   // op length << 4 | op (0 M, 1 I, 2 D)
};
// Reads of tiles [t0, t0 + n_chunk) (global tile indices, for the draws) of
// every sample: the fragment draws of the read kernel, each mate's bases
// built from the genome with the mutations its allele instance carries and
// the substitution errors of its error words.  Read r of the fragment j of
// (sample s, tile t0 + k) is written at 2 * (out_off[s * n_chunk + k] + j) +
// mate (one slot per fragment for single-end reads); seq holds max_len
// bytes per read.
void seq_sam_reads(const SeqRec* recs, uint32_t n_recs, const uint32_t* aux, const uint32_t* genome,
                   const SeqTiles& tiles, uint32_t t0, uint32_t n_chunk, const uint32_t* pair_cnt,
                   const SeqSample* samples, uint32_t n_samples, const uint32_t* leaf_tin, const SeqParams& prm,
                   uint64_t seed, const uint64_t* out_off, SamRead* out, char* seq, uint32_t max_len,
                   cudaStream_t st);

// ---------------------------------------------------------------- batched sequencing
// Per-instance descriptor of a batch.  The work items of instance i are its
// (sample, tile) pairs, sample-major; every table row below is relative to
// the instance's offsets, so each instance computes exactly what the plain
// path computes for it alone with the same tile size and seed.
struct SeqInst {
  SeqParams prm;
  uint32_t n_samples, sample_off;   // rows of the batch's SeqSample array
  uint32_t n_tiles, tile_off;       // rows of the batch's tile arrays
  uint32_t T;                       // tile size
  uint32_t slot_off;                // chromosome tables
  uint32_t n_blocks, blk_off;       // tile-split blocks of 64 tiles
  uint32_t etin_off;                // edge Euler table rows (n_nodes + 2)
  uint64_t pair_off;                // pair counts [sample][tile]
  uint64_t count_off;               // alt/depth of sample s: count_off + s * count_stride + record
  uint32_t count_stride;            // >= the instance's mutations
};
struct SeqBatch {
  uint32_t n_inst;
  const SeqInst* inst;
  const Key* keys;                  // sequencing key of each instance
  const uint32_t* rec_off;          // n_inst + 1: records of instance i (filled by placement)
  const uint32_t* item_off;         // n_inst + 1: first work item of each instance
  const uint32_t* cnt_off;          // n_inst + 1: first tile-split thread of each instance
  uint32_t n_items, n_cnt, n_tiles_all;
  const uint32_t *tile_start, *tile_len, *tile_end, *tile_inst;
  uint32_t *rec_lo, *rec_hi;        // per tile, relative to the instance's first record
  const uint32_t *c_first, *c_ntiles, *c_depth, *c_nstarts, *c_id;
  const uint64_t* c_pairs;
  const uint32_t *blk_slot, *blk_index;
  uint32_t* pair_cnt;
  const SeqSample* samples;
  const uint32_t* leaf_tin;
  const uint32_t *etin, *etout;
  uint32_t* counter;                // work-item counter of the persistent read kernel
  uint32_t *alt, *depth;
};
// batched placement (launchers in pg_place.cu): cells of instance i are
// [cell_off[i], cell_off[i+1]); node_off counts each instance's nodes plus its
// preneoplastic edge
void place_edge_counts_batch(const PlaceTables* tabs, uint32_t n_inst, const uint32_t* node_off, uint32_t n_nodes_all,
                             const uint32_t* cell_off, const Key* keys, const uint32_t* pre_snv, const uint32_t* pre_id,
                             uint32_t* cnt_snv, uint32_t* cnt_id, cudaStream_t st);
void place_mutations_batch(const PlaceTables* tabs, uint32_t n_inst, const uint32_t* cell_off, const Key* keys,
                           const PlaceOut& o, uint16_t* inst_of, const uint32_t* off_snv, const uint32_t* off_id,
                           uint32_t n_snv, const uint32_t* pending, uint32_t n_pending, int redraw, uint32_t* err,
                           cudaStream_t st, const uint32_t* n_dev = nullptr);
// hkeys NULL: no accepted set (the first round, whose candidate table then
// holds the taken keys); fkeys (optional): that first round's table, tested
// as taken by the later rounds
void sites_round_batch(const uint32_t* locus, const uint16_t* inst_of, const uint32_t* pending, uint32_t n,
                       uint64_t* hkeys, uint64_t hmask, uint64_t* ckeys, uint32_t* cvals, uint64_t cmask,
                       uint8_t* lost, uint32_t* next, uint32_t* n_next, uint32_t* err, cudaStream_t st,
                       const uint32_t* n_dev = nullptr, const uint64_t* fkeys = nullptr, uint64_t fmask = 0);
// every round after the first in one cooperative launch (k_sites_tail_b);
// list 0 of `a` holds the n0 losers of the first round; returns nullptr or
// a message when the launch could not be made
const char* sites_tail_batch(const PlaceTables* tabs, uint32_t n_inst, const uint32_t* cell_off, const Key* keys,
                             const PlaceOut& o, uint16_t* inst_of, const uint32_t* off_snv, const uint32_t* off_id,
                             uint32_t n_snv, const TailArgsB& a, uint32_t n0, TailCtl* ctl, uint32_t* err,
                             cudaStream_t st);
// sort by (instance, locus, slot); bcnt holds n_inst * sort_num_buckets(G)
// + 1 entries and ends as the exclusive scan of the bucket counts; keys: n
// 64-bit keys, recs: 2n 16-byte words
void sort_batch(const PlaceOut& o, const uint16_t* inst_of, uint32_t n, uint32_t n_inst, uint64_t G, uint32_t* bcnt,
                uint32_t* bfill, uint32_t* part, uint32_t* order, const PlaceOut& sorted, uint16_t* inst_sorted,
                unsigned long long* keys, uint4* recs, cudaStream_t st);
// resident CTAs per SM of the persistent read kernel
int seq_reads_batch_occupancy();
// records of the first *n_dev sorted mutations of a batch (cap >= *n_dev)
void seq_batch_records(const PlaceOut& sorted, const uint16_t* inst_sorted, const uint32_t* n_dev, uint32_t cap,
                       const SeqBatch& b, SeqRec* recs, cudaStream_t st);
// tile split, record ranges and the persistent read kernel over every work item
void seq_batch_reads(const SeqBatch& b, const SeqRec* recs, uint32_t grid, cudaStream_t st);
void seq_build_records(const PlaceOut& sorted, uint32_t n, const uint32_t* edge_tin, const uint32_t* edge_tout,
                       SeqRec* recs, cudaStream_t st);
void seq_tile_ranges(const SeqRec* recs, uint32_t n_recs, const uint32_t* start, const uint32_t* len,
                     uint32_t n_tiles, uint32_t span, uint32_t* rlo, uint32_t* rhi, cudaStream_t st);
// per (sample, tile) pair counts: multinomial split of each chromosome's
// pair count over its tiles by a binary tree of binomial draws, one launch
// per tree level (max_depth of them) with the node counts in `heap`
// (heap_total entries per sample; chromosome slot's heap at heap_base[slot],
// 2^(depth + 1) entries).  Tiles weigh their number of start positions, or
// (mass_cum != NULL) their DNA mass: mass_cum[s * n_tiles + t] is the
// sample's mass of the chromosome's tiles before t and
// mass_tot[s * n_slots + slot] the chromosome's total.
void seq_tile_counts(uint32_t n_samples, uint32_t n_slots, uint32_t max_depth, const uint32_t* chr_first_tile,
                     const uint32_t* chr_ntiles, const uint32_t* chr_depth, const uint32_t* chr_nstarts,
                     const uint32_t* chr_id, const uint64_t* chr_pairs, const uint64_t* heap_base,
                     uint64_t heap_total, uint32_t* heap, uint32_t tile_size, uint32_t n_tiles,
                     const double* mass_cum, const double* mass_tot, uint64_t seed, uint32_t* pair_cnt,
                     cudaStream_t st);
// observed rows: flag[m] = 1 when some sample has an alt read of mutation m;
// with pos the exclusive scan of the flags (n_active rows), the compact
// [sample][row] alt / depth tables and each row's mutation index
void seq_active_flags(const uint32_t* alt, uint32_t n_samples, uint64_t M, uint32_t* flag, cudaStream_t st);
void seq_active_gather(const uint32_t* alt, const uint32_t* depth, uint32_t n_samples, uint64_t M, const uint32_t* pos,
                       uint32_t n_active, uint32_t* index, uint32_t* a_out, uint32_t* d_out, cudaStream_t st);
void seq_reads(const SeqRec* recs, uint32_t n_recs, const SeqTiles& tiles, const uint32_t* pair_cnt,
               const SeqSample* samples, uint32_t n_samples, const uint32_t* leaf_tin, const SeqParams& prm,
               uint64_t seed, uint32_t* alt, uint32_t* depth, cudaStream_t st);

// ---------------------------------------------------------------- calibration
struct CalibArgs {
  uint32_t K, J, C, P;          // epochs, signatures, classes, parameters per replicate
  const int32_t* alt;           // sites of all replicates, concatenated
  const int32_t* depth;
  const int32_t* cls;
  const uint64_t* site_off;     // n_rep + 1
  const float* sig;             // J x C
  const float* epoch_w;         // n_rep x K  (L_k: relative length of epoch k)
  const float* phi;             // n_rep x K  (mean cellular fraction of epoch-k mutations)
  uint32_t chunk;               // sites per CTA
  uint32_t part_stride;         // floats per chunk partial (>= 1 + 3K + K J)
  uint32_t chunk0, rep0;        // first chunk / replicate of a launch (sub-range launches)
  const float* sig_rows;        // C x JP: S_j(c) by class, JP = 4 (J <= 4) or 8 floats, zero beyond J
  float* tab;                   // per replicate: log(exp(lr_k) L_k / Z), log v_k, log(1 - v_k), w_kj
  uint32_t tab_stride;          // floats per replicate in tab
};
struct AdamArgs {               // m == nullptr: no optimizer step
  float* m; float* v; uint32_t* step;
  float lr, beta1, beta2, eps;
};
// k_calib_sites over chunks [a.chunk0, a.chunk0 + n_chunks), then the
// epilogue for replicates [a.rep0, a.rep0 + n_rep)
void calib_launch(const CalibArgs& a, float* params, const uint32_t* chunk_rep, const uint64_t* chunk_start,
                  uint32_t n_chunks, const uint32_t* rep_first_chunk, uint32_t n_rep, float* partial, float* nll,
                  float* grad, const AdamArgs& adam, cudaStream_t st);

}  // namespace pg
