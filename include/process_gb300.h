/*
 * process_gb300 — C-ABI of the GB300 mutation-placement and bulk-sequencing
 * path of ProCESS.
 *
 * The two RACES call sites this library replaces are
 *   m_engine.place_mutations(...)      src/mutation_engine.cpp:1097-1101
 *   simulator(sequencer, ...)          src/seq_simulation.cpp:371,413,423
 * Everything above them (the Rcpp modules src/mutations.cpp:392-756,
 * src/sequencing.cpp:193-282 and the data-frame flatteners
 * src/seq_simulation.cpp:52-181) keeps its signatures; the Rcpp shim maps
 * each argument onto the calls below.
 *
 * Conventions
 *   - Every function returns a pg_status; 0 is success.  On failure
 *     pg_last_error() holds a message for the calling thread; the Rcpp shim
 *     rethrows it as std::runtime_error / std::domain_error, as the reference
 *     does (src/sequencers.cpp:78-105, src/seq_simulation.cpp:431-451).
 *   - Handles are opaque and owned by the library until their _destroy call.
 *     Inputs are copied during the call: the caller may free them afterwards.
 *   - Calls are synchronous on the engine's CUDA stream; device results stay
 *     in HBM until a _copy function moves them to caller-owned host memory.
 *   - Chromosome positions in/out are 1-based (chr_pos); absolute positions
 *     are 0-based offsets into the concatenated genome.
 */
#ifndef PROCESS_GB300_H
#define PROCESS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int pg_status;
enum {
  PG_OK = 0,
  PG_ERR_DOMAIN = 1,      /* invalid argument (reference: std::domain_error) */
  PG_ERR_RUNTIME = 2,     /* runtime failure (reference: std::runtime_error) */
  PG_ERR_CUDA = 3,        /* CUDA error or no device */
  PG_ERR_NOMEM = 4,       /* device allocation failed */
  PG_ERR_UNSUPPORTED = 5  /* feature not built in this library */
};

typedef struct pg_engine pg_engine;
typedef struct pg_forest pg_forest;
typedef struct pg_placed pg_placed;
typedef struct pg_seq_result pg_seq_result;

/* Message of the last failed call on this thread ("" if none). */
const char* pg_last_error(void);
/* Library version string. */
const char* pg_version(void);
/* Number of visible CUDA devices (0 when none). */
pg_status pg_device_count(int* n);

/* ------------------------------------------------------------------ engine
 * Replaces MutationEngine construction: build_MutationEngine /
 * init_mutation_engine (src/mutation_engine.cpp:489-496, 653-699), i.e. the
 * reference genome load plus build_contex_index (:211-275, call
 * ContextIndex::build_index :260) and build_rs_index (:289-359, call
 * RSIndex::build_index :344).  Both indices are built on the GPU. */
typedef struct {
  uint32_t n_chr;
  const uint32_t* chr_lengths;      /* bases per chromosome */
  const uint8_t* bases;             /* concatenated codes A=0 C=1 G=2 T=3, above 3 an unknown base (N,
                                       not indexed, read as 4 and as N in SAM), or NULL: synthetic genome */
  uint64_t synthetic_seed;          /* seeded i.i.d. bases when bases == NULL */
  double synthetic_gc;              /* GC fraction of the synthetic genome */
  uint32_t context_sampling;        /* keep 1 in N occurrences per context (reference default 100) */
  uint32_t max_repetition_storage;  /* positions kept per ID class (reference default 500000) */
  /* Regions to avoid: positions the SBS context index leaves out, as
   * build_contex_index does for the driver catalogue (each driver's position
   * and max(1, |ref|) bases; src/mutation_engine.cpp:240-250, 260); the ID
   * index keeps them (:323-334).  n_avoid 0: none. */
  uint32_t n_avoid;
  const uint32_t* avoid_chr;        /* chromosome index */
  const uint32_t* avoid_begin;      /* 1-based first position */
  const uint32_t* avoid_len;        /* bases, at least 1 */
  /* Directory of the index caches (the reference's .cif / .rsif files,
   * :199-209, 225-238, 277-318), or NULL / "": no cache.  The context index is
   * kept as context_index_<context_sampling>.pgcif and the ID index as
   * rs_index_<max_repetition_storage>.pgrsif, each with a format version, a
   * fingerprint of the genome and (context index) of the regions to avoid.
   * An existing file is loaded instead of building the index; a file of
   * another version, genome or regions is refused with PG_ERR_DOMAIN. */
  const char* index_cache_dir;
} pg_genome_desc;

pg_status pg_engine_create(const pg_genome_desc* genome, pg_engine** out);
pg_status pg_engine_destroy(pg_engine* eng);
/* Runs every later call of the engine on the caller's cudaStream_t (NULL =
 * the engine's own stream).  No reference counterpart: the reference has no
 * device; this lets a host framework order the calls with its own work. */
pg_status pg_engine_set_stream(pg_engine* eng, void* cuda_stream);
/* Number of kernels this library has launched in the process so far. */
pg_status pg_launch_count(uint64_t* n);

/* Per-class position counts of a genome the caller already holds in device
 * memory, computed without allocating any device memory.  No reference
 * counterpart: it exists for callers that must not call cudaMalloc, such as a
 * host framework whose pooling allocator owns the device memory, code that
 * runs while a stream is being captured, or a latency-bound loop that cannot
 * afford the device-wide synchronisation an allocation can cause.
 *   which          0: the 32 SBS trinucleotide contexts; 1: the 83 ID classes
 *   genome_words   device pointer, 2-bit codes (A=0 C=1 G=2 T=3), 16 bases per
 *                  u32 word, base i in bits 2*(i%16); at least
 *                  ceil(genome_len/16) words
 *   genome_len     total bases, at most 8,388,608 (larger genomes are rejected
 *                  with PG_ERR_DOMAIN)
 *   chr_off        device pointer, n_chr + 1 chromosome start offsets (the
 *                  last one is genome_len)
 *   class_totals   device pointer, 32 or 83 u64 counts (overwritten)
 *   stream         cudaStream_t the two kernels are queued on (NULL: legacy
 *                  default stream); the call returns without waiting.
 * The per-tile counts live in one fixed 2.7 MB array of the library's own
 * device memory, present on every GPU that loads the library until the
 * process exits.  The first call on a device looks up that array's device
 * address and keeps it for the life of the process (a cudaDeviceReset
 * invalidates it: do not call this after resetting the device); make the
 * first call before capturing a stream into a CUDA graph.  A CUDA error left
 * pending by earlier work on the calling thread makes the call fail with
 * PG_ERR_CUDA before launching anything, and stays pending.  All calls
 * share the array: calls whose kernels overlap on the GPU (different
 * streams, or concurrent host threads) race and return wrong counts;
 * serialise them on one stream.  The counts equal pg_engine_genome_info's
 * ctx_total / id_total for the same genome. */
pg_status pg_index_counts_noalloc(int which, const uint32_t* genome_words, uint64_t genome_len,
                                  const uint32_t* chr_off, uint32_t n_chr, uint64_t* class_totals, void* stream);

/* Genome size and per-class position counts of the indices (ctx: 32 entries,
 * id: 83 entries; either may be NULL).  get_genome_info, src/mutation_engine.cpp. */
pg_status pg_engine_genome_info(const pg_engine* eng, uint64_t* total_len, uint64_t* ctx_total,
                                uint64_t* id_total, uint32_t* ctx_stored, uint32_t* id_stored);
/* Copies n bases (codes 0..3) of the concatenated genome from `start`. */
pg_status pg_engine_read_genome(const pg_engine* eng, uint64_t start, uint64_t n, uint8_t* out);
/* Bases (codes 0..3; 4 outside the genome) at n absolute positions. */
pg_status pg_engine_gather_bases(const pg_engine* eng, uint64_t n, const uint32_t* positions, uint8_t* out);
/* Copies the stored positions of index class `cls` (which: 0 = SBS context, 1 = ID class). */
pg_status pg_engine_read_index(const pg_engine* eng, int which, uint32_t cls, uint32_t* out, uint32_t capacity,
                               uint32_t* n_out);

/* Signatures (Signature<SBSType|IDType>::read_from_stream,
 * src/mutation_engine.cpp:389-397): n_sigs rows of 96 (type 0, SBS) or 83
 * (type 1, ID) class probabilities in COSMIC order. */
pg_status pg_engine_set_signatures(pg_engine* eng, int type, uint32_t n_sigs, const double* probs);
/* MutationEngine::add_exposure(time, exposure) (src/mutation_engine.cpp:734-739):
 * coefficients over the n_sigs signatures of `type`, active from `time`. */
/* Signature<SBSType|IDType>::read_from_stream (src/mutation_engine.cpp:389-397):
 * a tab-separated table whose header is "Type" and the signature names, one
 * row per class labelled as COSMIC does ("A[C>A]A" for the 96 SBS classes,
 * "1:Del:C:0" .. "5:Del:M:5" for the 83 ID classes), rows in any order,
 * every class once.  load: sets the engine's signatures of the type (as
 * pg_engine_set_signatures) and their names.  read: the table alone, without
 * an engine or a device: *n_sigs, the names NUL-separated (*names_size
 * bytes) and probs [n_sigs][96 or 83]; outputs may be NULL. */
pg_status pg_engine_load_signatures_tsv(pg_engine* eng, int type, const char* path);
pg_status pg_signature_table_read(int type, const char* path, uint32_t* n_sigs, uint64_t* names_size, char* names,
                                  double* probs);
pg_status pg_engine_add_exposure(pg_engine* eng, int type, double time, const double* coeffs);
/* Passenger rates per base per division of a species (mutant + epistate),
 * MutationEngine::add_mutant / get_passenger_rates (src/mutation_engine.cpp:864-1083). */
pg_status pg_engine_set_species_rates(pg_engine* eng, uint32_t species, double snv, double indel, double cna);
/* Per-epoch passenger rates (epoch = interval between consecutive exposure
 * change times); overrides the constant rates of the species. */
pg_status pg_engine_set_species_epoch_rates(pg_engine* eng, uint32_t species, uint32_t n_epochs,
                                            const double* snv, const double* indel);
/* Mutant of a species: drivers are applied on the first edge whose mutant
 * differs from its parent's (driver lists, src/mutation_engine.cpp:789-862). */
pg_status pg_engine_set_species_mutant(pg_engine* eng, uint32_t species, uint32_t mutant);
/* Driver SNV/indel of a mutant, in application order (SIDMut, src/sid.cpp:18-146).
 * ref/alt are base strings (indels: VCF style, sharing the first base);
 * allele < 0 = random allele. */
pg_status pg_engine_add_driver_sid(pg_engine* eng, uint32_t mutant, uint32_t chr_index, uint32_t chr_pos,
                                   const char* ref, const char* alt, int32_t allele);
/* Driver CNA (CNA(type, chr, chr_pos, len, allele, src_allele), src/cna.cpp:21-138)
 * and whole-genome doubling (src/wg_doubling.hpp:28-40), appended to the
 * mutant's driver list in application order.  Alleles are ordinals among the
 * allele instances covering the region start (-1 = random). */
pg_status pg_engine_add_driver_cna(pg_engine* eng, uint32_t mutant, int type_amplification, uint32_t chr_index,
                                   uint32_t begin, uint32_t length, int32_t allele, int32_t src_allele);
pg_status pg_engine_add_driver_wgd(pg_engine* eng, uint32_t mutant);
/* Passenger CNA candidate (load_passenger_CNAs, src/mutation_engine.cpp:441-487):
 * each passenger CNA event draws one candidate uniformly. */
pg_status pg_engine_add_passenger_cna(pg_engine* eng, uint32_t chr_index, uint32_t begin, uint32_t length,
                                      int type_amplification);
/* avoid_homozygous_losses (src/mutation_engine.cpp:1356, src/mutations.cpp:837-840):
 * passenger deletions never remove the last allele of a region. */
pg_status pg_engine_set_avoid_homozygous_losses(pg_engine* eng, int on);
/* infinite_sites_model property (src/mutation_engine.hpp:148-156). */
pg_status pg_engine_set_infinite_sites(pg_engine* eng, int on);
pg_status pg_engine_get_infinite_sites(const pg_engine* eng, int* on);

/* ------------------------------------------------------------------ forest
 * SamplesForest (src/samples_forest.hpp:31, node fields src/forest.hpp:29-68):
 * nodes in topological order (parent index < node index, -1 for roots),
 * birth time, species id, sample index of leaves (-1 for internal nodes) and
 * the number of cell divisions on the edge into the node (NULL = 1 each). */
pg_status pg_forest_create(uint32_t n_nodes, const int32_t* parent, const double* birth, const uint32_t* species,
                           const int32_t* sample, const uint32_t* divisions, uint32_t n_samples, pg_forest** out);
pg_status pg_forest_destroy(pg_forest* forest);

/* ------------------------------------------------------------------ placement
 * MutationEngine::place_mutations(forest, #preneoplastic SNVs, SBS signature,
 * #preneoplastic indels, ID signature, seed) (src/mutation_engine.cpp:1085-1113;
 * R defaults "SBS1"/"ID1", src/mutation_engine.hpp:160-206): sig indices
 * select rows of the signature tables. */
pg_status pg_place_mutations(pg_engine* eng, const pg_forest* forest, uint32_t n_pre_snv, uint32_t pre_sbs_sig,
                             uint32_t n_pre_indel, uint32_t pre_id_sig, uint64_t seed, pg_placed** out);
pg_status pg_placed_destroy(pg_placed* placed);
pg_status pg_placed_count(const pg_placed* placed, uint64_t* n_mutations);
/* Placed mutations sorted by (absolute locus, slot); any pointer may be NULL.
 * aux: SNV alt base code; indel bit0 = insertion, bits1-3 = length, bits 8.. inserted bases. */
pg_status pg_placed_copy(const pg_placed* placed, uint32_t* locus, uint32_t* edge, uint32_t* aux, uint8_t* cls,
                         uint8_t* sig, uint16_t* allele, uint8_t* kind, uint8_t* nature);
/* Applied CNA / WGD events (type 0 deletion, 1 amplification, 2 WGD), with
 * the edge (node) they happened on, their 1-based inclusive region, the
 * allele instance they created (amplification) or acted on (deletion) and its
 * source instance, and whether they are drivers: the rows of the reference's
 * get_sampled_cell_CNAs (src/phylogenetic_forest.cpp:509-562) before they are
 * expanded per cell. */
pg_status pg_placed_cna_count(const pg_placed* placed, uint64_t* n);
pg_status pg_placed_cna_copy(const pg_placed* placed, uint32_t* node, uint8_t* type, uint32_t* chr, uint32_t* begin,
                             uint32_t* end, uint32_t* allele, uint32_t* src_allele, uint8_t* driver);
/* Genotype class of every node (n_nodes entries) and the class count / the
 * largest copy number of any position. */
pg_status pg_placed_node_classes(const pg_placed* placed, uint32_t* node_class, uint32_t* n_classes,
                                 uint32_t* cn_max);
/* The samples the next pg_simulate_seq calls sequence: sample_of_node[v] in
 * [0, n_samples) puts leaf v (a sampled cell) in that sample, -1 leaves it
 * out.  This is how the FACS labelling of simulate_seq(cell_labelling = f)
 * (src/seq_simulation.cpp:183-243, split_by_labels / apply_FACS_labels)
 * arrives: the shim evaluates f on each sampled cell before the call and
 * passes the partition; sample names stay with the caller. */
pg_status pg_placed_set_samples(pg_placed* placed, uint32_t n_samples, const int32_t* sample_of_node);
/* The allele-instance lineage behind the per-cell mutation lists of
 * get_sampled_cell_mutations (src/phylogenetic_forest.cpp:452-507, where an
 * SID sits on every allele copied from its allele after it and leaves with a
 * deleted allele): for instance y, its ancestors chain_anc[chain_off[y] ..
 * chain_off[y+1]) nearest first, each with the order key of the copy that
 * led towards y; order_key[m] is mutation m's key (tin of its edge << 16 |
 * order on the edge, in the order of pg_placed_copy).  Instance y carries
 * mutation m placed on instance x when y == x or x is in y's chain with a
 * key above order_key[m]. */
pg_status pg_placed_lineage_dims(const pg_placed* placed, uint32_t* n_instances, uint32_t* n_links);
pg_status pg_placed_lineage_copy(const pg_placed* placed, uint32_t* chain_off, uint16_t* chain_anc,
                                 uint64_t* chain_key, uint64_t* order_key);
/* Genotype classes as segments (for the allelic fragmentation getters,
 * src/phylogenetic_forest.cpp:767-927): class c covers the absolute 0-based
 * intervals [seg_start, seg_end) of its segments seg_off[c] .. seg_off[c+1]-1,
 * each with the allele instances inst_list[seg_ioff .. seg_ioff + seg_icnt);
 * inst_root gives the germline allele (0 or 1) every instance descends from.
 * Sizes: n_classes + 1, n_segments (x4), n_list, n_instances. */
pg_status pg_placed_class_dims(const pg_placed* placed, uint32_t* n_classes, uint32_t* n_segments, uint32_t* n_list,
                               uint32_t* n_instances);
pg_status pg_placed_class_copy(const pg_placed* placed, uint32_t* seg_off, uint32_t* seg_start, uint32_t* seg_end,
                               uint32_t* seg_ioff, uint32_t* seg_icnt, uint16_t* inst_list, uint8_t* inst_root);
/* Device time of the placement kernels of the last place call (ms). */
pg_status pg_placed_kernel_ms(const pg_placed* placed, float* ms);
// Redraw rounds of the placement (infinite sites collisions and loci drawn
// where the cell has no allele left): the round counter after the last
// round run, counting the first infinite-sites round as round 0; 0 when no
// round after the first ran.
pg_status pg_placed_redraw_rounds(const pg_placed* placed, uint32_t* rounds);
// Device time (ms) of the engine's index build: ms[0] SBS context count pass
// (with its scan over the units), ms[1] its emit pass, ms[2] and ms[3] the
// same for the ID83 index; zeros for an index read from a cache.
pg_status pg_engine_index_ms(const pg_engine* engine, float* ms);

/* ------------------------------------------------------------------ data frames
 * The data frames of the reference's PhylogeneticForest getters, built in
 * the library so that the Rcpp layer only turns columns into a data frame.
 * Cells are node ids of leaves (the shim maps them to cell ids); mutations
 * are row indices in the order of pg_placed_copy.  Each builder keeps its
 * result in the handle until the next call of the same builder, and its
 * _copy call fills caller buffers of the returned row count (any pointer may
 * be NULL).  Builders of one handle must not run concurrently.
 *
 * ref / alt strings: PG_SID_CHARS bytes per row, NUL-padded.  SNV: reference
 * base, alt base; insertion: anchor base, anchor + inserted bases; deletion:
 * anchor + deleted bases, anchor base.  Unknown reference bases read "N". */
#define PG_SID_CHARS 16

/* Names of the signatures of a type (0 SBS, 1 ID) as set by
 * pg_engine_set_signatures (one per signature, in that order), used for the
 * causes of the data frames; Signature::read_from_stream keeps them with the
 * probabilities (src/mutation_engine.cpp:389-397). */
pg_status pg_engine_set_signature_names(pg_engine* eng, int type, uint32_t n, const char* const* names);
/* Name of signature `index` of a type ("SBS#<index + 1>" / "ID#<index + 1>"
 * when none was set): *length characters, NUL-terminated into out when out
 * is not NULL (capacity bytes, truncated). */
pg_status pg_engine_signature_name(const pg_engine* eng, int type, uint32_t index, char* out, uint32_t capacity,
                                   uint32_t* length);
/* Columns of n placed mutations (rows[i], or rows 0..n-1 when rows is NULL):
 * chromosome index, 1-based position, ref, alt, kind (0 SNV, 1 indel), cause
 * (signature index of the kind, -1 none: drivers) and nature (0 passenger,
 * 1 driver, 2 preneoplastic).  The per-row columns of
 * get_sampled_cell_mutations (src/phylogenetic_forest.cpp:452-507). */
pg_status pg_placed_mutation_info(const pg_placed* placed, uint64_t n, const uint32_t* rows, uint32_t* chr,
                                  uint32_t* chr_pos, char* ref, char* alt, uint8_t* kind, int32_t* cause,
                                  uint8_t* nature);
/* get_sampled_cell_mutations (src/phylogenetic_forest.cpp:452-507): for each
 * cell (cells[i], or every sampled leaf by node id when cells is NULL), every
 * mutation it holds, once per allele instance of its genome that carries it
 * (the placed instance and its copies made after the mutation, while present
 * at the locus).  A cell's rows are ordered by chromosome, allele instance,
 * position, as fill_mutation_lists nests them (:323-351). */
pg_status pg_placed_cell_mutations(pg_placed* placed, uint32_t n_cells, const uint32_t* cells, uint64_t* n_rows);
pg_status pg_placed_cell_mutations_copy(const pg_placed* placed, uint32_t* cell, uint32_t* mutation,
                                        uint32_t* allele);
/* get_sampled_cell_CNAs (src/phylogenetic_forest.cpp:509-562): for each cell,
 * the CNA / WGD events on its root path, as indices of pg_placed_cna_copy,
 * in event order. */
pg_status pg_placed_cell_cnas(pg_placed* placed, uint32_t n_cells, const uint32_t* cells, uint64_t* n_rows);
pg_status pg_placed_cell_cnas_copy(const pg_placed* placed, uint32_t* cell, uint32_t* cna_index);
/* get_cell_allelic_fragmentation (src/phylogenetic_forest.cpp:867-927): for
 * each cell, its genome cut into maximal stretches of one allelic type
 * (copies of germline alleles 0 and 1; major the larger), per chromosome;
 * chromosome index, 1-based inclusive begin / end.  Deleted stretches have
 * type (0, 0). */
pg_status pg_placed_cell_fragmentation(pg_placed* placed, uint32_t n_cells, const uint32_t* cells,
                                       uint64_t* n_rows);
pg_status pg_placed_cell_fragmentation_copy(const pg_placed* placed, uint32_t* cell, uint32_t* chr, uint32_t* begin,
                                            uint32_t* end, uint32_t* major, uint32_t* minor);
/* get_bulk_allelic_fragmentation([sample_name]) (src/phylogenetic_forest.cpp:
 * 767-820): the genome cut where the allelic type of some sampled cell (of
 * the sample, or of every sample when sample < 0) changes; per stretch one
 * row per allelic type with the fraction of cells that show it (ratio),
 * types ascending, the cells without DNA there last as type (0, 0). */
pg_status pg_placed_bulk_fragmentation(pg_placed* placed, int32_t sample, uint64_t* n_rows);
pg_status pg_placed_bulk_fragmentation_copy(const pg_placed* placed, uint32_t* chr, uint32_t* begin, uint32_t* end,
                                            uint32_t* major, uint32_t* minor, double* ratio);
/* PhylogeneticForest$save / load_phylogenetic_forest (src/phylogenetic_forest.cpp:
 * 940-992, src/mutations.cpp:1466-1480).  The reference archives its RACES
 * forest; this library writes a versioned native archive of the placed
 * forest (Euler numbering and samples, placed mutations, genotype classes,
 * allele-instance lineage, CNA events) and a fingerprint of the engine's
 * genome.  Loading restores the handle without placing again; the engine
 * must hold the same genome (PG_ERR_DOMAIN otherwise, and for a file that is
 * missing, not a regular file, of another format version or truncated).
 * serialize: *size bytes, written to buf when buf is not NULL (capacity >=
 * *size); save / load: the same bytes in a file. */
pg_status pg_placed_serialize(const pg_placed* placed, uint8_t* buf, uint64_t capacity, uint64_t* size);
pg_status pg_placed_deserialize(pg_engine* eng, const uint8_t* buf, uint64_t size, pg_placed** out);
pg_status pg_placed_save(const pg_placed* placed, const char* path);
pg_status pg_placed_load(pg_engine* eng, const char* path, pg_placed** out);
/* get_samples_info (src/phylogenetic_forest.cpp:57-99): per sample its
 * sampled cells, its DNA quantity (the summed allelic size of their genomes)
 * and that in normal diploid genomes; arrays of n_samples entries. */
pg_status pg_placed_samples_info(const pg_placed* placed, uint32_t* n_cells, double* dna_quantity,
                                 double* equivalent_normal_cells);

/* ------------------------------------------------------------------ sequencing
 * simulate_seq / simulate_normal_seq (src/seq_simulation.cpp:517-679; R
 * defaults src/sequencing.cpp:193-209,268-282) down to the read simulator. */
enum { PG_INSERT_BINOMIAL = 0, PG_INSERT_NORMAL = 1 };
typedef struct {
  double coverage;              /* default 10 */
  uint32_t read_size;           /* default 150 */
  uint32_t insert_size_mean;    /* 0 = single-end reads */
  uint32_t insert_size_stddev;  /* default 10 */
  int insert_model;             /* PG_INSERT_BINOMIAL (reference get_bin_dist) or PG_INSERT_NORMAL */
  double error_rate;            /* BasicIlluminaSequencer error rate; 0 = ErrorlessIlluminaSequencer */
  double purity;                /* default 1 */
  int with_normal_sample;       /* default 1 */
  int preneoplastic_in_normal;  /* default 0 */
  int normal_only;              /* simulate_normal_seq: sequence only the normal sample */
  uint32_t n_chr_sel;           /* 0 = every chromosome */
  const uint32_t* chr_sel;      /* chromosome indices */
  uint32_t tile_size;           /* 0 = automatic */
} pg_seq_cfg;

pg_status pg_simulate_seq(const pg_placed* placed, const pg_seq_cfg* cfg, uint64_t seed, pg_seq_result** out);
pg_status pg_seq_result_destroy(pg_seq_result* res);
/* Sequenced samples = forest samples (+ the normal sample, last). */
pg_status pg_seq_result_dims(const pg_seq_result* res, uint32_t* n_samples, uint64_t* n_mutations,
                             uint64_t* n_reads);
/* alt ("occurrences") and depth ("coverage") as [n_samples][n_mutations]
 * int32, in the order of pg_placed_copy. */
pg_status pg_seq_result_copy(const pg_seq_result* res, int32_t* alt, int32_t* depth);
/* Device time of the read kernel of the call (ms). */
pg_status pg_seq_result_kernel_ms(const pg_seq_result* res, float* ms);
/* Tile size (bp of fragment starts per read-kernel work item) the call used:
 * cfg->tile_size, or the automatic choice when that was 0.  The draws depend
 * on it, so a replay of the call needs it.  No reference counterpart (the
 * reference has no tiles). */
pg_status pg_seq_result_tile_size(const pg_seq_result* res, uint32_t* tile_size);
/* The observed rows: mutations with an alt read in some sample, the rows the
 * reference's result data frame keeps by default (include_non_sequenced_
 * mutations = FALSE; src/seq_simulation.cpp:52-90, 142-181).  Built on the
 * device on the first call; n_active = their number. */
pg_status pg_seq_result_active(pg_seq_result* res, uint64_t* n_active);
/* Their mutation indices (n_active, ascending, in the order of
 * pg_placed_copy) and alt / depth as [n_samples][n_active] int32; any
 * pointer may be NULL.  Requires pg_seq_result_active first. */
pg_status pg_seq_result_copy_active(const pg_seq_result* res, uint32_t* index, int32_t* alt, int32_t* depth);
/* The result data frame of simulate_seq (get_result_dataframe,
 * src/seq_simulation.cpp:52-181), built from a result and the placed
 * mutations it was simulated from: one row per SID (chromosome, position,
 * ref, alt) in that order, over the observed mutations (alt read in some
 * sample) or, with include_non_sequenced, also every mutation present in the
 * cells of a sequenced sample.  Rows of one SID merge: occurrences add, the
 * coverage is the locus's, causes are the sorted union of signature names
 * joined by ';' (empty: NA), classes a bit set of natures (bit 0 passenger,
 * 1 driver, 2 preneoplastic; the reference joins their sorted names).  Per
 * sample occurrences, coverage and VAF = occurrences / coverage (0 without
 * coverage) as [n_samples][n_rows].  causes_off holds n_rows + 1 offsets
 * into the causes characters (pg_seq_result_frame_causes_size of them). */
pg_status pg_seq_result_frame(pg_seq_result* res, const pg_placed* placed, int include_non_sequenced,
                              uint64_t* n_rows);
pg_status pg_seq_result_frame_causes_size(const pg_seq_result* res, uint64_t* n_chars);
pg_status pg_seq_result_frame_copy(const pg_seq_result* res, uint32_t* chr, uint32_t* chr_pos, char* ref, char* alt,
                                   uint64_t* causes_off, char* causes, uint8_t* classes, int32_t* occurrences,
                                   int32_t* coverage, double* vaf);

/* simulate_seq with write_SAM = TRUE (src/seq_simulation.cpp:540-564; files
 * and naming of vignettes/sequencing.Rmd:137-180, 282-317): the counts of
 * pg_simulate_seq, and one SAM file per chromosome,
 * <output_dir>/<filename_prefix><chromosome name>.sam, holding the reads of
 * every sequenced sample as read groups named after the samples.  The
 * directory is created; when it exists the call fails unless `update` is set,
 * and then a chromosome whose file exists goes to the first free
 * <filename_prefix><chromosome name>_<n>.sam, n = 1, 2, ...  A read's bases
 * are the reference with the mutations its allele carries and its
 * substitution errors (the same draws as the counts); template names are
 * template_name_prefix followed by a number per file; qualities are the
 * Phred value of the error rate. */
typedef struct pg_sam_cfg {
  const char* output_dir;
  const char* filename_prefix;        /* R default "chr_" */
  const char* template_name_prefix;   /* R default "r" */
  int update;                         /* update_SAM */
  const char* const* sample_names;    /* one per sequenced sample (normal last) */
  const char* const* chr_names;       /* one per chromosome of the engine */
} pg_sam_cfg;
pg_status pg_simulate_seq_sam(const pg_placed* placed, const pg_seq_cfg* cfg, uint64_t seed, const pg_sam_cfg* sam,
                              pg_seq_result** out);

/* ------------------------------------------------------------------ calibration
 * Expected-VAF binomial-mixture negative log-likelihood of alt/depth tables
 * and its gradient (no reference counterpart: ProCESS has no calibration
 * path).  Per replicate r: sites (alt, depth, class) with class in [0, C);
 * K epochs of relative length L_k (epoch_weight) whose mutations have mean
 * cellular fraction phi_k; J signatures over the C classes.  Parameters per
 * replicate (P = K + K*J + 1 floats): log rates lr_k, exposure logits
 * theta_kj (softmax over j) and the purity logit rho:
 *   pi_k(c) = e^lr_k L_k sum_j softmax(theta_k)_j S_j(c) / sum_k' e^lr_k' L_k'
 *   v_k = sigmoid(rho) phi_k / 2
 *   NLL = -sum_i log sum_k pi_k(c_i) v_k^a_i (1 - v_k)^(d_i - a_i)
 * Computed in FP32 with compensated sums. */
typedef struct pg_calib pg_calib;
pg_status pg_calib_create(uint32_t n_rep, const uint64_t* site_off, const int32_t* alt, const int32_t* depth,
                          const int32_t* cls, uint32_t K, uint32_t J, uint32_t C, const double* signatures,
                          const double* epoch_weight, const double* phi, pg_calib** out);
pg_status pg_calib_destroy(pg_calib* cal);
pg_status pg_calib_num_params(const pg_calib* cal, uint32_t* P);
/* every later call of the handle runs on this cudaStream_t (NULL: its own stream) */
pg_status pg_calib_set_stream(pg_calib* cal, void* cuda_stream);
/* Batched: NLL and gradient of every replicate in one launch of each kernel.
 * params, nll and grad are device pointers (n_rep x P, n_rep, n_rep x P);
 * nll or grad may be NULL.  Asynchronous on the handle's stream. */
pg_status pg_calib_nll_grad(pg_calib* cal, const float* params, float* nll, float* grad);
/* One replicate only (the per-instance path): same layout, replicate `rep`. */
pg_status pg_calib_nll_grad_one(pg_calib* cal, uint32_t rep, const float* params, float* nll, float* grad);
/* `steps` Adam steps on every replicate's parameters (device, updated in
 * place), run entirely on the device as one CUDA graph; nll (device, n_rep,
 * may be NULL) receives the NLL of the last step's parameters before the
 * update.  The optimizer state restarts at zero on each call. */
pg_status pg_calib_adam(pg_calib* cal, float* params, uint32_t steps, float lr, float beta1, float beta2, float eps,
                        float* nll);

/* ------------------------------------------------------------------ batches
 * Many independent instances on one engine's genome and signatures (no
 * reference counterpart: the reference places and sequences one instance per
 * MutationEngine$place_mutations / simulate_seq call).  Instance i has its own
 * forest (every node of species 0), passenger rates snv_rate[i] /
 * indel_rate[i] per base per division, one exposure (row i of sbs_expo over
 * the engine's SBS signatures and of id_expo over its ID signatures; NULL =
 * zero), preneoplastic counts (NULL = none) of the signatures pre_sbs_sig /
 * pre_id_sig, and a sequencing configuration (cfgs[i].tile_size 0 = the
 * analytic size).  A run computes for every instance exactly what the plain
 * path computes for it alone (pg_place_mutations then pg_simulate_seq on an
 * engine whose species 0 has those rates and that exposure at time 0, with
 * the same seeds and the instance's tile size).  Placement runs as single
 * launches over all instances; sequencing as one persistent kernel over every
 * (instance, sample, tile), captured into a CUDA graph on the first run and
 * replayed afterwards. */
typedef struct pg_batch pg_batch;
pg_status pg_batch_create(pg_engine* eng, uint32_t n_inst, const pg_forest* const* forests, const double* snv_rate,
                          const double* indel_rate, const double* sbs_expo, const double* id_expo,
                          const uint32_t* n_pre_snv, uint32_t pre_sbs_sig, const uint32_t* n_pre_indel,
                          uint32_t pre_id_sig, const pg_seq_cfg* cfgs, pg_batch** out);
pg_status pg_batch_destroy(pg_batch* batch);
/* place and sequence every instance with its placement and sequencing seed */
pg_status pg_batch_run(pg_batch* batch, const uint64_t* place_seed, const uint64_t* seq_seed);
/* The autotuner: places once with these seeds, then times the whole
 * persistent read launch for candidate tile sizes (multiples 0.5, 0.75, 1,
 * 1.25 of every instance's analytic size) and keeps the fastest; tile_sizes
 * (may be NULL) receives the choice. */
pg_status pg_batch_autotune(pg_batch* batch, const uint64_t* place_seed, const uint64_t* seq_seed,
                            uint32_t* tile_sizes);
pg_status pg_batch_tile_sizes(const pg_batch* batch, uint32_t* tile_sizes);
pg_status pg_batch_set_tile_sizes(pg_batch* batch, const uint32_t* tile_sizes);
/* after a run: instance inst's mutations, sequenced samples and reads */
pg_status pg_batch_dims(const pg_batch* batch, uint32_t inst, uint64_t* n_mutations, uint32_t* n_samples,
                        uint64_t* n_reads);
/* instance inst's placed mutations (sorted by locus, the columns of
 * pg_placed_copy) and its alt/depth tables [sample][mutation]; any pointer may
 * be NULL */
pg_status pg_batch_copy(const pg_batch* batch, uint32_t inst, uint32_t* locus, uint32_t* edge, uint32_t* aux,
                        uint8_t* cls, uint8_t* sig, uint16_t* allele, uint8_t* kind, uint8_t* nature, int32_t* alt,
                        int32_t* depth);
/* device time of the last run's placement and sequencing stages (ms) */
pg_status pg_batch_kernel_ms(const pg_batch* batch, float* place_ms, float* seq_ms);

#ifdef __cplusplus
}
#endif

#endif /* PROCESS_GB300_H */
