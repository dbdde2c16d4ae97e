// C-ABI of the library (declared in include/process_gb300.h): handles,
// validation, host-side table preparation and orchestration of the kernels.
#include "../../include/process_gb300.h"
#include "pg_common.cuh"
#include "pg_kernels.h"
#include "pg_scan.cuh"
#include "pg_genome.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <thread>
#include <atomic>
#include <cmath>
#include <cstring>
#include <cstdlib>
#include <filesystem>
#include <fstream>
#include <map>
#include <memory>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

namespace {
std::atomic<uint64_t> g_launches{0};
}

void pg::note_launch(uint32_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

namespace {

thread_local std::string g_last_error;

struct DomainError : std::runtime_error { using std::runtime_error::runtime_error; };
struct Unsupported : std::runtime_error { using std::runtime_error::runtime_error; };
struct CudaError : std::runtime_error { using std::runtime_error::runtime_error; };
struct NoMem : std::runtime_error { using std::runtime_error::runtime_error; };

void ck(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    if (e == cudaErrorMemoryAllocation) { cudaGetLastError(); throw NoMem(std::string(what) + ": out of device memory"); }
    throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
  }
}

template <class F>
pg_status guarded(F&& f) {
  try {
    cudaGetLastError();   // a stale non-sticky error of an earlier call is not this call's error
    f();
    g_last_error.clear();
    return PG_OK;
  } catch (const DomainError& e) { g_last_error = e.what(); return PG_ERR_DOMAIN; }
  catch (const Unsupported& e) { g_last_error = e.what(); return PG_ERR_UNSUPPORTED; }
  catch (const CudaError& e) { g_last_error = e.what(); return PG_ERR_CUDA; }
  catch (const NoMem& e) { g_last_error = e.what(); return PG_ERR_NOMEM; }
  catch (const std::exception& e) { g_last_error = e.what(); return PG_ERR_RUNTIME; }
  catch (...) { g_last_error = "unknown error"; return PG_ERR_RUNTIME; }
}

void require(bool c, const std::string& msg) { if (!c) throw DomainError(msg); }
// literal messages: no string is built unless the check fails
void require(bool c, const char* msg) { if (!c) throw DomainError(msg); }

// ---------------------------------------------------------------- device memory
// A small caching pool: freed blocks are kept per engine and reused by size,
// so repeated place/sequence calls do not pay cudaMalloc/cudaFree.
class Pool {
 public:
  ~Pool() { release_all(); }
  void* get(size_t bytes) {
    if (bytes == 0) bytes = 256;
    bytes = (bytes + 255) & ~size_t(255);
    auto it = free_.lower_bound(bytes);
    if (it != free_.end() && it->first <= 2 * bytes) {
      void* p = it->second;
      sizes_[p] = it->first;
      free_.erase(it);
      return p;
    }
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      release_free();
      ck(cudaMalloc(&p, bytes), "cudaMalloc");
    }
    sizes_[p] = bytes;
    return p;
  }
  void put(void* p) {
    if (!p) return;
    auto it = sizes_.find(p);
    if (it == sizes_.end()) return;
    free_.emplace(it->second, p);
    sizes_.erase(it);
  }
  void release_free() {
    for (auto& kv : free_) cudaFree(kv.second);
    free_.clear();
  }
  void release_all() {
    release_free();
    for (auto& kv : sizes_) cudaFree(kv.first);
    sizes_.clear();
  }

 private:
  std::multimap<size_t, void*> free_;
  std::map<void*, size_t> sizes_;
};

template <class T>
struct DBuf {  // device buffer drawn from a pool
  Pool* pool = nullptr;
  T* p = nullptr;
  size_t n = 0;
  DBuf() = default;
  DBuf(Pool* pl, size_t count) : pool(pl), p(static_cast<T*>(pl->get(sizeof(T) * std::max<size_t>(count, 1)))), n(count) {}
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept { *this = std::move(o); }
  DBuf& operator=(DBuf&& o) noexcept {
    if (this != &o) { reset(); pool = o.pool; p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
    return *this;
  }
  ~DBuf() { reset(); }
  void reset() { if (p && pool) pool->put(p); p = nullptr; n = 0; }
};

template <class T>
DBuf<T> upload(Pool* pool, const std::vector<T>& v, cudaStream_t st) {
  DBuf<T> b(pool, v.size());
  if (!v.empty()) ck(cudaMemcpyAsync(b.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, st), "upload");
  return b;
}

// ---------------------------------------------------------------- CDF tables
// thresholds floor(CDF * 2^31); the last class with positive mass gets 2^31
std::vector<uint32_t> cdf_thresholds(const std::vector<double>& w) {
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

}  // namespace

// ---------------------------------------------------------------- handles
struct Species {
  double snv = 0, indel = 0, cna = 0;
  std::vector<double> snv_epoch, indel_epoch;  // optional per-epoch overrides
  uint32_t mutant = 0;
  bool has_rates = false;
};

struct DriverSpec {
  uint32_t chr, pos;  // 0-based chr index, 1-based position
  std::string ref, alt;
  int32_t allele;
};

struct CnaSpec {      // a driver CNA or a passenger CNA candidate
  bool amp;           // amplification (else deletion)
  uint32_t chr, begin, len;   // 0-based chr index, 1-based first position, length
  int32_t allele, src;        // allele ordinal among the covering instances, -1 = random
};

struct DriverEvent {  // one entry of a mutant's driver list, in application order
  int kind;           // 0 SNV/indel, 1 CNA, 2 whole-genome doubling
  DriverSpec sid;
  CnaSpec cna;
};

struct CnaOut {       // an applied CNA/WGD event (for the phylogenetic-forest getters)
  uint32_t node;
  uint8_t type;       // 0 deletion, 1 amplification, 2 WGD
  uint32_t chr, begin, end;   // 1-based inclusive region
  uint32_t allele, src;       // instance acted on / created, source instance
  uint8_t driver;
};

static void philox_host(uint64_t seed, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t out[4]) {
  uint32_t k0 = uint32_t(seed), k1 = uint32_t(seed >> 32);
  for (int i = 0; i < 10; ++i) {
    const uint64_t p0 = uint64_t(0xD2511F53u) * c0, p1 = uint64_t(0xCD9E8D57u) * c2;
    const uint32_t n0 = uint32_t(p1 >> 32) ^ c1 ^ k0, n2 = uint32_t(p0 >> 32) ^ c3 ^ k1;
    c0 = n0; c1 = uint32_t(p1); c2 = n2; c3 = uint32_t(p0);
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}
static inline uint32_t mulhi32(uint32_t a, uint32_t b) { return uint32_t((uint64_t(a) * b) >> 32); }

struct pg_engine {
  int device = 0;
  float index_ms[4] = {0, 0, 0, 0};  // device time of the index build: SBS count, emit; ID count, emit
  cudaStream_t st = nullptr;         // the stream every call of the engine runs on
  cudaStream_t own_st = nullptr;     // the engine's own stream (destroyed with it)
  Pool pool;
  uint32_t n_chr = 0;
  std::vector<uint32_t> chr_len, chr_off;  // chr_off: n_chr + 1 entries
  uint64_t G = 0;
  DBuf<uint32_t> genome, chr_off_d;
  DBuf<uint32_t> nmask;              // unknown bases (N), one bit each; empty when the genome has none
  DBuf<uint32_t> amask;              // positions of the regions to avoid (SBS index), one bit each; or empty
  uint64_t avoid_digest = 0;         // of the regions to avoid (index caches)
  std::string cache_dir;             // index caches (empty: none)
  uint32_t context_sampling = 100, max_rep = 500000;
  // index
  std::vector<uint64_t> ctx_total, id_total;
  std::vector<uint32_t> ctx_len, id_len;
  std::vector<uint64_t> ctx_off, id_off;
  DBuf<uint32_t> ctx_lists, id_lists, ctx_len_d, id_len_d;
  DBuf<uint64_t> ctx_off_d, id_off_d;
  // signatures and exposures
  uint32_t n_sig[2] = {0, 0};
  std::vector<double> sigs[2];
  std::vector<std::string> sig_names[2];   // optional (the causes of the data frames)
  std::map<double, std::vector<double>> expo[2];
  std::map<uint32_t, Species> species;
  std::map<uint32_t, std::vector<DriverEvent>> drivers;   // per mutant, application order
  std::vector<CnaSpec> cna_cands;                          // passenger CNA candidates
  bool infinite_sites = true;
  bool avoid_homozygous_losses = true;
  // device copies of the last placed forest's columns (a forest is immutable:
  // its uid keys them)
  uint64_t fc_uid = 0;
  DBuf<int32_t> fc_parent;
  DBuf<double> fc_birth;
  DBuf<uint32_t> fc_species, fc_div;
  // the caller's reference plus one per live placed/sequencing handle: the
  // engine (its pool and stream) outlives every handle that draws from it
  std::atomic<int> refs{1};

  ~pg_engine() {
    genome.reset(); chr_off_d.reset(); ctx_lists.reset(); id_lists.reset();
    ctx_len_d.reset(); id_len_d.reset(); ctx_off_d.reset(); id_off_d.reset();
    pool.release_all();
    if (own_st) cudaStreamDestroy(own_st);
  }
};

struct pg_forest {
  uint64_t uid = 0;                            // unique per forest (never reused): device-copy cache key
  uint32_t n = 0, n_samples = 0;
  std::vector<int32_t> parent, sample;
  std::vector<double> birth;
  std::vector<uint32_t> species, divisions;
  std::vector<uint32_t> tin, tout;             // Euler intervals (preorder)
  std::vector<std::vector<uint32_t>> leaves;   // per sample: tin of its leaves
};

static void engine_retain(pg_engine* e) { e->refs.fetch_add(1); }
static void engine_release(pg_engine* e) {
  if (e->refs.fetch_sub(1) == 1) {
    cudaSetDevice(e->device);
    delete e;
  }
}

struct pg_placed {
  pg_engine* eng = nullptr;
  uint32_t n_nodes = 0, n_samples = 0;
  std::vector<uint32_t> tin, tout;
  std::vector<int32_t> parent;
  std::vector<std::vector<uint32_t>> leaves;
  uint64_t M = 0;
  DBuf<uint32_t> locus, edge, aux, attempt;
  DBuf<uint8_t> cls, sig, kind, nature;
  DBuf<uint16_t> allele, seq;
  float kernel_ms = 0;
  uint32_t redraw_rounds = 0;   // the round counter after the last redraw round (0: none ran)
  // genotype classes (copy-number state) and allele-instance lineage
  bool has_cna = false;
  uint32_t cn_max = 2, n_classes = 1;
  std::vector<uint32_t> node_class_h;
  std::vector<std::vector<uint32_t>> leaf_cls;   // per sample, parallel to leaves
  // atoms: the coarsest partition of [0, G) on which every class's covering
  // instances are constant; per (atom, class) the covering instances as
  // (offset into inst_list, count)
  std::vector<uint32_t> atom_start_h, atom_icnt_h;
  // host copy of the class segments and each instance's germline allele
  std::vector<uint32_t> seg_off_h, seg_start_h, seg_end_h, seg_ioff_h, seg_icnt_h;
  std::vector<uint16_t> inst_list_h;
  std::vector<uint32_t> chain_off_h;   // instance lineage chains (host copies)
  std::vector<uint16_t> chain_anc_h;
  std::vector<uint64_t> chain_key_h;
  std::vector<uint8_t> inst_root_h;
  DBuf<uint32_t> atom_start, atom_ioff, atom_icnt;
  DBuf<uint32_t> node_class, seg_off, seg_start, seg_end, seg_ioff, seg_icnt, chain_off;
  DBuf<uint16_t> inst_list, chain_anc;
  DBuf<uint64_t> chain_key;
  std::vector<CnaOut> cnas;
  // results of the data-frame getters, built on request (pg_placed_cell_*,
  // pg_placed_bulk_fragmentation) and held until the next request
  std::vector<uint32_t> cm_cell, cm_row, cm_allele;
  std::vector<uint32_t> cc_cell, cc_index;
  std::vector<uint32_t> cf_cell, cf_chr, cf_begin, cf_end, cf_major, cf_minor;
  std::vector<uint32_t> bf_chr, bf_begin, bf_end, bf_major, bf_minor;
  std::vector<double> bf_ratio;
  pg::PlaceOut view() const {
    return {locus.p, edge.p, aux.p, cls.p, sig.p, allele.p, seq.p, kind.p, nature.p, attempt.p};
  }
  pg::GenomeClasses classes_view() const {
    return {n_classes, node_class.p, seg_off.p, seg_start.p, seg_end.p, seg_ioff.p, seg_icnt.p, inst_list.p};
  }
};

struct pg_seq_result {
  pg_engine* eng = nullptr;
  uint32_t n_samples = 0;
  uint64_t M = 0, n_reads = 0;
  uint32_t tile_size = 0;      // the tile size the call used (automatic or given)
  DBuf<uint32_t> alt, depth;
  float kernel_ms = 0;
  // observed rows (built on the first request)
  bool active_done = false;
  uint32_t n_active = 0;
  DBuf<uint32_t> a_index, a_alt, a_depth;
  // what the result data frame needs: the forest sample of each sequenced
  // sample (-1 the normal one) and whether normal cells carry the
  // preneoplastic mutations
  std::vector<int32_t> sample_src;
  bool pre_in_normal = false;
  // the result data frame (pg_seq_result_frame)
  uint64_t f_rows = 0;
  std::vector<uint32_t> f_chr, f_pos;
  std::vector<char> f_ref, f_alt;            // PG_SID_CHARS per row
  std::vector<uint64_t> f_cause_off;
  std::vector<char> f_causes;
  std::vector<uint8_t> f_classes;
  std::vector<int32_t> f_occ, f_cov;         // [sample][row]
  std::vector<double> f_vaf;
};

namespace {

struct Timer {
  cudaEvent_t a = nullptr, b = nullptr;
  cudaStream_t st;
  explicit Timer(cudaStream_t s) : st(s) {
    ck(cudaEventCreate(&a), "event"); ck(cudaEventCreate(&b), "event");
    ck(cudaEventRecord(a, st), "event");
  }
  float stop() {
    ck(cudaEventRecord(b, st), "event");
    ck(cudaEventSynchronize(b), "event");
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
  }
  ~Timer() { if (a) cudaEventDestroy(a); if (b) cudaEventDestroy(b); }
};

void select_device(const pg_engine* e) { ck(cudaSetDevice(e->device), "cudaSetDevice"); }

// fingerprint of an engine's genome: lengths and 4096 words at an even
// stride, FNV-1a (64 bit)
uint64_t fnv1a(uint64_t h, const void* p, size_t k) {
  const uint8_t* c = static_cast<const uint8_t*>(p);
  for (size_t i = 0; i < k; ++i) { h ^= c[i]; h *= 1099511628211ull; }
  return h;
}

uint64_t genome_fingerprint(const pg_engine* e) {
  uint64_t h = 1469598103934665603ull;
  h = fnv1a(h, &e->G, sizeof(e->G));
  h = fnv1a(h, e->chr_len.data(), sizeof(uint32_t) * e->chr_len.size());
  const uint64_t words = (e->G + 15) / 16;
  if (words) {
    const uint64_t k = std::min<uint64_t>(4096, words), stride = words / k;
    std::vector<uint32_t> smp(k);
    ck(cudaMemcpy2D(smp.data(), sizeof(uint32_t), e->genome.p, sizeof(uint32_t) * stride, sizeof(uint32_t), k,
                    cudaMemcpyDeviceToHost), "genome fingerprint");
    h = fnv1a(h, smp.data(), sizeof(uint32_t) * k);
  }
  return h;
}

// ---- index caches: "PGIX", version, which, genome fingerprint, parameter,
// regions digest, class count, per class total and stored count, the lists
constexpr uint32_t INDEX_CACHE_VERSION = 1;

std::string index_cache_path(const pg_engine* e, int which) {
  return e->cache_dir + (which == 0 ? "/context_index_" + std::to_string(e->context_sampling) + ".pgcif"
                                    : "/rs_index_" + std::to_string(e->max_rep) + ".pgrsif");
}

struct IndexTables {
  std::vector<uint64_t> total;
  std::vector<uint32_t> len;
  std::vector<uint32_t> lists;   // host copy (caches only)
};

void save_index_cache(const pg_engine* e, int which, uint64_t fp, const IndexTables& t) {
  std::ofstream f(index_cache_path(e, which), std::ios::binary | std::ios::trunc);
  if (!f) throw std::runtime_error("cannot write the index cache " + index_cache_path(e, which));
  auto put = [&](const void* p, size_t k) { f.write(static_cast<const char*>(p), std::streamsize(k)); };
  const uint32_t v = INDEX_CACHE_VERSION, w = uint32_t(which), prm = which == 0 ? e->context_sampling : e->max_rep,
                 nc = uint32_t(t.total.size());
  const uint64_t dg = which == 0 ? e->avoid_digest : 0, nl = t.lists.size();
  put("PGIX", 4); put(&v, 4); put(&w, 4); put(&fp, 8); put(&prm, 4); put(&dg, 8); put(&nc, 4);
  put(t.total.data(), 8 * nc); put(t.len.data(), 4 * nc); put(&nl, 8); put(t.lists.data(), 4 * nl);
  put("XIGP", 4);
  if (!f) throw std::runtime_error("cannot write the index cache " + index_cache_path(e, which));
}

bool load_index_cache(const pg_engine* e, int which, uint64_t fp, int NC, IndexTables& t) {
  const std::string path = index_cache_path(e, which);
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  auto get = [&](void* p, size_t k) {
    f.read(static_cast<char*>(p), std::streamsize(k));
    if (!f) throw DomainError("the index cache " + path + " is truncated");
  };
  char magic[4];
  uint32_t v = 0, w = 0, prm = 0, nc = 0;
  uint64_t fp2 = 0, dg = 0, nl = 0;
  get(magic, 4);
  if (std::memcmp(magic, "PGIX", 4) != 0) throw DomainError(path + " is not an index cache");
  get(&v, 4);
  if (v != INDEX_CACHE_VERSION)
    throw DomainError("the index cache " + path + " has format version " + std::to_string(v) +
                      ", this library reads version " + std::to_string(INDEX_CACHE_VERSION));
  get(&w, 4); get(&fp2, 8); get(&prm, 4); get(&dg, 8); get(&nc, 4);
  if (w != uint32_t(which) || nc != uint32_t(NC) || prm != (which == 0 ? e->context_sampling : e->max_rep))
    throw DomainError("the index cache " + path + " holds another index");
  if (fp2 != fp) throw DomainError("the index cache " + path + " was built for another reference genome");
  if (which == 0 && dg != e->avoid_digest)
    throw DomainError("the index cache " + path + " was built with other regions to avoid");
  t.total.resize(nc); t.len.resize(nc);
  get(t.total.data(), 8 * nc); get(t.len.data(), 4 * nc); get(&nl, 8);
  uint64_t want = 0;
  for (uint32_t k : t.len) want += k;
  if (nl != want || nl > (uint64_t(1) << 34)) throw DomainError("the index cache " + path + " is inconsistent");
  t.lists.resize(nl);
  get(t.lists.data(), 4 * nl);
  get(magic, 4);
  if (std::memcmp(magic, "XIGP", 4) != 0) throw DomainError("the index cache " + path + " is inconsistent");
  return true;
}

void build_indices(pg_engine* e) {
  const uint32_t ntiles = pg::index_num_tiles(e->G);
  const uint64_t fp = e->cache_dir.empty() ? 0 : genome_fingerprint(e);
  for (int which = 0; which < 2; ++which) {
    const int NC = pg::index_num_classes(which);
    IndexTables t;
    std::vector<uint64_t> off(NC + 1, 0);
    DBuf<uint32_t> lists;
    if (!e->cache_dir.empty() && load_index_cache(e, which, fp, NC, t)) {
      for (int k = 0; k < NC; ++k) off[k + 1] = off[k] + t.len[k];
      lists = upload(&e->pool, t.lists, e->st);
    } else {
      DBuf<uint32_t> cnt(&e->pool, uint64_t(NC) * ntiles);
      DBuf<uint32_t> part(&e->pool, pg::scan_part_elems(ntiles, NC));
      DBuf<uint32_t> tot(&e->pool, NC);
      const uint32_t* am = which == 0 ? e->amask.p : nullptr;
      Timer t_count(e->st);
      pg::index_count(which, e->genome.p, e->nmask.p, am, e->G, e->chr_off_d.p, int(e->n_chr), cnt.p, part.p, tot.p,
                      e->st);
      e->index_ms[2 * which] = t_count.stop();
      std::vector<uint32_t> tot_h(NC);
      ck(cudaMemcpyAsync(tot_h.data(), tot.p, sizeof(uint32_t) * NC, cudaMemcpyDeviceToHost, e->st), "index totals");
      ck(cudaStreamSynchronize(e->st), "index count");
      std::vector<uint32_t> stride(NC);
      t.total.assign(NC, 0); t.len.assign(NC, 0);
      for (int k = 0; k < NC; ++k) {
        t.total[k] = tot_h[k];
        uint64_t sd;
        if (which == 0) sd = e->context_sampling;
        else sd = std::max<uint64_t>(1, (uint64_t(tot_h[k]) + e->max_rep - 1) / e->max_rep);
        stride[k] = uint32_t(sd);
        t.len[k] = uint32_t((uint64_t(tot_h[k]) + sd - 1) / sd);
        off[k + 1] = off[k] + t.len[k];
      }
      auto stride_d = upload(&e->pool, stride, e->st);
      auto len_tmp = upload(&e->pool, t.len, e->st);
      std::vector<uint64_t> off_k(off.begin(), off.begin() + NC);
      auto off_tmp = upload(&e->pool, off_k, e->st);
      lists = DBuf<uint32_t>(&e->pool, off[NC]);
      Timer t_emit(e->st);
      const bool every = std::all_of(stride.begin(), stride.end(), [](uint32_t x) { return x == 1u; });
      pg::index_emit(which, e->genome.p, e->nmask.p, am, e->G, e->chr_off_d.p, int(e->n_chr), cnt.p, stride_d.p,
                     off_tmp.p, len_tmp.p, lists.p, every, e->st);
      e->index_ms[2 * which + 1] = t_emit.stop();
      ck(cudaStreamSynchronize(e->st), "index emit");
      ck(cudaGetLastError(), "index kernels");
      if (!e->cache_dir.empty()) {
        t.lists.resize(off[NC]);
        if (off[NC]) ck(cudaMemcpy(t.lists.data(), lists.p, 4 * off[NC], cudaMemcpyDeviceToHost), "index cache");
        save_index_cache(e, which, fp, t);
      }
    }
    std::vector<uint64_t> off_k(off.begin(), off.begin() + NC);
    auto len_d = upload(&e->pool, t.len, e->st);
    auto off_d = upload(&e->pool, off_k, e->st);
    ck(cudaStreamSynchronize(e->st), "index upload");
    if (which == 0) {
      e->ctx_total = t.total; e->ctx_len = t.len; e->ctx_off = off_k;
      e->ctx_lists = std::move(lists); e->ctx_len_d = std::move(len_d); e->ctx_off_d = std::move(off_d);
    } else {
      e->id_total = t.total; e->id_len = t.len; e->id_off = off_k;
      e->id_lists = std::move(lists); e->id_len_d = std::move(len_d); e->id_off_d = std::move(off_d);
    }
  }
}

uint32_t code_of(char c) {
  switch (c) {
    case 'A': case 'a': return 0;
    case 'C': case 'c': return 1;
    case 'G': case 'g': return 2;
    case 'T': case 't': return 3;
  }
  throw DomainError(std::string("invalid base '") + c + "'");
}

// Euler intervals of the forest (preorder index, subtree end)
void euler(pg_forest& f) {
  // children in CSR form, each node's in increasing index order
  std::vector<uint32_t> koff(f.n + 1, 0), kids(f.n), fill;
  std::vector<uint32_t> roots;
  for (uint32_t v = 0; v < f.n; ++v) {
    if (f.parent[v] < 0) roots.push_back(v); else ++koff[f.parent[v] + 1];
  }
  for (uint32_t v = 0; v < f.n; ++v) koff[v + 1] += koff[v];
  fill.assign(koff.begin(), koff.end() - 1);
  for (uint32_t v = 0; v < f.n; ++v)
    if (f.parent[v] >= 0) kids[fill[f.parent[v]]++] = v;
  f.tin.assign(f.n, 0); f.tout.assign(f.n, 0);
  uint32_t clock = 0;
  std::vector<std::pair<uint32_t, uint32_t>> stack;  // node, next child position
  for (uint32_t r : roots) {
    stack.push_back({r, koff[r]});
    f.tin[r] = clock++;
    while (!stack.empty()) {
      auto& top = stack.back();
      if (top.second < koff[top.first + 1]) {
        const uint32_t c = kids[top.second++];
        f.tin[c] = clock++;
        stack.push_back({c, koff[c]});
      } else {
        f.tout[top.first] = clock;
        stack.pop_back();
      }
    }
  }
  f.leaves.assign(f.n_samples, {});
  for (uint32_t v = 0; v < f.n; ++v) {
    if (koff[v] == koff[v + 1] && f.sample[v] >= 0) f.leaves[f.sample[v]].push_back(f.tin[v]);
  }
}

}  // namespace

// ====================================================================== C-ABI
extern "C" {

const char* pg_last_error(void) { return g_last_error.c_str(); }
const char* pg_version(void) { return "process_gb300 0.1 (sm_103a)"; }

pg_status pg_device_count(int* n) {
  return guarded([&] {
    require(n != nullptr, "n is NULL");
    int c = 0;
    cudaError_t e = cudaGetDeviceCount(&c);
    if (e != cudaSuccess) { cudaGetLastError(); c = 0; }
    *n = c;
  });
}

pg_status pg_engine_create(const pg_genome_desc* gd, pg_engine** out) {
  return guarded([&] {
    require(gd && out, "NULL argument");
    require(gd->n_chr > 0 && gd->chr_lengths, "the genome needs at least one chromosome");
    require(gd->context_sampling >= 1, "context_sampling must be positive");
    require(gd->max_repetition_storage >= 1, "max_repetition_storage must be positive");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
      cudaGetLastError();
      throw CudaError("no CUDA device: the GB300 kernels of process_gb300 need a GPU");
    }
    auto e = std::make_unique<pg_engine>();
    ck(cudaGetDevice(&e->device), "cudaGetDevice");
    ck(cudaStreamCreateWithFlags(&e->own_st, cudaStreamNonBlocking), "stream");
    e->st = e->own_st;
    e->n_chr = gd->n_chr;
    e->chr_len.assign(gd->chr_lengths, gd->chr_lengths + gd->n_chr);
    e->chr_off.assign(gd->n_chr + 1, 0);
    uint64_t G = 0;
    for (uint32_t c = 0; c < gd->n_chr; ++c) {
      require(e->chr_len[c] > 0, "chromosome lengths must be positive");
      e->chr_off[c] = uint32_t(G);
      G += e->chr_len[c];
      require(G < (uint64_t(1) << 32) - 1024, "genome longer than the u32 position space");
    }
    e->chr_off[gd->n_chr] = uint32_t(G);
    e->G = G;
    e->context_sampling = gd->context_sampling;
    e->max_rep = gd->max_repetition_storage;
    e->chr_off_d = upload(&e->pool, e->chr_off, e->st);
    const uint64_t nwords = (G + 15) / 16;
    e->genome = DBuf<uint32_t>(&e->pool, nwords + 4);
    ck(cudaMemsetAsync(e->genome.p, 0, sizeof(uint32_t) * (nwords + 4), e->st), "memset");
    if (gd->bases) {
      DBuf<uint8_t> codes(&e->pool, G);
      ck(cudaMemcpyAsync(codes.p, gd->bases, G, cudaMemcpyHostToDevice, e->st), "genome upload");
      pg::genome_pack(e->genome.p, codes.p, G, e->st);
      // codes above 3 (N and the other ambiguity codes) are unknown bases
      e->nmask = DBuf<uint32_t>(&e->pool, (G + 31) / 32 + 1);
      DBuf<uint32_t> any(&e->pool, 1);
      ck(cudaMemsetAsync(any.p, 0, sizeof(uint32_t), e->st), "memset");
      pg::genome_nmask(codes.p, G, e->nmask.p, any.p, e->st);
      uint32_t any_h = 0;
      ck(cudaMemcpyAsync(&any_h, any.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, e->st), "unknown bases");
      ck(cudaStreamSynchronize(e->st), "genome pack");
      if (!any_h) e->nmask.reset();
    } else {
      require(gd->synthetic_gc >= 0 && gd->synthetic_gc <= 1, "synthetic_gc must be in [0,1]");
      pg::genome_synth(e->genome.p, G, gd->synthetic_seed, gd->synthetic_gc, e->st);
    }
    ck(cudaGetLastError(), "genome kernels");
    // regions to avoid (SBS context index), as a bit per position
    if (gd->n_avoid) {
      require(gd->avoid_chr && gd->avoid_begin && gd->avoid_len, "NULL regions to avoid");
      std::vector<std::pair<uint32_t, uint32_t>> reg;
      for (uint32_t i = 0; i < gd->n_avoid; ++i) {
        const uint32_t c = gd->avoid_chr[i], b = gd->avoid_begin[i], l = gd->avoid_len[i];
        require(c < e->n_chr, "region to avoid on an unknown chromosome");
        require(b >= 1 && l >= 1 && uint64_t(b) - 1 + l <= e->chr_len[c], "region to avoid outside its chromosome");
        reg.push_back({e->chr_off[c] + b - 1, e->chr_off[c] + b - 1 + l});
      }
      std::vector<uint32_t> pos;     // every avoided position once, ascending
      for (auto [b, en] : reg)
        for (uint32_t q = b; q < en; ++q) pos.push_back(q);
      std::sort(pos.begin(), pos.end());
      pos.erase(std::unique(pos.begin(), pos.end()), pos.end());
      e->avoid_digest = fnv1a(1469598103934665603ull, pos.data(), sizeof(uint32_t) * pos.size());
      e->amask = DBuf<uint32_t>(&e->pool, (G + 31) / 32 + 1);
      ck(cudaMemsetAsync(e->amask.p, 0, sizeof(uint32_t) * ((G + 31) / 32 + 1), e->st), "memset");
      auto pos_d = upload(&e->pool, pos, e->st);
      pg::genome_avoid_mask(pos_d.p, pos.size(), e->amask.p, e->st);
      ck(cudaStreamSynchronize(e->st), "regions to avoid");
    }
    if (gd->index_cache_dir && gd->index_cache_dir[0]) {
      e->cache_dir = gd->index_cache_dir;
      std::error_code ec;
      std::filesystem::create_directories(e->cache_dir, ec);
      require(std::filesystem::is_directory(e->cache_dir), "index cache directory " + e->cache_dir + " is not a directory");
    }
    build_indices(e.get());
    *out = e.release();
  });
}

pg_status pg_engine_set_stream(pg_engine* e, void* stream) {
  return guarded([&] {
    require(e != nullptr, "NULL engine");
    select_device(e);
    ck(cudaStreamSynchronize(e->st), "stream switch");
    e->st = stream ? static_cast<cudaStream_t>(stream) : e->own_st;
  });
}

pg_status pg_index_counts_noalloc(int which, const uint32_t* genome_words, uint64_t genome_len,
                                  const uint32_t* chr_off, uint32_t n_chr, uint64_t* class_totals, void* stream) {
  return guarded([&] {
    require(which == 0 || which == 1, "which must be 0 (SBS contexts) or 1 (ID classes)");
    require(genome_words && chr_off && class_totals, "NULL device pointer");
    require(n_chr >= 1, "at least one chromosome");
    const char* msg = pg::index_counts_noalloc(which, genome_words, genome_len, chr_off, int(n_chr), class_totals,
                                               static_cast<cudaStream_t>(stream));
    if (msg) {
      if (genome_len == 0 || genome_len > uint64_t(pg::NOALLOC_MAX_TILES) * 1024) throw DomainError(msg);
      throw CudaError(msg);
    }
  });
}

pg_status pg_launch_count(uint64_t* n) {
  return guarded([&] { require(n != nullptr, "NULL argument"); *n = g_launches.load(); });
}

pg_status pg_engine_destroy(pg_engine* eng) {
  return guarded([&] { if (eng) engine_release(eng); });
}

pg_status pg_engine_genome_info(const pg_engine* e, uint64_t* total_len, uint64_t* ctx_total, uint64_t* id_total,
                                uint32_t* ctx_stored, uint32_t* id_stored) {
  return guarded([&] {
    require(e != nullptr, "NULL engine");
    if (total_len) *total_len = e->G;
    if (ctx_total) std::copy(e->ctx_total.begin(), e->ctx_total.end(), ctx_total);
    if (id_total) std::copy(e->id_total.begin(), e->id_total.end(), id_total);
    if (ctx_stored) std::copy(e->ctx_len.begin(), e->ctx_len.end(), ctx_stored);
    if (id_stored) std::copy(e->id_len.begin(), e->id_len.end(), id_stored);
  });
}

pg_status pg_engine_read_genome(const pg_engine* e, uint64_t start, uint64_t n, uint8_t* out) {
  return guarded([&] {
    require(e && out, "NULL argument");
    require(start + n <= e->G, "range outside the genome");
    select_device(e);
    const uint64_t w0 = start / 16, w1 = (start + n + 15) / 16;
    std::vector<uint32_t> words(w1 - w0);
    if (!words.empty())
      ck(cudaMemcpy(words.data(), e->genome.p + w0, sizeof(uint32_t) * words.size(), cudaMemcpyDeviceToHost), "read");
    // unknown bases read as 4
    const uint64_t m0 = start / 32, m1 = (start + n + 31) / 32;
    std::vector<uint32_t> mask(e->nmask.p ? m1 - m0 : 0);
    if (!mask.empty())
      ck(cudaMemcpy(mask.data(), e->nmask.p + m0, sizeof(uint32_t) * mask.size(), cudaMemcpyDeviceToHost), "read");
    for (uint64_t i = 0; i < n; ++i) {
      const uint64_t p = start + i;
      const bool unknown = !mask.empty() && ((mask[p / 32 - m0] >> (p % 32)) & 1u);
      out[i] = unknown ? uint8_t(4) : uint8_t((words[p / 16 - w0] >> (2 * (p % 16))) & 3u);
    }
  });
}

pg_status pg_engine_gather_bases(const pg_engine* e, uint64_t n, const uint32_t* pos, uint8_t* out) {
  return guarded([&] {
    require(e && (n == 0 || (pos && out)), "NULL argument");
    if (n == 0) return;
    select_device(e);
    Pool* P = const_cast<Pool*>(&e->pool);
    DBuf<uint32_t> pd(P, n);
    DBuf<uint8_t> od(P, n);
    ck(cudaMemcpyAsync(pd.p, pos, 4 * n, cudaMemcpyHostToDevice, e->st), "upload");
    pg::genome_gather(e->genome.p, e->nmask.p, e->G, pd.p, n, od.p, e->st);
    ck(cudaMemcpyAsync(out, od.p, n, cudaMemcpyDeviceToHost, e->st), "download");
    ck(cudaStreamSynchronize(e->st), "gather");
  });
}

pg_status pg_engine_read_index(const pg_engine* e, int which, uint32_t cls, uint32_t* out, uint32_t capacity,
                               uint32_t* n_out) {
  return guarded([&] {
    require(e && n_out, "NULL argument");
    require(which == 0 || which == 1, "which must be 0 (SBS) or 1 (ID)");
    const auto& len = which == 0 ? e->ctx_len : e->id_len;
    const auto& off = which == 0 ? e->ctx_off : e->id_off;
    require(cls < len.size(), "class out of range");
    *n_out = len[cls];
    if (out && len[cls]) {
      require(capacity >= len[cls], "output capacity too small");
      select_device(e);
      const uint32_t* base = (which == 0 ? e->ctx_lists.p : e->id_lists.p) + off[cls];
      ck(cudaMemcpy(out, base, sizeof(uint32_t) * len[cls], cudaMemcpyDeviceToHost), "read index");
    }
  });
}

pg_status pg_engine_set_signatures(pg_engine* e, int type, uint32_t n_sigs, const double* probs) {
  return guarded([&] {
    require(e && probs, "NULL argument");
    require(type == 0 || type == 1, "type must be 0 (SBS) or 1 (ID)");
    require(n_sigs > 0 && n_sigs < 255, "between 1 and 254 signatures");
    const uint32_t NC = type == 0 ? 96 : 83;
    for (uint64_t i = 0; i < uint64_t(n_sigs) * NC; ++i)
      require(probs[i] >= 0 && std::isfinite(probs[i]), "signature probabilities must be non-negative");
    e->n_sig[type] = n_sigs;
    e->sigs[type].assign(probs, probs + uint64_t(n_sigs) * NC);
    e->expo[type].clear();
    e->sig_names[type].clear();
  });
}

pg_status pg_engine_add_exposure(pg_engine* e, int type, double time, const double* coeffs) {
  return guarded([&] {
    require(e && coeffs, "NULL argument");
    require(type == 0 || type == 1, "type must be 0 (SBS) or 1 (ID)");
    require(e->n_sig[type] > 0, "set the signatures before adding exposures");
    require(std::isfinite(time), "exposure time must be finite");
    double tot = 0;
    for (uint32_t i = 0; i < e->n_sig[type]; ++i) {
      require(coeffs[i] >= 0, "exposure coefficients must be non-negative");
      tot += coeffs[i];
    }
    require(tot > 0, "exposure coefficients must not all be zero");
    e->expo[type][time] = std::vector<double>(coeffs, coeffs + e->n_sig[type]);
  });
}

pg_status pg_engine_set_species_rates(pg_engine* e, uint32_t sp, double snv, double indel, double cna) {
  return guarded([&] {
    require(e != nullptr, "NULL engine");
    require(snv >= 0, std::to_string(snv) + ": SNV rates must be non-negative");
    require(indel >= 0, std::to_string(indel) + ": indel rates must be non-negative");
    require(cna >= 0, std::to_string(cna) + ": CNA rates must be non-negative");
    auto& s = e->species[sp];
    s.snv = snv; s.indel = indel; s.cna = cna; s.has_rates = true;
  });
}

pg_status pg_engine_set_species_epoch_rates(pg_engine* e, uint32_t sp, uint32_t n_epochs, const double* snv,
                                            const double* indel) {
  return guarded([&] {
    require(e && snv && indel, "NULL argument");
    require(n_epochs >= 1 && n_epochs <= pg::MAX_EPOCHS, "between 1 and 16 epochs");
    for (uint32_t i = 0; i < n_epochs; ++i) require(snv[i] >= 0 && indel[i] >= 0, "rates must be non-negative");
    auto& s = e->species[sp];
    s.snv_epoch.assign(snv, snv + n_epochs);
    s.indel_epoch.assign(indel, indel + n_epochs);
    s.has_rates = true;
  });
}

pg_status pg_engine_set_species_mutant(pg_engine* e, uint32_t sp, uint32_t mutant) {
  return guarded([&] { require(e != nullptr, "NULL engine"); e->species[sp].mutant = mutant; });
}

pg_status pg_engine_add_driver_sid(pg_engine* e, uint32_t mutant, uint32_t chr, uint32_t pos, const char* ref,
                                   const char* alt, int32_t allele) {
  return guarded([&] {
    require(e && ref && alt, "NULL argument");
    require(chr < e->n_chr, "unknown chromosome");
    std::string r(ref), a(alt);
    require(!r.empty() && !a.empty(), "empty ref/alt");
    require(pos >= 1 && pos + r.size() - 1 <= e->chr_len[chr], "mutation outside the chromosome");
    require(r.size() == 1 || a.size() == 1, "indels share exactly their first base");
    if (r.size() != 1 || a.size() != 1) require(r[0] == a[0], "indel ref and alt must share their first base");
    require(r.size() <= 6 && a.size() <= 6, "driver indels up to 5 bases");
    for (char c : r) code_of(c);
    for (char c : a) code_of(c);
    require(allele >= -1 && allele <= 1, "allele must be 0, 1 or random (-1)");
    DriverEvent ev{};
    ev.kind = 0;
    ev.sid = {chr, pos, r, a, allele};
    e->drivers[mutant].push_back(ev);
  });
}

pg_status pg_engine_add_driver_cna(pg_engine* e, uint32_t mutant, int type_amplification, uint32_t chr,
                                   uint32_t begin, uint32_t length, int32_t allele, int32_t src_allele) {
  return guarded([&] {
    require(e != nullptr, "NULL engine");
    require(chr < e->n_chr, "unknown chromosome");
    require(begin >= 1 && length >= 1 && uint64_t(begin) + length - 1 <= e->chr_len[chr],
            "the CNA region must lie inside the chromosome");
    require(allele >= -1 && src_allele >= -1, "alleles are ordinals (>= 0) or random (-1)");
    DriverEvent ev{};
    ev.kind = 1;
    ev.cna = {type_amplification != 0, chr, begin, length, allele, src_allele};
    e->drivers[mutant].push_back(ev);
  });
}

pg_status pg_engine_add_driver_wgd(pg_engine* e, uint32_t mutant) {
  return guarded([&] {
    require(e != nullptr, "NULL engine");
    DriverEvent ev{};
    ev.kind = 2;
    e->drivers[mutant].push_back(ev);
  });
}

pg_status pg_engine_add_passenger_cna(pg_engine* e, uint32_t chr, uint32_t begin, uint32_t length,
                                      int type_amplification) {
  return guarded([&] {
    require(e != nullptr, "NULL engine");
    require(chr < e->n_chr, "unknown chromosome");
    require(begin >= 1 && length >= 1 && uint64_t(begin) + length - 1 <= e->chr_len[chr],
            "the CNA region must lie inside the chromosome");
    e->cna_cands.push_back({type_amplification != 0, chr, begin, length, -1, -1});
  });
}

pg_status pg_engine_set_avoid_homozygous_losses(pg_engine* e, int on) {
  return guarded([&] { require(e != nullptr, "NULL engine"); e->avoid_homozygous_losses = on != 0; });
}

pg_status pg_engine_set_infinite_sites(pg_engine* e, int on) {
  return guarded([&] { require(e != nullptr, "NULL engine"); e->infinite_sites = on != 0; });
}
pg_status pg_engine_get_infinite_sites(const pg_engine* e, int* on) {
  return guarded([&] { require(e && on, "NULL argument"); *on = e->infinite_sites ? 1 : 0; });
}

pg_status pg_forest_create(uint32_t n, const int32_t* parent, const double* birth, const uint32_t* species,
                           const int32_t* sample, const uint32_t* divisions, uint32_t n_samples, pg_forest** out) {
  return guarded([&] {
    require(out && parent && birth && species && sample, "NULL argument");
    require(n > 0, "empty forest");
    require(n < (1u << 30), "forest too large");
    static std::atomic<uint64_t> next_uid{0};
    auto f = std::make_unique<pg_forest>();
    f->uid = ++next_uid;
    f->n = n; f->n_samples = n_samples;
    f->parent.assign(parent, parent + n);
    f->birth.assign(birth, birth + n);
    f->species.assign(species, species + n);
    f->sample.assign(sample, sample + n);
    f->divisions.assign(n, 1);
    if (divisions) f->divisions.assign(divisions, divisions + n);
    for (uint32_t v = 0; v < n; ++v) {
      require(f->parent[v] < int32_t(v) && f->parent[v] >= -1, "nodes must be in topological order (parent < node)");
      require(std::isfinite(f->birth[v]), "birth times must be finite");
      require(f->divisions[v] >= 1 && f->divisions[v] <= 1000000, "divisions per edge in [1, 1e6]");
      require(f->sample[v] >= -1 && f->sample[v] < int32_t(n_samples), "sample index out of range");
      if (f->parent[v] >= 0) require(f->birth[v] >= f->birth[f->parent[v]], "a cell is born after its parent");
    }
    euler(*f);
    *out = f.release();
  });
}

pg_status pg_forest_destroy(pg_forest* f) {
  return guarded([&] { delete f; });
}

pg_status pg_place_mutations(pg_engine* e, const pg_forest* f, uint32_t n_pre_snv, uint32_t pre_sbs_sig,
                             uint32_t n_pre_id, uint32_t pre_id_sig, uint64_t seed, pg_placed** out) {
  return guarded([&] {
    require(e && f && out, "NULL argument");
    select_device(e);
    cudaStream_t st = e->st;
    // ---- epochs: union of exposure change times
    std::vector<double> times;
    for (int ty = 0; ty < 2; ++ty) for (auto& kv : e->expo[ty]) times.push_back(kv.first);
    std::sort(times.begin(), times.end());
    times.erase(std::unique(times.begin(), times.end()), times.end());
    if (times.empty()) times.push_back(0.0);
    require(times.size() <= pg::MAX_EPOCHS, "at most 16 exposure epochs");
    const uint32_t E = uint32_t(times.size());
    // ---- species
    uint32_t S = 0;
    for (uint32_t v = 0; v < f->n; ++v) S = std::max(S, f->species[v] + 1);
    std::vector<double> snv_rate(uint64_t(S) * E, 0.0), id_rate(uint64_t(S) * E, 0.0);
    bool need_sbs = n_pre_snv > 0, need_id = n_pre_id > 0;
    std::vector<uint8_t> used(S, 0);
    for (uint32_t v = 0; v < f->n; ++v) used[f->species[v]] = 1;
    for (uint32_t s = 0; s < S; ++s) {
      if (!used[s]) continue;
      auto it = e->species.find(s);
      require(it != e->species.end() && it->second.has_rates,
              "species " + std::to_string(s) + " has no passenger rates: add its mutant first");
      const Species& sp = it->second;
      for (uint32_t ep = 0; ep < E; ++ep) {
        double rs = sp.snv, ri = sp.indel;
        if (!sp.snv_epoch.empty()) {
          require(sp.snv_epoch.size() == E, "per-epoch rates must cover every exposure epoch");
          rs = sp.snv_epoch[ep]; ri = sp.indel_epoch[ep];
        }
        snv_rate[uint64_t(s) * E + ep] = rs;
        id_rate[uint64_t(s) * E + ep] = ri;
        need_sbs = need_sbs || rs > 0;
        need_id = need_id || ri > 0;
      }
    }
    // ---- CDF tables
    std::vector<uint32_t> sig_cdf[2], expo_cdf[2];
    for (int ty = 0; ty < 2; ++ty) {
      const uint32_t NC = ty == 0 ? 96 : 83;
      const bool need = ty == 0 ? need_sbs : need_id;
      const uint32_t ns = std::max<uint32_t>(e->n_sig[ty], 1);
      if (need) {
        require(e->n_sig[ty] > 0, ty == 0 ? "no SBS signatures set" : "no ID signatures set");
      }
      std::vector<uint8_t> usable(ns, 0);
      sig_cdf[ty].assign(uint64_t(ns) * NC, 0);
      for (uint32_t s = 0; s < e->n_sig[ty]; ++s) {
        std::vector<double> w(NC);
        for (uint32_t k = 0; k < NC; ++k) {
          const uint32_t list = ty == 0 ? uint32_t(pg::sbs_class_context(int(k))) : k;
          const uint32_t len = ty == 0 ? e->ctx_len[list] : e->id_len[list];
          w[k] = len > 0 ? e->sigs[ty][uint64_t(s) * NC + k] : 0.0;
          if (w[k] > 0) usable[s] = 1;
        }
        auto thr = cdf_thresholds(w);
        std::copy(thr.begin(), thr.end(), sig_cdf[ty].begin() + uint64_t(s) * NC);
      }
      expo_cdf[ty].assign(uint64_t(E + 1) * ns, 0);
      for (uint32_t ep = 0; ep < E; ++ep) {
        std::vector<double> w(ns, 0.0);
        if (!e->expo[ty].empty()) {
          auto it = e->expo[ty].upper_bound(times[ep]);
          if (it == e->expo[ty].begin()) w = it->second; else w = std::prev(it)->second;
        } else if (need && e->n_sig[ty] > 0) {
          bool used_type = false;
          for (uint32_t s = 0; s < S; ++s) if (used[s]) used_type = used_type || (ty == 0 ? snv_rate[uint64_t(s) * E + ep] > 0 : id_rate[uint64_t(s) * E + ep] > 0);
          require(!used_type, ty == 0 ? "no SBS exposure: add an exposure before placing mutations"
                                      : "no ID exposure: add an exposure before placing mutations");
        }
        for (uint32_t s = 0; s < ns && s < w.size(); ++s) {
          if (w[s] > 0 && !usable[s]) throw DomainError("signature " + std::to_string(s) +
                                                       " has no class with indexed positions");
        }
        auto thr = cdf_thresholds(w);
        std::copy(thr.begin(), thr.end(), expo_cdf[ty].begin() + uint64_t(ep) * ns);
      }
      const uint32_t pre_sig = ty == 0 ? pre_sbs_sig : pre_id_sig;
      const uint32_t n_pre = ty == 0 ? n_pre_snv : n_pre_id;
      if (n_pre > 0) {
        require(pre_sig < e->n_sig[ty], "unknown preneoplastic signature");
        require(usable[pre_sig], "the preneoplastic signature has no class with indexed positions");
        std::vector<double> w(ns, 0.0);
        w[pre_sig] = 1.0;
        auto thr = cdf_thresholds(w);
        std::copy(thr.begin(), thr.end(), expo_cdf[ty].begin() + uint64_t(E) * ns);
      }
    }
    // ---- device tables
    Pool* P = &e->pool;
    if (e->fc_uid != f->uid) {      // the last placed forest's columns stay on the device
      e->fc_uid = 0;
      e->fc_parent = upload(P, f->parent, st);
      e->fc_birth = upload(P, f->birth, st);
      e->fc_species = upload(P, f->species, st);
      e->fc_div = upload(P, f->divisions, st);
      e->fc_uid = f->uid;
    }
    auto times_d = upload(P, times, st);
    auto snv_d = upload(P, snv_rate, st);
    auto id_d = upload(P, id_rate, st);
    auto sbs_sig_d = upload(P, sig_cdf[0], st);
    auto id_sig_d = upload(P, sig_cdf[1], st);
    auto sbs_expo_d = upload(P, expo_cdf[0], st);
    auto id_expo_d = upload(P, expo_cdf[1], st);
    std::vector<double> cna_rate(S, 0.0);
    bool passenger_cnas = false;
    for (uint32_t s2 = 0; s2 < S; ++s2) {
      auto it = e->species.find(s2);
      if (used[s2] && it != e->species.end()) cna_rate[s2] = it->second.cna;
      passenger_cnas = passenger_cnas || (used[s2] && cna_rate[s2] > 0);
    }
    passenger_cnas = passenger_cnas && !e->cna_cands.empty();
    auto cna_d = upload(P, cna_rate, st);
    pg::PlaceTables t{};
    t.n_nodes = f->n; t.parent = e->fc_parent.p; t.birth = e->fc_birth.p; t.species = e->fc_species.p;
    t.divisions = e->fc_div.p;
    t.n_epochs = E; t.epoch_start = times_d.p; t.snv_rate = snv_d.p; t.indel_rate = id_d.p; t.cna_rate = cna_d.p;
    t.n_sbs_sigs = std::max<uint32_t>(e->n_sig[0], 1); t.n_id_sigs = std::max<uint32_t>(e->n_sig[1], 1);
    t.sbs_expo_cdf = sbs_expo_d.p; t.sbs_sig_cdf = sbs_sig_d.p; t.id_expo_cdf = id_expo_d.p; t.id_sig_cdf = id_sig_d.p;
    t.genome = e->genome.p;
    t.ctx_off = e->ctx_off_d.p; t.ctx_len = e->ctx_len_d.p; t.ctx_lists = e->ctx_lists.p;
    t.id_off = e->id_off_d.p; t.id_len = e->id_len_d.p; t.id_lists = e->id_lists.p;

    Timer timer(st);
    // ---- passenger CNA counts (germline-size rate, so they do not depend on the events)
    std::vector<uint32_t> cnt_cna(f->n, 0);
    if (passenger_cnas) {
      DBuf<uint32_t> cc(P, f->n);
      pg::place_cna_counts(t, cc.p, seed, 2.0 * double(e->G), st);
      ck(cudaMemcpyAsync(cnt_cna.data(), cc.p, sizeof(uint32_t) * f->n, cudaMemcpyDeviceToHost, st), "cna counts");
      ck(cudaStreamSynchronize(st), "cna counts");
    }
    // ---- replay drivers and CNA/WGD events into genotype classes (host)
    auto pl = std::make_unique<pg_placed>();
    std::vector<pg::GenomeFrags> classes(1);
    for (uint32_t c = 0; c < e->n_chr; ++c) {
      classes[0].push_back({0u, e->chr_off[c], e->chr_off[c + 1]});
      classes[0].push_back({1u, e->chr_off[c], e->chr_off[c + 1]});
    }
    std::vector<pg::InstInfo> insts{{-1, 0}, {-1, 0}};
    std::vector<uint32_t> node_class(f->n + 1, 0);
    std::vector<pg::DriverRec> drv;
    uint32_t drv_index = 0;
    std::vector<uint32_t> mutant_of(S, 0u);
    for (uint32_t s2 = 0; s2 < S; ++s2) {
      auto it = e->species.find(s2);
      if (it != e->species.end()) mutant_of[s2] = it->second.mutant;
    }
    auto mut_of = [&](uint32_t node) { return mutant_of[f->species[node]]; };
    // order key of the copy made by event j on edge v (see SEQ_PASSENGER)
    auto key_of = [&](uint32_t v, uint32_t j) { return (uint64_t(f->tin[v]) << 16) | (j + 1u); };
    for (uint32_t v = 0; v < f->n; ++v) {
      const uint32_t base = f->parent[v] >= 0 ? node_class[f->parent[v]] : 0u;
      const std::vector<DriverEvent>* devs = nullptr;
      const uint32_t m = mut_of(v);
      if (f->parent[v] < 0 || mut_of(uint32_t(f->parent[v])) != m) {
        auto it = e->drivers.find(m);
        if (it != e->drivers.end()) devs = &it->second;
      }
      const uint32_t nd = devs ? uint32_t(devs->size()) : 0u;
      require(uint64_t(nd) + cnt_cna[v] <= pg::SEQ_MAX_EVENTS, "too many driver and CNA events on one edge");
      bool touches = cnt_cna[v] > 0;
      for (uint32_t j = 0; j < nd; ++j) touches = touches || (*devs)[j].kind != 0;
      if (!touches && nd == 0) { node_class[v] = base; continue; }
      pg::GenomeFrags g = touches ? classes[base] : pg::GenomeFrags();
      const pg::GenomeFrags& gv = touches ? g : classes[base];
      bool changed = false;
      auto apply_cna = [&](const CnaSpec& c, uint32_t seq, uint32_t r_word, bool passenger) {
        const uint32_t b = e->chr_off[c.chr] + c.begin - 1;
        const uint32_t end = uint32_t(std::min<uint64_t>(uint64_t(b) + c.len, e->chr_off[c.chr + 1]));
        if (b >= end) return;
        const auto cov = pg::covering_insts(g, b);
        if (cov.empty()) return;
        CnaOut rec{v, uint8_t(c.amp ? 1 : 0), c.chr, c.begin, c.begin + (end - b) - 1, 0, 0, uint8_t(passenger ? 0 : 1)};
        if (c.amp) {
          const uint32_t ord = c.src >= 0 ? uint32_t(c.src) : mulhi32(r_word, uint32_t(cov.size()));
          if (ord >= cov.size()) throw DomainError("CNA source allele " + std::to_string(ord) + " does not cover the region");
          const uint32_t x = cov[ord], xn = uint32_t(insts.size());
          insts.push_back({int32_t(x), key_of(v, seq)});
          pg::frag_amplify(g, x, xn, b, end);
          rec.allele = xn; rec.src = x;
        } else {
          if (passenger && e->avoid_homozygous_losses && cov.size() <= 1) return;
          const uint32_t ord = c.allele >= 0 ? uint32_t(c.allele) : mulhi32(r_word, uint32_t(cov.size()));
          if (ord >= cov.size()) throw DomainError("CNA allele " + std::to_string(ord) + " does not cover the region");
          pg::frag_delete(g, cov[ord], b, end);
          rec.allele = cov[ord]; rec.src = cov[ord];
        }
        changed = true;
        pl->cnas.push_back(rec);
      };
      for (uint32_t j = 0; j < nd; ++j) {
        const DriverEvent& de = (*devs)[j];
        if (de.kind == 0) {
          const DriverSpec& d = de.sid;
          pg::DriverRec r{};
          r.locus = e->chr_off[d.chr] + d.pos - 1;   // SNV site, or the shared first base of an indel
          r.edge = v;
          r.seq = j;
          const auto cov = pg::covering_insts(gv, r.locus);
          if (cov.empty()) throw DomainError("a driver mutation lies where the cell has no allele left");
          uint32_t ord;
          if (d.allele >= 0) {
            ord = uint32_t(d.allele);
            if (ord >= cov.size()) throw DomainError("driver allele " + std::to_string(ord) + " does not exist there");
          } else {
            uint32_t w[4];
            philox_host(seed, drv_index, v, 0u, 6u /* TAG_DRIVER */, w);
            ord = mulhi32(w[0], uint32_t(cov.size()));
          }
          r.allele = cov[ord];
          if (d.ref.size() == 1 && d.alt.size() == 1) {
            r.kind = pg::KIND_SNV; r.aux = code_of(d.alt[0]);
          } else {
            r.kind = pg::KIND_INDEL;
            if (d.alt.size() > 1) {
              uint32_t bases = 0;
              for (size_t k = 1; k < d.alt.size(); ++k) bases |= code_of(d.alt[k]) << (2 * (k - 1));
              r.aux = 1u | (uint32_t(d.alt.size() - 1) << 1) | (bases << 8);
            } else {
              r.aux = 0u | (uint32_t(d.ref.size() - 1) << 1);
            }
          }
          drv.push_back(r);
          ++drv_index;
        } else if (de.kind == 1) {
          uint32_t w[4];
          philox_host(seed, j, v, 1u, 12u /* TAG_CNA */, w);
          apply_cna(de.cna, j, w[1], false);
        } else {                                  // whole-genome doubling
          std::vector<uint32_t> present;
          for (const auto& fr : g) present.push_back(fr.inst);
          std::sort(present.begin(), present.end());
          present.erase(std::unique(present.begin(), present.end()), present.end());
          for (uint32_t x : present) {
            const uint32_t xn = uint32_t(insts.size());
            insts.push_back({int32_t(x), key_of(v, j)});
            pg::frag_amplify(g, x, xn, 0u, 0xffffffffu);
          }
          pl->cnas.push_back({v, 2, 0, 0, 0, 0, 0, 1});
          changed = true;
        }
      }
      for (uint32_t k = 0; k < cnt_cna[v]; ++k) {
        uint32_t w[4];
        philox_host(seed, k, v, 0u, 12u /* TAG_CNA */, w);
        const CnaSpec& cand = e->cna_cands[mulhi32(w[0], uint32_t(e->cna_cands.size()))];
        apply_cna(cand, nd + k, w[1], true);
      }
      if (changed) {
        require(classes.size() < (1u << 24), "too many genotype classes");
        classes.push_back(std::move(g));
        node_class[v] = uint32_t(classes.size() - 1);
      } else {
        node_class[v] = base;
      }
    }
    require(insts.size() < 0xffff, "too many allele instances");
    // ---- node sizes, then the per-edge counts (they need nothing else of
    // the classes), launched before the host builds the class tables
    std::vector<double> class_size(classes.size());
    for (size_t c = 0; c < classes.size(); ++c) class_size[c] = double(pg::frag_size(classes[c]));
    std::vector<double> node_size(f->n + 1);
    for (uint32_t v = 0; v < f->n; ++v) node_size[v] = class_size[node_class[v]];
    node_size[f->n] = class_size[0];
    auto node_size_d = upload(P, node_size, st);
    t.node_size = node_size_d.p;
    const uint64_t ncell = uint64_t(f->n + 1) * E;
    DBuf<uint32_t> cnt_snv(P, ncell), cnt_id(P, ncell), off_snv(P, ncell), off_id(P, ncell);
    DBuf<uint32_t> part(P, pg::scan_part_elems(ncell, 1)), tot(P, 2);
    pg::place_edge_counts(t, cnt_snv.p, cnt_id.p, seed, n_pre_snv, n_pre_id, st);
    pg::scan_rows<uint32_t>(cnt_snv.p, off_snv.p, ncell, 1, part.p, tot.p, st);
    pg::scan_rows<uint32_t>(cnt_id.p, off_id.p, ncell, 1, part.p, tot.p + 1, st);
    // ---- class tables (segments) and instance lineage chains
    std::vector<uint32_t> seg_off{0}, seg_start, seg_end, seg_ioff, seg_icnt;
    std::vector<uint16_t> inst_list;
    uint32_t cn_max = 0;
    for (size_t c = 0; c < classes.size(); ++c) {
      for (const auto& sg : pg::segments_of(classes[c])) {
        seg_start.push_back(sg.b); seg_end.push_back(sg.e);
        seg_ioff.push_back(uint32_t(inst_list.size())); seg_icnt.push_back(uint32_t(sg.insts.size()));
        for (uint32_t x : sg.insts) inst_list.push_back(uint16_t(x));
        cn_max = std::max<uint32_t>(cn_max, uint32_t(sg.insts.size()));
      }
      seg_off.push_back(uint32_t(seg_start.size()));
    }
    std::vector<uint32_t> chain_off{0};
    std::vector<uint16_t> chain_anc;
    std::vector<uint64_t> chain_key;
    for (size_t y = 0; y < insts.size(); ++y) {
      for (int32_t cur = int32_t(y); insts[cur].parent >= 0; cur = insts[cur].parent) {
        chain_anc.push_back(uint16_t(insts[cur].parent));
        chain_key.push_back(insts[cur].key);
      }
      chain_off.push_back(uint32_t(chain_anc.size()));
    }
    pl->has_cna = classes.size() > 1 || insts.size() > 2;
    pl->chain_off_h = chain_off; pl->chain_anc_h = chain_anc; pl->chain_key_h = chain_key;
    pl->seg_off_h = seg_off; pl->seg_start_h = seg_start; pl->seg_end_h = seg_end;
    pl->seg_ioff_h = seg_ioff; pl->seg_icnt_h = seg_icnt; pl->inst_list_h = inst_list;
    pl->inst_root_h.resize(insts.size());
    for (size_t y = 0; y < insts.size(); ++y) {
      int32_t r = int32_t(y);
      while (insts[r].parent >= 0) r = insts[r].parent;
      pl->inst_root_h[y] = uint8_t(r);
    }
    pl->cn_max = std::max<uint32_t>(cn_max, 2);
    pl->n_classes = uint32_t(classes.size());
    pl->node_class_h = node_class;
    pl->node_class = upload(P, node_class, st);
    {
      // atoms: cut at every segment boundary of every class, then merge
      // neighbours on which every class sits in the same segment
      const uint32_t C = uint32_t(classes.size());
      std::vector<uint32_t> cuts{0u, uint32_t(e->G)};
      cuts.insert(cuts.end(), seg_start.begin(), seg_start.end());
      cuts.insert(cuts.end(), seg_end.begin(), seg_end.end());
      std::sort(cuts.begin(), cuts.end());
      cuts.erase(std::unique(cuts.begin(), cuts.end()), cuts.end());
      std::vector<uint32_t> cur(C), prev, ptr(seg_off.begin(), seg_off.end() - 1);
      std::vector<uint32_t> atom_ioff;
      for (size_t i = 0; i + 1 < cuts.size(); ++i) {
        const uint32_t b = cuts[i];
        for (uint32_t c = 0; c < C; ++c) {
          uint32_t& q = ptr[c];
          while (q < seg_off[c + 1] && seg_end[q] <= b) ++q;
          cur[c] = (q < seg_off[c + 1] && seg_start[q] <= b) ? q : 0xffffffffu;
        }
        if (!prev.empty() && cur == prev) continue;
        prev = cur;
        pl->atom_start_h.push_back(b);
        for (uint32_t c = 0; c < C; ++c) {
          const bool in = cur[c] != 0xffffffffu;
          atom_ioff.push_back(in ? seg_ioff[cur[c]] : 0u);
          pl->atom_icnt_h.push_back(in ? seg_icnt[cur[c]] : 0u);
        }
      }
      pl->atom_start = upload(P, pl->atom_start_h, st);
      pl->atom_ioff = upload(P, atom_ioff, st);
      pl->atom_icnt = upload(P, pl->atom_icnt_h, st);
    }
    pl->seg_off = upload(P, seg_off, st); pl->seg_start = upload(P, seg_start, st); pl->seg_end = upload(P, seg_end, st);
    pl->seg_ioff = upload(P, seg_ioff, st); pl->seg_icnt = upload(P, seg_icnt, st);
    if (inst_list.empty()) inst_list.push_back(0);
    pl->inst_list = upload(P, inst_list, st);
    if (chain_anc.empty()) { chain_anc.push_back(0); chain_key.push_back(0); }
    pl->chain_off = upload(P, chain_off, st); pl->chain_anc = upload(P, chain_anc, st); pl->chain_key = upload(P, chain_key, st);
    t.gc = pl->classes_view();
    // ---- the edge counts' totals size the outputs
    uint32_t tot_h[2];
    ck(cudaMemcpyAsync(tot_h, tot.p, sizeof(tot_h), cudaMemcpyDeviceToHost, st), "counts");
    ck(cudaStreamSynchronize(st), "edge counts");
    const uint64_t n_snv = tot_h[0], n_id = tot_h[1];
    const uint64_t n_all = n_snv + n_id + drv.size();
    require(n_all < (1ull << 31), "too many mutations for one placement call");
    // ---- outputs
    pl->M = n_all;
    DBuf<uint32_t> locus(P, n_all), edge(P, n_all), aux(P, n_all), attempt(P, n_all);
    DBuf<uint8_t> cls(P, n_all), sig(P, n_all), kind(P, n_all), nature(P, n_all);
    DBuf<uint16_t> allele(P, n_all), seqv(P, n_all);
    pg::PlaceOut o{locus.p, edge.p, aux.p, cls.p, sig.p, allele.p, seqv.p, kind.p, nature.p, attempt.p};
    DBuf<uint32_t> err(P, 1);
    ck(cudaMemsetAsync(err.p, 0, sizeof(uint32_t), st), "memset");
    // infinite sites: the first draw goes into the first round's table as it
    // is made (the drivers' loci follow; the losers are read back below)
    const bool unique = e->infinite_sites;
    const uint32_t n_slots = uint32_t(n_snv + n_id);
    DBuf<unsigned long long> first;
    DBuf<uint8_t> lost1;
    uint32_t fmask = 0;
    if (unique && n_slots > 0) {
      uint64_t fcap = 1024;
      while (fcap < 2 * n_all) fcap <<= 1;
      require(fcap <= (uint64_t(1) << 32), "too many mutations for one placement call");
      first = DBuf<unsigned long long>(P, fcap);
      fmask = uint32_t(fcap - 1);
      lost1 = DBuf<uint8_t>(P, n_slots);
      ck(cudaMemsetAsync(first.p, 0xff, sizeof(unsigned long long) * fcap, st), "memset");
      pg::place_first_round(t, o, seed, off_snv.p, off_id.p, uint32_t(n_snv), n_slots, first.p, fmask, lost1.p, err.p,
                            st);
    } else {
      pg::place_mutations_launch(t, o, seed, off_snv.p, off_id.p, uint32_t(n_snv), uint32_t(n_id), nullptr, n_slots, 0,
                                 err.p, st);
    }
    auto drv_d = upload(P, drv, st);
    pg::place_drivers(o, drv_d.p, uint32_t(drv.size()), n_slots, st);
    // the handle's host columns, while the first round runs
    pl->eng = e; pl->n_nodes = f->n; pl->n_samples = f->n_samples;
    pl->tin = f->tin; pl->tout = f->tout; pl->leaves = f->leaves; pl->parent = f->parent;
    pl->leaf_cls.assign(f->n_samples, {});
    {
      std::vector<uint8_t> has_kid(f->n, 0);
      for (uint32_t v = 0; v < f->n; ++v) if (f->parent[v] >= 0) has_kid[f->parent[v]] = 1;
      for (uint32_t v = 0; v < f->n; ++v)
        if (!has_kid[v] && f->sample[v] >= 0) pl->leaf_cls[f->sample[v]].push_back(node_class[v]);
    }
    // ---- infinite sites, and loci drawn where the cell has no allele left.
    // Infinite sites: the first round over all slots against one table of
    // its candidates (drivers first), read back once to size the later
    // rounds' tables; every later round runs in one cooperative launch.
    DBuf<pg::TailCtl> tail_ctl;
    if ((unique || pl->has_cna) && n_slots > 0) {
      uint32_t n_tail = 0;
      pg::TailArgs ta{};
      ta.unique = unique ? 1 : 0;
      DBuf<uint32_t> pend_a, pend_b, hkeys, ckeys, cvals, hpos;
      if (unique) {
        pend_a = DBuf<uint32_t>(P, n_slots);
        DBuf<uint32_t> n_next(P, 1);
        ck(cudaMemsetAsync(n_next.p, 0, sizeof(uint32_t), st), "memset");
        pg::sites_first_finish(locus.p + n_slots, uint32_t(drv.size()), first.p, fmask, lost1.p, n_slots, pend_a.p,
                               n_next.p, err.p, st);
        ck(cudaMemcpyAsync(&n_tail, n_next.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st), "round");
        ck(cudaStreamSynchronize(st), "first round");
        uint32_t cap = 1024;
        while (cap < 2 * uint64_t(n_tail)) cap <<= 1;
        pend_b = DBuf<uint32_t>(P, n_tail);
        hpos = DBuf<uint32_t>(P, n_tail);
        hkeys = DBuf<uint32_t>(P, cap); ckeys = DBuf<uint32_t>(P, cap); cvals = DBuf<uint32_t>(P, cap);
        ck(cudaMemsetAsync(hkeys.p, 0xff, sizeof(uint32_t) * cap, st), "memset");
        ck(cudaMemsetAsync(ckeys.p, 0xff, sizeof(uint32_t) * cap, st), "memset");
        ck(cudaMemsetAsync(cvals.p, 0xff, sizeof(uint32_t) * cap, st), "memset");
        ta.redraw_first = 1;
        ta.round0 = 1;
        ta.hkeys = hkeys.p; ta.hmask = cap - 1;
        ta.ckeys = ckeys.p; ta.cvals = cvals.p; ta.cmask = cap - 1;
        ta.hpos = hpos.p;
        ta.first = first.p; ta.fmask = fmask;
      } else {
        // loci without an allele: round 0 looks at every slot
        n_tail = n_slots;
        pend_a = DBuf<uint32_t>(P, n_slots);
        pend_b = DBuf<uint32_t>(P, n_slots);
        ta.identity_first = 1;
        ta.round0 = 0;
      }
      ta.list[0] = pend_a.p;
      ta.list[1] = pend_b.p;
      if (n_tail) {
        tail_ctl = DBuf<pg::TailCtl>(P, 1);
        pg::TailCtl c0{};
        c0.count[0] = n_tail;
        ck(cudaMemcpyAsync(tail_ctl.p, &c0, sizeof(c0), cudaMemcpyHostToDevice, st), "rounds");
        if (const char* msg = pg::sites_tail(t, o, seed, off_snv.p, off_id.p, uint32_t(n_snv), ta, n_tail, tail_ctl.p,
                                             err.p, st))
          throw std::runtime_error(msg);
      }
    }
    // ---- sort by locus
    const uint32_t nb = pg::sort_num_buckets(e->G);
    DBuf<uint32_t> bcnt(P, nb), bfill(P, nb), bpart(P, pg::scan_part_elems(nb, 1)), order(P, n_all);
    pl->locus = DBuf<uint32_t>(P, n_all); pl->edge = DBuf<uint32_t>(P, n_all); pl->aux = DBuf<uint32_t>(P, n_all);
    pl->attempt = DBuf<uint32_t>(P, n_all);
    pl->cls = DBuf<uint8_t>(P, n_all); pl->sig = DBuf<uint8_t>(P, n_all); pl->allele = DBuf<uint16_t>(P, n_all);
    pl->seq = DBuf<uint16_t>(P, n_all);
    pl->kind = DBuf<uint8_t>(P, n_all); pl->nature = DBuf<uint8_t>(P, n_all);
    DBuf<unsigned long long> skeys(P, n_all);
    DBuf<uint4> recs(P, 2 * n_all);   // 32-byte records of the gather
    pg::sort_by_locus(o, uint32_t(n_all), e->G, bcnt.p, bfill.p, bpart.p, order.p, pl->view(), skeys.p, recs.p, st);
    pl->kernel_ms = timer.stop();
    ck(cudaGetLastError(), "placement kernels");
    uint32_t err_h = 0;
    ck(cudaMemcpy(&err_h, err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost), "error flag");
    if (tail_ctl.p) {
      pg::TailCtl c{};
      ck(cudaMemcpy(&c, tail_ctl.p, sizeof(c), cudaMemcpyDeviceToHost), "rounds");
      if (c.status & pg::TAIL_BARRIER_TIMEOUT) throw std::runtime_error("a grid barrier of the redraw rounds timed out");
      require(!(c.status & pg::TAIL_ROUNDS_EXHAUSTED), unique ? "infinite sites model: no free locus left for some mutations"
                                                              : "no allele left where some mutations were drawn");
      pl->redraw_rounds = c.rounds;
    }
    if (err_h & pg::ERR_EMPTY_CLASS) throw std::runtime_error("a drawn mutation class has no indexed positions");
    if (err_h & pg::ERR_CAPACITY) throw std::runtime_error("internal hash table capacity exceeded");
    engine_retain(e);
    *out = pl.release();
  });
}

pg_status pg_placed_destroy(pg_placed* p) {
  return guarded([&] {
    if (!p) return;
    pg_engine* e = p->eng;
    cudaSetDevice(e->device);
    delete p;              // device buffers go back to the engine's pool
    engine_release(e);
  });
}

pg_status pg_placed_count(const pg_placed* p, uint64_t* n) {
  return guarded([&] { require(p && n, "NULL argument"); *n = p->M; });
}

pg_status pg_placed_cna_count(const pg_placed* p, uint64_t* n) {
  return guarded([&] { require(p && n, "NULL argument"); *n = p->cnas.size(); });
}

pg_status pg_placed_cna_copy(const pg_placed* p, uint32_t* node, uint8_t* type, uint32_t* chr, uint32_t* begin,
                             uint32_t* end, uint32_t* allele, uint32_t* src_allele, uint8_t* driver) {
  return guarded([&] {
    require(p != nullptr, "NULL handle");
    for (size_t i = 0; i < p->cnas.size(); ++i) {
      const CnaOut& c = p->cnas[i];
      if (node) node[i] = c.node;
      if (type) type[i] = c.type;
      if (chr) chr[i] = c.chr;
      if (begin) begin[i] = c.begin;
      if (end) end[i] = c.end;
      if (allele) allele[i] = c.allele;
      if (src_allele) src_allele[i] = c.src;
      if (driver) driver[i] = c.driver;
    }
  });
}

pg_status pg_placed_class_dims(const pg_placed* p, uint32_t* n_classes, uint32_t* n_segments, uint32_t* n_list,
                               uint32_t* n_instances) {
  return guarded([&] {
    require(p != nullptr, "NULL handle");
    if (n_classes) *n_classes = p->n_classes;
    if (n_segments) *n_segments = uint32_t(p->seg_start_h.size());
    if (n_list) *n_list = uint32_t(p->inst_list_h.size());
    if (n_instances) *n_instances = uint32_t(p->inst_root_h.size());
  });
}

pg_status pg_placed_class_copy(const pg_placed* p, uint32_t* seg_off, uint32_t* seg_start, uint32_t* seg_end,
                               uint32_t* seg_ioff, uint32_t* seg_icnt, uint16_t* inst_list, uint8_t* inst_root) {
  return guarded([&] {
    require(p != nullptr, "NULL handle");
    auto cp = [](auto* dst, const auto& v) { if (dst) std::copy(v.begin(), v.end(), dst); };
    cp(seg_off, p->seg_off_h); cp(seg_start, p->seg_start_h); cp(seg_end, p->seg_end_h);
    cp(seg_ioff, p->seg_ioff_h); cp(seg_icnt, p->seg_icnt_h); cp(inst_list, p->inst_list_h);
    cp(inst_root, p->inst_root_h);
  });
}

pg_status pg_placed_node_classes(const pg_placed* p, uint32_t* node_class, uint32_t* n_classes, uint32_t* cn_max) {
  return guarded([&] {
    require(p != nullptr, "NULL handle");
    if (node_class) std::copy(p->node_class_h.begin(), p->node_class_h.begin() + p->n_nodes, node_class);
    if (n_classes) *n_classes = p->n_classes;
    if (cn_max) *cn_max = p->cn_max;
  });
}

pg_status pg_placed_lineage_dims(const pg_placed* p, uint32_t* n_instances, uint32_t* n_links) {
  return guarded([&] {
    require(p != nullptr, "NULL handle");
    if (n_instances) *n_instances = p->chain_off_h.empty() ? 0u : uint32_t(p->chain_off_h.size() - 1);
    if (n_links) *n_links = uint32_t(p->chain_anc_h.size());
  });
}

pg_status pg_placed_lineage_copy(const pg_placed* p, uint32_t* chain_off, uint16_t* chain_anc, uint64_t* chain_key,
                                 uint64_t* order_key) {
  return guarded([&] {
    require(p != nullptr, "NULL handle");
    if (chain_off) std::copy(p->chain_off_h.begin(), p->chain_off_h.end(), chain_off);
    if (chain_anc) std::copy(p->chain_anc_h.begin(), p->chain_anc_h.end(), chain_anc);
    if (chain_key) std::copy(p->chain_key_h.begin(), p->chain_key_h.end(), chain_key);
    if (order_key && p->M) {
      // (tin of the mutation's edge << 16) | its order on the edge; the
      // preneoplastic edge has tin 0
      select_device(p->eng);
      std::vector<uint32_t> edge(p->M);
      std::vector<uint16_t> seq(p->M);
      ck(cudaMemcpy(edge.data(), p->edge.p, sizeof(uint32_t) * p->M, cudaMemcpyDeviceToHost), "copy");
      ck(cudaMemcpy(seq.data(), p->seq.p, sizeof(uint16_t) * p->M, cudaMemcpyDeviceToHost), "copy");
      for (uint64_t i = 0; i < p->M; ++i) {
        const uint64_t tin = edge[i] < p->n_nodes ? p->tin[edge[i]] : 0u;
        order_key[i] = (tin << 16) | (seq[i] & 0x7fffu);
      }
    }
  });
}

pg_status pg_placed_set_samples(pg_placed* p, uint32_t n_samples, const int32_t* sample_of_node) {
  return guarded([&] {
    require(p != nullptr && sample_of_node != nullptr, "NULL argument");
    std::vector<std::vector<uint32_t>> leaves(n_samples), leaf_cls(n_samples);
    for (uint32_t v = 0; v < p->n_nodes; ++v) {
      const int32_t s = sample_of_node[v];
      if (s < 0) continue;
      require(uint32_t(s) < n_samples, "sample index out of range");
      require(p->tout[v] == p->tin[v] + 1, "only leaves (sampled cells) can be assigned to a sample");
      leaves[s].push_back(p->tin[v]);
      leaf_cls[s].push_back(p->node_class_h.empty() ? 0u : p->node_class_h[v]);
    }
    p->leaves = std::move(leaves);
    p->leaf_cls = std::move(leaf_cls);
    p->n_samples = n_samples;
  });
}

pg_status pg_engine_index_ms(const pg_engine* e, float* ms) {
  return guarded([&] {
    require(e && ms, "NULL argument");
    for (int i = 0; i < 4; ++i) ms[i] = e->index_ms[i];
  });
}

pg_status pg_placed_redraw_rounds(const pg_placed* p, uint32_t* rounds) {
  return guarded([&] { require(p && rounds, "NULL argument"); *rounds = p->redraw_rounds; });
}

pg_status pg_placed_kernel_ms(const pg_placed* p, float* ms) {
  return guarded([&] { require(p && ms, "NULL argument"); *ms = p->kernel_ms; });
}

pg_status pg_placed_copy(const pg_placed* p, uint32_t* locus, uint32_t* edge, uint32_t* aux, uint8_t* cls,
                         uint8_t* sig, uint16_t* allele, uint8_t* kind, uint8_t* nature) {
  return guarded([&] {
    require(p != nullptr, "NULL handle");
    select_device(p->eng);
    const size_t n = p->M;
    if (n == 0) return;
    auto cp = [&](void* dst, const void* src, size_t bytes) {
      if (dst) ck(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, p->eng->st), "copy");
    };
    cp(locus, p->locus.p, 4 * n); cp(edge, p->edge.p, 4 * n); cp(aux, p->aux.p, 4 * n);
    cp(cls, p->cls.p, n); cp(sig, p->sig.p, n); cp(allele, p->allele.p, 2 * n); cp(kind, p->kind.p, n);
    cp(nature, p->nature.p, n);
    ck(cudaStreamSynchronize(p->eng->st), "copy");
  });
}

namespace {

// insert-size CDF table (min insert, thresholds)
void insert_table(const pg_seq_cfg& c, uint32_t R, uint32_t& ins_min, std::vector<uint32_t>& thr) {
  const double mean = c.insert_size_mean, sd = c.insert_size_stddev;
  std::vector<double> w;
  uint32_t k0 = 0;
  if (c.insert_model == PG_INSERT_BINOMIAL) {
    // src/seq_simulation.cpp:431-451: Binomial(t = mean/p, p = 1 - sd^2/mean)
    const double q = double(c.insert_size_stddev) * double(c.insert_size_stddev) / mean;
    const double p = 1 - q;
    if (p < 0) {
      throw std::runtime_error("The insert size mean (" + std::to_string(c.insert_size_mean) +
                               ") must be greater than or equal to its variance (" +
                               std::to_string(c.insert_size_stddev) + "*" + std::to_string(c.insert_size_stddev) +
                               "=" + std::to_string(c.insert_size_stddev * c.insert_size_stddev) + ").");
    }
    require(p > 0, "insert size variance equal to the mean gives an undefined binomial model");
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
    require(sd > 0, "the normal insert model needs a positive standard deviation");
    const double a = std::max(1.0, std::floor(mean - 10 * sd)), b = std::ceil(mean + 10 * sd);
    k0 = uint32_t(a);
    for (double k = a; k <= b; k += 1) {
      const double z0 = (k - 0.5 - mean) / (sd * std::sqrt(2.0)), z1 = (k + 0.5 - mean) / (sd * std::sqrt(2.0));
      w.push_back(0.5 * (std::erfc(z0) - std::erfc(z1)));
    }
  }
  // inserts shorter than a read are clamped to the read size
  if (k0 < R) {
    const uint32_t drop = std::min<uint32_t>(R - k0, uint32_t(w.size()) - 1);
    double mass = 0;
    for (uint32_t i = 0; i < drop; ++i) mass += w[i];
    w.erase(w.begin(), w.begin() + drop);
    w[0] += mass;
    k0 += drop;
    if (k0 < R) k0 = R;
  }
  ins_min = k0;
  thr = cdf_thresholds(w);
}

}  // namespace

namespace {

// SAM files of a sequencing call (see pg_sam_cfg): one per chromosome, the
// reads of every sample as read groups, built on the device chunk by chunk
void write_sam(pg_engine* e, const pg_placed* pl, const pg_sam_cfg& sam, uint64_t seed, const pg::SeqRec* recs,
               const pg::SeqTiles& tiles, const uint32_t* pair_cnt_d, const pg::SeqSample* samples_d,
               uint32_t n_samples, const uint32_t* leaf_d, const pg::SeqParams& prm,
               const std::vector<uint32_t>& c_id, const std::vector<uint32_t>& c_first,
               const std::vector<uint32_t>& c_ntiles, double error_rate) {
  namespace fs = std::filesystem;
  require(sam.output_dir && sam.filename_prefix && sam.template_name_prefix && sam.sample_names && sam.chr_names,
          "NULL SAM argument");
  cudaStream_t st = e->st;
  Pool* P = &e->pool;
  const fs::path dir(sam.output_dir);
  if (fs::exists(dir)) {
    require(sam.update != 0, "The output directory \"" + dir.string() + "\" already exists: set update_SAM to write into it");
    require(fs::is_directory(dir), "\"" + dir.string() + "\" is not a directory");
  } else {
    fs::create_directories(dir);
  }
  const uint32_t n_tiles = tiles.n_tiles, mates = prm.paired ? 2u : 1u, R = prm.read_len;
  std::vector<uint32_t> pc(uint64_t(n_samples) * n_tiles);
  ck(cudaMemcpyAsync(pc.data(), pair_cnt_d, sizeof(uint32_t) * pc.size(), cudaMemcpyDeviceToHost, st), "pair counts");
  ck(cudaStreamSynchronize(st), "pair counts");
  // Phred quality of the substitution rate (constant, as the reference's
  // constant-quality Illumina model)
  int q = error_rate > 0 ? int(std::lround(-10.0 * std::log10(error_rate))) : 41;
  q = std::max(2, std::min(41, q));
  const char qual = char('!' + q);
  uint64_t cap = uint64_t(1) << 22;   // reads per chunk
  DBuf<pg::SamRead> out(P, cap);
  DBuf<char> seq(P, cap * R);
  std::vector<pg::SamRead> h_out;
  std::vector<char> h_seq;
  std::string line;
  for (size_t slot = 0; slot < c_id.size(); ++slot) {
    const uint32_t chr = c_id[slot];
    const std::string name = sam.chr_names[chr];
    const std::string stem = std::string(sam.filename_prefix) + name;
    fs::path path = dir / (stem + ".sam");
    for (uint32_t n = 1; fs::exists(path); ++n) path = dir / (stem + "_" + std::to_string(n) + ".sam");
    std::ofstream f(path, std::ios::binary);
    require(bool(f), "cannot write " + path.string());
    const uint32_t off = e->chr_off[chr];
    f << "@HD\tVN:1.6\tSO:unsorted\n@SQ\tSN:" << name << "\tLN:" << e->chr_len[chr] << "\n";
    for (uint32_t s = 0; s < n_samples; ++s) f << "@RG\tID:" << sam.sample_names[s] << "\tSM:" << sam.sample_names[s] << "\n";
    uint64_t tmpl = 0;
    const uint32_t t_end = c_first[slot] + c_ntiles[slot];
    for (uint32_t k = c_first[slot]; k < t_end;) {
      // a chunk of whole tiles whose reads fit the buffers
      uint32_t k2 = k;
      uint64_t frags = 0;
      while (k2 < t_end) {
        uint64_t add = 0;
        for (uint32_t s = 0; s < n_samples; ++s) add += pc[uint64_t(s) * n_tiles + k2];
        if (k2 > k && (frags + add) * mates > cap) break;
        frags += add;
        ++k2;
      }
      if (frags * mates > cap) {        // one tile alone exceeds the buffers
        cap = frags * mates;
        out = DBuf<pg::SamRead>(P, cap);
        seq = DBuf<char>(P, cap * R);
      }
      const uint32_t n_chunk = k2 - k;
      std::vector<uint64_t> off_h(uint64_t(n_samples) * n_chunk);
      uint64_t acc = 0;
      for (uint32_t s = 0; s < n_samples; ++s)
        for (uint32_t x = 0; x < n_chunk; ++x) { off_h[uint64_t(s) * n_chunk + x] = acc; acc += pc[uint64_t(s) * n_tiles + k + x]; }
      auto off_d = upload(P, off_h, st);
      pg::seq_sam_reads(recs, uint32_t(pl->M), pl->aux.p, e->genome.p, tiles, k, n_chunk, pair_cnt_d, samples_d,
                        n_samples, leaf_d, prm, seed, off_d.p, out.p, seq.p, R, st);
      const uint64_t nr = acc * mates;
      h_out.resize(nr);
      h_seq.resize(nr * R);
      if (nr) {
        ck(cudaMemcpyAsync(h_out.data(), out.p, sizeof(pg::SamRead) * nr, cudaMemcpyDeviceToHost, st), "SAM reads");
        ck(cudaMemcpyAsync(h_seq.data(), seq.p, nr * R, cudaMemcpyDeviceToHost, st), "SAM reads");
      }
      ck(cudaStreamSynchronize(st), "SAM reads");
      static const char ops[3] = {'M', 'I', 'D'};
      for (uint32_t s = 0; s < n_samples; ++s) {
        const std::string rg = std::string("\tRG:Z:") + sam.sample_names[s] + "\n";
        for (uint32_t x = 0; x < n_chunk; ++x) {
          const uint64_t o = off_h[uint64_t(s) * n_chunk + x];
          const uint32_t np = pc[uint64_t(s) * n_tiles + k + x];
          for (uint32_t j = 0; j < np; ++j) {
            const std::string qname = std::string(sam.template_name_prefix) + std::to_string(tmpl + o + j);
            for (uint32_t m = 0; m < mates; ++m) {
              const uint64_t r = (o + j) * mates + m;
              const pg::SamRead& a = h_out[r];
              line.clear();
              line += qname; line += '\t';
              line += std::to_string(a.flag); line += '\t';
              if (a.flag & 4) { line += "*\t0\t0\t*\t*\t0\t0\t*\t*"; line += rg; f << line; continue; }
              line += name; line += '\t';
              line += std::to_string(a.pos - off + 1); line += "\t60\t";
              if (a.n_cigar == 0) line += '*';
              for (uint32_t c = 0; c < a.n_cigar; ++c) { line += std::to_string(a.cigar[c] >> 4); line += ops[a.cigar[c] & 15u]; }
              line += '\t';
              if (prm.paired) { line += "=\t"; line += std::to_string(a.mate_pos - off + 1); }
              else line += "*\t0";
              line += '\t'; line += std::to_string(a.tlen); line += '\t';
              line.append(h_seq.data() + r * R, a.seq_len); line += '\t';
              line.append(a.seq_len, qual);
              line += rg;
              f << line;
            }
          }
        }
      }
      tmpl += acc;
      k = k2;
    }
    require(bool(f), "error writing " + path.string());
  }
}

void simulate_seq_impl(const pg_placed* pl, const pg_seq_cfg* c, uint64_t seed, const pg_sam_cfg* sam,
                       pg_seq_result** out);

}  // namespace

pg_status pg_simulate_seq(const pg_placed* pl, const pg_seq_cfg* c, uint64_t seed, pg_seq_result** out) {
  return guarded([&] { simulate_seq_impl(pl, c, seed, nullptr, out); });
}

pg_status pg_simulate_seq_sam(const pg_placed* pl, const pg_seq_cfg* c, uint64_t seed, const pg_sam_cfg* sam,
                              pg_seq_result** out) {
  return guarded([&] {
    require(sam != nullptr, "NULL SAM configuration");
    simulate_seq_impl(pl, c, seed, sam, out);
  });
}

namespace {

void simulate_seq_impl(const pg_placed* pl, const pg_seq_cfg* c, uint64_t seed, const pg_sam_cfg* sam,
                       pg_seq_result** out) {
  {
    require(pl && c && out, "NULL argument");
    pg_engine* e = pl->eng;
    select_device(e);
    cudaStream_t st = e->st;
    Pool* P = &e->pool;
    require(c->coverage >= 0 && std::isfinite(c->coverage), "The coverage must be non-negative");
    require(c->read_size >= 1 && c->read_size <= 4096, "read_size must be in [1, 4096]");
    require(c->purity >= 0 && c->purity <= 1, "The purity must be a value in [0,1]");
    require(c->error_rate >= 0 && c->error_rate <= 1, "The parameter \"error_rate\" must be a positive real number.");
    const uint32_t R = c->read_size;
    const bool paired = c->insert_size_mean > 0;
    uint32_t ins_min = R;
    std::vector<uint32_t> ins_thr{2147483648u};
    if (paired) insert_table(*c, R, ins_min, ins_thr);
    const uint32_t span = std::max<uint32_t>(R, ins_min + uint32_t(ins_thr.size()) - 1);
    // ---- chromosome selection
    std::vector<uint32_t> chrs;
    if (c->n_chr_sel) {
      require(c->chr_sel != nullptr, "NULL chromosome list");
      for (uint32_t i = 0; i < c->n_chr_sel; ++i) { require(c->chr_sel[i] < e->n_chr, "unknown chromosome"); chrs.push_back(c->chr_sel[i]); }
      std::sort(chrs.begin(), chrs.end());
      chrs.erase(std::unique(chrs.begin(), chrs.end()), chrs.end());
    } else {
      for (uint32_t i = 0; i < e->n_chr; ++i) chrs.push_back(i);
    }
    // ---- tile size
    uint32_t T = c->tile_size;
    if (T == 0) {
      // fragments per tile: two shared-memory batches of the read kernel,
      // each 4 standard deviations below its capacity (one batch per tile
      // measured 1-3% slower: the per-tile set-up is paid twice as often);
      // at most 128 records per window, and a window that fits the start
      // buckets
      const double mates_per_frag = paired ? 2.0 : 1.0;
      const double cap = double(pg::SEQ_FRAGS_PER_BATCH);
      const double target = 2.0 * (cap - 4.0 * std::sqrt(cap));
      double t = c->coverage > 0 ? target * R * mates_per_frag / c->coverage : 8192.0;
      const double density = double(pl->M) / double(e->G);
      if (density > 0) t = std::min(t, 128.0 / density);
      t = std::min(t, double(16384 - 1 - span));
      T = uint32_t(std::max(256.0, std::floor(t / 64.0) * 64.0));
    }
    require(T >= 64 && T <= (1u << 24), "tile_size must be in [64, 2^24]");
    // ---- tiles
    // tiles are laid out on the device from the per-chromosome table
    std::vector<uint32_t> c_ntiles, c_nstarts, c_id, c_first, c_depth, c_start, c_end;
    std::vector<uint64_t> c_pairs, heap_base;   // per chromosome: its split tree's heap (2^(depth + 1) entries)
    uint64_t heap_total = 0;
    uint32_t max_depth = 0;
    uint32_t n_tiles = 0;
    const double mates = paired ? 2.0 : 1.0;
    uint64_t frags_per_sample = 0;
    for (uint32_t ci : chrs) {
      const uint32_t L = e->chr_len[ci];
      if (L < R) continue;
      const uint32_t slot = uint32_t(c_id.size());
      const uint32_t S = L - R + 1;
      const uint32_t nt = (S + T - 1) / T;
      const uint64_t pairs = uint64_t(std::floor(c->coverage * double(L) / (double(R) * mates)));
      require(pairs < (uint64_t(1) << 32), "too many fragments for one chromosome");
      uint32_t D = 0;
      while ((uint64_t(1) << D) < nt) ++D;
      c_id.push_back(ci); c_ntiles.push_back(nt); c_nstarts.push_back(S); c_pairs.push_back(pairs);
      c_first.push_back(n_tiles); c_depth.push_back(D);
      c_start.push_back(e->chr_off[ci]); c_end.push_back(e->chr_off[ci] + L);
      frags_per_sample += pairs;
      heap_base.push_back(heap_total);
      heap_total += uint64_t(2) << D;
      max_depth = std::max(max_depth, D);
      require(uint64_t(n_tiles) + nt < (uint64_t(1) << 31), "too many tiles");
      n_tiles += nt;
    }
    // ---- samples and Euler numbering of normal cells / preneoplastic edge
    const uint32_t N = pl->n_nodes;
    std::vector<pg::SeqSample> samples;
    std::vector<int32_t> sample_src;   // forest sample of each sequenced sample, -1 for the normal one
    std::vector<uint32_t> leaf_tin;
    if (!c->normal_only) {
      double nthr = std::floor((1.0 - c->purity) * 4294967296.0);
      if (nthr > 4294967295.0) nthr = 4294967295.0;
      for (uint32_t s = 0; s < pl->n_samples; ++s) {
        require(!pl->leaves[s].empty(), "sample " + std::to_string(s) + " has no sampled cells");
        pg::SeqSample ss{};
        ss.n_leaves = uint32_t(pl->leaves[s].size());
        ss.leaf_off = uint32_t(leaf_tin.size());
        ss.normal_thr = c->purity >= 1 ? 0u : uint32_t(nthr);
        ss.all_normal = c->purity <= 0 ? 1u : 0u;
        leaf_tin.insert(leaf_tin.end(), pl->leaves[s].begin(), pl->leaves[s].end());
        samples.push_back(ss);
        sample_src.push_back(int32_t(s));
      }
    }
    if (c->normal_only || c->with_normal_sample) {
      pg::SeqSample ss{};
      ss.n_leaves = 0; ss.leaf_off = 0; ss.normal_thr = 0; ss.all_normal = 1;
      samples.push_back(ss);
      sample_src.push_back(-1);
    }
    // ---- with copy-number events: the draws of (start, cell, instance)
    // follow the DNA of the sample's cells.  A cell is normal with
    // probability wn = normal_thr / 2^32 (1 for the normal sample), else one
    // of the sample's nl leaves; leaf class c holds n_c of them.  Over an
    // atom a, option o (the normal cells: class 0; leaf class c) weighs
    // wn * icnt(a, 0) or (1 - wn) / nl * (n_c * icnt(a, c)).  A stretch of
    // starts weighs wn * I0 + (1 - wn) / nl * S, where I0 sums icnt(a, 0) and
    // S sums n_c * icnt(a, c) over its positions (integers, exact); a tile's
    // mass is that expression over the whole tile, accumulated in tile order
    // per chromosome for the split (on the device, seq_tile_mass).
    std::vector<uint32_t> opt_class, opt_leaf_off, opt_nleaf, cls_leaf_tin, opt_cdf;
    std::vector<double> s_wn, s_wt;
    std::vector<uint64_t> s_nl, s_icnt0, s_copy;
    if (pl->has_cna) {
      const size_t NS = samples.size();
      const uint32_t C = pl->n_classes, NA = uint32_t(pl->atom_start_h.size());
      s_icnt0.assign(NS * NA, 0); s_copy.assign(NS * NA, 0);
      for (size_t s = 0; s < NS; ++s) {
        pg::SeqSample& sm = samples[s];
        const double wn = sm.all_normal ? 1.0 : double(sm.normal_thr) * (1.0 / 4294967296.0);
        const double wt = 1.0 - wn;
        // options: the normal cells, then the leaf classes (leaves grouped by class)
        std::map<uint32_t, std::vector<uint32_t>> by_class;
        if (sample_src[s] >= 0 && wt > 0) {
          const auto& lv = pl->leaves[sample_src[s]];
          const auto& lc = pl->leaf_cls[sample_src[s]];
          for (size_t i = 0; i < lv.size(); ++i) by_class[lc[i]].push_back(lv[i]);
        }
        sm.opt_off = uint32_t(opt_class.size());
        sm.n_opt = uint32_t(1 + by_class.size());
        sm.opt_cdf_off = uint32_t(opt_cdf.size());
        opt_class.push_back(0); opt_leaf_off.push_back(0); opt_nleaf.push_back(0);
        uint64_t nl = 0;
        std::vector<std::pair<uint32_t, uint64_t>> ncls;
        for (const auto& kv : by_class) {
          opt_class.push_back(kv.first); opt_leaf_off.push_back(uint32_t(cls_leaf_tin.size()));
          opt_nleaf.push_back(uint32_t(kv.second.size()));
          cls_leaf_tin.insert(cls_leaf_tin.end(), kv.second.begin(), kv.second.end());
          ncls.push_back({kv.first, kv.second.size()});
          nl += kv.second.size();
        }
        // per atom: option thresholds and the integer copy sums
        for (uint32_t a = 0; a < NA; ++a) {
          const uint32_t* ic = &pl->atom_icnt_h[uint64_t(a) * C];
          std::vector<double> w{wn * double(ic[0])};
          uint64_t S = 0;
          for (const auto& [cls, n] : ncls) {
            w.push_back((wt / double(nl)) * double(n * ic[cls]));
            S += n * ic[cls];
          }
          s_icnt0[s * NA + a] = ic[0];
          s_copy[s * NA + a] = S;
          const auto thr = cdf_thresholds(w);
          opt_cdf.insert(opt_cdf.end(), thr.begin(), thr.end());
        }
        s_wn.push_back(wn); s_wt.push_back(wt); s_nl.push_back(nl);
      }
      if (cls_leaf_tin.empty()) cls_leaf_tin.push_back(N);
    }
    if (leaf_tin.empty()) leaf_tin.push_back(N);
    std::vector<uint32_t> etin(N + 2), etout(N + 2);
    for (uint32_t v = 0; v < N; ++v) { etin[v] = pl->tin[v]; etout[v] = pl->tout[v]; }
    etin[N] = 0; etout[N] = c->preneoplastic_in_normal ? N + 1 : N;   // preneoplastic edge
    etin[N + 1] = 0; etout[N + 1] = N + 1;                             // germline
    // ---- device inputs
    auto res = std::make_unique<pg_seq_result>();
    res->eng = e;
    res->n_samples = uint32_t(samples.size());
    res->M = pl->M;
    res->n_reads = frags_per_sample * uint64_t(mates) * samples.size();
    res->tile_size = T;
    res->sample_src = sample_src;
    res->pre_in_normal = c->preneoplastic_in_normal != 0;
    res->alt = DBuf<uint32_t>(P, uint64_t(res->n_samples) * pl->M);
    res->depth = DBuf<uint32_t>(P, uint64_t(res->n_samples) * pl->M);
    ck(cudaMemsetAsync(res->alt.p, 0, sizeof(uint32_t) * res->n_samples * pl->M, st), "memset");
    ck(cudaMemsetAsync(res->depth.p, 0, sizeof(uint32_t) * res->n_samples * pl->M, st), "memset");
    if ((pl->M == 0 && !sam) || n_tiles == 0 || samples.empty()) {
      ck(cudaStreamSynchronize(st), "seq");
      engine_retain(e);
      *out = res.release();
      return;
    }
    auto etin_d = upload(P, etin, st), etout_d = upload(P, etout, st);
    DBuf<uint32_t> ts_d(P, n_tiles), tl_d(P, n_tiles), te_d(P, n_tiles);
    {
      auto cf = upload(P, c_first, st), cn = upload(P, c_ntiles, st), cs = upload(P, c_start, st);
      auto cns = upload(P, c_nstarts, st), cen = upload(P, c_end, st);
      pg::seq_make_tiles(uint32_t(c_first.size()), cf.p, cn.p, cs.p, cns.p, cen.p, T, n_tiles, ts_d.p, tl_d.p,
                         te_d.p, st);
    }
    auto hb_d = upload(P, heap_base, st);
    auto cnt_d = upload(P, c_ntiles, st), cns_d = upload(P, c_nstarts, st), cid_d = upload(P, c_id, st);
    auto cf_d = upload(P, c_first, st), cd_d = upload(P, c_depth, st);
    auto cp_d = upload(P, c_pairs, st);
    auto smp_d = upload(P, samples, st);
    auto leaf_d = upload(P, leaf_tin, st);
    auto ins_d = upload(P, ins_thr, st);
    // guide table of the insert CDF: first index whose threshold exceeds g * 2^23
    std::vector<uint16_t> guide(256);
    for (uint32_t g = 0; g < 256; ++g) {
      const uint32_t v = g << 23;
      const uint32_t k = uint32_t(std::upper_bound(ins_thr.begin(), ins_thr.end(), v) - ins_thr.begin());
      guide[g] = uint16_t(std::min<uint32_t>(k, uint32_t(ins_thr.size()) - 1));
    }
    auto guide_d = upload(P, guide, st);
    DBuf<pg::SeqRec> recs(P, pl->M);
    DBuf<uint32_t> pair_cnt(P, uint64_t(n_tiles) * samples.size()), rlo(P, n_tiles), rhi(P, n_tiles);
    pg::seq_build_records(pl->view(), uint32_t(pl->M), etin_d.p, etout_d.p, recs.p, st);
    DBuf<double> mcum_d, mtot_d;
    DBuf<uint32_t> poff_d, pstart_d, plen_d, patom_d, pcdf_d, ocls_d, oloff_d, onl_d, cltin_d, ocdf_d;
    uint32_t n_parts_cap = 0;
    if (pl->has_cna) {
      const uint32_t NS = uint32_t(samples.size()), NA = uint32_t(pl->atom_start_h.size());
      n_parts_cap = n_tiles + NA;   // each atom boundary splits at most one tile
      poff_d = DBuf<uint32_t>(P, uint64_t(n_tiles) + 1);
      pstart_d = DBuf<uint32_t>(P, n_parts_cap); plen_d = DBuf<uint32_t>(P, n_parts_cap);
      patom_d = DBuf<uint32_t>(P, n_parts_cap); pcdf_d = DBuf<uint32_t>(P, uint64_t(NS) * n_parts_cap);
      DBuf<uint32_t> scan_part(P, pg::scan_part_elems(n_tiles, 1));
      pg::seq_tile_parts(n_tiles, ts_d.p, tl_d.p, pl->atom_start.p, NA, uint32_t(e->G), poff_d.p, scan_part.p,
                         pstart_d.p, plen_d.p, patom_d.p, st);
      auto wn_d = upload(P, s_wn, st), wt_d = upload(P, s_wt, st);
      auto nl_d = upload(P, s_nl, st), i0_d = upload(P, s_icnt0, st), cs_d = upload(P, s_copy, st);
      auto cf_d2 = upload(P, c_first, st), cn_d2 = upload(P, c_ntiles, st);
      mcum_d = DBuf<double>(P, uint64_t(NS) * n_tiles);
      mtot_d = DBuf<double>(P, uint64_t(NS) * c_id.size());
      DBuf<uint64_t> tsums(P, 2 * uint64_t(NS) * n_tiles);
      pg::seq_tile_mass(NS, uint32_t(c_id.size()), cf_d2.p, cn_d2.p, poff_d.p, plen_d.p, patom_d.p, NA, wn_d.p,
                        wt_d.p, nl_d.p, i0_d.p, cs_d.p, n_tiles, n_parts_cap, tsums.p, mcum_d.p, mtot_d.p, pcdf_d.p,
                        st);
      ocls_d = upload(P, opt_class, st); oloff_d = upload(P, opt_leaf_off, st); onl_d = upload(P, opt_nleaf, st);
      cltin_d = upload(P, cls_leaf_tin, st); ocdf_d = upload(P, opt_cdf, st);
    }
    DBuf<uint32_t> heap(P, heap_total * samples.size());
    pg::seq_tile_counts(uint32_t(samples.size()), uint32_t(c_id.size()), max_depth, cf_d.p, cnt_d.p, cd_d.p, cns_d.p,
                        cid_d.p, cp_d.p, hb_d.p, heap_total, heap.p, T, n_tiles, pl->has_cna ? mcum_d.p : nullptr,
                        pl->has_cna ? mtot_d.p : nullptr, seed, pair_cnt.p, st);
    pg::seq_tile_ranges(recs.p, uint32_t(pl->M), ts_d.p, tl_d.p, n_tiles, span, rlo.p, rhi.p, st);
    pg::SeqTiles tiles{n_tiles, ts_d.p, tl_d.p, te_d.p, rlo.p, rhi.p};
    pg::SeqParams prm{};
    prm.read_len = R; prm.paired = paired ? 1u : 0u; prm.span = span;
    prm.ins_min = ins_min; prm.n_ins = uint32_t(ins_thr.size()); prm.ins_cdf = ins_d.p;
    prm.ins_guide = guide_d.p;
    double et = std::floor(c->error_rate * 4294967296.0);
    prm.err_thr = et >= 4294967295.0 ? 0xffffffffu : uint32_t(et);
    pg::err_thirds(prm.err_thr, prm.err_t1, prm.err_t2);
    prm.normal_tin = N;
    prm.n_alleles = 2;
    prm.has_cna = pl->has_cna ? 1u : 0u;
    prm.gc = pl->classes_view();
    prm.chain_off = pl->chain_off.p; prm.chain_anc = pl->chain_anc.p; prm.chain_key = pl->chain_key.p;
    prm.nmask = e->nmask.p;
    if (pl->has_cna) {
      prm.n_classes = pl->n_classes;
      prm.atom_ioff = pl->atom_ioff.p; prm.atom_icnt = pl->atom_icnt.p;
      prm.part_off = poff_d.p; prm.part_start = pstart_d.p; prm.part_len = plen_d.p; prm.part_atom = patom_d.p;
      prm.part_cdf = pcdf_d.p; prm.n_parts = n_parts_cap;
      prm.opt_class = ocls_d.p; prm.opt_leaf_off = oloff_d.p; prm.opt_nleaf = onl_d.p;
      prm.cls_leaf_tin = cltin_d.p; prm.opt_cdf = ocdf_d.p;
    }
    Timer timer(st);
    pg::seq_reads(recs.p, uint32_t(pl->M), tiles, pair_cnt.p, smp_d.p, uint32_t(samples.size()), leaf_d.p, prm, seed,
                  res->alt.p, res->depth.p, st);
    res->kernel_ms = timer.stop();
    ck(cudaGetLastError(), "sequencing kernels");
    if (sam) {
      write_sam(e, pl, *sam, seed, recs.p, tiles, pair_cnt.p, smp_d.p, uint32_t(samples.size()), leaf_d.p, prm, c_id,
                c_first, c_ntiles, c->error_rate);
      ck(cudaGetLastError(), "SAM kernels");
    }
    engine_retain(e);
    *out = res.release();
  }
}

}  // namespace

pg_status pg_seq_result_destroy(pg_seq_result* r) {
  return guarded([&] {
    if (!r) return;
    pg_engine* e = r->eng;
    cudaSetDevice(e->device);
    delete r;
    engine_release(e);
  });
}

pg_status pg_seq_result_dims(const pg_seq_result* r, uint32_t* n_samples, uint64_t* n_mut, uint64_t* n_reads) {
  return guarded([&] {
    require(r != nullptr, "NULL handle");
    if (n_samples) *n_samples = r->n_samples;
    if (n_mut) *n_mut = r->M;
    if (n_reads) *n_reads = r->n_reads;
  });
}

pg_status pg_seq_result_copy(const pg_seq_result* r, int32_t* alt, int32_t* depth) {
  return guarded([&] {
    require(r != nullptr, "NULL handle");
    select_device(r->eng);
    const size_t bytes = sizeof(int32_t) * r->n_samples * r->M;
    if (bytes == 0) return;
    if (alt) ck(cudaMemcpyAsync(alt, r->alt.p, bytes, cudaMemcpyDeviceToHost, r->eng->st), "copy alt");
    if (depth) ck(cudaMemcpyAsync(depth, r->depth.p, bytes, cudaMemcpyDeviceToHost, r->eng->st), "copy depth");
    ck(cudaStreamSynchronize(r->eng->st), "copy");
  });
}

pg_status pg_seq_result_active(pg_seq_result* r, uint64_t* n_active) {
  return guarded([&] {
    require(r != nullptr && n_active != nullptr, "NULL argument");
    select_device(r->eng);
    if (!r->active_done) {
      require(r->M < (uint64_t(1) << 32), "too many mutations for the observed-row tables");
      cudaStream_t st = r->eng->st;
      Pool* P = &r->eng->pool;
      DBuf<uint32_t> pos(P, r->M), part(P, pg::scan_part_elems(r->M, 1)), tot(P, 1);
      pg::seq_active_flags(r->alt.p, r->n_samples, r->M, pos.p, st);
      pg::scan_rows<uint32_t>(pos.p, pos.p, r->M, 1, part.p, tot.p, st);
      uint32_t na = 0;
      ck(cudaMemcpyAsync(&na, tot.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st), "observed rows");
      ck(cudaStreamSynchronize(st), "observed rows");
      r->a_index = DBuf<uint32_t>(P, na);
      r->a_alt = DBuf<uint32_t>(P, uint64_t(na) * r->n_samples);
      r->a_depth = DBuf<uint32_t>(P, uint64_t(na) * r->n_samples);
      pg::seq_active_gather(r->alt.p, r->depth.p, r->n_samples, r->M, pos.p, na, r->a_index.p, r->a_alt.p,
                            r->a_depth.p, st);
      ck(cudaGetLastError(), "observed rows");
      ck(cudaStreamSynchronize(st), "observed rows");
      r->n_active = na;
      r->active_done = true;
    }
    *n_active = r->n_active;
  });
}

pg_status pg_seq_result_copy_active(const pg_seq_result* r, uint32_t* index, int32_t* alt, int32_t* depth) {
  return guarded([&] {
    require(r != nullptr, "NULL handle");
    require(r->active_done, "pg_seq_result_active has not been called on this result");
    select_device(r->eng);
    cudaStream_t st = r->eng->st;
    const uint64_t na = r->n_active, nb = sizeof(uint32_t) * na * r->n_samples;
    if (na == 0) return;
    if (index) ck(cudaMemcpyAsync(index, r->a_index.p, sizeof(uint32_t) * na, cudaMemcpyDeviceToHost, st), "copy");
    if (alt) ck(cudaMemcpyAsync(alt, r->a_alt.p, nb, cudaMemcpyDeviceToHost, st), "copy alt");
    if (depth) ck(cudaMemcpyAsync(depth, r->a_depth.p, nb, cudaMemcpyDeviceToHost, st), "copy depth");
    ck(cudaStreamSynchronize(st), "copy");
  });
}

pg_status pg_seq_result_kernel_ms(const pg_seq_result* r, float* ms) {
  return guarded([&] { require(r && ms, "NULL argument"); *ms = r->kernel_ms; });
}

pg_status pg_seq_result_tile_size(const pg_seq_result* r, uint32_t* tile_size) {
  return guarded([&] { require(r && tile_size, "NULL argument"); *tile_size = r->tile_size; });
}

}  // extern "C"

// ====================================================================== calibration
constexpr uint32_t CALIB_CHUNK = 16384;   // sites per CTA of the site kernel

struct pg_calib {
  int device = 0;
  cudaStream_t st = nullptr, own_st = nullptr;
  Pool pool;
  uint32_t n_rep = 0, K = 0, J = 0, C = 0, P = 0, n_chunks = 0;
  DBuf<int32_t> alt, depth, cls;
  DBuf<uint64_t> site_off, chunk_start;
  DBuf<uint32_t> chunk_rep, rep_first_chunk, step;
  DBuf<float> sig, sig_rows, epoch_w, phi, partial, m, v, tab;
  std::vector<uint32_t> rep_first_chunk_h;
  uint32_t part_stride = 0, tab_stride = 0;
  cudaGraphExec_t graph = nullptr;
  struct { float* params = nullptr; uint32_t steps = 0; float lr = 0, b1 = 0, b2 = 0, eps = 0; float* nll = nullptr; cudaStream_t st = nullptr; } gkey;
  pg::CalibArgs args() const {
    pg::CalibArgs a{};
    a.K = K; a.J = J; a.C = C; a.P = P;
    a.alt = alt.p; a.depth = depth.p; a.cls = cls.p; a.site_off = site_off.p;
    a.sig = sig.p; a.epoch_w = epoch_w.p; a.phi = phi.p;
    a.chunk = CALIB_CHUNK; a.part_stride = part_stride;
    a.sig_rows = sig_rows.p; a.tab = tab.p; a.tab_stride = tab_stride;
    return a;
  }
  ~pg_calib() {
    if (graph) cudaGraphExecDestroy(graph);
    alt.reset(); depth.reset(); cls.reset(); site_off.reset(); chunk_start.reset(); chunk_rep.reset();
    rep_first_chunk.reset(); step.reset(); sig.reset(); epoch_w.reset(); phi.reset(); partial.reset(); m.reset();
    v.reset(); tab.reset(); sig_rows.reset();
    pool.release_all();
    if (own_st) cudaStreamDestroy(own_st);
  }
};

extern "C" {

pg_status pg_calib_create(uint32_t n_rep, const uint64_t* site_off, const int32_t* alt, const int32_t* depth,
                          const int32_t* cls, uint32_t K, uint32_t J, uint32_t C, const double* signatures,
                          const double* epoch_weight, const double* phi, pg_calib** out) {
  return guarded([&] {
    require(out && site_off && signatures && epoch_weight && phi, "NULL argument");
    require(n_rep >= 1, "at least one replicate");
    require(K >= 1 && K <= 8 && J >= 1 && J <= 8 && C >= 1 && C <= 128, "K and J in [1, 8], C in [1, 128]");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { cudaGetLastError(); throw CudaError("no CUDA device"); }
    const uint64_t n = site_off[n_rep];
    require(site_off[0] == 0, "site offsets start at 0");
    for (uint32_t r = 0; r < n_rep; ++r) require(site_off[r + 1] >= site_off[r], "site offsets must not decrease");
    require(n == 0 || (alt && depth && cls), "NULL site arrays");
    for (uint64_t i = 0; i < n; ++i) {
      require(depth[i] >= 0 && alt[i] >= 0 && alt[i] <= depth[i], "sites need 0 <= alt <= depth");
      require(cls[i] >= 0 && uint32_t(cls[i]) < C, "site class out of range");
    }
    for (uint64_t x = 0; x < uint64_t(J) * C; ++x) require(signatures[x] >= 0, "signature probabilities >= 0");
    for (uint64_t x = 0; x < uint64_t(n_rep) * K; ++x) {
      require(epoch_weight[x] > 0, "epoch weights must be positive");
      require(phi[x] > 0 && phi[x] <= 1, "phi must be in (0, 1]");
    }
    auto c = std::make_unique<pg_calib>();
    ck(cudaGetDevice(&c->device), "cudaGetDevice");
    ck(cudaStreamCreateWithFlags(&c->own_st, cudaStreamNonBlocking), "stream");
    c->st = c->own_st;
    c->n_rep = n_rep; c->K = K; c->J = J; c->C = C; c->P = K + K * J + 1;
    Pool* P = &c->pool;
    cudaStream_t st = c->st;
    std::vector<int32_t> va(alt, alt + n), vd(depth, depth + n), vc(cls, cls + n);
    c->alt = upload(P, va, st); c->depth = upload(P, vd, st); c->cls = upload(P, vc, st);
    c->site_off = upload(P, std::vector<uint64_t>(site_off, site_off + n_rep + 1), st);
    std::vector<float> fs(uint64_t(J) * C), fw(uint64_t(n_rep) * K), fp(uint64_t(n_rep) * K);
    for (uint32_t j = 0; j < J; ++j) {   // signatures normalised to sum 1 over the classes
      double tot = 0;
      for (uint32_t k = 0; k < C; ++k) tot += signatures[uint64_t(j) * C + k];
      require(tot > 0, "a signature has no mass");
      for (uint32_t k = 0; k < C; ++k) fs[uint64_t(j) * C + k] = float(signatures[uint64_t(j) * C + k] / tot);
    }
    for (uint64_t x = 0; x < fw.size(); ++x) { fw[x] = float(epoch_weight[x]); fp[x] = float(phi[x]); }
    c->sig = upload(P, fs, st); c->epoch_w = upload(P, fw, st); c->phi = upload(P, fp, st);
    {   // signatures by class, rows of 4 or 8 floats
      const uint32_t JP = J > 4 ? 8 : 4;
      std::vector<float> rows(size_t(C) * JP, 0.f);
      for (uint32_t j = 0; j < J; ++j)
        for (uint32_t cl = 0; cl < C; ++cl) rows[size_t(cl) * JP + j] = fs[size_t(j) * C + cl];
      c->sig_rows = upload(P, rows, st);
    }
    // chunks of CALIB_CHUNK sites, never across replicates
    std::vector<uint32_t> crep;
    std::vector<uint64_t> cstart;
    c->rep_first_chunk_h.assign(n_rep + 1, 0);
    for (uint32_t r = 0; r < n_rep; ++r) {
      c->rep_first_chunk_h[r] = uint32_t(crep.size());
      for (uint64_t i = site_off[r]; i < site_off[r + 1]; i += CALIB_CHUNK) { crep.push_back(r); cstart.push_back(i); }
    }
    c->rep_first_chunk_h[n_rep] = uint32_t(crep.size());
    c->n_chunks = uint32_t(crep.size());
    c->chunk_rep = upload(P, crep, st); c->chunk_start = upload(P, cstart, st);
    c->rep_first_chunk = upload(P, c->rep_first_chunk_h, st);
    c->part_stride = (1 + 3 * K + K * J + 3) & ~3u;
    // per replicate: log(exp(lr_k) L_k / Z), log v_k, log(1 - v_k) (K each), w_kj (K J)
    c->tab_stride = (3 * K + K * J + 3) & ~3u;
    c->tab = DBuf<float>(P, uint64_t(n_rep) * c->tab_stride);
    c->partial = DBuf<float>(P, uint64_t(std::max<uint32_t>(c->n_chunks, 1)) * c->part_stride);
    c->m = DBuf<float>(P, uint64_t(n_rep) * c->P);
    c->v = DBuf<float>(P, uint64_t(n_rep) * c->P);
    c->step = DBuf<uint32_t>(P, n_rep);
    ck(cudaStreamSynchronize(st), "calibration upload");
    *out = c.release();
  });
}

pg_status pg_calib_destroy(pg_calib* c) {
  return guarded([&] { if (c) { cudaSetDevice(c->device); delete c; } });
}

pg_status pg_calib_num_params(const pg_calib* c, uint32_t* P) {
  return guarded([&] { require(c && P, "NULL argument"); *P = c->P; });
}

pg_status pg_calib_set_stream(pg_calib* c, void* stream) {
  return guarded([&] {
    require(c != nullptr, "NULL handle");
    ck(cudaSetDevice(c->device), "cudaSetDevice");
    ck(cudaStreamSynchronize(c->st), "stream switch");
    c->st = stream ? static_cast<cudaStream_t>(stream) : c->own_st;
  });
}

pg_status pg_calib_nll_grad(pg_calib* c, const float* params, float* nll, float* grad) {
  return guarded([&] {
    require(c && params, "NULL argument");
    ck(cudaSetDevice(c->device), "cudaSetDevice");
    pg::AdamArgs no{};
    pg::calib_launch(c->args(), const_cast<float*>(params), c->chunk_rep.p, c->chunk_start.p, c->n_chunks,
                     c->rep_first_chunk.p, c->n_rep, c->partial.p, nll, grad, no, c->st);
    ck(cudaGetLastError(), "calibration kernels");
  });
}

pg_status pg_calib_nll_grad_one(pg_calib* c, uint32_t rep, const float* params, float* nll, float* grad) {
  return guarded([&] {
    require(c && params, "NULL argument");
    require(rep < c->n_rep, "replicate out of range");
    ck(cudaSetDevice(c->device), "cudaSetDevice");
    pg::CalibArgs a = c->args();
    a.chunk0 = c->rep_first_chunk_h[rep];
    a.rep0 = rep;
    pg::AdamArgs no{};
    pg::calib_launch(a, const_cast<float*>(params), c->chunk_rep.p, c->chunk_start.p,
                     c->rep_first_chunk_h[rep + 1] - c->rep_first_chunk_h[rep], c->rep_first_chunk.p, 1,
                     c->partial.p, nll, grad, no, c->st);
    ck(cudaGetLastError(), "calibration kernels");
  });
}

pg_status pg_calib_adam(pg_calib* c, float* params, uint32_t steps, float lr, float beta1, float beta2, float eps,
                        float* nll) {
  return guarded([&] {
    require(c && params, "NULL argument");
    require(steps >= 1 && steps <= 100000, "steps in [1, 100000]");
    require(lr > 0 && beta1 >= 0 && beta1 < 1 && beta2 >= 0 && beta2 < 1 && eps > 0, "invalid Adam hyperparameters");
    ck(cudaSetDevice(c->device), "cudaSetDevice");
    cudaStream_t st = c->st;
    ck(cudaMemsetAsync(c->m.p, 0, sizeof(float) * c->n_rep * c->P, st), "memset");
    ck(cudaMemsetAsync(c->v.p, 0, sizeof(float) * c->n_rep * c->P, st), "memset");
    ck(cudaMemsetAsync(c->step.p, 0, sizeof(uint32_t) * c->n_rep, st), "memset");
    const bool same = c->graph && c->gkey.params == params && c->gkey.steps == steps && c->gkey.lr == lr &&
                      c->gkey.b1 == beta1 && c->gkey.b2 == beta2 && c->gkey.eps == eps && c->gkey.nll == nll &&
                      c->gkey.st == st;
    if (!same) {
      if (c->graph) { cudaGraphExecDestroy(c->graph); c->graph = nullptr; }
      pg::AdamArgs ad{c->m.p, c->v.p, c->step.p, lr, beta1, beta2, eps};
      cudaGraph_t g = nullptr;
      const uint64_t counted = g_launches.load();   // captured kernels are not launches yet
      ck(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin capture");
      for (uint32_t s = 0; s < steps; ++s)
        pg::calib_launch(c->args(), params, c->chunk_rep.p, c->chunk_start.p, c->n_chunks, c->rep_first_chunk.p,
                         c->n_rep, c->partial.p, s + 1 == steps ? nll : nullptr, nullptr, ad, st);
      const cudaError_t ce = cudaStreamEndCapture(st, &g);
      ck(ce, "end capture");
      const cudaError_t ie = cudaGraphInstantiate(&c->graph, g, 0);
      cudaGraphDestroy(g);
      ck(ie, "graph instantiate");
      c->gkey = {params, steps, lr, beta1, beta2, eps, nll, st};
      g_launches.store(counted);
    }
    ck(cudaGraphLaunch(c->graph, st), "graph launch");
    pg::note_launch(2 * steps);
    ck(cudaGetLastError(), "calibration graph");
  });
}

}  // extern "C"

#include "pg_batch_impl.h"
#include "pg_frames_impl.h"
#include "pg_archive_impl.h"
#include "pg_inputs_impl.h"
