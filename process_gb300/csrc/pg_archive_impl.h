// The placed-forest archive (PhylogeneticForest$save / load_phylogenetic_forest,
// src/phylogenetic_forest.cpp:940-992, src/mutations.cpp:1466-1480).  The
// reference writes the RACES archive of its forest; RACES is not available,
// so this is a versioned native layout of everything a placed-forest handle
// holds: the forest's Euler numbering and samples, the placed mutations, the
// genotype classes and allele-instance lineage and the applied CNA events.
// Loading restores the handle without placing again, on an engine whose
// genome matches the archive's fingerprint.  Included by pg_api.cpp.
//
// Layout (little-endian): "PGPF", version (u32), then sections, each vector
// as its u64 element count and raw elements, and "FPGP" at the end.

namespace {

constexpr uint32_t ARCHIVE_VERSION = 1;

struct Writer {
  std::vector<uint8_t> b;
  void raw(const void* p, size_t n) { const uint8_t* c = static_cast<const uint8_t*>(p); b.insert(b.end(), c, c + n); }
  template <class T> void put(T v) { raw(&v, sizeof(T)); }
  template <class T> void vec(const std::vector<T>& v) { put<uint64_t>(v.size()); if (!v.empty()) raw(v.data(), sizeof(T) * v.size()); }
};

struct Reader {
  const uint8_t* p;
  size_t n, at = 0;
  void raw(void* dst, size_t k) {
    if (k > n - at) throw DomainError("the phylogenetic forest archive is truncated");
    std::memcpy(dst, p + at, k);
    at += k;
  }
  template <class T> T get() { T v; raw(&v, sizeof(T)); return v; }
  template <class T> std::vector<T> vec() {
    const uint64_t k = get<uint64_t>();
    if (k > (n - at) / sizeof(T)) throw DomainError("the phylogenetic forest archive is truncated");
    std::vector<T> v(k);
    if (k) raw(v.data(), sizeof(T) * k);
    return v;
  }
};

template <class T>
std::vector<T> download(const DBuf<T>& d, uint64_t n) {
  std::vector<T> v(n);
  if (n) ck(cudaMemcpy(v.data(), d.p, sizeof(T) * n, cudaMemcpyDeviceToHost), "download");
  return v;
}

std::vector<uint8_t> placed_serialize(const pg_placed* p) {
  const pg_engine* e = p->eng;
  Writer w;
  w.raw("PGPF", 4);
  w.put<uint32_t>(ARCHIVE_VERSION);
  w.put<uint64_t>(genome_fingerprint(e));
  w.put<uint64_t>(e->G);
  // forest
  w.put<uint32_t>(p->n_nodes); w.put<uint32_t>(p->n_samples);
  w.vec(p->tin); w.vec(p->tout); w.vec(p->parent);
  w.put<uint64_t>(p->leaves.size());
  for (const auto& v : p->leaves) w.vec(v);
  // placed mutations
  w.put<uint64_t>(p->M);
  w.vec(download(p->locus, p->M)); w.vec(download(p->edge, p->M)); w.vec(download(p->aux, p->M));
  w.vec(download(p->cls, p->M)); w.vec(download(p->sig, p->M)); w.vec(download(p->kind, p->M));
  w.vec(download(p->nature, p->M)); w.vec(download(p->allele, p->M)); w.vec(download(p->seq, p->M));
  // genotype classes and lineage
  w.put<uint8_t>(p->has_cna ? 1 : 0); w.put<uint32_t>(p->cn_max); w.put<uint32_t>(p->n_classes);
  w.vec(p->node_class_h);
  w.put<uint64_t>(p->leaf_cls.size());
  for (const auto& v : p->leaf_cls) w.vec(v);
  w.vec(p->atom_start_h); w.vec(p->atom_icnt_h);
  w.vec(download(p->atom_ioff, p->atom_icnt_h.size()));
  w.vec(p->seg_off_h); w.vec(p->seg_start_h); w.vec(p->seg_end_h); w.vec(p->seg_ioff_h); w.vec(p->seg_icnt_h);
  w.vec(p->inst_list_h); w.vec(p->chain_off_h); w.vec(p->chain_anc_h); w.vec(p->chain_key_h); w.vec(p->inst_root_h);
  // CNA events
  w.put<uint64_t>(p->cnas.size());
  for (const CnaOut& c : p->cnas) {
    w.put(c.node); w.put(c.type); w.put(c.chr); w.put(c.begin); w.put(c.end); w.put(c.allele); w.put(c.src);
    w.put(c.driver);
  }
  w.raw("FPGP", 4);
  return std::move(w.b);
}

std::unique_ptr<pg_placed> placed_deserialize(pg_engine* e, const uint8_t* buf, size_t n) {
  Reader r{buf, n};
  char magic[4];
  r.raw(magic, 4);
  if (std::memcmp(magic, "PGPF", 4) != 0) throw DomainError("not a phylogenetic forest archive");
  const uint32_t version = r.get<uint32_t>();
  if (version != ARCHIVE_VERSION)
    throw DomainError("the archive has format version " + std::to_string(version) + ", this library reads version " +
                      std::to_string(ARCHIVE_VERSION));
  const uint64_t fp = r.get<uint64_t>(), G = r.get<uint64_t>();
  if (G != e->G || fp != genome_fingerprint(e))
    throw DomainError("the archive was saved with another reference genome than the engine's");
  cudaStream_t st = e->st;
  Pool* P = &e->pool;
  auto p = std::make_unique<pg_placed>();
  p->eng = e;
  p->n_nodes = r.get<uint32_t>(); p->n_samples = r.get<uint32_t>();
  p->tin = r.vec<uint32_t>(); p->tout = r.vec<uint32_t>(); p->parent = r.vec<int32_t>();
  if (p->tin.size() != p->n_nodes || p->tout.size() != p->n_nodes || p->parent.size() != p->n_nodes)
    throw DomainError("the phylogenetic forest archive is inconsistent");
  p->leaves.resize(r.get<uint64_t>());
  for (auto& v : p->leaves) v = r.vec<uint32_t>();
  p->M = r.get<uint64_t>();
  auto up = [&](auto& dbuf, const auto& v) {
    if (v.size() != p->M) throw DomainError("the phylogenetic forest archive is inconsistent");
    dbuf = upload(P, v, st);
  };
  up(p->locus, r.vec<uint32_t>()); up(p->edge, r.vec<uint32_t>()); up(p->aux, r.vec<uint32_t>());
  up(p->cls, r.vec<uint8_t>()); up(p->sig, r.vec<uint8_t>()); up(p->kind, r.vec<uint8_t>());
  up(p->nature, r.vec<uint8_t>()); up(p->allele, r.vec<uint16_t>()); up(p->seq, r.vec<uint16_t>());
  p->attempt = DBuf<uint32_t>(P, p->M);
  p->has_cna = r.get<uint8_t>() != 0; p->cn_max = r.get<uint32_t>(); p->n_classes = r.get<uint32_t>();
  p->node_class_h = r.vec<uint32_t>();
  p->leaf_cls.resize(r.get<uint64_t>());
  for (auto& v : p->leaf_cls) v = r.vec<uint32_t>();
  p->atom_start_h = r.vec<uint32_t>(); p->atom_icnt_h = r.vec<uint32_t>();
  const auto atom_ioff = r.vec<uint32_t>();
  p->seg_off_h = r.vec<uint32_t>(); p->seg_start_h = r.vec<uint32_t>(); p->seg_end_h = r.vec<uint32_t>();
  p->seg_ioff_h = r.vec<uint32_t>(); p->seg_icnt_h = r.vec<uint32_t>();
  p->inst_list_h = r.vec<uint16_t>(); p->chain_off_h = r.vec<uint32_t>(); p->chain_anc_h = r.vec<uint16_t>();
  p->chain_key_h = r.vec<uint64_t>(); p->inst_root_h = r.vec<uint8_t>();
  p->cnas.resize(r.get<uint64_t>());
  for (CnaOut& c : p->cnas) {
    c.node = r.get<uint32_t>(); c.type = r.get<uint8_t>(); c.chr = r.get<uint32_t>(); c.begin = r.get<uint32_t>();
    c.end = r.get<uint32_t>(); c.allele = r.get<uint32_t>(); c.src = r.get<uint32_t>(); c.driver = r.get<uint8_t>();
  }
  r.raw(magic, 4);
  if (std::memcmp(magic, "FPGP", 4) != 0 || r.at != n)
    throw DomainError("the phylogenetic forest archive is inconsistent");
  if (p->node_class_h.size() < p->n_nodes || atom_ioff.size() != p->atom_icnt_h.size())
    throw DomainError("the phylogenetic forest archive is inconsistent");
  // device copies, as place_mutations leaves them
  p->node_class = upload(P, p->node_class_h, st);
  if (!p->atom_start_h.empty()) {
    p->atom_start = upload(P, p->atom_start_h, st);
    p->atom_ioff = upload(P, atom_ioff, st);
    p->atom_icnt = upload(P, p->atom_icnt_h, st);
  }
  p->seg_off = upload(P, p->seg_off_h, st); p->seg_start = upload(P, p->seg_start_h, st);
  p->seg_end = upload(P, p->seg_end_h, st); p->seg_ioff = upload(P, p->seg_ioff_h, st);
  p->seg_icnt = upload(P, p->seg_icnt_h, st);
  std::vector<uint16_t> il = p->inst_list_h, ca = p->chain_anc_h;
  std::vector<uint64_t> ckey = p->chain_key_h;
  if (il.empty()) il.push_back(0);
  if (ca.empty()) { ca.push_back(0); ckey.push_back(0); }
  p->inst_list = upload(P, il, st);
  p->chain_off = upload(P, p->chain_off_h, st); p->chain_anc = upload(P, ca, st); p->chain_key = upload(P, ckey, st);
  ck(cudaStreamSynchronize(st), "archive upload");
  return p;
}

}  // namespace

extern "C" {

pg_status pg_placed_serialize(const pg_placed* p, uint8_t* buf, uint64_t capacity, uint64_t* size) {
  return guarded([&] {
    require(p && size, "NULL argument");
    select_device(p->eng);
    const auto b = placed_serialize(p);
    *size = b.size();
    if (buf) {
      require(capacity >= b.size(), "archive buffer too small");
      std::memcpy(buf, b.data(), b.size());
    }
  });
}

pg_status pg_placed_deserialize(pg_engine* e, const uint8_t* buf, uint64_t size, pg_placed** out) {
  return guarded([&] {
    require(e && buf && out, "NULL argument");
    select_device(e);
    auto p = placed_deserialize(e, buf, size);
    engine_retain(e);
    *out = p.release();
  });
}

pg_status pg_placed_save(const pg_placed* p, const char* path) {
  return guarded([&] {
    require(p && path, "NULL argument");
    select_device(p->eng);
    const auto b = placed_serialize(p);
    std::ofstream f(path, std::ios::binary | std::ios::trunc);
    if (!f) throw std::runtime_error(std::string("cannot write \"") + path + "\"");
    f.write(reinterpret_cast<const char*>(b.data()), std::streamsize(b.size()));
    if (!f) throw std::runtime_error(std::string("cannot write \"") + path + "\"");
  });
}

pg_status pg_placed_load(pg_engine* e, const char* path, pg_placed** out) {
  return guarded([&] {
    require(e && path && out, "NULL argument");
    namespace fs = std::filesystem;
    if (!fs::exists(path)) throw DomainError(std::string("The file \"") + path + "\" does not exist.");
    if (!fs::is_regular_file(path)) throw DomainError(std::string("The file \"") + path + "\" is not a regular file.");
    std::ifstream f(path, std::ios::binary);
    std::vector<uint8_t> b((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    select_device(e);
    auto p = placed_deserialize(e, b.data(), b.size());
    engine_retain(e);
    *out = p.release();
  });
}

}  // extern "C"
