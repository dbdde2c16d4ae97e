// The output contract: the data frames of ProCESS's PhylogeneticForest
// getters and of simulate_seq, built here from the placed tables, so that a
// caller (the Rcpp layer) only turns columns into data frames.  Included by
// pg_api.cpp after the handle definitions.
//
//   sampled-cell mutations     src/phylogenetic_forest.cpp:452-507 (rows of a
//                              cell nested chromosome -> allele -> position as
//                              fill_mutation_lists walks them, :323-351)
//   sampled-cell CNAs          :509-562
//   allelic fragmentation      cells :867-927, bulk :767-820
//   samples' DNA quantity      :57-99
//   the result data frame      src/seq_simulation.cpp:52-181
//
// Row identifiers are node ids (cells) and row indices of pg_placed_copy
// (mutations); the caller maps them to cell ids and to the mutation columns
// of pg_placed_mutation_info.

namespace {

// rethrows the failure of a nested C-ABI call with its own status
void check_status(pg_status st) {
  if (st == PG_OK) return;
  const std::string msg = g_last_error;
  if (st == PG_ERR_DOMAIN) throw DomainError(msg);
  if (st == PG_ERR_CUDA) throw CudaError(msg);
  if (st == PG_ERR_NOMEM) throw NoMem(msg);
  throw std::runtime_error(msg);
}

// ref / alt string of a row-info code: up to 8 characters of "ACGNT"
void sid_string(uint32_t code, char* out) {
  static const char ch[6] = {0, 'A', 'C', 'G', 'N', 'T'};
  uint32_t n = 0;
  for (; n < 8; ++n) {
    const uint32_t c = (code >> (28 - 4 * n)) & 15u;
    if (c == 0 || c > 5) break;
    out[n] = ch[c];
  }
  for (; n < PG_SID_CHARS; ++n) out[n] = 0;
}

// per-row info of placed mutations rows (host indices; NULL = rows 0..n-1)
std::vector<uint4> placed_row_info(const pg_placed* p, uint64_t n, const uint32_t* rows) {
  pg_engine* e = p->eng;
  cudaStream_t st = e->st;
  Pool* P = &e->pool;
  std::vector<uint4> out(n);
  if (n == 0) return out;
  DBuf<uint32_t> rd;
  if (rows) {
    for (uint64_t i = 0; i < n; ++i) require(rows[i] < p->M, "mutation row out of range");
    rd = DBuf<uint32_t>(P, n);
    ck(cudaMemcpyAsync(rd.p, rows, sizeof(uint32_t) * n, cudaMemcpyHostToDevice, st), "upload");
  } else {
    require(n <= p->M, "more rows than placed mutations");
  }
  DBuf<uint4> od(P, n);
  pg::row_info(p->locus.p, p->aux.p, p->kind.p, p->sig.p, p->nature.p, rows ? rd.p : nullptr, n, e->genome.p,
               e->nmask.p, e->G, od.p, st);
  ck(cudaMemcpyAsync(out.data(), od.p, sizeof(uint4) * n, cudaMemcpyDeviceToHost, st), "download");
  ck(cudaStreamSynchronize(st), "row info");
  return out;
}

uint32_t chr_of(const pg_engine* e, uint32_t locus) {
  return uint32_t(std::upper_bound(e->chr_off.begin(), e->chr_off.end(), locus) - e->chr_off.begin()) - 1;
}

// node id of every Euler index
std::vector<uint32_t> node_of_tin(const pg_placed* p) {
  std::vector<uint32_t> v(p->n_nodes);
  for (uint32_t u = 0; u < p->n_nodes; ++u) v[p->tin[u]] = u;
  return v;
}

// the cells a getter covers: the given node ids (each a leaf), or every
// sampled leaf by ascending node id
std::vector<uint32_t> getter_cells(const pg_placed* p, uint32_t n_cells, const uint32_t* cells) {
  std::vector<uint32_t> out;
  if (cells) {
    for (uint32_t i = 0; i < n_cells; ++i) {
      require(cells[i] < p->n_nodes, "cell node out of range");
      require(p->tout[cells[i]] == p->tin[cells[i]] + 1, "Cell " + std::to_string(cells[i]) + " is not a leaf");
      out.push_back(cells[i]);
    }
    return out;
  }
  const auto node = node_of_tin(p);
  for (const auto& lv : p->leaves) for (uint32_t t : lv) out.push_back(node[t]);
  std::sort(out.begin(), out.end());
  out.erase(std::unique(out.begin(), out.end()), out.end());
  return out;
}

// class size (allelic size of a genome of that class) and, per class
// segment, copies of germline allele 0 and 1
struct ClassView {
  const pg_placed* p;
  uint32_t n_classes() const { return p->has_cna ? p->n_classes : 1u; }
  bool plain() const { return !p->has_cna || p->seg_off_h.empty(); }
  uint64_t size(uint32_t c) const {
    if (plain()) return 2 * p->eng->G;
    uint64_t s = 0;
    for (uint32_t k = p->seg_off_h[c]; k < p->seg_off_h[c + 1]; ++k)
      s += uint64_t(p->seg_end_h[k] - p->seg_start_h[k]) * p->seg_icnt_h[k];
    return s;
  }
  void copies(uint32_t k, uint32_t& a0, uint32_t& a1) const {
    a1 = 0;
    for (uint32_t q = 0; q < p->seg_icnt_h[k]; ++q) a1 += p->inst_root_h[p->inst_list_h[p->seg_ioff_h[k] + q]];
    a0 = p->seg_icnt_h[k] - a1;
  }
};

// Stretches of one allelic type (copies of germline alleles 0 and 1) of a
// genome of class c, chromosome by chromosome; uncovered stretches have type
// (0, 0).  Absolute half-open intervals.
struct Frag { uint32_t begin, end, a0, a1; };
std::vector<Frag> class_fragments(const pg_placed* p, uint32_t c) {
  const pg_engine* e = p->eng;
  const ClassView cv{p};
  std::vector<Frag> out;
  if (cv.plain()) {
    for (uint32_t k = 0; k < e->n_chr; ++k) out.push_back({e->chr_off[k], e->chr_off[k + 1], 1, 1});
    return out;
  }
  std::vector<uint32_t> cuts(e->chr_off.begin(), e->chr_off.end());
  const uint32_t lo = p->seg_off_h[c], hi = p->seg_off_h[c + 1];
  for (uint32_t k = lo; k < hi; ++k) { cuts.push_back(p->seg_start_h[k]); cuts.push_back(p->seg_end_h[k]); }
  std::sort(cuts.begin(), cuts.end());
  cuts.erase(std::unique(cuts.begin(), cuts.end()), cuts.end());
  for (size_t i = 0; i + 1 < cuts.size(); ++i) {
    const uint32_t b = cuts[i], en = cuts[i + 1];
    uint32_t a0 = 0, a1 = 0;
    // the segment covering b (segments of a class are disjoint and ascending)
    const auto it = std::upper_bound(p->seg_start_h.begin() + lo, p->seg_start_h.begin() + hi, b);
    if (it != p->seg_start_h.begin() + lo) {
      const uint32_t k = uint32_t(it - p->seg_start_h.begin()) - 1;
      if (b < p->seg_end_h[k]) cv.copies(k, a0, a1);
    }
    if (!out.empty() && out.back().end == b && out.back().a0 == a0 && out.back().a1 == a1 &&
        chr_of(e, out.back().begin) == chr_of(e, b))
      out.back().end = en;
    else
      out.push_back({b, en, a0, a1});
  }
  return out;
}

// does allele instance y carry a mutation placed on instance x with order
// key km?  (x itself, or a copy of it made after the mutation)
bool instance_carries(const pg_placed* p, uint32_t y, uint32_t x, uint64_t km) {
  if (y == x) return true;
  if (p->chain_off_h.empty() || y + 1 >= p->chain_off_h.size()) return false;
  for (uint32_t q = p->chain_off_h[y]; q < p->chain_off_h[y + 1]; ++q)
    if (p->chain_anc_h[q] == x) return p->chain_key_h[q] > km;
  return false;
}

}  // namespace

extern "C" {

pg_status pg_engine_set_signature_names(pg_engine* e, int type, uint32_t n, const char* const* names) {
  return guarded([&] {
    require(e && names, "NULL argument");
    require(type == 0 || type == 1, "type must be 0 (SBS) or 1 (ID)");
    require(n == e->n_sig[type], "one name per signature of the type is needed");
    std::vector<std::string> v;
    for (uint32_t i = 0; i < n; ++i) {
      require(names[i] != nullptr && names[i][0] != 0, "empty signature name");
      v.emplace_back(names[i]);
    }
    e->sig_names[type] = std::move(v);
  });
}

pg_status pg_engine_signature_name(const pg_engine* e, int type, uint32_t index, char* out, uint32_t capacity,
                                   uint32_t* length) {
  return guarded([&] {
    require(e != nullptr, "NULL handle");
    require(type == 0 || type == 1, "type must be 0 (SBS) or 1 (ID)");
    require(index < e->n_sig[type], "signature index out of range");
    const std::string name = index < e->sig_names[type].size()
                                 ? e->sig_names[type][index]
                                 : std::string(type == 0 ? "SBS#" : "ID#") + std::to_string(index + 1);
    if (length) *length = uint32_t(name.size());
    if (out && capacity) {
      const size_t k = std::min<size_t>(name.size(), capacity - 1);
      std::memcpy(out, name.data(), k);
      out[k] = 0;
    }
  });
}

pg_status pg_placed_mutation_info(const pg_placed* p, uint64_t n, const uint32_t* rows, uint32_t* chr,
                                  uint32_t* chr_pos, char* ref, char* alt, uint8_t* kind, int32_t* cause,
                                  uint8_t* nature) {
  return guarded([&] {
    require(p != nullptr, "NULL handle");
    select_device(p->eng);
    const auto info = placed_row_info(p, n, rows);
    const pg_engine* e = p->eng;
    for (uint64_t i = 0; i < n; ++i) {
      const uint4 r = info[i];
      const uint32_t c = chr_of(e, r.x), k = r.w & 0xffu, sg = (r.w >> 8) & 0xffu;
      if (chr) chr[i] = c;
      if (chr_pos) chr_pos[i] = r.x - e->chr_off[c] + 1;
      if (ref) sid_string(r.y, ref + i * PG_SID_CHARS);
      if (alt) sid_string(r.z, alt + i * PG_SID_CHARS);
      if (kind) kind[i] = uint8_t(k);
      if (cause) cause[i] = (sg == 0xffu || k > 1 || sg >= e->n_sig[k]) ? -1 : int32_t(sg);
      if (nature) nature[i] = uint8_t(r.w >> 16);
    }
  });
}

pg_status pg_placed_cell_mutations(pg_placed* p, uint32_t n_cells, const uint32_t* cells, uint64_t* n_rows) {
  return guarded([&] {
    require(p != nullptr && n_rows != nullptr, "NULL argument");
    select_device(p->eng);
    const std::vector<uint32_t> cs = getter_cells(p, n_cells, cells);
    p->cm_cell.clear(); p->cm_row.clear(); p->cm_allele.clear();
    const uint32_t N = p->n_nodes;
    const pg_engine* e = p->eng;
    // the placed columns on the host, and the rows of every edge
    std::vector<uint32_t> locus(p->M), edge(p->M);
    std::vector<uint16_t> allele(p->M), seq(p->M);
    if (p->M) {
      cudaStream_t st = e->st;
      ck(cudaMemcpyAsync(locus.data(), p->locus.p, 4 * p->M, cudaMemcpyDeviceToHost, st), "copy");
      ck(cudaMemcpyAsync(edge.data(), p->edge.p, 4 * p->M, cudaMemcpyDeviceToHost, st), "copy");
      ck(cudaMemcpyAsync(allele.data(), p->allele.p, 2 * p->M, cudaMemcpyDeviceToHost, st), "copy");
      ck(cudaMemcpyAsync(seq.data(), p->seq.p, 2 * p->M, cudaMemcpyDeviceToHost, st), "copy");
      ck(cudaStreamSynchronize(st), "copy");
    }
    std::vector<uint64_t> eoff(N + 3, 0);
    for (uint64_t m = 0; m < p->M; ++m) ++eoff[std::min<uint32_t>(edge[m], N + 1) + 1];
    for (uint32_t k = 0; k < N + 2; ++k) eoff[k + 1] += eoff[k];
    std::vector<uint32_t> erows(p->M);
    {
      std::vector<uint64_t> fill(eoff.begin(), eoff.end() - 1);
      for (uint64_t m = 0; m < p->M; ++m) erows[fill[std::min<uint32_t>(edge[m], N + 1)]++] = uint32_t(m);
    }
    const bool copies = p->has_cna && !p->seg_off_h.empty();
    struct Row { uint32_t chr, allele, locus, row; };
    std::vector<Row> rows;
    for (uint32_t v : cs) {
      rows.clear();
      auto take = [&](uint32_t ed) {
        for (uint64_t q = eoff[ed]; q < eoff[ed + 1]; ++q) {
          const uint32_t m = erows[q], L = locus[m], x = allele[m];
          if (!copies) { rows.push_back({chr_of(e, L), x, L, m}); continue; }
          const uint64_t km = (uint64_t(ed < N ? p->tin[ed] : 0u) << 16) | (seq[m] & 0x7fffu);
          const uint32_t c = p->node_class_h[v];
          const uint32_t lo = p->seg_off_h[c], hi = p->seg_off_h[c + 1];
          const auto it = std::upper_bound(p->seg_start_h.begin() + lo, p->seg_start_h.begin() + hi, L);
          if (it == p->seg_start_h.begin() + lo) continue;
          const uint32_t k = uint32_t(it - p->seg_start_h.begin()) - 1;
          if (L >= p->seg_end_h[k]) continue;
          for (uint32_t j = 0; j < p->seg_icnt_h[k]; ++j) {
            const uint32_t y = p->inst_list_h[p->seg_ioff_h[k] + j];
            if (instance_carries(p, y, x, km)) rows.push_back({chr_of(e, L), y, L, m});
          }
        }
      };
      for (int32_t u = int32_t(v); u >= 0; u = p->parent[u]) take(uint32_t(u));
      take(N);   // preneoplastic mutations: every cell holds them
      std::sort(rows.begin(), rows.end(), [](const Row& a, const Row& b) {
        if (a.chr != b.chr) return a.chr < b.chr;
        if (a.allele != b.allele) return a.allele < b.allele;
        if (a.locus != b.locus) return a.locus < b.locus;
        return a.row < b.row;
      });
      for (const Row& r : rows) { p->cm_cell.push_back(v); p->cm_row.push_back(r.row); p->cm_allele.push_back(r.allele); }
    }
    *n_rows = p->cm_cell.size();
  });
}

pg_status pg_placed_cell_mutations_copy(const pg_placed* p, uint32_t* cell, uint32_t* mutation, uint32_t* allele) {
  return guarded([&] {
    require(p != nullptr, "NULL handle");
    auto cp = [](auto* dst, const auto& v) { if (dst) std::copy(v.begin(), v.end(), dst); };
    cp(cell, p->cm_cell); cp(mutation, p->cm_row); cp(allele, p->cm_allele);
  });
}

pg_status pg_placed_cell_cnas(pg_placed* p, uint32_t n_cells, const uint32_t* cells, uint64_t* n_rows) {
  return guarded([&] {
    require(p != nullptr && n_rows != nullptr, "NULL argument");
    const std::vector<uint32_t> cs = getter_cells(p, n_cells, cells);
    p->cc_cell.clear(); p->cc_index.clear();
    for (uint32_t v : cs)
      for (uint32_t i = 0; i < p->cnas.size(); ++i) {
        const uint32_t u = p->cnas[i].node;
        if (u < p->n_nodes && p->tin[u] <= p->tin[v] && p->tin[v] < p->tout[u]) {
          p->cc_cell.push_back(v);
          p->cc_index.push_back(i);
        }
      }
    *n_rows = p->cc_cell.size();
  });
}

pg_status pg_placed_cell_cnas_copy(const pg_placed* p, uint32_t* cell, uint32_t* cna_index) {
  return guarded([&] {
    require(p != nullptr, "NULL handle");
    if (cell) std::copy(p->cc_cell.begin(), p->cc_cell.end(), cell);
    if (cna_index) std::copy(p->cc_index.begin(), p->cc_index.end(), cna_index);
  });
}

pg_status pg_placed_cell_fragmentation(pg_placed* p, uint32_t n_cells, const uint32_t* cells, uint64_t* n_rows) {
  return guarded([&] {
    require(p != nullptr && n_rows != nullptr, "NULL argument");
    const std::vector<uint32_t> cs = getter_cells(p, n_cells, cells);
    const pg_engine* e = p->eng;
    p->cf_cell.clear(); p->cf_chr.clear(); p->cf_begin.clear(); p->cf_end.clear();
    p->cf_major.clear(); p->cf_minor.clear();
    std::map<uint32_t, std::vector<Frag>> per_class;
    for (uint32_t v : cs) {
      const uint32_t c = p->has_cna ? p->node_class_h[v] : 0u;
      auto it = per_class.find(c);
      if (it == per_class.end()) it = per_class.emplace(c, class_fragments(p, c)).first;
      for (const Frag& f : it->second) {
        const uint32_t k = chr_of(e, f.begin);
        p->cf_cell.push_back(v); p->cf_chr.push_back(k);
        p->cf_begin.push_back(f.begin - e->chr_off[k] + 1); p->cf_end.push_back(f.end - e->chr_off[k]);
        p->cf_major.push_back(std::max(f.a0, f.a1)); p->cf_minor.push_back(std::min(f.a0, f.a1));
      }
    }
    *n_rows = p->cf_cell.size();
  });
}

pg_status pg_placed_cell_fragmentation_copy(const pg_placed* p, uint32_t* cell, uint32_t* chr, uint32_t* begin,
                                            uint32_t* end, uint32_t* major, uint32_t* minor) {
  return guarded([&] {
    require(p != nullptr, "NULL handle");
    auto cp = [](auto* dst, const auto& v) { if (dst) std::copy(v.begin(), v.end(), dst); };
    cp(cell, p->cf_cell); cp(chr, p->cf_chr); cp(begin, p->cf_begin); cp(end, p->cf_end);
    cp(major, p->cf_major); cp(minor, p->cf_minor);
  });
}

pg_status pg_placed_bulk_fragmentation(pg_placed* p, int32_t sample, uint64_t* n_rows) {
  return guarded([&] {
    require(p != nullptr && n_rows != nullptr, "NULL argument");
    require(sample < int32_t(p->n_samples), "Unknown sample.");
    const pg_engine* e = p->eng;
    // the cells (their classes) of the sample, or of every sample
    std::map<uint32_t, uint64_t> cls_cells;
    for (uint32_t s = 0; s < p->n_samples; ++s) {
      if (sample >= 0 && s != uint32_t(sample)) continue;
      for (size_t i = 0; i < p->leaves[s].size(); ++i)
        ++cls_cells[p->has_cna && !p->leaf_cls[s].empty() ? p->leaf_cls[s][i] : 0u];
    }
    uint64_t n_cells = 0;
    for (const auto& kv : cls_cells) n_cells += kv.second;
    p->bf_chr.clear(); p->bf_begin.clear(); p->bf_end.clear(); p->bf_major.clear(); p->bf_minor.clear();
    p->bf_ratio.clear();
    if (n_cells == 0) { *n_rows = 0; return; }
    std::vector<std::vector<Frag>> frags;
    std::vector<uint64_t> counts;
    std::vector<uint32_t> cuts;
    for (const auto& [c, n] : cls_cells) {
      frags.push_back(class_fragments(p, c));
      counts.push_back(n);
      for (const Frag& f : frags.back()) { cuts.push_back(f.begin); cuts.push_back(f.end); }
    }
    std::sort(cuts.begin(), cuts.end());
    cuts.erase(std::unique(cuts.begin(), cuts.end()), cuts.end());
    // the type of every class at each stretch; neighbouring stretches of one
    // chromosome with the same types in every class are one fragment
    std::vector<size_t> pos(frags.size(), 0);
    std::vector<std::pair<uint32_t, uint32_t>> cur, prev;
    uint32_t f_begin = 0, f_chr = 0;
    auto emit = [&](uint32_t end) {
      std::map<std::pair<uint32_t, uint32_t>, uint64_t> agg;
      for (size_t j = 0; j < prev.size(); ++j) agg[prev[j]] += counts[j];
      uint64_t zero = 0;
      auto row = [&](uint32_t a0, uint32_t a1, uint64_t n) {
        p->bf_chr.push_back(f_chr); p->bf_begin.push_back(f_begin - e->chr_off[f_chr] + 1);
        p->bf_end.push_back(end - e->chr_off[f_chr]);
        p->bf_major.push_back(std::max(a0, a1)); p->bf_minor.push_back(std::min(a0, a1));
        p->bf_ratio.push_back(double(n) / double(n_cells));
      };
      for (const auto& [t, n] : agg) {
        if (t.first == 0 && t.second == 0) { zero = n; continue; }
        row(t.first, t.second, n);
      }
      // the cells without DNA here come last, as the reference's remainder row
      if (zero) row(0, 0, zero);
    };
    for (size_t i = 0; i + 1 < cuts.size(); ++i) {
      const uint32_t b = cuts[i];
      cur.clear();
      for (size_t j = 0; j < frags.size(); ++j) {
        while (pos[j] + 1 < frags[j].size() && frags[j][pos[j]].end <= b) ++pos[j];
        cur.push_back({frags[j][pos[j]].a0, frags[j][pos[j]].a1});
      }
      const uint32_t k = chr_of(e, b);
      if (i == 0 || k != f_chr || cur != prev) {
        if (i > 0) emit(b);
        f_begin = b; f_chr = k; prev = cur;
      }
    }
    emit(cuts.back());
    *n_rows = p->bf_chr.size();
  });
}

pg_status pg_placed_bulk_fragmentation_copy(const pg_placed* p, uint32_t* chr, uint32_t* begin, uint32_t* end,
                                            uint32_t* major, uint32_t* minor, double* ratio) {
  return guarded([&] {
    require(p != nullptr, "NULL handle");
    auto cp = [](auto* dst, const auto& v) { if (dst) std::copy(v.begin(), v.end(), dst); };
    cp(chr, p->bf_chr); cp(begin, p->bf_begin); cp(end, p->bf_end); cp(major, p->bf_major);
    cp(minor, p->bf_minor); cp(ratio, p->bf_ratio);
  });
}

pg_status pg_placed_samples_info(const pg_placed* p, uint32_t* n_cells, double* dna_quantity,
                                 double* equivalent_normal_cells) {
  return guarded([&] {
    require(p != nullptr, "NULL handle");
    const ClassView cv{p};
    std::vector<uint64_t> size(cv.n_classes());
    for (uint32_t c = 0; c < size.size(); ++c) size[c] = cv.size(c);
    const double normal = 2.0 * double(p->eng->G);
    for (uint32_t s = 0; s < p->n_samples; ++s) {
      uint64_t dna = 0;
      for (size_t i = 0; i < p->leaves[s].size(); ++i)
        dna += size[p->has_cna && !p->leaf_cls[s].empty() ? p->leaf_cls[s][i] : 0u];
      if (n_cells) n_cells[s] = uint32_t(p->leaves[s].size());
      if (dna_quantity) dna_quantity[s] = double(dna);
      if (equivalent_normal_cells) equivalent_normal_cells[s] = double(dna) / normal;
    }
  });
}

pg_status pg_seq_result_frame(pg_seq_result* r, const pg_placed* p, int include_non_sequenced, uint64_t* n_rows) {
  return guarded([&] {
    require(r && p && n_rows, "NULL argument");
    require(p->eng == r->eng && p->M == r->M, "the placed mutations are not those the result was simulated from");
    select_device(r->eng);
    pg_engine* e = r->eng;
    const uint32_t S = r->n_samples;
    // the rows: the observed mutations (alt > 0 in some sample) or, with
    // include_non_sequenced, also every mutation present in the cells of a
    // sequenced sample (a preneoplastic one always)
    std::vector<uint32_t> idx;
    std::vector<int32_t> alt, dep;   // [sample][row]
    if (!include_non_sequenced) {
      uint64_t na = 0;
      check_status(pg_seq_result_active(r, &na));
      idx.resize(na); alt.resize(na * S); dep.resize(na * S);
      check_status(pg_seq_result_copy_active(r, idx.data(), alt.data(), dep.data()));
    } else {
      std::vector<int32_t> fa(uint64_t(S) * r->M), fd(uint64_t(S) * r->M);
      check_status(pg_seq_result_copy(r, fa.data(), fd.data()));
      std::vector<uint32_t> edge(r->M);
      if (r->M) ck(cudaMemcpy(edge.data(), p->edge.p, 4 * r->M, cudaMemcpyDeviceToHost), "copy");
      // sampled leaves below each Euler index, over the sequenced samples
      std::vector<uint32_t> cum(p->n_nodes + 1, 0);
      for (int32_t src : r->sample_src)
        if (src >= 0) for (uint32_t t : p->leaves[src]) ++cum[t + 1];
      for (uint32_t x = 1; x <= p->n_nodes; ++x) cum[x] += cum[x - 1];
      // preneoplastic mutations are in every tumour cell, and in the normal
      // cells when they carry them
      bool pre_present = false;
      for (int32_t src : r->sample_src) pre_present = pre_present || src >= 0 || r->pre_in_normal;
      for (uint64_t m = 0; m < r->M; ++m) {
        bool keep = false;
        for (uint32_t s = 0; s < S && !keep; ++s) keep = fa[uint64_t(s) * r->M + m] > 0;
        const uint32_t ed = edge[m];
        if (!keep) keep = ed >= p->n_nodes ? pre_present : cum[p->tout[ed]] > cum[p->tin[ed]];
        if (keep) idx.push_back(uint32_t(m));
      }
      const uint64_t n = idx.size();
      alt.resize(n * S); dep.resize(n * S);
      for (uint32_t s = 0; s < S; ++s)
        for (uint64_t i = 0; i < n; ++i) {
          alt[s * n + i] = fa[uint64_t(s) * r->M + idx[i]];
          dep[s * n + i] = fd[uint64_t(s) * r->M + idx[i]];
        }
    }
    const uint64_t n = idx.size();
    const auto info = placed_row_info(p, n, idx.data());
    // SIDs (chromosome, position, ref, alt) in the reference's map order; the
    // rows come sorted by locus, so only rows of one locus need ordering
    std::vector<uint32_t> order(n);
    for (uint64_t i = 0; i < n; ++i) order[i] = uint32_t(i);
    for (uint64_t i = 0; i < n;) {
      uint64_t j = i + 1;
      while (j < n && info[j].x == info[i].x) ++j;
      if (j - i > 1)
        std::sort(order.begin() + i, order.begin() + j, [&](uint32_t a, uint32_t b) {
          if (info[a].y != info[b].y) return info[a].y < info[b].y;
          if (info[a].z != info[b].z) return info[a].z < info[b].z;
          return a < b;
        });
      i = j;
    }
    r->f_chr.clear(); r->f_pos.clear(); r->f_ref.clear(); r->f_alt.clear(); r->f_cause_off.assign(1, 0);
    r->f_causes.clear(); r->f_classes.clear();
    r->f_chr.reserve(n); r->f_pos.reserve(n); r->f_ref.reserve(n * PG_SID_CHARS); r->f_alt.reserve(n * PG_SID_CHARS);
    r->f_cause_off.reserve(n + 1); r->f_classes.reserve(n);
    std::vector<std::vector<int32_t>> occ(S), cov(S);
    for (uint32_t s = 0; s < S; ++s) { occ[s].reserve(n); cov[s].reserve(n); }
    // signature names of each type, indexed by the row's signature byte
    std::vector<std::string> names[2];
    for (uint32_t k = 0; k < 2; ++k)
      for (uint32_t sg = 0; sg < e->n_sig[k]; ++sg)
        names[k].push_back(sg < e->sig_names[k].size() ? e->sig_names[k][sg]
                                                        : std::string(k == 0 ? "SBS#" : "ID#") + std::to_string(sg + 1));
    auto cause_of = [&](uint32_t w) -> const std::string* {
      const uint32_t k = w & 0xffu, sg = (w >> 8) & 0xffu;
      return (k <= 1 && sg < names[k].size()) ? &names[k][sg] : nullptr;
    };
    for (uint64_t a = 0; a < n;) {
      const uint4 f = info[order[a]];
      uint64_t b = a + 1;
      while (b < n && info[order[b]].x == f.x && info[order[b]].y == f.y && info[order[b]].z == f.z) ++b;
      uint8_t classes = 0;
      if (b == a + 1) {                     // one mutation: its cause, if any
        const std::string* c = cause_of(f.w);
        if (c) r->f_causes.insert(r->f_causes.end(), c->begin(), c->end());
        classes = uint8_t(1u << ((f.w >> 16) & 7u));
      } else {                              // several: the sorted union
        std::set<std::string> causes;
        for (uint64_t q = a; q < b; ++q) {
          const uint32_t w = info[order[q]].w;
          if (const std::string* c = cause_of(w)) causes.insert(*c);
          classes |= uint8_t(1u << ((w >> 16) & 7u));
        }
        bool first = true;
        for (const auto& cs : causes) {
          if (!first) r->f_causes.push_back(';');
          r->f_causes.insert(r->f_causes.end(), cs.begin(), cs.end());
          first = false;
        }
      }
      r->f_cause_off.push_back(r->f_causes.size());
      r->f_classes.push_back(classes);
      const uint32_t c = chr_of(e, f.x);
      r->f_chr.push_back(c);
      r->f_pos.push_back(f.x - e->chr_off[c] + 1);
      char buf[PG_SID_CHARS];
      sid_string(f.y, buf); r->f_ref.insert(r->f_ref.end(), buf, buf + PG_SID_CHARS);
      sid_string(f.z, buf); r->f_alt.insert(r->f_alt.end(), buf, buf + PG_SID_CHARS);
      for (uint32_t s = 0; s < S; ++s) {
        int64_t o = 0;
        for (uint64_t q = a; q < b; ++q) o += alt[uint64_t(s) * n + order[q]];
        occ[s].push_back(int32_t(o));
        cov[s].push_back(dep[uint64_t(s) * n + order[a]]);
      }
      a = b;
    }
    const uint64_t R = r->f_chr.size();
    r->f_rows = R;
    r->f_occ.resize(uint64_t(S) * R); r->f_cov.resize(uint64_t(S) * R); r->f_vaf.resize(uint64_t(S) * R);
    for (uint32_t s = 0; s < S; ++s)
      for (uint64_t i = 0; i < R; ++i) {
        r->f_occ[s * R + i] = occ[s][i];
        r->f_cov[s * R + i] = cov[s][i];
        r->f_vaf[s * R + i] = cov[s][i] > 0 ? double(occ[s][i]) / double(cov[s][i]) : 0.0;
      }
    *n_rows = R;
  });
}

pg_status pg_seq_result_frame_causes_size(const pg_seq_result* r, uint64_t* n_chars) {
  return guarded([&] { require(r && n_chars, "NULL argument"); *n_chars = r->f_causes.size(); });
}

pg_status pg_seq_result_frame_copy(const pg_seq_result* r, uint32_t* chr, uint32_t* chr_pos, char* ref, char* alt,
                                   uint64_t* causes_off, char* causes, uint8_t* classes, int32_t* occurrences,
                                   int32_t* coverage, double* vaf) {
  return guarded([&] {
    require(r != nullptr, "NULL handle");
    auto cp = [](auto* dst, const auto& v) { if (dst) std::copy(v.begin(), v.end(), dst); };
    cp(chr, r->f_chr); cp(chr_pos, r->f_pos); cp(ref, r->f_ref); cp(alt, r->f_alt);
    cp(causes_off, r->f_cause_off); cp(causes, r->f_causes); cp(classes, r->f_classes);
    cp(occurrences, r->f_occ); cp(coverage, r->f_cov); cp(vaf, r->f_vaf);
  });
}

}  // extern "C"
