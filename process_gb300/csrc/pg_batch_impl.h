// Batched instances: many forests, parameter sets and coverages on one
// engine's genome and signatures (no reference counterpart: the reference
// places and sequences one instance per call).  Included at the end of
// pg_api.cpp, whose handles and helpers it uses.
//
// Instance i has its own forest (every node of species 0), passenger rates,
// one exposure, preneoplastic counts, sequencing configuration and tile size.
// It computes exactly what the plain path computes for an engine whose
// species 0 has those rates and that exposure at time 0, called with the
// same seeds and tile size:
//   * placement runs as single launches over every instance (edge counts,
//     mutation placement, infinite-sites rounds keyed by (instance, locus),
//     one sort by (instance, locus)); slots of one instance keep their order;
//   * sequencing runs as one persistent read kernel over every (instance,
//     sample, tile), after batched tile splits and record ranges; the stage is
//     captured into a CUDA graph on its first run and replayed afterwards
//     (sizes it depends on live in device memory; capacities grow, and the
//     graph is captured again, only when an instance outgrows them);
//   * the autotuner times the persistent kernel over candidate tile sizes
//     for every instance and keeps the fastest.

struct BatchInst {
  pg_forest f;
  double snv = 0, indel = 0;
  std::vector<double> sbs_w, id_w;
  uint32_t n_pre_snv = 0, n_pre_id = 0;
  pg_seq_cfg cfg{};
  std::vector<uint32_t> chr_sel;
  uint32_t T = 0;          // tile size
  uint64_t M = 0;          // mutations placed by the last run
  uint64_t n_reads = 0;
  uint32_t n_samples = 0;
};

struct pg_batch {
  pg_engine* eng = nullptr;
  std::vector<BatchInst> in;
  uint32_t pre_sbs_sig = 0, pre_id_sig = 0;
  // placement tables (fixed per batch)
  std::vector<uint32_t> node_off, cell_off;     // n_inst + 1
  DBuf<int32_t> parent;
  DBuf<double> birth, epoch0, rates, node_size;
  DBuf<uint32_t> zeros, divisions, sig_cdf[2], expo_cdf[2];
  DBuf<uint32_t> gc_seg_off, gc_seg_start, gc_seg_end, gc_seg_ioff, gc_seg_icnt;
  DBuf<uint16_t> gc_inst;
  DBuf<pg::PlaceTables> tabs;
  DBuf<uint32_t> node_off_d, cell_off_d, pre_snv_d, pre_id_d;
  DBuf<pg::Key> pkeys, skeys;
  // placement outputs (capacity slot_cap)
  uint64_t slot_cap = 0, n_all = 0;
  DBuf<uint32_t> locus, edge, aux, attempt, s_locus, s_edge, s_aux, s_attempt;
  DBuf<uint8_t> cls, sig, kind, nature, s_cls, s_sig, s_kind, s_nature;
  DBuf<uint16_t> allele, seqo, inst_of, s_allele, s_seq, s_inst;
  DBuf<uint32_t> rec_off_d, n_all_d;
  std::vector<uint32_t> rec_off;
  // sequencing layout (rebuilt when tile sizes change or an instance outgrows its capacity)
  bool layout_ok = false;
  std::vector<uint32_t> stride;                  // per instance: alt/depth row length
  std::vector<pg::SeqInst> sinst;
  pg::SeqBatch sb{};
  DBuf<pg::SeqInst> sinst_d;
  DBuf<uint32_t> item_off_d, cnt_off_d, t_start, t_len, t_end, t_inst, rec_lo, rec_hi;
  DBuf<uint32_t> c_first, c_ntiles, c_depth, c_nstarts, c_id, blk_slot, blk_index, pair_cnt;
  DBuf<uint64_t> c_pairs;
  DBuf<pg::SeqSample> samples;
  DBuf<uint32_t> leaf_tin, etin, etout, ins_cdf, counter, alt, depth;
  DBuf<uint16_t> ins_guide;
  DBuf<pg::SeqRec> recs;
  uint64_t rec_cap = 0;
  cudaGraphExec_t graph = nullptr;
  uint32_t graph_kernels = 0;     // kernels one replay launches
  uint32_t grid = 0;
  float place_ms = 0, seq_ms = 0;

  ~pg_batch() {
    if (graph) cudaGraphExecDestroy(graph);
  }
  pg::PlaceOut out_view() {
    return {locus.p, edge.p, aux.p, cls.p, sig.p, allele.p, seqo.p, kind.p, nature.p, attempt.p};
  }
  pg::PlaceOut sorted_view() {
    return {s_locus.p, s_edge.p, s_aux.p, s_cls.p, s_sig.p, s_allele.p, s_seq.p, s_kind.p, s_nature.p, s_attempt.p};
  }
};

namespace {

// the plain auto tile size without the mutation-density term
uint32_t batch_default_tile(const pg_seq_cfg& c, uint32_t span) {
  const double mates = c.insert_size_mean > 0 ? 2.0 : 1.0;
  const double cap = double(pg::SEQ_FRAGS_PER_BATCH);
  const double target = cap - 4.0 * std::sqrt(cap);
  double t = c.coverage > 0 ? target * c.read_size * mates / c.coverage : 8192.0;
  t = std::min(t, double(16384 - 1 - span));
  return uint32_t(std::max(256.0, std::floor(t / 64.0) * 64.0));
}

uint32_t batch_span(const pg_seq_cfg& c, uint32_t& ins_min, std::vector<uint32_t>& thr) {
  const uint32_t R = c.read_size;
  ins_min = R;
  thr.assign(1, 2147483648u);
  if (c.insert_size_mean > 0) insert_table(c, R, ins_min, thr);
  return std::max<uint32_t>(R, ins_min + uint32_t(thr.size()) - 1);
}

void batch_place(pg_batch* b, const uint64_t* place_seed) {
  pg_engine* e = b->eng;
  cudaStream_t st = e->st;
  Pool* P = &e->pool;
  const uint32_t B = uint32_t(b->in.size());
  std::vector<pg::Key> keys(B);
  for (uint32_t i = 0; i < B; ++i) keys[i] = pg::make_key(place_seed[i]);
  ck(cudaMemcpyAsync(b->pkeys.p, keys.data(), sizeof(pg::Key) * B, cudaMemcpyHostToDevice, st), "keys");
  const uint32_t n_cells = b->cell_off[B];
  DBuf<uint32_t> cnt_snv(P, n_cells), cnt_id(P, n_cells), part(P, pg::scan_part_elems(n_cells, 1)), tot(P, 2);
  pg::place_edge_counts_batch(b->tabs.p, B, b->node_off_d.p, b->node_off[B], b->cell_off_d.p, b->pkeys.p,
                              b->pre_snv_d.p, b->pre_id_d.p, cnt_snv.p, cnt_id.p, st);
  pg::scan_rows<uint32_t>(cnt_snv.p, cnt_snv.p, n_cells, 1, part.p, tot.p, st);
  pg::scan_rows<uint32_t>(cnt_id.p, cnt_id.p, n_cells, 1, part.p, tot.p + 1, st);
  uint32_t tot_h[2];
  ck(cudaMemcpyAsync(tot_h, tot.p, sizeof(tot_h), cudaMemcpyDeviceToHost, st), "counts");
  ck(cudaStreamSynchronize(st), "batch counts");
  const uint64_t n_snv = tot_h[0], n_id = tot_h[1], n_all = n_snv + n_id;
  require(n_all < (1ull << 31), "too many mutations for one batch");
  b->n_all = n_all;
  if (n_all > b->slot_cap) {
    const uint64_t cap = n_all + n_all / 8 + 4096;
    b->locus = DBuf<uint32_t>(P, cap); b->edge = DBuf<uint32_t>(P, cap); b->aux = DBuf<uint32_t>(P, cap);
    b->attempt = DBuf<uint32_t>(P, cap);
    b->s_locus = DBuf<uint32_t>(P, cap); b->s_edge = DBuf<uint32_t>(P, cap); b->s_aux = DBuf<uint32_t>(P, cap);
    b->s_attempt = DBuf<uint32_t>(P, cap);
    b->cls = DBuf<uint8_t>(P, cap); b->sig = DBuf<uint8_t>(P, cap); b->kind = DBuf<uint8_t>(P, cap);
    b->nature = DBuf<uint8_t>(P, cap);
    b->s_cls = DBuf<uint8_t>(P, cap); b->s_sig = DBuf<uint8_t>(P, cap); b->s_kind = DBuf<uint8_t>(P, cap);
    b->s_nature = DBuf<uint8_t>(P, cap);
    b->allele = DBuf<uint16_t>(P, cap); b->seqo = DBuf<uint16_t>(P, cap); b->inst_of = DBuf<uint16_t>(P, cap);
    b->s_allele = DBuf<uint16_t>(P, cap); b->s_seq = DBuf<uint16_t>(P, cap); b->s_inst = DBuf<uint16_t>(P, cap);
    b->slot_cap = cap;
    b->layout_ok = false;          // the records buffer follows the slot capacity
  }
  const pg::PlaceOut o = b->out_view();
  DBuf<uint32_t> err(P, 1);
  DBuf<pg::TailCtl> tail_ctl;
  ck(cudaMemsetAsync(err.p, 0, sizeof(uint32_t), st), "memset");
  pg::place_mutations_batch(b->tabs.p, B, b->cell_off_d.p, b->pkeys.p, o, b->inst_of.p, cnt_snv.p, cnt_id.p,
                            uint32_t(n_snv), nullptr, uint32_t(n_all), 0, err.p, st);
  if (e->infinite_sites && n_all > 0) {
    DBuf<uint32_t> pend_a(P, n_all), pend_b(P, n_all), n_next(P, 1);
    DBuf<uint8_t> lost(P, n_all);
    const uint32_t* pending = nullptr;
    uint32_t n_pend = uint32_t(n_all);
    uint32_t* next = pend_a.p;
    // the first round (no drivers in a batch, so nothing is taken yet) keeps
    // its candidate table, which then holds exactly the taken keys; the
    // later rounds test it beside their own accepted set, sized by what the
    // first round leaves
    uint64_t fcap = 1024;
    while (fcap < 2 * n_all) fcap <<= 1;
    DBuf<uint64_t> fkeys(P, fcap);
    {
      DBuf<uint32_t> fvals(P, fcap);
      ck(cudaMemsetAsync(fkeys.p, 0xff, sizeof(uint64_t) * fcap, st), "memset");
      ck(cudaMemsetAsync(fvals.p, 0xff, sizeof(uint32_t) * fcap, st), "memset");
      ck(cudaMemsetAsync(n_next.p, 0, sizeof(uint32_t), st), "memset");
      pg::sites_round_batch(b->locus.p, b->inst_of.p, nullptr, n_pend, nullptr, 0, fkeys.p, fvals.p, fcap - 1, lost.p,
                            next, n_next.p, err.p, st);
      uint32_t nn = 0;
      ck(cudaMemcpyAsync(&nn, n_next.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st), "round");
      ck(cudaStreamSynchronize(st), "first round");
      pending = next;
      n_pend = nn;
    }
    // every later round (the losers' redraws first) in one cooperative
    // launch, its tables sized by what the first round leaves
    uint64_t cap = 1024;
    while (cap < 2 * uint64_t(n_pend)) cap <<= 1;
    if (n_pend) {
      DBuf<unsigned long long> hkeys(P, cap), ckeys(P, cap);
      DBuf<uint32_t> cvals(P, cap);
      DBuf<uint64_t> hpos(P, n_pend);
      ck(cudaMemsetAsync(hkeys.p, 0xff, sizeof(uint64_t) * cap, st), "memset");
      ck(cudaMemsetAsync(ckeys.p, 0xff, sizeof(uint64_t) * cap, st), "memset");
      ck(cudaMemsetAsync(cvals.p, 0xff, sizeof(uint32_t) * cap, st), "memset");
      tail_ctl = DBuf<pg::TailCtl>(P, 1);
      pg::TailCtl c0{};
      c0.count[0] = n_pend;
      ck(cudaMemcpyAsync(tail_ctl.p, &c0, sizeof(c0), cudaMemcpyHostToDevice, st), "rounds");
      pg::TailArgsB ta{};
      ta.list[0] = const_cast<uint32_t*>(pending);
      ta.list[1] = pend_b.p;
      ta.hkeys = hkeys.p; ta.hmask = cap - 1;
      ta.ckeys = ckeys.p; ta.cvals = cvals.p; ta.cmask = cap - 1;
      ta.hpos = hpos.p;
      ta.fkeys = fkeys.p; ta.fmask = fcap - 1;
      if (const char* msg = pg::sites_tail_batch(b->tabs.p, B, b->cell_off_d.p, b->pkeys.p, o, b->inst_of.p, cnt_snv.p,
                                                 cnt_id.p, uint32_t(n_snv), ta, n_pend, tail_ctl.p, err.p, st))
        throw std::runtime_error(msg);
      // the tables live until the launch ends: the engine's pool hands them
      // out again only to later work on this stream
    }
  }
  // sort by (instance, locus); the instance's first record is the exclusive
  // scan at its first bucket
  const uint32_t nb = pg::sort_num_buckets(e->G);
  const uint64_t nbt = uint64_t(nb) * B;
  DBuf<uint32_t> bcnt(P, nbt + 1), bfill(P, nbt), bpart(P, pg::scan_part_elems(nbt, 1)), order(P, n_all);
  DBuf<unsigned long long> skeys(P, n_all);
  DBuf<uint4> recs(P, 2 * n_all);
  pg::sort_batch(o, b->inst_of.p, uint32_t(n_all), B, e->G, bcnt.p, bfill.p, bpart.p, order.p, b->sorted_view(),
                 b->s_inst.p, skeys.p, recs.p, st);
  if (n_all > 0) {
    ck(cudaMemcpy2DAsync(b->rec_off_d.p, sizeof(uint32_t), bcnt.p, sizeof(uint32_t) * nb, sizeof(uint32_t), B,
                         cudaMemcpyDeviceToDevice, st), "record offsets");
  } else {
    ck(cudaMemsetAsync(b->rec_off_d.p, 0, sizeof(uint32_t) * B, st), "memset");
  }
  const uint32_t na = uint32_t(n_all);
  ck(cudaMemcpyAsync(b->rec_off_d.p + B, &na, sizeof(uint32_t), cudaMemcpyHostToDevice, st), "record offsets");
  ck(cudaMemcpyAsync(b->n_all_d.p, &na, sizeof(uint32_t), cudaMemcpyHostToDevice, st), "count");
  b->rec_off.assign(B + 1, 0);
  ck(cudaMemcpyAsync(b->rec_off.data(), b->rec_off_d.p, sizeof(uint32_t) * (B + 1), cudaMemcpyDeviceToHost, st),
     "record offsets");
  uint32_t err_h = 0;
  ck(cudaMemcpyAsync(&err_h, err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st), "error flag");
  pg::TailCtl tc{};
  if (tail_ctl.p) ck(cudaMemcpyAsync(&tc, tail_ctl.p, sizeof(tc), cudaMemcpyDeviceToHost, st), "rounds");
  ck(cudaStreamSynchronize(st), "batch placement");
  if (tc.status & pg::TAIL_BARRIER_TIMEOUT) throw std::runtime_error("a grid barrier of the redraw rounds timed out");
  require(!(tc.status & pg::TAIL_ROUNDS_EXHAUSTED), "infinite sites model: no free locus left for some mutations");
  if (err_h & pg::ERR_EMPTY_CLASS) throw std::runtime_error("a drawn mutation class has no indexed positions");
  if (err_h & pg::ERR_CAPACITY) throw std::runtime_error("internal hash table capacity exceeded");
  for (uint32_t i = 0; i < B; ++i) {
    const uint64_t m = uint64_t(b->rec_off[i + 1]) - b->rec_off[i];
    if (b->layout_ok && m > b->stride[i]) b->layout_ok = false;
    b->in[i].M = m;
  }
}

// sequencing layout: tiles, chromosome tables, samples, per-instance
// descriptors, count rows sized with headroom over the last placement
void batch_layout(pg_batch* b) {
  pg_engine* e = b->eng;
  cudaStream_t st = e->st;
  Pool* P = &e->pool;
  const uint32_t B = uint32_t(b->in.size());
  std::vector<uint32_t> t_start, t_len, t_end, t_inst, c_first, c_ntiles, c_depth, c_nstarts, c_id, blk_slot,
      blk_index, leaf_tin, etin, etout, ins_cdf, item_off{0}, cnt_off{0};
  std::vector<uint64_t> c_pairs;
  std::vector<uint16_t> guide_all;
  std::vector<pg::SeqSample> samples;
  b->sinst.assign(B, pg::SeqInst{});
  b->stride.assign(B, 0);
  uint64_t pair_total = 0, count_total = 0;
  for (uint32_t i = 0; i < B; ++i) {
    BatchInst& I = b->in[i];
    const pg_seq_cfg& c = I.cfg;
    const pg_forest& f = I.f;
    pg::SeqInst& S = b->sinst[i];
    uint32_t ins_min = 0;
    std::vector<uint32_t> thr;
    const uint32_t span = batch_span(c, ins_min, thr);
    const uint32_t R = c.read_size, T = I.T;
    const bool paired = c.insert_size_mean > 0;
    const double mates = paired ? 2.0 : 1.0;
    // chromosomes and tiles
    std::vector<uint32_t> chrs = I.chr_sel;
    if (chrs.empty()) for (uint32_t k = 0; k < e->n_chr; ++k) chrs.push_back(k);
    S.tile_off = uint32_t(t_start.size());
    S.slot_off = uint32_t(c_first.size());
    S.blk_off = uint32_t(blk_slot.size());
    S.T = T;
    uint32_t n_tiles = 0, n_slots = 0;
    uint64_t frags = 0;
    for (uint32_t ci : chrs) {
      const uint32_t L = e->chr_len[ci];
      if (L < R) continue;
      const uint32_t Sx = L - R + 1, nt = (Sx + T - 1) / T;
      const uint64_t pairs = uint64_t(std::floor(c.coverage * double(L) / (double(R) * mates)));
      require(pairs < (uint64_t(1) << 32), "too many fragments for one chromosome");
      uint32_t D = 0;
      while ((uint64_t(1) << D) < nt) ++D;
      c_id.push_back(ci); c_ntiles.push_back(nt); c_nstarts.push_back(Sx); c_pairs.push_back(pairs);
      c_first.push_back(n_tiles); c_depth.push_back(D);
      const uint32_t blk = 1u << std::min<uint32_t>(D, 6);
      for (uint32_t q = 0; q * blk < nt; ++q) { blk_slot.push_back(n_slots); blk_index.push_back(q); }
      for (uint32_t k = 0; k < nt; ++k) {
        t_start.push_back(e->chr_off[ci] + k * T);
        t_len.push_back(std::min<uint32_t>(T, Sx - k * T));
        t_end.push_back(e->chr_off[ci] + L);
        t_inst.push_back(i);
      }
      n_tiles += nt;
      ++n_slots;
      frags += pairs;
    }
    S.n_tiles = n_tiles;
    S.n_blocks = uint32_t(blk_slot.size()) - S.blk_off;
    // samples (the plain path's rules)
    S.sample_off = uint32_t(samples.size());
    const uint32_t N = f.n;
    if (!c.normal_only) {
      double nthr = std::floor((1.0 - c.purity) * 4294967296.0);
      if (nthr > 4294967295.0) nthr = 4294967295.0;
      for (uint32_t s = 0; s < f.n_samples; ++s) {
        require(!f.leaves[s].empty(), "sample " + std::to_string(s) + " has no sampled cells");
        pg::SeqSample ss{};
        ss.n_leaves = uint32_t(f.leaves[s].size());
        ss.leaf_off = uint32_t(leaf_tin.size());
        ss.normal_thr = c.purity >= 1 ? 0u : uint32_t(nthr);
        ss.all_normal = c.purity <= 0 ? 1u : 0u;
        leaf_tin.insert(leaf_tin.end(), f.leaves[s].begin(), f.leaves[s].end());
        samples.push_back(ss);
      }
    }
    if (c.normal_only || c.with_normal_sample) {
      pg::SeqSample ss{};
      ss.all_normal = 1;
      samples.push_back(ss);
    }
    S.n_samples = uint32_t(samples.size()) - S.sample_off;
    I.n_samples = S.n_samples;
    I.n_reads = frags * uint64_t(mates) * S.n_samples;
    // Euler table of the instance's edges (+ preneoplastic and germline rows)
    S.etin_off = uint32_t(etin.size());
    for (uint32_t v = 0; v < N; ++v) { etin.push_back(f.tin[v]); etout.push_back(f.tout[v]); }
    etin.push_back(0); etout.push_back(c.preneoplastic_in_normal ? N + 1 : N);
    etin.push_back(0); etout.push_back(N + 1);
    // parameters
    pg::SeqParams& prm = S.prm;
    prm.read_len = R; prm.paired = paired ? 1u : 0u; prm.span = span;
    prm.ins_min = ins_min; prm.n_ins = uint32_t(thr.size());
    double et = std::floor(c.error_rate * 4294967296.0);
    prm.err_thr = et >= 4294967295.0 ? 0xffffffffu : uint32_t(et);
    pg::err_thirds(prm.err_thr, prm.err_t1, prm.err_t2);
    prm.normal_tin = N;
    prm.n_alleles = 2;
    prm.has_cna = 0;
    // insert tables: positions into the concatenated arrays, patched below
    prm.ins_cdf = reinterpret_cast<const uint32_t*>(uintptr_t(ins_cdf.size()));
    prm.ins_guide = reinterpret_cast<const uint16_t*>(uintptr_t(guide_all.size()));
    ins_cdf.insert(ins_cdf.end(), thr.begin(), thr.end());
    for (uint32_t g = 0; g < 256; ++g) {
      const uint32_t v = g << 23;
      const uint32_t k = uint32_t(std::upper_bound(thr.begin(), thr.end(), v) - thr.begin());
      guide_all.push_back(uint16_t(std::min<uint32_t>(k, uint32_t(thr.size()) - 1)));
    }
    // counts and work items
    S.pair_off = pair_total;
    pair_total += uint64_t(S.n_samples) * n_tiles;
    const uint64_t m = std::max<uint64_t>(I.M, 1);
    b->stride[i] = uint32_t(std::min<uint64_t>(m + m / 4 + 1024, 0xffffffffu));
    S.count_stride = b->stride[i];
    S.count_off = count_total;
    count_total += uint64_t(S.n_samples) * S.count_stride;
    item_off.push_back(item_off.back() + S.n_samples * n_tiles);
    cnt_off.push_back(cnt_off.back() + S.n_samples * S.n_blocks);
  }
  if (leaf_tin.empty()) leaf_tin.push_back(0);
  b->t_start = upload(P, t_start, st); b->t_len = upload(P, t_len, st); b->t_end = upload(P, t_end, st);
  b->t_inst = upload(P, t_inst, st);
  b->rec_lo = DBuf<uint32_t>(P, t_start.size()); b->rec_hi = DBuf<uint32_t>(P, t_start.size());
  b->c_first = upload(P, c_first, st); b->c_ntiles = upload(P, c_ntiles, st); b->c_depth = upload(P, c_depth, st);
  b->c_nstarts = upload(P, c_nstarts, st); b->c_id = upload(P, c_id, st); b->c_pairs = upload(P, c_pairs, st);
  b->blk_slot = upload(P, blk_slot, st); b->blk_index = upload(P, blk_index, st);
  b->pair_cnt = DBuf<uint32_t>(P, pair_total);
  b->samples = upload(P, samples, st);
  b->leaf_tin = upload(P, leaf_tin, st);
  b->etin = upload(P, etin, st); b->etout = upload(P, etout, st);
  b->ins_cdf = upload(P, ins_cdf, st); b->ins_guide = upload(P, guide_all, st);
  for (auto& S : b->sinst) {
    S.prm.ins_cdf = b->ins_cdf.p + uintptr_t(S.prm.ins_cdf);
    S.prm.ins_guide = b->ins_guide.p + uintptr_t(S.prm.ins_guide);
  }
  b->sinst_d = upload(P, b->sinst, st);
  b->item_off_d = upload(P, item_off, st); b->cnt_off_d = upload(P, cnt_off, st);
  b->counter = DBuf<uint32_t>(P, 1);
  b->alt = DBuf<uint32_t>(P, count_total); b->depth = DBuf<uint32_t>(P, count_total);
  b->recs = DBuf<pg::SeqRec>(P, b->slot_cap);
  b->rec_cap = b->slot_cap;
  pg::SeqBatch& sb = b->sb;
  sb = pg::SeqBatch{};
  sb.n_inst = B; sb.inst = b->sinst_d.p; sb.keys = b->skeys.p; sb.rec_off = b->rec_off_d.p;
  sb.item_off = b->item_off_d.p; sb.cnt_off = b->cnt_off_d.p;
  sb.n_items = item_off.back(); sb.n_cnt = cnt_off.back(); sb.n_tiles_all = uint32_t(t_start.size());
  sb.tile_start = b->t_start.p; sb.tile_len = b->t_len.p; sb.tile_end = b->t_end.p; sb.tile_inst = b->t_inst.p;
  sb.rec_lo = b->rec_lo.p; sb.rec_hi = b->rec_hi.p;
  sb.c_first = b->c_first.p; sb.c_ntiles = b->c_ntiles.p; sb.c_depth = b->c_depth.p; sb.c_nstarts = b->c_nstarts.p;
  sb.c_id = b->c_id.p; sb.c_pairs = b->c_pairs.p; sb.blk_slot = b->blk_slot.p; sb.blk_index = b->blk_index.p;
  sb.pair_cnt = b->pair_cnt.p; sb.samples = b->samples.p; sb.leaf_tin = b->leaf_tin.p;
  sb.etin = b->etin.p; sb.etout = b->etout.p; sb.counter = b->counter.p; sb.alt = b->alt.p; sb.depth = b->depth.p;
  int sms = 0, per_sm = 0;
  ck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, e->device), "device attribute");
  per_sm = pg::seq_reads_batch_occupancy();
  b->grid = uint32_t(std::max(1, sms * std::max(1, per_sm)));
  if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
  ck(cudaStreamSynchronize(st), "batch layout");
  b->layout_ok = true;
}

// the sequencing stage, captured once per layout
void batch_sequence(pg_batch* b) {
  pg_engine* e = b->eng;
  cudaStream_t st = e->st;
  if (!b->graph) {
    cudaGraph_t g = nullptr;
    const uint64_t counted = g_launches.load();   // captured kernels are not launches yet
    ck(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "stream capture");
    const uint64_t nc = b->alt.n;
    cudaMemsetAsync(b->alt.p, 0, sizeof(uint32_t) * nc, st);
    cudaMemsetAsync(b->depth.p, 0, sizeof(uint32_t) * nc, st);
    pg::seq_batch_records(b->sorted_view(), b->s_inst.p, b->n_all_d.p, uint32_t(b->rec_cap), b->sb, b->recs.p, st);
    pg::seq_batch_reads(b->sb, b->recs.p, b->grid, st);
    ck(cudaStreamEndCapture(st, &g), "stream capture");
    b->graph_kernels = uint32_t(g_launches.load() - counted);
    g_launches.store(counted);
    const cudaError_t r = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    ck(r, "graph instantiate");
  }
  ck(cudaGraphLaunch(b->graph, st), "graph launch");
  pg::note_launch(b->graph_kernels);
}

}  // namespace

pg_status pg_batch_create(pg_engine* e, uint32_t n_inst, const pg_forest* const* forests, const double* snv_rate,
                          const double* indel_rate, const double* sbs_expo, const double* id_expo,
                          const uint32_t* n_pre_snv, uint32_t pre_sbs_sig, const uint32_t* n_pre_indel,
                          uint32_t pre_id_sig, const pg_seq_cfg* cfgs, pg_batch** out) {
  return guarded([&] {
    require(e && forests && snv_rate && indel_rate && cfgs && out, "NULL argument");
    require(n_inst > 0 && n_inst <= 65535, "a batch holds 1 to 65535 instances");
    select_device(e);
    cudaStream_t st = e->st;
    Pool* P = &e->pool;
    auto b = std::make_unique<pg_batch>();
    b->eng = e;
    b->pre_sbs_sig = pre_sbs_sig; b->pre_id_sig = pre_id_sig;
    const uint32_t ns[2] = {std::max<uint32_t>(e->n_sig[0], 1), std::max<uint32_t>(e->n_sig[1], 1)};
    b->in.resize(n_inst);
    uint32_t max_n = 0;
    b->node_off.assign(1, 0);
    b->cell_off.assign(1, 0);
    std::vector<int32_t> parent;
    std::vector<double> birth, rates;
    std::vector<uint32_t> divisions, pre_s, pre_i;
    for (uint32_t i = 0; i < n_inst; ++i) {
      require(forests[i] != nullptr, "NULL forest");
      BatchInst& I = b->in[i];
      I.f = *forests[i];
      I.snv = snv_rate[i]; I.indel = indel_rate[i];
      require(std::isfinite(I.snv) && I.snv >= 0 && std::isfinite(I.indel) && I.indel >= 0,
              "passenger rates must be non-negative");
      I.n_pre_snv = n_pre_snv ? n_pre_snv[i] : 0;
      I.n_pre_id = n_pre_indel ? n_pre_indel[i] : 0;
      I.cfg = cfgs[i];
      const pg_seq_cfg& c = I.cfg;
      require(c.coverage >= 0 && std::isfinite(c.coverage), "The coverage must be non-negative");
      require(c.read_size >= 1 && c.read_size <= 4096, "read_size must be in [1, 4096]");
      require(c.purity >= 0 && c.purity <= 1, "The purity must be a value in [0,1]");
      require(c.error_rate >= 0 && c.error_rate <= 1, "The parameter \"error_rate\" must be a positive real number.");
      if (c.n_chr_sel) {
        require(c.chr_sel != nullptr, "NULL chromosome list");
        for (uint32_t k = 0; k < c.n_chr_sel; ++k) {
          require(c.chr_sel[k] < e->n_chr, "unknown chromosome");
          I.chr_sel.push_back(c.chr_sel[k]);
        }
        std::sort(I.chr_sel.begin(), I.chr_sel.end());
        I.chr_sel.erase(std::unique(I.chr_sel.begin(), I.chr_sel.end()), I.chr_sel.end());
      }
      I.cfg.chr_sel = nullptr;
      uint32_t ins_min = 0;
      std::vector<uint32_t> thr;
      const uint32_t span = batch_span(c, ins_min, thr);   // validates the insert model
      I.T = c.tile_size ? c.tile_size : batch_default_tile(c, span);
      require(I.T >= 64 && I.T <= (1u << 24), "tile_size must be in [64, 2^24]");
      // exposures: one epoch, the plain path's thresholds
      for (int ty = 0; ty < 2; ++ty) {
        const double* src = ty == 0 ? sbs_expo : id_expo;
        std::vector<double>& w = ty == 0 ? I.sbs_w : I.id_w;
        w.assign(ns[ty], 0.0);
        if (src && e->n_sig[ty]) for (uint32_t k = 0; k < e->n_sig[ty]; ++k) w[k] = src[uint64_t(i) * e->n_sig[ty] + k];
      }
      const uint32_t n = I.f.n;
      max_n = std::max(max_n, n);
      for (uint32_t v = 0; v < n; ++v) {
        parent.push_back(I.f.parent[v]);
        birth.push_back(I.f.birth[v]);
        divisions.push_back(I.f.divisions[v]);
      }
      b->node_off.push_back(b->node_off.back() + n + 1);
      b->cell_off.push_back(b->cell_off.back() + n + 1);        // one epoch
      rates.push_back(I.snv); rates.push_back(I.indel);
      pre_s.push_back(I.n_pre_snv); pre_i.push_back(I.n_pre_id);
    }
    require(b->node_off.back() < (1u << 31), "batch forests too large");
    // signatures: the plain path's class thresholds (classes without indexed positions masked)
    std::vector<uint32_t> sig_cdf[2];
    for (int ty = 0; ty < 2; ++ty) {
      const uint32_t NC = ty == 0 ? 96 : 83;
      sig_cdf[ty].assign(uint64_t(ns[ty]) * NC, 0);
      std::vector<uint8_t> usable(ns[ty], 0);
      for (uint32_t s = 0; s < e->n_sig[ty]; ++s) {
        std::vector<double> w(NC);
        for (uint32_t k = 0; k < NC; ++k) {
          const uint32_t list = ty == 0 ? uint32_t(pg::sbs_class_context(int(k))) : k;
          const uint32_t len = ty == 0 ? e->ctx_len[list] : e->id_len[list];
          w[k] = len > 0 ? e->sigs[ty][uint64_t(s) * NC + k] : 0.0;
          if (w[k] > 0) usable[s] = 1;
        }
        const auto thr = cdf_thresholds(w);
        std::copy(thr.begin(), thr.end(), sig_cdf[ty].begin() + uint64_t(s) * NC);
      }
      // per-instance exposure rows: epoch 0, then the preneoplastic row
      std::vector<uint32_t> expo(uint64_t(n_inst) * 2 * ns[ty], 0);
      for (uint32_t i = 0; i < n_inst; ++i) {
        const BatchInst& I = b->in[i];
        const std::vector<double>& w = ty == 0 ? I.sbs_w : I.id_w;
        const double rate = ty == 0 ? I.snv : I.indel;
        const uint32_t n_pre = ty == 0 ? I.n_pre_snv : I.n_pre_id;
        if (rate > 0 || n_pre > 0) require(e->n_sig[ty] > 0, ty == 0 ? "no SBS signatures set" : "no ID signatures set");
        bool any = false;
        for (uint32_t k = 0; k < ns[ty]; ++k) {
          if (w[k] > 0) { any = true; if (!usable[k]) throw DomainError("signature " + std::to_string(k) + " has no class with indexed positions"); }
        }
        if (rate > 0) require(any, ty == 0 ? "an instance has no SBS exposure" : "an instance has no ID exposure");
        auto thr = cdf_thresholds(w);
        std::copy(thr.begin(), thr.end(), expo.begin() + (uint64_t(i) * 2) * ns[ty]);
        if (n_pre > 0) {
          const uint32_t ps = ty == 0 ? pre_sbs_sig : pre_id_sig;
          require(ps < e->n_sig[ty], "unknown preneoplastic signature");
          require(usable[ps], "the preneoplastic signature has no class with indexed positions");
          std::vector<double> pw(ns[ty], 0.0);
          pw[ps] = 1.0;
          thr = cdf_thresholds(pw);
          std::copy(thr.begin(), thr.end(), expo.begin() + (uint64_t(i) * 2 + 1) * ns[ty]);
        }
      }
      b->sig_cdf[ty] = upload(P, sig_cdf[ty], st);
      b->expo_cdf[ty] = upload(P, expo, st);
    }
    // device forests and shared tables
    b->parent = upload(P, parent, st); b->birth = upload(P, birth, st); b->divisions = upload(P, divisions, st);
    b->rates = upload(P, rates, st);
    b->epoch0 = upload(P, std::vector<double>{0.0, 0.0}, st);
    b->node_size = upload(P, std::vector<double>(max_n + 1, 2.0 * double(e->G)), st);
    b->zeros = upload(P, std::vector<uint32_t>(max_n + 2, 0u), st);
    b->gc_seg_off = upload(P, std::vector<uint32_t>{0u, 1u}, st);
    b->gc_seg_start = upload(P, std::vector<uint32_t>{0u}, st);
    b->gc_seg_end = upload(P, std::vector<uint32_t>{uint32_t(e->G)}, st);
    b->gc_seg_ioff = upload(P, std::vector<uint32_t>{0u}, st);
    b->gc_seg_icnt = upload(P, std::vector<uint32_t>{2u}, st);
    b->gc_inst = upload(P, std::vector<uint16_t>{0u, 1u}, st);
    std::vector<pg::PlaceTables> tabs(n_inst);
    for (uint32_t i = 0; i < n_inst; ++i) {
      pg::PlaceTables& t = tabs[i];
      const uint32_t base = b->node_off[i] - i;      // node arrays hold n (not n + 1) rows per instance
      t.n_nodes = b->in[i].f.n;
      t.parent = b->parent.p + base; t.birth = b->birth.p + base; t.species = b->zeros.p;
      t.divisions = b->divisions.p + base;
      t.n_epochs = 1; t.epoch_start = b->epoch0.p;
      t.snv_rate = b->rates.p + 2 * i; t.indel_rate = b->rates.p + 2 * i + 1; t.cna_rate = b->epoch0.p;
      t.node_size = b->node_size.p;
      t.gc = {1u, b->zeros.p, b->gc_seg_off.p, b->gc_seg_start.p, b->gc_seg_end.p, b->gc_seg_ioff.p,
              b->gc_seg_icnt.p, b->gc_inst.p};
      t.n_sbs_sigs = ns[0]; t.n_id_sigs = ns[1];
      t.sbs_expo_cdf = b->expo_cdf[0].p + uint64_t(i) * 2 * ns[0];
      t.id_expo_cdf = b->expo_cdf[1].p + uint64_t(i) * 2 * ns[1];
      t.sbs_sig_cdf = b->sig_cdf[0].p; t.id_sig_cdf = b->sig_cdf[1].p;
      t.genome = e->genome.p;
      t.ctx_off = e->ctx_off_d.p; t.ctx_len = e->ctx_len_d.p; t.ctx_lists = e->ctx_lists.p;
      t.id_off = e->id_off_d.p; t.id_len = e->id_len_d.p; t.id_lists = e->id_lists.p;
    }
    b->tabs = upload(P, tabs, st);
    b->node_off_d = upload(P, b->node_off, st); b->cell_off_d = upload(P, b->cell_off, st);
    b->pre_snv_d = upload(P, pre_s, st); b->pre_id_d = upload(P, pre_i, st);
    b->pkeys = DBuf<pg::Key>(P, n_inst); b->skeys = DBuf<pg::Key>(P, n_inst);
    b->rec_off_d = DBuf<uint32_t>(P, n_inst + 1); b->n_all_d = DBuf<uint32_t>(P, 1);
    ck(cudaStreamSynchronize(st), "batch create");
    engine_retain(e);
    *out = b.release();
  });
}

pg_status pg_batch_destroy(pg_batch* b) {
  return guarded([&] {
    if (!b) return;
    pg_engine* e = b->eng;
    cudaSetDevice(e->device);
    cudaStreamSynchronize(e->st);
    delete b;
    engine_release(e);
  });
}

pg_status pg_batch_run(pg_batch* b, const uint64_t* place_seed, const uint64_t* seq_seed) {
  return guarded([&] {
    require(b && place_seed && seq_seed, "NULL argument");
    pg_engine* e = b->eng;
    select_device(e);
    cudaStream_t st = e->st;
    Timer t1(st);
    batch_place(b, place_seed);
    b->place_ms = t1.stop();
    if (!b->layout_ok) batch_layout(b);
    const uint32_t B = uint32_t(b->in.size());
    std::vector<pg::Key> keys(B);
    for (uint32_t i = 0; i < B; ++i) keys[i] = pg::make_key(seq_seed[i]);
    ck(cudaMemcpyAsync(b->skeys.p, keys.data(), sizeof(pg::Key) * B, cudaMemcpyHostToDevice, st), "keys");
    Timer t2(st);
    batch_sequence(b);
    b->seq_ms = t2.stop();
    ck(cudaGetLastError(), "batch kernels");
  });
}

pg_status pg_batch_tile_sizes(const pg_batch* b, uint32_t* tile) {
  return guarded([&] {
    require(b && tile, "NULL argument");
    for (size_t i = 0; i < b->in.size(); ++i) tile[i] = b->in[i].T;
  });
}

pg_status pg_batch_set_tile_sizes(pg_batch* b, const uint32_t* tile) {
  return guarded([&] {
    require(b && tile, "NULL argument");
    for (size_t i = 0; i < b->in.size(); ++i) require(tile[i] >= 64 && tile[i] <= (1u << 24), "tile_size must be in [64, 2^24]");
    for (size_t i = 0; i < b->in.size(); ++i) b->in[i].T = tile[i];
    b->layout_ok = false;
  });
}

pg_status pg_batch_autotune(pg_batch* b, const uint64_t* place_seed, const uint64_t* seq_seed, uint32_t* tile_out) {
  return guarded([&] {
    require(b && place_seed && seq_seed, "NULL argument");
    pg_engine* e = b->eng;
    select_device(e);
    cudaStream_t st = e->st;
    const uint32_t B = uint32_t(b->in.size());
    std::vector<uint32_t> base(B);
    for (uint32_t i = 0; i < B; ++i) {
      uint32_t ins_min = 0;
      std::vector<uint32_t> thr;
      base[i] = batch_default_tile(b->in[i].cfg, batch_span(b->in[i].cfg, ins_min, thr));
    }
    batch_place(b, place_seed);
    std::vector<pg::Key> keys(B);
    for (uint32_t i = 0; i < B; ++i) keys[i] = pg::make_key(seq_seed[i]);
    ck(cudaMemcpyAsync(b->skeys.p, keys.data(), sizeof(pg::Key) * B, cudaMemcpyHostToDevice, st), "keys");
    // candidates: multiples of each instance's analytic size (the fragment
    // count of a tile 4 sigma below one shared-memory batch; 1.5 and 2 give
    // tiles of two batches), timed as one whole persistent launch; the best
    // of two repetitions counts
    const double mult[] = {0.5, 0.75, 1.0, 1.25, 1.5, 2.0};
    double best = 1e300;
    std::vector<uint32_t> best_T(B);
    for (double m : mult) {
      for (uint32_t i = 0; i < B; ++i) {
        uint32_t ins_min = 0;
        std::vector<uint32_t> thr;
        const uint32_t span = batch_span(b->in[i].cfg, ins_min, thr);
        const double t = std::min(double(base[i]) * m, double(16384 - 1 - span));
        b->in[i].T = uint32_t(std::max(256.0, std::floor(t / 64.0) * 64.0));
      }
      b->layout_ok = false;
      batch_layout(b);
      double ms = 1e300;
      for (int rep = 0; rep < 2; ++rep) {
        Timer t(st);
        batch_sequence(b);
        ms = std::min(ms, double(t.stop()));
      }
      if (ms < best) { best = ms; for (uint32_t i = 0; i < B; ++i) best_T[i] = b->in[i].T; }
    }
    for (uint32_t i = 0; i < B; ++i) b->in[i].T = best_T[i];
    b->layout_ok = false;
    if (tile_out) for (uint32_t i = 0; i < B; ++i) tile_out[i] = best_T[i];
  });
}

pg_status pg_batch_dims(const pg_batch* b, uint32_t inst, uint64_t* n_mut, uint32_t* n_samples, uint64_t* n_reads) {
  return guarded([&] {
    require(b != nullptr, "NULL handle");
    require(inst < b->in.size(), "instance index out of range");
    if (n_mut) *n_mut = b->in[inst].M;
    if (n_samples) *n_samples = b->in[inst].n_samples;
    if (n_reads) *n_reads = b->in[inst].n_reads;
  });
}

pg_status pg_batch_copy(const pg_batch* bc, uint32_t inst, uint32_t* locus, uint32_t* edge, uint32_t* aux,
                        uint8_t* cls, uint8_t* sig, uint16_t* allele, uint8_t* kind, uint8_t* nature, int32_t* alt,
                        int32_t* depth) {
  return guarded([&] {
    require(bc != nullptr, "NULL handle");
    auto* b = const_cast<pg_batch*>(bc);
    require(inst < b->in.size(), "instance index out of range");
    require(b->layout_ok || (!alt && !depth), "the batch has not been run");
    pg_engine* e = b->eng;
    select_device(e);
    cudaStream_t st = e->st;
    const uint64_t r0 = b->rec_off.empty() ? 0 : b->rec_off[inst], m = b->in[inst].M;
    auto cp = [&](void* dst, const void* src, size_t elem) {
      if (dst && m) ck(cudaMemcpyAsync(dst, static_cast<const char*>(src) + r0 * elem, m * elem,
                                       cudaMemcpyDeviceToHost, st), "copy");
    };
    cp(locus, b->s_locus.p, 4); cp(edge, b->s_edge.p, 4); cp(aux, b->s_aux.p, 4);
    cp(cls, b->s_cls.p, 1); cp(sig, b->s_sig.p, 1); cp(allele, b->s_allele.p, 2);
    cp(kind, b->s_kind.p, 1); cp(nature, b->s_nature.p, 1);
    const pg::SeqInst& S = b->sinst.empty() ? pg::SeqInst{} : b->sinst[inst];
    for (uint32_t s = 0; s < b->in[inst].n_samples && m; ++s) {
      const uint64_t row = S.count_off + uint64_t(s) * S.count_stride;
      if (alt) ck(cudaMemcpyAsync(alt + s * m, b->alt.p + row, m * 4, cudaMemcpyDeviceToHost, st), "copy");
      if (depth) ck(cudaMemcpyAsync(depth + s * m, b->depth.p + row, m * 4, cudaMemcpyDeviceToHost, st), "copy");
    }
    ck(cudaStreamSynchronize(st), "copy");
  });
}

pg_status pg_batch_kernel_ms(const pg_batch* b, float* place_ms, float* seq_ms) {
  return guarded([&] {
    require(b != nullptr, "NULL handle");
    if (place_ms) *place_ms = b->place_ms;
    if (seq_ms) *seq_ms = b->seq_ms;
  });
}
