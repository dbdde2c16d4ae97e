"""GPU parity: the CUDA path against the oracle.

* bit-exact (integers) against the Philox replay: genome, index lists,
  placed mutations (locus, edge, class, signature, allele, alt/indel
  descriptor, nature) and sequencing alt/depth tables;
* in distribution against the std::mt19937_64 reference-engine flavour over
  64 seeds (chi-square on contexts, KS on per-edge counts and on VAF), p > 0.01;
* edge cases of the reference API.
"""
import numpy as np
import pytest
from scipy import stats

pytestmark = pytest.mark.gpu


def make_pair(orc, w, **kw):
    from process_gb300 import synth
    eng = synth.build_engine(w)
    o = orc.OracleEngine.like(w, **kw) if kw else orc.OracleEngine.like(w)
    return eng, o


def oracle_species(e, forest):
    return np.array([e.species[(m, ep)] for m, ep in zip(forest.mutant, forest.epistate)], dtype=np.uint32)


def assert_tables_equal(a, b):
    assert len(a["locus"]) == len(b["locus"])
    for k in ("locus", "edge", "aux", "cls", "sig", "allele", "kind", "nature"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


def test_genome_and_index_bit_exact(gpu_lib, orc):
    from process_gb300 import GenomeSpec, MutationEngine
    g = GenomeSpec(["1", "2", "3", "4"], [70_001, 1_000, 333_333, 5], seed=77, gc=0.41)
    for cs, cap in ((1, 500000), (7, 300)):
        eng = MutationEngine(g, context_sampling=cs, max_repetition_storage=cap)
        o = orc.OracleEngine(g.chr_lengths, None, g.seed, g.gc, context_sampling=cs, max_rep=cap)
        np.testing.assert_array_equal(eng.read_genome(), o.read_genome())
        gi, oi = eng.index_info(), o.index_info()
        np.testing.assert_array_equal(gi["ctx_total"], oi["ctx_total"])
        np.testing.assert_array_equal(gi["id_total"], oi["id_total"])
        np.testing.assert_array_equal(gi["ctx_stored"], oi["ctx_stored"])
        np.testing.assert_array_equal(gi["id_stored"], oi["id_stored"])
        for c in range(32):
            np.testing.assert_array_equal(eng.read_index(0, c), o.read_index(0, c))
        for c in range(83):
            np.testing.assert_array_equal(eng.read_index(1, c), o.read_index(1, c))


def test_explicit_bases_genome(gpu_lib, orc):
    from process_gb300 import GenomeSpec, MutationEngine
    rng = np.random.default_rng(5)
    bases = rng.integers(0, 4, 50_000).astype(np.uint8)
    bases[1000:1040] = 1            # a long homopolymer run
    bases[2000:2030] = np.tile([0, 3], 15)   # a dinucleotide repeat
    g = GenomeSpec(["a", "b"], [20_000, 30_000], bases=bases)
    eng = MutationEngine(g, context_sampling=1, max_repetition_storage=1000)
    o = orc.OracleEngine(g.chr_lengths, bases, context_sampling=1, max_rep=1000)
    np.testing.assert_array_equal(eng.read_genome(), bases)
    for c in range(83):
        np.testing.assert_array_equal(eng.read_index(1, c), o.read_index(1, c))


@pytest.mark.parametrize("infinite", [True, False])
def test_placement_bit_exact_3mbp(gpu_lib, orc, infinite):
    from process_gb300 import synth
    w = synth.plain_3mbp(seed=3, n_leaves=800)
    eng, o = make_pair(orc, w)
    eng.infinite_sites_model = infinite
    o.set_infinite_sites(infinite)
    for seed in (1, 2, 12345678901):
        pf = eng.place_mutations(w.forest, 100, 10, seed=seed)
        ot = o.place(w.forest, oracle_species(o, w.forest), 100, 0, 10, 0, seed=seed).table()
        assert_tables_equal(pf.table(), ot)


def test_placement_bit_exact_epochs_drivers(gpu_lib, orc):
    """Three exposure epochs with per-epoch rates, compressed edges and drivers."""
    from process_gb300 import SNV, Mutation, synth
    w = synth.full_scale(seed=4, n_leaves_per_sample=300, genome_scale=2e-3)
    w.mutants = [("A", w.mutants[0][1], []),
                 ("B", w.mutants[1][1], [SNV("1", 1000, "T", allele=1), Mutation("2", 500, "A", "ACG"),
                                         SNV("3", 77, "G")])]
    eng, o = make_pair(orc, w)   # the oracle reads the "?" reference bases from its genome
    for seed in (5, 6):
        pf = eng.place_mutations(w.forest, 1000, 100, seed=seed)
        ot = o.place(w.forest, oracle_species(o, w.forest), 1000, 0, 100, 0, seed=seed).table()
        t = pf.table()
        assert_tables_equal(t, ot)
        assert (t["nature"] == 1).sum() == 3
        assert len(np.unique(t["locus"])) == len(t["locus"])


SEQ_CASES = [
    dict(coverage=30, read_size=150, insert_size_mean=350, insert_size_stddev=10, error_rate=1e-3, purity=0.7),
    dict(coverage=20, read_size=100, insert_size_mean=350, insert_size_stddev=30, insert_model="normal",
         error_rate=0.0, purity=1.0, preneoplastic_in_normal=True),
    dict(coverage=25, read_size=150, insert_size_mean=0, error_rate=5e-2, purity=0.5, with_normal_sample=False),
    dict(coverage=15, read_size=150, insert_size_mean=300, insert_size_stddev=5, error_rate=1e-3, purity=0.0,
         chromosomes=["3", "1"]),
    dict(coverage=40, read_size=150, insert_size_mean=250, insert_size_stddev=15, error_rate=1e-2,
         normal_only=True, preneoplastic_in_normal=True),
]


@pytest.mark.parametrize("case", range(len(SEQ_CASES)))
def test_sequencing_bit_exact(gpu_lib, orc, case):
    from process_gb300 import synth
    from process_gb300.engine import seq_cfg, sequence_counts
    cfg = dict(SEQ_CASES[case])
    w = synth.plain_3mbp(seed=8, n_leaves=400)
    eng, o = make_pair(orc, w)
    pf = eng.place_mutations(w.forest, 200, 20, seed=21)
    op = o.place(w.forest, oracle_species(o, w.forest), 200, 0, 20, 0, seed=21)
    assert_tables_equal(pf.table(), op.table())
    for tile in (2048, 16384):
        res = sequence_counts(pf, 99, tile_size=tile, **cfg)
        alt, dep = res.counts()
        c, _ = seq_cfg(chr_index=eng._chr_index, tile_size=tile, **cfg)
        oalt, odep, oreads = op.sequence(c, 99, flavour=0)
        np.testing.assert_array_equal(dep, odep)
        np.testing.assert_array_equal(alt, oalt)
        assert res.dims()[2] == oreads


def test_distribution_against_reference_engine(gpu_lib, orc):
    """64 seeds: chi-square on SBS context counts, KS on per-edge SNV counts
    and on VAF, GPU vs the std::mt19937_64 flavour; p > 0.01."""
    from process_gb300 import synth
    from process_gb300.engine import seq_cfg, sequence_counts
    w = synth.plain_3mbp(seed=11, n_leaves=300)
    w.genome.chr_lengths = [300_000] * 3
    eng, o = make_pair(orc, w)
    sp = oracle_species(o, w.forest)
    n = w.forest.num_of_nodes
    cfg = dict(coverage=30, read_size=150, insert_size_mean=350, insert_size_stddev=10, error_rate=1e-3,
               purity=0.8, with_normal_sample=False)
    c, _ = seq_cfg(chr_index=eng._chr_index, tile_size=16384, **cfg)
    g_ctx, m_ctx = np.zeros(96), np.zeros(96)
    g_edge, m_edge, g_vaf, m_vaf = [], [], [], []
    for s in range(64):
        pf = eng.place_mutations(w.forest, 50, 5, seed=1000 + s)
        t = pf.table()
        op = o.place(w.forest, sp, 50, 0, 5, 0, seed=1000 + s, flavour=1)
        ot = op.table()
        for tab, ctx, edges in ((t, g_ctx, g_edge), (ot, m_ctx, m_edge)):
            snv = tab["kind"] == 0
            ctx += np.bincount(tab["cls"][snv & (tab["nature"] == 0)], minlength=96)
            edges.append(np.bincount(tab["edge"][snv & (tab["nature"] == 0)], minlength=n))
        if s < 16:
            alt, dep = sequence_counts(pf, 500 + s, tile_size=16384, **cfg).counts()
            oalt, odep, _ = op.sequence(c, 500 + s, flavour=1)
            for a, d, out, tab in ((alt, dep, g_vaf, t), (oalt, odep, m_vaf, ot)):
                keep = (d[0] >= 10) & (tab["nature"] == 2)
                out.append(a[0][keep] / d[0][keep])
    keep = (g_ctx + m_ctx) > 0
    assert stats.chi2_contingency(np.vstack([g_ctx[keep], m_ctx[keep]]))[1] > 0.01
    assert stats.ks_2samp(np.concatenate(g_edge), np.concatenate(m_edge)).pvalue > 0.01
    assert stats.ks_2samp(np.concatenate(g_vaf), np.concatenate(m_vaf)).pvalue > 0.01


def test_edge_cases(gpu_lib, orc):
    from process_gb300 import (BasicIlluminaSequencer, ErrorlessIlluminaSequencer, ProcessError, simulate_seq,
                               simulate_normal_seq, synth)
    from process_gb300.engine import sequence_counts
    w = synth.plain_3mbp(seed=2, n_leaves=200)
    eng, _ = make_pair(orc, w)
    pf = eng.place_mutations(w.forest, 100, 10, seed=1)
    # error rate 0 is the error-less sequencer
    a = simulate_seq(pf, BasicIlluminaSequencer(0.0), coverage=10, seed=3)["mutations"]
    b = simulate_seq(pf, ErrorlessIlluminaSequencer(), coverage=10, seed=3)["mutations"]
    for k in b:
        np.testing.assert_array_equal(a[k], b[k])
    # purity 0: tumour reads all come from normal cells: no passenger is seen without errors
    alt, dep = sequence_counts(pf, 4, coverage=10, purity=0.0, error_rate=0.0).counts()
    assert alt[0].sum() == 0 and dep[0].sum() > 0
    # single-end reads (insert_size_mean = 0)
    alt, dep = sequence_counts(pf, 4, coverage=12, insert_size_mean=0).counts()
    assert abs(dep.mean() - 12) < 1.0
    # variance above the mean: the reference's binomial insert model throws
    with pytest.raises(ProcessError, match="variance"):
        simulate_seq(pf, coverage=1, insert_size_mean=350, insert_size_stddev=30, seed=1)
    # ... the normal model expresses it
    df = simulate_seq(pf, coverage=5, insert_size_mean=350, insert_size_stddev=30, insert_model="normal",
                      seed=1)["mutations"]
    assert {"chr", "chr_pos", "ref", "alt", "causes", "classes", "S_1.occurrences", "S_1.coverage", "S_1.VAF",
            "normal_sample.VAF"} <= set(df)
    # coverage 0: no reads, no observed mutation
    alt, dep = sequence_counts(pf, 4, coverage=0).counts()
    assert dep.sum() == 0
    # normal sequencing sees only preneoplastic mutations (when asked) and errors
    n = simulate_normal_seq(pf, coverage=20, with_preneoplastic=True, write_SAM=False, seed=2)["mutations"]
    assert set(n["classes"]) <= {"preneoplastic", "passenger"}
    assert list(n) == ["chr", "chr_pos", "ref", "alt", "causes", "classes", "normal_sample.occurrences",
                       "normal_sample.coverage", "normal_sample.VAF"]


def test_full_size_properties(gpu_lib):
    """The full-scale workload (3.1 Gbp, 3 x 1e4 leaves, 100x): properties
    that hold at any size — sorted unique loci, mean depth at the coverage,
    clonal VAF at purity/2, an error-only alt rate in the normal sample."""
    from process_gb300 import synth
    from process_gb300.engine import sequence_counts
    w = synth.full_scale(seed=2)
    w.mutants = [(n, r, []) for n, r, _ in w.mutants]     # copy number 2 everywhere
    eng = synth.build_engine(w)
    pf = eng.place_mutations(w.forest, w.n_pre_snv, w.n_pre_indel, seed=7)
    t = pf.table()
    assert np.all(np.diff(t["locus"].astype(np.int64)) > 0)
    assert 2e6 < len(t["locus"]) < 1e8
    res = sequence_counts(pf, 9, **w.seq)
    alt, dep = res.counts()
    assert abs(dep[:3].mean() - 100) < 2
    pre = (t["nature"] == 2) & (t["kind"] == 0)
    vaf = alt[0, pre].sum() / dep[0, pre].sum()
    assert abs(vaf - 0.35) < 0.02
    # normal sample: tumour passengers only through errors (rate e/3)
    pas = (t["nature"] == 0) & (t["kind"] == 0)
    rate = alt[3, pas].sum() / dep[3, pas].sum()
    assert rate < 1e-3


def test_full_size_copy_number_properties(gpu_lib):
    """The full-scale workload with its 20 CNAs and WGD branch: three
    genotype classes, one WGD record, passengers per edge scaled by the
    allelic size of the edge's genome (about 2x on the WGD branch), sorted
    unique loci and depth near the coverage."""
    from process_gb300 import synth
    from process_gb300.engine import sequence_counts
    w = synth.full_scale(seed=2)
    eng = synth.build_engine(w)
    pf = eng.place_mutations(w.forest, w.n_pre_snv, w.n_pre_indel, seed=7)
    t = pf.table()
    assert np.all(np.diff(t["locus"].astype(np.int64)) > 0)
    _, n_cls, cn_max = pf.node_classes()
    assert n_cls == 3 and cn_max >= 4
    c = pf.cna_table()
    assert (c["type"] == 2).sum() == 1 and len(c["type"]) <= 24
    w0 = synth.full_scale(seed=2)
    w0.mutants = [(n, r, []) for n, r, _ in w0.mutants]
    t0 = synth.build_engine(w0).place_mutations(w0.forest, w0.n_pre_snv, w0.n_pre_indel, seed=7).table()
    n = w.forest.num_of_nodes
    per = np.bincount(t["edge"][t["nature"] == 0], minlength=n)[:n].astype(float)
    per0 = np.bincount(t0["edge"][t0["nature"] == 0], minlength=n)[:n].astype(float)
    b = np.asarray(w.forest.mutant) == "B"
    assert 1.7 < per[b].sum() / per0[b].sum() < 2.3
    assert 0.85 < per[~b].sum() / per0[~b].sum() < 1.15
    res = sequence_counts(pf, 9, **w.seq)
    alt, dep = res.counts()
    assert 80 < dep[:3].mean() < 130


def test_unknown_bases_genome(gpu_lib, orc, tmp_path):
    """A genome with unknown bases (N runs, an isolated N, N across a
    chromosome boundary): the same genome codes (4 for N) and index lists as
    the oracle, placement and sequencing bit-exact, no mutation on or
    anchored at an N, and N in the SAM reads over them."""
    from pathlib import Path

    from process_gb300 import simulate_seq, synth
    from process_gb300.engine import seq_cfg, sequence_counts
    w = synth.plain_3mbp(seed=19, n_leaves=150)
    w.genome.chr_lengths = [60_000, 40_000, 40_000]
    rng = np.random.default_rng(4)
    b = rng.integers(0, 4, 140_000).astype(np.uint8)
    b[1000:3000] = 4
    b[7777] = 4
    b[59_990:60_010] = 4
    b[120_000:121_500] = 4
    w.genome.bases = b
    eng, o = make_pair(orc, w)
    np.testing.assert_array_equal(eng.read_genome(), b)
    np.testing.assert_array_equal(eng.read_genome(), o.read_genome())
    for c in range(32):
        np.testing.assert_array_equal(eng.read_index(0, c), o.read_index(0, c))
    for c in range(83):
        np.testing.assert_array_equal(eng.read_index(1, c), o.read_index(1, c))
    assert int(eng.gather_bases(np.array([7777], dtype=np.uint32))[0]) == 4
    pf = eng.place_mutations(w.forest, 100, 10, seed=6)
    op = o.place(w.forest, oracle_species(o, w.forest), 100, 0, 10, 0, seed=6)
    assert_tables_equal(pf.table(), op.table())
    loc = pf.table()["locus"].astype(np.int64)
    assert not (b[loc] == 4).any()
    cfg = dict(coverage=20, read_size=150, insert_size_mean=350, insert_size_stddev=10, error_rate=1e-3, purity=0.8)
    alt, dep = sequence_counts(pf, 12, tile_size=4096, **cfg).counts()
    c, _ = seq_cfg(chr_index=eng._chr_index, tile_size=4096, **cfg)
    oalt, odep, _ = op.sequence(c, 12, flavour=0)
    np.testing.assert_array_equal(dep, odep)
    np.testing.assert_array_equal(alt, oalt)
    out = tmp_path / "sam"
    simulate_seq(pf, coverage=5, write_SAM=True, output_dir=str(out), insert_size_mean=350, insert_size_stddev=10,
                 seed=2)
    n_count = 0
    for f in sorted(Path(out).glob("*.sam")):
        for line in f.read_text().splitlines():
            if not line.startswith("@"):
                n_count += line.split("\t")[9].count("N")
    assert n_count > 0


# ---------------------------------------------------------------- named workloads at their own sizes
def _replay_counts(o_placed, eng, res, seq, seed):
    """The oracle's replay of a sequencing call, at the tile size the call used."""
    from process_gb300.engine import seq_cfg
    c, _ = seq_cfg(chr_index=eng._chr_index, tile_size=res.tile_size(), **seq)
    return o_placed.sequence(c, seed, flavour=0)


@pytest.mark.parametrize("seed", [1, 2])
def test_plain_3mbp_workload_bit_exact(gpu_lib, orc, seed):
    """The 3 x 1 Mbp workload exactly as named: ~2.5k leaves (species A and
    the A+ subclone), SNV 1e-6 / indel 1e-7 per base per division, one SBS
    and one ID signature, 100 + 10 preneoplastic mutations; 80x paired
    150 bp reads with insert Normal(350, 30) and error rate 1e-3, at the
    automatic tile size.  Whole placed table and alt/depth tables bit for
    bit against the Philox replay."""
    from process_gb300 import synth
    from process_gb300.engine import sequence_counts
    w = synth.plain_3mbp(seed=1)
    assert w.forest.is_leaf.sum() == 2500
    assert w.seq["insert_model"] == "normal" and w.seq["insert_size_stddev"] == 30 and w.seq["coverage"] == 80
    eng, o = make_pair(orc, w)
    pf = eng.place_mutations(w.forest, w.n_pre_snv, w.n_pre_indel, seed=seed)
    op = o.place(w.forest, oracle_species(o, w.forest), w.n_pre_snv, 0, w.n_pre_indel, 0, seed=seed)
    t = pf.table()
    assert_tables_equal(t, op.table())
    assert len(t["locus"]) > 20_000
    res = sequence_counts(pf, 100 + seed, **w.seq)
    alt, dep = res.counts()
    oalt, odep, oreads = _replay_counts(op, eng, res, w.seq, 100 + seed)
    np.testing.assert_array_equal(dep, odep)
    np.testing.assert_array_equal(alt, oalt)
    assert res.dims()[2] == oreads > 3_000_000


def test_full_scale_slice_bit_exact(gpu_lib, orc):
    """1% of the 3.1 Gbp workload (31 Mbp over the same 24 chromosomes, the
    20 CNA segments and the WGD branch scaled with it) with the full
    3 x 1e4-leaf forest, 3 epochs, 100x, purity 0.7, error rate 1e-3: the
    slice the CPU baseline times.  Placement, CNA records, genotype classes
    and the alt/depth tables of all four samples bit for bit against the
    Philox replay."""
    from process_gb300 import synth
    from process_gb300.engine import sequence_counts
    w = synth.full_scale(seed=2, genome_scale=0.01)
    assert w.forest.is_leaf.sum() == 30_000
    eng, o = make_pair(orc, w)
    pf = eng.place_mutations(w.forest, w.n_pre_snv, w.n_pre_indel, seed=7)
    op = o.place(w.forest, oracle_species(o, w.forest), w.n_pre_snv, 0, w.n_pre_indel, 0, seed=7)
    assert_tables_equal(pf.table(), op.table())
    gc, oc = pf.cna_table(), op.cna_table()
    for k in oc:
        np.testing.assert_array_equal(gc[k], oc[k], err_msg=k)
    assert (gc["type"] == 2).sum() == 1
    g_cls, g_n, g_max = pf.node_classes()
    o_cls, o_n, o_max = op.node_classes(w.forest.num_of_nodes)
    np.testing.assert_array_equal(g_cls, o_cls)
    assert (g_n, g_max) == (o_n, o_max) and g_n >= 3
    res = sequence_counts(pf, 9, **w.seq)
    alt, dep = res.counts()
    oalt, odep, oreads = _replay_counts(op, eng, res, w.seq, 9)
    assert alt.shape[0] == 4
    np.testing.assert_array_equal(dep, odep)
    np.testing.assert_array_equal(alt, oalt)
    assert res.dims()[2] == oreads


def test_distribution_plain_3mbp_workload(gpu_lib, orc):
    """64 seeds on the 3 x 1 Mbp, ~2.5k-leaf workload (80x, insert
    Normal(350, 30), error 1e-3): chi-square on SBS context counts, KS on
    per-edge passenger SNV counts and on VAF, GPU vs the std::mt19937_64
    flavour; p > 0.01."""
    from process_gb300 import synth
    from process_gb300.engine import sequence_counts
    w = synth.plain_3mbp(seed=11)
    eng, o = make_pair(orc, w)
    sp = oracle_species(o, w.forest)
    n = w.forest.num_of_nodes
    seq = dict(w.seq, with_normal_sample=False)
    g_ctx, m_ctx = np.zeros(96), np.zeros(96)
    g_edge, m_edge, g_vaf, m_vaf = [], [], [], []
    for s in range(64):
        pf = eng.place_mutations(w.forest, w.n_pre_snv, w.n_pre_indel, seed=3000 + s)
        t = pf.table()
        op = o.place(w.forest, sp, w.n_pre_snv, 0, w.n_pre_indel, 0, seed=3000 + s, flavour=1)
        ot = op.table()
        for tab, ctx, edges in ((t, g_ctx, g_edge), (ot, m_ctx, m_edge)):
            snv = (tab["kind"] == 0) & (tab["nature"] == 0)
            ctx += np.bincount(tab["cls"][snv], minlength=96)
            edges.append(np.bincount(tab["edge"][snv], minlength=n)[:n])
        if s < 16:
            res = sequence_counts(pf, 700 + s, **seq)
            alt, dep = res.counts()
            from process_gb300.engine import seq_cfg
            c, _ = seq_cfg(chr_index=eng._chr_index, tile_size=res.tile_size(), **seq)
            oalt, odep, _ = op.sequence(c, 700 + s, flavour=1)
            for a, d, out, tab in ((alt, dep, g_vaf, t), (oalt, odep, m_vaf, ot)):
                keep = (d[0] >= 20) & (tab["kind"] == 0) & ((tab["nature"] == 2) | (a[0] >= 3))
                out.append(a[0][keep] / d[0][keep])
    keep = (g_ctx + m_ctx) > 0
    assert stats.chi2_contingency(np.vstack([g_ctx[keep], m_ctx[keep]]))[1] > 0.01
    assert stats.ks_2samp(np.concatenate(g_edge), np.concatenate(m_edge)).pvalue > 0.01
    assert stats.ks_2samp(np.concatenate(g_vaf), np.concatenate(m_vaf)).pvalue > 0.01


def test_regions_to_avoid(gpu_lib, orc):
    """Regions to avoid (the driver catalogue of build_contex_index,
    src/mutation_engine.cpp:240-262): the SBS context index leaves their
    positions out, the ID index keeps them; index lists and placement bit
    for bit against the oracle."""
    from process_gb300 import SNV, GenomeSpec, Mutation, MutationEngine, driver_regions, synth
    w = synth.plain_3mbp(seed=23, n_leaves=200)
    w.genome.chr_lengths = [200_000, 100_000, 100_000]
    catalogue = [SNV("1", 1000, "T"), Mutation("2", 500, "ACG", "A"), SNV("3", 77, "G")]
    regions = driver_regions(catalogue) + [("1", 50_001, 20_000)]
    assert regions[1] == ("2", 500, 3)
    eng = MutationEngine(w.genome, w.sbs, w.ids, context_sampling=1, regions_to_avoid=regions)
    plain = MutationEngine(w.genome, w.sbs, w.ids, context_sampling=1)
    o = orc.OracleEngine(w.genome.chr_lengths, None, w.genome.seed, w.genome.gc, context_sampling=1)
    o.set_regions_to_avoid(regions, eng._chr_index)
    gi, oi, pi = eng.index_info(), o.index_info(), plain.index_info()
    np.testing.assert_array_equal(gi["ctx_total"], oi["ctx_total"])
    np.testing.assert_array_equal(gi["id_total"], oi["id_total"])
    np.testing.assert_array_equal(gi["id_total"], pi["id_total"])          # ID index unchanged
    assert pi["ctx_total"].sum() - gi["ctx_total"].sum() == 20_000 + 1 + 3 + 1
    off = np.concatenate([[0], np.cumsum(w.genome.chr_lengths)])
    avoided = set()
    for c, b, n in regions:
        base = off[eng._chr_index(c)] + b - 1
        avoided.update(range(base, base + n))
    for c in range(32):
        lst = eng.read_index(0, c)
        np.testing.assert_array_equal(lst, o.read_index(0, c))
        assert not avoided & set(lst.tolist())
    for c in range(83):
        np.testing.assert_array_equal(eng.read_index(1, c), o.read_index(1, c))
    # placement over the index without those positions
    for name, rates, drivers in w.mutants:
        eng.add_mutant(name, rates, drivers)
    for t, coeffs in w.exposures:
        eng.add_exposure(t, coeffs)
    o2 = orc.OracleEngine.like(w)
    o2.set_regions_to_avoid(regions, eng._chr_index)
    pf = eng.place_mutations(w.forest, 40, 4, seed=2)
    ot = o2.place(w.forest, oracle_species(o2, w.forest), 40, 0, 4, 0, seed=2).table()
    assert_tables_equal(pf.table(), ot)


def test_index_cache(gpu_lib, tmp_path):
    """Index caches (the reference's .cif / .rsif files): the first engine
    writes them, the next one with the same genome, parameters and regions
    loads them and holds the same indices; a cache of another genome, other
    regions or another format version is refused."""
    import struct

    from process_gb300 import DomainError, GenomeSpec, MutationEngine, synth
    w = synth.plain_3mbp(seed=24, n_leaves=50)
    g = GenomeSpec(["1", "2"], [150_000, 80_000], seed=5, gc=0.45)
    d = tmp_path / "cache"
    regions = [("1", 101, 50)]
    a = MutationEngine(g, w.sbs, w.ids, context_sampling=3, max_repetition_storage=1000, regions_to_avoid=regions,
                       index_cache_dir=str(d))
    files = sorted(p.name for p in d.iterdir())
    assert files == ["context_index_3.pgcif", "rs_index_1000.pgrsif"]
    b = MutationEngine(g, w.sbs, w.ids, context_sampling=3, max_repetition_storage=1000, regions_to_avoid=regions,
                       index_cache_dir=str(d))
    ia, ib = a.index_info(), b.index_info()
    for k in ia:
        np.testing.assert_array_equal(ia[k], ib[k], err_msg=k)
    for c in range(32):
        np.testing.assert_array_equal(a.read_index(0, c), b.read_index(0, c))
    for c in range(83):
        np.testing.assert_array_equal(a.read_index(1, c), b.read_index(1, c))
    with pytest.raises(DomainError, match="another reference genome"):
        MutationEngine(GenomeSpec(["1", "2"], [150_000, 80_000], seed=6, gc=0.45), w.sbs, w.ids, context_sampling=3,
                       max_repetition_storage=1000, regions_to_avoid=regions, index_cache_dir=str(d))
    with pytest.raises(DomainError, match="other regions to avoid"):
        MutationEngine(g, w.sbs, w.ids, context_sampling=3, max_repetition_storage=1000,
                       regions_to_avoid=[("1", 102, 50)], index_cache_dir=str(d))
    f = d / "rs_index_1000.pgrsif"
    raw = bytearray(f.read_bytes())
    raw[4:8] = struct.pack("<I", 7)
    f.write_bytes(bytes(raw))
    with pytest.raises(DomainError, match="format version 7"):
        MutationEngine(g, w.sbs, w.ids, context_sampling=3, max_repetition_storage=1000, regions_to_avoid=regions,
                       index_cache_dir=str(d))
