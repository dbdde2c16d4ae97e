"""GPU parity with copy-number events: driver CNAs, whole-genome doubling,
passenger CNAs drawn from candidates, avoid_homozygous_losses.  Bit-exact
against the oracle's Philox replay: genotype classes, applied CNA records,
placed mutations and sequencing alt/depth tables."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _workload(seed, n_leaves, cna_rate=3e-9):
    from process_gb300 import CNA, SNV, WGD, synth
    w = synth.plain_3mbp(seed=seed, n_leaves=n_leaves)
    w.genome.chr_lengths = [600_000] * 3
    (na, ra, _), (nb, rb, _) = w.mutants
    w.mutants = [
        (na, dict(ra, CNA=cna_rate), [SNV("1", 1000, "T", allele=0), CNA("A", "2", 100_001, 200_000),
                                      WGD, CNA("D", "3", 500_001, 50_000, allele=1)]),
        (nb, dict(rb, CNA=cna_rate), [CNA("D", "1", 1, 300_000), SNV("2", 150_000, "G"),
                                      CNA("A", "2", 120_001, 10_000, src_allele=2)]),
    ]
    cands = [CNA("A", "1", 200_001, 30_000), CNA("D", "1", 400_001, 80_000), CNA("D", "2", 1, 50_000),
             CNA("A", "3", 10_001, 100_000), CNA("D", "3", 300_001, 5_000)]
    return w, cands


def _pair(orc, w, cands, avoid, infinite):
    from process_gb300 import synth
    eng = synth.build_engine(w)
    eng.add_passenger_CNAs(cands)
    eng.avoid_homozygous_losses = avoid
    eng.infinite_sites_model = infinite
    o = orc.OracleEngine.like(w)    # drivers included
    idx = {n: i for i, n in enumerate(w.genome.chr_names)}
    for c in cands:
        o.add_passenger_cna(idx[c.chr], c.chr_pos, c.len, c.type == "A")
    o.set_avoid_homozygous_losses(avoid)
    o.set_infinite_sites(infinite)
    return eng, o


def _species(o, forest):
    return np.array([o.species[(m, ep)] for m, ep in zip(forest.mutant, forest.epistate)], dtype=np.uint32)


def _tables_equal(a, b):
    assert len(a["locus"]) == len(b["locus"])
    for k in ("locus", "edge", "aux", "cls", "sig", "allele", "kind", "nature"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


@pytest.mark.parametrize("avoid,infinite", [(True, True), (False, True), (True, False)])
def test_cna_placement_bit_exact(gpu_lib, orc, avoid, infinite):
    w, cands = _workload(seed=3, n_leaves=500)
    eng, o = _pair(orc, w, cands, avoid, infinite)
    f = w.forest
    for seed in (1, 77):
        pf = eng.place_mutations(f, 100, 10, seed=seed)
        op = o.place(f, _species(o, f), 100, 0, 10, 0, seed=seed)
        gcls, gn, gcn = pf.node_classes()
        ocls, on, ocn = op.node_classes(f.num_of_nodes)
        np.testing.assert_array_equal(gcls, ocls)
        assert (gn, gcn) == (on, ocn)
        assert gn > 3 and gcn >= 4
        gc, oc = pf.cna_table(), op.cna_table()
        for k in oc:
            np.testing.assert_array_equal(gc[k], oc[k], err_msg=k)
        assert (gc["driver"] == 0).sum() > 0          # some passenger CNAs were applied
        _tables_equal(pf.table(), op.table())
        t = pf.table()
        assert t["allele"].max() > 1                  # mutations on copied instances


SEQ = [
    dict(coverage=25, read_size=150, insert_size_mean=350, insert_size_stddev=10, error_rate=1e-3, purity=0.7),
    dict(coverage=20, read_size=100, insert_size_mean=0, error_rate=0.0, purity=1.0, with_normal_sample=False),
]


@pytest.mark.parametrize("case", range(len(SEQ)))
def test_cna_sequencing_bit_exact(gpu_lib, orc, case):
    from process_gb300.engine import seq_cfg, sequence_counts
    w, cands = _workload(seed=4, n_leaves=300)
    eng, o = _pair(orc, w, cands, True, True)
    f = w.forest
    pf = eng.place_mutations(f, 200, 20, seed=5)
    op = o.place(f, _species(o, f), 200, 0, 20, 0, seed=5)
    _tables_equal(pf.table(), op.table())
    for tile in (2048, 16384):
        res = sequence_counts(pf, 31, tile_size=tile, **SEQ[case])
        alt, dep = res.counts()
        c, _ = seq_cfg(chr_index=eng._chr_index, tile_size=tile, **SEQ[case])
        oalt, odep, oreads = op.sequence(c, 31, flavour=0)
        np.testing.assert_array_equal(dep, odep)
        np.testing.assert_array_equal(alt, oalt)
        assert res.dims()[2] == oreads


def test_wgd_order_vaf_gpu(gpu_lib, orc):
    """The driver SNV before the doubling is on two of four alleles, after it on one."""
    from process_gb300 import SNV, WGD, synth
    from process_gb300.engine import sequence_counts
    vafs = []
    for drivers in ([SNV("1", 50_000, "T", allele=0), WGD], [WGD, SNV("1", 50_000, "T", allele=0)]):
        w = synth.plain_3mbp(seed=6, n_leaves=100)
        w.genome.chr_lengths = [200_000] * 3
        w.mutants = [(w.mutants[0][0], w.mutants[0][1], drivers), w.mutants[1]]
        eng = synth.build_engine(w)
        pf = eng.place_mutations(w.forest, 0, 0, seed=9)
        t = pf.table()
        d = np.nonzero(t["nature"] == 1)[0][0]
        alt, dep = sequence_counts(pf, 4, coverage=400, read_size=150, insert_size_mean=350, insert_size_stddev=10,
                                   error_rate=0.0, purity=1.0, with_normal_sample=False).counts()
        vafs.append(alt[0, d] / dep[0, d])
    assert abs(vafs[0] - 0.5) < 0.09 and abs(vafs[1] - 0.25) < 0.09


def _oracle_fragments(op, c, chr_off, roots):
    """Allelic-type stretches of oracle class c (an independent restatement)."""
    inst, b, e = op.class_pieces(c)
    cuts = np.unique(np.concatenate([chr_off, b, e]).astype(np.int64))
    rows = []
    for lo, hi in zip(cuts[:-1], cuts[1:]):
        cover = (b <= lo) & (lo < e)
        r = roots[inst[cover]]
        t = (int((r == 0).sum()), int((r == 1).sum()))
        ch = int(np.searchsorted(chr_off, lo, side="right") - 1)
        if rows and rows[-1][0] == ch and rows[-1][3] == t and rows[-1][2] == lo:
            rows[-1][2] = hi
        else:
            rows.append([ch, lo, hi, t])
    return [(ch, lo - chr_off[ch] + 1, hi - chr_off[ch], max(t), min(t)) for ch, lo, hi, t in rows]


def test_allelic_fragmentation_getters(gpu_lib, orc):
    w, cands = _workload(seed=6, n_leaves=200)
    eng, o = _pair(orc, w, cands, True, True)
    f = w.forest
    pf = eng.place_mutations(f, 50, 5, seed=8)
    op = o.place(f, _species(o, f), 50, 0, 5, 0, seed=8)
    chr_off = eng.chr_off.astype(np.int64)
    roots = op.inst_roots()
    cls, n_cls, _ = pf.node_classes()
    cell = pf.get_cell_allelic_fragmentation()
    leaves = np.nonzero(f.is_leaf & (f.sample >= 0))[0]
    assert len(np.unique(cell["cell_id"])) == len(leaves)
    for lf in leaves[:: max(1, len(leaves) // 25)]:
        m = cell["cell_id"] == f.cell_id[lf]
        got = [(eng.chr_names.index(c), int(b), int(e), int(mj), int(mn))
               for c, b, e, mj, mn in zip(cell["chr"][m], cell["begin"][m], cell["end"][m], cell["major"][m],
                                          cell["minor"][m])]
        assert got == _oracle_fragments(op, int(cls[lf]), chr_off, roots)
    bulk = pf.get_bulk_allelic_fragmentation()
    # every stretch's ratios sum to 1 and the stretches tile every chromosome
    keys = list(zip(bulk["chr"], bulk["begin"], bulk["end"]))
    for k in set(keys):
        assert abs(sum(r for kk, r in zip(keys, bulk["ratio"]) if kk == k) - 1.0) < 1e-12
    for ci, name in enumerate(eng.chr_names):
        spans = sorted({(b, e) for c, b, e in keys if c == name})
        assert spans[0][0] == 1 and spans[-1][1] == eng.chr_lengths[ci]
        assert all(spans[i][1] + 1 == spans[i + 1][0] for i in range(len(spans) - 1))
    info = pf.get_samples_info()
    assert np.all(info["DNA_quantity"] > 0) and np.any(info["equivalent_normal_cells"] != info["tumour_cells"])


def test_cna_distribution_against_reference_engine(gpu_lib, orc):
    """Copy-number events, 48 seeds: the GPU path against the std::mt19937_64
    flavour (which replays the events with sequential draws and draws reads by
    rejection over whole chromosomes): chi-square on SBS contexts, KS on
    per-edge passenger counts, on VAF and on depth; p > 0.01."""
    from scipy import stats

    from process_gb300.engine import seq_cfg, sequence_counts
    w, cands = _workload(seed=12, n_leaves=150, cna_rate=5e-9)
    eng, o = _pair(orc, w, cands, True, True)
    f = w.forest
    sp = _species(o, f)
    n = f.num_of_nodes
    cfg = dict(coverage=40, read_size=150, insert_size_mean=350, insert_size_stddev=10, error_rate=1e-3,
               purity=0.8, with_normal_sample=False)
    c, _ = seq_cfg(chr_index=eng._chr_index, tile_size=4096, **cfg)
    g_ctx, m_ctx = np.zeros(96), np.zeros(96)
    g_edge, m_edge, g_vaf, m_vaf, g_dep, m_dep = [], [], [], [], [], []
    for s in range(48):
        pf = eng.place_mutations(f, 40, 4, seed=3000 + s)
        t = pf.table()
        op = o.place(f, sp, 40, 0, 4, 0, seed=3000 + s, flavour=1)
        ot = op.table()
        for tab, ctx, edges in ((t, g_ctx, g_edge), (ot, m_ctx, m_edge)):
            snv = (tab["kind"] == 0) & (tab["nature"] == 0)
            ctx += np.bincount(tab["cls"][snv], minlength=96)
            edges.append(np.bincount(tab["edge"][snv], minlength=n)[:n])
        if s < 16:
            alt, dep = sequence_counts(pf, 700 + s, tile_size=4096, **cfg).counts()
            oalt, odep, _ = op.sequence(c, 700 + s, flavour=1)
            for a, d, vafs, deps, tab in ((alt, dep, g_vaf, g_dep, t), (oalt, odep, m_vaf, m_dep, ot)):
                keep = d[0] >= 10
                vafs.append(a[0][keep] / d[0][keep])
                deps.append(d[0])
    keep = (g_ctx + m_ctx) > 0
    assert stats.chi2_contingency(np.vstack([g_ctx[keep], m_ctx[keep]]))[1] > 0.01
    assert stats.ks_2samp(np.concatenate(g_edge), np.concatenate(m_edge)).pvalue > 0.01
    assert stats.ks_2samp(np.concatenate(g_vaf), np.concatenate(m_vaf)).pvalue > 0.01
    assert stats.ks_2samp(np.concatenate(g_dep), np.concatenate(m_dep)).pvalue > 0.01


def test_cell_mutations_follow_allele_copies(gpu_lib, orc):
    """get_sampled_cell_mutations with copy-number events (built in C++ by
    pg_placed_cell_mutations): in every sampled cell, each mutation on its
    root path once per allele instance of the cell's genome at the locus that
    carries it, rows by chromosome, allele, position.  The expectation comes
    from the oracle alone: the root path by walking the forest's parents, its
    class pieces (instances present per position) and its carrier closure
    over the copies."""
    w, cands = _workload(seed=5, n_leaves=300)
    eng, o = _pair(orc, w, cands, True, True)
    f = w.forest
    pf = eng.place_mutations(f, 60, 6, seed=9)
    op = o.place(f, _species(o, f), 60, 0, 6, 0, seed=9)
    _tables_equal(pf.table(), op.table())
    ot = op.table()
    off, lst = op.carriers()
    ocls, n_cls, _ = op.node_classes(f.num_of_nodes)
    assert n_cls > 3
    n = f.num_of_nodes
    leaves = np.nonzero(f.is_leaf & (f.sample >= 0))[0]
    picked = {}
    for lf in leaves:                                  # one leaf per genotype class
        picked.setdefault(int(ocls[lf]), int(lf))
    pieces = {c: op.class_pieces(c) for c in picked}
    chr_off = np.concatenate([[0], np.cumsum(np.asarray(w.genome.chr_lengths, dtype=np.int64))])
    copies = lost = 0
    for c, lf in picked.items():
        cell, rows, alle = pf.cell_mutation_rows(int(f.cell_id[lf]))
        assert (cell == lf).all()
        got = list(zip(rows.tolist(), alle.tolist()))
        path = set()
        v = lf
        while v >= 0:
            path.add(v)
            v = int(f.parent[v])
        inst, b, e = pieces[c]
        want = []
        for m in range(len(ot["locus"])):
            if int(ot["edge"][m]) < n and int(ot["edge"][m]) not in path:
                continue
            L = int(ot["locus"][m])
            present = set(inst[(b <= L) & (L < e)].tolist())
            car = [int(y) for y in lst[off[m]:off[m + 1]] if int(y) in present]
            want.extend((m, y) for y in car)
            copies += len(car) > 1
            lost += len(car) == 0
        key = lambda my: (int(np.searchsorted(chr_off, ot["locus"][my[0]], side="right")), my[1],
                          int(ot["locus"][my[0]]), my[0])
        assert got == sorted(want, key=key), (c, len(set(got) ^ set(want)))
    assert copies > 0 and lost > 0                     # amplified and deleted mutations both occur
    # the data frame of one cell: its rows, with their alleles, in that order
    lf = next(iter(picked.values()))
    df = pf.get_sampled_cell_mutations(int(f.cell_id[lf]))
    _, rows, alle = pf.cell_mutation_rows(int(f.cell_id[lf]))
    np.testing.assert_array_equal(df["allele"], alle)
    np.testing.assert_array_equal(df["chr_pos"], ot["locus"][rows].astype(np.int64) + 1
                                  - chr_off[np.searchsorted(chr_off, ot["locus"][rows], side="right") - 1])
