"""Copy-number events in the oracle (CPU): genotype classes, the order of a
driver SNV and a whole-genome doubling, deletions, and
avoid_homozygous_losses (src/mutations.cpp:837-840)."""
import numpy as np
import pytest


def _engine(orc, w):
    return orc.OracleEngine.like(w)


def _species(o, forest):
    return np.array([o.species[(m, ep)] for m, ep in zip(forest.mutant, forest.epistate)], dtype=np.uint32)


def _cfg(**kw):
    from process_gb300.engine import seq_cfg
    c, _ = seq_cfg(chr_index=lambda n: int(n) - 1, tile_size=4096, **kw)
    return c


def test_wgd_classes_and_copy_number(orc):
    from process_gb300 import synth
    w = synth.plain_3mbp(seed=5, n_leaves=200)
    o = _engine(orc, w)
    o.add_driver_wgd(0)                      # mutant A: every tumour cell
    f = w.forest
    p = o.place(f, _species(o, f), 10, 0, 0, 0, seed=3)
    cls, n_cls, cn_max = p.node_classes(f.num_of_nodes)
    assert n_cls >= 2 and cn_max == 4
    assert (cls > 0).all()
    c = p.cna_table()
    assert (c["type"] == 2).all() and (c["driver"] == 1).all()
    roots = np.nonzero(f.parent < 0)[0]
    assert sorted(c["node"].tolist()) == sorted(roots.tolist())
    # WGD doubles the allelic size: about twice the passengers of the same forest without it
    o2 = _engine(orc, w)
    p2 = o2.place(f, _species(o2, f), 10, 0, 0, 0, seed=3)
    n1, n2 = len(p.table()["locus"]), len(p2.table()["locus"])
    assert 1.7 < n1 / n2 < 2.3
    # every allele is a present instance id (0..5 with one WGD per root: 2 + 2 per root)
    assert p.table()["allele"].max() < 2 + 2 * len(roots)


@pytest.mark.parametrize("snv_first", [True, False])
def test_driver_then_wgd_vaf(orc, snv_first):
    """SNV then WGD: both copies of the mutated allele carry it (VAF 1/2 in a
    pure tumour); WGD then SNV: one allele of four (VAF 1/4)."""
    from process_gb300 import synth
    w = synth.plain_3mbp(seed=6, n_leaves=100)
    w.genome.chr_lengths = [200_000] * 3
    o = _engine(orc, w)
    g = o.read_genome()
    ref = "ACGT"[g[50_000 - 1]]
    alt = "C" if ref != "C" else "G"
    if snv_first:
        o.add_drivers(0, [_sid("1", 50_000, ref, alt, 0)], lambda n: int(n) - 1)
        o.add_driver_wgd(0)
    else:
        o.add_driver_wgd(0)
        o.add_drivers(0, [_sid("1", 50_000, ref, alt, 0)], lambda n: int(n) - 1)
    f = w.forest
    p = o.place(f, _species(o, f), 0, 0, 0, 0, seed=9)
    t = p.table()
    d = np.nonzero(t["nature"] == 1)[0]
    assert len(d) == 1
    alt_c, dep, _ = p.sequence(_cfg(coverage=400, read_size=150, insert_size_mean=350, insert_size_stddev=10,
                                    error_rate=0.0, purity=1.0, with_normal_sample=False), 4)
    vaf = alt_c[0, d[0]] / dep[0, d[0]]
    assert dep[0, d[0]] > 200
    want = 0.5 if snv_first else 0.25
    assert abs(vaf - want) < 0.09, (vaf, want)


def _sid(chr_, pos, ref, alt, allele):
    from process_gb300 import Mutation
    return Mutation(chr_, pos, ref, alt, allele)


@pytest.mark.parametrize("flavour", [0, 1])
def test_deletion_halves_depth_and_hides_mutations(orc, flavour):
    from process_gb300 import synth
    w = synth.plain_3mbp(seed=7, n_leaves=100)
    w.genome.chr_lengths = [300_000] * 3
    o = _engine(orc, w)
    # delete allele 0 of [100001, 200000] of chromosome 2 in every tumour cell
    o.add_driver_cna(0, False, 1, 100_001, 100_000, allele=0)
    f = w.forest
    p = o.place(f, _species(o, f), 200, 0, 0, 0, seed=2, flavour=flavour)
    t = p.table()
    lo, hi = 300_000 + 100_000, 300_000 + 200_000
    inside = (t["locus"] >= lo) & (t["locus"] < hi)
    # passengers inside the region sit on allele 1 (allele 0 is gone there), preneoplastic ones on either
    passenger = t["nature"] == 0
    assert inside.any() and (t["allele"][inside & passenger] == 1).all()
    _, dep, _ = p.sequence(_cfg(coverage=60, read_size=150, insert_size_mean=0, error_rate=0.0, purity=1.0,
                                with_normal_sample=False), 5, flavour=flavour)
    d_in = dep[0][inside & passenger].mean()
    d_out = dep[0][~inside & passenger & (t["locus"] >= 300_000) & (t["locus"] < 600_000)].mean()
    assert 0.35 < d_in / d_out < 0.65


@pytest.mark.parametrize("avoid", [True, False])
def test_avoid_homozygous_losses(orc, avoid):
    from process_gb300 import synth
    w = synth.plain_3mbp(seed=8, n_leaves=300)
    w.genome.chr_lengths = [100_000] * 3
    w.mutants = [(n, dict(r, CNA=2e-6), d) for n, r, d in w.mutants]
    o = _engine(orc, w)
    o.add_passenger_cna(0, 1001, 5000, False)       # one deletion candidate
    o.set_avoid_homozygous_losses(avoid)
    f = w.forest
    p = o.place(f, _species(o, f), 0, 0, 0, 0, seed=4)
    c = p.cna_table()
    assert len(c["node"]) > 0
    node_of = set(c["node"].tolist())
    worst = 0
    for lf in np.nonzero(f.is_leaf)[0]:
        k, v = 0, int(lf)
        while v >= 0:
            k += v in node_of
            v = int(f.parent[v])
        worst = max(worst, k)
    if avoid:
        assert worst == 1
    else:
        assert worst == 2
