"""CPU checks of the oracle: known-answer vectors, sampler distributions and the
model properties the reference documents.  No GPU."""
import ctypes as C
import math

import numpy as np
import pytest
from scipy import stats


def philox(orc, k0, k1, c0, c1, c2, c3):
    out = (C.c_uint32 * 4)()
    orc.lib().orc_philox(k0, k1, c0, c1, c2, c3, out)
    return list(out)


def test_philox_known_answers(orc):
    # Random123 known-answer vectors for philox4x32-10 (Salmon et al., SC'11)
    assert philox(orc, 0, 0, 0, 0, 0, 0) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    f = 0xFFFFFFFF
    assert philox(orc, f, f, f, f, f, f) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert philox(orc, 0xA4093822, 0x299F31D0, 0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_log_exp_accuracy(orc):
    L = orc.lib()
    rng = np.random.default_rng(0)
    for x in np.exp(rng.uniform(-700, 700, 5000)):
        assert abs(L.orc_log(x) - math.log(x)) <= 4e-16 * max(1.0, abs(math.log(x)))
    for y in rng.uniform(-700, 700, 5000):
        assert abs(L.orc_exp(y) - math.exp(y)) <= 4e-16 * math.exp(y)
    for k in [0, 1, 5, 9, 10, 11, 50, 1000, 1e6]:
        assert abs(L.orc_log_factorial(k) - math.lgamma(k + 1)) <= 1e-12 * max(1.0, math.lgamma(k + 1))


@pytest.mark.parametrize("lam", [0.3, 4.0, 9.9, 10.0, 37.5, 310.0, 5e4])
def test_poisson_sampler(orc, lam):
    L = orc.lib()
    x = np.array([L.orc_poisson(11, i, 3, 0, 1, lam) for i in range(20000)])
    assert abs(x.mean() - lam) < 5 * math.sqrt(lam / len(x))
    assert abs(x.var() / lam - 1) < 0.06
    if lam < 100:
        k = np.arange(0, int(lam + 8 * math.sqrt(lam) + 10))
        obs = np.bincount(x, minlength=len(k))[: len(k)]
        exp = stats.poisson.pmf(k, lam) * len(x)
        keep = exp > 5
        chi = ((obs[keep] - exp[keep]) ** 2 / exp[keep]).sum()
        assert stats.chi2.sf(chi, keep.sum() - 1) > 1e-3


@pytest.mark.parametrize("n,p", [(10, 0.3), (1000, 0.004), (490, 0.714), (100000, 0.37), (10**8, 0.5)])
def test_binomial_sampler(orc, n, p):
    L = orc.lib()
    x = np.array([L.orc_binomial(5, i, 0, 0, 7, n, p) for i in range(20000)], dtype=np.float64)
    mu, var = n * p, n * p * (1 - p)
    assert abs(x.mean() - mu) < 5 * math.sqrt(var / len(x)) + 1e-9
    assert abs(x.var() / var - 1) < 0.06
    assert x.min() >= 0 and x.max() <= n


def small_workload(seed=1, leaves=300):
    from process_gb300 import synth
    return synth.plain_3mbp(seed=seed, n_leaves=leaves)


def species_of(e, forest):
    return np.array([e.species[(m, ep)] for m, ep in zip(forest.mutant, forest.epistate)], dtype=np.uint32)


def test_index_lists_are_the_contexts(orc):
    w = small_workload()
    e = orc.OracleEngine.like(w)
    g = e.read_genome()
    info = e.index_info()
    assert info["ctx_total"].sum() == len(g) - 2 * len(w.genome.chr_lengths)
    comp = 3 - g
    for c in (0, 7, 19, 31):
        pos = e.read_index(0, c).astype(np.int64)
        assert np.all(np.diff(pos) > 0)
        x, y, z = g[pos - 1], g[pos], g[pos + 1]
        fwd = (y == 1) | (y == 3)
        ctx = np.where(fwd, np.where(y == 3, 16, 0) + x * 4 + z,
                       np.where(comp[pos] == 3, 16, 0) + comp[pos + 1] * 4 + comp[pos - 1])
        assert np.all(ctx == c)


def test_infinite_sites_property(orc):
    """vignettes/infinite_site_model.Rmd:150-220: with the model on, every
    mutation arises in exactly one cell; with it off, loci may repeat."""
    w = small_workload(leaves=600)
    for flavour in (0, 1):
        e = orc.OracleEngine.like(w)
        sp = species_of(e, w.forest)
        t = e.place(w.forest, sp, 50, 0, 5, 0, seed=3, flavour=flavour).table()
        assert len(np.unique(t["locus"])) == len(t["locus"])
        e.set_infinite_sites(False)
        t2 = e.place(w.forest, sp, 50, 0, 5, 0, seed=3, flavour=flavour).table()
        assert len(t2["locus"]) > 1000


def test_replay_is_deterministic_and_seeded(orc):
    w = small_workload()
    e = orc.OracleEngine.like(w)
    sp = species_of(e, w.forest)
    a = e.place(w.forest, sp, 10, 0, 2, 0, seed=9).table()
    b = e.place(w.forest, sp, 10, 0, 2, 0, seed=9).table()
    c = e.place(w.forest, sp, 10, 0, 2, 0, seed=10).table()
    for k in a:
        assert np.array_equal(a[k], b[k])
    assert not np.array_equal(a["locus"], c["locus"])


def test_preneoplastic_counts_and_signature(orc):
    w = small_workload()
    e = orc.OracleEngine.like(w)
    sp = species_of(e, w.forest)
    t = e.place(w.forest, sp, 123, 0, 17, 0, seed=4).table()
    pre = t["nature"] == 2
    assert (pre & (t["kind"] == 0)).sum() == 123 and (pre & (t["kind"] == 1)).sum() == 17
    assert np.all(t["edge"][pre] == w.forest.num_of_nodes)


def test_replay_and_reference_engine_agree_in_distribution(orc):
    """Per-edge count KS and context chi-square between the Philox replay and
    the std::mt19937_64 flavour (the GPU is compared with the latter in the
    GPU tests; this pins the replay's samplers on the CPU)."""
    w = small_workload(leaves=400)
    e = orc.OracleEngine.like(w)
    sp = species_of(e, w.forest)
    n = w.forest.num_of_nodes
    ca, cb = [], []
    ea, eb = np.zeros(96), np.zeros(96)
    for s in range(16):
        ta = e.place(w.forest, sp, 0, 0, 0, 0, seed=100 + s, flavour=0).table()
        tb = e.place(w.forest, sp, 0, 0, 0, 0, seed=100 + s, flavour=1).table()
        ca.append(np.bincount(ta["edge"][ta["kind"] == 0], minlength=n))
        cb.append(np.bincount(tb["edge"][tb["kind"] == 0], minlength=n))
        ea += np.bincount(ta["cls"][ta["kind"] == 0], minlength=96)
        eb += np.bincount(tb["cls"][tb["kind"] == 0], minlength=96)
    assert stats.ks_2samp(np.concatenate(ca), np.concatenate(cb)).pvalue > 0.01
    keep = (ea + eb) > 0
    assert stats.chi2_contingency(np.vstack([ea[keep], eb[keep]]))[1] > 0.01


def test_sequencing_replay_depth_and_vaf(orc):
    from process_gb300.engine import seq_cfg
    w = small_workload(leaves=300)
    e = orc.OracleEngine.like(w)
    sp = species_of(e, w.forest)
    p = e.place(w.forest, sp, 50, 0, 5, 0, seed=2)
    cfg, _ = seq_cfg(coverage=40, read_size=150, insert_size_mean=350, insert_size_stddev=10, error_rate=0.0,
                     tile_size=8192, chr_index=lambda x: int(x) - 1)
    alt, dep, reads = p.sequence(cfg, 5, flavour=0)
    assert reads == 2 * 3 * int(40 * 1e6 / 300) * 2  # 2 samples (tumour + normal), 3 chromosomes, 2 mates
    assert abs(dep.mean() - 40) < 1.5
    t = p.table()
    pre = t["nature"] == 2
    # clonal preneoplastic SNVs in a diploid genome: VAF about 1/2 in the tumour, 0 in the normal
    vaf = alt[0, pre].sum() / dep[0, pre].sum()
    assert abs(vaf - 0.5) < 0.05
    assert alt[1, pre].sum() == 0
    # errorless: never an alt read for a mutation not carried (normal sample, passengers)
    assert alt[1].sum() == 0


def test_sequencing_replay_error_thirds(orc):
    """Substitution errors: the normal sample carries no passenger, so each
    of its SNV depth units shows the alt base exactly when the visit's error
    word falls in the first third of [0, err_thr): a rate of e/3.  Indels
    see no substitution errors."""
    from process_gb300.engine import seq_cfg
    w = small_workload(leaves=200)
    e = orc.OracleEngine.like(w)
    sp = species_of(e, w.forest)
    p = e.place(w.forest, sp, 0, 0, 0, 0, seed=3)
    err = 0.09
    cfg, _ = seq_cfg(coverage=30, read_size=150, insert_size_mean=350, insert_size_stddev=10, error_rate=err,
                     tile_size=8192, chr_index=lambda x: int(x) - 1)
    alt, dep, _ = p.sequence(cfg, 7, flavour=0)
    t = p.table()
    snv, ind = t["kind"] == 0, t["kind"] == 1
    n = dep[1, snv].sum()
    rate = alt[1, snv].sum() / n
    assert abs(rate - err / 3) < 4 * np.sqrt(err / 3 / n)
    assert alt[1, ind].sum() == 0 and dep[1, ind].sum() > 0


def test_insert_size_model_rejects_large_variance(orc):
    from process_gb300.engine import seq_cfg
    w = small_workload(leaves=50)
    e = orc.OracleEngine.like(w)
    p = e.place(w.forest, species_of(e, w.forest), 5, 0, 0, 0, seed=1)
    cfg, _ = seq_cfg(coverage=1, insert_size_mean=350, insert_size_stddev=30, tile_size=4096,
                     chr_index=lambda x: int(x) - 1)
    with pytest.raises(RuntimeError):
        p.sequence(cfg, 1)
