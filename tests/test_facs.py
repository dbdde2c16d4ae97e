"""FACS labelling of simulate_seq(cell_labelling = f) (src/seq_simulation.cpp:183-243):
the cells of each sample split by their label into "<sample>_<label>"
samples (the empty label keeps the sample's name), in the order the labels
first appear; sequencing those samples is bit-exact against the oracle run
on a forest whose samples are the labelled groups."""
import types

import numpy as np
import pytest


def _forest_with_samples(f, part, names):
    from process_gb300 import SamplesForest
    anc = np.where(f.parent >= 0, f.cell_id[np.maximum(f.parent, 0)], -1)
    smp = np.array([names[p] if p >= 0 else None for p in part], dtype=object)
    return SamplesForest(f.cell_id, anc, f.mutant, f.epistate, smp, f.birth_time, f.divisions)


def test_partition_by_label():
    from process_gb300 import DomainError, synth
    from process_gb300.engine import _facs_partition, _forest_partition
    w = synth.plain_3mbp(seed=15, n_leaves=300)
    f = w.forest
    pf = types.SimpleNamespace(forest=f)
    base = _forest_partition(pf)
    part, names = _facs_partition(pf, lambda c: c.mutant)
    mutants = sorted({str(m) for m in f.mutant[base >= 0]})
    assert sorted(names) == sorted(f"{s}_{m}" for s in f.sample_names for m in mutants
                                   if ((base == f.sample_names.index(s)) & (f.mutant == m)).any())
    for v in np.nonzero(base >= 0)[0]:
        assert names[part[v]] == f"{f.sample_names[base[v]]}_{f.mutant[v]}"
    assert (part[base < 0] == -1).all()
    part0, names0 = _facs_partition(pf, lambda c: "")
    np.testing.assert_array_equal(part0, base)
    assert names0 == list(f.sample_names)
    with pytest.raises(DomainError, match="must be a function"):
        _facs_partition(pf, "not a function")
    with pytest.raises(DomainError, match="must return a string"):
        _facs_partition(pf, lambda c: 3)


@pytest.mark.gpu
def test_facs_sequencing_bit_exact(gpu_lib, orc):
    from process_gb300 import _lib, simulate_seq, synth
    from process_gb300.engine import _facs_partition, _forest_partition, seq_cfg, sequence_counts
    w = synth.plain_3mbp(seed=15, n_leaves=300)
    eng = synth.build_engine(w)
    pf = eng.place_mutations(w.forest, 30, 3, seed=4)
    label = lambda c: ("", "x", "y")[c.cell_id % 3]
    part, names = _facs_partition(pf, label)
    assert len(names) == 3 * len(w.forest.sample_names)
    cfg = dict(coverage=30, read_size=150, insert_size_mean=350, insert_size_stddev=10, error_rate=1e-3, purity=0.8)
    # a sample's index keys its reads' random streams: sequence the groups in
    # name order, the order of the oracle's forest built from them
    srt = sorted(names)
    part = np.where(part >= 0, np.array([srt.index(n) for n in names])[np.maximum(part, 0)], -1).astype(np.int32)
    names = srt
    _lib.check(_lib.lib().pg_placed_set_samples(pf._h, len(names), _lib.ptr(part, __import__("ctypes").c_int32)))
    try:
        alt, dep = sequence_counts(pf, 77, tile_size=4096, **cfg).counts()
    finally:
        base = _forest_partition(pf)
        _lib.check(_lib.lib().pg_placed_set_samples(pf._h, len(w.forest.sample_names),
                                                    _lib.ptr(base, __import__("ctypes").c_int32)))
    assert alt.shape[0] == len(names) + 1
    f2 = _forest_with_samples(w.forest, part, names)
    o = orc.OracleEngine.like(w)
    sp = np.array([o.species[(m, e)] for m, e in zip(f2.mutant, f2.epistate)], dtype=np.uint32)
    op = o.place(f2, sp, 30, 0, 3, 0, seed=4)
    c, _ = seq_cfg(chr_index=eng._chr_index, tile_size=4096, **cfg)
    oalt, odep, _ = op.sequence(c, 77, flavour=0)
    assert f2.sample_names == names
    np.testing.assert_array_equal(dep, odep)
    np.testing.assert_array_equal(alt, oalt)
    # through simulate_seq: the labelled samples' columns, and the plain
    # samples again afterwards
    out = simulate_seq(pf, coverage=20, seed=5, cell_labelling=label)["mutations"]
    assert all(f"{n}.occurrences" in out for n in names)
    assert sum(k.endswith(".occurrences") for k in out) == len(names) + 1
    plain = simulate_seq(pf, coverage=20, seed=5)["mutations"]
    again = simulate_seq(pf, coverage=20, seed=5, cell_labelling=lambda c: "")["mutations"]
    for k in plain:
        np.testing.assert_array_equal(plain[k], again[k], err_msg=k)
