"""PhylogeneticForest save / load (versioned native archive): a loaded forest
places the same mutations (digest-checked) and sequences identically."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_save_load_round_trip(gpu_lib, tmp_path):
    from process_gb300 import CNA, SNV, WGD, load_phylogenetic_forest, synth
    from process_gb300.engine import sequence_counts
    w = synth.config1(seed=4, n_leaves=150)
    w.genome.chr_lengths = [200_000, 100_000, 100_000]
    (na, ra, _), (nb, rb, _) = w.mutants
    w.mutants = [(na, dict(ra, CNA=1e-8), [SNV("1", 5000, "T"), CNA("A", "2", 10_001, 20_000)]),
                 (nb, rb, [WGD])]
    eng = synth.build_engine(w)
    eng.add_passenger_CNAs([CNA("D", "3", 1001, 5000)])
    eng.infinite_sites_model = False
    pf = eng.place_mutations(w.forest, 20, 3, seed=11)
    path = tmp_path / "phylo_forest.sff"
    pf.save(str(path))
    pf2 = load_phylogenetic_forest(str(path))
    for k, v in pf.table().items():
        np.testing.assert_array_equal(pf2.table()[k], v, err_msg=k)
    np.testing.assert_array_equal(pf2.forest.parent, pf.forest.parent)
    np.testing.assert_array_equal(pf2.forest.cell_id, pf.forest.cell_id)
    assert pf2.forest.sample_names == pf.forest.sample_names
    assert not pf2.engine.infinite_sites_model
    cfg = dict(coverage=10, read_size=150, insert_size_mean=350, insert_size_stddev=10, error_rate=1e-3)
    a1, d1 = sequence_counts(pf, 5, **cfg).counts()
    a2, d2 = sequence_counts(pf2, 5, **cfg).counts()
    np.testing.assert_array_equal(a1, a2)
    np.testing.assert_array_equal(d1, d2)
    c1, c2 = pf.cna_table(), pf2.cna_table()
    for k in c1:
        np.testing.assert_array_equal(c1[k], c2[k], err_msg=k)


def test_counts_into_page_locked_buffers(gpu_lib):
    """counts(out=...) fills caller-owned (here page-locked) arrays with the
    same tables as the allocating form, and rejects wrong shapes and types."""
    import torch
    from process_gb300 import synth
    from process_gb300.engine import sequence_counts
    w = synth.config1(seed=12, n_leaves=100)
    w.genome.chr_lengths = [100_000, 50_000, 50_000]
    eng = synth.build_engine(w)
    pf = eng.place_mutations(w.forest, 10, 2, seed=2)
    r = sequence_counts(pf, 3, coverage=12, read_size=100, insert_size_mean=250, insert_size_stddev=10)
    s, m, _ = r.dims()
    a1, d1 = r.counts()
    bufs = [torch.empty((s, m), dtype=torch.int32, pin_memory=True).numpy() for _ in range(2)]
    a2, d2 = r.counts(tuple(bufs))
    assert a2 is bufs[0] and d2 is bufs[1]
    np.testing.assert_array_equal(a1, a2)
    np.testing.assert_array_equal(d1, d2)
    with pytest.raises(ValueError, match="C-contiguous int32"):
        r.counts((np.empty((s, m), np.int64), bufs[1]))
    with pytest.raises(ValueError, match="C-contiguous int32"):
        r.counts((bufs[0][:, :-1], bufs[1]))


def test_observed_rows(gpu_lib):
    """observed() compacts, on the device, the rows with an alt read in some
    sample: the same indices and tables as filtering the full tables; the
    default result frame (those rows) and the include_non_sequenced frame
    carry the same occurrences."""
    import torch
    from process_gb300 import simulate_seq, synth
    from process_gb300.engine import sequence_counts
    w = synth.config1(seed=13, n_leaves=200)
    w.genome.chr_lengths = [120_000, 60_000, 60_000]
    eng = synth.build_engine(w)
    pf = eng.place_mutations(w.forest, 20, 4, seed=6)
    r = sequence_counts(pf, 5, coverage=25, read_size=120, insert_size_mean=300, insert_size_stddev=10,
                        error_rate=1e-3, purity=0.8)
    a, d = r.counts()
    keep = np.nonzero(a.sum(axis=0) > 0)[0]
    assert 0 < len(keep) < a.shape[1]
    idx, ao, do = r.observed()
    np.testing.assert_array_equal(idx, keep)
    np.testing.assert_array_equal(ao, a[:, keep])
    np.testing.assert_array_equal(do, d[:, keep])
    s = a.shape[0]
    bufs = (torch.empty(a.shape[1], dtype=torch.int32, pin_memory=True).numpy().view(np.uint32),
            torch.empty(s * a.shape[1], dtype=torch.int32, pin_memory=True).numpy(),
            torch.empty(s * a.shape[1], dtype=torch.int32, pin_memory=True).numpy())
    i2, a2, d2 = r.observed(bufs)
    np.testing.assert_array_equal(i2, keep)
    np.testing.assert_array_equal(a2, a[:, keep])
    np.testing.assert_array_equal(d2, d[:, keep])
    with pytest.raises(ValueError, match="at least"):
        r.observed((bufs[0][:1], bufs[1], bufs[2]))
    f0 = simulate_seq(pf, coverage=25, insert_size_mean=300, insert_size_stddev=10, seed=7)["mutations"]
    f1 = simulate_seq(pf, coverage=25, insert_size_mean=300, insert_size_stddev=10, seed=7,
                      include_non_sequenced_mutations=True)["mutations"]
    assert len(f1["chr"]) > len(f0["chr"])
    occ = [k for k in f0 if k.endswith(".occurrences")]
    assert occ and all(int(f0[k].sum()) == int(f1[k].sum()) for k in occ)
    rows0 = set(zip(f0["chr"], f0["chr_pos"], f0["ref"], f0["alt"]))
    rows1 = set(zip(f1["chr"], f1["chr_pos"], f1["ref"], f1["alt"]))
    assert rows0 <= rows1
