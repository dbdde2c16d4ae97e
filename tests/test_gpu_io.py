"""PhylogeneticForest save / load (versioned native archive of the placed
forest, pg_placed_serialize / pg_placed_deserialize): a loaded forest holds
the same tables and getters without placing again, and sequences
identically; SAM-free I/O helpers."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _frames_equal(a, b):
    assert set(a) == set(b)
    for k in a:
        assert np.asarray(a[k]).tolist() == np.asarray(b[k]).tolist(), k


def test_save_load_round_trip(gpu_lib, tmp_path):
    from process_gb300 import CNA, SNV, WGD, DomainError, GenomeSpec, MutationEngine, load_phylogenetic_forest, synth
    from process_gb300 import _lib
    from process_gb300.engine import sequence_counts
    w = synth.plain_3mbp(seed=4, n_leaves=150)
    w.genome.chr_lengths = [200_000, 100_000, 100_000]
    (na, ra, _), (nb, rb, _) = w.mutants
    w.mutants = [(na, dict(ra, CNA=1e-8), [SNV("1", 5000, "T"), CNA("A", "2", 10_001, 20_000)]),
                 (nb, rb, [WGD])]
    eng = synth.build_engine(w)
    eng.add_passenger_CNAs([CNA("D", "3", 1001, 5000)])
    eng.infinite_sites_model = False
    pf = eng.place_mutations(w.forest, 20, 3, seed=11)
    pf.set_reference_path("/data/genome.fa")
    expo = pf.get_exposures()
    # the engine changes after placement: the forest keeps what it was placed with
    eng.add_exposure(5.0, {"SBS1": 1.0})
    path = tmp_path / "phylo_forest.sff"
    pf.save(str(path))
    pf2 = load_phylogenetic_forest(str(path))
    for k, v in pf.table().items():
        np.testing.assert_array_equal(pf2.table()[k], v, err_msg=k)
    np.testing.assert_array_equal(pf2.forest.parent, pf.forest.parent)
    np.testing.assert_array_equal(pf2.forest.cell_id, pf.forest.cell_id)
    assert pf2.forest.sample_names == pf.forest.sample_names
    assert not pf2.engine.infinite_sites_model
    assert pf2.get_reference_path() == "/data/genome.fa"
    _frames_equal(pf2.get_exposures(), expo)
    _frames_equal(pf.get_exposures(), expo)
    for getter in ("get_sampled_cell_mutations", "get_sampled_cell_CNAs", "get_cell_allelic_fragmentation",
                   "get_bulk_allelic_fragmentation", "get_samples_info", "get_driver_mutations", "get_species_info"):
        _frames_equal(getattr(pf2, getter)(), getattr(pf, getter)())
    np.testing.assert_array_equal(pf2.node_classes()[0], pf.node_classes()[0])
    cfg = dict(coverage=10, read_size=150, insert_size_mean=350, insert_size_stddev=10, error_rate=1e-3)
    a1, d1 = sequence_counts(pf, 5, **cfg).counts()
    a2, d2 = sequence_counts(pf2, 5, **cfg).counts()
    np.testing.assert_array_equal(a1, a2)
    np.testing.assert_array_equal(d1, d2)
    c1, c2 = pf.cna_table(), pf2.cna_table()
    for k in c1:
        np.testing.assert_array_equal(c1[k], c2[k], err_msg=k)
    # the archive refuses an engine with another genome, and a truncated buffer
    n = C.c_uint64()
    _lib.check(_lib.lib().pg_placed_serialize(pf._h, None, 0, C.byref(n)))
    blob = np.empty(n.value, dtype=np.uint8)
    _lib.check(_lib.lib().pg_placed_serialize(pf._h, _lib.ptr(blob, C.c_uint8), n.value, C.byref(n)))
    other = MutationEngine(GenomeSpec(["1", "2", "3"], [200_000, 100_000, 100_000], seed=99), w.sbs, w.ids)
    h = C.c_void_p()
    assert _lib.lib().pg_placed_deserialize(other._h, _lib.ptr(blob, C.c_uint8), n.value, C.byref(h)) == \
        _lib.PG_ERR_DOMAIN
    assert b"another reference genome" in _lib.lib().pg_last_error()
    assert _lib.lib().pg_placed_deserialize(eng._h, _lib.ptr(blob, C.c_uint8), n.value // 2, C.byref(h)) == \
        _lib.PG_ERR_DOMAIN
    assert b"truncated" in _lib.lib().pg_last_error()
    with pytest.raises(DomainError):
        _lib.check(_lib.lib().pg_placed_load(eng._h, str(tmp_path / "none.pgpf").encode(), C.byref(h)))


def test_counts_into_page_locked_buffers(gpu_lib):
    """counts(out=...) fills caller-owned (here page-locked) arrays with the
    same tables as the allocating form, and rejects wrong shapes and types."""
    import torch
    from process_gb300 import synth
    from process_gb300.engine import sequence_counts
    w = synth.plain_3mbp(seed=12, n_leaves=100)
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
    w = synth.plain_3mbp(seed=13, n_leaves=200)
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


def _naive_frame(pf, alt, dep, names):
    """The result frame built row by row (the definition the library's
    builder must match): SIDs (locus, ref, alt) in the reference's map order
    (src/seq_simulation.cpp:52-181)."""
    from process_gb300.engine import BASES, NATURES
    t = pf.table()
    eng = pf.engine
    g = eng.read_genome()
    keep = np.nonzero(alt.sum(axis=0) > 0)[0]
    groups, order = {}, []
    for i in keep:
        a, k, loc = int(t["aux"][i]), int(t["kind"][i]), int(t["locus"][i])
        if k == 0:
            r, x = BASES[g[loc]], BASES[a & 3]
        else:
            ins, ln, b = a & 1, (a >> 1) & 7, a >> 8
            if ins:
                r = BASES[g[loc]]
                x = r + "".join(BASES[(b >> (2 * q)) & 3] for q in range(ln))
            else:
                r = "".join(BASES[g[loc:loc + ln + 1]])
                x = r[0]
        key = (loc, r, x)
        if key not in groups:
            groups[key] = []
            order.append(key)
        groups[key].append(i)
    order = sorted(order)
    out = {"ref": [k[1] for k in order], "alt": [k[2] for k in order], "locus": [k[0] for k in order]}
    for s, name in enumerate(names):
        out[f"{name}.occurrences"] = [int(alt[s, groups[k]].sum()) for k in order]
        out[f"{name}.coverage"] = [int(dep[s, groups[k][0]]) for k in order]
    out["classes"] = [";".join(sorted(set(NATURES[t["nature"][groups[k]]]))) for k in order]
    sig = [list(eng.sig_names[0]), list(eng.sig_names[1])]
    out["causes"] = [";".join(sorted({sig[int(t["kind"][i])][int(t["sig"][i])] for i in groups[k]
                                      if int(t["sig"][i]) < len(sig[int(t["kind"][i])])})) or None for k in order]
    return out


def test_result_frame_matches_row_by_row(gpu_lib):
    """The library's result frame (pg_seq_result_frame) equals the
    row-by-row definition, with indels and (infinite sites off) several SIDs
    on one locus."""
    from process_gb300 import synth
    from process_gb300.engine import _result_frame, sequence_counts
    w = synth.plain_3mbp(seed=14, n_leaves=150)
    w.genome.chr_lengths = [40_000, 20_000, 20_000]
    w.mutants = [(n, dict(r, SNV=r["SNV"] * 20, indel=2e-6), d) for n, r, d in w.mutants]
    eng = synth.build_engine(w)
    eng.infinite_sites_model = False
    pf = eng.place_mutations(w.forest, 50, 10, seed=8)
    t = pf.table()
    assert len(np.unique(t["locus"])) < len(t["locus"])        # repeated loci
    r = sequence_counts(pf, 9, coverage=60, read_size=100, insert_size_mean=250, insert_size_stddev=10,
                        error_rate=1e-3, purity=0.9)
    a, d = r.counts()
    names = [f"s{q}" for q in range(a.shape[0])]
    df = _result_frame(r, pf, False, names)
    ref = _naive_frame(pf, a, d, names)
    assert list(df["ref"]) == ref["ref"] and list(df["alt"]) == ref["alt"]
    assert (t["kind"][np.nonzero(a.sum(axis=0) > 0)[0]] == 1).any()   # some indels observed
    off = eng.chr_off.astype(np.int64)
    loc = np.array([off[eng.chr_names.index(c)] for c in df["chr"]]) + df["chr_pos"] - 1
    assert loc.tolist() == ref["locus"]
    assert list(df["classes"]) == ref["classes"]
    assert list(df["causes"]) == ref["causes"]
    for name in names:
        assert df[f"{name}.occurrences"].tolist() == ref[f"{name}.occurrences"]
        assert df[f"{name}.coverage"].tolist() == ref[f"{name}.coverage"]
