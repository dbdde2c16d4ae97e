"""The data frames built by the library (pg_placed_cell_fragmentation,
pg_placed_bulk_fragmentation, pg_placed_samples_info, pg_placed_cell_cnas,
pg_seq_result_frame) against the test-side numpy restatement of
tests/frames_ref.py, on a forest with driver and passenger CNAs and a WGD."""
import numpy as np
import pytest

import frames_ref as ref
from test_gpu_cna import _pair, _species, _tables_equal, _workload

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cna_forest(orc, gpu_lib):
    w, cands = _workload(seed=7, n_leaves=400)
    eng, o = _pair(orc, w, cands, True, True)
    pf = eng.place_mutations(w.forest, 80, 8, seed=3)
    op = o.place(w.forest, _species(o, w.forest), 80, 0, 8, 0, seed=3)
    _tables_equal(pf.table(), op.table())
    assert pf.node_classes()[1] > 3
    return w, eng, pf, op


def test_cell_fragmentation(cna_forest):
    _, _, pf, _ = cna_forest
    got = pf.get_cell_allelic_fragmentation()
    want = ref.get_cell_allelic_fragmentation(pf)
    # the restatement lists cells in node order, the reference (a std::map) by cell id
    o = np.argsort(np.asarray(want["cell_id"]), kind="stable")
    want = {k: np.asarray(v)[o] for k, v in want.items()}
    for k in ("cell_id", "chr", "begin", "end", "major", "minor"):
        np.testing.assert_array_equal(np.asarray(got[k]), np.asarray(want[k]), err_msg=k)
    assert (got["major"] != got["minor"]).any()           # some cell lost or gained an allele


@pytest.mark.parametrize("sample", [None, "S_1"])
def test_bulk_fragmentation(cna_forest, sample):
    """Same stretches and types as the restatement; per stretch the ratios
    add to 1, and cells without DNA come last as type (0, 0)."""
    _, _, pf, _ = cna_forest
    got = pf.get_bulk_allelic_fragmentation(sample)
    want = ref.get_bulk_allelic_fragmentation(pf, sample)
    key = lambda d, i: (str(d["chr"][i]), int(d["begin"][i]), int(d["end"][i]), int(d["major"][i]),
                        int(d["minor"][i]), round(float(d["ratio"][i]), 12))
    assert sorted(key(got, i) for i in range(len(got["chr"]))) == sorted(key(want, i) for i in range(len(want["chr"])))
    stretch = {}
    for i in range(len(got["chr"])):
        stretch.setdefault((got["chr"][i], got["begin"][i]), []).append(i)
    for rows in stretch.values():
        assert abs(sum(got["ratio"][i] for i in rows) - 1.0) < 1e-12
        zeros = [i for i in rows if got["major"][i] == 0]
        assert zeros in ([], [rows[-1]])


def test_samples_info(cna_forest):
    """DNA quantity = summed allelic size of the sample's cells' genomes."""
    w, eng, pf, _ = cna_forest
    f = w.forest
    d = ref.classes(pf)
    seg_cls = np.repeat(np.arange(d["n_classes"]), np.diff(d["seg_off"].astype(np.int64)))
    size = np.zeros(d["n_classes"])
    np.add.at(size, seg_cls, (d["end"].astype(np.float64) - d["start"]) * d["icnt"])
    cls, _, _ = pf.node_classes()
    info = pf.get_samples_info()
    for i, name in enumerate(info["name"]):
        j = f.sample_names.index(name)
        dna = size[cls[f.is_leaf & (f.sample == j)]].sum()
        assert info["DNA_quantity"][i] == dna
        assert info["equivalent_normal_cells"][i] == pytest.approx(dna / (2.0 * eng.genome.total), rel=1e-15)


def test_cell_cnas(cna_forest):
    """Each sampled cell's CNA rows are the events on its root path, in
    event order."""
    w, _, pf, op = cna_forest
    f = w.forest
    c = op.cna_table()
    got = pf.get_sampled_cell_CNAs()
    leaves = np.nonzero(f.is_leaf & (f.sample >= 0))[0]
    want_cell, want_begin = [], []
    for lf in leaves[np.argsort(f.cell_id[leaves])]:
        path = set()
        v = int(lf)
        while v >= 0:
            path.add(v)
            v = int(f.parent[v])
        for i in range(len(c["node"])):
            if int(c["node"][i]) in path:
                want_cell.append(int(f.cell_id[lf]))
                want_begin.append(-1 if c["type"][i] == 2 else int(c["begin"][i]))
    assert got["cell_id"].tolist() == want_cell
    assert got["begin"].tolist() == want_begin
    assert set(got["type"]) >= {"A", "D", "WGD"}


@pytest.mark.parametrize("include", [False, True])
def test_result_frame_matches_restatement(cna_forest, include):
    """simulate_seq's data frame from the library equals the restatement's,
    observed rows only and with every present mutation."""
    from process_gb300 import simulate_seq
    from process_gb300.engine import sequence_counts
    w, _, pf, _ = cna_forest
    names = list(w.forest.sample_names) + ["normal_sample"]
    df = simulate_seq(pf, coverage=30, insert_size_mean=350, insert_size_stddev=10, purity=0.8, seed=5,
                      include_non_sequenced_mutations=include)["mutations"]
    res = sequence_counts(pf, 5, coverage=30, read_size=150, insert_size_mean=350, insert_size_stddev=10,
                          error_rate=0.0, purity=0.8)
    present = ref.presence(pf, len(names), True, False) if include else None
    want = ref.result_frame(pf, *ref.result_rows(res, include, present), names)
    assert len(df["chr"]) == len(want["chr"]) > 0
    for k in want:
        a, b = np.asarray(df[k]), np.asarray(want[k])
        if a.dtype.kind == "f":
            np.testing.assert_allclose(a, b, rtol=0, atol=0, err_msg=k)
        else:
            assert a.tolist() == b.tolist(), k
