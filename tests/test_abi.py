"""The C-ABI library loads and exports every entry point include/process_gb300.h
declares; host-side validation that needs no GPU."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    text = "\n".join(p.read_text() for p in sorted((ROOT / "include").glob("*.h")))
    return sorted(set(re.findall(r"^\s*(?:pg_status|const char\*|void|int)\s+(pg_\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def lib():
    from process_gb300 import build, _lib
    build.build()
    return _lib.lib()


def test_header_declares_the_boundary():
    syms = declared_symbols()
    for must in ("pg_engine_create", "pg_place_mutations", "pg_simulate_seq", "pg_seq_result_copy",
                 "pg_last_error"):
        assert must in syms


def test_library_exports_every_declared_symbol(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_version_and_errors_without_device(lib):
    from process_gb300 import _lib
    assert b"sm_103a" in lib.pg_version()
    n = C.c_int(-1)
    assert lib.pg_device_count(C.byref(n)) == 0 and n.value >= 0
    if n.value == 0:
        d = _lib.GenomeDesc()
        lens = np.array([1000], dtype=np.uint32)
        d.n_chr = 1
        d.chr_lengths = lens.ctypes.data_as(C.POINTER(C.c_uint32))
        d.context_sampling = 1
        d.max_repetition_storage = 10
        h = C.c_void_p()
        assert lib.pg_engine_create(C.byref(d), C.byref(h)) == _lib.PG_ERR_CUDA
        assert b"no CUDA device" in lib.pg_last_error()


def test_null_and_domain_checks(lib):
    from process_gb300 import _lib
    assert lib.pg_engine_create(None, None) == _lib.PG_ERR_DOMAIN
    h = C.c_void_p()
    parent = np.array([-1, 0, 2], dtype=np.int32)   # node 2 is its own parent: not topological
    birth = np.zeros(3)
    sp = np.zeros(3, dtype=np.uint32)
    smp = np.array([-1, 0, 0], dtype=np.int32)
    st = lib.pg_forest_create(3, _lib.ptr(parent, C.c_int32), _lib.ptr(birth, C.c_double),
                              _lib.ptr(sp, C.c_uint32), _lib.ptr(smp, C.c_int32), None, 1, C.byref(h))
    assert st == _lib.PG_ERR_DOMAIN and b"topological" in lib.pg_last_error()
    parent = np.array([-1, 0, 0], dtype=np.int32)
    st = lib.pg_forest_create(3, _lib.ptr(parent, C.c_int32), _lib.ptr(birth, C.c_double),
                              _lib.ptr(sp, C.c_uint32), _lib.ptr(smp, C.c_int32), None, 1, C.byref(h))
    assert st == _lib.PG_OK
    assert lib.pg_forest_destroy(h) == _lib.PG_OK


def test_sequencer_validation():
    from process_gb300 import BasicIlluminaSequencer, DomainError
    with pytest.raises(DomainError):
        BasicIlluminaSequencer(-1e-3)
    with pytest.raises(DomainError):
        BasicIlluminaSequencer(1e-3, random_quality_scores="yes")
    assert BasicIlluminaSequencer(4e-3).error_rate == 4e-3


def test_samples_forest_topological_order():
    from process_gb300 import SamplesForest
    # children listed before parents, arbitrary cell ids
    f = SamplesForest([30, 10, 20], [10, -1, 10], ["A"] * 3, [""] * 3, ["S1", None, "S1"], [2.0, 0.0, 1.0])
    # depth-first order from the roots, children in input order
    assert list(f.cell_id) == [10, 30, 20]
    assert list(f.parent) == [-1, 0, 0]
    assert list(f.birth_time) == [0.0, 2.0, 1.0]
    assert f.sample_names == ["S1"]
    assert list(f.is_leaf) == [False, True, True]
    nodes = f.get_nodes()
    assert list(nodes["ancestor"]) == [-1, 10, 10]


def test_synthetic_workloads_shapes():
    from process_gb300 import synth
    w = synth.plain_3mbp(seed=3, n_leaves=200)
    assert w.forest.num_of_nodes == 399
    assert w.forest.is_leaf.sum() == 200
    assert w.genome.total == 3_000_000
    w2 = synth.full_scale(seed=3, n_leaves_per_sample=50, genome_scale=1e-3)
    assert len(w2.genome.chr_lengths) == 24 and len(w2.exposures) == 3
    assert sorted(set(w2.forest.sample_names)) == ["S_1", "S_2", "S_3"]


def test_load_phylogenetic_forest_errors(tmp_path):
    """File checks of load_phylogenetic_forest happen before any device work."""
    import numpy as np
    from process_gb300 import DomainError, load_phylogenetic_forest
    with pytest.raises(DomainError, match="does not exist"):
        load_phylogenetic_forest(str(tmp_path / "missing.sff"))
    with pytest.raises(DomainError, match="not a regular file"):
        load_phylogenetic_forest(str(tmp_path))
    bad = tmp_path / "bad.sff"
    with open(bad, "wb") as fh:
        np.savez(fh, meta=np.frombuffer(b'{"format": "other", "version": 1}', dtype=np.uint8))
    with pytest.raises(DomainError, match="not a phylogenetic forest"):
        load_phylogenetic_forest(str(bad))
    newer = tmp_path / "newer.sff"
    with open(newer, "wb") as fh:
        np.savez(fh, meta=np.frombuffer(b'{"format": "process_gb300.phylogenetic_forest", "version": 99}',
                                        dtype=np.uint8))
    with pytest.raises(DomainError, match="format version 99"):
        load_phylogenetic_forest(str(newer))


def test_forest_euler_and_path_carriers():
    """Euler intervals of a samples forest give the ancestor relation, and a
    cell's path mutations (edge an ancestor-or-self of the cell, or
    preneoplastic) match a walk up its parents."""
    import numpy as np
    from process_gb300 import PhylogeneticForest, synth
    w = synth.plain_3mbp(seed=4, n_leaves=300)
    f = w.forest
    tin, tout = f.euler()
    rng = np.random.default_rng(1)
    n = f.num_of_nodes
    edges = rng.integers(0, n + 1, 5000).astype(np.uint32)   # n: the preneoplastic edge
    pf = PhylogeneticForest.__new__(PhylogeneticForest)
    pf.forest = f
    pf._table = {"edge": edges}
    for leaf in rng.choice(np.nonzero(f.is_leaf)[0], 20, replace=False):
        path, v = set(), int(leaf)
        while v >= 0:
            path.add(v)
            v = int(f.parent[v])
        want = np.isin(edges, np.fromiter(path, dtype=np.int64)) | (edges == n)
        np.testing.assert_array_equal(pf.leaf_carriers(int(leaf)), want)
        anc = np.array(sorted(path))
        assert ((tin[anc] <= tin[leaf]) & (tin[leaf] < tout[anc])).all()
