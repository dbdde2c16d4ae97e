"""Signature tables in the reference's format (Signature::read_from_stream,
src/mutation_engine.cpp:389-397), read by the library without a device:
COSMIC class labels map to the class order the index and placement use,
rows in any order, and malformed tables are refused."""
import numpy as np
import pytest


def _write(path, labels, names, mat, order=None, header="Type"):
    rows = range(len(labels)) if order is None else order
    with open(path, "w") as fh:
        fh.write("\t".join([header] + names) + "\n")
        for i in rows:
            fh.write("\t".join([labels[i]] + [repr(float(v)) for v in mat[:, i]]) + "\n")


@pytest.mark.parametrize("type_", [0, 1])
def test_labels_map_to_class_order(tmp_path, type_):
    from process_gb300 import ID_CLASSES, SBS_CLASSES, read_signature_table
    labels = SBS_CLASSES if type_ == 0 else ID_CLASSES
    rng = np.random.default_rng(3 + type_)
    mat = rng.dirichlet(np.full(len(labels), 0.5), size=3)
    names = ["SBS1", "SBS2", "SBS17b"] if type_ == 0 else ["ID1", "ID2", "ID8"]
    path = tmp_path / "sig.tsv"
    _write(path, labels, names, mat, order=rng.permutation(len(labels)))
    got = read_signature_table(path, type_)
    assert list(got) == names
    for k, n in enumerate(names):
        np.testing.assert_array_equal(got[n], mat[k])


def test_plain_cosmic_id_labels(tmp_path):
    """The 5-base classes may be written "5" or "5+"."""
    from process_gb300 import ID_CLASSES, read_signature_table
    labels = [x.replace("5+", "5") for x in ID_CLASSES]
    mat = np.arange(83, dtype=float)[None, :] / 83.0
    path = tmp_path / "id.tsv"
    _write(path, labels, ["ID1"], mat)
    np.testing.assert_array_equal(read_signature_table(path, 1)["ID1"], mat[0])


def test_malformed_tables(tmp_path):
    from process_gb300 import SBS_CLASSES, DomainError, read_signature_table
    mat = np.full((1, 96), 1 / 96)
    cases = {
        "header": dict(header="Class"),
        "missing": dict(order=list(range(95))),
        "twice": dict(order=list(range(96)) + [7]),
    }
    for name, kw in cases.items():
        path = tmp_path / f"{name}.tsv"
        _write(path, SBS_CLASSES, ["SBS1"], mat, **kw)
        with pytest.raises(DomainError):
            read_signature_table(path, 0)
    bad = tmp_path / "label.tsv"
    _write(bad, ["A[A>C]A"] + SBS_CLASSES[1:], ["SBS1"], mat)
    with pytest.raises(DomainError, match="unknown SBS class"):
        read_signature_table(bad, 0)
    neg = tmp_path / "neg.tsv"
    _write(neg, SBS_CLASSES, ["SBS1"], -mat)
    with pytest.raises(DomainError, match="not a probability"):
        read_signature_table(neg, 0)
    with pytest.raises(DomainError, match="cannot read"):
        read_signature_table(tmp_path / "none.tsv", 0)
