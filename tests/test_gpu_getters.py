"""PhylogeneticForest getters beside the mutation tables: the declared
driver mutations, the timed exposures and the cells where a mutation first
occurs (src/phylogenetic_forest.cpp:172-218, 565-668)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _forest():
    from process_gb300 import CNA, SNV, WGD, synth
    w = synth.plain_3mbp(seed=21, n_leaves=200)
    w.genome.chr_lengths = [200_000, 100_000, 100_000]
    (na, ra, _), (nb, rb, _) = w.mutants
    w.mutants = [(na, ra, [SNV("1", 5000, "T"), CNA("A", "2", 10_001, 20_000), CNA("D", "3", 1_001, 5_000, allele=0)]),
                 (nb, rb, [WGD])]
    eng = synth.build_engine(w)
    return w, eng, eng.place_mutations(w.forest, 20, 2, seed=3)


def test_driver_mutations_and_exposures(gpu_lib):
    w, eng, pf = _forest()
    d = pf.get_driver_mutations()
    (na, _, _), (nb, _, _) = w.mutants
    rows = list(zip(d["mutant"], d["order"], d["type"], d["CNA_type"], d["chr"], d["start"], d["end"]))
    ref = eng.get_bases(0, 5000, 1)
    want = sorted([(na, 0, "SID", None, "1", 5000, 5000), (na, 1, "CNA", "A", "2", 10_001, 30_000),
                   (na, 2, "CNA", "D", "3", 1_001, 6_000), (nb, 0, "WGD", None, None, None, None)],
                  key=lambda r: (r[0], r[1]))
    assert rows == want
    sid = list(d["type"]).index("SID")
    dele = [k for k in range(len(rows)) if d["CNA_type"][k] == "D"][0]
    assert d["ref"][sid] == ref and d["alt"][sid] == "T" and d["allele"][dele] == 0
    sp = pf.get_species_info()
    assert set(sp) == {"mutant", "epistate", "SNV_rate", "indel_rate", "CNA_rate"} and len(sp["mutant"]) >= 2
    pf.set_reference_path("ref.fa")
    assert pf.get_reference_path() == "ref.fa"
    e = pf.get_exposures()
    n = sum(len([k for k in c if k in eng.sig_names[0]]) + len([k for k in c if k in eng.sig_names[1]])
            for _, c in eng._exposures)
    assert len(e["time"]) == n
    assert set(e["type"]) <= {"SNV", "indel"}
    snv = e["type"] == "SNV"
    assert np.all(np.diff(e["time"][snv]) >= 0) and np.all(np.diff(e["time"][~snv]) >= 0)


def test_first_occurrences(gpu_lib):
    from process_gb300 import CNA, DomainError, Mutation
    w, eng, pf = _forest()
    f = w.forest
    t = pf.table()
    # a passenger SNV: the cell at the end of its edge
    i = int(np.nonzero((t["kind"] == 0) & (t["nature"] == 0))[0][0])
    cols = pf.mutation_columns(np.array([i]))
    cells = pf.get_first_occurrences(Mutation(str(cols["chr"][0]), int(cols["chr_pos"][0]), str(cols["ref"][0]),
                                              str(cols["alt"][0])))
    assert int(f.cell_id[t["edge"][i]]) in cells
    # the driver SNV and the driver amplification: the first cell of the mutant's first edge
    c = pf.cna_table()
    amp = np.nonzero((c["type"] == 1) & (c["driver"] == 1))[0][0]
    assert pf.get_first_occurrences(CNA("A", "2", 10_001, 20_000)) == [int(f.cell_id[c["node"][amp]])]
    drv = np.nonzero(t["nature"] == 1)[0]
    cells = pf.get_first_occurrences(Mutation("1", 5000, "?", "T"))
    assert cells == sorted({int(f.cell_id[v]) for v in t["edge"][drv]})
    with pytest.raises(DomainError, match="does not occurs"):
        pf.get_first_occurrences(Mutation("1", 7, "A", "C"))


def test_signatures_from_table(gpu_lib, tmp_path):
    """An engine given the signatures as tables in the reference's format
    (pg_engine_load_signatures_tsv, and through set_signatures with a path)
    places exactly what the engine given the same probabilities does, and
    reports the table's names."""
    import ctypes as C

    from process_gb300 import ID_CLASSES, SBS_CLASSES, _lib, synth
    w = synth.plain_3mbp(seed=21, n_leaves=120)
    w.genome.chr_lengths = [100_000, 50_000, 50_000]
    paths = []
    for labels, sigs, name in ((SBS_CLASSES, w.sbs, "sbs.tsv"), (ID_CLASSES, w.ids, "id.tsv")):
        p = tmp_path / name
        with open(p, "w") as fh:
            fh.write("\t".join(["Type"] + list(sigs)) + "\n")
            for i in np.random.default_rng(0).permutation(len(labels)):
                fh.write("\t".join([labels[i]] + [repr(float(sigs[k][i])) for k in sigs]) + "\n")
        paths.append(p)
    a = synth.build_engine(w)
    w2 = synth.plain_3mbp(seed=21, n_leaves=120)
    w2.genome.chr_lengths = [100_000, 50_000, 50_000]
    w2.sbs, w2.ids = str(paths[0]), str(paths[1])
    b = synth.build_engine(w2)
    ta = a.place_mutations(w.forest, 30, 3, seed=4).table()
    tb = b.place_mutations(w.forest, 30, 3, seed=4).table()
    for k in ta:
        np.testing.assert_array_equal(ta[k], tb[k], err_msg=k)
    # the C entry point directly, and the names it keeps
    _lib.check(_lib.lib().pg_engine_load_signatures_tsv(a._h, 1, str(paths[1]).encode()))
    buf, n = C.create_string_buffer(64), C.c_uint32()
    _lib.check(_lib.lib().pg_engine_signature_name(a._h, 1, 0, buf, 64, C.byref(n)))
    assert buf.value.decode() == list(w.ids)[0]
