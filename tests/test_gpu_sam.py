"""SAM output of simulate_seq(write_SAM=TRUE): files, naming, read groups,
and reads that agree with the counts.  Counting, in the SAM files, the reads
that cover each SNV and those that show its alt base gives back the
alt/depth tables of the read kernel exactly (same seed and tile size), also
with copy-number events; reads with indels carry consistent CIGARs."""
import re
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CIG = re.compile(r"(\d+)([MID])")


def _parse(path):
    head, reads = [], []
    for line in Path(path).read_text().splitlines():
        if line.startswith("@"):
            head.append(line)
            continue
        f = line.split("\t")
        reads.append(f)
    return head, reads


def _sam_counts(files, t, sample_names, chr_off, chr_names, R):
    """alt/depth of every SNV of table t from the reads of the SAM files."""
    snv = np.nonzero(t["kind"] == 0)[0]
    loci = t["locus"][snv].astype(np.int64)
    alt_base = np.array(list("ACGT"))[t["aux"][snv] & 3]
    idx = {n: i for i, n in enumerate(sample_names)}
    dep = np.zeros((len(sample_names), len(t["locus"])), dtype=np.int64)
    alt = np.zeros_like(dep)
    for path in files:
        _, reads = _parse(path)
        for f in reads:
            if int(f[1]) & 4:
                continue
            ci = chr_names.index(f[2])
            pos = chr_off[ci] + int(f[3]) - 1
            seq = f[9]
            s = idx[f[11].split(":")[2]]
            ops = CIG.findall(f[5])
            assert sum(int(n) for n, o in ops if o in "MI") == len(seq)
            # aligned (reference, read) pairs of the M runs
            q, r = pos, 0
            for n, o in ops:
                n = int(n)
                if o == "M":
                    lo, hi = np.searchsorted(loci, [q, q + n])
                    for k in range(lo, hi):
                        m = snv[k]
                        dep[s, m] += 1
                        if seq[r + int(loci[k] - q)] == alt_base[k]:
                            alt[s, m] += 1
                    q += n
                    r += n
                elif o == "I":
                    r += n
                else:
                    q += n
    return alt, dep


def _check_against_counts(pf, eng, tmp_path, cfg, names, seed=17):
    from process_gb300.engine import sequence_counts
    out = tmp_path / "sam"
    res = sequence_counts(pf, seed, sam=dict(output_dir=str(out), sample_names=names), **cfg)
    alt, dep = res.counts()
    files = sorted(out.glob("chr_*.sam"))
    assert [f.name for f in files] == sorted(f"chr_{n}.sam" for n in eng.chr_names)
    head, _ = _parse(files[0])
    assert head[0].startswith("@HD") and any(h.startswith("@SQ") for h in head)
    assert [h.split("\t")[1] for h in head if h.startswith("@RG")] == [f"ID:{n}" for n in names]
    t = pf.table()
    salt, sdep = _sam_counts(files, t, names, eng.chr_off.astype(np.int64), eng.chr_names, cfg["read_size"])
    snv = t["kind"] == 0
    np.testing.assert_array_equal(sdep[:, snv], dep[:, snv])
    np.testing.assert_array_equal(salt[:, snv], alt[:, snv])
    n_lines = sum(len(_parse(f)[1]) for f in files)
    assert n_lines == res.dims()[2]
    return files


def test_sam_reads_match_counts(gpu_lib, tmp_path):
    from process_gb300 import synth
    w = synth.plain_3mbp(seed=9, n_leaves=150)
    w.genome.chr_lengths = [120_000, 80_000, 60_000]
    w.mutants = [(n, dict(r, indel=0.0), d) for n, r, d in w.mutants]
    eng = synth.build_engine(w)
    pf = eng.place_mutations(w.forest, 30, 0, seed=3)
    cfg = dict(coverage=15, read_size=120, insert_size_mean=300, insert_size_stddev=10, error_rate=5e-3,
               purity=0.8, with_normal_sample=True, tile_size=2048)
    names = list(w.forest.sample_names) + ["normal_sample"]
    _check_against_counts(pf, eng, tmp_path, cfg, names)


def test_sam_with_copy_number_and_single_end(gpu_lib, tmp_path):
    from process_gb300 import CNA, WGD, synth
    w = synth.plain_3mbp(seed=10, n_leaves=120)
    w.genome.chr_lengths = [150_000, 100_000, 50_000]
    (na, ra, _), (nb, rb, _) = w.mutants
    w.mutants = [(na, dict(ra, indel=0.0), [CNA("A", "1", 20_001, 40_000), CNA("D", "2", 10_001, 30_000, allele=0)]),
                 (nb, dict(rb, indel=0.0), [WGD])]
    eng = synth.build_engine(w)
    pf = eng.place_mutations(w.forest, 0, 0, seed=4)
    assert pf.node_classes()[1] > 1
    cfg = dict(coverage=20, read_size=100, insert_size_mean=0, error_rate=1e-2, purity=0.6,
               with_normal_sample=False, tile_size=4096)
    _check_against_counts(pf, eng, tmp_path, cfg, list(w.forest.sample_names))


def test_sam_indels_naming_and_update(gpu_lib, tmp_path):
    from process_gb300 import DomainError, simulate_seq, synth
    w = synth.plain_3mbp(seed=11, n_leaves=100)
    w.genome.chr_lengths = [100_000, 50_000, 50_000]
    w.mutants = [(n, dict(r, indel=2e-6), d) for n, r, d in w.mutants]
    eng = synth.build_engine(w)
    pf = eng.place_mutations(w.forest, 10, 10, seed=5)
    out = tmp_path / "ProCESS_SAM"
    simulate_seq(pf, coverage=10, write_SAM=True, output_dir=str(out), insert_size_mean=300,
                 insert_size_stddev=10, seed=1)
    assert sorted(p.name for p in out.iterdir()) == ["chr_1.sam", "chr_2.sam", "chr_3.sam"]
    n_id = 0
    for p in out.iterdir():
        _, reads = _parse(p)
        for f in reads:
            ops = CIG.findall(f[5])
            assert sum(int(n) for n, o in ops if o in "MI") == len(f[9]) == len(f[10])
            n_id += any(o in "ID" for _, o in ops)
            assert f[0].startswith("r")
    assert n_id > 0
    # an existing directory needs update_SAM; then files get the first free suffix
    with pytest.raises(DomainError, match="already exists"):
        simulate_seq(pf, coverage=2, write_SAM=True, output_dir=str(out), seed=2)
    simulate_seq(pf, coverage=2, write_SAM=True, update_SAM=True, output_dir=str(out), seed=2,
                 chromosomes=["2"], filename_prefix="chr_", template_name_prefix="t")
    assert (out / "chr_2_1.sam").exists()
    _, reads = _parse(out / "chr_2_1.sam")
    assert reads and all(f[0].startswith("t") for f in reads)


def test_sam_reads_match_oracle(gpu_lib, orc, tmp_path):
    """Every SAM read -- FLAG, POS, CIGAR, mate POS, TLEN and the bases --
    equals the oracle's own restatement of the read builder (reference
    window, carried SNVs and indels through its carrier closure, error
    substitutions, mate positions), read by read in file order, on a forest
    with CNAs, a WGD and frequent indels, at a high error rate."""
    from process_gb300.engine import seq_cfg, sequence_counts
    from test_gpu_cna import _pair, _species, _tables_equal, _workload
    w, cands = _workload(seed=13, n_leaves=120)
    w.mutants = [(n, dict(r, indel=3e-6, SNV=5e-6), d) for n, r, d in w.mutants]
    eng, o = _pair(orc, w, cands, True, True)
    pf = eng.place_mutations(w.forest, 60, 20, seed=3)
    op = o.place(w.forest, _species(o, w.forest), 60, 0, 20, 0, seed=3)
    _tables_equal(pf.table(), op.table())
    assert (pf.table()["kind"] == 1).sum() > 50
    cfg = dict(coverage=2, read_size=100, insert_size_mean=250, insert_size_stddev=10, error_rate=2e-2, purity=0.8)
    names = list(w.forest.sample_names) + ["normal_sample"]
    out = tmp_path / "sam"
    res = sequence_counts(pf, 31, sam=dict(output_dir=str(out), sample_names=names), **cfg)
    c, _ = seq_cfg(chr_index=eng._chr_index, tile_size=res.tile_size(), **cfg)
    want = op.sam_reads(c, 31, tmp_path / "expected.tsv")
    got = {}
    n_indel_reads = 0
    for path in sorted(out.glob("*.sam")):
        head, reads = _parse(path)
        chrom = [h.split("\t")[1][3:] for h in head if h.startswith("@SQ")][0]
        ci = eng._chr_index(chrom)
        for f in reads:
            s = names.index(f[11].split(":")[2])
            row = ("4", "*", "*", "*", "*", "*") if int(f[1]) & 4 else (f[1], f[3], f[5], f[7], f[8], f[9])
            n_indel_reads += ("I" in f[5]) or ("D" in f[5])
            got.setdefault((s, ci), []).append(row)
    assert set(got) == set(want)
    for k in want:
        assert got[k] == want[k], k
    assert n_indel_reads > 0
