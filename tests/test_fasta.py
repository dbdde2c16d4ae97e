"""Reference genomes from FASTA, with unknown bases: parsing (names, lengths,
codes, record selection, gzip) and the oracle's indices, which skip every
context and repeat site that touches an unknown base (N)."""
import gzip

import numpy as np
import pytest

FASTA = b""">chr1 the first
ACGTN
acgtr
>chr2
NNNNACGT
>chrUn_x extra
AC
"""


def test_from_fasta(tmp_path):
    from process_gb300 import DomainError, GenomeSpec
    p = tmp_path / "ref.fa"
    p.write_bytes(FASTA)
    g = GenomeSpec.from_fasta(str(p))
    assert list(g.chr_names) == ["chr1", "chr2", "chrUn_x"]
    assert list(g.chr_lengths) == [10, 8, 2]
    np.testing.assert_array_equal(g.bases, [0, 1, 2, 3, 4, 0, 1, 2, 3, 4, 4, 4, 4, 4, 0, 1, 2, 3, 0, 1])
    # a selection keeps the file's order
    g2 = GenomeSpec.from_fasta(str(p), chromosomes=["chr2", "chr1"])
    assert list(g2.chr_names) == ["chr1", "chr2"] and g2.total == 18
    pz = tmp_path / "ref.fa.gz"
    pz.write_bytes(gzip.compress(FASTA))
    np.testing.assert_array_equal(GenomeSpec.from_fasta(str(pz)).bases, g.bases)
    with pytest.raises(DomainError, match="not in"):
        GenomeSpec.from_fasta(str(p), chromosomes=["chr9"])


def test_oracle_indices_skip_unknown_bases(orc):
    rng = np.random.default_rng(3)
    b = rng.integers(0, 4, 60_000).astype(np.uint8)
    b[100:140] = 4                      # an N run
    b[5000] = 4                         # an isolated N
    b[29_998:30_003] = 4                # N across the chromosome boundary
    b[40_000:40_040] = 2                # a homopolymer beside
    b[40_040:40_050] = 4                #   an N run
    lengths = [30_000, 30_000]
    o = orc.OracleEngine(lengths, b, context_sampling=1, max_rep=10**9)
    g = o.read_genome()
    np.testing.assert_array_equal(g, b)
    unknown = np.nonzero(b == 4)[0]
    total = 0
    for c in range(32):
        pos = o.read_index(0, c).astype(np.int64)
        total += len(pos)
        assert not np.isin(pos, unknown).any() and not np.isin(pos - 1, unknown).any()
        assert not np.isin(pos + 1, unknown).any()
    # every triplet inside a chromosome with three known bases is indexed
    ok = 0
    for s, e in ((0, 30_000), (30_000, 60_000)):
        x = b[s:e]
        ok += int(((x[:-2] < 4) & (x[1:-1] < 4) & (x[2:] < 4)).sum())
    assert total == ok
    for c in range(83):
        pos = o.read_index(1, c).astype(np.int64)
        assert not np.isin(pos, unknown).any() and not np.isin(pos - 1, unknown).any()
