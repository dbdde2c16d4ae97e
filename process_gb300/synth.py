"""Seeded synthetic inputs of the named workloads.

The reference builds its inputs from downloaded data (FASTA, COSMIC
signatures, germline; src/mutation_engine.cpp:75-185) and from the lattice
simulation (SpatialSimulation, src/simulation.cpp); neither is available, so
the workloads use seeded synthetic genomes, Dirichlet signatures and
birth-process forests with the shapes of each configuration:

* ``plain_3mbp``: 3 x 1 Mbp uniform ACGT, ~2.5k leaves in one sample with a
  driver subclone (species A and A+), SNV 1e-6 and indel 1e-7 per base per
  division, one Dirichlet(0.5) SBS and one ID signature; 80x paired 150 bp,
  insert Normal(350, 30), error 1e-3.
* ``full_scale``: 3.1 Gbp in 24 chromosomes at GC 41%, 3 samples x 1e4 leaves,
  3 epochs with SNV {1.5e-8, 3e-8, 5e-8} and indels at 0.1x, 3 SBS + 2 ID
  Dirichlet(0.5) signatures with per-epoch exposures; 100x paired 150 bp,
  purity 0.7, error 1e-3.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .engine import GenomeSpec, SamplesForest


def dirichlet_signatures(rng: np.random.Generator, n: int, classes: int, alpha: float, prefix: str) -> dict:
    return {f"{prefix}{i + 1}": rng.dirichlet(np.full(classes, alpha)) for i in range(n)}


def birth_forest(n_leaves: int, n_samples: int, seed: int, birth_rate: float = 0.2, t0: float = 0.0,
                 subclone: tuple[str, float] | None = ("A+", 0.6), mutant: str = "A") -> SamplesForest:
    """A binary cell forest from a pure-birth (Yule) process at ``birth_rate``,
    grown until ``n_leaves`` lineages exist; every lineage alive at the end is a
    sampled leaf.  Leaves are split into ``n_samples`` consecutive blocks of
    the depth-first order (clade-correlated samples).  The number of cell
    divisions on an edge is its duration times the birth rate (at least 1).
    ``subclone=(species, fraction)`` marks the clade closest to that fraction
    of the leaves as the driver species."""
    from .engine import preorder
    rng = np.random.default_rng(seed)
    n_nodes = 2 * n_leaves - 1
    parent = np.full(n_nodes, -1, dtype=np.int64)
    birth = np.zeros(n_nodes, dtype=np.float64)
    birth[0] = t0
    # split j (k = j + 1 lineages alive) happens after an Exp(rate * k) wait
    # and splits a uniform lineage into nodes 2j+1 and 2j+2
    k = np.arange(1, n_leaves, dtype=np.float64)
    times = t0 + np.cumsum(rng.exponential(1.0, n_leaves - 1) / (birth_rate * k))
    picks = (rng.random(n_leaves - 1) * k).astype(np.int64).tolist()
    alive = [0]
    split_parent = [0] * (n_leaves - 1)
    for j, i in enumerate(picks):
        split_parent[j] = alive[i]
        alive[i] = 2 * j + 1
        alive.append(2 * j + 2)
    if n_leaves > 1:
        sp = np.asarray(split_parent, dtype=np.int64)
        parent[1::2] = sp
        parent[2::2] = sp
        birth[1::2] = times
        birth[2::2] = times
    t_end = (times[-1] if n_leaves > 1 else t0) + rng.exponential(1.0 / (birth_rate * n_leaves))
    leaf = np.zeros(n_nodes, dtype=bool)
    leaf[alive] = True
    # leaves are born at the end of the sampled time window
    birth[leaf] = t_end
    div = np.ones(n_nodes, dtype=np.uint32)
    if n_nodes > 1:
        dt = birth[1:] - birth[parent[1:]]
        div[1:] = np.maximum(1, np.rint(dt * birth_rate)).astype(np.uint32)
    # depth-first order of the leaves, and leaves below every node
    order, pos = preorder(parent)
    size = leaf.astype(np.int64)
    for v in range(n_nodes - 1, 0, -1):           # children have larger ids than parents
        size[parent[v]] += size[v]
    dfs_leaves = order[leaf[order]]
    sample = np.full(n_nodes, None, dtype=object)
    per = int(np.ceil(n_leaves / n_samples))
    names = np.array([f"S_{j + 1}" for j in range(n_samples)], dtype=object)
    sample[dfs_leaves] = names[np.arange(len(dfs_leaves)) // per]
    mut = np.full(n_nodes, mutant, dtype=object)
    epi = np.full(n_nodes, "", dtype=object)
    if subclone is not None:
        name, frac = subclone
        target = frac * n_leaves
        cand = np.nonzero(~leaf)[0]
        best = cand[np.argmin(np.abs(size[cand] - target))] if len(cand) else 0
        # the clade of `best` (2 L - 1 nodes for L leaves in a binary tree)
        # is the preorder block starting at it
        block = np.zeros(n_nodes, dtype=bool)
        block[order[pos[best]:pos[best] + 2 * size[best] - 1]] = True
        sub_mut = name.rstrip("+-")
        mut[block] = sub_mut
        epi[block] = name[len(sub_mut):]
    return SamplesForest(np.arange(n_nodes), parent, mut, epi, sample, birth, div)


@dataclass
class Workload:
    name: str
    genome: GenomeSpec
    sbs: dict
    ids: dict
    exposures: list            # (time, {name: coeff})
    mutants: list              # (name, rates, drivers)
    forest: SamplesForest
    n_pre_snv: int = 0
    n_pre_indel: int = 0
    seq: dict = field(default_factory=dict)
    context_sampling: int = 1


def plain_3mbp(seed: int = 1, n_leaves: int = 2500) -> Workload:
    rng = np.random.default_rng(seed)
    genome = GenomeSpec(["1", "2", "3"], [1_000_000] * 3, seed=seed, gc=0.5)
    sbs = dirichlet_signatures(rng, 1, 96, 0.5, "SBS")
    ids = dirichlet_signatures(rng, 1, 83, 0.5, "ID")
    forest = birth_forest(n_leaves, 1, seed, birth_rate=0.2, subclone=("B", 0.6), mutant="A")
    rates = {"SNV": 1e-6, "indel": 1e-7}
    return Workload("plain_3mbp: 3x1 Mbp, ~2.5k leaves, 80x paired 150 bp", genome, sbs, ids,
                    [(0.0, {"SBS1": 1.0, "ID1": 1.0})], [("A", rates, []), ("B", rates, [])], forest,
                    n_pre_snv=100, n_pre_indel=10,
                    seq=dict(coverage=80, read_size=150, insert_size_mean=350, insert_size_stddev=30,
                             insert_model="normal", error_rate=1e-3, purity=1.0))


def full_scale_cnas(rng: np.random.Generator, genome: GenomeSpec, scale: float) -> tuple[list, list]:
    """20 driver CNAs of 1-50 Mbp (times the genome scale) and one WGD branch.

    The founder clone A carries 10: four single-allele deletions (copy
    number 1), two regions deleted on both alleles (0), three amplifications
    (3) and one region amplified twice (4).  The subclone B starts with a
    whole-genome doubling followed by five deletions and five
    amplifications of random alleles."""
    from .engine import CNA, WGD
    names = list(genome.chr_names)
    lengths = np.asarray(genome.chr_lengths, dtype=np.int64)
    p_chr = lengths / lengths.sum()

    def region():
        c = int(rng.choice(len(names), p=p_chr))
        ln = int(max(1000, rng.uniform(1e6, 50e6) * scale))
        ln = int(min(ln, max(1, lengths[c] // 2)))
        begin = int(rng.integers(1, max(2, lengths[c] - ln + 1)))
        return names[c], begin, ln

    a = []
    for kind in ("D1", "D1", "D1", "D1", "D0", "D0", "A3", "A3", "A3", "A4"):
        ch, b, ln = region()
        if kind == "D1":
            a.append(CNA("D", ch, b, ln, allele=0))
        elif kind == "D0":
            a += [CNA("D", ch, b, ln, allele=0), CNA("D", ch, b, ln, allele=0)]
        elif kind == "A3":
            a.append(CNA("A", ch, b, ln))
        else:
            a += [CNA("A", ch, b, ln, src_allele=0), CNA("A", ch, b, ln, src_allele=0)]
    bl = [WGD]
    for kind in ("D",) * 5 + ("A",) * 5:
        ch, b2, ln = region()
        bl.append(CNA(kind, ch, b2, ln))
    return a, bl


def full_scale(seed: int = 2, n_leaves_per_sample: int = 10_000, genome_scale: float = 1.0) -> Workload:
    rng = np.random.default_rng(seed)
    total = int(3.1e9 * genome_scale)
    w = rng.dirichlet(np.full(24, 20.0))
    lengths = np.maximum((w * total).astype(np.int64), 1000)
    genome = GenomeSpec([str(i + 1) for i in range(22)] + ["X", "Y"], lengths.tolist(), seed=seed, gc=0.41)
    sbs = dirichlet_signatures(rng, 3, 96, 0.5, "SBS")
    ids = dirichlet_signatures(rng, 2, 83, 0.5, "ID")
    forest = birth_forest(3 * n_leaves_per_sample, 3, seed, birth_rate=0.2, subclone=("B", 0.5), mutant="A")
    t_end = float(forest.birth_time.max())
    times = [0.0, t_end / 3, 2 * t_end / 3]
    exposures = []
    for t in times:
        e_s = rng.dirichlet(np.ones(3))
        e_i = rng.dirichlet(np.ones(2))
        exposures.append((t, {**{f"SBS{i + 1}": float(e_s[i]) for i in range(3)},
                              **{f"ID{i + 1}": float(e_i[i]) for i in range(2)}}))
    snv = [1.5e-8, 3e-8, 5e-8]
    rates = {"SNV": snv, "indel": [0.1 * x for x in snv]}
    cna_a, cna_b = full_scale_cnas(rng, genome, genome_scale)
    return Workload("full_scale: 3.1 Gbp/24 chr, 3x1e4 leaves, 3 epochs, 20 CNAs + 1 WGD branch, "
                    "100x paired 150 bp, purity 0.7",
                    genome, sbs, ids, exposures, [("A", rates, cna_a), ("B", rates, cna_b)], forest,
                    n_pre_snv=1000, n_pre_indel=100,
                    seq=dict(coverage=100, read_size=150, insert_size_mean=350, insert_size_stddev=10,
                             insert_model="binomial", error_rate=1e-3, purity=0.7))


@dataclass
class BatchWorkload:
    name: str
    genome: GenomeSpec
    sbs: dict
    ids: dict
    forests: list
    snv: np.ndarray
    indel: np.ndarray
    sbs_expo: np.ndarray
    id_expo: np.ndarray
    seq: list                  # per-instance sequencing keywords
    context_sampling: int = 1


def batch_256(seed: int = 3, n_inst: int = 256, leaves=(1_000, 50_000), genome_len: int = 100_000_000) -> BatchWorkload:
    """Batched replicates: n_inst forests with log-uniform leaf counts on one
    synthetic genome (4 chromosomes); per instance an SNV rate log-uniform in
    [1e-8, 1e-7] (indels at 0.1x), exposures Dirichlet(1) over 3 SBS and 2 ID
    signatures, coverage uniform in [30, 200]x, paired 150 bp reads.  The
    engine indexes every position (context_sampling 1): the busiest instances
    place ~3 M mutations under the infinite-sites model, more than a
    1-in-100 index of 100 Mbp holds."""
    rng = np.random.default_rng(seed)
    w = rng.dirichlet(np.full(4, 20.0))
    lengths = np.maximum((w * genome_len).astype(np.int64), 1000)
    genome = GenomeSpec(["1", "2", "3", "4"], lengths.tolist(), seed=seed, gc=0.41)
    sbs = dirichlet_signatures(rng, 3, 96, 0.5, "SBS")
    ids = dirichlet_signatures(rng, 2, 83, 0.5, "ID")
    lo, hi = np.log(leaves[0]), np.log(leaves[1])
    n_leaves = np.exp(rng.uniform(lo, hi, n_inst)).astype(np.int64)
    forests = [birth_forest(int(n_leaves[i]), 1, seed * 100_003 + i, subclone=None, mutant="A")
               for i in range(n_inst)]
    snv = 10 ** rng.uniform(-8, -7, n_inst)
    seq = [dict(coverage=float(rng.uniform(30, 200)), read_size=150, insert_size_mean=350, insert_size_stddev=10,
                error_rate=1e-3, purity=1.0, with_normal_sample=False) for _ in range(n_inst)]
    return BatchWorkload(f"batch_256: {n_inst} forests of {leaves[0]}-{leaves[1]} leaves (log-uniform) on a "
                         f"{genome_len / 1e6:.0f} Mbp genome, SNV 1e-8-1e-7 (log-uniform), indel 0.1x, "
                         "exposures Dirichlet(1), coverage U(30, 200)x paired 150 bp",
                         genome, sbs, ids, forests, snv, 0.1 * snv, rng.dirichlet(np.ones(3), n_inst),
                         rng.dirichlet(np.ones(2), n_inst), seq)


def build_batch(w: BatchWorkload, engine=None):
    """(engine, Batch) for a batched workload."""
    from .engine import Batch, MutationEngine
    eng = engine if engine is not None else MutationEngine(w.genome, w.sbs, w.ids,
                                                           context_sampling=w.context_sampling)
    return eng, Batch(eng, w.forests, w.snv, w.indel, w.sbs_expo, w.id_expo, w.seq)


def build_engine(w: Workload):
    """MutationEngine configured for a workload."""
    from .engine import MutationEngine
    eng = MutationEngine(w.genome, w.sbs, w.ids, context_sampling=w.context_sampling)
    for name, rates, drivers in w.mutants:
        eng.add_mutant(name, rates, drivers)
    for t, coeffs in w.exposures:
        eng.add_exposure(t, coeffs)
    return eng
