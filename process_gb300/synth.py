"""Seeded synthetic inputs of the named workloads.

The reference builds its inputs from downloaded data (FASTA, COSMIC
signatures, germline; src/mutation_engine.cpp:75-185) and from the lattice
simulation (SpatialSimulation, src/simulation.cpp); neither is available, so
the workloads use seeded synthetic genomes, Dirichlet signatures and
birth-process forests with the shapes of each configuration:

* ``config1``: 3 x 1 Mbp uniform ACGT, ~2.5k leaves in one sample with a
  driver subclone (species A and A+), SNV 1e-6 and indel 1e-7 per base per
  division, one Dirichlet(0.5) SBS and one ID signature; 80x paired 150 bp,
  insert Normal(350, 30), error 1e-3.
* ``config2``: 3.1 Gbp in 24 chromosomes at GC 41%, 3 samples x 1e4 leaves,
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
    rng = np.random.default_rng(seed)
    n_nodes = 2 * n_leaves - 1
    parent = np.full(n_nodes, -1, dtype=np.int64)
    birth = np.zeros(n_nodes, dtype=np.float64)
    alive = [0]
    birth[0] = t0
    nxt = 1
    t = t0
    while len(alive) < n_leaves:
        k = len(alive)
        t += rng.exponential(1.0 / (birth_rate * k))
        i = int(rng.integers(k))
        v = alive[i]
        a, b = nxt, nxt + 1
        nxt += 2
        parent[a] = parent[b] = v
        birth[a] = birth[b] = t
        alive[i] = a
        alive.append(b)
    t_end = t + rng.exponential(1.0 / (birth_rate * len(alive)))
    # leaves are born at the end of the sampled time window
    div = np.ones(n_nodes, dtype=np.uint32)
    leaf = np.zeros(n_nodes, dtype=bool)
    leaf[alive] = True
    birth_leaf_end = birth.copy()
    birth_leaf_end[leaf] = t_end
    for v in range(1, n_nodes):
        dt = birth_leaf_end[v] - birth[parent[v]]
        div[v] = max(1, int(round(dt * birth_rate)))
    birth = birth_leaf_end
    # depth-first order of the leaves
    kids = [[] for _ in range(n_nodes)]
    for v in range(1, n_nodes):
        kids[parent[v]].append(v)
    order, stack = [], [0]
    size = np.zeros(n_nodes, dtype=np.int64)
    while stack:
        v = stack.pop()
        order.append(v)
        stack.extend(reversed(kids[v]))
    for v in reversed(order):
        size[v] = 1 if leaf[v] else sum(size[c] for c in kids[v])
    dfs_leaves = [v for v in order if leaf[v]]
    sample = np.full(n_nodes, None, dtype=object)
    per = int(np.ceil(n_leaves / n_samples))
    for j, v in enumerate(dfs_leaves):
        sample[v] = f"S_{j // per + 1}"
    mut = np.full(n_nodes, mutant, dtype=object)
    epi = np.full(n_nodes, "", dtype=object)
    if subclone is not None:
        name, frac = subclone
        target = frac * n_leaves
        cand = np.nonzero(~leaf)[0]
        best = cand[np.argmin(np.abs(size[cand] - target))] if len(cand) else 0
        stack = [best]
        sub_mut = name.rstrip("+-")
        sub_epi = name[len(sub_mut):]
        while stack:
            v = stack.pop()
            mut[v] = sub_mut
            epi[v] = sub_epi
            stack.extend(kids[v])
        if sub_mut == mutant:  # only the epistate differs
            pass
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


def config1(seed: int = 1, n_leaves: int = 2500) -> Workload:
    rng = np.random.default_rng(seed)
    genome = GenomeSpec(["1", "2", "3"], [1_000_000] * 3, seed=seed, gc=0.5)
    sbs = dirichlet_signatures(rng, 1, 96, 0.5, "SBS")
    ids = dirichlet_signatures(rng, 1, 83, 0.5, "ID")
    forest = birth_forest(n_leaves, 1, seed, birth_rate=0.2, subclone=("B", 0.6), mutant="A")
    rates = {"SNV": 1e-6, "indel": 1e-7}
    return Workload("config1: 3x1 Mbp, ~2.5k leaves, 80x paired 150 bp", genome, sbs, ids,
                    [(0.0, {"SBS1": 1.0, "ID1": 1.0})], [("A", rates, []), ("B", rates, [])], forest,
                    n_pre_snv=100, n_pre_indel=10,
                    seq=dict(coverage=80, read_size=150, insert_size_mean=350, insert_size_stddev=30,
                             insert_model="normal", error_rate=1e-3, purity=1.0))


def config2_cnas(rng: np.random.Generator, genome: GenomeSpec, scale: float) -> tuple[list, list]:
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


def config2(seed: int = 2, n_leaves_per_sample: int = 10_000, genome_scale: float = 1.0) -> Workload:
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
    cna_a, cna_b = config2_cnas(rng, genome, genome_scale)
    return Workload("config2: 3.1 Gbp/24 chr, 3x1e4 leaves, 3 epochs, 20 CNAs + 1 WGD branch, "
                    "100x paired 150 bp, purity 0.7",
                    genome, sbs, ids, exposures, [("A", rates, cna_a), ("B", rates, cna_b)], forest,
                    n_pre_snv=1000, n_pre_indel=100,
                    seq=dict(coverage=100, read_size=150, insert_size_mean=350, insert_size_stddev=10,
                             insert_model="binomial", error_rate=1e-3, purity=0.7))


def build_engine(w: Workload):
    """MutationEngine configured for a workload."""
    from .engine import MutationEngine
    eng = MutationEngine(w.genome, w.sbs, w.ids, context_sampling=w.context_sampling)
    for name, rates, drivers in w.mutants:
        eng.add_mutant(name, rates, drivers)
    for t, coeffs in w.exposures:
        eng.add_exposure(t, coeffs)
    return eng
