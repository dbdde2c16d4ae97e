"""Host-side mirror of the ProCESS API for the placement and sequencing path.

Names, arguments, defaults and returned data-frame columns follow the
reference's Rcpp modules:

* ``MutationEngine`` — ``src/mutations.cpp:392-756`` (methods) and the factory
  defaults ``:938-951``; ``place_mutations`` overloads
  ``src/mutation_engine.hpp:160-206``.
* ``PhylogeneticForest`` getters — ``src/phylogenetic_forest.cpp:57-99, 323-562``.
* ``simulate_seq`` / ``simulate_normal_seq`` — ``src/sequencing.cpp:193-209, 268-282``
  and the result flattening of ``src/seq_simulation.cpp:52-181``.
* ``BasicIlluminaSequencer`` / ``ErrorlessIlluminaSequencer`` —
  ``src/sequencers.cpp:78-105``.

Data frames are returned as ``dict[str, numpy.ndarray]`` with the reference's
column names (pandas is not a dependency).  All computation runs in the CUDA
library through the C-ABI; this module only validates and arranges inputs.
"""
from __future__ import annotations

import ctypes as C
import itertools
from dataclasses import dataclass, field
from typing import Iterable, Mapping, Sequence

import numpy as np

from . import _lib
from ._lib import DomainError, check, lib, ptr

BASES = np.array(list("ACGTN"))   # base codes; 4: unknown (N)
_SUBS = ["C>A", "C>G", "C>T", "T>A", "T>C", "T>G"]
SBS_CLASSES = [f"{f}[{s}]{t}" for s in _SUBS for f in "ACGT" for t in "ACGT"]
ID_CLASSES = (
    [f"1:Del:{b}:{k}" for b in "CT" for k in range(6)]
    + [f"1:Ins:{b}:{k}" for b in "CT" for k in range(6)]
    + [f"{ln}:Del:R:{k}" for ln in (2, 3, 4, "5+") for k in range(6)]
    + [f"{ln}:Ins:R:{k}" for ln in (2, 3, 4, "5+") for k in range(6)]
    + ["2:Del:M:1", "3:Del:M:1", "3:Del:M:2", "4:Del:M:1", "4:Del:M:2", "4:Del:M:3",
       "5:Del:M:1", "5:Del:M:2", "5:Del:M:3", "5:Del:M:4", "5:Del:M:5"]
)
assert len(SBS_CLASSES) == 96 and len(ID_CLASSES) == 83

NATURES = np.array(["passenger", "driver", "preneoplastic", "germinal"])


def _seed(seed) -> int:
    """Seed semantics of the reference: NULL draws one (src/utility.hpp:41-64)."""
    if seed is None:
        return int(np.random.default_rng().integers(0, 2**31 - 1))
    return int(seed) & 0xFFFFFFFFFFFFFFFF


# ---------------------------------------------------------------- genome
@dataclass
class GenomeSpec:
    """Reference genome: chromosome names and lengths plus either explicit base
    codes (A=0 C=1 G=2 T=3) or a seeded synthetic i.i.d. sequence."""

    chr_names: Sequence[str]
    chr_lengths: Sequence[int]
    bases: np.ndarray | None = None
    seed: int = 0
    gc: float = 0.5

    @property
    def total(self) -> int:
        return int(np.sum(np.asarray(self.chr_lengths, dtype=np.uint64)))

    @classmethod
    def from_fasta(cls, path: str, chromosomes: Sequence[str] | None = None) -> "GenomeSpec":
        """A reference genome read from a FASTA file (gzip-compressed when the
        name ends in .gz), the reference's input to its context and repeat
        indices (src/mutation_engine.cpp:211-359).  Each record's name is the
        first word of its header; ``chromosomes`` keeps only those records, in
        the file's order.  A, C, G, T (either case) become codes 0-3; every
        other letter (N and the other ambiguity codes) is an unknown base
        (code 4), which no context or repeat site that touches it indexes."""
        import gzip
        opener = gzip.open if str(path).endswith(".gz") else open
        with opener(path, "rb") as fh:
            data = fh.read()
        lut = np.full(256, 4, dtype=np.uint8)
        for k, c in enumerate(b"ACGT"):
            lut[c] = k
            lut[c + 32] = k                       # lower case
        keep = None if chromosomes is None else {str(c) for c in chromosomes}
        names, lengths, parts = [], [], []
        for rec in data.split(b">")[1:]:
            head, _, body = rec.partition(b"\n")
            name = head.split()[0].decode() if head.split() else ""
            if keep is not None and name not in keep:
                continue
            seq = body.translate(None, b"\r\n\t ")
            if not seq:
                raise DomainError(_lib.PG_ERR_DOMAIN, f'FASTA record "{name}" has no bases')
            names.append(name)
            lengths.append(len(seq))
            parts.append(lut[np.frombuffer(seq, dtype=np.uint8)])
        if keep is not None and len(set(names)) != len(keep):
            missing = sorted(keep - set(names))
            raise DomainError(_lib.PG_ERR_DOMAIN, f"chromosomes not in {path}: {', '.join(missing)}")
        if not names:
            raise DomainError(_lib.PG_ERR_DOMAIN, f"no chromosome read from {path}")
        return cls(names, lengths, bases=np.concatenate(parts))


# ---------------------------------------------------------------- driver specs
@dataclass
class Mutation:
    """Driver SNV/indel (``Mutation(chr, chr_pos, ref, alt, allele)``, src/mutations.cpp:30-120)."""

    chr: str
    chr_pos: int
    ref: str
    alt: str
    allele: int | None = None


def SNV(chr: str, chr_pos: int, alt: str, ref: str = "?", allele: int | None = None) -> Mutation:
    """``SNV(chr, chr_pos, alt, ref, allele)``; a "?" ref is read from the genome."""
    return Mutation(chr, chr_pos, ref, alt, allele)


@dataclass
class CNA:
    type: str
    chr: str
    chr_pos: int
    len: int
    allele: int | None = None
    src_allele: int | None = None


def load_passenger_CNAs(path, tumour_type: str = "", tumour_study: str = "") -> list[CNA]:
    """Passenger CNA candidates from a tab-separated table with a header row
    and the columns chr, begin, end, major, minor, tumour type, study
    (load_passenger_CNAs, src/mutation_engine.cpp:441-487): rows of the
    requested tumour type and study ("" = any) give an amplification when
    major is NA or above 1 and a deletion when minor is NA or below 1, over
    [begin, end]; duplicates are dropped."""
    out = set()
    with open(path) as fh:
        rows = [ln.rstrip("\n").split("\t") for ln in fh]
    for num, row in enumerate(rows[1:], start=2):
        if not row or row == [""]:
            continue
        if len(row) < 7:
            raise RuntimeError("The CNA CSV must contains at least 7 columns")
        if (tumour_type and row[5] != tumour_type) or (tumour_study and row[6] != tumour_study):
            continue
        try:
            begin, end = int(row[1]), int(row[2])
        except ValueError:
            raise DomainError(_lib.PG_ERR_DOMAIN, f"Unknown begin/end specification in row number {num}.")
        if begin > end:
            raise DomainError(_lib.PG_ERR_DOMAIN, f"The CNA begin lays after the end in row number {num}")
        for col, amp in ((3, True), (4, False)):
            v = row[col]
            try:
                hit = v == "NA" or (int(v) > 1 if amp else int(v) < 1)
            except ValueError:
                raise DomainError(_lib.PG_ERR_DOMAIN, f"Unknown major/minor specification {v} in row number {num}.")
            if hit:
                out.add(("A" if amp else "D", row[0], begin, end + 1 - begin))

    def key(c):
        return (0, int(c[1]), "") if c[1].isdigit() else (1, 0, c[1])
    return [CNA(t, ch, b, ln) for t, ch, b, ln in sorted(out, key=lambda c: (key(c), c[2], c[3], c[0]))]


class _WGD:
    def __repr__(self):
        return "WGD"


WGD = _WGD()


# ---------------------------------------------------------------- sequencers
@dataclass
class ErrorlessIlluminaSequencer:
    """An error-free Illumina sequencer (src/sequencers.hpp:25-38)."""

    @property
    def error_rate(self) -> float:
        return 0.0


@dataclass
class BasicIlluminaSequencer:
    """Illumina sequencer with a base-, position- and read-independent error
    rate (src/sequencers.hpp:40-72); validation of src/sequencers.cpp:78-105."""

    error_rate: float
    random_quality_scores: bool = True

    def __post_init__(self):
        if not isinstance(self.error_rate, (int, float)) or self.error_rate < 0:
            raise DomainError(_lib.PG_ERR_DOMAIN, 'The parameter "error_rate" must be a positive real number.')
        if not isinstance(self.random_quality_scores, bool):
            raise DomainError(_lib.PG_ERR_DOMAIN, 'The parameter "random_quality_scores" must be a Boolean value.')


# ---------------------------------------------------------------- forest
def preorder(par: np.ndarray, with_size: bool = False):
    """Depth-first preorder of a forest given parent indices (-1 for roots;
    roots and children visited in index order): the order and each node's
    position in it (and, with_size, each subtree's node count).  Level by
    level with numpy; raises on a cycle."""
    par = np.asarray(par, dtype=np.int64)
    n = len(par)
    root = par < 0
    kids = np.argsort(np.where(root, n, par), kind="stable")[: n - int(root.sum())]
    ptr = np.zeros(n + 1, dtype=np.int64)
    np.add.at(ptr, par[~root] + 1, 1)
    ptr = np.cumsum(ptr)
    roots = np.nonzero(root)[0]
    levels, frontier, seen = [roots], roots, len(roots)
    while True:
        cnt = ptr[frontier + 1] - ptr[frontier]
        tot = int(cnt.sum())
        if tot == 0:
            break
        first = np.cumsum(cnt) - cnt
        frontier = kids[np.repeat(ptr[frontier], cnt) + np.arange(tot) - np.repeat(first, cnt)]
        levels.append(frontier)
        seen += tot
        if seen > n:
            break
    if seen != n:
        raise DomainError(_lib.PG_ERR_DOMAIN, "the ancestor relation is not a forest")
    size = np.ones(n, dtype=np.int64)
    for lvl in reversed(levels[1:]):
        np.add.at(size, par[lvl], size[lvl])
    pos = np.empty(n, dtype=np.int64)
    pos[roots] = np.cumsum(size[roots]) - size[roots]
    for lvl in levels[1:]:
        p = par[lvl]
        sz = size[lvl]
        cs = np.cumsum(sz)
        start = np.r_[True, p[1:] != p[:-1]]
        head = np.maximum.accumulate(np.where(start, np.arange(len(lvl)), 0))
        pos[lvl] = pos[p] + 1 + (cs - sz) - (cs[head] - sz[head])
    order = np.empty(n, dtype=np.int64)
    order[pos] = np.arange(n)
    return (order, pos, size) if with_size else (order, pos)


class SamplesForest:
    """A samples forest (``DescendantsForest``, node columns of src/forest.hpp:29-68).

    ``divisions`` is the number of cell divisions on the edge into each node
    (1 for a forest that keeps every division as a node)."""

    def __init__(self, cell_id, ancestor, mutant, epistate, sample, birth_time, divisions=None):
        cell_id = np.asarray(cell_id, dtype=np.int64)
        n = len(cell_id)
        ancestor = np.asarray(ancestor, dtype=np.int64)  # -1 = root (NA)
        self.mutant = np.asarray(mutant, dtype=object)
        self.epistate = np.asarray(epistate, dtype=object)
        sample = np.asarray(sample, dtype=object)
        self.birth_time = np.asarray(birth_time, dtype=np.float64)
        self.divisions = (np.ones(n, dtype=np.uint32) if divisions is None
                          else np.asarray(divisions, dtype=np.uint32))
        # depth-first preorder (parents first, children in the given order)
        if np.array_equal(cell_id, np.arange(n)):
            par = np.where(ancestor >= 0, ancestor, -1)
            if np.any(par >= n):
                raise DomainError(_lib.PG_ERR_DOMAIN, "unknown ancestor id")
        else:
            srt = np.argsort(cell_id, kind="stable")
            at = np.searchsorted(cell_id[srt], ancestor)
            at = np.minimum(at, n - 1)
            found = (ancestor >= 0) & (cell_id[srt][at] == ancestor)
            if np.any((ancestor >= 0) & ~found):
                raise DomainError(_lib.PG_ERR_DOMAIN, "unknown ancestor id")
            par = np.where(found, srt[at], -1)
        order, _ = preorder(par)
        inv = np.empty(n, dtype=np.int64)
        inv[order] = np.arange(n)
        self.cell_id = cell_id[order]
        self.parent = np.where(par[order] >= 0, inv[np.maximum(par[order], 0)], -1).astype(np.int32)
        self.mutant = self.mutant[order]
        self.epistate = self.epistate[order]
        self.birth_time = self.birth_time[order]
        self.divisions = self.divisions[order]
        sample = sample[order]
        names = sorted({str(s) for s in sample if s is not None and str(s) != "" and str(s) != "nan"})
        self.sample_names = list(names)
        idx = {s: i for i, s in enumerate(names)}
        self.sample = np.array([idx.get(str(s), -1) if s is not None else -1 for s in sample], dtype=np.int32)
        is_parent = np.zeros(n, dtype=bool)
        is_parent[self.parent[self.parent >= 0]] = True
        self.is_leaf = ~is_parent

    def euler(self) -> tuple[np.ndarray, np.ndarray]:
        """(tin, tout) of every node: its depth-first preorder position and one
        past its subtree's last, so v is an ancestor-or-self of u iff
        tin[v] <= tin[u] < tout[v]."""
        if getattr(self, "_euler", None) is None:
            _, pos, size = preorder(self.parent, with_size=True)
            self._euler = (pos, pos + size)
        return self._euler

    def species_codes(self) -> tuple[list[tuple[str, str]], np.ndarray]:
        """The distinct (mutant, epistate) pairs and each node's index among
        them (computed once per pair of mutant/epistate arrays)."""
        cache = getattr(self, "_codes", None)
        if cache is not None and cache[0] is self.mutant and cache[1] is self.epistate:
            return cache[2], cache[3]
        table: dict[tuple[str, str], int] = {}
        code = np.fromiter((table.setdefault((str(m), "" if e is None else str(e)), len(table))
                            for m, e in zip(self.mutant.tolist(), self.epistate.tolist())),
                           dtype=np.int64, count=len(self.mutant))
        names = list(table)
        self._codes = (self.mutant, self.epistate, names, code)
        return names, code

    @property
    def num_of_nodes(self) -> int:
        return len(self.cell_id)

    def get_nodes(self) -> dict:
        anc = np.where(self.parent >= 0, self.cell_id[np.maximum(self.parent, 0)], -1)
        smp = np.array([self.sample_names[s] if s >= 0 else None for s in self.sample], dtype=object)
        return {"cell_id": self.cell_id.copy(), "ancestor": anc, "mutant": self.mutant.copy(),
                "epistate": self.epistate.copy(), "sample": smp, "birth_time": self.birth_time.copy()}

    def get_samples_info(self) -> dict:
        counts = np.bincount(self.sample[self.is_leaf & (self.sample >= 0)], minlength=len(self.sample_names))
        return {"name": np.array(self.sample_names, dtype=object), "tumour_cells": counts}


# ---------------------------------------------------------------- engine
class MutationEngine:
    """``MutationEngine`` over a GPU-resident genome and its context / repeat indices.

    The reference downloads a FASTA, signatures and germline data by setup
    code (src/mutation_engine.cpp:75-185); here the genome, signatures and
    species are given directly."""

    def __init__(self, genome: GenomeSpec, SBS_signatures: Mapping[str, Sequence[float]] | None = None,
                 indel_signatures: Mapping[str, Sequence[float]] | None = None, context_sampling: int = 100,
                 max_motif_size: int = 50, max_repetition_storage: int = 500000,
                 avoid_homozygous_losses: bool = True, passenger_CNAs: Iterable | None = None):
        self.genome = genome
        self.chr_names = [str(c) for c in genome.chr_names]
        self.chr_lengths = np.asarray(genome.chr_lengths, dtype=np.uint32)
        self.chr_off = np.concatenate([[0], np.cumsum(self.chr_lengths.astype(np.uint64))]).astype(np.uint64)
        self.context_sampling = int(context_sampling)
        self.max_motif_size = int(max_motif_size)
        self.max_repetition_storage = int(max_repetition_storage)
        d = _lib.GenomeDesc()
        d.n_chr = len(self.chr_lengths)
        d.chr_lengths = ptr(self.chr_lengths, C.c_uint32)
        bases = None
        if genome.bases is not None:
            bases = np.ascontiguousarray(genome.bases, dtype=np.uint8)
            if bases.size != genome.total:
                raise DomainError(_lib.PG_ERR_DOMAIN, "bases do not match the chromosome lengths")
            d.bases = ptr(bases, C.c_uint8)
        d.synthetic_seed = int(genome.seed)
        d.synthetic_gc = float(genome.gc)
        d.context_sampling = self.context_sampling
        d.max_repetition_storage = self.max_repetition_storage
        h = C.c_void_p()
        check(lib().pg_engine_create(C.byref(d), C.byref(h)))
        self._h = h
        self.sig_names: list[list[str]] = [[], []]
        self.mutants: list[str] = []
        self.species: dict[tuple[str, str], int] = {}
        self.species_rates: dict[tuple[str, str], dict] = {}
        self._exposures: list[tuple[float, dict]] = []
        self._sigs: list[dict] = [{}, {}]
        self._mutant_specs: list[tuple[str, dict, list]] = []   # add_mutant calls, in order
        self.passenger_CNAs: list[CNA] = []
        self.avoid_homozygous_losses = bool(avoid_homozygous_losses)
        if SBS_signatures:
            self.set_signatures(0, SBS_signatures)
        if indel_signatures:
            self.set_signatures(1, indel_signatures)
        if passenger_CNAs:
            self.add_passenger_CNAs(passenger_CNAs)

    @property
    def avoid_homozygous_losses(self) -> bool:
        """Passenger deletions never remove the last allele of a region
        (``avoid_homozygous_losses``, src/mutations.cpp:837-840, default TRUE)."""
        return self._avoid_losses

    @avoid_homozygous_losses.setter
    def avoid_homozygous_losses(self, value: bool) -> None:
        check(lib().pg_engine_set_avoid_homozygous_losses(self._h, 1 if value else 0))
        self._avoid_losses = bool(value)

    def add_passenger_CNAs(self, cnas: Iterable) -> None:
        """Appends passenger CNA candidates (``CNA`` objects; the reference
        loads them from its passenger-CNA table, src/mutation_engine.cpp:441-487,
        see :func:`load_passenger_CNAs`).  A species with CNA rate r draws
        Poisson(r * 2G * divisions) of them per edge, uniformly."""
        for c in cnas:
            if not isinstance(c, CNA) or c.type not in ("A", "D"):
                raise DomainError(_lib.PG_ERR_DOMAIN, "passenger CNA candidates are CNA(\"A\"|\"D\", ...) objects")
            ci = self._chr_index(c.chr)
            check(lib().pg_engine_add_passenger_cna(self._h, ci, int(c.chr_pos), int(c.len),
                                                    1 if c.type == "A" else 0))
            self.passenger_CNAs.append(c)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _lib._LIB is not None:
            _lib._LIB.pg_engine_destroy(h)
            self._h = None

    # -- signatures and exposures ------------------------------------------------
    def set_signatures(self, type_: int, sigs: Mapping[str, Sequence[float]]) -> None:
        nc = 96 if type_ == 0 else 83
        names = list(sigs.keys())
        mat = np.ascontiguousarray(np.array([np.asarray(sigs[k], dtype=np.float64) for k in names]))
        if mat.shape != (len(names), nc):
            raise DomainError(_lib.PG_ERR_DOMAIN, f"signatures must have {nc} classes")
        check(lib().pg_engine_set_signatures(self._h, type_, len(names), ptr(mat, C.c_double)))
        self.sig_names[type_] = names
        self._sigs[type_] = {k: mat[i].tolist() for i, k in enumerate(names)}

    def add_exposure(self, time: float = 0.0, coefficients: Mapping[str, float] | None = None) -> None:
        """``add_exposure(time, coefficients)`` (src/mutation_engine.cpp:734-739): one
        call may set SBS and ID exposures together; names select the type."""
        if coefficients is None:
            raise DomainError(_lib.PG_ERR_DOMAIN, "missing exposure coefficients")
        by_type = [np.zeros(len(self.sig_names[0])), np.zeros(len(self.sig_names[1]))]
        used = [False, False]
        for name, c in coefficients.items():
            if c < 0:
                raise DomainError(_lib.PG_ERR_DOMAIN, f"{name}: exposure coefficients must be non-negative")
            for ty in (0, 1):
                if name in self.sig_names[ty]:
                    by_type[ty][self.sig_names[ty].index(name)] = c
                    used[ty] = True
                    break
            else:
                raise DomainError(_lib.PG_ERR_DOMAIN, f"Unknown signature {name}")
        for ty in (0, 1):
            if used[ty]:
                s = by_type[ty].sum()
                if abs(s - 1.0) > 1e-6:
                    raise DomainError(_lib.PG_ERR_DOMAIN, "The exposure coefficients must sum up to 1")
                check(lib().pg_engine_add_exposure(self._h, ty, float(time), ptr(np.ascontiguousarray(by_type[ty]),
                                                                                    C.c_double)))
        self._exposures.append((float(time), dict(coefficients)))

    # -- mutants -----------------------------------------------------------------
    def _species_id(self, mutant: str, epistate: str) -> int:
        key = (mutant, epistate)
        if key not in self.species:
            self.species[key] = len(self.species)
        return self.species[key]

    def add_mutant(self, mutant_name: str, passenger_rates: Mapping, drivers: Iterable = ()) -> None:
        """``add_mutant(mutant_name, passenger_rates, drivers)`` (src/mutation_engine.cpp:864-1083).

        ``passenger_rates`` is ``{"SNV": r, "indel": r, "CNA": r}`` or
        ``{"+": {...}, "-": {...}}``; a rate may be a sequence giving one value
        per exposure epoch."""
        drivers = list(drivers)
        if mutant_name in self.mutants:
            raise DomainError(_lib.PG_ERR_DOMAIN, f"mutant {mutant_name} already declared")
        mut_id = len(self.mutants)
        self.mutants.append(mutant_name)
        keys = set(passenger_rates.keys())
        if keys <= {"SNV", "indel", "CNA"}:
            per_epi = {"": passenger_rates}
        elif keys <= {"+", "-"}:
            per_epi = dict(passenger_rates)
        else:
            raise DomainError(_lib.PG_ERR_DOMAIN, "Passenger rates list must be a named list whose names are in "
                              'the set {"SNV", "indel", "CNA"} or epistates "+"/"-".')
        for epi, rates in per_epi.items():
            for k in rates:
                if k not in ("SNV", "indel", "CNA"):
                    raise DomainError(_lib.PG_ERR_DOMAIN, f'"{k}" is an unsupported name in passenger rates list.')
            sid = self._species_id(mutant_name, epi)
            snv, indel, cna = rates.get("SNV", 0.0), rates.get("indel", 0.0), rates.get("CNA", 0.0)
            if np.ndim(snv) or np.ndim(indel):
                n = max(np.size(snv), np.size(indel))
                s_arr = np.ascontiguousarray(np.broadcast_to(np.asarray(snv, dtype=np.float64), (n,)))
                i_arr = np.ascontiguousarray(np.broadcast_to(np.asarray(indel, dtype=np.float64), (n,)))
                check(lib().pg_engine_set_species_epoch_rates(self._h, sid, n, ptr(s_arr, C.c_double),
                                                              ptr(i_arr, C.c_double)))
                check(lib().pg_engine_set_species_rates(self._h, sid, float(s_arr[0]), float(i_arr[0]), float(cna)))
            else:
                check(lib().pg_engine_set_species_rates(self._h, sid, float(snv), float(indel), float(cna)))
            check(lib().pg_engine_set_species_mutant(self._h, sid, mut_id))
            self.species_rates[(mutant_name, epi)] = {"SNV": snv, "indel": indel, "CNA": cna}
        for d in drivers:
            if isinstance(d, Mutation):
                chr_idx = self._chr_index(d.chr)
                ref = d.ref
                if ref == "?":
                    ref = self.get_bases(chr_idx, d.chr_pos, 1)
                al = -1 if d.allele is None else int(d.allele)
                check(lib().pg_engine_add_driver_sid(self._h, mut_id, chr_idx, int(d.chr_pos), ref.encode(),
                                                     d.alt.encode(), al))
            elif isinstance(d, CNA):
                al = -1 if d.allele is None else int(d.allele)
                src = -1 if d.src_allele is None else int(d.src_allele)
                check(lib().pg_engine_add_driver_cna(self._h, mut_id, 1 if d.type == "A" else 0,
                                                     self._chr_index(d.chr), int(d.chr_pos), int(d.len), al, src))
            elif d is WGD:
                check(lib().pg_engine_add_driver_wgd(self._h, mut_id))
            else:
                raise DomainError(_lib.PG_ERR_DOMAIN, "unsupported driver mutation specification")
        self._mutant_specs.append((mutant_name, passenger_rates, drivers))

    def get_species_rates(self) -> dict:
        rows = list(self.species_rates.items())
        return {"mutant": np.array([k[0] for k, _ in rows], dtype=object),
                "epistate": np.array([k[1] for k, _ in rows], dtype=object),
                "SNV": np.array([np.atleast_1d(v["SNV"])[0] for _, v in rows], dtype=float),
                "indel": np.array([np.atleast_1d(v["indel"])[0] for _, v in rows], dtype=float),
                "CNA": np.array([v["CNA"] for _, v in rows], dtype=float)}

    @property
    def infinite_sites_model(self) -> bool:
        on = C.c_int(0)
        check(lib().pg_engine_get_infinite_sites(self._h, C.byref(on)))
        return bool(on.value)

    @infinite_sites_model.setter
    def infinite_sites_model(self, value: bool) -> None:
        check(lib().pg_engine_set_infinite_sites(self._h, 1 if value else 0))

    # -- genome helpers ----------------------------------------------------------------
    def _chr_index(self, name) -> int:
        name = str(name)
        if name not in self.chr_names:
            raise DomainError(_lib.PG_ERR_DOMAIN, f"unknown chromosome {name}")
        return self.chr_names.index(name)

    def gather_bases(self, positions: np.ndarray) -> np.ndarray:
        pos = np.ascontiguousarray(positions, dtype=np.uint32)
        out = np.empty(pos.size, dtype=np.uint8)
        if pos.size:
            check(lib().pg_engine_gather_bases(self._h, pos.size, ptr(pos, C.c_uint32), ptr(out, C.c_uint8)))
        return out

    def get_bases(self, chr_idx: int, chr_pos: int, n: int) -> str:
        start = int(self.chr_off[chr_idx]) + chr_pos - 1
        return "".join(BASES[self.gather_bases(np.arange(start, start + n, dtype=np.uint32))])

    def read_genome(self, start: int = 0, n: int | None = None) -> np.ndarray:
        n = self.genome.total - start if n is None else n
        out = np.empty(n, dtype=np.uint8)
        check(lib().pg_engine_read_genome(self._h, start, n, ptr(out, C.c_uint8)))
        return out

    def index_info(self) -> dict:
        G = C.c_uint64()
        ct, it = np.zeros(32, np.uint64), np.zeros(83, np.uint64)
        cs, is_ = np.zeros(32, np.uint32), np.zeros(83, np.uint32)
        check(lib().pg_engine_genome_info(self._h, C.byref(G), ptr(ct, C.c_uint64), ptr(it, C.c_uint64),
                                          ptr(cs, C.c_uint32), ptr(is_, C.c_uint32)))
        return {"length": G.value, "ctx_total": ct, "id_total": it, "ctx_stored": cs, "id_stored": is_}

    def read_index(self, which: int, cls: int) -> np.ndarray:
        n = C.c_uint32()
        check(lib().pg_engine_read_index(self._h, which, cls, None, 0, C.byref(n)))
        out = np.empty(n.value, dtype=np.uint32)
        check(lib().pg_engine_read_index(self._h, which, cls, ptr(out, C.c_uint32), n.value, C.byref(n)))
        return out

    def get_genome_info(self) -> dict:
        return {"chr": np.array(self.chr_names, dtype=object), "length": self.chr_lengths.astype(np.int64)}

    # -- placement ------------------------------------------------------------------
    def forest_species(self, forest: SamplesForest) -> np.ndarray:
        """Species id of every node: its (mutant, epistate), else the mutant's
        epistate-free species."""
        names, code = forest.species_codes()
        ids = np.empty(len(names), dtype=np.uint32)
        for k, (m, e) in enumerate(names):
            key = (m, e) if (m, e) in self.species else (m, "")
            if key not in self.species:
                raise DomainError(_lib.PG_ERR_DOMAIN, f'unknown species "{m}{e}": add its mutant first')
            ids[k] = self.species[key]
        return ids[code]

    def place_mutations(self, samples_forest: SamplesForest, num_of_preneoplatic_SNVs: int = 0,
                        num_of_preneoplatic_indels: int = 0, seed=None,
                        preneoplatic_SNV_signature_name: str = "SBS1",
                        preneoplatic_indel_signature_name: str = "ID1") -> "PhylogeneticForest":
        """``place_mutations(samples_forest, #preneoplastic SNVs, #preneoplastic indels, seed)``."""
        f = samples_forest
        species = self.forest_species(f)

        def sig_index(ty, name, count):
            if count == 0:
                return 0
            if name not in self.sig_names[ty]:
                raise DomainError(_lib.PG_ERR_DOMAIN, f"Unknown signature {name}")
            return self.sig_names[ty].index(name)

        pre_s = sig_index(0, preneoplatic_SNV_signature_name, num_of_preneoplatic_SNVs)
        pre_i = sig_index(1, preneoplatic_indel_signature_name, num_of_preneoplatic_indels)
        fh = C.c_void_p()
        parent = np.ascontiguousarray(f.parent, dtype=np.int32)
        birth = np.ascontiguousarray(f.birth_time, dtype=np.float64)
        sample = np.ascontiguousarray(np.where(f.is_leaf, f.sample, -1), dtype=np.int32)
        div = np.ascontiguousarray(f.divisions, dtype=np.uint32)
        check(lib().pg_forest_create(f.num_of_nodes, ptr(parent, C.c_int32), ptr(birth, C.c_double),
                                     ptr(species, C.c_uint32), ptr(sample, C.c_int32), ptr(div, C.c_uint32),
                                     len(f.sample_names), C.byref(fh)))
        try:
            ph = C.c_void_p()
            s = _seed(seed)
            check(lib().pg_place_mutations(self._h, fh, int(num_of_preneoplatic_SNVs), pre_s,
                                           int(num_of_preneoplatic_indels), pre_i, s, C.byref(ph)))
        finally:
            lib().pg_forest_destroy(fh)
        pf = PhylogeneticForest(self, f, ph, s)
        pf._place_args = dict(num_of_preneoplatic_SNVs=int(num_of_preneoplatic_SNVs),
                              num_of_preneoplatic_indels=int(num_of_preneoplatic_indels), seed=s,
                              preneoplatic_SNV_signature_name=preneoplatic_SNV_signature_name,
                              preneoplatic_indel_signature_name=preneoplatic_indel_signature_name)
        return pf


class PhylogeneticForest:
    """Placement result: the samples forest plus the placed mutations (kept in
    HBM, sorted by locus) and the getters of src/phylogenetic_forest.cpp."""

    def __init__(self, engine: MutationEngine, forest: SamplesForest, handle: C.c_void_p, seed: int):
        self.engine = engine
        self.forest = forest
        self._h = handle
        self.seed = seed
        self._table = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _lib._LIB is not None:
            _lib._LIB.pg_placed_destroy(h)
            self._h = None

    @property
    def num_of_mutations(self) -> int:
        n = C.c_uint64()
        check(lib().pg_placed_count(self._h, C.byref(n)))
        return n.value

    def kernel_ms(self) -> float:
        v = C.c_float()
        check(lib().pg_placed_kernel_ms(self._h, C.byref(v)))
        return v.value

    def table(self) -> dict:
        """Placed mutations as arrays (sorted by absolute locus)."""
        if self._table is None:
            n = self.num_of_mutations
            t = {k: np.empty(n, dtype=np.uint32) for k in ("locus", "edge", "aux")}
            t.update({k: np.empty(n, dtype=np.uint8) for k in ("cls", "sig", "kind", "nature")})
            t["allele"] = np.empty(n, dtype=np.uint16)
            check(lib().pg_placed_copy(self._h, *(ptr(t[k], C.c_uint32) for k in ("locus", "edge", "aux")),
                                       ptr(t["cls"], C.c_uint8), ptr(t["sig"], C.c_uint8),
                                       ptr(t["allele"], C.c_uint16), ptr(t["kind"], C.c_uint8),
                                       ptr(t["nature"], C.c_uint8)))
            self._table = t
        return self._table

    # -- reference-facing getters ------------------------------------------------------
    def get_nodes(self) -> dict:
        return self.forest.get_nodes()

    def _ref_alt(self, t: dict, rows: np.ndarray | None = None) -> tuple[np.ndarray, np.ndarray]:
        """ref / alt strings of the rows (all when None): one base gather for
        the SNVs and one for the indels' anchor windows."""
        eng = self.engine
        rows = np.arange(len(t["locus"])) if rows is None else np.asarray(rows, dtype=np.int64)
        n = len(rows)
        kind, aux = t["kind"][rows], t["aux"][rows].astype(np.int64)
        locus = t["locus"][rows].astype(np.int64)
        ref = np.empty(n, dtype=object)
        alt = np.empty(n, dtype=object)
        snv = kind == 0
        rb = eng.gather_bases(locus[snv])
        ref[snv] = BASES[np.minimum(rb, 4)]
        alt[snv] = BASES[aux[snv] & 3]
        ind = np.nonzero(~snv)[0]
        if len(ind):
            a = aux[ind]
            ins, ln, bases = (a & 1).astype(bool), (a >> 1) & 7, a >> 8
            # the anchor and the 7 bases after it (a deletion spans at most 7)
            win = np.minimum(locus[ind][:, None] + np.arange(8)[None, :], eng.genome.total - 1)
            gch = BASES[np.minimum(eng.gather_bases(win.ravel()).reshape(-1, 8), 4)]
            added = BASES[(bases[:, None] >> (2 * np.arange(7))[None, :]) & 3]
            for length in np.unique(ln):
                L = int(length)
                # insertion: ref = anchor, alt = anchor + L inserted bases
                sel = np.nonzero(ins & (ln == L))[0]
                if len(sel):
                    ref[ind[sel]] = gch[sel, 0]
                    chars = np.ascontiguousarray(np.concatenate([gch[sel, :1], added[sel, :L]], axis=1))
                    alt[ind[sel]] = chars.view(f"<U{L + 1}").ravel()
                # deletion: ref = anchor + L deleted bases, alt = anchor
                sel = np.nonzero(~ins & (ln == L))[0]
                if len(sel):
                    ref[ind[sel]] = np.ascontiguousarray(gch[sel, :L + 1]).view(f"<U{L + 1}").ravel()
                    alt[ind[sel]] = gch[sel, 0]
        return ref, alt

    def _cause(self, t: dict, rows: np.ndarray | None = None) -> np.ndarray:
        """Signature name of each row (None for drivers and unknown indices)."""
        rows = np.arange(len(t["sig"])) if rows is None else np.asarray(rows, dtype=np.int64)
        sig, kind = t["sig"][rows].astype(np.int64), t["kind"][rows]
        out = np.full(len(rows), None, dtype=object)
        for k in np.unique(kind):
            names = list(self.engine.sig_names[int(k)]) if int(k) < len(self.engine.sig_names) else []
            table = np.array(names + [None], dtype=object)
            m = kind == k
            sk = sig[m]
            out[m] = table[np.where((sk == 0xFF) | (sk >= len(names)), len(names), sk)]
        return out

    def _chr_pos(self, locus: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
        off = self.engine.chr_off
        ci = np.searchsorted(off, locus.astype(np.uint64), side="right") - 1
        names = np.array(self.engine.chr_names, dtype=object)[ci]
        return names, (locus.astype(np.int64) - off[ci].astype(np.int64) + 1)

    def leaf_carriers(self, leaf: int) -> np.ndarray:
        """Mask of the placed mutations on the root path of node ``leaf``
        (their edge an ancestor-or-self of it) and the preneoplastic ones."""
        f = self.forest
        tin, tout = f.euler()
        e = self.table()["edge"].astype(np.int64)
        n = f.num_of_nodes
        inner = e < n
        ec = np.minimum(e, n - 1)
        x = tin[int(leaf)]
        return ~inner | ((tin[ec] <= x) & (x < tout[ec]))

    def _lineage(self) -> dict:
        """Instance lineage chains and every mutation's order key
        (pg_placed_lineage_copy)."""
        if getattr(self, "_lin_cache", None) is None:
            ni, nl = C.c_uint32(), C.c_uint32()
            check(lib().pg_placed_lineage_dims(self._h, C.byref(ni), C.byref(nl)))
            d = {"off": np.zeros(ni.value + 1, np.uint32), "anc": np.zeros(max(nl.value, 1), np.uint16),
                 "key": np.zeros(max(nl.value, 1), np.uint64),
                 "order": np.zeros(max(self.num_of_mutations, 1), np.uint64)}
            check(lib().pg_placed_lineage_copy(self._h, ptr(d["off"], C.c_uint32), ptr(d["anc"], C.c_uint16),
                                               ptr(d["key"], C.c_uint64), ptr(d["order"], C.c_uint64)))
            d["n_instances"] = ni.value
            self._lin_cache = d
        return self._lin_cache

    def _cell_rows(self, leaf: int) -> tuple[np.ndarray, np.ndarray]:
        """(mutation rows, allele instance) of the mutations sampled cell
        ``leaf`` holds: those on its root path, once per allele instance of
        its genome at the locus that carries them (the placed instance, and
        the copies of it made after the mutation), in mutation order."""
        t = self.table()
        idx = np.nonzero(self.leaf_carriers(leaf))[0]
        lin = self._lineage()
        cls, n_classes, _ = self.node_classes()
        if n_classes <= 1 and lin["n_instances"] <= 2:       # no copy-number event
            return idx, t["allele"][idx].astype(np.int64)
        d = self._classes()
        c = int(cls[leaf])
        lo, hi = int(d["seg_off"][c]), int(d["seg_off"][c + 1])
        st, en = d["start"][lo:hi].astype(np.int64), d["end"][lo:hi].astype(np.int64)
        loc = t["locus"][idx].astype(np.int64)
        k = np.searchsorted(st, loc, side="right") - 1
        inside = (k >= 0) & (loc < en[np.maximum(k, 0)]) if hi > lo else np.zeros(len(idx), bool)
        ks = np.maximum(k, 0)
        ioff = d["ioff"][lo:hi][ks].astype(np.int64) if hi > lo else np.zeros(len(idx), np.int64)
        icnt = np.where(inside, d["icnt"][lo:hi][ks], 0).astype(np.int64) if hi > lo else np.zeros(len(idx), np.int64)
        x = t["allele"][idx].astype(np.int64)
        km = lin["order"][idx]
        coff = lin["off"].astype(np.int64)
        rows, alle, slot = [], [], []
        for j in range(int(icnt.max()) if len(icnt) else 0):
            sel = np.nonzero(j < icnt)[0]
            y = d["list"][ioff[sel] + j].astype(np.int64)
            carry = y == x[sel]
            # y's lineage: x in its chain with a copy key above the mutation's
            b, ln = coff[y], coff[y + 1] - coff[y]
            found = carry.copy()
            for dep in range(int(ln.max()) if len(ln) else 0):
                act = ~found & (dep < ln)
                a = np.where(act, lin["anc"][np.where(act, b + dep, 0)].astype(np.int64), -1)
                hit = act & (a == x[sel])
                carry |= hit & (lin["key"][np.where(hit, b + dep, 0)] > km[sel])
                found |= hit
            rows.append(idx[sel][carry]); alle.append(y[carry]); slot.append(np.full(int(carry.sum()), j))
        if not rows:
            return idx[:0], idx[:0].astype(np.int64)
        r, a, s_ = np.concatenate(rows), np.concatenate(alle), np.concatenate(slot)
        o = np.lexsort((s_, r))
        return r[o], a[o]

    def get_sampled_cell_mutations(self, cell_id=None) -> dict:
        """Columns cell_id, chr, chr_pos, allele, ref, alt, type, cause, class
        (src/phylogenetic_forest.cpp:452-507): every mutation a sampled cell
        holds, once per allele instance of its genome carrying it (an SID is
        copied with its allele by an amplification or a WGD after it, and
        leaves with a deleted allele); ``allele`` is the instance."""
        f = self.forest
        t = self.table()
        leaves = np.nonzero(f.is_leaf & (f.sample >= 0))[0]
        if cell_id is not None:
            hit = np.nonzero(f.cell_id == int(cell_id))[0]
            if len(hit) == 0 or not f.is_leaf[hit[0]]:
                raise DomainError(_lib.PG_ERR_DOMAIN, f'Cell "{cell_id}" is not a leaf')
            leaves = hit
        per = [self._cell_rows(int(lf)) for lf in leaves]
        rows = np.concatenate([r for r, _ in per]) if per else np.zeros(0, np.int64)
        alle = np.concatenate([a for _, a in per]) if per else np.zeros(0, np.int64)
        cell = np.concatenate([np.full(len(r), f.cell_id[lf]) for lf, (r, _) in zip(leaves, per)]) if per else rows
        ref, alt = self._ref_alt(t, rows)
        chrn, pos = self._chr_pos(t["locus"][rows])
        return {"cell_id": cell, "chr": chrn, "chr_pos": pos, "allele": alle.astype(np.int64), "ref": ref, "alt": alt,
                "type": np.where(t["kind"][rows] == 0, "SNV", "indel"), "cause": self._cause(t, rows),
                "class": NATURES[t["nature"][rows]]}

    def cna_table(self) -> dict:
        """Applied CNA / WGD events: node, type (0 deletion, 1 amplification,
        2 WGD), chr index, 1-based begin/end, allele instance, source instance,
        driver flag."""
        n = C.c_uint64()
        check(lib().pg_placed_cna_count(self._h, C.byref(n)))
        m = n.value
        t = {k: np.empty(m, dtype=np.uint32) for k in ("node", "chr", "begin", "end", "allele", "src")}
        t.update({k: np.empty(m, dtype=np.uint8) for k in ("type", "driver")})
        check(lib().pg_placed_cna_copy(self._h, ptr(t["node"], C.c_uint32), ptr(t["type"], C.c_uint8),
                                       ptr(t["chr"], C.c_uint32), ptr(t["begin"], C.c_uint32),
                                       ptr(t["end"], C.c_uint32), ptr(t["allele"], C.c_uint32),
                                       ptr(t["src"], C.c_uint32), ptr(t["driver"], C.c_uint8)))
        return t

    def node_classes(self) -> tuple[np.ndarray, int, int]:
        """Genotype class of every node, the number of classes and the largest copy number."""
        f = self.forest
        out = np.empty(f.num_of_nodes, dtype=np.uint32)
        nc, cm = C.c_uint32(), C.c_uint32()
        check(lib().pg_placed_node_classes(self._h, ptr(out, C.c_uint32), C.byref(nc), C.byref(cm)))
        return out, nc.value, cm.value

    def get_sampled_cell_CNAs(self, cell_id=None) -> dict:
        """Columns cell_id, type ("A", "D"; "WGD" for a whole-genome doubling,
        whose chr/begin/end are empty), chr, begin, end, allele, src allele
        (NA, i.e. -1, for deletions) and class (src/phylogenetic_forest.cpp:509-562)."""
        f = self.forest
        c = self.cna_table()
        leaves = np.nonzero(f.is_leaf & (f.sample >= 0))[0]
        if cell_id is not None:
            hit = np.nonzero(f.cell_id == int(cell_id))[0]
            if len(hit) == 0 or not f.is_leaf[hit[0]]:
                raise DomainError(_lib.PG_ERR_DOMAIN, f'Cell "{cell_id}" is not a leaf')
            leaves = hit
        names = np.array(self.engine.chr_names + [""], dtype=object)
        tname = np.array(["D", "A", "WGD"], dtype=object)
        cols = {k: [] for k in ("cell_id", "type", "chr", "begin", "end", "allele", "src allele", "class")}
        for lf in leaves:
            path = set()
            v = int(lf)
            while v >= 0:
                path.add(v)
                v = int(f.parent[v])
            m = np.isin(c["node"], np.fromiter(path, dtype=np.int64))
            wgd = c["type"][m] == 2
            cols["cell_id"].append(np.full(m.sum(), f.cell_id[lf]))
            cols["type"].append(tname[c["type"][m]])
            cols["chr"].append(names[np.where(wgd, len(names) - 1, c["chr"][m])])
            cols["begin"].append(np.where(wgd, -1, c["begin"][m].astype(np.int64)))
            cols["end"].append(np.where(wgd, -1, c["end"][m].astype(np.int64)))
            cols["allele"].append(np.where(wgd, -1, c["allele"][m].astype(np.int64)))
            cols["src allele"].append(np.where(c["type"][m] == 1, c["src"][m].astype(np.int64), -1))
            cols["class"].append(np.where(c["driver"][m] == 1, "driver", "passenger"))
        return {k: (np.concatenate(v) if v else np.array([])) for k, v in cols.items()}

    # -- copy-number getters (allelic fragmentation) ------------------------------------
    def _classes(self) -> dict:
        """Genotype classes as segments with each instance's germline allele."""
        if getattr(self, "_cls_cache", None) is None:
            nc, ns, nl, ni = (C.c_uint32() for _ in range(4))
            check(lib().pg_placed_class_dims(self._h, C.byref(nc), C.byref(ns), C.byref(nl), C.byref(ni)))
            d = {"seg_off": np.empty(nc.value + 1, np.uint32), "start": np.empty(ns.value, np.uint32),
                 "end": np.empty(ns.value, np.uint32), "ioff": np.empty(ns.value, np.uint32),
                 "icnt": np.empty(ns.value, np.uint32), "list": np.empty(max(nl.value, 1), np.uint16),
                 "root": np.empty(max(ni.value, 1), np.uint8)}
            check(lib().pg_placed_class_copy(self._h, ptr(d["seg_off"], C.c_uint32), ptr(d["start"], C.c_uint32),
                                             ptr(d["end"], C.c_uint32), ptr(d["ioff"], C.c_uint32),
                                             ptr(d["icnt"], C.c_uint32), ptr(d["list"], C.c_uint16),
                                             ptr(d["root"], C.c_uint8)))
            # copies of germline allele 1 per segment (the rest descend from allele 0)
            roots = d["root"][d["list"][:max(nl.value, 1)]].astype(np.int64)
            csum = np.concatenate([[0], np.cumsum(roots)])
            d["a1"] = (csum[d["ioff"] + d["icnt"]] - csum[d["ioff"]]).astype(np.int64)
            d["a0"] = d["icnt"].astype(np.int64) - d["a1"]
            d["n_classes"] = nc.value
            self._cls_cache = d
        return self._cls_cache

    def _class_fragments(self, c: int) -> tuple[np.ndarray, np.ndarray, np.ndarray, np.ndarray]:
        """(absolute begin, end (half-open), copies of allele 0, of allele 1) of
        the maximal stretches of class c with one allelic type, chromosome by
        chromosome (uncovered stretches have type (0, 0))."""
        d = self._classes()
        lo, hi = int(d["seg_off"][c]), int(d["seg_off"][c + 1])
        st, en = d["start"][lo:hi].astype(np.int64), d["end"][lo:hi].astype(np.int64)
        off = self.engine.chr_off.astype(np.int64)
        cuts = np.unique(np.concatenate([off, st, en]))
        b, e = cuts[:-1], cuts[1:]
        k = np.searchsorted(st, b, side="right") - 1
        inside = (k >= 0) & (b < en[np.maximum(k, 0)])
        a0 = np.where(inside, d["a0"][lo:hi][np.maximum(k, 0)] if hi > lo else 0, 0)
        a1 = np.where(inside, d["a1"][lo:hi][np.maximum(k, 0)] if hi > lo else 0, 0)
        chrom = np.searchsorted(off, b, side="right") - 1
        new = np.r_[True, (chrom[1:] != chrom[:-1]) | (a0[1:] != a0[:-1]) | (a1[1:] != a1[:-1])]
        first = np.nonzero(new)[0]
        last = np.r_[first[1:], len(b)] - 1
        return b[first], e[last], a0[first], a1[first]

    def _frag_rows(self, b, e, a0, a1):
        off = self.engine.chr_off.astype(np.int64)
        ci = np.searchsorted(off, b, side="right") - 1
        names = np.array(self.engine.chr_names, dtype=object)[ci]
        return names, b - off[ci] + 1, e - off[ci], np.maximum(a0, a1), np.minimum(a0, a1)

    def get_cell_allelic_fragmentation(self) -> dict:
        """Columns cell_id, chr, begin, end, major, minor: every sampled cell's
        genome cut into stretches of one allelic type (copies of the two
        germline alleles; major = the larger), src/phylogenetic_forest.cpp:867-927."""
        f = self.forest
        cls, _, _ = self.node_classes()
        leaves = np.nonzero(f.is_leaf & (f.sample >= 0))[0]
        per = {}
        cols = {k: [] for k in ("cell_id", "chr", "begin", "end", "major", "minor")}
        for lf in leaves:
            c = int(cls[lf])
            if c not in per:
                per[c] = self._frag_rows(*self._class_fragments(c))
            names, b, e, mj, mn = per[c]
            cols["cell_id"].append(np.full(len(b), f.cell_id[lf]))
            cols["chr"].append(names); cols["begin"].append(b); cols["end"].append(e)
            cols["major"].append(mj); cols["minor"].append(mn)
        return {k: (np.concatenate(v) if v else np.array([])) for k, v in cols.items()}

    def get_bulk_allelic_fragmentation(self, sample_name: str | None = None) -> dict:
        """Columns chr, begin, end, major, minor, ratio: for every stretch of
        the genome on which the sampled cells (of one sample, or all) keep
        their allelic types, each type with the fraction of cells showing it
        (src/phylogenetic_forest.cpp:767-820)."""
        f = self.forest
        cls, _, _ = self.node_classes()
        sel = f.is_leaf & (f.sample >= 0)
        if sample_name is not None:
            if sample_name not in f.sample_names:
                raise DomainError(_lib.PG_ERR_DOMAIN, f'Unknown sample "{sample_name}".')
            sel &= f.sample == f.sample_names.index(sample_name)
        leaf_cls, counts = np.unique(cls[sel], return_counts=True)
        n_cells = float(counts.sum())
        frags = [self._class_fragments(int(c)) for c in leaf_cls]
        cuts = np.unique(np.concatenate([fr[0] for fr in frags] + [fr[1] for fr in frags]))
        b, e = cuts[:-1], cuts[1:]
        keep = np.ones(len(b), dtype=bool)
        types = []
        for (fb, fe, f0, f1) in frags:
            k = np.searchsorted(fb, b, side="right") - 1
            types.append((f0[k], f1[k]))
        # merge neighbouring stretches with the same type in every class and chromosome
        off = self.engine.chr_off.astype(np.int64)
        chrom = np.searchsorted(off, b, side="right") - 1
        same = np.ones(len(b) - 1, dtype=bool) if len(b) > 1 else np.zeros(0, dtype=bool)
        for t0, t1 in types:
            same &= (t0[1:] == t0[:-1]) & (t1[1:] == t1[:-1])
        same &= chrom[1:] == chrom[:-1]
        start = np.r_[True, ~same]
        first = np.nonzero(start)[0]
        last = np.r_[first[1:], len(b)] - 1
        cols = {k: [] for k in ("chr", "begin", "end", "major", "minor", "ratio")}
        for i0, i1 in zip(first, last):
            agg = {}
            for (t0, t1), n in zip(types, counts):
                key = (int(t0[i0]), int(t1[i0]))
                agg[key] = agg.get(key, 0) + int(n)
            names, bb, ee, _, _ = self._frag_rows(np.array([b[i0]]), np.array([e[i1]]), np.zeros(1), np.zeros(1))
            for (x0, x1), n in sorted(agg.items()):
                cols["chr"].append(names[0]); cols["begin"].append(int(bb[0])); cols["end"].append(int(ee[0]))
                cols["major"].append(max(x0, x1)); cols["minor"].append(min(x0, x1)); cols["ratio"].append(n / n_cells)
        return {k: np.array(v, dtype=object if k == "chr" else None) for k, v in cols.items()}

    def get_samples_info(self) -> dict:
        """name, tumour_cells, DNA_quantity, equivalent_normal_cells
        (src/phylogenetic_forest.cpp:57-99): the DNA of a sample is the summed
        allelic size of its sampled cells' genomes."""
        info = self.forest.get_samples_info()
        normal_dna = 2.0 * self.engine.genome.total
        f = self.forest
        d = self._classes()
        size = np.zeros(d["n_classes"], dtype=np.float64)
        seg_cls = np.repeat(np.arange(d["n_classes"]), np.diff(d["seg_off"].astype(np.int64)))
        np.add.at(size, seg_cls, (d["end"].astype(np.float64) - d["start"]) * d["icnt"])
        cls, _, _ = self.node_classes()
        dna = np.zeros(len(info["name"]), dtype=np.float64)
        for i, name in enumerate(info["name"]):
            j = f.sample_names.index(name)
            dna[i] = size[cls[f.is_leaf & (f.sample == j)]].sum()
        info["DNA_quantity"] = dna
        info["equivalent_normal_cells"] = dna / normal_dna
        return info

    def save(self, filename: str, quiet: bool = False) -> None:
        """``PhylogeneticForest$save(filename, quiet)``; see :func:`save_phylogenetic_forest`."""
        save_phylogenetic_forest(self, filename)

    def get_germline_mutations(self) -> dict:
        return {k: np.array([]) for k in ("chr", "chr_pos", "allele", "ref", "alt", "type", "cause", "class")}

    def get_species_info(self) -> dict:
        """The registered species (src/phylogenetic_forest.cpp:220-255):
        mutant, epistate, SNV_rate, indel_rate and CNA_rate."""
        r = self.engine.get_species_rates()
        return {"mutant": r["mutant"], "epistate": r["epistate"], "SNV_rate": r["SNV"], "indel_rate": r["indel"],
                "CNA_rate": r["CNA"]}

    def get_reference_path(self) -> str:
        """The reference genome path recorded with the forest (the FASTA the
        engine was built from, when it was)."""
        return getattr(self, "_reference_path", "")

    def set_reference_path(self, path: str) -> None:
        self._reference_path = str(path)

    def get_driver_mutations(self) -> dict:
        """The declared driver mutations (src/phylogenetic_forest.cpp:172-218):
        per mutant, in name order, its drivers in application order, with
        the columns mutant, order, type ("SID", "CNA" or "WGD"), CNA_type
        ("A" or "D"), chr, start, end, ref, alt, allele and src_allele (None
        where the reference reports NA)."""
        eng = self.engine
        specs = {}
        for name, _, drivers in eng._mutant_specs:
            specs[name] = list(drivers)
        cols = {k: [] for k in ("mutant", "order", "type", "CNA_type", "chr", "start", "end", "ref", "alt",
                                "allele", "src_allele")}

        def row(**kw):
            for k in cols:
                cols[k].append(kw.get(k))

        for name in sorted(specs):
            for k, d in enumerate(specs[name]):
                if d is WGD:
                    row(mutant=name, order=k, type="WGD")
                elif isinstance(d, CNA):
                    row(mutant=name, order=k, type="CNA", CNA_type=d.type, chr=str(d.chr), start=int(d.chr_pos),
                        end=int(d.chr_pos) + int(d.len) - 1, allele=d.allele,
                        src_allele=d.src_allele if d.type == "A" else None)
                else:
                    ref = d.ref
                    if "?" in ref:
                        ref = eng.get_bases(eng._chr_index(d.chr), int(d.chr_pos), max(1, len(ref)))
                    row(mutant=name, order=k, type="SID", chr=str(d.chr), start=int(d.chr_pos),
                        end=int(d.chr_pos) + len(ref) - 1, ref=ref, alt=d.alt, allele=d.allele)
        return {k: np.array(v, dtype=object) for k, v in cols.items()}

    def get_exposures(self) -> dict:
        """The timed exposures (src/phylogenetic_forest.cpp:644-668): time,
        signature, exposure and type, the SNV (SBS) rows then the indel (ID)
        rows, each by time and signature name."""
        eng = self.engine
        timed: list[dict] = [{}, {}]
        for t, coef in eng._exposures:
            for ty in (0, 1):
                part = {k: float(v) for k, v in coef.items() if k in eng.sig_names[ty]}
                if part:
                    timed[ty][float(t)] = part
        cols = {k: [] for k in ("time", "signature", "exposure", "type")}
        for ty, tname in ((0, "SNV"), (1, "indel")):
            for t in sorted(timed[ty]):
                for sig in sorted(timed[ty][t]):
                    cols["time"].append(t)
                    cols["signature"].append(sig)
                    cols["exposure"].append(timed[ty][t][sig])
                    cols["type"].append(tname)
        return {"time": np.array(cols["time"], dtype=np.float64), "signature": np.array(cols["signature"], dtype=object),
                "exposure": np.array(cols["exposure"], dtype=np.float64), "type": np.array(cols["type"], dtype=object)}

    def get_first_occurrences(self, mutation) -> list:
        """The identifiers of the cells in which a mutation (an SNV/indel
        ``Mutation`` or a ``CNA``) first occurs (src/phylogenetic_forest.cpp:565-622):
        the cells at the ends of the edges it was placed on (the forest's
        first cells for a preneoplastic mutation), ascending."""
        f = self.forest
        eng = self.engine
        roots = np.nonzero(f.parent < 0)[0]
        if isinstance(mutation, CNA):
            c = self.cna_table()
            ci = eng._chr_index(mutation.chr)
            typ = 1 if mutation.type == "A" else 0
            hit = ((c["type"] == typ) & (c["chr"] == ci) & (c["begin"] == int(mutation.chr_pos)) &
                   (c["end"] == int(mutation.chr_pos) + int(mutation.len) - 1))
            nodes = c["node"][hit].astype(np.int64)
        elif isinstance(mutation, Mutation):
            t = self.table()
            ci = eng._chr_index(mutation.chr)
            locus = int(eng.chr_off[ci]) + int(mutation.chr_pos) - 1
            cand = np.nonzero(t["locus"].astype(np.int64) == locus)[0]
            ref, alt = self._ref_alt(t, cand) if len(cand) else (np.array([]), np.array([]))
            want_ref = None if "?" in mutation.ref else mutation.ref
            keep = [i for j, i in enumerate(cand)
                    if alt[j] == mutation.alt and (want_ref is None or ref[j] == want_ref)]
            nodes = t["edge"][keep].astype(np.int64) if keep else np.zeros(0, dtype=np.int64)
        else:
            raise DomainError(_lib.PG_ERR_DOMAIN, "This methods exclusively accepts as the parameters "
                                                  "SNV, Indel, or CNA objects.")
        if len(nodes) == 0:
            raise DomainError(_lib.PG_ERR_DOMAIN, f"The mutation {mutation} does not occurs in the sampled cells.")
        cells = set()
        for v in nodes:
            cells.update(int(x) for x in (f.cell_id[roots] if v >= f.num_of_nodes else [f.cell_id[v]]))
        return sorted(cells)


# ---------------------------------------------------------------- save / load
FOREST_FORMAT = "process_gb300.phylogenetic_forest"
FOREST_VERSION = 1


def _plain(x):
    """JSON-ready copy of rates, exposures and driver specifications."""
    if isinstance(x, dict):
        return {str(k): _plain(v) for k, v in x.items()}
    if isinstance(x, (list, tuple)):
        return [_plain(v) for v in x]
    if isinstance(x, np.ndarray):
        return x.tolist()
    if isinstance(x, np.generic):
        return x.item()
    if isinstance(x, Mutation):
        return {"kind": "SID", "chr": x.chr, "chr_pos": int(x.chr_pos), "ref": x.ref, "alt": x.alt,
                "allele": x.allele}
    if isinstance(x, CNA):
        return {"kind": "CNA", "type": x.type, "chr": x.chr, "chr_pos": int(x.chr_pos), "len": int(x.len),
                "allele": x.allele, "src_allele": x.src_allele}
    if x is WGD:
        return {"kind": "WGD"}
    return x


def _driver(d):
    if d["kind"] == "SID":
        return Mutation(d["chr"], d["chr_pos"], d["ref"], d["alt"], d["allele"])
    if d["kind"] == "CNA":
        return CNA(d["type"], d["chr"], d["chr_pos"], d["len"], d["allele"], d["src_allele"])
    return WGD


def _table_digest(t: dict) -> str:
    import hashlib
    h = hashlib.sha256()
    for k in ("locus", "edge", "aux", "cls", "sig", "allele", "kind", "nature"):
        h.update(np.ascontiguousarray(t[k]).tobytes())
    return h.hexdigest()


def save_phylogenetic_forest(pf: "PhylogeneticForest", filename: str) -> None:
    """``PhylogeneticForest$save`` (src/phylogenetic_forest.cpp:940-955).  The
    RACES binary archive layout is unavailable, so the file is a versioned
    native archive (numpy .npz): the engine's configuration, the samples
    forest, the placement call and a digest of the placed mutations.  Loading
    places again (placement is a function of these inputs) and checks the
    digest."""
    import json
    e, f = pf.engine, pf.forest
    args = getattr(pf, "_place_args", None)
    if args is None:
        raise DomainError(_lib.PG_ERR_DOMAIN, "this phylogenetic forest was not made by place_mutations")
    meta = {
        "format": FOREST_FORMAT, "version": FOREST_VERSION,
        "genome": {"chr_names": list(e.chr_names), "chr_lengths": [int(x) for x in e.chr_lengths],
                   "seed": int(e.genome.seed), "gc": float(e.genome.gc), "bases": e.genome.bases is not None},
        "engine": {"context_sampling": e.context_sampling, "max_motif_size": e.max_motif_size,
                   "max_repetition_storage": e.max_repetition_storage,
                   "avoid_homozygous_losses": e.avoid_homozygous_losses,
                   "infinite_sites_model": e.infinite_sites_model,
                   "SBS_signatures": _plain(e._sigs[0]), "indel_signatures": _plain(e._sigs[1]),
                   "exposures": _plain(e._exposures), "mutants": _plain(e._mutant_specs),
                   "passenger_CNAs": _plain(e.passenger_CNAs)},
        "place": _plain(args),
        "digest": _table_digest(pf.table()),
    }
    ancestor = np.where(f.parent >= 0, f.cell_id[np.maximum(f.parent, 0)], -1)
    sample = np.array([f.sample_names[s] if s >= 0 else "" for s in f.sample], dtype=object)
    arrays = {"meta": np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8),
              "cell_id": f.cell_id, "ancestor": ancestor, "mutant": f.mutant.astype(str),
              "epistate": np.array(["" if x is None else str(x) for x in f.epistate]),
              "sample": sample.astype(str), "birth_time": f.birth_time, "divisions": f.divisions}
    if e.genome.bases is not None:
        arrays["bases"] = np.asarray(e.genome.bases, dtype=np.uint8)
    with open(filename, "wb") as fh:
        np.savez_compressed(fh, **arrays)


def load_phylogenetic_forest(filename: str, quiet: bool = False) -> "PhylogeneticForest":
    """``load_phylogenetic_forest(filename, quiet)`` (src/mutations.cpp:1466-1480):
    rebuilds the engine and the samples forest of a saved file, places the
    mutations again and checks them against the saved digest."""
    import json
    import os
    if not os.path.exists(filename):
        raise DomainError(_lib.PG_ERR_DOMAIN, f'The file "{filename}" does not exist.')
    if not os.path.isfile(filename):
        raise DomainError(_lib.PG_ERR_DOMAIN, f'The file "{filename}" is not a regular file.')
    with np.load(filename, allow_pickle=False) as z:
        meta = json.loads(bytes(z["meta"]).decode())
        if meta.get("format") != FOREST_FORMAT:
            raise DomainError(_lib.PG_ERR_DOMAIN, f'"{filename}" is not a phylogenetic forest file')
        if meta.get("version") != FOREST_VERSION:
            raise DomainError(_lib.PG_ERR_DOMAIN, f'"{filename}" has format version {meta.get("version")}, '
                              f"this library reads version {FOREST_VERSION}")
        g = meta["genome"]
        genome = GenomeSpec(g["chr_names"], g["chr_lengths"], z["bases"] if g["bases"] else None, g["seed"], g["gc"])
        em = meta["engine"]
        eng = MutationEngine(genome, em["SBS_signatures"], em["indel_signatures"],
                             context_sampling=em["context_sampling"], max_motif_size=em["max_motif_size"],
                             max_repetition_storage=em["max_repetition_storage"],
                             avoid_homozygous_losses=em["avoid_homozygous_losses"],
                             passenger_CNAs=[_driver(c) for c in em["passenger_CNAs"]])
        for name, rates, drivers in em["mutants"]:
            eng.add_mutant(name, rates, [_driver(d) for d in drivers])
        for t, coeffs in em["exposures"]:
            eng.add_exposure(t, coeffs)
        eng.infinite_sites_model = em["infinite_sites_model"]
        sample = np.array([s if s != "" else None for s in z["sample"]], dtype=object)
        forest = SamplesForest(z["cell_id"], z["ancestor"], z["mutant"].astype(object),
                               z["epistate"].astype(object), sample, z["birth_time"], z["divisions"])
    pf = eng.place_mutations(forest, **meta["place"])
    if _table_digest(pf.table()) != meta["digest"]:
        raise _lib.ProcessError(_lib.PG_ERR_RUNTIME, f'"{filename}": the placed mutations differ from the saved ones')
    return pf


# ---------------------------------------------------------------- batches
class Batch:
    """Many independent instances placed and sequenced together (no
    reference counterpart; ``pg_batch_*`` of include/process_gb300.h).

    Instance i: ``forests[i]`` (one species), passenger rates
    ``snv_rates[i]`` / ``indel_rates[i]``, exposure rows ``sbs_exposures[i]``
    / ``id_exposures[i]`` over the engine's signatures (in ``sig_names``
    order), preneoplastic counts and the sequencing keywords
    ``seq_cfgs[i]`` of :func:`sequence_counts`.  Each instance computes what
    the plain path computes for it alone (same seeds and tile size)."""

    def __init__(self, engine: MutationEngine, forests: Sequence[SamplesForest], snv_rates, indel_rates,
                 sbs_exposures, id_exposures, seq_cfgs: Sequence[Mapping], n_pre_snv=None, n_pre_indel=None,
                 preneoplatic_SNV_signature_name: str = "SBS1", preneoplatic_indel_signature_name: str = "ID1"):
        n = len(forests)
        self.engine, self.forests = engine, list(forests)
        self._h = None
        fh = []
        try:
            for f in forests:
                h = C.c_void_p()
                parent = np.ascontiguousarray(f.parent, dtype=np.int32)
                birth = np.ascontiguousarray(f.birth_time, dtype=np.float64)
                zeros = np.zeros(f.num_of_nodes, dtype=np.uint32)
                sample = np.ascontiguousarray(np.where(f.is_leaf, f.sample, -1), dtype=np.int32)
                div = np.ascontiguousarray(f.divisions, dtype=np.uint32)
                check(lib().pg_forest_create(f.num_of_nodes, ptr(parent, C.c_int32), ptr(birth, C.c_double),
                                             ptr(zeros, C.c_uint32), ptr(sample, C.c_int32), ptr(div, C.c_uint32),
                                             len(f.sample_names), C.byref(h)))
                fh.append(h)
            arr = (C.c_void_p * n)(*[h.value for h in fh])
            snv = np.ascontiguousarray(snv_rates, dtype=np.float64)
            ind = np.ascontiguousarray(indel_rates, dtype=np.float64)
            sbs = None if sbs_exposures is None else np.ascontiguousarray(sbs_exposures, dtype=np.float64)
            ids = None if id_exposures is None else np.ascontiguousarray(id_exposures, dtype=np.float64)
            pre_s = None if n_pre_snv is None else np.ascontiguousarray(n_pre_snv, dtype=np.uint32)
            pre_i = None if n_pre_indel is None else np.ascontiguousarray(n_pre_indel, dtype=np.uint32)

            def sig_index(ty, name, counts):
                if counts is None or not np.any(counts):
                    return 0
                if name not in engine.sig_names[ty]:
                    raise DomainError(_lib.PG_ERR_DOMAIN, f"Unknown signature {name}")
                return engine.sig_names[ty].index(name)
            cfgs = (_lib.SeqCfg * n)()
            self._chr_keep = []
            for i, kw in enumerate(seq_cfgs):
                c, sel = seq_cfg(chr_index=engine._chr_index, **kw)
                cfgs[i] = c
                self._chr_keep.append(sel)
            self.n = n
            h = C.c_void_p()
            check(lib().pg_batch_create(engine._h, n, C.cast(arr, C.POINTER(C.c_void_p)), ptr(snv, C.c_double),
                                        ptr(ind, C.c_double), ptr(sbs, C.c_double), ptr(ids, C.c_double),
                                        ptr(pre_s, C.c_uint32), sig_index(0, preneoplatic_SNV_signature_name, pre_s),
                                        ptr(pre_i, C.c_uint32), sig_index(1, preneoplatic_indel_signature_name, pre_i),
                                        cfgs, C.byref(h)))
            self._h = h
        finally:
            for h in fh:
                lib().pg_forest_destroy(h)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _lib._LIB is not None:
            _lib._LIB.pg_batch_destroy(h)
            self._h = None

    @staticmethod
    def _seeds(seeds, n):
        return np.ascontiguousarray(np.broadcast_to(np.asarray(seeds, dtype=np.uint64), (n,)))

    def run(self, place_seeds, seq_seeds) -> None:
        ps, ss = self._seeds(place_seeds, self.n), self._seeds(seq_seeds, self.n)
        check(lib().pg_batch_run(self._h, ptr(ps, C.c_uint64), ptr(ss, C.c_uint64)))

    def autotune(self, place_seeds, seq_seeds) -> np.ndarray:
        ps, ss = self._seeds(place_seeds, self.n), self._seeds(seq_seeds, self.n)
        out = np.empty(self.n, dtype=np.uint32)
        check(lib().pg_batch_autotune(self._h, ptr(ps, C.c_uint64), ptr(ss, C.c_uint64), ptr(out, C.c_uint32)))
        return out

    @property
    def tile_sizes(self) -> np.ndarray:
        out = np.empty(self.n, dtype=np.uint32)
        check(lib().pg_batch_tile_sizes(self._h, ptr(out, C.c_uint32)))
        return out

    @tile_sizes.setter
    def tile_sizes(self, value) -> None:
        v = np.ascontiguousarray(np.broadcast_to(np.asarray(value, dtype=np.uint32), (self.n,)))
        check(lib().pg_batch_set_tile_sizes(self._h, ptr(v, C.c_uint32)))

    def dims(self, i: int) -> tuple[int, int, int]:
        m, s, r = C.c_uint64(), C.c_uint32(), C.c_uint64()
        check(lib().pg_batch_dims(self._h, i, C.byref(m), C.byref(s), C.byref(r)))
        return m.value, s.value, r.value

    def table(self, i: int) -> dict:
        m, _, _ = self.dims(i)
        t = {k: np.empty(m, dtype=np.uint32) for k in ("locus", "edge", "aux")}
        t.update({k: np.empty(m, dtype=np.uint8) for k in ("cls", "sig", "kind", "nature")})
        t["allele"] = np.empty(m, dtype=np.uint16)
        check(lib().pg_batch_copy(self._h, i, ptr(t["locus"], C.c_uint32), ptr(t["edge"], C.c_uint32),
                                  ptr(t["aux"], C.c_uint32), ptr(t["cls"], C.c_uint8), ptr(t["sig"], C.c_uint8),
                                  ptr(t["allele"], C.c_uint16), ptr(t["kind"], C.c_uint8),
                                  ptr(t["nature"], C.c_uint8), None, None))
        return t

    def counts(self, i: int) -> tuple[np.ndarray, np.ndarray]:
        m, s, _ = self.dims(i)
        alt = np.empty((s, m), dtype=np.int32)
        dep = np.empty((s, m), dtype=np.int32)
        check(lib().pg_batch_copy(self._h, i, None, None, None, None, None, None, None, None,
                                  ptr(alt, C.c_int32), ptr(dep, C.c_int32)))
        return alt, dep

    def kernel_ms(self) -> tuple[float, float]:
        a, b = C.c_float(), C.c_float()
        check(lib().pg_batch_kernel_ms(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value


# ---------------------------------------------------------------- sequencing
class SeqResult:
    """Raw sequencing counts kept on the device until read."""

    def __init__(self, handle: C.c_void_p, source: "PhylogeneticForest | None" = None):
        self._h = handle
        self.source = source

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _lib._LIB is not None:
            _lib._LIB.pg_seq_result_destroy(h)
            self._h = None

    def dims(self) -> tuple[int, int, int]:
        s, m, r = C.c_uint32(), C.c_uint64(), C.c_uint64()
        check(lib().pg_seq_result_dims(self._h, C.byref(s), C.byref(m), C.byref(r)))
        return s.value, m.value, r.value

    def counts(self, out: tuple[np.ndarray, np.ndarray] | None = None) -> tuple[np.ndarray, np.ndarray]:
        """alt and depth tables (samples x mutations, int32).  ``out`` takes
        two preallocated C-contiguous int32 arrays of that shape, e.g. views
        of page-locked host memory, which the device copies straight into."""
        s, m, _ = self.dims()
        if out is None:
            alt = np.empty((s, m), dtype=np.int32)
            dep = np.empty((s, m), dtype=np.int32)
        else:
            alt, dep = out
            for a in (alt, dep):
                if a.dtype != np.int32 or a.shape != (s, m) or not a.flags.c_contiguous or not a.flags.writeable:
                    raise ValueError(f"out arrays must be writable C-contiguous int32 of shape {(s, m)}")
        check(lib().pg_seq_result_copy(self._h, ptr(alt, C.c_int32), ptr(dep, C.c_int32)))
        return alt, dep

    def observed(self, out: tuple[np.ndarray, np.ndarray, np.ndarray] | None = None
                 ) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        """The rows of mutations with an alt read in some sample (the rows
        the result data frame keeps by default), compacted on the device:
        (mutation indices (uint32, ascending), alt, depth ([samples][rows],
        int32)).  ``out`` takes three preallocated C-contiguous arrays of
        at least that size (e.g. page-locked host memory); views of their
        first rows are returned."""
        n = C.c_uint64()
        check(lib().pg_seq_result_active(self._h, C.byref(n)))
        s, _, _ = self.dims()
        na = n.value
        if out is None:
            idx = np.empty(na, dtype=np.uint32)
            alt = np.empty((s, na), dtype=np.int32)
            dep = np.empty((s, na), dtype=np.int32)
        else:
            bi, ba, bd = out
            for b, dt, need in ((bi, np.uint32, na), (ba, np.int32, s * na), (bd, np.int32, s * na)):
                if b.dtype != dt or not b.flags.c_contiguous or not b.flags.writeable or b.size < need:
                    raise ValueError(f"out arrays must be writable C-contiguous {np.dtype(dt).name} "
                                     f"with at least {need} elements")
            idx = bi.reshape(-1)[:na]
            alt = ba.reshape(-1)[:s * na].reshape(s, na)
            dep = bd.reshape(-1)[:s * na].reshape(s, na)
        check(lib().pg_seq_result_copy_active(self._h, ptr(idx, C.c_uint32), ptr(alt, C.c_int32),
                                              ptr(dep, C.c_int32)))
        return idx, alt, dep

    def kernel_ms(self) -> float:
        v = C.c_float()
        check(lib().pg_seq_result_kernel_ms(self._h, C.byref(v)))
        return v.value

    def tile_size(self) -> int:
        """The tile size the call used (the automatic choice when none was
        given); a replay of the call needs it."""
        v = C.c_uint32()
        check(lib().pg_seq_result_tile_size(self._h, C.byref(v)))
        return v.value


INSERT_MODELS = {"binomial": 0, "normal": 1}


def seq_cfg(coverage=10, read_size=150, insert_size_mean=0, insert_size_stddev=10, error_rate=0.0, purity=1.0,
            with_normal_sample=True, preneoplastic_in_normal=False, normal_only=False, chromosomes=None,
            tile_size=0, insert_model="binomial", chr_index=None) -> tuple[_lib.SeqCfg, np.ndarray | None]:
    c = _lib.SeqCfg()
    c.coverage = float(coverage)
    c.read_size = int(read_size)
    c.insert_size_mean = int(insert_size_mean)
    c.insert_size_stddev = int(insert_size_stddev)
    c.insert_model = INSERT_MODELS[insert_model]
    c.error_rate = float(error_rate)
    c.purity = float(purity)
    c.with_normal_sample = int(bool(with_normal_sample))
    c.preneoplastic_in_normal = int(bool(preneoplastic_in_normal))
    c.normal_only = int(bool(normal_only))
    c.tile_size = int(tile_size)
    sel = None
    if chromosomes is not None:
        sel = np.ascontiguousarray([chr_index(x) for x in chromosomes], dtype=np.uint32)
        c.n_chr_sel = len(sel)
        c.chr_sel = ptr(sel, C.c_uint32)
    return c, sel


def sequence_counts(phylo_forest: PhylogeneticForest, seed: int, sam: Mapping | None = None, **cfg) -> SeqResult:
    """Runs the read simulator and returns the device-resident counts.
    ``sam`` (keys output_dir, update, filename_prefix, template_name_prefix,
    sample_names) also writes the reads as SAM files."""
    c, _sel = seq_cfg(chr_index=phylo_forest.engine._chr_index, **cfg)
    h = C.c_void_p()
    if sam is None:
        check(lib().pg_simulate_seq(phylo_forest._h, C.byref(c), int(seed), C.byref(h)))
    else:
        names = [str(x).encode() for x in sam["sample_names"]]
        chrs = [str(x).encode() for x in phylo_forest.engine.chr_names]
        sn = (C.c_char_p * len(names))(*names)
        cn = (C.c_char_p * len(chrs))(*chrs)
        sc = _lib.SamCfg(str(sam["output_dir"]).encode(), str(sam.get("filename_prefix", "chr_")).encode(),
                         str(sam.get("template_name_prefix", "r")).encode(), int(bool(sam.get("update", False))),
                         sn, cn)
        check(lib().pg_simulate_seq_sam(phylo_forest._h, C.byref(c), int(seed), C.byref(sc), C.byref(h)))
    return SeqResult(h, phylo_forest)


def _sequencer_rate(sequencer) -> tuple[float, dict | None]:
    if sequencer is None:
        return 0.0, None
    if isinstance(sequencer, ErrorlessIlluminaSequencer):
        return 0.0, {"name": "ErrorlessIlluminaSequencer", "error_rate": 0.0}
    if isinstance(sequencer, BasicIlluminaSequencer):
        return float(sequencer.error_rate), {"name": "BasicIlluminaSequencer", "error_rate": sequencer.error_rate,
                                             "random_quality_scores": sequencer.random_quality_scores}
    raise DomainError(_lib.PG_ERR_DOMAIN, "Unsupported sequencer type")


def _result_frame(pf: PhylogeneticForest, idx: np.ndarray, alt: np.ndarray, dep: np.ndarray,
                  sample_names: list[str]) -> dict:
    """The wide data frame of get_result_dataframe (src/seq_simulation.cpp:142-181)
    over the rows idx (mutation indices, ascending; alt / dep are their
    [sample][row] tables), merged by (chr, pos, ref, alt) in the order of
    each SID's first row: occurrences add, the coverage is the first row's,
    causes and classes are the sorted unions."""
    t = pf.table()
    idx = np.asarray(idx, dtype=np.int64)
    ref, altb = pf._ref_alt(t, idx)
    cause = pf._cause(t, idx)
    nat = NATURES[t["nature"][idx]]
    loc = t["locus"][idx].astype(np.int64)
    n = len(idx)
    # group the rows by SID: a stable sort on (locus, ref, alt) keeps each
    # group's rows in index order
    _, rc = np.unique(ref.astype(str), return_inverse=True) if n else (None, np.zeros(0, np.int64))
    _, ac = np.unique(altb.astype(str), return_inverse=True) if n else (None, np.zeros(0, np.int64))
    order = np.lexsort((ac, rc, loc))
    if n:
        ks = np.stack([loc[order], rc[order], ac[order]], axis=1)
        new = np.ones(n, dtype=bool)
        new[1:] = np.any(ks[1:] != ks[:-1], axis=1)
    else:
        new = np.zeros(0, dtype=bool)
    gsorted = np.cumsum(new) - 1                     # group of each sorted row
    first_sorted = order[new]                        # each group's first row (smallest index)
    gorder = np.argsort(first_sorted, kind="stable")  # groups in the order of their first row
    rank = np.empty(len(gorder), dtype=np.int64)
    rank[gorder] = np.arange(len(gorder))
    group = np.empty(n, dtype=np.int64)
    group[order] = rank[gsorted]                     # output row of every input row
    first = first_sorted[gorder]
    ng = len(first)
    sizes = np.bincount(group, minlength=ng)
    chrn, pos = pf._chr_pos(loc[first] if ng else loc[:0])
    causes = cause[first].copy()
    classes = nat[first].astype(object)
    for g in np.nonzero(sizes > 1)[0]:
        members = np.nonzero(group == g)[0]
        causes[g] = ";".join(sorted({c for c in cause[members] if c is not None})) or None
        classes[g] = ";".join(sorted(set(nat[members])))
    df = {"chr": chrn, "chr_pos": pos, "ref": ref[first], "alt": altb[first], "causes": causes, "classes": classes}
    for s, name in enumerate(sample_names):
        occ = np.bincount(group, weights=alt[s], minlength=ng).astype(np.int32) if n else np.zeros(0, np.int32)
        cov = dep[s, first].astype(np.int32)
        with np.errstate(divide="ignore", invalid="ignore"):
            vaf = np.where(cov > 0, occ / np.maximum(cov, 1), 0.0)
        df[f"{name}.occurrences"] = occ
        df[f"{name}.coverage"] = cov
        df[f"{name}.VAF"] = vaf
    return df


def _result_rows(res: "SeqResult", include_non_sequenced: bool, present: np.ndarray):
    """Rows of the result frame: the observed rows compacted on the device,
    or (include_non_sequenced_mutations) those plus every mutation present
    in a sequenced sample's cells, from the full tables."""
    if not include_non_sequenced:
        return res.observed()
    alt, dep = res.counts()
    idx = np.nonzero((alt.sum(axis=0) > 0) | present)[0]
    return idx, alt[:, idx], dep[:, idx]


def _presence(pf: PhylogeneticForest, n_samples_seq: int, with_normal: bool, pre_in_normal: bool) -> np.ndarray:
    """Mutations present in the cells of some sequenced sample."""
    f = pf.forest
    t = pf.table()
    n = f.num_of_nodes
    tin, tout = f.euler()
    leaf_tins = np.sort(tin[f.is_leaf & (f.sample >= 0)])
    e = t["edge"].astype(np.int64)
    real = e < n
    present = np.zeros(len(e), dtype=bool)
    lo = np.searchsorted(leaf_tins, tin[np.minimum(e, n - 1)], side="left")
    hi = np.searchsorted(leaf_tins, tout[np.minimum(e, n - 1)], side="left")
    present[real] = (hi > lo)[real]
    present[~real] = True
    return present


class SampledCell:
    """A sampled cell as a ``cell_labelling`` function sees it (``SampledCell``
    of src/sequencing.cpp:284-330): its epistate, mutant, species, birth time
    and, on request, its mutations (the columns of
    ``get_sampled_cell_mutations``)."""

    def __init__(self, pf: "PhylogeneticForest", node: int):
        self._pf = pf
        self._node = int(node)

    @property
    def cell_id(self) -> int:
        return int(self._pf.forest.cell_id[self._node])

    @property
    def epistate(self) -> str:
        return str(self._pf.forest.epistate[self._node] or "")

    @property
    def mutant(self) -> str:
        return str(self._pf.forest.mutant[self._node])

    @property
    def species(self) -> str:
        return self.mutant + self.epistate

    @property
    def birth_time(self) -> float:
        return float(self._pf.forest.birth_time[self._node])

    @property
    def mutations(self) -> dict:
        return self._pf.get_sampled_cell_mutations(self.cell_id)


def _forest_partition(pf: "PhylogeneticForest") -> np.ndarray:
    f = pf.forest
    return np.ascontiguousarray(np.where(f.is_leaf & (f.sample >= 0), f.sample, -1), dtype=np.int32)


def _facs_partition(pf: "PhylogeneticForest", labelling) -> tuple[np.ndarray, list[str]]:
    """FACS split of every sample by the label of each of its cells
    (src/seq_simulation.cpp:183-243): the cells of a sample with one label
    form the sample "<sample>_<label>" ("<sample>" for the empty label), in
    the order the labels first appear, cells taken by identifier."""
    if not callable(labelling):
        raise DomainError(_lib.PG_ERR_DOMAIN, "The FACs_labelling_function must be a function.")
    f = pf.forest
    base = _forest_partition(pf)
    part = np.full(f.num_of_nodes, -1, dtype=np.int32)
    names: list[str] = []
    for s, sname in enumerate(f.sample_names):
        cells = np.nonzero(base == s)[0]
        cells = cells[np.argsort(f.cell_id[cells], kind="stable")]
        index: dict[str, int] = {}
        for v in cells:
            label = labelling(SampledCell(pf, v))
            if not isinstance(label, str):
                raise DomainError(_lib.PG_ERR_DOMAIN, "The FACS labelling function must return a string.")
            if label not in index:
                index[label] = len(names)
                names.append(sname if label == "" else f"{sname}_{label}")
            part[v] = index[label]
    return part, names


def simulate_seq(phylo_forest: PhylogeneticForest, sequencer=None, reference_genome=None, chromosomes=None,
                 coverage: float = 10, read_size: int = 150, insert_size_mean: int = 0, insert_size_stddev: int = 10,
                 output_dir: str = "ProCESS_SAM", write_SAM: bool = False, update_SAM: bool = False,
                 cell_labelling=None, purity: float = 1, with_normal_sample: bool = True,
                 preneoplastic_in_normal: bool = False, filename_prefix: str = "chr_",
                 template_name_prefix: str = "r", include_non_sequenced_mutations: bool = False, seed=None,
                 insert_model: str = "binomial", tile_size: int = 0) -> dict:
    """``simulate_seq`` (src/sequencing.cpp:193-209).  Returns
    ``{"mutations": data frame, "parameters": dict}``.  ``insert_model``
    "normal" adds a discretised normal insert size next to the reference's
    binomial model."""
    err, seq_data = _sequencer_rate(sequencer)
    s = _seed(seed)
    samples = list(phylo_forest.forest.sample_names)
    part = None
    if cell_labelling is not None:
        part, samples = _facs_partition(phylo_forest, cell_labelling)
    names = samples + (["normal_sample"] if with_normal_sample else [])
    sam = (dict(output_dir=output_dir, update=update_SAM, filename_prefix=filename_prefix,
                template_name_prefix=template_name_prefix, sample_names=names) if write_SAM else None)
    if part is not None:
        check(lib().pg_placed_set_samples(phylo_forest._h, len(samples), ptr(part, C.c_int32)))
    try:
        res = sequence_counts(phylo_forest, s, sam=sam, coverage=coverage, read_size=read_size,
                              insert_size_mean=insert_size_mean, insert_size_stddev=insert_size_stddev,
                              error_rate=err, purity=purity, with_normal_sample=with_normal_sample,
                              preneoplastic_in_normal=preneoplastic_in_normal, chromosomes=chromosomes,
                              tile_size=tile_size, insert_model=insert_model)
    finally:
        if part is not None:
            base = _forest_partition(phylo_forest)
            check(lib().pg_placed_set_samples(phylo_forest._h, len(phylo_forest.forest.sample_names),
                                              ptr(base, C.c_int32)))
    present = (_presence(phylo_forest, len(names), with_normal_sample, preneoplastic_in_normal)
               if include_non_sequenced_mutations else None)
    df = _result_frame(phylo_forest, *_result_rows(res, include_non_sequenced_mutations, present), names)
    params = {"sequencer": seq_data, "reference_genome": reference_genome, "chromosomes": chromosomes,
              "coverage": coverage, "read_size": read_size, "insert_size_mean": insert_size_mean,
              "insert_size_stddev": insert_size_stddev, "output_dir": output_dir, "write_SAM": write_SAM,
              "update_SAM": update_SAM, "cell_labelling": cell_labelling, "purity": purity,
              "with_normal_sample": with_normal_sample, "filename_prefix": filename_prefix,
              "template_name_prefix": template_name_prefix,
              "include_non_sequenced_mutations": include_non_sequenced_mutations, "seed": s}
    return {"mutations": df, "parameters": params}


def simulate_normal_seq(phylo_forest: PhylogeneticForest, sequencer=None, reference_genome=None, chromosomes=None,
                        coverage: float = 10, read_size: int = 150, insert_size_mean: int = 0,
                        insert_size_stddev: int = 10, output_dir: str = "ProCESS_normal_SAM",
                        write_SAM: bool = True, update_SAM: bool = False, with_preneoplastic: bool = False,
                        filename_prefix: str = "chr_", template_name_prefix: str = "r",
                        include_non_sequenced_mutations: bool = False, seed=None,
                        insert_model: str = "binomial", tile_size: int = 0) -> dict:
    """``simulate_normal_seq`` (src/sequencing.cpp:268-282)."""
    err, seq_data = _sequencer_rate(sequencer)
    s = _seed(seed)
    sam = (dict(output_dir=output_dir, update=update_SAM, filename_prefix=filename_prefix,
                template_name_prefix=template_name_prefix, sample_names=["normal_sample"]) if write_SAM else None)
    res = sequence_counts(phylo_forest, s, sam=sam, coverage=coverage, read_size=read_size,
                          insert_size_mean=insert_size_mean, insert_size_stddev=insert_size_stddev, error_rate=err,
                          purity=1.0, with_normal_sample=True, preneoplastic_in_normal=with_preneoplastic,
                          normal_only=True, chromosomes=chromosomes, tile_size=tile_size, insert_model=insert_model)
    t = phylo_forest.table()
    present = (t["edge"] == phylo_forest.forest.num_of_nodes) & bool(with_preneoplastic)
    df = _result_frame(phylo_forest, *_result_rows(res, include_non_sequenced_mutations, present), ["normal_sample"])
    params = {"sequencer": seq_data, "reference_genome": reference_genome, "chromosomes": chromosomes,
              "coverage": coverage, "read_size": read_size, "insert_size_mean": insert_size_mean,
              "insert_size_stddev": insert_size_stddev, "output_dir": output_dir, "write_SAM": write_SAM,
              "update_SAM": update_SAM, "with_preneoplastic": with_preneoplastic,
              "filename_prefix": filename_prefix, "template_name_prefix": template_name_prefix,
              "include_non_sequenced_mutations": include_non_sequenced_mutations, "seed": s}
    return {"mutations": df, "parameters": params}
