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
import os
import itertools
import weakref
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
    path: str = ""          # the FASTA file it was read from, if any (a forest's reference path)

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
        return cls(names, lengths, bases=np.concatenate(parts), path=str(path))


def driver_regions(drivers: Iterable) -> list:
    """The regions build_contex_index leaves out of the context index for a
    driver catalogue (src/mutation_engine.cpp:240-250): each driver
    mutation's position and max(1, len(ref)) bases, as (chr, begin, length)."""
    return [(str(m.chr), int(m.chr_pos), max(1, len(m.ref))) for m in drivers]


def read_signature_table(path, type_: int) -> dict:
    """A signature table in the reference's format
    (Signature::read_from_stream, src/mutation_engine.cpp:389-397): a
    tab-separated "Type" column of COSMIC class labels ("A[C>A]A" for SBS,
    type 0; "1:Del:C:0" .. "5:Del:M:5" for ID, type 1) and one probability
    column per signature.  Returns {name: probabilities in class order},
    parsed by the library (pg_signature_table_read)."""
    n, size = C.c_uint32(), C.c_uint64()
    p = str(path).encode()
    check(lib().pg_signature_table_read(type_, p, C.byref(n), C.byref(size), None, None))
    nc = 96 if type_ == 0 else 83
    names = C.create_string_buffer(max(size.value, 1))
    probs = np.empty((n.value, nc), dtype=np.float64)
    check(lib().pg_signature_table_read(type_, p, C.byref(n), C.byref(size), names, ptr(probs, C.c_double)))
    keys = names.raw[:size.value].split(b"\0")[:n.value]
    return {k.decode(): probs[i] for i, k in enumerate(keys)}


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
        # a samples forest does not change once built (as the reference's);
        # its columns are read-only, so the library's copy can be kept
        for a in (self.cell_id, self.parent, self.mutant, self.epistate, self.birth_time, self.divisions,
                  self.sample, self.is_leaf):
            a.flags.writeable = False

    def _library_forest(self, species: np.ndarray) -> C.c_void_p:
        """The library's forest (pg_forest) for these species ids, created once
        per species assignment and destroyed with this object."""
        cache = self.__dict__.get("_handles")
        if cache is None:
            cache = self._handles = {}
            weakref.finalize(self, _destroy_forests, cache)
        key = np.ascontiguousarray(species, dtype=np.uint32).tobytes()
        h = cache.get(key)
        if h is None:
            h = C.c_void_p()
            sp = np.ascontiguousarray(species, dtype=np.uint32)
            parent = np.ascontiguousarray(self.parent, dtype=np.int32)
            birth = np.ascontiguousarray(self.birth_time, dtype=np.float64)
            sample = np.ascontiguousarray(np.where(self.is_leaf, self.sample, -1), dtype=np.int32)
            div = np.ascontiguousarray(self.divisions, dtype=np.uint32)
            check(lib().pg_forest_create(self.num_of_nodes, ptr(parent, C.c_int32), ptr(birth, C.c_double),
                                         ptr(sp, C.c_uint32), ptr(sample, C.c_int32), ptr(div, C.c_uint32),
                                         len(self.sample_names), C.byref(h)))
            cache[key] = h
        return h

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
                 avoid_homozygous_losses: bool = True, passenger_CNAs: Iterable | None = None,
                 regions_to_avoid: Iterable | None = None, index_cache_dir: str | None = None):
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
        # positions the SBS context index leaves out (build_contex_index
        # leaves out the driver catalogue, src/mutation_engine.cpp:240-250)
        self.regions_to_avoid = [(str(c), int(b), int(n)) for c, b, n in (regions_to_avoid or [])]
        if self.regions_to_avoid:
            ac = np.ascontiguousarray([self._chr_index(c) for c, _, _ in self.regions_to_avoid], dtype=np.uint32)
            ab = np.ascontiguousarray([b for _, b, _ in self.regions_to_avoid], dtype=np.uint32)
            al = np.ascontiguousarray([n for _, _, n in self.regions_to_avoid], dtype=np.uint32)
            d.n_avoid = len(ac)
            d.avoid_chr, d.avoid_begin, d.avoid_len = ptr(ac, C.c_uint32), ptr(ab, C.c_uint32), ptr(al, C.c_uint32)
        self.index_cache_dir = index_cache_dir
        if index_cache_dir:
            d.index_cache_dir = str(index_cache_dir).encode()
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
    def set_signatures(self, type_: int, sigs) -> None:
        """Signatures of a type (0 SBS, 1 ID): a mapping name -> class
        probabilities, or the path of a signature table in the reference's
        format (see :func:`read_signature_table`)."""
        if isinstance(sigs, (str, os.PathLike)):
            sigs = read_signature_table(sigs, type_)
        nc = 96 if type_ == 0 else 83
        names = list(sigs.keys())
        mat = np.ascontiguousarray(np.array([np.asarray(sigs[k], dtype=np.float64) for k in names]))
        if mat.shape != (len(names), nc):
            raise DomainError(_lib.PG_ERR_DOMAIN, f"signatures must have {nc} classes")
        check(lib().pg_engine_set_signatures(self._h, type_, len(names), ptr(mat, C.c_double)))
        arr = (C.c_char_p * len(names))(*[str(k).encode() for k in names])
        check(lib().pg_engine_set_signature_names(self._h, type_, len(names), arr))
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
        fh = f._library_forest(species)
        ph = C.c_void_p()
        s = _seed(seed)
        check(lib().pg_place_mutations(self._h, fh, int(num_of_preneoplatic_SNVs), pre_s,
                                       int(num_of_preneoplatic_indels), pre_i, s, C.byref(ph)))
        pf = PhylogeneticForest(self, f, ph, s)
        pf._place_args = dict(num_of_preneoplatic_SNVs=int(num_of_preneoplatic_SNVs),
                              num_of_preneoplatic_indels=int(num_of_preneoplatic_indels), seed=s,
                              preneoplatic_SNV_signature_name=preneoplatic_SNV_signature_name,
                              preneoplatic_indel_signature_name=preneoplatic_indel_signature_name)
        # the forest keeps the configuration it was placed with (exposures,
        # mutants, species rates), as the reference's forest holds its own
        # copies: later add_exposure / add_mutant calls do not change it
        pf._config = self._config()
        pf._species_rates = self.get_species_rates()
        pf._reference_path = getattr(self.genome, "path", "") or ""
        return pf

    def _config(self) -> dict:
        """JSON-ready copy of the engine's configuration."""
        import copy
        return {"context_sampling": self.context_sampling, "max_motif_size": self.max_motif_size,
                "max_repetition_storage": self.max_repetition_storage,
                "avoid_homozygous_losses": self.avoid_homozygous_losses,
                "infinite_sites_model": self.infinite_sites_model,
                "SBS_signatures": _plain(self._sigs[0]), "indel_signatures": _plain(self._sigs[1]),
                "exposures": copy.deepcopy(_plain(self._exposures)),
                "mutants": copy.deepcopy(_plain(self._mutant_specs)),
                "passenger_CNAs": _plain(self.passenger_CNAs),
                "regions_to_avoid": _plain(getattr(self, "regions_to_avoid", []))}


def _destroy_forests(cache: dict) -> None:
    if _lib._LIB is not None:
        for h in cache.values():
            _lib._LIB.pg_forest_destroy(h)
    cache.clear()


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

    def mutation_columns(self, rows=None) -> dict:
        """The columns chr, chr_pos, ref, alt, type, cause and class of the
        placed mutations ``rows`` (indices into :meth:`table`; all when None),
        from pg_placed_mutation_info."""
        r = None if rows is None else np.ascontiguousarray(rows, dtype=np.uint32)
        n = self.num_of_mutations if r is None else len(r)
        chr_, pos = np.empty(n, np.uint32), np.empty(n, np.uint32)
        ref, alt = np.zeros(n * _lib.SID_CHARS, np.uint8), np.zeros(n * _lib.SID_CHARS, np.uint8)
        kind, cause, nat = np.empty(n, np.uint8), np.empty(n, np.int32), np.empty(n, np.uint8)
        if n:
            check(lib().pg_placed_mutation_info(self._h, n, ptr(r, C.c_uint32), ptr(chr_, C.c_uint32),
                                                ptr(pos, C.c_uint32), _cbuf(ref), _cbuf(alt), ptr(kind, C.c_uint8),
                                                ptr(cause, C.c_int32), ptr(nat, C.c_uint8)))
        names = np.array(self.engine.chr_names, dtype=object)
        sig = [np.array(list(self.engine.sig_names[k]) + [None], dtype=object) for k in (0, 1)]
        cz = np.where(cause < 0, 10 ** 6, cause)
        cnames = np.full(n, None, dtype=object)
        for k in (0, 1):
            m = kind == k
            cnames[m] = sig[k][np.minimum(cz[m], len(sig[k]) - 1)]
        return {"chr": names[chr_], "chr_pos": pos.astype(np.int64), "ref": _sid_strings(ref, n),
                "alt": _sid_strings(alt, n), "type": np.where(kind == 0, "SNV", "indel").astype(object),
                "cause": cnames, "class": NATURES[nat].astype(object)}

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

    def _getter_cells(self, cell_id=None) -> np.ndarray:
        """Node ids of the sampled cells by cell id (the reference's std::map
        order), or of the one cell ``cell_id``."""
        f = self.forest
        if cell_id is not None:
            hit = np.nonzero(f.cell_id == int(cell_id))[0]
            if len(hit) == 0 or not f.is_leaf[hit[0]]:
                raise DomainError(_lib.PG_ERR_DOMAIN, f'Cell "{cell_id}" is not a leaf')
            return np.ascontiguousarray(hit[:1], dtype=np.uint32)
        leaves = np.nonzero(f.is_leaf & (f.sample >= 0))[0]
        return np.ascontiguousarray(leaves[np.argsort(f.cell_id[leaves], kind="stable")], dtype=np.uint32)

    def cell_mutation_rows(self, cell_id=None) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        """(cell node, mutation row, allele instance) of every mutation each
        sampled cell holds (pg_placed_cell_mutations), in the order of
        :meth:`get_sampled_cell_mutations`."""
        cells = self._getter_cells(cell_id)
        n = C.c_uint64()
        check(lib().pg_placed_cell_mutations(self._h, len(cells), ptr(cells, C.c_uint32), C.byref(n)))
        cell, row, allele = (np.empty(n.value, np.uint32) for _ in range(3))
        check(lib().pg_placed_cell_mutations_copy(self._h, ptr(cell, C.c_uint32), ptr(row, C.c_uint32),
                                                  ptr(allele, C.c_uint32)))
        return cell, row, allele

    def get_sampled_cell_mutations(self, cell_id=None) -> dict:
        """Columns cell_id, chr, chr_pos, allele, ref, alt, type, cause, class
        (src/phylogenetic_forest.cpp:452-507), built by the library
        (pg_placed_cell_mutations): every mutation a sampled cell holds, once
        per allele instance of its genome carrying it (an SID is copied with
        its allele by an amplification or a WGD after it, and leaves with a
        deleted allele); ``allele`` is the instance.  Cells by cell id, each
        cell's rows by chromosome, allele, position."""
        cell, row, allele = self.cell_mutation_rows(cell_id)
        cols = self.mutation_columns(row)
        return {"cell_id": self.forest.cell_id[cell], "chr": cols["chr"], "chr_pos": cols["chr_pos"],
                "allele": allele.astype(np.int64), "ref": cols["ref"], "alt": cols["alt"], "type": cols["type"],
                "cause": cols["cause"], "class": cols["class"]}

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
        (NA, i.e. -1, for deletions) and class (src/phylogenetic_forest.cpp:509-562):
        the events on each sampled cell's root path (pg_placed_cell_cnas)."""
        cells = self._getter_cells(cell_id)
        c = self.cna_table()
        n = C.c_uint64()
        check(lib().pg_placed_cell_cnas(self._h, len(cells), ptr(cells, C.c_uint32), C.byref(n)))
        cell, idx = np.empty(n.value, np.uint32), np.empty(n.value, np.uint32)
        check(lib().pg_placed_cell_cnas_copy(self._h, ptr(cell, C.c_uint32), ptr(idx, C.c_uint32)))
        names = np.array(self.engine.chr_names + [""], dtype=object)
        tname = np.array(["D", "A", "WGD"], dtype=object)
        typ = c["type"][idx]
        wgd = typ == 2
        return {"cell_id": self.forest.cell_id[cell], "type": tname[typ],
                "chr": names[np.where(wgd, len(names) - 1, c["chr"][idx])],
                "begin": np.where(wgd, -1, c["begin"][idx].astype(np.int64)),
                "end": np.where(wgd, -1, c["end"][idx].astype(np.int64)),
                "allele": np.where(wgd, -1, c["allele"][idx].astype(np.int64)),
                "src allele": np.where(typ == 1, c["src"][idx].astype(np.int64), -1),
                "class": np.where(c["driver"][idx] == 1, "driver", "passenger").astype(object)}

    # -- copy-number getters (allelic fragmentation) ------------------------------------
    def get_cell_allelic_fragmentation(self) -> dict:
        """Columns cell_id, chr, begin, end, major, minor: every sampled cell's
        genome cut into stretches of one allelic type (copies of the two
        germline alleles; major = the larger), src/phylogenetic_forest.cpp:867-927
        (pg_placed_cell_fragmentation)."""
        cells = self._getter_cells()
        n = C.c_uint64()
        check(lib().pg_placed_cell_fragmentation(self._h, len(cells), ptr(cells, C.c_uint32), C.byref(n)))
        cell, chr_, b, e, mj, mn = (np.empty(n.value, np.uint32) for _ in range(6))
        check(lib().pg_placed_cell_fragmentation_copy(self._h, *(ptr(x, C.c_uint32) for x in (cell, chr_, b, e, mj,
                                                                                              mn))))
        names = np.array(self.engine.chr_names, dtype=object)
        return {"cell_id": self.forest.cell_id[cell], "chr": names[chr_], "begin": b.astype(np.int64),
                "end": e.astype(np.int64), "major": mj.astype(np.int64), "minor": mn.astype(np.int64)}

    def get_bulk_allelic_fragmentation(self, sample_name: str | None = None) -> dict:
        """Columns chr, begin, end, major, minor, ratio: for every stretch of
        the genome on which the sampled cells (of one sample, or all) keep
        their allelic types, each type with the fraction of cells showing it
        (src/phylogenetic_forest.cpp:767-820; pg_placed_bulk_fragmentation)."""
        f = self.forest
        s = -1
        if sample_name is not None:
            if sample_name not in f.sample_names:
                raise DomainError(_lib.PG_ERR_DOMAIN, f'Unknown sample "{sample_name}".')
            s = f.sample_names.index(sample_name)
        n = C.c_uint64()
        check(lib().pg_placed_bulk_fragmentation(self._h, s, C.byref(n)))
        chr_, b, e, mj, mn = (np.empty(n.value, np.uint32) for _ in range(5))
        ratio = np.empty(n.value, np.float64)
        check(lib().pg_placed_bulk_fragmentation_copy(self._h, *(ptr(x, C.c_uint32) for x in (chr_, b, e, mj, mn)),
                                                      ptr(ratio, C.c_double)))
        names = np.array(self.engine.chr_names, dtype=object)
        return {"chr": names[chr_], "begin": b.astype(np.int64), "end": e.astype(np.int64),
                "major": mj.astype(np.int64), "minor": mn.astype(np.int64), "ratio": ratio}

    def get_samples_info(self) -> dict:
        """name, tumour_cells, DNA_quantity, equivalent_normal_cells
        (src/phylogenetic_forest.cpp:57-99): the DNA of a sample is the summed
        allelic size of its sampled cells' genomes (pg_placed_samples_info)."""
        info = self.forest.get_samples_info()
        f = self.forest
        k = len(f.sample_names)
        cells, dna, eq = np.empty(max(k, 1), np.uint32), np.empty(max(k, 1)), np.empty(max(k, 1))
        check(lib().pg_placed_samples_info(self._h, ptr(cells, C.c_uint32), ptr(dna, C.c_double),
                                           ptr(eq, C.c_double)))
        order = [f.sample_names.index(name) for name in info["name"]]
        info["DNA_quantity"] = dna[order]
        info["equivalent_normal_cells"] = eq[order]
        return info

    def save(self, filename: str, quiet: bool = False) -> None:
        """``PhylogeneticForest$save(filename, quiet)``; see :func:`save_phylogenetic_forest`."""
        save_phylogenetic_forest(self, filename)

    def get_germline_mutations(self) -> dict:
        return {k: np.array([]) for k in ("chr", "chr_pos", "allele", "ref", "alt", "type", "cause", "class")}

    def get_species_info(self) -> dict:
        """The registered species (src/phylogenetic_forest.cpp:220-255):
        mutant, epistate, SNV_rate, indel_rate and CNA_rate."""
        r = getattr(self, "_species_rates", None) or self.engine.get_species_rates()
        return {"mutant": r["mutant"], "epistate": r["epistate"], "SNV_rate": r["SNV"], "indel_rate": r["indel"],
                "CNA_rate": r["CNA"]}

    def _mutants(self) -> list:
        """add_mutant calls in force when the forest was placed."""
        cfg = getattr(self, "_config", None)
        if cfg is None:
            return list(self.engine._mutant_specs)
        return [(name, rates, [_driver(d) for d in drivers]) for name, rates, drivers in cfg["mutants"]]

    def _exposure_list(self) -> list:
        """Timed exposures in force when the forest was placed."""
        cfg = getattr(self, "_config", None)
        return list(self.engine._exposures) if cfg is None else [(float(t), dict(c)) for t, c in cfg["exposures"]]

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
        for name, _, drivers in self._mutants():
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
        for t, coef in self._exposure_list():
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
            cols = self.mutation_columns(cand) if len(cand) else {"ref": np.array([]), "alt": np.array([])}
            ref, alt = cols["ref"], cols["alt"]
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
FOREST_VERSION = 2


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


def save_phylogenetic_forest(pf: "PhylogeneticForest", filename: str) -> None:
    """``PhylogeneticForest$save`` (src/phylogenetic_forest.cpp:940-955).  The
    RACES archive layout is unavailable, so the file is a versioned native
    archive (numpy .npz) holding the library's archive of the placed forest
    (pg_placed_serialize: placed mutations, genotype classes, allele
    lineage, CNA events), the samples forest, the engine configuration the
    forest was placed with and its reference path.  Loading restores the
    placed tables without placing again."""
    import json
    f = pf.forest
    n = C.c_uint64()
    check(lib().pg_placed_serialize(pf._h, None, 0, C.byref(n)))
    blob = np.empty(n.value, dtype=np.uint8)
    check(lib().pg_placed_serialize(pf._h, ptr(blob, C.c_uint8), n.value, C.byref(n)))
    e = pf.engine
    meta = {
        "format": FOREST_FORMAT, "version": FOREST_VERSION,
        "genome": {"chr_names": list(e.chr_names), "chr_lengths": [int(x) for x in e.chr_lengths],
                   "seed": int(e.genome.seed), "gc": float(e.genome.gc), "bases": e.genome.bases is not None},
        "engine": getattr(pf, "_config", None) or e._config(),
        "species_rates": _plain(getattr(pf, "_species_rates", None) or e.get_species_rates()),
        "place": _plain(getattr(pf, "_place_args", {"seed": pf.seed})),
        "reference_path": pf.get_reference_path(),
    }
    ancestor = np.where(f.parent >= 0, f.cell_id[np.maximum(f.parent, 0)], -1)
    sample = np.array([f.sample_names[s] if s >= 0 else "" for s in f.sample], dtype=object)
    arrays = {"meta": np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8), "placed": blob,
              "cell_id": f.cell_id, "ancestor": ancestor, "mutant": f.mutant.astype(str),
              "epistate": np.array(["" if x is None else str(x) for x in f.epistate]),
              "sample": sample.astype(str), "birth_time": f.birth_time, "divisions": f.divisions}
    if e.genome.bases is not None:
        arrays["bases"] = np.asarray(e.genome.bases, dtype=np.uint8)
    with open(filename, "wb") as fh:
        np.savez_compressed(fh, **arrays)


def load_phylogenetic_forest(filename: str, quiet: bool = False) -> "PhylogeneticForest":
    """``load_phylogenetic_forest(filename, quiet)`` (src/mutations.cpp:1466-1480):
    rebuilds the engine (genome, signatures, the configuration the forest was
    placed with) and the samples forest of a saved file, and restores the
    placed forest from its archive (pg_placed_deserialize)."""
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
                             passenger_CNAs=[_driver(c) for c in em["passenger_CNAs"]],
                             regions_to_avoid=[tuple(r) for r in em.get("regions_to_avoid", [])])
        for name, rates, drivers in em["mutants"]:
            eng.add_mutant(name, rates, [_driver(d) for d in drivers])
        for t, coeffs in em["exposures"]:
            eng.add_exposure(t, coeffs)
        eng.infinite_sites_model = em["infinite_sites_model"]
        sample = np.array([s if s != "" else None for s in z["sample"]], dtype=object)
        forest = SamplesForest(z["cell_id"], z["ancestor"], z["mutant"].astype(object),
                               z["epistate"].astype(object), sample, z["birth_time"], z["divisions"])
        blob = np.ascontiguousarray(z["placed"], dtype=np.uint8)
    ph = C.c_void_p()
    check(lib().pg_placed_deserialize(eng._h, ptr(blob, C.c_uint8), len(blob), C.byref(ph)))
    pf = PhylogeneticForest(eng, forest, ph, int(meta["place"].get("seed", 0)))
    pf._place_args = meta["place"]
    pf._config = em
    pf._species_rates = meta.get("species_rates")
    pf._reference_path = meta.get("reference_path", "")
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


def _sid_strings(buf: np.ndarray, n: int) -> np.ndarray:
    """Strings of a buffer of n NUL-padded SID_CHARS-byte fields."""
    if n == 0:
        return np.zeros(0, dtype=object)
    return buf.reshape(n, _lib.SID_CHARS).view(f"S{_lib.SID_CHARS}").ravel().astype(str).astype(object)


def _cbuf(arr: np.ndarray):
    return arr.ctypes.data_as(C.c_char_p)


_CLASS_NAMES = None


def _class_names() -> np.ndarray:
    """Joined nature names of every bit set of natures (sorted names, ';')."""
    global _CLASS_NAMES
    if _CLASS_NAMES is None:
        out = []
        for m in range(16):
            out.append(";".join(sorted(str(NATURES[b]) for b in range(4) if m >> b & 1)))
        _CLASS_NAMES = np.array(out, dtype=object)
    return _CLASS_NAMES


def _result_frame(res: "SeqResult", pf: PhylogeneticForest, include_non_sequenced: bool,
                  sample_names: list[str]) -> dict:
    """The wide data frame of get_result_dataframe (src/seq_simulation.cpp:52-181),
    built by the library (pg_seq_result_frame): one row per SID in
    (chromosome, position, ref, alt) order, occurrences summed over the
    SID's mutations, the coverage of its locus, causes and classes as the
    sorted unions joined by ';'."""
    n = C.c_uint64()
    check(lib().pg_seq_result_frame(res._h, pf._h, 1 if include_non_sequenced else 0, C.byref(n)))
    R = n.value
    nc = C.c_uint64()
    check(lib().pg_seq_result_frame_causes_size(res._h, C.byref(nc)))
    S = res.dims()[0]
    chr_, pos = np.empty(R, np.uint32), np.empty(R, np.uint32)
    ref, alt = np.zeros(R * _lib.SID_CHARS, np.uint8), np.zeros(R * _lib.SID_CHARS, np.uint8)
    coff = np.zeros(R + 1, np.uint64)
    cb = np.zeros(max(nc.value, 1), np.uint8)
    classes = np.zeros(R, np.uint8)
    occ, cov = np.empty((S, R), np.int32), np.empty((S, R), np.int32)
    vaf = np.empty((S, R), np.float64)
    check(lib().pg_seq_result_frame_copy(res._h, ptr(chr_, C.c_uint32), ptr(pos, C.c_uint32), _cbuf(ref), _cbuf(alt),
                                         ptr(coff, C.c_uint64), _cbuf(cb), ptr(classes, C.c_uint8),
                                         ptr(occ, C.c_int32), ptr(cov, C.c_int32), ptr(vaf, C.c_double)))
    # causes: the joined strings into fixed-width fields, empty ones NA (None)
    lens = np.diff(coff).astype(np.int64)
    width = int(lens.max()) if R else 0
    causes = np.full(R, None, dtype=object)
    if width:
        grid = np.zeros((R, width), np.uint8)
        rows = np.repeat(np.arange(R), lens)
        cols = np.arange(int(lens.sum())) - np.repeat(coff[:-1].astype(np.int64), lens)
        grid[rows, cols] = cb[:int(lens.sum())]
        txt = grid.view(f"S{width}").ravel().astype(str).astype(object)
        causes[lens > 0] = txt[lens > 0]
    names = np.array(pf.engine.chr_names, dtype=object)
    df = {"chr": names[chr_], "chr_pos": pos.astype(np.int64), "ref": _sid_strings(ref, R),
          "alt": _sid_strings(alt, R), "causes": causes, "classes": _class_names()[classes & 15]}
    for s, name in enumerate(sample_names):
        df[f"{name}.occurrences"] = occ[s]
        df[f"{name}.coverage"] = cov[s]
        df[f"{name}.VAF"] = vaf[s]
    return df


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
    df = _result_frame(res, phylo_forest, include_non_sequenced_mutations, names)
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
    df = _result_frame(res, phylo_forest, include_non_sequenced_mutations, ["normal_sample"])
    params = {"sequencer": seq_data, "reference_genome": reference_genome, "chromosomes": chromosomes,
              "coverage": coverage, "read_size": read_size, "insert_size_mean": insert_size_mean,
              "insert_size_stddev": insert_size_stddev, "output_dir": output_dir, "write_SAM": write_SAM,
              "update_SAM": update_SAM, "with_preneoplastic": with_preneoplastic,
              "filename_prefix": filename_prefix, "template_name_prefix": template_name_prefix,
              "include_non_sequenced_mutations": include_non_sequenced_mutations, "seed": s}
    return {"mutations": df, "parameters": params}
