"""ORACLE — test infrastructure only (the product never imports this package).

ctypes wrapper of ``oracle/_build/liboracle.so``, the sequential CPU
restatement of the placement and sequencing path (oracle.cpp).  PARITY
UNPINNED: RACES, which holds the reference arithmetic, is absent; the
restatement follows ProCESS's call sites and data contracts (see oracle.cpp).
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"
_L = None


def build() -> Path:
    r = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB_PATH


def lib() -> C.CDLL:
    global _L
    if _L is None:
        if not LIB_PATH.exists():
            build()
        L = C.CDLL(str(LIB_PATH))
        P = C.c_void_p
        u8p, u16p, u32p, i32p, u64p, f64p = (C.POINTER(t) for t in (C.c_uint8, C.c_uint16, C.c_uint32, C.c_int32,
                                                                      C.c_uint64, C.c_double))
        sig = {
            "orc_last_error": (C.c_char_p, []),
            "orc_philox": (None, [C.c_uint32] * 6 + [u32p]),
            "orc_log": (C.c_double, [C.c_double]),
            "orc_exp": (C.c_double, [C.c_double]),
            "orc_log_factorial": (C.c_double, [C.c_double]),
            "orc_poisson": (C.c_uint64, [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_double]),
            "orc_binomial": (C.c_uint64, [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64,
                                          C.c_double]),
            "orc_genome_synth": (None, [C.c_uint64, C.c_uint64, C.c_double, u8p]),
            "orc_engine_create": (P, [C.c_uint32, u32p, u8p, C.c_uint64, C.c_double, C.c_uint32, C.c_uint32]),
            "orc_engine_destroy": (None, [P]),
            "orc_engine_set_avoid": (None, [P, C.c_uint32, u32p, u32p, u32p]),
            "orc_engine_index_info": (None, [P, u64p, u64p, u32p, u32p]),
            "orc_engine_read_index": (None, [P, C.c_int, C.c_uint32, u32p]),
            "orc_engine_read_genome": (None, [P, u8p]),
            "orc_placed_carriers": (C.c_uint64, [P, u32p, u32p]),
            "orc_engine_set_signatures": (None, [P, C.c_int, C.c_uint32, f64p]),
            "orc_engine_add_exposure": (None, [P, C.c_int, C.c_double, f64p]),
            "orc_engine_set_species_rates": (None, [P, C.c_uint32, C.c_double, C.c_double, C.c_double]),
            "orc_engine_set_species_epoch_rates": (None, [P, C.c_uint32, C.c_uint32, f64p, f64p]),
            "orc_engine_set_species_mutant": (None, [P, C.c_uint32, C.c_uint32]),
            "orc_engine_add_driver_sid": (None, [P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_char_p, C.c_char_p,
                                                 C.c_int32]),
            "orc_engine_set_infinite_sites": (None, [P, C.c_int]),
            "orc_engine_add_driver_cna": (None, [P, C.c_uint32, C.c_int, C.c_uint32, C.c_uint32, C.c_uint32,
                                                 C.c_int32, C.c_int32]),
            "orc_engine_add_driver_wgd": (None, [P, C.c_uint32]),
            "orc_engine_add_passenger_cna": (None, [P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int]),
            "orc_engine_set_avoid_homozygous_losses": (None, [P, C.c_int]),
            "orc_placed_cna_count": (C.c_uint64, [P]),
            "orc_placed_cna_copy": (None, [P, u32p, u8p, u32p, u32p, u32p, u32p, u32p, u8p]),
            "orc_placed_node_classes": (None, [P, u32p, u32p, u32p]),
            "orc_placed_class_pieces": (C.c_uint64, [P, C.c_uint32, u32p, u32p, u32p]),
            "orc_placed_inst_roots": (C.c_uint32, [P, u8p]),
            "orc_place": (P, [P, C.c_uint32, i32p, f64p, u32p, i32p, u32p, C.c_uint32, C.c_uint32, C.c_uint32,
                              C.c_uint32, C.c_uint32, C.c_uint64, C.c_int]),
            "orc_placed_destroy": (None, [P]),
            "orc_placed_count": (C.c_uint64, [P]),
            "orc_placed_copy": (None, [P, u32p, u32p, u32p, u8p, u8p, u16p, u8p, u8p]),
            "orc_placed_set": (C.c_int, [P, C.c_uint64, u32p, u32p, u16p, u8p]),
            "orc_seq": (P, [P, C.c_void_p, C.c_uint64, C.c_int, C.c_double, C.c_int]),
            "orc_seq_destroy": (None, [P]),
            "orc_sam": (C.c_int, [P, C.c_void_p, C.c_uint64, C.c_char_p]),
            "orc_seq_samples": (C.c_uint32, [P]),
            "orc_seq_reads": (C.c_uint64, [P]),
            "orc_seq_copy": (None, [P, i32p, i32p]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _L = L
    return _L


def _p(a, t):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))


def _err():
    return lib().orc_last_error().decode()


class OracleEngine:
    """Mirror of process_gb300.MutationEngine over the CPU restatement."""

    def __init__(self, chr_lengths, bases=None, seed=0, gc=0.5, context_sampling=100, max_rep=500000):
        self.chr_lengths = np.ascontiguousarray(chr_lengths, dtype=np.uint32)
        b = None if bases is None else np.ascontiguousarray(bases, dtype=np.uint8)
        self._h = lib().orc_engine_create(len(self.chr_lengths), _p(self.chr_lengths, C.c_uint32),
                                          _p(b, C.c_uint8), int(seed), float(gc), int(context_sampling),
                                          int(max_rep))
        if not self._h:
            raise RuntimeError(_err())
        self.sig_names = [[], []]

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_engine_destroy(self._h)
            self._h = None

    @classmethod
    def like(cls, w, **kw):
        """An oracle engine configured like process_gb300.synth.build_engine(w)."""
        g = w.genome
        e = cls(g.chr_lengths, g.bases, g.seed, g.gc, context_sampling=w.context_sampling, **kw)
        e.set_signatures(0, w.sbs)
        e.set_signatures(1, w.ids)
        species = {}
        for mut_id, (name, rates, drivers) in enumerate(w.mutants):
            keys = set(rates.keys())
            per_epi = {"": rates} if keys <= {"SNV", "indel", "CNA"} else dict(rates)
            for epi, r in per_epi.items():
                sid = species.setdefault((name, epi), len(species))
                snv, indel, cna = r.get("SNV", 0.0), r.get("indel", 0.0), r.get("CNA", 0.0)
                if np.ndim(snv) or np.ndim(indel):
                    n = max(np.size(snv), np.size(indel))
                    e.set_epoch_rates(sid, np.broadcast_to(np.asarray(snv, float), (n,)),
                                      np.broadcast_to(np.asarray(indel, float), (n,)))
                    e.set_rates(sid, np.atleast_1d(snv)[0], np.atleast_1d(indel)[0], cna)
                else:
                    e.set_rates(sid, snv, indel, cna)
                lib().orc_engine_set_species_mutant(e._h, sid, mut_id)
        e.species = species
        for t, coeffs in w.exposures:
            e.add_exposure(t, coeffs)
        idx = {str(n): i for i, n in enumerate(g.chr_names)}
        off = np.concatenate([[0], np.cumsum(np.asarray(g.chr_lengths, dtype=np.int64))])
        genome = None
        for mut_id, (_, _, drivers) in enumerate(w.mutants):
            resolved = []
            for d in drivers:
                if type(d).__name__ == "Mutation" and d.ref == "?":
                    if genome is None:
                        genome = e.read_genome()
                    ref = "ACGT"[genome[off[idx[d.chr]] + d.chr_pos - 1]]
                    d = type(d)(d.chr, d.chr_pos, ref, d.alt, d.allele)
                resolved.append(d)
            e.add_drivers(mut_id, resolved, idx.__getitem__)
        return e

    def set_signatures(self, ty, sigs: dict):
        names = list(sigs)
        mat = np.ascontiguousarray(np.array([sigs[k] for k in names], dtype=np.float64))
        lib().orc_engine_set_signatures(self._h, ty, len(names), _p(mat, C.c_double))
        self.sig_names[ty] = names

    def add_exposure(self, time, coeffs: dict):
        for ty in (0, 1):
            v = np.zeros(len(self.sig_names[ty]))
            used = False
            for k, c in coeffs.items():
                if k in self.sig_names[ty]:
                    v[self.sig_names[ty].index(k)] = c
                    used = True
            if used:
                lib().orc_engine_add_exposure(self._h, ty, float(time), _p(np.ascontiguousarray(v), C.c_double))

    def set_rates(self, sid, snv, indel, cna=0.0):
        lib().orc_engine_set_species_rates(self._h, sid, float(snv), float(indel), float(cna))

    def set_epoch_rates(self, sid, snv, indel):
        s = np.ascontiguousarray(snv, dtype=np.float64)
        i = np.ascontiguousarray(indel, dtype=np.float64)
        lib().orc_engine_set_species_epoch_rates(self._h, sid, len(s), _p(s, C.c_double), _p(i, C.c_double))

    def add_driver_sid(self, mutant, chr_idx, pos, ref, alt, allele=-1):
        lib().orc_engine_add_driver_sid(self._h, mutant, chr_idx, pos, ref.encode(), alt.encode(), allele)

    def set_infinite_sites(self, on):
        lib().orc_engine_set_infinite_sites(self._h, 1 if on else 0)

    def add_driver_cna(self, mutant, amp, chr_idx, begin, length, allele=-1, src=-1):
        lib().orc_engine_add_driver_cna(self._h, mutant, 1 if amp else 0, chr_idx, begin, length, allele, src)

    def add_driver_wgd(self, mutant):
        lib().orc_engine_add_driver_wgd(self._h, mutant)

    def add_passenger_cna(self, chr_idx, begin, length, amp):
        lib().orc_engine_add_passenger_cna(self._h, chr_idx, begin, length, 1 if amp else 0)

    def set_avoid_homozygous_losses(self, on):
        lib().orc_engine_set_avoid_homozygous_losses(self._h, 1 if on else 0)

    def add_drivers(self, mutant, drivers, chr_index):
        """Driver lists as given to process_gb300.MutationEngine.add_mutant
        (SNV/Mutation with explicit ref, CNA, WGD); chr_index maps names."""
        for d in drivers:
            kind = type(d).__name__
            if kind == "Mutation":
                al = -1 if d.allele is None else int(d.allele)
                lib().orc_engine_add_driver_sid(self._h, mutant, chr_index(d.chr), int(d.chr_pos), d.ref.encode(),
                                                d.alt.encode(), al)
            elif kind == "CNA":
                self.add_driver_cna(mutant, d.type == "A", chr_index(d.chr), int(d.chr_pos), int(d.len),
                                    -1 if d.allele is None else int(d.allele),
                                    -1 if d.src_allele is None else int(d.src_allele))
            else:
                self.add_driver_wgd(mutant)

    def set_regions_to_avoid(self, regions, chr_index):
        """(chromosome, 1-based begin, length) triples; rebuilds the indices."""
        c = np.ascontiguousarray([chr_index(r[0]) for r in regions], dtype=np.uint32)
        b = np.ascontiguousarray([r[1] for r in regions], dtype=np.uint32)
        n = np.ascontiguousarray([r[2] for r in regions], dtype=np.uint32)
        lib().orc_engine_set_avoid(self._h, len(c), _p(c, C.c_uint32), _p(b, C.c_uint32), _p(n, C.c_uint32))

    def index_info(self):
        ct, it = np.zeros(32, np.uint64), np.zeros(83, np.uint64)
        cl, il = np.zeros(32, np.uint32), np.zeros(83, np.uint32)
        lib().orc_engine_index_info(self._h, _p(ct, C.c_uint64), _p(it, C.c_uint64), _p(cl, C.c_uint32),
                                    _p(il, C.c_uint32))
        return {"ctx_total": ct, "id_total": it, "ctx_stored": cl, "id_stored": il}

    def read_index(self, which, cls):
        n = self.index_info()["ctx_stored" if which == 0 else "id_stored"][cls]
        out = np.empty(n, dtype=np.uint32)
        lib().orc_engine_read_index(self._h, which, cls, _p(out, C.c_uint32))
        return out

    def read_genome(self):
        out = np.empty(int(self.chr_lengths.astype(np.uint64).sum()), dtype=np.uint8)
        lib().orc_engine_read_genome(self._h, _p(out, C.c_uint8))
        return out

    def place(self, forest, species, n_pre_snv=0, pre_sbs=0, n_pre_id=0, pre_id=0, seed=0, flavour=0):
        parent = np.ascontiguousarray(forest.parent, dtype=np.int32)
        birth = np.ascontiguousarray(forest.birth_time, dtype=np.float64)
        sp = np.ascontiguousarray(species, dtype=np.uint32)
        sample = np.ascontiguousarray(np.where(forest.is_leaf, forest.sample, -1), dtype=np.int32)
        div = np.ascontiguousarray(forest.divisions, dtype=np.uint32)
        h = lib().orc_place(self._h, forest.num_of_nodes, _p(parent, C.c_int32), _p(birth, C.c_double),
                            _p(sp, C.c_uint32), _p(sample, C.c_int32), _p(div, C.c_uint32),
                            len(forest.sample_names), n_pre_snv, pre_sbs, n_pre_id, pre_id, int(seed), flavour)
        if not h:
            raise RuntimeError(_err())
        return OraclePlaced(h)


class OraclePlaced:
    def __init__(self, h):
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_placed_destroy(self._h)
            self._h = None

    def table(self) -> dict:
        n = lib().orc_placed_count(self._h)
        t = {k: np.empty(n, dtype=np.uint32) for k in ("locus", "edge", "aux")}
        t.update({k: np.empty(n, dtype=np.uint8) for k in ("cls", "sig", "kind", "nature")})
        t["allele"] = np.empty(n, dtype=np.uint16)
        lib().orc_placed_copy(self._h, *(_p(t[k], C.c_uint32) for k in ("locus", "edge", "aux")),
                              _p(t["cls"], C.c_uint8), _p(t["sig"], C.c_uint8), _p(t["allele"], C.c_uint16),
                              _p(t["kind"], C.c_uint8), _p(t["nature"], C.c_uint8))
        return t

    def cna_table(self) -> dict:
        m = lib().orc_placed_cna_count(self._h)
        t = {k: np.empty(m, dtype=np.uint32) for k in ("node", "chr", "begin", "end", "allele", "src")}
        t.update({k: np.empty(m, dtype=np.uint8) for k in ("type", "driver")})
        lib().orc_placed_cna_copy(self._h, _p(t["node"], C.c_uint32), _p(t["type"], C.c_uint8),
                                  _p(t["chr"], C.c_uint32), _p(t["begin"], C.c_uint32), _p(t["end"], C.c_uint32),
                                  _p(t["allele"], C.c_uint32), _p(t["src"], C.c_uint32), _p(t["driver"], C.c_uint8))
        return t

    def node_classes(self, n_nodes):
        out = np.empty(n_nodes, dtype=np.uint32)
        nc, cm = C.c_uint32(), C.c_uint32()
        lib().orc_placed_node_classes(self._h, _p(out, C.c_uint32), C.byref(nc), C.byref(cm))
        return out, nc.value, cm.value

    def class_pieces(self, c):
        n = lib().orc_placed_class_pieces(self._h, c, None, None, None)
        inst, b, e = (np.empty(n, dtype=np.uint32) for _ in range(3))
        lib().orc_placed_class_pieces(self._h, c, _p(inst, C.c_uint32), _p(b, C.c_uint32), _p(e, C.c_uint32))
        return inst, b, e

    def carriers(self):
        """Per placed mutation the instances carrying it: (offsets, list)."""
        n = lib().orc_placed_carriers(self._h, None, None)
        off = np.empty(len(self.table()["locus"]) + 1, dtype=np.uint32)
        lst = np.empty(max(n, 1), dtype=np.uint32)
        lib().orc_placed_carriers(self._h, _p(off, C.c_uint32), _p(lst, C.c_uint32))
        return off, lst[:n]

    def inst_roots(self):
        n = lib().orc_placed_inst_roots(self._h, None)
        r = np.empty(n, dtype=np.uint8)
        lib().orc_placed_inst_roots(self._h, _p(r, C.c_uint8))
        return r

    def set_table(self, t: dict):
        arrs = [np.ascontiguousarray(t[k], dtype=d) for k, d in
                (("locus", np.uint32), ("edge", np.uint32), ("allele", np.uint16), ("kind", np.uint8))]
        if lib().orc_placed_set(self._h, len(arrs[0]), _p(arrs[0], C.c_uint32), _p(arrs[1], C.c_uint32),
                                _p(arrs[2], C.c_uint16), _p(arrs[3], C.c_uint8)):
            raise RuntimeError(_err())

    def sam_reads(self, cfg, seed, path) -> dict:
        """The replay's SAM reads: {(sample, chromosome index): [(FLAG, POS,
        CIGAR, mate POS, TLEN, SEQ), ...]} in file order (all strings)."""
        if lib().orc_sam(self._h, C.addressof(cfg), int(seed), str(path).encode()):
            raise RuntimeError(_err())
        out = {}
        with open(path) as fh:
            for line in fh:
                f = line.rstrip("\n").split("\t")
                out.setdefault((int(f[0]), int(f[1])), []).append(tuple(f[2:8]))
        return out

    def sequence(self, cfg, seed, flavour=0, fraction=1.0, threads=1):
        """cfg: a process_gb300._lib.SeqCfg (same layout as the oracle's)."""
        h = lib().orc_seq(self._h, C.addressof(cfg), int(seed), flavour, float(fraction), int(threads))
        if not h:
            raise RuntimeError(_err())
        try:
            s = lib().orc_seq_samples(h)
            n = lib().orc_placed_count(self._h)
            alt = np.empty((s, n), dtype=np.int32)
            dep = np.empty((s, n), dtype=np.int32)
            lib().orc_seq_copy(h, _p(alt, C.c_int32), _p(dep, C.c_int32))
            reads = lib().orc_seq_reads(h)
        finally:
            lib().orc_seq_destroy(h)
        return alt, dep, reads
