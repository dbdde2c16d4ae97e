"""Test-side restatement of the "PhylogeneticForest" getters and of the
result data frame in numpy, over the library's raw tables
(pg_placed_copy, pg_placed_class_copy, pg_placed_lineage_copy and the
alt/depth tables).  The library builds these frames in C++
(pg_placed_cell_mutations, pg_placed_cell_fragmentation,
pg_placed_bulk_fragmentation, pg_placed_samples_info, pg_seq_result_frame);
the tests compare the two.  Test infrastructure only."""
from __future__ import annotations

import ctypes as C

import numpy as np

from process_gb300 import _lib
from process_gb300._lib import DomainError, check, lib, ptr
from process_gb300.engine import BASES, NATURES


def ref_alt(pf, t: dict, rows: np.ndarray | None = None) -> tuple[np.ndarray, np.ndarray]:
    """ref / alt strings of the rows (all when None): one base gather for
    the SNVs and one for the indels' anchor windows."""
    eng = pf.engine
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

def cause(pf, t: dict, rows: np.ndarray | None = None) -> np.ndarray:
    """Signature name of each row (None for drivers and unknown indices)."""
    rows = np.arange(len(t["sig"])) if rows is None else np.asarray(rows, dtype=np.int64)
    sig, kind = t["sig"][rows].astype(np.int64), t["kind"][rows]
    out = np.full(len(rows), None, dtype=object)
    for k in np.unique(kind):
        names = list(pf.engine.sig_names[int(k)]) if int(k) < len(pf.engine.sig_names) else []
        table = np.array(names + [None], dtype=object)
        m = kind == k
        sk = sig[m]
        out[m] = table[np.where((sk == 0xFF) | (sk >= len(names)), len(names), sk)]
    return out

def chr_pos(pf, locus: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    off = pf.engine.chr_off
    ci = np.searchsorted(off, locus.astype(np.uint64), side="right") - 1
    names = np.array(pf.engine.chr_names, dtype=object)[ci]
    return names, (locus.astype(np.int64) - off[ci].astype(np.int64) + 1)

def lineage(pf) -> dict:
    """Instance lineage chains and every mutation's order key
    (pg_placed_lineage_copy)."""
    if getattr(pf, "_lin_cache", None) is None:
        ni, nl = C.c_uint32(), C.c_uint32()
        check(lib().pg_placed_lineage_dims(pf._h, C.byref(ni), C.byref(nl)))
        d = {"off": np.zeros(ni.value + 1, np.uint32), "anc": np.zeros(max(nl.value, 1), np.uint16),
             "key": np.zeros(max(nl.value, 1), np.uint64),
             "order": np.zeros(max(pf.num_of_mutations, 1), np.uint64)}
        check(lib().pg_placed_lineage_copy(pf._h, ptr(d["off"], C.c_uint32), ptr(d["anc"], C.c_uint16),
                                           ptr(d["key"], C.c_uint64), ptr(d["order"], C.c_uint64)))
        d["n_instances"] = ni.value
        pf._lin_cache = d
    return pf._lin_cache

def cell_rows(pf, leaf: int) -> tuple[np.ndarray, np.ndarray]:
    """(mutation rows, allele instance) of the mutations sampled cell
    ``leaf`` holds: those on its root path, once per allele instance of
    its genome at the locus that carries them (the placed instance, and
    the copies of it made after the mutation), in mutation order."""
    t = pf.table()
    idx = np.nonzero(pf.leaf_carriers(leaf))[0]
    lin = lineage(pf)
    cls, n_classes, _ = pf.node_classes()
    if n_classes <= 1 and lin["n_instances"] <= 2:       # no copy-number event
        return idx, t["allele"][idx].astype(np.int64)
    d = classes(pf)
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

def classes(pf) -> dict:
    """Genotype classes as segments with each instance's germline allele."""
    if getattr(pf, "_cls_cache", None) is None:
        nc, ns, nl, ni = (C.c_uint32() for _ in range(4))
        check(lib().pg_placed_class_dims(pf._h, C.byref(nc), C.byref(ns), C.byref(nl), C.byref(ni)))
        d = {"seg_off": np.empty(nc.value + 1, np.uint32), "start": np.empty(ns.value, np.uint32),
             "end": np.empty(ns.value, np.uint32), "ioff": np.empty(ns.value, np.uint32),
             "icnt": np.empty(ns.value, np.uint32), "list": np.empty(max(nl.value, 1), np.uint16),
             "root": np.empty(max(ni.value, 1), np.uint8)}
        check(lib().pg_placed_class_copy(pf._h, ptr(d["seg_off"], C.c_uint32), ptr(d["start"], C.c_uint32),
                                         ptr(d["end"], C.c_uint32), ptr(d["ioff"], C.c_uint32),
                                         ptr(d["icnt"], C.c_uint32), ptr(d["list"], C.c_uint16),
                                         ptr(d["root"], C.c_uint8)))
        # copies of germline allele 1 per segment (the rest descend from allele 0)
        roots = d["root"][d["list"][:max(nl.value, 1)]].astype(np.int64)
        csum = np.concatenate([[0], np.cumsum(roots)])
        d["a1"] = (csum[d["ioff"] + d["icnt"]] - csum[d["ioff"]]).astype(np.int64)
        d["a0"] = d["icnt"].astype(np.int64) - d["a1"]
        d["n_classes"] = nc.value
        pf._cls_cache = d
    return pf._cls_cache

def class_fragments(pf, c: int) -> tuple[np.ndarray, np.ndarray, np.ndarray, np.ndarray]:
    """(absolute begin, end (half-open), copies of allele 0, of allele 1) of
    the maximal stretches of class c with one allelic type, chromosome by
    chromosome (uncovered stretches have type (0, 0))."""
    d = classes(pf)
    lo, hi = int(d["seg_off"][c]), int(d["seg_off"][c + 1])
    st, en = d["start"][lo:hi].astype(np.int64), d["end"][lo:hi].astype(np.int64)
    off = pf.engine.chr_off.astype(np.int64)
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

def frag_rows(pf, b, e, a0, a1):
    off = pf.engine.chr_off.astype(np.int64)
    ci = np.searchsorted(off, b, side="right") - 1
    names = np.array(pf.engine.chr_names, dtype=object)[ci]
    return names, b - off[ci] + 1, e - off[ci], np.maximum(a0, a1), np.minimum(a0, a1)

def get_cell_allelic_fragmentation(pf) -> dict:
    """Columns cell_id, chr, begin, end, major, minor: every sampled cell's
    genome cut into stretches of one allelic type (copies of the two
    germline alleles; major = the larger), src/phylogenetic_forest.cpp:867-927."""
    f = pf.forest
    cls, _, _ = pf.node_classes()
    leaves = np.nonzero(f.is_leaf & (f.sample >= 0))[0]
    per = {}
    cols = {k: [] for k in ("cell_id", "chr", "begin", "end", "major", "minor")}
    for lf in leaves:
        c = int(cls[lf])
        if c not in per:
            per[c] = frag_rows(pf, *class_fragments(pf, c))
        names, b, e, mj, mn = per[c]
        cols["cell_id"].append(np.full(len(b), f.cell_id[lf]))
        cols["chr"].append(names); cols["begin"].append(b); cols["end"].append(e)
        cols["major"].append(mj); cols["minor"].append(mn)
    return {k: (np.concatenate(v) if v else np.array([])) for k, v in cols.items()}

def get_bulk_allelic_fragmentation(pf, sample_name: str | None = None) -> dict:
    """Columns chr, begin, end, major, minor, ratio: for every stretch of
    the genome on which the sampled cells (of one sample, or all) keep
    their allelic types, each type with the fraction of cells showing it
    (src/phylogenetic_forest.cpp:767-820)."""
    f = pf.forest
    cls, _, _ = pf.node_classes()
    sel = f.is_leaf & (f.sample >= 0)
    if sample_name is not None:
        if sample_name not in f.sample_names:
            raise DomainError(_lib.PG_ERR_DOMAIN, f'Unknown sample "{sample_name}".')
        sel &= f.sample == f.sample_names.index(sample_name)
    leaf_cls, counts = np.unique(cls[sel], return_counts=True)
    n_cells = float(counts.sum())
    frags = [class_fragments(pf, int(c)) for c in leaf_cls]
    cuts = np.unique(np.concatenate([fr[0] for fr in frags] + [fr[1] for fr in frags]))
    b, e = cuts[:-1], cuts[1:]
    keep = np.ones(len(b), dtype=bool)
    types = []
    for (fb, fe, f0, f1) in frags:
        k = np.searchsorted(fb, b, side="right") - 1
        types.append((f0[k], f1[k]))
    # merge neighbouring stretches with the same type in every class and chromosome
    off = pf.engine.chr_off.astype(np.int64)
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
        names, bb, ee, _, _ = frag_rows(pf, np.array([b[i0]]), np.array([e[i1]]), np.zeros(1), np.zeros(1))
        for (x0, x1), n in sorted(agg.items()):
            cols["chr"].append(names[0]); cols["begin"].append(int(bb[0])); cols["end"].append(int(ee[0]))
            cols["major"].append(max(x0, x1)); cols["minor"].append(min(x0, x1)); cols["ratio"].append(n / n_cells)
    return {k: np.array(v, dtype=object if k == "chr" else None) for k, v in cols.items()}

def result_frame(pf: "PhylogeneticForest", idx: np.ndarray, alt: np.ndarray, dep: np.ndarray,
                  sample_names: list[str]) -> dict:
    """The wide data frame of get_result_dataframe (src/seq_simulation.cpp:142-181)
    over the rows idx (mutation indices, ascending; alt / dep are their
    [sample][row] tables), merged by (chr, pos, ref, alt) in the order of
    each SID's first row: occurrences add, the coverage is the first row's,
    causes and classes are the sorted unions."""
    t = pf.table()
    idx = np.asarray(idx, dtype=np.int64)
    ref, altb = ref_alt(pf, t, idx)
    cause_all = cause(pf, t, idx)
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
    chrn, pos = chr_pos(pf, loc[first] if ng else loc[:0])
    causes = cause_all[first].copy()
    classes = nat[first].astype(object)
    for g in np.nonzero(sizes > 1)[0]:
        members = np.nonzero(group == g)[0]
        causes[g] = ";".join(sorted({c for c in cause_all[members] if c is not None})) or None
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


def result_rows(res: "SeqResult", include_non_sequenced: bool, present: np.ndarray):
    """Rows of the result frame: the observed rows compacted on the device,
    or (include_non_sequenced_mutations) those plus every mutation present
    in a sequenced sample's cells, from the full tables."""
    if not include_non_sequenced:
        return res.observed()
    alt, dep = res.counts()
    idx = np.nonzero((alt.sum(axis=0) > 0) | present)[0]
    return idx, alt[:, idx], dep[:, idx]


def presence(pf: "PhylogeneticForest", n_samples_seq: int, with_normal: bool, pre_in_normal: bool) -> np.ndarray:
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


