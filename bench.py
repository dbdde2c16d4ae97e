#!/usr/bin/env python
"""Benchmark: simulated reads/s (and placed mutations/s) of the GB300 path.

Workload: the full-scale configuration — synthetic 3.1 Gbp genome in 24
chromosomes (GC 41%), 3 samples x 1e4 leaves, 3 exposure epochs, 100x paired
150 bp reads, purity 0.7, error rate 1e-3, plus the normal sample.  One step =
place the mutations on the forest (new seed) and sequence all four samples.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

N > 1 runs one independent replica per GPU (the path does not exchange data
between instances), launched by torch.distributed.run.  ``--impl reference``
times the CPU restatement of the reference path (the oracle's std::mt19937_64
port) on the host cores, on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "reads/s + mutations placed/s on 1 GB300 vs host CPU; batched calib grad-evals/s"
WORKLOAD = ("full scale: 3.1 Gbp/24 chr GC 41%, 3 samples x 1e4 leaves, 3 epochs "
            "SNV {1.5e-8,3e-8,5e-8} indel 0.1x, 3 SBS + 2 ID signatures, 20 driver CNAs (1-50 Mbp, "
            "CN 0-4) + 1 WGD branch, 100x paired 150 bp, "
            "insert binomial(350, 10), purity 0.7, error 1e-3, + normal sample")
# algorithmic bytes of one simulated read and of one read-locus visit (alt+depth
# read-modify-write), the per-unit contract of the read kernel
BYTES_PER_READ = 38
BYTES_PER_SITE_HIT = 8
CPU_SAMPLE_SCALE = 0.01   # genome fraction of the CPU sample (31 Mbp over the 24 chromosomes)


def env_int(k, d):
    try:
        return int(os.environ.get(k, d))
    except ValueError:
        return d


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = Path(tempfile.mkstemp(suffix=".csv")[1])

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in self.path.read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def cpu_sample_workload():
    from process_gb300 import synth
    return synth.full_scale(seed=2, genome_scale=CPU_SAMPLE_SCALE)


def run_cpu(steps: int, warmup: int, threads: int, sample_desc: str):
    """Times the oracle's reference-engine port (std::mt19937_64) on the host."""
    import oracle
    from process_gb300.engine import seq_cfg
    oracle.build()
    w = cpu_sample_workload()
    e = oracle.OracleEngine.like(w)
    sp = np.array([e.species[(m, ep)] for m, ep in zip(w.forest.mutant, w.forest.epistate)], dtype=np.uint32)
    chr_index = {n: i for i, n in enumerate(w.genome.chr_names)}
    c, _ = seq_cfg(chr_index=lambda x: chr_index[x], **w.seq)
    reads = muts = 0
    t_place = t_seq = 0.0
    for s in range(warmup + steps):
        t0 = time.perf_counter()
        p = e.place(w.forest, sp, w.n_pre_snv, 0, w.n_pre_indel, 0, seed=100 + s, flavour=1)
        t1 = time.perf_counter()
        _, _, r = p.sequence(c, 200 + s, flavour=1, threads=threads)
        t2 = time.perf_counter()
        if s >= warmup:
            n = len(p.table()["locus"])
            reads += r
            muts += n
            t_place += t1 - t0
            t_seq += t2 - t1
    return {"reads_per_s": reads / (t_place + t_seq), "seq_reads_per_s": reads / t_seq,
            "mutations_placed_per_s": muts / t_place, "reads": reads, "mutations": muts,
            "seconds": t_place + t_seq, "threads": threads, "sample": sample_desc}


def cpu_model() -> str:
    """The host CPU's model name as the OS reports it (lscpu, else
    /proc/cpuinfo), for the CPU baseline's record."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def replica_rate(units: float, ms: list[float], world: int, device) -> tuple[float, float, list[float]]:
    """Whole-job throughput of independent replicas (no data-path
    collective): the units all ranks processed over the slowest rank's time.
    ``ms`` are this rank's timed spans (the first is the whole timed region);
    returns (rate per second, total units, the spans' maxima over ranks)."""
    import torch
    import torch.distributed as dist
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    t = torch.tensor([float(x) for x in ms], dtype=torch.float64, device=device)
    if world > 1:
        dist.all_reduce(u, op=dist.ReduceOp.SUM)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    spans = t.tolist()
    total = float(u[0])
    return total / (spans[0] / 1000.0), total, spans


def reference_arm(args):
    rank = env_int("RANK", 0)
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    desc = (f"oracle std::mt19937_64 port (oracle/oracle.cpp flavour 1) on {CPU_SAMPLE_SCALE:.0%} of the genome "
            "(31 Mbp over the same 24 chromosomes), full forest, 100x paired, purity 0.7, + normal; "
            "placement single-threaded, reads over all host threads")
    r = run_cpu(args.steps, args.warmup, threads, desc)
    line = {"metric": METRIC, "value": r["reads_per_s"], "unit": "reads/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * r["seconds"] / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD, "sample": desc},
            "secondary": {"mutations_placed_per_s": r["mutations_placed_per_s"],
                          "sequencing_reads_per_s": r["seq_reads_per_s"]},
            "cpu_baseline": {"value": r["reads_per_s"], "unit": "reads/s", "cores": threads, "kind": "port",
                             "sample": desc, "cpu_model": cpu_model()},
            "e2e": {"value": r["reads_per_s"], "unit": "reads/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def batch_bench(stream, n_inst: int, steps: int, warmup: int):
    """Batched replicates (256 forests on 100 Mbp): every instance placed and sequenced in
    one batch run (fused placement launches, one persistent read kernel under
    a CUDA graph, tile sizes from the autotuner).  Reads/s and placed
    mutations/s of whole runs, timed with CUDA events on the engine stream;
    beside them the plain path run instance by instance on the first 16."""
    import ctypes as C

    import torch

    from process_gb300 import _lib, synth
    from process_gb300.engine import sequence_counts
    w = synth.batch_256(seed=3, n_inst=n_inst)
    eng, b = synth.build_batch(w)
    _lib.check(_lib.lib().pg_engine_set_stream(eng._h, C.c_void_p(stream.cuda_stream)))
    seeds = np.arange(n_inst, dtype=np.uint64)
    tiles = b.autotune(seeds + 1, seeds + 2)
    for s in range(warmup):
        b.run(seeds + 100 * (s + 1), seeds + 100 * (s + 1) + 50)
    torch.cuda.synchronize()
    ms = place = seq = 0.0
    reads = muts = 0
    for s in range(steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.run(seeds + 10_000 * (s + 1), seeds + 10_000 * (s + 1) + 77)
        e1.record(stream)
        e1.synchronize()
        ms += e0.elapsed_time(e1)
        p_ms, s_ms = b.kernel_ms()
        place += p_ms
        seq += s_ms
        for i in range(n_inst):
            m, _, r = b.dims(i)
            reads += r
            muts += m
    # the plain path, instance by instance, on the first instances
    k = min(16, n_inst)
    from process_gb300 import MutationEngine
    torch.cuda.synchronize()
    plain_reads, plain_ms = 0, 0.0
    for i in range(k):
        e = MutationEngine(w.genome, w.sbs, w.ids, context_sampling=w.context_sampling)
        _lib.check(_lib.lib().pg_engine_set_stream(e._h, C.c_void_p(stream.cuda_stream)))
        e.add_mutant("A", {"SNV": float(w.snv[i]), "indel": float(w.indel[i])})
        e.add_exposure(0.0, {**{f"SBS{j + 1}": float(w.sbs_expo[i][j]) for j in range(3)},
                             **{f"ID{j + 1}": float(w.id_expo[i][j]) for j in range(2)}})
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        pf = e.place_mutations(w.forests[i], 0, 0, seed=int(seeds[i]) + 5)
        r = sequence_counts(pf, int(seeds[i]) + 6, tile_size=int(tiles[i]), **w.seq[i])
        e1.record(stream)
        e1.synchronize()
        plain_ms += e0.elapsed_time(e1)
        plain_reads += r.dims()[2]
    return {"workload": w.name, "instances": n_inst, "steps": steps, "warmup": warmup,
            "reads_per_s": reads / (ms / 1000.0), "mutations_placed_per_s": muts / (place / 1000.0),
            "ms_per_run": ms / steps, "place_ms_per_run": place / steps, "seq_ms_per_run": seq / steps,
            "reads_per_run": reads // steps, "mutations_per_run": muts // steps,
            "tile_sizes": {"min": int(tiles.min()), "median": int(np.median(tiles)), "max": int(tiles.max())},
            "plain_path_reads_per_s_first16": plain_reads / (plain_ms / 1000.0)}


def calibration_bench(world: int, n_rep: int = 512, n_sites: int = 100_000, steps: int = 200):
    """Batched calibration (512 replicates x 1e5 sites, Poisson depth means
    U(30, 200), K=4, 3 exposures): gradient evaluations per second of the
    batched kernels, of the graph-captured Adam loop, and of the per-instance
    path (one launch pair per replicate), plus the FP64 CPU oracle."""
    import torch

    import oracle.calib as oc
    from process_gb300 import calib
    rng = np.random.default_rng(5)
    d = calib.synthetic(n_rep, n_sites, rng.uniform(30, 200, n_rep), seed=5)
    b = calib.batch_of(d)
    s = b.stream
    p0 = torch.tensor(d.true_params + rng.normal(0, 0.3, d.true_params.shape), dtype=torch.float32, device="cuda")
    # batched gradient evaluations (every replicate per launch pair)
    for _ in range(3):
        b.nll_grad(p0)
    torch.cuda.synchronize()
    reps = 20
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ev[0].record(s)
    with torch.cuda.stream(s):
        for _ in range(reps):
            b.nll_grad(p0)
    ev[1].record(s)
    ev[1].synchronize()
    t_batched = ev[0].elapsed_time(ev[1]) / 1000.0 / reps
    # 200 Adam steps under one CUDA graph
    p = p0.clone()
    b.adam(p, steps)
    p = p0.clone()
    torch.cuda.synchronize()
    ev[0].record(s)
    with torch.cuda.stream(s):
        b.adam(p, steps)
    ev[1].record(s)
    ev[1].synchronize()
    t_adam = ev[0].elapsed_time(ev[1]) / 1000.0
    # per-instance path: one replicate per call (pg_calib_nll_grad_one),
    # stream-ordered with preallocated outputs and one synchronisation at
    # the end, timed with CUDA events on the handle's stream
    import ctypes as C
    n_one = min(64, n_rep)
    nll1 = torch.zeros(n_rep, dtype=torch.float32, device="cuda")
    grad1 = torch.zeros_like(p0)
    args = (C.c_void_p(p0.data_ptr()), C.c_void_p(nll1.data_ptr()), C.c_void_p(grad1.data_ptr()))
    for r in range(2):
        b.L.pg_calib_nll_grad_one(b._h, r, *args)
    torch.cuda.synchronize()
    ev[0].record(s)
    for r in range(n_one):
        b.L.pg_calib_nll_grad_one(b._h, r, *args)
    ev[1].record(s)
    ev[1].synchronize()
    t_one = ev[0].elapsed_time(ev[1]) / 1000.0 / n_one
    # FP64 CPU oracle, one replicate
    r0 = (d.alt[: n_sites], d.depth[: n_sites], d.cls[: n_sites], d.signatures, d.epoch_weight[0], d.phi[0], 4, 3)
    t0 = time.perf_counter()
    oc.nll_grad(d.true_params[0], *r0)
    t_cpu = time.perf_counter() - t0
    n_sites_total = int(d.site_off[-1])
    peak, _ = peaks()
    achieved = 12.0 * n_sites_total / t_batched / 1e9
    return {"workload": f"{n_rep} replicates x {n_sites} sites, depth Poisson(U(30,200)), K=4, J=3",
            "grad_evals_per_s_batched": world * n_rep / t_batched,
            "grad_evals_per_s_adam_graph": world * n_rep * steps / t_adam,
            "grad_evals_per_s_per_instance": world / t_one,
            "batched_over_per_instance": t_one / (t_batched / n_rep),
            "per_instance": "pg_calib_nll_grad_one per replicate, stream-ordered, one synchronisation at the end",
            "adam_200_steps_ms": t_adam * 1000.0,
            "cpu_fp64_grad_evals_per_s_1core": 1.0 / t_cpu,
            "roofline": {"kernel": "k_calib_sites+k_calib_epilogue", "bound": "hbm",
                         "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "per_unit": "12 B/site (alt, depth, class)"}}


def gpu_arm(args):
    import torch
    import torch.distributed as dist

    world = env_int("WORLD_SIZE", 1)
    rank = env_int("RANK", 0)
    local = env_int("LOCAL_RANK", 0)
    if world > 1:
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    import __graft_entry__
    __graft_entry__.build() if rank == 0 or world == 1 else None
    if world > 1:
        dist.barrier()
    from process_gb300 import _lib, synth
    from process_gb300.engine import sequence_counts
    import ctypes as C

    w = synth.full_scale(seed=2, genome_scale=args.genome_scale)
    eng = synth.build_engine(w)
    ims = (C.c_float * 4)()
    _lib.check(_lib.lib().pg_engine_index_ms(eng._h, ims))
    index_ms = {"sbs_count": ims[0], "sbs_emit": ims[1], "id_count": ims[2], "id_emit": ims[3],
                "total": sum(ims), "what": "device time of the engine's index build (count pass + scan, emit pass)"}
    # a dedicated (non-default) stream: the engine runs on it and the CUDA
    # events that time the steps are recorded on it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    _lib.check(_lib.lib().pg_engine_set_stream(eng._h, C.c_void_p(stream.cuda_stream)))
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    def launches():
        n = C.c_uint64()
        _lib.check(_lib.lib().pg_launch_count(C.byref(n)))
        return n.value

    seed0 = 1000 * rank
    for s in range(args.warmup):
        pf = eng.place_mutations(w.forest, w.n_pre_snv, w.n_pre_indel, seed=seed0 + s)
        sequence_counts(pf, seed0 + 500 + s, **w.seq)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    place_ms = seq_ms = read_kernel_ms = 0.0
    reads = muts = 0
    last = None
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        n0 = launches()
        wall0 = time.perf_counter()
        for s in range(args.steps):
            flush.fill_(s & 0xFF)                 # evict L2 between steps
            e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            e0.record(stream)
            pf = eng.place_mutations(w.forest, w.n_pre_snv, w.n_pre_indel, seed=seed0 + 10_000 + s)
            e1.record(stream)
            res = sequence_counts(pf, seed0 + 20_000 + s, **w.seq)
            e2.record(stream)
            e2.synchronize()
            place_ms += e0.elapsed_time(e1)
            seq_ms += e1.elapsed_time(e2)
            read_kernel_ms += res.kernel_ms()
            reads += res.dims()[2]
            muts += pf.num_of_mutations
            last = (pf, res)
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
        n_launch = launches() - n0
    value, _, t = replica_rate(reads, [place_ms + seq_ms, place_ms, seq_ms], world, "cuda")
    _, all_muts, _ = replica_rate(muts, [1.0], world, "cuda")
    step_ms = t[0] / args.steps
    # read-locus visits of the last step, for the roofline's algorithmic bytes
    pf, res = last
    rr = C.c_uint32()
    _lib.check(_lib.lib().pg_placed_redraw_rounds(pf._h, C.byref(rr)))
    redraw_rounds = rr.value
    alt, dep = res.counts()
    site_hits = int(dep.astype(np.int64).sum())
    reads_last = res.dims()[2]
    kms = res.kernel_ms()
    alg_bytes = BYTES_PER_READ * reads_last + BYTES_PER_SITE_HIT * site_hits
    peak, peak_kind = peaks()
    achieved = alg_bytes / (kms / 1000.0) / 1e9
    traffic = None
    tf = ROOT / "profiles" / "k_reads_traffic.json"
    if tf.exists():
        d = json.loads(tf.read_text())
        # traffic per read scaled to this launch (traffic grows with reads)
        traffic = d.get("dram_bytes_per_read", 0.0) * reads_last if d.get("dram_bytes_per_read") else None

    # end to end through the public API from host buffers: forest upload,
    # placement, sequencing and the alt/depth tables back to host memory
    e2e_steps = min(args.steps, 3)
    forest_bytes = w.forest.num_of_nodes * (4 + 8 + 4 + 4 + 4)
    # the result comes back into page-locked host memory (sized with
    # headroom for the step-to-step spread of the mutation count): the
    # observed rows, compacted on the device, as the reference's result frame
    # keeps them by default; beside it the same with the full alt/depth tables
    s_n, m_n, _ = res.dims()
    m_cap = int(m_n * 1.05) + 1024
    pinned = [torch.empty(s_n * m_cap, dtype=torch.int32, pin_memory=True).numpy() for _ in range(2)]
    pinned_idx = torch.empty(m_cap, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)

    def e2e_run(full: bool, seed_base: int):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        n_reads = n_bytes = 0
        for s in range(e2e_steps):
            pf2 = eng.place_mutations(w.forest, w.n_pre_snv, w.n_pre_indel, seed=seed_base + s)
            r2 = sequence_counts(pf2, seed_base + 10_000 + s, **w.seq)
            s2, m2, n_r = r2.dims()
            if m2 > m_cap:
                arrays = r2.counts() if full else r2.observed()
            elif full:
                arrays = r2.counts(tuple(b[:s2 * m2].reshape(s2, m2) for b in pinned))
            else:
                arrays = r2.observed((pinned_idx, pinned[0], pinned[1]))
            n_reads += n_r
            n_bytes += sum(x.nbytes for x in arrays)
        torch.cuda.synchronize()
        rate, _, _ = replica_rate(n_reads, [1000.0 * (time.perf_counter() - t0)], world, "cuda")
        return rate, n_bytes // max(1, e2e_steps)

    e2e_value, d2h_step = e2e_run(False, seed0 + 30_000)
    e2e_full_value, d2h_full_step = e2e_run(True, seed0 + 50_000)

    # the result data frame of the last step (simulate_seq's "mutations"):
    # built in C++ by the library, then turned into numpy columns
    from process_gb300.engine import _result_frame
    names = list(w.forest.sample_names) + ["normal_sample"]
    t0 = time.perf_counter()
    nrow = C.c_uint64()
    _lib.check(_lib.lib().pg_seq_result_frame(res._h, pf._h, 0, C.byref(nrow)))
    t_frame_lib = time.perf_counter() - t0
    t0 = time.perf_counter()
    frame = _result_frame(res, pf, False, names)
    t_frame_all = time.perf_counter() - t0
    frame_info = {"rows": int(nrow.value), "library_build_s": t_frame_lib, "build_and_columns_s": t_frame_all,
                  "columns": len(frame)}

    cal = None if args.no_calibration else calibration_bench(world, args.calib_replicates)
    batch = None if args.no_batch else batch_bench(stream, args.batch_instances, max(1, min(args.steps, 3)),
                                                   max(1, min(args.warmup, 2)))

    line = None
    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline:
            threads = os.cpu_count() or 1
            desc = (f"oracle std::mt19937_64 port on {CPU_SAMPLE_SCALE:.0%} of the genome (31 Mbp over the same "
                    "24 chromosomes), full forest, 100x paired, purity 0.7, + normal, 1 step")
            r = run_cpu(1, 0, threads, desc)
            r1 = run_cpu(1, 0, 1, desc)
            cpu = {"value": r["reads_per_s"], "unit": "reads/s", "cores": threads, "kind": "port", "sample": desc,
                   "single_core_value": r1["reads_per_s"],
                   "mutations_placed_per_s": r["mutations_placed_per_s"], "cpu_model": cpu_model()}
        clocks = clk.summary()
        line = {
            "metric": METRIC, "value": value, "unit": "reads/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "reads_per_step_per_gpu": reads // args.steps,
                       "mutations_per_step_per_gpu": muts // args.steps,
                       "l2": "flushed between steps (256 MiB write); record and count tables exceed L2",
                       "parallelism": f"replicas x{world}"},
            "secondary": {"mutations_placed_per_s": all_muts / (t[1] / 1000.0),
                          "sequencing_reads_per_s": value * t[0] / t[2],
                          "place_ms_per_step": float(t[1]) / args.steps, "seq_ms_per_step": float(t[2]) / args.steps,
                          "bracket_wall_s": wall,
                          "result_frame": frame_info,
                          "index_build_ms": index_ms,
                          "redraw_rounds_last_step": redraw_rounds,
                          "e2e_full_tables": {"value": e2e_full_value, "unit": "reads/s",
                                              "d2h_bytes_per_step": d2h_full_step}},
            "roofline": {"kernel": "k_reads", "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                         "algorithmic_bytes": alg_bytes, "kernel_ms": kms,
                         "per_unit": f"{BYTES_PER_READ} B/read + {BYTES_PER_SITE_HIT} B/site hit"},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "reads/s", "h2d_bytes_per_step": forest_bytes,
                    "d2h_bytes_per_step": d2h_step, "result": "observed rows (alt > 0 in some sample), "
                    "compacted on the device: indices + alt + depth"},
            "gpu_launches": n_launch,
            "calibration": cal,
            "batched": batch,
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-calibration", action="store_true")
    ap.add_argument("--calib-replicates", type=int, default=512)
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--batch-instances", type=int, default=256)
    ap.add_argument("--genome-scale", type=float, default=1.0,
                    help="fraction of the 3.1 Gbp genome (profiling runs on smaller cases; 1.0 for the bench)")
    args = ap.parse_args()
    if args.impl == "reference":
        return reference_arm(args)
    return gpu_arm(args)


if __name__ == "__main__":
    sys.exit(main())
