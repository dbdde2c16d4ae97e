"""The batched form: many forests, rates, exposures and coverages placed and
sequenced together (persistent read kernel under a CUDA graph).  Every
instance must equal, bit for bit, the plain path run on it alone with the
same seeds and tile size (the plain path is itself checked against the
oracle)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _instances(seed, n):
    from process_gb300 import GenomeSpec, synth
    rng = np.random.default_rng(seed)
    genome = GenomeSpec(["1", "2", "3"], [400_000, 250_000, 150_000], seed=seed, gc=0.45)
    sbs = synth.dirichlet_signatures(rng, 3, 96, 0.5, "SBS")
    ids = synth.dirichlet_signatures(rng, 2, 83, 0.5, "ID")
    insts = []
    for i in range(n):
        leaves = int(rng.integers(40, 400))
        f = synth.birth_forest(leaves, 1 + i % 2, seed * 100 + i, subclone=None, mutant="A")
        cfg = dict(coverage=float(rng.uniform(10, 60)), read_size=150, insert_size_mean=350 if i % 3 else 0,
                   insert_size_stddev=10, error_rate=1e-3, purity=float(rng.uniform(0.5, 1.0)),
                   with_normal_sample=bool(i % 2))
        insts.append(dict(forest=f, snv=float(10 ** rng.uniform(-7.5, -6.5)), indel=float(10 ** rng.uniform(-8.5, -7.5)),
                          sbs=rng.dirichlet(np.ones(3)), ids=rng.dirichlet(np.ones(2)), cfg=cfg,
                          n_pre=(int(rng.integers(0, 20)), int(rng.integers(0, 5)))))
    return genome, sbs, ids, insts


def _plain(genome, sbs, ids, inst, tile, place_seed, seq_seed, context_sampling=100):
    from process_gb300 import MutationEngine
    from process_gb300.engine import sequence_counts
    eng = MutationEngine(genome, sbs, ids, context_sampling=context_sampling)
    eng.add_mutant("A", {"SNV": inst["snv"], "indel": inst["indel"]})
    eng.add_exposure(0.0, {**{f"SBS{k + 1}": float(inst["sbs"][k]) for k in range(3)},
                           **{f"ID{k + 1}": float(inst["ids"][k]) for k in range(2)}})
    pf = eng.place_mutations(inst["forest"], inst["n_pre"][0], inst["n_pre"][1], seed=place_seed)
    alt, dep = sequence_counts(pf, seq_seed, tile_size=int(tile), **inst["cfg"]).counts()
    return pf.table(), alt, dep


def _batch(genome, sbs, ids, insts):
    from process_gb300 import Batch, MutationEngine
    eng = MutationEngine(genome, sbs, ids)
    b = Batch(eng, [x["forest"] for x in insts], [x["snv"] for x in insts], [x["indel"] for x in insts],
              np.array([x["sbs"] for x in insts]), np.array([x["ids"] for x in insts]), [x["cfg"] for x in insts],
              n_pre_snv=[x["n_pre"][0] for x in insts], n_pre_indel=[x["n_pre"][1] for x in insts])
    return eng, b


def _check(b, genome, sbs, ids, insts, pseeds, sseeds, context_sampling=100):
    tiles = b.tile_sizes
    for i, inst in enumerate(insts):
        t, alt, dep = _plain(genome, sbs, ids, inst, tiles[i], int(pseeds[i]), int(sseeds[i]), context_sampling)
        bt = b.table(i)
        for k in ("locus", "edge", "aux", "cls", "sig", "allele", "kind", "nature"):
            np.testing.assert_array_equal(bt[k], t[k], err_msg=f"instance {i} {k}")
        balt, bdep = b.counts(i)
        np.testing.assert_array_equal(bdep, dep, err_msg=f"instance {i} depth")
        np.testing.assert_array_equal(balt, alt, err_msg=f"instance {i} alt")


def test_batch_equals_plain_per_instance(gpu_lib):
    genome, sbs, ids, insts = _instances(3, 7)
    eng, b = _batch(genome, sbs, ids, insts)
    pseeds, sseeds = np.arange(7) + 100, np.arange(7) + 900
    b.run(pseeds, sseeds)
    assert sum(b.dims(i)[0] for i in range(7)) > 300
    _check(b, genome, sbs, ids, insts, pseeds, sseeds)
    # a second run replays the captured sequencing graph with new seeds
    pseeds2, sseeds2 = pseeds + 7, sseeds + 7
    b.run(pseeds2, sseeds2)
    _check(b, genome, sbs, ids, insts, pseeds2, sseeds2)


def test_batch_autotune_and_uneven_tiles(gpu_lib):
    genome, sbs, ids, insts = _instances(5, 5)
    eng, b = _batch(genome, sbs, ids, insts)
    pseeds, sseeds = np.arange(5) + 10, np.arange(5) + 20
    chosen = b.autotune(pseeds, sseeds)
    assert np.all(chosen % 64 == 0) and np.all(chosen >= 256)
    np.testing.assert_array_equal(b.tile_sizes, chosen)
    b.tile_sizes = [256, 512, 1024, 2048, 4096]       # uneven tiles across instances
    b.run(pseeds, sseeds)
    _check(b, genome, sbs, ids, insts, pseeds, sseeds)


def test_batch_at_batched_workload_sizes(gpu_lib):
    """32 instances drawn like the 256-instance batched workload (forests of
    1e3-5e4 leaves, log-uniform; SNV 1e-8-1e-7; coverage 30-200x; every
    position indexed) on a 10 Mbp genome: each instance equals the plain
    path run alone."""
    from process_gb300 import synth
    n = 32
    w = synth.batch_256(seed=11, n_inst=n, genome_len=10_000_000)
    leaves = [int(np.sum(np.asarray(f.is_leaf))) for f in w.forests]
    assert min(leaves) >= 1_000 and max(leaves) > 20_000
    eng, b = synth.build_batch(w)
    pseeds, sseeds = np.arange(n) + 300, np.arange(n) + 700
    b.run(pseeds, sseeds)
    insts = [dict(forest=w.forests[i], snv=float(w.snv[i]), indel=float(w.indel[i]), sbs=w.sbs_expo[i],
                  ids=w.id_expo[i], cfg=w.seq[i], n_pre=(0, 0)) for i in range(n)]
    assert sum(b.dims(i)[0] for i in range(n)) > 10_000
    _check(b, w.genome, w.sbs, w.ids, insts, pseeds, sseeds, context_sampling=w.context_sampling)
