"""The allocation-free class-count entry point (pg_index_counts_noalloc).

Some callers cannot allocate device memory themselves: a host framework
whose pooling allocator owns all device memory, code running while a stream
is captured into a CUDA graph, or a latency-bound loop that cannot take the
synchronisation an allocation may cause.  pg_index_counts_noalloc serves them
from a fixed array inside the library; this test checks it through the C-ABI
against the counts the engine computes with its own buffers, on two calls in
a row (the second call reuses the array the first one filled).

The file name makes pytest collect it last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _packed_words(codes: np.ndarray) -> np.ndarray:
    pad = (-len(codes)) % 16
    c = np.concatenate([codes.astype(np.uint32), np.zeros(pad, np.uint32)]).reshape(-1, 16)
    return (c << (2 * np.arange(16, dtype=np.uint32))).sum(axis=1, dtype=np.uint64).astype(np.uint32)


def test_noalloc_counts_match_engine_twice(gpu_lib):
    import torch

    from process_gb300 import GenomeSpec, MutationEngine, _lib

    g = GenomeSpec(["1", "2", "3"], [1_500_001, 700_000, 2_345], seed=31, gc=0.41)
    eng = MutationEngine(g, context_sampling=1, max_repetition_storage=1000)
    info = eng.index_info()
    words = torch.from_numpy(_packed_words(eng.read_genome()).view(np.int32)).cuda()
    off = np.concatenate([[0], np.cumsum(np.asarray(g.chr_lengths, dtype=np.int64))]).astype(np.uint32)
    chr_off = torch.from_numpy(off.view(np.int32)).cuda()
    stream = torch.cuda.current_stream()
    lb = _lib.lib()

    def counts(which):
        out = torch.full((32 if which == 0 else 83,), -1, dtype=torch.int64, device="cuda")
        _lib.check(lb.pg_index_counts_noalloc(which, C.c_void_p(words.data_ptr()), g.total,
                                              C.c_void_p(chr_off.data_ptr()), len(g.chr_lengths),
                                              C.c_void_p(out.data_ptr()), C.c_void_p(stream.cuda_stream)))
        stream.synchronize()
        return out.cpu().numpy().astype(np.uint64)

    for _ in range(2):    # two calls in a row per class family
        np.testing.assert_array_equal(counts(0), info["ctx_total"])
        np.testing.assert_array_equal(counts(1), info["id_total"])


def test_noalloc_rejects_genomes_above_its_array(gpu_lib):
    import torch

    from process_gb300 import DomainError, _lib

    words = torch.zeros(16, dtype=torch.int32, device="cuda")
    off = torch.tensor([0, 8_388_609], dtype=torch.int32, device="cuda")
    out = torch.zeros(32, dtype=torch.int64, device="cuda")
    st = _lib.lib().pg_index_counts_noalloc(0, C.c_void_p(words.data_ptr()), 8_388_609, C.c_void_p(off.data_ptr()),
                                            1, C.c_void_p(out.data_ptr()), None)
    assert st == _lib.PG_ERR_DOMAIN
    with pytest.raises(DomainError):
        _lib.check(st)
