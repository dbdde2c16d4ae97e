"""ctypes binding of ``libprocess_gb300.so`` (the C-ABI of include/process_gb300.h).

The library is built in-tree (``process_gb300/_lib``).  Loading fails loudly when
it is missing: there is no CPU fallback for any operation of this package.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_LIB = None
LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libprocess_gb300.so"

PG_OK, PG_ERR_DOMAIN, PG_ERR_RUNTIME, PG_ERR_CUDA, PG_ERR_NOMEM, PG_ERR_UNSUPPORTED = range(6)


class ProcessError(RuntimeError):
    """A failed library call (the reference raises R errors for the same cases)."""

    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status


class DomainError(ProcessError, ValueError):
    """Invalid argument (std::domain_error in the reference)."""


class UnsupportedError(ProcessError, NotImplementedError):
    """A feature this library does not build."""


class SeqCfg(C.Structure):
    _fields_ = [
        ("coverage", C.c_double), ("read_size", C.c_uint32), ("insert_size_mean", C.c_uint32),
        ("insert_size_stddev", C.c_uint32), ("insert_model", C.c_int), ("error_rate", C.c_double),
        ("purity", C.c_double), ("with_normal_sample", C.c_int), ("preneoplastic_in_normal", C.c_int),
        ("normal_only", C.c_int), ("n_chr_sel", C.c_uint32), ("chr_sel", C.POINTER(C.c_uint32)),
        ("tile_size", C.c_uint32),
    ]


class SamCfg(C.Structure):
    _fields_ = [
        ("output_dir", C.c_char_p), ("filename_prefix", C.c_char_p), ("template_name_prefix", C.c_char_p),
        ("update", C.c_int), ("sample_names", C.POINTER(C.c_char_p)), ("chr_names", C.POINTER(C.c_char_p)),
    ]


class GenomeDesc(C.Structure):
    _fields_ = [
        ("n_chr", C.c_uint32), ("chr_lengths", C.POINTER(C.c_uint32)), ("bases", C.POINTER(C.c_uint8)),
        ("synthetic_seed", C.c_uint64), ("synthetic_gc", C.c_double), ("context_sampling", C.c_uint32),
        ("max_repetition_storage", C.c_uint32), ("n_avoid", C.c_uint32), ("avoid_chr", C.POINTER(C.c_uint32)),
        ("avoid_begin", C.POINTER(C.c_uint32)), ("avoid_len", C.POINTER(C.c_uint32)), ("index_cache_dir", C.c_char_p),
    ]


P = C.c_void_p
u8p, u32p, i32p, u64p, f64p, f32p = (C.POINTER(t) for t in (C.c_uint8, C.c_uint32, C.c_int32, C.c_uint64,
                                                               C.c_double, C.c_float))

_PROTOS = {
    "pg_last_error": (C.c_char_p, []),
    "pg_version": (C.c_char_p, []),
    "pg_device_count": (C.c_int, [C.POINTER(C.c_int)]),
    "pg_engine_create": (C.c_int, [C.POINTER(GenomeDesc), C.POINTER(P)]),
    "pg_engine_destroy": (C.c_int, [P]),
    "pg_engine_set_stream": (C.c_int, [P, C.c_void_p]),
    "pg_launch_count": (C.c_int, [u64p]),
    "pg_index_counts_noalloc": (C.c_int, [C.c_int, C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint32, C.c_void_p,
                                          C.c_void_p]),
    "pg_engine_genome_info": (C.c_int, [P, u64p, u64p, u64p, u32p, u32p]),
    "pg_engine_read_genome": (C.c_int, [P, C.c_uint64, C.c_uint64, u8p]),
    "pg_engine_gather_bases": (C.c_int, [P, C.c_uint64, u32p, u8p]),
    "pg_engine_read_index": (C.c_int, [P, C.c_int, C.c_uint32, u32p, C.c_uint32, u32p]),
    "pg_engine_set_signatures": (C.c_int, [P, C.c_int, C.c_uint32, f64p]),
    "pg_engine_add_exposure": (C.c_int, [P, C.c_int, C.c_double, f64p]),
    "pg_engine_set_species_rates": (C.c_int, [P, C.c_uint32, C.c_double, C.c_double, C.c_double]),
    "pg_engine_set_species_epoch_rates": (C.c_int, [P, C.c_uint32, C.c_uint32, f64p, f64p]),
    "pg_engine_set_species_mutant": (C.c_int, [P, C.c_uint32, C.c_uint32]),
    "pg_engine_add_driver_sid": (C.c_int, [P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_char_p, C.c_char_p,
                                           C.c_int32]),
    "pg_engine_add_driver_cna": (C.c_int, [P, C.c_uint32, C.c_int, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int32,
                                           C.c_int32]),
    "pg_engine_add_driver_wgd": (C.c_int, [P, C.c_uint32]),
    "pg_engine_set_infinite_sites": (C.c_int, [P, C.c_int]),
    "pg_engine_get_infinite_sites": (C.c_int, [P, C.POINTER(C.c_int)]),
    "pg_forest_create": (C.c_int, [C.c_uint32, i32p, f64p, u32p, i32p, u32p, C.c_uint32, C.POINTER(P)]),
    "pg_forest_destroy": (C.c_int, [P]),
    "pg_place_mutations": (C.c_int, [P, P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64,
                                     C.POINTER(P)]),
    "pg_placed_destroy": (C.c_int, [P]),
    "pg_placed_count": (C.c_int, [P, u64p]),
    "pg_placed_copy": (C.c_int, [P, u32p, u32p, u32p, u8p, u8p, C.POINTER(C.c_uint16), u8p, u8p]),
    "pg_placed_cna_count": (C.c_int, [P, u64p]),
    "pg_placed_cna_copy": (C.c_int, [P, u32p, u8p, u32p, u32p, u32p, u32p, u32p, u8p]),
    "pg_placed_node_classes": (C.c_int, [P, u32p, u32p, u32p]),
    "pg_placed_class_dims": (C.c_int, [P, u32p, u32p, u32p, u32p]),
    "pg_placed_class_copy": (C.c_int, [P, u32p, u32p, u32p, u32p, u32p, C.POINTER(C.c_uint16), u8p]),
    "pg_engine_add_passenger_cna": (C.c_int, [P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int]),
    "pg_engine_set_avoid_homozygous_losses": (C.c_int, [P, C.c_int]),
    "pg_placed_kernel_ms": (C.c_int, [P, f32p]),
    "pg_placed_redraw_rounds": (C.c_int, [P, u32p]),
    "pg_engine_index_ms": (C.c_int, [P, f32p]),
    "pg_placed_set_samples": (C.c_int, [P, C.c_uint32, i32p]),
    "pg_placed_lineage_dims": (C.c_int, [P, u32p, u32p]),
    "pg_placed_lineage_copy": (C.c_int, [P, u32p, C.POINTER(C.c_uint16), u64p, u64p]),
    "pg_simulate_seq": (C.c_int, [P, C.POINTER(SeqCfg), C.c_uint64, C.POINTER(P)]),
    "pg_seq_result_destroy": (C.c_int, [P]),
    "pg_seq_result_dims": (C.c_int, [P, u32p, u64p, u64p]),
    "pg_seq_result_copy": (C.c_int, [P, i32p, i32p]),
    "pg_seq_result_kernel_ms": (C.c_int, [P, f32p]),
    "pg_seq_result_tile_size": (C.c_int, [P, u32p]),
    "pg_seq_result_active": (C.c_int, [P, u64p]),
    "pg_seq_result_copy_active": (C.c_int, [P, u32p, i32p, i32p]),
    "pg_simulate_seq_sam": (C.c_int, [P, C.POINTER(SeqCfg), C.c_uint64, C.POINTER(SamCfg), C.POINTER(P)]),
    "pg_batch_create": (C.c_int, [P, C.c_uint32, C.POINTER(P), f64p, f64p, f64p, f64p, u32p, C.c_uint32, u32p,
                                  C.c_uint32, C.POINTER(SeqCfg), C.POINTER(P)]),
    "pg_batch_destroy": (C.c_int, [P]),
    "pg_batch_run": (C.c_int, [P, u64p, u64p]),
    "pg_batch_autotune": (C.c_int, [P, u64p, u64p, u32p]),
    "pg_batch_tile_sizes": (C.c_int, [P, u32p]),
    "pg_batch_set_tile_sizes": (C.c_int, [P, u32p]),
    "pg_batch_dims": (C.c_int, [P, C.c_uint32, u64p, u32p, u64p]),
    "pg_batch_copy": (C.c_int, [P, C.c_uint32, u32p, u32p, u32p, u8p, u8p, C.POINTER(C.c_uint16), u8p, u8p, i32p,
                                i32p]),
    "pg_batch_kernel_ms": (C.c_int, [P, f32p, f32p]),
    # data frames
    "pg_engine_set_signature_names": (C.c_int, [P, C.c_int, C.c_uint32, C.POINTER(C.c_char_p)]),
    "pg_engine_signature_name": (C.c_int, [P, C.c_int, C.c_uint32, C.c_char_p, C.c_uint32, u32p]),
    "pg_placed_mutation_info": (C.c_int, [P, C.c_uint64, u32p, u32p, u32p, C.c_char_p, C.c_char_p, u8p, i32p,
                                          u8p]),
    "pg_placed_cell_mutations": (C.c_int, [P, C.c_uint32, u32p, u64p]),
    "pg_placed_cell_mutations_copy": (C.c_int, [P, u32p, u32p, u32p]),
    "pg_placed_cell_cnas": (C.c_int, [P, C.c_uint32, u32p, u64p]),
    "pg_placed_cell_cnas_copy": (C.c_int, [P, u32p, u32p]),
    "pg_placed_cell_fragmentation": (C.c_int, [P, C.c_uint32, u32p, u64p]),
    "pg_placed_cell_fragmentation_copy": (C.c_int, [P, u32p, u32p, u32p, u32p, u32p, u32p]),
    "pg_placed_bulk_fragmentation": (C.c_int, [P, C.c_int32, u64p]),
    "pg_placed_bulk_fragmentation_copy": (C.c_int, [P, u32p, u32p, u32p, u32p, u32p, f64p]),
    "pg_placed_samples_info": (C.c_int, [P, u32p, f64p, f64p]),
    "pg_engine_load_signatures_tsv": (C.c_int, [P, C.c_int, C.c_char_p]),
    "pg_signature_table_read": (C.c_int, [C.c_int, C.c_char_p, u32p, u64p, C.c_char_p, f64p]),
    "pg_placed_serialize": (C.c_int, [P, u8p, C.c_uint64, u64p]),
    "pg_placed_deserialize": (C.c_int, [P, u8p, C.c_uint64, C.POINTER(P)]),
    "pg_placed_save": (C.c_int, [P, C.c_char_p]),
    "pg_placed_load": (C.c_int, [P, C.c_char_p, C.POINTER(P)]),
    "pg_seq_result_frame": (C.c_int, [P, P, C.c_int, u64p]),
    "pg_seq_result_frame_causes_size": (C.c_int, [P, u64p]),
    "pg_seq_result_frame_copy": (C.c_int, [P, u32p, u32p, C.c_char_p, C.c_char_p, u64p, C.c_char_p, u8p, i32p,
                                           i32p, f64p]),
}

SID_CHARS = 16   # PG_SID_CHARS

# symbols added by later additions to the ABI are bound when present
OPTIONAL = set()


def lib() -> C.CDLL:
    """Loads the library (once); raises when it has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -m process_gb300.build` "
                          "(process_gb300 has no CPU fallback)")
    lb = C.CDLL(str(LIB_PATH))
    for name, (res, args) in _PROTOS.items():
        if not hasattr(lb, name):
            if name in OPTIONAL:
                continue
            raise ImportError(f"{LIB_PATH} does not export {name}")
        fn = getattr(lb, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lb
    return lb


def check(status: int) -> None:
    if status == PG_OK:
        return
    msg = lib().pg_last_error().decode(errors="replace")
    if status == PG_ERR_DOMAIN:
        raise DomainError(status, msg)
    if status == PG_ERR_UNSUPPORTED:
        raise UnsupportedError(status, msg)
    raise ProcessError(status, msg)


def ptr(arr, ctype):
    """ctypes pointer to the data of a contiguous numpy array (or NULL for None)."""
    if arr is None:
        return None
    return arr.ctypes.data_as(C.POINTER(ctype))


def device_count() -> int:
    n = C.c_int(0)
    check(lib().pg_device_count(C.byref(n)))
    return n.value
