"""Builds the CUDA library of process_gb300 in-tree.

``build()`` compiles every translation unit of ``process_gb300/csrc`` for
sm_103a with nvcc (in parallel) and links ``process_gb300/_lib/libprocess_gb300.so``.
Objects are cached by content hash under ``process_gb300/_build`` so an
unchanged source is not recompiled.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIBDIR = PKG / "_lib"
LIBNAME = "libprocess_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# Translation units and whether FMA contraction is allowed.  The placement,
# index and sequencing kernels are replayed bit-exactly on the CPU, so their
# floating-point expressions must not be contracted.
UNITS = {
    "pg_index.cu": False,
    "pg_place.cu": False,
    "pg_seq.cu": False,
    "pg_calib.cu": True,
    "pg_api.cpp": False,
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the process_gb300 CUDA library cannot be built")


def _flags(fmad: bool) -> list[str]:
    return ARCH + [
        "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
        f"--fmad={'true' if fmad else 'false'}", "-I", str(CSRC), "-I", str(PKG.parent / "include"),
    ]


def _digest(paths: list[Path], extra: str) -> str:
    h = hashlib.sha256(extra.encode())
    for p in paths:
        h.update(p.read_bytes())
    return h.hexdigest()[:16]


def _compile(unit: str, fmad: bool) -> Path:
    src = CSRC / unit
    headers = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + [PKG.parent / "include" / "process_gb300.h"]
    flags = _flags(fmad)
    tag = _digest([src] + headers, " ".join(flags))
    obj = BUILD / f"{src.stem}.{tag}.o"
    if obj.exists():
        return obj
    cmd = [nvcc(), "-c", "-x", "cu", str(src), "-o", str(obj) + ".tmp"] + flags
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {unit}:\n{r.stdout}\n{r.stderr}")
    os.replace(str(obj) + ".tmp", obj)
    return obj


def build(verbose: bool = False) -> Path:
    """Compile and link the library; returns its path."""
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    units = {u: f for u, f in UNITS.items() if (CSRC / u).exists()}
    with cf.ThreadPoolExecutor(max_workers=min(8, len(units))) as ex:
        objs = list(ex.map(lambda kv: _compile(*kv), units.items()))
    keep = {o.name for o in objs}
    for old in BUILD.glob("*.o"):            # objects of earlier sources
        if old.name not in keep:
            old.unlink()
    lib = LIBDIR / LIBNAME
    tag = _digest(objs, "link")
    stamp = LIBDIR / f".{LIBNAME}.{tag}"
    if lib.exists() and stamp.exists():
        return lib
    for old in LIBDIR.glob(f".{LIBNAME}.*"):
        old.unlink()
    cmd = [nvcc(), "-shared"] + ARCH + [str(o) for o in objs] + ["-o", str(lib) + ".tmp", "-lcuda"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(str(lib) + ".tmp", lib)
    stamp.touch()
    if verbose:
        print(f"built {lib}")
    return lib


if __name__ == "__main__":
    build(verbose=True)
