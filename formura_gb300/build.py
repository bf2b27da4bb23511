"""Build recipe for the native parts of formura_gb300.

* ``libformura_gb300.so`` — the CUDA kernels and the thin C ABI
  (``include/formura_gb300.h``), compiled with nvcc for sm_103a only.
* the emitted per-program host libraries (``lib<program>.so``) — see
  :mod:`formura_gb300.backend` — compiled with g++ against that C ABI.

Everything is written in-tree under ``formura_gb300/_build/`` (git-ignored).
Translation units compile in parallel; an object is rebuilt only when a
source, a shared header or the flags changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = BUILD / "libformura_gb300.so"

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = [
    ARCH,
    "-O3",
    "-lineinfo",
    "--fmad=false",  # generated-code parity: no silent FMA contraction
    "-std=c++17",
    "-Xcompiler=-fPIC",
    "-Xcompiler=-fvisibility=hidden",
    "-Xptxas=-warn-spills",
]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build formura_gb300")
    return cand


def _digest(paths, extra: str) -> str:
    h = hashlib.sha256(extra.encode())
    for p in sorted(paths):
        h.update(Path(p).read_bytes())
    return h.hexdigest()[:16]


def _run(cmd, cwd=None):
    r = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed (%d): %s\n%s" % (r.returncode, " ".join(cmd), r.stdout))
    return r.stdout


def cuda_sources():
    return sorted(CSRC.glob("*.cu"))


def build_library(verbose: bool = False, jobs: int | None = None) -> Path:
    """Compile every ``csrc/*.cu`` for sm_103a and link libformura_gb300.so."""
    nvcc = _nvcc()
    objdir = BUILD / "obj"
    objdir.mkdir(parents=True, exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    flags_key = " ".join(NVCC_FLAGS)
    jobs = jobs or max(1, min(len(cuda_sources()), os.cpu_count() or 4))

    def compile_one(src: Path):
        key = _digest([src] + headers, flags_key)
        obj = objdir / (src.stem + "." + key + ".o")
        if obj.exists():
            return obj, ""
        for old in objdir.glob(src.stem + ".*.o"):
            old.unlink()
        cmd = [nvcc, *NVCC_FLAGS, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj) + ".tmp"]
        out = _run(cmd)
        os.replace(str(obj) + ".tmp", obj)
        return obj, out

    with cf.ThreadPoolExecutor(jobs) as ex:
        results = list(ex.map(compile_one, cuda_sources()))
    objs = [o for o, _ in results]
    if verbose:
        for o, out in results:
            if out.strip():
                print(o.name, out, file=sys.stderr)
    link_key = _digest(objs, "link")
    stamp = BUILD / "libformura_gb300.stamp"
    if LIB.exists() and stamp.exists() and stamp.read_text() == link_key:
        return LIB
    tmp = str(LIB) + ".tmp"
    _run([nvcc, ARCH, "-shared", "-cudart=static", "-o", tmp, *map(str, objs)])
    os.replace(tmp, LIB)
    stamp.write_text(link_key)
    return LIB


def build_all(verbose: bool = False) -> Path:
    lib = build_library(verbose=verbose)
    from . import backend

    backend.build_programs(verbose=verbose)
    return lib


if __name__ == "__main__":
    print(build_all(verbose=True))
