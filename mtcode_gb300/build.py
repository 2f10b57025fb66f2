"""In-tree build of the sm_103a shared library ``mtcode_gb300/libmtcode_gb300.so``.

The translation units are compiled in parallel with nvcc (one ``-gencode``: compute_103a/sm_103a)
and linked into one shared object that exports the C ABI of ``include/mtcode_gb300.h``.  Objects
go to ``mtcode_gb300/_build/`` (git-ignored).  Run ``python -m mtcode_gb300.build``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "libmtcode_gb300.so"
BUILD = PKG / "_build"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I", str(ROOT / "include")]
CU_SOURCES = ["mtg_api.cu", "mtg_sys_f32.cu", "mtg_sys_f64.cu", "mtg_noalloc.cu"]
CPP_SOURCES = ["mtg_host.cpp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build mtcode_gb300")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed ({proc.returncode}): {' '.join(cmd)}\n{proc.stdout}")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compile (if out of date) and return the path of the shared library."""
    BUILD.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + [ROOT / "include" / "mtcode_gb300.h"]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        obj = BUILD / (src + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src] + headers):
            jobs.append([nvcc(), *ARCH, *NVCC_FLAGS, "-c", str(CSRC / src), "-o", str(obj)])
    for src in CPP_SOURCES:
        obj = BUILD / (src + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src] + headers):
            # no FMA contraction: seeded host inputs come out bit-identical on every host architecture
            jobs.append([nvcc(), *NVCC_FLAGS, "-Xcompiler", "-ffp-contract=off", "-x", "c++", "-c", str(CSRC / src),
                         "-o", str(obj)])
    if jobs:
        with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
            for _ in ex.map(_run, jobs):
                pass
    if force or jobs or _stale(OUT, objs):
        tmp = OUT.with_suffix(".so.tmp")
        _run([nvcc(), *ARCH, "-shared", *map(str, objs), "-o", str(tmp), "-lcudart"])
        os.replace(tmp, OUT)
    if verbose:
        print(f"built {OUT}")
    return OUT


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
