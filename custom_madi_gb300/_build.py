"""Build the native library ``_lib/libmadi_gb300.so`` in-tree with nvcc.

Every translation unit is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, then linked with the
static CUDA runtime into one shared object that exports the C ABI of
``include/madi_gb300.h``.  Objects are rebuilt when a source or header is newer.
"""

from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "_lib"
OBJDIR = LIBDIR / "obj"
LIBNAME = "libmadi_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["walk.cu", "classify.cu", "match.cu", "match_bf16.cu", "bayes.cu"]
CPP_SOURCES = ["host.cpp", "serve.cpp"]


def nvcc_path() -> str:
    found = shutil.which("nvcc")
    if found:
        return found
    for cand in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build custom_madi_gb300")


def library_path() -> Path:
    return LIBDIR / LIBNAME


def _deps() -> list[Path]:
    return sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + [ROOT / "include" / "madi_gb300.h"]


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src, *_deps()])


def build(force: bool = False, verbose: bool = False) -> Path:
    nvcc = nvcc_path()
    OBJDIR.mkdir(parents=True, exist_ok=True)
    jobs = []
    for name in CU_SOURCES:
        src, obj = CSRC / name, OBJDIR / (name + ".o")
        if force or _stale(obj, src):
            jobs.append([nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-c", str(src), "-o", str(obj)])
    for name in CPP_SOURCES:
        src, obj = CSRC / name, OBJDIR / (name + ".o")
        if force or _stale(obj, src):
            jobs.append([nvcc, "-O2", "-std=c++17", "-Xcompiler", "-fPIC,-pthread", "-x", "c++",
                         "-c", str(src), "-o", str(obj)])

    def run(cmd):
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
        if verbose and (res.stdout or res.stderr):
            print(res.stdout + res.stderr)

    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(run, jobs))
    out = library_path()
    objs = [OBJDIR / (n + ".o") for n in CU_SOURCES + CPP_SOURCES]
    if force or jobs or not out.exists():
        tmp = out.with_suffix(".so.tmp")
        run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs), "-lpthread"])
        os.replace(tmp, out)
    return out


if __name__ == "__main__":
    print(build(force=True, verbose=True))
