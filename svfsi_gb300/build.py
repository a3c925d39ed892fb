"""Build the gsls CUDA library (libgsls.so) in-tree for sm_103a.

Every translation unit is compiled by nvcc in parallel, then linked into
``svfsi_gb300/lib/libgsls.so``.  No cmake, no torch extension machinery: the
product is a plain C-ABI shared library.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "lib"
BUILD = PKG / "_build"
LIBNAME = "libgsls.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
    "--expt-relaxed-constexpr", "-Xptxas", "-O3",
]
SOURCES = [
    "gsls_lhs.cu",
    "gsls_krylov.cu",
    "gsls_assemble.cu",
    "gsls_eq.cu",
    "gsls_gmres.cu",
    "gsls_noalloc.cu",
    "gsls_ns.cu",
    "gsls_bicgs.cu",
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def lib_path() -> Path:
    return LIBDIR / LIBNAME


def _stale(out: Path, deps) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False, extra_flags=None) -> Path:
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "gsls.h"]
    cc = nvcc()
    flags = ARCH + NVCC_FLAGS + list(extra_flags or [])
    jobs = []
    objs = []
    for src in SOURCES:
        s = CSRC / src
        o = BUILD / (s.stem + ".o")
        objs.append(o)
        if force or _stale(o, [s, *headers]):
            jobs.append([cc, *flags, "-c", str(s), "-o", str(o)])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr, file=sys.stderr)
        return r

    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4) or 1) as ex:
        list(ex.map(run, jobs))
    out = lib_path()
    if force or jobs or _stale(out, objs):
        run([cc, *ARCH, "-shared", "-o", str(out), *map(str, objs), "-lcudart"])
    return out


if __name__ == "__main__":
    p = build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(p)
