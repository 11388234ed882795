"""Build libskyr.so (the CUDA kernels + C ABI) in-tree for sm_103a.

Each ``csrc/*.cu`` translation unit is compiled in parallel with one
``-gencode arch=compute_103a,code=sm_103a`` and linked into
``skyrendering_gb300/libskyr.so``.  Objects go to ``skyrendering_gb300/_build``.
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
BUILD = PKG / "_build"
LIB = PKG / "libskyr.so"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libskyr.so")


def _flags(extra: list[str] | None = None) -> list[str]:
    # Approximate division and square root (the kernels' formulas are
    # cancellation-free, so 2-ulp quotients do not amplify); no flush-to-zero,
    # so that denormal transmittances survive.
    f = [ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-prec-div=false",
         "-prec-sqrt=false", "-ftz=false", "-Xcompiler", "-Wall", "-Xptxas", "-warn-spills",
         "-I", str(PKG.parent / "include")]
    if os.environ.get("SKYR_PTXAS_VERBOSE"):
        f += ["-Xptxas", "-v"]
    return f + (extra or [])


def _needs(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    deps = [src] + list(CSRC.glob("*.cuh")) + list((PKG.parent / "include").glob("*.h"))
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def build(verbose: bool = False, force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    srcs = sorted(CSRC.glob("*.cu"))
    if not srcs:
        raise RuntimeError("no CUDA sources found")
    cc = nvcc()
    jobs = []
    for s in srcs:
        o = BUILD / (s.stem + ".o")
        if force or _needs(o, s):
            jobs.append((s, o))

    def compile_one(so):
        s, o = so
        cmd = [cc, *_flags(), "-c", str(s), "-o", str(o)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        return s, r, cmd

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for s, r, cmd in ex.map(compile_one, jobs):
                if verbose or r.returncode != 0:
                    sys.stderr.write(r.stdout + r.stderr)
                if r.returncode != 0:
                    raise RuntimeError(f"nvcc failed on {s.name}: {' '.join(cmd)}")
    objs = [BUILD / (s.stem + ".o") for s in srcs]
    if force or jobs or not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        cmd = [cc, ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link of libskyr.so failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
