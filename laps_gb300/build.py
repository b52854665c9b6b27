"""Build ``liblaps_gpu.so`` in-tree with nvcc for sm_103a.

Every ``csrc/*.cu`` translation unit is compiled in parallel into ``_build/`` and linked
into ``laps_gb300/liblaps_gpu.so``.  Objects are rebuilt only when a source or header is
newer than them.  ``python -m laps_gb300.build`` runs it from the command line.
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
LIB = PKG / "liblaps_gpu.so"
INCLUDE = PKG.parent / "include"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", f"-I{INCLUDE}"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and Path(c).exists():
            return c
    raise RuntimeError("nvcc not found")


def _newest_dep() -> float:
    deps = list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h")) + [Path(__file__)]
    return max(p.stat().st_mtime for p in deps)


def build(verbose: bool = False, jobs: int | None = None, extra_flags=(), build_dir: Path | None = None,
          lib: Path | None = None) -> Path:
    """Compile and link; ``extra_flags`` (e.g. ``-DNAME=VALUE`` tuning macros) go to every nvcc
    call, ``build_dir`` / ``lib`` redirect the objects and the library (another variant)."""
    nvcc = _nvcc()
    BUILD = Path(build_dir) if build_dir else PKG / "_build"
    LIB = Path(lib) if lib else PKG / "liblaps_gpu.so"
    BUILD.mkdir(parents=True, exist_ok=True)
    srcs = sorted(CSRC.glob("*.cu"))
    dep_t = _newest_dep()
    todo = []
    for s in srcs:
        o = BUILD / (s.stem + ".o")
        if not o.exists() or o.stat().st_mtime < max(dep_t, s.stat().st_mtime):
            todo.append((s, o))

    def compile_one(so):
        s, o = so
        cmd = [nvcc, *FLAGS, *extra_flags, *ARCH, "-c", str(s), "-o", str(o)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {s.name}:\n{r.stderr[-4000:]}")
        return s.name

    jobs = jobs or os.cpu_count() or 4
    # the slowest units first so the pool stays busy
    todo.sort(key=lambda so: ("_dd" not in so[0].name, so[0].name))
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        for name in ex.map(compile_one, todo):
            if verbose:
                print("compiled", name, flush=True)
    objs = [str(BUILD / (s.stem + ".o")) for s in srcs]
    if todo or not LIB.exists():
        cmd = [nvcc, "-shared", *ARCH, "-o", str(LIB), *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    print(LIB)
    sys.exit(0)
