"""Builds the engine's shared library in-tree for sm_103a.

``python -m dedispersion_gb300.build`` compiles every ``csrc/*.cu`` with nvcc
(one process per translation unit, in parallel) and links
``dedispersion_gb300/libdedisp_gb300.so``.  Host code is compiled with
``-ffp-contract=off`` so that no ``a + b * c`` in the delay and shift
arithmetic is fused into an FMA: the reference is built in ISO C++ mode,
which does not contract either (CMakeLists.txt:5 of the reference).
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libdedisp_gb300.so"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or Path(cand).exists()):
            return cand
    return "nvcc"


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed ({proc.returncode}): {' '.join(cmd)}\n"
                           f"{proc.stdout}\n{proc.stderr}")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compile and link the library; returns its path."""
    BUILD.mkdir(exist_ok=True)
    srcs = sources()
    deps = srcs + sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + \
        sorted((PKG.parent / "include").glob("*.h"))
    newest = max(p.stat().st_mtime for p in deps)
    if not force and LIB.exists() and LIB.stat().st_mtime >= newest:
        return LIB
    flags = ["-O3", "-std=c++17", ARCH, "-lineinfo", "-Xcompiler",
             "-fPIC,-ffp-contract=off,-fno-fast-math", "--expt-relaxed-constexpr",
             "-I", str(PKG.parent / "include")]
    objs = []
    cmds = []
    for src in srcs:
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        cmds.append([nvcc(), *flags, "-c", str(src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=min(8, len(cmds))) as pool:
        list(pool.map(_run, cmds))
    tmp = LIB.with_suffix(".so.tmp")
    _run([nvcc(), ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart_static",
          "-Xlinker", "--no-undefined", "-lpthread", "-ldl", "-lrt"])
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
