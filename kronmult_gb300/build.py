"""Build recipe of the CUDA library (``libkronmult_gb300.so``) for sm_103a.

Each ``csrc/*.cu`` translation unit is compiled in parallel with nvcc, then
linked into one shared library in this package directory (in-tree, so the
tests and the benchmark load exactly this file).  No cmake, no torch
extension machinery: the library has a plain C ABI and no torch types.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libkronmult_gb300.so")
OBJDIR = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _compile(src: str, flags: list[str]) -> str:
    obj = os.path.join(OBJDIR, os.path.basename(src)[:-3] + ".o")
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps.append(os.path.join(HERE, "..", "include", "kronmult_gb300.h"))
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps if os.path.exists(d)):
        return obj
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "--expt-relaxed-constexpr", "-c", src, "-o", obj, *flags]
    subprocess.run(cmd, check=True)
    return obj


def write_tune_header() -> None:
    """csrc/kmx_tune_table.h from the committed tuning table (rewritten only
    when its content changes, so unchanged builds stay incremental)."""
    sys.path.insert(0, os.path.dirname(HERE))
    from kronmult_gb300.tune import header_from_table

    text = header_from_table()
    path = os.path.join(CSRC, "kmx_tune_table.h")
    old = open(path).read() if os.path.exists(path) else None
    if old != text:
        with open(path, "w") as f:
            f.write(text)


def build(verbose: bool = False, extra_flags: list[str] | None = None) -> str:
    """Compile every translation unit and link the library; returns its path."""
    os.makedirs(OBJDIR, exist_ok=True)
    write_tune_header()
    flags = list(extra_flags or [])
    if verbose:
        flags += ["-Xptxas", "-v"]
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, flags), srcs))
    if not os.path.exists(OUT) or any(os.path.getmtime(OUT) < os.path.getmtime(o) for o in objs):
        tmp = OUT + ".tmp"
        subprocess.run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "shared"], check=True)
        os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
