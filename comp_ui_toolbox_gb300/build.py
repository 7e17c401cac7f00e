"""Build recipe for libcui_born.so (sm_103a only, in-tree).

Compiles every ``csrc/*.cu`` translation unit in parallel with nvcc for
``compute_103a/sm_103a`` and links them into ``libcui_born.so`` next to this
file.  No CMake, no torch extension machinery: the library is a plain C-ABI
shared object that MATLAB (through the MEX shim), C and Python all load.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIB = HERE / "libcui_born.so"
HARNESS_SRC = HERE / "harness" / "cui_harness.c"
HARNESS = HERE / "cui_harness"
ROOT = HERE.parent

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
          "--expt-relaxed-constexpr", f"-I{ROOT / 'include'}"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libcui_born")


def _run(cmd):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + res.stdout + res.stderr)
    return res.stdout + res.stderr


def sources():
    return sorted(CSRC.glob("*.cu"))


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    deps = list(CSRC.glob("*")) + list((ROOT / "include").glob("*.h")) + [Path(__file__), HARNESS_SRC]
    return HARNESS.exists() and all(d.stat().st_mtime <= t for d in deps)


def build(force: bool = False, verbose: bool = False, extra_flags=()) -> Path:
    """Compile libcui_born.so if any source is newer than it; return its path."""
    if not force and up_to_date():
        return LIB
    BUILD.mkdir(exist_ok=True)
    cc = nvcc()
    objs = []
    cmds = []
    for src in sources():
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        cmds.append([cc, *ARCH, *CFLAGS, *extra_flags, "-c", str(src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=min(len(cmds), os.cpu_count() or 4)) as ex:
        for out in ex.map(_run, cmds):
            if verbose and out.strip():
                print(out, file=sys.stderr)
    tmp = LIB.with_suffix(".so.tmp")
    _run([cc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread", "-ldl"])
    os.replace(tmp, LIB)
    build_harness()
    return LIB


def build_harness() -> Path:
    """Plain C driver of the C-ABI (gcc, links libcui_born.so with an $ORIGIN rpath)."""
    cc = shutil.which("cc") or shutil.which("gcc")
    if cc is None:
        raise RuntimeError("no C compiler for the harness")
    _run([cc, "-O2", "-std=c99", "-Wall", "-Wextra", f"-I{ROOT / 'include'}", str(HARNESS_SRC),
          f"-L{HERE}", "-lcui_born", "-lm", "-Wl,-rpath,$ORIGIN", "-o", str(HARNESS)])
    return HARNESS


if __name__ == "__main__":
    force = "--force" in sys.argv
    flags = ["-Xptxas", "-v"] if "--ptxas-v" in sys.argv else []
    print(build(force=force or bool(flags), verbose=True, extra_flags=flags))
