"""Build recipe of the reference runner: the reference's MEX gateway compiled from its source.

TEST INFRASTRUCTURE ONLY.  Compiles ``+scattering/combined_quick_gpu.cu`` where it lies in the
reference checkout, unchanged, with nvcc (host code; its one device kernel is compiled too but
never loaded), against this directory's ``mex.h`` / ``matrix.h``, and links it with the host
stand-ins of the MEX runtime (``mex_stub.cpp``) and of the CUDA runtime and cuBLAS
(``cuda_stub.cpp``) into ``oracle/_ref/libref_combined_quick_gpu.so``.  Nothing from the
reference is copied; the reference checkout is only read here, on the machine that has it.

    python -m oracle.ref_mex.build [--reference DIR]
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE.parent / "_ref"
LIB = OUT / "libref_combined_quick_gpu.so"
DEFAULT_REFERENCE = Path("/root/reference")


def reference_source(reference: Path = DEFAULT_REFERENCE) -> Path:
    return reference / "+scattering" / "combined_quick_gpu.cu"


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(map(str, cmd)) + "\n" + r.stdout + r.stderr)


def build(reference: Path = DEFAULT_REFERENCE, force: bool = False) -> Path | None:
    """Build the runner library; returns its path, or None when the reference source is absent."""
    src = reference_source(reference)
    if not src.exists():
        return None
    deps = [src, src.with_suffix(".h"), *HERE.glob("*.cpp"), *HERE.glob("*.h"), Path(__file__)]
    if not force and LIB.exists() and all(d.stat().st_mtime <= LIB.stat().st_mtime for d in deps if d.exists()):
        return LIB
    OUT.mkdir(exist_ok=True)
    nvcc = _nvcc()
    cuda_inc = Path(nvcc).resolve().parent.parent / "include"
    gw, cs, ms = OUT / "combined_quick_gpu.o", OUT / "cuda_stub.o", OUT / "mex_stub.o"
    _run([nvcc, "-std=c++17", "-O2", "-Xcompiler", "-fPIC", "-w", f"-I{HERE}", f"-I{src.parent}", "-c", str(src),
          "-o", str(gw)])
    _run(["g++", "-std=c++17", "-O2", "-fPIC", f"-I{cuda_inc}", f"-I{HERE}", "-c", str(HERE / "cuda_stub.cpp"),
          "-o", str(cs)])
    _run(["g++", "-std=c++17", "-O2", "-fPIC", f"-I{HERE}", "-c", str(HERE / "mex_stub.cpp"), "-o", str(ms)])
    tmp = LIB.with_suffix(".so.tmp")
    # -Bsymbolic: the gateway's CUDA, cuBLAS and MEX calls bind to the stand-ins linked here, never to a
    # real CUDA runtime another library of the process has loaded
    _run(["g++", "-shared", "-Wl,-Bsymbolic", "-o", str(tmp), str(gw), str(cs), str(ms)])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    ref = Path(sys.argv[sys.argv.index("--reference") + 1]) if "--reference" in sys.argv else DEFAULT_REFERENCE
    print(build(ref, force="--force" in sys.argv))
