"""Builds libfluids_gb300.so in-tree with nvcc for sm_103a.

Each translation unit compiles in its own nvcc process (in parallel), then
one nvcc call links the shared library next to this file. Forward kernel
units are compiled with --fmad=false (no FMA contraction), host units with
-ffp-contract=off, so every float expression rounds as written; the adjoint
unit keeps contraction on.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
BUILD = PKG / "_build"
LIB = PKG / "libfluids_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
          f"-I{INCLUDE}", f"-I{CSRC}"]
CU_FLAGS = ARCH + COMMON + ["--fmad=false", "-Xptxas", "-v"]
CPP_FLAGS = COMMON
# The adjoint kernels have no bit-exact target: FMA contraction on. Their
# decisions shared with the forward use explicitly rounded operations.
CONTRACTED = {"fl_adjoint.cu"}
CU_FLAGS_CONTRACTED = ARCH + COMMON + ["-Xptxas", "-v"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: set CUDA_HOME or put nvcc on PATH")
    return cand


def sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _compile(src: Path) -> tuple[Path, str]:
    obj = BUILD / (src.name + ".o")
    if src.suffix == ".cu":
        flags = CU_FLAGS_CONTRACTED if src.name in CONTRACTED else CU_FLAGS
    else:
        flags = CPP_FLAGS
    cmd = [nvcc(), *flags, "-c", str(src), "-o", str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    return obj, res.stderr


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = sources() + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h")) + [Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile and link the library if any source is newer than it."""
    if not force and not _stale():
        return LIB
    BUILD.mkdir(exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        results = list(ex.map(_compile, sources()))
    if verbose:
        for obj, log in results:
            if log.strip():
                print(f"--- {obj.name}\n{log}")
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *[str(o) for o, _ in results]]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, verbose=True))
