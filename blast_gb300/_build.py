"""Build the blastgpu CUDA library (sm_103a) in-tree, and the CPU oracle used by the tests.

The library is a plain shared object with a C ABI (include/blastgpu.h); it does not link against
PyTorch. Objects are compiled in parallel, one nvcc process per translation unit.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "lib" / "libblastgpu.so"
ORACLE = ROOT / "oracle"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
              "--expt-relaxed-constexpr", "-I", str(ROOT / "include")]


def nvcc() -> str:
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "bin" / "nvcc"
    if cand.exists():
        return str(cand)
    raise RuntimeError("nvcc not found: the blastgpu library needs the CUDA toolkit to build")


def _sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _needs_rebuild(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _compile(src: Path, verbose_regs: bool) -> Path:
    obj = BUILD / (src.stem + ".o")
    headers = list(CSRC.glob("*.cuh")) + [ROOT / "include" / "blastgpu.h"]
    if not _needs_rebuild(obj, [src] + headers):
        return obj
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
    if verbose_regs:
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stderr}")
    if verbose_regs and res.stderr:
        sys.stderr.write(res.stderr)
    return obj


def build_library(verbose_regs: bool = False, jobs: int | None = None) -> Path:
    """Compile every csrc/*.cu for sm_103a and link lib/libblastgpu.so. Returns the path."""
    BUILD.mkdir(parents=True, exist_ok=True)
    LIB.parent.mkdir(parents=True, exist_ok=True)
    srcs = _sources()
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose_regs), srcs))
    if _needs_rebuild(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart_static",
               "-Xcompiler", "-fPIC"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stderr}")
        os.replace(tmp, LIB)
    return LIB


def build_oracle() -> Path:
    """Build the CPU oracle (test infrastructure) with its Makefile."""
    res = subprocess.run(["make", "-s", "-C", str(ORACLE)], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    return ORACLE / "_build" / "libblast_oracle.so"


if __name__ == "__main__":
    print(build_library(verbose_regs="-v" in sys.argv))
    print(build_oracle())
