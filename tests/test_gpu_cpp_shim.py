"""The C++ shim (include/blastgpu/blast.hpp) compiles with the host C++ compiler against the C ABI
and runs BLAST-named calls on the GPU (tests/cpp/test_shim.cpp)."""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


def test_cpp_shim_builds_and_runs(gpu, tmp_path):
    from blast_gb300 import _build

    lib = _build.build_library()
    cuda = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.fail("no host C++ compiler")
    exe = tmp_path / "test_shim"
    cmd = [cxx, "-std=c++17", "-O2", str(ROOT / "tests" / "cpp" / "test_shim.cpp"), "-I", str(ROOT / "include"),
           "-I", str(cuda / "include"), "-L", str(lib.parent), "-lblastgpu", "-L", str(cuda / "lib64"),
           "-lcudart", f"-Wl,-rpath,{lib.parent}", f"-Wl,-rpath,{cuda / 'lib64'}", "-o", str(exe)]
    subprocess.run(cmd, check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "shim ok" in out.stdout
