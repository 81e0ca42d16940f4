"""The C ABI library builds, loads without a GPU, exports every declared entry point, and
rejects invalid arguments with LAPACK-style statuses before touching the device."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADERS = sorted((ROOT / "include").glob("*.h"))
DECL = re.compile(r"^\s*(?:const\s+)?(?:int|int64_t|size_t|char|void)\s*\*?\s*(blastgpu_\w+)\s*\(", re.M)


def declared():
    names = []
    for h in HEADERS:
        names += DECL.findall(h.read_text())
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from blast_gb300 import _build, _lib

    _build.build_library()
    return _lib.lib()


def test_header_declares_entry_points():
    names = declared()
    assert "blastgpu_dgemm_strided" in names and "blastgpu_dposv_strided" in names
    assert len(names) >= 10


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", str(Path(lib._name))], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\s[TW]\s(blastgpu_\w+)$", out, re.M))
    missing = [n for n in declared() if n not in exported]
    assert not missing, missing


def test_python_binding_covers_header():
    from blast_gb300 import _lib

    missing = [n for n in declared() if n not in _lib.SIGNATURES]
    assert not missing, missing


def test_status_strings(lib):
    assert lib.blastgpu_status_string(0) == b"success"
    assert lib.blastgpu_status_string(-3) == b"invalid argument"
    assert lib.blastgpu_version() >= 100


def test_argument_validation_without_device(lib):
    """Invalid arguments are rejected on the host (no CUDA call is made), LAPACK style."""
    from blast_gb300 import _lib

    f = lib.blastgpu_dgemm_strided
    assert f(2, 0, 1, 1, 1, 1.0, None, 1, 0, None, 1, 0, 1.0, None, 1, 0, None, 1, 0, 1, None) == -1
    assert f(0, 0, -1, 1, 1, 1.0, None, 1, 0, None, 1, 0, 1.0, None, 1, 0, None, 1, 0, 1, None) == -3
    assert f(0, 0, 4, 4, 4, 1.0, None, 2, 0, None, 4, 0, 1.0, None, 4, 0, None, 4, 0, 1, None) == -8
    # empty problems are a successful no-op
    assert f(0, 0, 0, 4, 4, 1.0, None, 1, 0, None, 4, 0, 1.0, None, 1, 0, None, 1, 0, 1, None) == 0
    assert lib.blastgpu_dpotrf_strided(-1, None, 1, 0, None, 1, 0, None, 1, None) == -1
    assert lib.blastgpu_dpotrf_strided(4, None, 4, 0, None, 4, 0, None, 1, None) == -2
    assert lib.blastgpu_dposv_strided(4, -2, None, 4, 0, None, 4, 0, None, 4, 0, None, 4, 0, None, 1,
                                      None) == -2
    with pytest.raises(_lib.BlastGpuError):
        _lib.call("blastgpu_dpotrs_strided", -1, 1, None, 1, 0, None, 1, 0, None, 1, 0, 1, None)


def test_argument_validation_blas2_and_extensions(lib):
    """The BLAS-2 entry points, the right-side solve, the fused Riccati step and the host-operand
    solve check their arguments on the host in declaration order. Every case below fails a check
    that precedes any CUDA call. The fake pointer (8) is never dereferenced, because a later
    argument is invalid."""
    p = 8  # non-null stand-in for a pointer argument that is checked only for null
    ger = lib.blastgpu_dger_strided
    assert ger(-1, 1, 1.0, None, 1, 0, None, 1, 0, None, 1, 0, None, 1, 0, 1, None) == -1
    assert ger(1, -1, 1.0, None, 1, 0, None, 1, 0, None, 1, 0, None, 1, 0, 1, None) == -2
    assert ger(2, 2, 1.0, None, 1, 0, None, 1, 0, None, 2, 0, None, 2, 0, 1, None) == -4
    assert ger(0, 0, 1.0, None, 0, 0, None, 1, 0, None, 1, 0, None, 1, 0, 1, None) == -5
    assert ger(0, 0, 1.0, None, 1, 0, None, 0, 0, None, 1, 0, None, 1, 0, 1, None) == -8
    assert ger(3, 2, 1.0, p, 1, 0, p, 1, 0, p, 2, 0, p, 3, 0, 1, None) == -11
    assert ger(3, 2, 1.0, p, 1, 0, p, 1, 0, p, 3, 0, p, 2, 0, 1, None) == -14
    assert ger(3, 2, 1.0, p, 1, 0, p, 1, 0, p, 3, 0, p, 3, 0, -1, None) == -16
    assert ger(0, 5, 1.0, None, 1, 0, None, 1, 0, None, 1, 0, None, 1, 0, 7, None) == 0  # empty: no-op

    iamax = lib.blastgpu_idamax_strided
    assert iamax(0, p, 1, 0, p, 1, None) == -1  # BLAST asserts a non-empty vector
    assert iamax(4, None, 1, 0, p, 1, None) == -2
    assert iamax(4, p, 0, 0, p, 1, None) == -3
    assert iamax(4, p, 1, 0, None, 1, None) == -5
    assert iamax(4, p, 1, 0, p, -1, None) == -6

    laswp = lib.blastgpu_dlaswp_strided
    assert laswp(-1, None, 1, 0, 0, 0, None, 0, 1, None) == -1
    assert laswp(0, None, 0, 0, 0, 0, None, 0, 1, None) == -3
    assert laswp(2, p, 4, 0, -1, 0, None, 0, 1, None) == -5
    assert laswp(2, p, 4, 0, 3, 2, None, 0, 1, None) == -6
    assert laswp(2, p, 4, 0, 0, 2, None, 0, 1, None) == -7
    assert laswp(2, p, 4, 0, 0, 2, p, 4, -1, None) == -9

    swap = lib.blastgpu_dswap_strided
    assert swap(-1, None, 1, 0, None, 1, 0, 1, None) == -1
    assert swap(0, None, 0, 0, None, 1, 0, 1, None) == -3
    assert swap(0, None, 1, 0, None, 0, 0, 1, None) == -6
    assert swap(3, p, 1, 0, p, 1, 0, -1, None) == -8

    tr = lib.blastgpu_dtrsm_right_strided
    assert tr(7, 0, 0, 1, 1, p, 1, 0, p, 1, 0, p, 1, 0, 1, None) == -1
    assert tr(0, 2, 0, 1, 1, p, 1, 0, p, 1, 0, p, 1, 0, 1, None) == -2
    assert tr(0, 0, 2, 1, 1, p, 1, 0, p, 1, 0, p, 1, 0, 1, None) == -3
    assert tr(0, 0, 0, 3, 4, p, 3, 0, p, 3, 0, p, 3, 0, 1, None) == -7  # lda < n
    assert tr(0, 0, 0, 3, 4, p, 4, 0, p, 2, 0, p, 3, 0, 1, None) == -10  # ldb < m
    assert tr(0, 0, 0, 3, 4, p, 4, 0, p, 3, 0, None, 3, 0, 1, None) == -12
    assert tr(0, 0, 0, 3, 4, p, 4, 0, p, 3, 0, p, 3, 0, -2, None) == -15

    sp = lib.blastgpu_dsyrk_potrf_strided
    assert sp(-1, 1, 0, 1.0, p, 1, 0, 1.0, p, 1, 0, p, 1, 0, None, 1, None) == -1
    assert sp(4, -1, 0, 1.0, p, 4, 0, 1.0, p, 4, 0, p, 4, 0, None, 1, None) == -2
    assert sp(4, 2, 2, 1.0, p, 4, 0, 1.0, p, 4, 0, p, 4, 0, None, 1, None) == -3
    assert sp(4, 2, 0, 1.0, None, 4, 0, 1.0, p, 4, 0, p, 4, 0, None, 1, None) == -5
    assert sp(4, 2, 1, 1.0, p, 1, 0, 1.0, p, 4, 0, p, 4, 0, None, 1, None) == -6  # trans: lda >= k
    assert sp(4, 2, 0, 1.0, p, 4, 0, 1.0, p, 4, 0, None, 4, 0, None, 1, None) == -12
    assert sp(4, 2, 0, 1.0, p, 4, 0, 1.0, p, 4, 0, p, 4, 0, None, -1, None) == -16

    mirror = lib.blastgpu_dposv_mirror_strided
    # n, nrhs, A, lda, sa, B, ldb, sb, L, ldl, sl, X, ldx, sx, L_work, X_work, info, batch, stream
    ok = (48, 8, p, 48, 0, p, 48, 0, p, 48, 0, p, 48, 0, p, p, None, 1, None)

    def call(**bad):
        args = list(ok)
        for i, v in bad.items():
            args[int(i[1:])] = v
        return mirror(*args)

    assert call(a0=-1) == -1
    assert call(a1=-1) == -2
    assert call(a2=None) == -3
    assert call(a3=47) == -4
    assert call(a5=None) == -6
    assert call(a9=40) == -10
    assert call(a14=None) == -15  # the device workspace for L
    assert call(a15=None) == -16  # the device workspace for X
    assert call(a17=-1) == -18

    # adjoints: invalid sizes, and a shared (stride 0) output for a batch of 2 (instances would race)
    assert lib.blastgpu_dpotrf_bwd_strided(-1, p, 1, 0, p, 1, 0, p, 1, 0, 1, None) == -1
    assert lib.blastgpu_dpotrf_bwd_strided(4, p, 3, 16, p, 4, 16, p, 4, 16, 1, None) == -3
    assert lib.blastgpu_dpotrf_bwd_strided(4, p, 4, 16, p, 4, 16, p, 4, 0, 2, None) == -10
    assert lib.blastgpu_dtrsm_bwd_strided(2, 0, 0, 4, 1, p, 4, 16, p, 4, 4, p, 4, 4, p, 4, 4, None, 4, 0, 1,
                                          None) == -1
    assert lib.blastgpu_dtrsm_bwd_strided(0, 0, 0, 4, 1, p, 4, 16, p, 4, 4, p, 4, 4, p, 4, 0, None, 4, 0, 2,
                                          None) == -17
    assert lib.blastgpu_dgemm_bwd_strided(0, 0, 2, 2, 2, 1.0, p, 2, 4, p, 2, 4, 1.0, p, 1, 4, None, 2, 0, None, 2,
                                          0, None, 2, 0, 1, None) == -15
    assert lib.blastgpu_dgemm_bwd_strided(0, 0, 2, 2, 2, 1.0, p, 2, 4, p, 2, 4, 1.0, p, 2, 4, p, 2, 0, None, 2, 0,
                                          None, 2, 0, 2, None) == -19


def test_descriptor_layouts_match_header(tmp_path):
    """The numpy descriptor dtypes of blast_gb300.desc have exactly the byte layout of the C
    structs in include/blastgpu.h (sizes and field offsets, as a C compiler lays them out)."""
    from blast_gb300 import desc

    structs = {
        "blastgpu_mat": (desc.MAT_DTYPE, ["data", "rows", "cols", "ld", "layout", "ps", "reserved"]),
        "blastgpu_gemm_desc": (desc.GEMM_DTYPE, ["A", "B", "C", "D", "alpha", "beta"]),
        "blastgpu_getrf_desc": (desc.GETRF_DTYPE, ["A", "ipiv", "B"]),
        "blastgpu_gesv_mixed_desc": (desc.GESV_MIXED_DTYPE, ["A", "ipiv", "B", "ws_offset"]),
        "blastgpu_posv_desc": (desc.POSV_DTYPE, ["A", "L", "B", "X", "ws_offset"]),
        "blastgpu_posv_bwd_desc": (desc.POSV_BWD_DTYPE, ["A", "L", "X", "Xbar", "Bbar", "Abar"]),
        "blastgpu_potrf_desc": (desc.POTRF_DTYPE, ["A", "L"]),
        "blastgpu_copy_desc": (desc.COPY_DTYPE, ["src", "dst"]),
        "blastgpu_syrk_desc": (desc.SYRK_DTYPE, ["A", "C", "D", "alpha", "beta"]),
        "blastgpu_trsm_desc": (desc.TRSM_DTYPE, ["A", "B", "X"]),
        "blastgpu_trmm_desc": (desc.TRMM_DTYPE, ["A", "B", "C", "alpha"]),
        "blastgpu_ger_desc": (desc.GER_DTYPE, ["x", "y", "A", "B", "alpha"]),
        "blastgpu_laswp_desc": (desc.LASWP_DTYPE, ["A", "ipiv", "k0", "k1"]),
        "blastgpu_swap_desc": (desc.SWAP_DTYPE, ["x", "y"]),
        "blastgpu_gemm_bwd_desc": (desc.GEMM_BWD_DTYPE, ["A", "B", "Dbar", "Abar", "Bbar", "Cbar", "alpha", "beta"]),
        "blastgpu_trsm_bwd_desc": (desc.TRSM_BWD_DTYPE, ["A", "X", "Xbar", "Bbar", "Abar"]),
        "blastgpu_potrf_bwd_desc": (desc.POTRF_BWD_DTYPE, ["L", "Lbar", "Abar"]),
    }
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "blastgpu.h"', "int main(void) {"]
    for name, (_, fields) in structs.items():
        lines.append(f'    printf("{name} %zu\\n", sizeof({name}));')
        for f in fields:
            lines.append(f'    printf("{name}.{f} %zu\\n", offsetof({name}, {f}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    got = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                           check=True).stdout.splitlines())
    for name, (dt, fields) in structs.items():
        assert int(got[name]) == dt.itemsize, name
        for f in fields:
            assert int(got[f"{name}.{f}"]) == dt.fields[f][1], (name, f)


def test_cpp_shim_compiles_and_links(lib, tmp_path):
    """include/blastgpu/blast.hpp (BLAST's names over the C ABI) and the example program that uses
    it compile with the host C++ compiler and link against the library (running it needs a GPU:
    tests/test_gpu_cpp_shim.py)."""
    import os
    import shutil

    cuda = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None or not (cuda / "include" / "cuda_runtime.h").exists():
        pytest.skip("no host C++ compiler or CUDA headers")
    libpath = Path(lib._name)
    exe = tmp_path / "test_shim"
    subprocess.run([cxx, "-std=c++17", "-Wall", str(ROOT / "tests" / "cpp" / "test_shim.cpp"), "-I",
                    str(ROOT / "include"), "-I", str(cuda / "include"), "-L", str(libpath.parent), "-lblastgpu", "-L",
                    str(cuda / "lib64"), "-lcudart", "-o", str(exe)], check=True)
    assert exe.exists()
