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
