"""The autotuner's cache is applied to the library's per-size-bin choices (host side only)."""
import json


def test_tune_cache_roundtrip(tmp_path, monkeypatch):
    from blast_gb300 import _build, _lib, tune

    _build.build_library()
    monkeypatch.setattr(tune, "cache_path", lambda: tmp_path / "gpu.json")
    (tmp_path / "gpu.json").write_text(json.dumps({"gpu": "test", "choices": {
        "posv.variant.n64": 2, "gemm.shape.m32": 1}}))
    applied = tune.apply()
    assert applied == {"posv.variant.n64": 2, "gemm.shape.m32": 1}
    assert _lib.tune_get("posv.variant.n64") == 2
    assert _lib.tune_get("gemm.shape.m32") == 1
    assert _lib.tune_get("never.set") is None
    assert tune.size_bin(48) == 64 and tune.size_bin(24) == 32 and tune.size_bin(3) == 8
