"""The allocation-free mixed-precision Cholesky solve (blastgpu_dposv_mixed_batched_noalloc),
called through the C ABI and checked against the workspace entry point
(blastgpu_dposv_mixed_batched) on the same ragged batch, on two calls in a row.

Its callers cannot allocate device memory when they solve: a model-predictive controller that
calls the batched solve from its control loop, where allocation is ruled out after start-up
because its latency is unbounded, or an application that owns every device allocation. The
binary32 factors therefore live in a fixed 32 MiB array inside the library instead of caller
workspace. This file runs last, so that a failure here does not hide the other tests' results.
"""
import numpy as np
import pytest

from helpers import normwise

pytestmark = pytest.mark.gpu


def _batch(rng, ns):
    mats = []
    for n in ns:
        Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
        lam = np.logspace(0, -4, n)
        A = (Q * lam) @ Q.T
        mats.append((A + A.T) / 2)
    return mats


def test_noalloc_matches_workspace_entry_point(gpu):
    import torch

    from blast_gb300 import _lib, desc
    from blast_gb300.ragged import Packed

    rng = np.random.default_rng(77)
    ns = np.array([64, 150, 300, 97, 256, 200, 128, 72])
    count, max_n = len(ns), int(ns.max())
    A = Packed(ns, ns, "cuda")
    A.fill_from(_batch(rng, ns))
    ones = np.ones_like(ns)
    B = Packed(ns, ones, "cuda")
    B.fill_from([rng.standard_normal((n, 1)) for n in ns])
    X_ref, X_na = Packed(ns, ones, "cuda"), Packed(ns, ones, "cuda")

    per = np.array([_lib.lib().blastgpu_dposv_mixed_workspace_bytes(int(n)) for n in ns], dtype=np.int64)
    offs = np.concatenate([[0], np.cumsum(per)[:-1]])
    scratch_bytes = int(per.sum())
    assert scratch_bytes <= _lib.NOALLOC_SCRATCH_BYTES

    def descriptors(X):
        recs = np.zeros(count, dtype=desc.POSV_DTYPE)
        for i in range(count):
            recs[i] = (A.record(i), desc.EMPTY_MAT, B.record(i), X.record(i), int(offs[i]))
        return desc.upload(recs, "cuda")

    d_ref, d_na = descriptors(X_ref), descriptors(X_na)
    stream = torch.cuda.current_stream().cuda_stream
    outs = [torch.zeros(count, dtype=torch.int32, device="cuda") for _ in range(2)]
    berrs = [torch.zeros(count, dtype=torch.float64, device="cuda") for _ in range(2)]
    infos = [torch.full((count,), -9, dtype=torch.int32, device="cuda") for _ in range(2)]

    # reference: caller-provided workspace
    workspace = torch.empty(scratch_bytes, dtype=torch.uint8, device="cuda")
    _lib.call("blastgpu_dposv_mixed_batched", d_ref.data_ptr(), count, max_n, workspace.data_ptr(),
              1e-12, 10, infos[0].data_ptr(), outs[0].data_ptr(), berrs[0].data_ptr(), stream)
    torch.cuda.synchronize()
    x_ref = X_ref.to_list()
    assert not infos[0].cpu().numpy().any()
    assert np.all(berrs[0].cpu().numpy() <= 1e-12)

    # the allocation-free entry point, twice in a row (the scratch keeps the first call's contents)
    for call in range(2):
        X_na.buf.zero_()
        infos[1].fill_(-9)
        _lib.call("blastgpu_dposv_mixed_batched_noalloc", d_na.data_ptr(), count, max_n, scratch_bytes,
                  1e-12, 10, infos[1].data_ptr(), outs[1].data_ptr(), berrs[1].data_ptr(), stream)
        torch.cuda.synchronize()
        assert not infos[1].cpu().numpy().any(), call
        assert np.all(berrs[1].cpu().numpy() <= 1e-12), call
        for n, xr, xn in zip(ns, x_ref, X_na.to_list()):
            assert normwise(xn, xr) <= 1e-12, (call, n)

    # a descriptor whose scratch range runs past the array (a miscounted scratch_bytes) is not
    # solved and reports info = -1; the other instances of the same batch are unaffected
    recs = np.zeros(count, dtype=desc.POSV_DTYPE)
    bad = 3
    for i in range(count):
        off = int(offs[i])
        if i == bad:
            off = _lib.NOALLOC_SCRATCH_BYTES - int(per[i]) + 256
        recs[i] = (A.record(i), desc.EMPTY_MAT, B.record(i), X_na.record(i), off)
    d_bad = desc.upload(recs, "cuda")
    X_na.buf.fill_(7.0)
    infos[1].fill_(-9)
    _lib.call("blastgpu_dposv_mixed_batched_noalloc", d_bad.data_ptr(), count, max_n, scratch_bytes,
              1e-12, 10, infos[1].data_ptr(), outs[1].data_ptr(), berrs[1].data_ptr(), stream)
    torch.cuda.synchronize()
    info_h, berr_h = infos[1].cpu().numpy(), berrs[1].cpu().numpy()
    assert info_h[bad] == -1 and np.isnan(berr_h[bad])
    assert np.all(X_na.to_list()[bad] == 7.0)  # nothing written for the refused instance
    for i, (n, xr, xn) in enumerate(zip(ns, x_ref, X_na.to_list())):
        if i != bad:
            assert info_h[i] == 0 and berr_h[i] <= 1e-12
            assert normwise(xn, xr) <= 1e-12, (i, n)

    # a batch that needs more scratch than the array holds is refused before any launch
    launches = _lib.launch_count()
    st = _lib.lib().blastgpu_dposv_mixed_batched_noalloc(
        d_na.data_ptr(), count, max_n, _lib.NOALLOC_SCRATCH_BYTES + 1, 1e-12, 10, infos[1].data_ptr(),
        outs[1].data_ptr(), berrs[1].data_ptr(), stream)
    assert st == -1004  # BLASTGPU_ERR_TOO_LARGE
    assert _lib.launch_count() == launches
