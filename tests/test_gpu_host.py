"""Host-resident batches (blast_gb300.host.PosvHostPipeline): the three transports — staged copies over
three streams; the kernel reading A, B from pinned host memory with staged result copies; and the
kernel that also writes L, X to host memory (blastgpu_dposv_mirror_strided) — give the
device-resident posv's results bit for bit, and so does the mirror transport with several batches
in flight."""
import numpy as np
import pytest

from helpers import spd_batch

pytestmark = pytest.mark.gpu


def _inputs(rng, batch, n, nrhs):
    import torch

    from blast_gb300.host import pinned_col_major

    hA, hB = pinned_col_major(batch, n, n), pinned_col_major(batch, n, nrhs)
    hA.copy_(torch.from_numpy(spd_batch(rng, batch, n)))
    hB.copy_(torch.from_numpy(rng.standard_normal((batch, n, nrhs))))
    return hA, hB


@pytest.mark.parametrize("transport", ["copy", "direct", "mirror"])
@pytest.mark.parametrize("n,nrhs,batch,chunk", [(48, 8, 1000, 300), (17, 3, 257, 257), (5, 1, 70, 32),
                                                (64, 0, 40, 16), (48, 8, 20000, 20000), (8, 3, 48657, 48657)])
def test_host_pipeline_matches_device_posv(gpu, transport, n, nrhs, batch, chunk):
    """The last two sizes run ten or more warps per SM (the last one partial in the second)."""
    import torch

    from blast_gb300.host import PosvHostPipeline, pinned_col_major

    rng = np.random.default_rng(n * 1000 + nrhs)
    hA, hB = _inputs(rng, batch, n, nrhs)
    hL, hX = pinned_col_major(batch, n, n), pinned_col_major(batch, n, nrhs)
    hL.zero_()
    hX.zero_()
    hinfo = torch.full((batch,), -5, dtype=torch.int32).pin_memory()
    pipe = PosvHostPipeline(n, nrhs, chunk, "cuda", transport=transport)
    pipe.run(hA, hB, hL, hX, hinfo)
    torch.cuda.synchronize()
    # device-resident reference: the same solve through blast.posv
    dA, dB = hA.cuda(), hB.cuda()
    dL, dX = gpu.col_major((batch,), n, n, "cuda"), gpu.col_major((batch,), n, nrhs, "cuda")
    dL.zero_()
    info = gpu.posv(dA, dL, dB, dX)
    torch.cuda.synchronize()
    assert not hinfo.any() and not info.any()
    assert torch.equal(torch.tril(hL), torch.tril(dL.cpu()))
    if nrhs:
        assert torch.equal(hX, dX.cpu())


@pytest.mark.parametrize("depth,steps", [(2, 5), (3, 7)])
def test_mirror_pipeline_batches_in_flight(gpu, depth, steps):
    """With depth > 1 consecutive run() calls overlap on the pipeline's own streams, each with its
    own device workspace; every batch (different inputs per call, output buffers per slot) still
    gives the device-resident posv's bits once wait() has joined them."""
    import torch

    from blast_gb300.host import PosvHostPipeline, pinned_col_major

    n, nrhs, batch = 48, 8, 6000
    rng = np.random.default_rng(depth * 100 + steps)
    inputs = [_inputs(rng, batch, n, nrhs) for _ in range(steps)]
    outs = [(pinned_col_major(batch, n, n), pinned_col_major(batch, n, nrhs),
             torch.full((batch,), -5, dtype=torch.int32).pin_memory()) for _ in range(steps)]
    for hL, hX, _ in outs:
        hL.zero_()
        hX.zero_()
    pipe = PosvHostPipeline(n, nrhs, batch, "cuda", transport="mirror", depth=depth)
    for (hA, hB), (hL, hX, hinfo) in zip(inputs, outs):
        pipe.run(hA, hB, hL, hX, hinfo)
    pipe.wait()
    torch.cuda.synchronize()
    for (hA, hB), (hL, hX, hinfo) in zip(inputs, outs):
        dA, dB = hA.cuda(), hB.cuda()
        dL, dX = gpu.col_major((batch,), n, n, "cuda"), gpu.col_major((batch,), n, nrhs, "cuda")
        dL.zero_()
        info = gpu.posv(dA, dL, dB, dX)
        torch.cuda.synchronize()
        assert not hinfo.any() and not info.any()
        assert torch.equal(torch.tril(hL), torch.tril(dL.cpu()))
        assert torch.equal(hX, dX.cpu())
    with pytest.raises(ValueError):
        PosvHostPipeline(n, nrhs, batch, "cuda", transport="copy", depth=2)


def test_zero_copy_rejects_pageable_buffers(gpu):
    import torch

    from blast_gb300.host import PosvHostPipeline, pinned_col_major

    n, batch = 8, 4
    hA = torch.zeros((batch, n, n), dtype=torch.float64).mT  # pageable
    for transport in ("direct", "mirror"):
        pipe = PosvHostPipeline(n, 1, batch, "cuda", transport=transport)
        with pytest.raises(ValueError):
            pipe.run(hA, pinned_col_major(batch, n, 1), pinned_col_major(batch, n, n),
                     pinned_col_major(batch, n, 1))


def test_mirror_entry_point_with_device_outputs(gpu):
    """blastgpu_dposv_mirror_strided with every operand in device memory is plain posv."""
    import torch

    from blast_gb300 import _lib

    rng = np.random.default_rng(5)
    batch, n, r = 100, 30, 2
    A = gpu.col_major((batch,), n, n, "cuda")
    A.copy_(torch.from_numpy(spd_batch(rng, batch, n)))
    B = gpu.col_major((batch,), n, r, "cuda")
    B.copy_(torch.from_numpy(rng.standard_normal((batch, n, r))))
    L, X = gpu.col_major((batch,), n, n, "cuda"), gpu.col_major((batch,), n, r, "cuda")
    wL = torch.empty(batch * n * n, dtype=torch.float64, device="cuda")
    wX = torch.empty(batch * n * r, dtype=torch.float64, device="cuda")
    info = torch.full((batch,), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    _lib.call("blastgpu_dposv_mirror_strided", n, r, A.data_ptr(), n, n * n, B.data_ptr(), n, n * r,
              L.data_ptr(), n, n * n, X.data_ptr(), n, n * r, wL.data_ptr(), wX.data_ptr(), info.data_ptr(),
              batch, stream)
    L2, X2 = gpu.col_major((batch,), n, n, "cuda"), gpu.col_major((batch,), n, r, "cuda")
    info2 = gpu.posv(A, L2, B, X2)
    torch.cuda.synchronize()
    assert not info.any() and not info2.any()
    assert torch.equal(torch.tril(L), torch.tril(L2)) and torch.equal(X, X2)
    assert _lib.lib().blastgpu_dposv_mirror_strided(n, r, A.data_ptr(), n, n * n, B.data_ptr(), n, n * r,
                                                    L.data_ptr(), n, n * n, X.data_ptr(), n, n * r, None,
                                                    wX.data_ptr(), info.data_ptr(), batch, stream) == -15
