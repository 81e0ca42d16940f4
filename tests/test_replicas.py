"""Replicas-only multi-GPU logic, on CPU with the gloo backend (world size 2): cost-balanced
sharding of a ragged batch, the max-over-ranks step time, and the host-side gather of per-instance
status, with each rank checking its shard against the oracle."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, result_dir):
    import torch.distributed as dist

    from blast_gb300.replicas import gather_info, max_over_ranks, shard_by_cost
    from oracle import oracle as orc

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    rng = np.random.default_rng(7)
    ns = rng.integers(4, 40, 37)
    parts = shard_by_cost(ns.astype(float) ** 3, world)
    mine = parts[rank]
    # each rank factors its own instances (the oracle stands in for the GPU work here)
    infos = []
    for i in mine:
        n = int(ns[i])
        G = np.random.default_rng(100 + int(i)).standard_normal((n, n))
        A = np.asfortranarray(G @ G.T + n * np.eye(n))
        if i % 9 == 0:
            A[0, 0] = -1.0  # a planted failure, reported through info
        L = np.zeros((n, n), order="F")
        infos.append(orc.potrf(A, L))
    t = max_over_ranks(float(rank + 1))
    full = gather_info(np.asarray(infos, dtype=np.int32), mine, len(ns))
    if rank == 0:
        np.save(os.path.join(result_dir, "full.npy"), full)
        np.save(os.path.join(result_dir, "t.npy"), np.array([t]))
    dist.barrier()
    dist.destroy_process_group()


def test_shard_by_cost_balances():
    from blast_gb300.replicas import shard_by_cost

    rng = np.random.default_rng(1)
    costs = rng.integers(4, 257, 1000).astype(float) ** 3
    parts = shard_by_cost(costs, 4)
    assert sorted(np.concatenate(parts).tolist()) == list(range(1000))
    loads = [costs[p].sum() for p in parts]
    assert max(loads) / min(loads) < 1.02


def test_gloo_world2_replicas(tmp_path):
    pytest.importorskip("torch.distributed")
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn")
    full = np.load(tmp_path / "full.npy")
    t = np.load(tmp_path / "t.npy")
    assert t[0] == 2.0  # the slowest rank's time
    ns = np.random.default_rng(7).integers(4, 40, 37)
    expect = np.array([1 if i % 9 == 0 else 0 for i in range(len(ns))], dtype=np.int32)
    assert np.array_equal(full, expect)


def test_bench_reference_arm_under_torchrun(tmp_path):
    """`bench.py --impl reference` launched like the N-GPU bench (torch.distributed.run, two ranks):
    rank 0 alone times the CPU restatement and prints one JSON line; the other rank exits 0."""
    import json
    import subprocess
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parent.parent
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), str(root / "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1"]
    out = subprocess.run(cmd, cwd=root, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [json.loads(x) for x in out.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["unit"] == "matrices/s" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
    # the workload-defining keys are the ones the GPU arm prints (bench.contract_config)
    sys.path.insert(0, str(root))
    import bench

    assert line["config"] == bench.contract_config()
