"""Multi-GPU here means independent replicas: acquisitions are sharded across
ranks, no data-path collective. This checks, with two gloo ranks on the CPU, that
sharding acquisitions by rank and reducing (sum of volumes, max of times) gives
the same volumes as one process computing them all."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def acquisitions():
    from bf_cases import small_params
    bp = small_params(S=256, C=8, T=8, points=(8, 1, 8))
    return bp, [3, 4, 5, 6]


def beamform_cpu(bp, seed):
    from bf_cases import small_raw
    from ogl_beamforming_cuda_gb300 import abi
    from oracle.bf_oracle import OraclePipeline
    orc = OraclePipeline()
    orc.bp = bp
    orc.shaders = [abi.SHADER["Decode"], abi.SHADER["Demodulate"], abi.SHADER["DAS"]]
    orc.create_kaiser(5.65, 5e6, 25e6, 16, 0)
    orc.focal[1::2] = np.inf
    return orc.compute(small_raw(bp, seed=seed, n_points=4, n_speckle=0))["frame"]


def worker(rank, world, port, out_path):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), BF_ORACLE_THREADS="1")
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    bp, seeds = acquisitions()
    mine = seeds[rank::world]
    vols = {s: beamform_cpu(bp, s) for s in mine}
    done = torch.tensor([float(len(vols)), 1.0 + rank], dtype=torch.float64)
    total = done.clone()
    dist.all_reduce(total[:1], op=dist.ReduceOp.SUM)
    tmax = done[1:].clone()
    dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
    np.savez(out_path + f".{rank}.npz", total=total[0].item(), tmax=tmax.item(),
             **{f"v{s}": v for s, v in vols.items()})
    dist.destroy_process_group()


def test_replicas_shard_acquisitions(tmp_path):
    import torch.multiprocessing as mp
    world = 2
    out = str(tmp_path / "r")
    mp.start_processes(worker, args=(world, free_port(), out), nprocs=world, start_method="spawn", join=True)
    bp, seeds = acquisitions()
    got = {}
    for r in range(world):
        d = np.load(out + f".{r}.npz")
        assert d["total"] == len(seeds)
        assert d["tmax"] == world
        got.update({int(k[1:]): d[k] for k in d.files if k.startswith("v")})
    assert sorted(got) == seeds
    for s in seeds:
        assert np.array_equal(got[s], beamform_cpu(bp, s))
