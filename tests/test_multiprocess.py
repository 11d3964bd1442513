"""Sharding the additive smoother across ranks (CPU, gloo, world size 2).

The reference distributes patches over MPI ranks and adds ghost contributions to their owners
after each color (compress(VectorOperation::add), schwarz_preconditioner.templates.h:658).
The additive smoother is a sum over patches, so ranks that apply disjoint patch ranges and
sum-reduce their partial vectors reproduce the single-process vmult.  This is the exchange a
multi-GPU run would do; this build runs one GPU per box, so bench.py --gpus N runs replicas.
"""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from oracle import oracle as O
    dim, k, nc = 3, 2, (5, 4, 6)
    N = int(np.prod(nc)) * (k + 1) ** dim
    src = np.random.Generator(np.random.Philox(3)).uniform(-1, 1, N)
    h = O.SchwarzHandle(dim, k, nc, patch_variant=1, omega=0.15)
    P = h.n_patches
    lo, hi = rank * P // world, (rank + 1) * P // world
    part = np.zeros(N)
    h.apply_range(lo, hi, part, src)
    t = torch.from_numpy(part)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    if rank == 0:
        ref = O.schwarz_vmult(dim, k, nc, src, patch_variant=1, omega=0.15)
        np.save(out, np.array([np.abs(t.numpy() - ref).max() / np.abs(ref).max()]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_sharded_vmult(tmp_path):
    import torch.multiprocessing as mp
    from oracle import oracle as O
    O.build()
    out = str(tmp_path / "err.npy")
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    err = float(np.load(out)[0])
    assert err <= 1e-13
