"""Shot sharding across two gloo ranks on CPU: the gradient summed over
rank blocks equals the single-process gradient, and data blocks tile the
full data.  The per-rank compute is the oracle (these are host-logic tests;
the GPU path is the same library call per rank)."""
import os
import socket

import numpy as np
import pytest

from cases import rel_l2, small_case


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    sys.path.insert(0, os.path.join(root, "wem-fwi_gb300"))
    sys.path.insert(0, os.path.join(root, "tests"))
    import torch
    import torch.distributed as dist
    from cases import small_case
    from oracle import oracle as O
    from wemgpu.params import make_params
    from wemgpu.shard import allreduce_sum, block_par
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    p, par, wav, s, rho = small_case(ns=5)
    bp = block_par(par, world, rank)
    pl = make_params(bp, nx=p.nx, nz=p.nz, dx=p.dx, dz=p.dz, nt=p.nt, dt=p.dt)
    d = O.wem_forward(pl, wav, s, rho, kind=0, prec=64)
    g0, _ = O.born_adjoint(pl, wav, s, rho, d, kind=0, prec=64)
    t = torch.from_numpy(g0.copy())
    allreduce_sum(t)
    if rank == 0:
        np.save(out + "_grad.npy", t.numpy())
    np.save(out + f"_data{rank}.npy", d)
    dist.barrier()
    dist.destroy_process_group()


def test_shot_blocks():
    from wemgpu.shard import shot_block
    blocks = [shot_block(10, 3, r) for r in range(3)]
    assert blocks == [(0, 4), (4, 3), (7, 3)]
    assert sum(c for _, c in blocks) == 10


def test_two_rank_gradient_matches_single_process(tmp_path, oracle):
    import torch.multiprocessing as mp
    world, port = 2, _free_port()
    out = str(tmp_path / "r")
    mp.start_processes(_rank, args=(world, port, out), nprocs=world, start_method="spawn")
    p, par, wav, s, rho = small_case(ns=5)
    d = oracle.wem_forward(p, wav, s, rho, kind=0, prec=64)
    g0, _ = oracle.born_adjoint(p, wav, s, rho, d, kind=0, prec=64)
    assert rel_l2(np.load(out + "_grad.npy"), g0) < 1e-6
    d_sh = np.concatenate([np.load(out + f"_data{r}.npy") for r in range(world)], 0)
    assert rel_l2(d_sh, d) < 1e-6
