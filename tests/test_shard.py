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


# ---------------------------------------------------------------- bench.py's
# weak-scaling path: every rank runs bench.rank_workload's block of one
# survey and bench.reduce_gradients sums the gradients (gloo here)

def _tiny_cfg():
    p, par, wav, s, rho = small_case(ns=3)
    # shot interval of 12 cells: two ranks interleave at 6 cells
    par = dict(par, osx=60.0, dsx=120.0)
    s_true = (s.real * (1 + 0.03 * np.cos(np.arange(s.shape[1]) / 5.0))[None, :] + 1j * s.imag).astype(np.complex64)
    return dict(par=par, nx=p.nx, nz=p.nz, dx=p.dx, dz=p.dz, nt=p.nt, dt=p.dt, wavelet=wav, slow=s,
                slow_true=s_true, rho=rho)


def _params(cfg):
    from wemgpu.params import make_params
    return make_params(cfg["par"], nx=cfg["nx"], nz=cfg["nz"], dx=cfg["dx"], dz=cfg["dz"], nt=cfg["nt"],
                       dt=cfg["dt"])


def _bench_rank(rank, world, port, out, use_gpu):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for d in (root, os.path.join(root, "wem-fwi_gb300"), os.path.join(root, "tests")):
        sys.path.insert(0, d)
    import torch
    import torch.distributed as dist
    import bench
    from test_shard import _params, _tiny_cfg
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    cfg = bench.rank_workload(_tiny_cfg(), rank, world)
    p = _params(cfg)
    if use_gpu:
        from wemgpu.core import FwiOp, WemOp
        dev = torch.device("cuda:0")
        st, s0, rh = (torch.from_numpy(cfg[k]).to(dev) for k in ("slow_true", "slow", "rho"))
        d = torch.zeros((p.ns, p.nr, p.nt), dtype=torch.float32, device=dev)
        WemOp(p, cfg["wavelet"]).forward(st, rh, d)
        g0, g1 = torch.zeros_like(s0), torch.zeros_like(s0)
        FwiOp(p, cfg["wavelet"]).gradient(s0, rh, d, g0, g1)
        torch.cuda.synchronize()
        g0, g1 = g0.cpu(), g1.cpu()
    else:
        from oracle import oracle as O
        d = O.wem_forward(p, cfg["wavelet"], cfg["slow_true"], cfg["rho"], kind=0, prec=64)
        syn = O.wem_forward(p, cfg["wavelet"], cfg["slow"], cfg["rho"], kind=0, prec=64)
        a0, a1 = O.born_adjoint(p, cfg["wavelet"], cfg["slow"], cfg["rho"], syn - d, kind=0, prec=64)
        g0, g1 = torch.from_numpy(a0.copy()), torch.from_numpy(a1.copy())
    bench.reduce_gradients(g0, g1, world)
    if rank == 0:
        np.save(out + "_g0.npy", g0.numpy())
        np.save(out + "_g1.npy", g1.numpy())
    dist.barrier()
    dist.destroy_process_group()


def _survey(world):
    from wemgpu.shard import survey_par
    cfg = _tiny_cfg()
    return dict(cfg, par=survey_par(cfg["par"], world))


def test_interleaved_blocks_tile_the_survey():
    from wemgpu.shard import interleave_par, survey_par
    import bench
    cfg = _tiny_cfg()
    xs = []
    for r in range(4):
        p = _params(bench.rank_workload(cfg, r, 4))
        xs += [p.osx + k * p.dsx for k in range(p.ns)]
    ps = _params(dict(cfg, par=survey_par(cfg["par"], 4)))
    assert np.allclose(sorted(xs), [ps.osx + k * ps.dsx for k in range(ps.ns)])
    assert interleave_par(cfg["par"], 1, 0) == dict(cfg["par"])


def test_bench_two_rank_gradient_matches_survey(tmp_path, oracle):
    import torch.multiprocessing as mp
    world, port = 2, _free_port()
    out = str(tmp_path / "b")
    mp.start_processes(_bench_rank, args=(world, port, out, False), nprocs=world, start_method="spawn")
    cfg = _survey(world)
    p = _params(cfg)
    d = oracle.wem_forward(p, cfg["wavelet"], cfg["slow_true"], cfg["rho"], kind=0, prec=64)
    syn = oracle.wem_forward(p, cfg["wavelet"], cfg["slow"], cfg["rho"], kind=0, prec=64)
    g0, g1 = oracle.born_adjoint(p, cfg["wavelet"], cfg["slow"], cfg["rho"], syn - d, kind=0, prec=64)
    assert rel_l2(np.load(out + "_g0.npy"), g0) < 1e-6
    assert rel_l2(np.load(out + "_g1.npy"), g1) < 1e-6


@pytest.mark.gpu
def test_bench_two_rank_gradient_on_gpu_matches_one_process(tmp_path, gpu_lib):
    """The library's fwi_gradient on each rank's block (both ranks on one
    GPU, gloo on host copies: no kernel waits on another rank) summed by
    bench.reduce_gradients equals one call over the whole survey."""
    import torch
    import torch.multiprocessing as mp
    from wemgpu.core import FwiOp, WemOp
    world, port = 2, _free_port()
    out = str(tmp_path / "g")
    mp.start_processes(_bench_rank, args=(world, port, out, True), nprocs=world, start_method="spawn")
    cfg = _survey(world)
    p = _params(cfg)
    dev = torch.device("cuda:0")
    st, s0, rh = (torch.from_numpy(cfg[k]).to(dev) for k in ("slow_true", "slow", "rho"))
    d = torch.zeros((p.ns, p.nr, p.nt), dtype=torch.float32, device=dev)
    WemOp(p, cfg["wavelet"]).forward(st, rh, d)
    g0, g1 = torch.zeros_like(s0), torch.zeros_like(s0)
    FwiOp(p, cfg["wavelet"]).gradient(s0, rh, d, g0, g1)
    torch.cuda.synchronize()
    assert rel_l2(np.load(out + "_g0.npy"), g0.cpu().numpy()) < 1e-5
    assert rel_l2(np.load(out + "_g1.npy"), g1.cpu().numpy()) < 1e-5
