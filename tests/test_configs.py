"""Parity on the benchmark configurations themselves (wemgpu.synthetic: c1,
c2, c3; the seeded synthetic stand-ins of the configurations the reference's
metric names).

* c1 (256 x 200, 1 shot, 64 frequencies, SSF, N = 256): WEM and the Born
  adjoint against the oracle at full size.
* c2 (1024 x 500, 48 shots, 128 frequencies, PSPI with 4 references,
  N = 1024): WEM, Born forward of the configuration's spike perturbation and
  the exact Born adjoint against the oracle on its first two shots (full
  grid and frequency axis); at the full 48 shots, properties that do not
  depend on the size: the first two shots' data and gradient equal the
  two-shot run's, and the exact adjoint passes its dot test.
* c3 (768 x 300, 32 shots, 96 frequencies, the FWI gradient workload):
  WEM and the compat Born adjoint against the oracle on its first two
  shots; the benchmarked fwi_gradient over all 32 shots against the sum of
  four 8-shot blocks, and a two-shot block against the oracle.
rel-L2 <= 1e-4 against the fp32 oracle and its fp64 twin; the measured
errors go to $WEM_PARITY_LOG (JSON lines) when it is set.
"""
import numpy as np
import pytest

from cases import rand_c, rel_l2
from wemgpu import synthetic as S
from wemgpu.params import WEM_DATA_TIME

pytestmark = pytest.mark.gpu
TOL = 1e-4
# a batch against the sum of its shot blocks: the same rows, their images
# added in another order (float sums over thousands of rows: measured
# 1.2e-6 on c2's density gradient)
TOL_SUM = 5e-6


def _cfg(name, **par):
    cfg = S.CONFIGS[name]()
    cfg["par"] = dict(cfg["par"], **par)
    return cfg, S.params_of(cfg)


def test_c1_full_size(gpu_lib, oracle):
    from wemgpu.core import BornOp, WemOp
    cfg, p = _cfg("c1")
    s, rho, wav = cfg["slow"], cfg["rho"], cfg["wavelet"]
    d = np.zeros((p.ns, p.nr, p.nt), np.float32)
    WemOp(p, wav).forward(s, rho, d)
    d_ref = oracle.wem_forward(p, wav, s, rho, kind=WEM_DATA_TIME)
    d64 = oracle.wem_forward(p, wav, s, rho, kind=WEM_DATA_TIME, prec=64)
    assert rel_l2(d, d_ref) <= TOL and rel_l2(d, d64) <= TOL
    g0, g1 = np.zeros_like(s), np.zeros_like(s)
    BornOp(p, wav, s, rho).adjoint(g0, g1, d_ref)
    o0, o1 = oracle.born_adjoint(p, wav, s, rho, d_ref, kind=WEM_DATA_TIME)
    q0, q1 = oracle.born_adjoint(p, wav, s, rho, d_ref, kind=WEM_DATA_TIME, prec=64)
    _record("c1 full size", wem_vs_fp32=rel_l2(d, d_ref), wem_vs_fp64=rel_l2(d, d64),
            born_adj_vs_fp32=max(rel_l2(g0, o0), rel_l2(g1, o1)),
            born_adj_vs_fp64=max(rel_l2(g0, q0), rel_l2(g1, q1)))
    assert rel_l2(g0, o0) <= TOL and rel_l2(g1, o1) <= TOL
    assert rel_l2(g0, q0) <= TOL and rel_l2(g1, q1) <= TOL


def test_c2_first_shots(gpu_lib, oracle):
    from wemgpu.core import BornOp, WemOp
    cfg, p = _cfg("c2", ns=2, adjoint_mode="exact")
    s, rho, wav = cfg["slow"], cfg["rho"], cfg["wavelet"]
    d = np.zeros((p.ns, p.nr, p.nt), np.float32)
    WemOp(p, wav).forward(s, rho, d)
    e = {"wem_vs_fp32": rel_l2(d, oracle.wem_forward(p, wav, s, rho, kind=WEM_DATA_TIME)),
         "wem_vs_fp64": rel_l2(d, oracle.wem_forward(p, wav, s, rho, kind=WEM_DATA_TIME, prec=64))}
    b = BornOp(p, wav, s, rho)
    bd = np.zeros_like(d)
    b.forward(cfg["dslow"], cfg["drho"], bd)
    bd_ref = oracle.born_forward(p, wav, s, rho, cfg["dslow"], cfg["drho"], kind=WEM_DATA_TIME)
    bd64 = oracle.born_forward(p, wav, s, rho, cfg["dslow"], cfg["drho"], kind=WEM_DATA_TIME, prec=64)
    e.update(born_fwd_vs_fp32=rel_l2(bd, bd_ref), born_fwd_vs_fp64=rel_l2(bd, bd64))
    g0, g1 = np.zeros_like(s), np.zeros_like(s)
    b.adjoint(g0, g1, bd_ref)
    o0, o1 = oracle.born_adjoint(p, wav, s, rho, bd_ref, kind=WEM_DATA_TIME, fchunks=16)
    q0, q1 = oracle.born_adjoint(p, wav, s, rho, bd_ref, kind=WEM_DATA_TIME, fchunks=16, prec=64)
    e.update(born_adj_vs_fp32=max(rel_l2(g0, o0), rel_l2(g1, o1)),
             born_adj_vs_fp64=max(rel_l2(g0, q0), rel_l2(g1, q1)))
    _record("c2 first 2 shots (exact adjoint)", **e)
    assert max(e.values()) <= TOL, e


def test_c2_full_size_properties(gpu_lib):
    from wemgpu.core import BornOp, WemOp
    cfg, p = _cfg("c2", adjoint_mode="exact")
    cfg2, p2 = _cfg("c2", ns=2, adjoint_mode="exact")
    s, rho, wav = cfg["slow"], cfg["rho"], cfg["wavelet"]
    # the first two shots of the full batch are the two-shot run
    d = np.zeros((p.ns, p.nr, p.nt), np.float32)
    WemOp(p, wav).forward(s, rho, d)
    d2 = np.zeros((2, p.nr, p.nt), np.float32)
    WemOp(p2, wav).forward(s, rho, d2)
    assert rel_l2(d[:2], d2) <= 1e-6
    # adjoint of data on the first two shots only
    b, b2 = BornOp(p, wav, s, rho), BornOp(p2, wav, s, rho)
    dd = np.zeros_like(d)
    dd[:2] = d2
    g, h = [np.zeros_like(s) for _ in range(2)], [np.zeros_like(s) for _ in range(2)]
    b.adjoint(g[0], g[1], dd)
    b2.adjoint(h[0], h[1], d2)
    assert rel_l2(g[0], h[0]) <= 1e-6 and rel_l2(g[1], h[1]) <= 1e-6
    # dot test of the exact adjoint at full size (d = L n, see test_born_dot_exact)
    rng = np.random.default_rng(21)
    m0, m1 = rand_c(rng, s.shape) * 1e-7, rand_c(rng, s.shape) * 1e-2
    n0, n1 = rand_c(rng, s.shape) * 1e-7, rand_c(rng, s.shape) * 1e-2
    dn = np.zeros_like(d)
    b.forward(n0 + 0.5 * m0, n1 + 0.5 * m1, dn)
    lm = np.zeros_like(d)
    b.forward(m0, m1, lm)
    a0, a1 = np.zeros_like(s), np.zeros_like(s)
    b.adjoint(a0, a1, dn)
    lhs = np.vdot(dn.astype(np.float64), lm.astype(np.float64))
    rhs = (np.vdot(a0.astype(np.complex128), m0.astype(np.complex128)).real +
           np.vdot(a1.astype(np.complex128), m1.astype(np.complex128)).real)
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs), (lhs, rhs)


def test_c3_first_shots(gpu_lib, oracle):
    from wemgpu.core import BornOp, WemOp
    cfg, p = _cfg("c3", ns=2)
    s, rho, wav = cfg["slow"], cfg["rho"], cfg["wavelet"]
    d = np.zeros((p.ns, p.nr, p.nt), np.float32)
    WemOp(p, wav).forward(s, rho, d)
    d_ref = oracle.wem_forward(p, wav, s, rho, kind=WEM_DATA_TIME)
    d64 = oracle.wem_forward(p, wav, s, rho, kind=WEM_DATA_TIME, prec=64)
    e = {"wem_vs_fp32": rel_l2(d, d_ref), "wem_vs_fp64": rel_l2(d, d64)}
    res = (d_ref - oracle.wem_forward(p, wav, cfg["slow_true"], rho, kind=WEM_DATA_TIME)).astype(np.float32)
    g0, g1 = np.zeros_like(s), np.zeros_like(s)
    BornOp(p, wav, s, rho).adjoint(g0, g1, res)
    o0, o1 = oracle.born_adjoint(p, wav, s, rho, res, kind=WEM_DATA_TIME)
    q0, q1 = oracle.born_adjoint(p, wav, s, rho, res, kind=WEM_DATA_TIME, prec=64)
    e.update(born_adj_vs_fp32=max(rel_l2(g0, o0), rel_l2(g1, o1)),
             born_adj_vs_fp64=max(rel_l2(g0, q0), rel_l2(g1, q1)))
    _record("c3 first 2 shots (compat adjoint)", **e)
    assert max(e.values()) <= TOL, e


def _record(name, **errs):
    """Append measured errors to $WEM_PARITY_LOG (a JSON-lines file), when set."""
    import json
    import os
    path = os.environ.get("WEM_PARITY_LOG")
    if path:
        with open(path, "a") as f:
            f.write(json.dumps(dict(config=name, **{k: float(v) for k, v in errs.items()})) + "\n")


def test_c3_full_batch_fwi_gradient(gpu_lib, oracle):
    """The benchmarked call at the benchmarked size: fwi_gradient over all 32
    shots x 96 frequencies (one launch per pass, groups of 8 shots and the
    shaped tail) equals the sum of fwi_gradient over four 8-shot blocks
    (born_prop.cpp:178-232 sums the shots' gradients), loss included, and a
    two-shot block equals the oracle's WEM + residual + Born adjoint."""
    import torch
    from wemgpu.core import FwiOp, WemOp
    from wemgpu.shard import block_par
    cfg, p = _cfg("c3")
    wav = cfg["wavelet"]
    dev = torch.device("cuda")
    st, s0, rho = (torch.from_numpy(cfg[k]).to(dev) for k in ("slow_true", "slow", "rho"))
    d_obs = torch.zeros((p.ns, p.nr, p.nt), dtype=torch.float32, device=dev)
    WemOp(p, wav).forward(st, rho, d_obs)
    g0, g1 = torch.zeros_like(s0), torch.zeros_like(s0)
    loss = FwiOp(p, wav).gradient(s0, rho, d_obs, g0, g1)
    h0, h1 = torch.zeros_like(s0), torch.zeros_like(s0)
    lsum, world = 0.0, 4
    for r in range(world):
        bp = dict(cfg, par=block_par(cfg["par"], world, r))
        pb = S.params_of(bp)
        a0, a1 = torch.zeros_like(s0), torch.zeros_like(s0)
        first = r * (p.ns // world)
        lsum += FwiOp(pb, wav).gradient(s0, rho, d_obs[first:first + pb.ns].contiguous(), a0, a1)
        h0 += a0
        h1 += a1
    torch.cuda.synchronize()
    assert abs(loss - lsum) <= 1e-6 * abs(loss)
    assert rel_l2(g0.cpu().numpy(), h0.cpu().numpy()) <= TOL_SUM
    assert rel_l2(g1.cpu().numpy(), h1.cpu().numpy()) <= TOL_SUM
    # two-shot block against the oracle (fp32 restatement and fp64 twin):
    # its modelling, and its gradient as the oracle's Born adjoint of the
    # block's residual (the residual is a small difference of two modelled
    # data sets, so each side's modelling error would be amplified by
    # |syn| / |res| were the oracle to form it from its own modelling)
    c2, p2 = _cfg("c3", ns=2)
    b0, b1 = torch.zeros_like(s0), torch.zeros_like(s0)
    obs2 = d_obs[:2].contiguous()
    loss2 = FwiOp(p2, wav).gradient(s0, rho, obs2, b0, b1)
    syn2 = torch.zeros_like(obs2)
    WemOp(p2, wav).forward(s0, rho, syn2)
    res = (syn2 - obs2).cpu().numpy()
    assert loss2 == pytest.approx(0.5 * float(np.sum(res.astype(np.float64) ** 2)), rel=1e-6)
    errs = {}
    for prec in (32, 64):
        syn = oracle.wem_forward(p2, wav, cfg["slow"], cfg["rho"], kind=WEM_DATA_TIME, prec=prec)
        o0, o1 = oracle.born_adjoint(p2, wav, cfg["slow"], cfg["rho"], res, kind=WEM_DATA_TIME, prec=prec)
        errs[f"wem_vs_fp{prec}"] = rel_l2(syn2.cpu().numpy(), syn)
        errs[f"grad_vs_fp{prec}"] = max(rel_l2(b0.cpu().numpy(), o0), rel_l2(b1.cpu().numpy(), o1))
    _record("c3 fwi_gradient, 2-shot block", **errs)
    assert max(errs.values()) <= TOL, errs


def test_c2_full_batch_born_adjoint_blocks(gpu_lib):
    """c2 at full size (48 shots, PSPI with 4 references): the Born adjoint of
    the whole batch equals the sum of the adjoints of two 24-shot blocks."""
    import torch
    from wemgpu.core import BornOp
    from wemgpu.shard import block_par
    cfg, p = _cfg("c2", adjoint_mode="exact")
    wav = cfg["wavelet"]
    dev = torch.device("cuda")
    s, rho = torch.from_numpy(cfg["slow"]).to(dev), torch.from_numpy(cfg["rho"]).to(dev)
    ds, dr = torch.from_numpy(cfg["dslow"]).to(dev), torch.from_numpy(cfg["drho"]).to(dev)
    b = BornOp(p, wav, s, rho)
    d = torch.zeros((p.ns, p.nr, p.nt), dtype=torch.float32, device=dev)
    b.forward(ds, dr, d)
    g0, g1 = torch.zeros_like(s), torch.zeros_like(s)
    b.adjoint(g0, g1, d)
    h0, h1 = torch.zeros_like(s), torch.zeros_like(s)
    for r in range(2):
        pb = S.params_of(dict(cfg, par=block_par(cfg["par"], 2, r)))
        a0, a1 = torch.zeros_like(s), torch.zeros_like(s)
        bb = BornOp(pb, wav, s, rho)
        db = torch.zeros((pb.ns, pb.nr, pb.nt), dtype=torch.float32, device=dev)
        bb.forward(ds, dr, db)
        first = r * (p.ns // 2)
        assert rel_l2(db.cpu().numpy(), d[first:first + pb.ns].cpu().numpy()) <= 1e-6
        bb.adjoint(a0, a1, d[first:first + pb.ns].contiguous())
        h0 += a0
        h1 += a1
    torch.cuda.synchronize()
    assert rel_l2(g0.cpu().numpy(), h0.cpu().numpy()) <= TOL_SUM
    assert rel_l2(g1.cpu().numpy(), h1.cpu().numpy()) <= TOL_SUM
