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
  shots.
rel-L2 <= 1e-4 against the fp32 oracle, as every parity test.
"""
import numpy as np
import pytest

from cases import rand_c, rel_l2
from wemgpu import synthetic as S
from wemgpu.params import WEM_DATA_TIME

pytestmark = pytest.mark.gpu
TOL = 1e-4


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
    assert rel_l2(d, d_ref) <= TOL
    g0, g1 = np.zeros_like(s), np.zeros_like(s)
    BornOp(p, wav, s, rho).adjoint(g0, g1, d_ref)
    o0, o1 = oracle.born_adjoint(p, wav, s, rho, d_ref, kind=WEM_DATA_TIME)
    assert rel_l2(g0, o0) <= TOL and rel_l2(g1, o1) <= TOL


def test_c2_first_shots(gpu_lib, oracle):
    from wemgpu.core import BornOp, WemOp
    cfg, p = _cfg("c2", ns=2, adjoint_mode="exact")
    s, rho, wav = cfg["slow"], cfg["rho"], cfg["wavelet"]
    d = np.zeros((p.ns, p.nr, p.nt), np.float32)
    WemOp(p, wav).forward(s, rho, d)
    assert rel_l2(d, oracle.wem_forward(p, wav, s, rho, kind=WEM_DATA_TIME)) <= TOL
    b = BornOp(p, wav, s, rho)
    bd = np.zeros_like(d)
    b.forward(cfg["dslow"], cfg["drho"], bd)
    bd_ref = oracle.born_forward(p, wav, s, rho, cfg["dslow"], cfg["drho"], kind=WEM_DATA_TIME)
    assert rel_l2(bd, bd_ref) <= TOL
    g0, g1 = np.zeros_like(s), np.zeros_like(s)
    b.adjoint(g0, g1, bd_ref)
    o0, o1 = oracle.born_adjoint(p, wav, s, rho, bd_ref, kind=WEM_DATA_TIME, fchunks=16)
    assert rel_l2(g0, o0) <= TOL and rel_l2(g1, o1) <= TOL


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
    assert rel_l2(d, d_ref) <= TOL
    res = (d_ref - oracle.wem_forward(p, wav, cfg["slow_true"], rho, kind=WEM_DATA_TIME)).astype(np.float32)
    g0, g1 = np.zeros_like(s), np.zeros_like(s)
    BornOp(p, wav, s, rho).adjoint(g0, g1, res)
    o0, o1 = oracle.born_adjoint(p, wav, s, rho, res, kind=WEM_DATA_TIME)
    assert rel_l2(g0, o0) <= TOL and rel_l2(g1, o1) <= TOL
