"""Conformal-map geometry (cmap = 1, 2; PropParam.h:88-137, conformal/src)
of WEM and BornFull.

CPU: the oracle's known answer (a rotation by 0 of a grid starting at the
origin is the identity, so cmap 2 must equal the unmapped operators
exactly), its fp32/fp64 twins, and host validation of the library.
GPU: the library against the oracle for both maps, WEM, Born forward and
both Born adjoints, on the warp-per-row and the shared-memory kernels, and
the single-call FWI gradient; rel-L2 <= 1e-4 as for the unmapped operators.
"""
import ctypes

import numpy as np
import pytest

from cases import cmap_case, rand_c, rel_l2
from wemgpu.params import WEM_DATA_TIME

TOL = 1e-4


def _unmapped(p):
    q = p.copy()
    q.cmap = 0
    return q


def test_oracle_rotation_by_zero_is_the_identity(oracle):
    p, _, wav, s, rho = cmap_case(2, angles=[0.0, 0.0, 0.0])
    q = _unmapped(p)
    d = oracle.wem_forward(p, wav, s, rho)
    assert np.array_equal(d, oracle.wem_forward(q, wav, s, rho))
    g = oracle.born_adjoint(p, wav, s, rho, d)
    g0 = oracle.born_adjoint(q, wav, s, rho, d)
    assert np.array_equal(g[0], g0[0]) and np.array_equal(g[1], g0[1])
    rng = np.random.default_rng(0)
    dm, dr = rand_c(rng, s.shape) * 1e-8, rand_c(rng, s.shape) * 1e-2
    assert np.array_equal(oracle.born_forward(p, wav, s, rho, dm, dr), oracle.born_forward(q, wav, s, rho, dm, dr))


@pytest.mark.parametrize("cmap", [1, 2])
def test_oracle_twins_agree(oracle, cmap):
    p, _, wav, s, rho = cmap_case(cmap)
    d = oracle.wem_forward(p, wav, s, rho)
    assert np.isfinite(d).all() and np.abs(d).max() > 0
    assert rel_l2(d, oracle.wem_forward(p, wav, s, rho, prec=64)) <= 1e-4
    g = oracle.born_adjoint(p, wav, s, rho, d)
    g64 = oracle.born_adjoint(p, wav, s, rho, d, prec=64)
    assert rel_l2(g[0], g64[0]) <= 1e-4 and rel_l2(g[1], g64[1]) <= 1e-4


def test_log_map_needs_two_receivers_and_angles(oracle):
    from wemgpu._lib import WemError, call
    p, _, wav, s, rho = cmap_case(1, nr=1)
    with pytest.raises(RuntimeError):
        oracle.wem_forward(p, wav, s, rho)
    h = ctypes.c_void_p()
    with pytest.raises(WemError) as e:
        call("wem_create", ctypes.byref(p), wav.ctypes.data_as(ctypes.c_void_p), ctypes.byref(h))
    assert e.value.code == 1
    p, _, wav, s, rho = cmap_case(2)
    p.cmap_angles = None
    with pytest.raises(WemError):
        call("wem_create", ctypes.byref(p), wav.ctypes.data_as(ctypes.c_void_p), ctypes.byref(h))


# (cmap, case options): warp-per-row kernels need N = nx + 2 (pad + tap) = 32 E
GPU_CASES = {
    "log_warp": (1, dict(nx=256, nz=40)),
    "log_warp_pad_tap": (1, dict(nx=240, nz=32, pad=4, tap=4, ngs=1)),
    "log_smem_pspi_nref2": (1, dict(nx=60, nz=24, pad=4, tap=2, prop="pspi", nref=2)),
    "rot_warp": (2, dict(nx=256, nz=40)),
    "rot_smem_pad": (2, dict(nx=70, nz=28, pad=5, tap=3, ngs=2, angles=[0.7, -0.3, 0.2])),
    "rot_warp_exact": (2, dict(nx=384, nz=24, adjoint_mode="exact")),
}


def _rel(a, b):
    return rel_l2(a, b)


@pytest.mark.gpu
@pytest.mark.parametrize("case", list(GPU_CASES))
def test_cmap_operators_match_oracle(gpu_lib, oracle, case):
    from wemgpu.core import BornOp, WemOp
    cm, kw = GPU_CASES[case]
    p, _, wav, s, rho = cmap_case(cm, **kw)
    # WEM forward, frequency and time data
    d_ref = oracle.wem_forward(p, wav, s, rho)
    w = WemOp(p, wav)
    d = np.zeros_like(d_ref)
    w.forward(s, rho, d)
    assert _rel(d, d_ref) <= TOL
    dt_ref = oracle.wem_forward(p, wav, s, rho, kind=WEM_DATA_TIME)
    dt = np.zeros_like(dt_ref)
    w.forward(s, rho, dt)
    assert _rel(dt, dt_ref) <= TOL
    # Born forward and adjoint at the same background
    rng = np.random.default_rng(3)
    dm, dr = rand_c(rng, s.shape) * 1e-8, rand_c(rng, s.shape) * 1e-2
    b = BornOp(p, wav, s, rho)
    bd_ref = oracle.born_forward(p, wav, s, rho, dm, dr)
    bd = np.zeros_like(bd_ref)
    b.forward(dm, dr, bd)
    assert _rel(bd, bd_ref) <= TOL
    # the log map's Jacobian spreads slowness^2 over four decades, and the
    # fp32 oracle's own gradient then differs from its fp64 twin by up to
    # ~2e-4: the library is held to the fp64 gradient within twice that
    # fp32 error (and never looser than TOL)
    g_ref = oracle.born_adjoint(p, wav, s, rho, d_ref)
    g64 = oracle.born_adjoint(p, wav, s, rho, d_ref, prec=64)
    g0, g1 = np.zeros_like(s), np.zeros_like(s)
    b.adjoint(g0, g1, d_ref)
    for got, o32, o64 in ((g0, g_ref[0], g64[0]), (g1, g_ref[1], g64[1])):
        assert _rel(got, o64) <= max(TOL, 2 * _rel(o32, o64))
    # add = 1 accumulates onto the caller's arrays
    h0, h1 = g0.copy(), g1.copy()
    b.adjoint(h0, h1, d_ref, add=True)
    assert _rel(h0, 2 * g0) <= 1e-6 and _rel(h1, 2 * g1) <= 1e-6


@pytest.mark.gpu
def test_cmap_rotation_by_zero_matches_unmapped_gpu(gpu_lib):
    from wemgpu.core import BornOp, WemOp
    p, _, wav, s, rho = cmap_case(2, nx=256, nz=40, angles=[0.0, 0.0, 0.0])
    q = _unmapped(p)
    d, d0 = np.zeros((3, p.nr, p.nt + p.tpad), np.complex64), None
    WemOp(p, wav).forward(s, rho, d)
    d0 = np.zeros_like(d)
    WemOp(q, wav).forward(s, rho, d0)
    assert _rel(d, d0) <= 1e-6
    g, g0 = [np.zeros_like(s) for _ in range(2)], [np.zeros_like(s) for _ in range(2)]
    BornOp(p, wav, s, rho).adjoint(g[0], g[1], d0)
    BornOp(q, wav, s, rho).adjoint(g0[0], g0[1], d0)
    assert _rel(g[0], g0[0]) <= 1e-6 and _rel(g[1], g0[1]) <= 1e-6


@pytest.mark.gpu
@pytest.mark.parametrize("cmap", [1, 2])
def test_cmap_fwi_gradient_is_wem_then_born_adjoint(gpu_lib, oracle, cmap):
    import torch

    from wemgpu.core import BornOp, FwiOp, WemOp
    p, _, wav, s, rho = cmap_case(cmap, nx=256, nz=40)
    zz, xx = np.meshgrid(np.arange(p.nz), np.arange(p.nx), indexing="ij")
    s_true = (s * (1 + 0.03 * np.exp(-((zz - 20) ** 2 + (xx - 128) ** 2) / 50.0))).astype(np.complex64)
    d_obs = oracle.wem_forward(p, wav, s_true, rho, kind=WEM_DATA_TIME)
    # the same gradient from the separate operators of the library
    syn = np.zeros_like(d_obs)
    WemOp(p, wav).forward(s, rho, syn)
    res = syn - d_obs
    g_ref = [np.zeros_like(s), np.zeros_like(s)]
    BornOp(p, wav, s, rho).adjoint(g_ref[0], g_ref[1], res)
    loss_ref = 0.5 * float(np.sum(res.astype(np.float64) ** 2))
    dev = torch.device("cuda")
    g0 = torch.zeros(s.shape, dtype=torch.complex64, device=dev)
    g1 = torch.zeros_like(g0)
    loss = FwiOp(p, wav).gradient(torch.from_numpy(s).to(dev), torch.from_numpy(rho).to(dev),
                                  torch.from_numpy(d_obs).to(dev), g0, g1)
    assert abs(loss - loss_ref) <= 1e-5 * loss_ref
    assert _rel(g0.cpu().numpy(), g_ref[0]) <= 1e-5 and _rel(g1.cpu().numpy(), g_ref[1]) <= 1e-5
    # and the oracle's loss
    loss_o = 0.5 * float(np.sum((oracle.wem_forward(p, wav, s, rho, kind=WEM_DATA_TIME) - d_obs).astype(np.float64) ** 2))
    assert abs(loss - loss_o) <= 1e-3 * loss_o
