"""3D one-way operators on planes (no reference counterpart: the reference
propagates 2D slices).  Pinned at ny = 1, where the 3D operators must equal
the 2D ones (WEM, propagator/src/wem_prop.cpp:9-78; BornRefl,
ext_born_refl.cpp:8-105; the SSF / PSPI step, SSF.cpp:8-60, PSPI.cpp:8-53):
the numpy 3D oracle against the C++ 2D oracle on the CPU, the GPU 3D path
against the GPU 2D path and the oracle.  Beyond ny = 1 the GPU is held to
the numpy 3D oracle, with dot tests and checkpointed = stored.
"""
import numpy as np
import pytest

from cases import layered_model, rand_c, rel_l2, ricker
from wemgpu.params import WEM_DATA_FREQ, WEM_DATA_TIME, make_params, make_params3d


def case3d(nx=24, ny=24, nz=8, pad=2, pady=2, prop="ssf", nref=1, ns=2, nt=64, dt=0.008, fmin=6.0, fmax=12.0,
           phase_law="ispc", seed=7, ngs=1, ngr=0, rstep=2, N=256, refl=False):
    """refl: the plane lengths of the reflectivity pair, which does not pad
    the model (pad, pad_y are taper widths there): N = nx + 2 tap."""
    rng = np.random.default_rng(seed)
    s2d, rho2d = layered_model(nz, nx, seed)
    # a slowness that varies along y too
    wob = 1 + 0.03 * np.sin(np.linspace(0, 3, ny))[None, :, None]
    s = (s2d.real[:, None, :] * wob - 1j * 1e-9).astype(np.complex64)
    rho = np.ascontiguousarray(np.repeat(rho2d[:, None, :], ny, 1))
    d = 10.0
    sx = [d * (nx // 3 + 4 * k) for k in range(ns)]
    sy = [d * (ny // 3 + 5 * k) if ny > 1 else 0.0 for k in range(ns)]
    sz = [0.0] * ns
    rx, ry = np.meshgrid(np.arange(0, nx, rstep) * d, np.arange(0, ny, rstep) * d)
    rx, ry = rx.ravel(), ry.ravel()
    rz = np.zeros_like(rx)
    grid_pad, grid_pady = (0, 0) if refl else (pad, pady)
    tap = (N - nx - 2 * grid_pad) // 2
    tapy = (N - ny - 2 * grid_pady) // 2 if ny > 1 else 0
    par = dict(prop=prop, nref=nref, tap=tap, pad=pad, fmin=fmin, fmax=fmax, ngs=ngs, ngr=ngr, phase_law=phase_law)
    q = make_params3d(par, nx=nx, ny=ny, nz=nz, dx=d, dy=d, dz=d, nt=nt, dt=dt, sx=sx, sy=sy, sz=sz, rx=rx, ry=ry,
                      rz=rz, pad_y=pady if ny > 1 else 0, tap_y=tapy)
    wav = ricker(nt, dt, 10.0)
    return q, par, wav, s, rho


def params2d(q, par):
    p = q.p
    m = dict(par, sx=[p.src_x[i] for i in range(p.ns)], sz=[p.src_z[i] for i in range(p.ns)],
             rx=[p.rec_x[i] for i in range(p.nr)], rz=[p.rec_z[i] for i in range(p.nr)])
    return make_params(m, nx=p.nx, nz=p.nz, dx=p.dx, dz=p.dz, nt=p.nt, dt=p.dt)


# ------------------------------------------------------------ oracle (CPU)

@pytest.mark.parametrize("prop,nref", [("ssf", 1), ("pspi", 3)])
def test_oracle3d_single_line_is_2d(oracle, prop, nref):
    from oracle import oracle3d as O3
    q, par, wav, s, rho = case3d(ny=1, prop=prop, nref=nref, nx=40, rstep=1)
    p2 = params2d(q, par)
    s2, r2 = np.ascontiguousarray(s[:, 0]), np.ascontiguousarray(rho[:, 0])
    for prec in (32, 64):
        d3 = O3.wem_forward(q, wav, s, rho, kind=WEM_DATA_FREQ, prec=prec)
        d2 = oracle.wem_forward(p2, wav, s2, r2, kind=WEM_DATA_FREQ, prec=prec)
        assert rel_l2(d3, d2) < (2e-5 if prec == 32 else 1e-10), (prec, rel_l2(d3, d2))
    nf = oracle.count_freqs(p2)[0]
    rng = np.random.default_rng(1)
    m = rand_c(rng, s.shape)
    d3 = O3.refl_forward(q, wav, s, m, kind=WEM_DATA_FREQ, prec=64)
    d2 = oracle.bornrefl_forward(p2, wav, s2, np.repeat(m[:, 0][None], nf, 0), kind=WEM_DATA_FREQ, prec=64)
    assert rel_l2(d3, d2) < 1e-6
    g = rand_c(rng, d3.shape)
    i3 = O3.refl_adjoint(q, wav, s, g, kind=WEM_DATA_FREQ, prec=64)
    i2 = oracle.bornrefl_adjoint(p2, wav, s2, g, kind=WEM_DATA_FREQ, prec=64).astype(np.complex128).sum(0)
    assert rel_l2(i3[:, 0], i2) < 1e-6


def test_oracle3d_dot():
    from oracle import oracle3d as O3
    q, par, wav, s, rho = case3d(nz=5, ns=1)
    rng = np.random.default_rng(2)
    m = rand_c(rng, s.shape)
    d = O3.refl_forward(q, wav, s, m, kind=WEM_DATA_FREQ, prec=64)
    g = rand_c(rng, d.shape)
    i = O3.refl_adjoint(q, wav, s, g, kind=WEM_DATA_FREQ, prec=64)
    a = np.vdot(d.astype(np.complex128), g.astype(np.complex128))
    b = np.vdot(m.astype(np.complex128), i.astype(np.complex128))
    assert abs(a - b) / abs(a) < 1e-6


# ------------------------------------------------------------------- GPU

@pytest.mark.gpu
@pytest.mark.parametrize("prop,nref", [("ssf", 1), ("pspi", 3)])
def test_3d_single_line_is_2d_gpu(gpu_lib, oracle, prop, nref):
    from wemgpu.core import BornReflOp, Refl3DOp, Wem3DOp, WemOp
    q, par, wav, s, rho = case3d(ny=1, prop=prop, nref=nref, nx=40, rstep=1)
    p2 = params2d(q, par)
    s2, r2 = np.ascontiguousarray(s[:, 0]), np.ascontiguousarray(rho[:, 0])
    d3 = np.zeros((q.p.ns, q.p.nr, q.p.nt), np.float32)
    Wem3DOp(q, wav).forward(s, rho, d3)
    d2 = np.zeros_like(d3)
    WemOp(p2, wav).forward(s2, r2, d2)
    assert rel_l2(d3, d2) < 1e-5
    o = oracle.wem_forward(p2, wav, s2, r2, kind=WEM_DATA_TIME, prec=64)
    assert rel_l2(d3, o) < 1e-4
    qr, par_r, _, _, _ = case3d(ny=1, prop=prop, nref=nref, nx=40, rstep=1, refl=True)
    op = Refl3DOp(qr, wav, s)
    ref = BornReflOp(params2d(qr, par_r), wav, s2)
    nf = ref.nfreq()
    rng = np.random.default_rng(3)
    m = rand_c(rng, s.shape)
    op.forward(m, d3)
    ref.forward(np.ascontiguousarray(np.repeat(m[:, 0][None], nf, 0)), d2)
    assert rel_l2(d3, d2) < 1e-5
    g = rng.standard_normal(d3.shape).astype(np.float32)
    i3 = np.zeros_like(m)
    op.adjoint(i3, g)
    i2 = np.zeros((nf,) + s2.shape, np.complex64)
    ref.adjoint(i2, g)
    assert rel_l2(i3[:, 0], i2.astype(np.complex128).sum(0)) < 1e-5


GPU3 = [dict(), dict(prop="pspi", nref=3), dict(phase_law="exact_kz", ngr=1), dict(N=384, nx=30, ny=20, pad=4, pady=0)]


@pytest.mark.gpu
@pytest.mark.parametrize("kw", GPU3, ids=lambda k: "-".join(f"{a}{b}" for a, b in k.items()) or "ssf")
def test_3d_matches_oracle(gpu_lib, kw):
    from oracle import oracle3d as O3
    from wemgpu.core import Refl3DOp, Wem3DOp
    q, par, wav, s, rho = case3d(**kw)
    d = np.zeros((q.p.ns, q.p.nr, q.p.nt), np.float32)
    Wem3DOp(q, wav).forward(s, rho, d)
    for prec in (32, 64):
        o = O3.wem_forward(q, wav, s, rho, kind=WEM_DATA_TIME, prec=prec)
        assert rel_l2(d, o) < 1e-4, (prec, rel_l2(d, o))
    q, par, wav, s, rho = case3d(refl=True, **kw)
    op = Refl3DOp(q, wav, s)
    rng = np.random.default_rng(4)
    m = rand_c(rng, s.shape)
    op.forward(m, d)
    o = O3.refl_forward(q, wav, s, m, kind=WEM_DATA_TIME, prec=64)
    assert rel_l2(d, o) < 1e-4, rel_l2(d, o)
    g = rng.standard_normal(d.shape).astype(np.float32)
    img = np.zeros_like(m)
    op.adjoint(img, g)
    o = O3.refl_adjoint(q, wav, s, g, kind=WEM_DATA_TIME, prec=64)
    assert rel_l2(img, o) < 1e-4, rel_l2(img, o)
    # dot test with bins
    nb = q.p.nt + q.p.tpad
    df = np.zeros((q.p.ns, q.p.nr, nb), np.complex64)
    op.forward(m, df)
    gf = rand_c(rng, df.shape)
    im2 = np.zeros_like(m)
    op.adjoint(im2, gf)
    a = np.vdot(df.astype(np.complex128), gf.astype(np.complex128))
    b = np.vdot(m.astype(np.complex128), im2.astype(np.complex128))
    assert abs(a - b) / abs(a) < 1e-5


@pytest.mark.gpu
def test_3d_checkpointing_is_bit_exact(gpu_lib):
    from wemgpu.core import Refl3DOp, Wem3DOp
    q, par, wav, s, rho = case3d(nz=11, prop="pspi", nref=2)
    qr = case3d(nz=11, prop="pspi", nref=2, refl=True)[0]
    rng = np.random.default_rng(5)
    m = rand_c(rng, s.shape)
    op = Refl3DOp(qr, wav, s)
    wem = Wem3DOp(q, wav)
    d0 = np.zeros((q.p.ns, q.p.nr, q.p.nt), np.float32)
    op.forward(m, d0)
    w0 = np.zeros_like(d0)
    wem.forward(s, rho, w0)
    for ck in (2, 3, 4, 20):
        d = np.zeros_like(d0)
        op.forward(m, d, checkpoint=ck)
        np.testing.assert_array_equal(d, d0)
        w = np.zeros_like(d0)
        wem.forward(s, rho, w, checkpoint=ck)
        np.testing.assert_array_equal(w, w0)


@pytest.mark.gpu
def test_3d_autograd_is_the_adjoint(gpu_lib):
    import torch
    from wemgpu.autograd import reflectivity_data_3d
    from wemgpu.core import Refl3DOp
    q, par, wav, s, rho = case3d(nz=6, refl=True)
    op = Refl3DOp(q, wav, s)
    rng = np.random.default_rng(6)
    m = torch.from_numpy(rand_c(rng, s.shape)).cuda().requires_grad_(True)
    d = reflectivity_data_3d(m, op, checkpoint=2)
    g = torch.from_numpy(rng.standard_normal(tuple(d.shape)).astype(np.float32)).cuda()
    (d * g).sum().backward()
    want = np.zeros(s.shape, np.complex64)
    op.adjoint(want, g.cpu().numpy())
    # torch's gradient of a real loss w.r.t. a complex leaf is the conjugate
    # Wirtinger form: 2 dL/d(conj m) = conj(J)^T g, the adjoint image here
    np.testing.assert_allclose(m.grad.cpu().numpy(), want, rtol=1e-6, atol=1e-12)
