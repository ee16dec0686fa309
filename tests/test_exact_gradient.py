"""The exact gradient of the nonlinear modelling (wem_gradient,
fwi_gradient_exact, wemgpu.autograd.WEMGradient) against central finite
differences of the oracle's fp64 modelling (the restatement of
wem_prop.cpp:9-78): per cell on 18 cells (among them the reference
slowness's sample points, where RefSampler.cpp:28-39 makes every depth's
reference depend on the model) and along directions of the whole model; and
the checkpointed gradient against the stored one, bit for bit.

Finite differences are central, per cell with h = 1e-3 of the cell's
value, along the direction with steps of 2.5e-4 of the model, and both
divide by the step actually taken after the model's rounding to complex64;
the GPU gradient is FP32.  Tolerances: per cell |g - fd| <= 2e-3 |fd| +
2e-3 max |fd|; directional derivative 1e-4.
"""
import numpy as np
import pytest

from cases import small_case
from wemgpu.params import WEM_DATA_TIME

pytestmark = pytest.mark.gpu

CASES = {
    # N = 256, tap 0 (the benchmark's kernel shape), SSF
    "ssf_t0": dict(nx=248, pad=4, tap=0, prop="ssf"),
    # N = 256 with an FFT pad, SSF
    "ssf_tap": dict(nx=240, pad=4, tap=4, prop="ssf"),
    # one-reference PSPI (no split step: the phase factor alone), N = 384
    "pspi1": dict(nx=376, pad=4, tap=0, prop="pspi"),
    # the exact-kz phase law
    "kz": dict(nx=248, pad=4, tap=0, prop="ssf", phase_law="exact_kz"),
}


def _problem(case, nz=14, ns=2):
    p, par, wav, s, rho = small_case(nz=nz, ns=ns, nref=1, fmin=6.0, fmax=10.0, **CASES[case])
    nzz, nx = s.shape
    zz, xx = np.meshgrid(np.arange(nzz), np.arange(nx), indexing="ij")
    bump = np.exp(-((zz - nzz / 2) ** 2 / 8.0 + (xx - nx / 2) ** 2 / 300.0))
    s_true = (s * (1 - 0.04 * bump)).astype(np.complex64)
    rho_true = (rho * (1 + 0.05 * bump)).astype(np.complex64)
    return p, wav, s, rho, s_true, rho_true


def _loss64(oracle, p, wav, s, rho, d_obs):
    d = oracle.wem_forward(p, wav, s, rho, kind=WEM_DATA_TIME, prec=64).astype(np.float64)
    return 0.5 * float(np.sum((d - d_obs) ** 2))


def _gpu_grad(p, wav, s, rho, d_obs, checkpoint=0):
    from wemgpu.core import FwiOp
    g0, g1 = np.zeros_like(s), np.zeros_like(s)
    loss = FwiOp(p, wav).gradient(s, rho, d_obs.astype(np.float32), g0, g1, exact=True, checkpoint=checkpoint)
    return loss, g0, g1


@pytest.mark.parametrize("case", list(CASES))
def test_exact_gradient_finite_differences(gpu_lib, oracle, case):
    p, wav, s, rho, s_true, rho_true = _problem(case)
    d_obs = oracle.wem_forward(p, wav, s_true, rho_true, kind=WEM_DATA_TIME, prec=64).astype(np.float64)
    loss, g0, g1 = _gpu_grad(p, wav, s, rho, d_obs)
    assert loss == pytest.approx(_loss64(oracle, p, wav, s, rho, d_obs), rel=1e-4)
    rng = np.random.default_rng(11)
    nz, nx = s.shape
    nxg = nx + 2 * p.pad
    xr = nxg // 2 - p.pad  # the reference slowness's sample column
    cells = [(int(z), xr) for z in rng.integers(1, nz - 1, 4)]
    cells += [(int(z), int(x)) for z, x in zip(rng.integers(0, nz, 12), rng.integers(0, nx, 12))]
    cells += [(0, 0), (nz - 1, nx - 1)]
    fd, gv, labels = [], [], []
    for z, x in cells:
        for which, g, part in (("s", g0, "re"), ("s", g0, "im"), ("rho", g1, "re")):
            base = s if which == "s" else rho
            h = 1e-3 * abs(base[z, x])
            step = h if part == "re" else 1j * h
            lp, lm = [], []
            for sign, out in ((1, lp), (-1, lm)):
                m = base.astype(np.complex128).copy()
                m[z, x] += sign * step
                m = m.astype(np.complex64)
                args = (m, rho) if which == "s" else (s, m)
                out.append(_loss64(oracle, p, wav, *args, d_obs))
            # the perturbation actually applied, after rounding to complex64
            mp = np.complex64(base.astype(np.complex128)[z, x] + step)
            mm = np.complex64(base.astype(np.complex128)[z, x] - step)
            dv = (mp - mm).real if part == "re" else (mp - mm).imag
            fd.append((lp[0] - lm[0]) / float(dv))
            gv.append(g[z, x].real if part == "re" else g[z, x].imag)
            labels.append((z, x, which, part))
    fd, gv = np.array(fd), np.array(gv)
    scale = np.abs(fd).max()
    bad = np.abs(gv - fd) > 2e-3 * np.abs(fd) + 2e-3 * scale
    assert not bad.any(), [(labels[i], gv[i], fd[i]) for i in np.flatnonzero(bad)]


@pytest.mark.parametrize("case", ["ssf_t0", "ssf_tap", "pspi1"])
def test_exact_gradient_directional(gpu_lib, oracle, case):
    """<g, dm> against the central difference of the loss along two
    directions of the whole model (slowness and density): the gradient
    itself (smoothed), where every cell adds with one sign, to 1e-4; and a
    random smooth direction, whose inner product is a sum of both signs, to
    1e-4 of the sum of its terms' magnitudes."""
    from scipy.ndimage import gaussian_filter
    p, wav, s, rho, s_true, rho_true = _problem(case)
    d_obs = oracle.wem_forward(p, wav, s_true, rho_true, kind=WEM_DATA_TIME, prec=64).astype(np.float64)
    _, g0, g1 = _gpu_grad(p, wav, s, rho, d_obs)
    rng = np.random.default_rng(4)
    sm = lambda: gaussian_filter(rng.standard_normal(s.shape), 2)
    smooth = lambda a: gaussian_filter(a.real, 1) + 1j * gaussian_filter(a.imag, 1)
    dirs = [(smooth(g0) * np.abs(s).max() / np.abs(g0).max(), smooth(g1) * np.abs(rho).max() / np.abs(g1).max(), False),
            (s.real * (sm() + 0.3j * sm()), rho.real * sm(), True)]
    t = 2.5e-4
    for dm0, dm1, mixed in dirs:
        dm0, dm1 = dm0.astype(np.complex128), dm1.astype(np.complex128)
        sp, sm_ = (s + t * dm0).astype(np.complex64), (s - t * dm0).astype(np.complex64)
        rp, rm = (rho + t * dm1).astype(np.complex64), (rho - t * dm1).astype(np.complex64)
        fd = (_loss64(oracle, p, wav, sp, rp, d_obs) - _loss64(oracle, p, wav, sm_, rm, d_obs)) / (2 * t)
        # the step actually taken, after the models' rounding to complex64
        e0 = (sp.astype(np.complex128) - sm_) / (2 * t)
        e1 = (rp.astype(np.complex128) - rm) / (2 * t)
        terms = np.concatenate([(g0.real * e0.real + g0.imag * e0.imag).ravel(),
                                (g1.real * e1.real + g1.imag * e1.imag).ravel()])
        ip = float(np.sum(terms))
        scale = float(np.sum(np.abs(terms))) if mixed else abs(fd)
        assert abs(ip - fd) <= 1e-4 * scale, (mixed, ip, fd, scale)


@pytest.mark.parametrize("case", ["ssf_t0", "ssf_tap"])
def test_exact_gradient_checkpointing_is_bit_exact(gpu_lib, oracle, case):
    p, wav, s, rho, s_true, rho_true = _problem(case, nz=17)
    d_obs = oracle.wem_forward(p, wav, s_true, rho_true, kind=WEM_DATA_TIME, prec=32).astype(np.float64)
    l0, a0, a1 = _gpu_grad(p, wav, s, rho, d_obs)
    for ck in (2, 4, 16):
        lk, b0, b1 = _gpu_grad(p, wav, s, rho, d_obs, checkpoint=ck)
        assert lk == l0
        assert np.array_equal(a0, b0) and np.array_equal(a1, b1), ck


def test_wem_gradient_and_autograd(gpu_lib, oracle):
    """wem_gradient of the residual is fwi_gradient_exact's gradient, and
    torch autograd through WEMGradient returns it for the L2 loss."""
    import torch
    from wemgpu.autograd import modelled_data
    from wemgpu.core import WemOp
    p, wav, s, rho, s_true, rho_true = _problem("ssf_t0")
    d_obs = oracle.wem_forward(p, wav, s_true, rho_true, kind=WEM_DATA_TIME, prec=32)
    loss, g0, g1 = _gpu_grad(p, wav, s, rho, d_obs)
    wem = WemOp(p, wav)
    d = np.zeros_like(d_obs)
    wem.forward(s, rho, d)
    h0, h1 = np.zeros_like(s), np.zeros_like(s)
    wem.gradient(s, rho, (d - d_obs).astype(np.float32), h0, h1)
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    assert rel(h0, g0) < 1e-6 and rel(h1, g1) < 1e-6
    dev = torch.device("cuda")
    ts = torch.from_numpy(s).to(dev).requires_grad_(True)
    tr = torch.from_numpy(rho).to(dev).requires_grad_(True)
    obs = torch.from_numpy(d_obs).to(dev)
    out = modelled_data(ts, tr, wem, exact=True, checkpoint=4)
    L = 0.5 * ((out - obs) ** 2).sum()
    L.backward()
    assert rel(ts.grad.cpu().numpy(), g0) < 1e-5 and rel(tr.grad.cpu().numpy(), g1) < 1e-5


def test_exact_gradient_rejects_what_it_does_not_cover(gpu_lib):
    """Several references, and rows whose length the warp kernels do not
    take, are refused with WEM_ENOTIMPL (5) before any work."""
    from wemgpu._lib import WemError
    p, wav, s, rho, _, _ = _problem("ssf_t0")
    p.nref, p.prop = 2, 1
    d = np.zeros((p.ns, p.nr, p.nt), np.float32)
    with pytest.raises(WemError) as e:
        _gpu_grad(p, wav, s, rho, d)
    assert e.value.code == 5 and "nref = 1" in str(e.value)
    q, _, wq, sq, rq = small_case(nx=50, nz=10, nref=1)  # N = 50 + 2 (4 + 6) = 70
    with pytest.raises(WemError) as e:
        _gpu_grad(q, wq, sq, rq, np.zeros((q.ns, q.nr, q.nt), np.float32))
    assert e.value.code == 5 and "warp kernels" in str(e.value)
