"""FWIGradient / FwiObjective (wemgpu.autograd): the reference's FWI
objective of scripts/fwi.py:70-113 through torch autograd on the CUDA
library."""
import numpy as np
import pytest

from cases import rel_l2, small_case
from test_gpu_parity import WARP_CASES

pytestmark = pytest.mark.gpu


def _setup(mode, case="n768t0"):
    import torch
    p, par, wav, s, rho = small_case(nz=12, ns=3, adjoint_mode=mode, **WARP_CASES[case])
    nz, nx = s.shape
    zz, xx = np.meshgrid(np.arange(nz), np.arange(nx), indexing="ij")
    bump = np.exp(-((zz - nz / 2) ** 2 / 8.0 + (xx - nx / 2) ** 2 / 400.0))
    s_true = (s * (1 - 0.05 * bump)).astype(np.complex64)
    from wemgpu.core import WemOp
    d_obs = np.zeros((p.ns, p.nr, p.nt), np.float32)
    WemOp(p, wav).forward(s_true, rho, d_obs)
    return p, wav, s, rho, d_obs, torch


@pytest.mark.parametrize("mode", ["compat", "exact"])
def test_objective_is_born_adjoint_of_residual(gpu_lib, mode):
    from wemgpu.autograd import FwiObjective
    from wemgpu.core import BornOp, WemOp
    p, wav, s, rho, d_obs, torch = _setup(mode)
    obj = FwiObjective(p, wav, d_obs)
    loss, g0, g1 = obj(s, rho)  # numpy in, numpy out
    d = np.zeros_like(d_obs)
    WemOp(p, wav).forward(s, rho, d)
    res = d - d_obs
    assert abs(loss - 0.5 * float(np.sum(res.astype(np.float64) ** 2))) < 1e-4 * loss
    a0, a1 = np.zeros_like(s), np.zeros_like(s)
    BornOp(p, wav, s, rho).adjoint(a0, a1, res)
    assert rel_l2(g0, a0) < 1e-6 and rel_l2(g1, a1) < 1e-6
    # device tensors in, device tensors out, same numbers
    dev = torch.device("cuda")
    l2, t0, t1 = obj(torch.from_numpy(s).to(dev), torch.from_numpy(rho).to(dev))
    assert l2 == pytest.approx(loss, rel=1e-6)
    assert rel_l2(t0.cpu().numpy(), g0) < 1e-6 and rel_l2(t1.cpu().numpy(), g1) < 1e-6


@pytest.mark.parametrize("case", ["n768t0", "n256"])
def test_fwi_gradient_matches_plain_launches(gpu_lib, case):
    """fwi_gradient with all rows in one launch per pass (grouped, shaped
    tail) against the same call forced onto one row per launch."""
    from wemgpu import _lib
    from wemgpu.core import FwiOp
    p, wav, s, rho, d_obs, torch = _setup("compat", case)
    op = FwiOp(p, wav)
    a0, a1 = np.zeros_like(s), np.zeros_like(s)
    la = op.gradient(s, rho, d_obs, a0, a1)
    _lib.call("wem_set_plain", 1)
    try:
        b0, b1 = np.zeros_like(s), np.zeros_like(s)
        lb = op.gradient(s, rho, d_obs, b0, b1)
    finally:
        _lib.call("wem_set_plain", 0)
    assert la == pytest.approx(lb, rel=1e-5)
    assert rel_l2(a0, b0) < 1e-5 and rel_l2(a1, b1) < 1e-5


def test_backward_is_the_transpose_of_born(gpu_lib):
    """Exact adjoint mode: for any data gradient r the leaves receive B^H r
    with Re<B^H r, dm> = <B dm, r> (torch's convention for complex leaves),
    to 1e-5.  r = B m' for an independent m' keeps both inner products far
    from cancellation (white random data alone moves the ratio by up to
    1e-4 through the float rounding of the outputs, test_born_dot_exact)."""
    from wemgpu.autograd import modelled_data
    from wemgpu.core import BornOp, WemOp
    p, wav, s, rho, d_obs, torch = _setup("exact")
    dev = torch.device("cuda")
    wem, born = WemOp(p, wav), BornOp(p, wav, s, rho)
    a = torch.from_numpy(s).to(dev).requires_grad_(True)
    b = torch.from_numpy(rho).to(dev).requires_grad_(True)
    d = modelled_data(a, b, wem, born)
    rng = np.random.default_rng(21)

    def rc(shape):
        return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)

    ds, dr = rc(s.shape), rc(s.shape)
    n0, n1 = rc(s.shape), rc(s.shape)
    born.set_background(s, rho)
    rd = np.zeros_like(d_obs)
    born.forward(n0 + 0.5 * ds, n1 + 0.5 * dr, rd)
    r = torch.from_numpy(rd).to(dev)
    d.backward(r)
    bd = np.zeros_like(d_obs)
    born.forward(ds, dr, bd)
    lhs = float(np.sum(bd.astype(np.float64) * rd.astype(np.float64)))
    rhs = float(np.sum((np.conj(a.grad.cpu().numpy().astype(np.complex128)) * ds).real)
                + np.sum((np.conj(b.grad.cpu().numpy().astype(np.complex128)) * dr).real))
    assert abs(lhs / rhs - 1) < 1e-5, (lhs, rhs)


def test_objective_pspi_shared_memory_path(gpu_lib):
    """fwi_gradient off the warp kernels (N = 72, PSPI with two references)
    equals the Born adjoint of its residual."""
    import torch
    from cases import small_case
    from wemgpu.core import BornOp, FwiOp, WemOp
    p, par, wav, s, rho = small_case(nz=12, ns=2, prop="pspi", nref=2)
    d_obs = np.zeros((p.ns, p.nr, p.nt), np.float32)
    WemOp(p, wav).forward((s * 1.02).astype(np.complex64), rho, d_obs)
    g0, g1 = np.zeros_like(s), np.zeros_like(s)
    loss = FwiOp(p, wav).gradient(s, rho, d_obs, g0, g1)
    d = np.zeros_like(d_obs)
    WemOp(p, wav).forward(s, rho, d)
    res = d - d_obs
    assert loss == pytest.approx(0.5 * float(np.sum(res.astype(np.float64) ** 2)), rel=1e-4)
    a0, a1 = np.zeros_like(s), np.zeros_like(s)
    BornOp(p, wav, s, rho).adjoint(a0, a1, res)
    assert rel_l2(g0, a0) < 1e-6 and rel_l2(g1, a1) < 1e-6
