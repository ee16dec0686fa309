"""Model-space interpolation of the FWI preconditioner (scripts/fwi.py:45-68):
LanczosInterpolation2D and Spline2D.

CPU: the numpy oracle against scalar loops written from the reference's
filter code, and its known answers (coarse nodes reproduced, partition of
unity of the cubic family, dot tests).  GPU: the library against the oracle
(rel-L2 <= 1e-5, fp32 sums of a few terms), host and device pointers,
add=1, the spline adjoint's edge copies, and the Python classes' dot tests.
"""
import math

import numpy as np
import pytest

from oracle.interp import Interp2D, lanczos_filter, spline_filter

# (coarse axes, fine axes): ((n1, d1), (n2, d2)); fine grids as scripts/fwi.py
# builds them: same extent, ds = (n - 1) d / (ns - 1)
CASES = {
    "fwi_like": (((17, 47.5), (9, 37.375)), ((77, 10.0), (24, 13.0))),
    "square": (((12, 3.0), (12, 3.0)), ((34, 1.0), (34, 1.0))),
    "unit": (((5, 1.0), (4, 1.0)), ((5, 1.0), (4, 1.0))),
    "bench_grid": (((49, 200.0), (26, 150.0)), ((768, 12.5), (300, 13.0))),
}


def _scalar_lanczos(nd, dd, nm, dm, a):
    f = [[0.0] * nm for _ in range(nd)]
    nf = int(2 * a / dd + 1)
    na = (nf - 1) // 2
    half = na * dd

    def w(x):
        return dm * a * math.sin(math.pi * x / dm) * math.sin(math.pi * x / a) / (math.pi ** 2 * x * x)

    for i in range(nd):
        for j in range(nm):
            x = i * dd - j * dm
            if abs(x) <= half:
                f[i][j] = 1.0 if x == 0 else w(x)
    for i in range(min(na, nd)):
        for j in range(nm):
            x, xx = i * dd - j * dm, i * dd + j * dm
            if abs(xx) < half and x != xx:
                f[i][j] += w(xx)
                f[nd - i - 1][nm - j - 1] += w(xx)
    return np.array(f)


def _scalar_spline(nd, dd, nm, dm, a, b):
    def w(y):
        if y < 1:
            return ((-6 * a - 9 * b + 12) * y ** 3 + (6 * a + 12 * b - 18) * y * y - 2 * b + 6) / 6
        if y < 2:
            return ((-6 * a - b) * y ** 3 + (30 * a + 6 * b) * y * y + (-48 * a - 12 * b) * y + 24 * a + 8 * b) / 6
        return 0.0

    f = [[w(abs(i * dd - j * dm) / dm) for j in range(nm)] for i in range(nd)]
    for i in range(nd):
        for j in range(1, nm - 1):
            v = w(abs(i * dd + j * dm) / dm)
            f[i][j] += v
            f[nd - i - 1][nm - j - 1] += v
    return np.array(f)


@pytest.mark.parametrize("case", ["fwi_like", "square", "unit"])
def test_oracle_filters_follow_the_reference_loops(case):
    (m1, m2), (d1, d2) = CASES[case]
    for (nm, dm), (nd, dd) in ((m1, d1), (m2, d2)):
        for a in (1.0, 3.0):
            got = lanczos_filter(nd, dd, nm, dm, a * dm)
            ref = _scalar_lanczos(nd, dd, nm, dm, a * dm)
            assert np.abs(got - ref).max() <= 1e-5 * max(1.0, np.abs(ref).max())
        for a, b in ((0.5, 0.0), (0.0, 1.0), (1 / 3, 1 / 3), (1.0, 0.0)):
            got = spline_filter(nd, dd, nm, dm, a, b)
            ref = _scalar_spline(nd, dd, nm, dm, a, b)
            assert np.abs(got - ref).max() <= 1e-5


def test_oracle_known_answers():
    (m1, m2), (d1, d2) = CASES["square"]
    rng = np.random.default_rng(3)
    m = (rng.standard_normal((m2[0], m1[0])) + 1j * rng.standard_normal((m2[0], m1[0]))).astype(np.complex64)
    # fine samples on coarse nodes (every 3rd) reproduce the node (sinc zeros)
    L = Interp2D("lanczos", (m1, m2), (d1, d2), (3, 3))
    d = L.forward(m)
    nodes = d[::3, ::3][1:-1, 1:-1]
    assert np.abs(nodes - m[1:-1, 1:-1]).max() <= 1e-5 * np.abs(m).max()
    # the cubic family is a partition of unity away from the edges
    for ab in ((0.5, 0.0), (0.0, 1.0), (1 / 3, 1 / 3)):
        S = Interp2D("spline", (m1, m2), (d1, d2), *ab)
        ones = S.forward(np.ones((m2[0], m1[0]), np.complex64))
        assert np.abs(ones[6:-6, 6:-6] - 1).max() <= 1e-5
    # B-spline (a=0, b=1) at a node: (1, 4, 1)/6 of its neighbours
    S = Interp2D("spline", (m1, m2), (d1, d2), 0.0, 1.0)
    assert abs(S.f1[15, 5] - 4 / 6) < 1e-6 and abs(S.f1[15, 4] - 1 / 6) < 1e-6


@pytest.mark.parametrize("kind", ["lanczos", "spline"])
def test_oracle_dot_test(kind):
    (m1, m2), (d1, d2) = CASES["fwi_like"]
    op = Interp2D(kind, (m1, m2), (d1, d2), (2, 3) if kind == "lanczos" else 0.5, 0.0)
    rng = np.random.default_rng(5)
    m = rng.standard_normal((m2[0], m1[0])) + 1j * rng.standard_normal((m2[0], m1[0]))
    d = rng.standard_normal((d2[0], d1[0])) + 1j * rng.standard_normal((d2[0], d1[0]))
    lhs = np.vdot(op.forward(m), d)
    rhs = np.vdot(m, op.adjoint(d, edges=False))
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.gpu
@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("kind", ["lanczos", "spline"])
def test_interp_matches_oracle(gpu_lib, case, kind):
    import torch

    from wemgpu.core import Interp2DOp
    (m1, m2), (d1, d2) = CASES[case]
    args = ((2, 3),) if kind == "lanczos" else (1 / 3, 1 / 3)
    op = Interp2DOp(kind, (m1, m2), (d1, d2), *args)
    ref = Interp2D(kind, (m1, m2), (d1, d2), *args)
    rng = np.random.default_rng(11)
    m = (rng.standard_normal(op.model_shape) + 1j * rng.standard_normal(op.model_shape)).astype(np.complex64)
    d0 = (rng.standard_normal(op.data_shape) + 1j * rng.standard_normal(op.data_shape)).astype(np.complex64)
    # host arrays, add=0 and add=1
    d = np.zeros(op.data_shape, np.complex64)
    op.forward(m, d)
    assert _rel(d, ref.forward(m)) <= 1e-5
    d_add = d0.copy()
    op.forward(m, d_add, add=True)
    assert _rel(d_add, ref.forward(m, d0, add=True)) <= 1e-5
    mo = np.zeros(op.model_shape, np.complex64)
    op.adjoint(mo, d0)
    assert _rel(mo, ref.adjoint(d0)) <= 1e-5
    m_add = m.copy()
    op.adjoint(m_add, d0, add=True)
    assert _rel(m_add, ref.adjoint(d0, m, add=True)) <= 1e-5
    # device tensors in place give the same numbers
    md, dd = torch.from_numpy(m).cuda(), torch.zeros(op.data_shape, dtype=torch.complex64, device="cuda")
    op.forward(md, dd)
    assert np.array_equal(dd.cpu().numpy(), d)
    mo_d = torch.zeros(op.model_shape, dtype=torch.complex64, device="cuda")
    op.adjoint(mo_d, torch.from_numpy(d0).cuda())
    assert np.array_equal(mo_d.cpu().numpy(), mo)


@pytest.mark.gpu
def test_spline_adjoint_copies_edges(gpu_lib):
    from wemgpu.core import Interp2DOp
    (m1, m2), (d1, d2) = CASES["fwi_like"]
    op = Interp2DOp("spline", (m1, m2), (d1, d2), 0.5, 0.0)
    rng = np.random.default_rng(2)
    d = (rng.standard_normal(op.data_shape) + 1j * rng.standard_normal(op.data_shape)).astype(np.complex64)
    m = np.zeros(op.model_shape, np.complex64)
    op.adjoint(m, d)
    assert np.array_equal(m[:, 0], m[:, 1]) and np.array_equal(m[:, -1], m[:, -2])
    assert np.array_equal(m[0], m[1]) and np.array_equal(m[-1], m[-2])


@pytest.mark.gpu
def test_python_classes_dot_test(gpu_lib):
    from wemgpu import LanczosInterpolation2D, Spline2D
    from wemgpu.vector import Hypercube, getSepVector
    (m1, m2), (d1, d2) = CASES["fwi_like"]
    model = getSepVector(Hypercube(ns=[m1[0], m2[0]], ds=[m1[1], m2[1]]), storage="dataComplex")
    data = getSepVector(Hypercube(ns=[d1[0], d2[0]], ds=[d1[1], d2[1]]), storage="dataComplex")
    op = LanczosInterpolation2D(model, data, a=[2, 3, 3])
    assert max(op.dotTest()) <= 1e-5
    sp = Spline2D(model, data, type="CR-spline")
    assert (sp.a, sp.b) == (0.5, 0.0)
    # the filter uses the a, b arguments (1, 0), as the reference's does
    ref = Interp2D("spline", (m1, m2), (d1, d2), 1.0, 0.0)
    m = model.clone().rand(4)
    d = data.clone().zero()
    sp.forward(False, m, d)
    assert _rel(np.asarray(d.getNdArray()), ref.forward(np.asarray(m.getNdArray()))) <= 1e-5
