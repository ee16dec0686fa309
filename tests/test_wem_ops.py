"""The per-operator classes of the reference (propagator/src/python/wem_ops.py)
on the library, with the set-ups of the reference's own operator tests
(propagator/test/test_wem_ops.py:13-235): a 200 x 100 slowness (1/1000^2,
1/2000^2 below depth 50, imaginary part -1e-8), tap = pad = 100, ten
frequencies from 1 Hz.

CPU: the oracle's own dot tests for the operators added to it here.
GPU: every class against the oracle (rel-L2 <= 1e-4; the transforms run in
fp32 on both sides) and the reference's dot tests (exact adjoints, 1e-4).
"""
import numpy as np
import pytest

from cases import rel_l2
from wemgpu.params import make_params

PAR = dict(ns=10, osx=1000, dsx=10, osz=50, nr=101, orx=0, drx=10, orz=0, eps=0.01, prop="ssf", nref=1, tap=100,
           pad=100, fmin=1, fmax=0, nfreq=10, ngs=3, ngr=3, ntaylor=1)
NX, NZ, D = 200, 100, 10.0


def _slow():
    s = np.full((NZ, NX), 1 / 1000 ** 2 - 1e-8j, np.complex64)
    s[50:, :] = 1 / 2000 ** 2 - 1e-8j
    return s


def _params(**over):
    return make_params(dict(PAR, **over), nx=NX, nz=NZ, dx=D, dz=D, nt=1, dt=1.0)


def _rand(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


def _dot_err(fwd, adj, mshape, dshape, seed=0):
    rng = np.random.default_rng(seed)
    m, d = _rand(rng, mshape), _rand(rng, dshape)
    lhs = np.vdot(fwd(m).astype(np.complex128), d.astype(np.complex128))
    rhs = np.vdot(m.astype(np.complex128), adj(d).astype(np.complex128))
    return abs(lhs - rhs) / max(abs(lhs), abs(rhs))


# ------------------------------------------------------------------ oracle
def test_oracle_row_operators_dot_tests(oracle):
    s = _slow()
    p = _params(adjoint_mode="exact")
    loc = np.random.default_rng(1).integers(0, NX, 50)
    # Phshift (test_wem_ops.py:132-144)
    assert _dot_err(lambda m: oracle.phshift(p, 200, 1.0, 10.0, 5.0, 1 / 1000, 0, m, prec=64),
                    lambda d: oracle.phshift(p, 200, 1.0, 10.0, 5.0, 1 / 1000, 1, d, prec=64), (NX,), (NX,)) < 1e-6
    # SplitStep (test_wem_ops.py:146-158); repeated points make it non-linear, use distinct ones
    uloc = np.unique(loc)
    assert _dot_err(lambda m: oracle.splitstep(p, s, 50, 5.0, 1 / 1000 ** 2, uloc, 0, m, prec=64),
                    lambda d: oracle.splitstep(p, s, 50, 5.0, 1 / 1000 ** 2, uloc, 1, d, prec=64), (NX,), (NX,)) < 1e-6
    # LinDown with the exact adjoint (test_wem_ops.py:219-229)
    bg = np.full((NZ, NX), 1 + 1j, np.complex64)
    assert _dot_err(lambda m: oracle.lindown(p, s, bg, 1.0, 0, m, prec=64),
                    lambda d: oracle.lindown(p, s, bg, 1.0, 1, d, prec=64), (NZ, NX), (NZ, NX)) < 1e-6
    # dReflect (test_wem_ops.py:240-247)
    rho = np.ones((NZ, NX), np.complex64)
    rng = np.random.default_rng(2)
    m0, m1, d = _rand(rng, (NZ, NX)), _rand(rng, (NZ, NX)), _rand(rng, (NZ, NX))
    fd = oracle.dreflect(s, rho, 0, m0=m0, m1=m1)
    a0, a1 = oracle.dreflect(s, rho, 1, data=d)
    lhs = np.vdot(fd.astype(np.complex128), d)
    rhs = np.vdot(m0.astype(np.complex128), a0) + np.vdot(m1.astype(np.complex128), a1)
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs)


# --------------------------------------------------------------------- GPU
def _vectors():
    from wemgpu.vector import Hypercube, SuperVector, Vector
    h2 = Hypercube(ns=[NX, NZ], ds=[D, D])
    slow = Vector(h2, _slow(), storage="dataComplex")
    den = Vector(h2, np.ones((NZ, NX), np.complex64), storage="dataComplex")
    row = Vector(Hypercube(ns=[NX], ds=[D]), np.zeros(NX, np.complex64), storage="dataComplex")
    return slow, den, SuperVector(slow, den), row


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["compat", "exact"])
def test_classes_match_oracle(gpu_lib, oracle, mode):
    from wemgpu import wem_ops as wem
    slow, den, model2d, row = _vectors()
    par = dict(PAR, adjoint_mode=mode)
    p = _params(adjoint_mode=mode)
    s = _slow()
    rng = np.random.default_rng(7)
    r_in, f_in = _rand(rng, (NX,)), _rand(rng, (NZ, NX))
    ref = wem.RefSampler(slow, PAR["nref"])
    sref, _ = oracle.refsampler(p, s)
    assert all(abs(ref.getRefSlow(iz, 0) - sref[iz, 0]) <= 1e-6 * abs(sref[iz, 0]) for iz in range(NZ))

    def run(op, x, out_shape, adj=False):
        from wemgpu.vector import Vector, Hypercube
        xv = Vector(Hypercube(ns=list(x.shape[::-1]), ds=[D] * x.ndim), x.copy(), storage="dataComplex")
        o = Vector(Hypercube(ns=list(out_shape[::-1]), ds=[D] * len(out_shape)), np.zeros(out_shape, np.complex64),
                   storage="dataComplex")
        if adj:
            op.adjoint(False, o, xv)
        else:
            op.forward(False, xv, o)
        return o.getNdArray()

    checks = []
    op = wem.SSF(row, row, slow, 5, 50, par, ref)
    checks.append((run(op, r_in, (NX,)), oracle.onestep(p, s, 50, 5.0, 0, r_in)))
    checks.append((run(op, r_in, (NX,), True), oracle.onestep(p, s, 50, 5.0, 1, r_in)))
    op = wem.Phshift(row, row, row.getHyper(), 10.0, 5, 1 / 1000, 1)
    p1 = make_params({}, nx=NX, nz=2, dx=D, dz=10.0, nt=1, dt=1.0)
    checks.append((run(op, r_in, (NX,)), oracle.phshift(p1, NX, D, 10.0, 5.0, 1 / 1000, 0, r_in)))
    checks.append((run(op, r_in, (NX,), True), oracle.phshift(p1, NX, D, 10.0, 5.0, 1 / 1000, 1, r_in)))
    loc = np.random.default_rng(3).integers(0, NX, 50)
    op = wem.SplitStep(row, row, slow, 5, loc.tolist(), 1 / 1000 ** 2, 50)
    p0 = make_params({}, nx=NX, nz=NZ, dx=D, dz=D, nt=1, dt=1.0)
    checks.append((run(op, r_in, (NX,)), oracle.splitstep(p0, s, 50, 5.0, 1 / 1000 ** 2, loc, 0, r_in)))
    checks.append((run(op, r_in, (NX,), True), oracle.splitstep(p0, s, 50, 5.0, 1 / 1000 ** 2, loc, 1, r_in)))
    op = wem.Scatter(row, row, slow, 1, 1, 50, par)
    checks.append((run(op, r_in, (NX,)), oracle.scatter(p, s, 50, 1.0, 0, r_in)))
    checks.append((run(op, r_in, (NX,), True), oracle.scatter(p, s, 50, 1.0, 1, r_in)))
    for cls, up in ((wem.Down, 0), (wem.Up, 1)):
        op = cls(slow, slow, slow, par, ref, 1)
        checks.append((run(op, f_in, (NZ, NX)), oracle.oneway(p, s, up, 1.0, 0, f_in)))
        checks.append((run(op, f_in, (NZ, NX), True), oracle.oneway(p, s, up, 1.0, 1, f_in)))
    bg = _rand(rng, (NZ, NX))
    bgv = slow.clone()
    bgv.getNdArray()[:] = bg
    op = wem.IC(row, row, bgv, 10)
    checks.append((run(op, r_in, (NX,)), bg[10] * r_in))
    checks.append((run(op, r_in, (NX,), True), np.conj(bg[10]) * r_in))
    op = wem.IC(slow, slow, bgv, 10)
    checks.append((run(op, f_in, (NZ, NX)), bg * f_in))
    bg1 = slow.clone()
    bg1.getNdArray()[:] = 1 + 1j
    down = wem.Down(slow, slow, slow, par, ref, 1)
    op = wem.LinDown(slow, slow, slow, par, bg1, down, 1)
    b1 = np.full((NZ, NX), 1 + 1j, np.complex64)
    checks.append((run(op, f_in, (NZ, NX)), oracle.lindown(p, s, b1, 1.0, 0, f_in)))
    checks.append((run(op, f_in, (NZ, NX), True), oracle.lindown(p, s, b1, 1.0, 1, f_in)))
    rho = np.ones((NZ, NX), np.complex64)
    op = wem.Reflect(slow, slow, model2d)
    checks.append((run(op, f_in, (NZ, NX)), oracle.reflect(s, rho, 0, f_in)))
    checks.append((run(op, f_in, (NZ, NX), True), oracle.reflect(s, rho, 1, f_in)))
    for got, want in checks:
        assert rel_l2(got, want) <= 1e-4
    # dReflect on a superVector model
    from wemgpu.vector import SuperVector
    op = wem.dReflect(model2d, slow, model2d)
    m = SuperVector(slow.clone(), den.clone())
    m.vecs[0].getNdArray()[:] = _rand(rng, (NZ, NX))
    m.vecs[1].getNdArray()[:] = _rand(rng, (NZ, NX))
    d = slow.clone()
    op.forward(False, m, d)
    want = oracle.dreflect(s, rho, 0, m0=m.vecs[0].getNdArray(), m1=m.vecs[1].getNdArray())
    assert rel_l2(d.getNdArray(), want) <= 1e-5
    op.adjoint(False, m, d)
    w0, w1 = oracle.dreflect(s, rho, 1, data=d.getNdArray())
    assert rel_l2(m.vecs[0].getNdArray(), w0) <= 1e-5 and rel_l2(m.vecs[1].getNdArray(), w1) <= 1e-5


@pytest.mark.gpu
def test_reference_dot_tests(gpu_lib):
    """The dot tests of test_wem_ops.py:118-247 on the classes (exact adjoints)."""
    from wemgpu import wem_ops as wem
    slow, den, model2d, row = _vectors()
    par = dict(PAR, adjoint_mode="exact")
    ref = wem.RefSampler(slow, PAR["nref"])
    bg = slow.clone()
    bg.getNdArray()[:] = 1 + 1j
    loc = np.unique(np.random.default_rng(0).integers(0, 200, 50)).tolist()
    rnd = slow.clone().rand(5)
    ops = {
        "SSF": wem.SSF(row, row.clone(), slow, 5, 50, par, ref),
        "Phshift": wem.Phshift(row, row.clone(), row.getHyper(), 10.0, 5, 1 / 1000, 1),
        "SplitStep": wem.SplitStep(row, row.clone(), slow, 5, loc, 1 / 1000 ** 2, 50),
        "Scatter": wem.Scatter(row, row.clone(), slow, PAR["ntaylor"], 1, 50, par),
        "Down": wem.Down(slow.clone(), slow.clone(), slow, par, ref, 1),
        "Up": wem.Up(slow.clone(), slow.clone(), slow, par, ref, 1),
        "IC": wem.IC(row, row.clone(), rnd, 10),
        "IC_2": wem.IC(slow.clone(), slow.clone(), slow, 10),
        "LinDown": wem.LinDown(slow.clone(), slow.clone(), slow, par, bg,
                               wem.Down(slow.clone(), slow.clone(), slow, par, ref, 1), 1),
        "Reflect": wem.Reflect(slow.clone(), slow.clone(), model2d),
        "dReflect": wem.dReflect(model2d.clone(), slow.clone(), model2d),
    }
    # SSF (Selector.cpp:5-10), Down/Up out of place (OneWay.cpp:32-109),
    # Reflect and SplitStep assign their outputs and LinDown clears its first
    # output row, as the reference's do, so only their add = False dot test
    # holds
    assign = {"SSF", "Down", "Up", "Reflect", "SplitStep", "LinDown"}
    bad = {}
    for name, op in ops.items():
        errs = op.dotTest()
        if (errs[0] if name in assign else max(errs)) > 1e-4:
            bad[name] = errs
    assert not bad, bad


@pytest.mark.gpu
def test_phshift_dot_reference_setup(gpu_lib):
    """propagator/test/dotPh.cpp:18-53: Phshift(dz 5) on rows of 500 samples at
    spacing 0.001, 5 Hz, slowness 0.002."""
    from wemgpu import wem_ops as wem
    from wemgpu.vector import Hypercube, Vector
    h = Hypercube(ns=[500], ds=[0.001])
    row = Vector(h, np.zeros(500, np.complex64), storage="dataComplex")
    op = wem.Phshift(row, row.clone(), h, 5.0, 5, 0.002, 0)
    assert max(op.dotTest()) <= 1e-5


def _inject_cases():
    import json
    import os
    f = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "refinject.npz"))
    return json.loads(bytes(f["meta"]).decode())["cases"], {k: f[k] for k in f.files if k != "meta"}


def _cvec(a):
    from wemgpu.vector import Hypercube, Vector
    return Vector(Hypercube(ns=list(reversed(a.shape))), np.ascontiguousarray(a, np.complex64), storage="dataComplex")


@pytest.mark.gpu
def test_injection_matches_reference_run(gpu_lib):
    """wem_ops.Injection against the reference's own Injection
    (Injection.cpp:8-33, 52-75; tests/golden/refinject.npz): forward,
    adjoint (which clears the whole model unless adding) and the add
    forms.  The roundings are the reference's; only the order of the sums
    may differ, so 1e-6."""
    from wemgpu import wem_ops as wem
    cases, F = _inject_cases()
    for c in cases:
        n, nz, nx = c["name"], c["nz"], c["nx"]
        m, d = F[n + "_m"], F[n + "_d"]
        mv, dv = _cvec(m), _cvec(np.zeros((nz, nx), np.complex64))
        op = wem.Injection(mv, dv, F[n + "_iz"].tolist(), F[n + "_ix"].tolist(), ng=c["ng"], tap=c["tap"])
        op.setStep(c["step"])
        op.setShot(c["shot"])
        dv.getNdArray()[:] = 3.0
        op.forward(False, mv, dv)
        assert rel_l2(dv.getNdArray(), F[n + "_fwd"]) < 1e-6, n
        op.forward(True, mv, dv)
        assert rel_l2(dv.getNdArray(), 2 * F[n + "_fwd"]) < 1e-6, n
        ma = _cvec(np.full(m.shape, 5.0 + 1j, np.complex64))
        op.adjoint(False, ma, _cvec(d))
        assert rel_l2(ma.getNdArray(), F[n + "_adj"]) < 1e-6, n
        op.adjoint(True, ma, _cvec(d))
        assert rel_l2(ma.getNdArray(), 2 * F[n + "_adj"]) < 1e-6, n


@pytest.mark.gpu
def test_injection_reference_dot_tests(gpu_lib):
    """The reference's two Injection dot tests (test_wem_ops.py:86-122):
    a trace [100] onto rows [100][200] along a line of 200 points (ng 1,
    tap 1, step 20), and shots x receivers x time [50][100][100] onto rows
    [200][200] (ng 0, step 20, shot 20)."""
    from wemgpu import wem_ops as wem
    x = np.linspace(0, 200 / 2, 200).astype(int).tolist()
    op = wem.Injection(_cvec(np.zeros(100, np.complex64)), _cvec(np.zeros((100, 200), np.complex64)),
                       [0] * 200, x, ng=1, tap=1)
    op.setStep(20)
    assert max(op.dotTest()) <= 1e-5
    x = np.linspace(0, 200 - 1, 100).astype(int).tolist()
    op = wem.Injection(_cvec(np.zeros((50, 100, 100), np.complex64)), _cvec(np.zeros((200, 200), np.complex64)),
                       [0] * 100, x, ng=0, tap=0)
    op.setStep(20)
    op.setShot(20)
    assert max(op.dotTest()) <= 1e-5

