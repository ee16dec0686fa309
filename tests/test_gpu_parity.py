"""GPU parity: the CUDA library through its C ABI against the CPU oracle.

Tolerance (rel. L2, complex64): 1e-4 against the fp32 restatement of the
reference and against its fp64 twin.  Single steps on random rows are also
held to 1e-5 against the fp64 twin: the fp32 restatement's own error there
reaches 3e-5 (its float phase-shift chain cancels in the evanescent band),
so fp64 is the sharper check.
"""
import numpy as np
import pytest

from cases import pad_edge, rand_c, rel_l2, small_case
from wemgpu.params import WEM_DATA_FREQ, WEM_DATA_TIME, make_params

pytestmark = pytest.mark.gpu

TOL_OP = 1e-4
TOL_STEP = 1e-5


@pytest.mark.parametrize("prop,nref,mode,nx,nz", [("ssf", 1, "ascoded", 52, 24), ("pspi", 3, "ascoded", 52, 24),
                                                  ("ssf", 3, "ascoded", 52, 24), ("pspi", 3, "nearest", 52, 24),
                                                  ("pspi", 4, "ascoded", 52, 24), ("pspi", 4, "nearest", 52, 24),
                                                  # the zero history runs out (nz nref > nxg - nref)
                                                  ("pspi", 4, "ascoded", 60, 40), ("pspi", 3, "ascoded", 20, 30),
                                                  ("ssf", 1, "ascoded", 20, 40)])
def test_refsampler_tables_bit_exact(gpu_lib, oracle, prop, nref, mode, nx, nz):
    """The device RefSampler (the operators' own partition kernels, through
    the row-level handle) equals the oracle's line-faithful restatement of
    RefSampler.cpp:41-84 point for point."""
    from wemgpu.core import RowOps
    p, par, wav, s, rho = small_case(prop=prop, nref=nref, nx=nx, nz=nz)
    p.refs_mode = 1 if mode == "nearest" else 0
    sp = pad_edge(s, p.pad)
    ops = RowOps(p, sp)
    sref_g, idx_g = ops.refsampler()
    sref_o, idx_o = oracle.refsampler(p, sp)
    assert np.array_equal(idx_g, idx_o)
    assert np.array_equal(sref_g, sref_o)


@pytest.mark.parametrize("name,nref", [("c2", 4), ("c2", 3), ("c3", 1)])
def test_refsampler_full_size_models(gpu_lib, oracle, name, nref):
    """The partition of the benchmark configurations' own models (c2: 1024 x
    500, c3: 768 x 300) and a history that runs out; bit-exact."""
    from wemgpu import synthetic as S
    from wemgpu.core import RowOps
    cfg = S.CONFIGS[name]()
    cfg["par"] = dict(cfg["par"], nref=nref, prop="pspi")
    p = S.params_of(cfg)
    sp = np.ascontiguousarray(cfg["slow"])
    sref_g, idx_g = RowOps(p, sp).refsampler()
    sref_o, idx_o = oracle.refsampler(p, sp)
    assert np.array_equal(sref_g, sref_o)
    assert np.array_equal(idx_g, idx_o)


def test_refsampler_rejects_nonpositive_reference(gpu_lib):
    """A reference slowness whose real part is not positive fails the call
    with the reference's message (RefSampler.cpp:35-36), on the operators'
    device path as on the row-level one."""
    from wemgpu._lib import WemError
    from wemgpu.core import BornOp, RowOps
    p, par, wav, s, rho = small_case(prop="pspi", nref=2)
    bad = s.copy()
    bad[5, :] = -1e-7
    with pytest.raises(WemError, match="Ref velocity .* at the layer 5"):
        BornOp(p, wav, bad, rho)
    op = BornOp(p, wav, s, rho)
    with pytest.raises(WemError, match="at the layer 5"):
        op.set_background(bad, rho)
    op.set_background(s, rho)
    with pytest.raises(WemError, match="at the layer 5"):
        RowOps(p, pad_edge(bad, p.pad))


@pytest.mark.parametrize("prop,nref", [("ssf", 1), ("pspi", 1), ("pspi", 3), ("ssf", 2)])
@pytest.mark.parametrize("adj", [0, 1])
def test_onestep(gpu_lib, oracle, prop, nref, adj):
    from wemgpu.core import RowOps
    p, par, wav, s, rho = small_case(prop=prop, nref=nref)
    sp = pad_edge(s, p.pad)
    rng = np.random.default_rng(3)
    x = rand_c(rng, (5, sp.shape[1]))
    ops = RowOps(p, sp)
    for iz in (0, 7, p.nz - 1):
        g = ops.onestep(iz, 9.5, adj, x)
        o32 = oracle.onestep(p, sp, iz, 9.5, adj, x, prec=32)
        o64 = oracle.onestep(p, sp, iz, 9.5, adj, x, prec=64)
        assert rel_l2(g, o32) < TOL_OP, (iz, rel_l2(g, o32))
        assert rel_l2(g, o64) < TOL_STEP, (iz, rel_l2(g, o64))


@pytest.mark.parametrize("up", [0, 1])
@pytest.mark.parametrize("adj", [0, 1])
@pytest.mark.parametrize("inplace", [True, False])
def test_oneway(gpu_lib, oracle, up, adj, inplace):
    from wemgpu.core import RowOps
    p, par, wav, s, rho = small_case(prop="pspi", nref=2)
    sp = pad_edge(s, p.pad)
    rng = np.random.default_rng(4)
    x = rand_c(rng, (3, p.nz, sp.shape[1]))
    ops = RowOps(p, sp)
    if inplace:
        g = x.copy()
        ops.oneway(up, 8.0, adj, g, out=g, add=True)
        o = oracle.oneway(p, sp, up, 8.0, adj, x.copy(), add=True)
    else:
        g = ops.oneway(up, 8.0, adj, x)
        o = oracle.oneway(p, sp, up, 8.0, adj, x, out=np.zeros_like(x))
    assert rel_l2(g, o) < TOL_OP, rel_l2(g, o)


@pytest.mark.parametrize("mode", ["compat", "exact"])
@pytest.mark.parametrize("adj", [0, 1])
@pytest.mark.parametrize("ntaylor", [0, 1, 2])
def test_scatter(gpu_lib, oracle, mode, adj, ntaylor):
    from wemgpu.core import RowOps
    p, par, wav, s, rho = small_case(ntaylor=ntaylor, adjoint_mode=mode)
    sp = pad_edge(s, p.pad)
    rng = np.random.default_rng(5)
    x = rand_c(rng, (4, sp.shape[1]))
    ops = RowOps(p, sp)
    g = ops.scatter(9, 11.0, adj, x)
    o = oracle.scatter(p, sp, 9, 11.0, adj, x, prec=64)
    assert rel_l2(g, o) < TOL_STEP, rel_l2(g, o)


@pytest.mark.parametrize("prop,nref", [("ssf", 1), ("pspi", 3)])
@pytest.mark.parametrize("kind", [WEM_DATA_FREQ, WEM_DATA_TIME])
def test_wem_forward(gpu_lib, oracle, prop, nref, kind):
    from wemgpu.core import WemOp
    p, par, wav, s, rho = small_case(prop=prop, nref=nref)
    op = WemOp(p, wav)
    shape = (p.ns, p.nr, p.nt if kind == WEM_DATA_TIME else p.nt + p.tpad)
    dt = np.float32 if kind == WEM_DATA_TIME else np.complex64
    g = np.zeros(shape, dt)
    op.forward(s, rho, g)
    o32 = oracle.wem_forward(p, wav, s, rho, kind=kind, prec=32)
    o64 = oracle.wem_forward(p, wav, s, rho, kind=kind, prec=64)
    assert np.abs(o64).max() > 0
    assert rel_l2(g, o32) < TOL_OP, rel_l2(g, o32)
    assert rel_l2(g, o64) < TOL_OP, rel_l2(g, o64)
    # add=True accumulates
    g2 = g.copy()
    op.forward(s, rho, g2, add=True)
    assert rel_l2(g2, 2 * g) < 1e-6


@pytest.mark.parametrize("prop,nref,ntaylor", [("ssf", 1, 1), ("pspi", 3, 1), ("ssf", 1, 2)])
def test_born_forward(gpu_lib, oracle, prop, nref, ntaylor):
    from wemgpu.core import BornOp
    p, par, wav, s, rho = small_case(prop=prop, nref=nref, ntaylor=ntaylor)
    rng = np.random.default_rng(6)
    ds = (rand_c(rng, s.shape) * 1e-8).astype(np.complex64)
    dr = (rand_c(rng, s.shape) * 0.1).astype(np.complex64)
    op = BornOp(p, wav, s, rho)
    g = np.zeros((p.ns, p.nr, p.nt + p.tpad), np.complex64)
    op.forward(ds, dr, g)
    o32 = oracle.born_forward(p, wav, s, rho, ds, dr, prec=32)
    o64 = oracle.born_forward(p, wav, s, rho, ds, dr, prec=64)
    assert rel_l2(g, o32) < TOL_OP, rel_l2(g, o32)
    assert rel_l2(g, o64) < TOL_OP, rel_l2(g, o64)


@pytest.mark.parametrize("mode", ["compat", "exact"])
@pytest.mark.parametrize("prop,nref", [("ssf", 1), ("pspi", 3)])
@pytest.mark.parametrize("kind", [WEM_DATA_FREQ, WEM_DATA_TIME])
def test_born_adjoint(gpu_lib, oracle, mode, prop, nref, kind):
    from wemgpu.core import BornOp
    p, par, wav, s, rho = small_case(prop=prop, nref=nref, adjoint_mode=mode)
    rng = np.random.default_rng(7)
    if kind == WEM_DATA_TIME:
        d = (rng.random((p.ns, p.nr, p.nt)) - .5).astype(np.float32)
    else:
        d = rand_c(rng, (p.ns, p.nr, p.nt + p.tpad))
    op = BornOp(p, wav, s, rho)
    g0 = np.zeros(s.shape, np.complex64)
    g1 = np.zeros(s.shape, np.complex64)
    op.adjoint(g0, g1, d)
    o0, o1 = oracle.born_adjoint(p, wav, s, rho, d, kind=kind, prec=32)
    q0, q1 = oracle.born_adjoint(p, wav, s, rho, d, kind=kind, prec=64)
    for g, o, q in ((g0, o0, q0), (g1, o1, q1)):
        assert rel_l2(g, o) < TOL_OP, rel_l2(g, o)
        assert rel_l2(g, q) < TOL_OP, rel_l2(g, q)


def test_born_dot_exact(gpu_lib):
    """Exact adjoint passes the dot test to 1e-5 for complex and time data.

    d = L m' with an independent m' keeps both inner products far from
    cancellation: with white random data the fp32 rounding of the outputs
    alone moves the ratio by up to 1e-4 (the fp64 oracle rounded to float
    shows 2e-6), which would hide the adjoint error being measured."""
    from wemgpu.core import BornOp
    p, par, wav, s, rho = small_case(prop="pspi", nref=3, adjoint_mode="exact")
    rng = np.random.default_rng(8)
    op = BornOp(p, wav, s, rho)
    m0, m1 = rand_c(rng, s.shape), rand_c(rng, s.shape)
    n0, n1 = rand_c(rng, s.shape), rand_c(rng, s.shape)
    for kind in (WEM_DATA_FREQ, WEM_DATA_TIME):
        dt = np.complex64 if kind == WEM_DATA_FREQ else np.float32
        nb = p.nt + p.tpad if kind == WEM_DATA_FREQ else p.nt
        d = np.zeros((p.ns, p.nr, nb), dt)
        op.forward(n0 + 0.5 * m0, n1 + 0.5 * m1, d)
        Lm = np.zeros_like(d)
        op.forward(m0, m1, Lm)
        a0, a1 = np.zeros_like(m0), np.zeros_like(m1)
        op.adjoint(a0, a1, d)
        lhs = np.vdot(d.astype(np.complex128), Lm.astype(np.complex128)).real
        rhs = (np.vdot(a0.astype(np.complex128), m0.astype(np.complex128)).real +
               np.vdot(a1.astype(np.complex128), m1.astype(np.complex128)).real)
        assert abs(lhs - rhs) / abs(lhs) < 1e-5, (kind, lhs, rhs)


def test_ext_wem_equals_wem(gpu_lib):
    """The reference's known-answer test (test_wem_ops.py:268-282): extWEM on
    a frequency-constant model equals WEM bit for bit."""
    from wemgpu.core import ExtWemOp, WemOp
    p, par, wav, s, rho = small_case(prop="pspi", nref=2)
    w = WemOp(p, wav)
    e = ExtWemOp(p, wav)
    nf = e.nfreq()
    d1 = np.zeros((p.ns, p.nr, p.nt + p.tpad), np.complex64)
    d2 = np.zeros_like(d1)
    w.forward(s, rho, d1)
    e.forward(np.repeat(s[None], nf, 0), np.repeat(rho[None], nf, 0), d2)
    assert np.array_equal(d1, d2)


@pytest.mark.parametrize("mode", ["compat", "exact"])
def test_ext_born(gpu_lib, oracle, mode):
    from wemgpu.core import ExtBornOp
    p, par, wav, s, rho = small_case(prop="ssf", nref=1, adjoint_mode=mode, ns=2)
    nf = oracle.count_freqs(p)[0]
    rng = np.random.default_rng(9)
    s3 = (np.repeat(s[None], nf, 0) * (1 + 0.02 * rng.standard_normal((nf, 1, 1)))).astype(np.complex64)
    r3 = np.repeat(rho[None], nf, 0)
    ds = (rand_c(rng, s3.shape) * 1e-8).astype(np.complex64)
    dr = (rand_c(rng, s3.shape) * 0.1).astype(np.complex64)
    op = ExtBornOp(p, wav, s3, r3)
    g = np.zeros((p.ns, p.nr, p.nt + p.tpad), np.complex64)
    op.forward(ds, dr, g)
    o = oracle.extborn_forward(p, wav, s3, r3, ds, dr, prec=32)
    assert rel_l2(g, o) < TOL_OP, rel_l2(g, o)
    d = rand_c(rng, g.shape)
    a0, a1 = np.zeros_like(s3), np.zeros_like(s3)
    op.adjoint(a0, a1, d)
    b0, b1 = oracle.extborn_adjoint(p, wav, s3, r3, d, prec=32)
    assert rel_l2(a0, b0) < TOL_OP, rel_l2(a0, b0)
    assert rel_l2(a1, b1) < TOL_OP, rel_l2(a1, b1)


# ---------------------------------------------------------------- warp path
# Row lengths N = 32 E run on the warp-per-row kernels (automatic choice);
# the same cases also run on the shared-memory kernels (path 1) so both
# families are held to the oracle.
WARP_CASES = {
    "n256": dict(nx=240, pad=4, tap=4, prop="ssf", nref=1),
    "n384": dict(nx=376, pad=0, tap=4, prop="pspi", nref=2),
    "n512": dict(nx=504, pad=4, tap=0, prop="pspi", nref=3),
    "n768": dict(nx=752, pad=4, tap=4, prop="ssf", nref=1),
    "n1024": dict(nx=1016, pad=0, tap=4, prop="pspi", nref=2),
    # tap = 0 (the reference's default): kernels built with every point on the grid
    "n768t0": dict(nx=760, pad=4, tap=0, prop="ssf", nref=1),
    "n384t0": dict(nx=384, pad=0, tap=0, prop="ssf", nref=1),
    "n512t0p": dict(nx=512, pad=0, tap=0, prop="pspi", nref=1),
}


@pytest.fixture
def kernel_path(gpu_lib, request):
    from wemgpu import _lib
    _lib.call("wem_set_kernel_path", request.param)
    yield request.param
    _lib.call("wem_set_kernel_path", 0)


@pytest.fixture
def row_ctas(gpu_lib, request):
    """Rows per CTA of the single-reference warp kernels: 1 grouped rows of a
    frequency, 2 one row per CTA (0 automatic: one-row CTAs when a pass has
    no more rows than SMs, which every small case here has)."""
    from wemgpu import _lib
    _lib.call("wem_set_row_ctas", request.param)
    yield request.param
    _lib.call("wem_set_row_ctas", 0)


ROWS = [pytest.param(1, id="grouped"), pytest.param(2, id="onerow")]


@pytest.mark.parametrize("case", list(WARP_CASES))
@pytest.mark.parametrize("kernel_path,row_ctas", [pytest.param(0, 1, id="warp-grouped"),
                                                  pytest.param(0, 2, id="warp-onerow"),
                                                  pytest.param(1, 0, id="smem")], indirect=True)
def test_paths_wem_and_born(gpu_lib, oracle, case, kernel_path, row_ctas):
    from wemgpu.core import BornOp, WemOp
    kw = WARP_CASES[case]
    for mode in ("compat", "exact"):
        p, par, wav, s, rho = small_case(nz=16, ns=2, adjoint_mode=mode, **kw)
        rng = np.random.default_rng(11)
        if mode == "compat":
            d = np.zeros((p.ns, p.nr, p.nt), np.float32)
            WemOp(p, wav).forward(s, rho, d)
            o = oracle.wem_forward(p, wav, s, rho, kind=WEM_DATA_TIME, prec=64)
            assert rel_l2(d, o) < TOL_OP, ("wem", rel_l2(d, o))
            ds = (rand_c(rng, s.shape) * 1e-8).astype(np.complex64)
            dr = (rand_c(rng, s.shape) * 0.1).astype(np.complex64)
            op = BornOp(p, wav, s, rho)
            g = np.zeros((p.ns, p.nr, p.nt), np.float32)
            op.forward(ds, dr, g)
            o = oracle.born_forward(p, wav, s, rho, ds, dr, kind=WEM_DATA_TIME, prec=64)
            assert rel_l2(g, o) < TOL_OP, ("born fwd", rel_l2(g, o))
        op = BornOp(p, wav, s, rho)
        dd = (rng.random((p.ns, p.nr, p.nt)) - .5).astype(np.float32)
        a0, a1 = np.zeros_like(s), np.zeros_like(s)
        op.adjoint(a0, a1, dd)
        q0, q1 = oracle.born_adjoint(p, wav, s, rho, dd, kind=WEM_DATA_TIME, prec=64)
        assert rel_l2(a0, q0) < TOL_OP, (mode, "adj s", rel_l2(a0, q0))
        assert rel_l2(a1, q1) < TOL_OP, (mode, "adj rho", rel_l2(a1, q1))


@pytest.mark.parametrize("case", ["n768t0", "n256"])
@pytest.mark.parametrize("row_ctas", ROWS, indirect=True)
def test_born_adjoint_many_shots(gpu_lib, oracle, case, row_ctas):
    """More shots than rows per CTA: full and partial groups of one frequency."""
    from wemgpu.core import BornOp
    p, par, wav, s, rho = small_case(nz=12, ns=11, **WARP_CASES[case])
    op = BornOp(p, wav, s, rho)
    d = (np.random.default_rng(13).random((p.ns, p.nr, p.nt)) - .5).astype(np.float32)
    a0, a1 = np.zeros_like(s), np.zeros_like(s)
    op.adjoint(a0, a1, d)
    q0, q1 = oracle.born_adjoint(p, wav, s, rho, d, kind=WEM_DATA_TIME, prec=64)
    assert rel_l2(a0, q0) < TOL_OP, rel_l2(a0, q0)
    assert rel_l2(a1, q1) < TOL_OP, rel_l2(a1, q1)


@pytest.mark.parametrize("case", ["n256", "n768t0"])
def test_shaped_tail(gpu_lib, oracle, case):
    """17 shots x 66 frequencies: 198 groups of up to 8 shots, more than one
    wave of CTAs, so the launch takes the shaped tail (the last frequencies in
    groups of 1-2 shots)."""
    from wemgpu.core import BornOp, WemOp
    p, par, wav, s, rho = small_case(nz=6, ns=17, nt=1024, **WARP_CASES[case])
    d = np.zeros((p.ns, p.nr, p.nt), np.float32)
    WemOp(p, wav).forward(s, rho, d)
    o = oracle.wem_forward(p, wav, s, rho, kind=WEM_DATA_TIME, prec=64)
    assert rel_l2(d, o) < TOL_OP, ("wem", rel_l2(d, o))
    op = BornOp(p, wav, s, rho)
    dd = (np.random.default_rng(14).random((p.ns, p.nr, p.nt)) - .5).astype(np.float32)
    a0, a1 = np.zeros_like(s), np.zeros_like(s)
    op.adjoint(a0, a1, dd)
    q0, q1 = oracle.born_adjoint(p, wav, s, rho, dd, kind=WEM_DATA_TIME, prec=64)
    assert rel_l2(a0, q0) < TOL_OP, rel_l2(a0, q0)
    assert rel_l2(a1, q1) < TOL_OP, rel_l2(a1, q1)


@pytest.mark.parametrize("case", ["n256", "n768", "n768t0"])
def test_warp_path_is_deterministic(gpu_lib, case):
    from wemgpu.core import BornOp
    p, par, wav, s, rho = small_case(nz=16, ns=2, **WARP_CASES[case])
    op = BornOp(p, wav, s, rho)
    d = (np.random.default_rng(12).random((p.ns, p.nr, p.nt)) - .5).astype(np.float32)
    outs = []
    for _ in range(2):
        a0, a1 = np.zeros_like(s), np.zeros_like(s)
        op.adjoint(a0, a1, d)
        outs.append((a0, a1))
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


def test_refsampler_history_exhausted(gpu_lib, oracle):
    """nref = 1 with nz > nxg - 2: the reference's zero history runs out and
    the as-coded partition drops points (RefSampler.cpp:63-81); the device
    RefSampler replays that history as the oracle does."""
    from wemgpu.core import WemOp
    p, par, wav, s, rho = small_case(nx=20, nz=24, pad=0, tap=6, ns=1)
    d = np.zeros((p.ns, p.nr, p.nt), np.float32)
    WemOp(p, wav).forward(s, rho, d)
    o = oracle.wem_forward(p, wav, s, rho, kind=WEM_DATA_TIME, prec=64)
    assert rel_l2(d, o) < TOL_OP, rel_l2(d, o)


@pytest.mark.parametrize("case", ["small", "n768t0"])
def test_exact_kz_phase_law(gpu_lib, oracle, case):
    """phase_law exact_kz (extPropagator/src/Phshift.cpp:41-126) through a
    depth step, the modelling and the Born adjoint."""
    from wemgpu.core import BornOp, RowOps, WemOp
    kw = {} if case == "small" else dict(WARP_CASES[case])
    p, par, wav, s, rho = small_case(nz=12, ns=2, phase_law="exact_kz", **kw)
    sp = pad_edge(s, p.pad)
    x = rand_c(np.random.default_rng(15), (3, sp.shape[1]))
    for adj in (0, 1):
        g = RowOps(p, sp).onestep(5, 9.5, adj, x)
        o = oracle.onestep(p, sp, 5, 9.5, adj, x, prec=64)
        assert rel_l2(g, o) < TOL_STEP, rel_l2(g, o)
    d = np.zeros((p.ns, p.nr, p.nt), np.float32)
    WemOp(p, wav).forward(s, rho, d)
    o = oracle.wem_forward(p, wav, s, rho, kind=WEM_DATA_TIME, prec=64)
    assert rel_l2(d, o) < TOL_OP, ("wem", rel_l2(d, o))
    dd = (np.random.default_rng(16).random((p.ns, p.nr, p.nt)) - .5).astype(np.float32)
    a0, a1 = np.zeros_like(s), np.zeros_like(s)
    BornOp(p, wav, s, rho).adjoint(a0, a1, dd)
    q0, q1 = oracle.born_adjoint(p, wav, s, rho, dd, kind=WEM_DATA_TIME, prec=64)
    assert rel_l2(a0, q0) < TOL_OP, rel_l2(a0, q0)
    assert rel_l2(a1, q1) < TOL_OP, rel_l2(a1, q1)


@pytest.mark.parametrize("case", ["small", "n256", "n768t0"])
@pytest.mark.parametrize("mode", ["compat", "exact"])
@pytest.mark.parametrize("row_ctas", ROWS, indirect=True)
def test_bornrefl_borntomo(gpu_lib, oracle, case, mode, row_ctas):
    """BornRefl / BornTomo (ext_born_refl.cpp, ext_born_tomo.cpp) on the Born
    passes against the oracle."""
    from wemgpu.core import BornReflOp, BornTomoOp
    kw = {} if case == "small" else dict(WARP_CASES[case])
    p, par, wav, s, rho = small_case(nz=12, ns=3, adjoint_mode=mode, **kw)
    nf = oracle.count_freqs(p)[0]
    rng = np.random.default_rng(41)
    m = rand_c(rng, (nf, p.nz, p.nx)) * 0.1
    d = (rng.random((p.ns, p.nr, p.nt)) - .5).astype(np.float32)
    op = BornReflOp(p, wav, s)
    g = np.zeros((p.ns, p.nr, p.nt), np.float32)
    op.forward(m, g)
    o = oracle.bornrefl_forward(p, wav, s, m, kind=WEM_DATA_TIME, prec=64)
    assert rel_l2(g, o) < TOL_OP, ("refl fwd", rel_l2(g, o))
    a = np.zeros((nf, p.nz, p.nx), np.complex64)
    op.adjoint(a, d)
    q = oracle.bornrefl_adjoint(p, wav, s, d, kind=WEM_DATA_TIME, prec=64)
    assert rel_l2(a, q) < TOL_OP, ("refl adj", rel_l2(a, q))
    refl = (rand_c(rng, (nf, p.nz, p.nx)) * 0.2).astype(np.complex64)
    dm = (rand_c(rng, (p.nz, p.nx)) * 1e-8).astype(np.complex64)
    op = BornTomoOp(p, wav, s)
    op.set_refl(refl)
    g = np.zeros((p.ns, p.nr, p.nt), np.float32)
    op.forward(dm, g)
    o = oracle.borntomo_forward(p, wav, s, refl, dm, kind=WEM_DATA_TIME, prec=64)
    assert rel_l2(g, o) < TOL_OP, ("tomo fwd", rel_l2(g, o))
    a = np.zeros((p.nz, p.nx), np.complex64)
    op.adjoint(a, d)
    q = oracle.borntomo_adjoint(p, wav, s, refl, d, kind=WEM_DATA_TIME, prec=64)
    assert rel_l2(a, q) < TOL_OP, ("tomo adj", rel_l2(a, q))


@pytest.mark.parametrize("case", ["n768t0", "n512t0p"])
@pytest.mark.parametrize("mode", ["compat", "exact"])
@pytest.mark.parametrize("row_ctas", ROWS, indirect=True)
def test_ext_born_warp_tap0(gpu_lib, oracle, case, mode, row_ctas):
    """Frequency-extended Born on the warp kernels at tap 0: per-frequency
    tables, the spectral reuse of the as-coded adjoint and the extended
    last-row rule (one shot's LinUp^H term)."""
    from wemgpu.core import ExtBornOp
    p, par, wav, s, rho = small_case(nz=10, ns=3, adjoint_mode=mode, **WARP_CASES[case])
    nf = oracle.count_freqs(p)[0]
    rng = np.random.default_rng(19)
    s3 = (np.repeat(s[None], nf, 0) * (1 + 0.02 * rng.standard_normal((nf, 1, 1)))).astype(np.complex64)
    r3 = np.repeat(rho[None], nf, 0)
    ds = (rand_c(rng, s3.shape) * 1e-8).astype(np.complex64)
    dr = (rand_c(rng, s3.shape) * 0.1).astype(np.complex64)
    op = ExtBornOp(p, wav, s3, r3)
    g = np.zeros((p.ns, p.nr, p.nt), np.float32)
    op.forward(ds, dr, g)
    o = oracle.extborn_forward(p, wav, s3, r3, ds, dr, kind=WEM_DATA_TIME, prec=64)
    assert rel_l2(g, o) < TOL_OP, rel_l2(g, o)
    d = (rng.random(g.shape) - .5).astype(np.float32)
    a0, a1 = np.zeros_like(s3), np.zeros_like(s3)
    op.adjoint(a0, a1, d)
    b0, b1 = oracle.extborn_adjoint(p, wav, s3, r3, d, kind=WEM_DATA_TIME, prec=64)
    assert rel_l2(a0, b0) < TOL_OP, rel_l2(a0, b0)
    assert rel_l2(a1, b1) < TOL_OP, rel_l2(a1, b1)


@pytest.mark.parametrize("kw", [dict(prop="pspi", nref=2), dict(ntaylor=0), dict(ntaylor=2)])
def test_bornrefl_borntomo_shared_memory_path(gpu_lib, oracle, kw):
    """BornRefl / BornTomo with several references (PSPI) and with Taylor
    orders the warp kernels do not serve (shared-memory kernels)."""
    from wemgpu.core import BornReflOp, BornTomoOp
    p, par, wav, s, rho = small_case(nz=10, ns=2, **kw)
    nf = oracle.count_freqs(p)[0]
    rng = np.random.default_rng(43)
    m = rand_c(rng, (nf, p.nz, p.nx)) * 0.1
    d = (rng.random((p.ns, p.nr, p.nt)) - .5).astype(np.float32)
    op = BornReflOp(p, wav, s)
    g = np.zeros((p.ns, p.nr, p.nt), np.float32)
    op.forward(m, g)
    assert rel_l2(g, oracle.bornrefl_forward(p, wav, s, m, prec=64)) < TOL_OP
    a = np.zeros((nf, p.nz, p.nx), np.complex64)
    op.adjoint(a, d)
    assert rel_l2(a, oracle.bornrefl_adjoint(p, wav, s, d, prec=64)) < TOL_OP
    refl = (rand_c(rng, (nf, p.nz, p.nx)) * 0.2).astype(np.complex64)
    dm = (rand_c(rng, (p.nz, p.nx)) * 1e-8).astype(np.complex64)
    op = BornTomoOp(p, wav, s)
    op.set_refl(refl)
    g = np.zeros((p.ns, p.nr, p.nt), np.float32)
    op.forward(dm, g)
    assert rel_l2(g, oracle.borntomo_forward(p, wav, s, refl, dm, prec=64)) < TOL_OP
    a = np.zeros((p.nz, p.nx), np.complex64)
    op.adjoint(a, d)
    assert rel_l2(a, oracle.borntomo_adjoint(p, wav, s, refl, d, prec=64)) < TOL_OP


@pytest.mark.parametrize("kw", [dict(), dict(nx=240, pad=4, tap=4), dict(nx=768, pad=0, tap=0)])
@pytest.mark.parametrize("nz,ns", [(2, 1), (3, 1), (5, 9)])
@pytest.mark.parametrize("row_ctas", ROWS, indirect=True)
def test_small_geometries(gpu_lib, oracle, kw, nz, ns, row_ctas):
    """Smallest depth axes (one step), one shot and more shots than rows per
    CTA, on the shared-memory kernels (N = 72) and the warp kernels (256, 768)."""
    from wemgpu.core import BornOp, WemOp
    p, par, wav, s, rho = small_case(nz=nz, ns=ns, **kw)
    d = np.zeros((p.ns, p.nr, p.nt), np.float32)
    WemOp(p, wav).forward(s, rho, d)
    o = oracle.wem_forward(p, wav, s, rho, kind=WEM_DATA_TIME, prec=64)
    assert rel_l2(d, o) < TOL_OP, ("wem", rel_l2(d, o))
    rng = np.random.default_rng(51)
    dd = (rng.random(d.shape) - .5).astype(np.float32)
    a0, a1 = np.zeros_like(s), np.zeros_like(s)
    BornOp(p, wav, s, rho).adjoint(a0, a1, dd)
    q0, q1 = oracle.born_adjoint(p, wav, s, rho, dd, kind=WEM_DATA_TIME, prec=64)
    assert rel_l2(a0, q0) < TOL_OP, ("adj s", rel_l2(a0, q0))
    assert rel_l2(a1, q1) < TOL_OP, ("adj rho", rel_l2(a1, q1))


def test_born_dot_reference_setup(gpu_lib):
    """The set-up of the reference's Born dot test (scripts/unit_tests/
    dot_test_born.py:13-77): 300 x 300 at 10 m, slowness 1/2000 as the script
    sets it, 5 shots 20 m apart, receivers every cell at 1000 m depth, 15
    frequencies from 1 Hz, SSF, N = 300 (shared-memory kernels).  The exact
    adjoint passes to 1e-5; the compat adjoint (the reference's own) is not
    a transpose and is only checked to be finite."""
    from wemgpu.core import BornOp
    n, nt, dt = 300, 1500, 0.002
    par = dict(ns=5, osx=0.0, dsx=20.0, osz=0.0, nr=n, orx=0.0, drx=10.0, orz=1000.0, prop="ssf", nref=1, tap=0,
               fmin=1, fmax=0, nfreq=15, ngs=0, ngr=0, ntaylor=1)
    t = np.arange(nt) * dt
    wav = ((1 - 2 * (np.pi * 5 * t) ** 2) * np.exp(-(np.pi * 5 * t) ** 2)).astype(np.float32)
    s = np.full((n, n), 1 / 2000, np.complex64)
    rho = np.ones((n, n), np.complex64)
    rng = np.random.default_rng(13)
    m0, m1 = rand_c(rng, s.shape), rand_c(rng, s.shape)
    n0, n1 = rand_c(rng, s.shape), rand_c(rng, s.shape)
    for mode in ("exact", "compat"):
        p = make_params(dict(par, adjoint_mode=mode), nx=n, nz=n, dx=10.0, dz=10.0, nt=nt, dt=dt)
        op = BornOp(p, wav, s, rho)
        d = np.zeros((p.ns, p.nr, p.nt), np.float32)
        op.forward(n0 + 0.5 * m0, n1 + 0.5 * m1, d)
        Lm = np.zeros_like(d)
        op.forward(m0, m1, Lm)
        a0, a1 = np.zeros_like(m0), np.zeros_like(m1)
        op.adjoint(a0, a1, d)
        lhs = np.vdot(d.astype(np.float64), Lm.astype(np.float64))
        rhs = (np.vdot(a0.astype(np.complex128), m0.astype(np.complex128)).real +
               np.vdot(a1.astype(np.complex128), m1.astype(np.complex128)).real)
        ratio = abs(lhs - rhs) / abs(lhs)
        if mode == "exact":
            assert ratio < 1e-5, ratio
        else:
            assert np.isfinite(ratio)


# time axes n = nt + tpad: the FFT path (every prime factor <= 7: 1536 =
# 2^9 3 as the benchmark's, 960 with a radix 5, 1176 with radix 7, and a
# time pad) and the restricted DFT (1018 = 2 x 509, 824 = 8 x 103 with a
# time pad, 10010 = 2 5 7 11 13)
@pytest.mark.parametrize("nt,tpad,dt", [(1536, 0, 0.004), (960, 0, 0.005), (1000, 176, 0.004), (1018, 0, 0.004),
                                        (700, 124, 0.005), (10010, 0, 0.0005)])
def test_time_axis_lengths(gpu_lib, oracle, nt, tpad, dt):
    from wemgpu.core import BornOp, FwiOp, WemOp
    p, par, wav, s, rho = small_case(nz=10, nt=nt, dt=dt)
    p.tpad = tpad
    d = np.zeros((p.ns, p.nr, p.nt), np.float32)
    WemOp(p, wav).forward(s, rho, d)
    o32 = oracle.wem_forward(p, wav, s, rho, kind=WEM_DATA_TIME, prec=32)
    o64 = oracle.wem_forward(p, wav, s, rho, kind=WEM_DATA_TIME, prec=64)
    assert rel_l2(d, o32) < TOL_OP and rel_l2(d, o64) < TOL_OP, (rel_l2(d, o32), rel_l2(d, o64))
    rng = np.random.default_rng(8)
    obs = (o32 * (1 + 0.1 * rng.standard_normal(o32.shape))).astype(np.float32)
    g0, g1 = np.zeros_like(s), np.zeros_like(s)
    loss = FwiOp(p, wav).gradient(s, rho, obs, g0, g1)
    res = (d - obs).astype(np.float32)
    assert loss == pytest.approx(0.5 * float(np.sum(res.astype(np.float64) ** 2)), rel=1e-5)
    q0, q1 = oracle.born_adjoint(p, wav, s, rho, res, kind=WEM_DATA_TIME, prec=64)
    assert rel_l2(g0, q0) < TOL_OP and rel_l2(g1, q1) < TOL_OP
    a0, a1 = np.zeros_like(s), np.zeros_like(s)
    BornOp(p, wav, s, rho).adjoint(a0, a1, res)
    assert rel_l2(g0, a0) < 1e-6 and rel_l2(g1, a1) < 1e-6


@pytest.mark.parametrize("case", ["n768t0", "n256", "n384t0"])
@pytest.mark.parametrize("row_ctas", [pytest.param(1, id="grouped")], indirect=True)
def test_fwi_gradient_split_matches_recompute(gpu_lib, oracle, case, row_ctas):
    """fwi_gradient with the source field stored by the modelling pass
    (kw_wem with wem_store_bg, the receiver side's down sweep in
    kw_adj_down, kw_born_adj2's up sweep) equals the gradient whose Born
    adjoint recomputes it, and the oracle's Born adjoint of the same
    residual; tap 0 with the spectral reuse of the scatter and tap 4
    without."""
    from wemgpu import _lib
    from wemgpu.core import FwiOp, WemOp
    p, par, wav, s, rho = small_case(nz=14, ns=4, **WARP_CASES[case])
    d = np.zeros((p.ns, p.nr, p.nt), np.float32)
    WemOp(p, wav).forward(s, rho, d)
    rng = np.random.default_rng(12)
    obs = (d * (1 + 0.1 * rng.standard_normal(d.shape))).astype(np.float32)
    out = {}
    try:
        for mode in (1, 0):
            _lib.call("wem_set_gradient_split", mode)
            g0, g1 = np.zeros_like(s), np.zeros_like(s)
            loss = FwiOp(p, wav).gradient(s, rho, obs, g0, g1)
            out[mode] = (loss, g0, g1)
    finally:
        _lib.call("wem_set_gradient_split", 1)
    l0, b0, b1 = out[0]
    for mode in (1,):
        l1, a0, a1 = out[mode]
        assert l1 == pytest.approx(l0, rel=1e-6)
        assert rel_l2(a0, b0) < 1e-5 and rel_l2(a1, b1) < 1e-5, (mode, rel_l2(a0, b0), rel_l2(a1, b1))
    a0, a1 = out[1][1], out[1][2]
    res = (d - obs).astype(np.float32)
    q0, q1 = oracle.born_adjoint(p, wav, s, rho, res, kind=WEM_DATA_TIME, prec=64)
    assert rel_l2(a0, q0) < TOL_OP and rel_l2(a1, q1) < TOL_OP, (rel_l2(a0, q0), rel_l2(a1, q1))
