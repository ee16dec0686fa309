"""CPU checks of the oracle (the restatement the GPU is held to).

The oracle is pinned to the reference run by tests/test_ref_pin.py (golden
outputs of the reference's own sources); these checks add the reference's
structural known-answer test, exact dot tests, numpy.fft, its fp64 twin and
the documented quirks of the reference code it reproduces.
"""
import numpy as np
import pytest

from cases import pad_edge, rand_c, rel_l2, small_case
from wemgpu.params import WEM_DATA_FREQ, WEM_DATA_TIME, make_params


@pytest.mark.parametrize("n", [1, 2, 3, 5, 6, 7, 12, 17, 60, 72, 97, 256, 384, 600, 768, 876, 1024])
def test_fft_matches_numpy(oracle, n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    ref = np.fft.fft(x)
    assert np.abs(oracle.fft(x, -1) - ref).max() <= 1e-12 * max(1, np.abs(ref).max())
    assert np.abs(oracle.fft(x, +1) - np.fft.ifft(x) * n).max() <= 1e-12 * max(1, np.abs(ref).max())


def test_frequency_axis(oracle):
    # PropParam.h:58-78 with the reference test's parameters (test_wem_ops.py:23-48)
    p = make_params(dict(ns=1, nr=1, drx=10, fmin=1, fmax=0, nfreq=10), nx=200, nz=100, dx=10, dz=10,
                    nt=1001, dt=0.004)
    n, bins, freqs = oracle.count_freqs(p)
    assert n == 10 and list(bins) == list(range(1, 11))
    assert np.allclose(freqs, 1 + np.arange(10) / 4.0)
    # fmax given: bins floor(fmin tmax) .. floor(fmax tmax + .5)
    p = make_params(dict(ns=1, nr=1, drx=10, fmin=2, fmax=20), nx=8, nz=4, dx=10, dz=10, nt=876, dt=0.004)
    n, bins, freqs = oracle.count_freqs(p)
    assert n == 64 and bins[0] == 7 and bins[-1] == 70


def test_devices_round_like_reference(oracle):
    p = make_params(dict(ns=3, osx=1000, dsx=10, osz=50, nr=101, orx=0, drx=10, orz=0), nx=200, nz=100,
                    dx=10, dz=10, nt=10, dt=0.004)
    sx, sz, rx, rz = oracle.devices(p)
    assert list(sx) == [100, 101, 102] and list(sz) == [5, 5, 5]
    assert list(rx) == list(range(101)) and (rz == 0).all()


def test_ext_wem_equals_wem(oracle):
    """The reference's only known-answer test (test_wem_ops.py:268-282) on its
    own setup: two-layer model 200x100, SSF, tap=pad=100, 10 shots."""
    nx, nz = 200, 100
    s = np.full((nz, nx), 1 / 1000 ** 2 - 1e-8j, np.complex64)
    s[50:, :] = 1 / 2000 ** 2 - 1e-8j
    rho = np.ones_like(s)
    par = dict(ns=10, osx=1000, dsx=10, osz=50, nr=101, orx=0, drx=10, orz=0, eps=0.01, prop="ssf", nref=1,
               tap=100, pad=100, fmin=1, fmax=0, nfreq=10, ngs=3, ngr=3, ntaylor=1)
    nt, dt = 1001, 0.004
    p = make_params(par, nx=nx, nz=nz, dx=10, dz=10, nt=nt, dt=dt)
    p.nbin = nt // 2  # the test's data axis of nt//2 bins
    t = np.linspace(0, (nt - 1) * dt, nt) - .5
    wav = ((1 - 2 * (np.pi * 5 * t) ** 2) * np.exp(-((np.pi * 5 * t) ** 2))).astype(np.float32)
    d1 = oracle.wem_forward(p, wav, s, rho, kind=WEM_DATA_FREQ)
    d2 = oracle.extwem_forward(p, wav, np.repeat(s[None], 10, 0), np.repeat(rho[None], 10, 0),
                               kind=WEM_DATA_FREQ)
    assert np.abs(d1).max() > 0
    assert (d1 == d2).all()


def _dot(a, b):
    return np.vdot(np.asarray(b, np.complex128), np.asarray(a, np.complex128)).real


@pytest.mark.parametrize("prop,nref", [("ssf", 1), ("pspi", 3)])
def test_row_operator_dot_tests(oracle, prop, nref):
    p, par, wav, s, rho = small_case(prop=prop, nref=nref, adjoint_mode="exact")
    sp = pad_edge(s, p.pad)
    rng = np.random.default_rng(1)
    m, d = rand_c(rng, sp.shape[1]), rand_c(rng, sp.shape[1])
    for fn, iz in ((oracle.onestep, 9), (oracle.scatter, 9)):
        Am = fn(p, sp, iz, 9.0, 0, m, prec=64)
        Ad = fn(p, sp, iz, 9.0, 1, d, prec=64)
        assert abs(_dot(Am, d) / _dot(m, Ad) - 1) < 1e-5
    M, D = rand_c(rng, sp.shape), rand_c(rng, sp.shape)
    for up in (0, 1):
        AM = oracle.oneway(p, sp, up, 9.0, 0, M, out=np.zeros_like(M), prec=64)
        AD = oracle.oneway(p, sp, up, 9.0, 1, D, out=np.zeros_like(D), prec=64)
        assert abs(_dot(AM, D) / _dot(M, AD) - 1) < 1e-5


def test_scatter_compat_adjoint_is_not_the_transpose(oracle):
    # Scatter.cpp:52-66 filters before scaling: on a laterally varying
    # model the as-coded adjoint differs from the transpose
    p, par, wav, s, rho = small_case(adjoint_mode="compat")
    sp = pad_edge(s, p.pad)
    rng = np.random.default_rng(2)
    d = rand_c(rng, sp.shape[1])
    a_compat = oracle.scatter(p, sp, 12, 9.0, 1, d, prec=64)
    p.adjoint_mode = 1
    a_exact = oracle.scatter(p, sp, 12, 9.0, 1, d, prec=64)
    assert rel_l2(a_compat, a_exact) > 1e-3


@pytest.mark.parametrize("kind", [WEM_DATA_FREQ, WEM_DATA_TIME])
def test_born_dot_exact(oracle, kind):
    p, par, wav, s, rho = small_case(prop="pspi", nref=3, adjoint_mode="exact")
    rng = np.random.default_rng(3)
    m0, m1 = rand_c(rng, s.shape), rand_c(rng, s.shape)
    d = oracle.born_forward(p, wav, s, rho, rand_c(rng, s.shape), rand_c(rng, s.shape), kind=kind, prec=64)
    Lm = oracle.born_forward(p, wav, s, rho, m0, m1, kind=kind, prec=64)
    a0, a1 = oracle.born_adjoint(p, wav, s, rho, d, kind=kind, prec=64)
    lhs, rhs = _dot(Lm, d), _dot(m0, a0) + _dot(m1, a1)
    assert abs(lhs - rhs) / abs(lhs) < 1e-5


def test_compat_last_row_depends_on_frequency_partition(oracle):
    # LinDown::adjoint clears the last depth row (LinOneWay.cpp:64-65): with
    # the frequencies of a shot split over two tasks that row keeps two
    # frequencies' LinUp terms instead of one; every other row is unchanged.
    p, par, wav, s, rho = small_case(adjoint_mode="compat", ns=2)
    rng = np.random.default_rng(4)
    d = rand_c(rng, (p.ns, p.nr, p.nt))
    a1, _ = oracle.born_adjoint(p, wav, s, rho, d, prec=64, fchunks=1)
    a2, _ = oracle.born_adjoint(p, wav, s, rho, d, prec=64, fchunks=2)
    assert rel_l2(a2[:-1], a1[:-1]) < 1e-6
    assert rel_l2(a2[-1], a1[-1]) > 1e-3


def test_fp32_restatement_tracks_fp64(oracle):
    p, par, wav, s, rho = small_case(prop="pspi", nref=3)
    d32 = oracle.wem_forward(p, wav, s, rho, kind=WEM_DATA_TIME, prec=32)
    d64 = oracle.wem_forward(p, wav, s, rho, kind=WEM_DATA_TIME, prec=64)
    assert rel_l2(d32, d64) < 1e-4


def test_refsampler_quirks(oracle):
    """RefSampler.cpp:41-84 as coded: while the zero-initialised history
    buffer still has zeros, every point goes to the largest-slowness
    reference; nref == 1 keeps all points."""
    p, par, wav, s, rho = small_case(prop="pspi", nref=4, nx=60, nz=24)
    sp = pad_edge(s, p.pad)
    sref, idx = oracle.refsampler(p, sp)
    nxg = sp.shape[1]
    for iz in range(nxg // p.nref - 2):
        big = int(np.argmax(sref[iz].real))
        assert (idx[iz] == big).all()
    p1, *_ = small_case(prop="ssf", nref=1)
    s1 = pad_edge(s, p1.pad)
    _, idx1 = oracle.refsampler(p1, s1)
    assert (idx1 == 0).all()
    p.refs_mode = 1  # nearest
    sref, idx = oracle.refsampler(p, sp)
    for iz in (0, 10, 20):
        dist = np.abs(sp[iz].real[:, None] - sref[iz].real[None, :])
        assert (np.take_along_axis(dist, idx[iz][:, None], 1)[:, 0] <= dist.min(1) + 0).all()


@pytest.mark.parametrize("adj", [0, 1])
def test_exact_kz_phase_law(oracle, adj):
    """phase_law exact_kz restates extPropagator/src/Phshift.cpp:59,81: on a
    constant model the split step is 1 and one depth step is the plane-wave
    factor exp(-i dz conj(sqrt(w^2 s - k^2 + 1e-5 i))) on the k grid of
    Phshift_cmplx.cpp:13,21-24 (adjoint: its conjugate)."""
    nx, nz, dx, dz, f = 64, 6, 10.0, 10.0, 11.0
    s = np.full((nz, nx), 1 / 2000.0 ** 2 + 2e-10j, np.complex64)
    par = dict(ns=1, osx=0.0, dsx=0.0, nr=1, orx=0.0, drx=dx, prop="ssf", nref=1, phase_law="exact_kz")
    p = make_params(par, nx=nx, nz=nz, dx=dx, dz=dz, nt=64, dt=0.004)
    x = rand_c(np.random.default_rng(5), (2, nx))
    got = oracle.onestep(p, s, 2, f, adj, x, prec=64)
    k = np.zeros(nx)
    dk = 2 * np.pi / (dx * (nx - 1))
    k[:nx // 2] = np.arange(nx // 2) * dk
    k[nx - np.arange(1, nx // 2)] = -k[1:nx // 2]
    w = 2 * np.pi * f
    kz = np.conj(np.sqrt(w * w * s[2, 0].astype(np.complex128) - k * k + 1e-5j))
    fac = np.exp(-1j * dz * kz)
    if adj:
        fac = np.conj(fac)
    want = np.fft.ifft(np.fft.fft(x.astype(np.complex128), axis=-1) * fac, axis=-1)
    assert rel_l2(got, want) < 1e-6  # complex64 output of an fp64 computation
    p.phase_law = 0
    ispc = oracle.onestep(p, s, 2, f, adj, x, prec=64)
    assert rel_l2(ispc, want) > 1e-3  # the two laws differ (eps damping)


@pytest.mark.parametrize("mode", ["compat", "exact"])
def test_bornrefl_dot(oracle, mode):
    """BornRefl (ext_born_refl.cpp:8-105): Up and Up^H are exact transposes,
    so forward and adjoint pass the dot test in either adjoint mode."""
    p, par, wav, s, rho = small_case(nz=12, ns=2, adjoint_mode=mode)
    nf = oracle.count_freqs(p)[0]
    rng = np.random.default_rng(31)
    m = rand_c(rng, (nf, p.nz, p.nx))
    d = (rng.random((p.ns, p.nr, p.nt)) - .5).astype(np.float32)
    Fm = oracle.bornrefl_forward(p, wav, s, m, kind=WEM_DATA_TIME, prec=64)
    Fd = oracle.bornrefl_adjoint(p, wav, s, d, kind=WEM_DATA_TIME, prec=64)
    lhs = float(np.sum(Fm.astype(np.float64) * d))
    rhs = float(np.sum((np.conj(Fd.astype(np.complex128)) * m).real))
    assert abs(lhs / rhs - 1) < 1e-5, (lhs, rhs)


def test_borntomo_dot_exact(oracle):
    """BornTomo (ext_born_tomo.cpp:9-119) with the exact scatter adjoint is
    the transpose of its forward."""
    p, par, wav, s, rho = small_case(nz=12, ns=2, adjoint_mode="exact")
    nf = oracle.count_freqs(p)[0]
    rng = np.random.default_rng(32)
    refl = (rand_c(rng, (nf, p.nz, p.nx)) * 0.2).astype(np.complex64)
    dm = (rand_c(rng, (p.nz, p.nx)) * 1e-8).astype(np.complex64)
    d = (rng.random((p.ns, p.nr, p.nt)) - .5).astype(np.float32)
    Fm = oracle.borntomo_forward(p, wav, s, refl, dm, kind=WEM_DATA_TIME, prec=64)
    Fd = oracle.borntomo_adjoint(p, wav, s, refl, d, kind=WEM_DATA_TIME, prec=64)
    lhs = float(np.sum(Fm.astype(np.float64) * d))
    rhs = float(np.sum((np.conj(Fd.astype(np.complex128)) * dm).real))
    assert abs(lhs / rhs - 1) < 1e-5, (lhs, rhs)
