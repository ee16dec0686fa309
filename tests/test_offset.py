"""Subsurface-offset extended reflectivity Born with per-shot apertures.

No reference implementation exists; the operator is pinned at its
reductions (the reference's own operators restated by the oracle):
* one lag on full apertures is BornRefl (propagator/src/ext_born_refl.cpp:
  8-105) with the same reflectivity at every frequency, the adjoint summed
  over frequencies (IC, ic.cpp:5-29);
* a shot on an aperture is that shot's BornRefl on the cropped model, the
  sub-problem WEM.from_subspace builds (propagator/src/python/WEM.py:24-30);
* forward and adjoint are transposes (dot test).
The GPU path is held to the oracle on uneven apertures with several lags.
"""
import ctypes

import numpy as np
import pytest

from cases import layered_model, rand_c, rel_l2, ricker
from wemgpu.params import WEM_DATA_FREQ, WEM_DATA_TIME, make_params

ROWS = (256, 384, 512, 768, 1024)


def row_of(w, pad, tap):
    """Row length and leading zero pad of an aperture row: the smallest of
    the warp kernels' lengths that holds w + 2 tap, padded equally (the
    aperture is not padded by `pad`, BornRefl's taper width)."""
    n = next(r for r in ROWS if r >= w + 2 * tap)
    return n, (n - w) // 2


def offset_case(nx=120, nz=20, ns=4, pad=4, tap=0, prop="ssf", phase_law="ispc", widths=(40, 64, 120, 80),
                nt=96, dt=0.008, fmin=6.0, fmax=13.0, seed=3, ngs=1, ngr=1):
    s, _ = layered_model(nz, nx, seed)
    sx = [nx * (k + 1) // (ns + 1) for k in range(ns)]
    par = dict(ns=ns, osx=10.0 * sx[0], dsx=10.0 * (sx[1] - sx[0]) if ns > 1 else 0.0, osz=0.0,
               nr=nx, orx=0.0, drx=10.0, orz=0.0, prop=prop, nref=1, tap=tap, pad=pad, fmin=fmin, fmax=fmax,
               ngs=ngs, ngr=ngr, phase_law=phase_law)
    p = make_params(par, nx=nx, nz=nz, dx=10.0, dz=10.0, nt=nt, dt=dt)
    srcx = [int(round(p.osx / 10.0)) + k * int(round(p.dsx / 10.0)) for k in range(ns)]
    ap = []
    for k in range(ns):
        w = min(widths[k % len(widths)], nx)
        x0 = min(max(srcx[k] - w // 2, 0), nx - w)
        ap.append((x0, w))
    taps = [row_of(w, pad, tap)[1] for _, w in ap]
    wav = ricker(nt, dt, 10.0)
    return p, par, wav, s, np.array(ap, np.int32), taps


def lag_model(rng, nh, nz, nx):
    m = np.zeros((nh, nz, nx), np.complex64)
    hm = (nh - 1) // 2
    spikes = rng.random((nz, nx)) < 0.05
    for k in range(nh):
        m[k] = spikes * rand_c(rng, (nz, nx)) * np.exp(-0.5 * ((k - hm) / max(hm / 2, 1)) ** 2)
    return m


def sub_params(p, par, ap, shot, srcx):
    """The single-shot problem on the cropped model of the shot's aperture."""
    x0, w = int(ap[shot][0]), int(ap[shot][1])
    sub = dict(par, ns=1, osx=10.0 * srcx, dsx=0.0, nr=w, orx=10.0 * x0, drx=10.0, ox=10.0 * x0)
    return make_params(sub, nx=w, nz=p.nz, dx=p.dx, dz=p.dz, nt=p.nt, dt=p.dt), x0, w


# ------------------------------------------------------------ oracle (CPU)

def test_oracle_one_lag_full_aperture_is_bornrefl(oracle):
    p, par, wav, s, _, _ = offset_case(widths=(120,))
    nf = oracle.count_freqs(p)[0]
    rng = np.random.default_rng(0)
    r = lag_model(rng, 1, p.nz, p.nx)
    ap = np.array([(0, p.nx)] * p.ns, np.int32)
    taps = [p.tap] * p.ns
    for prec in (32, 64):
        d = oracle.offborn_forward(p, wav, s, r, ap, taps, kind=WEM_DATA_FREQ, prec=prec)
        want = oracle.bornrefl_forward(p, wav, s, np.repeat(r, nf, 0), kind=WEM_DATA_FREQ, prec=prec)
        np.testing.assert_array_equal(d, want)
        dd = rand_c(rng, d.shape)
        img = oracle.offborn_adjoint(p, wav, s, 1, dd, ap, taps, kind=WEM_DATA_FREQ, prec=prec)
        ref = oracle.bornrefl_adjoint(p, wav, s, dd, kind=WEM_DATA_FREQ, prec=prec).astype(np.complex128).sum(0)
        assert rel_l2(img[0], ref) < 1e-6  # outputs are complex64; summation order differs


def test_oracle_aperture_is_cropped_bornrefl(oracle):
    """Shot by shot, one lag: the offset operator on an aperture equals BornRefl
    of the one-shot problem on the cropped model (receivers inside the
    aperture; the others record zero)."""
    p, par, wav, s, ap, taps = offset_case()
    nf = oracle.count_freqs(p)[0]
    rng = np.random.default_rng(1)
    r = lag_model(rng, 1, p.nz, p.nx)
    d = oracle.offborn_forward(p, wav, s, r, ap, taps, kind=WEM_DATA_TIME, prec=64)
    dd = rng.standard_normal(d.shape).astype(np.float32)
    img = oracle.offborn_adjoint(p, wav, s, 1, dd, ap, taps, kind=WEM_DATA_TIME, prec=64)
    acc = np.zeros((p.nz, p.nx), np.complex128)
    for k in range(p.ns):
        srcx = int(round((p.osx + k * p.dsx) / p.dx))
        q, x0, w = sub_params(p, par, ap, k, srcx)
        q.tap = taps[k]
        sc = np.ascontiguousarray(s[:, x0:x0 + w])
        rc = np.ascontiguousarray(np.repeat(r[:, :, x0:x0 + w], nf, 0))
        dk = oracle.bornrefl_forward(q, wav, sc, rc, kind=WEM_DATA_TIME, prec=64)
        assert rel_l2(d[k, x0:x0 + w], dk[0]) < 1e-6, k
        assert not np.any(d[k, :x0]) and not np.any(d[k, x0 + w:])
        ik = oracle.bornrefl_adjoint(q, wav, sc, np.ascontiguousarray(dd[k:k + 1, x0:x0 + w]), kind=WEM_DATA_TIME,
                                     prec=64)
        acc[:, x0:x0 + w] += ik.astype(np.complex128).sum(0)
    assert rel_l2(img[0], acc) < 1e-6


@pytest.mark.parametrize("nh", [1, 5])
def test_oracle_dot(oracle, nh):
    p, par, wav, s, ap, taps = offset_case()
    rng = np.random.default_rng(2)
    r = lag_model(rng, nh, p.nz, p.nx) + 0.1 * rand_c(rng, (nh, p.nz, p.nx))
    d = oracle.offborn_forward(p, wav, s, r, ap, taps, kind=WEM_DATA_FREQ, prec=64)
    dd = rand_c(rng, d.shape)
    img = oracle.offborn_adjoint(p, wav, s, nh, dd, ap, taps, kind=WEM_DATA_FREQ, prec=64)
    a = np.vdot(d.astype(np.complex128), dd.astype(np.complex128))
    b = np.vdot(r.astype(np.complex128), img.astype(np.complex128))
    assert abs(a - b) / abs(a) < 1e-6


def test_row_rule():
    assert row_of(40, 4, 0) == (256, 108)
    assert row_of(256, 0, 0) == (256, 0)
    assert row_of(258, 0, 0) == (384, 63)
    assert row_of(1000, 4, 6) == (1024, 12)


# ------------------------------------------------------------------- GPU

def _op(p, wav, s, nh, ap):
    from wemgpu.core import BornOffsetOp
    return BornOffsetOp(p, wav, s, nh, ap)


GPU_CASES = [
    dict(nh=5),
    dict(nh=21, widths=(52, 120, 96, 64)),
    dict(nh=3, pad=0, tap=3, widths=(256, 200, 120, 82), nx=256),
    dict(nh=5, prop="pspi"),
    dict(nh=5, phase_law="exact_kz", widths=(120,)),
    dict(nh=1, nx=300, widths=(300, 260, 40, 300), pad=6),
]


@pytest.mark.gpu
@pytest.mark.parametrize("kw", GPU_CASES, ids=lambda k: "-".join(f"{a}{b}" for a, b in k.items()))
def test_offset_matches_oracle(gpu_lib, oracle, kw):
    kw = dict(kw)
    nh = kw.pop("nh")
    p, par, wav, s, ap, taps = offset_case(**kw)
    op = _op(p, wav, s, nh, ap)
    n, t = op.rows()
    assert list(t) == taps and all(int(n[k]) == row_of(int(ap[k][1]), p.pad, p.tap)[0] for k in range(p.ns))
    rng = np.random.default_rng(4)
    r = lag_model(rng, nh, p.nz, p.nx)
    d = np.zeros((p.ns, p.nr, p.nt), np.float32)
    op.forward(r, d)
    for prec in (32, 64):
        o = oracle.offborn_forward(p, wav, s, r, ap, taps, kind=WEM_DATA_TIME, prec=prec)
        assert rel_l2(d, o) < 1e-4, (prec, rel_l2(d, o))
    dd = rng.standard_normal(d.shape).astype(np.float32)
    img = np.zeros((nh, p.nz, p.nx), np.complex64)
    op.adjoint(img, dd)
    for prec in (32, 64):
        o = oracle.offborn_adjoint(p, wav, s, nh, dd, ap, taps, kind=WEM_DATA_TIME, prec=prec)
        assert rel_l2(img, o) < 1e-4, (prec, rel_l2(img, o))
    # dot test, bins (complex data)
    nb = p.nt + p.tpad
    df = np.zeros((p.ns, p.nr, nb), np.complex64)
    op.forward(r, df)
    g = rand_c(rng, df.shape)
    im2 = np.zeros_like(img)
    op.adjoint(im2, g)
    a = np.vdot(df.astype(np.complex128), g.astype(np.complex128))
    b = np.vdot(r.astype(np.complex128), im2.astype(np.complex128))
    assert abs(a - b) / abs(a) < 1e-5


@pytest.mark.gpu
def test_offset_one_lag_is_bornrefl_gpu(gpu_lib):
    """One lag, full apertures: the GPU offset operator against the GPU
    BornRefl (its own oracle-pinned path) with the same row."""
    from wemgpu.core import BornReflOp
    p, par, wav, s, _, _ = offset_case(widths=(120,), tap=68)  # 120 + 136 = 256 points (pad is the taper)
    ap = np.array([(0, p.nx)] * p.ns, np.int32)
    op = _op(p, wav, s, 1, ap)
    assert list(op.rows()[1]) == [68] * p.ns
    ref = BornReflOp(p, wav, s)
    nf = ref.nfreq()
    rng = np.random.default_rng(5)
    r = lag_model(rng, 1, p.nz, p.nx)
    d = np.zeros((p.ns, p.nr, p.nt), np.float32)
    op.forward(r, d)
    dr = np.zeros_like(d)
    ref.forward(np.ascontiguousarray(np.repeat(r, nf, 0)), dr)
    assert rel_l2(d, dr) < 1e-5
    dd = rng.standard_normal(d.shape).astype(np.float32)
    img = np.zeros((1, p.nz, p.nx), np.complex64)
    op.adjoint(img, dd)
    ir = np.zeros((nf, p.nz, p.nx), np.complex64)
    ref.adjoint(ir, dd)
    assert rel_l2(img[0], ir.astype(np.complex128).sum(0)) < 1e-5


@pytest.mark.gpu
def test_offset_device_arrays_and_add(gpu_lib):
    import torch
    p, par, wav, s, ap, taps = offset_case()
    op = _op(p, wav, s, 5, ap)
    rng = np.random.default_rng(6)
    r = lag_model(rng, 5, p.nz, p.nx)
    d = np.zeros((p.ns, p.nr, p.nt), np.float32)
    op.forward(r, d)
    td = torch.zeros(d.shape, dtype=torch.float32, device="cuda")
    op.forward(torch.from_numpy(r).cuda(), td)
    np.testing.assert_array_equal(td.cpu().numpy(), d)
    op.forward(r, d, add=True)
    np.testing.assert_allclose(d, 2 * td.cpu().numpy(), rtol=1e-6, atol=1e-12)
    img = np.zeros((5, p.nz, p.nx), np.complex64)
    op.adjoint(img, d)
    timg = torch.zeros(img.shape, dtype=torch.complex64, device="cuda")
    op.adjoint(timg, torch.from_numpy(d).cuda())
    np.testing.assert_array_equal(timg.cpu().numpy(), img)


@pytest.mark.gpu
def test_offset_rejects_bad_set_ups(gpu_lib):
    from wemgpu._lib import WemError
    p, par, wav, s, ap, taps = offset_case()
    for nh, a, msg in [(4, ap, "odd"), (5, np.array([(0, 41)] + [tuple(x) for x in ap[1:]]), "even"),
                       (5, np.array([(60, 40)] + [tuple(x) for x in ap[1:]]), "source"),
                       (5, np.array([(100, 40)] + [tuple(x) for x in ap[1:]]), "outside the model")]:
        with pytest.raises(WemError) as e:
            _op(p, wav, s, nh, a)
        assert e.value.code == 1 and msg in str(e.value), str(e.value)
    q = p.copy()
    q.nref = 2
    with pytest.raises(WemError):
        _op(q, wav, s, 5, ap)
