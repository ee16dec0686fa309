"""Host-side logic of the reference-facing operator classes (wemgpu.ops),
without a GPU: the background and reflectivity chains of BornRefl and
BornTomo (propagator/src/python/WEM.py:85-134).  The library handle is
replaced by a recorder, so only the Python composition is under test."""
import numpy as np

from wemgpu import ops
from wemgpu.vector import Hypercube, Vector


class _Recorder:
    def __init__(self):
        self.bg = None
        self.refl = None

    def set_background(self, a):
        self.bg = np.array(a)

    def set_refl(self, a):
        self.refl = np.array(a)


class _Scale:
    """data = k * model on a larger grid: rows repeated twice (a stand-in
    for a coarse-to-fine interpolator)."""

    def __init__(self, model, k):
        nz, nx = model.getNdArray().shape
        self.range = Vector(Hypercube([nx, 2 * nz]), np.zeros((2 * nz, nx), np.complex64))
        self.k = k

    def forward(self, add, model, data):
        out = self.k * np.repeat(model.getNdArray(), 2, axis=0)
        if add:
            data.getNdArray()[:] += out
        else:
            data.getNdArray()[:] = out


class _PadX:
    """Edge-extended pad of w cells on both sides of the fastest axis."""

    def __init__(self, shape, w):
        self.w = w
        *lead, nx = shape
        self.range = Vector(Hypercube(list(reversed(list(lead) + [nx + 2 * w]))),
                            np.zeros(tuple(lead) + (nx + 2 * w,), np.complex64))

    def forward(self, add, model, data):
        a = model.getNdArray()
        pad = [(0, 0)] * (a.ndim - 1) + [(self.w, self.w)]
        out = np.pad(a, pad, mode="edge")
        if add:
            data.getNdArray()[:] += out
        else:
            data.getNdArray()[:] = out


def _slow(nz=4, nx=5, seed=0):
    rng = np.random.default_rng(seed)
    a = (rng.random((nz, nx)) + 1j * rng.random((nz, nx))).astype(np.complex64)
    return Vector(Hypercube([nx, nz]), a)


def _bornrefl():
    op = ops.BornRefl.__new__(ops.BornRefl)
    op.prec, op.pad, op.cppMode = None, None, _Recorder()
    return op


def test_bornrefl_background_without_chain():
    op, s = _bornrefl(), _slow()
    op.set_background(s)
    assert np.array_equal(op.cppMode.bg, s.getNdArray())


def test_bornrefl_background_through_prec_then_pad():
    """WEM.py:108-115: the preconditioner first, then the pad."""
    op, s = _bornrefl(), _slow()
    prec = _Scale(s, 3)
    op.add_prec(prec)
    op.add_pad(_PadX(prec.range.getNdArray().shape, 2))
    op.set_background(s)
    want = np.pad(3 * np.repeat(s.getNdArray(), 2, axis=0), [(0, 0), (2, 2)], mode="edge")
    assert np.array_equal(op.cppMode.bg, want)
    # a second call starts from the new model, not from what the first left
    s2 = _slow(seed=1)
    op.set_background(s2)
    want2 = np.pad(3 * np.repeat(s2.getNdArray(), 2, axis=0), [(0, 0), (2, 2)], mode="edge")
    assert np.array_equal(op.cppMode.bg, want2)


def test_bornrefl_background_through_pad_only():
    op, s = _bornrefl(), _slow()
    op.add_pad(_PadX(s.getNdArray().shape, 1))
    op.set_background(s)
    assert np.array_equal(op.cppMode.bg, np.pad(s.getNdArray(), [(0, 0), (1, 1)], mode="edge"))


def test_borntomo_reflectivity_through_pad():
    """WEM.py:123-131: setBgRefl pads the reflectivity first."""
    op = ops.BornTomo.__new__(ops.BornTomo)
    op.pad, op.cppMode = None, _Recorder()
    rng = np.random.default_rng(2)
    r = rng.random((3, 4, 5)).astype(np.complex64)  # [nfreq][nz][nx]
    refl = Vector(Hypercube([5, 4, 3]), r)
    op.setBgRefl(refl)
    assert np.array_equal(op.cppMode.refl, r)
    op.add_pad(_PadX(r.shape, 2))
    op.setBgRefl(refl)
    assert np.array_equal(op.cppMode.refl, np.pad(r, [(0, 0), (0, 0), (2, 2)], mode="edge"))
