"""The reference's per-operator Python classes (propagator/src/python/wem_ops.py:6-137),
on the GB300 library.

Class names, constructor arguments and ``forward(add, model, data)`` /
``adjoint(add, model, data)`` follow wem_ops.py, so the reference's operator
tests (propagator/test/test_wem_ops.py) read the same against this module.
Vectors are this package's ``Vector`` / ``SuperVector`` (wemgpu.vector), whose
hypercubes give the grid: axis 1 = x, axis 2 = z.  ``par`` is a dict or an
object with ``.pars`` holding the reference's keys (tap, pad, eps, prop, nref,
ntaylor, ...).  Every operator runs on the CUDA library.
"""
from __future__ import annotations

import numpy as np

from . import core
from .ops import Propagator
from .params import WEM_PROP_SSF, make_params


def _grid(slow, par=None, **over):
    """Parameter block of the slowness grid (axis 1 = x, axis 2 = z)."""
    h = slow.getHyper()
    ax1, ax2 = h.getAxis(1), h.getAxis(2)
    pars = dict(par.pars if hasattr(par, "pars") else (par or {}))
    pars.update(over)
    return make_params(pars, nx=ax1.n, nz=ax2.n, dx=ax1.d, dz=ax2.d, ox=ax1.o, oz=ax2.o, nt=1, dt=1.0)


def _arr(v):
    return v.getNdArray()


class _RowOperator(Propagator):
    """Base of the per-operator classes: domain/range and the dot test of
    the operator API (no Propagator set-up)."""

    def __init__(self, model, data):
        self.setDomainRange(model, data)

    def __getstate__(self):
        return {k: v for k, v in self.__dict__.items() if k != "cppMode"}


class SplitStep(_RowOperator):
    """Split-step correction of one depth on the points ``loc``
    (SplitStep.cpp:5-29; wem_ops.py:6-17)."""

    def __init__(self, model, data, slow, freq, loc, s0, depth):
        super().__init__(model, data)
        self.cppMode = core.RowOps(_grid(slow), _arr(slow))
        self.freq, self.loc, self.s0, self.depth = float(freq), list(loc), complex(s0), int(depth)

    def forward(self, add, model, data):
        self.cppMode.splitstep(self.depth, self.freq, self.s0, self.loc, 0, _arr(model), _arr(data), add)

    def adjoint(self, add, model, data):
        self.cppMode.splitstep(self.depth, self.freq, self.s0, self.loc, 1, _arr(data), _arr(model), add)


class Scatter(_RowOperator):
    """Taylor Born scatter of one depth (Scatter.cpp:6-111; wem_ops.py:19-28)."""

    def __init__(self, model, data, slow, ntaylor, freq, depth, par):
        super().__init__(model, data)
        self.cppMode = core.RowOps(_grid(slow, par, ntaylor=int(ntaylor)), _arr(slow))
        self.freq, self.depth = float(freq), int(depth)

    def forward(self, add, model, data):
        self.cppMode.scatter(self.depth, self.freq, 0, _arr(model), _arr(data), add)

    def adjoint(self, add, model, data):
        self.cppMode.scatter(self.depth, self.freq, 1, _arr(data), _arr(model), add)


class SSF(_RowOperator):
    """One split-step Fourier depth step (SSF.cpp:8-60; wem_ops.py:30-39).
    ``ref`` is the RefSampler of the same slowness; the library samples the
    references itself with the same rule."""

    def __init__(self, model, data, slow, freq, depth, par, ref):
        super().__init__(model, data)
        over = dict(prop=WEM_PROP_SSF)
        if isinstance(ref, RefSampler):
            over["nref"] = ref.nref
        self.cppMode = core.RowOps(_grid(slow, par, **over), _arr(slow))
        self.freq, self.depth = float(freq), int(depth)

    def forward(self, add, model, data):
        self.cppMode.onestep(self.depth, self.freq, 0, _arr(model), _arr(data), add)

    def adjoint(self, add, model, data):
        self.cppMode.onestep(self.depth, self.freq, 1, _arr(data), _arr(model), add)


class Reflect(_RowOperator):
    """Reflection coefficients of (slowness^2, density) (Reflect.h:12-48;
    wem_ops.py:41-49).  As the reference's, the output is assigned."""

    def __init__(self, model, data, slow):
        super().__init__(model, data)
        self.slow = [_arr(v) for v in slow.vecs]

    def forward(self, add, model, data):
        core.reflect(self.slow[0], self.slow[1], 0, _arr(model), _arr(data))

    def adjoint(self, add, model, data):
        core.reflect(self.slow[0], self.slow[1], 1, _arr(data), _arr(model))


class RefSampler:
    """Reference slownesses of each depth (RefSampler.cpp:10-91; wem_ops.py:51-56)."""

    def __init__(self, slow, nref):
        self.nref = int(nref)
        self.cppMode = core.RowOps(_grid(slow, nref=self.nref), _arr(slow))
        self._sref, self._idx = self.cppMode.refsampler()

    def getRefSlow(self, iz, iref):
        return complex(self._sref[iz, iref])


class Phshift(_RowOperator):
    """Phase shift in the wavenumber domain (Phshift_cmplx.cpp:47-113;
    wem_ops.py:58-68): rows on the hypercube ``hyper`` (axis 1 = k samples of
    a row of that length and spacing), slowness ``s0``, eps 0.04 (the
    reference's default).  ``iref`` selects a table of the reference's
    Phshift that the shift itself does not read."""

    def __init__(self, model, data, hyper, dz, freq, s0, iref):
        super().__init__(model, data)
        ax = hyper.getAxis(1)
        self.p = make_params({}, nx=ax.n, nz=2, dx=ax.d, dz=float(dz), nt=1, dt=1.0)
        self.dx, self.dz, self.freq, self.s0, self.iref = ax.d, float(dz), float(freq), complex(s0), int(iref)

    def forward(self, add, model, data):
        core.phshift(self.p, self.dx, self.dz, self.freq, self.s0, 0, _arr(model), _arr(data), add)

    def adjoint(self, add, model, data):
        core.phshift(self.p, self.dx, self.dz, self.freq, self.s0, 1, _arr(data), _arr(model), add)


class _OneWay(_RowOperator):
    UP = 0

    def __init__(self, model, data, slow, par, ref, freq):
        super().__init__(model, data)
        over = {"nref": ref.nref} if isinstance(ref, RefSampler) else {}
        self.cppMode = core.RowOps(_grid(slow, par, **over), _arr(slow))
        self.freq = float(freq)

    def forward(self, add, model, data):
        m, d = _arr(model), _arr(data)
        # the reference's Down/Up run in place when model is data (OneWay.cpp:32-109)
        self.cppMode.oneway(self.UP, self.freq, 0, m, d, add)

    def adjoint(self, add, model, data):
        self.cppMode.oneway(self.UP, self.freq, 1, _arr(data), _arr(model), add)


class Down(_OneWay):
    """Downward continuation over every depth (OneWay.cpp:32-68; wem_ops.py:70-78)."""
    UP = 0


class Up(_OneWay):
    """Upward continuation over every depth (OneWay.cpp:70-109; wem_ops.py:80-88)."""
    UP = 1


class IC(_RowOperator):
    """Imaging condition with the background wavefield ``bg`` (ic.cpp:5-45;
    wem_ops.py:90-98): on a row, the background's row ``depth``; on a field,
    the whole background."""

    def __init__(self, model, data, bg, depth):
        super().__init__(model, data)
        self.bg, self.depth = _arr(bg), int(depth)

    def _bg_for(self, x):
        if x.ndim == 1:
            return np.ascontiguousarray(self.bg[self.depth])
        return self.bg

    def forward(self, add, model, data):
        m = _arr(model)
        core.ic(self._bg_for(m), 0, m, _arr(data), add)

    def adjoint(self, add, model, data):
        d = _arr(data)
        core.ic(self._bg_for(d), 1, d, _arr(model), add)


class LinDown(_RowOperator):
    """Linearised downward continuation around ``bg`` (LinOneWay.cpp:33-85;
    wem_ops.py:100-108).  ``oneway`` is the Down operator it linearises; its
    parameters are those of ``par``."""

    def __init__(self, model, data, slow, par, bg, oneway, freq):
        super().__init__(model, data)
        over = {}
        ref = getattr(oneway, "cppMode", None)
        if ref is not None:
            over["nref"] = ref.p.nref
        self.cppMode = core.RowOps(_grid(slow, par, **over), _arr(slow))
        self.bg, self.freq = _arr(bg), float(freq)

    def forward(self, add, model, data):
        self.cppMode.lindown(self.bg, self.freq, 0, _arr(model), _arr(data), add)

    def adjoint(self, add, model, data):
        self.cppMode.lindown(self.bg, self.freq, 1, _arr(data), _arr(model), add)


class dReflect(_RowOperator):
    """Linearised reflection coefficients at (slowness^2, density)
    (dReflect.h:11-84; wem_ops.py:110-120); the model is a superVector
    (dslowness^2, ddensity)."""

    def __init__(self, model, data, slow):
        super().__init__(model, data)
        self.slow = [_arr(v) for v in slow.vecs]

    def forward(self, add, model, data):
        m = model.vecs
        core.dreflect(self.slow[0], self.slow[1], 0, _arr(m[0]), _arr(m[1]), _arr(data), add)

    def adjoint(self, add, model, data):
        m = model.vecs
        core.dreflect(self.slow[0], self.slow[1], 1, _arr(m[0]), _arr(m[1]), _arr(data), add)


class Injection(_RowOperator):
    """Point injection and its adjoint (Injection.h:19-65,
    Injection.cpp:8-33, 52-75; wem_ops.py:122-137): the points (z[i], x[i])
    of the data rows [nz][nx], each spread over x[i] + tap + [-ng, ng] by
    the cos^2 window.  The model is [nt] (every point takes its sample
    ``step``) or [nshot][npoints][nt] (point i takes [shot][i][step]);
    setStep / setShot choose them."""

    def __init__(self, model, data, z, x, ng=0, tap=0):
        super().__init__(model, data)
        self.z = [int(v) for v in z]
        self.x = [int(v) for v in x]
        self.ng, self.tap = int(ng), int(tap)
        self.step, self.shot = 0, 0

    def setStep(self, step):
        self.step = int(step)

    def setShot(self, shot):
        self.shot = int(shot)

    def forward(self, add, model, data):
        core.inject(self.z, self.x, self.ng, self.tap, self.step, self.shot, 0, _arr(model), _arr(data), add)

    def adjoint(self, add, model, data):
        core.inject(self.z, self.x, self.ng, self.tap, self.step, self.shot, 1, _arr(model), _arr(data), add)

