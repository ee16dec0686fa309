"""The reference's Python operator API, on the GB300 library.

Class names, constructor arguments and ``forward(add, model, data)`` /
``adjoint(add, model, data)`` follow propagator/src/python/WEM.py:8-134 and
newExtWEM.py:8-38, so FWI/EFWI scripts written against the reference
(scripts/fwi.py:70-71, scripts/efwi.py:97-98, scripts/mig.py:57-63) run on
these classes unchanged apart from the import.  Models are a
``superVector(slowness^2, density)``; data are real ``[ns][nr][nt]`` traces
or complex ``[ns][nr][nbin]`` bins (the dtype of the data vector decides).
"""
from __future__ import annotations

from typing import Any

import numpy as np

from . import core
from .params import make_params
from .vector import Hypercube, SuperVector, Vector


def _grid_params(par, model_hyper: Hypercube, wave: Vector, data: Vector = None):
    ax1, ax2 = model_hyper.getAxis(1), model_hyper.getAxis(2)
    wt = wave.getHyper().getAxis(1)
    p = make_params(par, nx=ax1.n, nz=ax2.n, dx=ax1.d, dz=ax2.d, ox=ax1.o, oz=ax2.o,
                    nt=wt.n, dt=wt.d, ot=wt.o)
    if data is not None and data.is_complex:
        p.nbin = data.getHyper().getAxis(1).n
    return p


def _refl_params(par, model_hyper: Hypercube, wave: Vector, data: Vector = None):
    """BornRefl / BornTomo read the source spreading from "ng"
    (ext_born_refl.cpp:18, ext_born_tomo.cpp:20) and record with point
    receivers; the library takes "ng" in ngs."""
    p = _grid_params(par, model_hyper, wave, data)
    m = par.pars if hasattr(par, "pars") else (par or {})
    p.ngs = int(m.get("ng", 0))
    p.ngr = 0
    return p


def _vecs(model):
    if isinstance(model, SuperVector):
        return model.vecs
    if isinstance(model, (list, tuple)):
        return list(model)
    raise TypeError("Model vector should be a superVector")


class Propagator:
    """Base of the modelling operators (WEM.py:8-35)."""

    def __init__(self, model, data, wave, par):
        if not isinstance(model, SuperVector):
            raise TypeError("Model vector should be a superVector")
        self.wave = wave
        self.par = par
        self.domain = model
        self.range = data

    def setDomainRange(self, model, data):
        self.domain, self.range = model, data

    def _op(self):
        raise NotImplementedError

    @classmethod
    def from_subspace(cls, subdomain, subrange, wave, par, *args, **kw):
        """Operator for a block of shots (WEM.py:24-30): ns and osx come from
        the sub-range's third axis."""
        pars = dict(par.pars if hasattr(par, "pars") else par)
        ax3 = subrange.getHyper().getAxis(3)
        pars["ns"] = ax3.n
        pars["osx"] = ax3.o
        return cls(subdomain, subrange, wave, pars, *args, **kw)

    def __getstate__(self):
        state = self.__dict__.copy()
        state.pop("cppMode", None)
        return state

    def dotTest(self, verbose=False, seed=0):
        """<L m, d> versus <m, L^H d> for random m and d, add=False and add=True
        (operator/src/Operator.h:23-48).  Returns the two relative errors."""
        m = self.domain.clone().rand(seed)
        d = self.range.clone().rand(seed + 7)
        m1, d1 = self.domain.clone().zero(), self.range.clone().zero()
        out = []
        for add in (False, True):
            if add:
                # the outputs' prior contents get the norms of L m and L^H d:
                # much larger ones would swamp the added part in fp32
                nd, nm = d1.norm(), m1.norm()
                m1.rand(seed + 11)
                d1.rand(seed + 13)
                if nm > 0:
                    m1.scale(nm / max(m1.norm(), 1e-300))
                if nd > 0:
                    d1.scale(nd / max(d1.norm(), 1e-300))
                m1c, d1c = m1.clone(), d1.clone()
            self.forward(add, m, d1)
            self.adjoint(add, m1, d)
            if add:
                lhs = d1.dot(d) - d1c.dot(d)
                rhs = m1.dot(m) - m1c.dot(m)
            else:
                lhs, rhs = d1.dot(d), m1.dot(m)
            err = abs(lhs - rhs) / max(abs(lhs), abs(rhs), 1e-300)
            if verbose:
                print(f"add={add}: <Lm,d>={lhs:.8e} <m,L'd>={rhs:.8e} rel={err:.3e}")
            out.append(err)
        return out


class WEM(Propagator):
    """Nonlinear one-way modelling (WEM.py:37-50; WEMnl.cpp, wem_prop.cpp)."""

    def __init__(self, model, data, wave, par):
        super().__init__(model, data, wave, par)
        self.params = _grid_params(par, _vecs(model)[0].getHyper(), wave, data)
        self.cppMode = core.WemOp(self.params, wave.getNdArray())

    def __setstate__(self, state):
        self.__dict__ = state.copy()
        self.cppMode = core.WemOp(self.params, self.wave.getNdArray())

    def get_nfreq(self):
        return self.cppMode.nfreq()

    def forward(self, add, model, data):
        m = _vecs(model)
        self.cppMode.forward(m[0].getNdArray(), m[1].getNdArray(), data.getNdArray(), add)


class Born(Propagator):
    """Born operator (WEM.py:52-80; BornFull).  ``mode='real'`` zeroes the
    imaginary part of the model around the calls, as the reference does."""

    def __init__(self, model, data, wave, par, mode=None):
        super().__init__(model, data, wave, par)
        self.mode = mode
        m = _vecs(model)
        self.params = _grid_params(par, m[0].getHyper(), wave, data)
        self.cppMode = core.BornOp(self.params, wave.getNdArray(), m[0].getNdArray(), m[1].getNdArray())

    def __setstate__(self, state):
        self.__dict__ = state.copy()
        m = _vecs(self.domain)
        self.cppMode = core.BornOp(self.params, self.wave.getNdArray(), m[0].getNdArray(), m[1].getNdArray())

    @classmethod
    def from_subspace(cls, subdomain, subrange, wave, par, mode=None):
        return super().from_subspace(subdomain, subrange, wave, par, mode=mode)

    def set_background(self, slow):
        m = _vecs(slow)
        self.cppMode.set_background(m[0].getNdArray(), m[1].getNdArray())

    def forward(self, add, model, data):
        m = _vecs(model)
        if self.mode == "real":
            for v in m:
                v.getNdArray().imag[...] = 0
        self.cppMode.forward(m[0].getNdArray(), m[1].getNdArray(), data.getNdArray(), add)

    def adjoint(self, add, model, data):
        m = _vecs(model)
        self.cppMode.adjoint(m[0].getNdArray(), m[1].getNdArray(), data.getNdArray(), add)
        if self.mode == "real":
            for v in m:
                v.getNdArray().imag[...] = 0


class extWEM(Propagator):
    """Frequency-extended modelling (newExtWEM.py:8-24): model axis 3 is the
    propagated frequency."""

    def __init__(self, model, data, wave, par):
        super().__init__(model, data, wave, par)
        self.params = _grid_params(par, _vecs(model)[0].getHyper(), wave, data)
        self.cppMode = core.ExtWemOp(self.params, wave.getNdArray())
        nw = _vecs(model)[0].getHyper().getAxis(3).n
        if nw != self.cppMode.nfreq():
            raise ValueError("Model is of the wrong size!")

    def forward(self, add, model, data):
        m = _vecs(model)
        self.cppMode.forward(m[0].getNdArray(), m[1].getNdArray(), data.getNdArray(), add)


class extBorn(Propagator):
    """Frequency-extended Born operator (newExtWEM.py:26-38)."""

    def __init__(self, model, data, wave, par):
        super().__init__(model, data, wave, par)
        m = _vecs(model)
        self.params = _grid_params(par, m[0].getHyper(), wave, data)
        self.cppMode = core.ExtBornOp(self.params, wave.getNdArray(), m[0].getNdArray(), m[1].getNdArray())

    def set_background(self, slow):
        m = _vecs(slow)
        self.cppMode.set_background(m[0].getNdArray(), m[1].getNdArray())

    def forward(self, add, model, data):
        m = _vecs(model)
        self.cppMode.forward(m[0].getNdArray(), m[1].getNdArray(), data.getNdArray(), add)

    def adjoint(self, add, model, data):
        m = _vecs(model)
        self.cppMode.adjoint(m[0].getNdArray(), m[1].getNdArray(), data.getNdArray(), add)


class BornRefl(Propagator):
    """Frequency-extended reflectivity Born (WEM.py:85-115; BornRefl,
    ext_born_refl.cpp:8-105).  model: reflectivity per frequency (a vector
    of shape [nfreq][nz][nx]); slowness: the background slowness^2."""

    def __init__(self, model, slowness, data, wave, par):
        self.wave, self.par, self.domain, self.range = wave, par, model, data
        self.params = _refl_params(par, slowness.getHyper(), wave, data)
        self.cppMode = core.BornReflOp(self.params, wave.getNdArray(), slowness.getNdArray())
        self.prec = None
        self.pad = None

    def add_prec(self, op):
        """The background passes through op.forward first (WEM.py:101-103):
        a coarse model and its interpolator (LanczosInterpolation2D,
        Spline2D)."""
        self.prec = op
        self.big_model = op.range.clone()

    def add_pad(self, op):
        """Then through op.forward (WEM.py:104-106): BornRefl propagates on
        the grid it is given, so a padding operator extends the slowness."""
        self.pad = op
        self.pad_model = op.range.clone()

    def set_background(self, slow):
        # WEM.py:108-115: preconditioner, then pad, then the background
        if self.prec is not None:
            self.prec.forward(False, slow, self.big_model)
            slow = self.big_model
        if self.pad is not None:
            self.pad.forward(False, slow, self.pad_model)
            slow = self.pad_model
        self.cppMode.set_background(slow.getNdArray())

    def forward(self, add, model, data):
        self.cppMode.forward(model.getNdArray(), data.getNdArray(), add)

    def adjoint(self, add, model, data):
        self.cppMode.adjoint(model.getNdArray(), data.getNdArray(), add)


class BornTomo(Propagator):
    """Frequency-extended tomographic Born (WEM.py:117-134; BornTomo,
    ext_born_tomo.cpp:9-119).  As in pyWEM.BornTomo(wave, slow, par), the
    constructor's model vector is the background slowness^2; forward and
    adjoint take a slowness^2 perturbation; setBgRefl sets the reflectivity
    per frequency ([nfreq][nz][nx])."""

    def __init__(self, model, data, wave, par):
        self.wave, self.par, self.domain, self.range = wave, par, model, data
        self.params = _refl_params(par, model.getHyper(), wave, data)
        self.cppMode = core.BornTomoOp(self.params, wave.getNdArray(), model.getNdArray())
        self.pad = None

    def add_pad(self, op):
        """The reflectivity passes through op.forward before it is set
        (WEM.py:123-131)."""
        self.pad = op
        self.pad_refl = op.range.clone()

    def setBgRefl(self, refl):
        if self.pad is not None:
            self.pad.forward(False, refl, self.pad_refl)
            refl = self.pad_refl
        self.cppMode.set_refl(refl.getNdArray())

    def set_background(self, slow):
        self.cppMode.set_background(slow.getNdArray())

    def forward(self, add, model, data):
        self.cppMode.forward(model.getNdArray(), data.getNdArray(), add)

    def adjoint(self, add, model, data):
        self.cppMode.adjoint(model.getNdArray(), data.getNdArray(), add)


class BornOffset(Propagator):
    """Subsurface-offset extended reflectivity Born with per-shot apertures
    (no reference counterpart; BornRefl's operator, ext_born_refl.cpp:8-105,
    with the imaging condition extended over nh horizontal lags).  model: a
    vector of shape [nh][nz][nx]; slowness: the background slowness^2;
    apertures: per shot (x0, w) in model columns, or None (whole model)."""

    def __init__(self, model, slowness, data, wave, par, nh, apertures=None):
        self.wave, self.par, self.domain, self.range = wave, par, model, data
        self.params = _grid_params(par, slowness.getHyper(), wave, data)
        self.cppMode = core.BornOffsetOp(self.params, wave.getNdArray(), slowness.getNdArray(), nh, apertures)

    def set_background(self, slow):
        self.cppMode.set_background(slow.getNdArray())

    def forward(self, add, model, data):
        self.cppMode.forward(model.getNdArray(), data.getNdArray(), add)

    def adjoint(self, add, model, data):
        self.cppMode.adjoint(model.getNdArray(), data.getNdArray(), add)


class LanczosInterpolation2D(Propagator):
    """Coarse-to-fine windowed-sinc interpolation of a 2D complex model
    (Operator.py:436-445; operator/src/LanczosInterpolation2D.h), the model
    preconditioner of scripts/fwi.py:45-68.  ``a`` holds the half widths in
    coarse samples along axes 1 and 2 (a third entry is ignored)."""

    def __init__(self, model, data, a=[3, 3, 3]):
        self.a = list(a)
        self.setDomainRange(model, data)
        self.cppMode = core.Interp2DOp("lanczos", _axes2(model), _axes2(data), self.a[:2])

    def __setstate__(self, state):
        self.__dict__ = state.copy()
        self.cppMode = core.Interp2DOp("lanczos", _axes2(self.domain), _axes2(self.range), self.a[:2])

    def forward(self, add, model, data):
        self.cppMode.forward(model.getNdArray(), data.getNdArray(), add)

    def adjoint(self, add, model, data):
        self.cppMode.adjoint(model.getNdArray(), data.getNdArray(), add)


class Spline(Propagator):
    """Cubic-spline interpolation base (Operator.py:447-465).  ``type`` names
    a member of the (a, b) family: 'CR-spline' (0.5, 0), 'B-spline' (0, 1),
    'MN-spline' (1/3, 1/3).  As in the reference, the filter is built from
    the ``a`` and ``b`` arguments; ``type`` sets the attributes ``a``, ``b``
    that an unpickled operator is rebuilt with."""

    _TYPES = {"CR-spline": (0.5, 0.0), "B-spline": (0.0, 1.0), "MN-spline": (1 / 3, 1 / 3)}

    def __init__(self, model, data, a=1, b=0, type=None):
        self.a, self.b = self._TYPES.get(type, (a, b))
        self.setDomainRange(model, data)

    def forward(self, add, model, data):
        self.cppMode.forward(model.getNdArray(), data.getNdArray(), add)

    def adjoint(self, add, model, data):
        self.cppMode.adjoint(model.getNdArray(), data.getNdArray(), add)


class Spline2D(Spline):
    """2D cubic-spline interpolation (Operator.py:467-478; operator/src/Spline2D.h).
    Its adjoint copies the model's edge columns and rows from their
    neighbours, as the reference's does, so a dot test fails at the edges."""

    def __init__(self, model, data, a=1, b=0, type=None):
        super().__init__(model, data, a, b, type=type)
        self.cppMode = core.Interp2DOp("spline", _axes2(model), _axes2(data), a, b)

    def __setstate__(self, state):
        self.__dict__ = state.copy()
        self.cppMode = core.Interp2DOp("spline", _axes2(self.domain), _axes2(self.range), self.a, self.b)


def _axes2(vec):
    h = vec.getHyper()
    return tuple((h.getAxis(i).n, h.getAxis(i).d) for i in (1, 2))
