"""Array-level handles over the C ABI.

Arrays may be numpy (host; the library stages them through the GPU and the
call returns when the result is back) or torch CUDA tensors (device; used
in place).  Shapes follow the reference: models ``[nz][nx]`` (or
``[nfreq][nz][nx]`` for the extended operators), data ``[ns][nr][nt]``
float32 for time traces or ``[ns][nr][nbin]`` complex64 for bins.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .params import WemParams, WEM_DATA_FREQ, WEM_DATA_TIME

try:
    import torch
except Exception:  # pragma: no cover
    torch = None


def _is_torch(a) -> bool:
    return torch is not None and isinstance(a, torch.Tensor)


def ptr(a, dtype, shape=None, name="array", writable=False):
    """Raw pointer of a C-contiguous numpy array or torch tensor of the
    expected dtype (complex64 / float32) and shape."""
    if a is None:
        raise ValueError(f"{name} is None")
    if _is_torch(a):
        tdt = {np.complex64: torch.complex64, np.float32: torch.float32}[dtype]
        if a.dtype != tdt or not a.is_contiguous():
            raise TypeError(f"{name}: need a contiguous {tdt} tensor, got {a.dtype}")
        if shape is not None and tuple(a.shape) != tuple(shape):
            raise ValueError(f"{name}: shape {tuple(a.shape)} != {tuple(shape)}")
        return ctypes.c_void_p(a.data_ptr())
    if not isinstance(a, np.ndarray) or a.dtype != dtype or not a.flags["C_CONTIGUOUS"]:
        raise TypeError(f"{name}: need a C-contiguous numpy {np.dtype(dtype)} array")
    if writable and not a.flags["WRITEABLE"]:
        raise ValueError(f"{name} is read-only")
    if shape is not None and tuple(a.shape) != tuple(shape):
        raise ValueError(f"{name}: shape {tuple(a.shape)} != {tuple(shape)}")
    return ctypes.c_void_p(a.ctypes.data)


def _data_kind(data):
    if _is_torch(data):
        return WEM_DATA_FREQ if data.is_complex() else WEM_DATA_TIME
    return WEM_DATA_FREQ if np.iscomplexobj(data) else WEM_DATA_TIME


class _Base:
    _destroy = None

    def __init__(self, p: WemParams, wavelet):
        self.p = p.copy()
        self.wavelet = np.ascontiguousarray(np.asarray(wavelet, dtype=np.float32)).reshape(-1)
        if self.wavelet.size != p.nt:
            raise ValueError(f"wavelet has {self.wavelet.size} samples, params say nt={p.nt}")
        self.h = ctypes.c_void_p()

    def __del__(self):
        h = getattr(self, "h", None)
        if h and h.value and self._destroy:
            try:
                getattr(_lib.load(), self._destroy)(h)
            except Exception:
                pass
            self.h = ctypes.c_void_p()

    # ---- shapes
    @property
    def model_shape(self):
        return (self.p.nz, self.p.nx)

    @property
    def nbin(self):
        return self.p.nbin if self.p.nbin else self.p.nt + self.p.tpad

    def data_shape(self, kind):
        return (self.p.ns, self.p.nr, self.p.nt if kind == WEM_DATA_TIME else self.nbin)

    def _data_ptr(self, data, writable):
        kind = _data_kind(data)
        dt = np.float32 if kind == WEM_DATA_TIME else np.complex64
        return ptr(data, dt, self.data_shape(kind), "data", writable), kind

    def nfreq(self) -> int:
        n = ctypes.c_int()
        _lib.call("wem_count_freqs", ctypes.byref(self.p), None, ctypes.byref(n))
        return n.value


class WemOp(_Base):
    """Nonlinear modelling (WEM::forward, propagator/src/WEMnl.cpp:39-82)."""

    _destroy = "wem_destroy"

    def __init__(self, p: WemParams, wavelet):
        super().__init__(p, wavelet)
        _lib.call("wem_create", ctypes.byref(self.p), self.wavelet.ctypes.data_as(ctypes.c_void_p),
                  ctypes.byref(self.h))

    def forward(self, s2, rho, data, add=False):
        d, kind = self._data_ptr(data, True)
        _lib.call("wem_forward", self.h, ptr(s2, np.complex64, self.model_shape, "slowness"),
                  ptr(rho, np.complex64, self.model_shape, "density"), d, kind, int(bool(add)))
        return data

    def gradient(self, s2, rho, data_grad, g_s2, g_rho, add=False, checkpoint=0):
        """(g_s2, g_rho) (+)= J^H data_grad: the exact derivative of the
        modelling at (s2, rho), transposed (wem_gradient); checkpoint k > 1
        keeps every k-th depth and recomputes between."""
        d, kind = self._data_ptr(data_grad, False)
        _lib.call("wem_gradient", self.h, ptr(s2, np.complex64, self.model_shape, "slowness"),
                  ptr(rho, np.complex64, self.model_shape, "density"), d, kind,
                  ptr(g_s2, np.complex64, self.model_shape, "g_slowness", True),
                  ptr(g_rho, np.complex64, self.model_shape, "g_density", True), int(bool(add)), int(checkpoint))
        return g_s2, g_rho


class BornOp(_Base):
    """Born operator (BornFull, propagator/src/BornFull.cpp:13-117)."""

    _destroy = "born_destroy"
    _prefix = "born"

    def __init__(self, p: WemParams, wavelet, bg_s2, bg_rho):
        super().__init__(p, wavelet)
        _lib.call(f"{self._prefix}_create", ctypes.byref(self.p), self.wavelet.ctypes.data_as(ctypes.c_void_p),
                  ptr(bg_s2, np.complex64, self.model_shape, "slowness"),
                  ptr(bg_rho, np.complex64, self.model_shape, "density"), ctypes.byref(self.h))

    def set_background(self, s2, rho):
        _lib.call(f"{self._prefix}_set_background", self.h, ptr(s2, np.complex64, self.model_shape, "slowness"),
                  ptr(rho, np.complex64, self.model_shape, "density"))

    def forward(self, ds2, drho, data, add=False):
        d, kind = self._data_ptr(data, True)
        _lib.call(f"{self._prefix}_forward", self.h, ptr(ds2, np.complex64, self.model_shape, "dslow"),
                  ptr(drho, np.complex64, self.model_shape, "drho"), d, kind, int(bool(add)))
        return data

    def adjoint(self, ds2, drho, data, add=False):
        d, kind = self._data_ptr(data, False)
        _lib.call(f"{self._prefix}_adjoint", self.h, ptr(ds2, np.complex64, self.model_shape, "dslow", True),
                  ptr(drho, np.complex64, self.model_shape, "drho", True), d, kind, int(bool(add)))
        return ds2, drho


class FwiOp(_Base):
    """FWI objective and gradient in one call (fwi_gradient): the loss
    1/2 ||WEM(m) - d_obs||^2 and the Born adjoint of the residual at m, as
    scripts/fwi.py:70-71,90 composes them from WEM and Born."""

    _destroy = "fwi_destroy"

    def __init__(self, p: WemParams, wavelet):
        super().__init__(p, wavelet)
        _lib.call("fwi_create", ctypes.byref(self.p), self.wavelet.ctypes.data_as(ctypes.c_void_p),
                  ctypes.byref(self.h))

    def gradient(self, s2, rho, d_obs, g_s2, g_rho, exact=False, checkpoint=0) -> float:
        """Loss and gradient; exact=True differentiates the modelling itself
        (fwi_gradient_exact) instead of the reference's Born adjoint."""
        loss = ctypes.c_double()
        args = [self.h, ptr(s2, np.complex64, self.model_shape, "slowness"),
                ptr(rho, np.complex64, self.model_shape, "density"),
                ptr(d_obs, np.float32, self.data_shape(WEM_DATA_TIME), "d_obs"),
                ptr(g_s2, np.complex64, self.model_shape, "g_slowness", True),
                ptr(g_rho, np.complex64, self.model_shape, "g_density", True), ctypes.byref(loss)]
        if exact:
            _lib.call("fwi_gradient_exact", *args, int(checkpoint))
        else:
            _lib.call("fwi_gradient", *args)
        return loss.value


class BornReflOp(_Base):
    """Frequency-extended reflectivity Born (BornRefl,
    propagator/src/ext_born_refl.cpp:8-105): model [nfreq][nz][nx] is a
    reflectivity per frequency; forward records Up(bg m_f), adjoint gives the
    per-frequency image sum_s conj(bg) Up^H(data)."""

    _destroy = "bornrefl_destroy"

    def __init__(self, p: WemParams, wavelet, bg_s2):
        super().__init__(p, wavelet)
        _lib.call("bornrefl_create", ctypes.byref(self.p), self.wavelet.ctypes.data_as(ctypes.c_void_p),
                  ptr(bg_s2, np.complex64, (self.p.nz, self.p.nx), "slowness"), ctypes.byref(self.h))

    @property
    def model_shape(self):
        return (self.nfreq(), self.p.nz, self.p.nx)

    def set_background(self, s2):
        _lib.call("bornrefl_set_background", self.h, ptr(s2, np.complex64, (self.p.nz, self.p.nx), "slowness"))

    def forward(self, model, data, add=False):
        d, kind = self._data_ptr(data, True)
        _lib.call("bornrefl_forward", self.h, ptr(model, np.complex64, self.model_shape, "model"), d, kind,
                  int(bool(add)))
        return data

    def adjoint(self, model, data, add=False):
        d, kind = self._data_ptr(data, False)
        _lib.call("bornrefl_adjoint", self.h, ptr(model, np.complex64, self.model_shape, "model", True), d, kind,
                  int(bool(add)))
        return model


class BornOffsetOp(_Base):
    """Subsurface-offset extended reflectivity Born with per-shot apertures
    (no reference counterpart; at one lag it is BornRefl,
    propagator/src/ext_born_refl.cpp:8-105, with one reflectivity for every
    frequency).  Model ``[nh][nz][nx]``: the reflectivity at horizontal lag
    ``i - (nh - 1) // 2`` cells.  ``apertures``: per shot ``(x0, w)`` model
    columns (even ``w``), or None for the whole model; each shot propagates on
    its aperture as a cropped model (``WEM.from_subspace``,
    propagator/src/python/WEM.py:24-30)."""

    _destroy = "bornoff_destroy"

    def __init__(self, p: WemParams, wavelet, bg_s2, nh: int, apertures=None):
        super().__init__(p, wavelet)
        self.nh = int(nh)
        x0 = w = None
        if apertures is not None:
            ap = np.ascontiguousarray(np.asarray(apertures, dtype=np.int32).reshape(p.ns, 2))
            self._x0 = np.ascontiguousarray(ap[:, 0])
            self._w = np.ascontiguousarray(ap[:, 1])
            x0, w = self._x0.ctypes.data_as(ctypes.c_void_p), self._w.ctypes.data_as(ctypes.c_void_p)
        _lib.call("bornoff_create", ctypes.byref(self.p), self.wavelet.ctypes.data_as(ctypes.c_void_p),
                  ptr(bg_s2, np.complex64, (self.p.nz, self.p.nx), "slowness"), self.nh, x0, w,
                  ctypes.byref(self.h))

    @property
    def model_shape(self):
        return (self.nh, self.p.nz, self.p.nx)

    def rows(self):
        """(row length, leading zero pad) of every shot's aperture row."""
        n = np.zeros(self.p.ns, np.int32)
        t = np.zeros(self.p.ns, np.int32)
        _lib.call("bornoff_rows", self.h, n.ctypes.data_as(ctypes.c_void_p), t.ctypes.data_as(ctypes.c_void_p))
        return n, t

    def set_background(self, s2):
        _lib.call("bornoff_set_background", self.h, ptr(s2, np.complex64, (self.p.nz, self.p.nx), "slowness"))

    def forward(self, model, data, add=False):
        d, kind = self._data_ptr(data, True)
        _lib.call("bornoff_forward", self.h, ptr(model, np.complex64, self.model_shape, "model"), d, kind,
                  int(bool(add)))
        return data

    def adjoint(self, model, data, add=False):
        d, kind = self._data_ptr(data, False)
        _lib.call("bornoff_adjoint", self.h, ptr(model, np.complex64, self.model_shape, "model", True), d, kind,
                  int(bool(add)))
        return model


class _Base3D:
    """3D operators: models ``[nz][ny][nx]``, data as in 2D."""

    _destroy = None

    def __init__(self, q, wavelet):
        self.q = q
        self.p = q.p
        self.wavelet = np.ascontiguousarray(np.asarray(wavelet, dtype=np.float32)).reshape(-1)
        if self.wavelet.size != self.p.nt:
            raise ValueError(f"wavelet has {self.wavelet.size} samples, params say nt={self.p.nt}")
        self.h = ctypes.c_void_p()

    def __del__(self):
        h = getattr(self, "h", None)
        if h and h.value and self._destroy:
            try:
                getattr(_lib.load(), self._destroy)(h)
            except Exception:
                pass
            self.h = ctypes.c_void_p()

    @property
    def model_shape(self):
        return (self.p.nz, self.q.ny, self.p.nx)

    @property
    def nbin(self):
        return self.p.nbin if self.p.nbin else self.p.nt + self.p.tpad

    def data_shape(self, kind):
        return (self.p.ns, self.p.nr, self.p.nt if kind == WEM_DATA_TIME else self.nbin)

    def _data_ptr(self, data, writable):
        kind = _data_kind(data)
        dt = np.float32 if kind == WEM_DATA_TIME else np.complex64
        return ptr(data, dt, self.data_shape(kind), "data", writable), kind

    def nfreq(self) -> int:
        n = ctypes.c_int()
        _lib.call("wem_count_freqs", ctypes.byref(self.p), None, ctypes.byref(n))
        return n.value


class Wem3DOp(_Base3D):
    """3D nonlinear modelling on planes (WEM's call sequence,
    propagator/src/wem_prop.cpp:9-78, with a 2D FFT per depth slice);
    ``checkpoint`` k > 1 keeps every k-th depth of the down field."""

    _destroy = "wem3d_destroy"

    def __init__(self, q, wavelet):
        super().__init__(q, wavelet)
        _lib.call("wem3d_create", ctypes.byref(q), self.wavelet.ctypes.data_as(ctypes.c_void_p), ctypes.byref(self.h))

    def forward(self, s2, rho, data, add=False, checkpoint=0):
        d, kind = self._data_ptr(data, True)
        _lib.call("wem3d_forward", self.h, ptr(s2, np.complex64, self.model_shape, "slowness"),
                  ptr(rho, np.complex64, self.model_shape, "density"), d, kind, int(bool(add)), int(checkpoint))
        return data


class Refl3DOp(_Base3D):
    """3D reflectivity Born (BornRefl's operator, ext_born_refl.cpp:8-105,
    one reflectivity for every frequency): forward records Up(r bg),
    adjoint is the migration image sum conj(bg) Up^H(data)."""

    _destroy = "refl3d_destroy"

    def __init__(self, q, wavelet, bg_s2):
        super().__init__(q, wavelet)
        _lib.call("refl3d_create", ctypes.byref(q), self.wavelet.ctypes.data_as(ctypes.c_void_p),
                  ptr(bg_s2, np.complex64, self.model_shape, "slowness"), ctypes.byref(self.h))

    def set_background(self, s2):
        _lib.call("refl3d_set_background", self.h, ptr(s2, np.complex64, self.model_shape, "slowness"))

    def forward(self, model, data, add=False, checkpoint=0):
        d, kind = self._data_ptr(data, True)
        _lib.call("refl3d_forward", self.h, ptr(model, np.complex64, self.model_shape, "model"), d, kind,
                  int(bool(add)), int(checkpoint))
        return data

    def adjoint(self, model, data, add=False):
        d, kind = self._data_ptr(data, False)
        _lib.call("refl3d_adjoint", self.h, ptr(model, np.complex64, self.model_shape, "model", True), d, kind,
                  int(bool(add)))
        return model


class BornTomoOp(_Base):
    """Frequency-extended tomographic Born (BornTomo,
    propagator/src/ext_born_tomo.cpp:9-119): model [nz][nx] is a slowness^2
    perturbation; the down- and up-scattering terms with the reflectivity per
    frequency of ``set_refl`` ([nfreq][nz][nx]) in place of R."""

    _destroy = "borntomo_destroy"

    def __init__(self, p: WemParams, wavelet, bg_s2):
        super().__init__(p, wavelet)
        _lib.call("borntomo_create", ctypes.byref(self.p), self.wavelet.ctypes.data_as(ctypes.c_void_p),
                  ptr(bg_s2, np.complex64, self.model_shape, "slowness"), ctypes.byref(self.h))

    def set_background(self, s2):
        _lib.call("borntomo_set_background", self.h, ptr(s2, np.complex64, self.model_shape, "slowness"))

    def set_refl(self, refl):
        _lib.call("borntomo_set_refl", self.h,
                  ptr(refl, np.complex64, (self.nfreq(), self.p.nz, self.p.nx), "reflectivity"))

    def forward(self, model, data, add=False):
        d, kind = self._data_ptr(data, True)
        _lib.call("borntomo_forward", self.h, ptr(model, np.complex64, self.model_shape, "model"), d, kind,
                  int(bool(add)))
        return data

    def adjoint(self, model, data, add=False):
        d, kind = self._data_ptr(data, False)
        _lib.call("borntomo_adjoint", self.h, ptr(model, np.complex64, self.model_shape, "model", True), d, kind,
                  int(bool(add)))
        return model


class ExtWemOp(WemOp):
    """Frequency-extended modelling (extWEM, propagator/src/extWEM.cpp:9-70)."""

    _destroy = "extwem_destroy"

    def __init__(self, p: WemParams, wavelet):
        _Base.__init__(self, p, wavelet)
        _lib.call("extwem_create", ctypes.byref(self.p), self.wavelet.ctypes.data_as(ctypes.c_void_p),
                  ctypes.byref(self.h))

    @property
    def model_shape(self):
        return (self.nfreq(), self.p.nz, self.p.nx)

    def forward(self, s2, rho, data, add=False):
        d, kind = self._data_ptr(data, True)
        _lib.call("extwem_forward", self.h, ptr(s2, np.complex64, self.model_shape, "slowness"),
                  ptr(rho, np.complex64, self.model_shape, "density"), d, kind, int(bool(add)))
        return data


class ExtBornOp(BornOp):
    """Frequency-extended Born operator (extBornFull, ext_born_prop.cpp:8-194)."""

    _destroy = "extborn_destroy"
    _prefix = "extborn"

    @property
    def model_shape(self):
        return (self.nfreq(), self.p.nz, self.p.nx)


class RowOps:
    """Row-level operators of one padded slowness grid [nz][nxg]
    (py_wem_ops: SSF/PSPI, Down/Up, Scatter, RefSampler)."""

    def __init__(self, p: WemParams, slow_padded):
        self.p = p.copy()
        self.nz, self.nxg = slow_padded.shape[-2], slow_padded.shape[-1]
        if self.nz != p.nz:
            raise ValueError("slowness depth axis does not match params.nz")
        self.h = ctypes.c_void_p()
        _lib.call("wemop_create", ctypes.byref(self.p), ptr(slow_padded, np.complex64, None, "slowness"),
                  self.nxg, ctypes.byref(self.h))

    def __del__(self):
        h = getattr(self, "h", None)
        if h and h.value:
            try:
                _lib.load().wemop_destroy(h)
            except Exception:
                pass

    def _rows(self, x, per_row):
        n = int(np.prod(x.shape)) if not _is_torch(x) else x.numel()
        if n % per_row:
            raise ValueError("input size is not a whole number of rows")
        return n // per_row

    def onestep(self, iz, freq, adj, x, out=None, add=False):
        out = _like(x) if out is None else out
        n = self._rows(x, self.nxg)
        _lib.call("wemop_onestep", self.h, int(iz), float(freq), int(adj), ptr(x, np.complex64), ptr(out, np.complex64),
                  n, int(bool(add)))
        return out

    def oneway(self, up, freq, adj, x, out=None, add=False):
        """``out is x`` (with add=True) is the drivers' in-place recursion."""
        out = _like(x) if out is None else out
        n = self._rows(x, self.nxg * self.nz)
        _lib.call("wemop_oneway", self.h, int(up), float(freq), int(adj), ptr(x, np.complex64),
                  ptr(out, np.complex64), n, int(bool(add)))
        return out

    def scatter(self, iz, freq, adj, x, out=None, add=False):
        out = _like(x) if out is None else out
        n = self._rows(x, self.nxg)
        _lib.call("wemop_scatter", self.h, int(iz), float(freq), int(adj), ptr(x, np.complex64),
                  ptr(out, np.complex64), n, int(bool(add)))
        return out

    def splitstep(self, iz, freq, sref, loc, adj, x, out=None, add=False):
        """SplitStep of depth iz on the points ``loc`` (wemop_splitstep)."""
        out = _like(x) if out is None else out
        n = self._rows(x, self.nxg)
        loc = np.ascontiguousarray(loc, dtype=np.int32).reshape(-1)
        _lib.call("wemop_splitstep", self.h, int(iz), float(freq), float(np.real(sref)), float(np.imag(sref)),
                  ctypes.c_void_p(loc.ctypes.data), int(loc.size), int(adj), ptr(x, np.complex64),
                  ptr(out, np.complex64, None, "out", True), n, int(bool(add)))
        return out

    def lindown(self, bg, freq, adj, x, out=None, add=False):
        """LinDown of one field [nz][nxg] around the background wavefield bg."""
        out = _like(x) if out is None else out
        shape = (self.nz, self.nxg)
        _lib.call("wemop_lindown", self.h, ptr(bg, np.complex64, shape, "bg"), float(freq), int(adj),
                  ptr(x, np.complex64, shape, "in"), ptr(out, np.complex64, shape, "out", True), int(bool(add)))
        return out

    def refsampler(self):
        sref = np.zeros((self.nz, self.p.nref), np.complex64)
        idx = np.zeros((self.nz, self.nxg), np.int32)
        _lib.call("wemop_refsampler", self.h, ptr(sref, np.complex64), ctypes.c_void_p(idx.ctypes.data))
        return sref, idx


def ic(bg, adj, x, out, add=False):
    """Imaging condition out (+)= bg x (adjoint conj(bg) x), element-wise."""
    n = int(np.prod(x.shape)) if not _is_torch(x) else x.numel()
    _lib.call("wem_ic", ptr(bg, np.complex64, tuple(x.shape), "bg"), n, int(adj), ptr(x, np.complex64),
              ptr(out, np.complex64, tuple(x.shape), "out", True), int(bool(add)))
    return out


def phshift(p: WemParams, dx, dz, freq, s, adj, x, out, add=False):
    """Phase shift of rows of wavenumber samples (wem_phshift)."""
    n = x.shape[-1]
    nrow = (int(np.prod(x.shape)) if not _is_torch(x) else x.numel()) // n
    _lib.call("wem_phshift", ctypes.byref(p), int(n), float(dx), float(dz), float(freq), float(np.real(s)),
              float(np.imag(s)), int(adj), ptr(x, np.complex64), ptr(out, np.complex64, tuple(x.shape), "out", True),
              nrow, int(bool(add)))
    return out


def inject(iz, ix, ng, tap, step, shot, adj, model, data, add=False):
    """Injection (wem_inject) between a model [nt] or [nshot][npt][nt] and
    rows data [nz][nx], complex: forward data (+)= the spread point
    values, adjoint model (+)= the gathered ones."""
    izs = np.ascontiguousarray(np.asarray(iz, dtype=np.int32).ravel())
    ixs = np.ascontiguousarray(np.asarray(ix, dtype=np.int32).ravel())
    if izs.size != ixs.size:
        raise ValueError("z and x lists differ in length")
    npt = int(izs.size)
    if len(model.shape) == 1:
        nshot, nt = 0, int(model.shape[0])
    elif len(model.shape) == 3:
        if int(model.shape[1]) != npt:
            raise ValueError(f"model has {model.shape[1]} points, the lists {npt}")
        nshot, nt = int(model.shape[0]), int(model.shape[2])
    else:
        raise ValueError("model must be [nt] or [nshot][npoints][nt]")
    nz, nx = int(data.shape[0]), int(data.shape[1])
    _lib.call("wem_inject", izs.ctypes.data_as(ctypes.c_void_p), ixs.ctypes.data_as(ctypes.c_void_p), npt, int(ng),
              int(tap), nx, nz, nt, nshot, int(step), int(shot), int(adj),
              ptr(model, np.complex64, tuple(model.shape), "model", bool(adj)),
              ptr(data, np.complex64, (nz, nx), "data", not adj), int(bool(add)))


def reflect(slow2, rho, adj, x, out):
    """Reflect of the grid (slow2, rho): out = r x (conj(r) x)."""
    nz, nx = slow2.shape[-2], slow2.shape[-1]
    shape = (nz, nx)
    _lib.call("wem_reflect", ptr(slow2, np.complex64, shape, "slowness"), ptr(rho, np.complex64, shape, "density"),
              nx, nz, int(adj), ptr(x, np.complex64, shape, "in"), ptr(out, np.complex64, shape, "out", True))
    return out


def dreflect(slow2, rho, adj, m0, m1, data, add=False):
    """dReflect at (slow2, rho): forward data (+)= dR(m0, m1), adjoint
    (m0, m1) (+)= dR^H data."""
    nz, nx = slow2.shape[-2], slow2.shape[-1]
    shape = (nz, nx)
    _lib.call("wem_dreflect", ptr(slow2, np.complex64, shape, "slowness"), ptr(rho, np.complex64, shape, "density"),
              nx, nz, int(adj), ptr(m0, np.complex64, shape, "dslowness", True),
              ptr(m1, np.complex64, shape, "ddensity", True), ptr(data, np.complex64, shape, "data", True),
              int(bool(add)))


class Interp2DOp:
    """Coarse-to-fine model interpolation (lanczos2d_* / spline2d_*): model
    complex ``[nm2][nm1]`` -> data complex ``[nd2][nd1]``.  ``m_axes`` and
    ``d_axes`` are ``((n1, d1), (n2, d2))``; ``kind`` is ``"lanczos"`` (``a`` =
    two half widths in coarse samples) or ``"spline"`` (``a``, ``b`` the cubic's
    parameters)."""

    def __init__(self, kind, m_axes, d_axes, a, b=0.0):
        (nm1, dm1), (nm2, dm2) = m_axes
        (nd1, dd1), (nd2, dd2) = d_axes
        self.model_shape = (int(nm2), int(nm1))
        self.data_shape = (int(nd2), int(nd1))
        self.h = ctypes.c_void_p()
        geo = (int(nm1), float(dm1), int(nm2), float(dm2), int(nd1), float(dd1), int(nd2), float(dd2))
        if kind == "lanczos":
            aa = (ctypes.c_float * 2)(float(a[0]), float(a[1]))
            _lib.call("lanczos2d_create", *geo, aa, ctypes.byref(self.h))
        elif kind == "spline":
            _lib.call("spline2d_create", *geo, float(a), float(b), ctypes.byref(self.h))
        else:
            raise ValueError(f"unknown interpolation {kind!r}")

    def __del__(self):
        h = getattr(self, "h", None)
        if h and h.value:
            try:
                _lib.load().interp2d_destroy(h)
            except Exception:
                pass

    def forward(self, model, data, add=False):
        _lib.call("interp2d_forward", self.h, ptr(model, np.complex64, self.model_shape, "model"),
                  ptr(data, np.complex64, self.data_shape, "data", True), int(bool(add)))

    def adjoint(self, model, data, add=False):
        _lib.call("interp2d_adjoint", self.h, ptr(model, np.complex64, self.model_shape, "model", True),
                  ptr(data, np.complex64, self.data_shape, "data"), int(bool(add)))


def _like(x):
    if _is_torch(x):
        return torch.zeros_like(x)
    return np.zeros_like(x)
