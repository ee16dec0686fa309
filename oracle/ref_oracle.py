"""REFERENCE RUN — test infrastructure only.

ctypes front end of ``oracle/_ref/libwemref.so``: the reference's own
propagator sources (propagator/src, operator/src FFT1_c/FFT1_r/Taper,
conformal/src, complex/SRC) compiled unchanged by ``oracle/ref/Makefile``
against the stand-ins of ``oracle/ref/stubs`` (serial TBB, an FFTW front end
over a double-precision DFT, minimal SEP vectors).  It exists only where the
reference checkout exists (this library is built from it); tests that use it
skip elsewhere, and the golden fixtures of ``tests/golden`` carry its outputs
to machines without it.

Every function takes the reference's own parameter dictionary (the keys its
``paramObj`` reads: ns, osx, dsx, osz, nr, orx, drx, orz, prop, nref, tap,
pad, tpad, eps, fmin, fmax, nfreq, ntaylor) and the model grid and wavelet
axes, builds the operator the way ``propagator/src/python/WEM.py:36-130``
does, and returns numpy arrays in the library's layouts: models [nz][nx]
(frequency-extended [nf][nz][nx]) complex64, data [ns][nr][nt] float32.
"""
from __future__ import annotations

import atexit
import ctypes
import json
import os
import shutil
import subprocess
import tempfile

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_ref", "libwemref.so")
REF_DEFAULT = "/root/reference"
_lib = None

# keys of the library's parameter block that the reference does not read;
# only their reference behaviour may be asked for
_OWN_KEYS = {"adjoint_mode": "compat", "refs_mode": "ascoded", "phase_law": "ispc", "nbin": 0}


def ref_root() -> str:
    return os.environ.get("WEM_REFERENCE", REF_DEFAULT)


def available() -> bool:
    """The reference checkout is present (so the library can be built)."""
    return os.path.isdir(os.path.join(ref_root(), "propagator", "src"))


def build() -> str:
    subprocess.run(["make", "-s", "-j8", "-C", os.path.join(_HERE, "ref"), f"REF={ref_root()}"], check=True)
    return _LIB


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(_LIB)
        _lib.ref_last_error.restype = ctypes.c_char_p
    return _lib


_TMP = None


def _json_file(obj) -> str:
    """A JSON file the reference reads by path (its "coord" geometry file,
    Device.h:65-85, and the "cmap_angles" file, PropParam.h:119-129)."""
    global _TMP
    if _TMP is None:
        _TMP = tempfile.mkdtemp(prefix="wemref_")
        atexit.register(shutil.rmtree, _TMP, True)
    fd, path = tempfile.mkstemp(suffix=".json", dir=_TMP)
    with os.fdopen(fd, "w") as f:
        json.dump(obj, f)
    return path


def _kv(par: dict) -> bytes:
    """The reference's parameters as "key=value;..."; coordinate lists (sx,
    sz, rx, rz) and rotation angles go into the JSON files it reads."""
    items = []
    coords = {}
    for k, v in par.items():
        if k in _OWN_KEYS:
            if str(v).lower() != str(_OWN_KEYS[k]):
                raise ValueError(f"the reference has no {k}={v!r} (it behaves as {k}={_OWN_KEYS[k]!r})")
            continue
        if k in ("sx", "sz", "rx", "rz"):
            coords[k] = [float(x) for x in np.asarray(v, np.float64).ravel()]
            continue
        if k == "cmap_angles" and not isinstance(v, str):
            v = _json_file({"a": [float(x) for x in np.asarray(v, np.float64).ravel()]})
        if isinstance(v, (list, tuple, np.ndarray)):
            raise ValueError(f"{k}: lists are not reference parameters")
        items.append(f"{k}={int(v) if isinstance(v, bool) else v}")
    if coords:
        items.append(f"coord={_json_file(coords)}")
    return ";".join(items).encode()


def _call(name, *args):
    rc = getattr(lib(), name)(*args)
    if rc != 0:
        raise RuntimeError(f"{name}: {lib().ref_last_error().decode()}")


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _c64(a):
    return np.ascontiguousarray(a, dtype=np.complex64)


class Grid:
    """Model and time axes: nx, nz, dx, dz (origins ox, oz) and nt, dt (ot)."""

    def __init__(self, nx, nz, dx, dz, nt, dt, ox=0.0, oz=0.0, ot=0.0):
        self.nx, self.nz, self.dx, self.dz = int(nx), int(nz), float(dx), float(dz)
        self.ox, self.oz = float(ox), float(oz)
        self.nt, self.dt, self.ot = int(nt), float(dt), float(ot)

    def head(self, par, wavelet):
        w = np.ascontiguousarray(wavelet, np.float32)
        assert w.size == self.nt
        return [_kv(par), ctypes.c_int(self.nt), ctypes.c_float(self.ot), ctypes.c_float(self.dt), _p(w),
                ctypes.c_int(self.nx), ctypes.c_int(self.nz), ctypes.c_float(self.ox), ctypes.c_float(self.oz),
                ctypes.c_float(self.dx), ctypes.c_float(self.dz)], w


def _counts(par):
    ns = len(par["sx"]) if "sx" in par else int(par["ns"])
    nr = len(par["rx"]) if "rx" in par else int(par["nr"])
    return ns, nr


def nfreq(par, g: Grid, wavelet) -> int:
    h, _w = g.head(par, wavelet)
    n = ctypes.c_int()
    _call("ref_nfreq", *h, ctypes.byref(n))
    return n.value


def wem_forward(par, g: Grid, wavelet, s2, rho):
    ns, nr = _counts(par)
    h, _w = g.head(par, wavelet)
    s2, rho = _c64(s2), _c64(rho)
    out = np.zeros((ns, nr, g.nt), np.float32)
    _call("ref_wem_forward", *h, _p(s2), _p(rho), ns, nr, _p(out))
    return out


def born_forward(par, g: Grid, wavelet, bs2, brho, ds2, drho):
    ns, nr = _counts(par)
    h, _w = g.head(par, wavelet)
    a = [_c64(x) for x in (bs2, brho, ds2, drho)]
    out = np.zeros((ns, nr, g.nt), np.float32)
    _call("ref_born_forward", *h, *[_p(x) for x in a], ns, nr, _p(out))
    return out


def born_adjoint(par, g: Grid, wavelet, bs2, brho, data):
    ns, nr = _counts(par)
    h, _w = g.head(par, wavelet)
    bs2, brho = _c64(bs2), _c64(brho)
    d = np.ascontiguousarray(data, np.float32)
    gs = np.zeros((g.nz, g.nx), np.complex64)
    gr = np.zeros((g.nz, g.nx), np.complex64)
    _call("ref_born_adjoint", *h, _p(bs2), _p(brho), _p(d), ns, nr, _p(gs), _p(gr))
    return gs, gr


def bornrefl_forward(par, g: Grid, wavelet, bs2, refl):
    ns, nr = _counts(par)
    h, _w = g.head(par, wavelet)
    r = _c64(refl).copy()
    out = np.zeros((ns, nr, g.nt), np.float32)
    _call("ref_bornrefl", h[0], 0, *h[1:], _p(_c64(bs2)), r.shape[0], _p(r), ns, nr, _p(out))
    return out


def bornrefl_adjoint(par, g: Grid, wavelet, bs2, data, nf):
    ns, nr = _counts(par)
    h, _w = g.head(par, wavelet)
    r = np.zeros((nf, g.nz, g.nx), np.complex64)
    d = np.ascontiguousarray(data, np.float32)
    _call("ref_bornrefl", h[0], 1, *h[1:], _p(_c64(bs2)), nf, _p(r), ns, nr, _p(d))
    return r


def borntomo_forward(par, g: Grid, wavelet, bs2, refl, ds2):
    ns, nr = _counts(par)
    h, _w = g.head(par, wavelet)
    refl = _c64(refl)
    m = _c64(ds2).copy()
    out = np.zeros((ns, nr, g.nt), np.float32)
    _call("ref_borntomo", h[0], 0, *h[1:], _p(_c64(bs2)), refl.shape[0], _p(refl), _p(m), ns, nr, _p(out))
    return out


def borntomo_adjoint(par, g: Grid, wavelet, bs2, refl, data):
    ns, nr = _counts(par)
    h, _w = g.head(par, wavelet)
    refl = _c64(refl)
    m = np.zeros((g.nz, g.nx), np.complex64)
    d = np.ascontiguousarray(data, np.float32)
    _call("ref_borntomo", h[0], 1, *h[1:], _p(_c64(bs2)), refl.shape[0], _p(refl), _p(m), ns, nr, _p(d))
    return m


def extwem_forward(par, g: Grid, wavelet, s2, rho):
    ns, nr = _counts(par)
    h, _w = g.head(par, wavelet)
    s2, rho = _c64(s2), _c64(rho)
    out = np.zeros((ns, nr, g.nt), np.float32)
    _call("ref_extwem_forward", *h, s2.shape[0], _p(s2), _p(rho), ns, nr, _p(out))
    return out


def extborn_forward(par, g: Grid, wavelet, bs2, brho, ds2, drho):
    ns, nr = _counts(par)
    h, _w = g.head(par, wavelet)
    bs2, brho = _c64(bs2), _c64(brho)
    ds2, drho = _c64(ds2).copy(), _c64(drho).copy()
    out = np.zeros((ns, nr, g.nt), np.float32)
    _call("ref_extborn", h[0], 0, *h[1:], bs2.shape[0], _p(bs2), _p(brho), _p(ds2), _p(drho), ns, nr, _p(out))
    return out


def extborn_adjoint(par, g: Grid, wavelet, bs2, brho, data):
    ns, nr = _counts(par)
    h, _w = g.head(par, wavelet)
    bs2, brho = _c64(bs2), _c64(brho)
    nf = bs2.shape[0]
    ds2 = np.zeros((nf, g.nz, g.nx), np.complex64)
    drho = np.zeros((nf, g.nz, g.nx), np.complex64)
    d = np.ascontiguousarray(data, np.float32)
    _call("ref_extborn", h[0], 1, *h[1:], nf, _p(bs2), _p(brho), _p(ds2), _p(drho), ns, nr, _p(d))
    return ds2, drho


def interp2d(kind, model_axes, data_axes, p0, p1, x, adj=False):
    """LanczosInterpolation2D ("lanczos": p0, p1 the half widths in coarse
    cells) or Spline2D ("spline": p0, p1 = a, b) from the coarse grid
    model_axes = ((n1, d1), (n2, d2)) to the fine grid data_axes; forward
    maps a model [n2][n1] to data, adjoint the reverse."""
    (mn1, md1), (mn2, md2) = model_axes
    (dn1, dd1), (dn2, dd2) = data_axes
    m = np.zeros((mn2, mn1), np.complex64)
    d = np.zeros((dn2, dn1), np.complex64)
    if adj:
        d[:] = x
    else:
        m[:] = x
    _call("ref_interp2d", 0 if kind == "lanczos" else 1, int(adj), mn1, ctypes.c_float(md1), mn2,
          ctypes.c_float(md2), dn1, ctypes.c_float(dd1), dn2, ctypes.c_float(dd2), ctypes.c_float(p0),
          ctypes.c_float(p1), _p(m), _p(d))
    return m if adj else d


def inject(iz, ix, ng, tap, nz, nx, step, shot, x, adj=False, nt=None, nshot=0):
    """Injection (propagator/src/Injection.cpp:8-33, 52-75): forward maps a
    model [nt] (nshot = 0) or [nshot][npt][nt] to rows [nz][nx], adjoint the
    reverse (nt, nshot: the model's sizes, needed for the adjoint)."""
    izs = np.ascontiguousarray(np.asarray(iz, np.int32))
    ixs = np.ascontiguousarray(np.asarray(ix, np.int32))
    npt = int(izs.size)
    if adj:
        d = _c64(x)
        m = np.zeros((nshot, npt, nt) if nshot else (nt,), np.complex64)
    else:
        m = _c64(x)
        nt = int(m.shape[-1])
        nshot = int(m.shape[0]) if m.ndim == 3 else 0
        d = np.zeros((nz, nx), np.complex64)
    _call("ref_inject", _p(izs), _p(ixs), npt, int(ng), int(tap), int(nx), int(nz), int(nt), int(nshot), int(step),
          int(shot), int(adj), _p(m), _p(d))
    return m if adj else d
