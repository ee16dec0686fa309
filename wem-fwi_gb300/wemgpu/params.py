"""Parameter block of the C ABI (include/wemgpu.h ``wem_params``).

The reference reads its operator parameters from a SEP ``paramObj`` filled
from a JSON/dict (``genericIO.pythonParams``, scripts/fwi.py:33-35) and takes
the grid from the model's hypercube.  :func:`make_params` accepts the same
keys (``ns, osx, dsx, osz, nr, orx, drx, orz, prop, nref, tap, pad, tpad, eps,
fmin, fmax, nfreq, ngs, ngr, ntaylor``) plus the grid and wavelet axes, with
the defaults the reference's ``getInt/getFloat`` calls use.
"""
from __future__ import annotations

import ctypes
import json
from typing import Any, Mapping

import numpy as np

WEM_OK, WEM_EINVAL, WEM_ENOMEM, WEM_EDEVICE, WEM_ETIMEOUT, WEM_ENOTIMPL = range(6)
WEM_PROP_SSF, WEM_PROP_PSPI = 0, 1
WEM_ADJ_COMPAT, WEM_ADJ_EXACT = 0, 1
WEM_REFS_ASCODED, WEM_REFS_NEAREST = 0, 1
WEM_DATA_TIME, WEM_DATA_FREQ = 0, 1
WEM_PHASE_ISPC, WEM_PHASE_EXACT_KZ = 0, 1

_fp = ctypes.POINTER(ctypes.c_float)


class WemParams(ctypes.Structure):
    """ctypes mirror of ``struct wem_params``; field order is the ABI."""

    _fields_ = [
        ("nx", ctypes.c_int), ("nz", ctypes.c_int),
        ("ox", ctypes.c_float), ("oz", ctypes.c_float),
        ("dx", ctypes.c_float), ("dz", ctypes.c_float),
        ("nt", ctypes.c_int), ("ot", ctypes.c_float), ("dt", ctypes.c_float),
        ("ns", ctypes.c_int), ("osx", ctypes.c_float), ("osz", ctypes.c_float),
        ("dsx", ctypes.c_float), ("dsz", ctypes.c_float),
        ("nr", ctypes.c_int), ("orx", ctypes.c_float), ("orz", ctypes.c_float),
        ("drx", ctypes.c_float), ("drz", ctypes.c_float),
        ("src_x", _fp), ("src_z", _fp), ("rec_x", _fp), ("rec_z", _fp),
        ("prop", ctypes.c_int), ("nref", ctypes.c_int), ("tap", ctypes.c_int),
        ("pad", ctypes.c_int), ("tpad", ctypes.c_int),
        ("ngs", ctypes.c_int), ("ngr", ctypes.c_int), ("ntaylor", ctypes.c_int),
        ("eps", ctypes.c_float), ("fmin", ctypes.c_float), ("fmax", ctypes.c_float),
        ("nfreq", ctypes.c_int),
        ("adjoint_mode", ctypes.c_int), ("refs_mode", ctypes.c_int), ("nbin", ctypes.c_int),
        ("phase_law", ctypes.c_int),
        ("cmap", ctypes.c_int), ("eps_log", ctypes.c_float), ("cmap_angles", _fp),
    ]

    def __init__(self, *a, **kw):
        super().__init__(*a, **kw)
        self._keep: list = []  # keeps coordinate arrays alive

    def copy(self) -> "WemParams":
        c = WemParams()
        ctypes.pointer(c)[0] = self
        c._keep = list(self._keep)
        return c

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, t in self._fields_ if t is not _fp}


_DEFAULTS = dict(
    ox=0.0, oz=0.0, ot=0.0,
    ns=0, osx=0.0, osz=0.0, dsx=0.0, dsz=0.0,
    nr=0, orx=0.0, orz=0.0, drx=0.0, drz=0.0,
    prop="ssf", nref=1, tap=0, pad=0, tpad=0, ngs=0, ngr=0, ntaylor=1,
    eps=0.04, fmin=1.0, fmax=0.0, nfreq=0,
    adjoint_mode="compat", refs_mode="ascoded", nbin=0, phase_law="ispc",
    cmap=0, eps_log=0.01,
)


def _as_mapping(par: Any) -> Mapping:
    if par is None:
        return {}
    if isinstance(par, Mapping):
        return par
    if hasattr(par, "pars"):  # genericIO.pythonParams
        return par.pars
    raise TypeError("par must be a dict or an object with a .pars dict")


def make_params(par: Any, *, nx: int, nz: int, dx: float, dz: float,
                nt: int, dt: float, ox: float = 0.0, oz: float = 0.0,
                ot: float = 0.0) -> WemParams:
    """Build the ABI parameter block from reference-style keys."""
    m = dict(_DEFAULTS)
    m.update({k: v for k, v in _as_mapping(par).items()})
    p = WemParams()
    p.nx, p.nz, p.dx, p.dz = int(nx), int(nz), float(dx), float(dz)
    given = _as_mapping(par)
    p.ox = float(given["ox"]) if "ox" in given else float(ox)
    p.oz = float(given["oz"]) if "oz" in given else float(oz)
    p.nt, p.dt, p.ot = int(nt), float(dt), float(ot)
    for k in ("ns", "nr", "nref", "tap", "pad", "tpad", "ngs", "ngr", "ntaylor", "nfreq", "nbin", "cmap"):
        setattr(p, k, int(m[k]))
    for k in ("osx", "osz", "dsx", "dsz", "orx", "orz", "drx", "drz", "eps", "fmin", "fmax", "eps_log"):
        setattr(p, k, float(m[k]))
    prop = m["prop"]
    p.prop = WEM_PROP_PSPI if str(prop).lower() == "pspi" or prop == WEM_PROP_PSPI else WEM_PROP_SSF
    am = m["adjoint_mode"]
    p.adjoint_mode = WEM_ADJ_EXACT if str(am).lower() == "exact" or am == WEM_ADJ_EXACT else WEM_ADJ_COMPAT
    rm = m["refs_mode"]
    p.refs_mode = WEM_REFS_NEAREST if str(rm).lower() == "nearest" or rm == WEM_REFS_NEAREST else WEM_REFS_ASCODED
    pl = m["phase_law"]
    p.phase_law = WEM_PHASE_EXACT_KZ if str(pl).lower() == "exact_kz" or pl == WEM_PHASE_EXACT_KZ else WEM_PHASE_ISPC
    # irregular geometry: explicit coordinate lists, or the JSON file named by
    # "coord" (keys sx, sz, rx, rz; Device.h:65-85), replace the regular grid
    if m.get("coord"):
        with open(m["coord"]) as f:
            coords = json.load(f)
        for key in ("sx", "sz", "rx", "rz"):
            if key in coords and key not in m:
                m[key] = coords[key]
    for key, field, count in (("sx", "src_x", "ns"), ("sz", "src_z", "ns"),
                              ("rx", "rec_x", "nr"), ("rz", "rec_z", "nr")):
        if key in m and m[key] is not None:
            arr = np.ascontiguousarray(np.asarray(m[key], dtype=np.float32))
            if count == "ns":
                p.ns = int(arr.size)
            else:
                p.nr = int(arr.size)
            p._keep.append(arr)
            setattr(p, field, arr.ctypes.data_as(_fp))
    # rotation angles of cmap = 2: a list, or the JSON file named by
    # "cmap_angles" with key "a" (PropParam.h:119-129)
    ang = m.get("cmap_angles")
    if ang is not None:
        if isinstance(ang, str):
            with open(ang) as f:
                ang = json.load(f)["a"]
        arr = np.ascontiguousarray(np.asarray(ang, dtype=np.float32)).reshape(-1)
        if p.cmap == 2 and arr.size < p.ns:
            raise ValueError(f"cmap_angles holds {arr.size} angles for {p.ns} shots")
        p._keep.append(arr)
        p.cmap_angles = arr.ctypes.data_as(_fp)
    return p


class WemParams3D(ctypes.Structure):
    """ctypes mirror of ``struct wem3d_params`` (3D operators)."""

    _fields_ = [("p", WemParams), ("ny", ctypes.c_int), ("oy", ctypes.c_float), ("dy", ctypes.c_float),
                ("pad_y", ctypes.c_int), ("tap_y", ctypes.c_int), ("src_y", _fp), ("rec_y", _fp)]

    def __init__(self, *a, **kw):
        super().__init__(*a, **kw)
        self._keep: list = []

    @property
    def ns(self):
        return self.p.ns

    @property
    def nr(self):
        return self.p.nr


def make_params3d(par: Any, *, nx: int, ny: int, nz: int, dx: float, dy: float, dz: float, nt: int, dt: float,
                  sx, sy, sz, rx, ry, rz, ox: float = 0.0, oy: float = 0.0, oz: float = 0.0,
                  pad_y: int = 0, tap_y: int = 0) -> WemParams3D:
    """3D parameter block: the 2D keys of :func:`make_params` for the x, z and
    time axes and the propagation, the y axis, and explicit device
    coordinates (x, y, z per source and per receiver)."""
    m = dict(_as_mapping(par))
    m.update(sx=list(sx), sz=list(sz), rx=list(rx), rz=list(rz))
    q = WemParams3D()
    base = make_params(m, nx=nx, nz=nz, dx=dx, dz=dz, nt=nt, dt=dt, ox=ox, oz=oz)
    q.p = base  # a field copy: the coordinate arrays stay alive in q._keep
    q._keep.extend(base._keep)
    q.ny, q.oy, q.dy, q.pad_y, q.tap_y = int(ny), float(oy), float(dy), int(pad_y), int(tap_y)
    ys = np.ascontiguousarray(np.asarray(sy, dtype=np.float32))
    yr = np.ascontiguousarray(np.asarray(ry, dtype=np.float32))
    if ys.size != q.p.ns or yr.size != q.p.nr:
        raise ValueError("sy / ry must give one y per source / receiver")
    q._keep.extend([ys, yr])
    q.src_y = ys.ctypes.data_as(_fp)
    q.rec_y = yr.ctypes.data_as(_fp)
    return q
