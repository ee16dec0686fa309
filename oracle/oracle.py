"""ORACLE — test infrastructure only.  ctypes front end of the CPU
restatement in ``wem_oracle.cpp``; only tests/, ``__graft_entry__.smoke()``
and bench.py's CPU-baseline leg import it, as the checker.

PARITY PINNED: the restatement is held to the outputs of the reference's
own sources (compiled by oracle/ref/Makefile against stand-ins for its
external libraries; golden fixtures tests/golden/ref_*.npz, checked by
tests/test_ref_pin.py), besides the reference's known-answer test (extWEM ==
WEM on a frequency-constant model), dot tests, its fp64 twin and numpy.fft.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_ROOT = os.path.dirname(_HERE)
sys.path.insert(0, os.path.join(_ROOT, "wem-fwi_gb300"))
from wemgpu.params import WemParams, WEM_DATA_TIME, WEM_DATA_FREQ  # noqa: E402

_LIB = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None


def build(force: bool = False) -> str:
    """Compile the restatement with g++ (no external libraries)."""
    # make rebuilds only what changed
    if force or _lib is None:
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(_LIB)
        _lib.oracle_last_error.restype = ctypes.c_char_p
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _call(name, *args):
    rc = getattr(lib(), name)(*args)
    if rc != 0:
        raise RuntimeError(f"{name}: {lib().oracle_last_error().decode()} (status {rc})")


def _c64(a):
    return np.ascontiguousarray(a, dtype=np.complex64)


def count_freqs(p: WemParams):
    n = ctypes.c_int()
    _call("oracle_count_freqs", ctypes.byref(p), ctypes.byref(n), None, None)
    bins = np.zeros(n.value, np.int32)
    freqs = np.zeros(n.value, np.float32)
    _call("oracle_count_freqs", ctypes.byref(p), ctypes.byref(n), _ptr(bins), _ptr(freqs))
    return n.value, bins, freqs


def devices(p: WemParams):
    sx, sz = np.zeros(p.ns, np.int32), np.zeros(p.ns, np.int32)
    rx, rz = np.zeros(p.nr, np.int32), np.zeros(p.nr, np.int32)
    _call("oracle_devices", ctypes.byref(p), _ptr(sx), _ptr(sz), _ptr(rx), _ptr(rz))
    return sx, sz, rx, rz


def fft(x, sign=-1):
    """Unnormalised DFT in double precision (sign -1 forward)."""
    v = np.ascontiguousarray(x, dtype=np.complex128).copy()
    _call("oracle_fft", ctypes.c_int(v.size), _ptr(v), ctypes.c_int(sign))
    return v


def _nbin(p):
    return p.nbin if p.nbin else p.nt + p.tpad


def _data_out(p, kind, data=None):
    if data is not None:
        return data
    if kind == WEM_DATA_TIME:
        return np.zeros((p.ns, p.nr, p.nt), np.float32)
    return np.zeros((p.ns, p.nr, _nbin(p)), np.complex64)


def wem_forward(p, wavelet, s2, rho, kind=WEM_DATA_FREQ, data=None, add=False, prec=32, nthreads=0):
    out = _data_out(p, kind, data)
    _call("oracle_wem_forward", ctypes.byref(p), _ptr(np.ascontiguousarray(wavelet, np.float32)),
          _ptr(_c64(s2)), _ptr(_c64(rho)), _ptr(out), kind, int(add), prec, nthreads)
    return out


def born_forward(p, wavelet, bs2, brho, ds2, drho, kind=WEM_DATA_FREQ, data=None, add=False,
                 prec=32, nthreads=0):
    out = _data_out(p, kind, data)
    _call("oracle_born_forward", ctypes.byref(p), _ptr(np.ascontiguousarray(wavelet, np.float32)),
          _ptr(_c64(bs2)), _ptr(_c64(brho)), _ptr(_c64(ds2)), _ptr(_c64(drho)), _ptr(out),
          kind, int(add), prec, nthreads)
    return out


def born_adjoint(p, wavelet, bs2, brho, data, kind=WEM_DATA_FREQ, ds2=None, drho=None, add=False,
                 prec=32, nthreads=0, fchunks=1):
    shape = (p.nz, p.nx)
    ds2 = np.zeros(shape, np.complex64) if ds2 is None else ds2
    drho = np.zeros(shape, np.complex64) if drho is None else drho
    d = np.ascontiguousarray(data, np.float32 if kind == WEM_DATA_TIME else np.complex64)
    _call("oracle_born_adjoint", ctypes.byref(p), _ptr(np.ascontiguousarray(wavelet, np.float32)),
          _ptr(_c64(bs2)), _ptr(_c64(brho)), _ptr(ds2), _ptr(drho), _ptr(d), kind, int(add), prec,
          nthreads, fchunks)
    return ds2, drho


def extwem_forward(p, wavelet, s2, rho, kind=WEM_DATA_FREQ, data=None, add=False, prec=32, nthreads=0):
    out = _data_out(p, kind, data)
    _call("oracle_extwem_forward", ctypes.byref(p), _ptr(np.ascontiguousarray(wavelet, np.float32)),
          _ptr(_c64(s2)), _ptr(_c64(rho)), _ptr(out), kind, int(add), prec, nthreads)
    return out


def extborn_forward(p, wavelet, bs2, brho, ds2, drho, kind=WEM_DATA_FREQ, data=None, add=False,
                    prec=32, nthreads=0):
    out = _data_out(p, kind, data)
    _call("oracle_extborn_forward", ctypes.byref(p), _ptr(np.ascontiguousarray(wavelet, np.float32)),
          _ptr(_c64(bs2)), _ptr(_c64(brho)), _ptr(_c64(ds2)), _ptr(_c64(drho)), _ptr(out),
          kind, int(add), prec, nthreads)
    return out


def extborn_adjoint(p, wavelet, bs2, brho, data, kind=WEM_DATA_FREQ, add=False, prec=32, nthreads=0):
    nf = count_freqs(p)[0]
    ds2 = np.zeros((nf, p.nz, p.nx), np.complex64)
    drho = np.zeros((nf, p.nz, p.nx), np.complex64)
    d = np.ascontiguousarray(data, np.float32 if kind == WEM_DATA_TIME else np.complex64)
    _call("oracle_extborn_adjoint", ctypes.byref(p), _ptr(np.ascontiguousarray(wavelet, np.float32)),
          _ptr(_c64(bs2)), _ptr(_c64(brho)), _ptr(ds2), _ptr(drho), _ptr(d), kind, int(add), prec,
          nthreads)
    return ds2, drho


def bornrefl_forward(p, wavelet, bs2, model, kind=WEM_DATA_TIME, data=None, add=False, prec=32, nthreads=0):
    """BornRefl (ext_born_refl.cpp:8-57): model [nfreq][nz][nx] reflectivity per frequency."""
    out = _data_out(p, kind, data)
    _call("oracle_bornrefl_forward", ctypes.byref(p), _ptr(np.ascontiguousarray(wavelet, np.float32)),
          _ptr(_c64(bs2)), _ptr(_c64(model)), _ptr(out), kind, int(add), prec, nthreads)
    return out


def bornrefl_adjoint(p, wavelet, bs2, data, kind=WEM_DATA_TIME, add=False, prec=32, nthreads=0):
    nf = count_freqs(p)[0]
    model = np.zeros((nf, p.nz, p.nx), np.complex64)
    d = np.ascontiguousarray(data, np.float32 if kind == WEM_DATA_TIME else np.complex64)
    _call("oracle_bornrefl_adjoint", ctypes.byref(p), _ptr(np.ascontiguousarray(wavelet, np.float32)),
          _ptr(_c64(bs2)), _ptr(model), _ptr(d), kind, int(add), prec, nthreads)
    return model


def _apertures(p, apertures, taps):
    ap = np.ascontiguousarray(np.asarray(apertures, dtype=np.int32).reshape(p.ns, 2))
    x0, w = np.ascontiguousarray(ap[:, 0]), np.ascontiguousarray(ap[:, 1])
    return x0, w, np.ascontiguousarray(np.asarray(taps, dtype=np.int32).reshape(p.ns))


def offborn_forward(p, wavelet, bs2, model, apertures, taps, kind=WEM_DATA_TIME, data=None, add=False, prec=32,
                    nthreads=0):
    """Subsurface-offset extended reflectivity Born (no reference counterpart):
    model [nh][nz][nx]; shot s on the aperture (x0, w) = apertures[s] with
    the row's leading zero pad taps[s]."""
    out = _data_out(p, kind, data)
    m = _c64(model)
    x0, w, t = _apertures(p, apertures, taps)
    _call("oracle_offborn_forward", ctypes.byref(p), _ptr(np.ascontiguousarray(wavelet, np.float32)),
          _ptr(_c64(bs2)), m.shape[0], _ptr(x0), _ptr(w), _ptr(t), _ptr(m), _ptr(out), kind, int(add), prec,
          nthreads)
    return out


def offborn_adjoint(p, wavelet, bs2, nh, data, apertures, taps, kind=WEM_DATA_TIME, add=False, prec=32,
                    nthreads=0):
    model = np.zeros((nh, p.nz, p.nx), np.complex64)
    d = np.ascontiguousarray(data, np.float32 if kind == WEM_DATA_TIME else np.complex64)
    x0, w, t = _apertures(p, apertures, taps)
    _call("oracle_offborn_adjoint", ctypes.byref(p), _ptr(np.ascontiguousarray(wavelet, np.float32)),
          _ptr(_c64(bs2)), nh, _ptr(x0), _ptr(w), _ptr(t), _ptr(model), _ptr(d), kind, int(add), prec, nthreads)
    return model


def borntomo_forward(p, wavelet, bs2, refl, dm, kind=WEM_DATA_TIME, data=None, add=False, prec=32, nthreads=0):
    """BornTomo (ext_born_tomo.cpp:9-57): dm [nz][nx], refl [nfreq][nz][nx]."""
    out = _data_out(p, kind, data)
    _call("oracle_borntomo_forward", ctypes.byref(p), _ptr(np.ascontiguousarray(wavelet, np.float32)),
          _ptr(_c64(bs2)), _ptr(_c64(refl)), _ptr(_c64(dm)), _ptr(out), kind, int(add), prec, nthreads)
    return out


def borntomo_adjoint(p, wavelet, bs2, refl, data, kind=WEM_DATA_TIME, add=False, prec=32, nthreads=0):
    dm = np.zeros((p.nz, p.nx), np.complex64)
    d = np.ascontiguousarray(data, np.float32 if kind == WEM_DATA_TIME else np.complex64)
    _call("oracle_borntomo_adjoint", ctypes.byref(p), _ptr(np.ascontiguousarray(wavelet, np.float32)),
          _ptr(_c64(bs2)), _ptr(_c64(refl)), _ptr(dm), _ptr(d), kind, int(add), prec, nthreads)
    return dm


def onestep(p, slow_padded, iz, freq, adj, x, out=None, add=False, prec=32):
    x = _c64(x)
    nxg = slow_padded.shape[-1]
    out = np.zeros_like(x) if out is None else out
    _call("oracle_onestep", ctypes.byref(p), _ptr(_c64(slow_padded)), nxg, iz, ctypes.c_float(freq),
          int(adj), _ptr(x), _ptr(out), x.size // nxg, int(add), prec)
    return out


def oneway(p, slow_padded, up, freq, adj, x, out=None, add=False, prec=32):
    """out=None with add=True means the in-place recursion (model is data)."""
    nxg = slow_padded.shape[-1]
    x = _c64(x)
    if out is None and add:
        out = x
    elif out is None:
        out = np.zeros_like(x)
    nrow = x.size // (nxg * p.nz)
    _call("oracle_oneway", ctypes.byref(p), _ptr(_c64(slow_padded)), nxg, int(up), ctypes.c_float(freq),
          int(adj), _ptr(x), _ptr(out), nrow, int(add), prec)
    return out


def scatter(p, slow_padded, iz, freq, adj, x, out=None, add=False, prec=32):
    x = _c64(x)
    nxg = slow_padded.shape[-1]
    out = np.zeros_like(x) if out is None else out
    _call("oracle_scatter", ctypes.byref(p), _ptr(_c64(slow_padded)), nxg, iz, ctypes.c_float(freq),
          int(adj), _ptr(x), _ptr(out), x.size // nxg, int(add), prec)
    return out


def refsampler(p, slow_padded):
    nxg = slow_padded.shape[-1]
    sref = np.zeros((p.nz, p.nref), np.complex64)
    idx = np.zeros((p.nz, nxg), np.int32)
    _call("oracle_refsampler", ctypes.byref(p), _ptr(_c64(slow_padded)), nxg, _ptr(sref), _ptr(idx))
    return sref, idx


def phshift(p, n, dx, dz, freq, s, adj, x, out=None, add=False, prec=32):
    """Phshift of rows of n wavenumber samples (Phshift_cmplx.cpp:47-113)."""
    x = _c64(x)
    out = np.zeros_like(x) if out is None else out
    _call("oracle_phshift", ctypes.byref(p), int(n), ctypes.c_float(dx), ctypes.c_float(dz), ctypes.c_float(freq),
          ctypes.c_float(np.real(s)), ctypes.c_float(np.imag(s)), int(adj), _ptr(x), _ptr(out), x.size // n,
          int(add), prec)
    return out


def splitstep(p, slow, iz, freq, sref, loc, adj, x, out=None, add=False, prec=32):
    """SplitStep of depth iz on the points loc (SplitStep.cpp:5-29)."""
    x = _c64(x)
    nxg = slow.shape[-1]
    out = np.zeros_like(x) if out is None else out
    loc = np.ascontiguousarray(loc, dtype=np.int32)
    _call("oracle_splitstep", ctypes.byref(p), _ptr(_c64(slow)), nxg, int(iz), ctypes.c_float(freq),
          ctypes.c_float(np.real(sref)), ctypes.c_float(np.imag(sref)), _ptr(loc), loc.size, int(adj), _ptr(x),
          _ptr(out), x.size // nxg, int(add), prec)
    return out


def lindown(p, slow, bg, freq, adj, x, out=None, add=False, prec=32):
    """LinDown of one field (LinOneWay.cpp:33-85)."""
    x = _c64(x)
    nxg = slow.shape[-1]
    out = np.zeros_like(x) if out is None else out
    _call("oracle_lindown", ctypes.byref(p), _ptr(_c64(slow)), nxg, _ptr(_c64(bg)), ctypes.c_float(freq), int(adj),
          _ptr(x), _ptr(out), int(add), prec)
    return out


def reflect(slow, rho, adj, x):
    """Reflect (Reflect.h:12-48), in double."""
    x = _c64(x)
    out = np.zeros_like(x)
    nz, nx = slow.shape
    _call("oracle_reflect", _ptr(_c64(slow)), _ptr(_c64(rho)), nx, nz, int(adj), _ptr(x), _ptr(out))
    return out


def dreflect(slow, rho, adj, m0=None, m1=None, data=None, add=False):
    """dReflect (dReflect.h:11-84), in double: forward returns data, adjoint
    (m0, m1)."""
    nz, nx = slow.shape
    m0 = np.zeros(slow.shape, np.complex64) if m0 is None else _c64(m0).copy()
    m1 = np.zeros(slow.shape, np.complex64) if m1 is None else _c64(m1).copy()
    data = np.zeros(slow.shape, np.complex64) if data is None else _c64(data).copy()
    _call("oracle_dreflect", _ptr(_c64(slow)), _ptr(_c64(rho)), nx, nz, int(adj), _ptr(m0), _ptr(m1), _ptr(data),
          int(add))
    return (m0, m1) if adj else data
