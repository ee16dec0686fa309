"""ORACLE — test infrastructure only.  numpy restatement of the model-space
interpolation operators of the FWI preconditioner; only tests/ import it,
as the checker of the library's ``lanczos2d_*`` / ``spline2d_*`` entry
points.

PARITY PINNED: the reference's own LanczosInterpolation2D.h / Spline2D.h
and lanczos_kernel.ispc, compiled by oracle/ref/Makefile, give the golden
outputs of tests/golden/refinterp.npz (tests/test_ref_pin.py, 1e-5); also
its dot test (Lanczos, and the spline before its edge copies), partition of
unity on the interior and exact reproduction of samples on coarse nodes.

Filters follow the reference's loops and arithmetic (float32 with the
Lanczos weights in float64, as the reference mixes them); the products are
evaluated in float64.
  LanczosInterpolation2D: operator/src/LanczosInterpolation2D.h:14-125
  Spline2D:               operator/src/Spline2D.h:14-130
"""
from __future__ import annotations

import numpy as np

f32 = np.float32


def lanczos_weight(x, dm, a):
    """Windowed sinc at offsets x != 0 (LanczosInterpolation2D.h:99-100)."""
    x = np.asarray(x, np.float64)
    return (np.float64(f32(dm) * f32(a)) * np.sin(np.pi * x / np.float64(f32(dm))) *
            np.sin(np.pi * x / np.float64(f32(a))) / (np.pi * np.pi * x * x)).astype(np.float32)


def lanczos_filter(nd, dd, nm, dm, a):
    """[nd][nm] filter of one axis; a = half width in the axis' units
    (LanczosInterpolation2D.h:91-121)."""
    dd, dm, a = f32(dd), f32(dm), f32(a)
    nf = int(f32(f32(f32(2) * a) / dd) + f32(1))
    na = (nf - 1) // 2
    half = f32(f32(na) * dd)
    i = np.arange(nd, dtype=np.float32)[:, None]
    j = np.arange(nm, dtype=np.float32)[None, :]
    x = (i * dd - j * dm).astype(np.float32)
    f = np.zeros((nd, nm), np.float32)
    inside = np.abs(x) <= half
    with np.errstate(divide="ignore", invalid="ignore"):
        w = lanczos_weight(x, dm, a)
    f[inside] = np.where(x[inside] == 0, f32(1), w[inside])
    for ii in range(min(na, nd)):
        for jj in range(nm):
            xv = f32(f32(ii) * dd - f32(jj) * dm)
            xx = f32(f32(ii) * dd + f32(jj) * dm)
            if abs(xx) < half and xv != xx:
                wv = lanczos_weight(xx, dm, a)
                f[ii, jj] = f32(f[ii, jj] + wv)
                f[nd - ii - 1, nm - jj - 1] = f32(f[nd - ii - 1, nm - jj - 1] + wv)
    return f


def spline_weight(y, a, b):
    """Two-parameter cubic at distance y in coarse samples (Spline2D.h:101-107)."""
    y = np.asarray(y, np.float32)
    a, b = f32(a), f32(b)
    c6 = f32(6)
    in1 = ((f32(-6) * a - f32(9) * b + f32(12)) * y * y * y + (f32(6) * a + f32(12) * b - f32(18)) * y * y
           - f32(2) * b + c6) / c6
    in2 = ((f32(-6) * a - b) * y * y * y + (f32(30) * a + f32(6) * b) * y * y + (f32(-48) * a - f32(12) * b) * y
           + f32(24) * a + f32(8) * b) / c6
    return np.where(y < 1, in1, np.where(y < 2, in2, f32(0))).astype(np.float32)


def spline_filter(nd, dd, nm, dm, a, b):
    """[nd][nm] filter of one axis (Spline2D.h:96-125)."""
    dd, dm = f32(dd), f32(dm)
    i = np.arange(nd, dtype=np.float32)[:, None]
    j = np.arange(nm, dtype=np.float32)[None, :]
    f = spline_weight(np.abs(i * dd - j * dm) / dm, a, b)
    for ii in range(nd):
        for jj in range(1, nm - 1):
            xx = f32(f32(ii) * dd + f32(jj) * dm)
            wv = spline_weight(abs(xx) / dm, a, b)
            f[ii, jj] = f32(f[ii, jj] + wv)
            f[nd - ii - 1, nm - jj - 1] = f32(f[nd - ii - 1, nm - jj - 1] + wv)
    return f


class Interp2D:
    """data [nd2][nd1] = F2 model [nm2][nm1] F1^T; m_axes / d_axes are
    ((n1, d1), (n2, d2)).  kind 'lanczos' (a = two half widths in coarse
    samples) or 'spline' (cubic parameters a, b)."""

    def __init__(self, kind, m_axes, d_axes, a, b=0.0):
        (nm1, dm1), (nm2, dm2) = m_axes
        (nd1, dd1), (nd2, dd2) = d_axes
        self.kind = kind
        if kind == "lanczos":
            # half widths in the axis' units (LanczosInterpolation2D.h:16-17)
            self.f1 = lanczos_filter(nd1, dd1, nm1, dm1, f32(a[0]) * f32(dm1))
            self.f2 = lanczos_filter(nd2, dd2, nm2, dm2, f32(a[1]) * f32(dm2))
        elif kind == "spline":
            self.f1 = spline_filter(nd1, dd1, nm1, dm1, a, b)
            self.f2 = spline_filter(nd2, dd2, nm2, dm2, a, b)
        else:
            raise ValueError(kind)

    def forward(self, model, data=None, add=False):
        f1, f2 = self.f1.astype(np.float64), self.f2.astype(np.float64)
        out = f2 @ (model.astype(np.complex128) @ f1.T)
        if add and data is not None:
            out = out + data.astype(np.complex128)
        return out

    def adjoint(self, data, model=None, add=False, edges=True):
        """``edges=False`` leaves out the spline's edge copies (the
        transpose proper)."""
        f1, f2 = self.f1.astype(np.float64), self.f2.astype(np.float64)
        out = (f2.T @ data.astype(np.complex128)) @ f1
        if add and model is not None:
            out = out + model.astype(np.complex128)
        if self.kind == "spline" and edges:
            # Spline2D.h:84-92: columns first, then rows
            out[:, 0] = out[:, 1]
            out[:, -1] = out[:, -2]
            out[0, :] = out[1, :]
            out[-1, :] = out[-2, :]
        return out
