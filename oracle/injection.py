"""ORACLE — test infrastructure only.  numpy restatement of the reference's
point Injection operator (propagator/src/Injection.h:19-65,
Injection.cpp:8-33, 52-75); only tests/ import it, as the checker of the
library's ``wem_inject`` entry point.

PARITY PINNED: the reference's own Injection class, compiled by
oracle/ref/Makefile (``ref_inject``), against this restatement in
tests/test_wem_ops.py, and the golden outputs of tests/golden/refinject.npz.

The cos^2 window is computed in float32 as Injection.h:53-65 does; the
spread values are summed in float32 in the reference's loop order.
"""
from __future__ import annotations

import numpy as np

f32 = np.float32


def window(ng):
    """Injection.h:53-65: (1 - cos(pi i / ng)) / 2 rising, (cos(...) + 1) / 2
    falling, in float32 (pi = 4 atan(1) rounded to float)."""
    sz = 2 * ng + 1
    g = np.ones(sz, np.float32)
    if ng == 0:
        return g
    pi = f32(4 * np.arctan(1.0))
    step = f32(pi / f32(ng))
    for i in range(sz // 2):
        g[i] = (-np.cos(f32(step * f32(i)), dtype=np.float32) + f32(1)) / f32(2)
    for i in range(sz // 2, sz):
        g[i] = (np.cos(f32(step * f32(i - sz + ng + 1)), dtype=np.float32) + f32(1)) / f32(2)
    return g


def forward(iz, ix, ng, tap, nz, nx, step, shot, model):
    """model [nt] (Injection.cpp:8-19: every point takes model[step]) or
    [nshot][npt][nt] (52-62: point i takes model[shot][i][step]) to rows
    [nz][nx]."""
    g = window(ng)
    d = np.zeros((nz, nx), np.complex64)
    m = np.asarray(model, np.complex64)
    for i in range(len(ix)):
        v = m[step] if m.ndim == 1 else m[shot, i, step]
        for ig in range(-ng, ng + 1):
            off = ix[i] + ig + tap
            if 0 <= off < nx:
                d[iz[i], off] += np.complex64(g[ig + ng] * v)
    return d


def adjoint(iz, ix, ng, tap, nz, nx, step, shot, data, nt, nshot=0):
    """The transpose: rows [nz][nx] to a model [nt] or [nshot][npt][nt]
    cleared elsewhere (Injection.cpp:21-33, 64-75)."""
    g = window(ng)
    npt = len(ix)
    m = np.zeros((nshot, npt, nt) if nshot else (nt,), np.complex64)
    d = np.asarray(data, np.complex64)
    for i in range(npt):
        for ig in range(-ng, ng + 1):
            off = ix[i] + ig + tap
            if 0 <= off < nx:
                v = np.complex64(g[ig + ng] * d[iz[i], off])
                if nshot:
                    m[shot, i, step] += v
                else:
                    m[step] += v
    return m
