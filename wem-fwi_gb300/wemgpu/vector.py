"""Vector types with the reference's interface.

The reference's operators take SEP vectors (``SepVector.getSepVector(
Hypercube.hypercube(ns=..., ds=..., os=...), storage='dataComplex')``) and a
python-solver ``superVector`` of ``[slowness^2, density]``
(propagator/test/test_wem_ops.py:50-57).  Those libraries are not available
here, so this module provides the part of their interface the operators and
tests use: ``getNdArray``, ``getHyper().getAxis(i)``, ``clone``, ``zero``,
``set``, ``rand``, ``scale``, ``dot``, ``norm`` and ``superVector.vecs``.

Axis 1 is the fastest axis, so ``ns=[nx, nz]`` gives an array of shape
``(nz, nx)``.  Storage is a numpy array or a torch tensor (host or CUDA);
the operators pass CUDA tensors to the library without copies.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Sequence

import numpy as np

try:  # torch is optional for the numpy path
    import torch
except Exception:  # pragma: no cover
    torch = None


@dataclass
class Axis:
    n: int
    d: float = 1.0
    o: float = 0.0


class Hypercube:
    def __init__(self, ns: Sequence[int] = None, ds: Sequence[float] = None, os: Sequence[float] = None,
                 axes: Sequence[Axis] = None):
        if axes is None:
            ns = list(ns)
            ds = list(ds) if ds is not None else [1.0] * len(ns)
            os = list(os) if os is not None else [0.0] * len(ns)
            axes = [Axis(int(n), float(d), float(o)) for n, d, o in zip(ns, ds, os)]
        self.axes: List[Axis] = list(axes)

    def getAxis(self, i: int) -> Axis:  # 1-based, as SEP hypercubes
        return self.axes[i - 1]

    def getNdim(self) -> int:
        return len(self.axes)

    @property
    def shape(self):
        return tuple(a.n for a in reversed(self.axes))

    def __eq__(self, other):
        return isinstance(other, Hypercube) and [(a.n, a.d, a.o) for a in self.axes] == \
            [(a.n, a.d, a.o) for a in other.axes]


def _is_torch(a) -> bool:
    return torch is not None and isinstance(a, torch.Tensor)


class Vector:
    """One regular-grid vector; ``arr`` is numpy or torch, C-contiguous."""

    def __init__(self, hyper: Hypercube, arr=None, storage: str = "dataFloat"):
        self.hyper = hyper
        if arr is None:
            dt = np.complex64 if storage == "dataComplex" else np.float32
            arr = np.zeros(hyper.shape, dtype=dt)
        if tuple(arr.shape) != hyper.shape:
            raise ValueError(f"array shape {tuple(arr.shape)} does not match hypercube {hyper.shape}")
        self.arr = arr

    # ---- SepVector surface
    def getNdArray(self):
        return self.arr

    def getHyper(self) -> Hypercube:
        return self.hyper

    @property
    def is_complex(self) -> bool:
        return self.arr.dtype in (np.complex64, np.complex128) or (
            _is_torch(self.arr) and self.arr.is_complex())

    def clone(self) -> "Vector":
        return Vector(self.hyper, self.arr.clone() if _is_torch(self.arr) else self.arr.copy())

    def cloneSpace(self) -> "Vector":
        v = self.clone()
        v.zero()
        return v

    def zero(self) -> "Vector":
        self.arr[...] = 0
        return self

    def set(self, val) -> "Vector":
        self.arr[...] = val
        return self

    def scale(self, s) -> "Vector":
        self.arr *= s
        return self

    def rand(self, seed=None) -> "Vector":
        """Uniform in (-.5, .5), real and imaginary parts (complexHyper.cc:43-53)."""
        rng = np.random.default_rng(seed)
        shape = self.hyper.shape
        vals = rng.random(shape) - .5
        if self.is_complex:
            vals = vals + 1j * (rng.random(shape) - .5)
        if _is_torch(self.arr):
            self.arr.copy_(torch.from_numpy(vals.astype(np.complex64 if self.is_complex else np.float32)))
        else:
            self.arr[...] = vals
        return self

    def dot(self, other: "Vector") -> float:
        """Re sum(self * conj(other)) accumulated in double (complexHyper.cc:69-81)."""
        a, b = _np(self.arr), _np(other.arr)
        return float(np.vdot(b.astype(np.complex128), a.astype(np.complex128)).real)

    def norm(self) -> float:
        return float(np.sqrt(self.dot(self)))


class SuperVector:
    """python-solver superVector: an ordered list of vectors."""

    def __init__(self, *vecs):
        if len(vecs) == 1 and isinstance(vecs[0], (list, tuple)):
            vecs = tuple(vecs[0])
        self.vecs: List[Vector] = list(vecs)

    def __getitem__(self, i) -> Vector:
        return self.vecs[i]

    def __len__(self):
        return len(self.vecs)

    def __iter__(self):
        return iter(self.vecs)

    def clone(self) -> "SuperVector":
        return SuperVector(*[v.clone() for v in self.vecs])

    def zero(self) -> "SuperVector":
        for v in self.vecs:
            v.zero()
        return self

    def rand(self, seed=None) -> "SuperVector":
        for i, v in enumerate(self.vecs):
            v.rand(None if seed is None else seed + i)
        return self

    def scale(self, s) -> "SuperVector":
        for v in self.vecs:
            v.scale(s)
        return self

    def dot(self, other: "SuperVector") -> float:
        return sum(a.dot(b) for a, b in zip(self.vecs, other.vecs))

    def norm(self) -> float:
        return float(np.sqrt(self.dot(self)))


superVector = SuperVector


def _np(a):
    if _is_torch(a):
        return a.detach().cpu().numpy()
    return np.asarray(a)


def getSepVector(hyper: Hypercube = None, ns=None, ds=None, os=None, storage: str = "dataFloat") -> Vector:
    """Same call shape as ``SepVector.getSepVector``."""
    if hyper is None:
        hyper = Hypercube(ns=ns, ds=ds, os=os)
    return Vector(hyper, storage=storage)
