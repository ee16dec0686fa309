"""wemgpu — GB300-native one-way wave-equation operators.

Drop-in for the hot path of arustam92/wem-fwi: the SSF/PSPI depth step and
the nonlinear (WEM) and Born operators built on it, with the reference's
Python API (``WEM``, ``Born``, ``extWEM``, ``extBorn``) over a C ABI
(include/wemgpu.h) whose kernels are hand-written CUDA for sm_103a.
"""
from .build import build  # noqa: F401
from .params import (  # noqa: F401
    WEM_ADJ_COMPAT, WEM_ADJ_EXACT, WEM_DATA_FREQ, WEM_DATA_TIME, WEM_PROP_PSPI, WEM_PROP_SSF,
    WEM_REFS_ASCODED, WEM_REFS_NEAREST, WemParams, make_params,
)
from .vector import Axis, Hypercube, SuperVector, Vector, getSepVector, superVector  # noqa: F401


def __getattr__(name):
    # operator classes load the CUDA library on first use
    if name in ("WEM", "Born", "extWEM", "extBorn", "BornRefl", "BornTomo", "BornOffset", "Propagator",
                "LanczosInterpolation2D", "Spline", "Spline2D"):
        from . import ops
        return getattr(ops, name)
    if name in ("WemOp", "BornOp", "ExtWemOp", "ExtBornOp", "BornReflOp", "BornTomoOp", "BornOffsetOp", "RowOps",
                "FwiOp", "Wem3DOp", "Refl3DOp",
                "Interp2DOp"):
        from . import core
        return getattr(core, name)
    raise AttributeError(name)
