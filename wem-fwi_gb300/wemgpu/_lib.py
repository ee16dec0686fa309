"""ctypes binding of ``libwemgpu.so`` (the C ABI in include/wemgpu.h).

The library is the only compute path: importing a compute entry point
without it raises, there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

from .params import WemParams

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libwemgpu.so")

_lib = None

_h = ctypes.c_void_p
_v = ctypes.c_void_p
_i = ctypes.c_int
_f = ctypes.c_float
_pp = ctypes.POINTER(WemParams)

_SIGS = {
    "wem_params_default": (None, [_pp]),
    "wem_count_freqs": (_i, [_pp, _v, ctypes.POINTER(_i)]),
    "wem_last_error": (ctypes.c_char_p, []),
    "wem_version": (ctypes.c_char_p, []),
    "wem_stats_enable": (_i, [_i]),
    "wem_stats_get": (_i, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_longlong)]),
    "wem_stats_reset": (_i, []),
    "wem_launch_count": (ctypes.c_longlong, []),
    "wem_set_plain": (_i, [_i]),
    "wem_set_kernel_path": (_i, [_i]),
    "wem_set_row_ctas": (_i, [_i]),
    "wem_set_gradient_split": (_i, [_i]),
    "wem_create": (_i, [_pp, _v, ctypes.POINTER(_h)]),
    "wem_destroy": (None, [_h]),
    "wem_get_nfreq": (_i, [_h, ctypes.POINTER(_i)]),
    "wem_forward": (_i, [_h, _v, _v, _v, _i, _i]),
    "born_create": (_i, [_pp, _v, _v, _v, ctypes.POINTER(_h)]),
    "born_destroy": (None, [_h]),
    "born_set_background": (_i, [_h, _v, _v]),
    "born_forward": (_i, [_h, _v, _v, _v, _i, _i]),
    "born_adjoint": (_i, [_h, _v, _v, _v, _i, _i]),
    "extwem_create": (_i, [_pp, _v, ctypes.POINTER(_h)]),
    "extwem_destroy": (None, [_h]),
    "extwem_forward": (_i, [_h, _v, _v, _v, _i, _i]),
    "extborn_create": (_i, [_pp, _v, _v, _v, ctypes.POINTER(_h)]),
    "extborn_destroy": (None, [_h]),
    "extborn_set_background": (_i, [_h, _v, _v]),
    "extborn_forward": (_i, [_h, _v, _v, _v, _i, _i]),
    "extborn_adjoint": (_i, [_h, _v, _v, _v, _i, _i]),
    "bornrefl_create": (_i, [_pp, _v, _v, ctypes.POINTER(_h)]),
    "bornrefl_destroy": (None, [_h]),
    "bornrefl_set_background": (_i, [_h, _v]),
    "bornrefl_forward": (_i, [_h, _v, _v, _i, _i]),
    "bornrefl_adjoint": (_i, [_h, _v, _v, _i, _i]),
    "bornoff_create": (_i, [_pp, _v, _v, _i, _v, _v, ctypes.POINTER(_h)]),
    "bornoff_destroy": (None, [_h]),
    "bornoff_set_background": (_i, [_h, _v]),
    "bornoff_forward": (_i, [_h, _v, _v, _i, _i]),
    "bornoff_adjoint": (_i, [_h, _v, _v, _i, _i]),
    "bornoff_rows": (_i, [_h, _v, _v]),
    "wem3d_create": (_i, [_v, _v, ctypes.POINTER(_h)]),
    "wem3d_destroy": (None, [_h]),
    "wem3d_get_nfreq": (_i, [_h, ctypes.POINTER(_i)]),
    "wem3d_forward": (_i, [_h, _v, _v, _v, _i, _i, _i]),
    "refl3d_create": (_i, [_v, _v, _v, ctypes.POINTER(_h)]),
    "refl3d_destroy": (None, [_h]),
    "refl3d_set_background": (_i, [_h, _v]),
    "refl3d_forward": (_i, [_h, _v, _v, _i, _i, _i]),
    "refl3d_adjoint": (_i, [_h, _v, _v, _i, _i]),
    "borntomo_create": (_i, [_pp, _v, _v, ctypes.POINTER(_h)]),
    "borntomo_destroy": (None, [_h]),
    "borntomo_set_background": (_i, [_h, _v]),
    "borntomo_set_refl": (_i, [_h, _v]),
    "borntomo_forward": (_i, [_h, _v, _v, _i, _i]),
    "borntomo_adjoint": (_i, [_h, _v, _v, _i, _i]),
    "fwi_create": (_i, [_pp, _v, ctypes.POINTER(_h)]),
    "fwi_destroy": (None, [_h]),
    "fwi_gradient": (_i, [_h, _v, _v, _v, _v, _v, ctypes.POINTER(ctypes.c_double)]),
    "fwi_gradient_exact": (_i, [_h, _v, _v, _v, _v, _v, ctypes.POINTER(ctypes.c_double), _i]),
    "wem_gradient": (_i, [_h, _v, _v, _v, _i, _v, _v, _i, _i]),
    "wemop_create": (_i, [_pp, _v, _i, ctypes.POINTER(_h)]),
    "wemop_destroy": (None, [_h]),
    "wemop_onestep": (_i, [_h, _i, _f, _i, _v, _v, _i, _i]),
    "wemop_oneway": (_i, [_h, _i, _f, _i, _v, _v, _i, _i]),
    "wemop_scatter": (_i, [_h, _i, _f, _i, _v, _v, _i, _i]),
    "wemop_refsampler": (_i, [_h, _v, _v]),
    "wemop_onestep_noalloc": (_i, [_pp, _v, _v, _v, _i, _f, _i, _v, _v, _i, _i, _v]),
    "wemop_splitstep": (_i, [_h, _i, _f, _f, _f, _v, _i, _i, _v, _v, _i, _i]),
    "wemop_lindown": (_i, [_h, _v, _f, _i, _v, _v, _i]),
    "wem_ic": (_i, [_v, _i, _i, _v, _v, _i]),
    "wem_phshift": (_i, [_pp, _i, _f, _f, _f, _f, _f, _i, _v, _v, _i, _i]),
    "wem_reflect": (_i, [_v, _v, _i, _i, _i, _v, _v]),
    "wem_inject": (_i, [_v, _v, _i, _i, _i, _i, _i, _i, _i, _i, _i, _i, _v, _v, _i]),
    "wem_dreflect": (_i, [_v, _v, _i, _i, _i, _v, _v, _v, _i]),
    "lanczos2d_create": (_i, [_i, _f, _i, _f, _i, _f, _i, _f, ctypes.POINTER(_f), ctypes.POINTER(_h)]),
    "spline2d_create": (_i, [_i, _f, _i, _f, _i, _f, _i, _f, _f, _f, ctypes.POINTER(_h)]),
    "interp2d_destroy": (None, [_h]),
    "interp2d_forward": (_i, [_h, _v, _v, _i]),
    "interp2d_adjoint": (_i, [_h, _v, _v, _i]),
}

EXPORTED = tuple(_SIGS)


def load(path: str = LIB_PATH):
    """Load (once) and type the library.  Raises when it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build the CUDA library first (python -c 'import wemgpu; wemgpu.build()')")
    lib = ctypes.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class WemError(RuntimeError):
    """A non-zero status of the C ABI, with the library's message."""

    def __init__(self, fn: str, code: int, msg: str):
        super().__init__(f"{fn}: {msg} (status {code})")
        self.code = code


def kernel_stats(name: str):
    """(total ms, launches) of one pass kernel since the last reset."""
    ms, n = ctypes.c_double(), ctypes.c_longlong()
    call("wem_stats_get", name.encode(), ctypes.byref(ms), ctypes.byref(n))
    return ms.value, n.value


def launch_count() -> int:
    """Kernel launches the library has made in this process."""
    return int(load().wem_launch_count())


def call(name: str, *args) -> None:
    lib = load()
    rc = getattr(lib, name)(*args)
    if rc != 0:
        raise WemError(name, rc, lib.wem_last_error().decode(errors="replace"))
