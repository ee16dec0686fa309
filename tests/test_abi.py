"""The C-ABI library builds, loads and exports what include/wemgpu.h
declares; host-side validation works without a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    import wemgpu
    wemgpu.build()
    from wemgpu import _lib
    return _lib.load()


def _declared():
    src = open(os.path.join(ROOT, "include", "wemgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b([a-z_][a-z0-9_]*)\s*\(", src)) - {"if", "sizeof", "for", "while"})


def test_exports_every_declared_symbol(lib):
    names = _declared()
    assert "wem_forward" in names and "born_adjoint" in names
    for n in names:
        assert hasattr(lib, n), n
    from wemgpu._lib import EXPORTED
    assert set(EXPORTED) == set(names)


def test_params_default_and_count(lib, oracle):
    from wemgpu.params import WemParams, make_params
    p = WemParams()
    lib.wem_params_default(ctypes.byref(p))
    assert p.nref == 1 and p.ntaylor == 1 and abs(p.eps - 0.04) < 1e-7 and p.fmin == 1.0
    q = make_params(dict(ns=1, nr=1, drx=10, fmin=2, fmax=20), nx=8, nz=4, dx=10, dz=10, nt=876, dt=0.004)
    n = ctypes.c_int()
    assert lib.wem_count_freqs(ctypes.byref(q), None, ctypes.byref(n)) == 0
    assert n.value == oracle.count_freqs(q)[0] == 64


@pytest.mark.parametrize("bad", [dict(nx=0), dict(pad=1), dict(nref=0), dict(ntaylor=7)])
def test_invalid_parameters_are_rejected_on_host(lib, bad):
    from wemgpu.params import make_params
    from wemgpu._lib import WemError, call
    kw = dict(nx=16, nz=8, dx=10.0, dz=10.0, nt=64, dt=0.004)
    par = dict(ns=1, osx=50, nr=4, drx=10, fmin=5, fmax=10)
    for k in ("pad", "nref", "ntaylor"):
        if k in bad:
            par[k] = bad[k]
    if "nx" in bad:
        kw["nx"] = bad["nx"]
    p = make_params(par, **kw)
    wav = np.zeros(64, np.float32)
    h = ctypes.c_void_p()
    with pytest.raises(WemError) as e:
        call("wem_create", ctypes.byref(p), wav.ctypes.data_as(ctypes.c_void_p), ctypes.byref(h))
    assert e.value.code == 1  # WEM_EINVAL, before any device call


@pytest.mark.parametrize("fn,bad", [("wem_set_kernel_path", 3), ("wem_set_row_ctas", 3), ("wem_set_row_ctas", -1),
                                    ("wem_set_gradient_split", 2), ("wem_set_gradient_split", -1)])
def test_launch_shape_knobs_validate_on_host(lib, fn, bad):
    from wemgpu._lib import WemError, call
    with pytest.raises(WemError) as e:
        call(fn, bad)
    assert e.value.code == 1  # WEM_EINVAL
    call(fn, 1 if fn == "wem_set_gradient_split" else 0)  # the default is always accepted


@pytest.mark.parametrize("bad", ["depth", "step", "shot", "window"])
def test_injection_arguments_validate_on_host(lib, bad):
    """wem_inject rejects a point below the rows (the reference would write
    outside them), a time sample or shot outside the model and a negative
    window before any device work."""
    from wemgpu._lib import WemError, call
    iz = np.array([0, 9 if bad == "depth" else 2], np.int32)
    ix = np.array([1, 3], np.int32)
    nz, nx, nt, nshot = 4, 8, 5, 2
    step = nt if bad == "step" else 1
    shot = nshot if bad == "shot" else 0
    ng = -1 if bad == "window" else 1
    m = np.zeros((nshot, 2, nt), np.complex64)
    d = np.zeros((nz, nx), np.complex64)
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    with pytest.raises(WemError) as e:
        call("wem_inject", p(iz), p(ix), 2, ng, 0, nx, nz, nt, nshot, step, shot, 0, p(m), p(d), 0)
    assert e.value.code == 1  # WEM_EINVAL
