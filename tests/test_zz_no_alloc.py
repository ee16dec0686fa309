"""The depth step that allocates nothing, against the handle-based one.

wemop_onestep_noalloc serves callers that cannot allocate device memory
while they run (a fixed arena or pool, a loop that must not touch the
allocator): it takes the depth's inputs directly and keeps its tables in a
device array the library owns.  Its output must match wemop_onestep on the
same rows, within the 1e-5 single-step tolerance of the parity tests, on
two calls in a row (the second call overwrites what the first left in the
shared array).  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from cases import pad_edge, rand_c, rel_l2, small_case

pytestmark = pytest.mark.gpu


def _dptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _noalloc(p, sp_row, sref_row, ref_row, freq, adj, x):
    import torch
    from wemgpu import _lib
    dev = torch.device("cuda")
    ts = torch.from_numpy(np.ascontiguousarray(sp_row)).to(dev)
    tsr = torch.from_numpy(np.ascontiguousarray(sref_row)).to(dev)
    tri = torch.from_numpy(np.ascontiguousarray(ref_row.astype(np.int8))).to(dev)
    tx = torch.from_numpy(x).to(dev)
    to = torch.zeros_like(tx)
    _lib.call("wemop_onestep_noalloc", ctypes.byref(p), _dptr(ts), _dptr(tsr), _dptr(tri), ts.numel(),
              ctypes.c_float(freq), adj, _dptr(tx), _dptr(to), x.shape[0], 0, None)
    torch.cuda.synchronize()
    return to.cpu().numpy()


def test_onestep_noalloc_matches_handle_path(gpu_lib):
    from wemgpu.core import RowOps
    rng = np.random.default_rng(21)
    # two calls in a row with different sizes, propagators and depths
    for prop, nref, nx, iz, freq, adj in (("pspi", 3, 52, 7, 9.5, 0), ("ssf", 1, 240, 12, 6.0, 1)):
        p, par, wav, s, rho = small_case(prop=prop, nref=nref, nx=nx)
        sp = pad_edge(s, p.pad)
        ops = RowOps(p, sp)
        sref, idx = ops.refsampler()
        x = rand_c(rng, (5, sp.shape[1]))
        want = ops.onestep(iz, freq, adj, x)
        got = _noalloc(p, sp[iz], sref[iz], idx[iz], freq, adj, x)
        assert rel_l2(got, want) < 1e-5, (prop, rel_l2(got, want))
        again = _noalloc(p, sp[iz], sref[iz], idx[iz], freq, adj, x)
        assert np.array_equal(again, got)


def test_onestep_noalloc_rejects_oversize_and_host_memory(gpu_lib):
    import torch
    from wemgpu import _lib
    from wemgpu._lib import WemError
    p, par, wav, s, rho = small_case(nx=52)
    dev = torch.device("cuda")
    big = 5000
    ts = torch.zeros(big, dtype=torch.complex64, device=dev)
    tsr = torch.ones(1, dtype=torch.complex64, device=dev)
    tri = torch.zeros(big, dtype=torch.int8, device=dev)
    tx = torch.zeros((1, big), dtype=torch.complex64, device=dev)
    with pytest.raises(WemError) as e:
        _lib.call("wemop_onestep_noalloc", ctypes.byref(p), _dptr(ts), _dptr(tsr), _dptr(tri), big,
                  ctypes.c_float(5.0), 0, _dptr(tx), _dptr(tx), 1, 0, None)
    assert e.value.code == 1 and "4096" in str(e.value)
    h = np.zeros(64, np.complex64)
    with pytest.raises(WemError) as e:
        _lib.call("wemop_onestep_noalloc", ctypes.byref(p), ctypes.c_void_p(h.ctypes.data), _dptr(tsr),
                  _dptr(tri), 64, ctypes.c_float(5.0), 0, _dptr(tx), _dptr(tx), 1, 0, None)
    assert e.value.code == 1 and "device memory" in str(e.value)
