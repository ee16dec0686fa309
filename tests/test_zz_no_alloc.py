"""The depth step that allocates nothing, against the handle-based one.

wemop_onestep_noalloc serves callers that cannot allocate device memory
while they run (a fixed arena or pool, a loop that must not touch the
allocator): it takes the depth's inputs directly and keeps its tables in a
device array the library owns.  Its output must match wemop_onestep on the
same rows, within the 1e-5 single-step tolerance of the parity tests, and the
oracle's fp64 depth step within the same tolerance, on calls in a row: a row
of N = 4096 points (the limit) first, then smaller rows, so that a call after
a larger one shows nothing of what the larger one left in the shared array.
This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from cases import pad_edge, rand_c, rel_l2, small_case

pytestmark = pytest.mark.gpu

TOL_STEP = 1e-5

# (prop, nref, nx, tap, pad, phase_law, iz, freq, adj, add): the first row
# has N = nx + 2 pad + 2 tap = 4096
CASES = [
    ("pspi", 3, 4064, 12, 4, "exact_kz", 5, 7.5, 0, 1),
    ("ssf", 1, 4064, 12, 4, "ispc", 9, 11.0, 1, 0),
    ("pspi", 3, 52, 6, 4, "ispc", 7, 9.5, 0, 0),
    ("ssf", 1, 240, 0, 0, "exact_kz", 12, 6.0, 1, 1),
    ("ssf", 2, 52, 6, 4, "ispc", 3, 8.0, 1, 0),
]


def _dptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _noalloc(p, sp_row, sref_row, ref_row, freq, adj, x, out0, add):
    import torch
    from wemgpu import _lib
    dev = torch.device("cuda")
    ts = torch.from_numpy(np.ascontiguousarray(sp_row)).to(dev)
    tsr = torch.from_numpy(np.ascontiguousarray(sref_row)).to(dev)
    tri = torch.from_numpy(np.ascontiguousarray(ref_row.astype(np.int8))).to(dev)
    tx = torch.from_numpy(x).to(dev)
    to = torch.from_numpy(out0.copy()).to(dev)
    _lib.call("wemop_onestep_noalloc", ctypes.byref(p), _dptr(ts), _dptr(tsr), _dptr(tri), ts.numel(),
              ctypes.c_float(freq), adj, _dptr(tx), _dptr(to), x.shape[0], add, None)
    torch.cuda.synchronize()
    return to.cpu().numpy()


def test_onestep_noalloc_matches_handle_path(gpu_lib, oracle):
    from wemgpu.core import RowOps
    rng = np.random.default_rng(21)
    for prop, nref, nx, tap, pad, law, iz, freq, adj, add in CASES:
        p, par, wav, s, rho = small_case(prop=prop, nref=nref, nx=nx, tap=tap, pad=pad, phase_law=law)
        sp = pad_edge(s, p.pad)
        ops = RowOps(p, sp)
        sref, idx = ops.refsampler()
        x = rand_c(rng, (5, sp.shape[1]))
        out0 = rand_c(rng, x.shape) if add else np.zeros_like(x)
        want = ops.onestep(iz, freq, adj, x, out=out0.copy(), add=bool(add))
        o64 = oracle.onestep(p, sp, iz, freq, adj, x, out=out0.copy(), add=bool(add), prec=64)
        got = _noalloc(p, sp[iz], sref[iz], idx[iz], freq, adj, x, out0, add)
        case = (prop, nref, nx, law, adj, add)
        assert rel_l2(got, want) < TOL_STEP, (case, rel_l2(got, want))
        assert rel_l2(got, o64) < TOL_STEP, (case, rel_l2(got, o64))
        again = _noalloc(p, sp[iz], sref[iz], idx[iz], freq, adj, x, out0, add)
        assert np.array_equal(again, got), case


def test_onestep_noalloc_out_of_range_reference_is_none(gpu_lib):
    """refidx entries outside [-1, nref) count as -1: the point gets no
    reference, as a -1 entry of the reference's own partition."""
    p, par, wav, s, rho = small_case(prop="pspi", nref=3, nx=52)
    sp = pad_edge(s, p.pad)
    from wemgpu.core import RowOps
    ops = RowOps(p, sp)
    sref, idx = ops.refsampler()
    rng = np.random.default_rng(5)
    x = rand_c(rng, (2, sp.shape[1]))
    zeros = np.zeros_like(x)
    bad = idx[4].copy()
    bad[::5] = -1
    wild = bad.copy()
    wild[::5] = np.where(np.arange(wild[::5].size) % 2, 3, -7)  # 3 == nref, -7 < -1
    a = _noalloc(p, sp[4], sref[4], bad, 8.0, 0, x, zeros, 0)
    b = _noalloc(p, sp[4], sref[4], wild, 8.0, 0, x, rand_c(rng, x.shape), 0)
    assert np.array_equal(a, b)
    assert np.all(a[:, ::5] == 0)


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
