"""Seeded synthetic problems shared by the CPU and GPU tests.

Shapes and parameters follow the reference's own test setup
(propagator/test/test_wem_ops.py:13-85) scaled down so the CPU oracle runs
in seconds, plus smooth random models like the benchmark configurations.
"""
import numpy as np

from wemgpu.params import make_params


def ricker(nt, dt, f0, t0=None):
    t = np.arange(nt) * dt - (t0 if t0 is not None else 1.0 / f0)
    a = (np.pi * f0 * t) ** 2
    return ((1 - 2 * a) * np.exp(-a)).astype(np.float32)


def smooth_noise(rng, shape, sigma):
    from scipy.ndimage import gaussian_filter
    return gaussian_filter(rng.uniform(-1, 1, shape), sigma)


def layered_model(nz, nx, seed=0, v0=1500.0, v1=3500.0, noise=0.05, sigma=4, q=1e-9):
    rng = np.random.default_rng(seed)
    v = v0 + (v1 - v0) * np.linspace(0, 1, nz)[:, None] * np.ones((1, nx))
    n = smooth_noise(rng, (nz, nx), sigma)
    n /= max(np.abs(n).max(), 1e-12)
    v = v * (1 + noise * n)
    s = (1.0 / v ** 2 - 1j * q).astype(np.complex64)
    rho = (1 + 0.2 * smooth_noise(rng, (nz, nx), sigma)).astype(np.complex64)
    return s, rho


def small_case(prop="ssf", nref=1, nx=52, nz=24, ns=3, tap=6, pad=4, ntaylor=1, adjoint_mode="compat",
               seed=0, nt=128, dt=0.008, fmin=6.0, fmax=14.0, ngs=2, ngr=1, eps=0.04, phase_law="ispc"):
    s, rho = layered_model(nz, nx, seed)
    par = dict(ns=ns, osx=10.0 * (nx // (ns + 1)), dsx=10.0 * (nx // (ns + 1)), osz=0.0,
               nr=nx, orx=0.0, drx=10.0, orz=0.0, eps=eps, prop=prop, nref=nref, tap=tap, pad=pad,
               fmin=fmin, fmax=fmax, ngs=ngs, ngr=ngr, ntaylor=ntaylor, adjoint_mode=adjoint_mode,
               phase_law=phase_law)
    p = make_params(par, nx=nx, nz=nz, dx=10.0, dz=10.0, nt=nt, dt=dt)
    wav = ricker(nt, dt, 10.0)
    return p, par, wav, s, rho


def rand_c(rng, shape):
    return ((rng.random(shape) - .5) + 1j * (rng.random(shape) - .5)).astype(np.complex64)


def pad_edge(a, pad):
    if pad == 0:
        return a.copy()
    return np.concatenate([np.repeat(a[..., :1], pad, -1), a, np.repeat(a[..., -1:], pad, -1)], -1)


def rel_l2(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def cmap_case(cmap, nx=64, nz=32, ns=3, nr=24, tap=0, pad=0, prop="ssf", nref=1, adjoint_mode="compat",
              angles=None, eps_log=0.01, seed=1, ngs=0, ngr=1, nt=128, dt=0.008, fmin=6.0, fmax=14.0):
    """Conformal-map problem (PropParam.h:88-137): grid spacing 12.5 m from
    the origin (so coordinates convert to grid cells exactly), sources
    inside the model, receivers along the surface."""
    s, rho = layered_model(nz, nx, seed)
    d = 12.5
    sx = [d * (nx * (k + 1) // (ns + 1)) for k in range(ns)]
    sz = [d * (nz // 2 + (k % 2) * 3) for k in range(ns)]
    rx = [d * (1 + (nx - 3) * k // max(nr - 1, 1)) for k in range(nr)]
    rz = [0.0] * nr
    par = dict(sx=sx, sz=sz, rx=rx, rz=rz, prop=prop, nref=nref, tap=tap, pad=pad, fmin=fmin, fmax=fmax,
               ngs=ngs, ngr=ngr, adjoint_mode=adjoint_mode, cmap=cmap, eps_log=eps_log)
    if cmap == 2:
        par["cmap_angles"] = list(angles if angles is not None else np.linspace(0.5, -0.5, ns))
    p = make_params(par, nx=nx, nz=nz, dx=d, dz=d, nt=nt, dt=dt)
    wav = ricker(nt, dt, 10.0)
    return p, par, wav, s, rho
