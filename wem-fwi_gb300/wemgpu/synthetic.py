"""Seeded synthetic workloads of the benchmark configurations.

The reference publishes no benchmark inputs (its notebooks' SEP data files
are absent), so the configurations are generated here from their stated
shapes and value distributions, deterministically from a seed:

* ``c1``: 2D SSF modelling + migration, 256x200, dx=dz=10 m, 1 shot, 64
  frequencies in 2-20 Hz, linear 1500->3500 m/s plus Gaussian-smoothed
  (sigma 8 cells) +-5 % noise, 10 Hz Ricker at x=nx/2, receivers every cell.
* ``c2``: 2D Born with PSPI nref=4, 1024x500, dx=dz=10 m, 48 shots, 128
  frequencies in 2-25 Hz, smooth background as c1, 1 % random spikes of
  amplitude N(0, 0.1) (relative slowness perturbation).
* ``c3``: FWI gradient, 768x300, dx=dz=12.5 m, 32 shots, 96 frequencies in
  3-18 Hz, SSF; true model of 6 dipping layers (1500-4500 m/s, dips within
  +-15 deg) with a smooth elliptical anomaly; start model = true smoothed
  with sigma 20 cells.
* ``c4``: extended Born with nh = 21 subsurface-offset lags, 1024x400,
  dx=dz=10 m, 64 shots, 80 frequencies in 3-20 Hz, uneven per-shot
  apertures of 256-1024 cells.
* ``c5``: 3D PSPI (nref 3) with a 2D FFT per depth slice, 256x256x300,
  dx=dy=dz=15 m, 16 shots on a 4x4 grid, 64 frequencies in 3-15 Hz.

Slowness is the complex squared slowness 1/v^2 - i q of the reference
(propagator/test/test_wem_ops.py:51-52); density is 1.
"""
from __future__ import annotations

import numpy as np


def ricker(nt, dt, f0, t0=None):
    t = np.arange(nt) * dt - (t0 if t0 is not None else 1.5 / f0)
    a = (np.pi * f0 * t) ** 2
    return ((1 - 2 * a) * np.exp(-a)).astype(np.float32)


def _smooth(a, sigma):
    from scipy.ndimage import gaussian_filter
    return gaussian_filter(a, sigma, mode="nearest")


def _slow(v, q=1e-10):
    return (1.0 / v.astype(np.float64) ** 2 - 1j * q).astype(np.complex64)


def gradient_velocity(nz, nx, v0, v1, noise, sigma, rng):
    v = v0 + (v1 - v0) * np.linspace(0, 1, nz)[:, None] * np.ones((1, nx))
    n = _smooth(rng.uniform(-1, 1, (nz, nx)), sigma)
    n /= max(np.abs(n).max(), 1e-12)
    return v * (1 + noise * n)


def _acquisition(nx, dx, ns):
    step = nx // ns
    return dict(ns=ns, osx=dx * (step // 2), dsx=dx * step, osz=0.0, nr=nx, orx=0.0, drx=dx, orz=0.0)


def c1(seed=0):
    nx, nz, dx = 256, 200, 10.0
    rng = np.random.default_rng(seed)
    v = gradient_velocity(nz, nx, 1500.0, 3500.0, 0.05, 8, rng)
    nt, dt = 876, 0.004  # tmax 3.5 s: 64 bins from 2 to 20 Hz
    par = dict(_acquisition(nx, dx, 1), osx=dx * (nx // 2), prop="ssf", nref=1, tap=0, pad=0,
               fmin=2.0, fmax=20.0, eps=0.04, ngs=0, ngr=0, ntaylor=1)
    s = _slow(v)
    return dict(name="c1", par=par, nx=nx, nz=nz, dx=dx, dz=dx, nt=nt, dt=dt,
                wavelet=ricker(nt, dt, 10.0), slow=s, rho=np.ones_like(s))


def c2(seed=0):
    nx, nz, dx = 1024, 500, 10.0
    rng = np.random.default_rng(seed)
    v = gradient_velocity(nz, nx, 1500.0, 3500.0, 0.05, 8, rng)
    # 128 bins from 2 to 25 Hz: tmax = 127/23 s
    dt = 0.004
    nt = int(round(127 / 23 / dt)) + 1
    par = dict(_acquisition(nx, dx, 48), prop="pspi", nref=4, tap=0, pad=0, fmin=2.0, fmax=25.0, eps=0.04,
               ngs=0, ngr=0, ntaylor=1)
    s = _slow(v)
    spikes = (rng.random((nz, nx)) < 0.01) * rng.normal(0, 0.1, (nz, nx))
    ds = (spikes * s.real).astype(np.complex64)
    return dict(name="c2", par=par, nx=nx, nz=nz, dx=dx, dz=dx, nt=nt, dt=dt,
                wavelet=ricker(nt, dt, 10.0), slow=s, rho=np.ones_like(s), dslow=ds,
                drho=np.zeros_like(s))


def layered_velocity(nz, nx, dx, rng, nlayer=6, vmin=1500.0, vmax=4500.0, maxdip=15.0):
    x = np.arange(nx) * dx
    z = np.arange(nz)[:, None] * dx
    depths = np.sort(rng.uniform(0.1, 0.95, nlayer - 1)) * nz * dx
    vel = np.sort(rng.uniform(vmin, vmax, nlayer))
    dips = np.tan(np.deg2rad(rng.uniform(-maxdip, maxdip, nlayer - 1)))
    v = np.full((nz, nx), vel[0])
    for k in range(nlayer - 1):
        iface = depths[k] + dips[k] * (x - x.mean())
        v = np.where(z >= iface[None, :], vel[k + 1], v)
    # smooth elliptical anomaly (-10 %)
    cx, cz = rng.uniform(0.3, 0.7) * nx * dx, rng.uniform(0.4, 0.7) * nz * dx
    ax, az = 0.12 * nx * dx, 0.08 * nz * dx
    r2 = ((x[None, :] - cx) / ax) ** 2 + ((z - cz) / az) ** 2
    v = v * (1 - 0.1 * np.exp(-r2))
    return v


def c3(seed=0):
    nx, nz, dx = 768, 300, 12.5
    rng = np.random.default_rng(seed)
    v_true = layered_velocity(nz, nx, dx, rng)
    v_start = _smooth(v_true, 20)
    # 96 bins from 3 to 18 Hz: nt 1536 (smooth FFT length), tmax 6.2935 s
    nt, dt = 1536, 0.0041
    par = dict(_acquisition(nx, dx, 32), prop="ssf", nref=1, tap=0, pad=0, fmin=3.0, fmax=18.0, eps=0.04,
               ngs=0, ngr=0, ntaylor=1)
    s_true, s0 = _slow(v_true), _slow(v_start)
    return dict(name="c3", par=par, nx=nx, nz=nz, dx=dx, dz=dx, nt=nt, dt=dt,
                wavelet=ricker(nt, dt, 10.0), slow_true=s_true, slow=s0, rho=np.ones_like(s0))


def c4(seed=0, nh=21):
    """Extended Born (subsurface offset): 1024 x 400, dx = dz = 10 m, 64
    shots, 80 frequencies in 3-20 Hz, nh = 21 lags; smooth random background
    (as c1); extended reflectivity of 1 % random spikes N(0, 0.1) spread over
    the lags with a Gaussian taper (sigma 3 lags); per-shot aperture widths
    uniform in [256, 1024] cells (even), centred on the source and moved
    inside the model."""
    nx, nz, dx = 1024, 400, 10.0
    rng = np.random.default_rng(seed)
    v = gradient_velocity(nz, nx, 1500.0, 3500.0, 0.05, 8, rng)
    nt, dt = 1152, 0.004  # 80 bins from 3 to 20 Hz, a smooth FFT length
    ns = 64
    par = dict(_acquisition(nx, dx, ns), prop="ssf", nref=1, tap=0, pad=0, fmin=3.0, fmax=20.0, eps=0.04,
               ngs=0, ngr=0, ntaylor=1)
    s = _slow(v)
    hm = (nh - 1) // 2
    spikes = (rng.random((nz, nx)) < 0.01) * rng.normal(0, 0.1, (nz, nx))
    taper = np.exp(-0.5 * ((np.arange(nh) - hm) / 3.0) ** 2)
    refl = (taper[:, None, None] * spikes[None]).astype(np.complex64)
    step = nx // ns
    srcx = step // 2 + step * np.arange(ns)
    widths = 2 * (rng.integers(256, 1025, ns) // 2)
    x0 = np.clip(srcx - widths // 2, 0, nx - widths)
    apertures = np.stack([x0, widths], 1).astype(np.int32)
    return dict(name="c4", par=par, nx=nx, nz=nz, dx=dx, dz=dx, nt=nt, dt=dt, nh=nh,
                wavelet=ricker(nt, dt, 10.0), slow=s, rho=np.ones_like(s), refl=refl, apertures=apertures)


def c5(seed=0, rstep=2):
    """3D PSPI with a 2D FFT per slice: 256 x 256 x 300, dx = dy = dz = 15 m,
    16 shots on a 4 x 4 grid, 64 frequencies in 3-15 Hz, nref = 3; velocity a
    linear gradient 1500 -> 3500 m/s in depth plus Gaussian-smoothed (sigma
    6 cells) +-8 % noise; receivers every ``rstep`` cells on the surface;
    the reflectivity of the migration pair is 1 % random spikes N(0, 0.1)."""
    from .params import make_params3d
    nx = ny = 256
    nz, d = 300, 15.0
    rng = np.random.default_rng(seed)
    v = 1500.0 + 2000.0 * np.linspace(0, 1, nz)[:, None, None] * np.ones((1, ny, nx))
    n = _smooth(rng.uniform(-1, 1, (nz, ny, nx)), 6)
    n /= max(np.abs(n).max(), 1e-12)
    v = v * (1 + 0.08 * n)
    s = _slow(v)
    nt, dt = 648, 0.008  # 64 bins from 3 to 15 Hz, a smooth FFT length
    g = (np.arange(4) + 0.5) * (nx / 4) * d
    sx, sy = np.meshgrid(g, g)
    sx, sy = sx.ravel(), sy.ravel()
    rx, ry = np.meshgrid(np.arange(0, nx, rstep) * d, np.arange(0, ny, rstep) * d)
    rx, ry = rx.ravel(), ry.ravel()
    par = dict(prop="pspi", nref=3, tap=0, pad=0, fmin=3.0, fmax=15.0, eps=0.04, ngs=0, ngr=0, ntaylor=1)
    q = make_params3d(par, nx=nx, ny=ny, nz=nz, dx=d, dy=d, dz=d, nt=nt, dt=dt, sx=sx, sy=sy,
                      sz=np.zeros_like(sx), rx=rx, ry=ry, rz=np.zeros_like(rx))
    refl = ((rng.random((nz, ny, nx)) < 0.01) * rng.normal(0, 0.1, (nz, ny, nx))).astype(np.complex64)
    return dict(name="c5", q=q, nx=nx, ny=ny, nz=nz, nt=nt, dt=dt, wavelet=ricker(nt, dt, 10.0), slow=s,
                rho=np.ones_like(s), refl=refl)


CONFIGS = {"c1": c1, "c2": c2, "c3": c3, "c4": c4}


def params_of(cfg):
    from .params import make_params
    return make_params(cfg["par"], nx=cfg["nx"], nz=cfg["nz"], dx=cfg["dx"], dz=cfg["dz"], nt=cfg["nt"],
                       dt=cfg["dt"])
