"""Generate the reference-run golden fixtures of tests/golden (ref_*.npz,
refc1.npz and refinterp.npz).

The outputs come from the reference's own operator classes (WEM, BornFull,
BornRefl, BornTomo, extWEM, extBornFull of propagator/src; the interpolators
LanczosInterpolation2D and Spline2D of operator/src), compiled from
the reference checkout by oracle/ref/Makefile and called through
oracle/ref_oracle.py; this script needs that checkout (WEM_REFERENCE, or the
default path in ref_oracle).  Each fixture holds its inputs (wavelet, models,
perturbations, data) and the reference's outputs, so the tests compare
against them on machines without the reference.

    python tests/golden/make_ref_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "wem-fwi_gb300"), os.path.join(ROOT, "tests")]

from cases import cmap_case, rand_c, small_case  # noqa: E402
from oracle import ref_oracle as R  # noqa: E402

# (name, case keywords, operators); keywords with "cmap" build a
# cmap_case (explicit device coordinates, a conformal map), the others a
# small_case
CASES = [
    ("ssf", dict(prop="ssf", nref=1, ns=2), ("wem", "born")),
    ("pspi3", dict(prop="pspi", nref=3, ns=2, tap=4, pad=2), ("wem", "born")),
    ("ssf_t2_tap0", dict(prop="ssf", nref=1, ns=1, nx=50, tap=0, pad=0, ntaylor=2), ("wem", "born")),
    ("pspi2_odd_t0", dict(prop="pspi", nref=2, ns=2, nx=51, ntaylor=0), ("wem", "born")),
    ("ssf_tpad", dict(prop="ssf", nref=1, ns=1, nz=20), ("wem", "born")),
    ("refl_tomo", dict(prop="pspi", nref=2, ns=2, nz=12, tap=4, pad=3), ("refl", "tomo")),
    ("ext", dict(prop="ssf", nref=1, ns=2, nz=16), ("extwem", "extborn")),
    ("coords", dict(cmap=0, prop="pspi", nref=2), ("wem", "born")),
    ("cmap_log", dict(cmap=1, prop="ssf", nref=1), ("wem", "born")),
    ("cmap_rot", dict(cmap=2, prop="pspi", nref=3), ("wem", "born")),
    ("pspi4_t4", dict(prop="pspi", nref=4, ns=2, nx=44, tap=3, pad=2, ntaylor=4), ("wem", "born")),
    ("refl_tomo_ssf", dict(prop="ssf", nref=1, ns=2, nx=48, nz=14, tap=0, pad=0), ("refl", "tomo")),
    ("ssf_point_eps0", dict(prop="ssf", nref=1, ns=2, nx=40, nz=16, tap=0, pad=0, eps=0.0, ngs=0, ngr=0),
     ("wem", "born")),
    ("pspi3_t3_band", dict(prop="pspi", nref=3, ns=2, nx=45, nz=18, ntaylor=3, fmin=4.0, fmax=18.0),
     ("wem", "born")),
    ("pspi2_buried", dict(prop="pspi", nref=2, ns=2, nx=48, nz=20), ("wem", "born")),
    # a prime trace length: the time <-> frequency step as a DFT over the bins
    ("ssf_nt_prime", dict(prop="ssf", nref=1, ns=2, nz=16, nt=127), ("wem", "born")),
    ("ext_pspi", dict(prop="pspi", nref=2, ns=2, nz=14, tap=3, pad=2), ("extwem", "extborn")),
]


def make_case(kw):
    return cmap_case(**kw) if "cmap" in kw else small_case(**kw)
# BornRefl and BornTomo spread the source over "ng" cells (ext_born_refl.cpp:18)
EXTRA_PAR = {"ssf_tpad": dict(tpad=32), "refl_tomo": dict(ng=2), "refl_tomo_ssf": dict(ng=1),
             # sources 3 and receivers 2 depth steps below the surface
             "pspi2_buried": dict(osz=30.0, orz=20.0)}


def run_case(name, kw, ops, seed):
    p, par, wav, s, rho = make_case(kw)
    par = dict(par, **EXTRA_PAR.get(name, {}))
    g = R.Grid(p.nx, p.nz, p.dx, p.dz, p.nt, p.dt)
    nf = R.nfreq(par, g, wav)
    rng = np.random.default_rng(seed)
    out = dict(wav=wav, s=s, rho=rho, nf=np.int32(nf))
    data_in = (rng.random((p.ns, p.nr, p.nt)) - .5).astype(np.float32)
    out["data_in"] = data_in
    if "wem" in ops:
        out["wem"] = R.wem_forward(par, g, wav, s, rho)
    if "born" in ops:
        ds = (rand_c(rng, s.shape) * 1e-8).astype(np.complex64)
        dr = (rand_c(rng, s.shape) * 0.1).astype(np.complex64)
        out.update(ds=ds, dr=dr)
        out["born_fwd"] = R.born_forward(par, g, wav, s, rho, ds, dr)
        out["born_adj_s"], out["born_adj_r"] = R.born_adjoint(par, g, wav, s, rho, data_in)
    if "refl" in ops:
        m = (rand_c(rng, (nf, p.nz, p.nx)) * 0.1).astype(np.complex64)
        out["refl_m"] = m
        out["refl_fwd"] = R.bornrefl_forward(par, g, wav, s, m)
        out["refl_adj"] = R.bornrefl_adjoint(par, g, wav, s, data_in, nf)
    if "tomo" in ops:
        refl = (rand_c(rng, (nf, p.nz, p.nx)) * 0.2).astype(np.complex64)
        dm = (rand_c(rng, s.shape) * 1e-8).astype(np.complex64)
        out.update(tomo_refl=refl, tomo_dm=dm)
        out["tomo_fwd"] = R.borntomo_forward(par, g, wav, s, refl, dm)
        out["tomo_adj"] = R.borntomo_adjoint(par, g, wav, s, refl, data_in)
    if "extwem" in ops or "extborn" in ops:
        s3 = (np.repeat(s[None], nf, 0) * (1 + 0.02 * rng.standard_normal((nf, 1, 1)))).astype(np.complex64)
        r3 = np.repeat(rho[None], nf, 0).astype(np.complex64)
        out.update(s3=s3, r3=r3)
        if "extwem" in ops:
            out["extwem"] = R.extwem_forward(par, g, wav, s3, r3)
        if "extborn" in ops:
            ds3 = (rand_c(rng, s3.shape) * 1e-8).astype(np.complex64)
            dr3 = (rand_c(rng, s3.shape) * 0.1).astype(np.complex64)
            out.update(ds3=ds3, dr3=dr3)
            out["extborn_fwd"] = R.extborn_forward(par, g, wav, s3, r3, ds3, dr3)
            out["extborn_adj_s"], out["extborn_adj_r"] = R.extborn_adjoint(par, g, wav, s3, r3, data_in)
    par = {k: (list(map(float, v)) if isinstance(v, (list, tuple, np.ndarray)) else v) for k, v in par.items()}
    meta = dict(name=name, case=kw, par=par, ops=list(ops), seed=seed,
                source="reference propagator/src compiled by oracle/ref/Makefile")
    out["meta"] = np.frombuffer(json.dumps(meta).encode(), np.uint8)
    return out


# model-space interpolators of the FWI preconditioner (operator/src
# LanczosInterpolation2D.h, Spline2D.h): (name, coarse axes, fine axes,
# kind, parameters); axes ((n1, d1), (n2, d2)) as scripts/fwi.py builds them
INTERP = [
    ("fwi_like_lanczos", ((17, 47.5), (9, 37.375)), ((77, 10.0), (24, 13.0)), "lanczos", (2.0, 3.0)),
    ("fwi_like_spline", ((17, 47.5), (9, 37.375)), ((77, 10.0), (24, 13.0)), "spline", (1 / 3, 1 / 3)),
    ("square_bspline", ((12, 3.0), (12, 3.0)), ((34, 1.0), (34, 1.0)), "spline", (0.0, 1.0)),
    ("bench_lanczos", ((13, 200.0), (9, 150.0)), ((193, 12.5), (93, 13.0)), "lanczos", (1.0, 1.0)),
]


def interp_fixture(seed):
    rng = np.random.default_rng(seed)
    out, meta = {}, []
    for name, ma, da, kind, (p0, p1) in INTERP:
        (m1, m2), (d1, d2) = ma, da
        m = (rng.standard_normal((m2[0], m1[0])) + 1j * rng.standard_normal((m2[0], m1[0]))).astype(np.complex64)
        d = (rng.standard_normal((d2[0], d1[0])) + 1j * rng.standard_normal((d2[0], d1[0]))).astype(np.complex64)
        out[name + "_m"], out[name + "_d"] = m, d
        out[name + "_fwd"] = R.interp2d(kind, ma, da, p0, p1, m)
        out[name + "_adj"] = R.interp2d(kind, ma, da, p0, p1, d, adj=True)
        meta.append(dict(name=name, model_axes=ma, data_axes=da, kind=kind, params=[p0, p1]))
    out["meta"] = np.frombuffer(json.dumps(dict(cases=meta, seed=seed,
                                                source="reference operator/src compiled by oracle/ref/Makefile")
                                           ).encode(), np.uint8)
    return out


# point Injection (propagator/src/Injection.cpp): (name, nz, nx, npt, ng, tap,
# nt, nshot); the points' depths and positions are seeded, some outside the
# row so that the window's bounds check is exercised
INJECT = [
    ("line_ng1_tap1", 6, 50, 30, 1, 1, 24, 0),
    ("scatter_ng3", 5, 41, 17, 3, 2, 12, 0),
    ("shots_ng0", 4, 36, 20, 0, 0, 10, 3),
    ("shots_ng2_tap3", 7, 45, 14, 2, 3, 9, 4),
]


def inject_fixture(seed):
    rng = np.random.default_rng(seed)
    out, cases = {}, []
    for name, nz, nx, npt, ng, tap, nt, nshot in INJECT:
        iz = rng.integers(0, nz, npt).astype(np.int32)
        ix = rng.integers(-ng - tap - 2, nx + 2, npt).astype(np.int32)
        step, shot = int(rng.integers(0, nt)), int(rng.integers(0, max(nshot, 1)))
        m = rand_c(rng, (nshot, npt, nt) if nshot else (nt,))
        d = rand_c(rng, (nz, nx))
        out[name + "_iz"], out[name + "_ix"] = iz, ix
        out[name + "_m"], out[name + "_d"] = m, d
        out[name + "_fwd"] = R.inject(iz, ix, ng, tap, nz, nx, step, shot, m)
        out[name + "_adj"] = R.inject(iz, ix, ng, tap, nz, nx, step, shot, d, adj=True, nt=nt, nshot=nshot)
        cases.append(dict(name=name, nz=nz, nx=nx, ng=ng, tap=tap, nt=nt, nshot=nshot, step=step, shot=shot))
    meta = dict(cases=cases, source="reference propagator/src/Injection.cpp compiled by oracle/ref/Makefile")
    out["meta"] = np.frombuffer(json.dumps(meta).encode(), np.uint8)
    return out


def c1_fixture():
    """Configuration c1 at full size (256 x 200, one shot, 64 frequencies,
    SSF): the reference's modelling of the seeded model and its Born adjoint
    (as coded) of that data at the same background."""
    from wemgpu import synthetic as S
    cfg = S.c1()
    par = dict(cfg["par"])
    g = R.Grid(cfg["nx"], cfg["nz"], cfg["dx"], cfg["dz"], cfg["nt"], cfg["dt"])
    s, rho, wav = cfg["slow"], cfg["rho"], cfg["wavelet"]
    d = R.wem_forward(par, g, wav, s, rho)
    gs, gr = R.born_adjoint(par, g, wav, s, rho, d)
    meta = dict(name="c1", par=par, source="reference propagator/src compiled by oracle/ref/Makefile")
    return dict(s=s, wem=d, born_adj_s=gs, born_adj_r=gr, meta=np.frombuffer(json.dumps(meta).encode(), np.uint8))


def c3_fixture():
    """Configuration c3's model and geometry (768 x 300: the 768-point warp
    kernels of the benchmarked gradient) on its first shot and the band's 21
    lowest frequencies (3-6 Hz): the reference's modelling, kept on every
    8th receiver, and its Born adjoint (as coded) of its own data, slowness
    part.  The model is not stored: the test rebuilds it from its seed and
    checks it against the sums kept here."""
    from wemgpu import synthetic as S
    cfg = S.c3()
    par = dict(cfg["par"], ns=1, fmax=6.0)
    g = R.Grid(cfg["nx"], cfg["nz"], cfg["dx"], cfg["dz"], cfg["nt"], cfg["dt"])
    s, rho, wav = cfg["slow"], cfg["rho"], cfg["wavelet"]
    d = R.wem_forward(par, g, wav, s, rho)
    gs, _ = R.born_adjoint(par, g, wav, s, rho, d)
    meta = dict(name="c3_shot0_3to6hz", par=par, source="reference propagator/src compiled by oracle/ref/Makefile")
    sums = np.array([np.sum(s.real, dtype=np.float64), np.sum(s.imag, dtype=np.float64),
                     np.sum(np.abs(s), dtype=np.float64)])
    return dict(s_sums=sums, wem_rx8=d[:, ::8, :], born_adj_s=gs,
                meta=np.frombuffer(json.dumps(meta).encode(), np.uint8))


def c2_fixture():
    """Configuration c2's model and geometry (1024 x 500, PSPI with four
    references: the several-reference 1024-point warp kernels) on its first
    shot and the band's lowest frequencies (2-3.5 Hz): the reference's
    modelling and Born forward of c2's perturbation, kept on every 8th
    receiver, and its Born adjoint (as coded) of its own modelled data,
    slowness part on every 4th depth.  The model is rebuilt from its seed
    by the test and checked against the sums kept here."""
    from wemgpu import synthetic as S
    cfg = S.c2()
    par = dict(cfg["par"], ns=1, fmax=3.5)
    g = R.Grid(cfg["nx"], cfg["nz"], cfg["dx"], cfg["dz"], cfg["nt"], cfg["dt"])
    s, rho, wav = cfg["slow"], cfg["rho"], cfg["wavelet"]
    d = R.wem_forward(par, g, wav, s, rho)
    b = R.born_forward(par, g, wav, s, rho, cfg["dslow"], cfg["drho"])
    gs, _ = R.born_adjoint(par, g, wav, s, rho, d)
    meta = dict(name="c2_shot0_2to3.5hz", par=par,
                source="reference propagator/src compiled by oracle/ref/Makefile")
    sums = np.array([np.sum(s.real, dtype=np.float64), np.sum(s.imag, dtype=np.float64),
                     np.sum(np.abs(cfg["dslow"]), dtype=np.float64)])
    return dict(sums=sums, wem_rx8=d[:, ::8, :], born_fwd_rx8=b[:, ::8, :], born_adj_s_z4=gs[::4],
                meta=np.frombuffer(json.dumps(meta).encode(), np.uint8))


def main():
    if not R.available():
        raise SystemExit(f"reference checkout not found at {R.ref_root()} (set WEM_REFERENCE)")
    R.build()
    path = os.path.join(HERE, "refc1.npz")
    np.savez_compressed(path, **c1_fixture())
    print(f"{path}: {os.path.getsize(path) / 1024:.0f} KB")
    path = os.path.join(HERE, "refc2.npz")
    np.savez_compressed(path, **c2_fixture())
    print(f"{path}: {os.path.getsize(path) / 1024:.0f} KB")
    path = os.path.join(HERE, "refc3.npz")
    np.savez_compressed(path, **c3_fixture())
    print(f"{path}: {os.path.getsize(path) / 1024:.0f} KB")
    path = os.path.join(HERE, "refinject.npz")
    np.savez_compressed(path, **inject_fixture(300))
    print(f"{path}: {os.path.getsize(path) / 1024:.0f} KB")
    path = os.path.join(HERE, "refinterp.npz")
    np.savez_compressed(path, **interp_fixture(200))
    print(f"{path}: {os.path.getsize(path) / 1024:.0f} KB")
    for i, (name, kw, ops) in enumerate(CASES):
        out = run_case(name, kw, ops, seed=100 + i)
        path = os.path.join(HERE, f"ref_{name}.npz")
        np.savez_compressed(path, **out)
        print(f"{path}: {os.path.getsize(path) / 1024:.0f} KB")


if __name__ == "__main__":
    main()
