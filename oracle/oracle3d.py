"""ORACLE -- test infrastructure only: never imported by the library.

3D restatement (numpy) of the one-way operators on planes.  The reference
has no 3D code; this file restates its 2D call sequence with the depth slice
as a plane: the SSF / PSPI step (propagator/src/SSF.cpp:8-60,
PSPI.cpp:8-53) with a unitary 2D FFT of the slice and k^2 = kx^2 + ky^2 in
the phase shift (phase_shift.ispc:2-16), the product of the x and y tapers
(Taper.h:11-23), edge padding along x and y (Pad.h:77-96), RefSampler
(RefSampler.cpp:10-91) of each slice flattened row by row (through the C++
oracle), Reflect (Reflect.h:19-26), the injection windows along x
(Injection.h:53-65), WEM (wem_prop.cpp:52-74) and BornRefl
(ext_born_refl.cpp:8-105) per (shot, frequency).  prec 32 computes in
complex64, prec 64 in complex128.

PARITY: pinned at ny = 1, where every function here reduces to the C++
oracle's 2D operator (tests/test_3d.py checks that); beyond ny = 1 there is
no reference to pin it to.
"""
from __future__ import annotations

import numpy as np

from . import oracle as O

WEM_PROP_SSF, WEM_PHASE_EXACT_KZ = 0, 1
WEM_DATA_TIME, WEM_DATA_FREQ = 0, 1


def _types(prec):
    return (np.float32, np.complex64) if prec == 32 else (np.float64, np.complex128)


def freqs(p):
    """PropParam.h:45-85 in float arithmetic: propagated frequencies and bins."""
    f32 = np.float32
    nt_pad = p.nt + p.tpad
    tmax = f32(p.ot) + f32(p.dt) * f32(nt_pad - 1)
    if p.fmax == 0:
        fmin = 1
        fmax = p.nfreq if p.nfreq else nt_pad // 2 + 1
    else:
        fmin = int(f32(p.fmin) * tmax)
        fmax = int(f32(p.fmax) * tmax + f32(.5))
    nf = fmax - fmin + 1
    return [f32(p.fmin) + f32(i) / tmax for i in range(nf)], [i + fmin for i in range(nf)], nt_pad


def window(ng, R):
    """Cosine-squared spreading window (Injection.h:53-65)."""
    if ng == 0:
        return np.ones(1, R)
    pi = R(4) * np.arctan(R(1))
    sz = 2 * ng + 1
    g = np.zeros(sz, R)
    for i in range(sz // 2):
        g[i] = (-np.cos(pi / R(ng) * R(i)) + R(1)) / R(2)
    for i in range(sz // 2, sz):
        g[i] = (np.cos(pi / R(ng) * R(i - sz + ng + 1)) + R(1)) / R(2)
    return g


def k_grid(n, d, R):
    """Phshift_cmplx.cpp:13,21-24: k[i] = i dk, k[n - i] = -k[i], dk = 2 pi / (d (n - 1))."""
    k = np.zeros(n, R)
    if n < 2:
        return k
    dk = R(2 * np.pi / (float(d) * (n - 1)))
    for i in range(n // 2):
        k[i] = R(i) * dk
    for i in range(1, n // 2):
        k[n - i] = -k[i]
    return k


def taper(n, pad, R):
    t = np.ones(n, R)
    for i in range(pad):
        t[i] = R(.5) * (R(1) - np.cos(R(np.pi) * R(i) / R(pad - 1)))
        t[n - 1 - i] = t[i]
    return t


def ps_factor(w, k2, dz, s, eps, law, R, C):
    """phase_shift.ispc:2-16 (and the exact-kz law) over an array of k^2."""
    if law == WEM_PHASE_EXACT_KZ:
        kz = np.conj(np.sqrt((w * w * C(s) - k2 + C(1j) * R(1e-5)).astype(C)))
        return np.exp(-C(1j) * R(dz) * kz).astype(C)
    s = C(s)
    a = w * w * R(s.real) - k2
    b = w * w * (R(s.imag) - R(eps) * R(s.real))
    c = np.sqrt(a * a + b * b)
    re = np.sqrt((c + a) / R(2))
    im = -np.sqrt((c - a) / R(2))
    e = np.exp(im * R(dz))
    return (e * np.cos(re * R(dz)) - C(1j) * e * np.sin(re * R(dz))).astype(C)


class Problem3D:
    """Everything a (shot, frequency) plane needs: grids, devices, tables."""

    def __init__(self, q, wavelet, s2, rho, prec=32, refl=False):
        # refl: the 2D BornRefl conventions (ext_born_refl.cpp:18-25): no
        # model padding, pad and pad_y the taper widths only, point receivers
        p = q.p
        R, C = _types(prec)
        self.R, self.C, self.p, self.prec = R, C, p, prec
        self.ny, self.pady, self.tapy = q.ny, (0 if refl else q.pad_y), q.tap_y
        self.nx, self.nz, self.pad, self.tapx = p.nx, p.nz, (0 if refl else p.pad), p.tap
        self.ngs, self.ngr = p.ngs, (0 if refl else p.ngr)
        self.nxg, self.nyg = p.nx + 2 * self.pad, q.ny + 2 * self.pady
        self.Nx, self.Ny = self.nxg + 2 * p.tap, self.nyg + 2 * q.tap_y
        self.freq, self.bin, self.nt_pad = freqs(p)
        # unitary FFT of the time-padded wavelet (FFT1_r.cpp:74-83)
        wp = np.zeros(self.nt_pad, C)
        wp[:p.nt] = np.asarray(wavelet, R)
        self.wave_f = (np.fft.fft(wp) / np.sqrt(R(self.nt_pad))).astype(C)
        f32 = np.float32

        def idx(v, o, d):
            return int((f32(v) - f32(o)) / f32(d) + f32(.5))

        ns, nr = p.ns, p.nr
        self.src = [(idx(p.src_x[i], p.ox, p.dx), idx(q.src_y[i], q.oy, q.dy), idx(p.src_z[i], p.oz, p.dz))
                    for i in range(ns)]
        self.rec = [(idx(p.rec_x[i], p.ox, p.dx), idx(q.rec_y[i], q.oy, q.dy), idx(p.rec_z[i], p.oz, p.dz))
                    for i in range(nr)]
        self.gs, self.gr = window(self.ngs, R), window(self.ngr, R)
        # padded slices (edge-extended) and their tables
        sp = self.pad3(np.asarray(s2, np.complex64))
        dp = self.pad3(np.asarray(rho, np.complex64))
        self.sp = sp.astype(C)
        flat = np.ascontiguousarray(sp.reshape(self.nz, -1))
        sref, ref = O.refsampler(p, flat)
        self.sref = sref.astype(C)
        self.ref = ref.reshape(self.nz, self.nyg, self.nxg)
        dpc = dp.astype(C)
        self.rc = np.zeros_like(self.sp)
        for z in range(1, self.nz):
            num = dpc[z] * np.sqrt(self.sp[z - 1]) - dpc[z - 1] * np.sqrt(self.sp[z])
            den = dpc[z] * np.sqrt(self.sp[z - 1]) + dpc[z - 1] * np.sqrt(self.sp[z])
            self.rc[z] = num / den
        kx, ky = k_grid(self.Nx, p.dx, R), k_grid(self.Ny, q.dy, R)
        self.k2 = (kx[None, :] * kx[None, :] + ky[:, None] * ky[:, None]).astype(R)
        self.taper = (taper(self.nyg, q.pad_y, R)[:, None] * taper(self.nxg, p.pad, R)[None, :]).astype(R)

    def pad3(self, m):
        m = np.asarray(m).reshape(self.nz, self.ny, self.nx)
        m = np.concatenate([np.repeat(m[..., :1], self.pad, -1), m, np.repeat(m[..., -1:], self.pad, -1)], -1)
        m = np.concatenate([np.repeat(m[:, :1], self.pady, 1), m, np.repeat(m[:, -1:], self.pady, 1)], 1)
        return m

    def omega(self, f):
        return self.R(2 * np.pi * float(self.freq[f]))

    def _fft(self, x, inv):
        n = self.R(np.sqrt(float(self.Nx * self.Ny)))
        return (np.fft.ifft2(x) * n if inv else np.fft.fft2(x) / n).astype(self.C)

    def _embed(self, w):
        P = np.zeros((self.Ny, self.Nx), self.C)
        P[self.tapy:self.tapy + self.nyg, self.tapx:self.tapx + self.nxg] = w
        return P

    def _grid(self, P):
        return P[self.tapy:self.tapy + self.nyg, self.tapx:self.tapx + self.nxg]

    def step(self, w, z, om, adj=False):
        """SSF / PSPI step of depth z on a padded slice (SSF.cpp:8-60)."""
        R, C, p = self.R, self.C, self.p
        out = np.zeros((self.nyg, self.nxg), C)
        ref = self.ref[z]
        if not adj:
            S = self._fft(self._embed(w), False)
        acc = np.zeros((self.Ny, self.Nx), C)
        for j in range(p.nref):
            sr = self.sref[z, j]
            ph = ps_factor(om, self.k2, p.dz, sr, p.eps, p.phase_law, R, C)
            loc = ref == j
            corr = None
            if p.prop == WEM_PROP_SSF:
                corr = (-C(1j) * om * R(p.dz) * (self.sp[z] - sr) / np.sqrt(sr)).astype(C)
            if not adj:
                wr = self._grid(self._fft(S * ph, True)) * self.taper
                if corr is not None:
                    wr = np.where(loc, wr * np.exp(corr), wr)
                out[loc] = wr[loc]
            else:
                wr = np.where(loc, w, C(0))
                if corr is not None:
                    wr = np.where(loc, wr * np.exp(np.conj(corr)), wr)
                wr = wr * self.taper
                acc += self._fft(self._embed(wr), False) * np.conj(ph)
        if adj:
            out = self._grid(self._fft(acc, True)).astype(C)
        return out

    def spread_src(self, W, s, f):
        x, y, z = self.src[s]
        v = self.wave_f[self.bin[f]]
        for g in range(-self.ngs, self.ngs + 1):
            xx = x + g + self.pad
            if 0 <= xx < self.nxg:
                W[z, y + self.pady, xx] += self.gs[g + self.ngs] * v

    def gather(self, W, vals):
        for i, (x, y, z) in enumerate(self.rec):
            for g in range(-self.ngr, self.ngr + 1):
                xx = x + g + self.pad
                if 0 <= xx < self.nxg:
                    vals[i] += self.gr[g + self.ngr] * W[z, y + self.pady, xx]

    def spread_rec(self, W, vals):
        for i, (x, y, z) in enumerate(self.rec):
            for g in range(-self.ngr, self.ngr + 1):
                xx = x + g + self.pad
                if 0 <= xx < self.nxg:
                    W[z, y + self.pady, xx] += self.gr[g + self.ngr] * vals[i]

    def down(self, M, om):
        W = M.copy()
        for z in range(self.nz - 1):
            W[z + 1] += self.step(W[z], z, om)
        return W

    def up(self, M, om):
        W = M.copy()
        for z in range(self.nz - 1, 0, -1):
            W[z - 1] += self.step(W[z], z, om)
        return W

    def up_adj(self, D, om):
        W = D.copy()
        for z in range(self.nz - 1):
            W[z + 1] += self.step(W[z], z + 1, om, adj=True)
        return W


def _emit(P, D, kind):
    p = P.p
    if kind == WEM_DATA_TIME:
        n = P.nt_pad
        t = np.fft.ifft(D.astype(np.complex128), axis=-1) * np.sqrt(n)
        return np.ascontiguousarray(t.real[..., :p.nt].astype(np.float32))
    nbin = p.nbin if p.nbin else P.nt_pad
    out = np.zeros(D.shape[:2] + (nbin,), np.complex64)
    m = min(nbin, P.nt_pad)
    out[..., :m] = D[..., :m]
    return out


def _absorb(P, data, kind):
    p = P.p
    D = np.zeros((p.ns, p.nr, P.nt_pad), P.C)
    if kind == WEM_DATA_TIME:
        x = np.zeros((p.ns, p.nr, P.nt_pad), np.complex128)
        x[..., :p.nt] = np.asarray(data, np.float32)
        D[:] = np.fft.fft(x, axis=-1) / np.sqrt(P.nt_pad)
    else:
        m = min(np.asarray(data).shape[-1], P.nt_pad)
        D[..., :m] = np.asarray(data)[..., :m]
    return D


def wem_forward(q, wavelet, s2, rho, kind=WEM_DATA_TIME, prec=32):
    """WEM per (shot, frequency): down, record, R D, up, record (wem_prop.cpp:52-74)."""
    P = Problem3D(q, wavelet, s2, rho, prec)
    p = P.p
    D = np.zeros((p.ns, p.nr, P.nt_pad), P.C)
    for f in range(len(P.freq)):
        om = P.omega(f)
        for s in range(p.ns):
            M = np.zeros((P.nz, P.nyg, P.nxg), P.C)
            P.spread_src(M, s, f)
            W = P.down(M, om)
            vals = np.zeros(p.nr, P.C)
            P.gather(W, vals)
            U = P.up(P.rc * W, om)
            P.gather(U, vals)
            D[s, :, P.bin[f]] += vals
    return _emit(P, D, kind)


def refl_forward(q, wavelet, s2, model, kind=WEM_DATA_TIME, prec=32):
    """BornRefl with one reflectivity [nz][ny][nx] for every frequency."""
    ones = np.ones_like(np.asarray(s2))
    P = Problem3D(q, wavelet, s2, ones, prec, refl=True)
    p = P.p
    m = np.zeros((P.nz, P.nyg, P.nxg), P.C)
    m[:, P.pady:P.pady + P.ny, P.pad:P.pad + P.nx] = np.asarray(model).reshape(P.nz, P.ny, P.nx)
    D = np.zeros((p.ns, p.nr, P.nt_pad), P.C)
    for f in range(len(P.freq)):
        om = P.omega(f)
        for s in range(p.ns):
            M = np.zeros((P.nz, P.nyg, P.nxg), P.C)
            P.spread_src(M, s, f)
            bg = P.down(M, om)
            U = P.up(bg * m, om)
            vals = np.zeros(p.nr, P.C)
            P.gather(U, vals)
            D[s, :, P.bin[f]] += vals
    return _emit(P, D, kind)


def refl_adjoint(q, wavelet, s2, data, kind=WEM_DATA_TIME, prec=32):
    """image = sum over (shot, frequency) of conj(bg) Up^H(rec^H data)."""
    ones = np.ones_like(np.asarray(s2))
    P = Problem3D(q, wavelet, s2, ones, prec, refl=True)
    p = P.p
    D = _absorb(P, data, kind)
    img = np.zeros((P.nz, P.nyg, P.nxg), P.C)
    for f in range(len(P.freq)):
        om = P.omega(f)
        for s in range(p.ns):
            M = np.zeros((P.nz, P.nyg, P.nxg), P.C)
            P.spread_src(M, s, f)
            bg = P.down(M, om)
            A = np.zeros_like(M)
            P.spread_rec(A, D[s, :, P.bin[f]])
            A = P.up_adj(A, om)
            img += np.conj(bg) * A
    return np.ascontiguousarray(img[:, P.pady:P.pady + P.ny, P.pad:P.pad + P.nx].astype(np.complex64))
