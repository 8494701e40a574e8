"""oracle/wem_np.py -- TEST INFRASTRUCTURE (CPU oracle), never the product path.

A NumPy FP64 restatement of the reference operator for tiny 2-D cases, written
independently of oracle/wem_oracle_impl.h so that the two oracles check each other.
Follows src/Imaging/c/wem.c: setup :28-89, spectra :112-140, extrap1f :206-287,
ssop :289-378, pspiop :380-471, linear_interp :473-478, f_op :480-514,
boundary_condition :546-564. Integer decisions (band, source cell, reference
indices) use the reference's float32 expressions, like the C FP64 oracle.
"""
from __future__ import annotations

import numpy as np

f32 = np.float32


def _grid(p):
    nt, padt, dt = int(p["nt"]), int(p["padt"]), f32(p["dt"])
    ntfft = int(f32(2 * padt) * f32(nt) / f32(2))
    nw = ntfft // 2 + 1
    fmax, fmin = f32(p["fmax"]), f32(p["fmin"])
    if fmax * dt * f32(ntfft) + f32(1) < nw:
        ifmax = int(f32(int(fmax)) * dt * f32(ntfft) + f32(1))
    else:
        ifmax = nw
    if fmin * dt * f32(ntfft) + f32(1) < ifmax:
        ifmin = int(f32(int(fmin)) * dt * f32(ntfft))
    else:
        ifmin = 0
    return ntfft, nw, ifmin, ifmax


def _tables(p, vel):
    nx, nz = vel.shape
    nref = int(p["nref"]) if p.get("pspi", 1) else 1
    vel = vel.astype(np.float32)
    po = nx / vel.astype(np.float64).sum(0)
    pd = 1.0 / vel.astype(np.float64) - po[None, :]
    vmin = vel.min(0)
    vmax = vel.max(0)
    vref32 = np.empty((nref, nz), np.float32)
    vref64 = np.empty((nref, nz))
    i1 = np.zeros((nx, nz), int)
    i2 = np.zeros((nx, nz), int)
    for iz in range(nz):
        for r in range(nref):
            vref32[r, iz] = (vmin[iz] + f32(r) * (vmax[iz] - vmin[iz]) / (f32(nref) - f32(1))) if nref > 1 else vmin[iz]
            lo, hi = float(vmin[iz]), float(vmax[iz])  # float64 (NumPy keeps float32 for mixed scalars)
            vref64[r, iz] = (lo + r * (hi - lo) / (nref - 1)) if nref > 1 else lo
        if vmax[iz] > vmin[iz] + f32(10):
            ir = (f32(nref - 1) * (vel[:, iz] - vmin[iz]) / (vmax[iz] - vmin[iz])).astype(np.int64)
            ir = np.maximum(ir, 0)
            a = ir.copy()
            b = ir + 1
            top = ir > nref - 2
            a[top] = nref - 1
            b[top] = nref - 1
            i1[:, iz], i2[:, iz] = a, b
    return po, pd, vref32, vref64, i1, i2


def _taper(nx):
    lmx = 30 if nx > 100 else 0
    t = np.ones(nx)
    for i in range(nx):
        if i < lmx:
            t[i] = np.exp(-(0.015 * (lmx - i)) ** 2)
        elif i > nx - lmx:
            t[i] = np.exp(-(0.015 * (i - nx + lmx)) ** 2)
    return t


def _kz_phase(w, slow2, kx, dz):
    s = w * w * slow2 - kx * kx
    out = np.empty(s.shape, complex)
    pos = s >= 0
    out[pos] = np.exp(1j * np.sqrt(s[pos]) * dz)
    out[~pos] = np.exp(-0.2 * np.sqrt(-s[~pos]) * abs(dz))
    return out


def wem(p, vel, wav, d=None, m=None, adj=True):
    """2-D (nmy = 1) operator in FP64. vel [nx, nz]; d [nx, nt]; m [nx, nz]."""
    nx, nz = vel.shape
    nt = int(p["nt"])
    # scalar inputs reach the C operator as float32 (wem.h:3-11); use the same values
    dt = float(f32(p["dt"]))
    dx, dz = float(f32(p["dmx"])), float(f32(p["dz"]))
    oz, sz, gz = float(f32(p.get("oz", 0.0))), float(f32(p.get("sz", 0.0))), float(f32(p.get("gz", 0.0)))
    pspi = int(p.get("pspi", 1))
    interp = p.get("interp", 0)
    interp = {"ref": 0, "linear": 1}.get(interp, interp)
    nkx = int(p["padx"]) * nx if nx > 1 else 1
    ntfft, nw, ifmin, ifmax = _grid(p)
    po, pd, vref32, vref64, i1, i2 = _tables(p, vel)
    kx = 2 * np.pi * np.fft.fftfreq(nkx, d=dx)
    taper = _taper(nx)
    igx = int(f32(int(f32(p["sx"]) - f32(p.get("omx", 0.0)))) / f32(dx))
    dw = 2 * np.pi / ntfft / dt
    wavf = np.fft.rfft(np.asarray(wav, float), ntfft)
    xs_all = np.zeros((nx, nw), complex)
    xs_all[igx] = wavf
    if adj:
        D = np.fft.rfft(np.asarray(d, float), ntfft, axis=1)
        w_all = np.arange(nw) * dw
        xg_all = np.where((np.arange(nw) >= ifmin) & (np.arange(nw) < ifmax), w_all ** 2, 0)[None, :] * D
        image = np.zeros((nx, nz))
    else:
        dg = np.zeros((nx, nw), complex)

    def step(u, w, dzs, iz, adj_op):
        if pspi:
            a = np.zeros(nkx, complex)
            a[:nx] = u
            A = np.fft.fft(a)
            nref = vref64.shape[0]
            dref = np.empty((nref, nx), complex)
            for r in range(nref):
                P = _kz_phase(w, 1.0 / vref64[r, iz] ** 2, kx, dzs)
                dref[r] = np.fft.ifft(A * P)[:nx]
            out = np.empty(nx, complex)
            for ix in range(nx):
                a1, b1 = i1[ix, iz], i2[ix, iz]
                if vref32[b1, iz] - vref32[a1, iz] > 10.0:
                    if interp == 1:
                        t = (float(vel[ix, iz]) - vref64[a1, iz]) / (vref64[b1, iz] - vref64[a1, iz])
                        out[ix] = dref[a1, ix] + (dref[b1, ix] - dref[a1, ix]) * t
                    else:
                        out[ix] = dref[a1, ix].real
                else:
                    out[ix] = dref[a1, ix]
            return out
        corr = np.exp(1j * w * pd[:, iz] * dzs)
        if not adj_op:
            u = u * taper
            u = u * corr
        a = np.zeros(nkx, complex)
        a[:nx] = u
        b = np.fft.ifft(np.fft.fft(a) * _kz_phase(w, po[iz] ** 2, kx, dzs))[:nx]
        if adj_op:
            b = b * corr * taper
        return b

    zs = oz + dz * np.arange(nz)
    for iw in range(ifmin, ifmax):
        w = iw * dw
        us = xs_all[:, iw] / np.sqrt(ntfft)
        if adj:
            factor = 1.0 if iw == 0 else 2.0
            ug = xg_all[:, iw] / np.sqrt(ntfft)
            for iz in range(nz):
                if zs[iz] >= sz:
                    us = step(us, w, -dz, iz, True)
                if zs[iz] >= gz:
                    ug = step(ug, w, dz, iz, True)
                    image[:, iz] += factor * (ug * np.conj(us)).real
        else:
            smig = np.zeros((nx, nz), complex)
            for iz in range(nz):
                if zs[iz] >= sz:
                    us = step(us, w, -dz, iz, True)
                    smig[:, iz] = us
            ug = np.zeros(nx, complex)
            for iz in range(nz - 1, -1, -1):
                if zs[iz] >= gz:
                    ug = ug + m[:, iz] * smig[:, iz]
                    ug = step(ug, w, -dz, iz, False)
            dg[:, iw] = ug / np.sqrt(ntfft)
    if adj:
        return image
    W = np.zeros(nw)
    W[ifmin:ifmax] = (np.arange(ifmin, ifmax) * dw) ** 2
    spec = dg * W[None, :]
    n = (nw - 1) * 2
    full = np.zeros((nx, n), complex)
    full[:, :nw] = spec
    full[:, nw:] = np.conj(spec[:, 1:n - nw + 1][:, ::-1])
    full[:, 0] = full[:, 0].real
    if n % 2 == 0:
        full[:, n // 2] = full[:, n // 2].real
    return (np.fft.ifft(full, axis=1).real * n)[:, :nt]
