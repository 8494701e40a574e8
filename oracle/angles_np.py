"""Test infrastructure (the oracle): NumPy restatement of the reference's source-side
incidence-angle computation, compute_angles / extrapolate_source / ssop_source /
calculate_derivatives (src/Imaging/c/wem.c:566-992), in float64.

Checked against the reference's own compute_angles() compiled in oracle/_ref
(tests/golden/angles_*.npz, made by tests/golden/make_golden.py). The scalar grid
quantities (frequency band, wavenumbers) follow the reference's float expressions,
rounded to float32, so that the same frequencies and wavenumbers are used.

Nothing outside tests/ and the bench's CPU leg imports this module.
"""
from __future__ import annotations

import numpy as np

f32 = np.float32
PI = 3.141592653589793  # seismic.h:18


def angle_band(nt: int, dt: float, fmin: float, fmax: float):
    """ntfft, nw, ifmin, ifmax of compute_angles (wem.c:589-603): no time padding."""
    ntfft = nt
    nw = ntfft // 2 + 1
    dtf = f32(dt)
    if f32(fmax) * dtf * f32(ntfft) + f32(1) < nw:
        ifmax = int(f32(int(fmax)) * dtf * f32(ntfft) + f32(1))
    else:
        ifmax = nw
    if f32(fmin) * dtf * f32(ntfft) + f32(1) < ifmax:
        ifmin = int(f32(int(fmin)) * dtf * f32(ntfft))
    else:
        ifmin = 0
    return ntfft, nw, ifmin, ifmax


def wavenumbers(n: int, d: float) -> np.ndarray:
    """k of index i (wem.c:802-803, 866-867): dk*i up to n/2, then -(dk*n - dk*i), float."""
    dk = f32(2 * PI / float(f32(n)) / float(f32(d)))  # double expression stored in a float
    i = np.arange(n)
    k = np.where(i <= n // 2, dk * i.astype(f32), -(dk * f32(n) - dk * i.astype(f32)))
    return k.astype(np.float64)


def taper(nm: int) -> np.ndarray:
    """boundary_condition (wem.c:546-564) weights along one axis."""
    lm = 30 if nm > 100 else 0
    t = np.ones(nm)
    for i in range(nm):
        if i < lm:
            t[i] = np.exp(-(0.015 * (lm - i)) ** 2)
        elif i > nm - lm:
            t[i] = np.exp(-(0.015 * (i - nm + lm)) ** 2)
    return t


def compute_angles(p: dict, vel: np.ndarray, wav: np.ndarray, sign_margin: bool = False):
    """angx, angy [nmx*nmy, nz] (float64) of one shot at (p["sx"], p["sy"]).
    vel [nmx*nmy, nz]; wav [nt].
    sign_margin: also return, per point and axis, |sign sum| / (sum of |u|/nw), the
    margin by which the side the energy arrives from is decided (0: undecided)."""
    nt, dt = int(p["nt"]), float(p["dt"])
    nmx, nmy, nz = int(p["nmx"]), int(p.get("nmy", 1)), int(p["nz"])
    dmx, dmy, dz = float(p["dmx"]), float(p.get("dmy", p["dmx"])), float(p["dz"])
    omx, omy, oz = float(p.get("omx", 0.0)), float(p.get("omy", 0.0)), float(p.get("oz", 0.0))
    sz = float(p.get("sz", 0.0))
    ntfft, nw, ifmin, ifmax = angle_band(nt, dt, float(p.get("fmin", 0.0)), float(p.get("fmax", 80.0)))
    dw = f32(2 * PI / float(f32(ntfft)) / float(f32(dt)))
    kx = wavenumbers(nmx, dmx)
    ky = wavenumbers(nmy, dmy)
    kz = wavenumbers(nz, dz)
    v = np.asarray(vel, np.float64).reshape(nmx, nmy, nz)
    po = 1.0 / v.mean(axis=(0, 1))                     # [nz]
    pd = 1.0 / v - po[None, None, :]                   # [nmx, nmy, nz]
    tap = taper(nmx)[:, None] * taper(nmy)[None, :]
    # igx = (int) (sx - omx)/dmx: the cast binds to the difference (wem.c:654-655)
    igx = int(f32(int(f32(p["sx"]) - f32(omx))) / f32(dmx))
    igy = int(f32(int(f32(p.get("sy", 0.0)) - f32(omy))) / f32(dmy))
    # source spectrum (f_op, ntfft = (nw-1)*2 inside it)
    nf_op = (nw - 1) * 2
    wpad = np.zeros(nf_op)
    wpad[:min(nt, nf_op)] = np.asarray(wav, np.float64)[:min(nt, nf_op)]
    dw_src = np.fft.rfft(wpad)[:nw]
    angx = np.zeros((nmx, nmy, nz))
    angy = np.zeros((nmx, nmy, nz))
    sgx = np.zeros((nmx, nmy, nz))
    sgy = np.zeros((nmx, nmy, nz))
    sgw = np.zeros((nmx, nmy, nz))
    KX, KY = np.meshgrid(kx, ky, indexing="ij")
    nk = nmx * nmy
    dzs = -dz  # extrapolate_source passes -dz to ssop_source (wem.c:719)
    for iw in range(ifmin, ifmax):
        w = float(f32(iw) * dw)
        d = np.zeros((nmx, nmy), complex)
        d[igx, igy] = dw_src[iw] / np.sqrt(ntfft)
        us = np.zeros((nmx, nmy, nz), complex)
        for iz in range(nz):
            z = oz + dz * iz
            if z < sz:
                continue
            d = d * tap
            a = d * np.exp(1j * w * pd[:, :, iz] * dzs)
            a = np.fft.fft2(a)
            s = (w * w) * (po[iz] * po[iz]) - KX ** 2 - KY ** 2
            L = np.where(s >= 0, np.exp(1j * np.sqrt(np.abs(s)) * dzs), np.exp(-0.2 * np.sqrt(np.abs(s)) * abs(dzs)))
            d = np.fft.ifft2(a * L / np.sqrt(nk)) * nk / np.sqrt(nk)
            us[:, :, iz] = d
        A = np.fft.fftn(us)
        ikx = 1j * kx[:, None, None]
        iky = 1j * ky[None, :, None]
        ikz = 1j * kz[None, None, :]
        usx = np.fft.ifftn(ikx * A)
        usy = np.fft.ifftn(iky * A)
        usz = np.fft.ifftn(ikz * A)
        half_x = np.arange(nmx) <= nmx // 2
        half_y = np.arange(nmy) <= nmy // 2
        kxl = np.where(half_x, 0.0, kx)[:, None, None]
        kxr = np.where(half_x, kx, 0.0)[:, None, None]
        kyl = np.where(half_y, 0.0, ky)[None, :, None]
        kyr = np.where(half_y, ky, 0.0)[None, :, None]
        ul, ur = np.abs(np.fft.ifftn(1j * kxl * A)), np.abs(np.fft.ifftn(1j * kxr * A))
        sgx += np.where(ul >= ur, 1.0, -1.0) * np.abs(us) / nw
        ul, ur = np.abs(np.fft.ifftn(1j * kyl * A)), np.abs(np.fft.ifftn(1j * kyr * A))
        sgy += np.where(ul >= ur, 1.0, -1.0) * np.abs(us) / nw
        sgw += np.abs(us) / nw
        angx += (180 / PI) * np.arctan(np.abs(usx) / (np.abs(usz) + 1e-10))
        angy += (180 / PI) * np.arctan(np.abs(usy) / (np.abs(usz) + 1e-10))
    nfreq = ifmax - ifmin + 1  # wem.c:676 divides by ifmax - ifmin + 1
    angx *= np.where(sgx >= 0, 1.0, -1.0) / nfreq
    angy *= np.where(sgy >= 0, 1.0, -1.0) / nfreq
    if sign_margin:
        with np.errstate(invalid="ignore", divide="ignore"):
            mx = np.where(sgw > 0, np.abs(sgx) / sgw, 0.0)
            my = np.where(sgw > 0, np.abs(sgy) / sgw, 0.0)
        return (angx.reshape(nmx * nmy, nz), angy.reshape(nmx * nmy, nz),
                mx.reshape(nmx * nmy, nz), my.reshape(nmx * nmy, nz))
    return angx.reshape(nmx * nmy, nz), angy.reshape(nmx * nmy, nz)
