"""oracle/ewem_np.py -- TEST INFRASTRUCTURE (CPU oracle), never the product path.

FP64 NumPy restatement of the reference's elastic shot-profile migration and its forward
operator, src/Imaging/c/ewem.c (2-D: nmy = 1, the case its separation handles):

  * ewem()               ewem.c:3-253   grids, slowness split, spectra, frequency loop, synthesis
  * elastic_extrap1f()   ewem.c:255-366 source continued down (ssop, -dz, kept per depth over
                                        max_source); receiver: separate -> ssop(P, vp) and
                                        ssop(S, vs) -> recombine; imaging of P and S2
  * elastic_separate_3d  ewem.c:553-741 components (ux, uz) <-> potentials (P, S2) per kx
  * ssop()               ewem.c:368-456 split-step with ewem's own conventions (cexpf, taper
                                        recomputed per call, kx sign by ikx < nkx/2.)
  * boundary_condition   ewem.c:533-551

Only the integer decisions (ntfft, ifmin, ifmax, igx) follow the reference's float
expressions; everything else is double. The y component and mps1 are zero on both sides
(the reference's separation leaves them out, ewem.c:579-587, 628-634).
"""
from __future__ import annotations

import math

import numpy as np

f32 = np.float32


def grids(p: dict):
    """ntfft, nw, ifmin, ifmax, nkx of ewem.c:44-57 (float expressions)."""
    nt, padt, padx, nmx = int(p["nt"]), int(p.get("padt", 1)), int(p.get("padx", 1)), int(p["nmx"])
    dt, fmin, fmax = f32(p["dt"]), f32(p.get("fmin", 0.0)), f32(p.get("fmax", 80.0))
    ntfft = int(2 * math.trunc(float(f32(f32(padt) * f32(nt)) / f32(2))))
    nw = int(math.trunc(ntfft // 2)) + 1
    nkx = padx * nmx if nmx > 1 else 1
    prod = f32(fmax * dt * f32(ntfft))
    ifmax = int(math.trunc(float(prod))) + 1 if prod + f32(1) < nw else nw
    prodn = f32(fmin * dt * f32(ntfft))
    ifmin = int(math.trunc(float(prodn))) if prodn + f32(1) < ifmax else 0
    return ntfft, nw, ifmin, ifmax, nkx


def taper(nmx: int) -> np.ndarray:
    """boundary_condition's weights (ewem.c:533-551), lmx = 30 when nmx > 100."""
    lmx = 30 if nmx > 100 else 0
    t = np.ones(nmx)
    for i in range(nmx):
        if i < lmx:
            t[i] = math.exp(-(0.015 * (lmx - i)) ** 2)
        elif i > nmx - lmx:
            t[i] = math.exp(-(0.015 * (i - nmx + lmx)) ** 2)
    return t


def kx_signed(nkx: int, dkx: float) -> np.ndarray:
    """kx = ikx < nkx/2. ? dkx*ikx : -(dkx*nkx - dkx*ikx) (ewem.c:414, 614)."""
    i = np.arange(nkx)
    return np.where(i < nkx / 2.0, dkx * i, -(dkx * nkx - dkx * i))


def ssop(d, w, kx, nkx, po, pd, dz, tap, adj):
    """ewem.c:368-456 on one row (nmx samples) of depth iz: po the layer slowness, pd the
    row's slowness perturbations."""
    nmx = len(d)
    a = np.zeros(nkx, complex)
    if adj:
        a[:nmx] = d
    else:
        d = d * tap
        a[:nmx] = d * np.exp(1j * w * pd * dz)
    A = np.fft.fft(a)
    s = (w * w) * (po * po) - kx * kx
    L = np.where(s >= 0, np.exp(1j * np.sqrt(np.abs(s)) * dz), np.exp(-0.2 * np.sqrt(np.abs(s)) * abs(dz)))
    b = np.fft.ifft(A * L / math.sqrt(nkx)) * nkx
    if adj:
        return b[:nmx] * np.exp(1j * w * pd * dz) / math.sqrt(nkx) * tap
    return b[:nmx] / math.sqrt(nkx)


def separation(w, kx, vp, vs):
    """The per-kx quantities of elastic_separate_3d (ewem.c:596-611): kxp, kzp, kxs, kzs, norm
    and the mask where the potentials are separated (norm >= 0.1 and w >= 20)."""
    sp = w * w / (vp * vp) - kx * kx
    ss = w * w / (vs * vs) - kx * kx
    kzp = np.where(sp > 0, np.sqrt(np.abs(sp)), 0.0)
    kzs = np.where(ss > 0, np.sqrt(np.abs(ss)), 0.0)
    with np.errstate(divide="ignore", invalid="ignore"):
        norm_p = np.sqrt(kx * kx + kzp * kzp)
        norm_s = np.sqrt(kx * kx + kzs * kzs)
        kxp, kxs = kx / norm_p, kx / norm_s
        kzp, kzs = kzp / norm_p, kzs / norm_s
        norm = kxp * kxs + kzp * kzs
        on = (norm >= 0.1) & (w >= 20.0)  # NaN compares false, as in C
    return kxp, kzp, kxs, kzs, norm, on


def separate(ux, uz, w, kx, nkx, vp, vs, adj):
    """Components -> potentials (P, S2), ewem.c:574-660."""
    nmx = len(ux)
    a = np.zeros(nkx, complex)
    a[:nmx] = ux
    uxk = np.fft.fft(a) / math.sqrt(nkx)
    a = np.zeros(nkx, complex)
    a[:nmx] = uz
    uzk = np.fft.fft(a) / math.sqrt(nkx)
    kxp, kzp, kxs, kzs, norm, on = separation(w, kx, vp, vs)
    with np.errstate(invalid="ignore", divide="ignore"):
        if adj:
            upk = kxp * uxk + kzp * uzk
            usk = -kzs * uxk + kxs * uzk
        else:
            upk = (kxs * uxk + kzs * uzk) / norm
            usk = (-kzp * uxk + kxp * uzk) / norm
    upk = np.where(on, upk, uzk)
    usk = np.where(on, usk, uxk)
    up = np.fft.ifft(upk)[:nmx] * nkx / math.sqrt(nkx)
    us = np.fft.ifft(usk)[:nmx] * nkx / math.sqrt(nkx)
    return up, us


def combine(up, us, w, kx, nkx, vp, vs, adj):
    """Potentials (P, S2) -> components (ux, uz), ewem.c:662-730."""
    nmx = len(up)
    a = np.zeros(nkx, complex)
    a[:nmx] = up
    upk = np.fft.fft(a) / math.sqrt(nkx)
    a = np.zeros(nkx, complex)
    a[:nmx] = us
    usk = np.fft.fft(a) / math.sqrt(nkx)
    kxp, kzp, kxs, kzs, norm, on = separation(w, kx, vp, vs)
    with np.errstate(invalid="ignore", divide="ignore"):
        if not adj:
            uxk = kxp * upk - kzs * usk
            uzk = kzp * upk + kxs * usk
        else:
            uxk = (kxs * upk - kzp * usk) / norm
            uzk = (kzs * upk + kxp * usk) / norm
    uxk = np.where(on, uxk, usk)
    uzk = np.where(on, uzk, upk)
    ux = np.fft.ifft(uxk)[:nmx] * nkx / math.sqrt(nkx)
    uz = np.fft.ifft(uzk)[:nmx] * nkx / math.sqrt(nkx)
    return ux, uz


def ewem(p: dict, vp, vs, wav, ux=None, uz=None, mpp=None, mps2=None, adj: bool = True):
    """One shot. vp, vs [nmx, nz]; ux, uz [nmx, nt] (adj) or mpp, mps2 [nmx, nz] (forward).
    Returns (mpp, mps1, mps2) or (ux, uy, uz) in float64 (mps1, uy zero)."""
    nmx, nz, nt = int(p["nmx"]), int(p["nz"]), int(p["nt"])
    assert int(p.get("nmy", 1)) == 1
    ntfft, nw, ifmin, ifmax, nkx = grids(p)
    dmx, dz, dt = float(p["dmx"]), float(p["dz"]), float(p["dt"])
    dkx = float(f32(2 * math.pi / f32(nkx) / f32(dmx)))
    dw = float(f32(2 * math.pi / f32(ntfft) / f32(dt)))
    kx = kx_signed(nkx, dkx)
    vp = np.asarray(vp, np.float64).reshape(nmx, nz)
    vs = np.asarray(vs, np.float64).reshape(nmx, nz)
    po_p = 1.0 / vp.mean(axis=0)
    po_s = 1.0 / vs.mean(axis=0)
    pd_p = 1.0 / vp - po_p[None, :]
    pd_s = 1.0 / vs - po_s[None, :]
    tap = taper(nmx)
    igx = int(math.trunc(float(f32((f32(p["sx"]) - f32(p.get("omx", 0.0))) / f32(dmx)))))
    w0 = np.zeros(ntfft)
    w0[:nt] = np.asarray(wav, np.float64)[:nt]
    W = np.fft.rfft(w0)[:nw]
    max_source = np.max(np.abs(np.asarray(wav, np.float64)[:nt])) / math.sqrt(ntfft)
    oz, sz, gz = float(p.get("oz", 0.0)), float(p.get("sz", 0.0)), float(p.get("gz", 0.0))
    zs = [oz + dz * iz for iz in range(nz)]
    if adj:
        dx = np.zeros((nmx, ntfft))
        dx[:, :nt] = np.asarray(ux, np.float64)
        dzz = np.zeros((nmx, ntfft))
        dzz[:, :nt] = np.asarray(uz, np.float64)
        UX = np.fft.rfft(dx, axis=1)[:, :nw]
        UZ = np.fft.rfft(dzz, axis=1)[:, :nw]
        m_pp = np.zeros((nmx, nz))
        m_s2 = np.zeros((nmx, nz))
    else:
        UXo = np.zeros((nmx, nw), complex)
        UZo = np.zeros((nmx, nw), complex)
        mpp = np.asarray(mpp, np.float64)
        mps2 = np.asarray(mps2, np.float64)
    for iw in range(ifmin, ifmax):
        factor = 1.0 if iw == 0 else 2.0
        w = iw * dw
        src = np.zeros(nmx, complex)
        src[igx] = W[iw] / math.sqrt(ntfft)
        smig = np.zeros((nmx, nz), complex)
        for iz in range(nz):
            if zs[iz] >= sz:
                src = ssop(src, w, kx, nkx, po_p[iz], pd_p[:, iz], -dz, tap, True)
                smig[:, iz] = src / max_source
        if adj:
            gx = UX[:, iw] / math.sqrt(ntfft)
            gzr = UZ[:, iw] / math.sqrt(ntfft)
            for iz in range(nz):
                if zs[iz] >= gz:
                    vpi, vsi = 1.0 / po_p[iz], 1.0 / po_s[iz]
                    up, us = separate(gx, gzr, w, kx, nkx, vpi, vsi, True)
                    up = ssop(up, w, kx, nkx, po_p[iz], pd_p[:, iz], dz, tap, True)
                    us = ssop(us, w, kx, nkx, po_s[iz], pd_s[:, iz], dz, tap, True)
                    gx, gzr = combine(up, us, w, kx, nkx, vpi, vsi, True)
                    m_pp[:, iz] += factor * np.real(np.conj(smig[:, iz]) * up)
                    m_s2[:, iz] += factor * np.real(np.conj(smig[:, iz]) * us)
        else:
            gx = np.zeros(nmx, complex)
            gzr = np.zeros(nmx, complex)
            for iz in range(nz - 1, -1, -1):
                if zs[iz] >= gz:
                    vpi, vsi = 1.0 / po_p[iz], 1.0 / po_s[iz]
                    up, us = separate(gx, gzr, w, kx, nkx, vpi, vsi, False)
                    up = up + smig[:, iz] * mpp[:, iz]
                    us = us + smig[:, iz] * mps2[:, iz]
                    up = ssop(up, w, kx, nkx, po_p[iz], pd_p[:, iz], -dz, tap, False)
                    us = ssop(us, w, kx, nkx, po_s[iz], pd_s[:, iz], -dz, tap, False)
                    gx, gzr = combine(up, us, w, kx, nkx, vpi, vsi, False)
            UXo[:, iw] = gx / math.sqrt(ntfft)
            UZo[:, iw] = gzr / math.sqrt(ntfft)
    if adj:
        return m_pp, np.zeros((nmx, nz)), m_s2
    nf = (nw - 1) * 2

    def synth(U):
        full = np.zeros((nmx, nf // 2 + 1), complex)
        full[:, :nw] = U
        return np.fft.irfft(full, nf, axis=1)[:, :nt] * nf
    return synth(UXo), np.zeros((nmx, nt)), synth(UZo)


# ------------------------------------------------------------------ 3-D grids (nmy > 1)
# The same operator on (x, y) planes with the reference's rank-2 transforms (ewem.c:84-96):
# the separation and recombination use kx alone, broadcast over ky (ewem.c:596-611, 680-695);
# ssop's phase uses kx and ky (ewem.c:412-421); boundary_condition tapers both axes.

def _pad2(d, nkx, nky):
    a = np.zeros((nkx, nky), complex)
    a[:d.shape[0], :d.shape[1]] = d
    return a


def ssop3(d, w, kx, ky, nkx, nky, po, pd, dz, tap, adj):
    """ewem.c:368-456 on one plane [nmx, nmy] of depth iz."""
    nmx, nmy = d.shape
    s_ = math.sqrt(nkx * nky)
    if adj:
        a = _pad2(d, nkx, nky)
    else:
        d = d * tap
        a = _pad2(d * np.exp(1j * w * pd * dz), nkx, nky)
    A = np.fft.fft2(a)
    s = (w * w) * (po * po) - kx[:, None] ** 2 - ky[None, :] ** 2
    L = np.where(s >= 0, np.exp(1j * np.sqrt(np.abs(s)) * dz), np.exp(-0.2 * np.sqrt(np.abs(s)) * abs(dz)))
    b = np.fft.ifft2(A * L / s_) * (nkx * nky)
    if adj:
        return b[:nmx, :nmy] * np.exp(1j * w * pd * dz) / s_ * tap
    return b[:nmx, :nmy] / s_


def _mix3(a0, a1, w, kx, nkx, nky, vp, vs, adj, sep):
    nmx, nmy = a0.shape
    s_ = math.sqrt(nkx * nky)
    k0 = np.fft.fft2(_pad2(a0, nkx, nky)) / s_
    k1 = np.fft.fft2(_pad2(a1, nkx, nky)) / s_
    kxp, kzp, kxs, kzs, norm, on = (q[:, None] for q in separation(w, kx, vp, vs))
    with np.errstate(invalid="ignore", divide="ignore"):
        if sep:
            if adj:
                o0, o1 = kxp * k0 + kzp * k1, -kzs * k0 + kxs * k1
            else:
                o0, o1 = (kxs * k0 + kzs * k1) / norm, (-kzp * k0 + kxp * k1) / norm
        else:
            if not adj:
                o0, o1 = kxp * k0 - kzs * k1, kzp * k0 + kxs * k1
            else:
                o0, o1 = (kxs * k0 - kzp * k1) / norm, (kzs * k0 + kxp * k1) / norm
    o0 = np.where(on, o0, k1)
    o1 = np.where(on, o1, k0)
    b0 = np.fft.ifft2(o0) * (nkx * nky) / s_
    b1 = np.fft.ifft2(o1) * (nkx * nky) / s_
    return b0[:nmx, :nmy], b1[:nmx, :nmy]


def ewem3d(p: dict, vp, vs, wav, ux=None, uz=None, mpp=None, mps2=None, adj: bool = True):
    """One shot on a 3-D grid. vp, vs [nmx*nmy, nz] (cell = imx*nmy + imy); ux, uz [nmx*nmy, nt]
    (adj) or mpp, mps2 [nmx*nmy, nz] (forward). Returns (mpp, mps1, mps2) or (ux, uy, uz) in
    float64 (mps1, uy zero)."""
    nmx, nmy, nz, nt = int(p["nmx"]), int(p["nmy"]), int(p["nz"]), int(p["nt"])
    nn = nmx * nmy
    ntfft, nw, ifmin, ifmax, nkx = grids(p)
    nky = int(p.get("padx", 1)) * nmy
    dmx, dmy, dz, dt = float(p["dmx"]), float(p["dmy"]), float(p["dz"]), float(p["dt"])
    dkx = float(f32(2 * math.pi / f32(nkx) / f32(dmx)))
    dky = float(f32(2 * math.pi / f32(nky) / f32(dmy)))
    dw = float(f32(2 * math.pi / f32(ntfft) / f32(dt)))
    kx, ky = kx_signed(nkx, dkx), kx_signed(nky, dky)
    vp = np.asarray(vp, np.float64).reshape(nn, nz)
    vs = np.asarray(vs, np.float64).reshape(nn, nz)
    po_p = 1.0 / vp.mean(axis=0)
    po_s = 1.0 / vs.mean(axis=0)
    pd_p = (1.0 / vp - po_p[None, :]).reshape(nmx, nmy, nz)
    pd_s = (1.0 / vs - po_s[None, :]).reshape(nmx, nmy, nz)
    tap = taper(nmx)[:, None] * taper(nmy)[None, :]
    igx = int(math.trunc(float(f32((f32(p["sx"]) - f32(p.get("omx", 0.0))) / f32(dmx)))))
    igy = int(math.trunc(float(f32((f32(p["sy"]) - f32(p.get("omy", 0.0))) / f32(dmy)))))
    w0 = np.zeros(ntfft)
    w0[:nt] = np.asarray(wav, np.float64)[:nt]
    W = np.fft.rfft(w0)[:nw]
    max_source = np.max(np.abs(np.asarray(wav, np.float64)[:nt])) / math.sqrt(ntfft)
    oz, sz, gz = float(p.get("oz", 0.0)), float(p.get("sz", 0.0)), float(p.get("gz", 0.0))
    zs = [oz + dz * iz for iz in range(nz)]
    if adj:
        def spec(u):
            d = np.zeros((nn, ntfft))
            d[:, :nt] = np.asarray(u, np.float64)
            return np.fft.rfft(d, axis=1)[:, :nw].reshape(nmx, nmy, nw)
        UX, UZ = spec(ux), spec(uz)
        m_pp = np.zeros((nmx, nmy, nz))
        m_s2 = np.zeros((nmx, nmy, nz))
    else:
        UXo = np.zeros((nmx, nmy, nw), complex)
        UZo = np.zeros((nmx, nmy, nw), complex)
        mpp = np.asarray(mpp, np.float64).reshape(nmx, nmy, nz)
        mps2 = np.asarray(mps2, np.float64).reshape(nmx, nmy, nz)
    for iw in range(ifmin, ifmax):
        factor = 1.0 if iw == 0 else 2.0
        w = iw * dw
        src = np.zeros((nmx, nmy), complex)
        src[igx, igy] = W[iw] / math.sqrt(ntfft)
        smig = np.zeros((nmx, nmy, nz), complex)
        for iz in range(nz):
            if zs[iz] >= sz:
                src = ssop3(src, w, kx, ky, nkx, nky, po_p[iz], pd_p[:, :, iz], -dz, tap, True)
                smig[:, :, iz] = src / max_source
        if adj:
            gx = UX[:, :, iw] / math.sqrt(ntfft)
            gzr = UZ[:, :, iw] / math.sqrt(ntfft)
            for iz in range(nz):
                if zs[iz] >= gz:
                    vpi, vsi = 1.0 / po_p[iz], 1.0 / po_s[iz]
                    up, us = _mix3(gx, gzr, w, kx, nkx, nky, vpi, vsi, True, True)
                    up = ssop3(up, w, kx, ky, nkx, nky, po_p[iz], pd_p[:, :, iz], dz, tap, True)
                    us = ssop3(us, w, kx, ky, nkx, nky, po_s[iz], pd_s[:, :, iz], dz, tap, True)
                    gx, gzr = _mix3(up, us, w, kx, nkx, nky, vpi, vsi, True, False)
                    m_pp[:, :, iz] += factor * np.real(np.conj(smig[:, :, iz]) * up)
                    m_s2[:, :, iz] += factor * np.real(np.conj(smig[:, :, iz]) * us)
        else:
            gx = np.zeros((nmx, nmy), complex)
            gzr = np.zeros((nmx, nmy), complex)
            for iz in range(nz - 1, -1, -1):
                if zs[iz] >= gz:
                    vpi, vsi = 1.0 / po_p[iz], 1.0 / po_s[iz]
                    up, us = _mix3(gx, gzr, w, kx, nkx, nky, vpi, vsi, False, True)
                    up = up + smig[:, :, iz] * mpp[:, :, iz]
                    us = us + smig[:, :, iz] * mps2[:, :, iz]
                    up = ssop3(up, w, kx, ky, nkx, nky, po_p[iz], pd_p[:, :, iz], -dz, tap, False)
                    us = ssop3(us, w, kx, ky, nkx, nky, po_s[iz], pd_s[:, :, iz], -dz, tap, False)
                    gx, gzr = _mix3(up, us, w, kx, nkx, nky, vpi, vsi, False, False)
            UXo[:, :, iw] = gx / math.sqrt(ntfft)
            UZo[:, :, iw] = gzr / math.sqrt(ntfft)
    if adj:
        return m_pp.reshape(nn, nz), np.zeros((nn, nz)), m_s2.reshape(nn, nz)
    nf = (nw - 1) * 2

    def synth(U):
        full = np.zeros((nn, nf // 2 + 1), complex)
        full[:, :nw] = U.reshape(nn, nw)
        return np.fft.irfft(full, nf, axis=1)[:, :nt] * nf
    return synth(UXo), np.zeros((nn, nt)), synth(UZo)
