"""Seeded synthetic surveys for the migration workloads (no external data).

Wavelet: Ricker, as src/Wavelets/Ricker.jl:21-28 (nw = 2/(f0 dt) samples,
t = dt*(-nc:nc), w = (1 - 2b) e^{-b}, b = (pi f0 t)^2), placed at the start of an
nt-sample trace (peak at nc*dt). Data: point diffractors, each trace the wavelet
delayed by the straight-ray traveltime source -> point -> receiver, amplitudes
U(0.5, 1). The cost of the migration does not depend on the data content.

Workloads (seed = 1000 + index):
  0  split-step, 3 flat layers 1500/2200/3000 m/s (interfaces at iz=67, 134),
     nz=200 x nx=256, 10 m; one shot at x=1280 m; nt=1000, dt=2 ms; 5-60 Hz
  1  PSPI, Gaussian random-field velocity (sigma 200 m, mean 3000, std 400 m/s,
     clipped to [1500, 4500]) nz=500 x nx=1024, 10 m; 64 shots, apertures
     U{200..800} traces centred on the source; nt=1500; 5-50 Hz; nref=8
  3  3-D PSPI, smooth random field in [1500, 4000] m/s, nz=300 x 256 x 256 at 12.5 m;
     one shot at the centre, 256 x 256 receivers; nt=2000; 3-60 Hz; nref=6
  4  PSPI, dipping layers 1500..3500 m/s, nz=300 x nx=512, 10 m; 32 shots with
     256..512 receivers; nt=1500; 5-45 Hz; nref=8
"""
from __future__ import annotations

import numpy as np
from scipy.ndimage import gaussian_filter

from .api import Shots


def ricker(f0: float, dt: float) -> np.ndarray:
    nw = 2.0 / (f0 * dt)
    nc = int(np.floor(nw / 2))
    t = dt * np.arange(-nc, nc + 1)
    b = (np.pi * f0 * t) ** 2
    return ((1 - 2 * b) * np.exp(-b)).astype(np.float32)


def wavelet_trace(nt: int, dt: float, f0: float = 20.0) -> np.ndarray:
    w = ricker(f0, dt)
    out = np.zeros(nt, np.float32)
    out[: min(nt, len(w))] = w[: min(nt, len(w))]
    return out


def _layer_time(zp, L, z_if, v_layers):
    """Straight-ray time over a segment of length L from the surface to depth zp
    through flat layers (interfaces z_if, velocities v_layers)."""
    zp = np.maximum(zp, 1e-6)
    t = np.zeros(np.broadcast(zp, L).shape)
    tops = np.concatenate([[0.0], z_if])
    bots = np.concatenate([z_if, [np.inf]])
    for top, bot, v in zip(tops, bots, v_layers):
        frac = np.clip(np.minimum(zp, bot) - top, 0, None) / zp
        t = t + frac * L / v
    return t


def diffraction_gather(xs_rec, sx, points, amps, nt, dt, wav, traveltime):
    """Sum of delayed wavelets for every receiver x; traveltime(sx, px, pz, xr)."""
    nr = len(xs_rec)
    spikes = np.zeros((nr, nt), np.float64)
    t0 = 0.0
    for (px, pz), a in zip(points, amps):
        tau = traveltime(sx, px, pz, xs_rec) + t0
        f = tau / dt
        i0 = np.floor(f).astype(np.int64)
        w1 = f - i0
        ok = (i0 >= 0) & (i0 + 1 < nt)
        r = np.nonzero(ok)[0]
        np.add.at(spikes, (r, i0[ok]), a * (1 - w1[ok]))
        np.add.at(spikes, (r, i0[ok] + 1), a * w1[ok])
    # convolve with the wavelet (causal: the wavelet's own delay stays)
    n = 1 << int(np.ceil(np.log2(nt + len(wav))))
    W = np.fft.rfft(wav.astype(np.float64), n)
    out = np.fft.irfft(np.fft.rfft(spikes, n, axis=1) * W[None, :], n, axis=1)[:, :nt]
    return out.astype(np.float32)


def config0(seed: int = 1000):
    rng = np.random.default_rng(seed)
    nx, nz, dx, dz, nt, dt = 256, 200, 10.0, 10.0, 1000, 0.002
    v_layers = np.array([1500.0, 2200.0, 3000.0])
    z_if = np.array([67 * dz, 134 * dz])
    vel = np.empty((nx, nz), np.float32)
    vel[:, :67] = 1500.0
    vel[:, 67:134] = 2200.0
    vel[:, 134:] = 3000.0
    wav = wavelet_trace(nt, dt)
    sx = 1280.0
    xs = np.arange(nx) * dx
    pts = np.stack([rng.uniform(0, 2550, 10), rng.uniform(200, 1990, 10)], 1)
    amps = rng.uniform(0.5, 1.0, 10)

    def tt(sx_, px, pz, xr):
        return (_layer_time(pz, np.hypot(px - sx_, pz), z_if, v_layers) +
                _layer_time(pz, np.hypot(xr - px, pz), z_if, v_layers))

    d = diffraction_gather(xs, sx, pts, amps, nt, dt, wav, tt)
    params = dict(nt=nt, ot=0.0, dt=dt, nmx=nx, omx=0.0, dmx=dx, nz=nz, oz=0.0, dz=dz, sx=sx,
                  fmin=5.0, fmax=60.0, padt=2, padx=2, pspi=0, nref=5)
    shots = Shots.full_grid([sx], d[None])
    return dict(name="2-D split-step, 1 shot, nz=200 x nx=256", params=params, vel=vel, wav=wav, shots=shots)


def grf_velocity(rng, nx, nz, sigma, mean, std, lo, hi):
    g = gaussian_filter(rng.standard_normal((nx, nz)), sigma, mode="reflect")
    g = (g - g.mean()) / g.std()
    return np.clip(mean + std * g, lo, hi).astype(np.float32)


def survey_shots(rng, nx, dx, sxs, ap_lo, ap_hi, nt, dt, wav, points, amps, vmean):
    xs_all = np.arange(nx) * dx
    offs = [0]
    cells = []
    datas = []

    def tt(sx_, px, pz, xr):
        return (np.hypot(px - sx_, pz) + np.hypot(xr - px, pz)) / vmean

    for sx in sxs:
        ap = int(rng.integers(ap_lo, ap_hi + 1))
        c = int(round(sx / dx))
        lo = max(0, c - ap // 2)
        hi = min(nx, lo + ap)
        cell = np.arange(lo, hi, dtype=np.int32)
        d = diffraction_gather(xs_all[lo:hi], sx, points, amps, nt, dt, wav, tt)
        cells.append(cell)
        datas.append(d)
        offs.append(offs[-1] + len(cell))
    return Shots(np.asarray(sxs, np.float32), np.zeros(len(sxs), np.float32), np.asarray(offs, np.int64),
                 np.concatenate(cells).astype(np.int32), np.concatenate(datas).astype(np.float32))


def config1(seed: int = 1001, nshot: int = 64, nx: int = 1024, nz: int = 500, nt: int = 1500,
            fmax: float = 50.0, npoints: int = 60):
    rng = np.random.default_rng(seed)
    dx = dz = 10.0
    dt = 0.002
    vel = grf_velocity(rng, nx, nz, 20.0, 3000.0, 400.0, 1500.0, 4500.0)
    wav = wavelet_trace(nt, dt)
    width = nx * dx
    sxs = (np.arange(nshot) + 0.5) * (width / nshot)
    pts = np.stack([rng.uniform(0, width - dx, npoints), rng.uniform(200, nz * dz - 10, npoints)], 1)
    amps = rng.uniform(0.5, 1.0, npoints)
    shots = survey_shots(rng, nx, dx, sxs, min(200, nx), min(800, nx), nt, dt, wav, pts, amps, 3000.0)
    params = dict(nt=nt, ot=0.0, dt=dt, nmx=nx, omx=0.0, dmx=dx, nz=nz, oz=0.0, dz=dz,
                  fmin=5.0, fmax=fmax, padt=2, padx=2, pspi=1, nref=8)
    return dict(name=f"2-D PSPI, {nshot} shots, nz={nz} x nx={nx}, nref=8", params=params, vel=vel, wav=wav,
                shots=shots)


def random_reflectivity(seed: int, nx: int, nz: int, density: float = 0.01) -> np.ndarray:
    """Seeded reflectivity [nx, nz]: `density` of the cells nonzero, N(0, 1) amplitudes."""
    rng = np.random.default_rng(seed)
    m = np.zeros((nx, nz), np.float32)
    k = int(round(density * m.size))
    m.flat[rng.choice(m.size, k, replace=False)] = rng.standard_normal(k).astype(np.float32)
    return m


def with_born_data(c: dict, ctx=None, seed: int | None = None, density: float = 0.01) -> dict:
    """The survey c with its traces replaced by Born data of a seeded random reflectivity
    (1 % of the cells, N(0, 1)): the reference's forward operator (wem.c:252-281, adj=false)
    run by the GPU library on every shot's receivers (wem_model, exact=0). The traces keep
    each shot's aperture. c["reflectivity"] holds the model."""
    from .api import Context
    p = c["params"]
    seed = (int(p["nmx"]) * 7919 + int(p["nz"])) if seed is None else seed
    m = random_reflectivity(seed, int(p["nmx"]) * int(p.get("nmy", 1)), int(p["nz"]), density)
    own = ctx is None
    ctx = Context() if own else ctx
    try:
        ctx.prepare(p, c["vel"], c["wav"])
        d = ctx.model(c["shots"], m, exact=False)
    finally:
        if own:
            ctx.close()
    s = c["shots"]
    out = dict(c)
    out["shots"] = Shots(s.sx, s.sy, s.trace_offset, s.trace_cell, np.ascontiguousarray(d, np.float32))
    out["reflectivity"] = m
    out["name"] = c["name"] + ", Born data of a 1 % random reflectivity"
    return out


def dipping_layers(rng, nx, nz, dx, dz, nlayer, vlo, vhi):
    x = np.arange(nx) * dx
    depths = np.sort(rng.uniform(0.1, 0.95, nlayer)) * nz * dz
    dips = np.tan(np.deg2rad(rng.uniform(-15, 15, nlayer)))
    vels = np.linspace(vlo, vhi, nlayer + 1)
    z = np.arange(nz)[None, :] * dz
    vel = np.full((nx, nz), vels[0], np.float32)
    for k in range(nlayer):
        zi = depths[k] + dips[k] * (x - x.mean())
        vel[z >= zi[:, None]] = vels[k + 1]
    return vel


def config4(seed: int = 1004, nshot: int = 32, nx: int = 512, nz: int = 300, nt: int = 1500):
    rng = np.random.default_rng(seed)
    dx = dz = 10.0
    dt = 0.002
    vel = dipping_layers(rng, nx, nz, dx, dz, 6, 1500.0, 3500.0)
    wav = wavelet_trace(nt, dt)
    width = nx * dx
    sxs = (np.arange(nshot) + 0.5) * (width / nshot)
    pts = np.stack([rng.uniform(0, width - dx, 40), rng.uniform(200, nz * dz - 10, 40)], 1)
    amps = rng.uniform(0.5, 1.0, 40)
    shots = survey_shots(rng, nx, dx, sxs, 256, 512, nt, dt, wav, pts, amps, 2500.0)
    params = dict(nt=nt, ot=0.0, dt=dt, nmx=nx, omx=0.0, dmx=dx, nz=nz, oz=0.0, dz=dz,
                  fmin=5.0, fmax=45.0, padt=2, padx=2, pspi=1, nref=8)
    return dict(name=f"2-D PSPI (LSM survey), {nshot} shots, nz={nz} x nx={nx}", params=params, vel=vel,
                wav=wav, shots=shots)


def small_case(seed: int, nx: int = 64, nz: int = 24, nt: int = 128, nshot: int = 3, pspi: int = 1,
               nref: int = 4, interp: str = "ref", fmax: float = 40.0, padx: int = 2, padt: int = 2):
    """Seeded small survey for parity tests (the CPU oracle finishes it in seconds)."""
    rng = np.random.default_rng(seed)
    dx = dz = 10.0
    dt = 0.004
    vel = grf_velocity(rng, nx, nz, 3.0, 2500.0, 300.0, 1500.0, 4500.0)
    wav = wavelet_trace(nt, dt, f0=15.0)
    width = nx * dx
    sxs = (np.arange(nshot) + 0.5) * (width / nshot)
    pts = np.stack([rng.uniform(0, width - dx, 6), rng.uniform(30, nz * dz - 10, 6)], 1)
    amps = rng.uniform(0.5, 1.0, 6)
    shots = survey_shots(rng, nx, dx, sxs, nx // 3, nx, nt, dt, wav, pts, amps, 2500.0)
    params = dict(nt=nt, ot=0.0, dt=dt, nmx=nx, omx=0.0, dmx=dx, nz=nz, oz=0.0, dz=dz,
                  fmin=3.0, fmax=fmax, padt=padt, padx=padx, pspi=pspi, nref=nref, interp=interp)
    return dict(name=f"small seed={seed}", params=params, vel=vel, wav=wav, shots=shots)


def diffraction_gather_3d(xr, yr, sx, sy, points, amps, nt, dt, wav, vmean):
    """Like diffraction_gather for receivers at (xr[i], yr[i]), constant-velocity times."""
    nr = len(xr)
    spikes = np.zeros((nr, nt), np.float64)
    for (px, py, pz), a in zip(points, amps):
        tau = (np.sqrt((px - sx) ** 2 + (py - sy) ** 2 + pz ** 2) +
               np.sqrt((xr - px) ** 2 + (yr - py) ** 2 + pz ** 2)) / vmean
        f = tau / dt
        i0 = np.floor(f).astype(np.int64)
        w1 = f - i0
        ok = (i0 >= 0) & (i0 + 1 < nt)
        r = np.nonzero(ok)[0]
        np.add.at(spikes, (r, i0[ok]), a * (1 - w1[ok]))
        np.add.at(spikes, (r, i0[ok] + 1), a * w1[ok])
    n = 1 << int(np.ceil(np.log2(nt + len(wav))))
    W = np.fft.rfft(wav.astype(np.float64), n)
    return np.fft.irfft(np.fft.rfft(spikes, n, axis=1) * W[None, :], n, axis=1)[:, :nt].astype(np.float32)


def smooth_field_3d(rng, nx, ny, nz, sigma, lo, hi):
    g = gaussian_filter(rng.standard_normal((nx, ny, nz)), sigma, mode="reflect")
    g = (g - g.min()) / (g.max() - g.min())
    return (lo + (hi - lo) * g).astype(np.float32)


def config3(seed: int = 1003, nx: int = 256, ny: int = 256, nz: int = 300, nt: int = 2000, fmax: float = 60.0,
            npoints: int = 50, d: float = 12.5):
    rng = np.random.default_rng(seed)
    dt = 0.002
    vel = smooth_field_3d(rng, nx, ny, nz, 8.0, 1500.0, 4000.0).reshape(nx * ny, nz)
    wav = wavelet_trace(nt, dt)
    sx, sy = (nx // 2) * d, (ny // 2) * d
    pts = np.stack([rng.uniform(0, (nx - 1) * d, npoints), rng.uniform(0, (ny - 1) * d, npoints),
                    rng.uniform(10 * d, (nz - 1) * d, npoints)], 1)
    amps = rng.uniform(0.5, 1.0, npoints)
    gx, gy = np.meshgrid(np.arange(nx) * d, np.arange(ny) * d, indexing="ij")
    data = diffraction_gather_3d(gx.ravel(), gy.ravel(), sx, sy, pts, amps, nt, dt, wav, float(vel.mean()))
    shots = Shots(np.array([sx], np.float32), np.array([sy], np.float32), np.array([0, nx * ny], np.int64),
                  np.arange(nx * ny, dtype=np.int32), data)
    params = dict(nt=nt, ot=0.0, dt=dt, nmx=nx, omx=0.0, dmx=d, nmy=ny, omy=0.0, dmy=d, nz=nz, oz=0.0, dz=d,
                  fmin=3.0, fmax=fmax, padt=2, padx=2, pspi=1, nref=6)
    return dict(name=f"3-D PSPI, 1 shot, nz={nz} x {nx} x {ny}, nref=6", params=params, vel=vel, wav=wav,
                shots=shots)


def small_case3d(seed: int, nx: int = 32, ny: int = 32, nz: int = 10, nt: int = 64, nshot: int = 1, pspi: int = 1,
                 nref: int = 3, interp: str = "ref", fmax: float = 40.0, padx: int = 2):
    """Seeded small 3-D survey; the velocity's minimum of every depth lies on the first
    x-plane (the reference takes vmin over the first nmx traces, wem.c:48-49)."""
    rng = np.random.default_rng(seed)
    d = 10.0
    dt = 0.004
    vel = smooth_field_3d(rng, nx, ny, nz, 2.0, 1800.0, 3200.0)
    vel[0, 0, :] = vel.min(axis=(0, 1)) - 1.0
    vel = vel.reshape(nx * ny, nz)
    wav = wavelet_trace(nt, dt, f0=15.0)
    srcs = [((nx // 2 + 3 * s) * d, (ny // 2 - 2 * s) * d) for s in range(nshot)]
    pts = np.stack([rng.uniform(0, (nx - 1) * d, 4), rng.uniform(0, (ny - 1) * d, 4),
                    rng.uniform(3 * d, (nz - 1) * d, 4)], 1)
    amps = rng.uniform(0.5, 1.0, 4)
    gx, gy = np.meshgrid(np.arange(nx) * d, np.arange(ny) * d, indexing="ij")
    datas = [diffraction_gather_3d(gx.ravel(), gy.ravel(), sx, sy, pts, amps, nt, dt, wav, 2500.0) for sx, sy in srcs]
    shots = Shots(np.array([q[0] for q in srcs], np.float32), np.array([q[1] for q in srcs], np.float32),
                  np.arange(nshot + 1, dtype=np.int64) * nx * ny, np.tile(np.arange(nx * ny, dtype=np.int32), nshot),
                  np.concatenate(datas))
    params = dict(nt=nt, ot=0.0, dt=dt, nmx=nx, omx=0.0, dmx=d, nmy=ny, omy=0.0, dmy=d, nz=nz, oz=0.0, dz=d,
                  fmin=3.0, fmax=fmax, padt=2, padx=padx, pspi=pspi, nref=nref, interp=interp)
    return dict(name=f"small 3-D seed={seed}", params=params, vel=vel, wav=wav, shots=shots)


def shot_gather_full(shots: Shots, s: int, ncell: int) -> np.ndarray:
    """Shot s on the full grid [ncell, nt], zeros where it has no trace (what the
    reference's per-shot files carry, wem.c:122-133)."""
    nt = shots.data.shape[1]
    g = np.zeros((ncell, nt), np.float32)
    lo, hi = int(shots.trace_offset[s]), int(shots.trace_offset[s + 1])
    g[shots.trace_cell[lo:hi]] = shots.data[lo:hi]
    return g
