"""File-level shot-profile migration / demigration: the interface of Seismic.jl's
`ShotProfileWEM(m, d, adj; ...)` (src/Imaging/ShotProfileWEM.jl:39) over seis files.

The reference windows the data into one file per shot (SeisWindow, :101-103), runs one
`shotwem` process per shot (:104-106, :288-290) and stacks the shot images through files
(:140-199). Here every shot goes to the GPU in one batched call (`wem_migrate` /
`wem_model`), and the image or the data is written once. Angle gathers (nangx, nangy > 1)
are not part of this path; with nangx = nangy = 1 the reference's bilinear binning puts
every sample in bin 1 with weight 1, which is what this does.

Differences, all where the reference is ill-defined:
  * traces are placed on the grid by their receiver position (gx, gy) headers; the
    reference's main() assumes each per-shot file holds the full grid in cell order
    (shotwem.c:70-74), which the two agree on for such files;
  * the shot images are summed on the GPU (compensated FP32) instead of in Float32
    read-add-write order.
"""
from __future__ import annotations

import numpy as np

from . import seis
from .api import Context, Shots


def grid_from_velocity(vel_name: str):
    """The grid of ShotProfileWEM.jl:42-55 (nx, ny from the imx/imy span of the velocity
    headers; ox = mx of the first trace; dx from the first two; dy = dx in 2-D)."""
    v, h, ext = seis.read(vel_name)
    nx = int(h[-1]["imx"] - h[0]["imx"] + 1)
    ny = int(h[-1]["imy"] - h[0]["imy"] + 1)
    ox = float(h[0]["mx"])
    dx = float(h[1]["mx"] - h[0]["mx"]) if len(h) > 1 else 1.0
    oy = float(h[0]["my"])
    dy = float(h[nx]["my"] - oy) if ny > 1 else dx
    g = dict(nmx=nx, omx=ox, dmx=dx, nmy=ny, omy=oy, dmy=dy, nz=int(h[0]["n1"]), dz=float(h[0]["d1"]),
             oz=float(h[0]["o1"]), min_imx=int(h[0]["imx"]), min_imy=int(h[0]["imy"]))
    return v, h, g


def window_shots(d: np.ndarray, h: np.ndarray, sx, sy, g: dict):
    """SeisWindow(d, key=["sx","sy"], minval=maxval=[sx_i, sy_i]) for every shot, in
    compact form: the traces of shot i and their grid cells from (gx, gy)."""
    offs = [0]
    cells, datas = [], []
    for x0, y0 in zip(sx, sy):
        sel = np.nonzero((h["sx"] == np.float32(x0)) & (h["sy"] == np.float32(y0)))[0]
        ix = np.rint((h["gx"][sel] - g["omx"]) / g["dmx"]).astype(np.int64)
        iy = np.rint((h["gy"][sel] - g["omy"]) / g["dmy"]).astype(np.int64) if g["nmy"] > 1 else np.zeros(len(sel), np.int64)
        ok = (ix >= 0) & (ix < g["nmx"]) & (iy >= 0) & (iy < g["nmy"])
        sel, ix, iy = sel[ok], ix[ok], iy[ok]
        cells.append((ix * g["nmy"] + iy).astype(np.int32))
        datas.append(d[sel])
        offs.append(offs[-1] + len(sel))
    nt = d.shape[1]
    return Shots(np.asarray(sx, np.float32), np.asarray(sy, np.float32), np.asarray(offs, np.int64),
                 np.concatenate(cells) if cells else np.zeros(0, np.int32),
                 np.concatenate(datas) if datas else np.zeros((0, nt), np.float32))


def image_headers(g: dict, dz: float):
    """Trace headers of the stacked image (ShotProfileWEM.jl:115-137, nangx=nangy=1):
    mx = dx*imx, my = dy*imy with the velocity's imx/imy numbering."""
    n = g["nmx"] * g["nmy"]
    h = seis.empty_headers(n)
    imx = np.repeat(np.arange(g["nmx"]), g["nmy"]) + g["min_imx"]
    imy = np.tile(np.arange(g["nmy"]), g["nmx"]) + g["min_imy"]
    h["tracenum"] = np.arange(1, n + 1) + 1
    h["o1"] = 0.0
    h["n1"] = g["nz"]
    h["d1"] = dz
    h["imx"] = imx
    h["imy"] = imy
    h["mx"] = g["dmx"] * imx
    h["my"] = g["dmy"] * imy
    return h


def ShotProfileWEM(m: str, d: str, adj: bool = True, *, pspi=True, nref=5, damping=1000.0, vel="vel",
                   angx="angx", angy="angy", wav="wav", sz=0.0, gz=0.0, nangx=1, oangx=0, dangx=1, nangy=1,
                   oangy=0, dangy=1, fmin=0, fmax=80, padt=2, padx=2, verbose=False, sx=(0.0,), sy=(0.0,),
                   interp="ref", device=0, ctx: Context | None = None):
    """Migration (adj=True: data file d -> image file m) or demigration (adj=False:
    image file m -> data file d) of the shots at (sx[i], sy[i]). Keyword names and
    defaults of ShotProfileWEM.jl:39; `damping` is accepted and unused, as there
    (shotwem.c never reads it)."""
    if nangx != 1 or nangy != 1:
        raise NotImplementedError("angle gathers (nangx, nangy > 1) are outside this path")
    velv, hv, g = grid_from_velocity(vel)
    w, hw, ew = seis.read(wav)
    nt, dt, ot = int(hw[0]["n1"]), float(hw[0]["d1"]), float(hw[0]["o1"])
    sx = [float(v) for v in np.atleast_1d(sx)]
    sy = [float(v) for v in np.atleast_1d(sy)]
    if len(sy) == 1 and len(sx) > 1:
        sy = sy * len(sx)
    params = dict(nt=nt, ot=ot, dt=dt, nmx=g["nmx"], omx=g["omx"], dmx=g["dmx"], nmy=g["nmy"], omy=g["omy"],
                  dmy=g["dmy"], nz=g["nz"], oz=g["oz"], dz=g["dz"], gz=gz, sz=sz, nref=nref, fmin=fmin,
                  fmax=fmax, padt=padt, padx=padx, pspi=int(bool(pspi)), interp=interp,
                  verbose=int(bool(verbose)))
    own = ctx is None
    ctx = ctx or Context(device)
    try:
        ctx.prepare(params, velv, w[0])
        if adj:
            data, hd, ed = seis.read(d)
            shots = window_shots(data, hd, sx, sy, g)
            image = ctx.migrate(shots)
            ext_n = [g["nz"], g["nmx"], g["nmy"], nangx, nangy]
            ext_o = [g["oz"], g["omx"], g["omy"], oangx, oangy]
            ext_d = [g["dz"], g["dmx"], g["dmy"], dangx, dangy]
            seis.write(m, image, image_headers(g, g["dz"]), ext_n, ext_o, ext_d,
                       labels=["Depth", "mx", "my", "angx", "angy"], units=["m", "m", "m", "degrees", "degrees"])
            return image
        # demigration: every shot recorded on every grid cell (ShotProfileWEM.jl:210-309)
        img, hm, em = seis.read(m)
        n = g["nmx"] * g["nmy"]
        shots = Shots(np.asarray(sx, np.float32), np.asarray(sy, np.float32), np.arange(len(sx) + 1, dtype=np.int64) * n,
                      np.tile(np.arange(n, dtype=np.int32), len(sx)), np.zeros((0, nt), np.float32))
        data = ctx.model(shots, img[:n], exact=False)
        hd = seis.empty_headers(len(sx) * n)
        mx = g["omx"] + g["dmx"] * np.repeat(np.arange(g["nmx"]), g["nmy"])
        my = g["omy"] + g["dmy"] * np.tile(np.arange(g["nmy"]), g["nmx"])
        for i, (x0, y0) in enumerate(zip(sx, sy)):
            q = hd[i * n:(i + 1) * n]
            q["tracenum"] = np.arange(1, n + 1) + i * n
            q["n1"], q["d1"], q["o1"] = nt, dt, ot
            q["sx"], q["sy"] = x0, y0
            q["gx"], q["gy"], q["mx"], q["my"] = mx, my, mx, my
            q["hx"], q["hy"] = mx - x0, my - y0
            q["imx"] = np.repeat(np.arange(g["nmx"]), g["nmy"])
            q["imy"] = np.tile(np.arange(g["nmy"]), g["nmx"])
        nsx = len(sx)
        seis.write(d, data, hd, [nt, g["nmx"], g["nmy"], nsx, 1], [ot, g["omx"], g["omy"], sx[0], sy[0]],
                   [dt, g["dmx"], g["dmy"], (sx[1] - sx[0]) if nsx > 1 else 1.0, 1.0],
                   labels=["Time", "gx", "gy", "sx", "sy"], units=["s", "m", "m", "m", "m"])
        return data
    finally:
        if own:
            ctx.close()
