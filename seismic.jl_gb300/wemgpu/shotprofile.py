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


def data_layout(g: dict, sx, sy, nt: int, dt: float, ot: float):
    """Trace headers and extent of modelled data: every shot recorded on every grid cell,
    shot after shot, receiver (gx, gy) = cell position, offsets hx, hy, keyed by sx, sy (the
    data files of ShotProfileWEM.jl:291-302, ShotProfileEWEM.jl:366-377). Returns the
    arguments of seis.write after the data."""
    n = g["nmx"] * g["nmy"]
    hd = seis.empty_headers(len(sx) * n)
    imx = np.repeat(np.arange(g["nmx"]), g["nmy"])
    imy = np.tile(np.arange(g["nmy"]), g["nmx"])
    mx, my = g["omx"] + g["dmx"] * imx, g["omy"] + g["dmy"] * imy
    for i, (x0, y0) in enumerate(zip(sx, sy)):
        q = hd[i * n:(i + 1) * n]
        q["tracenum"] = np.arange(1, n + 1) + i * n
        q["n1"], q["d1"], q["o1"] = nt, dt, ot
        q["sx"], q["sy"] = x0, y0
        q["gx"], q["gy"], q["mx"], q["my"] = mx, my, mx, my
        q["hx"], q["hy"] = mx - x0, my - y0
        q["imx"], q["imy"] = imx, imy
    nsx = len(sx)
    return (hd, [nt, g["nmx"], g["nmy"], nsx, 1], [ot, g["omx"], g["omy"], sx[0], sy[0]],
            [dt, g["dmx"], g["dmy"], (sx[1] - sx[0]) if nsx > 1 else 1.0, 1.0],
            ["Time", "gx", "gy", "sx", "sy"], ["s", "m", "m", "m", "m"])


# --------------------------------------------------------------------------- angles

def ComputeAngles(angx: str, angy: str, dip_flag=False, vel="vel", wav="wav", sz=0.0, fmin=0, fmax=80,
                  verbose=False, sx=(0.0,), sy=(0.0,), dipx="dipx", dipy="dipy", device=0,
                  ctx: Context | None = None):
    """Source-side incidence angles of every shot into the seis files angx and angy:
    Seismic.jl's ComputeAngles (src/Imaging/ComputeAngles.jl:55-100) over the GPU's
    wem_angles (compute_angles, src/Imaging/c/wem.c:566-684). Each shot's section has the
    velocity's trace headers with sx set (compute_angles.c:66-69); sections follow each
    other in shot order. dip_flag adds the dip sections of dipx/dipy
    (compute_angles.c:83-96)."""
    velv, hv, g = grid_from_velocity(vel)
    w, hw, ew = seis.read(wav)
    nt, dt, ot = int(hw[0]["n1"]), float(hw[0]["d1"]), float(hw[0]["o1"])
    sx = [float(v) for v in np.atleast_1d(sx)]
    sy = [float(v) for v in np.atleast_1d(sy)]
    if len(sy) == 1 and len(sx) > 1:
        sy = sy * len(sx)
    params = dict(nt=nt, ot=ot, dt=dt, nmx=g["nmx"], omx=g["omx"], dmx=g["dmx"], nmy=g["nmy"], omy=g["omy"],
                  dmy=g["dmy"], nz=g["nz"], oz=g["oz"], dz=g["dz"], sz=sz, fmin=fmin, fmax=fmax,
                  verbose=int(bool(verbose)))
    own = ctx is None
    ctx = ctx or Context(device)
    try:
        ax, ay = ctx.angles(params, velv, w[0], sx, sy)
    finally:
        if own:
            ctx.close()
    if dip_flag:
        ax = ax + seis.read(dipx)[0][None]
        ay = ay + seis.read(dipy)[0][None]
    n = g["nmx"] * g["nmy"]
    hs = []
    for i, x0 in enumerate(sx):
        h = hv.copy()
        h["sx"] = x0
        h["tracenum"] = np.arange(1, n + 1) + i * n
        hs.append(h)
    hh = np.concatenate(hs)
    # one section per shot along the 4th axis, so that the file's extent counts every trace
    ns = len(sx)
    ext = ([g["nz"], g["nmx"], g["nmy"], ns, 1], [g["oz"], g["omx"], g["omy"], sx[0], 0.0],
           [g["dz"], g["dmx"], g["dmy"], (sx[1] - sx[0]) if ns > 1 else 1.0, 1.0])
    seis.write(angx, ax.reshape(len(sx) * n, g["nz"]), hh, *ext)
    seis.write(angy, ay.reshape(len(sx) * n, g["nz"]), hh, *ext)
    return ax, ay


def angle_bins(ax, ay, nangx, oangx, dangx, nangy, oangy, dangy):
    """Bins and bilinear weights of every sample's angles (ShotProfileWEM.jl:161-176)."""
    ax = np.asarray(ax, np.float64)
    ay = np.asarray(ay, np.float64)
    iangx = np.floor((ax - oangx) / dangx).astype(np.int64) + 1
    iangy = np.floor((ay - oangy) / dangy).astype(np.int64) + 1
    angx1 = (iangx - 1) * dangx + oangx
    angx2 = angx1 + dangx
    angy1 = (iangy - 1) * dangy + oangy
    angy2 = angy1 + dangy
    den = (angx2 - angx1) * (angy2 - angy1)
    w1 = (angx2 - ax) * (angy2 - ay) / den
    w2 = (ax - angx1) * (angy2 - ay) / den
    w3 = (angx2 - ax) * (ay - angy1) / den
    w4 = (ax - angx1) * (ay - angy1) / den
    valid = (iangx >= 1) & (iangx <= nangx) & (iangy >= 1) & (iangy <= nangy)
    return iangx, iangy, (w1, w2, w3, w4), valid


def _bin_terms(iangx, iangy, w, valid, nangx, nangy):
    """(weight, bin index, mask) of the four bilinear terms; the last term's guard is
    iangx < nangx (ShotProfileWEM.jl:264-266; the adjoint side's `iang < nang` names no
    defined variable, :183, and is read as the same guard)."""
    b1 = (iangx - 1) * nangy + (iangy - 1)
    terms = [(w[0], b1, valid), (w[1], b1 + nangy, valid & (iangx < nangx))]
    if nangy > 1:
        terms += [(w[2], b1 + 1, valid), (w[3], b1 + nangy + 1, valid & (iangx < nangx))]
    return terms


def bin_shot(img, ax, ay, out, nangx, oangx, dangx, nangy, oangy, dangy):
    """Adds one shot's image [n, nz] into the angle gathers out [n, nangx*nangy, nz]
    (ShotProfileWEM.jl:155-188)."""
    iangx, iangy, w, valid = angle_bins(ax, ay, nangx, oangx, dangx, nangy, oangy, dangy)
    n, nz = img.shape
    cell = np.repeat(np.arange(n), nz).reshape(n, nz)
    z = np.tile(np.arange(nz), n).reshape(n, nz)
    for wk, b, ok in _bin_terms(iangx, iangy, w, valid, nangx, nangy):
        np.add.at(out, (cell[ok], b[ok], z[ok]), wk[ok] * img[ok])
    return out


def unbin_shot(gath, ax, ay, nangx, oangx, dangx, nangy, oangy, dangy):
    """One shot's image [n, nz] from the angle gathers gath [n, nangx*nangy, nz] at its
    own incidence angles (ShotProfileWEM.jl:246-270)."""
    iangx, iangy, w, valid = angle_bins(ax, ay, nangx, oangx, dangx, nangy, oangy, dangy)
    n, nb, nz = gath.shape
    cell = np.repeat(np.arange(n), nz).reshape(n, nz)
    z = np.tile(np.arange(nz), n).reshape(n, nz)
    img = np.zeros((n, nz))
    for wk, b, ok in _bin_terms(iangx, iangy, w, valid, nangx, nangy):
        bb = np.clip(b, 0, nb - 1)
        img += np.where(ok, wk * gath[cell, bb, z], 0.0)
    return img


def _shot_angles(name: str, x0: float, y0: float, n: int, nz: int) -> np.ndarray:
    """The section of the shot at (x0, y0) in an angle file written by ComputeAngles
    (SeisWindow by sx, sy: ShotProfileWEM.jl:93-97)."""
    a, h, e = seis.read(name)
    sel = np.nonzero((h["sx"] == np.float32(x0)) & (h["sy"] == np.float32(y0)))[0]
    if len(sel) != n:
        raise ValueError(f"{name}: {len(sel)} traces for the shot at sx={x0}, sy={y0}, need {n}")
    return a[sel].reshape(n, nz)


def gather_headers(g: dict, dz: float, nangx, oangx, dangx, nangy, oangy, dangy):
    """Trace headers of the angle-gather image (ShotProfileWEM.jl:115-137): one trace per
    (imx, imy, iangx, iangy), angles fastest."""
    nb = nangx * nangy
    base = image_headers(g, dz)
    h = np.repeat(base, nb)
    ia = np.tile(np.repeat(np.arange(nangx), nangy), len(base))
    iz = np.tile(np.tile(np.arange(nangy), nangx), len(base))
    h["tracenum"] = np.arange(1, len(h) + 1) + 1
    h["iang"] = ia
    h["ang"] = ia * dangx + oangx
    h["iaz"] = iz
    h["az"] = iz * dangy + oangy
    return h


def ShotProfileWEM(m: str, d: str, adj: bool = True, *, pspi=True, nref=5, damping=1000.0, vel="vel",
                   angx="angx", angy="angy", wav="wav", sz=0.0, gz=0.0, nangx=1, oangx=0, dangx=1, nangy=1,
                   oangy=0, dangy=1, fmin=0, fmax=80, padt=2, padx=2, verbose=False, sx=(0.0,), sy=(0.0,),
                   interp="ref", device=0, ctx: Context | None = None):
    """Migration (adj=True: data file d -> image file m) or demigration (adj=False:
    image file m -> data file d) of the shots at (sx[i], sy[i]). Keyword names and
    defaults of ShotProfileWEM.jl:39; `damping` is accepted and unused, as there
    (shotwem.c never reads it)."""
    gathers = nangx != 1 or nangy != 1
    abin = (nangx, float(oangx), float(dangx), nangy, float(oangy), float(dangy))
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
        n = g["nmx"] * g["nmy"]
        if adj and gathers:
            # angle gathers: every shot's image binned by its own incidence angles
            data, hd, ed = seis.read(d)
            out = np.zeros((n, nangx * nangy, g["nz"]))
            for x0, y0 in zip(sx, sy):
                img = ctx.migrate(window_shots(data, hd, [x0], [y0], g)).astype(np.float64)
                ax = _shot_angles(angx, x0, y0, n, g["nz"])
                ay = _shot_angles(angy, x0, y0, n, g["nz"])
                bin_shot(img, ax, ay, out, *abin)
            h = gather_headers(g, g["dz"], *abin)
            seis.write(m, out.reshape(n * nangx * nangy, g["nz"]).astype(np.float32), h,
                       [g["nz"], g["nmx"], g["nmy"], nangx, nangy], [g["oz"], g["omx"], g["omy"], oangx, oangy],
                       [g["dz"], g["dmx"], g["dmy"], dangx, dangy],
                       labels=["Depth", "mx", "my", "angx", "angy"], units=["m", "m", "m", "degrees", "degrees"])
            return out
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
        shots = Shots(np.asarray(sx, np.float32), np.asarray(sy, np.float32), np.arange(len(sx) + 1, dtype=np.int64) * n,
                      np.tile(np.arange(n, dtype=np.int32), len(sx)), np.zeros((0, nt), np.float32))
        if gathers:
            # each shot sees the gathers at its own incidence angles (ShotProfileWEM.jl:228-270)
            gath = img.reshape(n, nangx * nangy, g["nz"]).astype(np.float64)
            parts = []
            for i, (x0, y0) in enumerate(zip(sx, sy)):
                ax = _shot_angles(angx, x0, y0, n, g["nz"])
                ay = _shot_angles(angy, x0, y0, n, g["nz"])
                im = unbin_shot(gath, ax, ay, *abin).astype(np.float32)
                one = Shots(shots.sx[i:i + 1], shots.sy[i:i + 1], np.array([0, n], np.int64),
                            np.arange(n, dtype=np.int32), np.zeros((0, nt), np.float32))
                parts.append(ctx.model(one, im, exact=False))
            data = np.concatenate(parts)
        else:
            data = ctx.model(shots, img[:n], exact=False)
        seis.write(d, data, *data_layout(g, sx, sy, nt, dt, ot))
        return data
    finally:
        if own:
            ctx.close()


# --------------------------------------------------------------------------- elastic

def _signs(ax, ay):
    """signf(angx) * signf(angy) of ShotProfileEWEM.jl:434-438 (-1 below zero, else +1),
    the factor the S images carry into and out of the angle gathers."""
    return np.where(np.asarray(ax) < 0, -1.0, 1.0) * np.where(np.asarray(ay) < 0, -1.0, 1.0)


def _full_grid(data: np.ndarray, hd: np.ndarray, sx, sy, g: dict) -> np.ndarray:
    """Every shot's traces placed on the full receiver grid [nshot, n, nt] by (gx, gy)
    (SeisWindow by sx, sy: ShotProfileEWEM.jl:91-95), zeros where a cell has no trace."""
    n = g["nmx"] * g["nmy"]
    shots = window_shots(data, hd, sx, sy, g)
    out = np.zeros((len(sx), n, data.shape[1]), np.float32)
    for s in range(len(sx)):
        lo, hi = int(shots.trace_offset[s]), int(shots.trace_offset[s + 1])
        out[s, shots.trace_cell[lo:hi]] = shots.data[lo:hi]
    return out


def ShotProfileEWEM(m, d, adj: bool = True, *, damping=1000.0, vp="vp.seis", vs="vs.seis", angx="angx.seis",
                    angy="angy.seis", wav="wav.seis", sz=0.0, gz=0.0, nangx=1, oangx=0, dangx=1, nangy=1, oangy=0,
                    dangy=1, fmin=0, fmax=80, padt=1, padx=1, verbose=False, sx=(0.0,), sy=(0.0,), device=0):
    """Elastic migration (adj=True: data files d = [ux, uy, uz] -> image files m = [mpp, mps1,
    mps2]) or demigration (adj=False: m -> d) of the shots at (sx[i], sy[i]): the interface of
    Seismic.jl's ShotProfileEWEM (src/Imaging/ShotProfileEWEM.jl:38), keyword names and
    defaults included (`damping` is accepted and unused, as there). All shots go to the GPU in
    one wem_elastic call (per shot where angle gathers need each shot's image); with
    nangx, nangy > 1 the shot images are binned by the shot's incidence angles (the angx/angy
    files of ComputeAngles), the S images with the sign of the angles (ShotProfileEWEM.jl:
    155-230, 290-350). 2-D and 3-D grids; mps1 and uy are written as zeros (the separation has no S1
    potential, ewem.c:553-741). Differences, where the reference is ill-defined: traces are
    placed on the grid by their gx/gy headers, and the modelled traces carry gx = ox + dx*imx
    (the reference's per-shot images carry mx = dx*imx, ShotProfileEWEM.jl:274, which
    shotewem.c copies into gx: the same unless the grid starts at ox = 0)."""
    from .api import elastic
    gathers = nangx != 1 or nangy != 1
    abin = (nangx, float(oangx), float(dangx), nangy, float(oangy), float(dangy))
    vpv, hv, g = grid_from_velocity(vp)
    vsv, _, _ = seis.read(vs)
    w, hw, ew = seis.read(wav)
    nt, dt, ot = int(hw[0]["n1"]), float(hw[0]["d1"]), float(hw[0]["o1"])
    sx = [float(v) for v in np.atleast_1d(sx)]
    sy = [float(v) for v in np.atleast_1d(sy)]
    if len(sy) == 1 and len(sx) > 1:
        sy = sy * len(sx)
    n, nz, nb = g["nmx"] * g["nmy"], g["nz"], nangx * nangy
    params = dict(nt=nt, ot=ot, dt=dt, nmx=g["nmx"], omx=g["omx"], dmx=g["dmx"], nmy=g["nmy"], omy=g["omy"],
                  dmy=g["dmy"], nz=nz, oz=g["oz"], dz=g["dz"], gz=gz, sz=sz, fmin=fmin, fmax=fmax, padt=padt,
                  padx=padx, verbose=int(bool(verbose)))
    vpv, vsv = vpv[:n], vsv[:n]
    ext = ([nz, g["nmx"], g["nmy"], nangx, nangy], [g["oz"], g["omx"], g["omy"], oangx, oangy],
           [g["dz"], g["dmx"], g["dmy"], dangx, dangy])
    labels = dict(labels=["Depth", "mx", "my", "angx", "angy"], units=["m", "m", "m", "degrees", "degrees"])
    if adj:
        (ux, hx, _), (uz, hz, _) = seis.read(d[0]), seis.read(d[2])
        ux, uz = _full_grid(ux, hx, sx, sy, g), _full_grid(uz, hz, sx, sy, g)
        if not gathers:
            mpp, mps2 = elastic(params, vpv, vsv, w[0], sx, sy, ux=ux, uz=uz, adj=True, device=device)
            out = [mpp.astype(np.float64)[:, None], np.zeros((n, 1, nz)), mps2.astype(np.float64)[:, None]]
        else:
            out = [np.zeros((n, nb, nz)) for _ in range(3)]
            for i, (x0, y0) in enumerate(zip(sx, sy)):
                mpp, mps2 = elastic(params, vpv, vsv, w[0], [x0], [y0], ux=ux[i:i + 1], uz=uz[i:i + 1], adj=True,
                                    device=device)
                ax = _shot_angles(angx, x0, y0, n, nz)
                ay = _shot_angles(angy, x0, y0, n, nz)
                sg = _signs(ax, ay)
                bin_shot(mpp.astype(np.float64), ax, ay, out[0], *abin)
                bin_shot(sg * mps2, ax, ay, out[2], *abin)
        h = gather_headers(g, g["dz"], *abin)
        for name, a in zip(m, out):
            seis.write(name, a.reshape(n * nb, nz).astype(np.float32), h, *ext, **labels)
        return tuple(a.reshape(n, nb, nz) if gathers else a.reshape(n, nz) for a in out)
    # demigration: every shot recorded on every grid cell
    imgs = [seis.read(name)[0] for name in (m[0], m[2])]
    if not gathers:
        ux, uz = elastic(params, vpv, vsv, w[0], sx, sy, mpp=imgs[0][:n], mps2=imgs[1][:n], adj=False, device=device)
    else:
        gp, gs = (a.reshape(n, nb, nz).astype(np.float64) for a in imgs)
        ux, uz = np.zeros((len(sx), n, nt), np.float32), np.zeros((len(sx), n, nt), np.float32)
        for i, (x0, y0) in enumerate(zip(sx, sy)):
            ax = _shot_angles(angx, x0, y0, n, nz)
            ay = _shot_angles(angy, x0, y0, n, nz)
            ip = unbin_shot(gp, ax, ay, *abin).astype(np.float32)
            is2 = (_signs(ax, ay) * unbin_shot(gs, ax, ay, *abin)).astype(np.float32)
            a, b = elastic(params, vpv, vsv, w[0], [x0], [y0], mpp=ip, mps2=is2, adj=False, device=device)
            ux[i], uz[i] = a[0], b[0]
    layout = data_layout(g, sx, sy, nt, dt, ot)
    comps = (ux.reshape(-1, nt), np.zeros((len(sx) * n, nt), np.float32), uz.reshape(-1, nt))
    for name, a in zip(d, comps):
        seis.write(name, a, *layout)
    return ux, uz


# --------------------------------------------------------------------------- least squares

def _cost_writer(name: str):
    """The cost file of the file-level ConjugateGradients (src/Solvers/ConjugateGradients.jl:
    41-80): a first line with the start time, then cost[0] = 1 and one normalised cost per
    iteration, one number per line. Returns the per-iteration callback."""
    import time
    with open(name, "w") as f:
        f.write("began execution at: " + time.strftime("%a %b %d %H:%M:%S %Y") + "\n")
        f.write("1.0\n")

    def cb(it, m, cost):
        with open(name, "a") as f:
            f.write(repr(float(cost)) + "\n")
    return cb


def _live_traces(shots: Shots) -> Shots:
    """The traces CalculateSampling keeps (energy above 1e-10, CalculateSampling.jl:1-18): the
    others have weight 0, i.e. they take no part in the least-squares problem."""
    from .cg import trace_weights
    keep = trace_weights(shots.data) > 0
    offs = [0]
    for s in range(shots.nshot):
        lo, hi = int(shots.trace_offset[s]), int(shots.trace_offset[s + 1])
        offs.append(offs[-1] + int(keep[lo:hi].sum()))
    return Shots(shots.sx, shots.sy, np.asarray(offs, np.int64), shots.trace_cell[keep], shots.data[keep])


def ShotProfileLSWEM(m: str, m0: str, d: str, param=None, ctx: Context | None = None):
    """Least-squares shot-profile migration over seis files: the interface of Seismic.jl's
    ShotProfileLSWEM(m, m0, d, param) (src/Imaging/ShotProfileLSWEM.jl:1-20): ConjugateGradients
    over [ApplyDataWeights, SeisMute, ShotProfileWEM] with the sampling of the data as weights and
    the mute off (tmute = 0, vmute = 999999). param holds ShotProfileWEM's keywords (vel, wav,
    sx, sy, nref, pspi, fmin, fmax, padt, padx, sz, gz, interp) and the solver's Niter (10), mu
    (0), tol (1e-15) and cost (the cost file, "cost"); exact=True takes the exact adjoint of the
    migration as the forward operator instead of the reference's Born operator. m0 is accepted
    and unused, as there (the file-level CG starts from m = 0, ConjugateGradients.jl:55-57). The
    traces go to the GPU once per operator application (one batched call each way). Writes the
    image file m and returns (image, cost)."""
    from .cg import conjugate_gradients
    q = dict(param or {})
    vel, wav = q.get("vel", "vel"), q.get("wav", "wav")
    velv, hv, g = grid_from_velocity(vel)
    w, hw, ew = seis.read(wav)
    nt, dt, ot = int(hw[0]["n1"]), float(hw[0]["d1"]), float(hw[0]["o1"])
    sx = [float(v) for v in np.atleast_1d(q.get("sx", [0.0]))]
    sy = [float(v) for v in np.atleast_1d(q.get("sy", [0.0]))]
    if len(sy) == 1 and len(sx) > 1:
        sy = sy * len(sx)
    params = dict(nt=nt, ot=ot, dt=dt, nmx=g["nmx"], omx=g["omx"], dmx=g["dmx"], nmy=g["nmy"], omy=g["omy"],
                  dmy=g["dmy"], nz=g["nz"], oz=g["oz"], dz=g["dz"], gz=q.get("gz", 0.0), sz=q.get("sz", 0.0),
                  nref=q.get("nref", 5), fmin=q.get("fmin", 0), fmax=q.get("fmax", 80), padt=q.get("padt", 2),
                  padx=q.get("padx", 2), pspi=int(bool(q.get("pspi", True))), interp=q.get("interp", "ref"))
    data, hd, ed = seis.read(d)
    shots = _live_traces(window_shots(data, hd, sx, sy, g))
    own = ctx is None
    ctx = ctx or Context(q.get("device", 0))
    try:
        ctx.prepare(params, velv, w[0])
        exact = bool(q.get("exact", False))
        fwd = lambda mm: ctx.model(shots, np.asarray(mm, np.float32), exact=exact)  # noqa: E731
        adj = lambda r: ctx.migrate(Shots(shots.sx, shots.sy, shots.trace_offset, shots.trace_cell,  # noqa: E731
                                          np.ascontiguousarray(r, np.float32)))
        img, cost = conjugate_gradients(shots.data, fwd, adj, niter=int(q.get("Niter", 10)), mu=q.get("mu", 0.0),
                                        tol=float(q.get("tol", 1.0e-15)), callback=_cost_writer(q.get("cost", "cost")))
    finally:
        if own:
            ctx.close()
    img = np.asarray(img, np.float32)
    seis.write(m, img, image_headers(g, g["dz"]), [g["nz"], g["nmx"], g["nmy"], 1, 1],
               [g["oz"], g["omx"], g["omy"], 0.0, 0.0], [g["dz"], g["dmx"], g["dmy"], 1.0, 1.0],
               labels=["Depth", "mx", "my", "angx", "angy"], units=["m", "m", "m", "degrees", "degrees"])
    return img, cost


def ShotProfileLSEWEM(m, m0, d, param=None):
    """Elastic least-squares migration over seis files: the interface of Seismic.jl's
    ShotProfileLSEWEM(m, m0, d, param) (src/Imaging/ShotProfileLSEWEM.jl:1-19), m = [mpp, mps1,
    mps2] and d = [ux, uy, uz]: ConjugateGradients over [ApplyDataWeights, SeisMute,
    ShotProfileEWEM] (cg.least_squares_elastic). param holds ShotProfileEWEM's keywords (vp, vs,
    wav, sx, sy, sz, gz, fmin, fmax, padt, padx) and the solver's Niter (10), mu (one weight or
    one per image, 0), tol (1e-15) and cost ("cost.txt"). m0 is accepted and unused, as there.
    2-D and 3-D grids; mps1 is written as zeros. Returns (mpp, mps2, cost)."""
    from .cg import least_squares_elastic
    q = dict(param or {})
    vpv, hv, g = grid_from_velocity(q.get("vp", "vp.seis"))
    vsv, _, _ = seis.read(q.get("vs", "vs.seis"))
    w, hw, ew = seis.read(q.get("wav", "wav.seis"))
    nt, dt, ot = int(hw[0]["n1"]), float(hw[0]["d1"]), float(hw[0]["o1"])
    sx = [float(v) for v in np.atleast_1d(q.get("sx", [0.0]))]
    sy = [float(v) for v in np.atleast_1d(q.get("sy", [0.0]))]
    if len(sy) == 1 and len(sx) > 1:
        sy = sy * len(sx)
    n, nz = g["nmx"] * g["nmy"], g["nz"]
    params = dict(nt=nt, ot=ot, dt=dt, nmx=g["nmx"], omx=g["omx"], dmx=g["dmx"], nmy=g["nmy"], omy=g["omy"],
                  dmy=g["dmy"], nz=nz, oz=g["oz"], dz=g["dz"], gz=q.get("gz", 0.0), sz=q.get("sz", 0.0),
                  fmin=q.get("fmin", 0), fmax=q.get("fmax", 80), padt=q.get("padt", 1), padx=q.get("padx", 1))
    (ux, hx, _), (uz, hz, _) = seis.read(d[0]), seis.read(d[2])
    ux, uz = _full_grid(ux, hx, sx, sy, g), _full_grid(uz, hz, sx, sy, g)
    mu = q.get("mu", 0.0)
    mpp, mps2, cost = least_squares_elastic(params, vpv[:n], vsv[:n], w[0], sx, ux, uz, niter=int(q.get("Niter", 10)),
                                            mu=mu if np.ndim(mu) else (mu, mu), tol=float(q.get("tol", 1.0e-15)),
                                            sy=sy, device=q.get("device", 0),
                                            callback=_cost_writer(q.get("cost", "cost.txt")))
    h = gather_headers(g, g["dz"], 1, 0.0, 1.0, 1, 0.0, 1.0)
    ext = ([nz, g["nmx"], g["nmy"], 1, 1], [g["oz"], g["omx"], g["omy"], 0.0, 0.0], [g["dz"], g["dmx"], g["dmy"], 1.0, 1.0])
    for name, a in zip(m, (mpp, np.zeros_like(mpp), mps2)):
        seis.write(name, np.asarray(a, np.float32), h, *ext, labels=["Depth", "mx", "my", "angx", "angy"],
                   units=["m", "m", "m", "degrees", "degrees"])
    return mpp, mps2, cost
