"""Array-level API over the C ABI: one context per GPU, a survey of many shots per call.

The parameter names are those of the reference's wem() (src/Imaging/c/wem.h:3-11)
and of ShotProfileWEM's keywords (src/Imaging/ShotProfileWEM.jl:39).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L

_f32p = C.POINTER(C.c_float)
_i64p = C.POINTER(C.c_int64)
_i32p = C.POINTER(C.c_int32)


def make_params(**kw) -> L.Params:
    """Defaults follow shotwem.c:27-42 (padt=padx=1, nref=5, fmin=0, fmax=80)."""
    interp = kw.get("interp", "ref")
    prec = kw.get("precision", "fp32")
    p = L.Params(
        nt=int(kw["nt"]), ot=float(kw.get("ot", 0.0)), dt=float(kw["dt"]),
        nmx=int(kw["nmx"]), omx=float(kw.get("omx", 0.0)), dmx=float(kw["dmx"]),
        nmy=int(kw.get("nmy", 1)), omy=float(kw.get("omy", 0.0)), dmy=float(kw.get("dmy", kw["dmx"])),
        nz=int(kw["nz"]), oz=float(kw.get("oz", 0.0)), dz=float(kw["dz"]),
        gz=float(kw.get("gz", 0.0)), sz=float(kw.get("sz", 0.0)),
        nref=int(kw.get("nref", 5)), fmin=float(kw.get("fmin", 0.0)), fmax=float(kw.get("fmax", 80.0)),
        padt=int(kw.get("padt", 1)), padx=int(kw.get("padx", 1)),
        pspi=int(bool(kw.get("pspi", True))),
        interp=L.INTERP[interp] if isinstance(interp, str) else int(interp),
        precision=L.PRECISION[prec] if isinstance(prec, str) else int(prec),
        verbose=int(bool(kw.get("verbose", False))))
    return p


@dataclass
class Shots:
    """A batch of shots in compact form: shot s owns traces
    trace_offset[s]:trace_offset[s+1] of data ([ntrace, nt]); trace i sits on grid
    cell trace_cell[i] (= imx*nmy + imy)."""
    sx: np.ndarray
    sy: np.ndarray
    trace_offset: np.ndarray
    trace_cell: np.ndarray
    data: np.ndarray

    @staticmethod
    def full_grid(sx, data_per_shot, sy=None) -> "Shots":
        """Every shot recorded on every grid cell: data_per_shot [nshot, ncell, nt]."""
        d = np.ascontiguousarray(data_per_shot, dtype=np.float32)
        ns, ncell, nt = d.shape
        off = np.arange(ns + 1, dtype=np.int64) * ncell
        cell = np.tile(np.arange(ncell, dtype=np.int32), ns)
        sx = np.asarray(sx, np.float32)
        sy = np.zeros(ns, np.float32) if sy is None else np.asarray(sy, np.float32)
        return Shots(sx, sy, off, cell, d.reshape(ns * ncell, nt))

    @property
    def nshot(self) -> int:
        return len(self.sx)


class Context:
    """Owns a CUDA stream and device buffers (wem_ctx)."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        L.check(L.lib().wem_ctx_create(C.byref(self._h), int(device)))
        self.params = None

    def close(self):
        if self._h:
            L.lib().wem_ctx_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def prepare(self, params, vel: np.ndarray, wav: np.ndarray):
        p = params if isinstance(params, L.Params) else make_params(**params)
        vel = np.ascontiguousarray(vel, dtype=np.float32)
        wav = np.ascontiguousarray(np.asarray(wav, np.float32).reshape(-1))
        if vel.shape != (p.nmx * p.nmy, p.nz):
            raise ValueError(f"vel must be [nmx*nmy, nz] = {(p.nmx * p.nmy, p.nz)}, got {vel.shape}")
        if wav.size != p.nt:
            raise ValueError("wav must hold nt samples")
        L.check(L.lib().wem_prepare(self._h, C.byref(p), vel.ctypes.data_as(_f32p), wav.ctypes.data_as(_f32p)))
        self.params = p
        return self

    def migrate(self, shots: Shots) -> np.ndarray:
        p = self.params
        if p is None:
            raise RuntimeError("prepare() first")
        d = np.ascontiguousarray(shots.data, dtype=np.float32)
        sx = np.ascontiguousarray(shots.sx, dtype=np.float32)
        sy = np.ascontiguousarray(shots.sy, dtype=np.float32)
        off = np.ascontiguousarray(shots.trace_offset, dtype=np.int64)
        cell = np.ascontiguousarray(shots.trace_cell, dtype=np.int32)
        m = np.empty((p.nmx * p.nmy, p.nz), np.float32)
        L.check(L.lib().wem_migrate(self._h, len(sx), sx.ctypes.data_as(_f32p), sy.ctypes.data_as(_f32p),
                                    off.ctypes.data_as(_i64p), cell.ctypes.data_as(_i32p),
                                    d.ctypes.data_as(_f32p), m.ctypes.data_as(_f32p)))
        return m

    def model(self, shots: Shots, m: np.ndarray, exact: bool = False) -> np.ndarray:
        """Born modelling of the image m [nmx*nmy, nz] at the traces of `shots` (their
        data is ignored); returns [ntrace, nt]. exact=False: the reference's operator;
        exact=True: the exact adjoint of migrate()."""
        p = self.params
        if p is None:
            raise RuntimeError("prepare() first")
        m = np.ascontiguousarray(m, dtype=np.float32)
        if m.shape != (p.nmx * p.nmy, p.nz):
            raise ValueError(f"m must be [nmx*nmy, nz] = {(p.nmx * p.nmy, p.nz)}")
        sx = np.ascontiguousarray(shots.sx, dtype=np.float32)
        sy = np.ascontiguousarray(shots.sy, dtype=np.float32)
        off = np.ascontiguousarray(shots.trace_offset, dtype=np.int64)
        cell = np.ascontiguousarray(shots.trace_cell, dtype=np.int32)
        d = np.empty((int(off[-1]), p.nt), np.float32)
        L.check(L.lib().wem_model(self._h, len(sx), sx.ctypes.data_as(_f32p), sy.ctypes.data_as(_f32p),
                                  off.ctypes.data_as(_i64p), cell.ctypes.data_as(_i32p),
                                  m.ctypes.data_as(_f32p), d.ctypes.data_as(_f32p), int(bool(exact))))
        return d

    def migrate_device(self, shots: Shots, d_dev_ptr: int, m_dev_ptr: int, sync: bool = True):
        """Same, with the trace data and the image already in device memory (raw pointers)."""
        sx = np.ascontiguousarray(shots.sx, dtype=np.float32)
        sy = np.ascontiguousarray(shots.sy, dtype=np.float32)
        off = np.ascontiguousarray(shots.trace_offset, dtype=np.int64)
        cell = np.ascontiguousarray(shots.trace_cell, dtype=np.int32)
        L.check(L.lib().wem_migrate_device(self._h, len(sx), sx.ctypes.data_as(_f32p), sy.ctypes.data_as(_f32p),
                                           off.ctypes.data_as(_i64p), cell.ctypes.data_as(_i32p),
                                           C.c_void_p(d_dev_ptr), C.c_void_p(m_dev_ptr), int(sync)))

    def model_device(self, shots: Shots, m_dev_ptr: int, d_dev_ptr: int, exact: bool = False, sync: bool = True):
        """model() with the image [nmx*nmy, nz] and the traces [ntrace, nt] in device memory
        (raw pointers); the traces of `shots` give the geometry only."""
        sx = np.ascontiguousarray(shots.sx, dtype=np.float32)
        sy = np.ascontiguousarray(shots.sy, dtype=np.float32)
        off = np.ascontiguousarray(shots.trace_offset, dtype=np.int64)
        cell = np.ascontiguousarray(shots.trace_cell, dtype=np.int32)
        L.check(L.lib().wem_model_device(self._h, len(sx), sx.ctypes.data_as(_f32p), sy.ctypes.data_as(_f32p),
                                         off.ctypes.data_as(_i64p), cell.ctypes.data_as(_i32p),
                                         C.c_void_p(m_dev_ptr), C.c_void_p(d_dev_ptr), int(bool(exact)), int(sync)))

    def last_timing(self):
        """(device ms of the last call, kernels it launched)"""
        ms = C.c_float()
        k = C.c_int()
        L.check(L.lib().wem_last_timing(self._h, C.byref(ms), C.byref(k)))
        return ms.value, k.value

    def last_kernel_times(self):
        """device ms of (spectra, depth recursion, image reduction) of the last call"""
        a, b, c = C.c_float(), C.c_float(), C.c_float()
        L.check(L.lib().wem_last_kernel_times(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def angles(self, params, vel: np.ndarray, wav: np.ndarray, sx, sy=None):
        """Source-side incidence angles of the shots at sx (compute_angles, wem.c:566-684)
        on the grid of params (no prepare needed; any nmx, nz): (angx, angy), each
        [nshot, nmx*nmy, nz] float32."""
        p = params if isinstance(params, L.Params) else make_params(**params)
        vel = np.ascontiguousarray(vel, dtype=np.float32)
        wav = np.ascontiguousarray(np.asarray(wav, np.float32).reshape(-1))
        sx = np.ascontiguousarray(np.atleast_1d(sx), dtype=np.float32)
        sy = np.ascontiguousarray(np.zeros_like(sx) if sy is None else np.atleast_1d(sy), dtype=np.float32)
        ax = np.empty((len(sx), p.nmx * p.nmy, p.nz), np.float32)
        ay = np.empty_like(ax)
        L.check(L.lib().wem_angles(self._h, C.byref(p), vel.ctypes.data_as(_f32p), wav.ctypes.data_as(_f32p),
                                   len(sx), sx.ctypes.data_as(_f32p), sy.ctypes.data_as(_f32p),
                                   ax.ctypes.data_as(_f32p), ay.ctypes.data_as(_f32p)))
        return ax, ay

    def last_launch(self) -> dict:
        """How the last 2-D migration ran: threads per CTA, shots per CTA, grid, whether
        it replayed the captured CUDA graph and whether it timed the CTA shapes first."""
        v = [C.c_int() for _ in range(5)]
        L.check(L.lib().wem_last_launch(self._h, *[C.byref(x) for x in v]))
        out = dict(zip(["threads", "shots_per_cta", "grid", "graph_replayed", "tuned"], [x.value for x in v]))
        f, b = C.c_int(), C.c_int()
        L.check(L.lib().wem_last_launch_form(self._h, C.byref(f), C.byref(b)))
        out["form"] = {0: "fp32", 1: "split16", 2: "fp32-paired", 3: "fp32-bluestein", 4: "fp32-device-tables"}.get(f.value, str(f.value))
        out["bulk_table_copies"] = b.value
        return out

    def stream(self) -> int:
        """cudaStream_t of this context, as an integer handle."""
        s = C.c_void_p()
        L.check(L.lib().wem_ctx_stream(self._h, C.byref(s)))
        return int(s.value or 0)


def migrate(params: dict, vel, wav, shots: Shots, device: int = 0) -> np.ndarray:
    """One-shot convenience: prepare + migrate on a fresh context."""
    with Context(device) as ctx:
        return ctx.prepare(params, vel, wav).migrate(shots)


def _rows(a: np.ndarray):
    fp = _f32p
    rows = (fp * a.shape[0])()
    base = a.ctypes.data
    for i in range(a.shape[0]):
        rows[i] = C.cast(base + i * a.strides[0], fp)
    return rows


def wem_dropin(p: dict, vel, wav, d=None, m=None, adj=True) -> np.ndarray:
    """Calls the library's wem() exactly as the reference's wem.h:3-11 signature, with
    float** rows. Returns the image (adj) or the data."""
    n = int(p["nmx"]) * int(p.get("nmy", 1))
    vel = np.ascontiguousarray(vel, np.float32).copy()
    wav2 = np.ascontiguousarray(np.asarray(wav, np.float32).reshape(1, -1)).copy()
    dd = np.zeros((n, int(p["nt"])), np.float32) if d is None else np.ascontiguousarray(d, np.float32).copy()
    mm = np.zeros((n, int(p["nz"])), np.float32) if m is None else np.ascontiguousarray(m, np.float32).copy()
    rc = L.lib().wem(_rows(dd), _rows(mm), _rows(wav2), int(p["nt"]), float(p.get("ot", 0.0)), float(p["dt"]),
                     int(p["nmx"]), float(p.get("omx", 0.0)), float(p["dmx"]), int(p.get("nmy", 1)),
                     float(p.get("omy", 0.0)), float(p.get("dmy", p["dmx"])), float(p["sx"]),
                     float(p.get("sy", 0.0)), int(p["nz"]), float(p.get("oz", 0.0)), float(p["dz"]),
                     float(p.get("gz", 0.0)), float(p.get("sz", 0.0)), _rows(vel), int(p.get("nref", 5)),
                     float(p.get("fmin", 0.0)), float(p.get("fmax", 80.0)), int(p.get("padt", 1)),
                     int(p.get("padx", 1)), bool(adj), bool(p.get("pspi", True)), False)
    L.check(rc)
    return mm if adj else dd


def elastic(params: dict, vp, vs, wav, sx, sy=None, ux=None, uz=None, mpp=None, mps2=None, adj: bool = True,
            device: int = 0):
    """Elastic shot-profile migration (adj=True: the x and z components ux, uz [nshot, ncell, nt]
    recorded on every grid cell -> the P and S images mpp, mps2 [ncell, nz], stacked over the
    shots) or its forward operator (adj=False: mpp, mps2 -> ux, uz), wem_elastic (the
    reference's ewem, src/Imaging/c/ewem.c). ncell = nmx * nmy, cell = imx * nmy + imy (3-D
    grids when nmy > 1). Returns (mpp, mps2) or (ux, uz)."""
    p = make_params(**params)
    sx = np.ascontiguousarray(np.atleast_1d(sx), dtype=np.float32)
    sy = np.ascontiguousarray(np.zeros(len(sx)) if sy is None else np.atleast_1d(sy), dtype=np.float32)
    nshot, nmx, nz, nt = len(sx), p.nmx * max(p.nmy, 1), p.nz, p.nt
    vp = np.ascontiguousarray(vp, dtype=np.float32)
    vs = np.ascontiguousarray(vs, dtype=np.float32)
    wav = np.ascontiguousarray(wav, dtype=np.float32)
    if adj:
        ux = np.ascontiguousarray(ux, dtype=np.float32).reshape(nshot, nmx, nt)
        uz = np.ascontiguousarray(uz, dtype=np.float32).reshape(nshot, nmx, nt)
        mpp = np.empty((nmx, nz), np.float32)
        mps2 = np.empty((nmx, nz), np.float32)
    else:
        mpp = np.ascontiguousarray(mpp, dtype=np.float32).reshape(nmx, nz)
        mps2 = np.ascontiguousarray(mps2, dtype=np.float32).reshape(nmx, nz)
        ux = np.empty((nshot, nmx, nt), np.float32)
        uz = np.empty((nshot, nmx, nt), np.float32)
    L.check(L.lib().wem_elastic(device, C.byref(p), vp.ctypes.data_as(_f32p), vs.ctypes.data_as(_f32p),
                                wav.ctypes.data_as(_f32p), nshot, sx.ctypes.data_as(_f32p), sy.ctypes.data_as(_f32p),
                                ux.ctypes.data_as(_f32p), uz.ctypes.data_as(_f32p), mpp.ctypes.data_as(_f32p),
                                mps2.ctypes.data_as(_f32p), int(bool(adj))))
    return (mpp, mps2) if adj else (ux, uz)
