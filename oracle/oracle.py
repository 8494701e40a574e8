"""oracle/oracle.py -- TEST INFRASTRUCTURE (CPU oracle), never the product path.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
module, and only to check results or as the timed CPU baseline.

ctypes access to
  * oracle/liboracle.so   -- the C restatements of the reference operator
                             (src/Imaging/c/wem.c:3-564): ``wem_port`` keeps the
                             reference's float/double mixture, ``wem_fp64`` is the
                             same operator in double precision; plus the FFT.
  * oracle/_ref/libshotwem_ref.so -- the reference's own C core compiled unmodified
                             against oracle/fftw_subset.c (only where the reference
                             sources exist; see oracle/Makefile).
and the Python restatement of the multi-shot orchestration of
src/Imaging/ShotProfileWEM.jl:100-199 (adjoint: per-shot images stacked in
Float32, shot order) and :203-310 (forward: per-shot data gathers).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libshotwem_ref.so")
REF_EXE_PATH = os.path.join(HERE, "_ref", "shotwem_ref")
EWEM_REF_PATH = os.path.join(HERE, "_ref", "libewem_ref.so")

_lib = None
_ref = None
_ewem = None

_f = C.c_float
_i = C.c_int
_fp = C.POINTER(C.c_float)
_dp = C.POINTER(C.c_double)

_WEM_ARGS_TAIL = [_i, _f, _f,            # nt, ot, dt
                  _i, _f, _f,            # nmx, omx, dmx
                  _i, _f, _f,            # nmy, omy, dmy
                  _f, _f,                # sx, sy
                  _i, _f, _f, _f, _f]    # nz, oz, dz, gz, sz


def build(force: bool = False) -> str:
    """Compile liboracle.so with the committed recipe (oracle/Makefile)."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    return LIB_PATH


_ref_present = None


def ref_sources_available() -> bool:
    """Whether the reference's sources exist on this machine; the recipe (oracle/Makefile,
    REF= or WEM_REFERENCE_ROOT) is the one place that knows where they lie."""
    global _ref_present
    if _ref_present is None:
        _ref_present = subprocess.run(["make", "-s", "-C", HERE, "ref-present"],
                                      stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL).returncode == 0
    return _ref_present


def build_ref() -> str | None:
    """Compile the reference C core into oracle/_ref when its sources exist."""
    if not ref_sources_available():
        return None
    subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)
    return REF_LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.wemo_port_wem.restype = _i
        L.wemo_port_wem.argtypes = [_fp, _fp, _fp] + _WEM_ARGS_TAIL + [
            _fp, _i, _f, _f, _i, _i, _i, _i, _i, _i]
        L.wemo_fp64_wem.restype = _i
        L.wemo_fp64_wem.argtypes = [_dp, _dp, _fp] + _WEM_ARGS_TAIL + [
            _fp, _i, _f, _f, _i, _i, _i, _i, _i, _i]
        L.wemo_fft_f32.restype = _i
        L.wemo_fft_f32.argtypes = [_fp, _i, _i, _i]
        L.wemo_fft_f64.restype = _i
        L.wemo_fft_f64.argtypes = [_dp, _i, _i, _i]
        L.wemo_omp_max_threads.restype = _i
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_LIB_PATH)


def ref_lib():
    global _ref
    if _ref is None:
        if not ref_available():
            build_ref()
        if not ref_available():
            raise RuntimeError("reference C core not built (oracle/_ref missing)")
        L = C.CDLL(REF_LIB_PATH)
        fpp = C.POINTER(_fp)
        # wem.h:3-11 ; bool is C99 _Bool (1 byte)
        L.wem.restype = None
        L.wem.argtypes = [fpp, fpp, fpp] + _WEM_ARGS_TAIL + [
            fpp, _i, _f, _f, _i, _i, C.c_bool, C.c_bool, C.c_bool]
        L.main.restype = _i
        L.main.argtypes = [_i, C.POINTER(C.c_char_p)]
        # wem.h:44-50
        L.compute_angles.restype = None
        L.compute_angles.argtypes = [fpp, fpp, fpp, _i, _f, _f, _i, _f, _f, _i, _f, _f, _f, _f, _i, _f, _f, _f,
                                     fpp, _f, _f, C.c_bool]
        _ref = L
    return _ref


def ewem_ref(p: dict, vp: np.ndarray, vs: np.ndarray, wav: np.ndarray, ux=None, uz=None, mpp=None, mps2=None,
             adj: bool = True):
    """The reference's own elastic migration ewem() (oracle/_ref/libewem_ref.so,
    src/Imaging/c/ewem.c:3-253), one shot, via float** rows. adj=True: (ux, uz) data
    [nx*ny, nt] -> (mpp, mps1, mps2) images [nx*ny, nz]; adj=False: (mpp, mps2) -> (ux, uy,
    uz). The y component and mps1 take no part in the reference's 2-D separation
    (ewem.c:553-741), so they are zero in and out here."""
    global _ewem
    if _ewem is None:
        if not os.path.exists(EWEM_REF_PATH):
            build_ref()
        if not os.path.exists(EWEM_REF_PATH):
            raise RuntimeError("the reference's elastic core is not built (oracle/_ref missing)")
        L = C.CDLL(EWEM_REF_PATH)
        fpp = C.POINTER(_fp)
        L.ewem.restype = None
        L.ewem.argtypes = [fpp] * 7 + _WEM_ARGS_TAIL + [fpp, fpp, _f, _f, _i, _i, C.c_bool, C.c_bool]
        _ewem = L
    n = int(p["nmx"]) * int(p.get("nmy", 1))
    nt, nz = int(p["nt"]), int(p["nz"])

    def arr(a, cols):
        return np.zeros((n, cols), np.float32) if a is None else np.ascontiguousarray(a, np.float32).copy()
    dx, dy, dz_ = arr(ux, nt), np.zeros((n, nt), np.float32), arr(uz, nt)
    m1, m2, m3 = arr(mpp, nz), np.zeros((n, nz), np.float32), arr(mps2, nz)
    wav2 = np.ascontiguousarray(np.asarray(wav, np.float32).reshape(1, -1)).copy()
    vpa = np.ascontiguousarray(vp, np.float32).copy()
    vsa = np.ascontiguousarray(vs, np.float32).copy()
    _ewem.ewem(_rows(dx), _rows(dy), _rows(dz_), _rows(m1), _rows(m2), _rows(m3), _rows(wav2), *_common(p),
               _rows(vpa), _rows(vsa), float(p.get("fmin", 0.0)), float(p.get("fmax", 80.0)),
               int(p.get("padt", 1)), int(p.get("padx", 1)), bool(adj), False)
    return (m1, m2, m3) if adj else (dx, dy, dz_)


def angles_ref(p: dict, vel: np.ndarray, wav: np.ndarray):
    """The reference's own compute_angles() (oracle/_ref, src/Imaging/c/wem.c:566-684):
    angx, angy [nx*ny, nz] of the shot at (p["sx"], p["sy"]). Its frequency loop adds
    into shared arrays from every OpenMP thread without synchronisation, so only a
    process started with OMP_NUM_THREADS=1 gives a well-defined result."""
    L = ref_lib()
    n = int(p["nmx"]) * int(p.get("nmy", 1))
    nz = int(p["nz"])
    vel = np.ascontiguousarray(vel, dtype=np.float32).copy()
    wav2 = np.ascontiguousarray(np.asarray(wav, np.float32).reshape(1, -1)).copy()
    ax = np.zeros((n, nz), np.float32)
    ay = np.zeros((n, nz), np.float32)
    L.compute_angles(_rows(ax), _rows(ay), _rows(wav2), int(p["nt"]), float(p.get("ot", 0.0)), float(p["dt"]),
                     int(p["nmx"]), float(p.get("omx", 0.0)), float(p["dmx"]), int(p.get("nmy", 1)),
                     float(p.get("omy", 0.0)), float(p.get("dmy", p["dmx"])), float(p["sx"]), float(p.get("sy", 0.0)),
                     nz, float(p.get("oz", 0.0)), float(p["dz"]), float(p.get("sz", 0.0)), _rows(vel),
                     float(p.get("fmin", 0.0)), float(p.get("fmax", 80.0)), False)
    return ax, ay


def omp_threads() -> int:
    """Threads an OpenMP region of this process gets (fixed at the runtime's start)."""
    return int(lib().wemo_omp_max_threads())


# --------------------------------------------------------------------------- FFT

def fft_f32(x: np.ndarray, sign: int = -1) -> np.ndarray:
    """Unnormalised complex FFT along the last axis, complex64 arithmetic."""
    a = np.ascontiguousarray(x, dtype=np.complex64).copy()
    n = a.shape[-1]
    rc = lib().wemo_fft_f32(a.view(np.float32).ctypes.data_as(_fp), n, a.size // max(n, 1), sign)
    assert rc == 0
    return a


def fft_f64(x: np.ndarray, sign: int = -1) -> np.ndarray:
    a = np.ascontiguousarray(x, dtype=np.complex128).copy()
    n = a.shape[-1]
    rc = lib().wemo_fft_f64(a.view(np.float64).ctypes.data_as(_dp), n, a.size // max(n, 1), sign)
    assert rc == 0
    return a


# --------------------------------------------------------------------------- operator

def _interp(p: dict) -> int:
    v = p.get("interp", 0)
    return {"ref": 0, "linear": 1}[v] if isinstance(v, str) else int(v)


def _common(p: dict):
    return [int(p["nt"]), float(p.get("ot", 0.0)), float(p["dt"]),
            int(p["nmx"]), float(p["omx"]), float(p["dmx"]),
            int(p.get("nmy", 1)), float(p.get("omy", 0.0)), float(p.get("dmy", p["dmx"])),
            float(p["sx"]), float(p.get("sy", 0.0)),
            int(p["nz"]), float(p.get("oz", 0.0)), float(p["dz"]), float(p.get("gz", 0.0)),
            float(p.get("sz", 0.0))]


def wem_port(p: dict, vel: np.ndarray, wav: np.ndarray, d: np.ndarray | None = None,
             m: np.ndarray | None = None, adj: bool = True, nthreads: int = 0) -> np.ndarray:
    """Reference-semantics port of wem() (one shot). vel [nx*ny, nz]; d [nx*ny, nt];
    m [nx*ny, nz]. adj=True returns the image, adj=False the data."""
    n = int(p["nmx"]) * int(p.get("nmy", 1))
    vel = np.ascontiguousarray(vel, dtype=np.float32)
    wav = np.ascontiguousarray(wav, dtype=np.float32)
    dd = np.zeros((n, int(p["nt"])), np.float32) if d is None else np.ascontiguousarray(d, np.float32).copy()
    mm = np.zeros((n, int(p["nz"])), np.float32) if m is None else np.ascontiguousarray(m, np.float32).copy()
    rc = lib().wemo_port_wem(dd.ctypes.data_as(_fp), mm.ctypes.data_as(_fp), wav.ctypes.data_as(_fp),
                             *_common(p), vel.ctypes.data_as(_fp), int(p.get("nref", 5)),
                             float(p.get("fmin", 0.0)), float(p.get("fmax", 80.0)),
                             int(p.get("padt", 1)), int(p.get("padx", 1)), int(adj),
                             int(p.get("pspi", 1)), _interp(p), int(nthreads))
    if rc != 0:
        raise ValueError(f"wem_port rejected the arguments (rc={rc})")
    return mm if adj else dd


def wem_fp64(p: dict, vel: np.ndarray, wav: np.ndarray, d: np.ndarray | None = None,
             m: np.ndarray | None = None, adj: bool = True, nthreads: int = 0) -> np.ndarray:
    """The same operator in double precision (float64 in and out)."""
    n = int(p["nmx"]) * int(p.get("nmy", 1))
    vel = np.ascontiguousarray(vel, dtype=np.float32)
    wav = np.ascontiguousarray(wav, dtype=np.float32)
    dd = np.zeros((n, int(p["nt"])), np.float64) if d is None else np.ascontiguousarray(d, np.float64).copy()
    mm = np.zeros((n, int(p["nz"])), np.float64) if m is None else np.ascontiguousarray(m, np.float64).copy()
    rc = lib().wemo_fp64_wem(dd.ctypes.data_as(_dp), mm.ctypes.data_as(_dp), wav.ctypes.data_as(_fp),
                             *_common(p), vel.ctypes.data_as(_fp), int(p.get("nref", 5)),
                             float(p.get("fmin", 0.0)), float(p.get("fmax", 80.0)),
                             int(p.get("padt", 1)), int(p.get("padx", 1)), int(adj),
                             int(p.get("pspi", 1)), _interp(p), int(nthreads))
    if rc != 0:
        raise ValueError(f"wem_fp64 rejected the arguments (rc={rc})")
    return mm if adj else dd


def _rows(a: np.ndarray):
    fp = _fp
    rows = (fp * a.shape[0])()
    base = a.ctypes.data
    for i in range(a.shape[0]):
        rows[i] = C.cast(base + i * a.strides[0], fp)
    return rows


def wem_ref(p: dict, vel: np.ndarray, wav: np.ndarray, d: np.ndarray | None = None,
            m: np.ndarray | None = None, adj: bool = True) -> np.ndarray:
    """The reference's own wem() (oracle/_ref), via float** row pointers as
    alloc2float builds them (src/API/c/seismic.c:92-106). Thread count follows
    OMP_NUM_THREADS."""
    L = ref_lib()
    n = int(p["nmx"]) * int(p.get("nmy", 1))
    vel = np.ascontiguousarray(vel, dtype=np.float32).copy()
    wav2 = np.ascontiguousarray(np.asarray(wav, np.float32).reshape(1, -1)).copy()
    dd = np.zeros((n, int(p["nt"])), np.float32) if d is None else np.ascontiguousarray(d, np.float32).copy()
    mm = np.zeros((n, int(p["nz"])), np.float32) if m is None else np.ascontiguousarray(m, np.float32).copy()
    L.wem(_rows(dd), _rows(mm), _rows(wav2), *_common(p), _rows(vel), int(p.get("nref", 5)),
          float(p.get("fmin", 0.0)), float(p.get("fmax", 80.0)), int(p.get("padt", 1)),
          int(p.get("padx", 1)), bool(adj), bool(p.get("pspi", 1)), False)
    return mm if adj else dd


# --------------------------------------------------------------------------- multi-shot

def migrate_shots(op, p: dict, vel, wav, shots, **kw) -> np.ndarray:
    """ShotProfileWEM.jl:100-199 with nangx=nangy=1: migrate each shot over the
    full grid and add the shot images in Float32, in shot order.
    shots: iterable of (sx, d_shot[n, nt])."""
    img = None
    for sx, d in shots:
        q = dict(p, sx=sx)
        m = op(q, vel, wav, d=d, adj=True, **kw)
        img = m.astype(np.float32) if img is None else (img + m.astype(np.float32)).astype(np.float32)
    return img
