"""ctypes binding of lib/shotwem.so (C ABI in include/shotwem_gb300.h).

There is deliberately no fallback: if the CUDA library is not built, or no GPU is
present, calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))  # seismic.jl_gb300/
LIB_PATH = os.path.join(PKG_DIR, "lib", "shotwem.so")

WEM_OK = 0
WEM_ERR_ARG = -1
WEM_ERR_SIZE = -2
WEM_ERR_CUDA = -3
WEM_ERR_TIMEOUT = -4
WEM_ERR_IO = -5
WEM_ERR_NOMEM = -6
WEM_ERR_NODEV = -7

INTERP = {"ref": 0, "linear": 1}
PRECISION = {"fp32": 0, "split16": 1}

# every symbol the public header declares
EXPORTS = ["wem_last_error", "wem_version", "wem_ctx_create", "wem_ctx_destroy", "wem_prepare",
           "wem_migrate", "wem_migrate_device", "wem_migrate_survey", "wem_last_timing",
           "wem_last_kernel_times", "wem_last_launch", "wem_last_launch_form", "wem_ctx_stream", "wem_migrate_noalloc", "wem_model",
           "wem_model_device", "wem_angles", "wem", "wem_selftest_wait_timeout", "wem_measure_fp32_peak",
           "wem_elastic", "wem_elastic_last_ms", "ewem",
           "shotwem_main", "main"]


class WemError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"shotwem status {code}: {msg}")
        self.code = code


class Params(C.Structure):
    """wem_params of include/shotwem_gb300.h (field order matters)."""
    _fields_ = [("nt", C.c_int), ("ot", C.c_float), ("dt", C.c_float),
                ("nmx", C.c_int), ("omx", C.c_float), ("dmx", C.c_float),
                ("nmy", C.c_int), ("omy", C.c_float), ("dmy", C.c_float),
                ("nz", C.c_int), ("oz", C.c_float), ("dz", C.c_float),
                ("gz", C.c_float), ("sz", C.c_float),
                ("nref", C.c_int), ("fmin", C.c_float), ("fmax", C.c_float),
                ("padt", C.c_int), ("padx", C.c_int),
                ("pspi", C.c_int), ("interp", C.c_int), ("precision", C.c_int),
                ("verbose", C.c_int)]


_lib = None


def build(force: bool = False) -> str:
    """Compile lib/shotwem.so with the package Makefile (nvcc, sm_103a)."""
    if force or not os.path.exists(LIB_PATH):
        jobs = str(min(8, os.cpu_count() or 1))
        subprocess.run(["make", "-s", "-j", jobs, "-C", PKG_DIR], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"CUDA library not built: {LIB_PATH} (run __graft_entry__.build())")
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        fp = C.POINTER(C.c_float)
        i64p = C.POINTER(C.c_int64)
        i32p = C.POINTER(C.c_int32)
        L.wem_last_error.restype = C.c_char_p
        L.wem_version.restype = C.c_int
        L.wem_ctx_create.argtypes = [C.POINTER(vp), C.c_int]
        L.wem_ctx_destroy.argtypes = [vp]
        L.wem_prepare.argtypes = [vp, C.POINTER(Params), fp, fp]
        L.wem_migrate.argtypes = [vp, C.c_int, fp, fp, i64p, i32p, fp, fp]
        L.wem_migrate_device.argtypes = [vp, C.c_int, fp, fp, i64p, i32p, vp, vp, C.c_int]
        L.wem_model.argtypes = [vp, C.c_int, fp, fp, i64p, i32p, fp, fp, C.c_int]
        L.wem_model_device.argtypes = [vp, C.c_int, fp, fp, i64p, i32p, vp, vp, C.c_int, C.c_int]
        L.wem_migrate_survey.argtypes = [vp, C.POINTER(Params), fp, fp, C.c_int, fp, fp, i64p, i32p, fp, fp]
        L.wem_last_timing.argtypes = [vp, C.POINTER(C.c_float), C.POINTER(C.c_int)]
        f_p = C.POINTER(C.c_float)
        L.wem_last_kernel_times.argtypes = [vp, f_p, f_p, f_p]
        ip = C.POINTER(C.c_int)
        L.wem_last_launch.argtypes = [vp, ip, ip, ip, ip, ip]
        L.wem_last_launch_form.argtypes = [vp, ip, ip]
        L.wem_selftest_wait_timeout.argtypes = [C.c_int, ip, C.POINTER(C.c_float)]
        L.wem_measure_fp32_peak.argtypes = [C.c_int, C.POINTER(C.c_double)]
        L.wem_elastic.argtypes = [C.c_int, C.POINTER(Params), fp, fp, fp, C.c_int, fp, fp, fp, fp, fp, fp, C.c_int]
        L.wem_elastic_last_ms.restype = C.c_float
        L.wem_angles.argtypes = [vp, C.POINTER(Params), fp, fp, C.c_int, fp, fp, fp, fp]
        L.wem_ctx_stream.argtypes = [vp, C.POINTER(vp)]
        L.wem_migrate_noalloc.argtypes = [C.POINTER(Params), vp, vp, C.c_int, fp, fp, vp, vp, vp]
        L.shotwem_main.argtypes = [C.c_int, C.POINTER(C.c_char_p)]
        L.main.argtypes = [C.c_int, C.POINTER(C.c_char_p)]
        fpp = C.POINTER(fp)
        L.wem.restype = C.c_int
        L.wem.argtypes = [fpp, fpp, fpp, C.c_int, C.c_float, C.c_float, C.c_int, C.c_float, C.c_float,
                          C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int, C.c_float,
                          C.c_float, C.c_float, C.c_float, fpp, C.c_int, C.c_float, C.c_float, C.c_int,
                          C.c_int, C.c_bool, C.c_bool, C.c_bool]
        _lib = L
    return _lib


def measure_fp32_peak(device: int = 0) -> float:
    """Measured FP32 FMA throughput of the device in TFLOP/s (wem_measure_fp32_peak)."""
    v = C.c_double()
    check(lib().wem_measure_fp32_peak(device, C.byref(v)))
    return float(v.value)


def check(rc: int):
    if rc != WEM_OK:
        raise WemError(rc, lib().wem_last_error().decode(errors="replace"))
