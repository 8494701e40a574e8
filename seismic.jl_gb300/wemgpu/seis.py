"""The seis file format shared by Seismic.jl and its C core.

Text header of tab-indented key=value lines (src/ReadWrite/Header.jl:385-419,
src/API/c/seismic.c:423-461); `in` names the data file (ntraces x n1 native
float32) and `headers` the trace-header file (ntraces x 124-byte records with the
field order of type Header, src/ReadWrite/Header.jl:1-33). A key given twice takes
its last value (Header.jl:319-375 searches from the end).
"""
from __future__ import annotations

import os

import numpy as np

HEADER_FIELDS = [
    ("tracenum", "<i4"), ("o1", "<f4"), ("n1", "<i4"), ("d1", "<f4"),
    ("sx", "<f4"), ("sy", "<f4"), ("gx", "<f4"), ("gy", "<f4"), ("mx", "<f4"), ("my", "<f4"),
    ("hx", "<f4"), ("hy", "<f4"), ("h", "<f4"), ("az", "<f4"), ("ang", "<f4"),
    ("isx", "<i4"), ("isy", "<i4"), ("igx", "<i4"), ("igy", "<i4"), ("imx", "<i4"), ("imy", "<i4"),
    ("ihx", "<i4"), ("ihy", "<i4"), ("ih", "<i4"), ("iaz", "<i4"), ("iang", "<i4"),
    ("selev", "<f4"), ("gelev", "<f4"), ("sstat", "<f4"), ("gstat", "<f4"), ("trid", "<i4"),
]
HEADER_DTYPE = np.dtype(HEADER_FIELDS)
assert HEADER_DTYPE.itemsize == 124


def empty_headers(n: int) -> np.ndarray:
    return np.zeros(n, HEADER_DTYPE)


def read_text_header(name: str) -> dict:
    ext = {"n": [1] * 5, "o": [0.0] * 5, "d": [1.0] * 5, "in": None, "headers": None,
           "data_format": "native_float", "esize": 4, "title": "", "label": [""] * 5, "unit": [""] * 5}
    with open(name) as f:
        for line in f:
            line = line.strip()
            if "=" not in line:
                continue
            k, v = line.split("=", 1)
            k = k.strip()
            v = v.strip()
            q = v[1:-1] if len(v) >= 2 and v[0] == '"' and v[-1] == '"' else v
            if len(k) == 2 and k[0] in "nod" and k[1] in "12345":
                i = int(k[1]) - 1
                if k[0] == "n":
                    ext["n"][i] = int(q)
                elif k[0] == "o":
                    ext["o"][i] = float(q)
                else:
                    ext["d"][i] = float(q)
            elif k == "in":
                ext["in"] = q
            elif k == "headers":
                ext["headers"] = q
            elif k == "data_format":
                ext["data_format"] = q
            elif k == "esize":
                ext["esize"] = int(q)
            elif k == "title":
                ext["title"] = q
            elif k.startswith("label") and k[5:] in "12345" and len(k) == 6:
                ext["label"][int(k[5]) - 1] = q
            elif k.startswith("unit") and k[4:] in "12345" and len(k) == 5:
                ext["unit"][int(k[4]) - 1] = q
    return ext


def read(name: str):
    """Returns (data [ntraces, n1] float32, headers (structured array), extent dict)."""
    ext = read_text_header(name)
    n1 = ext["n"][0]
    ntr = int(np.prod(ext["n"][1:]))
    d = np.fromfile(ext["in"], dtype="<f4", count=ntr * n1).reshape(ntr, n1)
    h = np.fromfile(ext["headers"], dtype=HEADER_DTYPE, count=ntr) if ext["headers"] else empty_headers(ntr)
    return d, h, ext


def write(name: str, d: np.ndarray, h: np.ndarray, n, o, dd, labels=None, units=None, title=""):
    """Writes name, name@data@, name@headers@ (prefixed by $DATAPATH like
    SeisWrite.jl:21 / seismic.c:306)."""
    d = np.ascontiguousarray(d, dtype="<f4")
    dp = os.environ.get("DATAPATH", "")
    dname, hname = f"{dp}{name}@data@", f"{dp}{name}@headers@"
    n = list(n) + [1] * (5 - len(n))
    o = list(o) + [0.0] * (5 - len(o))
    dd = list(dd) + [1.0] * (5 - len(dd))
    labels = (labels or []) + [""] * (5 - len(labels or []))
    units = (units or []) + [""] * (5 - len(units or []))
    with open(name, "w") as f:
        for i in range(5):
            f.write(f"\tn{i + 1}={n[i]}\n")
        for i in range(5):
            f.write(f"\to{i + 1}={o[i]:f}\n")
        for i in range(5):
            f.write(f"\td{i + 1}={dd[i]:f}\n")
        for i in range(5):
            f.write(f'\tlabel{i + 1}="{labels[i]}"\n')
        for i in range(5):
            f.write(f'\tunit{i + 1}="{units[i]}"\n')
        f.write(f'\ttitle="{title}"\n\tdata_format="native_float"\n\tesize=4\n')
        f.write(f'\tin="{dname}"\n\theaders="{hname}"\n')
    d.tofile(dname)
    np.ascontiguousarray(h, dtype=HEADER_DTYPE).tofile(hname)


def remove(name: str):
    """SeisRemove: the text header and both binary files."""
    try:
        ext = read_text_header(name)
        for f in (ext["in"], ext["headers"]):
            if f and os.path.exists(f):
                os.remove(f)
    finally:
        if os.path.exists(name):
            os.remove(name)


# -- helpers for the 2-D grids the migration reads (shotwem.c:44-68 takes nz, dz, oz
#    from the velocity's n1/d1/o1, nx from the imx span of its headers, ox and dx
#    from the mx of its first two traces)

def grid_headers(nx: int, n1: int, o1: float, d1: float, ox: float, dx: float) -> np.ndarray:
    h = empty_headers(nx)
    h["tracenum"] = np.arange(1, nx + 1)
    h["n1"] = n1
    h["o1"] = o1
    h["d1"] = d1
    h["imx"] = np.arange(nx)
    h["mx"] = ox + dx * np.arange(nx, dtype=np.float64)
    return h


def write_grid(name: str, a: np.ndarray, o1: float, d1: float, ox: float, dx: float):
    nx, n1 = a.shape
    write(name, a, grid_headers(nx, n1, o1, d1, ox, dx), [n1, nx], [o1, ox], [d1, dx])


def write_wavelet(name: str, w: np.ndarray, dt: float, ot: float = 0.0):
    w = np.asarray(w, np.float32).reshape(1, -1)
    h = empty_headers(1)
    h["n1"] = w.shape[1]
    h["d1"] = dt
    h["o1"] = ot
    write(name, w, h, [w.shape[1], 1], [ot, 0.0], [dt, 1.0])


def write_shot(name: str, d: np.ndarray, sx: float, dt: float, ox: float, dx: float, ot: float = 0.0,
               sy: float = 0.0):
    """One shot gather on the full grid, receiver i at gx = ox + i*dx."""
    nx, nt = d.shape
    h = empty_headers(nx)
    h["tracenum"] = np.arange(1, nx + 1)
    h["n1"] = nt
    h["d1"] = dt
    h["o1"] = ot
    h["sx"] = sx
    h["sy"] = sy
    h["gx"] = ox + dx * np.arange(nx, dtype=np.float64)
    h["mx"] = h["gx"]
    h["imx"] = np.arange(nx)
    h["hx"] = h["gx"] - sx
    write(name, d, h, [nt, nx], [ot, ox], [dt, dx])
