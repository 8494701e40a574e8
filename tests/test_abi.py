"""C ABI and host logic, without a GPU (no compute calls).

* shotwem.so loads and exports every function include/shotwem_gb300.h declares
  (plus main, the symbol the Julia wrapper binds);
* without a device, entry points fail with a status instead of falling back;
* main() reports a missing argument as a status instead of exit(1);
* seis files round-trip; synthetic surveys are reproducible.
"""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "shotwem_gb300.h")


def declared_functions(header=HEADER):
    src = open(header).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:WEM_API\s+)?(?:const\s+)?\w+\s*\*?\s*(\w+)\s*\(", src, flags=re.M)
    return sorted(set(n for n in names if n not in ("if", "while")))


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ["wem", "shotwem_main", "wem_ctx_create", "wem_prepare", "wem_migrate", "wem_last_error"]:
        assert n in names


def test_library_exports_every_declared_symbol(gpu_lib):
    lib = C.CDLL(gpu_lib.LIB_PATH)
    for name in declared_functions() + ["main"]:
        assert hasattr(lib, name), f"shotwem.so does not export {name}"


def test_compute_angles_library_exports_its_entry_points(gpu_lib):
    """compute_angles.so (the drop-in for the reference's compute_angles library) exports
    main and what include/compute_angles_gb300.h declares, and reports a missing key as
    a status (compute_angles.c:27-33 calls exit(1))."""
    path = os.path.join(os.path.dirname(gpu_lib.LIB_PATH), "compute_angles.so")
    lib = C.CDLL(path)
    names = declared_functions(os.path.join(ROOT, "include", "compute_angles_gb300.h"))
    assert names == ["compute_angles_main"]
    for name in names + ["main"]:
        assert hasattr(lib, name)
    lib.main.argtypes = [C.c_int, C.POINTER(C.c_char_p)]
    argv = (C.c_char_p * 2)(b"0", b"angx=a")
    assert lib.main(2, argv) == gpu_lib._lib.WEM_ERR_ARG


def test_shotewem_library_exports_its_entry_points(gpu_lib):
    """shotewem.so (the drop-in for the reference's shotewem library) exports main and what
    include/shotewem_gb300.h declares, and reports a missing key as a status
    (shotewem.c:37-45 calls exit(1))."""
    path = os.path.join(os.path.dirname(gpu_lib.LIB_PATH), "shotewem.so")
    lib = C.CDLL(path)
    names = declared_functions(os.path.join(ROOT, "include", "shotewem_gb300.h"))
    assert names == ["shotewem_main"]
    for name in names + ["main"]:
        assert hasattr(lib, name)
    lib.main.argtypes = [C.c_int, C.POINTER(C.c_char_p)]
    argv = (C.c_char_p * 4)(b"0", b"ux=a", b"uy=b", b"uz=c")
    assert lib.main(4, argv) == gpu_lib._lib.WEM_ERR_ARG


def _has_gpu():
    lib = C.CDLL(__import__("wemgpu").LIB_PATH)
    h = C.c_void_p()
    rc = lib.wem_ctx_create(C.byref(h), 0)
    if rc == 0:
        lib.wem_ctx_destroy(h)
    return rc


def test_no_device_means_error_not_fallback(gpu_lib):
    rc = _has_gpu()
    if rc == 0:
        pytest.skip("a GPU is present")
    assert rc == gpu_lib._lib.WEM_ERR_NODEV
    msg = gpu_lib.lib().wem_last_error().decode()
    assert "no CUDA device" in msg


def test_main_missing_argument_returns_status(gpu_lib):
    L = gpu_lib.lib()
    argv = (C.c_char_p * 3)(b"0", b"adj=y", b"pspi=y")
    assert L.main(3, argv) == gpu_lib._lib.WEM_ERR_ARG
    assert L.shotwem_main(3, argv) == gpu_lib._lib.WEM_ERR_ARG


def test_main_unreadable_files_return_io_status(gpu_lib, tmp_path):
    L = gpu_lib.lib()
    args = [b"0", b"d=" + str(tmp_path / "nod").encode(), b"m=" + str(tmp_path / "m").encode(),
            b"vel=" + str(tmp_path / "novel").encode(), b"wav=" + str(tmp_path / "nowav").encode()]
    argv = (C.c_char_p * len(args))(*args)
    assert L.main(len(args), argv) == gpu_lib._lib.WEM_ERR_IO


def test_seis_roundtrip(tmp_path):
    from wemgpu import seis
    rng = np.random.default_rng(0)
    a = rng.standard_normal((7, 33)).astype(np.float32)
    name = str(tmp_path / "g")
    seis.write_grid(name, a, o1=0.0, d1=12.5, ox=100.0, dx=12.5)
    b, h, ext = seis.read(name)
    assert np.array_equal(a, b)
    assert ext["n"][:2] == [33, 7] and ext["d"][0] == 12.5
    assert list(h["imx"]) == list(range(7)) and h["mx"][1] - h["mx"][0] == 12.5
    seis.remove(name)
    assert not os.path.exists(name) and not os.path.exists(name + "@data@")


def test_seis_header_is_124_bytes():
    from wemgpu import seis
    assert seis.HEADER_DTYPE.itemsize == 124  # 31 four-byte fields, src/API/c/seismic.h:20-53


def test_synthetic_surveys_are_seeded():
    from wemgpu import synth
    a = synth.small_case(3)
    b = synth.small_case(3)
    assert np.array_equal(a["vel"], b["vel"]) and np.array_equal(a["shots"].data, b["shots"].data)
    c = synth.config0()
    assert c["vel"].shape == (256, 200) and c["shots"].data.shape == (256, 1000)
    assert set(np.unique(c["vel"])) == {1500.0, 2200.0, 3000.0}


def test_ricker_matches_reference_definition():
    """Ricker.jl:21-28: nw = 2/(f0 dt), nc = floor(nw/2), w = (1-2b)e^{-b}, b=(pi f0 t)^2."""
    from wemgpu import synth
    w = synth.ricker(20.0, 0.002)
    assert len(w) == 51 and np.argmax(w) == 25 and abs(w[25] - 1.0) < 1e-7


def test_shotewem_main_3d_grid_spacing_from_first_two_traces(gpu_lib, tmp_path):
    """shotewem.c:78 takes dx from the first two velocity traces' mx. A 3-D grid stored as the
    computation indexes it (cell = imx * ny + imy, y fastest) has the same mx on those two traces,
    so dx = 0: the reference goes on with a zero spacing, the drop-in refuses with WEM_ERR_ARG
    before any device work (no GPU is needed to see it)."""
    import numpy as np
    from wemgpu import seis
    nx, ny, nz, nt = 4, 4, 3, 8
    t = str(tmp_path)
    n = nx * ny
    h = seis.empty_headers(n)
    cell = np.arange(n)
    h["tracenum"] = cell + 1
    h["imx"], h["imy"] = cell // ny, cell % ny
    h["mx"], h["my"] = 10.0 * (cell // ny), 10.0 * (cell % ny)
    h["n1"], h["d1"] = nz, 10.0
    v = np.full((n, nz), 2000.0, np.float32)
    seis.write(t + "/vp", v, h, [nz, nx, ny], [0.0, 0.0, 0.0], [10.0, 10.0, 10.0])
    seis.write(t + "/vs", v / 1.8, h, [nz, nx, ny], [0.0, 0.0, 0.0], [10.0, 10.0, 10.0])
    seis.write_wavelet(t + "/wav", np.ones(nt, np.float32), dt=0.004)
    hd = seis.empty_headers(n)
    hd["n1"], hd["d1"], hd["gx"], hd["gy"] = nt, 0.004, h["mx"], h["my"]
    for k in ("ux", "uy", "uz"):
        seis.write(f"{t}/{k}", np.zeros((n, nt), np.float32), hd, [nt, nx, ny], [0.0] * 3, [0.004, 10.0, 10.0])
    lib = C.CDLL(os.path.join(os.path.dirname(gpu_lib.LIB_PATH), "shotewem.so"))
    lib.main.argtypes = [C.c_int, C.POINTER(C.c_char_p)]
    args = ["0", "adj=y"] + [f"{k}={t}/{k}" for k in ("ux", "uy", "uz", "mpp", "mps1", "mps2", "vp", "vs", "wav")]
    argv = (C.c_char_p * len(args))(*[a.encode() for a in args])
    assert lib.main(len(args), argv) == gpu_lib._lib.WEM_ERR_ARG
    assert "invalid grid" in gpu_lib.lib().wem_last_error().decode()


def test_elastic_3d_argument_checks_need_no_device(gpu_lib):
    """wem_elastic on a 3-D grid checks its sizes and source positions before any device
    work: planes whose sides are not powers of two in [64, 1024] give WEM_ERR_SIZE, and a
    source off the grid in y gives WEM_ERR_ARG."""
    import numpy as np
    from wemgpu._lib import WemError, WEM_ERR_ARG, WEM_ERR_SIZE
    p = dict(nt=16, dt=0.004, nmx=32, omx=0.0, dmx=10.0, nmy=32, omy=0.0, dmy=10.0, nz=4, oz=0.0, dz=10.0,
             fmin=3.0, fmax=30.0, padt=2, padx=2)
    wav = np.ones(16, np.float32)

    def call(q, sx, sy):
        n = q["nmx"] * q["nmy"]
        v = np.full((n, q["nz"]), 2000.0, np.float32)
        z = np.zeros((len(sx), n, q["nt"]), np.float32)
        with pytest.raises(WemError) as e:
            gpu_lib.elastic(q, v, v / 1.8, wav, sx, sy=sy, ux=z, uz=z, adj=True)
        return e.value.code

    assert call(dict(p, nmx=40, nmy=24), [100.0], [100.0]) == WEM_ERR_SIZE  # 80 x 48 planes
    assert call(dict(p, nmx=1024, nmy=32), [100.0], [100.0]) == WEM_ERR_SIZE  # 2048 x 64 planes
    assert call(p, [100.0], [1e6]) == WEM_ERR_ARG
