"""Elastic shot-profile migration and its forward operator on the GPU (wem_elastic and the
ewem() drop-in; the reference's src/Imaging/c/ewem.c, 2-D) against the reference's own output
(golden vectors) and the oracle's FP64 restatement (oracle/ewem_np.py).

Tolerance: relative L2 <= 1e-4 on each image (P, S2) and each data component (x, z)."""
import ctypes as C

import numpy as np
import pytest

from conftest import load_golden, rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-4


@pytest.mark.parametrize("case", ["ewem_64", "ewem_150_padx1", "ewem_64_buried"])
def test_elastic_matches_reference_golden(gpu_lib, case):
    g = load_golden(f"{case}.npz")
    p = g["params"]
    mpp, mps2 = gpu_lib.elastic(p, g["vp"], g["vs"], g["wav"], [p["sx"]], ux=g["ux"][None], uz=g["uz"][None], adj=True)
    assert rel_l2(mpp, g["mpp_ref"]) < TOL, rel_l2(mpp, g["mpp_ref"])
    assert rel_l2(mps2, g["mps2_ref"]) < TOL, rel_l2(mps2, g["mps2_ref"])
    ux, uz = gpu_lib.elastic(p, g["vp"], g["vs"], g["wav"], [p["sx"]], mpp=g["mpp_in"], mps2=g["mps2_in"], adj=False)
    assert rel_l2(ux[0], g["ux_ref"]) < TOL, rel_l2(ux[0], g["ux_ref"])
    assert rel_l2(uz[0], g["uz_ref"]) < TOL, rel_l2(uz[0], g["uz_ref"])


def _rows(a):
    fp = C.POINTER(C.c_float)
    rows = (fp * a.shape[0])()
    for i in range(a.shape[0]):
        rows[i] = C.cast(a.ctypes.data + i * a.strides[0], fp)
    return rows


def test_ewem_dropin_matches_reference_golden(gpu_lib):
    """ewem() with the reference's argument list and float** rows (ewem.h:3-16)."""
    g = load_golden("ewem_64.npz")
    p = g["params"]
    L = gpu_lib.lib()
    fpp = C.POINTER(C.POINTER(C.c_float))
    L.ewem.restype = C.c_int
    L.ewem.argtypes = [fpp] * 7 + [C.c_int, C.c_float, C.c_float, C.c_int, C.c_float, C.c_float, C.c_int, C.c_float,
                                   C.c_float, C.c_float, C.c_float, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float,
                                   fpp, fpp, C.c_float, C.c_float, C.c_int, C.c_int, C.c_bool, C.c_bool]
    n, nt, nz = p["nmx"], p["nt"], p["nz"]
    ux, uz = np.ascontiguousarray(g["ux"], np.float32), np.ascontiguousarray(g["uz"], np.float32)
    uy = np.full((n, nt), 7.0, np.float32)
    mpp, mps1, mps2 = (np.full((n, nz), 7.0, np.float32) for _ in range(3))
    wav = np.ascontiguousarray(g["wav"], np.float32).reshape(1, -1)
    vp, vs = np.ascontiguousarray(g["vp"], np.float32), np.ascontiguousarray(g["vs"], np.float32)
    args = [p["nt"], 0.0, p["dt"], n, p["omx"], p["dmx"], 1, 0.0, p["dmx"], p["sx"], 0.0, nz, p["oz"], p["dz"], 0.0,
            0.0, _rows(vp), _rows(vs), p["fmin"], p["fmax"], p["padt"], p["padx"]]
    rc = L.ewem(_rows(ux), _rows(uy), _rows(uz), _rows(mpp), _rows(mps1), _rows(mps2), _rows(wav), *args, True, False)
    assert rc == 0
    assert rel_l2(mpp, g["mpp_ref"]) < TOL and rel_l2(mps2, g["mps2_ref"]) < TOL and not np.any(mps1)


@pytest.mark.parametrize("nx,padx,nshot", [(128, 2, 3), (500, 2, 3), (256, 1, 3), (512, 2, 4), (64, 1, 5)])
def test_elastic_shots_stacked_match_fp64_oracle(gpu_lib, nx, padx, nshot):
    """Several shots in one call (the images stacked over the shots) against the FP64
    restatement shot by shot. nx 500 with padx 2 runs rows of nkx 1000 (Bluestein's form, one
    shot per CTA); the power-of-two rows carry three shots of a frequency per CTA, so 4 and 5
    shots leave a group part-filled (1024-point rows; 64-point rows with teams of 4 threads)."""
    import ewem_np as E
    from wemgpu import synth
    c = synth.small_case(70 + nx, nx=nx, nz=10, nt=128, nshot=nshot, pspi=0, fmax=30.0, padx=padx)
    rng = np.random.default_rng(nx)
    vp = c["vel"]
    vs = (vp / 1.7 * (1.0 + 0.05 * rng.standard_normal(vp.shape))).astype(np.float32)
    p = dict(c["params"], fmin=3.0)
    shots = c["shots"]
    uz = np.stack([synth.shot_gather_full(shots, s, nx) for s in range(shots.nshot)])
    ux = (0.5 * np.roll(uz, 2, axis=2)).astype(np.float32)
    mpp, mps2 = gpu_lib.elastic(p, vp, vs, c["wav"], shots.sx, ux=ux, uz=uz, adj=True)
    want_p = want_s = 0.0
    for s in range(shots.nshot):
        a, _, b = E.ewem(dict(p, sx=float(shots.sx[s])), vp, vs, c["wav"], ux=ux[s], uz=uz[s], adj=True)
        want_p, want_s = want_p + a, want_s + b
    assert rel_l2(mpp, want_p) < TOL and rel_l2(mps2, want_s) < TOL
    m1 = rng.standard_normal((nx, 10)).astype(np.float32)
    m2 = rng.standard_normal((nx, 10)).astype(np.float32)
    dx, dz = gpu_lib.elastic(p, vp, vs, c["wav"], shots.sx, mpp=m1, mps2=m2, adj=False)
    for s in range(shots.nshot):
        wx, _, wz = E.ewem(dict(p, sx=float(shots.sx[s])), vp, vs, c["wav"], mpp=m1, mps2=m2, adj=False)
        assert rel_l2(dx[s], wx) < TOL and rel_l2(dz[s], wz) < TOL


def test_shotewem_main_on_seis_files(gpu_lib, tmp_path):
    """main of shotewem.so (shotewem.c:13-222) on seis files, migration and the forward
    operator, against the reference's ewem() output; headers as shotewem.c writes them."""
    import os
    from wemgpu import seis
    g = load_golden("ewem_64.npz")
    p = g["params"]
    t = str(tmp_path)
    lib = C.CDLL(os.path.join(os.path.dirname(gpu_lib.LIB_PATH), "shotewem.so"))
    lib.main.argtypes = [C.c_int, C.POINTER(C.c_char_p)]
    seis.write_grid(t + "/vp", g["vp"], o1=p["oz"], d1=p["dz"], ox=p["omx"], dx=p["dmx"])
    seis.write_grid(t + "/vs", g["vs"], o1=p["oz"], d1=p["dz"], ox=p["omx"], dx=p["dmx"])
    seis.write_wavelet(t + "/wav", g["wav"], dt=p["dt"])
    for k in ("ux", "uz"):
        seis.write_shot(f"{t}/{k}", g[k], sx=p["sx"], dt=p["dt"], ox=p["omx"], dx=p["dmx"])
    seis.write_shot(t + "/uy", np.zeros_like(g["ux"]), sx=p["sx"], dt=p["dt"], ox=p["omx"], dx=p["dmx"])
    common = [f"{k}={t}/{k}" for k in ("ux", "uy", "uz", "mpp", "mps1", "mps2", "vp", "vs", "wav")] + [
        f"sx={p['sx']}", "sy=0", "sz=0", "gz=0", f"fmin={p['fmin']}", f"fmax={p['fmax']}", f"padt={p['padt']}",
        f"padx={p['padx']}"]

    def run(adj):
        args = ["0", "adj=" + ("y" if adj else "n")] + common
        argv = (C.c_char_p * len(args))(*[a.encode() for a in args])
        return lib.main(len(args), argv)

    assert run(True) == 0
    mpp, hp, ext = seis.read(t + "/mpp")
    mps1, _, _ = seis.read(t + "/mps1")
    mps2, hs, _ = seis.read(t + "/mps2")
    assert rel_l2(mpp, g["mpp_ref"]) < TOL and rel_l2(mps2, g["mps2_ref"]) < TOL and not np.any(mps1)
    assert np.all(hp["trid"] == 1) and np.all(hs["trid"] == 2)
    assert np.array_equal(hp["imx"], np.arange(p["nmx"])) and ext["n"][:2] == [p["nz"], p["nmx"]]

    seis.write_grid(t + "/mpp", g["mpp_in"], o1=p["oz"], d1=p["dz"], ox=p["omx"], dx=p["dmx"])
    seis.write_grid(t + "/mps1", np.zeros_like(g["mpp_in"]), o1=p["oz"], d1=p["dz"], ox=p["omx"], dx=p["dmx"])
    seis.write_grid(t + "/mps2", g["mps2_in"], o1=p["oz"], d1=p["dz"], ox=p["omx"], dx=p["dmx"])
    assert run(False) == 0
    ux, hx, ext = seis.read(t + "/ux")
    uy, _, _ = seis.read(t + "/uy")
    uz, _, _ = seis.read(t + "/uz")
    assert rel_l2(ux, g["ux_ref"]) < TOL and rel_l2(uz, g["uz_ref"]) < TOL and not np.any(uy)
    gx = p["omx"] + p["dmx"] * np.arange(p["nmx"])
    assert np.allclose(hx["gx"], gx) and np.allclose(hx["hx"], gx - p["sx"]) and np.all(hx["n1"] == p["nt"])
    assert ext["n"][:2] == [p["nt"], p["nmx"]]


def test_elastic_edge_cases(gpu_lib):
    """A source off the grid (in x, and in y on a 3-D grid), a row length with no kernel and
    a 3-D plane whose sides are not powers of two in [64, 1024] are refused with a status
    before anything runs. (ewem.c's band arithmetic always leaves at least one frequency,
    ewem.c:49-57, so there is no empty band to test.)"""
    from wemgpu import synth
    from wemgpu._lib import WemError, WEM_ERR_ARG, WEM_ERR_SIZE
    c = synth.small_case(91, nx=64, nz=8, nt=64, nshot=2, pspi=0, fmax=30.0)
    p, shots = c["params"], c["shots"]
    p3 = dict(p, nmx=32, nmy=32, omy=0.0, dmy=p["dmx"])
    for q, sx, sy, code in ((p, [1e6, 0.0], None, WEM_ERR_ARG), (dict(p, nmx=16, padx=2), shots.sx, None, WEM_ERR_SIZE),
                            (dict(p, nmx=40, nmy=4), shots.sx, [0.0, 0.0], WEM_ERR_SIZE),
                            (p3, [100.0, 100.0], [100.0, 1e6], WEM_ERR_ARG)):
        n = int(q["nmx"]) * int(q.get("nmy", 1))
        vp = np.resize(c["vel"], (n, c["vel"].shape[1]))
        zeros = np.zeros((2, n, int(q["nt"])), np.float32)
        with pytest.raises(WemError) as e:
            gpu_lib.elastic(q, vp, vp / 1.8, c["wav"], sx, sy=sy, ux=zeros, uz=zeros, adj=True)
        assert e.value.code == code


def test_elastic_least_squares_misfit_curve_vs_fp64_pair(gpu_lib):
    """Elastic least-squares migration (cg.least_squares_elastic, ShotProfileLSEWEM's solver):
    the misfit curve of CG over the GPU's migration / forward pair against CG over the FP64
    restatement's pair on the same data (modelled from a sparse random P and S reflectivity),
    within 1e-3 relative at every iteration."""
    import ewem_np as E
    from wemgpu import cg, synth
    c = synth.small_case(171, nx=64, nz=8, nt=64, nshot=2, pspi=0, fmax=25.0)
    p = dict(c["params"], fmin=3.0)
    vp = c["vel"]
    vs = (vp / 1.8).astype(np.float32)
    sx = [float(v) for v in c["shots"].sx]
    rng = np.random.default_rng(172)
    mask = rng.random((2, 64, 8)) < 0.05
    m_true = np.where(mask, rng.standard_normal((2, 64, 8)), 0.0).astype(np.float32)
    ux, uz = [], []
    for s in sx:
        a, _, b = E.ewem(dict(p, sx=s), vp, vs, c["wav"], mpp=m_true[0], mps2=m_true[1], adj=False)
        ux.append(a)
        uz.append(b)
    ux, uz = np.asarray(ux, np.float32), np.asarray(uz, np.float32)
    _, _, cost_gpu = cg.least_squares_elastic(p, vp, vs, c["wav"], sx, ux, uz, niter=4)
    w = cg.trace_weights(ux)[..., None]

    def fwd(m):
        out = [E.ewem(dict(p, sx=s), vp, vs, c["wav"], mpp=m[0], mps2=m[1], adj=False) for s in sx]
        return np.stack([np.stack([o[0] for o in out]) * w, np.stack([o[2] for o in out]) * w])

    def adj(r):
        a = b = 0.0
        for i, s in enumerate(sx):
            mp, _, ms = E.ewem(dict(p, sx=s), vp, vs, c["wav"], ux=r[0][i] * w[i], uz=r[1][i] * w[i], adj=True)
            a, b = a + mp, b + ms
        return np.stack([a, b])

    _, cost_cpu = cg.conjugate_gradients(np.stack([ux * w, uz * w]).astype(np.float64), fwd, adj, niter=4)
    print("misfit GPU", cost_gpu, "FP64", cost_cpu)
    assert len(cost_gpu) == len(cost_cpu) == 5
    assert np.all(np.abs(np.asarray(cost_gpu) - cost_cpu) <= 1e-3 * np.maximum(cost_cpu, 1e-3))


# ------------------------------------------------------------------ 3-D grids (nmy > 1)
def _ewem3d_ux(uz):
    """The x component the 3-D golden cases migrate (tests/golden/make_golden.py, ewem3d_ux)."""
    return (0.4 * uz + 0.1 * np.roll(uz, 3, axis=1)).astype(np.float32)


@pytest.mark.parametrize("case", ["ewem3d_32", "ewem3d_64x32_buried", "ewem3d_128x32_taper"])
def test_elastic3d_matches_reference_golden(gpu_lib, case):
    """3-D grids: the reference's ewem() with its rank-2 transforms over the x-y planes
    (64 x 64, 128 x 64 with the source and receivers below the surface, 256 x 64 with the
    taper on along x), migration and forward operator."""
    g = load_golden(f"{case}.npz")
    p = g["params"]
    ux = _ewem3d_ux(g["uz"])
    mpp, mps2 = gpu_lib.elastic(p, g["vp"], g["vs"], g["wav"], [p["sx"]], sy=[p["sy"]], ux=ux[None], uz=g["uz"][None],
                                adj=True)
    assert rel_l2(mpp, g["mpp_ref"]) < TOL, rel_l2(mpp, g["mpp_ref"])
    assert rel_l2(mps2, g["mps2_ref"]) < TOL, rel_l2(mps2, g["mps2_ref"])
    ux, uz = gpu_lib.elastic(p, g["vp"], g["vs"], g["wav"], [p["sx"]], sy=[p["sy"]], mpp=g["mpp_in"],
                             mps2=g["mps2_in"], adj=False)
    assert rel_l2(ux[0], g["ux_ref"]) < TOL, rel_l2(ux[0], g["ux_ref"])
    assert rel_l2(uz[0], g["uz_ref"]) < TOL, rel_l2(uz[0], g["uz_ref"])


def test_ewem_dropin_3d_matches_reference_golden(gpu_lib):
    """ewem() with the reference's argument list on a 3-D grid (nmy > 1, float** rows of the
    nmx * nmy cells)."""
    g = load_golden("ewem3d_32.npz")
    p = g["params"]
    L = gpu_lib.lib()
    fpp = C.POINTER(C.POINTER(C.c_float))
    L.ewem.restype = C.c_int
    L.ewem.argtypes = [fpp] * 7 + [C.c_int, C.c_float, C.c_float, C.c_int, C.c_float, C.c_float, C.c_int, C.c_float,
                                   C.c_float, C.c_float, C.c_float, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float,
                                   fpp, fpp, C.c_float, C.c_float, C.c_int, C.c_int, C.c_bool, C.c_bool]
    n, nt, nz = p["nmx"] * p["nmy"], p["nt"], p["nz"]
    uz = np.ascontiguousarray(g["uz"], np.float32)
    ux = _ewem3d_ux(uz)
    uy = np.full((n, nt), 7.0, np.float32)
    mpp, mps1, mps2 = (np.full((n, nz), 7.0, np.float32) for _ in range(3))
    wav = np.ascontiguousarray(g["wav"], np.float32).reshape(1, -1)
    vp, vs = np.ascontiguousarray(g["vp"], np.float32), np.ascontiguousarray(g["vs"], np.float32)
    args = [p["nt"], 0.0, p["dt"], p["nmx"], p["omx"], p["dmx"], p["nmy"], p["omy"], p["dmy"], p["sx"], p["sy"], nz,
            p["oz"], p["dz"], p["gz"], p["sz"], _rows(vp), _rows(vs), p["fmin"], p["fmax"], p["padt"], p["padx"]]
    rc = L.ewem(_rows(ux), _rows(uy), _rows(uz), _rows(mpp), _rows(mps1), _rows(mps2), _rows(wav), *args, True, False)
    assert rc == 0
    assert rel_l2(mpp, g["mpp_ref"]) < TOL and rel_l2(mps2, g["mps2_ref"]) < TOL and not np.any(mps1)


@pytest.mark.parametrize("nx,ny,padx,nshot", [(64, 32, 2, 3), (512, 32, 2, 2), (32, 512, 2, 2), (128, 64, 1, 3)])
def test_elastic3d_shots_stacked_match_fp64_oracle(gpu_lib, nx, ny, padx, nshot):
    """Several shots in one 3-D call against the FP64 restatement (oracle/ewem_np.py,
    ewem3d) shot by shot, migration and forward: planes of 128 x 64, 1024 x 64 (the column
    pass's widest transform), 64 x 1024 (the row pass's) and 128 x 64 without padding."""
    import ewem_np as E
    from wemgpu import synth
    nz = 5  # small_case3d places its scatterers between 3 dz and (nz - 1) dz
    c = synth.small_case3d(90 + nx + ny, nx=nx, ny=ny, nz=nz, nt=32, nshot=nshot, pspi=0, fmax=30.0, padx=padx)
    rng = np.random.default_rng(nx + 7 * ny)
    vp = c["vel"]
    vs = (vp / 1.7 * (1.0 + 0.05 * rng.standard_normal(vp.shape))).astype(np.float32)
    p = dict(c["params"], fmin=3.0)
    shots = c["shots"]
    uz = np.stack([synth.shot_gather_full(shots, s, nx * ny) for s in range(shots.nshot)])
    ux = (0.5 * np.roll(uz, 2, axis=2)).astype(np.float32)
    mpp, mps2 = gpu_lib.elastic(p, vp, vs, c["wav"], shots.sx, sy=shots.sy, ux=ux, uz=uz, adj=True)
    want_p = want_s = 0.0
    for s in range(shots.nshot):
        q = dict(p, sx=float(shots.sx[s]), sy=float(shots.sy[s]))
        a, _, b = E.ewem3d(q, vp, vs, c["wav"], ux=ux[s], uz=uz[s], adj=True)
        want_p, want_s = want_p + a, want_s + b
    assert rel_l2(mpp, want_p) < TOL, rel_l2(mpp, want_p)
    assert rel_l2(mps2, want_s) < TOL, rel_l2(mps2, want_s)
    m_in = [rng.standard_normal((nx * ny, nz)).astype(np.float32) for _ in range(2)]
    gx, gz = gpu_lib.elastic(p, vp, vs, c["wav"], shots.sx, sy=shots.sy, mpp=m_in[0], mps2=m_in[1], adj=False)
    for s in range(shots.nshot):
        q = dict(p, sx=float(shots.sx[s]), sy=float(shots.sy[s]))
        a, _, b = E.ewem3d(q, vp, vs, c["wav"], mpp=m_in[0], mps2=m_in[1], adj=False)
        assert rel_l2(gx[s], a) < TOL, (s, rel_l2(gx[s], a))
        assert rel_l2(gz[s], b) < TOL, (s, rel_l2(gz[s], b))


def test_elastic3d_linearity(gpu_lib):
    """The 3-D migration is linear in the data: twice the data gives exactly twice the images
    (a power-of-two scale passes every FP32 operation exactly), and the images of the x and z
    components migrated apart add up to the images of both at once."""
    from wemgpu import synth
    c = synth.small_case3d(97, nx=32, ny=32, nz=5, nt=32, nshot=2, pspi=0, fmax=25.0, padx=2)
    vp = c["vel"]
    vs = (vp / 1.8).astype(np.float32)
    p = dict(c["params"], fmin=3.0)
    shots = c["shots"]
    uz = np.stack([synth.shot_gather_full(shots, s, 32 * 32) for s in range(shots.nshot)])
    ux = (0.3 * np.roll(uz, 1, axis=2)).astype(np.float32)
    a = gpu_lib.elastic(p, vp, vs, c["wav"], shots.sx, sy=shots.sy, ux=ux, uz=uz, adj=True)
    b = gpu_lib.elastic(p, vp, vs, c["wav"], shots.sx, sy=shots.sy, ux=2 * ux, uz=2 * uz, adj=True)
    assert np.array_equal(2 * a[0], b[0]) and np.array_equal(2 * a[1], b[1])
    z = np.zeros_like(ux)
    ax = gpu_lib.elastic(p, vp, vs, c["wav"], shots.sx, sy=shots.sy, ux=ux, uz=z, adj=True)
    az = gpu_lib.elastic(p, vp, vs, c["wav"], shots.sx, sy=shots.sy, ux=z, uz=uz, adj=True)
    assert rel_l2(ax[0] + az[0], a[0]) < 1e-5 and rel_l2(ax[1] + az[1], a[1]) < 1e-5


def test_elastic3d_batches_agree(gpu_lib, monkeypatch):
    """The 3-D items (shot, frequency) run in batches when their planes exceed the memory
    budget; forcing batches of 5 items (WEM_E3_BATCH) gives the images and data of one batch to
    FP32 rounding (the imaging chunks sum the items in another grouping)."""
    from wemgpu import synth
    c = synth.small_case3d(98, nx=32, ny=32, nz=5, nt=32, nshot=3, pspi=0, fmax=25.0, padx=2)
    vp = c["vel"]
    vs = (vp / 1.8).astype(np.float32)
    p = dict(c["params"], fmin=3.0)
    shots = c["shots"]
    uz = np.stack([synth.shot_gather_full(shots, s, 32 * 32) for s in range(shots.nshot)])
    ux = (0.3 * np.roll(uz, 1, axis=2)).astype(np.float32)
    rng = np.random.default_rng(99)
    m_in = [rng.standard_normal((32 * 32, 5)).astype(np.float32) for _ in range(2)]
    one = gpu_lib.elastic(p, vp, vs, c["wav"], shots.sx, sy=shots.sy, ux=ux, uz=uz, adj=True)
    d_one = gpu_lib.elastic(p, vp, vs, c["wav"], shots.sx, sy=shots.sy, mpp=m_in[0], mps2=m_in[1], adj=False)
    monkeypatch.setenv("WEM_E3_BATCH", "5")
    many = gpu_lib.elastic(p, vp, vs, c["wav"], shots.sx, sy=shots.sy, ux=ux, uz=uz, adj=True)
    d_many = gpu_lib.elastic(p, vp, vs, c["wav"], shots.sx, sy=shots.sy, mpp=m_in[0], mps2=m_in[1], adj=False)
    assert rel_l2(many[0], one[0]) < 1e-6 and rel_l2(many[1], one[1]) < 1e-6
    assert np.array_equal(d_many[0], d_one[0]) and np.array_equal(d_many[1], d_one[1])
