"""The file-level operator ShotProfileWEM(m, d, adj; ...) over seis files
(src/Imaging/ShotProfileWEM.jl:39-310)."""
import os

import numpy as np
import pytest

from conftest import rel_l2


def _write_survey(tmp, c):
    """vel, wav and one data file holding every shot (headers sx, gx, ...), as SeisWindow
    expects to find them."""
    from wemgpu import seis, synth
    p, shots = c["params"], c["shots"]
    seis.write_grid(os.path.join(tmp, "vel"), c["vel"], o1=0.0, d1=p["dz"], ox=p["omx"], dx=p["dmx"])
    seis.write_wavelet(os.path.join(tmp, "wav"), c["wav"], dt=p["dt"])
    nx, nt = p["nmx"], p["nt"]
    datas, hs = [], []
    for s in range(shots.nshot):
        g = synth.shot_gather_full(shots, s, nx)
        h = seis.empty_headers(nx)
        h["n1"], h["d1"], h["sx"] = nt, p["dt"], shots.sx[s]
        h["gx"] = p["omx"] + p["dmx"] * np.arange(nx)
        h["imx"] = np.arange(nx)
        datas.append(g)
        hs.append(h)
    seis.write(os.path.join(tmp, "d"), np.concatenate(datas), np.concatenate(hs), [nt, nx, 1, shots.nshot, 1],
               [0.0, p["omx"], 0.0, float(shots.sx[0]), 0.0], [p["dt"], p["dmx"], 1.0, 1.0, 1.0])


def test_window_shots_selects_by_source_and_places_by_receiver(tmp_path):
    from wemgpu import seis, shotprofile
    h = seis.empty_headers(6)
    h["sx"] = [100, 100, 200, 200, 200, 300]
    h["gx"] = [0, 20, 10, 30, 40, 0]
    d = np.arange(6 * 4, dtype=np.float32).reshape(6, 4)
    g = dict(nmx=5, omx=0.0, dmx=10.0, nmy=1, omy=0.0, dmy=10.0)
    s = shotprofile.window_shots(d, h, [200.0, 100.0], [0.0, 0.0], g)
    assert list(s.trace_offset) == [0, 3, 5]
    assert list(s.trace_cell) == [1, 3, 4, 0, 2]
    assert np.array_equal(s.data[0], d[2]) and np.array_equal(s.data[3], d[0])


def test_image_headers_follow_the_reference():
    from wemgpu import shotprofile
    g = dict(nmx=3, nmy=2, dmx=10.0, dmy=5.0, nz=7, min_imx=4, min_imy=1)
    h = shotprofile.image_headers(g, 2.5)
    assert list(h["imx"]) == [4, 4, 5, 5, 6, 6] and list(h["imy"]) == [1, 2, 1, 2, 1, 2]
    assert list(h["mx"]) == [40, 40, 50, 50, 60, 60] and h["n1"][0] == 7 and h["tracenum"][0] == 2


@pytest.mark.gpu
@pytest.mark.parametrize("pspi", [0, 1])
def test_shotprofile_migration_and_demigration_on_files(gpu_lib, oracle_mod, tmp_path, pspi):
    from wemgpu import seis, synth, shotprofile
    c = synth.small_case(121, nx=64, nz=16, nt=128, nshot=3, pspi=pspi, nref=4)
    p = c["params"]
    _write_survey(str(tmp_path), c)
    sx = [float(v) for v in c["shots"].sx]
    kw = dict(pspi=bool(pspi), nref=p["nref"], vel=str(tmp_path / "vel"), wav=str(tmp_path / "wav"),
              fmin=p["fmin"], fmax=p["fmax"], padt=p["padt"], padx=p["padx"], sx=sx, sy=[0.0] * len(sx))
    shotprofile.ShotProfileWEM(str(tmp_path / "m"), str(tmp_path / "d"), True, **kw)
    m, hm, em = seis.read(str(tmp_path / "m"))
    want = None
    for s, x0 in enumerate(sx):
        g = synth.shot_gather_full(c["shots"], s, p["nmx"])
        w = oracle_mod.wem_port(dict(p, sx=x0), c["vel"], c["wav"], d=g, adj=True).astype(np.float64)
        want = w if want is None else want + w
    assert rel_l2(m, want) < 1e-4
    assert em["n"][:3] == [p["nz"], p["nmx"], 1]
    # demigration of that image back to data
    shotprofile.ShotProfileWEM(str(tmp_path / "m"), str(tmp_path / "dm"), False, **kw)
    dm, hd, ed = seis.read(str(tmp_path / "dm"))
    for s, x0 in enumerate(sx):
        w = oracle_mod.wem_port(dict(p, sx=x0), c["vel"], c["wav"], m=m, adj=False)
        assert rel_l2(dm[s * p["nmx"]:(s + 1) * p["nmx"]], w) < 1e-4
        assert np.all(hd["sx"][s * p["nmx"]:(s + 1) * p["nmx"]] == np.float32(x0))


def test_angle_binning_weights_and_adjoint():
    """Bilinear binning of ShotProfileWEM.jl:155-188 and its forward counterpart
    (:246-270) are adjoint to each other, and the weights of one sample add up to 1
    where both neighbouring bins exist."""
    from wemgpu import shotprofile as S
    rng = np.random.default_rng(5)
    n, nz = 7, 9
    spec = (6, -60.0, 20.0, 1, 0.0, 1.0)
    ax = rng.uniform(-59.0, 39.0, (n, nz))  # bins 1..5: the upper neighbour always exists
    ay = np.zeros((n, nz))
    img = rng.standard_normal((n, nz))
    out = S.bin_shot(img, ax, ay, np.zeros((n, 6, nz)), *spec)
    assert np.allclose(out.sum(axis=1), img)  # every sample lands in bins iangx < nangx
    g = rng.standard_normal((n, 6, nz))
    assert np.isclose(np.vdot(out, g), np.vdot(img, S.unbin_shot(g, ax, ay, *spec)))
    # one sample by hand: angle 5 deg, bins of 20 from -60: bin 4 (-0..) gets 0.75, bin 5 0.25
    one = S.bin_shot(np.ones((1, 1)), np.array([[5.0]]), np.zeros((1, 1)), np.zeros((1, 6, 1)), *spec)
    assert np.allclose(one[0, :, 0], [0, 0, 0, 0.75, 0.25, 0])


@pytest.mark.gpu
def test_compute_angles_and_angle_gathers_on_files(gpu_lib, tmp_path):
    """ComputeAngles on seis files (one section per shot, headers with sx), then
    ShotProfileWEM with angle bins: the gathers summed over the bins give the stacked
    image, and demigration from the gathers runs shot by shot."""
    import angles_np as A
    from wemgpu import seis, synth, shotprofile
    c = synth.small_case(123, nx=64, nz=16, nt=128, nshot=2, pspi=1, nref=3)
    p = c["params"]
    _write_survey(str(tmp_path), c)
    sx = [float(v) for v in c["shots"].sx]
    t = str(tmp_path)
    shotprofile.ComputeAngles(t + "/angx", t + "/angy", vel=t + "/vel", wav=t + "/wav", fmin=p["fmin"],
                              fmax=p["fmax"], sx=sx, sy=[0.0] * len(sx))
    a, ha, ea = seis.read(t + "/angx")
    assert a.shape == (2 * p["nmx"], p["nz"]) and list(np.unique(ha["sx"])) == sorted(np.float32(sx))
    want, _ = A.compute_angles(dict(p, sx=sx[1]), c["vel"], c["wav"])
    assert rel_l2(a[p["nmx"]:], want) < 1e-4
    kw = dict(pspi=True, nref=p["nref"], vel=t + "/vel", wav=t + "/wav", angx=t + "/angx", angy=t + "/angy",
              fmin=p["fmin"], fmax=p["fmax"], padt=p["padt"], padx=p["padx"], sx=sx, sy=[0.0] * len(sx))
    spec = dict(nangx=7, oangx=-90.0, dangx=30.0)
    gath = shotprofile.ShotProfileWEM(t + "/mg", t + "/d", True, **kw, **spec)
    stack = shotprofile.ShotProfileWEM(t + "/m", t + "/d", True, **kw)
    assert rel_l2(gath.sum(axis=1), stack) < 1e-5
    mg, hg, eg = seis.read(t + "/mg")
    assert eg["n"][:4] == [p["nz"], p["nmx"], 1, 7] and list(hg["ang"][:7]) == [-90, -60, -30, 0, 30, 60, 90]
    dd = shotprofile.ShotProfileWEM(t + "/mg", t + "/dg", False, **kw, **spec)
    assert dd.shape == (2 * p["nmx"], p["nt"]) and np.all(np.isfinite(dd)) and np.any(dd)


def _write_elastic_survey(tmp, c, vs, ux, uz):
    """vp, vs, wav and the three component files holding every shot (headers sx, gx)."""
    from wemgpu import seis
    p, shots = c["params"], c["shots"]
    grid = dict(o1=0.0, d1=p["dz"], ox=p["omx"], dx=p["dmx"])
    seis.write_grid(os.path.join(tmp, "vp"), c["vel"], **grid)
    seis.write_grid(os.path.join(tmp, "vs"), vs, **grid)
    seis.write_wavelet(os.path.join(tmp, "wav"), c["wav"], dt=p["dt"])
    nx, nt = p["nmx"], p["nt"]
    hs = []
    for s in range(shots.nshot):
        h = seis.empty_headers(nx)
        h["n1"], h["d1"], h["sx"] = nt, p["dt"], shots.sx[s]
        h["gx"] = p["omx"] + p["dmx"] * np.arange(nx)
        h["imx"] = np.arange(nx)
        hs.append(h)
    for name, a in (("ux", ux), ("uy", np.zeros_like(ux)), ("uz", uz)):
        seis.write(os.path.join(tmp, name), a.reshape(-1, nt), np.concatenate(hs), [nt, nx, 1, shots.nshot, 1],
                   [0.0, p["omx"], 0.0, float(shots.sx[0]), 0.0], [p["dt"], p["dmx"], 1.0, 1.0, 1.0])


def _write_shot_angles(name, values, sx, p):
    from wemgpu import seis
    nx, nz = p["nmx"], p["nz"]
    h = np.concatenate([seis.grid_headers(nx, nz, 0.0, p["dz"], p["omx"], p["dmx"]) for _ in sx])
    h["sx"] = np.repeat(np.asarray(sx, np.float32), nx)
    seis.write(name, values.reshape(-1, nz).astype(np.float32), h, [nz, nx, 1, len(sx), 1],
               [0.0, p["omx"], 0.0, sx[0], 0.0], [p["dz"], p["dmx"], 1.0, 1.0, 1.0])


@pytest.mark.gpu
def test_shotprofile_ewem_on_files_with_and_without_angle_gathers(gpu_lib, tmp_path):
    """ShotProfileEWEM (ShotProfileEWEM.jl:38-411) over seis files: the stacked P and S images
    against the FP64 restatement of ewem shot by shot; angle gathers summed over the bins give
    the P stack and the angle-signed S stack; demigration without gathers against the FP64
    forward operator."""
    import ewem_np as E
    from wemgpu import seis, synth, shotprofile
    c = synth.small_case(131, nx=64, nz=10, nt=128, nshot=2, pspi=0, fmax=30.0)
    p = dict(c["params"], fmin=3.0)
    rng = np.random.default_rng(5)
    vs = (c["vel"] / 1.7).astype(np.float32)
    shots, nx, nz = c["shots"], p["nmx"], p["nz"]
    uz = np.stack([synth.shot_gather_full(shots, s, nx) for s in range(shots.nshot)])
    ux = (0.5 * np.roll(uz, 3, axis=2)).astype(np.float32)
    t = str(tmp_path)
    _write_elastic_survey(t, c, vs, ux, uz)
    sx = [float(v) for v in shots.sx]
    kw = dict(vp=t + "/vp", vs=t + "/vs", wav=t + "/wav", fmin=p["fmin"], fmax=p["fmax"], padt=p["padt"],
              padx=p["padx"], sx=sx, sy=[0.0] * len(sx), angx=t + "/angx", angy=t + "/angy")
    m = [t + "/mpp", t + "/mps1", t + "/mps2"]
    d = [t + "/ux", t + "/uy", t + "/uz"]
    mpp, mps1, mps2 = shotprofile.ShotProfileEWEM(m, d, True, **kw)
    per = [E.ewem(dict(p, sx=x0), c["vel"], vs, c["wav"], ux=ux[s], uz=uz[s], adj=True) for s, x0 in enumerate(sx)]
    assert rel_l2(mpp, sum(a for a, _, _ in per)) < 1e-4 and rel_l2(mps2, sum(b for _, _, b in per)) < 1e-4
    assert not np.any(mps1)
    f, h, e = seis.read(t + "/mpp")
    assert e["n"][:2] == [nz, nx] and np.array_equal(h["imx"], np.arange(nx))

    ang = rng.uniform(-50.0, 50.0, (len(sx), nx, nz))
    _write_shot_angles(t + "/angx", ang, sx, p)
    _write_shot_angles(t + "/angy", np.zeros_like(ang), sx, p)
    spec = dict(nangx=7, oangx=-60.0, dangx=20.0)
    gp, g1, gs = shotprofile.ShotProfileEWEM([t + "/gpp", t + "/gps1", t + "/gps2"], d, True, **kw, **spec)
    assert gp.shape == (nx, 7, nz)
    signed = sum(np.where(ang[s] < 0, -1.0, 1.0) * per[s][2] for s in range(len(sx)))
    assert rel_l2(gp.sum(axis=1), mpp) < 1e-5 and rel_l2(gs.sum(axis=1), signed) < 1e-4 and not np.any(g1)

    ux2, uz2 = shotprofile.ShotProfileEWEM(m, [t + "/dx", t + "/dy", t + "/dz"], False, **kw)
    for s, x0 in enumerate(sx):
        wx, _, wz = E.ewem(dict(p, sx=x0), c["vel"], vs, c["wav"], mpp=mpp, mps2=mps2, adj=False)
        assert rel_l2(ux2[s], wx) < 1e-4 and rel_l2(uz2[s], wz) < 1e-4
    dx_, hdx, _ = seis.read(t + "/dx")
    assert dx_.shape == (len(sx) * nx, p["nt"]) and np.allclose(hdx["sx"][nx:], sx[1])
    gdx = shotprofile.ShotProfileEWEM([t + "/gpp", t + "/gps1", t + "/gps2"], [t + "/ex", t + "/ey", t + "/ez"],
                                      False, **kw, **spec)
    assert np.all(np.isfinite(gdx[0])) and np.any(gdx[0]) and np.any(gdx[1])


def test_shotprofile_ewem_file_plumbing_with_a_fake_operator(tmp_path, monkeypatch):
    """The host side of ShotProfileEWEM (ShotProfileEWEM.jl:38-411) on CPU: the GPU call is
    replaced by a deterministic fake (each shot's P image = sx * column sums of its ux traces,
    S image = -the same of uz; modelling = the images broadcast over time), so the test checks
    what the operator itself does with files: windowing by sx, placing traces by gx, stacking,
    angle binning with the S images signed by the angles, unbinning, and the data headers."""
    from wemgpu import seis, synth, shotprofile, api
    c = synth.small_case(131, nx=32, nz=6, nt=16, nshot=2, pspi=0, fmax=30.0)
    p, shots, nx, nz, nt = c["params"], c["shots"], 32, 6, 16
    rng = np.random.default_rng(9)
    uz = rng.standard_normal((shots.nshot, nx, nt)).astype(np.float32)
    ux = rng.standard_normal((shots.nshot, nx, nt)).astype(np.float32)
    calls = []

    def fake_elastic(params, vp, vs, wav, sx, sy=None, ux=None, uz=None, mpp=None, mps2=None, adj=True, device=0):
        sx = np.atleast_1d(sx).astype(np.float64)
        calls.append((adj, len(sx)))
        if adj:
            a = sum(x * np.repeat(u.sum(axis=1, keepdims=True), nz, 1) for x, u in zip(sx, ux))
            b = sum(-x * np.repeat(u.sum(axis=1, keepdims=True), nz, 1) for x, u in zip(sx, uz))
            return a.astype(np.float32), b.astype(np.float32)
        return (np.stack([np.repeat(mpp[:, :1], nt, 1) * x for x in sx]).astype(np.float32),
                np.stack([np.repeat(mps2[:, :1], nt, 1) * x for x in sx]).astype(np.float32))

    monkeypatch.setattr(api, "elastic", fake_elastic)
    t = str(tmp_path)
    _write_elastic_survey(t, c, (c["vel"] / 1.7).astype(np.float32), ux, uz)
    sx = [float(v) for v in shots.sx]
    kw = dict(vp=t + "/vp", vs=t + "/vs", wav=t + "/wav", sx=sx, sy=[0.0] * 2, angx=t + "/angx", angy=t + "/angy")
    m = [t + "/mpp", t + "/mps1", t + "/mps2"]
    d = [t + "/ux", t + "/uy", t + "/uz"]
    mpp, mps1, mps2 = shotprofile.ShotProfileEWEM(m, d, True, **kw)
    want_p, want_s = fake_elastic(p, None, None, None, sx, ux=ux, uz=uz)
    assert np.allclose(mpp, want_p) and np.allclose(mps2, want_s) and not np.any(mps1) and calls[-1] == (True, 2)
    got, h, e = seis.read(t + "/mpp")
    assert e["n"][:2] == [nz, nx] and np.allclose(got, want_p)

    ang = rng.uniform(-50.0, 50.0, (2, nx, nz))
    _write_shot_angles(t + "/angx", ang, sx, p)
    _write_shot_angles(t + "/angy", np.zeros_like(ang), sx, p)
    spec = dict(nangx=7, oangx=-60.0, dangx=20.0)
    gp, _, gs = shotprofile.ShotProfileEWEM([t + "/gpp", t + "/gps1", t + "/gps2"], d, True, **kw, **spec)
    per = [fake_elastic(p, None, None, None, [sx[i]], ux=ux[i:i + 1], uz=uz[i:i + 1]) for i in range(2)]
    assert np.allclose(gp.sum(axis=1), mpp, rtol=1e-5, atol=1e-3)
    signed = sum(np.where(ang[i] < 0, -1.0, 1.0) * per[i][1] for i in range(2))
    assert np.allclose(gs.sum(axis=1), signed, rtol=1e-5, atol=1e-3)
    _, hg, eg = seis.read(t + "/gpp")
    assert eg["n"][:4] == [nz, nx, 1, 7] and list(hg["ang"][:7]) == [-60, -40, -20, 0, 20, 40, 60]

    ux2, uz2 = shotprofile.ShotProfileEWEM(m, [t + "/dx", t + "/dy", t + "/dz"], False, **kw)
    assert np.allclose(ux2[1], np.repeat(mpp[:, :1], nt, 1) * sx[1]) and calls[-1] == (False, 2)
    dx_, hdx, edx = seis.read(t + "/dx")
    dy_, _, _ = seis.read(t + "/dy")
    gx = p["omx"] + p["dmx"] * np.arange(nx)
    assert dx_.shape == (2 * nx, nt) and not np.any(dy_) and edx["n"][:4] == [nt, nx, 1, 2]
    assert np.allclose(hdx["sx"][nx:], sx[1]) and np.allclose(hdx["gx"][:nx], gx) and np.allclose(hdx["hx"][:nx], gx - sx[0])


class _FakeContext:
    """Stands in for wemgpu.Context in a CPU test of the file plumbing: a shot's image is
    sx * the sum of its traces over time at each cell (nz copies); modelling puts the image's
    first depth sample times sx on every time sample."""

    def __init__(self, nz, nt):
        self.nz, self.nt, self.calls = nz, nt, []

    def prepare(self, params, vel, wav):
        self.params = params
        return self

    def migrate(self, shots):
        n = self.params["nmx"] * self.params["nmy"]
        img = np.zeros((n, self.nz))
        for s in range(shots.nshot):
            lo, hi = int(shots.trace_offset[s]), int(shots.trace_offset[s + 1])
            for cell, tr in zip(shots.trace_cell[lo:hi], shots.data[lo:hi]):
                img[cell] += float(shots.sx[s]) * tr.sum()
        self.calls.append(("migrate", shots.nshot))
        return img.astype(np.float32)

    def model(self, shots, m, exact=False):
        out = []
        for s in range(shots.nshot):
            lo, hi = int(shots.trace_offset[s]), int(shots.trace_offset[s + 1])
            out.append(np.repeat(m[shots.trace_cell[lo:hi], :1], self.nt, 1) * float(shots.sx[s]))
        self.calls.append(("model", shots.nshot))
        return np.concatenate(out).astype(np.float32)


def test_shotprofile_wem_file_plumbing_with_a_fake_context(tmp_path):
    """The host side of ShotProfileWEM (ShotProfileWEM.jl:39-310) on CPU with a fake context:
    the survey file windowed by sx and placed by gx, one batched call for the stack, one call
    per shot for angle gathers (their sum over the bins is the stack), and the modelled data's
    layout and headers."""
    from wemgpu import seis, synth, shotprofile
    c = synth.small_case(141, nx=32, nz=6, nt=16, nshot=3, pspi=1, nref=3)
    p, shots = c["params"], c["shots"]
    t = str(tmp_path)
    _write_survey(t, c)
    sx = [float(v) for v in shots.sx]
    fake = _FakeContext(p["nz"], p["nt"])
    kw = dict(vel=t + "/vel", wav=t + "/wav", sx=sx, sy=[0.0] * 3, ctx=fake, angx=t + "/angx", angy=t + "/angy")
    img = shotprofile.ShotProfileWEM(t + "/m", t + "/d", True, **kw)
    want = sum(s * np.repeat(synth.shot_gather_full(shots, i, 32).sum(axis=1, keepdims=True), p["nz"], 1)
               for i, s in enumerate(sx))
    assert np.allclose(img, want, rtol=1e-5) and fake.calls == [("migrate", 3)]
    got, h, e = seis.read(t + "/m")
    assert np.allclose(got, want, rtol=1e-5) and e["n"][:2] == [p["nz"], 32]

    ang = np.random.default_rng(2).uniform(-50.0, 50.0, (3, 32, p["nz"]))
    _write_shot_angles(t + "/angx", ang, sx, p)
    _write_shot_angles(t + "/angy", np.zeros_like(ang), sx, p)
    gath = shotprofile.ShotProfileWEM(t + "/mg", t + "/d", True, **kw, nangx=7, oangx=-60.0, dangx=20.0)
    assert gath.shape == (32, 7, p["nz"]) and np.allclose(gath.sum(axis=1), want, rtol=1e-5)
    assert fake.calls[1:] == [("migrate", 1)] * 3

    data = shotprofile.ShotProfileWEM(t + "/m", t + "/dm", False, **kw)
    assert data.shape == (3 * 32, p["nt"]) and fake.calls[-1] == ("model", 3)
    assert np.allclose(data[32:64], np.repeat(got[:, :1], p["nt"], 1) * sx[1], rtol=1e-5)
    _, hd, ed = seis.read(t + "/dm")
    assert ed["n"][:4] == [p["nt"], 32, 1, 3] and np.allclose(hd["sx"][64:], sx[2])
    assert np.allclose(hd["gx"][:32], p["omx"] + p["dmx"] * np.arange(32))


class _LinearContext:
    """A stand-in context whose model/migrate are an exact adjoint pair: every trace of shot s
    at cell c is (1 + s) K m[c], K a fixed random (nt x nz) matrix."""

    def __init__(self, nz, nt, seed=3):
        self.K = np.random.default_rng(seed).standard_normal((nt, nz)).astype(np.float64)

    def prepare(self, params, vel, wav):
        self.params = params
        return self

    def _each(self, shots):
        for s in range(shots.nshot):
            lo, hi = int(shots.trace_offset[s]), int(shots.trace_offset[s + 1])
            yield s, lo, hi

    def model(self, shots, m, exact=False):
        out = np.zeros((int(shots.trace_offset[-1]), self.K.shape[0]))
        for s, lo, hi in self._each(shots):
            out[lo:hi] = (1 + s) * m[shots.trace_cell[lo:hi]].astype(np.float64) @ self.K.T
        return out.astype(np.float32)

    def migrate(self, shots):
        img = np.zeros((self.params["nmx"] * self.params["nmy"], self.K.shape[1]))
        for s, lo, hi in self._each(shots):
            np.add.at(img, shots.trace_cell[lo:hi], (1 + s) * shots.data[lo:hi].astype(np.float64) @ self.K)
        return img.astype(np.float32)


def test_shotprofile_lswem_on_files_with_a_linear_stand_in(tmp_path):
    """ShotProfileLSWEM(m, m0, d, param) (ShotProfileLSWEM.jl:1-20) on CPU: the cost file of the
    file-level ConjugateGradients (start line, 1.0, one cost per iteration), a decreasing misfit,
    dead traces left out (CalculateSampling's weights), and the same result as conjugate_gradients
    on the same operator pair and live traces."""
    from wemgpu import seis, synth, shotprofile, cg
    c = synth.small_case(151, nx=24, nz=5, nt=12, nshot=2, pspi=1, nref=3)
    t = str(tmp_path)
    _write_survey(t, c)
    data, hd, ed = seis.read(t + "/d")
    data[3] = 0.0  # a dead trace: weight 0
    seis.write(t + "/d", data, hd, ed["n"], ed["o"], ed["d"])
    sx = [float(v) for v in c["shots"].sx]
    fake = _LinearContext(5, 12)
    param = dict(vel=t + "/vel", wav=t + "/wav", sx=sx, sy=[0.0, 0.0], Niter=6, cost=t + "/cost")
    img, cost = shotprofile.ShotProfileLSWEM(t + "/m", t + "/m0", t + "/d", param, ctx=fake)
    lines = open(t + "/cost").read().splitlines()
    assert lines[0].startswith("began execution at: ") and len(lines) == 2 + 6
    assert np.allclose([float(v) for v in lines[1:]], cost) and cost[0] == 1.0
    assert np.all(np.diff(cost) <= 1e-12) and cost[-1] < cost[1]  # CG on an exact pair: the misfit never grows
    g = shotprofile.grid_from_velocity(t + "/vel")[2]
    shots = shotprofile._live_traces(shotprofile.window_shots(data, hd, sx, [0.0, 0.0], g))
    live = int(np.sum(np.sum(data.astype(np.float64) ** 2, axis=1) > 1e-10))
    assert int(shots.trace_offset[-1]) == live < len(data)
    fake.prepare(dict(nmx=24, nmy=1), None, None)
    want, wcost = cg.conjugate_gradients(shots.data, lambda m: fake.model(shots, m),
                                         lambda r: fake.migrate(shotprofile.Shots(shots.sx, shots.sy, shots.trace_offset,
                                                                                  shots.trace_cell, r)), niter=6)
    assert np.allclose(img, want, rtol=1e-5, atol=1e-6) and np.allclose(cost, wcost)
    m_file, hm, em = seis.read(t + "/m")
    assert np.allclose(m_file, img) and em["n"][:2] == [5, 24]


def test_shotprofile_lsewem_on_files_with_a_linear_stand_in(tmp_path, monkeypatch):
    """ShotProfileLSEWEM(m, m0, d, param) (ShotProfileLSEWEM.jl:1-19) on CPU with a linear stand-in
    for wem_elastic (an exact adjoint pair): the two-image CG with one mu per image, its cost file,
    the three image files (mps1 zero)."""
    from wemgpu import seis, synth, shotprofile, api, cg
    c = synth.small_case(161, nx=16, nz=4, nt=10, nshot=2, pspi=0, fmax=30.0)
    p, shots = c["params"], c["shots"]
    rng = np.random.default_rng(4)
    Ka, Kb = rng.standard_normal((10, 4)), rng.standard_normal((10, 4))

    def fake_elastic(params, vp, vs, wav, sx, sy=None, ux=None, uz=None, mpp=None, mps2=None, adj=True, device=0):
        ns = len(np.atleast_1d(sx))
        if adj:
            a = sum((1 + s) * ux[s].astype(np.float64) @ Ka for s in range(ns))
            b = sum((1 + s) * uz[s].astype(np.float64) @ Kb for s in range(ns))
            return a.astype(np.float32), b.astype(np.float32)
        return (np.stack([(1 + s) * mpp.astype(np.float64) @ Ka.T for s in range(ns)]).astype(np.float32),
                np.stack([(1 + s) * mps2.astype(np.float64) @ Kb.T for s in range(ns)]).astype(np.float32))

    monkeypatch.setattr(api, "elastic", fake_elastic)
    ux = rng.standard_normal((2, 16, 10)).astype(np.float32)
    uz = rng.standard_normal((2, 16, 10)).astype(np.float32)
    t = str(tmp_path)
    _write_elastic_survey(t, c, (c["vel"] / 1.7).astype(np.float32), ux, uz)
    sx = [float(v) for v in shots.sx]
    param = dict(vp=t + "/vp", vs=t + "/vs", wav=t + "/wav", sx=sx, sy=[0.0, 0.0], Niter=5, mu=[0.1, 0.2],
                 cost=t + "/cost.txt")
    mpp, mps2, cost = shotprofile.ShotProfileLSEWEM([t + "/mpp", t + "/mps1", t + "/mps2"], None,
                                                   [t + "/ux", t + "/uy", t + "/uz"], param)
    a, b, wcost = cg.least_squares_elastic(p, None, None, None, sx, ux, uz, niter=5, mu=(0.1, 0.2))
    assert np.allclose(mpp, a, rtol=1e-5, atol=1e-6) and np.allclose(mps2, b, rtol=1e-5, atol=1e-6)
    assert np.allclose(cost, wcost) and cost[-1] < cost[1]
    lines = open(t + "/cost.txt").read().splitlines()
    assert lines[0].startswith("began execution at: ") and len(lines) == 2 + 5
    f1, _, e1 = seis.read(t + "/mps1")
    assert not np.any(f1) and e1["n"][:2] == [4, 16]
