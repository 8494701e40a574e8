"""Parity of the CUDA migration (called through the C ABI) with the oracle.

Tolerance: relative L2 image error <= 1e-4 against the reference's arithmetic (the
port / the reference's golden outputs) and against the FP64 operator. The GPU
computes in complex FP32 like the reference, so the expected error is the FP32
floor (1e-6 .. 1e-5).
"""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import load_golden, rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-4

GOLDEN_CASES = ["ss_64", "ss_128_taper", "pspi_64", "pspi_128_r8", "pspi_64_padx1", "pspi_500_padx2", "ss_300_padx2", "pspi_768_padx2", "pspi_97_padx1", "ss_50_padx1", "ss_64_buried", "pspi_64_buried"]


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_wem_dropin_matches_reference_golden(gpu_lib, case):
    """wem() (wem.h:3-11 signature, float** rows) vs the reference's own output."""
    g = load_golden(f"wem_{case}.npz")
    m = gpu_lib.wem_dropin(g["params"], g["vel"], g["wav"], d=g["d"], adj=True)
    assert rel_l2(m, g["m_ref"]) < TOL


@pytest.mark.parametrize("case", ["pspi_64_nt97_padt1", "ss_64_nt97_padt1"])
def test_odd_trace_length_with_padt1_matches_reference_golden(gpu_lib, case):
    """padt = 1 with an odd nt: the transform is one sample shorter than the trace, so the last
    sample takes no part in migration (wem.c:490-493); modelled traces match the reference on
    every sample but the last (the reference reads past its buffer there, wem.c:505-507)."""
    g = load_golden(f"wem_{case}.npz")
    p = g["params"]
    assert p["nt"] % 2 == 1 and p["padt"] == 1
    m = gpu_lib.wem_dropin(p, g["vel"], g["wav"], d=g["d"], adj=True)
    assert rel_l2(m, g["m_ref"]) < TOL
    d = gpu_lib.wem_dropin(p, g["vel"], g["wav"], m=g["m_in"], adj=False)
    assert rel_l2(d[:, :-1], g["d_ref"][:, :-1]) < TOL


def _port_stack(oracle_mod, p, vel, wav, shots, fp64=False):
    from wemgpu import synth
    op = oracle_mod.wem_fp64 if fp64 else oracle_mod.wem_port
    img = None
    for s in range(shots.nshot):
        q = dict(p, sx=float(shots.sx[s]), sy=float(shots.sy[s]))
        d = synth.shot_gather_full(shots, s, p["nmx"])
        m = op(q, vel, wav, d=d, adj=True).astype(np.float64)
        img = m if img is None else img + m
    return img


@pytest.mark.parametrize("pspi,interp", [(0, "ref"), (1, "ref"), (1, "linear")])
def test_batched_survey_matches_oracle(gpu_lib, oracle_mod, pspi, interp):
    """Several shots with uneven apertures in one call vs the oracle shot by shot,
    stacked like ShotProfileWEM.jl:140-199."""
    from wemgpu import synth
    c = synth.small_case(21, nx=64, nz=24, nt=128, nshot=5, pspi=pspi, nref=5, interp=interp)
    m = gpu_lib.migrate(c["params"], c["vel"], c["wav"], c["shots"])
    want = _port_stack(oracle_mod, c["params"], c["vel"], c["wav"], c["shots"])
    assert rel_l2(m, want) < TOL
    want64 = _port_stack(oracle_mod, c["params"], c["vel"], c["wav"], c["shots"], fp64=True)
    assert rel_l2(m, want64) < TOL


@pytest.mark.parametrize("nx,padx", [(16, 2), (32, 1), (128, 2), (256, 2), (512, 2), (1024, 2), (2048, 2)])
def test_row_lengths(gpu_lib, oracle_mod, nx, padx):
    """Every FFT length the kernel is built for (nkx = 32 .. 4096)."""
    from wemgpu import synth
    c = synth.small_case(31 + nx, nx=nx, nz=6, nt=64, nshot=2, pspi=1, nref=3, fmax=30.0, padx=padx)
    m = gpu_lib.migrate(c["params"], c["vel"], c["wav"], c["shots"])
    want = _port_stack(oracle_mod, c["params"], c["vel"], c["wav"], c["shots"])
    assert rel_l2(m, want) < TOL


@pytest.mark.parametrize("nx,padx,pspi,interp", [
    (500, 2, 1, "ref"), (500, 2, 1, "linear"), (300, 2, 0, "ref"), (768, 2, 1, "ref"), (1023, 2, 1, "linear"),
    (97, 1, 1, "ref"), (50, 1, 0, "ref"), (1000, 1, 1, "ref"), (9, 1, 1, "linear")])
def test_row_lengths_not_power_of_two(gpu_lib, oracle_mod, nx, padx, pspi, interp):
    """nkx = padx*nmx of any length in [9, 2048] (the reference plans FFTW transforms of any
    length, wem.c:103-104): nkx 1000, 600, 1536, 2046, 97 (prime), 50, 1000, 9. The depth
    kernels run them on power-of-two rows in Bluestein's chirp form; several shots against
    the port and the FP64 operator."""
    from wemgpu import synth
    c = synth.small_case(61 + nx + padx, nx=nx, nz=8, nt=128, nshot=3, pspi=pspi, nref=4, interp=interp,
                         fmax=30.0, padx=padx)
    m = gpu_lib.migrate(c["params"], c["vel"], c["wav"], c["shots"])
    want = _port_stack(oracle_mod, c["params"], c["vel"], c["wav"], c["shots"])
    want64 = _port_stack(oracle_mod, c["params"], c["vel"], c["wav"], c["shots"], fp64=True)
    assert rel_l2(want, want64) < TOL  # the reference's own FP32 floor on this case
    assert rel_l2(m, want64) < TOL
    assert rel_l2(m, want) < TOL


def test_row_length_limits(gpu_lib):
    """Lengths with no kernel are refused with WEM_ERR_SIZE instead of running anything:
    below 9, non-powers of two above 2048 (their chirp rows would exceed 4096 samples),
    and the split16 form off its 2048-point rows."""
    from wemgpu import synth
    from wemgpu._lib import WemError, WEM_ERR_SIZE
    c = synth.small_case(5, nx=64, nz=4, nt=64, nshot=1)
    for nmx, padx, prec in ((4, 2, "fp32"), (2049, 1, "fp32"), (500, 2, "split16")):
        p = dict(c["params"], nmx=nmx, padx=padx, precision=prec)
        vel = np.full((nmx, 4), 2000.0, np.float32)
        with gpu_lib.Context() as ctx:
            with pytest.raises(WemError) as e:
                ctx.prepare(p, vel, c["wav"])
            assert e.value.code == WEM_ERR_SIZE


# (nmx, nref, whether the tables leave shared memory: True when neither CTA shape holds them,
# False when both do, None when only the narrow one does and the autotuner decides); padx = 2,
# so rows of 2 nmx points. Shared memory holds up to 41 / 29 references (narrow / wide shape)
# at 1024 points, 19 / 13 at 2048, 5 at 4096.
MANY_REF_CASES = [(512, 24, False), (512, 64, True), (1024, 12, False), (1024, 16, None), (1024, 40, True),
                  (1024, 64, True), (2048, 5, False), (2048, 24, True), (2048, 64, True)]


@pytest.mark.parametrize("interp", ["ref", "linear"])
@pytest.mark.parametrize("nmx,nref,device_tables", MANY_REF_CASES)
def test_many_reference_velocities(gpu_lib, oracle_mod, interp, nmx, nref, device_tables):
    """Rows of 1024, 2048 and 4096 points: reference counts whose phase tables fit in shared
    memory beside the rows keep them there; larger counts (up to the reference's 64) read the
    precomputed tables in device memory instead. Every count matches the port."""
    from wemgpu import synth
    c = synth.small_case(83, nx=nmx, nz=6, nt=64, nshot=2, pspi=1, nref=nref, interp=interp, fmax=20.0)
    p = c["params"]
    assert p["nmx"] * p["padx"] == 2 * nmx and p["nref"] == nref
    with gpu_lib.Context() as ctx:
        m = ctx.prepare(p, c["vel"], c["wav"]).migrate(c["shots"])
        form = ctx.last_launch().get("form")
    want = _port_stack(oracle_mod, p, c["vel"], c["wav"], c["shots"])
    assert rel_l2(m, want) < TOL, (nref, form, rel_l2(m, want))
    if device_tables is not None:
        assert (form == "fp32-device-tables") == device_tables, (nref, form)


def test_untuned_shape_keeps_tables_in_shared_memory(gpu_lib, monkeypatch):
    """Without the autotuner the launch takes the wide CTA shape unless only the narrow one
    holds the phase tables in shared memory: 16 references at 2048 points run narrow."""
    from wemgpu import synth
    monkeypatch.setenv("WEM_AUTOTUNE", "0")
    c = synth.small_case(83, nx=1024, nz=6, nt=64, nshot=2, pspi=1, nref=16, interp="ref", fmax=20.0)
    with gpu_lib.Context() as ctx:
        ctx.prepare(c["params"], c["vel"], c["wav"]).migrate(c["shots"])
        ll = ctx.last_launch()
    assert ll["threads"] == 256 and ll["form"] != "fp32-device-tables", ll


def test_many_reference_velocities_without_tables(gpu_lib, monkeypatch):
    """With the precomputed tables switched off (WEM_PHASE_TABLES=0) the depth kernel builds
    each depth's tables in shared memory, so 40 references at 2048 points do not fit and the
    call is refused with WEM_ERR_SIZE instead of running."""
    from wemgpu import synth
    from wemgpu._lib import WemError, WEM_ERR_SIZE
    monkeypatch.setenv("WEM_PHASE_TABLES", "0")
    c = synth.small_case(83, nx=1024, nz=6, nt=64, nshot=2, pspi=1, nref=40, interp="ref", fmax=20.0)
    with gpu_lib.Context() as ctx:
        with pytest.raises(WemError) as e:
            ctx.prepare(c["params"], c["vel"], c["wav"]).migrate(c["shots"])
        assert e.value.code == WEM_ERR_SIZE


def test_deterministic(gpu_lib):
    from wemgpu import synth
    c = synth.small_case(41, nx=128, nz=16, nt=96, nshot=4)
    with gpu_lib.Context() as ctx:
        ctx.prepare(c["params"], c["vel"], c["wav"])
        a = ctx.migrate(c["shots"])
        b = ctx.migrate(c["shots"])
    assert np.array_equal(a, b)


def test_graph_replay_matches_direct_launch(gpu_lib, monkeypatch):
    """A second call with the same shots replays the captured CUDA graph of the whole
    launch sequence. Its image equals the directly launched one bit for bit, and new data
    in the same buffers is migrated afresh: data x2 gives exactly image x2 (scaling by a
    power of two commutes with every FP32 rounding)."""
    from wemgpu import synth
    from wemgpu.api import Shots
    c = synth.small_case(43, nx=128, nz=16, nt=96, nshot=4, pspi=1, nref=4)
    s = c["shots"]
    s2 = Shots(s.sx, s.sy, s.trace_offset, s.trace_cell, s.data * np.float32(2))
    with gpu_lib.Context() as ctx:
        ctx.prepare(c["params"], c["vel"], c["wav"])
        a = ctx.migrate(s)
        la = ctx.last_launch()
        b = ctx.migrate(s)
        lb = ctx.last_launch()
        d2 = ctx.migrate(s2)
        lc = ctx.last_launch()
    monkeypatch.setenv("WEM_GRAPH", "0")
    with gpu_lib.Context() as ctx:
        ctx.prepare(c["params"], c["vel"], c["wav"])
        direct = ctx.migrate(s)
        ld = ctx.last_launch()
    assert (la["graph_replayed"], lb["graph_replayed"], lc["graph_replayed"], ld["graph_replayed"]) == (0, 1, 1, 0)
    assert la["threads"] == ld["threads"] and la["grid"] == ld["grid"]
    assert np.array_equal(a, b) and np.array_equal(a, direct)
    assert np.array_equal(d2, a * np.float32(2))


def test_autotuned_cta_shape(gpu_lib, oracle_mod, monkeypatch):
    """The first migration of a geometry times both CTA shapes and keeps the faster one
    for the process; both shapes, forced, match the oracle."""
    from wemgpu import synth
    monkeypatch.delenv("WEM_CTA_SHAPE", raising=False)
    monkeypatch.delenv("WEM_AUTOTUNE", raising=False)
    c = synth.small_case(45, nx=256, nz=12, nt=96, nshot=3, pspi=1, nref=7)  # nref=7: a geometry no other test uses
    want = _port_stack(oracle_mod, c["params"], c["vel"], c["wav"], c["shots"])
    with gpu_lib.Context() as ctx:
        ctx.prepare(c["params"], c["vel"], c["wav"])
        m1 = ctx.migrate(c["shots"])
        l1 = ctx.last_launch()
    with gpu_lib.Context() as ctx:
        ctx.prepare(c["params"], c["vel"], c["wav"])
        ctx.migrate(c["shots"])
        l2 = ctx.last_launch()
    assert l1["tuned"] == 1 and l2["tuned"] == 0 and l1["threads"] == l2["threads"]
    assert rel_l2(m1, want) < TOL
    threads = set()
    for shape in ("wide", "narrow"):
        monkeypatch.setenv("WEM_CTA_SHAPE", shape)
        with gpu_lib.Context() as ctx:
            ctx.prepare(c["params"], c["vel"], c["wav"])
            m = ctx.migrate(c["shots"])
            threads.add(ctx.last_launch()["threads"])
        assert rel_l2(m, want) < TOL
    assert len(threads) == 2 and l1["threads"] in threads


@pytest.mark.parametrize("nref", [3, 8])
def test_paired_inverse_transforms(gpu_lib, oracle_mod, monkeypatch, nref):
    """The nearest-lower PSPI mode takes the real parts of two reference wavefields from
    one inverse transform wherever every point that takes them keeps the real part only
    (wem.c:454-455, 473-478). Depth levels of three kinds: random velocities (real parts;
    the reference of the row maximum taken whole), a velocity range of 40 m/s (reference
    spacing <= 10 m/s: every reference taken whole, wem.c:457-458) and constant velocity
    (vmax <= vmin + 10: reference 0 taken whole, wem.c:55-67); random levels whose maximum
    is taken by 3 points (their imaginary parts by direct sums) and by 5 points (the
    reference keeps a transform of its own). Against the port and against one transform
    per reference (WEM_PAIRED=0); the phase tables precomputed for every (frequency,
    depth) give the image bit for bit that tables built in each CTA give
    (WEM_PHASE_TABLES=0). The autotuner is off so that each run takes the form its switches
    name, in the same CTA shape."""
    from wemgpu import synth
    monkeypatch.setenv("WEM_AUTOTUNE", "0")  # the forms the switches name, not the tuner's pick
    c = synth.small_case(47, nx=256, nz=18, nt=96, nshot=3, pspi=1, nref=nref, interp="ref")
    rng = np.random.default_rng(48)
    vel = c["vel"].copy()
    vel[:, 6:9] = 2500.0
    vel[:, 9:12] = 2500.0 + 40.0 * rng.random((vel.shape[0], 3))
    for iz, pts in ((12, [3, 100, 200]), (13, [7, 8, 9, 150, 250])):
        vel[pts, iz] = vel[:, iz].max()
    want = _port_stack(oracle_mod, c["params"], vel, c["wav"], c["shots"])
    images = []
    for paired in ("1", "0"):
        monkeypatch.setenv("WEM_PAIRED", paired)
        with gpu_lib.Context() as ctx:
            ctx.prepare(c["params"], vel, c["wav"])
            images.append(ctx.migrate(c["shots"]))
        assert rel_l2(images[-1], want) < TOL, (paired, rel_l2(images[-1], want))
    assert rel_l2(images[0], images[1]) < 1e-5
    monkeypatch.setenv("WEM_PAIRED", "1")
    monkeypatch.setenv("WEM_PHASE_TABLES", "0")
    with gpu_lib.Context() as ctx:
        ctx.prepare(c["params"], vel, c["wav"])
        assert np.array_equal(ctx.migrate(c["shots"]), images[0])


def test_config0_full_size_matches_reference_port(gpu_lib, oracle_mod):
    """The split-step workload at full size (1 shot, 200 x 256, 221 frequencies)."""
    from wemgpu import synth
    c = synth.config0()
    m = gpu_lib.migrate(c["params"], c["vel"], c["wav"], c["shots"])
    p = dict(c["params"], sx=float(c["shots"].sx[0]))
    want = oracle_mod.wem_port(p, c["vel"], c["wav"], d=c["shots"].data, adj=True)
    assert rel_l2(m, want) < TOL


def test_config1_geometry_band_subset(gpu_lib, oracle_mod):
    """The PSPI survey's grid (500 x 1024, nkx 2048, nref 8) on 2 shots and a narrow
    band, so the oracle finishes in seconds."""
    from wemgpu import synth
    c = synth.config1(nshot=2, fmax=7.0, npoints=20)
    p = dict(c["params"], fmin=5.0, fmax=7.0)
    m = gpu_lib.migrate(p, c["vel"], c["wav"], c["shots"])
    want = _port_stack(oracle_mod, p, c["vel"], c["wav"], c["shots"])
    assert rel_l2(m, want) < TOL


def test_main_dropin_on_seis_files(gpu_lib, tmp_path):
    """main(argc, argv) on seis files (shotwem.c:12-140) vs the reference's main()."""
    from wemgpu import seis
    g = load_golden("main_pspi_64.npz")
    p = g["params"]
    seis.write_grid(str(tmp_path / "vel"), g["vel"], o1=0.0, d1=p["dz"], ox=p["omx"], dx=p["dmx"])
    seis.write_wavelet(str(tmp_path / "wav"), g["wav"], dt=p["dt"])
    seis.write_shot(str(tmp_path / "d"), g["d"], sx=p["sx"], dt=p["dt"], ox=p["omx"], dx=p["dmx"])
    args = [b"0", b"adj=y", b"pspi=y", f"nref={p['nref']}".encode(), b"d=" + str(tmp_path / "d").encode(),
            b"m=" + str(tmp_path / "m").encode(), b"vel=" + str(tmp_path / "vel").encode(),
            b"wav=" + str(tmp_path / "wav").encode(), b"damping=1000.0", f"sx={p['sx']}".encode(), b"sy=0",
            b"sz=0", b"gz=0", f"fmin={p['fmin']}".encode(), f"fmax={p['fmax']}".encode(),
            f"padt={p['padt']}".encode(), f"padx={p['padx']}".encode(), b"verbose=n"]
    argv = (C.c_char_p * len(args))(*args)
    assert gpu_lib.lib().main(len(args), argv) == 0
    m, h, ext = seis.read(str(tmp_path / "m"))
    assert rel_l2(m, g["m_ref"]) < TOL
    assert np.array_equal(h["imx"], g["imx"]) and np.allclose(h["mx"], g["mx"])
    assert ext["n"][:3] == list(g["n"][:3])


def test_edge_cases(gpu_lib):
    from wemgpu import synth, WemError
    c = synth.small_case(51, nx=64, nz=8, nt=64, nshot=2)
    p, vel, wav, shots = c["params"], c["vel"], c["wav"], c["shots"]
    with gpu_lib.Context() as ctx:
        ctx.prepare(p, vel, wav)
        # a shot without traces contributes nothing (its receiver wavefield is zero)
        empty = gpu_lib.Shots(shots.sx[:1], shots.sy[:1], np.array([0, 0], np.int64), np.zeros(0, np.int32),
                              np.zeros((0, p["nt"]), np.float32))
        assert not np.any(ctx.migrate(empty))
        # source outside the grid
        bad = gpu_lib.Shots(np.array([1e6], np.float32), np.zeros(1, np.float32), shots.trace_offset[:2],
                            shots.trace_cell[: shots.trace_offset[1]], shots.data[: shots.trace_offset[1]])
        with pytest.raises(WemError) as e:
            ctx.migrate(bad)
        assert e.value.code == -1
        # zero data gives a zero image
        zero = gpu_lib.Shots(shots.sx, shots.sy, shots.trace_offset, shots.trace_cell, np.zeros_like(shots.data))
        assert not np.any(ctx.migrate(zero))
        # a row length with no kernel (a non-power of two above 2048) and a single reference
        # velocity are rejected
        with pytest.raises(WemError) as e:
            ctx.prepare(dict(p, nmx=1100, padx=2), np.ones((1100, p["nz"]), np.float32) * 2000, wav)
        assert e.value.code == -2
        with pytest.raises(WemError) as e:
            ctx.prepare(dict(p, nref=1), vel, wav)
        assert e.value.code == -1


def test_source_and_receiver_depth(gpu_lib, oracle_mod):
    """sz, gz > 0: continuation and imaging start below them (wem.c:235-242)."""
    from wemgpu import synth
    c = synth.small_case(61, nx=64, nz=20, nt=96, nshot=1)
    p = dict(c["params"], sz=45.0, gz=95.0)
    m = gpu_lib.migrate(p, c["vel"], c["wav"], c["shots"])
    want = _port_stack(oracle_mod, p, c["vel"], c["wav"], c["shots"])
    assert rel_l2(m, want) < TOL
    assert not np.any(m[:, :10])


def test_measured_fp32_peak_is_plausible(gpu_lib):
    """wem_measure_fp32_peak (the denominator of the depth kernels' CUDA-core roofline):
    152 SMs x 128 FP32 lanes x 2 FLOPs at up to 2.07 GHz is 80.5 TFLOP/s nominal."""
    from wemgpu._lib import measure_fp32_peak
    v = measure_fp32_peak(0)
    assert 20.0 < v < 100.0, v


@pytest.mark.parametrize("interp", ["ref", "linear"])
def test_phase_tables_in_sub_bands(gpu_lib, oracle_mod, monkeypatch, interp):
    """When the whole band's phase tables do not fit the device, the migration and the
    modelling run sub-band by sub-band (one table launch, then the depth kernel on that
    sub-band's items); WEM_PTAB_CHUNK caps a sub-band so that this small case takes the
    path. The images and data agree with the single-band run to FP32 rounding (the CTAs see
    the items in another order) and with the port."""
    from wemgpu import synth
    c = synth.small_case(47, nx=128, nz=16, nt=128, nshot=3, pspi=1, nref=4, interp=interp)
    p, shots = c["params"], c["shots"]
    rng = np.random.default_rng(5)
    m_in = rng.standard_normal((p["nmx"], p["nz"])).astype(np.float32)
    out = []
    for chunk in (None, "3"):
        if chunk:
            monkeypatch.setenv("WEM_PTAB_CHUNK", chunk)
        with gpu_lib.Context() as ctx:
            ctx.prepare(p, c["vel"], c["wav"])
            out.append((ctx.migrate(shots), ctx.migrate(shots), ctx.model(shots, m_in, exact=True)))
    (m1, m1b, d1), (m2, m2b, d2) = out
    assert np.array_equal(m2, m2b)  # the captured graph of the sub-band launches replays
    assert rel_l2(m2, m1) < 1e-5 and rel_l2(d2, d1) < 1e-5
    assert rel_l2(m2, _port_stack(oracle_mod, p, c["vel"], c["wav"], shots)) < TOL
