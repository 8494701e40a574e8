"""The split16 precision mode: the FFTs' DFT stages of the migration on the tensor cores
(tcgen05, split fp16 hi+lo operands, FP32 accumulation), 2-D rows of nkx = 2048.

Tolerance: relative L2 image error <= 1e-4 against the FP64 operator (the oracle's
double-precision restatement of wem.c) and against the reference's FP32 arithmetic
(the port), the same bar as the FP32 mode.
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-4


def _stack(oracle_mod, p, vel, wav, shots, fp64):
    from wemgpu import synth
    op = oracle_mod.wem_fp64 if fp64 else oracle_mod.wem_port
    img = None
    for s in range(shots.nshot):
        d = synth.shot_gather_full(shots, s, p["nmx"])
        m = op(dict(p, sx=float(shots.sx[s]), sy=float(shots.sy[s])), vel, wav, d=d, adj=True).astype(np.float64)
        img = m if img is None else img + m
    return img


@pytest.mark.parametrize("pspi,interp", [(1, "ref"), (1, "linear"), (0, "ref")])
def test_split16_matches_fp64_oracle(gpu_lib, oracle_mod, pspi, interp):
    """3 shots with uneven apertures on a 1024-cell grid (nkx 2048), 40 depth steps."""
    from wemgpu import synth
    c = synth.small_case(51, nx=1024, nz=40, nt=128, nshot=3, pspi=pspi, nref=6, interp=interp, fmax=30.0)
    p = dict(c["params"], precision="split16")
    m = gpu_lib.migrate(p, c["vel"], c["wav"], c["shots"])
    m32 = gpu_lib.migrate(c["params"], c["vel"], c["wav"], c["shots"])
    want64 = _stack(oracle_mod, c["params"], c["vel"], c["wav"], c["shots"], fp64=True)
    want32 = _stack(oracle_mod, c["params"], c["vel"], c["wav"], c["shots"], fp64=False)
    e16 = rel_l2(m, want64)
    assert e16 < TOL, e16
    assert rel_l2(m, want32) < TOL
    assert rel_l2(m32, want64) < TOL


@pytest.mark.parametrize("interp", ["ref", "linear"])
def test_split16_precomputed_phase_tables_bit_identical(gpu_lib, monkeypatch, interp):
    """The split16 kernel reading the phase tables precomputed for every (frequency, depth)
    gives the image of tables built in each CTA (WEM_PHASE_TABLES=0) bit for bit."""
    from wemgpu import synth
    c = synth.small_case(53, nx=1024, nz=24, nt=128, nshot=3, pspi=1, nref=6, interp=interp, fmax=30.0)
    p = dict(c["params"], precision="split16")
    images = []
    monkeypatch.setenv("WEM_AUTOTUNE", "0")  # the same CTA shape for both runs
    for pt in ("1", "0"):
        monkeypatch.setenv("WEM_PHASE_TABLES", pt)
        with gpu_lib.Context() as ctx:
            ctx.prepare(p, c["vel"], c["wav"])
            images.append(ctx.migrate(c["shots"]))
            images.append(ctx.migrate(c["shots"]))  # the captured graph replayed
    assert np.array_equal(images[0], images[1])
    assert np.array_equal(images[0], images[2]) and np.array_equal(images[2], images[3])


def test_split16_survey_geometry_band_subset(gpu_lib, oracle_mod):
    """The PSPI survey's grid (500 x 1024, nref 8) on 2 shots and a narrow band, both
    CTA shapes of the tensor-core kernel."""
    import os
    from wemgpu import synth
    c = synth.config1(nshot=2, fmax=7.0, npoints=20)
    p = dict(c["params"], fmin=5.0, fmax=7.0)
    want64 = _stack(oracle_mod, p, c["vel"], c["wav"], c["shots"], fp64=True)
    for shape in ("wide", "narrow"):
        os.environ["WEM_CTA_SHAPE"] = shape
        try:
            with gpu_lib.Context() as ctx:
                ctx.prepare(dict(p, precision="split16"), c["vel"], c["wav"])
                m = ctx.migrate(c["shots"])
                threads = ctx.last_launch()["threads"]
        finally:
            del os.environ["WEM_CTA_SHAPE"]
        assert threads == (512 if shape == "wide" else 256)
        assert rel_l2(m, want64) < TOL, (shape, rel_l2(m, want64))


def test_split16_rejects_other_geometries(gpu_lib):
    from wemgpu import synth
    from wemgpu._lib import WemError
    c = synth.small_case(52, nx=256, nz=8, nt=64, nshot=1)
    with pytest.raises(WemError) as e:
        gpu_lib.migrate(dict(c["params"], precision="split16"), c["vel"], c["wav"], c["shots"])
    assert e.value.code == -2  # WEM_ERR_SIZE


def test_bounded_wait_reports_timeout_and_device_stays_usable(gpu_lib):
    """The tensor-core stages wait on an mbarrier with a time limit (about a second). A wait
    that nothing completes gives up, reports it, and the context stays usable: a migration
    on the same device right after it still matches the FP64 operator."""
    import ctypes as C
    from wemgpu import synth
    from wemgpu._lib import lib
    timed_out, ms = C.c_int(-1), C.c_float(0.0)
    assert lib().wem_selftest_wait_timeout(0, C.byref(timed_out), C.byref(ms)) == 0
    assert timed_out.value == 1
    assert 100.0 < ms.value < 20000.0, ms.value  # the wait ran to its limit, then returned
    c = synth.small_case(53, nx=64, nz=8, nt=64, nshot=1)
    m = gpu_lib.migrate(c["params"], c["vel"], c["wav"], c["shots"])
    assert np.isfinite(m).all() and np.abs(m).max() > 0
