"""Parity of every workload at its own grid size, against the oracle (CPU).

* the 64-shot PSPI survey (500 x 1024 grid, 2048-point rows, 8 reference velocities,
  all 271 frequencies of 5-50 Hz, Born data of a 1 % random reflectivity): the whole
  stacked image against the port of the reference's C (bit-identical to the compiled
  reference), shot by shot on the host cores;
* 4 shots of that survey over the full band against the FP64 operator, in both the FP32
  and the split16 (tensor-core) forms;
* the 3-D survey's 512 x 512 plane (256 x 256 cells, padx 2, 6 reference velocities) over
  a few depth steps and a narrow band, against the port and the FP64 operator;
* the least-squares workload's geometry (300 x 512, 8 reference velocities, linear
  interpolation): CG over the GPU's reference operator pair against CG over the port's
  pair, same data and start, on 4 shots and a 5 Hz band.

Tolerance: relative L2 image error <= 1e-4 (the contract's bar); misfit curves within
1e-3 of each other, relative.
"""
import os

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-4
CORES = os.cpu_count() or 1


def _stack(oracle_mod, p, vel, wav, shots, which, fp64=False):
    from wemgpu import synth
    op = oracle_mod.wem_fp64 if fp64 else oracle_mod.wem_port
    n = int(p["nmx"]) * int(p.get("nmy", 1))
    img = None
    for s in which:
        q = dict(p, sx=float(shots.sx[s]), sy=float(shots.sy[s]))
        m = op(q, vel, wav, d=synth.shot_gather_full(shots, s, n), adj=True, nthreads=CORES).astype(np.float64)
        img = m if img is None else img + m
    return img


def _subset(shots, which):
    from wemgpu import Shots
    offs, cells, data = [0], [], []
    for s in which:
        lo, hi = int(shots.trace_offset[s]), int(shots.trace_offset[s + 1])
        cells.append(shots.trace_cell[lo:hi])
        data.append(shots.data[lo:hi])
        offs.append(offs[-1] + hi - lo)
    return Shots(shots.sx[list(which)], shots.sy[list(which)], np.asarray(offs, np.int64),
                 np.concatenate(cells), np.concatenate(data))


@pytest.fixture(scope="module")
def survey64(gpu_lib):
    from wemgpu import synth
    return synth.with_born_data(synth.config1())


def test_survey64_whole_image_matches_the_reference_port(gpu_lib, oracle_mod, survey64):
    c = survey64
    p, shots = c["params"], c["shots"]
    assert shots.nshot == 64 and p["nz"] == 500 and p["nmx"] == 1024
    m = gpu_lib.migrate(p, c["vel"], c["wav"], shots)
    want = _stack(oracle_mod, p, c["vel"], c["wav"], shots, range(shots.nshot))
    err = rel_l2(m, want)
    print(f"64-shot survey, 271 frequencies: rel L2 vs the port {err:.3e}")
    assert err < TOL


@pytest.mark.parametrize("precision", ["fp32", "split16"])
def test_survey_four_shots_full_band_vs_fp64(gpu_lib, oracle_mod, survey64, precision):
    c = survey64
    p, shots = c["params"], c["shots"]
    which = [8, 24, 40, 56]
    sub = _subset(shots, which)
    m = gpu_lib.migrate(dict(p, precision=precision), c["vel"], c["wav"], sub)
    want = _stack(oracle_mod, p, c["vel"], c["wav"], shots, which, fp64=True)
    err = rel_l2(m, want)
    print(f"4 shots, 5-50 Hz, {precision}: rel L2 vs FP64 {err:.3e}")
    assert err < TOL


def test_3d_512_plane_matches_port_and_fp64(gpu_lib, oracle_mod):
    """The 3-D survey's geometry: 256 x 256 cells at 12.5 m, padx 2 (512 x 512 planes), 6
    reference velocities, the full receiver grid; 12 depth steps of the smooth random
    field and 3-5 Hz (17 frequencies) so that the CPU finishes in about a minute."""
    from wemgpu import synth
    c = synth.config3(nz=12, fmax=5.0, npoints=20)
    p = c["params"]
    assert p["nmx"] == 256 and p["nmy"] == 256 and p["padx"] == 2 and p["nref"] == 6
    m = gpu_lib.migrate(p, c["vel"], c["wav"], c["shots"])
    want = _stack(oracle_mod, p, c["vel"], c["wav"], c["shots"], [0])
    e32 = rel_l2(m, want)
    want64 = _stack(oracle_mod, p, c["vel"], c["wav"], c["shots"], [0], fp64=True)
    e64 = rel_l2(m, want64)
    print(f"3-D 512x512 planes: rel L2 vs the port {e32:.3e}, vs FP64 {e64:.3e}")
    assert e32 < TOL and e64 < TOL


def test_least_squares_geometry_misfit_curve_vs_port_pair(gpu_lib, oracle_mod):
    from wemgpu import synth
    from wemgpu.cg import conjugate_gradients
    c = synth.config4(nshot=4)
    p = dict(c["params"], interp="linear", fmax=10.0)
    shots = c["shots"]
    assert p["nmx"] == 512 and p["nz"] == 300 and p["nref"] == 8
    ctx = gpu_lib.Context()
    ctx.prepare(p, c["vel"], c["wav"])

    def fwd_gpu(m):
        return ctx.model(shots, np.asarray(m, np.float32), exact=False)

    def adj_gpu(d):
        return ctx.migrate(gpu_lib.Shots(shots.sx, shots.sy, shots.trace_offset, shots.trace_cell,
                                         np.ascontiguousarray(d, np.float32)))

    def fwd_ref(m):
        out = []
        for s in range(shots.nshot):
            lo, hi = int(shots.trace_offset[s]), int(shots.trace_offset[s + 1])
            full = oracle_mod.wem_port(dict(p, sx=float(shots.sx[s]), sy=float(shots.sy[s])), c["vel"], c["wav"],
                                       m=np.asarray(m, np.float32), adj=False, nthreads=CORES)
            out.append(full[shots.trace_cell[lo:hi]])
        return np.concatenate(out).astype(np.float64)

    def adj_ref(d):
        img = np.zeros((p["nmx"], p["nz"]))
        for s in range(shots.nshot):
            lo, hi = int(shots.trace_offset[s]), int(shots.trace_offset[s + 1])
            g = np.zeros((p["nmx"], p["nt"]), np.float32)
            g[shots.trace_cell[lo:hi]] = d[lo:hi]
            img += oracle_mod.wem_port(dict(p, sx=float(shots.sx[s]), sy=float(shots.sy[s])), c["vel"], c["wav"], d=g, adj=True,
                                       nthreads=CORES)
        return img

    m_true = synth.random_reflectivity(2004, p["nmx"], p["nz"])
    d = fwd_ref(m_true)
    assert rel_l2(fwd_gpu(m_true), d) < TOL
    _, cost_gpu = conjugate_gradients(d, fwd_gpu, lambda r: adj_gpu(r.astype(np.float32)), niter=6)
    _, cost_ref = conjugate_gradients(d, fwd_ref, lambda r: adj_ref(r.astype(np.float32)), niter=6)
    ctx.close()
    cost_gpu, cost_ref = np.array(cost_gpu), np.array(cost_ref)
    print("misfit GPU", cost_gpu, "port", cost_ref)
    assert np.all(np.abs(cost_gpu - cost_ref) <= 1e-3 * np.maximum(cost_ref, 1e-3)), (cost_gpu, cost_ref)


def test_elastic_workload_two_shots_full_band_vs_fp64(gpu_lib):
    """The elastic workload's geometry (300 x 512 grid, padx 2: 1024-point rows, vs = vp/1.8 with a
    5 % wobble) over its whole 5-30 Hz band (151 frequencies x 300 depth steps): two shots
    stacked, P and S images against the FP64 restatement of ewem.c (oracle/ewem_np.py), at
    1e-4. The reference's own FP32 arithmetic (ewem.c compiled in the build container) on the
    same two shots and band: 5.3e-5 (P) and 4.7e-5 (S) against the same FP64 images; this
    operator's 2 x 2 separation divides by norms down to 0.1 at every depth step."""
    import ewem_np as E
    from wemgpu import synth
    c = synth.config4(seed=1004, nshot=8)
    p = dict(c["params"], fmax=30.0)
    assert p["nmx"] == 512 and p["nz"] == 300
    rng = np.random.default_rng(2005)
    vp = c["vel"]
    vs = (vp / 1.8 * (1.0 + 0.05 * rng.standard_normal(vp.shape))).astype(np.float32)
    shots = c["shots"]
    which = [2, 5]
    uz = np.stack([synth.shot_gather_full(shots, s, 512) for s in which])
    ux = (0.5 * np.roll(uz, 3, axis=2)).astype(np.float32)
    sx = [float(shots.sx[s]) for s in which]
    mpp, mps2 = gpu_lib.elastic(p, vp, vs, c["wav"], sx, ux=ux, uz=uz, adj=True)
    want_p = want_s = 0.0
    for i, s in enumerate(sx):
        a, _, b = E.ewem(dict(p, sx=s), vp, vs, c["wav"], ux=ux[i], uz=uz[i], adj=True)
        want_p, want_s = want_p + a, want_s + b
    ep, es = rel_l2(mpp, want_p), rel_l2(mps2, want_s)
    print(f"elastic, 2 shots, 151 frequencies x 300 depth steps: rel L2 vs FP64 P {ep:.3e} S {es:.3e}")
    assert ep < TOL and es < TOL


def test_angles_workload_two_shots_full_band_vs_fp64(gpu_lib):
    """The incidence-angle workload's geometry (the 64-shot survey's 500 x 1024 grid, 5-50 Hz of
    the unpadded 1500-sample axis: 136 frequencies x 500 depth steps), two shots, against the
    FP64 restatement of compute_angles (oracle/angles_np.py): the angle magnitudes at 1e-4, and
    the side of arrival (the sign) at all but a few points per 100,000 (where both sides carry
    equal energy the side is ill-conditioned: the reference's own FP32 result flips the same
    way there)."""
    import angles_np as A
    from wemgpu import synth
    c = synth.config1(seed=1001, nshot=8)
    p = c["params"]
    assert p["nmx"] == 1024 and p["nz"] == 500
    sxs = [float(c["shots"].sx[2]), float(c["shots"].sx[5])]
    with gpu_lib.Context() as ctx:
        ax, _ = ctx.angles(p, c["vel"], c["wav"], sxs)
    for i, s in enumerate(sxs):
        want, _ = A.compute_angles(dict(p, sx=s), c["vel"], c["wav"])
        em = rel_l2(np.abs(ax[i]), np.abs(want))
        live = np.abs(want) > 1e-6
        flips = int(np.count_nonzero(np.sign(ax[i][live]) != np.sign(want[live])))
        print(f"angles, shot at {s:g} m, 136 frequencies x 500 depth steps: magnitudes {em:.3e}, "
              f"{flips} sign flips of {int(live.sum())} points")
        assert em < TOL and flips <= 1e-4 * live.sum()


def test_3d_survey_top_of_the_band_matches_port(gpu_lib, oracle_mod):
    """The 3-D survey (300 x 256 x 256, 512 x 512 planes, 6 reference velocities) over all 300
    depth steps at the top of its band, 58-60 Hz (17 frequencies, where most wavenumbers
    propagate), against the port of the reference's C at 1e-4."""
    from wemgpu import synth
    c = synth.config3(seed=1003)
    p = dict(c["params"], fmin=58.0, fmax=60.0)
    m = gpu_lib.migrate(p, c["vel"], c["wav"], c["shots"])
    want = _stack(oracle_mod, p, c["vel"], c["wav"], c["shots"], [0])
    err = rel_l2(m, want)
    print(f"3-D survey, 58-60 Hz x 300 depth steps: rel L2 vs the port {err:.3e}")
    assert err < TOL
