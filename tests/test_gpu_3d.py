"""3-D migration (nmy > 1: rank-2 x-y transforms, wem.c:100-104) on the GPU through the
C ABI, against the reference's own output (golden) and the oracle. Tolerance: relative L2
image error <= 1e-4."""
import numpy as np
import pytest

from conftest import load_golden, rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-4


@pytest.mark.parametrize("case", ["ss3d_32", "pspi3d_32"])
def test_3d_wem_dropin_matches_reference_golden(gpu_lib, case):
    g = load_golden(f"wem_{case}.npz")
    m = gpu_lib.wem_dropin(g["params"], g["vel"], g["wav"], d=g["d"], adj=True)
    assert rel_l2(m, g["m_ref"]) < TOL


def _port_stack(oracle_mod, p, vel, wav, shots, fp64=False):
    op = oracle_mod.wem_fp64 if fp64 else oracle_mod.wem_port
    n = p["nmx"] * p["nmy"]
    img = None
    for s in range(shots.nshot):
        lo, hi = shots.trace_offset[s], shots.trace_offset[s + 1]
        d = np.zeros((n, p["nt"]), np.float32)
        d[shots.trace_cell[lo:hi]] = shots.data[lo:hi]
        q = dict(p, sx=float(shots.sx[s]), sy=float(shots.sy[s]))
        m = op(q, vel, wav, d=d, adj=True).astype(np.float64)
        img = m if img is None else img + m
    return img


@pytest.mark.parametrize("pspi,interp", [(0, "ref"), (1, "ref"), (1, "linear")])
def test_3d_batched_matches_oracle(gpu_lib, oracle_mod, pspi, interp):
    from wemgpu import synth
    c = synth.small_case3d(31, nx=32, ny=32, nz=8, nt=64, nshot=2, pspi=pspi, nref=3, interp=interp)
    m = gpu_lib.migrate(c["params"], c["vel"], c["wav"], c["shots"])
    want = _port_stack(oracle_mod, c["params"], c["vel"], c["wav"], c["shots"])
    assert rel_l2(m, want) < TOL
    want64 = _port_stack(oracle_mod, c["params"], c["vel"], c["wav"], c["shots"], fp64=True)
    assert rel_l2(m, want64) < TOL


@pytest.mark.parametrize("nx,ny,padx", [(64, 32, 2), (32, 64, 2), (128, 128, 1), (256, 32, 2)])
def test_3d_plane_shapes(gpu_lib, oracle_mod, nx, ny, padx):
    from wemgpu import synth
    c = synth.small_case3d(41 + nx + ny, nx=nx, ny=ny, nz=5, nt=64, nshot=1, pspi=1, nref=3, fmax=25.0, padx=padx)
    m = gpu_lib.migrate(c["params"], c["vel"], c["wav"], c["shots"])
    want = _port_stack(oracle_mod, c["params"], c["vel"], c["wav"], c["shots"])
    assert rel_l2(m, want) < TOL


@pytest.mark.parametrize("nref", [3, 6])
def test_3d_paired_planes(gpu_lib, oracle_mod, monkeypatch, nref):
    """The nearest-lower mode in 3-D: the real parts of two reference wavefields come from
    one plane of passes B and C (Hermitian projection over (kx, ky): a(-kx, -ky) from the
    mirror column), references taken whole somewhere keep a plane of their own. Depth
    levels: random, a velocity range of 40 m/s (reference spacing <= 10 m/s at nref 6:
    every reference taken whole) and constant velocity; random levels whose maximum one or
    three points take (their references paired, the imaginary parts there from direct sums
    over kx in pass B and over ky in pass C). Against the port and against one plane per
    reference (WEM_PAIRED=0)."""
    from wemgpu import synth
    c = synth.small_case3d(81, nx=64, ny=32, nz=9, nt=64, nshot=2, pspi=1, nref=nref, fmax=30.0)
    rng = np.random.default_rng(82)
    vel = c["vel"].copy()
    vel[:, 3:5] = 2500.0
    vel[:, 5:7] = 2500.0 + 40.0 * rng.random((vel.shape[0], 2))
    vel[0, 5:7] = vel[:, 5:7].min(axis=0) - 1.0  # the depth's minimum on the first x-plane
    vel[[3, 700, 1500], 7] = vel[:, 7].max()  # a maximum taken by 3 points (direct sums)
    want = _port_stack(oracle_mod, c["params"], vel, c["wav"], c["shots"])
    images = []
    for paired in ("1", "0"):
        monkeypatch.setenv("WEM_PAIRED", paired)
        with gpu_lib.Context() as ctx:
            ctx.prepare(c["params"], vel, c["wav"])
            images.append(ctx.migrate(c["shots"]))
        assert rel_l2(images[-1], want) < TOL, (paired, rel_l2(images[-1], want))
    assert rel_l2(images[0], images[1]) < 1e-5


def test_3d_deterministic_and_depths(gpu_lib, oracle_mod):
    from wemgpu import synth
    c = synth.small_case3d(51, nx=32, ny=32, nz=10, nt=64, nshot=1, pspi=1, nref=3)
    p = dict(c["params"], sz=25.0, gz=35.0)
    with gpu_lib.Context() as ctx:
        ctx.prepare(p, c["vel"], c["wav"])
        a = ctx.migrate(c["shots"])
        b = ctx.migrate(c["shots"])
    assert np.array_equal(a, b)
    assert rel_l2(a, _port_stack(oracle_mod, p, c["vel"], c["wav"], c["shots"])) < TOL
    assert not np.any(a[:, :4])


@pytest.mark.parametrize("case", ["ss3d_32", "pspi3d_32"])
def test_3d_modelling_matches_reference_golden(gpu_lib, case):
    """wem() with adj=false on a 3-D grid (wem.c:252-281, 177-188): the reference's own
    modelled data of the golden image m_in."""
    g = load_golden(f"wem_{case}.npz")
    d = gpu_lib.wem_dropin(g["params"], g["vel"], g["wav"], m=g["m_in"], adj=False)
    assert rel_l2(d, g["d_ref"]) < TOL, rel_l2(d, g["d_ref"])


@pytest.mark.parametrize("pspi,interp", [(0, "ref"), (1, "ref"), (1, "linear")])
def test_3d_batched_modelling_matches_port(gpu_lib, oracle_mod, pspi, interp):
    """Several shots with source depth and receiver depth below the surface in one call,
    against the oracle's port shot by shot at the shots' receiver cells."""
    from wemgpu import synth
    c = synth.small_case3d(61, nx=32, ny=32, nz=8, nt=64, nshot=2, pspi=pspi, nref=3, interp=interp)
    p, s = dict(c["params"], sz=15.0, gz=25.0), c["shots"]
    rng = np.random.default_rng(3)
    m = rng.standard_normal((p["nmx"] * p["nmy"], p["nz"])).astype(np.float32)
    with gpu_lib.Context() as ctx:
        ctx.prepare(p, c["vel"], c["wav"])
        d = ctx.model(s, m, exact=False)
    for i in range(s.nshot):
        lo, hi = int(s.trace_offset[i]), int(s.trace_offset[i + 1])
        want = oracle_mod.wem_port(dict(p, sx=float(s.sx[i]), sy=float(s.sy[i])), c["vel"], c["wav"], m=m, adj=False)
        assert rel_l2(d[lo:hi], want[s.trace_cell[lo:hi]]) < TOL


@pytest.mark.parametrize("pspi,interp,nref", [(1, "linear", 3), (1, "ref", 6), (0, "ref", 1)])
def test_3d_exact_pair_dot_product(gpu_lib, pspi, interp, nref):
    """The exact modelling (exact = 1: the receiver goes up with the adjoint of the migration
    step, W_r^T, FFT2, conj(P_r), sum over r, IFFT2) and the 3-D migration are an adjoint
    pair: <d, L m> = <L' d, m> to FP32 rounding, with sources and receivers below the
    surface. Split-step: the reference's modelling operator already is the adjoint."""
    from wemgpu import synth
    from wemgpu.api import Shots
    from wemgpu.cg import dot_test
    c = synth.small_case3d(91, nx=64, ny=32, nz=8, nt=64, nshot=2, pspi=pspi, nref=nref, interp=interp, fmax=30.0)
    p, s = dict(c["params"], sz=15.0, gz=25.0), c["shots"]
    rng = np.random.default_rng(92)
    m = rng.standard_normal((p["nmx"] * p["nmy"], p["nz"])).astype(np.float32)
    d = rng.standard_normal(s.data.shape).astype(np.float32)
    with gpu_lib.Context() as ctx:
        ctx.prepare(p, c["vel"], c["wav"])
        geo = lambda r: Shots(s.sx, s.sy, s.trace_offset, s.trace_cell, np.ascontiguousarray(r, np.float32))
        a, b = dot_test(lambda x: ctx.model(s, np.asarray(x, np.float32), exact=True),
                        lambda r: ctx.migrate(geo(r)), m, d)
    assert abs(a - b) / abs(a) < 1e-5, (a, b)
