"""Born modelling (wem.c adj=false) on the GPU through the C ABI.

* the reference's operator vs the reference's own output (golden) and the port;
* the exact-adjoint operator against the migration: dot-product test to 1e-5 and the
  finite-difference gradient of the data misfit (least-squares migration);
* CG on the GPU operator pair decreases the misfit like CG on the FP64 oracle's pair.
"""
import numpy as np
import pytest

from conftest import load_golden, rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-4
GOLDEN_CASES = ["ss_64", "ss_128_taper", "pspi_64", "pspi_128_r8", "pspi_64_padx1", "pspi_500_padx2", "ss_300_padx2", "pspi_768_padx2", "pspi_97_padx1", "ss_50_padx1", "ss_64_buried", "pspi_64_buried"]


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_wem_dropin_modelling_matches_reference_golden(gpu_lib, case):
    g = load_golden(f"wem_{case}.npz")
    d = gpu_lib.wem_dropin(g["params"], g["vel"], g["wav"], m=g["m_in"], adj=False)
    assert rel_l2(d, g["d_ref"]) < TOL


@pytest.mark.parametrize("pspi,interp,nx", [(0, "ref", 64), (1, "ref", 64), (1, "linear", 64), (0, "ref", 300),
                                             (1, "ref", 500), (1, "linear", 97)])
def test_batched_modelling_matches_port(gpu_lib, oracle_mod, pspi, interp, nx):
    """Born modelling of several shots in one call vs the port shot by shot; nx 300, 500 and 97
    give rows of nkx 600, 1000 and 194 (Bluestein's form)."""
    from wemgpu import synth
    c = synth.small_case(81, nx=nx, nz=20, nt=128, nshot=3, pspi=pspi, nref=4, interp=interp)
    p, shots = c["params"], c["shots"]
    rng = np.random.default_rng(3)
    m = rng.standard_normal((p["nmx"], p["nz"])).astype(np.float32)
    with gpu_lib.Context() as ctx:
        d = ctx.prepare(p, c["vel"], c["wav"]).model(shots, m, exact=False)
    for s in range(shots.nshot):
        lo, hi = shots.trace_offset[s], shots.trace_offset[s + 1]
        want = oracle_mod.wem_port(dict(p, sx=float(shots.sx[s]), sy=float(shots.sy[s])), c["vel"], c["wav"], m=m, adj=False)
        assert rel_l2(d[lo:hi], want[shots.trace_cell[lo:hi]]) < TOL


def _pair(gpu_lib, c):
    ctx = gpu_lib.Context()
    ctx.prepare(c["params"], c["vel"], c["wav"])
    shots = c["shots"]

    def fwd(m):
        return ctx.model(shots, m, exact=True)

    def adj(d):
        return ctx.migrate(gpu_lib.Shots(shots.sx, shots.sy, shots.trace_offset, shots.trace_cell,
                                         np.ascontiguousarray(d, np.float32)))
    return ctx, fwd, adj


@pytest.mark.parametrize("pspi,interp,nx", [(0, "ref", 128), (1, "ref", 64), (1, "linear", 64), (1, "linear", 512),
                                             (1, "linear", 300), (0, "ref", 150)])
def test_dot_product_of_exact_pair(gpu_lib, pspi, interp, nx):
    """<d, L m> = <L' d, m> to 1e-5 (src/Tools/DotTest.jl), L = wem_model(exact), L' = wem_migrate."""
    from wemgpu import synth
    from wemgpu.cg import dot_test
    c = synth.small_case(91 + nx, nx=nx, nz=24, nt=128, nshot=3, pspi=pspi, nref=5, interp=interp)
    ctx, fwd, adj = _pair(gpu_lib, c)
    rng = np.random.default_rng(7)
    m = rng.standard_normal((c["params"]["nmx"], c["params"]["nz"])).astype(np.float32)
    d = rng.standard_normal(c["shots"].data.shape).astype(np.float32)
    a, b = dot_test(fwd, adj, m, d)
    ctx.close()
    assert abs(a - b) / max(abs(a), abs(b)) < 1e-5


def test_misfit_gradient_finite_difference(gpu_lib):
    """J(m) = 1/2 ||L m - d||^2: central difference along a random direction vs <L'(Lm - d), dm>."""
    from wemgpu import synth
    from wemgpu.cg import inner
    c = synth.small_case(101, nx=64, nz=20, nt=128, nshot=2, pspi=1, nref=4, interp="linear")
    ctx, fwd, adj = _pair(gpu_lib, c)
    rng = np.random.default_rng(11)
    m0 = rng.standard_normal((64, 20)).astype(np.float32)
    dm = rng.standard_normal((64, 20)).astype(np.float32)
    d = c["shots"].data

    def J(m):
        r = fwd(m).astype(np.float64) - d
        return 0.5 * inner(r, r)
    g = adj((fwd(m0).astype(np.float64) - d).astype(np.float32))
    eps = 1e-2
    fd = (J(m0 + eps * dm) - J(m0 - eps * dm)) / (2 * eps)
    ctx.close()
    assert abs(fd - inner(g, dm)) / abs(fd) < 1e-3


def test_least_squares_migration_reduces_misfit(gpu_lib):
    """CG (Scales 1987, ConjugateGradients.jl:1-39) on the GPU pair: the normalised misfit
    falls monotonically and fits data modelled from a known image."""
    from wemgpu import synth
    from wemgpu.cg import conjugate_gradients
    c = synth.small_case(111, nx=64, nz=20, nt=128, nshot=3, pspi=1, nref=4, interp="linear")
    ctx, fwd, adj = _pair(gpu_lib, c)
    rng = np.random.default_rng(13)
    m_true = np.zeros((64, 20), np.float32)
    m_true[rng.integers(0, 64, 30), rng.integers(2, 20, 30)] = rng.standard_normal(30)
    d = fwd(m_true)
    m, cost = conjugate_gradients(d, fwd, lambda r: adj(r.astype(np.float32)), niter=10)
    ctx.close()
    assert np.all(np.diff(cost) <= 1e-6) and cost[-1] < 0.2


def test_misfit_curve_matches_reference_operator_pair(gpu_lib, oracle_mod):
    """CG over the GPU's reference operator pair (wem_model with exact=0, wem_migrate)
    against CG over the oracle's restatement of the reference's own pair (wem.c adj and
    fwd, shot by shot), same data and start: the normalised misfit curves agree."""
    from wemgpu import synth
    from wemgpu.cg import conjugate_gradients
    c = synth.small_case(112, nx=64, nz=16, nt=96, nshot=2, pspi=1, nref=4, interp="linear")
    p, shots = c["params"], c["shots"]
    ctx = gpu_lib.Context()
    ctx.prepare(p, c["vel"], c["wav"])

    def fwd_gpu(m):
        return ctx.model(shots, m, exact=False)

    def adj_gpu(d):
        return ctx.migrate(gpu_lib.Shots(shots.sx, shots.sy, shots.trace_offset, shots.trace_cell,
                                         np.ascontiguousarray(d, np.float32)))

    def fwd_ref(m):
        out = []
        for s in range(shots.nshot):
            lo, hi = int(shots.trace_offset[s]), int(shots.trace_offset[s + 1])
            full = oracle_mod.wem_port(dict(p, sx=float(shots.sx[s]), sy=float(shots.sy[s])), c["vel"], c["wav"], m=m, adj=False)
            out.append(full[shots.trace_cell[lo:hi]])
        return np.concatenate(out).astype(np.float64)

    def adj_ref(d):
        img = np.zeros((p["nmx"], p["nz"]))
        for s in range(shots.nshot):
            lo, hi = int(shots.trace_offset[s]), int(shots.trace_offset[s + 1])
            g = np.zeros((p["nmx"], p["nt"]), np.float32)
            g[shots.trace_cell[lo:hi]] = d[lo:hi]
            img += oracle_mod.wem_port(dict(p, sx=float(shots.sx[s]), sy=float(shots.sy[s])), c["vel"], c["wav"], d=g, adj=True)
        return img

    rng = np.random.default_rng(14)
    m_true = np.zeros((p["nmx"], p["nz"]), np.float32)
    m_true[rng.integers(0, p["nmx"], 20), rng.integers(2, p["nz"], 20)] = rng.standard_normal(20)
    d = fwd_ref(m_true)
    _, cost_gpu = conjugate_gradients(d, lambda m: fwd_gpu(np.asarray(m, np.float32)),
                                      lambda r: adj_gpu(r.astype(np.float32)), niter=6)
    _, cost_ref = conjugate_gradients(d, lambda m: fwd_ref(np.asarray(m, np.float32)),
                                      lambda r: adj_ref(r.astype(np.float32)), niter=6)
    ctx.close()
    cost_gpu, cost_ref = np.array(cost_gpu), np.array(cost_ref)
    assert np.all(np.abs(cost_gpu - cost_ref) <= 1e-3 * np.maximum(cost_ref, 1e-3)), (cost_gpu, cost_ref)


def test_device_buffer_calls_match_host_calls(gpu_lib):
    """wem_model_device / wem_migrate_device on device tensors give the host-buffer calls'
    results bit for bit, and CG over them (device vectors, float64 inner products) follows
    the same misfit curve."""
    torch = pytest.importorskip("torch")
    from wemgpu import synth
    from wemgpu.api import Shots
    from wemgpu.cg import conjugate_gradients
    c = synth.small_case(71, nx=128, nz=20, nt=96, nshot=3, pspi=1, nref=4, interp="linear")
    p, s = c["params"], c["shots"]
    rng = np.random.default_rng(72)
    m = rng.standard_normal((p["nmx"], p["nz"])).astype(np.float32)
    dev = torch.device("cuda", 0)
    with gpu_lib.Context() as ctx:
        ctx.prepare(p, c["vel"], c["wav"])
        d_host = ctx.model(s, m, exact=True)
        m_host = ctx.migrate(s)
        m_t = torch.from_numpy(m).to(dev)
        d_t = torch.empty(d_host.shape, dtype=torch.float32, device=dev)
        torch.cuda.synchronize()
        ctx.model_device(s, m_t.data_ptr(), d_t.data_ptr(), exact=True)
        assert np.array_equal(d_t.cpu().numpy(), d_host)
        dd_t = torch.from_numpy(np.ascontiguousarray(s.data, np.float32)).to(dev)
        mm_t = torch.empty(m.shape, dtype=torch.float32, device=dev)
        torch.cuda.synchronize()
        ctx.migrate_device(s, dd_t.data_ptr(), mm_t.data_ptr())
        assert np.array_equal(mm_t.cpu().numpy(), m_host)

        geo = lambda d: Shots(s.sx, s.sy, s.trace_offset, s.trace_cell, np.ascontiguousarray(d, np.float32))

        def fwd_t(x):
            y = torch.empty(d_host.shape, dtype=torch.float32, device=dev)
            torch.cuda.synchronize()
            ctx.model_device(s, x.data_ptr(), y.data_ptr(), exact=True)
            return y

        def adj_t(r):
            y = torch.empty(m.shape, dtype=torch.float32, device=dev)
            torch.cuda.synchronize()
            ctx.migrate_device(s, r.data_ptr(), y.data_ptr())
            return y

        inner_t = lambda a, b: float(torch.dot(a.reshape(-1).double(), b.reshape(-1).double()))
        _, cost_t = conjugate_gradients(torch.from_numpy(d_host).to(dev), fwd_t, adj_t, niter=5, inner_fn=inner_t)
        _, cost_h = conjugate_gradients(d_host, lambda x: ctx.model(s, np.asarray(x, np.float32), exact=True),
                                        lambda r: ctx.migrate(geo(r)), niter=5)
    assert np.allclose(cost_t, cost_h, rtol=1e-4, atol=1e-7)


@pytest.mark.gpu
def test_least_squares_migration_host_call_matches_device_cg(gpu_lib):
    """least_squares_migration (host traces in, host image out, CG vectors in device
    memory) gives the misfit curve of CG over the per-application host-buffer calls and
    the image of the device-tensor CG bit for bit."""
    torch = pytest.importorskip("torch")
    from wemgpu import synth
    from wemgpu.api import Shots
    from wemgpu.cg import conjugate_gradients, least_squares_migration
    c = synth.small_case(73, nx=128, nz=20, nt=96, nshot=3, pspi=1, nref=4, interp="linear")
    p, s = c["params"], c["shots"]
    rng = np.random.default_rng(74)
    m_true = np.zeros((p["nmx"], p["nz"]), np.float32)
    m_true.flat[rng.choice(m_true.size, 40, replace=False)] = rng.standard_normal(40).astype(np.float32)
    dev = torch.device("cuda", 0)
    with gpu_lib.Context() as ctx:
        ctx.prepare(p, c["vel"], c["wav"])
        d_obs = ctx.model(s, m_true, exact=True)
        obs = Shots(s.sx, s.sy, s.trace_offset, s.trace_cell, d_obs)
        m_ls, cost_ls = least_squares_migration(ctx, obs, niter=6)

        def fwd_t(x):
            y = torch.empty(d_obs.shape, dtype=torch.float32, device=dev)
            torch.cuda.synchronize()
            ctx.model_device(s, x.data_ptr(), y.data_ptr(), exact=True)
            return y

        def adj_t(r):
            y = torch.empty(m_true.shape, dtype=torch.float32, device=dev)
            torch.cuda.synchronize()
            ctx.migrate_device(s, r.data_ptr(), y.data_ptr())
            return y

        inner_t = lambda a, b: float(torch.dot(a.reshape(-1).double(), b.reshape(-1).double()))
        m_t, cost_t = conjugate_gradients(torch.from_numpy(d_obs).to(dev), fwd_t, adj_t, niter=6, inner_fn=inner_t)
        geo = lambda d: Shots(s.sx, s.sy, s.trace_offset, s.trace_cell, np.ascontiguousarray(d, np.float32))
        _, cost_h = conjugate_gradients(d_obs, lambda x: ctx.model(s, np.asarray(x, np.float32), exact=True),
                                        lambda r: ctx.migrate(geo(r)), niter=6)
    assert m_ls.shape == m_true.shape and m_ls.dtype == np.float32
    assert np.array_equal(m_ls, m_t.cpu().numpy())
    assert np.array_equal(cost_ls, cost_t)
    assert np.allclose(cost_ls, cost_h, rtol=1e-4, atol=1e-7)
    assert np.all(np.diff(cost_ls) <= 1e-7) and cost_ls[-1] < 1.0  # CGLS: the residual never grows
