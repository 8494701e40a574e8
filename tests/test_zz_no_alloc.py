"""wem_migrate_noalloc: the migration entry point that allocates nothing.

It exists for callers that cannot call cudaMalloc/cudaFree while they run -- an
application that hands all device memory to its own pool at start-up, or a loop with
a fixed memory budget. They pass device buffers for the inputs and the output; the
library's working memory is one fixed device array. These tests call it through the C
ABI, twice in a row (the second call runs on the array the first one left behind),
and compare each result with the regular entry point wem_migrate on the same survey
and with the oracle's port of the reference, within the tolerance of the other parity
tests. The file's name sorts last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-4


def _full_grid(shots, nmx):
    from wemgpu import synth
    return np.stack([synth.shot_gather_full(shots, s, nmx) for s in range(shots.nshot)])


def _call(gpu_lib, prm, vel_d, wav_d, shots, d_d, m_d):
    sx = np.ascontiguousarray(shots.sx, np.float32)
    sy = np.ascontiguousarray(shots.sy, np.float32)
    fp = C.POINTER(C.c_float)
    return gpu_lib.lib().wem_migrate_noalloc(C.byref(prm), C.c_void_p(vel_d.data_ptr()), C.c_void_p(wav_d.data_ptr()),
                                             shots.nshot, sx.ctypes.data_as(fp), sy.ctypes.data_as(fp),
                                             C.c_void_p(d_d.data_ptr()), C.c_void_p(m_d.data_ptr()), None)


def _port_stack(oracle_mod, c):
    """The oracle's port of the reference (bit-identical to the compiled reference), one
    shot at a time on the full grid, stacked in shot order."""
    from wemgpu import synth
    p, shots = c["params"], c["shots"]
    out = None
    for s in range(shots.nshot):
        q = dict(p, sx=float(shots.sx[s]), sy=float(shots.sy[s]))
        m = oracle_mod.wem_port(q, c["vel"], c["wav"], d=synth.shot_gather_full(shots, s, p["nmx"]), adj=True)
        out = m.astype(np.float64) if out is None else out + m
    return out


def _cases():
    from wemgpu import synth
    return {
        "split_step": lambda: synth.small_case(71, nx=128, nz=30, nt=128, nshot=2, pspi=0),
        "pspi_ref": lambda: synth.small_case(72, nx=256, nz=24, nt=128, nshot=3, pspi=1, nref=5, interp="ref"),
        "pspi_linear": lambda: synth.small_case(72, nx=256, nz=24, nt=128, nshot=3, pspi=1, nref=5, interp="linear"),
        # 2048-point rows (one row team per wavefield) with the most reference velocities
        "pspi_2048_nref16": lambda: synth.small_case(74, nx=1024, nz=8, nt=64, nshot=2, pspi=1, nref=16,
                                                     interp="ref", fmax=20.0),
    }


@pytest.mark.parametrize("kind", ["split_step", "pspi_ref", "pspi_linear", "pspi_2048_nref16"])
def test_noalloc_matches_wem_migrate_twice(gpu_lib, oracle_mod, kind):
    torch = pytest.importorskip("torch")
    from wemgpu import make_params
    c = _cases()[kind]()
    p, vel, wav, shots = c["params"], c["vel"], c["wav"], c["shots"]
    want = gpu_lib.migrate(p, vel, wav, shots)  # the regular entry point
    port = _port_stack(oracle_mod, c)  # and the reference's arithmetic on the CPU
    assert rel_l2(want, port) < TOL

    dev = torch.device("cuda", 0)
    vel_d = torch.from_numpy(np.ascontiguousarray(vel)).to(dev)
    wav_d = torch.from_numpy(np.ascontiguousarray(wav)).to(dev)
    d_d = torch.from_numpy(np.ascontiguousarray(_full_grid(shots, p["nmx"]))).to(dev)
    m_d = torch.empty((p["nmx"], p["nz"]), dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    prm = make_params(**p)
    for _ in range(2):
        m_d.fill_(np.nan)
        torch.cuda.synchronize()
        rc = _call(gpu_lib, prm, vel_d, wav_d, shots, d_d, m_d)
        assert rc == 0, gpu_lib.lib().wem_last_error().decode()
        got = m_d.cpu().numpy()
        assert np.all(np.isfinite(got))
        assert rel_l2(got, want) < TOL
        assert rel_l2(got, port) < TOL


def test_noalloc_after_the_pool_took_the_memory(gpu_lib):
    """The documented order for a caller with its own pool: one small call first (CUDA
    loads the scratch array and the kernels at the library's first use on a device), then
    the pool takes nearly all free memory, and later calls still run."""
    torch = pytest.importorskip("torch")
    from wemgpu import make_params
    c = _cases()["pspi_ref"]()
    p, vel, wav, shots = c["params"], c["vel"], c["wav"], c["shots"]
    dev = torch.device("cuda", 0)
    vel_d = torch.from_numpy(np.ascontiguousarray(vel)).to(dev)
    wav_d = torch.from_numpy(np.ascontiguousarray(wav)).to(dev)
    d_d = torch.from_numpy(np.ascontiguousarray(_full_grid(shots, p["nmx"]))).to(dev)
    m_d = torch.empty((p["nmx"], p["nz"]), dtype=torch.float32, device=dev)
    prm = make_params(**p)
    assert _call(gpu_lib, prm, vel_d, wav_d, shots, d_d, m_d) == 0, gpu_lib.lib().wem_last_error().decode()
    first = m_d.cpu().numpy()
    torch.cuda.synchronize()
    free, _ = torch.cuda.mem_get_info(dev)
    keep = 64 << 20  # what is left to the driver
    pool = torch.empty(max(0, free - keep), dtype=torch.uint8, device=dev) if free > keep else None
    try:
        m_d.fill_(np.nan)
        torch.cuda.synchronize()
        rc = _call(gpu_lib, prm, vel_d, wav_d, shots, d_d, m_d)
        assert rc == 0, gpu_lib.lib().wem_last_error().decode()
        assert rel_l2(m_d.cpu().numpy(), first) < TOL
    finally:
        del pool
        torch.cuda.empty_cache()


def test_noalloc_rejects_sizes_beyond_its_limits(gpu_lib):
    torch = pytest.importorskip("torch")
    from wemgpu import synth, make_params
    c = synth.small_case(73, nx=64, nz=8, nt=64, nshot=1)
    dev = torch.device("cuda", 0)
    buf = torch.zeros(16, dtype=torch.float32, device=dev)
    fp = C.POINTER(C.c_float)
    L = gpu_lib.lib()

    def call(p, nshot):
        prm = make_params(**p)
        sx = np.full(nshot, 100.0, np.float32)
        # rejected before any device memory is touched: the buffers are never read
        return L.wem_migrate_noalloc(C.byref(prm), C.c_void_p(buf.data_ptr()), C.c_void_p(buf.data_ptr()), nshot,
                                     sx.ctypes.data_as(fp), None, C.c_void_p(buf.data_ptr()),
                                     C.c_void_p(buf.data_ptr()), None)

    # a grid above the 1024-cell limit
    assert call(dict(c["params"], nmx=2048, padx=1), 1) == gpu_lib._lib.WEM_ERR_SIZE
    assert "nmx <= 1024" in L.wem_last_error().decode()
    # within every per-axis limit, but the spectra of 64 shots x ~200 frequencies x 1024
    # cells (~100 MB) exceed the scratch array
    big = dict(c["params"], nmx=1024, padx=2, nz=64, nt=1000, dt=0.002, fmin=5.0, fmax=50.0)
    assert call(big, 64) == gpu_lib._lib.WEM_ERR_SIZE
    assert "scratch array" in L.wem_last_error().decode()
