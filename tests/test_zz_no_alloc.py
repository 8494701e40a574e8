"""wem_migrate_noalloc: the migration entry point that allocates nothing.

It exists for callers that cannot call cudaMalloc/cudaFree while they run -- an
application that hands all device memory to its own pool at start-up, or a loop with
a fixed memory budget. They pass device buffers for the inputs and the output; the
library's working memory is one fixed device array. This test calls it through the C
ABI, twice in a row (the second call runs on the array the first one left behind),
and compares each result with the regular entry point wem_migrate on the same
survey, within the tolerance of the other parity tests. The file's name sorts last
so that a run stopping at the first failure has already run every other test.
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


@pytest.mark.parametrize("kind", ["split_step", "pspi_ref", "pspi_linear"])
def test_noalloc_matches_wem_migrate_twice(gpu_lib, kind):
    torch = pytest.importorskip("torch")
    from wemgpu import synth, make_params
    if kind == "split_step":
        c = synth.small_case(71, nx=128, nz=30, nt=128, nshot=2, pspi=0)
    else:
        c = synth.small_case(72, nx=256, nz=24, nt=128, nshot=3, pspi=1, nref=5,
                             interp="ref" if kind == "pspi_ref" else "linear")
    p, vel, wav, shots = c["params"], c["vel"], c["wav"], c["shots"]
    want = gpu_lib.migrate(p, vel, wav, shots)  # the regular entry point

    dev = torch.device("cuda", 0)
    vel_d = torch.from_numpy(np.ascontiguousarray(vel)).to(dev)
    wav_d = torch.from_numpy(np.ascontiguousarray(wav)).to(dev)
    d_d = torch.from_numpy(np.ascontiguousarray(_full_grid(shots, p["nmx"]))).to(dev)
    m_d = torch.empty((p["nmx"], p["nz"]), dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    prm = make_params(**p)
    sx = np.ascontiguousarray(shots.sx, np.float32)
    sy = np.ascontiguousarray(shots.sy, np.float32)
    fp = C.POINTER(C.c_float)
    L = gpu_lib.lib()
    for _ in range(2):
        m_d.fill_(np.nan)
        torch.cuda.synchronize()
        rc = L.wem_migrate_noalloc(C.byref(prm), C.c_void_p(vel_d.data_ptr()), C.c_void_p(wav_d.data_ptr()),
                                   shots.nshot, sx.ctypes.data_as(fp), sy.ctypes.data_as(fp),
                                   C.c_void_p(d_d.data_ptr()), C.c_void_p(m_d.data_ptr()), None)
        assert rc == 0, L.wem_last_error().decode()
        got = m_d.cpu().numpy()
        assert np.all(np.isfinite(got))
        assert rel_l2(got, want) < TOL


def test_noalloc_rejects_sizes_beyond_its_limits(gpu_lib):
    torch = pytest.importorskip("torch")
    from wemgpu import synth, make_params
    c = synth.small_case(73, nx=64, nz=8, nt=64, nshot=1)
    p = dict(c["params"], nmx=2048, padx=1)  # above the 1024-cell limit
    prm = make_params(**p)
    dev = torch.device("cuda", 0)
    buf = torch.zeros(16, dtype=torch.float32, device=dev)
    sx = np.array([100.0], np.float32)
    fp = C.POINTER(C.c_float)
    L = gpu_lib.lib()
    rc = L.wem_migrate_noalloc(C.byref(prm), C.c_void_p(buf.data_ptr()), C.c_void_p(buf.data_ptr()), 1,
                               sx.ctypes.data_as(fp), None, C.c_void_p(buf.data_ptr()), C.c_void_p(buf.data_ptr()),
                               None)
    assert rc == gpu_lib._lib.WEM_ERR_SIZE
    assert "nmx <= 1024" in L.wem_last_error().decode()
