"""Full-size properties on the GPU (the oracle cannot finish these sizes in seconds):
the 64-shot PSPI survey (500 x 1024 grid, nkx 2048, nref 8, 271 frequencies) and the
least-squares workload (32 shots, 300 x 512).

* linearity of the migration in the data (a d1 + b d2), to FP32 rounding;
* additivity over shots: the survey's image equals the sum of the images of two
  disjoint shot subsets (ShotProfileWEM.jl:140-199 stacks shot images the same way);
* scaling the data by a power of two scales the image exactly (bit for bit);
* repeated calls are bit-identical;
* the exact modelling/migration pair passes the dot-product test at full size.
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def survey(gpu_lib):
    from wemgpu import synth
    c = synth.config1()
    ctx = gpu_lib.Context()
    ctx.prepare(c["params"], c["vel"], c["wav"])
    yield gpu_lib, ctx, c
    ctx.close()


def _with_data(gpu_lib, s, d):
    return gpu_lib.Shots(s.sx, s.sy, s.trace_offset, s.trace_cell, np.ascontiguousarray(d, np.float32))


def test_linearity_and_exact_scaling(survey):
    gpu_lib, ctx, c = survey
    s = c["shots"]
    rng = np.random.default_rng(7)
    d2 = rng.standard_normal(s.data.shape).astype(np.float32)
    m1 = ctx.migrate(s).astype(np.float64)
    m2 = ctx.migrate(_with_data(gpu_lib, s, d2)).astype(np.float64)
    m12 = ctx.migrate(_with_data(gpu_lib, s, 0.5 * s.data + 3.0 * d2)).astype(np.float64)
    assert rel_l2(m12, 0.5 * m1 + 3.0 * m2) < 1e-5
    m4 = ctx.migrate(_with_data(gpu_lib, s, 4.0 * s.data))
    assert np.array_equal(m4, (4.0 * m1).astype(np.float32))
    assert np.array_equal(ctx.migrate(s), m1.astype(np.float32))


def test_additivity_over_shots(survey):
    gpu_lib, ctx, c = survey
    s = c["shots"]
    whole = ctx.migrate(s).astype(np.float64)
    k = s.nshot // 3
    parts = []
    for lo, hi in ((0, k), (k, s.nshot)):
        t0, t1 = int(s.trace_offset[lo]), int(s.trace_offset[hi])
        parts.append(ctx.migrate(gpu_lib.Shots(s.sx[lo:hi], s.sy[lo:hi], s.trace_offset[lo:hi + 1] - t0,
                                               s.trace_cell[t0:t1], s.data[t0:t1])).astype(np.float64))
    # equal up to FP32 rounding: the shots pair up differently in the CTAs (2 shots share
    # an item) and the frequency sum of the image cancels strongly, so the rounding of
    # the partial sums shows at ~1e-5 of the image norm (the FP32-vs-FP64 floor of one
    # shot of this survey is 4e-6)
    assert rel_l2(parts[0] + parts[1], whole) < 5e-5


def test_dot_product_full_size_least_squares_pair(gpu_lib):
    from wemgpu import synth
    from wemgpu.cg import dot_test
    c = synth.config4()
    p, s = dict(c["params"], interp="linear"), c["shots"]
    with gpu_lib.Context() as ctx:
        ctx.prepare(p, c["vel"], c["wav"])
        rng = np.random.default_rng(8)
        m = rng.standard_normal((p["nmx"], p["nz"])).astype(np.float32)
        d = rng.standard_normal(s.data.shape).astype(np.float32)
        a, b = dot_test(lambda x: ctx.model(s, np.asarray(x, np.float32), exact=True),
                        lambda r: ctx.migrate(_with_data(gpu_lib, s, r)), m, d)
    assert abs(a - b) / abs(a) < 1e-5
