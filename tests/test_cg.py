"""The CG solver on the reference's own test problems (CPU).

test/test_CG.jl:1-23 solves a random 1000 x 300 least-squares problem with mu = 0.2 through
MatrixMultiplyOp and asserts a quality factor 10 log10(||m1|| / ||m2 - m1||) > 10 dB against
the closed-form ridge solution; the same here, plus the dot test of src/Tools/DotTest.jl.
"""
import numpy as np

from wemgpu.cg import conjugate_gradients, dot_test, inner


def test_cg_matches_closed_form_ridge_solution():
    rng = np.random.default_rng(0)
    A = rng.standard_normal((1000, 300))
    x = rng.standard_normal(300)
    d = A @ x + 0.1 * rng.standard_normal(1000)
    mu = 0.2
    m1 = np.linalg.solve(A.T @ A + mu * np.eye(300), A.T @ d)
    m2, cost = conjugate_gradients(d, lambda m: A @ m, lambda r: A.T @ r, niter=30, mu=mu)
    q = 10 * np.log10(np.linalg.norm(m1) / np.linalg.norm(m2 - m1))
    assert q > 10.0
    assert cost[0] == 1.0 and np.all(np.diff(cost) <= 1e-12)


def test_dot_test_matrix_operator():
    rng = np.random.default_rng(1)
    A = rng.standard_normal((50, 30))
    a, b = dot_test(lambda m: A @ m, lambda d: A.T @ d, rng.standard_normal(30), rng.standard_normal(50))
    assert abs(a - b) / abs(a) < 1e-12


def test_inner_is_float64():
    a = np.full(10_000_000, 0.1, np.float32)
    assert abs(inner(a, a) - 1e5) / 1e5 < 1e-6
