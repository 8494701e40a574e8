"""Conjugate gradients for least-squares migration.

Restates src/Solvers/ConjugateGradients.jl:1-39 (Algorithm 2 of Scales, 1987, "Tomographic
inversion via the conjugate gradient method"): minimise ||L m - d||^2 + mu ||m||^2 given a
forward operator L and its adjoint L'. Differences from the reference: inner products are
accumulated in float64 (the reference's InnerProduct returns Float32, src/Tools/InnerProduct.jl:1-5,
too coarse for a 1e-5 dot test), and the operator pair is two callables instead of a list of
Julia operators chained by LinearOperator (src/Operators/LinearOperator.jl:1-22).

The cost history is normalised by the initial residual <d, d> like the reference's.
"""
from __future__ import annotations

from typing import Callable

import numpy as np


def inner(a: np.ndarray, b: np.ndarray) -> float:
    """Re(sum(conj(a) * b)) in float64 (src/Tools/InnerProduct.jl:1-5 in FP32)."""
    a = np.asarray(a)
    b = np.asarray(b)
    if np.iscomplexobj(a) or np.iscomplexobj(b):
        return float(np.real(np.vdot(a.astype(np.complex128).ravel(), b.astype(np.complex128).ravel())))
    return float(np.dot(a.astype(np.float64).ravel(), b.astype(np.float64).ravel()))


def _copy(x):
    return x.clone() if hasattr(x, "clone") else np.array(x, copy=True)


def conjugate_gradients(d, forward: Callable, adjoint: Callable, niter: int = 10, mu=0.0,
                        tol: float = 1.0e-15, callback: Callable | None = None, inner_fn: Callable = inner):
    """Returns (m, cost) with cost[0] = 1 and cost[i] = (||r||^2 + mu ||m||^2)/||d||^2.
    d, and what forward/adjoint return, are NumPy arrays, or device tensors with inner_fn a
    float64 inner product of them. mu is one weight, or (NumPy models) one per component along
    the model's first axis, as the multi-component ConjugateGradients of
    src/Solvers/ConjugateGradients.jl:95-150 takes [mu1; mu2]."""
    inner_ = inner_fn
    mus = np.atleast_1d(np.asarray(mu, dtype=np.float64))
    if mus.size == 1:
        mu_dot = lambda x: float(mus[0]) * inner_(x, x)  # noqa: E731
        mu_times = lambda x: float(mus[0]) * x  # noqa: E731
    else:
        mu_dot = lambda x: sum(float(mk) * inner_(x[k], x[k]) for k, mk in enumerate(mus))  # noqa: E731
        mu_times = lambda x: x * mus.reshape((-1,) + (1,) * (np.ndim(x) - 1)).astype(x.dtype)  # noqa: E731
    cost = [1.0]
    r = _copy(d)
    g = adjoint(r)
    m = g * 0  # zeros of g's kind
    s = _copy(g)
    gamma = inner_(g, g)
    gamma00 = gamma
    cost0 = inner_(r, r)
    for it in range(1, niter + 1):
        t = forward(s)
        delta = inner_(t, t) + mu_dot(s)
        if delta <= tol:
            break
        alpha = gamma / delta
        m = m + alpha * s
        r = r - alpha * t
        g = adjoint(r)
        g = g - mu_times(m)
        gamma0 = gamma
        gamma = inner_(g, g)
        cost1 = inner_(r, r) + mu_dot(m)
        cost.append(cost1 / cost0 if cost0 > 0 else 0.0)
        beta = gamma / gamma0
        s = beta * s + g
        if callback is not None:
            callback(it, m, cost[-1])
        if np.sqrt(gamma) <= np.sqrt(gamma00) * tol:
            break
    return m, np.asarray(cost)


def least_squares_migration(ctx, shots, niter: int = 10, mu: float = 0.0, tol: float = 1.0e-15,
                            exact: bool = True, callback: Callable | None = None):
    """Least-squares migration of host trace data: ConjugateGradients(d, [WEM operator], ...;
    Niter, mu, tol) (src/Solvers/ConjugateGradients.jl:1-39) over the prepared context's
    Born modelling / migration pair, with the data, residual, image and search vectors held
    in device memory for the whole solve. The traces of `shots` (host, [ntrace, nt]) are
    copied to the device once from pinned memory; the image comes back once. exact=True
    takes the exact adjoint of migrate() as the forward operator (a symmetric pair for CG);
    exact=False the reference's Born operator. Returns (m [nmx*nmy, nz] float32, cost)."""
    import torch
    p = ctx.params
    if p is None:
        raise RuntimeError("prepare() first")
    dev = torch.device("cuda", torch.cuda.current_device())
    d_host = torch.from_numpy(np.ascontiguousarray(shots.data, np.float32)).pin_memory()
    d_obs = d_host.to(dev, non_blocking=True)
    ntr, nt = d_obs.shape
    nm = (p.nmx * p.nmy, p.nz)
    cur = torch.cuda.current_stream(dev)

    def fwd(m_t):
        d_t = torch.empty((ntr, nt), dtype=torch.float32, device=dev)
        cur.synchronize()  # the library works on its own stream
        ctx.model_device(shots, m_t.data_ptr(), d_t.data_ptr(), exact=exact)
        return d_t

    def adj(r_t):
        m_t = torch.empty(nm, dtype=torch.float32, device=dev)
        cur.synchronize()
        ctx.migrate_device(shots, r_t.data_ptr(), m_t.data_ptr())
        return m_t

    inner_dev = lambda x, y: float(torch.dot(x.reshape(-1).double(), y.reshape(-1).double()))
    m_t, cost = conjugate_gradients(d_obs, fwd, adj, niter=niter, mu=mu, tol=tol, callback=callback,
                                    inner_fn=inner_dev)
    m_out = torch.empty(nm, dtype=torch.float32).pin_memory()
    m_out.copy_(m_t)
    return m_out.numpy(), cost


def dot_test(forward, adjoint, m_rand: np.ndarray, d_rand: np.ndarray):
    """<d, L m> and <L' d, m> (src/Tools/DotTest.jl:1-12) in float64."""
    d_fwd = forward(m_rand)
    m_adj = adjoint(d_rand)
    return inner(d_rand, d_fwd), inner(m_rand, m_adj)


def trace_weights(d: np.ndarray, cutoff: float = 1e-10) -> np.ndarray:
    """1 for every trace (last axis = time) whose energy exceeds `cutoff`, else 0: the data
    weights of CalculateSampling (src/Tools/CalculateSampling.jl:1-18)."""
    d = np.asarray(d, np.float64)
    return (np.sum(d * d, axis=-1) > cutoff).astype(np.float32)


def least_squares_elastic(params: dict, vp, vs, wav, sx, ux, uz, niter: int = 10, mu=(0.0, 0.0),
                          tol: float = 1.0e-15, sy=None, device: int = 0, callback: Callable | None = None):
    """Elastic least-squares migration: ConjugateGradients over [ApplyDataWeights, SeisMute,
    ShotProfileEWEM] as ShotProfileLSEWEM builds it (src/Imaging/ShotProfileLSEWEM.jl:1-19; its
    mute has tmute = 0, vmute = 999999, so it keeps every sample). The model is (mpp, mps2)
    [2, nmx, nz], the data (ux, uz) [2, nshot, nmx, nt] on every grid cell, weighted by the
    sampling of the x component (CalculateSampling of d[1]); the operators are wem_elastic's
    migration and forward operator, the reference's pair. mu: one weight per image (the
    multi-component CG, ConjugateGradients.jl:95-150). Returns (mpp, mps2, cost)."""
    from .api import elastic
    ux = np.asarray(ux, np.float32)
    uz = np.asarray(uz, np.float32)
    w = trace_weights(ux)[..., None]  # [nshot, nmx, 1]
    d = np.stack([ux * w, uz * w])

    def fwd(m):
        a, b = elastic(params, vp, vs, wav, sx, sy, mpp=m[0], mps2=m[1], adj=False, device=device)
        return np.stack([a * w, b * w])

    def adj(r):
        a, b = elastic(params, vp, vs, wav, sx, sy, ux=r[0] * w, uz=r[1] * w, adj=True, device=device)
        return np.stack([a, b])

    m, cost = conjugate_gradients(d, fwd, adj, niter=niter, mu=mu, tol=tol, callback=callback)
    return m[0], m[1], cost
