"""Discrete energy of the reference's time loop (CPU oracle, no GPU).

Without sources, the explicit Newmark / velocity-Verlet loop of se2wave.c:4722-4775
(beta = 0, gamma = 1/2) is the central-difference scheme
M (u_{k+1} - 2 u_k + u_{k-1}) / dt^2 = -K u_k, and for symmetric K and diagonal M it
conserves E_{k+1/2} = 1/2 w^T M w + 1/2 u_{k+1}^T K u_k with w = (u_{k+1} - u_k) / dt,
exactly in exact arithmetic.  The oracle (bit-identical to the reference) must keep it
to rounding, and the stiffness it assembles must be symmetric and positive semi-definite.
"""
import numpy as np
import pytest

from oracle import oracle as O
from se2dr_fork_gb300 import spec as S


def _spec(p):
    rng = np.random.default_rng(40 + p)
    mx, my = 7, 5
    return S.explosion64(mx, my, p=p, tmax=1.0).replace(
        nt=10 ** 6, sources=[], receivers=[(0.0, 0.0)], nearest_internal_gll=(p > 1),
        cell_vp=rng.uniform(5000, 7000, mx * my), cell_vs=rng.uniform(2800, 3500, mx * my),
        cell_rho=rng.uniform(2000, 3000, mx * my))


@pytest.mark.parametrize("p", [1, 3, 4, 6])
def test_leapfrog_energy_is_conserved(p):
    o = O.OracleSolver(_spec(p))
    M = o.get("mass")
    rng = np.random.default_rng(p)
    u0 = rng.standard_normal(o.ndof) * 1e-3
    v0 = rng.standard_normal(o.ndof) * 1e-1
    a0 = o.force(u0) / M                     # consistent with u0 (no source)
    o.set_state(u0, v0, a0)
    us = [u0]
    for _ in range(40):
        o.run(1, traces=False)
        us.append(o.state()[0])
    Ku = [-o.force(u) for u in us]           # F = -K u
    E = np.array([0.5 * np.dot((us[k + 1] - us[k]) ** 2 / o.dt ** 2, M) + 0.5 * np.dot(us[k + 1], Ku[k])
                  for k in range(len(us) - 1)])
    assert E.min() > 0
    assert np.abs(E - E[0]).max() / E[0] < 1e-13, np.abs(E - E[0]).max() / E[0]   # measured ~3e-16


@pytest.mark.parametrize("p", [2, 5])
def test_stiffness_is_symmetric_positive_semidefinite(p):
    o = O.OracleSolver(_spec(p))
    rng = np.random.default_rng(p)
    x, y = rng.standard_normal(o.ndof), rng.standard_normal(o.ndof)
    Kx, Ky = -o.force(x), -o.force(y)
    assert abs(np.dot(y, Kx) - np.dot(x, Ky)) <= 1e-12 * np.linalg.norm(Kx) * np.linalg.norm(y)
    assert np.dot(x, Kx) > 0
    # rigid translations are in the null space
    t = np.tile([1.0, 0.0], o.ndof // 2)
    assert np.linalg.norm(o.force(t)) <= 1e-9 * np.linalg.norm(Kx) * np.linalg.norm(t) / np.linalg.norm(x)
