"""Seeded shot generator of the ensemble / surrogate workloads (host library, C)."""
import numpy as np
import pytest

from se2dr_fork_gb300 import host as H
from se2dr_fork_gb300 import spec as S


def test_draws_are_seeded_and_in_range():
    ds = [H.shot_draw(3, i) for i in range(200)]
    again = H.shot_draw(3, 17)
    assert bytes(again) == bytes(ds[17])
    assert bytes(H.shot_draw(4, 17)) != bytes(ds[17])
    for d in ds:
        assert 32 <= d.mx <= 512 and 32 <= d.my <= 512 and d.p in (3, 4, 6)
        assert d.nrec == 32 and d.nsteps == 5000 and d.ninc == 1
        for rock in (d.lower, d.upper, d.inc[0][5:8]):
            vp, vs, rho = rock
            assert 3000 <= vp <= 6000 and 1.6 <= vp / vs <= 1.9 and 2000 <= rho <= 3000
        assert 5 <= d.f0 <= 20 and d.t0 == pytest.approx(1.5 / d.f0)
        assert d.moment[1] == d.moment[2]
        assert 0.1 * d.Lx <= d.src_xy[0] <= 0.9 * d.Lx and 0.1 * d.Ly <= d.src_xy[1] <= 0.9 * d.Ly
    assert {d.p for d in ds} == {3, 4, 6}
    m = np.array([[d.moment[0], d.moment[1], d.moment[3]] for d in ds])
    assert abs(m.mean()) < 3e14 and 0.8e15 < m.std() < 1.2e15


def test_training_and_ood_draws():
    for i in range(50):
        t, o = H.shot_draw(1, i, H.SHOT_TRAINING), H.shot_draw(1, i, H.SHOT_OOD)
        assert (t.mx, t.my, t.p, t.nrec, t.ninc) == (128, 128, 4, 16, 1)
        assert o.ninc == 2 and max(o.lower[0], o.upper[0], o.inc[0][5], o.inc[1][5]) <= 7500
        assert t.src_xy[1] <= 0.5 * t.Ly
    assert max(max(H.shot_draw(1, i, H.SHOT_OOD).lower[0] for i in range(200)), 0) > 6000


def test_materials_layers_and_inclusion():
    d = H.shot_draw(3, 5)
    vp, vs, rho = H.shot_materials(d)
    grid = vp.reshape(d.my, d.mx)
    yc = (np.arange(d.my) + 0.5) * d.h
    xc = (np.arange(d.mx) + 0.5) * d.h
    X, Y = np.meshgrid(xc, yc)
    cx, cy, a, b, th = d.inc[0][:5]
    u = (np.cos(th) * (X - cx) + np.sin(th) * (Y - cy)) / a
    w = (-np.sin(th) * (X - cx) + np.cos(th) * (Y - cy)) / b
    inside = u * u + w * w <= 1.0
    expect = np.where(inside, d.inc[0][5], np.where(Y < d.interface_y, d.lower[0], d.upper[0]))
    assert np.array_equal(grid, expect)
    assert inside.sum() > 0


def test_shot_spec_sets_up():
    sp = S.shot(3, 2, size=(20, 16), nt=50)
    su = H.Setup(sp)
    assert (su.mx, su.my, su.nsteps, su.nsrc, su.nrec) == (20, 16, 50, 1, 32)
    assert su.gmin == pytest.approx((0.0, 0.0)) and su.gmax == pytest.approx((20 * 31.25, 16 * 31.25))
    # receivers snap to the top row of nodes
    assert np.all(su.rec_node // su.nx_g == su.ny_g - 1)
