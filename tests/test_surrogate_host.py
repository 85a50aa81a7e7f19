"""Host-side pieces of the surrogate pipeline (no GPU): output layout, mirror
augmentation, the disagreement gate, misfit, the workload's draws, and the coarse-solver
ladder used for the comparison at equal misfit."""
import numpy as np
import pytest

from se2dr_fork_gb300 import host as H
from se2dr_fork_gb300 import spec as S
from se2dr_fork_gb300 import surrogate as SU


def test_network_layout_round_trip():
    t = np.random.default_rng(0).standard_normal((3, 16, 2048)).astype(np.float32)
    n = SU.to_net_layout(t)
    assert np.array_equal(SU.from_net_layout(n), t)
    # row k of a receiver's column holds samples 8k..8k+7 of vx, then of vy
    assert n[1, 2, 5 * 16 + 3] == t[1, 2, 5 * 8 + 3] and n[1, 2, 5 * 16 + 8 + 3] == t[1, 2, 1024 + 5 * 8 + 3]


def test_mirror_is_an_involution_and_maps_receivers():
    rng = np.random.default_rng(1)
    d = SU.Dataset(rng.random((2, 128, 128, 3)).astype(np.float32), np.array([[10.5, 20.0], [100.0, 3.0]], np.float32),
                   rng.standard_normal((2, 16, 2048)).astype(np.float32), np.zeros(2))
    m = SU.mirrored(d)
    assert np.array_equal(m.traces[0, 15, :1024], -d.traces[0, 0, :1024])
    assert np.array_equal(m.traces[0, 15, 1024:], d.traces[0, 0, 1024:])
    assert np.array_equal(m.materials[1, :, 0], d.materials[1, :, 127])
    mm = SU.mirrored(m)
    assert np.array_equal(mm.traces, d.traces) and np.array_equal(mm.materials, d.materials)
    rc = SU.receiver_cells(SU.draw_spec(1, 0))
    assert np.array_equal(127 - rc[::-1], rc)


def test_disagreement_gate():
    rng = np.random.default_rng(2)
    base = rng.standard_normal((5, 16, 2048))
    same = np.stack([base, base, base])
    assert np.all(SU.disagreement(same) < 1e-15)
    assert np.all(np.isinf(SU.disagreement(base[None])))      # one member accepts nothing
    noisy = np.stack([base, base * 1.02, base * 0.98])
    np.testing.assert_allclose(SU.disagreement(noisy), (0 + 0.02 + 0.02) / 3, rtol=1e-9)
    np.testing.assert_allclose(SU.rel_l2(base * 1.1, base), 0.1, rtol=1e-12)


def test_draws_share_one_time_step_and_wavelet():
    a, b = SU.draw_spec(4, 0), SU.draw_spec(4, 1, H.SHOT_OOD)
    assert a.dt == b.dt == SU.surrogate_dt() and a.nt == b.nt == SU.NSTEPS
    assert a.sources[0].par == b.sources[0].par == (0.3, 5.0, 1.0)
    assert a.sources[0].y <= 0.5 * a.my * SU.CELL
    su = H.Setup(a)
    assert su.nsteps == SU.NSTEPS and su.nrec == 16
    assert np.all(su.rec_node // su.nx_g == su.ny_g - 1)
    assert SU.surrogate_dt() <= 0.5 * su.dt_cfl + 1e-15      # stable for every in-distribution draw


def test_coarse_spec_block_averages_and_steps_on_the_same_times():
    sp = SU.draw_spec(4, 3)
    fine_dt = sp.dt
    for mx, p in SU.LADDER:
        c, r = SU.coarse_spec(sp, mx, p, fine_dt)
        f = SU.GRID // mx
        assert (c.mx, c.my, c.p) == (mx, mx, p) and r in (1, 2, 4)
        assert c.dt == r * fine_dt and c.nt == SU.NSTEPS // r
        vp = np.asarray(sp.cell_vp).reshape(mx, f, mx, f)
        np.testing.assert_allclose(np.asarray(c.cell_vp).reshape(mx, mx), vp.mean(axis=(1, 3)), rtol=1e-15)
        np.testing.assert_allclose(np.mean(c.cell_vs), np.mean(sp.cell_vs), rtol=1e-12)   # averaging keeps the mean
        assert c.sources == sp.sources and c.receivers == sp.receivers
        # the coarse step is within the coarse mesh's stability limit at the fastest velocity
        probe = S.Spec(mx=mx, my=mx, p=p, scale=(SU.GRID * SU.CELL,) * 2, shift=(0.0, 0.0), vp=7500.0,
                          vs=7500.0 / 1.6, rho=2500.0, cfl=0.5, tmax=1.0e30, nt=1)
        assert c.dt <= H.Setup(probe).dt * (1 + 1e-12)
    with pytest.raises(ValueError):
        SU.coarse_spec(sp, 48, 4, fine_dt)       # 48 does not divide the 128-cell grid


def test_equal_misfit_picks_the_fastest_solver_at_least_as_accurate():
    ladder = [{"mx": 64, "misfit_mean": 0.01, "draws_per_s": 10.0, "wall_seconds": 2.0, "solver_seconds": 1.0},
              {"mx": 32, "misfit_mean": 0.05, "draws_per_s": 40.0, "wall_seconds": 0.5, "solver_seconds": 0.25},
              {"mx": 16, "misfit_mean": 0.30, "draws_per_s": 90.0, "wall_seconds": 0.2, "solver_seconds": 0.1}]
    eq = SU.equal_misfit(ladder, 0.06, 400.0)
    assert eq["solver"]["mx"] == 32 and eq["gain"] == 10.0
    # against device time: 20 draws in 0.25 s of solver time = 80 draws/s
    assert eq["gain_solver_time"] == 400.0 * 0.25 / 20.0
    assert SU.equal_misfit(ladder, 0.5, 400.0)["solver"]["mx"] == 16
    assert SU.equal_misfit(ladder, 0.001, 400.0) == {"solver": None, "gain": None, "gain_solver_time": None}
