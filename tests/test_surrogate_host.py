"""Host-side pieces of the surrogate pipeline (no GPU): output layout, mirror
augmentation, the disagreement gate, misfit, and the workload's draws."""
import numpy as np

from se2dr_fork_gb300 import host as H
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
