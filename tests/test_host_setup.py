"""The product's FP64 host set-up (libse2host.so) against the reference's golden
vectors and the oracle port, plus its input checks and the material generator."""
import platform

import numpy as np
import pytest

from golden_util import load, spec_of
from oracle import oracle as O
from se2dr_fork_gb300 import host as H
from se2dr_fork_gb300 import spec as S

BITWISE = platform.machine() in ("x86_64", "AMD64")


def same(x, ref, tol=1e-12):
    if BITWISE:
        return np.array_equal(x, ref)
    den = np.linalg.norm(ref)
    return np.linalg.norm(np.asarray(x) - ref) <= tol * (den if den > 0 else 1.0)


@pytest.mark.parametrize("p", range(1, 9))
def test_setup_vs_reference(p):
    d = load(f"hetero_p{p}")
    s = H.Setup(spec_of(d))
    assert same(s.D.ravel(), d["D"]) and same(s.xi, d["xi"]) and same(s.w1d, d["w1d"])
    assert same(s.src_vals.ravel(), d["src_values"])
    assert np.array_equal(np.stack([s.src_elem, s.src_gll], 1).ravel(), d["src_index"])
    assert same(np.array([s.dt_cfl]), d["dt_cfl"])
    assert s.nsteps == d["traces"].shape[0]
    if "mass" in d:
        assert same(s.mass_vec(), d["mass"]) and same(s.coords(), d["coords"])


@pytest.mark.parametrize("p", [1, 3, 6, 8])
def test_setup_vs_oracle_bitwise(p):
    """Same host, same libm: the product set-up and the oracle agree bit for bit."""
    rng = np.random.default_rng(p)
    mx, my = 9, 4
    sp = S.explosion64(mx, my, p=p).replace(
        nearest_internal_gll=(p > 1), cell_vp=rng.uniform(4000, 6000, mx * my),
        cell_vs=rng.uniform(2000, 3000, mx * my), cell_rho=rng.uniform(2000, 3000, mx * my),
        receivers=[(500.0, 500.0), (-1000.0, 999.99), (3.3, -444.4)])
    s, o = H.Setup(sp), O.OracleSolver(sp)
    assert np.array_equal(s.mass_vec(), o.get("mass"))
    assert np.array_equal(s.coords(), o.get("coords"))
    assert np.array_equal(s.D.ravel(), o.get("D"))
    assert s.dt == o.dt and s.nsteps == o.nsteps_planned
    assert np.array_equal(np.stack([s.rec_node, s.rec_elem, s.rec_gll], 1).ravel(), o.get("rec_index"))
    assert np.array_equal(s.src_vals.ravel(), o.get("src_values"))


def test_gll_closed_form():
    """GLL nodes are the roots of (1-x^2) P'_N and weights 2/(N(N+1) P_N(x)^2)."""
    from numpy.polynomial import legendre as L
    for p in range(1, 9):
        xi, w = H.gll(p)
        c = np.zeros(p + 1); c[-1] = 1
        interior = np.sort(L.legroots(L.legder(c)))
        np.testing.assert_allclose(xi, np.concatenate([[-1.0], interior, [1.0]]), atol=1e-14)
        np.testing.assert_allclose(np.sort(w), np.sort(2.0 / (p * (p + 1) * L.legval(xi, c) ** 2)), rtol=1e-13)
        assert abs(w.sum() - 2.0) < 1e-14


def test_derivative_matrix_closed_form():
    """D_ij = P_N(x_i) / (P_N(x_j) (x_i - x_j)), D_00 = -N(N+1)/4, D_NN = +N(N+1)/4, else 0."""
    from numpy.polynomial import legendre as L
    for p in range(1, 9):
        s = H.Setup(S.demo(2, p=max(p, 2)).replace(p=p, nearest_internal_gll=False, sources=[], receivers=[]))
        x = s.xi
        c = np.zeros(p + 1); c[-1] = 1
        PN = L.legval(x, c)
        Dc = np.zeros((p + 1, p + 1))
        for i in range(p + 1):
            for j in range(p + 1):
                if i != j:
                    Dc[i, j] = PN[i] / (PN[j] * (x[i] - x[j]))
        Dc[0, 0] = -p * (p + 1) / 4.0
        Dc[p, p] = p * (p + 1) / 4.0
        np.testing.assert_allclose(s.D, Dc, atol=1e-11 * max(1.0, np.abs(Dc).max()))


def test_stf_vs_reference():
    g = load("stf")
    t = g["ricker"][:, 0]
    vals = np.array([H.stf_eval(0, (0.15, 12.0, 1.0), x) for x in t])
    assert same(vals, g["ricker"][:, 1])
    t = g["yoffe_mode2"][:, 0]
    vals = np.array([H.stf_eval(2, (0.3, 0.45, 1.1), x) for x in t])
    assert same(vals, g["yoffe_mode2"][:, 1])


def test_setup_rejects_bad_input():
    bad = [S.demo(4).replace(sources=[S.Source(5000.0, 0.0, (1, 0, 0, 1))]),       # source outside
           S.demo(4, p=1),                                                        # p=1, interior GLL rule
           S.demo(4).replace(receivers=[(0.0, 1e6)]),                             # receiver outside
           S.demo(4).replace(p=9),                                                # degree beyond 8
           S.demo(4).replace(sources=[S.Source(0, 0, (1, 0, 0, 1), S.STF_YOFFE, (0.2, 0.2, 1.0))]),  # bad Yoffe
           S.demo(4).replace(rho=-1.0)]
    for sp in bad:
        with pytest.raises(ValueError):
            H.Setup(sp)


def test_gaussian_random_field_statistics():
    vp = H.gaussian_random_field(256, 256, 5000.0, 0.1, 8.0, seed=1)
    assert abs(vp.mean() - 5000.0) < 100.0
    assert 350.0 < vp.std() < 650.0
    assert vp.min() >= 5000.0 * 0.7 - 1e-9 and vp.max() <= 5000.0 * 1.3 + 1e-9
    z = (vp.reshape(256, 256) - vp.mean()) / vp.std()
    r1 = (z[:, :-1] * z[:, 1:]).mean()      # neighbour correlation of a Gaussian kernel, std 8 cells
    r16 = (z[:, :-16] * z[:, 16:]).mean()
    assert r1 > 0.95 and r16 < 0.5
    assert np.array_equal(vp, H.gaussian_random_field(256, 256, 5000.0, 0.1, 8.0, seed=1))


def test_nsteps_matches_reference_loop():
    d = load("explosion64")
    s = H.Setup(spec_of(d))
    assert s.nsteps == 4524 == d["traces"].shape[0]


def test_perturbed_materials_bitwise_vs_reference():
    """SpecFECtxSetPerturbedMaterialProperties_Velocity (RAND48 seeds 1, 2, 3), run by the reference."""
    from golden_util import load, spec_of
    from oracle import oracle as O
    d = load("perturbed_p3")
    sp = spec_of(d)
    su = H.Setup(sp)
    lmr = d["cell_lmr"].reshape(3, -1)
    assert np.array_equal(su.lam, lmr[0]) and np.array_equal(su.mu, lmr[1]) and np.array_equal(su.rho, lmr[2])
    assert np.array_equal(O.OracleSolver(sp).get("cell_lmr").reshape(3, -1), lmr)
    assert len(np.unique(su.rho)) == su.mx * su.my
    assert np.all(np.abs(su.rho - sp.rho) <= sp.perturb[2])


@pytest.mark.parametrize("p", [2, 4, 6])
def test_alternative_source_vectors_bitwise_vs_reference(p):
    """Pointwise (1716-1923), cubic-spline kernel (1925-2057, default radius and -sm_h) and P0
    (2059-2200) source vectors, against the reference's own assembly routines."""
    d = load(f"srcvec_p{p}")
    sp = spec_of(d)
    su = H.Setup(sp)
    src = sp.sources[0]
    for impl, h, key in [(0, 0.0, "g_impl0"), (2, 0.0, "g_impl2"), (3, 0.0, "g_impl3"), (2, 310.5, "g_impl2_h310p5")]:
        g = su.source_vector(impl, (src.x, src.y), src.moment, h)
        assert np.array_equal(g, d[key]), key


@pytest.mark.parametrize("impl", [0, 2, 3])
def test_source_entries_reassemble_the_vector(impl):
    d = load("srcvec_p4")
    sp = spec_of(d)
    base = H.Setup(sp)
    g = base.source_vector(impl, (sp.sources[0].x, sp.sources[0].y), sp.sources[0].moment)
    su = H.Setup(sp.replace(src_impl=impl))
    assert su.nsrc_phys == 1 and np.all(su.src_owner == 0)
    assert (su.nsrc == 1) == (impl != 2)
    acc = np.zeros_like(g)
    n1 = su.n1
    for k in range(su.nsrc):
        e = su.src_elem[k]
        ex, ey = e % su.mx, e // su.mx
        for q in range(su.npe):
            node = (ex * su.p + q % n1) + (ey * su.p + q // n1) * su.nx_g
            acc[2 * node:2 * node + 2] += su.src_vals[k, 2 * q:2 * q + 2]
    assert np.array_equal(acc, g)
    times, stf, _ = su.stf_block(0.0, 7)
    assert stf.shape == (7, su.nsrc) and np.all(stf == stf[:, :1])


@pytest.mark.parametrize("p", [3, 4])
def test_interp_receiver_vs_reference(p):
    """RecordUV_interp (se2wave.c:2445-2581): element, weights and interpolated coordinate of
    the host set-up; the weighted sum over the element's nodes of the reference's final
    fields reproduces the reference's last recorded row bit for bit."""
    d = load(f"interp_p{p}")
    sp = spec_of(d)
    su = H.Setup(sp)
    assert su.ninterp == 1 and su.nrec_sta == len(sp.receivers) and su.nrec == su.nrec_sta + su.npe
    # the coordinate the reference prints (%+1.8e)
    np.testing.assert_allclose(su.interp_xri[0], d["interp_xri_text"], rtol=1e-8, atol=1e-6)
    assert abs(su.interp_N[0].sum() - 1.0) < 1e-12
    # the appended receiver entries are the element's nodes in ascending local order
    e = int(su.interp_elem[0])
    base = su.nrec_sta
    for k in range(su.npe):
        node = (e % su.mx * su.p + k % su.n1) + (e // su.mx * su.p + k // su.n1) * su.nx_g
        assert su.rec_elem[base + k] == e and su.rec_gll[base + k] == k and su.rec_node[base + k] == node
    vals = []
    for arr in (d["u"], d["v"]):
        for c in range(2):
            acc = 0.0
            for k in range(su.npe):
                acc += float(su.interp_N[0, k]) * float(arr[2 * su.rec_node[base + k] + c])
            vals.append(acc)
    assert same(np.array(vals), d["interp"][-1, 1:])
    # se2_interp_rows combines receiver rows in the same order
    rng = np.random.default_rng(p)
    rows = rng.standard_normal((4, 7 * su.nrec))
    out = su.interp_rows(rows)
    for j in range(4):
        for c in range(7):
            acc = 0.0
            for k in range(su.npe):
                acc += float(su.interp_N[0, k]) * float(rows[j, 7 * (base + k) + c])
            assert out[j, 0, c] == acc


def test_interp_receiver_rejects_points_outside_the_mesh():
    sp = S.demo(9, 7, p=3, tmax=1.0)
    su = H.Setup(sp)
    for xy in [(1000.0, 0.0), (0.0, 1000.0), (-1000.1, 0.0), (0.0, -2000.0)]:
        with pytest.raises(ValueError, match="interpolating receiver"):
            su.interp_receiver(xy)
        with pytest.raises(ValueError, match="interpolating receiver"):
            H.Setup(sp.replace(interp_receivers=[xy]))
    e, N, xri = su.interp_receiver((-1000.0, -1000.0))     # the domain corner: element 0, xi = eta = -1
    assert e == 0 and N[0] == 1.0 and np.all(N[1:] == 0.0)


def test_write_vts_round_trip(tmp_path):
    """se2_write_vts (the VecView to a VTK viewer of se2wave.c:4764-4770): the grid extent,
    the node positions and every component come back bit for bit."""
    from golden_util import read_vts
    su = H.Setup(S.demo(5, 3, p=3))
    rng = np.random.default_rng(11)
    u, v = rng.standard_normal(su.ndof), rng.standard_normal(su.ndof)
    su.write_vts(tmp_path / "snap.vts", {"disp": u, "velo": v})
    (nx, ny), arrs = read_vts(tmp_path / "snap.vts")
    assert (nx, ny) == (su.nx_g, su.ny_g)
    assert set(arrs) == {"Position", "disp_x", "disp_y", "velo_x", "velo_y"}
    pos = arrs["Position"]
    assert np.array_equal(pos[:, 0], np.tile(su.xnode, ny)) and np.array_equal(pos[:, 1], np.repeat(su.ynode, nx))
    assert np.all(pos[:, 2] == 0)
    for name, f in (("disp", u), ("velo", v)):
        assert np.array_equal(arrs[name + "_x"][:, 0], f[0::2]) and np.array_equal(arrs[name + "_y"][:, 0], f[1::2])
    with pytest.raises(ValueError):
        su.write_vts(tmp_path / "bad.vts", {"disp": u[:-2]})
