"""Parity of the sm_103a library with the reference (golden vectors made by the
reference itself) and with the oracle port, through the C-ABI.

FP64 mode must be bit-identical (np.array_equal) to the reference; FP32 with
Kahan-compensated updates must stay within 1e-5 relative L2 of the FP64
receiver traces (the FP32 trace tolerance).
"""
import numpy as np
import pytest

from golden_util import FP32_COMPONENT_TOL, fp32_errors, fp32_errors_ok, load, rel_l2, spec_of
from oracle import oracle as O
from se2dr_fork_gb300 import gpu as G
from se2dr_fork_gb300 import host as H
from se2dr_fork_gb300 import spec as S

pytestmark = pytest.mark.gpu

FP32_TOL = 1e-5


@pytest.fixture(scope="module", autouse=True)
def _lib(gpu_lib):
    return gpu_lib


# ---------------------------------------------------------------- golden (the reference itself)
@pytest.mark.parametrize("p", range(1, 9))
def test_fp64_heterogeneous_traces_bitwise_vs_reference(p):
    d = load(f"hetero_p{p}")
    sol = G.Solver(H.Setup(spec_of(d)), "fp64")
    tr = sol.run()
    assert tr.shape == d["traces"].shape
    assert np.array_equal(tr, d["traces"])
    if "u" in d:
        u, v, a = sol.fields()
        assert np.array_equal(u, d["u"]) and np.array_equal(v, d["v"]) and np.array_equal(a, d["a"])


@pytest.mark.parametrize("name", ["ragged_p4", "demo8_p2"])
def test_fp64_fields_bitwise_vs_reference(name):
    d = load(name)
    sol = G.Solver(H.Setup(spec_of(d)), "fp64")
    tr = sol.run()
    assert np.array_equal(tr, d["traces"])
    u, v, a = sol.fields()
    assert np.array_equal(u, d["u"]) and np.array_equal(v, d["v"]) and np.array_equal(a, d["a"])


@pytest.mark.parametrize("p", [1, 3, 4, 7])
def test_fp64_internal_force_bitwise_vs_reference(p):
    d = load(f"force_p{p}")
    sol = G.Solver(H.Setup(spec_of(d)), "fp64")
    F = sol.assemble_linear_form(d["u"])
    assert np.array_equal(F, d["force"])


def test_fp64_perturbed_materials_bitwise_vs_reference():
    """Cell materials from SpecFECtxSetPerturbedMaterialProperties_Velocity (RAND48), traces and
    final fields against the reference run on them."""
    d = load("perturbed_p3")
    sol = G.Solver(H.Setup(spec_of(d)), "fp64")
    assert np.array_equal(sol.run(), d["traces"])
    u, v, a = sol.fields()
    assert np.array_equal(u, d["u"]) and np.array_equal(v, d["v"]) and np.array_equal(a, d["a"])


@pytest.mark.parametrize("p", [3, 4])
@pytest.mark.parametrize("precision", ["fp64", "fp32_kahan"])
def test_interp_receiver_vs_reference(p, precision):
    """The interpolating receiver (RecordUV_interp, se2wave.c:2445-2581): the element's nodes
    ride in the device receiver list and the host combines their rows.  FP64 is bit-identical
    to the reference's recorded u, v at every step; FP32+Kahan within the FP32 trace
    tolerance of the other receivers."""
    d = load(f"interp_p{p}")
    su = H.Setup(spec_of(d))
    tr = G.Solver(su, precision).run()
    ip = su.interp_rows(tr)
    ref = d["interp"]
    assert ip.shape == (ref.shape[0], 1, 7)
    assert np.array_equal(tr[:, 0], ref[:, 0])
    got = ip[:, 0, :4]
    if precision == "fp64":
        assert np.array_equal(got, ref[:, 1:])
        assert np.array_equal(tr[:, :1 + 7 * su.nrec_sta], d["traces"])
    else:
        for c, tol in enumerate(FP32_COMPONENT_TOL[:4]):
            assert rel_l2(got[:, c], ref[:, 1 + c]) <= tol, (c, rel_l2(got[:, c], ref[:, 1 + c]))


def test_fp64_explosion64_full_run_bitwise_vs_reference():
    d = load("explosion64")
    sol = G.Solver(H.Setup(spec_of(d)), "fp64")
    tr = sol.run()
    assert tr.shape == d["traces"].shape == (4524, 8)
    assert np.array_equal(tr, d["traces"])


def test_fp32_kahan_explosion64_within_tolerance_of_reference():
    d = load("explosion64")
    sol = G.Solver(H.Setup(spec_of(d)), "fp32_kahan")
    tr = sol.run()
    ref = d["traces"]
    assert np.array_equal(tr[:, 0], ref[:, 0])
    ok, errs = fp32_errors_ok(tr, ref)
    print("explosion64 FP32-Kahan relative L2 per component:", ["%.2e" % e for e in errs])
    assert ok, errs


def test_readme_demo_figure_features():
    """Receiver-0 vy of the README run (docs/figs/se2wave-demo-vy.png) from the GPU."""
    d = load("readme_demo64")
    sol = G.Solver(H.Setup(S.demo(64, p=6)), "fp64")
    tr = sol.run()
    assert np.array_equal(tr[:, 0], d["time"]) and np.array_equal(tr[:, 4], d["vy0"])
    t, vy = tr[:, 0], tr[:, 4]
    pk = (t > 0.145) & (t < 0.175)
    tr_ = (t > 0.175) & (t < 0.2)
    assert abs(vy[pk].max() - 5.2e-9) < 0.2e-9 and abs(t[pk][vy[pk].argmax()] - 0.16) < 0.005
    assert abs(vy[tr_].min() + 6.0e-9) < 0.2e-9 and abs(t[tr_][vy[tr_].argmin()] - 0.187) < 0.005


# ---------------------------------------------------------------- oracle port, other shapes
@pytest.mark.parametrize("p,mx,my", [(1, 40, 3), (2, 17, 33), (3, 12, 23), (4, 9, 17), (5, 7, 13),
                                     (6, 11, 6), (7, 5, 9), (8, 9, 5), (4, 1, 1), (6, 1, 7)])
def test_fp64_vs_oracle_ragged_meshes(p, mx, my):
    rng = np.random.default_rng(p * 100 + mx)
    Lx = 2000.0
    sp = S.explosion64(mx, my, p=p, tmax=1.0).replace(
        nt=25, nearest_internal_gll=(p > 1),
        cell_vp=rng.uniform(5000, 7000, mx * my), cell_vs=rng.uniform(2800, 3500, mx * my),
        cell_rho=rng.uniform(2000, 3000, mx * my),
        sources=[S.Source(rng.uniform(-1000, 1000), rng.uniform(-1000, 1000), tuple(rng.normal(0, 1e15, 4)),
                          S.STF_RICKER, (0.002, 60.0, 1.0)) for _ in range(3)],
        receivers=[tuple(rng.uniform(-Lx / 2, Lx / 2, 2)) for _ in range(4)] + [(-1000.0, -1000.0), (999.9, 999.9)])
    sol = G.Solver(H.Setup(sp), "fp64")
    tr = sol.run()
    ref = O.OracleSolver(sp)
    rr = ref.run(10 ** 6)
    assert np.array_equal(tr, rr["traces"])
    u, v, a = sol.fields()
    ru, rv, ra = ref.state()
    assert np.array_equal(u, ru) and np.array_equal(v, rv) and np.array_equal(a, ra)


def test_fp64_norms_vs_oracle():
    sp = S.demo(10, 7, p=4, tmax=1.0).replace(nt=200)
    sol = G.Solver(H.Setup(sp), "fp64")
    sol.run()
    ref = O.OracleSolver(sp)
    rr = ref.run(10 ** 6, norms=True)
    last = rr["norms"][-1, 1:]
    np.testing.assert_allclose(sol.norms(), last, rtol=1e-12, atol=0)


@pytest.mark.parametrize("bad", [np.nan, np.inf])
@pytest.mark.parametrize("precision", ["fp64", "fp32_kahan"])
def test_norms_report_non_finite_fields(precision, bad):
    """The log norms (se2wave.c:4747-4755) double as the blow-up detector: a non-finite
    value injected into the host fields before upload comes back as SE2GPU_ERR_NUMERIC."""
    setup = H.Setup(S.demo(6, 6, p=3, tmax=1.0).replace(nt=10))
    sol = G.Solver(setup, precision)
    sol.run(3)
    u, v, a = sol.fields()
    assert np.all(np.isfinite(sol.norms()))
    u[setup.ndof // 3] = bad
    sol.set_fields(u, v, a)
    with pytest.raises(G.GpuError, match="non-finite"):
        sol.norms()


def test_fp64_set_fields_then_step_matches_oracle():
    sp = S.demo(6, 6, p=5, tmax=1.0).replace(nt=10)
    setup = H.Setup(sp)
    rng = np.random.default_rng(5)
    u0, v0, a0 = (rng.standard_normal(setup.ndof) * s for s in (1e-6, 1e-3, 1.0))
    sol = G.Solver(setup, "fp64")
    sol.set_fields(u0, v0, a0)
    tr = sol.run()
    ref = O.OracleSolver(sp)
    ref.set_state(u0, v0, a0)
    rr = ref.run(10 ** 6)
    assert np.array_equal(tr, rr["traces"])
    assert all(np.array_equal(x, y) for x, y in zip(sol.fields(), ref.state()))


@pytest.mark.parametrize("precision", ["fp64", "fp32_kahan", "fp32"])
def test_deterministic_repeat(precision):
    d = load("hetero_p4")
    runs = []
    for _ in range(2):
        sol = G.Solver(H.Setup(spec_of(d)), precision)
        runs.append((sol.run(), *sol.fields()))
    assert all(np.array_equal(x, y) for x, y in zip(*runs))


@pytest.mark.parametrize("precision", ["fp32_kahan", "fp32"])
@pytest.mark.parametrize("p", range(1, 9))
def test_fp32_vs_fp64(p, precision):
    sp = S.explosion64(16, 13, p=p, tmax=0.25).replace(nearest_internal_gll=(p > 1))
    setup = H.Setup(sp)
    t64 = G.Solver(setup, "fp64").run()
    t32 = G.Solver(setup, precision).run()
    ok, errs = fp32_errors_ok(t32, t64)
    print(f"p={p} {precision} relative L2 per component:", ["%.2e" % e for e in errs])
    assert ok, errs


def test_internal_force_device_entry_point():
    import torch
    d = load("force_p4")
    sol = G.Solver(H.Setup(spec_of(d)), "fp64")
    u = torch.tensor(d["u"], dtype=torch.float64, device="cuda")
    F = torch.empty_like(u)
    sol.set_stream(torch.cuda.current_stream().cuda_stream)
    sol.assemble_linear_form_device(u.data_ptr(), F.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(F.cpu().numpy(), d["force"])


# ---------------------------------------------------------------- full-size properties (2048^2, degree 4)
# 67M nodes: too large for the CPU oracle, so these check size-independent
# properties with every tile active (random initial fields).
@pytest.fixture(scope="module")
def grf_setup():
    return H.Setup(S.grf2048(nt=24))


@pytest.fixture(scope="module")
def grf_u0(grf_setup):
    rng = np.random.default_rng(2048)
    return rng.standard_normal(grf_setup.ndof) * 1e-3


def _full_run(setup, precision, u0, scale, nsteps=24):
    sol = G.Solver(setup, precision)
    sol.set_fields(u=scale * u0)
    t = 0.0
    times, stf, t = setup.stf_block(t, nsteps)
    sol.advance(nsteps, stf=scale * stf)
    tr = sol.traces()
    u, v, a = sol.fields()
    sol.close()
    return tr, u, v, a


@pytest.mark.parametrize("precision", ["fp64", "fp32_kahan"])
def test_full_size_linearity(grf_setup, grf_u0, precision):
    """Doubling the initial field and the moment doubles every field exactly
    (scaling by 2 commutes with every rounding)."""
    r1 = _full_run(grf_setup, precision, grf_u0, 1.0)
    r2 = _full_run(grf_setup, precision, grf_u0, 2.0)
    for x1, x2 in zip(r1, r2):
        assert np.array_equal(x2[..., 1:] if x2.ndim == 2 else x2, 2.0 * (x1[..., 1:] if x1.ndim == 2 else x1))


def test_full_size_fp32_kahan_vs_fp64(grf_setup, grf_u0):
    r64 = _full_run(grf_setup, "fp64", grf_u0, 1.0)
    r32 = _full_run(grf_setup, "fp32_kahan", grf_u0, 1.0)
    for x32, x64 in zip(r32[1:], r64[1:]):
        assert rel_l2(x32, x64) <= FP32_TOL
    assert rel_l2(r32[0][:, 1:], r64[0][:, 1:]) <= FP32_TOL


def test_full_size_deterministic(grf_setup, grf_u0):
    r1 = _full_run(grf_setup, "fp32_kahan", grf_u0, 1.0, nsteps=8)
    r2 = _full_run(grf_setup, "fp32_kahan", grf_u0, 1.0, nsteps=8)
    assert all(np.array_equal(x, y) for x, y in zip(r1, r2))


# ---------------------------------------------------------------- errors are reported, not crashed
def test_errors_are_reported():
    sp = S.demo(4, 4, p=2, tmax=1.0).replace(nt=8)
    setup = H.Setup(sp)
    with pytest.raises(G.GpuError):
        G.Solver(setup, 17)
    sol = G.Solver(setup, "fp64", trace_capacity=4)
    with pytest.raises(G.GpuError):
        sol.advance(5)
    sol.advance(4)
    assert sol.traces().shape == (4, 22)


@pytest.mark.parametrize("precision", ["fp64", "fp32_kahan", "fp32"])
def test_no_sources_no_receivers_stays_at_rest(precision):
    """Empty source and receiver lists: the state stays exactly zero, the trace rows are empty,
    and zero or negative step counts through the C-ABI do nothing or are refused."""
    sp = S.demo(5, 4, p=3, tmax=1.0).replace(nt=12, sources=[], receivers=[])
    sol = G.Solver(H.Setup(sp), precision)
    tr = sol.run()
    assert tr.shape == (0, 1)
    assert all(not np.any(f) for f in sol.fields())
    assert np.array_equal(sol.norms(), np.zeros(6))
    lib = G.lib()
    assert lib.se2gpu_advance(sol._h, 0, None) == 0
    assert lib.se2gpu_advance(sol._h, -1, None) == -1 and b"negative" in lib.se2gpu_last_error(sol._h)


def test_sources_need_stf_values():
    sol = G.Solver(H.Setup(S.demo(4, 4, p=2, tmax=1.0).replace(nt=4)), "fp32_kahan")
    assert G.lib().se2gpu_advance(sol._h, 2, None) == -1
    assert b"stf values required" in G.lib().se2gpu_last_error(sol._h)
    sol.advance(2)                      # with the host's STF values it runs
    assert sol.traces().shape == (2, 22)


@pytest.mark.parametrize("precision", ["fp32_kahan", "fp32"])
@pytest.mark.parametrize("p", [3, 4, 6])
def test_fp32_tile_configs_agree(p, precision):
    """Every tile configuration gives the same fields (same arithmetic, different tiling)."""
    sp = S.demo(19, 17, p=p, tmax=1.0).replace(nt=30)
    setup = H.Setup(sp)
    ref = None
    sol = G.Solver(setup, precision)
    for c in range(len(sol.tile_configs())):
        s2 = G.Solver(setup, precision)
        s2.set_tile_config(c)
        out = (s2.run(), *s2.fields())
        if ref is None:
            ref = out
        else:
            assert all(np.array_equal(x, y) for x, y in zip(out, ref)), c


@pytest.mark.parametrize("precision", ["fp32_kahan", "fp32"])
def test_fp32_tile_configs_agree_many_tiles_per_cta(precision):
    """Degree 4 on 260 x 250 elements (1088-1892 tiles), several times what the persistent
    grid holds, so that every CTA walks at least four tiles through its copy pipeline (two
    region stages, one or two owned buffers; the cell constants, 1/M and the tile's bounds
    arriving with the copies), the last ones ragged: every configuration gives the same
    fields."""
    setup = H.Setup(S.demo(260, 250, p=4, tmax=1.0).replace(nt=12))
    ref = None
    ncfg = len(G.Solver(setup, precision).tile_configs())
    assert ncfg >= 6
    for c in range(ncfg):
        s2 = G.Solver(setup, precision)
        s2.set_tile_config(c)
        out = (s2.run(), *s2.fields())
        if ref is None:
            ref = out
        else:
            assert all(np.array_equal(x, y) for x, y in zip(out, ref)), c


def test_default_tile_config_and_getter():
    """A new plain or Kahan handle starts with its degree's default configuration (degree 4:
    configuration 1, 7x7 tiles with two owned buffers); the two-float and FP64 modes with 0;
    se2gpu_tile_config follows se2gpu_set_tile_config."""
    setup = H.Setup(S.demo(9, 7, p=4, tmax=1.0).replace(nt=4))
    for prec, want in [("fp32_kahan", 1), ("fp32", 1), ("fp32_df", 0), ("fp64", 0)]:
        sol = G.Solver(setup, prec)
        assert sol.tile_config == want, prec
        assert G.lib().se2gpu_tile_config(sol._h) == want
        if prec != "fp64":
            sol.set_tile_config(2)
            assert G.lib().se2gpu_tile_config(sol._h) == 2
        sol.close()


@pytest.mark.parametrize("p", [1, 3, 4, 8])
def test_tile_config_info(p):
    """se2gpu_tile_config_info agrees with se2gpu_tile_configs and reports one or two owned
    buffers and at least one resident CTA per SM for every FP32 configuration."""
    setup = H.Setup(S.demo(9, 7, p=p, tmax=1.0).replace(nt=4, nearest_internal_gll=(p > 1)))
    sol = G.Solver(setup, "fp32_kahan")
    cfgs = sol.tile_configs()
    for c, (edge, threads) in enumerate(cfgs):
        info = sol.tile_config_info(c)
        assert (info["edge"], info["threads"]) == (edge, threads)
        assert info["owned_buffers"] in (1, 2) and 1 <= info["ctas_per_sm"] <= 3, info
    with pytest.raises(G.GpuError):
        sol.tile_config_info(len(cfgs))
    f64 = G.Solver(setup, "fp64").tile_config_info(0)
    assert f64["owned_buffers"] == 0 and f64["ctas_per_sm"] == 0


@pytest.mark.parametrize("precision", ["fp64", "fp32_df", "fp32_kahan", "fp32"])
def test_checkpoint_resume_is_bitwise(precision):
    """Stop after 37 steps, checkpoint, resume in a new handle: identical traces and fields."""
    d = load("hetero_p4")
    setup = H.Setup(spec_of(d))
    ref = G.Solver(setup, precision)
    tr_ref = np.concatenate([ref.run(37), ref.run(23)])
    a = G.Solver(setup, precision)
    tr_a = a.run(37)
    blob = a.checkpoint()
    a.close()
    b = G.Solver(setup, precision)
    b.restore(blob)
    tr_b = b.run(23)
    assert np.array_equal(np.concatenate([tr_a, tr_b]), tr_ref)
    assert all(np.array_equal(x, y) for x, y in zip(b.fields(), ref.fields()))


def test_checkpoint_rejects_other_problems_and_buffered_rows():
    d = load("hetero_p4")
    s1 = H.Setup(spec_of(d))
    a = G.Solver(s1, "fp64")
    a.advance(3)
    with pytest.raises(G.GpuError, match="buffered"):
        a.checkpoint()
    a.traces()
    blob = a.checkpoint()
    other = G.Solver(H.Setup(spec_of(load("hetero_p3"))), "fp64")
    with pytest.raises(G.GpuError, match="another problem"):
        other.restore(blob)
    with pytest.raises(G.GpuError, match="another problem"):
        G.Solver(s1, "fp32").restore(blob)
    # a truncated buffer is rejected before the handle is touched: the full one loads after it
    n = G.lib().se2gpu_checkpoint_size(a.handle)
    b = G.Solver(s1, "fp64")
    assert G.lib().se2gpu_checkpoint_load(b.handle, blob[:n], n - 8) < 0
    assert "truncated" in G.lib().se2gpu_last_error(b.handle).decode()
    b.restore(blob)
    assert np.array_equal(b.run(5)[:, 1:], a.run(5)[:, 1:])


@pytest.mark.parametrize("impl", [0, 2, 3])
def test_alternative_source_representations_run(impl):
    """Source vectors of the pointwise, cubic-spline and P0 representations (their set-up is pinned
    bitwise against the reference on the host) drive the device loop: exactly linear in the moment in
    FP64, and FP32-Kahan within its error bars."""
    sp = spec_of(load("srcvec_p4")).replace(src_impl=impl, nt=120, receivers=[(300.0, 400.0), (-700.0, 150.0)],
                                            sources=[S.Source(137.3, -251.9, (1e15, 3e14, -2e14, 5e14),
                                                              S.STF_RICKER, (0.05, 8.0, 1.0))])
    t1 = G.Solver(H.Setup(sp), "fp64").run()
    sp2 = sp.replace(sources=[S.Source(137.3, -251.9, (2e15, 6e14, -4e14, 1e15), S.STF_RICKER, (0.05, 8.0, 1.0))])
    t2 = G.Solver(H.Setup(sp2), "fp64").run()
    assert np.abs(t1[:, 1:]).max() > 0
    assert np.array_equal(t2[:, 1:], 2.0 * t1[:, 1:])
    t32 = G.Solver(H.Setup(sp), "fp32_kahan").run()
    ok, errs = fp32_errors_ok(t32, t1, k=2 * np.pi * 8.0 / sp.vs)
    assert ok, errs


@pytest.mark.parametrize("precision", [64, 34, 33, 32])
def test_create_rejects_a_non_positive_mass_on_the_gpu(precision):
    """Where the device reads pageable host memory the FP32 modes check the mass in the
    kernel that forms 1/M (no host pass); the first bad node is reported either way, and
    a later create on good input succeeds."""
    import ctypes
    su = H.Setup(S.demo(4, 3, p=2, tmax=1.0).replace(nt=4))
    pr, keep = G._problem(su)
    m = np.array(su.mass)
    m[7] = 0.0
    m[9] = -1.0
    m[11] = np.nan
    pr.mass = m.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    h = ctypes.c_void_p()
    rc = G.lib().se2gpu_create(ctypes.byref(pr), precision, 4, ctypes.byref(h))
    assert rc == -1 and not h.value
    assert b"node 7 is not positive" in G.lib().se2gpu_create_error(), G.lib().se2gpu_create_error()
    name = {64: "fp64", 34: "fp32_df", 33: "fp32_kahan", 32: "fp32"}[precision]
    assert G.Solver(su, name).run().shape[0] == su.nsteps
