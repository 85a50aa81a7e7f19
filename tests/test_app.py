"""The C host application se2wave_gpu reproduces the reference executable's
stdout, receiver .dat file and .mpimeta file byte for byte (FP64 mode), with
the time loop running on the GPU."""
import os
import subprocess

import numpy as np
import pytest

from golden_util import load, read_vts

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
APP = os.path.join(ROOT, "se2dr_fork_gb300", "bin", "se2wave_gpu")


@pytest.fixture(scope="module")
def app(gpu_lib):
    from se2dr_fork_gb300 import build as B
    B.build_app()
    return APP


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["cli_demo_default", "cli_demo_6x4_p3"])
def test_app_matches_reference_executable(app, name, tmp_path):
    g = load(name)
    args = [str(a) for a in g["args"]]
    r = subprocess.run([app, *args], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout == str(g["stdout"])
    for key in g:
        if key.startswith("name_"):
            fname = str(g[key])
            with open(tmp_path / fname) as f:
                assert f.read() == str(g["file_" + key[5:]]), fname


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["cli_demo_default", "cli_demo_6x4_p3"])
def test_app_fp32_df_receiver_file_matches_reference_values(app, name, tmp_path):
    """With -precision fp32_df the application's receiver file carries the reference's
    values to the 9 significant digits it prints (within 1e-7 of each trace's largest
    value), with the same header and rows."""
    g = load(name)
    args = [str(a) for a in g["args"]] + ["-precision", "fp32_df"]
    r = subprocess.run([app, *args], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    for key in g:
        if key.startswith("name_") and str(g[key]).endswith(".dat"):
            fname = str(g[key])
            ref_text = str(g["file_" + key[5:]])
            got_text = open(tmp_path / fname).read()
            ref_head = [l for l in ref_text.splitlines() if l.startswith("#")]
            got_head = [l for l in got_text.splitlines() if l.startswith("#")]
            assert got_head == ref_head
            ref = np.array([[float(v) for v in l.split()] for l in ref_text.splitlines() if l and not l.startswith("#")])
            got = np.array([[float(v) for v in l.split()] for l in got_text.splitlines() if l and not l.startswith("#")])
            assert got.shape == ref.shape
            assert np.array_equal(got[:, 0], ref[:, 0])
            scale = np.maximum(np.abs(ref[:, 1:]).max(axis=0), 1e-300)
            assert np.max(np.abs(got[:, 1:] - ref[:, 1:]) / scale) < 1e-7


@pytest.mark.gpu
def test_app_fp32_kahan_runs(app, tmp_path):
    r = subprocess.run([app, "-mx", "16", "-bdegree", "4", "-precision", "fp32_kahan", "-tmax", "0.2"], cwd=tmp_path,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    dat = [f for f in os.listdir(tmp_path) if f.endswith(".dat")]
    rows = np.loadtxt(tmp_path / dat[0], comments="#")
    assert rows.shape[1] == 1 + 7 * 3 and np.isfinite(rows).all()


def test_app_verify_stf_matches_reference_ricker(tmp_path):
    """-verify_stf -stf_ricker needs no GPU (host STF tabulation, se2wave.c:4809-4914)."""
    from se2dr_fork_gb300 import build as B
    B.build_host()
    try:
        B.build_gpu()
        B.build_app()
    except Exception as e:  # pragma: no cover - nvcc is part of the build environment
        pytest.skip(f"application not buildable here: {e}")
    r = subprocess.run([APP, "-verify_stf", "-stf_ricker", "-tmax", "0.01", "-dt", "1e-4"], cwd=tmp_path,
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    lines = [l for l in open(tmp_path / "SeismicSTF_Ricker.log") if not l.startswith("#")]
    vals = np.array([float(l.split()[1]) for l in lines])
    assert len(vals) == 101  # accumulated time first reaches tmax after 101 samples
    from oracle import oracle as O
    ref = O.stf(0, (0.15, 12.0, 1.0), 0.0, 1.0e-4, 101)  # the literals the reference uses (se2wave.c:4837)
    np.testing.assert_allclose(vals, ref, rtol=1e-11, atol=1e-300)


@pytest.mark.gpu
def test_app_vts_snapshots_match_oracle_fields(app, tmp_path):
    """-dump_ic_src and -of write the initial displacement and periodic (u, v)
    snapshots named as the reference names them; the fields equal the oracle's
    (FP64, bit for bit) at those steps, and the last snapshot carries the loop's k."""
    from oracle import oracle as O
    from se2dr_fork_gb300 import host as H
    from se2dr_fork_gb300 import spec as S
    r = subprocess.run([app, "-mx", "6", "-my", "4", "-bdegree", "3", "-tmax", "0.5", "-of", "20", "-dump_ic_src"],
                       cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    sp = S.demo(6, 4, p=3, tmax=0.5)
    su = H.Setup(sp)
    (nx, ny), ic = read_vts(tmp_path / "uva.vts")
    assert (nx, ny) == (su.nx_g, su.ny_g) and set(ic) == {"Position", "disp_x", "disp_y"}
    assert np.array_equal(ic["Position"][:, 0], np.tile(su.xnode, ny)) and np.all(ic["disp_x"] == 0)
    ref = O.OracleSolver(sp)
    done = 0
    snaps = sorted(f for f in os.listdir(tmp_path) if f.startswith("step-"))
    steps = [int(f[5:-4]) for f in snaps]
    assert steps[:2] == [20, 40] and all(s % 20 == 0 for s in steps[:-1])
    t = 0.0
    for _ in range(su.nsteps):
        t += su.dt                      # time as the loop accumulates it (se2wave.c:4724)
    last = su.nsteps if t >= su.tmax else su.nsteps + 1
    assert steps[-1] == last
    for f, k in zip(snaps, steps):
        done += ref.run(min(k, su.nsteps) - done, traces=False)["nsteps"]
        u, v, _ = ref.state()
        _, arrs = read_vts(tmp_path / f)
        assert np.array_equal(arrs["disp_x"][:, 0], u[0::2]) and np.array_equal(arrs["disp_y"][:, 0], u[1::2]), f
        assert np.array_equal(arrs["velo_x"][:, 0], v[0::2]) and np.array_equal(arrs["velo_y"][:, 0], v[1::2]), f


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32_kahan"])
def test_app_checkpoint_restart_continues_bitwise(app, tmp_path, precision):
    """-checkpoint_every writes resumable states; -restart from one reproduces the rest of the
    uninterrupted run: the same receiver rows, snapshots and final log lines."""
    args = ["-mx", "6", "-my", "4", "-bdegree", "3", "-tmax", "2.0", "-of", "60", "-precision", precision]
    a, b = tmp_path / "a", tmp_path / "b"
    a.mkdir()
    b.mkdir()
    ra = subprocess.run([app, *args, "-checkpoint_every", "50"], cwd=a, capture_output=True, text=True, timeout=300)
    assert ra.returncode == 0, ra.stderr
    assert "checkpoint-000050.bin" in os.listdir(a)
    rb = subprocess.run([app, *args, "-restart", str(a / "checkpoint-000100.bin")], cwd=b, capture_output=True,
                        text=True, timeout=300)
    assert rb.returncode == 0, rb.stderr
    dat = [f for f in os.listdir(a) if f.endswith(".dat")][0]
    rows_a = [l for l in open(a / dat) if not l.startswith("#")]
    rows_b = open(b / dat).read().splitlines(keepends=True)
    assert len(rows_b) == len(rows_a) - 100 and rows_b == rows_a[100:]
    assert ra.stdout.splitlines()[-3:] == rb.stdout.splitlines()[-3:]
    for f in os.listdir(b):
        if f.endswith(".vts"):
            assert open(a / f, "rb").read() == open(b / f, "rb").read(), f


@pytest.mark.gpu
@pytest.mark.parametrize("p", [3, 4])
def test_app_interp_receiver_file_matches_reference(app, tmp_path, p):
    """-interp_receiver x,y writes RecordUV_interp's file (se2wave.c:2445-2581) byte for byte
    as the reference does (FP64), prints its interpolated-coordinate line, and leaves the
    multi-station file unchanged in layout."""
    g = load(f"interp_p{p}")
    mx, my = int(g["spec_mx"]), int(g["spec_my"])
    cells = np.concatenate([g["spec_cell_vp"], g["spec_cell_vs"], g["spec_cell_rho"]]).astype(np.float64)
    cells.tofile(tmp_path / "cells.bin")
    x, y = (float(v) for v in g["spec_interp_xy"][0])
    args = ["-mx", str(mx), "-my", str(my), "-bdegree", str(p), "-tmax", repr(float(g["spec_tmax"])),
            "-nt", str(int(g["spec_nt"])), "-cells", "cells.bin", "-interp_receiver", f"{x!r},{y!r}"]
    r = subprocess.run([app, *args], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    with open(tmp_path / str(g["dat_name"])) as f:
        assert f.read() == str(g["dat_text"])
    line = [l for l in r.stdout.splitlines() if "interpolated coordinate" in l]
    assert len(line) == 1
    assert np.array_equal([float(t) for t in line[0].split("-->")[1].split()], g["interp_xri_text"])
    sta = np.loadtxt(tmp_path / f"closestqpsource-receiverCP-uva-{mx}x{my}-p{p}-rank0.dat", comments="#")
    assert sta.shape == (g["traces"].shape[0], 1 + 7 * 3)
    np.testing.assert_allclose(sta[:, 1:], g["traces"][:, 1:], rtol=1e-8, atol=1e-30)


@pytest.mark.parametrize("args,message", [
    (["-verify_stf"], "No STF implementation specified. Use one of { -stf_ricker , -stf_yoffe }"),   # se2wave.c:4825
    (["-bdegree", "1"], "Cannot use basis degree = 1 and approximate the source location based on nearest "
                        "cell interior GLL point"),                                                      # se2wave.c:3129
    (["-precision", "fp16"], "unknown -precision fp16"),
    (["-of", "0"], "-of must be at least 1"),
    (["-source_impl", "7"], "-source_impl: valid choices are 0,1,2,3"),
    (["-interp_receiver", "100"], "-interp_receiver: expected x,y"),
])
def test_app_rejects_bad_options_before_the_gpu(tmp_path, args, message):
    """Option and set-up errors are reported (exit status 1, message on stderr) by the host
    code, before any device work; the reference's own messages where it has them."""
    from se2dr_fork_gb300 import build as B
    B.build_host()
    try:
        B.build_gpu()
        B.build_app()
    except Exception as e:  # pragma: no cover - nvcc is part of the build environment
        pytest.skip(f"application not buildable here: {e}")
    r = subprocess.run([APP, "-mx", "4", *args], cwd=tmp_path, capture_output=True, text=True, timeout=60)
    assert r.returncode == 1
    assert message in r.stderr, r.stderr
    assert not any(f.endswith(".dat") for f in os.listdir(tmp_path))


def test_app_rejects_bad_input_files_before_the_gpu(tmp_path):
    """-rec_file and -cells are read on the host: a missing file, a short cell file and a
    receiver outside the domain (the reference's message, se2wave.c:2727-2730) end the run
    with exit status 1 before any device work."""
    from se2dr_fork_gb300 import build as B
    B.build_host()
    try:
        B.build_gpu()
        B.build_app()
    except Exception as e:  # pragma: no cover - nvcc is part of the build environment
        pytest.skip(f"application not buildable here: {e}")

    def run(*args):
        return subprocess.run([APP, "-mx", "4", *args], cwd=tmp_path, capture_output=True, text=True, timeout=60)

    r = run("-rec_file", "missing.txt")
    assert r.returncode == 1 and "cannot open missing.txt" in r.stderr
    np.zeros(47).tofile(tmp_path / "short.bin")          # 3 x 4 x 4 = 48 doubles are needed
    r = run("-cells", "short.bin")
    assert r.returncode == 1 and "cannot read 48 doubles from short.bin" in r.stderr
    (tmp_path / "rec.txt").write_text("0.0 0.0\n1500.0 20.0\n")   # the demo's square is [-1000, 1000]^2
    r = run("-rec_file", "rec.txt")
    assert r.returncode == 1 and "Receiver 1, x-coordinate (+1.5000e+03) > max(domain).x (+1.0000e+03)" in r.stderr
