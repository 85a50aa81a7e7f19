"""Host-side arithmetic of bench.py (no GPU): the bytes per node the roofline divides by,
the whole-job value of replicas, and the clock-record summary."""
import bench


def test_bytes_per_node_at_degree_4():
    ne, nn = 2048 * 2048, 8193 * 8193
    cell = ne / nn
    # the plain and Kahan kernels read 16 bytes of constants per cell
    assert abs(bench.alg_bytes_per_node("fp32_kahan", ne, nn) - (68 + 16 * cell)) < 1e-12
    assert abs(bench.alg_bytes_per_node("fp32", ne, nn) - (36 + 16 * cell)) < 1e-12
    assert abs(bench.alg_bytes_per_node("fp64", ne, nn) - (104 + 16 * cell)) < 1e-12
    # the reference's update sequence: u, v, a (+ Kahan terms of u, v) read and written, 1/M, (lambda, mu)
    assert round(bench.reference_bytes_per_node("fp32_kahan", ne, nn), 1) == 84.5
    assert round(bench.reference_bytes_per_node("fp32", ne, nn), 1) == 52.5
    assert bench.reference_bytes_per_node("fp64", ne, nn) == bench.alg_bytes_per_node("fp64", ne, nn)
    rf = bench.reference_formulation("fp32_kahan", ne, nn, 1e-3, 6800.0)
    assert abs(rf["achieved"] - rf["bytes_per_node"] * nn / 1e-3 / 1e9) < 1e-6 and abs(rf["frac"] - rf["achieved"] / 6800.0) < 1e-15


def test_replica_value_is_the_whole_job():
    assert bench.replica_value(1000, 10, 4, 2.0) == 4 * 1000 * 10 / 2.0
    assert bench.replica_seconds(1.5) == 1.5          # single process: no collective


def test_clock_summary_reports_median_and_slowdowns():
    c = bench.ClockSampler(0)
    c.lines = ["0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active",
               "0, 1980, 2070, 1390.0, 0x4, Not Active, Not Active, Not Active, Active",
               "0, 2070, 2070, 1000.0, 0x0, Not Active, Not Active, Not Active, Not Active",
               "garbage line",
               "0, [N/A], 2070, 0, 0x0, Not Active, Not Active, Not Active, Not Active"]
    s = c.summary()
    assert s == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}
    c.lines.append("0, 1200, 2070, 700, 0x8, Active, Not Active, Not Active, Not Active")
    assert "hw_slowdown" in c.summary()["reasons"]
    assert bench.ClockSampler(0).summary()["sm_mhz"] is None


def test_median_job_reports_the_middle_run_with_its_parts():
    runs = [(0.0516, {"create_s": 0.0516}), (0.0243, {"create_s": 0.0042}), (0.0244, {"create_s": 0.0043})]
    assert bench.median_job(runs) == (0.0244, {"create_s": 0.0043})
    assert bench.median_job(runs[:1]) == runs[0]
