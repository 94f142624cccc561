"""The benchmark's error reports against the 1e-12 reference (host-side
arithmetic, on the golden vectors) and its guard that records a failed
report instead of ending the run."""
import numpy as np

import bench


def test_state_error_report_on_the_reference_itself():
    g, t = bench._gold("net20_fwd"), bench._gold("net20_fwd_tight")
    w = bench.workload()
    assert np.array_equal(w.p[g["idx"]], g["p"])  # the golden set is a subset of the benchmark batch
    r = bench.state_error_report(g["x"], g, t)
    assert r["instances"] == len(g["idx"])
    assert r["x_tol_units_max"] == r["reference_x_tol_units_max"] > 0
    r2 = bench.state_error_report(t["x"], g, t)
    assert r2["x_tol_units_max"] == 0.0 and r2["x_rel_err_max_where_above_1e3_atol"] == 0.0


def test_gradient_error_report_on_the_reference_itself():
    # the reference at the stated tolerances (rtol 1e-8, atol 1e-10) against
    # itself at 1e-12; with its default stability-limit detection one n = 200
    # instance (8192, stiffness ratio near 1e8) errs 1.4e-6 in llh
    for name, llh_bound in (("net100_asa", 1e-6), ("net50_fsa", 1e-6), ("net200_asa", 2e-6)):
        g, t = bench._gold(name), bench._gold(f"{name}_tight")
        r = bench.gradient_error_report(g["llh"], g["sllh"], g, t)
        assert r["llh_rel_max"] == r["reference_llh_rel_max"] < llh_bound
        assert r["sllh_rel_to_max"] == r["reference_sllh_rel_to_max"] < 1e-4
        assert bench.gradient_error_report(t["llh"], t["sllh"], g, t)["sllh_rel_to_max"] == 0.0


def test_guarded_report_records_the_exception():
    assert bench._guarded(lambda: {"ok": 1}) == {"ok": 1}
    r = bench._guarded(lambda: np.load("/nonexistent.npz"))
    assert set(r) == {"unavailable"} and "FileNotFoundError" in r["unavailable"]
