"""The CPU oracle against golden vectors from the reference's own CVODES."""
import platform
from pathlib import Path

import numpy as np
import pytest

from amici_gb300.networks import net20_workload, robertson_workload
from oracle.pyoracle import Oracle, reference_available

GOLD = Path(__file__).resolve().parent / "golden"
X86 = platform.machine() in ("x86_64", "AMD64")


def _load(name):
    return dict(np.load(GOLD / f"{name}.npz"))


def _close(a, b, rtol, atol):
    return np.all(np.abs(a - b) <= atol + rtol * np.abs(b))


@pytest.mark.parametrize("tag", ["robertson_fsa", "robertson_fsa_tight"])
def test_robertson_fsa_matches_reference(tag):
    g = _load(tag)
    w = robertson_workload()
    r = Oracle(w.model).run(g["p"], g["pscale"], np.zeros((1, 0)), g["ts"], g["my"],
                            rtol=float(g["rtol"]), atol=float(g["atol"]), sensi=1)
    assert r["status"][0] == 0
    if X86:  # same operations, same libm: the restatement reproduces CVODES bit for bit
        for key in ("x", "sx", "y", "sy", "llh", "sllh"):
            np.testing.assert_array_equal(r[key], g[key], err_msg=key)
        np.testing.assert_array_equal(r["numsteps"], g["numsteps"])
    else:
        for key in ("x", "sx", "llh", "sllh"):
            assert _close(r[key], g[key], 1e-6, 1e-12), key


@pytest.mark.parametrize("tag", ["net20_fwd", "net20_fwd_tight"])
def test_net20_matches_reference(tag):
    g = _load(tag)
    w = net20_workload(1024)
    r = Oracle(w.model).run(g["p"], g["pscale"], np.zeros((len(g["p"]), 0)), g["ts"],
                            rtol=float(g["rtol"]), atol=float(g["atol"]), maxsteps=100000,
                            nthreads=0)
    assert (r["status"] == 0).all()
    if X86:
        np.testing.assert_array_equal(r["x"], g["x"])
        np.testing.assert_array_equal(r["numsteps"], g["numsteps"])
    else:
        assert _close(r["x"], g["x"], 1e-5, 1e-9)


def test_golden_self_consistency():
    """Robertson conserves x1+x2+x3 = 1.  The reference at the stated
    tolerances meets the accuracy targets against its own 1e-12 run:
    llh within 1e-6 relative, sllh within 1e-4 relative.  States carry the
    global error of a local-error-controlled method (tens of tolerance units)."""
    a, b = _load("robertson_fsa"), _load("robertson_fsa_tight")
    np.testing.assert_allclose(a["x"].sum(-1), 1.0, atol=1e-9)
    assert abs(a["llh"][0] - b["llh"][0]) <= 1e-6 * abs(b["llh"][0])
    assert np.all(np.abs(a["sllh"] - b["sllh"]) <= 1e-4 * np.abs(b["sllh"]))
    assert _close(a["x"], b["x"], 100 * 1e-8, 100 * 1e-12)


@pytest.mark.skipif(not reference_available(), reason="reference sources not present")
def test_port_vs_live_reference_with_failure():
    """maxsteps exhaustion: the restated integrator fails at the same output
    with the same status as the reference."""
    w = robertson_workload()
    kw = dict(rtol=1e-8, atol=1e-12, sensi=0, maxsteps=300)
    a = Oracle(w.model).run(w.p, w.pscale, w.k, w.ts, **kw)
    b = Oracle(w.model, ref=True).run(w.p, w.pscale, w.k, w.ts, **kw)
    assert a["status"][0] == b["status"][0] == -1
    np.testing.assert_array_equal(np.isnan(a["x"]), np.isnan(b["x"]))
    np.testing.assert_array_equal(a["x"][~np.isnan(a["x"])], b["x"][~np.isnan(b["x"])])


@pytest.mark.parametrize("tag,frac_min,max_dev", [("robertson_fsa", 0.85, 100.0), ("net20_fwd", 0.95, 400.0)])
def test_reference_perturbation_envelope(tag, frac_min, max_dev):
    """The reference's own sensitivity to a few-ulp perturbation of its inputs:
    the envelope inside which the GPU parity tests assert agreement."""
    g = _load(tag)
    spec = robertson_workload().model if tag.startswith("rob") else net20_workload(1024).model
    n = len(g["p"])
    atol = float(g["atol"])
    r = Oracle(spec).run(g["p"] * (1 + 1e-15), g["pscale"], np.zeros((n, 0)), g["ts"],
                         rtol=float(g["rtol"]), atol=atol, nthreads=0)
    e = np.abs(r["x"] - g["x"]) / (float(g["rtol"]) * np.abs(g["x"]) + atol)
    assert e.max() > 10  # a few ulps already move outputs by more than 10 tolerance units
    assert np.mean(e <= 10) >= frac_min and e.max() <= max_dev


@pytest.mark.parametrize("tag", ["net50_fsa"])
def test_net50_fsa_matches_reference(tag):
    """Eight instances of the n=50 workload: 100 staggered forward sensitivities on the n=50 network."""
    from amici_gb300.networks import net50_fsa_workload
    g = _load(tag)
    spec = net50_fsa_workload(1).model
    r = Oracle(spec).run(g["p"], g["pscale"], np.zeros((len(g["p"]), 0)), g["ts"], g["my"],
                         rtol=float(g["rtol"]), atol=float(g["atol"]), sensi=1, maxsteps=100000,
                         nthreads=0)
    assert (r["status"] == 0).all()
    if X86:
        np.testing.assert_array_equal(r["x"], g["x"])
        np.testing.assert_array_equal(r["sllh"], g["sllh"])
        np.testing.assert_array_equal(r["numsteps"], g["numsteps"])
    else:
        np.testing.assert_allclose(r["llh"], g["llh"], rtol=1e-6)


# ---- adjoint sensitivities -------------------------------------------------
def _asa_spec(tag):
    from amici_gb300.networks import net100_adjoint_workload, net200_workload
    if tag.startswith("robertson"):
        return robertson_workload().model
    if tag.startswith("net200"):
        return net200_workload(1).model
    if tag.startswith("net20"):
        return net20_workload(16).model
    return net100_adjoint_workload(1).model


@pytest.mark.parametrize("tag", ["robertson_asa", "robertson_asa_tight", "net20_asa", "net100_asa",
                                 "net200_asa"])
def test_asa_matches_reference(tag):
    """The restated backward problem (AMICI's loop over outputs with an adjoint
    reinitialisation after every jump, CVODES' backward BDF with quadratures
    and polynomial interpolation of the stored forward steps) against the
    reference's own CVODES adjoint module on the same inputs."""
    g = _load(tag)
    n = len(g["p"])
    k = g["k"] if "k" in g else np.zeros((n, 0))
    r = Oracle(_asa_spec(tag)).run_asa(g["p"], g["pscale"], k, g["ts"], g["my"],
                                       rtol=float(g["rtol"]), atol=float(g["atol"]),
                                       maxsteps=100000, nthreads=0)
    assert (r["status"] == 0).all()
    if X86:
        np.testing.assert_array_equal(r["llh"], g["llh"])
        np.testing.assert_array_equal(r["sllh"], g["sllh"])
        np.testing.assert_array_equal(r["nst_b"], g["nst_b"])
        np.testing.assert_array_equal(r["numsteps"], g["numsteps"])
    else:
        np.testing.assert_allclose(r["llh"], g["llh"], rtol=1e-6)
        scale = np.abs(g["sllh"]).max(axis=1, keepdims=True)
        assert np.all(np.abs(r["sllh"] - g["sllh"]) <= 1e-4 * scale)


def test_asa_agrees_with_fsa_and_finite_differences():
    """Three independent gradients of the same llh (the reference's own test
    identity, python/tests/util.py:88-140): adjoint, forward sensitivities and
    central finite differences (h = 1e-5 in ln k) on Robertson."""
    g = _load("robertson_asa_tight")
    w = robertson_workload()
    o = Oracle(w.model)
    kw = dict(rtol=1e-12, atol=1e-12, maxsteps=100000)
    asa = o.run_asa(g["p"], g["pscale"], w.k, g["ts"], g["my"], **kw)["sllh"][0]
    fsa = o.run(g["p"], g["pscale"], w.k, g["ts"], g["my"], sensi=1, **kw)["sllh"][0]
    h = 1e-5
    fd = np.empty(3)
    for j in range(3):
        pp, pm = g["p"].copy(), g["p"].copy()
        pp[0, j] += h
        pm[0, j] -= h
        lp = o.run(pp, g["pscale"], w.k, g["ts"], g["my"], **kw)["llh"][0]
        lm = o.run(pm, g["pscale"], w.k, g["ts"], g["my"], **kw)["llh"][0]
        fd[j] = (lp - lm) / (2 * h)
    np.testing.assert_allclose(asa, fsa, rtol=1e-5)
    np.testing.assert_allclose(asa, fd, rtol=1e-4)


@pytest.mark.skipif(not reference_available(), reason="reference sources not present")
def test_asa_port_vs_live_reference_backward_budget():
    """A backward step budget too small to reach t0: both fail the same way
    (AMICI_ERROR from the exhausted budget) and report NaN gradients."""
    g = _load("robertson_asa")
    w = robertson_workload()
    kw = dict(rtol=1e-8, atol=1e-12, maxsteps=100000, maxsteps_b=500)
    a = Oracle(w.model).run_asa(g["p"], g["pscale"], w.k, g["ts"], g["my"], **kw)
    b = Oracle(w.model, ref=True).run_asa(g["p"], g["pscale"], w.k, g["ts"], g["my"], **kw)
    assert a["status"][0] == b["status"][0] != 0
    assert np.isnan(a["sllh"]).all() and np.isnan(b["sllh"]).all()


# ---- pre-equilibration and initial-state overrides -------------------------
@pytest.mark.parametrize("tag", ["preeq_fsa", "preeq_fsa_tight"])
def test_preeq_matches_reference(tag):
    """Simulation to steady state at the pre-equilibration's fixed parameters
    (forward sensitivities; the adjoint with its forward-sensitivity
    pre-equilibration), then the main simulation from x_ss / sx_ss; and the
    same instances started from given x0 / sx0: the restatement against the
    reference's CVODES driven by the same glue."""
    from amici_gb300.networks import preeq_workload
    g = _load(tag)
    spec = preeq_workload(1).model
    kw = dict(rtol=float(g["rtol"]), atol=float(g["atol"]), maxsteps=100000, nthreads=0)
    o = Oracle(spec)
    r = o.run(g["p"], g["pscale"], g["k"], g["ts"], g["my"], sensi=1, k_preeq=g["k_preeq"], **kw)
    a = o.run_asa(g["p"], g["pscale"], g["k"], g["ts"], g["my"], k_preeq=g["k_preeq"], **kw)
    v = o.run(g["p"], g["pscale"], g["k"], g["ts"], g["my"], sensi=1, x0=g["ov_x0"], sx0=g["ov_sx0"], **kw)
    assert (r["status"] == 0).all() and (r["preeq_status"] == 1).all() and (a["status"] == 0).all()
    if X86:
        for key in ("x", "llh", "sllh", "numsteps", "x_ss", "sx_ss", "preeq_numsteps", "preeq_t", "preeq_wrms"):
            np.testing.assert_array_equal(r[key], g[key], err_msg=key)
        np.testing.assert_array_equal(r["sx"][:, -1], g["sx_last"])
        np.testing.assert_array_equal(a["llh"], g["asa_llh"])
        np.testing.assert_array_equal(a["sllh"], g["asa_sllh"])
        np.testing.assert_array_equal(a["nst_b"], g["asa_nst_b"])
        for key in ("x", "llh", "sllh", "numsteps"):
            np.testing.assert_array_equal(v[key], g["ov_" + key], err_msg="override " + key)
    else:
        assert _close(r["x_ss"], g["x_ss"], 1e-5, 1e-9) and _close(r["llh"], g["llh"], 1e-6, 0)


def test_preeq_gradient_identities():
    """With pre-equilibration the forward-sensitivity and adjoint gradients
    agree (sx_ss enters the adjoint through sx0), and both match central
    finite differences of llh through the steady state."""
    g = _load("preeq_fsa_tight")
    np.testing.assert_allclose(g["asa_sllh"], g["sllh"], rtol=0,
                               atol=1e-8 * np.abs(g["sllh"]).max())
    from amici_gb300.networks import preeq_workload
    spec = preeq_workload(1).model
    o = Oracle(spec)
    i, h = 3, 1e-6
    args = lambda p: (p, g["pscale"], g["k"][i:i + 1], g["ts"][i:i + 1], g["my"][i:i + 1])
    kw = dict(rtol=1e-12, atol=1e-12, maxsteps=100000, k_preeq=g["k_preeq"][i:i + 1])
    fd = []
    for j in range(spec.np):
        pp, pm = g["p"][i:i + 1].copy(), g["p"][i:i + 1].copy()
        pp[0, j] += h
        pm[0, j] -= h
        fd.append((o.run(*args(pp), **kw)["llh"][0] - o.run(*args(pm), **kw)["llh"][0]) / (2 * h))
    assert np.max(np.abs(np.array(fd) - g["sllh"][i])) <= 1e-4 * np.abs(g["sllh"][i]).max()


# ---- observation model: nonlinear observables, noise distributions --------
@pytest.mark.parametrize("tag", ["obs6", "obs6_tight"])
def test_observation_model_matches_reference(tag):
    """Nonlinear and parameter-dependent observables, parameter-dependent
    noise scales and the six noise distributions (forward sensitivities and
    adjoint): the restatement against the reference's CVODES driven by the
    same glue."""
    from amici_gb300.networks import obs_workload
    g = _load(tag)
    spec = obs_workload(1).model
    kw = dict(rtol=float(g["rtol"]), atol=float(g["atol"]), maxsteps=100000, nthreads=0)
    o = Oracle(spec)
    k0 = np.zeros((len(g["p"]), 0))
    r = o.run(g["p"], g["pscale"], k0, g["ts"], g["my"], sensi=1, **kw)
    a = o.run_asa(g["p"], g["pscale"], k0, g["ts"], g["my"], **kw)
    if X86:
        for key in ("x", "y", "llh", "sllh", "numsteps"):
            np.testing.assert_array_equal(r[key], g[key], err_msg=key)
        np.testing.assert_array_equal(r["sy"][:, -1], g["sy_last"])
        np.testing.assert_array_equal(a["llh"], g["asa_llh"])
        np.testing.assert_array_equal(a["sllh"], g["asa_sllh"])
    else:
        assert _close(r["llh"], g["llh"], 1e-6, 0)


def test_observation_model_gradient_identities():
    """Forward-sensitivity and adjoint gradients agree, the noise-scale,
    scale and offset parameters included (their gradients are the direct
    objective terms dJy/dsigma dsigma/dp and dJy/dy dy/dp)."""
    g = _load("obs6_tight")
    np.testing.assert_allclose(g["asa_sllh"], g["sllh"], rtol=0, atol=1e-8 * np.abs(g["sllh"]).max())
    assert np.all(np.abs(g["sllh"][:, 10:]) > 1e-3)  # the observation parameters have gradients


# ---- general kinetics: Michaelis-Menten, Hill and inhibition rate laws ----
@pytest.mark.parametrize("tag", ["mapk9", "mapk9_tight"])
def test_general_kinetics_matches_reference(tag):
    """The MAPK cascade (general rate laws): the restatement against the
    reference's CVODES, forward sensitivities and adjoint, bit for bit on
    x86."""
    from amici_gb300.networks import mapk_model
    g = _load(tag)
    kw = dict(rtol=float(g["rtol"]), atol=float(g["atol"]), maxsteps=100000, nthreads=0)
    o = Oracle(mapk_model())
    r = o.run(g["p"], g["pscale"], g["k"], g["ts"], g["my"], sensi=1, **kw)
    a = o.run_asa(g["p"], g["pscale"], g["k"], g["ts"], g["my"], **kw)
    if X86:
        for key in ("x", "y", "llh", "sllh", "numsteps"):
            np.testing.assert_array_equal(r[key], g[key], err_msg=key)
        np.testing.assert_array_equal(r["sx"][:, -1], g["sx_last"])
        np.testing.assert_array_equal(a["llh"], g["asa_llh"])
        np.testing.assert_array_equal(a["sllh"], g["asa_sllh"])
        np.testing.assert_array_equal(a["nst_b"], g["asa_nst_b"])
        f = o.run(g["p"], g["pscale"], g["k"], g["ts"], g["my"], sensi=0, **kw)
        np.testing.assert_array_equal(f["x"], g["fwd_x"])
        np.testing.assert_array_equal(f["numsteps"], g["fwd_numsteps"])
    else:
        assert _close(r["llh"], g["llh"], 1e-6, 0)


def test_general_kinetics_gradient_identities():
    """Forward-sensitivity and adjoint gradients of the MAPK cascade agree at
    rtol = atol = 1e-12, and agree with central finite differences of the
    1e-12 log-likelihood for the first instance."""
    from amici_gb300.networks import mapk_model
    g = _load("mapk9_tight")
    np.testing.assert_allclose(g["asa_sllh"], g["sllh"], rtol=0, atol=1e-7 * np.abs(g["sllh"]).max())
    o = Oracle(mapk_model())
    kw = dict(rtol=1e-12, atol=1e-12, maxsteps=100000, nthreads=0)
    i, h = 0, 1e-5
    P = np.repeat(g["p"][i:i + 1], 2 * g["p"].shape[1], axis=0)
    for j in range(g["p"].shape[1]):
        P[2 * j, j] += h
        P[2 * j + 1, j] -= h
    n = len(P)
    r = o.run(P, g["pscale"], np.repeat(g["k"][i:i + 1], n, 0), np.repeat(g["ts"][i:i + 1], n, 0),
              np.repeat(g["my"][i:i + 1], n, 0), **kw)
    fd = (r["llh"][0::2] - r["llh"][1::2]) / (2 * h)
    np.testing.assert_allclose(fd, g["sllh"][i], rtol=0, atol=2e-5 * np.abs(g["sllh"][i]).max())


# ---- events with explicit trigger times -------------------------------------
@pytest.mark.parametrize("tag", ["dose4", "dose4_tight"])
def test_events_match_reference(tag):
    """Two doses (one at a parameter-dependent time) and a washout at a
    condition-specific time: the restatement of AMICI's event handling and
    solver reinitialisation, driving the restated integrator, against the
    same event handling driving the reference's CVODES; forward simulation
    and forward sensitivities, bit for bit on x86."""
    from amici_gb300.networks import dosing_model
    g = _load(tag)
    kw = dict(rtol=float(g["rtol"]), atol=float(g["atol"]), maxsteps=100000, nthreads=0)
    o = Oracle(dosing_model())
    r = o.run(g["p"], g["pscale"], g["k"], g["ts"], g["my"], sensi=1, **kw)
    f = o.run(g["p"], g["pscale"], g["k"], g["ts"], g["my"], sensi=0, **kw)
    if X86:
        for key in ("x", "y", "sx", "llh", "sllh", "numsteps"):
            np.testing.assert_array_equal(r[key], g[key], err_msg=key)
        np.testing.assert_array_equal(f["x"], g["fwd_x"])
        np.testing.assert_array_equal(f["numsteps"], g["fwd_numsteps"])
    else:
        assert _close(r["llh"], g["llh"], 1e-6, 0)


def test_event_sensitivities_match_finite_differences():
    """The sensitivity jumps at the events (the event-time sensitivity of the
    parameter-dependent dose time included) against central finite
    differences of the 1e-12 states, for every parameter."""
    from amici_gb300.networks import dosing_model
    g = _load("dose4_tight")
    o = Oracle(dosing_model())
    kw = dict(rtol=1e-12, atol=1e-12, maxsteps=200000, nthreads=0)
    i, h, npar = 0, 1e-4, g["p"].shape[1]
    P = np.repeat(g["p"][i:i + 1], 2 * npar, axis=0)
    for j in range(npar):
        P[2 * j, j] += h
        P[2 * j + 1, j] -= h
    n = len(P)
    f = o.run(P, g["pscale"], np.repeat(g["k"][i:i + 1], n, 0), np.repeat(g["ts"][i:i + 1], n, 0), **kw)
    fd = ((f["x"][0::2] - f["x"][1::2]) / (2 * h)).transpose(1, 0, 2)  # [nt, np, nx]
    sx = g["sx"][i]
    assert np.abs(fd - sx).max() <= 1e-6 * np.abs(sx).max()
    # the second dose's time (parameter 10) moves the states
    assert np.abs(sx[:, 10]).max() > 1e-2 * np.abs(sx).max()


def test_events_refused_where_not_restated():
    """Pre-equilibration and adjoint sensitivities of a model with events are
    refused (status -99, NaN outputs)."""
    from amici_gb300.networks import dosing_model
    g = _load("dose4")
    o = Oracle(dosing_model())
    kw = dict(rtol=float(g["rtol"]), atol=float(g["atol"]), maxsteps=100000, nthreads=0)
    a = o.run_asa(g["p"][:2], g["pscale"], g["k"][:2], g["ts"][:2], g["my"][:2], **kw)
    assert (a["status"] == -99).all() and np.isnan(a["llh"]).all()
    r = o.run(g["p"][:2], g["pscale"], g["k"][:2], g["ts"][:2], g["my"][:2], k_preeq=g["k"][:2], **kw)
    assert (r["status"] == -99).all()


# ---- events with trigger functions (root finding) ---------------------------
@pytest.mark.parametrize("tag", ["fire3", "fire3_tight"])
def test_root_finding_events_match_reference(tag):
    """An integrate-and-fire unit: the restatement of CVODES' root finding
    (cvRcheck1-3, cvRootfind) and of AMICI's event handling (roots_found,
    boluses, event-time sensitivities of a state trigger, secondary events,
    reinitialisation) against the reference's CVODES with CVodeRootInit
    driven by the same event handling; bit for bit on x86."""
    from amici_gb300.networks import fire_model
    g = _load(tag)
    kw = dict(rtol=float(g["rtol"]), atol=float(g["atol"]), maxsteps=500000, nthreads=0)
    o = Oracle(fire_model())
    r = o.run(g["p"], g["pscale"], g["k"], g["ts"], g["my"], sensi=1, **kw)
    f = o.run(g["p"], g["pscale"], g["k"], g["ts"], g["my"], sensi=0, **kw)
    assert (g["x"][:, -1, 1] >= 7).all()  # at least seven threshold crossings per instance
    if X86:
        for key in ("x", "y", "sx", "llh", "sllh", "numsteps"):
            np.testing.assert_array_equal(r[key], g[key], err_msg=key)
        np.testing.assert_array_equal(f["x"], g["fwd_x"])
        np.testing.assert_array_equal(f["numsteps"], g["fwd_numsteps"])
    else:
        assert _close(r["llh"], g["llh"], 1e-6, 0)


def test_root_finding_event_sensitivities_match_finite_differences():
    """Sensitivities across the threshold crossings (event-time sensitivity
    from the trigger's derivatives, reset and adaptation boluses) against
    central finite differences of the 1e-12 states."""
    from amici_gb300.networks import fire_model
    g = _load("fire3_tight")
    o = Oracle(fire_model())
    kw = dict(rtol=1e-12, atol=1e-12, maxsteps=500000, nthreads=0)
    i, h, npar = 0, 1e-5, g["p"].shape[1]
    P = np.repeat(g["p"][i:i + 1], 2 * npar, axis=0)
    for j in range(npar):
        P[2 * j, j] += h
        P[2 * j + 1, j] -= h
    n = len(P)
    f = o.run(P, g["pscale"], np.zeros((n, 0)), np.repeat(g["ts"][i:i + 1], n, 0), **kw)
    fd = ((f["x"][0::2] - f["x"][1::2]) / (2 * h)).transpose(1, 0, 2)
    sx = g["sx"][i]
    for j in range(npar - 1):  # the last parameter is a noise scale
        assert np.abs(fd[:, j] - sx[:, j]).max() <= 2e-5 * np.abs(sx[:, j]).max(), j


# ---- post-equilibration: outputs at t = inf --------------------------------
@pytest.mark.parametrize("tag", ["posteq", "posteq_tight"])
def test_posteq_matches_reference(tag):
    """After the last finite output the main solver continues in ONE_STEP
    mode to steady state and the outputs at t = inf are taken there: the
    restatement against the reference's CVODES driven by the same glue,
    forward simulation and forward sensitivities."""
    from amici_gb300.networks import preeq_model
    g = _load(tag)
    o = Oracle(preeq_model())
    kw = dict(rtol=float(g["rtol"]), atol=float(g["atol"]), maxsteps=100000, nthreads=0, k_preeq=g["k_preeq"])
    r = o.run(g["p"], g["pscale"], g["k"], g["ts"], g["my"], sensi=1, **kw)
    f = o.run(g["p"], g["pscale"], g["k"], g["ts"], g["my"], sensi=0, **kw)
    assert (r["status"] == 0).all() and (r["posteq_status"] == 1).all() and (f["posteq_status"] == 1).all()
    assert (r["numsteps"][:, -2:] == 0).all() and (r["posteq_numsteps"] > 0).all()
    np.testing.assert_array_equal(r["x"][:, -1], r["x"][:, -2])
    if X86:
        for key in ("x", "llh", "sllh", "numsteps", "posteq_status", "posteq_numsteps", "posteq_t", "posteq_wrms"):
            np.testing.assert_array_equal(r[key], g[key], err_msg=key)
        np.testing.assert_array_equal(r["sx"][:, -1], g["sx_last"])
        for key in ("x", "llh", "numsteps", "posteq_numsteps", "posteq_t"):
            np.testing.assert_array_equal(f[key], g["fwd_" + key], err_msg="forward " + key)
    else:
        assert _close(r["x"], g["x"], 1e-5, 1e-9) and _close(r["llh"], g["llh"], 1e-6, 0)


def test_posteq_sensitivities_match_finite_differences():
    """The steady-state sensitivities at t = inf (integrated along to the
    steady state) and sllh against central finite differences."""
    from amici_gb300.networks import preeq_model
    g = _load("posteq_tight")
    o = Oracle(preeq_model())
    i, h = 2, 1e-6
    args = lambda p: (p, g["pscale"], g["k"][i:i + 1], g["ts"][i:i + 1], g["my"][i:i + 1])
    kw = dict(rtol=1e-12, atol=1e-12, maxsteps=100000, k_preeq=g["k_preeq"][i:i + 1])
    fd, fdx = [], []
    for j in range(g["p"].shape[1]):
        pp, pm = g["p"][i:i + 1].copy(), g["p"][i:i + 1].copy()
        pp[0, j] += h
        pm[0, j] -= h
        a, b = o.run(*args(pp), **kw), o.run(*args(pm), **kw)
        fd.append((a["llh"][0] - b["llh"][0]) / (2 * h))
        fdx.append((a["x"][0, -1] - b["x"][0, -1]) / (2 * h))
    assert np.max(np.abs(np.array(fd) - g["sllh"][i])) <= 1e-4 * np.abs(g["sllh"][i]).max()
    assert np.max(np.abs(np.array(fdx) - g["sx_last"][i])) <= 1e-4 * np.abs(g["sx_last"][i]).max()


def test_posteq_refused_where_not_restated():
    from amici_gb300.networks import dosing_model, preeq_model
    g = _load("posteq")
    with pytest.raises(NotImplementedError, match="adjoint"):
        Oracle(preeq_model()).run_asa(g["p"][:1], g["pscale"], g["k"][:1], g["ts"][:1], g["my"][:1])
    d = dosing_model()
    with pytest.raises(NotImplementedError, match="events"):
        Oracle(d).run(np.zeros((1, d.np)), np.zeros(d.np, np.int32), np.zeros((1, d.nk)),
                      np.array([[1.0, np.inf]]))


# ---- Heaviside functions in the right-hand side -----------------------------
@pytest.mark.parametrize("tag", ["switch3", "switch3_tight"])
def test_heaviside_matches_reference(tag):
    """Fluxes switched by Heaviside functions of the states: each Heaviside
    becomes an indicator kept by the event handling (root finding on its
    argument and on minus its argument, update_heaviside at every crossing):
    the restatement against the reference's CVODES driven by the same glue."""
    from amici_gb300.networks import switch_model
    g = _load(tag)
    o = Oracle(switch_model())
    kw = dict(rtol=float(g["rtol"]), atol=float(g["atol"]), maxsteps=500000, nthreads=0)
    r = o.run(g["p"], g["pscale"], g["k"], g["ts"], g["my"], sensi=1, **kw)
    f = o.run(g["p"], g["pscale"], g["k"], g["ts"], g["my"], sensi=0, **kw)
    assert (r["status"] == 0).all() and (f["status"] == 0).all()
    if X86:
        for key in ("x", "llh", "sllh", "numsteps", "sx"):
            np.testing.assert_array_equal(r[key], g[key], err_msg=key)
        for key in ("x", "llh", "numsteps"):
            np.testing.assert_array_equal(f[key], g["fwd_" + key], err_msg="forward " + key)
    else:
        assert _close(r["x"], g["x"], 1e-5, 1e-9) and _close(r["llh"], g["llh"], 1e-6, 0)


def test_heaviside_sensitivities_match_finite_differences():
    """Sensitivities across the switches (the event-time sensitivity of each
    crossing times the jump of xdot) against central finite differences of
    the 1e-12 states."""
    from amici_gb300.networks import switch_model
    g = _load("switch3_tight")
    o = Oracle(switch_model())
    kw = dict(rtol=1e-12, atol=1e-12, maxsteps=500000, nthreads=0)
    i, h, npar = 0, 1e-5, g["p"].shape[1]
    P = np.repeat(g["p"][i:i + 1], 2 * npar, axis=0)
    for j in range(npar):
        P[2 * j, j] += h
        P[2 * j + 1, j] -= h
    n = len(P)
    f = o.run(P, g["pscale"], np.zeros((n, 0)), np.repeat(g["ts"][i:i + 1], n, 0), **kw)
    fd = ((f["x"][0::2] - f["x"][1::2]) / (2 * h)).transpose(1, 0, 2)
    sx = g["sx"][i]
    for j in range(npar):
        assert np.abs(fd[:, j] - sx[:, j]).max() <= 2e-5 * np.abs(sx[:, j]).max(), j


def test_heaviside_of_parameters_only_is_refused():
    import sympy as sp
    from amici_gb300.codegen import emit_oracle_c
    from amici_gb300.networks import switch_model
    m = switch_model()
    m.w[1] = m.p[1] * sp.Heaviside(m.p[2] - 0.5)
    with pytest.raises(ValueError, match="explicit trigger time"):
        emit_oracle_c(m)


def test_failed_posteq_keeps_outputs():
    """A model without a steady state (exponential growth): the
    post-equilibration fails (step budget or time overflow), the instance
    gets AMICI_ERROR, and, as in the reference (rdata.cpp:288-313,336-347),
    every output stays in place: the finite outputs, the outputs at t = inf
    from the last state reached, and the llh.  Restatement and reference
    CVODES agree."""
    import sympy as sp
    from amici_gb300.model_spec import ModelSpec
    x, p = sp.symbols("x0:1", real=True), sp.symbols("p0:1", real=True)
    spec = ModelSpec(name="growth1", state_ids=["x"], parameter_ids=["r"], fixed_parameter_ids=[],
                     observable_ids=["x"], x0=[sp.Integer(1)], w=[p[0] * x[0]], stoich={(0, 0): 1}, y=[x[0]],
                     sigma_y=[sp.Float(0.1)], x=list(x), p=list(p), k=[], p_nominal=[0.1], k_nominal=[])
    ts = np.array([[0.5, 1.0, np.inf]])
    my = np.array([[[1.0], [1.1], [2.0]]])
    kw = dict(rtol=1e-8, atol=1e-10, maxsteps=200, nthreads=0)
    r = Oracle(spec).run(np.log([[0.1]]), np.array([1], np.int32), np.zeros((1, 0)), ts, my, **kw)
    assert r["status"][0] == -99 and r["posteq_status"][0] in (-2, -5)
    assert np.isfinite(r["x"][0]).all() and np.isfinite(r["llh"][0])
    assert r["x"][0, 2, 0] > r["x"][0, 1, 0] and r["numsteps"][0, 2] == 0 and np.isnan(r["posteq_t"][0])
    if X86:
        q = Oracle(spec, ref=True).run(np.log([[0.1]]), np.array([1], np.int32), np.zeros((1, 0)), ts, my, **kw)
        for key in ("x", "llh", "status", "posteq_status", "posteq_numsteps"):
            np.testing.assert_array_equal(r[key], q[key], err_msg=key)
