"""Generate the golden vectors of tests/golden/ from the reference's own CVODES.

Runs the reference's vendored CVODES (compiled from the reference sources by
oracle/Makefile.ref, driven like amici::CVodeSolver by
oracle/ref_cvodes_driver.c) on the seeded workloads and stores inputs and
ReturnData outputs as .npz.  Needs the reference tree (AMICI_GB300_REFERENCE,
default /root/reference); the stored fixtures are what the tests read.

    python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from amici_gb300.networks import (dosing_workload, fire_workload, mapk_workload, net20_workload, switch_workload,  # noqa: E402
                                  net50_fsa_workload,
                                  net100_adjoint_workload, net200_workload, obs_workload, preeq_workload,
                                  robertson_workload)
from oracle.pyoracle import Oracle  # noqa: E402


def robertson_data(w, seed=1):
    """m = y(k_true) + N(0, sigma^2) with sigma = 0.01 (numpy default_rng(1))."""
    ref = Oracle(w.model, ref=True)
    r = ref.run(w.p, w.pscale, w.k, w.ts, rtol=1e-12, atol=1e-12, sensi=0)
    rng = np.random.default_rng(seed)
    return r["y"] + rng.normal(0.0, 0.01, r["y"].shape)


def save(name, **arrays):
    np.savez_compressed(HERE / f"{name}.npz", **arrays)
    print("wrote", name, {k: getattr(v, "shape", None) for k, v in arrays.items()})


def main():
    # Robertson, FSA w.r.t. ln k, at the stated tolerances and the 1e-12 oracle
    w = robertson_workload()
    my = robertson_data(w)
    ref = Oracle(w.model, ref=True)
    for tag, rtol, atol in (("robertson_fsa", 1e-8, 1e-12), ("robertson_fsa_tight", 1e-12, 1e-12)):
        r = ref.run(w.p, w.pscale, w.k, w.ts, my, rtol=rtol, atol=atol, sensi=1)
        save(tag, p=w.p, pscale=w.pscale, ts=w.ts, my=my, rtol=rtol, atol=atol,
             **{k: v for k, v in r.items() if v is not None})
    # 64 instances of the n=20 network, no sensitivities
    w2 = net20_workload(1024)
    idx = np.arange(0, 1024, 16)
    ref2 = Oracle(w2.model, ref=True)
    for tag, rtol, atol in (("net20_fwd", w2.rtol, w2.atol), ("net20_fwd_tight", 1e-12, 1e-12)):
        r = ref2.run(w2.p[idx], w2.pscale, w2.k[idx], w2.ts[idx], rtol=rtol, atol=atol,
                     maxsteps=100000)
        save(tag, idx=idx, p=w2.p[idx], pscale=w2.pscale, ts=w2.ts[idx], rtol=rtol, atol=atol,
             x=r["x"], llh=r["llh"], numsteps=r["numsteps"], status=r["status"])


def net50_fsa_golden():
    """Eight instances of the n=50 network with 100 forward
    sensitivities; data from the reference at theta_true (1e-12)."""
    def simulate(m, p, pscale, ts):
        ref = Oracle(m, ref=True)
        return ref.run(p, pscale, np.zeros((len(p), 0)), ts, rtol=1e-12, atol=1e-12, maxsteps=100000,
                       nthreads=0)["y"]
    w = net50_fsa_workload(8, simulate=simulate)
    ref = Oracle(w.model, ref=True)
    for tag, rtol, atol in (("net50_fsa", w.rtol, w.atol), ("net50_fsa_tight", 1e-12, 1e-12)):
        r = ref.run(w.p, w.pscale, w.k, w.ts, w.my, rtol=rtol, atol=atol, sensi=1, maxsteps=100000,
                    nthreads=0)
        save(tag, p=w.p, pscale=w.pscale, ts=w.ts, my=w.my, rtol=rtol, atol=atol, x=r["x"],
             llh=r["llh"], sllh=r["sllh"], sx_last=r["sx"][:, -1], numsteps=r["numsteps"],
             status=r["status"])


def net20_data(w, seed=2):
    """m = y(theta) * (1 + 0.05 N(0, 1)) from the reference at 1e-12 (y = x, sigma = 1)."""
    ref = Oracle(w.model, ref=True)
    r = ref.run(w.p, w.pscale, w.k, w.ts, rtol=1e-12, atol=1e-12, maxsteps=100000, nthreads=0)
    return r["y"] * (1.0 + 0.05 * np.random.default_rng(seed).normal(size=r["y"].shape))


def asa_golden():
    """Adjoint sensitivities (AMICI's backward problem with quadratures) from
    the reference's CVODES: Robertson (its FSA data), 16 instances of the
    n=20 network, and 4 conditions of the n=100 adjoint workload
    with data from the reference at theta_true; at the stated tolerances and
    at rtol = atol = 1e-12."""
    keep = ("x", "llh", "sllh", "numsteps", "status", "nst_b")
    w = robertson_workload()
    my = robertson_data(w)
    ref = Oracle(w.model, ref=True)
    for tag, rtol, atol in (("robertson_asa", 1e-8, 1e-12), ("robertson_asa_tight", 1e-12, 1e-12)):
        r = ref.run_asa(w.p, w.pscale, w.k, w.ts, my, rtol=rtol, atol=atol, maxsteps=100000)
        save(tag, p=w.p, pscale=w.pscale, ts=w.ts, my=my, rtol=rtol, atol=atol,
             **{k: r[k] for k in keep})
    w2 = net20_workload(1024)
    idx = np.arange(0, 1024, 64)
    w2 = w2.subset(idx)
    my2 = net20_data(w2)
    ref2 = Oracle(w2.model, ref=True)
    for tag, rtol, atol in (("net20_asa", 1e-8, 1e-10), ("net20_asa_tight", 1e-12, 1e-12)):
        r = ref2.run_asa(w2.p, w2.pscale, w2.k, w2.ts, my2, rtol=rtol, atol=atol, maxsteps=100000,
                         nthreads=0)
        save(tag, idx=idx, p=w2.p, pscale=w2.pscale, ts=w2.ts, my=my2, rtol=rtol, atol=atol,
             **{k: r[k] for k in keep})

    def simulate(m, p, pscale, k, ts):
        return Oracle(m, ref=True).run(p, pscale, k, ts, rtol=1e-12, atol=1e-12, maxsteps=100000,
                                       nthreads=0)["y"]
    w4 = net100_adjoint_workload(4, simulate=simulate)
    ref4 = Oracle(w4.model, ref=True)
    for tag, rtol, atol in (("net100_asa", w4.rtol, w4.atol), ("net100_asa_tight", 1e-12, 1e-12)):
        r = ref4.run_asa(w4.p, w4.pscale, w4.k, w4.ts, w4.my, rtol=rtol, atol=atol, maxsteps=100000,
                         nthreads=0)
        save(tag, p=w4.p, pscale=w4.pscale, k=w4.k, ts=w4.ts, my=w4.my, rtol=rtol, atol=atol,
             x_last=r["x"][:, -1], **{k: r[k] for k in keep if k != "x"})


def net200_golden():
    """Four instances of the n = 200 large-batch workload (instances 0, 4096,
    8192, 12288 of the 16,384): forward solve plus adjoint llh gradient, data
    from the reference at theta_true (1e-12); at the stated tolerances and at
    rtol = atol = 1e-12."""
    keep = ("llh", "sllh", "numsteps", "status", "nst_b")

    def simulate(m, p, pscale, ts):
        return Oracle(m, ref=True).run(p, pscale, np.zeros((len(p), 0)), ts, rtol=1e-12, atol=1e-12,
                                       maxsteps=1000000, nthreads=0)["y"]
    idx = np.array([0, 4096, 8192, 12288])
    w = net200_workload(16384, simulate=simulate).subset(idx)
    ref = Oracle(w.model, ref=True)
    for tag, rtol, atol in (("net200_asa", w.rtol, w.atol), ("net200_asa_tight", 1e-12, 1e-12)):
        r = ref.run_asa(w.p, w.pscale, w.k, w.ts, w.my, rtol=rtol, atol=atol, maxsteps=1000000,
                        nthreads=0)
        save(tag, idx=idx, p=w.p, pscale=w.pscale, ts=w.ts, my=w.my, rtol=rtol, atol=atol,
             x=r["x"], **{k: r[k] for k in keep})


def preeq_golden():
    """Sixteen instances of the pre-equilibration workload (the preeq12
    network at basal inputs to steady state, then the stimulus response):
    forward sensitivities and adjoint gradients, data from the reference at
    theta_true (1e-12); at the stated tolerances and at rtol = atol = 1e-12.
    Also the same instances started from given initial states and
    sensitivities (ExpData x0 / sx0) without pre-equilibration."""
    def simulate(m, p, pscale, k, ts, k_preeq):
        return Oracle(m, ref=True).run(p, pscale, k, ts, rtol=1e-12, atol=1e-12, maxsteps=100000,
                                       k_preeq=k_preeq, nthreads=0)["y"]
    w = preeq_workload(16, simulate=simulate)
    ref = Oracle(w.model, ref=True)
    keep = ("x", "llh", "sllh", "numsteps", "status", "x_ss", "sx_ss", "preeq_status",
            "preeq_numsteps", "preeq_t", "preeq_wrms")
    x0 = np.abs(np.random.default_rng(61).normal(0.0, 0.2, (16, w.model.nx)))
    sx0 = np.random.default_rng(62).normal(0.0, 0.05, (16, w.model.np, w.model.nx))
    for tag, rtol, atol in (("preeq_fsa", w.rtol, w.atol), ("preeq_fsa_tight", 1e-12, 1e-12)):
        r = ref.run(w.p, w.pscale, w.k, w.ts, w.my, rtol=rtol, atol=atol, sensi=1, maxsteps=100000,
                    k_preeq=w.k_preeq, nthreads=0)
        a = ref.run_asa(w.p, w.pscale, w.k, w.ts, w.my, rtol=rtol, atol=atol, maxsteps=100000,
                        k_preeq=w.k_preeq, nthreads=0)
        o = ref.run(w.p, w.pscale, w.k, w.ts, w.my, rtol=rtol, atol=atol, sensi=1, maxsteps=100000,
                    x0=x0, sx0=sx0, nthreads=0)
        save(tag, p=w.p, pscale=w.pscale, k=w.k, k_preeq=w.k_preeq, ts=w.ts, my=w.my, rtol=rtol, atol=atol,
             **{k: r[k] for k in keep}, sx_last=r["sx"][:, -1], asa_llh=a["llh"], asa_sllh=a["sllh"], asa_status=a["status"],
             asa_nst_b=a["nst_b"], ov_x0=x0, ov_sx0=sx0, ov_x=o["x"], ov_sx_last=o["sx"][:, -1], ov_llh=o["llh"],
             ov_sllh=o["sllh"], ov_numsteps=o["numsteps"])


def posteq_golden():
    """Sixteen instances of the preeq12 network with post-equilibration:
    pre-equilibrated at basal inputs, the stimulus response at ten outputs
    on [0.1, 10^0.5], then two outputs at t = inf (the steady state the
    continued solver reaches); data from the reference at theta_true
    (1e-12).  Forward simulation and forward sensitivities at the stated
    tolerances and at rtol = atol = 1e-12."""
    ts = np.concatenate([np.logspace(-1, 0.5, 10), [np.inf, np.inf]])

    def simulate(m, p, pscale, k, ts_, k_preeq):
        return Oracle(m, ref=True).run(p, pscale, k, ts, rtol=1e-12, atol=1e-12, maxsteps=100000,
                                       k_preeq=k_preeq, nthreads=0)["y"]
    w = preeq_workload(16, seed=16, simulate=simulate)
    ts = np.tile(ts, (16, 1))
    ref = Oracle(w.model, ref=True)
    post = ("posteq_status", "posteq_numsteps", "posteq_t", "posteq_wrms")
    for tag, rtol, atol in (("posteq", w.rtol, w.atol), ("posteq_tight", 1e-12, 1e-12)):
        r = ref.run(w.p, w.pscale, w.k, ts, w.my, rtol=rtol, atol=atol, sensi=1, maxsteps=100000,
                    k_preeq=w.k_preeq, nthreads=0)
        f = ref.run(w.p, w.pscale, w.k, ts, w.my, rtol=rtol, atol=atol, sensi=0, maxsteps=100000,
                    k_preeq=w.k_preeq, nthreads=0)
        save(tag, p=w.p, pscale=w.pscale, k=w.k, k_preeq=w.k_preeq, ts=ts, my=w.my, rtol=rtol, atol=atol,
             x=r["x"], llh=r["llh"], sllh=r["sllh"], sx_last=r["sx"][:, -1], numsteps=r["numsteps"],
             status=r["status"], **{k: r[k] for k in post}, fwd_x=f["x"], fwd_llh=f["llh"],
             fwd_numsteps=f["numsteps"], fwd_status=f["status"], **{"fwd_" + k: f[k] for k in post})


def obs_golden():
    """Sixteen instances of the observation-model workload (nonlinear and
    parameter-dependent observables, parameter-dependent noise scales, the
    six noise distributions): forward-sensitivity and adjoint gradients,
    data from the reference at theta_true (1e-12) with multiplicative noise;
    at the stated tolerances and at rtol = atol = 1e-12."""
    def simulate(m, p, pscale, ts):
        return Oracle(m, ref=True).run(p, pscale, np.zeros((len(p), 0)), ts, rtol=1e-12, atol=1e-12,
                                       maxsteps=100000, nthreads=0)["y"]
    w = obs_workload(16, simulate=simulate)
    ref = Oracle(w.model, ref=True)
    for tag, rtol, atol in (("obs6", w.rtol, w.atol), ("obs6_tight", 1e-12, 1e-12)):
        r = ref.run(w.p, w.pscale, w.k, w.ts, w.my, rtol=rtol, atol=atol, sensi=1, maxsteps=100000, nthreads=0)
        a = ref.run_asa(w.p, w.pscale, w.k, w.ts, w.my, rtol=rtol, atol=atol, maxsteps=100000, nthreads=0)
        save(tag, p=w.p, pscale=w.pscale, ts=w.ts, my=w.my, rtol=rtol, atol=atol, x=r["x"], y=r["y"],
             sy_last=r["sy"][:, -1], llh=r["llh"], sllh=r["sllh"], numsteps=r["numsteps"], status=r["status"],
             asa_llh=a["llh"], asa_sllh=a["sllh"], asa_status=a["status"], asa_nst_b=a["nst_b"])


def mapk_golden():
    """Sixteen instances of the general-kinetics workload (MAPK cascade with
    Michaelis-Menten, Hill and inhibition rate laws): states, observables,
    forward-sensitivity and adjoint gradients, data from the reference at
    theta_nominal (1e-12) with multiplicative noise; at the stated tolerances
    and at rtol = atol = 1e-12."""
    def simulate(m, p, pscale, k, ts):
        return Oracle(m, ref=True).run(p, pscale, k, ts, rtol=1e-12, atol=1e-12, maxsteps=100000,
                                       nthreads=0)["y"]
    w = mapk_workload(16, simulate=simulate)
    ref = Oracle(w.model, ref=True)
    for tag, rtol, atol in (("mapk9", w.rtol, w.atol), ("mapk9_tight", 1e-12, 1e-12)):
        r = ref.run(w.p, w.pscale, w.k, w.ts, w.my, rtol=rtol, atol=atol, sensi=1, maxsteps=100000, nthreads=0)
        a = ref.run_asa(w.p, w.pscale, w.k, w.ts, w.my, rtol=rtol, atol=atol, maxsteps=100000, nthreads=0)
        f = ref.run(w.p, w.pscale, w.k, w.ts, w.my, rtol=rtol, atol=atol, sensi=0, maxsteps=100000, nthreads=0)
        save(tag, p=w.p, pscale=w.pscale, k=w.k, ts=w.ts, my=w.my, rtol=rtol, atol=atol, x=r["x"], y=r["y"],
             fwd_x=f["x"], fwd_llh=f["llh"], fwd_numsteps=f["numsteps"],
             sx_last=r["sx"][:, -1], llh=r["llh"], sllh=r["sllh"], numsteps=r["numsteps"], status=r["status"],
             asa_llh=a["llh"], asa_sllh=a["sllh"], asa_status=a["status"], asa_nst_b=a["nst_b"])


def dosing_golden():
    """Sixteen instances of the event workload (two doses, one at a
    parameter-dependent time, and a washout at a condition-specific time):
    states, observables and forward sensitivities, data from the reference
    at theta_nominal (1e-12) with additive noise; the forward simulation
    without sensitivities beside them; at the stated tolerances and at
    rtol = atol = 1e-12."""
    def simulate(m, p, pscale, k, ts):
        return Oracle(m, ref=True).run(p, pscale, k, ts, rtol=1e-12, atol=1e-12, maxsteps=100000,
                                       nthreads=0)["y"]
    w = dosing_workload(16, simulate=simulate)
    ref = Oracle(w.model, ref=True)
    for tag, rtol, atol in (("dose4", w.rtol, w.atol), ("dose4_tight", 1e-12, 1e-12)):
        r = ref.run(w.p, w.pscale, w.k, w.ts, w.my, rtol=rtol, atol=atol, sensi=1, maxsteps=100000, nthreads=0)
        f = ref.run(w.p, w.pscale, w.k, w.ts, w.my, rtol=rtol, atol=atol, sensi=0, maxsteps=100000, nthreads=0)
        save(tag, p=w.p, pscale=w.pscale, k=w.k, ts=w.ts, my=w.my, rtol=rtol, atol=atol, x=r["x"], y=r["y"],
             sx=r["sx"], llh=r["llh"], sllh=r["sllh"], numsteps=r["numsteps"], status=r["status"],
             fwd_x=f["x"], fwd_llh=f["llh"], fwd_numsteps=f["numsteps"])


def fire_golden():
    """Sixteen instances of the root-finding workload (integrate-and-fire
    unit: a state-dependent trigger located by CVODES' root finding, a reset
    bolus, a counter and an adaptation bolus): states, observables and
    forward sensitivities, data from the reference at theta_nominal (1e-12)
    with additive noise; the forward simulation without sensitivities beside
    them; at the stated tolerances and at rtol = atol = 1e-12."""
    def simulate(m, p, pscale, k, ts):
        return Oracle(m, ref=True).run(p, pscale, k, ts, rtol=1e-12, atol=1e-12, maxsteps=500000,
                                       nthreads=0)["y"]
    w = fire_workload(16, simulate=simulate)
    ref = Oracle(w.model, ref=True)
    for tag, rtol, atol in (("fire3", w.rtol, w.atol), ("fire3_tight", 1e-12, 1e-12)):
        r = ref.run(w.p, w.pscale, w.k, w.ts, w.my, rtol=rtol, atol=atol, sensi=1, maxsteps=500000, nthreads=0)
        f = ref.run(w.p, w.pscale, w.k, w.ts, w.my, rtol=rtol, atol=atol, sensi=0, maxsteps=500000, nthreads=0)
        save(tag, p=w.p, pscale=w.pscale, k=w.k, ts=w.ts, my=w.my, rtol=rtol, atol=atol, x=r["x"], y=r["y"],
             sx=r["sx"], llh=r["llh"], sllh=r["sllh"], numsteps=r["numsteps"], status=r["status"],
             fwd_x=f["x"], fwd_llh=f["llh"], fwd_numsteps=f["numsteps"])


def switch_golden():
    """Sixteen instances of the Heaviside workload (two fluxes switched by
    Heavisides of the states, crossings in both directions located by root
    finding): states, observables and forward sensitivities, data from the
    reference at theta_nominal (1e-12) with additive noise; the forward
    simulation without sensitivities beside them; at the stated tolerances
    and at rtol = atol = 1e-12."""
    def simulate(m, p, pscale, k, ts):
        return Oracle(m, ref=True).run(p, pscale, k, ts, rtol=1e-12, atol=1e-12, maxsteps=500000,
                                       nthreads=0)["y"]
    w = switch_workload(16, simulate=simulate)
    ref = Oracle(w.model, ref=True)
    for tag, rtol, atol in (("switch3", w.rtol, w.atol), ("switch3_tight", 1e-12, 1e-12)):
        r = ref.run(w.p, w.pscale, w.k, w.ts, w.my, rtol=rtol, atol=atol, sensi=1, maxsteps=500000, nthreads=0)
        f = ref.run(w.p, w.pscale, w.k, w.ts, w.my, rtol=rtol, atol=atol, sensi=0, maxsteps=500000, nthreads=0)
        save(tag, p=w.p, pscale=w.pscale, k=w.k, ts=w.ts, my=w.my, rtol=rtol, atol=atol, x=r["x"], y=r["y"],
             sx=r["sx"], llh=r["llh"], sllh=r["sllh"], numsteps=r["numsteps"], status=r["status"],
             fwd_x=f["x"], fwd_llh=f["llh"], fwd_numsteps=f["numsteps"])


def stab_histories():
    """Inputs and results of the restated stability-limit detector (CVODES
    cvSLdet), recorded during forward runs of the n = 20 network (1024
    instances) and the n = 100 adjoint network's forward problem (8
    conditions): up to 400 calls per outcome, for the engine's detector."""
    import ctypes
    recs = []
    for w in (net20_workload(1024), net100_adjoint_workload(8)):
        o = Oracle(w.model)
        buf = np.zeros((400_000, 17))
        o.lib.oracle_record_stability_detector(buf.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                               ctypes.c_int64(len(buf)))
        o.lib.oracle_stability_detector_records.restype = ctypes.c_int64
        o.run(w.p, w.pscale, w.k, w.ts, rtol=w.rtol, atol=w.atol, maxsteps=100000, nthreads=1)
        n = o.lib.oracle_stability_detector_records()
        o.lib.oracle_record_stability_detector(None, ctypes.c_int64(0))
        recs.append(buf[:n].copy())
    r = np.concatenate(recs)
    rng = np.random.default_rng(0)
    keep = []
    for v in np.unique(r[:, 16]):
        idx = np.flatnonzero(r[:, 16] == v)
        keep.append(rng.choice(idx, min(400, len(idx)), replace=False))
    r = r[np.sort(np.concatenate(keep))]
    save("stab_histories", hist=r[:, :15], q=r[:, 15].astype(np.int32), kflag=r[:, 16].astype(np.int32))


if __name__ == "__main__":
    which = sys.argv[1:] or ["main", "net50", "asa", "net200", "preeq", "posteq", "obs", "mapk", "dose", "fire",
                             "switch", "stab"]
    if "main" in which:
        main()
    if "net50" in which:
        net50_fsa_golden()
    if "asa" in which:
        asa_golden()
    if "net200" in which:
        net200_golden()
    if "preeq" in which:
        preeq_golden()
    if "posteq" in which:
        posteq_golden()
    if "obs" in which:
        obs_golden()
    if "mapk" in which:
        mapk_golden()
    if "dose" in which:
        dosing_golden()
    if "fire" in which:
        fire_golden()
    if "switch" in which:
        switch_golden()
    if "stab" in which:
        stab_histories()
