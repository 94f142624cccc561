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

from amici_gb300.networks import config2_workload, config3_workload, robertson_workload  # noqa: E402
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
    # Config 1: Robertson, FSA w.r.t. ln k, at the stated tolerances and the 1e-12 oracle
    w = robertson_workload()
    my = robertson_data(w)
    ref = Oracle(w.model, ref=True)
    for tag, rtol, atol in (("robertson_fsa", 1e-8, 1e-12), ("robertson_fsa_tight", 1e-12, 1e-12)):
        r = ref.run(w.p, w.pscale, w.k, w.ts, my, rtol=rtol, atol=atol, sensi=1)
        save(tag, p=w.p, pscale=w.pscale, ts=w.ts, my=my, rtol=rtol, atol=atol,
             **{k: v for k, v in r.items() if v is not None})
    # Config 2 subset: 64 instances of the n=20 network, no sensitivities
    w2 = config2_workload(1024)
    idx = np.arange(0, 1024, 16)
    ref2 = Oracle(w2.model, ref=True)
    for tag, rtol, atol in (("net20_fwd", w2.rtol, w2.atol), ("net20_fwd_tight", 1e-12, 1e-12)):
        r = ref2.run(w2.p[idx], w2.pscale, w2.k[idx], w2.ts[idx], rtol=rtol, atol=atol,
                     maxsteps=100000)
        save(tag, idx=idx, p=w2.p[idx], pscale=w2.pscale, ts=w2.ts[idx], rtol=rtol, atol=atol,
             x=r["x"], llh=r["llh"], numsteps=r["numsteps"], status=r["status"])


def config3_golden():
    """Config 3 subset: 8 instances of the n=50 network with 100 forward
    sensitivities; data from the reference at theta_true (1e-12)."""
    def simulate(m, p, pscale, ts):
        ref = Oracle(m, ref=True)
        return ref.run(p, pscale, np.zeros((len(p), 0)), ts, rtol=1e-12, atol=1e-12, maxsteps=100000,
                       nthreads=0)["y"]
    w = config3_workload(8, simulate=simulate)
    ref = Oracle(w.model, ref=True)
    for tag, rtol, atol in (("net50_fsa", w.rtol, w.atol), ("net50_fsa_tight", 1e-12, 1e-12)):
        r = ref.run(w.p, w.pscale, w.k, w.ts, w.my, rtol=rtol, atol=atol, sensi=1, maxsteps=100000,
                    nthreads=0)
        save(tag, p=w.p, pscale=w.pscale, ts=w.ts, my=w.my, rtol=rtol, atol=atol, x=r["x"],
             llh=r["llh"], sllh=r["sllh"], sx_last=r["sx"][:, -1], numsteps=r["numsteps"],
             status=r["status"])


if __name__ == "__main__":
    main()
    config3_golden()
