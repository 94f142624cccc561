"""Small, self-contained cases of the sensitivity kernels for profiler captures.

A capture with many passes (``ncu --set full``) replays each launch dozens of
times, so it wants a case that ends in about a second: a few conditions and a
few outputs of a benchmark workload.  Each case times its calls with CUDA
events and prints one line per call.

    python -m amici_gb300.profile_case adjoint --n 16 --nt 10 --lu 32 --ck 50
    python -m amici_gb300.profile_case large --n 32 --lu 32
    python -m amici_gb300.profile_case fsa --n 512 --lu 32

``adjoint``: the n = 100 adjoint workload (first ``n`` conditions, first
``nt`` outputs, synthetic measurements 0.5 + 0.1 N(0, 1) from
``default_rng(5)``); ``large``: the n = 200 large-batch workload (first
``n`` instances, data from the engine at the true parameters plus noise);
``fsa``: the n = 50 forward-sensitivity workload (first ``n`` instances,
synthetic measurements 0.5 + 0.05 N(0, 1) from ``default_rng(3)``).
One warm-up call, then ``--reps`` timed calls.
"""
from __future__ import annotations

import argparse

import numpy as np


def _solver(ag, w, lu, ck, maxsteps=10000):
    s = ag.Solver()
    s.set_relative_tolerance(w.rtol)
    s.set_absolute_tolerance(w.atol)
    s.set_lu_precision(lu)
    s.set_control_precision(lu)
    s.set_checkpoint_steps(ck)
    s.set_max_steps(maxsteps)
    return s


def main(argv=None):
    import torch

    import amici_gb300 as ag
    from amici_gb300.networks import net50_fsa_workload, net100_adjoint_workload, net200_workload

    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("case", choices=["adjoint", "large", "fsa"])
    ap.add_argument("--n", type=int, default=16)
    ap.add_argument("--nt", type=int, default=0, help="first nt outputs (0: all)")
    ap.add_argument("--lu", type=int, default=32)
    ap.add_argument("--ck", type=int, default=50)
    ap.add_argument("--reps", type=int, default=1)
    a = ap.parse_args(argv)
    method = ag.SensitivityMethod.forward if a.case == "fsa" else ag.SensitivityMethod.adjoint
    if a.case == "fsa":
        w = net50_fsa_workload(a.n)
        nt = a.nt or w.ts.shape[1]
        w.ts = w.ts[:, :nt]
        my = 0.5 + 0.05 * np.random.default_rng(3).normal(size=(a.n, nt, w.model.ny))
        m = ag.Model(w.model)
    elif a.case == "adjoint":
        w = net100_adjoint_workload(a.n)
        nt = a.nt or w.ts.shape[1]
        w.ts = w.ts[:, :nt]
        my = 0.5 + 0.1 * np.random.default_rng(5).normal(size=(a.n, nt, w.model.ny))
        m = ag.Model(w.model)
    else:
        w = net200_workload(a.n)
        nt = a.nt or w.ts.shape[1]
        w.ts = w.ts[:, :nt]
        m = ag.Model(w.model)
        m.set_parameter_scale(w.pscale)
        y = ag.simulate_batch(m, _solver(ag, w, 64, a.ck, 100000), w.theta_true[None, :], np.zeros((1, 0)),
                              w.ts[:1], pscale=w.pscale)["y"]
        my = np.broadcast_to(y + np.random.default_rng(105).normal(0.0, 0.1, y.shape),
                             (a.n,) + y.shape[1:]).copy()
    m.set_parameter_scale(w.pscale)
    s = _solver(ag, w, a.lu, a.ck)
    theta = torch.tensor(w.p, device="cuda")
    ag.log_likelihood_and_gradient(m, s, theta, w.k, w.ts, my, method=method)  # warm-up (module load)
    torch.cuda.synchronize()
    for _ in range(a.reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        llh, sllh, st = ag.log_likelihood_and_gradient(m, s, theta, w.k, w.ts, my, method=method)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        print(f"{a.case} ck{a.ck} lu{a.lu} n={a.n} nt={nt}: {ms:.1f} ms -> {a.n / ms * 1e3:.2f} gradients/s; "
              f"failed {(st != 0).sum().item()}", flush=True)


if __name__ == "__main__":
    main()
