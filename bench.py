#!/usr/bin/env python3
"""Benchmark of AMICI's simulation path on one GB300 (solves/s and
llh-gradients/s on the five seeded configurations).

Headline (C2, net20): seeded random mass-action network, 20 species, 40
reactions (uni- or bimolecular), 1,024 parameter vectors with log10 k ~
U[-3, 3], x0 log-uniform in [1e-2, 1], 50 log-spaced outputs on [1e-3, 1e3],
FP64 states with an FP32 iteration matrix, rtol 1e-8, atol 1e-10, no
sensitivities.  One step = one batched simulation of all 1,024 instances.
  value  device-resident inputs/outputs, one persistent kernel launch per
         step, timed with CUDA events on the launching stream; a 512 MiB
         buffer is written between timed steps to flush the 129 MB L2.
  e2e    the same metric through the host-buffer C entry point (the call
         ``run_simulations`` makes): host->device copies of the inputs from
         pinned memory, the kernel and the device->host copies of every
         output inside the timed region.
Under torchrun each rank simulates its own 1,024 instances (weak scaling,
replicas; nothing is exchanged).  ``--impl reference`` times the CPU
restatement of the reference path (the oracle) on all host cores, the full
1,024-instance batch per step.

The line's ``legs`` object carries the other configurations, each with its
rate, its all-FP64 comparators and its error against the reference at
rtol = atol = 1e-12 on the golden instances (``*_err``, beside the
reference's own at the stated tolerances, ``ref_*_err``):
  C3  llh-gradients/s by staggered forward sensitivities: 50 species, 100
      reactions, 100 log-parameters, 4,096 instances, final times logU[1e1,
      1e4], 30 outputs, 10 observables; mixed precision and all-FP64
      batched; the HBM roofline of the sensitivity history traffic.
  C4  llh-gradients/s by adjoint sensitivities: 100 species, 300 reactions,
      256 log-parameters, 512 conditions, 100 outputs on [0, 500], forward
      check points every 50 steps; mixed precision, every-step storage,
      all-FP64 batched and with one launch per condition (a one-condition
      sample); the same 512 conditions as one Objective evaluation.
  C5  llh-gradients/s (forward solve plus adjoint gradient per instance):
      200 species, 500 reactions, 400 log10-parameters, the first
      ``--large-n`` of 16,384 instances (16384: all), AMICI's default budget
      of 10,000 steps; FP32 and FP64 iteration matrix on the same instances.
Each leg's CPU baseline is the oracle on the machine's host cores on a bounded
sample.  ``--detail PATH`` writes every leg's full report as JSON.

``--case {net20,fsa,adjoint,large}`` runs one small case of a leg for
profiler captures instead (one warm-up call, ``--reps`` timed calls, one
printed line per call): the first ``--n`` instances, first ``--nt``
outputs, iteration matrix precision ``--lu``, check-point spacing ``--ck``.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOAD = ("net20: mass-action network, 20 species, 40 reactions; 1024 parameter vectors; "
            "50 outputs on [1e-3,1e3]; rtol 1e-8, atol 1e-10; forward simulation")
METRIC = "solves/s"
DTYPE = "f64 states, f32 iteration matrix"
# DRAM bytes (read + write) of one forward_kernel launch on this workload, from
# one ncu capture (0.91 MB read, 0.05 MB written)
FWD_TRAFFIC_BYTES = 0.96e6
HBM_FALLBACK_GBS = 6800.0  # the pool's earlier GB300 copy-bandwidth measurement
GOLD = ROOT / "tests" / "golden"


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def workload():
    from amici_gb300.networks import net20_workload
    return net20_workload(1024)


def hbm_peak():
    """(GB/s, source): the measured copy bandwidth of the GB300s."""
    try:
        d = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
        for key in ("hbm_gbs", "hbm_GBs", "hbm"):
            if key in d and float(d[key]) > 0:
                return float(d[key]), "measured"
    except (OSError, ValueError, TypeError):
        pass
    return HBM_FALLBACK_GBS, "fallback"


def _r(x, digits=4):
    """Round to a few significant digits (keeps the line short)."""
    if x is None or isinstance(x, (bool, int, str)):
        return x
    x = float(x)
    if not math.isfinite(x) or x == 0.0:
        return x if math.isfinite(x) else None
    return float(f"{x:.{digits}g}")


# ---------------------------------------------------------------------------
# clocks during the timed region
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.path = tempfile.mktemp(suffix=".csv")
        self.proc = None
        self.gpu = gpu_index

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.strip()]
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            try:
                sm.append(float(r[1]))
                smax = float(r[2])
            except (ValueError, IndexError):
                continue
            for nm, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
def fp64_flops(spec, diag, q_avg=3.0):
    """Algorithmic FP64 work of one launch from the solver counters.

    Per accepted step (n states): predictor q(q+1)/2*n, history update
    2(q+1)*n, error weights and local error test 5n; per Newton iteration:
    residual, correction and convergence norm 10n; per right-hand-side
    evaluation: one multiply per reactant of every flux plus 2*nnz(S)
    (stoichiometry accumulation).  q_avg = 3 (the observed average order).
    """
    n = spec.nx
    mono = spec.flux_monomials()
    c_f = sum((m.a >= 0) + (m.b >= 0) for m in mono) + 2 * len(spec.stoich)
    steps, nfe, nni = diag[:, 0].sum(), diag[:, 1].sum(), diag[:, 2].sum()
    per_step = q_avg * (q_avg + 1) / 2 * n + 2 * (q_avg + 1) * n + 5 * n
    return float(steps * per_step + nni * 10 * n + nfe * c_f)


def fsa_history_bytes(spec, nplist, diag, q_avg=3.0):
    """Algorithmic DRAM bytes of one forward-sensitivity launch: every
    accepted step reads and writes the sensitivity columns' Nordsieck history,
    2 (q+1) n P doubles (q_avg = 3), which exceeds the L2 across the resident
    groups (400 KB per group for n = 50, P = 100)."""
    return float(diag[:, 0].sum()) * 2.0 * (q_avg + 1.0) * spec.nx * nplist * 8.0


def cpu_port_rate(w, seconds=8.0, threads=None):
    """The oracle (CPU restatement of the reference path) on all host cores:
    repeat the full batch until ``seconds`` of wall time have elapsed."""
    from oracle.pyoracle import Oracle
    threads = threads or os.cpu_count() or 1
    o = Oracle(w.model)
    t0 = time.perf_counter()
    solves, reps = 0, 0
    while True:
        o.run(w.p, w.pscale, w.k, w.ts, rtol=w.rtol, atol=w.atol, nthreads=threads)
        solves += w.n
        reps += 1
        el = time.perf_counter() - t0
        if el >= seconds or reps >= 50:
            break
    return solves / el, threads, reps, el


def run_reference(args, rank):
    """The reference arm: the oracle (CPU restatement of the reference's
    path) on all host threads, the full 1,024-instance batch per step."""
    if rank != 0:
        return
    w = workload()
    from oracle.pyoracle import Oracle
    threads = os.cpu_count() or 1
    o = Oracle(w.model)
    for _ in range(args.warmup):
        o.run(w.p, w.pscale, w.k, w.ts, rtol=w.rtol, atol=w.atol, nthreads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.run(w.p, w.pscale, w.k, w.ts, rtol=w.rtol, atol=w.atol, nthreads=threads)
    el = time.perf_counter() - t0
    value = w.n * args.steps / el
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "n_instances": w.n},
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port",
                         "sample": f"full 1024-instance batch per step, {args.steps} steps"},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gb300(args, ws, rank, local):
    import torch

    import amici_gb300 as ag
    from amici_gb300 import _native
    from amici_gb300.build import build_probe_library

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    w = workload()
    spec = w.model
    model = ag.Model(spec)
    model.set_parameter_scale(w.pscale)
    solver = ag.Solver()
    solver.set_relative_tolerance(w.rtol)
    solver.set_absolute_tolerance(w.atol)
    if args.lanes:
        solver.set_lanes_per_instance(args.lanes)
    lib = model.library
    opts = solver.to_options()
    n, nt, nx, ny = w.n, w.ts.shape[1], spec.nx, spec.ny

    # device-resident batch
    T = lambda a, dt=torch.float64: torch.as_tensor(np.ascontiguousarray(a)).to(dev, dt)
    dp, dts, dps = T(w.p), T(w.ts), T(w.pscale, torch.int32)
    dx = torch.empty((n, nt, nx), dtype=torch.float64, device=dev)
    dy = torch.empty((n, nt, ny), dtype=torch.float64, device=dev)
    dsy = torch.empty((n, nt, ny), dtype=torch.float64, device=dev)
    dllh = torch.empty(n, dtype=torch.float64, device=dev)
    dns = torch.empty((n, nt), dtype=torch.int32, device=dev)
    dst = torch.empty(n, dtype=torch.int32, device=dev)
    ddiag = torch.empty((n, 8), dtype=torch.int32, device=dev)
    b = _native.Batch()
    b.n_instances, b.nt, b.nplist = n, nt, 0
    b.p, b.pscale, b.k, b.ts = dp.data_ptr(), dps.data_ptr(), None, dts.data_ptr()
    b.my = b.sigma_y = b.plist = None
    b.x, b.y, b.sigmay, b.llh = dx.data_ptr(), dy.data_ptr(), dsy.data_ptr(), dllh.data_ptr()
    b.sx = b.sy = b.sllh = None
    b.numsteps, b.status, b.diag = dns.data_ptr(), dst.data_ptr(), ddiag.data_ptr()
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def step():
        lib.run_device(opts, b, stream.cuda_stream)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize(dev)
    if ws > 1:
        dist.barrier()
    events = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        torch.cuda.synchronize(dev)
        if ws > 1:
            dist.barrier()
        t_wall = time.perf_counter()
        for e0, e1 in events:
            flush.fill_(1.0)  # L2 flush between timed steps (outside the events)
            e0.record(stream)
            step()
            e1.record(stream)
        torch.cuda.synchronize(dev)
        t_wall = time.perf_counter() - t_wall
    ms = [e0.elapsed_time(e1) for e0, e1 in events]
    ms_step = sum(ms) / len(ms)
    if ws > 1:
        t = torch.tensor([ms_step], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_step = float(t.item())
    status = dst.cpu().numpy()
    diag = ddiag.cpu().numpy()
    value = ws * n / (ms_step * 1e-3)

    # end to end through the host-buffer entry point (the run_simulations path),
    # inputs from pinned host memory, every output copied back
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    hp, hts, hps = pin(w.p), pin(w.ts), pin(w.pscale.astype(np.int32))
    for _ in range(2):
        ag.simulate_batch(model, solver, hp, w.k, hts, pscale=hps)
    torch.cuda.synchronize(dev)
    te = time.perf_counter()
    for _ in range(args.steps):
        r = ag.simulate_batch(model, solver, hp, w.k, hts, pscale=hps)
    torch.cuda.synchronize(dev)
    te = (time.perf_counter() - te) / args.steps
    if ws > 1:
        t = torch.tensor([te], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        te = float(t.item())
    h2d = hp.nbytes + hts.nbytes + hps.nbytes
    d2h = sum(r[k].nbytes for k in ("x", "y", "sigmay", "llh", "numsteps", "status", "diag"))

    # roofline: FP64 issue (CUDA cores) bounds this kernel
    probe = _native_probe(build_probe_library())
    flops = fp64_flops(spec, diag)
    achieved = flops / (ms_step * 1e-3) / 1e9
    launches = args.steps  # one forward_kernel launch per step

    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": ws, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": DTYPE, "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "n_instances": n, "lanes_per_instance": int(opts.lanes_per_instance),
                   "lu_precision": int(opts.lu_precision), "stldet": int(opts.stldet),
                   "parallelism": f"replicas x{ws}", "l2": "512 MiB written between timed steps"},
        "e2e": {"value": ws * n / te, "unit": METRIC, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": probe, "unit": "GFLOP/s",
                     "frac": achieved / probe if probe > 0 else None, "traffic": FWD_TRAFFIC_BYTES,
                     "note": "FP64 CUDA-core bound; peak = live FP64 FMA probe (no FP64 figure among the "
                             "measured peaks); traffic = DRAM bytes of one launch (ncu)"},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    detail = {"headline": {"failed_instances": int((status != 0).sum()),
                           "steps_per_solve": float(diag[:, 0].mean()), "wall_s_timed_loop": t_wall,
                           "error_vs_fp64_oracle_1e-12": _guarded(lambda: state_error_report(
                               r["x"][_gold("net20_fwd")["idx"]], _gold("net20_fwd"), _gold("net20_fwd_tight")))}}
    legs = {"C2": {"v": _r(value), "e2e": _r(ws * n / te), "n": n,
                   "x_tu": _r(detail["headline"]["error_vs_fp64_oracle_1e-12"].get("x_tol_units_max"), 3),
                   "ref_x_tu": _r(detail["headline"]["error_vs_fp64_oracle_1e-12"].get(
                       "reference_x_tol_units_max"), 3)}}
    if rank == 0 and ws == 1 and not args.no_cpu:
        rate, threads, reps, el = cpu_port_rate(w)
        line["cpu_baseline"] = {"value": rate, "unit": METRIC, "cores": threads, "kind": "port",
                                "sample": f"full 1024-instance batch x{reps} ({el:.1f} s), oracle on all host threads"}
        legs["C2"]["cpu"] = _r(rate)
    if rank == 0 and not args.no_grad:
        for key, fn in (("C3", fsa_leg), ("C4", gradients_leg)) + ((("C5", large_leg),) if not args.no_large else ()):
            full, short = fn(args, dev)
            detail[key] = full
            legs[key] = short
    line["legs"] = legs
    if rank == 0 and args.detail:
        Path(args.detail).write_text(json.dumps(detail, indent=1, default=float))
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.barrier()
        dist.destroy_process_group()


def _errs_short(rep):
    """The compact error fields of a gradient error report."""
    if "unavailable" in rep:
        return {"err": rep["unavailable"][:60]}
    return {"llh_err": _r(rep["llh_rel_max"], 2), "sllh_err": _r(rep["sllh_rel_to_max"], 2),
            "ref_llh_err": _r(rep["reference_llh_rel_max"], 2), "ref_sllh_err": _r(rep["reference_sllh_rel_to_max"], 2)}


GRAD_WORKLOAD = ("net100: random mass-action network, 100 species, 300 reactions, 256 log-parameters; "
                 "512 conditions (5 input species scaled by logU[0.1,10]); 8 observables, 100 outputs "
                 "on [0,500], sigma 0.1; rtol 1e-8, atol 1e-10; adjoint llh gradient per condition")


def gradients_leg(args, dev):
    """C4: llh-gradients/s on the adjoint workload (see the module docstring)."""
    import torch

    import amici_gb300 as ag
    from amici_gb300.networks import net100_adjoint_workload
    from oracle.pyoracle import Oracle

    n = 512
    w = net100_adjoint_workload(n)
    spec = w.model
    # synthetic data: the engine's own y at the true parameters plus noise (sigma = 0.1)
    m = ag.Model(spec)
    m.set_parameter_scale(w.pscale)
    s0 = ag.Solver()
    s0.set_relative_tolerance(w.rtol)
    s0.set_absolute_tolerance(w.atol)
    y = ag.simulate_batch(m, s0, w.p, w.k, w.ts, pscale=w.pscale)["y"]
    my = y + np.random.default_rng(104).normal(0.0, 0.1, y.shape)
    theta = torch.tensor(w.p, device=dev)
    k = torch.tensor(w.k, device=dev)
    ts = torch.tensor(w.ts, device=dev)
    myd = torch.tensor(my, device=dev)
    stream = torch.cuda.current_stream(dev)

    def solver(bits, mode=0, ck=50):
        s = ag.Solver()
        s.set_relative_tolerance(w.rtol)
        s.set_absolute_tolerance(w.atol)
        s.set_lu_precision(bits)
        s.set_control_precision(bits)
        s.set_launch_mode(mode)
        s.set_checkpoint_steps(ck)
        return s

    def timed(s, rows, reps):
        out = None
        times = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            out = ag.log_likelihood_and_gradient(m, s, theta[rows], k[rows], ts[rows], myd[rows])
            e1.record(stream)
            torch.cuda.synchronize(dev)
            times.append(e0.elapsed_time(e1) * 1e-3)
        return min(times), out

    allr = slice(0, n)
    timed(solver(32), allr, 1)  # warm-up: module load, allocator, clocks
    t32, (llh32, sllh32, st32) = timed(solver(32), allr, max(1, args.grad_reps))
    t32all, _ = timed(solver(32, ck=0), allr, 1)
    t64, (llh64, sllh64, st64) = timed(solver(64), allr, 1)
    ns = 1  # per-instance launches: a one-condition sample (latency of a single warp)
    t64i, _ = timed(solver(64, 1), slice(0, ns), 1)
    rate32, rate64, rate64i = n / t32, n / t64, ns / t64i
    sl32, sl64 = sllh32.cpu().numpy(), sllh64.cpu().numpy()
    rel = np.abs(sl32 - sl64) / np.abs(sl64).max(axis=1, keepdims=True)
    out = {
        "metric": "llh-gradients/s", "workload": GRAD_WORKLOAD, "n_conditions": n,
        "value": rate32, "unit": "llh-gradients/s", "dtype": "f64 states/adjoint/quadratures, f32 iteration matrix",
        "ms_per_batch": t32 * 1e3,
        "checkpoint_steps": 50, "every_step_storage": n / t32all,
        "fp64_batched": rate64, "fp64_per_instance_launch": rate64i,
        "ratio_vs_fp64_per_instance_launch": rate32 / rate64i, "ratio_vs_fp64_batched": rate32 / rate64,
        "per_instance_sample": f"{ns} condition(s), one launch each, all-FP64",
        "failed": int((st32 != 0).sum().item()),
        "sllh_mixed_vs_fp64_max_rel": float(np.nanmax(rel)),
        "llh_mixed_vs_fp64_max_rel": float(np.nanmax(np.abs(llh32.cpu().numpy() - llh64.cpu().numpy())
                                                     / np.abs(llh64.cpu().numpy()))),
    }

    def gold_errors():
        g, t = _gold("net100_asa"), _gold("net100_asa_tight")
        lg, sg, _ = ag.log_likelihood_and_gradient(m, solver(32), g["p"], g["k"], g["ts"], g["my"])
        return gradient_error_report(lg.cpu().numpy(), sg.cpu().numpy(), g, t)
    out["error_vs_fp64_oracle_1e-12"] = _guarded(gold_errors)

    def objective_eval():
        # the same 512 conditions as one objective over the shared parameters
        # (PEtab-style mapping: every model parameter to the problem parameter
        # of the same id on ln scale, the fixed parameters per condition);
        # timed twice, and the device call it makes timed alone
        pids = list(spec.parameter_ids)
        maps = [ag.ConditionMapping({q: q for q in pids}, {q: "log" for q in pids},
                                    dict(zip(spec.fixed_parameter_ids, map(float, w.k[c])))) for c in range(n)]
        obj = ag.Objective(m, solver(32), pids, ["log"] * len(pids), maps, w.ts, my)
        ts_obj = []
        for _ in range(2):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize(dev)
            w0 = time.perf_counter()
            e0.record(stream)
            r = obj(w.p[0])
            e1.record(stream)
            torch.cuda.synchronize(dev)
            ts_obj.append((e0.elapsed_time(e1) * 1e-3, time.perf_counter() - w0))
        p_map = obj.map_parameters(torch.tensor(w.p[0], device=dev)).detach()
        t_call, _ = 0.0, None
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ag.log_likelihood_and_gradient(m, solver(32), p_map, obj.fixed_parameters(w.p[0]), obj.ts, obj.my)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        t_call = e0.elapsed_time(e1) * 1e-3
        ref = sllh32.cpu().numpy().sum(axis=0)
        return {"s_per_evaluation": ts_obj[-1][0], "s_per_evaluation_first": ts_obj[0][0],
                "wall_s_per_evaluation": ts_obj[-1][1], "device_call_s": t_call, "conditions": n,
                "failed": int((r["status"] != 0).sum()),
                "grad_vs_summed_sllh_max_rel": float(np.max(np.abs(r["sllh"] - ref)) / np.max(np.abs(ref)))
                if r["sllh"] is not None else None}
    out["objective"] = _guarded(objective_eval)
    if not args.no_cpu:
        sample = 32
        threads = os.cpu_count() or 1
        o = Oracle(spec)
        t0 = time.perf_counter()
        o.run_asa(w.p[:sample], w.pscale, w.k[:sample], w.ts[:sample], my[:sample], rtol=w.rtol,
                  atol=w.atol, nthreads=threads)
        el = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": sample / el, "unit": "llh-gradients/s", "cores": threads, "kind": "port",
                               "sample": f"first {sample} conditions, oracle adjoint on all host threads ({el:.1f} s)"}
    ob = out["objective"]
    short = {"v": _r(rate32), "u": "llh-grad/s", "n": n, "fp64": _r(rate64), "r64": _r(rate32 / rate64, 3),
             "fp64_1l": _r(rate64i), "r1l": _r(rate32 / rate64i, 3), "every": _r(n / t32all),
             "obj_s": _r(ob.get("s_per_evaluation"), 3), "obj_call_s": _r(ob.get("device_call_s"), 3),
             "failed": out["failed"], **_errs_short(out["error_vs_fp64_oracle_1e-12"])}
    if "cpu_baseline" in out:
        short["cpu"] = _r(out["cpu_baseline"]["value"])
    return out, short


FSA_WORKLOAD = ("net50: random mass-action network, 50 species, 100 reactions, 100 log-parameters; 4096 "
                "instances (theta_true + N(0,1)), final times logU[1e1,1e4], 30 outputs; 10 observables, "
                "sigma 0.05; rtol 1e-8, atol 1e-10; staggered forward sensitivities")


def fsa_leg(args, dev):
    """C3: llh-gradients/s by forward sensitivities (see the module docstring)."""
    import torch

    import amici_gb300 as ag
    from amici_gb300.networks import net50_fsa_workload
    from oracle.pyoracle import Oracle

    n = 4096
    w = net50_fsa_workload(n)
    spec = w.model
    m = ag.Model(spec)
    m.set_parameter_scale(w.pscale)
    s0 = ag.Solver()
    s0.set_relative_tolerance(w.rtol)
    s0.set_absolute_tolerance(w.atol)
    # synthetic data: the engine's y at theta_true on every instance's grid plus noise (sigma 0.05)
    y = ag.simulate_batch(m, s0, np.tile(w.theta_true, (n, 1)), w.k, w.ts, pscale=w.pscale)["y"]
    my = y + np.random.default_rng(103).normal(0.0, 0.05, y.shape)
    theta, k, ts, myd = (torch.tensor(a, device=dev) for a in (w.p, w.k, w.ts, my))
    stream = torch.cuda.current_stream(dev)
    diag = torch.zeros((n, 8), dtype=torch.int32, device=dev)

    def timed(bits):
        s = ag.Solver()
        s.set_relative_tolerance(w.rtol)
        s.set_absolute_tolerance(w.atol)
        s.set_lu_precision(bits)
        s.set_control_precision(bits)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = ag.log_likelihood_and_gradient(m, s, theta, k, ts, myd, method=ag.SensitivityMethod.forward,
                                             diag=diag)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1) * 1e-3, out

    timed(32)  # warm-up
    t32, (llh32, sllh32, st32) = timed(32)
    d32 = diag.cpu().numpy().copy()
    t64, (llh64, sllh64, st64) = timed(64)
    sl32, sl64 = sllh32.cpu().numpy(), sllh64.cpu().numpy()
    rel = np.abs(sl32 - sl64) / np.abs(sl64).max(axis=1, keepdims=True)
    peak, src = hbm_peak()
    hist = fsa_history_bytes(spec, spec.np, d32)
    achieved = hist / t32 / 1e9
    out = {"metric": "llh-gradients/s", "workload": FSA_WORKLOAD, "n_instances": n, "value": n / t32,
           "unit": "llh-gradients/s", "ms_per_batch": t32 * 1e3, "fp64_batched": n / t64,
           "ratio_vs_fp64_batched": t64 / t32, "failed": int((st32 != 0).sum().item()),
           "sllh_mixed_vs_fp64_max_rel": float(np.nanmax(rel)),
           "steps_per_instance": float(d32[:, 0].mean()),
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                        "frac": achieved / peak, "peak_source": src,
                        "algorithmic_bytes_per_launch": hist,
                        "note": "sensitivity Nordsieck history read and written every accepted step, "
                                "2 (q+1) n P doubles with q = 3"}}

    def gold_errors():
        g, t = _gold("net50_fsa"), _gold("net50_fsa_tight")
        s = ag.Solver()
        s.set_relative_tolerance(w.rtol)
        s.set_absolute_tolerance(w.atol)
        lg, sg, _ = ag.log_likelihood_and_gradient(m, s, g["p"], np.zeros((len(g["p"]), 0)), g["ts"], g["my"],
                                                   method=ag.SensitivityMethod.forward)
        return gradient_error_report(lg.cpu().numpy(), sg.cpu().numpy(), g, t)
    out["error_vs_fp64_oracle_1e-12"] = _guarded(gold_errors)
    if not args.no_cpu:
        sample = 32
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        Oracle(spec).run(w.p[:sample], w.pscale, w.k[:sample], w.ts[:sample], my[:sample], rtol=w.rtol,
                         atol=w.atol, sensi=1, nthreads=threads)
        el = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": sample / el, "unit": "llh-gradients/s", "cores": threads, "kind": "port",
                               "sample": f"first {sample} instances, oracle FSA on all host threads ({el:.1f} s)"}
    short = {"v": _r(n / t32), "u": "llh-grad/s", "n": n, "fp64": _r(n / t64), "r64": _r(t64 / t32, 3),
             "hbm_frac": _r(achieved / peak, 3), "failed": out["failed"],
             **_errs_short(out["error_vs_fp64_oracle_1e-12"])}
    if "cpu_baseline" in out:
        short["cpu"] = _r(out["cpu_baseline"]["value"])
    return out, short


LARGE_WORKLOAD = ("net200: random mass-action network, 200 species, 500 reactions, 400 log10-parameters; "
                  "16384 instances (log10 k ~ U[-4,4] per instance); 10 observables, 20 outputs "
                  "logspace(-2,4), sigma 0.1; rtol 1e-8, atol 1e-10; forward solve plus adjoint llh "
                  "gradient per instance (check points every 50 steps)")


def large_data(w, solver_fn, ag):
    """Synthetic data: the engine's y at theta_true plus noise (sigma 0.1), shared by all instances."""
    m = ag.Model(w.model)
    m.set_parameter_scale(w.pscale)
    y = ag.simulate_batch(m, solver_fn(64, maxsteps=100000), w.theta_true[None, :], np.zeros((1, 0)), w.ts[:1],
                          pscale=w.pscale)["y"]
    return np.broadcast_to(y + np.random.default_rng(105).normal(0.0, 0.1, y.shape), (w.n,) + y.shape[1:]).copy()


def large_solver(ag, w, bits, ck=50, maxsteps=10000):
    # AMICI's default step budget (10,000 steps over all outputs): instances
    # that need more fail with too much work, as in the reference
    s = ag.Solver()
    s.set_relative_tolerance(w.rtol)
    s.set_absolute_tolerance(w.atol)
    s.set_lu_precision(bits)
    s.set_control_precision(bits)
    s.set_checkpoint_steps(ck)
    s.set_max_steps(maxsteps)
    return s


def large_leg(args, dev):
    """C5: llh-gradients/s on the large-batch workload (see the module docstring)."""
    import torch

    import amici_gb300 as ag
    from amici_gb300.networks import net200_workload
    from oracle.pyoracle import Oracle

    n = args.large_n
    w = net200_workload(n)
    spec = w.model
    m = ag.Model(spec)
    m.set_parameter_scale(w.pscale)
    solver = lambda bits, **kw: large_solver(ag, w, bits, **kw)
    my = large_data(w, solver, ag)
    theta, k, ts, myd = (torch.tensor(a, device=dev) for a in (w.p, w.k, w.ts, my))
    stream = torch.cuda.current_stream(dev)

    def timed(bits, rows):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = ag.log_likelihood_and_gradient(m, solver(bits), theta[rows], k[rows], ts[rows], myd[rows])
        e1.record(stream)
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1) * 1e-3, out

    timed(32, slice(0, 64))  # warm-up: module load, allocator
    t32, (llh32, sllh32, st32) = timed(32, slice(0, n))
    ns = min(n, args.large_fp64_n or n)
    t64, (llh64, sllh64, st64) = timed(64, slice(0, ns))
    sl32, sl64 = sllh32[:ns].cpu().numpy(), sllh64.cpu().numpy()
    rel = np.abs(sl32 - sl64) / np.abs(sl64).max(axis=1, keepdims=True)
    ok32 = int((st32 == 0).sum().item())
    ok32s = int((st32[:ns] == 0).sum().item())
    ok64 = int((st64 == 0).sum().item())
    out = {"metric": "llh-gradients/s", "workload": LARGE_WORKLOAD, "n_instances": n,
           "sample": f"first {n} of the 16384 instances" if n < 16384 else "full batch",
           "value": ok32 / t32, "unit": "llh-gradients/s (successful instances)",
           "dtype": "f64 states/adjoint/quadratures, f32 iteration matrix",
           "s_per_batch": t32, "fp64_lu": ok64 / t64, "fp64_lu_instances": ns, "fp64_s": t64,
           "ratio_vs_fp64_same_instances": (ok32s / t32 * n / ns) / (ok64 / t64) if ns == n else None,
           "failed": n - ok32, "failed_fp64": ns - ok64, "sllh_f32lu_vs_fp64lu_max_rel": float(np.nanmax(rel)),
           "lu": "sparse (static minimum-degree order, factors in compressed rows); dense N x N storage "
                 "does not fit the shared memory at n = 200", "lanes_per_instance": 32}

    def gold_errors():
        g, t = _gold("net200_asa"), _gold("net200_asa_tight")
        gi = len(g["p"])
        lg, sg, _ = ag.log_likelihood_and_gradient(m, solver(32), g["p"], np.zeros((gi, 0)), g["ts"], g["my"])
        return gradient_error_report(lg.cpu().numpy(), sg.cpu().numpy(), g, t)
    out["error_vs_fp64_oracle_1e-12"] = _guarded(gold_errors)
    if not args.no_cpu:
        sample = 4
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        Oracle(spec).run_asa(w.p[:sample], w.pscale, w.k[:sample], w.ts[:sample], my[:sample], rtol=w.rtol,
                             atol=w.atol, maxsteps=10000, nthreads=threads)
        el = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": sample / el, "unit": "llh-gradients/s", "cores": min(threads, sample),
                               "kind": "port",
                               "sample": f"first {sample} instances, oracle adjoint, one host thread each ({el:.1f} s)"}
    short = {"v": _r(ok32 / t32), "u": "llh-grad/s", "n": n, "of": 16384, "fp64": _r(ok64 / t64),
             "fp64_n": ns, "r64": _r(out["ratio_vs_fp64_same_instances"], 3), "failed": n - ok32,
             **_errs_short(out["error_vs_fp64_oracle_1e-12"])}
    if "cpu_baseline" in out:
        short["cpu"] = _r(out["cpu_baseline"]["value"])
    return out, short


# ---------------------------------------------------------------------------
def run_case(args):
    """One small case of a leg for profiler captures (see the module docstring)."""
    import torch

    import amici_gb300 as ag
    from amici_gb300.networks import net20_workload, net50_fsa_workload, net100_adjoint_workload, net200_workload

    dev = torch.device("cuda", 0)
    if args.case == "net20":
        w = net20_workload(1024).subset(np.arange(args.n))
        nt = args.nt or w.ts.shape[1]
        w.ts = w.ts[:, :nt]
        m = ag.Model(w.model)
        s = large_solver(ag, w, args.lu, ck=args.ck)
        run = lambda: ag.simulate_batch(m, s, w.p, w.k, w.ts, pscale=w.pscale)["status"]
    else:
        if args.case == "fsa":
            w = net50_fsa_workload(args.n)
            my = 0.5 + 0.05 * np.random.default_rng(3).normal(size=(args.n, w.ts.shape[1], w.model.ny))
        elif args.case == "adjoint":
            w = net100_adjoint_workload(args.n)
            my = 0.5 + 0.1 * np.random.default_rng(5).normal(size=(args.n, w.ts.shape[1], w.model.ny))
        else:
            w = net200_workload(args.n)
            my = large_data(w, lambda bits, **kw: large_solver(ag, w, bits, **kw), ag)
        nt = args.nt or w.ts.shape[1]
        w.ts, my = w.ts[:, :nt], my[:, :nt]
        m = ag.Model(w.model)
        m.set_parameter_scale(w.pscale)
        s = large_solver(ag, w, args.lu, ck=args.ck)
        method = ag.SensitivityMethod.forward if args.case == "fsa" else ag.SensitivityMethod.adjoint
        theta = torch.tensor(w.p, device=dev)
        run = lambda: ag.log_likelihood_and_gradient(m, s, theta, w.k, w.ts, my, method=method)[2]
    run()  # warm-up (module load)
    torch.cuda.synchronize(dev)
    for _ in range(args.reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        st = run()
        e1.record()
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1)
        failed = int((np.asarray(st.cpu() if hasattr(st, "cpu") else st) != 0).sum())
        print(f"{args.case} ck{args.ck} lu{args.lu} n={args.n} nt={nt}: {ms:.1f} ms -> "
              f"{args.n / ms * 1e3:.2f} per s; failed {failed}", flush=True)


# ---------------------------------------------------------------------------
def _gold(name):
    return dict(np.load(GOLD / f"{name}.npz"))


def state_error_report(x, stated, tight):
    """States against the reference at rtol = atol = 1e-12, in units of the
    stated tolerances (rtol |x| + atol), beside the reference's own error at
    the stated tolerances; ``x`` holds the instances of the golden set."""
    rtol, atol = float(stated["rtol"]), float(stated["atol"])
    tu = lambda a: np.abs(a - tight["x"]) / (rtol * np.abs(tight["x"]) + atol)
    big = np.abs(tight["x"]) > 1e3 * atol
    rel = np.abs(x - tight["x"])[big] / np.abs(tight["x"])[big]
    return {"instances": int(len(x)), "x_tol_units_max": float(tu(x).max()),
            "reference_x_tol_units_max": float(tu(stated["x"]).max()),
            "x_rel_err_max_where_above_1e3_atol": float(rel.max()) if rel.size else None}


def gradient_error_report(llh, sllh, stated, tight):
    """llh (relative) and sllh (relative to each instance's largest
    component) against the reference at rtol = atol = 1e-12, beside the
    reference's own errors at the stated tolerances."""
    def errs(l, s):
        return (float(np.max(np.abs(l - tight["llh"]) / np.abs(tight["llh"]))),
                float(np.max(np.abs(s - tight["sllh"]) / np.abs(tight["sllh"]).max(axis=1, keepdims=True))))
    e_l, e_s = errs(np.asarray(llh), np.asarray(sllh))
    r_l, r_s = errs(stated["llh"], stated["sllh"])
    return {"instances": int(len(tight["llh"])), "llh_rel_max": e_l, "sllh_rel_to_max": e_s,
            "reference_llh_rel_max": r_l, "reference_sllh_rel_to_max": r_s}


def _guarded(fn):
    """A report that cannot end the benchmark: its exception is recorded."""
    try:
        return fn()
    except Exception as e:  # noqa: BLE001
        return {"unavailable": f"{type(e).__name__}: {e}"}


def _native_probe(path):
    import ctypes
    lib = ctypes.CDLL(str(path))
    lib.amici_gb300_probe_fp64_gflops.restype = ctypes.c_double
    lib.amici_gb300_probe_fp64_gflops.argtypes = [ctypes.c_int]
    return float(lib.amici_gb300_probe_fp64_gflops(4096))


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--lanes", type=int, default=0, help="lanes per instance (0 = autotuned)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baselines")
    ap.add_argument("--no-grad", action="store_true", help="skip the C3, C4 and C5 legs")
    ap.add_argument("--grad-reps", type=int, default=1, help="timed batches of the C4 leg")
    ap.add_argument("--no-large", action="store_true", help="skip the C5 (n = 200) leg")
    ap.add_argument("--large-n", type=int, default=608,
                    help="instances of the C5 leg (the first of the 16,384; 16384 = the full batch)")
    ap.add_argument("--large-fp64-n", type=int, default=0,
                    help="instances of the C5 leg timed with the FP64 iteration matrix (0: the same as --large-n)")
    ap.add_argument("--detail", default="", help="write every leg's full report to this JSON file")
    ap.add_argument("--case", choices=["net20", "fsa", "adjoint", "large"], default="",
                    help="run one small case of a leg for profiler captures instead")
    ap.add_argument("--n", type=int, default=16, help="--case: instances")
    ap.add_argument("--nt", type=int, default=0, help="--case: first nt outputs (0: all)")
    ap.add_argument("--lu", type=int, default=32, help="--case: iteration matrix precision (32 or 64)")
    ap.add_argument("--ck", type=int, default=50, help="--case: adjoint check-point spacing (0: every step)")
    ap.add_argument("--reps", type=int, default=1, help="--case: timed calls")
    args = ap.parse_args()
    if args.case:
        run_case(args)
        return
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, rank)
    else:
        run_gb300(args, ws, rank, local)


if __name__ == "__main__":
    main()
