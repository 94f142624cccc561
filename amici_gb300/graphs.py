"""CUDA-graph-captured simulation launches.

Repeated calls with the same batch shape (an optimiser evaluating llh and its
gradient at new parameter values, a sampler, a parameter sweep) re-issue the
same launch sequence: the work-queue reset, the persistent kernel and the
stream-ordered scratch allocation and release.  ``GraphedSimulation``
captures that sequence once on a side stream into a CUDA graph over fixed
device buffers; each ``run`` copies new inputs into those buffers (device to
device, or host to device from pinned memory) and replays the graph, so a
call costs one graph launch regardless of how many kernels the sequence
holds (one per instance in per-instance launch mode).
"""
from __future__ import annotations

import numpy as np

from . import _native
from .simulation import Model, SensitivityMethod, SensitivityOrder, Solver


class GraphedSimulation:
    """One captured call of the device entry point for a fixed batch shape.

    ``inputs`` (device tensors) ``p, k, ts, my`` and outputs ``llh, status,
    numsteps`` (plus ``sllh`` with sensitivities, ``x`` when ``want_x``) are
    owned by the object; ``run(p=..., k=..., ts=..., my=...)`` writes new
    values into them and replays."""

    def __init__(self, model: Model, solver: Solver, n: int, nt: int, *, with_data=True, want_x=False,
                 plist=None, device=None):
        import torch

        self.torch = torch
        spec = model.spec
        self.model, self.solver = model, solver
        self.dev = torch.device("cuda", torch.cuda.current_device()) if device is None else device
        f64 = dict(dtype=torch.float64, device=self.dev)
        self.p = torch.zeros((n, spec.np), **f64)
        self.k = torch.zeros((n, max(spec.nk, 1)), **f64)
        self.ts = torch.zeros((n, nt), **f64)
        self.my = torch.zeros((n, nt, spec.ny), **f64) if with_data else None
        self.pscale = torch.as_tensor(model.get_parameter_scale(), dtype=torch.int32, device=self.dev)
        sens = int(solver.sensi) > 0
        pl = np.arange(spec.np) if plist is None else np.asarray(plist)
        self.plist = torch.as_tensor(pl, dtype=torch.int32, device=self.dev)
        self.llh = torch.empty(n, **f64)
        self.sllh = torch.empty((n, len(pl)), **f64) if sens else None
        self.x = torch.empty((n, nt, spec.nx), **f64) if want_x else None
        self.numsteps = torch.empty((n, nt), dtype=torch.int32, device=self.dev)
        self.status = torch.empty(n, dtype=torch.int32, device=self.dev)
        if sens and solver.sensi_meth == SensitivityMethod.forward:
            raise ValueError("captured calls support forward simulation and adjoint sensitivities")
        b = _native.Batch()
        b.n_instances, b.nt, b.nplist = n, nt, len(pl) if sens else 0
        b.p, b.pscale, b.ts = self.p.data_ptr(), self.pscale.data_ptr(), self.ts.data_ptr()
        b.k = self.k.data_ptr() if spec.nk else None
        b.my = None if self.my is None else self.my.data_ptr()
        b.sigma_y = None
        b.plist = self.plist.data_ptr() if sens else None
        b.x = None if self.x is None else self.x.data_ptr()
        b.y = b.sigmay = b.sx = b.sy = b.diag = None
        b.llh = self.llh.data_ptr()
        b.sllh = None if self.sllh is None else self.sllh.data_ptr()
        b.numsteps, b.status = self.numsteps.data_ptr(), self.status.data_ptr()
        self._batch = b
        self._opts = solver.to_options()
        lib = model.library
        self.stream = torch.cuda.Stream(self.dev)
        # one eager call outside the capture: module load, function attributes, allocator pools
        with torch.cuda.stream(self.stream):
            lib.run_device(self._opts, b, self.stream.cuda_stream)
        self.stream.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, stream=self.stream, capture_error_mode="relaxed"):
            lib.run_device(self._opts, b, self.stream.cuda_stream)

    def run(self, p=None, k=None, ts=None, my=None):
        """Write new inputs (any that are given) and replay; returns after the
        replay is queued on torch's current stream (outputs are the object's
        tensors)."""
        for dst, src in ((self.p, p), (self.k, k), (self.ts, ts), (self.my, my)):
            if src is not None:
                dst.copy_(self.torch.as_tensor(src).reshape(dst.shape), non_blocking=True)
        self.graph.replay()
        return self
