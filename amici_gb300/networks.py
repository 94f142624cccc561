"""Seeded synthetic workloads: the Robertson ODE and random mass-action networks.

These stand in for the reference's test models.  The reference ships its
Robertson test model as a DAE (``python/sdist/amici/testing/models.py:90-127``);
the workloads here are the pure-ODE form and random mass-action networks with
the sizes, value distributions and output grids of the five benchmark
configurations.  Everything is drawn from ``numpy.random.default_rng(seed)``.

Random networks: each reaction draws 1–2 reactants and 1–2 products uniformly
from the species; its flux is ``k_r · Π x_reactant``.  Random topologies can
grow without bound (autocatalysis), so a topology is accepted only if the
oracle integrates a screening set of parameter draws with all states below
``1e6``; the accepted topology seed is recorded in ``ACCEPTED_TOPOLOGY_SEED``.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import sympy as sp

from .model_spec import TIME, Event, ModelSpec, mass_action_model

PSCALE_LIN, PSCALE_LN, PSCALE_LOG10 = 0, 1, 2


@dataclass
class Workload:
    """A model plus a batch of per-instance inputs (all numpy, row-major)."""

    name: str
    model: ModelSpec
    p: np.ndarray          # [N, np] scaled parameters
    pscale: np.ndarray     # [np] int32
    k: np.ndarray          # [N, nk]
    ts: np.ndarray         # [N, nt]
    my: np.ndarray | None  # [N, nt, ny] measurements (NaN = missing)
    sigma: np.ndarray | None  # [N, nt, ny] noise scales (NaN = model value)
    rtol: float
    atol: float
    sensi: int             # 0 none, 1 forward, 2 adjoint

    @property
    def n(self):
        return self.p.shape[0]

    def subset(self, idx):
        idx = np.asarray(idx)
        return Workload(self.name, self.model, self.p[idx], self.pscale, self.k[idx],
                        self.ts[idx], None if self.my is None else self.my[idx],
                        None if self.sigma is None else self.sigma[idx],
                        self.rtol, self.atol, self.sensi)


def robertson_model() -> ModelSpec:
    """Robertson kinetics: x1 -> x2 (k1), 2 x2 -> x2 + x3 (k2), x2 + x3 -> x1 + x3 (k3).

    dx1 = -k1 x1 + k3 x2 x3; dx2 = k1 x1 - k2 x2^2 - k3 x2 x3; dx3 = k2 x2^2.
    """
    reactions = [([0], [1]), ([1, 1], [1, 2]), ([1, 2], [0, 2])]
    return mass_action_model(
        "robertson", 3, reactions, [0, 1, 2], 3, x0=[1.0, 0.0, 0.0],
        observables=[{0: 1.0}, {1: 1.0}, {2: 1.0}], sigma=0.01,
        p_nominal=[0.04, 3e7, 1e4])


def robertson_workload(n_instances: int = 1, seed: int = 1) -> Workload:
    """One Robertson instance, 40 log-spaced outputs on [1e-4, 1e5],
    forward sensitivities w.r.t. ln k, y = x, sigma = 0.01, data = y(k) + N(0, sigma^2)."""
    m = robertson_model()
    k_true = np.array([0.04, 3e7, 1e4])
    ts = np.logspace(-4, 5, 40)
    p = np.tile(np.log(k_true), (n_instances, 1))
    return Workload("robertson", m, p, np.full(3, PSCALE_LN, np.int32),
                    np.zeros((n_instances, 0)), np.tile(ts, (n_instances, 1)),
                    None, None, 1e-8, 1e-12, 1)


def random_topology(n_species: int, n_reactions: int, seed: int):
    """Draw a mass-action topology: per reaction 1–2 reactants and 1–2 products,
    species uniform with replacement."""
    rng = np.random.default_rng(seed)
    reactions = []
    for _ in range(n_reactions):
        nr = int(rng.integers(1, 3))
        npd = int(rng.integers(1, 3))
        reac = sorted(int(s) for s in rng.integers(0, n_species, nr))
        prod = sorted(int(s) for s in rng.integers(0, n_species, npd))
        reactions.append((reac, prod))
    return reactions


def random_observables(n_species, n_obs, rng, per_obs=3):
    obs = []
    for _ in range(n_obs):
        sp_idx = rng.choice(n_species, per_obs, replace=False)
        wts = rng.uniform(0.0, 1.0, per_obs)
        obs.append({int(s): float(w) for s, w in zip(sp_idx, wts)})
    return obs


# Topology seeds accepted by the boundedness screen (see module docstring),
# keyed by (n_species, n_reactions).  Filled in by ``screen_topology``.
ACCEPTED_TOPOLOGY_SEED = {
    (20, 40): 1,
    (50, 100): 0,
    (100, 300): 0,
    (200, 500): 1,
}


def network_model(name, n_species, n_reactions, n_params, *, topology_seed=None,
                  n_obs=None, sigma=1.0, x0=None, input_species=None, obs_seed=7):
    if topology_seed is None:
        topology_seed = ACCEPTED_TOPOLOGY_SEED[(n_species, n_reactions)]
    reactions = random_topology(n_species, n_reactions, topology_seed)
    rate_idx = [r % n_params for r in range(n_reactions)]
    rng = np.random.default_rng(obs_seed)
    observables = None if n_obs is None else random_observables(n_species, n_obs, rng)
    nk = 0 if input_species is None else len(input_species)
    fixed = None if input_species is None else {s: j for j, s in enumerate(input_species)}
    if x0 is None:
        x0 = np.ones(n_species)
    return mass_action_model(name, n_species, reactions, rate_idx, n_params, nk=nk,
                             x0=list(map(float, x0)), observables=observables,
                             sigma=sigma, fixed_x0_scale=fixed)


def net20_workload(n_instances: int = 1024, seed: int = 2) -> Workload:
    """Batched forward simulation: n=20, R=40, log10 k ~ U[-3,3] per instance,
    x0 log-uniform in [1e-2, 1] (fixed per topology), 50 outputs logspace(-3, 3),
    rtol 1e-8, atol 1e-10, no sensitivities.  Parameters in log10 scale."""
    rng = np.random.default_rng(seed)
    x0 = 10.0 ** np.random.default_rng(1000 + seed).uniform(-2, 0, 20)
    m = network_model("net20", 20, 40, 40, x0=x0)
    m.families = ("fwd", "asa")
    p = rng.uniform(-3, 3, (n_instances, 40))
    ts = np.tile(np.logspace(-3, 3, 50), (n_instances, 1))
    return Workload("net20", m, p, np.full(40, PSCALE_LOG10, np.int32),
                    np.zeros((n_instances, 0)), ts, None, None, 1e-8, 1e-10, 0)


def net50_fsa_workload(n_instances: int = 4096, seed: int = 3, simulate=None) -> Workload:
    """Batched forward sensitivities with uneven work: n=50, R=100, one
    log-parameter per reaction (theta_r = ln k_r), theta = theta_true + N(0,1)
    per instance with log10 k_true ~ U[-3,3]; final times log-uniform in
    [1e1, 1e4], 30 outputs t_f * logspace(-4, 0); 10 observables, each a random
    nonnegative combination of 3 species, Gaussian noise sigma = 0.05.

    Synthetic data are y(theta_true) + N(0, 0.05^2) on every instance's grid,
    computed with ``simulate(model, p, pscale, ts) -> y`` if given (no data
    otherwise).  rtol 1e-8, atol 1e-10; forward sensitivities w.r.t. all 100
    parameters."""
    rng = np.random.default_rng(seed)
    x0 = 10.0 ** np.random.default_rng(1000 + seed).uniform(-2, 0, 50)
    m = network_model("net50", 50, 100, 100, n_obs=10, sigma=0.05, x0=x0)
    m.families = ("fwd", "fsa")
    theta_true = np.log(10.0 ** rng.uniform(-3, 3, 100))
    p = theta_true + rng.normal(0.0, 1.0, (n_instances, 100))
    tf = 10.0 ** rng.uniform(1, 4, n_instances)
    ts = tf[:, None] * np.logspace(-4, 0, 30)[None, :]
    pscale = np.full(100, PSCALE_LN, np.int32)
    my = None
    if simulate is not None:
        y = simulate(m, np.tile(theta_true, (n_instances, 1)), pscale, ts)
        my = y + np.random.default_rng(seed + 100).normal(0.0, 0.05, y.shape)
    w = Workload("net50_fsa", m, p, pscale, np.zeros((n_instances, 0)), ts, my, None, 1e-8, 1e-10, 1)
    w.theta_true = theta_true
    return w


def net100_adjoint_workload(n_instances: int = 512, seed: int = 4, simulate=None) -> Workload:
    """Adjoint gradients: n=100, R=300 (about 6 Jacobian nonzeros per row),
    256 log-parameters (theta = ln k, reaction r uses theta_{r mod 256}) with
    log10 k_true ~ U[-3, 3], shared by all conditions; 5 input species whose
    initial concentrations are scaled per condition by fixed parameters
    log-uniform in [0.1, 10]; 8 observables (random nonnegative combinations
    of 3 species), Gaussian noise sigma = 0.1; 100 outputs linspace(0, 500).

    Synthetic data are y(theta_true) + N(0, 0.1^2) per condition, computed
    with ``simulate(model, p, pscale, k, ts) -> y`` if given (no data
    otherwise).  rtol 1e-8, atol 1e-10; adjoint sensitivities w.r.t. all 256
    parameters."""
    rng = np.random.default_rng(seed)
    x0 = 10.0 ** np.random.default_rng(1000 + seed).uniform(-2, 0, 100)
    inputs = sorted(int(s) for s in np.random.default_rng(2000 + seed).choice(100, 5, replace=False))
    m = network_model("net100", 100, 300, 256, n_obs=8, sigma=0.1, x0=x0, input_species=inputs)
    m.families = ("fwd", "asa")
    theta_true = np.log(10.0 ** rng.uniform(-3, 3, 256))
    k = 10.0 ** rng.uniform(-1, 1, (n_instances, 5))
    p = np.tile(theta_true, (n_instances, 1))
    ts = np.tile(np.linspace(0.0, 500.0, 100), (n_instances, 1))
    pscale = np.full(256, PSCALE_LN, np.int32)
    my = None
    if simulate is not None:
        y = simulate(m, p, pscale, k, ts)
        my = y + np.random.default_rng(seed + 100).normal(0.0, 0.1, y.shape)
    w = Workload("net100_adjoint", m, p, pscale, k, ts, my, None, 1e-8, 1e-10, 2)
    w.theta_true = theta_true
    w.input_species = inputs
    return w


def net200_workload(n_instances: int = 16384, seed: int = 5, simulate=None) -> Workload:
    """Large batch, forward solve plus adjoint llh gradient per instance:
    n=200, R=500 (about 5 Jacobian nonzeros per row), 400 log10-parameters
    (reaction r uses theta_{r mod 400}), log10 k ~ U[-4, 4] drawn per
    instance (stiffness ratios up to 1e8); x0 log-uniform in [1e-2, 1] (fixed
    per topology); 20 outputs logspace(-2, 4); 10 observables (random
    nonnegative combinations of 3 species), Gaussian noise sigma = 0.1.

    Synthetic data are y(theta_true) + N(0, 0.1^2) on the output grid for one
    seeded true parameter set (log10 k_true ~ U[-4, 4]), computed with
    ``simulate(model, p, pscale, ts) -> y`` if given (no data otherwise) and
    shared by all instances.  rtol 1e-8, atol 1e-10; adjoint sensitivities
    w.r.t. all 400 parameters."""
    rng = np.random.default_rng(seed)
    x0 = 10.0 ** np.random.default_rng(1000 + seed).uniform(-2, 0, 200)
    m = network_model("net200", 200, 500, 400, n_obs=10, sigma=0.1, x0=x0)
    m.families = ("fwd", "asa")
    theta_true = rng.uniform(-4, 4, 400)
    p = rng.uniform(-4, 4, (n_instances, 400))
    ts = np.tile(np.logspace(-2, 4, 20), (n_instances, 1))
    pscale = np.full(400, PSCALE_LOG10, np.int32)
    my = None
    if simulate is not None:
        y = simulate(m, theta_true[None, :], pscale, ts[:1])
        my = np.broadcast_to(y + np.random.default_rng(seed + 100).normal(0.0, 0.1, y.shape),
                             (n_instances,) + y.shape[1:]).copy()
    w = Workload("net200", m, p, pscale, np.zeros((n_instances, 0)), ts, my, None, 1e-8, 1e-10, 2)
    w.theta_true = theta_true
    return w


def preeq_model(topology_seed: int = 11) -> ModelSpec:
    """A network with a steady state for pre-equilibration: 12 species;
    zero-order production of the two input species x0 and x1 at rates
    p0 * k0 and p1 * k1 (k: stimulus levels, fixed parameters); first-order
    degradation of every species (rates p2..p5, cyclically); a conversion
    chain x_i -> x_(i+1) and x1 -> x6 that reaches every species, and 6
    random conversions or bindings that never increase the molecule count (at
    most as many products as reactants); conversion rates p6..p13
    cyclically.  14 parameters; 4 observables (random nonnegative
    combinations of 3 species), sigma 0.1; x0 = 0."""
    nx = 12
    rng = np.random.default_rng(topology_seed)
    reactions, rate_idx = [([], [0]), ([], [1])], [0, 1]
    for i in range(nx):
        reactions.append(([i], []))
        rate_idx.append(2 + i % 4)
    conv = [([i], [i + 1]) for i in range(nx - 1)] + [([1], [6])]
    for _ in range(6):
        nr = int(rng.integers(1, 3))
        reac = sorted(int(s) for s in rng.integers(0, nx, nr))
        prod = sorted(int(s) for s in rng.integers(0, nx, int(rng.integers(1, nr + 1))))
        conv.append((reac, prod))
    for j, rc in enumerate(conv):
        reactions.append(rc)
        rate_idx.append(6 + j % 8)
    obs = random_observables(nx, 4, np.random.default_rng(topology_seed + 1))
    m = mass_action_model("preeq12", nx, reactions, rate_idx, 14, nk=2, x0=[0.0] * nx, observables=obs,
                          sigma=0.1)
    m.w[0] = m.w[0] * m.k[0]
    m.w[1] = m.w[1] * m.k[1]
    m.families = ("fwd", "fsa", "asa", "preeq", "posteq")
    return m


def preeq_workload(n_instances: int = 256, seed: int = 6, simulate=None) -> Workload:
    """Pre-equilibration, then the response to a stimulus: the ``preeq12``
    network pre-equilibrated at basal input levels k_preeq = (0.1, 0.1), then
    simulated from that steady state with per-instance stimulus levels k
    log-uniform in [1, 10]; theta = ln k_true + N(0, 0.3^2) per instance with
    log10 k_true ~ U[-1, 1]; 20 outputs logspace(-1, 2); rtol 1e-8, atol
    1e-10.  Synthetic data are y(theta_true) + N(0, 0.1^2), computed with
    ``simulate(model, p, pscale, k, ts, k_preeq) -> y`` if given.
    ``w.k_preeq`` holds the pre-equilibration parameters [N, 2]."""
    m = preeq_model()
    rng = np.random.default_rng(seed)
    theta_true = np.log(10.0 ** rng.uniform(-1, 1, 14))
    p = theta_true + rng.normal(0.0, 0.3, (n_instances, 14))
    k = 10.0 ** rng.uniform(0, 1, (n_instances, 2))
    k_preeq = np.full((n_instances, 2), 0.1)
    ts = np.tile(np.logspace(-1, 2, 20), (n_instances, 1))
    pscale = np.full(14, PSCALE_LN, np.int32)
    my = None
    if simulate is not None:
        y = simulate(m, np.tile(theta_true, (n_instances, 1)), pscale, k, ts, k_preeq)
        my = y + np.random.default_rng(seed + 100).normal(0.0, 0.1, y.shape)
    w = Workload("preeq12", m, p, pscale, k, ts, my, None, 1e-8, 1e-10, 1)
    w.theta_true = theta_true
    w.k_preeq = k_preeq
    return w


def obs_model() -> ModelSpec:
    """The observation model beyond affine Gaussian observables: a random
    mass-action network of 6 species and 10 reactions (rates p0..p9) with
    six observables, one per noise distribution of the reference (normal,
    log-normal, log10-normal, laplace, log-laplace, log10-laplace):
    y0 = x0 / (x0 + x1), y1 = p11 * x2 + p12, y2 = x3 + x4, y3 = x5,
    y4 = x1^2, y5 = x0 * x3; noise scales p10 (y0), p13 (y3) and 0.1
    otherwise.  14 parameters on the ln scale."""
    reactions = random_topology(6, 10, 17)
    m = mass_action_model("obs6", 6, reactions, list(range(10)), 14, x0=[1.0, 0.5, 0.2, 0.1, 0.3, 0.05],
                          sigma=0.1)
    x, p = m.x, m.p
    m.y = [x[0] / (x[0] + x[1]), p[11] * x[2] + p[12], x[3] + x[4], x[5], x[1] ** 2, x[0] * x[3]]
    m.observable_ids = [f"y{i}" for i in range(6)]
    m.sigma_y = [p[10], sp.Float(0.1), sp.Float(0.1), p[13], sp.Float(0.1), sp.Float(0.1)]
    m.noise_distributions = ["normal", "log-normal", "log10-normal", "laplace", "log-laplace", "log10-laplace"]
    m.families = ("fwd", "fsa", "asa")
    return m


def obs_workload(n_instances: int = 16, seed: int = 7, simulate=None) -> Workload:
    """Instances of ``obs6``: theta = theta_true + N(0, 0.2^2) with
    ln k_true ~ U[ln 0.1, ln 1] for the rates and sigma0 = 0.1, scale 2,
    offset 0.5, sigma3 = 0.05; 15 outputs logspace(-1, 1.5).  Synthetic
    data are y(theta_true) * exp(0.05 N(0, 1)) (positive, as the log
    distributions need), from ``simulate(model, p, pscale, ts) -> y`` if
    given."""
    m = obs_model()
    rng = np.random.default_rng(seed)
    theta_true = np.concatenate([np.log(10.0 ** rng.uniform(-1, 0, 10)), np.log([0.1, 2.0, 0.5, 0.05])])
    p = theta_true + rng.normal(0.0, 0.2, (n_instances, 14))
    ts = np.tile(np.logspace(-1, 1.5, 15), (n_instances, 1))
    pscale = np.full(14, PSCALE_LN, np.int32)
    my = None
    if simulate is not None:
        y = simulate(m, np.tile(theta_true, (n_instances, 1)), pscale, ts)
        my = y * np.exp(0.05 * np.random.default_rng(seed + 100).normal(size=y.shape))
    w = Workload("obs6", m, p, pscale, np.zeros((n_instances, 0)), ts, my, None, 1e-8, 1e-10, 1)
    w.theta_true = theta_true
    return w


# Kholodenko's MAPK cascade rate constants (Eur. J. Biochem. 267, 1583-1588,
# 2000): V1, Ki, K1, V2, K2, k3, K3, k4, K4, V5, K5, V6, K6, k7, K7, k8, K8,
# V9, K9, V10, K10; then the feedback loop kf, Kf, kd, the observable scale
# and its noise scale
MAPK_NOMINAL = (2.5, 9.0, 10.0, 0.25, 8.0, 0.025, 15.0, 0.025, 15.0, 0.75, 15.0, 0.75, 15.0, 0.025, 15.0,
                0.025, 15.0, 0.5, 15.0, 0.5, 15.0, 0.01, 50.0, 0.005, 0.01, 0.05)


def mapk_model() -> ModelSpec:
    """General kinetics: a three-tier MAPK cascade with Michaelis–Menten
    (de)phosphorylations, a Hill-type negative feedback of MAPK-PP on the
    first tier, and an inducible phosphatase activator F.  States: MKKK,
    MKKK-P, MKK, MKK-P, MKK-PP, MAPK, MAPK-P, MAPK-PP, F.  Fluxes:
    v1 = k0 V1 x0 / ((1 + (x7/Ki)^2)(K1 + x0)), v2 = V2 x1/(K2 + x1),
    v3 = k3 x1 x2/(K3 + x2), v4 = k4 x1 x3/(K4 + x3), v5 = V5 x4/(K5 + x4),
    v6 = V6 x3/(K6 + x3), v7 = k7 x4 x5/(K7 + x5), v8 = k8 x4 x6/(K8 + x6),
    v9 = V9 (1 + x8) x7/(K9 + x7), v10 = V10 x6/(K10 + x6),
    v11 = kf x7^2/(Kf^2 + x7^2) (production of F), v12 = kd x8 (mass action).
    k0: stimulus level (fixed parameter).  Observables: s (x6 + x7) (normal,
    sigma p25), x4 (normal, sigma 1) and the active fraction
    x7 / (x5 + x6 + x7) (log-normal, sigma 0.1).  26 parameters."""
    x = sp.symbols("x0:9", real=True)
    p = sp.symbols("p0:26", real=True)
    k = sp.symbols("k0:1", real=True)
    (V1, Ki, K1, V2, K2, k3, K3, k4, K4, V5, K5, V6, K6, k7, K7, k8, K8, V9, K9, V10, K10,
     kf, Kf, kd, s, sg) = p
    w = [k[0] * V1 * x[0] / ((1 + (x[7] / Ki) ** 2) * (K1 + x[0])),
         V2 * x[1] / (K2 + x[1]),
         k3 * x[1] * x[2] / (K3 + x[2]),
         k4 * x[1] * x[3] / (K4 + x[3]),
         V5 * x[4] / (K5 + x[4]),
         V6 * x[3] / (K6 + x[3]),
         k7 * x[4] * x[5] / (K7 + x[5]),
         k8 * x[4] * x[6] / (K8 + x[6]),
         V9 * (1 + x[8]) * x[7] / (K9 + x[7]),
         V10 * x[6] / (K10 + x[6]),
         kf * x[7] ** 2 / (Kf ** 2 + x[7] ** 2),
         kd * x[8]]
    conv = [(0, 1), (1, 0), (2, 3), (3, 4), (4, 3), (3, 2), (5, 6), (6, 7), (7, 6), (6, 5)]
    stoich = {}
    for r, (a, b) in enumerate(conv):
        stoich[(a, r)] = -1
        stoich[(b, r)] = 1
    stoich[(8, 10)] = 1
    stoich[(8, 11)] = -1
    x0 = [sp.Float(v) for v in (100.0, 0.0, 300.0, 0.0, 0.0, 300.0, 0.0, 0.0, 0.0)]
    y = [s * (x[6] + x[7]), x[4], x[7] / (x[5] + x[6] + x[7])]
    m = ModelSpec(name="mapk9", state_ids=["MKKK", "MKKK_P", "MKK", "MKK_P", "MKK_PP", "MAPK", "MAPK_P",
                                           "MAPK_PP", "F"],
                  parameter_ids=["V1", "Ki", "K1", "V2", "K2", "k3", "K3", "k4", "K4", "V5", "K5", "V6", "K6",
                                 "k7", "K7", "k8", "K8", "V9", "K9", "V10", "K10", "kf", "Kf", "kd", "scale",
                                 "sigma"],
                  fixed_parameter_ids=["stimulus"], observable_ids=["MAPK_act", "MKK_PP", "MAPK_frac"],
                  x0=x0, w=w, stoich=stoich, y=y, sigma_y=[sg, sp.Float(1.0), sp.Float(0.1)],
                  x=list(x), p=list(p), k=list(k), p_nominal=list(MAPK_NOMINAL), k_nominal=[1.0],
                  noise_distributions=["normal", "normal", "log-normal"])
    m.families = ("fwd", "fsa", "asa")
    return m


def mapk_workload(n_instances: int = 64, seed: int = 8, simulate=None) -> Workload:
    """Instances of ``mapk9``: theta = log10 of the nominal constants +
    N(0, 0.1^2) per instance, stimulus k0 log-uniform in [0.5, 2]; 20 outputs
    on [150, 3000]; rtol 1e-8, atol 1e-10.  Synthetic data are
    y(theta_nominal) * exp(0.05 N(0, 1)) (positive, for the log-normal
    observable), from ``simulate(model, p, pscale, k, ts) -> y`` if given."""
    m = mapk_model()
    rng = np.random.default_rng(seed)
    theta_true = np.log10(np.array(MAPK_NOMINAL))
    p = theta_true + rng.normal(0.0, 0.1, (n_instances, m.np))
    k = 10.0 ** rng.uniform(np.log10(0.5), np.log10(2.0), (n_instances, 1))
    ts = np.tile(np.linspace(150.0, 3000.0, 20), (n_instances, 1))
    pscale = np.full(m.np, PSCALE_LOG10, np.int32)
    my = None
    if simulate is not None:
        y = simulate(m, np.tile(theta_true, (n_instances, 1)), pscale, k, ts)
        my = y * np.exp(0.05 * np.random.default_rng(seed + 100).normal(size=y.shape))
    w = Workload("mapk9", m, p, pscale, k, ts, my, None, 1e-8, 1e-10, 1)
    w.theta_true = theta_true
    return w


# pharmacokinetic / turnover rates: ka, Vmax, Km, k12, k21, kin, Imax, IC50,
# kout, dose, second dose time, volume, noise scale
DOSE_NOMINAL = (1.2, 4.0, 2.0, 0.3, 0.15, 1.0, 0.8, 1.5, 0.1, 10.0, 12.0, 2.0, 0.1)


def dosing_model() -> ModelSpec:
    """Events: a pharmacokinetic model with two doses and a washout, and a
    pharmacodynamic turnover response.  States: depot x0, central x1,
    peripheral x2, response x3.  Fluxes: absorption ka x0, saturable
    elimination Vmax x1 / (Km + x1), distribution k12 x1 and k21 x2,
    production kin (1 - Imax x1 / (IC50 + x1)) and loss kout x3 of the
    response.  Events (explicit trigger times): a loading dose x0 += dose / 2
    at t = 0 (a trigger true at t0 whose initial value is false, so it fires
    at t0), a dose x0 += dose at t = 2, a second dose at t = td2 (a
    parameter, so the event time has parameter sensitivities), and at t = k0
    (a fixed parameter) half of the peripheral amount is removed
    (x2 := x2 / 2).  x3(0) = kin / kout.  Observables: the concentration
    x1 / V (sigma p12) and the response x3 (sigma 0.1)."""
    x = sp.symbols("x0:4", real=True)
    p = sp.symbols("p0:13", real=True)
    k = sp.symbols("k0:1", real=True)
    ka, Vmax, Km, k12, k21, kin, Imax, IC50, kout, dose, td2, V, sg = p
    w = [ka * x[0], Vmax * x[1] / (Km + x[1]), k12 * x[1], k21 * x[2],
         kin * (1 - Imax * x[1] / (IC50 + x[1])), kout * x[3]]
    stoich = {(0, 0): -1, (1, 0): 1, (1, 1): -1, (1, 2): -1, (2, 2): 1, (2, 3): -1, (1, 3): 1,
              (3, 4): 1, (3, 5): -1}
    m = ModelSpec(name="dose4", state_ids=["depot", "central", "peripheral", "response"],
                  parameter_ids=["ka", "Vmax", "Km", "k12", "k21", "kin", "Imax", "IC50", "kout", "dose", "td2",
                                 "V", "sigma"],
                  fixed_parameter_ids=["t_washout"], observable_ids=["conc", "response"],
                  x0=[sp.Integer(0), sp.Integer(0), sp.Integer(0), kin / kout], w=w, stoich=stoich,
                  y=[x[1] / V, x[3]], sigma_y=[sg, sp.Float(0.1)], x=list(x), p=list(p), k=list(k),
                  p_nominal=list(DOSE_NOMINAL), k_nominal=[20.0],
                  events=[Event(time=sp.Integer(0), bolus={0: dose / 2}, initial_value=False),
                          Event(time=sp.Integer(2), bolus={0: dose}),
                          Event(time=td2, bolus={0: dose}),
                          Event(time=k[0], bolus={2: -x[2] / 2})])
    m.families = ("fwd", "fsa")
    return m


def dosing_workload(n_instances: int = 64, seed: int = 9, simulate=None) -> Workload:
    """Instances of ``dose4``: theta = ln of the nominal constants +
    N(0, 0.15^2), washout time k0 uniform in [16, 30]; 30 outputs on
    [0.5, 48]; rtol 1e-8, atol 1e-10.  Synthetic data are y(theta_nominal)
    + N(0, 0.05^2), from ``simulate(model, p, pscale, k, ts) -> y`` if given."""
    m = dosing_model()
    rng = np.random.default_rng(seed)
    theta_true = np.log(np.array(DOSE_NOMINAL))
    p = theta_true + rng.normal(0.0, 0.15, (n_instances, m.np))
    k = rng.uniform(16.0, 30.0, (n_instances, 1))
    ts = np.tile(np.linspace(0.5, 48.0, 30), (n_instances, 1))
    pscale = np.full(m.np, PSCALE_LN, np.int32)
    my = None
    if simulate is not None:
        y = simulate(m, np.tile(theta_true, (n_instances, 1)), pscale, k, ts)
        my = y + np.random.default_rng(seed + 100).normal(0.0, 0.05, y.shape)
    w = Workload("dose4", m, p, pscale, k, ts, my, None, 1e-8, 1e-10, 1)
    w.theta_true = theta_true
    return w


def fire_model() -> ModelSpec:
    """Events with a trigger function (root finding): an integrate-and-fire
    unit with adaptation.  x0 integrates an input, x0' = I - g x0 - x2 x0;
    when x0 crosses the threshold theta upwards (trigger x0 - theta), x0 is
    reset to 0, the fire counter x1 increases by 1 and the adaptation x2 by
    a; x2 decays at rate r.  Parameters I, g, theta, a, r and the noise scale
    of the potential; observables x1 (sigma 0.5), x2 (sigma 0.05) and x0
    (sigma p5)."""
    x = sp.symbols("x0:3", real=True)
    p = sp.symbols("p0:6", real=True)
    I_in, gl, theta, a, r, sg = p
    w = [I_in, gl * x[0], x[2] * x[0], r * x[2]]
    stoich = {(0, 0): 1, (0, 1): -1, (0, 2): -1, (2, 3): -1}
    m = ModelSpec(name="fire3", state_ids=["potential", "count", "adaptation"],
                  parameter_ids=["I", "g", "theta", "a", "r", "sigma"], fixed_parameter_ids=[],
                  observable_ids=["count", "adaptation", "potential"],
                  x0=[sp.Integer(0), sp.Integer(0), sp.Integer(0)], w=w, stoich=stoich,
                  y=[x[1], x[2], x[0]], sigma_y=[sp.Float(0.5), sp.Float(0.05), sg], x=list(x), p=list(p), k=[],
                  p_nominal=[1.5, 0.2, 2.0, 0.3, 0.1, 0.1], k_nominal=[],
                  events=[Event(trigger=x[0] - theta, bolus={0: -x[0], 1: sp.Integer(1), 2: a})])
    m.families = ("fwd", "fsa")
    return m


def fire_workload(n_instances: int = 64, seed: int = 10, simulate=None) -> Workload:
    """Instances of ``fire3``: theta = ln of the nominal values + N(0, 0.1^2);
    40 outputs on [1, 40]; rtol 1e-8, atol 1e-10.  Synthetic data are
    y(theta_nominal) + N(0, 0.05^2), from ``simulate(model, p, pscale, k, ts)
    -> y`` if given."""
    m = fire_model()
    rng = np.random.default_rng(seed)
    theta_true = np.log(np.array(m.p_nominal))
    p = theta_true + rng.normal(0.0, 0.1, (n_instances, m.np))
    ts = np.tile(np.linspace(1.0, 40.0, 40), (n_instances, 1))
    pscale = np.full(m.np, PSCALE_LN, np.int32)
    k = np.zeros((n_instances, 0))
    my = None
    if simulate is not None:
        y = simulate(m, np.tile(theta_true, (n_instances, 1)), pscale, k, ts)
        my = y + np.random.default_rng(seed + 100).normal(0.0, 0.05, y.shape)
    w = Workload("fire3", m, p, pscale, k, ts, my, None, 1e-8, 1e-10, 1)
    w.theta_true = theta_true
    return w


def switch_model() -> ModelSpec:
    """Heaviside functions in the right-hand side: a decaying signal x0
    (rate p0) keeps the production of x1 (rate p1, degradation p3) on while
    it is above the threshold p2 (the flux p1 * Heaviside(x0 - p2)); x1 in
    turn keeps the production of x2 (rate p4) on while it is above p5
    (p4 * Heaviside(x1 - p5)).  Two switches in time: x0 is fed at rate p8
    until t = p9 (p8 * Heaviside(p9 - t)), and the degradation of x2 (rate
    p6) doubles from t = p7 on (p6 * x2 * (1 + Heaviside(t - p7))).  From
    x = (1, 0, 0): x0's feed stops, x1 crosses p5 upwards, x0 falls below p2,
    x1 falls below p5 and x2's degradation steps up: switches of the states
    located by root finding in both directions, and of time at explicit
    trigger times in both directions.  Observables x0, x1, x2 with sigma
    0.1."""
    x = sp.symbols("x0:3", real=True)
    p = sp.symbols("p0:10", real=True)
    t = TIME
    w = [p[0] * x[0], p[1] * sp.Heaviside(x[0] - p[2]), p[3] * x[1], p[4] * sp.Heaviside(x[1] - p[5]),
         p[6] * x[2] * (1 + sp.Heaviside(t - p[7])), p[8] * sp.Heaviside(p[9] - t)]
    stoich = {(0, 0): -1, (0, 5): 1, (1, 1): 1, (1, 2): -1, (2, 3): 1, (2, 4): -1}
    m = ModelSpec(name="switch3", state_ids=["signal", "response", "readout"],
                  parameter_ids=["k_decay", "k_on", "threshold_signal", "k_deg", "k_read", "threshold_response",
                                 "k_read_deg", "t_step", "k_feed", "t_feed"], fixed_parameter_ids=[],
                  observable_ids=["signal", "response", "readout"],
                  x0=[sp.Integer(1), sp.Integer(0), sp.Integer(0)], w=w, stoich=stoich,
                  y=[x[0], x[1], x[2]], sigma_y=[sp.Float(0.1)] * 3, x=list(x), p=list(p), k=[],
                  p_nominal=[0.3, 1.0, 0.2, 0.5, 1.0, 0.8, 0.4, 12.0, 0.5, 2.0], k_nominal=[])
    m.families = ("fwd", "fsa")
    return m


def switch_workload(n_instances: int = 64, seed: int = 12, simulate=None) -> Workload:
    """Instances of ``switch3``: theta = ln of the nominal values + N(0,
    0.1^2); 40 outputs on [0.5, 20]; rtol 1e-8, atol 1e-10.  Synthetic data
    are y(theta_nominal) + N(0, 0.1^2), from ``simulate(model, p, pscale, k,
    ts) -> y`` if given."""
    m = switch_model()
    rng = np.random.default_rng(seed)
    theta_true = np.log(np.array(m.p_nominal))
    p = theta_true + rng.normal(0.0, 0.1, (n_instances, m.np))
    ts = np.tile(np.linspace(0.5, 20.0, 40), (n_instances, 1))
    pscale = np.full(m.np, PSCALE_LN, np.int32)
    k = np.zeros((n_instances, 0))
    my = None
    if simulate is not None:
        y = simulate(m, np.tile(theta_true, (n_instances, 1)), pscale, k, ts)
        my = y + np.random.default_rng(seed + 100).normal(0.0, 0.1, y.shape)
    w = Workload("switch3", m, p, pscale, k, ts, my, None, 1e-8, 1e-10, 1)
    w.theta_true = theta_true
    return w
