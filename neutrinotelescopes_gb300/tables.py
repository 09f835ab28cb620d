"""Training tables for the arrival-time flow, generated by the MC kernel
(scripts/photon_tables.jl:52-230 of chrhck/NeutrinoTelescopes).

``make_flow_table`` draws simulations (distance log-uniform, source direction
isotropic relative to the module -> source axis, log10 E uniform), propagates
all of them in ONE launch around a single multi-PMT module (one source per
simulation, photons oversampled towards a target hit count and weighted back
to the source's light yield), weights the hits (calc_total_weight!) and calls
``ntp_make_table``: R random module orientations per simulation, PMT
assignment, per-(simulation, orientation, PMT) resampling and row output --
all on the device.  The table stays in device memory (torch CUDA tensors) and
feeds ``RQNormFlow.fit_table`` directly; ``FlowTable.save`` / ``load`` keep it
on disk as a NumPy ``.npz`` archive (the reference writes HDF5 groups with the
labels as attributes; here each row carries its condition).
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import _abi
from .detection import MultiPMTDetector, make_pom_pmt_coordinates
from .lightyield import ExtendedCherenkovEmitter, LongitudinalParameterisation
from .medium import make_simple_water
from .photon_prop import PhotonPropSetup, _check, pack_sources
from .spectrum import InverseSquareSpectrum

PMT_AREA = float(np.pi * (75e-3 / 2) ** 2)


@dataclass
class TableConfig:
    n_sims: int = 1024
    n_orientations: int = 16            # n_resample of run_sim (100 there)
    max_rows_per_group: int = 200       # create_pmt_table's limit
    zero_rows: bool = True              # count-only rows for groups without hits
    distance: tuple = (1.0, 200.0)      # m, log-uniform
    log10_energy: tuple = (2.0, 6.0)
    photons_per_gev: float = 1.3e5
    target_hits: float = 1000.0         # simulated hits aimed at per simulation
    min_photons: int = 100_000
    max_photons: int = 50_000_000
    downsample: float = 1.0
    module_radius: float = 0.21
    seed: int = 7
    # a fraction of the simulations drawn from a narrower region instead
    # (distance log-uniform over focus_distance, cos theta of the source
    # direction uniform over focus_cos_theta): the light of an event comes
    # mostly from modules 10-60 m away near the Cherenkov angle (the source
    # direction's cos theta about -0.74 relative to the module -> source
    # axis), where a uniform table holds few simulations.  The flow is
    # conditional on the features, so where its data lie moves its accuracy
    # but does not bias it.
    focus_fraction: float = 0.0
    focus_distance: tuple = (8.0, 80.0)
    focus_cos_theta: tuple = (-0.95, -0.5)


@dataclass
class FlowTable:
    """Rows (cond [n x 5], tres, nhits, has_time) and per-group truth
    (group_cond [G x 5], group_expec = sum of weights, group_count = drawn N),
    G = n_sims x n_orientations x 16 PMTs, as torch tensors on one device."""
    cond: object
    tres: object
    nhits: object
    has_time: object
    group_cond: object
    group_expec: object
    group_count: object
    n_photons: int = 0
    n_hits: int = 0
    meta: dict = field(default_factory=dict)
    row_group: object = None   # group index of every row
    sim_scale: object = None   # per simulation: emitted / simulated photons (the weight scale of its hits)

    def __len__(self) -> int:
        return int(self.tres.shape[0])

    def count_once_weights(self):
        """Per-row weights 1 / (rows of the row's group): with them each
        group's count term enters a training loss once (float32, device)."""
        import torch
        if self.row_group is None:
            raise ValueError("the table has no row_group")
        rg = self.row_group.long()
        n = torch.bincount(rg, minlength=int(self.group_cond.shape[0]))
        return (1.0 / n[rg].to(torch.float32)).contiguous()

    def information_weights(self):
        """Per-row count weights and count targets of the information-weighted
        count loss: (weight, target) float32 tensors on the table's device.

        A group's MC expectation is its simulation's weighted hits times the
        simulation's scale s (emitted / simulated photons), so its variance
        is about s times the expectation: the group's information on log
        lambda is the expectation / s, its simulated (weighted) hits.  The
        Poisson term c (N log lambda - lambda) with c = 1 / s and N = the
        expectation has exactly that curvature at its minimum, so each group
        pulls on the fit in proportion to the hits simulated for it, instead
        of in proportion to lambda, which spans about ten decades over the
        table (the reference's per-row Poisson term, dominated by the
        brightest PMTs).  Each group enters once (its c is split over its
        rows); the c are scaled to a mean of 1 over the groups, so the count
        term's total weight equals count_once's.  The target is the
        expectation itself rather than a Poisson draw of it, which would add
        noise on top of the simulation's own."""
        import torch
        if self.row_group is None or self.sim_scale is None:
            raise ValueError("the table needs row_group and sim_scale")
        G = int(self.group_cond.shape[0])
        S = int(self.sim_scale.shape[0])
        if S == 0 or G % S:
            raise ValueError(f"{G} groups do not split into {S} simulations")
        dev = self.row_group.device
        c_sim = 1.0 / torch.as_tensor(self.sim_scale, dtype=torch.float64, device=dev)
        c = c_sim.repeat_interleave(G // S)
        c = c / c.mean()
        rg = self.row_group.long()
        rows = torch.bincount(rg, minlength=G).to(torch.float64)
        w = (c[rg] / rows[rg]).to(torch.float32).contiguous()
        target = self.group_expec.to(dev)[rg].to(torch.float32).contiguous()
        return w, target

    def save(self, path) -> None:
        np.savez(path, **{k: getattr(self, k).cpu().numpy() for k in
                          ("cond", "tres", "nhits", "has_time", "group_cond", "group_expec", "group_count",
                           "row_group", "sim_scale") if getattr(self, k) is not None},
                 n_photons=self.n_photons, n_hits=self.n_hits,
                 meta=np.array([repr(sorted(self.meta.items()))]))

    @classmethod
    def load(cls, path, device="cuda") -> "FlowTable":
        import torch
        z = np.load(path)
        t = {k: torch.as_tensor(z[k]).to(device) for k in
             ("cond", "tres", "nhits", "has_time", "group_cond", "group_expec", "group_count", "row_group",
              "sim_scale") if k in z.files}
        return cls(**t, n_photons=int(z["n_photons"]), n_hits=int(z["n_hits"]))


def random_rotations(n: int, rng: np.random.Generator) -> np.ndarray:
    """n uniformly distributed rotation matrices [n x 3 x 3] (unit quaternions
    from a normal 4-vector)."""
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
        np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
        np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1),
    ], axis=1)


def draw_simulations(cfg: TableConfig, rng: np.random.Generator):
    """Simulation parameters: distance, cos theta and phi of the source
    direction (around the module -> source axis +z), log10 E, and the
    emitters: source at (0, 0, d), photons oversampled towards target_hits."""
    S = cfg.n_sims
    d = np.exp(rng.uniform(np.log(cfg.distance[0]), np.log(cfg.distance[1]), S))
    ct = rng.uniform(-1.0, 1.0, S)
    phi = rng.uniform(0.0, 2 * np.pi, S)
    le = rng.uniform(cfg.log10_energy[0], cfg.log10_energy[1], S)
    if cfg.focus_fraction > 0:
        f = rng.uniform(0.0, 1.0, S) < cfg.focus_fraction
        nf = int(f.sum())
        d[f] = np.exp(rng.uniform(np.log(cfg.focus_distance[0]), np.log(cfg.focus_distance[1]), nf))
        ct[f] = rng.uniform(cfg.focus_cos_theta[0], cfg.focus_cos_theta[1], nf)
    st = np.sqrt(1.0 - ct * ct)
    dirs = np.stack([st * np.cos(phi), st * np.sin(phi), ct], -1)
    e = 10.0 ** le
    n_true = cfg.photons_per_gev * e
    # geometric hit probability of a module of radius R at distance d
    p_hit = np.minimum(0.5, cfg.module_radius ** 2 / (4.0 * d * d))
    n_sim = np.clip(np.ceil(cfg.target_hits / p_hit), cfg.min_photons, cfg.max_photons).astype(np.int64)
    sources = []
    for i in range(S):
        lp = LongitudinalParameterisation(a=float(np.float32(2.0 + 0.6 * np.log(e[i]))), b=0.63, lrad=0.36)
        sources.append(ExtendedCherenkovEmitter((0.0, 0.0, float(d[i])), tuple(dirs[i]), 0.0, int(n_sim[i]), lp))
    scale = n_true / n_sim
    return dict(distance=d, cos_theta=ct, phi=phi, log10_energy=le, sources=sources, weight_scale=scale,
                n_simulated=n_sim)


def table_setup(cfg: TableConfig, medium=None, spectrum=None) -> PhotonPropSetup:
    module = MultiPMTDetector((0.0, 0.0, 0.0), cfg.module_radius, PMT_AREA, make_pom_pmt_coordinates(), 1)
    return PhotonPropSetup([], [module], medium or make_simple_water(),
                           spectrum or InverseSquareSpectrum(300.0, 600.0))


def propagate_to_device(setup: PhotonPropSetup, seed: int, capacity: int | None = None):
    """Propagates setup.sources with the hits kept on the device; returns
    (hits as a torch uint8 tensor of 64-byte records, n_hits, n_photons)."""
    import torch
    lib, ctx = setup.context()
    srcs = pack_sources(setup.sources)
    total = sum(int(s.photons) for s in setup.sources)
    cap = int(capacity or max(1 << 16, total // 2000))
    opts = setup.prop_opts()
    while True:
        buf = torch.empty(cap * 64, dtype=torch.uint8, device=f"cuda:{setup.device}")
        torch.cuda.synchronize()
        n_hits, n_sim = C.c_uint64(), C.c_uint64()
        st = lib.ntp_propagate(ctx, srcs, len(setup.sources), C.c_uint64(seed & (2 ** 64 - 1)), C.byref(opts),
                               buf.data_ptr(), cap, 1, C.byref(n_hits), C.byref(n_sim))
        if st == _abi.NTP_ERR_OVERFLOW:
            cap = int(n_hits.value)
            continue
        _check(lib, ctx, st)
        return buf, int(n_hits.value), int(n_sim.value)


def make_flow_table(cfg: TableConfig | None = None, medium=None, spectrum=None, setup=None) -> FlowTable:
    """Generates a training table on the device (see the module docstring)."""
    import torch
    cfg = cfg or TableConfig()
    rng = np.random.default_rng(cfg.seed)
    sims = draw_simulations(cfg, rng)
    setup = setup or table_setup(cfg, medium, spectrum)
    setup.sources = sims["sources"]
    lib, ctx = setup.context()
    dev = f"cuda:{setup.device}"
    hits, n, n_phot = propagate_to_device(setup, seed=cfg.seed)
    w = torch.empty(max(n, 1), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    _check(lib, ctx, lib.ntp_calc_total_weight(ctx, hits.data_ptr(), n, None, None, None, w.data_ptr(), 1, None))
    R = cfg.n_orientations
    orient = np.ascontiguousarray(random_rotations(cfg.n_sims * R, rng).reshape(-1), dtype=np.float64)
    n800 = float(np.float32(np.asarray(setup.medium.refractive_index(np.array([800.0])))[0]))
    spec = _abi.NtpTableSpec(n_sims=cfg.n_sims, n_orientations=R, max_rows_per_group=cfg.max_rows_per_group,
                             zero_rows=int(cfg.zero_rows), downsample=cfg.downsample, n800=n800,
                             seed=cfg.seed & (2 ** 64 - 1))
    srcs = pack_sources(setup.sources)
    le = np.ascontiguousarray(sims["log10_energy"], dtype=np.float32)
    scale = np.ascontiguousarray(sims["weight_scale"], dtype=np.float64)
    P = 16
    G = cfg.n_sims * R * P
    gcond = torch.empty((G, 5), dtype=torch.float32, device=dev)
    gexp = torch.empty(G, dtype=torch.float64, device=dev)
    gcnt = torch.empty(G, dtype=torch.int64, device=dev)
    ghit = torch.empty(G, dtype=torch.int64, device=dev)
    cap = max(G + n, 1)
    dp = C.POINTER(C.c_double)
    while True:
        cond = torch.empty((cap, 5), dtype=torch.float32, device=dev)
        tres = torch.empty(cap, dtype=torch.float32, device=dev)
        nh = torch.empty(cap, dtype=torch.float32, device=dev)
        has = torch.empty(cap, dtype=torch.int32, device=dev)
        rg = torch.empty(cap, dtype=torch.int32, device=dev)
        torch.cuda.synchronize()
        n_rows = C.c_uint64()
        st = lib.ntp_make_table(ctx, hits.data_ptr(), n, w.data_ptr(), srcs, _abi.fptr(le), scale.ctypes.data_as(dp),
                                orient.ctypes.data_as(dp), C.byref(spec), cond.data_ptr(), tres.data_ptr(),
                                nh.data_ptr(), has.data_ptr(), rg.data_ptr(), cap, C.byref(n_rows), gcond.data_ptr(),
                                gexp.data_ptr(), gcnt.data_ptr(), ghit.data_ptr(), None)
        if st == _abi.NTP_ERR_OVERFLOW:
            cap = int(n_rows.value)
            continue
        _check(lib, ctx, st)
        break
    m = int(n_rows.value)
    meta = dict(n_sims=cfg.n_sims, n_orientations=R, seed=cfg.seed, photons_per_gev=cfg.photons_per_gev)
    table = FlowTable(cond[:m], tres[:m], nh[:m], has[:m], gcond, gexp, gcnt, n_phot, n, meta, rg[:m],
                      torch.as_tensor(scale, device=dev))
    table.sims = sims
    table.hits = hits[: n * 64]
    table.weights = w[:n]
    table.orientations = orient.reshape(-1, 3, 3)
    table.group_hits = ghit
    return table


def flow_condition(distance, cos_theta_src, cos_theta_pmt, phi, log10_energy) -> np.ndarray:
    """The table's condition features for given geometry (the mapping of
    ntp_make_table; the same as neutrinotelescopes_gb300.flow.flow_features)."""
    from .flow import flow_features
    return flow_features(distance, cos_theta_src, cos_theta_pmt, phi, log10_energy)


def expected_hits_mc(table: FlowTable) -> np.ndarray:
    """Per group the MC expectation sum(w) (the truth the count head learns)."""
    return table.group_expec.cpu().numpy()


def poisson_nll(n: np.ndarray, log_lambda: np.ndarray) -> float:
    lam = np.exp(log_lambda)
    return float(np.mean(lam - n * log_lambda + np.array([math.lgamma(v + 1.0) for v in n])))
