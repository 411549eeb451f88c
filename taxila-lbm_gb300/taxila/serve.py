"""Request server for pore-scale solves on one GPU (continuous batching).

Requests (single-phase permeability solves and two-phase drainage runs of
different sizes) arrive over time.  The server admits a request as soon as
its lattice fits in the device-memory budget, into the batch of its kernel
form (tx_batch_*: one persistent tile-table launch per kernel for all
lattices of that form, replayed as a CUDA graph); batches of different forms
run on their own CUDA streams, so their work overlaps.  Every batch advances
in chunks of ``chunk`` steps; after each chunk the server probes every
lattice and retires the ones whose stop criterion holds:

* permeability: the mean flow (sum of u_z over pore sites) changed by at
  most tol relative over the last chunk (criterion="mean", the default), or
  max |u - u_prev| <= tol * max |u| over pore sites (criterion="max"; with
  FP16 storage the per-site rounding noise can keep this above small tol),
  or max_steps;
* drainage: the invading component's mass (the sum of its density over pore
  sites, from the same device probe) changed by at most tol relative over
  the last chunk (the saturation has levelled off: breakthrough, or a front
  held by capillary entry pressure), or max_steps.

Admission happens only between chunks, so every lattice is probed at
multiples of ``chunk`` of its own steps: its result does not depend on what
else was in flight (the populations equal those of the same request served
alone bit for bit).

The sequential plain-FP64 reference is the same server with the FP64 form and
one request in flight at a time.
"""
import dataclasses
import time

import numpy as np

from . import metrics
from . import params as P
from . import problems
from ._lib import Batch


@dataclasses.dataclass
class Request:
    rid: int
    kind: str              # "perm" or "drain"
    arrival: float         # seconds after the start of the run
    params: object         # TxParams (precision is set by the server)
    walls: np.ndarray
    rho: np.ndarray
    tol: float = 1e-5      # permeability stop criterion
    max_steps: int = 20000
    # drainage bookkeeping: invading component and its bulk densities
    invader: int = 0
    lo: float = 0.06
    hi: float = 2.0
    conc: object = None    # passive-species concentrations [N*ns] (drainage tracer)


@dataclasses.dataclass
class Result:
    rid: int
    kind: str
    sites: int
    steps: int
    arrival: float
    admitted: float
    finished: float
    value: float           # permeability (perm) or saturation of the invader (drain)
    front: float = 0.0     # drainage: mean front position (lattice units)
    tracer: float = 0.0    # drainage: mean position of the tracer along the flow axis

    @property
    def latency(self):
        return self.finished - self.arrival


def form_key(p):
    return (p.discretization, p.ncomponents, p.relaxation_mode, p.isotropy_order, p.precision, p.nspecies,
            p.species_relaxation_mode)


def _random_sides(rng, lo, hi, n):
    return [int(v) for v in rng.integers(lo, hi + 1, size=n)]


def perm_request(rid, arrival, sides, seed, tol, max_steps, gz=1e-5, radii=None):
    """Single-phase D3Q19 BGK (tau = 1) periodic sphere pack, body force along z.
    Porosity uniform in [0.25, 0.5]; sphere radii uniform in ``radii``
    (default [4, 10] scaled by the smallest side / 48)."""
    rng = np.random.default_rng(seed)
    nz, ny, nx = sides
    p = P.default_params()
    p.discretization = P.D3Q19
    p.nx, p.ny, p.nz = nx, ny, nz
    p.ncomponents = 1
    p.relaxation_mode = P.SRT
    p.isotropy_order = 4
    for f in range(6):
        p.bc_flags[f] = P.BC_PERIODIC
    p.tau[0] = 1.0
    p.nminerals = 1
    p.body_forces = 1
    p.gvt[2] = gz
    p.rho0[0] = 1.0
    if radii is None:
        scale = min(sides) / 48.0
        radii = (max(1.5, 4.0 * scale), max(2.0, 10.0 * scale))
    rmin, rmax = radii
    phi = float(rng.uniform(0.25, 0.5))
    solid = problems.sphere_pack((nz, ny, nx), phi, rmin, rmax, seed, periodic=True)
    walls = np.where(solid.ravel(), 1.0, 0.0)
    return Request(rid, "perm", arrival, p, walls, np.ones(p.nsites), tol=tol, max_steps=max_steps)


def drain_request(rid, arrival, sides, seed, steps, dims=3, tol=0.0):
    """Two-phase drainage: D3Q19 (or D2Q9) two-component BGK (tau = 1),
    seeded sphere (disk) pack of porosity 0.35 split into two minerals with
    adhesion (+a, -a) / (-a, +a); the pore starts with the wetting component 1
    (bulk density 1, the other 0.03); the non-wetting component 0 enters
    through a density face at the low end of the flow axis (rho 1.05, first
    three slices pre-filled) against the wetting phase at the high end (rho
    0.95); walls on the other axes.  One passive tracer species (tau_s =
    0.8) starts at concentration 1 where the injected phase is.  g_12 = 0.04
    and a = 0.03: with the stronger coupling g_12 = 0.15, adhesion 0.3 and
    densities 2.1 / 1.9 the reference algorithm (the FP64 oracle) diverges
    within 50 steps on small packs, and g_12 = 0.06, a = 0.05 diverge at the
    inlet-face corner after ~2,500 steps on a 256^3 pack; 0.04 / 0.03 stay
    stable there."""
    p = P.default_params()
    if dims == 3:
        nz, ny, nx = sides
        p.discretization = P.D3Q19
        p.nx, p.ny, p.nz = nx, ny, nz
        axis, shape = 2, (nz, ny, nx)
    else:
        ny, nx = sides
        p.discretization = P.D2Q9
        p.nx, p.ny, p.nz = nx, ny, 1
        axis, shape = 1, (1, ny, nx)
    p.ncomponents = 2
    p.relaxation_mode = P.SRT
    p.isotropy_order = 4
    p.tau[0] = p.tau[1] = 1.0
    p.g[0][1] = p.g[1][0] = 0.04
    p.nminerals = 2
    p.gw[0][0], p.gw[0][1] = 0.03, -0.03
    p.gw[1][0], p.gw[1][1] = -0.03, 0.03
    p.bc_flags[2 * axis] = P.BC_DENSITY
    p.bc_flags[2 * axis + 1] = P.BC_DENSITY
    p.bc_data[2 * axis][0], p.bc_data[2 * axis][1] = 1.05, 0.03
    p.bc_data[2 * axis + 1][0], p.bc_data[2 * axis + 1][1] = 0.03, 0.95
    rmin, rmax = max(2.0, min(sides) / 12.0), max(3.0, min(sides) / 6.0)
    if dims == 3:
        solid = problems.sphere_pack(shape, 0.35, rmin, rmax, seed, periodic=False)
    else:
        solid = problems.sphere_pack((1, ny, nx), 0.35, rmin, rmax, seed, periodic=False)
    # keep the inlet and outlet slices open
    sl = [slice(None)] * 3
    sl[2 - axis] = slice(0, 2)
    solid[tuple(sl)] = False
    sl[2 - axis] = slice(shape[2 - axis] - 2, None)
    solid[tuple(sl)] = False
    walls = problems.mineral_walls(solid, seed)
    pore = walls == 0
    inlet = np.indices(shape)[2 - axis].ravel() < 3
    rho = np.empty((p.nsites, 2))
    rho[:, 0] = np.where(pore, np.where(inlet, 1.05, 0.03), 0.0)
    rho[:, 1] = np.where(pore, np.where(inlet, 0.03, 1.0), 0.0)
    p.nspecies = 1
    p.species_relaxation_mode = P.SRT
    p.species_tau[0] = 0.8
    conc = np.where(pore & inlet, 1.0, 0.0)
    return Request(rid, "drain", arrival, p, walls, rho.ravel(), tol=tol, max_steps=steps, invader=0, lo=0.03, hi=1.05,
                   conc=conc)


def make_mix(seed=1, n=40, rate=30.0, perm_sides=(32, 64), drain3_sides=(32, 48), drain2_sides=(96, 192),
             frac_perm=0.7, perm_tol=1e-5, perm_max_steps=6000, drain_steps=1500, drain_tol=0.0, perm_radii=None,
             perm_gz=1e-5):
    """Seeded Poisson request stream: ``n`` requests at ``rate`` per second,
    70% permeability solves and 30% drainage runs (half D3Q19, half D2Q9),
    sides uniform in the given ranges (per axis for the 3D lattices)."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    for i in range(n):
        t += float(rng.exponential(1.0 / rate))
        s = int(rng.integers(0, 1 << 30))
        u = rng.random()
        if u < frac_perm:
            out.append(perm_request(i, t, _random_sides(rng, *perm_sides, 3), s, perm_tol, perm_max_steps,
                                    gz=perm_gz, radii=perm_radii))
        elif u < frac_perm + (1.0 - frac_perm) / 2:
            out.append(drain_request(i, t, _random_sides(rng, *drain3_sides, 3), s, drain_steps, dims=3, tol=drain_tol))
        else:
            out.append(drain_request(i, t, _random_sides(rng, *drain2_sides, 2), s, drain_steps, dims=2, tol=drain_tol))
    return out


# The serving mix of the workload specification: 70% single-phase
# permeability solves, sides 32-160 per axis, sphere radii 4-10, body force
# 1e-6, run to a relative change of the mean flow below 1e-7 per 100-step
# chunk; 30%
# two-phase drainage with two minerals and one tracer, D2Q9 256^2-1024^2 or
# D3Q19 64^3-128^3, run until the invader's mass changes by less than 1e-4
# per chunk; Poisson arrivals at 30 per second.  The step caps bound a
# request whose criterion is never met.
SPEC_MIX = dict(rate=30.0, perm_sides=(32, 160), drain3_sides=(64, 128), drain2_sides=(256, 1024), frac_perm=0.7,
                perm_tol=1e-7, perm_max_steps=20000, drain_steps=6000, drain_tol=1e-4, perm_radii=(4.0, 10.0),
                perm_gz=1e-6)


def make_spec_mix(n, seed=1, **overrides):
    """``n`` requests of the specification's mix (SPEC_MIX, with overrides)."""
    kw = dict(SPEC_MIX)
    kw.update(overrides)
    return make_mix(seed=seed, n=n, **kw)


class Server:
    """Continuous-batching server over one GPU.

    precision: the kernel form of every request (P.PREC_*); storage_scale:
    the FP16 storage scale; budget_bytes: device memory for lattices;
    max_active: requests in flight at once (None: as many as fit)."""

    def __init__(self, precision=P.PREC_F32_F16, storage_scale=4096.0, budget_bytes=150 << 30, chunk=100,
                 graph_steps=20, max_active=None, tiles=None, criterion="mean"):
        if criterion not in ("mean", "max"):
            raise ValueError("criterion must be 'mean' or 'max'")
        self.criterion = criterion
        self.precision = precision
        self.storage_scale = storage_scale
        self.budget = int(budget_bytes)
        self.chunk = int(chunk)
        self.graph_steps = graph_steps
        self.max_active = max_active
        self.tiles = tiles
        self.batches = {}

    def _params(self, req):
        q = P.copy_params(req.params)
        q.precision = self.precision
        q.exact = 0
        q.storage_scale = self.storage_scale if req.kind == "perm" else 1.0
        if req.kind == "drain":
            # two phases: no single rest density; plain storage (FP16 relative to each value)
            for m in range(P.MAXC):
                q.rho0[m] = 0.0
        return q

    def _batch(self, q):
        key = form_key(q)
        b = self.batches.get(key)
        if b is None:
            b = Batch(q)
            if self.graph_steps is not None:
                b.set_graph(self.graph_steps)
            if self.tiles:
                b.set_tiles(*self.tiles)
            self.batches[key] = b
        return key, b

    def in_use(self):
        return sum(b.bytes_in_use() for b in self.batches.values())

    def run(self, requests, realtime=True):
        """Serve ``requests`` (arrival times in seconds from now); returns the
        results in completion order.  realtime=False admits every request at
        once (arrival times only order them)."""
        pending = sorted(requests, key=lambda r: (r.arrival, r.rid))
        active, results = {}, []
        t0 = time.perf_counter()

        def now():
            return time.perf_counter() - t0

        while pending or active:
            t = now()
            # admission: first fit in arrival order among the arrived requests
            for req in list(pending):
                if realtime and req.arrival > t:
                    break
                if self.max_active is not None and len(active) >= self.max_active:
                    break
                q = self._params(req)
                need = Batch.lattice_bytes(q)
                if need > self.budget:
                    raise ValueError("request %d needs %d bytes, over the whole budget" % (req.rid, need))
                if self.in_use() + need > self.budget:
                    continue
                key, b = self._batch(q)
                lid = b.add(q, req.walls, req.rho, conc=req.conc)
                active[(key, lid)] = [req, q, now(), None]
                pending.remove(req)
            if not active:
                if pending and realtime:
                    time.sleep(max(0.0, min(pending[0].arrival - now(), 0.05)))
                continue
            busy = [b for b in self.batches.values() if b.count()]
            for b in busy:
                b.launch(self.chunk)
            for b in busy:
                b.sync()
            for key, b in list(self.batches.items()):
                if not b.count():
                    continue
                for lid, pr in b.probe().items():
                    slot = active[(key, lid)]
                    req, q, admitted, prev = slot
                    # the probed quantity of the stop criterion: mean flow or invader mass
                    cur = pr.u_sum[2] if req.kind == "perm" else pr.mass[req.invader]
                    slot[3] = cur
                    done = pr.steps >= req.max_steps
                    if req.kind == "perm":
                        if self.criterion == "max":
                            done = done or (pr.u_max > 0.0 and pr.du_max <= req.tol * pr.u_max)
                        elif prev is not None and cur != 0.0:
                            done = done or abs(cur - prev) <= req.tol * abs(cur)
                    elif req.tol > 0.0 and prev is not None and cur != 0.0:
                        done = done or abs(cur - prev) <= req.tol * abs(cur)
                    if not done:
                        continue
                    tracer = 0.0
                    if req.kind == "perm":
                        value = (q.tau[0] - 0.5) / 3.0 * (pr.u_sum[2] / q.nsites) / q.gvt[2]
                        front = 0.0
                    else:
                        if q.nspecies > 0:
                            c = b.download(lid, P.FIELD_SPECIES_RHO, q.nsites * q.nspecies)[::q.nspecies]
                            axis = 0 if q.discretization == P.D3Q19 else 1
                            pos = np.indices(q.shape)[axis].ravel()
                            tracer = float((c * pos).sum() / max(c.sum(), 1e-300))
                        rho = b.download(lid, P.FIELD_RHO, q.nsites * q.ncomponents)
                        value = metrics.saturation(rho, 2, req.invader, req.lo, req.hi, req.walls)
                        shape = q.shape
                        front = metrics.front_position(rho, shape, 2, req.invader, req.lo, req.hi, req.walls) \
                            if q.discretization == P.D3Q19 else 0.0
                    b.remove(lid)
                    del active[(key, lid)]
                    # without real-time arrivals every request is queued at t = 0
                    results.append(Result(req.rid, req.kind, q.nsites, int(pr.steps),
                                          req.arrival if realtime else 0.0, admitted, now(),
                                          float(value), float(front), tracer))
        return results

    def close(self):
        for b in self.batches.values():
            b.close()
        self.batches = {}


def summary(results, makespan=None):
    """solves/s over the makespan, latency percentiles, site-steps per second."""
    if not results:
        return {}
    lat = np.array([r.latency for r in results])
    span = makespan if makespan is not None else max(r.finished for r in results) - min(r.arrival for r in results)
    lups = sum(r.sites * r.steps for r in results)
    return {"solves": len(results), "makespan_s": round(span, 3), "solves_per_s": round(len(results) / span, 3),
            "p50_s": round(float(np.percentile(lat, 50)), 4), "p99_s": round(float(np.percentile(lat, 99)), 4),
            "mlups": round(lups / span / 1e6, 1)}
