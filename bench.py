"""Benchmark: D3Q19 two-component Shan-Chen step on one GB300 (per rank).

Workload (the reference's 3D bubble benchmark configuration): D3Q19, 128^3
fully periodic, two components, FP64, MRT with s_nu = 1/tau (tau_A = 1.0,
tau_B = 0.7) and all other rates 1.0, isotropy-4 psi gradient, psi = rho,
component A rho = 2.0 in a centred sphere of radius 24 and 0.06 outside, B
reversed, at rest.  The coupling G = 0.9 is the usual Shan-Chen constant
(F = -G psi grad psi); the reference scales its g_12 by c_0 = 6, so
g_12 = g_21 = G / 6 = 0.15.  Synthetic data: the initial state is generated.

One "step" is one LBM time step of the whole lattice (two kernel launches:
collide+push and density/boundary).  value = MLUPS with the state resident in
HBM (CUDA events on the library's stream); e2e = the same metric through the C
ABI with host buffers (upload walls + initial state, init, per-step steady-state
norm read back to the host, final fi download).  Populations (2 x 637 MB) are
larger than L2, so no flush is needed between steps.

--impl reference times the reference algorithm on the host cores: the
reference's Fortran/PETSc build is not buildable here (no Fortran compiler,
MPI or PETSc 3.6), so its C restatement (oracle/) stands in, OpenMP over all
host threads, on a bounded number of steps of the same lattice.
Multi-GPU (torchrun): replicas only - every rank steps its own lattice; value
sums the ranks' sites and takes the slowest rank's time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(REPO, "taxila-lbm_gb300"), os.path.join(REPO, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

from taxila import params as P  # noqa: E402
from taxila import problems  # noqa: E402

METRIC = "D3Q19 2-phase MLUPS"
UNIT = "MLUPS"
N_SIDE = 128
BYTES_PER_LUP_STEP = 2 * 19 * 2 * 8 + 1   # k_step: read + write 2x19 FP64 populations + mask
BYTES_PER_LUP_DENSITY = 19 * 2 * 8 + 2 * 8 + 1  # k_density: read populations, write rho, mask
# steps of the host-core baseline on the GPU line (about 10 s of CPU work)
CPU_BASELINE_STEPS = 40
# lattices of the batched workload run to convergence, and requests of the
# specification's serving mix, in the default run (each leg about a minute)
CONVERGED_LATTICES = 8
SPEC_REQUESTS = 16


FORMS = {"f64": P.PREC_F64, "f32": P.PREC_F32, "f16": P.PREC_F32_F16}
POP_BYTES = {P.PREC_F64: 8, P.PREC_F32: 4, P.PREC_F32_F16: 2}


def workload_params(precision=P.PREC_F64, n=N_SIDE):
    p = P.default_params()
    p.discretization = P.D3Q19
    p.nx = p.ny = p.nz = n
    p.ncomponents = 2
    p.relaxation_mode = P.MRT
    p.isotropy_order = 4
    for f in range(6):
        p.bc_flags[f] = P.BC_PERIODIC
    p.s_nu[0], p.s_nu[1] = 1.0 / 1.0, 1.0 / 0.7
    p.g[0][1] = p.g[1][0] = 0.9 / 6.0
    p.precision = precision
    p.rho0[0] = p.rho0[1] = 0.0  # two phases: plain storage of the populations
    return p


def workload_state(p):
    rho = problems.bubble_ball_state(p.nx, p.ny, p.nz, 24.0 * p.nx / N_SIDE, [2.0, 0.06], [0.06, 2.0])
    return np.zeros(p.nsites), rho


def peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi clock/throttle samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0 and out.stdout.strip():
                    self.rows.append([c.strip() for c in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 5 + i and r[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def reduce_max(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cpu" if dist.get_backend() == "gloo" else "cuda"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(ms_local, sites_local, steps, ws):
    """Replicas: every rank steps its own lattice of sites_local sites.  The job
    time is the slowest rank's; the value counts the sites of all ranks."""
    ms = reduce_max(ms_local, ws)
    return sites_local * ws * steps / (ms * 1e-3) / 1e6, ms


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def cpu_oracle_mlups(p, walls, rho, steps, threads):
    from oracle import Oracle
    o = Oracle(p, threads=threads)
    o.set_walls(walls)
    o.set_state(rho)
    o.init()
    o.step(1)  # warm
    t0 = time.perf_counter()
    o.step(steps)
    dt = time.perf_counter() - t0
    o.close()
    return p.nsites * steps / dt / 1e6, dt


def cpu_model():
    """Host CPU model name (for the record beside the core count)."""
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                k, _, v = line.partition(":")
                if k.strip() in ("model name", "Model", "CPU part") and v.strip():
                    name = v.strip()
                    if k.strip() == "CPU part":
                        name = {"0xd4f": "Neoverse V2 (Grace)"}.get(name, "Arm CPU part " + name)
                    return name
    except OSError:
        pass
    import platform
    return platform.processor() or platform.machine()


def run_reference(args):
    """The reference algorithm on the host cores: exactly --steps timed steps
    of the full 128^3 lattice after --warmup untimed ones."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import Oracle
    threads = os.cpu_count() or 1
    p = workload_params()
    walls, rho = workload_state(p)
    o = Oracle(p, threads=threads)
    o.set_walls(walls)
    o.set_state(rho)
    o.init()
    o.step(args.warmup)
    t0 = time.perf_counter()
    o.step(args.steps)
    dt = time.perf_counter() - t0
    o.close()
    v = p.nsites * args.steps / dt / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": round(v, 4), "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt * 1e3 / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "D3Q19 128^3 2-component MRT Shan-Chen bubble (r=24, rho 2.0/0.06, G=0.9 -> g_12=0.15), periodic, FP64",
                   "parallelism": "host OpenMP", "l2": "not applicable (CPU)"},
        "cpu_baseline": {"value": round(v, 4), "unit": UNIT, "cores": threads, "cpu": cpu_model(), "kind": "port",
                         "sample": "%d timed steps of the full 128^3 lattice after %d warm-up steps (%.1f s); the "
                                   "reference Fortran/PETSc 3.6 build is not buildable here, its C restatement runs "
                                   "instead" % (args.steps, args.warmup, dt)},
        "e2e": {"value": round(v, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def measure_form(precision, steps, warmup, p=None):
    """Device-timed MLUPS and per-kernel times for one storage form."""
    import torch
    from taxila._lib import Handle
    p = p or workload_params(precision)
    walls, rho = workload_state(p)
    h = Handle(p)
    h.upload_walls(walls)
    h.upload_state(rho)
    h.init()
    h.step(warmup)
    h.sync()
    stream = torch.cuda.ExternalStream(h.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    h.step(steps)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    # per-kernel split on a separate short timed run (events between the two launches)
    h.set_timing(True)
    h.step(min(steps, 20))
    h.sync()
    t_step, t_dens, nl = h.timing()
    h.set_timing(False)
    nk = min(steps, 20)
    res = {"ms_total": ms, "ms_per_step": ms / steps, "mlups": p.nsites * steps / (ms * 1e-3) / 1e6,
           "ms_k_step": t_step / nk, "ms_k_density": t_dens / nk, "kernel": h.kernel_name()}
    h.close()
    return res


def e2e_run(steps, warmup, repeats=5):
    """Through the C ABI with host buffers: upload, init, per-step host norm, final download.

    The timed region is taken ``repeats`` times on one handle; the value is the
    median, with the spread and the median split into upload+init, steps and
    download (each part closed by a stream synchronize, so the split adds up to
    a little more than the unsplit region)."""
    import torch
    from taxila._lib import Handle
    p = workload_params()
    walls, rho = workload_state(p)
    walls_pinned = torch.from_numpy(walls).pin_memory().numpy()
    rho_pinned = torch.from_numpy(rho).pin_memory().numpy()
    fi_out = torch.empty(p.nsites * 2 * 19, dtype=torch.float64).pin_memory().numpy()
    h = Handle(p)
    h.upload_walls(walls_pinned)
    h.upload_state(rho_pinned)
    h.init()
    h.step(warmup)
    h.delta_norm(P.FIELD_RHO)
    h.download(P.FIELD_FI, fi_out)
    h.sync()
    torch.cuda.synchronize()
    whole, parts = [], []
    for _ in range(repeats):
        t0 = time.perf_counter()
        h.upload_walls(walls_pinned)
        h.upload_state(rho_pinned)
        h.init()
        for _ in range(steps):
            h.step(1)
            h.delta_norm(P.FIELD_RHO)
        h.download(P.FIELD_FI, fi_out)
        whole.append(time.perf_counter() - t0)
    for _ in range(repeats):
        t0 = time.perf_counter()
        h.upload_walls(walls_pinned)
        h.upload_state(rho_pinned)
        h.init()
        h.sync()
        t1 = time.perf_counter()
        for _ in range(steps):
            h.step(1)
            h.delta_norm(P.FIELD_RHO)
        h.sync()
        t2 = time.perf_counter()
        h.download(P.FIELD_FI, fi_out)
        t3 = time.perf_counter()
        parts.append((t1 - t0, t2 - t1, t3 - t2))
    h.close()
    dt = statistics.median(whole)
    split = [statistics.median(x[i] for x in parts) * 1e3 for i in range(3)]
    h2d = walls.nbytes + rho.nbytes
    d2h = 8 * steps + fi_out.nbytes
    mlups = [p.nsites * steps / t / 1e6 for t in whole]
    return {"value": p.nsites * steps / dt / 1e6, "unit": UNIT,
            "h2d_bytes_per_step": int(round(h2d / steps)), "d2h_bytes_per_step": int(round(d2h / steps)),
            "repeats": repeats, "min": round(min(mlups), 1), "max": round(max(mlups), 1),
            "ms_upload_init": round(split[0], 3), "ms_steps": round(split[1], 3),
            "ms_download": round(split[2], 3),
            "download_gbs": round(fi_out.nbytes / split[2] / 1e6, 1)}


def traffic_from_profile():
    path = os.path.join(REPO, "profiles", "k_step_d3q19_2c_mrt_fp64_traffic.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["dram_bytes_per_lup"])
    except Exception:
        return None


def bubble_2d_run(steps=1000, check_steps=200):
    """The D2Q9 case the reference runs on its CPU build: two-component
    Shan-Chen bubble, 200 x 200 fully periodic, FP64 BGK with tau = 1 for both
    components, unit molecular masses, psi = rho, G = 0.9 (g_12 = G / c0 =
    0.15), a centred disk of radius 30 at rho 2.0 in 0.06 (B reversed), zero
    velocity, 1,000 steps.  Device-timed MLUPS of the plain FP64 form; the
    oracle on the host cores over the first ``check_steps`` steps (a bounded
    sample), whose densities the device's must match."""
    import torch
    from oracle import Oracle
    from taxila._lib import Handle
    p = P.default_params()
    p.discretization = P.D2Q9
    p.nx = p.ny = 200
    p.nz = 1
    p.ncomponents = 2
    for f in range(4):
        p.bc_flags[f] = P.BC_PERIODIC
    p.g[0][1] = p.g[1][0] = 0.9 / 6.0
    walls = np.zeros(p.nsites)
    rho = problems.bubble_ball_state(p.nx, p.ny, 1, 30.0, [2.0, 0.06], [0.06, 2.0])

    def started():
        h = Handle(p)
        h.upload_walls(walls)
        h.upload_state(rho)
        h.init()
        return h

    h = started()
    h.step(5)
    h.sync()
    stream = torch.cuda.ExternalStream(h.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    h.step(steps)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    h.close()
    g = started()
    g.step(check_steps)
    r_dev = g.download(P.FIELD_RHO)
    g.close()
    threads = os.cpu_count() or 1
    o = Oracle(p, threads=threads)
    o.set_walls(walls)
    o.set_state(rho)
    o.init()
    t0 = time.perf_counter()
    o.step(check_steps)
    dt = time.perf_counter() - t0
    r_ref = o.get(P.FIELD_RHO)
    o.close()
    return {"workload": "D2Q9 200^2 2-component BGK Shan-Chen bubble (r=30, rho 2.0/0.06, G=0.9 -> g_12=0.15), "
                        "periodic, FP64 plain form",
            "steps": steps, "ms_per_step": round(ms / steps, 5),
            "mlups": round(p.nsites * steps / (ms * 1e-3) / 1e6, 2),
            "l2": "populations 5.8 MB stay in L2: MLUPS only, no HBM figure",
            "cpu_oracle": {"mlups": round(p.nsites * check_steps / dt / 1e6, 3), "cores": threads,
                           "sample": "first %d steps (%.1f s)" % (check_steps, dt)},
            "rho_rel_err_vs_oracle_after_%d_steps" % check_steps:
                float(np.max(np.abs(r_dev - r_ref)) / np.max(np.abs(r_ref)))}


def batched_run(n_lat=96, steps=40, seed=4, compare=8, sides=(48, 192)):
    """Many uneven single-phase permeability lattices (D3Q19 BGK tau = 1, sides
    uniform in 48..192 per axis, seeded sphere packs with radii 4..10 and
    porosity 0.25..0.5, periodic, body force 1e-6 along z) in one batch of the
    FP32 form: tile shape from the autotuner, steps replayed as a CUDA graph.
    Every lattice is also stepped alone in a tx_handle (the first ``compare``
    reported on their own as well)."""
    import torch
    from taxila import serve
    from taxila._lib import Batch, Handle
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n_lat):
        dims = [int(v) for v in rng.integers(sides[0], sides[1] + 1, size=3)]
        reqs.append(serve.perm_request(i, 0.0, dims, int(rng.integers(0, 1 << 30)), 1e-7, 10 ** 9, gz=1e-6,
                                       radii=(4.0, 10.0) if sides[0] >= 48 else (2.0, 5.0)))
    form = P.copy_params(reqs[0].params)
    form.precision = P.PREC_F32

    def params_of(r):
        q = P.copy_params(r.params)
        q.precision = P.PREC_F32
        return q

    def timed(b, k):
        stream = torch.cuda.ExternalStream(b.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.launch(k)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1)

    b = Batch(form)
    for r in reqs:
        b.add(params_of(r), r.walls, r.rho)
    sites = sum(r.params.nsites for r in reqs)
    tiles = b.tune(2)
    b.set_graph(20)
    b.step(20)
    ms = timed(b, steps)
    probes = b.probe()
    finite = all(np.isfinite(pr.u_sum[2]) for pr in probes.values())
    b.close()
    # the first lattices batched and one by one
    sub = reqs[:compare]
    sub_sites = sum(r.params.nsites for r in sub)
    bs = Batch(form)
    for r in sub:
        bs.add(params_of(r), r.walls, r.rho)
    bs.set_tiles(*tiles)
    bs.set_graph(20)
    bs.step(20)
    ms_sub = timed(bs, steps)
    bs.close()
    ms_one = 0.0
    ms_all = 0.0
    handles = []
    for i, r in enumerate(reqs):
        h = Handle(params_of(r))
        h.upload_walls(r.walls)
        h.upload_state(r.rho)
        h.init()
        h.step(5)
        h.sync()
        stream = torch.cuda.ExternalStream(h.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        h.step(steps)
        e1.record(stream)
        e1.synchronize()
        if i < compare:
            ms_one += e0.elapsed_time(e1)
        ms_all += e0.elapsed_time(e1)
        handles.append(h)
    # a driver stepping every lattice in turn, one step each, waiting for each
    # (states evicted from L2 between visits, as in the batch)
    t0 = time.perf_counter()
    for _ in range(steps):
        for h in handles:
            h.step(1)
            h.sync()
    ms_rr = (time.perf_counter() - t0) * 1e3
    for h in handles:
        h.close()
    mlups = sites * steps / (ms * 1e-3) / 1e6
    fluid = sum(int(np.count_nonzero(np.asarray(r.walls) == 0)) for r in reqs)
    bpl = 2 * 19 * 4 + 1 + 19 * 4 + 4  # collide-push read+write, mask; density read + write
    return {"workload": "%d single-phase D3Q19 BGK sphere packs, sides %d-%d per axis (%d sites), FP32 form, "
                        "body force 1e-6, periodic" % (n_lat, sides[0], sides[1], sites),
            "steps": steps, "ms_per_step": round(ms / steps, 4), "mlups": round(mlups, 1),
            "mflups_fluid_sites": round(fluid * steps / (ms * 1e-3) / 1e6, 1),
            "gbs_algorithmic": round(mlups * 1e6 * bpl / 1e9, 1), "bytes_per_lup": bpl,
            "tiles": {"bx": tiles[0], "by": tiles[1], "bz": tiles[2], "blocks_per_sm": tiles[3]},
            "graph_steps": 20, "finite": finite,
            "first_%d_batched_mlups" % compare: round(sub_sites * steps / (ms_sub * 1e-3) / 1e6, 1),
            "first_%d_one_by_one_mlups" % compare: round(sub_sites * steps / (ms_one * 1e-3) / 1e6, 1),
            "all_one_by_one_mlups": round(sites * steps / (ms_all * 1e-3) / 1e6, 1),
            "all_round_robin_mlups": round(sites * steps / (ms_rr * 1e-3) / 1e6, 1),
            "one_by_one": "each lattice in its own tx_handle: device time of its steps alone (states of lattices "
                          "under ~80^3 stay in L2; launch gaps not counted), and round robin: wall time of a "
                          "driver stepping every lattice once per round and waiting for it"}


def serving_run(n=30, rate=30.0, seed=1):
    """The request mix of the server (70% permeability solves, sides 32-64,
    stop at 1e-5 relative change of the mean flow; 30% drainage, D3Q19
    32-48 / D2Q9 96-192, 1500 steps) at ``rate`` Poisson arrivals per second,
    served by the FP16-storage and FP32 forms and, one request at a time, by
    the plain FP64 form."""
    from taxila import serve
    reqs = serve.make_mix(seed=seed, n=n, rate=rate)
    out = {"mix": "%d requests, Poisson %.0f/s, seed %d: 70%% permeability (D3Q19 sides 32-64, tol 1e-5 on the "
                  "mean flow), 30%% drainage with one passive tracer (D3Q19 32-48 or D2Q9 96-192, 1500 steps)"
                  % (n, rate, seed)}
    for name, prec, maxa in (("fp32_fp16_storage", P.PREC_F32_F16, None), ("fp32", P.PREC_F32, None),
                             ("fp64_sequential", P.PREC_F64, 1)):
        for mode, realtime in (("", True), ("_saturated", False)):
            srv = serve.Server(precision=prec, max_active=maxa, chunk=100)
            res = srv.run(reqs, realtime=realtime)
            srv.close()
            out[name + mode] = serve.summary(res)
    for mode in ("", "_saturated"):
        f, s = out["fp32_fp16_storage" + mode], out["fp64_sequential" + mode]
        if f and s:
            out["fp16_storage_vs_fp64_sequential_solves" + mode] = round(f["solves_per_s"] / s["solves_per_s"], 2)
    out["saturated"] = "the same requests all queued at once: solves/s is the server's capacity"
    return out


def peaks_run(gpu):
    """Measured issue rates of the FP64 (DFMA, DADD, DMUL) and FP32 (FFMA,
    packed FFMA2) pipes over the whole GPU, with the SM clock sampled during
    the probes: G operations per second and lanes per SM per cycle."""
    import torch
    from taxila import peaks
    sms = torch.cuda.get_device_properties(gpu).multi_processor_count
    with Clocks(gpu) as clk:
        rates = peaks.pipe_rates(sms)
    c = clk.summary()
    mhz = c["sm_mhz"] or c["sm_max_mhz"]
    out = {"sms": sms, "clocks": c, "unit": "G operations/s (DFMA/FFMA: one FMA per operation)"}
    for op, r in rates.items():
        out[op] = {"g_per_s": round(r["ops_per_s"] / 1e9, 2), "ms_per_launch": round(r["ms_per_launch"], 3),
                   "per_sm_per_cycle": round(peaks.per_sm_cycle(r["ops_per_s"], sms, mhz), 3) if mhz else None}
    out["fp64_tflops_dfma"] = round(2 * rates["dfma"]["ops_per_s"] / 1e12, 3)
    return out


def fp64_counts():
    """FP64 instructions per lattice site of the FP64 k_step, from its ncu capture."""
    with open(os.path.join(REPO, "profiles", "k_step_d3q19_2c_mrt_fp64_instr.json")) as f:
        return json.load(f)


def fp64_bound(pk, sites, k_ms):
    """k_step of the FP64 form against the measured FP64 pipe: the time its
    FP64 instructions need at the probes' rates, as a fraction of the
    kernel's event-timed duration."""
    c = fp64_counts()
    n = {op: c["per_site"][op] for op in ("dadd", "dfma", "dmul")}
    t_pipe = sum(sites * n[op] / (pk[op]["g_per_s"] * 1e9) for op in n)
    instr = sum(n.values())
    return {"pipe": "fp64", "fp64_instr_per_lup": instr, "per_lup": n,
            "fp64_flop_per_lup": n["dadd"] + n["dmul"] + 2 * n["dfma"],
            "achieved_g_instr_per_s": round(sites * instr / (k_ms * 1e-3) / 1e9, 1),
            "peak_g_instr_per_s": round(pk["dfma"]["g_per_s"], 1),
            "frac": round(t_pipe / (k_ms * 1e-3), 4),
            "peak_source": "measured (peaks: DFMA/DADD/DMUL probes, this run)",
            "counts_source": c["source"]}


def batched_converged_run(n_lat=16, seed=4):
    """A bounded subset of the batched-permeability workload run to its stop
    criterion (relative change of the mean flow < 1e-7 per 100-step chunk):
    the first ``n_lat`` lattices of the 96 (sides 48-192, sphere packs, body
    force 1e-6), one batch per form; time to solution and the permeability
    errors of the FP32 and FP16-storage forms against the FP64 form."""
    from taxila import precision
    r = precision.batch_permeability_study(n_lat, seed)
    return {"case": r["case"], "forms": r["forms"]}


def serving_spec_run(n=40, seed=1):
    """The specification's serving mix (serve.SPEC_MIX: 70% permeability
    solves, sides 32-160, to a relative mean-flow change < 1e-7 per chunk; 30%
    drainage with two minerals and a tracer, D2Q9 256^2-1024^2 or D3Q19
    64^3-128^3, until the invader's mass levels off) with ``n`` seeded
    requests: the FP16-storage form served at the Poisson arrival rate (p50 /
    p99 latency) and with every request queued at once (capacity), the FP32
    form at capacity, and the plain FP64 form one request at a time."""
    from taxila import serve
    reqs = serve.make_spec_mix(n, seed=seed)
    sites = sum(r.params.nsites for r in reqs)
    out = {"mix": "%d requests of the specification's mix, seed %d (%d perm, %d drain, %d sites): Poisson %.0f/s; "
                  "perm sides %d-%d to mean-flow change < %g per chunk (cap %d steps); drainage D2Q9 %d-%d / D3Q19 "
                  "%d-%d with 2 minerals and a tracer to invader-mass change < %g per chunk (cap %d steps)"
                  % (n, seed, sum(r.kind == "perm" for r in reqs), sum(r.kind == "drain" for r in reqs), sites,
                     serve.SPEC_MIX["rate"], *serve.SPEC_MIX["perm_sides"], serve.SPEC_MIX["perm_tol"],
                     serve.SPEC_MIX["perm_max_steps"], *serve.SPEC_MIX["drain2_sides"], *serve.SPEC_MIX["drain3_sides"],
                     serve.SPEC_MIX["drain_tol"], serve.SPEC_MIX["drain_steps"])}
    runs = (("fp32_fp16_storage", P.PREC_F32_F16, None, True), ("fp32_fp16_storage_saturated", P.PREC_F32_F16, None, False),
            ("fp32_saturated", P.PREC_F32, None, False), ("fp64_sequential_saturated", P.PREC_F64, 1, False))
    values = {}
    for name, prec, maxa, realtime in runs:
        srv = serve.Server(precision=prec, max_active=maxa, chunk=100)
        res = srv.run(reqs, realtime=realtime)
        srv.close()
        out[name] = serve.summary(res)
        values[name] = {r.rid: r.value for r in res}
    f, s = out["fp32_fp16_storage_saturated"], out["fp64_sequential_saturated"]
    out["fp16_storage_vs_fp64_sequential_solves_saturated"] = round(f["solves_per_s"] / s["solves_per_s"], 2)
    perm = [r.rid for r in reqs if r.kind == "perm"]
    ref = values["fp64_sequential_saturated"]
    for name in ("fp32_fp16_storage_saturated", "fp32_saturated"):
        errs = [abs(values[name][i] / ref[i] - 1.0) for i in perm if ref.get(i)]
        out[name]["perm_rel_err_max_vs_fp64"] = max(errs) if errs else None
    out["saturated"] = "every request queued at once: solves/s is the server's capacity"
    return out


def conservation_mass(h):
    """Each component's mass from tx_conservation, or the error text."""
    try:
        return [float(v) for v in h.conservation()[0]]
    except Exception as ex:  # report, do not hide
        return "tx_conservation: %s" % ex


def run_gpu(args):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    gpu = torch.cuda.current_device()
    from taxila._lib import Handle
    prec = FORMS[args.form]
    p = workload_params(prec, args.n)
    walls, rho = workload_state(p)
    h = Handle(p)
    h.upload_walls(walls)
    h.upload_state(rho)
    h.init()
    mass0 = conservation_mass(h)
    h.step(args.warmup)
    h.sync()
    stream = torch.cuda.ExternalStream(h.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(ws)
    torch.cuda.synchronize()
    with Clocks(gpu) as clk:
        e0.record(stream)
        h.step(args.steps)
        e1.record(stream)
        e1.synchronize()
    torch.cuda.synchronize()
    barrier(ws)
    value, ms = replica_throughput(e0.elapsed_time(e1), p.nsites, args.steps, ws)
    # per-kernel durations (events around each launch)
    h.set_timing(True)
    nk = min(args.steps, 20)
    h.step(nk)
    h.sync()
    t_step, t_dens, _ = h.timing()
    h.set_timing(False)
    rho_check = h.delta_norm(P.FIELD_RHO)  # non-finite states raise here
    mass1 = conservation_mass(h)
    kname = h.kernel_name()
    h.close()
    if rank != 0:
        if ws > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return 0
    peak, peak_kind = peaks()
    k_ms = t_step / nk
    bpl = 2 * 19 * 2 * POP_BYTES[prec] + 1
    achieved = p.nsites * bpl / (k_ms * 1e-3) / 1e9
    bpl_dram = traffic_from_profile() if args.form == "f64" else None
    traffic = round(bpl_dram * p.nsites) if bpl_dram else None
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": {"f64": "f64", "f32": "f32", "f16": "f32 (f16 storage)"}[args.form],
        "data": "synthetic",
        "config": {"workload": "D3Q19 %d^3 2-component MRT Shan-Chen bubble (r=%g, rho 2.0/0.06, G=0.9 -> g_12=0.15), "
                               "periodic, isotropy 4, %s form" % (args.n, 24.0 * args.n / N_SIDE,
                                                                  {"f64": "FP64 plain", "f32": "FP32", "f16": "FP32-arithmetic FP16-storage"}[args.form]),
                   "global_lattice": [args.n] * 3, "sites_per_gpu": p.nsites, "parallelism": "replicas x%d" % ws,
                   "l2": "inputs larger than L2 (2 x %d MB population buffers); no flush" % (p.nsites * 38 * POP_BYTES[prec] // 1000000),
                   "kernel": "k_step/k_density (%s)" % kname},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic,
                     "kernel": "k_step (collide + push, %d B/LUP algorithmic)" % bpl,
                     "ms_per_launch": round(k_ms, 4), "ms_k_density": round(t_dens / nk, 4),
                     "peak_source": peak_kind,
                     "compute_bound": None,
                     "note": "the FP64 form is bound by GB300's FP64 pipe, not HBM (compute_bound: its FP64 "
                             "instructions per site against the measured FP64 instruction rate); the fp32/fp16 "
                             "forms are the HBM-bound ones"},
        "gpu_launches": 2 * args.steps,
        "clocks": clk.summary(),
    }
    small = {}
    if args.form == "f64" and not args.quick:
        # measured FP64 ceiling of the step kernel (pipe probes, sampled clock)
        try:
            small["peaks"] = peaks_run(gpu)
            line["roofline"]["compute_bound"] = fp64_bound(small["peaks"], p.nsites, k_ms)
        except Exception as ex:  # report, do not hide
            small["peaks"] = {"error": str(ex)}
    if ws == 1 and not args.quick and args.form == "f64" and args.n == N_SIDE:
        try:
            line["e2e"] = e2e_run(args.steps, 2)
        except Exception as ex:  # report, do not hide
            line["e2e"] = {"value": None, "unit": UNIT, "error": str(ex)}
        # the long legs first: the end of the line (what a tail of the output
        # keeps) holds the short per-form figures
        legs = (("batched", batched_run),
                ("batched_small", lambda: batched_run(n_lat=192, steps=100, seed=5, sides=(16, 48))),
                ("batched_converged", lambda: batched_converged_run(n_lat=CONVERGED_LATTICES)),
                ("serving_spec", lambda: serving_spec_run(n=SPEC_REQUESTS)),
                ("bubble_2d", bubble_2d_run))
        for key, fn in legs:
            try:
                line[key] = fn()
            except Exception as ex:  # report, do not hide
                line[key] = {"error": str(ex)}
        forms = {}
        for name, prec in (("fp32", P.PREC_F32), ("fp16_storage", P.PREC_F32_F16)):
            try:
                r = measure_form(prec, max(20, args.steps // 2), args.warmup)
                bpl = 2 * 19 * 2 * (4 if prec == P.PREC_F32 else 2) + 1
                r["k_step_gbs"] = p.nsites * bpl / (r["ms_k_step"] * 1e-3) / 1e9
                r["k_step_frac"] = r["k_step_gbs"] / peak
                forms[name] = {k: (round(v, 4) if isinstance(v, float) else v) for k, v in r.items()}
            except Exception as ex:
                forms[name] = {"error": str(ex)}
        small["precision_forms"] = forms
        try:
            # the same workload with the isotropy-8 psi gradient (the higher-order variant)
            q8 = workload_params(P.PREC_F64)
            q8.isotropy_order = 8
            r = measure_form(P.PREC_F64, max(20, args.steps // 4), args.warmup, p=q8)
            small["fp64_iso8"] = {k: (round(v, 4) if isinstance(v, float) else v) for k, v in r.items()}
        except Exception as ex:
            small["fp64_iso8"] = {"error": str(ex)}
        try:
            threads = os.cpu_count() or 1
            nb = CPU_BASELINE_STEPS
            v, dt = cpu_oracle_mlups(p, walls, rho, nb, threads)
            line["cpu_baseline"] = {"value": round(v, 4), "unit": UNIT, "cores": threads, "cpu": cpu_model(),
                                    "kind": "port",
                                    "sample": "%d steps of the full 128^3 lattice (%.1f s), C restatement of the "
                                              "reference step, OpenMP" % (nb, dt)}
        except Exception as ex:
            line["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": 0, "kind": "port", "sample": str(ex)}
    line.update(small)
    line["state_check"] = {"rho_delta_norm_last": rho_check}
    if isinstance(mass0, list) and isinstance(mass1, list):
        # each component's mass (FP64 device sums) after init and after every step of this run
        line["state_check"]["mass_after_init"] = mass0
        line["state_check"]["mass_at_end"] = mass1
        line["state_check"]["mass_rel_drift"] = [abs(b / a - 1.0) if a else None for a, b in zip(mass0, mass1)]
    else:
        line["state_check"]["mass_error"] = str(mass0 if not isinstance(mass0, list) else mass1)
    print(json.dumps(line))
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--quick", action="store_true", help="skip the e2e, precision-form, batched, serving and CPU legs")
    ap.add_argument("--n", type=int, default=N_SIDE, help="lattice side (profiling runs use a smaller case)")
    ap.add_argument("--form", default="f64", choices=sorted(FORMS), help="storage/arithmetic form of the timed run")
    ap.add_argument("--leg", default="all", choices=["all", "batched", "serving", "serving_spec", "batched_converged"],
                    help="run one extra leg alone and print its JSON (profiling)")
    ap.add_argument("--lattices", type=int, default=96, help="lattices of the batched leg")
    ap.add_argument("--requests", type=int, default=40, help="requests of the specification's serving mix")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.leg == "batched":
        print(json.dumps(batched_run(n_lat=args.lattices, steps=args.steps, compare=min(8, args.lattices))))
        return 0
    if args.leg == "serving":
        print(json.dumps(serving_run()))
        return 0
    if args.leg == "serving_spec":
        print(json.dumps(serving_spec_run(n=args.requests)))
        return 0
    if args.leg == "batched_converged":
        print(json.dumps(batched_converged_run(n_lat=args.lattices)))
        return 0
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
