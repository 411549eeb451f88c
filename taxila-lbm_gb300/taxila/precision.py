"""Precision study: the FP32-arithmetic forms (FP32 or FP16 storage of
deviations) against the FP64 form on the same inputs.

Two workloads, seeded:

* porous drainage (D3Q19, two components, sphere pack with two minerals,
  density faces along z, walls on x/y): density-field error, saturation and
  mean front position of the invading phase at checkpoints;
* single-phase permeability (D3Q19 BGK, periodic sphere pack, body force
  along z): permeability.

The FP64 reference is the GPU's FP64 form, which agrees with the CPU oracle
to 1e-12 after 1,000 steps (its exact variant bit for bit), so full-size
runs that the CPU oracle cannot finish still have an FP64 anchor.

    python -m taxila.precision --n 256 --steps 20000 --out study.json
    python -m taxila.precision --batch 96 --out batch.json   # the batched-permeability set
"""
import argparse
import json
import time

import numpy as np

from . import metrics
from . import params as P
from . import problems
from . import serve
from ._lib import Batch, Handle


def drainage_case(n, seed=1234):
    """n^3 drainage: the serving drainage request scaled to n, grain radii
    6..12 voxels at n = 256 (scaled with n), porosity 0.35."""
    req = serve.drain_request(0, 0.0, (n, n, n), seed, 0, dims=3)
    p = req.params
    p.nspecies = 0
    scale = n / 256.0
    solid = problems.sphere_pack(p.shape, 0.35, max(2.0, 6.0 * scale), max(3.0, 12.0 * scale), seed, periodic=False)
    solid[0:2] = False
    solid[-2:] = False
    walls = problems.mineral_walls(solid, seed)
    pore = walls == 0
    inlet = np.indices(p.shape)[0].ravel() < 3
    rho = np.empty((p.nsites, 2))
    rho[:, 0] = np.where(pore, np.where(inlet, 1.05, 0.03), 0.0)
    rho[:, 1] = np.where(pore, np.where(inlet, 0.03, 1.0), 0.0)
    return p, walls, rho.ravel()


def permeability_case(n, seed=4321, gz=1e-5):
    req = serve.perm_request(0, 0.0, (n, n, n), seed, 0.0, 0, gz=gz, radii=(4.0 * n / 96, 10.0 * n / 96))
    return req.params, req.walls, req.rho


# the FP64 reference runs the fast FP64 form: within 1e-12 of the oracle after
# 1,000 steps (tests/test_gpu_parity.py), far below the errors measured here
FORMS = (("fp64", P.PREC_F64, 0), ("fp32", P.PREC_F32, 0), ("fp32_fp16_storage", P.PREC_F32_F16, 0))


def _handle(p, walls, rho, prec, exact, rho0, scale):
    q = P.copy_params(p)
    q.precision = prec
    q.exact = exact
    for m in range(P.MAXC):
        q.rho0[m] = rho0[m] if m < len(rho0) else 0.0
    q.storage_scale = scale
    h = Handle(q)
    h.upload_walls(walls)
    h.upload_state(rho)
    h.init()
    return h


def drainage_study(n, steps, checkpoints, seed=1234):
    p, walls, rho = drainage_case(n, seed)
    pore = walls == 0
    out = {"case": "D3Q19 %d^3 two-phase drainage, seed %d, porosity %.3f" % (n, seed, pore.mean()),
           "steps": steps, "checkpoints": {}}
    fields = {}
    for name, prec, exact in FORMS:
        t = time.perf_counter()
        h = _handle(p, walls, rho, prec, exact, (0.0, 0.0), 1.0)
        done = 0
        for c in checkpoints:
            h.step(c - done)
            done = c
            fields[(name, c)] = h.download(P.FIELD_RHO)
        h.close()
        out.setdefault("seconds", {})[name] = round(time.perf_counter() - t, 1)
    for c in checkpoints:
        ref = fields[("fp64", c)]
        row = {}
        for name, _, _ in FORMS:
            r = fields[(name, c)]
            m = np.repeat(pore, 2)
            row[name] = {
                "saturation": metrics.saturation(r, 2, 0, 0.03, 1.05, walls),
                "front": metrics.front_position(r, p.shape, 2, 0, 0.03, 1.05, walls),
                "rho_max_err": metrics.rel_err(r, ref, m),
                "rho_mean_abs_err": float(np.mean(np.abs(r[m] - ref[m]))),
            }
        for name in ("fp32", "fp32_fp16_storage"):
            row[name]["saturation_err"] = abs(row[name]["saturation"] - row["fp64"]["saturation"])
            row[name]["front_err"] = abs(row[name]["front"] - row["fp64"]["front"])
        out["checkpoints"][str(c)] = row
    return out


def permeability_study(n, steps, seed=4321):
    p, walls, rho = permeability_case(n, seed)
    out = {"case": "D3Q19 %d^3 single-phase permeability, seed %d, porosity %.3f" % (n, seed, (walls == 0).mean()),
           "steps": steps}
    ks = {}
    for name, prec, exact in FORMS:
        h = _handle(p, walls, rho, prec, exact, (1.0,), 4096.0)
        h.step(steps)
        ks[name] = metrics.permeability(p.tau[0], p.gvt[2], h.download(P.FIELD_FLUX), walls, p.nsites)
        h.close()
    out["permeability"] = ks
    out["rel_err"] = {k: abs(v / ks["fp64"] - 1.0) for k, v in ks.items() if k != "fp64"}
    return out


def batch_lattices(n_lat=96, seed=4, sides=(48, 192), tol=1e-7, max_steps=40000, gz=1e-6):
    """The batched-permeability workload: ``n_lat`` single-phase D3Q19 BGK
    (tau = 1) lattices, each side uniform in ``sides``, seeded periodic sphere
    packs (radii 4..10, porosity uniform 0.25..0.5), body force ``gz`` along
    z, run until the mean flow changes by less than ``tol`` relative per
    100-step chunk."""
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n_lat):
        dims = [int(v) for v in rng.integers(sides[0], sides[1] + 1, size=3)]
        reqs.append(serve.perm_request(i, 0.0, dims, int(rng.integers(0, 1 << 30)), tol, max_steps, gz=gz,
                                       radii=(4.0, 10.0)))
    return reqs


def batch_permeability_study(n_lat=96, seed=4, tol=1e-7, max_steps=40000, chunk=100):
    """Every lattice of the batched-permeability workload run to its stop
    criterion in one batch per form (persistent tile-table launches replayed
    as CUDA graphs, tuned tiles): time to solution of the whole set, and
    each lattice's steps and permeability, with the FP32-arithmetic forms'
    permeability errors against the FP64 form's."""
    reqs = batch_lattices(n_lat, seed, tol=tol, max_steps=max_steps)
    sites = sum(r.params.nsites for r in reqs)
    # tile shape and grid from the autotuner, on a batch of the same lattices
    # that is then discarded (its trial steps would shift the probe chunks)
    tiles = {}
    for name, prec, _ in FORMS:
        form = P.copy_params(reqs[0].params)
        form.precision = prec
        tb = Batch(form)
        for r in reqs:
            q = P.copy_params(r.params)
            q.precision = prec
            tb.add(q, r.walls, r.rho)
        tiles[name] = tuple(tb.tune(2))
        tb.close()
    out = {"case": "%d single-phase D3Q19 BGK periodic sphere packs, sides 48-192 per axis (%d sites), body force "
                   "1e-6, stop at a relative change of the mean flow < %g per %d-step chunk (cap %d steps)"
                   % (n_lat, sites, tol, chunk, max_steps), "forms": {}}
    perms = {}
    for name, prec, _ in FORMS:
        srv = serve.Server(precision=prec, chunk=chunk, budget_bytes=200 << 30, tiles=tiles[name])
        t = time.perf_counter()
        res = srv.run(reqs, realtime=False)
        span = time.perf_counter() - t
        srv.close()
        steps = {r.rid: r.steps for r in res}
        perms[name] = {r.rid: r.value for r in res}
        out["forms"][name] = {"time_to_solution_s": round(span, 2), "tiles": list(tiles[name]),
                              "lattice_steps_mean": round(float(np.mean(list(steps.values()))), 1),
                              "lattice_steps_max": int(max(steps.values())),
                              "capped": int(sum(1 for v in steps.values() if v >= max_steps)),
                              "gsite_steps": round(sum(r.sites * r.steps for r in res) / 1e9, 2)}
    ref = perms["fp64"]
    out["lattices"] = [{"rid": r.rid, "dims": [r.params.nx, r.params.ny, r.params.nz],
                        "porosity": round(float(np.mean(np.asarray(r.walls) == 0)), 4),
                        "k_fp64": ref[r.rid],
                        "rel_err": {name: abs(perms[name][r.rid] / ref[r.rid] - 1.0)
                                    for name in perms if name != "fp64"}} for r in reqs]
    for name in perms:
        if name != "fp64":
            errs = [l["rel_err"][name] for l in out["lattices"]]
            out["forms"][name]["perm_rel_err_max"] = max(errs)
            out["forms"][name]["perm_rel_err_median"] = float(np.median(errs))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--checkpoints", type=int, default=4)
    ap.add_argument("--perm-n", type=int, default=96)
    ap.add_argument("--perm-steps", type=int, default=4000)
    ap.add_argument("--out", default="")
    ap.add_argument("--batch", type=int, default=0,
                    help="run the batched-permeability study on this many lattices instead (96: the full set)")
    a = ap.parse_args()
    if a.batch:
        res = {"batched_permeability": batch_permeability_study(a.batch)}
    else:
        cps = [a.steps * (i + 1) // a.checkpoints for i in range(a.checkpoints)]
        res = {"drainage": drainage_study(a.n, a.steps, cps), "permeability": permeability_study(a.perm_n, a.perm_steps)}
    text = json.dumps(res, indent=1)
    if a.out:
        with open(a.out, "w") as f:
            f.write(text)
    print(text)


if __name__ == "__main__":
    main()
