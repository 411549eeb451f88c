"""Request server (continuous batching over tx_batch).

* every request's result is the same served alone and served in the mix
  (same step count, same permeability / saturation bit for bit): lattices
  only interact through scheduling, and admission happens at chunk
  boundaries;
* requests that do not fit the device-memory budget wait and are admitted
  as memory frees up; the budget is never exceeded;
* a served FP16-storage permeability agrees with the FP64 oracle to 1e-3.
"""
import numpy as np
import pytest

from oracle import Oracle
from taxila import metrics
from taxila import params as P
from taxila import serve

pytestmark = pytest.mark.gpu


def small_mix(seed=3, n=9):
    """n requests of all three kinds (permeability, D3Q19 and D2Q9 drainage), sizes drawn per seed."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        s = int(rng.integers(0, 1 << 30))
        kind = i % 3
        if kind == 0:
            sides = [int(v) for v in rng.integers(14, 23, size=3)]
            out.append(serve.perm_request(i, 0.001 * i, sides, s, tol=1e-4, max_steps=2000))
        elif kind == 1:
            sides = [int(v) for v in rng.integers(14, 19, size=3)]
            out.append(serve.drain_request(i, 0.001 * i, sides, s, 300, dims=3))
        else:
            sides = [int(v) for v in rng.integers(28, 41, size=2)]
            out.append(serve.drain_request(i, 0.001 * i, sides, s, 300, dims=2))
    return out


@pytest.mark.parametrize("prec", [P.PREC_F32, P.PREC_F32_F16], ids=["f32", "f32_f16"])
def test_same_result_alone_and_in_mix(prec):
    reqs = small_mix()
    assert {(r.kind, r.params.discretization) for r in reqs} == {("perm", P.D3Q19), ("drain", P.D3Q19),
                                                                   ("drain", P.D2Q9)}
    srv = serve.Server(precision=prec, chunk=50, tiles=(32, 4, 1, 4))
    mix = {r.rid: r for r in srv.run(reqs, realtime=False)}
    srv.close()
    assert sorted(mix) == sorted(r.rid for r in reqs)
    for req in reqs:
        one = serve.Server(precision=prec, chunk=50, tiles=(32, 4, 1, 4))
        (res,) = one.run([req], realtime=False)
        one.close()
        m = mix[req.rid]
        assert (res.steps, res.value, res.front, res.tracer) == (m.steps, m.value, m.front, m.tracer), \
            (req.rid, req.kind, res, m)
        if req.kind == "drain":
            assert m.tracer > 0.0


def test_budget_admission_waits_for_memory():
    reqs = small_mix(seed=5, n=6)
    srv = serve.Server(precision=P.PREC_F32, chunk=50)
    need = max(serve.Batch.lattice_bytes(srv._params(r)) for r in reqs)
    srv.budget = int(1.5 * need)  # at most one of the largest in flight
    peak = [0]
    orig = srv._batch

    def tracked(q):
        key, b = orig(q)
        peak[0] = max(peak[0], srv.in_use())
        return key, b
    srv._batch = tracked
    res = srv.run(reqs, realtime=False)
    srv.close()
    assert len(res) == len(reqs)
    assert peak[0] <= srv.budget


def test_served_fp16_permeability_matches_fp64_oracle():
    req = serve.perm_request(0, 0.0, (18, 16, 20), seed=17, tol=1e-9, max_steps=600)
    srv = serve.Server(precision=P.PREC_F32_F16, storage_scale=4096.0, chunk=100)
    (res,) = srv.run([req], realtime=False)
    srv.close()
    assert res.steps == 600
    o = Oracle(req.params)
    o.set_walls(req.walls)
    o.set_state(req.rho)
    o.init()
    o.step(600)
    k_ref = metrics.permeability(1.0, req.params.gvt[2], o.get(P.FIELD_FLUX), req.walls, req.params.nsites)
    assert abs(res.value / k_ref - 1.0) < 1e-3, (res.value, k_ref)


def test_served_fp16_permeability_converged_matches_fp64_oracle():
    # served to its stop criterion (relative change of the mean flow < 1e-7
    # per chunk), the FP16-storage permeability is within 1e-3 of the FP64
    # oracle run for the same number of steps
    req = serve.perm_request(0, 0.0, (22, 18, 26), seed=23, tol=1e-7, max_steps=20000, gz=1e-6, radii=(2.5, 5.0))
    srv = serve.Server(precision=P.PREC_F32_F16, storage_scale=4096.0, chunk=100)
    (res,) = srv.run([req], realtime=False)
    srv.close()
    assert res.steps < 20000, "the stop criterion was never met"
    o = Oracle(req.params)
    o.set_walls(req.walls)
    o.set_state(req.rho)
    o.init()
    o.step(res.steps)
    k_ref = metrics.permeability(1.0, req.params.gvt[2], o.get(P.FIELD_FLUX), req.walls, req.params.nsites)
    assert abs(res.value / k_ref - 1.0) < 1e-3, (res.steps, res.value, k_ref)


def test_drainage_stops_when_the_invader_mass_levels_off():
    # the drainage criterion ends a run before its step cap, and the run is
    # the same alone and with a second request in flight
    reqs = [serve.drain_request(0, 0.0, (16, 14, 20), 11, 20000, dims=3, tol=2e-3),
            serve.perm_request(1, 0.0, (14, 16, 18), 12, tol=1e-4, max_steps=2000)]
    srv = serve.Server(precision=P.PREC_F32, chunk=50)
    mix = {r.rid: r for r in srv.run(reqs, realtime=False)}
    srv.close()
    one = serve.Server(precision=P.PREC_F32, chunk=50)
    (alone,) = one.run(reqs[:1], realtime=False)
    one.close()
    assert mix[0].steps < 20000 and mix[0].steps % 50 == 0
    assert (alone.steps, alone.value) == (mix[0].steps, mix[0].value)
