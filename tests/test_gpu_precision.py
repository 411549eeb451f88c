"""Reduced-precision forms on the GPU against the FP64 oracle.

The FP32-arithmetic forms store population deviations f - w rho0 (FP32, or
FP16 times a storage scale).  Bounds, after the stated steps:

* single-phase permeability flow, rho0 = 1: permeability within 1e-3 relative
  (FP32 and FP16 storage), density within 1e-6;
* two-phase bubble, plain storage (rho0 = 0): densities within 2e-5 (FP32) /
  2e-3 (FP16) of the largest density, bubble radius within 1e-3 relative.
"""
import numpy as np
import pytest

import cases
from oracle import Oracle
from taxila import metrics
from taxila import params as P
from taxila._lib import Batch, Handle

pytestmark = pytest.mark.gpu


def oracle_after(p, walls, rho, steps):
    o = Oracle(p)
    o.set_walls(walls)
    o.set_state(rho)
    o.init()
    o.step(steps)
    return o


def gpu_after(q, walls, rho, steps):
    h = Handle(q)
    h.upload_walls(walls)
    h.upload_state(rho)
    h.init()
    h.step(steps)
    return h


@pytest.mark.parametrize("prec,scale", [(P.PREC_F32, 1.0), (P.PREC_F32_F16, 4096.0)], ids=["f32", "f32_f16"])
@pytest.mark.parametrize("shape", [(20, 18, 24), (20, 18, 23), (19, 17, 23)], ids=["even_nx", "odd_nx", "odd_sites"])
def test_permeability_reduced_precision(prec, scale, shape):
    # even nx: the paired step everywhere; odd nx: pairs that span a row end
    # take the per-site kernel; an odd site count: the per-site kernel alone
    p, walls, rho = cases.permeability_case(shape, seed=9)
    steps = 300
    o = oracle_after(p, walls, rho, steps)
    q = P.copy_params(p)
    q.precision = prec
    q.rho0[0] = 1.0
    q.storage_scale = scale
    h = gpu_after(q, walls, rho, steps)
    k_ref = metrics.permeability(1.0, p.gvt[2], o.get(P.FIELD_FLUX), walls, p.nsites)
    k_gpu = metrics.permeability(1.0, p.gvt[2], h.download(P.FIELD_FLUX), walls, p.nsites)
    assert abs(k_gpu / k_ref - 1.0) < 1e-3, (k_gpu, k_ref)
    pore = walls == 0
    assert metrics.rel_err(h.download(P.FIELD_RHO), o.get(P.FIELD_RHO), pore) < 1e-6
    # the same lattice in a batch of that form evolves identically
    b = Batch(q)
    lid = b.add(q, walls, rho)
    b.step(steps)
    assert np.array_equal(b.download(lid, P.FIELD_FI, p.nsites * 19), h.download(P.FIELD_FI))


@pytest.mark.parametrize("prec,tol", [(P.PREC_F32, 2e-5), (P.PREC_F32_F16, 2e-3)], ids=["f32", "f32_f16"])
@pytest.mark.parametrize("shape,nu_only", [((24, 24, 24), False), ((24, 24, 23), True)],
                         ids=["mixed_rates", "odd_nx_s_nu_only"])
def test_bubble_reduced_precision(prec, tol, shape, nu_only):
    p, walls, rho = cases.sc_bubble(P.D3Q19, shape, P.MRT, 4, g=0.15, r=6, nu_only=nu_only)
    steps = 200
    o = oracle_after(p, walls, rho, steps)
    q = P.copy_params(p)
    q.precision = prec
    h = gpu_after(q, walls, rho, steps)
    r_ref, r_gpu = o.get(P.FIELD_RHO), h.download(P.FIELD_RHO)
    assert metrics.rel_err(r_gpu, r_ref) < tol
    R_ref = metrics.equivalent_radius(r_ref, 2, 0, 0.06, 2.0, 3)
    R_gpu = metrics.equivalent_radius(r_gpu, 2, 0, 0.06, 2.0, 3)
    assert abs(R_gpu / R_ref - 1.0) < 1e-3, (R_gpu, R_ref)
    # the same lattice in a batch of that form evolves identically
    b = Batch(q)
    lid = b.add(q, walls, rho)
    b.step(steps)
    assert np.array_equal(b.download(lid, P.FIELD_FI, p.nsites * 2 * 19), h.download(P.FIELD_FI))
