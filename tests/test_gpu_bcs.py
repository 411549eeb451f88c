"""Exterior boundary conditions on the GPU against the oracle (C ABI).

Pressure, flux, momentum, velocity and reflecting faces, one- and
two-component outlets, and BCApply's class order at shared edges
(FlowApplyBCs, src/lbm/lbm_flow.F90:1958-1991; lbm_bc.F90:781-1865).  The
exact form is bit-identical (within 1e-12 where an EOS calls exp); the fast
form stays within 1e-12.
"""
import numpy as np
import pytest

import cases
from oracle import Oracle
from taxila import params as P
from taxila._lib import Batch, Handle, TxError

pytestmark = pytest.mark.gpu
FIELDS = (P.FIELD_FI, P.FIELD_RHO, P.FIELD_FLUX, P.FIELD_FORCES, P.FIELD_PRS)


def run_both(p, walls, rho, steps, exact, bc_values=None):
    o = Oracle(p)
    o.set_walls(walls)
    o.set_state(rho)
    q = P.copy_params(p)
    q.exact = 1 if exact else 0
    h = Handle(q)
    h.upload_walls(walls)
    h.upload_state(rho)
    for face, vals in (bc_values or {}).items():
        o.set_bc_values(face, vals)
        h.upload_bc_values(face, vals)
    o.init()
    h.init()
    o.step(steps)
    h.step(steps)
    return o, h


def check(o, h, walls, exact):
    pore = np.asarray(walls).ravel() == 0
    for f in FIELDS:
        a, b = o.get(f), h.download(f)
        m = np.repeat(pore, a.size // pore.size)
        if exact:
            bad = np.nonzero((a != b) & m)[0]
            assert bad.size == 0, "field %d: %d values differ, first %s: %r vs %r" % (f, bad.size, bad[:3], a[bad[:3]],
                                                                                    b[bad[:3]])
        else:
            scale = np.max(np.abs(a[m])) or 1.0
            err = np.max(np.abs(a[m] - b[m])) / scale
            assert err <= 1e-12, "field %d: max rel err %.3e > 1e-12" % (f, err)


@pytest.mark.parametrize("name,make,steps", cases.BCS, ids=[c[0] for c in cases.BCS])
@pytest.mark.parametrize("exact", [True, False], ids=["exact", "fast"])
def test_exterior_bcs_match_oracle(name, make, steps, exact):
    p, walls, rho = make()
    o, h = run_both(p, walls, rho, steps, exact)
    # the Shan-Chen and thermo EOS call exp, whose device and host results may differ by an ulp
    uses_exp = p.use_nonideal_eos and p.eos[0] in (P.EOS_SC, P.EOS_THERMO)
    check(o, h, walls, exact and not uses_exp)


def test_uploaded_face_values_match_oracle():
    # initialize_bcs: a momentum profile across the inlet face instead of the uniform value
    name, make, steps = next(c for c in cases.BCS if c[0] == "d3_reflect_momentum")
    p, walls, rho = make()
    area = p.nx * p.nz  # YM face: nodes in (x, z) order
    s, d = p.ncomponents, p.ndims
    vals = np.zeros((area, s * d))
    x = np.arange(area) % p.nx
    vals[:, 1 * s] = 0.002 * (x + 0.5) * (p.nx - x - 0.5) / (0.25 * p.nx * p.nx)
    o, h = run_both(p, walls, rho, steps, True, {P.YM: vals.ravel()})
    check(o, h, walls, True)


def test_bc_errors_are_status_codes():
    name, make, steps = cases.BCS[0]
    p, walls, rho = make()
    # a reflecting XM face in 2D reads past the reference's direction table
    q = P.copy_params(cases.BCS[6][1]()[0])
    q.bc_flags[0] = P.BC_REFLECTING
    with pytest.raises(TxError):
        Handle(q)
    # pressure and flux outlets together
    q = P.copy_params(p)
    q.bc_flags[4] = P.BC_FLUX_OUTLET
    with pytest.raises(TxError):
        Handle(q)
    # closed faces carry no values
    h = Handle(p)
    with pytest.raises(TxError):
        h.upload_bc_values(P.XM, np.zeros(p.ny * p.nz))


def _alone(p, walls, rho, steps):
    h = Handle(p)
    h.upload_walls(walls)
    h.upload_state(rho)
    h.init()
    h.step(steps)
    return h


@pytest.mark.parametrize("names", [["d3_pressure_s1", "d3_reflect_momentum", "d3_neumann_then_dirichlet"],
                                   ["d3_two_phase_pressure"]], ids=["one_component", "two_component_outlet"])
@pytest.mark.parametrize("prec", [P.PREC_F64, P.PREC_F32_F16], ids=["f64", "f16"])
def test_exterior_bcs_in_a_batch_equal_alone(names, prec):
    # face pass and outlet refresh as batched tile kernels: each lattice as alone,
    # bit for bit, including one that joins a running batch
    mk = {n: m for n, m, _ in cases.BCS}
    lats = []
    for n in names:
        p, w, r = mk[n]()
        q = P.copy_params(p)
        q.exact = 0
        q.precision = prec
        if prec != P.PREC_F64:
            q.rho0[0] = 1.0
            q.storage_scale = 4096.0
        lats.append((q, w, r))
    b = Batch(lats[0][0])
    ids = [b.add(q, w, r) for q, w, r in lats]
    b.step(23)
    late = mk[names[0]]()
    ql = P.copy_params(lats[0][0])
    il = b.add(ql, late[1], late[2])
    b.step(9)
    for (q, w, r), lid, steps in list(zip(lats, ids, [32] * len(ids))) + [((ql, late[1], late[2]), il, 9)]:
        h = _alone(q, w, r, steps)
        n = q.nsites * q.ncomponents * q.Q
        assert np.array_equal(b.download(lid, P.FIELD_FI, n), h.download(P.FIELD_FI))
        assert np.array_equal(b.download(lid, P.FIELD_RHO, q.nsites * q.ncomponents), h.download(P.FIELD_RHO))


@pytest.mark.parametrize("name", ["d3_two_phase_pressure", "d3_flux_velocity_mrt", "d2_velocity_outlet"])
def test_fast_form_1000_steps_with_exterior_bcs(name):
    # the stated tolerance (1e-12 relative after 1,000 steps) through driven faces
    p, walls, rho = next(m for n, m, _ in cases.BCS if n == name)()
    o, h = run_both(p, walls, rho, 1000, False)
    check(o, h, walls, False)
