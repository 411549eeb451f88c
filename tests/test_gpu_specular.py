"""Specular (no-stick) walls 900/901/902 on the GPU against the oracle, through the C ABI.

DistributionBouncebackD3/D2 (src/lbm/lbm_distribution_function.F90:668-784)
sweeps the ghosted box in k-j-i order; a specular wall reflects only the
component of c normal to it and may write into wall cells the sweep has
already cleared, so wall cells end steps holding populations.  The library
resolves every population slot's source once per wall upload and applies the
exceptions to its ordinary push after the step kernel (csrc/tx_specular.cuh).

* exact FP64 form: every cell's populations (wall cells included), densities,
  velocities and forces identical to the oracle bit for bit;
* fast FP64 form: within 1e-12 relative;
* the FP32/FP16 forms within their bounds of the FP64 oracle;
* restarts with populations in wall cells, and batches, which refuse these codes.
"""
import numpy as np
import pytest

import cases
from oracle import Oracle
from taxila import params as P
from taxila._lib import Batch, Handle, TxError

pytestmark = pytest.mark.gpu
FIELDS = (P.FIELD_FI, P.FIELD_RHO, P.FIELD_FLUX, P.FIELD_FORCES)


def run_pair(p, walls, rho, steps, exact, fi=None):
    o = Oracle(p)
    o.set_walls(walls)
    q = P.copy_params(p)
    q.exact = 1 if exact else 0
    h = Handle(q)
    h.upload_walls(walls)
    if fi is not None:
        o.set_fi(fi)
        h.upload_fi(fi)
    else:
        o.set_state(rho)
        h.upload_state(rho)
    o.init()
    h.init()
    if steps:
        o.step(steps)
        h.step(steps)
    return o, h


def compare_all_cells(o, h, exact, rtol=1e-12):
    for f in FIELDS:
        a, b = o.get(f), h.download(f)
        assert np.all(np.isfinite(a)), f
        if exact:
            bad = np.nonzero(a != b)[0]
            assert bad.size == 0, "field %d: %d values differ, first %s: %r vs %r" % (f, bad.size, bad[:3], a[bad[:3]], b[bad[:3]])
        else:
            err = float(np.max(np.abs(a - b)) / (np.max(np.abs(a)) or 1.0))
            assert err <= rtol, "field %d: max rel err %.3e > %.1e" % (f, err, rtol)


def wall_content(o, p, walls):
    return float(np.abs(o.get(P.FIELD_FI).reshape(p.nsites, -1)[np.asarray(walls) > 0]).sum())


@pytest.mark.parametrize("name,make,steps", cases.SPECULAR, ids=[c[0] for c in cases.SPECULAR])
@pytest.mark.parametrize("exact", [True, False], ids=["exact", "fast"])
def test_specular_walls_match_oracle(name, make, steps, exact):
    p, walls, rho = make()
    o, h = run_pair(p, walls, rho, steps, exact)
    assert wall_content(o, p, walls) > 0.0  # the case exercises populations left in wall cells
    compare_all_cells(o, h, exact)
    # the delta norms see the wall cells' populations as the reference's do
    o.step(1)
    h.step(1)
    for field in (P.FIELD_RHO, P.FIELD_FI):
        a, b = o.delta_norm(field), h.delta_norm(field)
        assert (a == b) if exact else abs(a - b) <= 1e-10 * max(abs(a), 1e-300), (field, a, b)


@pytest.mark.parametrize("name,make,steps", cases.SPECULAR_BCS, ids=[c[0] for c in cases.SPECULAR_BCS])
def test_specular_walls_with_exterior_bcs(name, make, steps):
    # bit for bit, except where an equation of state calls exp (the device's
    # and the host libm's may differ by an ulp): there within 1e-12
    p, walls, rho = make()
    o, h = run_pair(p, walls, rho, steps, True)
    compare_all_cells(o, h, not p.use_nonideal_eos)


@pytest.mark.parametrize("name,make,steps", cases.SPECIES_SPECULAR, ids=[c[0] for c in cases.SPECIES_SPECULAR])
def test_species_with_specular_walls(name, make, steps):
    # species stream and bounce back through the same sweep as the flow (in 2D
    # the reference also collides the wall cells that hold them)
    p, walls, rho, conc = make()
    o = Oracle(p)
    o.set_walls(walls)
    o.set_state(rho)
    o.set_species(conc)
    o.init()
    o.step(steps)
    q = P.copy_params(p)
    q.exact = 1
    h = Handle(q)
    h.upload_walls(walls)
    h.upload_state(rho)
    h.upload_species(conc)
    h.init()
    h.step(steps)
    for f in (P.FIELD_FI, P.FIELD_SPECIES_FI, P.FIELD_SPECIES_RHO, P.FIELD_SPECIES_FLUX):
        a, b = o.get(f), h.download(f)
        assert np.all(np.isfinite(a)), f
        assert np.array_equal(a, b), (f, int(np.sum(a != b)))
    h.close()
    o.close()


FORM_TOL = {P.PREC_F32: 2e-5, P.PREC_F32_F16: 2e-3}


@pytest.mark.parametrize("prec,rho0,scale", [(P.PREC_F32, 1.0, 1.0), (P.PREC_F32_F16, 1.0, 4096.0)],
                         ids=["f32", "f32_f16"])
def test_specular_walls_reduced_precision(prec, rho0, scale):
    # deviation storage: exceptions copy stored values between slots of one
    # speed, empty slots take the stored value of f = 0
    p, walls, rho = cases.SPECULAR[0][1]()
    o = Oracle(p)
    o.set_walls(walls)
    o.set_state(rho)
    o.init()
    o.step(6)
    q = P.copy_params(p)
    q.precision = prec
    q.rho0[0] = rho0
    q.storage_scale = scale
    h = Handle(q)
    h.upload_walls(walls)
    h.upload_state(rho)
    h.init()
    h.step(6)
    for f in (P.FIELD_FI, P.FIELD_RHO):
        a, b = o.get(f), h.download(f)
        err = float(np.max(np.abs(a - b)) / np.max(np.abs(a)))
        assert err <= FORM_TOL[prec], (f, err)
    h.close()
    o.close()


def test_specular_restart_with_wall_content():
    p, walls, rho = cases.specular_porous(P.D3Q19, (12, 10, 11), 8)
    o0 = Oracle(p)
    o0.set_walls(walls)
    o0.set_state(rho)
    o0.init()
    o0.step(3)
    fi = o0.get(P.FIELD_FI)
    o0.close()
    assert np.abs(fi.reshape(p.nsites, -1)[walls > 0]).sum() > 0.0
    o, h = run_pair(p, walls, None, 6, True, fi=fi)
    compare_all_cells(o, h, True)


def test_specular_larger_lattice_fast_form():
    # more steps on a larger lattice: long wall-to-wall chains and many exceptions
    p, walls, rho = cases.specular_case(P.D3Q19, (24, 28, 32), (1, 0, 1), 2, cases.SPEC3, 0.2, 11)
    o, h = run_pair(p, walls, rho, 40, exact=False)
    compare_all_cells(o, h, False)


def test_specular_walls_refused_where_unsupported():
    p, walls, rho = cases.SPECULAR[0][1]()
    # a refused upload (a negative code) leaves the handle usable with other walls
    h = Handle(p)
    bad = np.array(walls)
    bad[0] = -3.0
    with pytest.raises(TxError):
        h.upload_walls(bad)
    h.upload_walls(np.where(walls >= 900.0, 1.0, walls))
    h.upload_state(rho)
    h.init()
    h.step(2)
    h.close()
    form = P.copy_params(p)
    form.exact = 0
    b = Batch(form)
    with pytest.raises(TxError):
        b.add(p, walls, rho)
    b.close()


def test_specular_walls_download_as_uploaded():
    p, walls, _ = cases.SPECULAR[3][1]()
    h = Handle(p)
    h.upload_walls(walls)
    assert np.array_equal(h.download(P.FIELD_WALLS), walls)
    h.close()


SPECIES_FORM_CASES = [("d3_mrt_two_species_specular", P.PREC_F32, 6), ("d3_mrt_two_species_specular", P.PREC_F32_F16, 6),
                      ("d2_species_specular", P.PREC_F32, 10), ("d2_mrt_species_specular", P.PREC_F32, 12)]


@pytest.mark.parametrize("name,prec,steps", SPECIES_FORM_CASES, ids=["d3_mrt_f32", "d3_mrt_f16", "d2_srt_f32", "d2_mrt_f32"])
def test_species_specular_reduced_precision(name, prec, steps):
    # species (no rest state: empty slots store zero) next to the flow's
    # deviation storage, each component's rest density at its mean
    p, walls, rho, conc = dict((c[0], c[1]) for c in cases.SPECIES_SPECULAR)[name]()
    o = Oracle(p)
    o.set_walls(walls)
    o.set_state(rho)
    o.set_species(conc)
    o.init()
    o.step(steps)
    q = P.copy_params(p)
    q.exact = 0
    q.precision = prec
    q.storage_scale = 4096.0 if prec == P.PREC_F32_F16 else 1.0
    for m in range(p.ncomponents):
        q.rho0[m] = float(np.mean(np.asarray(rho).reshape(-1, p.ncomponents)[:, m]))
    h = Handle(q)
    h.upload_walls(walls)
    h.upload_state(rho)
    h.upload_species(conc)
    h.init()
    h.step(steps)
    for f in (P.FIELD_FI, P.FIELD_SPECIES_FI, P.FIELD_SPECIES_RHO):
        a, b = o.get(f), h.download(f)
        err = float(np.max(np.abs(a - b)) / np.max(np.abs(a)))
        assert err <= FORM_TOL[prec], (f, err)
    h.close()
    o.close()


@pytest.mark.parametrize("name,make,steps", cases.SPECIES_SPECULAR_BCS, ids=[c[0] for c in cases.SPECIES_SPECULAR_BCS])
def test_species_specular_with_exterior_bcs(name, make, steps):
    # the species' own exception list: no BCPreStream copies (their transport
    # applies no boundary condition); bit for bit, within 1e-12 where an
    # equation of state calls exp
    p, walls, rho, conc = make()
    o = Oracle(p)
    o.set_walls(walls)
    o.set_state(rho)
    o.set_species(conc)
    o.init()
    o.step(steps)
    q = P.copy_params(p)
    q.exact = 1
    h = Handle(q)
    h.upload_walls(walls)
    h.upload_state(rho)
    h.upload_species(conc)
    h.init()
    h.step(steps)
    tol = 1e-12 if p.use_nonideal_eos else 0.0
    for f in (P.FIELD_FI, P.FIELD_SPECIES_FI, P.FIELD_SPECIES_RHO, P.FIELD_SPECIES_FLUX):
        a, b = o.get(f), h.download(f)
        assert np.all(np.isfinite(a)), f
        bad = int(np.sum(np.abs(a - b) > tol * np.max(np.abs(a))))
        assert bad == 0, (f, bad)
    h.close()
    o.close()
