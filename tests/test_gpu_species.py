"""Passive species transport on the GPU against the oracle (C ABI).

* exact FP64 form: species populations, concentrations and fluxes identical
  to the oracle bit for bit (and the flow populations still are);
* fast FP64 form: within 1e-12 of the largest value;
* species mass is conserved.
"""
import numpy as np
import pytest

import cases
from oracle import Oracle
from taxila import params as P
from taxila._lib import Handle

pytestmark = pytest.mark.gpu
SPECIES_FIELDS = (P.FIELD_SPECIES_FI, P.FIELD_SPECIES_RHO, P.FIELD_SPECIES_FLUX, P.FIELD_FI)


def run(p, walls, rho, conc, steps, exact):
    o = Oracle(p)
    o.set_walls(walls)
    o.set_state(rho)
    o.set_species(conc)
    o.init()
    o.step(steps)
    q = P.copy_params(p)
    q.exact = 1 if exact else 0
    h = Handle(q)
    h.upload_walls(walls)
    h.upload_state(rho)
    h.upload_species(conc)
    h.init()
    h.step(steps)
    return o, h


@pytest.mark.parametrize("name,make,steps", cases.SPECIES, ids=[c[0] for c in cases.SPECIES])
@pytest.mark.parametrize("exact", [True, False], ids=["exact", "fast"])
def test_species_match_oracle(name, make, steps, exact):
    p, walls, rho, conc = make()
    o, h = run(p, walls, rho, conc, steps, exact)
    pore = np.asarray(walls).ravel() == 0
    for f in SPECIES_FIELDS:
        a, b = o.get(f), h.download(f)
        m = np.repeat(pore, a.size // p.nsites)
        if exact:
            bad = np.nonzero((a != b) & m)[0]
            assert bad.size == 0, "field %d: %d values differ" % (f, bad.size)
        else:
            scale = np.max(np.abs(a[m])) or 1.0
            assert np.max(np.abs(a[m] - b[m])) / scale <= 1e-12, f
    mass = h.download(P.FIELD_SPECIES_RHO).reshape(p.nsites, -1)[pore].sum(axis=0)
    assert np.allclose(mass, np.asarray(conc).reshape(p.nsites, -1)[pore].sum(axis=0), rtol=1e-12)


def test_species_errors():
    p, walls, rho = cases.porous_case(P.D3Q19, (8, 8, 8))
    h = Handle(p)
    with pytest.raises(Exception):
        h.upload_species(np.zeros(p.nsites))  # created without species


@pytest.mark.parametrize("name,make,steps", cases.SPECIES, ids=[c[0] for c in cases.SPECIES])
def test_species_only_steps(name, make, steps):
    # the steady-flow mode (-steadystate_flow): after k full steps, m
    # species-only steps leave the flow as it was and move the species exactly
    # as m more full steps do, since the species feel no flow in this model
    p, walls, rho, conc = make()
    k, m = 3, 5

    def started():
        h = Handle(p)
        h.upload_walls(walls)
        h.upload_state(rho)
        h.upload_species(conc)
        h.init()
        return h

    a = started()
    a.step(k)
    flow_k = a.download(P.FIELD_FI)
    a.step_species(m)
    b = started()
    b.step(k + m)
    assert np.array_equal(a.download(P.FIELD_FI), flow_k)
    for f in (P.FIELD_SPECIES_FI, P.FIELD_SPECIES_RHO, P.FIELD_SPECIES_FLUX):
        assert np.array_equal(a.download(f), b.download(f)), f
    a.close()
    b.close()


def test_species_only_step_needs_species():
    from taxila._lib import TxError
    p, walls, rho = cases.porous_case(P.D3Q19, (8, 8, 8))
    h = Handle(p)
    h.upload_walls(walls)
    h.upload_state(rho)
    h.init()
    with pytest.raises(TxError) as e:
        h.step_species(1)
    assert e.value.code == 2
    h.close()
