"""tx_conservation: global mass and momentum summed in FP64 on the device.

* the device totals equal FP64 sums of the downloaded populations (within
  1e-12 relative: only the order of summation differs), for the FP64, FP32
  and FP16-storage forms, in 3D and 2D, with walls and density faces;
* a second call on the same state returns the same bits;
* on a periodic two-component bubble each component's mass stays constant
  over the steps, to round-off;
* the call before tx_init is a TX_ERR_STATE error.
"""
import numpy as np
import pytest

import cases
from taxila import params as P
from taxila._lib import Handle, TxError

pytestmark = pytest.mark.gpu

# direction vectors in the reference's order (rest, axis links, diagonals)
C3 = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [-1, 0, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
               [1, 1, 0], [-1, 1, 0], [-1, -1, 0], [1, -1, 0], [1, 0, 1], [-1, 0, 1], [-1, 0, -1],
               [1, 0, -1], [0, 1, 1], [0, -1, 1], [0, -1, -1], [0, 1, -1]], dtype=np.float64)
C2 = np.array([[0, 0], [1, 0], [0, 1], [-1, 0], [0, -1], [1, 1], [-1, 1], [-1, -1], [1, -1]],
              dtype=np.float64)


def host_totals(p, fi):
    s, q = p.ncomponents, p.Q
    f = fi.reshape(p.nsites, q, s)
    c = C3 if p.ndims == 3 else C2
    mass = f.sum(axis=(0, 1))
    mom = np.einsum("iqm,qd->md", f, c)
    return mass, mom


def bubble_f16():
    p, walls, rho = cases.sc_bubble(P.D3Q19, (16, 12, 14), P.MRT, 4, nu_only=True)
    p.precision = P.PREC_F32_F16
    return p, walls, rho


def perm_f16():
    p, walls, rho = cases.permeability_case((20, 18, 24), seed=9, precision=P.PREC_F32_F16)
    p.storage_scale = 4096.0
    return p, walls, rho


CASES = [
    ("d3_bubble_mrt_f64", lambda: cases.sc_bubble(P.D3Q19, (16, 12, 14), P.MRT, 4)),
    ("d3_porous_dirichlet_body_f64", lambda: cases.porous_case(P.D3Q19, (12, 10, 14), mode=P.MRT, body=True)),
    ("d2_porous_dirichlet_f64", lambda: cases.porous_case(P.D2Q9, (1, 30, 26), body=True)),
    ("d2_bubble_one_component_f64", lambda: cases.sc_bubble(P.D2Q9, (1, 40, 48), P.SRT, 4, ncomp=1)),
    ("d3_bubble_f16_storage", bubble_f16),
    ("d3_permeability_f32", lambda: cases.permeability_case((20, 18, 24), seed=9, precision=P.PREC_F32)),
    ("d3_permeability_f16_storage_shifted", perm_f16),
]


@pytest.mark.parametrize("name", [n for n, _ in CASES])
def test_conservation_equals_host_sums(name):
    p, walls, rho = dict(CASES)[name]()
    h = Handle(p)
    h.upload_walls(walls)
    h.upload_state(rho)
    h.init()
    h.step(7)
    mass, mom = h.conservation()
    mass_h, mom_h = host_totals(p, h.download(P.FIELD_FI))
    assert mass.shape == (p.ncomponents,) and mom.shape == (p.ncomponents, p.ndims)
    assert np.all(np.abs(mass / mass_h - 1.0) <= 1e-12), (mass, mass_h)
    scale = np.abs(mass_h).max()
    assert np.all(np.abs(mom - mom_h) <= 1e-12 * scale), (mom, mom_h)
    mass2, mom2 = h.conservation()
    assert np.array_equal(mass, mass2) and np.array_equal(mom, mom2)
    h.close()


def test_periodic_bubble_conserves_mass():
    p, walls, rho = cases.sc_bubble(P.D3Q19, (16, 12, 14), P.MRT, 4)
    h = Handle(p)
    h.upload_walls(walls)
    h.upload_state(rho)
    h.init()
    m0, _ = h.conservation()
    h.step(20)
    m1, _ = h.conservation()
    h.close()
    assert np.all(np.abs(m1 / m0 - 1.0) < 1e-10), (m0, m1)


def test_conservation_before_init_is_an_error():
    p, walls, rho = cases.sc_bubble(P.D3Q19, (8, 8, 8), P.SRT, 4)
    h = Handle(p)
    h.upload_walls(walls)
    with pytest.raises(TxError) as e:
        h.conservation()
    assert e.value.code == 2
    h.close()
