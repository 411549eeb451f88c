"""GPU parity: the CUDA library against the CPU oracle through the C ABI.

* exact FP64 form (reference operation order, no FMA): populations, densities,
  velocities and forces identical to the oracle bit for bit;
* fast FP64 form: populations, densities and velocities within 1e-12 relative
  of the oracle after the stated number of steps;
* the reference's own golden (tests/bubble_2D, 100 steps) reproduced through
  the GPU bit for bit by the exact form.
"""
import json
import os

import numpy as np
import pytest

import cases
from golden.make_golden import digest
from oracle import Oracle
from taxila import params as P
from taxila._lib import Handle, TxError

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
FIELDS = (P.FIELD_FI, P.FIELD_RHO, P.FIELD_FLUX, P.FIELD_FORCES)


def run_pair(p, walls, rho, steps, exact, fi=None, u=None):
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
        o.set_state(rho, u)
        h.upload_state(rho, u)
    o.init()
    h.init()
    if steps:
        o.step(steps)
        h.step(steps)
    return o, h


def pore(p, walls, dof):
    return np.repeat(np.asarray(walls).ravel() == 0, dof)


def compare(o, h, p, walls, exact, rtol=1e-12):
    out = {}
    for f in FIELDS:
        a, b = o.get(f), h.download(f)
        dof = a.size // p.nsites
        mask = pore(p, walls, dof)
        if exact:
            bad = np.nonzero((a != b) & mask)[0]
            assert bad.size == 0, "field %d: %d sites differ, first %s: %r vs %r" % (
                f, bad.size, bad[:3], a[bad[:3]], b[bad[:3]])
        else:
            scale = np.max(np.abs(a[mask])) or 1.0
            err = np.max(np.abs(a[mask] - b[mask])) / scale
            out[f] = err
            assert err <= rtol, "field %d: max rel err %.3e > %.1e" % (f, err, rtol)
        # wall sites hold zeros on the device
        assert np.all(b[~mask] == 0.0)
    return out


PARITY = cases.PARITY


@pytest.mark.parametrize("name,make,steps", PARITY, ids=[c[0] for c in PARITY])
def test_exact_form_bit_identical(name, make, steps):
    p, walls, rho = make()
    o, h = run_pair(p, walls, rho, steps, exact=True)
    compare(o, h, p, walls, exact=True)


@pytest.mark.parametrize("name,make,steps", PARITY, ids=[c[0] for c in PARITY])
def test_fast_form_within_1e12(name, make, steps):
    p, walls, rho = make()
    o, h = run_pair(p, walls, rho, steps, exact=False)
    compare(o, h, p, walls, exact=False)


def test_init_state_bit_identical():
    # FlowFiInit + FlowUpdateMoments alone, with a nonzero initial velocity
    p, walls, rho = cases.porous_case(P.D3Q19, (10, 10, 10), body=True)
    rng = np.random.default_rng(5)
    u = 1e-3 * rng.standard_normal(p.nsites * p.ndims * p.ncomponents)
    o, h = run_pair(p, walls, rho, 0, exact=True, u=u)
    compare(o, h, p, walls, exact=True)


def test_upload_fi_restart_bit_identical():
    p, walls, rho = cases.sc_bubble(P.D3Q19, (10, 12, 10), P.MRT, 4)
    o0 = Oracle(p)
    o0.set_walls(walls)
    o0.set_state(rho)
    o0.init()
    o0.step(3)
    fi = o0.get(P.FIELD_FI)
    o, h = run_pair(p, walls, None, 5, exact=True, fi=fi)
    compare(o, h, p, walls, exact=True)


def test_reference_golden_through_gpu():
    p = cases.bubble_2d_reference_deck()
    p.exact = 1
    h = Handle(p)
    h.upload_walls(np.zeros(p.nsites))
    h.upload_state(cases.bubble_2d_reference_state(p))
    h.init()
    h.step(100)
    fi = h.download(P.FIELD_FI)
    with open(os.path.join(HERE, "golden", "bubble_2D_fi001.json")) as f:
        g = json.load(f)
    assert digest(fi) == g["sha256_be"]


def test_fast_form_1000_steps_within_1e12():
    # the tolerance is stated after 1,000 steps; a smaller lattice keeps the oracle quick
    p, walls, rho = cases.sc_bubble(P.D3Q19, (16, 16, 16), P.MRT, 4, g=0.15, r=4)
    o, h = run_pair(p, walls, rho, 1000, exact=False)
    errs = compare(o, h, p, walls, exact=False)
    print("fast FP64 after 1000 steps:", errs)


def test_diagnostics_match_oracle():
    p, walls, rho = cases.porous_case(P.D3Q19, (10, 12, 8), body=True)
    o, h = run_pair(p, walls, rho, 7, exact=True)
    for f in (P.FIELD_PRS, P.FIELD_VELT, P.FIELD_RHOT):
        a, b = o.get(f), h.download(f)
        assert np.array_equal(a, b), f


@pytest.mark.parametrize("make", [lambda: cases.sc_bubble(P.D2Q9, (1, 32, 32), P.SRT, 4),
                                  lambda: cases.sc_bubble(P.D3Q19, (12, 14, 16), P.MRT, 4),
                                  lambda: cases.porous_case(P.D3Q19, (10, 12, 14), mode=P.MRT, body=True)],
                         ids=["d2_periodic", "d3_periodic", "d3_porous_density_faces"])
def test_delta_norm_matches_oracle(make):
    # periodic lattices read the density in place, density faces stage it; both
    # screen the FP64 divisions and must return the oracle's norm bit for bit
    p, walls, rho = make()
    o, h = run_pair(p, walls, rho, 0, exact=True)
    for k in range(6):
        o.step(1 + k % 2)
        h.step(1 + k % 2)
        assert o.delta_norm(P.FIELD_RHO) == h.delta_norm(P.FIELD_RHO)
        assert o.delta_norm(P.FIELD_FI) == h.delta_norm(P.FIELD_FI)


def test_errors_are_status_codes():
    p = cases.base(P.D3Q19, (4, 4, 4))
    p.isotropy_order = 10
    with pytest.raises(TxError) as e:
        Handle(p)
    assert e.value.code == 1
    p.isotropy_order = 4
    h = Handle(p)
    with pytest.raises(TxError) as e:
        h.step(1)  # before init
    assert e.value.code == 2
    w = np.zeros(p.nsites)
    w[3] = -1.0
    with pytest.raises(TxError):
        h.upload_walls(w)


def test_refused_wall_codes_leave_the_walls():
    # wall codes are converted on the device; a refused upload (negative, NaN,
    # infinite) changes nothing, and the next run equals the oracle
    p, walls, rho = cases.porous_case(P.D3Q19, (10, 12, 8), body=True)
    o, h = run_pair(p, walls, rho, 0, exact=True)
    for bad in (-1.0, float("nan"), float("inf"), -float("inf")):
        w = np.array(walls, dtype=np.float64)
        w[17] = bad
        with pytest.raises(TxError) as e:
            h.upload_walls(w)
        assert e.value.code == 1
        assert np.array_equal(h.download(P.FIELD_WALLS), np.where(walls >= 998.0, 999.0, walls))
    h.step(5)
    o.step(5)
    compare(o, h, p, walls, exact=True)
    # an unknown mineral or a code at or above 998 is a plain wall
    w = np.array(walls, dtype=np.float64)
    w[w == 2.0] = 7.0
    w[w == 1.0] = 1e300
    h.upload_walls(w)
    assert set(np.unique(h.download(P.FIELD_WALLS))) <= {0.0, 999.0}
