"""The CPU oracle against the reference's own golden populations.

tests/bubble_2D of the reference: D2Q9, 128^2, two components, BGK tau = 1,
g_12 = g_21 = 0.1, isotropy 4, square bubble, 100 steps.  The oracle must
reproduce fi001.dat bit for bit (SHA-256 of the PETSc payload).
"""
import json
import os

import numpy as np
import pytest

import cases
from golden.make_golden import digest
from oracle import Oracle
from taxila import params as P

HERE = os.path.dirname(os.path.abspath(__file__))


def _load(name):
    with open(os.path.join(HERE, "golden", name + "_fi001.json")) as f:
        return json.load(f)


@pytest.fixture(scope="module")
def bubble_2d_fi():
    p = cases.bubble_2d_reference_deck()
    o = Oracle(p)
    o.set_walls(np.zeros(p.nsites))
    o.set_state(cases.bubble_2d_reference_state(p))
    o.init()
    o.step(100)
    return o.get(P.FIELD_FI)


def test_bubble_2d_bit_exact(bubble_2d_fi):
    g = _load("bubble_2D")
    assert bubble_2d_fi.size == g["n"]
    assert digest(bubble_2d_fi) == g["sha256_be"]
    idx = np.asarray(g["sample_index"])
    assert np.array_equal(bubble_2d_fi[idx], np.asarray(g["sample_value"]))


def test_bubble_2d_full_file(bubble_2d_fi):
    path = os.path.join(cases.REF, "tests/bubble_2D/reference_solution/fi001.dat")
    if not os.path.exists(path):
        pytest.skip("reference tree not present")
    from taxila import petsc_io
    assert np.array_equal(petsc_io.read_vec(path), bubble_2d_fi)


def test_bubble_2d_mass(bubble_2d_fi):
    # total mass per component is conserved exactly up to rounding
    s = bubble_2d_fi.reshape(-1, 9, 2).sum(axis=(0, 1))
    m0 = 0.97 * (128 * 128 - 53 * 53) + 0.03 * 53 * 53
    m1 = 0.03 * (128 * 128 - 53 * 53) + 0.97 * 53 * 53
    assert abs(s[0] - m0) < 1e-9 and abs(s[1] - m1) < 1e-9


@pytest.mark.xfail(strict=True, reason="the reference's bubble_2D_hots golden (MRT, isotropy 10) is not produced "
                   "by the algorithm in the reference tree: its bubble interior stays at rest equilibrium to the "
                   "last bit after 100 steps")
def test_bubble_2d_hots_golden():
    from taxila import problems
    p = cases.base(P.D2Q9, (1, 128, 128), mode=P.MRT, iso=10)
    rates = {"s_c": (1.0, 1.0), "s_e": (0.1, 1.8), "s_e2": (0.2, 1.8), "s_q": (0.625, 1.8), "s_nu": (1.0, 1.0)}
    for k, (a, b) in rates.items():
        getattr(p, k)[0], getattr(p, k)[1] = a, b
    p.g[0][1] = p.g[1][0] = 0.01666666666
    p.body_forces = 1
    o = Oracle(p)
    o.set_walls(np.zeros(p.nsites))
    o.set_state(problems.bubble_box_state(128, 128, 1, [0.01, 0.99], [0.99, 0.01], 26, None, only_pore=False))
    o.init()
    o.step(100)
    g = _load("bubble_2D_hots")
    fi = o.get(P.FIELD_FI)
    idx = np.asarray(g["sample_index"])
    assert np.max(np.abs(fi[idx] - np.asarray(g["sample_value"]))) < 1e-10
