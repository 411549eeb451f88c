"""The bench workload at its full size (D3Q19 128^3, two components, MRT,
FP64): parity with the oracle and size-independent properties.

* the exact form is bit-identical to the oracle after 10 steps over all
  2,097,152 sites (the oracle runs them on the host cores in seconds);
* over 200 steps of the periodic lattice, each component's mass is conserved
  and the total momentum stays zero (the Shan-Chen force of a symmetric
  coupling sums to zero over a periodic lattice), to round-off; the fast
  form drifts no more than the reference-order (exact) form.
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import bench  # noqa: E402
from oracle import Oracle  # noqa: E402
from taxila import params as P  # noqa: E402
from taxila._lib import Handle  # noqa: E402

pytestmark = pytest.mark.gpu


def test_full_size_exact_form_bit_identical():
    p = bench.workload_params(P.PREC_F64)
    walls, rho = bench.workload_state(p)
    q = P.copy_params(p)
    q.exact = 1
    h = Handle(q)
    h.upload_walls(walls)
    h.upload_state(rho)
    h.init()
    h.step(10)
    o = Oracle(p)
    o.set_walls(walls)
    o.set_state(rho)
    o.init()
    o.step(10)
    for f in (P.FIELD_RHO, P.FIELD_FI):
        a, b = o.get(f), h.download(f)
        bad = np.count_nonzero(a != b)
        assert bad == 0, "field %d: %d of %d values differ" % (f, bad, a.size)
    h.close()


def _drift(exact, steps):
    p = bench.workload_params(P.PREC_F64)
    p.exact = 1 if exact else 0
    walls, rho = bench.workload_state(p)
    h = Handle(p)
    h.upload_walls(walls)
    h.upload_state(rho)
    h.init()
    s = p.ncomponents
    m0 = h.download(P.FIELD_RHO).reshape(p.nsites, s).sum(axis=0)
    h.step(steps)
    r = h.download(P.FIELD_RHO).reshape(p.nsites, s)
    m1 = r.sum(axis=0)
    # common velocity times the total density: the lattice's momentum per unit mass
    u = h.download(P.FIELD_FLUX).reshape(p.nsites, p.ndims, s)[:, :, 0]
    mom = (u * r.sum(axis=1)[:, None]).sum(axis=0) / m1.sum()
    h.close()
    return np.abs(m1 / m0 - 1.0), np.abs(mom)


def test_full_size_mass_and_momentum_conserved():
    # both forms drift by round-off only; the fast form no more than the
    # reference-order (exact) form, within a factor, and both far below 1e-9
    dm_fast, mom_fast = _drift(False, 200)
    dm_exact, mom_exact = _drift(True, 200)
    print("mass drift fast", dm_fast, "exact", dm_exact, "momentum fast", mom_fast, "exact", mom_exact)
    assert np.all(dm_fast < 1e-9) and np.all(dm_exact < 1e-9)
    assert np.all(dm_fast <= 10 * dm_exact + 1e-13)
    assert np.all(mom_fast < 1e-12) and np.all(mom_exact < 1e-12)
