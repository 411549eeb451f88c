"""Non-ideal equations of state on the GPU against the oracle (C ABI).

psi(rho) replaces rho in the fluid-fluid force and the pressure diagnostic.
The exact form is bit-identical for psi = rho and Peng-Robinson (IEEE
divide and square root); the Shan-Chen and thermo EOS call exp, whose
device implementation is not the host library's, so those compare within
1e-12, as does the fast form.
"""
import numpy as np
import pytest

import cases
from oracle import Oracle
from taxila import params as P
from taxila._lib import Handle

pytestmark = pytest.mark.gpu
FIELDS = (P.FIELD_FI, P.FIELD_RHO, P.FIELD_FORCES, P.FIELD_PSI, P.FIELD_PRS)


@pytest.mark.parametrize("name,make,steps", cases.EOS, ids=[c[0] for c in cases.EOS])
@pytest.mark.parametrize("exact", [True, False], ids=["exact", "fast"])
def test_eos_matches_oracle(name, make, steps, exact):
    p, walls, rho = make()
    o = Oracle(p)
    o.set_walls(walls)
    o.set_state(rho)
    o.init()
    o.step(steps)
    q = P.copy_params(p)
    q.exact = 1 if exact else 0
    h = Handle(q)
    h.upload_walls(walls)
    h.upload_state(rho)
    h.init()
    h.step(steps)
    bitwise = exact and p.eos[0] in (P.EOS_RHO, P.EOS_PR)
    for f in FIELDS:
        a, b = o.get(f), h.download(f)
        if bitwise:
            assert np.array_equal(a, b), f
        else:
            scale = np.max(np.abs(a)) or 1.0
            assert np.max(np.abs(a - b)) / scale <= 1e-12, (f, np.max(np.abs(a - b)) / scale)
