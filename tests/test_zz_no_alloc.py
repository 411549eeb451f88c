"""tx_step_static: the flow step for callers that cannot allocate device memory.

Callers that own all device memory themselves (an application arena, a plugin
handed buffers by its host) pass their own device arrays; the entry point
takes its working storage from the library's static device array instead of
allocating.  Its result must equal the handle-based path it mirrors
(tx_upload_fi + tx_init + tx_step + tx_download), on two calls in a row.
This file is collected last so that a failure here leaves every other test
already run.
"""
import numpy as np
import pytest

import cases
from taxila import params as P
from taxila._lib import Handle, TxError, step_static

pytestmark = pytest.mark.gpu
RTOL = 1e-12


def handle_path(p, walls, fi_in, n):
    h = Handle(p)
    h.upload_walls(walls)
    h.upload_fi(fi_in)
    h.init()
    h.step(n)
    out = h.download(P.FIELD_FI)
    h.close()
    return out


def rel_err(a, b, pore):
    return np.max(np.abs(a[pore] - b[pore])) / np.max(np.abs(a[pore]))


def test_static_step_matches_handle_twice():
    import torch
    p, walls, rho = cases.porous_case(P.D3Q19, (12, 10, 14), mode=P.MRT, body=True)
    h0 = Handle(p)
    h0.upload_walls(walls)
    h0.upload_state(rho)
    h0.init()
    h0.step(3)
    fi0 = h0.download(P.FIELD_FI)
    h0.close()
    pore = np.repeat(np.asarray(walls) == 0, p.ncomponents * p.Q)

    d_walls = torch.tensor(walls, dtype=torch.float64, device="cuda")
    d_in = torch.tensor(fi0, dtype=torch.float64, device="cuda")
    d_out = torch.empty_like(d_in)
    step_static(p, d_walls.data_ptr(), d_in.data_ptr(), d_out.data_ptr(), 5)
    out1 = d_out.cpu().numpy()
    assert np.array_equal(d_in.cpu().numpy(), fi0), "fi_in must not be modified"
    assert rel_err(handle_path(p, walls, fi0, 5), out1, pore) <= RTOL

    # second call in a row, continuing from the first output (the static array keeps the last call's contents)
    d_in2 = d_out.clone()
    d_out2 = torch.empty_like(d_in2)
    step_static(p, d_walls.data_ptr(), d_in2.data_ptr(), d_out2.data_ptr(), 4)
    out2 = d_out2.cpu().numpy()
    assert rel_err(handle_path(p, walls, out1, 4), out2, pore) <= RTOL
    assert np.all(out2[~pore] == 0.0)


@pytest.mark.parametrize("name", ["d3_two_phase_pressure", "d3_reflect_momentum", "d2_velocity_outlet"])
def test_static_step_with_exterior_bcs(name):
    # outlet refresh and face pass in the allocation-free step
    import torch
    p, walls, rho = next(m for n, m, _ in cases.BCS if n == name)()
    h0 = Handle(p)
    h0.upload_walls(walls)
    h0.upload_state(rho)
    h0.init()
    h0.step(2)
    fi0 = h0.download(P.FIELD_FI)
    h0.close()
    pore = np.repeat(np.asarray(walls) == 0, p.ncomponents * p.Q)
    d_walls = torch.tensor(walls, dtype=torch.float64, device="cuda")
    d_in = torch.tensor(fi0, dtype=torch.float64, device="cuda")
    d_out = torch.empty_like(d_in)
    step_static(p, d_walls.data_ptr(), d_in.data_ptr(), d_out.data_ptr(), 6)
    assert np.array_equal(handle_path(p, walls, fi0, 6)[pore], d_out.cpu().numpy()[pore])


def test_static_step_rejects_lattices_beyond_the_static_area():
    import torch
    p = cases.base(P.D3Q19, (64, 64, 64))
    p.g[0][1] = p.g[1][0] = 0.1
    d = torch.zeros(8, dtype=torch.float64, device="cuda")
    with pytest.raises(TxError) as e:
        step_static(p, d.data_ptr(), d.data_ptr(), d.data_ptr(), 1)
    assert e.value.code == 1 and "bytes of working storage" in str(e.value)


def test_static_step_rejects_bad_wall_codes_before_stepping():
    # a negative wall code is refused before any step: fi_out keeps what the caller put there
    import torch
    p, walls, rho = cases.porous_case(P.D3Q19, (12, 10, 14), mode=P.MRT, body=True)
    bad = np.array(walls, dtype=np.float64)
    bad[5] = -1.0
    d_walls = torch.tensor(bad, dtype=torch.float64, device="cuda")
    n = p.nsites * p.ncomponents * p.Q
    d_in = torch.ones(n, dtype=torch.float64, device="cuda")
    d_out = torch.full((n,), 7.0, dtype=torch.float64, device="cuda")
    with pytest.raises(TxError) as e:
        step_static(p, d_walls.data_ptr(), d_in.data_ptr(), d_out.data_ptr(), 3)
    assert e.value.code == 1 and "wall codes" in str(e.value)
    assert torch.all(d_out == 7.0).item()
