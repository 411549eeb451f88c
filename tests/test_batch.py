"""Batched lattices (tx_batch_*): one persistent tile-table launch per kernel
for many lattices of one form, replayed as a CUDA graph.

* every lattice of a batch evolves exactly as the same lattice alone in a
  tx_handle of the same form (identical per-site code: populations equal bit
  for bit), whatever else is in the batch, whenever it joined, whatever the
  tile shape;
* the probe statistics equal the ones computed from the downloaded velocity;
* the device-memory budget gates admission.
"""
import numpy as np
import pytest

import cases
from taxila import params as P
from taxila._lib import Batch, Handle, TxError

pytestmark = pytest.mark.gpu


def form_of(p):
    q = P.copy_params(p)
    q.exact = 0
    return q


def alone(p, walls, rho, steps):
    q = form_of(p)
    h = Handle(q)
    h.upload_walls(walls)
    h.upload_state(rho)
    h.init()
    if steps:
        h.step(steps)
    return h


def two_phase_mix():
    a = cases.sc_bubble(P.D3Q19, (16, 12, 14), P.MRT, 4)
    b = cases.porous_case(P.D3Q19, (12, 10, 14), mode=P.MRT, body=True)
    c = cases.sc_bubble(P.D3Q19, (10, 18, 12), P.MRT, 4, g=0.1, r=3)
    # the batch form is that of the first; the others share it
    return [a, b, c]


def nfi(p):
    return p.nsites * p.ncomponents * p.Q


def test_batch_equals_lattices_alone():
    mix = two_phase_mix()
    b = Batch(form_of(mix[0][0]))
    ids = [b.add(form_of(p), w, r) for p, w, r in mix]
    b.step(25)  # one 20-step graph and 5 direct steps: ends on the odd buffer
    for (p, w, r), lid in zip(mix, ids):
        h = alone(p, w, r, 25)
        got = b.download(lid, P.FIELD_FI, nfi(p))
        assert np.array_equal(got, h.download(P.FIELD_FI))
        assert np.array_equal(b.download(lid, P.FIELD_RHO, p.nsites * p.ncomponents), h.download(P.FIELD_RHO))


def test_join_and_leave_between_steps():
    mix = two_phase_mix()
    b = Batch(form_of(mix[0][0]))
    ia = b.add(form_of(mix[0][0]), mix[0][1], mix[0][2])
    b.step(7)
    ib = b.add(form_of(mix[1][0]), mix[1][1], mix[1][2])
    b.step(30)
    b.remove(ia)
    ic = b.add(form_of(mix[2][0]), mix[2][1], mix[2][2])
    b.step(12)
    assert b.count() == 2
    for (p, w, r), lid, steps in ((mix[1], ib, 42), (mix[2], ic, 12)):
        h = alone(p, w, r, steps)
        assert np.array_equal(b.download(lid, P.FIELD_FI, nfi(p)), h.download(P.FIELD_FI))
    with pytest.raises(TxError):
        b.download(ia, P.FIELD_FI, nfi(mix[0][0]))


def test_tile_shapes_and_tuner_keep_results():
    mix = two_phase_mix()
    b = Batch(form_of(mix[0][0]))
    ids = [b.add(form_of(p), w, r) for p, w, r in mix]
    b.set_tiles(128, 1, 1, 8)
    b.step(3)
    b.set_tiles(16, 4, 2, 4)
    b.step(3)
    chosen = b.tune(2)  # 12 candidates x 3 steps
    assert chosen[0] * chosen[1] * chosen[2] == 128
    b.step(4)
    total = 10 + 12 * 3
    probes = b.probe()
    for (p, w, r), lid in zip(mix, ids):
        assert probes[lid].steps == total
        h = alone(p, w, r, total)
        assert np.array_equal(b.download(lid, P.FIELD_FI, nfi(p)), h.download(P.FIELD_FI))


def test_probe_matches_downloaded_velocity():
    p, w, r = cases.permeability_case((14, 12, 16), seed=5)
    b = Batch(form_of(p))
    lid = b.add(form_of(p), w, r)
    b.step(10)
    pr1 = b.probe()[lid]
    u1 = b.download(lid, P.FIELD_FLUX, p.nsites * 3).reshape(p.nsites, 3)
    b.step(6)
    pr2 = b.probe()[lid]
    u2 = b.download(lid, P.FIELD_FLUX, p.nsites * 3).reshape(p.nsites, 3)
    pore = w == 0
    assert pr1.pore_sites == pore.sum() == pr2.pore_sites
    assert pr1.du_max == np.max(np.abs(u1[pore]))   # first probe compares with zero
    assert pr2.du_max == np.max(np.abs(u2[pore] - u1[pore]))
    assert pr2.u_max == np.max(np.abs(u2[pore]))
    for d in range(3):
        assert pr2.u_sum[d] == pytest.approx(u2[pore, d].sum(), rel=1e-12, abs=1e-300)
    assert pr2.steps == 16


def test_budget_gates_admission():
    p, w, r = cases.permeability_case((12, 12, 12), seed=2)
    need = Batch.lattice_bytes(p)
    b = Batch(form_of(p), hbm_budget_bytes=int(2.5 * need))
    b.add(form_of(p), w, r)
    b.add(form_of(p), w, r)
    with pytest.raises(TxError) as e:
        b.add(form_of(p), w, r)
    assert e.value.code == 4
    assert b.bytes_in_use() == 2 * need


def test_form_mismatch_is_rejected():
    p, w, r = cases.permeability_case((8, 8, 8))
    b = Batch(form_of(p))
    q = P.copy_params(p)
    q.precision = P.PREC_F32
    with pytest.raises(TxError):
        b.add(q, w, r)


def test_batch_with_species_equals_alone():
    mk = [cases.porous_case(P.D3Q19, (12, 10, 14), body=True), cases.porous_case(P.D3Q19, (10, 12, 9), body=True, seed=8)]
    items = []
    for p, w, r in mk:
        conc = cases.with_species(p, w, mode=P.SRT, tau=0.8)
        items.append((p, w, r, conc))
    b = Batch(form_of(items[0][0]))
    ids = [b.add(form_of(p), w, r, conc=c) for p, w, r, c in items]
    b.step(23)
    for (p, w, r, c), lid in zip(items, ids):
        q = form_of(p)
        h = Handle(q)
        h.upload_walls(w)
        h.upload_state(r)
        h.upload_species(c)
        h.init()
        h.step(23)
        for f in (P.FIELD_FI, P.FIELD_SPECIES_FI, P.FIELD_SPECIES_RHO):
            assert np.array_equal(b.download(lid, f, h.L.tx_field_size(h.h, f)), h.download(f)), f


def test_probe_mass_matches_downloaded_density():
    # each component's mass in the probe is the sum of the downloaded density
    # over pore sites (a periodic two-phase bubble: no density faces)
    p, w, r = cases.sc_bubble(P.D3Q19, (16, 12, 14), P.MRT, 4)
    q = form_of(p)
    q.precision = P.PREC_F32
    b = Batch(q)
    lid = b.add(q, w, r)
    b.step(8)
    pr = b.probe()[lid]
    rho = b.download(lid, P.FIELD_RHO, p.nsites * p.ncomponents).reshape(p.nsites, p.ncomponents)
    pore = np.asarray(w) == 0
    for m in range(p.ncomponents):
        assert pr.mass[m] == pytest.approx(rho[pore, m].sum(), rel=1e-6)
    b.close()
