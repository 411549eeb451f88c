"""Host emulation of the CUDA kernels against the oracle (CPU only).

The kernels of taxila-lbm_gb300/csrc/tx_kernels.cuh, compiled as C++ with
AddressSanitizer/UBSan (tests/hostemu), run the GPU parity matrix on the CPU
with the library's own parameter translation and launch shapes:

* exact FP64 form: populations, densities, velocities and forces identical to
  the oracle bit for bit (the device build adds only --fmad=false, which the
  host compiler matches with -ffp-contract=off);
* fast FP64 form: within 1e-12 relative of the oracle;
* FP32 arithmetic forms: within the bounds stated in FORM_TOL.

Every index a kernel forms is checked by the sanitizers, so an out-of-bounds
read or write in a kernel fails here before it reaches a GPU.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

import cases
from oracle import Oracle
from taxila import params as P

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "hostemu"))
import build_emu  # noqa: E402

FIELDS = ("fi", "rho", "flux", "forces")
ORACLE_FIELDS = {"fi": P.FIELD_FI, "rho": P.FIELD_RHO, "flux": P.FIELD_FLUX, "forces": P.FIELD_FORCES}
# bound on max |emu - oracle| / max |oracle| over pore sites after 20 steps of the
# D3Q19 MRT bubble: FP32 arithmetic and storage; FP32 arithmetic with FP16 storage of
# f - w rho0 (11-bit significand: ~5e-4 of the deviation; the flux, a small
# difference of populations, carries the largest relative error)
FORM_TOL = {P.PREC_F32: {"fi": 2e-5, "rho": 2e-5, "flux": 2e-5, "forces": 2e-5},
            P.PREC_F32_F16: {"fi": 2e-3, "rho": 2e-3, "flux": 3e-2, "forces": 3e-3}}


@pytest.fixture(scope="module")
def emu_exe():
    os.environ.setdefault("ASAN_OPTIONS", "detect_leaks=0")
    return build_emu.build()


SPECIES_FIELDS = ("sfi", "srho", "sflux")


def run_emu(exe, p, walls, init, steps, from_fi, tmp_path, conc=None):
    case = os.path.join(str(tmp_path), "case.bin")
    res = os.path.join(str(tmp_path), "result.bin")
    with open(case, "wb") as f:
        f.write(C.string_at(C.addressof(p), C.sizeof(p)))
        f.write(np.array([steps, 1 if from_fi else 0], dtype=np.int32).tobytes())
        f.write(np.ascontiguousarray(walls, dtype=np.float64).tobytes())
        f.write(np.ascontiguousarray(init, dtype=np.float64).tobytes())
        if p.nspecies > 0:
            f.write(np.ascontiguousarray(conc, dtype=np.float64).tobytes())
    r = subprocess.run([exe, case, res], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, "emu exit %d: %s" % (r.returncode, r.stderr[-3000:])
    raw = np.fromfile(res, dtype=np.float64)
    n, s, d, q, ns = p.nsites, p.ncomponents, p.ndims, p.Q, p.nspecies
    sizes = {"fi": n * s * q, "rho": n * s, "flux": n * s * d, "forces": n * s * d,
             "sfi": n * ns * q, "srho": n * ns, "sflux": n * ns * d}
    out, o = {}, 0
    for k in FIELDS + (SPECIES_FIELDS if ns else ()):
        out[k] = raw[o:o + sizes[k]]
        o += sizes[k]
    assert o == raw.size
    return out


def oracle_run(p, walls, rho, steps, fi=None):
    o = Oracle(p)
    o.set_walls(walls)
    if fi is not None:
        o.set_fi(fi)
    else:
        o.set_state(rho)
    o.init()
    if steps:
        o.step(steps)
    return {k: o.get(v) for k, v in ORACLE_FIELDS.items()}


def compare(ref, got, p, walls, tol, fields=FIELDS):
    pore = np.asarray(walls).ravel() == 0
    errs = {}
    for k in fields:
        a, b = ref[k], got[k]
        t = tol[k] if isinstance(tol, dict) else tol
        m = np.repeat(pore, a.size // p.nsites)
        assert np.all(b[~m] == 0.0), k
        if t == 0.0:
            bad = np.nonzero((a != b) & m)[0]
            assert bad.size == 0, "%s: %d values differ, first %s: %r vs %r" % (k, bad.size, bad[:3], a[bad[:3]], b[bad[:3]])
        else:
            scale = np.max(np.abs(a[m])) or 1.0
            errs[k] = float(np.max(np.abs(a[m] - b[m])) / scale)
            assert errs[k] <= t, "%s: max rel err %.3e > %.1e" % (k, errs[k], t)
    return errs


@pytest.mark.parametrize("name,make,steps", cases.PARITY, ids=[c[0] for c in cases.PARITY])
@pytest.mark.parametrize("exact", [True, False], ids=["exact", "fast"])
def test_emulated_kernels_match_oracle(emu_exe, tmp_path, name, make, steps, exact):
    p, walls, rho = make()
    ref = oracle_run(p, walls, rho, steps)
    q = P.copy_params(p)
    q.exact = 1 if exact else 0
    got = run_emu(emu_exe, q, walls, rho, steps, False, tmp_path)
    compare(ref, got, p, walls, 0.0 if exact else 1e-12)


def test_emulated_restart_from_fi(emu_exe, tmp_path):
    p, walls, rho = cases.porous_case(P.D3Q19, (10, 12, 10), mode=P.MRT, body=True)
    o = Oracle(p)
    o.set_walls(walls)
    o.set_state(rho)
    o.init()
    o.step(3)
    fi = o.get(P.FIELD_FI)
    ref = oracle_run(p, walls, None, 5, fi=fi)
    q = P.copy_params(p)
    q.exact = 1
    got = run_emu(emu_exe, q, walls, fi, 5, True, tmp_path)
    compare(ref, got, p, walls, 0.0)


@pytest.mark.parametrize("prec", [P.PREC_F32, P.PREC_F32_F16], ids=["f32", "f32_f16"])
@pytest.mark.parametrize("shape,nu_only", [((12, 12, 14), False), ((12, 12, 13), False), ((12, 12, 13), True)],
                         ids=["mixed_rates", "odd_nx", "odd_nx_s_nu_only"])
def test_emulated_reduced_precision_forms(emu_exe, tmp_path, prec, shape, nu_only):
    # odd nx: paired cells span row ends; s_nu only: the closed-form stress correction
    p, walls, rho = cases.sc_bubble(P.D3Q19, shape, P.MRT, 4, g=0.15, nu_only=nu_only)
    ref = oracle_run(p, walls, rho, 20)
    q = P.copy_params(p)
    q.precision = prec
    q.rho0[0] = q.rho0[1] = 0.0  # two phases: no single rest density; plain storage
    got = run_emu(emu_exe, q, walls, rho, 20, False, tmp_path)
    errs = compare(ref, got, p, walls, FORM_TOL[prec])
    print("form %d after 20 steps:" % prec, errs)


@pytest.mark.parametrize("prec,scale", [(P.PREC_F32, 1.0), (P.PREC_F32_F16, 4096.0)], ids=["f32", "f32_f16"])
@pytest.mark.parametrize("shape", [(14, 12, 16), (14, 12, 15)], ids=["even_nx", "odd_nx"])
def test_emulated_permeability_precision(emu_exe, tmp_path, prec, scale, shape):
    # single-phase body-force flow through a sphere pack, deviations stored
    # from rho0 = 1: the Darcy velocity (hence the permeability) within 1e-3 of
    # the FP64 oracle, populations and density far tighter
    p, walls, rho = cases.permeability_case(shape, seed=5)
    ref = oracle_run(p, walls, rho, 40)
    q = P.copy_params(p)
    q.precision = prec
    q.rho0[0] = 1.0
    q.storage_scale = scale
    got = run_emu(emu_exe, q, walls, rho, 40, False, tmp_path)
    compare(ref, got, p, walls, {"fi": 1e-6, "rho": 1e-6, "flux": 1e-3, "forces": 1e-6})
    pore = walls == 0
    k_ref = cases.permeability(p, ref["flux"].reshape(-1, 3)[pore, 2].sum(), p.nsites)
    k_got = cases.permeability(p, got["flux"].reshape(-1, 3)[pore, 2].sum(), p.nsites)
    assert abs(k_got / k_ref - 1.0) < 1e-3


@pytest.mark.parametrize("name,make,steps", cases.SPECIES, ids=[c[0] for c in cases.SPECIES])
@pytest.mark.parametrize("exact", [True, False], ids=["exact", "fast"])
def test_emulated_species_match_oracle(emu_exe, tmp_path, name, make, steps, exact):
    p, walls, rho, conc = make()
    o = Oracle(p)
    o.set_walls(walls)
    o.set_state(rho)
    o.set_species(conc)
    o.init()
    o.step(steps)
    ref = {"sfi": o.get(P.FIELD_SPECIES_FI), "srho": o.get(P.FIELD_SPECIES_RHO),
           "sflux": o.get(P.FIELD_SPECIES_FLUX), "fi": o.get(P.FIELD_FI)}
    q = P.copy_params(p)
    q.exact = 1 if exact else 0
    got = run_emu(emu_exe, q, walls, rho, steps, False, tmp_path, conc=conc)
    compare(ref, got, p, walls, 0.0 if exact else 1e-12, fields=("fi",) + SPECIES_FIELDS)
    pore = walls == 0
    mass0 = np.asarray(conc).reshape(p.nsites, -1)[pore].sum(axis=0)
    assert np.allclose(got["srho"].reshape(p.nsites, -1)[pore].sum(axis=0), mass0, rtol=1e-12)


@pytest.mark.parametrize("name,make,steps", cases.EOS, ids=[c[0] for c in cases.EOS])
@pytest.mark.parametrize("exact", [True, False], ids=["exact", "fast"])
def test_emulated_eos_match_oracle(emu_exe, tmp_path, name, make, steps, exact):
    # psi(rho) from the EOS in the fluid-fluid force; the host's exp is the oracle's
    p, walls, rho = make()
    ref = oracle_run(p, walls, rho, steps)
    q = P.copy_params(p)
    q.exact = 1 if exact else 0
    got = run_emu(emu_exe, q, walls, rho, steps, False, tmp_path)
    compare(ref, got, p, walls, 0.0 if exact else 1e-12)


@pytest.mark.parametrize("name,make,steps", cases.BCS, ids=[c[0] for c in cases.BCS])
@pytest.mark.parametrize("exact", [True, False], ids=["exact", "fast"])
def test_emulated_exterior_bcs_match_oracle(emu_exe, tmp_path, name, make, steps, exact):
    # pressure, flux, momentum, velocity and reflecting faces, outlets, BCApply's class order
    p, walls, rho = make()
    ref = oracle_run(p, walls, rho, steps)
    q = P.copy_params(p)
    q.exact = 1 if exact else 0
    got = run_emu(emu_exe, q, walls, rho, steps, False, tmp_path)
    compare(ref, got, p, walls, 0.0 if exact else 1e-12)


BC_FORM_CASES = ["d3_pressure_s1", "d3_reflect_momentum", "d3_neumann_then_dirichlet"]


@pytest.mark.parametrize("name", BC_FORM_CASES)
@pytest.mark.parametrize("prec,scale", [(P.PREC_F32, 1.0), (P.PREC_F32_F16, 4096.0)], ids=["f32", "f32_f16"])
def test_emulated_exterior_bcs_reduced_precision(emu_exe, tmp_path, name, prec, scale):
    # the face pass in the FP32-arithmetic forms, deviations from rho0 = 1,
    # against the FP64 oracle
    make, steps = next((m, s) for n, m, s in cases.BCS if n == name)
    p, walls, rho = make()
    ref = oracle_run(p, walls, rho, steps)
    q = P.copy_params(p)
    q.precision = prec
    q.rho0[0] = 1.0
    q.storage_scale = scale
    got = run_emu(emu_exe, q, walls, rho, steps, False, tmp_path)
    tol = 1e-5 if prec == P.PREC_F32 else 2e-3
    errs = compare(ref, got, p, walls, {"fi": tol, "rho": tol, "flux": 50 * tol, "forces": 50 * tol})
    print(name, prec, errs)


@pytest.mark.parametrize("name", ["d3_two_phase_pressure", "d3_flux_velocity_mrt"])
def test_emulated_exterior_bcs_fast_form_1000_steps(emu_exe, tmp_path, name):
    # the fast form's tolerance is stated after 1,000 steps; driven flows through
    # pressure, flux and velocity faces hold it too
    make = next(m for n, m, _ in cases.BCS if n == name)
    p, walls, rho = make()
    ref = oracle_run(p, walls, rho, 1000)
    q = P.copy_params(p)
    q.exact = 0
    got = run_emu(emu_exe, q, walls, rho, 1000, False, tmp_path)
    errs = compare(ref, got, p, walls, 1e-12)
    print(name, errs)


def compare_all_cells(ref, got, tol):
    """Like compare, but every cell's populations count: with specular walls,
    wall cells hold populations (the moments stay zero on walls)."""
    for k in FIELDS:
        a, b = ref[k], got[k]
        assert np.all(np.isfinite(a)), k
        if tol == 0.0:
            bad = np.nonzero(a != b)[0]
            assert bad.size == 0, "%s: %d values differ, first %s: %r vs %r" % (k, bad.size, bad[:3], a[bad[:3]], b[bad[:3]])
        else:
            err = float(np.max(np.abs(a - b)) / (np.max(np.abs(a)) or 1.0))
            assert err <= tol, "%s: max rel err %.3e > %.1e" % (k, err, tol)


@pytest.mark.parametrize("name,make,steps", cases.SPECULAR, ids=[c[0] for c in cases.SPECULAR])
@pytest.mark.parametrize("exact", [True, False], ids=["exact", "fast"])
def test_emulated_specular_walls_match_oracle(emu_exe, tmp_path, name, make, steps, exact):
    # specular walls 900/901/902 next to ordinary walls: the step kernels plus the
    # route exceptions resolved at wall upload reproduce the reference's ordered
    # bounceback sweep, wall cells' populations included
    p, walls, rho = make()
    ref = oracle_run(p, walls, rho, steps)
    assert np.abs(ref["fi"].reshape(p.nsites, -1)[walls > 0]).sum() > 0.0  # wall cells do hold populations
    q = P.copy_params(p)
    q.exact = 1 if exact else 0
    got = run_emu(emu_exe, q, walls, rho, steps, False, tmp_path)
    compare_all_cells(ref, got, 0.0 if exact else 1e-12)


@pytest.mark.parametrize("name", ["d3_porous_mrt_iso8_dirichlet", "d2_periodic_2c"])
def test_emulated_specular_restart_with_wall_content(emu_exe, tmp_path, name):
    # populations uploaded into wall cells (a restart file) move on as the
    # reference's sweep moves them
    make = dict((c[0], c[1]) for c in cases.SPECULAR)[name]
    p, walls, rho = make()
    o = Oracle(p)
    o.set_walls(walls)
    o.set_state(rho)
    o.init()
    o.step(3)
    fi = o.get(P.FIELD_FI)
    o.close()
    assert np.abs(fi.reshape(p.nsites, -1)[walls > 0]).sum() > 0.0
    ref = oracle_run(p, walls, None, 5, fi=fi)
    q = P.copy_params(p)
    q.exact = 1
    got = run_emu(emu_exe, q, walls, fi, 5, True, tmp_path)
    compare_all_cells(ref, got, 0.0)


def test_delta_norm_screen_is_exact(emu_exe):
    # the delta norm divides in FP64 only where a single-precision screen says
    # the quotient may reach the running maximum; on sequences of ordinary,
    # near-tied, extreme and special values the result equals the plain
    # maximum of every FP64 quotient bit for bit
    r = subprocess.run([emu_exe, "norm"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]


@pytest.mark.parametrize("name,make,steps", cases.SPECULAR_BCS, ids=[c[0] for c in cases.SPECULAR_BCS])
def test_emulated_specular_walls_with_exterior_bcs(emu_exe, tmp_path, name, make, steps):
    # specular walls next to every exterior BC kind: the faces' pre-stream
    # copies and corrections act on the populations the sweep leaves
    p, walls, rho = make()
    ref = oracle_run(p, walls, rho, steps)
    q = P.copy_params(p)
    q.exact = 1
    got = run_emu(emu_exe, q, walls, rho, steps, False, tmp_path)
    compare_all_cells(ref, got, 0.0)


@pytest.mark.parametrize("name,make,steps", cases.SPECIES_SPECULAR, ids=[c[0] for c in cases.SPECIES_SPECULAR])
def test_emulated_species_with_specular_walls(emu_exe, tmp_path, name, make, steps):
    # the species stream and bounce back through the flow's sweep: the same
    # exceptions move their populations, wall cells included; in 2D the wall
    # cells are also collided (under MRT that mixes their slots)
    p, walls, rho, conc = make()
    o = Oracle(p)
    o.set_walls(walls)
    o.set_state(rho)
    o.set_species(conc)
    o.init()
    o.step(steps)
    ref = {"fi": o.get(P.FIELD_FI), "sfi": o.get(P.FIELD_SPECIES_FI), "srho": o.get(P.FIELD_SPECIES_RHO),
           "sflux": o.get(P.FIELD_SPECIES_FLUX)}
    o.close()
    sfi = ref["sfi"].reshape(p.nsites, -1)
    assert np.abs(sfi[walls > 0]).sum() > 0.0  # species populations held in wall cells
    q = P.copy_params(p)
    q.exact = 1
    got = run_emu(emu_exe, q, walls, rho, steps, False, tmp_path, conc=conc)
    for k, v in ref.items():
        assert np.all(np.isfinite(v)), k
        bad = np.nonzero(v != got[k])[0]
        assert bad.size == 0, "%s: %d values differ" % (k, bad.size)


@pytest.mark.parametrize("name,prec,rho0,scale", [("d3_periodic_1c", P.PREC_F32, 1.0, 1.0),
                                                  ("d3_periodic_1c", P.PREC_F32_F16, 1.0, 4096.0),
                                                  ("d3_periodic_1c", P.PREC_F32, 0.0, 1.0),
                                                  ("d2_periodic_2c", P.PREC_F32, 0.0, 1.0)],
                         ids=["d3_f32_rho0", "d3_f16_rho0", "d3_f32_plain", "d2_f32_two_components"])
def test_emulated_specular_walls_reduced_precision(emu_exe, tmp_path, name, prec, rho0, scale):
    # the FP32/FP16 forms store deviations from a rest state: the exceptions
    # copy stored values between slots of one speed (same weight, same offset)
    # and empty slots take the stored value of f = 0; every cell within the
    # forms' bounds of the FP64 oracle
    make = dict((c[0], c[1]) for c in cases.SPECULAR)[name]
    p, walls, rho = make()
    ref = oracle_run(p, walls, rho, 6)
    q = P.copy_params(p)
    q.precision = prec
    q.rho0[0] = rho0
    q.storage_scale = scale
    got = run_emu(emu_exe, q, walls, rho, 6, False, tmp_path)
    for k in FIELDS:
        a, b = ref[k], got[k]
        err = float(np.max(np.abs(a - b)) / np.max(np.abs(a)))
        assert err <= FORM_TOL[prec][k], "%s: max rel err %.3e" % (k, err)


SPECIES_FORM_CASES = [("d3_mrt_two_species_specular", P.PREC_F32, 6), ("d3_mrt_two_species_specular", P.PREC_F32_F16, 6),
                      ("d2_species_specular", P.PREC_F32, 10)]


@pytest.mark.parametrize("name,prec,steps", SPECIES_FORM_CASES, ids=["d3_mrt_f32", "d3_mrt_f16", "d2_srt_f32"])
def test_emulated_species_specular_reduced_precision(emu_exe, tmp_path, name, prec, steps):
    # species in the FP32/FP16 forms (no rest state: their empty slots store
    # zero) next to the flow's deviation storage, with each component's rest
    # density at its mean; species and flow populations within the forms' bounds
    p, walls, rho, conc = dict((c[0], c[1]) for c in cases.SPECIES_SPECULAR)[name]()
    o = Oracle(p)
    o.set_walls(walls)
    o.set_state(rho)
    o.set_species(conc)
    o.init()
    o.step(steps)
    ref = {"fi": o.get(P.FIELD_FI), "sfi": o.get(P.FIELD_SPECIES_FI), "srho": o.get(P.FIELD_SPECIES_RHO)}
    o.close()
    assert np.abs(ref["sfi"].reshape(p.nsites, -1)[np.asarray(walls) > 0]).sum() > 0.0
    q = P.copy_params(p)
    q.exact = 0
    q.precision = prec
    q.storage_scale = 4096.0 if prec == P.PREC_F32_F16 else 1.0
    for m in range(p.ncomponents):
        q.rho0[m] = float(np.mean(np.asarray(rho).reshape(-1, p.ncomponents)[:, m]))
    got = run_emu(emu_exe, q, walls, rho, steps, False, tmp_path, conc=conc)
    tol = FORM_TOL[prec]["fi"]
    for k, v in ref.items():
        err = float(np.max(np.abs(v - got[k])) / np.max(np.abs(v)))
        assert err <= tol, "%s: max rel err %.3e" % (k, err)


@pytest.mark.parametrize("name,make,steps", cases.SPECIES_SPECULAR_BCS, ids=[c[0] for c in cases.SPECIES_SPECULAR_BCS])
def test_emulated_species_specular_with_exterior_bcs(emu_exe, tmp_path, name, make, steps):
    # the species' exceptions are resolved without the flow's BCPreStream
    # copies (their transport applies no boundary condition); flow and species
    # bit for bit (within 1e-12 where an equation of state calls exp)
    p, walls, rho, conc = make()
    o = Oracle(p)
    o.set_walls(walls)
    o.set_state(rho)
    o.set_species(conc)
    o.init()
    o.step(steps)
    ref = {"fi": o.get(P.FIELD_FI), "sfi": o.get(P.FIELD_SPECIES_FI), "srho": o.get(P.FIELD_SPECIES_RHO),
           "sflux": o.get(P.FIELD_SPECIES_FLUX)}
    o.close()
    q = P.copy_params(p)
    q.exact = 1
    got = run_emu(emu_exe, q, walls, rho, steps, False, tmp_path, conc=conc)
    tol = 1e-12 if p.use_nonideal_eos else 0.0
    for k, v in ref.items():
        assert np.all(np.isfinite(v)), k
        bad = int(np.sum(np.abs(v - got[k]) > tol * np.max(np.abs(v))))
        assert bad == 0, "%s: %d values differ" % (k, bad)


@pytest.mark.parametrize("seed", range(32))
def test_emulated_specular_random_configurations(emu_exe, tmp_path, seed):
    # seeded random lattices with specular walls among ordinary ones: periodic
    # axes, components, relaxation, exterior BCs, species and restarts with
    # wall content drawn at random; every cell bit for bit
    p, walls, rho, conc, steps, restart = cases.random_specular(seed)
    init, from_fi = rho, False
    if restart:
        o0 = Oracle(p)
        o0.set_walls(walls)
        o0.set_state(rho)
        o0.init()
        o0.step(restart)
        init, from_fi = o0.get(P.FIELD_FI), True
        o0.close()
    o = Oracle(p)
    o.set_walls(walls)
    if from_fi:
        o.set_fi(init)
    else:
        o.set_state(rho)
    if conc is not None:
        o.set_species(conc)
    o.init()
    o.step(steps)
    fields = {"fi": P.FIELD_FI, "rho": P.FIELD_RHO, "flux": P.FIELD_FLUX}
    if conc is not None:
        fields.update({"sfi": P.FIELD_SPECIES_FI, "srho": P.FIELD_SPECIES_RHO})
    ref = {k: o.get(f) for k, f in fields.items()}
    o.close()
    q = P.copy_params(p)
    q.exact = 1
    got = run_emu(emu_exe, q, walls, init, steps, from_fi, tmp_path, conc=conc)
    for k, v in ref.items():
        assert np.all(np.isfinite(v)), k
        bad = int(np.sum(v != got[k]))
        assert bad == 0, "%s: %d values differ" % (k, bad)
