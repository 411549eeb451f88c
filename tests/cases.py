"""Parameter sets and initial states shared by the oracle and GPU tests."""
import os

import numpy as np

from taxila import params as P
from taxila import problems

REF = os.environ.get("TAXILA_REFERENCE", "/root/reference")  # the reference checkout


def base(disc, shape, ncomp=2, mode=P.SRT, iso=4, periodic=(1, 1, 1)):
    p = P.default_params()
    p.discretization = disc
    p.nz, p.ny, p.nx = shape
    if disc == P.D2Q9:
        p.nz = 1
    p.ncomponents = ncomp
    p.relaxation_mode = mode
    p.isotropy_order = iso
    for a in range(p.ndims):
        if periodic[a]:
            p.bc_flags[2 * a] = p.bc_flags[2 * a + 1] = P.BC_PERIODIC
    return p


def bubble_2d_reference_deck():
    """tests/bubble_2D/input_data of the reference as tx_params."""
    p = base(P.D2Q9, (1, 128, 128))
    p.tau[0] = p.tau[1] = 1.0
    p.g[0][1] = p.g[1][0] = 0.1
    return p


def bubble_2d_reference_state(p):
    return problems.bubble_box_state(p.nx, p.ny, 1, [0.03, 0.97], [0.97, 0.03], 26, np.zeros(p.nsites))


def sc_bubble(disc, shape, mode, iso, g=0.12, r=None, ncomp=2, nu_only=False, base_rate=1.0):
    """Two-component Shan-Chen bubble; MRT rates mixed (s_e, s_q, s_nu differ
    from 1) or, with nu_only, only s_nu of the second component differs from
    the others (base_rate; 1 in the bench's viscosity contrast)."""
    p = base(disc, shape, ncomp=ncomp, mode=mode, iso=iso)
    p.tau[0], p.tau[1] = 1.0, 0.8
    if mode == P.MRT:
        for key in ("s_c", "s_e", "s_e2", "s_q", "s_pi", "s_m"):
            getattr(p, key)[1] = base_rate
        p.s_nu[0], p.s_nu[1] = 1.0, 1.0 / 0.7
        if not nu_only:
            p.s_e[0], p.s_q[1] = 1.2, 1.1
    if ncomp == 2:
        p.g[0][1] = p.g[1][0] = g
    z, y, x = p.shape
    r = r if r is not None else max(2.0, min(x, y) / 5.0)
    rho = problems.bubble_ball_state(x, y, z, r, [2.0, 0.06][:ncomp], [0.06, 2.0][:ncomp])
    return p, np.zeros(p.nsites), rho


def porous_case(disc, shape, mode=P.SRT, iso=4, seed=3, dirichlet=True, body=False, ncomp=2):
    """Seeded sphere pack with two minerals, ghost walls on x/y, density faces on z
    (D2Q9: on y), plus optional body force."""
    periodic = (0, 0, 1) if disc == P.D3Q19 else (0, 1, 1)
    if disc == P.D3Q19 and not dirichlet:
        periodic = (1, 1, 1)
    p = base(disc, shape, ncomp=ncomp, mode=mode, iso=iso, periodic=periodic)
    p.nminerals = 2
    p.tau[0], p.tau[1] = 1.0, 0.9
    if mode == P.MRT:
        p.s_nu[0], p.s_nu[1] = 1.0, 1.0 / 0.9
    if ncomp == 2:
        p.g[0][1] = p.g[1][0] = 0.1
        p.gw[0][0], p.gw[0][1] = 0.3, -0.3
        p.gw[1][0], p.gw[1][1] = -0.3, 0.3
    else:
        p.gw[0][0], p.gw[1][0] = 0.05, -0.05
    z, y, x = p.shape
    solid = problems.sphere_pack((z, y, x), 0.55, 1.2, 2.5, seed, periodic=True)
    walls = problems.mineral_walls(solid, seed)
    rng = np.random.default_rng(seed)
    s = p.ncomponents
    rho = np.empty((p.nsites, s))
    rho[:, 0] = 1.0 + 0.02 * rng.standard_normal(p.nsites)
    if s == 2:
        rho[:, 1] = 0.06 + 0.005 * rng.standard_normal(p.nsites)
    if dirichlet:
        a = 2 if disc == P.D3Q19 else 1
        p.bc_flags[2 * a] = P.BC_DENSITY
        p.bc_flags[2 * a + 1] = P.BC_DENSITY
        p.bc_data[2 * a][0], p.bc_data[2 * a + 1][0] = 1.03, 0.97
        if s == 2:
            p.bc_data[2 * a][1], p.bc_data[2 * a + 1][1] = 0.07, 0.05
    if body:
        p.body_forces = 1
        p.gvt[0], p.gvt[1] = 1e-5, -2e-5
        if disc == P.D3Q19:
            p.gvt[2] = 3e-5
    return p, walls, rho.ravel()


# (name, case factory, steps): the parity matrix of the GPU and host-emulation tests
PARITY = [
    ("d2_srt_iso4", lambda: sc_bubble(P.D2Q9, (1, 40, 48), P.SRT, 4), 30),
    ("d2_mrt_iso8", lambda: sc_bubble(P.D2Q9, (1, 44, 40), P.MRT, 8), 30),
    ("d2_mrt_iso10", lambda: sc_bubble(P.D2Q9, (1, 40, 40), P.MRT, 10), 30),
    ("d3_srt_iso4", lambda: sc_bubble(P.D3Q19, (12, 14, 16), P.SRT, 4), 20),
    ("d3_mrt_iso4", lambda: sc_bubble(P.D3Q19, (16, 12, 14), P.MRT, 4), 20),
    ("d3_mrt_iso8", lambda: sc_bubble(P.D3Q19, (14, 16, 12), P.MRT, 8), 20),
    ("d3_mrt_nu_only", lambda: sc_bubble(P.D3Q19, (12, 14, 12), P.MRT, 4, nu_only=True), 20),
    ("d2_mrt_nu_only_iso8", lambda: sc_bubble(P.D2Q9, (1, 36, 40), P.MRT, 8, nu_only=True), 30),
    ("d3_mrt_nu_only_base_rate", lambda: sc_bubble(P.D3Q19, (12, 12, 14), P.MRT, 4, nu_only=True, base_rate=1.2), 20),
    ("d3_porous_dirichlet_srt", lambda: porous_case(P.D3Q19, (14, 12, 10)), 20),
    ("d3_porous_dirichlet_mrt_body", lambda: porous_case(P.D3Q19, (12, 10, 14), mode=P.MRT, body=True), 20),
    ("d3_porous_periodic_iso8", lambda: porous_case(P.D3Q19, (12, 12, 12), iso=8, dirichlet=False), 15),
    ("d2_porous_dirichlet", lambda: porous_case(P.D2Q9, (1, 30, 26), body=True), 30),
    ("d3_single_component_porous", lambda: porous_case(P.D3Q19, (10, 12, 14), ncomp=1, body=True), 20),
]


def bc_case(disc, shape, faces, ncomp=1, mode=P.SRT, iso=4, periodic=(0, 0, 0), seed=5, body=False,
            porosity=0.8, rho_init=(1.0, 0.05), g12=0.0, eos=None):
    """A channel with exterior BCs: ``faces`` maps face index (0..5) to
    (kind, bc_data values); a sparse seeded sphere pack with two minerals
    (some grains cut by the faces), fluid-solid adhesion, optional body force
    and component coupling.  The initial density is rho_init per component
    with 1% noise."""
    p = base(disc, shape, ncomp=ncomp, mode=mode, iso=iso, periodic=periodic)
    p.nminerals = 2
    p.tau[0], p.tau[1] = 1.0, 0.9
    if mode == P.MRT:
        p.s_nu[0], p.s_nu[1] = 1.0, 1.0 / 0.9
        p.s_e[0], p.s_q[1] = 1.2, 1.1
    if ncomp == 2:
        p.g[0][1] = p.g[1][0] = g12
        p.gw[0][0], p.gw[0][1] = 0.1, -0.1
        p.gw[1][0], p.gw[1][1] = -0.1, 0.1
    else:
        p.gw[0][0], p.gw[1][0] = 0.05, -0.05
    for f, (kind, vals) in faces.items():
        p.bc_flags[f] = kind
        for k, v in enumerate(vals):
            p.bc_data[f][k] = v
    if body:
        p.body_forces = 1
        p.gvt[0], p.gvt[1] = 2e-6, -1e-6
        if disc == P.D3Q19:
            p.gvt[2] = 3e-6
    if eos is not None:
        p.use_nonideal_eos = 1
        for m in range(ncomp):
            p.eos[m] = eos[0]
            for k, v in enumerate(eos[1]):
                p.eos_coef[m][k] = v
    z, y, x = p.shape
    solid = problems.sphere_pack((z, y, x), porosity, 1.0, 2.0, seed, periodic=True)
    walls = problems.mineral_walls(solid, seed)
    rng = np.random.default_rng(seed)
    rho = np.empty((p.nsites, ncomp))
    for m in range(ncomp):
        rho[:, m] = rho_init[m] * (1.0 + 0.01 * rng.standard_normal(p.nsites))
    return p, walls, rho.ravel()


# (name, case factory, steps): exterior boundary conditions.  Face index:
# 0 XM, 1 XP, 2 YM, 3 YP, 4 ZM, 5 ZP.
BCS = [
    # one component: pressure inlet, pressure outlet (its value is the density itself)
    ("d3_pressure_s1", lambda: bc_case(P.D3Q19, (12, 8, 10), {4: (P.BC_PRESSURE, (0.345,)),
                                                                5: (P.BC_PRESSURE_OUTLET, (0.99,))},
                                        periodic=(1, 1, 0), body=True), 20),
    # flux inlet, velocity outlet, a reflecting and a closed side; MRT
    ("d3_flux_velocity_mrt", lambda: bc_case(P.D3Q19, (12, 10, 8), {2: (P.BC_REFLECTING, ()),
                                                                     4: (P.BC_FLUX, (0.002,)),
                                                                     5: (P.BC_VELOCITY, (0.0, 0.0, 0.0021))},
                                              mode=P.MRT, periodic=(1, 0, 0)), 20),
    # reflecting x faces (XM with the reference's z comparison), momentum and flux outlet on y
    ("d3_reflect_momentum", lambda: bc_case(P.D3Q19, (8, 12, 10), {0: (P.BC_REFLECTING, ()),
                                                                    1: (P.BC_REFLECTING, ()),
                                                                    2: (P.BC_MOMENTUM, (0.0, 0.0015, 0.0002)),
                                                                    3: (P.BC_FLUX_OUTLET, (0.0015,))},
                                             periodic=(0, 0, 1), body=True), 20),
    # Neumann class before Dirichlet at the shared edge (BCApply's order of first appearance)
    ("d3_neumann_then_dirichlet", lambda: bc_case(P.D3Q19, (8, 10, 10), {0: (P.BC_FLUX, (0.001,)),
                                                                          2: (P.BC_DENSITY, (1.01,)),
                                                                          3: (P.BC_PRESSURE, (0.33,))},
                                                   periodic=(0, 0, 1)), 20),
    # two components: pressure inlet with a mass fraction, pressure outlet refreshed every step
    ("d3_two_phase_pressure", lambda: bc_case(P.D3Q19, (12, 8, 8), {4: (P.BC_PRESSURE_INLET, (0.35, 0.95)),
                                                                     5: (P.BC_PRESSURE_OUTLET, (0.33,))},
                                               ncomp=2, g12=0.1, rho_init=(0.9, 0.05), periodic=(1, 0, 0)), 20),
    # two components: flux inlet, per-component momentum outlet, density and velocity sides; MRT iso 8
    ("d3_two_phase_flux_mrt_iso8", lambda: bc_case(P.D3Q19, (12, 10, 8), {
        2: (P.BC_DENSITY, (0.92, 0.05)), 3: (P.BC_VELOCITY, (0.0, 0.0, 0.0)),
        4: (P.BC_FLUX_INLET, (0.003, 0.9)), 5: (P.BC_MOMENTUM, (0.0, 0.0, 0.0027, 0.0, 0.0, 0.0003))},
        ncomp=2, mode=P.MRT, iso=8, g12=0.1, rho_init=(0.9, 0.05), periodic=(1, 0, 0)), 15),
    # 2D: velocity inlet, pressure outlet, reflecting y faces
    ("d2_velocity_outlet", lambda: bc_case(P.D2Q9, (1, 20, 28), {0: (P.BC_VELOCITY, (0.004, 0.0)),
                                                                  1: (P.BC_PRESSURE_OUTLET, (1.0,)),
                                                                  2: (P.BC_REFLECTING, ()),
                                                                  3: (P.BC_REFLECTING, ())}, body=True), 30),
    # 2D two components: pressure inlet / outlet on y, MRT iso 10
    ("d2_two_phase_pressure_iso10", lambda: bc_case(P.D2Q9, (1, 30, 24), {
        2: (P.BC_PRESSURE_INLET, (0.35, 0.9)), 3: (P.BC_PRESSURE_OUTLET, (0.34,))},
        ncomp=2, mode=P.MRT, iso=10, g12=0.1, rho_init=(0.9, 0.05), periodic=(1, 0, 0)), 30),
    # 2D two components with a Shan-Chen EOS: momentum inlet, flux outlet, flux inlet sides
    ("d2_momentum_flux_eos", lambda: bc_case(P.D2Q9, (1, 24, 26), {
        0: (P.BC_MOMENTUM, (0.002, 0.0, 0.0002, 0.0)), 1: (P.BC_FLUX_OUTLET, (0.0022,)),
        2: (P.BC_FLUX_INLET, (0.0, 0.5))},
        ncomp=2, g12=0.1, rho_init=(0.9, 0.05), eos=(P.EOS_SC, (1.0,))), 30),
]


def permeability_case(shape, seed=11, porosity=0.45, rmin=2.0, rmax=4.0, precision=P.PREC_F64, gz=1e-5):
    """Single-phase D3Q19 BGK (tau = 1) periodic sphere pack driven by a body
    force along z: the batched permeability workload at test size."""
    p = base(P.D3Q19, shape, ncomp=1, mode=P.SRT, iso=4)
    p.tau[0] = 1.0
    p.nminerals = 1
    p.body_forces = 1
    p.gvt[2] = gz
    p.precision = precision
    p.rho0[0] = 1.0
    solid = problems.sphere_pack(p.shape, porosity, rmin, rmax, seed, periodic=True)
    walls = np.where(solid.ravel(), 1.0, 0.0)
    rho = np.ones(p.nsites)
    return p, walls, rho


def permeability(p, u_sum_z, nsites):
    """k = nu <u_z> phi / g, with <u_z> phi = sum of u_z over pore sites / all sites."""
    nu = (p.tau[0] - 0.5) / 3.0
    return nu * (u_sum_z / nsites) / p.gvt[2]


def with_species(p, walls, mode=P.SRT, tau=0.8, ns=1, front=4):
    """Adds ns passive species to p (in place): concentration 1 in the first
    ``front`` slices along the last axis of the lattice (z in 3D, y in 2D) on
    pore sites, 0 elsewhere; species s has tau + 0.1 s (MRT: s_nu = 1/tau,
    s_e = 1.1, other rates 1).  Returns the concentration array [N*ns]."""
    p.nspecies = ns
    p.species_relaxation_mode = mode
    axis = 0 if p.ndims == 3 else 1
    first = np.indices(p.shape)[axis].ravel() < front
    pore = np.asarray(walls).ravel() == 0
    conc = np.zeros((p.nsites, ns))
    for s in range(ns):
        p.species_tau[s] = tau + 0.1 * s
        for k in range(7):
            p.species_rates[s][k] = 1.0
        if mode == P.MRT:
            p.species_rates[s][4] = 1.0 / (tau + 0.1 * s)
            p.species_rates[s][1] = 1.1
        conc[:, s] = np.where(first & pore, 1.0 - 0.2 * s, 0.0)
    return conc.ravel()


# (name, case factory returning (p, walls, rho, conc), steps): species parity matrix
def _sp(make, mode, ns=1):
    def f():
        p, w, r = make()
        return p, w, r, with_species(p, w, mode=mode, ns=ns)
    return f


SPECIES = [
    ("d3_srt_species", _sp(lambda: porous_case(P.D3Q19, (12, 10, 14), body=True), P.SRT), 20),
    ("d3_mrt_two_species", _sp(lambda: sc_bubble(P.D3Q19, (12, 12, 10), P.MRT, 4), P.MRT, ns=2), 20),
    ("d2_species_streaming", _sp(lambda: porous_case(P.D2Q9, (1, 30, 26), body=True), P.SRT), 30),
]


def eos_drop(disc, shape, eos, coef, g11, mode=P.SRT, r=None, rho_in=2.0, rho_out=0.2):
    """Single-component Shan-Chen with a non-ideal EOS psi(rho): a drop of
    rho_in in rho_out, self coupling g11, periodic."""
    p = base(disc, shape, ncomp=1, mode=mode, iso=4)
    p.tau[0] = 1.0
    p.g[0][0] = g11
    p.use_nonideal_eos = 1
    p.eos[0] = eos
    for k, v in enumerate(coef):
        p.eos_coef[0][k] = v
    z, y, x = p.shape
    r = r if r is not None else max(2.0, min(x, y) / 5.0)
    rho = problems.bubble_ball_state(x, y, z, r, [rho_in], [rho_out])
    return p, np.zeros(p.nsites), rho


def _pr_coef():
    a, b = 2.0 / 49.0, 2.0 / 21.0
    f = lambda v: float(np.float32(v))  # single-precision literals of lbm_eos.F90
    tc = a / b * f(0.0778) / f(0.45724)
    return (a, b, f(0.9) * tc, f(0.344))


# (name, case factory, steps): EOS parity cases
EOS = [
    ("d2_eos_sc", lambda: eos_drop(P.D2Q9, (1, 36, 40), P.EOS_SC, (1.0,), -0.28), 40),
    ("d2_eos_thermo", lambda: eos_drop(P.D2Q9, (1, 32, 32), P.EOS_THERMO, (1.0, 1.0), -0.5), 40),
    ("d3_eos_pr", lambda: eos_drop(P.D3Q19, (14, 12, 16), P.EOS_PR, _pr_coef(), -1.0 / 6.0,
                                   rho_in=6.5, rho_out=0.4), 20),
    ("d3_eos_sc_mrt", lambda: eos_drop(P.D3Q19, (12, 14, 12), P.EOS_SC, (1.0,), -0.28, mode=P.MRT), 20),
]


def specular_case(disc, shape, periodic, ncomp, codes, frac, seed):
    """Seeded random walls mixing ordinary and specular (no-stick) codes:
    900/901/902 reflect normal to x/y/z (902 is an ordinary wall in 2D); one
    or two components with coupling, body force, slightly uneven densities."""
    p = base(disc, shape, ncomp=ncomp, mode=P.SRT, periodic=periodic)
    rng = np.random.default_rng(seed)
    p.nminerals = 1
    if ncomp == 2:
        p.g[0][1] = p.g[1][0] = 0.1
        p.tau[1] = 0.8
    p.body_forces = 1
    p.gvt[0], p.gvt[1] = 1e-4, -2e-4
    walls = np.where(rng.random(p.nsites) < frac, rng.choice(codes, size=p.nsites), 0.0)
    rho = np.repeat(np.where(walls == 0, 1.0, 0.0), ncomp) * (1.0 + 0.1 * rng.random(p.nsites * ncomp))
    return p, walls, rho


def specular_porous(disc, shape, iso, seed=7):
    """porous_case (two minerals, density faces, body force, MRT) with half of
    its wall cells turned into specular walls."""
    p, walls, rho = porous_case(disc, shape, mode=P.MRT, iso=iso, body=True)
    rng = np.random.default_rng(seed)
    codes = [900.0, 901.0, 902.0] if disc == P.D3Q19 else [900.0, 901.0]
    pick = (walls > 0) & (rng.random(p.nsites) < 0.5)
    return p, np.where(pick, rng.choice(codes, size=p.nsites), walls), rho


SPEC3 = [1.0, 900.0, 901.0, 902.0]
# (name, case factory, steps): specular walls next to ordinary walls
SPECULAR = [
    ("d3_periodic_1c", lambda: specular_case(P.D3Q19, (10, 12, 14), (1, 1, 1), 1, SPEC3, 0.25, 0), 6),
    ("d3_ghost_xy_2c", lambda: specular_case(P.D3Q19, (10, 12, 14), (0, 0, 1), 2, SPEC3, 0.25, 1), 6),
    ("d3_ghost_xz_1c", lambda: specular_case(P.D3Q19, (9, 11, 13), (0, 1, 0), 1, SPEC3 + [999.0], 0.3, 2), 6),
    ("d2_periodic_2c", lambda: specular_case(P.D2Q9, (1, 20, 24), (1, 1, 1), 2, SPEC3, 0.25, 3), 6),
    ("d2_ghost_x_1c", lambda: specular_case(P.D2Q9, (1, 20, 24), (0, 1, 1), 1, SPEC3[:3], 0.3, 4), 6),
    ("d3_porous_mrt_iso8_dirichlet", lambda: specular_porous(P.D3Q19, (12, 10, 11), 8), 30),
    ("d2_porous_mrt_iso10_dirichlet", lambda: specular_porous(P.D2Q9, (1, 22, 18), 10), 8),
]


def with_specular(make, seed=5):
    """A case factory whose wall cells turn half into specular walls."""
    def made():
        p, walls, rho = make()
        rng = np.random.default_rng(seed)
        codes = [900.0, 901.0, 902.0] if p.ndims == 3 else [900.0, 901.0]
        pick = (walls > 0) & (rng.random(p.nsites) < 0.5)
        return p, np.where(pick, rng.choice(codes, size=p.nsites), walls), rho
    return made


# (name, case factory, steps): every exterior BC kind with specular walls among the grains
SPECULAR_BCS = [(name, with_specular(make), steps) for name, make, steps in BCS]


def _sp_specular(make, mode, ns=1, seed=6):
    """_sp with half of the wall cells specular (the species stream and bounce
    back through the same sweep; in 2D their wall cells are also collided)."""
    def f():
        p, w, r = with_specular(make, seed)()
        return p, w, r, with_species(p, w, mode=mode, ns=ns)
    return f


SPECIES_SPECULAR = [
    ("d3_srt_species_specular", _sp_specular(lambda: porous_case(P.D3Q19, (12, 10, 14), body=True), P.SRT), 20),
    ("d3_mrt_two_species_specular", _sp_specular(lambda: porous_case(P.D3Q19, (10, 12, 12), mode=P.MRT), P.MRT, ns=2), 15),
    # 2D: the reference collides wall cells, and the species near the walls move on within a few steps
    ("d2_species_specular", _sp_specular(lambda: porous_case(P.D2Q9, (1, 30, 26), body=True), P.SRT), 3),
    ("d2_mrt_species_specular", _sp_specular(lambda: porous_case(P.D2Q9, (1, 28, 30), mode=P.MRT, iso=8), P.MRT, seed=9), 12),
]

# species with specular walls next to exterior BCs: the flow's BCPreStream
# copies fill its ghost layer, the species' transport applies no boundary
# condition, so their exceptions differ there
_SPB = dict((c[0], c) for c in BCS)
SPECIES_SPECULAR_BCS = [(name + ("_mrt" if mode == P.MRT else "_srt") + "_species", _sp_specular(_SPB[name][1], mode), _SPB[name][2])
                        for name, mode in (("d3_reflect_momentum", P.SRT), ("d3_reflect_momentum", P.MRT),
                                           ("d3_flux_velocity_mrt", P.MRT), ("d2_momentum_flux_eos", P.MRT))]


def random_specular(seed):
    """A seeded random configuration with specular walls: D2Q9 or D3Q19, random
    periodic axes, wall fraction and codes, one or two components, SRT or MRT,
    optional exterior BCs (one component), optional species (SRT or MRT, one or
    two) and a random step count.  Returns (p, walls, rho, conc or None, steps,
    restart_steps): restart_steps > 0 asks for a restart from the populations
    after that many steps."""
    rng = np.random.default_rng(1000 + seed)
    D = 3 if rng.random() < 0.5 else 2
    disc = P.D3Q19 if D == 3 else P.D2Q9
    shape = tuple(int(v) for v in rng.integers(5, 12, size=3)) if D == 3 else (1, int(rng.integers(6, 22)), int(rng.integers(6, 22)))
    per = tuple(int(v) for v in rng.integers(0, 2, size=3))
    ncomp = int(rng.integers(1, 3))
    codes = [1.0, 900.0, 901.0, 902.0] if D == 3 else [1.0, 2.0, 900.0, 901.0]
    p, walls, rho = specular_case(disc, shape, per, ncomp, codes, float(rng.uniform(0.1, 0.45)), int(rng.integers(0, 10**6)))
    p.nminerals = 2
    if D == 3 and rng.random() < 0.4:
        p.relaxation_mode = P.MRT
    elif D == 2 and ncomp == 2 and rng.random() < 0.4:
        p.relaxation_mode, p.isotropy_order = P.MRT, 8
    if ncomp == 1 and rng.random() < 0.6:
        for a in range(D):
            if per[a]:
                continue
            for f in (2 * a, 2 * a + 1):
                r = rng.random()
                if r < 0.25:
                    p.bc_flags[f], p.bc_data[f][0] = P.BC_DENSITY, 1.0 + 0.02 * rng.random()
                elif r < 0.45:
                    p.bc_flags[f], p.bc_data[f][0] = P.BC_FLUX, 0.001 * (1 if f % 2 == 0 else -1)
                elif r < 0.6 and not (D == 2 and f == 0):
                    p.bc_flags[f] = P.BC_REFLECTING
    sp = int(rng.integers(0, 3))
    conc = None
    if sp:
        conc = with_species(p, walls, mode=P.SRT if sp == 1 else P.MRT, ns=int(rng.integers(1, 3)),
                            front=int(rng.integers(1, 5)))
    steps = int(rng.integers(1, 14))
    restart = int(rng.integers(1, 5)) if rng.random() < 0.5 else 0
    return p, walls, rho, conc, steps, restart
