"""Deck parsing mirrors the reference's options (lbm_options.F90, lbm_flow.F90)."""
import pytest

from taxila import options as O
from taxila import params as P

DECK_2D = """
## Bubble problem, in 2D
-NX 128
-NY 128
-flow_relaxation_mode 0 # SRT
-discretization d2q9
-ncomponents 2
-component1_name outer
-mm_outer 1.0
-tau_outer 1.0
-component2_name inner
-mm_inner 1.0
-tau_inner 1.0
-g_11 0.0
-g_22 0.0
-g_12 0.1
-g_21 0.1
-rho_outer 0.97,0.03
-rho_inner 0.03,0.97
-bc_periodic_x
-bc_periodic_y
-npasses 100
-kwrite 100
-walls_type 2
-output_file_prefix test_solution/
-output_flow_fi
"""


def test_bubble_deck():
    p, run = O.params_from_options(O.parse_deck_text(DECK_2D))
    assert p.discretization == P.D2Q9 and (p.nx, p.ny, p.nz) == (128, 128, 1)
    assert p.ncomponents == 2 and p.relaxation_mode == P.SRT and p.isotropy_order == 4
    assert p.g[0][1] == 0.1 and p.g[1][0] == 0.1 and p.g[0][0] == 0.0
    assert list(p.bc_flags)[:4] == [P.BC_PERIODIC] * 4
    assert run.nsteps == 100 and run.kwrite == 100 and run.walls_type == 2
    assert run.component_names == ["outer", "inner"] and run.output_flow_fi
    assert O._reals(run.extra["rho_inner"]) == [0.03, 0.97]


def test_mrt_and_derivative_order():
    deck = DECK_2D.replace("-flow_relaxation_mode 0 # SRT", "-flow_relaxation_mode 1\n-derivative_order 10\n-s_e_outer 0.1\n-s_nu_inner 1.5")
    p, _ = O.params_from_options(O.parse_deck_text(deck))
    assert p.relaxation_mode == P.MRT and p.isotropy_order == 10
    assert p.s_e[0] == 0.1 and p.s_nu[1] == 1.5 and p.tau[0] == 1.0


def test_density_faces_and_minerals():
    deck = """-NX 8
-NY 8
-NZ 16
-discretization d3q19
-ncomponents 2
-nminerals 2
-bc_density_zm
-bc_density_zm_component1 2.1
-bc_density_zm_component2 0.06
-bc_density_zp
-bc_density_zp_component1 1.9
-bc_density_zp_component2 0.06
-gw_mineral1_component1 0.3
-gw_mineral2_component2 -0.3
-gvt 0,0,1e-6
"""
    p, _ = O.params_from_options(O.parse_deck_text(deck))
    assert p.bc_flags[4] == P.BC_DENSITY and p.bc_flags[5] == P.BC_DENSITY and p.bc_flags[0] == P.BC_NULL
    assert p.bc_data[4][0] == 2.1 and p.bc_data[5][1] == 0.06
    assert p.gw[0][0] == 0.3 and p.gw[1][1] == -0.3 and p.gw[0][1] == 0.0
    assert p.body_forces == 1 and p.gvt[2] == 1e-6


def test_conflicting_bcs_rejected():
    deck = "-NX 4\n-NY 4\n-NZ 4\n-bc_periodic_z\n-bc_density_zm\n"
    with pytest.raises(O.DeckError):
        O.params_from_options(O.parse_deck_text(deck))


def test_exterior_bcs_parsed():
    deck = """
-NX 4
-NY 4
-NZ 6
-bc_periodic_x
-bc_velocity_ym
-bc_velocity_ym_values 0.0,0.01,0.0
-bc_reflecting_yp
-bc_pressure_zm
-bc_pressure_zm_value 0.34
-bc_flux_outlet_zp
-bc_flux_outlet_zp_value 0.002
"""
    p, _ = O.params_from_options(O.parse_deck_text(deck))
    assert list(p.bc_flags) == [P.BC_PERIODIC, P.BC_PERIODIC, P.BC_VELOCITY, P.BC_REFLECTING,
                                P.BC_PRESSURE, P.BC_FLUX_OUTLET]
    assert list(p.bc_data[2][:3]) == [0.0, 0.01, 0.0]
    assert p.bc_data[4][0] == 0.34 and p.bc_data[4][1] == -1.0
    assert p.bc_data[5][0] == 0.002
    # velocity with the wrong number of components, two kinds on one face
    with pytest.raises(O.DeckError):
        O.params_from_options(O.parse_deck_text(deck.replace("0.0,0.01,0.0", "0.0,0.01")))
    with pytest.raises(O.DeckError):
        O.params_from_options(O.parse_deck_text(deck + "-bc_density_zm\n"))


def test_two_component_exterior_bcs():
    deck = """
-NX 4
-NY 4
-NZ 6
-ncomponents 2
-bc_pressure_inlet_zm
-bc_pressure_zm_value 0.35
-bc_rho1_fraction_zm_value 0.9
-bc_momentum_zp
-bc_momentum_zp_component1 0.0,0.0,-0.01
-bc_momentum_zp_component2 0.0,0.0,-0.002
-bc_flux_inlet_xm
-bc_flux_inlet_xm_value 0.01
"""
    p, _ = O.params_from_options(O.parse_deck_text(deck))
    assert p.bc_flags[4] == P.BC_PRESSURE_INLET and list(p.bc_data[4][:2]) == [0.35, 0.9]
    assert p.bc_flags[5] == P.BC_MOMENTUM and list(p.bc_data[5][:6]) == [0.0, 0.0, -0.01, 0.0, 0.0, -0.002]
    assert p.bc_flags[0] == P.BC_FLUX_INLET and p.bc_data[0][0] == 0.01 and p.bc_data[0][1] == -1.0
    # -bc_pressure / -bc_flux are read for one component only
    p2, _ = O.params_from_options(O.parse_deck_text(deck + "-bc_pressure_ym\n"))
    assert p2.bc_flags[2] == P.BC_NULL


def test_viscosity_consistency():
    deck = "-NX 4\n-NY 4\n-NZ 4\n-ncomponents 2\n-tau_component1 1.0\n-viscosity_component1 0.1\n-viscosity_component2 0.05\n"
    p, _ = O.params_from_options(O.parse_deck_text(deck))
    # time scale = (tau1 - 0.5)/(3 nu1); tau2 = 3 ts nu2 + 0.5
    ts = (1.0 - 0.5) / (0.1 * 3.0)
    assert abs(p.tau[1] - (3 * ts * 0.05 + 0.5)) < 1e-15


def test_transport_options():
    from taxila import options
    deck = """
-flow_discretization d3q19
-NX 8
-NY 8
-NZ 8
-transport_discretization d3q19
-nspecies 2
-specie2_name salt
-tau_specie1 0.8
-tau_salt 1.2
"""
    p, run = options.params_from_options(options.parse_deck_text(deck))
    assert p.nspecies == 2 and p.species_relaxation_mode == 0
    assert p.species_tau[0] == 0.8 and p.species_tau[1] == 1.2
    assert run.species_names == ["specie1", "salt"]
    bad = deck.replace("-transport_discretization d3q19", "-transport_discretization d2q9")
    import pytest
    with pytest.raises(options.DeckError):
        options.params_from_options(options.parse_deck_text(bad))



def test_eos_options():
    from taxila import options
    from taxila import params as P
    deck = """
-flow_discretization d2q9
-NX 8
-NY 8
-ncomponents 2
-flow_use_nonideal_eos true
-eos_component1 sc
-eos_sc_rho0_component1 2.0
-eos_component2 pr
-eos_pr_reduced_T_component2 0.8
"""
    p, _ = options.params_from_options(options.parse_deck_text(deck))
    assert p.use_nonideal_eos == 1
    assert p.eos[0] == P.EOS_SC and p.eos_coef[0][0] == 2.0
    a, b = 2.0 / 49.0, 2.0 / 21.0
    assert p.eos[1] == P.EOS_PR and abs(p.eos_coef[1][2] - 0.8 * a / b * 0.0778 / 0.45724) < 1e-8
    import pytest
    with pytest.raises(options.DeckError):
        options.params_from_options(options.parse_deck_text(deck.replace("-eos_component1 sc", "-eos_component1 vdw")))


def test_spec_serving_mix_sizes():
    # the specification's serving mix: request kinds and lattice sizes in range
    from taxila import serve
    reqs = serve.make_spec_mix(40, seed=1)
    perm = [r for r in reqs if r.kind == "perm"]
    drain = [r for r in reqs if r.kind == "drain"]
    assert 0.5 < len(perm) / len(reqs) < 0.9 and drain
    for r in perm:
        assert all(32 <= v <= 160 for v in (r.params.nx, r.params.ny, r.params.nz))
        assert r.tol == 1e-7 and r.params.gvt[2] == 1e-6
    for r in drain:
        if r.params.discretization == P.D2Q9:
            assert all(256 <= v <= 1024 for v in (r.params.nx, r.params.ny))
        else:
            assert all(64 <= v <= 128 for v in (r.params.nx, r.params.ny, r.params.nz))
        assert r.params.nspecies == 1 and r.params.nminerals == 2 and r.tol == 1e-4
    assert all(a.arrival < b.arrival for a, b in zip(reqs, reqs[1:]))
