"""The host driver's initial output, time loop and outputs follow LBMInit2, LBMRun2 and LBMOutput
(src/lbm/lbm.F90:183-442) and FlowOutputDiagnostics (src/lbm/lbm_flow.F90:576-601):
-kwrite cadence, -waypointN, fi at the last step (-output_flow_last_fi),
-output_last, the steady-state exit, the per-field output flags and the
physical scales of the written fields.  The device handle is replaced by a
fake that records the steps it is asked for, so this runs on the CPU.
"""
import os

import numpy as np
import pytest

from taxila import options as O
from taxila import params as P
from taxila import petsc_io
from taxila.lbm import LBM, main

BASE = """
-NX 4
-NY 3
-discretization d2q9
-ncomponents 1
-component1_name water
-tau_water 1.0
-bc_periodic_x
-bc_periodic_y
-walls_type 2
"""


class FakeHandle:
    """Counts steps; downloads return the step count plus field / 100 everywhere."""

    def __init__(self, p, norms=()):
        self.p = p
        self.t = 0
        self.calls = []
        self.norms = list(norms)

    def init(self):
        self.inited = True

    def upload_walls(self, walls):
        self.walls = np.array(walls)

    def upload_state(self, rho, u=None):
        self.rho = np.array(rho)

    def upload_fi(self, fi):
        self.fi = np.array(fi)

    def upload_bc_values(self, face, vals):
        self.bc = getattr(self, "bc", {})
        self.bc[face] = np.array(vals)

    def close(self):
        self.closed = True

    def step(self, n):
        assert n > 0
        self.calls.append(n)
        self.t += n

    def step_species(self, n):
        assert n > 0
        self.calls.append(("species", n))
        self.t += n

    def download(self, field):
        p = self.p
        dof = {P.FIELD_FI: p.ncomponents * p.Q, P.FIELD_RHO: p.ncomponents, P.FIELD_VELT: p.ndims,
               P.FIELD_PRS: 1, P.FIELD_RHOT: 1, P.FIELD_SPECIES_FI: p.nspecies * p.Q,
               P.FIELD_SPECIES_RHO: p.nspecies}[field]
        return np.full(p.nsites * dof, self.t + field / 100.0)

    def delta_norm(self, field):
        return self.norms.pop(0)


def driver(tmp_path, extra, norms=()):
    lbm = LBM.from_deck(BASE + extra + "\n-output_file_prefix %s/o_\n" % tmp_path)
    lbm.handle = FakeHandle(lbm.params, norms)
    return lbm


def written(tmp_path, name, counter):
    path = petsc_io.output_name(str(tmp_path) + "/o_", name, counter)
    return petsc_io.read_vec(path) if os.path.exists(path) else None


def steps_of(tmp_path, name="rho"):
    out, c = [], 0
    while written(tmp_path, name, c) is not None:
        out.append(int(written(tmp_path, name, c)[0]))
        c += 1
    return out


def test_kwrite_and_waypoints(tmp_path):
    lbm = driver(tmp_path, "-npasses 10\n-kwrite 5\n-waypoint1 3\n-waypoint2 7")
    assert lbm.run_opts.waypoints == [3, 7]
    assert lbm.run() == 10
    assert lbm.handle.calls == [3, 2, 2, 3]
    assert steps_of(tmp_path) == [3, 5, 7, 10]
    assert steps_of(tmp_path, "u") == [3, 5, 7, 10] and steps_of(tmp_path, "prs") == [3, 5, 7, 10]
    assert written(tmp_path, "fi", 0) is None and written(tmp_path, "rhot", 0) is None


def test_waypoint_on_a_kwrite_step_outputs_once_and_numbering_stops_at_a_gap(tmp_path):
    lbm = driver(tmp_path, "-npasses 10\n-kwrite 5\n-waypoint1 5\n-waypoint3 8")
    assert lbm.run_opts.waypoints == [5]
    lbm.run()
    assert steps_of(tmp_path) == [5, 10]


def test_waypoints_without_kwrite(tmp_path):
    lbm = driver(tmp_path, "-npasses 9\n-waypoint1 2\n-waypoint2 6")
    lbm.run()
    assert lbm.handle.calls == [2, 4, 3]
    assert steps_of(tmp_path) == [2, 6]


def test_last_fi_and_output_last(tmp_path):
    lbm = driver(tmp_path, "-npasses 6\n-kwrite 3\n-output_flow_last_fi\n-output_last")
    lbm.run()
    # outputs at steps 3 and 6, then the one of -output_last (state still at step 6)
    assert steps_of(tmp_path) == [3, 6, 6]
    assert written(tmp_path, "fi", 0) is None
    assert written(tmp_path, "fi", 1) is not None and written(tmp_path, "fi", 2) is not None
    assert written(tmp_path, "fi", 1).size == lbm.params.nsites * lbm.params.Q


def test_steady_state_exit(tmp_path):
    # the norm is below the tolerance from the start; the loop exits once step > istep + 2
    lbm = driver(tmp_path, "-npasses 100\n-kwrite 50\n-run_to_steadystate\n-steadystate_tolerance 1e-3\n-output_last",
                 norms=[1e-4] * 10)
    assert lbm.run() == 3
    assert lbm.handle.calls == [1, 1, 1]
    assert steps_of(tmp_path) == [3]


def test_field_flags(tmp_path):
    lbm = driver(tmp_path, "-npasses 2\n-kwrite 2\n-output_rho 0\n-output_rhot\n-output_pressure 0")
    lbm.run()
    assert written(tmp_path, "rho", 0) is None and written(tmp_path, "prs", 0) is None
    assert written(tmp_path, "rhot", 0) is not None and written(tmp_path, "u", 0) is not None


def test_physical_scales_of_the_outputs(tmp_path):
    # spacing 2 on both axes; mass scale mm * density * L^3, velocity scale
    # L / time scale with time scale L^2 (tau - 1/2) / (3 viscosity)
    lbm = driver(tmp_path, "-npasses 2\n-kwrite 2\n-x_end 8\n-y_end 6\n-mm_water 1.5\n-density_water 2.0\n"
                           "-viscosity_water 0.5")
    ro = lbm.run_opts
    assert ro.length_scale == 2.0
    assert ro.mass_scale == pytest.approx(1.5 * 2.0 * 8.0)
    assert ro.velocity_scale == pytest.approx(2.0 / (4.0 * 0.5 / 1.5))
    lbm.run()
    assert np.allclose(written(tmp_path, "rho", 0), (2 + P.FIELD_RHO / 100.0) * 1.5 * 2.0)
    assert np.allclose(written(tmp_path, "u", 0), (2 + P.FIELD_VELT / 100.0) * 1.5)
    assert np.allclose(written(tmp_path, "prs", 0), 2 + P.FIELD_PRS / 100.0)


def test_unequal_spacing_is_an_error():
    with pytest.raises(O.DeckError):
        LBM.from_deck(BASE + "-x_end 8\n")


def test_init_output_and_counter(tmp_path):
    # LBMInit2 writes the walls and the initial fields to file 000 and
    # advances the counter: the first output of the run is file 001
    lbm = driver(tmp_path, "-npasses 4\n-kwrite 4")
    lbm.walls = np.zeros(lbm.params.nsites)
    lbm.init()
    assert written(tmp_path, "walls", 0) is not None
    lbm.run()
    assert steps_of(tmp_path) == [0, 4]


def test_suppressed_initial_output_still_advances_the_counter(tmp_path):
    lbm = driver(tmp_path, "-npasses 4\n-kwrite 4\n-supress_ic_output")
    lbm.walls = np.zeros(lbm.params.nsites)
    lbm.init()
    lbm.run()
    assert written(tmp_path, "walls", 0) is None and written(tmp_path, "rho", 0) is None
    assert int(written(tmp_path, "rho", 1)[0]) == 4


def test_main_with_plugins(tmp_path):
    deck = BASE + "-npasses 4\n-kwrite 2\n-output_file_prefix %s/o_\n" % tmp_path
    seen = {}

    def walls(p, run):
        return np.zeros(p.nsites)

    def state(p, run, w):
        seen["rho"] = np.full(p.nsites, 1.25)
        return seen["rho"]

    def bcs(p, run):
        return {1: np.ones(3)}

    fake = FakeHandle(LBM.from_deck(deck).params)
    main(deck, initialize_state=state, initialize_walls=walls, initialize_bcs=bcs, handle=fake)
    assert fake.inited and fake.closed
    assert np.array_equal(fake.rho, seen["rho"]) and np.array_equal(fake.walls, np.zeros(12))
    assert 1 in fake.bc
    assert fake.calls == [2, 2]
    assert steps_of(tmp_path) == [0, 2, 4]


def test_main_restart_reads_the_counter_file(tmp_path):
    # -restart at istep 4 with -kwrite 2 reads fi002 and runs steps 5..6
    deck = BASE + "-npasses 6\n-kwrite 2\n-restart\n-istep 4\n-output_file_prefix %s/o_\n" % tmp_path
    p = LBM.from_deck(deck).params
    fi = np.arange(p.nsites * p.Q, dtype=np.float64)
    petsc_io.write_vec(petsc_io.output_name(str(tmp_path) + "/o_", "fi", 2), fi)
    fake = FakeHandle(p)
    main(deck, initialize_walls=lambda p, run: np.zeros(p.nsites), handle=fake)
    assert np.array_equal(fake.fi, fi)
    assert fake.calls == [2]
    # the initial output rewrites file 002; step 6 goes to file 003 (the fake counts the 2 steps it ran)
    assert int(written(tmp_path, "rho", 3)[0]) == 2


def test_main_restart_needs_a_counter(tmp_path):
    deck = BASE + "-npasses 6\n-restart\n-istep 4\n-output_file_prefix %s/o_\n" % tmp_path
    fake = FakeHandle(LBM.from_deck(deck).params)
    with pytest.raises(O.DeckError):
        main(deck, initialize_walls=lambda p, run: np.zeros(p.nsites), handle=fake)
    assert fake.closed


def test_main_needs_an_initial_state(tmp_path):
    deck = BASE + "-npasses 2\n-output_file_prefix %s/o_\n" % tmp_path
    fake = FakeHandle(LBM.from_deck(deck).params)
    with pytest.raises(O.DeckError):
        main(deck, initialize_walls=lambda p, run: np.zeros(p.nsites), handle=fake)


def test_steady_flow_after_rampup(tmp_path):
    # the flow steps while lcv_step < rampup (steps 1..3), then only the
    # species; flow fields are written only for outputs before the ramp-up ends
    lbm = driver(tmp_path, "-npasses 10\n-kwrite 2\n-transport_discretization d2q9\n-nspecies 1\n"
                           "-steadystate_flow\n-steadystate_rampup_steps 4")
    ro = lbm.run_opts
    assert ro.steadystate_flow and ro.steadystate_rampup_steps == 4
    lbm.run()
    assert lbm.handle.calls == [2, 1, ("species", 1), ("species", 2), ("species", 2), ("species", 2)]
    assert steps_of(tmp_path, "rho") == [2]
    assert steps_of(tmp_path, "psi") == [2, 4, 6, 8, 10]


def test_steady_flow_file_means_no_rampup(tmp_path):
    lbm = driver(tmp_path, "-npasses 4\n-transport_discretization d2q9\n-nspecies 1\n-steadystate_flow\n"
                           "-steadystate_flow_file flow.dat\n-steadystate_rampup_steps 3")
    assert lbm.run_opts.steadystate_rampup_steps == 0
    lbm.run()
    assert lbm.handle.calls == [("species", 4)]


class OracleHandle:
    """The CPU oracle behind the device handle's method names (test only)."""

    def __init__(self, p):
        from oracle import Oracle
        self.o = Oracle(p)

    def upload_walls(self, walls):
        self.o.set_walls(walls)

    def upload_state(self, rho, u=None):
        self.o.set_state(rho, u)

    def upload_fi(self, fi):
        self.o.set_fi(fi)

    def upload_bc_values(self, face, vals):
        self.o.set_bc_values(face, vals)

    def init(self):
        self.o.init()

    def step(self, n):
        self.o.step(n)

    def download(self, field):
        return self.o.get(field)

    def delta_norm(self, field):
        return self.o.delta_norm(field)

    def close(self):
        self.o.close()


def test_reference_bubble_2d_deck_through_main_on_the_oracle(tmp_path, monkeypatch):
    # the reference's own test: its deck and initial state through main(),
    # which writes test_solution/fi001.dat after 100 steps; its payload is the
    # reference golden's bit for bit
    import json

    import cases
    import test_options
    from golden.make_golden import digest
    from taxila import problems
    monkeypatch.chdir(tmp_path)
    p, run = O.params_from_options(O.parse_deck_text(test_options.DECK_2D))
    plugin = problems.bubble_plugin()
    walls = np.zeros(p.nsites)
    assert np.array_equal(plugin(p, run, walls), cases.bubble_2d_reference_state(p))
    main(test_options.DECK_2D, initialize_state=plugin, handle=OracleHandle(p))
    assert os.path.exists(os.path.join("test_solution", "fi000.dat"))
    fi = petsc_io.read_vec(os.path.join("test_solution", "fi001.dat"))
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "golden", "bubble_2D_fi001.json")) as f:
        assert digest(fi) == json.load(f)["sha256_be"]


def test_bubble_plugin_on_the_reference_3d_deck():
    # tests/bubble_3D of the reference: a 21^3 box of rho_inner (N+1)/2 +- 10
    import cases
    from taxila import problems
    path = os.path.join(cases.REF, "tests", "bubble_3D", "input_data")
    if not os.path.exists(path):
        pytest.skip("reference test decks not present")
    p, run = O.load_deck(path)
    rho = problems.bubble_plugin(only_pore=False)(p, run, np.zeros(p.nsites)).reshape(p.shape + (p.ncomponents,))
    inner = np.asarray(O._reals(run.extra["rho_inner"])[:p.ncomponents])
    box = np.all(rho == inner, axis=-1)
    assert box.sum() == 21 ** 3
    c = (p.nx + 1) // 2 - 1  # 0-based index of the 1-based centre (N+1)/2
    assert box[c - 10:c + 11, c - 10:c + 11, c - 10:c + 11].all()


def test_duct_walls_plugin():
    from taxila import problems
    p, run = O.params_from_options(O.parse_deck_text(BASE))
    w = problems.duct_walls(p, run).reshape(p.shape)
    assert w[:, [0, -1], :].all() and not w[:, 1:-1, :].any()  # default normal: y
    p3, run3 = O.params_from_options(O.parse_deck_text(
        "-NX 4\n-NY 5\n-NZ 6\n-discretization d3q19\n-duct_normal_direction 3\n"))
    w3 = problems.duct_walls(p3, run3).reshape(p3.shape)
    # as in the reference, the top z wall needs NZ == NY
    assert w3[0].all() and not w3[1:].any()
    p4, run4 = O.params_from_options(O.parse_deck_text(
        "-NX 4\n-NY 5\n-NZ 5\n-discretization d3q19\n-duct_normal_direction 1\n"))
    w4 = problems.duct_walls(p4, run4).reshape(p4.shape)
    assert w4[:, :, [0, -1]].all() and not w4[:, :, 1:-1].any()
    assert not problems.no_walls(p, run).any()


SINGLE = """
-NX 5
-NY 3
-NZ 4
-discretization d3q19
-ncomponents 1
"""


@pytest.mark.parametrize("faces,rho_expect,u_expect", [
    ("-bc_pressure_xm\n-bc_pressure_xm_value 0.4\n-bc_pressure_xp\n-bc_pressure_xp_value 0.3",
     lambda t: 3.0 * (0.4 * (1 - t) + 0.3 * t), 0.0),
    ("-bc_pressure_xm\n-bc_pressure_xm_value 0.4\n-bc_flux_xp\n-bc_flux_xp_value 0.01",
     lambda t: 1.2 + 0 * t, -0.01 / 1.2),
    ("-bc_flux_xm\n-bc_flux_xm_value 0.02\n-bc_flux_xp\n-bc_flux_xp_value 0.01", lambda t: 1.0 + 0 * t, 0.005),
    ("-bc_velocity_xm\n-bc_velocity_xm_values 0.02,0,0\n-bc_velocity_xp\n-bc_velocity_xp_values 0.04,0,0",
     lambda t: 1.0 + 0 * t, 0.03),
])
def test_singlephase_plugin(faces, rho_expect, u_expect):
    # initialize_state_singlephase: the first component along -flow_direction
    # (x here): a linear pressure profile over the 1-based x index, or the
    # closed forms of the mixed face kinds
    from taxila import problems
    p, run = O.params_from_options(O.parse_deck_text(SINGLE + faces))
    rho, u = problems.singlephase_state(p, run, np.zeros(p.nsites))
    x = np.tile(np.arange(p.nx), p.ny * p.nz)
    assert np.allclose(rho, rho_expect(x / (p.nx - 1.0)), rtol=0, atol=1e-15)
    u = u.reshape(p.nsites, 3)
    assert np.allclose(u[:, 0], u_expect, rtol=0, atol=1e-15) and not u[:, 1:].any()


def test_singlephase_plugin_without_faces_is_rest():
    from taxila import problems
    p, run = O.params_from_options(O.parse_deck_text(SINGLE + "-flow_direction 3\n"))
    rho, u = problems.singlephase_state(p, run, np.zeros(p.nsites))
    assert np.all(rho == 1.0) and not u.any()
