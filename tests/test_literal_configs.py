"""Why the benchmark workloads rescale the configurations' Shan-Chen
constants: run literally, the reference algorithm (the FP64 oracle, CPU)
blows up within a few steps.

* Bubbles: the configurations give G = 0.9 with densities 2.0 / 0.06.  The
  reference's force is -c0 g psi grad psi with c0 = 6 on a weight-normalised
  gradient, so g_12 = 0.9 as written diverges; g_12 = G / c0 = 0.15 (what
  the bench uses) stays finite.
* Drainage: adhesion +-0.3 with inlet/outlet densities 2.1 / 1.9 diverges
  with g_12 = 0.15 and with 0.9; the served drainage requests use g_12 =
  0.04, adhesion +-0.03 and faces 1.05 / 0.95, which stay finite.
"""
import numpy as np
import pytest

from oracle import Oracle
from taxila import params as P
from taxila import problems
from taxila import serve


def first_nonfinite(p, walls, rho, nmax, chunk=5):
    """The step (a multiple of chunk) at which some density is no longer finite, or None."""
    o = Oracle(p)
    o.set_walls(walls)
    o.set_state(rho)
    o.init()
    t = 0
    try:
        while t < nmax:
            o.step(chunk)
            t += chunk
            if not np.all(np.isfinite(o.get(P.FIELD_RHO))):
                return t
    finally:
        o.close()
    return None


def bubble_2d(g12):
    """D2Q9 200^2 periodic BGK bubble (tau = 1), disk of radius 30, rho 2.0 / 0.06."""
    p = P.default_params()
    p.discretization = P.D2Q9
    p.nx = p.ny = 200
    p.nz = 1
    p.ncomponents = 2
    for f in range(4):
        p.bc_flags[f] = P.BC_PERIODIC
    p.g[0][1] = p.g[1][0] = g12
    return p, np.zeros(p.nsites), problems.bubble_ball_state(200, 200, 1, 30.0, [2.0, 0.06], [0.06, 2.0])


def bubble_3d(g12, n=32):
    """D3Q19 periodic MRT bubble (s_nu 1/1.0 and 1/0.7, other rates 1), the
    128^3 benchmark case scaled to n^3 (sphere radius 24 n / 128)."""
    p = P.default_params()
    p.discretization = P.D3Q19
    p.nx = p.ny = p.nz = n
    p.ncomponents = 2
    p.relaxation_mode = P.MRT
    for f in range(6):
        p.bc_flags[f] = P.BC_PERIODIC
    p.s_nu[0], p.s_nu[1] = 1.0, 1.0 / 0.7
    p.g[0][1] = p.g[1][0] = g12
    return p, np.zeros(p.nsites), problems.bubble_ball_state(n, n, n, 24.0 * n / 128, [2.0, 0.06], [0.06, 2.0])


def drainage(g12, ads, rho_in, rho_out, n=24, seed=3):
    """A served D3Q19 drainage request (n^3 two-mineral sphere pack, density
    faces along z) with the given coupling, adhesion +-ads and face
    densities; bulk densities 2.0 / 0.06 as in the bubbles when the literal
    values are used."""
    r = serve.drain_request(0, 0.0, [n, n, n], seed, 100)
    p = r.params
    p.nspecies = 0
    p.g[0][1] = p.g[1][0] = g12
    p.gw[0][0], p.gw[0][1] = ads, -ads
    p.gw[1][0], p.gw[1][1] = -ads, ads
    p.bc_data[4][0] = rho_in
    p.bc_data[5][1] = rho_out
    rho = r.rho.reshape(-1, 2).copy()
    pore = np.asarray(r.walls) == 0
    inlet = rho[:, 0] > 0.5
    rho[:, 0] = np.where(pore, np.where(inlet, rho_in, 0.06), 0.0)
    rho[:, 1] = np.where(pore, np.where(inlet, 0.06, 2.0), 0.0)
    return p, r.walls, rho.ravel()


@pytest.mark.parametrize("case", [bubble_2d, bubble_3d])
def test_bubble_literal_g_diverges(case):
    t = first_nonfinite(*case(0.9), 50)
    assert t is not None and t <= 50, "g_12 = 0.9 stayed finite for 50 steps"


def test_bubble_2d_rescaled_g_stays_finite():
    assert first_nonfinite(*bubble_2d(0.15), 200, chunk=50) is None


def test_bubble_3d_rescaled_g_stays_finite():
    assert first_nonfinite(*bubble_3d(0.15), 300, chunk=50) is None


@pytest.mark.parametrize("g12", [0.15, 0.9])
def test_drainage_literal_values_diverge(g12):
    t = first_nonfinite(*drainage(g12, 0.3, 2.1, 1.9), 50)
    assert t is not None and t <= 50, "drainage with adhesion 0.3 and faces 2.1/1.9 stayed finite for 50 steps"


def test_served_drainage_values_stay_finite():
    r = serve.drain_request(0, 0.0, [24, 24, 24], 3, 300)
    p = r.params
    p.nspecies = 0
    assert first_nonfinite(p, r.walls, r.rho, 300, chunk=50) is None


def test_specular_walls_leave_populations_in_wall_cells():
    # Why the device keeps wall cells' populations when specular wall codes
    # 900-902 are present: in the reference's bounceback sweep (k-j-i order
    # over the ghosted box, restated by the oracle) a specular wall moves a
    # population along one axis only, possibly into a wall cell that the sweep
    # has already cleared.  Those populations stay in wall cells, stream into
    # pore cells on the next step and decide the result; with ordinary walls
    # alone, wall cells end every step empty.
    rng = np.random.default_rng(0)
    for codes, expect_left in (([1.0], False), ([1.0, 900.0, 901.0, 902.0], True)):
        p = P.default_params()
        p.discretization = P.D3Q19
        p.nx, p.ny, p.nz = 14, 12, 10
        p.ncomponents = 1
        for f in range(6):
            p.bc_flags[f] = P.BC_PERIODIC
        p.body_forces = 1
        p.gvt[0] = 1e-5
        u = rng.random(p.nsites)
        walls = np.where(u < 0.25, rng.choice(codes, size=p.nsites), 0.0)
        o = Oracle(p)
        o.set_walls(walls)
        o.set_state(np.where(walls == 0, 1.0, 0.0))
        o.init()
        o.step(3)
        fi = o.get(P.FIELD_FI).reshape(p.nsites, p.Q)
        o.close()
        left = np.abs(fi[walls > 0]).sum()
        assert (left > 0.0) == expect_left, (codes, left)
