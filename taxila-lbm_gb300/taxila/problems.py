"""Problem plugins: initial states and wall geometries, natural order.

The reference fills host arrays through link-time plugins
(``initialize_state``, ``initialize_walls``; src/lbm/lbm.F90:444-453,
src/lbm/lbm_walls.F90:172).  These functions produce the same arrays as numpy
vectors for tx_upload_state / tx_upload_walls: rho has s values per site
(component fastest), walls one code per site, x fastest then y, z.
"""
import numpy as np


def _grid(nx, ny, nz):
    k, j, i = np.meshgrid(np.arange(1, nz + 1), np.arange(1, ny + 1), np.arange(1, nx + 1), indexing="ij")
    return i, j, k


def bubble_box_state(nx, ny, nz, rho_inner, rho_outer, half, walls=None, only_pore=True):
    """The reference tests' bubble (tests/bubble_2D/initialize_state.F90:149-206,
    :45-124): rho_inner on the box (N+1)/2 +- half (integer division), 1-based
    inclusive bounds, rho_outer elsewhere; ``only_pore`` skips wall sites like
    the bubble_2D plugin (the *_hots plugin sets every site)."""
    s = len(rho_inner)
    i, j, k = _grid(nx, ny, nz)
    inside = (i >= (nx + 1) // 2 - half) & (i <= (nx + 1) // 2 + half)
    inside &= (j >= (ny + 1) // 2 - half) & (j <= (ny + 1) // 2 + half)
    if nz > 1:
        inside &= (k >= (nz + 1) // 2 - half) & (k <= (nz + 1) // 2 + half)
    rho = np.where(inside.ravel()[:, None], np.asarray(rho_inner, float)[None, :], np.asarray(rho_outer, float)[None, :])
    if only_pore and walls is not None:
        rho[np.asarray(walls).ravel() != 0] = 0.0
    return rho.reshape(-1, s).ravel()


def bubble_ball_state(nx, ny, nz, radius, rho_in, rho_out):
    """Centred disk (2D) or sphere (3D) of radius ``radius`` in 1-based cell
    centres: rho_in inside (distance <= radius), rho_out outside."""
    i, j, k = _grid(nx, ny, nz)
    r2 = (i - (nx + 1) / 2.0) ** 2 + (j - (ny + 1) / 2.0) ** 2
    if nz > 1:
        r2 = r2 + (k - (nz + 1) / 2.0) ** 2
    inside = (r2 <= radius * radius).ravel()
    return np.where(inside[:, None], np.asarray(rho_in, float)[None, :], np.asarray(rho_out, float)[None, :]).ravel()


def sphere_pack(shape, porosity, rmin, rmax, seed, periodic=True, max_spheres=1_000_000):
    """Seeded random overlapping spheres added until the pore fraction drops
    to ``porosity``.  shape = (nz, ny, nx); radii uniform in [rmin, rmax];
    centres uniform in the box; periodic images wrap (nearest image) when
    ``periodic``.  Returns a bool array (True = solid), natural order.
    Each sphere touches only its bounding box."""
    nz, ny, nx = shape
    dims = (nz, ny, nx)
    rng = np.random.default_rng(seed)
    solid = np.zeros(shape, dtype=bool)
    target = (1.0 - porosity) * solid.size
    nsolid = 0
    count = 0

    def axis(cc, r, n):
        if periodic:
            if 2 * r + 2 >= n:
                idx = np.arange(n)
            else:
                idx = np.arange(int(np.floor(cc - r)), int(np.ceil(cc + r)) + 1) % n
            d = (idx - cc + n / 2.0) % n - n / 2.0
        else:
            idx = np.arange(max(0, int(np.floor(cc - r))), min(n - 1, int(np.ceil(cc + r))) + 1)
            d = idx - cc
        return idx, d

    while nsolid < target and count < max_spheres:
        r = rng.uniform(rmin, rmax)
        c = rng.uniform(0, 1, 3) * np.array([nz, ny, nx])
        (iz, dz), (iy, dy), (ix, dx) = (axis(c[k], r, dims[k]) for k in range(3))
        count += 1
        if not (len(iz) and len(iy) and len(ix)):
            continue
        ball = (dz[:, None, None] ** 2 + dy[None, :, None] ** 2 + dx[None, None, :] ** 2) <= r * r
        box = np.ix_(iz, iy, ix)
        sub = solid[box]
        nsolid += int(np.count_nonzero(ball & ~sub))
        solid[box] = sub | ball
    return solid


def mineral_walls(solid, seed, nminerals=2):
    """Split solid voxels among minerals 1..nminerals with a seeded fair coin."""
    rng = np.random.default_rng(seed + 7919)
    walls = np.zeros(solid.shape, dtype=np.float64)
    ids = rng.integers(1, nminerals + 1, size=solid.shape)
    walls[solid] = ids[solid]
    return walls.ravel()


def bubble_plugin(only_pore=True):
    """The reference tests' initialize_state plugin as a driver plugin
    (plugin(params, run, walls) -> rho): reads -rho_inner and -rho_outer from
    the deck (tests/bubble_2D/initialize_state.F90:80-95, :163-180) and fills
    the box (N+1)/2 +- 10 in 3D, +- 26 in 2D (:104-109, :187-190).  The
    bubble_2D plugin leaves wall sites at 0 (only_pore=True); the bubble_3D
    and bubble_2D_hots plugins and the stock initialize_state_bubble
    (src/problem_specs/initialize_state_bubble.F90) fill every site
    (only_pore=False)."""
    def plugin(params, run, walls):
        from .options import DeckError, _reals
        s = params.ncomponents
        vals = []
        for key in ("rho_inner", "rho_outer"):
            v = run.extra.get(key)
            r = _reals(v) if v else []
            if len(r) < s:
                raise DeckError("-%s needs %d values" % (key, s))
            vals.append(r[:s])
        half = 10 if params.ndims == 3 else 26
        nz = params.nz if params.ndims == 3 else 1
        return bubble_box_state(params.nx, params.ny, nz, vals[0], vals[1], half, walls, only_pore)
    return plugin


def duct_walls(params, run):
    """The stock initialize_walls_duct plugin as a driver plugin
    (plugin(params, run) -> walls): walls of code 1 on the two faces normal to
    -duct_normal_direction (1 = x, 2 = y (default), 3 = z; src/problem_specs/
    initialize_walls_duct.F90:33-52, :63-77), in one process.  As written
    there, the top z wall is set only when NZ equals NY (the test compares the
    upper z index with NY), and a 2D lattice takes no z walls."""
    normal = int(run.extra.get("duct_normal_direction") or 2)
    nz, ny, nx = params.shape
    w = np.zeros((nz, ny, nx))
    if normal == 1:
        w[:, :, 0] = 1.0
        w[:, :, nx - 1] = 1.0
    elif normal == 2:
        w[:, 0, :] = 1.0
        w[:, ny - 1, :] = 1.0
    elif normal == 3 and params.ndims == 3:
        w[0] = 1.0
        if params.nz == params.ny:
            w[nz - 1] = 1.0
    return w.ravel()


def no_walls(params, run):
    """The stock initialize_walls_nowalls plugin: every site is pore."""
    return np.zeros(params.nsites)


def _singlephase_face(extra, face, direction):
    # the first of pressure, flux, velocity given for the face (:95-120)
    if ("bc_pressure_%s_value" % face) in extra:
        return "pressure", float(extra["bc_pressure_%s_value" % face])
    if ("bc_flux_%s_value" % face) in extra:
        return "flux", float(extra["bc_flux_%s_value" % face])
    if ("bc_velocity_%s_values" % face) in extra:
        from .options import _reals
        v = _reals(extra["bc_velocity_%s_values" % face] or "")
        return "velocity", v[direction - 1] if len(v) >= direction else 0.0
    return None, 0.0


def singlephase_state(params, run, walls):
    """The stock initialize_state_singlephase plugin as a driver plugin
    (plugin(params, run, walls) -> (rho, u)), following
    src/problem_specs/initialize_state_singlephase.F90:66-299 as written.
    Along -flow_direction (1 = x default, 2 = y, 3 = z) the two faces' values
    are read as pressure, flux or velocity (the first given).  Every
    component starts at rho = 1, u = 0; the first component then gets: for
    two pressures a linear profile 3 (p_left (1 - t) + p_right t), t = (i - 1)
    / (N - 1) over the 1-based index along the axis; for pressure and flux
    rho = 3 p, u = -flux / (3 p) (flux on the left: u = flux / (3 p)); for two
    fluxes rho = 1, u = (flux_left - flux_right) / 2; for two velocities
    rho = 1, u = mean; and the mixed velocity cases as in the source.  Every
    site is set, walls included."""
    nd, s = params.ndims, params.ncomponents
    direction = int(run.extra.get("flow_direction") or 1)
    rho = np.ones((params.nsites, s))
    u = np.zeros((params.nsites, nd, s))
    if not 1 <= direction <= nd:
        return rho.ravel(), u.ravel()
    ax = "xyz"[direction - 1]
    (bl, vl), (br, vr) = (_singlephase_face(run.extra, ax + side, direction) for side in ("m", "p"))
    r0, u0 = None, None
    if bl == "pressure":
        if br == "pressure":
            n = (params.nx, params.ny, params.nz)[direction - 1]
            i, j, k = _grid(params.nx, params.ny, params.nz if nd == 3 else 1)
            idx = (i, j, k)[direction - 1].ravel()
            t = (idx - 1.0) / (n - 1.0)
            r0 = (vl * (1 - t) + vr * t) * 3.0
        elif br == "flux":
            r0, u0 = vl * 3.0, -vr / (vl * 3.0)
        elif br == "velocity":
            r0, u0 = vl * 3.0, vr
    elif bl == "flux":
        if br == "pressure":
            r0, u0 = vr * 3.0, vl / (vr * 3.0)
        elif br == "flux":
            r0, u0 = 1.0, (vl - vr) / 2.0
        elif br == "velocity":
            r0, u0 = vl / vr, vr
    elif bl == "velocity":
        if br == "pressure":
            r0, u0 = vr * 3.0, vl
        elif br == "flux":
            r0, u0 = -vr / vl, vl
        elif br == "velocity":
            r0, u0 = 1.0, (vl + vr) / 2.0
    if r0 is not None:
        rho[:, 0] = r0
    if u0 is not None:
        u[:, direction - 1, 0] = u0
    return rho.ravel(), u.ravel()


# The stock defaults: default_initialize_state.F90 is the single-phase plugin
# (the two files are identical) and default_initialize_walls.F90 sets no walls.
default_state = singlephase_state
default_walls = no_walls
