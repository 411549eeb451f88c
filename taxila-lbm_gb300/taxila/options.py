"""The reference's input deck (a PETSc options file) mapped onto tx_params.

Mirrors OptionsSetUp (lbm_options.F90:163-365), FlowSetFromOptions
(lbm_flow.F90:188-284), FlowParseBC (lbm_flow.F90:1031-1309),
ComponentSetFromOptions (lbm_component.F90:131-176), RelaxationSetFromOptions
(lbm_relaxation.F90:117-151), MineralSetFromOptions (lbm_mineral.F90:103-134),
GridSetFromOptions/InfoSetFromOptions (lbm_grid.F90:97-132,
lbm_info.F90:116-238), FlowSetPhysicalScales (lbm_flow.F90:295-376) and
EOSSetFromOptions (lbm_eos.F90:90-300).  Option names and defaults are the
reference's, so an unchanged deck drives this library.
"""
import struct
from dataclasses import dataclass, field

from . import params as P


class DeckError(ValueError):
    """Raised where the reference would call LBMError on the deck."""


def parse_deck_text(text):
    """PETSc options-file syntax: ``-name value`` per line, ``#`` comments."""
    opts = {}
    for raw in text.splitlines():
        line = raw.split("#", 1)[0].strip()
        if not line:
            continue
        parts = line.split(None, 1)
        key = parts[0]
        if not key.startswith("-"):
            raise DeckError("option must start with '-': %r" % raw)
        opts[key[1:]] = parts[1].strip() if len(parts) > 1 else None
    return opts


def _f32(v):
    """A Fortran default-kind real literal: the value rounded to single precision."""
    return struct.unpack("f", struct.pack("f", v))[0]


def _parse_face_bc(p, f, fname, s, nd, names, has, get):
    """FlowParseBC (lbm_flow.F90:1031-1309) for one face: the kind, then its
    values in flow%bc_data(:, face) order; -1 where the deck gives none (0
    for -bc_flux).  A second kind on one face is an error, as in the
    reference; a periodic axis takes no other kind here."""
    nbcs = s * nd
    done = p.bc_flags[f] == P.BC_PERIODIC

    def on(name):
        return has(name) and _bool(get(name))

    def claim(kind, fill):
        nonlocal done
        if done:
            raise DeckError("Multiple BCs provided for boundary " + fname)
        done = True
        p.bc_flags[f] = kind
        for k in range(nbcs):
            p.bc_data[f][k] = fill

    def real(key, k):
        if has(key):
            p.bc_data[f][k] = float(get(key))

    def reals(key, k0):
        if has(key):
            vals = _reals(get(key))
            if len(vals) != nd:
                raise DeckError("%s was provided the wrong number of components." % key)
            for d, v in enumerate(vals):
                p.bc_data[f][k0 + d] = v

    if on("bc_reflecting_" + fname):
        claim(P.BC_REFLECTING, 0.0)
    if on("bc_density_" + fname):
        claim(P.BC_DENSITY, -1.0)
        for m in range(s):
            real(("bc_density_%s_value" % fname) if s == 1 else ("bc_density_%s_%s" % (fname, names[m])), m)
    if s == 1:
        if on("bc_pressure_" + fname):
            claim(P.BC_PRESSURE, -1.0)
            real("bc_pressure_%s_value" % fname, 0)
        if on("bc_flux_" + fname):
            claim(P.BC_FLUX, 0.0)
            real("bc_flux_%s_value" % fname, 0)
    if on("bc_pressure_inlet_" + fname):
        claim(P.BC_PRESSURE_INLET, -1.0)
        real("bc_pressure_%s_value" % fname, 0)
        if s > 1:
            real("bc_rho1_fraction_%s_value" % fname, 1)
    if on("bc_pressure_outlet_" + fname):
        claim(P.BC_PRESSURE_OUTLET, -1.0)
        real("bc_pressure_%s_value" % fname, 0)
    if on("bc_momentum_" + fname):
        claim(P.BC_MOMENTUM, -1.0)
        if s == 1:
            reals("bc_momentum_%s_value" % fname, 0)
        else:
            for m in range(s):
                reals("bc_momentum_%s_%s" % (fname, names[m]), m * nd)
    if on("bc_flux_inlet_" + fname):
        claim(P.BC_FLUX_INLET, -1.0)
        real("bc_flux_inlet_%s_value" % fname, 0)
        if s > 1:
            real("bc_rho1_fraction_%s_value" % fname, 1)
    if on("bc_flux_outlet_" + fname):
        claim(P.BC_FLUX_OUTLET, -1.0)
        real("bc_flux_outlet_%s_value" % fname, 0)
    if on("bc_velocity_" + fname):
        claim(P.BC_VELOCITY, -1.0)
        reals("bc_velocity_%s_values" % fname, 0)


def _bool(v):
    if v is None:
        return True
    s = v.strip().lower()
    if s in ("1", "true", "yes", "on"):
        return True
    if s in ("0", "false", "no", "off"):
        return False
    raise DeckError("not a boolean: %r" % v)


def _reals(v):
    return [float(x) for x in v.replace(" ", "").split(",") if x != ""]


@dataclass
class RunOptions:
    """Driver-level options that stay on the host (the time loop's controls)."""
    npasses: int = 1
    ntimes: int = 1
    kwrite: int = -1
    istep: int = 0
    run_to_steadystate: bool = False
    steadystate_tolerance: float = 1e-6
    steadystate_field_rho: bool = True
    steadystate_field_fi: bool = False
    walls_type: int = 1
    walls_file: str = "geometry.dat"
    output_prefix: str = ""
    output_flow_fi: bool = False
    output_flow_last_fi: bool = False  # -output_flow_last_fi: fi also at the last step
    output_last: bool = False          # -output_last: one more output after the loop
    supress_ic_output: bool = False    # -supress_ic_output: no output of the initial state
    restart: bool = False              # -restart: fi from an earlier output
    restart_counter: int = -1          # -restart_counter: its file number (else istep / kwrite)
    # -steadystate_flow: the flow stops after steadystate_rampup_steps (0 with
    # -steadystate_flow_file) and only the species step on
    steadystate_flow: bool = False
    steadystate_flow_file: str = ""
    steadystate_rampup_steps: int = 0
    # fields of each output (FlowCreate defaults, lbm_flow.F90:137-142)
    output_rho: bool = True
    output_velocity: bool = True
    output_rhot: bool = False
    output_pressure: bool = True
    waypoints: list = field(default_factory=list)  # -waypoint1, -waypoint2, ...: extra output steps
    # physical scales (GridSetPhysicalScales, FlowSetPhysicalScales): outputs of
    # rho are scaled by mass_scale / length_scale**3, of u by velocity_scale
    length_scale: float = 1.0
    mass_scale: float = 1.0
    velocity_scale: float = 1.0
    ic_file: str = ""
    ic_file_rho: str = ""
    component_names: list = field(default_factory=list)
    species_names: list = field(default_factory=list)
    mineral_names: list = field(default_factory=list)
    extra: dict = field(default_factory=dict)

    @property
    def nsteps(self):
        return self.ntimes * self.npasses


def params_from_options(opts):
    """Return (tx_params, RunOptions) for a parsed options dict."""
    p = P.default_params()
    run = RunOptions()
    get = opts.get

    def has(k):
        return k in opts

    # discretization (lbm_options.F90:303-324)
    name = get("flow_discretization") or get("discretization") or "D3Q19"
    name = name.strip().lower()
    if name.startswith("d3q19"):
        p.discretization = P.D3Q19
    elif name.startswith("d2q9"):
        p.discretization = P.D2Q9
    else:
        raise DeckError("Invalid Discretization")
    nd = p.ndims

    # grid (lbm_info.F90:150-163)
    p.nx = int(get("NX", -1))
    p.ny = int(get("NY", -1))
    p.nz = int(get("NZ", -1)) if nd == 3 else 1
    if p.nx < 1 or p.ny < 1 or p.nz < 1:
        raise DeckError("grid size -NX/-NY(/-NZ) must be given")
    for a, ax in enumerate("xyz"[:nd]):
        if has("bc_periodic_" + ax) and _bool(get("bc_periodic_" + ax)):
            p.bc_flags[2 * a] = P.BC_PERIODIC
            p.bc_flags[2 * a + 1] = P.BC_PERIODIC

    p.relaxation_mode = int(get("flow_relaxation_mode", 0))
    p.ncomponents = int(get("ncomponents", 1))
    p.nminerals = int(get("nminerals", 1))
    if not 1 <= p.ncomponents <= P.MAXC:
        raise DeckError("ncomponents must be 1..%d" % P.MAXC)
    if not 0 <= p.nminerals <= P.MAXMIN:
        raise DeckError("nminerals must be 0..%d" % P.MAXMIN)
    if has("isotropy_order"):
        p.isotropy_order = int(get("isotropy_order"))
    elif has("derivative_order"):
        p.isotropy_order = int(get("derivative_order"))

    # components (lbm_component.F90:82-176, lbm_relaxation.F90:117-151)
    s = p.ncomponents
    names = []
    for m in range(s):
        nm = get("component%d_name" % (m + 1)) or "component%d" % (m + 1)
        names.append(nm.strip())
    run.component_names = names
    viscosity = [-999.0] * s
    density = [-999.0] * s
    for m, nm in enumerate(names):
        if p.relaxation_mode == P.SRT:
            if has("tau_" + nm):
                p.tau[m] = float(get("tau_" + nm))
        else:
            for key in ("s_c", "s_e", "s_e2", "s_q", "s_nu", "s_pi", "s_m"):
                if has(key + "_" + nm):
                    getattr(p, key)[m] = float(get(key + "_" + nm))
        if has("mm_" + nm):
            p.mm[m] = float(get("mm_" + nm))
        if has("viscosity_" + nm):
            viscosity[m] = float(get("viscosity_" + nm))
        if has("density_" + nm):
            density[m] = float(get("density_" + nm))
        for q in range(s):
            key = "g_%d%d" % (m + 1, q + 1)
            if has(key):
                p.g[m][q] = float(get(key))

    # non-ideal EOS per component (EOSSetFromOptions, lbm_eos.F90:90-300)
    if _bool(get("flow_use_nonideal_eos", "0")):
        p.use_nonideal_eos = 1
        for m, nm in enumerate(names):
            kind = (get("eos_" + nm) or "").strip().lower()
            if kind.startswith("rho"):
                p.eos[m] = P.EOS_RHO
            elif kind.startswith("sc"):
                p.eos[m] = P.EOS_SC
                p.eos_coef[m][0] = float(get("eos_sc_rho0_" + nm, 1.0))
            elif kind.startswith("thermo"):
                p.eos[m] = P.EOS_THERMO
                p.eos_coef[m][0] = float(get("eos_thermo_psi0_" + nm, 1.0))
                p.eos_coef[m][1] = float(get("eos_thermo_rho0_" + nm, 1.0))
            elif kind.startswith("pr"):
                p.eos[m] = P.EOS_PR
                a = float(get("eos_pr_a_" + nm, 2.0 / 49.0))
                b = float(get("eos_pr_b_" + nm, 2.0 / 21.0))
                # lbm_eos.F90:296 and the 0.9 / 0.344 defaults are single-precision literals
                tc = a / b * _f32(0.0778) / _f32(0.45724) / 1.0
                if has("eos_pr_T_" + nm):
                    t = float(get("eos_pr_T_" + nm))
                else:
                    t = (float(get("eos_pr_reduced_T_" + nm)) if has("eos_pr_reduced_T_" + nm) else _f32(0.9)) * tc
                p.eos_coef[m][0], p.eos_coef[m][1], p.eos_coef[m][2] = a, b, t
                p.eos_coef[m][3] = float(get("eos_pr_omega_" + nm)) if has("eos_pr_omega_" + nm) else _f32(0.344)
            else:
                raise DeckError("Invalid EOS type")

    # minerals (lbm_mineral.F90:64-134)
    mnames = []
    for q in range(p.nminerals):
        nm = get("mineral%d_name" % (q + 1)) or "mineral%d" % (q + 1)
        mnames.append(nm.strip())
        for m in range(s):
            key = "gw_%s_%s" % (nm.strip(), names[m])
            if has(key):
                p.gw[q][m] = float(get(key))
    run.mineral_names = mnames

    # body force (lbm_flow.F90:224-231)
    if has("gvt"):
        g = _reals(get("gvt"))
        p.body_forces = 1
        for d in range(min(nd, len(g))):
            p.gvt[d] = g[d]

    # boundary conditions (FlowParseBC, lbm_flow.F90:1031-1309)
    for f, fname in enumerate(P.FACE_NAMES[: 2 * nd]):
        _parse_face_bc(p, f, fname, s, nd, names, has, get)

    run.length_scale = _length_scale(p, get)
    run.mass_scale, run.velocity_scale = _physical_scales(p, viscosity, density, run.length_scale)

    # transport (lbm_options.F90:326-361, TransportSetFromOptions lbm_transport.F90:130-245,
    # SpecieSetFromOptions lbm_species.F90:111-133)
    if has("transport_discretization"):
        tname = get("transport_discretization").strip().lower()
        if tname.startswith("d3q19"):
            tdims = 3
        elif tname.startswith("d2q9"):
            tdims = 2
        else:
            raise DeckError("Invalid Discretization")
        if tdims != nd:
            raise DeckError("Flow and transport discretization dimensions don't match")
        p.nspecies = int(get("nspecies", 1))
        if not 1 <= p.nspecies <= P.MAXC:
            raise DeckError("nspecies must be 1..%d" % P.MAXC)
        p.species_relaxation_mode = int(get("transport_relaxation_mode", 0))
        if _bool(get("reactive_matrix", "0")):
            raise DeckError("-reactive_matrix: dissolution/precipitation is not on this path")
        snames = []
        rate_keys = ("s_c", "s_e", "s_e2", "s_q", "s_nu", "s_pi", "s_m")
        for sp in range(p.nspecies):
            nm = "specie%d" % (sp + 1)
            nm = (get(nm + "_name") or nm).strip()
            snames.append(nm)
            if p.species_relaxation_mode == P.SRT:
                if has("tau_" + nm):
                    p.species_tau[sp] = float(get("tau_" + nm))
            else:
                for k, key in enumerate(rate_keys):
                    if has(key + "_" + nm):
                        p.species_rates[sp][k] = float(get(key + "_" + nm))
        run.species_names = snames

    # driver options (lbm_options.F90:184-262)
    run.npasses = int(get("npasses", 1))
    run.ntimes = int(get("ntimes", 1))
    run.kwrite = int(get("kwrite", -1))
    run.istep = int(get("istep", 0))
    run.run_to_steadystate = _bool(get("run_to_steadystate", "0"))
    if run.run_to_steadystate:
        run.steadystate_tolerance = float(get("steadystate_tolerance", 1e-6))
        run.steadystate_field_rho = _bool(get("steadystate_field_rho", "1"))
        run.steadystate_field_fi = _bool(get("steadystate_field_fi", "0"))
    run.walls_type = int(get("walls_type", 1))
    run.walls_file = (get("walls_file") or "geometry.dat").strip()
    run.output_prefix = (get("output_file_prefix") or "").strip()
    run.output_flow_fi = _bool(get("output_flow_fi", "0"))
    # output options (lbm_options.F90:240-241, lbm_flow.F90:262-279)
    run.output_flow_last_fi = _bool(get("output_flow_last_fi", "0"))
    run.output_last = _bool(get("output_last", "0"))
    run.supress_ic_output = _bool(get("supress_ic_output", "0"))
    run.restart = _bool(get("restart", "0"))
    run.restart_counter = int(get("restart_counter", -1))
    # steady flow (lbm_options.F90:204-215): ramp-up steps only without a flow file
    run.steadystate_flow = _bool(get("steadystate_flow", "0"))
    if run.steadystate_flow:
        run.steadystate_flow_file = (get("steadystate_flow_file") or "").strip()
        if not has("steadystate_flow_file"):
            run.steadystate_rampup_steps = int(get("steadystate_rampup_steps", 0))
    run.output_rho = _bool(get("output_rho", "1"))
    run.output_velocity = _bool(get("output_velocity", "1"))
    run.output_rhot = _bool(get("output_rhot", "0"))
    run.output_pressure = _bool(get("output_pressure", "1"))
    # waypoints (lbm_options.F90:243-276): -waypoint1, -waypoint2, ... up to
    # the first number that is not given
    wps = []
    while has("waypoint%d" % (len(wps) + 1)):
        wps.append(int(get("waypoint%d" % (len(wps) + 1))))
    run.waypoints = wps
    run.ic_file = (get("ic_file") or "").strip()
    run.ic_file_rho = (get("ic_file_rho") or "").strip()
    run.extra = dict(opts)
    return p, run


def _length_scale(p, get):
    """Lattice spacing (InfoSetFromOptions, lbm_info.F90:164-222, and
    GridSetPhysicalScales, lbm_grid.F90:80-95): corners default to 0 and N
    (periodic axis) or N - 1, overridden by -x_start/-x_end etc.; the spacing
    (end - start) / N (periodic) or / (N - 1) must be the same on every axis."""
    sizes = []
    for a, (ax, n) in enumerate(zip("xyz"[:p.ndims], (p.nx, p.ny, p.nz))):
        per = p.bc_flags[2 * a] == P.BC_PERIODIC
        start = float(get(ax + "_start", 0.0))
        end = float(get(ax + "_end", n if per else n - 1))
        sizes.append((end - start) / (n if per else n - 1) if (per or n > 1) else float("nan"))
    for h in sizes[1:]:
        if abs(h - sizes[0]) > 1.e-8:  # as in the reference, a NaN spacing (N = 1, not periodic) passes
            raise DeckError("Lattice sizes must be equal, check grid parameters.")
    return sizes[0]


def _physical_scales(p, viscosity, density, length_scale=1.0):
    """FlowSetPhysicalScales (lbm_flow.F90:295-376): tau / mm consistency.

    Component 1's tau and mm are taken as correct; other components' tau/mm
    are derived from -viscosity_<c>/-density_<c> when those are given.
    Returns (mass_scale, velocity_scale)."""
    eps = 1.e-8
    if viscosity[0] < -990.0:
        time_scale = 1.0
    else:
        time_scale = length_scale * length_scale * (p.tau[0] - 0.5) / (viscosity[0] * 3.)
    if density[0] < -990.0:
        density[0] = 1.0
    mass_scale = p.mm[0] * density[0] * length_scale ** 3
    for m in range(1, p.ncomponents):
        if viscosity[m] >= -990.0:
            consistent_tau = (3. * time_scale * viscosity[m]) / (length_scale * length_scale) + 0.5
            if abs(p.tau[m] - 1.) < eps:
                p.tau[m] = consistent_tau
            elif abs(p.tau[m] - consistent_tau) > eps:
                raise DeckError("Viscosities and relaxation times specified for components are not consistent.")
        if density[m] >= -990.0:
            consistent_mm = mass_scale / density[0] / length_scale ** 3
            if abs(p.mm[m] - 1.) < eps:
                p.mm[m] = consistent_mm
            elif abs(p.mm[m] - consistent_mm) > eps:
                raise DeckError("Densities and molecular masses specified for components are not consistent.")
    return mass_scale, length_scale / time_scale


def load_deck(path):
    with open(path) as f:
        return params_from_options(parse_deck_text(f.read()))
