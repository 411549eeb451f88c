"""Host driver mirroring the reference's LBM object (src/lbm/lbm.F90).

    lbm = LBM.from_deck("input_data")              # LBMCreate + LBMSetFromOptions
    lbm.setup(initialize_walls=...)                # LBMSetUp (walls file or plugin)
    lbm.initialize_state(initialize_state)         # LBMInitializeState (plugin)
    lbm.init()                                     # LBMInit   -> tx_init
    lbm.run()                                      # LBMRun    -> tx_step + outputs
    lbm.destroy()                                  # LBMDestroy

or, all of it in the order of the reference's main program (restart and
initial-condition files included): main(deck, initialize_state=..., ...).

The time loop, output cadence (-kwrite, -waypointN, -output_last), steady-state exit and
PETSc-binary output stay on the host exactly as in LBMRun2 (lbm.F90:262-422);
each flow step is one tx_step on the GPU.
"""
import os

import numpy as np

from . import options as O
from . import params as P
from . import petsc_io
from ._lib import Handle


class LBM:
    def __init__(self, params, run, name=""):
        self.params = P.copy_params(params)
        self.run_opts = run
        self.name = name
        self.handle = None
        self.walls = None
        self.counter = 0
        self.nd = self.params.ndims
        self.io_fi = run.output_flow_fi  # flow%io_fi: -output_last_fi turns it on at the last step, for good
        self.waypoint = 0                # index of the next waypoint (current_waypoint - 1)

    # LBMCreate + OptionsSetUp + LBMSetFromOptions
    @classmethod
    def from_deck(cls, path_or_text, **overrides):
        text = open(path_or_text).read() if os.path.exists(str(path_or_text)) else str(path_or_text)
        p, run = O.params_from_options(O.parse_deck_text(text))
        for k, v in overrides.items():
            setattr(p, k, v)
        return cls(p, run)

    # LBMSetUp (lbm.F90:140-175): device state and walls
    def setup(self, initialize_walls=None, handle=None):
        # handle: an already created device handle for these parameters (default: a new one)
        self.handle = Handle(self.params) if handle is None else handle
        z, y, x = self.params.shape
        if self.run_opts.walls_type == 2 or initialize_walls is not None:
            w = np.zeros(self.params.nsites) if initialize_walls is None else initialize_walls(self.params, self.run_opts)
        else:
            w = petsc_io.read_field(self.run_opts.walls_file, self.params.nsites, 1)
        self.walls = np.ascontiguousarray(w, dtype=np.float64).ravel()
        self.handle.upload_walls(self.walls)
        return self

    # LBMInitializeState (lbm.F90:444-453): the plugin fills rho (and u)
    def initialize_state(self, initialize_state):
        res = initialize_state(self.params, self.run_opts, self.walls)
        rho, u = res if isinstance(res, tuple) else (res, None)
        self.handle.upload_state(rho, u)

    # LBMInitializeStateFromFile (lbm.F90:482-517)
    # LBMInitializeState_FlowTransport (lbm.F90:455-480): the transport plugin's
    # concentrations [N*ns] and, optionally, fluxes [N*ndims*ns]
    def initialize_species(self, conc, flux=None):
        self.handle.upload_species(conc, flux)

    def initialize_state_from_file(self):
        n, s, q = self.params.nsites, self.params.ncomponents, self.params.Q
        if self.run_opts.ic_file:
            self.handle.upload_fi(petsc_io.read_field(self.run_opts.ic_file, n, s * q))
        elif self.run_opts.ic_file_rho:
            self.handle.upload_state(petsc_io.read_field(self.run_opts.ic_file_rho, n, s))
        else:
            raise O.DeckError("-ic_file or -ic_file_rho required")

    # LBMInitializeStateRestarted (lbm.F90:519-544): the file number is
    # -restart_counter, else istep / kwrite
    def initialize_state_restarted(self, counter=None):
        ro = self.run_opts
        if counter is None:
            if ro.restart_counter > -1:
                counter = ro.restart_counter
            elif ro.kwrite > 0:
                counter = ro.istep // ro.kwrite
            else:
                raise O.DeckError("must set -restart_counter to define which file to restart from")
        self.counter = counter
        name = petsc_io.output_name(self.run_opts.output_prefix, "fi", counter)
        n, s, q = self.params.nsites, self.params.ncomponents, self.params.Q
        self.handle.upload_fi(petsc_io.read_field(name, n, s * q))

    # LBMInit2 (lbm.F90:183-253): walls (step 0 only) and the initial fields
    # unless -supress_ic_output; the output counter advances either way, so
    # the first output of the run is file 001
    def init(self, istep=0, suppress_output=None):
        if suppress_output is None:
            suppress_output = self.run_opts.supress_ic_output
        self.handle.init()
        if not suppress_output:
            if istep == 0:
                self._write("walls", self.walls, 1)
            self._write_fields()
        self.counter += 1

    # LBMOutput (lbm.F90:424-442) / FlowOutputDiagnostics (lbm_flow.F90:576-601)
    def output(self, istep, with_fi=None):
        ro = self.run_opts
        # a flow held at steady state writes no flow fields after its ramp-up
        flow = not ro.steadystate_flow or istep < ro.steadystate_rampup_steps
        self._write_fields(with_fi, flow=flow)
        self.counter += 1

    def _write_fields(self, with_fi=None, flow=True):
        h = self.handle
        if flow:
            self._write_flow(h, with_fi)
        if self.params.nspecies > 0:
            # TransportOutputDiagnostics (lbm_transport.F90:342-356): gi and psi
            ns = self.params.nspecies
            self._write("gi", h.download(P.FIELD_SPECIES_FI), ns * self.params.Q)
            self._write("psi", h.download(P.FIELD_SPECIES_RHO), ns)

    def _write_flow(self, h, with_fi):
        ro = self.run_opts
        if with_fi if with_fi is not None else self.io_fi:
            self._write("fi", h.download(P.FIELD_FI), self.params.ncomponents * self.params.Q)
        if ro.output_rho:
            rho = h.download(P.FIELD_RHO)
            if ro.mass_scale != 1.0 or ro.length_scale != 1.0:
                rho = rho * (ro.mass_scale / ro.length_scale ** 3)
            self._write("rho", rho, self.params.ncomponents)
        if ro.output_velocity:
            u = h.download(P.FIELD_VELT)
            if ro.velocity_scale != 1.0:
                u = u * ro.velocity_scale
            self._write("u", u, self.nd)
        if ro.output_rhot:
            self._write("rhot", h.download(P.FIELD_RHOT), 1)
        if ro.output_pressure:
            self._write("prs", h.download(P.FIELD_PRS), 1)

    def _write(self, name, arr, dof):
        pre = self.run_opts.output_prefix
        if pre and os.path.dirname(pre):
            os.makedirs(os.path.dirname(pre), exist_ok=True)
        petsc_io.write_vec(petsc_io.output_name(pre, name, self.counter), arr, dof)

    # the output check of LBMRun2 (lbm.F90:373-391): the next waypoint, else
    # the -kwrite cadence; at the last step -output_flow_last_fi adds fi
    def _output_check(self, step, kstep):
        ro = self.run_opts
        wps = ro.waypoints
        hit = False
        if self.waypoint < len(wps) and wps[self.waypoint] == step:
            hit = True
            self.waypoint += 1
        elif ro.kwrite > 0 and step % ro.kwrite == 0:
            hit = True
        if hit:
            if step == kstep:
                self.io_fi = self.io_fi or ro.output_flow_last_fi
            self.output(step)

    # LBMRun2 (lbm.F90:262-422)
    def run(self, istep=None, kstep=None, write_output=True):
        ro = self.run_opts
        istep = ro.istep if istep is None else istep
        kstep = ro.nsteps if kstep is None else kstep
        kw = ro.kwrite
        steady = ro.run_to_steadystate
        field = P.FIELD_FI if ro.steadystate_field_fi else P.FIELD_RHO
        step = istep
        last = kstep + 1  # the loop variable after a loop that ran to the end
        while step < kstep:
            # advance to the next step that needs host work
            nxt = kstep
            if steady:
                nxt = step + 1
            elif write_output:
                if kw > 0:
                    nxt = min(nxt, (step // kw + 1) * kw)
                if self.waypoint < len(ro.waypoints) and ro.waypoints[self.waypoint] > step:
                    nxt = min(nxt, ro.waypoints[self.waypoint])
            if ro.steadystate_flow and step + 1 >= ro.steadystate_rampup_steps:
                # -steadystate_flow after the ramp-up: the flow calls of the
                # loop are skipped (lbm.F90:283-363), the species step on
                if self.params.nspecies > 0:
                    self.handle.step_species(nxt - step)
            else:
                if ro.steadystate_flow:
                    nxt = min(nxt, ro.steadystate_rampup_steps - 1)
                self.handle.step(nxt - step)
            step = nxt
            if write_output:
                self._output_check(step, kstep)
            if steady:
                norm = self.handle.delta_norm(field)
                if norm < ro.steadystate_tolerance and step > istep + 2:
                    last = step
                    break
        # -output_last: one more output after the loop (lbm.F90:407-416)
        if write_output and ro.output_last:
            self.io_fi = self.io_fi or ro.output_flow_last_fi
            self.output(last)
        return step

    def download(self, field):
        return self.handle.download(field)

    def destroy(self):
        if self.handle is not None:
            self.handle.close()
            self.handle = None


def main(deck, initialize_state=None, initialize_walls=None, initialize_bcs=None, initialize_species=None,
         handle=None, overrides=None):
    """One run of a deck, in the order of the reference's main program
    (src/lbm/main.F90:45-104).  The plugins are the reference's link-time
    externals as callables: initialize_walls(params, run) -> walls (else the
    walls file), initialize_bcs(params, run) -> {face: values of
    tx_upload_bc_values} (else the deck's constant face values),
    initialize_state(params, run, walls) -> rho or (rho, u), and
    initialize_species(params, run, walls) -> conc or (conc, flux).  A restart
    (-restart) reads fi from the output file of -restart_counter (else
    istep / kwrite); -ic_file / -ic_file_rho read the initial state from
    PETSc-binary files.  overrides: tx_params members to set after the deck
    is read (e.g. {"exact": 1}).  Returns the LBM object after its last
    step, with the device handle released."""
    lbm = LBM.from_deck(deck, **(overrides or {}))
    ro = lbm.run_opts
    try:
        lbm.setup(initialize_walls, handle=handle)
        if initialize_bcs is not None:
            for face, vals in initialize_bcs(lbm.params, ro).items():
                lbm.handle.upload_bc_values(face, vals)
        if ro.restart:
            lbm.initialize_state_restarted()
            istep = ro.istep
        elif ro.ic_file or ro.ic_file_rho:
            lbm.initialize_state_from_file()
            istep = 0
        else:
            if initialize_state is None:
                raise O.DeckError("an initialize_state plugin, -ic_file/-ic_file_rho or -restart is required")
            lbm.initialize_state(initialize_state)
            istep = 0
        if lbm.params.nspecies > 0 and not ro.restart:
            if initialize_species is None:
                raise O.DeckError("a deck with species needs an initialize_species plugin")
            res = initialize_species(lbm.params, ro, lbm.walls)
            conc, flux = res if isinstance(res, tuple) else (res, None)
            lbm.initialize_species(conc, flux)
        lbm.init(istep)
        lbm.run(istep, ro.nsteps)
    finally:
        lbm.destroy()
    return lbm
