"""Host driver mirroring the reference's LBM object (src/lbm/lbm.F90).

    lbm = LBM.from_deck("input_data")              # LBMCreate + LBMSetFromOptions
    lbm.setup(initialize_walls=...)                # LBMSetUp (walls file or plugin)
    lbm.initialize_state(initialize_state)         # LBMInitializeState (plugin)
    lbm.init()                                     # LBMInit   -> tx_init
    lbm.run()                                      # LBMRun    -> tx_step + outputs
    lbm.destroy()                                  # LBMDestroy

The time loop, output cadence (-kwrite, waypoints), steady-state exit and
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

    # LBMCreate + OptionsSetUp + LBMSetFromOptions
    @classmethod
    def from_deck(cls, path_or_text, **overrides):
        text = open(path_or_text).read() if os.path.exists(str(path_or_text)) else str(path_or_text)
        p, run = O.params_from_options(O.parse_deck_text(text))
        for k, v in overrides.items():
            setattr(p, k, v)
        return cls(p, run)

    # LBMSetUp (lbm.F90:140-175): device state and walls
    def setup(self, initialize_walls=None):
        self.handle = Handle(self.params)
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

    # LBMInitializeStateRestarted (lbm.F90:519-544)
    def initialize_state_restarted(self, counter):
        self.counter = counter
        name = petsc_io.output_name(self.run_opts.output_prefix, "fi", counter)
        n, s, q = self.params.nsites, self.params.ncomponents, self.params.Q
        self.handle.upload_fi(petsc_io.read_field(name, n, s * q))

    # LBMInit2 (lbm.F90:183-253)
    def init(self, istep=0, suppress_output=True):
        self.handle.init()
        if not suppress_output and istep == 0:
            self._write("walls", self.walls, 1)
            self.output(istep)

    # LBMOutput (lbm.F90:424-442) / FlowOutputDiagnostics (lbm_flow.F90:576-601)
    def output(self, istep, with_fi=None):
        pre = self.run_opts.output_prefix
        if pre and os.path.dirname(pre):
            os.makedirs(os.path.dirname(pre), exist_ok=True)
        h = self.handle
        if with_fi if with_fi is not None else self.run_opts.output_flow_fi:
            self._write("fi", h.download(P.FIELD_FI), self.params.ncomponents * self.params.Q)
        self._write("rho", h.download(P.FIELD_RHO), self.params.ncomponents)
        self._write("u", h.download(P.FIELD_VELT), self.nd)
        self._write("prs", h.download(P.FIELD_PRS), 1)
        if self.params.nspecies > 0:
            # TransportOutputDiagnostics (lbm_transport.F90:342-356): gi and psi
            ns = self.params.nspecies
            self._write("gi", h.download(P.FIELD_SPECIES_FI), ns * self.params.Q)
            self._write("psi", h.download(P.FIELD_SPECIES_RHO), ns)
        self.counter += 1

    def _write(self, name, arr, dof):
        petsc_io.write_vec(petsc_io.output_name(self.run_opts.output_prefix, name, self.counter), arr, dof)

    # LBMRun2 (lbm.F90:262-422)
    def run(self, istep=None, kstep=None, write_output=True):
        istep = self.run_opts.istep if istep is None else istep
        kstep = self.run_opts.nsteps if kstep is None else kstep
        kw = self.run_opts.kwrite
        steady = self.run_opts.run_to_steadystate
        field = P.FIELD_FI if self.run_opts.steadystate_field_fi else P.FIELD_RHO
        step = istep
        while step < kstep:
            # advance to the next step that needs host work
            nxt = kstep
            if steady:
                nxt = step + 1
            elif write_output and kw > 0:
                nxt = min(kstep, (step // kw + 1) * kw)
            self.handle.step(nxt - step)
            step = nxt
            if write_output and kw > 0 and step % kw == 0:
                self.output(step, with_fi=self.run_opts.output_flow_fi)
            if steady:
                norm = self.handle.delta_norm(field)
                if norm < self.run_opts.steadystate_tolerance and step > istep + 2:
                    break
        return step

    def download(self, field):
        return self.handle.download(field)

    def destroy(self):
        if self.handle is not None:
            self.handle.close()
            self.handle = None
