/*
 * taxila_gb300.h - C ABI of the GB300 Shan-Chen lattice-Boltzmann step.
 *
 * This library is a drop-in for the flow part of Taxila LBM's time step.  The
 * reference runs, once per step, the Fortran module procedures
 *
 *   FlowCollision              (src/lbm/lbm_flow.F90:936-958)
 *   DistributionCommunicateFi  (src/lbm/lbm_distribution_function.F90:309-314)
 *   FlowStream                 (src/lbm/lbm_flow.F90:810-814)
 *   FlowBounceback             (src/lbm/lbm_flow.F90:816-820)
 *   FlowApplyBCs               (src/lbm/lbm_flow.F90:1958-1991)
 *   FlowUpdateFlux             (src/lbm/lbm_flow.F90:458-464)
 *
 * from LBMRun2 (src/lbm/lbm.F90:279-406), and FlowFiInit + FlowUpdateMoments
 * from LBMInit2 (src/lbm/lbm.F90:212, :238).  tx_init and tx_step replace those
 * calls; the Fortran host keeps the options deck, the plugins, I/O and the
 * loop.  All arrays crossing this boundary are host arrays in the reference's
 * natural (PETSc global vector) order: for a field with `dof` values per
 * lattice site the value (d, i, j, k) is at d + dof*(i + NX*(j + NY*k)),
 * i.e. the dof index fastest, then x, y, z.  Populations use
 * dof = m + s*n (component fastest), exactly as the reference's fi vector
 * (src/lbm/lbm_distribution_function.F90:197-202).
 *
 * Every entry point returns 0 on success and a nonzero TX_ERR_* code on
 * failure (the reference's PetscErrorCode convention, src/lbm/lbm.F90:122-136);
 * tx_last_error() gives the message.  The device never traps: NaN/Inf
 * populations and exhausted step budgets come back as status codes.
 * A handle is single-threaded and owns one CUDA stream and all device memory.
 */
#ifndef TAXILA_GB300_H
#define TAXILA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TX_MAX_COMPONENTS 4  /* reference NMAX_COMPONENTS = 5 (include/lbm_definitions.h:79) */
#define TX_MAX_MINERALS 16

/* discretization enum values of include/lbm_definitions.h:9-11 */
#define TX_D3Q19 1
#define TX_D2Q9 2

/* relaxation modes, include/lbm_definitions.h:68-69 */
#define TX_RELAX_SRT 0
#define TX_RELAX_MRT 1

/* per-face flow BC kinds (flow%bc_flags), include/lbm_definitions.h:30-43, and
 * what tx_params.bc_data[face] holds for each (flow%bc_data(:, face),
 * FlowParseBC, src/lbm/lbm_flow.F90:1031-1309).  Node values per kind are set
 * up as FlowSetUpBCsD3/D2 do (lbm_flow.F90:1311-1956). */
#define TX_BC_NULL 0            /* non-periodic face closed by ghost walls (bounceback) */
#define TX_BC_PERIODIC 1
#define TX_BC_REFLECTING 2      /* -bc_reflecting_<face>: mirror the incoming populations */
#define TX_BC_VELOCITY 5        /* -bc_velocity_<face>_values: bc_data[0..ndims-1] = u */
#define TX_BC_DENSITY 6         /* -bc_density_<face>_<c>: bc_data[m] = rho_m */
#define TX_BC_MOMENTUM 7        /* -bc_momentum_<face>_<c>: bc_data[m*ndims + d] = (rho u)_m,d */
#define TX_BC_PRESSURE 8        /* one component: bc_data[0] = p, rho = 3 p */
#define TX_BC_PRESSURE_INLET 9  /* bc_data[0] = p, bc_data[1] = rho_1 / sum(rho) */
#define TX_BC_PRESSURE_OUTLET 10 /* bc_data[0] = p; two components: rho_1 / sum(rho) from the
                                   neighbour inside, every step */
#define TX_BC_FLUX 11           /* one component: bc_data[0] = inward flux */
#define TX_BC_FLUX_INLET 12     /* bc_data[0] = flux, bc_data[1] = rho_1 / sum(rho) */
#define TX_BC_FLUX_OUTLET 13    /* bc_data[0] = flux */

/* faces, include/lbm_definitions.h:47-52 (index = value - 1 in arrays below) */
#define TX_XM 1
#define TX_XP 2
#define TX_YM 3
#define TX_YP 4
#define TX_ZM 5
#define TX_ZP 6

/* storage/arithmetic forms */
#define TX_PREC_F64 0      /* plain form: FP64 populations and arithmetic */
#define TX_PREC_F32 1      /* FP32 arithmetic, FP32 populations stored as f - w_n*rho0[m] */
#define TX_PREC_F32_F16 2  /* FP32 arithmetic, FP16 populations stored as (f - w_n*rho0[m]) * storage_scale */

/* fields for tx_download / tx_delta_norm */
#define TX_FIELD_FI 1      /* s*Q dof: populations after the step (reference fi)          */
#define TX_FIELD_RHO 2     /* s dof: component densities (reference rho)                  */
#define TX_FIELD_FLUX 3    /* s*ndims dof: reference flux array = common velocity u_eq    */
#define TX_FIELD_FORCES 4  /* s*ndims dof: Shan-Chen + fluid-solid + body forces          */
#define TX_FIELD_PRS 5     /* 1 dof: pressure diagnostic (FlowUpdateDiagnostics)          */
#define TX_FIELD_VELT 6    /* ndims dof: total velocity diagnostic                        */
#define TX_FIELD_RHOT 7    /* 1 dof: total mass density diagnostic                        */
#define TX_FIELD_WALLS 8   /* 1 dof: wall codes as uploaded                               */
#define TX_FIELD_PSI 12    /* s dof: Shan-Chen potential psi(rho) (= rho without an EOS)  */
#define TX_FIELD_SPECIES_FI 9    /* ns*Q dof: transported species populations (reference gi) */
#define TX_FIELD_SPECIES_RHO 10  /* ns dof: species concentrations (reference psi)           */
#define TX_FIELD_SPECIES_FLUX 11 /* ns*ndims dof: species flux sum_n g_n c_n                 */

/* error codes */
#define TX_OK 0
#define TX_EOS_RHO 0        /* psi = rho */
#define TX_EOS_SC 1         /* psi = rho0 (1 - exp(-rho / rho0))       (Shan & Chen 1993) */
#define TX_EOS_THERMO 2     /* psi = psi0 exp(-rho0 / rho)             (Shan & Chen 1994) */
#define TX_EOS_PR 3         /* Peng-Robinson: psi = sqrt(2 (p(rho) - rho/3) / (c0 g_mm)) */

#define TX_ERR_ARG 1       /* invalid argument / unsupported parameter combination */
#define TX_ERR_STATE 2     /* call out of order (e.g. tx_step before tx_init) */
#define TX_ERR_CUDA 3      /* CUDA runtime error (message has the CUDA string) */
#define TX_ERR_NOMEM 4     /* device allocation failed or over the memory budget */
#define TX_ERR_NONFINITE 5 /* NaN/Inf detected in a reduction */
#define TX_ERR_NODEVICE 6  /* no CUDA device / kernels not built for this device */

typedef struct tx_params {
  int32_t discretization;   /* TX_D2Q9 or TX_D3Q19 (-discretization) */
  int32_t nx, ny, nz;       /* -NX -NY -NZ (nz = 1 for D2Q9) */
  int32_t ncomponents;      /* -ncomponents, 1..TX_MAX_COMPONENTS */
  int32_t nminerals;        /* -nminerals, 0..TX_MAX_MINERALS */
  int32_t relaxation_mode;  /* -flow_relaxation_mode */
  int32_t isotropy_order;   /* -isotropy_order / -derivative_order: 4, 8 (D2Q9 also 10) */
  int32_t bc_flags[6];      /* TX_BC_* per face XM..ZP; periodic faces come in pairs */
  double tau[TX_MAX_COMPONENTS];  /* -tau_<c> (SRT) */
  double s_c[TX_MAX_COMPONENTS];  /* -s_c_<c> .. -s_m_<c> (MRT rates) */
  double s_e[TX_MAX_COMPONENTS];
  double s_e2[TX_MAX_COMPONENTS];
  double s_q[TX_MAX_COMPONENTS];
  double s_nu[TX_MAX_COMPONENTS];
  double s_pi[TX_MAX_COMPONENTS];
  double s_m[TX_MAX_COMPONENTS];
  double mm[TX_MAX_COMPONENTS];                       /* -mm_<c> molecular masses */
  double g[TX_MAX_COMPONENTS][TX_MAX_COMPONENTS];     /* -g_<mn>: g[m][n] */
  double gw[TX_MAX_MINERALS][TX_MAX_COMPONENTS];      /* -gw_<mineral>_<c> */
  int32_t body_forces;      /* 1 when -gvt was given */
  double gvt[3];            /* -gvt */
  double bc_data[6][3 * TX_MAX_COMPONENTS];  /* per face: the kind's values (see TX_BC_*) */
  int32_t literal_kind;     /* 4: the reference's default-REAL literals (1./6. etc.) are
                               single precision, as built without -fdefault-real-8; 8: double */
  int32_t precision;        /* TX_PREC_* */
  int32_t exact;            /* 1: reference operation order, IEEE divides, no FMA (FP64 only) */
  double rho0[TX_MAX_COMPONENTS]; /* precision forms: per-component rest density rho0 of the
                               deviation storage f - w_n*rho0 (0 = plain storage; pick the density
                               the component mostly has, e.g. 1 for single-phase flow) */
  double storage_scale;     /* FP16 form: populations stored as (f - w_n*rho0) * storage_scale
                               (a power of two keeps the scaling exact; 0 = 1) */
  /* passive species (LBM_Transport_module, src/lbm/lbm_transport.F90): the
   * -nspecies / -transport_relaxation_mode / -tau_<specie> / -s_*_<specie>
   * options.  The transport lattice is the flow's (same discretization and
   * faces); species feel no force and no boundary condition. */
  /* non-ideal equation of state psi(rho) per component: -flow_use_nonideal_eos
   * with -eos_<component> {rho,sc,thermo,pr} (LBM_EOS_module,
   * src/lbm/lbm_eos.F90:183-350).  psi replaces rho in the fluid-fluid force
   * and the pressure diagnostic (FlowCalcForces, lbm_flow.F90:790-806). */
  int32_t use_nonideal_eos;
  int32_t eos[TX_MAX_COMPONENTS];          /* TX_EOS_RHO, TX_EOS_SC, TX_EOS_THERMO, TX_EOS_PR */
  double eos_coef[TX_MAX_COMPONENTS][4];   /* SC: rho0 | thermo: psi0, rho0 | PR: a, b, T, omega */
  int32_t nspecies;                        /* 0 = no transport */
  int32_t species_relaxation_mode;         /* TX_RELAX_SRT or TX_RELAX_MRT */
  double species_tau[TX_MAX_COMPONENTS];   /* SRT relaxation time */
  double species_rates[TX_MAX_COMPONENTS][7]; /* MRT s_c, s_e, s_e2, s_q, s_nu, s_pi, s_m */
} tx_params;

typedef struct tx_handle tx_handle;

/* Fill *p with the reference's defaults (lbm_options.F90:105-148,
 * lbm_relaxation.F90:65-84, lbm_component.F90:99-111). */
int tx_params_default(tx_params* p);

/* LBMSetUp (src/lbm/lbm.F90:140-175) for the flow: validates the parameters
 * (FlowSetFromOptions, lbm_flow.F90:188-284) and allocates device state. */
int tx_create(const tx_params* p, tx_handle** out);

/* LBMDestroy (src/lbm/lbm.F90:99-108). */
int tx_destroy(tx_handle* h);

/* Last error message of this handle.  With h NULL: the message of the calling
 * host thread's last failed call that has no handle (tx_create,
 * tx_step_static, tx_batch_create); each host thread keeps its own, and the
 * pointer stays valid until that thread's next such failure. */
const char* tx_last_error(const tx_handle* h);

/* WallsSetValues (src/lbm/lbm_walls.F90:151-177): natural-order wall codes,
 * NX*NY*NZ doubles.  0 = pore, 1..nminerals = mineral, other positive values
 * (e.g. 800, 999) = plain wall.  Ghost walls on non-periodic faces are added
 * by the library (WallsSetGhostNodes, lbm_walls.F90:179-231).  The specular
 * codes 900/901/902 (WALL_NORMAL_X/Y/Z, lbm_definitions.h; 902 is a plain
 * wall in 2D) reflect as DistributionBounceback does
 * (lbm_distribution_function.F90:668-784): their routes are resolved on the
 * host at upload, and wall cells then hold populations, which tx_upload_fi,
 * tx_download, tx_delta_norm and tx_conservation include (species
 * populations too, which stream through the same sweep).  Batches and
 * tx_step_static refuse them (TX_ERR_ARG).  A refused upload leaves the
 * handle's walls unchanged. */
int tx_upload_walls(tx_handle* h, const double* walls);

/* The initialize_state plugin's output (src/lbm/lbm.F90:444-453): rho
 * (s dof) and u (s*ndims dof, the reference flux array) in natural order;
 * u may be NULL for a fluid at rest. */
int tx_upload_state(tx_handle* h, const double* rho, const double* u);

/* -ic_file / restart (src/lbm/lbm.F90:482-544): populations, s*Q dof. */
int tx_upload_fi(tx_handle* h, const double* fi);

/* The initialize_bcs plugin's face arrays (src/lbm/lbm_bc.F90:215-228):
 * vals has nbcs = s*ndims values per face node, the reference's (s, ndims)
 * block with the component fastest (densities in the first s for Dirichlet
 * faces, momenta for Neumann faces, the velocity in entries 0, s, 2s for
 * velocity faces), face nodes in natural order of the two tangential axes.
 * Optional: tx_create fills the faces from bc_data.  Faces without values
 * (periodic, closed, reflecting) return TX_ERR_ARG. */
int tx_upload_bc_values(tx_handle* h, int32_t face, const double* vals);

/* Species concentrations [N*ns] and fluxes [N*ndims*ns] (NULL = 0), natural
 * order with the species fastest: the initial state of the transported
 * species (LBMInitializeState_FlowTransport, src/lbm/lbm.F90:455-480).
 * tx_init then sets gi = geq (TransportFiInit, lbm_transport.F90:320-334). */
int tx_upload_species(tx_handle* h, const double* conc, const double* flux);

/* LBMInit2 for istep = 0 (src/lbm/lbm.F90:183-253): FlowFiInit (unless
 * populations were uploaded) then FlowUpdateMoments; with species,
 * TransportFiInit and TransportUpdateMoments. */
int tx_init(tx_handle* h);

/* nsteps iterations of the flow part of LBMRun2's loop body (lbm.F90:283-363),
 * and of its transport part when the handle has species. */
int tx_step(tx_handle* h, int32_t nsteps);

/* nsteps iterations of the transport part of LBMRun2's loop body alone
 * (TransportCollision, TransportStream and the species bounceback and moments,
 * lbm.F90:290-370): the steady-flow mode of -steadystate_flow, in which the
 * flow calls of the loop are skipped once the ramp-up steps are done
 * (lbm.F90:283-363).  The flow state and its step count stay unchanged.
 * TX_ERR_STATE without species. */
int tx_step_species(tx_handle* h, int32_t nsteps);

/* DistributionCalcDeltaNorm (lbm_distribution_function.F90:809-833):
 * ||(old - new)/new||_inf of TX_FIELD_RHO or TX_FIELD_FI against the values
 * saved by the previous call (first call: against zero).  Sites where new
 * is 0 contribute 0.  FP64 device reduction. */
int tx_delta_norm(tx_handle* h, int32_t field, double* norm);

/* No counterpart in the reference, whose step keeps no conservation totals.
 * Global mass and momentum of the current state, summed over all sites in
 * FP64 on the device from the populations (the precision forms add their rest
 * state back first): out[m] = sum of f(m, n) over sites and directions, and
 * out[s + m*ndims + d] = sum of f(m, n) * c_n[d], for m < s, d < ndims
 * (s + s*ndims doubles).  The order of summation is fixed, so repeated calls
 * on the same state return the same bits.  Non-finite totals return
 * TX_ERR_NONFINITE. */
int tx_conservation(tx_handle* h, double* out);

/* Copy a field to a host array in natural order (see TX_FIELD_*). */
int tx_download(tx_handle* h, int32_t field, double* out);

/* Number of doubles tx_download writes for a field. */
int64_t tx_field_size(const tx_handle* h, int32_t field);

/* Block until all work queued on the handle's stream is done. */
int tx_sync(tx_handle* h);

/* ---- the step for callers that cannot allocate device memory ---- */

/* Size of the library's one static device work area (every GPU that loads the
 * library holds it until the process exits). */
#define TX_STATIC_SCRATCH_BYTES (64ll << 20)

/* No counterpart in the reference.  For callers that are not allowed to call
 * cudaMalloc (hosts that own all device memory in their own arena, plugins
 * handed device buffers by their host): runs nsteps flow steps from fi_in to
 * fi_out without allocating any device memory.  walls (NX*NY*NZ codes),
 * fi_in and fi_out (s*Q dof) are the caller's DEVICE arrays in natural order;
 * fi_in is read only.  The result equals tx_create + tx_upload_walls +
 * tx_upload_fi(fi_in) + tx_init + tx_step(nsteps) + tx_download(TX_FIELD_FI)
 * (the reference's restart path) for the FP64 form.  All working storage comes
 * from one static device array of TX_STATIC_SCRATCH_BYTES; lattices that need
 * more return TX_ERR_ARG.  The first call on a device looks up that array's
 * address, so make it before any stream capture; after a cudaDeviceReset of
 * that device the address is stale, so do not call this on a reset device in
 * the same process.  Calls share the array: calls whose GPU work overlaps
 * race.  Bad wall codes are rejected before any step, with fi_out untouched.
 * The call is synchronous on `stream` (a cudaStream_t; NULL = default
 * stream), also when it fails.  Errors: tx_last_error(NULL). */
int tx_step_static(const tx_params* p, const double* walls, const double* fi_in, double* fi_out, int32_t nsteps,
                   void* stream);


/* ------------------------------------------------------------ batches
 * Many independent lattices of one kernel form, stepped together by
 * persistent tile-table launches that are replayed as a CUDA graph.  There is
 * no counterpart in the reference, which runs one lattice per process; these
 * entry points serve batched permeability runs and the request server.
 * A batch owns one CUDA stream; every call is synchronous with respect to the
 * host unless stated.  Lattice ids are assigned by tx_batch_add and never
 * reused within a batch. */
typedef struct tx_batch tx_batch;

/* Velocity statistics of one lattice from tx_batch_probe, over pore sites:
 * the largest change of any velocity component since the previous probe
 * (the first probe compares with zero), the largest component, the sum of
 * each component, the pore-site count, the steps taken so far, and each
 * component's mass (the sum of its density, as the collision sees it). */
typedef struct {
  int32_t id;
  int32_t pad_;
  double du_max;
  double u_max;
  double u_sum[3];
  int64_t pore_sites;
  int64_t steps;
  double mass[TX_MAX_COMPONENTS];
} tx_probe;

/* form: discretization, ncomponents, relaxation_mode, isotropy_order,
 * precision, nspecies and species_relaxation_mode shared by every lattice of
 * the batch (exact must be 0).
 * hbm_budget_bytes > 0 caps the device memory of all lattices together;
 * tx_batch_add fails with TX_ERR_NOMEM above it. */
int tx_batch_create(const tx_params* form, int64_t hbm_budget_bytes, tx_batch** out);
int tx_batch_destroy(tx_batch* b);
const char* tx_batch_last_error(const tx_batch* b);
/* device bytes one lattice with these parameters occupies in a batch */
int64_t tx_batch_lattice_bytes(const tx_params* p);
int64_t tx_batch_bytes_in_use(const tx_batch* b);
int32_t tx_batch_count(const tx_batch* b);

/* Adds a lattice (walls and initial state as tx_upload_walls + tx_upload_state
 * [+ tx_upload_species(conc, NULL)], then tx_init) and returns its id.  It
 * joins the next step of the batch.  conc is required when the batch form has
 * species and ignored otherwise. */
int tx_batch_add(tx_batch* b, const tx_params* p, const double* walls, const double* rho, const double* u,
                 const double* conc, int32_t* id);
int tx_batch_remove(tx_batch* b, int32_t id);
/* nsteps flow steps of every lattice in the batch */
int tx_batch_step(tx_batch* b, int32_t nsteps);
/* tx_batch_step without waiting: the steps are queued on the batch's stream,
 * so that the work of several batches overlaps on the device; tx_batch_sync
 * waits for them.  The other calls order themselves after queued steps. */
int tx_batch_launch(tx_batch* b, int32_t nsteps);
int tx_batch_sync(tx_batch* b);
/* Probes every lattice; writes up to cap records, *n = lattices probed. */
int tx_batch_probe(tx_batch* b, int32_t cap, tx_probe* out, int32_t* n);
/* a field of one lattice, as tx_download */
int tx_batch_download(tx_batch* b, int32_t id, int32_t field, double* out);
/* tile shape (bx*by*bz must be 128; bz = 1 for D2Q9) and persistent blocks per SM */
int tx_batch_set_tiles(tx_batch* b, int32_t bx, int32_t by, int32_t bz, int32_t blocks_per_sm);
/* Times the candidate tile shapes and grid sizes on the lattices in the batch
 * (steps_per_trial steps each; these are real steps of every lattice) and
 * keeps the fastest; chosen = {bx, by, bz, blocks_per_sm}. */
int tx_batch_tune(tx_batch* b, int32_t steps_per_trial, int32_t* chosen);
/* steps per captured graph (even, >= 2); 0 launches every step directly */
int tx_batch_set_graph(tx_batch* b, int32_t steps_per_graph);
void* tx_batch_stream(tx_batch* b);

/* ---- instrumentation (no counterpart in the reference; used by bench.py) ---- */
/* Per-kernel CUDA-event timing of tx_step on the handle's stream (resets the totals). */
int tx_set_timing(tx_handle* h, int32_t on);

/* Accumulated milliseconds of the collide-push and density launches and the
 * number of kernel launches since tx_set_timing. */
int tx_get_timing(tx_handle* h, double* ms_step, double* ms_density, int64_t* launches);

/* The handle's cudaStream_t (as void*), for callers that order their own work after it. */
void* tx_get_stream(tx_handle* h);

/* Name of the kernel variant selected by tx_create. */
const char* tx_kernel_name(const tx_handle* h);

#ifdef __cplusplus
}
#endif
#endif /* TAXILA_GB300_H */
