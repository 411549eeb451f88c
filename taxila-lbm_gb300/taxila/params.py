"""ctypes mirror of ``tx_params`` (include/taxila_gb300.h) and its defaults."""
import ctypes as C

MAXC = 4
MAXMIN = 16

D3Q19 = 1
D2Q9 = 2
SRT = 0
MRT = 1
BC_NULL = 0
BC_PERIODIC = 1
BC_REFLECTING = 2
BC_VELOCITY = 5
BC_DENSITY = 6
BC_MOMENTUM = 7
BC_PRESSURE = 8
BC_PRESSURE_INLET = 9
BC_PRESSURE_OUTLET = 10
BC_FLUX = 11
BC_FLUX_INLET = 12
BC_FLUX_OUTLET = 13
XM, XP, YM, YP, ZM, ZP = 1, 2, 3, 4, 5, 6
FACE_NAMES = ("xm", "xp", "ym", "yp", "zm", "zp")
PREC_F64, PREC_F32, PREC_F32_F16 = 0, 1, 2

FIELD_FI, FIELD_RHO, FIELD_FLUX, FIELD_FORCES = 1, 2, 3, 4
FIELD_PRS, FIELD_VELT, FIELD_RHOT, FIELD_WALLS = 5, 6, 7, 8
FIELD_SPECIES_FI, FIELD_SPECIES_RHO, FIELD_SPECIES_FLUX = 9, 10, 11
FIELD_PSI = 12
EOS_RHO, EOS_SC, EOS_THERMO, EOS_PR = 0, 1, 2, 3

ERR_NAMES = {0: "TX_OK", 1: "TX_ERR_ARG", 2: "TX_ERR_STATE", 3: "TX_ERR_CUDA",
             4: "TX_ERR_NOMEM", 5: "TX_ERR_NONFINITE", 6: "TX_ERR_NODEVICE"}

_D = C.c_double
_I = C.c_int32


class TxParams(C.Structure):
    _fields_ = [
        ("discretization", _I), ("nx", _I), ("ny", _I), ("nz", _I),
        ("ncomponents", _I), ("nminerals", _I), ("relaxation_mode", _I),
        ("isotropy_order", _I), ("bc_flags", _I * 6),
        ("tau", _D * MAXC), ("s_c", _D * MAXC), ("s_e", _D * MAXC), ("s_e2", _D * MAXC),
        ("s_q", _D * MAXC), ("s_nu", _D * MAXC), ("s_pi", _D * MAXC), ("s_m", _D * MAXC),
        ("mm", _D * MAXC), ("g", (_D * MAXC) * MAXC), ("gw", (_D * MAXC) * MAXMIN),
        ("body_forces", _I), ("gvt", _D * 3),
        ("bc_data", (_D * (3 * MAXC)) * 6),
        ("literal_kind", _I), ("precision", _I), ("exact", _I), ("rho0", _D * MAXC), ("storage_scale", _D),
        ("use_nonideal_eos", _I), ("eos", _I * MAXC), ("eos_coef", (_D * 4) * MAXC),
        ("nspecies", _I), ("species_relaxation_mode", _I), ("species_tau", _D * MAXC),
        ("species_rates", (_D * 7) * MAXC),
    ]

    @property
    def ndims(self):
        return 3 if self.discretization == D3Q19 else 2

    @property
    def Q(self):
        return 19 if self.discretization == D3Q19 else 9

    @property
    def shape(self):
        """Lattice shape in natural (x fastest) order as (nz, ny, nx)."""
        return (self.nz if self.ndims == 3 else 1, self.ny, self.nx)

    @property
    def nsites(self):
        z, y, x = self.shape
        return x * y * z


def default_params():
    """Reference defaults (lbm_options.F90:105-148, lbm_relaxation.F90:65-84,
    lbm_component.F90:99-111)."""
    p = TxParams()
    p.discretization = D3Q19
    p.nx = p.ny = p.nz = 1
    p.ncomponents = 1
    p.nminerals = 1
    p.relaxation_mode = SRT
    p.isotropy_order = 4
    for f in range(6):
        p.bc_flags[f] = BC_NULL
    for m in range(MAXC):
        p.tau[m] = 1.0
        p.s_c[m] = p.s_e[m] = p.s_e2[m] = p.s_q[m] = 1.0
        p.s_nu[m] = p.s_pi[m] = p.s_m[m] = 1.0
        p.mm[m] = 1.0
    p.body_forces = 0
    p.literal_kind = 4
    p.precision = PREC_F64
    p.exact = 0
    for m in range(MAXC):
        p.rho0[m] = 0.0
    p.storage_scale = 1.0
    p.nspecies = 0
    p.species_relaxation_mode = SRT
    for m in range(MAXC):
        p.species_tau[m] = 1.0
        for k in range(7):
            p.species_rates[m][k] = 1.0
    return p


def copy_params(p):
    q = TxParams()
    C.memmove(C.addressof(q), C.addressof(p), C.sizeof(TxParams))
    return q
