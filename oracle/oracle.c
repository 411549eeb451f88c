/*
 * CPU oracle of the Shan-Chen flow step - TEST INFRASTRUCTURE ONLY.
 *
 * This file restates, routine by routine and loop by loop, the reference's
 * Fortran flow step so that tests can check the CUDA library against it.  It
 * keeps the reference's data layout (fi(m,n,i,j,k) with component fastest and
 * one ghost layer; rho and walls with isotropy-dependent ghost width), its
 * sweep order, its expression shapes (so that IEEE rounding matches) and its
 * single-precision literals.  Only tests/, __graft_entry__.smoke() and the CPU
 * baseline of bench.py use it.  Build: oracle/Makefile (gcc -O2
 * -ffp-contract=off -fopenmp); contraction to FMA must stay off because the
 * reference's goldens were produced without it.
 *
 * Single rank: the reference's PETSc DMDA ghost exchange (DMLocalToLocal)
 * becomes a periodic copy of ghost cells (halo_* below); results of the
 * reference are decomposition-invariant, so one rank reproduces them.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "ff_stencil_oracle.h"

#define MAXQ 19
#define MAXC TX_MAX_COMPONENTS

struct orc {
  tx_params p;
  int nd, N[3], s, b, Q, iso;
  int per[3];
  int gs[3], ge[3], gl[3];   /* fi-ghosted ranges (width 1) */
  int rs[3], re[3], rl[3];   /* rho/walls-ghosted ranges (width stencil_size_rho) */
  int ci[MAXQ][3];
  double w[MAXQ];
  int opp[MAXQ], refl[3][MAXQ];
  double mt[MAXQ][MAXQ];     /* mt[i][k] = mt_mrt(i,k) */
  double mmt[MAXQ];
  double ffw[48];
  double c0;
  double tau_mrt[MAXC][MAXQ];
  double tau[MAXC], cs2[MAXC], dk[MAXC], s_c[MAXC], mm[MAXC];
  int mode;
  int ff_on, fs_on, body_on;
  double fs_w_axis, fs_w_diag;
  double *fi, *tmp, *rho, *walls, *flux, *forces, *fieq;
  double *psi;               /* psi_of_rho (rho layout) when use_nonideal_eos */
  double eos_alpha[MAXC];    /* Peng-Robinson alpha(T) */
  double *bcv[6];            /* nbcs * face area per face with values (Dirichlet, Neumann, velocity) */
  double *old_rho, *old_fi;
  int have_fi, have_state, inited;
  /* passive species: a second distribution over the same lattice, kept as
   * an orc of its own with transport = 1 (LBM_Transport_module) */
  int transport;
  struct orc* tr;
  int have_species;
};

/* ---------------------------------------------------------------- indexing */
static inline long cidx(const orc* o, int i, int j, int k) {
  return (long)(i - o->gs[0]) + (long)o->gl[0] * ((long)(j - o->gs[1]) + (long)o->gl[1] * (long)(k - o->gs[2]));
}
static inline long ridx(const orc* o, int i, int j, int k) {
  return (long)(i - o->rs[0]) + (long)o->rl[0] * ((long)(j - o->rs[1]) + (long)o->rl[1] * (long)(k - o->rs[2]));
}
#define FI(o, m, n, i, j, k) (o)->fi[((cidx(o, i, j, k)) * (o)->Q + (n)) * (o)->s + (m)]
#define TMP(o, m, n, i, j, k) (o)->tmp[((cidx(o, i, j, k)) * (o)->Q + (n)) * (o)->s + (m)]
#define FEQ(o, m, n, i, j, k) (o)->fieq[((cidx(o, i, j, k)) * (o)->Q + (n)) * (o)->s + (m)]
#define RHO(o, m, i, j, k) (o)->rho[(ridx(o, i, j, k)) * (o)->s + (m)]
#define WALL(o, i, j, k) (o)->walls[ridx(o, i, j, k)]
#define FLUX(o, m, d, i, j, k) (o)->flux[((cidx(o, i, j, k)) * (o)->nd + (d)) * (o)->s + (m)]
#define FRC(o, m, d, i, j, k) (o)->forces[((cidx(o, i, j, k)) * (o)->nd + (d)) * (o)->s + (m)]

/* owned-cell loops; k outermost like the reference's do k / do j / do i */
#define OWNED_LOOP(o) \
  for (int k = 1; k <= (o)->N[2]; ++k) \
    for (int j = 1; j <= (o)->N[1]; ++j) \
      for (int i = 1; i <= (o)->N[0]; ++i)

/* ------------------------------------------------------------ lattice setup */
/* DiscretizationSetup_D3Q19 (lbm_discretization_d3q19.F90:64-232) and
 * DiscretizationSetUp_D2Q9 (lbm_discretization_d2q9.F90:53-144). */
static void setup_lattice(orc* o) {
  static const int d3x[19] = {0, 1, 0, -1, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1, 0, 0, 0, 0};
  static const int d3y[19] = {0, 0, 1, 0, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, -1, 1};
  static const int d3z[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};
  static const int d3mt[19][19] = {
      {1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1},
      {-30, -11, -11, -11, -11, -11, -11, 8, 8, 8, 8, 8, 8, 8, 8, 8, 8, 8, 8},
      {12, -4, -4, -4, -4, -4, -4, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1},
      {0, 1, 0, -1, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1, 0, 0, 0, 0},
      {0, -4, 0, 4, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1, 0, 0, 0, 0},
      {0, 0, 1, 0, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, -1, 1},
      {0, 0, -4, 0, 4, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, -1, 1},
      {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1},
      {0, 0, 0, 0, 0, -4, 4, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1},
      {0, 2, -1, 2, -1, -1, -1, 1, 1, 1, 1, 1, 1, 1, 1, -2, -2, -2, -2},
      {0, -4, 2, -4, 2, 2, 2, 1, 1, 1, 1, 1, 1, 1, 1, -2, -2, -2, -2},
      {0, 0, 1, 0, 1, -1, -1, 1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 0, 0},
      {0, 0, -2, 0, -2, 2, 2, 1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 0, 0},
      {0, 0, 0, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 0, 0, 0, 0, 0, 0},
      {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, -1, 1, -1},
      {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 0, 0},
      {0, 0, 0, 0, 0, 0, 0, 1, -1, -1, 1, -1, 1, 1, -1, 0, 0, 0, 0},
      {0, 0, 0, 0, 0, 0, 0, -1, -1, 1, 1, 0, 0, 0, 0, 1, -1, -1, 1},
      {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, -1, -1, -1, -1, 1, 1}};
  static const int d3mmt[19] = {19, 2394, 252, 10, 40, 10, 40, 10, 40, 36, 72, 12, 24, 4, 4, 4, 8, 8, 8};
  static const int d2x[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
  static const int d2y[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
  static const int d2mt[9][9] = {{1, 1, 1, 1, 1, 1, 1, 1, 1},   {-4, -1, -1, -1, -1, 2, 2, 2, 2},
                                 {4, -2, -2, -2, -2, 1, 1, 1, 1}, {0, 1, 0, -1, 0, 1, -1, -1, 1},
                                 {0, -2, 0, 2, 0, 1, -1, -1, 1},  {0, 0, 1, 0, -1, 1, 1, -1, -1},
                                 {0, 0, -2, 0, 2, 1, 1, -1, -1},  {0, 1, -1, 1, -1, 0, 0, 0, 0},
                                 {0, 0, 0, 0, 0, 1, -1, 1, -1}};
  static const int d2mmt[9] = {9, 36, 36, 6, 12, 6, 12, 4, 4};
  memset(o->ffw, 0, sizeof(o->ffw));
  memset(o->ci, 0, sizeof(o->ci));
  if (o->nd == 3) {
    o->b = 18;
    for (int n = 0; n < 19; ++n) {
      o->ci[n][0] = d3x[n]; o->ci[n][1] = d3y[n]; o->ci[n][2] = d3z[n];
      o->w[n] = n == 0 ? 1.0 / 3.0 : (n <= 6 ? 1.0 / 18.0 : 1.0 / 36.0);
      o->mmt[n] = d3mmt[n];
      for (int i = 0; i < 19; ++i) o->mt[i][n] = d3mt[n][i];
    }
    if (o->iso == 4) { o->ffw[1] = 1.0 / 6.0; o->ffw[2] = 1.0 / 12.0; }
    if (o->iso == 8) {
      o->ffw[1] = 4.0 / 45.0; o->ffw[2] = 1.0 / 21.0; o->ffw[3] = 2.0 / 105.0; o->ffw[4] = 5.0 / 504.0;
      o->ffw[5] = 1.0 / 315.0; o->ffw[6] = 1.0 / 630.0; o->ffw[8] = 1.0 / 5040.0;
    }
  } else {
    o->b = 8;
    for (int n = 0; n < 9; ++n) {
      o->ci[n][0] = d2x[n]; o->ci[n][1] = d2y[n];
      o->w[n] = n == 0 ? 4.0 / 9.0 : (n <= 4 ? 1.0 / 9.0 : 1.0 / 36.0);
      o->mmt[n] = d2mmt[n];
      for (int i = 0; i < 9; ++i) o->mt[i][n] = d2mt[n][i];
    }
    if (o->iso == 4) { o->ffw[1] = 1.0 / 3.0; o->ffw[2] = 1.0 / 12.0; }
    if (o->iso == 8) {
      o->ffw[1] = 4.0 / 21.0; o->ffw[2] = 4.0 / 45.0; o->ffw[4] = 1.0 / 60.0; o->ffw[5] = 2.0 / 315.0;
      o->ffw[8] = 1.0 / 5040.0;
    }
    if (o->iso == 10) {
      o->ffw[1] = 262.0 / 1785.0; o->ffw[2] = 93.0 / 1190.0; o->ffw[4] = 7.0 / 340.0; o->ffw[5] = 6.0 / 595.0;
      o->ffw[8] = 9.0 / 9520.0; o->ffw[9] = 2.0 / 5355.0; o->ffw[10] = 1.0 / 7140.0;
    }
  }
  o->Q = o->b + 1;
  o->c0 = 6.0;
  /* opposites / reflect_x,y,z: the direction with the negated (component of) c */
  for (int n = 0; n < o->Q; ++n) {
    for (int m = 0; m < o->Q; ++m) {
      const int* a = o->ci[n]; const int* c = o->ci[m];
      if (c[0] == -a[0] && c[1] == -a[1] && c[2] == -a[2]) o->opp[n] = m;
      if (c[0] == -a[0] && c[1] == a[1] && c[2] == a[2]) o->refl[0][n] = m;
      if (c[0] == a[0] && c[1] == -a[1] && c[2] == a[2]) o->refl[1][n] = m;
      if (c[0] == a[0] && c[1] == a[1] && c[2] == -a[2]) o->refl[2][n] = m;
    }
  }
  /* DiscretizationSetupRelax_D3Q19 (:234-263) / _D2Q9 (:147-166) */
  for (int m = 0; m < o->s; ++m) {
    const tx_params* p = &o->p;
    if (o->nd == 3) {
      const double r[19] = {p->s_c[m], p->s_e[m], p->s_e2[m], p->s_c[m], p->s_q[m], p->s_c[m], p->s_q[m],
                            p->s_c[m], p->s_q[m], p->s_nu[m], p->s_pi[m], p->s_nu[m], p->s_pi[m], p->s_nu[m],
                            p->s_nu[m], p->s_nu[m], p->s_m[m], p->s_m[m], p->s_m[m]};
      memcpy(o->tau_mrt[m], r, sizeof(r));
    } else {
      const double r[9] = {p->s_c[m], p->s_e[m], p->s_e2[m], p->s_c[m], p->s_q[m],
                           p->s_c[m], p->s_q[m], p->s_nu[m], p->s_nu[m]};
      memcpy(o->tau_mrt[m], r, sizeof(r));
    }
  }
}

/* ---------------------------------------------------------------- creation */
static orc* orc_create_transport(const tx_params* p);

/* ------------------------------------------------------------ exterior BCs */
/* bc%flags classes next to flow%bc_flags (FlowParseBC, lbm_flow.F90:1031-1309;
 * include/lbm_definitions.h:30-43) */
enum { CLS_NONE = 0, CLS_REFL = 2, CLS_DIR = 3, CLS_NEU = 4, CLS_VEL = 5 };
static int face_class(const orc* o, int f) {
  if (f >= 2 * o->nd) return CLS_NONE;
  switch (o->p.bc_flags[f]) {
    case TX_BC_REFLECTING: return CLS_REFL;
    case TX_BC_DENSITY: case TX_BC_PRESSURE: case TX_BC_PRESSURE_INLET: case TX_BC_PRESSURE_OUTLET: return CLS_DIR;
    case TX_BC_FLUX: case TX_BC_MOMENTUM: case TX_BC_FLUX_INLET: case TX_BC_FLUX_OUTLET: return CLS_NEU;
    case TX_BC_VELOCITY: return CLS_VEL;
  }
  return CLS_NONE;
}
static int has_values(const orc* o, int f) {
  const int c = face_class(o, f);
  return c == CLS_DIR || c == CLS_NEU || c == CLS_VEL;
}
static long face_area(const orc* o, int f) {
  const int a = f / 2, t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
  return (long)o->N[t1] * (o->nd == 3 ? o->N[t2] : 1);
}

/* FlowUpdateDensityFromPressure (lbm_flow.F90:2235-2263) */
static void density_from_pressure(const orc* o, double pressure, double rho1frac, double* rho) {
  const double eps = 1.e-10;
  if (o->s == 1) {
    rho[0] = pressure * 3.0;
  } else {
    if (rho1frac < eps) {
      rho[0] = 0.0;
      rho[1] = pressure * 3.0;
    } else if (rho1frac > 1 - eps) {
      rho[0] = pressure * 3.0;
      rho[1] = 0.0;
    } else {
      const double alpha = 1.0 / (1.0 / rho1frac - 1.0);
      const double g21 = o->p.g[1][0]; /* components(2)%gf(1) */
      rho[0] = (-((1.0 + alpha) / 3.0) + sqrt((1.0 + alpha) / 3.0 * (1.0 + alpha) / 3.0 + 4. * o->c0 * g21 * alpha * pressure)) /
               (2 * o->c0 * g21);
      rho[1] = rho[0] / alpha;
    }
  }
}

/* FlowSetUpBCsD3/D2 (lbm_flow.F90:1311-1956): node values per face, the same
 * at every node, in the (s, ndims) block xm_vals(m, d) = v[d * s + m] */
static void setup_bc_values(orc* o) {
  const tx_params* p = &o->p;
  const int s = o->s, nd = o->nd, nbcs = s * nd;
  for (int f = 0; f < 2 * nd; ++f) {
    if (!has_values(o, f)) continue;
    const int a = f / 2, plus = f % 2;
    const double* bd = p->bc_data[f];
    double v[3 * MAXC];
    for (int k = 0; k < nbcs; ++k) v[k] = 0.0;
    switch (p->bc_flags[f]) {
      case TX_BC_DENSITY:
        for (int m = 0; m < s; ++m) v[m] = bd[m];
        break;
      case TX_BC_PRESSURE_INLET:
      case TX_BC_PRESSURE: {
        double density[MAXC] = {0.0};
        density_from_pressure(o, bd[0], bd[1], density);
        for (int m = 0; m < s; ++m) v[m] = density[m];
        break;
      }
      case TX_BC_PRESSURE_OUTLET:
        v[0] = bd[0];
        break;
      case TX_BC_MOMENTUM:
        for (int m = 0; m < s; ++m)
          for (int d = 0; d < nd; ++d) v[d * s + m] = bd[m * nd + d];
        break;
      case TX_BC_FLUX_INLET:
      case TX_BC_FLUX:
        if (s == 1) {
          v[a * s] = plus ? -bd[0] : bd[0];
        } else {
          v[a * s] = bd[0] * bd[1];
          v[a * s + 1] = bd[0] * (1.0 - bd[1]);
        }
        break;
      case TX_BC_FLUX_OUTLET:
        v[a * s] = plus ? -bd[0] : bd[0];
        break;
      case TX_BC_VELOCITY:
        for (int d = 0; d < nd; ++d) v[d * s] = bd[d];
        break;
    }
    const long area = face_area(o, f);
    o->bcv[f] = (double*)calloc((size_t)area * nbcs, sizeof(double));
    for (long q = 0; q < area; ++q)
      for (int k = 0; k < nbcs; ++k) o->bcv[f][q * nbcs + k] = v[k];
  }
}

orc* orc_create(const tx_params* p) {
  orc* o = (orc*)calloc(1, sizeof(orc));
  if (!o) return NULL;
  o->p = *p;
  o->nd = p->discretization == TX_D3Q19 ? 3 : 2;
  o->N[0] = p->nx; o->N[1] = p->ny; o->N[2] = o->nd == 3 ? p->nz : 1;
  o->s = p->ncomponents;
  o->iso = p->isotropy_order;
  o->mode = p->relaxation_mode;
  for (int a = 0; a < 3; ++a) o->per[a] = (a < o->nd) && p->bc_flags[2 * a] == TX_BC_PERIODIC;
  /* GridSetFromOptions (lbm_grid.F90:107-120): rho ghost width from isotropy */
  int rw = o->iso == 8 ? 2 : (o->iso == 10 ? 3 : 1);
  for (int a = 0; a < 3; ++a) {
    if (a < o->nd) {
      o->gs[a] = 0; o->ge[a] = o->N[a] + 1;
      o->rs[a] = 1 - rw; o->re[a] = o->N[a] + rw;
    } else {
      o->gs[a] = o->ge[a] = 1; o->rs[a] = o->re[a] = 1;
    }
    o->gl[a] = o->ge[a] - o->gs[a] + 1;
    o->rl[a] = o->re[a] - o->rs[a] + 1;
  }
  setup_lattice(o);
  /* RelaxationCreate / RelaxationSetFromOptions / ComponentSetFromOptions */
  for (int m = 0; m < o->s; ++m) {
    o->tau[m] = p->tau[m];
    o->cs2[m] = 1.0 / 3.0;
    o->mm[m] = p->mm[m];
    o->dk[m] = 1. - 2. / (3. * p->mm[m]);
    o->s_c[m] = o->mode == TX_RELAX_SRT ? 1.0 / p->tau[m] : p->s_c[m];
  }
  /* force switches (lbm_flow.F90:221-239, lbm_walls.F90:115-122) */
  const double eps15 = (double)1.e-15f;
  for (int m = 0; m < o->s; ++m)
    for (int n = 0; n < o->s; ++n)
      if (fabs(p->g[m][n]) > eps15) o->ff_on = 1;
  for (int q = 0; q < p->nminerals; ++q)
    for (int m = 0; m < o->s; ++m)
      if (fabs(p->gw[q][m]) > eps15) o->fs_on = 1;
  o->body_on = p->body_forces != 0;
  /* lbm_forcing.F90:1355,1364 (D3) and :1406,1414 (D2): default-REAL literals */
  if (p->literal_kind == 8) {
    o->fs_w_axis = o->nd == 3 ? 1.0 / 6.0 : 1.0 / 3.0;
    o->fs_w_diag = 1.0 / 12.0;
  } else {
    o->fs_w_axis = o->nd == 3 ? (double)(1.0f / 6.0f) : (double)(1.0f / 3.0f);
    o->fs_w_diag = (double)(1.0f / 12.0f);
  }
  long ncell = (long)o->gl[0] * o->gl[1] * o->gl[2];
  long nrc = (long)o->rl[0] * o->rl[1] * o->rl[2];
  o->fi = (double*)calloc((size_t)ncell * o->Q * o->s, sizeof(double));
  o->tmp = (double*)calloc((size_t)ncell * o->Q * o->s, sizeof(double));
  o->fieq = (double*)calloc((size_t)ncell * o->Q * o->s, sizeof(double));
  o->flux = (double*)calloc((size_t)ncell * o->nd * o->s, sizeof(double));
  o->forces = (double*)calloc((size_t)ncell * o->nd * o->s, sizeof(double));
  o->rho = (double*)calloc((size_t)nrc * o->s, sizeof(double));
  o->walls = (double*)calloc((size_t)nrc, sizeof(double));
  o->psi = (double*)calloc((size_t)nrc * o->s, sizeof(double));
  /* EOSSetFromOptions_PR (lbm_eos.F90:253-300): T_c from a and b with R = 1 */
  for (int m = 0; m < o->s; ++m) {
    if (p->eos[m] != TX_EOS_PR) continue;
    const double a = p->eos_coef[m][0], b = p->eos_coef[m][1], T = p->eos_coef[m][2], om = p->eos_coef[m][3];
    /* single-precision literals in the Fortran source (lbm_eos.F90:296,336) */
    const double Tc = a / b * (double)0.0778f / (double)0.45724f / 1.;
    const double t = 1. + ((double)0.37464f + (double)1.54226f * om - (double)0.26992f * (om * om)) * (1. - sqrt(T / Tc));
    o->eos_alpha[m] = t * t;
  }
  long nown = (long)o->N[0] * o->N[1] * o->N[2];
  o->old_rho = (double*)calloc((size_t)nown * o->s, sizeof(double));
  o->old_fi = (double*)calloc((size_t)nown * o->s * o->Q, sizeof(double));
  setup_bc_values(o);
  if (p->nspecies > 0) o->tr = orc_create_transport(p);
  return o;
}

/* TransportSetFromOptions / TransportSetUp (lbm_transport.F90:130-286) and
 * SpecieSetFromOptions (lbm_species.F90:111-133): nspecies "components" on the
 * flow's lattice with the species' relaxation (RelaxationCreate leaves d_k =
 * 0 for species, lbm_relaxation.F90:80), no forces, and no boundary
 * condition but the periodic faces (TransportApplyBCs is not called by
 * LBMRun2, lbm.F90:348-352). */
static orc* orc_create_transport(const tx_params* p) {
  tx_params q = *p;
  q.ncomponents = p->nspecies;
  q.relaxation_mode = p->species_relaxation_mode;
  q.nspecies = 0;
  q.body_forces = 0;
  for (int m = 0; m < TX_MAX_COMPONENTS; ++m) {
    q.tau[m] = p->species_tau[m];
    q.s_c[m] = p->species_rates[m][0];
    q.s_e[m] = p->species_rates[m][1];
    q.s_e2[m] = p->species_rates[m][2];
    q.s_q[m] = p->species_rates[m][3];
    q.s_nu[m] = p->species_rates[m][4];
    q.s_pi[m] = p->species_rates[m][5];
    q.s_m[m] = p->species_rates[m][6];
    q.mm[m] = 1.0;
    for (int n = 0; n < TX_MAX_COMPONENTS; ++n) q.g[m][n] = 0.0;
  }
  for (int w = 0; w < TX_MAX_MINERALS; ++w)
    for (int m = 0; m < TX_MAX_COMPONENTS; ++m) q.gw[w][m] = 0.0;
  for (int f = 0; f < 6; ++f)
    if (q.bc_flags[f] != TX_BC_PERIODIC) q.bc_flags[f] = TX_BC_NULL;
  orc* t = orc_create(&q);
  if (!t) return NULL;
  t->transport = 1;
  for (int m = 0; m < t->s; ++m) t->dk[m] = 0.0;
  return t;
}

int orc_lattice(const tx_params* p, int* ci, double* w, int* mt, int* mmt, double* ffw, double* rate) {
  orc* o = orc_create(p);
  if (!o) return TX_ERR_ARG;
  for (int n = 0; n < o->Q; ++n) {
    for (int a = 0; a < 3; ++a) ci[n * 3 + a] = o->ci[n][a];
    w[n] = o->w[n];
    mmt[n] = o->mmt[n];
    rate[n] = o->tau_mrt[0][n];
    for (int k = 0; k < o->Q; ++k) mt[n * o->Q + k] = o->mt[n][k];
  }
  for (int i = 0; i < 12; ++i) ffw[i] = o->ffw[i];
  orc_destroy(o);
  return 0;
}

void orc_destroy(orc* o) {
  if (!o) return;
  orc_destroy(o->tr);
  free(o->fi); free(o->tmp); free(o->fieq); free(o->flux); free(o->forces);
  free(o->rho); free(o->walls); free(o->old_rho); free(o->old_fi); free(o->psi);
  for (int f = 0; f < 6; ++f) free(o->bcv[f]);
  free(o);
}

int orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

/* ------------------------------------------------------------ ghost exchange */
/* DMLocalToLocal with a BOX stencil: a ghost point is refreshed from its
 * periodic image when every out-of-range coordinate lies on a periodic axis;
 * ghost points on DM_BOUNDARY_GHOSTED axes keep their values. */
static int wrap(const orc* o, int a, int v, int* out) {
  if (v >= 1 && v <= o->N[a]) { *out = v; return 1; }
  if (!o->per[a]) return 0;
  int n = o->N[a];
  *out = ((v - 1) % n + n) % n + 1;
  return 1;
}

static void halo_fi(orc* o) {
  const int SQ = o->s * o->Q;
  for (int k = o->gs[2]; k <= o->ge[2]; ++k)
    for (int j = o->gs[1]; j <= o->ge[1]; ++j)
      for (int i = o->gs[0]; i <= o->ge[0]; ++i) {
        int owned = i >= 1 && i <= o->N[0] && j >= 1 && j <= o->N[1] && k >= 1 && k <= o->N[2];
        if (owned) continue;
        int si, sj, sk;
        if (!wrap(o, 0, i, &si) || !wrap(o, 1, j, &sj) || !wrap(o, 2, k, &sk)) continue;
        memcpy(&o->fi[cidx(o, i, j, k) * SQ], &o->fi[cidx(o, si, sj, sk) * SQ], sizeof(double) * SQ);
      }
}

static void halo_rho_like(orc* o, double* arr, int dof) {
  for (int k = o->rs[2]; k <= o->re[2]; ++k)
    for (int j = o->rs[1]; j <= o->re[1]; ++j)
      for (int i = o->rs[0]; i <= o->re[0]; ++i) {
        int owned = i >= 1 && i <= o->N[0] && j >= 1 && j <= o->N[1] && k >= 1 && k <= o->N[2];
        if (owned) continue;
        int si, sj, sk;
        if (!wrap(o, 0, i, &si) || !wrap(o, 1, j, &sj) || !wrap(o, 2, k, &sk)) continue;
        memcpy(&arr[ridx(o, i, j, k) * dof], &arr[ridx(o, si, sj, sk) * dof], sizeof(double) * dof);
      }
}
static void halo_rho(orc* o) { halo_rho_like(o, o->rho, o->s); }

/* ------------------------------------------------------------------- walls */
/* WallsSetValues + WallsSetGhostNodesD3/D2 (lbm_walls.F90:151-231) */
int orc_set_walls(orc* o, const double* walls) {
  long q = 0;
  for (int k = o->rs[2]; k <= o->re[2]; ++k)
    for (int j = o->rs[1]; j <= o->re[1]; ++j)
      for (int i = o->rs[0]; i <= o->re[0]; ++i) WALL(o, i, j, k) = 0.0;
  OWNED_LOOP(o) WALL(o, i, j, k) = walls[q++];
  for (int a = 0; a < o->nd; ++a) {
    if (o->per[a]) continue;
    for (int k = o->rs[2]; k <= o->re[2]; ++k)
      for (int j = o->rs[1]; j <= o->re[1]; ++j)
        for (int i = o->rs[0]; i <= o->re[0]; ++i) {
          int v = a == 0 ? i : (a == 1 ? j : k);
          if (v < 1 || v > o->N[a]) WALL(o, i, j, k) = 999.0;
        }
  }
  if (o->tr) orc_set_walls(o->tr, walls);
  return 0;
}

/* ----------------------------------------------------------------- moments */
/* DistributionCalcDensityD3/D2 (lbm_distribution_function.F90:379-428) */
static void calc_density(orc* o) {
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= o->N[2]; ++k)
    for (int j = 1; j <= o->N[1]; ++j)
      for (int i = 1; i <= o->N[0]; ++i) {
        if (WALL(o, i, j, k) == 0) {
          for (int m = 0; m < o->s; ++m) {
            double acc = 0.0;
            for (int n = 0; n < o->Q; ++n) acc = acc + FI(o, m, n, i, j, k);
            RHO(o, m, i, j, k) = acc;
          }
        } else {
          for (int m = 0; m < o->s; ++m) RHO(o, m, i, j, k) = 0.;
        }
      }
}

/* DistributionCalcFluxD3/D2 (lbm_distribution_function.F90:451-508) */
static void calc_flux(orc* o, double* out) {
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= o->N[2]; ++k)
    for (int j = 1; j <= o->N[1]; ++j)
      for (int i = 1; i <= o->N[0]; ++i) {
        long c = cidx(o, i, j, k);
        for (int m = 0; m < o->s; ++m)
          for (int d = 0; d < o->nd; ++d) {
            double acc = 0.0;
            if (WALL(o, i, j, k) == 0)
              for (int n = 0; n < o->Q; ++n) acc = acc + FI(o, m, n, i, j, k) * (double)o->ci[n][d];
            out[(c * o->nd + d) * o->s + m] = WALL(o, i, j, k) == 0 ? acc : 0.;
          }
      }
}

/* FlowUpdateUED3/D2 (lbm_flow.F90:494-574) */
static void update_ue(orc* o) {
  double mmot[MAXC];
  for (int m = 0; m < o->s; ++m) mmot[m] = o->mm[m] * o->s_c[m];
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= o->N[2]; ++k)
    for (int j = 1; j <= o->N[1]; ++j)
      for (int i = 1; i <= o->N[0]; ++i) {
        if (WALL(o, i, j, k) != 0) continue;
        double up[3];
        for (int m = 0; m < o->s; ++m)
          for (int d = 0; d < o->nd; ++d) FLUX(o, m, d, i, j, k) = FLUX(o, m, d, i, j, k) + .5 * FRC(o, m, d, i, j, k);
        for (int d = 0; d < o->nd; ++d) {
          double num = 0.0, den = 0.0;
          for (int m = 0; m < o->s; ++m) num = num + FLUX(o, m, d, i, j, k) * mmot[m];
          for (int m = 0; m < o->s; ++m) den = den + RHO(o, m, i, j, k) * mmot[m];
          up[d] = num / den;
        }
        for (int m = 0; m < o->s; ++m)
          for (int d = 0; d < o->nd; ++d) FLUX(o, m, d, i, j, k) = up[d];
      }
}

/* ------------------------------------------------------------------ forces */
/* LBMAddFluidSolidForcesD3/D2 (lbm_forcing.F90:1326-1421) with the gather of
 * DistributionGatherValueToDirection (lbm_distribution_function.F90:786-807) */
static void add_fluid_solid(orc* o) {
  const int na = 2 * o->nd;
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= o->N[2]; ++k)
    for (int j = 1; j <= o->N[1]; ++j)
      for (int i = 1; i <= o->N[0]; ++i) {
        if (WALL(o, i, j, k) != 0) continue;
        for (int n = 1; n <= o->b; ++n) {
          double v = WALL(o, i + o->ci[n][0], j + o->ci[n][1], k + o->ci[n][2]);
          if (!(v > 0. && v < 998.)) continue;
          int mineral = (int)v;
          const double wgt = n <= na ? o->fs_w_axis : o->fs_w_diag;
          for (int d = 0; d < o->nd; ++d)
            for (int m = 0; m < o->s; ++m) {
              double gw = (mineral >= 1 && mineral <= o->p.nminerals) ? o->p.gw[mineral - 1][m] : 0.0;
              FRC(o, m, d, i, j, k) = FRC(o, m, d, i, j, k) - wgt * RHO(o, m, i, j, k) * gw * (double)o->ci[n][d];
            }
        }
      }
}

/* LBMAddBodyForcesD3/D2 (lbm_forcing.F90:1440-1496) */
static void add_body(orc* o) {
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= o->N[2]; ++k)
    for (int j = 1; j <= o->N[1]; ++j)
      for (int i = 1; i <= o->N[0]; ++i) {
        if (WALL(o, i, j, k) != 0) continue;
        for (int m = 0; m < o->s; ++m)
          for (int d = 0; d < o->nd; ++d)
            FRC(o, m, d, i, j, k) = FRC(o, m, d, i, j, k) + o->p.gvt[d] * o->mm[m] * RHO(o, m, i, j, k);
      }
}

/* LBMAddFluidFluidForcesD3/D2 (lbm_forcing.F90:51-958, :960-1299) */
/* EOSApply_Rho/_SC/_Thermo/_PR (lbm_eos.F90:183-350) with R = 1 */
static double eos_psi(const orc* o, int m, double rho) {
  const int t = o->p.eos[m];
  const double* c = o->p.eos_coef[m];
  if (t == TX_EOS_SC) return c[0] * (1. - exp(-rho / c[0]));
  if (t == TX_EOS_THERMO) return c[0] * exp(-c[1] / rho);
  if (t == TX_EOS_PR) {
    const double a = c[0], b = c[1], T = c[2], alpha = o->eos_alpha[m];
    const double tmp = 2. * (rho * 1. * T / (1. - b * rho) - (a * alpha) * (rho * rho) / (1. + 2. * b * rho - (b * rho) * (b * rho)) -
                             rho / 3.) / (o->c0 * o->p.g[m][m]);
    return sqrt(tmp);
  }
  return rho;
}

/* FlowCalcForces with use_nonideal_eos (lbm_flow.F90:795-805): psi over the
 * whole rho-ghosted box */
static void apply_eos(orc* o) {
  const long nrc = (long)o->rl[0] * o->rl[1] * o->rl[2];
  for (long q = 0; q < nrc; ++q)
    for (int m = 0; m < o->s; ++m) o->psi[q * o->s + m] = eos_psi(o, m, o->rho[q * o->s + m]);
}

static void add_fluid_fluid(orc* o) {
  const double* fld = o->p.use_nonideal_eos ? o->psi : o->rho;
  const double eps = (double)1.e-12f;
  const int ISO = o->iso;
  const int NS = o->s;
  const double* FFW = o->ffw;
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= o->N[2]; ++k)
    for (int j = 1; j <= o->N[1]; ++j)
      for (int i = 1; i <= o->N[0]; ++i) {
        if (WALL(o, i, j, k) != 0) continue;
        double gr[MAXC][3] = {{0}};
        double ws[3] = {0., 0., 0.};
#define O_WALL(dx, dy, dz) (WALL(o, i + (dx), j + (dy), k + (dz)) == 0)
#define O_RHO(m, dx, dy, dz) fld[(ridx(o, i + (dx), j + (dy), k + (dz))) * o->s + (m)]
#define O_GR(m, a) gr[m][a]
        if (o->nd == 3) {
          ORC_FF_GRADIENT_D3(O_WALL, O_RHO, O_GR, ws, FFW, NS);
        } else {
          ORC_FF_GRADIENT_D2(O_WALL, O_RHO, O_GR, ws, FFW, NS);
        }
#undef O_WALL
#undef O_RHO
#undef O_GR
        for (int m = 0; m < o->s; ++m)
          for (int d = 0; d < o->nd; ++d) {
            if (ws[d] > eps) {
              double acc = 0.0;
              for (int q = 0; q < o->s; ++q) acc = acc + o->p.g[m][q] * (gr[q][d] / ws[d]);
              FRC(o, m, d, i, j, k) = FRC(o, m, d, i, j, k) - o->c0 * fld[ridx(o, i, j, k) * o->s + m] * acc;
            }
          }
      }
}

/* FlowCalcForces (lbm_flow.F90:760-808): zero, fluid-solid, body, fluid-fluid */
static void calc_forces(orc* o) {
  long ncell = (long)o->gl[0] * o->gl[1] * o->gl[2];
  memset(o->forces, 0, sizeof(double) * (size_t)ncell * o->nd * o->s);
  if (o->fs_on) add_fluid_solid(o);
  if (o->body_on) add_body(o);
  if (o->ff_on) {
    halo_rho(o);
    if (o->p.use_nonideal_eos) apply_eos(o);
    add_fluid_fluid(o);
  }
}

/* -------------------------------------------------------- equilibrium/collide */
/* DiscretizationEquilf_D3Q19 (lbm_discretization_d3q19.F90:265-305) and
 * DiscretizationEquilf_D2Q9 (lbm_discretization_d2q9.F90:168-205) */
static void update_feq(orc* o) {
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= o->N[2]; ++k)
    for (int j = 1; j <= o->N[1]; ++j)
      for (int i = 1; i <= o->N[0]; ++i) {
        if (WALL(o, i, j, k) != 0) continue;
        for (int m = 0; m < o->s; ++m) {
          const double cs2 = o->cs2[m], dk = o->dk[m];
          const double r = RHO(o, m, i, j, k);
          double usqr = 0.0;
          for (int d = 0; d < o->nd; ++d) usqr = usqr + FLUX(o, m, d, i, j, k) * FLUX(o, m, d, i, j, k);
          if (o->nd == 3)
            FEQ(o, m, 0, i, j, k) = r * (dk - usqr / 2.);
          else
            FEQ(o, m, 0, i, j, k) = r * ((1. + dk * 5.) / 6. - 2. * usqr / 3.);
          for (int n = 1; n <= o->b; ++n) {
            double udote = 0.0;
            for (int d = 0; d < o->nd; ++d) udote = udote + (double)o->ci[n][d] * FLUX(o, m, d, i, j, k);
            FEQ(o, m, n, i, j, k) = o->w[n] * r *
                                    (1.5 * (1. - dk) + udote / cs2 + udote * udote / (2. * cs2 * cs2) -
                                     usqr / (2. * cs2));
          }
        }
      }
}

/* FlowFiBarEqPrefactor (lbm_flow.F90:836-851) */
static inline void prefactor(const orc* o, int i, int j, int k, double P[MAXC][MAXQ]) {
  for (int n = 0; n < o->Q; ++n)
    for (int m = 0; m < o->s; ++m) {
      double acc = 0.0;
      for (int d = 0; d < o->nd; ++d)
        acc = acc + FRC(o, m, d, i, j, k) * ((double)o->ci[n][d] - FLUX(o, m, d, i, j, k));
      P[m][n] = acc / (RHO(o, m, i, j, k) * o->cs2[m]);
    }
}

/* FlowCollisionD3/D2 (lbm_flow.F90:960-1029) with RelaxationCollideSRT/MRT
 * (lbm_relaxation.F90:171-200) */
static void collision(orc* o) {
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= o->N[2]; ++k)
    for (int j = 1; j <= o->N[1]; ++j)
      for (int i = 1; i <= o->N[0]; ++i) {
        if (WALL(o, i, j, k) != 0) continue;
        double P[MAXC][MAXQ], fb[MAXC][MAXQ];
        prefactor(o, i, j, k, P);
        for (int m = 0; m < o->s; ++m)
          for (int n = 0; n < o->Q; ++n) fb[m][n] = (1. - .5 * P[m][n]) * FEQ(o, m, n, i, j, k);
        for (int m = 0; m < o->s; ++m) {
          if (o->mode == TX_RELAX_SRT) {
            for (int n = 0; n < o->Q; ++n)
              FI(o, m, n, i, j, k) = FI(o, m, n, i, j, k) - (FI(o, m, n, i, j, k) - fb[m][n]) / o->tau[m];
          } else {
            double dfi[MAXQ];
            for (int n = 0; n < o->Q; ++n) dfi[n] = FI(o, m, n, i, j, k) - fb[m][n];
            for (int q = 0; q < o->Q; ++q) {
              double mdiff = 0.0;
              for (int n = 0; n < o->Q; ++n) mdiff = mdiff + o->mt[n][q] * dfi[n];
              const double coef = o->tau_mrt[m][q] * mdiff / o->mmt[q];
              for (int n = 0; n < o->Q; ++n) FI(o, m, n, i, j, k) = FI(o, m, n, i, j, k) - coef * o->mt[n][q];
            }
          }
        }
        for (int m = 0; m < o->s; ++m)
          for (int n = 0; n < o->Q; ++n)
            FI(o, m, n, i, j, k) = FI(o, m, n, i, j, k) + P[m][n] * FEQ(o, m, n, i, j, k);
      }
}

/* FlowFeqBarD3/D2 (lbm_flow.F90:867-921): f = (1 - P/2) feq on pore sites */
static void fibar_init(orc* o) {
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= o->N[2]; ++k)
    for (int j = 1; j <= o->N[1]; ++j)
      for (int i = 1; i <= o->N[0]; ++i) {
        if (WALL(o, i, j, k) != 0) continue;
        double P[MAXC][MAXQ];
        prefactor(o, i, j, k, P);
        for (int m = 0; m < o->s; ++m)
          for (int n = 0; n < o->Q; ++n) FI(o, m, n, i, j, k) = (1. - 0.5 * P[m][n]) * FEQ(o, m, n, i, j, k);
      }
}

/* --------------------------------------------------------- stream/bounceback */
static int is_dirichlet(const orc* o, int f) { return face_class(o, f) == CLS_DIR; }

/* BCPreStream_D3/D2 (lbm_bc.F90:613-779): Dirichlet, Neumann and velocity faces */
static void bc_prestream(orc* o) {
  for (int f = 0; f < 2 * o->nd; ++f) {
    if (!has_values(o, f)) continue;
    const int a = f / 2, minus = (f % 2) == 0;
    const int face = minus ? 1 : o->N[a];
    for (int n = 1; n <= o->b; ++n) {
      const int c = o->ci[n][a];
      if (!(minus ? c > 0 : c < 0)) continue;
      for (int k = 1; k <= o->N[2]; ++k)
        for (int j = 1; j <= o->N[1]; ++j)
          for (int i = 1; i <= o->N[0]; ++i) {
            int x[3] = {i, j, k};
            if (x[a] != face) continue;
            for (int m = 0; m < o->s; ++m)
              FI(o, m, n, i - o->ci[n][0], j - o->ci[n][1], k - o->ci[n][2]) = FI(o, m, n, i, j, k);
          }
    }
  }
}

/* DistributionStreamD3/D2 (lbm_distribution_function.F90:545-652): push of
 * every direction over the owned box into tmp (ghost destinations included),
 * then fi = tmp.  tmp starts as NaN: the reference's automatic array is
 * uninitialised, and any read of an unwritten slot must show up. */
static void stream(orc* o) {
  long ntot = (long)o->gl[0] * o->gl[1] * o->gl[2] * o->Q * o->s;
  const double qnan = nan("");
  for (long q = 0; q < ntot; ++q) o->tmp[q] = qnan;
  for (int n = 0; n < o->Q; ++n) {
    int lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
      const int c = o->ci[n][a];
      lo[a] = 1; hi[a] = o->N[a];
      if (c < 0) lo[a] = 1 + c;
      else if (c > 0) hi[a] = o->N[a] + c;
    }
#pragma omp parallel for schedule(static)
    for (int k = lo[2]; k <= hi[2]; ++k)
      for (int j = lo[1]; j <= hi[1]; ++j)
        for (int i = lo[0]; i <= hi[0]; ++i)
          for (int m = 0; m < o->s; ++m)
            TMP(o, m, n, i, j, k) = FI(o, m, n, i - o->ci[n][0], j - o->ci[n][1], k - o->ci[n][2]);
  }
  double* t = o->fi; o->fi = o->tmp; o->tmp = t;
}

/* DistributionBouncebackD3/D2 (lbm_distribution_function.F90:654-784): over
 * the fi-ghosted box in k-j-i order; wall codes 900/901/902 reflect. */
static void bounceback(orc* o) {
  for (int k = o->gs[2]; k <= o->ge[2]; ++k)
    for (int j = o->gs[1]; j <= o->ge[1]; ++j)
      for (int i = o->gs[0]; i <= o->ge[0]; ++i) {
        const double wv = WALL(o, i, j, k);
        int spec = -1;
        if (wv == 900.0) spec = 0;
        else if (wv == 901.0) spec = 1;
        else if (wv == 902.0 && o->nd == 3) spec = 2;
        if (spec < 0 && !(wv > 0)) continue;
        for (int n = 0; n < o->Q; ++n) {
          int ni = i, nj = j, nk = k, nn;
          if (spec >= 0) {
            int x[3] = {i, j, k};
            x[spec] -= o->ci[n][spec];
            if (!(x[spec] >= 1 && x[spec] <= o->N[spec])) continue;
            ni = x[0]; nj = x[1]; nk = x[2];
            nn = o->refl[spec][n];
          } else {
            ni = i - o->ci[n][0]; nj = j - o->ci[n][1]; nk = k - o->ci[n][2];
            if (!(ni >= 1 && ni <= o->N[0] && nj >= 1 && nj <= o->N[1] && nk >= 1 && nk <= o->N[2])) continue;
            nn = o->opp[n];
          }
          for (int m = 0; m < o->s; ++m) FI(o, m, nn, ni, nj, nk) = FI(o, m, n, i, j, k);
        }
        for (int n = 0; n < o->Q; ++n)
          for (int m = 0; m < o->s; ++m) FI(o, m, n, i, j, k) = 0.0;
      }
}

/* ------------------------------------------------------------ Dirichlet BCs */
static long face_node(const orc* o, int f, int i, int j, int k) {
  const int a = f / 2;
  int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
  int x[3] = {i, j, k};
  if (o->nd == 2) return (long)(x[t1] - 1);
  return (long)(x[t1] - 1) + (long)o->N[t1] * (long)(x[t2] - 1);
}

/* BCApplyDirichletToRho_D3/D2 (lbm_bc.F90:252-434) */
static void bc_dirichlet_to_rho(orc* o) {
  const int nbcs = o->s * o->nd;
  for (int f = 0; f < 2 * o->nd; ++f) {
    if (!is_dirichlet(o, f)) continue;
    const int a = f / 2, face = (f % 2) == 0 ? 1 : o->N[a];
    OWNED_LOOP(o) {
      int x[3] = {i, j, k};
      if (x[a] != face || WALL(o, i, j, k) != 0) continue;
      for (int m = 0; m < o->s; ++m) RHO(o, m, i, j, k) = o->bcv[f][face_node(o, f, i, j, k) * nbcs + m];
    }
  }
}

/* BCApplyDirichletNode (lbm_bc.F90:1273-1333) with the local frames of
 * DiscSetLocalDirections (lbm_discretization_d3q19.F90:566-714, d2q9:372-434):
 * normal axis a with inward sign sg; tangential axes in CARDINAL order. */
static void dirichlet_node(orc* o, int f, int i, int j, int k, const double* pv) {
  const int a = f / 2;
  const int sg = (f % 2) == 0 ? 1 : -1;
  int tang[2], nt = 0;
  if (o->nd == 3) {
    if (a == 0) { tang[0] = 1; tang[1] = 2; }
    else if (a == 1) { tang[0] = 2; tang[1] = 0; }
    else { tang[0] = 0; tang[1] = 1; }
    nt = 2;
  } else {
    tang[0] = a == 0 ? 1 : 0;
    nt = 1;
  }
  for (int m = 0; m < o->s; ++m) {
    double ws[3] = {0.0, 0.0, 0.0}, Q[3] = {0.0, 0.0, 0.0}, mom[3] = {0.0, 0.0, 0.0};
    for (int n = 1; n <= o->b; ++n)
      if (sg * o->ci[n][a] == 1) ws[a] = ws[a] + o->w[n];
    double sum = 0.0;
    for (int n = 0; n < o->Q; ++n) sum = sum + FI(o, m, n, i, j, k);
    Q[a] = (double)sg * (pv[m] - sum) / ws[a];
    for (int p = 0; p < nt; ++p) {
      const int t = tang[p];
      for (int n = 1; n <= o->b; ++n) {
        mom[t] = mom[t] + FI(o, m, n, i, j, k) * (double)o->ci[n][t];
        if (sg * o->ci[n][a] == 1 && o->ci[n][t] != 0) ws[t] = ws[t] + o->w[n];
      }
      Q[t] = -(mom[t] / ws[t]);
    }
    for (int n = 1; n <= o->b; ++n) {
      if (sg * o->ci[n][a] != 1) continue;
      double cq = 0.0;
      for (int d = 0; d < o->nd; ++d) cq = cq + (double)o->ci[n][d] * Q[d];
      FI(o, m, n, i, j, k) = FI(o, m, n, i, j, k) + o->w[n] * cq;
    }
  }
}

/* BCApplyNeumannNode (lbm_bc.F90:1533-1593): mv = the node's (s, ndims) block */
static void neumann_node(orc* o, int f, int i, int j, int k, const double* mv) {
  const int a = f / 2;
  const int sg = (f % 2) == 0 ? 1 : -1;
  for (int m = 0; m < o->s; ++m) {
    double ws[3] = {0.0, 0.0, 0.0}, mom[3] = {0.0, 0.0, 0.0}, Q[3] = {0.0, 0.0, 0.0};
    for (int p = 0; p < o->nd; ++p) {
      for (int n = 1; n <= o->b; ++n) {
        mom[p] = mom[p] + FI(o, m, n, i, j, k) * (double)o->ci[n][p];
        if (sg * o->ci[n][a] == 1 && o->ci[n][p] != 0) ws[p] = ws[p] + o->w[n];
      }
      Q[p] = (mv[p * o->s + m] - FRC(o, m, p, i, j, k) / 2.0 - mom[p]) / ws[p];
    }
    for (int n = 1; n <= o->b; ++n) {
      if (sg * o->ci[n][a] != 1) continue;
      double cq = 0.0;
      for (int d = 0; d < o->nd; ++d) cq = cq + (double)o->ci[n][d] * Q[d];
      FI(o, m, n, i, j, k) = FI(o, m, n, i, j, k) + o->w[n] * cq;
    }
  }
}

/* BCApplyVelocityNode (lbm_bc.F90:1793-1865): uvals(1, :) = uv[d * s] */
static void velocity_node(orc* o, int f, int i, int j, int k, const double* uv) {
  const int a = f / 2;
  const int sg = (f % 2) == 0 ? 1 : -1;
  int tang[2], nt = 0;
  if (o->nd == 3) {
    if (a == 0) { tang[0] = 1; tang[1] = 2; }
    else if (a == 1) { tang[0] = 2; tang[1] = 0; }
    else { tang[0] = 0; tang[1] = 1; }
    nt = 2;
  } else {
    tang[0] = a == 0 ? 1 : 0;
    nt = 1;
  }
  for (int m = 0; m < o->s; ++m) {
    double ws[3] = {0.0, 0.0, 0.0}, mom[3] = {0.0, 0.0, 0.0}, Q[3] = {0.0, 0.0, 0.0};
    for (int n = 1; n <= o->b; ++n) {
      mom[a] = mom[a] + FI(o, m, n, i, j, k) * (double)o->ci[n][a];
      if (sg * o->ci[n][a] == 1) ws[a] = ws[a] + o->w[n];
    }
    double sum = 0.0;
    for (int n = 0; n < o->Q; ++n) sum = sum + FI(o, m, n, i, j, k);
    Q[a] = (sum * uv[a * o->s] - mom[a] - FRC(o, m, a, i, j, k) / 2.0) / (1.0 - (double)sg * uv[a * o->s]) / ws[a];
    const double rho = sum + ws[a] * Q[a] * (double)sg;
    for (int p = 0; p < nt; ++p) {
      const int t = tang[p];
      for (int n = 1; n <= o->b; ++n) {
        mom[t] = mom[t] + FI(o, m, n, i, j, k) * (double)o->ci[n][t];
        if (sg * o->ci[n][a] == 1 && o->ci[n][t] != 0) ws[t] = ws[t] + o->w[n];
      }
      Q[t] = (rho * uv[t * o->s] - FRC(o, m, t, i, j, k) / 2.0 - mom[t]) / ws[t];
    }
    for (int n = 1; n <= o->b; ++n) {
      if (sg * o->ci[n][a] != 1) continue;
      double cq = 0.0;
      for (int d = 0; d < o->nd; ++d) cq = cq + (double)o->ci[n][d] * Q[d];
      FI(o, m, n, i, j, k) = FI(o, m, n, i, j, k) + o->w[n] * cq;
    }
  }
}

/* BCApplyReflectingD3/D2 (lbm_bc.F90:825-1073) at one node, as written: on
 * the XM face in 3D the normal component of n is compared with the z
 * component of p (:851).  (The 2D XM face compares with ci(p, Z), past the
 * D2Q9 table; the library rejects that face.) */
static void reflect_node(orc* o, int f, int i, int j, int k) {
  const int a = f / 2;
  const int sg = (f % 2) == 0 ? 1 : -1;
  const int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
  const int b3 = (o->nd == 3 && f == 0) ? 2 : a;
  for (int n = 1; n <= o->b; ++n) {
    if (!(sg * o->ci[n][a] > 0)) continue;
    for (int q = 1; q <= o->b; ++q) {
      if (o->ci[n][t1] != o->ci[q][t1]) continue;
      if (o->nd == 3 && o->ci[n][t2] != o->ci[q][t2]) continue;
      if (o->ci[n][a] != -o->ci[q][b3]) continue;
      for (int m = 0; m < o->s; ++m) FI(o, m, n, i, j, k) = FI(o, m, q, i, j, k);
    }
  }
}

/* BCApplyReflecting / BCApplyDirichlet / BCApplyNeumann / BCApplyVelocity
 * D3/D2 (lbm_bc.F90:809-1865) for one class: its faces in XM..ZP order, pore
 * nodes of each face */
static void apply_class(orc* o, int cls) {
  const int nbcs = o->s * o->nd;
  for (int f = 0; f < 2 * o->nd; ++f) {
    if (face_class(o, f) != cls) continue;
    const int a = f / 2, face = (f % 2) == 0 ? 1 : o->N[a];
    OWNED_LOOP(o) {
      int x[3] = {i, j, k};
      if (x[a] != face || WALL(o, i, j, k) != 0) continue;
      if (cls == CLS_REFL) {
        reflect_node(o, f, i, j, k);
        continue;
      }
      const double* v = &o->bcv[f][face_node(o, f, i, j, k) * nbcs];
      if (cls == CLS_DIR) dirichlet_node(o, f, i, j, k, v);
      else if (cls == CLS_NEU) neumann_node(o, f, i, j, k, v);
      else velocity_node(o, f, i, j, k, v);
    }
  }
}

/* BCApply (lbm_bc.F90:781-807): each class once, in order of first appearance
 * over the six sides (periodic and closed sides apply nothing) */
static void bc_apply(orc* o) {
  int done[8] = {0};
  for (int side = 0; side < 6; ++side) {
    const int cls = face_class(o, side);
    if (cls == CLS_NONE || done[cls]) continue;
    apply_class(o, cls);
    done[cls] = 1;
  }
}

/* BCUpdateRho_D3/D2 (lbm_bc.F90:436-611): Dirichlet, Neumann and velocity faces */
static void bc_update_rho(orc* o) {
  for (int f = 0; f < 2 * o->nd; ++f) {
    if (!has_values(o, f)) continue;
    const int a = f / 2, face = (f % 2) == 0 ? 1 : o->N[a];
    OWNED_LOOP(o) {
      int x[3] = {i, j, k};
      if (x[a] != face || WALL(o, i, j, k) != 0) continue;
      for (int m = 0; m < o->s; ++m) {
        double acc = 0.0;
        for (int n = 0; n < o->Q; ++n) acc = acc + FI(o, m, n, i, j, k);
        RHO(o, m, i, j, k) = acc;
      }
    }
  }
}

/* FlowUpdateBCPressureOutletD3/D2 (lbm_flow.F90:2020-2233), two components:
 * the mass fraction of the neighbour inside (of the node when that neighbour
 * is a wall) at the start of FlowApplyBCs */
static void update_pressure_outlets(orc* o) {
  const int nbcs = o->s * o->nd;
  for (int f = 0; f < 2 * o->nd; ++f) {
    if (o->p.bc_flags[f] != TX_BC_PRESSURE_OUTLET) continue;
    const int a = f / 2, minus = (f % 2) == 0;
    const int face = minus ? 1 : o->N[a];
    OWNED_LOOP(o) {
      int x[3] = {i, j, k};
      if (x[a] != face || WALL(o, i, j, k) != 0) continue;
      int q[3] = {i, j, k};
      q[a] += minus ? 1 : -1;
      if (WALL(o, q[0], q[1], q[2]) != 0) { q[0] = i; q[1] = j; q[2] = k; }
      double tot = 0.0;
      for (int m = 0; m < o->s; ++m) tot = tot + RHO(o, m, q[0], q[1], q[2]);
      const double rho1frac = RHO(o, 0, q[0], q[1], q[2]) / tot;
      density_from_pressure(o, o->p.bc_data[f][0], rho1frac, &o->bcv[f][face_node(o, f, i, j, k) * nbcs]);
    }
  }
}

/* ------------------------------------------------------------- transport */
/* TransportCollisionD3 (lbm_transport.F90:403-431) collides pore cells
 * (walls == 0); TransportCollisionD2 (:433-458) collides cells with walls > 0,
 * which the reference does as written: in 2D the species are only streamed
 * and bounced back.  RelaxationCollideSRT/MRT (lbm_relaxation.F90:171-200)
 * toward fi_eq, no forcing. */
static void transport_collision(orc* o) {
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= o->N[2]; ++k)
    for (int j = 1; j <= o->N[1]; ++j)
      for (int i = 1; i <= o->N[0]; ++i) {
        const int on = o->nd == 3 ? WALL(o, i, j, k) == 0 : WALL(o, i, j, k) > 0;
        if (!on) continue;
        for (int m = 0; m < o->s; ++m) {
          if (o->mode == TX_RELAX_SRT) {
            for (int n = 0; n < o->Q; ++n)
              FI(o, m, n, i, j, k) = FI(o, m, n, i, j, k) - (FI(o, m, n, i, j, k) - FEQ(o, m, n, i, j, k)) / o->tau[m];
          } else {
            double dfi[MAXQ];
            for (int n = 0; n < o->Q; ++n) dfi[n] = FI(o, m, n, i, j, k) - FEQ(o, m, n, i, j, k);
            for (int q = 0; q < o->Q; ++q) {
              double mdiff = 0.0;
              for (int n = 0; n < o->Q; ++n) mdiff = mdiff + o->mt[n][q] * dfi[n];
              const double coef = o->tau_mrt[m][q] * mdiff / o->mmt[q];
              for (int n = 0; n < o->Q; ++n) FI(o, m, n, i, j, k) = FI(o, m, n, i, j, k) - coef * o->mt[n][q];
            }
          }
        }
      }
}

/* TransportFiInit (lbm_transport.F90:320-334): fi_eq from the initial
 * concentration and flux, fi = fi_eq over the whole local array, then
 * TransportUpdateMoments (:312-318). */
static void transport_init(orc* t) {
  halo_rho_like(t, t->walls, 1);
  update_feq(t);
  long ntot = (long)t->gl[0] * t->gl[1] * t->gl[2] * t->Q * t->s;
  memcpy(t->fi, t->fieq, sizeof(double) * (size_t)ntot);
  calc_density(t);
  calc_flux(t, t->flux);
  t->inited = 1;
}

/* The transport part of LBMRun2's loop body (lbm.F90:290-370): collision with
 * the equilibrium of the species' own density and flux (TransportUpdateFeq,
 * lbm_transport.F90:363-378, passes the flux array as the velocity), halo,
 * stream, bounceback (TransportReactWithWalls without a reactive matrix),
 * moments. */
static void transport_step(orc* t) {
  update_feq(t);
  transport_collision(t);
  halo_fi(t);
  stream(t);
  bounceback(t);
  calc_density(t);
  calc_flux(t, t->flux);
}

int orc_set_species(orc* o, const double* conc, const double* flux) {
  if (!o->tr) return TX_ERR_STATE;
  orc_set_state(o->tr, conc, flux);
  o->have_species = 1;
  return 0;
}

/* ------------------------------------------------------------ step drivers */
/* FlowUpdateMoments (lbm_flow.F90:466-478) */
static void update_moments(orc* o) {
  calc_density(o);
  calc_flux(o, o->flux);
  calc_forces(o);
  update_ue(o);
}

int orc_set_state(orc* o, const double* rho, const double* u) {
  long q = 0;
  OWNED_LOOP(o) {
    for (int m = 0; m < o->s; ++m) RHO(o, m, i, j, k) = rho[q * o->s + m];
    for (int d = 0; d < o->nd; ++d)
      for (int m = 0; m < o->s; ++m) FLUX(o, m, d, i, j, k) = u ? u[(q * o->nd + d) * o->s + m] : 0.0;
    ++q;
  }
  o->have_state = 1;
  o->have_fi = 0;
  return 0;
}

int orc_set_fi(orc* o, const double* fi) {
  long q = 0;
  OWNED_LOOP(o) {
    for (int n = 0; n < o->Q; ++n)
      for (int m = 0; m < o->s; ++m) FI(o, m, n, i, j, k) = fi[(q * o->Q + n) * o->s + m];
    ++q;
  }
  o->have_fi = 1;
  return 0;
}

int orc_set_bc_values(orc* o, int face, const double* vals) {
  int f = face - 1;
  if (f < 0 || f >= 2 * o->nd || !o->bcv[f]) return TX_ERR_ARG;
  const int a = f / 2;
  int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
  long area = (long)o->N[t1] * (o->nd == 3 ? o->N[t2] : 1);
  memcpy(o->bcv[f], vals, sizeof(double) * (size_t)area * o->s * o->nd);
  return 0;
}

/* LBMInit2 with istep = 0 (lbm.F90:183-253) */
int orc_init(orc* o) {
  halo_rho_like(o, o->walls, 1); /* WallsCommunicate */
  if (!o->have_fi) {
    /* FlowFiInit (lbm_flow.F90:923-934) */
    calc_forces(o);
    update_feq(o);
    fibar_init(o);
  }
  update_moments(o);
  if (o->tr && o->have_species) transport_init(o->tr);
  o->inited = 1;
  return 0;
}

/* One iteration of LBMRun2's loop for the flow (lbm.F90:283-363) */
static void one_step(orc* o) {
  update_feq(o);          /* FlowCollision: FlowUpdateFeq */
  collision(o);           /*                FlowCollisionD3/D2 */
  halo_fi(o);             /* DistributionCommunicateFi */
  bc_prestream(o);        /* FlowStream: BCPreStream */
  stream(o);              /*             DistributionStream */
  bounceback(o);          /* FlowBounceback */
  /* FlowApplyBCs (lbm_flow.F90:1958-1991): two-component pressure outlets first;
   * the flux-outlet update acts on pressure-outlet faces only (:2282-2497)
   * and the library rejects the two outlets together */
  if (o->s != 1)
    for (int f = 0; f < 2 * o->nd; ++f)
      if (o->p.bc_flags[f] == TX_BC_PRESSURE_OUTLET) {
        update_pressure_outlets(o);
        break;
      }
  calc_density(o);        /*              -> FlowCalcRhoForces */
  bc_dirichlet_to_rho(o);
  calc_forces(o);
  bc_apply(o);            /*              -> BCApply */
  bc_update_rho(o);       /*              -> BCUpdateRho */
  calc_flux(o, o->flux);  /* FlowUpdateFlux */
  update_ue(o);
}

int orc_step(orc* o, int nsteps) {
  if (!o->inited) return TX_ERR_STATE;
  const int species = o->tr && o->have_species;
  for (int t = 0; t < nsteps; ++t) {
    one_step(o);
    if (species) transport_step(o->tr);
  }
  return 0;
}

/* ---------------------------------------------------------------- outputs */
long orc_field_size(const orc* o, int field) {
  long n = (long)o->N[0] * o->N[1] * o->N[2];
  switch (field) {
    case TX_FIELD_FI: return n * o->s * o->Q;
    case TX_FIELD_RHO: return n * o->s;
    case TX_FIELD_FLUX:
    case TX_FIELD_FORCES: return n * o->s * o->nd;
    case TX_FIELD_PRS:
    case TX_FIELD_RHOT:
    case TX_FIELD_WALLS: return n;
    case TX_FIELD_VELT: return n * o->nd;
    case TX_FIELD_SPECIES_FI: return o->tr ? n * o->tr->s * o->Q : -1;
    case TX_FIELD_SPECIES_RHO: return o->tr ? n * o->tr->s : -1;
    case TX_FIELD_SPECIES_FLUX: return o->tr ? n * o->tr->s * o->nd : -1;
    case TX_FIELD_PSI: return n * o->s;
  }
  return -1;
}

/* FlowUpdateDiagnosticsD3/D2 (lbm_flow.F90:654-758) for psi = rho */
static void diagnostics(orc* o, double* rhot, double* prs, double* velt) {
  long ncell = (long)o->gl[0] * o->gl[1] * o->gl[2];
  double* u = (double*)calloc((size_t)ncell * o->nd * o->s, sizeof(double));
  calc_flux(o, u);
  long q = 0;
  OWNED_LOOP(o) {
    long c = cidx(o, i, j, k);
    if (WALL(o, i, j, k) == 0) {
      double rt = 0.0;
      for (int m = 0; m < o->s; ++m) rt = rt + RHO(o, m, i, j, k) * o->mm[m];
      double pr = rt / 3.;
      if (o->s > 1 || o->p.use_nonideal_eos) {
        double ps[MAXC];
        for (int m = 0; m < o->s; ++m)
          ps[m] = o->p.use_nonideal_eos ? eos_psi(o, m, RHO(o, m, i, j, k)) : RHO(o, m, i, j, k);
        for (int m = 0; m < o->s; ++m) {
          double acc = 0.0;
          for (int n = 0; n < o->s; ++n) acc = acc + o->p.g[m][n] * ps[n];
          pr = pr + o->c0 / 2. * ps[m] * acc;
        }
      }
      for (int m = 0; m < o->s; ++m)
        for (int d = 0; d < o->nd; ++d)
          u[(c * o->nd + d) * o->s + m] = u[(c * o->nd + d) * o->s + m] + .5 * FRC(o, m, d, i, j, k);
      if (rhot) rhot[q] = rt;
      if (prs) prs[q] = pr;
      for (int d = 0; d < o->nd; ++d) {
        double acc = 0.0;
        for (int m = 0; m < o->s; ++m) acc = acc + u[(c * o->nd + d) * o->s + m] * o->mm[m];
        if (velt) velt[q * o->nd + d] = acc / rt;
      }
    } else {
      if (rhot) rhot[q] = 0.0;
      if (prs) prs[q] = 0.0;
      for (int d = 0; d < o->nd; ++d)
        if (velt) velt[q * o->nd + d] = 0.0;
    }
    ++q;
  }
  free(u);
}

int orc_get(orc* o, int field, double* out) {
  long q = 0;
  switch (field) {
    case TX_FIELD_FI:
      OWNED_LOOP(o) {
        for (int n = 0; n < o->Q; ++n)
          for (int m = 0; m < o->s; ++m) out[(q * o->Q + n) * o->s + m] = FI(o, m, n, i, j, k);
        ++q;
      }
      return 0;
    case TX_FIELD_RHO:
      OWNED_LOOP(o) {
        for (int m = 0; m < o->s; ++m) out[q * o->s + m] = RHO(o, m, i, j, k);
        ++q;
      }
      return 0;
    case TX_FIELD_FLUX:
    case TX_FIELD_FORCES:
      OWNED_LOOP(o) {
        for (int d = 0; d < o->nd; ++d)
          for (int m = 0; m < o->s; ++m)
            out[(q * o->nd + d) * o->s + m] = field == TX_FIELD_FLUX ? FLUX(o, m, d, i, j, k) : FRC(o, m, d, i, j, k);
        ++q;
      }
      return 0;
    case TX_FIELD_WALLS:
      OWNED_LOOP(o) out[q++] = WALL(o, i, j, k);
      return 0;
    case TX_FIELD_PRS: diagnostics(o, NULL, out, NULL); return 0;
    case TX_FIELD_RHOT: diagnostics(o, out, NULL, NULL); return 0;
    case TX_FIELD_VELT: diagnostics(o, NULL, NULL, out); return 0;
    case TX_FIELD_PSI:
      OWNED_LOOP(o) {
        for (int m = 0; m < o->s; ++m)
          out[q * o->s + m] = WALL(o, i, j, k) == 0 ? (o->p.use_nonideal_eos ? eos_psi(o, m, RHO(o, m, i, j, k))
                                                                              : RHO(o, m, i, j, k)) : 0.0;
        ++q;
      }
      return 0;
    case TX_FIELD_SPECIES_FI: return o->tr ? orc_get(o->tr, TX_FIELD_FI, out) : TX_ERR_ARG;
    case TX_FIELD_SPECIES_RHO: return o->tr ? orc_get(o->tr, TX_FIELD_RHO, out) : TX_ERR_ARG;
    case TX_FIELD_SPECIES_FLUX: return o->tr ? orc_get(o->tr, TX_FIELD_FLUX, out) : TX_ERR_ARG;
  }
  return TX_ERR_ARG;
}

/* DistributionCalcDeltaNorm (lbm_distribution_function.F90:809-833); sites
 * whose new value is 0 contribute 0 (pointwise divide by zero guarded). */
double orc_delta_norm(orc* o, int field) {
  long n = orc_field_size(o, field);
  double* cur = (double*)malloc(sizeof(double) * (size_t)n);
  orc_get(o, field, cur);
  double* old = field == TX_FIELD_FI ? o->old_fi : o->old_rho;
  double norm = 0.0;
  for (long q = 0; q < n; ++q) {
    double v = cur[q] != 0.0 ? (old[q] - cur[q]) / cur[q] : 0.0;
    v = fabs(v);
    if (v > norm) norm = v;
    old[q] = cur[q];
  }
  free(cur);
  return norm;
}
