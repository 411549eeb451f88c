/*
 * CPU oracle for the Shan-Chen flow step - TEST INFRASTRUCTURE ONLY.
 *
 * A line-for-line restatement of the reference's Fortran step, used by the
 * tests, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the
 * checker.  It is never linked into or called by the product library.
 * Arrays follow the reference's ghosted Fortran layout; the interface takes
 * and returns natural-order global vectors like the C ABI.
 */
#ifndef TAXILA_ORACLE_H
#define TAXILA_ORACLE_H
#include "../include/taxila_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc orc;

orc* orc_create(const tx_params* p);
void orc_destroy(orc* o);
int orc_set_walls(orc* o, const double* walls);
int orc_set_state(orc* o, const double* rho, const double* u);
int orc_set_fi(orc* o, const double* fi);
int orc_set_bc_values(orc* o, int face, const double* vals);
int orc_init(orc* o);
int orc_step(orc* o, int nsteps);
double orc_delta_norm(orc* o, int field);
int orc_get(orc* o, int field, double* out);
/* The lattice tables of an oracle built from p, for the tests that pin them
 * to the reference source: ci[Q*3], w[Q], mt[Q*Q] (M^T(i,k) at i*Q+k),
 * mmt[Q], ffw[12] (isotropy weights by |e|^2) and the MRT rate of every
 * moment of component 0, rate[Q] (tau_mrt). */
int orc_lattice(const tx_params* p, int* ci, double* w, int* mt, int* mmt, double* ffw, double* rate);
long orc_field_size(const orc* o, int field);
int orc_set_threads(int n);
int orc_set_species(orc* o, const double* conc, const double* flux);

#ifdef __cplusplus
}
#endif
#endif
