/*
 * fcs_oracle.h -- CPU restatement of the FastChemistrySolver per-cell stiff
 * chemistry path, used ONLY as a checker (tests, smoke, bench cpu_baseline).
 * It is never linked into or called by the product library.
 *
 * Every function restates the reference algorithm and cites the reference
 * file:line it follows.  The restatement is validated against the reference
 * itself compiled from its own sources (oracle/Makefile -> oracle/_ref/) and
 * against the golden fixtures in tests/golden/.
 */
#ifndef FCS_ORACLE_H
#define FCS_ORACLE_H
#include <stdint.h>
#include "../include/fcs.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_mech orc_mech;

typedef struct orc_options {
    int32_t solver;          /* FCS_SOLVER_* */
    int32_t jacobian;        /* FCS_JACOBIAN_* */
    int32_t conversion_as_written; /* 1: O(N^3) dC/dY conversion exactly as
                                      Jacobian.C:2814-2858 writes it; 0: the
                                      algebraically identical O(N^2) form */
    int32_t max_steps;
    double abs_tol, rel_tol;
    double T_react;
    double delta_t_chem_max;
    int32_t n_threads;
} orc_options;

/* Counters summed over cells: attempts, accepted, jacobians, lu, rhs, solves,
 * integrated cells, failed cells. */
enum { ORC_ATTEMPTS = 0, ORC_ACCEPTED, ORC_JAC, ORC_LU, ORC_RHS, ORC_SOLVES,
       ORC_CELLS, ORC_FAILED, ORC_NCOUNTERS };

orc_mech* orc_mech_create(const fcs_mechanism_desc* desc, int32_t* status);
void orc_mech_destroy(orc_mech* m);
int32_t orc_mech_n_species(const orc_mech* m);
/* reference-order reaction index -> file-order index */
int32_t orc_mech_order(const orc_mech* m, int32_t* file_index_out);

void orc_default_options(orc_options* o);

int32_t orc_integrate(const orc_mech* m, const orc_options* o, int64_t n_cells,
                      double delta_t, const double* delta_t_per_cell,
                      const double* p, const double* rho0, double* T, double* Y,
                      double* sub_dt, double* RR, int32_t* cell_status,
                      double* delta_t_min, int64_t* counters);

/* f = [dY/dt, dT/dt] per cell (species-major [(Ns+1)*n]) */
int32_t orc_rhs(const orc_mech* m, int64_t n_cells, const double* p, const double* T,
                const double* Y, double* dydt);
/* J per cell [n][(Ns+1)^2] and f */
int32_t orc_jacobian(const orc_mech* m, const orc_options* o, int64_t n_cells,
                     const double* p, const double* T, const double* Y,
                     double* J, double* dydt);
/* calculate(): RR [Ns*n] and Qdot [n] from (p, T, rho, Y) */
int32_t orc_rates(const orc_mech* m, int64_t n_cells, const double* p, const double* T, const double* rho,
                  const double* Y, double* RR, double* Qdot);
/* FastChemistryModel::tc (chemical time scale) per cell from (p, T, rho, Y) */
int32_t orc_tc(const orc_mech* m, int64_t n_cells, const double* p, const double* T, const double* rho,
               const double* Y, double* tc);
/* Dense LU with the reference's 4-row-panel pivoting on one n x n row-major
 * matrix; solves nrhs right-hand sides in place (b is [nrhs][n]). */
int32_t orc_lu_solve(int32_t n, double* a, int32_t nrhs, double* b, int32_t* piv,
                     double* invD);

#ifdef __cplusplus
}
#endif
#endif
