/*
 * flint_oracle.h -- FP64 CPU oracle of the per-cell chemistry path.
 *
 * TEST INFRASTRUCTURE ONLY.  This code is the checker for the GPU library and
 * the timed CPU baseline; the product path never links, loads or calls it.
 *
 * Parity pin: the oracle's thermo and rate constants reproduce the reference's
 * own tables (test/WD/INPUT/chemistry-Arrhenius.dat, test/Pelucchi/INPUT/
 * {thermo,chemistry-Troe,chemistry-Lindemann}.dat) to their printed digits;
 * tests/golden/ holds the sampled rows and tests/test_oracle_golden.py checks
 * them.  The reference's integrator (OSlo) is absent from the reference tree,
 * so the reactor part is pinned only against tighter-tolerance runs of itself.
 */
#ifndef FLINT_ORACLE_H
#define FLINT_ORACLE_H

#include <stdint.h>
#include "../include/flint_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* NASA-7 species thermo at T: cp/R, h/(RT), s/R, d(cp/R)/dT. */
void orc_species_thermo(const flint_mech_desc* m, double T, double* cpR, double* hRT,
                        double* sR, double* dcpR);

/* Rate constants at T: kf (high-P for falloff), Kc (concentration units,
 * 0 for irreversible), k0 (falloff), Fcent (Troe; 1 otherwise). */
void orc_rate_constants(const flint_mech_desc* m, double T, double* kf, double* Kc,
                        double* k0, double* fcent);

/* One cell: wdot [kg/m^3/s] and its absolute scale sum_r |nu| (|fwd|+|rev|) W,
 * mixture cp [J/kg/K], h [J/kg].  Any output may be NULL. */
void orc_wdot_cell(const flint_mech_desc* m, double T, double p, const double* Y,
                   double* wdot, double* wscale, double* cp, double* h);

/* One cell: constant-pressure RHS f[ns+1] = (dY/dt, dT/dt). */
void orc_rhs_constp_cell(const flint_mech_desc* m, double T, double p, const double* Y,
                         double* f);

/* One cell: RHS f[ns+1], Jacobian J[(ns+1)^2] column-major
 * (J[col*(ns+1)+row] = d f_row / d x_col, x = (Y, T)) and an absolute scale of
 * every entry (sum of |terms|), for the parity metric.  Jscale may be NULL. */
void orc_jac_cell(const flint_mech_desc* m, double T, double p, const double* Y,
                  double* f, double* J, double* Jscale);

/* Batches over cells with OpenMP (nthreads <= 0: all).  layout = FLINT_*_MAJOR. */
void orc_wdot_batch(const flint_mech_desc* m, int64_t n, int layout, const double* T,
                    const double* p, const double* Y, double* wdot, double* wscale,
                    double* cp, double* h, int nthreads);
void orc_wdot_jac_batch(const flint_mech_desc* m, int64_t n, int layout, const double* T,
                        const double* p, const double* Y, double* wdot, double* jac,
                        double* jscale, int nthreads);

/* Batched constant-pressure reactor advance: the same variable-order
 * fixed-leading-coefficient BDF / Newton algorithm the GPU runs, with a dense
 * partial-pivoting LU.  T, Y (cell-major) updated in place. */
/* Constant-volume RHS and Jacobian (rho fixed; rhs_native's system). */
void orc_rhs_constv_cell(const flint_mech_desc* m, double T, double rho, const double* Y, double* f);
void orc_jac_constv_cell(const flint_mech_desc* m, double T, double rho, const double* Y,
                         double* f, double* J, double* Js);
void orc_jac_constv_batch(const flint_mech_desc* m, int64_t n, const double* T, const double* rho,
                          const double* Y, double* f, double* jac, double* jscale, int nthreads);
void orc_reactor_advance(const flint_mech_desc* m, int64_t n, double* T, const double* p,
                         double* Y, const double* dt, const flint_reactor_opts* o,
                         int* status, int* nsteps, int nthreads);

/* Reference restatement of FLINT's general loop and rhs_native on the tabulated
 * mechanism of include/flint_gpu.h (flint_table_desc). */
typedef flint_table_desc orc_table_mech;

/* general(roi, temp, omegadot), Lib_Chemistry_wdot.f90:96-220. */
void orc_general(const orc_table_mech* m, const double* roi, double temp, double* omegadot);
/* rhs_native(nz, time, Z, F), Lib_Chemistry_rhs.f90:15-52 (constant volume). */
void orc_rhs_native(const orc_table_mech* m, int nz, const double* Z, double* F);
void orc_general_batch(const orc_table_mech* m, int64_t n, const double* roi, const double* T,
                       double* omegadot, int nthreads);
void orc_rhs_native_batch(const orc_table_mech* m, int64_t n, const double* Z, double* F,
                          int nthreads);

/* cons2prim(cons, T), Lib_ThermoTransport.f90:129-165: prim = (rho_s, u_d, p)
 * from cons = (rho_s, rho u_d, rho E0); np = ns + ndim + 1 per cell. */
void orc_cons2prim(const orc_table_mech* m, int np, const double* cons, double T, double* prim,
                   double* Tout, int* iters);
void orc_cons2prim_batch(const orc_table_mech* m, int64_t n, int np, const double* cons,
                         const double* T, double* prim, double* Tout, int nthreads);

/* co_k_mi_lam_Wilke (Lib_ThermoTransport.f90:407-462): Wilke viscosity and
 * conductivity from the tabulated species values; rho = sum(rhoi). */
void orc_transport(const orc_table_mech* m, const double* rhoi, double T, double* mu, double* lam);
void orc_transport_batch(const orc_table_mech* m, int64_t n, const double* rhoi, const double* T, double* mu,
                         double* lam, int nthreads);

int orc_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
