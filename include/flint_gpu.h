/*
 * flint_gpu.h -- C-ABI of the GB300 (sm_103a) per-cell chemistry library.
 *
 * This is the drop-in boundary below FLINT's Fortran API.  Every entry point is
 * plain C: opaque handles, plain pointers, 64-bit sizes, an explicit CUDA
 * stream passed as `void*` (NULL = legacy default stream), and an `int` status
 * (FLINT_OK = 0).  No C++ exception and no torch type crosses it.  The Fortran
 * interface block a FLINT caller binds is include/flint_gpu.f90.
 *
 * Reference interfaces replaced (paths within the FLINT project):
 *   read_idealgas_thermo(folder)          src/lib/Load_ThermoTransport.f90:7
 *   read_chemistry(folder, mech_name)     src/lib/Load_Chemistry.f90:7
 *   Assign_Mechanism(name)                src/lib/Lib_Chemistry_wdot.f90:24
 *   chemistry_source(roi, temp, omegadot) src/lib/Lib_Chemistry_wdot.f90:6-20
 *   general(roi, temp, omegadot)          src/lib/Lib_Chemistry_wdot.f90:96-220
 *   f_cp / H (mixture cp and h)           src/lib/Lib_ThermoTransport.f90:251-271, :40-52
 *   rhs_native(nz, time, Z, F)            src/lib/Lib_Chemistry_rhs.f90:15-52
 *   setup_odesolver / run_odesolver       OSlo, call sites src/test/Fortran/test-batchF.f90:81,105
 *   free_chemistry_data()                 src/lib/Lib_Chemistry_data.f90:168
 *   cons2prim(cons, T)                    src/lib/Lib_ThermoTransport.f90:129-165
 *   co_k_mi_lam_Wilke(rhoi, rho, T, ...)  src/lib/Lib_ThermoTransport.f90:407-462
 *
 * Threads: a handle (mechanism or surrogate) serves one thread at a time;
 * different handles may be used concurrently.  The allocation-free reactor
 * entry's static scratch is shared by every handle of a device.
 *
 * Device-pointer entry points take device (or managed) memory and are
 * asynchronous on `stream`; the *_host variants take host memory, stage it
 * through device buffers owned by the handle and return after the results are
 * back on the host.
 *
 * Units: SI with kmol.  T [K], p [Pa], Y mass fractions, rho_i [kg/m^3],
 * wdot [kg/m^3/s], cp [J/kg/K], h [J/kg].
 */
#ifndef FLINT_GPU_H
#define FLINT_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
enum {
  FLINT_OK = 0,
  FLINT_ERR_ARG = 1,        /* bad argument (NULL pointer, size, layout)       */
  FLINT_ERR_CUDA = 2,       /* a CUDA runtime call failed                       */
  FLINT_ERR_MECH = 3,       /* mechanism outside what the kernels support       */
  FLINT_ERR_IO = 4,         /* input file missing or malformed                  */
  FLINT_ERR_NOMEM = 5       /* device allocation failed                         */
};

/* Per-cell status written by the reactor (one int per cell). */
enum {
  FLINT_CELL_OK = 0,
  FLINT_CELL_T_OUT_OF_RANGE = 1,  /* T outside the mechanism's valid range     */
  FLINT_CELL_NAN_INPUT = 2,       /* NaN/Inf or non-positive p in the input    */
  FLINT_CELL_MAX_STEPS = 3,       /* internal step limit reached               */
  FLINT_CELL_NEWTON_FAIL = 4,     /* repeated Newton convergence failures      */
  FLINT_CELL_ERRTEST_FAIL = 5,    /* repeated local error test failures        */
  FLINT_CELL_SURROGATE_REJECTED = 6 /* surrogate rejected; cell re-solved      */
};

/* Layout of per-species arrays (Y, rho_i, wdot) of N cells. */
enum {
  FLINT_CELL_MAJOR = 0,     /* Fortran (ns, N): a[cell*ns + k]                   */
  FLINT_SPECIES_MAJOR = 1   /* structure of arrays (N, ns): a[k*N + cell]        */
};

/* Reaction forms (the reference's rxn_type plus the three-body flag). */
enum {
  FLINT_RXN_ELEMENTARY = 0,
  FLINT_RXN_THREEBODY = 1,
  FLINT_RXN_LINDEMANN = 2,
  FLINT_RXN_TROE = 3
};

#define FLINT_MAXSP_PER_SIDE 3

typedef struct flint_mech_s* flint_mech_t;
/* FLINT input files parsed on the host (flint_tables_read). */
typedef struct flint_table_set_s* flint_table_set_t;
/* A parsed mechanism IR blob (flint_ir_parse). */
typedef struct flint_ir_s* flint_ir_t;

/* Analytic mechanism description: NASA-7 (or NASA-9) thermo + Arrhenius / third-body /
 * falloff kinetics with reverse rates from Kc (Gibbs).  All arrays are host
 * memory, row-major, read once by flint_mech_create. */
typedef struct {
  int ns;                 /* species                                        */
  int nr;                 /* reactions                                      */
  const double* mw;       /* [ns] molar mass, kg/kmol                       */
  const double* nasa7;    /* [ns][17]: Tlow, Tmid, Thigh, a_low[7], a_high[7] */
  const int* rtype;       /* [nr] FLINT_RXN_*                               */
  const int* reversible;  /* [nr] 1 = reverse rate from Kc, 0 = irreversible */
  const double* arrh;     /* [nr][3] A (SI kmol), b, Ea/R [K]; high-P limit for falloff */
  const double* arrh0;    /* [nr][3] low-pressure limit (falloff only)       */
  const double* troe;     /* [nr][4] a, T3, T1, T2 (T2 = 0: term absent)     */
  const int* rsp;         /* [nr][3] reactant species (-1 = unused slot)     */
  const double* rnu;      /* [nr][3] reactant stoichiometric coefficients    */
  const double* rord;     /* [nr][3] forward orders (= rnu unless custom)    */
  const int* psp;         /* [nr][3] product species (-1 = unused slot)      */
  const double* pnu;      /* [nr][3] product stoichiometric coefficients     */
  const double* eff;      /* [nr][ns] third-body efficiencies (types 1-3)    */
  double r_eos;           /* gas constant of the EOS and energy equation (FLINT Runiv 8314.51) */
  double r_thermo;        /* gas constant of the polynomials -> cp,h,s and Kc (8314.46261815324) */
  double p_ref;           /* standard pressure of Kc, Pa (101325)            */
  /* optional NASA-9 thermo (NULL: nasa7 serves): [ns][32] = nranges (1-3),
   * T0..T3 (range i is [T_i, T_i+1]; unused +inf), 3 x (a1..a7, b1, b2);
   * when given it replaces nasa7 for every species (NASA-7 data enter it as
   * a1 = a2 = 0) */
  const double* nasa9;
} flint_mech_desc;

/* Tabulated mechanism: FLINT's own module arrays as read_idealgas_thermo and
 * read_chemistry leave them (Lib_ThermoTransport.f90:10-23,
 * Lib_Chemistry_data.f90:4-32), in their Fortran layout, 1-K rows.  A FLINT
 * caller passes c_loc() of its arrays; flint_gb300.tables reads the same files
 * in Python.  Rows run tmin..tmax (thermo) and ti1..ti2 (rates). */
typedef struct {
  int ns;
  int nr_arrh, nr_troe, nr_lind;
  int tmin, tmax;              /* thermo rows tmin..tmax                       */
  int ti1, ti2;                /* rate-table rows ti1..ti2                     */
  const double* wm;            /* [ns] molar mass                              */
  const double* cp_tab;        /* cp_tab(tmin:tmax, ns)  J/kg/K                */
  const double* h_tab;         /* h_tab(tmin:tmax, ns)   J/kg                  */
  const double* kf_tab;        /* kf_tab(ti1:ti2, nr_arrh)                     */
  const double* kb_tab;        /* kb_tab(ti1:ti2, nr_arrh)                     */
  const double* kinf_troe;     /* (ti1:ti2, nr_troe), likewise k0, kc, Fcent    */
  const double* k0_troe;
  const double* kc_troe;
  const double* fcent_troe;
  const double* kinf_lind;     /* (ti1:ti2, nr_lind), likewise k0, kc           */
  const double* k0_lind;
  const double* kc_lind;
  const double* ni1_arrh;      /* ni1_arrh_tab(ns+1, nr_arrh); row ns+1 = "M"   */
  const double* ni2_arrh;
  const double* eps_arrh;
  const double* ni1_troe;      /* (ns+1, nr_troe)                               */
  const double* ni2_troe;
  const double* eps_troe;
  const double* ni1_lind;      /* (ns+1, nr_lind)                               */
  const double* ni2_lind;
  const double* eps_lind;
  double runiv;                /* Runiv of the EOS terms (8314.51)             */
  /* optional transport tables as read_idealgas_transport leaves them
   * (Load_ThermoTransport.f90:129-174), rows tmin..tmax like cp_tab; NULL when
   * the caller has none (flint_transport_batch then refuses)                  */
  const double* mi_tab;        /* mi_tab(tmin:tmax, ns)  laminar viscosity, Pa s */
  const double* k_tab;         /* k_tab(tmin:tmax, ns)   conductivity, W/m/K    */
} flint_table_desc;

/* Integrator options of the batched 0D reactor. */
typedef struct {
  double rtol;            /* relative tolerance (all components)            */
  double atol;            /* absolute tolerance (all components)            */
  int max_steps;          /* internal step limit per cell (bounded loop)    */
  int max_order;          /* BDF order limit, 1..5                           */
  int constant_volume;    /* 0: constant pressure (default); 1: constant volume,
                             the density fixed at p/(R T sum Y/W) of the input
                             state and the energy equation of rhs_native
                             (Lib_Chemistry_rhs.f90:43-50); p is not updated */
  int reserved;
  double tmin, tmax;      /* valid temperature range; outside -> T_OUT_OF_RANGE */
} flint_reactor_opts;

/* ------------------------------------------------------------ life cycle */
/* Replaces read_idealgas_thermo + read_chemistry + Assign_Mechanism for an
 * analytic mechanism: copies the description to device memory owned by *out. */
int flint_mech_create(const flint_mech_desc* desc, flint_mech_t* out);
/* Replaces read_idealgas_thermo + read_chemistry + Assign_Mechanism for the
 * reference's tabulated data (the `general` path, Lib_Chemistry_wdot.f90:96-220):
 * copies the tables to device memory owned by *out.  Handles made this way
 * serve flint_chemistry_source_batch and flint_rhs_native_batch. */
int flint_mech_create_tables(const flint_table_desc* desc, flint_mech_t* out);
/* Replaces read_idealgas_thermo, read_idealgas_transport and read_chemistry
 * (Load_ThermoTransport.f90:7-95, :129-174, Load_Chemistry.f90:7-164) for
 * callers without FLINT's Fortran loaders: parses <folder>/<prefix>phase.txt,
 * thermo, chemistry-info.txt, chemistry-Arrhenius and, when the mechanism has
 * such reactions, chemistry-Troe / chemistry-Lindemann, plus transport.dat
 * when present (1-K rows; a thermo table starting at 1 K gains the cloned row
 * 0 with h = 0, as the reference builds it).  Each table is read as Tecplot
 * ASCII POINT zones (.dat) or, when that file is absent, as SZL binary
 * (.szplt, ordered zones of float32 or float64 values), the loaders' own
 * fallback (Load_Chemistry.f90:95-96, Load_ThermoTransport.f90:57-60).
 * Host only, no GPU needed.  A missing or malformed
 * file returns FLINT_ERR_IO with the reason in flint_last_error(), where the
 * reference prints [ERROR] and returns or stops.  prefix may be NULL. */
int flint_tables_read(const char* folder, const char* prefix, flint_table_set_t* out);
/* Fill *desc with pointers into the set (valid until flint_tables_free). */
int flint_tables_desc(flint_table_set_t set, flint_table_desc* desc);
/* Name of species k (0-based) as phase.txt gives it. */
const char* flint_tables_species_name(flint_table_set_t set, int k);
int flint_tables_free(flint_table_set_t set);
/* flint_tables_read + flint_mech_create_tables + flint_tables_free. */
int flint_mech_create_from_files(const char* folder, const char* prefix, flint_mech_t* out);

/* Mechanism IR blob: flint_mech_desc serialized as one byte string, the
 * form a caller stores or sends an analytic mechanism in (flint_gb300.mech
 * writes it: Mechanism.to_ir()).  Little-endian, packed, no padding:
 *   header (48 bytes): "FLIR", uint32 version = 1, int32 ns, int32 nr,
 *     uint32 flags (bit 0: NASA-9 section present), uint32 0,
 *     double r_eos, r_thermo, p_ref;
 *   then, in this order: double mw[ns], nasa7[ns][17]; int32 rtype[nr],
 *     reversible[nr]; double arrh[nr][3], arrh0[nr][3], troe[nr][4];
 *     int32 rsp[nr][3]; double rnu[nr][3], rord[nr][3]; int32 psp[nr][3];
 *     double pnu[nr][3], eff[nr][ns]; [double nasa9[ns][32] if flags bit 0].
 * The meaning of each array is that of the flint_mech_desc field of the same
 * name.  The blob's length must equal flint_ir_bytes(ns, nr, nasa9); a bad
 * magic, version, count, flag or length returns FLINT_ERR_ARG before any
 * array is read.  Host only, no GPU needed. */
int flint_ir_parse(const void* blob, int64_t bytes, flint_ir_t* out);
/* Fill *desc with pointers into the parsed IR (valid until flint_ir_free). */
int flint_ir_desc(flint_ir_t ir, flint_mech_desc* desc);
int flint_ir_free(flint_ir_t ir);
/* Exact blob length for ns species, nr reactions (nasa9: 0 or 1); -1 if invalid. */
int64_t flint_ir_bytes(int ns, int nr, int nasa9);
/* flint_ir_parse + flint_mech_create + flint_ir_free. */
int flint_mech_create_from_ir(const void* blob, int64_t bytes, flint_mech_t* out);
/* Replaces free_chemistry_data (Lib_Chemistry_data.f90:168). */
int flint_mech_destroy(flint_mech_t mech);
/* Text of the last error on the calling thread ("" if none). */
const char* flint_last_error(void);
/* Library version string. */
const char* flint_version(void);
/* Species / reaction counts of a handle. */
int flint_mech_sizes(flint_mech_t mech, int* ns, int* nr);

/* -------------------------------------------------------------- thermo */
/* Mixture cp [J/kg/K] and h [J/kg] for N cells (NASA-7 / NASA-9, f_cp / H of
 * Lib_ThermoTransport.f90:251-271, :40-52).  Either output may be NULL. */
int flint_thermo_batch(flint_mech_t mech, int64_t n, int layout, const double* T,
                       const double* Y, double* cp, double* h, void* stream);
/* Species cp [J/kg/K], h [J/kg], s at p_ref [J/kg/K] and g = h - T s [J/kg]
 * for N temperatures (cpi, H0i, S0i of Lib_ThermoTransport.f90:40-97,
 * :233-248, from the NASA-7 / NASA-9 polynomials), cell-major (N, ns) outputs;
 * any output may be NULL.  Analytic handles. */
int flint_species_thermo_batch(flint_mech_t mech, int64_t n, const double* T, double* cp,
                               double* h, double* s, double* g, void* stream);

/* ----------------------------------------------------------- source term */
/* Net mass production rates wdot [kg/m^3/s] of N cells at (T, p, Y), plus the
 * mixture cp and h (either may be NULL).  Replaces the per-cell
 * chemistry_source loop of a CFD caller (Lib_Chemistry_wdot.f90:6-20). */
int flint_wdot_batch(flint_mech_t mech, int64_t n, int layout, const double* T,
                     const double* p, const double* Y, double* wdot, double* cp,
                     double* h, void* stream);

/* chemistry_source(roi, temp, omegadot) over N cells, cell-major rho_i input
 * (Fortran (ns, N)).  Analytic handles clamp negative rho_i to zero in place, as
 * the reference mechanisms do (WD.f90:19, Lib_Chemistry_rhs.f90:37-39);
 * tabulated handles run the general loop on roi as given, as `general` does.
 * For a tabulated handle, temperatures outside the rate table use its edge
 * rows (the reference reads past the table there). */
int flint_chemistry_source_batch(flint_mech_t mech, int64_t n, double* roi,
                                 const double* T, double* omegadot, void* stream);

/* rhs_native(nz, time, Z, F) over N cells (Lib_Chemistry_rhs.f90:15-52):
 * Z, F cell-major (ns+1) per cell, Z = (rho_1..rho_ns, T); constant-volume
 * energy equation from the tabulated h and cp; F = -1 for a cell whose T is
 * outside the thermo table or NaN, as the reference returns.  Tabulated handles. */
int flint_rhs_native_batch(flint_mech_t mech, int64_t n, const double* Z, double* F, void* stream);

/* Mixture laminar viscosity and conductivity by Wilke's rule over N cells:
 * co_k_mi_lam_Wilke(rhoi, rho, T, milam, klam) (Lib_ThermoTransport.f90:407-462)
 * with rho = sum(rhoi); rhoi cell-major (ns, N), T, mu, lambda (N).  Species
 * values from the handle's mi_tab / k_tab.  Tabulated handles with transport. */
int flint_transport_batch(flint_mech_t mech, int64_t n, const double* rhoi, const double* T, double* mu,
                          double* lambda, void* stream);

/* cons2prim(cons, T) over N cells (Lib_ThermoTransport.f90:129-165):
 * cons, prim cell-major, np = ns + ndim + 1 per cell; cons = (rho_1..rho_ns,
 * rho u_1..rho u_ndim, rho E0), prim = (rho_1..rho_ns, u_1..u_ndim, p).  T is
 * the Newton start per cell (the caller's previous temperature, as in the
 * reference); T_out (may be NULL) gets the last iterate.  The reference's
 * iteration: at most 20 Newton steps on the static energy from the tabulated
 * h and cp, stopping at a relative energy change below 1e-6.  Tabulated handles. */
int flint_cons2prim_batch(flint_mech_t mech, int64_t n, int ndim, const double* cons, const double* T,
                          double* prim, double* T_out, void* stream);

/* wdot and the analytic Jacobian of the constant-pressure reactor right-hand
 * side, J = d(dY/dt, dT/dt)/d(Y, T), (ns+1)^2 per cell stored column-major
 * per cell: jac[cell*(ns+1)^2 + col*(ns+1) + row] (Fortran (ns+1, ns+1, N)). */
int flint_wdot_jac_batch(flint_mech_t mech, int64_t n, int layout, const double* T,
                         const double* p, const double* Y, double* wdot, double* jac,
                         void* stream);

/* Constant-volume forms of the two calls below and above (the system of
 * rhs_native, Lib_Chemistry_rhs.f90:15-52, from the analytic mechanism):
 * rho [kg/m^3] per cell replaces p, dT/dt = -sum_k u_k wdot_k / (rho cv), and
 * J = d(dY/dt, dT/dt)/d(Y, T) at fixed rho (same storage as
 * flint_wdot_jac_batch). */
int flint_wdot_jac_constv_batch(flint_mech_t mech, int64_t n, int layout, const double* T,
                                const double* rho, const double* Y, double* wdot, double* jac,
                                void* stream);
int flint_rhs_constv_batch(flint_mech_t mech, int64_t n, const double* T, const double* rho,
                           const double* Y, double* f, void* stream);

/* Constant-pressure reactor right-hand side f = (dY/dt, dT/dt), cell-major
 * (ns+1) per cell. */
int flint_rhs_constp_batch(flint_mech_t mech, int64_t n, const double* T, const double* p,
                           const double* Y, double* f, void* stream);

/* ---------------------------------------------------------------- reactor */
/* Advance N independent 0D reactors over their own dt (setup_odesolver +
 * run_odesolver of OSlo as called at test-batchF.f90:81,105) with a batched
 * variable-order BDF / Newton integrator and dense LU of the (ns+1) system.
 * T and Y (cell-major) are updated in place; status[cell] gets FLINT_CELL_*,
 * nsteps[cell] the internal steps taken (either may be NULL).  Constant
 * pressure by default; opts->constant_volume = 1 integrates at the cell's
 * initial density, as run_odesolver does with rhs_native. */
int flint_reactor_advance(flint_mech_t mech, int64_t n, double* T, const double* p,
                          double* Y, const double* dt, const flint_reactor_opts* opts,
                          int* status, int* nsteps, void* stream);

/* Empirical choice of the reactor's layout for this mechanism: the Newton
 * matrix and Jacobian work area in shared memory (blocks of 8 warps), or in
 * each warp's global slot with blocks of 8 or of 4 warps (shared memory left to
 * the L1 cache that holds the slots).  Times flint_reactor_advance under each
 * possible layout on a sample of cells (n of them, device arrays; the caller's
 * arrays are not modified), keeps the fastest for later calls on this handle,
 * and reports it in *layout (1 shared, 2 global / 8 warps, 3 global / 4 warps,
 * 4 global / two blocks of 8 warps per SM from a build capped at 128 registers).
 * No reference counterpart. */
int flint_reactor_autotune(flint_mech_t mech, int64_t n, const double* T, const double* p, const double* Y,
                           const double* dt, const flint_reactor_opts* opts, int* layout, void* stream);
/* The layouts the last flint_reactor_autotune on this handle timed and their
 * times [ms] (at most cap of them; *count = how many were timed).  No
 * reference counterpart. */
int flint_reactor_autotune_times(flint_mech_t mech, int* layouts, float* ms, int cap, int* count);
/* The tuning a handle runs with: the reactor layout (0 = by size, 1-4 as
 * flint_reactor_autotune reports them) and the threads per block of the
 * warp-per-cell source-term kernels, for wdot (flint_wdot_batch) and for
 * wdot + Jacobian (flint_wdot_jac_batch): 64, 128 or 256, 0 = 256.  No
 * reference counterpart. */
typedef struct {
  int reactor_layout;
  int wdot_threads;
  int jac_threads;
  int reserved;
} flint_tuning;
int flint_tuning_get(flint_mech_t mech, flint_tuning* tuning);
/* Apply a tuning chosen earlier (a tuning cache) without timing; a layout or
 * block size that does not fit this mechanism on the current device is
 * refused (FLINT_ERR_ARG) and nothing changes. */
int flint_tuning_set(flint_mech_t mech, const flint_tuning* tuning);
/* Empirical choice of the source-term kernels' block size: times
 * flint_wdot_batch and flint_wdot_jac_batch at every block size on a sample
 * of cells (n of them, device arrays, cell-major; outputs go to private
 * buffers), keeps the fastest for this handle and reports the handle's tuning
 * in *tuning (may be NULL).  No reference counterpart. */
int flint_wdot_autotune(flint_mech_t mech, int64_t n, const double* T, const double* p, const double* Y,
                        flint_tuning* tuning, void* stream);

/* flint_reactor_advance without any device allocation.  No counterpart in the
 * reference.  For callers that must not have a library call cudaMalloc: CFD
 * codes that hand their whole device memory to their own pool at start-up and
 * codes whose rules forbid allocation after initialisation.  The scratch (work
 * counters and one saved Jacobian per resident warp) is a static device array
 * of 1280 slots of 32 x 32 doubles plus 256 bytes of counters (10 MiB + 256 B),
 * which every GPU that loads the library holds until exit.  Mechanisms of up to
 * 31 species fit; larger ones are rejected with FLINT_ERR_MECH.
 * Warm-up: a call with n = 0 (the arrays may then be NULL) advances nothing
 * and does the one-time set-up on the current device: under CUDA's default
 * lazy module loading the array gets its device memory only then (or on the
 * first real call); the call also looks the array's address up
 * (cudaGetSymbolAddress), uploads the BDF table and sets the kernel's
 * shared-memory attribute.  Make that call, with the device current, before
 * the caller's pool reserves its device memory and before any stream capture
 * (CUDA_MODULE_LOADING=EAGER instead makes the array resident when the library
 * loads).  The kernel always runs the shared-memory layout, the only one whose
 * per-warp scratch fits a slot; a layout chosen by flint_reactor_autotune
 * applies to flint_reactor_advance only.  Every call shares the one array and
 * zeroes its counters: calls that overlap on the GPU (two streams, two
 * threads) race and must be serialised by the caller.  flint_reactor_stats
 * does not report these calls. */
int flint_reactor_advance_noalloc(flint_mech_t mech, int64_t n, double* T, const double* p,
                                  double* Y, const double* dt, const flint_reactor_opts* opts,
                                  int* status, int* nsteps, void* stream);

/* ------------------------------------------------------------- surrogate */
/* Learned surrogate of the reactor advance (no reference counterpart: a new
 * path next to run_odesolver).  An MLP maps (log10 Y of all species but the
 * bath, T, log10 p, log10 dt), normalised, to (dY, dT) normalised; BF16
 * weights and activations as tensor-core operands, FP32 accumulation, FP32
 * master weights trained by Adam on the device. */
typedef struct flint_surrogate_s* flint_surrogate_t;

typedef struct {
  int n_layers;           /* GEMM layers (5 = four hidden layers)            */
  int hidden;             /* hidden width (256)                              */
  int n_nets;             /* 1, or 2 for a two-network ensemble               */
  int bath;               /* species implied by sum Y = 1 (not an input)      */
  int n_elements;         /* rows of elem                                    */
  int reserved;
  const float* weights;   /* [n_nets][P] initial parameters, per layer W[out][in] then b[out] */
  const float* x_mean;    /* [ns+2] input normalisation                      */
  const float* x_std;
  const float* y_mean;    /* [ns+1] target normalisation (dY_k, dT)          */
  const float* y_std;
  const double* elem;     /* [n_elements][ns] atoms of each element per species */
} flint_surrogate_desc;

/* Gate of a surrogate step: a cell is accepted only if every test passes,
 * else it is re-solved by the BDF integrator from its original state. */
typedef struct {
  double max_dT_resid;    /* |T(h conservation) - (T0 + dT_net)| limit [K]     */
  double max_elem_resid;  /* max_e |sum_k a_ek dY_net,k / W_k| [kmol/kg]        */
  double min_Y;           /* -(mass clipped to keep Y >= 0) must be >= min_Y   */
  double max_ens_dT;      /* two networks: |dT_1 - dT_2| limit [K]              */
  double max_ens_dY;      /* two networks: max_k |dY_1,k - dY_2,k| limit        */
  double T_lo, T_hi;      /* input domain of the training data                 */
  double log10p_lo, log10p_hi;
  double log10dt_lo, log10dt_hi;
} flint_surrogate_gate;

int flint_surrogate_create(flint_mech_t mech, const flint_surrogate_desc* desc, flint_surrogate_t* out);
int flint_surrogate_destroy(flint_surrogate_t s);
/* Number of parameters of one network. */
int64_t flint_surrogate_nparams(flint_surrogate_t s);
/* Normalised inputs X[n][ns+2] (float, device) of cells (T, p, Y, dt). */
int flint_surrogate_features(flint_surrogate_t s, int64_t n, const double* T, const double* p,
                             const double* Y, const double* dt, float* X, void* stream);
/* Normalised targets Yt[n][ns+1] from states before (T0, Y0) and after (T1, Y1). */
int flint_surrogate_targets(flint_surrogate_t s, int64_t n, const double* T0, const double* Y0,
                            const double* T1, const double* Y1, float* Yt, void* stream);
/* One Adam step of network `net` on a device batch; *loss (may be NULL) gets
 * the batch MSE before the update (synchronises the stream when non-NULL). */
int flint_surrogate_train_step(flint_surrogate_t s, int net, int64_t n, const float* X,
                               const float* Yt, float lr, double* loss, void* stream);
/* Forward pass of network `net`: normalised outputs Yn[n][ns+1] (device). */
int flint_surrogate_predict(flint_surrogate_t s, int net, int64_t n, const float* X, float* Yn,
                            void* stream);
/* Training state of network `net` (host buffer of 3*P floats: weights, Adam
 * first and second moments) and its Adam step: get = 1 reads, 0 writes. */
int flint_surrogate_state(flint_surrogate_t s, int net, float* host, int64_t* step, int get);
/* Surrogate + fallback advance with the arguments of flint_reactor_advance.
 * Accepted cells: status FLINT_CELL_OK, nsteps 0; rejected cells are re-solved
 * by the BDF integrator (status FLINT_CELL_SURROGATE_REJECTED when it
 * succeeds, else its failure code; nsteps its step count).  counts (may be
 * NULL) gets {accepted, rejected} and the call waits for `stream`; with
 * counts NULL it returns without waiting (every operation stays on `stream`,
 * so a call made after a first, sizing call can be captured in a CUDA graph). */
int flint_surrogate_advance(flint_surrogate_t s, int64_t n, double* T, const double* p, double* Y,
                            const double* dt, const flint_reactor_opts* opts,
                            const flint_surrogate_gate* gate, int* status, int* nsteps,
                            int64_t* counts, void* stream);
/* {accepted, rejected} of the last flint_surrogate_advance, read from the
 * device after waiting for it (the form for advances made without counts, such
 * as replays of a captured CUDA graph).  No reference counterpart. */
int flint_surrogate_counts(flint_surrogate_t s, int64_t* counts);

/* Which implementation runs the networks' inference forward: 0 (default) the
 * fused Blackwell kernel -- all layers of a 128-cell tile on one SM,
 * tcgen05.mma with the accumulator in tensor memory, weights streamed from
 * L2 by bulk copies -- wherever the network fits it (hidden layers of 256,
 * inputs and outputs of up to 64); 1 one mma.sync GEMM launch per layer
 * (always; training uses it).  *kind (may be NULL) reports what mode 0/1
 * resolves to for this network (0 fused, 1 per-layer).  No reference
 * counterpart. */
int flint_surrogate_set_forward(flint_surrogate_t s, int mode, int* kind);
/* Waits for the device and reads the fused forward's error word: *err != 0
 * when one of its bounded waits gave up (the outputs of that call are not
 * valid).  No reference counterpart. */
int flint_surrogate_check(flint_surrogate_t s, int* err);
/* Apply the surrogate to every cell (no gate, no fallback; T, Y in place) and
 * write the gate quantities per cell, metrics[cell][6] = {energy residual [K],
 * element residual, realizability (the smaller of -(clipped mass) and the
 * smallest mass fraction), ensemble |dT| spread, ensemble max |dY| spread,
 * 1 if the input is inside the gate's domain and the projected mass fractions
 * are non-negative else 0}: the calibration of the gate thresholds. */
int flint_surrogate_evaluate(flint_surrogate_t s, int64_t n, double* T, const double* p, double* Y,
                             const double* dt, const flint_surrogate_gate* gate, double* metrics,
                             void* stream);

/* Work counters of the last flint_reactor_advance on this handle (blocks until
 * it has finished): out[0] RHS evaluations, out[1] Jacobian evaluations,
 * out[2] Newton iterations (one LU solve each), out[3] accepted steps,
 * out[4] rejected step attempts, out[5] LU factorizations.  No reference
 * counterpart: instrumentation (the CVODE statistics test-batchCXX.cpp:25-48
 * prints are its nearest kin). */
int flint_reactor_stats(flint_mech_t mech, int64_t out[6]);

/* Default options: rtol 1e-8, atol 1e-14, 20000 steps, order 5, constant p. */
void flint_reactor_default_opts(flint_reactor_opts* opts);

/* ------------------------------------------------------------ host forms */
int flint_wdot_batch_host(flint_mech_t mech, int64_t n, int layout, const double* T,
                          const double* p, const double* Y, double* wdot, double* cp,
                          double* h);
int flint_wdot_jac_batch_host(flint_mech_t mech, int64_t n, int layout, const double* T,
                              const double* p, const double* Y, double* wdot, double* jac);
int flint_reactor_advance_host(flint_mech_t mech, int64_t n, double* T, const double* p,
                               double* Y, const double* dt, const flint_reactor_opts* opts,
                               int* status, int* nsteps);

/* FP64 FMA throughput of the current GPU in TFLOP/s (FMA = 2 flops), timed on
 * the default stream with an independent-FMA-chain kernel; the denominator of
 * the FP64 roofline.  No reference counterpart: instrumentation. */
int flint_probe_fp64_peak(double* tflops);

/* Diagnostic: y[2i] = the kernels' table-driven exp(x[i]), y[2i+1] = CUDA's
 * exp(x[i]) (device pointers).  No reference counterpart: lets tests bound the
 * kernels' exp against the CUDA library. */
int flint_selftest_exp(flint_mech_t mech, int64_t n, const double* x, double* y, void* stream);

/* Diagnostic: y[2i] = the kernels' table-driven ln(x[i]), y[2i+1] = CUDA's
 * log(x[i]) (device pointers).  No reference counterpart: lets tests bound the
 * kernels' log against the CUDA library. */
int flint_selftest_log(flint_mech_t mech, int64_t n, const double* x, double* y, void* stream);

/* Number of kernels the library launched since load (instrumentation). */
int64_t flint_kernel_launch_count(void);

#ifdef __cplusplus
}
#endif

#endif /* FLINT_GPU_H */
