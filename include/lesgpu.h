/*
 * lesgpu.h -- C ABI of the GB300 (sm_103a) LES time-step library.
 *
 * The library replaces the body of the time loop of LESwHT's `solver_exec`
 * (02_solver/f90/solver.f90:85-183): one call to lesgpu_step() performs the
 * three RK3/Crank-Nicolson substeps of stepinit .. convergence_check on the
 * device, with the whole solver state resident in HBM.
 *
 * Conventions
 *   - Plain C, POD structs, int64_t for every integer that the Fortran code
 *     holds as integer(8) (the reference builds with -fdefault-integer-8).
 *   - Every 3-D field crossing the boundary is a host array in the Fortran
 *     layout of the reference, dimension (0:n1,0:n2,0:n3), i fastest:
 *     element (i,j,k) sits at  i + (n1+1)*(j + (n2+1)*k).
 *   - 1-D grid vectors are passed exactly as the Fortran driver holds them
 *     after readgeom (misc_init.f90:204-251): a vector declared x(1:n1) is a
 *     pointer to n1 doubles (x[0] is x(1)); a vector declared c2cx(0:n1) is a
 *     pointer to n1+1 doubles (c2cx[0] is c2cx(0)).
 *   - Every entry point returns 0 on success or a negative LESGPU_ERR_* code.
 *     Nothing in the library calls exit(), abort() or traps the device.
 *   - The caller owns host buffers; the library owns device memory.
 *     One host thread drives a case at a time; each case has its own stream.
 */
#ifndef LESGPU_H
#define LESGPU_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LESGPU_ABI_VERSION 2

/* ---- error codes ------------------------------------------------------ */
#define LESGPU_OK                 0
#define LESGPU_ERR_ARG          (-1)  /* bad pointer / size / option value          */
#define LESGPU_ERR_CONFIG       (-2)  /* option combination the reference rejects   */
#define LESGPU_ERR_CUDA         (-3)  /* a CUDA runtime call failed                 */
#define LESGPU_ERR_OOM          (-4)  /* device allocation failed                   */
#define LESGPU_ERR_NOT_CONVERGED (-5) /* iterative Poisson solver hit its limit     */
#define LESGPU_ERR_NAN          (-6)  /* non-finite value detected in the state     */
#define LESGPU_ERR_STATE        (-7)  /* call out of order (e.g. step before start) */
#define LESGPU_ERR_UNSUPPORTED  (-8)  /* option valid in the reference, not built    */
#define LESGPU_ERR_TOO_LARGE    (-9)  /* grid exceeds the fixed scratch of the
                                         allocation-free entry point              */

/* ---- option values ---------------------------------------------------- */
/* Poisson solver: chosen at link time in the reference (02_solver/Makefile:23-34). */
#define LESGPU_POISSON_FTFT  0   /* poiss_ftft.f90  FFT x & z + y Thomas          */
#define LESGPU_POISSON_Z_FT  1   /* poiss_z_ft.f90  FFT z + 2-D x-semicoarsened MG */
#define LESGPU_POISSON_MGRD  2   /* poiss_mgrd.f90  BiCGSTAB + MG3D V-cycle        */
#define LESGPU_POISSON_X_FT  3   /* poiss_x_ft.f90  FFT x + 2-D z-semicoarsened MG */

/* Arithmetic of the step. */
#define LESGPU_PREC_FP64   0     /* every kernel in FP64 (the plain form)          */
#define LESGPU_PREC_MIXED  1     /* FP32 stencils/SGS/FFT; FP64 Thomas-y, Poisson
                                    residual, flow-rate and divergence checks      */

/* Body geometry: the reference links one `funcbody(x,y,z,t)` at compile time
 * (geometry/funcbody.f90).  Value <= 0 inside the body, > 0 in the fluid. */
#define LESGPU_BODY_NONE      0  /* funcbody = +1 everywhere                        */
#define LESGPU_BODY_CHANNEL   1  /* (1 + p0) - |y|      (funcbody_channel.f90)      */
#define LESGPU_BODY_CYLINDER  2  /* sqrt((x-cx)^2+(y-cy)^2) - r  (funcbody_cylinder) */
#define LESGPU_BODY_SPHERE    3  /* sqrt((x-cx)^2+(y-cy)^2+(z-cz)^2) - r            */
#define LESGPU_BODY_SQUARE    4  /* max(|x-cx|,|y-cy|) - r  (square prism)          */

typedef struct lesgpu_body {
    int64_t kind;
    double cx, cy, cz;   /* centre                                               */
    double r;            /* radius / half side                                    */
    double p0;           /* channel half-width offset (EPS in funcbody_channel)   */
} lesgpu_body;

/* Scalars of settings.input and boundary.input (misc_init.f90:19-158) plus
 * the periodicity flags of output/ibmpre/ibmpre_prdic.bin. */
typedef struct lesgpu_config {
    /* settings.input */
    double re, pr, gr;
    int64_t grdir;
    double tflu_i, tsol_i;
    int64_t ireset, iread, iavg, ipzero;
    double eps_ptr, udrv_i;
    int64_t nend, nprint, npriavg, npin;
    double tend, ptb_tst, avg_tst;
    int64_t idtopt;
    double dt_size, cflfac;
    double resid1;
    int64_t nlev, nbli, ioldv, mgitr, imgsor;
    double wwsor;
    int64_t iles, insmdl, itemdl, idvmon;
    double csgsts, csgshf;
    int64_t filter;
    int64_t ibmon, masson, imovingon, ihtrans, idecomp;
    /* boundary.input */
    int64_t bc_ybtm, bc_ytop, bc_zbtm, bc_ztop;
    int64_t bc_t_ybtm, bc_t_ytop;
    double val_t_ybtm, val_t_ytop;
    int64_t bc_t_zbtm, bc_t_ztop;
    double val_t_zbtm, val_t_ztop;
    int64_t ich, iconjg;
    /* ibmpre_prdic.bin */
    int64_t xprdic, yprdic, zprdic, iintp;
    /* choices that are compile/link time in the reference */
    int64_t poisson;     /* LESGPU_POISSON_*  */
    int64_t precision;   /* LESGPU_PREC_*     */
    lesgpu_body body;
} lesgpu_config;

/* The grid as readgeom (misc_init.f90:204-251) leaves it. */
typedef struct lesgpu_grid {
    int64_t n1, n2, n3;        /* gridlines      */
    int64_t n1m, n2m, n3m;     /* cells          */
    double xl, yl, zl;
    const double *x, *y, *z;                    /* x(1:n1) y(1:n2) z(1:n3)   */
    const int64_t *ipv, *jpv, *kpv;             /* (1:n?m)                   */
    const int64_t *imv, *jmv, *kmv;
    const int64_t *fixil, *fixjl, *fixkl;
    const int64_t *fixiu, *fixju, *fixku;
    const double *c2cx, *c2cy, *c2cz;           /* (0:n?)                    */
    const double *c2cxi, *c2cyi, *c2czi;
    const double *f2fx, *f2fy, *f2fz;
    const double *f2fxi, *f2fyi, *f2fzi;
    const double *xmp, *ymp, *zmp;
} lesgpu_grid;

/* Immersed-boundary tables of output/ibmpre (misc_init.f90:254-440).
 * Component l = 0..3 is u, v, w, T (T only when ihtrans = 1).
 * fc[l]       : nbody[l]*3 int64, row n = (ifc, jfc, kfc) of forcing point n
 *               (rows 0..nintp[l]-1 interpolated, the rest inner points)
 * intpindx[l] : nintp[l]*3 int64, row n = direction offsets (-1/0/+1)
 * geomfac[l]  : nintp[l]*27 double, row n = geomfac(n,l,i,j,k) at
 *               i*9 + j*3 + k for i,j,k in 0..2 (the file's record order)
 * nzero, inz/jnz/knz : zero-eddy-viscosity list exactly as ibmpre_nutzero.bin
 *               holds it; the solver uses the values as Fortran (1-based)
 *               indices (sgs.f90:893) although the pre-processor writes
 *               0-based ones, and so does this library
 * nwall_dvm   : (1:n1m,1:n2m,1:n3m) int64 mask, i fastest, or NULL (= 1)
 * cstar       : (1:n1m,1:n2m,1:n3m) double or NULL (= 1)
 * kstar       : (1:n1m,1:n2m,1:n3m,6) double or NULL (= 1)
 * omega       : (1:n1m,1:n2m,1:n3m) int64 or NULL (= 1)                     */
typedef struct lesgpu_ibm {
    int64_t nintp[4], nbody[4];
    const int64_t *fc[4];
    const int64_t *intpindx[4];
    const double  *geomfac[4];
    int64_t nzero;
    const int64_t *inz, *jnz, *knz;
    const int64_t *nwall_dvm;
    const double  *cstar;
    const double  *kstar;
    const int64_t *omega;
} lesgpu_ibm;

/* What one step reports; the quantities writehistory / writeftrtime print. */
typedef struct lesgpu_step_report {
    int64_t ntime, ihist, m;
    double time, dt;
    double cflmax;          /* cfl() of this step (slv_auxi.f90:53)          */
    double dvmax;           /* convergence_check (misc_init.f90:1047)        */
    double qmmax;           /* masscheck (misc_init.f90:1080)                */
    double pmi[5];          /* meanpg after the last substep                 */
    double pmiavg;
    double qvol[3];         /* qvolcalc values of the last substep           */
    double tvol[3];
    double csgsts, csgshf;  /* dynamic coefficients of this step             */
    double nutavg, nutmax, alpavg, alpmax;
    double cd[3];           /* draglift forces (IBMON = 1)                    */
    double heat_flux[3];    /* heatflux (IHTRANS = 1)                         */
    double ubulk;           /* bulk velocity (writehistory)                   */
    double tbulk_fluid, tbulk_solid;
    int64_t poisson_iters[3];   /* iterations of each substep's Poisson solve */
    double phase_ms[4];     /* SGS, RHS+LHS, Poisson, whole step (device ms)  */
    double qflux;           /* flow rate qvol_u / xl (writehistory)           */
    /* Iterative Poisson solves of this step (substeps x z or x modes, or
     * BiCGSTAB solves) that stopped at MGITR above the tolerance: the
     * reference prints 'ITERATION LIMIT EXCEEDED.' and goes on
     * (poiss_z_ft.f90:289, poiss_mgrd.f90:204), as lesgpu_step does unless
     * lesgpu_set_strict is on. */
    int64_t poisson_unconverged;
    /* Heat the thermal IB forcing adds to the fluid per unit time over the
     * step, sum of fcvavg(n,4) * f2fx f2fy f2fz over the thermal forcing
     * points (the thermal counterpart of draglift's force integral,
     * slv_auxi.f90:705-716; fcvavg(:,4) is accumulated in slv_engy.f90:
     * 299-303).  For a body at T = 0 in fluid at T = -1 the mean Nusselt
     * number is heat_body * Re * Pr / (surface area * (0 - (-1))). */
    double heat_body;
} lesgpu_step_report;

/* Fields of lesgpu_get_array / lesgpu_set_array (phase-level parity tests). */
#define LESGPU_F_U       0
#define LESGPU_F_V       1
#define LESGPU_F_W       2
#define LESGPU_F_P       3
#define LESGPU_F_T       4
#define LESGPU_F_NUSGS   5
#define LESGPU_F_NUSGS1  6   /* 3 components, stride (n1+1)(n2+1)(n3+1) */
#define LESGPU_F_ALSGS   7
#define LESGPU_F_ALSGS1  8   /* 3 components                              */
#define LESGPU_F_RHS1    9   /* 4 components                              */
#define LESGPU_F_RK3O    10  /* 4 components: rk3xo, rk3yo, rk3zo, rk3to  */
#define LESGPU_F_RK3OO   11  /* 4 components                              */
#define LESGPU_F_DIVGSUM 12
#define LESGPU_F_PHI     13
#define LESGPU_F_QMASS   14

/* Phases of lesgpu_run_phase: the reference subroutines of one substep. */
#define LESGPU_PH_SUBSTEPINIT 0  /* substepinit(msub)                     */
#define LESGPU_PH_SGS         1  /* sgscalc (+ sgscalc_t)                 */
#define LESGPU_PH_RHSNLHS     2  /* rhsnlhs                               */
#define LESGPU_PH_DIVGS       3  /* divgs                                 */
#define LESGPU_PH_POISSON     4  /* poisson                               */
#define LESGPU_PH_UCALC       5  /* ucalc + pcalc (+ qvol bookkeeping)    */
#define LESGPU_PH_MEANPG      6  /* meanpg                                */
#define LESGPU_PH_ENERGY      7  /* rhsnlhs_t + tvol/tcalc                */
#define LESGPU_PH_STEPINIT    8  /* stepinit (CFL, dt)                    */

typedef struct lesgpu_case lesgpu_case;

/* Build a case: allocates the device state and computes every init-time
 * table (lhsinit slv_mmtm.f90:180, sgsfilterinit sgs.f90:2, poisinit of the
 * chosen solver).  Replaces readsettings..poisinit of solver.f90:28-62. */
int lesgpu_create(const lesgpu_config *cfg, const lesgpu_grid *grid,
                  lesgpu_case **out);

/* IB / LES / conjugate tables (ibmpreread misc_init.f90:312, nutzeroread
 * :381, conjgread :412).  Call before lesgpu_start. */
int lesgpu_load_ibm(lesgpu_case *c, const lesgpu_ibm *ibm);

/* The field state after prefld/makefld (misc_init.f90:443-786): host arrays
 * in the (0:n1,0:n2,0:n3) layout; t may be NULL when ihtrans = 0. */
int lesgpu_set_fields(lesgpu_case *c, const double *u, const double *v,
                      const double *w, const double *p, const double *t,
                      double time, double dt, int64_t ihist, int64_t m);

/* meanpg (ICH != 0), dttimeinit and the cflmax seed of solver.f90:56-75. */
int lesgpu_start(lesgpu_case *c);

/* One full time step, solver.f90:85-151 + convergence_check/masscheck and
 * the per-step diagnostics (draglift, heatflux, bulk quantities). */
int lesgpu_step(lesgpu_case *c, lesgpu_step_report *rep);

/* Copy the field state back (writefield misc_hist.f90:212). */
int lesgpu_get_fields(lesgpu_case *c, double *u, double *v, double *w,
                      double *p, double *t);

/* Running time averages of field_avg (misc_hist.f90:287-527).  With IAVG = 1
 * every lesgpu_step after time > AVG_TST adds dt-weighted cell-centre
 * statistics on the device.  lesgpu_get_averages copies them out in the
 * record order of the reference's fav file -- uavg, vavg, wavg, uiujavg(1..6),
 * pavg, p2avg, voravg(1..3), vor2avg(1..6), ssavg, then tavg, t2avg when
 * IHTRANS = 1 -- each an (n1m, n2m, n3m) array in Fortran order, so `out`
 * holds LESGPU_NAVG (or LESGPU_NAVG - 2) * n1m*n2m*n3m doubles; *nsamples
 * is the number of steps summed; reset != 0 zeroes the sums (the reference
 * does so after writing each fav file, every NPRIAVG samples). */
#define LESGPU_NAVG 23
int lesgpu_get_averages(lesgpu_case *c, double *out, int64_t *nsamples, int reset);

/* Serving loop (no reference counterpart; the reference runs one case per
 * process).  A server owns one worker thread on `device`.  Cases submitted at
 * any time wait until their device footprint fits `hbm_budget_bytes` and fewer
 * than `max_active` cases are resident; an admitted case keeps its fields on
 * the device for its whole run and advances `steps_in_flight` steps at a time
 * on its own stream and captured step graph, so the work of all resident
 * cases overlaps on the GPU.  A finished case is copied back and freed at
 * once, which admits the next waiting case.  Submission copies every input;
 * results (the five fields, the last step report and the seconds from
 * submission to completion) are copied out by lesgpu_server_result.
 * Request states: 0 waiting, 1 running, 2 done, 3 failed, 4 cancelled. */
typedef struct lesgpu_server lesgpu_server;
int lesgpu_server_create(int64_t device, int64_t hbm_budget_bytes, int64_t max_active,
                         int64_t steps_in_flight, lesgpu_server **out);
int lesgpu_server_submit(lesgpu_server *s, const lesgpu_config *cfg, const lesgpu_grid *grid,
                         const lesgpu_ibm *ibm, const double *u, const double *v, const double *w,
                         const double *p, const double *t, double time, double dt, int64_t ihist,
                         int64_t m, int64_t nsteps, int64_t *ticket);
int lesgpu_server_poll(lesgpu_server *s, int64_t ticket, int64_t *state, int64_t *steps_done);
int lesgpu_server_result(lesgpu_server *s, int64_t ticket, double *u, double *v, double *w,
                         double *p, double *t, lesgpu_step_report *rep, double *seconds_to_solution);
int lesgpu_server_release(lesgpu_server *s, int64_t ticket);
int lesgpu_server_stats(lesgpu_server *s, int64_t *pending, int64_t *active, int64_t *bytes_used,
                        double *cell_steps);
int lesgpu_server_destroy(lesgpu_server *s);

/* Immersed-boundary pre-processing on the GPU (the pre-processor's
 * ibm_body.f90 find_inout :14, findbdy_intp :49, geomfac_preset :126,
 * geomfac_intp :160, find_zero_nu_sgs :357 as preprocessing.py drives them
 * and lib_preprocessing.py writes them).  The tables are exactly what the
 * solver reads back from output/ibmpre: forcing points in the reference's
 * k, j, i order (interpolated first), geomfac rounded to its '%15.8f' text,
 * the zero-viscosity list 0-based, the wall mask; c*, k*, omega are left
 * NULL (= 1, the placeholders).  axes = {xc, xm, yc, ym, zc, zm}: the
 * coordinate and centre vectors (0:n?) the pre-processor holds in full
 * precision, n? + 1 values each.  lesgpu_ibmpre_tables fills a lesgpu_ibm
 * for lesgpu_load_ibm with pointers owned by the handle. */
typedef struct lesgpu_ibmpre lesgpu_ibmpre;
int lesgpu_ibmpre_run(const lesgpu_config *cfg, const lesgpu_grid *grid, const double *const axes[6],
                      lesgpu_ibmpre **out);
int lesgpu_ibmpre_tables(lesgpu_ibmpre *h, lesgpu_ibm *tables);
int lesgpu_ibmpre_free(lesgpu_ibmpre *h);

/* conjg_intp (ibm_body.f90:402-550, called by preprocessing.py:286 for
 * CONJG-HTRANS): on the GPU, the conjugate heat-transfer tables of the cells
 * 1..n?m -- c* = (1 - fp) cratio + fp from the cell's fluid fraction fp
 * (fluid_portion, a flood fill on 6x6x6 sub-cells), the fluid mask omega
 * (fp >= 1 - 1e-12), and k* of the east, west, north, south, top and bottom
 * faces from the fluid fraction between the two cell centres (harmonic mean
 * across the interface) -- for the body and periodicity of cfg, the
 * pre-processor's coordinate vectors axes (as lesgpu_ibmpre_run) and the
 * solid/fluid ratios cratio (heat capacity) and kratio (conductivity).
 * Host outputs in lesgpu_ibm's layout: cstar[ncell], kstar[6 * ncell],
 * omega[ncell], cells i fastest. */
int lesgpu_conjg_run(const lesgpu_config *cfg, const lesgpu_grid *grid, const double *const axes[6],
                     double cratio, double kratio, double *cstar, double *kstar, int64_t *omega);

/* Phase-level access for parity tests (not needed by a driver). */
int lesgpu_get_array(lesgpu_case *c, int64_t field, double *out);
int lesgpu_set_array(lesgpu_case *c, int64_t field, const double *in);
int lesgpu_run_phase(lesgpu_case *c, int64_t phase, int64_t msub);
int lesgpu_get_report(lesgpu_case *c, lesgpu_step_report *rep);

/* Benchmark / driver helpers (no reference counterpart).
 * lesgpu_step_async enqueues n steps on the case's stream without reading
 * anything back; lesgpu_stream returns that cudaStream_t (as void*) so a
 * caller can record events on it; lesgpu_use_graph(0) disables the CUDA
 * graph replay of steps. */
int lesgpu_step_async(lesgpu_case *c, int64_t n);
int lesgpu_stream(lesgpu_case *c, void **stream);
int lesgpu_use_graph(lesgpu_case *c, int on);

/* Strict convergence (no reference counterpart; the reference only prints
 * a warning): with on != 0, lesgpu_step returns LESGPU_ERR_NOT_CONVERGED
 * after completing a step in which report.poisson_unconverged > 0 (the
 * state has advanced and the report is filled, as without it). */
int lesgpu_set_strict(lesgpu_case *c, int on);

/* Kernel launches one step makes (counted from the captured step graph). */
int lesgpu_launch_count(lesgpu_case *c, int64_t *kernels_per_step);

/* The autotuner's choices for this case's shape (no reference counterpart).
 * At lesgpu_start every feasible lanes-per-line count of each ADI sweep class
 * (direction, components batched, FP32 or FP64) is timed on the case's own
 * sweeps and the fastest kept for the process; LESGPU_AUTOTUNE=0 in the
 * environment turns it off for cases started afterwards (defaults are then
 * used, and results are reproducible across processes); LESGPU_TUNE_FILE
 * names a text file the table is read from before tuning and written back to
 * after, so several processes share one set of choices.  Writes up to maxn
 * tuples (dir 0..2 = x,y,z; components; fp32 0/1; lanes, 1 = one thread per
 * line, + 64 when the register-capped variant of the warp-scan kernel won)
 * to out as 4 int64 each and their number to *nclasses (lanes = 128: the
 * tiled FP32 sweep, lines staged in shared memory); the Poisson FFTs'
 * lines per block, also timed at start, follow as (3, 2 = z | 0 = x, 0,
 * lines), for poiss_z_ft / poiss_x_ft the multigrid's blocks per cluster
 * as (4, 0, 0, blocks), and for poiss_ftft in the mixed form the solve chosen
 * as (5, 0, 0, 1 = FP32 transforms under an FP64 defect correction | 0 =
 * FP64 transforms); LESGPU_FFT_MIXED=1 / 0 forces either. */
int lesgpu_tuning(lesgpu_case *c, int64_t *out, int64_t maxn, int64_t *nclasses);

/* Event instrumentation of one kernel class for roofline measurements:
 * lesgpu_instrument(c, cls) makes the following steps run without the graph
 * and brackets every launch of class `cls` (LESGPU_K_*) with CUDA events on
 * the case's stream; lesgpu_instrument_read returns the summed device time
 * (ms) and the number of launches since the call, and cls = 0 switches the
 * instrumentation off. */
#define LESGPU_K_RHS      1   /* fused rhs + rhssgs (momentum)          */
#define LESGPU_K_ADI      2   /* tridiagonal sweeps, momentum and T     */
#define LESGPU_K_SGS      3   /* SGS passes and test filters            */
#define LESGPU_K_POISSON  4   /* FFT + y-Thomas Poisson solve           */
#define LESGPU_K_RHS_T    5   /* rhs_t                                  */
int lesgpu_instrument(lesgpu_case *c, int64_t cls);
/* Select the CUDA device used by the cases this thread creates next
 * (one process per GPU when several GPUs run replicas). */
int lesgpu_set_device(int64_t device);
int lesgpu_instrument_read(lesgpu_case *c, double *ms, int64_t *launches);

/* Allocation-free pressure Poisson solve.  No counterpart in the reference:
 * it serves callers that cannot call cudaMalloc (a runtime that hands out
 * device memory only from its own pool, a real-time loop that must not enter
 * the driver's allocator, a plugin that must not bypass its host's
 * allocator).  It runs the poiss_ftft solve of a case -- FFT in x and z,
 * Thomas in y, the (1,1) mode pinned -- on caller-owned DEVICE buffers
 * divgsum (input) and phi (output, interior written), both in the
 * (0:n1,0:n2,0:n3) layout, on `stream` (a cudaStream_t, or NULL), and keeps
 * all its temporaries in one fixed 32 MiB device array per GPU.  The grid is
 * read from host memory; it must be periodic and uniform in x and z (ipv and
 * kpv wrap to 1, every 1/dx and 1/dz within 1e-6 relative of the first),
 * else LESGPU_ERR_UNSUPPORTED; a NULL grid vector is LESGPU_ERR_ARG.
 *   - It calls no cudaMalloc/cudaFree; grids needing more than the fixed
 *     array (24*n1m*(n3m/2+1)*n2m bytes plus tables, about 128^3 at most,
 *     and at most 1024 cells per direction) return LESGPU_ERR_TOO_LARGE.
 *   - It copies nothing from host memory: its tables are built on the device
 *     and the wall-normal vectors travel as kernel parameters.
 *   - The first call on a device sets it up (resolves the array's device
 *     address); that first call must not be made during a stream capture.
 *   - All calls on a device share the array and leave their contents in it;
 *     calls that overlap on the GPU race with each other -- serialise them.
 *   - An error already pending in the calling thread's CUDA state is left
 *     untouched and the call returns LESGPU_ERR_CUDA without launching.
 *   - Returns after enqueueing; synchronise `stream` before reading phi. */
int lesgpu_poisson_ftft_noalloc(const lesgpu_grid *grid, const double *d_divgsum,
                                double *d_phi, void *stream);

int lesgpu_destroy(lesgpu_case *c);
const char *lesgpu_strerror(int code);
int lesgpu_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* LESGPU_H */
