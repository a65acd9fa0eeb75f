/*
 * ORACLE -- test infrastructure only.
 *
 * lesref: a CPU (C11 + OpenMP) restatement of the LESwHT per-time-step
 * solver routines, used by the tests as the parity checker for the GPU
 * library and by bench.py as the timed CPU baseline.  It is never linked
 * into, loaded by, or called from the product library.
 *
 * Parity status: the reference solver is Fortran and cannot be built in the
 * development container (no Fortran compiler), and the reference ships no
 * golden outputs for the solver, so this restatement is pinned only by
 * invariants (FFT round trips, tridiagonal residuals, discrete Poisson
 * residuals, divergence after projection, periodic symmetry) and, for the
 * grid metrics it consumes, by fixtures produced with the reference's own
 * Python pre-processor.  Each routine cites the Fortran it restates.
 *
 * Storage: every 3-D array, including the reference's interior-only arrays
 * (rk3xo(n1m,n2m,n3m), qmass, ...), is held in the full (0:n1,0:n2,0:n3)
 * layout, i fastest, so one index macro serves all of them.  1-D vectors
 * are indexed with the Fortran index (x[1..n1], c2cx[0..n1], ipv[1..n1m]).
 */
#ifndef LESREF_INTERNAL_H
#define LESREF_INTERNAL_H

#include <stdint.h>
#include <stddef.h>
#include "../include/lesgpu.h"

typedef long long ll;

typedef struct { double re, im; } cplx;

typedef struct ref_fft_plan {
    int n;
    int nfac;
    int fac[32];
    cplx *tw;      /* exp(-2 pi i m / n), m = 0..n-1 */
} ref_fft_plan;

typedef struct ref_case {
    lesgpu_config c;
    ll n1, n2, n3, n1m, n2m, n3m, n1md, n2md, n3md, n1mh, n2mh, n3mh;
    double xl, yl, zl;
    size_t sx, sxy, nt;          /* strides and total size of a 3-D array */

    /* grid (Fortran indices) */
    double *x, *y, *z, *xmp, *ymp, *zmp;
    ll *ipv, *jpv, *kpv, *imv, *jmv, *kmv;
    ll *fixil, *fixiu, *fixjl, *fixju, *fixkl, *fixku;
    double *f2fx, *f2fy, *f2fz, *f2fxi, *f2fyi, *f2fzi;
    double *c2cx, *c2cy, *c2cz, *c2cxi, *c2cyi, *c2czi;

    /* funcbody values at the evaluation points the solver uses */
    double *fb_u;   /* funcbody(x(i),   ymp(j), zmp(k)) */
    double *fb_c;   /* funcbody(xmp(i), ymp(j), zmp(k)) */

    /* fields */
    double *u, *v, *w, *p, *t;
    double *rhs1[4];
    double *rk3o[4], *rk3oo[4];
    double *nusgs, *nusgs1[3], *alsgs, *alsgs1[3];
    double *qmass, *divgsum, *phi;
    double *cstar, *kstar[6];
    ll *omega, *nwall;

    /* IB tables */
    ll nintp[4], nbody[4];
    ll *ifc[4], *jfc[4], *kfc[4];
    ll *intpindx[4];            /* [n*3 + d] */
    double *geomfac[4];         /* [n*27 + a*9 + b*3 + cc] */
    double *fcv[4], *fcvavg[4], *dudtr[3];
    ll nzero;
    ll *inz, *jnz, *knz;

    /* convective outlet planes (0:n2,0:n3) */
    double *uout, *vout, *wout, *tout, *duout, *dvout, *dwout, *dtout;

    /* ADI coefficients (lhsinit) */
    double *aiu, *ciu, *aivw, *civw, *ajv, *cjv, *ajuw, *cjuw, *akw, *ckw, *akuv, *ckuv;
    ll i_bgpx, j_bgpy, k_bgpz;

    /* test filter coefficients cf?1(n?m,-1:1) */
    double *cfx1, *cfy1, *cfz1;

    /* Poisson */
    double *ak1, *ak3;                 /* modified wavenumbers (ftft, z_ft) */
    ref_fft_plan fftx, fftz;
    /* z_ft / mgrd multigrid */
    ll iimg[21][3], kkmg[21][3];
    double *aw, *ae, *as, *an, *ab, *af;
    double *coi1, *coi2, *cor1, *cor2;
    double *fidw, *fkdw, *fiup, *fkup;
    ll *ih1, *ih2, *kh1, *kh2, *il1, *il2, *kl1, *kl2;
    ll *ipm, *imm, *kpm, *kmm;
    double *ac, *gam, *bet;            /* z_ft: (n1md,n2m,n3mh); mgrd: (n1md,n2m,n3md) */
    ll poisson_iters[3];               /* per substep: most cycles any mode took */
    ll poisson_unconv;                 /* solves of the step that stopped at MGITR above the test */
    double heat_body;                  /* draglift's thermal term: sum fcvavg(n,4) f2fx f2fy f2fz */

    /* scalars (mod_common) */
    ll ntime, ihist, m, msub;
    double dt, time, subdt;
    double dvmax, cflmax, qmmax;
    double gamma[4], ro[4];
    double alpha, dtconst, dtconsti, test1, acoef, acoefi;
    double pmi[5], pmiavg, qvol[3], tvol[3], phcap, thcap;
    double csgsts, csgshf;
    double nutavg, nutmax, alpavg, alpmax;
    double err_integral;          /* meanpg's SAVEd controller state */
    double dudta, dvdta, dwdta;
    double cd[3], heat_flux[3];
    double ubulk, qflux, tbulk_fluid, tbulk_solid;
    /* field_avg accumulators: LESGPU_NAVG arrays in the full layout, record order of the fav file */
    double *avg;
    ll avg_count;
    int started;
} ref_case;

#define IX(c, i, j, k) ((size_t)(i) + (c)->sx * (size_t)(j) + (c)->sxy * (size_t)(k))

/* allocation helpers */
double *ref_zalloc(size_t n);
ll *ref_izalloc(size_t n);

/* funcbody descriptor (geometry/funcbody.f90 and funcbody_example/) */
double ref_funcbody(const lesgpu_body *b, double x, double y, double z);

/* FFT with FFTE conventions (ffte-7.0/zfft1d.f:18-84) */
int ref_fft_plan_init(ref_fft_plan *p, int n);
void ref_fft_plan_free(ref_fft_plan *p);
void ref_fft(const ref_fft_plan *p, cplx *a, cplx *work, int iopt);

/* routines, grouped by reference file */
/* slv_auxi.f90 */
void ref_stepinit(ref_case *c);
void ref_cfl(ref_case *c);
void ref_substepinit(ref_case *c, ll msub);
double ref_qvolcalc(ref_case *c);
double ref_tvolcalc(ref_case *c);
void ref_qvolcorr(ref_case *c);
void ref_tvolcorr(ref_case *c);
void ref_ucalc(ref_case *c);
void ref_pcalc(ref_case *c);
void ref_tcalc(ref_case *c);
void ref_lagforce(ref_case *c);
void ref_heatflux(ref_case *c);
void ref_draglift(ref_case *c);
/* slv_mmtm.f90 */
void ref_meanpg(ref_case *c);
void ref_lhsinit(ref_case *c);
void ref_rhsnlhs(ref_case *c);
void ref_rhs(ref_case *c);
void ref_rhs_ibm(ref_case *c);
void ref_convbc(ref_case *c);
void ref_rhsincorpbc(ref_case *c);
void ref_lhsu(ref_case *c);
void ref_lhsv(ref_case *c);
void ref_lhsw(ref_case *c);
void ref_retrv_uvw(ref_case *c);
void ref_prdic_adj_uvw(ref_case *c, int isp);
void ref_trdiag(const double *a, const double *b, const double *cc, double *r,
                ll l1, ll l2, ll ll1, ll ll2, ll ld);
void ref_trdiagp(const double *a, const double *b, const double *cc, double *f,
                 ll j1, ll j2, ll l1, ll l2, ll ld);
/* slv_cont.f90 */
void ref_divgs(ref_case *c);
/* sgs.f90 */
void ref_sgsfilterinit(ref_case *c);
void ref_sgscalc(ref_case *c);
void ref_sgscalc_t(ref_case *c);
void ref_rhssgs(ref_case *c);
void ref_velgrad(const ref_case *c, ll i, ll j, ll k, double a[9], double sr[6]);
void ref_test_filter(const ref_case *c, double *a0, double *tmp, double *src);
/* slv_engy.f90 */
void ref_rhsnlhs_t(ref_case *c);
/* poisson */
int ref_poisinit(ref_case *c);
void ref_poisson(ref_case *c);
/* misc_init.f90 */
void ref_convergence_check(ref_case *c);
/* misc_hist.f90 */
void ref_field_avg(ref_case *c);
void ref_masscheck(ref_case *c);
void ref_bulk_diag(ref_case *c);

#endif
