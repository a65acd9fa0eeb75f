/*
 * ORACLE -- test infrastructure only (see lesref_internal.h).
 *
 * Case lifetime, the time-step driver and the auxiliary routines of
 * 02_solver/f90/lib/slv_auxi.f90 and misc_init.f90.
 */
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "lesref_internal.h"
#include "lesref.h"
#ifdef _OPENMP
#include <omp.h>
#endif

double *ref_zalloc(size_t n) { return (double *)calloc(n ? n : 1, sizeof(double)); }
ll *ref_izalloc(size_t n) { return (ll *)calloc(n ? n : 1, sizeof(ll)); }

/* geometry/funcbody.f90 and geometry/funcbody_example/funcbody_*.f90 */
double ref_funcbody(const lesgpu_body *b, double x, double y, double z)
{
    switch (b->kind) {
    case LESGPU_BODY_CHANNEL: return (1.0 + b->p0) - fabs(y);
    case LESGPU_BODY_CYLINDER: {
        double dx = x - b->cx, dy = y - b->cy;
        return sqrt(dx * dx + dy * dy) - b->r;
    }
    case LESGPU_BODY_SPHERE: {
        double dx = x - b->cx, dy = y - b->cy, dz = z - b->cz;
        return sqrt(dx * dx + dy * dy + dz * dz) - b->r;
    }
    case LESGPU_BODY_SQUARE: {
        double ax = fabs(x - b->cx), ay = fabs(y - b->cy);
        return (ax > ay ? ax : ay) - b->r;
    }
    default: return 1.0;
    }
}

static double *copy_vec0(const double *src, ll n)   /* (0:n) */
{
    double *d = ref_zalloc((size_t)n + 2);
    for (ll i = 0; i <= n; i++) d[i] = src[i];
    return d;
}
static double *copy_vec1(const double *src, ll n)   /* (1:n) */
{
    double *d = ref_zalloc((size_t)n + 2);
    for (ll i = 1; i <= n; i++) d[i] = src[i - 1];
    return d;
}
static ll *copy_ivec1(const int64_t *src, ll n)
{
    ll *d = ref_izalloc((size_t)n + 2);
    for (ll i = 1; i <= n; i++) d[i] = src[i - 1];
    return d;
}

int ref_create(const lesgpu_config *cfg, const lesgpu_grid *g, ref_case **out)
{
    if (!cfg || !g || !out) return LESGPU_ERR_ARG;
    ref_case *c = (ref_case *)calloc(1, sizeof(ref_case));
    if (!c) return LESGPU_ERR_OOM;
    c->c = *cfg;
    c->n1 = g->n1; c->n2 = g->n2; c->n3 = g->n3;
    c->n1m = g->n1m; c->n2m = g->n2m; c->n3m = g->n3m;
    if (c->n1 != c->n1m + 1 || c->n2 != c->n2m + 1 || c->n3 != c->n3m + 1) { free(c); return LESGPU_ERR_ARG; }
    /* mod_common.f90:118-123 */
    c->n1md = c->n1m * 2; c->n2md = c->n2m * 2; c->n3md = c->n3m * 2;
    c->n1mh = c->n1m / 2 + 1; c->n2mh = c->n2m / 2 + 1; c->n3mh = c->n3m / 2 + 1;
    c->xl = g->xl; c->yl = g->yl; c->zl = g->zl;
    c->sx = (size_t)(c->n1 + 1);
    c->sxy = c->sx * (size_t)(c->n2 + 1);
    c->nt = c->sxy * (size_t)(c->n3 + 1);

    c->x = copy_vec1(g->x, c->n1); c->y = copy_vec1(g->y, c->n2); c->z = copy_vec1(g->z, c->n3);
    c->ipv = copy_ivec1(g->ipv, c->n1m); c->jpv = copy_ivec1(g->jpv, c->n2m); c->kpv = copy_ivec1(g->kpv, c->n3m);
    c->imv = copy_ivec1(g->imv, c->n1m); c->jmv = copy_ivec1(g->jmv, c->n2m); c->kmv = copy_ivec1(g->kmv, c->n3m);
    c->fixil = copy_ivec1(g->fixil, c->n1m); c->fixjl = copy_ivec1(g->fixjl, c->n2m); c->fixkl = copy_ivec1(g->fixkl, c->n3m);
    c->fixiu = copy_ivec1(g->fixiu, c->n1m); c->fixju = copy_ivec1(g->fixju, c->n2m); c->fixku = copy_ivec1(g->fixku, c->n3m);
    c->c2cx = copy_vec0(g->c2cx, c->n1); c->c2cy = copy_vec0(g->c2cy, c->n2); c->c2cz = copy_vec0(g->c2cz, c->n3);
    c->c2cxi = copy_vec0(g->c2cxi, c->n1); c->c2cyi = copy_vec0(g->c2cyi, c->n2); c->c2czi = copy_vec0(g->c2czi, c->n3);
    c->f2fx = copy_vec0(g->f2fx, c->n1); c->f2fy = copy_vec0(g->f2fy, c->n2); c->f2fz = copy_vec0(g->f2fz, c->n3);
    c->f2fxi = copy_vec0(g->f2fxi, c->n1); c->f2fyi = copy_vec0(g->f2fyi, c->n2); c->f2fzi = copy_vec0(g->f2fzi, c->n3);
    c->xmp = copy_vec0(g->xmp, c->n1); c->ymp = copy_vec0(g->ymp, c->n2); c->zmp = copy_vec0(g->zmp, c->n3);

    size_t nt = c->nt;
    c->fb_u = ref_zalloc(nt); c->fb_c = ref_zalloc(nt);
    for (ll k = 0; k <= c->n3; k++)
        for (ll j = 0; j <= c->n2; j++)
            for (ll i = 0; i <= c->n1; i++) {
                double xi = (i >= 1) ? c->x[i] : 0.0;
                c->fb_u[IX(c, i, j, k)] = ref_funcbody(&cfg->body, xi, c->ymp[j], c->zmp[k]);
                c->fb_c[IX(c, i, j, k)] = ref_funcbody(&cfg->body, c->xmp[i], c->ymp[j], c->zmp[k]);
            }

    c->u = ref_zalloc(nt); c->v = ref_zalloc(nt); c->w = ref_zalloc(nt);
    c->p = ref_zalloc(nt); c->t = ref_zalloc(nt);
    for (int l = 0; l < 4; l++) {
        c->rhs1[l] = ref_zalloc(nt); c->rk3o[l] = ref_zalloc(nt); c->rk3oo[l] = ref_zalloc(nt);
    }
    c->nusgs = ref_zalloc(nt); c->alsgs = ref_zalloc(nt);
    for (int l = 0; l < 3; l++) { c->nusgs1[l] = ref_zalloc(nt); c->alsgs1[l] = ref_zalloc(nt); }
    c->qmass = ref_zalloc(nt); c->divgsum = ref_zalloc(nt); c->phi = ref_zalloc(nt);
    c->cstar = ref_zalloc(nt);
    for (int l = 0; l < 6; l++) c->kstar[l] = ref_zalloc(nt);
    c->omega = ref_izalloc(nt); c->nwall = ref_izalloc(nt);
    for (size_t q = 0; q < nt; q++) {          /* conjg_allo / les_allo defaults */
        c->cstar[q] = 1.0; c->omega[q] = 1; c->nwall[q] = 1;
        for (int l = 0; l < 6; l++) c->kstar[l][q] = 1.0;
    }
    size_t np = (size_t)(c->n2 + 1) * (size_t)(c->n3 + 1);
    c->uout = ref_zalloc(np); c->vout = ref_zalloc(np); c->wout = ref_zalloc(np); c->tout = ref_zalloc(np);
    c->duout = ref_zalloc(np); c->dvout = ref_zalloc(np); c->dwout = ref_zalloc(np); c->dtout = ref_zalloc(np);
    for (int l = 0; l < 4; l++) { c->fcv[l] = ref_zalloc(1); c->fcvavg[l] = ref_zalloc(1); c->ifc[l] = ref_izalloc(1); c->jfc[l] = ref_izalloc(1); c->kfc[l] = ref_izalloc(1); c->intpindx[l] = ref_izalloc(1); c->geomfac[l] = ref_zalloc(1); }
    for (int l = 0; l < 3; l++) c->dudtr[l] = ref_zalloc(1);
    c->inz = ref_izalloc(1); c->jnz = ref_izalloc(1); c->knz = ref_izalloc(1);

    /* rk3coefinit (misc_init.f90:1031-1044) */
    c->gamma[1] = 8.0 / 15.0; c->gamma[2] = 5.0 / 12.0; c->gamma[3] = 3.0 / 4.0;
    c->ro[1] = 0.0; c->ro[2] = -17.0 / 60.0; c->ro[3] = -5.0 / 12.0;

    ref_lhsinit(c);
    if (cfg->iles == 1) ref_sgsfilterinit(c);
    int rc = ref_poisinit(c);
    if (rc) { ref_destroy(c); return rc; }
    *out = c;
    return 0;
}

int ref_load_ibm(ref_case *c, const lesgpu_ibm *b)
{
    if (!c || !b) return LESGPU_ERR_ARG;
    int nl = (c->c.ihtrans == 1) ? 4 : 3;
    for (int l = 0; l < nl; l++) {
        ll nb = b->nbody[l], ni = b->nintp[l];
        if (nb < ni || ni < 0) return LESGPU_ERR_ARG;
        c->nbody[l] = nb; c->nintp[l] = ni;
        free(c->ifc[l]); free(c->jfc[l]); free(c->kfc[l]); free(c->intpindx[l]); free(c->geomfac[l]);
        free(c->fcv[l]); free(c->fcvavg[l]);
        c->ifc[l] = ref_izalloc(nb + 1); c->jfc[l] = ref_izalloc(nb + 1); c->kfc[l] = ref_izalloc(nb + 1);
        c->intpindx[l] = ref_izalloc(3 * (ni + 1)); c->geomfac[l] = ref_zalloc(27 * (ni + 1));
        c->fcv[l] = ref_zalloc(nb + 1); c->fcvavg[l] = ref_zalloc(nb + 1);
        for (ll n = 0; n < nb; n++) {
            c->ifc[l][n + 1] = b->fc[l][3 * n]; c->jfc[l][n + 1] = b->fc[l][3 * n + 1]; c->kfc[l][n + 1] = b->fc[l][3 * n + 2];
        }
        for (ll n = 0; n < ni; n++) {
            for (int d = 0; d < 3; d++) c->intpindx[l][3 * (n + 1) + d] = b->intpindx[l][3 * n + d];
            for (int q = 0; q < 27; q++) c->geomfac[l][27 * (n + 1) + q] = b->geomfac[l][27 * n + q];
        }
        if (l < 3) { free(c->dudtr[l]); c->dudtr[l] = ref_zalloc(nb + 1); }
    }
    c->nzero = b->nzero;
    free(c->inz); free(c->jnz); free(c->knz);
    c->inz = ref_izalloc(c->nzero + 1); c->jnz = ref_izalloc(c->nzero + 1); c->knz = ref_izalloc(c->nzero + 1);
    for (ll n = 0; n < c->nzero; n++) { c->inz[n + 1] = b->inz[n]; c->jnz[n + 1] = b->jnz[n]; c->knz[n + 1] = b->knz[n]; }
    ll n1m = c->n1m, n2m = c->n2m, n3m = c->n3m;
    for (ll k = 1; k <= n3m; k++)
        for (ll j = 1; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++) {
                size_t q = (size_t)(i - 1) + (size_t)n1m * ((size_t)(j - 1) + (size_t)n2m * (size_t)(k - 1));
                size_t s = IX(c, i, j, k);
                if (b->nwall_dvm) c->nwall[s] = b->nwall_dvm[q];
                if (b->cstar) c->cstar[s] = b->cstar[q];
                if (b->omega) c->omega[s] = b->omega[q];
                if (b->kstar)
                    for (int l = 0; l < 6; l++) c->kstar[l][s] = b->kstar[q + (size_t)l * n1m * n2m * n3m];
            }
    return 0;
}

int ref_set_fields(ref_case *c, const double *u, const double *v, const double *w,
                   const double *p, const double *t, double time, double dt,
                   int64_t ihist, int64_t m)
{
    if (!c || !u || !v || !w || !p) return LESGPU_ERR_ARG;
    memcpy(c->u, u, c->nt * sizeof(double));
    memcpy(c->v, v, c->nt * sizeof(double));
    memcpy(c->w, w, c->nt * sizeof(double));
    memcpy(c->p, p, c->nt * sizeof(double));
    if (t) memcpy(c->t, t, c->nt * sizeof(double));
    c->time = time; c->dt = dt; c->ihist = ihist; c->m = m;
    return 0;
}

/* solver.f90:56-75: meanpg, dttimeinit (misc_init.f90:1001), cflmax seed */
int ref_start(ref_case *c)
{
    if (!c) return LESGPU_ERR_ARG;
    if (c->c.ich != 0) ref_meanpg(c);
    if (c->c.idtopt == 0) c->dt = c->c.dt_size;
    if (c->c.idtopt != 0 && c->c.iread == 0) c->dt = c->c.dt_size;
    if (c->c.ireset == 1) { c->ihist = 0; c->time = 0.0; }
    c->ntime = 0;
    c->cflmax = c->c.cflfac;
    c->err_integral = 0.0;
    c->started = 1;
    return 0;
}

/* solver.f90:85-175 without file output */
int ref_step(ref_case *c, lesgpu_step_report *rep)
{
    if (!c) return LESGPU_ERR_ARG;
    if (!c->started) return LESGPU_ERR_STATE;
    const lesgpu_config *g = &c->c;
    ref_stepinit(c);
    c->subdt = 0.0;
    for (ll msub = 1; msub <= 3; msub++) {
        ref_substepinit(c, msub);
        if (g->ich == 1) c->qvol[1] = ref_qvolcalc(c);
        if (g->iles == 1) {
            ref_sgscalc(c);
            if (g->ihtrans == 1) ref_sgscalc_t(c);
        }
        ref_rhsnlhs(c);
        memset(c->divgsum, 0, c->nt * sizeof(double));
        memset(c->phi, 0, c->nt * sizeof(double));
        ref_divgs(c);
        ref_poisson(c);
        if (g->ich == 1) { c->qvol[2] = ref_qvolcalc(c); ref_qvolcorr(c); }
        ref_ucalc(c);
        if (g->ich == 1) c->qvol[0] = ref_qvolcalc(c);
        ref_pcalc(c);
        if (g->ich != 0) ref_meanpg(c);
        if (g->ibmon == 1) ref_lagforce(c);
        if (g->ihtrans == 1) {
            if (g->ich == 1) c->tvol[1] = ref_tvolcalc(c);
            ref_rhsnlhs_t(c);
            if (g->ich == 1) { c->tvol[2] = ref_tvolcalc(c); ref_tvolcorr(c); }
            ref_tcalc(c);
            if (g->ich == 1) c->tvol[0] = ref_tvolcalc(c);
        }
    }
    c->time = c->time + c->dt;
    ref_convergence_check(c);
    if (g->ibmon == 1 && g->masson == 1) ref_masscheck(c);
    ref_bulk_diag(c);
    if (g->ibmon == 1) ref_draglift(c);
    if (g->ihtrans == 1) ref_heatflux(c);
    if (g->iavg == 1) ref_field_avg(c);
    if (rep) ref_get_report(c, rep);
    return 0;
}

int ref_get_report(ref_case *c, lesgpu_step_report *r)
{
    if (!c || !r) return LESGPU_ERR_ARG;
    memset(r, 0, sizeof(*r));
    r->ntime = c->ntime; r->ihist = c->ihist; r->m = c->m;
    r->time = c->time; r->dt = c->dt;
    r->cflmax = c->cflmax; r->dvmax = c->dvmax; r->qmmax = c->qmmax;
    for (int i = 0; i < 5; i++) r->pmi[i] = c->pmi[i];
    r->pmiavg = c->pmiavg;
    for (int i = 0; i < 3; i++) { r->qvol[i] = c->qvol[i]; r->tvol[i] = c->tvol[i]; r->cd[i] = c->cd[i]; r->heat_flux[i] = c->heat_flux[i]; }
    r->csgsts = c->csgsts; r->csgshf = c->csgshf;
    r->nutavg = c->nutavg; r->nutmax = c->nutmax; r->alpavg = c->alpavg; r->alpmax = c->alpmax;
    r->ubulk = c->ubulk; r->qflux = c->qflux; r->tbulk_fluid = c->tbulk_fluid; r->tbulk_solid = c->tbulk_solid;
    for (int i = 0; i < 3; i++) r->poisson_iters[i] = c->poisson_iters[i];
    r->poisson_unconverged = c->poisson_unconv;
    r->heat_body = c->heat_body;
    return 0;
}

int ref_get_fields(ref_case *c, double *u, double *v, double *w, double *p, double *t)
{
    if (!c) return LESGPU_ERR_ARG;
    if (u) memcpy(u, c->u, c->nt * sizeof(double));
    if (v) memcpy(v, c->v, c->nt * sizeof(double));
    if (w) memcpy(w, c->w, c->nt * sizeof(double));
    if (p) memcpy(p, c->p, c->nt * sizeof(double));
    if (t) memcpy(t, c->t, c->nt * sizeof(double));
    return 0;
}

static int field_ptrs(ref_case *c, int64_t f, double **ptr, int *ncomp)
{
    *ncomp = 1;
    switch (f) {
    case LESGPU_F_U: ptr[0] = c->u; return 0;
    case LESGPU_F_V: ptr[0] = c->v; return 0;
    case LESGPU_F_W: ptr[0] = c->w; return 0;
    case LESGPU_F_P: ptr[0] = c->p; return 0;
    case LESGPU_F_T: ptr[0] = c->t; return 0;
    case LESGPU_F_NUSGS: ptr[0] = c->nusgs; return 0;
    case LESGPU_F_ALSGS: ptr[0] = c->alsgs; return 0;
    case LESGPU_F_NUSGS1: *ncomp = 3; for (int l = 0; l < 3; l++) ptr[l] = c->nusgs1[l]; return 0;
    case LESGPU_F_ALSGS1: *ncomp = 3; for (int l = 0; l < 3; l++) ptr[l] = c->alsgs1[l]; return 0;
    case LESGPU_F_RHS1: *ncomp = 4; for (int l = 0; l < 4; l++) ptr[l] = c->rhs1[l]; return 0;
    case LESGPU_F_RK3O: *ncomp = 4; for (int l = 0; l < 4; l++) ptr[l] = c->rk3o[l]; return 0;
    case LESGPU_F_RK3OO: *ncomp = 4; for (int l = 0; l < 4; l++) ptr[l] = c->rk3oo[l]; return 0;
    case LESGPU_F_DIVGSUM: ptr[0] = c->divgsum; return 0;
    case LESGPU_F_PHI: ptr[0] = c->phi; return 0;
    case LESGPU_F_QMASS: ptr[0] = c->qmass; return 0;
    default: return LESGPU_ERR_ARG;
    }
}

int ref_get_array(ref_case *c, int64_t f, double *out)
{
    double *ptr[4]; int nc;
    if (!c || !out || field_ptrs(c, f, ptr, &nc)) return LESGPU_ERR_ARG;
    for (int l = 0; l < nc; l++) memcpy(out + (size_t)l * c->nt, ptr[l], c->nt * sizeof(double));
    return 0;
}

int ref_set_array(ref_case *c, int64_t f, const double *in)
{
    double *ptr[4]; int nc;
    if (!c || !in || field_ptrs(c, f, ptr, &nc)) return LESGPU_ERR_ARG;
    for (int l = 0; l < nc; l++) memcpy(ptr[l], in + (size_t)l * c->nt, c->nt * sizeof(double));
    return 0;
}

/* one reference subroutine group at a time, for phase-level parity */
int ref_run_phase(ref_case *c, int64_t phase, int64_t msub)
{
    const lesgpu_config *g = &c->c;
    switch (phase) {
    case LESGPU_PH_STEPINIT: ref_stepinit(c); c->subdt = 0.0; return 0;
    case LESGPU_PH_SUBSTEPINIT: ref_substepinit(c, msub); return 0;
    case LESGPU_PH_SGS:
        if (g->iles == 1) { ref_sgscalc(c); if (g->ihtrans == 1) ref_sgscalc_t(c); }
        return 0;
    case LESGPU_PH_RHSNLHS: ref_rhsnlhs(c); return 0;
    case LESGPU_PH_DIVGS:
        memset(c->divgsum, 0, c->nt * sizeof(double));
        ref_divgs(c); return 0;
    case LESGPU_PH_POISSON:
        memset(c->phi, 0, c->nt * sizeof(double));
        ref_poisson(c); return 0;
    case LESGPU_PH_UCALC:
        if (g->ich == 1) { c->qvol[2] = ref_qvolcalc(c); ref_qvolcorr(c); }
        ref_ucalc(c);
        if (g->ich == 1) c->qvol[0] = ref_qvolcalc(c);
        ref_pcalc(c);
        return 0;
    case LESGPU_PH_MEANPG: if (g->ich != 0) ref_meanpg(c); return 0;
    case LESGPU_PH_ENERGY:
        if (g->ihtrans == 1) {
            if (g->ich == 1) c->tvol[1] = ref_tvolcalc(c);
            ref_rhsnlhs_t(c);
            if (g->ich == 1) { c->tvol[2] = ref_tvolcalc(c); ref_tvolcorr(c); }
            ref_tcalc(c);
            if (g->ich == 1) c->tvol[0] = ref_tvolcalc(c);
        }
        return 0;
    default: return LESGPU_ERR_ARG;
    }
}

/* Thread count of the OpenMP loops (the stated core count of a CPU timing). */
int ref_set_threads(int n)
{
#ifdef _OPENMP
    if (n < 1) return -1;
    omp_set_num_threads(n);
    return 0;
#else
    return n == 1 ? 0 : -1;
#endif
}

int ref_get_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int ref_destroy(ref_case *c)
{
    if (!c) return 0;
    /* process-lifetime test helper: the few KB of vectors are released with
       the large arrays below */
    double *big[] = { c->fb_u, c->fb_c, c->u, c->v, c->w, c->p, c->t, c->nusgs, c->alsgs,
                      c->qmass, c->divgsum, c->phi, c->cstar, c->uout, c->vout, c->wout, c->tout,
                      c->duout, c->dvout, c->dwout, c->dtout };
    for (size_t q = 0; q < sizeof(big) / sizeof(big[0]); q++) free(big[q]);
    for (int l = 0; l < 4; l++) { free(c->rhs1[l]); free(c->rk3o[l]); free(c->rk3oo[l]); }
    for (int l = 0; l < 3; l++) { free(c->nusgs1[l]); free(c->alsgs1[l]); }
    for (int l = 0; l < 6; l++) free(c->kstar[l]);
    free(c->omega); free(c->nwall);
    free(c->ac); free(c->gam); free(c->bet);
    free(c->aw); free(c->ae); free(c->as); free(c->an); free(c->coi1); free(c->coi2); free(c->cor1); free(c->cor2);
    free(c->ipm); free(c->imm); free(c->ak1); free(c->ak3); free(c->avg);
    free(c->ab); free(c->af); free(c->fidw); free(c->fkdw); free(c->fiup); free(c->fkup);
    free(c->ih1); free(c->ih2); free(c->kh1); free(c->kh2); free(c->il1); free(c->il2); free(c->kl1); free(c->kl2);
    free(c->kpm); free(c->kmm);
    ref_fft_plan_free(&c->fftx); ref_fft_plan_free(&c->fftz);
    free(c);
    return 0;
}

/* ===================== slv_auxi.f90 ===================================== */

/* stepinit, slv_auxi.f90:2-50 */
void ref_stepinit(ref_case *c)
{
    const lesgpu_config *g = &c->c;
    c->ntime += 1;
    c->m = c->ntime;
    c->poisson_unconv = 0;
    c->heat_body = 0.0;
    for (int l = 0; l < 4; l++)
        for (ll n = 1; n <= c->nbody[l]; n++) c->fcvavg[l][n] = 0.0;
    if (g->ich != 0) c->pmiavg = 0.0;
    if (g->idtopt == 0) c->dt = g->dt_size;
    ref_cfl(c);
    if (g->idtopt != 0 && c->cflmax != 0.0) {
        double a = c->dt * g->cflfac / c->cflmax;
        double b = c->dt * (0.80 + 0.20 * g->cflfac / c->cflmax);
        double dtcfl = a < b ? a : b;
        if (g->idtopt == 1) c->dt = dtcfl;
    }
    double eps_t = 1.0e-12 * (fabs(c->time) > 1.0 ? fabs(c->time) : 1.0);
    double dt_evt = c->dt;
    if (g->ptb_tst > c->time + eps_t) dt_evt = fmin(dt_evt, g->ptb_tst - c->time);
    if (g->avg_tst > c->time + eps_t) dt_evt = fmin(dt_evt, g->avg_tst - c->time);
    if (g->tend > c->time + eps_t) dt_evt = fmin(dt_evt, g->tend - c->time);
    if (dt_evt < c->dt) c->dt = dt_evt;
}

/* cfl, slv_auxi.f90:53-102 */
void ref_cfl(ref_case *c)
{
    double cflm = 0.0;
    #pragma omp parallel for reduction(max:cflm)
    for (ll k = 1; k <= c->n3m; k++)
        for (ll j = 1; j <= c->n2m; j++)
            for (ll i = 1; i <= c->n1m; i++) {
                double c1 = fabs(c->u[IX(c, i, j, k)] + c->u[IX(c, i + 1, j, k)]) * 0.5 * c->f2fxi[i];
                double c2 = fabs(c->v[IX(c, i, j, k)] + c->v[IX(c, i, j + 1, k)]) * 0.5 * c->f2fyi[j];
                double c3 = fabs(c->w[IX(c, i, j, k)] + c->w[IX(c, i, j, k + 1)]) * 0.5 * c->f2fzi[k];
                double c0 = (c1 + c2 + c3) * c->dt;
                if (c0 >= cflm) cflm = c0;
            }
    c->cflmax = cflm;
}

/* substepinit, slv_auxi.f90:105-123 */
void ref_substepinit(ref_case *c, ll s)
{
    c->alpha = 0.5 * (c->gamma[s] + c->ro[s]);
    c->dtconst = c->dt * (c->gamma[s] + c->ro[s]);
    c->dtconsti = 1.0 / c->dtconst;
    c->test1 = c->c.resid1 * c->dtconsti;
    c->acoef = c->alpha * c->dt / c->c.re;
    c->acoefi = 1.0 / c->acoef;
    c->pmiavg = c->pmiavg + c->pmi[0] * 2.0 * c->alpha;
    c->subdt = c->subdt + c->dtconst;
    c->msub = s;
}

/* qvolcalc, slv_auxi.f90:126-149 */
double ref_qvolcalc(ref_case *c)
{
    double qq = 0.0;
    #pragma omp parallel for reduction(+:qq)
    for (ll k = 1; k <= c->n3m; k++)
        for (ll j = 1; j <= c->n2m; j++)
            for (ll i = 1; i <= c->n1m; i++)
                if (c->fb_u[IX(c, i, j, k)] >= 1.0e-10)
                    qq += c->u[IX(c, i, j, k)] * c->c2cx[i] * c->f2fy[j] * c->f2fz[k];
    return qq;
}

/* tvolcalc, slv_auxi.f90:152-173 (cstar defaults to 1 when ICONJG = 0) */
double ref_tvolcalc(ref_case *c)
{
    double qq = 0.0;
    #pragma omp parallel for reduction(+:qq)
    for (ll k = 1; k <= c->n3m; k++)
        for (ll j = 1; j <= c->n2m; j++)
            for (ll i = 1; i <= c->n1m; i++)
                qq += c->t[IX(c, i, j, k)] / c->cstar[IX(c, i, j, k)] * c->f2fx[i] * c->f2fy[j] * c->f2fz[k];
    return qq;
}

/* qvolcorr, slv_auxi.f90:176-203: the correction is disabled (phcap = 0) */
void ref_qvolcorr(ref_case *c) { c->phcap = 0.0; }

/* tvolcorr, slv_auxi.f90:206-230 */
void ref_tvolcorr(ref_case *c)
{
    double cvol = 0.0;
    #pragma omp parallel for reduction(+:cvol)
    for (ll k = 1; k <= c->n3m; k++)
        for (ll j = 1; j <= c->n2m; j++)
            for (ll i = 1; i <= c->n1m; i++)
                cvol += 1.0 / c->cstar[IX(c, i, j, k)] * c->f2fx[i] * c->f2fy[j] * c->f2fz[k];
    c->thcap = (c->tvol[2] - c->tvol[1]) / cvol;
}

/* ucalc, slv_auxi.f90:233-416 (the jut..kvb branches never fire: those flags
   are declared in mod_common.f90:22 but never assigned) */
void ref_ucalc(ref_case *c)
{
    ll n1 = c->n1, n2 = c->n2, n3 = c->n3, n1m = c->n1m, n2m = c->n2m, n3m = c->n3m;
    double dtc = c->dtconst;
    double *u = c->u, *v = c->v, *w = c->w, *phi = c->phi;
    #pragma omp parallel for
    for (ll k = 1; k <= n3m; k++)
        for (ll j = 1; j <= n2m; j++)
            for (ll i = c->i_bgpx; i <= n1m; i++) {
                ll im = c->imv[i];
                u[IX(c, i, j, k)] = u[IX(c, i, j, k)] - dtc * (phi[IX(c, i, j, k)] - phi[IX(c, im, j, k)]) * c->c2cxi[i];
            }
    #pragma omp parallel for
    for (ll k = 1; k <= n3m; k++)
        for (ll j = 2; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++)
                v[IX(c, i, j, k)] = v[IX(c, i, j, k)] - dtc * (phi[IX(c, i, j, k)] - phi[IX(c, i, j - 1, k)]) * c->c2cyi[j];
    #pragma omp parallel for
    for (ll k = c->k_bgpz; k <= n3m; k++) {
        ll km = c->kmv[k];
        for (ll j = 1; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++)
                w[IX(c, i, j, k)] = w[IX(c, i, j, k)] - dtc * (phi[IX(c, i, j, k)] - phi[IX(c, i, j, km)]) * c->c2czi[k];
    }
    if (c->c.zprdic == 1) {
        for (ll j = 0; j <= n2; j++)
            for (ll i = 1; i <= n1; i++) { u[IX(c, i, j, 0)] = u[IX(c, i, j, n3m)]; u[IX(c, i, j, n3)] = u[IX(c, i, j, 1)]; }
        for (ll j = 1; j <= n2; j++)
            for (ll i = 0; i <= n1; i++) { v[IX(c, i, j, 0)] = v[IX(c, i, j, n3m)]; v[IX(c, i, j, n3)] = v[IX(c, i, j, 1)]; }
        for (ll j = 0; j <= n2; j++)
            for (ll i = 0; i <= n1; i++) { w[IX(c, i, j, 0)] = w[IX(c, i, j, n3m)]; w[IX(c, i, j, n3)] = w[IX(c, i, j, 1)]; }
    }
    if (c->c.xprdic == 1) {
        for (ll k = 0; k <= n3; k++)
            for (ll j = 0; j <= n2; j++) { u[IX(c, 0, j, k)] = u[IX(c, n1m, j, k)]; u[IX(c, n1, j, k)] = u[IX(c, 1, j, k)]; }
        for (ll k = 0; k <= n3; k++)
            for (ll j = 1; j <= n2; j++) { v[IX(c, 0, j, k)] = v[IX(c, n1m, j, k)]; v[IX(c, n1, j, k)] = v[IX(c, 1, j, k)]; }
        for (ll k = 1; k <= n3; k++)
            for (ll j = 0; j <= n2; j++) { w[IX(c, 0, j, k)] = w[IX(c, n1m, j, k)]; w[IX(c, n1, j, k)] = w[IX(c, 1, j, k)]; }
    }
}

/* pcalc, slv_auxi.f90:419-493 */
void ref_pcalc(ref_case *c)
{
    ll n1 = c->n1, n3 = c->n3, n1m = c->n1m, n2m = c->n2m, n3m = c->n3m;
    double *p = c->p, *phi = c->phi, *dv = c->divgsum;
    double dtc = c->dtconst, re = c->c.re;
    #pragma omp parallel for
    for (ll k = 1; k <= n3m; k++)
        for (ll j = 1; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++)
                p[IX(c, i, j, k)] = p[IX(c, i, j, k)] + phi[IX(c, i, j, k)] - 0.5 * dtc * dv[IX(c, i, j, k)] * 1.0 / re;
    double phiref = 0.0;
    for (ll k = 1; k <= n3m; k++)
        for (ll j = 1; j <= n2m; j++)
            phiref = phi[IX(c, n1m, j, k)] * c->f2fy[j] * c->f2fz[k] + phiref;
    phiref = phiref / (c->yl * c->zl);
    #pragma omp parallel for
    for (ll k = 1; k <= n3m; k++)
        for (ll j = 1; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++)
                p[IX(c, i, j, k)] = p[IX(c, i, j, k)] - phiref;
    if (c->c.zprdic == 1)
        for (ll j = 1; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++) { p[IX(c, i, j, 0)] = p[IX(c, i, j, n3m)]; p[IX(c, i, j, n3)] = p[IX(c, i, j, 1)]; }
    if (c->c.xprdic == 1)
        for (ll k = 1; k <= n3m; k++)
            for (ll j = 1; j <= n2m; j++) { p[IX(c, 0, j, k)] = p[IX(c, n1m, j, k)]; p[IX(c, n1, j, k)] = p[IX(c, 1, j, k)]; }
}

/* tcalc, slv_auxi.f90:496-516 */
void ref_tcalc(ref_case *c)
{
    if (c->c.ich == 1 && c->c.xprdic == 0) {
        for (ll k = 1; k <= c->n3m; k++)
            for (ll j = 1; j <= c->n2m; j++)
                for (ll i = 1; i <= c->n1m; i++) c->t[IX(c, i, j, k)] -= c->thcap;
    }
}

/* lagforce, slv_auxi.f90:519-570 */
void ref_lagforce(ref_case *c)
{
    ll s = c->msub;
    if (s == 1) { c->dudta = 0.0; c->dvdta = 0.0; c->dwdta = 0.0; }
    double acc[3] = { 0.0, 0.0, 0.0 };
    for (int l = 0; l < 3; l++) {
        for (ll n = 1; n <= c->nbody[l]; n++) {
            ll ii = c->ifc[l][n], jj = c->jfc[l][n], kk = c->kfc[l][n];
            double vol = (l == 0) ? c->c2cx[ii] * c->f2fy[jj] * c->f2fz[kk]
                       : (l == 1) ? c->f2fx[ii] * c->c2cy[jj] * c->f2fz[kk]
                                  : c->f2fx[ii] * c->f2fy[jj] * c->c2cz[kk];
            size_t q = IX(c, ii, jj, kk);
            acc[l] += vol * (c->dudtr[l][n] - (c->gamma[s] * c->rk3o[l][q] + c->ro[s] * c->rk3oo[l][q]));
        }
    }
    c->dudta += acc[0]; c->dvdta += acc[1]; c->dwdta += acc[2];
}

/* heatflux, slv_auxi.f90:573-663 (history bookkeeping is host work) */
void ref_heatflux(ref_case *c)
{
    const lesgpu_body *b = &c->c.body;
    ll n1 = c->n1, n2 = c->n2, n3 = c->n3, n1m = c->n1m, n2m = c->n2m, n3m = c->n3m;
    double fxm = 0, fxp = 0, fym = 0, fyp = 0, fzm = 0, fzp = 0;
    double *t = c->t;
    for (ll k = 1; k <= n3m; k++)
        for (ll j = 1; j <= n2m; j++) {
            double area = c->f2fy[j] * c->f2fz[k];
            if (ref_funcbody(b, c->x[1], c->ymp[j], c->zmp[k]) >= 1.0e-10)
                fxm += c->u[IX(c, 1, j, k)] * (0.5 * (t[IX(c, 1, j, k)] + t[IX(c, 0, j, k)])) * area;
            if (ref_funcbody(b, c->x[n1], c->ymp[j], c->zmp[k]) >= 1.0e-10)
                fxp += c->u[IX(c, n1, j, k)] * (0.5 * (t[IX(c, n1m, j, k)] + t[IX(c, n1, j, k)])) * area;
        }
    for (ll k = 1; k <= n3m; k++)
        for (ll i = 1; i <= n1m; i++) {
            double area = c->f2fx[i] * c->f2fz[k];
            if (ref_funcbody(b, c->xmp[i], c->y[1], c->zmp[k]) >= 1.0e-10)
                fym += c->v[IX(c, i, 1, k)] * (0.5 * (t[IX(c, i, 1, k)] + t[IX(c, i, 0, k)])) * area;
            if (ref_funcbody(b, c->xmp[i], c->y[n2], c->zmp[k]) >= 1.0e-10)
                fyp += c->v[IX(c, i, n2, k)] * (0.5 * (t[IX(c, i, n2m, k)] + t[IX(c, i, n2, k)])) * area;
        }
    for (ll j = 1; j <= n2m; j++)
        for (ll i = 1; i <= n1m; i++) {
            double area = c->f2fx[i] * c->f2fy[j];
            if (ref_funcbody(b, c->xmp[i], c->ymp[j], c->z[1]) >= 1.0e-10)
                fzm += c->w[IX(c, i, j, 1)] * (0.5 * (t[IX(c, i, j, 1)] + t[IX(c, i, j, 0)])) * area;
            if (ref_funcbody(b, c->xmp[i], c->ymp[j], c->z[n3]) >= 1.0e-10)
                fzp += c->w[IX(c, i, j, n3)] * (0.5 * (t[IX(c, i, j, n3m)] + t[IX(c, i, j, n3)])) * area;
        }
    c->heat_flux[0] = fxp - fxm; c->heat_flux[1] = fyp - fym; c->heat_flux[2] = fzp - fzm;
}

/* draglift, slv_auxi.f90:666-840 (instantaneous force; averaging is host work) */
void ref_draglift(ref_case *c)
{
    ll n1m = c->n1m, n2m = c->n2m, n3m = c->n3m, n2 = c->n2, n3 = c->n3;
    double cd[3] = { 0, 0, 0 };
    const lesgpu_config *g = &c->c;
    for (int l = 0; l < 3; l++)
        for (ll n = 1; n <= c->nbody[l]; n++) {
            ll ii = c->ifc[l][n], jj = c->jfc[l][n], kk = c->kfc[l][n];
            cd[l] = cd[l] - c->fcvavg[l][n] * (c->c2cx[ii] * c->f2fy[jj] * c->f2fz[kk]);
        }
    cd[0] += c->dudta; cd[1] += c->dvdta; cd[2] += c->dwdta;
    /* the thermal forcing's heat rate, with the cell-centre volume of the T points */
    double hb = 0.0;
    if (g->ihtrans == 1)
        for (ll n = 1; n <= c->nbody[3]; n++) {
            ll ii = c->ifc[3][n], jj = c->jfc[3][n], kk = c->kfc[3][n];
            hb = hb + c->fcvavg[3][n] * (c->f2fx[ii] * c->f2fy[jj] * c->f2fz[kk]);
        }
    c->heat_body = hb;
    double *u = c->u, *v = c->v, *w = c->w, re = g->re;
    if (g->bc_ybtm == 0) {
        double dy1 = 1.0 / c->c2cyi[1], dy2 = dy1 + 1.0 / c->c2cyi[2];
        for (ll k = 1; k <= n3m; k++)
            for (ll i = 1; i <= n1m; i++)
                if (c->fb_u[IX(c, i, 1, k)] >= 1.0e-10) {
                    double gu = (u[IX(c, i, 1, k)] * dy2 * dy2 - u[IX(c, i, 2, k)] * dy1 * dy1) / (dy1 * dy2 * (dy2 - dy1));
                    cd[0] += gu * c->c2cx[i] * c->f2fz[k] / re;
                    double gw = (w[IX(c, i, 1, k)] * dy2 * dy2 - w[IX(c, i, 2, k)] * dy1 * dy1) / (dy1 * dy2 * (dy2 - dy1));
                    cd[2] += gw * c->c2cx[i] * c->f2fz[k] / re;
                }
    }
    if (g->bc_ytop == 0) {
        double dy1 = 1.0 / c->c2cyi[n2], dy2 = dy1 + 1.0 / c->c2cyi[n2m];
        for (ll k = 1; k <= n3m; k++)
            for (ll i = 1; i <= n1m; i++)
                if (c->fb_u[IX(c, i, n2m, k)] >= 1.0e-10) {
                    double gu = (u[IX(c, i, n2m, k)] * dy2 * dy2 - u[IX(c, i, n2m - 1, k)] * dy1 * dy1) / (dy1 * dy2 * (dy2 - dy1));
                    cd[0] += gu * c->c2cx[i] * c->f2fz[k] / re;
                    double gw = (w[IX(c, i, n2m, k)] * dy2 * dy2 - w[IX(c, i, n2m - 1, k)] * dy1 * dy1) / (dy1 * dy2 * (dy2 - dy1));
                    cd[2] += gw * c->c2cx[i] * c->f2fz[k] / re;
                }
    }
    if (g->bc_zbtm == 0) {
        double dz1 = 1.0 / c->c2czi[1], dz2 = dz1 + 1.0 / c->c2czi[2];
        for (ll j = 1; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++)
                if (c->fb_u[IX(c, i, j, 1)] >= 1.0e-10) {
                    double gu = (u[IX(c, i, j, 1)] * dz2 * dz2 - u[IX(c, i, j, 2)] * dz1 * dz1) / (dz1 * dz2 * (dz2 - dz1));
                    cd[0] += gu * c->c2cx[i] * c->f2fy[j] / re;
                    double gv = (v[IX(c, i, j, 1)] * dz2 * dz2 - v[IX(c, i, j, 2)] * dz1 * dz1) / (dz1 * dz2 * (dz2 - dz1));
                    cd[1] += gv * c->c2cx[i] * c->f2fy[j] / re;
                }
    }
    if (g->bc_ztop == 0) {
        double dz1 = 1.0 / c->c2czi[n3], dz2 = dz1 + 1.0 / c->c2czi[n3m];
        for (ll j = 1; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++)
                if (c->fb_u[IX(c, i, j, n3m)] >= 1.0e-10) {
                    double gu = (u[IX(c, i, j, n3m)] * dz2 * dz2 - u[IX(c, i, j, n3m - 1)] * dz1 * dz1) / (dz1 * dz2 * (dz2 - dz1));
                    cd[0] += gu * c->c2cx[i] * c->f2fy[j] / re;
                    double gv = (v[IX(c, i, j, n3m)] * dz2 * dz2 - v[IX(c, i, j, n3m - 1)] * dz1 * dz1) / (dz1 * dz2 * (dz2 - dz1));
                    cd[1] += gv * c->c2cx[i] * c->f2fy[j] / re;
                }
    }
    double vol = c->xl * c->yl * c->zl;
    for (int l = 0; l < 3; l++) c->cd[l] = cd[l] / vol;
}

/* ===================== misc_init.f90 ==================================== */

/* convergence_check, misc_init.f90:1047-1077 */
void ref_convergence_check(ref_case *c)
{
    double dvmax = 0.0;
    int masson = (int)c->c.masson;
    #pragma omp parallel for reduction(max:dvmax)
    for (ll k = 1; k <= c->n3m; k++)
        for (ll j = 1; j <= c->n2m; j++)
            for (ll i = 1; i <= c->n1m; i++) {
                double d1 = (c->u[IX(c, i + 1, j, k)] - c->u[IX(c, i, j, k)]) * c->f2fxi[i];
                double d2 = (c->v[IX(c, i, j + 1, k)] - c->v[IX(c, i, j, k)]) * c->f2fyi[j];
                double d3 = (c->w[IX(c, i, j, k + 1)] - c->w[IX(c, i, j, k)]) * c->f2fzi[k];
                double dv = (masson == 1) ? d1 + d2 + d3 - c->qmass[IX(c, i, j, k)] : d1 + d2 + d3;
                if (fabs(dv) > dvmax) dvmax = fabs(dv);
            }
    c->dvmax = dvmax;
}

/* masscheck, misc_init.f90:1080-1104 */
void ref_masscheck(ref_case *c)
{
    double q = 0.0;
    for (ll k = 1; k <= c->n3m; k++)
        for (ll j = 1; j <= c->n2m; j++)
            for (ll i = 1; i <= c->n1m; i++)
                if (fabs(c->qmass[IX(c, i, j, k)]) > q) q = fabs(c->qmass[IX(c, i, j, k)]);
    c->qmmax = q;
}

/* bulk quantities of writehistory, misc_hist.f90:73-181 */
void ref_bulk_diag(ref_case *c)
{
    double qv = 0, fv = 0, tfv = 0, tsv = 0, tfi = 0, tsi = 0;
    for (ll k = 1; k <= c->n3m; k++)
        for (ll j = 1; j <= c->n2m; j++)
            for (ll i = 1; i <= c->n1m; i++) {
                double cv = c->c2cx[i] * c->f2fy[j] * c->f2fz[k];
                if (c->fb_u[IX(c, i, j, k)] >= 1.0e-10) { qv += c->u[IX(c, i, j, k)] * cv; fv += cv; }
                if (c->c.ihtrans == 1) {
                    if (c->fb_c[IX(c, i, j, k)] >= 1.0e-10) { tfv += cv; tfi += c->t[IX(c, i, j, k)] * cv; }
                    else { tsv += cv; tsi += c->t[IX(c, i, j, k)] * cv; }
                }
            }
    c->ubulk = fv > 0 ? qv / fv : 0.0;
    c->qflux = qv / c->xl;
    c->tbulk_fluid = tfv > 0 ? tfi / tfv : 0.0;
    c->tbulk_solid = tsv > 0 ? tsi / tsv : 0.0;
}

/* ===================== misc_hist.f90 ==================================== */

/* field_avg, misc_hist.f90:287-527: running sums of dt-weighted cell-centre
   statistics once time > AVG_TST.  The fav file write and the reset every
   NPRIAVG samples are host work (ref_get_averages). */
void ref_field_avg(ref_case *c)
{
    const lesgpu_config *g = &c->c;
    if (c->time <= g->avg_tst) return;
    size_t nt = c->nt;
    if (!c->avg) c->avg = ref_zalloc(nt * LESGPU_NAVG);
    double *A[LESGPU_NAVG];
    for (int q = 0; q < LESGPU_NAVG; q++) A[q] = c->avg + nt * (size_t)q;
    double dt = c->dt;
    const double *u = c->u, *v = c->v, *w = c->w, *p = c->p, *t = c->t;
    ll n1 = c->n1, n2 = c->n2, n3 = c->n3;
    #pragma omp parallel for
    for (ll k = 1; k <= c->n3m; k++)
        for (ll j = 1; j <= c->n2m; j++)
            for (ll i = 1; i <= c->n1m; i++) {
                size_t q = IX(c, i, j, k);
                double ucc = 0.5 * (u[q] + u[IX(c, i + 1, j, k)]);
                double vcc = 0.5 * (v[q] + v[IX(c, i, j + 1, k)]);
                double wcc = 0.5 * (w[q] + w[IX(c, i, j, k + 1)]);
                A[0][q] = A[0][q] + ucc * dt;
                A[1][q] = A[1][q] + vcc * dt;
                A[2][q] = A[2][q] + wcc * dt;
                A[3][q] = A[3][q] + ucc * ucc * dt;
                A[4][q] = A[4][q] + ucc * vcc * dt;
                A[5][q] = A[5][q] + ucc * wcc * dt;
                A[6][q] = A[6][q] + vcc * vcc * dt;
                A[7][q] = A[7][q] + vcc * wcc * dt;
                A[8][q] = A[8][q] + wcc * wcc * dt;
                A[9][q] = A[9][q] + p[q] * dt;
                A[10][q] = A[10][q] + p[q] * p[q] * dt;
                if (g->ihtrans == 1) {
                    A[21][q] = A[21][q] + t[q] * dt;
                    A[22][q] = A[22][q] + t[q] * t[q] * dt;
                }
                /* velocity gradients at the cell centre (misc_hist.f90:379-455) */
                double fju = (double)c->fixju[j], fjl = (double)c->fixjl[j];
                double fku = (double)c->fixku[k], fkl = (double)c->fixkl[k];
                double fiu = (double)c->fixiu[i], fil = (double)c->fixil[i];
                double vg11 = c->f2fxi[i] * (u[IX(c, i + 1, j, k)] - u[q]);
                double up = c->c2cyi[j + 1] * 0.25 * (c->f2fy[j + 1] * (u[q] + u[IX(c, i + 1, j, k)])
                            + c->f2fy[j] * (u[IX(c, i, j + 1, k)] + u[IX(c, i + 1, j + 1, k)])) * (1. - fju)
                            + 0.5 * (u[IX(c, i, n2, k)] + u[IX(c, i + 1, n2, k)]) * fju;
                double um = c->c2cyi[j] * 0.25 * (c->f2fy[j] * (u[IX(c, i, j - 1, k)] + u[IX(c, i + 1, j - 1, k)])
                            + c->f2fy[j - 1] * (u[q] + u[IX(c, i + 1, j, k)])) * (1. - fjl)
                            + 0.5 * (u[IX(c, i, 0, k)] + u[IX(c, i + 1, 0, k)]) * fjl;
                double vg12 = c->f2fyi[j] * (up - um);
                up = c->c2czi[k + 1] * 0.25 * (c->f2fz[k + 1] * (u[q] + u[IX(c, i + 1, j, k)])
                     + c->f2fz[k] * (u[IX(c, i, j, k + 1)] + u[IX(c, i + 1, j, k + 1)])) * (1. - fku)
                     + 0.5 * (u[IX(c, i, j, n3)] + u[IX(c, i + 1, j, n3)]) * fku;
                um = c->c2czi[k] * 0.25 * (c->f2fz[k] * (u[IX(c, i, j, k - 1)] + u[IX(c, i + 1, j, k - 1)])
                     + c->f2fz[k - 1] * (u[q] + u[IX(c, i + 1, j, k)])) * (1. - fkl)
                     + 0.5 * (u[IX(c, i, j, 0)] + u[IX(c, i + 1, j, 0)]) * fkl;
                double vg13 = c->f2fzi[k] * (up - um);
                double vp = c->c2cxi[i + 1] * 0.25 * (c->f2fx[i + 1] * (v[q] + v[IX(c, i, j + 1, k)])
                            + c->f2fx[i] * (v[IX(c, i + 1, j, k)] + v[IX(c, i + 1, j + 1, k)])) * (1. - fiu)
                            + 0.5 * (v[IX(c, n1, j, k)] + v[IX(c, n1, j + 1, k)]) * fiu;
                double vm = c->c2cxi[i] * 0.25 * (c->f2fx[i] * (v[IX(c, i - 1, j, k)] + v[IX(c, i - 1, j + 1, k)])
                            + c->f2fx[i - 1] * (v[q] + v[IX(c, i, j + 1, k)])) * (1. - fil)
                            + 0.5 * (v[IX(c, 0, j, k)] + v[IX(c, 0, j + 1, k)]) * fil;
                double vg21 = c->f2fxi[i] * (vp - vm);
                double vg22 = c->f2fyi[j] * (v[IX(c, i, j + 1, k)] - v[q]);
                vp = c->c2czi[k + 1] * 0.25 * (c->f2fz[k + 1] * (v[q] + v[IX(c, i, j + 1, k)])
                     + c->f2fz[k] * (v[IX(c, i, j, k + 1)] + v[IX(c, i, j + 1, k + 1)])) * (1. - fku)
                     + 0.5 * (v[IX(c, i, j, n3)] + v[IX(c, i, j + 1, n3)]) * fku;
                vm = c->c2czi[k] * 0.25 * (c->f2fz[k] * (v[IX(c, i, j, k - 1)] + v[IX(c, i, j + 1, k - 1)])
                     + c->f2fz[k - 1] * (v[q] + v[IX(c, i, j + 1, k)])) * (1. - fkl)
                     + 0.5 * (v[IX(c, i, j, 0)] + v[IX(c, i, j + 1, 0)]) * fkl;
                double vg23 = c->f2fzi[k] * (vp - vm);
                double wp = c->c2cxi[i + 1] * 0.25 * (c->f2fx[i + 1] * (w[q] + w[IX(c, i, j, k + 1)])
                            + c->f2fx[i] * (w[IX(c, i + 1, j, k)] + w[IX(c, i + 1, j, k + 1)])) * (1. - fiu)
                            + 0.5 * (w[IX(c, n1, j, k)] + w[IX(c, n1, j, k + 1)]) * fiu;
                double wm = c->c2cxi[i] * 0.25 * (c->f2fx[i] * (w[IX(c, i - 1, j, k)] + w[IX(c, i - 1, j, k + 1)])
                            + c->f2fx[i - 1] * (w[q] + w[IX(c, i, j, k + 1)])) * (1. - fil)
                            + 0.5 * (w[IX(c, 0, j, k)] + w[IX(c, 0, j, k + 1)]) * fil;
                double vg31 = c->f2fxi[i] * (wp - wm);
                wp = c->c2cyi[j + 1] * 0.25 * (c->f2fy[j + 1] * (w[q] + w[IX(c, i, j, k + 1)])
                     + c->f2fy[j] * (w[IX(c, i, j + 1, k)] + w[IX(c, i, j + 1, k + 1)])) * (1. - fju)
                     + 0.5 * (w[IX(c, i, n2, k)] + w[IX(c, i, n2, k + 1)]) * fju;
                wm = c->c2cyi[j] * 0.25 * (c->f2fy[j] * (w[IX(c, i, j - 1, k)] + w[IX(c, i, j - 1, k + 1)])
                     + c->f2fy[j - 1] * (w[q] + w[IX(c, i, j, k + 1)])) * (1. - fjl)
                     + 0.5 * (w[IX(c, i, 0, k)] + w[IX(c, i, 0, k + 1)]) * fjl;
                double vg32 = c->f2fyi[j] * (wp - wm);
                double vg33 = c->f2fzi[k] * (w[IX(c, i, j, k + 1)] - w[q]);
                double s1 = vg11, s2 = 0.5 * (vg12 + vg21), s3 = 0.5 * (vg13 + vg31);
                double s4 = vg22, s5 = 0.5 * (vg23 + vg32), s6 = vg33;
                double wx = vg32 - vg23, wy = vg13 - vg31, wz = vg21 - vg12;
                A[11][q] = A[11][q] + wx * dt;
                A[12][q] = A[12][q] + wy * dt;
                A[13][q] = A[13][q] + wz * dt;
                A[14][q] = A[14][q] + wx * wx * dt;
                A[15][q] = A[15][q] + wx * wy * dt;
                A[16][q] = A[16][q] + wx * wz * dt;
                A[17][q] = A[17][q] + wy * wy * dt;
                A[18][q] = A[18][q] + wy * wz * dt;
                A[19][q] = A[19][q] + wz * wz * dt;
                double srsr = 2. * (s2 * s2) + s1 * s1 + 2. * (s3 * s3) + s4 * s4 + 2. * (s5 * s5) + s6 * s6;
                A[20][q] = A[20][q] + srsr * dt;
            }
    c->avg_count += 1;
}

int ref_get_averages(ref_case *c, double *out, int64_t *nsamples, int reset)
{
    if (!c) return LESGPU_ERR_ARG;
    int na = c->c.ihtrans == 1 ? LESGPU_NAVG : LESGPU_NAVG - 2;
    ll n1m = c->n1m, n2m = c->n2m, n3m = c->n3m;
    size_t nc = (size_t)n1m * n2m * n3m;
    if (out)
        for (int a = 0; a < na; a++)
            for (ll k = 1; k <= n3m; k++)
                for (ll j = 1; j <= n2m; j++)
                    for (ll i = 1; i <= n1m; i++)
                        out[nc * a + (size_t)(i - 1) + (size_t)n1m * ((size_t)(j - 1) + (size_t)n2m * (size_t)(k - 1))] =
                            c->avg ? c->avg[c->nt * (size_t)a + IX(c, i, j, k)] : 0.0;
    if (nsamples) *nsamples = c->avg_count;
    if (reset) {
        if (c->avg) memset(c->avg, 0, sizeof(double) * c->nt * LESGPU_NAVG);
        c->avg_count = 0;
    }
    return 0;
}
