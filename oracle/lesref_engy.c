/*
 * ORACLE -- test infrastructure only (see lesref_internal.h).
 *
 * Temperature equation: 02_solver/f90/lib/slv_engy.f90.
 */
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "lesref_internal.h"

double ref_ibm_target(const ref_case *c, int l, ll n, const double *fld, const double *rtmp);

#define PL(c, j, k) ((size_t)(j) + (size_t)((c)->n2 + 1) * (size_t)(k))

/* rhs_t, slv_engy.f90:29-198 (rhssgs_t, sgs.f90:1776, zeroes rhs1(:,:,:,4)
   first; its stress terms are identically zero for the linear model) */
static void rhs_t(ref_case *c)
{
    const lesgpu_config *g = &c->c;
    ll n1 = c->n1, n1m = c->n1m, n2m = c->n2m, n3m = c->n3m;
    ll s = c->msub;
    double *t = c->t, *u = c->u, *v = c->v, *w = c->w, *r4 = c->rhs1[3];
    double u_bulk = 1.0;
    if (g->idecomp == 1) {
        double fv = 0.0, qv = 0.0;
        #pragma omp parallel for reduction(+:fv, qv)
        for (ll k = 1; k <= n3m; k++)
            for (ll j = 1; j <= n2m; j++)
                for (ll i = 1; i <= n1m; i++)
                    if (c->fb_c[IX(c, i, j, k)] >= 1.0e-10) {
                        double cv = c->c2cx[i] * c->f2fy[j] * c->f2fz[k];
                        double ucc = 0.5 * (u[IX(c, i, j, k)] + u[IX(c, i + 1, j, k)]);
                        fv += cv;
                        qv += ucc * cv;
                    }
        if (fv > 1.0e-12) u_bulk = qv / fv;
        else if (fabs(g->udrv_i) > 1.0e-12) u_bulk = g->udrv_i;
        else u_bulk = 1.0;
    }
    double gam = c->gamma[s], ro = c->ro[s], alpha = c->alpha, dt = c->dt;
    double inv_repr = 1.0 / (g->re * g->pr);
    int iconjg = (int)g->iconjg, iles = (int)g->iles;
    #pragma omp parallel for
    for (ll k = 1; k <= n3m; k++)
        for (ll j = 1; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++) {
                size_t q = IX(c, i, j, k);
                ll kp = c->kpv[k], km = c->kmv[k], jp = c->jpv[j], jm = c->jmv[j], ip = c->ipv[i], im = c->imv[i];
                if (g->xprdic == 1 && g->idecomp == 0) {
                    if (i == n1m) ip = n1;
                    if (i == 1) im = 0;
                }
                double fiu = (double)c->fixiu[i], fil = (double)c->fixil[i], fju = (double)c->fixju[j], fjl = (double)c->fixjl[j];
                double fku = (double)c->fixku[k], fkl = (double)c->fixkl[k];
                double tq = t[q];
                double tip = t[IX(c, ip, j, k)], tim = t[IX(c, im, j, k)];
                double tjp = t[IX(c, i, jp, k)], tjm = t[IX(c, i, jm, k)];
                double tkp = t[IX(c, i, j, kp)], tkm = t[IX(c, i, j, km)];
                double te = 0.5 * (c->f2fx[i] * tip + c->f2fx[ip] * tq) * c->c2cxi[ip] * (1.0 - fiu) + tip * fiu;
                double tw = 0.5 * (c->f2fx[im] * tq + c->f2fx[i] * tim) * c->c2cxi[i] * (1.0 - fil) + tim * fil;
                double tn = 0.5 * (c->f2fy[j] * tjp + c->f2fy[jp] * tq) * c->c2cyi[jp] * (1.0 - fju) + tjp * fju;
                double ts = 0.5 * (c->f2fy[jm] * tq + c->f2fy[j] * tjm) * c->c2cyi[j] * (1.0 - fjl) + tjm * fjl;
                double tc = 0.5 * (c->f2fz[k] * tkp + c->f2fz[kp] * tq) * c->c2czi[kp] * (1.0 - fku) + tkp * fku;
                double tf = 0.5 * (c->f2fz[km] * tq + c->f2fz[k] * tkm) * c->c2czi[k] * (1.0 - fkl) + tkm * fkl;
                double ant1 = (te * u[IX(c, ip, j, k)] - tw * u[q]) * c->f2fxi[i];
                double ant2 = (tn * v[IX(c, i, jp, k)] - ts * v[q]) * c->f2fyi[j];
                double ant3 = (tc * w[IX(c, i, j, kp)] - tf * w[q]) * c->f2fzi[k];
                double omega = (iconjg == 1 && g->imovingon == 0) ? (double)c->omega[q] : 1.0;
                double src = 0.0;
                if (g->idecomp == 1) {
                    double ucc = 0.5 * (u[q] + u[IX(c, i + 1, j, k)]);
                    src = omega * (ucc / u_bulk);
                }
                double rk3t = -omega * (ant1 + ant2 + ant3) + src;
                double a1 = (tip - tq) * c->c2cxi[ip];
                double a2 = (tq - tim) * c->c2cxi[i];
                double a3 = (tjp - tq) * c->c2cyi[jp];
                double a4 = (tq - tjm) * c->c2cyi[j];
                double a5 = (tkp - tq) * c->c2czi[kp];
                double a6 = (tq - tkm) * c->c2czi[k];
                double altx, alty, altz;
                if (iconjg == 1) {
                    double cs = c->cstar[q];
                    altx = cs * (c->kstar[0][q] * a1 - c->kstar[1][q] * a2) * c->f2fxi[i];
                    alty = cs * (c->kstar[2][q] * a3 - c->kstar[3][q] * a4) * c->f2fyi[j];
                    altz = cs * (c->kstar[4][q] * a5 - c->kstar[5][q] * a6) * c->f2fzi[k];
                } else {
                    altx = (a1 - a2) * c->f2fxi[i];
                    alty = (a3 - a4) * c->f2fyi[j];
                    altz = (a5 - a6) * c->f2fzi[k];
                }
                double alt = inv_repr * (altx + alty + altz);
                if (iles == 1) {
                    double tx = c->f2fxi[i] * (c->alsgs1[0][IX(c, ip, j, k)] * c->c2cxi[ip] * (tip - tq)
                                              - c->alsgs1[0][q] * c->c2cxi[i] * (tq - tim));
                    double ty = c->f2fyi[j] * (c->alsgs1[1][IX(c, i, jp, k)] * c->c2cyi[jp] * (tjp - tq)
                                              - c->alsgs1[1][q] * c->c2cyi[j] * (tq - tjm));
                    double tz = c->f2fzi[k] * (c->alsgs1[2][IX(c, i, j, kp)] * c->c2czi[kp] * (tkp - tq)
                                              - c->alsgs1[2][q] * c->c2czi[k] * (tq - tkm));
                    alt = alt + omega * (tx + ty + tz);
                    rk3t = rk3t + omega * 0.0;   /* rhs1(:,:,:,4) holds rhssgs_t = 0 */
                }
                r4[q] = dt * (gam * rk3t + ro * c->rk3o[3][q] + 2.0 * alpha * alt);
                c->rk3oo[3][q] = c->rk3o[3][q];
                c->rk3o[3][q] = rk3t;
            }
    (void)n1;
}

/* rhs_ibm_t, slv_engy.f90:201-306 (target temperature tbody = 0) */
static void rhs_ibm_t(ref_case *c)
{
    double dti = 1.0 / c->dt;
    double *r = c->rhs1[3];
    double *tmp = ref_zalloc(c->nt);
    for (ll k = 1; k <= c->n3m; k++)
        for (ll j = 1; j <= c->n2m; j++)
            for (ll i = 1; i <= c->n1m; i++) tmp[IX(c, i, j, k)] = r[IX(c, i, j, k)];
    for (ll n = 1; n <= c->nintp[3]; n++) {
        double targ = ref_ibm_target(c, 3, n, c->t, tmp);
        size_t q = IX(c, c->ifc[3][n], c->jfc[3][n], c->kfc[3][n]);
        c->fcv[3][n] = (targ - c->t[q] - tmp[q]) * dti;
        r[q] = targ - c->t[q];
    }
    free(tmp);
    for (ll n = c->nintp[3] + 1; n <= c->nbody[3]; n++) {
        size_t q = IX(c, c->ifc[3][n], c->jfc[3][n], c->kfc[3][n]);
        double targ = 0.0;
        c->fcv[3][n] = (targ - c->t[q] - r[q]) * dti;
        r[q] = targ - c->t[q];
    }
    for (ll n = 1; n <= c->nbody[3]; n++) c->fcvavg[3][n] += c->fcv[3][n];
}

/* convbc_t, slv_engy.f90:309-413 */
static void convbc_t(ref_case *c)
{
    const lesgpu_config *g = &c->c;
    ll n1 = c->n1, n2 = c->n2, n3 = c->n3, n1m = c->n1m, n2m = c->n2m, n3m = c->n3m;
    double *u = c->u, *v = c->v, *w = c->w, *t = c->t;
    if (g->ich != 1) {
        double qin = 0.0;
        for (ll k = 1; k <= n3m; k++)
            for (ll j = 1; j <= n2m; j++) qin = u[IX(c, 1, j, k)] * c->f2fy[j] * c->f2fz[k] + qin;
        for (ll k = 1; k <= n3m; k++)
            for (ll i = 1; i <= n1m; i++) qin = (v[IX(c, i, 1, k)] - v[IX(c, i, n2, k)]) * c->f2fx[i] * c->f2fz[k] + qin;
        for (ll j = 1; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++) qin = (w[IX(c, i, j, 1)] - w[IX(c, i, j, n3)]) * c->f2fx[i] * c->f2fy[j] + qin;
        double ubar = 0.0;
        for (ll k = 1; k <= n3m; k++)
            for (ll j = 1; j <= n2m; j++) ubar = u[IX(c, n1, j, k)] * c->f2fy[j] * c->f2fz[k] + ubar;
        ubar = ubar / (c->yl * c->zl);
        double ucoef = ubar * c->dtconst * c->f2fxi[n1m];
        double vwcoef = ubar * c->dtconst * c->c2cxi[n1];
        double qout = 0.0;
        for (ll k = 1; k <= n3m; k++)
            for (ll j = 1; j <= n2m; j++) {
                size_t pq = PL(c, j, k);
                double uo = u[IX(c, n1, j, k)] - ucoef * (u[IX(c, n1, j, k)] - u[IX(c, n1m, j, k)]);
                if (c->fb_c[IX(c, n1m, j, k)] <= 1.0e-10 && g->imovingon == 0)
                    c->tout[pq] = t[IX(c, n1m, j, k)];
                else
                    c->tout[pq] = t[IX(c, n1, j, k)] - vwcoef * (t[IX(c, n1, j, k)] - t[IX(c, n1m, j, k)]);
                qout = uo * c->f2fy[j] * c->f2fz[k] + qout;
            }
        double qratio = fabs(qout) > 1.0e-14 ? qin / qout : 1.0;
        for (ll k = 1; k <= n3m; k++)
            for (ll j = 1; j <= n2m; j++) {
                size_t pq = PL(c, j, k);
                if (c->fb_c[IX(c, n1m, j, k)] > 1.0e-10) c->tout[pq] *= qratio;
                c->dtout[pq] = c->tout[pq] - t[IX(c, n1, j, k)];
            }
        if (g->yprdic == 1)
            for (ll k = 0; k <= n3; k++) { c->dtout[PL(c, n2, k)] = c->dtout[PL(c, 1, k)]; c->dtout[PL(c, 0, k)] = c->dtout[PL(c, n2m, k)]; }
        if (g->zprdic == 1)
            for (ll j = 0; j <= n2; j++) { c->dtout[PL(c, j, n3)] = c->dtout[PL(c, j, 1)]; c->dtout[PL(c, j, 0)] = c->dtout[PL(c, j, n3m)]; }
    } else {
        memset(c->tout, 0, (size_t)(n2 + 1) * (size_t)(n3 + 1) * sizeof(double));
    }
}

/* rhsincorpbc_t, slv_engy.f90:416-457 */
static void rhsincorpbc_t(ref_case *c)
{
    const lesgpu_config *g = &c->c;
    ll n1m = c->n1m, n2m = c->n2m, n3m = c->n3m;
    double cre2 = g->iles == 1 ? 2.0 * g->re * g->pr : 0.0;
    for (ll k = 1; k <= n3m; k++)
        for (ll j = 1; j <= n2m; j++) {
            size_t q = IX(c, n1m, j, k);
            double cs = 1.0, ks = 1.0, omc = 1.0;
            if (g->iconjg == 1) {
                cs = c->cstar[q];
                ks = (c->kstar[0][q] + c->kstar[1][q] + c->kstar[2][q] + c->kstar[3][q] + c->kstar[4][q] + c->kstar[5][q]) / 6.0;
                omc = g->imovingon == 0 ? (double)c->omega[q] : 1.0;
            }
            c->rhs1[3][q] -= c->acoef * cs * ks * c->ciu[n1m] * (1.0 + cre2 * omc * c->alsgs[q]) * c->dtout[PL(c, j, k)];
        }
}

/* lhs_t, slv_engy.f90:460-609 */
static void lhs_t(ref_case *c)
{
    const lesgpu_config *g = &c->c;
    ll n1 = c->n1, n2 = c->n2, n3 = c->n3, n1m = c->n1m, n2m = c->n2m, n3m = c->n3m;
    double cre = (double)g->iles * g->re * g->pr;
    double api = c->acoefi * g->pr;
    double *r4 = c->rhs1[3];
    int iconjg = (int)g->iconjg;
#define CSK(q, ka) double cs = 1.0, ks1 = 1.0, ks2 = 1.0, omc = 1.0; \
    if (iconjg == 1) { cs = c->cstar[q]; ks1 = c->kstar[(ka)][q]; ks2 = c->kstar[(ka) - 1][q]; \
                       omc = g->imovingon == 0 ? (double)c->omega[q] : 1.0; }
    if (n3m != 1) {
        ll ld = n1 + 1;
        #pragma omp parallel
        {
            double *A = ref_zalloc((size_t)ld * (n3 + 2)), *B = ref_zalloc((size_t)ld * (n3 + 2));
            double *C = ref_zalloc((size_t)ld * (n3 + 2)), *R = ref_zalloc((size_t)ld * (n3 + 2));
            #pragma omp for
            for (ll j = 1; j <= n2m; j++) {
                for (ll k = 1; k <= n3m; k++)
                    for (ll i = 1; i <= n1m; i++) {
                        size_t q = IX(c, i, j, k);
                        CSK(q, 5)
                        size_t p = (size_t)i + (size_t)ld * (size_t)k;
                        A[p] = c->akuv[k] * (cs * ks1 + cre * omc * c->alsgs1[1][q]);
                        C[p] = c->ckuv[k] * (cs * ks2 + cre * omc * c->alsgs1[1][IX(c, i, j, k + 1)]);
                        B[p] = api - A[p] - C[p];
                        R[p] = api * r4[q];
                    }
                if (g->zprdic == 0) ref_trdiag(A, B, C, R, 1, n3m, 1, n1m, ld);
                else ref_trdiagp(A, B, C, R, 1, n3m, 1, n1m, ld);
                for (ll k = 1; k <= n3m; k++)
                    for (ll i = 1; i <= n1m; i++) r4[IX(c, i, j, k)] = R[(size_t)i + (size_t)ld * (size_t)k];
            }
            free(A); free(B); free(C); free(R);
        }
    }
    #pragma omp parallel
    {
        ll ldj = n1 + 1, ldi = n2 + 1;
        double *AJ = ref_zalloc((size_t)ldj * (n2 + 2)), *BJ = ref_zalloc((size_t)ldj * (n2 + 2));
        double *CJ = ref_zalloc((size_t)ldj * (n2 + 2)), *GJ = ref_zalloc((size_t)ldj * (n2 + 2));
        double *AI = ref_zalloc((size_t)ldi * (n1 + 2)), *BI = ref_zalloc((size_t)ldi * (n1 + 2));
        double *CI = ref_zalloc((size_t)ldi * (n1 + 2)), *GI = ref_zalloc((size_t)ldi * (n1 + 2));
        #pragma omp for
        for (ll k = 1; k <= n3m; k++) {
            for (ll j = 1; j <= n2m; j++)
                for (ll i = 1; i <= n1m; i++) {
                    size_t q = IX(c, i, j, k);
                    CSK(q, 3)
                    size_t p = (size_t)i + (size_t)ldj * (size_t)j;
                    AJ[p] = c->ajuw[j] * (cs * ks1 + cre * omc * c->alsgs1[2][q]);
                    CJ[p] = c->cjuw[j] * (cs * ks2 + cre * omc * c->alsgs1[2][IX(c, i, j + 1, k)]);
                    BJ[p] = api - AJ[p] - CJ[p];
                    GJ[p] = api * r4[q];
                }
            ref_trdiag(AJ, BJ, CJ, GJ, 1, n2m, 1, n1m, ldj);
            for (ll i = 1; i <= n1m; i++)
                for (ll j = 1; j <= n2m; j++) {
                    size_t q = IX(c, i, j, k);
                    CSK(q, 1)
                    size_t p = (size_t)j + (size_t)ldi * (size_t)i;
                    AI[p] = c->aivw[i] * (cs * ks1 + cre * omc * c->alsgs1[0][q]);
                    CI[p] = c->civw[i] * (cs * ks2 + cre * omc * c->alsgs1[0][IX(c, i + 1, j, k)]);
                    BI[p] = api - AI[p] - CI[p];
                    GI[p] = api * GJ[(size_t)i + (size_t)ldj * (size_t)j];
                }
            if (g->xprdic == 0) ref_trdiag(AI, BI, CI, GI, 1, n1m, 1, n2m, ldi);
            else ref_trdiagp(AI, BI, CI, GI, 1, n1m, 1, n2m, ldi);
            for (ll j = 1; j <= n2m; j++)
                for (ll i = 1; i <= n1m; i++) c->t[IX(c, i, j, k)] += GI[(size_t)j + (size_t)ldi * (size_t)i];
        }
        free(AJ); free(BJ); free(CJ); free(GJ); free(AI); free(BI); free(CI); free(GI);
    }
#undef CSK
}

/* prdic_adj_t, slv_engy.f90:637-740 */
static void prdic_adj_t(ref_case *c)
{
    const lesgpu_config *g = &c->c;
    ll n1 = c->n1, n2 = c->n2, n3 = c->n3, n1m = c->n1m, n2m = c->n2m, n3m = c->n3m;
    double *t = c->t, *u = c->u;
    if (g->xprdic == 1) {
        if (g->idecomp == 1) {
            for (ll k = 0; k <= n3; k++)
                for (ll j = 0; j <= n2; j++) { t[IX(c, 0, j, k)] = t[IX(c, n1m, j, k)]; t[IX(c, n1, j, k)] = t[IX(c, 1, j, k)]; }
        } else {
            double tw = g->tsol_i, tbi = g->tflu_i, tbo = 0.0, md = 0.0;
            for (ll k = 1; k <= n3m; k++)
                for (ll j = 1; j <= n2m; j++)
                    if (c->fb_c[IX(c, n1m, j, k)] >= 1.0e-10) {
                        md += u[IX(c, n1m, j, k)] * c->f2fy[j] * c->f2fz[k];
                        tbo += t[IX(c, n1m, j, k)] * u[IX(c, n1m, j, k)] * c->f2fy[j] * c->f2fz[k];
                    }
            tbo = fabs(md) > 1.0e-14 ? tbo / md : tbi;
            double numer = tw - tbi, denom = tw - tbo, ratio;
            if (fabs(numer) <= 1.0e-14) ratio = 1.0;
            else if (fabs(denom) > 1.0e-14) { ratio = numer / denom; if (fabs(ratio) <= 1.0e-14) ratio = 1.0; }
            else ratio = 1.0;
            for (ll k = 0; k <= n3; k++)
                for (ll j = 0; j <= n2; j++) {
                    t[IX(c, 0, j, k)] = tw - (tw - t[IX(c, n1m, j, k)]) * ratio;
                    t[IX(c, n1, j, k)] = tw - (tw - t[IX(c, 1, j, k)]) / ratio;
                }
        }
    }
    if (g->yprdic == 1)
        for (ll k = 0; k <= n3; k++)
            for (ll i = 0; i <= n1; i++) { t[IX(c, i, 0, k)] = t[IX(c, i, n2m, k)]; t[IX(c, i, n2, k)] = t[IX(c, i, 1, k)]; }
    if (g->zprdic == 1)
        for (ll j = 0; j <= n2; j++)
            for (ll i = 0; i <= n1; i++) { t[IX(c, i, j, 0)] = t[IX(c, i, j, n3m)]; t[IX(c, i, j, n3)] = t[IX(c, i, j, 1)]; }
}

/* wallbc_t, slv_engy.f90:743-812 */
static void wallbc_t(ref_case *c)
{
    const lesgpu_config *g = &c->c;
    ll n1 = c->n1, n2 = c->n2, n3 = c->n3, n2m = c->n2m, n3m = c->n3m;
    double *t = c->t;
    if (g->xprdic == 0)
        for (ll k = 0; k <= n3; k++)
            for (ll j = 0; j <= n2; j++)
                t[IX(c, 0, j, k)] = (c->fb_c[IX(c, 0, j, k)] <= 1.0e-10) ? g->tsol_i : g->tflu_i;
    if (g->yprdic == 0)
        for (ll k = 0; k <= n3; k++)
            for (ll i = 0; i <= n1; i++) {
                if (g->bc_t_ybtm == 0) t[IX(c, i, 0, k)] = g->val_t_ybtm;
                else if (g->bc_t_ybtm == 1) t[IX(c, i, 0, k)] = t[IX(c, i, 1, k)] - g->val_t_ybtm / c->c2cyi[1];
                if (g->bc_t_ytop == 0) t[IX(c, i, n2, k)] = g->val_t_ytop;
                else if (g->bc_t_ytop == 1) t[IX(c, i, n2, k)] = t[IX(c, i, n2m, k)] + g->val_t_ytop / c->c2cyi[n2];
            }
    if (g->zprdic == 0)
        for (ll j = 0; j <= n2; j++)
            for (ll i = 0; i <= n1; i++) {
                if (g->bc_t_zbtm == 0) t[IX(c, i, j, 0)] = g->val_t_zbtm;
                else if (g->bc_t_zbtm == 1) t[IX(c, i, j, 0)] = t[IX(c, i, j, 1)] - g->val_t_zbtm / c->c2czi[1];
                if (g->bc_t_ztop == 0) t[IX(c, i, j, n3)] = g->val_t_ztop;
                else if (g->bc_t_ztop == 1) t[IX(c, i, j, n3)] = t[IX(c, i, j, n3m)] + g->val_t_ztop / c->c2czi[n3];
            }
}

/* rhsnlhs_t, slv_engy.f90:2-26 */
void ref_rhsnlhs_t(ref_case *c)
{
    const lesgpu_config *g = &c->c;
    rhs_t(c);
    if (g->ibmon != 0 && g->iconjg == 0) rhs_ibm_t(c);
    if (g->xprdic == 0) {
        convbc_t(c);
        if (g->ich != 1) rhsincorpbc_t(c);
    }
    lhs_t(c);
    if (g->xprdic == 0)
        for (ll k = 1; k <= c->n3m; k++)
            for (ll j = 1; j <= c->n2m; j++) c->t[IX(c, c->n1, j, k)] = c->tout[PL(c, j, k)];
    prdic_adj_t(c);
    wallbc_t(c);
}
