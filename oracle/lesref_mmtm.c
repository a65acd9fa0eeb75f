/*
 * ORACLE -- test infrastructure only (see lesref_internal.h).
 *
 * Momentum equation: 02_solver/f90/lib/slv_mmtm.f90 and slv_cont.f90.
 */
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "lesref_internal.h"
#include "lesref.h"

#define FIX(a) ((double)(a))

/* meanpg, slv_mmtm.f90:2-177.  err_integral is the routine's SAVEd state. */
void ref_meanpg(ref_case *c)
{
    const lesgpu_config *g = &c->c;
    ll n1m = c->n1m, n2m = c->n2m, n3m = c->n3m, n2 = c->n2, n3 = c->n3;
    double *u = c->u, re = g->re;
    double flowvol = 0.0, qcur = 0.0;
    #pragma omp parallel for reduction(+:flowvol, qcur)
    for (ll k = 1; k <= n3m; k++)
        for (ll j = 1; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++)
                if (c->fb_u[IX(c, i, j, k)] >= 1.0e-10) {
                    flowvol += c->c2cx[i] * c->f2fy[j] * c->f2fz[k];
                    qcur += u[IX(c, i, j, k)] * c->c2cx[i] * c->f2fy[j] * c->f2fz[k];
                }
    double ubulk = flowvol > 0.0 ? qcur / flowvol : 0.0;
    for (int q = 0; q < 5; q++) c->pmi[q] = 0.0;
    if (g->bc_ybtm == 0) {
        double tmp = 0.0, dy1 = 1.0 / c->c2cyi[1], dy2 = dy1 + 1.0 / c->c2cyi[2];
        for (ll k = 1; k <= n3m; k++)
            for (ll i = 1; i <= n1m; i++)
                if (c->fb_u[IX(c, i, 1, k)] >= 1.0e-10) {
                    double gu = (u[IX(c, i, 1, k)] * (dy2 * dy2) - u[IX(c, i, 2, k)] * (dy1 * dy1)) / (dy1 * dy2 * (dy2 - dy1));
                    tmp += gu * c->c2cx[i] * c->f2fz[k] / re;
                }
        c->pmi[1] += tmp;
    }
    if (g->bc_ytop == 0) {
        double tmp = 0.0, dy1 = 1.0 / c->c2cyi[n2], dy2 = dy1 + 1.0 / c->c2cyi[n2m];
        for (ll k = 1; k <= n3m; k++)
            for (ll i = 1; i <= n1m; i++)
                if (c->fb_u[IX(c, i, n2m, k)] >= 1.0e-10) {
                    double gu = (u[IX(c, i, n2m, k)] * (dy2 * dy2) - u[IX(c, i, n2m - 1, k)] * (dy1 * dy1)) / (dy1 * dy2 * (dy2 - dy1));
                    tmp += gu * c->c2cx[i] * c->f2fz[k] / re;
                }
        c->pmi[2] += tmp;
    }
    if (g->bc_zbtm == 0) {
        double tmp = 0.0, dz1 = 1.0 / c->c2czi[1], dz2 = dz1 + 1.0 / c->c2czi[2];
        for (ll j = 1; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++)
                if (c->fb_u[IX(c, i, j, 1)] >= 1.0e-10) {
                    double gu = (u[IX(c, i, j, 1)] * (dz2 * dz2) - u[IX(c, i, j, 2)] * (dz1 * dz1)) / (dz1 * dz2 * (dz2 - dz1));
                    tmp += gu * c->c2cx[i] * c->f2fy[j] / re;
                }
        c->pmi[3] += tmp;
    }
    if (g->bc_ztop == 0) {
        double tmp = 0.0, dz1 = 1.0 / c->c2czi[n3], dz2 = dz1 + 1.0 / c->c2czi[n3m];
        for (ll j = 1; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++)
                if (c->fb_u[IX(c, i, j, n3m)] >= 1.0e-10) {
                    double gu = (u[IX(c, i, j, n3m)] * (dz2 * dz2) - u[IX(c, i, j, n3m - 1)] * (dz1 * dz1)) / (dz1 * dz2 * (dz2 - dz1));
                    tmp += gu * c->c2cx[i] * c->f2fy[j] / re;
                }
        c->pmi[4] += tmp;
    }
    c->pmi[0] = c->pmi[1] + c->pmi[2] + c->pmi[3] + c->pmi[4];
    /* the reference stops when ICH != 0 and no wall exists; lesgpu_create
       rejects that configuration up front */
    double tmp = 0.0;
    for (ll n = 1; n <= c->nbody[0]; n++)
        tmp += c->fcv[0][n] * c->c2cx[c->ifc[0][n]] * c->f2fy[c->jfc[0][n]] * c->f2fz[c->kfc[0][n]];
    c->pmi[0] += tmp;
    double volume = c->xl * c->yl * c->zl;
    for (int q = 0; q < 5; q++) c->pmi[q] = c->pmi[q] / volume;
    if (g->ich == 0) {
        c->pmi[0] = 0.0;
    } else if (g->ich == 1) {
        if (c->ntime > 0 && c->dt > 0.0) {
            double err = g->udrv_i - ubulk;
            c->err_integral = c->err_integral + err * c->dtconst;
            c->pmi[0] = c->pmi[0] - (1.0 * err + 0.1 * c->err_integral);
        }
    } else if (g->ich == 2) {
        c->pmi[0] = -g->udrv_i;
    }
}

/* lhsinit, slv_mmtm.f90:180-249 */
void ref_lhsinit(ref_case *c)
{
    const lesgpu_config *g = &c->c;
    c->i_bgpx = g->xprdic == 1 ? 1 : 2;
    c->j_bgpy = g->yprdic == 1 ? 1 : 2;
    c->k_bgpz = g->zprdic == 1 ? 1 : 2;
    c->aiu = ref_zalloc(c->n1 + 2); c->ciu = ref_zalloc(c->n1 + 2);
    c->aivw = ref_zalloc(c->n1 + 2); c->civw = ref_zalloc(c->n1 + 2);
    c->ajv = ref_zalloc(c->n2 + 2); c->cjv = ref_zalloc(c->n2 + 2);
    c->ajuw = ref_zalloc(c->n2 + 2); c->cjuw = ref_zalloc(c->n2 + 2);
    c->akw = ref_zalloc(c->n3 + 2); c->ckw = ref_zalloc(c->n3 + 2);
    c->akuv = ref_zalloc(c->n3 + 2); c->ckuv = ref_zalloc(c->n3 + 2);
    for (ll i = c->i_bgpx; i <= c->n1m; i++) {
        ll im = c->imv[i];
        c->aiu[i] = -c->c2cxi[i] * c->f2fxi[im];
        c->ciu[i] = -c->c2cxi[i] * c->f2fxi[i];
    }
    for (ll i = 1; i <= c->n1m; i++) {
        ll ip = c->ipv[i];
        c->aivw[i] = -c->c2cxi[i] * c->f2fxi[i];
        c->civw[i] = -c->c2cxi[ip] * c->f2fxi[i];
    }
    for (ll j = c->j_bgpy; j <= c->n2m; j++) {
        ll jm = c->jmv[j];
        c->ajv[j] = -c->c2cyi[j] * c->f2fyi[jm];
        c->cjv[j] = -c->c2cyi[j] * c->f2fyi[j];
    }
    for (ll j = 1; j <= c->n2m; j++) {
        ll jp = c->jpv[j];
        c->ajuw[j] = -c->c2cyi[j] * c->f2fyi[j];
        c->cjuw[j] = -c->c2cyi[jp] * c->f2fyi[j];
    }
    for (ll k = c->k_bgpz; k <= c->n3m; k++) {
        ll km = c->kmv[k];
        c->akw[k] = -c->c2czi[k] * c->f2fzi[km];
        c->ckw[k] = -c->c2czi[k] * c->f2fzi[k];
    }
    for (ll k = 1; k <= c->n3m; k++) {
        ll kp = c->kpv[k];
        c->akuv[k] = -c->c2czi[k] * c->f2fzi[k];
        c->ckuv[k] = -c->c2czi[kp] * c->f2fzi[k];
    }
}

/* rhsnlhs, slv_mmtm.f90:252-293 */
void ref_rhsnlhs(ref_case *c)
{
    const lesgpu_config *g = &c->c;
    if (g->iles == 1) ref_rhssgs(c);
    ref_rhs(c);
    if (g->ibmon != 0) ref_rhs_ibm(c);
    ref_convbc(c);
    if (g->ich != 1) ref_rhsincorpbc(c);
    ref_lhsu(c);
    ref_lhsv(c);
    if (c->n3m != 1) ref_lhsw(c);
    ref_retrv_uvw(c);
    ref_prdic_adj_uvw(c, 0);
}

/* rhs, slv_mmtm.f90:315-567 (jut..kvb are never assigned, so the
   (1 - fix*float(jut)) factors are 1) */
void ref_rhs(ref_case *c)
{
    const lesgpu_config *g = &c->c;
    ll n2 = c->n2, n3 = c->n3, n1m = c->n1m, n2m = c->n2m, n3m = c->n3m;
    ll s = c->msub;
    double *u = c->u, *v = c->v, *w = c->w, *p = c->p, *t = c->t;
    double *nu = c->nusgs, *nu1 = c->nusgs1[0], *nu2 = c->nusgs1[1], *nu3 = c->nusgs1[2];
    double gam = c->gamma[s], ro = c->ro[s], alpha = c->alpha, dt = c->dt, re = g->re;
    double ichfac = g->ich != 0 ? 1.0 : 0.0;
    int iles = (int)g->iles;
    const double *f2fx = c->f2fx, *f2fy = c->f2fy, *f2fz = c->f2fz;
    const double *f2fxi = c->f2fxi, *f2fyi = c->f2fyi, *f2fzi = c->f2fzi;
    const double *c2cxi = c->c2cxi, *c2cyi = c->c2cyi, *c2czi = c->c2czi;
    double *r1 = c->rhs1[0], *r2 = c->rhs1[1], *r3 = c->rhs1[2];

    #pragma omp parallel for
    for (ll k = 1; k <= n3m; k++)
        for (ll j = 1; j <= n2m; j++)
            for (ll i = c->i_bgpx; i <= n1m; i++) {
                size_t q = IX(c, i, j, k);
                double fju = FIX(c->fixju[j]), fjl = FIX(c->fixjl[j]), fku = FIX(c->fixku[k]), fkl = FIX(c->fixkl[k]);
                double un = 0.5 * (f2fy[j + 1] * u[q] + f2fy[j] * u[IX(c, i, j + 1, k)]) * c2cyi[j + 1] * (1.0 - fju) + u[IX(c, i, n2, k)] * fju;
                double us = 0.5 * (f2fy[j] * u[IX(c, i, j - 1, k)] + f2fy[j - 1] * u[q]) * c2cyi[j] * (1.0 - fjl) + u[IX(c, i, 0, k)] * fjl;
                double uc = 0.5 * (f2fz[k + 1] * u[q] + f2fz[k] * u[IX(c, i, j, k + 1)]) * c2czi[k + 1] * (1.0 - fku) + u[IX(c, i, j, n3)] * fku;
                double uf = 0.5 * (f2fz[k] * u[IX(c, i, j, k - 1)] + f2fz[k - 1] * u[q]) * c2czi[k] * (1.0 - fkl) + u[IX(c, i, j, 0)] * fkl;
                double vnx = 0.5 * (f2fx[i - 1] * v[IX(c, i, j + 1, k)] + f2fx[i] * v[IX(c, i - 1, j + 1, k)]) * c2cxi[i];
                double vsx = 0.5 * (f2fx[i - 1] * v[q] + f2fx[i] * v[IX(c, i - 1, j, k)]) * c2cxi[i];
                double wcx = 0.5 * (f2fx[i - 1] * w[IX(c, i, j, k + 1)] + f2fx[i] * w[IX(c, i - 1, j, k + 1)]) * c2cxi[i];
                double wfx = 0.5 * (f2fx[i - 1] * w[q] + f2fx[i] * w[IX(c, i - 1, j, k)]) * c2cxi[i];
                double anxe = 0.5 * (u[IX(c, i + 1, j, k)] + u[q]);
                double anxw = 0.5 * (u[q] + u[IX(c, i - 1, j, k)]);
                double anxx = (anxe * anxe - anxw * anxw) * c2cxi[i];
                double anx1 = (un * vnx - us * vsx) * f2fyi[j];
                double anx2 = (uc * wcx - uf * wfx) * f2fzi[k];
                double rk3x = -anxx - anx1 - anx2;
                double alx1 = (u[IX(c, i + 1, j, k)] - u[q]) * f2fxi[i];
                double alx2 = (u[q] - u[IX(c, i - 1, j, k)]) * f2fxi[i - 1];
                double alx3 = (u[IX(c, i, j + 1, k)] - u[q]) * c2cyi[j + 1];
                double alx4 = (u[q] - u[IX(c, i, j - 1, k)]) * c2cyi[j];
                double alx5 = (u[IX(c, i, j, k + 1)] - u[q]) * c2czi[k + 1];
                double alx6 = (u[q] - u[IX(c, i, j, k - 1)]) * c2czi[k];
                double alxx = (alx1 - alx2) * c2cxi[i];
                double alxy = (alx3 - alx4) * f2fyi[j];
                double alxz = (alx5 - alx6) * f2fzi[k];
                double alx = 1.0 / re * (alxx + alxy + alxz);
                if (iles == 1) {
                    double tx = (nu[q] * alx1 - nu[IX(c, i - 1, j, k)] * alx2) * c2cxi[i];
                    double ty = (nu3[IX(c, i, j + 1, k)] * alx3 - nu3[q] * alx4) * f2fyi[j];
                    double tz = (nu2[IX(c, i, j, k + 1)] * alx5 - nu2[q] * alx6) * f2fzi[k];
                    alx = alx + (2.0 * tx + ty + tz);
                    rk3x = rk3x + r1[q];
                }
                if (g->ihtrans == 1 && g->grdir == 1) rk3x = rk3x + g->gr / (re * re) * t[q];
                r1[q] = dt * (gam * rk3x + ro * c->rk3o[0][q] + 2.0 * alpha * alx
                              - 2.0 * alpha * (p[q] - p[IX(c, i - 1, j, k)]) * c2cxi[i]
                              - 2.0 * alpha * c->pmi[0] * ichfac);
                c->rk3oo[0][q] = c->rk3o[0][q];
                c->rk3o[0][q] = rk3x;
            }

    #pragma omp parallel for
    for (ll k = 1; k <= n3m; k++)
        for (ll j = c->j_bgpy; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++) {
                size_t q = IX(c, i, j, k);
                double fiu = FIX(c->fixiu[i]), fil = FIX(c->fixil[i]), fku = FIX(c->fixku[k]), fkl = FIX(c->fixkl[k]);
                double ve = (0.5 * (f2fx[i + 1] * v[q] + f2fx[i] * v[IX(c, i + 1, j, k)]) * c2cxi[i + 1]) * (1.0 - fiu) + v[IX(c, c->n1, j, k)] * fiu;
                double vw = (0.5 * (f2fx[i] * v[IX(c, i - 1, j, k)] + f2fx[i - 1] * v[q]) * c2cxi[i]) * (1.0 - fil) + v[IX(c, 0, j, k)] * fil;
                double vc = (0.5 * (f2fz[k + 1] * v[q] + f2fz[k] * v[IX(c, i, j, k + 1)]) * c2czi[k + 1]) * (1.0 - fku) + v[IX(c, i, j, n3)] * fku;
                double vf = (0.5 * (f2fz[k] * v[IX(c, i, j, k - 1)] + f2fz[k - 1] * v[q]) * c2czi[k]) * (1.0 - fkl) + v[IX(c, i, j, 0)] * fkl;
                double uey = 0.5 * (f2fy[j - 1] * u[IX(c, i + 1, j, k)] + f2fy[j] * u[IX(c, i + 1, j - 1, k)]) * c2cyi[j];
                double uwy = 0.5 * (f2fy[j - 1] * u[q] + f2fy[j] * u[IX(c, i, j - 1, k)]) * c2cyi[j];
                double wcy = 0.5 * (f2fy[j - 1] * w[IX(c, i, j, k + 1)] + f2fy[j] * w[IX(c, i, j - 1, k + 1)]) * c2cyi[j];
                double wfy = 0.5 * (f2fy[j - 1] * w[q] + f2fy[j] * w[IX(c, i, j - 1, k)]) * c2cyi[j];
                double anyn = 0.5 * (v[IX(c, i, j + 1, k)] + v[q]);
                double anys = 0.5 * (v[q] + v[IX(c, i, j - 1, k)]);
                double anyy = c2cyi[j] * (anyn * anyn - anys * anys);
                double any1 = (uey * ve - uwy * vw) * f2fxi[i];
                double any2 = (vc * wcy - vf * wfy) * f2fzi[k];
                double rk3y = -anyy - any1 - any2;
                double aly1 = (v[IX(c, i + 1, j, k)] - v[q]) * c2cxi[i + 1];
                double aly2 = (v[q] - v[IX(c, i - 1, j, k)]) * c2cxi[i];
                double aly3 = (v[IX(c, i, j + 1, k)] - v[q]) * f2fyi[j];
                double aly4 = (v[q] - v[IX(c, i, j - 1, k)]) * f2fyi[j - 1];
                double aly5 = (v[IX(c, i, j, k + 1)] - v[q]) * c2czi[k + 1];
                double aly6 = (v[q] - v[IX(c, i, j, k - 1)]) * c2czi[k];
                double alyx = (aly1 - aly2) * f2fxi[i];
                double alyy = (aly3 - aly4) * c2cyi[j];
                double alyz = (aly5 - aly6) * f2fzi[k];
                double aly = 1.0 / re * (alyx + alyy + alyz);
                if (iles == 1) {
                    double tx = (nu3[IX(c, i + 1, j, k)] * aly1 - nu3[q] * aly2) * f2fxi[i];
                    double ty = (nu[q] * aly3 - nu[IX(c, i, j - 1, k)] * aly4) * c2cyi[j];
                    double tz = (nu1[IX(c, i, j, k + 1)] * aly5 - nu1[q] * aly6) * f2fzi[k];
                    aly = aly + (tx + 2.0 * ty + tz);
                    rk3y = rk3y + r2[q];
                }
                if (g->ihtrans == 1 && g->grdir == 2) rk3y = rk3y + g->gr / (re * re) * t[q];
                r2[q] = dt * (gam * rk3y + ro * c->rk3o[1][q] + 2.0 * alpha * aly
                              - 2.0 * alpha * (p[q] - p[IX(c, i, j - 1, k)]) * c2cyi[j]);
                c->rk3oo[1][q] = c->rk3o[1][q];
                c->rk3o[1][q] = rk3y;
            }

    if (n3m == 1) return;
    #pragma omp parallel for
    for (ll k = c->k_bgpz; k <= n3m; k++)
        for (ll j = 1; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++) {
                size_t q = IX(c, i, j, k);
                double fiu = FIX(c->fixiu[i]), fil = FIX(c->fixil[i]), fju = FIX(c->fixju[j]), fjl = FIX(c->fixjl[j]);
                double we = 0.5 * (f2fx[i + 1] * w[q] + f2fx[i] * w[IX(c, i + 1, j, k)]) * c2cxi[i + 1] * (1.0 - fiu) + fiu * w[IX(c, c->n1, j, k)];
                double ww = 0.5 * (f2fx[i] * w[IX(c, i - 1, j, k)] + f2fx[i - 1] * w[q]) * c2cxi[i] * (1.0 - fil) + fil * w[IX(c, 0, j, k)];
                double wn = (0.5 * (f2fy[j + 1] * w[q] + f2fy[j] * w[IX(c, i, j + 1, k)]) * c2cyi[j + 1]) * (1.0 - fju) + fju * w[IX(c, i, n2, k)];
                double ws = (0.5 * (f2fy[j] * w[IX(c, i, j - 1, k)] + f2fy[j - 1] * w[q]) * c2cyi[j]) * (1.0 - fjl) + fjl * w[IX(c, i, 0, k)];
                double uez = 0.5 * (f2fz[k - 1] * u[IX(c, i + 1, j, k)] + f2fz[k] * u[IX(c, i + 1, j, k - 1)]) * c2czi[k];
                double uwz = 0.5 * (f2fz[k - 1] * u[q] + f2fz[k] * u[IX(c, i, j, k - 1)]) * c2czi[k];
                double vnz = 0.5 * (f2fz[k - 1] * v[IX(c, i, j + 1, k)] + f2fz[k] * v[IX(c, i, j + 1, k - 1)]) * c2czi[k];
                double vsz = 0.5 * (f2fz[k - 1] * v[q] + f2fz[k] * v[IX(c, i, j, k - 1)]) * c2czi[k];
                double anzc = 0.5 * (w[IX(c, i, j, k + 1)] + w[q]);
                double anzf = 0.5 * (w[q] + w[IX(c, i, j, k - 1)]);
                double anzz = (anzc * anzc - anzf * anzf) * c2czi[k];
                double anz1 = (uez * we - uwz * ww) * f2fxi[i];
                double anz2 = (vnz * wn - vsz * ws) * f2fyi[j];
                double rk3z = -anzz - anz1 - anz2;
                double alz1 = (w[IX(c, i + 1, j, k)] - w[q]) * c2cxi[i + 1];
                double alz2 = (w[q] - w[IX(c, i - 1, j, k)]) * c2cxi[i];
                double alz3 = (w[IX(c, i, j + 1, k)] - w[q]) * c2cyi[j + 1];
                double alz4 = (w[q] - w[IX(c, i, j - 1, k)]) * c2cyi[j];
                double alz5 = (w[IX(c, i, j, k + 1)] - w[q]) * f2fzi[k];
                double alz6 = (w[q] - w[IX(c, i, j, k - 1)]) * f2fzi[k - 1];
                double alzx = (alz1 - alz2) * f2fxi[i];
                double alzy = (alz3 - alz4) * f2fyi[j];
                double alzz = (alz5 - alz6) * c2czi[k];
                double alz = 1.0 / re * (alzx + alzy + alzz);
                if (iles == 1) {
                    double tx = (nu2[IX(c, i + 1, j, k)] * alz1 - nu2[q] * alz2) * f2fxi[i];
                    double ty = (nu1[IX(c, i, j + 1, k)] * alz3 - nu1[q] * alz4) * f2fyi[j];
                    double tz = (nu[q] * alz5 - nu[IX(c, i, j, k - 1)] * alz6) * c2czi[k];
                    alz = alz + (tx + ty + 2.0 * tz);
                    rk3z = rk3z + r3[q];
                }
                if (g->ihtrans == 1 && g->grdir == 3) rk3z = rk3z + g->gr / (re * re) * t[q];
                r3[q] = dt * (gam * rk3z + ro * c->rk3o[2][q] + 2.0 * alpha * alz
                              - 2.0 * alpha * (p[q] - p[IX(c, i, j, k - 1)]) * c2czi[k]);
                c->rk3oo[2][q] = c->rk3o[2][q];
                c->rk3o[2][q] = rk3z;
            }
}

/* reindex_i / reindex_k, slv_mmtm.f90:821-870 */
static void reindex(ll n, ll nm, ll *ip, ll *ipp)
{
    if (*ipp == n) *ipp = 1;
    else if (*ipp == n + 1) { *ip = 1; *ipp = 2; }
    else if (*ipp == 0) *ipp = nm;
    else if (*ipp == -1) { *ip = nm; *ipp = nm - 1; }
}

/* target value of one interpolated forcing point (rhs_ibm :615-651 for u;
   the same 27-point sum for v, w and, in slv_engy.f90:236-272, for T).
   The stationary body value (ubody/tbody) is 0. */
double ref_ibm_target(const ref_case *c, int l, ll n, const double *fld, const double *rtmp)
{
    ll ii = c->ifc[l][n], jj = c->jfc[l][n], kk = c->kfc[l][n];
    const ll *d = &c->intpindx[l][3 * n];
    ll ip = ii + d[0], jp = jj + d[1], kp = kk + d[2];
    ll ipp = ii + d[0] * 2, jpp = jj + d[1] * 2, kpp = kk + d[2] * 2;
    if (ipp >= c->n1 || ipp <= 0) reindex(c->n1, c->n1m, &ip, &ipp);
    if (kpp >= c->n3 || kpp <= 0) reindex(c->n3, c->n3m, &kp, &kpp);
    ll is[3] = { ii, ip, ipp }, js[3] = { jj, jp, jpp }, ks[3] = { kk, kp, kpp };
    const double *gf = &c->geomfac[l][27 * n];
    double s = gf[0] * 0.0;
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++)
            for (int e = 0; e < 3; e++) {
                if (a == 0 && b == 0 && e == 0) continue;
                size_t q = IX(c, is[a], js[b], ks[e]);
                s = s + gf[a * 9 + b * 3 + e] * (fld[q] + rtmp[q]);
            }
    return s;
}

/* rhs_ibm, slv_mmtm.f90:569-819 */
void ref_rhs_ibm(ref_case *c)
{
    double dti = 1.0 / c->dt;
    double *fld[3] = { c->u, c->v, c->w };
    double *tmp = ref_zalloc(c->nt);
    for (int l = 0; l < 3; l++) {
        double *r = c->rhs1[l];
        for (ll k = 1; k <= c->n3m; k++)
            for (ll j = 1; j <= c->n2m; j++)
                for (ll i = 1; i <= c->n1m; i++) tmp[IX(c, i, j, k)] = r[IX(c, i, j, k)];
        for (ll n = 1; n <= c->nintp[l]; n++) {
            double targ = ref_ibm_target(c, l, n, fld[l], tmp);
            size_t q = IX(c, c->ifc[l][n], c->jfc[l][n], c->kfc[l][n]);
            c->fcv[l][n] = (targ - fld[l][q] - tmp[q]) * dti;
            c->dudtr[l][n] = (targ - fld[l][q]) * dti;
            r[q] = targ - fld[l][q];
        }
    }
    free(tmp);
    for (int l = 0; l < 3; l++) {
        double *r = c->rhs1[l];
        for (ll n = c->nintp[l] + 1; n <= c->nbody[l]; n++) {
            size_t q = IX(c, c->ifc[l][n], c->jfc[l][n], c->kfc[l][n]);
            double targ = 0.0;
            c->fcv[l][n] = (targ - fld[l][q] - r[q]) * dti;
            c->dudtr[l][n] = (targ - fld[l][q]) * dti;
            r[q] = targ - fld[l][q];
        }
    }
    for (int l = 0; l < 3; l++)
        for (ll n = 1; n <= c->nbody[l]; n++) c->fcvavg[l][n] += c->fcv[l][n];
}

#define PL(c, j, k) ((size_t)(j) + (size_t)((c)->n2 + 1) * (size_t)(k))

/* convbc, slv_mmtm.f90:873-988 */
void ref_convbc(ref_case *c)
{
    const lesgpu_config *g = &c->c;
    ll n1 = c->n1, n2 = c->n2, n3 = c->n3, n1m = c->n1m, n2m = c->n2m, n3m = c->n3m;
    double *u = c->u, *v = c->v, *w = c->w;
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
                if (c->fb_c[IX(c, n1m, j, k)] <= 1.0e-10 && g->imovingon == 0) {
                    c->uout[pq] = u[IX(c, n1m, j, k)];
                    c->vout[pq] = v[IX(c, n1m, j, k)];
                    c->wout[pq] = w[IX(c, n1m, j, k)];
                } else {
                    c->uout[pq] = u[IX(c, n1, j, k)] - ucoef * (u[IX(c, n1, j, k)] - u[IX(c, n1m, j, k)]);
                    c->vout[pq] = v[IX(c, n1, j, k)] - vwcoef * (v[IX(c, n1, j, k)] - v[IX(c, n1m, j, k)]);
                    c->wout[pq] = w[IX(c, n1, j, k)] - vwcoef * (w[IX(c, n1, j, k)] - w[IX(c, n1m, j, k)]);
                }
                qout = c->uout[pq] * c->f2fy[j] * c->f2fz[k] + qout;
            }
        double qratio = qin / qout;
        for (ll k = 1; k <= n3m; k++)
            for (ll j = 1; j <= n2m; j++) {
                size_t pq = PL(c, j, k);
                if (c->fb_c[IX(c, n1m, j, k)] > 1.0e-10) {
                    c->uout[pq] *= qratio; c->vout[pq] *= qratio; c->wout[pq] *= qratio;
                }
                c->duout[pq] = c->uout[pq] - u[IX(c, n1, j, k)];
                c->dvout[pq] = c->vout[pq] - v[IX(c, n1, j, k)];
                c->dwout[pq] = c->wout[pq] - w[IX(c, n1, j, k)];
            }
        if (g->yprdic == 1)
            for (ll k = 0; k <= n3; k++) {
                c->duout[PL(c, n2, k)] = c->duout[PL(c, 1, k)]; c->duout[PL(c, 0, k)] = c->duout[PL(c, n2m, k)];
                c->dvout[PL(c, n2, k)] = c->dvout[PL(c, 1, k)]; c->dvout[PL(c, 0, k)] = c->dvout[PL(c, n2m, k)];
                c->dwout[PL(c, n2, k)] = c->dwout[PL(c, 1, k)]; c->dwout[PL(c, 0, k)] = c->dwout[PL(c, n2m, k)];
            }
        if (g->zprdic == 1)
            for (ll j = 0; j <= n2; j++) {
                c->duout[PL(c, j, n3)] = c->duout[PL(c, j, 1)]; c->duout[PL(c, j, 0)] = c->duout[PL(c, j, n3m)];
                c->dvout[PL(c, j, n3)] = c->dvout[PL(c, j, 1)]; c->dvout[PL(c, j, 0)] = c->dvout[PL(c, j, n3m)];
                c->dwout[PL(c, j, n3)] = c->dwout[PL(c, j, 1)]; c->dwout[PL(c, j, 0)] = c->dwout[PL(c, j, n3m)];
            }
    } else {
        size_t np = (size_t)(n2 + 1) * (size_t)(n3 + 1);
        memset(c->uout, 0, np * sizeof(double));
        memset(c->vout, 0, np * sizeof(double));
        memset(c->wout, 0, np * sizeof(double));
    }
}

/* rhsincorpbc, slv_mmtm.f90:991-1041 */
void ref_rhsincorpbc(ref_case *c)
{
    const lesgpu_config *g = &c->c;
    ll n1 = c->n1, n1m = c->n1m, n2m = c->n2m, n3m = c->n3m;
    double cre = g->iles == 1 ? g->re : 0.0, cre2 = g->iles == 1 ? 2.0 * g->re : 0.0;
    for (ll k = 1; k <= n3m; k++)
        for (ll j = 1; j <= n2m; j++)
            c->rhs1[0][IX(c, n1m, j, k)] -= c->acoef * c->ciu[n1m] * (1.0 + cre2 * c->nusgs[IX(c, n1m, j, k)]) * c->duout[PL(c, j, k)];
    for (ll k = 1; k <= n3m; k++)
        for (ll j = 2; j <= n2m; j++)
            c->rhs1[1][IX(c, n1m, j, k)] -= c->acoef * c->civw[n1m] * (1.0 + cre * c->nusgs1[2][IX(c, n1, j, k)]) * c->dvout[PL(c, j, k)];
    for (ll k = c->k_bgpz; k <= n3m; k++)
        for (ll j = 1; j <= n2m; j++)
            c->rhs1[2][IX(c, n1m, j, k)] -= c->acoef * c->civw[n1m] * (1.0 + cre * c->nusgs1[1][IX(c, n1, j, k)]) * c->dwout[PL(c, j, k)];
}

/* trdiag1/2/3, slv_mmtm.f90:1365-1498: batch index i (ll1..ll2) first,
   line index j (l1..l2) second, a[i + ld*j]; r is overwritten with the
   solution (every call site passes the same array as r and uu). */
void ref_trdiag(const double *a, const double *b, const double *cc, double *r,
                ll l1, ll l2, ll ll1, ll ll2, ll ld)
{
    double *gam = ref_zalloc((size_t)ld * (size_t)(l2 + 2));
    double *bet = ref_zalloc((size_t)ld + 1);
    for (ll i = ll1; i <= ll2; i++) {
        bet[i] = 1.0 / b[i + ld * l1];
        r[i + ld * l1] = r[i + ld * l1] * bet[i];
    }
    for (ll j = l1 + 1; j <= l2; j++)
        for (ll i = ll1; i <= ll2; i++) {
            gam[i + ld * j] = cc[i + ld * (j - 1)] * bet[i];
            bet[i] = 1.0 / (b[i + ld * j] - a[i + ld * j] * gam[i + ld * j]);
            r[i + ld * j] = (r[i + ld * j] - a[i + ld * j] * r[i + ld * (j - 1)]) * bet[i];
        }
    for (ll j = l2 - 1; j >= l1; j--)
        for (ll i = ll1; i <= ll2; i++)
            r[i + ld * j] = r[i + ld * j] - gam[i + ld * (j + 1)] * r[i + ld * (j + 1)];
    free(gam); free(bet);
}

/* trdiag1p/3p, slv_mmtm.f90:1501-1641 (periodic lines j1..j2, batch l1..l2) */
void ref_trdiagp(const double *a, const double *b, const double *cc, double *f,
                 ll j1, ll j2, ll l1, ll l2, ll ld)
{
    size_t sz = (size_t)ld * (size_t)(j2 + 2);
    double *q = ref_zalloc(sz), *s = ref_zalloc(sz), *qe = ref_zalloc(sz);
    double *fn = ref_zalloc((size_t)ld + 1);
    ll ja = j1 + 1, jj = j1 + j2;
#define A2(arr, k, j) arr[(k) + ld * (j)]
    for (ll k = l1; k <= l2; k++) {
        double binv = 1.0 / A2(b, k, j1);
        A2(q, k, j1) = -A2(cc, k, j1) * binv;
        A2(s, k, j1) = -A2(a, k, j1) * binv;
        fn[k] = A2(f, k, j2);
        A2(f, k, j1) = A2(f, k, j1) * binv;
    }
    for (ll j = ja; j <= j2; j++)
        for (ll k = l1; k <= l2; k++) {
            double pn = 1.0 / (A2(b, k, j) + A2(a, k, j) * A2(q, k, j - 1));
            A2(q, k, j) = -A2(cc, k, j) * pn;
            A2(s, k, j) = -A2(a, k, j) * A2(s, k, j - 1) * pn;
            A2(f, k, j) = (A2(f, k, j) - A2(a, k, j) * A2(f, k, j - 1)) * pn;
        }
    for (ll k = l1; k <= l2; k++) { A2(s, k, j2) = 1.0; A2(qe, k, j2) = 0.0; }
    for (ll i = ja; i <= j2; i++) {
        ll j = jj - i;
        for (ll k = l1; k <= l2; k++) {
            A2(s, k, j) = A2(s, k, j) + A2(q, k, j) * A2(s, k, j + 1);
            A2(qe, k, j) = A2(f, k, j) + A2(q, k, j) * A2(qe, k, j + 1);
        }
    }
    for (ll k = l1; k <= l2; k++)
        A2(f, k, j2) = (fn[k] - A2(cc, k, j2) * A2(qe, k, j1) - A2(a, k, j2) * A2(qe, k, j2 - 1))
                     / (A2(cc, k, j2) * A2(s, k, j1) + A2(a, k, j2) * A2(s, k, j2 - 1) + A2(b, k, j2));
    for (ll i = ja; i <= j2; i++) {
        ll j = jj - i;
        for (ll k = l1; k <= l2; k++) A2(f, k, j) = A2(f, k, j2) * A2(s, k, j) + A2(qe, k, j);
    }
#undef A2
    free(q); free(s); free(qe); free(fn);
}

/* exposed for the tridiagonal invariant tests: one line, 0-based arrays */
int ref_thomas(int64_t n, const double *a, const double *b, const double *cc,
               const double *r, double *x, int periodic)
{
    if (n < 2) return LESGPU_ERR_ARG;
    double *A = ref_zalloc(n + 2), *B = ref_zalloc(n + 2), *C = ref_zalloc(n + 2), *R = ref_zalloc(n + 2);
    for (ll j = 0; j < n; j++) { A[j + 1] = a[j]; B[j + 1] = b[j]; C[j + 1] = cc[j]; R[j + 1] = r[j]; }
    if (periodic) ref_trdiagp(A, B, C, R, 1, n, 0, 0, 1);
    else ref_trdiag(A, B, C, R, 1, n, 0, 0, 1);
    for (ll j = 0; j < n; j++) x[j] = R[j + 1];
    free(A); free(B); free(C); free(R);
    return 0;
}

/* Scratch planes of one ADI sweep. */
typedef struct { double *a, *b, *cc, *r; } plane4;
static plane4 plane_alloc(size_t n)
{
    plane4 p = { ref_zalloc(n), ref_zalloc(n), ref_zalloc(n), ref_zalloc(n) };
    return p;
}
static void plane_free(plane4 *p) { free(p->a); free(p->b); free(p->cc); free(p->r); }

/* One component of the approximately factorised CN solve
   (lhsu :1044-1148, lhsv :1151-1256, lhsw :1259-1362). */
typedef struct {
    int comp;                     /* 0 u, 1 v, 2 w */
} adi_desc;

static void adi_solve(ref_case *c, int comp)
{
    const lesgpu_config *g = &c->c;
    ll n1 = c->n1, n2 = c->n2, n3 = c->n3, n1m = c->n1m, n2m = c->n2m, n3m = c->n3m;
    double cre = (double)g->iles * g->re, cre2 = 2.0 * (double)g->iles * g->re;
    double acoefi = c->acoefi;
    double *rhs = c->rhs1[comp];
    double *nu = c->nusgs, *nu1 = c->nusgs1[0], *nu2 = c->nusgs1[1], *nu3 = c->nusgs1[2];
    double *fld = comp == 0 ? c->u : comp == 1 ? c->v : c->w;
    ll ib = comp == 0 ? c->i_bgpx : 1;           /* x range of this component   */
    ll jb = comp == 1 ? 2 : 1;                   /* y range (v starts at j = 2) */
    ll kb = comp == 2 ? c->k_bgpz : 1;           /* z range                     */

    /* ---- z direction, one (n1, n3) plane per j ---- */
    if (!(comp != 2 && n3m == 1)) {
        ll ld = n1 + 1;
        #pragma omp parallel
        {
            plane4 P = plane_alloc((size_t)ld * (size_t)(n3 + 2));
            #pragma omp for
            for (ll j = jb; j <= n2m; j++) {
                ll kl = (comp == 2) ? kb : 1;
                for (ll k = kl; k <= n3m; k++)
                    for (ll i = ib; i <= n1m; i++) {
                        double ak, ck;
                        if (comp == 0) {
                            ak = c->akuv[k] * (1.0 + cre * nu2[IX(c, i, j, k)]);
                            ck = c->ckuv[k] * (1.0 + cre * nu2[IX(c, i, j, k + 1)]);
                        } else if (comp == 1) {
                            ak = c->akuv[k] * (1.0 + cre * nu1[IX(c, i, j, k)]);
                            ck = c->ckuv[k] * (1.0 + cre * nu1[IX(c, i, j, k + 1)]);
                        } else {
                            ak = c->akw[k] * (1.0 + cre2 * nu[IX(c, i, j, k - 1)]);
                            ck = c->ckw[k] * (1.0 + cre2 * nu[IX(c, i, j, k)]);
                        }
                        size_t q = (size_t)i + (size_t)ld * (size_t)k;
                        P.a[q] = ak; P.cc[q] = ck;
                        P.b[q] = acoefi - ak - ck;
                        P.r[q] = acoefi * rhs[IX(c, i, j, k)];
                    }
                if (g->zprdic == 0) {
                    ll l1 = (comp == 2) ? 2 : 1;
                    ref_trdiag(P.a, P.b, P.cc, P.r, l1, n3m, ib, n1m, ld);
                } else {
                    ref_trdiagp(P.a, P.b, P.cc, P.r, 1, n3m, ib, n1m, ld);
                }
                for (ll k = kl; k <= n3m; k++)
                    for (ll i = ib; i <= n1m; i++) rhs[IX(c, i, j, k)] = P.r[(size_t)i + (size_t)ld * (size_t)k];
            }
            plane_free(&P);
        }
    }

    /* ---- y then x direction, one k plane at a time ---- */
    #pragma omp parallel
    {
        ll ldj = n1 + 1, ldi = n2 + 1;
        plane4 J = plane_alloc((size_t)ldj * (size_t)(n2 + 2));
        plane4 I = plane_alloc((size_t)ldi * (size_t)(n1 + 2));
        #pragma omp for
        for (ll k = kb; k <= n3m; k++) {
            for (ll j = jb; j <= n2m; j++)
                for (ll i = ib; i <= n1m; i++) {
                    double aj, cj;
                    if (comp == 0) {
                        aj = c->ajuw[j] * (1.0 + cre * nu3[IX(c, i, j, k)]);
                        cj = c->cjuw[j] * (1.0 + cre * nu3[IX(c, i, j + 1, k)]);
                    } else if (comp == 1) {
                        aj = c->ajv[j] * (1.0 + cre2 * nu[IX(c, i, j - 1, k)]);
                        cj = c->cjv[j] * (1.0 + cre2 * nu[IX(c, i, j, k)]);
                    } else {
                        aj = c->ajuw[j] * (1.0 + cre * nu1[IX(c, i, j, k)]);
                        cj = c->cjuw[j] * (1.0 + cre * nu1[IX(c, i, j + 1, k)]);
                    }
                    size_t q = (size_t)i + (size_t)ldj * (size_t)j;
                    J.a[q] = aj; J.cc[q] = cj;
                    J.b[q] = acoefi - aj - cj;
                    J.r[q] = acoefi * rhs[IX(c, i, j, k)];
                }
            ref_trdiag(J.a, J.b, J.cc, J.r, jb, n2m, ib, n1m, ldj);
            for (ll i = ib; i <= n1m; i++)
                for (ll j = jb; j <= n2m; j++) {
                    double ai, ci;
                    if (comp == 0) {
                        ai = c->aiu[i] * (1.0 + cre2 * nu[IX(c, i - 1, j, k)]);
                        ci = c->ciu[i] * (1.0 + cre2 * nu[IX(c, i, j, k)]);
                    } else if (comp == 1) {
                        ai = c->aivw[i] * (1.0 + cre * nu3[IX(c, i, j, k)]);
                        ci = c->civw[i] * (1.0 + cre * nu3[IX(c, i + 1, j, k)]);
                    } else {
                        ai = c->aivw[i] * (1.0 + cre * nu2[IX(c, i, j, k)]);
                        ci = c->civw[i] * (1.0 + cre * nu2[IX(c, i + 1, j, k)]);
                    }
                    size_t q = (size_t)j + (size_t)ldi * (size_t)i;
                    I.a[q] = ai; I.cc[q] = ci;
                    I.b[q] = acoefi - ai - ci;
                    I.r[q] = acoefi * J.r[(size_t)i + (size_t)ldj * (size_t)j];
                }
            if (g->xprdic == 0) ref_trdiag(I.a, I.b, I.cc, I.r, ib, n1m, jb, n2m, ldi);
            else ref_trdiagp(I.a, I.b, I.cc, I.r, ib, n1m, jb, n2m, ldi);
            for (ll j = jb; j <= n2m; j++)
                for (ll i = ib; i <= n1m; i++)
                    fld[IX(c, i, j, k)] = I.r[(size_t)j + (size_t)ldi * (size_t)i] + fld[IX(c, i, j, k)];
        }
        plane_free(&J); plane_free(&I);
    }
}

void ref_lhsu(ref_case *c) { adi_solve(c, 0); }
void ref_lhsv(ref_case *c) { adi_solve(c, 1); }
void ref_lhsw(ref_case *c) { adi_solve(c, 2); }

/* retrv_uvw, slv_mmtm.f90:1710-1743 */
void ref_retrv_uvw(ref_case *c)
{
    ll n1 = c->n1, n2m = c->n2m, n3m = c->n3m;
    for (ll k = 1; k <= n3m; k++)
        for (ll j = 1; j <= n2m; j++) c->u[IX(c, n1, j, k)] = c->uout[PL(c, j, k)];
    for (ll k = 1; k <= n3m; k++)
        for (ll j = 2; j <= n2m; j++) c->v[IX(c, n1, j, k)] = c->vout[PL(c, j, k)];
    for (ll k = c->k_bgpz; k <= n3m; k++)
        for (ll j = 1; j <= n2m; j++) c->w[IX(c, n1, j, k)] = c->wout[PL(c, j, k)];
}

/* prdic_adj_uvw, slv_mmtm.f90:1746-1857 */
void ref_prdic_adj_uvw(ref_case *c, int isp)
{
    ll n1 = c->n1, n2 = c->n2, n3 = c->n3, n1m = c->n1m, n2m = c->n2m, n3m = c->n3m;
    double *u = c->u, *v = c->v, *w = c->w, *p = c->p;
    if (c->c.xprdic == 1) {
        for (ll k = 0; k <= n3; k++)
            for (ll j = 0; j <= n2; j++) { u[IX(c, 0, j, k)] = u[IX(c, n1m, j, k)]; u[IX(c, n1, j, k)] = u[IX(c, 1, j, k)]; }
        for (ll k = 0; k <= n3; k++)
            for (ll j = 1; j <= n2; j++) { v[IX(c, 0, j, k)] = v[IX(c, n1m, j, k)]; v[IX(c, n1, j, k)] = v[IX(c, 1, j, k)]; }
        for (ll k = 1; k <= n3; k++)
            for (ll j = 0; j <= n2; j++) { w[IX(c, 0, j, k)] = w[IX(c, n1m, j, k)]; w[IX(c, n1, j, k)] = w[IX(c, 1, j, k)]; }
        if (isp)
            for (ll k = 1; k <= n3m; k++)
                for (ll j = 1; j <= n2m; j++) { p[IX(c, 0, j, k)] = p[IX(c, n1m, j, k)]; p[IX(c, n1, j, k)] = p[IX(c, 1, j, k)]; }
    }
    if (c->c.yprdic == 1) {
        for (ll k = 1; k <= n3; k++)
            for (ll i = 0; i <= n1; i++) { u[IX(c, i, 0, k)] = u[IX(c, i, n2m, k)]; u[IX(c, i, n2, k)] = u[IX(c, i, 1, k)]; }
        for (ll k = 0; k <= n3; k++)
            for (ll i = 0; i <= n1; i++) { v[IX(c, i, 0, k)] = v[IX(c, i, n2m, k)]; v[IX(c, i, n2, k)] = v[IX(c, i, 1, k)]; }
        for (ll k = 0; k <= n3; k++)
            for (ll i = 1; i <= n1; i++) { w[IX(c, i, 0, k)] = w[IX(c, i, n2m, k)]; w[IX(c, i, n2, k)] = w[IX(c, i, 1, k)]; }
        if (isp)
            for (ll k = 1; k <= n3m; k++)
                for (ll i = 1; i <= n1m; i++) { p[IX(c, i, 0, k)] = p[IX(c, i, n2m, k)]; p[IX(c, i, n2, k)] = p[IX(c, i, 1, k)]; }
    }
    if (c->c.zprdic == 1) {
        for (ll j = 0; j <= n2; j++)
            for (ll i = 1; i <= n1; i++) { u[IX(c, i, j, 0)] = u[IX(c, i, j, n3m)]; u[IX(c, i, j, n3)] = u[IX(c, i, j, 1)]; }
        for (ll j = 1; j <= n2; j++)
            for (ll i = 0; i <= n1; i++) { v[IX(c, i, j, 0)] = v[IX(c, i, j, n3m)]; v[IX(c, i, j, n3)] = v[IX(c, i, j, 1)]; }
        for (ll j = 0; j <= n2; j++)
            for (ll i = 0; i <= n1; i++) { w[IX(c, i, j, 0)] = w[IX(c, i, j, n3m)]; w[IX(c, i, j, n3)] = w[IX(c, i, j, 1)]; }
        if (isp)
            for (ll j = 1; j <= n2m; j++)
                for (ll i = 1; i <= n1m; i++) { p[IX(c, i, j, 0)] = p[IX(c, i, j, n3m)]; p[IX(c, i, j, n3)] = p[IX(c, i, j, 1)]; }
    }
}

/* divgs, slv_cont.f90:2-208 (stationary-body branch) */
void ref_divgs(ref_case *c)
{
    const lesgpu_config *g = &c->c;
    ll n1m = c->n1m, n2m = c->n2m, n3m = c->n3m;
    double *u = c->u, *v = c->v, *w = c->w, *dv = c->divgsum, *qm = c->qmass;
    #pragma omp parallel for
    for (ll k = 1; k <= n3m; k++)
        for (ll j = 1; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++) {
                double d1 = (u[IX(c, i + 1, j, k)] - u[IX(c, i, j, k)]) * c->f2fxi[i];
                double d2 = (v[IX(c, i, j + 1, k)] - v[IX(c, i, j, k)]) * c->f2fyi[j];
                double d3 = (w[IX(c, i, j, k + 1)] - w[IX(c, i, j, k)]) * c->f2fzi[k];
                dv[IX(c, i, j, k)] = (d1 + d2 + d3);
            }
    if (g->masson == 1 && g->imovingon == 0) {
        memset(qm, 0, c->nt * sizeof(double));
        for (ll n = 1; n <= c->nbody[0]; n++) {
            ll ii = c->ifc[0][n], jj = c->jfc[0][n], kk = c->kfc[0][n];
            size_t q = IX(c, ii, jj, kk);
            qm[q] = qm[q] - u[q] * c->f2fxi[ii];
            dv[q] = dv[q] + u[q] * c->f2fxi[ii];
        }
        for (ll n = 1; n <= c->nbody[0]; n++) {
            ll ii = c->ifc[0][n], jj = c->jfc[0][n], kk = c->kfc[0][n], imm = c->imv[ii];
            size_t q = IX(c, imm, jj, kk);
            qm[q] = qm[q] + u[IX(c, ii, jj, kk)] * c->f2fxi[imm];
            dv[q] = dv[q] - u[IX(c, ii, jj, kk)] * c->f2fxi[imm];
        }
        for (ll n = 1; n <= c->nbody[1]; n++) {
            ll ii = c->ifc[1][n], jj = c->jfc[1][n], kk = c->kfc[1][n];
            size_t q = IX(c, ii, jj, kk);
            qm[q] = qm[q] - v[q] * c->f2fyi[jj];
            dv[q] = dv[q] + v[q] * c->f2fyi[jj];
        }
        for (ll n = 1; n <= c->nbody[1]; n++) {
            ll ii = c->ifc[1][n], jj = c->jfc[1][n], kk = c->kfc[1][n], jmm = c->jmv[jj];
            size_t q = IX(c, ii, jmm, kk);
            qm[q] = qm[q] + v[IX(c, ii, jj, kk)] * c->f2fyi[jmm];
            dv[q] = dv[q] - v[IX(c, ii, jj, kk)] * c->f2fyi[jmm];
        }
        for (ll n = 1; n <= c->nbody[2]; n++) {
            ll ii = c->ifc[2][n], jj = c->jfc[2][n], kk = c->kfc[2][n];
            size_t q = IX(c, ii, jj, kk);
            qm[q] = qm[q] - w[q] * c->f2fzi[kk];
            dv[q] = dv[q] + w[q] * c->f2fzi[kk];
        }
        for (ll n = 1; n <= c->nbody[2]; n++) {
            ll ii = c->ifc[2][n], jj = c->jfc[2][n], kk = c->kfc[2][n], kmm = c->kmv[kk];
            size_t q = IX(c, ii, jj, kmm);
            qm[q] = qm[q] + w[IX(c, ii, jj, kk)] * c->f2fzi[kmm];
            dv[q] = dv[q] - w[IX(c, ii, jj, kk)] * c->f2fzi[kmm];
        }
    }
    double dti = c->dtconsti;
    #pragma omp parallel for
    for (ll k = 1; k <= n3m; k++)
        for (ll j = 1; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++) dv[IX(c, i, j, k)] = dv[IX(c, i, j, k)] * dti;
}
