/*
 * ORACLE -- test infrastructure only (see lesref_internal.h).
 *
 * Dynamic Vreman eddy viscosity and dynamic eddy diffusivity:
 * 02_solver/f90/lib/sgs.f90.
 */
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "lesref_internal.h"

#define CF(arr, i, d) (arr)[3 * (size_t)(i) + (size_t)((d) + 1)]

/* sgsfilterinit, sgs.f90:2-285 (only the 3-point cf?1 weights are used by
   test_filter; the 5-point cf?2 weights are computed there but never read) */
static void filter_coefs(double *cf, const double *c2c, ll nm)
{
    if (nm == 1) return;
    for (ll i = 1; i <= nm; i++) {
        double h1 = c2c[i], h2 = c2c[i + 1];
        CF(cf, i, -1) = (2.0 * h1 - h2) / 6.0 / h1;
        CF(cf, i, 0) = ((h1 + h2) * (h1 + h2)) / 6.0 / h1 / h2;
        CF(cf, i, 1) = (2.0 * h2 - h1) / 6.0 / h2;
    }
}

void ref_sgsfilterinit(ref_case *c)
{
    c->cfx1 = ref_zalloc(3 * (c->n1m + 2));
    c->cfy1 = ref_zalloc(3 * (c->n2m + 2));
    c->cfz1 = ref_zalloc(3 * (c->n3m + 2));
    filter_coefs(c->cfx1, c->c2cx, c->n1m);
    filter_coefs(c->cfy1, c->c2cy, c->n2m);
    filter_coefs(c->cfz1, c->c2cz, c->n3m);
}

/* test_filter, sgs.f90:641-769: Simpson test filter along x and/or z on an
   interior array held in the full layout.  tmp, src: scratch of c->nt. */
void ref_test_filter(const ref_case *c, double *a0, double *tmp, double *src)
{
    ll n1m = c->n1m, n2m = c->n2m, n3m = c->n3m;
    int xf = 0, yf = 0, zf = 0;
    if (c->c.filter == 1) xf = 1;
    else if (c->c.filter == 2) zf = 1;
    else { xf = 1; zf = 1; }
    memcpy(tmp, a0, c->nt * sizeof(double));
    if (xf) {
        memcpy(src, tmp, c->nt * sizeof(double));
        for (ll k = 1; k <= n3m; k++)
            for (ll j = 1; j <= n2m; j++) {
                for (ll i = 2; i <= n1m - 1; i++)
                    tmp[IX(c, i, j, k)] = CF(c->cfx1, i, -1) * src[IX(c, i - 1, j, k)] + CF(c->cfx1, i, 0) * src[IX(c, i, j, k)]
                                        + CF(c->cfx1, i, 1) * src[IX(c, i + 1, j, k)];
                if (c->c.xprdic == 1) {
                    tmp[IX(c, 1, j, k)] = CF(c->cfx1, 1, -1) * src[IX(c, n1m, j, k)] + CF(c->cfx1, 1, 0) * src[IX(c, 1, j, k)]
                                        + CF(c->cfx1, 1, 1) * src[IX(c, 2, j, k)];
                    tmp[IX(c, n1m, j, k)] = CF(c->cfx1, n1m, -1) * src[IX(c, n1m - 1, j, k)] + CF(c->cfx1, n1m, 0) * src[IX(c, n1m, j, k)]
                                          + CF(c->cfx1, n1m, 1) * src[IX(c, 1, j, k)];
                }
            }
    }
    if (yf) {
        memcpy(src, tmp, c->nt * sizeof(double));
        for (ll k = 1; k <= n3m; k++)
            for (ll i = 1; i <= n1m; i++) {
                for (ll j = 2; j <= n2m - 1; j++)
                    tmp[IX(c, i, j, k)] = CF(c->cfy1, j, -1) * src[IX(c, i, j - 1, k)] + CF(c->cfy1, j, 0) * src[IX(c, i, j, k)]
                                        + CF(c->cfy1, j, 1) * src[IX(c, i, j + 1, k)];
                if (c->c.yprdic == 1) {
                    tmp[IX(c, i, 1, k)] = CF(c->cfy1, 1, -1) * src[IX(c, i, n2m, k)] + CF(c->cfy1, 1, 0) * src[IX(c, i, 1, k)]
                                        + CF(c->cfy1, 1, 1) * src[IX(c, i, 2, k)];
                    tmp[IX(c, i, n2m, k)] = CF(c->cfy1, n2m, -1) * src[IX(c, i, n2m - 1, k)] + CF(c->cfy1, n2m, 0) * src[IX(c, i, n2m, k)]
                                          + CF(c->cfy1, n2m, 1) * src[IX(c, i, 1, k)];
                }
            }
    }
    if (zf) {
        memcpy(src, tmp, c->nt * sizeof(double));
        for (ll j = 1; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++) {
                for (ll k = 2; k <= n3m - 1; k++)
                    tmp[IX(c, i, j, k)] = CF(c->cfz1, k, -1) * src[IX(c, i, j, k - 1)] + CF(c->cfz1, k, 0) * src[IX(c, i, j, k)]
                                        + CF(c->cfz1, k, 1) * src[IX(c, i, j, k + 1)];
                if (c->c.zprdic == 1) {
                    tmp[IX(c, i, j, 1)] = CF(c->cfz1, 1, -1) * src[IX(c, i, j, n3m)] + CF(c->cfz1, 1, 0) * src[IX(c, i, j, 1)]
                                        + CF(c->cfz1, 1, 1) * src[IX(c, i, j, 2)];
                    tmp[IX(c, i, j, n3m)] = CF(c->cfz1, n3m, -1) * src[IX(c, i, j, n3m - 1)] + CF(c->cfz1, n3m, 0) * src[IX(c, i, j, n3m)]
                                          + CF(c->cfz1, n3m, 1) * src[IX(c, i, j, 1)];
                }
            }
    }
    memcpy(a0, tmp, c->nt * sizeof(double));
}

/* velgrad, sgs.f90:772-875: the nine velocity gradients at a cell centre */
void ref_velgrad(const ref_case *c, ll i, ll j, ll k, double a[9], double sr[6])
{
    ll kp = c->kpv[k], km = c->kmv[k], jp = c->jpv[j], jm = c->jmv[j], ip = c->ipv[i], im = c->imv[i];
    ll n1 = c->n1, n2 = c->n2, n3 = c->n3;
    const double *u = c->u, *v = c->v, *w = c->w;
    const double *f2fx = c->f2fx, *f2fy = c->f2fy, *f2fz = c->f2fz;
    double fju = (double)c->fixju[j], fjl = (double)c->fixjl[j], fku = (double)c->fixku[k], fkl = (double)c->fixkl[k];
    double fiu = (double)c->fixiu[i], fil = (double)c->fixil[i];
#define U(a_, b_, c_) u[IX(c, a_, b_, c_)]
#define V(a_, b_, c_) v[IX(c, a_, b_, c_)]
#define W(a_, b_, c_) w[IX(c, a_, b_, c_)]
    double vg11 = c->f2fxi[i] * (U(ip, j, k) - U(i, j, k));
    double up = c->c2cyi[jp] * 0.25 * (f2fy[jp] * (U(i, j, k) + U(ip, j, k)) + f2fy[j] * (U(i, jp, k) + U(ip, jp, k))) * (1.0 - fju)
              + 0.5 * (U(i, n2, k) + U(ip, n2, k)) * fju;
    double um = c->c2cyi[j] * 0.25 * (f2fy[j] * (U(i, jm, k) + U(ip, jm, k)) + f2fy[jm] * (U(i, j, k) + U(ip, j, k))) * (1.0 - fjl)
              + 0.5 * (U(i, 0, k) + U(ip, 0, k)) * fjl;
    double vg12 = c->f2fyi[j] * (up - um);
    up = c->c2czi[kp] * 0.25 * (f2fz[kp] * (U(i, j, k) + U(ip, j, k)) + f2fz[k] * (U(i, j, kp) + U(ip, j, kp))) * (1.0 - fku)
       + 0.5 * (U(i, j, n3) + U(ip, j, n3)) * fku;
    um = c->c2czi[k] * 0.25 * (f2fz[k] * (U(i, j, km) + U(ip, j, km)) + f2fz[km] * (U(i, j, k) + U(ip, j, k))) * (1.0 - fkl)
       + 0.5 * (U(i, j, 0) + U(ip, j, 0)) * fkl;
    double vg13 = c->f2fzi[k] * (up - um);
    double vp = c->c2cxi[ip] * 0.25 * (f2fx[ip] * (V(i, j, k) + V(i, jp, k)) + f2fx[i] * (V(ip, j, k) + V(ip, jp, k))) * (1.0 - fiu)
              + 0.5 * (V(n1, j, k) + V(n1, jp, k)) * fiu;
    double vm = c->c2cxi[i] * 0.25 * (f2fx[i] * (V(im, j, k) + V(im, jp, k)) + f2fx[im] * (V(i, j, k) + V(i, jp, k))) * (1.0 - fil)
              + 0.5 * (V(0, j, k) + V(0, jp, k)) * fil;
    double vg21 = c->f2fxi[i] * (vp - vm);
    double vg22 = c->f2fyi[j] * (V(i, jp, k) - V(i, j, k));
    vp = c->c2czi[kp] * 0.25 * (f2fz[kp] * (V(i, j, k) + V(i, jp, k)) + f2fz[k] * (V(i, j, kp) + V(i, jp, kp))) * (1.0 - fku)
       + 0.5 * (V(i, j, n3) + V(i, jp, n3)) * fku;
    vm = c->c2czi[k] * 0.25 * (f2fz[k] * (V(i, j, km) + V(i, jp, km)) + f2fz[km] * (V(i, j, k) + V(i, jp, k))) * (1.0 - fkl)
       + 0.5 * (V(i, j, 0) + V(i, jp, 0)) * fkl;
    double vg23 = c->f2fzi[k] * (vp - vm);
    double wp = c->c2cxi[ip] * 0.25 * (f2fx[ip] * (W(i, j, k) + W(i, j, kp)) + f2fx[i] * (W(ip, j, k) + W(ip, j, kp))) * (1.0 - fiu)
              + 0.5 * (W(n1, j, k) + W(n1, j, kp)) * fiu;
    double wm = c->c2cxi[i] * 0.25 * (f2fx[i] * (W(im, j, k) + W(im, j, kp)) + f2fx[im] * (W(i, j, k) + W(i, j, kp))) * (1.0 - fil)
              + 0.5 * (W(0, j, k) + W(0, j, kp)) * fil;
    double vg31 = c->f2fxi[i] * (wp - wm);
    wp = c->c2cyi[jp] * 0.25 * (f2fy[jp] * (W(i, j, k) + W(i, j, kp)) + f2fy[j] * (W(i, jp, k) + W(i, jp, kp))) * (1.0 - fju)
       + 0.5 * (W(i, n2, k) + W(i, n2, kp)) * fju;
    wm = c->c2cyi[j] * 0.25 * (f2fy[j] * (W(i, jm, k) + W(i, jm, kp)) + f2fy[jm] * (W(i, j, k) + W(i, j, kp))) * (1.0 - fjl)
       + 0.5 * (W(i, 0, k) + W(i, 0, kp)) * fjl;
    double vg32 = c->f2fyi[j] * (wp - wm);
    double vg33 = c->f2fzi[k] * (W(i, j, kp) - W(i, j, k));
#undef U
#undef V
#undef W
    a[0] = vg11; a[1] = vg21; a[2] = vg31;
    a[3] = vg12; a[4] = vg22; a[5] = vg32;
    a[6] = vg13; a[7] = vg23; a[8] = vg33;
    sr[0] = vg11; sr[1] = 0.5 * (vg12 + vg21); sr[2] = 0.5 * (vg13 + vg31);
    sr[3] = vg22; sr[4] = 0.5 * (vg23 + vg32); sr[5] = vg33;
}

/* temgrad, sgs.f90:1480-1525 */
static void temgrad(const ref_case *c, ll i, ll j, ll k, double a[3])
{
    ll kp = c->kpv[k], km = c->kmv[k], jp = c->jpv[j], jm = c->jmv[j], ip = c->ipv[i], im = c->imv[i];
    const double *t = c->t;
    double fiu = (double)c->fixiu[i], fil = (double)c->fixil[i], fju = (double)c->fixju[j], fjl = (double)c->fixjl[j];
    double fku = (double)c->fixku[k], fkl = (double)c->fixkl[k];
    double tc = t[IX(c, i, j, k)];
    double tp = 0.5 * (c->f2fx[i] * t[IX(c, ip, j, k)] + c->f2fx[ip] * tc) * c->c2cxi[ip] * (1.0 - fiu) + t[IX(c, ip, j, k)] * fiu;
    double tm = 0.5 * (c->f2fx[im] * tc + c->f2fx[i] * t[IX(c, im, j, k)]) * c->c2cxi[i] * (1.0 - fil) + t[IX(c, im, j, k)] * fil;
    a[0] = c->f2fxi[i] * (tp - tm);
    tp = 0.5 * (c->f2fy[j] * t[IX(c, i, jp, k)] + c->f2fy[jp] * tc) * c->c2cyi[jp] * (1.0 - fju) + t[IX(c, i, jp, k)] * fju;
    tm = 0.5 * (c->f2fy[jm] * tc + c->f2fy[j] * t[IX(c, i, jm, k)]) * c->c2cyi[j] * (1.0 - fjl) + t[IX(c, i, jm, k)] * fjl;
    a[1] = c->f2fyi[j] * (tp - tm);
    tp = 0.5 * (c->f2fz[k] * t[IX(c, i, j, kp)] + c->f2fz[kp] * tc) * c->c2czi[kp] * (1.0 - fku) + t[IX(c, i, j, kp)] * fku;
    tm = 0.5 * (c->f2fz[km] * tc + c->f2fz[k] * t[IX(c, i, j, km)]) * c->c2czi[k] * (1.0 - fkl) + t[IX(c, i, j, km)] * fkl;
    a[2] = c->f2fzi[k] * (tp - tm);
}

static void vreman_b(const double alp[9], double sdx2, double sdy2, double sdz2, double *aaa, double *bbb)
{
    double b1 = sdx2 * alp[0] * alp[0] + sdy2 * alp[3] * alp[3] + sdz2 * alp[6] * alp[6];
    double b2 = sdx2 * alp[0] * alp[1] + sdy2 * alp[3] * alp[4] + sdz2 * alp[6] * alp[7];
    double b3 = sdx2 * alp[0] * alp[2] + sdy2 * alp[3] * alp[5] + sdz2 * alp[6] * alp[8];
    double b4 = sdx2 * alp[1] * alp[1] + sdy2 * alp[4] * alp[4] + sdz2 * alp[7] * alp[7];
    double b5 = sdx2 * alp[1] * alp[2] + sdy2 * alp[4] * alp[5] + sdz2 * alp[7] * alp[8];
    double b6 = sdx2 * alp[2] * alp[2] + sdy2 * alp[5] * alp[5] + sdz2 * alp[8] * alp[8];
    double a = 0.0;
    for (int q = 0; q < 9; q++) a += alp[q] * alp[q];
    double b = b1 * b4 + b4 * b6 + b6 * b1 - b2 * b2 - b3 * b3 - b5 * b5;
    if (b < 1.0e-16) b = 1.0e-16;
    *aaa = a; *bbb = b;
}

/* sgs_cvm, sgs.f90:335-402 */
static void sgs_cvm(ref_case *c)
{
    #pragma omp parallel for
    for (ll k = 1; k <= c->n3m; k++)
        for (ll j = 1; j <= c->n2m; j++)
            for (ll i = 1; i <= c->n1m; i++) {
                double a[9], s[6], aaa, bbb;
                ref_velgrad(c, i, j, k, a, s);
                vreman_b(a, c->f2fx[i] * c->f2fx[i], c->f2fy[j] * c->f2fy[j], c->f2fz[k] * c->f2fz[k], &aaa, &bbb);
                c->nusgs[IX(c, i, j, k)] = (aaa == 0.0) ? 0.0 : c->c.csgsts * sqrt(bbb / aaa);
            }
}

/* sgs_dvmg, sgs.f90:405-638: dynamic Vreman model with one global
   coefficient from the least-squares Germano identity. */
static void sgs_dvmg(ref_case *c)
{
    ll n1m = c->n1m, n2m = c->n2m, n3m = c->n3m;
    size_t nt = c->nt;
    double *aalp[9], *llij[6], *mmij[6], *uui[3];
    for (int q = 0; q < 9; q++) aalp[q] = ref_zalloc(nt);
    for (int q = 0; q < 6; q++) { llij[q] = ref_zalloc(nt); mmij[q] = ref_zalloc(nt); }
    for (int q = 0; q < 3; q++) uui[q] = ref_zalloc(nt);
    c->csgsts = 0.0;

    #pragma omp parallel for
    for (ll k = 1; k <= n3m; k++)
        for (ll j = 1; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++) {
                double alp[9], str[6], aaa, bbb;
                ref_velgrad(c, i, j, k, alp, str);
                vreman_b(alp, c->f2fx[i] * c->f2fx[i], c->f2fy[j] * c->f2fy[j], c->f2fz[k] * c->f2fz[k], &aaa, &bbb);
                size_t q = IX(c, i, j, k);
                double nu = (aaa == 0.0) ? 0.0 : sqrt(bbb / aaa);
                c->nusgs[q] = nu;
                for (int m = 0; m < 6; m++) mmij[m][q] = nu * str[m];
                for (int m = 0; m < 9; m++) aalp[m][q] = alp[m];
            }

    #pragma omp parallel
    {
        double *tmp = ref_zalloc(nt), *src = ref_zalloc(nt);
        #pragma omp for
        for (int m = 0; m < 15; m++) {
            if (m < 6) ref_test_filter(c, mmij[m], tmp, src);
            else ref_test_filter(c, aalp[m - 6], tmp, src);
        }
        free(tmp); free(src);
    }

    #pragma omp parallel for
    for (ll k = 1; k <= n3m; k++)
        for (ll j = 1; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++) {
                size_t q = IX(c, i, j, k);
                double alp[9], str[6], aaa, bbb;
                for (int m = 0; m < 9; m++) alp[m] = aalp[m][q];
                str[0] = alp[0]; str[1] = 0.5 * (alp[3] + alp[1]); str[2] = 0.5 * (alp[6] + alp[2]);
                str[3] = alp[4]; str[4] = 0.5 * (alp[7] + alp[5]); str[5] = alp[8];
                double sx = 0.5 * c->f2fx[i - 1] * (1.0 - (double)c->fixiu[i]) + c->f2fx[i] + 0.5 * c->f2fx[i + 1] * (1.0 - (double)c->fixil[i]);
                double sy = 0.5 * c->f2fy[j - 1] * (1.0 - (double)c->fixju[j]) + c->f2fy[j] + 0.5 * c->f2fy[j + 1] * (1.0 - (double)c->fixjl[j]);
                double sz = 0.5 * c->f2fz[k - 1] * (1.0 - (double)c->fixku[k]) + c->f2fz[k] + 0.5 * c->f2fz[k + 1] * (1.0 - (double)c->fixkl[k]);
                vreman_b(alp, sx * sx, sy * sy, sz * sz, &aaa, &bbb);
                double ami = (aaa == 0.0) ? 0.0 : sqrt(bbb / aaa);
                for (int m = 0; m < 6; m++) mmij[m][q] = ami * str[m] - mmij[m][q];
                double u1 = 0.5 * (c->u[q] + c->u[IX(c, i + 1, j, k)]);
                double u2 = 0.5 * (c->v[q] + c->v[IX(c, i, j + 1, k)]);
                double u3 = 0.5 * (c->w[q] + c->w[IX(c, i, j, k + 1)]);
                uui[0][q] = u1; uui[1][q] = u2; uui[2][q] = u3;
                llij[0][q] = u1 * u1; llij[1][q] = u1 * u2; llij[2][q] = u1 * u3;
                llij[3][q] = u2 * u2; llij[4][q] = u2 * u3; llij[5][q] = u3 * u3;
            }

    #pragma omp parallel
    {
        double *tmp = ref_zalloc(nt), *src = ref_zalloc(nt);
        #pragma omp for
        for (int m = 0; m < 9; m++) {
            if (m < 3) ref_test_filter(c, uui[m], tmp, src);
            else ref_test_filter(c, llij[m - 3], tmp, src);
        }
        free(tmp); free(src);
    }

    double lm = 0.0, mm = 0.0;
    #pragma omp parallel for reduction(+:lm, mm)
    for (ll k = 1; k <= n3m; k++)
        for (ll j = 1; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++) {
                size_t q = IX(c, i, j, k);
                double vol = c->f2fx[i] * c->f2fy[j] * c->f2fz[k];
                double L[6];
                L[0] = llij[0][q] - uui[0][q] * uui[0][q];
                L[1] = llij[1][q] - uui[0][q] * uui[1][q];
                L[2] = llij[2][q] - uui[0][q] * uui[2][q];
                L[3] = llij[3][q] - uui[1][q] * uui[1][q];
                L[4] = llij[4][q] - uui[1][q] * uui[2][q];
                L[5] = llij[5][q] - uui[2][q] * uui[2][q];
                double M0 = mmij[0][q], M1 = mmij[1][q], M2 = mmij[2][q], M3 = mmij[3][q], M4 = mmij[4][q], M5 = mmij[5][q];
                double nw = (double)c->nwall[q];
                lm += (2.0 * L[1] * M1 + L[0] * M0 + 2.0 * L[2] * M2 + L[3] * M3 + 2.0 * L[4] * M4 + L[5] * M5) * nw * vol;
                mm += (2.0 * M1 * M1 + M0 * M0 + 2.0 * M2 * M2 + M3 * M3 + 2.0 * M4 * M4 + M5 * M5) * nw * vol;
            }
    for (int q = 0; q < 9; q++) free(aalp[q]);
    for (int q = 0; q < 6; q++) { free(llij[q]); free(mmij[q]); }
    for (int q = 0; q < 3; q++) free(uui[q]);

    double cs = -0.5 * lm / mm;
    c->csgsts = cs > 0.0 ? cs : 0.0;
    #pragma omp parallel for
    for (ll k = 1; k <= n3m; k++)
        for (ll j = 1; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++) c->nusgs[IX(c, i, j, k)] = c->csgsts * c->nusgs[IX(c, i, j, k)];
}

/* nutzero / alpzero, sgs.f90:878-938 / 1528-1588 */
static void zero_in_body(ref_case *c, double *f, double *avg_out, double *max_out)
{
    for (ll l = 1; l <= c->nzero; l++) f[IX(c, c->inz[l], c->jnz[l], c->knz[l])] = 0.0;
    double avg = 0.0, area = 0.0, mx = 0.0;
    for (ll k = 1; k <= c->n3m; k++)
        for (ll j = 1; j <= c->n2m; j++)
            for (ll i = 1; i <= c->n1m; i++) {
                size_t q = IX(c, i, j, k);
                if (c->fb_c[q] >= 1.0e-10) {
                    double vol = c->f2fx[i] * c->f2fy[j] * c->f2fz[k];
                    avg += f[q] * vol;
                    area += vol;
                    if (f[q] > mx) mx = f[q];
                } else {
                    f[q] = 0.0;
                }
            }
    *avg_out = avg / area;
    *max_out = mx;
}

/* nutinterpol / alpinterpol, sgs.f90:941-1133 / 1591-1773: cell-centre
   viscosity to the three edge locations.  'full' selects the alpinterpol
   index ranges (all of 1..n?m) instead of the *_bgp? starts. */
static void edge_interpol(ref_case *c, double *f, double *f1[3], int full)
{
    const lesgpu_config *g = &c->c;
    ll n1 = c->n1, n2 = c->n2, n3 = c->n3, n1m = c->n1m, n2m = c->n2m, n3m = c->n3m;
    for (int l = 0; l < 3; l++) memset(f1[l], 0, c->nt * sizeof(double));
    if (g->xprdic == 1)
        for (ll k = 0; k <= n3; k++)
            for (ll j = 0; j <= n2; j++) { f[IX(c, 0, j, k)] = f[IX(c, n1m, j, k)]; f[IX(c, n1, j, k)] = f[IX(c, 1, j, k)]; }
    if (g->yprdic == 1)
        for (ll k = 0; k <= n3; k++)
            for (ll i = 0; i <= n1; i++) { f[IX(c, i, 0, k)] = f[IX(c, i, n2m, k)]; f[IX(c, i, n2, k)] = f[IX(c, i, 1, k)]; }
    if (g->zprdic == 1)
        for (ll j = 0; j <= n2; j++)
            for (ll i = 0; i <= n1; i++) { f[IX(c, i, j, 0)] = f[IX(c, i, j, n3m)]; f[IX(c, i, j, n3)] = f[IX(c, i, j, 1)]; }
    ll ib = full ? 1 : c->i_bgpx, jb = full ? 1 : c->j_bgpy, kb = full ? 1 : c->k_bgpz;
    const double *f2fx = c->f2fx, *f2fy = c->f2fy, *f2fz = c->f2fz;
    #pragma omp parallel for
    for (ll k = kb; k <= n3m; k++)
        for (ll j = jb; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++)
                f1[0][IX(c, i, j, k)] = c->c2cyi[j] * c->c2czi[k] * 0.25
                    * (f2fy[j - 1] * (f2fz[k - 1] * f[IX(c, i, j, k)] + f2fz[k] * f[IX(c, i, j, k - 1)])
                       + f2fy[j] * (f2fz[k - 1] * f[IX(c, i, j - 1, k)] + f2fz[k] * f[IX(c, i, j - 1, k - 1)]));
    #pragma omp parallel for
    for (ll k = kb; k <= n3m; k++)
        for (ll j = 1; j <= n2m; j++)
            for (ll i = ib; i <= n1m; i++)
                f1[1][IX(c, i, j, k)] = c->c2czi[k] * c->c2cxi[i] * 0.25
                    * (f2fz[k - 1] * (f2fx[i - 1] * f[IX(c, i, j, k)] + f2fx[i] * f[IX(c, i - 1, j, k)])
                       + f2fz[k] * (f2fx[i - 1] * f[IX(c, i, j, k - 1)] + f2fx[i] * f[IX(c, i - 1, j, k - 1)]));
    #pragma omp parallel for
    for (ll k = 1; k <= n3m; k++)
        for (ll j = jb; j <= n2m; j++)
            for (ll i = ib; i <= n1m; i++)
                f1[2][IX(c, i, j, k)] = c->c2cxi[i] * c->c2cyi[j] * 0.25
                    * (f2fx[i - 1] * (f2fy[j - 1] * f[IX(c, i, j, k)] + f2fy[j] * f[IX(c, i, j - 1, k)])
                       + f2fx[i] * (f2fy[j - 1] * f[IX(c, i - 1, j, k)] + f2fy[j] * f[IX(c, i - 1, j - 1, k)]));

    /* x boundaries */
    for (ll j = jb; j <= n2m; j++)
        for (ll k = kb; k <= n3m; k++) {
            ll jm = c->jmv[j], km = c->kmv[k];
            if (g->xprdic == 1) {
                for (int l = 0; l < 3; l++) f1[l][IX(c, n1, j, k)] = f1[l][IX(c, 1, j, k)];
            } else {
                /* readbcs (misc_init.f90:124-130) makes a non-periodic x
                   direction an inlet (2) and a convective outlet (3), so the
                   wall branch (bc == 0) of the reference never applies */
                f1[1][IX(c, 1, j, k)] = c->c2czi[k] * 0.5 * (f2fz[k] * f[IX(c, 2, j, km)] + f2fz[km] * f[IX(c, 2, j, k)]);
                f1[2][IX(c, 1, j, k)] = c->c2cyi[j] * 0.5 * (f2fy[j] * f[IX(c, 2, jm, k)] + f2fy[jm] * f[IX(c, 2, j, k)]);
                f1[1][IX(c, n1, j, k)] = c->c2czi[k] * 0.5 * (f2fz[k] * f[IX(c, n1m, j, km)] + f2fz[km] * f[IX(c, n1m, j, k)]);
                f1[2][IX(c, n1, j, k)] = c->c2cyi[j] * 0.5 * (f2fy[j] * f[IX(c, n1m, jm, k)] + f2fy[jm] * f[IX(c, n1m, j, k)]);
            }
        }
    /* y boundaries */
    for (ll k = kb; k <= n3m; k++)
        for (ll i = ib; i <= n1m; i++) {
            ll im = c->imv[i], km = c->kmv[k];
            if (g->yprdic == 1) {
                for (int l = 0; l < 3; l++) f1[l][IX(c, i, n2, k)] = f1[l][IX(c, i, 1, k)];
            } else {
                if (g->bc_ybtm == 0) {
                    for (int l = 0; l < 3; l++) f1[l][IX(c, i, 1, k)] = 0.0;
                } else {
                    f1[1][IX(c, i, 1, k)] = c->c2czi[k] * 0.5 * (f2fz[k] * f[IX(c, i, 2, km)] + f2fz[km] * f[IX(c, i, 2, k)]);
                    f1[2][IX(c, i, 1, k)] = c->c2cxi[i] * 0.5 * (f2fx[i] * f[IX(c, im, 2, k)] + f2fx[im] * f[IX(c, i, 2, k)]);
                }
                if (g->bc_ytop == 0) {
                    for (int l = 0; l < 3; l++) f1[l][IX(c, i, n2, k)] = 0.0;
                } else {
                    f1[1][IX(c, i, n2, k)] = c->c2czi[k] * 0.5 * (f2fz[k] * f[IX(c, i, n2m, km)] + f2fz[km] * f[IX(c, i, n2m, k)]);
                    f1[2][IX(c, i, n2, k)] = c->c2cxi[i] * 0.5 * (f2fx[i] * f[IX(c, im, n2m, k)] + f2fx[im] * f[IX(c, i, n2m, k)]);
                }
            }
        }
    /* z boundaries.  nutinterpol's z-top branch reads c2cyi(k) with k left at
       n3 by the preceding loop (sgs.f90:1124); alpinterpol reads c2cyi(j). */
    for (ll i = ib; i <= n1m; i++)
        for (ll j = jb; j <= n2m; j++) {
            ll im = c->imv[i], jm = c->jmv[j];
            if (g->zprdic == 1) {
                for (int l = 0; l < 3; l++) f1[l][IX(c, i, j, n3)] = f1[l][IX(c, i, j, 1)];
            } else {
                if (g->bc_zbtm == 0) {
                    for (int l = 0; l < 3; l++) f1[l][IX(c, i, j, 1)] = 0.0;
                } else {
                    f1[1][IX(c, i, j, 1)] = c->c2cyi[j] * 0.5 * (f2fy[j] * f[IX(c, i, jm, 2)] + f2fy[jm] * f[IX(c, i, j, 2)]);
                    f1[2][IX(c, i, j, 1)] = c->c2cxi[i] * 0.5 * (f2fx[i] * f[IX(c, im, j, 2)] + f2fx[im] * f[IX(c, i, j, 2)]);
                }
                if (g->bc_ztop == 0) {
                    for (int l = 0; l < 3; l++) f1[l][IX(c, i, j, n3)] = 0.0;
                } else {
                    double cyk = full ? c->c2cyi[j] : (n3 <= n2 ? c->c2cyi[n3] : 0.0);
                    f1[1][IX(c, i, j, n3)] = cyk * 0.5 * (f2fy[j] * f[IX(c, i, jm, n3m)] + f2fy[jm] * f[IX(c, i, j, n3m)]);
                    f1[2][IX(c, i, j, n3)] = c->c2cxi[i] * 0.5 * (f2fx[i] * f[IX(c, im, j, n3m)] + f2fx[im] * f[IX(c, i, j, n3m)]);
                }
            }
        }
}

/* sgscalc, sgs.f90:288-332 */
void ref_sgscalc(ref_case *c)
{
    if (c->msub != 1) return;
    if (c->c.iread == 0 && c->ntime == 1) {
        memset(c->nusgs, 0, c->nt * sizeof(double));
    } else {
        if (c->c.idvmon == 1) sgs_dvmg(c);
        else sgs_cvm(c);
    }
    zero_in_body(c, c->nusgs, &c->nutavg, &c->nutmax);
    c->nutavg *= c->c.re;
    c->nutmax *= c->c.re;
    edge_interpol(c, c->nusgs, c->nusgs1, 0);
}

/* sgs_cedm, sgs.f90:1250-1294 */
static void sgs_cedm(ref_case *c)
{
    #pragma omp parallel for
    for (ll k = 1; k <= c->n3m; k++)
        for (ll j = 1; j <= c->n2m; j++)
            for (ll i = 1; i <= c->n1m; i++) {
                double d[9], s[6];
                ref_velgrad(c, i, j, k, d, s);
                double del = pow(c->f2fx[i] * c->f2fy[j] * c->f2fz[k], 1.0 / 3.0);
                double sss = s[0] * s[0] + 2.0 * s[1] * s[1] + 2.0 * s[2] * s[2] + s[3] * s[3] + 2.0 * s[4] * s[4] + s[5] * s[5];
                if (sss < 1.0e-16) sss = 1.0e-16;
                c->alsgs[IX(c, i, j, k)] = c->c.csgshf * (del * del) * sqrt(2.0 * sss);
            }
}

/* sgs_edm, sgs.f90:1297-1478 */
static void sgs_edm(ref_case *c)
{
    ll n1m = c->n1m, n2m = c->n2m, n3m = c->n3m;
    size_t nt = c->nt;
    double *aalp[9], *llij[3], *mmij[3], *uui[3];
    for (int q = 0; q < 9; q++) aalp[q] = ref_zalloc(nt);
    for (int q = 0; q < 3; q++) { llij[q] = ref_zalloc(nt); mmij[q] = ref_zalloc(nt); uui[q] = ref_zalloc(nt); }
    c->csgshf = 0.0;

    #pragma omp parallel for
    for (ll k = 1; k <= n3m; k++)
        for (ll j = 1; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++) {
                double d[9], s[6], alp[3];
                ref_velgrad(c, i, j, k, d, s);
                temgrad(c, i, j, k, alp);
                double del = pow(c->f2fx[i] * c->f2fy[j] * c->f2fz[k], 1.0 / 3.0);
                double sss = s[0] * s[0] + 2.0 * s[1] * s[1] + 2.0 * s[2] * s[2] + s[3] * s[3] + 2.0 * s[4] * s[4] + s[5] * s[5];
                if (sss < 1.0e-16) sss = 1.0e-16;
                size_t q = IX(c, i, j, k);
                double al = (del * del) * sqrt(2.0 * sss);
                c->alsgs[q] = al;
                for (int m = 0; m < 3; m++) mmij[m][q] = al * alp[m];
                for (int m = 0; m < 6; m++) aalp[m][q] = s[m];
                for (int m = 0; m < 3; m++) aalp[6 + m][q] = alp[m];
            }

    #pragma omp parallel
    {
        double *tmp = ref_zalloc(nt), *src = ref_zalloc(nt);
        #pragma omp for
        for (int m = 0; m < 12; m++) {
            if (m < 3) ref_test_filter(c, mmij[m], tmp, src);
            else ref_test_filter(c, aalp[m - 3], tmp, src);
        }
        free(tmp); free(src);
    }

    #pragma omp parallel for
    for (ll k = 1; k <= n3m; k++)
        for (ll j = 1; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++) {
                size_t q = IX(c, i, j, k);
                double d1 = 0.5 * c->f2fx[i - 1] * (1.0 - (double)c->fixiu[i]) + c->f2fx[i] + 0.5 * c->f2fx[i + 1] * (1.0 - (double)c->fixil[i]);
                double d2 = 0.5 * c->f2fy[j - 1] * (1.0 - (double)c->fixju[j]) + c->f2fy[j] + 0.5 * c->f2fy[j + 1] * (1.0 - (double)c->fixjl[j]);
                double d3 = 0.5 * c->f2fz[k - 1] * (1.0 - (double)c->fixku[k]) + c->f2fz[k] + 0.5 * c->f2fz[k + 1] * (1.0 - (double)c->fixkl[k]);
                double del = pow(d1 * d2 * d3, 1.0 / 3.0);
                double sss = aalp[0][q] * aalp[0][q] + 2.0 * aalp[1][q] * aalp[1][q] + 2.0 * aalp[2][q] * aalp[2][q]
                           + aalp[3][q] * aalp[3][q] + 2.0 * aalp[4][q] * aalp[4][q] + aalp[5][q] * aalp[5][q];
                if (sss < 1.0e-16) sss = 1.0e-16;
                double ami = (del * del) * sqrt(2.0 * sss);
                for (int m = 0; m < 3; m++) mmij[m][q] = ami * aalp[6 + m][q] - mmij[m][q];
                double u1 = 0.5 * (c->u[q] + c->u[IX(c, i + 1, j, k)]);
                double u2 = 0.5 * (c->v[q] + c->v[IX(c, i, j + 1, k)]);
                double u3 = 0.5 * (c->w[q] + c->w[IX(c, i, j, k + 1)]);
                uui[0][q] = u1; uui[1][q] = u2; uui[2][q] = u3;
                double tt = c->t[q];
                aalp[0][q] = tt; aalp[1][q] = tt; aalp[2][q] = tt;
                llij[0][q] = u1 * tt; llij[1][q] = u2 * tt; llij[2][q] = u3 * tt;
            }

    #pragma omp parallel
    {
        double *tmp = ref_zalloc(nt), *src = ref_zalloc(nt);
        #pragma omp for
        for (int m = 0; m < 9; m++) {
            if (m < 3) ref_test_filter(c, uui[m], tmp, src);
            else if (m < 6) ref_test_filter(c, aalp[m - 3], tmp, src);
            else ref_test_filter(c, llij[m - 6], tmp, src);
        }
        free(tmp); free(src);
    }

    double lm = 0.0, mm = 0.0;
    #pragma omp parallel for reduction(+:lm, mm)
    for (ll k = 1; k <= n3m; k++)
        for (ll j = 1; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++) {
                size_t q = IX(c, i, j, k);
                double vol = c->f2fx[i] * c->f2fy[j] * c->f2fz[k];
                double L0 = llij[0][q] - uui[0][q] * aalp[0][q];
                double L1 = llij[1][q] - uui[1][q] * aalp[1][q];
                double L2 = llij[2][q] - uui[2][q] * aalp[2][q];
                double nw = (double)c->nwall[q];
                lm += (L0 * mmij[0][q] + L1 * mmij[1][q] + L2 * mmij[2][q]) * nw * vol;
                mm += (mmij[0][q] * mmij[0][q] + mmij[1][q] * mmij[1][q] + mmij[2][q] * mmij[2][q]) * nw * vol;
            }
    for (int q = 0; q < 9; q++) free(aalp[q]);
    for (int q = 0; q < 3; q++) { free(llij[q]); free(mmij[q]); free(uui[q]); }
    double cs = -lm / mm;
    c->csgshf = cs > 0.0 ? cs : 0.0;
    #pragma omp parallel for
    for (ll k = 1; k <= n3m; k++)
        for (ll j = 1; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++) c->alsgs[IX(c, i, j, k)] = c->csgshf * c->alsgs[IX(c, i, j, k)];
}

/* sgscalc_t, sgs.f90:1203-1247 */
void ref_sgscalc_t(ref_case *c)
{
    if (c->msub != 1) return;
    if (c->c.iread == 0 && c->ntime == 1) {
        memset(c->alsgs, 0, c->nt * sizeof(double));
    } else {
        if (c->c.idvmon == 1) sgs_edm(c);
        else sgs_cedm(c);
    }
    zero_in_body(c, c->alsgs, &c->alpavg, &c->alpmax);
    c->alpavg *= c->c.re * c->c.pr;
    c->alpmax *= c->c.re * c->c.pr;
    edge_interpol(c, c->alsgs, c->alsgs1, 1);
}

/* rhssgs, sgs.f90:1136-1200: off-diagonal SGS stress divergence */
void ref_rhssgs(ref_case *c)
{
    ll n1m = c->n1m, n2m = c->n2m, n3m = c->n3m;
    double *u = c->u, *v = c->v, *w = c->w;
    double *n1_ = c->nusgs1[0], *n2_ = c->nusgs1[1], *n3_ = c->nusgs1[2];
    #pragma omp parallel for
    for (ll k = 1; k <= n3m; k++)
        for (ll j = 1; j <= n2m; j++)
            for (ll i = c->i_bgpx; i <= n1m; i++) {
                double a = c->f2fyi[j] * c->c2cxi[i] * (n3_[IX(c, i, j + 1, k)] * (v[IX(c, i, j + 1, k)] - v[IX(c, i - 1, j + 1, k)])
                                                        - n3_[IX(c, i, j, k)] * (v[IX(c, i, j, k)] - v[IX(c, i - 1, j, k)]));
                double b = c->f2fzi[k] * c->c2cxi[i] * (n2_[IX(c, i, j, k + 1)] * (w[IX(c, i, j, k + 1)] - w[IX(c, i - 1, j, k + 1)])
                                                        - n2_[IX(c, i, j, k)] * (w[IX(c, i, j, k)] - w[IX(c, i - 1, j, k)]));
                c->rhs1[0][IX(c, i, j, k)] = a + b;
            }
    #pragma omp parallel for
    for (ll k = 1; k <= n3m; k++)
        for (ll j = c->j_bgpy; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++) {
                double a = c->f2fxi[i] * c->c2cyi[j] * (n3_[IX(c, i + 1, j, k)] * (u[IX(c, i + 1, j, k)] - u[IX(c, i + 1, j - 1, k)])
                                                        - n3_[IX(c, i, j, k)] * (u[IX(c, i, j, k)] - u[IX(c, i, j - 1, k)]));
                double b = c->f2fzi[k] * c->c2cyi[j] * (n1_[IX(c, i, j, k + 1)] * (w[IX(c, i, j, k + 1)] - w[IX(c, i, j - 1, k + 1)])
                                                        - n1_[IX(c, i, j, k)] * (w[IX(c, i, j, k)] - w[IX(c, i, j - 1, k)]));
                c->rhs1[1][IX(c, i, j, k)] = a + b;
            }
    #pragma omp parallel for
    for (ll k = c->k_bgpz; k <= n3m; k++)
        for (ll j = 1; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++) {
                double a = c->f2fxi[i] * c->c2czi[k] * (n2_[IX(c, i + 1, j, k)] * (u[IX(c, i + 1, j, k)] - u[IX(c, i + 1, j, k - 1)])
                                                        - n2_[IX(c, i, j, k)] * (u[IX(c, i, j, k)] - u[IX(c, i, j, k - 1)]));
                double b = c->f2fyi[j] * c->c2czi[k] * (n1_[IX(c, i, j + 1, k)] * (v[IX(c, i, j + 1, k)] - v[IX(c, i, j + 1, k - 1)])
                                                        - n1_[IX(c, i, j, k)] * (v[IX(c, i, j, k)] - v[IX(c, i, j, k - 1)]));
                c->rhs1[2][IX(c, i, j, k)] = a + b;
            }
}
