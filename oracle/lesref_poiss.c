/*
 * ORACLE -- test infrastructure only (see lesref_internal.h).
 *
 * Pressure Poisson solvers: 02_solver/f90/lib/poiss/poiss_ftft.f90 (FFT x & z,
 * Thomas y), poiss_z_ft.f90 (FFT z, 2-D multigrid x-y) and poiss_mgrd.f90
 * (BiCGSTAB with one MG3D V-cycle as preconditioner).
 *
 * The FFT is this file's own mixed-radix (2,3,4,5 and a direct DFT for other
 * factors) transform with the conventions of FFTE 7.0's ZFFT1D (vendored at
 * 02_solver/f90/lib/poiss/ffte-7.0/zfft1d.f:18-84): IOPT = -1 is the forward
 * transform A_k = sum_n a_n exp(-2 pi i n k / N), unnormalised; IOPT = +1 is
 * conj -> forward -> conj -> scale by 1/N.
 */
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "lesref_internal.h"
#include "lesref.h"

/* ---------------------------------------------------------------- FFT -- */
int ref_fft_plan_init(ref_fft_plan *p, int n)
{
    memset(p, 0, sizeof(*p));
    if (n < 1) return LESGPU_ERR_ARG;
    p->n = n;
    int m = n;
    while (m > 1) {
        int r;
        if (m % 4 == 0) r = 4;
        else if (m % 2 == 0) r = 2;
        else if (m % 3 == 0) r = 3;
        else if (m % 5 == 0) r = 5;
        else r = m;                       /* remaining prime: direct DFT */
        p->fac[p->nfac++] = r;
        m /= r;
    }
    p->tw = (cplx *)malloc(sizeof(cplx) * (size_t)n);
    for (int e = 0; e < n; e++) {
        long double ang = -2.0L * 3.14159265358979323846264338327950288L * (long double)e / (long double)n;
        p->tw[e].re = (double)cosl(ang);
        p->tw[e].im = (double)sinl(ang);
    }
    return 0;
}

void ref_fft_plan_free(ref_fft_plan *p)
{
    free(p->tw);
    p->tw = NULL;
}

/* decimation in time: x (stride s) -> y (contiguous, length m) */
static void fft_rec(const ref_fft_plan *p, const cplx *x, cplx *y, int m, int s, int fi, cplx *tmp)
{
    if (m == 1) { y[0] = x[0]; return; }
    int r = p->fac[fi], q = m / r;
    for (int a = 0; a < r; a++) fft_rec(p, x + (size_t)a * s, y + (size_t)a * q, q, s * r, fi + 1, tmp);
    int step = p->n / m;               /* W_m^e = tw[e*step] */
    for (int k = 0; k < q; k++) {
        cplx t[64];
        for (int a = 0; a < r; a++) {
            cplx v = y[(size_t)a * q + k];
            int e = (a * k) % m;
            cplx w = p->tw[(size_t)e * step];
            t[a].re = v.re * w.re - v.im * w.im;
            t[a].im = v.re * w.im + v.im * w.re;
        }
        for (int b = 0; b < r; b++) {
            cplx acc = { 0.0, 0.0 };
            for (int a = 0; a < r; a++) {
                int e = ((a * b) % r) * (p->n / r);
                cplx w = p->tw[e];
                acc.re += t[a].re * w.re - t[a].im * w.im;
                acc.im += t[a].re * w.im + t[a].im * w.re;
            }
            tmp[(size_t)b * q + k] = acc;
        }
    }
    memcpy(y, tmp, sizeof(cplx) * (size_t)m);
}

void ref_fft(const ref_fft_plan *p, cplx *a, cplx *work, int iopt)
{
    int n = p->n;
    if (n == 1) return;
    cplx *y = work, *tmp = work + n;
    if (iopt == 1)
        for (int i = 0; i < n; i++) a[i].im = -a[i].im;
    fft_rec(p, a, y, n, 1, 0, tmp);
    if (iopt == 1) {
        double dn = 1.0 / (double)n;
        for (int i = 0; i < n; i++) { a[i].re = y[i].re * dn; a[i].im = -y[i].im * dn; }
    } else {
        memcpy(a, y, sizeof(cplx) * (size_t)n);
    }
}

int ref_fft_1d(int n, const double *in, double *out, int iopt)
{
    ref_fft_plan p;
    if (ref_fft_plan_init(&p, n)) return LESGPU_ERR_ARG;
    for (int f = 0; f < p.nfac; f++)
        if (p.fac[f] > 64) { ref_fft_plan_free(&p); return LESGPU_ERR_ARG; }
    cplx *a = (cplx *)malloc(sizeof(cplx) * n), *wk = (cplx *)malloc(sizeof(cplx) * 2 * n);
    for (int i = 0; i < n; i++) { a[i].re = in[2 * i]; a[i].im = in[2 * i + 1]; }
    ref_fft(&p, a, wk, iopt);
    for (int i = 0; i < n; i++) { out[2 * i] = a[i].re; out[2 * i + 1] = a[i].im; }
    free(a); free(wk);
    ref_fft_plan_free(&p);
    return 0;
}

/* -------------------------------------------------------- poiss_ftft -- */

/* poisinit, poiss_ftft.f90:164-204: modified wavenumbers */
static void ftft_init(ref_case *c)
{
    ll n1m = c->n1m, n3m = c->n3m, n1mh = c->n1mh, n3mh = c->n3mh;
    double pi = 2.0 * asin(1.0);
    c->ak1 = ref_zalloc(c->n1 + 2);
    c->ak3 = ref_zalloc(n3mh + 2);
    double sdzis = c->f2fzi[1], sdxis = c->f2fxi[1];
    for (ll k = 1; k <= n3mh; k++) {
        double ai = (k == 1) ? 0.0 : (double)(k - 1) * 2.0 * pi;
        c->ak3[k] = 2.0 * (1.0 - cos(ai / (double)n3m)) * sdzis * sdzis;
    }
    for (ll i = 1; i <= n1mh; i++) {
        double ai = (i == 1) ? 0.0 : (double)(i - 1) * 2.0 * pi;
        c->ak1[i] = 2.0 * (1.0 - cos(ai / (double)n1m)) * sdxis * sdxis;
    }
    for (ll i = n1m; i >= n1mh + 1; i--) c->ak1[i] = c->ak1[n1m + 2 - i];
}

/* ctrdiag, poiss_ftft.f90:207-244: one complex line, real coefficients */
static void ctrdiag_line(const double *a, const double *b, const double *cc, cplx *r, double *gam, ll ni, ll nf)
{
    double bet = 1.0 / b[ni];
    r[ni].re *= bet; r[ni].im *= bet;
    for (ll j = ni + 1; j <= nf; j++) {
        gam[j] = cc[j - 1] * bet;
        bet = 1.0 / (b[j] - a[j] * gam[j]);
        r[j].re = (r[j].re - a[j] * r[j - 1].re) * bet;
        r[j].im = (r[j].im - a[j] * r[j - 1].im) * bet;
    }
    for (ll j = nf - 1; j >= ni; j--) {
        r[j].re -= gam[j + 1] * r[j + 1].re;
        r[j].im -= gam[j + 1] * r[j + 1].im;
    }
}

/* poisson, poiss_ftft.f90:21-161 */
static void ftft_poisson(ref_case *c)
{
    ll n1m = c->n1m, n2m = c->n2m, n3m = c->n3m, n3mh = c->n3mh;
    size_t sk = (size_t)n3mh, ski = sk * (size_t)n1m;
    cplx *ccap = (cplx *)malloc(sizeof(cplx) * ski * (size_t)(n2m + 1));
#define CC(k, i, j) ccap[(size_t)((k) - 1) + sk * (size_t)((i) - 1) + ski * (size_t)(j)]
    #pragma omp parallel
    {
        cplx *zzz = (cplx *)malloc(sizeof(cplx) * (size_t)n3m * (size_t)n1m);
        cplx *xx = (cplx *)malloc(sizeof(cplx) * (size_t)n1m);
        cplx *wk = (cplx *)malloc(sizeof(cplx) * 2 * (size_t)(n1m > n3m ? n1m : n3m));
        #pragma omp for
        for (ll j = 1; j <= n2m; j++) {
            for (ll k = 1; k <= n3m; k++)
                for (ll i = 1; i <= n1m; i++) {
                    cplx *z = &zzz[(size_t)(k - 1) + (size_t)n3m * (size_t)(i - 1)];
                    z->re = c->divgsum[IX(c, i, j, k)]; z->im = 0.0;
                }
            for (ll i = 1; i <= n1m; i++) ref_fft(&c->fftz, &zzz[(size_t)n3m * (size_t)(i - 1)], wk, -1);
            for (ll k = 1; k <= n3mh; k++) {
                for (ll i = 1; i <= n1m; i++) xx[i - 1] = zzz[(size_t)(k - 1) + (size_t)n3m * (size_t)(i - 1)];
                ref_fft(&c->fftx, xx, wk, -1);
                for (ll i = 1; i <= n1m; i++) CC(k, i, j) = xx[i - 1];
            }
        }
        free(zzz); free(xx); free(wk);
    }

    #pragma omp parallel
    {
        double *am = ref_zalloc(n2m + 2), *ap = ref_zalloc(n2m + 2), *ac = ref_zalloc(n2m + 2), *gam = ref_zalloc(n2m + 2);
        cplx *cr = (cplx *)malloc(sizeof(cplx) * (size_t)(n2m + 2));
        #pragma omp for
        for (ll k = 1; k <= n3mh; k++)
            for (ll i = 1; i <= n1m; i++) {
                for (ll j = 1; j <= n2m; j++) {
                    ll jjp = c->jpv[j];
                    double fl = (double)c->fixjl[j], fu = (double)c->fixju[j];
                    am[j] = c->f2fyi[j] * c->c2cyi[j] * (1.0 - fl);
                    ap[j] = c->f2fyi[j] * c->c2cyi[jjp] * (1.0 - fu);
                    double akk = c->ak1[i] + c->ak3[k];
                    ac[j] = -((am[j] + ap[j] + akk) * (1.0 - fl) * (1.0 - fu)
                              + (c->f2fyi[1] * c->c2cyi[2] + akk) * fl
                              + (c->f2fyi[n2m] * c->c2cyi[n2m] + akk) * fu);
                    cr[j] = CC(k, i, j);
                }
                if (k == 1 && i == 1) {
                    cplx crhsref = cr[n2m];
                    double ajcref = ac[n2m], ajmref = am[n2m];
                    cr[n2m].re = 0.0; cr[n2m].im = 0.0;
                    ac[n2m] = 1.0; am[n2m] = 0.0; ap[n2m] = 0.0;
                    ctrdiag_line(am, ac, ap, cr, gam, 1, n2m);
                    cplx phref;
                    phref.re = (-ajmref * cr[n2m - 1].re + crhsref.re) / ajcref;
                    phref.im = (-ajmref * cr[n2m - 1].im + crhsref.im) / ajcref;
                    for (ll j = 1; j <= n2m; j++) { cr[j].re -= phref.re; cr[j].im -= phref.im; }
                    cr[n2m].re = 0.0; cr[n2m].im = 0.0;
                } else {
                    ctrdiag_line(am, ac, ap, cr, gam, 1, n2m);
                }
                for (ll j = 1; j <= n2m; j++) CC(k, i, j) = cr[j];
            }
        free(am); free(ap); free(ac); free(gam); free(cr);
    }

    #pragma omp parallel
    {
        cplx *zzz = (cplx *)malloc(sizeof(cplx) * (size_t)n3m * (size_t)n1m);
        cplx *xx = (cplx *)malloc(sizeof(cplx) * (size_t)n1m);
        cplx *wk = (cplx *)malloc(sizeof(cplx) * 2 * (size_t)(n1m > n3m ? n1m : n3m));
        #pragma omp for
        for (ll j = 1; j <= n2m; j++) {
            for (ll k = 1; k <= n3mh; k++) {
                for (ll i = 1; i <= n1m; i++) xx[i - 1] = CC(k, i, j);
                ref_fft(&c->fftx, xx, wk, 1);
                for (ll i = 1; i <= n1m; i++) zzz[(size_t)(k - 1) + (size_t)n3m * (size_t)(i - 1)] = xx[i - 1];
            }
            for (ll i = 1; i <= n1m; i++)
                for (ll k = n3mh + 1; k <= n3m; k++) {
                    cplx s = zzz[(size_t)(n3m + 2 - k - 1) + (size_t)n3m * (size_t)(i - 1)];
                    s.im = -s.im;
                    zzz[(size_t)(k - 1) + (size_t)n3m * (size_t)(i - 1)] = s;
                }
            for (ll i = 1; i <= n1m; i++) {
                ref_fft(&c->fftz, &zzz[(size_t)n3m * (size_t)(i - 1)], wk, 1);
                for (ll k = 1; k <= n3m; k++) c->phi[IX(c, i, j, k)] = zzz[(size_t)(k - 1) + (size_t)n3m * (size_t)(i - 1)].re;
            }
        }
        free(zzz); free(xx); free(wk);
    }
#undef CC
    free(ccap);
}

/* -------------------------------------------------------- poiss_z_ft -- */
/* FFT in z, then for every z-mode a 2-D problem in x-y solved by multigrid
   semi-coarsened in x with zebra x-line relaxation (y-Thomas per line).
   Level ilev occupies x slots iimg[ilev][0]..iimg[ilev][1] of the 1-D
   coefficient vectors; the finest level nlev is 1..n1m. */

#define ZAC(c, i, j, k) ((size_t)((i) - 1) + (size_t)(c)->n1md * ((size_t)((j) - 1) + (size_t)(c)->n2m * (size_t)((k) - 1)))

/* pmat + mwavenumber, poiss_z_ft.f90:55-113 */
static void zft_pmat(ref_case *c)
{
    ll n1m = c->n1m, n2m = c->n2m, n3m = c->n3m;
    for (ll i = 1; i <= n1m; i++) {
        ll ip = c->ipv[i];
        c->aw[i] = (1.0 - (double)c->fixil[i]) * c->c2cxi[i] * c->f2fxi[i];
        c->ae[i] = (1.0 - (double)c->fixiu[i]) * c->c2cxi[ip] * c->f2fxi[i];
    }
    for (ll j = 1; j <= n2m; j++) {
        ll jp = c->jpv[j];
        c->as[j] = (1.0 - (double)c->fixjl[j]) * c->c2cyi[j] * c->f2fyi[j];
        c->an[j] = (1.0 - (double)c->fixju[j]) * c->c2cyi[jp] * c->f2fyi[j];
    }
    for (ll j = 1; j <= n2m; j++)
        for (ll i = 1; i <= n1m; i++)
            c->ac[ZAC(c, i, j, 1)] = -1.0 * (c->aw[i] + c->ae[i] + c->as[j] + c->an[j]);
    if (n3m > 1) {
        double pi = acos(-1.0);
        for (ll k = 1; k <= c->n3mh; k++)
            c->ak3[k] = 2.0 * (1.0 - cos(2.0 * (double)(k - 1) * pi / (double)n3m)) * c->f2fzi[1] * c->f2fzi[1];
    }
    for (ll k = 2; k <= c->n3mh; k++)
        for (ll j = 1; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++) c->ac[ZAC(c, i, j, k)] = c->ac[ZAC(c, i, j, 1)] - c->ak3[k];
}

/* coefmg, poiss_z_ft.f90:643-798 */
static void zft_coefmg(ref_case *c)
{
    ll n1m = c->n1m, n2m = c->n2m, n1md = c->n1md, nlev = c->c.nlev, n1 = c->n1;
    ll minrow = n1m / (1LL << nlev);
    double *xmpm = ref_zalloc((size_t)n1md + 2), *iwz = ref_zalloc((size_t)n1md + 2), *iez = ref_zalloc((size_t)n1md + 2);
    const double *x = c->x;
    c->iimg[nlev][0] = 1; c->iimg[nlev][1] = n1m; c->iimg[nlev][2] = n1m;
    for (ll i = 1; i <= n1m; i++) {
        xmpm[i] = c->xmp[i];
        iwz[i] = (double)(1 - 1 / i);
        iez[i] = (double)(1 - i / n1m);
    }
    for (ll ilev = nlev - 1; ilev >= 0; ilev--) {
        c->iimg[ilev][0] = c->iimg[ilev + 1][0] + c->iimg[ilev + 1][2];
        c->iimg[ilev][2] = minrow * (1LL << ilev);
        c->iimg[ilev][1] = c->iimg[ilev][0] + c->iimg[ilev][2] - 1;
        ll ibg = c->iimg[ilev][0], iend = c->iimg[ilev][1], isp = 1LL << (nlev - ilev);
        ll ic = 0;
        for (ll i = ibg; i <= iend; i++) {
            ic++;
            xmpm[i] = 0.5 * (x[ic * isp + 1] + x[(ic - 1) * isp + 1]);
            iwz[i] = (double)(1 - ibg / i);
            iez[i] = (double)(1 - i / iend);
        }
        ic = 0;
        for (ll i = ibg; i <= iend; i++) {
            ic++;
            double w = x[ic * isp + 1] - x[(ic - 1) * isp + 1];
            c->aw[i] = iwz[i] / ((xmpm[i] - xmpm[i - 1]) * w);
            c->ae[i] = iez[i] / ((xmpm[i + 1] - xmpm[i]) * w);
        }
        for (ll j = 1; j <= n2m; j++)
            for (ll i = ibg; i <= iend; i++)
                c->ac[ZAC(c, i, j, 1)] = -1.0 * (c->aw[i] + c->ae[i] + c->as[j] + c->an[j]);
        for (ll k = 2; k <= c->n3mh; k++)
            for (ll j = 1; j <= n2m; j++)
                for (ll i = ibg; i <= iend; i++) c->ac[ZAC(c, i, j, k)] = c->ac[ZAC(c, i, j, 1)] - c->ak3[k];
    }
    for (ll ilev = nlev; ilev >= 1; ilev--) {
        ll ibgh = c->iimg[ilev][0];
        for (ll i = c->iimg[ilev - 1][0]; i <= c->iimg[ilev - 1][1]; i++) {
            c->cor1[i] = (xmpm[ibgh + 1] - xmpm[i]) / (xmpm[ibgh + 1] - xmpm[ibgh]);
            c->cor2[i] = 1.0 - c->cor1[i];
            ibgh += 2;
        }
    }
    for (ll ilev = 0; ilev <= nlev - 1; ilev++) {
        ll ibgh = c->iimg[ilev + 1][0] + 1;
        for (ll i = c->iimg[ilev][0]; i <= c->iimg[ilev][1] - 1; i++) {
            c->coi1[i] = (xmpm[i + 1] - xmpm[ibgh]) / (xmpm[i + 1] - xmpm[i]);
            c->coi2[i] = 1.0 - c->coi1[i];
            ibgh += 2;
        }
        c->coi1[c->iimg[ilev][1]] = 1.0;
    }
    for (ll ilev = nlev; ilev >= 0; ilev--)
        for (ll i = c->iimg[ilev][0]; i <= c->iimg[ilev][1]; i++) { c->ipm[i] = i + 1; c->imm[i] = i - 1; }
    if (c->c.xprdic == 1) {
        for (ll ilev = nlev; ilev >= 0; ilev--) {
            ll ibg = c->iimg[ilev][0], iend = c->iimg[ilev][1];
            c->ipm[iend] = ibg;
            c->imm[ibg] = iend;
        }
        for (ll ilev = nlev - 1; ilev >= 0; ilev--) {
            ll ibg = c->iimg[ilev][0], iend = c->iimg[ilev][1], isp = 1LL << (nlev - ilev);
            double vdx = xmpm[ibg] - x[1] + x[n1] - xmpm[iend];
            double sdx_b = x[1 + isp] - x[1], sdx_e = x[n1] - x[n1 - isp];
            c->aw[ibg] = 1.0 / (vdx * sdx_b);
            c->ae[iend] = 1.0 / (vdx * sdx_e);
        }
        for (ll ilev = nlev - 1; ilev >= 0; ilev--) {
            for (ll j = 1; j <= n2m; j++)
                for (ll i = c->iimg[ilev][0]; i <= c->iimg[ilev][1]; i++)
                    c->ac[ZAC(c, i, j, 1)] = -1.0 * (c->aw[i] + c->ae[i] + c->as[j] + c->an[j]);
            for (ll k = 2; k <= c->n3mh; k++)
                for (ll j = 1; j <= n2m; j++)
                    for (ll i = c->iimg[ilev][0]; i <= c->iimg[ilev][1]; i++)
                        c->ac[ZAC(c, i, j, k)] = c->ac[ZAC(c, i, j, 1)] - c->ak3[k];
        }
        for (ll ilev = 0; ilev <= nlev - 1; ilev++) {
            ll ibg = c->iimg[ilev][0], iend = c->iimg[ilev][1];
            double vdx = xmpm[ibg] - x[1] + x[n1] - xmpm[iend];
            c->coi2[iend] = (xmpm[c->iimg[ilev + 1][1]] - xmpm[iend]) / vdx;
            c->coi1[iend] = 1.0 - c->coi2[iend];
        }
    }
    free(xmpm); free(iwz); free(iez);
}

/* poisinit, poiss_z_ft.f90:18-52 */
static int zft_init(ref_case *c)
{
    ll n1md = c->n1md, n2m = c->n2m, n3mh = c->n3mh, nlev = c->c.nlev;
    if (nlev < 1 || nlev > 20 || c->n1m % (1LL << nlev) != 0) return LESGPU_ERR_CONFIG;
    if (c->n3m > 1 && ref_fft_plan_init(&c->fftz, (int)c->n3m)) return LESGPU_ERR_ARG;
    size_t nv = (size_t)n1md + 2, na = (size_t)n1md * (size_t)n2m * (size_t)n3mh;
    c->aw = ref_zalloc(nv); c->ae = ref_zalloc(nv);
    c->as = ref_zalloc((size_t)n2m + 2); c->an = ref_zalloc((size_t)n2m + 2);
    c->coi1 = ref_zalloc(nv); c->coi2 = ref_zalloc(nv); c->cor1 = ref_zalloc(nv); c->cor2 = ref_zalloc(nv);
    c->ipm = ref_izalloc(nv); c->imm = ref_izalloc(nv);
    c->ak3 = ref_zalloc((size_t)n3mh + 2);
    c->ac = ref_zalloc(na); c->gam = ref_zalloc(na); c->bet = ref_zalloc(na);
    zft_pmat(c);
    zft_coefmg(c);
    for (ll ilev = 0; ilev <= nlev; ilev++)
        for (ll k = 1; k <= n3mh; k++) {
            for (ll i = c->iimg[ilev][0]; i <= c->iimg[ilev][1]; i++) c->bet[ZAC(c, i, 1, k)] = 1.0 / c->ac[ZAC(c, i, 1, k)];
            for (ll j = 2; j <= n2m; j++)
                for (ll i = c->iimg[ilev][0]; i <= c->iimg[ilev][1]; i++) {
                    c->gam[ZAC(c, i, j, k)] = c->an[j - 1] * c->bet[ZAC(c, i, j - 1, k)];
                    c->bet[ZAC(c, i, j, k)] = 1.0 / (c->ac[ZAC(c, i, j, k)] - c->as[j] * c->gam[ZAC(c, i, j, k)]);
                }
        }
    return 0;
}

/* Work arrays of one mode: pc(0:n1,0:n2), rhs(n1,n2), resd(n1md,n2m), ggii(0:n1md,0:n2). */
typedef struct {
    ll ld_p, ld_g;            /* leading dimensions: n1+1 and n1md+1 */
    cplx *pc, *rhs, *resd, *gg;
} zmode;

#define PC(z, i, j) (z)->pc[(size_t)(i) + (size_t)(z)->ld_p * (size_t)(j)]
#define RH(z, i, j) (z)->rhs[(size_t)(i) + (size_t)(z)->ld_p * (size_t)(j)]
#define RS(z, i, j) (z)->resd[(size_t)(i) + (size_t)(z)->ld_g * (size_t)(j)]
#define GG(z, i, j) (z)->gg[(size_t)(i) + (size_t)(z)->ld_g * (size_t)(j)]

static inline cplx cx_axpy(cplx y, double a, cplx x) { cplx r = { y.re - a * x.re, y.im - a * x.im }; return r; }

/* trdiag1m, poiss_z_ft.f90:383-408: y-Thomas on x-lines l1, l1+2, ..., l2 (in place) */
static void zft_trdiag(const ref_case *c, zmode *z, ll l1, ll l2, ll kv)
{
    ll n2m = c->n2m;
    for (ll i = l1; i <= l2; i += 2) {
        double b = c->bet[ZAC(c, i, 1, kv)];
        GG(z, i, 1).re *= b; GG(z, i, 1).im *= b;
    }
    for (ll j = 2; j <= n2m; j++)
        for (ll i = l1; i <= l2; i += 2) {
            double b = c->bet[ZAC(c, i, j, kv)];
            cplx t = cx_axpy(GG(z, i, j), c->as[j], GG(z, i, j - 1));
            GG(z, i, j).re = t.re * b; GG(z, i, j).im = t.im * b;
        }
    for (ll j = n2m - 1; j >= 1; j--)
        for (ll i = l1; i <= l2; i += 2)
            GG(z, i, j) = cx_axpy(GG(z, i, j), c->gam[ZAC(c, i, j + 1, kv)], GG(z, i, j + 1));
}

/* rhs - aw*g(imm) - ae*g(ipm) - as*g(j-1) - an*g(j+1) - ac*g */
static inline cplx zft_defect(const ref_case *c, cplx r, const cplx *g, ll ld, ll i, ll j, ll kv)
{
    const cplx *gm = &g[(size_t)c->imm[i] + (size_t)ld * (size_t)j], *gp = &g[(size_t)c->ipm[i] + (size_t)ld * (size_t)j];
    const cplx *gs = &g[(size_t)i + (size_t)ld * (size_t)(j - 1)], *gn = &g[(size_t)i + (size_t)ld * (size_t)(j + 1)];
    const cplx *gc = &g[(size_t)i + (size_t)ld * (size_t)j];
    double ac = c->ac[ZAC(c, i, j, kv)];
    r = cx_axpy(r, c->aw[i], *gm);
    r = cx_axpy(r, c->ae[i], *gp);
    r = cx_axpy(r, c->as[j], *gs);
    r = cx_axpy(r, c->an[j], *gn);
    r = cx_axpy(r, ac, *gc);
    return r;
}

/* toplevel, poiss_z_ft.f90:302-380 (zebra version) */
static void zft_toplevel(const ref_case *c, zmode *z, int id, double *sumres, double oldv, double test, ll kv)
{
    ll n1m = c->n1m, n2m = c->n2m, nlev = c->c.nlev;
    if (id == 1) {
        ll ic = 0;
        for (ll i = c->iimg[nlev - 1][0]; i <= c->iimg[nlev - 1][1] - 1; i++) {
            ic += 2;
            for (ll j = 1; j <= n2m; j++) {
                cplx p = PC(z, ic, j), a = GG(z, i, j), b = GG(z, c->ipm[i], j);
                p.re = p.re + c->coi1[i] * a.re + c->coi2[i] * b.re;
                p.im = p.im + c->coi1[i] * a.im + c->coi2[i] * b.im;
                PC(z, ic, j) = p;
            }
        }
        ll i = c->iimg[nlev - 1][1];
        ic += 2;
        for (ll j = 1; j <= n2m; j++) {
            PC(z, ic, j).re = PC(z, ic, j).re + c->coi1[i] * GG(z, i, j).re;
            PC(z, ic, j).im = PC(z, ic, j).im + c->coi1[i] * GG(z, i, j).im;
        }
    }
    for (ll j = 1; j <= n2m; j++)
        for (ll i = 1; i <= n1m; i += 2) {
            cplx pm = PC(z, c->imm[i], j), pp = PC(z, c->ipm[i], j), r = RH(z, i, j);
            double sre = c->aw[i] * pm.re + c->ae[i] * pp.re, sim = c->aw[i] * pm.im + c->ae[i] * pp.im;
            GG(z, i, j).re = r.re - oldv * sre;
            GG(z, i, j).im = r.im - oldv * sim;
        }
    zft_trdiag(c, z, 1, n1m, kv);
    cplx tt = { 0.0, 0.0 };
    if (kv == 1) tt = GG(z, 1, n2m - 1);
    for (ll j = 1; j <= n2m; j++)
        for (ll i = 2; i <= n1m; i += 2) {
            GG(z, i - 1, j).re -= tt.re; GG(z, i - 1, j).im -= tt.im;
            cplx gm = GG(z, c->imm[i], j), gp = GG(z, c->ipm[i], j), r = RH(z, i, j);
            GG(z, i, j).re = r.re - c->aw[i] * gm.re - c->ae[i] * (gp.re - tt.re);
            GG(z, i, j).im = r.im - c->aw[i] * gm.im - c->ae[i] * (gp.im - tt.im);
        }
    zft_trdiag(c, z, 2, n1m, kv);
    double sr = 0.0;
    for (ll j = 1; j <= n2m; j++)
        for (ll i = 1; i <= n1m; i++) {
            cplx d = zft_defect(c, RH(z, i, j), z->gg, z->ld_g, i, j, kv);
            RS(z, i, j) = d;
            double a = hypot(d.re, d.im);
            if (a > sr) sr = a;
            PC(z, i, j) = GG(z, i, j);
        }
    *sumres = sr;
    if (sr < test || id == 2) return;
    ll ic = -1;
    for (ll i = c->iimg[nlev - 1][0]; i <= c->iimg[nlev - 1][1]; i++) {
        ic += 2;
        for (ll j = 1; j <= n2m; j++) {
            cplx a = RS(z, ic, j), b = RS(z, ic + 1, j);
            RS(z, i, j).re = a.re * c->cor1[i] + b.re * c->cor2[i];
            RS(z, i, j).im = a.im * c->cor1[i] + b.im * c->cor2[i];
        }
    }
}

/* relax, poiss_z_ft.f90:466-511 (zebra version) */
static void zft_relax(const ref_case *c, zmode *z, ll ilev, double oldv, ll iiter, ll kv)
{
    ll n2m = c->n2m, ibg = c->iimg[ilev][0], iend = c->iimg[ilev][1];
    for (ll it = 0; it < iiter; it++) {
        double ov = it == 0 ? oldv : 1.0;
        for (ll j = 1; j <= n2m; j++)
            for (ll i = ibg; i <= iend; i += 2) {
                cplx gm = GG(z, c->imm[i], j), gp = GG(z, c->ipm[i], j), r = RS(z, i, j);
                double sre = c->aw[i] * gm.re + c->ae[i] * gp.re, sim = c->aw[i] * gm.im + c->ae[i] * gp.im;
                GG(z, i, j).re = r.re - ov * sre;
                GG(z, i, j).im = r.im - ov * sim;
            }
        zft_trdiag(c, z, ibg, iend, kv);
        for (ll j = 1; j <= n2m; j++)
            for (ll i = ibg + 1; i <= iend; i += 2) {
                cplx gm = GG(z, c->imm[i], j), gp = GG(z, c->ipm[i], j), r = RS(z, i, j);
                GG(z, i, j).re = r.re - c->aw[i] * gm.re - c->ae[i] * gp.re;
                GG(z, i, j).im = r.im - c->aw[i] * gm.im - c->ae[i] * gp.im;
            }
        zft_trdiag(c, z, ibg + 1, iend, kv);
    }
}

/* godown, poiss_z_ft.f90:438-463: residual of level ilev, restricted to ilev-1 */
static void zft_godown(const ref_case *c, zmode *z, ll ilev, ll kv)
{
    ll n2m = c->n2m;
    for (ll j = 1; j <= n2m; j++)
        for (ll i = c->iimg[ilev][0]; i <= c->iimg[ilev][1]; i++)
            RS(z, i, j) = zft_defect(c, RS(z, i, j), z->gg, z->ld_g, i, j, kv);
    ll ibg = c->iimg[ilev][0] - 2;
    for (ll i = c->iimg[ilev - 1][0]; i <= c->iimg[ilev - 1][1]; i++) {
        ibg += 2;
        for (ll j = 1; j <= n2m; j++) {
            cplx a = RS(z, ibg, j), b = RS(z, ibg + 1, j);
            RS(z, i, j).re = a.re * c->cor1[i] + b.re * c->cor2[i];
            RS(z, i, j).im = a.im * c->cor1[i] + b.im * c->cor2[i];
        }
    }
}

/* goup, poiss_z_ft.f90:411-435: coarse correction onto the even lines of ilev+1 */
static void zft_goup(const ref_case *c, zmode *z, ll ilev)
{
    ll n2m = c->n2m, ibgh = c->iimg[ilev + 1][0] - 1;
    for (ll i = c->iimg[ilev][0]; i <= c->iimg[ilev][1] - 1; i++) {
        ibgh += 2;
        for (ll j = 1; j <= n2m; j++) {
            cplx g = GG(z, ibgh, j), a = GG(z, i, j), b = GG(z, c->ipm[i], j);
            GG(z, ibgh, j).re = g.re + c->coi1[i] * a.re + c->coi2[i] * b.re;
            GG(z, ibgh, j).im = g.im + c->coi1[i] * a.im + c->coi2[i] * b.im;
        }
    }
    ll i = c->iimg[ilev][1];
    ibgh += 2;
    for (ll j = 1; j <= n2m; j++) {
        GG(z, ibgh, j).re = GG(z, ibgh, j).re + c->coi1[i] * GG(z, i, j).re;
        GG(z, ibgh, j).im = GG(z, ibgh, j).im + c->coi1[i] * GG(z, i, j).im;
    }
}

/* mg2d, poiss_z_ft.f90:239-299; returns the number of V-cycles */
static ll zft_mg2d(const ref_case *c, zmode *z, ll kv, double test, double oldv, int *unconv)
{
    ll nlev = c->c.nlev, kk = 0;
    double sumres;
    zft_toplevel(c, z, 0, &sumres, oldv, test, kv);
    if (sumres < test) return 0;
    for (kk = 1; kk <= c->c.mgitr; kk++) {
        for (ll ilev = nlev - 1; ilev >= 1; ilev--) {
            zft_relax(c, z, ilev, 0.0, 1, kv);
            zft_godown(c, z, ilev, kv);
        }
        zft_relax(c, z, 0, 0.0, c->c.nbli, kv);
        for (ll ilev = 0; ilev <= nlev - 2; ilev++) {
            zft_goup(c, z, ilev);
            zft_relax(c, z, ilev + 1, 1.0, 1, kv);
        }
        zft_toplevel(c, z, 1, &sumres, 1.0, test, kv);
        if (sumres < test) return kk;
    }
    *unconv = 1;
    return kk;   /* iteration limit (the reference prints a warning and goes on) */
}

/* resid3, poiss_z_ft.f90:619-641 */
static double zft_resid3(const ref_case *c, zmode *z, ll kv)
{
    double e = 0.0;
    for (ll j = 1; j <= c->n2m; j++)
        for (ll i = 1; i <= c->n1m; i++) {
            cplx d = zft_defect(c, RH(z, i, j), z->pc, z->ld_p, i, j, kv);
            double a = hypot(d.re, d.im);
            if (a > e) e = a;
        }
    return e;
}

/* gsor2d, poiss_z_ft.f90:513-616: zebra line SOR on pc (= u) */
static ll zft_gsor2d(const ref_case *c, zmode *z, ll kv, double test, double oldv, int *unconv)
{
    ll n1m = c->n1m, n2m = c->n2m;
    double ww = c->c.wwsor, ww2 = 1.0 - ww;
    for (ll kk = 0; kk <= c->c.mgitr; kk++) {
        double ov = kk == 0 ? oldv : 1.0;
        for (int half = 0; half < 2; half++) {
            ll i0 = half == 0 ? 1 : 2;
            for (ll j = 1; j <= n2m; j++)
                for (ll i = i0; i <= n1m; i += 2) {
                    cplx um = PC(z, c->imm[i], j), up = PC(z, c->ipm[i], j), r = RH(z, i, j);
                    double sre = c->aw[i] * um.re + c->ae[i] * up.re, sim = c->aw[i] * um.im + c->ae[i] * up.im;
                    double f = half == 0 ? ov : 1.0;
                    GG(z, i, j).re = r.re - f * sre;
                    GG(z, i, j).im = r.im - f * sim;
                }
            zft_trdiag(c, z, i0, n1m, kv);
            double o2 = ov * ww2;
            for (ll j = 1; j <= n2m; j++)
                for (ll i = i0; i <= n1m; i += 2) {
                    PC(z, i, j).re = ww * GG(z, i, j).re + o2 * PC(z, i, j).re;
                    PC(z, i, j).im = ww * GG(z, i, j).im + o2 * PC(z, i, j).im;
                }
        }
        if (zft_resid3(c, z, kv) < test) return kk;
    }
    *unconv = 1;
    return c->c.mgitr;
}

/* poisson, poiss_z_ft.f90:116-236 */
static void zft_poisson(ref_case *c)
{
    ll n1 = c->n1, n2 = c->n2, n1m = c->n1m, n2m = c->n2m, n3m = c->n3m, n3mh = c->n3mh, n1md = c->n1md;
    ll ld_p = n1 + 1, ld_g = n1md + 1;
    size_t np = (size_t)ld_p * (size_t)(n2 + 1), ng = (size_t)ld_g * (size_t)(n2 + 1);
    cplx *ccap = (cplx *)calloc(np * (size_t)n3mh, sizeof(cplx));
    ll itmax = 0, nunc = 0;
    if (n3m == 1) {
        for (ll j = 1; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++) { ccap[(size_t)i + (size_t)ld_p * (size_t)j].re = c->divgsum[IX(c, i, j, 1)]; }
    } else {
        #pragma omp parallel
        {
            cplx *line = (cplx *)malloc(sizeof(cplx) * (size_t)n3m), *wk = (cplx *)malloc(sizeof(cplx) * 2 * (size_t)n3m);
            #pragma omp for
            for (ll j = 1; j <= n2m; j++)
                for (ll i = 1; i <= n1m; i++) {
                    for (ll k = 1; k <= n3m; k++) { line[k - 1].re = c->divgsum[IX(c, i, j, k)]; line[k - 1].im = 0.0; }
                    ref_fft(&c->fftz, line, wk, -1);
                    for (ll k = 1; k <= n3mh; k++) ccap[(size_t)i + (size_t)ld_p * (size_t)j + np * (size_t)(k - 1)] = line[k - 1];
                }
            free(line); free(wk);
        }
    }
    double test = n3m == 1 ? c->test1 : c->test1 / (double)n3mh * (double)n3m * 0.8;
    #pragma omp parallel reduction(max:itmax) reduction(+:nunc)
    {
        zmode z;
        z.ld_p = ld_p; z.ld_g = ld_g;
        z.pc = (cplx *)malloc(sizeof(cplx) * np);
        z.resd = (cplx *)malloc(sizeof(cplx) * ng);
        z.gg = (cplx *)malloc(sizeof(cplx) * ng);
        #pragma omp for schedule(dynamic, 1)
        for (ll kkk = 1; kkk <= n3mh; kkk++) {
            z.rhs = ccap + np * (size_t)(kkk - 1);
            memset(z.pc, 0, sizeof(cplx) * np);
            memset(z.resd, 0, sizeof(cplx) * ng);
            memset(z.gg, 0, sizeof(cplx) * ng);
            int unc = 0;
            ll it = kkk <= c->c.imgsor ? zft_mg2d(c, &z, kkk, test, 0.0, &unc) : zft_gsor2d(c, &z, kkk, test, 0.0, &unc);
            if (it > itmax) itmax = it;
            nunc += unc;
            for (ll j = 1; j <= n2m; j++)
                for (ll i = 1; i <= n1m; i++) z.rhs[(size_t)i + (size_t)ld_p * (size_t)j] = PC(&z, i, j);
        }
        free(z.pc); free(z.resd); free(z.gg);
    }
    if (n3m == 1) {
        for (ll j = 1; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++) c->phi[IX(c, i, j, 1)] = ccap[(size_t)i + (size_t)ld_p * (size_t)j].re;
    } else {
        #pragma omp parallel
        {
            cplx *line = (cplx *)malloc(sizeof(cplx) * (size_t)n3m), *wk = (cplx *)malloc(sizeof(cplx) * 2 * (size_t)n3m);
            #pragma omp for
            for (ll j = 1; j <= n2m; j++)
                for (ll i = 1; i <= n1m; i++) {
                    for (ll k = 1; k <= n3mh; k++) line[k - 1] = ccap[(size_t)i + (size_t)ld_p * (size_t)j + np * (size_t)(k - 1)];
                    for (ll k = n3mh + 1; k <= n3m; k++) {
                        cplx s = line[n3m + 2 - k - 1];
                        s.im = -s.im;
                        line[k - 1] = s;
                    }
                    ref_fft(&c->fftz, line, wk, 1);
                    for (ll k = 1; k <= n3m; k++) c->phi[IX(c, i, j, k)] = line[k - 1].re;
                }
            free(line); free(wk);
        }
    }
    free(ccap);
    c->poisson_iters[c->msub >= 1 && c->msub <= 3 ? c->msub - 1 : 0] = itmax;
    c->poisson_unconv += nunc;
}

/* -------------------------------------------------------- poiss_x_ft -- */
/* FFT in x, then for every x mode a 2-D problem in z-y solved by multigrid
   semi-coarsened in z with zebra z-line relaxation (y-Thomas per line).
   Level ilev occupies z slots kkmg[ilev][0]..kkmg[ilev][1] of ab, af,
   coi?, cor?, kpm, kmm; the finest level nlev is 1..n3m.  ak1 holds ai3,
   the x modified wavenumbers.  The work arrays of one mode reuse zmode:
   pc(0:n3,0:n2), rhs(n3,n2), resd(n3md,n2m), ggii(0:n3md,0:n2). */

#define XAC(c, k, j, i) ((size_t)((k) - 1) + (size_t)(c)->n3md * ((size_t)((j) - 1) + (size_t)(c)->n2m * (size_t)((i) - 1)))

/* pmat + mwavenumber, poiss_x_ft.f90:54-112 */
static void xft_pmat(ref_case *c)
{
    ll n1m = c->n1m, n2m = c->n2m, n3m = c->n3m;
    for (ll k = 1; k <= n3m; k++) {
        ll kp = c->kpv[k];
        c->ab[k] = (1.0 - (double)c->fixkl[k]) * c->c2czi[k] * c->f2fzi[k];
        c->af[k] = (1.0 - (double)c->fixku[k]) * c->c2czi[kp] * c->f2fzi[k];
    }
    for (ll j = 1; j <= n2m; j++) {
        ll jp = c->jpv[j];
        c->as[j] = (1.0 - (double)c->fixjl[j]) * c->c2cyi[j] * c->f2fyi[j];
        c->an[j] = (1.0 - (double)c->fixju[j]) * c->c2cyi[jp] * c->f2fyi[j];
    }
    for (ll j = 1; j <= n2m; j++)
        for (ll k = 1; k <= n3m; k++)
            c->ac[XAC(c, k, j, 1)] = -1.0 * (c->ab[k] + c->af[k] + c->as[j] + c->an[j]);
    double pi = acos(-1.0);
    for (ll i = 1; i <= c->n1mh; i++)
        c->ak1[i] = 2.0 * (1.0 - cos(2.0 * pi * (double)(i - 1) / (double)n1m)) * c->f2fxi[1] * c->f2fxi[1];
    for (ll i = 2; i <= c->n1mh; i++)
        for (ll j = 1; j <= n2m; j++)
            for (ll k = 1; k <= n3m; k++) c->ac[XAC(c, k, j, i)] = c->ac[XAC(c, k, j, 1)] - c->ak1[i];
}

/* coefmg, poiss_x_ft.f90:644-794.  Without z periodicity the reference
   leaves kpm/kmm unset; every coefficient that multiplies them there (ab at
   a level's first point, af and coi2 at its last) is zero, so k+1 / k-1 are
   used, which read finite work-array entries. */
static void xft_coefmg(ref_case *c)
{
    ll n2m = c->n2m, n3m = c->n3m, n3md = c->n3md, nlev = c->c.nlev, n3 = c->n3;
    ll minrow = n3m / (1LL << nlev);
    double *zmpm = ref_zalloc((size_t)n3md + 2), *kbz = ref_zalloc((size_t)n3md + 2), *kfz = ref_zalloc((size_t)n3md + 2);
    const double *z = c->z;
    c->kkmg[nlev][0] = 1; c->kkmg[nlev][1] = n3m; c->kkmg[nlev][2] = n3m;
    for (ll k = 1; k <= n3m; k++) {
        zmpm[k] = c->zmp[k];
        kbz[k] = (double)(1 - 1 / k);
        kfz[k] = (double)(1 - k / n3m);
    }
    for (ll ilev = nlev - 1; ilev >= 0; ilev--) {
        c->kkmg[ilev][0] = c->kkmg[ilev + 1][0] + c->kkmg[ilev + 1][2];
        c->kkmg[ilev][2] = minrow * (1LL << ilev);
        c->kkmg[ilev][1] = c->kkmg[ilev][0] + c->kkmg[ilev][2] - 1;
        ll kbg = c->kkmg[ilev][0], kend = c->kkmg[ilev][1], ksp = 1LL << (nlev - ilev);
        ll kc = 0;
        for (ll k = kbg; k <= kend; k++) {
            kc++;
            zmpm[k] = 0.5 * (z[kc * ksp + 1] + z[(kc - 1) * ksp + 1]);
            kbz[k] = (double)(1 - kbg / k);
            kfz[k] = (double)(1 - k / kend);
        }
        kc = 0;
        for (ll k = kbg; k <= kend; k++) {
            kc++;
            double w = z[kc * ksp + 1] - z[(kc - 1) * ksp + 1];
            c->ab[k] = kbz[k] / ((zmpm[k] - zmpm[k - 1]) * w);
            c->af[k] = kfz[k] / ((zmpm[k + 1] - zmpm[k]) * w);
        }
        for (ll j = 1; j <= n2m; j++)
            for (ll k = kbg; k <= kend; k++)
                c->ac[XAC(c, k, j, 1)] = -1.0 * (c->ab[k] + c->af[k] + c->as[j] + c->an[j]);
        for (ll i = 2; i <= c->n1mh; i++)
            for (ll j = 1; j <= n2m; j++)
                for (ll k = kbg; k <= kend; k++) c->ac[XAC(c, k, j, i)] = c->ac[XAC(c, k, j, 1)] - c->ak1[i];
    }
    for (ll ilev = nlev; ilev >= 1; ilev--) {
        ll kbgh = c->kkmg[ilev][0];
        for (ll k = c->kkmg[ilev - 1][0]; k <= c->kkmg[ilev - 1][1]; k++) {
            c->cor1[k] = (zmpm[kbgh + 1] - zmpm[k]) / (zmpm[kbgh + 1] - zmpm[kbgh]);
            c->cor2[k] = 1.0 - c->cor1[k];
            kbgh += 2;
        }
    }
    for (ll ilev = 0; ilev <= nlev - 1; ilev++) {
        ll kbgh = c->kkmg[ilev + 1][0] + 1;
        for (ll k = c->kkmg[ilev][0]; k <= c->kkmg[ilev][1] - 1; k++) {
            c->coi1[k] = (zmpm[k + 1] - zmpm[kbgh]) / (zmpm[k + 1] - zmpm[k]);
            c->coi2[k] = 1.0 - c->coi1[k];
            kbgh += 2;
        }
        c->coi1[c->kkmg[ilev][1]] = 1.0;
    }
    for (ll ilev = nlev; ilev >= 0; ilev--)
        for (ll k = c->kkmg[ilev][0]; k <= c->kkmg[ilev][1]; k++) { c->kpm[k] = k + 1; c->kmm[k] = k - 1; }
    if (c->c.zprdic == 1) {
        for (ll ilev = nlev; ilev >= 0; ilev--) {
            ll kbg = c->kkmg[ilev][0], kend = c->kkmg[ilev][1];
            c->kpm[kend] = kbg;
            c->kmm[kbg] = kend;
        }
        for (ll ilev = nlev - 1; ilev >= 0; ilev--) {
            ll kbg = c->kkmg[ilev][0], kend = c->kkmg[ilev][1], ksp = 1LL << (nlev - ilev);
            double vdz_kbg = zmpm[kbg] - z[1] + z[n3] - zmpm[kend];
            double vdz_kend = zmpm[kbg] - z[1] + z[n3] - zmpm[kend];
            double sdz_kbg = z[1 + ksp] - z[1], sdz_kend = z[n3] - z[n3 - ksp];
            c->ab[kbg] = 1.0 / (vdz_kbg * sdz_kbg);
            c->af[kend] = 1.0 / (vdz_kend * sdz_kend);
        }
        for (ll ilev = nlev - 1; ilev >= 0; ilev--) {
            for (ll j = 1; j <= n2m; j++)
                for (ll k = c->kkmg[ilev][0]; k <= c->kkmg[ilev][1]; k++)
                    c->ac[XAC(c, k, j, 1)] = -1.0 * (c->ab[k] + c->af[k] + c->as[j] + c->an[j]);
            for (ll i = 2; i <= c->n1mh; i++)
                for (ll j = 1; j <= n2m; j++)
                    for (ll k = c->kkmg[ilev][0]; k <= c->kkmg[ilev][1]; k++)
                        c->ac[XAC(c, k, j, i)] = c->ac[XAC(c, k, j, 1)] - c->ak1[i];
        }
        for (ll ilev = 0; ilev <= nlev - 1; ilev++) {
            ll kbg = c->kkmg[ilev][0], kend = c->kkmg[ilev][1];
            double vdz_kend = zmpm[kbg] - z[1] + z[n3] - zmpm[kend];
            c->coi2[kend] = (zmpm[c->kkmg[ilev + 1][1]] - zmpm[kend]) / vdz_kend;
            c->coi1[kend] = 1.0 - c->coi2[kend];
        }
    }
    free(zmpm); free(kbz); free(kfz);
}

/* poisinit, poiss_x_ft.f90:18-52 */
static int xft_init(ref_case *c)
{
    ll n3md = c->n3md, n2m = c->n2m, n1mh = c->n1mh, nlev = c->c.nlev;
    if (c->c.xprdic != 1) return LESGPU_ERR_CONFIG;                 /* the x transform needs periodic x */
    if (nlev < 1 || nlev > 20 || c->n3m % (1LL << nlev) != 0) return LESGPU_ERR_CONFIG;
    if (ref_fft_plan_init(&c->fftx, (int)c->n1m)) return LESGPU_ERR_ARG;
    size_t nv = (size_t)n3md + 2, na = (size_t)n3md * (size_t)n2m * (size_t)n1mh;
    c->ab = ref_zalloc(nv); c->af = ref_zalloc(nv);
    c->as = ref_zalloc((size_t)n2m + 2); c->an = ref_zalloc((size_t)n2m + 2);
    c->coi1 = ref_zalloc(nv); c->coi2 = ref_zalloc(nv); c->cor1 = ref_zalloc(nv); c->cor2 = ref_zalloc(nv);
    c->kpm = ref_izalloc(nv); c->kmm = ref_izalloc(nv);
    c->ak1 = ref_zalloc((size_t)n1mh + 2);
    c->ac = ref_zalloc(na); c->gam = ref_zalloc(na); c->bet = ref_zalloc(na);
    xft_pmat(c);
    xft_coefmg(c);
    for (ll ilev = 0; ilev <= nlev; ilev++)
        for (ll i = 1; i <= n1mh; i++) {
            for (ll k = c->kkmg[ilev][0]; k <= c->kkmg[ilev][1]; k++) c->bet[XAC(c, k, 1, i)] = 1.0 / c->ac[XAC(c, k, 1, i)];
            for (ll j = 2; j <= n2m; j++)
                for (ll k = c->kkmg[ilev][0]; k <= c->kkmg[ilev][1]; k++) {
                    c->gam[XAC(c, k, j, i)] = c->an[j - 1] * c->bet[XAC(c, k, j - 1, i)];
                    c->bet[XAC(c, k, j, i)] = 1.0 / (c->ac[XAC(c, k, j, i)] - c->as[j] * c->gam[XAC(c, k, j, i)]);
                }
        }
    return 0;
}

/* trdiag1m, poiss_x_ft.f90:373-398: y-Thomas on z-lines l1, l1+2, ..., l2 (in place) */
static void xft_trdiag(const ref_case *c, zmode *z, ll l1, ll l2, ll iv)
{
    ll n2m = c->n2m;
    for (ll k = l1; k <= l2; k += 2) {
        double b = c->bet[XAC(c, k, 1, iv)];
        GG(z, k, 1).re *= b; GG(z, k, 1).im *= b;
    }
    for (ll j = 2; j <= n2m; j++)
        for (ll k = l1; k <= l2; k += 2) {
            double b = c->bet[XAC(c, k, j, iv)];
            cplx t = cx_axpy(GG(z, k, j), c->as[j], GG(z, k, j - 1));
            GG(z, k, j).re = t.re * b; GG(z, k, j).im = t.im * b;
        }
    for (ll j = n2m - 1; j >= 1; j--)
        for (ll k = l1; k <= l2; k += 2)
            GG(z, k, j) = cx_axpy(GG(z, k, j), c->gam[XAC(c, k, j + 1, iv)], GG(z, k, j + 1));
}

/* rhs - ab*g(kmm) - af*g(kpm) - as*g(j-1) - an*g(j+1) - ac*g */
static inline cplx xft_defect(const ref_case *c, cplx r, const cplx *g, ll ld, ll k, ll j, ll iv)
{
    const cplx *gm = &g[(size_t)c->kmm[k] + (size_t)ld * (size_t)j], *gp = &g[(size_t)c->kpm[k] + (size_t)ld * (size_t)j];
    const cplx *gs = &g[(size_t)k + (size_t)ld * (size_t)(j - 1)], *gn = &g[(size_t)k + (size_t)ld * (size_t)(j + 1)];
    const cplx *gc = &g[(size_t)k + (size_t)ld * (size_t)j];
    double ac = c->ac[XAC(c, k, j, iv)];
    r = cx_axpy(r, c->ab[k], *gm);
    r = cx_axpy(r, c->af[k], *gp);
    r = cx_axpy(r, c->as[j], *gs);
    r = cx_axpy(r, c->an[j], *gn);
    r = cx_axpy(r, ac, *gc);
    return r;
}

/* rhs - f*(ab*u(kmm) + af*u(kpm)) on the lines k0, k0+2, ..., k1 of the level */
static void xft_line_rhs(const ref_case *c, zmode *z, const cplx *u, ll ldu, int from_rhs, ll k0, ll k1, double f)
{
    for (ll j = 1; j <= c->n2m; j++)
        for (ll k = k0; k <= k1; k += 2) {
            cplx um = u[(size_t)c->kmm[k] + (size_t)ldu * (size_t)j], up = u[(size_t)c->kpm[k] + (size_t)ldu * (size_t)j];
            cplx r = from_rhs ? RH(z, k, j) : RS(z, k, j);
            double sre = c->ab[k] * um.re + c->af[k] * up.re, sim = c->ab[k] * um.im + c->af[k] * up.im;
            GG(z, k, j).re = r.re - f * sre;
            GG(z, k, j).im = r.im - f * sim;
        }
}

/* toplevel, poiss_x_ft.f90:296-371 (zebra version) */
static void xft_toplevel(const ref_case *c, zmode *z, int id, double *sumres, double oldv, double test, ll iv)
{
    ll n3m = c->n3m, n2m = c->n2m, nlev = c->c.nlev;
    if (id == 1) {
        ll kc = 0;
        for (ll k = c->kkmg[nlev - 1][0]; k <= c->kkmg[nlev - 1][1]; k++) {
            kc += 2;
            for (ll j = 1; j <= n2m; j++) {
                cplx p = PC(z, kc, j), a = GG(z, k, j), b = GG(z, c->kpm[k], j);
                p.re = p.re + c->coi1[k] * a.re + c->coi2[k] * b.re;
                p.im = p.im + c->coi1[k] * a.im + c->coi2[k] * b.im;
                PC(z, kc, j) = p;
            }
        }
    }
    xft_line_rhs(c, z, z->pc, z->ld_p, 1, 1, n3m, oldv);
    xft_trdiag(c, z, 1, n3m, iv);
    if (iv == 1) {
        cplx tt = GG(z, 1, n2m);
        for (ll j = 1; j <= n2m; j++)
            for (ll k = 1; k <= n3m; k += 2) { GG(z, k, j).re -= tt.re; GG(z, k, j).im -= tt.im; }
    }
    xft_line_rhs(c, z, z->gg, z->ld_g, 1, 2, n3m, 1.0);
    xft_trdiag(c, z, 2, n3m, iv);
    double sr = 0.0;
    for (ll j = 1; j <= n2m; j++)
        for (ll k = 1; k <= n3m; k++) {
            cplx d = xft_defect(c, RH(z, k, j), z->gg, z->ld_g, k, j, iv);
            RS(z, k, j) = d;
            double a = hypot(d.re, d.im);
            if (a > sr) sr = a;
            PC(z, k, j) = GG(z, k, j);
        }
    *sumres = sr;
    if (sr < test || id == 2) return;
    ll kc = -1;
    for (ll k = c->kkmg[nlev - 1][0]; k <= c->kkmg[nlev - 1][1]; k++) {
        kc += 2;
        for (ll j = 1; j <= n2m; j++) {
            cplx a = RS(z, kc, j), b = RS(z, kc + 1, j);
            RS(z, k, j).re = a.re * c->cor1[k] + b.re * c->cor2[k];
            RS(z, k, j).im = a.im * c->cor1[k] + b.im * c->cor2[k];
        }
    }
}

/* relax, poiss_x_ft.f90:450-495 (zebra version): the first pass scales the
   odd lines' neighbours by oldv; the even lines and later passes do not */
static void xft_relax(const ref_case *c, zmode *z, ll ilev, double oldv, ll iiter, ll iv)
{
    ll n2m = c->n2m, kbg = c->kkmg[ilev][0], kend = c->kkmg[ilev][1];
    for (ll it = 0; it < iiter; it++) {
        xft_line_rhs(c, z, z->gg, z->ld_g, 0, kbg, kend, it == 0 ? oldv : 1.0);
        xft_trdiag(c, z, kbg, kend, iv);
        for (ll j = 1; j <= n2m; j++)
            for (ll k = kbg + 1; k <= kend; k += 2) {
                cplx gm = GG(z, c->kmm[k], j), gp = GG(z, c->kpm[k], j), r = RS(z, k, j);
                GG(z, k, j).re = r.re - c->ab[k] * gm.re - c->af[k] * gp.re;
                GG(z, k, j).im = r.im - c->ab[k] * gm.im - c->af[k] * gp.im;
            }
        xft_trdiag(c, z, kbg + 1, kend, iv);
    }
}

/* godown, poiss_x_ft.f90:422-447: residual of level ilev, restricted to ilev-1 */
static void xft_godown(const ref_case *c, zmode *z, ll ilev, ll iv)
{
    ll n2m = c->n2m;
    for (ll j = 1; j <= n2m; j++)
        for (ll k = c->kkmg[ilev][0]; k <= c->kkmg[ilev][1]; k++)
            RS(z, k, j) = xft_defect(c, RS(z, k, j), z->gg, z->ld_g, k, j, iv);
    ll kbg = c->kkmg[ilev][0] - 2;
    for (ll k = c->kkmg[ilev - 1][0]; k <= c->kkmg[ilev - 1][1]; k++) {
        kbg += 2;
        for (ll j = 1; j <= n2m; j++) {
            cplx a = RS(z, kbg, j), b = RS(z, kbg + 1, j);
            RS(z, k, j).re = a.re * c->cor1[k] + b.re * c->cor2[k];
            RS(z, k, j).im = a.im * c->cor1[k] + b.im * c->cor2[k];
        }
    }
}

/* goup, poiss_x_ft.f90:401-419: coarse correction onto the even lines of
   ilev+1, every coarse point through coi1 and coi2 (the last one's coi2 is
   the periodic weight, or zero) */
static void xft_goup(const ref_case *c, zmode *z, ll ilev)
{
    ll n2m = c->n2m, kbgh = c->kkmg[ilev + 1][0] - 1;
    for (ll k = c->kkmg[ilev][0]; k <= c->kkmg[ilev][1]; k++) {
        kbgh += 2;
        for (ll j = 1; j <= n2m; j++) {
            cplx g = GG(z, kbgh, j), a = GG(z, k, j), b = GG(z, c->kpm[k], j);
            GG(z, kbgh, j).re = g.re + c->coi1[k] * a.re + c->coi2[k] * b.re;
            GG(z, kbgh, j).im = g.im + c->coi1[k] * a.im + c->coi2[k] * b.im;
        }
    }
}

/* mg2d, poiss_x_ft.f90:238-294; returns the number of V-cycles */
static ll xft_mg2d(const ref_case *c, zmode *z, ll iv, double test, double oldv, int *unconv)
{
    ll nlev = c->c.nlev;
    double sumres;
    xft_toplevel(c, z, 0, &sumres, oldv, test, iv);
    if (sumres < test) return 0;
    for (ll ii = 1; ii <= c->c.mgitr; ii++) {
        for (ll ilev = nlev - 1; ilev >= 1; ilev--) {
            xft_relax(c, z, ilev, 0.0, 1, iv);
            xft_godown(c, z, ilev, iv);
        }
        xft_relax(c, z, 0, 0.0, c->c.nbli, iv);
        for (ll ilev = 0; ilev <= nlev - 2; ilev++) {
            xft_goup(c, z, ilev);
            xft_relax(c, z, ilev + 1, 1.0, 1, iv);
        }
        xft_toplevel(c, z, 1, &sumres, 1.0, test, iv);
        if (sumres < test) return ii;
    }
    *unconv = 1;
    return c->c.mgitr;   /* iteration limit (the reference prints a warning and goes on) */
}

/* resid3, poiss_x_ft.f90:620-642 */
static double xft_resid3(const ref_case *c, zmode *z, ll iv)
{
    double e = 0.0;
    for (ll j = 1; j <= c->n2m; j++)
        for (ll k = 1; k <= c->n3m; k++) {
            cplx d = xft_defect(c, RH(z, k, j), z->pc, z->ld_p, k, j, iv);
            double a = hypot(d.re, d.im);
            if (a > e) e = a;
        }
    return e;
}

/* gsor2d, poiss_x_ft.f90:497-617: zebra line SOR on pc (= u); the zero
   wavenumber's odd lines are shifted by u(1,n2m) after their update */
static ll xft_gsor2d(const ref_case *c, zmode *z, ll iv, double test, double oldv, int *unconv)
{
    ll n3m = c->n3m, n2m = c->n2m;
    double ww = c->c.wwsor, ww2 = 1.0 - ww;
    for (ll ii = 0; ii <= c->c.mgitr; ii++) {
        double ov = ii == 0 ? oldv : 1.0, o2 = ii == 0 ? oldv * ww2 : ww2;
        for (int half = 0; half < 2; half++) {
            ll k0 = half == 0 ? 1 : 2;
            xft_line_rhs(c, z, z->pc, z->ld_p, 1, k0, n3m, half == 0 ? ov : 1.0);
            xft_trdiag(c, z, k0, n3m, iv);
            for (ll j = 1; j <= n2m; j++)
                for (ll k = k0; k <= n3m; k += 2) {
                    PC(z, k, j).re = ww * GG(z, k, j).re + o2 * PC(z, k, j).re;
                    PC(z, k, j).im = ww * GG(z, k, j).im + o2 * PC(z, k, j).im;
                }
            if (half == 0 && iv == 1) {
                cplx tt = PC(z, 1, n2m);
                for (ll j = 1; j <= n2m; j++)
                    for (ll k = 1; k <= n3m; k += 2) { PC(z, k, j).re -= tt.re; PC(z, k, j).im -= tt.im; }
            }
        }
        if (xft_resid3(c, z, iv) < test) return ii;
    }
    *unconv = 1;
    return c->c.mgitr;
}

/* poisson, poiss_x_ft.f90:115-235 */
static void xft_poisson(ref_case *c)
{
    ll n1m = c->n1m, n2m = c->n2m, n3m = c->n3m, n3 = c->n3, n2 = c->n2, n1mh = c->n1mh, n3md = c->n3md;
    ll ld_p = n3 + 1, ld_g = n3md + 1;
    size_t np = (size_t)ld_p * (size_t)(n2 + 1), ng = (size_t)ld_g * (size_t)(n2 + 1);
    cplx *ccap = (cplx *)calloc(np * (size_t)n1mh, sizeof(cplx));
    ll itmax = 0, nunc = 0;
    #pragma omp parallel
    {
        cplx *line = (cplx *)malloc(sizeof(cplx) * (size_t)n1m), *wk = (cplx *)malloc(sizeof(cplx) * 2 * (size_t)n1m);
        #pragma omp for
        for (ll j = 1; j <= n2m; j++)
            for (ll k = 1; k <= n3m; k++) {
                for (ll i = 1; i <= n1m; i++) { line[i - 1].re = c->divgsum[IX(c, i, j, k)]; line[i - 1].im = 0.0; }
                ref_fft(&c->fftx, line, wk, -1);
                for (ll i = 1; i <= n1mh; i++) ccap[(size_t)k + (size_t)ld_p * (size_t)j + np * (size_t)(i - 1)] = line[i - 1];
            }
        free(line); free(wk);
    }
    double test = c->test1 / (double)n1mh * (double)n1m * 0.9;
    #pragma omp parallel reduction(max:itmax) reduction(+:nunc)
    {
        zmode z;
        z.ld_p = ld_p; z.ld_g = ld_g;
        z.pc = (cplx *)malloc(sizeof(cplx) * np);
        z.resd = (cplx *)malloc(sizeof(cplx) * ng);
        z.gg = (cplx *)malloc(sizeof(cplx) * ng);
        #pragma omp for schedule(dynamic, 1)
        for (ll iii = 1; iii <= n1mh; iii++) {
            z.rhs = ccap + np * (size_t)(iii - 1);
            memset(z.pc, 0, sizeof(cplx) * np);
            memset(z.resd, 0, sizeof(cplx) * ng);
            memset(z.gg, 0, sizeof(cplx) * ng);
            int unc = 0;
            ll it = iii <= c->c.imgsor ? xft_mg2d(c, &z, iii, test, 0.0, &unc) : xft_gsor2d(c, &z, iii, test, 0.0, &unc);
            if (it > itmax) itmax = it;
            nunc += unc;
            for (ll j = 1; j <= n2m; j++)
                for (ll k = 1; k <= n3m; k++) z.rhs[(size_t)k + (size_t)ld_p * (size_t)j] = PC(&z, k, j);
        }
        free(z.pc); free(z.resd); free(z.gg);
    }
    #pragma omp parallel
    {
        cplx *line = (cplx *)malloc(sizeof(cplx) * (size_t)n1m), *wk = (cplx *)malloc(sizeof(cplx) * 2 * (size_t)n1m);
        #pragma omp for
        for (ll j = 1; j <= n2m; j++)
            for (ll k = 1; k <= n3m; k++) {
                for (ll i = 1; i <= n1mh; i++) line[i - 1] = ccap[(size_t)k + (size_t)ld_p * (size_t)j + np * (size_t)(i - 1)];
                for (ll i = n1mh + 1; i <= n1m; i++) {
                    cplx s = ccap[(size_t)k + (size_t)ld_p * (size_t)j + np * (size_t)(n1m + 2 - i - 1)];
                    s.im = -s.im;
                    line[i - 1] = s;
                }
                ref_fft(&c->fftx, line, wk, 1);
                for (ll i = 1; i <= n1m; i++) c->phi[IX(c, i, j, k)] = line[i - 1].re;
            }
        free(line); free(wk);
    }
    free(ccap);
    if (c->c.ich == 1) {   /* the f2fx-weighted mean of phi(:,n2m,1) becomes zero */
        double phiref = 0.0;
        for (ll i = 1; i <= n1m; i++) phiref = phiref + c->phi[IX(c, i, n2m, 1)] * c->f2fx[i];
        phiref = phiref / c->xl;
        for (ll k = 1; k <= n3m; k++)
            for (ll j = 1; j <= n2m; j++)
                for (ll i = 1; i <= n1m; i++) c->phi[IX(c, i, j, k)] = c->phi[IX(c, i, j, k)] - phiref;
    }
    c->poisson_iters[c->msub >= 1 && c->msub <= 3 ? c->msub - 1 : 0] = itmax;
    c->poisson_unconv += nunc;
}

/* ------------------------------------------------------------ mgrd ---- */
/* BiCGSTAB with a one-V-cycle MG3D preconditioner (poiss_mgrd.f90).  The
   levels are laid side by side along x and along z as in the reference
   (level ilev occupies i = iimg[ilev][0..1], k = kkmg[ilev][0..1]); y is never
   coarsened.  gi is (0:n1md, 0:n2, 0:n3md), resid and bet/gam are
   (n1md, n2m, n3md).  gi starts at zero in every mg3d call (the reference's
   automatic array is uninitialised; every read of a never-written element is
   multiplied by a zero coefficient). */
#define MG_G(c, i, j, k) ((size_t)(i) + (size_t)((c)->n1md + 1) * ((size_t)(j) + (size_t)((c)->n2 + 1) * (size_t)(k)))
#define MG_R(c, i, j, k) ((size_t)((i) - 1) + (size_t)(c)->n1md * ((size_t)((j) - 1) + (size_t)(c)->n2m * (size_t)((k) - 1)))

/* mgcoef + tridcoef, poiss_mgrd.f90:717-993 (poisinit :678-715 gives the
   finest-level coefficients) */
static int mgrd_init(ref_case *c)
{
    ll n1 = c->n1, n3 = c->n3, n1m = c->n1m, n2m = c->n2m, n3m = c->n3m, n1md = c->n1md, n3md = c->n3md;
    ll nlev = c->c.nlev;
    if (nlev < 0 || nlev > 20 || n1m % (1LL << nlev) != 0 || n3m % (1LL << nlev) != 0) return LESGPU_ERR_CONFIG;
    if (c->c.yprdic == 1) return LESGPU_ERR_UNSUPPORTED;
    for (ll l = 0; l <= nlev; l++) {      /* periodic directions need even level sizes (a proper zebra) */
        if (c->c.xprdic == 1 && ((n1m >> (nlev - l)) % 2) != 0 && (n1m >> (nlev - l)) > 1) return LESGPU_ERR_CONFIG;
        if (c->c.zprdic == 1 && ((n3m >> (nlev - l)) % 2) != 0 && (n3m >> (nlev - l)) > 1) return LESGPU_ERR_CONFIG;
    }
    size_t nvx = (size_t)n1md + 2, nvz = (size_t)n3md + 2;
    c->aw = ref_zalloc(nvx); c->ae = ref_zalloc(nvx); c->as = ref_zalloc((size_t)n2m + 2); c->an = ref_zalloc((size_t)n2m + 2);
    c->ab = ref_zalloc(nvz); c->af = ref_zalloc(nvz);
    c->fidw = ref_zalloc(nvx); c->fiup = ref_zalloc(nvx); c->fkdw = ref_zalloc(nvz); c->fkup = ref_zalloc(nvz);
    c->ih1 = ref_izalloc(nvx); c->ih2 = ref_izalloc(nvx); c->il1 = ref_izalloc(nvx); c->il2 = ref_izalloc(nvx);
    c->kh1 = ref_izalloc(nvz); c->kh2 = ref_izalloc(nvz); c->kl1 = ref_izalloc(nvz); c->kl2 = ref_izalloc(nvz);
    c->ipm = ref_izalloc(nvx); c->imm = ref_izalloc(nvx); c->kpm = ref_izalloc(nvz); c->kmm = ref_izalloc(nvz);
    size_t na = (size_t)n1md * (size_t)n2m * (size_t)n3md;
    c->gam = ref_zalloc(na); c->bet = ref_zalloc(na);
    /* poisinit */
    for (ll i = 1; i <= n1m; i++) {
        ll ip = c->ipv[i];
        c->aw[i] = (1.0 - (double)c->fixil[i]) * c->c2cxi[i] * c->f2fxi[i];
        c->ae[i] = (1.0 - (double)c->fixiu[i]) * c->c2cxi[ip] * c->f2fxi[i];
    }
    for (ll j = 1; j <= n2m; j++) {
        ll jp = c->jpv[j];
        c->as[j] = (1.0 - (double)c->fixjl[j]) * c->c2cyi[j] * c->f2fyi[j];
        c->an[j] = (1.0 - (double)c->fixju[j]) * c->c2cyi[jp] * c->f2fyi[j];
    }
    for (ll k = 1; k <= n3m; k++) {
        ll kp = c->kpv[k];
        c->ab[k] = (1.0 - (double)c->fixkl[k]) * c->c2czi[k] * c->f2fzi[k];
        c->af[k] = (1.0 - (double)c->fixku[k]) * c->c2czi[kp] * c->f2fzi[k];
    }
    /* mgcoef: level index ranges */
    c->iimg[nlev][0] = 1; c->iimg[nlev][1] = n1m; c->iimg[nlev][2] = n1m;
    c->kkmg[nlev][0] = 1; c->kkmg[nlev][1] = n3m; c->kkmg[nlev][2] = n3m;
    for (ll l = nlev - 1; l >= 0; l--) {
        c->iimg[l][0] = c->iimg[l + 1][0] + c->iimg[l + 1][2];
        c->iimg[l][2] = (n1m / (1LL << nlev)) * (1LL << l);
        c->iimg[l][1] = c->iimg[l][0] + c->iimg[l][2] - 1;
        c->kkmg[l][0] = c->kkmg[l + 1][0] + c->kkmg[l + 1][2];
        c->kkmg[l][2] = (n3m / (1LL << nlev)) * (1LL << l);
        c->kkmg[l][1] = c->kkmg[l][0] + c->kkmg[l][2] - 1;
    }
    double *xmpm = ref_zalloc(nvx), *zmpm = ref_zalloc(nvz);
    ll *iwest = ref_izalloc(nvx), *ieast = ref_izalloc(nvx), *kback = ref_izalloc(nvz), *kforw = ref_izalloc(nvz);
    const double *x = c->x, *z = c->z;
    for (ll i = 1; i <= n1m; i++) { xmpm[i] = c->xmp[i]; iwest[i] = 1 - 1 / i; ieast[i] = 1 - i / n1m; }
    for (ll k = 1; k <= n3m; k++) { zmpm[k] = c->zmp[k]; kback[k] = 1 - 1 / k; kforw[k] = 1 - k / n3m; }
    for (ll l = nlev - 1; l >= 0; l--) {
        ll ibg = c->iimg[l][0], iend = c->iimg[l][1], kbg = c->kkmg[l][0], kend = c->kkmg[l][1];
        ll sp = 1LL << (nlev - l), ic = 0;
        for (ll i = ibg; i <= iend; i++) {
            ic++;
            xmpm[i] = 0.5 * (x[(ic - 1) * sp + 1] + x[ic * sp + 1]);
            iwest[i] = 1 - ibg / i; ieast[i] = 1 - i / iend;
        }
        ic = 0;
        for (ll k = kbg; k <= kend; k++) {
            ic++;
            zmpm[k] = 0.5 * (z[(ic - 1) * sp + 1] + z[ic * sp + 1]);
            kback[k] = 1 - kbg / k; kforw[k] = 1 - k / kend;
        }
        /* a factor that is zero (the non-periodic edges) multiplies a
           difference with a point outside the level: left at zero here */
        ic = 0;
        for (ll i = ibg; i <= iend; i++) {
            ic++;
            double w = x[ic * sp + 1] - x[(ic - 1) * sp + 1];
            c->aw[i] = iwest[i] ? 1.0 / ((xmpm[i] - xmpm[i - 1]) * w) : 0.0;
            c->ae[i] = ieast[i] ? 1.0 / ((xmpm[i + 1] - xmpm[i]) * w) : 0.0;
        }
        ic = 0;
        for (ll k = kbg; k <= kend; k++) {
            ic++;
            double w = z[ic * sp + 1] - z[(ic - 1) * sp + 1];
            c->ab[k] = kback[k] ? 1.0 / ((zmpm[k] - zmpm[k - 1]) * w) : 0.0;
            c->af[k] = kforw[k] ? 1.0 / ((zmpm[k + 1] - zmpm[k]) * w) : 0.0;
        }
    }
    /* restriction */
    for (ll l = 0; l <= nlev - 1; l++) {
        ll h = c->iimg[l + 1][0];
        for (ll i = c->iimg[l][0]; i <= c->iimg[l][1]; i++, h += 2) {
            c->fidw[i] = (xmpm[i] - xmpm[h]) / (xmpm[h + 1] - xmpm[h]);
            c->ih1[i] = h; c->ih2[i] = h + 1;
        }
        h = c->kkmg[l + 1][0];
        for (ll k = c->kkmg[l][0]; k <= c->kkmg[l][1]; k++, h += 2) {
            c->fkdw[k] = (zmpm[k] - zmpm[h]) / (zmpm[h + 1] - zmpm[h]);
            c->kh1[k] = h; c->kh2[k] = h + 1;
        }
    }
    /* prolongation (the first and last points get the Neumann weights 1 and
       0; their other index points outside the coarser level) */
    for (ll l = 1; l <= nlev; l++) {
        ll lo = c->iimg[l - 1][0];
        for (ll i = c->iimg[l][0]; i <= c->iimg[l][1]; i += 2, lo++) {
            if (i > c->iimg[l][0]) c->fiup[i] = (xmpm[i] - xmpm[lo - 1]) / (xmpm[lo] - xmpm[lo - 1]);
            if (i + 1 < c->iimg[l][1]) c->fiup[i + 1] = (xmpm[i + 1] - xmpm[lo]) / (xmpm[lo + 1] - xmpm[lo]);
            c->il1[i] = lo - 1; c->il2[i] = lo; c->il1[i + 1] = lo; c->il2[i + 1] = lo + 1;
        }
        c->fiup[c->iimg[l][0]] = 1.0;
        c->fiup[c->iimg[l][1]] = 0.0;
        lo = c->kkmg[l - 1][0];
        for (ll k = c->kkmg[l][0]; k <= c->kkmg[l][1]; k += 2, lo++) {
            if (k > c->kkmg[l][0]) c->fkup[k] = (zmpm[k] - zmpm[lo - 1]) / (zmpm[lo] - zmpm[lo - 1]);
            if (k + 1 < c->kkmg[l][1]) c->fkup[k + 1] = (zmpm[k + 1] - zmpm[lo]) / (zmpm[lo + 1] - zmpm[lo]);
            c->kl1[k] = lo - 1; c->kl2[k] = lo; c->kl1[k + 1] = lo; c->kl2[k + 1] = lo + 1;
        }
        c->fkup[c->kkmg[l][0]] = 1.0;
        c->fkup[c->kkmg[l][1]] = 0.0;
    }
    for (ll l = nlev; l >= 0; l--) {
        for (ll k = c->kkmg[l][0]; k <= c->kkmg[l][1]; k++) { c->kpm[k] = k + 1; c->kmm[k] = k - 1; }
        for (ll i = c->iimg[l][0]; i <= c->iimg[l][1]; i++) { c->ipm[i] = i + 1; c->imm[i] = i - 1; }
    }
    if (c->c.xprdic == 1) {
        for (ll l = nlev; l >= 0; l--) { c->ipm[c->iimg[l][1]] = c->iimg[l][0]; c->imm[c->iimg[l][0]] = c->iimg[l][1]; }
        for (ll l = nlev - 1; l >= 0; l--) {
            ll ibg = c->iimg[l][0], iend = c->iimg[l][1], sp = 1LL << (nlev - l);
            double vdx = xmpm[ibg] - x[1] + x[n1] - xmpm[iend];
            c->aw[ibg] = 1.0 / (vdx * (x[1 + sp] - x[1]));
            c->ae[iend] = 1.0 / (vdx * (x[n1] - x[n1 - sp]));
        }
        for (ll l = 1; l <= nlev; l++) {
            ll ibg = c->iimg[l][0], iend = c->iimg[l][1], ibgl = c->iimg[l - 1][0], iendl = c->iimg[l - 1][1];
            double dx = xmpm[ibgl] - x[1] + x[n1] - xmpm[iendl];
            c->fiup[ibg] = (x[n1] - xmpm[iendl] + xmpm[ibg] - x[1]) / dx;
            c->fiup[iend] = (xmpm[iend] - xmpm[iendl]) / dx;
            c->il1[ibg] = iendl; c->il2[ibg] = ibgl; c->il1[iend] = iendl; c->il2[iend] = ibgl;
        }
    }
    if (c->c.zprdic == 1) {
        for (ll l = nlev; l >= 0; l--) { c->kpm[c->kkmg[l][1]] = c->kkmg[l][0]; c->kmm[c->kkmg[l][0]] = c->kkmg[l][1]; }
        for (ll l = nlev - 1; l >= 0; l--) {
            ll kbg = c->kkmg[l][0], kend = c->kkmg[l][1], sp = 1LL << (nlev - l);
            double vdz = zmpm[kbg] - z[1] + z[n3] - zmpm[kend];
            c->ab[kbg] = 1.0 / (vdz * (z[1 + sp] - z[1]));
            c->af[kend] = 1.0 / (vdz * (z[n3] - z[n3 - sp]));
        }
        for (ll l = 1; l <= nlev; l++) {
            ll kbg = c->kkmg[l][0], kend = c->kkmg[l][1], kbgl = c->kkmg[l - 1][0], kendl = c->kkmg[l - 1][1];
            double dz = zmpm[kbgl] - z[1] + z[n3] - zmpm[kendl];
            c->fkup[kbg] = (z[n3] - zmpm[kendl] + zmpm[kbg] - z[1]) / dz;
            c->fkup[kend] = (zmpm[kend] - zmpm[kendl]) / dz;
            c->kl1[kbg] = kendl; c->kl2[kbg] = kbgl; c->kl1[kend] = kendl; c->kl2[kend] = kbgl;
        }
    }
    /* tridcoef */
    for (ll l = 0; l <= nlev; l++)
        for (ll k = c->kkmg[l][0]; k <= c->kkmg[l][1]; k++)
            for (ll i = c->iimg[l][0]; i <= c->iimg[l][1]; i++) {
                double acc = -1.0 * (c->aw[i] + c->ae[i] + c->as[1] + c->an[1] + c->ab[k] + c->af[k]);
                c->bet[MG_R(c, i, 1, k)] = 1.0 / acc;
                for (ll j = 2; j <= n2m; j++) {
                    acc = -1.0 * (c->aw[i] + c->ae[i] + c->as[j] + c->an[j] + c->ab[k] + c->af[k]);
                    double g = c->an[j - 1] * c->bet[MG_R(c, i, j - 1, k)];
                    c->gam[MG_R(c, i, j, k)] = g;
                    c->bet[MG_R(c, i, j, k)] = 1.0 / (acc - c->as[j] * g);
                }
            }
    free(xmpm); free(zmpm); free(iwest); free(ieast); free(kback); free(kforw);
    return 0;
}

/* One zebra half-sweep at level l: the y lines (i, k) with
   i = i0(k), i0(k)+2, ... take rhs - iold * (x and z neighbours) and are
   solved with the stored LU (relax / toplevel, poiss_mgrd.f90:271-330,
   502-568).  color 0 starts at iimg + mod(kpm(k), 2), color 1 at
   iimg + mod(k, 2).  src(i, j, k) gives the right-hand side. */
typedef double (*mg_src_fn)(const ref_case *c, const double *src, ll i, ll j, ll k);
static double mg_src_resid(const ref_case *c, const double *src, ll i, ll j, ll k) { return src[MG_R(c, i, j, k)]; }
static double mg_src_full(const ref_case *c, const double *src, ll i, ll j, ll k) { return src[IX(c, i, j, k)]; }

static void mg_half(const ref_case *c, double *gi, const double *src, mg_src_fn fs, ll l, int color, double iold)
{
    ll n2m = c->n2m;
    for (ll k = c->kkmg[l][0]; k <= c->kkmg[l][1]; k++) {
        ll i0 = c->iimg[l][0] + (color == 0 ? c->kpm[k] % 2 : k % 2);
        for (ll i = i0; i <= c->iimg[l][1]; i += 2) {
            for (ll j = 1; j <= n2m; j++)
                gi[MG_G(c, i, j, k)] = fs(c, src, i, j, k) - iold * (c->aw[i] * gi[MG_G(c, c->imm[i], j, k)] + c->ae[i] * gi[MG_G(c, c->ipm[i], j, k)]
                                                                     + c->ab[k] * gi[MG_G(c, i, j, c->kmm[k])] + c->af[k] * gi[MG_G(c, i, j, c->kpm[k])]);
        }
    }
    for (ll k = c->kkmg[l][0]; k <= c->kkmg[l][1]; k++) {
        ll i0 = c->iimg[l][0] + (color == 0 ? c->kpm[k] % 2 : k % 2);
        for (ll i = i0; i <= c->iimg[l][1]; i += 2) {
            gi[MG_G(c, i, 1, k)] = gi[MG_G(c, i, 1, k)] * c->bet[MG_R(c, i, 1, k)];
            for (ll j = 2; j <= n2m; j++)
                gi[MG_G(c, i, j, k)] = (gi[MG_G(c, i, j, k)] - c->as[j] * gi[MG_G(c, i, j - 1, k)]) * c->bet[MG_R(c, i, j, k)];
            for (ll j = n2m - 1; j >= 1; j--)
                gi[MG_G(c, i, j, k)] = gi[MG_G(c, i, j, k)] - c->gam[MG_R(c, i, j + 1, k)] * gi[MG_G(c, i, j + 1, k)];
        }
    }
}

/* rhs - A gi at (i, j, k) of any level (rescal / toplevel's residual) */
static inline double mg_defect(const ref_case *c, const double *gi, double rhs, ll i, ll j, ll k)
{
    double acc = -1.0 * (c->aw[i] + c->ae[i] + c->as[j] + c->an[j] + c->ab[k] + c->af[k]);
    return rhs - acc * gi[MG_G(c, i, j, k)] - c->aw[i] * gi[MG_G(c, c->imm[i], j, k)] - c->ae[i] * gi[MG_G(c, c->ipm[i], j, k)]
           - c->as[j] * gi[MG_G(c, i, j - 1, k)] - c->an[j] * gi[MG_G(c, i, j + 1, k)]
           - c->ab[k] * gi[MG_G(c, i, j, c->kmm[k])] - c->af[k] * gi[MG_G(c, i, j, c->kpm[k])];
}

/* godown, poiss_mgrd.f90:455-476: restrict resid from level l+1 to l */
static void mg_godown(const ref_case *c, double *resid, ll l)
{
    for (ll k = c->kkmg[l][0]; k <= c->kkmg[l][1]; k++)
        for (ll j = 1; j <= c->n2m; j++)
            for (ll i = c->iimg[l][0]; i <= c->iimg[l][1]; i++) {
                double fi = c->fidw[i], fk = c->fkdw[k];
                resid[MG_R(c, i, j, k)] = (1.0 - fi) * (1.0 - fk) * resid[MG_R(c, c->ih1[i], j, c->kh1[k])]
                                          + fi * (1.0 - fk) * resid[MG_R(c, c->ih2[i], j, c->kh1[k])]
                                          + (1.0 - fi) * fk * resid[MG_R(c, c->ih1[i], j, c->kh2[k])]
                                          + fi * fk * resid[MG_R(c, c->ih2[i], j, c->kh2[k])];
            }
}

/* goup, poiss_mgrd.f90:479-500: add the interpolated correction of level
   l-1 to the points i = iimg + mod(k, 2), +2, ... of level l.  An index
   outside the coarser level carries a zero weight and reads zero. */
static void mg_goup(const ref_case *c, double *gi, ll l)
{
    ll lo_i = c->iimg[l - 1][0], hi_i = c->iimg[l - 1][1], lo_k = c->kkmg[l - 1][0], hi_k = c->kkmg[l - 1][1];
    for (ll k = c->kkmg[l][0]; k <= c->kkmg[l][1]; k++) {
        ll i0 = c->iimg[l][0] + k % 2;
        for (ll j = 1; j <= c->n2m; j++)
            for (ll i = i0; i <= c->iimg[l][1]; i += 2) {
                double fi = c->fiup[i], fk = c->fkup[k];
                ll a1 = c->il1[i], a2 = c->il2[i], b1 = c->kl1[k], b2 = c->kl2[k];
#define MG_C(ii, kk) (((ii) >= lo_i && (ii) <= hi_i && (kk) >= lo_k && (kk) <= hi_k) ? gi[MG_G(c, ii, j, kk)] : 0.0)
                gi[MG_G(c, i, j, k)] = gi[MG_G(c, i, j, k)] + (1.0 - fi) * (1.0 - fk) * MG_C(a1, b1) + fi * (1.0 - fk) * MG_C(a2, b1)
                                       + (1.0 - fi) * fk * MG_C(a1, b2) + fi * fk * MG_C(a2, b2);
#undef MG_C
            }
    }
}

/* mg3d, poiss_mgrd.f90:227-268 (+ toplevel :271-400, rescal :403-425,
   relax :502-675); sol and rhs are full arrays, only their interior is used */
static void mg3d(const ref_case *c, double *sol, const double *rhs, double *gi, double *resid, double iold)
{
    ll nlev = c->c.nlev, n2m = c->n2m, nbli = c->c.nbli;
    memset(gi, 0, sizeof(double) * (size_t)(c->n1md + 1) * (size_t)(c->n2 + 1) * (size_t)(c->n3md + 1));
    for (int pass = 0; pass < 2; pass++) {
        double io = pass == 0 ? iold : 1.0;
        /* toplevel */
        mg_half(c, gi, rhs, mg_src_full, nlev, 0, io);
        mg_half(c, gi, rhs, mg_src_full, nlev, 1, 1.0);
        if (pass == 1) break;              /* the closing toplevel's residual is discarded */
        for (ll k = 1; k <= c->n3m; k++)
            for (ll j = 1; j <= n2m; j++)
                for (ll i = 1; i <= c->n1m; i++)
                    resid[MG_R(c, i, j, k)] = mg_defect(c, gi, rhs[IX(c, i, j, k)], i, j, k);
        if (nlev > 0) {
            mg_godown(c, resid, nlev - 1);
            for (ll l = nlev - 1; l >= 1; l--) {
                mg_half(c, gi, resid, mg_src_resid, l, 0, 0.0);
                mg_half(c, gi, resid, mg_src_resid, l, 1, 1.0);
                for (ll k = c->kkmg[l][0]; k <= c->kkmg[l][1]; k++)
                    for (ll j = 1; j <= n2m; j++)
                        for (ll i = c->iimg[l][0]; i <= c->iimg[l][1]; i++)
                            resid[MG_R(c, i, j, k)] = mg_defect(c, gi, resid[MG_R(c, i, j, k)], i, j, k);
                mg_godown(c, resid, l - 1);
            }
            mg_half(c, gi, resid, mg_src_resid, 0, 0, 0.0);
            mg_half(c, gi, resid, mg_src_resid, 0, 1, 1.0);
            for (ll it = 1; it < nbli; it++) {
                mg_half(c, gi, resid, mg_src_resid, 0, 0, 1.0);
                mg_half(c, gi, resid, mg_src_resid, 0, 1, 1.0);
            }
            for (ll l = 1; l <= nlev - 1; l++) {
                mg_goup(c, gi, l);
                mg_half(c, gi, resid, mg_src_resid, l, 0, 1.0);
                mg_half(c, gi, resid, mg_src_resid, l, 1, 1.0);
            }
            mg_goup(c, gi, nlev);
        }
    }
    for (ll k = 1; k <= c->n3m; k++)
        for (ll j = 1; j <= n2m; j++)
            for (ll i = 1; i <= c->n1m; i++) sol[IX(c, i, j, k)] = gi[MG_G(c, i, j, k)];
}

/* A q at an interior point (the 7-point operator of poisson :113-122) */
static inline double mg_apply(const ref_case *c, const double *q, ll i, ll j, ll k)
{
    double acc = -1.0 * (c->aw[i] + c->ae[i] + c->as[j] + c->an[j] + c->ab[k] + c->af[k]);
    return c->aw[i] * q[IX(c, c->imm[i], j, k)] + c->ae[i] * q[IX(c, c->ipm[i], j, k)] + c->as[j] * q[IX(c, i, j - 1, k)]
           + c->an[j] * q[IX(c, i, j + 1, k)] + c->ab[k] * q[IX(c, i, j, c->kmm[k])] + c->af[k] * q[IX(c, i, j, c->kpm[k])]
           + acc * q[IX(c, i, j, k)];
}

/* poisson, poiss_mgrd.f90:25-224 (IOLDV = 1 starts from phi = 0 as well:
   solver.f90 zeroes phi before every call) */
static void mgrd_poisson(ref_case *c)
{
    ll n1m = c->n1m, n2m = c->n2m, n3m = c->n3m;
    size_t nt = (size_t)(c->n1 + 1) * (size_t)(c->n2 + 1) * (size_t)(c->n3 + 1);
    double *p = ref_zalloc(nt), *s = ref_zalloc(nt), *y = ref_zalloc(nt), *zz = ref_zalloc(nt), *v = ref_zalloc(nt);
    double *t = ref_zalloc(nt), *res = ref_zalloc(nt);
    double *gi = ref_zalloc((size_t)(c->n1md + 1) * (size_t)(c->n2 + 1) * (size_t)(c->n3md + 1));
    double *resid = ref_zalloc((size_t)c->n1md * (size_t)n2m * (size_t)c->n3md);
    const double *b = c->divgsum;
    double *phi = c->phi;
    for (size_t q = 0; q < nt; q++) phi[q] = 0.0;
    for (ll k = 1; k <= n3m; k++)
        for (ll j = 1; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++) res[IX(c, i, j, k)] = b[IX(c, i, j, k)];
    double rho_ol = 1.0, alp = 1.0, w = 1.0;
    ll it, done = c->c.mgitr;
    for (it = 1; it <= c->c.mgitr; it++) {
        double rho = 0.0;
        for (ll k = 1; k <= n3m; k++)
            for (ll j = 1; j <= n2m; j++)
                for (ll i = 1; i <= n1m; i++) rho += b[IX(c, i, j, k)] * res[IX(c, i, j, k)];
        double bet = rho / rho_ol * alp / w;
        for (ll k = 1; k <= n3m; k++)
            for (ll j = 1; j <= n2m; j++)
                for (ll i = 1; i <= n1m; i++) {
                    size_t q = IX(c, i, j, k);
                    p[q] = res[q] + bet * (p[q] - w * v[q]);
                }
        mg3d(c, y, p, gi, resid, (double)c->c.ioldv);
        double rv = 0.0;
        for (ll k = 1; k <= n3m; k++)
            for (ll j = 1; j <= n2m; j++)
                for (ll i = 1; i <= n1m; i++) {
                    size_t q = IX(c, i, j, k);
                    v[q] = mg_apply(c, y, i, j, k);
                    rv += b[q] * v[q];
                }
        alp = rho / rv;
        for (ll k = 1; k <= n3m; k++)
            for (ll j = 1; j <= n2m; j++)
                for (ll i = 1; i <= n1m; i++) {
                    size_t q = IX(c, i, j, k);
                    s[q] = res[q] - alp * v[q];
                }
        mg3d(c, zz, s, gi, resid, (double)c->c.ioldv);
        double up = 0.0, bt = 0.0;
        for (ll k = 1; k <= n3m; k++)
            for (ll j = 1; j <= n2m; j++)
                for (ll i = 1; i <= n1m; i++) {
                    size_t q = IX(c, i, j, k);
                    t[q] = mg_apply(c, zz, i, j, k);
                    up += t[q] * s[q];
                    bt += t[q] * t[q];
                }
        w = up / bt;
        double resm = 0.0;
        for (ll k = 1; k <= n3m; k++)
            for (ll j = 1; j <= n2m; j++)
                for (ll i = 1; i <= n1m; i++) {
                    size_t q = IX(c, i, j, k);
                    phi[q] = phi[q] + alp * y[q] + w * zz[q];
                    res[q] = s[q] - w * t[q];
                    if (fabs(res[q]) > resm) resm = fabs(res[q]);
                }
        rho_ol = rho;
        if (resm < c->test1) { done = it; break; }
    }
    if (it > c->c.mgitr) c->poisson_unconv += 1;   /* poiss_mgrd.f90:204: NOT CONVERGED, goes on */
    double phiref = phi[IX(c, 1, n2m, 1)];
    for (ll k = 1; k <= n3m; k++)
        for (ll j = 1; j <= n2m; j++)
            for (ll i = 1; i <= n1m; i++) phi[IX(c, i, j, k)] = phi[IX(c, i, j, k)] - phiref;
    free(p); free(s); free(y); free(zz); free(v); free(t); free(res); free(gi); free(resid);
    c->poisson_iters[c->msub >= 1 && c->msub <= 3 ? c->msub - 1 : 0] = done;
}

/* ------------------------------------------------------------ dispatch -- */
int ref_poisinit(ref_case *c)
{
    switch (c->c.poisson) {
    case LESGPU_POISSON_FTFT:
        if (c->c.xprdic != 1 || c->c.zprdic != 1) return LESGPU_ERR_CONFIG;
        if (ref_fft_plan_init(&c->fftx, (int)c->n1m) || ref_fft_plan_init(&c->fftz, (int)c->n3m)) return LESGPU_ERR_ARG;
        ftft_init(c);
        return 0;
    case LESGPU_POISSON_Z_FT:
        if (c->c.zprdic != 1 && c->n3m > 1) return LESGPU_ERR_CONFIG;
        return zft_init(c);
    case LESGPU_POISSON_MGRD:
        return mgrd_init(c);
    case LESGPU_POISSON_X_FT:
        return xft_init(c);
    default:
        return LESGPU_ERR_UNSUPPORTED;
    }
}

void ref_poisson(ref_case *c)
{
    switch (c->c.poisson) {
    case LESGPU_POISSON_FTFT: ftft_poisson(c); break;
    case LESGPU_POISSON_Z_FT: zft_poisson(c); break;
    case LESGPU_POISSON_MGRD: mgrd_poisson(c); break;
    case LESGPU_POISSON_X_FT: xft_poisson(c); break;
    default: break;
    }
}
