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

/* ------------------------------------------------------------ dispatch -- */
int ref_poisinit(ref_case *c)
{
    switch (c->c.poisson) {
    case LESGPU_POISSON_FTFT:
        if (c->c.xprdic != 1 || c->c.zprdic != 1) return LESGPU_ERR_CONFIG;
        if (ref_fft_plan_init(&c->fftx, (int)c->n1m) || ref_fft_plan_init(&c->fftz, (int)c->n3m)) return LESGPU_ERR_ARG;
        ftft_init(c);
        return 0;
    default:
        return LESGPU_ERR_UNSUPPORTED;
    }
}

void ref_poisson(ref_case *c)
{
    c->poisson_iters = 0;
    switch (c->c.poisson) {
    case LESGPU_POISSON_FTFT: ftft_poisson(c); break;
    default: break;
    }
}
