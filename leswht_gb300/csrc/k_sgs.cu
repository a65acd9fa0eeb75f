// Dynamic SGS models of 02_solver/f90/lib/sgs.f90: the dynamic Vreman eddy
// viscosity with one global coefficient (sgs_dvmg :405-638, constant form
// sgs_cvm :335), the dynamic eddy diffusivity (sgs_edm :1297-1478, constant
// form sgs_cedm :1250), the Simpson test filter (test_filter :641-769),
// nutzero/alpzero and the edge interpolations nutinterpol/alpinterpol.
//
// The reference filters each of its 24 temporaries with two full-array
// passes (x, then z) through stack copies.  Here one kernel filters a whole
// batch of arrays in a single pass: for output (i,k) it rebuilds the three
// x-filtered values at k-1, k, k+1 in registers and applies the z weights to
// them, which is the reference's arithmetic with its rounding order and a
// third of its memory traffic.
#include "lesgpu_internal.cuh"

namespace lg {

// velgrad, sgs.f90:772-875
__device__ void velgrad(const KP &p, int i, int j, int k, double a[9], double sr[6]) {
    const DGrid &g = p.g;
    const double *u = p.f.u, *v = p.f.v, *w = p.f.w;
    int kp = g.kpv[k], km = g.kmv[k], jp = g.jpv[j], jm = g.jmv[j], ip = g.ipv[i], im = g.imv[i];
    int n1 = g.n1, n2 = g.n2, n3 = g.n3;
    double fju = fixd(g.fixju[j]), fjl = fixd(g.fixjl[j]), fku = fixd(g.fixku[k]), fkl = fixd(g.fixkl[k]);
    double fiu = fixd(g.fixiu[i]), fil = fixd(g.fixil[i]);
    const double *f2fx = g.f2fx, *f2fy = g.f2fy, *f2fz = g.f2fz;
#define U(a_, b_, c_) u[g.ix(a_, b_, c_)]
#define V(a_, b_, c_) v[g.ix(a_, b_, c_)]
#define W(a_, b_, c_) w[g.ix(a_, b_, c_)]
    double vg11 = g.f2fxi[i] * (U(ip, j, k) - U(i, j, k));
    double up = g.c2cyi[jp] * 0.25 * (f2fy[jp] * (U(i, j, k) + U(ip, j, k)) + f2fy[j] * (U(i, jp, k) + U(ip, jp, k))) * (1.0 - fju)
              + 0.5 * (U(i, n2, k) + U(ip, n2, k)) * fju;
    double um = g.c2cyi[j] * 0.25 * (f2fy[j] * (U(i, jm, k) + U(ip, jm, k)) + f2fy[jm] * (U(i, j, k) + U(ip, j, k))) * (1.0 - fjl)
              + 0.5 * (U(i, 0, k) + U(ip, 0, k)) * fjl;
    double vg12 = g.f2fyi[j] * (up - um);
    up = g.c2czi[kp] * 0.25 * (f2fz[kp] * (U(i, j, k) + U(ip, j, k)) + f2fz[k] * (U(i, j, kp) + U(ip, j, kp))) * (1.0 - fku)
       + 0.5 * (U(i, j, n3) + U(ip, j, n3)) * fku;
    um = g.c2czi[k] * 0.25 * (f2fz[k] * (U(i, j, km) + U(ip, j, km)) + f2fz[km] * (U(i, j, k) + U(ip, j, k))) * (1.0 - fkl)
       + 0.5 * (U(i, j, 0) + U(ip, j, 0)) * fkl;
    double vg13 = g.f2fzi[k] * (up - um);
    double vp = g.c2cxi[ip] * 0.25 * (f2fx[ip] * (V(i, j, k) + V(i, jp, k)) + f2fx[i] * (V(ip, j, k) + V(ip, jp, k))) * (1.0 - fiu)
              + 0.5 * (V(n1, j, k) + V(n1, jp, k)) * fiu;
    double vm = g.c2cxi[i] * 0.25 * (f2fx[i] * (V(im, j, k) + V(im, jp, k)) + f2fx[im] * (V(i, j, k) + V(i, jp, k))) * (1.0 - fil)
              + 0.5 * (V(0, j, k) + V(0, jp, k)) * fil;
    double vg21 = g.f2fxi[i] * (vp - vm);
    double vg22 = g.f2fyi[j] * (V(i, jp, k) - V(i, j, k));
    vp = g.c2czi[kp] * 0.25 * (f2fz[kp] * (V(i, j, k) + V(i, jp, k)) + f2fz[k] * (V(i, j, kp) + V(i, jp, kp))) * (1.0 - fku)
       + 0.5 * (V(i, j, n3) + V(i, jp, n3)) * fku;
    vm = g.c2czi[k] * 0.25 * (f2fz[k] * (V(i, j, km) + V(i, jp, km)) + f2fz[km] * (V(i, j, k) + V(i, jp, k))) * (1.0 - fkl)
       + 0.5 * (V(i, j, 0) + V(i, jp, 0)) * fkl;
    double vg23 = g.f2fzi[k] * (vp - vm);
    double wp = g.c2cxi[ip] * 0.25 * (f2fx[ip] * (W(i, j, k) + W(i, j, kp)) + f2fx[i] * (W(ip, j, k) + W(ip, j, kp))) * (1.0 - fiu)
              + 0.5 * (W(n1, j, k) + W(n1, j, kp)) * fiu;
    double wm = g.c2cxi[i] * 0.25 * (f2fx[i] * (W(im, j, k) + W(im, j, kp)) + f2fx[im] * (W(i, j, k) + W(i, j, kp))) * (1.0 - fil)
              + 0.5 * (W(0, j, k) + W(0, j, kp)) * fil;
    double vg31 = g.f2fxi[i] * (wp - wm);
    wp = g.c2cyi[jp] * 0.25 * (f2fy[jp] * (W(i, j, k) + W(i, j, kp)) + f2fy[j] * (W(i, jp, k) + W(i, jp, kp))) * (1.0 - fju)
       + 0.5 * (W(i, n2, k) + W(i, n2, kp)) * fju;
    wm = g.c2cyi[j] * 0.25 * (f2fy[j] * (W(i, jm, k) + W(i, jm, kp)) + f2fy[jm] * (W(i, j, k) + W(i, j, kp))) * (1.0 - fjl)
       + 0.5 * (W(i, 0, k) + W(i, 0, kp)) * fjl;
    double vg32 = g.f2fyi[j] * (wp - wm);
    double vg33 = g.f2fzi[k] * (W(i, j, kp) - W(i, j, k));
#undef U
#undef V
#undef W
    a[0] = vg11; a[1] = vg21; a[2] = vg31;
    a[3] = vg12; a[4] = vg22; a[5] = vg32;
    a[6] = vg13; a[7] = vg23; a[8] = vg33;
    sr[0] = vg11; sr[1] = 0.5 * (vg12 + vg21); sr[2] = 0.5 * (vg13 + vg31);
    sr[3] = vg22; sr[4] = 0.5 * (vg23 + vg32); sr[5] = vg33;
}

// temgrad, sgs.f90:1480-1525
__device__ void temgrad(const KP &p, int i, int j, int k, double a[3]) {
    const DGrid &g = p.g;
    const double *t = p.f.t;
    int kp = g.kpv[k], km = g.kmv[k], jp = g.jpv[j], jm = g.jmv[j], ip = g.ipv[i], im = g.imv[i];
    double fiu = fixd(g.fixiu[i]), fil = fixd(g.fixil[i]), fju = fixd(g.fixju[j]), fjl = fixd(g.fixjl[j]);
    double fku = fixd(g.fixku[k]), fkl = fixd(g.fixkl[k]);
    double tc = t[g.ix(i, j, k)];
    double tip = t[g.ix(ip, j, k)], tim = t[g.ix(im, j, k)];
    double tp = 0.5 * (g.f2fx[i] * tip + g.f2fx[ip] * tc) * g.c2cxi[ip] * (1.0 - fiu) + tip * fiu;
    double tm = 0.5 * (g.f2fx[im] * tc + g.f2fx[i] * tim) * g.c2cxi[i] * (1.0 - fil) + tim * fil;
    a[0] = g.f2fxi[i] * (tp - tm);
    double tjp = t[g.ix(i, jp, k)], tjm = t[g.ix(i, jm, k)];
    tp = 0.5 * (g.f2fy[j] * tjp + g.f2fy[jp] * tc) * g.c2cyi[jp] * (1.0 - fju) + tjp * fju;
    tm = 0.5 * (g.f2fy[jm] * tc + g.f2fy[j] * tjm) * g.c2cyi[j] * (1.0 - fjl) + tjm * fjl;
    a[1] = g.f2fyi[j] * (tp - tm);
    double tkp = t[g.ix(i, j, kp)], tkm = t[g.ix(i, j, km)];
    tp = 0.5 * (g.f2fz[k] * tkp + g.f2fz[kp] * tc) * g.c2czi[kp] * (1.0 - fku) + tkp * fku;
    tm = 0.5 * (g.f2fz[km] * tc + g.f2fz[k] * tkm) * g.c2czi[k] * (1.0 - fkl) + tkm * fkl;
    a[2] = g.f2fzi[k] * (tp - tm);
}

__device__ __forceinline__ void vreman(const double alp[9], double sdx2, double sdy2, double sdz2, double &aaa, double &bbb) {
    double b1 = sdx2 * alp[0] * alp[0] + sdy2 * alp[3] * alp[3] + sdz2 * alp[6] * alp[6];
    double b2 = sdx2 * alp[0] * alp[1] + sdy2 * alp[3] * alp[4] + sdz2 * alp[6] * alp[7];
    double b3 = sdx2 * alp[0] * alp[2] + sdy2 * alp[3] * alp[5] + sdz2 * alp[6] * alp[8];
    double b4 = sdx2 * alp[1] * alp[1] + sdy2 * alp[4] * alp[4] + sdz2 * alp[7] * alp[7];
    double b5 = sdx2 * alp[1] * alp[2] + sdy2 * alp[4] * alp[5] + sdz2 * alp[7] * alp[8];
    double b6 = sdx2 * alp[2] * alp[2] + sdy2 * alp[5] * alp[5] + sdz2 * alp[8] * alp[8];
    double a = 0.0;
#pragma unroll
    for (int q = 0; q < 9; q++) a += alp[q] * alp[q];
    double b = b1 * b4 + b4 * b6 + b6 * b1 - b2 * b2 - b3 * b3 - b5 * b5;
    if (b < 1.0e-16) b = 1.0e-16;
    aaa = a;
    bbb = b;
}

// Test-filter width at a cell: the sum of the three test-filter cell widths
// used in the second Vreman / eddy-diffusivity evaluation (sgs.f90:528-533).
__device__ __forceinline__ double tf_width(const double *f2f, const int *fl, const int *fu, int i) {
    return 0.5 * f2f[i - 1] * (1.0 - fixd(fu[i])) + f2f[i] + 0.5 * f2f[i + 1] * (1.0 - fixd(fl[i]));
}

#define GRID_LOOP(b)                                                                                   \
    for (long long tt = (long long)blockIdx.x * blockDim.x + threadIdx.x, nn_ = (b).count(); tt < nn_; \
         tt += (long long)gridDim.x * blockDim.x)

// pass 1 of sgs_dvmg (:434-491) and the constant model sgs_cvm
__global__ void __launch_bounds__(kThreads) k_vreman1(KP p, Box b, int dynamic) {
    const DGrid &g = p.g;
    double **A = p.f.scr + 3;       // mm[0..5] in scr[3..8], alp[0..8] in scr[9..17]
    GRID_LOOP(b) {
        int i, j, k;
        b.at(tt, i, j, k);
        double alp[9], str[6], aaa, bbb;
        velgrad(p, i, j, k, alp, str);
        vreman(alp, g.f2fx[i] * g.f2fx[i], g.f2fy[j] * g.f2fy[j], g.f2fz[k] * g.f2fz[k], aaa, bbb);
        long long q = g.ix(i, j, k);
        if (!dynamic) {
            p.f.nusgs[q] = (aaa == 0.0) ? 0.0 : p.c.csgsts * sqrt(bbb / aaa);
            continue;
        }
        double nu = (aaa == 0.0) ? 0.0 : sqrt(bbb / aaa);
        p.f.nusgs[q] = nu;
#pragma unroll
        for (int m = 0; m < 6; m++) A[m][q] = nu * str[m];
#pragma unroll
        for (int m = 0; m < 9; m++) A[6 + m][q] = alp[m];
    }
}

// Batched test filter: dst[a] = filter(src[a]) on the interior, a < na.
struct FiltBatch {
    const double *src[16];
    double *dst[16];
    int na;
};

__device__ __forceinline__ double filt_x(const KP &p, const double *s, int i, long long qrow, int xf) {
    const DGrid &g = p.g;
    // qrow = index of (0, j, k)
    if (!xf) return s[qrow + i];
    const double *cf = p.f.cfx1 + 3 * i;
    if (i >= 2 && i <= g.n1m - 1)
        return cf[0] * s[qrow + i - 1] + cf[1] * s[qrow + i] + cf[2] * s[qrow + i + 1];
    if (p.c.xprdic == 1) {
        if (g.n1m == 1) return s[qrow + i];
        if (i == 1) return cf[0] * s[qrow + g.n1m] + cf[1] * s[qrow + 1] + cf[2] * s[qrow + 2];
        return cf[0] * s[qrow + g.n1m - 1] + cf[1] * s[qrow + g.n1m] + cf[2] * s[qrow + 1];
    }
    return s[qrow + i];
}

__global__ void __launch_bounds__(kThreads) k_filter(KP p, Box b, FiltBatch F) {
    const DGrid &g = p.g;
    int xf = (p.c.filter == 1 || p.c.filter == 3) ? 1 : 0;
    int zf = (p.c.filter == 2 || p.c.filter == 3) ? 1 : 0;
    long long n = b.count();
    long long tot = n * F.na;
    for (long long tt = (long long)blockIdx.x * blockDim.x + threadIdx.x; tt < tot; tt += (long long)gridDim.x * blockDim.x) {
        int a = (int)(tt / n);
        int i, j, k;
        b.at(tt - (long long)a * n, i, j, k);
        const double *s = F.src[a];
        double out;
        // z-periodic ends use the wrapped neighbours; with n3m = 1 the weights
        // are zero (sgsfilterinit skips them), so the filtered value is 0 as
        // in test_filter (sgs.f90:735-764)
        bool zin = zf && ((k >= 2 && k <= g.n3m - 1) || p.c.zprdic == 1);
        if (!zin) {
            out = filt_x(p, s, i, g.ix(0, j, k), xf);
        } else {
            int km = k - 1, kp = k + 1;
            if (k == 1) km = g.n3m;
            if (k == g.n3m) kp = 1;
            const double *cf = p.f.cfz1 + 3 * k;
            double xm = filt_x(p, s, i, g.ix(0, j, km), xf);
            double x0 = filt_x(p, s, i, g.ix(0, j, k), xf);
            double xp = filt_x(p, s, i, g.ix(0, j, kp), xf);
            out = cf[0] * xm + cf[1] * x0 + cf[2] * xp;
        }
        F.dst[a][g.ix(i, j, k)] = out;
    }
}

static void filter_batch(lesgpu_case *c, FiltBatch &F) {
    const DGrid &g = c->kp.g;
    Box b{1, 1, 1, g.n1m, g.n2m, g.n3m};
    inst_begin(c, LESGPU_K_SGS);
    k_filter<<<blocks_for(b.count() * F.na), kThreads, 0, c->stream>>>(c->kp, b, F);
    inst_end(c, LESGPU_K_SGS);
}

// pass 2 of sgs_dvmg (:504-580): filtered gradients -> test-level Vreman
// viscosity, M_ij update, resolved velocities and their products.
__global__ void __launch_bounds__(kThreads) k_vreman2(KP p, Box b) {
    const DGrid &g = p.g;
    double **FM = p.f.scr + 18;     // filtered mm[0..5]  (updated in place)
    double **FA = p.f.scr + 24;     // filtered alp[0..8] (scr[24..32])
    double **OUT = p.f.scr + 3;     // uui[0..2], llij[0..5] -> scr[3..11]
    GRID_LOOP(b) {
        int i, j, k;
        b.at(tt, i, j, k);
        long long q = g.ix(i, j, k);
        double alp[9], str[6], aaa, bbb;
#pragma unroll
        for (int m = 0; m < 9; m++) alp[m] = FA[m][q];
        str[0] = alp[0]; str[1] = 0.5 * (alp[3] + alp[1]); str[2] = 0.5 * (alp[6] + alp[2]);
        str[3] = alp[4]; str[4] = 0.5 * (alp[7] + alp[5]); str[5] = alp[8];
        double sx = tf_width(g.f2fx, g.fixil, g.fixiu, i);
        double sy = tf_width(g.f2fy, g.fixjl, g.fixju, j);
        double sz = tf_width(g.f2fz, g.fixkl, g.fixku, k);
        vreman(alp, sx * sx, sy * sy, sz * sz, aaa, bbb);
        double ami = (aaa == 0.0) ? 0.0 : sqrt(bbb / aaa);
#pragma unroll
        for (int m = 0; m < 6; m++) FM[m][q] = ami * str[m] - FM[m][q];
        double u1 = 0.5 * (p.f.u[q] + p.f.u[q + 1]);
        double u2 = 0.5 * (p.f.v[q] + p.f.v[q + g.sx]);
        double u3 = 0.5 * (p.f.w[q] + p.f.w[q + g.sxy]);
        OUT[0][q] = u1; OUT[1][q] = u2; OUT[2][q] = u3;
        OUT[3][q] = u1 * u1; OUT[4][q] = u1 * u2; OUT[5][q] = u1 * u3;
        OUT[6][q] = u2 * u2; OUT[7][q] = u2 * u3; OUT[8][q] = u3 * u3;
    }
}

// global least-squares sums (:593-618)
struct LmMmTerm {
    __device__ void operator()(const KP &p, int i, int j, int k, double *w) const {
        const DGrid &g = p.g;
        long long q = g.ix(i, j, k);
        double *const *FM = p.f.scr + 18;   // M_ij
        double *const *FU = p.f.scr + 24;   // filtered uui (scr[24..26]) and llij (scr[27..32])
        double vol = g.f2fx[i] * g.f2fy[j] * g.f2fz[k];
        double u1 = FU[0][q], u2 = FU[1][q], u3 = FU[2][q];
        double L0 = FU[3][q] - u1 * u1, L1 = FU[4][q] - u1 * u2, L2 = FU[5][q] - u1 * u3;
        double L3 = FU[6][q] - u2 * u2, L4 = FU[7][q] - u2 * u3, L5 = FU[8][q] - u3 * u3;
        double M0 = FM[0][q], M1 = FM[1][q], M2 = FM[2][q], M3 = FM[3][q], M4 = FM[4][q], M5 = FM[5][q];
        double nw = (double)p.f.nwall[q];
        w[0] = (2.0 * L1 * M1 + L0 * M0 + 2.0 * L2 * M2 + L3 * M3 + 2.0 * L4 * M4 + L5 * M5) * nw * vol;
        w[1] = (2.0 * M1 * M1 + M0 * M0 + 2.0 * M2 * M2 + M3 * M3 + 2.0 * M4 * M4 + M5 * M5) * nw * vol;
    }
};
struct CsgstsFinal {
    __device__ void operator()(const KP &p, const double *o) const {
        double cs = -0.5 * o[0] / o[1];
        p.S->csgsts = cs > 0.0 ? cs : 0.0;
    }
};

__global__ void k_scale(KP p, Box b, double *f, int which) {
    double cs = which == 0 ? p.S->csgsts : p.S->csgshf;
    GRID_LOOP(b) {
        int i, j, k;
        b.at(tt, i, j, k);
        long long q = p.g.ix(i, j, k);
        f[q] = cs * f[q];
    }
}

__global__ void k_zero_list(KP p, double *f) {
    for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < p.c.nzero; l += gridDim.x * blockDim.x)
        f[p.g.ix(p.f.inz[l + 1], p.f.jnz[l + 1], p.f.knz[l + 1])] = 0.0;
}

// nutzero / alpzero statistics with the in-body zeroing (sgs.f90:898-925)
struct ZeroSumTerm {
    double *f;
    __device__ void operator()(const KP &p, int i, int j, int k, double *w) const {
        long long q = p.g.ix(i, j, k);
        if (p.f.fb_c[q] >= 1.0e-10) {
            double vol = p.g.f2fx[i] * p.g.f2fy[j] * p.g.f2fz[k];
            w[0] = f[q] * vol;
            w[1] = vol;
        } else {
            f[q] = 0.0;
            w[0] = 0.0;
            w[1] = 0.0;
        }
    }
};
struct ZeroMaxTerm {
    const double *f;
    __device__ void operator()(const KP &p, int i, int j, int k, double *w) const {
        long long q = p.g.ix(i, j, k);
        w[0] = (p.f.fb_c[q] >= 1.0e-10) ? fmax(f[q], 0.0) : 0.0;
    }
};
struct ZeroSumFinal {
    int thermal;
    __device__ void operator()(const KP &p, const double *o) const {
        double avg = o[0] / o[1];
        if (thermal) p.S->alpavg = avg * p.c.re * p.c.pr;
        else p.S->nutavg = avg * p.c.re;
    }
};
struct ZeroMaxFinal {
    int thermal;
    __device__ void operator()(const KP &p, const double *o) const {
        if (thermal) p.S->alpmax = o[0] * p.c.re * p.c.pr;
        else p.S->nutmax = o[0] * p.c.re;
    }
};

// nutinterpol / alpinterpol main loops (sgs.f90:981-1004 / 1627-1650)
__global__ void __launch_bounds__(kThreads) k_edge_interp(KP p, Box b, const double *f, double *f1, double *f2,
                                                           double *f3, int ib, int jb, int kb) {
    const DGrid &g = p.g;
    const double *f2fx = g.f2fx, *f2fy = g.f2fy, *f2fz = g.f2fz;
    GRID_LOOP(b) {
        int i, j, k;
        b.at(tt, i, j, k);
        long long q = g.ix(i, j, k);
        double c = f[q], cim = f[q - 1], cjm = f[q - g.sx], ckm = f[q - g.sxy];
        if (k >= kb && j >= jb)
            f1[q] = g.c2cyi[j] * g.c2czi[k] * 0.25
                  * (f2fy[j - 1] * (f2fz[k - 1] * c + f2fz[k] * ckm) + f2fy[j] * (f2fz[k - 1] * cjm + f2fz[k] * f[q - g.sx - g.sxy]));
        if (k >= kb && i >= ib)
            f2[q] = g.c2czi[k] * g.c2cxi[i] * 0.25
                  * (f2fz[k - 1] * (f2fx[i - 1] * c + f2fx[i] * cim) + f2fz[k] * (f2fx[i - 1] * ckm + f2fx[i] * f[q - 1 - g.sxy]));
        if (j >= jb && i >= ib)
            f3[q] = g.c2cxi[i] * g.c2cyi[j] * 0.25
                  * (f2fx[i - 1] * (f2fy[j - 1] * c + f2fy[j] * cjm) + f2fx[i] * (f2fy[j - 1] * cim + f2fy[j] * f[q - 1 - g.sx]));
    }
}

// boundary fix-ups of nutinterpol/alpinterpol, one direction per launch in
// the reference's order (x, then y, then z)
__global__ void k_edge_bc(KP p, int dir, const double *f, double *f1, double *f2, double *f3,
                          int lo0, int hi0, int lo1, int hi1, int full) {
    const DGrid &g = p.g;
    const DCfg &c = p.c;
    const double *f2fx = g.f2fx, *f2fy = g.f2fy, *f2fz = g.f2fz;
    double *F[3] = {f1, f2, f3};
    int n0 = hi0 - lo0 + 1, nm = hi1 - lo1 + 1;
    long long n = (long long)n0 * nm;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        int a = lo0 + (int)(t % n0), bq = lo1 + (int)(t / n0);
        if (dir == 0) {           // loop j = a, k = bq
            int j = a, k = bq, jm = g.jmv[j], km = g.kmv[k];
            if (c.xprdic == 1) {
                for (int l = 0; l < 3; l++) F[l][g.ix(g.n1, j, k)] = F[l][g.ix(1, j, k)];
            } else {
                F[1][g.ix(1, j, k)] = g.c2czi[k] * 0.5 * (f2fz[k] * f[g.ix(2, j, km)] + f2fz[km] * f[g.ix(2, j, k)]);
                F[2][g.ix(1, j, k)] = g.c2cyi[j] * 0.5 * (f2fy[j] * f[g.ix(2, jm, k)] + f2fy[jm] * f[g.ix(2, j, k)]);
                F[1][g.ix(g.n1, j, k)] = g.c2czi[k] * 0.5 * (f2fz[k] * f[g.ix(g.n1m, j, km)] + f2fz[km] * f[g.ix(g.n1m, j, k)]);
                F[2][g.ix(g.n1, j, k)] = g.c2cyi[j] * 0.5 * (f2fy[j] * f[g.ix(g.n1m, jm, k)] + f2fy[jm] * f[g.ix(g.n1m, j, k)]);
            }
        } else if (dir == 1) {    // loop i = a, k = bq
            int i = a, k = bq, im = g.imv[i], km = g.kmv[k];
            if (c.yprdic == 1) {
                for (int l = 0; l < 3; l++) F[l][g.ix(i, g.n2, k)] = F[l][g.ix(i, 1, k)];
            } else {
                if (c.bc_ybtm == 0) {
                    for (int l = 0; l < 3; l++) F[l][g.ix(i, 1, k)] = 0.0;
                } else {
                    F[1][g.ix(i, 1, k)] = g.c2czi[k] * 0.5 * (f2fz[k] * f[g.ix(i, 2, km)] + f2fz[km] * f[g.ix(i, 2, k)]);
                    F[2][g.ix(i, 1, k)] = g.c2cxi[i] * 0.5 * (f2fx[i] * f[g.ix(im, 2, k)] + f2fx[im] * f[g.ix(i, 2, k)]);
                }
                if (c.bc_ytop == 0) {
                    for (int l = 0; l < 3; l++) F[l][g.ix(i, g.n2, k)] = 0.0;
                } else {
                    F[1][g.ix(i, g.n2, k)] = g.c2czi[k] * 0.5 * (f2fz[k] * f[g.ix(i, g.n2m, km)] + f2fz[km] * f[g.ix(i, g.n2m, k)]);
                    F[2][g.ix(i, g.n2, k)] = g.c2cxi[i] * 0.5 * (f2fx[i] * f[g.ix(im, g.n2m, k)] + f2fx[im] * f[g.ix(i, g.n2m, k)]);
                }
            }
        } else {                  // loop i = a, j = bq
            int i = a, j = bq, im = g.imv[i], jm = g.jmv[j];
            if (c.zprdic == 1) {
                for (int l = 0; l < 3; l++) F[l][g.ix(i, j, g.n3)] = F[l][g.ix(i, j, 1)];
            } else {
                if (c.bc_zbtm == 0) {
                    for (int l = 0; l < 3; l++) F[l][g.ix(i, j, 1)] = 0.0;
                } else {
                    F[1][g.ix(i, j, 1)] = g.c2cyi[j] * 0.5 * (f2fy[j] * f[g.ix(i, jm, 2)] + f2fy[jm] * f[g.ix(i, j, 2)]);
                    F[2][g.ix(i, j, 1)] = g.c2cxi[i] * 0.5 * (f2fx[i] * f[g.ix(im, j, 2)] + f2fx[im] * f[g.ix(i, j, 2)]);
                }
                if (c.bc_ztop == 0) {
                    for (int l = 0; l < 3; l++) F[l][g.ix(i, j, g.n3)] = 0.0;
                } else {
                    // nutinterpol reads c2cyi(k) with k = n3 left by its
                    // previous loop (sgs.f90:1124); alpinterpol reads c2cyi(j)
                    double cyk = full ? g.c2cyi[j] : (g.n3 <= g.n2 ? g.c2cyi[g.n3] : 0.0);
                    F[1][g.ix(i, j, g.n3)] = cyk * 0.5 * (f2fy[j] * f[g.ix(i, jm, g.n3m)] + f2fy[jm] * f[g.ix(i, j, g.n3m)]);
                    F[2][g.ix(i, j, g.n3)] = g.c2cxi[i] * 0.5 * (f2fx[i] * f[g.ix(im, j, g.n3m)] + f2fx[im] * f[g.ix(i, j, g.n3m)]);
                }
            }
        }
    }
}

// nutinterpol (full = 0) / alpinterpol (full = 1)
static void edge_interpol(lesgpu_case *c, double *f, double **f1, int full) {
    const DGrid &g = c->kp.g;
    const DCfg &cf = c->kp.c;
    for (int l = 0; l < 3; l++) cudaMemsetAsync(f1[l], 0, sizeof(double) * g.nt, c->stream);
    if (cf.xprdic == 1) { GhostSpec s[1] = {{f, 0, g.n2, 0, g.n3}}; ghost(c, 0, s, 1); }
    if (cf.yprdic == 1) { GhostSpec s[1] = {{f, 0, g.n1, 0, g.n3}}; ghost(c, 1, s, 1); }
    if (cf.zprdic == 1) { GhostSpec s[1] = {{f, 0, g.n1, 0, g.n2}}; ghost(c, 2, s, 1); }
    int ib = full ? 1 : g.i_bgpx, jb = full ? 1 : g.j_bgpy, kb = full ? 1 : g.k_bgpz;
    Box b{1, 1, 1, g.n1m, g.n2m, g.n3m};
    k_edge_interp<<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b, f, f1[0], f1[1], f1[2], ib, jb, kb);
    long long nx = (long long)(g.n2m - jb + 1) * (g.n3m - kb + 1);
    long long ny = (long long)(g.n1m - ib + 1) * (g.n3m - kb + 1);
    long long nz = (long long)(g.n1m - ib + 1) * (g.n2m - jb + 1);
    k_edge_bc<<<blocks_for(nx), kThreads, 0, c->stream>>>(c->kp, 0, f, f1[0], f1[1], f1[2], jb, g.n2m, kb, g.n3m, full);
    k_edge_bc<<<blocks_for(ny), kThreads, 0, c->stream>>>(c->kp, 1, f, f1[0], f1[1], f1[2], ib, g.n1m, kb, g.n3m, full);
    k_edge_bc<<<blocks_for(nz), kThreads, 0, c->stream>>>(c->kp, 2, f, f1[0], f1[1], f1[2], ib, g.n1m, jb, g.n2m, full);
}

static void zero_in_body(lesgpu_case *c, double *f, int thermal) {
    const DGrid &g = c->kp.g;
    Box b{1, 1, 1, g.n1m, g.n2m, g.n3m};
    if (c->kp.c.nzero > 0) k_zero_list<<<blocks_for(c->kp.c.nzero), kThreads, 0, c->stream>>>(c->kp, f);
    reduce<2, false>(c, b, ZeroSumTerm{f}, ZeroSumFinal{thermal});
    reduce<1, true>(c, b, ZeroMaxTerm{f}, ZeroMaxFinal{thermal});
}

void launch_sgs_zero_first(lesgpu_case *c, int thermal) {
    double *f = thermal ? c->kp.f.alsgs : c->kp.f.nusgs;
    cudaMemsetAsync(f, 0, sizeof(double) * c->kp.g.nt, c->stream);
}

// sgscalc, sgs.f90:288-332 (the msub == 1 / first-step logic is the host's)
void launch_sgs(lesgpu_case *c) {
    const DGrid &g = c->kp.g;
    DFields &f = c->kp.f;
    Box b{1, 1, 1, g.n1m, g.n2m, g.n3m};
    if (c->kp.c.idvmon == 1) {
        k_vreman1<<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b, 1);
        FiltBatch F{};
        F.na = 15;
        for (int m = 0; m < 6; m++) { F.src[m] = f.scr[3 + m]; F.dst[m] = f.scr[18 + m]; }
        for (int m = 0; m < 9; m++) { F.src[6 + m] = f.scr[9 + m]; F.dst[6 + m] = f.scr[24 + m]; }
        filter_batch(c, F);
        k_vreman2<<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b);
        FiltBatch G{};
        G.na = 9;
        for (int m = 0; m < 9; m++) { G.src[m] = f.scr[3 + m]; G.dst[m] = f.scr[24 + m]; }
        filter_batch(c, G);
        reduce<2, false>(c, b, LmMmTerm{}, CsgstsFinal{});
        k_scale<<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b, f.nusgs, 0);
    } else {
        k_vreman1<<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b, 0);
    }
}

void launch_sgs_post(lesgpu_case *c) {
    zero_in_body(c, c->kp.f.nusgs, 0);
    edge_interpol(c, c->kp.f.nusgs, c->kp.f.nusgs1, 0);
}

// ------------------------------------------------------------ thermal EDM
__global__ void __launch_bounds__(kThreads) k_edm1(KP p, Box b, int dynamic) {
    const DGrid &g = p.g;
    double **A = p.f.scr + 3;   // mm[0..2] scr[3..5]; s[0..5] scr[6..11]; tgrad[0..2] scr[12..14]
    GRID_LOOP(b) {
        int i, j, k;
        b.at(tt, i, j, k);
        double d[9], s[6], alp[3];
        velgrad(p, i, j, k, d, s);
        double del = pow(g.f2fx[i] * g.f2fy[j] * g.f2fz[k], 1.0 / 3.0);
        double sss = s[0] * s[0] + 2.0 * s[1] * s[1] + 2.0 * s[2] * s[2] + s[3] * s[3] + 2.0 * s[4] * s[4] + s[5] * s[5];
        if (sss < 1.0e-16) sss = 1.0e-16;
        long long q = g.ix(i, j, k);
        if (!dynamic) {
            p.f.alsgs[q] = p.c.csgshf * (del * del) * sqrt(2.0 * sss);
            continue;
        }
        temgrad(p, i, j, k, alp);
        double al = (del * del) * sqrt(2.0 * sss);
        p.f.alsgs[q] = al;
#pragma unroll
        for (int m = 0; m < 3; m++) A[m][q] = al * alp[m];
#pragma unroll
        for (int m = 0; m < 6; m++) A[3 + m][q] = s[m];
#pragma unroll
        for (int m = 0; m < 3; m++) A[9 + m][q] = alp[m];
    }
}

__global__ void __launch_bounds__(kThreads) k_edm2(KP p, Box b) {
    const DGrid &g = p.g;
    double **FM = p.f.scr + 18;   // filtered mm[0..2] (updated in place)
    double **FS = p.f.scr + 21;   // filtered s[0..5] scr[21..26], tgrad[0..2] scr[27..29]
    double **OUT = p.f.scr + 3;   // uui[0..2] scr[3..5], t scr[6], llij[0..2] scr[7..9]
    GRID_LOOP(b) {
        int i, j, k;
        b.at(tt, i, j, k);
        long long q = g.ix(i, j, k);
        double d1 = tf_width(g.f2fx, g.fixil, g.fixiu, i);
        double d2 = tf_width(g.f2fy, g.fixjl, g.fixju, j);
        double d3 = tf_width(g.f2fz, g.fixkl, g.fixku, k);
        double del = pow(d1 * d2 * d3, 1.0 / 3.0);
        double s0 = FS[0][q], s1 = FS[1][q], s2 = FS[2][q], s3 = FS[3][q], s4 = FS[4][q], s5 = FS[5][q];
        double sss = s0 * s0 + 2.0 * s1 * s1 + 2.0 * s2 * s2 + s3 * s3 + 2.0 * s4 * s4 + s5 * s5;
        if (sss < 1.0e-16) sss = 1.0e-16;
        double ami = (del * del) * sqrt(2.0 * sss);
#pragma unroll
        for (int m = 0; m < 3; m++) FM[m][q] = ami * FS[6 + m][q] - FM[m][q];
        double u1 = 0.5 * (p.f.u[q] + p.f.u[q + 1]);
        double u2 = 0.5 * (p.f.v[q] + p.f.v[q + g.sx]);
        double u3 = 0.5 * (p.f.w[q] + p.f.w[q + g.sxy]);
        double tq = p.f.t[q];
        OUT[0][q] = u1; OUT[1][q] = u2; OUT[2][q] = u3;
        OUT[3][q] = tq;
        OUT[4][q] = u1 * tq; OUT[5][q] = u2 * tq; OUT[6][q] = u3 * tq;
    }
}

struct LmMmTTerm {
    __device__ void operator()(const KP &p, int i, int j, int k, double *w) const {
        const DGrid &g = p.g;
        long long q = g.ix(i, j, k);
        double *const *FM = p.f.scr + 18;   // M_j
        double *const *FU = p.f.scr + 24;   // filtered uui [24..26], t [27], llij [28..30]
        double vol = g.f2fx[i] * g.f2fy[j] * g.f2fz[k];
        double tf = FU[3][q];
        double L0 = FU[4][q] - FU[0][q] * tf, L1 = FU[5][q] - FU[1][q] * tf, L2 = FU[6][q] - FU[2][q] * tf;
        double nw = (double)p.f.nwall[q];
        w[0] = (L0 * FM[0][q] + L1 * FM[1][q] + L2 * FM[2][q]) * nw * vol;
        w[1] = (FM[0][q] * FM[0][q] + FM[1][q] * FM[1][q] + FM[2][q] * FM[2][q]) * nw * vol;
    }
};
struct CsgshfFinal {
    __device__ void operator()(const KP &p, const double *o) const {
        double cs = -o[0] / o[1];
        p.S->csgshf = cs > 0.0 ? cs : 0.0;
    }
};

void launch_sgs_t(lesgpu_case *c) {
    const DGrid &g = c->kp.g;
    DFields &f = c->kp.f;
    Box b{1, 1, 1, g.n1m, g.n2m, g.n3m};
    if (c->kp.c.idvmon == 1) {
        k_edm1<<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b, 1);
        FiltBatch F{};
        F.na = 12;
        for (int m = 0; m < 3; m++) { F.src[m] = f.scr[3 + m]; F.dst[m] = f.scr[18 + m]; }
        for (int m = 0; m < 9; m++) { F.src[3 + m] = f.scr[6 + m]; F.dst[3 + m] = f.scr[21 + m]; }
        filter_batch(c, F);
        k_edm2<<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b);
        FiltBatch G{};
        G.na = 7;
        for (int m = 0; m < 7; m++) { G.src[m] = f.scr[3 + m]; G.dst[m] = f.scr[24 + m]; }
        filter_batch(c, G);
        reduce<2, false>(c, b, LmMmTTerm{}, CsgshfFinal{});
        k_scale<<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b, f.alsgs, 1);
    } else {
        k_edm1<<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b, 0);
    }
}

void launch_sgs_t_post(lesgpu_case *c) {
    zero_in_body(c, c->kp.f.alsgs, 1);
    edge_interpol(c, c->kp.f.alsgs, c->kp.f.alsgs1, 1);
}

}  // namespace lg
