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

// velgrad, sgs.f90:772-875.  R: arithmetic type (float in the mixed form).
template <class R>
__device__ void velgrad(const KP &p, int i, int j, int k, R a[9], R sr[6]) {
    const Mir<R> &M = mir<R>(p);
    const DGrid &g = p.g;
    const R *u = M.u, *v = M.v, *w = M.w;
    int kp = g.kpv[k], km = g.kmv[k], jp = g.jpv[j], jm = g.jmv[j], ip = g.ipv[i], im = g.imv[i];
    int n1 = g.n1, n2 = g.n2, n3 = g.n3;
    R fju = M.fixju[j], fjl = M.fixjl[j], fku = M.fixku[k], fkl = M.fixkl[k];
    R fiu = M.fixiu[i], fil = M.fixil[i];
    const R *f2fx = M.f2fx, *f2fy = M.f2fy, *f2fz = M.f2fz;
#define U(a_, b_, c_) R(u[g.ix(a_, b_, c_)])
#define V(a_, b_, c_) R(v[g.ix(a_, b_, c_)])
#define W(a_, b_, c_) R(w[g.ix(a_, b_, c_)])
    R vg11 = R(M.f2fxi[i]) * (U(ip, j, k) - U(i, j, k));
    R up = R(M.c2cyi[jp]) * R(0.25) * (R(f2fy[jp]) * (U(i, j, k) + U(ip, j, k)) + R(f2fy[j]) * (U(i, jp, k) + U(ip, jp, k))) * (R(1.0) - fju)
              + R(0.5) * (U(i, n2, k) + U(ip, n2, k)) * fju;
    R um = R(M.c2cyi[j]) * R(0.25) * (R(f2fy[j]) * (U(i, jm, k) + U(ip, jm, k)) + R(f2fy[jm]) * (U(i, j, k) + U(ip, j, k))) * (R(1.0) - fjl)
              + R(0.5) * (U(i, 0, k) + U(ip, 0, k)) * fjl;
    R vg12 = R(M.f2fyi[j]) * (up - um);
    up = R(M.c2czi[kp]) * R(0.25) * (R(f2fz[kp]) * (U(i, j, k) + U(ip, j, k)) + R(f2fz[k]) * (U(i, j, kp) + U(ip, j, kp))) * (R(1.0) - fku)
       + R(0.5) * (U(i, j, n3) + U(ip, j, n3)) * fku;
    um = R(M.c2czi[k]) * R(0.25) * (R(f2fz[k]) * (U(i, j, km) + U(ip, j, km)) + R(f2fz[km]) * (U(i, j, k) + U(ip, j, k))) * (R(1.0) - fkl)
       + R(0.5) * (U(i, j, 0) + U(ip, j, 0)) * fkl;
    R vg13 = R(M.f2fzi[k]) * (up - um);
    R vp = R(M.c2cxi[ip]) * R(0.25) * (R(f2fx[ip]) * (V(i, j, k) + V(i, jp, k)) + R(f2fx[i]) * (V(ip, j, k) + V(ip, jp, k))) * (R(1.0) - fiu)
              + R(0.5) * (V(n1, j, k) + V(n1, jp, k)) * fiu;
    R vm = R(M.c2cxi[i]) * R(0.25) * (R(f2fx[i]) * (V(im, j, k) + V(im, jp, k)) + R(f2fx[im]) * (V(i, j, k) + V(i, jp, k))) * (R(1.0) - fil)
              + R(0.5) * (V(0, j, k) + V(0, jp, k)) * fil;
    R vg21 = R(M.f2fxi[i]) * (vp - vm);
    R vg22 = R(M.f2fyi[j]) * (V(i, jp, k) - V(i, j, k));
    vp = R(M.c2czi[kp]) * R(0.25) * (R(f2fz[kp]) * (V(i, j, k) + V(i, jp, k)) + R(f2fz[k]) * (V(i, j, kp) + V(i, jp, kp))) * (R(1.0) - fku)
       + R(0.5) * (V(i, j, n3) + V(i, jp, n3)) * fku;
    vm = R(M.c2czi[k]) * R(0.25) * (R(f2fz[k]) * (V(i, j, km) + V(i, jp, km)) + R(f2fz[km]) * (V(i, j, k) + V(i, jp, k))) * (R(1.0) - fkl)
       + R(0.5) * (V(i, j, 0) + V(i, jp, 0)) * fkl;
    R vg23 = R(M.f2fzi[k]) * (vp - vm);
    R wp = R(M.c2cxi[ip]) * R(0.25) * (R(f2fx[ip]) * (W(i, j, k) + W(i, j, kp)) + R(f2fx[i]) * (W(ip, j, k) + W(ip, j, kp))) * (R(1.0) - fiu)
              + R(0.5) * (W(n1, j, k) + W(n1, j, kp)) * fiu;
    R wm = R(M.c2cxi[i]) * R(0.25) * (R(f2fx[i]) * (W(im, j, k) + W(im, j, kp)) + R(f2fx[im]) * (W(i, j, k) + W(i, j, kp))) * (R(1.0) - fil)
              + R(0.5) * (W(0, j, k) + W(0, j, kp)) * fil;
    R vg31 = R(M.f2fxi[i]) * (wp - wm);
    wp = R(M.c2cyi[jp]) * R(0.25) * (R(f2fy[jp]) * (W(i, j, k) + W(i, j, kp)) + R(f2fy[j]) * (W(i, jp, k) + W(i, jp, kp))) * (R(1.0) - fju)
       + R(0.5) * (W(i, n2, k) + W(i, n2, kp)) * fju;
    wm = R(M.c2cyi[j]) * R(0.25) * (R(f2fy[j]) * (W(i, jm, k) + W(i, jm, kp)) + R(f2fy[jm]) * (W(i, j, k) + W(i, j, kp))) * (R(1.0) - fjl)
       + R(0.5) * (W(i, 0, k) + W(i, 0, kp)) * fjl;
    R vg32 = R(M.f2fyi[j]) * (wp - wm);
    R vg33 = R(M.f2fzi[k]) * (W(i, j, kp) - W(i, j, k));
#undef U
#undef V
#undef W
    a[0] = vg11; a[1] = vg21; a[2] = vg31;
    a[3] = vg12; a[4] = vg22; a[5] = vg32;
    a[6] = vg13; a[7] = vg23; a[8] = vg33;
    sr[0] = vg11; sr[1] = R(0.5) * (vg12 + vg21); sr[2] = R(0.5) * (vg13 + vg31);
    sr[3] = vg22; sr[4] = R(0.5) * (vg23 + vg32); sr[5] = vg33;
}

// temgrad, sgs.f90:1480-1525
template <class R>
__device__ void temgrad(const KP &p, int i, int j, int k, R a[3]) {
    const Mir<R> &M = mir<R>(p);
    const DGrid &g = p.g;
    const R *t = M.t;
    int kp = g.kpv[k], km = g.kmv[k], jp = g.jpv[j], jm = g.jmv[j], ip = g.ipv[i], im = g.imv[i];
    R fiu = M.fixiu[i], fil = M.fixil[i], fju = M.fixju[j], fjl = M.fixjl[j];
    R fku = M.fixku[k], fkl = M.fixkl[k];
    R tc = R(t[g.ix(i, j, k)]);
    R tip = R(t[g.ix(ip, j, k)]), tim = R(t[g.ix(im, j, k)]);
    R tp = R(0.5) * (R(M.f2fx[i]) * tip + R(M.f2fx[ip]) * tc) * R(M.c2cxi[ip]) * (R(1.0) - fiu) + tip * fiu;
    R tm = R(0.5) * (R(M.f2fx[im]) * tc + R(M.f2fx[i]) * tim) * R(M.c2cxi[i]) * (R(1.0) - fil) + tim * fil;
    a[0] = R(M.f2fxi[i]) * (tp - tm);
    R tjp = R(t[g.ix(i, jp, k)]), tjm = R(t[g.ix(i, jm, k)]);
    tp = R(0.5) * (R(M.f2fy[j]) * tjp + R(M.f2fy[jp]) * tc) * R(M.c2cyi[jp]) * (R(1.0) - fju) + tjp * fju;
    tm = R(0.5) * (R(M.f2fy[jm]) * tc + R(M.f2fy[j]) * tjm) * R(M.c2cyi[j]) * (R(1.0) - fjl) + tjm * fjl;
    a[1] = R(M.f2fyi[j]) * (tp - tm);
    R tkp = R(t[g.ix(i, j, kp)]), tkm = R(t[g.ix(i, j, km)]);
    tp = R(0.5) * (R(M.f2fz[k]) * tkp + R(M.f2fz[kp]) * tc) * R(M.c2czi[kp]) * (R(1.0) - fku) + tkp * fku;
    tm = R(0.5) * (R(M.f2fz[km]) * tc + R(M.f2fz[k]) * tkm) * R(M.c2czi[k]) * (R(1.0) - fkl) + tkm * fkl;
    a[2] = R(M.f2fzi[k]) * (tp - tm);
}

template <class R>
__device__ __forceinline__ void vreman(const R alp[9], R sdx2, R sdy2, R sdz2, R &aaa, R &bbb) {
    R b1 = sdx2 * R(alp[0]) * R(alp[0]) + sdy2 * R(alp[3]) * R(alp[3]) + sdz2 * R(alp[6]) * R(alp[6]);
    R b2 = sdx2 * R(alp[0]) * R(alp[1]) + sdy2 * R(alp[3]) * R(alp[4]) + sdz2 * R(alp[6]) * R(alp[7]);
    R b3 = sdx2 * R(alp[0]) * R(alp[2]) + sdy2 * R(alp[3]) * R(alp[5]) + sdz2 * R(alp[6]) * R(alp[8]);
    R b4 = sdx2 * R(alp[1]) * R(alp[1]) + sdy2 * R(alp[4]) * R(alp[4]) + sdz2 * R(alp[7]) * R(alp[7]);
    R b5 = sdx2 * R(alp[1]) * R(alp[2]) + sdy2 * R(alp[4]) * R(alp[5]) + sdz2 * R(alp[7]) * R(alp[8]);
    R b6 = sdx2 * R(alp[2]) * R(alp[2]) + sdy2 * R(alp[5]) * R(alp[5]) + sdz2 * R(alp[8]) * R(alp[8]);
    R a = R(0.0);
#pragma unroll
    for (int q = 0; q < 9; q++) a += R(alp[q]) * R(alp[q]);
    R b = b1 * b4 + b4 * b6 + b6 * b1 - b2 * b2 - b3 * b3 - b5 * b5;
    if (b < R(1.0e-16)) b = R(1.0e-16);
    aaa = a;
    bbb = b;
}

// Test-filter width at a cell: the sum of the three test-filter cell widths
// used in the second Vreman / eddy-diffusivity evaluation (sgs.f90:528-533).
template <class R, class T>
__device__ __forceinline__ R tf_width(const T *f2f, const int *fl, const int *fu, int i) {
    return R(0.5) * R(f2f[i - 1]) * (R(1.0) - R(fu[i])) + R(f2f[i]) + R(0.5) * R(f2f[i + 1]) * (R(1.0) - R(fl[i]));
}

#define GRID_LOOP(b)                                                                                   \
    for (long long tt = (long long)blockIdx.x * blockDim.x + threadIdx.x, nn_ = (b).count(); tt < nn_; \
         tt += (long long)gridDim.x * blockDim.x)

// SGS scratch arrays (scr[3..32]) hold R values: float in the mixed form,
// where they take half of each nt-double buffer.
template <class R>
__device__ __forceinline__ R *scr(const KP &p, int s) { return reinterpret_cast<R *>(p.f.scr[s]); }

// pass 1 of sgs_dvmg (:434-491) and the constant model sgs_cvm
template <class R>
__global__ void __launch_bounds__(kThreads) k_vreman1(KP p, Box b, int dynamic) {
    const Mir<R> &M = mir<R>(p);
    const DGrid &g = p.g;
    GRID_LOOP(b) {      // mm[0..5] in scr[3..8], alp[0..8] in scr[9..17]
        int i, j, k;
        b.at(tt, i, j, k);
        R alp[9], str[6], aaa, bbb;
        velgrad<R>(p, i, j, k, alp, str);
        const R fx = R(M.f2fx[i]), fy = R(M.f2fy[j]), fz = R(M.f2fz[k]);
        vreman<R>(alp, fx * fx, fy * fy, fz * fz, aaa, bbb);
        long long q = g.ix(i, j, k);
        if (!dynamic) {
            p.f.nusgs[q] = (aaa == R(0.0)) ? R(0.0) : R(p.c.csgsts) * sqrt(bbb / aaa);
            continue;
        }
        R nu = (aaa == R(0.0)) ? R(0.0) : sqrt(bbb / aaa);
        p.f.nusgs[q] = nu;
#pragma unroll
        for (int m = 0; m < 6; m++) scr<R>(p, 3 + m)[q] = nu * str[m];
#pragma unroll
        for (int m = 0; m < 9; m++) scr<R>(p, 9 + m)[q] = alp[m];
    }
}

// Batched test filter: dst[a] = filter(src[a]) on the interior, a < na
// (arrays of R).
struct FiltBatch {
    const void *src[16];
    void *dst[16];
    int na;
};

// One cell's x filter (sgs.f90:650-733) of the rows qm, q0, qp of every array
// of the batch is formed from the same offsets and weights: the cell's index
// decoding, periodic wrap and weights are computed once for all arrays.
struct FiltX {
    int im, ip;              // x neighbours (wrapped); == i when x is not filtered here
    bool filt;
};

template <class R>
__global__ void __launch_bounds__(kThreads) k_filter(KP p, Box b, FiltBatch F) {
    const DGrid &g = p.g;
    const int xf = (p.c.filter == 1 || p.c.filter == 3) ? 1 : 0;
    const int zf = (p.c.filter == 2 || p.c.filter == 3) ? 1 : 0;
    const long long n = b.count();
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        b.at(t, i, j, k);
        // x: interior points use i-1, i, i+1; x-periodic ends wrap (with n1m = 1
        // the value is unfiltered); other ends are unfiltered
        FiltX X{i, i, false};
        if (xf) {
            if (i >= 2 && i <= g.n1m - 1) X = FiltX{i - 1, i + 1, true};
            else if (p.c.xprdic == 1 && g.n1m > 1) X = FiltX{i == 1 ? g.n1m : g.n1m - 1, i == 1 ? 2 : 1, true};
        }
        const R *cfx = mir<R>(p).cfx1 + 3 * i;
        const R c0 = X.filt ? R(cfx[0]) : R(0.0), c1 = X.filt ? R(cfx[1]) : R(0.0), c2 = X.filt ? R(cfx[2]) : R(0.0);
        // z-periodic ends use the wrapped neighbours; with n3m = 1 the weights
        // are zero (sgsfilterinit skips them), so the filtered value is 0 as
        // in test_filter (sgs.f90:735-764)
        const bool zin = zf && ((k >= 2 && k <= g.n3m - 1) || p.c.zprdic == 1);
        const int km = k == 1 ? g.n3m : k - 1, kp = k == g.n3m ? 1 : k + 1;
        const R *cfz = mir<R>(p).cfz1 + 3 * k;
        const R z0 = zin ? R(cfz[0]) : R(0.0), z1 = zin ? R(cfz[1]) : R(0.0), z2 = zin ? R(cfz[2]) : R(0.0);
        const long long r0 = g.ix(0, j, k), rm = g.ix(0, j, km), rp = g.ix(0, j, kp);
        // sources and destinations are distinct arrays: two arrays' loads
        // can be in flight at once
#pragma unroll 2
        for (int a = 0; a < F.na; a++) {
            const R *__restrict__ s = static_cast<const R *>(F.src[a]);
            R *__restrict__ d = static_cast<R *>(F.dst[a]);
            R out;
            if (!zin) {
                out = X.filt ? c0 * s[r0 + X.im] + c1 * s[r0 + i] + c2 * s[r0 + X.ip] : s[r0 + i];
            } else if (X.filt) {
                const R xm = c0 * s[rm + X.im] + c1 * s[rm + i] + c2 * s[rm + X.ip];
                const R x0 = c0 * s[r0 + X.im] + c1 * s[r0 + i] + c2 * s[r0 + X.ip];
                const R xp = c0 * s[rp + X.im] + c1 * s[rp + i] + c2 * s[rp + X.ip];
                out = z0 * xm + z1 * x0 + z2 * xp;
            } else {
                out = z0 * s[rm + i] + z1 * s[r0 + i] + z2 * s[rp + i];
            }
            d[r0 + i] = out;
        }
    }
}

static bool mixed(const lesgpu_case *c) { return c->cfg.precision == LESGPU_PREC_MIXED; }

static void filter_batch(lesgpu_case *c, FiltBatch &F) {
    const DGrid &g = c->kp.g;
    Box b{1, 1, 1, g.n1m, g.n2m, g.n3m};
    inst_begin(c, LESGPU_K_SGS);
    if (mixed(c)) k_filter<float><<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b, F);
    else k_filter<double><<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b, F);
    inst_end(c, LESGPU_K_SGS);
}

// pass 2 of sgs_dvmg (:504-580): filtered gradients -> test-level Vreman
// viscosity, M_ij update, resolved velocities and their products.
// filtered mm[0..5] in scr[18..23] (updated in place), filtered alp[0..8] in
// scr[24..32]; out: uui[0..2], llij[0..5] in scr[3..11]
template <class R>
__global__ void __launch_bounds__(kThreads) k_vreman2(KP p, Box b) {
    const Mir<R> &M = mir<R>(p);
    const DGrid &g = p.g;
    GRID_LOOP(b) {
        int i, j, k;
        b.at(tt, i, j, k);
        long long q = g.ix(i, j, k);
        R alp[9], str[6], aaa, bbb;
#pragma unroll
        for (int m = 0; m < 9; m++) alp[m] = scr<R>(p, 24 + m)[q];
        str[0] = alp[0]; str[1] = R(0.5) * (alp[3] + alp[1]); str[2] = R(0.5) * (alp[6] + alp[2]);
        str[3] = alp[4]; str[4] = R(0.5) * (alp[7] + alp[5]); str[5] = alp[8];
        R sx = tf_width<R>(M.f2fx, g.fixil, g.fixiu, i);
        R sy = tf_width<R>(M.f2fy, g.fixjl, g.fixju, j);
        R sz = tf_width<R>(M.f2fz, g.fixkl, g.fixku, k);
        vreman<R>(alp, sx * sx, sy * sy, sz * sz, aaa, bbb);
        R ami = (aaa == R(0.0)) ? R(0.0) : sqrt(bbb / aaa);
#pragma unroll
        for (int m = 0; m < 6; m++) scr<R>(p, 18 + m)[q] = ami * str[m] - scr<R>(p, 18 + m)[q];
        R u1 = R(0.5) * (R(M.u[q]) + R(M.u[q + 1]));
        R u2 = R(0.5) * (R(M.v[q]) + R(M.v[q + g.sx]));
        R u3 = R(0.5) * (R(M.w[q]) + R(M.w[q + g.sxy]));
        scr<R>(p, 3)[q] = u1; scr<R>(p, 4)[q] = u2; scr<R>(p, 5)[q] = u3;
        scr<R>(p, 6)[q] = u1 * u1; scr<R>(p, 7)[q] = u1 * u2; scr<R>(p, 8)[q] = u1 * u3;
        scr<R>(p, 9)[q] = u2 * u2; scr<R>(p, 10)[q] = u2 * u3; scr<R>(p, 11)[q] = u3 * u3;
    }
}

// global least-squares sums (:593-618): M_ij in scr[18..23], filtered uui in
// scr[24..26], filtered llij in scr[27..32]
template <class R>
struct LmMmTerm {
    __device__ void operator()(const KP &p, int i, int j, int k, double *w) const {
        const Mir<R> &M = mir<R>(p);
        const DGrid &g = p.g;
        long long q = g.ix(i, j, k);
        R vol = R(M.f2fx[i]) * R(M.f2fy[j]) * R(M.f2fz[k]);
        R u1 = scr<R>(p, 24)[q], u2 = scr<R>(p, 25)[q], u3 = scr<R>(p, 26)[q];
        R L0 = scr<R>(p, 27)[q] - u1 * u1, L1 = scr<R>(p, 28)[q] - u1 * u2, L2 = scr<R>(p, 29)[q] - u1 * u3;
        R L3 = scr<R>(p, 30)[q] - u2 * u2, L4 = scr<R>(p, 31)[q] - u2 * u3, L5 = scr<R>(p, 32)[q] - u3 * u3;
        R M0 = scr<R>(p, 18)[q], M1 = scr<R>(p, 19)[q], M2 = scr<R>(p, 20)[q];
        R M3 = scr<R>(p, 21)[q], M4 = scr<R>(p, 22)[q], M5 = scr<R>(p, 23)[q];
        R nw = R(p.f.nwall[q]);
        w[0] = (R(2.0) * L1 * M1 + L0 * M0 + R(2.0) * L2 * M2 + L3 * M3 + R(2.0) * L4 * M4 + L5 * M5) * nw * vol;
        w[1] = (R(2.0) * M1 * M1 + M0 * M0 + R(2.0) * M2 * M2 + M3 * M3 + R(2.0) * M4 * M4 + M5 * M5) * nw * vol;
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
// Each edge value is c2c?i c2c?i / 4 times a bilinear combination of the four
// surrounding cell values (sgs.f90:1002-1040); the four products of the 1-D
// weights are formed once per edge line (ew1..3), so a value costs four FP64
// operations instead of nine -- the pass is FP64-pipe bound on GB300.
__global__ void __launch_bounds__(kThreads) k_edge_interp(KP p, Box b, const double *f, double *f1, double *f2,
                                                           double *f3, int ib, int jb, int kb) {
    const DGrid &g = p.g;
    const long long n2 = g.n2 + 1, n3 = g.n3 + 1;
    GRID_LOOP(b) {
        int i, j, k;
        b.at(tt, i, j, k);
        long long q = g.ix(i, j, k);
        double c = f[q], cim = f[q - 1], cjm = f[q - g.sx], ckm = f[q - g.sxy];
        if (k >= kb && j >= jb) {
            const double *w = p.f.ew1 + 4 * (j + n2 * k);
            f1[q] = w[0] * c + w[1] * ckm + w[2] * cjm + w[3] * f[q - g.sx - g.sxy];
        }
        if (k >= kb && i >= ib) {
            const double *w = p.f.ew2 + 4 * (k + n3 * i);
            f2[q] = w[0] * c + w[1] * cim + w[2] * ckm + w[3] * f[q - 1 - g.sxy];
        }
        if (j >= jb && i >= ib) {
            const double *w = p.f.ew3 + 4 * (i + (long long)(g.n1 + 1) * j);
            f3[q] = w[0] * c + w[1] * cjm + w[2] * cim + w[3] * f[q - 1 - g.sx];
        }
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
        if (mixed(c)) k_vreman1<float><<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b, 1);
        else k_vreman1<double><<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b, 1);
        FiltBatch F{};
        F.na = 15;
        for (int m = 0; m < 6; m++) { F.src[m] = f.scr[3 + m]; F.dst[m] = f.scr[18 + m]; }
        for (int m = 0; m < 9; m++) { F.src[6 + m] = f.scr[9 + m]; F.dst[6 + m] = f.scr[24 + m]; }
        filter_batch(c, F);
        if (mixed(c)) k_vreman2<float><<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b);
        else k_vreman2<double><<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b);
        FiltBatch G{};
        G.na = 9;
        for (int m = 0; m < 9; m++) { G.src[m] = f.scr[3 + m]; G.dst[m] = f.scr[24 + m]; }
        filter_batch(c, G);
        if (mixed(c)) reduce<2, false>(c, b, LmMmTerm<float>{}, CsgstsFinal{});
        else reduce<2, false>(c, b, LmMmTerm<double>{}, CsgstsFinal{});
        k_scale<<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b, f.nusgs, 0);
    } else {
        if (mixed(c)) k_vreman1<float><<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b, 0);
        else k_vreman1<double><<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b, 0);
    }
}

void launch_sgs_post(lesgpu_case *c) {
    zero_in_body(c, c->kp.f.nusgs, 0);
    edge_interpol(c, c->kp.f.nusgs, c->kp.f.nusgs1, 0);
}

// ------------------------------------------------------------ thermal EDM
// pass 1 of sgs_edm: mm[0..2] scr[3..5]; s[0..5] scr[6..11]; tgrad[0..2] scr[12..14]
template <class R>
__global__ void __launch_bounds__(kThreads) k_edm1(KP p, Box b, int dynamic) {
    const Mir<R> &M = mir<R>(p);
    const DGrid &g = p.g;
    GRID_LOOP(b) {
        int i, j, k;
        b.at(tt, i, j, k);
        R d[9], s[6], alp[3];
        velgrad<R>(p, i, j, k, d, s);
        R del = pow(R(M.f2fx[i]) * R(M.f2fy[j]) * R(M.f2fz[k]), R(1.0) / R(3.0));
        R sss = s[0] * s[0] + R(2.0) * s[1] * s[1] + R(2.0) * s[2] * s[2] + s[3] * s[3] + R(2.0) * s[4] * s[4] + s[5] * s[5];
        if (sss < R(1.0e-16)) sss = R(1.0e-16);
        long long q = g.ix(i, j, k);
        if (!dynamic) {
            p.f.alsgs[q] = R(p.c.csgshf) * (del * del) * sqrt(R(2.0) * sss);
            continue;
        }
        temgrad<R>(p, i, j, k, alp);
        R al = (del * del) * sqrt(R(2.0) * sss);
        p.f.alsgs[q] = al;
#pragma unroll
        for (int m = 0; m < 3; m++) scr<R>(p, 3 + m)[q] = al * alp[m];
#pragma unroll
        for (int m = 0; m < 6; m++) scr<R>(p, 6 + m)[q] = s[m];
#pragma unroll
        for (int m = 0; m < 3; m++) scr<R>(p, 12 + m)[q] = alp[m];
    }
}

// pass 2: filtered mm[0..2] scr[18..20] (updated in place), filtered s[0..5]
// scr[21..26] and tgrad[0..2] scr[27..29]; out uui[0..2] scr[3..5], t scr[6],
// llij[0..2] scr[7..9]
template <class R>
__global__ void __launch_bounds__(kThreads) k_edm2(KP p, Box b) {
    const Mir<R> &M = mir<R>(p);
    const DGrid &g = p.g;
    GRID_LOOP(b) {
        int i, j, k;
        b.at(tt, i, j, k);
        long long q = g.ix(i, j, k);
        R d1 = tf_width<R>(M.f2fx, g.fixil, g.fixiu, i);
        R d2 = tf_width<R>(M.f2fy, g.fixjl, g.fixju, j);
        R d3 = tf_width<R>(M.f2fz, g.fixkl, g.fixku, k);
        R del = pow(d1 * d2 * d3, R(1.0) / R(3.0));
        R s0 = scr<R>(p, 21)[q], s1 = scr<R>(p, 22)[q], s2 = scr<R>(p, 23)[q];
        R s3 = scr<R>(p, 24)[q], s4 = scr<R>(p, 25)[q], s5 = scr<R>(p, 26)[q];
        R sss = s0 * s0 + R(2.0) * s1 * s1 + R(2.0) * s2 * s2 + s3 * s3 + R(2.0) * s4 * s4 + s5 * s5;
        if (sss < R(1.0e-16)) sss = R(1.0e-16);
        R ami = (del * del) * sqrt(R(2.0) * sss);
#pragma unroll
        for (int m = 0; m < 3; m++) scr<R>(p, 18 + m)[q] = ami * scr<R>(p, 27 + m)[q] - scr<R>(p, 18 + m)[q];
        R u1 = R(0.5) * (R(M.u[q]) + R(M.u[q + 1]));
        R u2 = R(0.5) * (R(M.v[q]) + R(M.v[q + g.sx]));
        R u3 = R(0.5) * (R(M.w[q]) + R(M.w[q + g.sxy]));
        R tq = R(M.t[q]);
        scr<R>(p, 3)[q] = u1; scr<R>(p, 4)[q] = u2; scr<R>(p, 5)[q] = u3;
        scr<R>(p, 6)[q] = tq;
        scr<R>(p, 7)[q] = u1 * tq; scr<R>(p, 8)[q] = u2 * tq; scr<R>(p, 9)[q] = u3 * tq;
    }
}

// M_j in scr[18..20]; filtered uui [24..26], t [27], llij [28..30]
template <class R>
struct LmMmTTerm {
    __device__ void operator()(const KP &p, int i, int j, int k, double *w) const {
        const Mir<R> &M = mir<R>(p);
        const DGrid &g = p.g;
        long long q = g.ix(i, j, k);
        R vol = R(M.f2fx[i]) * R(M.f2fy[j]) * R(M.f2fz[k]);
        R tf = scr<R>(p, 27)[q];
        R L0 = scr<R>(p, 28)[q] - scr<R>(p, 24)[q] * tf;
        R L1 = scr<R>(p, 29)[q] - scr<R>(p, 25)[q] * tf;
        R L2 = scr<R>(p, 30)[q] - scr<R>(p, 26)[q] * tf;
        R M0 = scr<R>(p, 18)[q], M1 = scr<R>(p, 19)[q], M2 = scr<R>(p, 20)[q];
        R nw = R(p.f.nwall[q]);
        w[0] = (L0 * M0 + L1 * M1 + L2 * M2) * nw * vol;
        w[1] = (M0 * M0 + M1 * M1 + M2 * M2) * nw * vol;
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
        if (mixed(c)) k_edm1<float><<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b, 1);
        else k_edm1<double><<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b, 1);
        FiltBatch F{};
        F.na = 12;
        for (int m = 0; m < 3; m++) { F.src[m] = f.scr[3 + m]; F.dst[m] = f.scr[18 + m]; }
        for (int m = 0; m < 9; m++) { F.src[3 + m] = f.scr[6 + m]; F.dst[3 + m] = f.scr[21 + m]; }
        filter_batch(c, F);
        if (mixed(c)) k_edm2<float><<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b);
        else k_edm2<double><<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b);
        FiltBatch G{};
        G.na = 7;
        for (int m = 0; m < 7; m++) { G.src[m] = f.scr[3 + m]; G.dst[m] = f.scr[24 + m]; }
        filter_batch(c, G);
        if (mixed(c)) reduce<2, false>(c, b, LmMmTTerm<float>{}, CsgshfFinal{});
        else reduce<2, false>(c, b, LmMmTTerm<double>{}, CsgshfFinal{});
        k_scale<<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b, f.alsgs, 1);
    } else {
        if (mixed(c)) k_edm1<float><<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b, 0);
        else k_edm1<double><<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b, 0);
    }
}

void launch_sgs_t_post(lesgpu_case *c) {
    zero_in_body(c, c->kp.f.alsgs, 1);
    edge_interpol(c, c->kp.f.alsgs, c->kp.f.alsgs1, 1);
}

}  // namespace lg
