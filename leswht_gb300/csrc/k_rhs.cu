// Explicit right-hand sides: rhs (slv_mmtm.f90:315-567) fused with the SGS
// cross terms rhssgs (sgs.f90:1136-1200), divgs (slv_cont.f90:2-208) and
// rhs_t (slv_engy.f90:29-198).
//
// One thread per cell computes all three momentum components, so u, v, w, p
// and the eddy viscosities around a cell are read once per cell from L1/L2
// instead of once per component; the SGS cross term never goes to memory.
// Each expression keeps the reference's operation order.
#include "lesgpu_internal.cuh"

namespace lg {

__global__ void __launch_bounds__(kThreads) k_rhs(KP p, Box b, double gam, double ro) {
    const DGrid &g = p.g;
    const DCfg &c = p.c;
    const double *u = p.f.u, *v = p.f.v, *w = p.f.w, *pp = p.f.p, *t = p.f.t;
    const double *nu = p.f.nusgs, *nu1 = p.f.nusgs1[0], *nu2 = p.f.nusgs1[1], *nu3 = p.f.nusgs1[2];
    const double dt = p.S->dt, alpha = p.S->alpha, pmi0 = p.S->pmi[0];
    const double ichfac = c.ich != 0 ? 1.0 : 0.0;
    const double rei = 1.0 / c.re;
    const long long sx = g.sx, sxy = g.sxy;
    long long n = b.count();
    for (long long tt = (long long)blockIdx.x * blockDim.x + threadIdx.x; tt < n; tt += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        b.at(tt, i, j, k);
        long long q = g.ix(i, j, k);
        const double fju = fixd(g.fixju[j]), fjl = fixd(g.fixjl[j]), fku = fixd(g.fixku[k]), fkl = fixd(g.fixkl[k]);
        const double fiu = fixd(g.fixiu[i]), fil = fixd(g.fixil[i]);
        const double f2fxm = g.f2fx[i - 1], f2fx0 = g.f2fx[i], f2fxp = g.f2fx[i + 1];
        const double f2fym = g.f2fy[j - 1], f2fy0 = g.f2fy[j], f2fyp = g.f2fy[j + 1];
        const double f2fzm = g.f2fz[k - 1], f2fz0 = g.f2fz[k], f2fzp = g.f2fz[k + 1];

        // ---------------- u momentum
        if (i >= g.i_bgpx) {
            double uq = u[q];
            double un = 0.5 * (f2fyp * uq + f2fy0 * u[q + sx]) * g.c2cyi[j + 1] * (1.0 - fju) + u[g.ix(i, g.n2, k)] * fju;
            double us = 0.5 * (f2fy0 * u[q - sx] + f2fym * uq) * g.c2cyi[j] * (1.0 - fjl) + u[g.ix(i, 0, k)] * fjl;
            double uc = 0.5 * (f2fzp * uq + f2fz0 * u[q + sxy]) * g.c2czi[k + 1] * (1.0 - fku) + u[g.ix(i, j, g.n3)] * fku;
            double uf = 0.5 * (f2fz0 * u[q - sxy] + f2fzm * uq) * g.c2czi[k] * (1.0 - fkl) + u[g.ix(i, j, 0)] * fkl;
            double vnx = 0.5 * (f2fxm * v[q + sx] + f2fx0 * v[q + sx - 1]) * g.c2cxi[i];
            double vsx = 0.5 * (f2fxm * v[q] + f2fx0 * v[q - 1]) * g.c2cxi[i];
            double wcx = 0.5 * (f2fxm * w[q + sxy] + f2fx0 * w[q + sxy - 1]) * g.c2cxi[i];
            double wfx = 0.5 * (f2fxm * w[q] + f2fx0 * w[q - 1]) * g.c2cxi[i];
            double anxe = 0.5 * (u[q + 1] + uq);
            double anxw = 0.5 * (uq + u[q - 1]);
            double anxx = (anxe * anxe - anxw * anxw) * g.c2cxi[i];
            double anx1 = (un * vnx - us * vsx) * g.f2fyi[j];
            double anx2 = (uc * wcx - uf * wfx) * g.f2fzi[k];
            double rk3x = -anxx - anx1 - anx2;
            double alx1 = (u[q + 1] - uq) * g.f2fxi[i];
            double alx2 = (uq - u[q - 1]) * g.f2fxi[i - 1];
            double alx3 = (u[q + sx] - uq) * g.c2cyi[j + 1];
            double alx4 = (uq - u[q - sx]) * g.c2cyi[j];
            double alx5 = (u[q + sxy] - uq) * g.c2czi[k + 1];
            double alx6 = (uq - u[q - sxy]) * g.c2czi[k];
            double alx = rei * ((alx1 - alx2) * g.c2cxi[i] + (alx3 - alx4) * g.f2fyi[j] + (alx5 - alx6) * g.f2fzi[k]);
            if (c.iles == 1) {
                // rhssgs u-part (sgs.f90:1146-1156)
                double a = g.f2fyi[j] * g.c2cxi[i] * (nu3[q + sx] * (v[q + sx] - v[q + sx - 1]) - nu3[q] * (v[q] - v[q - 1]));
                double bb = g.f2fzi[k] * g.c2cxi[i] * (nu2[q + sxy] * (w[q + sxy] - w[q + sxy - 1]) - nu2[q] * (w[q] - w[q - 1]));
                double tx = (nu[q] * alx1 - nu[q - 1] * alx2) * g.c2cxi[i];
                double ty = (nu3[q + sx] * alx3 - nu3[q] * alx4) * g.f2fyi[j];
                double tz = (nu2[q + sxy] * alx5 - nu2[q] * alx6) * g.f2fzi[k];
                alx = alx + (2.0 * tx + ty + tz);
                rk3x = rk3x + (a + bb);
            }
            if (c.ihtrans == 1 && c.grdir == 1) rk3x = rk3x + c.gr / (c.re * c.re) * t[q];
            p.f.rhs1[0][q] = dt * (gam * rk3x + ro * p.f.rk3o[0][q] + 2.0 * alpha * alx
                                   - 2.0 * alpha * (pp[q] - pp[q - 1]) * g.c2cxi[i]
                                   - 2.0 * alpha * pmi0 * ichfac);
            p.f.rk3oo[0][q] = p.f.rk3o[0][q];
            p.f.rk3o[0][q] = rk3x;
        }
        // ---------------- v momentum
        if (j >= g.j_bgpy) {
            double vq = v[q];
            double ve = (0.5 * (f2fxp * vq + f2fx0 * v[q + 1]) * g.c2cxi[i + 1]) * (1.0 - fiu) + v[g.ix(g.n1, j, k)] * fiu;
            double vw = (0.5 * (f2fx0 * v[q - 1] + f2fxm * vq) * g.c2cxi[i]) * (1.0 - fil) + v[g.ix(0, j, k)] * fil;
            double vc = (0.5 * (f2fzp * vq + f2fz0 * v[q + sxy]) * g.c2czi[k + 1]) * (1.0 - fku) + v[g.ix(i, j, g.n3)] * fku;
            double vf = (0.5 * (f2fz0 * v[q - sxy] + f2fzm * vq) * g.c2czi[k]) * (1.0 - fkl) + v[g.ix(i, j, 0)] * fkl;
            double uey = 0.5 * (f2fym * u[q + 1] + f2fy0 * u[q + 1 - sx]) * g.c2cyi[j];
            double uwy = 0.5 * (f2fym * u[q] + f2fy0 * u[q - sx]) * g.c2cyi[j];
            double wcy = 0.5 * (f2fym * w[q + sxy] + f2fy0 * w[q + sxy - sx]) * g.c2cyi[j];
            double wfy = 0.5 * (f2fym * w[q] + f2fy0 * w[q - sx]) * g.c2cyi[j];
            double anyn = 0.5 * (v[q + sx] + vq);
            double anys = 0.5 * (vq + v[q - sx]);
            double anyy = g.c2cyi[j] * (anyn * anyn - anys * anys);
            double any1 = (uey * ve - uwy * vw) * g.f2fxi[i];
            double any2 = (vc * wcy - vf * wfy) * g.f2fzi[k];
            double rk3y = -anyy - any1 - any2;
            double aly1 = (v[q + 1] - vq) * g.c2cxi[i + 1];
            double aly2 = (vq - v[q - 1]) * g.c2cxi[i];
            double aly3 = (v[q + sx] - vq) * g.f2fyi[j];
            double aly4 = (vq - v[q - sx]) * g.f2fyi[j - 1];
            double aly5 = (v[q + sxy] - vq) * g.c2czi[k + 1];
            double aly6 = (vq - v[q - sxy]) * g.c2czi[k];
            double aly = rei * ((aly1 - aly2) * g.f2fxi[i] + (aly3 - aly4) * g.c2cyi[j] + (aly5 - aly6) * g.f2fzi[k]);
            if (c.iles == 1) {
                double a = g.f2fxi[i] * g.c2cyi[j] * (nu3[q + 1] * (u[q + 1] - u[q + 1 - sx]) - nu3[q] * (u[q] - u[q - sx]));
                double bb = g.f2fzi[k] * g.c2cyi[j] * (nu1[q + sxy] * (w[q + sxy] - w[q + sxy - sx]) - nu1[q] * (w[q] - w[q - sx]));
                double tx = (nu3[q + 1] * aly1 - nu3[q] * aly2) * g.f2fxi[i];
                double ty = (nu[q] * aly3 - nu[q - sx] * aly4) * g.c2cyi[j];
                double tz = (nu1[q + sxy] * aly5 - nu1[q] * aly6) * g.f2fzi[k];
                aly = aly + (tx + 2.0 * ty + tz);
                rk3y = rk3y + (a + bb);
            }
            if (c.ihtrans == 1 && c.grdir == 2) rk3y = rk3y + c.gr / (c.re * c.re) * t[q];
            p.f.rhs1[1][q] = dt * (gam * rk3y + ro * p.f.rk3o[1][q] + 2.0 * alpha * aly
                                   - 2.0 * alpha * (pp[q] - pp[q - sx]) * g.c2cyi[j]);
            p.f.rk3oo[1][q] = p.f.rk3o[1][q];
            p.f.rk3o[1][q] = rk3y;
        }
        // ---------------- w momentum
        if (k >= g.k_bgpz && g.n3m != 1) {
            double wq = w[q];
            double we = 0.5 * (f2fxp * wq + f2fx0 * w[q + 1]) * g.c2cxi[i + 1] * (1.0 - fiu) + fiu * w[g.ix(g.n1, j, k)];
            double ww = 0.5 * (f2fx0 * w[q - 1] + f2fxm * wq) * g.c2cxi[i] * (1.0 - fil) + fil * w[g.ix(0, j, k)];
            double wn = (0.5 * (f2fyp * wq + f2fy0 * w[q + sx]) * g.c2cyi[j + 1]) * (1.0 - fju) + fju * w[g.ix(i, g.n2, k)];
            double ws = (0.5 * (f2fy0 * w[q - sx] + f2fym * wq) * g.c2cyi[j]) * (1.0 - fjl) + fjl * w[g.ix(i, 0, k)];
            double uez = 0.5 * (f2fzm * u[q + 1] + f2fz0 * u[q + 1 - sxy]) * g.c2czi[k];
            double uwz = 0.5 * (f2fzm * u[q] + f2fz0 * u[q - sxy]) * g.c2czi[k];
            double vnz = 0.5 * (f2fzm * v[q + sx] + f2fz0 * v[q + sx - sxy]) * g.c2czi[k];
            double vsz = 0.5 * (f2fzm * v[q] + f2fz0 * v[q - sxy]) * g.c2czi[k];
            double anzc = 0.5 * (w[q + sxy] + wq);
            double anzf = 0.5 * (wq + w[q - sxy]);
            double anzz = (anzc * anzc - anzf * anzf) * g.c2czi[k];
            double anz1 = (uez * we - uwz * ww) * g.f2fxi[i];
            double anz2 = (vnz * wn - vsz * ws) * g.f2fyi[j];
            double rk3z = -anzz - anz1 - anz2;
            double alz1 = (w[q + 1] - wq) * g.c2cxi[i + 1];
            double alz2 = (wq - w[q - 1]) * g.c2cxi[i];
            double alz3 = (w[q + sx] - wq) * g.c2cyi[j + 1];
            double alz4 = (wq - w[q - sx]) * g.c2cyi[j];
            double alz5 = (w[q + sxy] - wq) * g.f2fzi[k];
            double alz6 = (wq - w[q - sxy]) * g.f2fzi[k - 1];
            double alz = rei * ((alz1 - alz2) * g.f2fxi[i] + (alz3 - alz4) * g.f2fyi[j] + (alz5 - alz6) * g.c2czi[k]);
            if (c.iles == 1) {
                double a = g.f2fxi[i] * g.c2czi[k] * (nu2[q + 1] * (u[q + 1] - u[q + 1 - sxy]) - nu2[q] * (u[q] - u[q - sxy]));
                double bb = g.f2fyi[j] * g.c2czi[k] * (nu1[q + sx] * (v[q + sx] - v[q + sx - sxy]) - nu1[q] * (v[q] - v[q - sxy]));
                double tx = (nu2[q + 1] * alz1 - nu2[q] * alz2) * g.f2fxi[i];
                double ty = (nu1[q + sx] * alz3 - nu1[q] * alz4) * g.f2fyi[j];
                double tz = (nu[q] * alz5 - nu[q - sxy] * alz6) * g.c2czi[k];
                alz = alz + (tx + ty + 2.0 * tz);
                rk3z = rk3z + (a + bb);
            }
            if (c.ihtrans == 1 && c.grdir == 3) rk3z = rk3z + c.gr / (c.re * c.re) * t[q];
            p.f.rhs1[2][q] = dt * (gam * rk3z + ro * p.f.rk3o[2][q] + 2.0 * alpha * alz
                                   - 2.0 * alpha * (pp[q] - pp[q - sxy]) * g.c2czi[k]);
            p.f.rk3oo[2][q] = p.f.rk3o[2][q];
            p.f.rk3o[2][q] = rk3z;
        }
    }
}

void launch_rhs(lesgpu_case *c, int msub) {
    const double gam[4] = {0.0, 8.0 / 15.0, 5.0 / 12.0, 3.0 / 4.0};
    const double ro[4] = {0.0, 0.0, -17.0 / 60.0, -5.0 / 12.0};
    const DGrid &g = c->kp.g;
    Box b{1, 1, 1, g.n1m, g.n2m, g.n3m};
    inst_begin(c, LESGPU_K_RHS);
    k_rhs<<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b, gam[msub], ro[msub]);
    inst_end(c, LESGPU_K_RHS);
}

// ------------------------------------------------------------------- divgs
__global__ void __launch_bounds__(kThreads) k_divgs(KP p, Box b, int scale) {
    const DGrid &g = p.g;
    double dti = p.S->dtconsti;
    long long n = b.count();
    for (long long tt = (long long)blockIdx.x * blockDim.x + threadIdx.x; tt < n; tt += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        b.at(tt, i, j, k);
        long long q = g.ix(i, j, k);
        double d1 = (p.f.u[q + 1] - p.f.u[q]) * g.f2fxi[i];
        double d2 = (p.f.v[q + g.sx] - p.f.v[q]) * g.f2fyi[j];
        double d3 = (p.f.w[q + g.sxy] - p.f.w[q]) * g.f2fzi[k];
        double s = (d1 + d2 + d3);
        p.f.divgsum[q] = scale ? s * dti : s;
    }
}

__global__ void k_scale_div(KP p, Box b) {
    double dti = p.S->dtconsti;
    long long n = b.count();
    for (long long tt = (long long)blockIdx.x * blockDim.x + threadIdx.x; tt < n; tt += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        b.at(tt, i, j, k);
        long long q = p.g.ix(i, j, k);
        p.f.divgsum[q] = p.f.divgsum[q] * dti;
    }
}

void launch_divgs(lesgpu_case *c) {
    const DGrid &g = c->kp.g;
    Box b{1, 1, 1, g.n1m, g.n2m, g.n3m};
    bool ibm = c->kp.c.masson == 1 && c->kp.c.imovingon == 0 && c->kp.c.ibmon == 1;
    k_divgs<<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b, ibm ? 0 : 1);
    if (ibm) {
        cudaMemsetAsync(c->kp.f.qmass, 0, sizeof(double) * g.nt, c->stream);
        launch_divgs_ibm(c);       // slv_cont.f90:48-113
        k_scale_div<<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b);
    }
}

// ------------------------------------------------------------------- rhs_t
struct UbulkTTerm;   // defined in k_energy via reduce; see launch_rhs_t there

__global__ void __launch_bounds__(kThreads) k_rhs_t(KP p, Box b, double gam, double ro) {
    const DGrid &g = p.g;
    const DCfg &c = p.c;
    const double *t = p.f.t, *u = p.f.u, *v = p.f.v, *w = p.f.w;
    const double dt = p.S->dt, alpha = p.S->alpha, u_bulk = p.S->u_bulk_t;
    const double inv_repr = 1.0 / (c.re * c.pr);
    long long n = b.count();
    for (long long tt = (long long)blockIdx.x * blockDim.x + threadIdx.x; tt < n; tt += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        b.at(tt, i, j, k);
        long long q = g.ix(i, j, k);
        int kp = g.kpv[k], km = g.kmv[k], jp = g.jpv[j], jm = g.jmv[j], ip = g.ipv[i], im = g.imv[i];
        if (c.xprdic == 1 && c.idecomp == 0) {
            if (i == g.n1m) ip = g.n1;
            if (i == 1) im = 0;
        }
        const double fiu = fixd(g.fixiu[i]), fil = fixd(g.fixil[i]), fju = fixd(g.fixju[j]), fjl = fixd(g.fixjl[j]);
        const double fku = fixd(g.fixku[k]), fkl = fixd(g.fixkl[k]);
        double tq = t[q];
        long long qip = g.ix(ip, j, k), qim = g.ix(im, j, k), qjp = g.ix(i, jp, k), qjm = g.ix(i, jm, k);
        long long qkp = g.ix(i, j, kp), qkm = g.ix(i, j, km);
        double tip = t[qip], tim = t[qim], tjp = t[qjp], tjm = t[qjm], tkp = t[qkp], tkm = t[qkm];
        double te = 0.5 * (g.f2fx[i] * tip + g.f2fx[ip] * tq) * g.c2cxi[ip] * (1.0 - fiu) + tip * fiu;
        double tw = 0.5 * (g.f2fx[im] * tq + g.f2fx[i] * tim) * g.c2cxi[i] * (1.0 - fil) + tim * fil;
        double tn = 0.5 * (g.f2fy[j] * tjp + g.f2fy[jp] * tq) * g.c2cyi[jp] * (1.0 - fju) + tjp * fju;
        double ts = 0.5 * (g.f2fy[jm] * tq + g.f2fy[j] * tjm) * g.c2cyi[j] * (1.0 - fjl) + tjm * fjl;
        double tc = 0.5 * (g.f2fz[k] * tkp + g.f2fz[kp] * tq) * g.c2czi[kp] * (1.0 - fku) + tkp * fku;
        double tf = 0.5 * (g.f2fz[km] * tq + g.f2fz[k] * tkm) * g.c2czi[k] * (1.0 - fkl) + tkm * fkl;
        double ant1 = (te * u[qip] - tw * u[q]) * g.f2fxi[i];
        double ant2 = (tn * v[qjp] - ts * v[q]) * g.f2fyi[j];
        double ant3 = (tc * w[qkp] - tf * w[q]) * g.f2fzi[k];
        double omega = (c.iconjg == 1 && c.imovingon == 0) ? (double)p.f.omega[q] : 1.0;
        double src = 0.0;
        if (c.idecomp == 1) {
            double ucc = 0.5 * (u[q] + u[q + 1]);
            src = omega * (ucc / u_bulk);
        }
        double rk3t = -omega * (ant1 + ant2 + ant3) + src;
        double a1 = (tip - tq) * g.c2cxi[ip];
        double a2 = (tq - tim) * g.c2cxi[i];
        double a3 = (tjp - tq) * g.c2cyi[jp];
        double a4 = (tq - tjm) * g.c2cyi[j];
        double a5 = (tkp - tq) * g.c2czi[kp];
        double a6 = (tq - tkm) * g.c2czi[k];
        double altx, alty, altz;
        if (c.iconjg == 1) {
            double cs = p.f.cstar[q];
            altx = cs * (p.f.kstar[0][q] * a1 - p.f.kstar[1][q] * a2) * g.f2fxi[i];
            alty = cs * (p.f.kstar[2][q] * a3 - p.f.kstar[3][q] * a4) * g.f2fyi[j];
            altz = cs * (p.f.kstar[4][q] * a5 - p.f.kstar[5][q] * a6) * g.f2fzi[k];
        } else {
            altx = (a1 - a2) * g.f2fxi[i];
            alty = (a3 - a4) * g.f2fyi[j];
            altz = (a5 - a6) * g.f2fzi[k];
        }
        double alt = inv_repr * (altx + alty + altz);
        if (c.iles == 1) {
            const double *al1 = p.f.alsgs1[0], *al2 = p.f.alsgs1[1], *al3 = p.f.alsgs1[2];
            double tx = g.f2fxi[i] * (al1[qip] * g.c2cxi[ip] * (tip - tq) - al1[q] * g.c2cxi[i] * (tq - tim));
            double ty = g.f2fyi[j] * (al2[qjp] * g.c2cyi[jp] * (tjp - tq) - al2[q] * g.c2cyi[j] * (tq - tjm));
            double tz = g.f2fzi[k] * (al3[qkp] * g.c2czi[kp] * (tkp - tq) - al3[q] * g.c2czi[k] * (tq - tkm));
            alt = alt + omega * (tx + ty + tz);
        }
        p.f.rhs1[3][q] = dt * (gam * rk3t + ro * p.f.rk3o[3][q] + 2.0 * alpha * alt);
        p.f.rk3oo[3][q] = p.f.rk3o[3][q];
        p.f.rk3o[3][q] = rk3t;
    }
}

void launch_rhs_t_kernel(lesgpu_case *c, int msub) {
    const double gam[4] = {0.0, 8.0 / 15.0, 5.0 / 12.0, 3.0 / 4.0};
    const double ro[4] = {0.0, 0.0, -17.0 / 60.0, -5.0 / 12.0};
    const DGrid &g = c->kp.g;
    Box b{1, 1, 1, g.n1m, g.n2m, g.n3m};
    inst_begin(c, LESGPU_K_RHS_T);
    k_rhs_t<<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b, gam[msub], ro[msub]);
    inst_end(c, LESGPU_K_RHS_T);
}

}  // namespace lg
