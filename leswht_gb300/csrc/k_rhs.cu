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

// R: arithmetic type (double; float in the mixed-precision form).  Every
// load is converted to R, so the whole stencil runs in R; the reference's
// operation order is kept either way.
template <class R>
__global__ void __launch_bounds__(kThreads, sizeof(R) == 4 ? 3 : 1) k_rhs(KP p, Box b, R gam, R ro) {
    const Mir<R> &M = mir<R>(p);
    const DGrid &g = p.g;
    const DCfg &c = p.c;
    const R *u = M.u, *v = M.v, *w = M.w, *pp = M.p, *t = M.t;
    const R *nu = M.nusgs, *nu1 = M.nusgs1[0], *nu2 = M.nusgs1[1], *nu3 = M.nusgs1[2];
    const R dt = p.S->dt, alpha = p.S->alpha, pmi0 = p.S->pmi[0];
    const R ichfac = c.ich != 0 ? R(1.0) : R(0.0);
    const R rei = pickr<R>(c.rei_d, c.rei_f);
    const long long sx = g.sx, sxy = g.sxy;
    // buoyancy in the grdir equation only (decided once, not per cell)
    const bool gbx = c.ihtrans == 1 && c.grdir == 1 && c.gterm != 0.0;
    const bool gby = c.ihtrans == 1 && c.grdir == 2 && c.gterm != 0.0;
    const bool gbz = c.ihtrans == 1 && c.grdir == 3 && c.gterm != 0.0;
    long long n = b.count();
    for (long long tt = (long long)blockIdx.x * blockDim.x + threadIdx.x; tt < n; tt += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        b.at(tt, i, j, k);
        long long q = g.ix(i, j, k);
        const R fju = M.fixju[j], fjl = M.fixjl[j], fku = M.fixku[k], fkl = M.fixkl[k];
        const R fiu = M.fixiu[i], fil = M.fixil[i];
        const R f2fxm = R(M.f2fx[i - 1]), f2fx0 = R(M.f2fx[i]), f2fxp = R(M.f2fx[i + 1]);
        const R f2fym = R(M.f2fy[j - 1]), f2fy0 = R(M.f2fy[j]), f2fyp = R(M.f2fy[j + 1]);
        const R f2fzm = R(M.f2fz[k - 1]), f2fz0 = R(M.f2fz[k]), f2fzp = R(M.f2fz[k + 1]);

        // ---------------- u momentum
        if (i >= g.i_bgpx) {
            R uq = R(u[q]);
            R un = R(0.5) * (f2fyp * uq + f2fy0 * R(u[q + sx])) * R(M.c2cyi[j + 1]) * (R(1.0) - fju) + R(u[g.ix(i, g.n2, k)]) * fju;
            R us = R(0.5) * (f2fy0 * R(u[q - sx]) + f2fym * uq) * R(M.c2cyi[j]) * (R(1.0) - fjl) + R(u[g.ix(i, 0, k)]) * fjl;
            R uc = R(0.5) * (f2fzp * uq + f2fz0 * R(u[q + sxy])) * R(M.c2czi[k + 1]) * (R(1.0) - fku) + R(u[g.ix(i, j, g.n3)]) * fku;
            R uf = R(0.5) * (f2fz0 * R(u[q - sxy]) + f2fzm * uq) * R(M.c2czi[k]) * (R(1.0) - fkl) + R(u[g.ix(i, j, 0)]) * fkl;
            R vnx = R(0.5) * (f2fxm * R(v[q + sx]) + f2fx0 * R(v[q + sx - 1])) * R(M.c2cxi[i]);
            R vsx = R(0.5) * (f2fxm * R(v[q]) + f2fx0 * R(v[q - 1])) * R(M.c2cxi[i]);
            R wcx = R(0.5) * (f2fxm * R(w[q + sxy]) + f2fx0 * R(w[q + sxy - 1])) * R(M.c2cxi[i]);
            R wfx = R(0.5) * (f2fxm * R(w[q]) + f2fx0 * R(w[q - 1])) * R(M.c2cxi[i]);
            R anxe = R(0.5) * (R(u[q + 1]) + uq);
            R anxw = R(0.5) * (uq + R(u[q - 1]));
            R anxx = (anxe * anxe - anxw * anxw) * R(M.c2cxi[i]);
            R anx1 = (un * vnx - us * vsx) * R(M.f2fyi[j]);
            R anx2 = (uc * wcx - uf * wfx) * R(M.f2fzi[k]);
            R rk3x = -anxx - anx1 - anx2;
            R alx1 = (R(u[q + 1]) - uq) * R(M.f2fxi[i]);
            R alx2 = (uq - R(u[q - 1])) * R(M.f2fxi[i - 1]);
            R alx3 = (R(u[q + sx]) - uq) * R(M.c2cyi[j + 1]);
            R alx4 = (uq - R(u[q - sx])) * R(M.c2cyi[j]);
            R alx5 = (R(u[q + sxy]) - uq) * R(M.c2czi[k + 1]);
            R alx6 = (uq - R(u[q - sxy])) * R(M.c2czi[k]);
            R alx = rei * ((alx1 - alx2) * R(M.c2cxi[i]) + (alx3 - alx4) * R(M.f2fyi[j]) + (alx5 - alx6) * R(M.f2fzi[k]));
            if (c.iles == 1) {
                // rhssgs u-part (sgs.f90:1146-1156)
                R a = R(M.f2fyi[j]) * R(M.c2cxi[i]) * (R(nu3[q + sx]) * (R(v[q + sx]) - R(v[q + sx - 1])) - R(nu3[q]) * (R(v[q]) - R(v[q - 1])));
                R bb = R(M.f2fzi[k]) * R(M.c2cxi[i]) * (R(nu2[q + sxy]) * (R(w[q + sxy]) - R(w[q + sxy - 1])) - R(nu2[q]) * (R(w[q]) - R(w[q - 1])));
                R tx = (R(nu[q]) * alx1 - R(nu[q - 1]) * alx2) * R(M.c2cxi[i]);
                R ty = (R(nu3[q + sx]) * alx3 - R(nu3[q]) * alx4) * R(M.f2fyi[j]);
                R tz = (R(nu2[q + sxy]) * alx5 - R(nu2[q]) * alx6) * R(M.f2fzi[k]);
                alx = alx + (R(2.0) * tx + ty + tz);
                rk3x = rk3x + (a + bb);
            }
            if (gbx) rk3x = rk3x + c.gterm * R(t[q]);
            p.f.rhs1[0][q] = dt * (gam * rk3x + ro * hist_o<R>(p, 0)[q] + R(2.0) * alpha * alx
                                   - R(2.0) * alpha * (R(pp[q]) - R(pp[q - 1])) * R(M.c2cxi[i])
                                   - R(2.0) * alpha * pmi0 * ichfac);
            hist_oo<R>(p, 0)[q] = hist_o<R>(p, 0)[q];
            hist_o<R>(p, 0)[q] = rk3x;
        }
        // ---------------- v momentum
        if (j >= g.j_bgpy) {
            R vq = R(v[q]);
            R ve = (R(0.5) * (f2fxp * vq + f2fx0 * R(v[q + 1])) * R(M.c2cxi[i + 1])) * (R(1.0) - fiu) + R(v[g.ix(g.n1, j, k)]) * fiu;
            R vw = (R(0.5) * (f2fx0 * R(v[q - 1]) + f2fxm * vq) * R(M.c2cxi[i])) * (R(1.0) - fil) + R(v[g.ix(0, j, k)]) * fil;
            R vc = (R(0.5) * (f2fzp * vq + f2fz0 * R(v[q + sxy])) * R(M.c2czi[k + 1])) * (R(1.0) - fku) + R(v[g.ix(i, j, g.n3)]) * fku;
            R vf = (R(0.5) * (f2fz0 * R(v[q - sxy]) + f2fzm * vq) * R(M.c2czi[k])) * (R(1.0) - fkl) + R(v[g.ix(i, j, 0)]) * fkl;
            R uey = R(0.5) * (f2fym * R(u[q + 1]) + f2fy0 * R(u[q + 1 - sx])) * R(M.c2cyi[j]);
            R uwy = R(0.5) * (f2fym * R(u[q]) + f2fy0 * R(u[q - sx])) * R(M.c2cyi[j]);
            R wcy = R(0.5) * (f2fym * R(w[q + sxy]) + f2fy0 * R(w[q + sxy - sx])) * R(M.c2cyi[j]);
            R wfy = R(0.5) * (f2fym * R(w[q]) + f2fy0 * R(w[q - sx])) * R(M.c2cyi[j]);
            R anyn = R(0.5) * (R(v[q + sx]) + vq);
            R anys = R(0.5) * (vq + R(v[q - sx]));
            R anyy = R(M.c2cyi[j]) * (anyn * anyn - anys * anys);
            R any1 = (uey * ve - uwy * vw) * R(M.f2fxi[i]);
            R any2 = (vc * wcy - vf * wfy) * R(M.f2fzi[k]);
            R rk3y = -anyy - any1 - any2;
            R aly1 = (R(v[q + 1]) - vq) * R(M.c2cxi[i + 1]);
            R aly2 = (vq - R(v[q - 1])) * R(M.c2cxi[i]);
            R aly3 = (R(v[q + sx]) - vq) * R(M.f2fyi[j]);
            R aly4 = (vq - R(v[q - sx])) * R(M.f2fyi[j - 1]);
            R aly5 = (R(v[q + sxy]) - vq) * R(M.c2czi[k + 1]);
            R aly6 = (vq - R(v[q - sxy])) * R(M.c2czi[k]);
            R aly = rei * ((aly1 - aly2) * R(M.f2fxi[i]) + (aly3 - aly4) * R(M.c2cyi[j]) + (aly5 - aly6) * R(M.f2fzi[k]));
            if (c.iles == 1) {
                R a = R(M.f2fxi[i]) * R(M.c2cyi[j]) * (R(nu3[q + 1]) * (R(u[q + 1]) - R(u[q + 1 - sx])) - R(nu3[q]) * (R(u[q]) - R(u[q - sx])));
                R bb = R(M.f2fzi[k]) * R(M.c2cyi[j]) * (R(nu1[q + sxy]) * (R(w[q + sxy]) - R(w[q + sxy - sx])) - R(nu1[q]) * (R(w[q]) - R(w[q - sx])));
                R tx = (R(nu3[q + 1]) * aly1 - R(nu3[q]) * aly2) * R(M.f2fxi[i]);
                R ty = (R(nu[q]) * aly3 - R(nu[q - sx]) * aly4) * R(M.c2cyi[j]);
                R tz = (R(nu1[q + sxy]) * aly5 - R(nu1[q]) * aly6) * R(M.f2fzi[k]);
                aly = aly + (tx + R(2.0) * ty + tz);
                rk3y = rk3y + (a + bb);
            }
            if (gby) rk3y = rk3y + c.gterm * R(t[q]);
            p.f.rhs1[1][q] = dt * (gam * rk3y + ro * hist_o<R>(p, 1)[q] + R(2.0) * alpha * aly
                                   - R(2.0) * alpha * (R(pp[q]) - R(pp[q - sx])) * R(M.c2cyi[j]));
            hist_oo<R>(p, 1)[q] = hist_o<R>(p, 1)[q];
            hist_o<R>(p, 1)[q] = rk3y;
        }
        // ---------------- w momentum
        if (k >= g.k_bgpz && g.n3m != 1) {
            R wq = R(w[q]);
            R we = R(0.5) * (f2fxp * wq + f2fx0 * R(w[q + 1])) * R(M.c2cxi[i + 1]) * (R(1.0) - fiu) + fiu * R(w[g.ix(g.n1, j, k)]);
            R ww = R(0.5) * (f2fx0 * R(w[q - 1]) + f2fxm * wq) * R(M.c2cxi[i]) * (R(1.0) - fil) + fil * R(w[g.ix(0, j, k)]);
            R wn = (R(0.5) * (f2fyp * wq + f2fy0 * R(w[q + sx])) * R(M.c2cyi[j + 1])) * (R(1.0) - fju) + fju * R(w[g.ix(i, g.n2, k)]);
            R ws = (R(0.5) * (f2fy0 * R(w[q - sx]) + f2fym * wq) * R(M.c2cyi[j])) * (R(1.0) - fjl) + fjl * R(w[g.ix(i, 0, k)]);
            R uez = R(0.5) * (f2fzm * R(u[q + 1]) + f2fz0 * R(u[q + 1 - sxy])) * R(M.c2czi[k]);
            R uwz = R(0.5) * (f2fzm * R(u[q]) + f2fz0 * R(u[q - sxy])) * R(M.c2czi[k]);
            R vnz = R(0.5) * (f2fzm * R(v[q + sx]) + f2fz0 * R(v[q + sx - sxy])) * R(M.c2czi[k]);
            R vsz = R(0.5) * (f2fzm * R(v[q]) + f2fz0 * R(v[q - sxy])) * R(M.c2czi[k]);
            R anzc = R(0.5) * (R(w[q + sxy]) + wq);
            R anzf = R(0.5) * (wq + R(w[q - sxy]));
            R anzz = (anzc * anzc - anzf * anzf) * R(M.c2czi[k]);
            R anz1 = (uez * we - uwz * ww) * R(M.f2fxi[i]);
            R anz2 = (vnz * wn - vsz * ws) * R(M.f2fyi[j]);
            R rk3z = -anzz - anz1 - anz2;
            R alz1 = (R(w[q + 1]) - wq) * R(M.c2cxi[i + 1]);
            R alz2 = (wq - R(w[q - 1])) * R(M.c2cxi[i]);
            R alz3 = (R(w[q + sx]) - wq) * R(M.c2cyi[j + 1]);
            R alz4 = (wq - R(w[q - sx])) * R(M.c2cyi[j]);
            R alz5 = (R(w[q + sxy]) - wq) * R(M.f2fzi[k]);
            R alz6 = (wq - R(w[q - sxy])) * R(M.f2fzi[k - 1]);
            R alz = rei * ((alz1 - alz2) * R(M.f2fxi[i]) + (alz3 - alz4) * R(M.f2fyi[j]) + (alz5 - alz6) * R(M.c2czi[k]));
            if (c.iles == 1) {
                R a = R(M.f2fxi[i]) * R(M.c2czi[k]) * (R(nu2[q + 1]) * (R(u[q + 1]) - R(u[q + 1 - sxy])) - R(nu2[q]) * (R(u[q]) - R(u[q - sxy])));
                R bb = R(M.f2fyi[j]) * R(M.c2czi[k]) * (R(nu1[q + sx]) * (R(v[q + sx]) - R(v[q + sx - sxy])) - R(nu1[q]) * (R(v[q]) - R(v[q - sxy])));
                R tx = (R(nu2[q + 1]) * alz1 - R(nu2[q]) * alz2) * R(M.f2fxi[i]);
                R ty = (R(nu1[q + sx]) * alz3 - R(nu1[q]) * alz4) * R(M.f2fyi[j]);
                R tz = (R(nu[q]) * alz5 - R(nu[q - sxy]) * alz6) * R(M.c2czi[k]);
                alz = alz + (tx + ty + R(2.0) * tz);
                rk3z = rk3z + (a + bb);
            }
            if (gbz) rk3z = rk3z + c.gterm * R(t[q]);
            p.f.rhs1[2][q] = dt * (gam * rk3z + ro * hist_o<R>(p, 2)[q] + R(2.0) * alpha * alz
                                   - R(2.0) * alpha * (R(pp[q]) - R(pp[q - sxy])) * R(M.c2czi[k]));
            hist_oo<R>(p, 2)[q] = hist_o<R>(p, 2)[q];
            hist_o<R>(p, 2)[q] = rk3z;
        }
    }
}

void launch_rhs(lesgpu_case *c, int msub) {
    const double gam[4] = {0.0, 8.0 / 15.0, 5.0 / 12.0, 3.0 / 4.0};
    const double ro[4] = {0.0, 0.0, -17.0 / 60.0, -5.0 / 12.0};
    const DGrid &g = c->kp.g;
    Box b{1, 1, 1, g.n1m, g.n2m, g.n3m};
    inst_begin(c, LESGPU_K_RHS);
    if (c->cfg.precision == LESGPU_PREC_MIXED)
        k_rhs<float><<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b, (float)gam[msub], (float)ro[msub]);
    else
        k_rhs<double><<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b, gam[msub], ro[msub]);
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

// conj: the conjugate tables (c*, k*, omega) are read; 0 when ICONJG = 0 or
// when every loaded table value is 1, where each product with them is exact
// and the terms reduce to the plain ones
template <class R>
__global__ void __launch_bounds__(kThreads) k_rhs_t(KP p, Box b, R gam, R ro, int conj) {
    const Mir<R> &M = mir<R>(p);
    const DGrid &g = p.g;
    const DCfg &c = p.c;
    const R *t = M.t, *u = M.u, *v = M.v, *w = M.w;
    const R dt = p.S->dt, alpha = p.S->alpha, u_bulk = p.S->u_bulk_t;
    const R inv_repr = pickr<R>(c.inv_repr_d, c.inv_repr_f);
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
        const R fiu = M.fixiu[i], fil = M.fixil[i], fju = M.fixju[j], fjl = M.fixjl[j];
        const R fku = M.fixku[k], fkl = M.fixkl[k];
        R tq = R(t[q]);
        long long qip = g.ix(ip, j, k), qim = g.ix(im, j, k), qjp = g.ix(i, jp, k), qjm = g.ix(i, jm, k);
        long long qkp = g.ix(i, j, kp), qkm = g.ix(i, j, km);
        R tip = R(t[qip]), tim = R(t[qim]), tjp = R(t[qjp]), tjm = R(t[qjm]), tkp = R(t[qkp]), tkm = R(t[qkm]);
        R te = R(0.5) * (R(M.f2fx[i]) * tip + R(M.f2fx[ip]) * tq) * R(M.c2cxi[ip]) * (R(1.0) - fiu) + tip * fiu;
        R tw = R(0.5) * (R(M.f2fx[im]) * tq + R(M.f2fx[i]) * tim) * R(M.c2cxi[i]) * (R(1.0) - fil) + tim * fil;
        R tn = R(0.5) * (R(M.f2fy[j]) * tjp + R(M.f2fy[jp]) * tq) * R(M.c2cyi[jp]) * (R(1.0) - fju) + tjp * fju;
        R ts = R(0.5) * (R(M.f2fy[jm]) * tq + R(M.f2fy[j]) * tjm) * R(M.c2cyi[j]) * (R(1.0) - fjl) + tjm * fjl;
        R tc = R(0.5) * (R(M.f2fz[k]) * tkp + R(M.f2fz[kp]) * tq) * R(M.c2czi[kp]) * (R(1.0) - fku) + tkp * fku;
        R tf = R(0.5) * (R(M.f2fz[km]) * tq + R(M.f2fz[k]) * tkm) * R(M.c2czi[k]) * (R(1.0) - fkl) + tkm * fkl;
        R ant1 = (te * R(u[qip]) - tw * R(u[q])) * R(M.f2fxi[i]);
        R ant2 = (tn * R(v[qjp]) - ts * R(v[q])) * R(M.f2fyi[j]);
        R ant3 = (tc * R(w[qkp]) - tf * R(w[q])) * R(M.f2fzi[k]);
        R omega = (conj && c.imovingon == 0) ? R(p.f.omega[q]) : R(1.0);
        R src = R(0.0);
        if (c.idecomp == 1) {
            R ucc = R(0.5) * (R(u[q]) + R(u[q + 1]));
            src = omega * (ucc / u_bulk);
        }
        R rk3t = -omega * (ant1 + ant2 + ant3) + src;
        R a1 = (tip - tq) * R(M.c2cxi[ip]);
        R a2 = (tq - tim) * R(M.c2cxi[i]);
        R a3 = (tjp - tq) * R(M.c2cyi[jp]);
        R a4 = (tq - tjm) * R(M.c2cyi[j]);
        R a5 = (tkp - tq) * R(M.c2czi[kp]);
        R a6 = (tq - tkm) * R(M.c2czi[k]);
        R altx, alty, altz;
        if (conj) {
            R cs = R(M.cstar[q]);
            altx = cs * (R(M.kstar[0][q]) * a1 - R(M.kstar[1][q]) * a2) * R(M.f2fxi[i]);
            alty = cs * (R(M.kstar[2][q]) * a3 - R(M.kstar[3][q]) * a4) * R(M.f2fyi[j]);
            altz = cs * (R(M.kstar[4][q]) * a5 - R(M.kstar[5][q]) * a6) * R(M.f2fzi[k]);
        } else {
            altx = (a1 - a2) * R(M.f2fxi[i]);
            alty = (a3 - a4) * R(M.f2fyi[j]);
            altz = (a5 - a6) * R(M.f2fzi[k]);
        }
        R alt = inv_repr * (altx + alty + altz);
        if (c.iles == 1) {
            const R *al1 = M.alsgs1[0], *al2 = M.alsgs1[1], *al3 = M.alsgs1[2];
            R tx = R(M.f2fxi[i]) * (R(al1[qip]) * R(M.c2cxi[ip]) * (tip - tq) - R(al1[q]) * R(M.c2cxi[i]) * (tq - tim));
            R ty = R(M.f2fyi[j]) * (R(al2[qjp]) * R(M.c2cyi[jp]) * (tjp - tq) - R(al2[q]) * R(M.c2cyi[j]) * (tq - tjm));
            R tz = R(M.f2fzi[k]) * (R(al3[qkp]) * R(M.c2czi[kp]) * (tkp - tq) - R(al3[q]) * R(M.c2czi[k]) * (tq - tkm));
            alt = alt + omega * (tx + ty + tz);
        }
        p.f.rhs1[3][q] = dt * (gam * rk3t + ro * hist_o<R>(p, 3)[q] + R(2.0) * alpha * alt);
        hist_oo<R>(p, 3)[q] = hist_o<R>(p, 3)[q];
        hist_o<R>(p, 3)[q] = rk3t;
    }
}

void launch_rhs_t_kernel(lesgpu_case *c, int msub) {
    const double gam[4] = {0.0, 8.0 / 15.0, 5.0 / 12.0, 3.0 / 4.0};
    const double ro[4] = {0.0, 0.0, -17.0 / 60.0, -5.0 / 12.0};
    const DGrid &g = c->kp.g;
    Box b{1, 1, 1, g.n1m, g.n2m, g.n3m};
    inst_begin(c, LESGPU_K_RHS_T);
    const int conj = c->kp.c.iconjg == 1 && c->conj_general;
    if (c->cfg.precision == LESGPU_PREC_MIXED)
        k_rhs_t<float><<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b, (float)gam[msub], (float)ro[msub], conj);
    else
        k_rhs_t<double><<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b, gam[msub], ro[msub], conj);
    inst_end(c, LESGPU_K_RHS_T);
}

}  // namespace lg
