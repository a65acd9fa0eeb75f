// Direct-forcing immersed boundary: rhs_ibm (slv_mmtm.f90:569-819),
// rhs_ibm_t (slv_engy.f90:201-306), the mass source/sink of divgs
// (slv_cont.f90:48-113), lagforce (slv_auxi.f90:519-570), draglift
// (:666-840) and heatflux (:573-663).
//
// The reference copies the whole right-hand side (rhstmp, 3 full arrays per
// substep) so that the 27-point gathers read values no forcing point has
// overwritten yet.  Here the forcing runs in two phases instead: phase A
// computes every target from the untouched right-hand side into a per-point
// buffer, phase B writes rhs1 at the forcing points.  Same values, no
// full-array copy: the traffic is the gathers themselves.
#include "lesgpu_internal.cuh"

namespace lg {

// reindex_i / reindex_k, slv_mmtm.f90:821-870
__device__ __forceinline__ void reindex(int n, int nm, int &ip, int &ipp) {
    if (ipp == n) ipp = 1;
    else if (ipp == n + 1) { ip = 1; ipp = 2; }
    else if (ipp == 0) ipp = nm;
    else if (ipp == -1) { ip = nm; ipp = nm - 1; }
}

// phase A: targets, fcv and dudtr of every forcing point of component l
__global__ void k_ibm_target(KP p, int l, const double *fld, const double *rhs, double *targ) {
    const DGrid &g = p.g;
    const int nintp = p.c.nintp[l], nbody = p.c.nbody[l];
    const double dti = 1.0 / p.S->dt;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nbody; t += gridDim.x * blockDim.x) {
        const int n = t + 1;
        const int ii = p.f.ifc[l][n], jj = p.f.jfc[l][n], kk = p.f.kfc[l][n];
        const long long q = g.ix(ii, jj, kk);
        double tv = 0.0;                         // stationary body value (ubody = tbody = 0)
        if (n <= nintp) {
            const int *d = p.f.intpindx[l] + 3 * n;
            int ip = ii + d[0], jp = jj + d[1], kp = kk + d[2];
            int ipp = ii + d[0] * 2, jpp = jj + d[1] * 2, kpp = kk + d[2] * 2;
            if (ipp >= g.n1 || ipp <= 0) reindex(g.n1, g.n1m, ip, ipp);
            if (kpp >= g.n3 || kpp <= 0) reindex(g.n3, g.n3m, kp, kpp);
            const int is[3] = {ii, ip, ipp}, js[3] = {jj, jp, jpp}, ks[3] = {kk, kp, kpp};
            const double *gf = p.f.geomfac[l] + 27 * n;
            double s = gf[0] * 0.0;
#pragma unroll
            for (int a = 0; a < 3; a++)
#pragma unroll
                for (int b = 0; b < 3; b++)
#pragma unroll
                    for (int e = 0; e < 3; e++) {
                        if (a == 0 && b == 0 && e == 0) continue;
                        const long long r = g.ix(is[a], js[b], ks[e]);
                        s = s + gf[a * 9 + b * 3 + e] * (fld[r] + rhs[r]);
                    }
            tv = s;
        }
        targ[n] = tv;
        p.f.fcv[l][n] = (tv - fld[q] - rhs[q]) * dti;
        if (l < 3) p.f.dudtr[l][n] = (tv - fld[q]) * dti;
    }
}

// phase B: rhs1 at the forcing points, running sum of the forcing
__global__ void k_ibm_write(KP p, int l, const double *fld, double *rhs, const double *targ) {
    const DGrid &g = p.g;
    const int nbody = p.c.nbody[l];
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nbody; t += gridDim.x * blockDim.x) {
        const int n = t + 1;
        const long long q = g.ix(p.f.ifc[l][n], p.f.jfc[l][n], p.f.kfc[l][n]);
        rhs[q] = targ[n] - fld[q];
        p.f.fcvavg[l][n] = p.f.fcvavg[l][n] + p.f.fcv[l][n];
    }
}

void launch_rhs_ibm(lesgpu_case *c) {
    DFields &f = c->kp.f;
    double *fld[3] = {f.u, f.v, f.w};
    for (int l = 0; l < 3; l++) {
        int nb = c->kp.c.nbody[l];
        if (nb <= 0) continue;
        k_ibm_target<<<blocks_for(nb), kThreads, 0, c->stream>>>(c->kp, l, fld[l], f.rhs1[l], f.ibtarg[l]);
    }
    for (int l = 0; l < 3; l++) {
        int nb = c->kp.c.nbody[l];
        if (nb <= 0) continue;
        k_ibm_write<<<blocks_for(nb), kThreads, 0, c->stream>>>(c->kp, l, fld[l], f.rhs1[l], f.ibtarg[l]);
    }
}

void launch_rhs_ibm_t(lesgpu_case *c) {
    DFields &f = c->kp.f;
    int nb = c->kp.c.nbody[3];
    if (nb <= 0) return;
    k_ibm_target<<<blocks_for(nb), kThreads, 0, c->stream>>>(c->kp, 3, f.t, f.rhs1[3], f.ibtarg[3]);
    k_ibm_write<<<blocks_for(nb), kThreads, 0, c->stream>>>(c->kp, 3, f.t, f.rhs1[3], f.ibtarg[3]);
}

// divgs mass source/sink: one pass over one list; the six passes run in the
// reference's order so every cell accumulates in the same sequence.  Within
// one pass the touched cells are distinct.
__global__ void k_divgs_ibm_pass(KP p, int l, int pass) {
    const DGrid &g = p.g;
    double *qm = p.f.qmass, *dv = p.f.divgsum;
    const double *vel = l == 0 ? p.f.u : l == 1 ? p.f.v : p.f.w;
    const int nb = p.c.nbody[l];
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nb; t += gridDim.x * blockDim.x) {
        const int n = t + 1;
        const int ii = p.f.ifc[l][n], jj = p.f.jfc[l][n], kk = p.f.kfc[l][n];
        const double val = vel[g.ix(ii, jj, kk)];
        if (pass == 0) {
            const long long q = g.ix(ii, jj, kk);
            const double ds = l == 0 ? g.f2fxi[ii] : l == 1 ? g.f2fyi[jj] : g.f2fzi[kk];
            qm[q] = qm[q] - val * ds;
            dv[q] = dv[q] + val * ds;
        } else {
            const int im = l == 0 ? g.imv[ii] : ii, jm = l == 1 ? g.jmv[jj] : jj, km = l == 2 ? g.kmv[kk] : kk;
            const long long q = g.ix(im, jm, km);
            const double ds = l == 0 ? g.f2fxi[im] : l == 1 ? g.f2fyi[jm] : g.f2fzi[km];
            qm[q] = qm[q] + val * ds;
            dv[q] = dv[q] - val * ds;
        }
    }
}

void launch_divgs_ibm(lesgpu_case *c) {
    for (int l = 0; l < 3; l++) {
        int nb = c->kp.c.nbody[l];
        if (nb <= 0) continue;
        for (int pass = 0; pass < 2; pass++)
            k_divgs_ibm_pass<<<blocks_for(nb), kThreads, 0, c->stream>>>(c->kp, l, pass);
    }
}

// A forcing-point index t over the concatenated lists of u, v, w.
__device__ __forceinline__ int ibm_split(const KP &p, int t, int &n) {
    int l = 0;
    while (l < 2 && t >= p.c.nbody[l]) { t -= p.c.nbody[l]; l++; }
    n = t + 1;
    return l;
}

// lagforce, slv_auxi.f90:519-570: sum over the three forcing lists
struct LagTerm {
    double gam, ro;
    __device__ void operator()(const KP &p, int t, int, int, double *w) const {
        const DGrid &g = p.g;
        int n, l = ibm_split(p, t, n);
        w[0] = w[1] = w[2] = 0.0;
        const int ii = p.f.ifc[l][n], jj = p.f.jfc[l][n], kk = p.f.kfc[l][n];
        const double vol = l == 0 ? g.c2cx[ii] * g.f2fy[jj] * g.f2fz[kk]
                         : l == 1 ? g.f2fx[ii] * g.c2cy[jj] * g.f2fz[kk]
                                  : g.f2fx[ii] * g.f2fy[jj] * g.c2cz[kk];
        const long long q = g.ix(ii, jj, kk);
        const double ho = p.f.rk3of[l] ? (double)p.f.rk3of[l][q] : p.f.rk3o[l][q];
        const double hoo = p.f.rk3oof[l] ? (double)p.f.rk3oof[l][q] : p.f.rk3oo[l][q];
        w[l] = vol * (p.f.dudtr[l][n] - (gam * ho + ro * hoo));
    }
};
struct LagFinal {
    int s;
    __device__ void operator()(const KP &p, const double *o) const {
        DScal *S = p.S;
        if (s == 1) { S->dudta = 0.0; S->dvdta = 0.0; S->dwdta = 0.0; }
        S->dudta += o[0];
        S->dvdta += o[1];
        S->dwdta += o[2];
    }
};

static Box ibm_box(const lesgpu_case *c) {
    const DCfg &k = c->kp.c;
    return Box{0, 0, 0, k.nbody[0] + k.nbody[1] + k.nbody[2], 1, 1};
}

void launch_lagforce(lesgpu_case *c, int msub) {
    const double gam[4] = {0.0, 8.0 / 15.0, 5.0 / 12.0, 3.0 / 4.0};
    const double ro[4] = {0.0, 0.0, -17.0 / 60.0, -5.0 / 12.0};
    reduce<3, false>(c, ibm_box(c), LagTerm{gam[msub], ro[msub]}, LagFinal{msub});
}

// draglift, slv_auxi.f90:666-840: IB forcing integral + inertia, then the
// shear on the computational walls, over the volume
struct DragIbTerm {
    __device__ void operator()(const KP &p, int t, int, int, double *w) const {
        const DGrid &g = p.g;
        int n, l = ibm_split(p, t, n);
        w[0] = w[1] = w[2] = 0.0;
        const int ii = p.f.ifc[l][n], jj = p.f.jfc[l][n], kk = p.f.kfc[l][n];
        w[l] = -p.f.fcvavg[l][n] * (g.c2cx[ii] * g.f2fy[jj] * g.f2fz[kk]);
    }
};
struct DragIbFinal {
    __device__ void operator()(const KP &p, const double *o) const {
        DScal *S = p.S;
        S->cd[0] = o[0] + S->dudta;
        S->cd[1] = o[1] + S->dvdta;
        S->cd[2] = o[2] + S->dwdta;
    }
};

// one-sided second-order wall gradient (u1 dy2^2 - u2 dy1^2) / (dy1 dy2 (dy2 - dy1))
__device__ __forceinline__ double wall_grad(double a1, double a2, double d1, double d2) {
    return (a1 * (d2 * d2) - a2 * (d1 * d1)) / (d1 * d2 * (d2 - d1));
}

// Faces of the shear sum: y walls (n1m x n3m each) then z walls (n1m x n2m each).
struct WallShearTerm {
    __device__ void operator()(const KP &p, int t, int, int, double *w) const {
        const DGrid &g = p.g;
        const DCfg &c = p.c;
        const double *u = p.f.u, *v = p.f.v, *wv = p.f.w;
        w[0] = w[1] = w[2] = 0.0;
        const int ny = g.n1m * g.n3m, nz = g.n1m * g.n2m;
        int face;
        if (t < 2 * ny) { face = t / ny; t -= face * ny; }
        else { t -= 2 * ny; face = 2 + t / nz; t -= (face - 2) * nz; }
        if (face < 2) {
            const int i = 1 + t % g.n1m, k = 1 + t / g.n1m;
            if ((face == 0 && c.bc_ybtm != 0) || (face == 1 && c.bc_ytop != 0)) return;
            const int j = face == 0 ? 1 : g.n2m;
            const long long q = g.ix(i, j, k), q2 = face == 0 ? q + g.sx : q - g.sx;
            if (p.f.fb_u[q] < 1.0e-10) return;
            const double d1 = 1.0 / g.c2cyi[face == 0 ? 1 : g.n2];
            const double d2 = d1 + 1.0 / g.c2cyi[face == 0 ? 2 : g.n2m];
            w[0] = wall_grad(u[q], u[q2], d1, d2) * g.c2cx[i] * g.f2fz[k] / c.re;
            w[2] = wall_grad(wv[q], wv[q2], d1, d2) * g.c2cx[i] * g.f2fz[k] / c.re;
        } else {
            const int i = 1 + t % g.n1m, j = 1 + t / g.n1m;
            if ((face == 2 && c.bc_zbtm != 0) || (face == 3 && c.bc_ztop != 0)) return;
            const int k = face == 2 ? 1 : g.n3m;
            const long long q = g.ix(i, j, k), q2 = face == 2 ? q + g.sxy : q - g.sxy;
            if (p.f.fb_u[q] < 1.0e-10) return;
            const double d1 = 1.0 / g.c2czi[face == 2 ? 1 : g.n3];
            const double d2 = d1 + 1.0 / g.c2czi[face == 2 ? 2 : g.n3m];
            w[0] = wall_grad(u[q], u[q2], d1, d2) * g.c2cx[i] * g.f2fy[j] / c.re;
            w[1] = wall_grad(v[q], v[q2], d1, d2) * g.c2cx[i] * g.f2fy[j] / c.re;
        }
    }
};
struct DragFinal {
    __device__ void operator()(const KP &p, const double *o) const {
        DScal *S = p.S;
        const double vol = p.g.xl * p.g.yl * p.g.zl;
        for (int l = 0; l < 3; l++) S->cd[l] = (S->cd[l] + o[l]) / vol;
    }
};

// The thermal counterpart of the force integral: the heat the thermal
// forcing adds over the step, sum of fcvavg(n,4) times the cell-centre
// volume of the T forcing points (fcvavg(:,4) accumulates in rhs_ibm_t,
// slv_engy.f90:299-303; the reference computes no such sum).
struct HeatIbTerm {
    __device__ void operator()(const KP &p, int t, int, int, double *w) const {
        const DGrid &g = p.g;
        const int n = t + 1;
        const int ii = p.f.ifc[3][n], jj = p.f.jfc[3][n], kk = p.f.kfc[3][n];
        w[0] = p.f.fcvavg[3][n] * (g.f2fx[ii] * g.f2fy[jj] * g.f2fz[kk]);
    }
};
struct HeatIbFinal {
    __device__ void operator()(const KP &p, const double *o) const { p.S->heat_body = o[0]; }
};

void launch_draglift(lesgpu_case *c) {
    const DGrid &g = c->kp.g;
    reduce<3, false>(c, ibm_box(c), DragIbTerm{}, DragIbFinal{});
    if (c->kp.c.ihtrans == 1 && c->kp.c.nbody[3] > 0)
        reduce<1, false>(c, Box{0, 0, 0, c->kp.c.nbody[3], 1, 1}, HeatIbTerm{}, HeatIbFinal{});
    Box faces{0, 0, 0, 2 * g.n1m * g.n3m + 2 * g.n1m * g.n2m, 1, 1};
    reduce<3, false>(c, faces, WallShearTerm{}, DragFinal{});
}

// heatflux, slv_auxi.f90:573-663: convective heat flux through the six
// domain faces where the face point lies in the fluid.  Faces: x (n2m x n3m
// each), y (n1m x n3m each), z (n1m x n2m each); the body function at the
// face points comes from tables built at create.
struct HeatFluxTerm {
    __device__ void operator()(const KP &p, int t, int, int, double *w) const {
        const DGrid &g = p.g;
        const double *T = p.f.t;
        w[0] = w[1] = w[2] = w[3] = w[4] = w[5] = 0.0;
        const int nx = g.n2m * g.n3m, ny = g.n1m * g.n3m, nz = g.n1m * g.n2m;
        if (t < 2 * nx) {
            const int side = t / nx, r = t - side * nx;
            const int j = 1 + r % g.n2m, k = 1 + r / g.n2m;
            const double area = g.f2fy[j] * g.f2fz[k];
            const int ib = side == 0 ? 1 : g.n1;
            if (p.f.fb_u[g.ix(ib, j, k)] < 1.0e-10) return;
            const double tf = side == 0 ? 0.5 * (T[g.ix(1, j, k)] + T[g.ix(0, j, k)])
                                        : 0.5 * (T[g.ix(g.n1m, j, k)] + T[g.ix(g.n1, j, k)]);
            w[side] = p.f.u[g.ix(ib, j, k)] * tf * area;
            return;
        }
        t -= 2 * nx;
        if (t < 2 * ny) {
            const int side = t / ny, r = t - side * ny;
            const int i = 1 + r % g.n1m, k = 1 + r / g.n1m;
            const double area = g.f2fx[i] * g.f2fz[k];
            const double *fb = side == 0 ? p.f.fb_vb : p.f.fb_vt;
            if (fb[i + (long long)(g.n1 + 1) * k] < 1.0e-10) return;
            const int jb = side == 0 ? 1 : g.n2;
            const double tf = side == 0 ? 0.5 * (T[g.ix(i, 1, k)] + T[g.ix(i, 0, k)])
                                        : 0.5 * (T[g.ix(i, g.n2m, k)] + T[g.ix(i, g.n2, k)]);
            w[2 + side] = p.f.v[g.ix(i, jb, k)] * tf * area;
            return;
        }
        t -= 2 * ny;
        const int side = t / nz, r = t - side * nz;
        const int i = 1 + r % g.n1m, j = 1 + r / g.n1m;
        const double area = g.f2fx[i] * g.f2fy[j];
        const double *fb = side == 0 ? p.f.fb_wb : p.f.fb_wt;
        if (fb[i + (long long)(g.n1 + 1) * j] < 1.0e-10) return;
        const int kb = side == 0 ? 1 : g.n3;
        const double tf = side == 0 ? 0.5 * (T[g.ix(i, j, 1)] + T[g.ix(i, j, 0)])
                                    : 0.5 * (T[g.ix(i, j, g.n3m)] + T[g.ix(i, j, g.n3)]);
        w[4 + side] = p.f.w[g.ix(i, j, kb)] * tf * area;
    }
};
struct HeatFluxFinal {
    __device__ void operator()(const KP &p, const double *o) const {
        p.S->heat_flux[0] = o[1] - o[0];
        p.S->heat_flux[1] = o[3] - o[2];
        p.S->heat_flux[2] = o[5] - o[4];
    }
};

void launch_heatflux(lesgpu_case *c) {
    const DGrid &g = c->kp.g;
    Box faces{0, 0, 0, 2 * (g.n2m * g.n3m + g.n1m * g.n3m + g.n1m * g.n2m), 1, 1};
    reduce<6, false>(c, faces, HeatFluxTerm{}, HeatFluxFinal{});
}

}  // namespace lg
