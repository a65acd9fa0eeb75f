// Convective outlet at i = n1 for flows that are not periodic in x:
// convbc (slv_mmtm.f90:873-988), rhsincorpbc (:991-1041), convbc_t
// (slv_engy.f90:309-413) and rhsincorpbc_t (:416-457).
//
// The outlet values follow du/dt + U_c du/dx = 0 with U_c the mean outlet
// velocity, then are scaled so the outflow matches the inflow through the
// other five faces (global mass conservation).  Work is 2-D: the three
// face sums are deterministic two-stage reductions, the plane updates are
// one thread per (j, k).
#include "lesgpu_internal.cuh"

namespace lg {

// inflow through the x inlet, the y faces and the z faces (qin), and the
// outlet flux (ubar); faces are enumerated x (n2m n3m), y (n1m n3m), z (n1m n2m)
struct OutletQTerm {
    __device__ void operator()(const KP &p, int t, int, int, double *w) const {
        const DGrid &g = p.g;
        const double *u = p.f.u, *v = p.f.v, *wv = p.f.w;
        w[0] = w[1] = 0.0;
        const int nx = g.n2m * g.n3m, ny = g.n1m * g.n3m;
        if (t < nx) {
            const int j = 1 + t % g.n2m, k = 1 + t / g.n2m;
            const double a = g.f2fy[j] * g.f2fz[k];
            w[0] = u[g.ix(1, j, k)] * a;
            w[1] = u[g.ix(g.n1, j, k)] * a;
            return;
        }
        t -= nx;
        if (t < ny) {
            const int i = 1 + t % g.n1m, k = 1 + t / g.n1m;
            w[0] = (v[g.ix(i, 1, k)] - v[g.ix(i, g.n2, k)]) * g.f2fx[i] * g.f2fz[k];
            return;
        }
        t -= ny;
        const int i = 1 + t % g.n1m, j = 1 + t / g.n1m;
        w[0] = (wv[g.ix(i, j, 1)] - wv[g.ix(i, j, g.n3)]) * g.f2fx[i] * g.f2fy[j];
    }
};
struct OutletQFinal {
    __device__ void operator()(const KP &p, const double *o) const {
        DScal *S = p.S;
        const DGrid &g = p.g;
        const double ubar = o[1] / (g.yl * g.zl);
        S->cb[0] = o[0];                                  // qin
        S->cb[1] = ubar * S->dtconst * g.f2fxi[g.n1m];    // ucoef
        S->cb[2] = ubar * S->dtconst * g.c2cxi[g.n1];     // vwcoef
    }
};

// outlet values of the substep and the outflow they carry
struct OutletOutTerm {
    int thermal;
    __device__ void operator()(const KP &p, int t, int, int, double *w) const {
        const DGrid &g = p.g;
        const DFields &f = p.f;
        const int j = 1 + t % g.n2m, k = 1 + t / g.n2m;
        const long long pq = j + (long long)(g.n2 + 1) * k;
        const long long qo = g.ix(g.n1, j, k), qi = g.ix(g.n1m, j, k);
        const double ucoef = p.S->cb[1], vwcoef = p.S->cb[2];
        const bool solid = f.fb_c[qi] <= 1.0e-10 && p.c.imovingon == 0;
        double uo;
        if (!thermal) {
            if (solid) {
                f.uout[pq] = f.u[qi]; f.vout[pq] = f.v[qi]; f.wout[pq] = f.w[qi];
            } else {
                f.uout[pq] = f.u[qo] - ucoef * (f.u[qo] - f.u[qi]);
                f.vout[pq] = f.v[qo] - vwcoef * (f.v[qo] - f.v[qi]);
                f.wout[pq] = f.w[qo] - vwcoef * (f.w[qo] - f.w[qi]);
            }
            uo = f.uout[pq];
        } else {
            uo = f.u[qo] - ucoef * (f.u[qo] - f.u[qi]);
            f.tout[pq] = solid ? f.t[qi] : f.t[qo] - vwcoef * (f.t[qo] - f.t[qi]);
        }
        w[0] = uo * g.f2fy[j] * g.f2fz[k];
    }
};
struct OutletOutFinal {
    int thermal;
    __device__ void operator()(const KP &p, const double *o) const {
        const double qin = p.S->cb[0], qout = o[0];
        p.S->cb[3] = thermal ? (fabs(qout) > 1.0e-14 ? qin / qout : 1.0) : qin / qout;
    }
};

__global__ void k_outlet_scale(KP p, int thermal) {
    const DGrid &g = p.g;
    const DFields &f = p.f;
    const double qr = p.S->cb[3];
    const long long n = (long long)g.n2m * g.n3m;
    for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += (long long)gridDim.x * blockDim.x) {
        const int j = 1 + (int)(s % g.n2m), k = 1 + (int)(s / g.n2m);
        const long long pq = j + (long long)(g.n2 + 1) * k, qo = g.ix(g.n1, j, k);
        const bool fluid = f.fb_c[g.ix(g.n1m, j, k)] > 1.0e-10;
        if (!thermal) {
            if (fluid) { f.uout[pq] *= qr; f.vout[pq] *= qr; f.wout[pq] *= qr; }
            f.duout[pq] = f.uout[pq] - f.u[qo];
            f.dvout[pq] = f.vout[pq] - f.v[qo];
            f.dwout[pq] = f.wout[pq] - f.w[qo];
        } else {
            if (fluid) f.tout[pq] *= qr;
            f.dtout[pq] = f.tout[pq] - f.t[qo];
        }
    }
}

// periodic copies of the outlet increments: dir 1 (y, all k), then dir 2 (z, all j)
__global__ void k_outlet_ghost(KP p, int thermal, int dir) {
    const DGrid &g = p.g;
    const DFields &f = p.f;
    double *a[3] = {thermal ? f.dtout : f.duout, f.dvout, f.dwout};
    const int na = thermal ? 1 : 3;
    const long long sp = g.n2 + 1;
    const int n = dir == 1 ? g.n3 + 1 : g.n2 + 1;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x)
        for (int q = 0; q < na; q++) {
            if (dir == 1) {
                a[q][g.n2 + sp * s] = a[q][1 + sp * s];
                a[q][0 + sp * s] = a[q][g.n2m + sp * s];
            } else {
                a[q][s + sp * g.n3] = a[q][s + sp * 1];
                a[q][s + sp * 0] = a[q][s + sp * g.n3m];
            }
        }
}

__global__ void k_rhsincorpbc(KP p) {
    const DGrid &g = p.g;
    const DFields &f = p.f;
    const double acoef = p.S->acoef;
    const double cre = p.c.iles == 1 ? p.c.re : 0.0, cre2 = p.c.iles == 1 ? 2.0 * p.c.re : 0.0;
    const long long n = (long long)g.n2m * g.n3m;
    for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += (long long)gridDim.x * blockDim.x) {
        const int j = 1 + (int)(s % g.n2m), k = 1 + (int)(s / g.n2m);
        const long long pq = j + (long long)(g.n2 + 1) * k;
        const long long qi = g.ix(g.n1m, j, k), qo = g.ix(g.n1, j, k);
        f.rhs1[0][qi] -= acoef * f.ciu[g.n1m] * (1.0 + cre2 * f.nusgs[qi]) * f.duout[pq];
        if (j >= 2) f.rhs1[1][qi] -= acoef * f.civw[g.n1m] * (1.0 + cre * f.nusgs1[2][qo]) * f.dvout[pq];
        if (k >= g.k_bgpz) f.rhs1[2][qi] -= acoef * f.civw[g.n1m] * (1.0 + cre * f.nusgs1[1][qo]) * f.dwout[pq];
    }
}

__global__ void k_rhsincorpbc_t(KP p) {
    const DGrid &g = p.g;
    const DFields &f = p.f;
    const DCfg &c = p.c;
    const double acoef = p.S->acoef;
    const double cre2 = c.iles == 1 ? 2.0 * c.re * c.pr : 0.0;
    const long long n = (long long)g.n2m * g.n3m;
    for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += (long long)gridDim.x * blockDim.x) {
        const int j = 1 + (int)(s % g.n2m), k = 1 + (int)(s / g.n2m);
        const long long pq = j + (long long)(g.n2 + 1) * k, q = g.ix(g.n1m, j, k);
        double cs = 1.0, ks = 1.0, omc = 1.0;
        if (c.iconjg == 1) {
            cs = f.cstar[q];
            ks = (f.kstar[0][q] + f.kstar[1][q] + f.kstar[2][q] + f.kstar[3][q] + f.kstar[4][q] + f.kstar[5][q]) / 6.0;
            omc = c.imovingon == 0 ? (double)f.omega[q] : 1.0;
        }
        f.rhs1[3][q] -= acoef * cs * ks * f.ciu[g.n1m] * (1.0 + cre2 * omc * f.alsgs[q]) * f.dtout[pq];
    }
}

static void outlet(lesgpu_case *c, int thermal) {
    const DGrid &g = c->kp.g;
    const DCfg &cf = c->kp.c;
    // ICH = 1: the reference zeroes the outlet planes; they are zero from
    // create on and nothing else writes them
    if (cf.ich == 1) return;
    const long long nplane = (long long)g.n2m * g.n3m;
    reduce<2, false>(c, Box{0, 0, 0, (int)(nplane + (long long)g.n1m * g.n3m + (long long)g.n1m * g.n2m), 1, 1},
                     OutletQTerm{}, OutletQFinal{});
    reduce<1, false>(c, Box{0, 0, 0, (int)nplane, 1, 1}, OutletOutTerm{thermal}, OutletOutFinal{thermal});
    k_outlet_scale<<<blocks_for(nplane), kThreads, 0, c->stream>>>(c->kp, thermal);
    if (cf.yprdic == 1) k_outlet_ghost<<<blocks_for(g.n3 + 1), kThreads, 0, c->stream>>>(c->kp, thermal, 1);
    if (cf.zprdic == 1) k_outlet_ghost<<<blocks_for(g.n2 + 1), kThreads, 0, c->stream>>>(c->kp, thermal, 2);
}

// convbc + rhsincorpbc (momentum), called between rhs(_ibm) and the ADI sweeps
void launch_convbc(lesgpu_case *c) {
    const DGrid &g = c->kp.g;
    outlet(c, 0);
    if (c->kp.c.ich != 1) k_rhsincorpbc<<<blocks_for((long long)g.n2m * g.n3m), kThreads, 0, c->stream>>>(c->kp);
}

// convbc_t + rhsincorpbc_t, only for flows not periodic in x
void launch_convbc_t(lesgpu_case *c) {
    const DGrid &g = c->kp.g;
    if (c->kp.c.xprdic != 0) return;
    outlet(c, 1);
    if (c->kp.c.ich != 1) k_rhsincorpbc_t<<<blocks_for((long long)g.n2m * g.n3m), kThreads, 0, c->stream>>>(c->kp);
}

}  // namespace lg
