// Step/substep bookkeeping, global reductions, projection and pressure
// update: the routines of 02_solver/f90/lib/slv_auxi.f90, meanpg of
// slv_mmtm.f90:2-177 and the checks of misc_init.f90:1047-1104.
//
// Every global sum is a two-stage deterministic reduction: a fixed grid of
// kRedBlocks blocks strides over the cells in a fixed order, each block
// writes its partials, and a one-block kernel folds them in a fixed tree and
// applies the scalar logic of the reference routine.  The result is the same
// bit pattern on every run.
#include "lesgpu_internal.cuh"

namespace lg {

static Box interior(const DGrid &g) { return Box{1, 1, 1, g.n1m, g.n2m, g.n3m}; }

// ------------------------------------------------------------ stepinit/cfl
// cfl, slv_auxi.f90:53-102: max over cells of the cell-centre |u|/dx sum.
// The reference multiplies each cell's sum by dt before the max; dt > 0 so
// max(s)*dt is the same rounded value.
struct CflTerm {
    __device__ void operator()(const KP &p, int i, int j, int k, double *w) const {
        const DGrid &g = p.g;
        long long q = g.ix(i, j, k);
        double c1 = fabs(p.f.u[q] + p.f.u[q + 1]) * 0.5 * g.f2fxi[i];
        double c2 = fabs(p.f.v[q] + p.f.v[q + g.sx]) * 0.5 * g.f2fyi[j];
        double c3 = fabs(p.f.w[q] + p.f.w[q + g.sxy]) * 0.5 * g.f2fzi[k];
        w[0] = c1 + c2 + c3;
    }
};

// stepinit, slv_auxi.f90:2-50
__device__ void stepinit_pre(KP p);
// The last block of the CFL reduction first does stepinit's scalar updates
// (k_stepinit_pre's work; the per-cell terms read none of them), saving a
// launch per step.
struct StepinitFinal {
    __device__ void operator()(const KP &p, const double *out) const {
        stepinit_pre(p);
        DScal *S = p.S;
        const DCfg &c = p.c;
        double cflm = out[0] * S->dt;
        if (cflm < 0.0) cflm = 0.0;
        S->cflmax = cflm;
        if (c.idtopt != 0 && cflm != 0.0) {
            double a = S->dt * c.cflfac / cflm;
            double b = S->dt * (0.80 + 0.20 * c.cflfac / cflm);
            double dtcfl = a < b ? a : b;
            if (c.idtopt == 1) S->dt = dtcfl;
        }
        double at = fabs(S->time);
        double eps_t = 1.0e-12 * (at > 1.0 ? at : 1.0);
        double dt_evt = S->dt;
        if (c.ptb_tst > S->time + eps_t) dt_evt = fmin(dt_evt, c.ptb_tst - S->time);
        if (c.avg_tst > S->time + eps_t) dt_evt = fmin(dt_evt, c.avg_tst - S->time);
        if (c.tend > S->time + eps_t) dt_evt = fmin(dt_evt, c.tend - S->time);
        if (dt_evt < S->dt) S->dt = dt_evt;
        if (!(S->dt > 0.0) || !isfinite(S->dt)) S->err |= 1;
    }
};

__device__ void stepinit_pre(KP p) {
    DScal *S = p.S;
    S->ntime += 1;
    S->m = S->ntime;
    S->poisson_unconv = 0;
    S->heat_body = 0.0;
    if (p.c.ich != 0) S->pmiavg = 0.0;
    if (p.c.idtopt == 0) S->dt = p.c.dt_size;
    S->subdt = 0.0;
}

__global__ void k_zero_fcvavg(KP p) {
    for (int l = 0; l < 4; l++) {
        int n = p.c.nbody[l];
        for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
            p.f.fcvavg[l][t + 1] = 0.0;
    }
}

void launch_stepinit(lesgpu_case *c) {
    if (c->kp.c.ibmon == 1) k_zero_fcvavg<<<64, kThreads, 0, c->stream>>>(c->kp);
    reduce<1, true>(c, interior(c->kp.g), CflTerm{}, StepinitFinal{});
}

// substepinit, slv_auxi.f90:105-123 (RK3 coefficients of rk3coefinit,
// misc_init.f90:1031-1044)
__global__ void k_substepinit(KP p, int s) {
    const double gam[4] = {0.0, 8.0 / 15.0, 5.0 / 12.0, 3.0 / 4.0};
    const double ro[4] = {0.0, 0.0, -17.0 / 60.0, -5.0 / 12.0};
    DScal *S = p.S;
    S->alpha = 0.5 * (gam[s] + ro[s]);
    S->dtconst = S->dt * (gam[s] + ro[s]);
    S->dtconsti = 1.0 / S->dtconst;
    S->test1 = p.c.resid1 * S->dtconsti;
    S->acoef = S->alpha * S->dt / p.c.re;
    S->acoefi = 1.0 / S->acoef;
    S->pmiavg = S->pmiavg + S->pmi[0] * 2.0 * S->alpha;
    S->subdt = S->subdt + S->dtconst;
}

void launch_substepinit(lesgpu_case *c, int msub) { k_substepinit<<<1, 1, 0, c->stream>>>(c->kp, msub); }

// ------------------------------------------------------------ qvol / tvol
struct QvolTerm {   // qvolcalc, slv_auxi.f90:126-149
    __device__ void operator()(const KP &p, int i, int j, int k, double *w) const {
        long long q = p.g.ix(i, j, k);
        w[0] = p.f.u[q] * p.f.wq[q];     // u c2cx f2fy f2fz over the fluid u points
    }
};
struct QvolFinal {
    int slot;
    __device__ void operator()(const KP &p, const double *out) const { p.S->qvol[slot] = out[0]; }
};
void launch_qvolcalc(lesgpu_case *c, int slot) { reduce<1, false>(c, interior(c->kp.g), QvolTerm{}, QvolFinal{slot}); }

struct TvolTerm {   // tvolcalc, slv_auxi.f90:152-173
    __device__ void operator()(const KP &p, int i, int j, int k, double *w) const {
        long long q = p.g.ix(i, j, k);
        w[0] = p.f.t[q] * p.f.wt[q];     // t / c* f2fx f2fy f2fz
    }
};
struct TvolFinal {
    int slot;
    __device__ void operator()(const KP &p, const double *out) const { p.S->tvol[slot] = out[0]; }
};
void launch_tvolcalc(lesgpu_case *c, int slot) { reduce<1, false>(c, interior(c->kp.g), TvolTerm{}, TvolFinal{slot}); }

// Weights of the volume reductions: the cell-volume products and fluid masks
// of qvolcalc / meanpg (fb_u), the bulk velocity (fb_c) and tvolcalc (1/c*),
// formed once so each reduction does one multiply per cell.
__global__ void k_red_weights(KP p, Box b) {
    const DGrid &g = p.g;
    const long long n = b.count();
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        b.at(t, i, j, k);
        const long long q = g.ix(i, j, k);
        const double cv = g.c2cx[i] * g.f2fy[j] * g.f2fz[k];
        p.f.wq[q] = p.f.fb_u[q] >= 1.0e-10 ? cv : 0.0;
        p.f.wb[q] = p.f.fb_c[q] >= 1.0e-10 ? cv : 0.0;
        p.f.wt[q] = g.f2fx[i] * g.f2fy[j] * g.f2fz[k] / p.f.cstar[q];
    }
}
void launch_red_weights(lesgpu_case *c) {
    Box b = interior(c->kp.g);
    k_red_weights<<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b);
}

// tvolcorr, slv_auxi.f90:206-230.  The volume integral of 1/c* does not
// change in time; it is reduced once (lesgpu_start) into S->cvol.
struct CvolTerm {
    __device__ void operator()(const KP &p, int i, int j, int k, double *w) const {
        long long q = p.g.ix(i, j, k);
        w[0] = p.f.wt[q];                // 1 / c* f2fx f2fy f2fz
    }
};
struct CvolFinal {
    __device__ void operator()(const KP &p, const double *out) const { p.S->cvol = out[0]; }
};
// tvolcalc(tvol(2)) followed by tvolcorr in one launch: the reduction's last
// block stores tvol(2) and forms thcap from it
// (slot0: tcalc leaves t unchanged, so the following tvolcalc(tvol(0)) is the
// same sum and is stored here too)
struct TvolCorrFinal {
    int slot0;
    __device__ void operator()(const KP &p, const double *out) const {
        p.S->tvol[2] = out[0];
        p.S->thcap = (p.S->tvol[2] - p.S->tvol[1]) / p.S->cvol;
        if (slot0) p.S->tvol[0] = out[0];
    }
};
void launch_tvolcalc_corr(lesgpu_case *c, bool slot0) {
    reduce<1, false>(c, interior(c->kp.g), TvolTerm{}, TvolCorrFinal{slot0 ? 1 : 0});
}
void launch_cvol(lesgpu_case *c) { reduce<1, false>(c, interior(c->kp.g), CvolTerm{}, CvolFinal{}); }

// tcalc, slv_auxi.f90:496-516
__global__ void k_tcalc(KP p, Box b) {
    long long n = b.count();
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        b.at(t, i, j, k);
        p.f.t[p.g.ix(i, j, k)] -= p.S->thcap;
    }
}
void launch_tcalc(lesgpu_case *c) {
    if (c->kp.c.ich == 1 && c->kp.c.xprdic == 0) {
        Box b = interior(c->kp.g);
        k_tcalc<<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b);
    }
}

// ------------------------------------------------------------------ meanpg
// Two passes: flow volume and flow rate over every cell, and the four
// wall-shear sums over the planes next to no-slip walls only (the terms are
// zero elsewhere; carrying them through the volume pass cost it two thirds
// of its time).  The wall pass runs first and leaves its sums in pmiw.
struct MeanpgTerm {
    __device__ void operator()(const KP &p, int i, int j, int k, double *w) const {
        const long long q = p.g.ix(i, j, k);
        const double vol = p.f.wq[q];    // c2cx f2fy f2fz over the fluid u points, else 0
        w[0] = vol;
        w[1] = p.f.u[q] * vol;
    }
};
// Box (i, plane, c): plane 0 / 1 = the y-bottom / top wall (j = 1 / n2m,
// k = c), 2 / 3 = the z-bottom / top wall (k = 1 / n3m, j = c); c beyond the
// plane's extent contributes nothing.  A cell on two walls is visited once
// per wall, as the one-pass form tested each wall for every cell.
struct MeanpgWallTerm {
    __device__ void operator()(const KP &p, int i, int plane, int cc, double *w) const {
        const DGrid &g = p.g;
        const DCfg &c = p.c;
        const double *u = p.f.u;
        w[0] = w[1] = w[2] = w[3] = 0.0;
        int j, k;
        if (plane <= 1) {
            j = plane == 0 ? 1 : g.n2m;
            k = cc;
            if (k > g.n3m || (plane == 0 && c.bc_ybtm != 0) || (plane == 1 && c.bc_ytop != 0)) return;
        } else {
            k = plane == 2 ? 1 : g.n3m;
            j = cc;
            if (j > g.n2m || (plane == 2 && c.bc_zbtm != 0) || (plane == 3 && c.bc_ztop != 0)) return;
        }
        const long long q = g.ix(i, j, k);
        if (p.f.fb_u[q] < 1.0e-10) return;
        if (plane == 0) {
            double dy1 = 1.0 / g.c2cyi[1], dy2 = dy1 + 1.0 / g.c2cyi[2];
            double gu = (u[q] * (dy2 * dy2) - u[q + g.sx] * (dy1 * dy1)) / (dy1 * dy2 * (dy2 - dy1));
            w[0] = gu * g.c2cx[i] * g.f2fz[k] / c.re;
        } else if (plane == 1) {
            double dy1 = 1.0 / g.c2cyi[g.n2], dy2 = dy1 + 1.0 / g.c2cyi[g.n2m];
            double gu = (u[q] * (dy2 * dy2) - u[q - g.sx] * (dy1 * dy1)) / (dy1 * dy2 * (dy2 - dy1));
            w[1] = gu * g.c2cx[i] * g.f2fz[k] / c.re;
        } else if (plane == 2) {
            double dz1 = 1.0 / g.c2czi[1], dz2 = dz1 + 1.0 / g.c2czi[2];
            double gu = (u[q] * (dz2 * dz2) - u[q + g.sxy] * (dz1 * dz1)) / (dz1 * dz2 * (dz2 - dz1));
            w[2] = gu * g.c2cx[i] * g.f2fy[j] / c.re;
        } else {
            double dz1 = 1.0 / g.c2czi[g.n3], dz2 = dz1 + 1.0 / g.c2czi[g.n3m];
            double gu = (u[q] * (dz2 * dz2) - u[q - g.sxy] * (dz1 * dz1)) / (dz1 * dz2 * (dz2 - dz1));
            w[3] = gu * g.c2cx[i] * g.f2fy[j] / c.re;
        }
    }
};
struct MeanpgWallFinal {
    __device__ void operator()(const KP &p, const double *o) const {
        for (int q = 0; q < 4; q++) p.S->pmiw[q] = o[q];
    }
};

// IB streamwise forcing term of meanpg (slv_mmtm.f90:141-146)
__global__ void k_meanpg_ibm(KP p) {
    double v[1] = {0.0};
    int n = p.c.nbody[0];
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        int m = t + 1;
        v[0] += p.f.fcv[0][m] * p.g.c2cx[p.f.ifc[0][m]] * p.g.f2fy[p.f.jfc[0][m]] * p.g.f2fz[p.f.kfc[0][m]];
    }
    block_reduce<1, false>(v);
    if (threadIdx.x == 0) p.f.part[(size_t)kRedBlocks * kMaxRed] = v[0];
}

struct MeanpgFinal {
    __device__ void operator()(const KP &p, const double *o) const {
        DScal *S = p.S;
        const DCfg &c = p.c;
        double flowvol = o[0], qcur = o[1];
        double ubulk = flowvol > 0.0 ? qcur / flowvol : 0.0;
        for (int q = 0; q < 5; q++) S->pmi[q] = 0.0;
        if (c.bc_ybtm == 0) S->pmi[1] += S->pmiw[0];
        if (c.bc_ytop == 0) S->pmi[2] += S->pmiw[1];
        if (c.bc_zbtm == 0) S->pmi[3] += S->pmiw[2];
        if (c.bc_ztop == 0) S->pmi[4] += S->pmiw[3];
        S->pmi[0] = S->pmi[1] + S->pmi[2] + S->pmi[3] + S->pmi[4];
        double ibm = (c.nbody[0] > 0) ? p.f.part[(size_t)kRedBlocks * kMaxRed] : 0.0;
        S->pmi[0] = S->pmi[0] + ibm;
        double volume = p.g.xl * p.g.yl * p.g.zl;
        for (int q = 0; q < 5; q++) S->pmi[q] = S->pmi[q] / volume;
        if (c.ich == 0) {
            S->pmi[0] = 0.0;
        } else if (c.ich == 1) {
            if (S->ntime > 0 && S->dt > 0.0) {
                double err = c.udrv_i - ubulk;
                S->err_integral = S->err_integral + err * S->dtconst;
                S->pmi[0] = S->pmi[0] - (1.0 * err + 0.1 * S->err_integral);
            }
        } else if (c.ich == 2) {
            S->pmi[0] = -c.udrv_i;
        }
    }
};

void launch_meanpg(lesgpu_case *c) {
    const DGrid &g = c->kp.g;
    if (c->kp.c.nbody[0] > 0) k_meanpg_ibm<<<1, kThreads, 0, c->stream>>>(c->kp);
    reduce<4, false>(c, Box{1, 0, 1, g.n1m, 4, g.n2m > g.n3m ? g.n2m : g.n3m}, MeanpgWallTerm{}, MeanpgWallFinal{});
    reduce<2, false>(c, interior(g), MeanpgTerm{}, MeanpgFinal{});
}

// ------------------------------------------------------------------- ucalc
// ucalc, slv_auxi.f90:233-416 (interior update; ghosts by launch_ghost_*)
__global__ void __launch_bounds__(kThreads) k_ucalc(KP p, Box b) {
    long long n = b.count();
    const DGrid &g = p.g;
    double dtc = p.S->dtconst;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        b.at(t, i, j, k);
        long long q = g.ix(i, j, k);
        const double *phi = p.f.phi;
        double ph = phi[q];
        if (i >= g.i_bgpx) {
            int im = g.imv[i];
            p.f.u[q] = p.f.u[q] - dtc * (ph - phi[g.ix(im, j, k)]) * g.c2cxi[i];
        }
        if (j >= 2) p.f.v[q] = p.f.v[q] - dtc * (ph - phi[q - g.sx]) * g.c2cyi[j];
        if (k >= g.k_bgpz) {
            int km = g.kmv[k];
            p.f.w[q] = p.f.w[q] - dtc * (ph - phi[g.ix(i, j, km)]) * g.c2czi[k];
        }
    }
}

// Periodic ghost copy of one plane pair for up to 4 arrays.
//  dir 0: a(0,j,k) = a(n1m,j,k), a(n1,j,k) = a(1,j,k) over j in [j0,j1], k in [k0,k1]
//  dir 1: a(i,0,k) = a(i,n2m,k), a(i,n2,k) = a(i,1,k) over i, k
//  dir 2: a(i,j,0) = a(i,j,n3m), a(i,j,n3) = a(i,j,1) over i, j

__global__ void k_ghost(KP p, int dir, GhostSpec s0, GhostSpec s1, GhostSpec s2, GhostSpec s3, int na) {
    const DGrid &g = p.g;
    GhostSpec ss[4] = {s0, s1, s2, s3};
    for (int a = 0; a < na; a++) {
        const GhostSpec &s = ss[a];
        int n0 = s.hi0 - s.lo0 + 1, n1 = s.hi1 - s.lo1 + 1;
        long long n = (long long)n0 * n1;
        for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
            int x0 = s.lo0 + (int)(t % n0), x1 = s.lo1 + (int)(t / n0);
            if (dir == 0) {
                s.a[g.ix(0, x0, x1)] = s.a[g.ix(g.n1m, x0, x1)];
                s.a[g.ix(g.n1, x0, x1)] = s.a[g.ix(1, x0, x1)];
            } else if (dir == 1) {
                s.a[g.ix(x0, 0, x1)] = s.a[g.ix(x0, g.n2m, x1)];
                s.a[g.ix(x0, g.n2, x1)] = s.a[g.ix(x0, 1, x1)];
            } else {
                s.a[g.ix(x0, x1, 0)] = s.a[g.ix(x0, x1, g.n3m)];
                s.a[g.ix(x0, x1, g.n3)] = s.a[g.ix(x0, x1, 1)];
            }
        }
    }
}

void ghost(lesgpu_case *c, int dir, GhostSpec *s, int na) {
    GhostSpec z{nullptr, 0, -1, 0, -1};
    GhostSpec a0 = na > 0 ? s[0] : z, a1 = na > 1 ? s[1] : z, a2 = na > 2 ? s[2] : z, a3 = na > 3 ? s[3] : z;
    long long mx = 0;
    for (int q = 0; q < na; q++) {
        long long n = (long long)(s[q].hi0 - s[q].lo0 + 1) * (s[q].hi1 - s[q].lo1 + 1);
        if (n > mx) mx = n;
    }
    k_ghost<<<blocks_for(mx), kThreads, 0, c->stream>>>(c->kp, dir, a0, a1, a2, a3, na);
}

// qvolcalc(qvol(2)), ucalc and qvolcalc(qvol(0)) in one pass: per cell the
// flow-rate term of the predicted u, the projection of u, v, w (which reads
// only phi's neighbours), then the flow-rate term of the projected u.  The
// sums run in the reduction kernel's own order, so qvol(2) and qvol(0) are
// bitwise those of two separate qvolcalc launches.
struct UcalcQvolTerm {
    __device__ void operator()(const KP &p, int i, int j, int k, double *w) const {
        const DGrid &g = p.g;
        const long long q = g.ix(i, j, k);
        const double dtc = p.S->dtconst;
        const double *phi = p.f.phi;
        w[0] = p.f.u[q] * p.f.wq[q];
        const double ph = phi[q];
        if (i >= g.i_bgpx) p.f.u[q] = p.f.u[q] - dtc * (ph - phi[g.ix(g.imv[i], j, k)]) * g.c2cxi[i];
        if (j >= 2) p.f.v[q] = p.f.v[q] - dtc * (ph - phi[q - g.sx]) * g.c2cyi[j];
        if (k >= g.k_bgpz) p.f.w[q] = p.f.w[q] - dtc * (ph - phi[g.ix(i, j, g.kmv[k])]) * g.c2czi[k];
        w[1] = p.f.u[q] * p.f.wq[q];
    }
};
struct UcalcQvolFinal {
    __device__ void operator()(const KP &p, const double *o) const { p.S->qvol[2] = o[0]; p.S->qvol[0] = o[1]; }
};

static void ucalc_interior(lesgpu_case *c, bool with_qvol) {
    Box b = interior(c->kp.g);
    if (with_qvol) reduce<2, false>(c, b, UcalcQvolTerm{}, UcalcQvolFinal{});
    else k_ucalc<<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b);
}

// prdic_adj_uvw(0), slv_mmtm.f90:1746-1857: x, then y, then z
void launch_ghost_uvw(lesgpu_case *c) {
    const DGrid &g = c->kp.g;
    DFields &f = c->kp.f;
    if (c->kp.c.xprdic == 1) {
        GhostSpec s[3] = {{f.u, 0, g.n2, 0, g.n3}, {f.v, 1, g.n2, 0, g.n3}, {f.w, 0, g.n2, 1, g.n3}};
        ghost(c, 0, s, 3);
    }
    if (c->kp.c.yprdic == 1) {
        GhostSpec s[3] = {{f.u, 0, g.n1, 1, g.n3}, {f.v, 0, g.n1, 0, g.n3}, {f.w, 1, g.n1, 0, g.n3}};
        ghost(c, 1, s, 3);
    }
    if (c->kp.c.zprdic == 1) {
        GhostSpec s[3] = {{f.u, 1, g.n1, 0, g.n2}, {f.v, 0, g.n1, 1, g.n2}, {f.w, 0, g.n1, 0, g.n2}};
        ghost(c, 2, s, 3);
    }
}

// ------------------------------------------------------------------- pcalc
// pcalc, slv_auxi.f90:419-493
struct PhirefTerm {
    __device__ void operator()(const KP &p, int i, int j, int k, double *w) const {
        w[0] = p.f.phi[p.g.ix(p.g.n1m, j, k)] * p.g.f2fy[j] * p.g.f2fz[k];
    }
};
struct PhirefFinal {
    __device__ void operator()(const KP &p, const double *o) const { p.S->phiref = o[0] / (p.g.yl * p.g.zl); }
};

__global__ void __launch_bounds__(kThreads) k_pcalc(KP p, Box b) {
    long long n = b.count();
    const DGrid &g = p.g;
    // 1/re (formed once) in place of a per-cell division: an FP64 division
    // is some ten operations on the narrow FP64 pipe
    double dtc = p.S->dtconst, phiref = p.S->phiref, rei = p.c.rei_d;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        b.at(t, i, j, k);
        long long q = g.ix(i, j, k);
        double pn = p.f.p[q] + p.f.phi[q] - 0.5 * dtc * p.f.divgsum[q] * rei;
        p.f.p[q] = pn - phiref;
    }
}

// ucalc then pcalc.  pcalc reads p, phi and divgsum but no velocity ghost,
// so the periodic ghost copies of u, v, w (ucalc, slv_auxi.f90:360-412) and of
// p (pcalc, :470-490) run after both interiors, the four arrays sharing one
// launch per direction; each array still gets z first, then x.
void launch_ucalc_pcalc(lesgpu_case *c, bool with_qvol) {
    const DGrid &g = c->kp.g;
    ucalc_interior(c, with_qvol);
    reduce<1, false>(c, Box{1, 1, 1, 1, g.n2m, g.n3m}, PhirefTerm{}, PhirefFinal{});
    Box b = interior(g);
    k_pcalc<<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b);
    DFields &f = c->kp.f;
    if (c->kp.c.zprdic == 1) {
        GhostSpec s[4] = {{f.u, 1, g.n1, 0, g.n2}, {f.v, 0, g.n1, 1, g.n2}, {f.w, 0, g.n1, 0, g.n2}, {f.p, 1, g.n1m, 1, g.n2m}};
        ghost(c, 2, s, 4);
    }
    if (c->kp.c.xprdic == 1) {
        GhostSpec s[4] = {{f.u, 0, g.n2, 0, g.n3}, {f.v, 1, g.n2, 0, g.n3}, {f.w, 0, g.n2, 1, g.n3}, {f.p, 1, g.n2m, 1, g.n3m}};
        ghost(c, 0, s, 4);
    }
}

// ------------------------------------------------------- end-of-step checks
struct DivTerm {   // convergence_check, misc_init.f90:1047-1077
    __device__ void operator()(const KP &p, int i, int j, int k, double *w) const {
        const DGrid &g = p.g;
        long long q = g.ix(i, j, k);
        double d1 = (p.f.u[q + 1] - p.f.u[q]) * g.f2fxi[i];
        double d2 = (p.f.v[q + g.sx] - p.f.v[q]) * g.f2fyi[j];
        double d3 = (p.f.w[q + g.sxy] - p.f.w[q]) * g.f2fzi[k];
        double dv = (p.c.masson == 1) ? d1 + d2 + d3 - p.f.qmass[q] : d1 + d2 + d3;
        w[0] = fabs(dv);
        w[1] = fabs(p.f.qmass[q]);
        double fin = p.f.u[q] + p.f.v[q] + p.f.w[q] + p.f.p[q];
        w[2] = isfinite(fin) ? 0.0 : 1.0;
    }
};
// the last block also advances time (k_time_advance's work; the divergence
// terms do not read it), one launch fewer per step
struct DivFinal {
    __device__ void operator()(const KP &p, const double *o) const {
        p.S->time = p.S->time + p.S->dt;
        p.S->dvmax = o[0];
        if (p.c.ibmon == 1 && p.c.masson == 1) p.S->qmmax = o[1];
        if (o[2] > 0.0 || !isfinite(o[0])) p.S->err |= 2;
    }
};
void launch_advance_and_convergence(lesgpu_case *c) { reduce<3, true>(c, interior(c->kp.g), DivTerm{}, DivFinal{}); }

// writehistory's bulk quantities, misc_hist.f90:73-181: the flow rate and
// the fluid cells' temperature sums in one pass; the solid cells' sums
// (temperature inside bodies) in a second pass only when some cell centre
// lies inside a body -- carried through one pass they cost it half its time
// on bodiless cases, where they are zero.
struct BulkTerm {
    __device__ void operator()(const KP &p, int i, int j, int k, double *w) const {
        const DGrid &g = p.g;
        long long q = g.ix(i, j, k);
        double cv = g.c2cx[i] * g.f2fy[j] * g.f2fz[k];
        bool flu = p.f.fb_u[q] >= 1.0e-10;
        w[0] = flu ? p.f.u[q] * cv : 0.0;
        w[1] = flu ? cv : 0.0;
        w[2] = w[3] = 0.0;
        if (p.c.ihtrans == 1 && p.f.fb_c[q] >= 1.0e-10) { w[2] = cv; w[3] = p.f.t[q] * cv; }
    }
};
struct BulkSolidTerm {
    __device__ void operator()(const KP &p, int i, int j, int k, double *w) const {
        const DGrid &g = p.g;
        long long q = g.ix(i, j, k);
        w[0] = w[1] = 0.0;
        if (p.f.fb_c[q] < 1.0e-10) {
            double cv = g.c2cx[i] * g.f2fy[j] * g.f2fz[k];
            w[0] = cv;
            w[1] = p.f.t[q] * cv;
        }
    }
};
struct BulkFinal {
    int solid;      // the solid pass follows (else the solid bulk temperature is 0)
    __device__ void operator()(const KP &p, const double *o) const {
        DScal *S = p.S;
        S->ubulk = o[1] > 0.0 ? o[0] / o[1] : 0.0;
        S->qflux = o[0] / p.g.xl;
        S->tbulk_fluid = o[2] > 0.0 ? o[3] / o[2] : 0.0;
        if (!solid) S->tbulk_solid = 0.0;
    }
};
struct BulkSolidFinal {
    __device__ void operator()(const KP &p, const double *o) const {
        p.S->tbulk_solid = o[0] > 0.0 ? o[1] / o[0] : 0.0;
    }
};
void launch_bulk_diag(lesgpu_case *c) {
    const bool solid = c->kp.c.ihtrans == 1 && c->bulk_solid;
    reduce<4, false>(c, interior(c->kp.g), BulkTerm{}, BulkFinal{solid ? 1 : 0});
    if (solid) reduce<2, false>(c, interior(c->kp.g), BulkSolidTerm{}, BulkSolidFinal{});
}


}  // namespace lg
