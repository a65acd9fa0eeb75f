// Temperature equation around the fused rhs_t kernel: the bulk velocity of
// the decomposition source (slv_engy.f90:63-89), the recycling / periodic
// ghost update prdic_adj_t (:637-740), retrv_t (:612-634) and the wall
// conditions wallbc_t (:743-812).
#include "lesgpu_internal.cuh"

namespace lg {

struct UbulkTerm {
    __device__ void operator()(const KP &p, int i, int j, int k, double *w) const {
        const long long q = p.g.ix(i, j, k);
        const double cv = p.f.wb[q];     // c2cx f2fy f2fz over the fluid cells, else 0
        w[0] = cv;
        w[1] = 0.5 * (p.f.u[q] + p.f.u[q + 1]) * cv;
    }
};
struct UbulkFinal {
    __device__ void operator()(const KP &p, const double *o) const {
        double ub;
        if (o[0] > 1.0e-12) ub = o[1] / o[0];
        else if (fabs(p.c.udrv_i) > 1.0e-12) ub = p.c.udrv_i;
        else ub = 1.0;
        p.S->u_bulk_t = ub;
    }
};
__global__ void k_set_ubulk_one(KP p) { p.S->u_bulk_t = 1.0; }

// tvolcalc(tvol(1)) and the bulk velocity in one reduction (both read every
// interior cell; each sum keeps the order of its own launch, bitwise)
struct TvolUbulkTerm {
    __device__ void operator()(const KP &p, int i, int j, int k, double *w) const {
        const long long q = p.g.ix(i, j, k);
        w[0] = p.f.t[q] * p.f.wt[q];
        UbulkTerm{}(p, i, j, k, w + 1);
    }
};
struct TvolUbulkFinal {
    __device__ void operator()(const KP &p, const double *o) const {
        p.S->tvol[1] = o[0];
        UbulkFinal{}(p, o + 1);
    }
};

void launch_rhs_t(lesgpu_case *c, int msub, bool with_tvol) {
    const DGrid &g = c->kp.g;
    const Box b{1, 1, 1, g.n1m, g.n2m, g.n3m};
    if (c->kp.c.idecomp == 1) {
        if (with_tvol) reduce<3, false>(c, b, TvolUbulkTerm{}, TvolUbulkFinal{});
        else reduce<2, false>(c, b, UbulkTerm{}, UbulkFinal{});
    } else {
        if (with_tvol) launch_tvolcalc(c, 1);
        k_set_ubulk_one<<<1, 1, 0, c->stream>>>(c->kp);
    }
    launch_rhs_t_kernel(c, msub);
}

// recycling scaling of prdic_adj_t for X-periodic flows without the
// decomposition (slv_engy.f90:663-711)
struct RecycTerm {
    __device__ void operator()(const KP &p, int i, int j, int k, double *w) const {
        const DGrid &g = p.g;
        long long q = g.ix(g.n1m, j, k);
        if (p.f.fb_c[q] >= 1.0e-10) {
            w[0] = p.f.u[q] * g.f2fy[j] * g.f2fz[k];
            w[1] = p.f.t[q] * p.f.u[q] * g.f2fy[j] * g.f2fz[k];
        } else {
            w[0] = 0.0;
            w[1] = 0.0;
        }
    }
};
struct RecycFinal {
    __device__ void operator()(const KP &p, const double *o) const {
        double tw = p.c.tsol_i, tbi = p.c.tflu_i;
        double md = o[0], tbo = o[1];
        tbo = fabs(md) > 1.0e-14 ? tbo / md : tbi;
        double numer = tw - tbi, denom = tw - tbo, ratio;
        if (fabs(numer) <= 1.0e-14) ratio = 1.0;
        else if (fabs(denom) > 1.0e-14) { ratio = numer / denom; if (fabs(ratio) <= 1.0e-14) ratio = 1.0; }
        else ratio = 1.0;
        p.S->phiref = ratio;      // reused slot: the ratio of this substep
    }
};
__global__ void k_recyc_apply(KP p) {
    const DGrid &g = p.g;
    double tw = p.c.tsol_i, ratio = p.S->phiref;
    long long n = (long long)(g.n2 + 1) * (g.n3 + 1);
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        int j = (int)(t % (g.n2 + 1)), k = (int)(t / (g.n2 + 1));
        p.f.t[g.ix(0, j, k)] = tw - (tw - p.f.t[g.ix(g.n1m, j, k)]) * ratio;
        p.f.t[g.ix(g.n1, j, k)] = tw - (tw - p.f.t[g.ix(1, j, k)]) / ratio;
    }
}

// wallbc_t, one direction per launch (x, then y, then z)
__global__ void k_wallbc_t(KP p, int dir) {
    const DGrid &g = p.g;
    const DCfg &c = p.c;
    double *t = p.f.t;
    if (dir == 0) {
        long long n = (long long)(g.n2 + 1) * (g.n3 + 1);
        for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += (long long)gridDim.x * blockDim.x) {
            int j = (int)(s % (g.n2 + 1)), k = (int)(s / (g.n2 + 1));
            t[g.ix(0, j, k)] = (p.f.fb_c[g.ix(0, j, k)] <= 1.0e-10) ? c.tsol_i : c.tflu_i;
        }
    } else if (dir == 1) {
        long long n = (long long)(g.n1 + 1) * (g.n3 + 1);
        for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += (long long)gridDim.x * blockDim.x) {
            int i = (int)(s % (g.n1 + 1)), k = (int)(s / (g.n1 + 1));
            if (c.bc_t_ybtm == 0) t[g.ix(i, 0, k)] = c.val_t_ybtm;
            else if (c.bc_t_ybtm == 1) t[g.ix(i, 0, k)] = t[g.ix(i, 1, k)] - c.val_t_ybtm / g.c2cyi[1];
            if (c.bc_t_ytop == 0) t[g.ix(i, g.n2, k)] = c.val_t_ytop;
            else if (c.bc_t_ytop == 1) t[g.ix(i, g.n2, k)] = t[g.ix(i, g.n2m, k)] + c.val_t_ytop / g.c2cyi[g.n2];
        }
    } else {
        long long n = (long long)(g.n1 + 1) * (g.n2 + 1);
        for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += (long long)gridDim.x * blockDim.x) {
            int i = (int)(s % (g.n1 + 1)), j = (int)(s / (g.n1 + 1));
            if (c.bc_t_zbtm == 0) t[g.ix(i, j, 0)] = c.val_t_zbtm;
            else if (c.bc_t_zbtm == 1) t[g.ix(i, j, 0)] = t[g.ix(i, j, 1)] - c.val_t_zbtm / g.c2czi[1];
            if (c.bc_t_ztop == 0) t[g.ix(i, j, g.n3)] = c.val_t_ztop;
            else if (c.bc_t_ztop == 1) t[g.ix(i, j, g.n3)] = t[g.ix(i, j, g.n3m)] + c.val_t_ztop / g.c2czi[g.n3];
        }
    }
}

__global__ void k_retrv_t(KP p) {
    const DGrid &g = p.g;
    long long n = (long long)g.n2m * g.n3m;
    for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += (long long)gridDim.x * blockDim.x) {
        int j = 1 + (int)(s % g.n2m), k = 1 + (int)(s / g.n2m);
        p.f.t[g.ix(g.n1, j, k)] = p.f.tout[j + (long long)(g.n2 + 1) * k];
    }
}

// retrv_t (when X is not periodic), prdic_adj_t and wallbc_t
void launch_energy_bc(lesgpu_case *c) {
    const DGrid &g = c->kp.g;
    const DCfg &cf = c->kp.c;
    double *t = c->kp.f.t;
    if (cf.xprdic == 0) k_retrv_t<<<blocks_for((long long)g.n2m * g.n3m), kThreads, 0, c->stream>>>(c->kp);
    if (cf.xprdic == 1) {
        if (cf.idecomp == 1) {
            GhostSpec s[1] = {{t, 0, g.n2, 0, g.n3}};
            ghost(c, 0, s, 1);
        } else {
            reduce<2, false>(c, Box{1, 1, 1, 1, g.n2m, g.n3m}, RecycTerm{}, RecycFinal{});
            k_recyc_apply<<<blocks_for((long long)(g.n2 + 1) * (g.n3 + 1)), kThreads, 0, c->stream>>>(c->kp);
        }
    }
    if (cf.yprdic == 1) { GhostSpec s[1] = {{t, 0, g.n1, 0, g.n3}}; ghost(c, 1, s, 1); }
    if (cf.zprdic == 1) { GhostSpec s[1] = {{t, 0, g.n1, 0, g.n2}}; ghost(c, 2, s, 1); }
    if (cf.xprdic == 0) k_wallbc_t<<<blocks_for((long long)(g.n2 + 1) * (g.n3 + 1)), kThreads, 0, c->stream>>>(c->kp, 0);
    if (cf.yprdic == 0) k_wallbc_t<<<blocks_for((long long)(g.n1 + 1) * (g.n3 + 1)), kThreads, 0, c->stream>>>(c->kp, 1);
    if (cf.zprdic == 0) k_wallbc_t<<<blocks_for((long long)(g.n1 + 1) * (g.n2 + 1)), kThreads, 0, c->stream>>>(c->kp, 2);
}

}  // namespace lg
