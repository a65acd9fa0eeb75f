// C ABI of the GB300 LES time-step library (include/lesgpu.h).
//
// lesgpu_create allocates the whole solver state in device memory and builds
// the init-time tables of the reference (lhsinit slv_mmtm.f90:180,
// sgsfilterinit sgs.f90:2, poisinit of the Poisson solver, and the body
// function values that the reference re-evaluates inside its reductions).
// lesgpu_step enqueues one time step (solver.f90:85-151 plus the per-step
// checks) on the case's stream; from the second eligible step on, the step
// is replayed from a captured CUDA graph, so one step costs one graph launch
// and one 400-byte read-back of the step scalars.
#include "lesgpu_internal.cuh"
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <vector>

using namespace lg;

namespace lg {
void launch_sgs_post(lesgpu_case *c);
void launch_sgs_t_post(lesgpu_case *c);
}

// ------------------------------------------------------------------ helpers
namespace {

struct Alloc {
    std::vector<void *> ptrs;
    bool ok = true;
    template <class T> T *get(size_t n) {
        void *p = nullptr;
        if (n == 0) n = 1;
        if (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess) { ok = false; return nullptr; }
        cudaMemset(p, 0, n * sizeof(T));
        ptrs.push_back(p);
        return (T *)p;
    }
};

// FP32 mirrors of the mixed form: source and destination of every 3-D
// mirror, in the order of the kMir* bits
struct MirState {
    const double *src[20];
    float *dst[20];
    int n = 0;
};

struct CaseExtra {
    Alloc alloc;
    MirState mir;
};

double funcbody(const lesgpu_body &b, double x, double y, double z) {
    switch (b.kind) {
    case LESGPU_BODY_CHANNEL: return (1.0 + b.p0) - fabs(y);
    case LESGPU_BODY_CYLINDER: { double dx = x - b.cx, dy = y - b.cy; return sqrt(dx * dx + dy * dy) - b.r; }
    case LESGPU_BODY_SPHERE: { double dx = x - b.cx, dy = y - b.cy, dz = z - b.cz; return sqrt(dx * dx + dy * dy + dz * dz) - b.r; }
    case LESGPU_BODY_SQUARE: { double ax = fabs(x - b.cx), ay = fabs(y - b.cy); return (ax > ay ? ax : ay) - b.r; }
    default: return 1.0;
    }
}

template <class T> T *upload(Alloc &A, const T *h, size_t n) {
    T *d = A.get<T>(n);
    if (d && h) cudaMemcpy(d, h, n * sizeof(T), cudaMemcpyHostToDevice);
    return d;
}

// (0:n) vector -> device array of n+2
double *vec0(Alloc &A, const double *src, long long n) {
    std::vector<double> h(n + 2, 0.0);
    for (long long i = 0; i <= n; i++) h[i] = src[i];
    return upload(A, h.data(), h.size());
}
// (1:n) vector -> device array of n+2 with Fortran index
double *vec1(Alloc &A, const double *src, long long n) {
    std::vector<double> h(n + 2, 0.0);
    for (long long i = 1; i <= n; i++) h[i] = src[i - 1];
    return upload(A, h.data(), h.size());
}
int *ivec1(Alloc &A, const int64_t *src, long long n) {
    std::vector<int> h(n + 2, 0);
    for (long long i = 1; i <= n; i++) h[i] = (int)src[i - 1];
    return upload(A, h.data(), h.size());
}

int check_config(const lesgpu_config *c, const lesgpu_grid *g) {
    if (g->n1 != g->n1m + 1 || g->n2 != g->n2m + 1 || g->n3 != g->n3m + 1) return LESGPU_ERR_ARG;
    if (g->n1m < 2 || g->n2m < 2 || g->n3m < 1) return LESGPU_ERR_ARG;
    if ((long long)(g->n1 + 1) * (g->n2 + 1) * (g->n3 + 1) > (1LL << 40)) return LESGPU_ERR_ARG;
    if (c->precision != LESGPU_PREC_FP64 && c->precision != LESGPU_PREC_MIXED) return LESGPU_ERR_ARG;
    if (c->poisson != LESGPU_POISSON_FTFT && c->poisson != LESGPU_POISSON_Z_FT && c->poisson != LESGPU_POISSON_MGRD &&
        c->poisson != LESGPU_POISSON_X_FT)
        return LESGPU_ERR_UNSUPPORTED;
    if (c->imovingon != 0) return LESGPU_ERR_UNSUPPORTED;     // moving bodies: not built
    // poiss_ftft transforms x and z: both must be periodic
    if (c->poisson == LESGPU_POISSON_FTFT && (c->xprdic != 1 || c->zprdic != 1)) return LESGPU_ERR_CONFIG;
    if (c->iles == 1 && c->insmdl != 1) return LESGPU_ERR_CONFIG;   // sgs.f90:314 stops
    if (c->ihtrans == 1 && c->iles == 1 && c->itemdl != 0) return LESGPU_ERR_CONFIG;
    if (c->filter < 1 || c->filter > 3) return LESGPU_ERR_CONFIG;
    if (c->ich != 0 && c->bc_ybtm != 0 && c->bc_ytop != 0 && c->bc_zbtm != 0 && c->bc_ztop != 0)
        return LESGPU_ERR_CONFIG;                                    // meanpg stops
    if (c->idecomp == 1) {                                            // check_idecomp_input
        if (c->xprdic != 1 || c->bc_ybtm != 0 || c->bc_ytop != 0 || c->bc_t_ybtm != 0 || c->bc_t_ytop != 0)
            return LESGPU_ERR_CONFIG;
        if (fabs(c->val_t_ybtm) > 1e-12 || fabs(c->val_t_ytop) > 1e-12) return LESGPU_ERR_CONFIG;
    }
    return 0;
}

int cuda_rc(cudaError_t e) { return e == cudaSuccess ? 0 : LESGPU_ERR_CUDA; }

}  // namespace

// ------------------------------------------------------------- FP32 mirrors
namespace lg {
struct MirBatch {
    const double *src[20];
    float *dst[20];
    int n;
};

// FP64 -> FP32 (round to nearest, as the per-load conversions it replaces)
__global__ void __launch_bounds__(kThreads) k_mirror(MirBatch b, long long nt) {
    const long long npair = nt >> 1;
    const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x, st = (long long)gridDim.x * blockDim.x;
    for (int a = 0; a < b.n; a++) {
        const double2 *s = reinterpret_cast<const double2 *>(b.src[a]);
        float2 *d = reinterpret_cast<float2 *>(b.dst[a]);
        for (long long q = t0; q < npair; q += st) {
            const double2 x = s[q];
            d[q] = make_float2((float)x.x, (float)x.y);
        }
        if ((nt & 1) && t0 == 0) b.dst[a][nt - 1] = (float)b.src[a][nt - 1];
    }
}

// Refresh the FP32 mirrors of the requested sets that are out of date.
void launch_mirror(lesgpu_case *c, unsigned sets) {
    const MirState &ms = ((CaseExtra *)c->dmem_pool)->mir;
    if (ms.n == 0) return;                       // FP64 form
    sets &= c->mir_dirty;
    c->mir_dirty &= ~sets;
    MirBatch b;
    b.n = 0;
    auto take = [&](int first, int count) {
        for (int q = first; q < first + count; q++) { b.src[b.n] = ms.src[q]; b.dst[b.n] = ms.dst[q]; b.n++; }
    };
    if (sets & kMirU) take(0, 1);
    if (sets & kMirV) take(1, 1);
    if (sets & kMirW) take(2, 1);
    if (sets & kMirP) take(3, 1);
    if (sets & kMirT) take(4, 1);
    if (sets & kMirNu) take(5, 4);
    if (sets & kMirAl) take(9, 4);
    if (sets & kMirConj) take(13, 7);
    if (b.n == 0) return;
    const long long nt = c->kp.g.nt;
    int nb = blocks_for(nt / 2 + 1);
    if (nb > 4 * 152) nb = 4 * 152;
    k_mirror<<<nb, kThreads, 0, c->stream>>>(b, nt);
}
}  // namespace lg

// ------------------------------------------------------------------ create
extern "C" int lesgpu_create(const lesgpu_config *cfg, const lesgpu_grid *g, lesgpu_case **out) {
    if (!cfg || !g || !out) return LESGPU_ERR_ARG;
    *out = nullptr;
    int rc = check_config(cfg, g);
    if (rc) return rc;
    lesgpu_case *c = (lesgpu_case *)calloc(1, sizeof(lesgpu_case));
    if (!c) return LESGPU_ERR_OOM;
    CaseExtra *X = new CaseExtra();
    c->dmem_pool = X;
    c->cfg = *cfg;
    c->use_graph = 1;
    c->mir_dirty = ~0u;
    Alloc &A = X->alloc;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) { lesgpu_destroy(c); return LESGPU_ERR_CUDA; }

    DGrid &d = c->kp.g;
    d.n1 = (int)g->n1; d.n2 = (int)g->n2; d.n3 = (int)g->n3;
    d.n1m = (int)g->n1m; d.n2m = (int)g->n2m; d.n3m = (int)g->n3m;
    d.n1mh = d.n1m / 2 + 1; d.n3mh = d.n3m / 2 + 1;
    d.sx = d.n1 + 1; d.sxy = d.sx * (d.n2 + 1); d.nt = d.sxy * (d.n3 + 1);
    d.xl = g->xl; d.yl = g->yl; d.zl = g->zl;
    d.x = vec1(A, g->x, d.n1); d.y = vec1(A, g->y, d.n2); d.z = vec1(A, g->z, d.n3);
    d.xmp = vec0(A, g->xmp, d.n1); d.ymp = vec0(A, g->ymp, d.n2); d.zmp = vec0(A, g->zmp, d.n3);
    d.f2fx = vec0(A, g->f2fx, d.n1); d.f2fy = vec0(A, g->f2fy, d.n2); d.f2fz = vec0(A, g->f2fz, d.n3);
    d.f2fxi = vec0(A, g->f2fxi, d.n1); d.f2fyi = vec0(A, g->f2fyi, d.n2); d.f2fzi = vec0(A, g->f2fzi, d.n3);
    d.c2cx = vec0(A, g->c2cx, d.n1); d.c2cy = vec0(A, g->c2cy, d.n2); d.c2cz = vec0(A, g->c2cz, d.n3);
    d.c2cxi = vec0(A, g->c2cxi, d.n1); d.c2cyi = vec0(A, g->c2cyi, d.n2); d.c2czi = vec0(A, g->c2czi, d.n3);
    d.ipv = ivec1(A, g->ipv, d.n1m); d.jpv = ivec1(A, g->jpv, d.n2m); d.kpv = ivec1(A, g->kpv, d.n3m);
    d.imv = ivec1(A, g->imv, d.n1m); d.jmv = ivec1(A, g->jmv, d.n2m); d.kmv = ivec1(A, g->kmv, d.n3m);
    d.fixil = ivec1(A, g->fixil, d.n1m); d.fixjl = ivec1(A, g->fixjl, d.n2m); d.fixkl = ivec1(A, g->fixkl, d.n3m);
    d.fixiu = ivec1(A, g->fixiu, d.n1m); d.fixju = ivec1(A, g->fixju, d.n2m); d.fixku = ivec1(A, g->fixku, d.n3m);
    d.i_bgpx = cfg->xprdic == 1 ? 1 : 2;
    d.j_bgpy = cfg->yprdic == 1 ? 1 : 2;
    d.k_bgpz = cfg->zprdic == 1 ? 1 : 2;

    DCfg &k = c->kp.c;
    k.re = cfg->re; k.pr = cfg->pr; k.gr = cfg->gr; k.udrv_i = cfg->udrv_i; k.tflu_i = cfg->tflu_i; k.tsol_i = cfg->tsol_i;
    k.val_t_ybtm = cfg->val_t_ybtm; k.val_t_ytop = cfg->val_t_ytop; k.val_t_zbtm = cfg->val_t_zbtm; k.val_t_ztop = cfg->val_t_ztop;
    k.resid1 = cfg->resid1; k.csgsts = cfg->csgsts; k.csgshf = cfg->csgshf; k.cflfac = cfg->cflfac; k.dt_size = cfg->dt_size;
    k.ptb_tst = cfg->ptb_tst; k.avg_tst = cfg->avg_tst; k.tend = cfg->tend;
    k.grdir = (int)cfg->grdir; k.iles = (int)cfg->iles; k.ihtrans = (int)cfg->ihtrans; k.ich = (int)cfg->ich;
    k.iconjg = (int)cfg->iconjg; k.idecomp = (int)cfg->idecomp; k.idvmon = (int)cfg->idvmon; k.filter = (int)cfg->filter;
    k.ibmon = (int)cfg->ibmon; k.masson = (int)cfg->masson; k.imovingon = (int)cfg->imovingon; k.iread = (int)cfg->iread;
    k.xprdic = (int)cfg->xprdic; k.yprdic = (int)cfg->yprdic; k.zprdic = (int)cfg->zprdic;
    k.bc_ybtm = (int)cfg->bc_ybtm; k.bc_ytop = (int)cfg->bc_ytop; k.bc_zbtm = (int)cfg->bc_zbtm; k.bc_ztop = (int)cfg->bc_ztop;
    k.bc_t_ybtm = (int)cfg->bc_t_ybtm; k.bc_t_ytop = (int)cfg->bc_t_ytop; k.bc_t_zbtm = (int)cfg->bc_t_zbtm; k.bc_t_ztop = (int)cfg->bc_t_ztop;
    k.idtopt = (int)cfg->idtopt;
    {
        const double re = cfg->re, pr = cfg->pr, iles = (double)cfg->iles;
        const double re_f = (double)(float)re;
        k.rei_d = 1.0 / re; k.rei_f = (float)(1.0 / re);
        k.inv_repr_d = 1.0 / (re * pr); k.inv_repr_f = (float)(1.0 / (re * pr));
        k.gterm = cfg->gr / (re * re);
        k.adi_cd[0] = iles * re; k.adi_cd[1] = 2.0 * iles * re; k.adi_cd[2] = iles * re * pr;
        k.adi_cf[0] = (float)(iles * re_f); k.adi_cf[1] = (float)(2.0 * iles * re_f); k.adi_cf[2] = (float)(iles * re_f * pr);
    }

    size_t nt = (size_t)d.nt;
    DFields &f = c->kp.f;
    f.u = A.get<double>(nt); f.v = A.get<double>(nt); f.w = A.get<double>(nt);
    f.p = A.get<double>(nt); f.t = A.get<double>(nt);
    for (int l = 0; l < 4; l++) { f.rhs1[l] = A.get<double>(nt); f.rk3o[l] = A.get<double>(nt); f.rk3oo[l] = A.get<double>(nt); }
    if (cfg->precision == LESGPU_PREC_MIXED)
        for (int l = 0; l < 4; l++) { f.rk3of[l] = A.get<float>(nt); f.rk3oof[l] = A.get<float>(nt); }
    f.nusgs = A.get<double>(nt); f.alsgs = A.get<double>(nt);
    for (int l = 0; l < 3; l++) { f.nusgs1[l] = A.get<double>(nt); f.alsgs1[l] = A.get<double>(nt); }
    f.qmass = A.get<double>(nt); f.divgsum = A.get<double>(nt); f.phi = A.get<double>(nt);
    if (cfg->iavg == 1) f.avg = A.get<double>(nt * LESGPU_NAVG);
    int nscr = (cfg->iles == 1) ? 33 : 9;   // ADI uses scr[0..8] (three components), SGS scr[3..32]
    for (int s = 0; s < nscr; s++) f.scr[s] = A.get<double>(nt);
    f.part = A.get<double>((size_t)(kRedBlocks + 1) * kMaxRed);
    f.red_count = A.get<unsigned>(1);
    size_t np = (size_t)(d.n2 + 1) * (d.n3 + 1);
    f.uout = A.get<double>(np); f.vout = A.get<double>(np); f.wout = A.get<double>(np); f.tout = A.get<double>(np);
    f.duout = A.get<double>(np); f.dvout = A.get<double>(np); f.dwout = A.get<double>(np); f.dtout = A.get<double>(np);

    // conjugate / LES defaults (conjg_allo, les_allo): c* = k* = 1, omega = nwall = 1
    {
        std::vector<double> one(nt, 1.0);
        std::vector<int> ione(nt, 1);
        f.cstar = upload(A, one.data(), nt);
        for (int l = 0; l < 6; l++) f.kstar[l] = upload(A, one.data(), nt);
        f.omega = upload(A, ione.data(), nt);
        f.nwall = upload(A, ione.data(), nt);
    }
    // body function at the u points and at the cell centres
    {
        std::vector<double> fbu(nt), fbc(nt);
        for (long long kk = 0; kk <= d.n3; kk++)
            for (long long jj = 0; jj <= d.n2; jj++)
                for (long long ii = 0; ii <= d.n1; ii++) {
                    double xi = ii >= 1 ? g->x[ii - 1] : 0.0;
                    size_t q = (size_t)(ii + d.sx * jj + d.sxy * kk);
                    fbu[q] = funcbody(cfg->body, xi, g->ymp[jj], g->zmp[kk]);
                    fbc[q] = funcbody(cfg->body, g->xmp[ii], g->ymp[jj], g->zmp[kk]);
                }
        f.fb_u = upload(A, fbu.data(), nt);
        f.fb_c = upload(A, fbc.data(), nt);
        c->bulk_solid = 0;
        for (long long kk = 1; kk <= d.n3 - 1 && !c->bulk_solid; kk++)
            for (long long jj = 1; jj <= d.n2 - 1 && !c->bulk_solid; jj++)
                for (long long ii = 1; ii <= d.n1 - 1; ii++)
                    if (fbc[(size_t)(ii + d.sx * jj + d.sxy * kk)] < 1.0e-10) { c->bulk_solid = 1; break; }
        f.wq = A.get<double>(nt); f.wb = A.get<double>(nt); f.wt = A.get<double>(nt);
        // nutinterpol's edge weights (sgs.f90:1002-1040), 4 per edge line
        {
            const long long N1 = d.n1 + 1, N2 = d.n2 + 1, N3 = d.n3 + 1;
            std::vector<double> e1(4 * N2 * N3, 0.0), e2(4 * N3 * N1, 0.0), e3(4 * N1 * N2, 0.0);
            const double *cxi = g->c2cxi, *cyi = g->c2cyi, *czi = g->c2czi, *fx = g->f2fx, *fy = g->f2fy, *fz = g->f2fz;
            for (long long kk = 1; kk < N3; kk++)
                for (long long jj = 1; jj < N2; jj++) {
                    const double W = cyi[jj] * czi[kk] * 0.25;
                    double *w = &e1[4 * (jj + N2 * kk)];
                    w[0] = W * fy[jj - 1] * fz[kk - 1]; w[1] = W * fy[jj - 1] * fz[kk];
                    w[2] = W * fy[jj] * fz[kk - 1];     w[3] = W * fy[jj] * fz[kk];
                }
            for (long long ii = 1; ii < N1; ii++)
                for (long long kk = 1; kk < N3; kk++) {
                    const double W = czi[kk] * cxi[ii] * 0.25;
                    double *w = &e2[4 * (kk + N3 * ii)];
                    w[0] = W * fz[kk - 1] * fx[ii - 1]; w[1] = W * fz[kk - 1] * fx[ii];
                    w[2] = W * fz[kk] * fx[ii - 1];     w[3] = W * fz[kk] * fx[ii];
                }
            for (long long jj = 1; jj < N2; jj++)
                for (long long ii = 1; ii < N1; ii++) {
                    const double W = cxi[ii] * cyi[jj] * 0.25;
                    double *w = &e3[4 * (ii + N1 * jj)];
                    w[0] = W * fx[ii - 1] * fy[jj - 1]; w[1] = W * fx[ii - 1] * fy[jj];
                    w[2] = W * fx[ii] * fy[jj - 1];     w[3] = W * fx[ii] * fy[jj];
                }
            f.ew1 = upload(A, e1.data(), e1.size());
            f.ew2 = upload(A, e2.data(), e2.size());
            f.ew3 = upload(A, e3.data(), e3.size());
        }
        // face points of heatflux (slv_auxi.f90:573-663)
        size_t nxz = (size_t)(d.n1 + 1) * (d.n3 + 1), nxy = (size_t)(d.n1 + 1) * (d.n2 + 1);
        std::vector<double> vb(nxz, 0.0), vt(nxz, 0.0), wb(nxy, 0.0), wt(nxy, 0.0);
        for (long long kk = 0; kk <= d.n3; kk++)
            for (long long ii = 0; ii <= d.n1; ii++) {
                vb[ii + (d.n1 + 1) * kk] = funcbody(cfg->body, g->xmp[ii], g->y[0], g->zmp[kk]);
                vt[ii + (d.n1 + 1) * kk] = funcbody(cfg->body, g->xmp[ii], g->y[d.n2 - 1], g->zmp[kk]);
            }
        for (long long jj = 0; jj <= d.n2; jj++)
            for (long long ii = 0; ii <= d.n1; ii++) {
                wb[ii + (d.n1 + 1) * jj] = funcbody(cfg->body, g->xmp[ii], g->ymp[jj], g->z[0]);
                wt[ii + (d.n1 + 1) * jj] = funcbody(cfg->body, g->xmp[ii], g->ymp[jj], g->z[d.n3 - 1]);
            }
        f.fb_vb = upload(A, vb.data(), nxz); f.fb_vt = upload(A, vt.data(), nxz);
        f.fb_wb = upload(A, wb.data(), nxy); f.fb_wt = upload(A, wt.data(), nxy);
    }
    // lhsinit (slv_mmtm.f90:180-249)
    {
        long long n1 = d.n1, n2 = d.n2, n3 = d.n3;
        std::vector<double> aiu(n1 + 2, 0), ciu(n1 + 2, 0), aivw(n1 + 2, 0), civw(n1 + 2, 0);
        std::vector<double> ajv(n2 + 2, 0), cjv(n2 + 2, 0), ajuw(n2 + 2, 0), cjuw(n2 + 2, 0);
        std::vector<double> akw(n3 + 2, 0), ckw(n3 + 2, 0), akuv(n3 + 2, 0), ckuv(n3 + 2, 0);
        auto C2CXI = [&](long long i) { return g->c2cxi[i]; };
        auto C2CYI = [&](long long j) { return g->c2cyi[j]; };
        auto C2CZI = [&](long long kk) { return g->c2czi[kk]; };
        for (long long i = d.i_bgpx; i <= d.n1m; i++) {
            long long im = g->imv[i - 1];
            aiu[i] = -C2CXI(i) * g->f2fxi[im];
            ciu[i] = -C2CXI(i) * g->f2fxi[i];
        }
        for (long long i = 1; i <= d.n1m; i++) {
            long long ip = g->ipv[i - 1];
            aivw[i] = -C2CXI(i) * g->f2fxi[i];
            civw[i] = -C2CXI(ip) * g->f2fxi[i];
        }
        for (long long j = d.j_bgpy; j <= d.n2m; j++) {
            long long jm = g->jmv[j - 1];
            ajv[j] = -C2CYI(j) * g->f2fyi[jm];
            cjv[j] = -C2CYI(j) * g->f2fyi[j];
        }
        for (long long j = 1; j <= d.n2m; j++) {
            long long jp = g->jpv[j - 1];
            ajuw[j] = -C2CYI(j) * g->f2fyi[j];
            cjuw[j] = -C2CYI(jp) * g->f2fyi[j];
        }
        for (long long kk = d.k_bgpz; kk <= d.n3m; kk++) {
            long long km = g->kmv[kk - 1];
            akw[kk] = -C2CZI(kk) * g->f2fzi[km];
            ckw[kk] = -C2CZI(kk) * g->f2fzi[kk];
        }
        for (long long kk = 1; kk <= d.n3m; kk++) {
            long long kp = g->kpv[kk - 1];
            akuv[kk] = -C2CZI(kk) * g->f2fzi[kk];
            ckuv[kk] = -C2CZI(kp) * g->f2fzi[kk];
        }
        f.aiu = upload(A, aiu.data(), aiu.size()); f.ciu = upload(A, ciu.data(), ciu.size());
        f.aivw = upload(A, aivw.data(), aivw.size()); f.civw = upload(A, civw.data(), civw.size());
        f.ajv = upload(A, ajv.data(), ajv.size()); f.cjv = upload(A, cjv.data(), cjv.size());
        f.ajuw = upload(A, ajuw.data(), ajuw.size()); f.cjuw = upload(A, cjuw.data(), cjuw.size());
        f.akw = upload(A, akw.data(), akw.size()); f.ckw = upload(A, ckw.data(), ckw.size());
        f.akuv = upload(A, akuv.data(), akuv.size()); f.ckuv = upload(A, ckuv.data(), ckuv.size());
    }
    // sgsfilterinit (sgs.f90:2-285): the 3-point weights cf?1
    {
        auto coefs = [&](const double *c2c, long long nm) {
            std::vector<double> cf(3 * (nm + 2), 0.0);
            if (nm != 1)
                for (long long i = 1; i <= nm; i++) {
                    double h1 = c2c[i], h2 = c2c[i + 1];
                    cf[3 * i + 0] = (2.0 * h1 - h2) / 6.0 / h1;
                    cf[3 * i + 1] = ((h1 + h2) * (h1 + h2)) / 6.0 / h1 / h2;
                    cf[3 * i + 2] = (2.0 * h2 - h1) / 6.0 / h2;
                }
            return cf;
        };
        auto cx = coefs(g->c2cx, d.n1m), cy = coefs(g->c2cy, d.n2m), cz = coefs(g->c2cz, d.n3m);
        f.cfx1 = upload(A, cx.data(), cx.size());
        f.cfy1 = upload(A, cy.data(), cy.size());
        f.cfz1 = upload(A, cz.data(), cz.size());
    }
    // IB placeholders (no forcing points until lesgpu_load_ibm)
    for (int l = 0; l < 4; l++) {
        f.ifc[l] = A.get<int>(1); f.jfc[l] = A.get<int>(1); f.kfc[l] = A.get<int>(1); f.intpindx[l] = A.get<int>(3);
        f.geomfac[l] = A.get<double>(27); f.fcv[l] = A.get<double>(1); f.fcvavg[l] = A.get<double>(1);
    }
    for (int l = 0; l < 3; l++) f.dudtr[l] = A.get<double>(1);
    for (int l = 0; l < 4; l++) f.ibtarg[l] = A.get<double>(1);
    f.inz = A.get<int>(1); f.jnz = A.get<int>(1); f.knz = A.get<int>(1);

    // stencil operand views (Mir<double> aliases the state) and, in the mixed
    // form, their FP32 mirrors: 1-D tables converted here, 3-D arrays
    // allocated here and filled by launch_mirror
    {
        Mir<double> &m = c->kp.md;
        m.u = f.u; m.v = f.v; m.w = f.w; m.p = f.p; m.t = f.t;
        m.nusgs = f.nusgs; m.alsgs = f.alsgs;
        for (int l = 0; l < 3; l++) { m.nusgs1[l] = f.nusgs1[l]; m.alsgs1[l] = f.alsgs1[l]; }
        m.cstar = f.cstar;
        for (int l = 0; l < 6; l++) m.kstar[l] = f.kstar[l];
        m.f2fx = d.f2fx; m.f2fy = d.f2fy; m.f2fz = d.f2fz; m.f2fxi = d.f2fxi; m.f2fyi = d.f2fyi; m.f2fzi = d.f2fzi;
        m.c2cxi = d.c2cxi; m.c2cyi = d.c2cyi; m.c2czi = d.c2czi;
        m.aiu = f.aiu; m.ciu = f.ciu; m.aivw = f.aivw; m.civw = f.civw; m.ajv = f.ajv; m.cjv = f.cjv;
        m.ajuw = f.ajuw; m.cjuw = f.cjuw; m.akw = f.akw; m.ckw = f.ckw; m.akuv = f.akuv; m.ckuv = f.ckuv;
        m.cfx1 = f.cfx1; m.cfy1 = f.cfy1; m.cfz1 = f.cfz1;
        auto flags = [&](const int64_t *src, long long n) {     // (1:n) int64 -> (0:n+1) double
            std::vector<double> h(n + 2, 0.0);
            for (long long q = 1; q <= n; q++) h[q] = (double)src[q - 1];
            return (const double *)upload(A, h.data(), h.size());
        };
        m.fixil = flags(g->fixil, d.n1m); m.fixiu = flags(g->fixiu, d.n1m);
        m.fixjl = flags(g->fixjl, d.n2m); m.fixju = flags(g->fixju, d.n2m);
        m.fixkl = flags(g->fixkl, d.n3m); m.fixku = flags(g->fixku, d.n3m);
        if (cfg->precision == LESGPU_PREC_MIXED) {
            Mir<float> &r = c->kp.mf;
            MirState &ms = X->mir;
            auto add = [&](const double *src, const float *&dst) {
                float *q = A.get<float>(nt);
                dst = q;
                ms.src[ms.n] = src; ms.dst[ms.n] = q; ms.n++;
            };
            // order = the kMir* bits: u v w p t | nusgs nusgs1(3) | alsgs alsgs1(3) | cstar kstar(6)
            add(f.u, r.u); add(f.v, r.v); add(f.w, r.w); add(f.p, r.p); add(f.t, r.t);
            add(f.nusgs, r.nusgs);
            for (int l = 0; l < 3; l++) add(f.nusgs1[l], r.nusgs1[l]);
            add(f.alsgs, r.alsgs);
            for (int l = 0; l < 3; l++) add(f.alsgs1[l], r.alsgs1[l]);
            add(f.cstar, r.cstar);
            for (int l = 0; l < 6; l++) add(f.kstar[l], r.kstar[l]);
            auto v32 = [&](const double *dev, long long n) -> const float * {
                std::vector<double> h((size_t)n);
                cudaMemcpy(h.data(), dev, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost);
                std::vector<float> hf(h.begin(), h.end());
                return upload(A, hf.data(), hf.size());
            };
            const long long nx = d.n1 + 2, ny = d.n2 + 2, nz = d.n3 + 2;
            r.f2fx = v32(d.f2fx, nx); r.f2fy = v32(d.f2fy, ny); r.f2fz = v32(d.f2fz, nz);
            r.f2fxi = v32(d.f2fxi, nx); r.f2fyi = v32(d.f2fyi, ny); r.f2fzi = v32(d.f2fzi, nz);
            r.c2cxi = v32(d.c2cxi, nx); r.c2cyi = v32(d.c2cyi, ny); r.c2czi = v32(d.c2czi, nz);
            r.aiu = v32(f.aiu, nx); r.ciu = v32(f.ciu, nx); r.aivw = v32(f.aivw, nx); r.civw = v32(f.civw, nx);
            r.ajv = v32(f.ajv, ny); r.cjv = v32(f.cjv, ny); r.ajuw = v32(f.ajuw, ny); r.cjuw = v32(f.cjuw, ny);
            r.akw = v32(f.akw, nz); r.ckw = v32(f.ckw, nz); r.akuv = v32(f.akuv, nz); r.ckuv = v32(f.ckuv, nz);
            r.cfx1 = v32(f.cfx1, 3 * (d.n1m + 2)); r.cfy1 = v32(f.cfy1, 3 * (d.n2m + 2)); r.cfz1 = v32(f.cfz1, 3 * (d.n3m + 2));
            r.fixil = v32(m.fixil, d.n1m + 2); r.fixiu = v32(m.fixiu, d.n1m + 2);
            r.fixjl = v32(m.fixjl, d.n2m + 2); r.fixju = v32(m.fixju, d.n2m + 2);
            r.fixkl = v32(m.fixkl, d.n3m + 2); r.fixku = v32(m.fixku, d.n3m + 2);
        }
    }
    c->S = A.get<DScal>(1);
    c->kp.S = c->S;
    c->h_f2fx = (double *)calloc(d.n1 + 2, sizeof(double));
    c->h_f2fz = (double *)calloc(d.n3 + 2, sizeof(double));
    for (long long i = 0; i <= d.n1; i++) c->h_f2fx[i] = g->f2fxi[i];
    for (long long kk = 0; kk <= d.n3; kk++) c->h_f2fz[kk] = g->f2fzi[kk];
    if (!A.ok) { lesgpu_destroy(c); return LESGPU_ERR_OOM; }
    // the tables went up by cudaMemcpy on the legacy stream, whose DMA may
    // still be in flight; the case stream (non-blocking) is ordered after it
    // only by this wait
    if (cudaStreamSynchronize(cudaStreamLegacy) != cudaSuccess) { lesgpu_destroy(c); return LESGPU_ERR_CUDA; }
    launch_red_weights(c);
    c->h_grid = g;
    rc = poisson_init(c);
    c->h_grid = nullptr;
    if (rc) { lesgpu_destroy(c); return rc; }
    if (cudaDeviceSynchronize() != cudaSuccess) { lesgpu_destroy(c); return LESGPU_ERR_CUDA; }
    *out = c;
    return 0;
}

// --------------------------------------------------------------- load_ibm
extern "C" int lesgpu_load_ibm(lesgpu_case *c, const lesgpu_ibm *b) {
    if (!c || !b) return LESGPU_ERR_ARG;
    const DGrid &d = c->kp.g;
    DFields &f = c->kp.f;
    Alloc &A = ((CaseExtra *)c->dmem_pool)->alloc;
    int nl = c->cfg.ihtrans == 1 ? 4 : 3;
    for (int l = 0; l < nl; l++) {
        if (b->nbody[l] < b->nintp[l] || b->nintp[l] < 0 || b->nbody[l] > 0x7ffffff0LL) return LESGPU_ERR_ARG;
        if (b->nbody[l] > 0 && c->cfg.ibmon == 0) return LESGPU_ERR_CONFIG;
        if (b->nbody[l] > 0 && (!b->fc[l] || (b->nintp[l] > 0 && (!b->intpindx[l] || !b->geomfac[l]))))
            return LESGPU_ERR_ARG;
    }
    // forcing lists (ibmpreread, misc_init.f90:312-378): 1-based rows on the
    // device.  Every index is checked against the grid before anything is
    // uploaded, so a rejected table leaves the case as it was and no gather
    // can leave the arrays.
    struct HostList { std::vector<int> fi, fj, fk, ix; std::vector<double> gf; };
    HostList H[4];
    for (int l = 0; l < nl; l++) {
        long long nb = b->nbody[l], ni = b->nintp[l];
        HostList &h = H[l];
        h.fi.assign(nb + 1, 0); h.fj.assign(nb + 1, 0); h.fk.assign(nb + 1, 0);
        h.ix.assign(3 * (ni + 1), 0); h.gf.assign(27 * (ni + 1), 0.0);
        for (long long n = 0; n < nb; n++) {
            long long i = b->fc[l][3 * n], j = b->fc[l][3 * n + 1], k = b->fc[l][3 * n + 2];
            if (i < 1 || i > d.n1m || j < 1 || j > d.n2m || k < 1 || k > d.n3m) return LESGPU_ERR_ARG;
            h.fi[n + 1] = (int)i; h.fj[n + 1] = (int)j; h.fk[n + 1] = (int)k;
        }
        for (long long n = 0; n < ni; n++) {
            for (int q = 0; q < 3; q++) {
                long long dq = b->intpindx[l][3 * n + q];
                if (dq < -1 || dq > 1) return LESGPU_ERR_ARG;
                h.ix[3 * (n + 1) + q] = (int)dq;
            }
            // x and z wrap through reindex_i / reindex_k; y must stay in 0..n2
            long long jpp = h.fj[n + 1] + 2 * h.ix[3 * (n + 1) + 1];
            if (jpp < 0 || jpp > d.n2) return LESGPU_ERR_ARG;
            for (int q = 0; q < 27; q++) h.gf[27 * (n + 1) + q] = b->geomfac[l][27 * n + q];
        }
    }
    // zero-eddy-viscosity list: the file's 0-based numbers are used as
    // indices as they are (sgs.f90:893-895), so 0..n?m-1 are valid
    if (b->nzero < 0 || b->nzero > 0x7ffffff0LL || (b->nzero > 0 && (!b->inz || !b->jnz || !b->knz)))
        return LESGPU_ERR_ARG;
    for (long long n = 0; n < b->nzero; n++)
        if (b->inz[n] < 0 || b->inz[n] > d.n1 || b->jnz[n] < 0 || b->jnz[n] > d.n2 || b->knz[n] < 0 || b->knz[n] > d.n3)
            return LESGPU_ERR_ARG;
    for (int l = 0; l < nl; l++) {
        long long nb = b->nbody[l];
        HostList &h = H[l];
        f.ifc[l] = upload(A, h.fi.data(), h.fi.size()); f.jfc[l] = upload(A, h.fj.data(), h.fj.size());
        f.kfc[l] = upload(A, h.fk.data(), h.fk.size());
        f.intpindx[l] = upload(A, h.ix.data(), h.ix.size()); f.geomfac[l] = upload(A, h.gf.data(), h.gf.size());
        f.fcv[l] = A.get<double>(nb + 1); f.fcvavg[l] = A.get<double>(nb + 1);
        f.ibtarg[l] = A.get<double>(nb + 1);
        if (l < 3) f.dudtr[l] = A.get<double>(nb + 1);
        c->kp.c.nbody[l] = (int)nb; c->kp.c.nintp[l] = b->nintp[l] > 0 ? (int)b->nintp[l] : 0;
    }
    if (c->graph_ok) { cudaGraphExecDestroy(c->graph); c->graph_ok = 0; }
    c->kp.c.nzero = (int)b->nzero;
    if (b->nzero > 0) {
        std::vector<int> a(b->nzero + 2), bb(b->nzero + 2), cc(b->nzero + 2);
        for (long long n = 0; n < b->nzero; n++) { a[n + 1] = (int)b->inz[n]; bb[n + 1] = (int)b->jnz[n]; cc[n + 1] = (int)b->knz[n]; }
        f.inz = upload(A, a.data(), a.size()); f.jnz = upload(A, bb.data(), bb.size()); f.knz = upload(A, cc.data(), cc.size());
    }
    size_t nt = (size_t)d.nt;
    long long n1m = d.n1m, n2m = d.n2m, n3m = d.n3m, ncell = n1m * n2m * n3m;
    auto scatter_d = [&](const double *src, double *dst) {
        std::vector<double> h(nt, 1.0);
        for (long long kk = 1; kk <= n3m; kk++)
            for (long long j = 1; j <= n2m; j++)
                for (long long i = 1; i <= n1m; i++)
                    h[i + d.sx * j + d.sxy * kk] = src[(i - 1) + n1m * ((j - 1) + n2m * (kk - 1))];
        cudaMemcpy(dst, h.data(), nt * sizeof(double), cudaMemcpyHostToDevice);
    };
    auto scatter_i = [&](const int64_t *src, int *dst) {
        std::vector<int> h(nt, 1);
        for (long long kk = 1; kk <= n3m; kk++)
            for (long long j = 1; j <= n2m; j++)
                for (long long i = 1; i <= n1m; i++)
                    h[i + d.sx * j + d.sxy * kk] = (int)src[(i - 1) + n1m * ((j - 1) + n2m * (kk - 1))];
        cudaMemcpy(dst, h.data(), nt * sizeof(int), cudaMemcpyHostToDevice);
    };
    if (b->nwall_dvm) scatter_i(b->nwall_dvm, f.nwall);
    if (b->omega) scatter_i(b->omega, f.omega);
    if (b->cstar) scatter_d(b->cstar, f.cstar);
    if (b->kstar)
        for (int l = 0; l < 6; l++) scatter_d(b->kstar + (size_t)l * ncell, f.kstar[l]);
    // unit tables (a channel whose ICONJG = 1 only provides the arrays tvolcalc
    // reads) make the temperature coefficients c* k* + cre omega alpha equal
    // to 1 + cre alpha, so the sweeps may use their factored form
    for (size_t q = 0; b->omega && q < (size_t)ncell; q++)
        if (b->omega[q] != 1) c->conj_general = 1;
    for (size_t q = 0; b->cstar && q < (size_t)ncell; q++)
        if (b->cstar[q] != 1.0) c->conj_general = 1;
    for (size_t q = 0; b->kstar && q < 6 * (size_t)ncell; q++)
        if (b->kstar[q] != 1.0) c->conj_general = 1;
    c->kp.c.conj_tables = c->kp.c.iconjg == 1 && c->conj_general;
    if (!A.ok) return LESGPU_ERR_OOM;
    // the tables above went up by cudaMemcpy on the legacy stream, whose DMA
    // may still be in flight; the case stream (non-blocking) is ordered after
    // it only by this wait
    if (cudaStreamSynchronize(cudaStreamLegacy) != cudaSuccess) return LESGPU_ERR_CUDA;
    launch_red_weights(c);
    mark_mirror(c, kMirConj);
    launch_mirror(c, kMirConj);
    return cuda_rc(cudaDeviceSynchronize());
}

// ------------------------------------------------------------- set_fields
extern "C" int lesgpu_set_fields(lesgpu_case *c, const double *u, const double *v, const double *w,
                                 const double *p, const double *t, double time, double dt, int64_t ihist, int64_t m) {
    if (!c || !u || !v || !w || !p) return LESGPU_ERR_ARG;
    size_t bytes = sizeof(double) * (size_t)c->kp.g.nt;
    DFields &f = c->kp.f;
    mark_mirror(c, kMirVel | kMirP | kMirT);
    cudaMemcpyAsync(f.u, u, bytes, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(f.v, v, bytes, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(f.w, w, bytes, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(f.p, p, bytes, cudaMemcpyHostToDevice, c->stream);
    if (t) cudaMemcpyAsync(f.t, t, bytes, cudaMemcpyHostToDevice, c->stream);
    DScal s;
    cudaMemcpyAsync(&s, c->S, sizeof(DScal), cudaMemcpyDeviceToHost, c->stream);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return LESGPU_ERR_CUDA;
    s.time = time; s.dt = dt; s.ihist = ihist; s.m = m;
    cudaMemcpyAsync(c->S, &s, sizeof(DScal), cudaMemcpyHostToDevice, c->stream);
    return cuda_rc(cudaStreamSynchronize(c->stream));
}

// ------------------------------------------------------------------ start
__global__ void k_start(KP p) {
    DScal *S = p.S;
    S->ntime = 0;
    S->cflmax = p.c.cflfac;
    S->err_integral = 0.0;
    S->err = 0;
}

extern "C" int lesgpu_start(lesgpu_case *c) {
    if (!c) return LESGPU_ERR_ARG;
    const lesgpu_config &g = c->cfg;
    DScal s;
    cudaMemcpyAsync(&s, c->S, sizeof(DScal), cudaMemcpyDeviceToHost, c->stream);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return LESGPU_ERR_CUDA;
    // dttimeinit, misc_init.f90:1001-1028
    if (g.idtopt == 0) s.dt = g.dt_size;
    if (g.idtopt != 0 && g.iread == 0) s.dt = g.dt_size;
    if (g.ireset == 1) { s.ihist = 0; s.time = 0.0; }
    cudaMemcpyAsync(c->S, &s, sizeof(DScal), cudaMemcpyHostToDevice, c->stream);
    k_start<<<1, 1, 0, c->stream>>>(c->kp);
    launch_mirror(c, kMirConj | kMirNu | kMirAl);
    if (g.ich != 0) launch_meanpg(c);
    if (g.ihtrans == 1 && g.ich == 1) launch_cvol(c);
    c->ntime_host = 0;
    {
        const char *ff = getenv("LESGPU_ADI_FP32_FORM");
        const int v = ff ? atoi(ff) : 0;
        const int wl = v & 63;
        c->adi_force_f32 = (v == 128 || (v == 1) || ((wl == 8 || wl == 16 || wl == 32) && (v == wl || v == (wl | 64)))) ? v : 0;
    }
    c->started = 1;
    if (c->graph_ok) { cudaGraphExecDestroy(c->graph); c->graph_ok = 0; }
    // autotuner: on unless LESGPU_AUTOTUNE=0 (a tuned choice changes the
    // rounding of the scan-form sweeps, so runs that must agree bitwise across
    // processes turn it off)
    const char *at = getenv("LESGPU_AUTOTUNE");
    c->autotune = !(at && at[0] == '0');
    if (c->autotune) {
        int rc = adi_autotune(c);
        if (!rc) rc = fft_autotune(c);
        if (!rc) rc = mg2d_autotune(c);
        if (rc) return rc;
    }
    return cuda_rc(cudaStreamSynchronize(c->stream));
}

// ------------------------------------------------------------------- step
__global__ void k_retrv_uvw(KP p) {   // retrv_uvw, slv_mmtm.f90:1710-1743
    const DGrid &g = p.g;
    long long n = (long long)g.n2m * g.n3m;
    for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += (long long)gridDim.x * blockDim.x) {
        int j = 1 + (int)(s % g.n2m), k = 1 + (int)(s / g.n2m);
        long long pq = j + (long long)(g.n2 + 1) * k;
        p.f.u[g.ix(g.n1, j, k)] = p.f.uout[pq];
        if (j >= 2) p.f.v[g.ix(g.n1, j, k)] = p.f.vout[pq];
        if (k >= g.k_bgpz) p.f.w[g.ix(g.n1, j, k)] = p.f.wout[pq];
    }
}

static void enqueue_sgs(lesgpu_case *c, bool first) {
    const lesgpu_config &g = c->cfg;
    launch_mirror(c, kMirVel | kMirT);
    if (first) launch_sgs_zero_first(c, 0);
    else launch_sgs(c);
    launch_sgs_post(c);
    mark_mirror(c, kMirNu);
    launch_mirror(c, kMirNu);
    if (g.ihtrans == 1) {
        if (first) launch_sgs_zero_first(c, 1);
        else launch_sgs_t(c);
        launch_sgs_t_post(c);
        mark_mirror(c, kMirAl);
        launch_mirror(c, kMirAl);
    }
}

static void enqueue_rhsnlhs(lesgpu_case *c, int msub) {
    launch_mirror(c, kMirVel | kMirP | kMirT);
    launch_rhs(c, msub);
    if (c->cfg.ibmon != 0) launch_rhs_ibm(c);
    launch_convbc(c);
    launch_adi_uvw(c);
    k_retrv_uvw<<<blocks_for((long long)c->kp.g.n2m * c->kp.g.n3m), kThreads, 0, c->stream>>>(c->kp);
    launch_ghost_uvw(c);
    mark_mirror(c, kMirVel);
}

static void enqueue_energy(lesgpu_case *c, int msub) {
    const lesgpu_config &g = c->cfg;
    launch_mirror(c, kMirVel | kMirT);     // the projected velocity
    launch_rhs_t(c, msub, g.ich == 1);              // with tvolcalc(tvol(1)) when ICH = 1
    if (g.ibmon != 0 && g.iconjg == 0) launch_rhs_ibm_t(c);
    launch_convbc_t(c);
    launch_adi_t(c);
    launch_energy_bc(c);
    // tvolcalc(tvol(2)) + tvolcorr; tcalc changes t only when x is not
    // periodic, otherwise tvolcalc(tvol(0)) is the same sum
    const bool tcalc_runs = g.ich == 1 && g.xprdic == 0;
    if (g.ich == 1) launch_tvolcalc_corr(c, !tcalc_runs);
    launch_tcalc(c);
    if (tcalc_runs) launch_tvolcalc(c, 0);
    mark_mirror(c, kMirT);
}

// A substep up to the Poisson solve (with stepinit before the first one)
// and from the solve's result on (with the step's checks and diagnostics
// after the last one): solver.f90:85-151, 154-173.
static void enqueue_substep_pre(lesgpu_case *c, int msub, bool first) {
    const lesgpu_config &g = c->cfg;
    if (msub == 1) launch_stepinit(c);
    launch_substepinit(c, msub);
    if (g.ich == 1) launch_qvolcalc(c, 1);
    if (g.iles == 1 && msub == 1) enqueue_sgs(c, first);
    enqueue_rhsnlhs(c, msub);
    launch_divgs(c);
}

static void enqueue_substep_post(lesgpu_case *c, int msub) {
    const lesgpu_config &g = c->cfg;
    launch_ucalc_pcalc(c, g.ich == 1);        // qvolcalc(qvol(2)), ucalc, qvolcalc(qvol(0)), pcalc
    mark_mirror(c, kMirVel | kMirP);
    if (g.ich != 0) launch_meanpg(c);
    if (g.ibmon == 1) launch_lagforce(c, msub);
    if (g.ihtrans == 1) enqueue_energy(c, msub);
    if (msub == 3) {
        launch_advance_and_convergence(c);          // time += dt, convergence_check
        launch_bulk_diag(c);
        if (g.ibmon == 1) launch_draglift(c);
        if (g.ihtrans == 1) launch_heatflux(c);
        if (g.iavg == 1) launch_field_avg(c);
    }
}

static void enqueue_step(lesgpu_case *c, bool first) {
    for (int msub = 1; msub <= 3; msub++) {
        enqueue_substep_pre(c, msub, first);
        launch_poisson(c, msub);
        enqueue_substep_post(c, msub);
    }
}

// The out-of-date mirror sets a step leaves behind (and the captured step
// assumes at its start): p (pcalc), and t after the energy phase's sweeps or,
// without heat transfer, the projected velocity.
static unsigned mir_steady(const lesgpu_case *c) { return kMirP | (c->cfg.ihtrans == 1 ? kMirT : kMirVel); }

// Before a replay of the captured step: refresh eagerly what is out of date
// beyond the steady state (after set_fields, set_array, start).
static void mirror_prologue(lesgpu_case *c) {
    const unsigned extra = c->mir_dirty & ~mir_steady(c);
    if (extra) launch_mirror(c, extra);
}

// Capture one steady-state step into a CUDA graph and count its kernels.
static int capture_step(lesgpu_case *c) {
    cudaGraph_t gr;
    if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return LESGPU_ERR_CUDA;
    c->mir_dirty = mir_steady(c);
    enqueue_step(c, false);
    if (cudaStreamEndCapture(c->stream, &gr) != cudaSuccess) return LESGPU_ERR_CUDA;
    size_t nn = 0;
    cudaGraphGetNodes(gr, nullptr, &nn);
    std::vector<cudaGraphNode_t> nodes(nn);
    if (nn) cudaGraphGetNodes(gr, nodes.data(), &nn);
    long long nk = 0;
    for (size_t q = 0; q < nn; q++) {
        cudaGraphNodeType t;
        cudaGraphNodeGetType(nodes[q], &t);
        if (t == cudaGraphNodeTypeKernel) nk++;
    }
    c->kernels_per_step = nk;
    if (cudaGraphInstantiate(&c->graph, gr, 0) != cudaSuccess) { cudaGraphDestroy(gr); return LESGPU_ERR_CUDA; }
    cudaGraphDestroy(gr);
    c->graph_ok = 1;
    return 0;
}

// ---- the serving loop's size buckets: one step of every case of a bucket
// (cases of one grid shape and options) captured as one CUDA graph on the
// bucket's stream.  Each case's kernels run on its own stream branch, forked
// from and joined to the bucket stream; for poiss_z_ft / poiss_x_ft the
// branches join before each substep's Poisson solve, whose mode solves run
// as one batched launch over all the cases, and fork again after it.
namespace lg {

int bucket_prologue(lesgpu_case **cs, int n) {
    for (int q = 0; q < n; q++) {
        lesgpu_case *c = cs[q];
        const unsigned extra = c->mir_dirty & ~mir_steady(c);
        if (extra) {
            launch_mirror(c, extra);
            if (cudaStreamSynchronize(c->stream) != cudaSuccess) return LESGPU_ERR_CUDA;
        }
    }
    return 0;
}

void bucket_replayed(lesgpu_case **cs, int n, int steps) {
    for (int q = 0; q < n; q++) {
        cs[q]->ntime_host += steps;
        cs[q]->mir_dirty = mir_steady(cs[q]);
    }
}

void free_bucket_graph(BucketGraph *bg) {
    if (bg->exec) cudaGraphExecDestroy(bg->exec);
    if (bg->d_args) cudaFree(bg->d_args);
    bg->exec = nullptr;
    bg->d_args = nullptr;
    bg->kernels = 0;
}

int capture_bucket_step(lesgpu_case **cs, int n, cudaStream_t st, BucketGraph *bg) {
    free_bucket_graph(bg);
    if (n < 1) return LESGPU_ERR_ARG;
    const int pk = (int)cs[0]->cfg.poisson;
    const bool batched = pk == LESGPU_POISSON_Z_FT || pk == LESGPU_POISSON_X_FT;
    for (int q = 1; q < n; q++)
        if (cs[q]->cfg.poisson != pk || (batched && mg2d_batch_key(cs[q]) != mg2d_batch_key(cs[0])))
            return LESGPU_ERR_ARG;
    const size_t sz = batched ? (size_t)mg2d_batch_size(cs[0]) : 0;
    if (batched) {
        std::vector<unsigned char> h(3 * (size_t)n * sz);
        for (int msub = 1; msub <= 3; msub++)
            for (int q = 0; q < n; q++) mg2d_batch_args(cs[q], msub, h.data() + ((size_t)(msub - 1) * n + q) * sz);
        if (cudaMalloc(&bg->d_args, h.size()) != cudaSuccess) return LESGPU_ERR_OOM;
        // on the bucket stream, which the graph is launched on: a plain
        // cudaMemcpy from pageable memory may return before its DMA lands and
        // is ordered on the legacy stream only, which the non-blocking bucket
        // stream does not wait for -- the batched solve would read the
        // pointers in these arguments before they are there
        if (cudaMemcpyAsync(bg->d_args, h.data(), h.size(), cudaMemcpyHostToDevice, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            return LESGPU_ERR_CUDA;
    }
    int rc = bucket_prologue(cs, n);
    if (rc) return rc;
    std::vector<cudaEvent_t> ev(n + 1, nullptr);
    for (auto &e : ev)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) rc = LESGPU_ERR_CUDA;
    auto fork = [&]() {
        cudaEventRecord(ev[n], st);
        for (int q = 0; q < n; q++) cudaStreamWaitEvent(cs[q]->stream, ev[n], 0);
    };
    auto join = [&]() {
        for (int q = 0; q < n; q++) {
            cudaEventRecord(ev[q], cs[q]->stream);
            cudaStreamWaitEvent(st, ev[q], 0);
        }
    };
    cudaGraph_t gr = nullptr;
    if (!rc && cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) rc = LESGPU_ERR_CUDA;
    if (!rc) {
        for (int q = 0; q < n; q++) cs[q]->mir_dirty = mir_steady(cs[q]);
        fork();
        for (int msub = 1; msub <= 3; msub++) {
            for (int q = 0; q < n; q++) {
                enqueue_substep_pre(cs[q], msub, false);
                if (batched) mg2d_launch_pre(cs[q], msub);
                else launch_poisson(cs[q], msub);
            }
            if (batched) {
                join();
                mg2d_launch_batch(cs[0], (const unsigned char *)bg->d_args + (size_t)(msub - 1) * n * sz, n, st);
                fork();
                for (int q = 0; q < n; q++) mg2d_launch_post(cs[q]);
            }
            for (int q = 0; q < n; q++) enqueue_substep_post(cs[q], msub);
        }
        join();
        if (cudaStreamEndCapture(st, &gr) != cudaSuccess) rc = LESGPU_ERR_CUDA;
    }
    for (auto &e : ev)
        if (e) cudaEventDestroy(e);
    if (rc) {
        if (gr) cudaGraphDestroy(gr);
        return rc;
    }
    size_t nn = 0;
    cudaGraphGetNodes(gr, nullptr, &nn);
    std::vector<cudaGraphNode_t> nodes(nn);
    if (nn) cudaGraphGetNodes(gr, nodes.data(), &nn);
    for (size_t q = 0; q < nn; q++) {
        cudaGraphNodeType t;
        cudaGraphNodeGetType(nodes[q], &t);
        if (t == cudaGraphNodeTypeKernel) bg->kernels++;
    }
    if (cudaGraphInstantiate(&bg->exec, gr, 0) != cudaSuccess) rc = LESGPU_ERR_CUDA;
    cudaGraphDestroy(gr);
    return rc;
}

}  // namespace lg

static void fill_report(const lesgpu_case *c, const DScal &s, lesgpu_step_report *r) {
    memset(r, 0, sizeof(*r));
    r->ntime = s.ntime; r->ihist = s.ihist; r->m = s.m;
    r->time = s.time; r->dt = s.dt;
    r->cflmax = s.cflmax; r->dvmax = s.dvmax; r->qmmax = s.qmmax;
    for (int q = 0; q < 5; q++) r->pmi[q] = s.pmi[q];
    r->pmiavg = s.pmiavg;
    for (int q = 0; q < 3; q++) { r->qvol[q] = s.qvol[q]; r->tvol[q] = s.tvol[q]; r->cd[q] = s.cd[q]; r->heat_flux[q] = s.heat_flux[q]; }
    r->csgsts = s.csgsts; r->csgshf = s.csgshf;
    r->nutavg = s.nutavg; r->nutmax = s.nutmax; r->alpavg = s.alpavg; r->alpmax = s.alpmax;
    r->ubulk = s.ubulk; r->qflux = s.qflux; r->tbulk_fluid = s.tbulk_fluid; r->tbulk_solid = s.tbulk_solid;
    for (int q = 0; q < 3; q++) r->poisson_iters[q] = s.poisson_iters[q];
    r->poisson_unconverged = s.poisson_unconv;
    r->heat_body = s.heat_body;
}

extern "C" int lesgpu_step(lesgpu_case *c, lesgpu_step_report *rep) {
    if (!c) return LESGPU_ERR_ARG;
    if (!c->started) return LESGPU_ERR_STATE;
    c->ntime_host += 1;
    bool first = (c->cfg.iread == 0 && c->ntime_host == 1);
    if (c->use_graph && !first && c->inst_cls == 0) {
        mirror_prologue(c);
        if (!c->graph_ok) {
            int rc = capture_step(c);
            if (rc) return rc;
        }
        if (cudaGraphLaunch(c->graph, c->stream) != cudaSuccess) return LESGPU_ERR_CUDA;
        c->mir_dirty = mir_steady(c);
    } else {
        enqueue_step(c, first);
    }
    if (cudaMemcpyAsync(&c->hS, c->S, sizeof(DScal), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess) return LESGPU_ERR_CUDA;
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return LESGPU_ERR_CUDA;
    if (rep) fill_report(c, c->hS, rep);
    if (c->hS.err) return LESGPU_ERR_NAN;
    if (c->strict && c->hS.poisson_unconv > 0) return LESGPU_ERR_NOT_CONVERGED;
    return 0;
}

// Enqueue n steps without reading anything back (benchmark path; the
// caller synchronises the stream).  n must be >= 1; steps follow the same
// graph path as lesgpu_step.
extern "C" int lesgpu_step_async(lesgpu_case *c, int64_t n) {
    if (!c || n < 1) return LESGPU_ERR_ARG;
    if (!c->started) return LESGPU_ERR_STATE;
    for (int64_t s = 0; s < n; s++) {
        c->ntime_host += 1;
        bool first = (c->cfg.iread == 0 && c->ntime_host == 1);
        if (c->use_graph && !first && c->inst_cls == 0) {
            mirror_prologue(c);
            if (!c->graph_ok) {
                int rc = capture_step(c);
                if (rc) return rc;
            }
            if (cudaGraphLaunch(c->graph, c->stream) != cudaSuccess) return LESGPU_ERR_CUDA;
            c->mir_dirty = mir_steady(c);
        } else {
            enqueue_step(c, first);
        }
    }
    return 0;
}

extern "C" int lesgpu_stream(lesgpu_case *c, void **stream) {
    if (!c || !stream) return LESGPU_ERR_ARG;
    *stream = (void *)c->stream;
    return 0;
}

extern "C" int lesgpu_set_strict(lesgpu_case *c, int on) {
    if (!c) return LESGPU_ERR_ARG;
    c->strict = on ? 1 : 0;
    return 0;
}

extern "C" int lesgpu_use_graph(lesgpu_case *c, int on) {
    if (!c) return LESGPU_ERR_ARG;
    c->use_graph = on ? 1 : 0;
    return 0;
}

extern "C" int lesgpu_tuning(lesgpu_case *c, int64_t *out, int64_t maxn, int64_t *nclasses) {
    if (!c || !nclasses || maxn < 0 || (maxn > 0 && !out)) return LESGPU_ERR_ARG;
    int buf[4 * 72];
    int n = c->autotune ? adi_tuned(c, buf, 4 * 64) : 0;
    if (c->autotune && c->pois.Lz > 0) { buf[4 * n] = 3; buf[4 * n + 1] = 2; buf[4 * n + 2] = 0; buf[4 * n + 3] = c->pois.Lz; n++; }
    if (c->autotune && c->pois.Lx > 0) { buf[4 * n] = 3; buf[4 * n + 1] = 0; buf[4 * n + 2] = 0; buf[4 * n + 3] = c->pois.Lx; n++; }
    if (c->autotune && mg2d_cluster(c) > 0) { buf[4 * n] = 4; buf[4 * n + 1] = 0; buf[4 * n + 2] = 0; buf[4 * n + 3] = mg2d_cluster(c); n++; }
    if (c->cfg.poisson == LESGPU_POISSON_FTFT && c->cfg.precision == LESGPU_PREC_MIXED) {
        buf[4 * n] = 5; buf[4 * n + 1] = 0; buf[4 * n + 2] = 0; buf[4 * n + 3] = c->pois.mixed_fft; n++;
    }
    *nclasses = n;
    for (int q = 0; q < n && q < maxn; q++)
        for (int e = 0; e < 4; e++) out[4 * q + e] = buf[4 * q + e];
    return 0;
}

extern "C" int lesgpu_launch_count(lesgpu_case *c, int64_t *kernels_per_step) {
    if (!c || !kernels_per_step) return LESGPU_ERR_ARG;
    if (!c->graph_ok) {
        if (!c->started) return LESGPU_ERR_STATE;
        int rc = capture_step(c);
        if (rc) return rc;
    }
    *kernels_per_step = c->kernels_per_step;
    return 0;
}

extern "C" int lesgpu_instrument(lesgpu_case *c, int64_t cls) {
    if (!c || cls < 0 || cls > 5) return LESGPU_ERR_ARG;
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return LESGPU_ERR_CUDA;
    if (cls != 0 && c->inst_ev[0] == nullptr)
        for (int q = 0; q < 2 * 4096; q++)
            if (cudaEventCreate(&c->inst_ev[q]) != cudaSuccess) return LESGPU_ERR_CUDA;
    c->inst_cls = (int)cls;
    c->inst_n = 0;
    return 0;
}

extern "C" int lesgpu_instrument_read(lesgpu_case *c, double *ms, int64_t *launches) {
    if (!c || !ms || !launches) return LESGPU_ERR_ARG;
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return LESGPU_ERR_CUDA;
    double tot = 0.0;
    for (int q = 0; q < c->inst_n; q++) {
        float m = 0.f;
        if (cudaEventElapsedTime(&m, c->inst_ev[2 * q], c->inst_ev[2 * q + 1]) != cudaSuccess) return LESGPU_ERR_CUDA;
        tot += m;
    }
    *ms = tot;
    *launches = c->inst_n;
    c->inst_n = 0;
    return 0;
}

extern "C" int lesgpu_get_report(lesgpu_case *c, lesgpu_step_report *rep) {
    if (!c || !rep) return LESGPU_ERR_ARG;
    if (cudaMemcpyAsync(&c->hS, c->S, sizeof(DScal), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess) return LESGPU_ERR_CUDA;
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return LESGPU_ERR_CUDA;
    fill_report(c, c->hS, rep);
    return 0;
}

extern "C" int lesgpu_get_fields(lesgpu_case *c, double *u, double *v, double *w, double *p, double *t) {
    if (!c) return LESGPU_ERR_ARG;
    size_t bytes = sizeof(double) * (size_t)c->kp.g.nt;
    DFields &f = c->kp.f;
    if (u) cudaMemcpyAsync(u, f.u, bytes, cudaMemcpyDeviceToHost, c->stream);
    if (v) cudaMemcpyAsync(v, f.v, bytes, cudaMemcpyDeviceToHost, c->stream);
    if (w) cudaMemcpyAsync(w, f.w, bytes, cudaMemcpyDeviceToHost, c->stream);
    if (p) cudaMemcpyAsync(p, f.p, bytes, cudaMemcpyDeviceToHost, c->stream);
    if (t) cudaMemcpyAsync(t, f.t, bytes, cudaMemcpyDeviceToHost, c->stream);
    return cuda_rc(cudaStreamSynchronize(c->stream));
}

static int field_ptrs(lesgpu_case *c, int64_t fld, double **ptr, int *nc) {
    DFields &f = c->kp.f;
    *nc = 1;
    switch (fld) {
    case LESGPU_F_U: ptr[0] = f.u; return 0;
    case LESGPU_F_V: ptr[0] = f.v; return 0;
    case LESGPU_F_W: ptr[0] = f.w; return 0;
    case LESGPU_F_P: ptr[0] = f.p; return 0;
    case LESGPU_F_T: ptr[0] = f.t; return 0;
    case LESGPU_F_NUSGS: ptr[0] = f.nusgs; return 0;
    case LESGPU_F_ALSGS: ptr[0] = f.alsgs; return 0;
    case LESGPU_F_NUSGS1: *nc = 3; for (int l = 0; l < 3; l++) ptr[l] = f.nusgs1[l]; return 0;
    case LESGPU_F_ALSGS1: *nc = 3; for (int l = 0; l < 3; l++) ptr[l] = f.alsgs1[l]; return 0;
    case LESGPU_F_RHS1: *nc = 4; for (int l = 0; l < 4; l++) ptr[l] = f.rhs1[l]; return 0;
    case LESGPU_F_RK3O: *nc = 4; for (int l = 0; l < 4; l++) ptr[l] = f.rk3o[l]; return 0;
    case LESGPU_F_RK3OO: *nc = 4; for (int l = 0; l < 4; l++) ptr[l] = f.rk3oo[l]; return 0;
    case LESGPU_F_DIVGSUM: ptr[0] = f.divgsum; return 0;
    case LESGPU_F_PHI: ptr[0] = f.phi; return 0;
    case LESGPU_F_QMASS: ptr[0] = f.qmass; return 0;
    default: return LESGPU_ERR_ARG;
    }
}

// the mixed form's FP32 RK3 histories, for the array copies below (null otherwise)
static float *const *hist32(lesgpu_case *c, int64_t fld) {
    DFields &f = c->kp.f;
    if (!f.rk3of[0]) return nullptr;
    if (fld == LESGPU_F_RK3O) return f.rk3of;
    if (fld == LESGPU_F_RK3OO) return f.rk3oof;
    return nullptr;
}

extern "C" int lesgpu_get_array(lesgpu_case *c, int64_t fld, double *out) {
    double *ptr[4];
    int nc;
    if (!c || !out || field_ptrs(c, fld, ptr, &nc)) return LESGPU_ERR_ARG;
    size_t nt = (size_t)c->kp.g.nt;
    if (float *const *h = hist32(c, fld)) {
        std::vector<float> tmp(nt);
        for (int l = 0; l < nc; l++) {
            if (cudaMemcpyAsync(tmp.data(), h[l], nt * sizeof(float), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
                cudaStreamSynchronize(c->stream) != cudaSuccess)
                return LESGPU_ERR_CUDA;
            for (size_t q = 0; q < nt; q++) out[l * nt + q] = (double)tmp[q];
        }
        return 0;
    }
    for (int l = 0; l < nc; l++) cudaMemcpyAsync(out + l * nt, ptr[l], nt * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    return cuda_rc(cudaStreamSynchronize(c->stream));
}

extern "C" int lesgpu_set_array(lesgpu_case *c, int64_t fld, const double *in) {
    double *ptr[4];
    int nc;
    if (!c || !in || field_ptrs(c, fld, ptr, &nc)) return LESGPU_ERR_ARG;
    size_t nt = (size_t)c->kp.g.nt;
    if (float *const *h = hist32(c, fld)) {      // rounded to the FP32 the mixed form keeps
        std::vector<float> tmp(nt);
        for (int l = 0; l < nc; l++) {
            for (size_t q = 0; q < nt; q++) tmp[q] = (float)in[l * nt + q];
            if (cudaMemcpyAsync(h[l], tmp.data(), nt * sizeof(float), cudaMemcpyHostToDevice, c->stream) != cudaSuccess ||
                cudaStreamSynchronize(c->stream) != cudaSuccess)
                return LESGPU_ERR_CUDA;
        }
        return 0;
    }
    for (int l = 0; l < nc; l++) cudaMemcpyAsync(ptr[l], in + l * nt, nt * sizeof(double), cudaMemcpyHostToDevice, c->stream);
    mark_mirror(c, ~0u);
    launch_mirror(c, ~0u);
    return cuda_rc(cudaStreamSynchronize(c->stream));
}

extern "C" int lesgpu_run_phase(lesgpu_case *c, int64_t phase, int64_t msub) {
    if (!c || msub < 1 || msub > 3) return LESGPU_ERR_ARG;
    const lesgpu_config &g = c->cfg;
    c->mir_dirty = ~0u;        // a phase on its own refreshes every mirror it reads
    switch (phase) {
    case LESGPU_PH_STEPINIT: launch_stepinit(c); c->ntime_host += 1; break;
    case LESGPU_PH_SUBSTEPINIT: launch_substepinit(c, (int)msub); break;
    case LESGPU_PH_SGS:
        if (g.iles == 1 && msub == 1) enqueue_sgs(c, g.iread == 0 && c->ntime_host == 1);
        break;
    case LESGPU_PH_RHSNLHS: enqueue_rhsnlhs(c, (int)msub); break;
    case LESGPU_PH_DIVGS:
        cudaMemsetAsync(c->kp.f.divgsum, 0, sizeof(double) * c->kp.g.nt, c->stream);
        launch_divgs(c);
        break;
    case LESGPU_PH_POISSON:
        cudaMemsetAsync(c->kp.f.phi, 0, sizeof(double) * c->kp.g.nt, c->stream);
        launch_poisson(c, (int)msub);
        break;
    case LESGPU_PH_UCALC:
        launch_ucalc_pcalc(c, g.ich == 1);        // qvolcalc(qvol(2)), ucalc, qvolcalc(qvol(0)), pcalc
        break;
    case LESGPU_PH_MEANPG: if (g.ich != 0) launch_meanpg(c); break;
    case LESGPU_PH_ENERGY: if (g.ihtrans == 1) enqueue_energy(c, (int)msub); break;
    default: return LESGPU_ERR_ARG;
    }
    return cuda_rc(cudaStreamSynchronize(c->stream));
}

// ----------------------------------------------------------- field_avg
__global__ void k_avg_reset_count(KP p) { p.S->avg_count = 0; }

extern "C" int lesgpu_get_averages(lesgpu_case *c, double *out, int64_t *nsamples, int reset) {
    if (!c) return LESGPU_ERR_ARG;
    const DGrid &g = c->kp.g;
    const int na = c->cfg.ihtrans == 1 ? LESGPU_NAVG : LESGPU_NAVG - 2;
    double *avg = c->kp.f.avg;
    const size_t nt = (size_t)g.nt, nc = (size_t)g.n1m * g.n2m * g.n3m;
    if (out) {
        if (!avg) {
            memset(out, 0, sizeof(double) * nc * na);
        } else {
            for (int a = 0; a < na; a++) {
                cudaMemcpy3DParms m = {};
                m.srcPtr = make_cudaPitchedPtr(avg + nt * a, sizeof(double) * g.sx, g.sx, g.n2 + 1);
                m.srcPos = make_cudaPos(sizeof(double) * 1, 1, 1);
                m.dstPtr = make_cudaPitchedPtr(out + nc * a, sizeof(double) * g.n1m, g.n1m, g.n2m);
                m.dstPos = make_cudaPos(0, 0, 0);
                m.extent = make_cudaExtent(sizeof(double) * g.n1m, g.n2m, g.n3m);
                m.kind = cudaMemcpyDeviceToHost;
                if (cudaMemcpy3DAsync(&m, c->stream) != cudaSuccess) return LESGPU_ERR_CUDA;
            }
        }
    }
    DScal s;
    cudaMemcpyAsync(&s, c->S, sizeof(DScal), cudaMemcpyDeviceToHost, c->stream);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return LESGPU_ERR_CUDA;
    if (nsamples) *nsamples = s.avg_count;
    if (reset) {
        if (avg) cudaMemsetAsync(avg, 0, sizeof(double) * nt * LESGPU_NAVG, c->stream);
        k_avg_reset_count<<<1, 1, 0, c->stream>>>(c->kp);
        if (cudaStreamSynchronize(c->stream) != cudaSuccess) return LESGPU_ERR_CUDA;
    }
    return 0;
}

extern "C" int lesgpu_destroy(lesgpu_case *c) {
    if (!c) return 0;
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->graph_ok) cudaGraphExecDestroy(c->graph);
    if (c->inst_ev[0])
        for (int q = 0; q < 2 * 4096; q++) cudaEventDestroy(c->inst_ev[q]);
    poisson_free(c);
    CaseExtra *X = (CaseExtra *)c->dmem_pool;
    if (X) {
        for (void *p : X->alloc.ptrs) cudaFree(p);
        delete X;
    }
    if (c->stream) cudaStreamDestroy(c->stream);
    free(c->h_f2fx);
    free(c->h_f2fz);
    free(c);
    return 0;
}

extern "C" const char *lesgpu_strerror(int code) {
    switch (code) {
    case LESGPU_OK: return "ok";
    case LESGPU_ERR_ARG: return "invalid argument";
    case LESGPU_ERR_CONFIG: return "option combination rejected by the reference solver";
    case LESGPU_ERR_CUDA: return "CUDA runtime error";
    case LESGPU_ERR_OOM: return "device memory exhausted";
    case LESGPU_ERR_NOT_CONVERGED: return "Poisson iteration limit exceeded";
    case LESGPU_ERR_NAN: return "non-finite value in the solver state";
    case LESGPU_ERR_STATE: return "call out of order";
    case LESGPU_ERR_UNSUPPORTED: return "option not built in this library";
    case LESGPU_ERR_TOO_LARGE: return "grid exceeds the fixed scratch of the allocation-free entry point";
    default: return "unknown error";
    }
}

extern "C" int lesgpu_abi_version(void) { return LESGPU_ABI_VERSION; }

extern "C" int lesgpu_set_device(int64_t device) {
    if (device < 0) return LESGPU_ERR_ARG;
    return cuda_rc(cudaSetDevice((int)device));
}
