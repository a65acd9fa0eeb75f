// Internal declarations of the GB300 LES time-step library.
//
// Data layout in HBM: every 3-D array (fields, right-hand sides, RK3
// histories, eddy viscosities, Poisson source and solution) is a dense FP64
// array in the reference's Fortran (0:n1,0:n2,0:n3) layout, i fastest:
// element (i,j,k) at i + sx*j + sxy*k with sx = n1+1, sxy = (n1+1)(n2+1).
// Keeping the reference layout makes lesgpu_set_fields / get_fields a single
// contiguous copy and lets a warp read 32 consecutive i with one 256-byte
// transaction.  1-D metric vectors keep their Fortran index (x[1..n1],
// c2cx[0..n1]); index vectors are int32 on the device.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>
#include "../../include/lesgpu.h"

#define LG_HD __host__ __device__ __forceinline__

namespace lg {

constexpr int kThreads = 256;
constexpr int kRedBlocks = 608;        // 4 x 152 SMs: reduction grid, fixed for determinism
constexpr int kMaxRed = 8;             // values reduced together in one pass

struct DGrid {
    int n1, n2, n3, n1m, n2m, n3m, n1mh, n3mh;
    long long sx, sxy, nt;
    double xl, yl, zl;
    const double *x, *y, *z, *xmp, *ymp, *zmp;
    const double *f2fx, *f2fy, *f2fz, *f2fxi, *f2fyi, *f2fzi;
    const double *c2cx, *c2cy, *c2cz, *c2cxi, *c2cyi, *c2czi;
    const int *ipv, *jpv, *kpv, *imv, *jmv, *kmv;
    const int *fixil, *fixiu, *fixjl, *fixju, *fixkl, *fixku;
    int i_bgpx, j_bgpy, k_bgpz;
    LG_HD long long ix(long long i, long long j, long long k) const { return i + sx * j + sxy * k; }
};

struct DCfg {
    double re, pr, gr, udrv_i, tflu_i, tsol_i;
    double val_t_ybtm, val_t_ytop, val_t_zbtm, val_t_ztop;
    double resid1, csgsts, csgshf, cflfac, dt_size, ptb_tst, avg_tst, tend;
    int grdir, iles, ihtrans, ich, iconjg, idecomp, idvmon, filter, ibmon, masson, imovingon, iread;
    int xprdic, yprdic, zprdic;
    int bc_ybtm, bc_ytop, bc_zbtm, bc_ztop, bc_t_ybtm, bc_t_ytop, bc_t_zbtm, bc_t_ztop;
    int idtopt;
    int nintp[4], nbody[4];
    int nzero;
    int conj_tables;          // 1: ICONJG = 1 with a loaded c*, k* or omega value other than 1
    // constants of the R-templated stencils, formed once on the host exactly
    // as the kernels formed them per cell: [0] in FP64, [1] the FP32 form's
    // value (FP64 arithmetic on the FP32-rounded re, then rounded)
    double rei_d, inv_repr_d, gterm;   // 1/re, 1/(re pr), gr/re^2
    float rei_f, inv_repr_f;
    double adi_cd[3];                   // ADI: iles re, 2 iles re, iles re pr
    float adi_cf[3];
};

// Scalars of mod_common that change during a step.  They live in device
// memory so a whole step can run (and be captured in a CUDA graph) without
// a host round trip; the host reads them once at the end of the step.
struct DScal {
    double dt, time, subdt;
    double cflmax, dvmax, qmmax;
    double alpha, dtconst, dtconsti, test1, acoef, acoefi;
    double pmi[5], pmiavg, qvol[3], tvol[3], thcap;
    double pmiw[4];           // meanpg's wall-shear sums (y bottom, y top, z bottom, z top)
    double csgsts, csgshf, nutavg, nutmax, alpavg, alpmax;
    double err_integral;
    double dudta, dvdta, dwdta;
    double cd[3], heat_flux[3];
    double ubulk, qflux, tbulk_fluid, tbulk_solid;
    double u_bulk_t;          // rhs_t's bulk velocity of the current substep
    double phiref;            // pcalc's outlet-plane mean of phi
    double cvol;              // tvolcorr's volume integral of 1/c*
    double cb[4];             // convective outlet: qin, ucoef, vwcoef, qratio
    double mg_test;           // z_ft / x_ft multigrid convergence criterion of the substep
    long long avg_count;      // field_avg samples since the last reset
    long long ntime, m, ihist;
    long long poisson_iters[3];
    long long poisson_unconv; // solves of the step that stopped at MGITR above the tolerance
    double heat_body;         // thermal IB forcing's heat rate over the step (draglift's thermal term)
    int err;                  // device-side error flag (non-finite values etc.)
};

struct DFields {
    double *u, *v, *w, *p, *t;
    double *rhs1[4], *rk3o[4], *rk3oo[4];
    // the mixed form keeps the RK3 histories in FP32 (its FP32 stencils
    // produce them, so the storage is exact); null in the FP64 form
    float *rk3of[4], *rk3oof[4];
    double *nusgs, *nusgs1[3], *alsgs, *alsgs1[3];
    double *qmass, *divgsum, *phi;
    double *cstar, *kstar[6];
    int *omega, *nwall;
    double *fb_u, *fb_c;
    // per-cell weights of the volume reductions, formed once (k_red_weights):
    // wq = c2cx f2fy f2fz where fb_u >= 1e-10 (flow rate), wb the same where
    // fb_c >= 1e-10 (bulk velocity), wt = f2fx f2fy f2fz / c* (temperature)
    double *wq, *wb, *wt;
    // weights of the edge interpolation of nutinterpol / alpinterpol, 4 per
    // edge: ew1 over (j, k), ew2 over (k, i), ew3 over (i, j) (k_edge_interp)
    double *ew1, *ew2, *ew3;
    // body function on the y faces (xmp_i, y_1 | y_n2, zmp_k) and the z faces
    // (xmp_i, ymp_j, z_1 | z_n3), planes indexed i + (n1+1) * (k | j)
    double *fb_vb, *fb_vt, *fb_wb, *fb_wt;
    // convective outlet planes (0:n2,0:n3)
    double *uout, *vout, *wout, *tout, *duout, *dvout, *dwout, *dtout;
    // ADI coefficient vectors (lhsinit)
    double *aiu, *ciu, *aivw, *civw, *ajv, *cjv, *ajuw, *cjuw, *akw, *ckw, *akuv, *ckuv;
    // Simpson test-filter weights cf?1(n?m,-1:1)
    double *cfx1, *cfy1, *cfz1;
    // IB tables (component l = 0..3); 1-based rows
    int *ifc[4], *jfc[4], *kfc[4], *intpindx[4];
    double *geomfac[4], *fcv[4], *fcvavg[4], *dudtr[3];
    double *ibtarg[4];        // forcing targets of the current substep (two-phase forcing)
    int *inz, *jnz, *knz;
    // scratch
    double *scr[34];          // SGS temporaries / tridiagonal work, nt each
    double *part;             // reduction partials kRedBlocks * kMaxRed
    unsigned *red_count;      // blocks of the running reduction that have written their partials
    double *avg;              // field_avg sums: LESGPU_NAVG arrays of nt (IAVG = 1 only)
};

// Poisson FFT plan of one line length.
struct FftPlan {
    int n;
    int nst;
    int rad[24];
    double2 *tw;              // exp(-2 pi i e / n), e = 0..n-1 (device)
    float2 *twf;              // the same rounded to FP32
};

struct MgTables;              // poiss_z_ft multigrid tables (k_mg.cu)

struct MgrdTables;
struct DPois {
    double *ak1, *ak3;
    double2 *ccap;            // spectrum; ftft: (n1m, n3mh, n2m) i fastest, then k, then j;
                              // z_ft: (n1m, n2m, n3mh), one x-y plane per z mode;
                              // x_ft: (n3m, n2m, n1mh), one z-y plane per x mode
    FftPlan fx, fz;
    MgTables *mg;
    MgrdTables *mgrd;         // poiss_mgrd (BiCGSTAB + MG3D)
    double *ybet, *ygam, *yam, *pinref;   // poiss_ftft: LU of the y systems (k_ytri_lu)
    float *ybetf, *ygamf, *yamf, *pinreff;  // their FP32 copies (mixed form)
    int Lz, Lx;               // FFT lines per block (0 = the shared-memory rule; set by the autotuner)
    int mixed_fft;            // poiss_ftft in the mixed form: FP32 transforms, FP64 defect correction
    double *yres;             // its FP64 residual's y rows and diagonal, 3 per j
};

// The arrays a kernel of arithmetic type T reads in its stencils.  Mir<double>
// aliases the FP64 state; in the mixed form Mir<float> holds FP32 mirrors
// (1-D metrics and ADI tables converted once; fields, eddy viscosities and
// c*/k* refreshed by k_mirror where they change), so an FP32 kernel loads
// FP32 and converts nothing -- on GB300 an FP64->FP32 conversion issues on the
// narrow FP64 pipe, and a stencil converting every operand is bound by it.
template <class T>
struct Mir {
    const T *u, *v, *w, *p, *t;
    const T *nusgs, *nusgs1[3], *alsgs, *alsgs1[3];
    const T *cstar, *kstar[6];
    const T *f2fx, *f2fy, *f2fz, *f2fxi, *f2fyi, *f2fzi, *c2cxi, *c2cyi, *c2czi;
    const T *aiu, *ciu, *aivw, *civw, *ajv, *cjv, *ajuw, *cjuw, *akw, *ckw, *akuv, *ckuv;
    const T *cfx1, *cfy1, *cfz1;     // test-filter weights
    // the wall flags fix?? (1-based) as T: a stencil loads them instead of
    // converting an int per cell (conversions issue on GB300's FP64 pipe)
    const T *fixil, *fixiu, *fixjl, *fixju, *fixkl, *fixku;
};

struct KP {                   // everything a kernel may read, passed by value
    DGrid g;
    DCfg c;
    DFields f;
    DScal *S;
    Mir<double> md;
    Mir<float> mf;            // mixed form only (null otherwise)
};

template <class R> __device__ __forceinline__ R pickr(double d, float f);
template <> __device__ __forceinline__ double pickr<double>(double d, float) { return d; }
template <> __device__ __forceinline__ float pickr<float>(double, float f) { return f; }

// RK3 histories N^{k-1} and N^{k-2} of component l in the arithmetic type
template <class R> __device__ __forceinline__ R *hist_o(const KP &p, int l);
template <> __device__ __forceinline__ double *hist_o<double>(const KP &p, int l) { return p.f.rk3o[l]; }
template <> __device__ __forceinline__ float *hist_o<float>(const KP &p, int l) { return p.f.rk3of[l]; }
template <class R> __device__ __forceinline__ R *hist_oo(const KP &p, int l);
template <> __device__ __forceinline__ double *hist_oo<double>(const KP &p, int l) { return p.f.rk3oo[l]; }
template <> __device__ __forceinline__ float *hist_oo<float>(const KP &p, int l) { return p.f.rk3oof[l]; }

template <class R> __device__ __forceinline__ const Mir<R> &mir(const KP &p);
template <> __device__ __forceinline__ const Mir<double> &mir<double>(const KP &p) { return p.md; }
template <> __device__ __forceinline__ const Mir<float> &mir<float>(const KP &p) { return p.mf; }

// FP32 mirror refresh sets (k_mirror)
constexpr unsigned kMirU = 1, kMirV = 2, kMirW = 4, kMirP = 8, kMirT = 16, kMirNu = 32, kMirAl = 64, kMirConj = 128;
constexpr unsigned kMirVel = kMirU | kMirV | kMirW;

// ------------------------------------------------------------------ helpers
__device__ __forceinline__ double fixd(int v) { return (double)v; }

// Division of 0 <= n < 2^31 by an invariant d >= 1 as a multiply and a shift
// (Granlund & Montgomery, "Division by invariant integers using
// multiplication", PLDI 1994, theorem 4.2 with N = 31): l = ceil(log2 d),
// m = ceil(2^(31+l) / d) <= 2^32, n / d = (n m) >> (31 + l), n m < 2^63.
// A 64-bit integer division costs a GPU thread some sixty instructions.
struct IDiv {
    unsigned long long m;
    int s;
    LG_HD static IDiv make(int d) {
        int l = 0;
        while (l < 31 && (1LL << l) < (long long)d) l++;
        const int s = 31 + l;
        const unsigned long long dd = d > 0 ? (unsigned long long)d : 1ULL;
        return IDiv{((1ULL << s) + dd - 1ULL) / dd, s};
    }
    LG_HD unsigned div(unsigned n) const { return (unsigned)(((unsigned long long)n * m) >> s); }
};

// Decode a linear thread index over the interior box [i0..i1]x[j0..j1]x[k0..k1].
// Boxes of fewer than 2^31 points (every grid that fits in memory) decode
// with two multiply-shift divisions; larger ones fall back to 64-bit division.
struct Box {
    int i0, j0, k0, ni, nj, nk;
    IDiv di = IDiv::make(ni), dj = IDiv::make(nj);
    LG_HD long long count() const { return (long long)ni * nj * nk; }
    LG_HD void at(long long t, int &i, int &j, int &k) const {
        if (t < (1LL << 31)) {
            const unsigned t32 = (unsigned)t, r = di.div(t32), kk = dj.div(r);
            i = i0 + (int)(t32 - r * (unsigned)ni);
            j = j0 + (int)(r - kk * (unsigned)nj);
            k = k0 + (int)kk;
            return;
        }
        i = i0 + (int)(t % ni);
        long long r = t / ni;
        j = j0 + (int)(r % nj);
        k = k0 + (int)(r / nj);
    }
};

inline int blocks_for(long long n, int threads = kThreads) {
    long long b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > 0x7fffffffLL) b = 0x7fffffffLL;
    return (int)b;
}

// Deterministic block reduction of NV doubles (sum or max); result valid in thread 0.
template <int NV, bool MAX>
__device__ __forceinline__ void block_reduce(double (&v)[NV]) {
    __shared__ double sh[NV][kThreads / 32];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; q++) {
        double x = v[q];
        for (int o = 16; o > 0; o >>= 1) {
            double y = __shfl_down_sync(0xffffffffu, x, o);
            x = MAX ? fmax(x, y) : x + y;
        }
        if (lane == 0) sh[q][wid] = x;
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int q = 0; q < NV; q++) {
            double x = (lane < (int)(blockDim.x >> 5)) ? sh[q][lane] : (MAX ? -1.0e308 : 0.0);
            for (int o = 16; o > 0; o >>= 1) {
                double y = __shfl_down_sync(0xffffffffu, x, o);
                x = MAX ? fmax(x, y) : x + y;
            }
            v[q] = x;
        }
    }
    __syncthreads();
}

}  // namespace lg

// --------------------------------------------------------------- the case
struct lesgpu_case {
    lesgpu_config cfg;
    lg::KP kp;
    lg::DPois pois;
    cudaStream_t stream;
    cudaEvent_t ev[8];
    void *dmem_pool;           // single device allocation backing every array
    size_t dmem_bytes;
    lg::DScal *S;              // == kp.S
    lg::DScal hS;              // host copy after the last step
    int started;
    int ntime_host;
    cudaGraphExec_t graph;     // captured steady-state step
    int graph_ok;
    int use_graph;
    int autotune;              // use the autotuner's choices (LESGPU_AUTOTUNE != 0 at start)
    int strict;                // lesgpu_set_strict: unconverged Poisson solves are an error
    int bulk_solid;            // some interior cell centre lies inside a body (fb_c < 1e-10)
    // LESGPU_ADI_FP32_FORM at start: the form every FP32 sweep uses (lanes
    // per line, + 64 register-capped, 128 tiled; 0 = the autotuner's)
    int adi_force_f32;
    // FP32 mirror sets (kMir*) whose FP64 arrays changed since their last
    // refresh, as the enqueued work stands (host-side bookkeeping of the
    // mixed form; launch_mirror converts only these)
    unsigned mir_dirty;
    // 1 once a loaded conjugate table (c*, k*, omega) holds a value other
    // than 1; while 0 the temperature sweeps use the factored coefficients
    int conj_general;
    // host mirrors of metrics used for init-time tables
    double *h_f2fx, *h_f2fy, *h_f2fz;
    const lesgpu_grid *h_grid;  // the caller's grid, valid only inside lesgpu_create
    // kernel launches per step (from the captured graph)
    long long kernels_per_step;
    // event instrumentation of one kernel class (lesgpu_instrument)
    int inst_cls;
    int inst_n;
    cudaEvent_t inst_ev[2 * 4096];
    double inst_ms;
    long long inst_launches;
};

namespace lg {
// bracket a launch of class `cls` with events when that class is instrumented
inline void inst_begin(lesgpu_case *c, int cls) {
    if (c->inst_cls == cls && c->inst_n < 4096) cudaEventRecord(c->inst_ev[2 * c->inst_n], c->stream);
}
inline void inst_end(lesgpu_case *c, int cls) {
    if (c->inst_cls == cls && c->inst_n < 4096) { cudaEventRecord(c->inst_ev[2 * c->inst_n + 1], c->stream); c->inst_n++; }
}
}  // namespace lg

namespace lg {
// launch wrappers implemented in the k_*.cu files
void launch_stepinit(lesgpu_case *c);
void launch_substepinit(lesgpu_case *c, int msub);
void launch_qvolcalc(lesgpu_case *c, int slot);
void launch_tvolcalc(lesgpu_case *c, int slot);
// tvolcalc(tvol(2)) + tvolcorr; slot0: also tvol(0) (tcalc will not change t)
void launch_tvolcalc_corr(lesgpu_case *c, bool slot0);
void launch_meanpg(lesgpu_case *c);
// ucalc; with_qvol: fused with the qvolcalc before (qvol(2)) and after (qvol(0))
void launch_ucalc_pcalc(lesgpu_case *c, bool with_qvol);
void launch_tcalc(lesgpu_case *c);
void launch_advance_and_convergence(lesgpu_case *c);
void launch_bulk_diag(lesgpu_case *c);
void launch_rhs(lesgpu_case *c, int msub);
void launch_divgs(lesgpu_case *c);
void launch_ghost_uvw(lesgpu_case *c);
// rhs_t with its bulk velocity; with_tvol: tvolcalc(tvol(1)) in the same reduction
void launch_rhs_t(lesgpu_case *c, int msub, bool with_tvol);
void launch_energy_bc(lesgpu_case *c);
void launch_adi_uvw(lesgpu_case *c);
void launch_adi_t(lesgpu_case *c);
void launch_sgs(lesgpu_case *c);
void launch_sgs_t(lesgpu_case *c);
void launch_poisson(lesgpu_case *c, int msub);
int poisson_init(lesgpu_case *c);
void poisson_free(lesgpu_case *c);
void launch_sgs_zero_first(lesgpu_case *c, int thermal);
void launch_rhs_ibm(lesgpu_case *c);
void launch_rhs_ibm_t(lesgpu_case *c);
void launch_divgs_ibm(lesgpu_case *c);
void launch_lagforce(lesgpu_case *c, int msub);
void launch_draglift(lesgpu_case *c);
void launch_heatflux(lesgpu_case *c);
void launch_convbc(lesgpu_case *c);
void launch_convbc_t(lesgpu_case *c);
void launch_field_avg(lesgpu_case *c);
}  // namespace lg

namespace lg {
// ----------------------------------------------------------- generic sums
// One-launch reduction: every block writes its partials; the last block to
// finish (counted with an atomic ticket after a release fence) sums all the
// partials in block order -- the same fixed order as a separate finalize
// kernel, so results are deterministic -- applies g and resets the ticket.
template <int NV, bool MAX, class F, class G>
__global__ void __launch_bounds__(kThreads, 4) k_reduce_fin(KP p, Box b, F f, G g) {
    __shared__ int last;
    double v[NV];
#pragma unroll
    for (int q = 0; q < NV; q++) v[q] = MAX ? -1.0e308 : 0.0;
    const long long n = b.count();
    const long long S = (long long)gridDim.x * blockDim.x;
    // a sum skips exact +0 terms (integer test): FP64 adds issue on the
    // narrow FP64 pipe, and several reductions carry terms that are zero
    // almost everywhere (the wall-shear sums of meanpg)
    auto add_terms = [&](const double (&w)[NV]) {
#pragma unroll
        for (int q = 0; q < NV; q++) {
            if (MAX) v[q] = fmax(v[q], w[q]);
            else if (__double_as_longlong(w[q]) != 0LL) v[q] = v[q] + w[q];
        }
    };
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    // U elements of the thread's sequence per pass (4, 2 for six sums: 4
    // blocks of 256 threads an SM leave 64 registers a thread): their terms
    // are all formed (loads in flight together) before they are added, in
    // the sequence's order -- the sums of the one-at-a-time loop, bit for bit
    constexpr int U = NV >= 6 ? 2 : 4;
    for (; t + (U - 1) * S < n; t += U * S) {
        double w[U][NV];
#pragma unroll
        for (int u = 0; u < U; u++) {
            int i, j, k;
            b.at(t + u * S, i, j, k);
            f(p, i, j, k, w[u]);
        }
#pragma unroll
        for (int u = 0; u < U; u++) add_terms(w[u]);
    }
    for (; t < n; t += S) {
        int i, j, k;
        b.at(t, i, j, k);
        double w[NV];
        f(p, i, j, k, w);
        add_terms(w);
    }
    block_reduce<NV, MAX>(v);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NV; q++) p.f.part[(size_t)blockIdx.x * kMaxRed + q] = v[q];
        __threadfence();
        last = atomicAdd(p.f.red_count, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double acc[NV];
#pragma unroll
    for (int q = 0; q < NV; q++) acc[q] = MAX ? -1.0e308 : 0.0;
    for (int bk = threadIdx.x; bk < (int)gridDim.x; bk += blockDim.x)
#pragma unroll
        for (int q = 0; q < NV; q++) {
            const double x = __ldcg(p.f.part + (size_t)bk * kMaxRed + q);
            acc[q] = MAX ? fmax(acc[q], x) : acc[q] + x;
        }
    block_reduce<NV, MAX>(acc);
    if (threadIdx.x == 0) {
        g(p, acc);
        *p.f.red_count = 0u;
    }
}

template <int NV, bool MAX, class F, class G>
inline void reduce(lesgpu_case *c, Box b, F f, G g) {
    int nb = blocks_for(b.count());
    if (nb > kRedBlocks) nb = kRedBlocks;
    k_reduce_fin<NV, MAX><<<nb, kThreads, 0, c->stream>>>(c->kp, b, f, g);
}


// Periodic ghost copy of one plane pair (see k_ghost in k_aux.cu).
struct GhostSpec {
    double *a;
    int lo0, hi0, lo1, hi1;   // ranges of the two in-plane indices (in index order)
};
void ghost(lesgpu_case *c, int dir, GhostSpec *s, int na);
// refresh FP32 mirrors (mixed form; no-op in the FP64 form)
void launch_mirror(lesgpu_case *c, unsigned sets);
// note that enqueued work changes the FP64 arrays of `sets`
inline void mark_mirror(lesgpu_case *c, unsigned sets) { c->mir_dirty |= sets; }
// autotuner (k_adi.cu): time the sweep classes of this shape once per process
int adi_autotune(lesgpu_case *c);
// autotuner (k_fft.cu): FFT lines per block of the case's Poisson transforms
int fft_autotune(lesgpu_case *c);
// autotuner (k_mg.cu): cluster size of the z_ft multigrid; the chosen size
int mg2d_autotune(lesgpu_case *c);
int mg2d_cluster(const lesgpu_case *c);
int adi_tuned(const lesgpu_case *c, int *out, int maxn);
// cap on the z_ft multigrid's cluster size for cases created by this thread (0 = none)
void set_mg_cluster_cap(int cap);
void launch_cvol(lesgpu_case *c);
// the reduction weights (DFields wq, wb, wt); after fb_u/fb_c or c* change
void launch_red_weights(lesgpu_case *c);
void launch_rhs_t_kernel(lesgpu_case *c, int msub);
// poiss_z_ft / poiss_x_ft in pieces, for the serving loop's batched solve
// (k_mg.cu): the transforms before and after the mode solves, the solve's
// arguments of one case (mg2d_batch_size bytes), one launch over n cases of
// one shape, and what the cases must share for it (cluster size, levels)
void mg2d_launch_pre(lesgpu_case *c, int msub);
void mg2d_launch_post(lesgpu_case *c);
int mg2d_batch_size(const lesgpu_case *c);
void mg2d_batch_args(lesgpu_case *c, int msub, void *out);
void mg2d_launch_batch(const lesgpu_case *c0, const void *d_args, int n, cudaStream_t st);
long long mg2d_batch_key(const lesgpu_case *c);
// one step of n cases of one shape captured as a CUDA graph on stream st
// (lesgpu_api.cu), the host bookkeeping after each replay of it, and the
// out-of-date mirrors refreshed before the first replay
struct BucketGraph {
    cudaGraphExec_t exec = nullptr;
    void *d_args = nullptr;      // batched solve arguments, 3 substeps x n cases
    long long kernels = 0;       // kernel nodes of the graph
};
int capture_bucket_step(lesgpu_case **cs, int n, cudaStream_t st, BucketGraph *bg);
void free_bucket_graph(BucketGraph *bg);
int bucket_prologue(lesgpu_case **cs, int n);
void bucket_replayed(lesgpu_case **cs, int n, int steps);
}  // namespace lg
