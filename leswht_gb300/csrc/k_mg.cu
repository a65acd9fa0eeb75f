// Pressure Poisson solves of poiss_z_ft.f90 and poiss_x_ft.f90.  z_ft: FFT
// in z, then for each of the n3mh z modes a complex 2-D problem in x-y
// solved by the reference's multigrid -- semi-coarsened in x (levels of n1m,
// n1m/2, ... x-lines), zebra x-line relaxation with y-Thomas solves, linear
// restriction and the prolongation onto the even lines only -- or, for modes
// above IMGSOR, by zebra line SOR.  x_ft is the same with x and z exchanged
// (FFT in x, n1mh modes, each a z-y problem semi-coarsened in z), except
// where poiss_x_ft.f90 differs: the zero wavenumber's odd lines are shifted
// by ggii(1,n2m) before the even lines are formed (toplevel and gsor2d), the
// prolongation runs over every coarse point with coi2 (the last one's is the
// periodic weight or zero), the convergence criterion carries 0.9, and phi
// gets the upper-wall mean removed when ICH = 1.  Below, "line" / i is the
// semi-coarsened direction (x for z_ft, z for x_ft) and kv the mode.
//
// GPU design: one thread block per z mode runs that mode's whole solve
// (every V-cycle and its convergence test) as one launch; the phases of a
// cycle are separated by block barriers, so the iteration count needs no
// host round trip and the solve can sit inside the step's CUDA graph.
// Within a phase, the y-Thomas solve of an x-line is done by one warp: each
// lane composes the affine maps of its chunk of rows, a 5-step shuffle scan
// joins the chunks, and each lane re-runs its chunk with the reference's
// recurrence from the scanned incoming value (forward elimination with the
// precomputed LU factors, then back substitution the same way).  That cuts
// the dependent chain of a 192-row line from 384 steps to about 30.
//
// Tables (pmat :55-94, mwavenumber :97-113, coefmg :643-798, the LU factors
// of poisinit :18-52) are built on the host in the reference's arithmetic
// order and uploaded once.
#include "k_fft.cuh"
#include <cooperative_groups.h>
#include <new>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <vector>
#include <array>
#include <map>
#include <mutex>

namespace lg {

// threads per block: 256, so a thread may hold up to 255 registers -- the
// 128 of a 512-thread block spill the sweeps' line arrays and the values
// live across the phase calls to local memory, which 512 threads' stacks
// push out of L1
constexpr int kMgThreads = 256;
constexpr int kMC = 8;            // rows per lane: y lines of up to 32 * kMC = 256 cells
constexpr int kMaxLev = 20;

int mg_cluster_cap();

template <class T> struct V2;
template <> struct V2<double> {
    using t = double2;
    __host__ __device__ static double2 mk(double x, double y) { return make_double2(x, y); }
};
template <> struct V2<float> {
    using t = float2;
    __host__ __device__ static float2 mk(float x, float y) { return make_float2(x, y); }
};

// Coefficient tables and per-mode work arrays of one arithmetic type.
template <class T>
struct MgSet {
    T *aw, *ae, *as, *an, *coi1, *coi2, *cor1, *cor2;   // 1-based
    T *ac, *bet, *gam;          // (i-1) + nld*((j-1) + n2m*(kv-1))
    typename V2<T>::t *pc, *gg, *rs;
    // rd: the defect of a level partitioned over the cluster (its godown
    // result, kept apart from the restricted residual in rs that neighbouring
    // blocks still read in the same phase); gu: prolonged even lines; gb:
    // a copy of a partitioned level's even lines after its down-sweep
    // relaxation, the base its prolongation adds to (read by neighbouring
    // blocks while the owner overwrites gg)
    typename V2<T>::t *rd, *gu, *gb;
};

struct MgTables {
    int nl, nld, nlev;          // cells along the semi-coarsened direction, 2 nl, levels
    int nmodes, xft;            // modes solved (n3mh / n1mh); 1 for poiss_x_ft
    int mixed;                  // FP32 cycles under an FP64 defect correction
    int cs;                     // blocks per cluster (one cluster per z mode)
    int lc;                     // levels 0..lc run on one block of the cluster
    int cap;                    // cap on cs set by the creator (0 = none)
    int iimg[kMaxLev + 1][3];
    int *ipm, *imm;
    MgSet<double> d;            // FP64 tables and work arrays
    MgSet<float> f;             // their FP32 copies (mixed form)
    long long *iters;           // per mode, last solve
    long long pc_plane, gg_plane;
};

struct MgArgs {
    int nl, n2m, nld, nlev, nbli, mgitr, imgsor;
    int xft;                    // poiss_x_ft's pinning and prolongation
    int mixed;
    double wwsor;
    int ldp, ldg;
    int iimg[kMaxLev + 1][3];
    const int *ipm, *imm;
    MgSet<double> d;
    MgSet<float> f;
    double2 *ccap;
    long long pc_plane, gg_plane;
    long long *iters;
    DScal *S;
    int slot;
    int fixed_cycles;           // > 0: run exactly this many cycles (autotuner timing), no test
    int lc;                     // levels 0..lc (at most kCoarseLines lines) run on one block
};

// ------------------------------------------------------------- device side
// One z mode is solved by one thread-block cluster; tid() / nt() number the
// threads of the whole cluster and sync() is the cluster barrier (release /
// acquire at cluster scope, so global writes of a phase are visible to every
// block of the cluster in the next phase).  ModeT<T> views the mode's tables
// and work arrays of arithmetic type T.  A view holds only what is the same
// for every thread of a block, so one copy of it (and of the launch's
// MgArgs) sits in the block's shared memory: the phases, compiled apart,
// read their fields from there instead of each thread keeping its own copy
// on the stack.
template <class T>
struct ModeT {
    using V = typename V2<T>::t;
    const MgArgs &a;
    const MgSet<T> &s;
    int kv;
    int rank, csz;                      // the block's rank in the cluster, blocks in it
    bool local;                         // the threads are one block's: sync() is the block barrier
    V *pc, *gg, *rs, *rd, *gu, *gb;
    const double2 *rhs;                 // ccap plane of the mode, (i-1) + nl*(j-1)
    size_t cb;                          // coefficient base of the mode
    __device__ void sync() const {
        if (local) __syncthreads();
        else cooperative_groups::this_cluster().sync();
    }
    // thread index / count over the cluster (or the block).  Warp w of
    // block r is the cluster's warp w*csz + r: consecutive lines and 32-point
    // chunks go to different SMs (the work of a phase is spread over every
    // block, each warp still touches 32 consecutive points).
    __device__ int tid() const {
        if (local) return (int)threadIdx.x;
        return (((int)threadIdx.x >> 5) * csz + rank) * 32 + ((int)threadIdx.x & 31);
    }
    __device__ int nt() const { return local ? (int)blockDim.x : csz * (int)blockDim.x; }
    __device__ ModeT(const MgArgs &a_, const MgSet<T> &s_, int kv_, bool local_, int rank_, int csz_)
        : a(a_), s(s_), kv(kv_), rank(rank_), csz(csz_), local(local_) {
        pc = s.pc + a.pc_plane * (kv - 1);
        gg = s.gg + a.gg_plane * (kv - 1);
        rs = s.rs + a.gg_plane * (kv - 1);
        rd = s.rd + a.gg_plane * (kv - 1);
        gu = s.gu + a.gg_plane * (kv - 1);
        gb = s.gb + a.gg_plane * (kv - 1);
        rhs = a.ccap + (size_t)a.nl * a.n2m * (kv - 1);
        cb = (size_t)a.nld * a.n2m * (kv - 1);
    }
    __device__ V &P(int i, int j) const { return pc[i + (size_t)a.ldp * j]; }
    __device__ V &G(int i, int j) const { return gg[i + (size_t)a.ldg * j]; }
    __device__ V &R(int i, int j) const { return rs[i + (size_t)a.ldg * j]; }
    __device__ V &D(int i, int j) const { return rd[i + (size_t)a.ldg * j]; }
    __device__ V &U(int i, int j) const { return gu[i + (size_t)a.ldg * j]; }
    __device__ V &GB(int i, int j) const { return gb[i + (size_t)a.ldg * j]; }
    __device__ double2 B(int i, int j) const { return rhs[(i - 1) + (size_t)a.nl * (j - 1)]; }
    __device__ T AC(int i, int j) const { return s.ac[cb + (i - 1) + (size_t)a.nld * (j - 1)]; }
};
using Mode = ModeT<double>;

template <class V, class T>
__device__ __forceinline__ V axmy(V y, T s, V x) {   // y - s*x
    return V{y.x - s * x.x, y.y - s * x.y};
}

// trdiag1m (poiss_z_ft.f90:383-408) of one x-line held in registers: lane
// `lane` owns rows j0..j0+cnt-1 (v, with as_j, bet_j and gam_{j+1} beside
// them; gam_{n2m+1} = 0).  Affine maps of the chunks are composed, joined by
// a shuffle scan, then each chunk is re-run with the reference recurrence
// from its scanned incoming value (see the file comment).
template <int MC, class T, class V>
__device__ __forceinline__ void line_solve(V (&v)[MC], const T (&as_)[MC], const T (&bt)[MC],
                                           const T (&gm)[MC], int cnt, int lane) {
    T A = T(1.0);
    V Bv = V{T(0.0), T(0.0)};
#pragma unroll
    for (int q = 0; q < MC; q++)
        if (q < cnt) {
            const T aj = -as_[q] * bt[q];
            Bv = V{aj * Bv.x + v[q].x * bt[q], aj * Bv.y + v[q].y * bt[q]};
            A = aj * A;
        }
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const T Ap = __shfl_up_sync(0xffffffffu, A, d);
        const T bx = __shfl_up_sync(0xffffffffu, Bv.x, d), by = __shfl_up_sync(0xffffffffu, Bv.y, d);
        if (lane >= d) { Bv = V{A * bx + Bv.x, A * by + Bv.y}; A = A * Ap; }
    }
    T yx = __shfl_up_sync(0xffffffffu, Bv.x, 1), yy = __shfl_up_sync(0xffffffffu, Bv.y, 1);
    if (lane == 0) { yx = T(0.0); yy = T(0.0); }
#pragma unroll
    for (int q = 0; q < MC; q++)
        if (q < cnt) {
            yx = (v[q].x - as_[q] * yx) * bt[q];
            yy = (v[q].y - as_[q] * yy) * bt[q];
            v[q] = V{yx, yy};
        }
    T C = T(1.0);
    V D = V{T(0.0), T(0.0)};
#pragma unroll
    for (int q = MC - 1; q >= 0; q--)
        if (q < cnt) {
            const T cj = -gm[q];
            D = V{cj * D.x + v[q].x, cj * D.y + v[q].y};
            C = cj * C;
        }
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const T Cn = __shfl_down_sync(0xffffffffu, C, d);
        const T dx = __shfl_down_sync(0xffffffffu, D.x, d), dy = __shfl_down_sync(0xffffffffu, D.y, d);
        if (lane + d < 32) { D = V{C * dx + D.x, C * dy + D.y}; C = C * Cn; }
    }
    T xx = __shfl_down_sync(0xffffffffu, D.x, 1), xy = __shfl_down_sync(0xffffffffu, D.y, 1);
    if (lane == 31) { xx = T(0.0); xy = T(0.0); }
#pragma unroll
    for (int q = MC - 1; q >= 0; q--)
        if (q < cnt) {
            xx = v[q].x - gm[q] * xx;
            xy = v[q].y - gm[q] * xy;
            v[q] = V{xx, xy};
        }
}

// How the right-hand side of a line is formed before its y solve.
enum HalfKind {
    H_ODD = 0,      // src - ov*(aw*nb(imm) + ae*nb(ipm))      toplevel/relax odd lines, gsor
    H_EVEN = 1,     // src - aw*nb(imm) - ae*nb(ipm)            relax even lines
    H_EVEN_TT = 2,  // src - aw*(nb(imm)-tt) - ae*(nb(ipm)-tt)   toplevel even lines (pinned mode)
};

// One zebra half sweep: lines l1, l1+2, ..., l2; one warp per line.
//   src: the rhs plane (top level) or resd; nb: the array the neighbours come from
//   out: G(i,j) = solution, or for gsor P(i,j) = ww*solution + o2*P(i,j)
template <int MC, class T>
__device__ __noinline__ void mg_half(const ModeT<T> &m, int l1, int l2, int kind, bool src_rhs,
                                     const typename V2<T>::t *nb, int ldn, T ov, typename V2<T>::t tt, bool gsor,
                                     T ww, T o2) {
    using V = typename V2<T>::t;
    const MgArgs &a = m.a;
    const MgSet<T> &s = m.s;
    if (l2 < l1) return;
    const int tid = m.tid(), lane = tid & 31, warp = tid >> 5, nw = m.nt() >> 5;
    const int n2m = a.n2m, nl = (l2 - l1) / 2 + 1;
    const int ch = (n2m + 31) / 32;
    const int j0 = 1 + lane * ch;
    const int cnt = max(0, min(ch, n2m - j0 + 1));
    const size_t sj = (size_t)a.nld;
    for (int li = warp; li < nl; li += nw) {
        const int i = l1 + 2 * li;
        const int im = a.imm[i], ip = a.ipm[i];
        const T aw = s.aw[i], ae = s.ae[i];
        const T *bet = s.bet + m.cb + (i - 1);
        const T *gam = s.gam + m.cb + (i - 1);
        V v[MC];
        T as_[MC], bt[MC], gm[MC];
#pragma unroll
        for (int q = 0; q < MC; q++)
            if (q < cnt) {
                const int j = j0 + q;
                V sr;
                if (src_rhs) {
                    const double2 b = m.B(i, j);
                    sr = V{T(b.x), T(b.y)};
                } else {
                    sr = m.R(i, j);
                }
                V nm = nb[im + (size_t)ldn * j], np = nb[ip + (size_t)ldn * j];
                if (kind == H_ODD) {
                    const T sx = aw * nm.x + ae * np.x, sy = aw * nm.y + ae * np.y;
                    v[q] = V{sr.x - ov * sx, sr.y - ov * sy};
                } else if (kind == H_EVEN) {
                    v[q] = V{sr.x - aw * nm.x - ae * np.x, sr.y - aw * nm.y - ae * np.y};
                } else {
                    nm = V{nm.x - tt.x, nm.y - tt.y};
                    if (ip < i) np = V{np.x - tt.x, np.y - tt.y};   // x-periodic wrap: shifted already
                    v[q] = V{sr.x - aw * nm.x - ae * (np.x - tt.x), sr.y - aw * nm.y - ae * (np.y - tt.y)};
                }
                as_[q] = s.as[j];
                bt[q] = bet[sj * (j - 1)];
                gm[q] = j < n2m ? gam[sj * j] : T(0.0);
            }
        line_solve<MC>(v, as_, bt, gm, cnt, lane);
#pragma unroll
        for (int q = 0; q < MC; q++)
            if (q < cnt) {
                const int j = j0 + q;
                if (gsor) {
                    const V u = m.P(i, j);
                    m.P(i, j) = V{ww * v[q].x + o2 * u.x, ww * v[q].y + o2 * u.y};
                } else {
                    m.G(i, j) = v[q];
                }
            }
    }
}

// src - aw*g(imm) - ae*g(ipm) - as*g(j-1) - an*g(j+1) - ac*g  on the array g
template <class T>
__device__ __forceinline__ typename V2<T>::t mg_defect(const ModeT<T> &m, typename V2<T>::t src,
                                                      const typename V2<T>::t *g, int ld, int i, int j) {
    const MgArgs &a = m.a;
    const MgSet<T> &s = m.s;
    src = axmy(src, s.aw[i], g[a.imm[i] + (size_t)ld * j]);
    src = axmy(src, s.ae[i], g[a.ipm[i] + (size_t)ld * j]);
    src = axmy(src, s.as[j], g[i + (size_t)ld * (j - 1)]);
    src = axmy(src, s.an[j], g[i + (size_t)ld * (j + 1)]);
    src = axmy(src, m.AC(i, j), g[i + (size_t)ld * j]);
    return src;
}

// The max of every block's *v (a shared-memory variable at the same place in
// each block) through distributed shared memory: lane q reads block q's
// (clusters have at most 16 blocks), then a warp max; every thread gets the
// same result (max is exact and order-free).
__device__ __forceinline__ double dsm_max(cooperative_groups::cluster_group &cl, double *v) {
    const int lane = threadIdx.x & 31;
    double r = lane < (int)cl.num_blocks() ? *cl.map_shared_rank(v, lane) : 0.0;
    for (int o = 16; o > 0; o >>= 1) r = fmax(r, __shfl_xor_sync(0xffffffffu, r, o));
    return r;
}

// Max over the cluster: warp shuffles, one value per block in shared memory,
// then every thread reads every block's value through distributed shared
// memory, so all threads get the same result.
__device__ double cluster_max(double v) {
    __shared__ double sh[kMgThreads / 32];
    __shared__ double blk;
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    if (lane == 0) sh[w] = v;
    cl.sync();
    if (threadIdx.x == 0) {
        double r = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) r = fmax(r, sh[q]);
        blk = r;
    }
    cl.sync();
    const double r = dsm_max(cl, &blk);
    cl.sync();          // nobody overwrites blk before every block has read it
    return r;
}

// Subtract tt from the odd lines of u (ld: leading dimension) -- the zero
// wavenumber's pin of poiss_x_ft.f90:328-335, 533-540 and 582-589.  tt was read by
// every thread before the barrier in front of this.
template <class T>
__device__ void mg_shift_odd(const ModeT<T> &m, typename V2<T>::t *u, int ld, typename V2<T>::t tt) {
    const int nh = m.a.nl / 2, n2m = m.a.n2m;
    for (int t = m.tid(); t < nh * n2m; t += m.nt()) {
        const int i = 1 + 2 * (t % nh), j = 1 + t / nh;
        typename V2<T>::t &g = u[i + (size_t)ld * j];
        g = typename V2<T>::t{g.x - tt.x, g.y - tt.y};
    }
}

// relax, poiss_z_ft.f90:466-511 (zebra version)
template <int MC, class T>
__device__ __noinline__ void mg_relax(const ModeT<T> &m, int ilev, T oldv, int iiter) {
    const MgArgs &a = m.a;
    const int ibg = a.iimg[ilev][0], iend = a.iimg[ilev][1];
    const typename V2<T>::t zero{T(0.0), T(0.0)};
    for (int it = 0; it < iiter; it++) {
        const T ov = it == 0 ? oldv : T(1.0);
        mg_half<MC, T>(m, ibg, iend, H_ODD, false, m.gg, a.ldg, ov, zero, false, T(0.0), T(0.0));
        m.sync();
        mg_half<MC, T>(m, ibg + 1, iend, H_EVEN, false, m.gg, a.ldg, T(1.0), zero, false, T(0.0), T(0.0));
        m.sync();
    }
}

// Points of godown and goup go kMgBatch<T> at a time per thread: all of
// their loads before any of their stores (no point of either phase reads
// what another point of it writes), so the loads are in flight together
// instead of one round trip per point behind the previous point's store.
// FP32 phases only: batched FP64 points raise the register demand of the
// whole call graph, and ptxas then spills in the 192- and 256-row instances.
template <class T> constexpr int kMgBatch = sizeof(T) == 4 ? 4 : 1;

// godown, poiss_z_ft.f90:438-463
template <class T>
__device__ __noinline__ void mg_godown(const ModeT<T> &m, int ilev) {
    using V = typename V2<T>::t;
    constexpr int B = kMgBatch<T>;
    const MgArgs &a = m.a;
    const int ibg = a.iimg[ilev][0], iend = a.iimg[ilev][1], n2m = a.n2m, nt = m.nt();
    const int nf = iend - ibg + 1;
    for (int t0 = m.tid(); t0 < nf * n2m; t0 += B * nt) {
        V d[B];
#pragma unroll
        for (int q = 0; q < B; q++) {
            const int t = t0 + q * nt;
            if (t < nf * n2m) {
                const int i = ibg + t % nf, j = 1 + t / nf;
                d[q] = mg_defect(m, m.R(i, j), m.gg, a.ldg, i, j);
            }
        }
#pragma unroll
        for (int q = 0; q < B; q++) {
            const int t = t0 + q * nt;
            if (t < nf * n2m) m.R(ibg + t % nf, 1 + t / nf) = d[q];
        }
    }
    m.sync();
    const int cl = a.iimg[ilev - 1][0], nc = a.iimg[ilev - 1][1] - cl + 1;
    for (int t0 = m.tid(); t0 < nc * n2m; t0 += B * nt) {
        V d[B];
#pragma unroll
        for (int q = 0; q < B; q++) {
            const int t = t0 + q * nt;
            if (t < nc * n2m) {
                const int i = cl + t % nc, j = 1 + t / nc, f = ibg + 2 * (i - cl);
                const V r1 = m.R(f, j), r2 = m.R(f + 1, j);
                d[q] = V{r1.x * m.s.cor1[i] + r2.x * m.s.cor2[i], r1.y * m.s.cor1[i] + r2.y * m.s.cor2[i]};
            }
        }
#pragma unroll
        for (int q = 0; q < B; q++) {
            const int t = t0 + q * nt;
            if (t < nc * n2m) m.R(cl + t % nc, 1 + t / nc) = d[q];
        }
    }
    m.sync();
}

// goup, poiss_z_ft.f90:411-435 / poiss_x_ft.f90:401-419
template <class T>
__device__ __noinline__ void mg_goup(const ModeT<T> &m, int ilev) {
    using V = typename V2<T>::t;
    constexpr int B = kMgBatch<T>;
    const MgArgs &a = m.a;
    const MgSet<T> &s = m.s;
    const int cl = a.iimg[ilev][0], ce = a.iimg[ilev][1], n2m = a.n2m, nt = m.nt();
    const int fb = a.iimg[ilev + 1][0], nc = ce - cl + 1;
    for (int t0 = m.tid(); t0 < nc * n2m; t0 += B * nt) {
        V d[B];
#pragma unroll
        for (int q = 0; q < B; q++) {
            const int t = t0 + q * nt;
            if (t < nc * n2m) {
                const int i = cl + t % nc, j = 1 + t / nc, f = fb + 1 + 2 * (i - cl);
                const V g = m.G(f, j), g1 = m.G(i, j);
                if (i < ce || a.xft) {
                    const V g2 = m.G(a.ipm[i], j);
                    d[q] = V{g.x + s.coi1[i] * g1.x + s.coi2[i] * g2.x, g.y + s.coi1[i] * g1.y + s.coi2[i] * g2.y};
                } else {
                    d[q] = V{g.x + s.coi1[i] * g1.x, g.y + s.coi1[i] * g1.y};
                }
            }
        }
#pragma unroll
        for (int q = 0; q < B; q++) {
            const int t = t0 + q * nt;
            if (t < nc * n2m) m.G(fb + 1 + 2 * (t % nc), 1 + t / nc) = d[q];
        }
    }
    m.sync();
}

// gsor2d + resid3, poiss_z_ft.f90:513-641 / poiss_x_ft.f90:497-642 (pc is the iterate u)
template <int MC>
__device__ __noinline__ int mg_gsor2d(const Mode &m, double test, bool &unconv) {
    const MgArgs &a = m.a;
    const int n1m = a.nl, n2m = a.n2m, nt = m.nt();
    const double ww = a.wwsor, ww2 = 1.0 - ww;
    for (int kk = 0; kk <= a.mgitr; kk++) {
        const double ov = kk == 0 ? 0.0 : 1.0, o2 = ov * ww2;
        for (int half = 0; half < 2; half++) {
            const double f = half == 0 ? ov : 1.0;
            mg_half<MC, double>(m, 1 + half, n1m, H_ODD, true, m.pc, a.ldp, f, make_double2(0.0, 0.0), true, ww, o2);
            m.sync();
            if (half == 0 && a.xft && m.kv == 1) {     // poiss_x_ft pins the zero wavenumber by u(1,n2m)
                const double2 tt = m.P(1, n2m);
                m.sync();
                mg_shift_odd(m, m.pc, a.ldp, tt);
                m.sync();
            }
        }
        double mx = 0.0;
        for (int t = m.tid(); t < n1m * n2m; t += nt) {
            const int i = 1 + t % n1m, j = 1 + t / n1m;
            const double2 d = mg_defect(m, m.B(i, j), m.pc, a.ldp, i, j);
            mx = fmax(mx, d.x * d.x + d.y * d.y);
        }
        const double e = sqrt(cluster_max(mx));
        if (e < test) return kk;
    }
    unconv = true;
    return a.mgitr;
}

// ---------------------------------------------------------------------------
// Level-partitioned V-cycle (the cycle of mg_mg2d / mg_mg2d_mixed with the
// same per-point arithmetic).  The phases above spread every level's lines
// over the whole cluster and put a cluster barrier after each half sweep,
// defect, restriction and prolongation: about forty barriers per V-cycle,
// which bound the solve.  Here:
//   * on the top level and on every level of more than kCoarseLines lines,
//     block r of the cluster owns a contiguous, even-aligned range of lines
//     [a, b]; the few lines just outside it that its own lines depend on
//     inside one phase (the halo: at most the two lines before a and the
//     two after b, cyclically on a periodic level) are recomputed by the
//     block into shared memory, so a whole relaxation + defect +
//     restriction, or a prolongation + relaxation, needs one cluster
//     barrier at its end and only block barriers inside;
//   * the levels of at most kCoarseLines lines run on block 0 alone with
//     block barriers (the phases above with a block-local mode view), the
//     other blocks waiting at one cluster barrier -- or, in the mixed form
//     with 16-block clusters, spread over the cluster with a cluster barrier
//     per phase, all but the coarsest level's relaxations (measured faster
//     both ways on the 256x192 modes, slower with small clusters);
//   * the defect of a partitioned level goes to rd, not over the restricted
//     residual in rs that neighbouring blocks still read in the same phase
//     (the reference overwrites resd with it, poiss_z_ft.f90:447-452; the
//     post-smoothing of the level reads it from rd, the same values), and
//     prolonged even lines go to gu (scratch) for the same reason;
//   * the max-norm test exchanges one value per block through distributed
//     shared memory at the phase's closing barrier.
// A V-cycle takes 2 + 2 (levels above kCoarseLines lines below the top) + 1
// cluster barriers.
constexpr int kCoarseLines = 32;
constexpr int kHalo = 6;
constexpr int kHaloRows = 32 * kMC + 2;

// lines [ibg, iend] of a level; the block owns [a, b]
struct Part {
    int ibg, iend, a, b;
    __device__ bool in(int i) const { return i >= ibg && i <= iend; }
    __device__ bool own(int i) const { return i >= a && i <= b; }
};
__device__ __forceinline__ Part part_of(int ibg, int iend, int r, int cs) {
    const int nb = (iend - ibg + 1) / cs;
    return Part{ibg, iend, ibg + r * nb, ibg + r * nb + nb - 1};
}

// halo lines of a phase and their rows in shared memory
template <class V>
struct Halo {
    int line[kHalo];
    V *buf;
    __device__ int slot(int i) const {
#pragma unroll
        for (int s = 0; s < kHalo; s++)
            if (line[s] == i) return s;
        return -1;
    }
    __device__ V &at(int s, int j) const { return buf[s * kHaloRows + j]; }
    __device__ void add(int i) {        // i >= 1, deduplicated
        if (slot(i) >= 0) return;
#pragma unroll
        for (int s = 0; s < kHalo; s++)
            if (line[s] < 0) { line[s] = i; return; }
    }
};

// the value of neighbour line `line`, row j: from the halo, else from
// `in` (lines of the level) or `out` (lines outside it, weight zero)
template <class V>
__device__ __forceinline__ V nbval(const Halo<V> &h, const Part &pt, const V *in, int ldi, const V *out, int ldo,
                                   int line, int j) {
    const int s = h.slot(line);
    if (s >= 0) return h.at(s, j);
    return pt.in(line) ? in[line + (size_t)ldi * j] : out[line + (size_t)ldo * j];
}

// the rows of neighbour line `line` as a base and a stride (row j at
// p[st * j]), resolved once per line: the same source nbval picks
template <class V>
struct LineRef {
    const V *p;
    size_t st;
};
template <class V>
__device__ __forceinline__ LineRef<V> nbline(const Halo<V> &h, const Part &pt, const V *in, int ldi, const V *out,
                                             int ldo, int line) {
    const int s = h.slot(line);
    if (s >= 0) return LineRef<V>{h.buf + (size_t)s * kHaloRows, 1};
    return pt.in(line) ? LineRef<V>{in + line, (size_t)ldi} : LineRef<V>{out + line, (size_t)ldo};
}

// The y solves of one zebra half on a partitioned level: the block's own
// lines of parity par (0: a, a+2, ..; 1: a+1, a+3, ..) and the halo lines
// of that parity listed in xl (their results go to the halo).  Right-hand
// sides as mg_half forms them (kind), from src (rhs plane if src == null);
// neighbours from nbval(h, ...).  With kind H_ODD and ov == 0 the right-hand
// side is the source itself (the neighbour terms vanish).
template <int MC, class T>
__device__ __noinline__ void part_half(const ModeT<T> &m, const Part &pt, int par, const int *xl, int nx, int kind,
                                       const typename V2<T>::t *src, const typename V2<T>::t *nin, int ldi,
                                       const typename V2<T>::t *nout, int ldo, Halo<typename V2<T>::t> &h, T ov,
                                       typename V2<T>::t tt) {
    using V = typename V2<T>::t;
    const MgArgs &a = m.a;
    const MgSet<T> &s = m.s;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int n2m = a.n2m;
    const int ch = (n2m + 31) / 32;
    const int j0 = 1 + lane * ch;
    const int cnt = max(0, min(ch, n2m - j0 + 1));
    const size_t sj = (size_t)a.nld;
    const int nown = (pt.b - pt.a + 1) / 2;
    for (int li = warp; li < nown + nx; li += nw) {
        const int i = li < nown ? pt.a + par + 2 * li : xl[li - nown];
        const int im = a.imm[i], ip = a.ipm[i];
        const T aw = s.aw[i], ae = s.ae[i];
        const T *bet = s.bet + m.cb + (i - 1);
        const T *gam = s.gam + m.cb + (i - 1);
        const bool nbr = !(kind == H_ODD && ov == T(0.0));
        LineRef<V> lm{nullptr, 0}, lp{nullptr, 0};
        if (nbr) {
            lm = nbline(h, pt, nin, ldi, nout, ldo, im);
            lp = nbline(h, pt, nin, ldi, nout, ldo, ip);
        }
        V v[MC];
        T as_[MC], bt[MC], gm[MC];
#pragma unroll
        for (int q = 0; q < MC; q++)
            if (q < cnt) {
                const int j = j0 + q;
                V sr;
                if (!src) {
                    const double2 b = m.B(i, j);
                    sr = V{T(b.x), T(b.y)};
                } else {
                    sr = src[i + (size_t)a.ldg * j];
                }
                if (!nbr) {
                    v[q] = sr;
                } else {
                    V nm = lm.p[lm.st * j], np = lp.p[lp.st * j];
                    if (kind == H_ODD) {
                        const T sx = aw * nm.x + ae * np.x, sy = aw * nm.y + ae * np.y;
                        v[q] = V{sr.x - ov * sx, sr.y - ov * sy};
                    } else if (kind == H_EVEN) {
                        v[q] = V{sr.x - aw * nm.x - ae * np.x, sr.y - aw * nm.y - ae * np.y};
                    } else {
                        nm = V{nm.x - tt.x, nm.y - tt.y};
                        if (ip < i) np = V{np.x - tt.x, np.y - tt.y};
                        v[q] = V{sr.x - aw * nm.x - ae * (np.x - tt.x), sr.y - aw * nm.y - ae * (np.y - tt.y)};
                    }
                }
                as_[q] = s.as[j];
                bt[q] = bet[sj * (j - 1)];
                gm[q] = j < n2m ? gam[sj * j] : T(0.0);
            }
        line_solve<MC>(v, as_, bt, gm, cnt, lane);
        const int hs = li < nown ? -1 : h.slot(i);
#pragma unroll
        for (int q = 0; q < MC; q++)
            if (q < cnt) {
                const int j = j0 + q;
                if (hs < 0) m.G(i, j) = v[q];
                else h.at(hs, j) = v[q];
            }
    }
}

// src - aw*g(imm) - ae*g(ipm) - as*g(j-1) - an*g(j+1) - ac*g (mg_defect) with
// the line neighbours through the halo
template <class T>
__device__ __forceinline__ typename V2<T>::t part_defect(const ModeT<T> &m, const Part &pt,
                                                        const Halo<typename V2<T>::t> &h, typename V2<T>::t src,
                                                        const typename V2<T>::t *g, int ld, int i, int j) {
    const MgArgs &a = m.a;
    const MgSet<T> &s = m.s;
    src = axmy(src, s.aw[i], nbval(h, pt, g, ld, g, ld, a.imm[i], j));
    src = axmy(src, s.ae[i], nbval(h, pt, g, ld, g, ld, a.ipm[i], j));
    src = axmy(src, s.as[j], g[i + (size_t)ld * (j - 1)]);
    src = axmy(src, s.an[j], g[i + (size_t)ld * (j + 1)]);
    src = axmy(src, m.AC(i, j), g[i + (size_t)ld * j]);
    return src;
}

// prolongation of coarse line i (level range [cl, ce]) onto a fine even
// line: base + coi1 g(i) + coi2 g(ipm i) (mg_goup / mg_top_prolong)
template <class T>
__device__ __forceinline__ typename V2<T>::t prolong_val(const ModeT<T> &m, typename V2<T>::t p, int i, int ce, int j) {
    const MgArgs &a = m.a;
    const MgSet<T> &s = m.s;
    const typename V2<T>::t g1 = m.G(i, j);
    if (i < ce || a.xft) {
        const typename V2<T>::t g2 = m.G(a.ipm[i], j);
        return typename V2<T>::t{p.x + s.coi1[i] * g1.x + s.coi2[i] * g2.x, p.y + s.coi1[i] * g1.y + s.coi2[i] * g2.y};
    }
    return typename V2<T>::t{p.x + s.coi1[i] * g1.x, p.y + s.coi1[i] * g1.y};
}

__device__ __forceinline__ void hinit(int (&l)[kHalo]) {
#pragma unroll
    for (int s = 0; s < kHalo; s++) l[s] = -1;
}

// One level down (relax(ilev, 0, 1) + godown(ilev)) on a partitioned level:
// restricted residual R -> relaxed G (own lines), defect -> D, restricted
// defect -> R of level ilev - 1 (own coarse lines).  Ends at the cluster barrier.
template <int MC, class T>
__device__ __noinline__ void part_down(const ModeT<T> &m, int ilev, int r, int cs, typename V2<T>::t *hbuf) {
    using V = typename V2<T>::t;
    const MgArgs &a = m.a;
    const Part pt = part_of(a.iimg[ilev][0], a.iimg[ilev][1], r, cs);
    const int n2m = a.n2m;
    Halo<V> h;
    hinit(h.line);
    h.buf = hbuf;
    int xo[2], nxo = 0, xe[1], nxe = 0;
    const int l1 = a.imm[pt.a], r1 = a.ipm[pt.b];
    if (pt.in(r1) && !pt.own(r1)) { h.add(r1); xo[nxo++] = r1; }
    if (pt.in(l1) && !pt.own(l1)) {
        const int l2 = a.imm[l1];
        if (pt.in(l2) && !pt.own(l2) && h.slot(l2) < 0) { h.add(l2); xo[nxo++] = l2; }
        h.add(l1);
        xe[nxe++] = l1;
    }
    const V zero{T(0.0), T(0.0)};
    part_half<MC, T>(m, pt, 0, xo, nxo, H_ODD, m.rs, m.gg, a.ldg, m.gg, a.ldg, h, T(0.0), zero);
    __syncthreads();
    part_half<MC, T>(m, pt, 1, xe, nxe, H_EVEN, m.rs, m.gg, a.ldg, m.gg, a.ldg, h, T(1.0), zero);
    __syncthreads();
    const int nown = pt.b - pt.a + 1;
    for (int t = threadIdx.x; t < nown * n2m; t += blockDim.x) {
        const int i = pt.a + t % nown, j = 1 + t / nown;
        m.D(i, j) = part_defect(m, pt, h, m.R(i, j), m.gg, a.ldg, i, j);
        if (((i - pt.ibg) & 1) == 1) m.GB(i, j) = m.G(i, j);     // even line: the base of its prolongation
    }
    __syncthreads();
    const int cl = a.iimg[ilev - 1][0], c0 = cl + (pt.a - pt.ibg) / 2, nc = nown / 2;
    for (int t = threadIdx.x; t < nc * n2m; t += blockDim.x) {
        const int i = c0 + t % nc, j = 1 + t / nc, f = pt.ibg + 2 * (i - cl);
        const V r1v = m.D(f, j), r2v = m.D(f + 1, j);
        m.R(i, j) = V{r1v.x * m.s.cor1[i] + r2v.x * m.s.cor2[i], r1v.y * m.s.cor1[i] + r2v.y * m.s.cor2[i]};
    }
    cooperative_groups::this_cluster().sync();
}

// One level up (goup(ilev) + relax(ilev + 1, 1, 1)) onto a partitioned
// level: prolonged even lines (own -> U, halo), relaxation against the
// level's defect D.  Ends at the cluster barrier.
template <int MC, class T>
__device__ __noinline__ void part_up(const ModeT<T> &m, int ilev, int r, int cs, typename V2<T>::t *hbuf) {
    using V = typename V2<T>::t;
    const MgArgs &a = m.a;
    const int F = ilev + 1;
    const Part pt = part_of(a.iimg[F][0], a.iimg[F][1], r, cs);
    const int n2m = a.n2m, cl = a.iimg[ilev][0], ce = a.iimg[ilev][1], fb = pt.ibg;
    Halo<V> h;
    hinit(h.line);
    h.buf = hbuf;
    int xo[1], nxo = 0;
    int xe[2], nxe = 0;
    const int l1 = a.imm[pt.a], r1 = a.ipm[pt.b];
    if (pt.in(l1) && !pt.own(l1)) { h.add(l1); xe[nxe++] = l1; }
    if (pt.in(r1) && !pt.own(r1)) {
        h.add(r1);
        xo[nxo++] = r1;
        const int r2 = a.ipm[r1];
        if (pt.in(r2) && !pt.own(r2) && h.slot(r2) < 0) { h.add(r2); xe[nxe++] = r2; }
    }
    // prolongation onto the own even lines (-> U) and the halo even lines
    const int ne = (pt.b - pt.a + 1) / 2;
    for (int t = threadIdx.x; t < (ne + nxe) * n2m; t += blockDim.x) {
        const int q = t % (ne + nxe), j = 1 + t / (ne + nxe);
        const int f = q < ne ? pt.a + 1 + 2 * q : xe[q - ne];
        const int i = cl + (f - fb - 1) / 2;
        const V v = prolong_val(m, m.GB(f, j), i, ce, j);
        if (q < ne) m.U(f, j) = v;
        else h.at(h.slot(f), j) = v;
    }
    __syncthreads();
    const V zero{T(0.0), T(0.0)};
    part_half<MC, T>(m, pt, 0, xo, nxo, H_ODD, m.rd, m.gu, a.ldg, m.gg, a.ldg, h, T(1.0), zero);
    __syncthreads();
    part_half<MC, T>(m, pt, 1, xo, 0, H_EVEN, m.rd, m.gg, a.ldg, m.gg, a.ldg, h, T(1.0), zero);
    cooperative_groups::this_cluster().sync();
}

// The top level's relaxation (toplevel's prolongation and zebra sweep with
// the zero wavenumber's pin) on the partitioned top level.  prolong: the
// coarse correction is added to (FP64 form) or becomes (assign, the mixed
// form's correction) the even lines' neighbour values, in U; src: the
// right-hand side plane (null) or the FP32 residual.  The mixed form then
// adds the correction to the FP64 solution of its own lines.  Ends at the
// cluster barrier.
template <int MC, class T>
__device__ __noinline__ void part_top_relax(const ModeT<T> &m, int r, int cs, T oldv, bool prolong, bool assign,
                               const typename V2<T>::t *src, typename V2<T>::t *hbuf, const Mode *x64, bool first) {
    using V = typename V2<T>::t;
    const MgArgs &a = m.a;
    const Part pt = part_of(1, a.nl, r, cs);
    const int n2m = a.n2m, nlev = a.nlev;
    const int cl = a.iimg[nlev - 1][0], ce = a.iimg[nlev - 1][1];
    Halo<V> h;
    hinit(h.line);
    h.buf = hbuf;
    int xo[2], nxo = 0, xe[4], nxe = 0;
    const int l1 = a.imm[pt.a], r1 = a.ipm[pt.b];
    if (prolong && pt.in(l1) && !pt.own(l1)) { h.add(l1); xe[nxe++] = l1; }
    if (pt.in(r1) && !pt.own(r1)) {
        h.add(r1);
        xo[nxo++] = r1;
        const int r2 = a.ipm[r1];
        if (prolong && pt.in(r2) && !pt.own(r2) && h.slot(r2) < 0) { h.add(r2); xe[nxe++] = r2; }
    }
    const bool pin = m.kv == 1;
    if (pin && !pt.own(1) && h.slot(1) < 0) {
        // line 1 gives the zero wavenumber's shift: recomputed by every
        // block, with the prolonged even lines beside it
        h.add(1);
        xo[nxo++] = 1;
        if (prolong)
            for (int q = 0; q < 2; q++) {
                const int e = q == 0 ? a.imm[1] : a.ipm[1];
                if (pt.in(e) && !pt.own(e) && h.slot(e) < 0) { h.add(e); xe[nxe++] = e; }
            }
    }
    if (prolong) {
        const int ne = (pt.b - pt.a + 1) / 2;
        for (int t = threadIdx.x; t < (ne + nxe) * n2m; t += blockDim.x) {
            const int q = t % (ne + nxe), j = 1 + t / (ne + nxe);
            const int ic = q < ne ? pt.a + 1 + 2 * q : xe[q - ne];
            const int i = cl + ic / 2 - 1;
            const V base = assign ? V{T(0.0), T(0.0)} : m.P(ic, j);
            const V v = prolong_val(m, base, i, ce, j);
            if (q < ne) m.U(ic, j) = v;
            else h.at(h.slot(ic), j) = v;
        }
        __syncthreads();
    }
    const V zero{T(0.0), T(0.0)};
    // odd lines: neighbours are the even lines' prolonged values (U, halo),
    // or P outside the level
    part_half<MC, T>(m, pt, 0, xo, nxo, H_ODD, src, prolong ? m.gu : m.pc, prolong ? a.ldg : a.ldp, m.pc, a.ldp, h,
                      oldv, zero);
    __syncthreads();
    auto gval = [&](int i, int j) -> V {
        const int s = h.slot(i);
        return s >= 0 ? h.at(s, j) : m.G(i, j);
    };
    if (a.xft) {
        // poiss_x_ft: shift the odd lines by ggii(1,n2m) (own and halo), then
        // the even lines from the shifted values
        if (pin) {
            const V tt = gval(1, n2m);
            __syncthreads();
            const int no = (pt.b - pt.a + 1) / 2;
            for (int t = threadIdx.x; t < (no + nxo) * n2m; t += blockDim.x) {
                const int q = t % (no + nxo), j = 1 + t / (no + nxo);
                const int i = q < no ? pt.a + 2 * q : xo[q - no];
                V &g = q < no ? m.G(i, j) : h.at(h.slot(i), j);
                g = V{g.x - tt.x, g.y - tt.y};
            }
            __syncthreads();
        }
        part_half<MC, T>(m, pt, 1, xe, 0, H_ODD, src, m.gg, a.ldg, m.gg, a.ldg, h, T(1.0), zero);
        __syncthreads();
    } else {
        // poiss_z_ft: the even lines see the odd ones shifted by
        // ggii(1,n2m-1) inside their right-hand side; the odd lines are
        // shifted afterwards
        const V tt = pin ? gval(1, n2m - 1) : zero;
        part_half<MC, T>(m, pt, 1, xe, 0, H_EVEN_TT, src, m.gg, a.ldg, m.gg, a.ldg, h, T(1.0), tt);
        __syncthreads();
        if (pin) {
            const int no = (pt.b - pt.a + 1) / 2;
            for (int t = threadIdx.x; t < no * n2m; t += blockDim.x) {
                const int i = pt.a + 2 * (t % no), j = 1 + t / no;
                V &g = m.G(i, j);
                g = V{g.x - tt.x, g.y - tt.y};
            }
            __syncthreads();
        }
    }
    if (x64) {            // the mixed form: x += e on the own lines (x = e on the first pass)
        const int nown = pt.b - pt.a + 1;
        for (int t = threadIdx.x; t < nown * n2m; t += blockDim.x) {
            const int i = pt.a + t % nown, j = 1 + t / nown;
            const V e = m.G(i, j);
            const double2 x = first ? make_double2(0.0, 0.0) : x64->P(i, j);
            x64->P(i, j) = make_double2(x.x + (double)e.x, x.y + (double)e.y);
        }
    }
    cooperative_groups::this_cluster().sync();
}

// Max over the cluster through distributed shared memory: one value per
// block, slot `par` (alternating between calls, so a slot is rewritten only
// after every block has passed the barrier that follows its reads).  A
// cluster barrier must follow before the slot is written again and before
// any block of the cluster exits.
__device__ double part_cluster_max(double v, int par) {
    __shared__ double sh[kMgThreads / 32];
    __shared__ double blk[2];
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    if (lane == 0) sh[w] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) r = fmax(r, sh[q]);
        blk[par] = r;
    }
    cl.sync();
    return dsm_max(cl, &blk[par]);
}

// toplevel's residual on the partitioned top level (FP64 form): R = B - A G
// on the own lines, P = G, the residual restricted onto level nlev-1 (own
// coarse lines), the max norm over the cluster.
__device__ __noinline__ double part_top_resid(const Mode &m, int r, int cs, int par) {
    const MgArgs &a = m.a;
    const Part pt = part_of(1, a.nl, r, cs);
    const int n2m = a.n2m, nown = pt.b - pt.a + 1;
    double mx = 0.0;
    Halo<double2> h0;
    hinit(h0.line);
    h0.buf = nullptr;
    for (int t = threadIdx.x; t < nown * n2m; t += blockDim.x) {
        const int i = pt.a + t % nown, j = 1 + t / nown;
        const double2 d = part_defect(m, pt, h0, m.B(i, j), m.gg, a.ldg, i, j);
        m.R(i, j) = d;
        mx = fmax(mx, d.x * d.x + d.y * d.y);
        m.P(i, j) = m.G(i, j);
    }
    __syncthreads();
    const int cl = a.iimg[a.nlev - 1][0], c0 = cl + (pt.a - 1) / 2, nc = nown / 2;
    for (int t = threadIdx.x; t < nc * n2m; t += blockDim.x) {
        const int i = c0 + t % nc, j = 1 + t / nc, ic = 2 * (i - cl) + 1;
        const double2 r1 = m.R(ic, j), r2 = m.R(ic + 1, j);
        m.R(i, j) = double2{r1.x * m.s.cor1[i] + r2.x * m.s.cor2[i], r1.y * m.s.cor1[i] + r2.y * m.s.cor2[i]};
    }
    return sqrt(part_cluster_max(mx, par));
}

// the mixed form's residual: r = b - A x in FP64 (x in m.P) -> the FP32
// residual f.R, restricted in FP32 onto level nlev-1; the max norm
__device__ __noinline__ double part_top_resid_mixed(const Mode &m, const ModeT<float> &f, int r, int cs, int par) {
    const MgArgs &a = m.a;
    const Part pt = part_of(1, a.nl, r, cs);
    const int n2m = a.n2m, nown = pt.b - pt.a + 1;
    double mx = 0.0;
    for (int t = threadIdx.x; t < nown * n2m; t += blockDim.x) {
        const int i = pt.a + t % nown, j = 1 + t / nown;
        const double2 d = mg_defect(m, m.B(i, j), m.pc, a.ldp, i, j);
        f.R(i, j) = make_float2((float)d.x, (float)d.y);
        mx = fmax(mx, d.x * d.x + d.y * d.y);
    }
    __syncthreads();
    const int cl = a.iimg[a.nlev - 1][0], c0 = cl + (pt.a - 1) / 2, nc = nown / 2;
    for (int t = threadIdx.x; t < nc * n2m; t += blockDim.x) {
        const int i = c0 + t % nc, j = 1 + t / nc, ic = 2 * (i - cl) + 1;
        const float2 r1 = f.R(ic, j), r2 = f.R(ic + 1, j);
        f.R(i, j) = float2{r1.x * f.s.cor1[i] + r2.x * f.s.cor2[i], r1.y * f.s.cor1[i] + r2.y * f.s.cor2[i]};
    }
    return sqrt(part_cluster_max(mx, par));
}

// mg2d (poiss_z_ft.f90:239-299) with the level-partitioned phases
template <int MC>
__device__ int part_mg2d(const Mode &m, const Mode &mb, double test, bool &unconv, int r, int cs, double2 *hbuf) {
    const MgArgs &a = m.a;
    const int nlev = a.nlev, lc = a.lc;
    int par = 0;
    part_top_relax<MC>(m, r, cs, 0.0, false, false, nullptr, hbuf, nullptr, true);
    double sumres = part_top_resid(m, r, cs, par);
    par ^= 1;
    if (sumres < test) return 0;
    for (int kk = 1; kk <= a.mgitr; kk++) {
        for (int ilev = nlev - 1; ilev > lc; ilev--) part_down<MC>(m, ilev, r, cs, hbuf);
        if (r == 0) {
            for (int ilev = lc; ilev >= 1; ilev--) {
                mg_relax<MC>(mb, ilev, 0.0, 1);
                mg_godown(mb, ilev);
            }
            mg_relax<MC>(mb, 0, 0.0, a.nbli);
            for (int ilev = 0; ilev < lc; ilev++) {
                mg_goup(mb, ilev);
                mg_relax<MC>(mb, ilev + 1, 1.0, 1);
            }
        }
        cooperative_groups::this_cluster().sync();
        for (int ilev = lc; ilev <= nlev - 2; ilev++) part_up<MC>(m, ilev, r, cs, hbuf);
        part_top_relax<MC>(m, r, cs, 1.0, true, false, nullptr, hbuf, nullptr, false);
        sumres = part_top_resid(m, r, cs, par);
        par ^= 1;
        if (sumres < test) return kk;
    }
    unconv = true;
    return a.xft ? a.mgitr : a.mgitr + 1;
}

// mg_mg2d_mixed with the level-partitioned phases
template <int MC>
__device__ int part_mg2d_mixed(const Mode &m, const ModeT<float> &f, const ModeT<float> &fb, double test,
                               bool &unconv, int r, int cs, double2 *hbuf) {
    const MgArgs &a = m.a;
    const int nlev = a.nlev, lc = a.lc, n2m = a.n2m;
    float2 *hf = reinterpret_cast<float2 *>(hbuf);
    int par = 0;
    {   // the first source is b itself, rounded (own lines; the halo lines
        // read other blocks' after the barrier)
        const Part pt = part_of(1, a.nl, r, cs);
        const int nown = pt.b - pt.a + 1;
        for (int t = threadIdx.x; t < nown * n2m; t += blockDim.x) {
            const int i = pt.a + t % nown, j = 1 + t / nown;
            const double2 b = m.B(i, j);
            f.R(i, j) = make_float2((float)b.x, (float)b.y);
        }
        cooperative_groups::this_cluster().sync();
    }
    part_top_relax<MC>(f, r, cs, 0.0f, false, true, f.rs, hf, &m, true);
    double sumres = part_top_resid_mixed(m, f, r, cs, par);
    par ^= 1;
    if (sumres < test) return 0;
    // with 16-block clusters the coarse levels (up to kCoarseLines lines, two
    // per warp of one block) run faster spread over the cluster despite a
    // cluster barrier per phase; with smaller clusters, on block 0
    const bool wide = cs >= 16;
    for (int kk = 1; kk <= a.mgitr; kk++) {
        for (int ilev = nlev - 1; ilev > lc; ilev--) part_down<MC>(f, ilev, r, cs, hf);
        if (wide) {
            // the coarse levels' relaxations, defects, restrictions and
            // prolongations spread over the cluster (a cluster barrier per
            // phase), the coarsest level's relaxations on block 0
            for (int ilev = lc; ilev >= 1; ilev--) {
                mg_relax<MC>(f, ilev, 0.0f, 1);
                mg_godown(f, ilev);
            }
            if (r == 0) mg_relax<MC>(fb, 0, 0.0f, a.nbli);
            cooperative_groups::this_cluster().sync();
            for (int ilev = 0; ilev < lc; ilev++) {
                mg_goup(f, ilev);
                mg_relax<MC>(f, ilev + 1, 1.0f, 1);
            }
        } else {
            if (r == 0) {
                for (int ilev = lc; ilev >= 1; ilev--) {
                    mg_relax<MC>(fb, ilev, 0.0f, 1);
                    mg_godown(fb, ilev);
                }
                // the coarsest level's nbli relaxations in FP32 too: GB300's
                // FP64 latency made their dependent line recurrences a third of
                // the cycle in FP64, and they only refine the FP32 correction
                mg_relax<MC>(fb, 0, 0.0f, a.nbli);
                for (int ilev = 0; ilev < lc; ilev++) {
                    mg_goup(fb, ilev);
                    mg_relax<MC>(fb, ilev + 1, 1.0f, 1);
                }
            }
            cooperative_groups::this_cluster().sync();
        }
        for (int ilev = lc; ilev <= nlev - 2; ilev++) part_up<MC>(f, ilev, r, cs, hf);
        part_top_relax<MC>(f, r, cs, 1.0f, true, true, f.rs, hf, &m, false);
        sumres = part_top_resid_mixed(m, f, r, cs, par);
        par ^= 1;
        if (sumres < test) return kk;
    }
    unconv = true;
    return a.xft ? a.mgitr : a.mgitr + 1;
}

// What a block keeps in shared memory for its mode: the launch's arguments
// and the four views of the mode (cluster-wide and block-local, FP64 and
// FP32), built once by thread 0.
struct MgBlock {
    MgArgs a;
    alignas(16) unsigned char m[sizeof(ModeT<double>)], f[sizeof(ModeT<float>)];
    alignas(16) unsigned char mb[sizeof(ModeT<double>)], fb[sizeof(ModeT<float>)];
};

// One cluster's solve of mode kv of the case described by ga.
template <int MC>
__device__ __forceinline__ void zft_mode(const MgArgs &ga, int kv, double2 *hbuf, MgBlock &sb) {
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    const int cs = (int)cl.num_blocks();
    const int r = (int)cl.block_rank();
    if (threadIdx.x == 0) {
        sb.a = ga;
        new (sb.m) Mode(sb.a, sb.a.d, kv, false, r, cs);
        new (sb.f) ModeT<float>(sb.a, sb.a.f, kv, false, r, cs);
        new (sb.mb) Mode(sb.a, sb.a.d, kv, true, 0, 1);
        new (sb.fb) ModeT<float>(sb.a, sb.a.f, kv, true, 0, 1);
    }
    __syncthreads();
    const MgArgs &a = sb.a;
    const Mode &m = *reinterpret_cast<const Mode *>(sb.m);
    const double test = a.fixed_cycles > 0 ? -1.0 : a.S->mg_test;
    int it;
    bool unconv = false;
    if (kv > a.imgsor) {
        it = mg_gsor2d<MC>(m, test, unconv);
    } else if (a.mixed) {
        it = part_mg2d_mixed<MC>(m, *reinterpret_cast<const ModeT<float> *>(sb.f),
                                 *reinterpret_cast<const ModeT<float> *>(sb.fb), test, unconv, r, cs, hbuf);
    } else {
        it = part_mg2d<MC>(m, *reinterpret_cast<const Mode *>(sb.mb), test, unconv, r, cs, hbuf);
    }
    // the last max-norm test read every block's slot through distributed
    // shared memory with no barrier after it: no block may exit (and take
    // its shared memory with it) before all have read
    cl.sync();
    // the mode's solution replaces its right-hand side (ccap(i,j,kkk) = cp(i,j))
    double2 *out = a.ccap + (size_t)a.nl * a.n2m * (kv - 1);
    const int tid = m.tid(), nt = m.nt();
    for (int t = tid; t < a.nl * a.n2m; t += nt) {
        const int i = 1 + t % a.nl, j = 1 + t / a.nl;
        out[t] = m.P(i, j);
    }
    if (tid == 0) {
        a.iters[kv - 1] = it;
        atomicMax((unsigned long long *)&a.S->poisson_iters[a.slot], (unsigned long long)it);
        // the timing runs of the autotuner fix the cycle count: not a failure
        if (unconv && a.fixed_cycles <= 0) atomicAdd((unsigned long long *)&a.S->poisson_unconv, 1ULL);
    }
}

template <int MC>
__global__ void __launch_bounds__(kMgThreads, 1) k_zft_modes(MgArgs a) {
    __shared__ __align__(16) double2 hbuf[kHalo * kHaloRows];
    __shared__ MgBlock sb;
    const int cs = (int)cooperative_groups::this_cluster().num_blocks();
    zft_mode<MC>(a, blockIdx.x / cs + 1, hbuf, sb);
}

// The modes of several cases of one grid shape in one launch (the serving
// loop's batched solve): cluster b solves mode b % nmodes + 1 of case
// b / nmodes, each case's tables, work arrays and scalars from its own
// MgArgs; per case the arithmetic is that of k_zft_modes.
template <int MC>
__global__ void __launch_bounds__(kMgThreads, 1) k_zft_modes_batch(const MgArgs *as, int nmodes) {
    __shared__ __align__(16) double2 hbuf[kHalo * kHaloRows];
    __shared__ MgBlock sb;
    const int cs = (int)cooperative_groups::this_cluster().num_blocks();
    const int b = blockIdx.x / cs;
    zft_mode<MC>(as[b / nmodes], b % nmodes + 1, hbuf, sb);
}

// the instance for y lines of n2m cells: MC = ceil(n2m / 32) rounded up to
// 2, 4, 6 or 8 rows per lane (fewer registers, no spills, on shorter lines)
inline int mg_mc(int n2m) { return n2m <= 64 ? 2 : n2m <= 128 ? 4 : n2m <= 192 ? 6 : 8; }
typedef void (*ZftKernel)(MgArgs);
inline ZftKernel zft_kernel(int n2m) {
    switch (mg_mc(n2m)) {
    case 2: return k_zft_modes<2>;
    case 4: return k_zft_modes<4>;
    case 6: return k_zft_modes<6>;
    default: return k_zft_modes<8>;
    }
}
typedef void (*ZftBatchKernel)(const MgArgs *, int);
inline ZftBatchKernel zft_batch_kernel(int n2m) {
    switch (mg_mc(n2m)) {
    case 2: return k_zft_modes_batch<2>;
    case 4: return k_zft_modes_batch<4>;
    case 6: return k_zft_modes_batch<6>;
    default: return k_zft_modes_batch<8>;
    }
}

// convergence criterion of the substep: test1 / nmodes * nfft * fac -- 0.8 in
// poiss_z_ft.f90:179 (test1 itself in 2-D), 0.9 in poiss_x_ft.f90:158
__global__ void k_mg_begin(DScal *S, int slot, int nfft, int nmodes, double fac) {
    S->poisson_iters[slot] = 0;
    S->mg_test = nfft == 1 ? S->test1 : S->test1 / (double)nmodes * (double)nfft * fac;
}

// ---------------------------------------------------------------- host side
// The semi-coarsened axis of a solve, in the reference's Fortran indexing:
// x for poiss_z_ft, z for poiss_x_ft.
struct MgAxis {
    int nm, n;                                      // cells, nodes (nm + 1)
    bool prdic;
    std::vector<double> x, xmp, c2ci, f2fi;         // x(1..n); xmp, c2c?i, f2f?i (0..n)
    std::vector<long long> pv, fixl, fixu;          // ipv / kpv, fixil / fixkl, fixiu / fixku (1..nm)
};

// pmat, mwavenumber, coefmg and the LU factors of poisinit, in the
// reference's arithmetic order: poiss_z_ft.f90:18-113, 643-798 and
// poiss_x_ft.f90:18-112, 644-794.  ab/af of x_ft land in aw/ae, kpm/kmm in
// ipm/imm, kkmg in iimg.
static int set_up_tables(lesgpu_case *c, MgTables &T) {
    const DGrid &g = c->kp.g;
    const lesgpu_config &cf = c->cfg;
    const bool xft = T.xft != 0;
    const int n2m = g.n2m, nmodes = T.nmodes, n1md = T.nld, nlev = T.nlev;
    const lesgpu_grid *hg = c->h_grid;
    auto v0 = [&](const double *p, int n) { std::vector<double> v(n + 2, 0.0); for (int q = 0; q <= n; q++) v[q] = p[q]; return v; };
    auto v1 = [&](const double *p, int n) { std::vector<double> v(n + 2, 0.0); for (int q = 1; q <= n; q++) v[q] = p[q - 1]; return v; };
    auto i1 = [&](const int64_t *p, int n) { std::vector<long long> v(n + 2, 0); for (int q = 1; q <= n; q++) v[q] = p[q - 1]; return v; };
    MgAxis A;
    if (xft) {
        A.nm = g.n3m; A.n = g.n3; A.prdic = cf.zprdic == 1;
        A.x = v1(hg->z, g.n3); A.xmp = v0(hg->zmp, g.n3); A.c2ci = v0(hg->c2czi, g.n3); A.f2fi = v0(hg->f2fzi, g.n3);
        A.pv = i1(hg->kpv, g.n3m); A.fixl = i1(hg->fixkl, g.n3m); A.fixu = i1(hg->fixku, g.n3m);
    } else {
        A.nm = g.n1m; A.n = g.n1; A.prdic = cf.xprdic == 1;
        A.x = v1(hg->x, g.n1); A.xmp = v0(hg->xmp, g.n1); A.c2ci = v0(hg->c2cxi, g.n1); A.f2fi = v0(hg->f2fxi, g.n1);
        A.pv = i1(hg->ipv, g.n1m); A.fixl = i1(hg->fixil, g.n1m); A.fixu = i1(hg->fixiu, g.n1m);
    }
    const int n1m = A.nm, n1 = A.n;
    const std::vector<double> &x = A.x;
    std::vector<double> c2cyi = v0(hg->c2cyi, g.n2), f2fyi = v0(hg->f2fyi, g.n2);
    std::vector<long long> jpv = i1(hg->jpv, n2m), fixjl = i1(hg->fixjl, n2m), fixju = i1(hg->fixju, n2m);

    const size_t nv = (size_t)n1md + 2, na = (size_t)n1md * n2m * nmodes;
    std::vector<double> aw(nv, 0.0), ae(nv, 0.0), as(n2m + 2, 0.0), an(n2m + 2, 0.0);
    std::vector<double> coi1(nv, 0.0), coi2(nv, 0.0), cor1(nv, 0.0), cor2(nv, 0.0);
    std::vector<int> ipm(nv, 0), imm(nv, 0);
    std::vector<double> ac(na, 0.0), bet(na, 0.0), gam(na, 0.0);
    std::vector<double> ak(nmodes + 2, 0.0);          // modified wavenumbers: ak3 (z_ft) / ai3 (x_ft)
    auto AC = [&](int i, int j, int k) -> double & { return ac[(size_t)(i - 1) + (size_t)n1md * ((size_t)(j - 1) + (size_t)n2m * (size_t)(k - 1))]; };
    // pmat
    for (int i = 1; i <= n1m; i++) {
        long long ip = A.pv[i];
        aw[i] = (1.0 - (double)A.fixl[i]) * A.c2ci[i] * A.f2fi[i];
        ae[i] = (1.0 - (double)A.fixu[i]) * A.c2ci[ip] * A.f2fi[i];
    }
    for (int j = 1; j <= n2m; j++) {
        long long jp = jpv[j];
        as[j] = (1.0 - (double)fixjl[j]) * c2cyi[j] * f2fyi[j];
        an[j] = (1.0 - (double)fixju[j]) * c2cyi[jp] * f2fyi[j];
    }
    for (int j = 1; j <= n2m; j++)
        for (int i = 1; i <= n1m; i++) AC(i, j, 1) = -1.0 * (aw[i] + ae[i] + as[j] + an[j]);
    const double pi = acos(-1.0);
    if (xft) {
        const double sdx = hg->f2fxi[1];
        for (int i = 1; i <= nmodes; i++)
            ak[i] = 2.0 * (1.0 - cos(2.0 * pi * (double)(i - 1) / (double)g.n1m)) * sdx * sdx;
    } else if (g.n3m > 1) {
        const double sdz = hg->f2fzi[1];
        for (int k = 1; k <= nmodes; k++)
            ak[k] = 2.0 * (1.0 - cos(2.0 * (double)(k - 1) * pi / (double)g.n3m)) * sdz * sdz;
    }
    for (int k = 2; k <= nmodes; k++)
        for (int j = 1; j <= n2m; j++)
            for (int i = 1; i <= n1m; i++) AC(i, j, k) = AC(i, j, 1) - ak[k];
    // coefmg
    const int minrow = n1m / (1 << nlev);
    std::vector<double> xmpm(nv, 0.0), iwz(nv, 0.0), iez(nv, 0.0);
    int (&iimg)[kMaxLev + 1][3] = T.iimg;
    iimg[nlev][0] = 1; iimg[nlev][1] = n1m; iimg[nlev][2] = n1m;
    for (int i = 1; i <= n1m; i++) xmpm[i] = A.xmp[i];
    for (int ilev = nlev - 1; ilev >= 0; ilev--) {
        iimg[ilev][0] = iimg[ilev + 1][0] + iimg[ilev + 1][2];
        iimg[ilev][2] = minrow * (1 << ilev);
        iimg[ilev][1] = iimg[ilev][0] + iimg[ilev][2] - 1;
        const int ibg = iimg[ilev][0], iend = iimg[ilev][1], isp = 1 << (nlev - ilev);
        int ic = 0;
        for (int i = ibg; i <= iend; i++) {
            ic++;
            xmpm[i] = 0.5 * (x[ic * isp + 1] + x[(ic - 1) * isp + 1]);
            iwz[i] = (double)(1 - ibg / i);
            iez[i] = (double)(1 - i / iend);
        }
        ic = 0;
        for (int i = ibg; i <= iend; i++) {
            ic++;
            const double w = x[ic * isp + 1] - x[(ic - 1) * isp + 1];
            aw[i] = iwz[i] / ((xmpm[i] - xmpm[i - 1]) * w);
            ae[i] = iez[i] / ((xmpm[i + 1] - xmpm[i]) * w);
        }
        for (int j = 1; j <= n2m; j++)
            for (int i = ibg; i <= iend; i++) AC(i, j, 1) = -1.0 * (aw[i] + ae[i] + as[j] + an[j]);
        for (int k = 2; k <= nmodes; k++)
            for (int j = 1; j <= n2m; j++)
                for (int i = ibg; i <= iend; i++) AC(i, j, k) = AC(i, j, 1) - ak[k];
    }
    for (int ilev = nlev; ilev >= 1; ilev--) {
        int ibgh = iimg[ilev][0];
        for (int i = iimg[ilev - 1][0]; i <= iimg[ilev - 1][1]; i++) {
            cor1[i] = (xmpm[ibgh + 1] - xmpm[i]) / (xmpm[ibgh + 1] - xmpm[ibgh]);
            cor2[i] = 1.0 - cor1[i];
            ibgh += 2;
        }
    }
    for (int ilev = 0; ilev <= nlev - 1; ilev++) {
        int ibgh = iimg[ilev + 1][0] + 1;
        for (int i = iimg[ilev][0]; i <= iimg[ilev][1] - 1; i++) {
            coi1[i] = (xmpm[i + 1] - xmpm[ibgh]) / (xmpm[i + 1] - xmpm[i]);
            coi2[i] = 1.0 - coi1[i];
            ibgh += 2;
        }
        coi1[iimg[ilev][1]] = 1.0;
    }
    // neighbours; without periodicity x_ft leaves kpm/kmm unset, and the
    // coefficients that multiply them at the level ends are zero, so i+1 / i-1
    // (finite work-array entries) serve both
    for (int ilev = nlev; ilev >= 0; ilev--)
        for (int i = iimg[ilev][0]; i <= iimg[ilev][1]; i++) { ipm[i] = i + 1; imm[i] = i - 1; }
    if (A.prdic) {
        for (int ilev = nlev; ilev >= 0; ilev--) { ipm[iimg[ilev][1]] = iimg[ilev][0]; imm[iimg[ilev][0]] = iimg[ilev][1]; }
        for (int ilev = nlev - 1; ilev >= 0; ilev--) {
            const int ibg = iimg[ilev][0], iend = iimg[ilev][1], isp = 1 << (nlev - ilev);
            const double vdx = xmpm[ibg] - x[1] + x[n1] - xmpm[iend];
            aw[ibg] = 1.0 / (vdx * (x[1 + isp] - x[1]));
            ae[iend] = 1.0 / (vdx * (x[n1] - x[n1 - isp]));
        }
        for (int ilev = nlev - 1; ilev >= 0; ilev--) {
            for (int j = 1; j <= n2m; j++)
                for (int i = iimg[ilev][0]; i <= iimg[ilev][1]; i++) AC(i, j, 1) = -1.0 * (aw[i] + ae[i] + as[j] + an[j]);
            for (int k = 2; k <= nmodes; k++)
                for (int j = 1; j <= n2m; j++)
                    for (int i = iimg[ilev][0]; i <= iimg[ilev][1]; i++) AC(i, j, k) = AC(i, j, 1) - ak[k];
        }
        for (int ilev = 0; ilev <= nlev - 1; ilev++) {
            const int ibg = iimg[ilev][0], iend = iimg[ilev][1];
            const double vdx = xmpm[ibg] - x[1] + x[n1] - xmpm[iend];
            coi2[iend] = (xmpm[iimg[ilev + 1][1]] - xmpm[iend]) / vdx;
            coi1[iend] = 1.0 - coi2[iend];
        }
    }
    // poisinit: LU factors of every level's y-operator
    auto IX3 = [&](int i, int j, int k) { return (size_t)(i - 1) + (size_t)n1md * ((size_t)(j - 1) + (size_t)n2m * (size_t)(k - 1)); };
    for (int ilev = 0; ilev <= nlev; ilev++)
        for (int k = 1; k <= nmodes; k++) {
            for (int i = iimg[ilev][0]; i <= iimg[ilev][1]; i++) bet[IX3(i, 1, k)] = 1.0 / ac[IX3(i, 1, k)];
            for (int j = 2; j <= n2m; j++)
                for (int i = iimg[ilev][0]; i <= iimg[ilev][1]; i++) {
                    gam[IX3(i, j, k)] = an[j - 1] * bet[IX3(i, j - 1, k)];
                    bet[IX3(i, j, k)] = 1.0 / (ac[IX3(i, j, k)] - as[j] * gam[IX3(i, j, k)]);
                }
        }
    // upload
    bool ok = true;
    auto up = [&](auto *&dst, const auto &v) {
        using T0 = typename std::remove_reference<decltype(v[0])>::type;
        if (cudaMalloc((void **)&dst, sizeof(T0) * v.size()) != cudaSuccess) { ok = false; return; }
        cudaMemcpy(dst, v.data(), sizeof(T0) * v.size(), cudaMemcpyHostToDevice);
    };
    up(T.d.aw, aw); up(T.d.ae, ae); up(T.d.as, as); up(T.d.an, an);
    up(T.d.coi1, coi1); up(T.d.coi2, coi2); up(T.d.cor1, cor1); up(T.d.cor2, cor2);
    up(T.ipm, ipm); up(T.imm, imm); up(T.d.ac, ac); up(T.d.bet, bet); up(T.d.gam, gam);
    if (T.mixed) {   // FP32 copies (the LU factors rounded from their FP64 values)
        auto upf = [&](float *&dst, const std::vector<double> &v) {
            std::vector<float> h(v.begin(), v.end());
            up(dst, h);
        };
        upf(T.f.aw, aw); upf(T.f.ae, ae); upf(T.f.as, as); upf(T.f.an, an);
        upf(T.f.coi1, coi1); upf(T.f.coi2, coi2); upf(T.f.cor1, cor1); upf(T.f.cor2, cor2);
        upf(T.f.ac, ac); upf(T.f.bet, bet); upf(T.f.gam, gam);
    }
    return ok ? 0 : LESGPU_ERR_OOM;
}

// A cluster of cs blocks splits the top level and every level above lc into
// cs ranges of an even number of lines each.
static bool cs_splits(const MgTables &T, int cs) {
    if (T.nl % (2 * cs) != 0) return false;
    for (int l = T.lc + 1; l < T.nlev; l++)
        if (T.iimg[l][2] % (2 * cs) != 0) return false;
    return true;
}

static void cluster_cfg(cudaLaunchConfig_t &lc, cudaLaunchAttribute (&at)[1], int nmodes, int cs) {
    lc = {};
    lc.gridDim = dim3(nmodes * cs);
    lc.blockDim = dim3(kMgThreads);
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cs; at[0].val.clusterDim.y = 1; at[0].val.clusterDim.z = 1;
    lc.attrs = at;
    lc.numAttrs = 1;
}

int mg2d_init(lesgpu_case *c) {
    const DGrid &g = c->kp.g;
    const lesgpu_config &cf = c->cfg;
    DPois &P = c->pois;
    const bool xft = cf.poisson == LESGPU_POISSON_X_FT;
    const int nlev = (int)cf.nlev, nl = xft ? g.n3m : g.n1m, nmodes = xft ? g.n1mh : g.n3mh;
    if (nlev < 1 || nlev > kMaxLev || nl % (1 << nlev) != 0) return LESGPU_ERR_CONFIG;
    if (!xft && g.n3m > 1 && cf.zprdic != 1) return LESGPU_ERR_CONFIG;   // the z transform needs periodic z
    if (xft && cf.xprdic != 1) return LESGPU_ERR_CONFIG;                 // the x transform needs periodic x
    if (cf.mgitr < 0 || cf.nbli < 1) return LESGPU_ERR_CONFIG;
    if (g.n2m > 32 * kMC) return LESGPU_ERR_UNSUPPORTED;    // one warp per y line, kMC rows per lane
    int rc = xft ? make_plan(P.fx, g.n1m) : make_plan(P.fz, g.n3m);
    if (rc) return rc;
    MgTables *T = new MgTables();
    memset(T, 0, sizeof(*T));
    P.mg = T;
    T->nl = nl;
    T->nld = 2 * nl;
    T->nlev = nlev;
    T->nmodes = nmodes;
    T->xft = xft ? 1 : 0;
    // the mixed form runs the multigrid cycles in FP32 under an FP64 defect
    // correction (LESGPU_MG_FP64=1 keeps them in FP64)
    const char *mg64 = getenv("LESGPU_MG_FP64");
    T->mixed = cf.precision == LESGPU_PREC_MIXED && !(mg64 && mg64[0] == '1');
    rc = set_up_tables(c, *T);
    if (rc) return rc;
    const int ldp = nl + 2, ldg = T->nld + 1;
    T->pc_plane = (long long)ldp * (g.n2m + 2);
    T->gg_plane = (long long)ldg * (g.n2m + 2);
    const size_t nm = (size_t)nmodes;
    if (cudaMalloc(&T->d.pc, sizeof(double2) * T->pc_plane * nm) != cudaSuccess ||
        cudaMalloc(&T->d.gg, sizeof(double2) * T->gg_plane * nm) != cudaSuccess ||
        cudaMalloc(&T->d.rs, sizeof(double2) * T->gg_plane * nm) != cudaSuccess ||
        cudaMalloc(&T->d.rd, sizeof(double2) * T->gg_plane * nm) != cudaSuccess ||
        cudaMalloc(&T->d.gu, sizeof(double2) * T->gg_plane * nm) != cudaSuccess ||
        cudaMalloc(&T->d.gb, sizeof(double2) * T->gg_plane * nm) != cudaSuccess ||
        cudaMalloc(&T->iters, sizeof(long long) * nm) != cudaSuccess ||
        cudaMalloc(&P.ccap, sizeof(double2) * (size_t)nl * g.n2m * nm) != cudaSuccess)
        return LESGPU_ERR_OOM;
    // the boundary rows and columns of pc / gg are read as zeros and never written
    cudaMemset(T->d.pc, 0, sizeof(double2) * T->pc_plane * nm);
    cudaMemset(T->d.gg, 0, sizeof(double2) * T->gg_plane * nm);
    cudaMemset(T->d.rs, 0, sizeof(double2) * T->gg_plane * nm);
    cudaMemset(T->d.rd, 0, sizeof(double2) * T->gg_plane * nm);
    cudaMemset(T->d.gu, 0, sizeof(double2) * T->gg_plane * nm);
    cudaMemset(T->d.gb, 0, sizeof(double2) * T->gg_plane * nm);
    if (T->mixed) {
        if (cudaMalloc(&T->f.pc, sizeof(float2) * T->pc_plane * nm) != cudaSuccess ||
            cudaMalloc(&T->f.gg, sizeof(float2) * T->gg_plane * nm) != cudaSuccess ||
            cudaMalloc(&T->f.rs, sizeof(float2) * T->gg_plane * nm) != cudaSuccess ||
            cudaMalloc(&T->f.rd, sizeof(float2) * T->gg_plane * nm) != cudaSuccess ||
            cudaMalloc(&T->f.gu, sizeof(float2) * T->gg_plane * nm) != cudaSuccess ||
            cudaMalloc(&T->f.gb, sizeof(float2) * T->gg_plane * nm) != cudaSuccess)
            return LESGPU_ERR_OOM;
        cudaMemset(T->f.pc, 0, sizeof(float2) * T->pc_plane * nm);
        cudaMemset(T->f.gg, 0, sizeof(float2) * T->gg_plane * nm);
        cudaMemset(T->f.rs, 0, sizeof(float2) * T->gg_plane * nm);
        cudaMemset(T->f.rd, 0, sizeof(float2) * T->gg_plane * nm);
        cudaMemset(T->f.gu, 0, sizeof(float2) * T->gg_plane * nm);
        cudaMemset(T->f.gb, 0, sizeof(float2) * T->gg_plane * nm);
    }
    // levels of at most kCoarseLines lines run on one block; the others
    // (and the top) are split over the cluster
    T->lc = 0;
    for (int l = 0; l < nlev; l++)
        if (T->iimg[l][2] <= kCoarseLines) T->lc = l;
    cudaMemset(T->iters, 0, sizeof(long long) * nm);
    if (xft) {
        if (cudaFuncSetAttribute(k_fft_xr_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, kFftSmemMax) != cudaSuccess ||
            cudaFuncSetAttribute(k_fft_xr_inv, cudaFuncAttributeMaxDynamicSharedMemorySize, kFftSmemMax) != cudaSuccess)
            return LESGPU_ERR_CUDA;
    } else {
        if (fft_smem64(kFftSmemMax)) return LESGPU_ERR_CUDA;
    }
    // Cluster size: the mode solves are FP64-throughput bound (a GB300 SM
    // retires few FP64 FMAs per clock), so each mode gets as many SMs as the
    // GPU can co-schedule for all modes: minimise waves / blocks-per-mode.
    const ZftKernel kz = zft_kernel(g.n2m);
    cudaFuncSetAttribute(kz, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cudaFuncSetAttribute(zft_batch_kernel(g.n2m), cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    T->cs = 1;
    double best = 1e300;
    const int cands[5] = {16, 8, 4, 2, 1};
    for (int q = 0; q < 5; q++) {
        const int cs = cands[q];
        if (!cs_splits(*T, cs)) continue;
        cudaLaunchConfig_t lc;
        cudaLaunchAttribute at[1];
        cluster_cfg(lc, at, nmodes, cs);
        int nact = 0;
        if (cudaOccupancyMaxActiveClusters(&nact, kz, &lc) != cudaSuccess || nact < 1) {
            cudaGetLastError();
            continue;
        }
        const double waves = (double)((nmodes + nact - 1) / nact);
        const double cost = waves / cs;
        if (cost < best - 1e-12) { best = cost; T->cs = cs; }
    }
    // A caller sharing the GPU among many cases caps the cluster size: the
    // solve is latency-bound, so smaller clusters leave SMs to the other cases'
    // solves (the serving loop sets a cap on its worker thread; the
    // LESGPU_MG_CLUSTER_MAX environment variable sets one for every case).
    int cap = mg_cluster_cap();
    const char *env = getenv("LESGPU_MG_CLUSTER_MAX");
    if (env && atoi(env) >= 1) cap = atoi(env);
    T->cap = cap;
    if (cap >= 1)
        while (T->cs > cap) T->cs >>= 1;
    while (!cs_splits(*T, T->cs)) T->cs >>= 1;
    return 0;
}

static thread_local int t_mg_cluster_cap = 0;
int mg_cluster_cap() { return t_mg_cluster_cap; }
void set_mg_cluster_cap(int cap) { t_mg_cluster_cap = cap; }

void mg2d_free(lesgpu_case *c) {
    MgTables *T = c->pois.mg;
    if (!T) return;
    void *ptrs[] = {T->d.aw, T->d.ae, T->d.as, T->d.an, T->d.coi1, T->d.coi2, T->d.cor1, T->d.cor2, T->ipm, T->imm,
                    T->d.ac, T->d.bet, T->d.gam, T->d.pc, T->d.gg, T->d.rs, T->d.rd, T->d.gu, T->d.gb, T->iters,
                    T->f.aw, T->f.ae, T->f.as, T->f.an, T->f.coi1, T->f.coi2, T->f.cor1, T->f.cor2,
                    T->f.ac, T->f.bet, T->f.gam, T->f.pc, T->f.gg, T->f.rs, T->f.rd, T->f.gu, T->f.gb};
    for (void *q : ptrs) cudaFree(q);
    delete T;
    c->pois.mg = nullptr;
}

static MgArgs mg_args(lesgpu_case *c, int slot, int fixed_cycles) {
    const DGrid &g = c->kp.g;
    const lesgpu_config &cf = c->cfg;
    DPois &P = c->pois;
    MgTables *T = P.mg;
    MgArgs a;
    memset(&a, 0, sizeof(a));
    a.nl = T->nl; a.n2m = g.n2m; a.nld = T->nld; a.nlev = T->nlev;
    a.xft = T->xft;
    a.nbli = (int)cf.nbli; a.mgitr = fixed_cycles > 0 ? fixed_cycles : (int)cf.mgitr;
    a.imgsor = (int)cf.imgsor; a.wwsor = cf.wwsor;
    a.ldp = T->nl + 2; a.ldg = T->nld + 1;
    memcpy(a.iimg, T->iimg, sizeof(a.iimg));
    a.ipm = T->ipm; a.imm = T->imm;
    a.d = T->d; a.f = T->f;
    a.mixed = T->mixed;
    a.ccap = P.ccap;
    a.pc_plane = T->pc_plane; a.gg_plane = T->gg_plane;
    a.iters = T->iters; a.S = c->S; a.slot = slot;
    a.fixed_cycles = fixed_cycles;
    a.lc = T->lc;
    return a;
}

static void launch_modes(lesgpu_case *c, const MgArgs &a, int cs, int nmodes = 0) {
    cudaLaunchConfig_t lc;
    cudaLaunchAttribute at[1];
    cluster_cfg(lc, at, nmodes > 0 ? nmodes : c->pois.mg->nmodes, cs);
    lc.stream = c->stream;
    cudaLaunchKernelEx(&lc, zft_kernel(c->kp.g.n2m), a);
}

// can a cluster of cs blocks be scheduled at all
static bool cluster_fits(lesgpu_case *c, int cs) {
    cudaLaunchConfig_t lc;
    cudaLaunchAttribute at[1];
    cluster_cfg(lc, at, c->pois.mg->nmodes, cs);
    int nact = 0;
    if (cudaOccupancyMaxActiveClusters(&nact, zft_kernel(c->kp.g.n2m), &lc) != cudaSuccess) { cudaGetLastError(); return false; }
    return nact >= 1;
}

// The transforms around the mode solves: pre = the criterion of the
// substep and the forward transform into the modes, post = the inverse
// transform back to phi (z_ft: z; x_ft: x).
static void mg2d_pre(lesgpu_case *c, int slot) {
    const DGrid &g = c->kp.g;
    DPois &P = c->pois;
    if (P.mg->xft) {
        k_mg_begin<<<1, 1, 0, c->stream>>>(c->S, slot, g.n1m, g.n1mh, 0.9);
        const DevPlan px = devplan(P.fx);
        const int Lx = fft_lx(c);
        k_fft_xr_fwd<<<dim3((g.n3m + Lx - 1) / Lx, g.n2m), kThreads, (size_t)2 * g.n1m * Lx * sizeof(double2),
                       c->stream>>>(c->kp, P.ccap, px, Lx);
    } else {
        k_mg_begin<<<1, 1, 0, c->stream>>>(c->S, slot, g.n3m, g.n3mh, 0.8);
        const DevPlan pz = devplan(P.fz);
        const int Lz = fft_lz(c);
        const size_t smz = (size_t)2 * (g.n3m > 1 ? g.n3m : 1) * Lz * sizeof(double2);
        const dim3 gz((g.n1m + 2 * Lz - 1) / (2 * Lz), g.n2m);   // 2 Lz real lines per block
        const long long sk = (long long)g.n1m * g.n2m, sj = g.n1m;
        fft_z_fwd64(gz, smz, c->stream, c->kp, c->kp.f.divgsum, P.ccap, pz, Lz, sk, sj);
    }
}

static void mg2d_post(lesgpu_case *c) {
    const DGrid &g = c->kp.g;
    DPois &P = c->pois;
    if (P.mg->xft) {
        const DevPlan px = devplan(P.fx);
        const int Lx = fft_lx(c), pin = c->cfg.ich == 1 ? 1 : 0;
        const int Li = fft_xr_inv_lines(g.n1m, Lx, pin);
        k_fft_xr_inv<<<dim3((g.n3m + Li - 1) / Li, g.n2m), kThreads, (size_t)2 * g.n1m * (Li + pin) * sizeof(double2),
                       c->stream>>>(c->kp, P.ccap, px, Li, pin);
    } else {
        const DevPlan pz = devplan(P.fz);
        const int Lz = fft_lz(c);
        const size_t smz = (size_t)2 * (g.n3m > 1 ? g.n3m : 1) * Lz * sizeof(double2);
        const dim3 gz((g.n1m + 2 * Lz - 1) / (2 * Lz), g.n2m);
        const long long sk = (long long)g.n1m * g.n2m, sj = g.n1m;
        fft_z_inv64(gz, smz, c->stream, c->kp, P.ccap, pz, Lz, sk, sj);
    }
}

void launch_mg2d(lesgpu_case *c, int msub) {
    MgTables *T = c->pois.mg;
    const int slot = (msub >= 1 && msub <= 3) ? msub - 1 : 0;
    inst_begin(c, LESGPU_K_POISSON);
    mg2d_pre(c, slot);
    launch_modes(c, mg_args(c, slot, 0), T->cs);
    mg2d_post(c);
    inst_end(c, LESGPU_K_POISSON);
}

// ---- the serving loop's batched solve: the pieces of launch_mg2d apart,
// the mode solves of several cases of one shape in one launch
void mg2d_launch_pre(lesgpu_case *c, int msub) { mg2d_pre(c, (msub >= 1 && msub <= 3) ? msub - 1 : 0); }
void mg2d_launch_post(lesgpu_case *c) { mg2d_post(c); }
int mg2d_batch_size(const lesgpu_case *) { return (int)sizeof(MgArgs); }
void mg2d_batch_args(lesgpu_case *c, int msub, void *out) {
    const MgArgs a = mg_args(c, (msub >= 1 && msub <= 3) ? msub - 1 : 0, 0);
    memcpy(out, &a, sizeof(MgArgs));
}
// d_args: n MgArgs of cases with equal mg2d_batch_key
void mg2d_launch_batch(const lesgpu_case *c0, const void *d_args, int n, cudaStream_t st) {
    const MgTables *T = c0->pois.mg;
    cudaLaunchConfig_t lc;
    cudaLaunchAttribute at[1];
    cluster_cfg(lc, at, T->nmodes * n, T->cs);
    lc.stream = st;
    cudaLaunchKernelEx(&lc, zft_batch_kernel(c0->kp.g.n2m), (const MgArgs *)d_args, T->nmodes);
}
// what cases of one grid shape must share to be solved by one batched
// launch: the cluster size and the level layout it was checked against
long long mg2d_batch_key(const lesgpu_case *c) {
    const MgTables *T = c->pois.mg;
    if (!T) return 0;
    return (((long long)T->cs * 64 + T->nlev) * 64 + T->lc) * 4096 + T->nmodes;
}

// ---- autotuner: cluster size per mode.  A solve lasts as long as its
// slowest mode -- the zero wavenumber, which needs the most V-cycles while
// the others finish early -- and its cycle count depends on the data, so the
// candidates are timed on that mode alone, three V-cycles with the
// convergence test off (results go to scratch).
static std::map<std::array<int, 7>, int> g_zft_cs;
static std::mutex g_zft_mu;

int mg2d_autotune(lesgpu_case *c) {
    const DGrid &g = c->kp.g;
    MgTables *T = c->pois.mg;
    if (!T || (c->cfg.poisson != LESGPU_POISSON_Z_FT && c->cfg.poisson != LESGPU_POISSON_X_FT)) return 0;
    const std::array<int, 7> key{T->xft, g.n1m, g.n2m, g.n3m, T->nlev, (int)c->cfg.imgsor, T->cap};
    {
        std::lock_guard<std::mutex> lk(g_zft_mu);
        auto it = g_zft_cs.find(key);
        if (it != g_zft_cs.end()) { T->cs = it->second; return 0; }
    }
    const MgArgs a = mg_args(c, 0, 3);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int best = T->cs;
    float best_ms = 3.0e38f;
    for (int cs = 16; cs >= 1; cs >>= 1) {
        if (T->cap >= 1 && cs > T->cap) continue;
        if (!cs_splits(*T, cs) || !cluster_fits(c, cs)) continue;
        launch_modes(c, a, cs, 1);              // warm-up
        cudaEventRecord(e0, c->stream);
        for (int r = 0; r < 2; r++) launch_modes(c, a, cs, 1);
        cudaEventRecord(e1, c->stream);
        float ms = 0.0f;
        if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) break;
        if (ms < best_ms) { best_ms = ms; best = cs; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    T->cs = best;
    std::lock_guard<std::mutex> lk(g_zft_mu);
    g_zft_cs[key] = best;
    return cudaStreamSynchronize(c->stream) == cudaSuccess ? 0 : LESGPU_ERR_CUDA;
}
int mg2d_cluster(const lesgpu_case *c) { return c->pois.mg ? c->pois.mg->cs : 0; }

}  // namespace lg
