// poiss_mgrd: BiCGSTAB with a one-V-cycle MG3D preconditioner
// (poiss_mgrd.f90:25-993), the reference's third pressure solver.
//
// The whole solve -- every BiCGSTAB iteration, both V-cycles of each, the
// convergence test and the final pinning of phi -- is ONE cooperative
// persistent kernel.  Its phases are separated by grid-wide barriers; the
// scalars of the iteration (rho, alpha, omega) are reduced deterministically
// (fixed-order partials per block, summed in the same order by every block)
// so all blocks take the same branch at the convergence test.  A BiCGSTAB
// iteration is ~6 nlev + 2 nbli + 5 barriers instead of as many kernel
// launches, and the loop needs no host round trip, so it sits inside the
// captured step graph.
//
// MG3D levels are stored compactly, one (nx_l, n2+1, nz_l) block per level
// (level nlev is the caller's full-layout solution array), where the
// reference lays them side by side in (0:n1md, 0:n2, 0:n3md).  The 1-D
// coefficient and transfer tables keep the reference's concatenated index
// (iimg / kkmg ranges), so a neighbour or transfer index outside the level
// reads zero -- it always carries a zero coefficient or weight.
//
// Fusions (exact: the fused operands are disjoint): the right-hand side of a
// zebra half-sweep is formed in the same pass as the forward elimination;
// the finest residual and its restriction (toplevel) are one pass, and so
// are rescal and godown (every fine point belongs to one coarse point); the
// closing toplevel's residual, which mg3d discards, is not computed.
#include <cooperative_groups.h>

#include <cstring>
#include <vector>

#include "k_fft.cuh"
#include "lesgpu_internal.cuh"

namespace cg = cooperative_groups;

namespace lg {

constexpr int kMgrdThreads = 256;
constexpr int kMgrdMaxLev = 20;
constexpr int kMgrdSlots = 8;   // partial-sum slots per block

struct MgrdLevel {
    int ibg, iend, nx, kbg, kend, nz;
    long long goff, roff, loff;   // offsets in gc (rows 0..n2), rs and bet/gam (rows 1..n2m)
};

struct MgrdTables {
    int nlev, nblocks;
    MgrdLevel h_lev[kMgrdMaxLev + 1];
    MgrdLevel *lev;
    double *aw, *ae, *as, *an, *ab, *af, *fidw, *fkdw, *fiup, *fkup;
    int *imm, *ipm, *kmm, *kpm, *ih1, *ih2, *kh1, *kh2, *il1, *il2, *kl1, *kl2;
    double *bet, *gam, *gc, *rs;
    double *p, *s, *y, *z, *v, *t, *res, *part;
};

struct MgrdArgs {
    int n1m, n2m, n3m, n2, nlev, nbli, mgitr, slot;
    long long sx, sxy;
    const MgrdLevel *lev;
    const double *aw, *ae, *as, *an, *ab, *af, *fidw, *fkdw, *fiup, *fkup;
    const int *imm, *ipm, *kmm, *kpm, *ih1, *ih2, *kh1, *kh2, *il1, *il2, *kl1, *kl2;
    const double *bet, *gam;
    double *gc, *rs;
    double *p, *s, *y, *z, *v, *t, *res, *part;
    double *phi;
    const double *b;
    DScal *S;
};

// ------------------------------------------------------------ level access
struct LevelView {            // one level's storage, resolved once per phase
    MgrdLevel L;
    double *g;                // gi of the level
    long long sj, sk, gbase;  // gi index = gbase + i + sj * j + sk * k
    bool finest;
    __device__ LevelView(const MgrdArgs &a, double *sol, int l) {
        L = a.lev[l];
        finest = (l == a.nlev);
        if (finest) { g = sol; sj = a.sx; sk = a.sxy; gbase = 0; }
        else {
            g = a.gc; sj = L.nx; sk = (long long)L.nx * (a.n2 + 1);
            gbase = L.goff - L.ibg - sk * L.kbg;
        }
    }
    __device__ bool inside(int i, int k) const { return i >= L.ibg && i <= L.iend && k >= L.kbg && k <= L.kend; }
    __device__ long long gi(int i, int j, int k) const { return gbase + i + sj * j + sk * k; }
    __device__ double get(int i, int j, int k) const { return inside(i, k) ? g[gi(i, j, k)] : 0.0; }
    // resid and bet/gam: rows 1..n2m
    __device__ long long ri(const MgrdArgs &a, int i, int j, int k) const {
        return (long long)(i - L.ibg) + (long long)L.nx * ((j - 1) + (long long)a.n2m * (k - L.kbg));
    }
};

// rhs - A gi at a point of a level (rescal / toplevel residual, :353-364, :414-421)
__device__ __forceinline__ double mg_defect(const MgrdArgs &a, const LevelView &V, double rhs, int i, int j, int k) {
    const double acc = -1.0 * (a.aw[i] + a.ae[i] + a.as[j] + a.an[j] + a.ab[k] + a.af[k]);
    return rhs - acc * V.g[V.gi(i, j, k)] - a.aw[i] * V.get(a.imm[i], j, k) - a.ae[i] * V.get(a.ipm[i], j, k)
           - a.as[j] * V.g[V.gi(i, j - 1, k)] - a.an[j] * V.g[V.gi(i, j + 1, k)]
           - a.ab[k] * V.get(i, j, a.kmm[k]) - a.af[k] * V.get(i, j, a.kpm[k]);
}

// One zebra half-sweep of level l (relax :502-675 / toplevel :281-348): the y
// lines (i, k), i = ibg + (color 0: mod(kpm(k), 2); color 1: mod(k, 2)) + 2q,
// take src - iold * (x and z neighbours) and are solved with the stored LU.
// src is the full-layout right-hand side at the finest level, else resid.
__device__ void mg_half(const MgrdArgs &a, double *sol, const double *src, int l, int color, double iold,
                        long long tid, long long nthr) {
    const LevelView V(a, sol, l);
    const MgrdLevel &L = V.L;
    const int half = (L.nx + 1) >> 1;
    const long long nlines = (long long)half * L.nz;
    const int n2m = a.n2m;
    for (long long q = tid; q < nlines; q += nthr) {
        const int kk = (int)(q / half), hh = (int)(q - (long long)kk * half);
        const int k = L.kbg + kk;
        const int i = L.ibg + (color == 0 ? (a.kpm[k] & 1) : (k & 1)) + 2 * hh;
        if (i > L.iend) continue;
        const int im = a.imm[i], ip = a.ipm[i], km = a.kmm[k], kp = a.kpm[k];
        const bool vim = V.inside(im, k), vip = V.inside(ip, k), vkm = V.inside(i, km), vkp = V.inside(i, kp);
        const double cw = a.aw[i], ce = a.ae[i], cb = a.ab[k], cf = a.af[k];
        const long long g0 = V.gi(i, 0, k);
        const long long gw = vim ? V.gi(im, 0, k) : 0, ge = vip ? V.gi(ip, 0, k) : 0;
        const long long gb = vkm ? V.gi(i, 0, km) : 0, gf = vkp ? V.gi(i, 0, kp) : 0;
        const long long lu0 = L.loff + V.ri(a, i, 1, k) - L.nx;    // + nx * j
        const long long s0 = V.finest ? (long long)i + a.sxy * k : L.roff + V.ri(a, i, 1, k) - L.nx;
        const long long ss = V.finest ? a.sx : L.nx;
        double *g = V.g;
        double prev = 0.0;
        for (int j = 1; j <= n2m; j++) {
            const long long o = V.sj * j;
            double r = V.finest ? src[s0 + ss * j] : a.rs[s0 + ss * j];
            if (iold != 0.0) {
                const double nb = cw * (vim ? g[gw + o] : 0.0) + ce * (vip ? g[ge + o] : 0.0)
                                  + cb * (vkm ? g[gb + o] : 0.0) + cf * (vkp ? g[gf + o] : 0.0);
                r = r - iold * nb;
            }
            const double bt = a.bet[lu0 + (long long)L.nx * j];
            const double gv = (j == 1) ? r * bt : (r - a.as[j] * prev) * bt;
            g[g0 + o] = gv;
            prev = gv;
        }
        double next = prev;
        for (int j = n2m - 1; j >= 1; j--) {
            const long long o = V.sj * j;
            const double gv = g[g0 + o] - a.gam[lu0 + (long long)L.nx * (j + 1)] * next;
            g[g0 + o] = gv;
            next = gv;
        }
    }
}

// toplevel's residual at the finest level restricted to level nlev-1
// (:352-378), one coarse point per thread
__device__ void mg_top_restrict(const MgrdArgs &a, double *sol, const double *rhs, long long tid, long long nthr) {
    const LevelView F(a, sol, a.nlev);
    const MgrdLevel C = a.lev[a.nlev - 1];
    const long long n = (long long)C.nx * a.n2m * C.nz;
    for (long long q = tid; q < n; q += nthr) {
        const int ii = (int)(q % C.nx);
        const long long r = q / C.nx;
        const int j = 1 + (int)(r % a.n2m), kk = (int)(r / a.n2m);
        const int ic = C.ibg + ii, kc = C.kbg + kk;
        const int i1 = a.ih1[ic], i2 = a.ih2[ic], k1 = a.kh1[kc], k2 = a.kh2[kc];
        const double fi = a.fidw[ic], fk = a.fkdw[kc];
        const double r11 = mg_defect(a, F, rhs[i1 + a.sx * j + a.sxy * k1], i1, j, k1);
        const double r21 = mg_defect(a, F, rhs[i2 + a.sx * j + a.sxy * k1], i2, j, k1);
        const double r12 = mg_defect(a, F, rhs[i1 + a.sx * j + a.sxy * k2], i1, j, k2);
        const double r22 = mg_defect(a, F, rhs[i2 + a.sx * j + a.sxy * k2], i2, j, k2);
        a.rs[C.roff + q] = (1.0 - fi) * (1.0 - fk) * r11 + fi * (1.0 - fk) * r21 + (1.0 - fi) * fk * r12 + fi * fk * r22;
    }
}

// rescal(l) (:403-425) then godown(l-1) (:455-476), one coarse point per
// thread: the four level-l defects replace resid there and are restricted
__device__ void mg_rescal_godown(const MgrdArgs &a, double *sol, int l, long long tid, long long nthr) {
    const LevelView F(a, sol, l);
    const MgrdLevel C = a.lev[l - 1];
    const long long n = (long long)C.nx * a.n2m * C.nz;
    for (long long q = tid; q < n; q += nthr) {
        const int ii = (int)(q % C.nx);
        const long long r = q / C.nx;
        const int j = 1 + (int)(r % a.n2m), kk = (int)(r / a.n2m);
        const int ic = C.ibg + ii, kc = C.kbg + kk;
        const int i1 = a.ih1[ic], i2 = a.ih2[ic], k1 = a.kh1[kc], k2 = a.kh2[kc];
        const double fi = a.fidw[ic], fk = a.fkdw[kc];
        const long long q11 = F.L.roff + F.ri(a, i1, j, k1), q21 = F.L.roff + F.ri(a, i2, j, k1);
        const long long q12 = F.L.roff + F.ri(a, i1, j, k2), q22 = F.L.roff + F.ri(a, i2, j, k2);
        const double r11 = mg_defect(a, F, a.rs[q11], i1, j, k1);
        const double r21 = mg_defect(a, F, a.rs[q21], i2, j, k1);
        const double r12 = mg_defect(a, F, a.rs[q12], i1, j, k2);
        const double r22 = mg_defect(a, F, a.rs[q22], i2, j, k2);
        a.rs[q11] = r11; a.rs[q21] = r21; a.rs[q12] = r12; a.rs[q22] = r22;
        a.rs[C.roff + q] = (1.0 - fi) * (1.0 - fk) * r11 + fi * (1.0 - fk) * r21 + (1.0 - fi) * fk * r12 + fi * fk * r22;
    }
}

// goup(l) (:479-500): the points i = ibg + mod(k, 2) + 2q of level l gain
// the interpolated correction of level l-1
__device__ void mg_goup(const MgrdArgs &a, double *sol, int l, long long tid, long long nthr) {
    const LevelView F(a, sol, l), C(a, sol, l - 1);
    const MgrdLevel &L = F.L;
    const int half = (L.nx + 1) >> 1;
    const long long n = (long long)half * a.n2m * L.nz;
    for (long long q = tid; q < n; q += nthr) {
        const int hh = (int)(q % half);
        const long long r = q / half;
        const int j = 1 + (int)(r % a.n2m), k = L.kbg + (int)(r / a.n2m);
        const int i = L.ibg + (k & 1) + 2 * hh;
        if (i > L.iend) continue;
        const double fi = a.fiup[i], fk = a.fkup[k];
        const int a1 = a.il1[i], a2 = a.il2[i], b1 = a.kl1[k], b2 = a.kl2[k];
        const long long o = F.gi(i, j, k);
        F.g[o] = F.g[o] + (1.0 - fi) * (1.0 - fk) * C.get(a1, j, b1) + fi * (1.0 - fk) * C.get(a2, j, b1)
                 + (1.0 - fi) * fk * C.get(a1, j, b2) + fi * fk * C.get(a2, j, b2);
    }
}

// mg3d (:227-268): one V-cycle, sol = M^-1 rhs.  The first half-sweep takes
// no neighbours (IOLD = 0; with IOLD = 1 the reference reads its
// uninitialised work array there, which is zero here).
__device__ void mg3d(const MgrdArgs &a, cg::grid_group &grid, double *sol, const double *rhs, long long tid, long long nthr) {
    const int nlev = a.nlev;
    mg_half(a, sol, rhs, nlev, 0, 0.0, tid, nthr); grid.sync();
    mg_half(a, sol, rhs, nlev, 1, 1.0, tid, nthr); grid.sync();
    if (nlev > 0) {
        mg_top_restrict(a, sol, rhs, tid, nthr); grid.sync();
        for (int l = nlev - 1; l >= 1; l--) {
            mg_half(a, sol, nullptr, l, 0, 0.0, tid, nthr); grid.sync();
            mg_half(a, sol, nullptr, l, 1, 1.0, tid, nthr); grid.sync();
            mg_rescal_godown(a, sol, l, tid, nthr); grid.sync();
        }
        mg_half(a, sol, nullptr, 0, 0, 0.0, tid, nthr); grid.sync();
        mg_half(a, sol, nullptr, 0, 1, 1.0, tid, nthr); grid.sync();
        for (int it = 1; it < a.nbli; it++) {
            mg_half(a, sol, nullptr, 0, 0, 1.0, tid, nthr); grid.sync();
            mg_half(a, sol, nullptr, 0, 1, 1.0, tid, nthr); grid.sync();
        }
        for (int l = 1; l <= nlev - 1; l++) {
            mg_goup(a, sol, l, tid, nthr); grid.sync();
            mg_half(a, sol, nullptr, l, 0, 1.0, tid, nthr); grid.sync();
            mg_half(a, sol, nullptr, l, 1, 1.0, tid, nthr); grid.sync();
        }
        mg_goup(a, sol, nlev, tid, nthr); grid.sync();
    }
    mg_half(a, sol, rhs, nlev, 0, 1.0, tid, nthr); grid.sync();
    mg_half(a, sol, rhs, nlev, 1, 1.0, tid, nthr); grid.sync();
}

// ------------------------------------------------------------ reductions
// Sum (or max) of N values over the block; every thread gets the same
// totals (warp trees, then the warps' sums in a fixed order).
template <int N>
__device__ void block_reduce(double (&v)[N], const bool (&is_max)[N], double *sh) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int q = 0; q < N; q++) {
        double x = v[q];
        for (int o = 16; o > 0; o >>= 1) {
            const double y = __shfl_xor_sync(0xffffffffu, x, o);
            x = is_max[q] ? fmax(x, y) : x + y;
        }
        if (lane == 0) sh[q * 32 + wid] = x;
    }
    __syncthreads();
    for (int q = 0; q < N; q++) {
        double x = 0.0;                 // the maxima are of absolute values
        for (int w = 0; w < nw; w++) x = is_max[q] ? fmax(x, sh[q * 32 + w]) : x + sh[q * 32 + w];
        v[q] = x;
    }
    __syncthreads();
}

// Grid-wide totals: block partials to slots, barrier, every block reduces
// all partials in the same order.
template <int N>
__device__ void grid_reduce(const MgrdArgs &a, cg::grid_group &grid, double (&v)[N], const bool (&is_max)[N],
                            const int (&slot)[N], double *sh) {
    block_reduce<N>(v, is_max, sh);
    if (threadIdx.x == 0)
        for (int q = 0; q < N; q++) a.part[(long long)blockIdx.x * kMgrdSlots + slot[q]] = v[q];
    grid.sync();
    double w[N];
    for (int q = 0; q < N; q++) {
        w[q] = 0.0;
        for (int bk = threadIdx.x; bk < (int)gridDim.x; bk += blockDim.x) {
            const double x = a.part[(long long)bk * kMgrdSlots + slot[q]];
            w[q] = is_max[q] ? fmax(w[q], x) : w[q] + x;
        }
    }
    block_reduce<N>(w, is_max, sh);
    for (int q = 0; q < N; q++) v[q] = w[q];
}

// A q at an interior point: the 7-point operator of poisson (:113-122)
__device__ __forceinline__ double mg_apply(const MgrdArgs &a, const double *q, int i, int j, int k) {
    const double acc = -1.0 * (a.aw[i] + a.ae[i] + a.as[j] + a.an[j] + a.ab[k] + a.af[k]);
    const long long c = i + a.sx * j + a.sxy * k;
    return a.aw[i] * q[a.imm[i] + a.sx * j + a.sxy * k] + a.ae[i] * q[a.ipm[i] + a.sx * j + a.sxy * k]
           + a.as[j] * q[c - a.sx] + a.an[j] * q[c + a.sx]
           + a.ab[k] * q[i + a.sx * j + a.sxy * a.kmm[k]] + a.af[k] * q[i + a.sx * j + a.sxy * a.kpm[k]] + acc * q[c];
}

// poisson (:25-224): phi = A^-1 divgsum to max|res| < test1, then
// phi -= phi(1, n2m, 1).  IOLDV = 1 also starts from phi = 0 (solver.f90
// zeroes phi before every call).
__global__ void __launch_bounds__(kMgrdThreads) k_mgrd_solve(MgrdArgs a) {
    cg::grid_group grid = cg::this_grid();
    __shared__ double sh[4 * 32];
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long nthr = (long long)gridDim.x * blockDim.x;
    const int n1m = a.n1m, n2m = a.n2m;
    const long long nin = (long long)n1m * n2m * a.n3m;
    const long long ntot = a.sxy * (a.n3m + 2);
    auto at = [&](long long q, int &i, int &j, int &k) {
        i = 1 + (int)(q % n1m);
        const long long r = q / n1m;
        j = 1 + (int)(r % n2m);
        k = 1 + (int)(r / n2m);
        return i + a.sx * j + a.sxy * k;
    };
    for (long long q = tid; q < ntot; q += nthr) a.phi[q] = 0.0;
    double r1[1] = {0.0};
    const bool sum1[1] = {false};
    for (long long q = tid; q < nin; q += nthr) {
        int i, j, k;
        const long long c = at(q, i, j, k);
        const double bb = a.b[c];
        a.res[c] = bb;
        a.p[c] = 0.0;
        a.v[c] = 0.0;
        r1[0] += bb * bb;
    }
    const int sl0[1] = {0};
    grid_reduce<1>(a, grid, r1, sum1, sl0, sh);
    double rho = r1[0], rho_ol = 1.0, alp = 1.0, w = 1.0;
    const double test1 = a.S->test1;
    int done = a.mgitr;
    bool conv = false;
    for (int it = 1; it <= a.mgitr; it++) {
        const double bet = rho / rho_ol * alp / w;
        for (long long q = tid; q < nin; q += nthr) {
            int i, j, k;
            const long long c = at(q, i, j, k);
            a.p[c] = a.res[c] + bet * (a.p[c] - w * a.v[c]);
        }
        grid.sync();
        mg3d(a, grid, a.y, a.p, tid, nthr);
        double rv[1] = {0.0};
        for (long long q = tid; q < nin; q += nthr) {
            int i, j, k;
            const long long c = at(q, i, j, k);
            const double vv = mg_apply(a, a.y, i, j, k);
            a.v[c] = vv;
            rv[0] += a.b[c] * vv;
        }
        const int sl1[1] = {1};
        grid_reduce<1>(a, grid, rv, sum1, sl1, sh);
        alp = rho / rv[0];
        for (long long q = tid; q < nin; q += nthr) {
            int i, j, k;
            const long long c = at(q, i, j, k);
            a.s[c] = a.res[c] - alp * a.v[c];
        }
        grid.sync();
        mg3d(a, grid, a.z, a.s, tid, nthr);
        double ub[2] = {0.0, 0.0};
        const bool sum2[2] = {false, false};
        for (long long q = tid; q < nin; q += nthr) {
            int i, j, k;
            const long long c = at(q, i, j, k);
            const double tt = mg_apply(a, a.z, i, j, k);
            a.t[c] = tt;
            ub[0] += tt * a.s[c];
            ub[1] += tt * tt;
        }
        const int sl2[2] = {2, 3};
        grid_reduce<2>(a, grid, ub, sum2, sl2, sh);
        w = ub[0] / ub[1];
        double mr[2] = {0.0, 0.0};
        const bool mx[2] = {true, false};
        for (long long q = tid; q < nin; q += nthr) {
            int i, j, k;
            const long long c = at(q, i, j, k);
            a.phi[c] = a.phi[c] + alp * a.y[c] + w * a.z[c];
            const double rr = a.s[c] - w * a.t[c];
            a.res[c] = rr;
            mr[0] = fmax(mr[0], fabs(rr));
            mr[1] += a.b[c] * rr;        // the next iteration's rho
        }
        const int sl3[2] = {4, 0};
        grid_reduce<2>(a, grid, mr, mx, sl3, sh);
        rho_ol = rho;
        rho = mr[1];
        if (mr[0] < test1) { done = it; conv = true; break; }
    }
    const double phiref = a.phi[1 + a.sx * n2m + a.sxy * 1];
    grid.sync();
    for (long long q = tid; q < nin; q += nthr) {
        int i, j, k;
        const long long c = at(q, i, j, k);
        a.phi[c] = a.phi[c] - phiref;
    }
    if (tid == 0) {
        a.S->poisson_iters[a.slot] = done;
        if (!conv) a.S->poisson_unconv += 1;   // poiss_mgrd.f90:204 prints NOT CONVERGED and goes on
    }
}

// ------------------------------------------------------------ host side
// poisinit + mgcoef + tridcoef (:678-993)
int mgrd_init(lesgpu_case *c) {
    const DGrid &g = c->kp.g;
    const lesgpu_config &cf = c->cfg;
    const lesgpu_grid *hg = c->h_grid;
    const int n1 = g.n1, n3 = g.n3, n1m = g.n1m, n2m = g.n2m, n3m = g.n3m;
    const int nlev = (int)cf.nlev, n1md = 2 * n1m, n3md = 2 * n3m;
    if (nlev < 0 || nlev > kMgrdMaxLev || n1m % (1 << nlev) != 0 || n3m % (1 << nlev) != 0) return LESGPU_ERR_CONFIG;
    if (cf.yprdic == 1) return LESGPU_ERR_UNSUPPORTED;
    if (cf.mgitr < 0 || cf.mgitr > 1000000 || cf.nbli < 1) return LESGPU_ERR_CONFIG;
    for (int l = 0; l <= nlev; l++) {          // periodic directions need a proper zebra on every level
        const int nx = n1m >> (nlev - l), nz = n3m >> (nlev - l);
        if ((cf.xprdic == 1 && nx > 1 && nx % 2) || (cf.zprdic == 1 && nz > 1 && nz % 2)) return LESGPU_ERR_CONFIG;
    }
    auto v0 = [](const double *p, int n) { std::vector<double> v(n + 2, 0.0); for (int q = 0; q <= n; q++) v[q] = p[q]; return v; };
    auto v1 = [](const double *p, int n) { std::vector<double> v(n + 2, 0.0); for (int q = 1; q <= n; q++) v[q] = p[q - 1]; return v; };
    auto i1 = [](const int64_t *p, int n) { std::vector<long long> v(n + 2, 0); for (int q = 1; q <= n; q++) v[q] = p[q - 1]; return v; };
    const std::vector<double> x = v1(hg->x, n1), z = v1(hg->z, n3), xmp = v0(hg->xmp, n1), zmp = v0(hg->zmp, n3);
    const std::vector<double> c2cxi = v0(hg->c2cxi, n1), f2fxi = v0(hg->f2fxi, n1), c2cyi = v0(hg->c2cyi, g.n2);
    const std::vector<double> f2fyi = v0(hg->f2fyi, g.n2), c2czi = v0(hg->c2czi, n3), f2fzi = v0(hg->f2fzi, n3);
    const std::vector<long long> ipv = i1(hg->ipv, n1m), jpv = i1(hg->jpv, n2m), kpv = i1(hg->kpv, n3m);
    const std::vector<long long> fixil = i1(hg->fixil, n1m), fixiu = i1(hg->fixiu, n1m), fixjl = i1(hg->fixjl, n2m);
    const std::vector<long long> fixju = i1(hg->fixju, n2m), fixkl = i1(hg->fixkl, n3m), fixku = i1(hg->fixku, n3m);
    const size_t nvx = (size_t)n1md + 2, nvz = (size_t)n3md + 2;
    std::vector<double> aw(nvx, 0.0), ae(nvx, 0.0), as(n2m + 2, 0.0), an(n2m + 2, 0.0), ab(nvz, 0.0), af(nvz, 0.0);
    std::vector<double> fidw(nvx, 0.0), fiup(nvx, 0.0), fkdw(nvz, 0.0), fkup(nvz, 0.0);
    std::vector<int> ih1(nvx, 0), ih2(nvx, 0), il1(nvx, 0), il2(nvx, 0), imm(nvx, 0), ipm(nvx, 0);
    std::vector<int> kh1(nvz, 0), kh2(nvz, 0), kl1(nvz, 0), kl2(nvz, 0), kmm(nvz, 0), kpm(nvz, 0);
    // poisinit: finest-level coefficients
    for (int i = 1; i <= n1m; i++) {
        aw[i] = (1.0 - (double)fixil[i]) * c2cxi[i] * f2fxi[i];
        ae[i] = (1.0 - (double)fixiu[i]) * c2cxi[ipv[i]] * f2fxi[i];
    }
    for (int j = 1; j <= n2m; j++) {
        as[j] = (1.0 - (double)fixjl[j]) * c2cyi[j] * f2fyi[j];
        an[j] = (1.0 - (double)fixju[j]) * c2cyi[jpv[j]] * f2fyi[j];
    }
    for (int k = 1; k <= n3m; k++) {
        ab[k] = (1.0 - (double)fixkl[k]) * c2czi[k] * f2fzi[k];
        af[k] = (1.0 - (double)fixku[k]) * c2czi[kpv[k]] * f2fzi[k];
    }
    // mgcoef: level ranges (iimg / kkmg)
    int ib[kMgrdMaxLev + 1], ie[kMgrdMaxLev + 1], kb[kMgrdMaxLev + 1], ke[kMgrdMaxLev + 1];
    ib[nlev] = 1; ie[nlev] = n1m; kb[nlev] = 1; ke[nlev] = n3m;
    for (int l = nlev - 1; l >= 0; l--) {
        const int nx = (n1m >> nlev) << l, nz = (n3m >> nlev) << l;
        ib[l] = ie[l + 1] + 1; ie[l] = ib[l] + nx - 1;
        kb[l] = ke[l + 1] + 1; ke[l] = kb[l] + nz - 1;
    }
    std::vector<double> xmpm(nvx, 0.0), zmpm(nvz, 0.0);
    std::vector<int> iwest(nvx, 0), ieast(nvx, 0), kback(nvz, 0), kforw(nvz, 0);
    for (int i = 1; i <= n1m; i++) { xmpm[i] = xmp[i]; iwest[i] = i > 1; ieast[i] = i < n1m; }
    for (int k = 1; k <= n3m; k++) { zmpm[k] = zmp[k]; kback[k] = k > 1; kforw[k] = k < n3m; }
    for (int l = nlev - 1; l >= 0; l--) {
        const int sp = 1 << (nlev - l);
        for (int i = ib[l], ic = 1; i <= ie[l]; i++, ic++) {
            xmpm[i] = 0.5 * (x[(ic - 1) * sp + 1] + x[ic * sp + 1]);
            iwest[i] = i > ib[l]; ieast[i] = i < ie[l];
        }
        for (int k = kb[l], kc = 1; k <= ke[l]; k++, kc++) {
            zmpm[k] = 0.5 * (z[(kc - 1) * sp + 1] + z[kc * sp + 1]);
            kback[k] = k > kb[l]; kforw[k] = k < ke[l];
        }
        // a zero factor (non-periodic edge) multiplies a difference with a point
        // outside the level; the coefficient is zero
        for (int i = ib[l], ic = 1; i <= ie[l]; i++, ic++) {
            const double w = x[ic * sp + 1] - x[(ic - 1) * sp + 1];
            aw[i] = iwest[i] ? 1.0 / ((xmpm[i] - xmpm[i - 1]) * w) : 0.0;
            ae[i] = ieast[i] ? 1.0 / ((xmpm[i + 1] - xmpm[i]) * w) : 0.0;
        }
        for (int k = kb[l], kc = 1; k <= ke[l]; k++, kc++) {
            const double w = z[kc * sp + 1] - z[(kc - 1) * sp + 1];
            ab[k] = kback[k] ? 1.0 / ((zmpm[k] - zmpm[k - 1]) * w) : 0.0;
            af[k] = kforw[k] ? 1.0 / ((zmpm[k + 1] - zmpm[k]) * w) : 0.0;
        }
    }
    for (int l = 0; l <= nlev - 1; l++) {          // restriction
        for (int i = ib[l], h = ib[l + 1]; i <= ie[l]; i++, h += 2) {
            fidw[i] = (xmpm[i] - xmpm[h]) / (xmpm[h + 1] - xmpm[h]);
            ih1[i] = h; ih2[i] = h + 1;
        }
        for (int k = kb[l], h = kb[l + 1]; k <= ke[l]; k++, h += 2) {
            fkdw[k] = (zmpm[k] - zmpm[h]) / (zmpm[h + 1] - zmpm[h]);
            kh1[k] = h; kh2[k] = h + 1;
        }
    }
    for (int l = 1; l <= nlev; l++) {              // prolongation; Neumann weights at the ends
        for (int i = ib[l], lo = ib[l - 1]; i <= ie[l]; i += 2, lo++) {
            if (i > ib[l]) fiup[i] = (xmpm[i] - xmpm[lo - 1]) / (xmpm[lo] - xmpm[lo - 1]);
            if (i + 1 < ie[l]) fiup[i + 1] = (xmpm[i + 1] - xmpm[lo]) / (xmpm[lo + 1] - xmpm[lo]);
            il1[i] = lo - 1; il2[i] = lo; il1[i + 1] = lo; il2[i + 1] = lo + 1;
        }
        fiup[ib[l]] = 1.0; fiup[ie[l]] = 0.0;
        for (int k = kb[l], lo = kb[l - 1]; k <= ke[l]; k += 2, lo++) {
            if (k > kb[l]) fkup[k] = (zmpm[k] - zmpm[lo - 1]) / (zmpm[lo] - zmpm[lo - 1]);
            if (k + 1 < ke[l]) fkup[k + 1] = (zmpm[k + 1] - zmpm[lo]) / (zmpm[lo + 1] - zmpm[lo]);
            kl1[k] = lo - 1; kl2[k] = lo; kl1[k + 1] = lo; kl2[k + 1] = lo + 1;
        }
        fkup[kb[l]] = 1.0; fkup[ke[l]] = 0.0;
    }
    for (int l = nlev; l >= 0; l--) {
        for (int k = kb[l]; k <= ke[l]; k++) { kpm[k] = k + 1; kmm[k] = k - 1; }
        for (int i = ib[l]; i <= ie[l]; i++) { ipm[i] = i + 1; imm[i] = i - 1; }
    }
    if (cf.xprdic == 1) {
        for (int l = nlev; l >= 0; l--) { ipm[ie[l]] = ib[l]; imm[ib[l]] = ie[l]; }
        for (int l = nlev - 1; l >= 0; l--) {
            const int sp = 1 << (nlev - l);
            const double vdx = xmpm[ib[l]] - x[1] + x[n1] - xmpm[ie[l]];
            aw[ib[l]] = 1.0 / (vdx * (x[1 + sp] - x[1]));
            ae[ie[l]] = 1.0 / (vdx * (x[n1] - x[n1 - sp]));
        }
        for (int l = 1; l <= nlev; l++) {
            const double dx = xmpm[ib[l - 1]] - x[1] + x[n1] - xmpm[ie[l - 1]];
            fiup[ib[l]] = (x[n1] - xmpm[ie[l - 1]] + xmpm[ib[l]] - x[1]) / dx;
            fiup[ie[l]] = (xmpm[ie[l]] - xmpm[ie[l - 1]]) / dx;
            il1[ib[l]] = ie[l - 1]; il2[ib[l]] = ib[l - 1]; il1[ie[l]] = ie[l - 1]; il2[ie[l]] = ib[l - 1];
        }
    }
    if (cf.zprdic == 1) {
        for (int l = nlev; l >= 0; l--) { kpm[ke[l]] = kb[l]; kmm[kb[l]] = ke[l]; }
        for (int l = nlev - 1; l >= 0; l--) {
            const int sp = 1 << (nlev - l);
            const double vdz = zmpm[kb[l]] - z[1] + z[n3] - zmpm[ke[l]];
            ab[kb[l]] = 1.0 / (vdz * (z[1 + sp] - z[1]));
            af[ke[l]] = 1.0 / (vdz * (z[n3] - z[n3 - sp]));
        }
        for (int l = 1; l <= nlev; l++) {
            const double dz = zmpm[kb[l - 1]] - z[1] + z[n3] - zmpm[ke[l - 1]];
            fkup[kb[l]] = (z[n3] - zmpm[ke[l - 1]] + zmpm[kb[l]] - z[1]) / dz;
            fkup[ke[l]] = (zmpm[ke[l]] - zmpm[ke[l - 1]]) / dz;
            kl1[kb[l]] = ke[l - 1]; kl2[kb[l]] = kb[l - 1]; kl1[ke[l]] = ke[l - 1]; kl2[ke[l]] = kb[l - 1];
        }
    }
    // compact level storage and tridcoef's LU, level by level
    MgrdTables *T = new MgrdTables();
    memset(T, 0, sizeof(*T));
    c->pois.mgrd = T;
    T->nlev = nlev;
    long long goff = 0, roff = 0, loff = 0;
    for (int l = 0; l <= nlev; l++) {
        MgrdLevel &L = T->h_lev[l];
        L.ibg = ib[l]; L.iend = ie[l]; L.nx = ie[l] - ib[l] + 1;
        L.kbg = kb[l]; L.kend = ke[l]; L.nz = ke[l] - kb[l] + 1;
        const long long plane = (long long)L.nx * L.nz;
        L.goff = goff; L.roff = roff; L.loff = loff;
        if (l < nlev) { goff += plane * (g.n2 + 1); roff += plane * n2m; }
        loff += plane * n2m;
    }
    std::vector<double> bet((size_t)loff, 0.0), gam((size_t)loff, 0.0);
    for (int l = 0; l <= nlev; l++) {
        const MgrdLevel &L = T->h_lev[l];
        auto at = [&](int i, int j, int k) { return (size_t)(L.loff + (i - L.ibg) + (long long)L.nx * ((j - 1) + (long long)n2m * (k - L.kbg))); };
        for (int k = L.kbg; k <= L.kend; k++)
            for (int i = L.ibg; i <= L.iend; i++) {
                double acc = -1.0 * (aw[i] + ae[i] + as[1] + an[1] + ab[k] + af[k]);
                bet[at(i, 1, k)] = 1.0 / acc;
                for (int j = 2; j <= n2m; j++) {
                    acc = -1.0 * (aw[i] + ae[i] + as[j] + an[j] + ab[k] + af[k]);
                    const double gm = an[j - 1] * bet[at(i, j - 1, k)];
                    gam[at(i, j, k)] = gm;
                    bet[at(i, j, k)] = 1.0 / (acc - as[j] * gm);
                }
            }
    }
    bool ok = true;
    auto up = [&](auto *&dst, const auto &v) {
        using T0 = typename std::remove_reference<decltype(v[0])>::type;
        if (cudaMalloc((void **)&dst, sizeof(T0) * v.size()) != cudaSuccess) { ok = false; return; }
        cudaMemcpy(dst, v.data(), sizeof(T0) * v.size(), cudaMemcpyHostToDevice);
    };
    up(T->aw, aw); up(T->ae, ae); up(T->as, as); up(T->an, an); up(T->ab, ab); up(T->af, af);
    up(T->fidw, fidw); up(T->fkdw, fkdw); up(T->fiup, fiup); up(T->fkup, fkup);
    up(T->imm, imm); up(T->ipm, ipm); up(T->kmm, kmm); up(T->kpm, kpm);
    up(T->ih1, ih1); up(T->ih2, ih2); up(T->kh1, kh1); up(T->kh2, kh2);
    up(T->il1, il1); up(T->il2, il2); up(T->kl1, kl1); up(T->kl2, kl2);
    up(T->bet, bet); up(T->gam, gam);
    std::vector<MgrdLevel> lev(T->h_lev, T->h_lev + nlev + 1);
    up(T->lev, lev);
    if (!ok) return LESGPU_ERR_OOM;
    const size_t nt = (size_t)g.nt;
    double **vecs[7] = {&T->p, &T->s, &T->y, &T->z, &T->v, &T->t, &T->res};
    for (double **pv : vecs) {
        if (cudaMalloc((void **)pv, sizeof(double) * nt) != cudaSuccess) return LESGPU_ERR_OOM;
        cudaMemset(*pv, 0, sizeof(double) * nt);      // ghost cells are read as zeros and never written
    }
    if (cudaMalloc(&T->gc, sizeof(double) * (size_t)(goff > 0 ? goff : 1)) != cudaSuccess ||
        cudaMalloc(&T->rs, sizeof(double) * (size_t)(roff > 0 ? roff : 1)) != cudaSuccess)
        return LESGPU_ERR_OOM;
    cudaMemset(T->gc, 0, sizeof(double) * (size_t)(goff > 0 ? goff : 1));   // ghost rows j = 0, n2 stay zero
    // persistent grid: every block co-resident (a cooperative launch checks
    // it); at most two blocks per SM keeps the barriers short
    int dev = 0, nsm = 0, occ = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_mgrd_solve, kMgrdThreads, 0) != cudaSuccess || occ < 1)
        return LESGPU_ERR_CUDA;
    T->nblocks = nsm * (occ < 2 ? occ : 2);
    if (cudaMalloc(&T->part, sizeof(double) * kMgrdSlots * (size_t)T->nblocks) != cudaSuccess) return LESGPU_ERR_OOM;
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : LESGPU_ERR_CUDA;
}

void mgrd_free(lesgpu_case *c) {
    MgrdTables *T = c->pois.mgrd;
    if (!T) return;
    void *ptrs[] = {T->lev, T->aw, T->ae, T->as, T->an, T->ab, T->af, T->fidw, T->fkdw, T->fiup, T->fkup,
                    T->imm, T->ipm, T->kmm, T->kpm, T->ih1, T->ih2, T->kh1, T->kh2, T->il1, T->il2, T->kl1, T->kl2,
                    T->bet, T->gam, T->gc, T->rs, T->p, T->s, T->y, T->z, T->v, T->t, T->res, T->part};
    for (void *q : ptrs) cudaFree(q);
    delete T;
    c->pois.mgrd = nullptr;
}

void launch_mgrd(lesgpu_case *c, int msub) {
    const DGrid &g = c->kp.g;
    const lesgpu_config &cf = c->cfg;
    MgrdTables *T = c->pois.mgrd;
    MgrdArgs a;
    memset(&a, 0, sizeof(a));
    a.n1m = g.n1m; a.n2m = g.n2m; a.n3m = g.n3m; a.n2 = g.n2;
    a.nlev = T->nlev; a.nbli = (int)cf.nbli; a.mgitr = (int)cf.mgitr;
    a.slot = (msub >= 1 && msub <= 3) ? msub - 1 : 0;
    a.sx = g.sx; a.sxy = g.sxy;
    a.lev = T->lev;
    a.aw = T->aw; a.ae = T->ae; a.as = T->as; a.an = T->an; a.ab = T->ab; a.af = T->af;
    a.fidw = T->fidw; a.fkdw = T->fkdw; a.fiup = T->fiup; a.fkup = T->fkup;
    a.imm = T->imm; a.ipm = T->ipm; a.kmm = T->kmm; a.kpm = T->kpm;
    a.ih1 = T->ih1; a.ih2 = T->ih2; a.kh1 = T->kh1; a.kh2 = T->kh2;
    a.il1 = T->il1; a.il2 = T->il2; a.kl1 = T->kl1; a.kl2 = T->kl2;
    a.bet = T->bet; a.gam = T->gam; a.gc = T->gc; a.rs = T->rs;
    a.p = T->p; a.s = T->s; a.y = T->y; a.z = T->z; a.v = T->v; a.t = T->t; a.res = T->res; a.part = T->part;
    a.phi = c->kp.f.phi; a.b = c->kp.f.divgsum; a.S = c->S;
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3(T->nblocks);
    lc.blockDim = dim3(kMgrdThreads);
    lc.stream = c->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    lc.attrs = at;
    lc.numAttrs = 1;
    inst_begin(c, LESGPU_K_POISSON);
    cudaLaunchKernelEx(&lc, k_mgrd_solve, a);
    inst_end(c, LESGPU_K_POISSON);
}

}  // namespace lg
