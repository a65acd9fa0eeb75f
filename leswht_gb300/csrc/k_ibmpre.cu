// Immersed-boundary pre-processing on the GPU: the geometry routines the
// reference's pre-processor runs through f2py (ibm_body.f90 find_inout :14-46,
// findbdy_intp :49-123, geomfac_preset :126-157, geomfac_intp :160-322,
// find_zero_nu_sgs :357-399, driven by preprocessing.py and written by
// lib_preprocessing.py:223-328).  The tables come out exactly as the
// pre-processor's files would give them back to the solver:
//   * forcing points in the reference's k, j, i loop order, interpolated
//     points first, found by order-preserving compaction (a block-level
//     prefix sum, deterministic);
//   * geomfac rounded to the 8 decimals of its '%15.8f' text (an exact
//     round-half-even of v * 1e8 using the FMA residual of the product, then
//     k / 1e8 correctly rounded -- the value strtod reads back);
//   * the zero-viscosity list in numpy's nonzero order of the (i, j, k)
//     transposed mask, 0-based as written.
// Every floating-point operation is the round-to-nearest intrinsic of the
// host restatement's operation in the same order, so no contraction changes
// a bisection step or a weight.
#include <cstring>
#include <vector>

#include "lesgpu_internal.cuh"

struct lesgpu_ibmpre {
    int nl;
    int64_t nintp[4], nbody[4], nzero;
    std::vector<int64_t> fc[4], ix[4], inz, jnz, knz, nwall;
    std::vector<double> gf[4];
};

namespace lg {
namespace ibp {

struct Body {
    int kind;
    double cx, cy, cz, r, p0;
};

__device__ double fbody(const Body &b, double x, double y, double z) {
    switch (b.kind) {
    case LESGPU_BODY_CHANNEL:
        return __dadd_rn(__dadd_rn(__dsub_rn(__dadd_rn(1.0, b.p0), fabs(y)), __dmul_rn(0.0, x)), __dmul_rn(0.0, z));
    case LESGPU_BODY_CYLINDER: {
        const double dx = __dsub_rn(x, b.cx), dy = __dsub_rn(y, b.cy);
        return __dadd_rn(__dsub_rn(__dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy))), b.r), __dmul_rn(0.0, z));
    }
    case LESGPU_BODY_SPHERE: {
        const double dx = __dsub_rn(x, b.cx), dy = __dsub_rn(y, b.cy), dz = __dsub_rn(z, b.cz);
        return __dsub_rn(__dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz))), b.r);
    }
    case LESGPU_BODY_SQUARE: {
        const double ax = fabs(__dsub_rn(x, b.cx)), ay = fabs(__dsub_rn(y, b.cy));
        return __dadd_rn(__dsub_rn(ax >= ay ? ax : ay, b.r), __dmul_rn(0.0, z));
    }
    default:
        return 1.0;
    }
}

#define GLOOP(t, n) for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < (n); t += (long long)gridDim.x * blockDim.x)

// find_inout: 0 inside the body (funcbody <= 1e-10), 1 outside; [k][j][i]
__global__ void k_inout(Body b, const double *xc, const double *yc, const double *zc, int nx1, int ny1, int nz1,
                        unsigned char *out) {
    const long long n = (long long)nx1 * ny1 * nz1;
    GLOOP(t, n) {
        const int i = (int)(t % nx1);
        const long long r = t / nx1;
        const int j = (int)(r % ny1), k = (int)(r / ny1);
        out[t] = fbody(b, xc[i], yc[j], zc[k]) <= 1.0e-10 ? 0 : 1;
    }
}

// findbdy_intp's tests over the interior box, enumerated k, j, i (the
// reference's loop order): flag 1 interpolated, 2 inner, 0 neither
struct Classify {
    const unsigned char *c;
    int nx1, ny1, nz1;             // inout dims
    int ist, jst, kst, ni, nj, nk; // box origin and extents
    const int *ufx, *lfx, *ufy, *lfy, *ufz, *lfz;   // fix flags of cells 1..n-1 (0-based)
};

__global__ void k_classify(Classify C, unsigned char *flag, signed char *dir3) {
    const long long n = (long long)C.ni * C.nj * C.nk;
    GLOOP(t, n) {
        const int ii = (int)(t % C.ni);
        const long long r = t / C.ni;
        const int jj = (int)(r % C.nj), kk = (int)(r / C.nj);
        const int i = C.ist + ii, j = C.jst + jj, k = C.kst + kk;
        auto at = [&](int a, int bq, int cq) { return (int)C.c[((long long)cq * C.ny1 + bq) * C.nx1 + a]; };
        const int ctr = at(i, j, k);
        const int dxi = at(i + 1, j, k) - at(i - 1, j, k);
        const int dyi = at(i, j + 1, k) - at(i, j - 1, k);
        const int dzi = at(i, j, k + 1) - at(i, j, k - 1);
        const int s = abs(dxi) * (1 - C.ufx[i - 1]) * (1 - C.lfx[i - 1]) + abs(dyi) * (1 - C.ufy[j - 1]) * (1 - C.lfy[j - 1])
                      + abs(dzi) * (1 - C.ufz[k - 1]) * (1 - C.lfz[k - 1]);
        flag[t] = ctr == 0 ? (s > 0 ? 1 : 2) : 0;
        dir3[3 * t] = (signed char)dxi; dir3[3 * t + 1] = (signed char)dyi; dir3[3 * t + 2] = (signed char)dzi;
    }
}

// ---- order-preserving compaction of the elements whose flag equals `want`
constexpr int kCT = 256, kCE = 4;                  // threads per block, elements per thread
constexpr int kCB = kCT * kCE;                     // elements per block

__device__ int block_excl_scan(int v, int *sh, int &total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[w] = x;
    __syncthreads();
    if (w == 0) {
        int s = lane < (kCT >> 5) ? sh[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < (kCT >> 5)) sh[lane] = s;
    }
    __syncthreads();
    const int before = w > 0 ? sh[w - 1] : 0;
    total = sh[(kCT >> 5) - 1];
    __syncthreads();
    return before + x - v;
}

__global__ void __launch_bounds__(kCT) k_count(const unsigned char *flag, long long n, int want, int *bcount) {
    __shared__ int sh[32];
    const long long base = (long long)blockIdx.x * kCB + (long long)threadIdx.x * kCE;
    int c = 0;
    for (int e = 0; e < kCE; e++)
        if (base + e < n && flag[base + e] == want) c++;
    int total;
    block_excl_scan(c, sh, total);
    if (threadIdx.x == 0) bcount[blockIdx.x] = total;
}

// exclusive scan of the block counts (one block); total in boff[nb]
__global__ void __launch_bounds__(kCT) k_scan_counts(const int *bcount, int nb, long long *boff) {
    __shared__ int sh[32];
    long long carry = 0;
    for (int b0 = 0; b0 < nb; b0 += kCT) {
        const int v = b0 + (int)threadIdx.x < nb ? bcount[b0 + threadIdx.x] : 0;
        int total;
        const int ex = block_excl_scan(v, sh, total);
        if (b0 + (int)threadIdx.x < nb) boff[b0 + threadIdx.x] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) boff[nb] = carry;
}

__global__ void __launch_bounds__(kCT) k_rank(const unsigned char *flag, long long n, int want, const long long *boff,
                                              long long *rank) {
    __shared__ int sh[32];
    const long long base = (long long)blockIdx.x * kCB + (long long)threadIdx.x * kCE;
    int c = 0;
    for (int e = 0; e < kCE; e++)
        if (base + e < n && flag[base + e] == want) c++;
    int total;
    int r = block_excl_scan(c, sh, total);
    for (int e = 0; e < kCE; e++)
        if (base + e < n) {
            if (flag[base + e] == want) rank[base + e] = boff[blockIdx.x] + r++;
            else rank[base + e] = -1;
        }
}

// forcing-point rows (i, j, k) and, for interpolated points, the directions
__global__ void k_fill_fc(Classify C, const unsigned char *flag, const signed char *dir3, const long long *rank_i,
                          const long long *rank_n, long long nintp, int *fc, int *ix) {
    const long long n = (long long)C.ni * C.nj * C.nk;
    GLOOP(t, n) {
        if (flag[t] == 0) continue;
        const int ii = (int)(t % C.ni);
        const long long r = t / C.ni;
        const int jj = (int)(r % C.nj), kk = (int)(r / C.nj);
        const long long row = flag[t] == 1 ? rank_i[t] : nintp + rank_n[t];
        fc[3 * row] = C.ist + ii; fc[3 * row + 1] = C.jst + jj; fc[3 * row + 2] = C.kst + kk;
        if (flag[t] == 1)
            for (int q = 0; q < 3; q++) ix[3 * row + q] = dir3[3 * t + q];
    }
}

// '%15.8f' then strtod: round v * 1e8 to the nearest integer (ties to even)
// on its exact value, then divide by 1e8 with one rounding
__device__ double round8(double v) {
    const double s = 1.0e8;
    const double p = __dmul_rn(v, s);
    const double e = __fma_rn(v, s, -p);           // v * s = p + e exactly
    double k = rint(p);
    const double d = __dsub_rn(p, k);              // exact
    if (d == 0.5 && e > 0.0) k = __dadd_rn(k, 1.0);
    else if (d == -0.5 && e < 0.0) k = __dsub_rn(k, 1.0);
    return __ddiv_rn(k, s);
}

// geomfac_intp: the surface point on the segment to the fluid neighbour by
// the reference's search (20 sub-segments, three levels), then the 3x3x3
// weights; xpre etc. are geomfac_preset's tables (index + 1; the ghost
// entries stay 0 as the reference's periodic branch is never taken)
__global__ void k_geomfac(Body b, const double *xpre, const double *ypre, const double *zpre, const int *fc,
                          const int *ix, long long nintp, double *gf) {
    GLOOP(n, nintp) {
        const int fi = fc[3 * n], fj = fc[3 * n + 1], fk = fc[3 * n + 2];
        const int di = ix[3 * n], dj = ix[3 * n + 1], dk = ix[3 * n + 2];
        const double x1 = xpre[fi + 1], y1 = ypre[fj + 1], z1 = zpre[fk + 1];
        const double x2 = xpre[fi + di + 1], y2 = ypre[fj + dj + 1], z2 = zpre[fk + dk + 1];
        const double ffs = fbody(b, x1, y1, z1), ffe = fbody(b, x2, y2, z2);
        const bool bad = __dmul_rn(ffs, ffe) > 0.0;
        double x0 = x1, y0 = y1, z0 = z1;
        bool done = bad;
        double t1[3] = {x1, y1, z1}, t2[3] = {x2, y2, z2};
        double xx1[3] = {x1, y1, z1}, xx2[3] = {x2, y2, z2};
        for (int m = 1; m <= 3; m++) {
            if (m > 1)
                for (int q = 0; q < 3; q++) { t1[q] = xx1[q]; t2[q] = xx2[q]; }
            bool found = false;
            for (int s = 0; s < 20; s++) {
                if (done || found) break;
                double a1[3], a2[3];
                for (int q = 0; q < 3; q++) {
                    const double d = __dsub_rn(t2[q], t1[q]);
                    a1[q] = __dadd_rn(t1[q], __ddiv_rn(__dmul_rn(d, (double)s), 20.0));
                    a2[q] = __dadd_rn(t1[q], __ddiv_rn(__dmul_rn(d, (double)(s + 1)), 20.0));
                    xx1[q] = a1[q];
                    xx2[q] = a2[q];
                }
                const double ff1 = fbody(b, a1[0], a1[1], a1[2]), ff2 = fbody(b, a2[0], a2[1], a2[2]);
                if (ff1 == 0.0) { x0 = a1[0]; y0 = a1[1]; z0 = a1[2]; done = true; }
                else if (ff2 == 0.0) { x0 = a2[0]; y0 = a2[1]; z0 = a2[2]; done = true; }
                else if (__dmul_rn(ff1, ff2) < 0.0) {
                    x0 = __dmul_rn(0.5, __dadd_rn(a1[0], a2[0]));
                    y0 = __dmul_rn(0.5, __dadd_rn(a1[1], a2[1]));
                    z0 = __dmul_rn(0.5, __dadd_rn(a1[2], a2[2]));
                    if (m == 3) done = true;
                    else found = true;
                }
            }
        }
        const double x3 = xpre[fi + 2 * di + 1], y3 = ypre[fj + 2 * dj + 1], z3 = zpre[fk + 2 * dk + 1];
        auto wts = [](int ind, double d1, double d2, double d3, double &c0, double &c1) {
            if (ind == 0) { c0 = 1.0; c1 = 1.0; return; }
            if (d2 >= d1) {
                const double den = __dadd_rn(d1, d2);
                c0 = __ddiv_rn(d2, den == 0.0 ? 1.0 : den);
                c1 = 1.0;
            } else {
                const double den = __dsub_rn(d3, d2);
                c0 = 0.5;
                c1 = __ddiv_rn(__dsub_rn(d3, d1), den == 0.0 ? 1.0 : den);
            }
        };
        double a0, a1w, b0, b1w, c0, c1w;
        wts(di, fabs(__dsub_rn(x1, x0)), fabs(__dsub_rn(x2, x0)), fabs(__dsub_rn(x3, x0)), a0, a1w);
        wts(dj, fabs(__dsub_rn(y1, y0)), fabs(__dsub_rn(y2, y0)), fabs(__dsub_rn(y3, y0)), b0, b1w);
        wts(dk, fabs(__dsub_rn(z1, z0)), fabs(__dsub_rn(z2, z0)), fabs(__dsub_rn(z3, z0)), c0, c1w);
        const double inv = __ddiv_rn(1.0, __dmul_rn(__dmul_rn(a0, b0), c0));
        const double F[3][3] = {{a0, __dsub_rn(1.0, a0), __dsub_rn(1.0, a0)},
                                {b0, __dsub_rn(1.0, b0), __dsub_rn(1.0, b0)},
                                {c0, __dsub_rn(1.0, c0), __dsub_rn(1.0, c0)}};
        const double G[3][3] = {{0.0, a1w, __dsub_rn(1.0, a1w)}, {0.0, b1w, __dsub_rn(1.0, b1w)}, {0.0, c1w, __dsub_rn(1.0, c1w)}};
        double *out = gf + 27 * n;
        for (int p = 0; p < 3; p++)
            for (int q = 0; q < 3; q++)
                for (int r = 0; r < 3; r++) {
                    double v = __dmul_rn(__dmul_rn(__dmul_rn(-inv, F[0][p]), F[1][q]), F[2][r]);
                    if (p > 0) v = __dmul_rn(v, G[0][p]);
                    if (q > 0) v = __dmul_rn(v, G[1][q]);
                    if (r > 0) v = __dmul_rn(v, G[2][r]);
                    if (bad) v = 0.0;
                    out[9 * p + 3 * q + r] = round8(v);
                }
        out[0] = round8(bad ? 1.0 : inv);
    }
}

// find_zero_nu_sgs: iszero of the cells (0 where the cell or one of its six
// neighbours is solid), [k][j][i]; flag 1 where zero, enumerated i, j, k
__global__ void k_zero_nu(Body b, const double *xm, const double *ym, const double *zm, int nx1, int ny1, int nz1,
                          int *isz, unsigned char *flag_ijk) {
    const int ni = nx1 - 2, nj = ny1 - 2, nk = nz1 - 2;
    const long long n = (long long)ni * nj * nk;
    GLOOP(t, n) {
        const int ii = (int)(t % ni);
        const long long r = t / ni;
        const int jj = (int)(r % nj), kk = (int)(r / nj);
        const int i = ii + 1, j = jj + 1, k = kk + 1;
        auto sol = [&](int a, int bq, int cq) { return fbody(b, xm[a], ym[bq], zm[cq]) <= 1.0e-10; };
        const bool z = sol(i, j, k) || sol(i - 1, j, k) || sol(i + 1, j, k) || sol(i, j - 1, k) || sol(i, j + 1, k)
                       || sol(i, j, k - 1) || sol(i, j, k + 1);
        isz[t] = z ? 0 : 1;
        flag_ijk[((long long)ii * nj + jj) * nk + kk] = z ? 1 : 0;
    }
}

// ---- conjg_intp (ibm_body.f90:402-550) and fluid_portion (:553-667) ------
// fluid_portion flood-fills a 6x6x6 sub-cell grid from sub-cell (1,1,1)
// through 6-connected sub-cells of its phase; the sub-cells it never reaches
// take the opposite phase.  The result is therefore the start sub-cell's
// same-phase component, whatever the order of the fill: here the phases are
// one 36-bit word per z layer (bit i + 6 j) and the component grows by bit
// dilation (x: shift by 1 within a row, y: by 6, z: the neighbouring words)
// until it stops changing.
__device__ double fluid_portion(const Body &b, double x1, double x2, double y1, double y2, double z1, double z2) {
    const double tx = __ddiv_rn(__dsub_rn(x2, x1), 6.0), ty = __ddiv_rn(__dsub_rn(y2, y1), 6.0),
                 tz = __ddiv_rn(__dsub_rn(z2, z1), 6.0);
    const unsigned long long full = (1ULL << 36) - 1ULL;
    const unsigned long long notI0 = full & ~0x041041041ULL, notI5 = full & ~0x820820820ULL;
    unsigned long long sol[6];
    for (int k = 0; k < 6; k++) {
        const double zc = __dadd_rn(z1, __dmul_rn(tz, (double)k + 0.5));   // dble(2 kk - 1) / 2
        unsigned long long w = 0ULL;
        for (int j = 0; j < 6; j++) {
            const double yc = __dadd_rn(y1, __dmul_rn(ty, (double)j + 0.5));
            for (int i = 0; i < 6; i++) {
                const double xc = __dadd_rn(x1, __dmul_rn(tx, (double)i + 0.5));
                if (fbody(b, xc, yc, zc) <= 1.0e-10) w |= 1ULL << (i + 6 * j);
            }
        }
        sol[k] = w;
    }
    const bool s0 = (sol[0] & 1ULL) != 0ULL;
    unsigned long long same[6], r[6];
    for (int k = 0; k < 6; k++) { same[k] = s0 ? sol[k] : (~sol[k] & full); r[k] = 0ULL; }
    r[0] = 1ULL;
    for (int it = 0; it < 216; it++) {          // the component gains a sub-cell per pass or stops
        unsigned long long nr[6];
        bool changed = false;
        for (int k = 0; k < 6; k++) {
            unsigned long long gw = r[k] | ((r[k] << 1) & notI0) | ((r[k] >> 1) & notI5) | ((r[k] << 6) & full) | (r[k] >> 6);
            if (k > 0) gw |= r[k - 1];
            if (k < 5) gw |= r[k + 1];
            nr[k] = gw & same[k];
            changed |= nr[k] != r[k];
        }
        for (int k = 0; k < 6; k++) r[k] = nr[k];
        if (!changed) break;
    }
    int comp = 0;
    for (int k = 0; k < 6; k++) comp += __popcll(r[k]);
    const int nsolid = s0 ? comp : 216 - comp;
    return __dsub_rn(1.0, __ddiv_rn((double)nsolid, 216.0));
}

struct ConjgArgs {
    Body b;
    const double *x, *xm, *y, *ym, *z, *zm;   // 0..n? (the pre-processor's vectors)
    int nx, ny, nz, xpr, ypr, zpr;
    double cratio, kratio;
    double *cstar, *kstar;                     // cells i fastest; kstar: 6 faces of ncell
    long long *omega;
};

// one thread per (cell, box): box 0 is the cell (c*, omega), boxes 1..6 the
// east, west, north, south, top and bottom faces (k*)
__global__ void k_conjg(ConjgArgs A) {
    const int mx = A.nx - 1, my = A.ny - 1, mz = A.nz - 1;
    const long long ncell = (long long)mx * my * mz;
    GLOOP(t, 7 * ncell) {
        const int f = (int)(t % 7);
        const long long c = t / 7;
        const int i = 1 + (int)(c % mx), j = 1 + (int)((c / mx) % my), k = 1 + (int)(c / ((long long)mx * my));
        double x1 = A.x[i], x2 = A.x[i + 1], y1 = A.y[j], y2 = A.y[j + 1], z1 = A.z[k], z2 = A.z[k + 1];
        double nxc = A.xm[i], nyc = A.ym[j], nzc = A.zm[k];       // neighbour centre of the face
        const double lx = __dsub_rn(A.x[A.nx], A.x[1]), ly = __dsub_rn(A.y[A.ny], A.y[1]), lz = __dsub_rn(A.z[A.nz], A.z[1]);
        switch (f) {
        case 1: nxc = (A.xpr == 1 && i == A.nx - 1) ? __dadd_rn(A.xm[1], lx) : A.xm[i + 1]; x1 = A.xm[i]; x2 = nxc; break;
        case 2: nxc = (A.xpr == 1 && i == 1) ? __dsub_rn(A.xm[A.nx - 1], lx) : A.xm[i - 1]; x1 = nxc; x2 = A.xm[i]; break;
        case 3: nyc = (A.ypr == 1 && j == A.ny - 1) ? __dadd_rn(A.ym[1], ly) : A.ym[j + 1]; y1 = A.ym[j]; y2 = nyc; break;
        case 4: nyc = (A.ypr == 1 && j == 1) ? __dsub_rn(A.ym[A.ny - 1], ly) : A.ym[j - 1]; y1 = nyc; y2 = A.ym[j]; break;
        case 5: nzc = (A.zpr == 1 && k == A.nz - 1) ? __dadd_rn(A.zm[1], lz) : A.zm[k + 1]; z1 = A.zm[k]; z2 = nzc; break;
        case 6: nzc = (A.zpr == 1 && k == 1) ? __dsub_rn(A.zm[A.nz - 1], lz) : A.zm[k - 1]; z1 = nzc; z2 = A.zm[k]; break;
        default: break;
        }
        const double fp = fluid_portion(A.b, x1, x2, y1, y2, z1, z2);
        const double mix = __dadd_rn(__dmul_rn(__dsub_rn(1.0, fp), f == 0 ? A.cratio : A.kratio), __dmul_rn(fp, 1.0));
        if (f == 0) {
            A.cstar[c] = mix;
            A.omega[c] = fp >= (1.0 - 1.0e-12) ? 1 : 0;
        } else {
            const double aa = fbody(A.b, A.xm[i], A.ym[j], A.zm[k]);
            const bool same = __dmul_rn(aa, fbody(A.b, nxc, nyc, nzc)) >= 0.0;
            A.kstar[(long long)(f - 1) * ncell + c] =
                same ? mix : __ddiv_rn(A.kratio, __dadd_rn(__dmul_rn(A.kratio, fp), __dmul_rn(1.0, __dsub_rn(1.0, fp))));
        }
    }
}

struct DevBuf {
    std::vector<void *> p;
    bool ok = true;
    template <class T> T *get(size_t n) {
        void *q = nullptr;
        if (cudaMalloc(&q, (n ? n : 1) * sizeof(T)) != cudaSuccess) { ok = false; return nullptr; }
        cudaMemset(q, 0, (n ? n : 1) * sizeof(T));
        p.push_back(q);
        return (T *)q;
    }
    template <class T> T *up(const T *h, size_t n) {
        T *d = get<T>(n);
        if (d && n) cudaMemcpy(d, h, n * sizeof(T), cudaMemcpyHostToDevice);
        return d;
    }
    ~DevBuf() { for (void *q : p) cudaFree(q); }
};

// ranks of the elements flagged `want` (-1 elsewhere); returns their number
static long long compact(DevBuf &B, const unsigned char *flag, long long n, int want, long long *rank) {
    const int nb = (int)((n + kCB - 1) / kCB);
    int *bcount = B.get<int>(nb);
    long long *boff = B.get<long long>(nb + 1);
    if (!B.ok || n == 0) return 0;
    k_count<<<nb, kCT>>>(flag, n, want, bcount);
    k_scan_counts<<<1, kCT>>>(bcount, nb, boff);
    k_rank<<<nb, kCT>>>(flag, n, want, boff, rank);
    long long total = 0;
    cudaMemcpy(&total, boff + nb, sizeof(long long), cudaMemcpyDeviceToHost);
    return total;
}

}  // namespace ibp
}  // namespace lg

using namespace lg;
using namespace lg::ibp;

extern "C" int lesgpu_ibmpre_run(const lesgpu_config *cfg, const lesgpu_grid *g, const double *const axes[6],
                                 lesgpu_ibmpre **out) {
    if (!cfg || !g || !axes || !out) return LESGPU_ERR_ARG;
    *out = nullptr;
    for (int a = 0; a < 6; a++)
        if (!axes[a]) return LESGPU_ERR_ARG;
    if (g->n1 != g->n1m + 1 || g->n2 != g->n2m + 1 || g->n3 != g->n3m + 1 || g->n1m < 2 || g->n2m < 2 || g->n3m < 1)
        return LESGPU_ERR_ARG;
    const int n[3] = {(int)g->n1, (int)g->n2, (int)g->n3};
    const int nm[3] = {(int)g->n1m, (int)g->n2m, (int)g->n3m};
    DevBuf B;
    const double *dc[3], *dm[3];
    for (int a = 0; a < 3; a++) {
        dc[a] = B.up(axes[2 * a], (size_t)n[a] + 1);
        dm[a] = B.up(axes[2 * a + 1], (size_t)n[a] + 1);
    }
    // geomfac_preset tables, index + 1: coordinate / centre columns, ghosts 0
    const double *pre_c[3], *pre_m[3];
    for (int a = 0; a < 3; a++) {
        std::vector<double> hc((size_t)n[a] + 3, 0.0), hm((size_t)n[a] + 3, 0.0);
        for (int q = 0; q <= n[a]; q++) { hc[q + 1] = axes[2 * a][q]; hm[q + 1] = axes[2 * a + 1][q]; }
        pre_c[a] = B.up(hc.data(), hc.size());
        pre_m[a] = B.up(hm.data(), hm.size());
    }
    const int64_t *fixu[3] = {g->fixiu, g->fixju, g->fixku}, *fixl[3] = {g->fixil, g->fixjl, g->fixkl};
    const int *du[3], *dl[3];
    for (int a = 0; a < 3; a++) {
        std::vector<int> hu(nm[a]), hl(nm[a]);
        for (int q = 0; q < nm[a]; q++) { hu[q] = (int)fixu[a][q]; hl[q] = (int)fixl[a][q]; }
        du[a] = B.up(hu.data(), hu.size());
        dl[a] = B.up(hl.data(), hl.size());
    }
    if (!B.ok) return LESGPU_ERR_OOM;
    Body body{(int)cfg->body.kind, cfg->body.cx, cfg->body.cy, cfg->body.cz, cfg->body.r, cfg->body.p0};
    lesgpu_ibmpre *h = new lesgpu_ibmpre();
    h->nl = cfg->ihtrans == 1 ? 4 : 3;
    for (int l = 0; l < 4; l++) { h->nintp[l] = 0; h->nbody[l] = 0; }
    const int nx1 = n[0] + 1, ny1 = n[1] + 1, nz1 = n[2] + 1;
    const long long nfull = (long long)nx1 * ny1 * nz1;
    unsigned char *inout = B.get<unsigned char>((size_t)nfull);
    // variable d = 1..4 sits at (x, ym, zm), (xm, y, zm), (xm, ym, z), (xm, ym, zm)
    for (int l = 0; l < h->nl; l++) {
        const double *lx = l == 0 ? dc[0] : dm[0], *ly = l == 1 ? dc[1] : dm[1], *lz = l == 2 ? dc[2] : dm[2];
        const double *px = l == 0 ? pre_c[0] : pre_m[0], *py = l == 1 ? pre_c[1] : pre_m[1];
        const double *pz = l == 2 ? pre_c[2] : pre_m[2];
        k_inout<<<blocks_for(nfull), kThreads>>>(body, lx, ly, lz, nx1, ny1, nz1, inout);
        Classify C{inout, nx1, ny1, nz1, l == 0 ? 2 : 1, l == 1 ? 2 : 1, l == 2 ? 2 : 1, 0, 0, 0,
                   du[0], dl[0], du[1], dl[1], du[2], dl[2]};
        C.ni = n[0] - C.ist; C.nj = n[1] - C.jst; C.nk = n[2] - C.kst;
        const long long nbox = (long long)(C.ni > 0 ? C.ni : 0) * (C.nj > 0 ? C.nj : 0) * (C.nk > 0 ? C.nk : 0);
        unsigned char *flag = B.get<unsigned char>((size_t)nbox);
        signed char *dir3 = B.get<signed char>((size_t)nbox * 3);
        long long *ri = B.get<long long>((size_t)nbox), *rn = B.get<long long>((size_t)nbox);
        if (!B.ok) { delete h; return LESGPU_ERR_OOM; }
        if (nbox > 0) k_classify<<<blocks_for(nbox), kThreads>>>(C, flag, dir3);
        const long long ni = compact(B, flag, nbox, 1, ri), nn = compact(B, flag, nbox, 2, rn);
        const long long nb = ni + nn;
        int *fc = B.get<int>((size_t)nb * 3), *ix = B.get<int>((size_t)(ni > 0 ? ni : 1) * 3);
        double *gf = B.get<double>((size_t)(ni > 0 ? ni : 1) * 27);
        if (!B.ok) { delete h; return LESGPU_ERR_OOM; }
        if (nbox > 0) k_fill_fc<<<blocks_for(nbox), kThreads>>>(C, flag, dir3, ri, rn, ni, fc, ix);
        if (ni > 0) k_geomfac<<<blocks_for(ni, 128), 128>>>(body, px, py, pz, fc, ix, ni, gf);
        std::vector<int> hfc((size_t)nb * 3), hix((size_t)ni * 3);
        h->gf[l].resize((size_t)ni * 27);
        if (nb) cudaMemcpy(hfc.data(), fc, hfc.size() * sizeof(int), cudaMemcpyDeviceToHost);
        if (ni) {
            cudaMemcpy(hix.data(), ix, hix.size() * sizeof(int), cudaMemcpyDeviceToHost);
            cudaMemcpy(h->gf[l].data(), gf, h->gf[l].size() * sizeof(double), cudaMemcpyDeviceToHost);
        }
        h->nintp[l] = ni;
        h->nbody[l] = nb;
        h->fc[l].assign(hfc.begin(), hfc.end());
        h->ix[l].assign(hix.begin(), hix.end());
    }
    // zero-viscosity cells and the wall mask
    const long long ncell = (long long)nm[0] * nm[1] * nm[2];
    int *isz = B.get<int>((size_t)ncell);
    unsigned char *fz = B.get<unsigned char>((size_t)ncell);
    long long *rz = B.get<long long>((size_t)ncell);
    if (!B.ok) { delete h; return LESGPU_ERR_OOM; }
    k_zero_nu<<<blocks_for(ncell), kThreads>>>(body, dm[0], dm[1], dm[2], nx1, ny1, nz1, isz, fz);
    const long long nz = compact(B, fz, ncell, 1, rz);
    std::vector<int> hisz((size_t)ncell);
    std::vector<long long> hrz((size_t)ncell);
    cudaMemcpy(hisz.data(), isz, hisz.size() * sizeof(int), cudaMemcpyDeviceToHost);
    cudaMemcpy(hrz.data(), rz, hrz.size() * sizeof(long long), cudaMemcpyDeviceToHost);
    if (cudaDeviceSynchronize() != cudaSuccess) { delete h; return LESGPU_ERR_CUDA; }
    h->nwall.assign(hisz.begin(), hisz.end());
    h->nzero = nz;
    h->inz.assign((size_t)nz, 0); h->jnz.assign((size_t)nz, 0); h->knz.assign((size_t)nz, 0);
    const long long nj = nm[1], nk = nm[2];
    for (long long t = 0; t < ncell; t++)        // t enumerates (i, j, k), k fastest
        if (hrz[t] >= 0) {
            const long long r = hrz[t];
            h->inz[r] = t / (nj * nk); h->jnz[r] = (t / nk) % nj; h->knz[r] = t % nk;
        }
    *out = h;
    return 0;
}

extern "C" int lesgpu_ibmpre_tables(lesgpu_ibmpre *h, lesgpu_ibm *t) {
    if (!h || !t) return LESGPU_ERR_ARG;
    memset(t, 0, sizeof(*t));
    for (int l = 0; l < 4; l++) {
        t->nintp[l] = h->nintp[l];
        t->nbody[l] = h->nbody[l];
        t->fc[l] = h->fc[l].empty() ? nullptr : h->fc[l].data();
        t->intpindx[l] = h->ix[l].empty() ? nullptr : h->ix[l].data();
        t->geomfac[l] = h->gf[l].empty() ? nullptr : h->gf[l].data();
    }
    t->nzero = h->nzero;
    t->inz = h->inz.empty() ? nullptr : h->inz.data();
    t->jnz = h->jnz.empty() ? nullptr : h->jnz.data();
    t->knz = h->knz.empty() ? nullptr : h->knz.data();
    t->nwall_dvm = h->nwall.data();
    return 0;
}

extern "C" int lesgpu_ibmpre_free(lesgpu_ibmpre *h) {
    delete h;
    return 0;
}

extern "C" int lesgpu_conjg_run(const lesgpu_config *cfg, const lesgpu_grid *g, const double *const axes[6],
                                double cratio, double kratio, double *cstar, double *kstar, int64_t *omega) {
    if (!cfg || !g || !axes || !cstar || !kstar || !omega) return LESGPU_ERR_ARG;
    for (int a = 0; a < 6; a++)
        if (!axes[a]) return LESGPU_ERR_ARG;
    if (g->n1 != g->n1m + 1 || g->n2 != g->n2m + 1 || g->n3 != g->n3m + 1 || g->n1m < 1 || g->n2m < 1 || g->n3m < 1)
        return LESGPU_ERR_ARG;
    const int n[3] = {(int)g->n1, (int)g->n2, (int)g->n3};
    const long long ncell = (long long)g->n1m * g->n2m * g->n3m;
    DevBuf B;
    ConjgArgs A;
    const double *d[6];
    for (int a = 0; a < 6; a++) d[a] = B.up(axes[a], (size_t)n[a / 2] + 1);
    A.x = d[0]; A.xm = d[1]; A.y = d[2]; A.ym = d[3]; A.z = d[4]; A.zm = d[5];
    A.b = Body{(int)cfg->body.kind, cfg->body.cx, cfg->body.cy, cfg->body.cz, cfg->body.r, cfg->body.p0};
    A.nx = n[0]; A.ny = n[1]; A.nz = n[2];
    A.xpr = (int)cfg->xprdic; A.ypr = (int)cfg->yprdic; A.zpr = (int)cfg->zprdic;
    A.cratio = cratio; A.kratio = kratio;
    A.cstar = B.get<double>((size_t)ncell);
    A.kstar = B.get<double>((size_t)6 * ncell);
    A.omega = B.get<long long>((size_t)ncell);
    if (!B.ok) return LESGPU_ERR_OOM;
    k_conjg<<<blocks_for(7 * ncell, 128), 128>>>(A);
    if (cudaMemcpy(cstar, A.cstar, sizeof(double) * (size_t)ncell, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(kstar, A.kstar, sizeof(double) * 6 * (size_t)ncell, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(omega, A.omega, sizeof(int64_t) * (size_t)ncell, cudaMemcpyDeviceToHost) != cudaSuccess)
        return LESGPU_ERR_CUDA;
    return 0;
}

