// Approximately factorised Crank-Nicolson solves: lhsu/lhsv/lhsw
// (slv_mmtm.f90:1044-1362) and lhs_t (slv_engy.f90:460-609), with the
// tridiagonal algorithms trdiag1/2/3 (:1365-1498) and the periodic two-sweep
// variant trdiag1p/3p (:1501-1641).
//
// Each thread solves one line.  The coefficients a, b, c of an element are
// rebuilt from the metric vectors and the eddy viscosities when the forward
// sweep reaches it, so no coefficient plane is ever stored; the forward
// sweep keeps the elimination factors in a scratch array that the backward
// sweep reads once.  z- and y-lines are laid out so that the 32 threads of a
// warp hold 32 consecutive i: every load and store of a step is one
// coalesced 256-byte row.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>

#include "lesgpu_internal.cuh"

namespace lg {

// coefficient sets: component (u, v, w, T) x direction (x, y, z)
enum { CU = 0, CV = 1, CW = 2, CT = 3 };

struct AdiArgs {
    int comp, dir;          // component and sweep direction (0 x, 1 y, 2 z)
    int l1, l2;             // line index range
    int a0, a1, b0, b1;     // ranges of the two batch indices (see line_coords)
    const double *src;      // right-hand side source (scaled by diag)
    double *dst;            // solution destination (or the field to add to)
    int add;                // 1: dst += solution
    double *gam;            // scratch (forward factors)
    double *sarr;           // scratch (periodic second vector)
    int periodic;
};

__device__ __forceinline__ void line_coords(int dir, int l, int x0, int x1, int &i, int &j, int &k) {
    if (dir == 2) { i = x0; j = x1; k = l; }        // z-lines: batch (i, j)
    else if (dir == 1) { i = x0; k = x1; j = l; }   // y-lines: batch (i, k)
    else { j = x0; k = x1; i = l; }                 // x-lines: batch (j, k)
}

// a and c of the element (i,j,k); b = diag - a - c.  R is the arithmetic
// type (double; float for the x and z sweeps of the mixed-precision form).
template <class R>
__device__ __forceinline__ void adi_coef(const KP &p, int comp, int dir, int i, int j, int k, R &a, R &c) {
    const Mir<R> &M = mir<R>(p);
    const DGrid &g = p.g;
    const DFields &f = p.f;
    long long q = g.ix(i, j, k);
    if (comp == CT) {
        const R cre = pickr<R>(p.c.adi_cd[2], p.c.adi_cf[2]);   // iles re pr
        R cs = R(1.0), ks1 = R(1.0), ks2 = R(1.0), omc = R(1.0);
        int ka = dir == 2 ? 5 : dir == 1 ? 3 : 1;
        if (p.c.conj_tables) {        // unit tables: the same expression with the values 1
            cs = R(M.cstar[q]);
            ks1 = R(M.kstar[ka][q]);
            ks2 = R(M.kstar[ka - 1][q]);
            omc = p.c.imovingon == 0 ? R(f.omega[q]) : R(1.0);
        }
        if (dir == 2) {
            a = R(M.akuv[k]) * (cs * ks1 + cre * omc * R(M.alsgs1[1][q]));
            c = R(M.ckuv[k]) * (cs * ks2 + cre * omc * R(M.alsgs1[1][q + g.sxy]));
        } else if (dir == 1) {
            a = R(M.ajuw[j]) * (cs * ks1 + cre * omc * R(M.alsgs1[2][q]));
            c = R(M.cjuw[j]) * (cs * ks2 + cre * omc * R(M.alsgs1[2][q + g.sx]));
        } else {
            a = R(M.aivw[i]) * (cs * ks1 + cre * omc * R(M.alsgs1[0][q]));
            c = R(M.civw[i]) * (cs * ks2 + cre * omc * R(M.alsgs1[0][q + 1]));
        }
        return;
    }
    const R cre = pickr<R>(p.c.adi_cd[0], p.c.adi_cf[0]), cre2 = pickr<R>(p.c.adi_cd[1], p.c.adi_cf[1]);
    const R *nu = M.nusgs, *nu1 = M.nusgs1[0], *nu2 = M.nusgs1[1], *nu3 = M.nusgs1[2];
    switch (comp * 3 + dir) {
    case CU * 3 + 2: a = R(M.akuv[k]) * (R(1.0) + cre * R(nu2[q])); c = R(M.ckuv[k]) * (R(1.0) + cre * R(nu2[q + g.sxy])); break;
    case CU * 3 + 1: a = R(M.ajuw[j]) * (R(1.0) + cre * R(nu3[q])); c = R(M.cjuw[j]) * (R(1.0) + cre * R(nu3[q + g.sx])); break;
    case CU * 3 + 0: a = R(M.aiu[i]) * (R(1.0) + cre2 * R(nu[q - 1])); c = R(M.ciu[i]) * (R(1.0) + cre2 * R(nu[q])); break;
    case CV * 3 + 2: a = R(M.akuv[k]) * (R(1.0) + cre * R(nu1[q])); c = R(M.ckuv[k]) * (R(1.0) + cre * R(nu1[q + g.sxy])); break;
    case CV * 3 + 1: a = R(M.ajv[j]) * (R(1.0) + cre2 * R(nu[q - g.sx])); c = R(M.cjv[j]) * (R(1.0) + cre2 * R(nu[q])); break;
    case CV * 3 + 0: a = R(M.aivw[i]) * (R(1.0) + cre * R(nu3[q])); c = R(M.civw[i]) * (R(1.0) + cre * R(nu3[q + 1])); break;
    case CW * 3 + 2: a = R(M.akw[k]) * (R(1.0) + cre2 * R(nu[q - g.sxy])); c = R(M.ckw[k]) * (R(1.0) + cre2 * R(nu[q])); break;
    case CW * 3 + 1: a = R(M.ajuw[j]) * (R(1.0) + cre * R(nu1[q])); c = R(M.cjuw[j]) * (R(1.0) + cre * R(nu1[q + g.sx])); break;
    default:         a = R(M.aivw[i]) * (R(1.0) + cre * R(nu2[q])); c = R(M.civw[i]) * (R(1.0) + cre * R(nu2[q + 1])); break;
    }
}

// The same coefficients in factored form, a = ma[l] (1 + cre nv[q + oa]) and
// c = mc[l] (1 + cre nv[q + oa + s]) at line index l and line stride s.  The
// c factor of element l is the a factor of element l + 1 (the same viscosity
// value), so a serial sweep carries it over and reads and forms each factor
// once.  This holds for every velocity coefficient and for the temperature
// one without conjugate tables; with them, c* and k* differ between the two
// sides of a face and adi_coef is used.
template <class R>
struct AdiFacs {
    const R *ma, *mc, *nv;
    R cre;
    long long oa;
};

template <class R>
__device__ __forceinline__ AdiFacs<R> adi_facs(const KP &p, int comp, int dir) {
    const Mir<R> &M = mir<R>(p);
    const R cre = pickr<R>(p.c.adi_cd[0], p.c.adi_cf[0]), cre2 = pickr<R>(p.c.adi_cd[1], p.c.adi_cf[1]);
    const long long s = dir == 2 ? p.g.sxy : dir == 1 ? p.g.sx : 1;
    switch (comp * 3 + dir) {
    case CU * 3 + 2: return {M.akuv, M.ckuv, M.nusgs1[1], cre, 0};
    case CU * 3 + 1: return {M.ajuw, M.cjuw, M.nusgs1[2], cre, 0};
    case CU * 3 + 0: return {M.aiu, M.ciu, M.nusgs, cre2, -1};
    case CV * 3 + 2: return {M.akuv, M.ckuv, M.nusgs1[0], cre, 0};
    case CV * 3 + 1: return {M.ajv, M.cjv, M.nusgs, cre2, -s};
    case CV * 3 + 0: return {M.aivw, M.civw, M.nusgs1[2], cre, 0};
    case CW * 3 + 2: return {M.akw, M.ckw, M.nusgs, cre2, -s};
    case CW * 3 + 1: return {M.ajuw, M.cjuw, M.nusgs1[0], cre, 0};
    case CW * 3 + 0: return {M.aivw, M.civw, M.nusgs1[1], cre, 0};
    default: {
        const R c3 = pickr<R>(p.c.adi_cd[2], p.c.adi_cf[2]);
        if (dir == 2) return {M.akuv, M.ckuv, M.alsgs1[1], c3, 0};
        if (dir == 1) return {M.ajuw, M.cjuw, M.alsgs1[2], c3, 0};
        return {M.aivw, M.civw, M.alsgs1[0], c3, 0};
    }
    }
}

// a and c of the elements c0 .. c0 + CHN - 1 (below nline) of the line that
// starts at q0 with line index l1; factored when shared, fprev carrying the c
// factor from element to element.
template <class R, int CHN>
__device__ __forceinline__ void adi_chunk_coefs(const KP &p, int comp, int dir, const AdiFacs<R> &F, bool shared,
                                                int l1, int c0, int nline, int x0, int x1, long long q0,
                                                long long stride, R &fprev, R (&av)[CHN], R (&cv)[CHN]) {
#pragma unroll
    for (int u = 0; u < CHN; u++) {
        if (c0 + u < nline) {
            const int l = l1 + c0 + u;
            if (shared) {
                const R fc = R(1.0) + F.cre * R(F.nv[q0 + (long long)(c0 + u) * stride + F.oa + stride]);
                av[u] = R(F.ma[l]) * fprev;
                cv[u] = R(F.mc[l]) * fc;
                fprev = fc;
            } else {
                int i, j, k;
                line_coords(dir, l, x0, x1, i, j, k);
                adi_coef(p, comp, dir, i, j, k, av[u], cv[u]);
            }
        }
    }
}

// Reciprocal of a pivot.  FP32: the division.  FP64: Newton-Raphson
// iteration for 1/d, r <- r + r (1 - d r), from an FP32 reciprocal seed; each
// step squares the relative error (2^-22 -> 2^-44 -> below the final
// rounding), so the result is within 2 ulp of the quotient.  The seed's
// FP64 <-> FP32 moves are done on the bit patterns with integer operations
// (exponent rebias, mantissa truncated to 23 bits), not by conversions, which
// on GB300 issue on the narrow FP64 pipe: the reciprocal then costs that pipe
// four FMAs where a correctly rounded division takes more.  Pivots whose
// binary exponent lies outside [-99, 99], where the FP32 seed or its
// reciprocal would leave the normal FP32 range, take the division.
template <class R>
__device__ __forceinline__ R rcp_pivot(R d) {
    if (sizeof(R) == 4) return R(1.0) / d;
    const unsigned long long bits = (unsigned long long)__double_as_longlong((double)d);
    const unsigned hi = (unsigned)(bits >> 32);
    const int ed = (int)((hi >> 20) & 0x7ffu);                // biased FP64 exponent
    if ((unsigned)(ed - (1023 - 99)) > 198u) return R(1.0) / d;
    const unsigned fs = (hi & 0x80000000u) | ((unsigned)(ed - 1023 + 127) << 23) | ((unsigned)(bits >> 29) & 0x7fffffu);
    const unsigned rs = __float_as_uint(__frcp_rn(__uint_as_float(fs)));
    const unsigned long long rb = ((unsigned long long)(rs & 0x80000000u) << 32)
                                | ((unsigned long long)(((rs >> 23) & 0xffu) - 127u + 1023u) << 52)
                                | ((unsigned long long)(rs & 0x7fffffu) << 29);
    double r = __longlong_as_double((long long)rb);
    double e = fma(-(double)d, r, 1.0);
    r = fma(r, e, r);
    e = fma(-(double)d, r, 1.0);
    r = fma(r, e, r);
    return R(r);
}

// Elements per chunk: a thread issues the loads of CH consecutive line
// elements before it runs the (serial) recurrence over them, so CH loads are
// in flight instead of one.  Stores of a chunk follow all its loads, which
// keeps in-place sweeps (src == dst) correct.  The kernel is instantiated per
// direction and periodicity, and its registers are capped so that 32 warps
// fit on an SM: at large grids (lines >> threads) the serial sweep is
// bound by memory latency and FP64 issue, both of which want occupancy.
constexpr int CH = 4;

struct AdiBatch {
    AdiArgs a[3];
};

template <class R, int DIR, bool PER, bool FAC>
__global__ void __launch_bounds__(128, 6) k_adi(KP p, AdiBatch B) {
    const AdiArgs &A = B.a[blockIdx.y];
    const DGrid &g = p.g;
    const R diag = (A.comp == CT) ? p.S->acoefi * p.c.pr : p.S->acoefi;
    int na = A.a1 - A.a0 + 1, nb = A.b1 - A.b0 + 1;
    long long nl = (long long)na * nb;
    const long long stride = DIR == 2 ? g.sxy : DIR == 1 ? g.sx : 1;
    const int nline = A.l2 - A.l1 + 1;
    if (nl <= 0 || A.l2 < A.l1) return;
    // Forward-pass scratch in the arithmetic type: in FP32 the factors and
    // provisional values never pass through FP64 (on GB300 a conversion issues
    // on the narrow FP64 pipe) and move half the bytes.  An FP32 sweep keeps
    // its three periodic vectors in the two scratch arrays (the gam array of
    // nt doubles holds two float vectors).
    constexpr bool F32 = sizeof(R) == 4;
    R *const sg = reinterpret_cast<R *>(A.gam);
    R *const ss = reinterpret_cast<R *>(A.sarr);
    R *const sf = F32 ? reinterpret_cast<R *>(A.gam) + g.nt : nullptr;
    constexpr bool shared = FAC;
    const AdiFacs<R> F = FAC ? adi_facs<R>(p, A.comp, DIR) : AdiFacs<R>{};
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < nl; t += (long long)gridDim.x * blockDim.x) {
        const int x0 = A.a0 + (int)(t % na), x1 = A.b0 + (int)(t / na);
        int i0, j0, k0;
        line_coords(DIR, A.l1, x0, x1, i0, j0, k0);
        const long long q0 = g.ix(i0, j0, k0);
        if (!PER) {
            // ---- trdiag: forward elimination, chunk by chunk; the provisional
            // solution goes to the scratch (FP32, or when adding) or to dst
            R *xs = (F32 || A.add) ? ss : reinterpret_cast<R *>(A.dst);
            R bet = R(0.0), x = R(0.0), cprev = R(0.0);
            R fprev = shared ? R(1.0) + F.cre * R(F.nv[q0 + F.oa]) : R(0.0);
            for (int c0 = 0; c0 < nline; c0 += CH) {
                R av[CH], cv[CH], rv[CH];
                adi_chunk_coefs<R, CH>(p, A.comp, DIR, F, shared, A.l1, c0, nline, x0, x1, q0, stride, fprev, av, cv);
#pragma unroll
                for (int u = 0; u < CH; u++)
                    if (c0 + u < nline) rv[u] = R(A.src[q0 + (long long)(c0 + u) * stride]);
#pragma unroll
                for (int u = 0; u < CH; u++) {
                    if (c0 + u < nline) {
                        const long long q = q0 + (long long)(c0 + u) * stride;
                        const R a = av[u], c = cv[u];
                        const R b = diag - a - c;
                        if (c0 + u == 0) {
                            bet = rcp_pivot(b);
                            x = diag * rv[u] * bet;
                        } else {
                            const R gm = cprev * bet;
                            bet = rcp_pivot(b - a * gm);
                            x = (diag * rv[u] - a * x) * bet;
                            sg[q] = gm;
                        }
                        xs[q] = x;
                        cprev = c;
                    }
                }
            }
            // ---- back substitution, chunk by chunk from the end
            R xn = x;
            const long long qlast = q0 + (long long)(nline - 1) * stride;
            if (A.add) A.dst[qlast] += xn;
            else if (F32) A.dst[qlast] = xn;
            for (int c1 = nline - 2; c1 >= 0; c1 -= CH) {
                R ov[CH], gv[CH], fv[CH];
#pragma unroll
                for (int u = 0; u < CH; u++) {
                    const int l = c1 - u;
                    if (l >= 0) {
                        const long long q = q0 + (long long)l * stride;
                        ov[u] = xs[q];
                        gv[u] = sg[q + stride];
                        if (A.add) fv[u] = R(A.dst[q]);
                    }
                }
#pragma unroll
                for (int u = 0; u < CH; u++) {
                    const int l = c1 - u;
                    if (l >= 0) {
                        const long long q = q0 + (long long)l * stride;
                        const R xl = ov[u] - gv[u] * xn;
                        if (A.add) A.dst[q] = fv[u] + xl;
                        else if (F32) A.dst[q] = xl;
                        else xs[q] = xl;
                        xn = xl;
                    }
                }
            }
        } else {
            // ---- trdiagp: forward sweep; q factors, s and f vectors in the
            // scratch (FP64: q in gam, s in sarr, f in the source when adding,
            // else in dst; FP32: q, f in gam's two halves, s in sarr)
            R *fw = F32 ? sf : reinterpret_cast<R *>(A.add ? (double *)A.src : A.dst);
            const long long qn_last = q0 + (long long)(nline - 1) * stride;
            const R fn = diag * R(A.src[qn_last]);   // original right-hand side at the last element
            R qq = R(0.0), sv0 = R(0.0), ff = R(0.0);
            R a_last = R(0.0), b_last = R(0.0), c_last = R(0.0);
            R fprev = shared ? R(1.0) + F.cre * R(F.nv[q0 + F.oa]) : R(0.0);
            for (int c0 = 0; c0 < nline; c0 += CH) {
                R av[CH], cv[CH], rv[CH];
                adi_chunk_coefs<R, CH>(p, A.comp, DIR, F, shared, A.l1, c0, nline, x0, x1, q0, stride, fprev, av, cv);
#pragma unroll
                for (int u = 0; u < CH; u++)
                    if (c0 + u < nline) rv[u] = R(A.src[q0 + (long long)(c0 + u) * stride]);
#pragma unroll
                for (int u = 0; u < CH; u++) {
                    if (c0 + u < nline) {
                        const long long q = q0 + (long long)(c0 + u) * stride;
                        const R a = av[u], c = cv[u];
                        const R b = diag - a - c;
                        if (c0 + u == 0) {
                            const R binv = rcp_pivot(b);
                            qq = -c * binv;
                            sv0 = -a * binv;
                            ff = diag * rv[u] * binv;
                        } else {
                            const R pn = rcp_pivot(b + a * qq);
                            const R qn = -c * pn;
                            const R sn = -a * sv0 * pn;
                            ff = (diag * rv[u] - a * ff) * pn;
                            qq = qn;
                            sv0 = sn;
                        }
                        sg[q] = qq;
                        ss[q] = sv0;
                        fw[q] = ff;
                        a_last = a; b_last = b; c_last = c;
                    }
                }
            }
            // backward pass: s(j) += q(j) s(j+1); qe(j) = f(j) + q(j) qe(j+1)
            R s_next = R(1.0), qe_next = R(0.0), s_j2m1 = R(0.0), qe_j2m1 = R(0.0);
            for (int c1 = nline - 2; c1 >= 0; c1 -= CH) {
                R qv[CH], sv[CH], fv[CH];
#pragma unroll
                for (int u = 0; u < CH; u++) {
                    const int l = c1 - u;
                    if (l >= 0) {
                        const long long q = q0 + (long long)l * stride;
                        qv[u] = sg[q];
                        sv[u] = ss[q];
                        fv[u] = fw[q];
                    }
                }
#pragma unroll
                for (int u = 0; u < CH; u++) {
                    const int l = c1 - u;
                    if (l >= 0) {
                        const long long q = q0 + (long long)l * stride;
                        const R sj = sv[u] + qv[u] * s_next;
                        const R qej = fv[u] + qv[u] * qe_next;
                        ss[q] = sj;
                        fw[q] = qej;
                        if (l == nline - 2) { s_j2m1 = sj; qe_j2m1 = qej; }
                        s_next = sj;
                        qe_next = qej;
                    }
                }
            }
            const R s_j1 = s_next, qe_j1 = qe_next;
            const R fj2 = (fn - c_last * qe_j1 - a_last * qe_j2m1) / (c_last * s_j1 + a_last * s_j2m1 + b_last);
            if (A.add) A.dst[qn_last] += fj2;
            else if (F32) A.dst[qn_last] = fj2;
            else fw[qn_last] = fj2;
            for (int c1 = nline - 2; c1 >= 0; c1 -= CH) {
                R sv[CH], ev[CH], dv[CH];
#pragma unroll
                for (int u = 0; u < CH; u++) {
                    const int l = c1 - u;
                    if (l >= 0) {
                        const long long q = q0 + (long long)l * stride;
                        sv[u] = ss[q];
                        ev[u] = fw[q];
                        if (A.add) dv[u] = R(A.dst[q]);
                    }
                }
#pragma unroll
                for (int u = 0; u < CH; u++) {
                    const int l = c1 - u;
                    if (l >= 0) {
                        const long long q = q0 + (long long)l * stride;
                        const R val = fj2 * sv[u] + ev[u];
                        if (A.add) A.dst[q] = dv[u] + val;
                        else if (F32) A.dst[q] = val;
                        else fw[q] = val;
                    }
                }
            }
        }
    }
}

template <class R, int DIR>
static void k_adi_launch_dir(bool per, bool fac, dim3 grid, int tpb, cudaStream_t st, const KP &kp, const AdiBatch &B) {
    if (per) { if (fac) k_adi<R, DIR, true, true><<<grid, tpb, 0, st>>>(kp, B); else k_adi<R, DIR, true, false><<<grid, tpb, 0, st>>>(kp, B); }
    else { if (fac) k_adi<R, DIR, false, true><<<grid, tpb, 0, st>>>(kp, B); else k_adi<R, DIR, false, false><<<grid, tpb, 0, st>>>(kp, B); }
}

template <class R>
static void k_adi_launch(int dir, bool per, bool fac, dim3 grid, int tpb, cudaStream_t st, const KP &kp, const AdiBatch &B) {
    if (dir == 0) k_adi_launch_dir<R, 0>(per, fac, grid, tpb, st, kp, B);
    else if (dir == 1) k_adi_launch_dir<R, 1>(per, fac, grid, tpb, st, kp, B);
    else k_adi_launch_dir<R, 2>(per, fac, grid, tpb, st, kp, B);
}

// ------------------------------------------------------------------------
// Warp-per-line sweeps.  One thread per line leaves a 64^3 grid with ~2.5
// warps per SM and a 2n-step dependent chain per line, so the sweep is
// latency bound in FP64 and FP32 alike.  Here a warp solves a line: lane l
// owns rows [l*m, l*m+m) (m = ceil(n/32) <= MC, held in registers), and each
// recurrence of the reference's algorithm is split into
//   1. the chunk's composed map (a 2x2 matrix for the pivots, whose
//      recurrence bet_j = 1/(b_j - a_j c_{j-1} bet_{j-1}) is a Moebius map;
//      an affine map for the substitutions),
//   2. a 5-step shuffle scan over the lanes,
//   3. the chunk re-run with the reference's recurrence from the scanned
//      incoming value.
// The dependent chain of a 64-row line drops from 128 steps to ~30 and the
// GPU holds 32 times as many threads.  Matrix products are rescaled by their
// largest entry (the pivot is a ratio), so nothing overflows in FP32.
template <class R>
struct M22 { R a, b, c, d; };     // [[a, b], [c, d]]

template <class R>
__device__ __forceinline__ M22<R> mmul_raw(const M22<R> &x, const M22<R> &y) {   // x * y
    return M22<R>{x.a * y.a + x.b * y.c, x.a * y.b + x.b * y.d, x.c * y.a + x.d * y.c, x.c * y.b + x.d * y.d};
}
template <class R>
__device__ __forceinline__ M22<R> mmul(const M22<R> &x, const M22<R> &y) {   // x * y, rescaled
    M22<R> r = mmul_raw(x, y);
    R m = fmax(fmax(fabs(r.a), fabs(r.b)), fmax(fabs(r.c), fabs(r.d)));
    if (m > R(0.0)) {
        const R s = R(1.0) / m;
        r.a *= s; r.b *= s; r.c *= s; r.d *= s;
    }
    return r;
}
// Inside a chunk FP64 needs no rescaling (at most 12 rows of ~1e8 entries);
// FP32 rescales every row.
template <class R>
__device__ __forceinline__ M22<R> mmul_chunk(const M22<R> &x, const M22<R> &y) {
    if (sizeof(R) == 8) return mmul_raw(x, y);
    return mmul(x, y);
}

template <class R, int W>
__device__ __forceinline__ M22<R> shfl_up_m(const M22<R> &x, int d) {
    return M22<R>{__shfl_up_sync(0xffffffffu, x.a, d, W), __shfl_up_sync(0xffffffffu, x.b, d, W),
                  __shfl_up_sync(0xffffffffu, x.c, d, W), __shfl_up_sync(0xffffffffu, x.d, d, W)};
}

// exclusive prefix over lanes of a matrix product applied to (0, 1):
// returns the column vector (P, Q) entering this lane's chunk
template <class R, int W>
__device__ __forceinline__ void scan_moebius(M22<R> T, int lane, R &P, R &Q) {
#pragma unroll
    for (int d = 1; d < W; d <<= 1) {
        M22<R> o = shfl_up_m<R, W>(T, d);
        if (lane >= d) T = mmul(T, o);
    }
    // inclusive product S_l = T_l ... T_0; the incoming vector is S_{l-1} (0, 1)^T
    R pb = __shfl_up_sync(0xffffffffu, T.b, 1, W), qd = __shfl_up_sync(0xffffffffu, T.d, 1, W);
    if (lane == 0) { pb = R(0.0); qd = R(1.0); }
    P = pb;
    Q = qd;
}

// exclusive forward scan of affine maps y = A y_prev + B; y_(-1) = y0
template <class R, int W>
__device__ __forceinline__ R scan_affine_up(R A, R B, int lane, R y0) {
#pragma unroll
    for (int d = 1; d < W; d <<= 1) {
        const R Ap = __shfl_up_sync(0xffffffffu, A, d, W), Bp = __shfl_up_sync(0xffffffffu, B, d, W);
        if (lane >= d) { B = A * Bp + B; A = A * Ap; }
    }
    R Ai = __shfl_up_sync(0xffffffffu, A, 1, W), Bi = __shfl_up_sync(0xffffffffu, B, 1, W);
    if (lane == 0) return y0;
    return Ai * y0 + Bi;
}

// exclusive backward scan of x = C x_next + D; x past the end = 0
template <class R, int W>
__device__ __forceinline__ R scan_affine_down(R C, R D, int lane) {
#pragma unroll
    for (int d = 1; d < W; d <<= 1) {
        const R Cn = __shfl_down_sync(0xffffffffu, C, d, W), Dn = __shfl_down_sync(0xffffffffu, D, d, W);
        if (lane + d < W) { D = C * Dn + D; C = C * Cn; }
    }
    R Di = __shfl_down_sync(0xffffffffu, D, 1, W);
    return lane == W - 1 ? R(0.0) : Di;
}

// MINB > 1 caps the registers (65536 / (128 MINB) per thread) so that MINB
// blocks fit on an SM: more warps in flight for some spilling -- which of the
// two is faster depends on the shape, and the autotuner times both.
template <class R, int MC, int W, int MINB>
__global__ void __launch_bounds__(128, MINB) k_adis(KP p, AdiBatch B) {
    const AdiArgs &A = B.a[blockIdx.y];
    const DGrid &g = p.g;
    const R diag = (A.comp == CT) ? p.S->acoefi * p.c.pr : p.S->acoefi;
    const int na = A.a1 - A.a0 + 1, nb = A.b1 - A.b0 + 1;
    const long long nl = (long long)na * nb;
    const long long stride = A.dir == 2 ? g.sxy : A.dir == 1 ? g.sx : 1;
    const int n = A.l2 - A.l1 + 1;
    if (nl <= 0 || n <= 0) return;
    const int lane = threadIdx.x & (W - 1);       // W lanes per line, 32/W lines per warp
    const int m = (n + W - 1) / W;
    const int r0 = lane * m;
    const int cnt = max(0, min(m, n - r0));
    const long long lpb = blockDim.x / W;
    // every lane of a warp runs the same number of iterations (shuffles need the full warp)
    const long long nl_pad = (nl + (32 / W) - 1) / (32 / W) * (32 / W);
    for (long long t = blockIdx.x * lpb + threadIdx.x / W; t < nl_pad; t += (long long)gridDim.x * lpb) {
        const bool live = t < nl;
        const long long tl = live ? t : nl - 1;     // a dead lane repeats the last line, stores nothing
        const int x0 = A.a0 + (int)(tl % na), x1 = A.b0 + (int)(tl / na);
        int i0, j0, k0;
        line_coords(A.dir, A.l1, x0, x1, i0, j0, k0);
        const long long q0 = g.ix(i0, j0, k0);
        R av[MC], bv[MC], cv[MC], rv[MC];
#pragma unroll
        for (int u = 0; u < MC; u++)
            if (u < cnt) {
                int i, j, k;
                line_coords(A.dir, A.l1 + r0 + u, x0, x1, i, j, k);
                adi_coef<R>(p, A.comp, A.dir, i, j, k, av[u], cv[u]);
                bv[u] = diag - av[u] - cv[u];
                rv[u] = diag * R(A.src[q0 + (long long)(r0 + u) * stride]);
            }
        // c of the row before this chunk
        R clast = R(0.0);
#pragma unroll
        for (int u = 0; u < MC; u++)
            if (u == cnt - 1) clast = cv[u];
        R cprev0 = __shfl_up_sync(0xffffffffu, clast, 1, W);
        if (lane == 0) cprev0 = R(0.0);
        R xv[MC];
        if (!A.periodic) {
            // 1. pivots bet_j (Moebius in bet_{j-1})
            M22<R> T{R(1.0), R(0.0), R(0.0), R(1.0)};
            {
                R cp = cprev0;
#pragma unroll
                for (int u = 0; u < MC; u++)
                    if (u < cnt) {
                        M22<R> Tj{R(0.0), R(1.0), -av[u] * cp, bv[u]};
                        T = mmul_chunk(Tj, T);
                        cp = cv[u];
                    }
            }
            R P, Q;
            scan_moebius<R, W>(T, lane, P, Q);
            R bet = (lane == 0) ? R(0.0) : P / Q;     // bet of the row before the chunk
            R gmv[MC];
            {
                R cp = cprev0;
#pragma unroll
                for (int u = 0; u < MC; u++)
                    if (u < cnt) {
                        if (lane == 0 && u == 0) {
                            bet = rcp_pivot(bv[u]);
                            gmv[u] = R(0.0);
                        } else {
                            const R gm = cp * bet;
                            bet = rcp_pivot(bv[u] - av[u] * gm);
                            gmv[u] = gm;
                        }
                        bv[u] = bet;          // bv now holds bet_j
                        cp = cv[u];
                    }
            }
            // 2. forward substitution y_j = (r_j - a_j y_{j-1}) bet_j
            R Aa = R(1.0), Bb = R(0.0);
#pragma unroll
            for (int u = 0; u < MC; u++)
                if (u < cnt) {
                    const R mj = (lane == 0 && u == 0) ? R(0.0) : -av[u] * bv[u];
                    Bb = mj * Bb + rv[u] * bv[u];
                    Aa = mj * Aa;
                }
            R y = scan_affine_up<R, W>(Aa, Bb, lane, R(0.0));
#pragma unroll
            for (int u = 0; u < MC; u++)
                if (u < cnt) {
                    y = (lane == 0 && u == 0) ? rv[u] * bv[u] : (rv[u] - av[u] * y) * bv[u];
                    rv[u] = y;            // rv now holds y_j
                }
            // 3. back substitution x_j = y_j - gm_{j+1} x_{j+1}
            R gnext0 = __shfl_down_sync(0xffffffffu, gmv[0], 1, W);   // gm of the row after the chunk
            R Cc = R(1.0), Dd = R(0.0);
#pragma unroll
            for (int u = MC - 1; u >= 0; u--)
                if (u < cnt) {
                    const bool last = (r0 + u == n - 1);
                    const R gn = last ? R(0.0) : (u + 1 < cnt ? gmv[u + 1] : gnext0);
                    Dd = -gn * Dd + rv[u];
                    Cc = -gn * Cc;
                }
            R x = scan_affine_down<R, W>(Cc, Dd, lane);
#pragma unroll
            for (int u = MC - 1; u >= 0; u--)
                if (u < cnt) {
                    const bool last = (r0 + u == n - 1);
                    const R gn = last ? R(0.0) : (u + 1 < cnt ? gmv[u + 1] : gnext0);
                    x = rv[u] - gn * x;
                    xv[u] = x;
                }
        } else {
            // trdiagp: q_j = -c_j / (b_j + a_j q_{j-1}) (Moebius), pn_j the pivots
            M22<R> T{R(1.0), R(0.0), R(0.0), R(1.0)};
#pragma unroll
            for (int u = 0; u < MC; u++)
                if (u < cnt) {
                    M22<R> Tj{R(0.0), -cv[u], av[u], bv[u]};
                    T = mmul_chunk(Tj, T);
                }
            R P, Q;
            scan_moebius<R, W>(T, lane, P, Q);
            R qq = (lane == 0) ? R(0.0) : P / Q;
            R qv[MC], pv[MC];
#pragma unroll
            for (int u = 0; u < MC; u++)
                if (u < cnt) {
                    const R pn = rcp_pivot((lane == 0 && u == 0) ? bv[u] : bv[u] + av[u] * qq);
                    qq = -cv[u] * pn;
                    qv[u] = qq;
                    pv[u] = pn;
                }
            // s_j = (-a_j pn_j) s_{j-1}, s_{-1} = 1;  f_j = (-a_j pn_j) f_{j-1} + r_j pn_j, f_{-1} = 0
            R Aa = R(1.0), Bb = R(0.0);
#pragma unroll
            for (int u = 0; u < MC; u++)
                if (u < cnt) {
                    const R mj = -av[u] * pv[u];
                    Bb = mj * Bb + rv[u] * pv[u];
                    Aa = mj * Aa;
                }
            // incoming s and f: run the same scan for the pair
            R sA = Aa, fA = Aa, fB = Bb;
#pragma unroll
            for (int d = 1; d < W; d <<= 1) {
                const R sp = __shfl_up_sync(0xffffffffu, sA, d, W);
                const R Ap = __shfl_up_sync(0xffffffffu, fA, d, W), Bp = __shfl_up_sync(0xffffffffu, fB, d, W);
                if (lane >= d) { sA = sA * sp; fB = fA * Bp + fB; fA = fA * Ap; }
            }
            R s_in = __shfl_up_sync(0xffffffffu, sA, 1, W), f_in = __shfl_up_sync(0xffffffffu, fB, 1, W);
            if (lane == 0) { s_in = R(1.0); f_in = R(0.0); }
            R sv[MC], fv[MC];
            {
                R sc = s_in, fc = f_in;
#pragma unroll
                for (int u = 0; u < MC; u++)
                    if (u < cnt) {
                        if (lane == 0 && u == 0) {
                            sc = -av[u] * pv[u];
                            fc = rv[u] * pv[u];
                        } else {
                            sc = -av[u] * sc * pv[u];
                            fc = (rv[u] - av[u] * fc) * pv[u];
                        }
                        sv[u] = sc;
                        fv[u] = fc;
                    }
            }
            // backward: S_j = s_j + q_j S_{j+1}, QE_j = f_j + q_j QE_{j+1}; S_{n-1} = 1, QE_{n-1} = 0
            R Cs = R(1.0), Ds = R(0.0), De = R(0.0);
#pragma unroll
            for (int u = MC - 1; u >= 0; u--)
                if (u < cnt) {
                    const bool last = (r0 + u == n - 1);
                    const R mq = last ? R(0.0) : qv[u];
                    const R os = last ? R(1.0) : sv[u], oe = last ? R(0.0) : fv[u];
                    Ds = mq * Ds + os;
                    De = mq * De + oe;
                    Cs = mq * Cs;
                }
#pragma unroll
            for (int d = 1; d < W; d <<= 1) {
                const R Cn = __shfl_down_sync(0xffffffffu, Cs, d, W);
                const R Dsn = __shfl_down_sync(0xffffffffu, Ds, d, W), Den = __shfl_down_sync(0xffffffffu, De, d, W);
                if (lane + d < W) { Ds = Cs * Dsn + Ds; De = Cs * Den + De; Cs = Cs * Cn; }
            }
            R S_in = __shfl_down_sync(0xffffffffu, Ds, 1, W), E_in = __shfl_down_sync(0xffffffffu, De, 1, W);
            if (lane == W - 1) { S_in = R(0.0); E_in = R(0.0); }
            {
                R Sc = S_in, Ec = E_in;
#pragma unroll
                for (int u = MC - 1; u >= 0; u--)
                    if (u < cnt) {
                        if (r0 + u == n - 1) { Sc = R(1.0); Ec = R(0.0); }
                        else {
                            Sc = sv[u] + qv[u] * Sc;
                            Ec = fv[u] + qv[u] * Ec;
                        }
                        sv[u] = Sc;          // S_j
                        fv[u] = Ec;          // QE_j
                    }
            }
            // fj2 from S_0, QE_0, S_{n-2}, QE_{n-2} and the last row
            const int own_last = (n - 1) / m, u_last = (n - 1) - own_last * m;
            const int own_pen = (n - 2) / m, u_pen = (n - 2) - own_pen * m;
            R al = R(0.0), bl = R(0.0), cl = R(0.0), fnl = R(0.0), Sp = R(0.0), Ep = R(0.0);
#pragma unroll
            for (int u = 0; u < MC; u++) {
                if (u == u_last) { al = av[u]; bl = bv[u]; cl = cv[u]; fnl = rv[u]; }
                if (u == u_pen) { Sp = sv[u]; Ep = fv[u]; }
            }
            al = __shfl_sync(0xffffffffu, al, own_last, W);
            bl = __shfl_sync(0xffffffffu, bl, own_last, W);
            cl = __shfl_sync(0xffffffffu, cl, own_last, W);
            fnl = __shfl_sync(0xffffffffu, fnl, own_last, W);
            Sp = __shfl_sync(0xffffffffu, Sp, own_pen, W);
            Ep = __shfl_sync(0xffffffffu, Ep, own_pen, W);
            const R S0 = __shfl_sync(0xffffffffu, sv[0], 0, W), E0 = __shfl_sync(0xffffffffu, fv[0], 0, W);
            const R fj2 = (fnl - cl * E0 - al * Ep) / (cl * S0 + al * Sp + bl);
#pragma unroll
            for (int u = 0; u < MC; u++)
                if (u < cnt) xv[u] = (r0 + u == n - 1) ? fj2 : fj2 * sv[u] + fv[u];
        }
        // store: the solution, or added to the field
#pragma unroll
        for (int u = 0; u < MC; u++)
            if (live && u < cnt) {
                const long long q = q0 + (long long)(r0 + u) * stride;
                if (A.add) A.dst[q] = A.dst[q] + xv[u];
                else A.dst[q] = xv[u];
            }
    }
}

// ------------------------------------------------------------------------
// Tiled warp-scan sweeps (x and z sweeps in FP32).  A block stages a tile
// of kTileLines lines -- consecutive i for z lines, consecutive j for x
// lines -- in shared memory with coalesced loads: the right-hand side
// (times the diagonal, in R) and every row's coefficients a and c (the
// metric terms times the viscosity factors 1 + cre nu of the row's two
// faces), formed once there; one warp then solves one line from shared
// memory with the recurrences and chunk layout of k_adis (W = 32 lanes,
// lane l owning rows l*m .. l*m+m-1), reading the coefficients from shared
// memory in each pass instead of holding them in registers, and the tile is
// written back coalesced.  The serial z sweep moved each line's elimination factors
// through HBM (2.6 times the sweep's algorithmic bytes) and k_adis held a
// 12-row chunk's coefficients in registers (16 warps an SM); here the HBM
// traffic is the operands once and 32 warps fit on an SM.  Results equal
// the 32-lane k_adis's: the same arithmetic on the same chunks.
constexpr int kTileLines = 16;
constexpr size_t kTileSmemMax = 110 * 1024;   // two blocks an SM

// position of row r of a line in shared memory: lane chunks of m rows with
// a pitch pm (odd: the 32 lanes' rows fall in 32 different banks)
__device__ __forceinline__ int tpos(int r, int m, int pm) { return (r / m) * pm + r % m; }

template <class R, int DIR, bool PER, int MC>
__global__ void __launch_bounds__(kTileLines * 32, 2) k_adit(KP p, AdiBatch B, int m, int pm, int lp) {
    extern __shared__ __align__(16) unsigned char adit_smem[];
    R *S = reinterpret_cast<R *>(adit_smem);             // lines x lp: diag*rhs -> y -> x
    R *Ca = S + kTileLines * lp;                          // lines x lp: a of rows 0..n-1
    R *Cc = Ca + kTileLines * lp;                         // lines x lp: c of rows 0..n-1
    const AdiArgs &A = B.a[blockIdx.y];
    const DGrid &g = p.g;
    const R diag = (A.comp == CT) ? p.S->acoefi * p.c.pr : p.S->acoefi;
    const int na = A.a1 - A.a0 + 1, nb = A.b1 - A.b0 + 1;
    const int n = A.l2 - A.l1 + 1;
    const long long stride = DIR == 2 ? g.sxy : 1;
    const long long lstride = DIR == 2 ? 1 : g.sx;       // between consecutive lines of a tile
    const int ntx = (na + kTileLines - 1) / kTileLines;
    if ((int)blockIdx.x >= ntx * nb || n <= 0) return;
    const int x0 = A.a0 + (int)(blockIdx.x % ntx) * kTileLines, x1 = A.b0 + (int)(blockIdx.x / ntx);
    const int nl = min(kTileLines, A.a1 - x0 + 1);
    int i0, j0, k0;
    line_coords(DIR, A.l1, x0, x1, i0, j0, k0);
    const long long qb = g.ix(i0, j0, k0);                // row 0 of line 0
    const AdiFacs<R> F = adi_facs<R>(p, A.comp, DIR);
    // ---- stage the tile (z: lines fastest, x: rows fastest: both coalesced);
    // each thread issues the loads of four elements before it stores them.
    // tp[r]: row r's slot in a line (rows 0..n), formed once per block.
    const int nt = blockDim.x;
    int *tp = reinterpret_cast<int *>(Cc + kTileLines * lp);
    for (int r = threadIdx.x; r <= n; r += nt) tp[r] = tpos(r, m, pm);
    __syncthreads();
    if (DIR == 2) {
        const int ntot = kTileLines * (n + 1);
        for (int t0 = threadIdx.x; t0 < ntot; t0 += 4 * nt) {
            double sv[4];
            R fv[4];
            int pos[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int t = t0 + u * nt;
                pos[u] = -1;
                if (t < ntot) {
                    const int w = t % kTileLines, r = t / kTileLines;
                    if (w < nl) {
                        const long long q = qb + w * lstride + (long long)r * stride;
                        pos[u] = w * lp + tp[r];
                        fv[u] = R(F.nv[q + F.oa]);
                        sv[u] = r < n ? A.src[q] : 0.0;
                        if (r >= n) pos[u] = -2 - pos[u];      // the factor row only
                    }
                }
            }
#pragma unroll
            for (int u = 0; u < 4; u++) {
                if (pos[u] == -1) continue;
                const int ps = pos[u] >= 0 ? pos[u] : -2 - pos[u];
                const int r = (t0 + u * nt) / kTileLines, w = (t0 + u * nt) % kTileLines;
                const R f = R(1.0) + F.cre * fv[u];
                if (pos[u] >= 0) {
                    S[ps] = diag * R(sv[u]);
                    Ca[ps] = R(F.ma[A.l1 + r]) * f;
                }
                if (r >= 1) Cc[w * lp + tp[r - 1]] = R(F.mc[A.l1 + r - 1]) * f;
            }
        }
    } else {
        // a thread takes one row of four lines at a time
        for (int r = threadIdx.x; r <= n; r += nt) {
            const int pr = tp[r], pr1 = r >= 1 ? tp[r - 1] : 0;
            const R ma_r = r < n ? R(F.ma[A.l1 + r]) : R(0.0), mc_r1 = r >= 1 ? R(F.mc[A.l1 + r - 1]) : R(0.0);
            for (int w0 = 0; w0 < nl; w0 += 4) {
                double sv[4];
                R fv[4];
#pragma unroll
                for (int u = 0; u < 4; u++)
                    if (w0 + u < nl) {
                        const long long q = qb + (w0 + u) * lstride + (long long)r * stride;
                        fv[u] = R(F.nv[q + F.oa]);
                        sv[u] = r < n ? A.src[q] : 0.0;
                    }
#pragma unroll
                for (int u = 0; u < 4; u++)
                    if (w0 + u < nl) {
                        const int ps = (w0 + u) * lp + pr;
                        const R f = R(1.0) + F.cre * fv[u];
                        if (r < n) {
                            S[ps] = diag * R(sv[u]);
                            Ca[ps] = ma_r * f;
                        }
                        if (r >= 1) Cc[(w0 + u) * lp + pr1] = mc_r1 * f;
                    }
            }
        }
    }
    __syncthreads();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (w < nl) {
        R *Sl = S + w * lp;
        const R *Al = Ca + w * lp, *Cl = Cc + w * lp;
        const int r0 = lane * m;
        const int cnt = max(0, min(m, n - r0));
        // the lane's rows sit at lb .. lb + m - 1
        const int lb = lane * pm;
        auto coef = [&](int u, R &a, R &c) {
            a = Al[lb + u];
            c = Cl[lb + u];
        };
        if (!PER) {
            // c of the row before the chunk
            R cprev0 = R(0.0);
            if (lane > 0 && r0 - 1 < n) cprev0 = Cl[lb - pm + m - 1];
            if (r0 - 1 >= n) cprev0 = R(0.0);
            // 1. pivots: Moebius composition, scan, re-run
            M22<R> T{R(1.0), R(0.0), R(0.0), R(1.0)};
            {
                R cp = cprev0;
#pragma unroll
                for (int u = 0; u < MC; u++)
                    if (u < cnt) {
                        R a, c;
                        coef(u, a, c);
                        const R b = diag - a - c;
                        M22<R> Tj{R(0.0), R(1.0), -a * cp, b};
                        T = mmul_chunk(Tj, T);
                        cp = c;
                    }
            }
            R P, Q;
            scan_moebius<R, 32>(T, lane, P, Q);
            R bet = (lane == 0) ? R(0.0) : P / Q;
            // gm of the chunk's first row, c_{r0-1} times the scanned pivot
            // (k_adis keeps it, and the previous chunk's last row uses it)
            const R gm_first = (lane == 0) ? R(0.0) : cprev0 * bet;
            const R gnext0 = __shfl_down_sync(0xffffffffu, gm_first, 1);
            R betv[MC];
            {
                R cp = cprev0;
#pragma unroll
                for (int u = 0; u < MC; u++)
                    if (u < cnt) {
                        R a, c;
                        coef(u, a, c);
                        const R b = diag - a - c;
                        if (lane == 0 && u == 0) bet = rcp_pivot(b);
                        else bet = rcp_pivot(b - a * (cp * bet));
                        betv[u] = bet;
                        cp = c;
                    }
            }
            // 2. forward substitution y_j = (r_j - a_j y_{j-1}) bet_j
            R Aa = R(1.0), Bb = R(0.0);
#pragma unroll
            for (int u = 0; u < MC; u++)
                if (u < cnt) {
                    R a, c;
                    coef(u, a, c);
                    const R mj = (lane == 0 && u == 0) ? R(0.0) : -a * betv[u];
                    Bb = mj * Bb + Sl[lb + u] * betv[u];
                    Aa = mj * Aa;
                }
            R y = scan_affine_up<R, 32>(Aa, Bb, lane, R(0.0));
#pragma unroll
            for (int u = 0; u < MC; u++)
                if (u < cnt) {
                    R a, c;
                    coef(u, a, c);
                    const int ps = lb + u;
                    y = (lane == 0 && u == 0) ? Sl[ps] * betv[u] : (Sl[ps] - a * y) * betv[u];
                    Sl[ps] = y;
                }
            // 3. back substitution x_j = y_j - gm_{j+1} x_{j+1}, gm_{j+1} = c_j bet_j
            R Cc = R(1.0), Dd = R(0.0);
#pragma unroll
            for (int u = MC - 1; u >= 0; u--)
                if (u < cnt) {
                    R a, c;
                    coef(u, a, c);
                    const R gn = (r0 + u == n - 1) ? R(0.0) : (u + 1 < cnt ? c * betv[u] : gnext0);
                    Dd = -gn * Dd + Sl[lb + u];
                    Cc = -gn * Cc;
                }
            R x = scan_affine_down<R, 32>(Cc, Dd, lane);
#pragma unroll
            for (int u = MC - 1; u >= 0; u--)
                if (u < cnt) {
                    R a, c;
                    coef(u, a, c);
                    const R gn = (r0 + u == n - 1) ? R(0.0) : (u + 1 < cnt ? c * betv[u] : gnext0);
                    const int ps = lb + u;
                    x = Sl[ps] - gn * x;
                    Sl[ps] = x;
                }
        } else {
            // trdiagp: q_j = -c_j / (b_j + a_j q_{j-1}) (Moebius), pn_j the pivots
            M22<R> T{R(1.0), R(0.0), R(0.0), R(1.0)};
#pragma unroll
            for (int u = 0; u < MC; u++)
                if (u < cnt) {
                    R a, c;
                    coef(u, a, c);
                    const R b = diag - a - c;
                    M22<R> Tj{R(0.0), -c, a, b};
                    T = mmul_chunk(Tj, T);
                }
            R P, Q;
            scan_moebius<R, 32>(T, lane, P, Q);
            R qq = (lane == 0) ? R(0.0) : P / Q;
            R pv[MC], sv[MC];
            R Aa = R(1.0), Bb = R(0.0);
#pragma unroll
            for (int u = 0; u < MC; u++)
                if (u < cnt) {
                    R a, c;
                    coef(u, a, c);
                    const R b = diag - a - c;
                    const R pn = rcp_pivot((lane == 0 && u == 0) ? b : b + a * qq);
                    qq = -c * pn;
                    pv[u] = pn;
                    const R mj = -a * pn;
                    Bb = mj * Bb + Sl[lb + u] * pn;
                    Aa = mj * Aa;
                }
            // incoming s and f
            R sA = Aa, fA = Aa, fB = Bb;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const R sp = __shfl_up_sync(0xffffffffu, sA, d);
                const R Ap = __shfl_up_sync(0xffffffffu, fA, d), Bp = __shfl_up_sync(0xffffffffu, fB, d);
                if (lane >= d) { sA = sA * sp; fB = fA * Bp + fB; fA = fA * Ap; }
            }
            R s_in = __shfl_up_sync(0xffffffffu, sA, 1), f_in = __shfl_up_sync(0xffffffffu, fB, 1);
            if (lane == 0) { s_in = R(1.0); f_in = R(0.0); }
            // the last row's a, b, c and right-hand side, kept for fj2
            R al = R(0.0), bl = R(0.0), cl = R(0.0), fnl = R(0.0);
            {
                R sc = s_in, fc = f_in;
#pragma unroll
                for (int u = 0; u < MC; u++)
                    if (u < cnt) {
                        R a, c;
                        coef(u, a, c);
                        const int ps = lb + u;
                        const R rv = Sl[ps];
                        if (r0 + u == n - 1) { al = a; bl = diag - a - c; cl = c; fnl = rv; }
                        if (lane == 0 && u == 0) {
                            sc = -a * pv[u];
                            fc = rv * pv[u];
                        } else {
                            sc = -a * sc * pv[u];
                            fc = (rv - a * fc) * pv[u];
                        }
                        sv[u] = sc;
                        Sl[ps] = fc;
                    }
            }
            // backward: S_j = s_j + q_j S_{j+1}, QE_j = f_j + q_j QE_{j+1}; S_{n-1} = 1, QE_{n-1} = 0
            R Cs = R(1.0), Ds = R(0.0), De = R(0.0);
#pragma unroll
            for (int u = MC - 1; u >= 0; u--)
                if (u < cnt) {
                    R a, c;
                    coef(u, a, c);
                    const bool last = (r0 + u == n - 1);
                    const R mq = last ? R(0.0) : -c * pv[u];
                    const R os = last ? R(1.0) : sv[u], oe = last ? R(0.0) : Sl[lb + u];
                    Ds = mq * Ds + os;
                    De = mq * De + oe;
                    Cs = mq * Cs;
                }
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const R Cn = __shfl_down_sync(0xffffffffu, Cs, d);
                const R Dsn = __shfl_down_sync(0xffffffffu, Ds, d), Den = __shfl_down_sync(0xffffffffu, De, d);
                if (lane + d < 32) { Ds = Cs * Dsn + Ds; De = Cs * Den + De; Cs = Cs * Cn; }
            }
            R S_in = __shfl_down_sync(0xffffffffu, Ds, 1), E_in = __shfl_down_sync(0xffffffffu, De, 1);
            if (lane == 31) { S_in = R(0.0); E_in = R(0.0); }
            R Sp = R(0.0), Ep = R(0.0);
            {
                R Sc = S_in, Ec = E_in;
#pragma unroll
                for (int u = MC - 1; u >= 0; u--)
                    if (u < cnt) {
                        R a, c;
                        coef(u, a, c);
                        const int ps = lb + u;
                        if (r0 + u == n - 1) { Sc = R(1.0); Ec = R(0.0); }
                        else {
                            const R qj = -c * pv[u];
                            Sc = sv[u] + qj * Sc;
                            Ec = Sl[ps] + qj * Ec;
                        }
                        sv[u] = Sc;          // S_j
                        Sl[ps] = Ec;         // QE_j
                        if (r0 + u == n - 2) { Sp = Sc; Ep = Ec; }
                    }
            }
            // fj2 from S_0, QE_0, S_{n-2}, QE_{n-2} and the last row
            const int own_last = (n - 1) / m, own_pen = (n - 2) / m;
            al = __shfl_sync(0xffffffffu, al, own_last);
            bl = __shfl_sync(0xffffffffu, bl, own_last);
            cl = __shfl_sync(0xffffffffu, cl, own_last);
            fnl = __shfl_sync(0xffffffffu, fnl, own_last);
            Sp = __shfl_sync(0xffffffffu, Sp, own_pen);
            Ep = __shfl_sync(0xffffffffu, Ep, own_pen);
            const R S0 = __shfl_sync(0xffffffffu, sv[0], 0);
            const R E0 = Sl[0];
            const R fj2 = (fnl - cl * E0 - al * Ep) / (cl * S0 + al * Sp + bl);
            __syncwarp();
#pragma unroll
            for (int u = 0; u < MC; u++)
                if (u < cnt) {
                    const int ps = lb + u;
                    Sl[ps] = (r0 + u == n - 1) ? fj2 : fj2 * sv[u] + Sl[ps];
                }
        }
    }
    __syncthreads();
    // ---- write back: the solution, or added to the field (four elements a
    // thread at a time, the field's loads first)
    if (DIR == 2) {
        for (int t0 = threadIdx.x; t0 < kTileLines * n; t0 += 4 * nt) {
            long long qv[4];
            double dv[4];
            R xv[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int t = t0 + u * nt;
                qv[u] = -1;
                if (t < kTileLines * n) {
                    const int w2 = t % kTileLines, r = t / kTileLines;
                    if (w2 < nl) {
                        qv[u] = qb + w2 * lstride + (long long)r * stride;
                        xv[u] = S[w2 * lp + tp[r]];
                        if (A.add) dv[u] = A.dst[qv[u]];
                    }
                }
            }
#pragma unroll
            for (int u = 0; u < 4; u++)
                if (qv[u] >= 0) A.dst[qv[u]] = A.add ? dv[u] + xv[u] : (double)xv[u];
        }
    } else {
        for (int r = threadIdx.x; r < n; r += nt) {
            const int pr = tp[r];
            for (int w0 = 0; w0 < nl; w0 += 4) {
                double dv[4];
#pragma unroll
                for (int u = 0; u < 4; u++)
                    if (w0 + u < nl && A.add) dv[u] = A.dst[qb + (w0 + u) * lstride + (long long)r * stride];
#pragma unroll
                for (int u = 0; u < 4; u++)
                    if (w0 + u < nl) {
                        const long long q = qb + (w0 + u) * lstride + (long long)r * stride;
                        const R xv = S[(w0 + u) * lp + pr];
                        A.dst[q] = A.add ? dv[u] + xv : (double)xv;
                    }
            }
        }
    }
}

// rows per lane of the tiled sweep (compile-time chunk bound), its shared memory
struct TileShape {
    int m, pm, lp, mc;
    size_t smem;
};
static TileShape tile_shape(int nmax) {
    TileShape t;
    t.m = (nmax + 31) / 32;
    t.pm = (t.m % 2 == 0) ? t.m + 1 : t.m + 2;
    t.lp = 32 * t.pm + 1;
    t.mc = t.m <= 4 ? 4 : t.m <= 8 ? 8 : t.m <= 12 ? 12 : t.m <= 16 ? 16 : 0;
    // the three tile arrays, then the row-slot table (rows 0 .. 32 m)
    t.smem = (size_t)3 * kTileLines * t.lp * sizeof(float) + (size_t)(32 * t.m + 1) * sizeof(int);
    return t;
}

template <int DIR, bool PER, int MC>
static void adit_launch3(dim3 grid, const TileShape &ts, cudaStream_t st, const KP &kp, const AdiBatch &B) {
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_adit<float, DIR, PER, MC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTileSmemMax);
        attr = true;
    }
    k_adit<float, DIR, PER, MC><<<grid, kTileLines * 32, ts.smem, st>>>(kp, B, ts.m, ts.pm, ts.lp);
}

template <int DIR, bool PER>
static bool adit_launch2(dim3 grid, const TileShape &ts, cudaStream_t st, const KP &kp, const AdiBatch &B) {
    switch (ts.mc) {
    case 4: adit_launch3<DIR, PER, 4>(grid, ts, st, kp, B); return true;
    case 8: adit_launch3<DIR, PER, 8>(grid, ts, st, kp, B); return true;
    case 12: adit_launch3<DIR, PER, 12>(grid, ts, st, kp, B); return true;
    case 16: adit_launch3<DIR, PER, 16>(grid, ts, st, kp, B); return true;
    }
    return false;
}

// The tiled FP32 sweep of a batch (x or z, factored coefficients); false
// when it does not apply (the caller falls back).
static bool adit_launch(lesgpu_case *c, const AdiBatch &B, int ncomp, int nmax) {
    const int dir = B.a[0].dir;
    if (dir == 1) return false;
    const TileShape ts = tile_shape(nmax);
    if (ts.mc == 0 || ts.smem > kTileSmemMax) return false;
    int tiles = 0;
    for (int q = 0; q < ncomp; q++) {
        const AdiArgs &A = B.a[q];
        const int na = A.a1 - A.a0 + 1, nb = A.b1 - A.b0 + 1;
        tiles = std::max(tiles, ((na + kTileLines - 1) / kTileLines) * nb);
    }
    if (tiles <= 0) return true;
    const dim3 grid((unsigned)tiles, (unsigned)ncomp);
    const bool per = B.a[0].periodic != 0;
    if (dir == 2) return per ? adit_launch2<2, true>(grid, ts, c->stream, c->kp, B) : adit_launch2<2, false>(grid, ts, c->stream, c->kp, B);
    return per ? adit_launch2<0, true>(grid, ts, c->stream, c->kp, B) : adit_launch2<0, false>(grid, ts, c->stream, c->kp, B);
}

template <class R, int W>
static bool adis_launch(lesgpu_case *c, const AdiBatch &B, int ncomp, long long mx, int nmax, bool capped) {
    const int m = (nmax + W - 1) / W;
    const long long lpb = 128 / W;
    dim3 grid((unsigned)((mx + lpb - 1) / lpb), (unsigned)ncomp);
    // up to 4 rows per lane the kernel fits the cap anyway
    if (m <= 2) k_adis<R, 2, W, 1><<<grid, 128, 0, c->stream>>>(c->kp, B);
    else if (m <= 4) k_adis<R, 4, W, 1><<<grid, 128, 0, c->stream>>>(c->kp, B);
    else if (m <= 8) {
        if (capped) k_adis<R, 8, W, 4><<<grid, 128, 0, c->stream>>>(c->kp, B);
        else k_adis<R, 8, W, 1><<<grid, 128, 0, c->stream>>>(c->kp, B);
    } else if (m <= 12) {
        if (capped) k_adis<R, 12, W, 4><<<grid, 128, 0, c->stream>>>(c->kp, B);
        else k_adis<R, 12, W, 1><<<grid, 128, 0, c->stream>>>(c->kp, B);
    } else {
        return false;
    }
    return true;
}

// One launch sweeps the same direction for up to three components at once
// (blockIdx.y = component): the u, v and w solves of lhsu/lhsv/lhsw are
// independent of each other, and three times the lines keep three times as
// many FP64 pipes busy on small grids.
//
// Lanes per line (W) of each sweep class -- 1 = one thread per line
// (k_adi), else the warp-scan form k_adis -- are picked by an autotuner: at
// the first start of a case of a given shape every feasible W is timed on the
// case's own sweeps (results redirected to scratch) and the fastest kept in a
// process-wide table, so later cases of the shape (the serving loop) reuse it.
// Mixed form: FP32 arithmetic for the x and z sweeps, the wall-normal
// (stretched) y sweep stays FP64.
struct AdiShape {
    long long mx;
    int nmax, ncomp;
    bool f32;
};

static AdiShape adi_shape(const lesgpu_case *c, const AdiBatch &B, int ncomp) {
    AdiShape h{0, 0, ncomp, c->cfg.precision == LESGPU_PREC_MIXED && B.a[0].dir != 1};
    for (int q = 0; q < ncomp; q++) {
        const AdiArgs &A = B.a[q];
        h.mx = std::max(h.mx, (long long)(A.a1 - A.a0 + 1) * (A.b1 - A.b0 + 1));
        h.nmax = std::max(h.nmax, A.l2 - A.l1 + 1);
    }
    return h;
}

// launch with W = w & 63 lanes per line (w & 64: the register-capped warp-scan
// kernel; w == kTiled: the tiled FP32 sweep); false if that form cannot take
// the batch (W cannot hold the line, MC <= 12; the tiled form needs FP32
// and factored coefficients)
constexpr int kTiled = 128;
static bool adi_run(lesgpu_case *c, const AdiBatch &B, const AdiShape &h, int wcode) {
    if (h.mx <= 0) return true;
    // factored coefficients unless a temperature sweep reads conjugate
    // tables that are not all 1
    const bool fac = !(B.a[0].comp == CT && c->kp.c.iconjg == 1 && c->conj_general);
    if (wcode == kTiled) {
        if (!h.f32 || !fac) return false;
        return adit_launch(c, B, h.ncomp, h.nmax);
    }
    const int w = wcode & 63;
    const bool capped = (wcode & 64) != 0;
    if (w <= 1) {
        // 128-thread blocks once the lines fill the GPU several times over,
        // single-warp blocks (more SMs busy) below that
        const int tpb = h.mx * h.ncomp >= 152LL * 512 ? 128 : 32;
        const dim3 grid((unsigned)((h.mx + tpb - 1) / tpb), (unsigned)h.ncomp);
        const int dir = B.a[0].dir;
        const bool per = B.a[0].periodic != 0;
        if (h.f32) k_adi_launch<float>(dir, per, fac, grid, tpb, c->stream, c->kp, B);
        else k_adi_launch<double>(dir, per, fac, grid, tpb, c->stream, c->kp, B);
        return true;
    }
    if (h.f32) {
        switch (w) {
        case 8: return adis_launch<float, 8>(c, B, h.ncomp, h.mx, h.nmax, capped);
        case 16: return adis_launch<float, 16>(c, B, h.ncomp, h.mx, h.nmax, capped);
        case 32: return adis_launch<float, 32>(c, B, h.ncomp, h.mx, h.nmax, capped);
        }
    } else {
        switch (w) {
        case 8: return adis_launch<double, 8>(c, B, h.ncomp, h.mx, h.nmax, capped);
        case 16: return adis_launch<double, 16>(c, B, h.ncomp, h.mx, h.nmax, capped);
        case 32: return adis_launch<double, 32>(c, B, h.ncomp, h.mx, h.nmax, capped);
        }
    }
    return false;
}

struct AdiTuneKey {
    int n1m, n2m, n3m, dir, ncomp, f32, periodic, nmax;
    bool operator<(const AdiTuneKey &o) const {
        const int a[8] = {n1m, n2m, n3m, dir, ncomp, f32, periodic, nmax};
        const int b[8] = {o.n1m, o.n2m, o.n3m, o.dir, o.ncomp, o.f32, o.periodic, o.nmax};
        return std::lexicographical_compare(a, a + 8, b, b + 8);
    }
};
static std::map<AdiTuneKey, int> g_adi_w;
static std::mutex g_adi_mu;

static AdiTuneKey adi_key(const lesgpu_case *c, const AdiBatch &B, const AdiShape &h) {
    const DGrid &g = c->kp.g;
    return AdiTuneKey{g.n1m, g.n2m, g.n3m, B.a[0].dir, h.ncomp, h.f32 ? 1 : 0, B.a[0].periodic, h.nmax};
}

// W used until a shape is tuned: the FP32 form 32 lanes; FP64 about 64k threads
static int adi_default_w(const AdiShape &h) {
    if (h.f32) return 32;
    const long long lines = h.mx * h.ncomp;
    int w = 1;
    while (w < 32 && lines * w < 65536) w <<= 1;
    return w < 8 ? 1 : w;
}

static void adi_launch(lesgpu_case *c, const AdiBatch &B, int ncomp) {
    const AdiShape h = adi_shape(c, B, ncomp);
    if (h.mx <= 0) return;
    int w = adi_default_w(h);
    if (c->autotune) {
        std::lock_guard<std::mutex> lk(g_adi_mu);
        auto it = g_adi_w.find(adi_key(c, B, h));
        if (it != g_adi_w.end()) w = it->second;
    }
    if (h.f32 && c->adi_force_f32) w = c->adi_force_f32;
    inst_begin(c, LESGPU_K_ADI);
    if (!adi_run(c, B, h, w)) adi_run(c, B, h, 1);
    inst_end(c, LESGPU_K_ADI);
}

// Time every feasible W of one sweep class with its results sent to scratch
// (z: in place on rhs -> the component's scratch G; x: adds into rhs, whose
// contents are dead between steps; y already writes G).
static void adi_tune_batch(lesgpu_case *c, AdiBatch B, int ncomp) {
    const AdiShape h = adi_shape(c, B, ncomp);
    if (h.mx <= 0) return;
    const AdiTuneKey key = adi_key(c, B, h);
    {
        std::lock_guard<std::mutex> lk(g_adi_mu);
        if (g_adi_w.count(key)) return;
    }
    DFields &f = c->kp.f;
    for (int q = 0; q < ncomp; q++) {
        AdiArgs &A = B.a[q];
        if (A.dir == 2) A.dst = f.scr[3 * q];
        else if (A.dir == 0) A.dst = f.rhs1[A.comp];
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    // the register-capped warp-scan variant only differs where a lane holds
    // more than 4 rows
    const int cand[8] = {1, 8, 16, 32, 8 | 64, 16 | 64, 32 | 64, kTiled};
    int best = adi_default_w(h);
    float best_ms = 3.0e38f;
    for (int q = 0; q < 8; q++) {
        if (cand[q] == kTiled && (!h.f32 || B.a[0].dir == 1)) continue;
        if (cand[q] != kTiled && (cand[q] & 64) && (h.nmax + (cand[q] & 63) - 1) / (cand[q] & 63) <= 4) continue;
        if (!adi_run(c, B, h, cand[q])) continue;          // warm-up launch (also the feasibility check)
        cudaEventRecord(e0, c->stream);
        for (int r = 0; r < 3; r++) adi_run(c, B, h, cand[q]);
        cudaEventRecord(e1, c->stream);
        float ms = 0.0f;
        if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) break;
        if (ms < best_ms) { best_ms = ms; best = cand[q]; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::lock_guard<std::mutex> lk(g_adi_mu);
    g_adi_w[key] = best;
}

// The three sweeps of one component (the structure of lhsu :1044-1148):
// z in place on rhs1, y into the scratch G, x added to the field.  Scratch
// arrays per component slot: G, factor, second vector.
static void adi_args(lesgpu_case *c, int comp, int slot, int dir, AdiArgs &A) {
    const DGrid &g = c->kp.g;
    const DCfg &cf = c->kp.c;
    DFields &f = c->kp.f;
    double *rhs = f.rhs1[comp];
    double *fld = comp == CU ? f.u : comp == CV ? f.v : comp == CW ? f.w : f.t;
    int ib = comp == CU ? g.i_bgpx : 1;
    int jb = comp == CV ? 2 : 1;
    int kb = comp == CW ? g.k_bgpz : 1;
    double *G = f.scr[3 * slot], *GAM = f.scr[3 * slot + 1], *SA = f.scr[3 * slot + 2];
    A = AdiArgs{};
    A.comp = comp;
    A.dir = dir;
    A.gam = GAM;
    A.sarr = SA;
    if (dir == 2) {
        A.periodic = cf.zprdic == 1;
        A.l1 = (comp == CW && !A.periodic) ? kb : 1;
        A.l2 = g.n3m;
        A.a0 = ib; A.a1 = g.n1m; A.b0 = jb; A.b1 = g.n2m;
        A.src = rhs; A.dst = rhs; A.add = 0;
    } else if (dir == 1) {
        A.periodic = 0;
        A.l1 = jb; A.l2 = g.n2m;
        A.a0 = ib; A.a1 = g.n1m; A.b0 = kb; A.b1 = g.n3m;
        A.src = rhs; A.dst = G; A.add = 0;
    } else {
        A.periodic = cf.xprdic == 1;
        A.l1 = ib; A.l2 = g.n1m;
        A.a0 = jb; A.a1 = g.n2m; A.b0 = kb; A.b1 = g.n3m;
        A.src = G; A.dst = fld; A.add = 1;
    }
}

static void adi_components(lesgpu_case *c, const int *comps, int n) {
    const DGrid &g = c->kp.g;
    for (int dir = 2; dir >= 0; dir--) {
        AdiBatch B{};
        int m = 0;
        for (int q = 0; q < n; q++) {
            // lhsu/lhsv skip their z sweep when n3m = 1 (lhsw is not called then)
            if (dir == 2 && comps[q] != CW && g.n3m == 1) continue;
            adi_args(c, comps[q], q, dir, B.a[m++]);
        }
        if (m) adi_launch(c, B, m);
    }
}

void launch_adi_uvw(lesgpu_case *c) {
    const int comps3[3] = {CU, CV, CW};
    adi_components(c, comps3, c->kp.g.n3m != 1 ? 3 : 2);
}

void launch_adi_t(lesgpu_case *c) {
    const int comps[1] = {CT};
    adi_components(c, comps, 1);
}

// The table can persist in a text file named by LESGPU_TUNE_FILE (one
// "adi n1m n2m n3m dir ncomp f32 periodic nmax lanes" line per class): read
// before tuning, rewritten after, so another process -- a profiler run of the
// same command, the compiled driver -- uses the same choices.
static void adi_table_load(const char *path) {
    FILE *f = fopen(path, "r");
    if (!f) return;
    char tag[16];
    AdiTuneKey k;
    int w;
    std::lock_guard<std::mutex> lk(g_adi_mu);
    while (fscanf(f, "%15s %d %d %d %d %d %d %d %d %d", tag, &k.n1m, &k.n2m, &k.n3m, &k.dir, &k.ncomp, &k.f32,
                  &k.periodic, &k.nmax, &w) == 10)
        if (!strcmp(tag, "adi") && !g_adi_w.count(k)) {
            const int wl = w & 63;    // lanes; + 64: the register-capped warp-scan kernel; 128: tiled
            if ((wl == 1 && w == 1) || ((wl == 8 || wl == 16 || wl == 32) && (w == wl || w == (wl | 64))) ||
                w == kTiled)
                g_adi_w[k] = w;
        }
    fclose(f);
}

static void adi_table_save(const char *path) {
    std::lock_guard<std::mutex> lk(g_adi_mu);
    FILE *f = fopen(path, "w");
    if (!f) return;
    for (const auto &kv : g_adi_w) {
        const AdiTuneKey &k = kv.first;
        fprintf(f, "adi %d %d %d %d %d %d %d %d %d\n", k.n1m, k.n2m, k.n3m, k.dir, k.ncomp, k.f32, k.periodic, k.nmax,
                kv.second);
    }
    fclose(f);
}

// Autotune the sweep classes of this case's shape (momentum and, with heat
// transfer, temperature); a no-op for shapes already tuned in this process.
int adi_autotune(lesgpu_case *c) {
    const char *tf = getenv("LESGPU_TUNE_FILE");
    if (tf && tf[0]) adi_table_load(tf);
    const DGrid &g = c->kp.g;
    const int comps3[3] = {CU, CV, CW};
    const int ct[1] = {CT};
    const int nm = g.n3m != 1 ? 3 : 2;
    for (int pass = 0; pass < (c->cfg.ihtrans == 1 ? 2 : 1); pass++) {
        const int *comps = pass == 0 ? comps3 : ct;
        const int n = pass == 0 ? nm : 1;
        for (int dir = 2; dir >= 0; dir--) {
            AdiBatch B{};
            int m = 0;
            for (int q = 0; q < n; q++) {
                if (dir == 2 && comps[q] != CW && g.n3m == 1) continue;
                adi_args(c, comps[q], q, dir, B.a[m++]);
            }
            if (m) adi_tune_batch(c, B, m);
        }
    }
    if (tf && tf[0]) adi_table_save(tf);
    return cudaStreamSynchronize(c->stream) == cudaSuccess ? 0 : LESGPU_ERR_CUDA;
}

// the autotuner's choices, for reports: "dir:ncomp:f32:W" per tuned class of this shape
int adi_tuned(const lesgpu_case *c, int *out, int maxn) {
    const DGrid &g = c->kp.g;
    std::lock_guard<std::mutex> lk(g_adi_mu);
    int n = 0;
    for (const auto &kv : g_adi_w) {
        const AdiTuneKey &k = kv.first;
        if (k.n1m != g.n1m || k.n2m != g.n2m || k.n3m != g.n3m || n + 4 > maxn) continue;
        out[n++] = k.dir; out[n++] = k.ncomp; out[n++] = k.f32; out[n++] = kv.second;
    }
    return n / 4;
}

}  // namespace lg

// Self-check of the FP64 pivot reciprocal (no reference counterpart): r[q] =
// rcp_pivot(x[q]) for n host values, so a test can bound its error.
namespace lg {
__global__ void k_rcp_check(const double *x, double *r, long long n) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) r[q] = rcp_pivot<double>(x[q]);
}
}  // namespace lg

extern "C" int lesgpu_check_rcp(const double *x, double *r, int64_t n) {
    if (n < 0 || (n > 0 && (!x || !r))) return LESGPU_ERR_ARG;
    if (n == 0) return 0;
    double *d = nullptr;
    if (cudaMalloc(&d, sizeof(double) * 2 * (size_t)n) != cudaSuccess) return LESGPU_ERR_OOM;
    int rc = 0;
    if (cudaMemcpy(d, x, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice) != cudaSuccess) rc = LESGPU_ERR_CUDA;
    if (!rc) {
        lg::k_rcp_check<<<(unsigned)((n + 255) / 256), 256>>>(d, d + n, (long long)n);
        if (cudaMemcpy(r, d + n, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost) != cudaSuccess) rc = LESGPU_ERR_CUDA;
    }
    cudaFree(d);
    return rc;
}
