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

// a and c of the element (i,j,k); b = diag - a - c.
__device__ __forceinline__ void adi_coef(const KP &p, int comp, int dir, int i, int j, int k, double &a, double &c) {
    const DGrid &g = p.g;
    const DFields &f = p.f;
    const double re = p.c.re;
    long long q = g.ix(i, j, k);
    if (comp == CT) {
        const double cre = (double)p.c.iles * re * p.c.pr;
        double cs = 1.0, ks1 = 1.0, ks2 = 1.0, omc = 1.0;
        int ka = dir == 2 ? 5 : dir == 1 ? 3 : 1;
        if (p.c.iconjg == 1) {
            cs = f.cstar[q];
            ks1 = f.kstar[ka][q];
            ks2 = f.kstar[ka - 1][q];
            omc = p.c.imovingon == 0 ? (double)f.omega[q] : 1.0;
        }
        if (dir == 2) {
            a = f.akuv[k] * (cs * ks1 + cre * omc * f.alsgs1[1][q]);
            c = f.ckuv[k] * (cs * ks2 + cre * omc * f.alsgs1[1][q + g.sxy]);
        } else if (dir == 1) {
            a = f.ajuw[j] * (cs * ks1 + cre * omc * f.alsgs1[2][q]);
            c = f.cjuw[j] * (cs * ks2 + cre * omc * f.alsgs1[2][q + g.sx]);
        } else {
            a = f.aivw[i] * (cs * ks1 + cre * omc * f.alsgs1[0][q]);
            c = f.civw[i] * (cs * ks2 + cre * omc * f.alsgs1[0][q + 1]);
        }
        return;
    }
    const double cre = (double)p.c.iles * re, cre2 = 2.0 * (double)p.c.iles * re;
    const double *nu = f.nusgs, *nu1 = f.nusgs1[0], *nu2 = f.nusgs1[1], *nu3 = f.nusgs1[2];
    switch (comp * 3 + dir) {
    case CU * 3 + 2: a = f.akuv[k] * (1.0 + cre * nu2[q]); c = f.ckuv[k] * (1.0 + cre * nu2[q + g.sxy]); break;
    case CU * 3 + 1: a = f.ajuw[j] * (1.0 + cre * nu3[q]); c = f.cjuw[j] * (1.0 + cre * nu3[q + g.sx]); break;
    case CU * 3 + 0: a = f.aiu[i] * (1.0 + cre2 * nu[q - 1]); c = f.ciu[i] * (1.0 + cre2 * nu[q]); break;
    case CV * 3 + 2: a = f.akuv[k] * (1.0 + cre * nu1[q]); c = f.ckuv[k] * (1.0 + cre * nu1[q + g.sxy]); break;
    case CV * 3 + 1: a = f.ajv[j] * (1.0 + cre2 * nu[q - g.sx]); c = f.cjv[j] * (1.0 + cre2 * nu[q]); break;
    case CV * 3 + 0: a = f.aivw[i] * (1.0 + cre * nu3[q]); c = f.civw[i] * (1.0 + cre * nu3[q + 1]); break;
    case CW * 3 + 2: a = f.akw[k] * (1.0 + cre2 * nu[q - g.sxy]); c = f.ckw[k] * (1.0 + cre2 * nu[q]); break;
    case CW * 3 + 1: a = f.ajuw[j] * (1.0 + cre * nu1[q]); c = f.cjuw[j] * (1.0 + cre * nu1[q + g.sx]); break;
    default:         a = f.aivw[i] * (1.0 + cre * nu2[q]); c = f.civw[i] * (1.0 + cre * nu2[q + 1]); break;
    }
}

// Elements per chunk: a thread issues the loads of CH consecutive line
// elements before it runs the (serial) recurrence over them, so CH loads are
// in flight instead of one.  Stores of a chunk follow all its loads, which
// keeps in-place sweeps (src == dst) correct.
constexpr int CH = 8;

struct AdiBatch {
    AdiArgs a[3];
};

__global__ void __launch_bounds__(64) k_adi(KP p, AdiBatch B) {
    const AdiArgs &A = B.a[blockIdx.y];
    const DGrid &g = p.g;
    const double diag = (A.comp == CT) ? p.S->acoefi * p.c.pr : p.S->acoefi;
    int na = A.a1 - A.a0 + 1, nb = A.b1 - A.b0 + 1;
    long long nl = (long long)na * nb;
    const long long stride = A.dir == 2 ? g.sxy : A.dir == 1 ? g.sx : 1;
    const int nline = A.l2 - A.l1 + 1;
    if (nl <= 0 || A.l2 < A.l1) return;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < nl; t += (long long)gridDim.x * blockDim.x) {
        const int x0 = A.a0 + (int)(t % na), x1 = A.b0 + (int)(t / na);
        int i0, j0, k0;
        line_coords(A.dir, A.l1, x0, x1, i0, j0, k0);
        const long long q0 = g.ix(i0, j0, k0);
        if (!A.periodic) {
            // ---- trdiag: forward elimination, chunk by chunk
            double *out = A.add ? A.sarr : A.dst;    // provisional solution
            double bet = 0.0, x = 0.0, cprev = 0.0;
            for (int c0 = 0; c0 < nline; c0 += CH) {
                double av[CH], cv[CH], rv[CH];
#pragma unroll
                for (int u = 0; u < CH; u++) {
                    if (c0 + u < nline) {
                        int i, j, k;
                        line_coords(A.dir, A.l1 + c0 + u, x0, x1, i, j, k);
                        adi_coef(p, A.comp, A.dir, i, j, k, av[u], cv[u]);
                        rv[u] = A.src[q0 + (long long)(c0 + u) * stride];
                    }
                }
#pragma unroll
                for (int u = 0; u < CH; u++) {
                    if (c0 + u < nline) {
                        const long long q = q0 + (long long)(c0 + u) * stride;
                        const double a = av[u], c = cv[u];
                        const double b = diag - a - c;
                        if (c0 + u == 0) {
                            bet = 1.0 / b;
                            x = diag * rv[u] * bet;
                        } else {
                            const double gm = cprev * bet;
                            bet = 1.0 / (b - a * gm);
                            x = (diag * rv[u] - a * x) * bet;
                            A.gam[q] = gm;
                        }
                        out[q] = x;
                        cprev = c;
                    }
                }
            }
            // ---- back substitution, chunk by chunk from the end
            double xn = x;
            const long long qlast = q0 + (long long)(nline - 1) * stride;
            if (A.add) A.dst[qlast] += xn;
            for (int c1 = nline - 2; c1 >= 0; c1 -= CH) {
                double ov[CH], gv[CH], fv[CH];
#pragma unroll
                for (int u = 0; u < CH; u++) {
                    const int l = c1 - u;
                    if (l >= 0) {
                        const long long q = q0 + (long long)l * stride;
                        ov[u] = out[q];
                        gv[u] = A.gam[q + stride];
                        if (A.add) fv[u] = A.dst[q];
                    }
                }
#pragma unroll
                for (int u = 0; u < CH; u++) {
                    const int l = c1 - u;
                    if (l >= 0) {
                        const long long q = q0 + (long long)l * stride;
                        const double xl = ov[u] - gv[u] * xn;
                        if (A.add) A.dst[q] = fv[u] + xl;
                        else out[q] = xl;
                        xn = xl;
                    }
                }
            }
        } else {
            // ---- trdiagp: forward sweep; q factors in gam, s in sarr, f in fw
            double *fw = A.add ? (double *)A.src : A.dst;
            const long long qn_last = q0 + (long long)(nline - 1) * stride;
            const double fn = diag * A.src[qn_last];   // original right-hand side at the last element
            double qq = 0.0, ss = 0.0, ff = 0.0;
            double a_last = 0.0, b_last = 0.0, c_last = 0.0;
            for (int c0 = 0; c0 < nline; c0 += CH) {
                double av[CH], cv[CH], rv[CH];
#pragma unroll
                for (int u = 0; u < CH; u++) {
                    if (c0 + u < nline) {
                        int i, j, k;
                        line_coords(A.dir, A.l1 + c0 + u, x0, x1, i, j, k);
                        adi_coef(p, A.comp, A.dir, i, j, k, av[u], cv[u]);
                        rv[u] = A.src[q0 + (long long)(c0 + u) * stride];
                    }
                }
#pragma unroll
                for (int u = 0; u < CH; u++) {
                    if (c0 + u < nline) {
                        const long long q = q0 + (long long)(c0 + u) * stride;
                        const double a = av[u], c = cv[u];
                        const double b = diag - a - c;
                        if (c0 + u == 0) {
                            const double binv = 1.0 / b;
                            qq = -c * binv;
                            ss = -a * binv;
                            ff = diag * rv[u] * binv;
                        } else {
                            const double pn = 1.0 / (b + a * qq);
                            const double qn = -c * pn;
                            const double sn = -a * ss * pn;
                            ff = (diag * rv[u] - a * ff) * pn;
                            qq = qn;
                            ss = sn;
                        }
                        A.gam[q] = qq;
                        A.sarr[q] = ss;
                        fw[q] = ff;
                        a_last = a; b_last = b; c_last = c;
                    }
                }
            }
            // backward pass: s(j) += q(j) s(j+1); qe(j) = f(j) + q(j) qe(j+1)
            double s_next = 1.0, qe_next = 0.0, s_j2m1 = 0.0, qe_j2m1 = 0.0;
            for (int c1 = nline - 2; c1 >= 0; c1 -= CH) {
                double qv[CH], sv[CH], fv[CH];
#pragma unroll
                for (int u = 0; u < CH; u++) {
                    const int l = c1 - u;
                    if (l >= 0) {
                        const long long q = q0 + (long long)l * stride;
                        qv[u] = A.gam[q];
                        sv[u] = A.sarr[q];
                        fv[u] = fw[q];
                    }
                }
#pragma unroll
                for (int u = 0; u < CH; u++) {
                    const int l = c1 - u;
                    if (l >= 0) {
                        const long long q = q0 + (long long)l * stride;
                        const double sj = sv[u] + qv[u] * s_next;
                        const double qej = fv[u] + qv[u] * qe_next;
                        A.sarr[q] = sj;
                        fw[q] = qej;
                        if (l == nline - 2) { s_j2m1 = sj; qe_j2m1 = qej; }
                        s_next = sj;
                        qe_next = qej;
                    }
                }
            }
            const double s_j1 = s_next, qe_j1 = qe_next;
            const double fj2 = (fn - c_last * qe_j1 - a_last * qe_j2m1) / (c_last * s_j1 + a_last * s_j2m1 + b_last);
            if (A.add) A.dst[qn_last] += fj2; else fw[qn_last] = fj2;
            for (int c1 = nline - 2; c1 >= 0; c1 -= CH) {
                double sv[CH], ev[CH], dv[CH];
#pragma unroll
                for (int u = 0; u < CH; u++) {
                    const int l = c1 - u;
                    if (l >= 0) {
                        const long long q = q0 + (long long)l * stride;
                        sv[u] = A.sarr[q];
                        ev[u] = fw[q];
                        if (A.add) dv[u] = A.dst[q];
                    }
                }
#pragma unroll
                for (int u = 0; u < CH; u++) {
                    const int l = c1 - u;
                    if (l >= 0) {
                        const long long q = q0 + (long long)l * stride;
                        const double val = fj2 * sv[u] + ev[u];
                        if (A.add) A.dst[q] = dv[u] + val; else fw[q] = val;
                    }
                }
            }
        }
    }
}

// One launch sweeps the same direction for up to three components at once
// (blockIdx.y = component): the u, v and w solves of lhsu/lhsv/lhsw are
// independent of each other, and three times the lines keep three times as
// many FP64 pipes busy on small grids.
static void adi_launch(lesgpu_case *c, const AdiBatch &B, int ncomp) {
    long long mx = 0;
    for (int q = 0; q < ncomp; q++) {
        const AdiArgs &A = B.a[q];
        long long nl = (long long)(A.a1 - A.a0 + 1) * (A.b1 - A.b0 + 1);
        if (nl > mx) mx = nl;
    }
    if (mx <= 0) return;
    dim3 grid((unsigned)((mx + 31) / 32), (unsigned)ncomp);
    inst_begin(c, LESGPU_K_ADI);
    k_adi<<<grid, 32, 0, c->stream>>>(c->kp, B);
    inst_end(c, LESGPU_K_ADI);
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

}  // namespace lg
