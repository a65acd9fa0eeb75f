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

__global__ void __launch_bounds__(128) k_adi(KP p, AdiArgs A) {
    const DGrid &g = p.g;
    const double diag = (A.comp == CT) ? p.S->acoefi * p.c.pr : p.S->acoefi;
    int na = A.a1 - A.a0 + 1, nb = A.b1 - A.b0 + 1;
    long long nl = (long long)na * nb;
    long long stride = A.dir == 2 ? g.sxy : A.dir == 1 ? g.sx : 1;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < nl; t += (long long)gridDim.x * blockDim.x) {
        int x0 = A.a0 + (int)(t % na), x1 = A.b0 + (int)(t / na);
        int i, j, k;
        line_coords(A.dir, A.l1, x0, x1, i, j, k);
        long long q0 = g.ix(i, j, k);
        if (!A.periodic) {
            // ---- trdiag: forward elimination
            double a, c;
            adi_coef(p, A.comp, A.dir, i, j, k, a, c);
            double b = diag - a - c;
            double bet = 1.0 / b;
            double x = diag * A.src[q0] * bet;
            double cprev = c;
            double *out = A.add ? A.gam + 0 : A.dst;   // solution holder during the sweep
            // when adding to the field the provisional solution lives in sarr
            if (A.add) out = A.sarr;
            out[q0] = x;
            long long q = q0;
            for (int l = A.l1 + 1; l <= A.l2; l++) {
                q += stride;
                line_coords(A.dir, l, x0, x1, i, j, k);
                adi_coef(p, A.comp, A.dir, i, j, k, a, c);
                b = diag - a - c;
                double gm = cprev * bet;
                bet = 1.0 / (b - a * gm);
                x = (diag * A.src[q] - a * x) * bet;
                A.gam[q] = gm;
                out[q] = x;
                cprev = c;
            }
            // ---- back substitution
            double xn = x;
            if (A.add) A.dst[q] += xn;
            for (int l = A.l2 - 1; l >= A.l1; l--) {
                long long qn = q;
                q -= stride;
                double xl = out[q] - A.gam[qn] * xn;
                if (A.add) A.dst[q] += xl;
                else out[q] = xl;
                xn = xl;
            }
        } else {
            // ---- trdiagp: forward sweep (q in gam, s in sarr, f in dst/work)
            double *f = A.add ? nullptr : A.dst;
            double a, c;
            adi_coef(p, A.comp, A.dir, i, j, k, a, c);
            double b = diag - a - c;
            long long q = q0;
            long long qn_last = q0 + (long long)(A.l2 - A.l1) * stride;
            double fn;
            {
                // original right-hand side at the last element
                fn = diag * A.src[qn_last];
            }
            double binv = 1.0 / b;
            double qq = -c * binv, ss = -a * binv;
            double ff = diag * A.src[q0] * binv;
            // when adding to the field, the f/qe vector lives in a private
            // region of dst's companion: reuse the src array only if it is a
            // scratch (x sweeps read the y-sweep result G, which is private)
            double *fw = A.add ? (double *)A.src : f;
            A.gam[q] = qq;
            A.sarr[q] = ss;
            fw[q] = ff;
            double a_last = 0.0, b_last = 0.0, c_last = 0.0;
            for (int l = A.l1 + 1; l <= A.l2; l++) {
                q += stride;
                line_coords(A.dir, l, x0, x1, i, j, k);
                adi_coef(p, A.comp, A.dir, i, j, k, a, c);
                b = diag - a - c;
                double pn = 1.0 / (b + a * qq);
                double qn = -c * pn;
                double sn = -a * ss * pn;
                double fnw = (diag * A.src[q] - a * ff) * pn;
                qq = qn; ss = sn; ff = fnw;
                A.gam[q] = qq;
                A.sarr[q] = ss;
                fw[q] = ff;
                a_last = a; b_last = b; c_last = c;
            }
            // backward pass: s(j) += q(j) s(j+1); qe(j) = f(j) + q(j) qe(j+1)
            double s_next = 1.0, qe_next = 0.0;
            double s_j2m1 = 0.0, qe_j2m1 = 0.0;
            long long qe_pos = qn_last;
            for (int l = A.l2 - 1; l >= A.l1; l--) {
                qe_pos -= stride;
                double qj = A.gam[qe_pos];
                double sj = A.sarr[qe_pos] + qj * s_next;
                double qej = fw[qe_pos] + qj * qe_next;
                A.sarr[qe_pos] = sj;
                fw[qe_pos] = qej;
                if (l == A.l2 - 1) { s_j2m1 = sj; qe_j2m1 = qej; }
                s_next = sj; qe_next = qej;
            }
            double s_j1 = s_next, qe_j1 = qe_next;
            double fj2 = (fn - c_last * qe_j1 - a_last * qe_j2m1) / (c_last * s_j1 + a_last * s_j2m1 + b_last);
            if (A.add) A.dst[qn_last] += fj2; else fw[qn_last] = fj2;
            long long qp = qn_last;
            for (int l = A.l2 - 1; l >= A.l1; l--) {
                qp -= stride;
                double val = fj2 * A.sarr[qp] + fw[qp];
                if (A.add) A.dst[qp] += val; else fw[qp] = val;
            }
        }
    }
}

static void adi_launch(lesgpu_case *c, const AdiArgs &A) {
    long long nl = (long long)(A.a1 - A.a0 + 1) * (A.b1 - A.b0 + 1);
    if (nl <= 0 || A.l2 < A.l1) return;
    int nb = (int)((nl + 127) / 128);
    inst_begin(c, LESGPU_K_ADI);
    k_adi<<<nb, 128, 0, c->stream>>>(c->kp, A);
    inst_end(c, LESGPU_K_ADI);
}

// One component: z sweep in place on rhs1, y sweep into scratch G, x sweep
// added to the field (the structure of lhsu :1044-1148).
static void adi_component(lesgpu_case *c, int comp) {
    const DGrid &g = c->kp.g;
    const DCfg &cf = c->kp.c;
    DFields &f = c->kp.f;
    double *rhs = f.rhs1[comp];
    double *fld = comp == CU ? f.u : comp == CV ? f.v : comp == CW ? f.w : f.t;
    int ib = comp == CU ? g.i_bgpx : 1;
    int jb = comp == CV ? 2 : 1;
    int kb = comp == CW ? g.k_bgpz : 1;
    double *G = f.scr[0], *GAM = f.scr[1], *SA = f.scr[2];
    bool zsweep = (comp == CW) || g.n3m != 1;
    if (zsweep) {
        AdiArgs A{};
        A.comp = comp; A.dir = 2;
        A.periodic = cf.zprdic == 1;
        A.l1 = (comp == CW && !A.periodic) ? 2 : 1;
        if (comp == CW && !A.periodic) A.l1 = kb;
        A.l2 = g.n3m;
        A.a0 = ib; A.a1 = g.n1m; A.b0 = jb; A.b1 = g.n2m;
        A.src = rhs; A.dst = rhs; A.add = 0; A.gam = GAM; A.sarr = SA;
        adi_launch(c, A);
    }
    {
        AdiArgs A{};
        A.comp = comp; A.dir = 1; A.periodic = 0;
        A.l1 = jb; A.l2 = g.n2m;
        A.a0 = ib; A.a1 = g.n1m; A.b0 = kb; A.b1 = g.n3m;
        A.src = rhs; A.dst = G; A.add = 0; A.gam = GAM; A.sarr = SA;
        adi_launch(c, A);
    }
    {
        AdiArgs A{};
        A.comp = comp; A.dir = 0; A.periodic = cf.xprdic == 1;
        A.l1 = ib; A.l2 = g.n1m;
        A.a0 = jb; A.a1 = g.n2m; A.b0 = kb; A.b1 = g.n3m;
        A.src = G; A.dst = fld; A.add = 1; A.gam = GAM; A.sarr = SA;
        adi_launch(c, A);
    }
}

void launch_adi_uvw(lesgpu_case *c) {
    adi_component(c, CU);
    adi_component(c, CV);
    if (c->kp.g.n3m != 1) adi_component(c, CW);
}

void launch_adi_t(lesgpu_case *c) { adi_component(c, CT); }

}  // namespace lg
