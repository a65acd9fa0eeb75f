// Pressure Poisson solve of poiss_ftft.f90 (FFT in x and z, Thomas in y)
// with this library's own batched FFT.
//
// FFT: a Stockham auto-sort transform (Govindaraju et al., "High
// performance discrete Fourier transforms on graphics processors", SC'08)
// with radix-4/2/3/5 stages, executed by one thread block on a batch of L
// lines held in shared memory.  Lines are interleaved (element e of line l at
// e*L + l) so consecutive threads touch consecutive words.  Conventions are
// those of FFTE's ZFFT1D (zfft1d.f:18-84): forward = sum a_n exp(-2 pi i nk/N)
// unnormalised; inverse = exp(+...) scaled by 1/N.  Twiddles come from a
// table computed once on the host in long double.
//
// Data flow of one solve (spectrum ccap laid out i fastest, then k, then j):
//   k_fft_z_fwd : divgsum(i,j,:) real -> z-spectrum, keep modes 1..n3mh
//   k_fft_x     : complex x transform of every (k,j) line, in place
//   k_ytri      : complex Thomas along y for every (k,i) wavenumber pair,
//                 with the (1,1) mode pinned as poiss_ftft.f90:93-112
//   k_fft_x     : inverse x transform
//   k_fft_z_inv : conjugate-symmetric completion, inverse z, real part -> phi
#include "k_fft.cuh"
#include <math.h>
#include <stdlib.h>
#include <array>
#include <functional>
#include <map>
#include <mutex>
#include <vector>

namespace lg {

// complex arithmetic on double2 / float2 and the twiddle table of the type
template <class V> __device__ __forceinline__ V cmul(V a, V b) { return V{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
template <class V> __device__ __forceinline__ V cadd(V a, V b) { return V{a.x + b.x, a.y + b.y}; }
template <class V> __device__ __forceinline__ V csub(V a, V b) { return V{a.x - b.x, a.y - b.y}; }
template <class V> __device__ __forceinline__ const V *twid(const DevPlan &P);
template <> __device__ __forceinline__ const double2 *twid<double2>(const DevPlan &P) { return P.tw; }
template <> __device__ __forceinline__ const float2 *twid<float2>(const DevPlan &P) { return P.twf; }

// x / d for 0 <= x, 1 <= d and x d < 2^32 by one high multiply with
// m = ceil(2^32 / d): x m / 2^32 exceeds x / d by less than x / 2^32 < 1 / d,
// which never reaches the next integer.  (d = 1: m = 0, the quotient is x.)
// The index arithmetic of the transforms divides by run-time line counts and
// stage strides; an integer division costs some twenty instructions.
struct FastDiv {
    unsigned m;
    __device__ explicit FastDiv(int d) : m(d > 1 ? 0xFFFFFFFFu / (unsigned)d + 1u : 0u) {}
    __device__ int div(int x) const { return m ? (int)__umulhi((unsigned)x, m) : x; }
};

// One radix-R stage of block_fft on L interleaved lines, R a compile-time
// constant (the plans hold radices 4, 2, 3 and 5 only), so the butterfly and
// its loads, twiddles and stores unroll.  Twiddle index jm r twstep < Ns R
// N / (Ns R) = N: inside the table.
template <class V, int R>
__device__ __forceinline__ void fft_stage(const V *in, V *out, int L, const FastDiv &dL, int N, int Ns,
                                          const V *tw, int inv) {
    const int NR = N / R;
    const int twstep = N / (Ns * R);
    const int work = NR * L;
    const FastDiv dNs(Ns);
    for (int w = threadIdx.x; w < work; w += blockDim.x) {
        const int jb = dL.div(w), l = w - jb * L;
        const int jq = dNs.div(jb), jm = jb - jq * Ns;
        V v[R];
#pragma unroll
        for (int r = 0; r < R; r++) {
            V x = in[(jb + r * NR) * L + l];
            if (r > 0 && jm > 0) {
                V t = tw[jm * r * twstep];
                if (inv) t.y = -t.y;
                x = cmul(x, t);
            }
            v[r] = x;
        }
        V y[R];
        if constexpr (R == 2) {
            y[0] = cadd(v[0], v[1]);
            y[1] = csub(v[0], v[1]);
        } else if constexpr (R == 4) {
            V s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
            V s13 = cadd(v[1], v[3]), d13 = csub(v[1], v[3]);
            // forward: W4 = -i; inverse: +i
            V jd13 = inv ? V{-d13.y, d13.x} : V{d13.y, -d13.x};
            y[0] = cadd(s02, s13);
            y[2] = csub(s02, s13);
            y[1] = cadd(d02, jd13);
            y[3] = csub(d02, jd13);
        } else {
#pragma unroll
            for (int m = 0; m < R; m++) {
                V acc = v[0];
#pragma unroll
                for (int r = 1; r < R; r++) {
                    V t = tw[((m * r) % R) * NR];
                    if (inv) t.y = -t.y;
                    acc = cadd(acc, cmul(v[r], t));
                }
                y[m] = acc;
            }
        }
        const int idxD = jq * Ns * R + jm;
#pragma unroll
        for (int r = 0; r < R; r++) out[(idxD + r * Ns) * L + l] = y[r];
    }
}

// Run all stages on L interleaved lines; returns the buffer holding the result.
template <class V>
__device__ V *block_fft(V *b0, V *b1, int L, const DevPlan &P, int inv) {
    const int N = P.n;
    const V *tw = twid<V>(P);
    const FastDiv dL(L);
    int Ns = 1;
    V *in = b0, *out = b1;
    for (int st = 0; st < P.nst; st++) {
        const int code = (int)(P.radc >> (2 * st)) & 3;
        const int R = code == 0 ? 4 : code == 1 ? 2 : code == 2 ? 3 : 5;
        switch (R) {
        case 4: fft_stage<V, 4>(in, out, L, dL, N, Ns, tw, inv); break;
        case 2: fft_stage<V, 2>(in, out, L, dL, N, Ns, tw, inv); break;
        case 3: fft_stage<V, 3>(in, out, L, dL, N, Ns, tw, inv); break;
        default: fft_stage<V, 5>(in, out, L, dL, N, Ns, tw, inv); break;
        }
        __syncthreads();
        V *tmp = in; in = out; out = tmp;
        Ns *= R;
    }
    return in;
}

void pack_radices(DevPlan &d) {
    d.radc = 0ULL;
    for (int s = 0; s < d.nst && s < 24; s++) {
        const unsigned long long c = d.rad[s] == 4 ? 0ULL : d.rad[s] == 2 ? 1ULL : d.rad[s] == 3 ? 2ULL : 3ULL;
        d.radc |= c << (2 * s);
    }
}

DevPlan devplan(const FftPlan &p) {
    DevPlan d;
    d.n = p.n;
    d.nst = p.nst;
    for (int s = 0; s < 24; s++) d.rad[s] = p.rad[s];
    pack_radices(d);
    d.tw = p.tw;
    d.twf = p.twf;
    return d;
}

// ---- z transforms: block = (i-tile of 2L real lines) x j ------------------
// Two real lines share one complex transform (the two-for-one real FFT):
// c = a + i b, C = FFT(c), A_k = (C_k + conj C_{N-k}) / 2 and
// B_k = (C_k - conj C_{N-k}) / (2i); the inverse transforms X + i Y of two
// conjugate-symmetric spectra and takes x = Re, y = Im.  Half the transforms
// of the real z lines, each exact up to rounding (on GB300 the FP64 pipe, not
// memory, bounds these passes).  Line pair l holds i = i0 + 2l and i0 + 2l + 1.
template <class V>
__global__ void k_fft_z_fwd(KP p, const double *src, V *ccap, DevPlan P, int L, long long sk, long long sj) {
    using T = decltype(V{}.x);
    extern __shared__ __align__(16) unsigned char smraw[];
    V *sm = reinterpret_cast<V *>(smraw);
    const DGrid &g = p.g;
    const int N = P.n;
    V *b0 = sm, *b1 = sm + (size_t)N * L;
    const int i0 = 1 + blockIdx.x * 2 * L, j = 1 + blockIdx.y;
    const FastDiv d2L(2 * L);
    for (int w = threadIdx.x; w < N * 2 * L; w += blockDim.x) {
        const int e = d2L.div(w), l2 = w - e * 2 * L;       // consecutive threads: consecutive i
        const int i = i0 + l2;
        const T val = (i <= g.n1m) ? T(src[g.ix(i, j, e + 1)]) : T(0.0);
        T *slot = reinterpret_cast<T *>(&b0[e * L + (l2 >> 1)]);
        slot[l2 & 1] = val;
    }
    __syncthreads();
    const V *res = block_fft(b0, b1, L, P, 0);
    const int n3mh = g.n3mh;
    for (int w = threadIdx.x; w < n3mh * 2 * L; w += blockDim.x) {
        const int kk = d2L.div(w), l2 = w - kk * 2 * L;
        const int i = i0 + l2, l = l2 >> 1;
        if (i > g.n1m) continue;
        const V c = res[kk * L + l], cn = res[(kk == 0 ? 0 : N - kk) * L + l];
        // A_k = (C_k + conj C_{N-k}) / 2 ; B_k = -i (C_k - conj C_{N-k}) / 2
        const V v = (l2 & 1) ? V{T(0.5) * (c.y + cn.y), T(-0.5) * (c.x - cn.x)}
                             : V{T(0.5) * (c.x + cn.x), T(0.5) * (c.y - cn.y)};
        ccap[(i - 1) + sk * kk + sj * (j - 1)] = v;
    }
}

// ADD: phi += the result (the correction pass of the mixed form), else phi =
template <class V, bool ADD>
__global__ void k_fft_z_inv(KP p, const V *ccap, DevPlan P, int L, long long sk, long long sj) {
    using T = decltype(V{}.x);
    extern __shared__ __align__(16) unsigned char smraw[];
    V *sm = reinterpret_cast<V *>(smraw);
    const DGrid &g = p.g;
    const int N = P.n;
    V *b0 = sm, *b1 = sm + (size_t)N * L;
    const int i0 = 1 + blockIdx.x * 2 * L, j = 1 + blockIdx.y;
    const int n3mh = g.n3mh;
    // coefficient e of line i (conjugate completion above n3mh, poiss_ftft.f90:143-147);
    // the k = 0 and Nyquist coefficients enter through their real part only
    // (the reference takes Re of the inverse)
    auto coef = [&](int i, int e) -> V {
        if (i > g.n1m) return V{T(0.0), T(0.0)};
        if (e < n3mh) {
            V v = ccap[(i - 1) + sk * e + sj * (j - 1)];
            if (e == 0 || 2 * e == N) v.y = T(0.0);
            return v;
        }
        const V s = ccap[(i - 1) + sk * (N - e) + sj * (j - 1)];
        return V{s.x, -s.y};
    };
    const FastDiv dL(L), d2L(2 * L);
    for (int w = threadIdx.x; w < N * L; w += blockDim.x) {
        const int e = dL.div(w), l = w - e * L;
        const V x = coef(i0 + 2 * l, e), y = coef(i0 + 2 * l + 1, e);
        b0[e * L + l] = V{x.x - y.y, x.y + y.x};     // Z = X + i Y
    }
    __syncthreads();
    const V *res = block_fft(b0, b1, L, P, 1);
    const double dn = 1.0 / (double)N;
    for (int w = threadIdx.x; w < N * 2 * L; w += blockDim.x) {
        const int e = d2L.div(w), l2 = w - e * 2 * L;
        const int i = i0 + l2;
        if (i <= g.n1m) {
            const V r = res[e * L + (l2 >> 1)];
            const double v = (double)((l2 & 1) ? r.y : r.x) * dn;
            double &ph = p.f.phi[g.ix(i, j, e + 1)];
            ph = ADD ? ph + v : v;
        }
    }
}

// ---- x transforms of the (k,j) lines of ccap, in place -------------------
template <class V>
__global__ void k_fft_x(V *ccap, int nlines, DevPlan P, int L, int inv) {
    using T = decltype(V{}.x);
    extern __shared__ __align__(16) unsigned char smraw[];
    V *sm = reinterpret_cast<V *>(smraw);
    const int N = P.n;
    V *b0 = sm, *b1 = sm + (size_t)N * L;
    int line0 = blockIdx.x * L;
    const FastDiv dN(N);
    for (int w = threadIdx.x; w < N * L; w += blockDim.x) {
        int l = dN.div(w), e = w - l * N;   // coalesced global read along the line
        int line = line0 + l;
        b0[e * L + l] = (line < nlines) ? ccap[(size_t)line * N + e] : V{T(0.0), T(0.0)};
    }
    __syncthreads();
    V *res = block_fft(b0, b1, L, P, inv);
    const T dn = T(1.0 / (double)N);
    for (int w = threadIdx.x; w < N * L; w += blockDim.x) {
        int l = dN.div(w), e = w - l * N;
        int line = line0 + l;
        if (line < nlines) {
            V v = res[e * L + l];
            if (inv) { v.x *= dn; v.y *= dn; }
            ccap[(size_t)line * N + e] = v;
        }
    }
}

// ---- poiss_x_ft transforms (poiss_x_ft.f90:121-150, 182-232) ------------
// Forward: the real x lines of divgsum -> modes 1..n1mh, stored one z-y plane
// per mode, (k-1) + n3m*(j-1) + n3m*n2m*(iv-1).  Block = (k-tile of L lines)
// x j: lines are read along x (contiguous) and written along k.
__global__ void k_fft_xr_fwd(KP p, double2 *ccap, DevPlan P, int L) {
    extern __shared__ double2 sm[];
    const DGrid &g = p.g;
    const int N = P.n;
    double2 *b0 = sm, *b1 = sm + (size_t)N * L;
    const int k0 = 1 + blockIdx.x * L, j = 1 + blockIdx.y;
    for (int w = threadIdx.x; w < N * L; w += blockDim.x) {
        const int e = w % N, l = w / N;
        const int k = k0 + l;
        const double val = k <= g.n3m ? p.f.divgsum[g.ix(e + 1, j, k)] : 0.0;
        b0[e * L + l] = make_double2(val, 0.0);
    }
    __syncthreads();
    const double2 *res = block_fft<double2>(b0, b1, L, P, 0);
    const size_t plane = (size_t)g.n3m * g.n2m;
    for (int w = threadIdx.x; w < g.n1mh * L; w += blockDim.x) {
        const int l = w % L, iv = w / L;
        const int k = k0 + l;
        if (k <= g.n3m) ccap[(k - 1) + (size_t)g.n3m * (j - 1) + plane * iv] = res[iv * L + l];
    }
}

// Inverse: conjugate-symmetric completion over the modes, inverse x
// transform, real part -> phi.  With pin = 1 (ICH = 1) every block also
// transforms the line (j = n2m, k = 1) as its slot L and subtracts that
// line's f2fx-weighted mean, phiref = sum_i phi(i,n2m,1) f2fx(i) / xl, from
// what it stores: the sum is formed in one fixed order, so every block gets
// the same phiref and the reference's extra pass over phi is not needed.
__global__ void k_fft_xr_inv(KP p, const double2 *ccap, DevPlan P, int L, int pin) {
    extern __shared__ double2 sm[];
    __shared__ double s_ref;
    const DGrid &g = p.g;
    const int N = P.n, Ls = L + pin;
    double2 *b0 = sm, *b1 = sm + (size_t)N * Ls;
    const int k0 = 1 + blockIdx.x * L, j = 1 + blockIdx.y;
    const size_t plane = (size_t)g.n3m * g.n2m;
    for (int w = threadIdx.x; w < N * Ls; w += blockDim.x) {
        const int l = w % Ls, e = w / Ls;
        const int k = l < L ? k0 + l : 1, jj = l < L ? j : g.n2m;
        double2 val = make_double2(0.0, 0.0);
        if (k <= g.n3m) {
            const size_t base = (size_t)(k - 1) + (size_t)g.n3m * (jj - 1);
            if (e < g.n1mh) {
                val = ccap[base + plane * e];
            } else {
                // xxx(i) = conjg(ccap(k,j,n1m+2-i)), poiss_x_ft.f90:192-196
                const double2 s = ccap[base + plane * (N - e)];
                val = make_double2(s.x, -s.y);
            }
        }
        b0[e * Ls + l] = val;
    }
    __syncthreads();
    const double2 *res = block_fft<double2>(b0, b1, Ls, P, 1);
    const double dn = 1.0 / (double)N;
    double phiref = 0.0;
    if (pin) {
        if (threadIdx.x < 32) {
            double acc = 0.0;
            for (int e = threadIdx.x; e < N; e += 32) acc += __dmul_rn(res[e * Ls + L].x, dn) * g.f2fx[e + 1];
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
            if (threadIdx.x == 0) s_ref = acc / g.xl;
        }
        __syncthreads();
        phiref = s_ref;
    }
    for (int w = threadIdx.x; w < N * L; w += blockDim.x) {
        const int e = w % N, l = w / N;
        const int k = k0 + l;
        if (k <= g.n3m) p.f.phi[g.ix(e + 1, j, k)] = __dmul_rn(res[e * Ls + l].x, dn) - phiref;
    }
}

// lines per block of k_fft_xr_inv: L, or fewer if the extra line does not fit
int fft_xr_inv_lines(int n, int L, int pin) {
    while (L > 1 && (size_t)2 * n * (L + pin) * sizeof(double2) > (size_t)kFftSmemMax) L >>= 1;
    return L;
}

// ---- complex Thomas along y, ctrdiag (poiss_ftft.f90:207-244) ------------
__device__ __forceinline__ void ycoef(const DGrid &g, const double *ak1, const double *ak3, int i, int k, int j,
                                      double &am, double &ac, double &ap) {
    double fl = fixd(g.fixjl[j]), fu = fixd(g.fixju[j]);
    am = g.f2fyi[j] * g.c2cyi[j] * (1.0 - fl);
    ap = g.f2fyi[j] * g.c2cyi[g.jpv[j]] * (1.0 - fu);
    double akk = ak1[i] + ak3[k];
    ac = -((am + ap + akk) * (1.0 - fl) * (1.0 - fu) + (g.f2fyi[1] * g.c2cyi[2] + akk) * fl
           + (g.f2fyi[g.n2m] * g.c2cyi[g.n2m] + akk) * fu);
}

// Elimination and substitution in one pass (the allocation-free entry point,
// which keeps no per-case tables).
__global__ void k_ytri_elim(KP p, double2 *ccap, const double *ak1, const double *ak3, double *gam) {
    const DGrid &g = p.g;
    const int n1m = g.n1m, n2m = g.n2m, n3mh = g.n3mh;
    long long nl = (long long)n1m * n3mh;
    const long long sj = (long long)n1m * n3mh;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < nl; t += (long long)gridDim.x * blockDim.x) {
        int i = 1 + (int)(t % n1m), k = 1 + (int)(t / n1m);
        double2 *r = ccap + (i - 1) + (size_t)n1m * (k - 1);
        double *gm = gam + (i - 1) + (size_t)n1m * (k - 1);
        bool pin = (i == 1 && k == 1);
        double am, ac, ap;
        double ajcref = 0.0, ajmref = 0.0;
        double2 crhsref = make_double2(0.0, 0.0);
        if (pin) crhsref = r[(n2m - 1) * sj];
        // forward
        ycoef(g, ak1, ak3, i, k, 1, am, ac, ap);
        if (pin && n2m == 1) { ajcref = ac; ajmref = am; ac = 1.0; am = 0.0; ap = 0.0; }
        double bet = 1.0 / ac;
        double2 x = r[0];
        if (pin && n2m == 1) x = make_double2(0.0, 0.0);
        x.x *= bet; x.y *= bet;
        r[0] = x;
        double cprev = ap;
        for (int j = 2; j <= n2m; j++) {
            ycoef(g, ak1, ak3, i, k, j, am, ac, ap);
            double2 rj = r[(j - 1) * sj];
            if (pin && j == n2m) {
                ajcref = ac; ajmref = am;
                ac = 1.0; am = 0.0; ap = 0.0;
                rj = make_double2(0.0, 0.0);
            }
            double gj = cprev * bet;
            bet = 1.0 / (ac - am * gj);
            x = make_double2((rj.x - am * x.x) * bet, (rj.y - am * x.y) * bet);
            gm[(j - 1) * sj] = gj;
            r[(j - 1) * sj] = x;
            cprev = ap;
        }
        // backward
        double2 xn = x;
        for (int j = n2m - 1; j >= 1; j--) {
            double2 xj = r[(j - 1) * sj];
            double gn = gm[j * sj];
            xj = make_double2(xj.x - gn * xn.x, xj.y - gn * xn.y);
            r[(j - 1) * sj] = xj;
            xn = xj;
        }
        if (pin) {
            // phref = (-ajmref*crhs(n2m-1,1) + crhsref)/ajcref; shift; crhs(n2m,1) = 0
            double2 cm = n2m >= 2 ? r[(n2m - 2) * sj] : make_double2(0.0, 0.0);
            double2 ph = make_double2((-ajmref * cm.x + crhsref.x) / ajcref, (-ajmref * cm.y + crhsref.y) / ajcref);
            for (int j = 1; j <= n2m; j++) {
                double2 v = r[(j - 1) * sj];
                r[(j - 1) * sj] = make_double2(v.x - ph.x, v.y - ph.y);
            }
            r[(n2m - 1) * sj] = make_double2(0.0, 0.0);
        }
    }
}

// The y systems' LU (ctrdiag's forward pivots bet_j and multipliers gam_j)
// depends only on the grid and the wavenumber pair, so it is computed once per
// case by k_ytri_lu -- with the same device arithmetic as the reference's
// per-call elimination -- and every solve only substitutes.  Pivot tables are
// (i, k, j) with i fastest; yam holds am_j; pinref the (1,1) mode's
// (ajcref, ajmref) of poiss_ftft.f90:93-112.
__global__ void k_ytri_lu(KP p, const double *ak1, const double *ak3, double *ybet, double *ygam, double *yam,
                          double *pinref) {
    const DGrid &g = p.g;
    const int n1m = g.n1m, n2m = g.n2m, n3mh = g.n3mh;
    const long long nl = (long long)n1m * n3mh;
    const long long sj = nl;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < nl; t += (long long)gridDim.x * blockDim.x) {
        const int i = 1 + (int)(t % n1m), k = 1 + (int)(t / n1m);
        const bool pin = (i == 1 && k == 1);
        double am, ac, ap;
        ycoef(g, ak1, ak3, i, k, 1, am, ac, ap);
        if (t == 0) yam[1] = am;
        if (pin && n2m == 1) { pinref[0] = ac; pinref[1] = am; ac = 1.0; am = 0.0; ap = 0.0; }
        double bet = 1.0 / ac;
        ybet[t] = bet;
        double cprev = ap;
        for (int j = 2; j <= n2m; j++) {
            ycoef(g, ak1, ak3, i, k, j, am, ac, ap);
            if (t == 0) yam[j] = am;
            if (pin && j == n2m) { pinref[0] = ac; pinref[1] = am; ac = 1.0; am = 0.0; ap = 0.0; }
            const double gj = cprev * bet;
            bet = 1.0 / (ac - am * gj);
            ybet[t + (j - 1) * sj] = bet;
            ygam[t + (j - 1) * sj] = gj;
            cprev = ap;
        }
    }
}

// complex Thomas substitutions along y for every (k, i) pair, the (1,1) mode
// pinned as poiss_ftft.f90:93-112.  The coefficients are real, so the real
// and imaginary parts are independent recurrences: one thread each (twice
// the lines in flight); operands are loaded 8 rows ahead.
// S: the spectrum's storage and the arithmetic type: double, or float in the
// mixed form's FP32 solves (with FP32 copies of the LU tables), whose result
// the FP64 defect correction refines
template <class S>
__global__ void __launch_bounds__(64) k_ytri(KP p, S *ccap, const S *ybet, const S *ygam,
                                             const S *yam, const S *pinref) {
    const DGrid &g = p.g;
    const int n1m = g.n1m, n2m = g.n2m, n3mh = g.n3mh;
    const long long nl = (long long)n1m * n3mh;
    const long long sj = nl;
    constexpr int U = 8;
    for (long long tt = (long long)blockIdx.x * blockDim.x + threadIdx.x; tt < 2 * nl; tt += (long long)gridDim.x * blockDim.x) {
        const long long t = tt >> 1;
        const int part = (int)(tt & 1);
        S *r = ccap + 2 * t + part;                                   // element j at r[2 * (j-1) * sj]
        const long long s2 = 2 * sj;
        const bool pin = (t == 0);
        const S crhsref = pin ? r[(n2m - 1) * s2] : S(0.0);
        // forward: the next chunk's operands are loaded while one is computed
        // (two register buffers, alternated by unrolling the chunk loop by two)
        S x = S(0.0);
        S rA[U], bA[U], aA[U], rB[U], bB[U], aB[U];
        auto load_f = [&](S (&rv)[U], S (&bv)[U], S (&av)[U], int j0) {
#pragma unroll
            for (int u = 0; u < U; u++) {
                const int j = j0 + u;
                if (j <= n2m) { rv[u] = r[(j - 1) * s2]; bv[u] = ybet[t + (j - 1) * sj]; av[u] = yam[j]; }
            }
        };
        auto solve_f = [&](const S (&rv)[U], const S (&bv)[U], const S (&av)[U], int j0) {
#pragma unroll
            for (int u = 0; u < U; u++) {
                const int j = j0 + u;
                if (j > n2m) break;
                S rj = rv[u], am = av[u];
                if (pin && j == n2m) { am = S(0.0); rj = S(0.0); }
                x = (j == 1) ? rj * bv[u] : (rj - am * x) * bv[u];
                r[(j - 1) * s2] = x;
            }
        };
        load_f(rA, bA, aA, 1);
        for (int j0 = 1; j0 <= n2m; j0 += 2 * U) {
            if (j0 + U <= n2m) load_f(rB, bB, aB, j0 + U);
            solve_f(rA, bA, aA, j0);
            if (j0 + U > n2m) break;
            if (j0 + 2 * U <= n2m) load_f(rA, bA, aA, j0 + 2 * U);
            solve_f(rB, bB, aB, j0 + U);
        }
        // backward, pipelined the same way (the rows re-read here were written
        // above by this thread, so program order makes them visible)
        S xn = x;
        S xA[U], gA[U], xB[U], gB[U];
        auto load_b = [&](S (&xv)[U], S (&gv)[U], int j0) {
#pragma unroll
            for (int u = 0; u < U; u++) {
                const int j = j0 - u;
                if (j >= 1) { xv[u] = r[(j - 1) * s2]; gv[u] = ygam[t + j * sj]; }
            }
        };
        auto solve_b = [&](const S (&xv)[U], const S (&gv)[U], int j0) {
#pragma unroll
            for (int u = 0; u < U; u++) {
                const int j = j0 - u;
                if (j < 1) break;
                const S xj = xv[u] - gv[u] * xn;
                r[(j - 1) * s2] = xj;
                xn = xj;
            }
        };
        if (n2m >= 2) load_b(xA, gA, n2m - 1);
        for (int j0 = n2m - 1; j0 >= 1; j0 -= 2 * U) {
            if (j0 - U >= 1) load_b(xB, gB, j0 - U);
            solve_b(xA, gA, j0);
            if (j0 - U < 1) break;
            if (j0 - 2 * U >= 1) load_b(xA, gA, j0 - 2 * U);
            solve_b(xB, gB, j0 - U);
        }
        if (pin) {
            // phref = (-ajmref*crhs(n2m-1,1) + crhsref)/ajcref; shift; crhs(n2m,1) = 0
            const S ajcref = pinref[0], ajmref = pinref[1];
            const S cm = n2m >= 2 ? r[(n2m - 2) * s2] : S(0.0);
            const S ph = (-ajmref * cm + crhsref) / ajcref;
            for (int j = 1; j <= n2m; j++) r[(j - 1) * s2] = r[(j - 1) * s2] - ph;
            r[(n2m - 1) * s2] = S(0.0);
        }
    }
}

// FP64 -> FP32 copies of the y systems' LU tables
__global__ void k_to_f32(const double *a, float *b, long long n) {
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
        b[q] = (float)a[q];
}

// the LU tables of the y systems in the arithmetic type of k_ytri<T>
template <class T> struct YtriTabs { const T *bet, *gam, *am, *pin; };
template <class T> YtriTabs<T> ytri_tabs(const DPois &P);
template <> YtriTabs<double> ytri_tabs<double>(const DPois &P) { return {P.ybet, P.ygam, P.yam, P.pinref}; }
template <> YtriTabs<float> ytri_tabs<float>(const DPois &P) { return {P.ybetf, P.ygamf, P.yamf, P.pinreff}; }

// The mixed form's FP64 defect of the poiss_ftft system, r = divgsum - L phi,
// for the operator the transforms diagonalise (poiss_ftft.f90:79-88,
// :164-204): periodic second differences in x and z on the uniform spacings
// (-ak1, -ak3 in wavenumber space) and the y rows ajm, ajp with the walls'
// Neumann closure.  One FP32 solve of L e = r then corrects phi.
// yc[3 j .. 3 j + 2] = (ajm, ajp, 2 sdx^2 + 2 sdz^2 + ajm + ajp) of row j, so a
// cell costs a handful of FP64 operations (the FP64 pipe bounds this pass)
__global__ void __launch_bounds__(kThreads) k_pois_resid(KP p, Box b, const double *yc, double *res) {
    const DGrid &g = p.g;
    const double sdx = g.f2fxi[1], sdz = g.f2fzi[1];
    const double sx2 = sdx * sdx, sz2 = sdz * sdz;
    const long long n = b.count();
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        b.at(t, i, j, k);
        const long long q = g.ix(i, j, k);
        const double *phi = p.f.phi;
        const int ip = i < g.n1m ? i + 1 : 1, im = i > 1 ? i - 1 : g.n1m;
        const int kp = k < g.n3m ? k + 1 : 1, km = k > 1 ? k - 1 : g.n3m;
        const double am = yc[3 * j], ap = yc[3 * j + 1], dg = yc[3 * j + 2];
        const double ys = (j > 1 ? am * phi[q - g.sx] : 0.0) + (j < g.n2m ? ap * phi[q + g.sx] : 0.0);
        const double lap = sx2 * (phi[g.ix(ip, j, k)] + phi[g.ix(im, j, k)]) + sz2 * (phi[g.ix(i, j, kp)] + phi[g.ix(i, j, km)])
                         + ys - dg * phi[q];
        res[q] = p.f.divgsum[q] - lap;
    }
}

// ------------------------------------------------------------ host side
int make_plan(FftPlan &p, int n) {
    p.n = n;
    p.nst = 0;
    int m = n;
    while (m > 1) {
        int r;
        if (m % 4 == 0) r = 4;
        else if (m % 2 == 0) r = 2;
        else if (m % 3 == 0) r = 3;
        else if (m % 5 == 0) r = 5;
        else return LESGPU_ERR_UNSUPPORTED;      // FFTE supports 2^p 3^q 5^r only
        if (p.nst >= 24) return LESGPU_ERR_UNSUPPORTED;
        p.rad[p.nst++] = r;
        m /= r;
    }
    double2 *h = (double2 *)malloc(sizeof(double2) * (size_t)(n > 0 ? n : 1));
    float2 *hf = (float2 *)malloc(sizeof(float2) * (size_t)(n > 0 ? n : 1));
    for (int e = 0; e < n; e++) {
        long double ang = -2.0L * 3.14159265358979323846264338327950288L * (long double)e / (long double)n;
        h[e] = make_double2((double)cosl(ang), (double)sinl(ang));
        hf[e] = make_float2((float)cosl(ang), (float)sinl(ang));
    }
    if (cudaMalloc(&p.tw, sizeof(double2) * (size_t)n) != cudaSuccess ||
        cudaMalloc(&p.twf, sizeof(float2) * (size_t)n) != cudaSuccess) { free(h); free(hf); return LESGPU_ERR_OOM; }
    cudaMemcpy(p.tw, h, sizeof(double2) * (size_t)n, cudaMemcpyHostToDevice);
    cudaMemcpy(p.twf, hf, sizeof(float2) * (size_t)n, cudaMemcpyHostToDevice);
    free(h);
    free(hf);
    return 0;
}

static int lines_per_block(int n, size_t elem = sizeof(double2)) {
    int L = 32;
    while (L > 1 && (size_t)2 * n * L * elem > 200 * 1024) L >>= 1;
    return L;
}

int fft_lines_per_block(int n) { return lines_per_block(n); }
int fft_lz(const lesgpu_case *c) { return c->pois.Lz > 0 ? c->pois.Lz : lines_per_block(c->kp.g.n3m); }
int fft_lx(const lesgpu_case *c) { return c->pois.Lx > 0 ? c->pois.Lx : lines_per_block(c->kp.g.n1m); }

// ---- autotuner: lines per block of the z (and, for poiss_ftft, x) transforms.
// More lines per block make longer coalesced rows but take more shared memory
// (2 n L complex), hence fewer resident blocks; the best L depends on n and
// on the number of lines, so it is timed per shape (forward transforms on the
// case's own arrays, whose contents are scratch outside a solve) and cached.
static std::map<std::array<int, 4>, int> g_fft_l;

// LESGPU_FFT_MIXED: 1 = the mixed form always solves poiss_ftft with FP32
// transforms under the FP64 defect correction, 0 = always FP64; unset = timed
static int fft_mixed_forced() {
    const char *e = getenv("LESGPU_FFT_MIXED");
    if (!e || (e[0] != '0' && e[0] != '1')) return -1;
    return e[0] - '0';
}
static std::mutex g_fft_mu;

static int fft_time_pick(lesgpu_case *c, std::array<int, 4> key, int n, int dflt,
                         const std::function<void(int)> &run) {
    {
        std::lock_guard<std::mutex> lk(g_fft_mu);
        auto it = g_fft_l.find(key);
        if (it != g_fft_l.end()) return it->second;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int best = dflt;
    float best_ms = 3.0e38f;
    for (int L = 1; L <= 32; L <<= 1) {
        if ((size_t)2 * n * L * sizeof(double2) > 200 * 1024) break;
        run(L);                                  // warm-up
        cudaEventRecord(e0, c->stream);
        for (int r = 0; r < 3; r++) run(L);
        cudaEventRecord(e1, c->stream);
        float ms = 0.0f;
        if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) break;
        if (ms < best_ms) { best_ms = ms; best = L; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::lock_guard<std::mutex> lk(g_fft_mu);
    g_fft_l[key] = best;
    return best;
}

int fft_autotune(lesgpu_case *c) {
    const DGrid &g = c->kp.g;
    DPois &P = c->pois;
    const int pois = (int)c->cfg.poisson;
    if (pois == LESGPU_POISSON_MGRD) return 0;
    if (pois == LESGPU_POISSON_X_FT) {     // forward x transforms of the real lines
        const DevPlan px = devplan(P.fx);
        P.Lx = fft_time_pick(c, {2, g.n1m, g.n2m, g.n3m}, g.n1m, lines_per_block(g.n1m), [&](int L) {
            k_fft_xr_fwd<<<dim3((g.n3m + L - 1) / L, g.n2m), kThreads, (size_t)2 * g.n1m * L * sizeof(double2),
                           c->stream>>>(c->kp, P.ccap, px, L);
        });
        return cudaStreamSynchronize(c->stream) == cudaSuccess ? 0 : LESGPU_ERR_CUDA;
    }
    if (g.n3m <= 1) return 0;
    const DevPlan pz = devplan(P.fz);
    const bool ftft = pois == LESGPU_POISSON_FTFT;
    const long long sk = ftft ? g.n1m : (long long)g.n1m * g.n2m;
    const long long sj = ftft ? (long long)g.n1m * g.n3mh : g.n1m;
    P.Lz = fft_time_pick(c, {0, g.n1m, g.n2m, g.n3m}, g.n3m, lines_per_block(g.n3m), [&](int L) {
        const dim3 gz((g.n1m + 2 * L - 1) / (2 * L), g.n2m);   // 2L real lines per block
        k_fft_z_fwd<double2><<<gz, kThreads, (size_t)2 * g.n3m * L * sizeof(double2), c->stream>>>(c->kp, c->kp.f.divgsum, P.ccap, pz, L, sk, sj);
    });
    if (ftft) {
        const DevPlan px = devplan(P.fx);
        const int nxl = g.n3mh * g.n2m;
        P.Lx = fft_time_pick(c, {1, g.n1m, g.n2m, g.n3m}, g.n1m, lines_per_block(g.n1m), [&](int L) {
            k_fft_x<double2><<<(nxl + L - 1) / L, kThreads, (size_t)2 * g.n1m * L * sizeof(double2), c->stream>>>(P.ccap, nxl, px, L, 0);
        });
        // the mixed form: one FP64 solve, or two FP32 solves under an FP64
        // defect correction -- whichever is faster for the shape
        if (c->cfg.precision == LESGPU_PREC_MIXED && fft_mixed_forced() < 0) {
            cudaEvent_t e0, e1;
            cudaEventCreate(&e0);
            cudaEventCreate(&e1);
            float ms[2] = {0.0f, 0.0f};
            for (int v = 0; v < 2; v++) {
                P.mixed_fft = v;
                launch_poisson(c, 1);                 // warm-up
                cudaEventRecord(e0, c->stream);
                for (int r = 0; r < 3; r++) launch_poisson(c, 1);
                cudaEventRecord(e1, c->stream);
                if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms[v], e0, e1) != cudaSuccess)
                    ms[v] = 3.0e38f;
            }
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            P.mixed_fft = ms[1] < ms[0] ? 1 : 0;
        }
    }
    return cudaStreamSynchronize(c->stream) == cudaSuccess ? 0 : LESGPU_ERR_CUDA;
}

// poisinit, poiss_ftft.f90:164-204
int poisson_init(lesgpu_case *c) {
    const DGrid &g = c->kp.g;
    DPois &P = c->pois;
    if (c->cfg.poisson == LESGPU_POISSON_Z_FT || c->cfg.poisson == LESGPU_POISSON_X_FT) return mg2d_init(c);
    if (c->cfg.poisson == LESGPU_POISSON_MGRD) return mgrd_init(c);
    if (c->cfg.poisson != LESGPU_POISSON_FTFT) return LESGPU_ERR_UNSUPPORTED;
    if (c->cfg.xprdic != 1 || c->cfg.zprdic != 1) return LESGPU_ERR_CONFIG;
    // mixed form: FP32 transforms under the FP64 defect correction when forced
    // (LESGPU_FFT_MIXED) or, until the autotuner times both, on grids of 4M
    // cells and more (the FP64 transforms are FP64-pipe bound there)
    {
        const int forced = fft_mixed_forced();
        const bool mixed = c->cfg.precision == LESGPU_PREC_MIXED;
        P.mixed_fft = mixed && (forced == 1 || (forced < 0 && (long long)g.n1m * g.n2m * g.n3m >= (4LL << 20)));
    }
    int rc = make_plan(P.fx, g.n1m);
    if (rc) return rc;
    rc = make_plan(P.fz, g.n3m);
    if (rc) return rc;
    double pi = 2.0 * asin(1.0);
    double *ak1 = (double *)calloc(g.n1 + 2, sizeof(double));
    double *ak3 = (double *)calloc(g.n3mh + 2, sizeof(double));
    double sdzis = c->h_f2fz[1], sdxis = c->h_f2fx[1];
    for (int k = 1; k <= g.n3mh; k++) {
        double ai = (k == 1) ? 0.0 : (double)(k - 1) * 2.0 * pi;
        ak3[k] = 2.0 * (1.0 - cos(ai / (double)g.n3m)) * sdzis * sdzis;
    }
    for (int i = 1; i <= g.n1mh; i++) {
        double ai = (i == 1) ? 0.0 : (double)(i - 1) * 2.0 * pi;
        ak1[i] = 2.0 * (1.0 - cos(ai / (double)g.n1m)) * sdxis * sdxis;
    }
    for (int i = g.n1m; i >= g.n1mh + 1; i--) ak1[i] = ak1[g.n1m + 2 - i];
    if (cudaMalloc(&P.ak1, sizeof(double) * (g.n1 + 2)) != cudaSuccess) return LESGPU_ERR_OOM;
    if (cudaMalloc(&P.ak3, sizeof(double) * (g.n3mh + 2)) != cudaSuccess) return LESGPU_ERR_OOM;
    cudaMemcpy(P.ak1, ak1, sizeof(double) * (g.n1 + 2), cudaMemcpyHostToDevice);
    cudaMemcpy(P.ak3, ak3, sizeof(double) * (g.n3mh + 2), cudaMemcpyHostToDevice);
    free(ak1); free(ak3);
    size_t nspec = (size_t)g.n1m * g.n3mh * g.n2m;
    if (cudaMalloc(&P.ccap, sizeof(double2) * nspec) != cudaSuccess) return LESGPU_ERR_OOM;
    // LU of the y systems, fixed for the case
    if (cudaMalloc(&P.ybet, sizeof(double) * nspec) != cudaSuccess ||
        cudaMalloc(&P.ygam, sizeof(double) * nspec) != cudaSuccess ||
        cudaMalloc(&P.yam, sizeof(double) * (g.n2m + 2)) != cudaSuccess ||
        cudaMalloc(&P.pinref, sizeof(double) * 2) != cudaSuccess)
        return LESGPU_ERR_OOM;
    {   // the residual's y rows (poiss_ftft.f90:81-84) and diagonal
        const lesgpu_grid *hg = c->h_grid;
        const double sx2 = hg->f2fxi[1] * hg->f2fxi[1], sz2 = hg->f2fzi[1] * hg->f2fzi[1];
        std::vector<double> yc(3 * (size_t)(g.n2m + 2), 0.0);
        for (int j = 1; j <= g.n2m; j++) {
            const int jp = (int)hg->jpv[j - 1];
            const double am = hg->f2fyi[j] * hg->c2cyi[j] * (1.0 - (double)hg->fixjl[j - 1]);
            const double ap = hg->f2fyi[j] * hg->c2cyi[jp] * (1.0 - (double)hg->fixju[j - 1]);
            yc[3 * j] = am; yc[3 * j + 1] = ap; yc[3 * j + 2] = 2.0 * sx2 + 2.0 * sz2 + am + ap;
        }
        if (cudaMalloc(&P.yres, sizeof(double) * yc.size()) != cudaSuccess) return LESGPU_ERR_OOM;
        cudaMemcpy(P.yres, yc.data(), sizeof(double) * yc.size(), cudaMemcpyHostToDevice);
    }
    cudaMemset(P.ygam, 0, sizeof(double) * nspec);
    cudaMemset(P.pinref, 0, sizeof(double) * 2);
    {
        const long long nl = (long long)g.n1m * g.n3mh;
        k_ytri_lu<<<blocks_for(nl, 128), 128>>>(c->kp, P.ak1, P.ak3, P.ybet, P.ygam, P.yam, P.pinref);
        if (cudaDeviceSynchronize() != cudaSuccess) return LESGPU_ERR_CUDA;
    }
    // their FP32 copies, for the mixed form's FP32 solves
    if (c->cfg.precision == LESGPU_PREC_MIXED) {
        if (cudaMalloc(&P.ybetf, sizeof(float) * nspec) != cudaSuccess ||
            cudaMalloc(&P.ygamf, sizeof(float) * nspec) != cudaSuccess ||
            cudaMalloc(&P.yamf, sizeof(float) * (g.n2m + 2)) != cudaSuccess ||
            cudaMalloc(&P.pinreff, sizeof(float) * 2) != cudaSuccess)
            return LESGPU_ERR_OOM;
        k_to_f32<<<blocks_for((long long)nspec), kThreads>>>(P.ybet, P.ybetf, (long long)nspec);
        k_to_f32<<<blocks_for((long long)nspec), kThreads>>>(P.ygam, P.ygamf, (long long)nspec);
        k_to_f32<<<1, kThreads>>>(P.yam, P.yamf, (long long)(g.n2m + 2));
        k_to_f32<<<1, kThreads>>>(P.pinref, P.pinreff, 2LL);
        if (cudaDeviceSynchronize() != cudaSuccess) return LESGPU_ERR_CUDA;
    }
    // the attribute is per function and shared by every case: set it to the
    // largest size lines_per_block() can ask for
    if (cudaFuncSetAttribute(k_fft_z_fwd<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, kFftSmemMax) != cudaSuccess ||
        cudaFuncSetAttribute(k_fft_z_inv<double2, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kFftSmemMax) != cudaSuccess ||
        cudaFuncSetAttribute(k_fft_x<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, kFftSmemMax) != cudaSuccess ||
        cudaFuncSetAttribute(k_fft_z_fwd<float2>, cudaFuncAttributeMaxDynamicSharedMemorySize, kFftSmemMax) != cudaSuccess ||
        cudaFuncSetAttribute(k_fft_z_inv<float2, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kFftSmemMax) != cudaSuccess ||
        cudaFuncSetAttribute(k_fft_z_inv<float2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kFftSmemMax) != cudaSuccess ||
        cudaFuncSetAttribute(k_fft_x<float2>, cudaFuncAttributeMaxDynamicSharedMemorySize, kFftSmemMax) != cudaSuccess)
        return LESGPU_ERR_CUDA;
    return 0;
}

void poisson_free(lesgpu_case *c) {
    DPois &P = c->pois;
    mg2d_free(c);
    mgrd_free(c);
    cudaFree(P.ak1); cudaFree(P.ak3); cudaFree(P.ccap);
    cudaFree(P.ybet); cudaFree(P.ygam); cudaFree(P.yam); cudaFree(P.pinref); cudaFree(P.yres);
    cudaFree(P.ybetf); cudaFree(P.ygamf); cudaFree(P.yamf); cudaFree(P.pinreff);
    P.yres = nullptr;
    P.ybet = P.ygam = P.yam = P.pinref = nullptr;
    P.ybetf = P.ygamf = P.yamf = P.pinreff = nullptr;
    cudaFree(P.fx.tw); cudaFree(P.fz.tw); cudaFree(P.fx.twf); cudaFree(P.fz.twf);
    P.ak1 = P.ak3 = nullptr; P.ccap = nullptr; P.fx.tw = P.fz.tw = nullptr; P.fx.twf = P.fz.twf = nullptr;
}

// One poiss_ftft solve of L x = src on the transforms of type V (FP64, or FP32
// with FP64 y-Thomas arithmetic); ADD: phi += x, else phi = x.
template <class V, bool ADD>
static void ftft_solve(lesgpu_case *c, const double *src) {
    const DGrid &g = c->kp.g;
    DPois &P = c->pois;
    const DevPlan px = devplan(P.fx), pz = devplan(P.fz);
    // the FP64 transforms' lines per block (the FP32 blocks then take half the
    // shared memory, so more of them are resident)
    const int Lz = fft_lz(c), Lx = fft_lx(c);
    const size_t smz = (size_t)2 * g.n3m * Lz * sizeof(V), smx = (size_t)2 * g.n1m * Lx * sizeof(V);
    const dim3 gz((g.n1m + 2 * Lz - 1) / (2 * Lz), g.n2m);   // 2 Lz real lines per block
    const int nxl = g.n3mh * g.n2m;
    const long long sk = g.n1m, sj = (long long)g.n1m * g.n3mh;
    V *spec = reinterpret_cast<V *>(P.ccap);
    using T = decltype(V{}.x);
    k_fft_z_fwd<V><<<gz, kThreads, smz, c->stream>>>(c->kp, src, spec, pz, Lz, sk, sj);
    k_fft_x<V><<<(nxl + Lx - 1) / Lx, kThreads, smx, c->stream>>>(spec, nxl, px, Lx, 0);
    const long long nl = (long long)g.n1m * g.n3mh;
    const YtriTabs<T> yt = ytri_tabs<T>(P);
    k_ytri<T><<<blocks_for(2 * nl, 64), 64, 0, c->stream>>>(c->kp, reinterpret_cast<T *>(spec), yt.bet, yt.gam, yt.am, yt.pin);
    k_fft_x<V><<<(nxl + Lx - 1) / Lx, kThreads, smx, c->stream>>>(spec, nxl, px, Lx, 1);
    k_fft_z_inv<V, ADD><<<gz, kThreads, smz, c->stream>>>(c->kp, spec, pz, Lz, sk, sj);
}

void launch_poisson(lesgpu_case *c, int msub) {
    DPois &P = c->pois;
    if (c->cfg.poisson == LESGPU_POISSON_Z_FT || c->cfg.poisson == LESGPU_POISSON_X_FT) { launch_mg2d(c, msub); return; }
    if (c->cfg.poisson == LESGPU_POISSON_MGRD) { launch_mgrd(c, msub); return; }
    inst_begin(c, LESGPU_K_POISSON);
    if (P.mixed_fft) {
        // FP32 transforms under an FP64 defect correction: phi = S32 divgsum,
        // r = divgsum - L phi in FP64, phi += S32 r.  Each FP32 solve is within
        // ~1e-6 of the FP64 one in relative terms, so the correction leaves a
        // relative error of order 1e-12 (the constant of phi, which L does not
        // see, keeps the first solve's FP32 rounding).
        double *res = c->kp.f.scr[0];
        ftft_solve<float2, false>(c, c->kp.f.divgsum);
        const DGrid &g = c->kp.g;
        Box b{1, 1, 1, g.n1m, g.n2m, g.n3m};
        k_pois_resid<<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b, P.yres, res);
        ftft_solve<float2, true>(c, res);
    } else {
        ftft_solve<double2, false>(c, c->kp.f.divgsum);
    }
    inst_end(c, LESGPU_K_POISSON);
}

// FP64 launches for the other translation units
void fft_z_fwd64(dim3 grid, size_t smem, cudaStream_t st, KP p, const double *src, double2 *ccap, DevPlan P, int L,
                 long long sk, long long sj) {
    k_fft_z_fwd<double2><<<grid, kThreads, smem, st>>>(p, src, ccap, P, L, sk, sj);
}
void fft_z_inv64(dim3 grid, size_t smem, cudaStream_t st, KP p, const double2 *ccap, DevPlan P, int L, long long sk,
                 long long sj) {
    k_fft_z_inv<double2, false><<<grid, kThreads, smem, st>>>(p, ccap, P, L, sk, sj);
}
void fft_x64(int nblocks, size_t smem, cudaStream_t st, double2 *ccap, int nlines, DevPlan P, int L, int inv) {
    k_fft_x<double2><<<nblocks, kThreads, smem, st>>>(ccap, nlines, P, L, inv);
}
int fft_smem64(int bytes) {
    return (cudaFuncSetAttribute(k_fft_z_fwd<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) == cudaSuccess &&
            cudaFuncSetAttribute(k_fft_z_inv<double2, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) == cudaSuccess &&
            cudaFuncSetAttribute(k_fft_x<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) == cudaSuccess)
               ? 0 : LESGPU_ERR_CUDA;
}

}  // namespace lg
