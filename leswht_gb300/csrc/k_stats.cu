// Running time averages of field_avg (misc_hist.f90:287-527): after each step
// with time > AVG_TST, dt-weighted sums of the cell-centre velocity, pressure,
// temperature, their products, the vorticity and S:S are added to
// LESGPU_NAVG accumulators.  One thread per cell reads the staggered
// neighbours once and updates the 21 (23 with temperature) sums in place.
#include "lesgpu_internal.cuh"

namespace lg {

__global__ void __launch_bounds__(kThreads) k_field_avg(KP p, Box b, double *avg) {
    const DGrid &g = p.g;
    const DScal *S = p.S;
    if (!(S->time > p.c.avg_tst)) return;          // field_avg returns while time <= AVG_TST
    const double dt = S->dt;
    const double *u = p.f.u, *v = p.f.v, *w = p.f.w, *pp = p.f.p, *t = p.f.t;
    const long long n = b.count(), nt = g.nt, sx = g.sx, sxy = g.sxy;
    const int n1 = g.n1, n2 = g.n2, n3 = g.n3;
    if (blockIdx.x == 0 && threadIdx.x == 0) p.S->avg_count += 1;
    for (long long tt = (long long)blockIdx.x * blockDim.x + threadIdx.x; tt < n; tt += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        b.at(tt, i, j, k);
        const long long q = g.ix(i, j, k);
        double *A = avg + q;
#define ACC(a, x) A[(long long)(a) * nt] = A[(long long)(a) * nt] + (x)
        const double ucc = 0.5 * (u[q] + u[q + 1]);
        const double vcc = 0.5 * (v[q] + v[q + sx]);
        const double wcc = 0.5 * (w[q] + w[q + sxy]);
        ACC(0, ucc * dt);
        ACC(1, vcc * dt);
        ACC(2, wcc * dt);
        ACC(3, ucc * ucc * dt);
        ACC(4, ucc * vcc * dt);
        ACC(5, ucc * wcc * dt);
        ACC(6, vcc * vcc * dt);
        ACC(7, vcc * wcc * dt);
        ACC(8, wcc * wcc * dt);
        ACC(9, pp[q] * dt);
        ACC(10, pp[q] * pp[q] * dt);
        if (p.c.ihtrans == 1) {
            ACC(21, t[q] * dt);
            ACC(22, t[q] * t[q] * dt);
        }
        // velocity gradients at the cell centre (misc_hist.f90:379-455)
        const double fju = fixd(g.fixju[j]), fjl = fixd(g.fixjl[j]);
        const double fku = fixd(g.fixku[k]), fkl = fixd(g.fixkl[k]);
        const double fiu = fixd(g.fixiu[i]), fil = fixd(g.fixil[i]);
        const double u0 = u[q], u1 = u[q + 1];
        const double vg11 = g.f2fxi[i] * (u1 - u0);
        double up = g.c2cyi[j + 1] * 0.25 * (g.f2fy[j + 1] * (u0 + u1) + g.f2fy[j] * (u[q + sx] + u[q + sx + 1])) * (1. - fju)
                    + 0.5 * (u[g.ix(i, n2, k)] + u[g.ix(i + 1, n2, k)]) * fju;
        double um = g.c2cyi[j] * 0.25 * (g.f2fy[j] * (u[q - sx] + u[q - sx + 1]) + g.f2fy[j - 1] * (u0 + u1)) * (1. - fjl)
                    + 0.5 * (u[g.ix(i, 0, k)] + u[g.ix(i + 1, 0, k)]) * fjl;
        const double vg12 = g.f2fyi[j] * (up - um);
        up = g.c2czi[k + 1] * 0.25 * (g.f2fz[k + 1] * (u0 + u1) + g.f2fz[k] * (u[q + sxy] + u[q + sxy + 1])) * (1. - fku)
             + 0.5 * (u[g.ix(i, j, n3)] + u[g.ix(i + 1, j, n3)]) * fku;
        um = g.c2czi[k] * 0.25 * (g.f2fz[k] * (u[q - sxy] + u[q - sxy + 1]) + g.f2fz[k - 1] * (u0 + u1)) * (1. - fkl)
             + 0.5 * (u[g.ix(i, j, 0)] + u[g.ix(i + 1, j, 0)]) * fkl;
        const double vg13 = g.f2fzi[k] * (up - um);
        const double v0 = v[q], v1 = v[q + sx];
        double vp = g.c2cxi[i + 1] * 0.25 * (g.f2fx[i + 1] * (v0 + v1) + g.f2fx[i] * (v[q + 1] + v[q + 1 + sx])) * (1. - fiu)
                    + 0.5 * (v[g.ix(n1, j, k)] + v[g.ix(n1, j + 1, k)]) * fiu;
        double vm = g.c2cxi[i] * 0.25 * (g.f2fx[i] * (v[q - 1] + v[q - 1 + sx]) + g.f2fx[i - 1] * (v0 + v1)) * (1. - fil)
                    + 0.5 * (v[g.ix(0, j, k)] + v[g.ix(0, j + 1, k)]) * fil;
        const double vg21 = g.f2fxi[i] * (vp - vm);
        const double vg22 = g.f2fyi[j] * (v1 - v0);
        vp = g.c2czi[k + 1] * 0.25 * (g.f2fz[k + 1] * (v0 + v1) + g.f2fz[k] * (v[q + sxy] + v[q + sx + sxy])) * (1. - fku)
             + 0.5 * (v[g.ix(i, j, n3)] + v[g.ix(i, j + 1, n3)]) * fku;
        vm = g.c2czi[k] * 0.25 * (g.f2fz[k] * (v[q - sxy] + v[q + sx - sxy]) + g.f2fz[k - 1] * (v0 + v1)) * (1. - fkl)
             + 0.5 * (v[g.ix(i, j, 0)] + v[g.ix(i, j + 1, 0)]) * fkl;
        const double vg23 = g.f2fzi[k] * (vp - vm);
        const double w0 = w[q], w1 = w[q + sxy];
        double wp = g.c2cxi[i + 1] * 0.25 * (g.f2fx[i + 1] * (w0 + w1) + g.f2fx[i] * (w[q + 1] + w[q + 1 + sxy])) * (1. - fiu)
                    + 0.5 * (w[g.ix(n1, j, k)] + w[g.ix(n1, j, k + 1)]) * fiu;
        double wm = g.c2cxi[i] * 0.25 * (g.f2fx[i] * (w[q - 1] + w[q - 1 + sxy]) + g.f2fx[i - 1] * (w0 + w1)) * (1. - fil)
                    + 0.5 * (w[g.ix(0, j, k)] + w[g.ix(0, j, k + 1)]) * fil;
        const double vg31 = g.f2fxi[i] * (wp - wm);
        wp = g.c2cyi[j + 1] * 0.25 * (g.f2fy[j + 1] * (w0 + w1) + g.f2fy[j] * (w[q + sx] + w[q + sx + sxy])) * (1. - fju)
             + 0.5 * (w[g.ix(i, n2, k)] + w[g.ix(i, n2, k + 1)]) * fju;
        wm = g.c2cyi[j] * 0.25 * (g.f2fy[j] * (w[q - sx] + w[q - sx + sxy]) + g.f2fy[j - 1] * (w0 + w1)) * (1. - fjl)
             + 0.5 * (w[g.ix(i, 0, k)] + w[g.ix(i, 0, k + 1)]) * fjl;
        const double vg32 = g.f2fyi[j] * (wp - wm);
        const double vg33 = g.f2fzi[k] * (w1 - w0);
        const double s1 = vg11, s2 = 0.5 * (vg12 + vg21), s3 = 0.5 * (vg13 + vg31);
        const double s4 = vg22, s5 = 0.5 * (vg23 + vg32), s6 = vg33;
        const double wx = vg32 - vg23, wy = vg13 - vg31, wz = vg21 - vg12;
        ACC(11, wx * dt);
        ACC(12, wy * dt);
        ACC(13, wz * dt);
        ACC(14, wx * wx * dt);
        ACC(15, wx * wy * dt);
        ACC(16, wx * wz * dt);
        ACC(17, wy * wy * dt);
        ACC(18, wy * wz * dt);
        ACC(19, wz * wz * dt);
        const double srsr = 2. * (s2 * s2) + s1 * s1 + 2. * (s3 * s3) + s4 * s4 + 2. * (s5 * s5) + s6 * s6;
        ACC(20, srsr * dt);
#undef ACC
    }
}

void launch_field_avg(lesgpu_case *c) {
    const DGrid &g = c->kp.g;
    Box b{1, 1, 1, g.n1m, g.n2m, g.n3m};
    k_field_avg<<<blocks_for(b.count()), kThreads, 0, c->stream>>>(c->kp, b, c->kp.f.avg);
}

}  // namespace lg
