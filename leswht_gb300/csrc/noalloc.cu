// Pressure Poisson solve (the poiss_ftft algorithm of k_fft.cu) for callers
// that cannot allocate device memory.
//
// Who needs this: code that runs where cudaMalloc is unavailable or not
// allowed -- a host runtime that hands out device memory only from its own
// pre-sized pool, a real-time loop that must not enter the driver's allocator
// (cudaMalloc can synchronise the device and take milliseconds), or a plugin
// loaded into a process whose allocator it must not bypass.  Such a caller
// owns its input and output buffers already; what it cannot provide is the
// solver's temporary memory.  This entry point keeps that temporary memory --
// the half spectrum, the elimination factors of the y-Thomas sweeps and the
// small wavenumber/metric/twiddle tables -- in one fixed file-scope device
// array, so it calls no cudaMalloc, cudaFree or other allocating routine.
//
// Limits and sharing
//   * The array holds kNoAllocScratchBytes (32 MiB) on every GPU that loads
//     this library, for the life of the process.  A grid needs
//     24 * n1m * (n3m/2+1) * n2m bytes plus a few KB of tables (64x64x64:
//     3.2 MiB; the largest cube that fits is about 128^3); each direction is
//     limited to 1024 cells.  Larger grids are rejected with
//     LESGPU_ERR_TOO_LARGE before any device work.
//   * Every call on a device uses the same array and leaves its contents
//     behind.  Nothing in it needs to start at zero: each call writes every
//     table, spectrum and factor it later reads.  Calls that overlap on the
//     GPU (two host threads, or two streams, on the same device) race on the
//     array and corrupt each other; serialise them.
//   * The first call on a device sets that device up: it resolves the
//     device address of the array (cudaGetSymbolAddress, with that device
//     current) and raises the FFT kernels' shared-memory limit.  That first
//     call must not be made while a stream of the device is being captured.
//   * A call copies nothing from host memory: the wavenumber and twiddle
//     tables are computed on the device by a first small kernel, and the
//     wall-normal metric and index tables reach it as kernel parameters, so
//     a call neither stages pageable host memory nor waits for the stream.
//   * The grid must be periodic and uniform in x and z (the transforms'
//     assumptions): a grid whose ipv(n1m) or kpv(n3m) does not wrap to 1, or
//     whose 1/dx or 1/dz varies by more than 1e-6 relative, is rejected with
//     LESGPU_ERR_UNSUPPORTED.
#include "k_fft.cuh"
#include <math.h>
#include <mutex>
#include <string.h>

namespace {

constexpr size_t kNoAllocScratchBytes = (size_t)32 << 20;
constexpr int kMaxDir = 1024;
constexpr int kMaxDevices = 64;

// The solver's scratch.  In host code `g_noalloc_scratch` is only a
// host-side handle of the symbol: its device address comes from
// cudaGetSymbolAddress (per device) and is what the kernels receive.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_mu;
std::mutex g_ymu;
void *g_base[kMaxDevices];

int setup_device(int dev, unsigned char **base) {
    if (dev < 0 || dev >= kMaxDevices) return LESGPU_ERR_ARG;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_base[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return LESGPU_ERR_CUDA;
        const int kMaxSmem = 200 * 1024;
        if (lg::fft_smem64(kMaxSmem)) return LESGPU_ERR_CUDA;
        g_base[dev] = p;
    }
    *base = (unsigned char *)g_base[dev];
    return 0;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

int plan_radices(int n, int *rad, int *nst) {
    *nst = 0;
    int m = n;
    while (m > 1) {
        int r;
        if (m % 4 == 0) r = 4;
        else if (m % 2 == 0) r = 2;
        else if (m % 3 == 0) r = 3;
        else if (m % 5 == 0) r = 5;
        else return LESGPU_ERR_UNSUPPORTED;
        if (*nst >= 24) return LESGPU_ERR_UNSUPPORTED;
        rad[(*nst)++] = r;
        m /= r;
    }
    return 0;
}


// The wall-normal tables of the solve, passed by value as kernel parameters:
// f2fyi(0:n2+1), c2cyi(0:n2+1) and jpv, fixjl, fixju over 0..n2m+1 (the
// unused ends zero), at most kMaxDir cells.  About 20.6 KB, below the 32 KB
// kernel-parameter limit of CUDA 12.1 and later.
struct YTables {
    double f2fyi[kMaxDir + 3], c2cyi[kMaxDir + 3];
    short jpv[kMaxDir + 2];
    unsigned char fixjl[kMaxDir + 2], fixju[kMaxDir + 2];
};

struct TableDst {
    double *ak1, *ak3, *f2fyi, *c2cyi;
    int *jpv, *fixjl, *fixju;
    double2 *twx, *twz;
};

// poisinit of poiss_ftft.f90:164-204 on the device: the modified wavenumbers
// ak1 = 2 (1 - cos(2 pi (i-1) / n1m)) / dx^2 (mirrored above n1mh) and
// ak3 likewise over z, the twiddles exp(-2 pi i e / n) of both transforms,
// and the y tables copied out of the parameter block.
__global__ void k_noalloc_tables(YTables y, TableDst d, int n1m, int n2m, int n3m, double sdxis, double sdzis) {
    const int n1mh = n1m / 2 + 1, n3mh = n3m / 2 + 1, n2 = n2m + 1;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < kMaxDir + 3; t += gridDim.x * blockDim.x) {
        if (t <= n1m + 2) {
            double v = 0.0;
            const int i = (t >= n1mh + 1 && t <= n1m) ? n1m + 2 - t : t;
            if (t >= 1 && t <= n1m) v = 2.0 * (1.0 - cospi(2.0 * (double)(i - 1) / (double)n1m)) * sdxis * sdxis;
            d.ak1[t] = v;
        }
        if (t <= n3mh + 1)
            d.ak3[t] = (t >= 1 && t <= n3mh) ? 2.0 * (1.0 - cospi(2.0 * (double)(t - 1) / (double)n3m)) * sdzis * sdzis : 0.0;
        if (t <= n2 + 1) { d.f2fyi[t] = y.f2fyi[t]; d.c2cyi[t] = y.c2cyi[t]; }
        if (t <= n2m + 1) { d.jpv[t] = y.jpv[t]; d.fixjl[t] = y.fixjl[t]; d.fixju[t] = y.fixju[t]; }
        double s, c;
        if (t < n1m) { sincospi(-2.0 * (double)t / (double)n1m, &s, &c); d.twx[t] = make_double2(c, s); }
        if (t < n3m) { sincospi(-2.0 * (double)t / (double)n3m, &s, &c); d.twz[t] = make_double2(c, s); }
    }
}

// x and z must wrap (ipv(n1m) = 1, kpv(n3m) = 1) and be uniform: every 1/dx
// within 1e-6 relative of the first, which the transforms use throughout.
bool periodic_uniform(const int64_t *pv, const double *fi, int nm) {
    if (pv[nm - 1] != 1) return false;
    const double f1 = fi[1];
    if (!(f1 > 0.0)) return false;
    for (int i = 1; i <= nm; i++)
        if (!(fabs(fi[i] - f1) <= 1e-6 * f1)) return false;
    return true;
}

}  // namespace

// See include/lesgpu.h.  Enqueues the solve on `stream` and returns; the
// caller synchronises before reading phi.
extern "C" int lesgpu_poisson_ftft_noalloc(const lesgpu_grid *g, const double *d_divgsum, double *d_phi, void *stream) {
    if (!g || !d_divgsum || !d_phi) return LESGPU_ERR_ARG;
    if (!g->ipv || !g->kpv || !g->jpv || !g->fixjl || !g->fixju || !g->f2fxi || !g->f2fzi || !g->f2fyi || !g->c2cyi)
        return LESGPU_ERR_ARG;
    if (g->n1 != g->n1m + 1 || g->n2 != g->n2m + 1 || g->n3 != g->n3m + 1) return LESGPU_ERR_ARG;
    if (g->n1m < 1 || g->n2m < 2 || g->n3m < 1) return LESGPU_ERR_ARG;
    if (g->n1m > kMaxDir || g->n2m > kMaxDir || g->n3m > kMaxDir) return LESGPU_ERR_TOO_LARGE;
    const int n1m = (int)g->n1m, n2m = (int)g->n2m, n3m = (int)g->n3m;
    const int n1 = n1m + 1, n2 = n2m + 1, n3mh = n3m / 2 + 1, n1mh = n1m / 2 + 1;
    if (!periodic_uniform(g->ipv, g->f2fxi, n1m) || !periodic_uniform(g->kpv, g->f2fzi, n3m))
        return LESGPU_ERR_UNSUPPORTED;
    lg::DevPlan px{}, pz{};
    if (plan_radices(n1m, px.rad, &px.nst) || plan_radices(n3m, pz.rad, &pz.nst)) return LESGPU_ERR_UNSUPPORTED;
    px.n = n1m;
    pz.n = n3m;
    lg::pack_radices(px);
    lg::pack_radices(pz);

    // layout of the scratch array
    const size_t nspec = (size_t)n1m * n3mh * n2m;
    size_t off = 0;
    const size_t o_ak1 = off; off = align256(off + sizeof(double) * (n1 + 2));
    const size_t o_ak3 = off; off = align256(off + sizeof(double) * (n3mh + 2));
    const size_t o_f2fyi = off; off = align256(off + sizeof(double) * (n2 + 2));
    const size_t o_c2cyi = off; off = align256(off + sizeof(double) * (n2 + 2));
    const size_t o_jpv = off; off = align256(off + sizeof(int) * (n2m + 2));
    const size_t o_fixjl = off; off = align256(off + sizeof(int) * (n2m + 2));
    const size_t o_fixju = off; off = align256(off + sizeof(int) * (n2m + 2));
    const size_t o_twx = off; off = align256(off + sizeof(double2) * n1m);
    const size_t o_twz = off; off = align256(off + sizeof(double2) * n3m);
    const size_t o_ccap = off; off = align256(off + sizeof(double2) * nspec);
    const size_t o_gam = off; off = align256(off + sizeof(double) * nspec);
    if (off > kNoAllocScratchBytes) return LESGPU_ERR_TOO_LARGE;

    // an error left pending by the caller's earlier work is theirs: return
    // without touching it rather than blame (and clear) it here
    if (cudaPeekAtLastError() != cudaSuccess) return LESGPU_ERR_CUDA;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return LESGPU_ERR_CUDA;
    unsigned char *base = nullptr;
    int rc = setup_device(dev, &base);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;

    // the wall-normal tables go to the device as kernel parameters (static:
    // the block is too large for a small thread stack; guarded by g_ymu until
    // the launch has copied it)
    static YTables y;
    std::lock_guard<std::mutex> lk(g_ymu);
    memset(&y, 0, sizeof(y));
    for (int j = 0; j <= n2; j++) { y.f2fyi[j] = g->f2fyi[j]; y.c2cyi[j] = g->c2cyi[j]; }
    for (int j = 1; j <= n2m; j++) {
        y.jpv[j] = (short)g->jpv[j - 1];
        y.fixjl[j] = (unsigned char)(g->fixjl[j - 1] != 0);
        y.fixju[j] = (unsigned char)(g->fixju[j - 1] != 0);
    }

    TableDst d;
    d.ak1 = (double *)(base + o_ak1);
    d.ak3 = (double *)(base + o_ak3);
    d.f2fyi = (double *)(base + o_f2fyi);
    d.c2cyi = (double *)(base + o_c2cyi);
    d.jpv = (int *)(base + o_jpv);
    d.fixjl = (int *)(base + o_fixjl);
    d.fixju = (int *)(base + o_fixju);
    d.twx = (double2 *)(base + o_twx);
    d.twz = (double2 *)(base + o_twz);
    k_noalloc_tables<<<(kMaxDir + 3 + 255) / 256, 256, 0, st>>>(y, d, n1m, n2m, n3m, g->f2fxi[1], g->f2fzi[1]);

    lg::KP p;
    memset(&p, 0, sizeof(p));
    p.g.n1 = n1; p.g.n2 = n2; p.g.n3 = n3m + 1;
    p.g.n1m = n1m; p.g.n2m = n2m; p.g.n3m = n3m; p.g.n1mh = n1mh; p.g.n3mh = n3mh;
    p.g.sx = n1 + 1; p.g.sxy = p.g.sx * (n2 + 1); p.g.nt = p.g.sxy * (n3m + 2);
    p.g.f2fyi = d.f2fyi;
    p.g.c2cyi = d.c2cyi;
    p.g.jpv = d.jpv;
    p.g.fixjl = d.fixjl;
    p.g.fixju = d.fixju;
    p.f.divgsum = (double *)d_divgsum;
    p.f.phi = d_phi;
    px.tw = d.twx;
    pz.tw = d.twz;
    px.twf = nullptr;   // FP64 transforms only
    pz.twf = nullptr;
    double2 *ccap = (double2 *)(base + o_ccap);
    double *gam = (double *)(base + o_gam);

    // the same launch sequence as the case-based solve (k_fft.cu launch_poisson)
    int Lz = lg::fft_lines_per_block(n3m), Lx = lg::fft_lines_per_block(n1m);
    size_t smz = (size_t)2 * n3m * Lz * sizeof(double2), smx = (size_t)2 * n1m * Lx * sizeof(double2);
    dim3 gz((n1m + 2 * Lz - 1) / (2 * Lz), n2m);   // 2 Lz real lines per block
    int nxl = n3mh * n2m;
    const long long sk = n1m, sj = (long long)n1m * n3mh;
    lg::fft_z_fwd64(gz, smz, st, p, p.f.divgsum, ccap, pz, Lz, sk, sj);
    lg::fft_x64((nxl + Lx - 1) / Lx, smx, st, ccap, nxl, px, Lx, 0);
    long long nl = (long long)n1m * n3mh;
    lg::k_ytri_elim<<<lg::blocks_for(nl, 128), 128, 0, st>>>(p, ccap, d.ak1, d.ak3, gam);
    lg::fft_x64((nxl + Lx - 1) / Lx, smx, st, ccap, nxl, px, Lx, 1);
    lg::fft_z_inv64(gz, smz, st, p, ccap, pz, Lz, sk, sj);
    // a launch that failed leaves its error pending; report it, leave it for the caller to see
    return cudaPeekAtLastError() == cudaSuccess ? 0 : LESGPU_ERR_CUDA;
}
