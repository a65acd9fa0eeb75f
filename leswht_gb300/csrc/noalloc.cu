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
//     current) and raises the FFT kernels' shared-memory limit.  Make that
//     first call before any stream capture on the device.
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

}  // namespace

// See include/lesgpu.h.  Enqueues the solve on `stream` and returns; the
// caller synchronises before reading phi.
extern "C" int lesgpu_poisson_ftft_noalloc(const lesgpu_grid *g, const double *d_divgsum, double *d_phi, void *stream) {
    if (!g || !d_divgsum || !d_phi) return LESGPU_ERR_ARG;
    if (g->n1 != g->n1m + 1 || g->n2 != g->n2m + 1 || g->n3 != g->n3m + 1) return LESGPU_ERR_ARG;
    if (g->n1m < 1 || g->n2m < 2 || g->n3m < 1) return LESGPU_ERR_ARG;
    if (g->n1m > kMaxDir || g->n2m > kMaxDir || g->n3m > kMaxDir) return LESGPU_ERR_TOO_LARGE;
    const int n1m = (int)g->n1m, n2m = (int)g->n2m, n3m = (int)g->n3m;
    const int n1 = n1m + 1, n2 = n2m + 1, n3mh = n3m / 2 + 1, n1mh = n1m / 2 + 1;
    lg::DevPlan px{}, pz{};
    if (plan_radices(n1m, px.rad, &px.nst) || plan_radices(n3m, pz.rad, &pz.nst)) return LESGPU_ERR_UNSUPPORTED;
    px.n = n1m;
    pz.n = n3m;

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

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return LESGPU_ERR_CUDA;
    unsigned char *base = nullptr;
    int rc = setup_device(dev, &base);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;

    // host tables (stack, bounded by kMaxDir): poisinit of poiss_ftft.f90:164-204
    double ak1[kMaxDir + 2], ak3[kMaxDir / 2 + 3], f2fyi[kMaxDir + 3], c2cyi[kMaxDir + 3];
    int jpv[kMaxDir + 2], fixjl[kMaxDir + 2], fixju[kMaxDir + 2];
    double2 twx[kMaxDir], twz[kMaxDir];
    memset(ak1, 0, sizeof(ak1));
    memset(ak3, 0, sizeof(ak3));
    const double pi = 2.0 * asin(1.0);
    const double sdzis = g->f2fzi[1], sdxis = g->f2fxi[1];
    for (int k = 1; k <= n3mh; k++) {
        double ai = (k == 1) ? 0.0 : (double)(k - 1) * 2.0 * pi;
        ak3[k] = 2.0 * (1.0 - cos(ai / (double)n3m)) * sdzis * sdzis;
    }
    for (int i = 1; i <= n1mh; i++) {
        double ai = (i == 1) ? 0.0 : (double)(i - 1) * 2.0 * pi;
        ak1[i] = 2.0 * (1.0 - cos(ai / (double)n1m)) * sdxis * sdxis;
    }
    for (int i = n1m; i >= n1mh + 1; i--) ak1[i] = ak1[n1m + 2 - i];
    for (int j = 0; j <= n2; j++) { f2fyi[j] = g->f2fyi[j]; c2cyi[j] = g->c2cyi[j]; }
    f2fyi[n2 + 1] = c2cyi[n2 + 1] = 0.0;
    jpv[0] = fixjl[0] = fixju[0] = 0;
    for (int j = 1; j <= n2m; j++) { jpv[j] = (int)g->jpv[j - 1]; fixjl[j] = (int)g->fixjl[j - 1]; fixju[j] = (int)g->fixju[j - 1]; }
    jpv[n2m + 1] = fixjl[n2m + 1] = fixju[n2m + 1] = 0;
    for (int e = 0; e < n1m; e++) {
        long double a = -2.0L * 3.14159265358979323846264338327950288L * (long double)e / (long double)n1m;
        twx[e] = make_double2((double)cosl(a), (double)sinl(a));
    }
    for (int e = 0; e < n3m; e++) {
        long double a = -2.0L * 3.14159265358979323846264338327950288L * (long double)e / (long double)n3m;
        twz[e] = make_double2((double)cosl(a), (double)sinl(a));
    }
    struct { size_t o; const void *h; size_t b; } cp[] = {
        {o_ak1, ak1, sizeof(double) * (n1 + 2)}, {o_ak3, ak3, sizeof(double) * (n3mh + 2)},
        {o_f2fyi, f2fyi, sizeof(double) * (n2 + 2)}, {o_c2cyi, c2cyi, sizeof(double) * (n2 + 2)},
        {o_jpv, jpv, sizeof(int) * (n2m + 2)}, {o_fixjl, fixjl, sizeof(int) * (n2m + 2)},
        {o_fixju, fixju, sizeof(int) * (n2m + 2)}, {o_twx, twx, sizeof(double2) * n1m}, {o_twz, twz, sizeof(double2) * n3m}};
    // pageable sources: each copy returns once its source has been staged
    for (auto &c : cp)
        if (cudaMemcpyAsync(base + c.o, c.h, c.b, cudaMemcpyHostToDevice, st) != cudaSuccess) return LESGPU_ERR_CUDA;

    lg::KP p;
    memset(&p, 0, sizeof(p));
    p.g.n1 = n1; p.g.n2 = n2; p.g.n3 = n3m + 1;
    p.g.n1m = n1m; p.g.n2m = n2m; p.g.n3m = n3m; p.g.n1mh = n1mh; p.g.n3mh = n3mh;
    p.g.sx = n1 + 1; p.g.sxy = p.g.sx * (n2 + 1); p.g.nt = p.g.sxy * (n3m + 2);
    p.g.f2fyi = (const double *)(base + o_f2fyi);
    p.g.c2cyi = (const double *)(base + o_c2cyi);
    p.g.jpv = (const int *)(base + o_jpv);
    p.g.fixjl = (const int *)(base + o_fixjl);
    p.g.fixju = (const int *)(base + o_fixju);
    p.f.divgsum = (double *)d_divgsum;
    p.f.phi = d_phi;
    px.tw = (const double2 *)(base + o_twx);
    pz.tw = (const double2 *)(base + o_twz);
    px.twf = nullptr;   // FP64 transforms only
    pz.twf = nullptr;
    double2 *ccap = (double2 *)(base + o_ccap);
    double *gam = (double *)(base + o_gam);
    const double *dak1 = (const double *)(base + o_ak1), *dak3 = (const double *)(base + o_ak3);

    // the same launch sequence as the case-based solve (k_fft.cu launch_poisson)
    int Lz = lg::fft_lines_per_block(n3m), Lx = lg::fft_lines_per_block(n1m);
    size_t smz = (size_t)2 * n3m * Lz * sizeof(double2), smx = (size_t)2 * n1m * Lx * sizeof(double2);
    dim3 gz((n1m + 2 * Lz - 1) / (2 * Lz), n2m);   // 2 Lz real lines per block
    int nxl = n3mh * n2m;
    const long long sk = n1m, sj = (long long)n1m * n3mh;
    lg::fft_z_fwd64(gz, smz, st, p, p.f.divgsum, ccap, pz, Lz, sk, sj);
    lg::fft_x64((nxl + Lx - 1) / Lx, smx, st, ccap, nxl, px, Lx, 0);
    long long nl = (long long)n1m * n3mh;
    lg::k_ytri_elim<<<lg::blocks_for(nl, 128), 128, 0, st>>>(p, ccap, dak1, dak3, gam);
    lg::fft_x64((nxl + Lx - 1) / Lx, smx, st, ccap, nxl, px, Lx, 1);
    lg::fft_z_inv64(gz, smz, st, p, ccap, pz, Lz, sk, sj);
    return cudaGetLastError() == cudaSuccess ? 0 : LESGPU_ERR_CUDA;
}
