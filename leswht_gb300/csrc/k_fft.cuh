// Declarations of the FFT / poiss_ftft kernels of k_fft.cu, shared with the
// allocation-free entry point of noalloc.cu.
#pragma once
#include "lesgpu_internal.cuh"

namespace lg {

struct DevPlan {
    int n, nst;
    int rad[24];
    // the radices again, two bits a stage (0: 4, 1: 2, 2: 3, 3: 5): the
    // device reads its stage's radix from this word, where indexing rad[]
    // with the stage number would copy the whole plan to local memory
    unsigned long long radc;
    const double2 *tw;
    const float2 *twf;
};
// fill radc from rad[0 .. nst-1]
void pack_radices(DevPlan &d);

// dynamic shared memory a transform block may take (below the per-block
// opt-in limit, with room for the kernels' static shared memory)
constexpr int kFftSmemMax = 200 * 1024;

// z transforms; the spectrum element (i, k, j) sits at (i-1) + sk*(k-1) + sj*(j-1)
// FP64 launches of the transforms (kernel templates of k_fft.cu, which other
// translation units cannot launch directly): src is the real field transformed
void fft_z_fwd64(dim3 grid, size_t smem, cudaStream_t st, KP p, const double *src, double2 *ccap, DevPlan P, int L,
                 long long sk, long long sj);
void fft_z_inv64(dim3 grid, size_t smem, cudaStream_t st, KP p, const double2 *ccap, DevPlan P, int L, long long sk,
                 long long sj);
void fft_x64(int nblocks, size_t smem, cudaStream_t st, double2 *ccap, int nlines, DevPlan P, int L, int inv);
// opt the FP64 transform kernels into `bytes` of dynamic shared memory
int fft_smem64(int bytes);
// poiss_x_ft: real x lines <-> modes 1..n1mh, one z-y plane per mode
__global__ void k_fft_xr_fwd(KP p, double2 *ccap, DevPlan P, int L);
__global__ void k_fft_xr_inv(KP p, const double2 *ccap, DevPlan P, int L, int pin);
int fft_xr_inv_lines(int n, int L, int pin);
__global__ void k_ytri_elim(KP p, double2 *ccap, const double *ak1, const double *ak3, double *gam);
__global__ void k_ytri_lu(KP p, const double *ak1, const double *ak3, double *ybet, double *ygam, double *yam,
                          double *pinref);
int fft_lines_per_block(int n);
int fft_lz(const lesgpu_case *c);
int fft_lx(const lesgpu_case *c);
int make_plan(FftPlan &p, int n);
DevPlan devplan(const FftPlan &p);
// poiss_z_ft and poiss_x_ft (k_mg.cu)
int mg2d_init(lesgpu_case *c);
void mg2d_free(lesgpu_case *c);
void launch_mg2d(lesgpu_case *c, int msub);
// poiss_mgrd (k_mgrd.cu)
int mgrd_init(lesgpu_case *c);
void mgrd_free(lesgpu_case *c);
void launch_mgrd(lesgpu_case *c, int msub);

}  // namespace lg
