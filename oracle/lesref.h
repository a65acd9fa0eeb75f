/*
 * ORACLE -- test infrastructure only.
 *
 * Public entry points of liblesref.so, the CPU restatement of the LESwHT
 * time step.  They mirror the lesgpu_* C ABI one for one so a parity test
 * drives both with the same inputs.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg load this library.
 */
#ifndef LESREF_H
#define LESREF_H
#include "../include/lesgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ref_case ref_case;

int ref_create(const lesgpu_config *cfg, const lesgpu_grid *grid, ref_case **out);
int ref_load_ibm(ref_case *c, const lesgpu_ibm *ibm);
int ref_set_fields(ref_case *c, const double *u, const double *v, const double *w,
                   const double *p, const double *t, double time, double dt,
                   int64_t ihist, int64_t m);
int ref_start(ref_case *c);
int ref_step(ref_case *c, lesgpu_step_report *rep);
int ref_get_fields(ref_case *c, double *u, double *v, double *w, double *p, double *t);
int ref_get_array(ref_case *c, int64_t field, double *out);
int ref_set_array(ref_case *c, int64_t field, const double *in);
int ref_run_phase(ref_case *c, int64_t phase, int64_t msub);
int ref_get_report(ref_case *c, lesgpu_step_report *rep);
int ref_get_averages(ref_case *c, double *out, int64_t *nsamples, int reset);
int ref_destroy(ref_case *c);
/* OpenMP threads of the loops (omp_set_num_threads); the current count */
int ref_set_threads(int n);
int ref_get_threads(void);

/* building blocks exposed for invariant tests */
int ref_fft_1d(int n, const double *in_reim, double *out_reim, int iopt);
int ref_thomas(int64_t n, const double *a, const double *b, const double *c,
               const double *r, double *x, int periodic);

#ifdef __cplusplus
}
#endif
#endif
