/*
 * fftw3.h -- FFTW-API shim for building the reference library here (oracle/_ref).
 *
 * TEST INFRASTRUCTURE ONLY.  The reference (build/init.C:1146-1607, build/templ.C:1293-1366,
 * include/p3dfft.h:93-100, 185-190, 274-280) delegates its 1D arithmetic to FFTW 3, which is not
 * installed on this machine or on the GPU host.  This header declares exactly the FFTW 3 entry
 * points and constants the reference uses, with FFTW's published signatures and meanings (FFTW 3
 * manual: "Advanced Complex DFTs", "Advanced Real-data DFTs", "Advanced Real-to-real
 * Transforms", "New-array Execute Functions", "What FFTW Really Computes").  fftw_shim.c
 * implements them on the oracle's double-precision 1D arithmetic, so the reference's own planner,
 * reorders, derivative and wrappers run unchanged with only the 1D math substituted.
 */
#ifndef ORC_FFTW3_SHIM_H
#define ORC_FFTW3_SHIM_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef float fftwf_complex[2];
typedef struct orc_fftw_plan_s *fftw_plan;
typedef struct orc_fftw_plan_s *fftwf_plan;

/* r2r kinds (FFTW 3 manual, "Real-to-Real Transform Kinds") */
typedef enum {
  FFTW_R2HC = 0, FFTW_HC2R = 1, FFTW_DHT = 2,
  FFTW_REDFT00 = 3, FFTW_REDFT01 = 4, FFTW_REDFT10 = 5, FFTW_REDFT11 = 6,
  FFTW_RODFT00 = 7, FFTW_RODFT01 = 8, FFTW_RODFT10 = 9, FFTW_RODFT11 = 10
} fftw_r2r_kind;
typedef fftw_r2r_kind fftwf_r2r_kind;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_DESTROY_INPUT (1U << 0)
#define FFTW_PRESERVE_INPUT (1U << 4)
#define FFTW_PATIENT (1U << 5)
#define FFTW_ESTIMATE (1U << 6)

void *fftw_malloc(size_t n);
void fftw_free(void *p);
void fftw_destroy_plan(fftw_plan p);
void fftwf_destroy_plan(fftwf_plan p);
void fftw_cleanup(void);
void fftwf_cleanup(void);

fftw_plan fftw_plan_many_dft(int rank, const int *n, int howmany, fftw_complex *in, const int *inembed,
                             int istride, int idist, fftw_complex *out, const int *onembed, int ostride,
                             int odist, int sign, unsigned flags);
fftw_plan fftw_plan_many_dft_r2c(int rank, const int *n, int howmany, double *in, const int *inembed,
                                 int istride, int idist, fftw_complex *out, const int *onembed,
                                 int ostride, int odist, unsigned flags);
fftw_plan fftw_plan_many_dft_c2r(int rank, const int *n, int howmany, fftw_complex *in, const int *inembed,
                                 int istride, int idist, double *out, const int *onembed, int ostride,
                                 int odist, unsigned flags);
fftw_plan fftw_plan_many_r2r(int rank, const int *n, int howmany, double *in, const int *inembed,
                             int istride, int idist, double *out, const int *onembed, int ostride,
                             int odist, const fftw_r2r_kind *kind, unsigned flags);
void fftw_execute_dft(const fftw_plan p, fftw_complex *in, fftw_complex *out);
void fftw_execute_dft_r2c(const fftw_plan p, double *in, fftw_complex *out);
void fftw_execute_dft_c2r(const fftw_plan p, fftw_complex *in, double *out);
void fftw_execute_r2r(const fftw_plan p, double *in, double *out);

fftwf_plan fftwf_plan_many_dft(int rank, const int *n, int howmany, fftwf_complex *in, const int *inembed,
                               int istride, int idist, fftwf_complex *out, const int *onembed,
                               int ostride, int odist, int sign, unsigned flags);
fftwf_plan fftwf_plan_many_dft_r2c(int rank, const int *n, int howmany, float *in, const int *inembed,
                                   int istride, int idist, fftwf_complex *out, const int *onembed,
                                   int ostride, int odist, unsigned flags);
fftwf_plan fftwf_plan_many_dft_c2r(int rank, const int *n, int howmany, fftwf_complex *in,
                                   const int *inembed, int istride, int idist, float *out,
                                   const int *onembed, int ostride, int odist, unsigned flags);
fftwf_plan fftwf_plan_many_r2r(int rank, const int *n, int howmany, float *in, const int *inembed,
                               int istride, int idist, float *out, const int *onembed, int ostride,
                               int odist, const fftwf_r2r_kind *kind, unsigned flags);
void fftwf_execute_dft(const fftwf_plan p, fftwf_complex *in, fftwf_complex *out);
void fftwf_execute_dft_r2c(const fftwf_plan p, float *in, fftwf_complex *out);
void fftwf_execute_dft_c2r(const fftwf_plan p, fftwf_complex *in, float *out);
void fftwf_execute_r2r(const fftwf_plan p, float *in, float *out);

#ifdef __cplusplus
}
#endif
#endif
