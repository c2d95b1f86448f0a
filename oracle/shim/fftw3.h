/* Minimal FFTW-API header for compiling the reference CPU imaging library as the oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  FFTW is not installed in this image and is not vendored by
 * the reference (bullseye/mo/cmake/FindFFTW.cmake finds a system copy; no version is
 * pinned).  The reference calls exactly five entry points per precision
 * (bullseye/mo/cpu_gpu_common/fft_and_repacking_routines.cpp:52-99, 122-157):
 * plan_many_dft, execute, execute_dft, destroy_plan.  This header declares those with
 * FFTW's published signatures; oracle/fftw_shim.c implements them with a
 * project-written DFT (unnormalised, FFTW sign convention), so the reference's own
 * finalize/shift/packing code runs unchanged.
 */
#ifndef BULLSEYE_ORACLE_FFTW3_SHIM_H
#define BULLSEYE_ORACLE_FFTW3_SHIM_H
#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef float fftwf_complex[2];
typedef struct oracle_dft_plan *fftw_plan;
typedef struct oracle_dft_planf *fftwf_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_UNALIGNED (1U << 1)

fftw_plan fftw_plan_many_dft(int rank, const int *n, int howmany, fftw_complex *in,
                             const int *inembed, int istride, int idist, fftw_complex *out,
                             const int *onembed, int ostride, int odist, int sign,
                             unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_execute_dft(const fftw_plan p, fftw_complex *in, fftw_complex *out);
void fftw_destroy_plan(fftw_plan p);

fftwf_plan fftwf_plan_many_dft(int rank, const int *n, int howmany, fftwf_complex *in,
                               const int *inembed, int istride, int idist, fftwf_complex *out,
                               const int *onembed, int ostride, int odist, int sign,
                               unsigned flags);
void fftwf_execute(const fftwf_plan p);
void fftwf_execute_dft(const fftwf_plan p, fftwf_complex *in, fftwf_complex *out);
void fftwf_destroy_plan(fftwf_plan p);

#ifdef __cplusplus
}
#endif
#endif
