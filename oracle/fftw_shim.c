/* Project-written DFT behind the FFTW entry points the reference CPU library calls.
 *
 * TEST INFRASTRUCTURE ONLY (never linked into the product).  Implements the subset of
 * FFTW's published API that bullseye/mo/cpu_gpu_common/fft_and_repacking_routines.cpp
 * uses: rank-2, contiguous (stride 1), batched ("howmany" slices idist apart), in-place
 * or out-of-place, unnormalised, sign convention X[k] = sum_j x[j] exp(sign * 2 pi i jk/n)
 * (FFTW_BACKWARD = +1).  Arithmetic is double precision for both the double and the
 * float API, so the float variant is slightly more accurate than FFTW's own single
 * precision transform (differences are at the 1e-7 level).
 *
 * Method: row transforms then column transforms.  Power-of-two lengths use an iterative
 * radix-2 Cooley-Tukey transform; other lengths use a direct O(n^2) DFT.  Twiddles are
 * evaluated with libm sin/cos of the exact angle 2 pi jk/n (index reduced mod n first).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "shim/fftw3.h"

struct oracle_dft_plan {
    int ny, nx, howmany, idist, odist, sign;
    double *in, *out; /* double planes */
};
struct oracle_dft_planf {
    int ny, nx, howmany, idist, odist, sign;
    float *in, *out; /* float planes */
};

static int is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

/* In-place 1-D transform of n complex doubles at stride `stride` (in complex units). */
static void dft1d(double *data, int n, int stride, int sign, double *scratch) {
    const double two_pi = 6.283185307179586476925286766559;
    for (int j = 0; j < n; ++j) {
        scratch[2 * j] = data[2 * (size_t)j * stride];
        scratch[2 * j + 1] = data[2 * (size_t)j * stride + 1];
    }
    double *out = scratch + 2 * n;
    if (is_pow2(n)) {
        /* bit-reversal permutation into out */
        int bits = 0;
        while ((1 << bits) < n) ++bits;
        for (int j = 0; j < n; ++j) {
            int r = 0;
            for (int b = 0; b < bits; ++b)
                if (j & (1 << b)) r |= 1 << (bits - 1 - b);
            out[2 * r] = scratch[2 * j];
            out[2 * r + 1] = scratch[2 * j + 1];
        }
        for (int len = 2; len <= n; len <<= 1) {
            int half = len >> 1;
            for (int k = 0; k < half; ++k) {
                /* twiddle exp(sign * 2 pi i k / len) */
                double ang = sign * two_pi * (double)k / (double)len;
                double wr = cos(ang), wi = sin(ang);
                for (int s = 0; s < n; s += len) {
                    double *a = out + 2 * (s + k);
                    double *b = out + 2 * (s + k + half);
                    double tr = b[0] * wr - b[1] * wi;
                    double ti = b[0] * wi + b[1] * wr;
                    b[0] = a[0] - tr;
                    b[1] = a[1] - ti;
                    a[0] += tr;
                    a[1] += ti;
                }
            }
        }
    } else {
        for (int k = 0; k < n; ++k) {
            double sr = 0.0, si = 0.0;
            for (int j = 0; j < n; ++j) {
                long idx = ((long)j * (long)k) % n;
                double ang = sign * two_pi * (double)idx / (double)n;
                double wr = cos(ang), wi = sin(ang);
                sr += scratch[2 * j] * wr - scratch[2 * j + 1] * wi;
                si += scratch[2 * j] * wi + scratch[2 * j + 1] * wr;
            }
            out[2 * k] = sr;
            out[2 * k + 1] = si;
        }
    }
    for (int j = 0; j < n; ++j) {
        data[2 * (size_t)j * stride] = out[2 * j];
        data[2 * (size_t)j * stride + 1] = out[2 * j + 1];
    }
}

/* One 2-D transform of an ny x nx row-major complex-double plane, in place. */
static void dft2d(double *plane, int ny, int nx, int sign) {
    int m = nx > ny ? nx : ny;
    double *scratch = (double *)malloc(sizeof(double) * 4 * (size_t)m);
    for (int y = 0; y < ny; ++y) dft1d(plane + 2 * (size_t)y * nx, nx, 1, sign, scratch);
    for (int x = 0; x < nx; ++x) dft1d(plane + 2 * (size_t)x, ny, nx, sign, scratch);
    free(scratch);
}

fftw_plan fftw_plan_many_dft(int rank, const int *n, int howmany, fftw_complex *in,
                             const int *inembed, int istride, int idist, fftw_complex *out,
                             const int *onembed, int ostride, int odist, int sign,
                             unsigned flags) {
    (void)inembed; (void)onembed; (void)flags;
    if (rank != 2 || istride != 1 || ostride != 1) return NULL;
    fftw_plan p = (fftw_plan)calloc(1, sizeof(*p));
    p->ny = n[0]; p->nx = n[1]; p->howmany = howmany;
    p->idist = idist; p->odist = odist; p->sign = sign;
    p->in = (double *)in; p->out = (double *)out;
    return p;
}

void fftw_execute_dft(const fftw_plan p, fftw_complex *in, fftw_complex *out) {
    size_t plane = (size_t)p->ny * p->nx;
    for (int b = 0; b < p->howmany; ++b) {
        double *src = (double *)in + 2 * (size_t)b * p->idist;
        double *dst = (double *)out + 2 * (size_t)b * p->odist;
        if (src != dst) memcpy(dst, src, sizeof(double) * 2 * plane);
        dft2d(dst, p->ny, p->nx, p->sign);
    }
}

void fftw_execute(const fftw_plan p) { fftw_execute_dft(p, (fftw_complex *)p->in, (fftw_complex *)p->out); }
void fftw_destroy_plan(fftw_plan p) { free(p); }

fftwf_plan fftwf_plan_many_dft(int rank, const int *n, int howmany, fftwf_complex *in,
                               const int *inembed, int istride, int idist, fftwf_complex *out,
                               const int *onembed, int ostride, int odist, int sign,
                               unsigned flags) {
    (void)inembed; (void)onembed; (void)flags;
    if (rank != 2 || istride != 1 || ostride != 1) return NULL;
    fftwf_plan p = (fftwf_plan)calloc(1, sizeof(*p));
    p->ny = n[0]; p->nx = n[1]; p->howmany = howmany;
    p->idist = idist; p->odist = odist; p->sign = sign;
    p->in = (float *)in; p->out = (float *)out;
    return p;
}

void fftwf_execute_dft(const fftwf_plan p, fftwf_complex *in, fftwf_complex *out) {
    size_t plane = (size_t)p->ny * p->nx;
    double *tmp = (double *)malloc(sizeof(double) * 2 * plane);
    for (int b = 0; b < p->howmany; ++b) {
        float *src = (float *)in + 2 * (size_t)b * p->idist;
        float *dst = (float *)out + 2 * (size_t)b * p->odist;
        for (size_t i = 0; i < 2 * plane; ++i) tmp[i] = src[i];
        dft2d(tmp, p->ny, p->nx, p->sign);
        for (size_t i = 0; i < 2 * plane; ++i) dst[i] = (float)tmp[i];
    }
    free(tmp);
}

void fftwf_execute(const fftwf_plan p) { fftwf_execute_dft(p, (fftwf_complex *)p->in, (fftwf_complex *)p->out); }
void fftwf_destroy_plan(fftwf_plan p) { free(p); }
