/* CPU restatement of the reference's facet-imaging path (the oracle).
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU drop-in: only the
 * tests, the smoke check and the CPU-baseline leg of the benchmark load it.  The product
 * never links, loads or calls it.
 *
 * It restates the algorithm of the reference CPU imaging library
 * (the bullseye/mo/cpu_algorithm and bullseye/mo/cpu_gpu_common sources) in plain C with the same
 * arithmetic types and operation order, so that its results agree bit-for-bit with the
 * reference built from source (oracle/build_ref.sh) on x86-64; tests/test_oracle_golden.py
 * holds that check.  It exports the same C-ABI (bullseye/mo/cpu_gpu_common/wrapper.h:41-61)
 * so one harness drives the reference, this restatement and the GPU drop-in alike.
 *
 * Compiled twice: -DORACLE_SINGLE (float data, double normalisation, like BULLSEYE_SINGLE,
 * bullseye/mo/cpu_gpu_common/base_types.h:41-50) and -DORACLE_DOUBLE.
 *
 * Differences from the reference that do not change results:
 *   - gridding runs synchronously inside the call (the reference uses std::async,
 *     bullseye/mo/cpu_algorithm/wrapper.cpp:184); gridding_barrier() is then a no-op;
 *   - no progress printing;
 *   - a singular Jones matrix sets an error flag readable via oracle_last_error() instead of
 *     throwing through extern "C" (bullseye/mo/cpu_gpu_common/jones_2x2.h:118-123).
 */
#define _GNU_SOURCE
#include <complex.h>
#include <fenv.h>
#include <math.h>
#include <omp.h>
#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "shim/fftw3.h"

#if defined(ORACLE_SINGLE)
typedef float real_t;
typedef float _Complex cplx_t;
#define RLRINT lrintf
#define RSINCOS sincosf
#define RCOS cosf
#define RSIN sinf
#define RSQRT sqrtf
#define RFABS fabsf
#elif defined(ORACLE_DOUBLE)
typedef double real_t;
typedef double _Complex cplx_t;
#define RLRINT lrint
#define RSINCOS sincos
#define RCOS cos
#define RSIN sin
#define RSQRT sqrt
#define RFABS fabs
#else
#error "define ORACLE_SINGLE or ORACLE_DOUBLE"
#endif
typedef double norm_t;

/* bullseye/mo/cpu_gpu_common/cu_common.h:63 -- a float constant even in double mode. */
static const float ARCSEC_TO_RAD = (float)(3.14159265358979323846 / (180.0 * 3600.0));

typedef struct { real_t u, v, w; } uvw_t;
typedef struct { real_t re, im; } rc_t; /* layout of basic_complex / std::complex */

/* Same field order and types as bullseye/mo/cpu_gpu_common/gridding_parameters.h:44-109. */
typedef struct gridding_parameters {
    rc_t *visibilities;
    uvw_t *uvw_coords;
    real_t *reference_wavelengths;
    real_t *visibility_weights;
    bool *flags;
    bool *flagged_rows;
    unsigned int *field_array;
    unsigned int *spw_index_array;
    unsigned int imaging_field;
    size_t baseline_count, row_count, chunk_max_row_count, channel_count;
    size_t number_of_polarization_terms, number_of_polarization_terms_being_gridded;
    size_t spw_count, no_timestamps_read, nx, ny;
    real_t cell_size_x, cell_size_y;
    real_t *conv;
    size_t conv_support, conv_oversample, polarization_index, second_polarization_index;
    rc_t *output_buffer;
    real_t phase_centre_ra, phase_centre_dec;
    real_t *facet_centres;
    size_t num_facet_centres;
    rc_t *jones_terms;
    bool should_invert_jones_terms;
    unsigned int *antenna_1_ids, *antenna_2_ids;
    size_t *timestamp_ids;
    size_t antenna_count;
    bool *enabled_channels;
    size_t *channel_grid_indicies;
    size_t cube_channel_dim_size;
    bool should_grid_sampling_function;
    rc_t *sampling_function_buffer;
    size_t *sampling_function_channel_grid_indicies;
    size_t sampling_function_channel_count;
    bool is_final_data_chunk;
    size_t wplanes;
    real_t wmax_est;
    size_t *baseline_starting_indexes;
    size_t *antenna_jones_starting_indexes;
    size_t *jones_time_indicies_per_antenna;
    norm_t *normalization_terms;
} gp_t;

_Static_assert(sizeof(gp_t) == (sizeof(real_t) == 4 ? 392 : 408), "gridding_parameters layout");

enum corr_mode { CORR_SINGLE = 1, CORR_DUAL = 2, CORR_QUAD = 4, CORR_QUAD_JONES = 5, CORR_SAMPLING = 8 };
enum conv_mode { CONV_AA_1D, CONV_W_2D, CONV_NN };

static norm_t *g_norm = NULL;
static int g_initialized = 0;
static int g_error = 0;
static double g_grid_seconds = 0.0, g_inv_seconds = 0.0;

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + ts.tv_nsec * 1e-9;
}

/* ---- complex helpers matching basic_complex (cu_basic_complex.h:42-92) ---- */
static inline rc_t rc_mul(rc_t a, rc_t b) {
    rc_t r;
    r.re = a.re * b.re - a.im * b.im;
    r.im = a.re * b.im + a.im * b.re;
    return r;
}

/* ---- 2x2 Jones algebra with C99 complex (lowered like std::complex by GCC) ----
 * jones_2x2.h:52-126 and correlation_gridding_traits.h:137-160 */
typedef struct { cplx_t c[4]; } jones_t;

#if defined(ORACLE_SINGLE)
#define MKC(re, im) CMPLXF((re), (im))
#else
#define MKC(re, im) CMPLX((re), (im))
#endif
static inline cplx_t to_c(rc_t a) { return MKC(a.re, a.im); }

static inline jones_t j_mul(jones_t a, jones_t b) {
    jones_t o;
    o.c[0] = a.c[0] * b.c[0] + a.c[1] * b.c[2];
    o.c[1] = a.c[0] * b.c[1] + a.c[1] * b.c[3];
    o.c[2] = a.c[2] * b.c[0] + a.c[3] * b.c[2];
    o.c[3] = a.c[2] * b.c[1] + a.c[3] * b.c[3];
    return o;
}

/* In-place inverse, jones_2x2.h:86-105; returns 0 when the determinant is exactly zero. */
static int j_invert(jones_t *m) {
    cplx_t det = m->c[0] * m->c[3] - m->c[1] * m->c[2];
    if (det == 0) return 0;
    cplx_t one = 1;
    cplx_t det_inv = one / det;
    m->c[1] *= -det_inv;
    m->c[2] *= -det_inv;
    cplx_t swp = m->c[0];
    m->c[0] = m->c[3] * det_inv;
    m->c[3] = swp * det_inv;
    return 1;
}

/* ---- per-facet transforms ---- */
typedef struct { real_t l, m, n; } lmn_t;

/* phase_transform_policies.h:110-134 */
static void delta_lmn(real_t old_ra, real_t old_dec, real_t new_ra, real_t new_dec, lmn_t *r) {
    real_t d_ra = (new_ra - old_ra) * ARCSEC_TO_RAD, d_dec = new_dec * ARCSEC_TO_RAD,
           d_decp = old_dec * ARCSEC_TO_RAD, c_d_dec = RCOS(d_dec), s_d_dec = RSIN(d_dec),
           s_d_ra = RSIN(d_ra), c_d_ra = RCOS(d_ra), c_d_decp = RCOS(d_decp), s_d_decp = RSIN(d_decp);
    r->l = -c_d_dec * s_d_ra;
    r->m = -(s_d_dec * c_d_decp - c_d_dec * s_d_decp * c_d_ra);
    r->n = 1 - RSQRT(1 - r->l * r->l - r->m * r->m);
}

/* baseline_transform_policies.h:117-149 (Kogan & Greisen planar approximation) */
static void planar_terms(real_t old_ra, real_t old_dec, real_t new_ra, real_t new_dec, real_t *ut, real_t *vt) {
    real_t d_ra = (new_ra - old_ra) * ARCSEC_TO_RAD, n_dec = new_dec * ARCSEC_TO_RAD,
           o_dec = old_dec * ARCSEC_TO_RAD, c_d_ra = RCOS(d_ra), s_d_ra = RSIN(d_ra),
           c_new_dec = RCOS(n_dec), c_old_dec = RCOS(o_dec), s_new_dec = RSIN(n_dec),
           s_old_dec = RSIN(o_dec), li0 = c_new_dec * s_d_ra,
           mi0 = s_new_dec * c_old_dec - c_new_dec * s_old_dec * c_d_ra,
           ni0 = s_new_dec * s_old_dec + c_new_dec * c_old_dec * c_d_ra;
    *ut = li0 / ni0;
    *vt = mi0 / ni0;
}

/* ---- gridding (templated_gridder.h:17-103 with the policies it composes) ---- */
struct modes {
    int corr;     /* enum corr_mode */
    int phase;    /* enable_faceting_phase_shift */
    int uvxform;  /* transform_planar_approx_with_w */
    int conv;     /* enum conv_mode */
};

/* Test instrumentation (not in the reference): when set, the AA and w-projection branches write
 * every (facet, row, channel)'s footprint corner and tap offsets {du, dv, fu, fv} (-1 x 4 when the
 * reference rejects it) into g_tap_log[((f x rows + row) x channels + c) x 4 ...] instead of
 * gridding it, so that a test can compare the cell choices of the two precisions. */
static long long *g_tap_log = NULL;
static size_t g_tap_log_n = 0;

void oracle_record_taps(long long *log, size_t n) {
    g_tap_log = log;
    g_tap_log_n = n;
}

static int record_taps(gp_t *p, size_t f, size_t row, size_t c, int ok, size_t du, size_t dv, size_t fu, size_t fv) {
    if (!g_tap_log) return 0;
    const size_t i = ((f * p->row_count + row) * p->channel_count + c) * 4;
    if (i + 3 < g_tap_log_n) {
        g_tap_log[i] = ok ? (long long)du : -1;
        g_tap_log[i + 1] = ok ? (long long)dv : -1;
        g_tap_log[i + 2] = ok ? (long long)fu : -1;
        g_tap_log[i + 3] = ok ? (long long)fv : -1;
    }
    return 1;
}

static void grid_one_facet(gp_t *p, const struct modes *md, size_t f) {
    const size_t W = (p->conv_support << 1) + 1;
    const size_t padded = W + 2;
    const size_t os = p->conv_oversample;
    const int ncorr = (md->corr == CORR_QUAD || md->corr == CORR_QUAD_JONES) ? 4
                      : (md->corr == CORR_DUAL ? 2 : 1);
    real_t u_scale = p->nx * p->cell_size_x * ARCSEC_TO_RAD;
    real_t v_scale = -(p->ny * p->cell_size_y * ARCSEC_TO_RAD);
    real_t gcx = p->nx / 2 - p->conv_support;
    real_t gcy = p->ny / 2 - p->conv_support;
    size_t slice = p->nx * p->ny << 1; /* grid_size_in_floats */

    real_t *facet_grid;
    if (md->corr == CORR_SAMPLING)
        facet_grid = (real_t *)p->sampling_function_buffer + slice * p->sampling_function_channel_count * f;
    else
        facet_grid = (real_t *)p->output_buffer +
                     slice * p->number_of_polarization_terms_being_gridded * p->cube_channel_dim_size * f;

    /* the disabled phase policy reports the phase centre as the facet centre
       (phase_transform_policies.h:77-82); the uv transform is computed from that. */
    real_t new_ra = p->phase_centre_ra, new_dec = p->phase_centre_dec;
    if (md->phase) {
        new_ra = p->facet_centres[f << 1];
        new_dec = p->facet_centres[(f << 1) + 1];
    }
    real_t u_term = 0, v_term = 0;
    if (md->uvxform) planar_terms(p->phase_centre_ra, p->phase_centre_dec, new_ra, new_dec, &u_term, &v_term);
    lmn_t dlmn = {0, 0, 0};
    if (md->phase) delta_lmn(p->phase_centre_ra, p->phase_centre_dec, new_ra, new_dec, &dlmn);

    const size_t K = padded + (padded - 1) * (os - 1); /* conv_dim_size */

    for (size_t row = 0; row < p->row_count; ++row) {
        uvw_t uvw = p->uvw_coords[row];
        bool row_flagged = p->flagged_rows[row];
        bool in_field = (p->field_array[row] == p->imaging_field);
        size_t spw = p->spw_index_array[row];
        for (size_t c = 0; c < p->channel_count; ++c) {
            size_t sc = spw * p->channel_count + c;
            if (!p->enabled_channels[sc]) continue;
            size_t g = (md->corr == CORR_SAMPLING) ? p->sampling_function_channel_grid_indicies[sc]
                                                    : p->channel_grid_indicies[sc];
            real_t inv_lambda = 1 / p->reference_wavelengths[sc];

            rc_t vis[4];
            real_t wt[4];
            bool fl[4];
            size_t npol = p->number_of_polarization_terms;
            if (md->corr == CORR_SAMPLING) {
                vis[0].re = 1; vis[0].im = 0; wt[0] = 1; fl[0] = false;
            } else if (md->corr == CORR_SINGLE) {
                size_t vi = (row * p->channel_count + c) * npol + p->polarization_index;
                fl[0] = p->flags[vi]; wt[0] = p->visibility_weights[vi]; vis[0] = p->visibilities[vi];
            } else if (md->corr == CORR_DUAL) {
                size_t vi = (row * p->channel_count + c) * npol;
                fl[0] = p->flags[vi + p->polarization_index];
                fl[1] = p->flags[vi + p->second_polarization_index];
                wt[0] = p->visibility_weights[vi + p->polarization_index];
                wt[1] = p->visibility_weights[vi + p->second_polarization_index];
                vis[0] = p->visibilities[vi + p->polarization_index];
                vis[1] = p->visibilities[vi + p->second_polarization_index];
            } else { /* quad: the 4 correlations of (row, c) read as one vec4 */
                size_t vi = (row * p->channel_count + c) * 4;
                for (int k = 0; k < 4; ++k) {
                    fl[k] = p->flags[vi + k]; wt[k] = p->visibility_weights[vi + k]; vis[k] = p->visibilities[vi + k];
                }
            }
            uvw_t uvl = uvw;
            uvl.u *= inv_lambda;
            uvl.v *= inv_lambda;
            uvl.w *= inv_lambda;

            if (md->corr == CORR_QUAD_JONES) {
                /* correlation_gridding_policies.h:523-542 (terms pre-inverted) */
                size_t t = p->timestamp_ids[row];
                size_t a1 = p->antenna_1_ids[row], a2 = p->antenna_2_ids[row];
                size_t i1 = (((t * p->antenna_count + a1) * p->num_facet_centres + f) * p->spw_count + spw) * p->channel_count + c;
                size_t i2 = (((t * p->antenna_count + a2) * p->num_facet_centres + f) * p->spw_count + spw) * p->channel_count + c;
                jones_t pinv, qinv, v;
                for (int k = 0; k < 4; ++k) {
                    pinv.c[k] = to_c(p->jones_terms[i1 * 4 + k]);
                    qinv.c[k] = to_c(p->jones_terms[i2 * 4 + k]);
                    v.c[k] = to_c(vis[k]);
                }
                /* hermitian transpose of q (jones_2x2.h:57-67) */
                cplx_t swp = conj(qinv.c[1]);
                qinv.c[0] = MKC(creal(qinv.c[0]), -cimag(qinv.c[0]));
                qinv.c[1] = conj(qinv.c[2]);
                qinv.c[2] = swp;
                qinv.c[3] = MKC(creal(qinv.c[3]), -cimag(qinv.c[3]));
                jones_t o = j_mul(pinv, j_mul(v, qinv));
                for (int k = 0; k < 4; ++k) { vis[k].re = creal(o.c[k]); vis[k].im = cimag(o.c[k]); }
            }
            bool keep[4];
            real_t cw[4];
            for (int k = 0; k < ncorr; ++k) {
                keep[k] = !(fl[k] || row_flagged) && in_field;
                cw[k] = wt[k] * (real_t)(int)keep[k];
                vis[k].re = vis[k].re * cw[k];
                vis[k].im = vis[k].im * cw[k];
            }
            if (md->phase) {
                real_t x = 2 * 3.14159265358979323846 * (uvl.u * dlmn.l + uvl.v * dlmn.m + uvl.w * (dlmn.n));
                real_t s, co;
                RSINCOS(x, &s, &co);
                rc_t ph = {co, s};
                for (int k = 0; k < ncorr; ++k) vis[k] = rc_mul(vis[k], ph);
            }
            if (md->uvxform) {
                uvl.u = uvl.u - uvl.w * u_term;
                uvl.v = uvl.v - uvl.w * v_term;
            }
            uvl.u *= u_scale;
            uvl.v *= v_scale;

            norm_t norm_acc = 0;
            real_t *gbase;
            if (md->corr == CORR_SAMPLING) gbase = facet_grid + g * slice;
            else gbase = facet_grid + (g * p->number_of_polarization_terms_being_gridded) * slice;

            if (md->conv == CONV_NN) {
                /* convolution_policies.h:35-65 */
                real_t tu = uvl.u + (p->nx >> 1), tv = uvl.v + (p->ny >> 1);
                size_t du = (size_t)RLRINT(tu), dv = (size_t)RLRINT(tv);
                if (dv >= p->ny || du >= p->nx) goto next;
                for (int k = 0; k < ncorr; ++k) {
                    real_t *cell = gbase + k * slice + ((dv * p->nx + du) << 1);
                    cell[0] += vis[k].re;
                    cell[1] += vis[k].im;
                }
                norm_acc += 1.0;
            } else if (md->conv == CONV_AA_1D) {
                /* convolution_policies.h:70-118; FE_DOWNWARD is in force (lrint == floor) */
                real_t tu = uvl.u + gcx, tv = uvl.v + gcy;
                size_t du = (size_t)RLRINT(tu), dv = (size_t)RLRINT(tv);
                size_t fu = (size_t)((1 - uvl.u + (real_t)RLRINT(uvl.u)) * (real_t)os);
                size_t fv = (size_t)((1 - uvl.v + (real_t)RLRINT(uvl.v)) * (real_t)os);
                if (record_taps(p, f, row, c, !(dv + padded >= p->ny || du + padded >= p->nx || dv >= p->ny || du >= p->nx),
                                du, dv, fu, fv))
                    goto next;
                if (dv + padded >= p->ny || du + padded >= p->nx || dv >= p->ny || du >= p->nx) goto next;
                size_t cv = fv;
                for (size_t sv = 0; sv < W; ++sv) {
                    real_t kv = p->conv[cv];
                    size_t cu = fu;
                    for (size_t su = 0; su < W; ++su) {
                        real_t ku = p->conv[cu];
                        real_t tap = ku * kv;
                        real_t *cell = gbase + (((dv + sv) * p->nx + (du + su)) << 1);
                        for (int k = 0; k < ncorr; ++k) {
                            cell[k * slice] += vis[k].re * tap;
                            cell[k * slice + 1] += vis[k].im * tap;
                        }
                        norm_acc += tap;
                        cu += os;
                    }
                    cv += os;
                }
            } else {
                /* convolution_policies.h:231-289 (2-D complex w-projection stack) */
                if (uvl.w < 0) {
                    for (int k = 0; k < ncorr; ++k) vis[k].im *= -1;
                    uvl.u *= -1; uvl.v *= -1; uvl.w *= -1;
                }
                real_t tu = uvl.u + gcx, tv = uvl.v + gcy;
                size_t du = (size_t)RLRINT(tu), dv = (size_t)RLRINT(tv);
                size_t fu = (size_t)((1 - uvl.u + (real_t)RLRINT(uvl.u)) * (real_t)os);
                size_t fv = (size_t)((1 - uvl.v + (real_t)RLRINT(uvl.v)) * (real_t)os);
                size_t plane = (size_t)RLRINT(RFABS(uvl.w) / (float)p->wmax_est * (real_t)(p->wplanes - 1));
                size_t foff = plane * K * K;
                if (record_taps(p, f, row, c,
                                !(dv + padded >= p->ny || du + padded >= p->nx || dv >= p->ny || du >= p->nx ||
                                  plane >= p->wplanes),
                                du, dv, fu, fv))
                    goto next;
                if (dv + padded >= p->ny || du + padded >= p->nx || dv >= p->ny || du >= p->nx ||
                    plane >= p->wplanes) goto next;
                const rc_t *tab = (const rc_t *)p->conv;
                size_t cv = foff + fv * K;
                for (size_t sv = 0; sv < W; ++sv) {
                    size_t cu = fu;
                    for (size_t su = 0; su < W; ++su) {
                        rc_t tap = tab[cv + cu];
                        real_t *cell = gbase + (((dv + sv) * p->nx + (du + su)) << 1);
                        for (int k = 0; k < ncorr; ++k) {
                            rc_t cvv = rc_mul(vis[k], tap);
                            cell[k * slice] += cvv.re;
                            cell[k * slice + 1] += cvv.im;
                        }
                        norm_acc += tap.re;
                        cu += os;
                    }
                    cv += os * K;
                }
            }
            if (md->corr != CORR_SAMPLING) {
                /* templated_gridder.h:97 then store_normalization_term */
                real_t nf = (real_t)norm_acc;
                size_t base = (f * p->cube_channel_dim_size + g) * (size_t)ncorr;
                for (int k = 0; k < ncorr; ++k) p->normalization_terms[base + k] += (norm_t)(cw[k] * nf);
            }
        next:;
        }
    }
}

/* Runs one gridding pass over all facets.  The reference sets the rounding mode per
 * convolution policy (FE_DOWNWARD for the 1-D AA policy, FE_TONEAREST otherwise,
 * convolution_policies.h:37,73,124,233) on the thread that then opens the OpenMP team
 * (templated_gridder.h:18,29); every team member here sets it explicitly.  OpenMP runs over
 * facets only, schedule(static), as templated_gridder.h:29. */
static void run_gridder(gp_t *p, const struct modes *md) {
    const int mode = (md->conv == CONV_AA_1D) ? FE_DOWNWARD : FE_TONEAREST;
    double t0 = now_s();
#pragma omp parallel
    {
        int saved = fegetround();
        fesetround(mode);
#pragma omp for schedule(static)
        for (long f = 0; f < (long)p->num_facet_centres; ++f) grid_one_facet(p, md, (size_t)f);
        fesetround(saved);
    }
    g_grid_seconds += now_s() - t0;
}

static void grid_dispatch(gp_t *p, int corr, int faceting) {
    struct modes md;
    md.corr = corr;
    md.phase = faceting && corr != CORR_SAMPLING;
    md.uvxform = faceting;
    md.conv = (p->wplanes <= 1) ? CONV_AA_1D : CONV_W_2D;
    run_gridder(p, &md);
}

/* ---------------- exported C-ABI (wrapper.h:41-61) ---------------- */
double get_gridding_walltime(void) { return g_grid_seconds; }
double get_inversion_walltime(void) { return g_inv_seconds; }
void gridding_barrier(void) {}
int oracle_last_error(void) { return g_error; }

/* wrapper.cpp:82-106 -- the library owns the normalisation terms and publishes the pointer */
void initLibrary(gp_t *p) {
    if (g_initialized) return;
    g_initialized = 1;
    g_error = 0;
    g_grid_seconds = g_inv_seconds = 0.0;
    size_t n = p->num_facet_centres * p->cube_channel_dim_size * p->number_of_polarization_terms_being_gridded;
    g_norm = (norm_t *)calloc(n ? n : 1, sizeof(norm_t));
    p->normalization_terms = g_norm;
}

void releaseLibrary(void) {
    if (!g_initialized) return;
    g_initialized = 0;
    free(g_norm);
    g_norm = NULL;
}

/* wrapper.cpp:116-135 (channel_grid_indicies compared with the sampling-function channel
 * index c, as in the reference) */
void weight_uniformly(gp_t *p) {
    const real_t eps = 0.0000001f;
    size_t nxy = p->nx * p->ny;
    for (size_t f = 0; f < p->num_facet_centres; ++f)
        for (size_t g = 0; g < p->cube_channel_dim_size; ++g)
            for (size_t y = 0; y < p->ny; ++y)
                for (size_t x = 0; x < p->nx; ++x) {
                    real_t count = eps;
                    for (size_t c = 0; c < p->sampling_function_channel_count; ++c)
                        count += (int)(p->channel_grid_indicies[c] == g) *
                                 p->sampling_function_buffer[((f * p->sampling_function_channel_count + c) * p->ny + y) * p->nx + x].re;
                    count = 1 / count;
                    for (size_t corr = 0; corr < p->number_of_polarization_terms_being_gridded; ++corr) {
                        rc_t *cell = &p->output_buffer[(((f * p->cube_channel_dim_size + g) *
                                                          p->number_of_polarization_terms_being_gridded + corr) * p->ny + y) * p->nx + x];
                        cell->re *= count;
                        cell->im *= count;
                    }
                    (void)nxy;
                }
}

/* wrapper.cpp:136-163; complex<float> /= double converts the divisor to float first */
void normalize(gp_t *p) {
    size_t C = p->number_of_polarization_terms_being_gridded;
    for (size_t f = 0; f < p->num_facet_centres; ++f)
        for (size_t ch = 0; ch < p->cube_channel_dim_size; ++ch)
            for (size_t corr = 0; corr < C; ++corr) {
                norm_t nv = p->normalization_terms[(f * p->cube_channel_dim_size + ch) * C + corr];
                real_t d = (real_t)nv;
                rc_t *g = p->output_buffer + ((f * p->cube_channel_dim_size + ch) * C + corr) * p->ny * p->nx;
                for (size_t i = 0; i < p->ny * p->nx; ++i) {
                    g[i].re /= d;
                    g[i].im /= d;
                }
            }
}

/* numpy-convention shifts (fft_shift_utils.cpp:41-112 realise the same permutation in
 * place; the reference notebook "Fourier Shifting" asserts equality with numpy) */
static void shift_plane(rc_t *plane, size_t nx, size_t ny, int inverse, rc_t *tmp) {
    size_t sx = nx / 2, sy = ny / 2;
    for (size_t y = 0; y < ny; ++y)
        for (size_t x = 0; x < nx; ++x) {
            size_t srcy, srcx;
            if (!inverse) { srcy = (y + ny - sy) % ny; srcx = (x + nx - sx) % nx; }
            else { srcy = (y + sy) % ny; srcx = (x + sx) % nx; }
            tmp[y * nx + x] = plane[srcy * nx + srcx];
        }
    memcpy(plane, tmp, sizeof(rc_t) * nx * ny);
}

static void transform_slices(rc_t *base, size_t nx, size_t ny, size_t nslices) {
    int dims[2] = {(int)ny, (int)nx};
    rc_t *tmp = (rc_t *)malloc(sizeof(rc_t) * nx * ny);
    for (size_t s = 0; s < nslices; ++s) shift_plane(base + s * nx * ny, nx, ny, 1, tmp);
#if defined(ORACLE_SINGLE)
    fftwf_plan pl = fftwf_plan_many_dft(2, dims, (int)nslices, (fftwf_complex *)base, dims, 1, (int)(nx * ny),
                                        (fftwf_complex *)base, dims, 1, (int)(nx * ny), FFTW_BACKWARD, FFTW_ESTIMATE);
    fftwf_execute(pl);
    fftwf_destroy_plan(pl);
#else
    fftw_plan pl = fftw_plan_many_dft(2, dims, (int)nslices, (fftw_complex *)base, dims, 1, (int)(nx * ny),
                                      (fftw_complex *)base, dims, 1, (int)(nx * ny), FFTW_BACKWARD, FFTW_ESTIMATE);
    fftw_execute(pl);
    fftw_destroy_plan(pl);
#endif
    for (size_t s = 0; s < nslices; ++s) shift_plane(base + s * nx * ny, nx, ny, 0, tmp);
    free(tmp);
}

/* fft_and_repacking_routines.cpp:83-118: per facet, shift -> unnormalised backward c2c over
 * the first cube slices -> shift; then float32 real parts packed at float index offset*f */
static void finalize_buffer(rc_t *buf, size_t nx, size_t ny, size_t nf, size_t per_facet_slices, size_t nslices) {
    double t0 = now_s();
    size_t offset = nx * ny * per_facet_slices;
    for (size_t f = 0; f < nf; ++f) transform_slices(buf + f * offset, nx, ny, nslices);
    real_t *src = (real_t *)buf;
    float *dst = (float *)buf;
    for (size_t f = 0; f < nf; ++f) {
        size_t lo = offset * f, hi = lo + nx * ny * nslices;
        for (size_t i = lo; i < hi; ++i) dst[i] = (float)src[i * 2];
    }
    g_inv_seconds += now_s() - t0;
}

void finalize(gp_t *p) {
    finalize_buffer(p->output_buffer, p->nx, p->ny, p->num_facet_centres,
                    p->cube_channel_dim_size * p->number_of_polarization_terms_being_gridded,
                    p->cube_channel_dim_size);
}

void finalize_psf(gp_t *p) {
    finalize_buffer(p->sampling_function_buffer, p->nx, p->ny, p->num_facet_centres,
                    p->sampling_function_channel_count, p->sampling_function_channel_count);
}

/* wrapper.cpp:171-181: the CPU library has no repacking step (it throws); flag instead */
void repack_input_data(gp_t *p) { (void)p; g_error = 2; }

void grid_single_pol(gp_t *p) { grid_dispatch(p, CORR_SINGLE, 0); }
void facet_single_pol(gp_t *p) { grid_dispatch(p, CORR_SINGLE, 1); }
void grid_duel_pol(gp_t *p) { grid_dispatch(p, CORR_DUAL, 0); }
void facet_duel_pol(gp_t *p) { grid_dispatch(p, CORR_DUAL, 1); }
void grid_4_cor(gp_t *p) { grid_dispatch(p, CORR_QUAD, 0); }
void facet_4_cor(gp_t *p) { grid_dispatch(p, CORR_QUAD, 1); }

/* wrapper.cpp:351-381: invert every Jones matrix in place, then grid with corrections */
void facet_4_cor_corrections(gp_t *p) {
    size_t n = p->no_timestamps_read * p->antenna_count * p->num_facet_centres * p->spw_count * p->channel_count;
    int bad = 0;
#pragma omp parallel for reduction(| : bad)
    for (long j = 0; j < (long)n; ++j) {
        jones_t m;
        for (int k = 0; k < 4; ++k) m.c[k] = to_c(p->jones_terms[(size_t)j * 4 + k]);
        if (!j_invert(&m)) { bad |= 1; continue; }
        for (int k = 0; k < 4; ++k) {
            p->jones_terms[(size_t)j * 4 + k].re = creal(m.c[k]);
            p->jones_terms[(size_t)j * 4 + k].im = cimag(m.c[k]);
        }
    }
    if (bad) { g_error = 1; return; }
    grid_dispatch(p, CORR_QUAD_JONES, 1);
}

void grid_sampling_function(gp_t *p) { grid_dispatch(p, CORR_SAMPLING, 0); }
void facet_sampling_function(gp_t *p) { grid_dispatch(p, CORR_SAMPLING, 1); }

/* Integer sampling counts: the reference's nearest-neighbour policy
 * (convolution_policies.h:35-65) applied to the sampling function, grid or facet mode. */
void oracle_sampling_counts_nn(gp_t *p, int faceting) {
    struct modes md = {CORR_SAMPLING, 0, faceting, CONV_NN};
    run_gridder(p, &md);
}
