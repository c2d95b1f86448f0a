// Shared definitions of the GB300 imaging library: precision types, the ABI struct and
// error reporting.  Compiled twice, with -DBULLSEYE_SINGLE (libgpu_imaging32.so) and
// -DBULLSEYE_DOUBLE (libgpu_imaging64.so), like the reference's two libraries.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#if defined(BULLSEYE_SINGLE)
// bullseye/mo/cpu_gpu_common/base_types.h:41-50: single precision data, double normalisation
typedef float vis_real;  // visibilities, uvw, wavelengths, weights, conv taps, grids
#define BZ_PRECISION_BITS 32
#elif defined(BULLSEYE_DOUBLE)
typedef double vis_real;  // base_types.h:51-58
#define BZ_PRECISION_BITS 64
#else
#error "compile with -DBULLSEYE_SINGLE or -DBULLSEYE_DOUBLE"
#endif
typedef double norm_real;

struct vis_complex { vis_real re, im; };  // std::complex<vis_real> layout
struct uvw_coord { vis_real u, v, w; };    // imaging::uvw_coord<uvw_base_type>

// Field order, types and meaning follow bullseye/mo/cpu_gpu_common/gridding_parameters.h:44-109
// exactly: the pipeliner fills this struct through ctypes (bullseye/mo/gridding_parameters.py).
struct gridding_parameters {
  vis_complex *visibilities;          // [rows][channels][pol terms]
  uvw_coord *uvw_coords;              // [rows] metres
  vis_real *reference_wavelengths;    // [spw][channels] metres
  vis_real *visibility_weights;       // [rows][channels][pol terms]
  bool *flags;                        // [rows][channels][pol terms]
  bool *flagged_rows;                 // [rows]
  unsigned int *field_array;          // [rows]
  unsigned int *spw_index_array;      // [rows]
  unsigned int imaging_field;
  size_t baseline_count;              // N(N-1)/2 + N (autocorrelations included)
  size_t row_count;
  size_t chunk_max_row_count;
  size_t channel_count;
  size_t number_of_polarization_terms;
  size_t number_of_polarization_terms_being_gridded;
  size_t spw_count;
  size_t no_timestamps_read;
  size_t nx;
  size_t ny;
  vis_real cell_size_x;               // arcsec
  vis_real cell_size_y;
  vis_real *conv;                     // real [K] (no w) or complex [wplanes][K] (separable w)
  size_t conv_support;                // half support
  size_t conv_oversample;
  size_t polarization_index;
  size_t second_polarization_index;
  vis_complex *output_buffer;         // [facets][cube][corr][ny][nx]
  vis_real phase_centre_ra;           // arcsec
  vis_real phase_centre_dec;
  vis_real *facet_centres;            // [facets][2] arcsec
  size_t num_facet_centres;
  vis_complex *jones_terms;           // [time][antenna][facet][spw][channel][2x2]
  bool should_invert_jones_terms;
  unsigned int *antenna_1_ids;
  unsigned int *antenna_2_ids;
  size_t *timestamp_ids;
  size_t antenna_count;
  bool *enabled_channels;             // [spw][channels]
  size_t *channel_grid_indicies;      // [spw][channels]
  size_t cube_channel_dim_size;
  bool should_grid_sampling_function;
  vis_complex *sampling_function_buffer;  // [facets][sf channels][ny][nx]
  size_t *sampling_function_channel_grid_indicies;
  size_t sampling_function_channel_count;
  bool is_final_data_chunk;
  size_t wplanes;
  vis_real wmax_est;
  size_t *baseline_starting_indexes;  // [baselines + 1], filled by repack_input_data
  size_t *antenna_jones_starting_indexes;
  size_t *jones_time_indicies_per_antenna;
  norm_real *normalization_terms;     // library-owned, published by initLibrary
};

#if defined(BULLSEYE_SINGLE)
static_assert(sizeof(gridding_parameters) == 392, "gridding_parameters must match the reference FP32 layout");
static_assert(offsetof(gridding_parameters, cell_size_x) == 152, "layout");
static_assert(offsetof(gridding_parameters, conv) == 160, "layout");
static_assert(offsetof(gridding_parameters, phase_centre_ra) == 208, "layout");
static_assert(offsetof(gridding_parameters, wmax_est) == 352, "layout");
static_assert(offsetof(gridding_parameters, normalization_terms) == 384, "layout");
#else
static_assert(sizeof(gridding_parameters) == 408, "gridding_parameters must match the reference FP64 layout");
static_assert(offsetof(gridding_parameters, conv) == 168, "layout");
static_assert(offsetof(gridding_parameters, phase_centre_ra) == 216, "layout");
static_assert(offsetof(gridding_parameters, wmax_est) == 368, "layout");
static_assert(offsetof(gridding_parameters, normalization_terms) == 400, "layout");
#endif

// bullseye/mo/cpu_gpu_common/cu_common.h:63 declares this as a float even in double mode;
// every scale derived from it inherits that rounding, so it is kept as a float here too.
static const float kArcsecToRad = (float)(3.14159265358979323846 / (180.0 * 3600.0));

// ---- error reporting (sticky; the reference exits or throws instead) ----
enum bz_status {
  BZ_OK = 0,
  BZ_ERR_NOT_INITIALISED = 1,
  BZ_ERR_INVALID_ARGUMENT = 2,
  BZ_ERR_CUDA = 3,
  BZ_ERR_SINGULAR_JONES = 4,
  BZ_ERR_UNSUPPORTED = 5,
  BZ_ERR_CUFFT = 6,
};

void bz_record_error(int code, const char *fmt, ...);
int bz_error_code();

#define BZ_CUDA_TRY(expr)                                                                  \
  do {                                                                                     \
    cudaError_t _e = (expr);                                                               \
    if (_e != cudaSuccess) {                                                               \
      bz_record_error(BZ_ERR_CUDA, "%s failed: %s (%s:%d)", #expr, cudaGetErrorString(_e), \
                      __FILE__, __LINE__);                                                 \
      return;                                                                              \
    }                                                                                      \
  } while (0)

#define BZ_CUDA_TRY_RET(expr, ret)                                                         \
  do {                                                                                     \
    cudaError_t _e = (expr);                                                               \
    if (_e != cudaSuccess) {                                                               \
      bz_record_error(BZ_ERR_CUDA, "%s failed: %s (%s:%d)", #expr, cudaGetErrorString(_e), \
                      __FILE__, __LINE__);                                                 \
      return ret;                                                                          \
    }                                                                                      \
  } while (0)

// One facet of an uneven layout (bullseye_grid_batched_facets): centre and cell size in arcsec,
// grid size, and the complex-element offset of its [cube][4][ny][nx] block in the caller's grids.
extern "C" {
struct bullseye_facet {
  double ra, dec;
  double cell_x, cell_y;
  size_t nx, ny;
  size_t grid_offset;
};
}
static_assert(sizeof(bullseye_facet) == 56, "bullseye_facet layout");
