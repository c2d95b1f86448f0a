// Integer sampling-function counts with the reference's nearest-neighbour policy.
//
// The reference's sampling-function gridder (cpu_algorithm/wrapper.cpp:383-425, policy
// correlation_gridding_policies.h:190-245) grids V = 1 with unit weight, zeroed for flagged rows
// and rows outside the imaged field (templated_gridder.h:70-77).  With the nearest-neighbour
// convolution policy (convolution_policies.h:35-65) every kept (row, channel) adds exactly 1 to
// one cell, so the grid holds integer counts; this kernel produces them bit for bit.  Cell
// selection repeats the reference's arithmetic in the library's data precision, operation by
// operation and without contraction (the __*_rn intrinsics are never fused):
//   u = u_m * (1 / lambda);  u *= nx * cell * ARCSEC_TO_RAD;  x = lrint(u + (nx >> 1))  (nearest even)
//   v likewise with -(ny * cell_y * ARCSEC_TO_RAD);  rejected when x or y is outside [0, n).
// In facet mode the sampling function's uv transform is the identity: its phase policy reports the
// phase centre as the facet centre (phase_transform_policies.h:77-82), so u_term = v_term = 0
// exactly and u - w * 0 = u.  Every facet therefore receives the same counts.
#include <cstring>

#include "common.h"

namespace {

#if defined(BULLSEYE_SINGLE)
__device__ __forceinline__ vis_real mul_rn(vis_real a, vis_real b) { return __fmul_rn(a, b); }
__device__ __forceinline__ vis_real add_rn(vis_real a, vis_real b) { return __fadd_rn(a, b); }
__device__ __forceinline__ vis_real rcp_rn(vis_real a) { return __fdiv_rn(1.0f, a); }
__device__ __forceinline__ vis_real round_even(vis_real a) { return rintf(a); }
#else
__device__ __forceinline__ vis_real mul_rn(vis_real a, vis_real b) { return __dmul_rn(a, b); }
__device__ __forceinline__ vis_real add_rn(vis_real a, vis_real b) { return __dadd_rn(a, b); }
__device__ __forceinline__ vis_real rcp_rn(vis_real a) { return __ddiv_rn(1.0, a); }
__device__ __forceinline__ vis_real round_even(vis_real a) { return rint(a); }
#endif

struct NNArgs {
  const vis_real *uvw;
  const vis_real *wavelengths;
  const unsigned *spw;
  const unsigned *field;
  const uint8_t *flagged_rows;
  const uint8_t *enabled;
  const size_t *sf_cgi;
  unsigned *counts;  // [sf_ch][ny][nx] of facet 0
  int *error;
  long long nrows;
  int nchan, nspw, nx, ny, sf_ch;
  unsigned imaging_field;
  vis_real u_scale, v_scale, half_x, half_y;
};

__global__ void sampling_counts_nn_kernel(const NNArgs a) {
  const long long n = a.nrows * a.nchan;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const long long row = i / a.nchan;
    const int c = (int)(i - row * a.nchan);
    const unsigned spw = a.spw[row];
    if (spw >= (unsigned)a.nspw) {
      atomicOr(a.error, 1);
      continue;
    }
    const long long sc = (long long)spw * a.nchan + c;
    if (!a.enabled[sc]) continue;
    // the kept weight is 0 for flagged rows and rows of other fields: the reference adds 0 there
    if (a.flagged_rows[row] || a.field[row] != a.imaging_field) continue;
    const size_t g = a.sf_cgi[sc];
    if (g >= (size_t)a.sf_ch) {
      atomicOr(a.error, 2);
      continue;
    }
    const vis_real inv = rcp_rn(a.wavelengths[sc]);
    const vis_real u = mul_rn(mul_rn(a.uvw[3 * row], inv), a.u_scale);
    const vis_real v = mul_rn(mul_rn(a.uvw[3 * row + 1], inv), a.v_scale);
    const vis_real x = round_even(add_rn(u, a.half_x));
    const vis_real y = round_even(add_rn(v, a.half_y));
    // lrint's result converted to size_t: negatives wrap to huge values and are rejected
    if (!(x >= (vis_real)0 && y >= (vis_real)0 && x < (vis_real)a.nx && y < (vis_real)a.ny)) continue;
    atomicAdd(a.counts + ((long long)g * a.ny + (long long)y) * a.nx + (long long)x, 1u);
  }
}

__device__ int g_nn_error;

}  // namespace

// See include/bullseye_gb300.h.
extern "C" int bullseye_sampling_counts_nn(const gridding_parameters *params, unsigned int *counts, int faceting,
                                           void *stream) {
  (void)faceting;  // the sampling function's uv transform is the identity in facet mode
  if (!params || !counts) return BZ_ERR_INVALID_ARGUMENT;
  const gridding_parameters &p = *params;
  if (p.row_count && (!p.uvw_coords || !p.reference_wavelengths || !p.spw_index_array || !p.field_array ||
                      !p.flagged_rows || !p.enabled_channels || !p.sampling_function_channel_grid_indicies))
    return BZ_ERR_INVALID_ARGUMENT;
  if (p.nx == 0 || p.ny == 0 || p.sampling_function_channel_count == 0) return BZ_ERR_INVALID_ARGUMENT;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t F = p.num_facet_centres ? p.num_facet_centres : 1;
  const size_t slab = p.sampling_function_channel_count * p.nx * p.ny;
  NNArgs a;
  std::memset(&a, 0, sizeof a);
  a.uvw = (const vis_real *)p.uvw_coords;
  a.wavelengths = p.reference_wavelengths;
  a.spw = p.spw_index_array;
  a.field = p.field_array;
  a.flagged_rows = (const uint8_t *)p.flagged_rows;
  a.enabled = (const uint8_t *)p.enabled_channels;
  a.sf_cgi = p.sampling_function_channel_grid_indicies;
  a.counts = counts;
  a.nrows = (long long)p.row_count;
  a.nchan = (int)p.channel_count;
  a.nspw = (int)p.spw_count;
  a.nx = (int)p.nx;
  a.ny = (int)p.ny;
  a.sf_ch = (int)p.sampling_function_channel_count;
  a.imaging_field = p.imaging_field;
  // templated_gridder.h:23-24 in the data precision: nx (size_t) x cell x ARCSEC_TO_RAD (a float
  // constant, cu_common.h:63), evaluated left to right
  volatile vis_real sx = (vis_real)p.nx * p.cell_size_x;
  volatile vis_real sy = (vis_real)p.ny * p.cell_size_y;
  a.u_scale = sx * (vis_real)kArcsecToRad;
  a.v_scale = -(sy * (vis_real)kArcsecToRad);
  a.half_x = (vis_real)(p.nx >> 1);
  a.half_y = (vis_real)(p.ny >> 1);
  int *err = nullptr;
  if (cudaGetSymbolAddress((void **)&err, g_nn_error) != cudaSuccess) return BZ_ERR_CUDA;
  a.error = err;
  if (cudaMemsetAsync(err, 0, sizeof(int), st) != cudaSuccess) return BZ_ERR_CUDA;
  const long long n = a.nrows * a.nchan;
  if (n > 0) {
    const long long blocks = std::min<long long>((n + 255) / 256, 152LL * 32);
    sampling_counts_nn_kernel<<<(unsigned)blocks, 256, 0, st>>>(a);
    if (cudaGetLastError() != cudaSuccess) return BZ_ERR_CUDA;
  }
  for (size_t f = 1; f < F; ++f)
    if (cudaMemcpyAsync(counts + f * slab, counts, slab * sizeof(unsigned), cudaMemcpyDeviceToDevice, st) != cudaSuccess)
      return BZ_ERR_CUDA;
  int host_err = 0;
  if (cudaMemcpyAsync(&host_err, err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return BZ_ERR_CUDA;
  if (host_err) {
    bz_record_error(BZ_ERR_INVALID_ARGUMENT, "bullseye_sampling_counts_nn: %s index out of range",
                    (host_err & 1) ? "spw" : "sampling-function channel grid");
    return BZ_ERR_INVALID_ARGUMENT;
  }
  return BZ_OK;
}
