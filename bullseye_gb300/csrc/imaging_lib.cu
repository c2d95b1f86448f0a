// GB300 drop-in for the reference's GPU imaging libraries (libgpu_imaging32.so / 64.so).
//
// Exports the C-ABI of bullseye/mo/cpu_gpu_common/wrapper.h:41-61 with the call-sequencing
// contract of bullseye/mo/gpu_algorithm/wrapper.cu:
//   * initLibrary allocates device mirrors for chunk_max_row_count rows, uploads the tables and
//     the caller's grids, and publishes a library-owned normalisation array through
//     params.normalization_terms ([facets][cube][corr][W*W] float64, wrapper.cu:222-230; the sum
//     lands in bin 0, so normalize() -- which sums the bins -- sees the same value);
//   * gridding calls are asynchronous on one library stream; grids stay device resident and are
//     copied back to the caller's buffers when is_final_data_chunk is set (wrapper.cu:293-314);
//     gridding_barrier() synchronises;
//   * weight_uniformly / normalize operate on the caller's host buffers after the copy-back,
//     exactly as the reference (wrapper.cu:275-339);
//   * finalize / finalize_psf run the inverse FFT on the device (cuFFT) with the reference's
//     shift and float32 packing (fft_and_repacking_routines.cpp:83-161).
// Deliberate differences (none changes results):
//   * no cudaDeviceReset and no device selection: the current device is used (the reference
//     resets and picks the device with most SMs, wrapper.cu:89-112);
//   * errors never exit or throw: they are recorded (sticky) and readable through
//     bullseye_last_error(); calls after an error return without work until initLibrary;
//   * single/dual correlation selection happens on the device; caller arrays are not compacted
//     in place (the reference compacts them, wrapper.cu:482-490, 666-680);
//   * Jones terms are inverted on the device into a library buffer; the caller's array is left
//     unmodified (the reference GPU library inverts a host copy, wrapper.cu:1088);
//   * the Jones correction is applied (the reference GPU library launches the plain 4-correlation
//     policy for facet_4_cor_corrections, wrapper.cu:1125, so its GPU results ignore the terms;
//     the CPU library applies them, correlation_gridding_policies.h:523-542, and is the oracle).
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <numeric>
#include <string>
#include <chrono>
#include <thread>
#include <vector>

#include "common.h"
#include "gridder.cuh"
#include "kernels_misc.cuh"

using namespace bz;

// ------------------------------------------------------------------ error state
static std::mutex g_err_mutex;
static int g_err_code = BZ_OK;
static std::string g_err_msg;

void bz_record_error(int code, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  std::lock_guard<std::mutex> lk(g_err_mutex);
  if (g_err_code == BZ_OK) {  // keep the first error
    g_err_code = code;
    g_err_msg = buf;
  }
}
int bz_error_code() {
  std::lock_guard<std::mutex> lk(g_err_mutex);
  return g_err_code;
}
static void bz_clear_error() {
  std::lock_guard<std::mutex> lk(g_err_mutex);
  g_err_code = BZ_OK;
  g_err_msg.clear();
}

#include "context.h"

Context g_ctx;
void bz_release_batched();
void bz_release_fft_plans();

static bool check_ready(const char *fn) {
  if (!g_ctx.initialized) {
    bz_record_error(BZ_ERR_NOT_INITIALISED, "%s called before initLibrary", fn);
    return false;
  }
  return bz_error_code() == BZ_OK;
}

static void drain_device_error() {
  int h = 0;
  if (g_ctx.dev_error.ptr && cudaMemcpy(&h, g_ctx.dev_error.ptr, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess && h) {
    if (h & DEV_ERR_SINGULAR) bz_record_error(BZ_ERR_SINGULAR_JONES, "Jones matrix set contains singular matrices");
    if (h & DEV_ERR_GRID_INDEX) bz_record_error(BZ_ERR_INVALID_ARGUMENT, "channel grid index out of range of the cube");
    if (h & DEV_ERR_JONES_INDEX) bz_record_error(BZ_ERR_INVALID_ARGUMENT, "timestamp or antenna id out of range of the Jones terms");
    if (h & DEV_ERR_WAIT_TIMEOUT) bz_record_error(BZ_ERR_CUDA, "gridder: a bounded wait for staged kernel taps ran out");
    if (h & DEV_ERR_ANTENNA) bz_record_error(BZ_ERR_INVALID_ARGUMENT, "antenna pair outside baseline_count");
    int z = 0;
    cudaMemcpy(g_ctx.dev_error.ptr, &z, sizeof(int), cudaMemcpyHostToDevice);
  }
}

// Fold the previous gridder launch's event interval into the per-kind totals.
static void settle_kernel_timing() {
  Context &c = g_ctx;
  if (!c.kernel_timing_pending) return;
  float ms = 0;
  cudaEventSynchronize(c.ev_k1);
  if (cudaEventElapsedTime(&ms, c.ev_k0, c.ev_k1) == cudaSuccess) c.kernel_ms[c.kernel_timing_kind] += ms;
  c.kernel_timing_pending = false;
}

// ------------------------------------------------------------------ exported API

extern "C" int bullseye_last_error(char *buf, size_t n) {
  std::lock_guard<std::mutex> lk(g_err_mutex);
  if (buf && n) {
    snprintf(buf, n, "%s", g_err_msg.c_str());
  }
  return g_err_code;
}

extern "C" void bullseye_clear_error() { bz_clear_error(); }

extern "C" int bullseye_precision_bits() { return BZ_PRECISION_BITS; }

extern "C" void bullseye_set_compensated(int on) { g_ctx.compensated = on != 0; }

// See include/bullseye_gb300.h.
extern "C" void bullseye_set_batched_calls(int on) { g_ctx.batched_calls = on != 0; }

// See include/bullseye_gb300.h.
extern "C" void bullseye_set_jones_time_major(int on) {
  g_ctx.jones_time_major = on != 0;
  if (!on) g_ctx.jones_inv_t.release();  // stream-ordered: after the calls already queued
}

// ---------------------------------------------------------------- phase tracing
namespace {
struct Trace {
  bool on = false;
  std::chrono::steady_clock::time_point last;
  std::string log;  // "phase ms; " entries since the last report
} g_trace;
}  // namespace

void bz_trace_begin() {
  if (!g_trace.on) return;
  if (g_ctx.stream) cudaStreamSynchronize(g_ctx.stream);
  g_trace.last = std::chrono::steady_clock::now();
}

void bz_trace_mark(const char *phase) {
  if (!g_trace.on) return;
  if (g_ctx.stream) cudaStreamSynchronize(g_ctx.stream);
  if (g_ctx.copy_stream) cudaStreamSynchronize(g_ctx.copy_stream);
  if (g_ctx.jones_stream) cudaStreamSynchronize(g_ctx.jones_stream);
  const auto now = std::chrono::steady_clock::now();
  const double ms = std::chrono::duration<double, std::milli>(now - g_trace.last).count();
  g_trace.last = now;
  char buf[96];
  snprintf(buf, sizeof buf, "%s %.3f; ", phase, ms);
  if (g_trace.log.size() < (1u << 16)) g_trace.log += buf;
}

bool bz_tracing() { return g_trace.on; }

void bz_trace_note(const char *fmt, ...) {
  if (!g_trace.on) return;
  char buf[160];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (g_trace.log.size() < (1u << 16)) (g_trace.log += buf) += "; ";
}

const char *bz_host_kind(const void *p) {
  cudaPointerAttributes at{};
  if (!p) return "null";
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return "unknown";
  }
  switch (at.type) {
    case cudaMemoryTypeHost: return "pinned";
    case cudaMemoryTypeDevice: return "device";
    case cudaMemoryTypeManaged: return "managed";
    default: return "pageable";
  }
}

// See include/bullseye_gb300.h.
extern "C" void bullseye_set_tracing(int on) {
  g_trace.on = on != 0;
  g_trace.log.clear();
}

// See include/bullseye_gb300.h.
extern "C" size_t bullseye_trace_report(char *buf, size_t n) {
  const size_t len = g_trace.log.size();
  if (buf && n) {
    snprintf(buf, n, "%s", g_trace.log.c_str());
    g_trace.log.clear();
  }
  return len;
}

// Device-resident inputs: when on, the row arrays (visibilities, weights, flags, uvw, flagged
// rows, field, spw, antenna and timestamp ids), jones_terms and baseline_starting_indexes in
// gridding_parameters are device pointers already in baseline-major order; the gridding calls
// then copy nothing from the host.  Tables and grids are still owned by the library.
extern "C" void bullseye_set_device_inputs(int on) { g_ctx.device_inputs = on != 0; }

// The library's CUDA stream (all its work is ordered on it); null before initLibrary.
extern "C" void *bullseye_get_stream() { return (void *)g_ctx.stream; }

// Number of kernels this library launched since initLibrary (cuFFT's internal launches excluded).
extern "C" long long bullseye_kernel_launches() { return g_ctx.launches; }

// Accumulated device time of the gridder kernels (ms, CUDA events around each launch) and the
// number of gridder launches timed, since initLibrary or the last reset.
// kind 0: visibility gridding launches, kind 1: sampling-function launches.
extern "C" double bullseye_gridder_kernel_ms(int kind, long long *count) {
  Context &c = g_ctx;
  if (kind < 0 || kind > 1) return 0.0;
  settle_kernel_timing();
  if (count) *count = c.kernel_count[kind];
  return c.kernel_ms[kind];
}

extern "C" void bullseye_reset_counters() {
  Context &c = g_ctx;
  settle_kernel_timing();
  c.kernel_ms[0] = c.kernel_ms[1] = 0;
  c.kernel_count[0] = c.kernel_count[1] = 0;
  c.launches = 0;
}

// Measured FP32 FMA throughput of this GPU (TFLOP/s): independent FMA chains in registers on
// every SM, timed with CUDA events.  The denominator of the gridder's FP32 roofline.
extern "C" double bullseye_fp32_fma_tflops(int iters) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return 0.0;
  const int threads = 256, blocks = sms * 8;
  float *out = nullptr;
  if (cudaMalloc(&out, sizeof(float) * threads * blocks) != cudaSuccess) return 0.0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fma_probe_kernel<<<blocks, threads>>>(out, iters);  // warm-up
  cudaEventRecord(e0);
  fma_probe_kernel<<<blocks, threads>>>(out, iters);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  double flops = 2.0 * kFmaProbeChains * (double)iters * threads * blocks;
  return ms > 0 ? flops / (ms * 1e-3) / 1e12 : 0.0;
}

// Zero the device-resident grids, compensation grids and normalisation sums (a fresh image
// without reallocating; the caller's host buffers are untouched).
extern "C" void bullseye_zero_grids() {
  Context &c = g_ctx;
  if (!check_ready("bullseye_zero_grids")) return;
  const size_t nxy = c.nx * c.ny;
  BZ_CUDA_TRY(cudaMemsetAsync(c.grid.ptr, 0, sizeof(vis_complex) * c.F * c.cube * c.C * nxy, c.stream));
  if (c.grid_lo.ptr) BZ_CUDA_TRY(cudaMemsetAsync(c.grid_lo.ptr, 0, sizeof(vis_complex) * c.F * c.cube * c.C * nxy, c.stream));
  if (c.sf.ptr) BZ_CUDA_TRY(cudaMemsetAsync(c.sf.ptr, 0, sizeof(vis_complex) * c.F * c.sf_count * nxy, c.stream));
  if (c.sf_acc.ptr) BZ_CUDA_TRY(cudaMemsetAsync(c.sf_acc.ptr, 0, sizeof(vis_complex) * c.sf_count * nxy, c.stream));
  if (c.sf_lo.ptr) BZ_CUDA_TRY(cudaMemsetAsync(c.sf_lo.ptr, 0, sizeof(vis_complex) * c.sf_count * nxy, c.stream));
  BZ_CUDA_TRY(cudaMemsetAsync(c.norm.ptr, 0, sizeof(double) * c.F * c.cube * c.C, c.stream));
}

extern "C" double get_gridding_walltime() {
  if (g_ctx.grid_timing_pending && g_ctx.ev_g1) {
    cudaEventSynchronize(g_ctx.ev_g1);
  }
  return g_ctx.grid_seconds;
}

extern "C" double get_inversion_walltime() { return g_ctx.inv_seconds; }

// Publishes the normalisation sums of the last copy-back (copied into pinned memory on the copy
// stream) as the library-owned host terms, in the reference GPU library's [F][cube][C][W*W] layout
// (the sum in bin 0).
static void publish_norms() {
  Context &c = g_ctx;
  if (!c.norm_pending) return;
  const size_t bins = c.W * c.W, n = c.F * c.cube * c.C;
  std::fill(c.host_norm.begin(), c.host_norm.end(), 0.0);
  for (size_t i = 0; i < n; ++i) c.host_norm[i * bins] = c.norm_host[i];
  c.norm_pending = false;
}

// Waits for the library stream and the copy stream (row uploads, copy-backs); after it the caller
// may change its arrays, so rows on the device are no longer taken for the caller's.
extern "C" void gridding_barrier() {
  if (!g_ctx.initialized || !g_ctx.stream) return;
  cudaError_t e = cudaStreamSynchronize(g_ctx.stream);
  if (e == cudaSuccess && g_ctx.copy_stream) e = cudaStreamSynchronize(g_ctx.copy_stream);
  if (e == cudaSuccess && g_ctx.jones_stream) e = cudaStreamSynchronize(g_ctx.jones_stream);
  if (e != cudaSuccess) {
    bz_record_error(BZ_ERR_CUDA, "gridding_barrier: %s", cudaGetErrorString(e));
    return;
  }
  publish_norms();
  bz_forget_rows();
  drain_device_error();
}

static void timer_start() {
  if (g_ctx.grid_timing_pending) {
    float ms = 0;
    cudaEventSynchronize(g_ctx.ev_g1);
    if (cudaEventElapsedTime(&ms, g_ctx.ev_g0, g_ctx.ev_g1) == cudaSuccess) g_ctx.grid_seconds += ms * 1e-3;
    g_ctx.grid_timing_pending = false;
  }
  cudaEventRecord(g_ctx.ev_g0, g_ctx.stream);
}
static void timer_stop() {
  cudaEventRecord(g_ctx.ev_g1, g_ctx.stream);
  g_ctx.grid_timing_pending = true;
}

extern "C" void releaseLibrary();

extern "C" void initLibrary(gridding_parameters *pp) {
  if (g_ctx.initialized) return;  // as the reference (wrapper.cu:82)
  bz_clear_error();
  gridding_parameters &p = *pp;
  Context &c = g_ctx;
  if (cudaGetDevice(&c.device) != cudaSuccess) {
    bz_record_error(BZ_ERR_CUDA, "no CUDA device available");
    return;
  }
  if (p.nx == 0 || p.ny == 0 || p.conv_oversample == 0 || p.channel_count == 0 || p.spw_count == 0) {
    bz_record_error(BZ_ERR_INVALID_ARGUMENT, "initLibrary: nx, ny, conv_oversample, channel_count and spw_count must be > 0");
    return;
  }
  c.F = std::max<size_t>(1, p.num_facet_centres);
  c.cube = p.cube_channel_dim_size;
  c.C = p.number_of_polarization_terms_being_gridded;
  c.nx = p.nx;
  c.ny = p.ny;
  c.W = 2 * p.conv_support + 1;
  c.os = p.conv_oversample;
  c.K = (c.W + 2) + (c.W + 1) * (c.os - 1);
  c.P = std::max<size_t>(1, p.wplanes);
  c.nchan = p.channel_count;
  c.nspw = p.spw_count;
  c.npol = p.number_of_polarization_terms;
  c.max_rows = p.chunk_max_row_count;
  c.baselines = p.baseline_count;
  c.want_sf = p.should_grid_sampling_function;
  c.sf_count = c.want_sf ? p.sampling_function_channel_count : 0;
  c.grid_seconds = c.inv_seconds = 0;
  c.grid_timing_pending = c.inv_timing_pending = false;
  if (c.C != 1 && c.C != 2 && c.C != 4) {
    bz_record_error(BZ_ERR_INVALID_ARGUMENT, "number_of_polarization_terms_being_gridded must be 1, 2 or 4");
    return;
  }
  if (c.cube == 0) {
    bz_record_error(BZ_ERR_INVALID_ARGUMENT, "cube_channel_dim_size must be > 0");
    return;
  }
  if (!p.conv) {
    bz_record_error(BZ_ERR_INVALID_ARGUMENT, "initLibrary: conv is null");
    return;
  }
  BZ_CUDA_TRY(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
  BZ_CUDA_TRY(cudaStreamCreateWithFlags(&c.copy_stream, cudaStreamNonBlocking));
  BZ_CUDA_TRY(cudaStreamCreateWithFlags(&c.jones_stream, cudaStreamNonBlocking));
  for (cudaEvent_t *ev : {&c.ev_stage_full[0], &c.ev_stage_full[1], &c.ev_stage_free[0], &c.ev_stage_free[1], &c.ev_jones_up,
                          &c.ev_jones_read, &c.ev_ready_vis, &c.ev_ready_sf, &c.ev_copied_vis, &c.ev_copied_sf})
    BZ_CUDA_TRY(cudaEventCreateWithFlags(ev, cudaEventDisableTiming));
  c.norm_pending = false;
  c.stage_rows = 0;
  bz_forget_rows();
  BZ_CUDA_TRY(cudaEventCreate(&c.ev_g0));
  BZ_CUDA_TRY(cudaEventCreate(&c.ev_g1));
  BZ_CUDA_TRY(cudaEventCreate(&c.ev_i0));
  BZ_CUDA_TRY(cudaEventCreate(&c.ev_i1));
  BZ_CUDA_TRY(cudaEventCreate(&c.ev_k0));
  BZ_CUDA_TRY(cudaEventCreate(&c.ev_k1));
  c.launches = 0;
  c.kernel_ms[0] = c.kernel_ms[1] = 0;
  c.kernel_count[0] = c.kernel_count[1] = 0;
  c.kernel_timing_pending = false;
  const size_t sc = c.nchan * c.nspw;
  const size_t nxy = c.nx * c.ny;
  const bool wproj = p.wplanes > 1;
  const size_t conv_elems = wproj ? c.P * c.K * 2 : c.K;
  bool ok = c.conv.alloc(conv_elems) && c.wavelengths.alloc(sc) && c.enabled.alloc(sc) && c.cgi.alloc(sc) &&
            c.sf_cgi.alloc(sc) && c.facet_centres.alloc(2 * c.F) && c.facets.alloc(c.F) &&
            c.dev_error.alloc(1) && c.norm.alloc(c.F * c.cube * c.C);
  if (!ok) return;
  BZ_CUDA_TRY(cudaMemcpy(c.conv.ptr, p.conv, sizeof(vis_real) * conv_elems, cudaMemcpyHostToDevice));
  c.conv_host.assign(p.conv, p.conv + conv_elems);
  {
    // row sums of the kernel for every (plane, tap offset): tap offsets span [0, 2 os]
    c.tap_f = 2 * c.os + 1;
    std::vector<double> sums(2 * c.P * c.tap_f, 0.0);
    const size_t W = c.W;
    for (size_t pl = 0; pl < c.P; ++pl)
      for (size_t f = 0; f < c.tap_f; ++f) {
        double re = 0, im = 0;
        for (size_t j = 0; j < W; ++j) {
          const size_t i = f + j * c.os;
          if (i >= c.K) break;
          if (wproj) {
            re += (double)c.conv_host[2 * (pl * c.K + i)];
            im += (double)c.conv_host[2 * (pl * c.K + i) + 1];
          } else {
            re += (double)c.conv_host[i];
          }
        }
        sums[2 * (pl * c.tap_f + f)] = re;
        sums[2 * (pl * c.tap_f + f) + 1] = im;
      }
    if (!c.tap_sums.alloc(sums.size())) return;
    BZ_CUDA_TRY(cudaMemcpy(c.tap_sums.ptr, sums.data(), sizeof(double) * sums.size(), cudaMemcpyHostToDevice));
    std::vector<float> sums_f(sums.begin(), sums.end());
    if (!c.tap_sums_f.alloc(sums_f.size())) return;
    BZ_CUDA_TRY(cudaMemcpy(c.tap_sums_f.ptr, sums_f.data(), sizeof(float) * sums_f.size(), cudaMemcpyHostToDevice));
    // regrouped table: entry (plane, f, j) = conv[plane][f + j os], zero past the row
    const size_t ncomp = wproj ? 2 : 1;
    std::vector<vis_real> regrouped(ncomp * c.P * c.tap_f * W, (vis_real)0);
    for (size_t pl = 0; pl < c.P; ++pl)
      for (size_t f = 0; f < c.tap_f; ++f)
        for (size_t j = 0; j < W; ++j) {
          const size_t i = f + j * c.os;
          if (i >= c.K) break;
          for (size_t q = 0; q < ncomp; ++q)
            regrouped[ncomp * ((pl * c.tap_f + f) * W + j) + q] = c.conv_host[ncomp * (pl * c.K + i) + q];
        }
    if (!c.conv_t.alloc(regrouped.size())) return;
    BZ_CUDA_TRY(cudaMemcpy(c.conv_t.ptr, regrouped.data(), sizeof(vis_real) * regrouped.size(), cudaMemcpyHostToDevice));
  }
  BZ_CUDA_TRY(cudaMemcpy(c.wavelengths.ptr, p.reference_wavelengths, sizeof(vis_real) * sc, cudaMemcpyHostToDevice));
  BZ_CUDA_TRY(cudaMemcpy(c.enabled.ptr, p.enabled_channels, sc, cudaMemcpyHostToDevice));
  BZ_CUDA_TRY(cudaMemcpy(c.cgi.ptr, p.channel_grid_indicies, sizeof(size_t) * sc, cudaMemcpyHostToDevice));
  if (c.want_sf && p.sampling_function_channel_grid_indicies)
    BZ_CUDA_TRY(cudaMemcpy(c.sf_cgi.ptr, p.sampling_function_channel_grid_indicies, sizeof(size_t) * sc,
                           cudaMemcpyHostToDevice));
  if (p.facet_centres)
    BZ_CUDA_TRY(cudaMemcpy(c.facet_centres.ptr, p.facet_centres, sizeof(vis_real) * 2 * c.F, cudaMemcpyHostToDevice));
  BZ_CUDA_TRY(cudaMemset(c.dev_error.ptr, 0, sizeof(int)));
  BZ_CUDA_TRY(cudaMemset(c.norm.ptr, 0, sizeof(double) * c.F * c.cube * c.C));
  BZ_CUDA_TRY(cudaHostAlloc((void **)&c.norm_host, sizeof(double) * c.F * c.cube * c.C, cudaHostAllocDefault));
  // row buffers are allocated on the first host-input gridding call (ensure_row_buffers)
  // grids: the caller's initial contents are uploaded (wrapper.cu:179-186)
  const size_t ng = c.F * c.cube * c.C * nxy;
  if (!c.grid.alloc(ng) || !c.scratch.alloc(std::max(ng, c.F * std::max<size_t>(1, c.sf_count) * nxy))) return;
  if (p.output_buffer) {
    if (!bz_copy_async(c.grid.ptr, p.output_buffer, sizeof(vis_complex) * ng, cudaMemcpyHostToDevice, c.stream)) return;
    BZ_CUDA_TRY(cudaStreamSynchronize(c.stream));
  } else
    BZ_CUDA_TRY(cudaMemset(c.grid.ptr, 0, sizeof(vis_complex) * ng));
#if defined(BULLSEYE_SINGLE)
  if (!c.grid_lo.alloc(ng)) return;
  BZ_CUDA_TRY(cudaMemset(c.grid_lo.ptr, 0, sizeof(vis_complex) * ng));
#endif
  if (c.want_sf) {
    const size_t ns = c.F * c.sf_count * nxy;
    if (!c.sf.alloc(ns)) return;
    if (p.sampling_function_buffer) {
      if (!bz_copy_async(c.sf.ptr, p.sampling_function_buffer, sizeof(vis_complex) * ns, cudaMemcpyHostToDevice,
                         c.stream))
        return;
      BZ_CUDA_TRY(cudaStreamSynchronize(c.stream));
    } else
      BZ_CUDA_TRY(cudaMemset(c.sf.ptr, 0, sizeof(vis_complex) * ns));
    if (!c.sf_out.alloc(ns)) return;
    const size_t na = c.sf_count * nxy;
    if (!c.sf_acc.alloc(na)) return;
    BZ_CUDA_TRY(cudaMemset(c.sf_acc.ptr, 0, sizeof(vis_complex) * na));
#if defined(BULLSEYE_SINGLE)
    if (!c.sf_lo.alloc(na)) return;
    BZ_CUDA_TRY(cudaMemset(c.sf_lo.ptr, 0, sizeof(vis_complex) * na));
#endif
  }
  // library-owned normalisation terms in the GPU library's layout
  const size_t bins = c.W * c.W;
  c.host_norm.assign(c.F * c.cube * c.C * bins, 0.0);
  p.normalization_terms = c.host_norm.data();
  c.have_corr = false;
  c.initialized = true;
}

extern "C" void releaseLibrary() {
  Context &c = g_ctx;
  if (!c.initialized) return;
  if (c.stream) cudaStreamSynchronize(c.stream);
  if (c.copy_stream) cudaStreamSynchronize(c.copy_stream);
  if (c.jones_stream) cudaStreamSynchronize(c.jones_stream);
  // buffers go back to the library's memory pool (ordered on the library stream)
  c.conv.release(); c.tap_sums.release(); c.tap_sums_f.release(); c.conv_t.release(); c.wavelengths.release(); c.facet_centres.release(); c.enabled.release();
  c.cgi.release(); c.sf_cgi.release(); c.vis.release(); c.weights.release(); c.uvw.release();
  c.flags.release(); c.flagged_rows.release(); c.field.release(); c.spw.release(); c.ant1.release();
  c.ant2.release(); c.time_ids.release(); c.starts.release(); c.jones_raw.release(); c.jones_inv.release(); c.jones_inv_t.release();
  c.facets.release(); c.facets_sf.release(); c.grid.release(); c.grid_lo.release(); c.sf.release(); c.sf_acc.release(); c.sf_lo.release();
  c.scratch.release(); c.sf_out.release(); c.norm.release(); c.dev_error.release(); c.corr_x.release(); c.corr_y.release();
  for (StageBuf &g : c.stage) {
    g.vis.release(); g.weights.release(); g.uvw.release(); g.flags.release(); g.flagged_rows.release();
    g.field.release(); g.spw.release(); g.ant1.release(); g.ant2.release(); g.time_ids.release();
  }
  c.sort_keys.release(); c.sort_vals.release(); c.sort_tmp.release(); c.track_starts.release();
  c.stage_rows = 0;
  bz_forget_rows();
  bz_release_batched();
  bz_release_fft_plans();
  if (c.stream) cudaStreamSynchronize(c.stream);
  for (cudaEvent_t *ev : {&c.ev_g0, &c.ev_g1, &c.ev_i0, &c.ev_i1, &c.ev_k0, &c.ev_k1, &c.ev_stage_full[0],
                          &c.ev_stage_full[1], &c.ev_stage_free[0], &c.ev_stage_free[1], &c.ev_jones_up, &c.ev_jones_read,
                          &c.ev_ready_vis, &c.ev_ready_sf, &c.ev_copied_vis, &c.ev_copied_sf}) {
    if (*ev) cudaEventDestroy(*ev);
    *ev = nullptr;
  }
  if (c.copy_stream) cudaStreamDestroy(c.copy_stream);
  c.copy_stream = nullptr;
  if (c.jones_stream) cudaStreamDestroy(c.jones_stream);
  c.jones_stream = nullptr;
  if (c.stream) cudaStreamDestroy(c.stream);
  c.stream = nullptr;
  if (c.norm_host) cudaFreeHost(c.norm_host);
  c.norm_host = nullptr;
  c.norm_pending = false;
  c.host_norm.clear();
  c.host_norm.shrink_to_fit();
  c.conv_host.clear();
  c.initialized = false;
}

// ---------------------------------------------------------------- repack (host, as reference)
static long baseline_slot(long a1, long a2, long n) {
  long s = std::min(a1, a2);
  return (s * (-s + (2 * n + 1))) / 2 + std::labs(a1 - a2);
}

// Stable counting sort of the chunk's rows into baseline-major order, in place on the caller's
// arrays, filling baseline_starting_indexes (bullseye/mo/gpu_algorithm/wrapper.cu:367-454).
extern "C" void repack_input_data(gridding_parameters *pp) {
  gridding_parameters &p = *pp;
  // pure host work: usable before initLibrary, like the reference (wrapper.cu:367)
  if (bz_error_code() != BZ_OK) return;
  if (!p.baseline_starting_indexes || !p.antenna_1_ids || !p.antenna_2_ids) {
    bz_record_error(BZ_ERR_INVALID_ARGUMENT, "repack_input_data: baseline_starting_indexes and antenna ids are required");
    return;
  }
  const size_t R = p.row_count, B = p.baseline_count, per = p.channel_count * p.number_of_polarization_terms;
  std::vector<size_t> slot(R);
  std::fill(p.baseline_starting_indexes, p.baseline_starting_indexes + B + 1, 0);
  for (size_t r = 0; r < R; ++r) {
    long b = baseline_slot(p.antenna_1_ids[r], p.antenna_2_ids[r], (long)p.antenna_count);
    if (b < 0 || (size_t)b >= B) {
      bz_record_error(BZ_ERR_INVALID_ARGUMENT, "repack_input_data: antenna pair outside baseline_count");
      return;
    }
    slot[r] = (size_t)b;
    ++p.baseline_starting_indexes[b + 1];
  }
  std::partial_sum(p.baseline_starting_indexes, p.baseline_starting_indexes + B + 1, p.baseline_starting_indexes);
  // bullseye_set_host_repack(0): the gridding calls sort their rows by baseline on the device, so
  // the caller's arrays stay in place and only the baseline starts are reported
  if (!g_ctx.host_repack) return;
  std::vector<size_t> dest(R), cursor(p.baseline_starting_indexes, p.baseline_starting_indexes + B);
  for (size_t r = 0; r < R; ++r) dest[r] = cursor[slot[r]]++;
  auto permute = [&](auto *arr, size_t width) {
    if (!arr) return;
    const size_t esz = sizeof(*arr) * width;
    unsigned char *bytes = reinterpret_cast<unsigned char *>(arr);
    std::vector<unsigned char> tmp(bytes, bytes + R * esz);
    for (size_t r = 0; r < R; ++r) std::memcpy(bytes + dest[r] * esz, tmp.data() + r * esz, esz);
  };
  permute(p.uvw_coords, 1);
  permute(p.visibilities, per);
  permute(p.visibility_weights, per);
  permute(p.flags, per);
  permute(p.flagged_rows, 1);
  permute(p.spw_index_array, 1);
  permute(p.antenna_1_ids, 1);
  permute(p.antenna_2_ids, 1);
  permute(p.field_array, 1);
  if (p.should_invert_jones_terms) permute(p.timestamp_ids, 1);
}

// ---------------------------------------------------------------- gridding launch
FacetXform bz_facet_xform(double ra0, double dec0, double ra, double dec, bool phase, bool uvx) {
  // phase_transform_policies.h:110-134 and baseline_transform_policies.h:117-149, in FP64
  FacetXform x;
  std::memset(&x, 0, sizeof x);
  const double k = (double)kArcsecToRad;
  double d_ra = (ra - ra0) * k, n_dec = dec * k, o_dec = dec0 * k;
  double c_d_ra = cos(d_ra), s_d_ra = sin(d_ra), c_n = cos(n_dec), s_n = sin(n_dec), c_o = cos(o_dec),
         s_o = sin(o_dec);
  if (uvx) {
    double li0 = c_n * s_d_ra, mi0 = s_n * c_o - c_n * s_o * c_d_ra, ni0 = s_n * s_o + c_n * c_o * c_d_ra;
    x.u_term = li0 / ni0;
    x.v_term = mi0 / ni0;
  }
  if (phase) {
    x.dl = -c_n * s_d_ra;
    x.dm = -(s_n * c_o - c_n * s_o * c_d_ra);
    x.dn = 1.0 - sqrt(1.0 - x.dl * x.dl - x.dm * x.dm);
  }
  return x;
}

struct LaunchShape {
  int J, NT, V;
  bool wide;
  size_t smem;
};

// Ownership layout for full support W: J rows per thread; WIDE pads columns to a multiple of 32
// (chosen when that wastes at most 1/8 of the columns) so each warp holds one strip.
template <int NC, bool WPROJ>
static LaunchShape choose_shape(int W) {
  LaunchShape s;
  s.J = 0;
  s.wide = false;
  const int cols = ((W + 31) / 32) * 32;
  if ((cols - W) * 8 <= W) {
    for (int j : {2, 8}) {
      if (cols * ((W + j - 1) / j) <= 512) {
        s.J = j;
        s.wide = true;
        break;
      }
    }
  }
  if (!s.J) {
    for (int j : {1, 2, 4, 8, 16}) {
      if (W * ((W + j - 1) / j) <= 512) {
        s.J = j;
        break;
      }
    }
  }
  if (!s.J) s.J = 16;
  const int owners = s.wide ? cols * ((W + s.J - 1) / s.J) : W * ((W + s.J - 1) / s.J);
  s.NT = std::max(32, ((owners + 31) / 32) * 32);
  s.V = grid_chunk_size<NC, WPROJ>(W, s.NT, s.J);
  s.smem = grid_smem_bytes<NC, WPROJ>(s.V, W, s.NT, s.J);
  return s;
}

template <int NC, bool WPROJ, int J, bool WIDE>
static bool launch_j(const GridArgs &a, const LaunchShape &s, long long blocks, cudaStream_t st, bool comp) {
  void (*kern)(const GridArgs);
#if defined(BULLSEYE_SINGLE)
  if (comp)
    kern = romein_grid_kernel<NC, WPROJ, J, true, WIDE>;
  else
    kern = romein_grid_kernel<NC, WPROJ, J, false, WIDE>;
#else
  (void)comp;  // FP64 accumulation needs no compensation
  kern = romein_grid_kernel<NC, WPROJ, J, false, WIDE>;
#endif
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s.smem) != cudaSuccess) {
    bz_record_error(BZ_ERR_CUDA, "cudaFuncSetAttribute failed");
    return false;
  }
  kern<<<(unsigned)blocks, s.NT, s.smem, st>>>(a);
  g_ctx.launches++;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    bz_record_error(BZ_ERR_CUDA, "gridder launch failed: %s", cudaGetErrorString(e));
    return false;
  }
  return true;
}

template <int NC, bool WPROJ>
static bool launch_nc(GridArgs a, long long blocks, cudaStream_t st, bool comp) {
  LaunchShape s = choose_shape<NC, WPROJ>(a.W);
  if (s.NT > 512) {
    bz_record_error(BZ_ERR_UNSUPPORTED, "full support %d is larger than this build supports", a.W);
    return false;
  }
  a.V = s.V;
  if (s.wide) {
    if (s.J == 2) return launch_j<NC, WPROJ, 2, true>(a, s, blocks, st, comp);
    return launch_j<NC, WPROJ, 8, true>(a, s, blocks, st, comp);
  }
  switch (s.J) {
    case 1: return launch_j<NC, WPROJ, 1, false>(a, s, blocks, st, comp);
    case 2: return launch_j<NC, WPROJ, 2, false>(a, s, blocks, st, comp);
    case 4: return launch_j<NC, WPROJ, 4, false>(a, s, blocks, st, comp);
    case 8: return launch_j<NC, WPROJ, 8, false>(a, s, blocks, st, comp);
    default: return launch_j<NC, WPROJ, 16, false>(a, s, blocks, st, comp);
  }
}

static bool launch_gridder(const GridArgs &a, int nc, bool wproj, long long blocks, cudaStream_t st, bool comp) {
  if (blocks <= 0) return true;
  if (blocks > 0x7fffffffLL) {
    bz_record_error(BZ_ERR_UNSUPPORTED, "too many gridding work items in one chunk");
    return false;
  }
  if (nc == 1) return wproj ? launch_nc<1, true>(a, blocks, st, comp) : launch_nc<1, false>(a, blocks, st, comp);
  if (nc == 2) return wproj ? launch_nc<2, true>(a, blocks, st, comp) : launch_nc<2, false>(a, blocks, st, comp);
  return wproj ? launch_nc<4, true>(a, blocks, st, comp) : launch_nc<4, false>(a, blocks, st, comp);
}

// Track setup of device-resident inputs (bullseye_set_device_inputs): the caller's baseline starts
// (device pointer) or fixed 256-row segments.
static void device_tracks(const gridding_parameters &p, int &nslots, int &seg, const size_t **starts_dev) {
  if (p.baseline_starting_indexes) {
    *starts_dev = p.baseline_starting_indexes;
    nslots = (int)p.baseline_count;
    seg = 0;
    return;
  }
  *starts_dev = nullptr;
  seg = 256;
  nslots = (int)((p.row_count + seg - 1) / seg);
}

bool bz_check_ready(const char *fn) { return check_ready(fn); }
void bz_copy_back_grids(gridding_parameters &p, bool sampling);
// Final-chunk copy-back, queued without waiting: the resolved grids (hi + lo) and the normalisation
// sums are copied to the caller's buffers on the copy stream, overlapping whatever the library
// stream does next (the sampling-function call of the chunk); gridding_barrier waits for them and
// publishes the normalisation terms.  A copy-back buffer is rewritten only after its previous copy.
static void copy_back_grids(gridding_parameters &p, bool sampling) {
  Context &c = g_ctx;
  const size_t nxy = c.nx * c.ny;
  if (!sampling) {
    const size_t n = c.F * c.cube * c.C * nxy;
    BZ_CUDA_TRY(cudaStreamWaitEvent(c.stream, c.ev_copied_vis, 0));
    resolve_compensated_kernel<<<1024, 256, 0, c.stream>>>(c.grid.ptr, c.grid_lo.ptr, c.scratch.ptr, (long long)n);
    c.launches++;
    BZ_CUDA_TRY(cudaEventRecord(c.ev_ready_vis, c.stream));
    BZ_CUDA_TRY(cudaStreamWaitEvent(c.copy_stream, c.ev_ready_vis, 0));
    if (p.output_buffer && !bz_copy_async(p.output_buffer, c.scratch.ptr, sizeof(vis_complex) * n, cudaMemcpyDeviceToHost,
                                          c.copy_stream))
      return;
    BZ_CUDA_TRY(cudaMemcpyAsync(c.norm_host, c.norm.ptr, sizeof(double) * c.F * c.cube * c.C, cudaMemcpyDeviceToHost,
                                c.copy_stream));
    BZ_CUDA_TRY(cudaEventRecord(c.ev_copied_vis, c.copy_stream));
    c.norm_pending = true;
  } else {
    const size_t n = c.F * c.sf_count * nxy;
    BZ_CUDA_TRY(cudaStreamWaitEvent(c.stream, c.ev_copied_sf, 0));
    broadcast_add_kernel<<<1024, 256, 0, c.stream>>>(c.sf.ptr, c.sf_acc.ptr, c.sf_lo.ptr, c.sf_out.ptr,
                                                    (long long)(c.sf_count * nxy), (long long)c.F);
    c.launches++;
    BZ_CUDA_TRY(cudaEventRecord(c.ev_ready_sf, c.stream));
    BZ_CUDA_TRY(cudaStreamWaitEvent(c.copy_stream, c.ev_ready_sf, 0));
    if (p.sampling_function_buffer && !bz_copy_async(p.sampling_function_buffer, c.sf_out.ptr, sizeof(vis_complex) * n,
                                                     cudaMemcpyDeviceToHost, c.copy_stream))
      return;
    BZ_CUDA_TRY(cudaEventRecord(c.ev_copied_sf, c.copy_stream));
  }
}

// Validation, uploads, Jones inversion, track setup and the per-facet transforms of one gridding
// call; fills the kernel arguments.  Shared by the per-call and the batched paths.
bool bz_prepare_grid_args(const gridding_parameters &p, int nc, int mode, bool faceting, GridArgs &a, int &nslots,
                          const char *name, bool upload) {
  Context &c = g_ctx;
  const bool sampling = mode == CORR_SAMPLING;
  if (sampling && !c.want_sf) {
    bz_record_error(BZ_ERR_INVALID_ARGUMENT, "%s: library initialised without should_grid_sampling_function", name);
    return false;
  }
  if (!sampling && (size_t)nc != c.C) {
    bz_record_error(BZ_ERR_INVALID_ARGUMENT, "%s grids %d correlations but the library was initialised for %zu", name, nc, c.C);
    return false;
  }
  if (nc == 4 && !sampling && c.npol != 4) {
    bz_record_error(BZ_ERR_INVALID_ARGUMENT, "%s needs 4 polarisation terms per visibility", name);
    return false;
  }
  if (!sampling && (p.polarization_index >= c.npol || (nc == 2 && p.second_polarization_index >= c.npol))) {
    bz_record_error(BZ_ERR_INVALID_ARGUMENT, "%s: polarization index out of range", name);
    return false;
  }
  const bool jones = mode == CORR_QUAD_JONES;
  // rows: device-resident inputs are used as they are; host inputs are streamed in chunks and
  // sorted by baseline on the device (rows.cu), into the library's row buffers and track table
  int seg = 0;
  const size_t *starts = nullptr;
  RowsPlan plan;
  if (c.device_inputs) {
    device_tracks(p, nslots, seg, &starts);
  } else {
    if (upload) {
      if (!bz_upload_rows(p, !sampling, jones, plan)) return false;
    } else if (!bz_plan_rows(p, plan)) {
      return false;
    }
    starts = c.track_starts.ptr;
    nslots = plan.chunks * (int)plan.slots;
  }
  bz_trace_mark("rows_h2d");
  bool jones_t_valid = false;
  if (jones) {
    const size_t nj = p.no_timestamps_read * p.antenna_count * c.F * c.nspw * c.nchan;
    if (!p.jones_terms || nj == 0) {
      bz_record_error(BZ_ERR_INVALID_ARGUMENT, "%s: jones_terms missing", name);
      return false;
    }
    if (c.jones_inv.n < 4 * nj && !c.jones_inv.alloc(4 * nj)) return false;
    const vis_complex *jsrc = p.jones_terms;
    if (!c.device_inputs) {
      // on its own stream, beside the row upload on the copy stream
      if (c.jones_raw.n < 4 * nj && !c.jones_raw.alloc(4 * nj)) return false;
      // the previous call's inversion must have read the buffer before it is refilled
      BZ_CUDA_TRY_RET(cudaStreamWaitEvent(c.jones_stream, c.ev_jones_read, 0), false);
      cudaEvent_t t0 = nullptr, t1 = nullptr;
      if (bz_tracing()) {
        bz_trace_mark("jones_alloc");
        cudaEventCreate(&t0);
        cudaEventCreate(&t1);
        cudaEventRecord(t0, c.jones_stream);
      }
      if (!bz_copy_async(c.jones_raw.ptr, p.jones_terms, sizeof(vis_complex) * 4 * nj, cudaMemcpyHostToDevice,
                         c.jones_stream))
        return false;
      if (t0) {
        cudaEventRecord(t1, c.jones_stream);
        cudaEventSynchronize(t1);
        float ms = 0;
        cudaEventElapsedTime(&ms, t0, t1);
        bz_trace_note("jones_copy %s%s %.1f MB %.3f ms %.1f GB/s", bz_host_kind(p.jones_terms),
                      c.host_copy_sm && bz_mapped_host(p.jones_terms, sizeof(vis_complex) * 4 * nj) ? " (SM copy)" : "",
                      sizeof(vis_complex) * 4.0 * nj / 1e6, ms, sizeof(vis_complex) * 4.0 * nj / (ms * 1e6));
        cudaEventDestroy(t0);
        cudaEventDestroy(t1);
      }
      BZ_CUDA_TRY_RET(cudaEventRecord(c.ev_jones_up, c.jones_stream), false);
      BZ_CUDA_TRY_RET(cudaStreamWaitEvent(c.stream, c.ev_jones_up, 0), false);
      jsrc = c.jones_raw.ptr;
    }
    bz_trace_mark("jones_h2d");
    // the batched gridder's record kernel reads a time-innermost copy (the 32 rows of a warp are
    // consecutive times): allocated when there is room, never an error when there is not
    const bool want_t = c.batched_calls && c.jones_time_major;
    if (want_t && c.jones_inv_t.n < 4 * nj) {
      c.jones_inv_t.release();
      void *pt = nullptr;
      if (bz_dev_alloc(&pt, sizeof(vis_complex) * 4 * nj)) {
        c.jones_inv_t.ptr = static_cast<vis_complex *>(pt);
        c.jones_inv_t.n = 4 * nj;
      } else {
        cudaGetLastError();
      }
    }
    vis_complex *jt = want_t && c.jones_inv_t.n >= 4 * nj ? c.jones_inv_t.ptr : nullptr;
    const JonesDims jd{(long long)p.no_timestamps_read, (long long)p.antenna_count, (long long)c.F, (long long)c.nspw,
                       (long long)c.nchan};
    invert_jones_kernel<<<(unsigned)((nj + 255) / 256), 256, 0, c.stream>>>(jsrc, c.jones_inv.ptr, (long long)nj,
                                                                             c.dev_error.ptr, jt, jd);
    jones_t_valid = jt != nullptr;
    BZ_CUDA_TRY_RET(cudaEventRecord(c.ev_jones_read, c.stream), false);
    c.launches++;
    bz_trace_mark("jones_invert");
  }
  // per-facet transforms (FP64, host)
  std::vector<FacetXform> fx(c.F);
  const double ra0 = (double)p.phase_centre_ra, dec0 = (double)p.phase_centre_dec;
  const bool phase = faceting && !sampling;
  for (size_t f = 0; f < c.F; ++f) {
    double ra = ra0, dec = dec0;
    if (phase && p.facet_centres) {
      ra = (double)p.facet_centres[2 * f];
      dec = (double)p.facet_centres[2 * f + 1];
    }
    // the sampling-function policy reports the phase centre as facet centre
    // (phase_transform_policies.h:77-82), so its uv transform is the identity
    fx[f] = bz_facet_xform(ra0, dec0, ra, dec, phase, faceting);
    // every facet shares the library's grid size: u_scale = nx * cell * ARCSEC_TO_RAD,
    // v_scale = -(ny * cell * ARCSEC_TO_RAD) (templated_gridder.h:23-24)
    fx[f].nx = (int)c.nx;
    fx[f].ny = (int)c.ny;
    fx[f].u_scale = (double)c.nx * (double)p.cell_size_x * (double)kArcsecToRad;
    fx[f].v_scale = -((double)c.ny * (double)p.cell_size_y * (double)kArcsecToRad);
    fx[f].gcx = (double)(c.nx / 2 - p.conv_support);
    fx[f].gcy = (double)(c.ny / 2 - p.conv_support);
    fx[f].grid_base = (long long)f * (long long)(sampling ? c.sf_count : c.cube) * (sampling ? 1 : nc) *
                      (long long)(c.nx * c.ny);
  }
  DevBuf<FacetXform> &table = sampling ? c.facets_sf : c.facets;
  if (table.n < c.F && !table.alloc(c.F)) return false;
  BZ_CUDA_TRY_RET(cudaMemcpyAsync(table.ptr, fx.data(), sizeof(FacetXform) * c.F, cudaMemcpyHostToDevice, c.stream), false);

  std::memset(&a, 0, sizeof a);
  if (c.device_inputs) {
    a.vis = p.visibilities; a.weights = p.visibility_weights; a.flags = (const uint8_t *)p.flags;
    a.uvw = (const vis_real *)p.uvw_coords; a.flagged_rows = (const uint8_t *)p.flagged_rows;
    a.field = p.field_array; a.spw = p.spw_index_array; a.ant1 = p.antenna_1_ids; a.ant2 = p.antenna_2_ids;
    a.time_ids = p.timestamp_ids;
  } else {
    a.vis = c.vis.ptr; a.weights = c.weights.ptr; a.flags = c.flags.ptr; a.uvw = c.uvw.ptr;
    a.flagged_rows = c.flagged_rows.ptr; a.field = c.field.ptr; a.spw = c.spw.ptr;
    a.ant1 = c.ant1.ptr; a.ant2 = c.ant2.ptr; a.time_ids = c.time_ids.ptr;
  }
  a.jones_inv = jones ? c.jones_inv.ptr : nullptr;
  a.jones_inv_t = jones && jones_t_valid ? c.jones_inv_t.ptr : nullptr;
  a.starts = starts;
  a.wavelengths = c.wavelengths.ptr; a.enabled = c.enabled.ptr;
  a.cgi = sampling ? c.sf_cgi.ptr : c.cgi.ptr;
  a.conv = c.conv.ptr;
  a.tap_sums = c.tap_sums.ptr;
  a.tap_sums_f = c.tap_sums_f.ptr;
  a.tap_f = (int)c.tap_f;
  a.conv_t = c.conv_t.ptr;
  a.facets = table.ptr;
  a.grid = sampling ? c.sf_acc.ptr : c.grid.ptr;
  a.grid_lo = nullptr;
#if defined(BULLSEYE_SINGLE)
  if (c.compensated) a.grid_lo = sampling ? c.sf_lo.ptr : c.grid_lo.ptr;
#endif
  a.norm = sampling ? nullptr : c.norm.ptr;
  a.error = c.dev_error.ptr;
  a.nrows = (long long)p.row_count;
  a.nchan = (int)c.nchan; a.npol = (int)c.npol;
  a.pol0 = (int)p.polarization_index; a.pol1 = (int)p.second_polarization_index;
  a.nspw = (int)c.nspw; a.nant = (int)p.antenna_count; a.ntimes = (int)p.no_timestamps_read;
  a.facet_base = 0; a.nfacets_total = (int)c.F;
  a.groups = (int)(sampling ? c.sf_count : c.cube);
  a.nx = (int)c.nx; a.ny = (int)c.ny; a.W = (int)c.W; a.os = (int)c.os; a.K = (int)c.K; a.P = (int)c.P;
  a.W_full = (int)c.W;
  a.mode = mode; a.phase = phase ? 1 : 0; a.uvx = faceting ? 1 : 0;
  a.nslots = nslots; a.seg = seg;
  a.imaging_field = p.imaging_field;
  // u_scale = nx * cell * ARCSEC_TO_RAD, v_scale = -(ny * cell * ARCSEC_TO_RAD) (templated_gridder.h:23-24)
  a.u_scale = (double)c.nx * (double)p.cell_size_x * (double)kArcsecToRad;
  a.v_scale = -((double)c.ny * (double)p.cell_size_y * (double)kArcsecToRad);
  a.gcx = (double)(c.nx / 2 - p.conv_support);
  a.gcy = (double)(c.ny / 2 - p.conv_support);
  a.wmax = (double)(float)p.wmax_est;  // the reference divides by (float)wmax_est
  return true;
}

static void grid_common(gridding_parameters *pp, int nc, int mode, bool faceting, const char *name) {
  gridding_parameters &p = *pp;
  if (!check_ready(name)) return;
  Context &c = g_ctx;
  const bool sampling = mode == CORR_SAMPLING;
  timer_start();
  if (c.batched_calls && c.C == 4 && (sampling || nc == 4)) {
    // the support-aware batched gridder (same results; see batched.cu)
    settle_kernel_timing();
    bz_trace_begin();
    cudaEventRecord(c.ev_k0, c.stream);
    if (!bz_grid_batched_call(p, mode, faceting, name)) return;
    cudaEventRecord(c.ev_k1, c.stream);
    c.kernel_timing_pending = true;
    c.kernel_timing_kind = sampling ? 1 : 0;
    c.kernel_count[c.kernel_timing_kind]++;
    if (p.is_final_data_chunk) {
      copy_back_grids(p, sampling);
      bz_trace_mark(sampling ? "sf.copy_back" : "vis.copy_back");
    }
    timer_stop();
    return;
  }
  GridArgs a;
  int nslots = 0;
  if (!bz_prepare_grid_args(p, nc, mode, faceting, a, nslots, name)) return;
  const int nc_launch = sampling ? 1 : nc;
  // the sampling function is identical for every facet: grid it once (facet 0)
  const long long blocks = (long long)(sampling ? 1 : c.F) * nslots * (long long)c.nchan;
  settle_kernel_timing();
  cudaEventRecord(c.ev_k0, c.stream);
  if (p.row_count > 0 && !launch_gridder(a, nc_launch, p.wplanes > 1, blocks, c.stream, a.grid_lo != nullptr)) return;
  cudaEventRecord(c.ev_k1, c.stream);
  c.kernel_timing_pending = true;
  c.kernel_timing_kind = sampling ? 1 : 0;
  c.kernel_count[c.kernel_timing_kind]++;
  if (p.is_final_data_chunk) copy_back_grids(p, sampling);
  timer_stop();
}

extern "C" void grid_single_pol(gridding_parameters *p) { grid_common(p, 1, CORR_SINGLE, false, "grid_single_pol"); }
extern "C" void facet_single_pol(gridding_parameters *p) { grid_common(p, 1, CORR_SINGLE, true, "facet_single_pol"); }
extern "C" void grid_duel_pol(gridding_parameters *p) { grid_common(p, 2, CORR_DUAL, false, "grid_duel_pol"); }
extern "C" void facet_duel_pol(gridding_parameters *p) { grid_common(p, 2, CORR_DUAL, true, "facet_duel_pol"); }
extern "C" void grid_4_cor(gridding_parameters *p) { grid_common(p, 4, CORR_QUAD, false, "grid_4_cor"); }
extern "C" void facet_4_cor(gridding_parameters *p) { grid_common(p, 4, CORR_QUAD, true, "facet_4_cor"); }
extern "C" void facet_4_cor_corrections(gridding_parameters *p) {
  grid_common(p, 4, CORR_QUAD_JONES, true, "facet_4_cor_corrections");
}
extern "C" void grid_sampling_function(gridding_parameters *p) {
  grid_common(p, 1, CORR_SAMPLING, false, "grid_sampling_function");
}
extern "C" void facet_sampling_function(gridding_parameters *p) {
  grid_common(p, 1, CORR_SAMPLING, true, "facet_sampling_function");
}

void bz_copy_back_grids(gridding_parameters &p, bool sampling) { copy_back_grids(p, sampling); }
void bz_timer_start() { timer_start(); }
void bz_timer_stop() { timer_stop(); }

// ---------------------------------------------------------------- host post-processing
template <typename Fn>
static void parallel_for(size_t n, Fn fn) {
  unsigned nt = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
  if (n < 4096 || nt == 1) {
    fn(0, n);
    return;
  }
  std::vector<std::thread> th;
  size_t step = (n + nt - 1) / nt;
  for (unsigned t = 0; t < nt; ++t) {
    size_t lo = t * step, hi = std::min(n, lo + step);
    if (lo >= hi) break;
    th.emplace_back([=] { fn(lo, hi); });
  }
  for (auto &x : th) x.join();
}

// wrapper.cu:275-291 (identical to the CPU library, wrapper.cpp:116-135): per cell,
// divide by 1e-7 + sum of the sampling-function real parts whose channel maps to the cube slice
// (channel_grid_indicies compared with the sampling-function channel index, as the reference).
extern "C" void weight_uniformly(gridding_parameters *pp) {
  gridding_parameters &p = *pp;
  if (!check_ready("weight_uniformly")) return;
  gridding_barrier();
  if (!p.sampling_function_buffer || !p.output_buffer) {
    bz_record_error(BZ_ERR_INVALID_ARGUMENT, "weight_uniformly: sampling function and output buffers are required");
    return;
  }
  const size_t F = std::max<size_t>(1, p.num_facet_centres), G = p.cube_channel_dim_size, nx = p.nx, ny = p.ny,
               S = p.sampling_function_channel_count, C = p.number_of_polarization_terms_being_gridded;
  const vis_real eps = (vis_real)0.0000001f;
  parallel_for(F * G * ny, [&](size_t lo, size_t hi) {
    for (size_t idx = lo; idx < hi; ++idx) {
      size_t y = idx % ny, fg = idx / ny, g = fg % G, f = fg / G;
      for (size_t x = 0; x < nx; ++x) {
        vis_real count = eps;
        for (size_t s = 0; s < S; ++s)
          count += (int)(p.channel_grid_indicies[s] == g) *
                   p.sampling_function_buffer[((f * S + s) * ny + y) * nx + x].re;
        count = 1 / count;
        for (size_t corr = 0; corr < C; ++corr) {
          vis_complex &v = p.output_buffer[(((f * G + g) * C + corr) * ny + y) * nx + x];
          v.re *= count;
          v.im *= count;
        }
      }
    }
  });
}

// wrapper.cu:315-339: sum the normalisation bins, divide each (facet, cube, corr) slice.
// complex<float> /= double divides by the value rounded to float (as the reference).
extern "C" void normalize(gridding_parameters *pp) {
  gridding_parameters &p = *pp;
  if (!check_ready("normalize")) return;
  gridding_barrier();
  if (!p.output_buffer || !p.normalization_terms) return;
  const size_t F = std::max<size_t>(1, p.num_facet_centres), G = p.cube_channel_dim_size, C = p.number_of_polarization_terms_being_gridded,
               nxy = p.nx * p.ny, bins = (2 * p.conv_support + 1) * (2 * p.conv_support + 1);
  std::vector<vis_real> div(F * G * C);
  for (size_t s = 0; s < F * G * C; ++s) {
    double v = 0;
    for (size_t b = 0; b < bins; ++b) v += p.normalization_terms[s * bins + b];
    div[s] = (vis_real)v;
  }
  parallel_for(F * G * C * p.ny, [&](size_t lo, size_t hi) {
    for (size_t idx = lo; idx < hi; ++idx) {
      size_t s = idx / p.ny, y = idx % p.ny;
      vis_real d = div[s];
      vis_complex *row = p.output_buffer + s * nxy + y * p.nx;
      for (size_t x = 0; x < p.nx; ++x) {
        row[x].re /= d;
        row[x].im /= d;
      }
    }
  });
}

// ---------------------------------------------------------------- finalize (cuFFT)
// Combination applied by bullseye_finalize_stokes before the transform: slice c of facet f becomes
// (G[f][c][a] + sign G[f][c][b]) / 2.
struct StokesPair {
  int a, b, sign;
};

// The inverse transform of finalize, planned once per batch size while the library is initialised
// (finalize and finalize_psf may transform different slice counts).
static cufftHandle g_fft_plans[2] = {0, 0};
static int g_fft_batches[2] = {-1, -1};

static cufftHandle fft_plan(int batch) {
  Context &c = g_ctx;
  for (int i = 0; i < 2; ++i)
    if (g_fft_plans[i] && g_fft_batches[i] == batch) return g_fft_plans[i];
  const int slot = g_fft_plans[0] ? (g_fft_plans[1] ? 0 : 1) : 0;
  if (g_fft_plans[slot]) cufftDestroy(g_fft_plans[slot]);
  g_fft_plans[slot] = 0;
  g_fft_batches[slot] = -1;
  cufftHandle plan;
  int dims[2] = {(int)c.ny, (int)c.nx};
  const int nxy = (int)(c.nx * c.ny);
#if defined(BULLSEYE_SINGLE)
  const cufftType type = CUFFT_C2C;
#else
  const cufftType type = CUFFT_Z2Z;
#endif
  if (cufftPlanMany(&plan, 2, dims, nullptr, 1, nxy, nullptr, 1, nxy, type, batch) != CUFFT_SUCCESS) return 0;
  g_fft_plans[slot] = plan;
  g_fft_batches[slot] = batch;
  return plan;
}

void bz_release_fft_plans() {
  for (int i = 0; i < 2; ++i) {
    if (g_fft_plans[i]) cufftDestroy(g_fft_plans[i]);
    g_fft_plans[i] = 0;
    g_fft_batches[i] = -1;
  }
}

static void finalize_buffer(vis_complex *host, size_t per_facet_slices, size_t nslices, const char *name,
                            const StokesPair *stokes = nullptr) {
  Context &c = g_ctx;
  const size_t nxy = c.nx * c.ny, F = c.F;
  if (!host || nslices == 0) return;
  const size_t total = F * nslices * nxy;
  DevBuf<vis_complex> work, shifted;
  DevBuf<float> packed;
  // with a Stokes combination the whole facet blocks are uploaded into `work` first
  if (!work.alloc(stokes ? F * per_facet_slices * nxy : total) || !shifted.alloc(total) || !packed.alloc(total)) return;
  cudaStream_t s = c.stream;
  cudaEventRecord(c.ev_i0, s);
  if (stokes) {
    if (!bz_copy_async(work.ptr, host, sizeof(vis_complex) * F * per_facet_slices * nxy, cudaMemcpyHostToDevice, s))
      return;
    stokes_combine_kernel<<<2048, 256, 0, s>>>(work.ptr, shifted.ptr, (long long)nxy, (int)F, (int)nslices,
                                               (int)(per_facet_slices / nslices), stokes->a, stokes->b, stokes->sign);
    c.launches++;
  } else {
    // upload the first nslices slices of every facet block
    for (size_t f = 0; f < F; ++f)
      if (!bz_copy_async(shifted.ptr + f * nslices * nxy, host + f * per_facet_slices * nxy,
                         sizeof(vis_complex) * nslices * nxy, cudaMemcpyHostToDevice, s))
        return;
  }
  ifftshift_gather_kernel<<<2048, 256, 0, s>>>(shifted.ptr, work.ptr, (int)c.nx, (int)c.ny, (long long)(F * nslices));
  c.launches += 2;  // the gather and the packing kernel (cuFFT's own launches are not counted)
  cufftHandle plan = fft_plan((int)(F * nslices));
  if (!plan) {
    bz_record_error(BZ_ERR_CUFFT, "%s: cufftPlanMany failed", name);
    return;
  }
  cufftSetStream(plan, s);
#if defined(BULLSEYE_SINGLE)
  cufftResult r = cufftExecC2C(plan, (cufftComplex *)work.ptr, (cufftComplex *)work.ptr, CUFFT_INVERSE);
#else
  cufftResult r = cufftExecZ2Z(plan, (cufftDoubleComplex *)work.ptr, (cufftDoubleComplex *)work.ptr, CUFFT_INVERSE);
#endif
  if (r != CUFFT_SUCCESS) {
    bz_record_error(BZ_ERR_CUFFT, "%s: cufftExec failed", name);
    return;
  }
  const double *cx = c.have_corr ? c.corr_x.ptr : nullptr, *cy = c.have_corr ? c.corr_y.ptr : nullptr;
  fftshift_pack_kernel<<<2048, 256, 0, s>>>(work.ptr, shifted.ptr, packed.ptr, (int)c.nx, (int)c.ny,
                                            (long long)(F * nslices), cx, cy);
  // transformed complex slices back into their facet blocks, then the packed float32 images at
  // float index (per_facet_slices * nxy) * f, in that order (fft_and_repacking_routines.cpp:85-117)
  for (size_t f = 0; f < F; ++f)
    if (!bz_copy_async(host + f * per_facet_slices * nxy, shifted.ptr + f * nslices * nxy,
                       sizeof(vis_complex) * nslices * nxy, cudaMemcpyDeviceToHost, s))
      return;
  float *hf = reinterpret_cast<float *>(host);
  for (size_t f = 0; f < F; ++f)
    if (!bz_copy_async(hf + f * per_facet_slices * nxy, packed.ptr + f * nslices * nxy, sizeof(float) * nslices * nxy,
                       cudaMemcpyDeviceToHost, s))
      return;
  cudaEventRecord(c.ev_i1, s);
  BZ_CUDA_TRY(cudaStreamSynchronize(s));
  float ms = 0;
  if (cudaEventElapsedTime(&ms, c.ev_i0, c.ev_i1) == cudaSuccess) c.inv_seconds += ms * 1e-3;
  work.release();
  shifted.release();
  packed.release();
}

extern "C" void finalize(gridding_parameters *pp) {
  if (!check_ready("finalize")) return;
  gridding_barrier();
  finalize_buffer(pp->output_buffer, pp->cube_channel_dim_size * pp->number_of_polarization_terms_being_gridded,
                  pp->cube_channel_dim_size, "finalize");
}

// See include/bullseye_gb300.h.
extern "C" void bullseye_finalize_stokes(gridding_parameters *pp, int corr_a, int corr_b, int sign) {
  if (!check_ready("bullseye_finalize_stokes")) return;
  const int C = (int)pp->number_of_polarization_terms_being_gridded;
  if (corr_a < 0 || corr_a >= C || corr_b < 0 || corr_b >= C || (sign != 1 && sign != -1)) {
    bz_record_error(BZ_ERR_INVALID_ARGUMENT, "bullseye_finalize_stokes: correlations %d, %d of %d and sign %d", corr_a,
                    corr_b, C, sign);
    return;
  }
  gridding_barrier();
  const StokesPair sp{corr_a, corr_b, sign};
  finalize_buffer(pp->output_buffer, pp->cube_channel_dim_size * (size_t)C, pp->cube_channel_dim_size,
                  "bullseye_finalize_stokes", &sp);
}

extern "C" void finalize_psf(gridding_parameters *pp) {
  if (!check_ready("finalize_psf")) return;
  gridding_barrier();
  if (!g_ctx.want_sf) return;
  finalize_buffer(pp->sampling_function_buffer, pp->sampling_function_channel_count,
                  pp->sampling_function_channel_count, "finalize_psf");
}

// Gridding correction (detaper) for finalize: image[y][x] /= corr_x[x] * corr_y[y].  Passing
// null pointers switches it off (the default, which reproduces the reference's finalize).
extern "C" void bullseye_set_gridding_correction(const double *corr_x, size_t nx, const double *corr_y, size_t ny) {
  Context &c = g_ctx;
  if (!check_ready("bullseye_set_gridding_correction")) return;
  if (!corr_x || !corr_y) {
    c.have_corr = false;
    return;
  }
  if (nx != c.nx || ny != c.ny) {
    bz_record_error(BZ_ERR_INVALID_ARGUMENT, "gridding correction sizes must equal nx, ny");
    return;
  }
  if (!c.corr_x.alloc(nx) || !c.corr_y.alloc(ny)) return;
  BZ_CUDA_TRY(cudaMemcpy(c.corr_x.ptr, corr_x, sizeof(double) * nx, cudaMemcpyHostToDevice));
  BZ_CUDA_TRY(cudaMemcpy(c.corr_y.ptr, corr_y, sizeof(double) * ny, cudaMemcpyHostToDevice));
  c.have_corr = true;
}

