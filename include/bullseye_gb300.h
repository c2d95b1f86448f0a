/* C-ABI of the GB300 imaging libraries libgpu_imaging32.so / libgpu_imaging64.so.
 *
 * Drop-in for the reference's GPU imaging libraries: the same 19 entry points, the same
 * argument (a gridding_parameters struct passed by reference, i.e. by pointer in C) and the same
 * call sequencing (bullseye/bin/bullseye_pipeliner.py:260-424).  Each declaration below cites the
 * reference interface it replaces.  Precision is chosen by which library is loaded (32: float
 * data, 64: double data; normalisation terms are double in both), exactly as the reference's
 * BULLSEYE_SINGLE / BULLSEYE_DOUBLE builds (bullseye/mo/cpu_gpu_common/base_types.h:41-59).
 *
 * The struct layout is bullseye/mo/cpu_gpu_common/gridding_parameters.h:44-109 (392 bytes in
 * the 32-bit library, 408 in the 64-bit one); bullseye_gb300/csrc/common.h defines it with
 * static_asserts on size and offsets.  It is opaque here.
 *
 * Errors never terminate the process: every entry point records the first error (sticky) and
 * later calls return without work until it is cleared; bullseye_last_error() reports it.
 */
#ifndef BULLSEYE_GB300_H
#define BULLSEYE_GB300_H
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gridding_parameters gridding_parameters;

/* One facet of an uneven facet layout (bullseye_grid_batched_facets): centre (ra, dec) and cell
 * sizes in arcsec, grid size, and the offset in complex elements of the facet's [cube][4][ny][nx]
 * block within the caller's grid buffer. */
typedef struct bullseye_facet {
  double ra, dec;
  double cell_x, cell_y;
  size_t nx, ny;
  size_t grid_offset;
} bullseye_facet;

/* ---- reference entry points (bullseye/mo/cpu_gpu_common/wrapper.h:41-61) ---- */

/* Seconds of device time spent in gridding calls (wrapper.cu:73-75, gpu_algorithm/timer.h). */
double get_gridding_walltime(void);
/* Seconds of device time spent in finalize / finalize_psf (wrapper.cu:76-78). */
double get_inversion_walltime(void);
/* Wait for queued gridding work and copy-backs (wrapper.cu:79-81). */
void gridding_barrier(void);
/* Allocate device state, upload tables and the caller's grids, publish the library-owned
 * normalisation terms [facets][cube][corr][W*W] through params->normalization_terms
 * (wrapper.cu:82-232).  No device reset, no device selection: the current device is used. */
void initLibrary(gridding_parameters *params);
/* Free all device state (wrapper.cu:233-274; no cudaDeviceReset). */
void releaseLibrary(void);
/* Uniform weighting of the host grids by the sampling function (wrapper.cu:275-291). */
void weight_uniformly(gridding_parameters *params);
/* Divide each host grid slice by its normalisation sum (wrapper.cu:315-339). */
void normalize(gridding_parameters *params);
/* Baseline-major stable repacking of the caller's row arrays, filling
 * baseline_starting_indexes[baseline_count + 1] (wrapper.cu:367-454).  Host-only. */
void repack_input_data(gridding_parameters *params);
/* Inverse FFT of the first cube slices of every facet with the reference's shifts, float32
 * real parts packed at float index (cube * corr * nx * ny) * facet
 * (wrapper.cu:340-352, fft_and_repacking_routines.cpp:83-118). */
void finalize(gridding_parameters *params);
/* Same for the sampling-function grids (wrapper.cu:353-362, fft_and_repacking_routines.cpp:120-161). */
void finalize_psf(gridding_parameters *params);
/* Grid one correlation (polarization_index), no faceting (wrapper.cu:456-545). */
void grid_single_pol(gridding_parameters *params);
/* One correlation, faceted: phase rotation + planar uv transform per facet (wrapper.cu:546-639). */
void facet_single_pol(gridding_parameters *params);
/* Two correlations (polarization_index, second_polarization_index) (wrapper.cu:640-735). */
void grid_duel_pol(gridding_parameters *params);
/* Two correlations, faceted (wrapper.cu:736-831). */
void facet_duel_pol(gridding_parameters *params);
/* The four-correlation and sampling-function calls below run the batched, support-aware gridder
 * (see bullseye_grid_batched) when the library is initialised for 4 correlations, unless
 * bullseye_set_batched_calls(0) selects the per-track kernels; the grids are the same. */
/* Four correlations, no faceting (wrapper.cu:832-909). */
void grid_4_cor(gridding_parameters *params);
/* Four correlations, faceted (wrapper.cu:910-987). */
void facet_4_cor(gridding_parameters *params);
/* Four correlations, faceted, with J_p^-1 V J_q^-H Jones correction (wrapper.cu:988-1150; the
 * correction follows the CPU library, correlation_gridding_policies.h:503-542). */
void facet_4_cor_corrections(gridding_parameters *params);
/* Sampling function (V = 1, unit weight, row flags only), no faceting (wrapper.cu:1151-1217). */
void grid_sampling_function(gridding_parameters *params);
/* Sampling function, faceted (wrapper.cu:1218-1284). */
void facet_sampling_function(gridding_parameters *params);

/* ---- extensions (no counterpart in the reference) ---- */

/* First recorded error: returns its code (0 = none) and copies the message into buf. */
int bullseye_last_error(char *buf, size_t n);
/* Clear the sticky error so the library accepts calls again. */
void bullseye_clear_error(void);
/* 32 or 64: the data precision of the loaded library. */
int bullseye_precision_bits(void);
/* 32-bit library: compensated (hi/lo TwoSum) grid accumulation on (1, default) or off (0). */
void bullseye_set_compensated(int on);
/* When on, the row arrays, jones_terms and baseline_starting_indexes in gridding_parameters are
 * device pointers in baseline-major order and gridding calls copy nothing from the host. */
void bullseye_set_device_inputs(int on);
/* Gridding correction for finalize: image[y][x] /= corr_x[x] * corr_y[y]; nulls switch it off. */
void bullseye_set_gridding_correction(const double *corr_x, size_t nx, const double *corr_y, size_t ny);
/* The library's CUDA stream (cudaStream_t), valid between initLibrary and releaseLibrary. */
void *bullseye_get_stream(void);
/* Kernels launched by the library since initLibrary or the last counter reset. */
long long bullseye_kernel_launches(void);
/* Accumulated gridder kernel time in ms for kind 0 (visibilities) or 1 (sampling function). */
double bullseye_gridder_kernel_ms(int kind, long long *count);
/* Reset the launch and kernel-time counters. */
void bullseye_reset_counters(void);
/* Zero the device-resident grids and normalisation sums. */
void bullseye_zero_grids(void);
/* Measured FP32 FMA throughput of the current GPU in TFLOP/s (roofline denominator). */
double bullseye_fp32_fma_tflops(int iters);

/* Device memory: every buffer of the library comes from a device memory pool of the library that
 * keeps freed memory mapped, so releaseLibrary followed by initLibrary (a pipeliner imaging several
 * runs) reuses memory the GPU has already touched.  This returns the pooled memory to the driver. */
void bullseye_trim_memory(void);
/* Host inputs are uploaded on a copy stream and sorted by baseline on the device (one chunk per
 * call unless bullseye_set_max_stage_bytes or bullseye_set_grid_groups splits it).  With this off,
 * repack_input_data fills baseline_starting_indexes without permuting the caller's arrays (the
 * reference permutes them, wrapper.cu:422-452); gridding results do not depend on the row order.
 * On by default. */
void bullseye_set_host_repack(int on);
/* Host-input visibilities of a batched gridding call are gridded in `groups` groups of row chunks,
 * each while the next group's rows upload; 1 (the default) grids every row after the last chunk
 * is sorted, in one set of class launches.  More groups hide more of the upload but split every
 * class launch, adding a launch tail per group. */
void bullseye_set_grid_groups(int groups);
/* Bulk copies between the caller's host buffers (rows, Jones terms, grids) and the device: with
 * mode 1 (the default) a buffer that lies in one page-locked allocation mapped into the device's
 * address space (cudaHostAlloc, cudaHostRegister, a pinned torch tensor) is copied by an SM kernel
 * over the coherent CPU-GPU link; other memory, and every copy with mode 0, goes through
 * cudaMemcpyAsync (the copy engines).  Results are the same either way. */
void bullseye_set_host_copy(int mode);
/* Host-input rows gridded in one group are staged on the device as one chunk per call, so each
 * baseline's rows form one track; a call whose rows exceed `bytes` of staging (0: the default,
 * 8 GB) is split into even chunks, sorted and tracked chunk by chunk. */
void bullseye_set_max_stage_bytes(size_t bytes);
/* Visibility records (on by default): before its per-class launches, a batched call writes one
 * record per (row, facet, channel) of its work (footprint corner, tap rows, grid group, and the
 * weighted, Jones-corrected, phase-rotated visibility, 64 bytes in single precision) and its
 * normalisation sums, by a kernel that takes every row in parallel; the class launches then stage
 * records and tap rows by bulk copies only.  The records take at most the record budget (0: the
 * default, 30 % of the device's memory) and the free memory; work past it is prepared in place, as
 * with records off.  Results are the same either way. */
void bullseye_set_visibility_records(int on);
void bullseye_set_record_budget(size_t bytes);
/* Jones terms of the batched record kernel (on by default): the inversion also writes the inverses
 * time-innermost ([antenna][spw][channel][facet][time][4], 16 bytes per complex term in double
 * precision, 8 in single), so that a warp's rows (consecutive times of one baseline) read one
 * contiguous run per antenna and facet.  It takes a second copy of the terms' memory, allocated
 * when there is room; off (or without room), the record kernel reads the original table.  Results
 * are the same either way. */
void bullseye_set_jones_time_major(int on);

/* Batched, support-aware gridding of every facet of the current chunk: `call` 0 grids like
 * facet_4_cor_corrections, 1 like facet_4_cor, 2 like grid_4_cor; with_sampling != 0 also grids
 * the sampling function (like facet_/grid_sampling_function).  Same results as those calls: each
 * visibility is gridded over its w plane's nonzero support window (read from the kernel table)
 * instead of the padded W x W, by persistent per-support-class launches over (track run, facet)
 * work items; the schedule is built on the device and the whole call is replayed as a CUDA graph
 * after its first use (layouts per support class are picked by timing on that first use).
 * Returns 0 or the error code (also reported by bullseye_last_error). */
int bullseye_grid_batched(gridding_parameters *params, int call, int with_sampling);
/* Batched gridding of facets of UNEVEN sizes and cell sizes, each with its own rows: the same
 * support-aware persistent schedule and graph replay as bullseye_grid_batched, over `nfacets`
 * facets described by `facets` (host array), accumulated into CALLER-OWNED device buffers:
 * grids (complex, each facet's block at its grid_offset), grid_lo (the 32-bit library's
 * compensation buffer, same size as grids and zeroed by the caller, or null for plain FP32
 * accumulation; a cell's value is then grids + grid_lo; ignored by the 64-bit library) and norms
 * (float64 [nfacets][cube][4]).  Work is queued on the library stream (bullseye_get_stream).
 * row_mask, if not null, is a device array [nfacets][row_count] of bytes (device-resident inputs
 * only, bullseye_set_device_inputs; rejected with BZ_ERR_UNSUPPORTED otherwise): 0 leaves that row out of
 * that facet (the facet then sees fewer visibilities).  `call` 1 grids like facet_4_cor, 2 like
 * grid_4_cor, 0 like facet_4_cor_corrections (then nfacets must equal the facet count given to
 * initLibrary, which lays out the Jones terms).  Tables (kernel, wavelengths, channels) and rows
 * come from params as for the other gridding calls, after initLibrary; the library's own grids
 * are not touched and nothing is copied back.  The sampling function is not gridded.  No
 * counterpart in the reference (its ABI has one grid size for every facet). */
int bullseye_grid_batched_facets(gridding_parameters *params, const bullseye_facet *facets, int nfacets,
                                 const unsigned char *row_mask, void *grids, void *grid_lo, double *norms,
                                 int call);
/* Profiling mode of bullseye_grid_batched (off by default): when on, each call runs eagerly (no
 * graph) with a CUDA event pair around every support-class launch, synchronising after each. */
void bullseye_set_batched_profiling(int on);
/* The last profiled call's class launches: support width, correlations (4 visibilities, 1
 * sampling function), layout (J rows per thread; `wide` bit 0 = WIDE, bits 1.. = the build's register
 * cap), (track run, facet) work items and
 * milliseconds, up to max entries; returns the number of launches recorded. */
int bullseye_batched_profile(int *width, int *nc, int *J, int *wide, int *items, float *ms, int max);
/* Support-class width the batched gridder uses for every w plane (the plane's nonzero window,
 * rounded up to a class width), up to max planes; returns the plane count (0 before the first
 * batched call after initLibrary). */
int bullseye_batched_plane_classes(int *width, int max);
/* The reference's 4-correlation gridding exports (grid_4_cor, facet_4_cor,
 * facet_4_cor_corrections) and sampling-function exports run the batched, support-aware gridder
 * (the same grids: each w plane's taps outside its nonzero window are exactly zero) when this is
 * on (the default, when the library is initialised for 4 correlations); off selects the plain
 * per-track kernels, which grid the full padded support.  Single and dual polarisation calls
 * always use the plain kernels. */
void bullseye_set_batched_calls(int on);
/* finalize with the Stokes (or correlation) combination and facet compaction done on the device:
 * for every facet f and cube slice c, (G[f][c][corr_a] + sign * G[f][c][corr_b]) / 2 of the host
 * grids (after weight_uniformly / normalize; corr_a and corr_b index the gridded correlation
 * slices) is placed at cube slice c of the facet block, then transformed and packed as finalize
 * does.  These are the combinations bullseye/data/stokes.py:90-172 forms on the host: linear feeds
 * I = (XX, YY, +1), Q = (XX, YY, -1), U = (XY, YX, +1), V = (XY, YX, -1); circular feeds
 * I = (RR, LL, +1), V = (RR, LL, -1), Q = (RL, LR, +1), U = (RL, LR, -1).  corr_a == corr_b with
 * sign +1 selects one correlation.  No counterpart in the reference library. */
void bullseye_finalize_stokes(gridding_parameters *params, int corr_a, int corr_b, int sign);
/* Phase tracing of the batched gridding calls: when on, each call synchronises its stream at phase
 * boundaries (upload and prepare, schedule/tune/capture, the class kernels, copy-back) and records
 * their host times; bullseye_trace_report writes "phase ms; ..." for the calls since the last
 * report into buf (up to n bytes) and returns the length of the log.  Tracing changes the overlap
 * of those phases: use it to see where a call's time goes, not to time it. */
void bullseye_set_tracing(int on);
size_t bullseye_trace_report(char *buf, size_t n);
/* Self-test of the batched gridder's bounded waits: runs one CTA whose tap-copy barrier never
 * completes and returns the device error bits it recorded (16 = the wait ran out, as expected),
 * or -1 on a CUDA error.  Takes about 0.2 s; touches no library state. */
int bullseye_selftest_bounded_wait(void);

/* Allocation-free facet_4_cor_corrections, for callers that cannot allocate device memory while
 * they grid (a fixed device arena with no further cudaMalloc/cudaFree, or code where a device
 * allocation would synchronise or is not permitted).  No counterpart in the reference.
 * Every pointer in *params is a DEVICE pointer: row arrays in baseline-major order (with
 * baseline_starting_indexes, or null for fixed row segments), jones_terms (inverted IN PLACE, as
 * the reference CPU library does), conv, reference_wavelengths, enabled_channels,
 * channel_grid_indicies, facet_centres, output_buffer (grids, accumulated into) and
 * normalization_terms (float64 [facets][cube][4], accumulated into); sizes and scalars are read
 * from the struct.  Work is queued on `stream` (a cudaStream_t); nothing is allocated and the
 * call does not synchronise.  Scratch is one fixed file-scope device array of the library
 * (40 MiB + 64 KiB, held by every GPU that loads the library until exit): in the 32-bit library,
 * grids beyond 5,242,880 complex cells (facets x cube x 4 x ny x nx) are rejected with
 * BZ_ERR_UNSUPPORTED (5)
 * and a message in bullseye_last_error().  Calls whose work overlaps on one GPU race on the shared
 * scratch.  The first call on each device resolves the scratch address and must come before any
 * stream capture on that device (a first call made while `stream` is capturing is rejected).
 * Device-side errors are read with bullseye_facet_4_cor_corrections_status.  Returns 0 when
 * queued. */
int bullseye_facet_4_cor_corrections_noalloc(const gridding_parameters *params, void *stream);

/* The same gridding on device pointers with a CALLER-PROVIDED device workspace instead of the fixed
 * scratch array, so grids of any size are accepted and concurrent calls with their own workspaces
 * do not share state.  It is support-aware: each w plane's nonzero kernel window is found on the
 * device and the visibilities are gridded by persistent per-support-class launches over a run
 * schedule built in the workspace (the same grids as the full padded support).  The workspace must
 * be 256-byte aligned and at least bullseye_facet_4_cor_corrections_ws_bytes(params) bytes (the
 * 32-bit library's compensation grid, the facet table, an error word, and the support windows,
 * window table and run schedule: about 33 bytes per (row, channel)); its contents need not be
 * initialised.  jones_terms is inverted in place.  No counterpart in the reference. */
size_t bullseye_facet_4_cor_corrections_ws_bytes(const gridding_parameters *params);
int bullseye_facet_4_cor_corrections_ws(const gridding_parameters *params, void *workspace, size_t bytes,
                                        void *stream);
/* Device-side errors of the last bullseye_facet_4_cor_corrections_noalloc call on the current device
 * (workspace null; params may be null) or of the last bullseye_facet_4_cor_corrections_ws call on
 * `workspace` (params as passed to that call): waits for `stream`, reads the call's error word
 * (singular Jones matrices, which are zeroed as in the reference's jones_2x2.h; channel grid index,
 * spw, antenna or timestamp ids out of range; a bounded wait that ran out), records the first
 * error for bullseye_last_error, clears the word and returns its status (0 = none, else
 * BZ_ERR_SINGULAR_JONES (4), BZ_ERR_INVALID_ARGUMENT (2) or BZ_ERR_CUDA (3)).  Allocates nothing.
 * Both entries reject bad arguments before queuing any work, so a rejected call leaves
 * jones_terms as it was.  No counterpart in the reference (its CPU library throws from
 * invert_all, bullseye/mo/cpu_gpu_common/jones_2x2.h:118-123). */
int bullseye_facet_4_cor_corrections_status(const gridding_parameters *params, const void *workspace, void *stream);

/* Adjoint of four-correlation gridding (a degridder): given grad_grid = dL/dG for the grids
 * G [facets][cube][4][ny][nx] that facet_4_cor_corrections (jones_terms set, faceting != 0),
 * facet_4_cor (jones_terms null, faceting != 0) or grid_4_cor (faceting == 0) produce from these
 * inputs, writes grad_vis = dL/dV [rows][channels][4] and, when jones_terms and grad_jones are
 * both set, ACCUMULATES dL/dJ into grad_jones [T][A][F][S][Ch][4] (zero it first).  Complex
 * gradients follow the real-inner-product convention dL = Re sum conj(g) dz (PyTorch's).  Cells,
 * taps, w planes, phase rotation and flags are selected exactly as the gridder selects them; the
 * normalisation sums carry no gradient.  No counterpart in the reference (its only degridder is
 * the prototype in writing_and_wiki/notebooks/Resampling.ipynb, cell 17: with unit weights, no
 * faceting and grad_grid = the model grid, grad_vis divided by the tap sum is that degridder).
 * Every pointer in *params and the three arrays are DEVICE pointers; jones_terms holds the raw
 * (not inverted) terms.  Rows may be in any order.  Work is queued on `stream`; nothing is
 * allocated.  Returns 0 when queued. */
int bullseye_grid_adjoint(const gridding_parameters *params, const void *grad_grid, void *grad_vis,
                          void *grad_jones, int faceting, void *stream);

/* Prediction (degridding as a forward operator): model visibilities from per-facet model images.
 * `model` holds complex [facets][cube][4][ny][nx] images (each facet's model sky per cube slice and
 * correlation, image pixels laid out as finalize writes them).  Each slice is divided by the
 * gridding correction taper_y[y] * taper_x[x] (the tapers finalize divides by, see
 * bullseye_set_gridding_correction; both null for none), transformed to a uv grid with the inverse
 * of finalize's shifts (grid = fftshift(FFT(ifftshift(image))), unnormalised forward transform), and
 * every (row, channel) visibility of vis_out [rows][channels][4] is OVERWRITTEN with
 *   sum over facets of  J_p (e^{-i phi_f} D_f') J_q^H,
 *   D_f = sum over the visibility's footprint of grid_f x conj(tap)      (flags & 1: divided by the
 *         real part of the footprint's tap sum, the normalised form of the reference's prototype
 *         degridder, writing_and_wiki/notebooks/Resampling.ipynb cell 17),
 * with D_f' = D_f, or conj(D_f) for w < 0; the cells, taps, w plane, phase rotation (phi_f, applied
 * with the opposite sign to the gridder's) and planar uv transform are selected exactly as the
 * gridder selects them (faceting != 0: facet_4_cor geometry; 0: grid_4_cor), and jones_terms (raw,
 * not inverted; null for none) are applied forward.  Weights and flags are not applied.  flags & 2:
 * `model` already holds the uv grids (no taper, no transform, no workspace needed).  Otherwise
 * `workspace` (256-byte aligned, at least bullseye_predict_ws_bytes(params) bytes: two grids)
 * holds the transform.  Every pointer is a DEVICE pointer; row arrays may be in any order.  Work
 * is queued on `stream`; the library's batched forward transform plans are created on first use
 * per (device, size, batch) and kept.  Returns 0 when queued.  No counterpart in the reference's
 * library (its only degridder is the notebook prototype). */
size_t bullseye_predict_ws_bytes(const gridding_parameters *params);
int bullseye_predict(const gridding_parameters *params, const void *model, const double *taper_x,
                     const double *taper_y, int faceting, int flags, void *vis_out, void *workspace,
                     size_t ws_bytes, void *stream);

/* Integer sampling-function counts with the reference's nearest-neighbour policy
 * (bullseye/mo/cpu_algorithm/convolution_policies.h:35-65 composed with the sampling-function policy,
 * correlation_gridding_policies.h:190-245): every kept (row, channel) adds 1 to the cell
 * lrint(u * u_scale + nx/2), lrint(v * v_scale + ny/2), computed in the library's data precision with
 * the reference's operation order, so the counts are bit-exact.  ACCUMULATES into counts
 * [facets][sampling_function_channel_count][ny][nx] (uint32, device; zero it first); the facets all
 * receive the same counts (the sampling function's uv transform is the identity in facet mode).
 * Row arrays, reference_wavelengths, enabled_channels and sampling_function_channel_grid_indicies
 * are DEVICE pointers.  Synchronises `stream` to report index errors.  Returns 0 or a bz status. */
int bullseye_sampling_counts_nn(const gridding_parameters *params, unsigned int *counts, int faceting, void *stream);

#ifdef __cplusplus
}
#endif
#endif
