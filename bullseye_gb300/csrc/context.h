// Library context of the GB300 imaging library (shared by its translation units).
#pragma once
#include <cstring>
#include <functional>
#include <vector>

#include "common.h"
#include "gridder.cuh"

using bz::FacetXform;
using bz::GridArgs;

// ------------------------------------------------------------------ device buffer helper
// Library device memory (rows.cu): a stream-ordered pool that keeps freed memory mapped, so
// buffers released by releaseLibrary are reused by the next initLibrary without first-touch costs.
bool bz_dev_alloc(void **p, size_t bytes);
void bz_dev_free(void *p);

template <typename T>
struct DevBuf {
  T *ptr = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { release(); }
  bool alloc(size_t count) {
    release();
    if (count == 0) count = 1;
    if (!bz_dev_alloc((void **)&ptr, sizeof(T) * count)) {
      ptr = nullptr;
      bz_record_error(BZ_ERR_CUDA, "device allocation of %zu bytes failed", sizeof(T) * count);
      return false;
    }
    n = count;
    return true;
  }
  void release() {
    if (ptr) bz_dev_free(ptr);
    ptr = nullptr;
    n = 0;
  }
};

// One staging buffer of the chunked row upload (rows.cu): a chunk's rows in the caller's order.
struct StageBuf {
  DevBuf<vis_complex> vis;
  DevBuf<vis_real> weights, uvw;
  DevBuf<uint8_t> flags, flagged_rows;
  DevBuf<unsigned> field, spw, ant1, ant2;
  DevBuf<size_t> time_ids;
};

// How the rows of a call are streamed: chunks of consecutive rows, baseline slots per chunk.
struct RowsPlan {
  int chunks = 0;
  unsigned slots = 0;
  long long chunk_rows = 0;
};

// ------------------------------------------------------------------ library context
struct Context {
  bool initialized = false;
  int device = 0;
  cudaStream_t stream = nullptr;
  // host <-> device copies of the row chunks and the grids overlap the library stream's kernels
  cudaStream_t copy_stream = nullptr;
  cudaStream_t jones_stream = nullptr;  // the Jones terms' upload, beside the rows on the copy stream
  cudaEvent_t ev_stage_full[2] = {nullptr, nullptr}, ev_stage_free[2] = {nullptr, nullptr};
  cudaEvent_t ev_jones_up = nullptr, ev_jones_read = nullptr, ev_ready_vis = nullptr, ev_ready_sf = nullptr;
  cudaEvent_t ev_copied_vis = nullptr, ev_copied_sf = nullptr;
  bool host_repack = true;      // repack_input_data permutes the caller's arrays (the reference's behaviour)
  int grid_groups = 1;          // groups of row chunks gridded while later chunks upload (1: after all)
  bool host_copy_sm = true;     // bulk copies of mapped page-locked host memory run as SM kernels
  size_t max_stage_bytes = 0;   // row staging of one chunk, bytes (0: 8 GB)
  bool norm_pending = false;    // host normalisation terms are published by the next gridding_barrier
  double *norm_host = nullptr;  // pinned copy of the device normalisation sums [F][cube][C]
  cudaEvent_t ev_g0 = nullptr, ev_g1 = nullptr, ev_i0 = nullptr, ev_i1 = nullptr;
  bool grid_timing_pending = false, inv_timing_pending = false;
  double grid_seconds = 0.0, inv_seconds = 0.0;
  bool compensated = true;  // FP32: compensated (hi/lo) grid accumulation
  bool device_inputs = false;  // row arrays, Jones terms and baseline starts are device pointers
  bool batched_calls = true;   // 4-correlation and sampling-function exports run the batched gridder
  bool jones_time_major = true;  // batched calls: the record kernel reads a time-innermost Jones copy
  long long launches = 0;      // kernels launched by this library since initLibrary
  cudaEvent_t ev_k0 = nullptr, ev_k1 = nullptr;  // around the last gridder launch
  bool kernel_timing_pending = false;
  int kernel_timing_kind = 0;  // 0 visibilities, 1 sampling function
  double kernel_ms[2] = {0.0, 0.0};  // accumulated gridder kernel time (ms) per kind
  long long kernel_count[2] = {0, 0};

  // sizes fixed at init
  size_t F = 1, cube = 1, C = 1, nx = 0, ny = 0, sf_count = 0, W = 1, os = 1, K = 1, P = 1;
  size_t nchan = 1, nspw = 1, npol = 1, max_rows = 0, baselines = 0;
  bool want_sf = false;

  // device tables
  DevBuf<vis_real> conv, wavelengths, facet_centres;
  std::vector<vis_real> conv_host;  // host copy of the kernel table (support windows)
  // sum over the W taps of every (plane, tap offset) kernel row, FP64 complex [P][2 os + 1][2]:
  // a visibility's normalisation term is Re(S[plane][fu] * S[plane][fv])
  DevBuf<double> tap_sums;
  DevBuf<float> tap_sums_f;  // the same rounded to FP32 (the single-precision record kernel)
  size_t tap_f = 0;
  // the kernel table regrouped by tap offset, [P][tap_f][W] (real or complex like conv): the W taps
  // a visibility reads are contiguous, so staging them is a coalesced copy
  DevBuf<vis_real> conv_t;
  DevBuf<uint8_t> enabled;
  DevBuf<size_t> cgi, sf_cgi;
  // device row buffers (chunk_max_row_count rows)
  DevBuf<vis_complex> vis;
  DevBuf<vis_real> weights, uvw;
  DevBuf<uint8_t> flags, flagged_rows;
  DevBuf<unsigned> field, spw, ant1, ant2;
  DevBuf<size_t> time_ids, starts;
  // chunked upload: two staging buffers, the sort's keys/values/scratch, and the track table
  // [chunks][baseline slots] + 1 of absolute row starts (track k*slots + b = baseline slot b of chunk k)
  StageBuf stage[2];
  size_t stage_rows = 0;
  DevBuf<unsigned> sort_keys;
  DevBuf<int> sort_vals;
  DevBuf<unsigned char> sort_tmp;
  DevBuf<size_t> track_starts;
  RowsPlan rows_plan;           // of the rows now on the device
  const void *rows_key[3] = {nullptr, nullptr, nullptr};  // host uvw, ant1, vis of those rows
  size_t rows_key_count = 0;
  bool rows_with_vis = false, rows_with_time = false;
  DevBuf<vis_complex> jones_raw, jones_inv;
  DevBuf<vis_complex> jones_inv_t;  // the inverses time-innermost, for the batched record kernel (optional)
  DevBuf<FacetXform> facets, facets_sf;
  // grids
  // sf holds the caller's initial sampling grids [facets][sf][ny][nx]; every facet receives the
  // same sampling-function contribution (the phase policy of the sampling function reports the
  // phase centre as facet centre, phase_transform_policies.h:77-82, so the uv transform is the
  // identity), which is gridded once into sf_acc/sf_lo [sf][ny][nx] and added to every facet.
  DevBuf<vis_complex> grid, grid_lo, sf, sf_acc, sf_lo, scratch, sf_out;
  DevBuf<double> norm;
  DevBuf<int> dev_error;
  std::vector<double> host_norm;  // published through params.normalization_terms
  // gridding correction (detaper) factors for finalize, optional
  DevBuf<double> corr_x, corr_y;
  bool have_corr = false;
};


extern Context g_ctx;

// helpers defined in imaging_lib.cu
bool bz_check_ready(const char *fn);
void bz_copy_back_grids(gridding_parameters &p, bool sampling);
// Phase-rotation and uv-transform constants of a facet centred at (ra, dec), arcsec (FP64, host).
FacetXform bz_facet_xform(double ra0, double dec0, double ra, double dec, bool phase, bool uvx);
void bz_timer_start();
void bz_timer_stop();
// The batched (support-aware, persistent per-class) gridder behind one reference export: grids
// the visibilities (mode != CORR_SAMPLING, 4 correlations) or the sampling function; false on
// error (recorded).
bool bz_grid_batched_call(gridding_parameters &p, int mode, bool faceting, const char *name);
// Phase tracing (bullseye_set_tracing): when on, bz_trace_begin() and bz_trace_mark() synchronise
// the library stream and record the host time of each phase of a call; off, they do nothing.
void bz_trace_begin();
void bz_trace_mark(const char *phase);
// Whether tracing is on; a free-form trace entry; the CUDA memory kind of a caller's pointer
// ("pinned", "pageable", "device", "managed") for the trace.
bool bz_tracing();
void bz_trace_note(const char *fmt, ...);
const char *bz_host_kind(const void *p);
// Support-aware gridding without library state (the workspace entry): bytes of workspace it needs,
// and the call itself (a: the prepared arguments over the full support; ws: 256-byte aligned).
size_t bz_support_aware_ws_bytes(long long rows, int nchan, int nslots, int P, int os, int W, bool wproj);
bool bz_grid_support_aware(const GridArgs &a, int nfacets, unsigned char *ws, size_t bytes, cudaStream_t st);
// upload = false reuses the rows a preceding prepare of the same call already uploaded.  With host
// inputs, prepare only sets the arguments up (device row buffers, Jones terms, the track table of
// `plan`); the rows themselves are streamed by bz_stream_rows (or bz_upload_rows) afterwards.
bool bz_prepare_grid_args(const gridding_parameters &p, int nc, int mode, bool faceting, GridArgs &a,
                          int &nslots, const char *name, bool upload = true);
// Chunked row upload with the device sort (rows.cu): on_chunk(k, row_begin, row_end) runs after the
// chunk's sort is queued, so its gridding launches overlap the next chunk's upload.
bool bz_stream_rows(const gridding_parameters &p, bool need_vis, bool need_time, RowsPlan &plan,
                    const std::function<bool(int, long long, long long)> &on_chunk);
// Streams every chunk of a host-input call unless the rows of the same host arrays are still on the
// device (the sampling-function call that follows a visibility call); returns the plan in use.
bool bz_upload_rows(const gridding_parameters &p, bool need_vis, bool need_time, RowsPlan &plan,
                    const std::function<bool(int, long long, long long)> &on_chunk = nullptr);
// The plan a host-input call will stream with (chunks, baseline slots), allocating the device rows.
bool bz_plan_rows(const gridding_parameters &p, RowsPlan &plan);
// Forget which host arrays the device rows came from (gridding_barrier: the caller may change them).
void bz_forget_rows();
// Device address of host bytes [p, p + n) when they lie in one page-locked allocation mapped into
// the device's address space; nullptr otherwise (pageable memory, or a range that leaves it).
const void *bz_mapped_host(const void *p, size_t n);
// A host <-> device (or device <-> device) copy on stream s: an SM kernel when the host side is
// mapped page-locked memory and SM copies are on (bullseye_set_host_copy), else cudaMemcpyAsync.
// false on error (recorded).
bool bz_copy_async(void *dst, const void *src, size_t bytes, cudaMemcpyKind kind, cudaStream_t s);
