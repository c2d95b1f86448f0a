// Allocation-free gridding entry point.
//
// Some callers cannot allocate device memory at the time they grid: a host application that
// hands the library a fixed device-memory arena and forbids further cudaMalloc/cudaFree (to keep
// its memory footprint and fragmentation under its own control, or because allocation would
// synchronise the device in the middle of its pipeline), or code running where a device
// allocation is not permitted at all.  For them, bullseye_facet_4_cor_corrections_noalloc grids
// exactly like facet_4_cor_corrections but touches only memory the caller passes in plus one
// fixed, file-scope device scratch array of this library (g_noalloc_scratch below); it calls no
// cudaMalloc, cudaFree or allocating library routine.
//
// The scratch array holds the compensation (lo) half of the single-precision grid accumulation,
// the per-facet transform table and an error word.  It is BZ_NOALLOC_SCRATCH_BYTES bytes (40 MiB
// for the compensation grid, so at most 40 MiB / 8 bytes = 5,242,880 complex cells over
// facets x cube x 4 correlations x ny x nx, plus 64 KiB for the table), and every GPU that loads
// the library keeps it until the process exits.  All calls share it and it keeps the last call's
// contents: each call clears the parts that must start at zero, and calls whose work overlaps on
// the GPU (different streams, or different host threads, on one device) race on it.
//
// So that no buffer is needed for inverted Jones terms, the entry point inverts the caller's
// jones_terms in place before gridding, as the reference CPU library does
// (bullseye/mo/cpu_algorithm/wrapper.cpp:356-360).
#include <cstdint>
#include <cstring>

#include <algorithm>
#include <atomic>
#include <mutex>

#include "common.h"
#include "gridder.cuh"

// Support-aware form of the batched gridder (batched.cu), used by the workspace entry.
size_t bz_support_aware_ws_bytes(long long rows, int nchan, int nslots, int P, int os, int W, bool wproj);
bool bz_support_aware_check(const bz::GridArgs &a, size_t bytes);
bool bz_grid_support_aware(const bz::GridArgs &a, int nfacets, unsigned char *ws, size_t bytes, cudaStream_t st);

using namespace bz;

#define BZ_NOALLOC_LO_BYTES (40u << 20)
#define BZ_NOALLOC_TABLE_BYTES (64u << 10)
#define BZ_NOALLOC_SCRATCH_BYTES (BZ_NOALLOC_LO_BYTES + BZ_NOALLOC_TABLE_BYTES)
#define BZ_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) unsigned char g_noalloc_scratch[BZ_NOALLOC_SCRATCH_BYTES];

// Device address of g_noalloc_scratch per device, resolved once with that device current.  In
// host code the symbol is only a host-side stand-in, never a device address.  Host threads may
// call concurrently: the addresses are atomics and the first resolution per device is serialised.
static std::atomic<void *> g_noalloc_addr[BZ_NOALLOC_MAX_DEVICES];
static std::mutex g_noalloc_resolve_mutex;

namespace {

// Per-facet transform constants (FP64) from device-resident facet centres (arcsec):
// phase_transform_policies.h:110-134 and baseline_transform_policies.h:117-149.
__global__ void noalloc_facet_table_kernel(FacetXform *out, const vis_real *centres, int nf, double ra0, double dec0,
                                           int nx, int ny, double u_scale, double v_scale, double gcx, double gcy,
                                           long long facet_elems) {
  int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const double k = (double)kArcsecToRad;
  const double ra = centres ? (double)centres[2 * f] : ra0, dec = centres ? (double)centres[2 * f + 1] : dec0;
  double d_ra = (ra - ra0) * k, n_dec = dec * k, o_dec = dec0 * k;
  double c_d_ra = cos(d_ra), s_d_ra = sin(d_ra), c_n = cos(n_dec), s_n = sin(n_dec), c_o = cos(o_dec), s_o = sin(o_dec);
  FacetXform x;
  double li0 = c_n * s_d_ra, mi0 = s_n * c_o - c_n * s_o * c_d_ra, ni0 = s_n * s_o + c_n * c_o * c_d_ra;
  x.u_term = li0 / ni0;
  x.v_term = mi0 / ni0;
  x.dl = -c_n * s_d_ra;
  x.dm = -(s_n * c_o - c_n * s_o * c_d_ra);
  x.dn = 1.0 - sqrt(1.0 - x.dl * x.dl - x.dm * x.dm);
  x.nx = nx;
  x.ny = ny;
  x.u_scale = u_scale;
  x.v_scale = v_scale;
  x.gcx = gcx;
  x.gcy = gcy;
  x.grid_base = (long long)f * facet_elems;
  out[f] = x;
}

// In-place 2x2 inverse of every Jones matrix (jones_2x2.h:86-126); a singular matrix becomes zero
// and sets bit DEV_ERR_SINGULAR of the scratch error word.
__global__ void noalloc_invert_kernel(vis_complex *m, long long n, int *err) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  typedef vis_real T;
  vis_complex a = m[4 * i], b = m[4 * i + 1], c = m[4 * i + 2], d = m[4 * i + 3];
  T dr = (a.re * d.re - a.im * d.im) - (b.re * c.re - b.im * c.im);
  T di = (a.re * d.im + a.im * d.re) - (b.re * c.im + b.im * c.re);
  vis_complex z = {0, 0};
  if (dr == (T)0 && di == (T)0) {
    atomicOr(err, DEV_ERR_SINGULAR);
    m[4 * i] = z; m[4 * i + 1] = z; m[4 * i + 2] = z; m[4 * i + 3] = z;
    return;
  }
  T n2 = dr * dr + di * di, ir = dr / n2, ii = -di / n2;
  auto mul = [](vis_complex x, T yr, T yi) {
    vis_complex o;
    o.re = x.re * yr - x.im * yi;
    o.im = x.re * yi + x.im * yr;
    return o;
  };
  m[4 * i] = mul(d, ir, ii);
  m[4 * i + 1] = mul(b, -ir, -ii);
  m[4 * i + 2] = mul(c, -ir, -ii);
  m[4 * i + 3] = mul(a, ir, ii);
}

__global__ void noalloc_fold_kernel(vis_complex *__restrict__ grid, const vis_complex *__restrict__ lo, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    vis_complex l = lo[i];
    grid[i].re += l.re;
    grid[i].im += l.im;
  }
}

// Ownership layout for full support W (same rule as the library's other gridding calls).
struct Shape {
  int J, NT, V;
  bool wide;
  size_t smem;
};
template <bool WPROJ>
Shape noalloc_shape(int W) {
  Shape s;
  s.J = 0;
  s.wide = false;
  const int cols = ((W + 31) / 32) * 32;
  if ((cols - W) * 8 <= W) {
    for (int j : {2, 8})
      if (cols * ((W + j - 1) / j) <= 512) { s.J = j; s.wide = true; break; }
  }
  if (!s.J)
    for (int j : {1, 2, 4, 8, 16})
      if (W * ((W + j - 1) / j) <= 512) { s.J = j; break; }
  if (!s.J) s.J = 16;
  const int owners = s.wide ? cols * ((W + s.J - 1) / s.J) : W * ((W + s.J - 1) / s.J);
  s.NT = std::max(32, ((owners + 31) / 32) * 32);
  s.V = grid_chunk_size<4, WPROJ>(W, s.NT, s.J);
  s.smem = grid_smem_bytes<4, WPROJ>(s.V, W, s.NT, s.J);
  return s;
}

template <bool WPROJ, int J, bool WIDE>
bool noalloc_launch(const GridArgs &a, const Shape &s, long long blocks, cudaStream_t st) {
#if defined(BULLSEYE_SINGLE)
  void (*kern)(const GridArgs) = romein_grid_kernel<4, WPROJ, J, true, WIDE>;
#else
  void (*kern)(const GridArgs) = romein_grid_kernel<4, WPROJ, J, false, WIDE>;
#endif
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s.smem) != cudaSuccess) return false;
  kern<<<(unsigned)blocks, s.NT, s.smem, st>>>(a);
  return cudaGetLastError() == cudaSuccess;
}

template <bool WPROJ>
bool noalloc_dispatch(GridArgs a, long long blocks, cudaStream_t st) {
  Shape s = noalloc_shape<WPROJ>(a.W);
  if (s.NT > 512) return false;
  a.V = s.V;
  if (s.wide) return s.J == 2 ? noalloc_launch<WPROJ, 2, true>(a, s, blocks, st) : noalloc_launch<WPROJ, 8, true>(a, s, blocks, st);
  switch (s.J) {
    case 1: return noalloc_launch<WPROJ, 1, false>(a, s, blocks, st);
    case 2: return noalloc_launch<WPROJ, 2, false>(a, s, blocks, st);
    case 4: return noalloc_launch<WPROJ, 4, false>(a, s, blocks, st);
    case 8: return noalloc_launch<WPROJ, 8, false>(a, s, blocks, st);
    default: return noalloc_launch<WPROJ, 16, false>(a, s, blocks, st);
  }
}

}  // namespace

namespace {

// Device scratch of one gridding call: the compensation grid (single precision), the facet table
// and an error word, with the capacities the call checks its sizes against.
struct Workspace {
  vis_complex *lo;
  size_t lo_bytes;
  FacetXform *table;
  size_t table_bytes;
  int *err;
  unsigned char *sched = nullptr;  // support-aware schedule and tables (workspace entry), or null
  size_t sched_bytes = 0;
};

// Every rejection happens before the first launch, so a rejected call leaves the caller's arrays
// (jones_terms included) untouched.  Only a launch failure reported by the runtime after the Jones
// inversion was queued (the device is then unusable anyway) returns with the terms inverted.
int grid_4cor_jones(const gridding_parameters &p, const Workspace &ws, void *stream, const char *name) {
  const size_t F = p.num_facet_centres ? p.num_facet_centres : 1;
  const size_t nxy = p.nx * p.ny;
  const size_t grid_elems = F * p.cube_channel_dim_size * 4 * nxy;
  const int W = (int)(2 * p.conv_support + 1);
  const bool wproj = p.wplanes > 1;
  if (p.number_of_polarization_terms_being_gridded != 4 || p.number_of_polarization_terms != 4) {
    bz_record_error(BZ_ERR_INVALID_ARGUMENT, "%s: four polarisation terms are gridded", name);
    return BZ_ERR_INVALID_ARGUMENT;
  }
  if (!p.visibilities || !p.uvw_coords || !p.visibility_weights || !p.flags || !p.flagged_rows || !p.field_array ||
      !p.spw_index_array || !p.antenna_1_ids || !p.antenna_2_ids || !p.timestamp_ids || !p.jones_terms || !p.conv ||
      !p.reference_wavelengths || !p.enabled_channels || !p.channel_grid_indicies || !p.output_buffer ||
      !p.normalization_terms) {
    bz_record_error(BZ_ERR_INVALID_ARGUMENT, "%s: a required device array is null", name);
    return BZ_ERR_INVALID_ARGUMENT;
  }
  if (p.nx == 0 || p.ny == 0 || p.channel_count == 0 || p.spw_count == 0 || p.conv_oversample == 0 ||
      p.cube_channel_dim_size == 0) {
    bz_record_error(BZ_ERR_INVALID_ARGUMENT, "%s: nx, ny, channels, spws, oversampling and cube must be > 0", name);
    return BZ_ERR_INVALID_ARGUMENT;
  }
#if defined(BULLSEYE_SINGLE)
  if (grid_elems * sizeof(vis_complex) > ws.lo_bytes) {
    bz_record_error(BZ_ERR_UNSUPPORTED,
                    "%s: %zu grid cells need %zu bytes of compensation scratch, more than the %zu bytes available "
                    "(the fixed scratch array of the allocation-free entry)",
                    name, grid_elems, grid_elems * sizeof(vis_complex), ws.lo_bytes);
    return BZ_ERR_UNSUPPORTED;
  }
#endif
  if (F * sizeof(FacetXform) > ws.table_bytes) {
    bz_record_error(BZ_ERR_UNSUPPORTED, "%s: %zu facets exceed the scratch facet table", name, F);
    return BZ_ERR_UNSUPPORTED;
  }

  GridArgs a;
  std::memset(&a, 0, sizeof a);
  a.vis = p.visibilities; a.weights = p.visibility_weights; a.flags = (const uint8_t *)p.flags;
  a.uvw = (const vis_real *)p.uvw_coords; a.flagged_rows = (const uint8_t *)p.flagged_rows;
  a.field = p.field_array; a.spw = p.spw_index_array; a.ant1 = p.antenna_1_ids; a.ant2 = p.antenna_2_ids;
  a.time_ids = p.timestamp_ids;
  a.jones_inv = p.jones_terms;  // inverted in place before gridding
  a.starts = p.baseline_starting_indexes;
  a.wavelengths = p.reference_wavelengths; a.enabled = (const uint8_t *)p.enabled_channels; a.cgi = p.channel_grid_indicies;
  a.conv = p.conv;
  a.facets = ws.table;
  a.grid = p.output_buffer;
#if defined(BULLSEYE_SINGLE)
  a.grid_lo = ws.lo;
#endif
  a.norm = p.normalization_terms;
  a.error = ws.err;
  a.nrows = (long long)p.row_count;
  a.nchan = (int)p.channel_count; a.npol = 4; a.pol0 = 0; a.pol1 = 0;
  a.nspw = (int)p.spw_count; a.nant = (int)p.antenna_count; a.ntimes = (int)p.no_timestamps_read;
  a.facet_base = 0; a.nfacets_total = (int)F; a.groups = (int)p.cube_channel_dim_size;
  a.nx = (int)p.nx; a.ny = (int)p.ny; a.W = W; a.os = (int)p.conv_oversample;
  a.K = (W + 2) + (W + 1) * ((int)p.conv_oversample - 1);
  a.P = (int)(p.wplanes > 1 ? p.wplanes : 1);
  a.mode = CORR_QUAD_JONES; a.phase = 1; a.uvx = 1;
  if (p.baseline_starting_indexes) {
    a.nslots = (int)p.baseline_count;
    a.seg = 0;
  } else {
    a.seg = 256;
    a.nslots = (int)((p.row_count + 255) / 256);
  }
  a.imaging_field = p.imaging_field;
  a.u_scale = (double)p.nx * (double)p.cell_size_x * (double)kArcsecToRad;
  a.v_scale = -((double)p.ny * (double)p.cell_size_y * (double)kArcsecToRad);
  a.gcx = (double)(p.nx / 2 - p.conv_support);
  a.gcy = (double)(p.ny / 2 - p.conv_support);
  a.wmax = (double)(float)p.wmax_est;
  const long long blocks = (long long)F * a.nslots * (long long)a.nchan;
  if (p.row_count > 0) {
    if (ws.sched) {
      // workspace entry: persistent per-class launches (no limit on work items); the workspace size
      // and a thread layout for every class width are checked here
      if (!bz_support_aware_check(a, ws.sched_bytes)) return bz_error_code() ? bz_error_code() : BZ_ERR_UNSUPPORTED;
    } else {
      // plain entry: one CTA per (facet, track, channel)
      if (blocks > 0x7fffffffLL) {
        bz_record_error(BZ_ERR_UNSUPPORTED, "%s: %lld (facet, track, channel) work items exceed one launch", name, blocks);
        return BZ_ERR_UNSUPPORTED;
      }
      if ((wproj ? noalloc_shape<true>(W) : noalloc_shape<false>(W)).NT > 512) {
        bz_record_error(BZ_ERR_UNSUPPORTED, "%s: full support %d is not supported", name, W);
        return BZ_ERR_UNSUPPORTED;
      }
    }
  }

  // launches
  cudaStream_t st = static_cast<cudaStream_t>(stream);
#if defined(BULLSEYE_SINGLE)
  if (cudaMemsetAsync(ws.lo, 0, grid_elems * sizeof(vis_complex), st) != cudaSuccess) return BZ_ERR_CUDA;
#endif
  if (cudaMemsetAsync(ws.err, 0, sizeof(int), st) != cudaSuccess) return BZ_ERR_CUDA;
  noalloc_facet_table_kernel<<<(unsigned)((F + 127) / 128), 128, 0, st>>>(
      ws.table, p.facet_centres, (int)F, (double)p.phase_centre_ra, (double)p.phase_centre_dec, (int)p.nx, (int)p.ny,
      a.u_scale, a.v_scale, a.gcx, a.gcy, (long long)(p.cube_channel_dim_size * 4 * nxy));
  if (cudaGetLastError() != cudaSuccess) return BZ_ERR_CUDA;
  const long long nj = (long long)(p.no_timestamps_read * p.antenna_count * F * p.spw_count * p.channel_count);
  if (nj > 0) noalloc_invert_kernel<<<(unsigned)((nj + 255) / 256), 256, 0, st>>>(p.jones_terms, nj, ws.err);
  if (cudaGetLastError() != cudaSuccess) return BZ_ERR_CUDA;
  if (p.row_count == 0) return BZ_OK;
  if (ws.sched) {
    // workspace entry: support-aware (each w plane's nonzero window only; the same grids)
    if (!bz_grid_support_aware(a, (int)F, ws.sched, ws.sched_bytes, st)) return bz_error_code() ? bz_error_code() : BZ_ERR_CUDA;
  } else if (!(wproj ? noalloc_dispatch<true>(a, blocks, st) : noalloc_dispatch<false>(a, blocks, st))) {
    bz_record_error(BZ_ERR_CUDA, "%s: gridder launch failed", name);
    return BZ_ERR_CUDA;
  }
#if defined(BULLSEYE_SINGLE)
  noalloc_fold_kernel<<<1024, 256, 0, st>>>(p.output_buffer, ws.lo, (long long)grid_elems);
  if (cudaGetLastError() != cudaSuccess) return BZ_ERR_CUDA;
#endif
  return BZ_OK;
}

// Maps the error bits of a call's error word to the library's sticky error (as the regular entry
// points do when they synchronise); returns the first status, 0 when the word is clear.
int report_device_error(int h, const char *name) {
  if (!h) return BZ_OK;
  if (h & DEV_ERR_SINGULAR) bz_record_error(BZ_ERR_SINGULAR_JONES, "%s: Jones matrix set contains singular matrices", name);
  if (h & DEV_ERR_GRID_INDEX)
    bz_record_error(BZ_ERR_INVALID_ARGUMENT, "%s: channel grid index, spw or schedule entry out of range", name);
  if (h & DEV_ERR_JONES_INDEX)
    bz_record_error(BZ_ERR_INVALID_ARGUMENT, "%s: timestamp or antenna id out of range of the Jones terms", name);
  if (h & DEV_ERR_WAIT_TIMEOUT) bz_record_error(BZ_ERR_CUDA, "%s: a bounded wait for staged kernel taps ran out", name);
  if (h & DEV_ERR_SINGULAR) return BZ_ERR_SINGULAR_JONES;
  if (h & (DEV_ERR_GRID_INDEX | DEV_ERR_JONES_INDEX)) return BZ_ERR_INVALID_ARGUMENT;
  return BZ_ERR_CUDA;
}

// Device address of the scratch array on the current device (resolved on the first call there).
// Resolution loads the module's symbol table, which a stream capture does not allow: a first call
// made while `st` is capturing is rejected.
unsigned char *noalloc_scratch(cudaStream_t st, bool resolve, const char *name) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= BZ_NOALLOC_MAX_DEVICES) {
    bz_record_error(BZ_ERR_CUDA, "%s: no current CUDA device below %d", name, BZ_NOALLOC_MAX_DEVICES);
    return nullptr;
  }
  void *ptr = g_noalloc_addr[dev].load(std::memory_order_acquire);
  if (ptr || !resolve) return static_cast<unsigned char *>(ptr);
  std::lock_guard<std::mutex> lk(g_noalloc_resolve_mutex);
  ptr = g_noalloc_addr[dev].load(std::memory_order_acquire);
  if (ptr) return static_cast<unsigned char *>(ptr);
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
    cudaGetLastError();
    bz_record_error(BZ_ERR_UNSUPPORTED, "%s: the first call on a device must come before any stream capture", name);
    return nullptr;
  }
  const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
  if (e != cudaSuccess || !ptr) {
    bz_record_error(BZ_ERR_CUDA, "%s: cudaGetSymbolAddress of the scratch array failed (%s)", name, cudaGetErrorString(e));
    return nullptr;
  }
  g_noalloc_addr[dev].store(ptr, std::memory_order_release);
  return static_cast<unsigned char *>(ptr);
}

Workspace noalloc_workspace(unsigned char *scratch) {
  Workspace ws;
  ws.lo = reinterpret_cast<vis_complex *>(scratch);
  ws.lo_bytes = BZ_NOALLOC_LO_BYTES;
  ws.table = reinterpret_cast<FacetXform *>(scratch + BZ_NOALLOC_LO_BYTES);
  ws.table_bytes = BZ_NOALLOC_TABLE_BYTES - 256;
  ws.err = reinterpret_cast<int *>(scratch + BZ_NOALLOC_LO_BYTES + BZ_NOALLOC_TABLE_BYTES - 256);
  return ws;
}

}  // namespace

// See include/bullseye_gb300.h.  Every pointer in *params is a device pointer; returns 0 when
// the work was queued on `stream`, or a bz_status code (nothing queued) when the arguments are
// rejected.  The first call on each device resolves the scratch array's device address
// (cudaGetSymbolAddress) and must therefore come before any stream capture on that device.
extern "C" int bullseye_facet_4_cor_corrections_noalloc(const gridding_parameters *params, void *stream) {
  const char *name = "bullseye_facet_4_cor_corrections_noalloc";
  if (!params) return BZ_ERR_INVALID_ARGUMENT;
  unsigned char *scratch = noalloc_scratch(static_cast<cudaStream_t>(stream), true, name);
  if (!scratch) return bz_error_code() ? bz_error_code() : BZ_ERR_CUDA;
  return grid_4cor_jones(*params, noalloc_workspace(scratch), stream, name);
}

// Bytes of caller workspace bullseye_facet_4_cor_corrections_ws needs for these parameters.
static size_t ws_lo_bytes(const gridding_parameters &p) {
#if defined(BULLSEYE_SINGLE)
  const size_t F = p.num_facet_centres ? p.num_facet_centres : 1;
  return (F * p.cube_channel_dim_size * 4 * p.nx * p.ny * sizeof(vis_complex) + 255) / 256 * 256;
#else
  (void)p;
  return 0;
#endif
}
static size_t ws_table_bytes(const gridding_parameters &p) {
  const size_t F = p.num_facet_centres ? p.num_facet_centres : 1;
  return (F * sizeof(FacetXform) + 255) / 256 * 256;
}

static size_t ws_sched_bytes(const gridding_parameters &p) {
  const int nslots = p.baseline_starting_indexes ? (int)p.baseline_count : (int)((p.row_count + 255) / 256);
  return bz_support_aware_ws_bytes((long long)p.row_count, (int)p.channel_count, nslots,
                                   (int)(p.wplanes > 1 ? p.wplanes : 1), (int)p.conv_oversample,
                                   (int)(2 * p.conv_support + 1), p.wplanes > 1);
}

// See include/bullseye_gb300.h.
extern "C" size_t bullseye_facet_4_cor_corrections_ws_bytes(const gridding_parameters *params) {
  if (!params) return 0;
  return ws_lo_bytes(*params) + ws_table_bytes(*params) + 256 + ws_sched_bytes(*params);
}

// Workspace pieces of bullseye_facet_4_cor_corrections_ws: compensation grid, facet table, error
// word, support-aware schedule.
static Workspace caller_workspace(const gridding_parameters &p, unsigned char *w) {
  Workspace ws;
  ws.lo = reinterpret_cast<vis_complex *>(w);
  ws.lo_bytes = ws_lo_bytes(p);
  ws.table = reinterpret_cast<FacetXform *>(w + ws.lo_bytes);
  ws.table_bytes = ws_table_bytes(p);
  ws.err = reinterpret_cast<int *>(w + ws.lo_bytes + ws.table_bytes);
  ws.sched = w + ws.lo_bytes + ws.table_bytes + 256;
  ws.sched_bytes = ws_sched_bytes(p);
  return ws;
}

// See include/bullseye_gb300.h.
extern "C" int bullseye_facet_4_cor_corrections_ws(const gridding_parameters *params, void *workspace, size_t bytes,
                                                   void *stream) {
  const char *name = "bullseye_facet_4_cor_corrections_ws";
  if (!params || !workspace) {
    bz_record_error(BZ_ERR_INVALID_ARGUMENT, "%s: params and workspace are required", name);
    return BZ_ERR_INVALID_ARGUMENT;
  }
  const size_t need = bullseye_facet_4_cor_corrections_ws_bytes(params);
  if (bytes < need || (reinterpret_cast<uintptr_t>(workspace) & 255)) {
    bz_record_error(BZ_ERR_INVALID_ARGUMENT, "%s: workspace of %zu bytes at %p, need %zu bytes 256-byte aligned", name,
                    bytes, workspace, need);
    return BZ_ERR_INVALID_ARGUMENT;
  }
  return grid_4cor_jones(*params, caller_workspace(*params, static_cast<unsigned char *>(workspace)), stream, name);
}

// See include/bullseye_gb300.h.
extern "C" int bullseye_facet_4_cor_corrections_status(const gridding_parameters *params, const void *workspace,
                                                       void *stream) {
  const char *name = workspace ? "bullseye_facet_4_cor_corrections_ws" : "bullseye_facet_4_cor_corrections_noalloc";
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int *err = nullptr;
  if (workspace) {
    if (!params) {
      bz_record_error(BZ_ERR_INVALID_ARGUMENT, "bullseye_facet_4_cor_corrections_status: params are required");
      return BZ_ERR_INVALID_ARGUMENT;
    }
    err = caller_workspace(*params, static_cast<unsigned char *>(const_cast<void *>(workspace))).err;
  } else {
    unsigned char *scratch = noalloc_scratch(st, false, name);
    if (!scratch) return bz_error_code();  // no call on this device yet: nothing to report
    err = noalloc_workspace(scratch).err;
  }
  int h = 0;
  cudaError_t e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaMemcpy(&h, err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && h) e = cudaMemset(err, 0, sizeof(int));
  if (e != cudaSuccess) {
    bz_record_error(BZ_ERR_CUDA, "bullseye_facet_4_cor_corrections_status: %s", cudaGetErrorString(e));
    return BZ_ERR_CUDA;
  }
  return report_device_error(h, name);
}
