// Device memory, host copies and row streaming of the GB300 imaging library.
//
// Memory.  Every library buffer comes from a stream-ordered device memory pool of the library (one
// per device) whose release threshold keeps freed memory mapped: releaseLibrary returns buffers
// to the pool and the next initLibrary reuses them without cudaMalloc / cudaFree (which
// synchronise the device).  bullseye_trim_memory() hands the pooled memory back.
//
// Host copies.  Bulk copies of the caller's page-locked buffers run as SM kernels over the
// coherent CPU-GPU link (bz_copy_async): copy-engine transfers of host buffers that have sat idle
// between calls were measured at 13-30 GB/s, SM copies of the same buffers at 110-211 GB/s.
//
// Rows.  A gridding call with host inputs uploads its rows (in the caller's order) into a staging
// buffer on a copy stream; on the library stream they are sorted by baseline slot (a stable radix
// sort, so rows of a baseline stay in the caller's time order) and gathered into the device row
// buffers, baseline-major, as repack_input_data orders them on the host
// (bullseye/mo/gpu_algorithm/wrapper.cu:367-454).  A call is one chunk unless its rows exceed the
// staging limit or are gridded in several groups (bullseye_set_grid_groups); then chunks of
// consecutive rows use two staging buffers in turn, the upload of chunk k + 1 overlapping the
// sort (and, with groups, the gridding) of chunk k.  Each chunk's track starts (rows of each
// baseline slot) go into a table of chunks x slots + 1 entries, so that the tracks of every chunk
// together describe all rows.  Rows sorted on the device need no host permutation, so
// repack_input_data can leave the caller's arrays in place (bullseye_set_host_repack(0)); results
// do not depend on the row order.
#include <cub/device/device_radix_sort.cuh>
#include <cuda.h>

#include <algorithm>
#include <cmath>
#include <atomic>
#include <cstdint>
#include <mutex>

#include "context.h"

using namespace bz;

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_pool_mutex;
cudaMemPool_t g_pools[kMaxDevices];

cudaMemPool_t device_pool() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return nullptr;
  std::lock_guard<std::mutex> lk(g_pool_mutex);
  if (!g_pools[dev]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool = nullptr;
    if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) return nullptr;
    uint64_t keep = UINT64_MAX;  // freed memory stays mapped in the pool
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    g_pools[dev] = pool;
  }
  return g_pools[dev];
}

}  // namespace

// Allocations are ordered on the library stream and completed before they are handed out, so the
// memory may be used on any stream; frees are ordered after the stream's queued work.
bool bz_dev_alloc(void **p, size_t bytes) {
  cudaMemPool_t pool = device_pool();
  cudaStream_t s = g_ctx.stream;
  if (!pool) return cudaMalloc(p, bytes) == cudaSuccess;
  if (cudaMallocFromPoolAsync(p, bytes, pool, s) != cudaSuccess) return false;
  return cudaStreamSynchronize(s) == cudaSuccess;
}

void bz_dev_free(void *p) {
  if (p) cudaFreeAsync(p, g_ctx.stream);
}

// See include/bullseye_gb300.h.
extern "C" void bullseye_trim_memory(void) {
  if (g_ctx.stream) cudaStreamSynchronize(g_ctx.stream);
  if (g_ctx.copy_stream) cudaStreamSynchronize(g_ctx.copy_stream);
  if (g_ctx.jones_stream) cudaStreamSynchronize(g_ctx.jones_stream);
  cudaMemPool_t pool = device_pool();
  if (pool) cudaMemPoolTrimTo(pool, 0);
}

// See include/bullseye_gb300.h.
extern "C" void bullseye_set_host_repack(int on) { g_ctx.host_repack = on != 0; }

// ---------------------------------------------------------------- host <-> device bulk copies
//
// A GB300's CPU-GPU link is coherent: SM loads and stores reach page-locked host memory mapped
// into the device's address space directly.  Bulk copies between such memory and the device run as
// a kernel of 16-byte accesses, which keeps its rate where copy-engine transfers of host buffers
// that have sat idle for a while fall to a fraction of the link's rate.  Other host memory
// (pageable, or a range that leaves its page-locked allocation) goes through cudaMemcpyAsync.
namespace {

using PointerAttrFn = CUresult (*)(void *, CUpointer_attribute, CUdeviceptr);

PointerAttrFn pointer_attr_fn() {
  static const PointerAttrFn fn = [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuPointerGetAttribute", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      f = nullptr;
    }
    return reinterpret_cast<PointerAttrFn>(f);
  }();
  return fn;
}

// Device address of host byte p when it is page-locked and mapped; nullptr otherwise.
const unsigned char *mapped_byte(const void *p) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (at.type != cudaMemoryTypeHost || !at.devicePointer) return nullptr;
  return static_cast<const unsigned char *>(at.devicePointer);
}

// Copies n bytes: in 16-byte units when src and dst share their alignment mod 16 (4-byte units
// mod 4, else bytes); the bytes before src is aligned and after the last unit go one per thread.
__global__ void link_copy_kernel(const unsigned char *__restrict__ src, unsigned char *__restrict__ dst, size_t n,
                                 int unit) {
  const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (size_t)gridDim.x * blockDim.x;
  const size_t mis = (size_t)(0 - (uintptr_t)src) & (size_t)(unit - 1);
  const size_t head = mis < n ? mis : n;
  const size_t units = (n - head) / unit;
  if (unit == 16) {
    // eight independent 16-byte loads in flight per thread before their stores (the link's
    // latency is long); the tail goes one unit at a time
    const int4 *s = reinterpret_cast<const int4 *>(src + head);
    int4 *d = reinterpret_cast<int4 *>(dst + head);
    size_t i = tid;
    for (; i + 7 * stride < units; i += 8 * stride) {
      int4 a[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) a[q] = s[i + q * stride];
#pragma unroll
      for (int q = 0; q < 8; ++q) d[i + q * stride] = a[q];
    }
    for (; i < units; i += stride) d[i] = s[i];
  } else if (unit == 4) {
    const unsigned *s = reinterpret_cast<const unsigned *>(src + head);
    unsigned *d = reinterpret_cast<unsigned *>(dst + head);
    for (size_t i = tid; i < units; i += stride) d[i] = s[i];
  } else {
    for (size_t i = tid; i < units; i += stride) dst[head + i] = src[head + i];
  }
  const size_t tail0 = head + units * unit, edge = head + (n - tail0);
  for (size_t i = tid; i < edge; i += stride) {
    const size_t b = i < head ? i : tail0 + (i - head);
    dst[b] = src[b];
  }
}

}  // namespace

const void *bz_mapped_host(const void *p, size_t n) {
  if (!p || n == 0) return nullptr;
  const unsigned char *first = mapped_byte(p);
  if (!first) return nullptr;
  const unsigned char *last = mapped_byte(static_cast<const unsigned char *>(p) + (n - 1));
  if (last != first + (n - 1)) return nullptr;
  // both ends must lie in the same page-locked allocation
  const PointerAttrFn fn = pointer_attr_fn();
  if (!fn) return nullptr;
  unsigned long long start = 0, size = 0;
  if (fn(&start, CU_POINTER_ATTRIBUTE_RANGE_START_ADDR, (CUdeviceptr)(uintptr_t)first) != CUDA_SUCCESS ||
      fn(&size, CU_POINTER_ATTRIBUTE_RANGE_SIZE, (CUdeviceptr)(uintptr_t)first) != CUDA_SUCCESS)
    return nullptr;
  const unsigned long long a = (unsigned long long)(uintptr_t)first;
  if (size == 0 || a < start || a - start + n > size) return nullptr;
  return first;
}

bool bz_copy_async(void *dst, const void *src, size_t bytes, cudaMemcpyKind kind, cudaStream_t s) {
  if (bytes == 0) return true;
  Context &c = g_ctx;
  if (c.host_copy_sm && (kind == cudaMemcpyHostToDevice || kind == cudaMemcpyDeviceToHost)) {
    const bool h2d = kind == cudaMemcpyHostToDevice;
    const void *mapped = bz_mapped_host(h2d ? src : dst, bytes);
    if (mapped) {
      const unsigned char *from = h2d ? static_cast<const unsigned char *>(mapped) : static_cast<const unsigned char *>(src);
      unsigned char *to = h2d ? static_cast<unsigned char *>(dst) : const_cast<unsigned char *>(static_cast<const unsigned char *>(mapped));
      const uintptr_t x = (uintptr_t)from ^ (uintptr_t)to;
      const int unit = (x & 15) == 0 ? 16 : (x & 3) == 0 ? 4 : 1;
      const size_t units = (bytes + unit - 1) / unit;
      static int sms = 0;  // four 512-thread CTAs per SM at most
      if (!sms) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            sms <= 0)
          sms = 1;
      }
      const unsigned blocks = (unsigned)std::min<size_t>((units + 511) / 512, (size_t)sms * 4);
      link_copy_kernel<<<blocks, 512, 0, s>>>(from, to, bytes, unit);
      c.launches++;
      BZ_CUDA_TRY_RET(cudaGetLastError(), false);
      return true;
    }
  }
  BZ_CUDA_TRY_RET(cudaMemcpyAsync(dst, src, bytes, kind, s), false);
  return true;
}

// See include/bullseye_gb300.h.
extern "C" void bullseye_set_host_copy(int mode) { g_ctx.host_copy_sm = mode != 0; }

// See include/bullseye_gb300.h.
extern "C" void bullseye_set_max_stage_bytes(size_t bytes) { g_ctx.max_stage_bytes = bytes; }

namespace {

// Sort key of every row of a chunk: its baseline slot S(2N+1-S)/2 + |a1 - a2| (S = min(a1, a2),
// wrapper.cu:358-366), or, without antenna ids, its 256-row segment; the value is the row index.
__global__ void row_keys_kernel(const unsigned *__restrict__ a1, const unsigned *__restrict__ a2, long long n,
                                long long nant, unsigned nslots, unsigned *__restrict__ keys, int *__restrict__ vals,
                                int *err) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    unsigned k;
    if (a1) {
      const long long x = a1[i], y = a2[i];
      const long long s = x < y ? x : y;
      const long long slot = (s * (2 * nant + 1 - s)) / 2 + (x > y ? x - y : y - x);
      if (slot < 0 || slot >= (long long)nslots) {
        atomicOr(err, DEV_ERR_ANTENNA);
        k = nslots - 1;
      } else {
        k = (unsigned)slot;
      }
    } else {
      k = (unsigned)(i >> 8);
    }
    keys[i] = k;
    vals[i] = (int)i;
  }
}

// Track starts of a sorted chunk: starts[k] = r0 + (first sorted position with key >= k) for every
// slot k < nslots, and starts[nslots] = r0 + n, the end of the chunk's last track (also the start
// of the next chunk's first track, written again with the same value when that chunk is sorted,
// so a chunk gridded before the next one arrives has its end), from the sorted keys (one thread
// per sorted position fills the slots it opens).
__global__ void chunk_starts_kernel(const unsigned *__restrict__ sorted_keys, long long n, unsigned nslots,
                                    long long r0, size_t *__restrict__ starts) {
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p <= n; p += (long long)gridDim.x * blockDim.x) {
    const unsigned hi = p < n ? sorted_keys[p] : nslots;  // slots <= hi start at or before p
    const unsigned lo = p > 0 ? sorted_keys[p - 1] + 1 : 0;
    for (unsigned k = lo; k <= hi && k <= nslots; ++k) starts[k] = (size_t)(r0 + p);
  }
}

// Gathers the chunk's rows from staging (caller order) into the device row buffers at row0,
// in sorted order: one warp per row, the per-row arrays copied element by element.
struct RowArrays {
  vis_complex *vis;
  vis_real *weights;
  uint8_t *flags;
  vis_real *uvw;
  uint8_t *flagged_rows;
  unsigned *field, *spw, *ant1, *ant2;
  size_t *time_ids;
};

__global__ void gather_rows_kernel(RowArrays dst, RowArrays src, const int *__restrict__ order, long long n,
                                   long long row0, int per) {
  const int lane = threadIdx.x & 31;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long p = warp; p < n; p += nwarps) {
    const long long s = order[p], d = row0 + p;
    if (src.vis)
      for (int j = lane; j < per; j += 32) dst.vis[d * per + j] = src.vis[s * per + j];
    if (src.weights)
      for (int j = lane; j < per; j += 32) dst.weights[d * per + j] = src.weights[s * per + j];
    if (src.flags)
      for (int j = lane; j < per; j += 32) dst.flags[d * per + j] = src.flags[s * per + j];
    if (lane < 3) dst.uvw[3 * d + lane] = src.uvw[3 * s + lane];
    if (lane == 3) dst.flagged_rows[d] = src.flagged_rows[s];
    if (lane == 4) dst.field[d] = src.field[s];
    if (lane == 5) dst.spw[d] = src.spw[s];
    if (lane == 6 && src.ant1) dst.ant1[d] = src.ant1[s];
    if (lane == 7 && src.ant2) dst.ant2[d] = src.ant2[s];
    if (lane == 8 && src.time_ids) dst.time_ids[d] = src.time_ids[s];
  }
}

// One host-to-device copy of a row array; with `trace` set (tracing, first chunk) it is timed alone.
template <typename T>
bool h2d(T *dst, const void *src, size_t count, cudaStream_t s, const char *trace = nullptr) {
  if (!src || count == 0) return true;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  if (trace) {
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    cudaEventRecord(t0, s);
  }
  if (!bz_copy_async(dst, src, sizeof(T) * count, cudaMemcpyHostToDevice, s)) return false;
  if (trace) {
    cudaEventRecord(t1, s);
    cudaEventSynchronize(t1);
    float ms = 0;
    cudaEventElapsedTime(&ms, t0, t1);
    bz_trace_note("%s %s%s %.2f MB %.3f ms %.1f GB/s", trace, bz_host_kind(src),
                  g_ctx.host_copy_sm && bz_mapped_host(src, sizeof(T) * count) ? " (SM copy)" : "",
                  sizeof(T) * count / 1e6, ms, sizeof(T) * count / (ms * 1e6));
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
  }
  return true;
}

__global__ void set_size_kernel(size_t *dst, size_t v) { *dst = v; }

int bits_for(unsigned n) {
  int b = 1;
  while (b < 32 && (1u << b) < n) ++b;
  return b;
}

}  // namespace

// Rows per chunk.  Gridded in one group (the default), every row of a call goes in one chunk, so
// each baseline's rows form one track, as they do for device-resident rows; the staging buffer
// then holds the whole call, up to 8 GB (bullseye_set_max_stage_bytes), beyond which the call is
// split evenly.  Gridded in G > 1 groups, calls above 64 K rows go in chunks of at least 64 K
// rows, at most max(8, G).
static constexpr double kMaxStageBytes = 8e9;

static long long chunk_rows_for(long long R, double row_bytes, int groups, size_t stage_cap) {
  const double cap = stage_cap ? (double)stage_cap : kMaxStageBytes;
  long long k;
  if (groups <= 1) {
    k = std::max<long long>(1, (long long)std::ceil(R * row_bytes / cap));
    return std::max<long long>(1, (R + k - 1) / k);
  }
  if (R <= 65536) return std::max<long long>(R, 1);
  k = std::min<long long>(std::max(8, groups), (R + 65535) / 65536);
  return (R + k - 1) / k;
}

// See context.h.
bool bz_plan_rows(const gridding_parameters &p, RowsPlan &plan) {
  Context &c = g_ctx;
  const long long R = (long long)p.row_count;
  const bool ants = p.antenna_1_ids && p.antenna_2_ids;
  const long long nant = (long long)p.antenna_count;
  const int per_row = (int)(c.nchan * c.npol);
  const double row_bytes = per_row * (sizeof(vis_complex) + sizeof(vis_real) + 1.0) + 3.0 * sizeof(vis_real) + 1 +
                           4.0 * sizeof(unsigned) + sizeof(size_t);
  const long long chunk = chunk_rows_for(R, row_bytes, c.grid_groups, c.max_stage_bytes);
  if (R > (long long)c.max_rows) {
    bz_record_error(BZ_ERR_INVALID_ARGUMENT, "row_count %zu exceeds chunk_max_row_count %zu", p.row_count, c.max_rows);
    return false;
  }
  if (ants) {
    const long long slots = p.baseline_count ? (long long)p.baseline_count : nant * (nant - 1) / 2 + nant;
    if (slots <= 0 || slots > (1ll << 30)) {
      bz_record_error(BZ_ERR_INVALID_ARGUMENT, "baseline_count %zu is out of range", p.baseline_count);
      return false;
    }
    plan.slots = (unsigned)slots;
  } else {
    plan.slots = (unsigned)((chunk + 255) / 256);
  }
  plan.chunks = R ? (int)((R + chunk - 1) / chunk) : 0;
  plan.chunk_rows = chunk;
  if ((long long)plan.chunks * plan.slots + 1 > 0x7fffffffLL) {
    bz_record_error(BZ_ERR_UNSUPPORTED, "%d row chunks x %u baseline slots exceed the track table", plan.chunks, plan.slots);
    return false;
  }
  const int per = (int)(c.nchan * c.npol);
  const size_t Rm = std::max<size_t>(1, c.max_rows);
  if (!c.vis.ptr) {
    if (!(c.vis.alloc(Rm * per) && c.weights.alloc(Rm * per) && c.flags.alloc(Rm * per) && c.uvw.alloc(3 * Rm) &&
          c.flagged_rows.alloc(Rm) && c.field.alloc(Rm) && c.spw.alloc(Rm) && c.ant1.alloc(Rm) && c.ant2.alloc(Rm) &&
          c.time_ids.alloc(Rm)))
      return false;
  }
  // staging buffers in use: one for a single chunk, two (used in turn) otherwise; a buffer's
  // capacity in rows is its time_ids length
  for (int s = 0; R && s < (plan.chunks > 1 ? 2 : 1); ++s) {
    StageBuf &g = c.stage[s];
    if (g.time_ids.n >= (size_t)chunk) continue;
    if (!(g.vis.alloc((size_t)chunk * per) && g.weights.alloc((size_t)chunk * per) &&
          g.flags.alloc((size_t)chunk * per) && g.uvw.alloc(3 * (size_t)chunk) && g.flagged_rows.alloc(chunk) &&
          g.field.alloc(chunk) && g.spw.alloc(chunk) && g.ant1.alloc(chunk) && g.ant2.alloc(chunk) &&
          g.time_ids.alloc(chunk)))
      return false;
  }
  // the sort's keys and values (input and output halves) and its scratch, for `stage_rows` rows
  if (R && c.stage_rows < (size_t)chunk) {
    size_t tmp = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tmp, (const unsigned *)nullptr, (unsigned *)nullptr, (const int *)nullptr,
                                    (int *)nullptr, (int)chunk, 0, 32, c.stream);
    if (!(c.sort_keys.alloc(2 * (size_t)chunk) && c.sort_vals.alloc(2 * (size_t)chunk) && c.sort_tmp.alloc(tmp)))
      return false;
    c.stage_rows = (size_t)chunk;
  }
  const size_t tracks = (size_t)plan.chunks * plan.slots + 1;
  if (c.track_starts.n < tracks && !c.track_starts.alloc(tracks)) return false;
  return true;
}

// See context.h.
bool bz_stream_rows(const gridding_parameters &p, bool need_vis, bool need_time, RowsPlan &plan,
                    const std::function<bool(int, long long, long long)> &on_chunk) {
  Context &c = g_ctx;
  if (!bz_plan_rows(p, plan)) return false;
  const long long R = (long long)p.row_count;
  if (R == 0) return true;
  const bool ants = p.antenna_1_ids && p.antenna_2_ids;
  const long long nant = (long long)p.antenna_count;
  const long long chunk = plan.chunk_rows;
  const int K = plan.chunks;
  const unsigned B = plan.slots;
  const int per = (int)(c.nchan * c.npol);
  // the last entry of the track table closes the last chunk's last track
  set_size_kernel<<<1, 1, 0, c.stream>>>(c.track_starts.ptr + (size_t)K * B, (size_t)R);
  RowArrays dst{c.vis.ptr, c.weights.ptr, c.flags.ptr, c.uvw.ptr, c.flagged_rows.ptr, c.field.ptr, c.spw.ptr,
                c.ant1.ptr, c.ant2.ptr, c.time_ids.ptr};
  const int bits = bits_for(B);
  // tracing only: copy times of the first chunk and of all chunks (the span includes waits for
  // staging buffers), and the memory kind of the caller's row arrays
  cudaEvent_t tr[3] = {nullptr, nullptr, nullptr};
  if (bz_tracing()) {
    for (cudaEvent_t &e : tr) cudaEventCreate(&e);
    bz_trace_note("rows vis %s weights %s flags %s uvw %s", bz_host_kind(p.visibilities),
                  bz_host_kind(p.visibility_weights), bz_host_kind(p.flags), bz_host_kind(p.uvw_coords));
  }
  double copied = 0, copied0 = 0;
  for (int k = 0; k < K; ++k) {
    const long long r0 = (long long)k * chunk, n = std::min<long long>(chunk, R - r0);
    StageBuf &g = c.stage[k & 1];
    // copy stream: this staging buffer is free once the gather of chunk k - 2 has run
    BZ_CUDA_TRY_RET(cudaStreamWaitEvent(c.copy_stream, c.ev_stage_free[k & 1], 0), false);
    const cudaStream_t cs = c.copy_stream;
    if (tr[0] && k == 0) cudaEventRecord(tr[0], cs);
    copied += (double)n * ((need_vis ? per * (sizeof(vis_complex) + sizeof(vis_real) + 1.0) : 0.0) +
                           3.0 * sizeof(vis_real) + 1 + 2 * sizeof(unsigned) + (ants ? 2 * sizeof(unsigned) : 0) +
                           (need_time ? sizeof(size_t) : 0));
    if (k == 0) copied0 = copied;
    const bool t = tr[0] && k == 0;
    if (need_vis) {
      if (!h2d(g.vis.ptr, p.visibilities + r0 * per, (size_t)n * per, cs, t ? "vis" : nullptr) ||
          !h2d(g.weights.ptr, p.visibility_weights + r0 * per, (size_t)n * per, cs, t ? "weights" : nullptr) ||
          !h2d(g.flags.ptr, reinterpret_cast<const uint8_t *>(p.flags) + r0 * per, (size_t)n * per, cs,
               t ? "flags" : nullptr))
        return false;
    }
    if (!h2d(g.uvw.ptr, reinterpret_cast<const vis_real *>(p.uvw_coords) + 3 * r0, 3 * (size_t)n, cs,
             t ? "uvw" : nullptr) ||
        !h2d(g.flagged_rows.ptr, reinterpret_cast<const uint8_t *>(p.flagged_rows) + r0, (size_t)n, cs,
             t ? "flagged_rows" : nullptr) ||
        !h2d(g.field.ptr, p.field_array + r0, (size_t)n, cs, t ? "field" : nullptr) ||
        !h2d(g.spw.ptr, p.spw_index_array + r0, (size_t)n, cs, t ? "spw" : nullptr))
      return false;
    if (ants && (!h2d(g.ant1.ptr, p.antenna_1_ids + r0, (size_t)n, cs, t ? "ant1" : nullptr) ||
                 !h2d(g.ant2.ptr, p.antenna_2_ids + r0, (size_t)n, cs, t ? "ant2" : nullptr)))
      return false;
    if (need_time && !h2d(g.time_ids.ptr, p.timestamp_ids + r0, (size_t)n, cs, t ? "time" : nullptr)) return false;
    if (tr[1] && k == 0) cudaEventRecord(tr[1], cs);
    if (tr[2] && k == K - 1) cudaEventRecord(tr[2], cs);
    BZ_CUDA_TRY_RET(cudaEventRecord(c.ev_stage_full[k & 1], cs), false);
    // library stream: sort by baseline slot, gather baseline-major, the chunk's track starts
    BZ_CUDA_TRY_RET(cudaStreamWaitEvent(c.stream, c.ev_stage_full[k & 1], 0), false);
    unsigned *keys = c.sort_keys.ptr, *keys_out = c.sort_keys.ptr + c.stage_rows;
    int *vals = c.sort_vals.ptr, *vals_out = c.sort_vals.ptr + c.stage_rows;
    row_keys_kernel<<<(unsigned)std::min<long long>((n + 255) / 256, 4096), 256, 0, c.stream>>>(
        ants ? g.ant1.ptr : nullptr, ants ? g.ant2.ptr : nullptr, n, nant, B, keys, vals, c.dev_error.ptr);
    size_t tmp = c.sort_tmp.n;
    BZ_CUDA_TRY_RET(cub::DeviceRadixSort::SortPairs(c.sort_tmp.ptr, tmp, keys, keys_out, vals, vals_out, (int)n, 0,
                                                    bits, c.stream), false);
    RowArrays src{need_vis ? g.vis.ptr : nullptr, need_vis ? g.weights.ptr : nullptr,
                  need_vis ? g.flags.ptr : nullptr, g.uvw.ptr, g.flagged_rows.ptr, g.field.ptr, g.spw.ptr,
                  ants ? g.ant1.ptr : nullptr, ants ? g.ant2.ptr : nullptr, need_time ? g.time_ids.ptr : nullptr};
    gather_rows_kernel<<<(unsigned)std::min<long long>((n * 32 + 255) / 256, 8192), 256, 0, c.stream>>>(
        dst, src, vals_out, n, r0, per);
    BZ_CUDA_TRY_RET(cudaEventRecord(c.ev_stage_free[k & 1], c.stream), false);
    chunk_starts_kernel<<<(unsigned)std::min<long long>((n + 256) / 256, 4096), 256, 0, c.stream>>>(
        keys_out, n, B, r0, c.track_starts.ptr + (size_t)k * B);
    c.launches += 3;
    BZ_CUDA_TRY_RET(cudaGetLastError(), false);
    if (on_chunk && !on_chunk(k, r0, r0 + n)) return false;
  }
  c.launches += 1;
  if (tr[0]) {
    cudaEventSynchronize(tr[2]);
    float first = 0, all = 0;
    cudaEventElapsedTime(&first, tr[0], tr[1]);
    cudaEventElapsedTime(&all, tr[0], tr[2]);
    bz_trace_note("rows_copy %d chunks %.1f MB; first chunk %.3f ms %.1f GB/s; all %.3f ms %.1f GB/s", K, copied / 1e6,
                  first, copied0 / (first * 1e6), all, copied / (all * 1e6));
    for (cudaEvent_t e : tr) cudaEventDestroy(e);
  }
  c.rows_plan = plan;
  c.rows_key[0] = p.uvw_coords;
  c.rows_key[1] = p.antenna_1_ids;
  c.rows_key[2] = need_vis ? (const void *)p.visibilities : nullptr;
  c.rows_key_count = p.row_count;
  c.rows_with_vis = need_vis;
  c.rows_with_time = need_time;
  return true;
}

// See context.h.
bool bz_upload_rows(const gridding_parameters &p, bool need_vis, bool need_time, RowsPlan &plan,
                    const std::function<bool(int, long long, long long)> &on_chunk) {
  Context &c = g_ctx;
  const bool same = c.rows_key_count == p.row_count && c.rows_key[0] == p.uvw_coords &&
                    c.rows_key[1] == p.antenna_1_ids && (!need_vis || (c.rows_with_vis && c.rows_key[2] == p.visibilities)) &&
                    (!need_time || c.rows_with_time) && p.uvw_coords != nullptr;
  if (same && !on_chunk) {
    plan = c.rows_plan;
    return true;
  }
  return bz_stream_rows(p, need_vis, need_time, plan, on_chunk);
}

// Forget the rows on the device (after gridding_barrier the caller may change its arrays).
void bz_forget_rows() {
  Context &c = g_ctx;
  c.rows_key[0] = c.rows_key[1] = c.rows_key[2] = nullptr;
  c.rows_key_count = 0;
  c.rows_with_vis = c.rows_with_time = false;
}
