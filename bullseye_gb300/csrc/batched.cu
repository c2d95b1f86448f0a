// Batched, support-aware gridding: one call grids every facet (and the sampling function) of a
// chunk with a schedule built on the device and replayed as a CUDA graph.
//
// Support awareness.  The reference's ABI carries one padded kernel support W for every w plane
// (bullseye/mo/cpu_gpu_common/gridding_parameters.h:66-67), so each visibility is spread over
// W x W cells even when its plane's kernel is much narrower; the taps outside a plane's window
// are exactly zero.  The window of every plane is read from the kernel table once, rounded up to
// a support class (a few widths), and each visibility is gridded over its class's window only:
// the same sums, computed over nonzero (or possibly nonzero) taps.
//
// Schedule (all on the device, so it can be captured and replayed):
//   classify     class of every (channel, row) from its w plane (FP64, as the gridder);
//   seg_count    per track (baseline, channel): number of runs of one class;
//   scan         track offsets;
//   seg_write    the runs {row_begin, row_end, channel, class};
//   bucket       runs ordered by class;
//   per class    one persistent Romein launch (romein_segment_kernel) over (run, facet) items,
//                with the thread layout chosen for that class width by the autotuner; then the
//                same for the sampling function (facet-invariant, gridded once).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

#include "context.h"

using namespace bz;

namespace {

constexpr int kMaxClasses = 32;

// Rows [r0, r0 + n) of R: cls[c * R + r].
__global__ void classify_kernel(const vis_real *__restrict__ uvw, const unsigned *__restrict__ spw,
                                const vis_real *__restrict__ wavelengths, int nchan, int nspw, long long R,
                                double wmax, int P, const int *__restrict__ plane_class, unsigned char *__restrict__ cls,
                                long long r0, long long n) {
  const double plane_scale = P > 1 ? (double)(P - 1) / wmax : 0.0;  // as the gridder's prologue
  const long long total = (long long)nchan * n;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(i / n);
    const long long r = r0 + (i - (long long)c * n);
    int k = plane_class[0];
    if (P > 1) {
      const unsigned s = spw[r];
      if (s < (unsigned)nspw) {
        const double inv = 1.0 / (double)wavelengths[(long long)s * nchan + c];
        const double w = (double)uvw[3 * r + 2] * inv;
        const double pl = rint(fabs(w) * plane_scale);
        if (pl >= 0.0 && pl < (double)P) k = plane_class[(int)pl];
      }
    }
    cls[(long long)c * R + r] = (unsigned char)k;
  }
}

__device__ __forceinline__ void track_rows(int t, int nchan, int nslots, int seg_len, long long R, const size_t *starts,
                                           int &c, long long &r0, long long &r1) {
  const int b = t / nchan;
  c = t - b * nchan;
  if (starts) {
    r0 = (long long)starts[b];
    r1 = (long long)starts[b + 1];
  } else {
    r0 = (long long)b * seg_len;
    r1 = r0 + seg_len;
  }
  if (r1 > R) r1 = R;
  if (r0 > r1) r0 = r1;
}

__global__ void seg_count_kernel(const size_t *starts, int nslots, int seg_len, long long R, int nchan,
                                 const unsigned char *__restrict__ cls, int *__restrict__ nseg) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nslots * nchan) return;
  int c;
  long long r0, r1;
  track_rows(t, nchan, nslots, seg_len, R, starts, c, r0, r1);
  const unsigned char *k = cls + (long long)c * R;
  int n = 0;
  int prev = -1;
  for (long long r = r0; r < r1; ++r) {
    if (k[r] != prev) {
      ++n;
      prev = k[r];
    }
  }
  nseg[t] = n;
}

// Exclusive scan of n ints by one block; total -> *total.
__global__ void scan_kernel(const int *__restrict__ in, int *__restrict__ out, int n, int *total) {
  __shared__ int part[1024];
  const int tid = threadIdx.x, nt = blockDim.x;
  const int per = (n + nt - 1) / nt;
  const int lo = tid * per, hi = min(n, lo + per);
  int s = 0;
  for (int i = lo; i < hi; ++i) s += in[i];
  part[tid] = s;
  __syncthreads();
  for (int off = 1; off < nt; off <<= 1) {
    int v = tid >= off ? part[tid - off] : 0;
    __syncthreads();
    part[tid] += v;
    __syncthreads();
  }
  int run = tid ? part[tid - 1] : 0;
  for (int i = lo; i < hi; ++i) {
    out[i] = run;
    run += in[i];
  }
  if (tid == nt - 1) *total = part[nt - 1];
}

// Class indices come from plane_class (< the class count, <= kMaxClasses); a run whose class lies
// outside the table is left out and reported rather than counted out of bounds.
__global__ void seg_write_kernel(const size_t *starts, int nslots, int seg_len, long long R, int nchan,
                                 const unsigned char *__restrict__ cls, const int *__restrict__ off,
                                 int4 *__restrict__ segs, int *__restrict__ class_count, int ncls, int *err) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nslots * nchan) return;
  int c;
  long long r0, r1;
  track_rows(t, nchan, nslots, seg_len, R, starts, c, r0, r1);
  const unsigned char *k = cls + (long long)c * R;
  int o = off[t];
  long long begin = r0;
  for (long long r = r0; r < r1; ++r) {
    if (r + 1 == r1 || k[r + 1] != k[r]) {
      const int kc = k[r] < ncls ? (int)k[r] : -1;
      if (kc < 0) atomicOr(err, DEV_ERR_GRID_INDEX);
      segs[o++] = make_int4((int)begin, (int)(r + 1), c, kc);
      if (kc >= 0) atomicAdd(&class_count[kc], 1);
      begin = r + 1;
    }
  }
}

__global__ void class_offsets_kernel(const int *class_count, int *class_off, int *class_cursor, int ncls) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int s = 0;
  for (int k = 0; k < ncls; ++k) {
    class_off[k] = s;
    class_cursor[k] = 0;
    s += class_count[k];
  }
}

__global__ void bucket_kernel(const int4 *__restrict__ segs, const int *total, int4 *__restrict__ sorted,
                              int *class_cursor, const int *class_off) {
  const int n = *total;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int4 s = segs[i];
    if (s.w < 0) continue;  // reported by seg_write_kernel
    const int pos = class_off[s.w] + atomicAdd(&class_cursor[s.w], 1);
    sorted[pos] = s;
  }
}

// Exclusive scan of the scheduled segments' row counts by one block: rec_off[i] = rows of the
// segments before i (in class order), rec_off[n] = all rows; n = the segments of every class.
__global__ void rec_offsets_kernel(const int4 *__restrict__ sorted, const int *__restrict__ class_count, int ncls,
                                   long long *__restrict__ rec_off) {
  __shared__ long long part[1024];
  int n = 0;
  for (int k = 0; k < ncls; ++k) n += class_count[k];
  const int tid = threadIdx.x, nt = blockDim.x;
  const int per = (n + nt - 1) / nt;
  const int lo = min(n, tid * per), hi = min(n, lo + per);
  long long sum = 0;
  for (int i = lo; i < hi; ++i) sum += sorted[i].y - sorted[i].x;
  part[tid] = sum;
  __syncthreads();
  for (int off = 1; off < nt; off <<= 1) {
    const long long v = tid >= off ? part[tid - off] : 0;
    __syncthreads();
    part[tid] += v;
    __syncthreads();
  }
  long long run = tid ? part[tid - 1] : 0;
  for (int i = lo; i < hi; ++i) {
    rec_off[i] = run;
    run += sorted[i].y - sorted[i].x;
  }
  if (tid == nt - 1) rec_off[n] = part[nt - 1];
}

// Facets a warp of the record kernel takes at once (its per-facet range and sums sit in shared
// memory); more facets are taken in blocks, each block reloading the segment's rows.
constexpr int kRecordFacetBlock = 32;
constexpr int kRecordWarps = 8;

template <int NC>
constexpr size_t record_smem_bytes() {
  return (size_t)kRecordWarps * kRecordFacetBlock * (NC * sizeof(double) + sizeof(int2) + sizeof(int) + sizeof(DfFacet));
}

// Visibility records of every scheduled segment, one warp per segment taking segments from a
// counter.  Each lane loads one row of the segment (load_row) and writes its record for every
// facet (facet_record: the in-place gridder's prologue, so the same cells, taps, corrections and
// weights) at rec_off[si] x F + f x len + row, with the footprint residues for the segment's class
// width.  Per facet the warp keeps, in shared memory, the first and last valid row (the work item's
// range) and the normalisation sums of the current grid group (added to the global sums when the
// group changes and when the segment ends).  A segment whose records would pass `capacity` is left
// to the segment kernel's in-place prologue.
template <int NC, bool WPROJ>
__global__ void __launch_bounds__(kRecordWarps * 32) record_kernel(
    const GridArgs a, const int4 *__restrict__ sorted, const int *__restrict__ class_count, int ncls,
    const long long *__restrict__ rec_off, const int *__restrict__ widths, int nfacets, GridRec<NC> *__restrict__ out,
    long long capacity, int2 *__restrict__ range, long long range_items, int *next) {
  extern __shared__ __align__(16) unsigned char rk_smem[];
  constexpr int FB = kRecordFacetBlock;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double *s_norm = reinterpret_cast<double *>(rk_smem) + (size_t)warp * FB * NC;                  // [FB][NC]
  int2 *s_rng = reinterpret_cast<int2 *>(rk_smem + (size_t)kRecordWarps * FB * NC * sizeof(double)) +
                (size_t)warp * FB;                                                                 // [FB]
  int *s_ng = reinterpret_cast<int *>(rk_smem + (size_t)kRecordWarps * FB * (NC * sizeof(double) + sizeof(int2))) +
              (size_t)warp * FB;                                                                   // [FB]
  // single precision: the facets' double-float constants for the segment's spw
  DfFacet *s_df = reinterpret_cast<DfFacet *>(rk_smem + (size_t)kRecordWarps * FB *
                                                           (NC * sizeof(double) + sizeof(int2) + sizeof(int))) +
                  (size_t)warp * FB;                                                               // [FB]
  (void)s_df;
  int nseg = 0;
  for (int k = 0; k < ncls; ++k) nseg += class_count[k];
  const double plane_scale = WPROJ ? (double)(a.P - 1) / a.wmax : 0.0;
  const bool want_norm = a.norm != nullptr;
  for (;;) {
    int si = 0;
    if (lane == 0) si = atomicAdd(next, 1);
    si = __shfl_sync(0xffffffffu, si, 0);
    if (si >= nseg) break;
    const int4 sg = sorted[si];
    if (sg.x < 0 || sg.x > sg.y || (long long)sg.y > a.nrows || sg.z < 0 || sg.z >= a.nchan || sg.w < 0 ||
        sg.w >= ncls) {
      if (lane == 0) atomicOr(a.error, DEV_ERR_GRID_INDEX);
      continue;
    }
    const int len = sg.y - sg.x;
    if ((rec_off[si] + len) * nfacets > capacity) continue;
    GridRec<NC> *seg_out = out + rec_off[si] * nfacets;
    // residues mod the class width by a multiply-high (exact for corners below 2^26), corrected
    const unsigned Wc = (unsigned)widths[sg.w];
    const unsigned mag = 0xffffffffu / Wc + 1u;
    // the segment's spw (its first row's): rows of that spw use the double-float cell choice
    unsigned dspw = 0xffffffffu;
    double dinv = 0.0;
#if defined(BULLSEYE_SINGLE)
    {
      const unsigned s0 = a.spw[sg.x];
      if (len > 0 && s0 < (unsigned)a.nspw) {
        dspw = s0;
        dinv = 1.0 / (double)a.wavelengths[(long long)s0 * a.nchan + sg.z];
      }
    }
#else
    (void)dinv;  // the 64-bit library keeps the FP64 cell choice
#endif
    for (int f0 = 0; f0 < nfacets; f0 += FB) {
      const int fb = min(FB, nfacets - f0);
      for (int j = lane; j < fb; j += 32) {
        s_rng[j] = make_int2(0x7fffffff, 0);
        s_ng[j] = -1;
#pragma unroll
        for (int k = 0; k < NC; ++k) s_norm[j * NC + k] = 0.0;
#if defined(BULLSEYE_SINGLE)
        if (dspw != 0xffffffffu) df_facet(a.facets[f0 + j], dinv, a.os, s_df[j]);
#endif
      }
      __syncwarp();
      unsigned cspw = 0xffffffffu;
      double inv = 0.0;
      for (int b = 0; b < len; b += 32) {
        const int i = b + lane;
        RowInputs<NC> ri;
        load_row<NC>(a, sg.z, (long long)sg.x + i, i < len, ri);
        if (ri.use && ri.spw != cspw) {
          cspw = ri.spw;
          inv = 1.0 / (double)a.wavelengths[ri.sc];
        }
        // the w plane does not depend on the facet: choose_cells' FP64 expression, once per row
        const bool use_df = ri.use && ri.spw == dspw;
        int plane_df = 0;
        if (WPROJ && use_df) {
          const double pl = rint(fabs(ri.wm) * (inv * plane_scale));
          plane_df = (pl >= 0.0 && pl < (double)a.P) ? (int)pl : -1;
        }
        for (int fj = 0; fj < fb; ++fj) {
          const int f = f0 + fj;
          VisRec<NC> rec;
          facet_record<NC, WPROJ>(a, f, sg.z, (long long)sg.x + i, ri, inv, rec, plane_scale,
                                  use_df ? &s_df[fj] : nullptr, plane_df);
          const bool v = i < len && rec.valid;
          if (i < len) {
            GridRec<NC> g;
            if (v) {
              const unsigned u0 = (unsigned)rec.u0, v0 = (unsigned)rec.v0;
              int ru = (int)(u0 - __umulhi(u0, mag) * Wc), rv = (int)(v0 - __umulhi(v0, mag) * Wc);
              ru += ru < 0 ? (int)Wc : 0;
              rv += rv < 0 ? (int)Wc : 0;
              g.u0 = rec.u0; g.v0 = rec.v0; g.ru = ru; g.rv = rv;
              g.g = rec.g; g.valid = 1; g.fu = rec.fu; g.fv = rec.fv;
#pragma unroll
              for (int k = 0; k < NC; ++k) g.vis[k] = rec.vis[k];
            } else {
              g.u0 = g.v0 = g.ru = g.rv = g.g = g.valid = g.fu = g.fv = 0;
#pragma unroll
              for (int k = 0; k < NC; ++k) g.vis[k].re = g.vis[k].im = 0;
            }
            seg_out[(long long)f * len + i] = g;
          }
          const unsigned m = __ballot_sync(0xffffffffu, v);
          if (!m) continue;
          if (lane == 0) {
            int2 r = s_rng[fj];
            if (r.x == 0x7fffffff) r.x = b + __ffs(m) - 1;
            r.y = b + 32 - __clz(m);
            s_rng[fj] = r;
          }
          if (!want_norm) continue;
          NormTerm t[NC];
          const int gv = v ? rec.g : -1;
          if (v) {
            NormTerm nt;
#if defined(BULLSEYE_SINGLE)
            if (a.tap_sums_f) {  // single precision: the row sums rounded to FP32, multiplied in FP32
              const float *su = a.tap_sums_f + 2 * ((long long)rec.plane * a.tap_f + rec.fu0);
              const float *sv = a.tap_sums_f + 2 * ((long long)rec.plane * a.tap_f + rec.fv0);
              nt = fmaf(su[0], sv[0], -__fmul_rn(su[1], sv[1]));
            } else
#endif
            {
              const double *su = a.tap_sums + 2 * ((long long)rec.plane * a.tap_f + rec.fu0);
              const double *sv = a.tap_sums + 2 * ((long long)rec.plane * a.tap_f + rec.fv0);
              nt = (NormTerm)(su[0] * sv[0] - su[1] * sv[1]);
            }
#pragma unroll
            for (int k = 0; k < NC; ++k) t[k] = (NormTerm)rec.cw[k] * nt;
          } else {
#pragma unroll
            for (int k = 0; k < NC; ++k) t[k] = 0;
          }
          const int g0 = __shfl_sync(0xffffffffu, gv, __ffs(m) - 1);
          const long long fslice = (long long)(a.facet_base + f) * a.groups;
          if (__all_sync(0xffffffffu, gv < 0 || gv == g0)) {
            __syncwarp();  // the lanes' earlier additions to s_norm are seen by lane 0
            if (lane == 0 && s_ng[fj] != g0) {
              if (s_ng[fj] >= 0) {
#pragma unroll
                for (int k = 0; k < NC; ++k)
                  if (s_norm[fj * NC + k] != 0.0) atomicAdd(&a.norm[(fslice + s_ng[fj]) * NC + k], s_norm[fj * NC + k]);
              }
#pragma unroll
              for (int k = 0; k < NC; ++k) s_norm[fj * NC + k] = 0.0;
              s_ng[fj] = g0;
            }
            __syncwarp();  // lane 0's reset is seen by the lanes that add below
            // a warp's 32 terms are summed in the working precision (positive terms: a relative
            // error of a few FP32 units at most), the sums of the warps in FP64.  The butterfly
            // leaves the same sum in every lane (each step adds the same two partials), and lane k
            // adds correlation k: the NC FP64 additions are one warp instruction, not NC.
            NormTerm mine = 0;
#pragma unroll
            for (int k = 0; k < NC; ++k) {
              NormTerm x = t[k];
#pragma unroll
              for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
              if (lane == k) mine = x;
            }
            if (lane < NC) s_norm[fj * NC + lane] += (double)mine;
          } else if (v) {
#pragma unroll
            for (int k = 0; k < NC; ++k)
              if (t[k] != 0) atomicAdd(&a.norm[(fslice + gv) * NC + k], (double)t[k]);
          }
        }
      }
      __syncwarp();
      // the block's work-item ranges and remaining sums
      for (int j = lane; j < fb; j += 32) {
        const long long item = (long long)si * nfacets + f0 + j;
        const int2 r = s_rng[j];
        if (item < range_items) range[item] = r.x == 0x7fffffff ? make_int2(0, 0) : r;
        if (want_norm && s_ng[j] >= 0) {
          const long long fslice = (long long)(a.facet_base + f0 + j) * a.groups;
#pragma unroll
          for (int k = 0; k < NC; ++k)
            if (s_norm[j * NC + k] != 0.0) atomicAdd(&a.norm[(fslice + s_ng[j]) * NC + k], s_norm[j * NC + k]);
        }
      }
      __syncwarp();
    }
  }
}

// ---------------------------------------------------------------- launch variants
// A thread layout of one support class; NT = 0 marks a layout not chosen for the current build.
struct Variant {
  int J = 0;
  bool wide = false;
  int regs = 0;  // register cap of the build
  int NT = 0, V = 0, grid = 0;
  size_t smem = 0;
};

template <int NC, bool WPROJ, bool COMP>
using SegKernel = void (*)(const GridArgs, const int);

template <int NC, bool WPROJ, bool COMP, bool WIDE>
SegKernel<NC, WPROJ, COMP> seg_kernel_of(int J, int regs) {
  if (J == 8) return romein_segment_kernel<NC, WPROJ, 8, COMP, WIDE>;
#if defined(BULLSEYE_SINGLE)
  if constexpr (NC == 4 && WPROJ) {
    if (J == 6) return romein_segment_kernel<NC, WPROJ, 6, COMP, WIDE, kSegRegs6>;
  }
#endif
  if constexpr (NC == 4 && WPROJ) {
    if (regs == 64) return romein_segment_kernel<NC, WPROJ, 4, COMP, WIDE, 64>;
    if (regs == 72) return romein_segment_kernel<NC, WPROJ, 4, COMP, WIDE, 72>;
  }
  return romein_segment_kernel<NC, WPROJ, 4, COMP, WIDE>;
}

template <int NC, bool WPROJ, bool COMP>
SegKernel<NC, WPROJ, COMP> seg_kernel(int J, bool wide, int regs) {
  return wide ? seg_kernel_of<NC, WPROJ, COMP, true>(J, regs) : seg_kernel_of<NC, WPROJ, COMP, false>(J, regs);
}

// Register caps the tuner tries for a layout.
template <int NC, bool WPROJ>
std::vector<int> reg_caps(int J) {
  if (J == 8) return {kSegRegs<8>};
  if (J == 6) return {kSegRegs6};
  if (NC == 4 && WPROJ) return {kSegRegs<4>, 72, 64};
  return {kSegRegs<4>};
}

template <int NC, bool WPROJ>
bool make_variant(int W, int J, bool wide, int regs, Variant &v) {
  const int cols = ((W + 31) / 32) * 32;
  if (wide && (cols - W) * 8 > W) return false;
  const int owners = wide ? cols * ((W + J - 1) / J) : W * ((W + J - 1) / J);
  v.J = J;
  v.wide = wide;
  v.regs = regs;
  v.NT = std::max(32, ((owners + 31) / 32) * 32);
  if (v.NT > 512) return false;
  v.V = grid_chunk_size<NC, WPROJ>(W, v.NT, J, regs);
  v.smem = grid_smem_bytes<NC, WPROJ>(v.V, W, v.NT, J);
  return true;
}

struct ClassInfo {
  int width;
  Variant vis, sf;  // chosen layouts for the visibility (NC = c.C) and sampling (NC = 1) launches
};

struct BatchedState {
  bool planned = false;
  int ncls = 0;
  ClassInfo cls[kMaxClasses];
  DevBuf<int> plane_class, plane_lo;
  DevBuf<unsigned char> row_class;
  DevBuf<int> nseg, seg_off, seg_total, class_count, class_off, class_cursor, work_next, sample_count;
  DevBuf<int4> segs, sorted;
  DevBuf<FacetXform> facet_table;  // per-facet geometry of bullseye_grid_batched_facets
  DevBuf<vis_real> conv_w;         // support-window table [P][tap_f][conv_w_stride] (plan_classes)
  int conv_w_stride = 0;
  size_t rows_cap = 0, tracks_cap = 0, segs_cap = 0;
  // tuning decisions, by (class width, NC, WPROJ, COMP)
  std::map<std::tuple<int, int, int, int>, std::tuple<int, int, int>> tuned;  // -> (J, wide, regs)
  // captured graphs, by launch arguments (two slots: the reference's exports alternate between
  // the visibilities and the sampling function); least recently used is replaced
  struct GraphSlot {
    cudaGraphExec_t exec = nullptr;
    std::vector<unsigned char> key;
    unsigned long long used = 0;
  };
  GraphSlot graphs[2];
  unsigned long long graph_clock = 0;
  void drop_graphs() {
    for (auto &g : graphs) {
      if (g.exec) cudaGraphExecDestroy(g.exec);
      g.exec = nullptr;
      g.key.clear();
      g.used = 0;
    }
  }
  // eager, per-class timed mode (bullseye_set_batched_profiling)
  bool profile = false;
  struct ClassRecord {
    int width, nc, J, wide, items;
    float ms;
  };
  std::vector<ClassRecord> records;
  std::vector<int> plane_width;  // class width of every w plane (plan_classes)
  // precomputed visibility records (record_kernel): the buffer and its budget, the per-segment
  // record offsets, the per-item valid ranges, the class widths on the device, a work counter
  bool vrec_on = true;
  size_t vrec_budget = 0;        // bytes; 0: 30 % of the device's memory
  DevBuf<unsigned char> vrec;
  DevBuf<long long> vrec_off;    // [segs_cap + 1]
  DevBuf<int2> vrec_range;
  long long vrec_range_items = 0;
  DevBuf<int> cls_width, vrec_next;
};
BatchedState g_bs;

// Support windows of every w plane, rounded up to a class width.  A cell s of the footprint
// reads table sample fu + s*os, where fu = trunc((1 - u + round(u)) * os) spans
// [floor(os/2), floor(3 os/2)] with round-to-nearest (w-projection) and [0, os] with floor (AA);
// the window keeps every s that can reach a nonzero sample for some fu in that range, so the
// taps left out are exactly zero.  Only the class widths some plane uses get a launch.
// Candidate class widths for full support W, ascending; the last is W itself.
// The library's batched calls (fine = true) take every even width from 16: each class launch
// grids its planes' windows with less padding, and only the widths some plane uses are launched.
// The workspace entry launches every candidate and keeps the coarser list.
std::vector<int> class_candidates(int W, bool fine = false) {
  std::vector<int> cand;
  if (fine) {
    for (int w = 16; w < W && (int)cand.size() < kMaxClasses - 1; w += 2) cand.push_back(w);
  } else {
    for (int w : {16, 18, 20, 22, 24, 28, 32, 36, 40, 44, 48, 56})
      if (w < W) cand.push_back(w);
  }
  cand.push_back(W);
  return cand;
}

bool plan_classes() {
  Context &c = g_ctx;
  BatchedState &b = g_bs;
  const int W = (int)c.W, os = (int)c.os, K = (int)c.K, P = (int)c.P;
  const bool wproj = c.P > 1;
  const std::vector<int> cand = class_candidates(W, true);
  const int fu_min = wproj ? (int)std::floor(0.5 * os - 1e-6) : 0;
  const int fu_max = wproj ? (int)std::floor(1.5 * os + 1e-6) : os;
  std::vector<int> pw(P), plo(P);
  for (int p = 0; p < P; ++p) {
    int nzlo = -1, nzhi = -1;
    for (int i = 0; i < K; ++i) {
      bool nz;
      if (wproj) nz = c.conv_host[2 * ((size_t)p * K + i)] != 0 || c.conv_host[2 * ((size_t)p * K + i) + 1] != 0;
      else nz = c.conv_host[i] != 0;
      if (nz) {
        if (nzlo < 0) nzlo = i;
        nzhi = i;
      }
    }
    int slo = 0, shi = 0;
    if (nzlo >= 0) {
      slo = std::max(0, (int)std::ceil((double)(nzlo - fu_max) / os));
      shi = std::min(W - 1, (int)std::floor((double)(nzhi - fu_min) / os));
      if (shi < slo) shi = slo;
    }
    const int width = shi - slo + 1;
    int cw = W;
    for (int w : cand)
      if (w >= width) { cw = w; break; }
    pw[p] = cw;
    plo[p] = std::min(slo, W - cw);
  }
  std::vector<int> widths;
  for (int w : cand)
    if (std::find(pw.begin(), pw.end(), w) != pw.end()) widths.push_back(w);
  std::vector<int> pcls(P);
  for (int p = 0; p < P; ++p) pcls[p] = (int)(std::find(widths.begin(), widths.end(), pw[p]) - widths.begin());
  // Support-window table: row (plane p, tap offset f) holds the taps s = plo[p] + j,
  // j < pw[p] (conv[p][f + s os]), then its first 7 taps again (the J - 1 <= 7 repeated leading
  // row taps of a Romein strip), zero-padded to a multiple of 16 bytes.  A staged tap row is then
  // one 16-byte aligned bulk copy from the row start.
  {
    const size_t ncomp = wproj ? 2 : 1;
    const int E = (int)(16 / (ncomp * sizeof(vis_real)));
    const int pwmax = *std::max_element(pw.begin(), pw.end());
    const int L = (pwmax + 7 + E - 1) / E * E;
    const size_t tf = c.tap_f;
    std::vector<vis_real> tab(ncomp * (size_t)P * tf * L, (vis_real)0);
    for (int p = 0; p < P; ++p)
      for (size_t f = 0; f < tf; ++f) {
        vis_real *row = tab.data() + ncomp * (((size_t)p * tf + f) * L);
        for (int j = 0; j < pw[p]; ++j) {
          const size_t i = f + (size_t)(plo[p] + j) * os;
          if (i >= (size_t)K) break;
          for (size_t q = 0; q < ncomp; ++q) row[ncomp * j + q] = c.conv_host[ncomp * ((size_t)p * K + i) + q];
        }
        for (int j = pw[p]; j < pw[p] + 7; ++j)
          for (size_t q = 0; q < ncomp; ++q) row[ncomp * j + q] = row[ncomp * (j - pw[p]) + q];
      }
    if (!b.conv_w.alloc(tab.size())) return false;
    BZ_CUDA_TRY_RET(cudaMemcpy(b.conv_w.ptr, tab.data(), sizeof(vis_real) * tab.size(), cudaMemcpyHostToDevice), false);
    b.conv_w_stride = L;
  }
  b.plane_width = pw;
  b.ncls = (int)widths.size();
  if (b.ncls > kMaxClasses) return false;
  for (int k = 0; k < b.ncls; ++k) {
    b.cls[k].width = widths[k];
    b.cls[k].vis = Variant();  // chosen again (from the tuned decisions) for each call's build
    b.cls[k].sf = Variant();
  }
  {
    int wd[kMaxClasses] = {0};
    for (int k = 0; k < b.ncls; ++k) wd[k] = widths[k];
    if (!b.cls_width.alloc(kMaxClasses)) return false;
    BZ_CUDA_TRY_RET(cudaMemcpy(b.cls_width.ptr, wd, sizeof(wd), cudaMemcpyHostToDevice), false);
  }
  if (!b.plane_class.alloc(P) || !b.plane_lo.alloc(P)) return false;
  BZ_CUDA_TRY_RET(cudaMemcpy(b.plane_class.ptr, pcls.data(), sizeof(int) * P, cudaMemcpyHostToDevice), false);
  BZ_CUDA_TRY_RET(cudaMemcpy(b.plane_lo.ptr, plo.data(), sizeof(int) * P, cudaMemcpyHostToDevice), false);
  if (!b.class_count.alloc(kMaxClasses) || !b.class_off.alloc(kMaxClasses) || !b.class_cursor.alloc(kMaxClasses) ||
      !b.work_next.alloc(2 * kMaxClasses) || !b.seg_total.alloc(1) || !b.sample_count.alloc(2 * kMaxClasses))
    return false;
  b.planned = true;
  return true;
}

// Grows the schedule buffers; a reallocation invalidates the captured graph (it holds the
// buffer addresses).
bool ensure_capacity(size_t rows, size_t tracks) {
  Context &c = g_ctx;
  BatchedState &b = g_bs;
  const void *before[3] = {b.row_class.ptr, b.nseg.ptr, b.segs.ptr};
  if (rows * c.nchan > b.rows_cap) {
    if (!b.row_class.alloc(rows * c.nchan)) return false;
    b.rows_cap = rows * c.nchan;
  }
  if (tracks > b.tracks_cap) {
    if (!b.nseg.alloc(tracks) || !b.seg_off.alloc(tracks)) return false;
    b.tracks_cap = tracks;
  }
  // runs: at most one per (track, class change); bound by rows x channels
  const size_t maxseg = std::max<size_t>(rows * c.nchan, 1);
  if (maxseg > b.segs_cap) {
    if (!b.segs.alloc(maxseg) || !b.sorted.alloc(maxseg)) return false;
    b.segs_cap = maxseg;
  }
  if (before[0] != b.row_class.ptr || before[1] != b.nseg.ptr || before[2] != b.segs.ptr) b.drop_graphs();
  return true;
}

// The dynamic shared-memory limit is an attribute of the kernel function that a graph launch reads
// when it runs, not when it was captured, and support classes of different sizes can share one
// instantiation: open each instantiation to the device's opt-in maximum instead of a class's size.
template <typename Kern>
bool open_smem(Kern kern) {
  cudaFuncAttributes fa;
  int dev = 0, optin = 0;
  if (cudaFuncGetAttributes(&fa, kern) != cudaSuccess || cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
    return false;
  return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes) ==
         cudaSuccess;
}

// Sizes the visibility-record buffers for a call of `rows` rows over nfacets facets (before any
// capture: the captured launches hold their addresses).  The records take at most the record
// budget and the free memory; segments past the capacity are gridded in place.  `segments` (the
// schedule's segment count, 0 when unknown) sizes the per-item range table.
bool ensure_records(int nfacets, long long rows, int nchan, long long segments) {
  BatchedState &b = g_bs;
  if (!b.vrec_on || !b.conv_w.ptr || rows <= 0) return true;
  size_t fr = 0, tot = 0;
  if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
    cudaGetLastError();
    return true;
  }
  const size_t budget = b.vrec_budget ? b.vrec_budget : tot / 10 * 3;
  const double need = (double)std::max(nfacets, 1) * (double)rows * nchan * sizeof(GridRec<4>);
  const void *before[3] = {b.vrec.ptr, b.vrec_off.ptr, b.vrec_range.ptr};
  const double room = (double)b.vrec.n + (double)fr * 0.8;
  const size_t want = (size_t)(std::min(need, std::min((double)budget, room)) / 256) * 256;
  if (want > b.vrec.n && want >= (1u << 20)) {
    b.vrec.release();
    if (!b.vrec.alloc(want)) return false;
  }
  if (b.vrec_off.n < b.segs_cap + 1 && !b.vrec_off.alloc(b.segs_cap + 1)) return false;
  const long long seg = segments > 0 ? segments + segments / 4 + 4096 : std::min<long long>((long long)b.segs_cap, 1 << 20);
  const long long items = seg * std::max(nfacets, 1);
  if (items > b.vrec_range_items) {
    if (!b.vrec_range.alloc((size_t)items)) return false;
    b.vrec_range_items = items;
  }
  if (!b.vrec_next.ptr && !b.vrec_next.alloc(1)) return false;
  if (before[0] != b.vrec.ptr || before[1] != b.vrec_off.ptr || before[2] != b.vrec_range.ptr) b.drop_graphs();
  return true;
}

template <int NC>
void set_record_args(GridArgs &a) {
  BatchedState &b = g_bs;
  a.records = b.vrec.ptr;
  a.rec_off = b.vrec_off.ptr;
  a.item_range = b.vrec_range.ptr;
  a.rec_capacity = (long long)(b.vrec.n / sizeof(GridRec<NC>));
  a.range_capacity = b.vrec_range_items;
}

// The visibility records of this build's work items (all classes) ahead of its class launches;
// `out` is `base` with the record arguments, or `base` itself when records are off or cannot be
// used (no record buffer, no support-window table, or normalisation without kernel row sums).
template <int NC, bool WPROJ>
bool launch_records(const GridArgs &base, int nfacets, cudaStream_t st, GridArgs &out) {
  BatchedState &b = g_bs;
  out = base;
  if (!b.vrec_on || !b.vrec.ptr || !b.vrec_off.ptr || !b.vrec_range.ptr || !b.conv_w.ptr || !b.cls_width.ptr ||
      (base.norm && !base.tap_sums))
    return true;
  GridArgs a = base;
  a.plane_lo = b.plane_lo.ptr;
  a.conv_w = b.conv_w.ptr;
  a.conv_w_stride = b.conv_w_stride;
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  BZ_CUDA_TRY_RET(cudaMemsetAsync(b.vrec_next.ptr, 0, sizeof(int), st), false);
  rec_offsets_kernel<<<1, 1024, 0, st>>>(b.sorted.ptr, b.class_count.ptr, b.ncls, b.vrec_off.ptr);
  record_kernel<NC, WPROJ><<<sms * 4, kRecordWarps * 32, record_smem_bytes<NC>(), st>>>(
      a, b.sorted.ptr, b.class_count.ptr, b.ncls, b.vrec_off.ptr,
                                                    b.cls_width.ptr, nfacets, reinterpret_cast<GridRec<NC> *>(b.vrec.ptr),
                                                    (long long)(b.vrec.n / sizeof(GridRec<NC>)), b.vrec_range.ptr,
                                                    b.vrec_range_items, b.vrec_next.ptr);
  g_ctx.launches += 2;
  BZ_CUDA_TRY_RET(cudaGetLastError(), false);
  set_record_args<NC>(out);
  return true;
}

template <int NC, bool WPROJ, bool COMP>
bool launch_class(const GridArgs &base, int k, const Variant &v, int nfacets, const int *count, int *next,
                  cudaStream_t st) {
  GridArgs a = base;
  a.W = g_bs.cls[k].width;
  a.V = v.V;
  a.plane_lo = g_bs.plane_lo.ptr;
  a.conv_w = g_bs.conv_w.ptr;
  a.conv_w_stride = g_bs.conv_w_stride;
  a.segments = g_bs.sorted.ptr;
  a.segment_base = g_bs.class_off.ptr + k;
  a.segment_capacity = (long long)g_bs.segs_cap;
  a.work_count = count;
  a.work_next = next;
  if (v.NT <= 0 || v.grid <= 0) {
    bz_record_error(BZ_ERR_CUDA, "batched: no layout chosen for support class %d", a.W);
    return false;
  }
  auto kern = seg_kernel<NC, WPROJ, COMP>(v.J, v.wide, v.regs);
  if (!open_smem(kern)) {
    bz_record_error(BZ_ERR_CUDA, "batched: cudaFuncSetAttribute failed");
    return false;
  }
  BZ_CUDA_TRY_RET(cudaMemsetAsync(next, 0, sizeof(int), st), false);
  kern<<<v.grid, v.NT, v.smem, st>>>(a, nfacets);
  g_ctx.launches++;
  BZ_CUDA_TRY_RET(cudaGetLastError(), false);
  return true;
}

template <int NC, bool WPROJ, bool COMP>
bool finish_variant(Variant &v) {
  auto kern = seg_kernel<NC, WPROJ, COMP>(v.J, v.wide, v.regs);
  if (!open_smem(kern)) return false;
  int per_sm = 0, dev = 0, sms = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, v.NT, v.smem) != cudaSuccess || per_sm < 1) return false;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  v.grid = per_sm * sms;
  return true;
}

// Autotuner: time every valid layout of a class on a sample of its own work items, gridding into
// scratch grids, and keep the fastest.  Decisions are cached by (width, NC, WPROJ, COMP).
template <int NC, bool WPROJ, bool COMP>
bool tune_class(const GridArgs &base, int k, int nfacets, Variant &out, int host_count) {
  BatchedState &b = g_bs;
  Context &c = g_ctx;
  const int W = b.cls[k].width;
  auto key = std::make_tuple(W, NC, (int)WPROJ, (int)COMP);
  auto it = b.tuned.find(key);
  std::vector<Variant> cands;
  // J = 6 (single precision, four correlations, w-projection): 48 accumulator registers, the
  // column tap shared by 6 rows
  const bool six = BZ_PRECISION_BITS == 32 && NC == 4 && WPROJ;
  for (int J : {8, 6, 4})
    for (bool wide : {true, false})
      for (int regs : reg_caps<NC, WPROJ>(J)) {
        if (J == 6 && !six) continue;
        Variant v;
        if (make_variant<NC, WPROJ>(W, J, wide, regs, v) && finish_variant<NC, WPROJ, COMP>(v)) cands.push_back(v);
      }
  if (cands.empty()) {
    bz_record_error(BZ_ERR_UNSUPPORTED, "batched: no layout for support class %d", W);
    return false;
  }
  if (it != b.tuned.end()) {
    for (auto &v : cands)
      if (v.J == std::get<0>(it->second) && (int)v.wide == std::get<1>(it->second) && v.regs == std::get<2>(it->second)) {
        out = v;
        return true;
      }
  }
  if (cands.size() == 1 || host_count == 0) {
    out = cands[0];
    b.tuned[key] = std::make_tuple(out.J, (int)out.wide, out.regs);
    return true;
  }
  // Each candidate grids a quarter of the class's runs (at least 4096, when there are that many)
  // into the scratch grid (no effect on results): smaller samples leave the persistent grid
  // underfilled and favour the wrong layout.  A short first launch loads the variant's code.
  const int counts2[2] = {std::min(host_count, 64), std::min(host_count, std::max(4096, host_count / 4))};
  BZ_CUDA_TRY_RET(cudaMemcpyAsync(b.sample_count.ptr + 2 * k, counts2, sizeof(counts2), cudaMemcpyHostToDevice, c.stream),
                  false);
  BZ_CUDA_TRY_RET(cudaStreamSynchronize(c.stream), false);
  GridArgs a = base;
  a.grid = c.scratch.ptr;
  a.grid_lo = COMP ? c.scratch.ptr : nullptr;
  a.norm = nullptr;
  BZ_CUDA_TRY_RET(cudaStreamWaitEvent(c.stream, c.ev_copied_vis, 0), false);  // a copy-back may read the scratch grid
  float best = 1e30f;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  for (auto &v : cands) {
    if (!launch_class<NC, WPROJ, COMP>(a, k, v, nfacets, b.sample_count.ptr + 2 * k, b.work_next.ptr + k, c.stream))
      break;
    cudaEventRecord(e0, c.stream);
    launch_class<NC, WPROJ, COMP>(a, k, v, nfacets, b.sample_count.ptr + 2 * k + 1, b.work_next.ptr + k, c.stream);
    cudaEventRecord(e1, c.stream);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) {
      best = ms;
      out = v;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  BZ_CUDA_TRY_RET(cudaMemsetAsync(c.scratch.ptr, 0, sizeof(vis_complex) * c.scratch.n, c.stream), false);
  b.tuned[key] = std::make_tuple(out.J, (int)out.wide, out.regs);
  return bz_error_code() == BZ_OK;
}

template <int NC, bool WPROJ, bool COMP>
bool tune_all(const GridArgs &base, int nfacets, bool sampling, const std::vector<int> &counts) {
  // records for the timing runs only when some class has work and no layout decided yet (a
  // decided class takes its layout without launching)
  bool timing = false;
  for (int k = 0; k < g_bs.ncls; ++k)
    if (counts[k] > 0 && !g_bs.tuned.count(std::make_tuple(g_bs.cls[k].width, NC, (int)WPROJ, (int)COMP))) timing = true;
  GridArgs tb = base, rb = base;
  tb.norm = nullptr;  // tuning launches leave the normalisation alone
  if (timing && !launch_records<NC, WPROJ>(tb, nfacets, g_ctx.stream, rb)) return false;
  for (int k = 0; k < g_bs.ncls; ++k) {
    Variant &v = sampling ? g_bs.cls[k].sf : g_bs.cls[k].vis;
    if (!tune_class<NC, WPROJ, COMP>(rb, k, nfacets, v, counts[k])) return false;
  }
  return true;
}

template <int NC, bool WPROJ, bool COMP>
bool launch_all(const GridArgs &base_in, int nfacets, bool sampling, cudaStream_t st, const std::vector<int> *counts) {
  BatchedState &b = g_bs;
  GridArgs base;
  {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (b.profile) {
      cudaEventCreate(&e0);
      cudaEventCreate(&e1);
      cudaEventRecord(e0, st);
    }
    if (!launch_records<NC, WPROJ>(base_in, nfacets, st, base)) return false;
    if (b.profile) {
      cudaEventRecord(e1, st);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      if (base.records) b.records.push_back({0, NC, 0, 0, 0, ms});  // width 0: the record kernel
    }
  }
  for (int k = 0; k < b.ncls; ++k) {
    const Variant &v = sampling ? b.cls[k].sf : b.cls[k].vis;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (b.profile) {
      cudaEventCreate(&e0);
      cudaEventCreate(&e1);
      cudaEventRecord(e0, st);
    }
    const bool ok = launch_class<NC, WPROJ, COMP>(base, k, v, nfacets, b.class_count.ptr + k,
                                                  b.work_next.ptr + (sampling ? kMaxClasses : 0) + k, st);
    if (b.profile) {
      cudaEventRecord(e1, st);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      b.records.push_back({b.cls[k].width, NC, v.J, (int)v.wide | (v.regs << 1), counts ? (*counts)[k] * nfacets : 0, ms});
    }
    if (!ok) return false;
  }
  return true;
}

// vis = false launches (and tunes) only the sampling function's classes; va then only feeds the
// schedule.
template <bool WPROJ, bool COMP>
bool dispatch(const GridArgs &va, const GridArgs *sa, int nfacets, bool tune, const std::vector<int> &counts,
              cudaStream_t st, bool vis) {
  if (tune) {
    if (vis && !tune_all<4, WPROJ, COMP>(va, nfacets, false, counts)) return false;
    if (sa && !tune_all<1, WPROJ, COMP>(*sa, 1, true, counts)) return false;
    return true;
  }
  if (vis && !launch_all<4, WPROJ, COMP>(va, nfacets, false, st, &counts)) return false;
  if (sa && !launch_all<1, WPROJ, COMP>(*sa, 1, true, st, &counts)) return false;
  return true;
}

bool run_dispatch(const GridArgs &va, const GridArgs *sa, bool wproj, bool comp, bool tune, const std::vector<int> &counts,
                  cudaStream_t st, int nfacets, bool vis) {
  const int F = nfacets > 0 ? nfacets : (int)g_ctx.F;
#if defined(BULLSEYE_SINGLE)
  if (comp)
    return wproj ? dispatch<true, true>(va, sa, F, tune, counts, st, vis)
                 : dispatch<false, true>(va, sa, F, tune, counts, st, vis);
#else
  (void)comp;
#endif
  return wproj ? dispatch<true, false>(va, sa, F, tune, counts, st, vis)
               : dispatch<false, false>(va, sa, F, tune, counts, st, vis);
}

// The schedule-building kernels (everything before the per-class launches), for the tracks of
// va.starts / va.nslots, whose rows lie in [r0, r0 + n) (n < 0: all rows).
bool enqueue_schedule(const GridArgs &va, cudaStream_t st, long long r0 = 0, long long n = -1) {
  Context &c = g_ctx;
  BatchedState &b = g_bs;
  const long long R = va.nrows;
  if (n < 0) n = R - r0;
  const int tracks = va.nslots * va.nchan;
  BZ_CUDA_TRY_RET(cudaMemsetAsync(b.class_count.ptr, 0, sizeof(int) * kMaxClasses, st), false);
  classify_kernel<<<1024, 256, 0, st>>>(va.uvw, va.spw, c.wavelengths.ptr, va.nchan, va.nspw, R, va.wmax, va.P,
                                        b.plane_class.ptr, b.row_class.ptr, r0, n);
  seg_count_kernel<<<(tracks + 127) / 128, 128, 0, st>>>(va.starts, va.nslots, va.seg, R, va.nchan, b.row_class.ptr,
                                                         b.nseg.ptr);
  scan_kernel<<<1, 1024, 0, st>>>(b.nseg.ptr, b.seg_off.ptr, tracks, b.seg_total.ptr);
  seg_write_kernel<<<(tracks + 127) / 128, 128, 0, st>>>(va.starts, va.nslots, va.seg, R, va.nchan, b.row_class.ptr,
                                                         b.seg_off.ptr, b.segs.ptr, b.class_count.ptr, b.ncls, va.error);
  class_offsets_kernel<<<1, 1, 0, st>>>(b.class_count.ptr, b.class_off.ptr, b.class_cursor.ptr, b.ncls);
  bucket_kernel<<<1024, 256, 0, st>>>(b.segs.ptr, b.seg_total.ptr, b.sorted.ptr, b.class_cursor.ptr, b.class_off.ptr);
  c.launches += 6;
  BZ_CUDA_TRY_RET(cudaGetLastError(), false);
  return true;
}

}  // namespace

void bz_release_batched() {
  BatchedState &b = g_bs;
  b.drop_graphs();
  b.plane_class.release(); b.plane_lo.release(); b.row_class.release(); b.nseg.release(); b.seg_off.release();
  b.seg_total.release(); b.class_count.release(); b.class_off.release(); b.class_cursor.release();
  b.work_next.release(); b.sample_count.release(); b.segs.release(); b.sorted.release(); b.facet_table.release();
  b.conv_w.release();
  b.conv_w_stride = 0;
  b.vrec.release(); b.vrec_off.release(); b.vrec_range.release(); b.cls_width.release(); b.vrec_next.release();
  b.vrec_range_items = 0;
  b.rows_cap = b.tracks_cap = b.segs_cap = 0;
  b.planned = false;
  b.ncls = 0;
}

// See include/bullseye_gb300.h.
extern "C" void bullseye_set_batched_profiling(int on) { g_bs.profile = on != 0; }

// See include/bullseye_gb300.h.
extern "C" void bullseye_set_grid_groups(int groups) { g_ctx.grid_groups = groups < 1 ? 1 : groups; }

// See include/bullseye_gb300.h.
extern "C" void bullseye_set_visibility_records(int on) {
  if (g_bs.vrec_on != (on != 0)) g_bs.drop_graphs();
  g_bs.vrec_on = on != 0;
}

// See include/bullseye_gb300.h.
extern "C" void bullseye_set_record_budget(size_t bytes) { g_bs.vrec_budget = bytes; }

namespace {
// Self-test of the bounded tap-barrier wait: the barrier expects two arrivals and gets one, so
// every thread's wait must run out (about 0.2 s) and record DEV_ERR_WAIT_TIMEOUT.  No copy is in
// flight, so nothing is left pending when the CTA exits.
__global__ void bounded_wait_selftest_kernel(int *err) {
  __shared__ __align__(8) unsigned long long bar;
  if (threadIdx.x == 0) bar_init(&bar, 2);
  __syncthreads();
  if (threadIdx.x == 0) bar_arrive(&bar);
  if (!bar_wait(&bar, 0) && threadIdx.x == 0) atomicOr(err, DEV_ERR_WAIT_TIMEOUT);
}
}  // namespace

// See include/bullseye_gb300.h.
extern "C" int bullseye_selftest_bounded_wait(void) {
  int *d = nullptr, h = 0;
  if (cudaMalloc(&d, sizeof(int)) != cudaSuccess) return -1;
  bool ok = cudaMemset(d, 0, sizeof(int)) == cudaSuccess;
  if (ok) {
    bounded_wait_selftest_kernel<<<1, 32>>>(d);
    ok = cudaGetLastError() == cudaSuccess && cudaDeviceSynchronize() == cudaSuccess &&
         cudaMemcpy(&h, d, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess;
  }
  cudaFree(d);
  return ok ? h : -1;
}

// See include/bullseye_gb300.h.
extern "C" int bullseye_batched_plane_classes(int *width, int max) {
  const auto &w = g_bs.plane_width;
  for (int i = 0; i < (int)w.size() && i < max; ++i) width[i] = w[i];
  return g_bs.planned ? (int)w.size() : 0;
}

// See include/bullseye_gb300.h.
extern "C" int bullseye_batched_profile(int *width, int *nc, int *J, int *wide, int *items, float *ms, int max) {
  const auto &r = g_bs.records;
  const int n = (int)std::min<size_t>(r.size(), max > 0 ? (size_t)max : 0);
  for (int i = 0; i < n; ++i) {
    if (width) width[i] = r[i].width;
    if (nc) nc[i] = r[i].nc;
    if (J) J[i] = r[i].J;
    if (wide) wide[i] = r[i].wide;
    if (items) items[i] = r[i].items;
    if (ms) ms[i] = r[i].ms;
  }
  return (int)r.size();
}

namespace {

// Runs one batched call: builds the schedule on the device, on first use tunes every support class
// (tuning launches use `ta` over `tune_facets` facets and grid into the library's scratch grid),
// then replays the call as a CUDA graph keyed on the launch arguments; eager with per-class events
// in profiling mode.  vis = false grids only the sampling function (sa), with va feeding the
// schedule.
int run_batched(const GridArgs &va, const GridArgs *sa, int nfacets, const GridArgs &ta, int tune_facets, bool wproj,
                bool comp, const char *name, bool vis = true) {
  Context &c = g_ctx;
  BatchedState &b = g_bs;
  const bool sf = sa != nullptr;
  // graph key: everything the captured launches read by value
  std::vector<unsigned char> key(sizeof(GridArgs) * 2 + 16);
  std::memcpy(key.data(), &va, sizeof(GridArgs));
  if (sf) std::memcpy(key.data() + sizeof(GridArgs), sa, sizeof(GridArgs));
  key[sizeof(GridArgs) * 2] = (unsigned char)sf;
  key[sizeof(GridArgs) * 2 + 1] = (unsigned char)comp;
  key[sizeof(GridArgs) * 2 + 2] = (unsigned char)vis;
  std::memcpy(key.data() + sizeof(GridArgs) * 2 + 4, &nfacets, sizeof(int));

  // the eager schedule's class counts; the record buffers are sized from them before any tuning
  // or capture
  auto schedule_counts = [&](std::vector<int> &counts) -> bool {
    if (!enqueue_schedule(va, c.stream)) return false;
    BZ_CUDA_TRY_RET(cudaMemcpyAsync(counts.data(), b.class_count.ptr, sizeof(int) * kMaxClasses, cudaMemcpyDeviceToHost,
                                    c.stream), false);
    BZ_CUDA_TRY_RET(cudaStreamSynchronize(c.stream), false);
    long long nseg = 0;
    for (int k = 0; k < b.ncls; ++k) nseg += counts[k];
    return ensure_records(std::max(nfacets, tune_facets), va.nrows, va.nchan, nseg);
  };
  if (b.profile) {
    std::vector<int> counts(kMaxClasses, 0);
    if (!schedule_counts(counts)) return bz_error_code() ? bz_error_code() : BZ_ERR_CUDA;
    if (!run_dispatch(ta, sa, wproj, comp, true, counts, c.stream, tune_facets, vis)) return bz_error_code();
    b.records.clear();
    if (!run_dispatch(va, sa, wproj, comp, false, counts, c.stream, nfacets, vis)) return bz_error_code();
    return BZ_OK;
  }
  BatchedState::GraphSlot *slot = nullptr;
  for (auto &g : b.graphs)
    if (g.exec && g.key == key) slot = &g;
  if (!slot) {
    // first run of this configuration: build the schedule eagerly, tune each class, then capture
    // into the least recently used slot
    slot = &b.graphs[0];
    for (auto &g : b.graphs)
      if (g.used < slot->used) slot = &g;
    std::vector<int> counts(kMaxClasses, 0);
    if (!schedule_counts(counts)) return bz_error_code() ? bz_error_code() : BZ_ERR_CUDA;
    if (!run_dispatch(ta, sa, wproj, comp, true, counts, c.stream, tune_facets, vis)) return bz_error_code();
    if (slot->exec) cudaGraphExecDestroy(slot->exec);
    slot->exec = nullptr;
    slot->key.clear();
    cudaGraph_t graph;
    BZ_CUDA_TRY_RET(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal), BZ_ERR_CUDA);
    const long long launches0 = c.launches;
    bool ok = enqueue_schedule(va, c.stream) && run_dispatch(va, sa, wproj, comp, false, counts, c.stream, nfacets, vis);
    cudaError_t ce = cudaStreamEndCapture(c.stream, &graph);
    if (!ok || ce != cudaSuccess) {
      bz_record_error(BZ_ERR_CUDA, "%s: graph capture failed (%s)", name, cudaGetErrorString(ce));
      return BZ_ERR_CUDA;
    }
    c.launches = launches0;  // counted again when the graph is launched
    ce = cudaGraphInstantiate(&slot->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) {
      slot->exec = nullptr;
      bz_record_error(BZ_ERR_CUDA, "%s: graph instantiation failed (%s)", name, cudaGetErrorString(ce));
      return BZ_ERR_CUDA;
    }
    slot->key = key;
  }
  slot->used = ++b.graph_clock;
  bz_trace_mark("schedule_tune_capture");
  BZ_CUDA_TRY_RET(cudaGraphLaunch(slot->exec, c.stream), BZ_ERR_CUDA);
  const int rec = b.vrec_on && b.vrec.ptr && b.conv_w.ptr ? 2 : 0;  // record offsets + record kernel per build
  c.launches += 6 + (long long)(b.ncls + rec) * ((vis ? 1 : 0) + (sf ? 1 : 0));
  return BZ_OK;
}

bool call_mode(int call, int &mode, bool &faceting, const char *name) {
  switch (call) {
    case 0: mode = CORR_QUAD_JONES; faceting = true; return true;  // facet_4_cor_corrections
    case 1: mode = CORR_QUAD; faceting = true; return true;        // facet_4_cor
    case 2: mode = CORR_QUAD; faceting = false; return true;       // grid_4_cor
    default:
      bz_record_error(BZ_ERR_INVALID_ARGUMENT, "%s: unknown call %d", name, call);
      return false;
  }
}

// Whether every support class has a tuned layout for these visibility launches.
bool classes_tuned(int nc, bool wproj, bool comp) {
  for (int k = 0; k < g_bs.ncls; ++k)
    if (!g_bs.tuned.count(std::make_tuple(g_bs.cls[k].width, nc, (int)wproj, (int)comp))) return false;
  return true;
}

// Host inputs: the visibilities are streamed in row chunks (rows.cu): the upload of chunk k + 1
// overlaps the device sort of chunk k.  With one gridding group (the default) every row is gridded
// after the last chunk is sorted, by the same graph-replayed launches as device-resident rows;
// with G groups, the chunks of each group are gridded (eager launches) while the next group's rows
// upload.  More groups hide more of the upload but split every class launch, and each split adds
// a launch tail.
bool stream_visibilities(gridding_parameters &p, const GridArgs &va, int nfacets, bool jones, const char *name) {
  Context &c = g_ctx;
  const bool wproj = va.P > 1, comp = va.grid_lo != nullptr;
  RowsPlan plan;
  if (!bz_plan_rows(p, plan)) return false;
  if (!ensure_capacity(p.row_count, (size_t)plan.chunks * plan.slots * c.nchan)) return false;
  const int K = plan.chunks, G = std::max(1, std::min(c.grid_groups, K));
  if (G == 1) {
    if (!bz_stream_rows(p, true, jones, plan, nullptr)) {
      if (!bz_error_code()) bz_record_error(BZ_ERR_CUDA, "%s: row upload failed", name);
      return false;
    }
    bz_trace_mark("vis.rows_sorted");
    return run_batched(va, nullptr, nfacets, va, nfacets, wproj, comp, name, true) == BZ_OK;
  }
  std::vector<int> counts(kMaxClasses, 0);
  if (!ensure_records(nfacets, (long long)p.row_count, (int)c.nchan, 0)) return false;
  int k0 = 0;
  long long g_r0 = 0;
  auto chunk = [&](int k, long long r0, long long r1) -> bool {
    if (k == k0) g_r0 = r0;
    if (k + 1 < K && (long long)(k + 1) * G / K == (long long)k * G / K) return true;  // group not complete
    GridArgs vk = va;
    vk.starts = c.track_starts.ptr + (size_t)k0 * plan.slots;
    vk.nslots = (k - k0 + 1) * (int)plan.slots;
    if (!enqueue_schedule(vk, c.stream, g_r0, r1 - g_r0)) return false;
    if (k0 == 0) {
      // every call sets its classes' layouts up for this build (NC, w-projection, compensation) from
      // the tuned decisions; classes without a decision yet are timed on this group's runs
      if (!classes_tuned(4, wproj, comp)) {
        BZ_CUDA_TRY_RET(cudaMemcpyAsync(counts.data(), g_bs.class_count.ptr, sizeof(int) * kMaxClasses,
                                        cudaMemcpyDeviceToHost, c.stream), false);
        BZ_CUDA_TRY_RET(cudaStreamSynchronize(c.stream), false);
      }
      if (!run_dispatch(vk, nullptr, wproj, comp, true, counts, c.stream, nfacets, true)) return false;
    }
    const bool ok = run_dispatch(vk, nullptr, wproj, comp, false, counts, c.stream, nfacets, true);
    bz_trace_mark("vis.group_grid");
    k0 = k + 1;
    return ok;
  };
  if (!bz_stream_rows(p, true, jones, plan, chunk)) {
    if (!bz_error_code()) bz_record_error(BZ_ERR_CUDA, "%s: streamed gridding failed", name);
    return false;
  }
  return true;
}

}  // namespace

// The batched gridder behind the reference's 4-correlation and sampling-function exports (one
// kind of grid per call; the two graph slots keep both captured).
bool bz_grid_batched_call(gridding_parameters &p, int mode, bool faceting, const char *name) {
  Context &c = g_ctx;
  BatchedState &b = g_bs;
  const bool sampling = mode == CORR_SAMPLING;
  GridArgs a;
  int nslots = 0;
  // host-input visibilities are streamed (and gridded chunk by chunk) below, not uploaded here
  const bool stream = !c.device_inputs && !sampling;
  if (!bz_prepare_grid_args(p, sampling ? 1 : 4, mode, faceting, a, nslots, name, !stream)) return false;
  bz_trace_mark(sampling ? "sf.upload_prepare" : "vis.upload_prepare");
  if (p.row_count == 0) return true;
  if (!b.planned && !plan_classes()) {
    if (!bz_error_code()) bz_record_error(BZ_ERR_CUDA, "%s: support-class planning failed", name);
    return false;
  }
  const bool wproj = p.wplanes > 1, comp = a.grid_lo != nullptr;
  if (stream) {
    const bool ok = stream_visibilities(p, a, (int)c.F, mode == CORR_QUAD_JONES, name);
    bz_trace_mark("vis.grid");
    return ok;
  }
  if (!ensure_capacity(p.row_count, (size_t)nslots * c.nchan)) return false;
  const int rc = sampling ? run_batched(a, &a, 1, a, 1, wproj, comp, name, false)
                          : run_batched(a, nullptr, (int)c.F, a, (int)c.F, wproj, comp, name, true);
  bz_trace_mark(sampling ? "sf.grid" : "vis.grid");
  return rc == BZ_OK;
}

// See include/bullseye_gb300.h.
extern "C" int bullseye_grid_batched(gridding_parameters *pp, int call, int with_sampling) {
  if (!bz_check_ready("bullseye_grid_batched")) return bz_error_code() ? bz_error_code() : BZ_ERR_NOT_INITIALISED;
  gridding_parameters &p = *pp;
  Context &c = g_ctx;
  BatchedState &b = g_bs;
  int mode;
  bool faceting;
  if (!call_mode(call, mode, faceting, "bullseye_grid_batched")) return BZ_ERR_INVALID_ARGUMENT;
  if (c.C != 4) {
    bz_record_error(BZ_ERR_UNSUPPORTED, "bullseye_grid_batched grids 4 correlations");
    return BZ_ERR_UNSUPPORTED;
  }
  const bool sf = with_sampling && c.want_sf;
  bz_timer_start();
  GridArgs va, sa;
  int nslots = 0, nslots_sf = 0;
  const bool stream = !c.device_inputs;
  if (!bz_prepare_grid_args(p, 4, mode, faceting, va, nslots, "bullseye_grid_batched", !stream)) return bz_error_code();
  if (p.row_count == 0) {
    bz_timer_stop();
    return BZ_OK;
  }
  if (!b.planned && !plan_classes()) return bz_error_code() ? bz_error_code() : BZ_ERR_CUDA;
  if (stream) {
    // host inputs: the visibilities gridded chunk by chunk as their rows arrive, then the sampling
    // function over the rows now on the device
    if (!stream_visibilities(p, va, (int)c.F, mode == CORR_QUAD_JONES, "bullseye_grid_batched")) return bz_error_code();
    if (sf) {
      if (!bz_prepare_grid_args(p, 1, CORR_SAMPLING, faceting, sa, nslots_sf, "bullseye_grid_batched")) return bz_error_code();
      if (!ensure_capacity(p.row_count, (size_t)nslots_sf * c.nchan)) return bz_error_code();
      const int rc = run_batched(sa, &sa, 1, sa, 1, p.wplanes > 1, sa.grid_lo != nullptr, "bullseye_grid_batched", false);
      if (rc != BZ_OK) return rc;
    }
  } else {
    // the sampling function reads the rows the visibility prepare set up
    if (sf && !bz_prepare_grid_args(p, 1, CORR_SAMPLING, faceting, sa, nslots_sf, "bullseye_grid_batched", false))
      return bz_error_code();
    if (!ensure_capacity(p.row_count, (size_t)nslots * c.nchan)) return bz_error_code();
    const int rc = run_batched(va, sf ? &sa : nullptr, (int)c.F, va, (int)c.F, p.wplanes > 1, va.grid_lo != nullptr,
                               "bullseye_grid_batched");
    if (rc != BZ_OK) return rc;
  }
  if (p.is_final_data_chunk) {
    bz_copy_back_grids(p, false);
    if (sf) bz_copy_back_grids(p, true);
  }
  bz_timer_stop();
  return bz_error_code();
}

// See include/bullseye_gb300.h.
extern "C" int bullseye_grid_batched_facets(gridding_parameters *pp, const bullseye_facet *facets, int nfacets,
                                            const unsigned char *row_mask, void *grids, void *grid_lo, double *norms,
                                            int call) {
  const char *name = "bullseye_grid_batched_facets";
  if (!bz_check_ready(name)) return bz_error_code() ? bz_error_code() : BZ_ERR_NOT_INITIALISED;
  gridding_parameters &p = *pp;
  Context &c = g_ctx;
  BatchedState &b = g_bs;
  int mode;
  bool faceting;
  if (!call_mode(call, mode, faceting, name)) return BZ_ERR_INVALID_ARGUMENT;
  if (!facets || nfacets <= 0 || !grids || !norms) {
    bz_record_error(BZ_ERR_INVALID_ARGUMENT, "%s: facets, grids and norms are required", name);
    return BZ_ERR_INVALID_ARGUMENT;
  }
  if (c.C != 4) {
    bz_record_error(BZ_ERR_UNSUPPORTED, "%s grids 4 correlations", name);
    return BZ_ERR_UNSUPPORTED;
  }
  if (call == 0 && (size_t)nfacets != c.F) {
    bz_record_error(BZ_ERR_INVALID_ARGUMENT, "%s: Jones terms are laid out for %zu facets, not %d", name, c.F, nfacets);
    return BZ_ERR_INVALID_ARGUMENT;
  }
  if (row_mask && !c.device_inputs) {
    // host rows are reordered by baseline on the device; a row mask is indexed in the caller's order
    bz_record_error(BZ_ERR_UNSUPPORTED, "%s: a row mask needs device-resident inputs (bullseye_set_device_inputs)", name);
    return BZ_ERR_UNSUPPORTED;
  }
  const long long s = (long long)p.conv_support;
  for (int f = 0; f < nfacets; ++f) {
    const bullseye_facet &d = facets[f];
    if (d.nx < (size_t)(2 * s + 4) || d.ny < (size_t)(2 * s + 4) || d.nx > (1u << 20) || d.ny > (1u << 20)) {
      bz_record_error(BZ_ERR_INVALID_ARGUMENT, "%s: facet %d has a %zu x %zu grid", name, f, d.nx, d.ny);
      return BZ_ERR_INVALID_ARGUMENT;
    }
  }
  bz_timer_start();
  GridArgs va;
  int nslots = 0;
  if (!bz_prepare_grid_args(p, 4, mode, faceting, va, nslots, name)) return bz_error_code();
  if (p.row_count == 0) {
    bz_timer_stop();
    return BZ_OK;
  }
  // tuning runs on facet 0 of the library's own layout, into its scratch grid
  const GridArgs ta = va;
  std::vector<FacetXform> fx(nfacets);
  const double ra0 = (double)p.phase_centre_ra, dec0 = (double)p.phase_centre_dec;
  for (int f = 0; f < nfacets; ++f) {
    const bullseye_facet &d = facets[f];
    fx[f] = bz_facet_xform(ra0, dec0, faceting ? d.ra : ra0, faceting ? d.dec : dec0, faceting, faceting);
    fx[f].nx = (int)d.nx;
    fx[f].ny = (int)d.ny;
    fx[f].u_scale = (double)d.nx * d.cell_x * (double)kArcsecToRad;
    fx[f].v_scale = -((double)d.ny * d.cell_y * (double)kArcsecToRad);
    fx[f].gcx = (double)((long long)(d.nx / 2) - s);
    fx[f].gcy = (double)((long long)(d.ny / 2) - s);
    fx[f].grid_base = (long long)d.grid_offset;
  }
  if (b.facet_table.n < (size_t)nfacets && !b.facet_table.alloc(nfacets)) return bz_error_code();
  BZ_CUDA_TRY_RET(cudaMemcpyAsync(b.facet_table.ptr, fx.data(), sizeof(FacetXform) * nfacets, cudaMemcpyHostToDevice,
                                  c.stream), BZ_ERR_CUDA);
  va.facets = b.facet_table.ptr;
  va.nfacets_total = nfacets;
  va.facet_base = 0;
  va.jones_inv_t = nullptr;  // its facet count is the library's, not this call's
  va.facet_row_mask = row_mask;
  va.grid = static_cast<vis_complex *>(grids);
  va.grid_lo = nullptr;
#if defined(BULLSEYE_SINGLE)
  va.grid_lo = static_cast<vis_complex *>(grid_lo);
#else
  (void)grid_lo;
#endif
  va.norm = norms;
  if (!b.planned && !plan_classes()) return bz_error_code() ? bz_error_code() : BZ_ERR_CUDA;
  if (!ensure_capacity(p.row_count, (size_t)nslots * c.nchan)) return bz_error_code();
  const int rc = run_batched(va, nullptr, nfacets, ta, 1, p.wplanes > 1, va.grid_lo != nullptr, name);
  if (rc != BZ_OK) return rc;
  bz_timer_stop();
  return bz_error_code();
}

// ---------------------------------------------------------------- support-aware workspace form
// The batched gridder without library state, for the allocation-free workspace entry: the
// per-plane windows, the support-window table and the run schedule are built on the device in the
// caller's workspace from the call's own (device) tables, and every candidate class width gets
// one persistent launch (a class no plane uses finds no work items).  The layout of a class is
// fixed, J = 4 (J = 8 where the J = 4 layout needs more than 512 threads), so that concurrent
// calls with their own workspaces read no shared state.

namespace {

struct ClassList {
  int n;
  int w[kMaxClasses];
};

// One warp per w plane: the plane's nonzero window, its class and window start (the same rule as
// plan_classes, evaluated on the device).
__global__ void plane_window_kernel(const void *conv, int P, int K, int W, int os, int wproj, ClassList cl,
                                    int *plane_class, int *plane_lo, int *plane_w) {
  const int lane = threadIdx.x & 31;
  const int pl = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (pl >= P) return;  // whole warps
  int lo = 0x7fffffff, hi = -1;
  for (int i = lane; i < K; i += 32) {
    bool nz;
    if (wproj) {
      const vis_complex t = ((const vis_complex *)conv)[(long long)pl * K + i];
      nz = t.re != (vis_real)0 || t.im != (vis_real)0;
    } else {
      nz = ((const vis_real *)conv)[i] != (vis_real)0;
    }
    if (nz) {
      lo = min(lo, i);
      hi = max(hi, i);
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, off));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, off));
  }
  if (lane != 0) return;
  const int fu_min = wproj ? (int)floor(0.5 * os - 1e-6) : 0;
  const int fu_max = wproj ? (int)floor(1.5 * os + 1e-6) : os;
  int slo = 0, shi = 0;
  if (hi >= 0) {
    slo = max(0, (int)ceil((double)(lo - fu_max) / os));
    shi = min(W - 1, (int)floor((double)(hi - fu_min) / os));
    if (shi < slo) shi = slo;
  }
  const int width = shi - slo + 1;
  int k = cl.n - 1;
  for (int i = 0; i < cl.n; ++i)
    if (cl.w[i] >= width) {
      k = i;
      break;
    }
  plane_class[pl] = k;
  plane_w[pl] = cl.w[k];
  plane_lo[pl] = min(slo, W - cl.w[k]);
}

// Support-window table [P][tap_f][L] (real or complex like conv), as plan_classes builds it.
__global__ void window_table_kernel(const void *conv, int P, int K, int tap_f, int os, int wproj,
                                    const int *__restrict__ plane_lo, const int *__restrict__ plane_w, int L,
                                    vis_real *__restrict__ out) {
  const long long n = (long long)P * tap_f * L;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(e % L);
    const long long pf = e / L;
    const int f = (int)(pf % tap_f), p = (int)(pf / tap_f);
    const int pw = plane_w[p];
    const int jj = j < pw ? j : (j < pw + 7 ? j - pw : -1);
    vis_real re = 0, im = 0;
    if (jj >= 0) {
      const long long i = f + (long long)(plane_lo[p] + jj) * os;
      if (i < K) {
        if (wproj) {
          const vis_complex t = ((const vis_complex *)conv)[(long long)p * K + i];
          re = t.re;
          im = t.im;
        } else {
          re = ((const vis_real *)conv)[i];
        }
      }
    }
    if (wproj) {
      out[2 * e] = re;
      out[2 * e + 1] = im;
    } else {
      out[e] = re;
    }
  }
}

// Workspace layout of the support-aware form (every piece 256-byte aligned).
struct SupportWs {
  size_t plane_class, plane_lo, plane_w, table, row_class, nseg, seg_off, seg_total, segs, sorted, class_count,
      class_off, class_cursor, work_next, bytes;
  int L, tap_f;
  long long maxseg;
};

SupportWs support_ws_layout(long long R, int nchan, int nslots, int P, int os, int W, bool wproj) {
  SupportWs l;
  const size_t ncomp = wproj ? 2 : 1;
  const int E = (int)(16 / (ncomp * sizeof(vis_real)));
  l.L = (W + 7 + E - 1) / E * E;
  l.tap_f = 2 * os + 1;
  l.maxseg = std::max<long long>(1, R * nchan);
  const long long tracks = std::max<long long>(1, (long long)nslots * nchan);
  size_t off = 0;
  auto take = [&](size_t n) {
    const size_t at = off;
    off += (n + 255) / 256 * 256;
    return at;
  };
  l.plane_class = take(sizeof(int) * P);
  l.plane_lo = take(sizeof(int) * P);
  l.plane_w = take(sizeof(int) * P);
  l.table = take(sizeof(vis_real) * ncomp * (size_t)P * l.tap_f * l.L);
  l.row_class = take((size_t)std::max<long long>(1, R * nchan));
  l.nseg = take(sizeof(int) * tracks);
  l.seg_off = take(sizeof(int) * tracks);
  l.seg_total = take(sizeof(int));
  l.segs = take(sizeof(int4) * l.maxseg);
  l.sorted = take(sizeof(int4) * l.maxseg);
  l.class_count = take(sizeof(int) * kMaxClasses);
  l.class_off = take(sizeof(int) * kMaxClasses);
  l.class_cursor = take(sizeof(int) * kMaxClasses);
  l.work_next = take(sizeof(int) * kMaxClasses);
  l.bytes = off;
  return l;
}

// Thread layout of one support class of the workspace form: J = 4 (J = 8 where the J = 4 layout
// needs more than 512 threads), fixed so that concurrent calls share no tuning state.
template <bool WPROJ, bool COMP>
bool support_aware_variant(int W, Variant &v) {
  for (int J : {4, 8})
    if (make_variant<4, WPROJ>(W, J, false, kSegRegs<4>, v) && finish_variant<4, WPROJ, COMP>(v)) return true;
  return make_variant<4, WPROJ>(W, 8, true, kSegRegs<8>, v) && finish_variant<4, WPROJ, COMP>(v);
}

template <bool WPROJ, bool COMP>
bool support_aware_layouts(const ClassList &cl, Variant *vs) {
  for (int k = 0; k < cl.n; ++k)
    if (!support_aware_variant<WPROJ, COMP>(cl.w[k], vs[k])) {
      bz_record_error(BZ_ERR_UNSUPPORTED, "support-aware gridding: no layout for class width %d", cl.w[k]);
      return false;
    }
  return true;
}

bool support_aware_layouts(const ClassList &cl, bool wproj, bool comp, Variant *vs) {
#if defined(BULLSEYE_SINGLE)
  if (comp) return wproj ? support_aware_layouts<true, true>(cl, vs) : support_aware_layouts<false, true>(cl, vs);
#else
  (void)comp;
#endif
  return wproj ? support_aware_layouts<true, false>(cl, vs) : support_aware_layouts<false, false>(cl, vs);
}

template <bool WPROJ, bool COMP>
bool support_aware_launches(const GridArgs &a, const ClassList &cl, const Variant *vs, int nfacets, int *class_count,
                            int *class_off, int *work_next, cudaStream_t st) {
  for (int k = 0; k < cl.n; ++k) {
    const Variant &v = vs[k];
    GridArgs ak = a;
    ak.W = cl.w[k];
    ak.V = v.V;
    ak.segment_base = class_off + k;
    ak.work_count = class_count + k;
    ak.work_next = work_next + k;
    auto kern = seg_kernel<4, WPROJ, COMP>(v.J, v.wide, v.regs);
    if (cudaMemsetAsync(work_next + k, 0, sizeof(int), st) != cudaSuccess) return false;
    kern<<<v.grid, v.NT, v.smem, st>>>(ak, nfacets);
    if (cudaGetLastError() != cudaSuccess) return false;
  }
  return true;
}

ClassList candidate_classes(int W) {
  const std::vector<int> cand = class_candidates(W);
  ClassList cl;
  cl.n = (int)cand.size();
  for (int i = 0; i < cl.n; ++i) cl.w[i] = cand[i];
  return cl;
}

}  // namespace

size_t bz_support_aware_ws_bytes(long long rows, int nchan, int nslots, int P, int os, int W, bool wproj) {
  return support_ws_layout(rows, nchan, nslots, P, os, W, wproj).bytes;
}

bool bz_support_aware_check(const GridArgs &a, size_t bytes) {
  const bool wproj = a.P > 1;
  const SupportWs l = support_ws_layout(a.nrows, a.nchan, a.nslots, a.P, a.os, a.W, wproj);
  if (bytes < l.bytes) {
    bz_record_error(BZ_ERR_INVALID_ARGUMENT, "support-aware gridding: workspace of %zu bytes, need %zu", bytes, l.bytes);
    return false;
  }
  const ClassList cl = candidate_classes(a.W);
  Variant vs[kMaxClasses];
  return support_aware_layouts(cl, wproj, a.grid_lo != nullptr, vs);
}

bool bz_grid_support_aware(const GridArgs &a_in, int nfacets, unsigned char *ws, size_t bytes, cudaStream_t st) {
  const bool wproj = a_in.P > 1;
  const int W = a_in.W;
  const SupportWs l = support_ws_layout(a_in.nrows, a_in.nchan, a_in.nslots, a_in.P, a_in.os, W, wproj);
  if (bytes < l.bytes) {
    bz_record_error(BZ_ERR_INVALID_ARGUMENT, "support-aware gridding: workspace of %zu bytes, need %zu", bytes, l.bytes);
    return false;
  }
  const ClassList cl = candidate_classes(W);
  Variant vs[kMaxClasses];
  const bool comp = a_in.grid_lo != nullptr;
  if (!support_aware_layouts(cl, wproj, comp, vs)) return false;
  int *plane_class = reinterpret_cast<int *>(ws + l.plane_class);
  int *plane_lo = reinterpret_cast<int *>(ws + l.plane_lo);
  int *plane_w = reinterpret_cast<int *>(ws + l.plane_w);
  vis_real *table = reinterpret_cast<vis_real *>(ws + l.table);
  unsigned char *row_class = ws + l.row_class;
  int *nseg = reinterpret_cast<int *>(ws + l.nseg);
  int *seg_off = reinterpret_cast<int *>(ws + l.seg_off);
  int *seg_total = reinterpret_cast<int *>(ws + l.seg_total);
  int4 *segs = reinterpret_cast<int4 *>(ws + l.segs);
  int4 *sorted = reinterpret_cast<int4 *>(ws + l.sorted);
  int *class_count = reinterpret_cast<int *>(ws + l.class_count);
  int *class_off = reinterpret_cast<int *>(ws + l.class_off);
  int *class_cursor = reinterpret_cast<int *>(ws + l.class_cursor);
  int *work_next = reinterpret_cast<int *>(ws + l.work_next);
  const int P = a_in.P, K = a_in.K;
  const long long R = a_in.nrows;
  const int tracks = a_in.nslots * a_in.nchan;
  if (cudaMemsetAsync(class_count, 0, sizeof(int) * kMaxClasses, st) != cudaSuccess) return false;
  plane_window_kernel<<<(unsigned)((P * 32 + 255) / 256), 256, 0, st>>>(a_in.conv, P, K, W, a_in.os, wproj ? 1 : 0, cl,
                                                                        plane_class, plane_lo, plane_w);
  window_table_kernel<<<256, 256, 0, st>>>(a_in.conv, P, K, l.tap_f, a_in.os, wproj ? 1 : 0, plane_lo, plane_w, l.L,
                                           table);
  classify_kernel<<<1024, 256, 0, st>>>(a_in.uvw, a_in.spw, a_in.wavelengths, a_in.nchan, a_in.nspw, R, a_in.wmax, P,
                                        plane_class, row_class, 0, R);
  seg_count_kernel<<<(tracks + 127) / 128, 128, 0, st>>>(a_in.starts, a_in.nslots, a_in.seg, R, a_in.nchan, row_class,
                                                         nseg);
  scan_kernel<<<1, 1024, 0, st>>>(nseg, seg_off, tracks, seg_total);
  seg_write_kernel<<<(tracks + 127) / 128, 128, 0, st>>>(a_in.starts, a_in.nslots, a_in.seg, R, a_in.nchan, row_class,
                                                         seg_off, segs, class_count, cl.n, a_in.error);
  class_offsets_kernel<<<1, 1, 0, st>>>(class_count, class_off, class_cursor, cl.n);
  bucket_kernel<<<1024, 256, 0, st>>>(segs, seg_total, sorted, class_cursor, class_off);
  if (cudaGetLastError() != cudaSuccess) return false;
  GridArgs a = a_in;
  a.W_full = W;
  a.tap_f = l.tap_f;
  a.plane_lo = plane_lo;
  a.conv_w = table;
  a.conv_w_stride = l.L;
  a.segments = sorted;
  a.segment_capacity = l.maxseg;
#if defined(BULLSEYE_SINGLE)
  if (comp)
    return wproj ? support_aware_launches<true, true>(a, cl, vs, nfacets, class_count, class_off, work_next, st)
                 : support_aware_launches<false, true>(a, cl, vs, nfacets, class_count, class_off, work_next, st);
#endif
  return wproj ? support_aware_launches<true, false>(a, cl, vs, nfacets, class_count, class_off, work_next, st)
               : support_aware_launches<false, false>(a, cl, vs, nfacets, class_count, class_off, work_next, st);
}
