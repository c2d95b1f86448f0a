// Romein-strategy convolutional gridder for GB300 (sm_103a).
//
// Work decomposition.  One CTA grids one *track*: the visibilities of one (facet, baseline,
// channel) in time order (rows of a baseline are contiguous after repack_input_data, as in
// bullseye/mo/gpu_algorithm/wrapper.cu:367-454).  Consecutive samples of a track move slowly
// across the uv grid, which is what Romein's ownership scheme exploits (J. W. Romein, "An
// efficient work-distribution strategy for gridding radio-telescope data on GPUs", ICS 2012).
//
// Ownership.  For full support W, the W x W cells under any visibility's kernel footprint
// contain exactly one cell of every (x mod W, y mod W) class.  Thread (du, strip) owns the
// classes x = du (mod W) and y in {strip*J .. strip*J+J-1} (mod W): for each visibility it
// updates exactly the J cells of its classes inside the footprint, accumulating in registers
// while the owned cell stays the same and flushing with a global atomic when it changes.  The
// reference GPU kernel instead binds each thread to a fixed footprint offset
// (bullseye/mo/gpu_algorithm/templated_gridder.h:59-69), which flushes on every cell move.
//
// Per-visibility work (the prologue) is done once per CTA, not once per thread: V threads each
// prepare one visibility (correlation selection, weights x flags, Jones J_p^-1 V J_q^-H, facet
// phase rotation, planar uv transform, cell and tap-offset selection) into shared memory, the
// CTA then stages the 2W + J - 1 taps of each staged visibility (in the persistent batched
// kernel: two TMA bulk copies per visibility from the support-window table, completed on an
// mbarrier; otherwise per-tap asynchronous copies from the ABI's table), and all threads grid
// the staged chunk.
//
// Numerics (matching the reference CPU library, bullseye/mo/cpu_algorithm/*):
//  * uvw / lambda, the phase argument 2 pi (u dl + v dm + w dn), the uv transform and the
//    cell/tap selection are evaluated in FP64 in both libraries;
//  * 1-D AA kernels select cells and taps with floor (the reference sets FE_DOWNWARD,
//    convolution_policies.h:73-75); w-projection uses round-half-even (FE_TONEAREST, :233);
//  * tap index = trunc((1 - u + round(u)) * os) + j*os; a visibility is dropped when
//    disc + W + 2 >= n or disc < 0 (convolution_policies.h:86-97);
//  * single-precision library: visibilities, taps and the register accumulation are FP32,
//    the phase is evaluated by sincospif on the argument reduced in FP64 to turns; grid
//    flushes can be compensated (hi/lo pair, TwoSum on the value returned by the atomic);
//  * normalisation: sum over taps of the real tap weight times weight x flag
//    (templated_gridder.h:97 and store_normalization_term), computed per visibility as
//    Re(sum_j k_u[j] * sum_i k_v[i]) from kernel row sums precomputed in FP64, accumulated per
//    staging slot (FP32 with Kahan compensation in the single library, FP64 in the double one)
//    and reduced per warp into FP64.
#pragma once
#include <algorithm>
#include <type_traits>

#include "common.h"

namespace bz {

#if defined(BULLSEYE_SINGLE)
typedef float acc_real;
#else
typedef double acc_real;
#endif

struct cplx {
  acc_real re, im;
};
__device__ __forceinline__ cplx cmul(cplx a, cplx b) {
  cplx r;
  r.re = a.re * b.re - a.im * b.im;
  r.im = a.re * b.im + a.im * b.re;
  return r;
}

enum CorrMode { CORR_SINGLE = 0, CORR_DUAL = 1, CORR_QUAD = 2, CORR_QUAD_JONES = 3, CORR_SAMPLING = 4 };

// Per-facet transform constants, evaluated on the host in FP64
// (phase_transform_policies.h:110-134, baseline_transform_policies.h:117-149).
struct FacetXform {
  double u_term, v_term;  // planar uv transform: u -= w u_term, v -= w v_term
  double dl, dm, dn;      // phase rotation offsets
  // the facet's grid: uv scale (pixels per wavelength), footprint-corner offsets nx/2 - s and
  // ny/2 - s, the complex-element offset of its [groups][NC][ny][nx] block, and its size
  double u_scale, v_scale, gcx, gcy;
  long long grid_base;
  int nx, ny;
};

struct GridArgs {
  // row inputs (device)
  const vis_complex *vis;
  const vis_real *weights;
  const uint8_t *flags;
  const vis_real *uvw;
  const uint8_t *flagged_rows;
  const unsigned *field;
  const unsigned *spw;
  const unsigned *ant1;
  const unsigned *ant2;
  const size_t *time_ids;
  const vis_complex *jones_inv;  // inverted 2x2 terms [T][A][F][S][Ch][4]
  const vis_complex *jones_inv_t;  // the same terms time-innermost, [A][S][Ch][F][T][4], or null (record kernel)
  const size_t *starts;          // baseline row starts [slots + 1] or null (fixed segments)
  // per-run tables (device)
  const vis_real *wavelengths;
  const uint8_t *enabled;
  const size_t *cgi;
  const void *conv;              // real [K] or complex [P][K]
  const double *tap_sums;        // FP64 complex [P][tap_f] row sums of the kernel, or null
  const float *tap_sums_f;       // the same rounded to FP32 (the single-precision record kernel), or null
  int tap_f;
  const void *conv_t;            // kernel regrouped by tap offset [P][tap_f][W], or null
  const void *conv_w;            // support-window rows [P][tap_f][conv_w_stride], or null (see
                                 // the batched planner): a staged tap row is one bulk copy
  int conv_w_stride;
  const uint8_t *facet_row_mask; // [facets][rows]: 0 leaves the row out of that facet, or null
  const FacetXform *facets;
  // outputs
  vis_complex *grid;             // slices [(f*groups + g)*NC + k][ny][nx]
  vis_complex *grid_lo;          // compensation slices (same layout) or null
  double *norm;                  // [f][groups][NC] or null (sampling function)
  int *error;                    // sticky device error word
  // sizes and scalars
  long long nrows;
  int nchan, npol, pol0, pol1, nspw, nant, ntimes;
  int facet_base;                // facet index of launch facet 0 in the ABI facet list
  int nfacets_total;             // ABI num_facet_centres (Jones indexing)
  int groups;                    // cube channels (or sampling-function channels)
  int nx, ny, W, os, K, P;
  int W_full;                    // the ABI's full support (visibility acceptance test); 0 means W
  int mode;                      // CorrMode
  int phase, uvx;                // faceting phase rotation / planar uv transform
  int nslots, seg;               // track slots (baselines or fixed segments), segment length
  int V;                         // visibilities staged per chunk
  const int *plane_lo;           // per w plane: first tap of its nonzero window (support-aware), or null
  const int4 *segments;          // persistent mode: {row_begin, row_end, channel, -} per segment, or null
  const int *work_count;         // persistent mode: number of segments of this launch (device)
  const int *segment_base;       // persistent mode: index of this launch's first segment (device)
  long long segment_capacity;    // persistent mode: entries in segments
  int *work_next;                // persistent mode: work-item counter (device, zeroed before launch)
  // persistent mode with precomputed visibility records (or null: records are computed in place)
  const void *records;           // GridRec<NC> of every work item, item (si, f) at rec_off[si] x F + f x len
  const long long *rec_off;      // per scheduled segment: records of the segments before it
  const int2 *item_range;        // per work item si x F + f: its valid records [x, y) (x >= y: none)
  long long rec_capacity;        // records the buffer holds (a segment past it is gridded in place)
  long long range_capacity;      // entries of item_range (items past it grid all their records)
  unsigned imaging_field;
  double u_scale, v_scale, gcx, gcy, wmax;
};

// Error bits written to GridArgs::error (host decodes them)
enum DeviceError {
  DEV_ERR_GRID_INDEX = 1,
  DEV_ERR_JONES_INDEX = 2,
  DEV_ERR_SINGULAR = 4,
  DEV_ERR_POL_INDEX = 8,
  DEV_ERR_WAIT_TIMEOUT = 16,  // a bounded wait on the tap-copy barrier ran out
  DEV_ERR_ANTENNA = 32        // an antenna pair outside baseline_count (row sort)
};

template <bool WPROJ>
struct TapT;
template <>
struct TapT<false> {
  typedef acc_real type;
};
template <>
struct TapT<true> {
  typedef cplx type;
};

// One staged visibility, prepared by the prologue (16-byte aligned header for vector loads).
template <int NC>
struct __align__(16) VisRec {
  int u0, v0, ru, rv;      // footprint corner and its residues mod W
  int g, valid, fu, fv;    // grid group, validity, tap offsets
  int plane, fu0, fv0, pad0;  // w plane; tap offsets before the support-window shift
  cplx vis[NC];            // weighted, corrected, rotated visibility
  acc_real cw[NC];         // weight x flag per correlation (normalisation)
};

// What the multiply-add loop reads of a staged visibility: a VisRec without its normalisation
// fields.  The visibility-record kernel writes one per (row, facet, channel) of a call; the
// persistent segment kernel then stages them by bulk copies (sizes a multiple of 16 bytes).
template <int NC>
struct __align__(16) GridRec {
  int u0, v0, ru, rv;      // footprint corner and its residues mod the class width
  int g, valid, fu, fv;    // grid group, validity, support-window table rows
  cplx vis[NC];            // weighted, corrected, rotated visibility
};

__device__ __forceinline__ void load_tap(const void *conv, long long idx, acc_real &t) {
  t = (acc_real)((const vis_real *)conv)[idx];
}
__device__ __forceinline__ void load_tap(const void *conv, long long idx, cplx &t) {
  vis_complex c = ((const vis_complex *)conv)[idx];
  t.re = (acc_real)c.re;
  t.im = (acc_real)c.im;
}

__device__ __forceinline__ cplx tap_mul(acc_real a, acc_real b, cplx v) {
  acc_real t = a * b;
  cplx r;
  r.re = v.re * t;
  r.im = v.im * t;
  return r;
}
__device__ __forceinline__ cplx tap_mul(cplx a, cplx b, cplx v) { return cmul(v, cmul(a, b)); }

// 2x2 complex products on row-major [a b; c d] stored as 4 cplx
__device__ __forceinline__ void jmul(const cplx *A, const cplx *B, cplx *O) {
  cplx t0 = cmul(A[0], B[0]), t1 = cmul(A[1], B[2]);
  cplx t2 = cmul(A[0], B[1]), t3 = cmul(A[1], B[3]);
  cplx t4 = cmul(A[2], B[0]), t5 = cmul(A[3], B[2]);
  cplx t6 = cmul(A[2], B[1]), t7 = cmul(A[3], B[3]);
  O[0].re = t0.re + t1.re; O[0].im = t0.im + t1.im;
  O[1].re = t2.re + t3.re; O[1].im = t2.im + t3.im;
  O[2].re = t4.re + t5.re; O[2].im = t4.im + t5.im;
  O[3].re = t6.re + t7.re; O[3].im = t6.im + t7.im;
}

// Phase factor e^{i x} for an FP64 argument (double-precision library; the single-precision
// library evaluates sincospif on the argument reduced to turns, in choose_cells).
#if !defined(BULLSEYE_SINGLE)
__device__ __forceinline__ cplx phase_factor(double x) {
  cplx r;
  double s, c;
  sincos(x, &s, &c);
  r.re = c;
  r.im = s;
  return r;
}
#endif

// Flush one owned cell's register accumulator into the grid.  Compensated mode adds with
// atomics that return the previous value, then recovers each addition's rounding error exactly
// (TwoSum: s = a + b, e = (a - (s - (s - a))) + (b - (s - a))) and adds it to the lo grid; the
// final grid is hi + lo.  The NC atomics of a cell are issued before any result is consumed.
template <int NC, bool COMP>
__device__ __forceinline__ void flush_cell(const GridArgs &a, long long base, long long nxy, int nx, int x, int y,
                                           cplx (&acc)[NC]) {
  const long long cell = base + (long long)y * nx + x;
#if defined(BULLSEYE_SINGLE)
  if (COMP) {
    float2 old[NC];
#pragma unroll
    for (int k = 0; k < NC; ++k)
      old[k] = atomicAdd(reinterpret_cast<float2 *>(a.grid + k * nxy + cell), make_float2(acc[k].re, acc[k].im));
#pragma unroll
    for (int k = 0; k < NC; ++k) {
      float s0 = old[k].x + acc[k].re, b0 = s0 - old[k].x;
      float e0 = (old[k].x - (s0 - b0)) + (acc[k].re - b0);
      float s1 = old[k].y + acc[k].im, b1 = s1 - old[k].y;
      float e1 = (old[k].y - (s1 - b1)) + (acc[k].im - b1);
      if (e0 != 0.0f || e1 != 0.0f)
        atomicAdd(reinterpret_cast<float2 *>(a.grid_lo + k * nxy + cell), make_float2(e0, e1));
    }
  } else {
#pragma unroll
    for (int k = 0; k < NC; ++k)
      atomicAdd(reinterpret_cast<float2 *>(a.grid + k * nxy + cell), make_float2(acc[k].re, acc[k].im));
  }
#else
#pragma unroll
  for (int k = 0; k < NC; ++k) {
    atomicAdd(&a.grid[k * nxy + cell].re, acc[k].re);
    atomicAdd(&a.grid[k * nxy + cell].im, acc[k].im);
  }
#endif
#pragma unroll
  for (int k = 0; k < NC; ++k) {
    acc[k].re = 0;
    acc[k].im = 0;
  }
}

// Compensated flushes go through a per-warp queue in shared memory: a lane that must flush a
// cell appends (cell, values) and carries on; when a queue holds kDrainAt records the warp drains
// it with one record per lane, so the atomics' round trips overlap instead of serialising in the
// lane that owns the cells.
constexpr int kFlushQueueCap = 64;
constexpr int kDrainAt = 32;

template <int NC>
struct FlushRec {
  long long cell;        // grid element of correlation 0 (base + y * nx + x)
  float2 v[NC];
};

template <int NC>
__device__ __forceinline__ void compensated_add(const GridArgs &a, long long idx, float2 val, float2 old) {
  float s0 = old.x + val.x, b0 = s0 - old.x;
  float e0 = (old.x - (s0 - b0)) + (val.x - b0);
  float s1 = old.y + val.y, b1 = s1 - old.y;
  float e1 = (old.y - (s1 - b1)) + (val.y - b1);
  if (e0 != 0.0f || e1 != 0.0f) atomicAdd(reinterpret_cast<float2 *>(a.grid_lo + idx), make_float2(e0, e1));
}

// Drain the calling warp's queue (warp-uniform call).
template <int NC>
__device__ __forceinline__ void drain_queue(const GridArgs &a, long long nxy, FlushRec<NC> *q, int *qn) {
#if defined(BULLSEYE_SINGLE)
  __syncwarp();
  const int n = min(*qn, kFlushQueueCap);
  const int lane = threadIdx.x & 31;
  for (int i = lane; i < n; i += 32) {
    const FlushRec<NC> r = q[i];
    float2 old[NC];
#pragma unroll
    for (int k = 0; k < NC; ++k) old[k] = atomicAdd(reinterpret_cast<float2 *>(a.grid + r.cell + k * nxy), r.v[k]);
#pragma unroll
    for (int k = 0; k < NC; ++k) compensated_add<NC>(a, r.cell + k * nxy, r.v[k], old[k]);
  }
  __syncwarp();
  if (lane == 0) *qn = 0;
  __syncwarp();
#endif
}

// Queue one owned cell's accumulator (falls back to a direct flush when the queue is full).
template <int NC>
__device__ __forceinline__ void queue_cell(const GridArgs &a, long long base, long long nxy, int nx, int x, int y,
                                           cplx (&acc)[NC], FlushRec<NC> *q, int *qn) {
#if defined(BULLSEYE_SINGLE)
  const int slot = atomicAdd(qn, 1);
  if (slot < kFlushQueueCap) {
    FlushRec<NC> r;
    r.cell = base + (long long)y * nx + x;
#pragma unroll
    for (int k = 0; k < NC; ++k) r.v[k] = make_float2(acc[k].re, acc[k].im);
    q[slot] = r;
#pragma unroll
    for (int k = 0; k < NC; ++k) { acc[k].re = 0; acc[k].im = 0; }
  } else {
    flush_cell<NC, true>(a, base, nxy, nx, x, y, acc);
  }
#endif
}

// Per-visibility normalisation partial sums of a staged chunk (8 bytes per correlation either way).
// The single-precision library accumulates them in FP32 with Kahan compensation and widens to
// FP64 only when a partial sum leaves the CTA; the double library accumulates in FP64.
#if defined(BULLSEYE_SINGLE)
struct NormAcc {
  float s, c;
};
__device__ __forceinline__ void norm_zero(NormAcc &n) { n.s = 0.f; n.c = 0.f; }
__device__ __forceinline__ void norm_add(NormAcc &n, float x) {
  const float y = x - n.c;
  const float t = n.s + y;
  n.c = (t - n.s) - y;
  n.s = t;
}
__device__ __forceinline__ double norm_value(const NormAcc &n) { return (double)n.s - (double)n.c; }
typedef float NormTerm;
#else
typedef double NormAcc;
__device__ __forceinline__ void norm_zero(NormAcc &n) { n = 0.0; }
__device__ __forceinline__ void norm_add(NormAcc &n, double x) { n += x; }
__device__ __forceinline__ double norm_value(const NormAcc &n) { return n; }
typedef double NormTerm;
#endif
static_assert(sizeof(NormAcc) == sizeof(double), "normalisation partial sums keep the shared-memory layout");

// Per-channel constants of the prologue, recomputed only when the spw changes along a track.
struct ChanCache {
  unsigned spw = 0xffffffffu;
  double inv = 0;     // 1 / lambda
  double su = 0, sv = 0, sw = 0;  // (1 / lambda) x u_scale, v_scale, plane scale
};

// Cells, taps, w plane and phase factor of one visibility in one facet: the geometry shared by
// the gridder and its adjoint, so both select exactly the same footprint.
struct CellChoice {
  int du, dv;    // footprint corner (full support)
  int fu, fv;    // tap offsets into the plane's kernel row
  int plane;     // w plane
  bool flip;     // w < 0 with w-projection: grid the conjugate at (-u, -v)
};

// Returns false when the footprint leaves the grid or the w plane is out of range (the reference's
// acceptance test: corner >= 0 and corner + W + 2 < n, convolution_policies.h:81-83,241-243).
template <bool WPROJ>
__device__ __forceinline__ bool choose_cells(double um, double vm, double wm, const ChanCache &cc,
                                             const FacetXform &fx, bool phase, bool uvx, double u_scale,
                                             double v_scale, double plane_scale, double gcx, double gcy, int nx,
                                             int ny, int Wf, int P, int os, cplx &ph, CellChoice &out) {
  ph.re = 1;
  ph.im = 0;
#if defined(BULLSEYE_SINGLE)
  // Single-precision library: the same mathematics with fewer FP64 operations (GB300 issues FP64
  // at 1/64 of FP32).  FP64 is kept for the phase argument, reduced in turns:
  //   t = (u dl + v dm + w dn) / lambda (metres x 1/lambda),  phase = e^{2 pi i (t - rint(t))},
  // and for the pixel coordinates, scaled from metres by the per-channel constants
  // (1/lambda) x u_scale and (1/lambda) x v_scale, and the tap offsets.
  (void)u_scale;
  (void)v_scale;
  (void)plane_scale;
  if (phase) {
    const double t = (um * fx.dl + vm * fx.dm + wm * fx.dn) * cc.inv;
    const float f = (float)(t - rint(t));
    float sn, cs;
    sincospif(2.0f * f, &sn, &cs);
    ph.re = cs;
    ph.im = sn;
  }
  double u = um, v = vm;
  if (uvx) {
    u = fma(-wm, fx.u_term, um);
    v = fma(-wm, fx.v_term, vm);
  }
  u *= cc.su;
  v *= cc.sv;
  double wabs = wm;
  out.flip = WPROJ && wm < 0;
  if (out.flip) {
    u = -u; v = -v; wabs = -wm;
  }
  const double ru_ = WPROJ ? rint(u) : floor(u);
  const double rv_ = WPROJ ? rint(v) : floor(v);
  // the corner offsets nx/2 - s are integers, so round(u + gcx) = round(u) + gcx
  const double du_d = ru_ + gcx;
  const double dv_d = rv_ + gcy;
  long long plane = 0;
  if (WPROJ) {
    double pl = rint(fabs(wabs) * cc.sw);
    plane = (pl >= 0.0 && pl < (double)P) ? (long long)pl : -1;  // NaN and out of range -> dropped
  }
  if (!(du_d >= 0.0 && dv_d >= 0.0 && du_d + (Wf + 2) < (double)nx && dv_d + (Wf + 2) < (double)ny && plane >= 0 &&
        plane < P))
    return false;
  // tap offsets in FP64: an FP32 fraction moves a tap by one oversampled step about once in 1e5
  // samples, which shows in the dirty image at the 1e-5 level
  out.fu = (int)((1.0 - (u - ru_)) * (double)os);
  out.fv = (int)((1.0 - (v - rv_)) * (double)os);
#else
  // Double-precision library: the reference's operation order (parity at 1e-12 needs the same
  // cells and taps): uvw / lambda, phase, uv transform, scale, round, tap offsets.
  double u = um * cc.inv, v = vm * cc.inv, w = wm * cc.inv;
  if (phase) ph = phase_factor(6.283185307179586476925286766559 * (u * fx.dl + v * fx.dm + w * fx.dn));
  if (uvx) {
    u = u - w * fx.u_term;
    v = v - w * fx.v_term;
  }
  u *= u_scale;
  v *= v_scale;
  out.flip = WPROJ && w < 0;
  if (out.flip) {
    u = -u; v = -v; w = -w;
  }
  const double ru_ = WPROJ ? rint(u) : floor(u);
  const double rv_ = WPROJ ? rint(v) : floor(v);
  const double du_d = WPROJ ? rint(u + gcx) : floor(u + gcx);
  const double dv_d = WPROJ ? rint(v + gcy) : floor(v + gcy);
  long long plane = 0;
  if (WPROJ) {
    double pl = rint(fabs(w) * plane_scale);
    plane = (pl >= 0.0 && pl < (double)P) ? (long long)pl : -1;  // NaN and out of range -> dropped
  }
  if (!(du_d >= 0.0 && dv_d >= 0.0 && du_d + (Wf + 2) < (double)nx && dv_d + (Wf + 2) < (double)ny && plane >= 0 &&
        plane < P))
    return false;
  out.fu = (int)((1.0 - u + ru_) * (double)os);
  out.fv = (int)((1.0 - v + rv_) * (double)os);
#endif
  out.du = (int)du_d;
  out.dv = (int)dv_d;
  out.plane = (int)plane;
  return true;
}

// ------------------------------------------------------------ double-float cell choice
// Single-precision library, record kernel: the cell, tap and phase choice of choose_cells with
// pairs of floats in place of FP64 (GB300 issues FP64 at 1/64 of FP32, and the FP64 pipe bounds a
// prologue that keeps about 40 FP64 operations per visibility and facet).  A pair hi + lo
// (|lo| <= ulp(hi) / 2) carries about 48 significant bits; sums use Knuth's error-free TwoSum,
// products the FMA form of Dekker's TwoProduct (products by __fmul_rn, which is never contracted
// into an FMA).  Per facet and spw the FP64 constants are split into pairs once (DfFacet); each
// visibility then needs FP32 arithmetic only.  Roundings decide on the exact high part and use
// the low part at ties, so cells and taps agree with the FP64 choice except where the two
// computations round a value within about 1e-12 pixel of a boundary differently.
struct DF {
  float hi, lo;
};
struct DfFacet {
  DF pu, pv, pw;  // phase: dl / lambda, dm / lambda, dn / lambda (turns per metre)
  DF su, sv;      // pixels per metre: (1 / lambda) x u_scale, (1 / lambda) x v_scale
  DF ut, vt;      // planar uv transform terms
  int gcx, gcy;   // footprint-corner offsets nx/2 - s, ny/2 - s
  float osf;      // oversampling factor
};
#if defined(BULLSEYE_SINGLE)
__device__ __forceinline__ DF df_split(double x) {
  DF r;
  r.hi = (float)x;
  r.lo = (float)(x - (double)r.hi);
  return r;
}
__device__ __forceinline__ DF df_quick(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return DF{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ DF df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return DF{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ DF df_add(DF a, DF b) {
  const DF s = df_two_sum(a.hi, b.hi);
  return df_quick(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ DF df_mul_f(DF a, float b) {
  const float p = __fmul_rn(a.hi, b);
  const float e = fmaf(a.lo, b, fmaf(a.hi, b, -p));
  return df_quick(p, e);
}
__device__ __forceinline__ DF df_mul(DF a, DF b) {
  const float p = __fmul_rn(a.hi, b.hi);
  const float e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, fmaf(a.hi, b.hi, -p)));
  return df_quick(p, e);
}

// Round half to even, and the int of an integer-valued float, for |x| < 2^22: adding 1.5 x 2^23
// leaves unit spacing, so the sum is the rounded value and its bits count it (FP32 adds on the
// FMA pipe instead of the rounding and conversion instructions).
__device__ __forceinline__ float rint22(float x) { return __fsub_rn(__fadd_rn(x, 12582912.f), 12582912.f); }
__device__ __forceinline__ int int22(float k) { return __float_as_int(__fadd_rn(k, 12582912.f)) - 0x4B400000; }
__device__ __forceinline__ float floor22(float x) {
  const float r = rint22(x);
  return r > x ? __fsub_rn(r, 1.f) : r;
}

__device__ __forceinline__ void df_facet(const FacetXform &fx, double inv, int os, DfFacet &k) {
  k.osf = (float)os;
  k.pu = df_split(fx.dl * inv);
  k.pv = df_split(fx.dm * inv);
  k.pw = df_split(fx.dn * inv);
  k.su = df_split(inv * fx.u_scale);
  k.sv = df_split(inv * fx.v_scale);
  k.ut = df_split(fx.u_term);
  k.vt = df_split(fx.v_term);
  k.gcx = (int)fx.gcx;
  k.gcy = (int)fx.gcy;
}

// Rounds x (|x| < 2^22) to the nearest integer, halves to even like rint (round = true), or down
// like floor; d = x - r as a pair.  hi - r is exact (Sterbenz), and a low part cannot carry x past
// the next rounding boundary unless hi sits on it.
__device__ __forceinline__ void df_round(DF x, bool round, float &r, DF &d) {
  if (round) {
    r = rint22(x.hi);
    const float h = __fsub_rn(x.hi, r);
    if (h == 0.5f && x.lo > 0.f) {
      r = __fadd_rn(r, 1.f);
      d = DF{-0.5f, x.lo};
    } else if (h == -0.5f && x.lo < 0.f) {
      r = __fsub_rn(r, 1.f);
      d = DF{0.5f, x.lo};
    } else {
      d = DF{h, x.lo};
    }
  } else {
    r = floor22(x.hi);
    const float h = __fsub_rn(x.hi, r);
    if (h == 0.f && x.lo < 0.f) {
      r = __fsub_rn(r, 1.f);
      d = DF{1.f, x.lo};
    } else {
      d = DF{h, x.lo};
    }
  }
}

// trunc((1 - d) x os) for 1 - d > 0 (the tap offset), with the low part deciding at integers.
__device__ __forceinline__ int df_tap(DF d, float osf) {
  DF e = df_two_sum(1.f, -d.hi);
  e = df_quick(e.hi, __fsub_rn(e.lo, d.lo));
  e = df_mul_f(e, osf);
  float k = floor22(e.hi);
  if (e.hi == k && e.lo < 0.f) k = __fsub_rn(k, 1.f);
  return int22(k);
}

// choose_cells with the facet's pairs k and the row's w plane (computed per row in FP64: it does
// not depend on the facet; -1 when out of range).
template <bool WPROJ>
__device__ __forceinline__ bool choose_cells_df(float um, float vm, float wm, const DfFacet &k, int plane, bool phase,
                                                bool uvx, int nx, int ny, int Wf, int P, int os, cplx &ph,
                                                CellChoice &out) {
  ph.re = 1;
  ph.im = 0;
  if (phase) {
    const DF t = df_add(df_add(df_mul_f(k.pu, um), df_mul_f(k.pv, vm)), df_mul_f(k.pw, wm));
    const float r = fabsf(t.hi) < 4194304.f ? rint22(t.hi) : rintf(t.hi);
    const float f = __fadd_rn(__fsub_rn(t.hi, r), t.lo);
    float sn, cs;
    sincospif(2.0f * f, &sn, &cs);
    ph.re = cs;
    ph.im = sn;
  }
  DF u, v;
  if (uvx) {
    const DF pu = df_mul_f(k.ut, wm), pv = df_mul_f(k.vt, wm);
    u = df_mul(df_add(DF{um, 0.f}, DF{-pu.hi, -pu.lo}), k.su);
    v = df_mul(df_add(DF{vm, 0.f}, DF{-pv.hi, -pv.lo}), k.sv);
  } else {
    u = df_mul_f(k.su, um);
    v = df_mul_f(k.sv, vm);
  }
  out.flip = WPROJ && wm < 0;
  if (out.flip) {
    u = DF{-u.hi, -u.lo};
    v = DF{-v.hi, -v.lo};
  }
  // corners far off the grid (or not finite) are rejected before rounding
  if (!(fabsf(u.hi) < 4194304.f && fabsf(v.hi) < 4194304.f)) return false;
  float ru, rv;
  DF du_f, dv_f;
  df_round(u, WPROJ, ru, du_f);
  df_round(v, WPROJ, rv, dv_f);
  const int du = int22(ru) + k.gcx, dv = int22(rv) + k.gcy;
  if (!(du >= 0 && dv >= 0 && du + (Wf + 2) < nx && dv + (Wf + 2) < ny && plane >= 0 && plane < P)) return false;
  out.fu = df_tap(du_f, k.osf);
  out.fv = df_tap(dv_f, k.osf);
  out.du = du;
  out.dv = dv;
  out.plane = plane;
  return true;
}
#endif

// The facet-independent part of a visibility's prologue: one (row, channel)'s checks and inputs.
// Four consecutive values starting at a multiple of four elements (a 2x2 Jones term; a row's four
// correlations, weights or flags): vector loads when the array's base allows them (`vec`, the same
// for every thread of a launch), element loads otherwise (a caller's device array may sit at any
// element boundary).
__device__ __forceinline__ bool vec16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }
__device__ __forceinline__ void load_c4(const vis_complex *p, bool vec, cplx out[4]) {
  if (vec) {
#if defined(BULLSEYE_SINGLE)
    const float4 x = __ldg(reinterpret_cast<const float4 *>(p)), y = __ldg(reinterpret_cast<const float4 *>(p) + 1);
    out[0].re = x.x; out[0].im = x.y; out[1].re = x.z; out[1].im = x.w;
    out[2].re = y.x; out[2].im = y.y; out[3].re = y.z; out[3].im = y.w;
#else
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const double2 v = __ldg(reinterpret_cast<const double2 *>(p) + k);
      out[k].re = v.x; out[k].im = v.y;
    }
#endif
  } else {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      out[k].re = p[k].re;
      out[k].im = p[k].im;
    }
  }
}
__device__ __forceinline__ void load_r4(const vis_real *p, bool vec, acc_real out[4]) {
  if (vec) {
#if defined(BULLSEYE_SINGLE)
    const float4 x = __ldg(reinterpret_cast<const float4 *>(p));
    out[0] = x.x; out[1] = x.y; out[2] = x.z; out[3] = x.w;
#else
    const double2 x = __ldg(reinterpret_cast<const double2 *>(p)), y = __ldg(reinterpret_cast<const double2 *>(p) + 1);
    out[0] = x.x; out[1] = x.y; out[2] = y.x; out[3] = y.y;
#endif
  } else {
#pragma unroll
    for (int k = 0; k < 4; ++k) out[k] = (acc_real)p[k];
  }
}
__device__ __forceinline__ void load_f4(const uint8_t *p, bool vec, bool out[4]) {
  if (vec) {
    const unsigned x = __ldg(reinterpret_cast<const unsigned *>(p));
#pragma unroll
    for (int k = 0; k < 4; ++k) out[k] = ((x >> (8 * k)) & 0xffu) != 0;  // little-endian byte k
  } else {
#pragma unroll
    for (int k = 0; k < 4; ++k) out[k] = p[k] != 0;
  }
}

template <int NC>
struct RowInputs {
  bool use;            // in range, channel enabled, spw and grid group valid, Jones indices valid
  bool row_ok;         // not flagged, in the imaging field
  unsigned spw;
  int g;               // grid group (cube channel)
  long long sc;        // spw x nchan + channel
  long long jt1, jt2;  // Jones rows t x nant + antenna; with jones_inv_t, ((antenna x S + spw) x Ch + channel) x F
  long long tt;        // the row's time index (with jones_inv_t)
  double um, vm, wm;
  vis_real uvw_in[3];  // as stored (the double-float cell choice starts from them)
  cplx vis[NC];
  acc_real wt[NC];
  bool fl[NC];
};

template <int NC>
__device__ __forceinline__ void load_row(const GridArgs &a, int chan, long long row, bool in_range, RowInputs<NC> &ri) {
  ri.use = false;
  if (!in_range) return;
  const int c = chan;
  const unsigned spw = a.spw[row];
  if (spw >= (unsigned)a.nspw) {
    atomicOr(a.error, DEV_ERR_GRID_INDEX);
    return;
  }
  const long long sc = (long long)spw * a.nchan + c;
  if (!a.enabled[sc]) return;
  const size_t g = a.cgi[sc];
  if (g >= (size_t)a.groups) {
    atomicOr(a.error, DEV_ERR_GRID_INDEX);
    return;
  }
  ri.spw = spw;
  ri.sc = sc;
  ri.g = (int)g;
  ri.uvw_in[0] = a.uvw[3 * row];
  ri.uvw_in[1] = a.uvw[3 * row + 1];
  ri.uvw_in[2] = a.uvw[3 * row + 2];
  ri.um = (double)ri.uvw_in[0];
  ri.vm = (double)ri.uvw_in[1];
  ri.wm = (double)ri.uvw_in[2];
  ri.row_ok = !a.flagged_rows[row] && (a.field[row] == a.imaging_field);
  const long long base = ((long long)row * a.nchan + c) * a.npol;
  if (a.mode == CORR_SAMPLING) {
#pragma unroll
    for (int k = 0; k < NC; ++k) { ri.vis[k].re = 1; ri.vis[k].im = 0; ri.wt[k] = 1; ri.fl[k] = false; }
  } else if constexpr (NC == 4) {
    // a row's 4 correlations start at a multiple of 4 elements when npol = 4
    const bool v4 = a.npol == 4;
    load_c4(a.vis + base, v4 && vec16(a.vis), ri.vis);
    load_r4(a.weights + base, v4 && vec16(a.weights), ri.wt);
    load_f4(a.flags + base, v4 && (reinterpret_cast<uintptr_t>(a.flags) & 3) == 0, ri.fl);
  } else {
#pragma unroll
    for (int k = 0; k < NC; ++k) {
      int pi = (k == 0) ? a.pol0 : a.pol1;
      vis_complex vv = a.vis[base + pi];
      ri.vis[k].re = vv.re; ri.vis[k].im = vv.im;
      ri.wt[k] = (acc_real)a.weights[base + pi];
      ri.fl[k] = a.flags[base + pi] != 0;
    }
  }
  ri.jt1 = ri.jt2 = ri.tt = 0;
  if (NC == 4 && a.mode == CORR_QUAD_JONES) {
    const long long t = (long long)a.time_ids[row];
    const unsigned a1 = a.ant1[row], a2 = a.ant2[row];
    if (t < 0 || t >= a.ntimes || a1 >= (unsigned)a.nant || a2 >= (unsigned)a.nant) {
      atomicOr(a.error, DEV_ERR_JONES_INDEX);
      return;
    }
    if (a.jones_inv_t) {
      ri.jt1 = (((long long)a1 * a.nspw + spw) * a.nchan + c) * a.nfacets_total;
      ri.jt2 = (((long long)a2 * a.nspw + spw) * a.nchan + c) * a.nfacets_total;
      ri.tt = t;
    } else {
      ri.jt1 = t * a.nant + a1;
      ri.jt2 = t * a.nant + a2;
    }
  }
  ri.use = true;
}

// The facet part of the prologue: the row's Jones correction for facet f_local, weights and flags,
// cells, taps, phase rotation and flip, into rec (valid = 0 when the row is left out of the facet
// or its footprint is off the grid).  inv = 1 / lambda of the row's channel.
template <int NC, bool WPROJ>
__device__ __forceinline__ void facet_record(const GridArgs &a, int f_local, int chan, long long row,
                                             const RowInputs<NC> &ri, double inv, VisRec<NC> &rec,
                                             const double plane_scale, const DfFacet *dk = nullptr,
                                             int plane_df = -1) {
  rec.valid = 0;
  if (!ri.use) return;
  const int c = chan;
  const int fglob = a.facet_base + f_local;
  // a row left out of this facet (uneven facet layouts) is skipped like an off-grid visibility
  if (a.facet_row_mask && !a.facet_row_mask[(long long)fglob * a.nrows + row]) return;
  const FacetXform &fx = a.facets[f_local];
  cplx vis[NC];
#pragma unroll
  for (int k = 0; k < NC; ++k) vis[k] = ri.vis[k];
  if (NC == 4 && a.mode == CORR_QUAD_JONES) {
    // V <- J_p^-1 (V J_q^-H)   (correlation_gridding_policies.h:523-542; terms pre-inverted).
    // With the time-innermost copy, the 32 rows of a warp (consecutive times of one baseline and
    // channel) read one contiguous run of terms per antenna and facet.
    cplx P[4], Q[4], T[4], O[4];
    if (a.jones_inv_t) {
      const bool jv = vec16(a.jones_inv_t);
      load_c4(a.jones_inv_t + ((ri.jt1 + fglob) * a.ntimes + ri.tt) * 4, jv, P);
      load_c4(a.jones_inv_t + ((ri.jt2 + fglob) * a.ntimes + ri.tt) * 4, jv, Q);
    } else {
      const long long i1 = (((ri.jt1 * a.nfacets_total + fglob) * a.nspw + ri.spw) * a.nchan + c) * 4;
      const long long i2 = (((ri.jt2 * a.nfacets_total + fglob) * a.nspw + ri.spw) * a.nchan + c) * 4;
      const bool jv = vec16(a.jones_inv);
      load_c4(a.jones_inv + i1, jv, P);
      load_c4(a.jones_inv + i2, jv, Q);
    }
    // hermitian transpose of Q
    cplx qh[4];
    qh[0].re = Q[0].re; qh[0].im = -Q[0].im;
    qh[1].re = Q[2].re; qh[1].im = -Q[2].im;
    qh[2].re = Q[1].re; qh[2].im = -Q[1].im;
    qh[3].re = Q[3].re; qh[3].im = -Q[3].im;
    jmul(vis, qh, T);
    jmul(P, T, O);
#pragma unroll
    for (int k = 0; k < 4; ++k) vis[k] = O[k];
  }
#pragma unroll
  for (int k = 0; k < NC; ++k) {
    bool keep = !(ri.fl[k] || !ri.row_ok);
    acc_real cw = keep ? ri.wt[k] : (acc_real)0;
    rec.cw[k] = cw;
    vis[k].re *= cw;
    vis[k].im *= cw;
  }
  CellChoice cell;
  cplx ph;
#if defined(BULLSEYE_SINGLE)
  if (dk) {
    if (!choose_cells_df<WPROJ>((float)ri.uvw_in[0], (float)ri.uvw_in[1], (float)ri.uvw_in[2], *dk, plane_df,
                                a.phase != 0, a.uvx != 0, fx.nx, fx.ny, a.W_full ? a.W_full : a.W, a.P, a.os, ph,
                                cell))
      return;
  } else
#endif
  {
    ChanCache cc;
    cc.spw = ri.spw;
    cc.inv = inv;
    cc.su = inv * fx.u_scale;
    cc.sv = inv * fx.v_scale;
    cc.sw = inv * plane_scale;
    if (!choose_cells<WPROJ>(ri.um, ri.vm, ri.wm, cc, fx, a.phase != 0, a.uvx != 0, fx.u_scale, fx.v_scale,
                             plane_scale, fx.gcx, fx.gcy, fx.nx, fx.ny, a.W_full ? a.W_full : a.W, a.P, a.os, ph, cell))
      return;
  }
  if (a.phase) {
#pragma unroll
    for (int k = 0; k < NC; ++k) vis[k] = cmul(vis[k], ph);
  }
  if (cell.flip) {
#pragma unroll
    for (int k = 0; k < NC; ++k) vis[k].im = -vis[k].im;
  }
  const long long plane = cell.plane;
  int du = cell.du, dv = cell.dv;
  rec.fu = cell.fu;
  rec.fv = cell.fv;
  rec.fu0 = cell.fu;
  rec.fv0 = cell.fv;
  int lo = 0;
  if (a.plane_lo) {
    // support-aware: grid only the plane's nonzero window of a.W taps (the taps outside it are
    // exactly zero), shifting the footprint corner and the tap offsets by the window start
    lo = a.plane_lo[plane];
    du += lo;
    dv += lo;
    rec.fu += lo * a.os;
    rec.fv += lo * a.os;
  }
  if (a.conv_w) {
    // start of the (plane, tap offset) row of the support-window table (window start included)
    rec.fu = (int)(((long long)plane * a.tap_f + cell.fu) * a.conv_w_stride);
    rec.fv = (int)(((long long)plane * a.tap_f + cell.fv) * a.conv_w_stride);
  } else if (a.conv_t) {
    // index of the first staged tap in the regrouped table
    const int Wfull = a.W_full ? a.W_full : a.W;
    rec.fu = (int)(((long long)plane * a.tap_f + cell.fu) * Wfull + lo);
    rec.fv = (int)(((long long)plane * a.tap_f + cell.fv) * Wfull + lo);
  }
  rec.plane = (int)plane;
  rec.u0 = du;
  rec.v0 = dv;
  rec.ru = du % a.W;
  rec.rv = dv % a.W;
  rec.g = ri.g;
#pragma unroll
  for (int k = 0; k < NC; ++k) rec.vis[k] = vis[k];
  rec.valid = 1;
}

// One visibility's prologue in one facet, in one piece for the in-place gridder (fewer values live
// at once than load_row + facet_record, which the record kernel uses; both make the same record
// from the same arithmetic).  cc keeps the per-channel constants while the spw stays the same.
template <int NC, bool WPROJ>
__device__ __forceinline__ void prologue(const GridArgs &a, int f_local, int chan, long long row, bool in_range,
                                         VisRec<NC> &rec, ChanCache &cc, const double plane_scale) {
  rec.valid = 0;
  if (!in_range) return;
  const int c = chan;
  unsigned spw = a.spw[row];
  if (spw >= (unsigned)a.nspw) {
    atomicOr(a.error, DEV_ERR_GRID_INDEX);
    return;
  }
  long long sc = (long long)spw * a.nchan + c;
  if (!a.enabled[sc]) return;
  size_t g = a.cgi[sc];
  if (g >= (size_t)a.groups) {
    atomicOr(a.error, DEV_ERR_GRID_INDEX);
    return;
  }
  const int fglob = a.facet_base + f_local;
  // a row left out of this facet (uneven facet layouts) is skipped like an off-grid visibility
  if (a.facet_row_mask && !a.facet_row_mask[(long long)fglob * a.nrows + row]) return;
  const FacetXform &fx = a.facets[f_local];
  if (spw != cc.spw) {  // 1/lambda is constant along a track unless the spw changes
    cc.spw = spw;
    cc.inv = 1.0 / (double)a.wavelengths[sc];
    cc.su = cc.inv * fx.u_scale;
    cc.sv = cc.inv * fx.v_scale;
    cc.sw = cc.inv * plane_scale;
  }
  const double um = (double)a.uvw[3 * row], vm = (double)a.uvw[3 * row + 1], wm = (double)a.uvw[3 * row + 2];
  bool row_ok = !a.flagged_rows[row] && (a.field[row] == a.imaging_field);

  cplx vis[NC];
  acc_real wt[NC];
  bool fl[NC];
  const long long base = ((long long)row * a.nchan + c) * a.npol;
  if (a.mode == CORR_SAMPLING) {
#pragma unroll
    for (int k = 0; k < NC; ++k) { vis[k].re = 1; vis[k].im = 0; wt[k] = 1; fl[k] = false; }
  } else if (NC == 1 || NC == 2) {
#pragma unroll
    for (int k = 0; k < NC; ++k) {
      int pi = (k == 0) ? a.pol0 : a.pol1;
      vis_complex vv = a.vis[base + pi];
      vis[k].re = vv.re; vis[k].im = vv.im;
      wt[k] = (acc_real)a.weights[base + pi];
      fl[k] = a.flags[base + pi] != 0;
    }
  } else {
#pragma unroll
    for (int k = 0; k < NC; ++k) {
      vis_complex vv = a.vis[base + k];
      vis[k].re = vv.re; vis[k].im = vv.im;
      wt[k] = (acc_real)a.weights[base + k];
      fl[k] = a.flags[base + k] != 0;
    }
  }
  if (NC == 4 && a.mode == CORR_QUAD_JONES) {
    // V <- J_p^-1 (V J_q^-H)   (correlation_gridding_policies.h:523-542; terms pre-inverted)
    long long t = (long long)a.time_ids[row];
    unsigned a1 = a.ant1[row], a2 = a.ant2[row];
    if (t < 0 || t >= a.ntimes || a1 >= (unsigned)a.nant || a2 >= (unsigned)a.nant) {
      atomicOr(a.error, DEV_ERR_JONES_INDEX);
      return;
    }
    long long i1 = ((((t * a.nant + a1) * a.nfacets_total + fglob) * a.nspw + spw) * a.nchan + c) * 4;
    long long i2 = ((((t * a.nant + a2) * a.nfacets_total + fglob) * a.nspw + spw) * a.nchan + c) * 4;
    cplx P[4], Q[4], T[4], O[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      vis_complex p = a.jones_inv[i1 + k], q = a.jones_inv[i2 + k];
      P[k].re = p.re; P[k].im = p.im;
      Q[k].re = q.re; Q[k].im = q.im;
    }
    // hermitian transpose of Q
    cplx qh[4];
    qh[0].re = Q[0].re; qh[0].im = -Q[0].im;
    qh[1].re = Q[2].re; qh[1].im = -Q[2].im;
    qh[2].re = Q[1].re; qh[2].im = -Q[1].im;
    qh[3].re = Q[3].re; qh[3].im = -Q[3].im;
    jmul(vis, qh, T);
    jmul(P, T, O);
#pragma unroll
    for (int k = 0; k < 4; ++k) vis[k] = O[k];
  }
#pragma unroll
  for (int k = 0; k < NC; ++k) {
    bool keep = !(fl[k] || !row_ok);
    acc_real cw = keep ? wt[k] : (acc_real)0;
    rec.cw[k] = cw;
    vis[k].re *= cw;
    vis[k].im *= cw;
  }
  CellChoice cell;
  cplx ph;
  if (!choose_cells<WPROJ>(um, vm, wm, cc, fx, a.phase != 0, a.uvx != 0, fx.u_scale, fx.v_scale, plane_scale, fx.gcx,
                           fx.gcy, fx.nx, fx.ny, a.W_full ? a.W_full : a.W, a.P, a.os, ph, cell))
    return;
  if (a.phase) {
#pragma unroll
    for (int k = 0; k < NC; ++k) vis[k] = cmul(vis[k], ph);
  }
  if (cell.flip) {
#pragma unroll
    for (int k = 0; k < NC; ++k) vis[k].im = -vis[k].im;
  }
  const long long plane = cell.plane;
  int du = cell.du, dv = cell.dv;
  rec.fu = cell.fu;
  rec.fv = cell.fv;
  rec.fu0 = cell.fu;
  rec.fv0 = cell.fv;
  int lo = 0;
  if (a.plane_lo) {
    // support-aware: grid only the plane's nonzero window of a.W taps (the taps outside it are
    // exactly zero), shifting the footprint corner and the tap offsets by the window start
    lo = a.plane_lo[plane];
    du += lo;
    dv += lo;
    rec.fu += lo * a.os;
    rec.fv += lo * a.os;
  }
  if (a.conv_w) {
    // start of the (plane, tap offset) row of the support-window table (window start included)
    rec.fu = (int)(((long long)plane * a.tap_f + cell.fu) * a.conv_w_stride);
    rec.fv = (int)(((long long)plane * a.tap_f + cell.fv) * a.conv_w_stride);
  } else if (a.conv_t) {
    // index of the first staged tap in the regrouped table
    const int Wfull = a.W_full ? a.W_full : a.W;
    rec.fu = (int)(((long long)plane * a.tap_f + cell.fu) * Wfull + lo);
    rec.fv = (int)(((long long)plane * a.tap_f + cell.fv) * Wfull + lo);
  }
  rec.plane = (int)plane;
  rec.u0 = du;
  rec.v0 = dv;
  rec.ru = du % a.W;
  rec.rv = dv % a.W;
  rec.g = (int)g;
#pragma unroll
  for (int k = 0; k < NC; ++k) rec.vis[k] = vis[k];
  rec.valid = 1;
}

// Shared-memory bytes for a launch with V staged visibilities.
// Per-warp flush queues (compensated single precision only): nwarps record arrays, then one
// 16-byte counter slot per warp.
template <int NC>
__host__ __device__ inline size_t flush_queue_bytes(int nwarps) {
#if defined(BULLSEYE_SINGLE)
  return (size_t)nwarps * (sizeof(FlushRec<NC>) * kFlushQueueCap + 16);
#else
  (void)nwarps;
  return 0;
#endif
}

// Row taps are stored W + J - 1 long per visibility: the first J - 1 taps are repeated after the
// last, so a thread's J consecutive owned rows read J consecutive taps without a wrap.

// Staged tap rows per visibility: W column taps, then W + J - 1 row taps (the first J - 1 repeated
// after the last), each row padded to a multiple of 16 bytes so that it can be one bulk copy.
template <bool WPROJ>
__host__ __device__ inline int tap_row_u(int W) {
  constexpr int E = (int)(16 / sizeof(typename TapT<WPROJ>::type));
  return (W + E - 1) / E * E;
}
template <bool WPROJ>
__host__ __device__ inline int tap_row_v(int W, int J) {
  constexpr int E = (int)(16 / sizeof(typename TapT<WPROJ>::type));
  return (W + J - 1 + E - 1) / E * E;
}

// Bytes before the tap arrays, rounded up to 16: computed in place, V staged records, their
// normalisation state (partial sums, grid group) and the V + 1 run starts of the chunk; from
// precomputed records, two buffers of V GridRecs (one filled while the other is gridded) and the
// run starts.  A launch reserves the larger, so each work item may take either form.
template <int NC>
__host__ __device__ inline size_t stage_head_per_vis() {
  const size_t own = sizeof(VisRec<NC>) + sizeof(NormAcc) * NC + 2 * sizeof(int);
  const size_t pre = 2 * sizeof(GridRec<NC>) + sizeof(int);
  return own > pre ? own : pre;
}
template <int NC>
__host__ __device__ inline size_t stage_head_bytes(int V) {
  return (stage_head_per_vis<NC>() * (size_t)V + sizeof(int) + 15) / 16 * 16;
}

template <int NC, bool WPROJ>
__host__ __device__ inline size_t grid_smem_bytes(int V, int W, int nthreads, int J) {
  size_t taps = sizeof(typename TapT<WPROJ>::type) * (size_t)V * (tap_row_u<WPROJ>(W) + tap_row_v<WPROJ>(W, J));
  return stage_head_bytes<NC>(V) + taps + flush_queue_bytes<NC>((nthreads + 31) / 32) + 64;
}

// Staged-chunk size V for a CTA of nthreads: one visibility per thread at most, and shared memory
// small enough that the CTAs the register file allows (regs registers per thread) fit on an SM.
template <int NC, bool WPROJ>
__host__ inline int grid_chunk_size(int W, int nthreads, int J, int regs = 128) {
  const int ctas = std::max(1, std::min(8, 65536 / (nthreads * regs)));
  const size_t smem_sm = 227 * 1024;
  size_t budget = std::min<size_t>(200 * 1024, smem_sm / ctas - 1024);
  const size_t fixed = flush_queue_bytes<NC>((nthreads + 31) / 32) + 64 + sizeof(int) + 15;
  budget = budget > fixed ? budget - fixed : 0;
  const size_t per = stage_head_per_vis<NC>() +
                     sizeof(typename TapT<WPROJ>::type) * (size_t)(tap_row_u<WPROJ>(W) + tap_row_v<WPROJ>(W, J));
  return std::max(1, (int)std::min<size_t>(nthreads, budget / per));
}

// premultiplied visibility times the column tap
__device__ __forceinline__ cplx premul(cplx v, acc_real t) {
  cplx r;
  r.re = v.re * t;
  r.im = v.im * t;
  return r;
}
__device__ __forceinline__ cplx premul(cplx v, cplx t) { return cmul(v, t); }
__device__ __forceinline__ void mac(cplx &acc, cplx a, acc_real t) {
  acc.re = fma(a.re, t, acc.re);
  acc.im = fma(a.im, t, acc.im);
}
__device__ __forceinline__ void mac(cplx &acc, cplx a, cplx t) {
  acc.re = fma(a.re, t.re, acc.re);
  acc.re = fma(-a.im, t.im, acc.re);
  acc.im = fma(a.re, t.im, acc.im);
  acc.im = fma(a.im, t.re, acc.im);
}

// Thread -> owned (column, strip) map.  WIDE pads the columns to a multiple of 32 so that every
// warp covers one strip: the row taps it reads are then warp-uniform (shared-memory broadcast).
template <bool WIDE>
__device__ __forceinline__ void owner_map(int tid, int W, int J, int &du, int &strip, bool &owner) {
  const int nstrips = (W + J - 1) / J;
  if (WIDE) {
    const int wpr = (W + 31) >> 5;  // warps per strip
    const int warp = tid >> 5, lane = tid & 31;
    du = (warp % wpr) * 32 + lane;
    strip = warp / wpr;
    owner = du < W && strip < nstrips;
  } else {
    du = tid % W;
    strip = tid / W;
    owner = strip < nstrips;
  }
}

// Register state of a Romein owner thread: the accumulators of its J cells and the footprint they
// belong to.  For the last footprint corner (pu0, pv0) the owned cells are
// (pu0 + ou, pv0 + wrap(ov0 + j)), wrap(i) = i - W when i >= W.
template <int NC, int J>
struct OwnerState {
  cplx acc[J][NC];
  unsigned dirty;
  int cg, pu0, pv0, ou, ov0;
};

// Prologue of one staging slot: the visibility of `row` staged into recs[slot].
template <int NC, bool WPROJ>
__device__ __forceinline__ void stage_slot(const GridArgs &a, int f_local, int chan, long long row, bool in_range,
                                           int slot, VisRec<NC> *recs, ChanCache &cc, double plane_scale) {
  VisRec<NC> rec;
  prologue<NC, WPROJ>(a, f_local, chan, row, in_range, rec, cc, plane_scale);
  recs[slot] = rec;
}

// Normalisation term of a staged visibility from the precomputed kernel row sums, added to its
// slot's running sums (which go to the global normalisation when the slot's grid group changes).
// Runs after the chunk's records are published, so its table loads overlap the tap copies instead
// of lengthening the prologue.
template <int NC>
__device__ __forceinline__ void norm_slot(const GridArgs &a, const VisRec<NC> &rec, int slot, NormAcc *s_nacc,
                                          int *s_ng, long long fslice) {
  if (!rec.valid) return;
  const double *su = a.tap_sums + 2 * ((long long)rec.plane * a.tap_f + rec.fu0);
  const double *sv = a.tap_sums + 2 * ((long long)rec.plane * a.tap_f + rec.fv0);
  const NormTerm nt = (NormTerm)(su[0] * sv[0] - su[1] * sv[1]);
  NormAcc *na = s_nacc + slot * NC;
  if (s_ng[slot] != rec.g) {
    if (s_ng[slot] >= 0) {
#pragma unroll
      for (int k = 0; k < NC; ++k)
        if (norm_value(na[k]) != 0.0) atomicAdd(&a.norm[(fslice + s_ng[slot]) * NC + k], norm_value(na[k]));
    }
#pragma unroll
    for (int k = 0; k < NC; ++k) norm_zero(na[k]);
    s_ng[slot] = rec.g;
  }
#pragma unroll
  for (int k = 0; k < NC; ++k) norm_add(na[k], (NormTerm)rec.cw[k] * nt);
}

// Runs of a staged chunk, found by one warp: maximal stretches of valid staged visibilities with
// one footprint corner and grid group (a Romein thread keeps its cells across a run); an invalid
// slot is a run of its own.  runs[0..n) are the first slots of the runs, runs[n] = nv.
template <class Rec>
__device__ __forceinline__ void find_runs(const Rec *recs, int nv, int *runs, int *nruns) {
  const int lane = threadIdx.x & 31;
  int count = 0;
  for (int b = 0; b < nv; b += 32) {
    const int t = b + lane;
    bool start = false;
    if (t < nv) {
      const int4 c0 = *reinterpret_cast<const int4 *>(&recs[t].u0);
      const int4 c1 = *reinterpret_cast<const int4 *>(&recs[t].g);
      start = !c1.y || t == 0;
      if (!start) {
        const int4 p0 = *reinterpret_cast<const int4 *>(&recs[t - 1].u0);
        const int4 p1 = *reinterpret_cast<const int4 *>(&recs[t - 1].g);
        start = !p1.y || p0.x != c0.x || p0.y != c0.y || p1.x != c1.x;
      }
    }
    const unsigned m = __ballot_sync(0xffffffffu, start);
    if (start) runs[count + __popc(m & ((1u << lane) - 1u))] = t;
    count += __popc(m);
  }
  if (lane == 0) {
    runs[count] = nv;
    *nruns = count;
  }
}

// Asynchronous global -> shared copy of one tap (cp.async: no register staging, so a thread has its
// whole share of a chunk's taps in flight at once).  Kernel tables are stored in the working
// precision, so a tap is copied as it is (4, 8 or 16 bytes, aligned to its size).
template <int BYTES>
__device__ __forceinline__ void copy_tap_async(void *dst_smem, const void *src) {
  static_assert(BYTES == 4 || BYTES == 8 || BYTES == 16, "cp.async copies 4, 8 or 16 bytes");
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst_smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(d), "l"(src), "n"(BYTES) : "memory");
}
// Waits for this thread's outstanding tap copies; a CTA barrier then publishes them.
__device__ __forceinline__ void wait_taps() { asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory"); }

// Taps of every valid staged visibility: W column taps, then W + J - 1 row taps, issued as
// asynchronous copies (the caller runs wait_taps() before the barrier that publishes them).  Thread
// tid walks (visibility, tap) pairs with a stride of blockDim.x pairs, stepped without division.
// Rows are stored with strides TUS and TVS (padded to 16 bytes).
template <int NC, bool WPROJ>
__device__ __forceinline__ void stage_taps(const GridArgs &a, const VisRec<NC> *recs, int nv, int J, int TUS, int TVS,
                                           typename TapT<WPROJ>::type *tu, typename TapT<WPROJ>::type *tv) {
  typedef typename TapT<WPROJ>::type tap_t;
  typedef typename std::conditional<WPROJ, vis_complex, vis_real>::type stored_t;
  static_assert(sizeof(stored_t) == sizeof(tap_t), "kernel tables are stored in the working precision");
  const stored_t *table = reinterpret_cast<const stored_t *>(a.conv_t ? a.conv_t : a.conv);
  // a caller-owned table (the allocation-free entries) may be only element-part aligned: such a
  // table is read through registers
  const bool aligned = (reinterpret_cast<uintptr_t>(table) & (sizeof(tap_t) - 1)) == 0;
  const int W = a.W;
  const int per = 2 * W + J - 1;
  const int tid = threadIdx.x;
  int vi = tid / per, j = tid - vi * per;
  const int svi = (int)blockDim.x / per, sj = (int)blockDim.x - svi * per;
  while (vi < nv) {
    const int4 h1 = *reinterpret_cast<const int4 *>(&recs[vi].g);  // g, valid, fu, fv
    if (h1.y) {
      const bool isv = j >= W;
      const int js = isv ? j - W : j;  // slot in the staged row
      int jj = js >= W ? js - W : js;  // repeated leading row taps
      if (jj >= W) jj = W - 1;
      const long long idx = a.conv_t ? (long long)(isv ? h1.w : h1.z) + jj
                                     : (long long)recs[vi].plane * a.K + (isv ? h1.w : h1.z) + (long long)jj * a.os;
      tap_t *dst = isv ? &tv[vi * TVS + js] : &tu[vi * TUS + js];
      if (aligned) {
        copy_tap_async<sizeof(tap_t)>(dst, table + idx);
      } else {
        load_tap(table, idx, *dst);
      }
    }
    vi += svi;
    j += sj;
    if (j >= per) {
      j -= per;
      ++vi;
    }
  }
}

// Tap-copy barrier (mbarrier) of the bulk-copy staging: V arrivals per chunk, one per staging
// slot, each announcing the bytes of its two row copies.  Waits are bounded.
__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void bar_init(unsigned long long *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ __forceinline__ void bar_arrive(unsigned long long *bar) {
  asm volatile("{\n.reg .b64 st;\nmbarrier.arrive.shared::cta.b64 st, [%0];\n}\n" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void bar_arrive_tx(unsigned long long *bar, unsigned bytes) {
  asm volatile("{\n.reg .b64 st;\nmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}\n" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}
// Non-blocking test of the phase of the given parity.
__device__ __forceinline__ bool bar_test(unsigned long long *bar, unsigned parity) {
  unsigned done;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
// Bounded wait for the phase of the given parity (polls, then polls with short sleeps: about 0.2 s
// at most); false when the bound ran out.
__device__ __forceinline__ bool bar_wait(unsigned long long *bar, unsigned parity) {
  for (int i = 0; i < (1 << 22); ++i) {
    if (bar_test(bar, parity)) return true;
    if (i >= 64) __nanosleep(32);
  }
  return false;
}
// Orders this thread's earlier shared-memory accesses (and those a CTA barrier published to it)
// before its following bulk copies into shared memory.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
// One bulk (TMA) copy global -> shared of `bytes` (16-byte aligned addresses, a multiple of 16
// bytes) that completes its bytes on the barrier.
__device__ __forceinline__ void bulk_copy(void *dst, const void *src, unsigned bytes, unsigned long long *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

// Bulk-copy staging of a chunk's taps from the support-window table: staging slot tid copies its
// visibility's column row (TUS taps) and row row (TVS taps, the repeated leading taps included) as
// two bulk copies and arrives on the barrier with their bytes; an empty slot arrives without bytes.
template <int NC, bool WPROJ, class Rec>
__device__ __forceinline__ void stage_taps_bulk(const GridArgs &a, const Rec *recs, int nv, int TUS, int TVS,
                                                typename TapT<WPROJ>::type *tu, typename TapT<WPROJ>::type *tv,
                                                unsigned long long *bar) {
  typedef typename TapT<WPROJ>::type tap_t;
  const int tid = threadIdx.x;
  if (tid >= a.V) return;
  const int4 h1 = *reinterpret_cast<const int4 *>(&recs[tid].g);  // g, valid, fu, fv
  if (tid < nv && h1.y) {
    const tap_t *table = reinterpret_cast<const tap_t *>(a.conv_w);
    const unsigned bu = (unsigned)(sizeof(tap_t) * TUS), bv = (unsigned)(sizeof(tap_t) * TVS);
    bar_arrive_tx(bar, bu + bv);
    bulk_copy(tu + tid * TUS, table + h1.z, bu, bar);
    bulk_copy(tv + tid * TVS, table + h1.w, bv, bar);
  } else {
    bar_arrive(bar);
  }
}

// Normalisation without precomputed row sums (the allocation-free entry), four lanes per staged
// visibility: Re(sum_u k_u * sum_v k_v) x weight x flag (loop bounds are warp-uniform so the
// shuffles always see full warps); lane 4i owns the running sums of staged slot i.
template <int NC, bool WPROJ>
__device__ __forceinline__ void norm_from_taps(const GridArgs &a, const VisRec<NC> *recs, int nv, int TUS, int TVS,
                                               const typename TapT<WPROJ>::type *tu,
                                               const typename TapT<WPROJ>::type *tv, NormAcc *s_nacc, int *s_ng,
                                               long long fslice) {
  const int W = a.W;
  const int tid = threadIdx.x;
  for (int b4 = tid & ~31; b4 < 4 * nv; b4 += blockDim.x) {
    const int q = b4 + (tid & 31);
    const int vi = q >> 2, part = q & 3;
    const bool act = vi < nv;
    // tap sums in the library's working precision (FP64 units are scarce on this GPU)
    acc_real sur = 0, sui = 0, svr = 0, svi = 0;
    if (act) {
      if (WPROJ) {
        const cplx *pu = reinterpret_cast<const cplx *>(tu) + vi * TUS;
        const cplx *pv = reinterpret_cast<const cplx *>(tv) + vi * TVS;
        for (int j = part; j < W; j += 4) { sur += pu[j].re; sui += pu[j].im; svr += pv[j].re; svi += pv[j].im; }
      } else {
        const acc_real *pu = reinterpret_cast<const acc_real *>(tu) + vi * TUS;
        const acc_real *pv = reinterpret_cast<const acc_real *>(tv) + vi * TVS;
        for (int j = part; j < W; j += 4) { sur += pu[j]; svr += pv[j]; }
      }
    }
#pragma unroll
    for (int off = 1; off < 4; off <<= 1) {
      sur += __shfl_xor_sync(0xffffffffu, sur, off);
      sui += __shfl_xor_sync(0xffffffffu, sui, off);
      svr += __shfl_xor_sync(0xffffffffu, svr, off);
      svi += __shfl_xor_sync(0xffffffffu, svi, off);
    }
    if (act && part == 0 && recs[vi].valid) {
      const VisRec<NC> &r = recs[vi];
      const NormTerm nt = (NormTerm)sur * (NormTerm)svr - (NormTerm)sui * (NormTerm)svi;
      NormAcc *na = s_nacc + vi * NC;
      if (s_ng[vi] != r.g) {
        if (s_ng[vi] >= 0) {
#pragma unroll
          for (int k = 0; k < NC; ++k)
            if (norm_value(na[k]) != 0.0) atomicAdd(&a.norm[(fslice + s_ng[vi]) * NC + k], norm_value(na[k]));
        }
#pragma unroll
        for (int k = 0; k < NC; ++k) norm_zero(na[k]);
        s_ng[vi] = r.g;
      }
#pragma unroll
      for (int k = 0; k < NC; ++k) norm_add(na[k], (NormTerm)r.cw[k] * nt);
    }
  }
}

// Multiply-adds of a staged chunk's runs into an owner thread's cells.  When the footprint moves,
// the owned cells are recomputed and those that changed are flushed (queued for the warp's
// compensated flush in single precision; the queue is drained when it fills and at the end of the
// track).  Every lane of a warp with any owned cell calls this, so the queue drains are
// warp-uniform.
template <int NC, bool WPROJ, int J, bool COMP, class Rec>
__device__ __forceinline__ void grid_runs(const GridArgs &a, const Rec *recs,
                                          const typename TapT<WPROJ>::type *tu,
                                          const typename TapT<WPROJ>::type *tv, const int *runs, int nruns,
                                          int TUS, int TVS, int du, int strip, unsigned rows_mask, long long fbase,
                                          long long nxy, int gnx, FlushRec<NC> *fq, int *fqn,
                                          OwnerState<NC, J> &st) {
  typedef typename TapT<WPROJ>::type tap_t;
  const int W = a.W;
  for (int ri = 0; ri < nruns; ++ri) {
    const int rs = runs[ri], re = runs[ri + 1];
    const int4 h0 = *reinterpret_cast<const int4 *>(&recs[rs].u0);
    const int4 h1 = *reinterpret_cast<const int4 *>(&recs[rs].g);
    if (!h1.y) continue;
    if (h0.x != st.pu0 || h0.y != st.pv0 || h1.x != st.cg) {
      // footprint moved: recompute the owned cells, flush those that changed
      int o = du - h0.z;
      o += (o < 0) ? W : 0;
      int nov0 = strip * J - h0.w;
      nov0 += (nov0 < 0) ? W : 0;
      if (h0.x + o != st.pu0 + st.ou || h1.x != st.cg) {
        if (st.dirty) {
#pragma unroll
          for (int j = 0; j < J; ++j)
            if (st.dirty & (1u << j)) {
              const int oy = st.ov0 + j >= W ? st.ov0 + j - W : st.ov0 + j;
              if (COMP)
                queue_cell<NC>(a, fbase + (long long)st.cg * NC * nxy, nxy, gnx, st.pu0 + st.ou, st.pv0 + oy,
                               st.acc[j], fq, fqn);
              else
                flush_cell<NC, false>(a, fbase + (long long)st.cg * NC * nxy, nxy, gnx, st.pu0 + st.ou,
                                      st.pv0 + oy, st.acc[j]);
            }
          st.dirty = 0;
        }
        st.cg = h1.x;
      }
      if (st.dirty) {
#pragma unroll
        for (int j = 0; j < J; ++j) {
          const int oy = st.ov0 + j >= W ? st.ov0 + j - W : st.ov0 + j;
          const int ny = nov0 + j >= W ? nov0 + j - W : nov0 + j;
          if ((st.dirty & (1u << j)) && h0.y + ny != st.pv0 + oy) {
            if (COMP)
              queue_cell<NC>(a, fbase + (long long)st.cg * NC * nxy, nxy, gnx, st.pu0 + st.ou, st.pv0 + oy,
                             st.acc[j], fq, fqn);
            else
              flush_cell<NC, false>(a, fbase + (long long)st.cg * NC * nxy, nxy, gnx, st.pu0 + st.ou, st.pv0 + oy,
                                    st.acc[j]);
            st.dirty &= ~(1u << j);
          }
        }
      }
      // columns beyond W (padding lanes) read in-bounds taps and are never flushed
      st.ou = o < W ? o : W - 1;
      st.ov0 = nov0 < W ? nov0 : 0;  // lanes past the last strip own nothing: keep their reads in bounds
      st.pu0 = h0.x;
      st.pv0 = h0.y;
      if (COMP) {  // the queue only grows here; the branch is uniform over the warp
        __syncwarp();
        if (*fqn >= kDrainAt) drain_queue<NC>(a, nxy, fq, fqn);
      }
    }
    // the run's visibilities share the owned cells: a branch-free multiply-add loop over the J
    // owned rows (offsets modulo W; rows of non-owning lanes stay in bounds and are never flushed)
#pragma unroll 2
    for (int vi = rs; vi < re; ++vi) {
      const tap_t tuv = tu[vi * TUS + st.ou];
      cplx pre[NC];
#pragma unroll
      for (int k = 0; k < NC; ++k) pre[k] = premul(recs[vi].vis[k], tuv);
      const tap_t *tvrow = tv + vi * TVS + st.ov0;
#pragma unroll
      for (int j = 0; j < J; ++j) {
        const tap_t t = tvrow[j];
#pragma unroll
        for (int k = 0; k < NC; ++k) mac(st.acc[j][k], pre[k], t);
      }
    }
    st.dirty = rows_mask;
  }
}

// One track (facet, channel, rows [r0, r1)) of one CTA: the rows are staged V at a time (prologue,
// runs, taps) and gridded by the Romein owner threads.  With a tap-copy barrier (`bar`, whose
// phase parity `phase` carries over from track to track) and the support-window table, a staged
// visibility's tap rows are two bulk copies; otherwise per-tap asynchronous copies.
template <int NC, bool WPROJ, int J, bool COMP, bool WIDE>
__device__ __forceinline__ void grid_track(const GridArgs &a, const int f_local, const int chan, long long r0,
                                           long long r1, unsigned long long *bar, unsigned &phase) {
  typedef typename TapT<WPROJ>::type tap_t;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int V = a.V, W = a.W;
  const int TUS = tap_row_u<WPROJ>(W), TVS = tap_row_v<WPROJ>(W, J);  // staged row strides
  const bool bulk = bar != nullptr && a.conv_w != nullptr;
  VisRec<NC> *recs = reinterpret_cast<VisRec<NC> *>(smem_raw);                          // [V]
  NormAcc *s_nacc = reinterpret_cast<NormAcc *>(smem_raw + sizeof(VisRec<NC>) * (size_t)V);  // [V][NC]
  int *s_ng = reinterpret_cast<int *>(s_nacc + (size_t)V * NC);                             // [V]
  int *s_runs = s_ng + V;                                                                   // [V + 1]
  tap_t *tu = reinterpret_cast<tap_t *>(smem_raw + stage_head_bytes<NC>(V));               // [V][TUS]
  tap_t *tv = tu + V * TUS;                                                                 // [V][TVS]
  // per-warp flush queues follow the taps
  unsigned char *qbase = reinterpret_cast<unsigned char *>(tv + V * TVS);
  qbase = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(qbase) + 15) & ~(uintptr_t)15);
  const int warp_id = threadIdx.x >> 5, nwarps = (blockDim.x + 31) >> 5;
  FlushRec<NC> *fq = reinterpret_cast<FlushRec<NC> *>(qbase) + warp_id * kFlushQueueCap;
  int *fqn = reinterpret_cast<int *>(qbase + nwarps * sizeof(FlushRec<NC>) * kFlushQueueCap) + warp_id * 4;
  if (COMP && (threadIdx.x & 31) == 0) *fqn = 0;
  __shared__ int s_nruns;

  const FacetXform &fxt = a.facets[f_local];
  const int gnx = fxt.nx;
  const long long nxy = (long long)fxt.nx * fxt.ny;
  const long long fbase = fxt.grid_base;  // element offset of this facet's grid block
  if (r1 > a.nrows) r1 = a.nrows;
  if (r0 >= r1) return;

  const int tid = threadIdx.x;
  int du, strip;
  bool owner;
  owner_map<WIDE>(tid, W, J, du, strip, owner);
  unsigned rows_mask = 0;
#pragma unroll
  for (int j = 0; j < J; ++j)
    if (strip * J + j < W) rows_mask |= 1u << j;
  if (!owner) rows_mask = 0;
  const bool grids = __any_sync(0xffffffffu, rows_mask != 0);
  const long long fslice = (long long)(a.facet_base + f_local) * a.groups;
  const bool want_norm = a.norm != nullptr;
  if (want_norm && tid < V) {
#pragma unroll
    for (int k = 0; k < NC; ++k) norm_zero(s_nacc[tid * NC + k]);
    s_ng[tid] = -1;
  }

  OwnerState<NC, J> st;
#pragma unroll
  for (int j = 0; j < J; ++j) {
#pragma unroll
    for (int k = 0; k < NC; ++k) { st.acc[j][k].re = 0; st.acc[j][k].im = 0; }
  }
  st.dirty = 0;
  st.cg = -1;
  st.pu0 = -1;
  st.pv0 = -1;
  st.ou = 0;
  st.ov0 = 0;
  ChanCache cc;
  const double plane_scale = WPROJ ? (double)(a.P - 1) / a.wmax : 0.0;

  for (long long base = r0; base < r1; base += V) {
    const int nv = (int)min((long long)V, r1 - base);
    if (tid < V) stage_slot<NC, WPROJ>(a, f_local, chan, base + tid, tid < nv, tid, recs, cc, plane_scale);
    __syncthreads();
    if (bulk)
      stage_taps_bulk<NC, WPROJ>(a, recs, nv, TUS, TVS, tu, tv, bar);
    else
      stage_taps<NC, WPROJ>(a, recs, nv, J, TUS, TVS, tu, tv);
    if (warp_id == 0) find_runs(recs, nv, s_runs, &s_nruns);
    if (want_norm && a.tap_sums && tid < nv) norm_slot<NC>(a, recs[tid], tid, s_nacc, s_ng, fslice);
    if (bulk) {
      // every thread observes the phase (the copies' data is visible to the threads that do);
      // a wait that runs out is recorded, then waited for once more before the data is used
      if (!bar_wait(bar, phase)) {
        atomicOr(a.error, DEV_ERR_WAIT_TIMEOUT);
        bar_wait(bar, phase);
      }
      phase ^= 1u;
    } else {
      wait_taps();
    }
    __syncthreads();
    if (want_norm && !a.tap_sums) norm_from_taps<NC, WPROJ>(a, recs, nv, TUS, TVS, tu, tv, s_nacc, s_ng, fslice);
    if (grids)
      grid_runs<NC, WPROJ, J, COMP>(a, recs, tu, tv, s_runs, s_nruns, TUS, TVS, du, strip, rows_mask, fbase, nxy, gnx,
                                    fq, fqn, st);
    __syncthreads();
  }
  // the flush queues carry over from chunk to chunk; empty them before the final flush
  if (COMP && grids) drain_queue<NC>(a, nxy, fq, fqn);
  // final flush of owned cells
  if (st.dirty) {
#pragma unroll
    for (int j = 0; j < J; ++j) {
      const int oy = st.ov0 + j >= W ? st.ov0 + j - W : st.ov0 + j;
      if (st.dirty & (1u << j))
        flush_cell<NC, COMP>(a, fbase + (long long)st.cg * NC * nxy, nxy, gnx, st.pu0 + st.ou, st.pv0 + oy, st.acc[j]);
    }
  }
  // normalisation: the slots' current partial sums (earlier grid groups went out when the group
  // changed), summed over each warp by shuffles when its slots share one group (one atomic per
  // correlation and warp), added slot by slot otherwise.  The slots' state was last written before
  // the chunk loop's final barrier.
  if (want_norm) {
    const bool has = tid < V && s_ng[tid] >= 0;
    const int my_g = has ? s_ng[tid] : -1;
    const unsigned m = __ballot_sync(0xffffffffu, has);
    if (m) {
      const int g0 = __shfl_sync(0xffffffffu, my_g, __ffs(m) - 1);
      const NormAcc *na = s_nacc + (has ? tid : 0) * NC;
      if (__all_sync(0xffffffffu, !has || my_g == g0)) {
#pragma unroll
        for (int k = 0; k < NC; ++k) {
          double v = has ? norm_value(na[k]) : 0.0;
#pragma unroll
          for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
          if ((tid & 31) == 0 && v != 0.0) atomicAdd(&a.norm[(fslice + g0) * NC + k], v);
        }
      } else if (has) {
#pragma unroll
        for (int k = 0; k < NC; ++k)
          if (norm_value(na[k]) != 0.0) atomicAdd(&a.norm[(fslice + my_g) * NC + k], norm_value(na[k]));
      }
    }
  }
}

// One work item from precomputed records: its n records (src, 16-byte aligned) are staged V at a
// time by one bulk copy each into two buffers used in turn, the next chunk's copy in flight while
// the current chunk's taps arrive and its runs are gridded; the tap rows are bulk copies as in
// grid_track.  No prologue and no normalisation here (the record kernel did both).  rbar are the
// two record barriers (one arrival each), rphase their phase parities (bit b for buffer b); a
// copy is only issued for a chunk of this item, so none is in flight when the item ends.
template <int NC, bool WPROJ, int J, bool COMP, bool WIDE>
__device__ __forceinline__ void grid_track_pre(const GridArgs &a, const int f_local, const GridRec<NC> *src, int n,
                                               unsigned long long *rbar, unsigned &rphase, unsigned long long *bar,
                                               unsigned &phase) {
  typedef typename TapT<WPROJ>::type tap_t;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int V = a.V, W = a.W;
  const int TUS = tap_row_u<WPROJ>(W), TVS = tap_row_v<WPROJ>(W, J);
  GridRec<NC> *rb = reinterpret_cast<GridRec<NC> *>(smem_raw);  // [2][V]
  int *s_runs = reinterpret_cast<int *>(rb + 2 * V);             // [V + 1]
  tap_t *tu = reinterpret_cast<tap_t *>(smem_raw + stage_head_bytes<NC>(V));
  tap_t *tv = tu + V * TUS;
  unsigned char *qbase = reinterpret_cast<unsigned char *>(tv + V * TVS);
  qbase = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(qbase) + 15) & ~(uintptr_t)15);
  const int warp_id = threadIdx.x >> 5, nwarps = (blockDim.x + 31) >> 5;
  FlushRec<NC> *fq = reinterpret_cast<FlushRec<NC> *>(qbase) + warp_id * kFlushQueueCap;
  int *fqn = reinterpret_cast<int *>(qbase + nwarps * sizeof(FlushRec<NC>) * kFlushQueueCap) + warp_id * 4;
  if (COMP && (threadIdx.x & 31) == 0) *fqn = 0;
  __shared__ int s_nruns_pre;
  if (n <= 0) return;

  const FacetXform &fxt = a.facets[f_local];
  const int gnx = fxt.nx;
  const long long nxy = (long long)fxt.nx * fxt.ny;
  const long long fbase = fxt.grid_base;
  const int tid = threadIdx.x;
  int du, strip;
  bool owner;
  owner_map<WIDE>(tid, W, J, du, strip, owner);
  unsigned rows_mask = 0;
#pragma unroll
  for (int j = 0; j < J; ++j)
    if (strip * J + j < W) rows_mask |= 1u << j;
  if (!owner) rows_mask = 0;
  const bool grids = __any_sync(0xffffffffu, rows_mask != 0);

  OwnerState<NC, J> st;
#pragma unroll
  for (int j = 0; j < J; ++j) {
#pragma unroll
    for (int k = 0; k < NC; ++k) { st.acc[j][k].re = 0; st.acc[j][k].im = 0; }
  }
  st.dirty = 0;
  st.cg = -1;
  st.pu0 = -1;
  st.pv0 = -1;
  st.ou = 0;
  st.ov0 = 0;

  const int nchunks = (n + V - 1) / V;
  if (tid == 0) {
    // the buffers may last have been written by plain stores (an item prepared in place)
    fence_proxy_async();
    const unsigned bytes = (unsigned)(sizeof(GridRec<NC>) * (size_t)min(V, n));
    bar_arrive_tx(&rbar[0], bytes);
    bulk_copy(rb, src, bytes, &rbar[0]);
  }
  int cur = 0;
  for (int c = 0; c < nchunks; ++c, cur ^= 1) {
    const int nv = min(V, n - c * V);
    const unsigned par = (rphase >> cur) & 1u;
    if (!bar_wait(&rbar[cur], par)) {
      atomicOr(a.error, DEV_ERR_WAIT_TIMEOUT);
      bar_wait(&rbar[cur], par);
    }
    rphase ^= 1u << cur;
    const GridRec<NC> *recs = rb + cur * V;
    stage_taps_bulk<NC, WPROJ>(a, recs, nv, TUS, TVS, tu, tv, bar);
    if (tid == 0 && c + 1 < nchunks) {
      // the other buffer was last read by the previous chunk, which every thread has finished
      const unsigned bytes = (unsigned)(sizeof(GridRec<NC>) * (size_t)min(V, n - (c + 1) * V));
      fence_proxy_async();
      bar_arrive_tx(&rbar[cur ^ 1], bytes);
      bulk_copy(rb + (cur ^ 1) * V, src + (size_t)(c + 1) * V, bytes, &rbar[cur ^ 1]);
    }
    if (warp_id == 0) find_runs(recs, nv, s_runs, &s_nruns_pre);
    if (!bar_wait(bar, phase)) {
      atomicOr(a.error, DEV_ERR_WAIT_TIMEOUT);
      bar_wait(bar, phase);
    }
    phase ^= 1u;
    __syncthreads();
    if (grids)
      grid_runs<NC, WPROJ, J, COMP>(a, recs, tu, tv, s_runs, s_nruns_pre, TUS, TVS, du, strip, rows_mask, fbase, nxy,
                                    gnx, fq, fqn, st);
    __syncthreads();
  }
  if (COMP && grids) drain_queue<NC>(a, nxy, fq, fqn);
  if (st.dirty) {
#pragma unroll
    for (int j = 0; j < J; ++j) {
      const int oy = st.ov0 + j >= W ? st.ov0 + j - W : st.ov0 + j;
      if (st.dirty & (1u << j))
        flush_cell<NC, COMP>(a, fbase + (long long)st.cg * NC * nxy, nxy, gnx, st.pu0 + st.ou, st.pv0 + oy, st.acc[j]);
    }
  }
}

// Default register budget of the persistent segment kernel: the J = 4 layout (32 accumulator
// registers) is capped at 80 registers per thread so that more warps stay resident; J = 8 keeps the
// 128 that 512 threads allow.  The w-projection visibility launches also offer J = 4 builds at 64 and
// 72 registers to the tuner (different support classes prefer different caps).
template <int J>
constexpr int kSegRegs = J == 4 ? 80 : 128;
// the J = 6 layout of the single-precision w-projection visibility launches
constexpr int kSegRegs6 = 96;

// One CTA per track: blockIdx -> (facet, baseline slot or row segment, channel).
template <int NC, bool WPROJ, int J, bool COMP, bool WIDE>
__global__ void __launch_bounds__(512, 1) romein_grid_kernel(const GridArgs a) {
  long long track = blockIdx.x;
  const int chan = (int)(track % a.nchan);
  track /= a.nchan;
  const int slot = (int)(track % a.nslots);
  const int f_local = (int)(track / a.nslots);
  long long r0, r1;
  if (a.starts) {
    r0 = (long long)a.starts[slot];
    r1 = (long long)a.starts[slot + 1];
  } else {
    r0 = (long long)slot * a.seg;
    r1 = min(a.nrows, r0 + a.seg);
  }
  unsigned phase = 0;
  grid_track<NC, WPROJ, J, COMP, WIDE>(a, f_local, chan, r0, r1, nullptr, phase);
}

// Persistent form: a fixed grid of CTAs takes (segment, facet) work items from a device counter
// until the device-side item count is exhausted; every segment is a run of one track's rows
// whose w planes share this launch's support class (a.W).  Items of one segment are adjacent, so
// the facets of a segment are gridded while its rows are hot in L2.  The loop ends on the count,
// never waits on other CTAs.  The tap-copy barrier is set up once (V arrivals per phase).
template <int NC, bool WPROJ, int J, bool COMP, bool WIDE, int REGS = kSegRegs<J>>
__global__ void __launch_bounds__(512, 1) __maxnreg__(REGS) romein_segment_kernel(const GridArgs a, const int nfacets) {
  __shared__ int s_item;
  __shared__ int s_first, s_last;  // unmasked row range of the item (facet row masks)
  __shared__ __align__(8) unsigned long long s_tap_bar;
  __shared__ __align__(8) unsigned long long s_rec_bar[2];
  unsigned phase = 0, rphase = 0;
  if (threadIdx.x == 0) {
    bar_init(&s_tap_bar, (unsigned)a.V);
    bar_init(&s_rec_bar[0], 1);
    bar_init(&s_rec_bar[1], 1);
  }
  const int count = *a.work_count;
  const long long total = (long long)count * nfacets;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) {
      s_item = atomicAdd(a.work_next, 1);
      s_first = 0x7fffffff;
      s_last = -1;
    }
    __syncthreads();
    const long long item = s_item;
    if (item >= total) break;
    const int seg = (int)(item / nfacets);
    const int f_local = (int)(item - (long long)seg * nfacets);
    const long long si = (long long)*a.segment_base + seg;
    if (si < 0 || si >= a.segment_capacity) {  // schedule out of range: record and stop
      if (threadIdx.x == 0) atomicOr(a.error, DEV_ERR_GRID_INDEX);
      break;
    }
    const int4 sg = a.segments[si];
    if (sg.x < 0 || sg.x > sg.y || (long long)sg.y > a.nrows || sg.z < 0 || sg.z >= a.nchan) {
      if (threadIdx.x == 0) atomicOr(a.error, DEV_ERR_GRID_INDEX);
      continue;
    }
    if (a.records) {
      // records of this item, when the record kernel had room for its segment: only the item's
      // first to last valid record (all of them past the range table)
      const long long len = (long long)sg.y - sg.x;
      const long long first = a.rec_off[si] * nfacets;
      if ((a.rec_off[si] + len) * nfacets <= a.rec_capacity) {
        const long long it = si * nfacets + f_local;
        int lo = 0, hi = (int)len;
        if (it < a.range_capacity) {
          const int2 rg = a.item_range[it];
          lo = rg.x;
          hi = rg.y;
        }
        if (lo < hi) {
          const GridRec<NC> *src =
              reinterpret_cast<const GridRec<NC> *>(a.records) + first + (long long)f_local * len + lo;
          grid_track_pre<NC, WPROJ, J, COMP, WIDE>(a, f_local, src, hi - lo, s_rec_bar, rphase, &s_tap_bar, phase);
        }
        continue;
      }
    }
    long long r0 = sg.x, r1 = sg.y;
    if (a.facet_row_mask) {
      // a facet that leaves rows out grids only the item's first to last row it keeps, and skips
      // the item when it keeps none (the rows in between are still tested in the prologue)
      const uint8_t *m = a.facet_row_mask + (long long)(a.facet_base + f_local) * a.nrows;
      int first = 0x7fffffff, last = -1;
      for (int r = sg.x + (int)threadIdx.x; r < sg.y; r += (int)blockDim.x)
        if (m[r]) {
          first = min(first, r);
          last = max(last, r);
        }
      if (last >= 0) {
        atomicMin(&s_first, first);
        atomicMax(&s_last, last);
      }
      __syncthreads();
      if (s_last < 0) continue;  // uniform: every thread reads the same shared values
      r0 = s_first;
      r1 = (long long)s_last + 1;
    }
    grid_track<NC, WPROJ, J, COMP, WIDE>(a, f_local, sg.z, r0, r1, &s_tap_bar, phase);
  }
}

}  // namespace bz
