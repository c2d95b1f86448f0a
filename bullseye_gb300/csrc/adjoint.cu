// Adjoint of facet gridding (a degridder): gradients of a real loss with respect to the
// visibilities and the per-antenna 2x2 Jones terms, given the gradient with respect to the grids.
//
// Forward (per facet f, visibility (row, channel), correlation c, footprint cell (x, y)):
//   M   = J_p^-1 V J_q^-H                       (Jones correction, 2x2)
//   V'  = s M,  s = weight x flag x e^{i phi_f} (phase rotation to the facet centre)
//   y   = V' (w >= 0) or conj(V') (w < 0, gridded at (-u, -v))
//   G  += y tap(x - u0, y - v0)
// With the real-inner-product convention dL = Re <g_z, dz> (torch's complex gradient):
//   g_y  = sum over the footprint of g_G conj(tap)         (a gather: no atomics)
//   g_V' = g_y or conj(g_y)
//   g_M  = conj(s) g_V'
//   g_V  = P^H g_M Q                                      (P = J_p^-1, Q = J_q^-1)
//   g_Jp = -P^H g_M M^H,   g_Jq = -Q^H g_M^H M            (d(J^-1) = -J^-1 dJ J^-1)
// Cells, taps, w plane and phase come from the gridder's own choose_cells (floor for 1-D AA
// kernels, round-half-even for w-projection, full-support acceptance), so the adjoint reads exactly
// the footprint the gridder wrote.  The normalisation sums depend only on weights and taps, so they
// carry no gradient.
//
// Prediction (bullseye_predict) is the physical forward model of the same measurement, on the same
// gather: from model grids G_f (the model images divided by the gridding correction, transformed
// with the reference's shifts, or given as grids),
//   D   = sum over the footprint of G_f conj(tap)            [/ Re sum tap: the normalised form of
//                                                              the reference's prototype degridder,
//                                                              Resampling.ipynb cell 17]
//   V'  = D (w >= 0) or conj(D) (w < 0),   M = e^{-i phi_f} V'
//   V  += J_p M J_q^H   (the gains applied forward; no weights, no flags), summed over facets.
//
// Work layout: a warp takes 32 (row, channel) items; each lane resolves its own item's Jones terms
// and geometry, the warp gathers the footprints item by item with every lane, and shuffles reduce
// each item's sums into its lane.  The visibility result (summed over facets) is written once;
// Jones gradients are accumulated with atomics because every antenna appears on many baselines.
#include <cufft.h>

#include <cstring>
#include <map>
#include <mutex>
#include <tuple>

#include "common.h"
#include "gridder.cuh"

using namespace bz;

namespace {

struct AdjointArgs {
  const vis_complex *vis;
  const vis_real *weights;
  const uint8_t *flags;
  const vis_real *uvw;
  const uint8_t *flagged_rows;
  const unsigned *field;
  const unsigned *spw;
  const unsigned *ant1, *ant2;
  const size_t *time_ids;
  const vis_complex *jones;  // raw terms [T][A][F][S][Ch][4], or null (no correction)
  const vis_real *wavelengths;
  const uint8_t *enabled;
  const size_t *cgi;
  const void *conv;
  const vis_real *facet_centres;  // [F][2] arcsec, or null (no faceting)
  const vis_complex *grad_grid;   // [F][cube][4][ny][nx], or [F][cube][ny][nx][4] with grid_interleaved
  vis_complex *grad_vis;          // [R][Ch][4]
  vis_complex *grad_jones;        // like jones, accumulated; or null
  long long nrows;
  int nchan, nspw, nant, ntimes, nfacets, cube, nx, ny, W, os, K, P, faceting;
  int normalise;  // prediction: divide each facet's gathered value by the real part of its tap sum
  int grid_interleaved;  // prediction from its own model grids: a cell's 4 correlations are adjacent
  unsigned imaging_field;
  double u_scale, v_scale, gcx, gcy, wmax, ra0, dec0;
};

// Dynamic shared memory of the gather kernel: the facet transforms, the w planes' windows, then
// (16-byte aligned) each warp's staged taps.
__host__ __device__ inline size_t degrid_taps_offset(int nfacets, int P) {
  return (sizeof(FacetXform) * (size_t)nfacets + sizeof(int2) * (size_t)P + 15) / 16 * 16;
}

// The 4 adjacent correlations of one cell (32 bytes in single precision, 16-byte aligned): two
// 16-byte loads.
__device__ __forceinline__ void load_cell4(const vis_complex *p, cplx out[4]) {
#if defined(BULLSEYE_SINGLE)
  const float4 a = *reinterpret_cast<const float4 *>(p), b = *reinterpret_cast<const float4 *>(p + 2);
  out[0].re = a.x; out[0].im = a.y;
  out[1].re = a.z; out[1].im = a.w;
  out[2].re = b.x; out[2].im = b.y;
  out[3].re = b.z; out[3].im = b.w;
#else
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    out[k].re = p[k].re;
    out[k].im = p[k].im;
  }
#endif
}

__device__ __forceinline__ cplx cconj(cplx a) {
  a.im = -a.im;
  return a;
}
__device__ __forceinline__ cplx cadd(cplx a, cplx b) {
  a.re += b.re;
  a.im += b.im;
  return a;
}
// 2x2 products with optional hermitian transposes: O = op(A) op(B)
__device__ __forceinline__ void mat2(const cplx *A, bool ha, const cplx *B, bool hb, cplx *O) {
  cplx a[4], b[4];
  if (ha) { a[0] = cconj(A[0]); a[1] = cconj(A[2]); a[2] = cconj(A[1]); a[3] = cconj(A[3]); }
  else { a[0] = A[0]; a[1] = A[1]; a[2] = A[2]; a[3] = A[3]; }
  if (hb) { b[0] = cconj(B[0]); b[1] = cconj(B[2]); b[2] = cconj(B[1]); b[3] = cconj(B[3]); }
  else { b[0] = B[0]; b[1] = B[1]; b[2] = B[2]; b[3] = B[3]; }
  jmul(a, b, O);
}

__device__ __forceinline__ bool inv2(cplx *m) {
  cplx det;
  det.re = (m[0].re * m[3].re - m[0].im * m[3].im) - (m[1].re * m[2].re - m[1].im * m[2].im);
  det.im = (m[0].re * m[3].im + m[0].im * m[3].re) - (m[1].re * m[2].im + m[1].im * m[2].re);
  if (det.re == (acc_real)0 && det.im == (acc_real)0) return false;
  const acc_real n2 = det.re * det.re + det.im * det.im;
  cplx inv;
  inv.re = det.re / n2;
  inv.im = -det.im / n2;
  cplx neg;
  neg.re = -inv.re;
  neg.im = -inv.im;
  const cplx a0 = m[0];
  m[0] = cmul(m[3], inv);
  m[3] = cmul(a0, inv);
  m[1] = cmul(m[1], neg);
  m[2] = cmul(m[2], neg);
  return true;
}

template <bool WPROJ>
__device__ __forceinline__ cplx tap_at(const void *conv, long long idx) {
  cplx t;
  if (WPROJ) {
    const vis_complex c = ((const vis_complex *)conv)[idx];
    t.re = (acc_real)c.re;
    t.im = (acc_real)c.im;
  } else {
    t.re = (acc_real)((const vis_real *)conv)[idx];
    t.im = 0;
  }
  return t;
}

__device__ __forceinline__ void atomic_add_c(vis_complex *dst, cplx v) {
  atomicAdd(&dst->re, (vis_real)v.re);
  atomicAdd(&dst->im, (vis_real)v.im);
}

// PREDICT = false: the adjoint (grad_grid -> grad_vis, grad_jones).  PREDICT = true: prediction
// (model grids in grad_grid -> visibilities in grad_vis).
template <bool WPROJ, bool PREDICT>
__global__ void __launch_bounds__(256) degrid_adjoint_kernel(const AdjointArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  FacetXform *fx = reinterpret_cast<FacetXform *>(smem_raw);
  for (int f = threadIdx.x; f < a.nfacets; f += blockDim.x) {
    double ra = a.ra0, dec = a.dec0;
    if (a.faceting && a.facet_centres) {
      ra = (double)a.facet_centres[2 * f];
      dec = (double)a.facet_centres[2 * f + 1];
    }
    // same constants as the gridder (phase_transform_policies.h:110-134, baseline_transform_policies.h:117-149)
    const double k = (double)kArcsecToRad;
    double d_ra = (ra - a.ra0) * k, n_dec = dec * k, o_dec = a.dec0 * k;
    double c_d_ra = cos(d_ra), s_d_ra = sin(d_ra), c_n = cos(n_dec), s_n = sin(n_dec), c_o = cos(o_dec), s_o = sin(o_dec);
    FacetXform x;
    memset(&x, 0, sizeof x);
    if (a.faceting) {
      double li0 = c_n * s_d_ra, mi0 = s_n * c_o - c_n * s_o * c_d_ra, ni0 = s_n * s_o + c_n * c_o * c_d_ra;
      x.u_term = li0 / ni0;
      x.v_term = mi0 / ni0;
      x.dl = -c_n * s_d_ra;
      x.dm = -(s_n * c_o - c_n * s_o * c_d_ra);
      x.dn = 1.0 - sqrt(1.0 - x.dl * x.dl - x.dm * x.dm);
    }
    fx[f] = x;
  }
  // nonzero window [lo, hi] of every w plane's kernel row, one warp per plane: a footprint cell s
  // reads sample fu + s*os with fu in [floor(os/2), floor(3 os/2)] (w-projection, round to nearest)
  // or [0, os] (AA, floor); cells that cannot reach a nonzero sample carry a zero tap and are skipped
  int2 *win = reinterpret_cast<int2 *>(smem_raw + sizeof(FacetXform) * a.nfacets);
  {
    const int ln = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int fu_min = WPROJ ? (int)floor(0.5 * a.os - 1e-6) : 0;
    const int fu_max = WPROJ ? (int)floor(1.5 * a.os + 1e-6) : a.os;
    for (int pl = wid; pl < a.P; pl += nw) {
      int lo = 0x7fffffff, hi = -1;
      for (int i = ln; i < a.K; i += 32) {
        const cplx t = tap_at<WPROJ>(a.conv, (long long)pl * a.K + i);
        if (t.re != (acc_real)0 || t.im != (acc_real)0) {
          lo = min(lo, i);
          hi = max(hi, i);
        }
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, off));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, off));
      }
      if (ln == 0) {
        int2 w2 = make_int2(0, -1);  // empty window: an all-zero row
        if (hi >= 0) {
          w2.x = max(0, (int)ceil((double)(lo - fu_max) / a.os));
          w2.y = min(a.W - 1, (int)floor((double)(hi - fu_min) / a.os));
        }
        win[pl] = w2;
      }
    }
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  // this warp's staged column and row taps of the item it gathers ([2][W])
  cplx *s_taps = reinterpret_cast<cplx *>(smem_raw + degrid_taps_offset(a.nfacets, a.P)) +
                 (size_t)(threadIdx.x >> 5) * 2 * a.W;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  const int W = a.W;
  const long long nxy = (long long)a.nx * a.ny;
  const double plane_scale = WPROJ ? (double)(a.P - 1) / a.wmax : 0.0;
  const bool jones_vec = vec16(a.jones);  // 16-byte loads of the 2x2 terms (every term starts at 4 x 8 bytes)

  // Each warp takes 32 consecutive (row, channel) items at a time.  Lane i does the scalar work
  // of item i: its loads, the FP64 geometry, the Jones inverses and the chain rule.  FP64 and the
  // 2x2 algebra therefore run 32 items per instruction, not one (GB300 issues FP64 at 1/64 of
  // FP32).  The warp then gathers the footprints one item at a time with every lane, and each
  // item's sums land in its own lane.
  const long long total = a.nrows * a.nchan;
  for (long long base0 = warp * 32; base0 < total; base0 += nwarps * 32) {
    const long long item = base0 + lane;
    bool live = item < total;
    long long row = 0, sc = 0;
    int c = 0;
    unsigned spw = 0;
    size_t g = 0;
    if (live) {
      row = item / a.nchan;
      c = (int)(item - row * a.nchan);
      spw = a.spw[row];
      live = spw < (unsigned)a.nspw;
    }
    if (live) {
      sc = (long long)spw * a.nchan + c;
      live = a.enabled[sc] != 0;
    }
    if (live) {
      g = a.cgi[sc];
      live = g < (size_t)a.cube;
    }
    ChanCache cc;
    double um = 0, vm = 0, wm = 0;
    if (live) {
      cc.spw = spw;
      cc.inv = 1.0 / (double)a.wavelengths[sc];
      cc.su = cc.inv * a.u_scale;
      cc.sv = cc.inv * a.v_scale;
      cc.sw = cc.inv * plane_scale;
      um = (double)a.uvw[3 * row];
      vm = (double)a.uvw[3 * row + 1];
      wm = (double)a.uvw[3 * row + 2];
    }
    const long long base = (row * a.nchan + c) * 4;
    cplx gV[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) { gV[k].re = 0; gV[k].im = 0; }

    for (int f = 0; f < a.nfacets; ++f) {
      // this lane's item: Jones indices and the geometry (the gridder's own cell choice: same
      // cells, taps, plane and phase)
      long long i1 = 0, i2 = 0;
      CellChoice cell;
      cell.du = cell.dv = cell.fu = cell.fv = cell.plane = 0;
      cell.flip = false;
      cplx ph;
      ph.re = 1;
      ph.im = 0;
      bool ok = live;
      if (ok && a.jones) {
        const long long t = (long long)a.time_ids[row];
        const unsigned a1 = a.ant1[row], a2 = a.ant2[row];
        if (t < 0 || t >= a.ntimes || a1 >= (unsigned)a.nant || a2 >= (unsigned)a.nant) {
          ok = false;
        } else {
          i1 = ((((t * a.nant + a1) * a.nfacets + f) * a.nspw + spw) * a.nchan + c) * 4;
          i2 = ((((t * a.nant + a2) * a.nfacets + f) * a.nspw + spw) * a.nchan + c) * 4;
        }
      }
      if (ok)
        ok = choose_cells<WPROJ>(um, vm, wm, cc, fx[f], a.faceting != 0, a.faceting != 0, a.u_scale, a.v_scale,
                                 plane_scale, a.gcx, a.gcy, a.nx, a.ny, W, a.P, a.os, ph, cell);
      // gather, item by item: D_k = sum over the footprint of g_G conj(tap)
      cplx myD[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) { myD[k].re = 0; myD[k].im = 0; }
      acc_real myTS = 0;  // prediction: real part of the item's tap sum
      const bool want_ts = PREDICT && a.normalise;
      unsigned todo = __ballot_sync(0xffffffffu, ok);
      while (todo) {
        const int it = __ffs(todo) - 1;
        todo &= todo - 1;
        const int u0 = __shfl_sync(0xffffffffu, cell.du, it), v0 = __shfl_sync(0xffffffffu, cell.dv, it);
        const int plane = __shfl_sync(0xffffffffu, cell.plane, it);
        const long long fu = (long long)plane * a.K + __shfl_sync(0xffffffffu, cell.fu, it);
        const long long fv = (long long)plane * a.K + __shfl_sync(0xffffffffu, cell.fv, it);
        const long long git = __shfl_sync(0xffffffffu, (long long)g, it);
        const long long slice0 = ((long long)f * a.cube + git) * 4;
        const long long cube0 = ((long long)f * a.cube + git) * nxy;  // interleaved layout
        // lane walks the cells lane, lane + 32, ... of the plane's nonzero window as (ju, jv)
        // without division
        const int2 w2 = win[plane];
        const int ww = w2.y - w2.x + 1;
        if (ww <= 0) continue;  // an all-zero kernel row: the item's sums stay zero
        // the item's W column taps and W row taps, once per item instead of once per cell
        for (int j = lane; j < ww; j += 32) {
          s_taps[j] = tap_at<WPROJ>(a.conv, fu + (long long)(w2.x + j) * a.os);
          s_taps[a.W + j] = tap_at<WPROJ>(a.conv, fv + (long long)(w2.x + j) * a.os);
        }
        __syncwarp();
        cplx D[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) { D[k].re = 0; D[k].im = 0; }
        acc_real TS = 0;
        // (ru, rv): the lane's cell relative to the window corner; off: its offset in the grid.
        // The trip count is fixed before the loop, so prediction's loads of consecutive cells
        // overlap (two cells per iteration); the adjoint's four strided slices run one cell at a time.
        const int ncell = ww * ww, sju = 32 % ww, sjv = 32 / ww;
        int ru = lane % ww, rv = lane / ww;
        const long long corner = (long long)(v0 + w2.x) * a.nx + (u0 + w2.x);
        long long off = (long long)rv * a.nx + ru;
        const long long step = (long long)sjv * a.nx + sju, wrap = (long long)a.nx - ww;
#pragma unroll(PREDICT ? 2 : 1)
        for (int idx = lane; idx < ncell; idx += 32) {
          const cplx tap = cmul(s_taps[ru], s_taps[a.W + rv]);
          const cplx ct = cconj(tap);
          if (want_ts) TS += tap.re;
          const long long cidx = corner + off;
          cplx gc[4];
          if (PREDICT && a.grid_interleaved) {
            load_cell4(a.grad_grid + (cube0 + cidx) * 4, gc);
          } else {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              const vis_complex gg = a.grad_grid[(slice0 + k) * nxy + cidx];
              gc[k].re = gg.re;
              gc[k].im = gg.im;
            }
          }
#pragma unroll
          for (int k = 0; k < 4; ++k) D[k] = cadd(D[k], cmul(gc[k], ct));
          ru += sju;
          rv += sjv;
          off += step;
          if (ru >= ww) {  // one wrap at most: sju < ww, or ww > 32 and sju = 32
            ru -= ww;
            ++rv;
            off += wrap;
          }
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
#pragma unroll
          for (int off = 16; off > 0; off >>= 1) {
            D[k].re += __shfl_xor_sync(0xffffffffu, D[k].re, off);
            D[k].im += __shfl_xor_sync(0xffffffffu, D[k].im, off);
          }
        }
        if (want_ts) {
#pragma unroll
          for (int off = 16; off > 0; off >>= 1) TS += __shfl_xor_sync(0xffffffffu, TS, off);
        }
        if (lane == it) {
#pragma unroll
          for (int k = 0; k < 4; ++k) myD[k] = D[k];
          myTS = TS;
        }
        __syncwarp();  // every lane has read the staged taps before the next item's
      }
      if (!ok) continue;
      if (PREDICT) {
        // V' = D or conj(D) (w < 0), normalised by the tap sum; M = e^{-i phi} V'; V += J_p M J_q^H
        const acc_real inv = (want_ts && myTS != (acc_real)0) ? (acc_real)1 / myTS : (acc_real)1;
        const cplx cph = cconj(ph);
        cplx X[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          cplx v = cell.flip ? cconj(myD[k]) : myD[k];
          v.re *= inv;
          v.im *= inv;
          X[k] = cmul(cph, v);
        }
        if (a.jones) {
          cplx Pm[4], Qm[4], T[4], O[4];
          load_c4(a.jones + i1, jones_vec, Pm);
          load_c4(a.jones + i2, jones_vec, Qm);
          mat2(Pm, false, X, false, T);  // J_p M
          mat2(T, false, Qm, true, O);   // (J_p M) J_q^H
#pragma unroll
          for (int k = 0; k < 4; ++k) gV[k] = cadd(gV[k], O[k]);
        } else {
#pragma unroll
          for (int k = 0; k < 4; ++k) gV[k] = cadd(gV[k], X[k]);
        }
        continue;
      }
      // chain rule back to V (and the Jones terms), each lane for its own item
      cplx Pm[4], Qm[4];
      if (a.jones) {
        load_c4(a.jones + i1, jones_vec, Pm);
        load_c4(a.jones + i2, jones_vec, Qm);
        if (!inv2(Pm) || !inv2(Qm)) continue;  // a singular term: no gradient through it
      }
      const bool row_ok = !a.flagged_rows[row] && a.field[row] == a.imaging_field;
      acc_real cw[4];
      bool fl[4];
      load_r4(a.weights + base, vec16(a.weights), cw);
      load_f4(a.flags + base, (reinterpret_cast<uintptr_t>(a.flags) & 3) == 0, fl);
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (!row_ok || fl[k]) cw[k] = (acc_real)0;
      cplx gM[4];
      const cplx cph = cconj(ph);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const cplx gvp = cell.flip ? cconj(myD[k]) : myD[k];
        cplx t = cmul(cph, gvp);
        t.re *= cw[k];
        t.im *= cw[k];
        gM[k] = t;
      }
      if (a.jones) {
        cplx T[4], G1[4];
        mat2(Pm, true, gM, false, T);  // P^H gM
        mat2(T, false, Qm, false, G1);  // (P^H gM) Q
#pragma unroll
        for (int k = 0; k < 4; ++k) gV[k] = cadd(gV[k], G1[k]);
        if (a.grad_jones) {
          cplx V[4];
          load_c4(a.vis + base, vec16(a.vis), V);
          cplx VQ[4], M[4], gp[4], gq[4];
          mat2(V, false, Qm, true, VQ);  // V Q^H
          mat2(Pm, false, VQ, false, M);  // M = P V Q^H
          mat2(T, false, M, true, gp);    // P^H gM M^H
          cplx T2[4];
          mat2(Qm, true, gM, true, T2);   // Q^H gM^H
          mat2(T2, false, M, false, gq);  // Q^H gM^H M
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            gp[k].re = -gp[k].re; gp[k].im = -gp[k].im;
            gq[k].re = -gq[k].re; gq[k].im = -gq[k].im;
            atomic_add_c(a.grad_jones + i1 + k, gp[k]);
            atomic_add_c(a.grad_jones + i2 + k, gq[k]);
          }
        }
      } else {
#pragma unroll
        for (int k = 0; k < 4; ++k) gV[k] = cadd(gV[k], gM[k]);
      }
    }
    if (live) {
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        vis_complex o;
        o.re = (vis_real)gV[k].re;
        o.im = (vis_real)gV[k].im;
        a.grad_vis[base + k] = o;
      }
    }
  }
}

// Arguments shared by the adjoint and the prediction (device pointers, sizes from the struct).
AdjointArgs degrid_args(const gridding_parameters &p, int faceting) {
  AdjointArgs a;
  std::memset(&a, 0, sizeof a);
  a.vis = p.visibilities; a.weights = p.visibility_weights; a.flags = (const uint8_t *)p.flags;
  a.uvw = (const vis_real *)p.uvw_coords; a.flagged_rows = (const uint8_t *)p.flagged_rows;
  a.field = p.field_array; a.spw = p.spw_index_array; a.ant1 = p.antenna_1_ids; a.ant2 = p.antenna_2_ids;
  a.time_ids = p.timestamp_ids; a.jones = p.jones_terms;
  a.wavelengths = p.reference_wavelengths; a.enabled = (const uint8_t *)p.enabled_channels; a.cgi = p.channel_grid_indicies;
  a.conv = p.conv; a.facet_centres = p.facet_centres;
  a.nrows = (long long)p.row_count;
  a.nchan = (int)p.channel_count; a.nspw = (int)p.spw_count; a.nant = (int)p.antenna_count;
  a.ntimes = (int)p.no_timestamps_read;
  a.nfacets = (int)(p.num_facet_centres ? p.num_facet_centres : 1);
  a.cube = (int)p.cube_channel_dim_size;
  a.nx = (int)p.nx; a.ny = (int)p.ny;
  a.W = (int)(2 * p.conv_support + 1);
  a.os = (int)p.conv_oversample;
  a.K = (a.W + 2) + (a.W + 1) * (a.os - 1);
  a.P = (int)(p.wplanes > 1 ? p.wplanes : 1);
  a.faceting = faceting ? 1 : 0;
  a.imaging_field = p.imaging_field;
  a.u_scale = (double)p.nx * (double)p.cell_size_x * (double)kArcsecToRad;
  a.v_scale = -((double)p.ny * (double)p.cell_size_y * (double)kArcsecToRad);
  a.gcx = (double)(p.nx / 2 - p.conv_support);
  a.gcy = (double)(p.ny / 2 - p.conv_support);
  a.wmax = (double)(float)p.wmax_est;
  a.ra0 = (double)p.phase_centre_ra;
  a.dec0 = (double)p.phase_centre_dec;
  return a;
}

// Zeroes the output, then one persistent-style launch of the gather (32 items per warp pass).
template <bool PREDICT>
int launch_degrid(const AdjointArgs &a, bool wproj, cudaStream_t st) {
  const size_t smem = degrid_taps_offset(a.nfacets, a.P) + (size_t)8 * 2 * a.W * sizeof(cplx);  // 8 warps
  if (smem > 200 * 1024) return BZ_ERR_UNSUPPORTED;
  if (cudaMemsetAsync(a.grad_vis, 0, sizeof(vis_complex) * (size_t)a.nrows * a.nchan * 4, st) != cudaSuccess) return BZ_ERR_CUDA;
  if (a.nrows == 0) return BZ_OK;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long warps_needed = (a.nrows * a.nchan + 31) / 32;  // 32 items per warp pass
  const long long blocks = std::min<long long>((warps_needed + 7) / 8, (long long)sms * 16);
  auto kern = wproj ? degrid_adjoint_kernel<true, PREDICT> : degrid_adjoint_kernel<false, PREDICT>;
  if (smem > 48 * 1024 && cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return BZ_ERR_CUDA;
  kern<<<(unsigned)blocks, 256, smem, st>>>(a);
  return cudaGetLastError() == cudaSuccess ? BZ_OK : BZ_ERR_CUDA;
}

// Model images -> the FFT input: dst[s][y][x] = img[s][(y+ny/2)%ny][(x+nx/2)%nx] / (taper_x[x'] taper_y[y'])
// at the source pixel (x', y') (numpy's ifftshift; the tapers are the gridding correction c(l) c(m)
// that finalize divides by, or null).
__global__ void predict_taper_shift_kernel(const vis_complex *__restrict__ img, vis_complex *__restrict__ dst, int nx,
                                           int ny, long long slices, const double *__restrict__ taper_x,
                                           const double *__restrict__ taper_y) {
  const long long nxy = (long long)nx * ny, total = nxy * slices;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const long long s = i / nxy, r = i - s * nxy;
    const int y = (int)(r / nx), x = (int)(r - (long long)y * nx);
    const int sy = (y + ny / 2) % ny, sx = (x + nx / 2) % nx;
    vis_complex v = img[s * nxy + (long long)sy * nx + sx];
    if (taper_x) {
      const double c = taper_x[sx] * taper_y[sy];
      v.re = (vis_real)((double)v.re / c);
      v.im = (vis_real)((double)v.im / c);
    }
    dst[i] = v;
  }
}

// After the forward transform: numpy's fftshift, cell (y, x) = src[(y-ny/2)%ny][(x-nx/2)%nx], written
// with the 4 correlations of a cell adjacent, dst[(f cube + g)][y][x][k] for source slice
// (f cube + g) x 4 + k (the gather then reads a cell's correlations with two 16-byte loads).
__global__ void predict_fftshift_kernel(const vis_complex *__restrict__ src, vis_complex *__restrict__ dst, int nx,
                                        int ny, long long slices) {
  const long long nxy = (long long)nx * ny, total = nxy * slices;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(i & 3);
    const long long cell = i >> 2, q = cell / nxy, r = cell - q * nxy;
    const int y = (int)(r / nx), x = (int)(r - (long long)y * nx);
    const int sy = (y + ny - ny / 2) % ny, sx = (x + nx - nx / 2) % nx;
    dst[i] = src[(q * 4 + k) * nxy + (long long)sy * nx + sx];
  }
}

// Batched 2-D forward plans, one per (device, ny, nx, batch), kept for the life of the process.
// Plans are shared by host threads: setting the stream and executing happen under the lock.
std::mutex g_plan_mutex;
std::map<std::tuple<int, int, int, int>, cufftHandle> g_plans;

int forward_fft(vis_complex *data, int nx, int ny, int batch, cudaStream_t st) {
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(g_plan_mutex);
  const auto key = std::make_tuple(dev, ny, nx, batch);
  auto it = g_plans.find(key);
  if (it == g_plans.end()) {
    cufftHandle plan;
    int dims[2] = {ny, nx};
    const int dist = nx * ny;
#if defined(BULLSEYE_SINGLE)
    const cufftType type = CUFFT_C2C;
#else
    const cufftType type = CUFFT_Z2Z;
#endif
    if (cufftPlanMany(&plan, 2, dims, nullptr, 1, dist, nullptr, 1, dist, type, batch) != CUFFT_SUCCESS) return BZ_ERR_CUFFT;
    it = g_plans.emplace(key, plan).first;
  }
  if (cufftSetStream(it->second, st) != CUFFT_SUCCESS) return BZ_ERR_CUFFT;
#if defined(BULLSEYE_SINGLE)
  const cufftResult r = cufftExecC2C(it->second, (cufftComplex *)data, (cufftComplex *)data, CUFFT_FORWARD);
#else
  const cufftResult r = cufftExecZ2Z(it->second, (cufftDoubleComplex *)data, (cufftDoubleComplex *)data, CUFFT_FORWARD);
#endif
  return r == CUFFT_SUCCESS ? BZ_OK : BZ_ERR_CUFFT;
}

constexpr int kPredictNormalise = 1;
constexpr int kPredictFromGrid = 2;

}  // namespace

// See include/bullseye_gb300.h.  Every pointer is a device pointer (as for the allocation-free
// gridding entry); jones_terms holds the raw (not inverted) terms or is null.
extern "C" int bullseye_grid_adjoint(const gridding_parameters *params, const void *grad_grid, void *grad_vis,
                                     void *grad_jones, int faceting, void *stream) {
  const char *name = "bullseye_grid_adjoint";
  if (!params || !grad_grid || !grad_vis) {
    bz_record_error(BZ_ERR_INVALID_ARGUMENT, "%s: params, grad_grid and grad_vis are required", name);
    return BZ_ERR_INVALID_ARGUMENT;
  }
  const gridding_parameters &p = *params;
  if (p.number_of_polarization_terms != 4 || p.number_of_polarization_terms_being_gridded != 4 || !p.visibilities ||
      !p.uvw_coords || !p.visibility_weights || !p.flags || !p.flagged_rows || !p.field_array || !p.spw_index_array ||
      !p.conv || !p.reference_wavelengths || !p.enabled_channels || !p.channel_grid_indicies ||
      (p.jones_terms && (!p.antenna_1_ids || !p.antenna_2_ids || !p.timestamp_ids))) {
    bz_record_error(BZ_ERR_INVALID_ARGUMENT, "%s: four polarisation terms and the row and table arrays are required", name);
    return BZ_ERR_INVALID_ARGUMENT;
  }
  AdjointArgs a = degrid_args(p, faceting);
  a.grad_grid = (const vis_complex *)grad_grid;
  a.grad_vis = (vis_complex *)grad_vis;
  a.grad_jones = p.jones_terms ? (vis_complex *)grad_jones : nullptr;
  const int rc = launch_degrid<false>(a, p.wplanes > 1, static_cast<cudaStream_t>(stream));
  if (rc != BZ_OK) bz_record_error(rc, "%s: launch failed (status %d)", name, rc);
  return rc;
}

// See include/bullseye_gb300.h.
extern "C" size_t bullseye_predict_ws_bytes(const gridding_parameters *params) {
  if (!params) return 0;
  const gridding_parameters &p = *params;
  const size_t F = p.num_facet_centres ? p.num_facet_centres : 1;
  return 2 * F * p.cube_channel_dim_size * 4 * p.nx * p.ny * sizeof(vis_complex);
}

// See include/bullseye_gb300.h.
extern "C" int bullseye_predict(const gridding_parameters *params, const void *model, const double *taper_x,
                                const double *taper_y, int faceting, int flags, void *vis_out, void *workspace,
                                size_t ws_bytes, void *stream) {
  const char *name = "bullseye_predict";
  if (!params || !model || !vis_out) {
    bz_record_error(BZ_ERR_INVALID_ARGUMENT, "%s: params, model and vis_out are required", name);
    return BZ_ERR_INVALID_ARGUMENT;
  }
  const gridding_parameters &p = *params;
  if (p.number_of_polarization_terms != 4 || p.number_of_polarization_terms_being_gridded != 4 || !p.uvw_coords ||
      !p.spw_index_array || !p.conv || !p.reference_wavelengths || !p.enabled_channels || !p.channel_grid_indicies ||
      (p.jones_terms && (!p.antenna_1_ids || !p.antenna_2_ids || !p.timestamp_ids)) || p.nx == 0 || p.ny == 0 ||
      p.cube_channel_dim_size == 0 || p.conv_oversample == 0 || (flags & ~(kPredictNormalise | kPredictFromGrid))) {
    bz_record_error(BZ_ERR_INVALID_ARGUMENT, "%s: four polarisation terms, uvw, spw and the tables are required", name);
    return BZ_ERR_INVALID_ARGUMENT;
  }
  if ((taper_x == nullptr) != (taper_y == nullptr)) {
    bz_record_error(BZ_ERR_INVALID_ARGUMENT, "%s: give both gridding-correction tapers or neither", name);
    return BZ_ERR_INVALID_ARGUMENT;
  }
  const bool from_grid = (flags & kPredictFromGrid) != 0;
  const size_t need = from_grid ? 0 : bullseye_predict_ws_bytes(params);
  if (need && (!workspace || ws_bytes < need || (reinterpret_cast<uintptr_t>(workspace) & 255))) {
    bz_record_error(BZ_ERR_INVALID_ARGUMENT, "%s: workspace of %zu bytes at %p, need %zu bytes 256-byte aligned", name,
                    ws_bytes, workspace, need);
    return BZ_ERR_INVALID_ARGUMENT;
  }
  const size_t F = p.num_facet_centres ? p.num_facet_centres : 1;
  const long long slices = (long long)(F * p.cube_channel_dim_size * 4);
  if (!from_grid && ((long long)p.nx * (long long)p.ny > 0x7fffffffLL || slices > 0x7fffffffLL)) {
    bz_record_error(BZ_ERR_UNSUPPORTED, "%s: %lld model slices of %zu x %zu exceed one batched transform", name, slices,
                    p.nx, p.ny);
    return BZ_ERR_UNSUPPORTED;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const vis_complex *grids = static_cast<const vis_complex *>(model);
  if (!from_grid) {
    vis_complex *buf = static_cast<vis_complex *>(workspace);
    vis_complex *out = buf + (size_t)slices * p.nx * p.ny;
    predict_taper_shift_kernel<<<2048, 256, 0, st>>>(grids, buf, (int)p.nx, (int)p.ny, slices, taper_x, taper_y);
    int rc = cudaGetLastError() == cudaSuccess ? BZ_OK : BZ_ERR_CUDA;
    if (rc == BZ_OK) rc = forward_fft(buf, (int)p.nx, (int)p.ny, (int)slices, st);
    if (rc == BZ_OK) {
      predict_fftshift_kernel<<<2048, 256, 0, st>>>(buf, out, (int)p.nx, (int)p.ny, slices);
      rc = cudaGetLastError() == cudaSuccess ? BZ_OK : BZ_ERR_CUDA;
    }
    if (rc != BZ_OK) {
      bz_record_error(rc, "%s: model transform failed (status %d)", name, rc);
      return rc;
    }
    grids = out;
  }
  AdjointArgs a = degrid_args(p, faceting);
  a.grad_grid = grids;
  a.grid_interleaved = from_grid ? 0 : 1;  // the model grids made above interleave the correlations
  a.grad_vis = static_cast<vis_complex *>(vis_out);
  a.normalise = (flags & kPredictNormalise) ? 1 : 0;
  const int rc = launch_degrid<true>(a, p.wplanes > 1, st);
  if (rc != BZ_OK) bz_record_error(rc, "%s: launch failed (status %d)", name, rc);
  return rc;
}
