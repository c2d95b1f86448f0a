// Small device kernels around the gridder: Jones inversion, compensated-grid resolution,
// and the finalize (shift / real-part packing / gridding correction) passes.
#pragma once
#include "common.h"

namespace bz {

// Time-innermost position of term i of a [T][A][F][S][Ch] table: [A][S][Ch][F][T].
struct JonesDims {
  long long T, A, F, S, C;
};
__device__ __forceinline__ long long jones_time_major(long long i, const JonesDims &d) {
  const long long c = i % d.C;
  long long r = i / d.C;
  const long long s = r % d.S;
  r /= d.S;
  const long long f = r % d.F;
  r /= d.F;
  const long long a = r % d.A;
  const long long t = r / d.A;
  return (((a * d.S + s) * d.C + c) * d.F + f) * d.T + t;
}

// Invert every 2x2 Jones matrix (jones_2x2.h:86-126).  Singular matrices (determinant exactly
// zero) are replaced by zeros and flagged; the reference throws instead.  With out_t, each
// inverse is also written time-innermost (the record kernel's copy).
__global__ void invert_jones_kernel(const vis_complex *__restrict__ in, vis_complex *__restrict__ out,
                                    long long n, int *error, vis_complex *__restrict__ out_t = nullptr,
                                    JonesDims dims = JonesDims{0, 0, 0, 0, 0}) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  vis_complex *o2 = out_t ? out_t + 4 * jones_time_major(i, dims) : nullptr;
  typedef vis_real T;
  vis_complex a = in[4 * i], b = in[4 * i + 1], c = in[4 * i + 2], d = in[4 * i + 3];
  T dr = (a.re * d.re - a.im * d.im) - (b.re * c.re - b.im * c.im);
  T di = (a.re * d.im + a.im * d.re) - (b.re * c.im + b.im * c.re);
  vis_complex z = {0, 0};
  if (dr == (T)0 && di == (T)0) {
    atomicOr(error, 4);
    out[4 * i] = z; out[4 * i + 1] = z; out[4 * i + 2] = z; out[4 * i + 3] = z;
    if (o2) { o2[0] = z; o2[1] = z; o2[2] = z; o2[3] = z; }
    return;
  }
  // 1 / det with scaling (Smith's method) to avoid overflow
  T ir, ii;
  if (fabs((double)dr) >= fabs((double)di)) {
    T r = di / dr, den = dr + di * r;
    ir = (T)1 / den;
    ii = -r / den;
  } else {
    T r = dr / di, den = dr * r + di;
    ir = r / den;
    ii = (T)-1 / den;
  }
  auto mul = [](vis_complex x, T yr, T yi) {
    vis_complex o;
    o.re = x.re * yr - x.im * yi;
    o.im = x.re * yi + x.im * yr;
    return o;
  };
  const vis_complex r0 = mul(d, ir, ii), r1 = mul(b, -ir, -ii), r2 = mul(c, -ir, -ii), r3 = mul(a, ir, ii);
  out[4 * i] = r0;
  out[4 * i + 1] = r1;
  out[4 * i + 2] = r2;
  out[4 * i + 3] = r3;
  if (o2) { o2[0] = r0; o2[1] = r1; o2[2] = r2; o2[3] = r3; }
}

// out = hi + lo (compensated grid resolution), element-wise over complex values.
__global__ void resolve_compensated_kernel(const vis_complex *__restrict__ hi, const vis_complex *__restrict__ lo,
                                           vis_complex *__restrict__ out, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    vis_complex h = hi[i];
    if (lo) {
      vis_complex l = lo[i];
      h.re += l.re;
      h.im += l.im;
    }
    out[i] = h;
  }
}

// out[f][i] = init[f][i] + hi[i] + lo[i] for f < nf, i < per: a facet-invariant accumulated
// contribution added to every facet's initial grid.
__global__ void broadcast_add_kernel(const vis_complex *__restrict__ init, const vis_complex *__restrict__ hi,
                                     const vis_complex *__restrict__ lo, vis_complex *__restrict__ out, long long per,
                                     long long nf) {
  const long long total = per * nf;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const long long r = i % per;
    vis_complex h = hi[r];
    if (lo) {
      h.re += lo[r].re;
      h.im += lo[r].im;
    }
    vis_complex o = init[i];
    o.re += h.re;
    o.im += h.im;
    out[i] = o;
  }
}

// Gather with the inverse shift of numpy's ifftshift: dst[y][x] = src[(y+ny/2)%ny][(x+nx/2)%nx]
// for each of `slices` planes.  Equivalent to bullseye/mo/cpu_gpu_common/fft_shift_utils.cpp:75-111.
// Stokes (or correlation) term of every (facet, cube slice): dst[f][c] = (src[f][c][a] +
// sign * src[f][c][b]) / 2 over nxy cells, from facet blocks of `cube` x `corr` slices into
// compact [facet][cube] slices (bullseye/data/stokes.py:90-172 combines the same pairs on the host).
__global__ void stokes_combine_kernel(const vis_complex *__restrict__ src, vis_complex *__restrict__ dst, long long nxy,
                                      int facets, int cube, int corr, int a, int b, int sign) {
  const long long total = (long long)facets * cube * nxy;
  const vis_real half = (vis_real)0.5, sg = (vis_real)sign;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const long long fc = i / nxy, r = i - fc * nxy;
    const long long base = fc * corr * nxy + r;  // slice (f, c, 0) of the facet block
    const vis_complex va = src[base + (long long)a * nxy], vb = src[base + (long long)b * nxy];
    vis_complex o;
    o.re = (va.re + sg * vb.re) * half;
    o.im = (va.im + sg * vb.im) * half;
    dst[i] = o;
  }
}

__global__ void ifftshift_gather_kernel(const vis_complex *__restrict__ src, vis_complex *__restrict__ dst, int nx,
                                        int ny, long long slices) {
  long long nxy = (long long)nx * ny;
  long long total = nxy * slices;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    long long s = i / nxy, r = i - s * nxy;
    int y = (int)(r / nx), x = (int)(r - (long long)y * nx);
    int sy = (y + ny / 2) % ny, sx = (x + nx / 2) % nx;
    dst[i] = src[s * nxy + (long long)sy * nx + sx];
  }
}

// After the transform: fftshift (dst[y][x] = src[(y-ny/2)%ny][(x-nx/2)%nx]) into `shifted`,
// and the float32 real parts into `packed`, optionally divided by the separable gridding
// correction corr_x[x] * corr_y[y].
__global__ void fftshift_pack_kernel(const vis_complex *__restrict__ src, vis_complex *__restrict__ shifted,
                                     float *__restrict__ packed, int nx, int ny, long long slices,
                                     const double *__restrict__ corr_x, const double *__restrict__ corr_y) {
  long long nxy = (long long)nx * ny;
  long long total = nxy * slices;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    long long s = i / nxy, r = i - s * nxy;
    int y = (int)(r / nx), x = (int)(r - (long long)y * nx);
    int sy = (y + ny - ny / 2) % ny, sx = (x + nx - nx / 2) % nx;
    vis_complex v = src[s * nxy + (long long)sy * nx + sx];
    if (shifted) shifted[i] = v;
    double re = (double)v.re;
    if (corr_x) re = re / (corr_x[x] * corr_y[y]);
    packed[i] = (float)re;
  }
}

// FP32 FMA throughput probe: kFmaProbeChains independent dependency chains per thread.
constexpr int kFmaProbeChains = 16;
__global__ void fma_probe_kernel(float *out, int iters) {
  float acc[kFmaProbeChains];
#pragma unroll
  for (int k = 0; k < kFmaProbeChains; ++k) acc[k] = (float)(threadIdx.x + k) * 1e-3f;
  const float m = 0.999999f, a = 1e-7f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < kFmaProbeChains; ++k) acc[k] = fmaf(acc[k], m, a);
  }
  float s = 0;
#pragma unroll
  for (int k = 0; k < kFmaProbeChains; ++k) s += acc[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace bz
