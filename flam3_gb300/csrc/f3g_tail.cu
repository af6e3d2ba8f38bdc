/*
 * f3g_tail.cu -- the render tail: log-density scaling, density estimation,
 * spatial filter, gamma/vibrancy/highlight tonemap and 8/16-bit packing.
 *
 * Replaces rect.c:933-974 (k1/k2 log scaling), rect.c:57-251 (de_thread),
 * rect.c:1067-1247 (earlyclip, filter, tonemap, pack) and the helpers of
 * palettes.c:199-349.  Arithmetic is FP32 (FP64 reads when the histogram is
 * FP64).
 *
 * Kernels:
 *   k_logscale        acc += ls(bucket) * bucket           (no DE)
 *   k_de_gather       DE as a gather over shared-memory tiles (see below)
 *   k_earlyclip       tonemap the accumulator in place     (earlyclip=1)
 *   k_filter_tonemap  spatial filter + tonemap + pack      (one output pixel per thread)
 *   k_fused_log_filter: log scaling + filter + tonemap + pack in one pass over
 *                     the histogram, for one batch without DE
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "f3g_common.h"
#include "f3g_launch.h"

namespace f3g {

/* ---------------------------------------------------------------------
 * histogram / accumulator access
 * ------------------------------------------------------------------- */
__device__ __forceinline__ float4 load_bucket(const void *b, int kind, long long i) {
  if (kind == F3G_BK_F32) return __ldg((const float4 *)b + i);
  const double2 *d = (const double2 *)b + 2 * i;
  double2 a = __ldg(d), c = __ldg(d + 1);
  return make_float4((float)a.x, (float)a.y, (float)c.x, (float)c.y);
}

__device__ __forceinline__ float load_count(const void *b, int kind, const void *count, long long i) {
  if (count) return kind == F3G_BK_F32 ? __ldg((const float *)count + i) : (float)__ldg((const double *)count + i);
  return load_bucket(b, kind, i).w;
}

__device__ __forceinline__ void acc_add(void *acc, int kind, long long i, float4 v) {
  if (kind == F3G_BK_F32) {
    atomicAdd((float4 *)acc + i, v);
  } else {
    double *d = (double *)acc + 4 * i;
    atomicAdd(d + 0, (double)v.x);
    atomicAdd(d + 1, (double)v.y);
    atomicAdd(d + 2, (double)v.z);
    atomicAdd(d + 3, (double)v.w);
  }
}

__device__ __forceinline__ float4 acc_load(const void *acc, int kind, long long i) {
  if (kind == F3G_BK_F32) return ((const float4 *)acc)[i];
  const double *d = (const double *)acc + 4 * i;
  return make_float4((float)d[0], (float)d[1], (float)d[2], (float)d[3]);
}

__device__ __forceinline__ void acc_store(void *acc, int kind, long long i, float4 v) {
  if (kind == F3G_BK_F32) ((float4 *)acc)[i] = v;
  else {
    double *d = (double *)acc + 4 * i;
    d[0] = v.x; d[1] = v.y; d[2] = v.z; d[3] = v.w;
  }
}

/* ls = k1 * log(1 + c3*k2) / c3  (rect.c:963) */
__device__ __forceinline__ float log_scale(float c3, float k1, float k2) {
  return k1 * log1pf(c3 * k2) / c3;
}

/* ---------------------------------------------------------------------
 * tonemap (rect.c:1167-1203 with palettes.c:199-349)
 * ------------------------------------------------------------------- */
__device__ __forceinline__ void rgb2hsv(const float *rgb, float *hsv) {
  float rd = rgb[0], gd = rgb[1], bd = rgb[2], h, s, v, mx, mn, del;
  if (rd >= gd) mx = (rd >= bd) ? rd : bd;
  else mx = (gd >= bd) ? gd : bd;
  if (rd <= gd) mn = (rd <= bd) ? rd : bd;
  else mn = (gd <= bd) ? gd : bd;
  del = mx - mn;
  v = mx;
  s = (mx != 0.0f) ? del / mx : 0.0f;
  h = 0.0f;
  if (s != 0.0f) {
    float rc = (mx - rd) / del, gc = (mx - gd) / del, bc = (mx - bd) / del;
    if (rd == mx) h = bc - gc;
    else if (gd == mx) h = 2.0f + rc - bc;
    else if (bd == mx) h = 4.0f + gc - rc;
    if (h < 0.0f) h += 6.0f;
  }
  hsv[0] = h; hsv[1] = s; hsv[2] = v;
}

__device__ __forceinline__ void hsv2rgb(const float *hsv, float *rgb) {
  float h = hsv[0], s = hsv[1], v = hsv[2];
  while (h >= 6.0f) h -= 6.0f;
  while (h < 0.0f) h += 6.0f;
  int j = (int)floorf(h);
  float f = h - j, p = v * (1.0f - s), q = v * (1.0f - s * f), t = v * (1.0f - s * (1.0f - f));
  float r, g, b;
  switch (j) {
    case 0: r = v; g = t; b = p; break;
    case 1: r = q; g = v; b = p; break;
    case 2: r = p; g = v; b = t; break;
    case 3: r = p; g = q; b = v; break;
    case 4: r = t; g = p; b = v; break;
    case 5: r = v; g = p; b = q; break;
    default: r = v; g = t; b = p; break;
  }
  rgb[0] = r; rgb[1] = g; rgb[2] = b;
}

__device__ __forceinline__ float calc_alpha(float density, float gamma, float linrange, float funcval) {
  if (density > 0.0f) {
    if (density < linrange) {
      float frac = density / linrange;
      return (1.0f - frac) * density * (funcval / linrange) + frac * powf(density, gamma);
    }
    return powf(density, gamma);
  }
  return 0.0f;
}

__device__ __forceinline__ void calc_newrgb(const float *cbuf, float ls, float highpow, float *newrgb) {
  if (ls == 0.0f || (cbuf[0] == 0.0f && cbuf[1] == 0.0f && cbuf[2] == 0.0f)) {
    newrgb[0] = newrgb[1] = newrgb[2] = 0.0f;
    return;
  }
  float maxa = -1.0f, maxc = 0.0f;
  for (int k = 0; k < 3; k++) {
    float a = ls * (cbuf[k] / 255.0f);
    if (a > maxa) { maxa = a; maxc = cbuf[k] / 255.0f; }
  }
  if (maxa > 255.0f && highpow >= 0.0f) {
    float newls = 255.0f / maxc, lsratio = powf(newls / ls, highpow), hsv[3];
    for (int k = 0; k < 3; k++) newrgb[k] = newls * (cbuf[k] / 255.0f) / 255.0f;
    rgb2hsv(newrgb, hsv);
    hsv[1] *= lsratio;
    hsv2rgb(hsv, newrgb);
    for (int k = 0; k < 3; k++) newrgb[k] *= 255.0f;
  } else {
    float newls = 255.0f / maxc, adjhlp = -highpow;
    if (adjhlp > 1.0f) adjhlp = 1.0f;
    if (maxa <= 255.0f) adjhlp = 1.0f;
    for (int k = 0; k < 3; k++) newrgb[k] = ((1.0f - adjhlp) * newls + adjhlp * ls) * (cbuf[k] / 255.0f);
  }
}

__device__ __forceinline__ void tonemap(float *t, const F3GTonemap &tp) {
  float alpha, ls, tmp = t[3] / 255.0f, newrgb[3];
  if (t[3] <= 0.0f) {
    alpha = 0.0f;
    ls = 0.0f;
  } else {
    alpha = calc_alpha(tmp, tp.g, tp.linrange, tp.funcval);
    ls = tp.vibrancy * 256.0f * alpha / tmp;
    alpha = fminf(fmaxf(alpha, 0.0f), 1.0f);
  }
  calc_newrgb(t, ls, tp.highpow, newrgb);
  for (int k = 0; k < 3; k++) {
    float a = newrgb[k];
    if (tp.vibrancy != 1.0f) a += (1.0f - tp.vibrancy) * 256.0f * powf(t[k] / 255.0f, tp.g);
    if (tp.nchan <= 3 || tp.transp == 0) a += (1.0f - alpha) * tp.background[k];
    else a = (alpha > 0.0f) ? a / alpha : 0.0f;
    t[k] = fminf(fmaxf(a, 0.0f), 255.0f);
  }
  t[3] = alpha;
}

/* rect.c:1205-1241: clamp and pack one pixel */
__device__ __forceinline__ void pack_pixel(unsigned char *p, const float *t, const F3GTonemap &tp) {
  if (tp.bpc == 2) {
    unsigned short *p16 = (unsigned short *)p;
    for (int k = 0; k < 3; k++) p16[k] = (unsigned short)(fminf(fmaxf(t[k], 0.0f), 255.0f) * 256.0f);
    if (tp.nchan > 3) {
      float a = fminf(fmaxf(t[3], 0.0f), 1.0f);
      p16[3] = tp.transp == 1 ? (unsigned short)(a * 65535.0f) : (unsigned short)65535;
    }
  } else {
    for (int k = 0; k < 3; k++) p[k] = (unsigned char)fminf(fmaxf(t[k], 0.0f), 255.0f);
    if (tp.nchan > 3) {
      float a = fminf(fmaxf(t[3], 0.0f), 1.0f);
      p[3] = tp.transp == 1 ? (unsigned char)(a * 255.0f) : (unsigned char)255;
    }
  }
}

/* ---------------------------------------------------------------------
 * kernels
 * ------------------------------------------------------------------- */
__global__ void k_logscale(const void *__restrict__ buckets, int bkind, long long n, float k1, float k2, void *acc,
                           int akind) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float4 c = load_bucket(buckets, bkind, i);
    if (c.w == 0.0f) continue;
    float ls = log_scale(c.w, k1, k2);
    float4 v = make_float4(c.x * ls, c.y * ls, c.z * ls, c.w * ls);
    if (akind == F3G_BK_F32) {
      float4 *a = (float4 *)acc + i;
      float4 o = *a;
      *a = make_float4(o.x + v.x, o.y + v.y, o.z + v.z, o.w + v.w);
    } else {
      double *d = (double *)acc + 4 * i;
      d[0] += v.x; d[1] += v.y; d[2] += v.z; d[3] += v.w;
    }
  }
}

/* Density estimation (rect.c:57-251) as a gather.  The reference scatters
 * each source bucket with a kernel chosen by the density around it; here a
 * block owns a TxT tile of destination buckets and
 *   1. stages the sources of the tile plus a halo of R (the widest kernel's
 *      reach) in shared memory: log-scaled colour (float4), kernel index and
 *      reach (-1 for empty sources);
 *   2. each thread sums, for its destination, every staged source whose
 *      reach covers it, with the octant coefficient of that source's kernel.
 * Sources outside the reference's DE loop bounds contribute nothing. */
#define DE_TILE 16

__global__ void __launch_bounds__(256) k_de_gather(const void *__restrict__ buckets, int bkind,
                                                   const void *__restrict__ count, int W, int H, int oversample,
                                                   float k1, float k2, float curve, int max_filtered_counts,
                                                   int max_filter_index, int kernel_size,
                                                   const float *__restrict__ widths,
                                                   const float *__restrict__ coefs, int R, void *acc, int akind) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int S = DE_TILE + 2 * R;
  float4 *sv = (float4 *)smem_raw;
  short2 *sk = (short2 *)(sv + S * S); /* x: kernel index, y: reach (-1 = none) */
  const int tx0 = blockIdx.x * DE_TILE, ty0 = blockIdx.y * DE_TILE;
  const int ss = oversample / 2;
  const int scf = !(oversample & 1);
  const float scfact = powf(oversample / (oversample + 1.0f), 2.0f);
  const int istart = oversample - 1, iend = W - (oversample - 1);
  const int jstart = oversample - 1, jend = (oversample - 1) + (H - 2 * (oversample - 1) + 1);
  for (int k = threadIdx.x; k < S * S; k += blockDim.x) {
    int i = tx0 - R + k % S, j = ty0 - R + k / S;
    float4 v = make_float4(0, 0, 0, 0);
    short2 kr = make_short2(0, -1);
    if (i >= istart && i < iend && j >= jstart && j < jend && j < H) {
      long long bi = (long long)i + (long long)j * W;
      float4 c = load_bucket(buckets, bkind, bi);
      float cnt = count ? load_count(buckets, bkind, count, bi) : c.w;
      if (cnt != 0.0f && c.w != 0.0f) {
        float f = 0.0f;
        for (int ii = -ss; ii <= ss; ii++)
          for (int jj = -ss; jj <= ss; jj++) {
            int ni = i + ii, nj = j + jj;
            if (ni >= 0 && ni < W && nj >= 0 && nj < H)
              f += load_count(buckets, bkind, count, (long long)ni + (long long)nj * W) / 255.0f;
          }
        if (scf) f *= scfact;
        int fi;
        if (f > (float)max_filtered_counts) fi = max_filter_index;
        else if (f <= 100.0f) fi = (int)ceilf(f) - 1;
        else fi = 100 + (int)floorf(powf(f - 100.0f, curve));
        if (fi > max_filter_index) fi = max_filter_index;
        if (fi < 0) fi = 0;
        int reach = (int)ceilf(widths[fi]) - 1;
        float ls = k1 * log1pf(c.w * k2) / c.w;
        v = make_float4(c.x * ls, c.y * ls, c.z * ls, c.w * ls);
        kr = make_short2((short)fi, (short)reach);
      }
    }
    sv[k] = v;
    sk[k] = kr;
  }
  __syncthreads();
  const int lx = threadIdx.x % DE_TILE, ly = threadIdx.x / DE_TILE;
  const int di = tx0 + lx, dj = ty0 + ly;
  if (di >= W || dj >= H) return;
  float4 sum = make_float4(0, 0, 0, 0);
  for (int dy = -R; dy <= R; dy++) {
    const int ady = dy < 0 ? -dy : dy;
    const int row = (ly + R + dy) * S + lx + R;
    for (int dx = -R; dx <= R; dx++) {
      short2 kr = sk[row + dx];
      const int adx = dx < 0 ? -dx : dx;
      const int hi = adx > ady ? adx : ady, lo = adx > ady ? ady : adx;
      if (kr.y < hi) continue;
      float cf = __ldg(coefs + (long long)kr.x * kernel_size + hi * (hi + 1) / 2 + lo);
      if (cf == 0.0f) continue;
      float4 v = sv[row + dx];
      sum.x += cf * v.x; sum.y += cf * v.y; sum.z += cf * v.z; sum.w += cf * v.w;
    }
  }
  long long di_lin = (long long)di + (long long)dj * W;
  float4 o = acc_load(acc, akind, di_lin);
  acc_store(acc, akind, di_lin, make_float4(o.x + sum.x, o.y + sum.y, o.z + sum.z, o.w + sum.w));
}

__global__ void k_earlyclip(void *acc, int akind, long long n, F3GTonemap tp) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float4 a = acc_load(acc, akind, i);
    float t[4] = {a.x, a.y, a.z, a.w};
    tonemap(t, tp);
    acc_store(acc, akind, i, make_float4(t[0], t[1], t[2], t[3]));
  }
}

__global__ void k_filter_tonemap(const void *__restrict__ acc, int akind, int W, int de_offset, int oversample,
                                 const float *__restrict__ filter, int fw, int image_w, int image_h,
                                 unsigned char *out, int earlyclip, F3GTonemap tp) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= image_w || j >= image_h) return;
  int x = de_offset + i * oversample, y = de_offset + j * oversample;
  float t[4] = {0, 0, 0, 0};
  for (int jj = 0; jj < fw; jj++)
    for (int ii = 0; ii < fw; ii++) {
      float k = __ldg(filter + ii + jj * fw);
      float4 a = acc_load(acc, akind, (long long)(x + ii) + (long long)(y + jj) * W);
      t[0] += k * a.x; t[1] += k * a.y; t[2] += k * a.z; t[3] += k * a.w;
    }
  if (!earlyclip) tonemap(t, tp);
  pack_pixel(out + (size_t)tp.nchan * tp.bpc * ((size_t)i + (size_t)j * image_w), t, tp);
}

/* One batch without DE: read each histogram bucket once, log-scale it into a
 * shared tile, filter and tonemap the output pixels of the tile, pack. */
#define FL_TX 32
#define FL_TY 8
__global__ void __launch_bounds__(256) k_fused_log_filter(const void *__restrict__ buckets, int bkind, int W, int H,
                                                          float k1, float k2, int de_offset, int oversample,
                                                          const float *__restrict__ filter, int fw, int image_w,
                                                          int image_h, unsigned char *out, int earlyclip,
                                                          F3GTonemap tp) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int sw = FL_TX * oversample + fw - oversample, sh = FL_TY * oversample + fw - oversample;
  float4 *tile = (float4 *)smem_raw;
  float *sf = (float *)(tile + sw * sh);
  const int i0 = blockIdx.x * FL_TX, j0 = blockIdx.y * FL_TY;
  const int bx0 = de_offset + i0 * oversample, by0 = de_offset + j0 * oversample;
  const int tid = threadIdx.x + threadIdx.y * blockDim.x, nt = blockDim.x * blockDim.y;
  for (int k = tid; k < fw * fw; k += nt) sf[k] = filter[k];
  for (int k = tid; k < sw * sh; k += nt) {
    int bx = bx0 + k % sw, by = by0 + k / sw;
    float4 v = make_float4(0, 0, 0, 0);
    if (bx < W && by < H) {
      float4 c = load_bucket(buckets, bkind, (long long)bx + (long long)by * W);
      if (c.w != 0.0f) {
        float ls = log_scale(c.w, k1, k2);
        v = make_float4(c.x * ls, c.y * ls, c.z * ls, c.w * ls);
        if (earlyclip) {
          float t[4] = {v.x, v.y, v.z, v.w};
          tonemap(t, tp);
          v = make_float4(t[0], t[1], t[2], t[3]);
        }
      } else if (earlyclip) {
        float t[4] = {0, 0, 0, 0};
        tonemap(t, tp);
        v = make_float4(t[0], t[1], t[2], t[3]);
      }
    }
    tile[k] = v;
  }
  __syncthreads();
  const int i = i0 + threadIdx.x, j = j0 + threadIdx.y;
  if (i >= image_w || j >= image_h) return;
  const int lx = threadIdx.x * oversample, ly = threadIdx.y * oversample;
  float t[4] = {0, 0, 0, 0};
  for (int jj = 0; jj < fw; jj++)
    for (int ii = 0; ii < fw; ii++) {
      float k = sf[ii + jj * fw];
      float4 a = tile[(lx + ii) + (ly + jj) * sw];
      t[0] += k * a.x; t[1] += k * a.y; t[2] += k * a.z; t[3] += k * a.w;
    }
  if (!earlyclip) tonemap(t, tp);
  pack_pixel(out + (size_t)tp.nchan * tp.bpc * ((size_t)i + (size_t)j * image_w), t, tp);
}

}  // namespace f3g

using namespace f3g;

static int grid_for(long long n, int threads) {
  long long b = (n + threads - 1) / threads;
  if (b > 152 * 32) b = 152 * 32;
  if (b < 1) b = 1;
  return (int)b;
}

extern "C" int f3g_launch_logscale(const void *buckets, int bkind, long long n, double k1, double k2, void *acc,
                                   int akind, cudaStream_t st) {
  k_logscale<<<grid_for(n, 256), 256, 0, st>>>(buckets, bkind, n, (float)k1, (float)k2, acc, akind);
  return (int)cudaGetLastError();
}

extern "C" int f3g_launch_de(const void *buckets, int bkind, const void *count, int W, int H, int oversample,
                             double k1, double k2, double curve, int max_filtered_counts, int max_filter_index,
                             int kernel_size, const float *widths, const float *coefs, int R, void *acc, int akind,
                             cudaStream_t st) {
  int S = DE_TILE + 2 * R;
  size_t smem = (size_t)S * S * (sizeof(float4) + sizeof(short2));
  cudaError_t e = cudaFuncSetAttribute(k_de_gather, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  dim3 grid((W + DE_TILE - 1) / DE_TILE, (H + DE_TILE - 1) / DE_TILE);
  k_de_gather<<<grid, DE_TILE * DE_TILE, smem, st>>>(buckets, bkind, count, W, H, oversample, (float)k1, (float)k2,
                                                     (float)curve, max_filtered_counts, max_filter_index, kernel_size,
                                                     widths, coefs, R, acc, akind);
  return (int)cudaGetLastError();
}

extern "C" int f3g_de_max_reach(void) {
  /* shared memory bound of k_de_gather: (16 + 2R)^2 * 20 B <= 220 KB */
  return 44;
}

extern "C" int f3g_launch_earlyclip(void *acc, int akind, long long n, const F3GTonemap *tp, cudaStream_t st) {
  k_earlyclip<<<grid_for(n, 256), 256, 0, st>>>(acc, akind, n, *tp);
  return (int)cudaGetLastError();
}

extern "C" int f3g_launch_filter_tonemap(const void *acc, int akind, int W, int de_offset, int oversample,
                                         const float *filter, int fw, int image_w, int image_h, unsigned char *out,
                                         int earlyclip, const F3GTonemap *tp, cudaStream_t st) {
  dim3 block(32, 8), grid((image_w + 31) / 32, (image_h + 7) / 8);
  k_filter_tonemap<<<grid, block, 0, st>>>(acc, akind, W, de_offset, oversample, filter, fw, image_w, image_h, out,
                                           earlyclip, *tp);
  return (int)cudaGetLastError();
}

extern "C" int f3g_launch_fused_log_filter(const void *buckets, int bkind, int W, int H, double k1, double k2,
                                           int de_offset, int oversample, const float *filter, int fw, int image_w,
                                           int image_h, unsigned char *out, int earlyclip, const F3GTonemap *tp,
                                           cudaStream_t st) {
  int sw = FL_TX * oversample + fw - oversample, sh = FL_TY * oversample + fw - oversample;
  size_t smem = (size_t)sw * sh * sizeof(float4) + (size_t)fw * fw * sizeof(float);
  if (smem > 200 * 1024) return -1;
  cudaError_t e = cudaFuncSetAttribute(k_fused_log_filter, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  dim3 block(FL_TX, FL_TY), grid((image_w + FL_TX - 1) / FL_TX, (image_h + FL_TY - 1) / FL_TY);
  k_fused_log_filter<<<grid, block, smem, st>>>(buckets, bkind, W, H, (float)k1, (float)k2, de_offset, oversample,
                                                filter, fw, image_w, image_h, out, earlyclip, *tp);
  return (int)cudaGetLastError();
}
