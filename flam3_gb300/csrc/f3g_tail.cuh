/*
 * f3g_tail.cuh -- device helpers of the render tail: histogram and
 * accumulator access, log-density scaling, and the tonemap of
 * rect.c:1167-1241 with palettes.c:199-349 (FP32).
 */
#ifndef F3G_TAIL_CUH
#define F3G_TAIL_CUH

#include <cuda_runtime.h>

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

/* Tail arithmetic is FP32 with hardware approximations (a few ulp) unless
 * F3G_ACCURATE_MATH is defined; the output is quantised to 8 or 16 bits. */
#ifndef F3G_ACCURATE_MATH
__device__ __forceinline__ float t_div(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ float t_pow(float x, float y) { return __powf(x, y); }
/* log(1 + x) for x >= 0: below 1 from log1p(x) = 2 atanh(s), s = x / (2 + x)
 * <= 1/3, with the atanh Taylor series to s^13 (truncation < 2e-8
 * relative); above 1 from the hardware logarithm, whose relative error is
 * small there because the result exceeds ln 2. */
__device__ __forceinline__ float t_log1p(float x) {
  if (x >= 1.0f) return __logf(1.0f + x);
  const float s = __fdividef(x, 2.0f + x), z = s * s;
  float p = 1.0f / 13.0f;
  p = fmaf(p, z, 1.0f / 11.0f);
  p = fmaf(p, z, 1.0f / 9.0f);
  p = fmaf(p, z, 1.0f / 7.0f);
  p = fmaf(p, z, 1.0f / 5.0f);
  p = fmaf(p, z, 1.0f / 3.0f);
  p = fmaf(p, z, 1.0f);
  return 2.0f * s * p;
}
#else
__device__ __forceinline__ float t_div(float a, float b) { return a / b; }
__device__ __forceinline__ float t_pow(float x, float y) { return powf(x, y); }
__device__ __forceinline__ float t_log1p(float x) { return log1pf(x); }
#endif

/* ls = k1 * log(1 + c3*k2) / c3  (rect.c:963) */
__device__ __forceinline__ float log_scale(float c3, float k1, float k2) {
  return t_div(k1 * t_log1p(c3 * k2), c3);
}

/* log_scale for any c3 >= 0, 0 for an empty bucket */
__device__ __forceinline__ float log_scale_nz(float c3, float k1, float k2) {
  return c3 != 0.0f ? log_scale(c3, k1, k2) : 0.0f;
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
  s = (mx != 0.0f) ? t_div(del, mx) : 0.0f;
  h = 0.0f;
  if (s != 0.0f) {
    const float id = t_div(1.0f, del);
    float rc = (mx - rd) * id, gc = (mx - gd) * id, bc = (mx - bd) * id;
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
      float frac = t_div(density, linrange);
      return (1.0f - frac) * density * t_div(funcval, linrange) + frac * t_pow(density, gamma);
    }
    return t_pow(density, gamma);
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
    float a = ls * (cbuf[k] * (1.0f / 255.0f));
    if (a > maxa) { maxa = a; maxc = cbuf[k] * (1.0f / 255.0f); }
  }
  if (maxa > 255.0f && highpow >= 0.0f) {
    float newls = t_div(255.0f, maxc), lsratio = t_pow(t_div(newls, ls), highpow), hsv[3];
    for (int k = 0; k < 3; k++) newrgb[k] = newls * (cbuf[k] * (1.0f / 255.0f)) * (1.0f / 255.0f);
    rgb2hsv(newrgb, hsv);
    hsv[1] *= lsratio;
    hsv2rgb(hsv, newrgb);
    for (int k = 0; k < 3; k++) newrgb[k] *= 255.0f;
  } else {
    float newls = t_div(255.0f, maxc), adjhlp = -highpow;
    if (adjhlp > 1.0f) adjhlp = 1.0f;
    if (maxa <= 255.0f) adjhlp = 1.0f;
    for (int k = 0; k < 3; k++) newrgb[k] = ((1.0f - adjhlp) * newls + adjhlp * ls) * (cbuf[k] * (1.0f / 255.0f));
  }
}

__device__ __forceinline__ void tonemap(float *t, const F3GTonemap &tp) {
  float alpha, ls, tmp = t[3] * (1.0f / 255.0f), newrgb[3];
  if (t[3] <= 0.0f) {
    alpha = 0.0f;
    ls = 0.0f;
  } else {
    alpha = calc_alpha(tmp, tp.g, tp.linrange, tp.funcval);
    ls = t_div(tp.vibrancy * 256.0f * alpha, tmp);
    alpha = fminf(fmaxf(alpha, 0.0f), 1.0f);
  }
  calc_newrgb(t, ls, tp.highpow, newrgb);
  for (int k = 0; k < 3; k++) {
    float a = newrgb[k];
    if (tp.vibrancy != 1.0f) a += (1.0f - tp.vibrancy) * 256.0f * t_pow(t[k] * (1.0f / 255.0f), tp.g);
    if (tp.nchan <= 3 || tp.transp == 0) a += (1.0f - alpha) * tp.background[k];
    else a = (alpha > 0.0f) ? t_div(a, alpha) : 0.0f;
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

}  // namespace f3g

#endif
