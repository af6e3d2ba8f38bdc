/*
 * f3g_device.cuh -- device side of the chaos game: the counter-based random
 * stream, the 99 variations and apply_xform, templated on the iteration
 * precision R (float by default, double for parity work).
 *
 * The formulas follow variations.c:142-1938 and apply_xform
 * variations.c:2129-2399 term for term, including the order in which random
 * words are drawn, so a given word stream produces the same point sequence
 * as the reference (to the rounding of R).
 */
#ifndef F3G_DEVICE_CUH
#define F3G_DEVICE_CUH

#include <stdint.h>

#include "f3g_common.h"

namespace f3g {

/* ---------------------------------------------------------------------
 * Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
 * easy as 1, 2, 3", SC'11): a counter-based generator; one call maps a
 * 128-bit counter and a 64-bit key to four 32-bit words.
 * ------------------------------------------------------------------- */
__device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
    uint32_t lo0 = 0xD2511F53u * c[0];
    uint32_t hi0 = __umulhi(0xD2511F53u, c[0]);
    uint32_t lo1 = 0xCD9E8D57u * c[2];
    uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]);
    uint32_t n0 = hi1 ^ c[1] ^ k0;
    uint32_t n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

/* A stream of 32-bit words: counter (c0, block, c2, c3) under key k;
 * each refill bumps the block word and yields four words in order. */
/* One Philox block, kept out of line (one copy of the ten rounds instead of
 * one per draw site); arguments and result stay in registers. */
static __device__ __noinline__ uint4 philox_block(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                                           uint32_t k1) {
  uint32_t c[4] = {c0, c1, c2, c3};
  philox4x32_10(c, k0, k1);
  return make_uint4(c[0], c[1], c[2], c[3]);
}

struct Rng {
  uint32_t k0, k1, c0, blk, c2, c3;
  uint32_t b0, b1, b2, b3;
  int pos;
  __device__ __forceinline__ void init(uint32_t key0, uint32_t key1, uint32_t ctr0, uint32_t ctr2, uint32_t ctr3) {
    k0 = key0; k1 = key1; c0 = ctr0; blk = 0; c2 = ctr2; c3 = ctr3; pos = 4;
  }
  __device__ __forceinline__ uint32_t word() {
    if (pos == 4) {
      uint4 r = philox_block(c0, blk, c2, c3, k0, k1);
      b0 = r.x; b1 = r.y; b2 = r.z; b3 = r.w;
      blk++;
      pos = 0;
    }
    uint32_t w = (pos == 0) ? b0 : (pos == 1) ? b1 : (pos == 2) ? b2 : b3;
    pos++;
    return w;
  }
};

/* Caller-given words, consumed in order (0 once exhausted). */
struct ArrayRng {
  const uint32_t *w;
  int n, pos;
  __device__ __forceinline__ uint32_t word() { return pos < n ? w[pos++] : 0u; }
};

/* flam3.c:2519-2544: U(0,1) and U(-1,1) from the low 28 bits, one bit. */
template <typename R> __device__ __forceinline__ R u01(uint32_t w) {
  return (R)(int)(w & 0xfffffffu) * (R)(1.0 / 268435455.0);
}
template <> __device__ __forceinline__ double u01<double>(uint32_t w) {
  return (double)(int)(w & 0xfffffffu) / 268435455.0;
}
template <typename R> __device__ __forceinline__ R u11(uint32_t w) {
  return (R)((int)(w & 0xfffffffu) - 0x7ffffff) * (R)(1.0 / 134217727.0);
}
template <> __device__ __forceinline__ double u11<double>(uint32_t w) {
  return (double)((int)(w & 0xfffffffu) - 0x7ffffff) / 134217727.0;
}

/* ---------------------------------------------------------------------
 * precision-generic math
 * ------------------------------------------------------------------- */
/* FP32 iteration uses the hardware approximations of sin, cos, exp, log and
 * pow (the chain is chaotic; the FP32 bound of the apply_xform tests covers
 * them, and whole-render error against a 16x-quality render is unchanged);
 * build with F3G_ACCURATE_MATH for the libm-accurate FP32 functions.  FP64
 * always uses the accurate functions. */
#if !defined(F3G_ACCURATE_MATH) && !defined(F3G_FAST_MATH)
#define F3G_FAST_MATH
#endif
#ifdef F3G_FAST_MATH
__device__ __forceinline__ float m_sin(float x) { return __sinf(x); }
__device__ __forceinline__ float m_cos(float x) { return __cosf(x); }
__device__ __forceinline__ void m_sincos(float x, float *s, float *c) { __sincosf(x, s, c); }
__device__ __forceinline__ float m_exp(float x) { return __expf(x); }
__device__ __forceinline__ float m_log(float x) { return __logf(x); }
__device__ __forceinline__ float m_pow(float x, float y) { return __powf(x, y); }
#else
__device__ __forceinline__ float m_sin(float x) { return sinf(x); }
__device__ __forceinline__ float m_cos(float x) { return cosf(x); }
__device__ __forceinline__ void m_sincos(float x, float *s, float *c) { sincosf(x, s, c); }
__device__ __forceinline__ float m_exp(float x) { return expf(x); }
__device__ __forceinline__ float m_log(float x) { return logf(x); }
__device__ __forceinline__ float m_pow(float x, float y) { return powf(x, y); }
#endif
/* quotient: with fast math FP32 uses the approximate divide (2 ulp) */
#ifdef F3G_FAST_MATH
__device__ __forceinline__ float m_div(float a, float b) { return __fdividef(a, b); }
#else
__device__ __forceinline__ float m_div(float a, float b) { return a / b; }
#endif
__device__ __forceinline__ double m_div(double a, double b) { return a / b; }
__device__ __forceinline__ double m_sin(double x) { return sin(x); }
__device__ __forceinline__ double m_cos(double x) { return cos(x); }
__device__ __forceinline__ void m_sincos(double x, double *s, double *c) { sincos(x, s, c); }
__device__ __forceinline__ double m_exp(double x) { return exp(x); }
__device__ __forceinline__ double m_log(double x) { return log(x); }
__device__ __forceinline__ double m_pow(double x, double y) { return pow(x, y); }
__device__ __forceinline__ float m_tan(float x) { return tanf(x); }
__device__ __forceinline__ double m_tan(double x) { return tan(x); }
#ifdef F3G_FAST_MATH
/* atan2 from atan on [0, 1] by octant reduction; atan(a) ~ a * P(a^2), P of
 * degree 6 fitted to arctangent on [0, 1] by iteratively reweighted least
 * squares (Lawson) for this project: max abs error 2.5e-7 rad. */
__device__ __forceinline__ float m_atan2(float y, float x) {
  const float ax = fabsf(x), ay = fabsf(y);
  const float mx = fmaxf(ax, ay), mn = fminf(ax, ay);
  const float a = mx > 0.0f ? __fdividef(mn, mx) : 0.0f;
  const float s = a * a;
  float p = 0.006811756f;
  p = fmaf(p, s, -0.033604111f);
  p = fmaf(p, s, 0.079623550f);
  p = fmaf(p, s, -0.132333356f);
  p = fmaf(p, s, 0.198078140f);
  p = fmaf(p, s, -0.333173679f);
  p = fmaf(p, s, 0.999996112f);
  float r = a * p;
  if (ay > ax) r = 1.57079632679489662f - r;
  if (x < 0.0f) r = 3.14159265358979324f - r;
  if (x != x || y != y) r = x + y;
  return copysignf(r, y);
}
/* square root: the hardware approximation (PTX sqrt.approx.f32: one
 * instruction, 0 for 0, NaN below 0) */
__device__ __forceinline__ float m_sqrt(float x) {
  float r;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
#else
__device__ __forceinline__ float m_atan2(float y, float x) { return atan2f(y, x); }
__device__ __forceinline__ float m_sqrt(float x) { return sqrtf(x); }
#endif
__device__ __forceinline__ double m_atan2(double y, double x) { return atan2(y, x); }
__device__ __forceinline__ double m_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float m_log10(float x) { return log10f(x); }
__device__ __forceinline__ double m_log10(double x) { return log10(x); }
__device__ __forceinline__ float m_sinh(float x) { return sinhf(x); }
__device__ __forceinline__ double m_sinh(double x) { return sinh(x); }
__device__ __forceinline__ float m_cosh(float x) { return coshf(x); }
__device__ __forceinline__ double m_cosh(double x) { return cosh(x); }
__device__ __forceinline__ float m_acos(float x) { return acosf(x); }
__device__ __forceinline__ double m_acos(double x) { return acos(x); }
__device__ __forceinline__ float m_fmod(float x, float y) { return fmodf(x, y); }
__device__ __forceinline__ double m_fmod(double x, double y) { return fmod(x, y); }
__device__ __forceinline__ float m_floor(float x) { return floorf(x); }
__device__ __forceinline__ double m_floor(double x) { return floor(x); }
__device__ __forceinline__ float m_trunc(float x) { return truncf(x); }
__device__ __forceinline__ double m_trunc(double x) { return trunc(x); }
__device__ __forceinline__ float m_rint(float x) { return rintf(x); }
__device__ __forceinline__ double m_rint(double x) { return rint(x); }
__device__ __forceinline__ float m_fabs(float x) { return fabsf(x); }
__device__ __forceinline__ double m_fabs(double x) { return fabs(x); }

/* F3G_LAZY_ANGLES: see var_basic */
#ifndef F3G_LAZY_ANGLES
#define F3G_LAZY_ANGLES 1
#endif

/* F3G_ANGLES_RSQ (with the fast FP32 math): FP32 sin and cos of the angle
 * (x/r, y/r) from one reciprocal square root instead of two divides */
#ifndef F3G_ANGLES_RSQ
#ifdef F3G_FAST_MATH
#define F3G_ANGLES_RSQ 1
#else
#define F3G_ANGLES_RSQ 0
#endif
#endif

/* NaN, or |x| > 1e10 (flam3.c:269-272), as one compare of |x| (false for
 * NaN) */
template <typename R> __device__ __forceinline__ bool badvalue(R x) { return !(fabs(x) <= (R)1e10); }

/* One xform staged in shared memory in the iteration precision. */
/* 16-byte aligned: apply_xform loads its FP32 fields as vectors */
template <typename R> struct __align__(16) XfS {
  R c[6], post[6];
  R color, color_speed, vis_adjusted, opacity, preblur;
  int flags, var_off, nvars;
  R prm[PRM_COUNT];
};

template <typename R> struct Helper {
  R tx, ty, atan_xy, sina, cosa, sqrtv, sumsq, atan_yx, p0, p1;
};

#define PI_R ((R)3.14159265358979323846)
#define PI_2_R ((R)1.57079632679489661923)
#define PI_4_R ((R)0.78539816339744830962)
#define ONE_PI_R ((R)0.31830988618379067154)
#define TWO_PI_R ((R)0.63661977236758134308)
#define EPS_R ((R)1e-10)
#define P(name) x.prm[PRM_##name]

/* variations 0-19 (the set the common genomes use) */
/* The angle terms of apply_xform (variations.c:2153-2170): atan2(tx, ty)
 * and (sin, cos) of the point's angle as (tx/r, ty/r) -- FP32 from one
 * reciprocal square root when F3G_ANGLES_RSQ, else two divides. */
template <typename R> __device__ __forceinline__ R pre_atan_xy(const Helper<R> &f) { return m_atan2(f.tx, f.ty); }
template <typename R> __device__ __forceinline__ void pre_angles(const Helper<R> &f, R &sina, R &cosa) {
#if F3G_ANGLES_RSQ
  if (sizeof(R) == 4) {
    const R r = (R)rsqrtf((float)f.sumsq);
    sina = f.tx * r;
    cosa = f.ty * r;
    return;
  }
#endif
  sina = m_div(f.tx, f.sqrtv);
  cosa = m_div(f.ty, f.sqrtv);
}

/* Variations 0-19.  LAZY: the angle terms are computed here, by the
 * variations that use them, instead of once per xform by apply_xform (the
 * same values: they live only inside the case, which matters at the
 * iterate kernel's register cap). */
template <typename R, class G, bool LAZY>
__device__ __forceinline__ void var_basic(int v, R w, Helper<R> &f, const XfS<R> &x, G &rng) {
#define ATAN_XY (LAZY ? pre_atan_xy<R>(f) : f.atan_xy)
#define ANGLES(sa_, ca_)          \
  R sa_, ca_;                     \
  if (LAZY) pre_angles<R>(f, sa_, ca_); \
  else {                          \
    sa_ = f.sina;                 \
    ca_ = f.cosa;                 \
  }
  switch (v) {
    case 0: f.p0 += w * f.tx; f.p1 += w * f.ty; break;
    case 1: f.p0 += w * m_sin(f.tx); f.p1 += w * m_sin(f.ty); break;
    case 2: { R r2 = m_div(w, f.sumsq + EPS_R); f.p0 += r2 * f.tx; f.p1 += r2 * f.ty; } break;
    case 3: {
      R c1, c2; m_sincos(f.sumsq, &c1, &c2);
      R nx = c1 * f.tx - c2 * f.ty, ny = c2 * f.tx + c1 * f.ty;
      f.p0 += w * nx; f.p1 += w * ny;
    } break;
    case 4: {
      R r = m_div(w, f.sqrtv + EPS_R);
      f.p0 += (f.tx - f.ty) * (f.tx + f.ty) * r; f.p1 += (R)2.0 * f.tx * f.ty * r;
    } break;
    case 5: f.p0 += w * (ATAN_XY * ONE_PI_R); f.p1 += w * (f.sqrtv - (R)1.0); break;
    case 6: {
      R a = ATAN_XY, r = f.sqrtv;
      f.p0 += w * r * m_sin(a + r); f.p1 += w * r * m_cos(a - r);
    } break;
    case 7: {
      R a = f.sqrtv * ATAN_XY, sa, ca, r = w * f.sqrtv; m_sincos(a, &sa, &ca);
      f.p0 += r * sa; f.p1 += (-r) * ca;
    } break;
    case 8: {
      R a = ATAN_XY * ONE_PI_R, r = PI_R * f.sqrtv, sr, cr; m_sincos(r, &sr, &cr);
      f.p0 += w * sr * a; f.p1 += w * cr * a;
    } break;
    case 9: {
      R r = f.sqrtv + EPS_R, r1 = m_div(w, r), sr, cr; m_sincos(r, &sr, &cr);
      ANGLES(sina, cosa)
      f.p0 += r1 * (cosa + sr); f.p1 += r1 * (sina - cr);
    } break;
    case 10: { ANGLES(sina, cosa) R r = f.sqrtv + EPS_R; f.p0 += m_div(w * sina, r); f.p1 += w * cosa * r; } break;
    case 11: {
      R sr, cr; m_sincos(f.sqrtv, &sr, &cr);
      ANGLES(sina, cosa)
      f.p0 += w * sina * cr; f.p1 += w * cosa * sr;
    } break;
    case 12: {
      R a = ATAN_XY, r = f.sqrtv, n0 = m_sin(a + r), n1 = m_cos(a - r);
      R m0 = n0 * n0 * n0 * r, m1 = n1 * n1 * n1 * r;
      f.p0 += w * (m0 + m1); f.p1 += w * (m0 - m1);
    } break;
    case 13: {
      /* julia draws one word (variations.c:350-372) */
      R a = (R)0.5 * ATAN_XY, sa, ca;
      if (rng.word() & 1u) a += PI_R;
      R r = w * m_sqrt(f.sqrtv); m_sincos(a, &sa, &ca);
      f.p0 += r * ca; f.p1 += r * sa;
    } break;
    case 14: {
      R nx = f.tx, ny = f.ty;
      if (nx < (R)0.0) nx = nx * (R)2.0;
      if (ny < (R)0.0) ny = ny / (R)2.0;
      f.p0 += w * nx; f.p1 += w * ny;
    } break;
    case 15: {
      R nx = f.tx + x.c[2] * m_sin(f.ty * P(waves_dx2));
      R ny = f.ty + x.c[3] * m_sin(f.tx * P(waves_dy2));
      f.p0 += w * nx; f.p1 += w * ny;
    } break;
    case 16: { R r = m_div((R)2 * w, f.sqrtv + (R)1); f.p0 += r * f.ty; f.p1 += r * f.tx; } break;
    case 17: {
      R dx = m_tan((R)3 * f.ty), dy = m_tan((R)3 * f.tx);
      R nx = f.tx + x.c[4] * m_sin(dx), ny = f.ty + x.c[5] * m_sin(dy);
      f.p0 += w * nx; f.p1 += w * ny;
    } break;
    case 18: {
      R dx = w * m_exp(f.tx - (R)1.0), dy = PI_R * f.ty, sdy, cdy; m_sincos(dy, &sdy, &cdy);
      f.p0 += dx * cdy; f.p1 += dx * sdy;
    } break;
    case 19: {
      ANGLES(sina, cosa)
      R r = w * m_pow(f.sqrtv, sina);
      f.p0 += r * cosa; f.p1 += r * sina;
    } break;
    default: break;
  }
#undef ATAN_XY
#undef ANGLES
}

/* variations 20-98 */
/* Random words each of these variations draws, in order (variations.c). */
__device__ __forceinline__ int ext_draws(int v) {
  switch (v) {
    case 35: return 5;
    case 36: return 4;
    case 37: return 3;
    case 31: case 34: case 43: case 53: return 2;
    case 32: case 33: case 41: case 44: case 45: case 47: case 50: case 51: case 52: case 56: case 59: case 78:
      return 1;
    default: return 0;
  }
}

/* Kept out of line and free of references: inputs by value (the random words
 * already drawn, in the order the variation consumes them), result (p0, p1)
 * returned, so the call stays in registers. */
template <typename R> struct Vec2;
template <> struct Vec2<float> { typedef float2 T; };
template <> struct Vec2<double> { typedef double2 T; };

template <typename R>
__device__ __noinline__ typename Vec2<R>::T var_extended_impl(int v, R w, R tx, R ty, R sumsq, R sqrtv, R atan_xy, R sina,
                                                             R cosa, R atan_yx, R p0, R p1,
                                                             const XfS<R> *__restrict__ xp, uint32_t w0, uint32_t w1,
                                                             uint32_t w2, uint32_t w3, uint32_t w4) {
  Helper<R> f;
  f.tx = tx; f.ty = ty; f.sumsq = sumsq; f.sqrtv = sqrtv; f.atan_xy = atan_xy; f.sina = sina; f.cosa = cosa;
  f.atan_yx = atan_yx; f.p0 = p0; f.p1 = p1;
  const XfS<R> &x = *xp;
  switch (v) {
    case 20: {
      R a = f.tx * PI_R, sa, ca; m_sincos(a, &sa, &ca);
      R nx = ca * m_cosh(f.ty), ny = -sa * m_sinh(f.ty);
      f.p0 += w * nx; f.p1 += w * ny;
    } break;
    case 21: {
      R dx = x.c[4] * x.c[4] + EPS_R, r = f.sqrtv;
      r = w * (m_fmod(r + dx, (R)2 * dx) - dx + r * ((R)1 - dx));
      f.p0 += r * f.cosa; f.p1 += r * f.sina;
    } break;
    case 22: {
      R dx = PI_R * (x.c[4] * x.c[4] + EPS_R), dy = x.c[5], dx2 = (R)0.5 * dx;
      R a = f.atan_xy, r = w * f.sqrtv, sa, ca;
      a += (m_fmod(a + dy, dx) > dx2) ? -dx2 : dx2;
      m_sincos(a, &sa, &ca);
      f.p0 += r * ca; f.p1 += r * sa;
    } break;
    case 23: {
      R r = f.sqrtv, a = f.atan_xy, bdiff = P(blob_high) - P(blob_low);
      r = r * (P(blob_low) + bdiff * ((R)0.5 + (R)0.5 * m_sin(P(blob_waves) * a)));
      f.p0 += w * f.sina * r; f.p1 += w * f.cosa * r;
    } break;
    case 24: {
      R nx1 = m_cos(P(pdj_b) * f.tx), nx2 = m_sin(P(pdj_c) * f.tx);
      R ny1 = m_sin(P(pdj_a) * f.ty), ny2 = m_cos(P(pdj_d) * f.ty);
      f.p0 += w * (ny1 - nx1); f.p1 += w * (nx2 - ny2);
    } break;
    case 25: {
      R dy = P(fan2_y), dx = PI_R * (P(fan2_x) * P(fan2_x) + EPS_R), dx2 = (R)0.5 * dx;
      R a = f.atan_xy, sa, ca, r = w * f.sqrtv;
      R t = a + dy - dx * (R)(int)((a + dy) / dx);
      if (t > dx2) a = a - dx2; else a = a + dx2;
      m_sincos(a, &sa, &ca);
      f.p0 += r * sa; f.p1 += r * ca;
    } break;
    case 26: {
      R r = f.sqrtv, dx = P(rings2_val) * P(rings2_val) + EPS_R;
      r += (R)-2.0 * dx * (R)(int)((r + dx) / ((R)2.0 * dx)) + r * ((R)1.0 - dx);
      f.p0 += w * f.sina * r; f.p1 += w * f.cosa * r;
    } break;
    case 27: { R r = (w * (R)2.0) / (f.sqrtv + (R)1.0); f.p0 += r * f.tx; f.p1 += r * f.ty; } break;
    case 28: { R r = w / ((R)0.25 * f.sumsq + (R)1); f.p0 += r * f.tx; f.p1 += r * f.ty; } break;
    case 29: f.p0 += w * m_sin(f.tx); f.p1 += w * f.ty; break;
    case 30: {
      R t = (R)1.0 / (P(perspective_dist) - f.ty * P(persp_vsin));
      f.p0 += w * P(perspective_dist) * f.tx * t; f.p1 += w * P(persp_vfcos) * f.ty * t;
    } break;
    case 31: {
      R tmpr = u01<R>(w0) * (R)2 * PI_R, sinr, cosr; m_sincos(tmpr, &sinr, &cosr);
      R r = w * u01<R>(w1);
      f.p0 += f.tx * r * cosr; f.p1 += f.ty * r * sinr;
    } break;
    case 32: {
      int t_rnd = (int)m_trunc(P(julian_rN) * u01<R>(w0));
      R tmpr = (f.atan_yx + (R)2 * PI_R * (R)t_rnd) / P(julian_power);
      R r = w * m_pow(f.sumsq, P(julian_cn)), sina, cosa; m_sincos(tmpr, &sina, &cosa);
      f.p0 += r * cosa; f.p1 += r * sina;
    } break;
    case 33: {
      int t_rnd = (int)m_trunc(P(juliascope_rN) * u01<R>(w0));
      R tmpr, sina, cosa;
      if ((t_rnd & 1) == 0) tmpr = ((R)2 * PI_R * (R)t_rnd + f.atan_yx) / P(juliascope_power);
      else tmpr = ((R)2 * PI_R * (R)t_rnd - f.atan_yx) / P(juliascope_power);
      m_sincos(tmpr, &sina, &cosa);
      R r = w * m_pow(f.sumsq, P(juliascope_cn));
      f.p0 += r * cosa; f.p1 += r * sina;
    } break;
    case 34: {
      R tmpr = u01<R>(w0) * (R)2 * PI_R, sinr, cosr; m_sincos(tmpr, &sinr, &cosr);
      R r = w * u01<R>(w1);
      f.p0 += r * cosr; f.p1 += r * sinr;
    } break;
    case 35: {
      R ang = u01<R>(w0) * (R)2 * PI_R, sina, cosa; m_sincos(ang, &sina, &cosa);
      R g1 = u01<R>(w1), g2 = u01<R>(w2), g3 = u01<R>(w3), g4 = u01<R>(w4);
      R r = w * (g1 + g2 + g3 + g4 - (R)2.0);
      f.p0 += r * cosa; f.p1 += r * sina;
    } break;
    case 36: {
      R g1 = u01<R>(w0), g2 = u01<R>(w1), g3 = u01<R>(w2), g4 = u01<R>(w3);
      R rndG = w * (g1 + g2 + g3 + g4 - (R)2.0), sa, ca;
      R ra = f.sqrtv, tmpa = f.atan_yx + P(radialBlur_spinvar) * rndG;
      m_sincos(tmpa, &sa, &ca);
      R rz = P(radialBlur_zoomvar) * rndG - (R)1;
      f.p0 += ra * ca + rz * f.tx; f.p1 += ra * sa + rz * f.ty;
    } break;
    case 37: {
      int sl = (int)(u01<R>(w0) * P(pie_slices) + (R)0.5);
      R a = P(pie_rotation) + (R)2.0 * PI_R * ((R)sl + u01<R>(w1) * P(pie_thickness)) / P(pie_slices);
      R r = w * u01<R>(w2), sa, ca; m_sincos(a, &sa, &ca);
      f.p0 += r * ca; f.p1 += r * sa;
    } break;
    case 38: {
      R r_factor = m_pow(f.sumsq, P(ngon_power) / (R)2.0), theta = f.atan_yx;
      R b = (R)2 * PI_R / P(ngon_sides), phi = theta - (b * m_floor(theta / b));
      if (phi > b / (R)2) phi -= b;
      R amp = P(ngon_corners) * ((R)1.0 / (m_cos(phi) + EPS_R) - (R)1.0) + P(ngon_circle);
      amp /= (r_factor + EPS_R);
      f.p0 += w * f.tx * amp; f.p1 += w * f.ty * amp;
    } break;
    case 39: {
      R re = (R)1.0 + P(curl_c1) * f.tx + P(curl_c2) * (f.tx * f.tx - f.ty * f.ty);
      R im = P(curl_c1) * f.ty + (R)2.0 * P(curl_c2) * f.tx * f.ty;
      R r = w / (re * re + im * im);
      f.p0 += (f.tx * re + f.ty * im) * r; f.p1 += (f.ty * re - f.tx * im) * r;
    } break;
    case 40: {
      R rx = P(rectangles_x), ry = P(rectangles_y);
      if (rx == (R)0) f.p0 += w * f.tx;
      else f.p0 += w * (((R)2 * m_floor(f.tx / rx) + (R)1) * rx - f.tx);
      if (ry == (R)0) f.p1 += w * f.ty;
      else f.p1 += w * (((R)2 * m_floor(f.ty / ry) + (R)1) * ry - f.ty);
    } break;
    case 41: {
      R ang = u01<R>(w0) * w * PI_R, sinr, cosr; m_sincos(ang, &sinr, &cosr);
      f.p0 += w * sinr; f.p1 += w * (sinr * sinr) / cosr;
    } break;
    case 42: f.p0 += w * m_sin(f.tx) / m_cos(f.ty); f.p1 += w * m_tan(f.ty); break;
    case 43: {
      R a = u01<R>(w0); f.p0 += w * (a - (R)0.5);
      R b = u01<R>(w1); f.p1 += w * (b - (R)0.5);
    } break;
    case 44: {
      R ang = w * u01<R>(w0) * PI_R, r = w / (f.sumsq + EPS_R);
      R tanr = w * m_tan(ang) * r;
      f.p0 += tanr * m_cos(f.tx); f.p1 += tanr * m_sin(f.ty);
    } break;
    case 45: {
      R r = u01<R>(w0) * w * f.sqrtv, sinr, cosr; m_sincos(r, &sinr, &cosr);
      f.p0 += w * f.tx * (cosr + sinr); f.p1 += w * f.tx * (cosr - sinr);
    } break;
    case 46: {
      R r = w * f.sqrtv, cr = m_cos(r), icr = (R)1.0 / cr;
      f.p0 += w * f.tx;
      if (cr < (R)0) f.p1 += w * (icr + (R)1); else f.p1 += w * (icr - (R)1);
    } break;
    case 47: {
      R r = u01<R>(w0) * w * f.sqrtv, sinr, cosr; m_sincos(r, &sinr, &cosr);
      R diff = m_log10(sinr * sinr) + cosr;
      if (badvalue(diff)) diff = (R)-30.0;
      f.p0 += w * f.tx * diff; f.p1 += w * f.tx * (diff - sinr * PI_R);
    } break;
    case 48: {
      R s = f.tx * f.tx - f.ty * f.ty, r = w * m_sqrt((R)1.0 / (s * s + EPS_R));
      f.p0 += f.tx * r; f.p1 += f.ty * r;
    } break;
    case 49: {
      R t = P(disc2_timespi) * (f.tx + f.ty), sinr, cosr; m_sincos(t, &sinr, &cosr);
      R r = w * f.atan_xy / PI_R;
      f.p0 += (sinr + P(disc2_cosadd)) * r; f.p1 += (cosr + P(disc2_sinadd)) * r;
    } break;
    case 50: {
      R theta = P(super_shape_pm_4) * f.atan_yx + PI_4_R, st, ct; m_sincos(theta, &st, &ct);
      R t1 = m_pow(m_fabs(ct), P(super_shape_n2)), t2 = m_pow(m_fabs(st), P(super_shape_n3));
      R myrnd = P(super_shape_rnd);
      R r = w * ((myrnd * u01<R>(w0) + ((R)1.0 - myrnd) * f.sqrtv) - P(super_shape_holes)) *
            m_pow(t1 + t2, P(super_shape_pneg1_n1)) / f.sqrtv;
      f.p0 += r * f.tx; f.p1 += r * f.ty;
    } break;
    case 51: {
      R theta = f.atan_yx;
      R r = w * (u01<R>(w0) - P(flower_holes)) * m_cos(P(flower_petals) * theta) / f.sqrtv;
      f.p0 += r * f.tx; f.p1 += r * f.ty;
    } break;
    case 52: {
      R ct = f.tx / f.sqrtv;
      R r = w * (u01<R>(w0) - P(conic_holes)) * P(conic_eccentricity) /
            ((R)1 + P(conic_eccentricity) * ct) / f.sqrtv;
      f.p0 += r * f.tx; f.p1 += r * f.ty;
    } break;
    case 53: {
      R sr, cr; m_sincos(f.sqrtv, &sr, &cr);
      f.p0 += P(parabola_height) * w * sr * sr * u01<R>(w0);
      f.p1 += P(parabola_width) * w * cr * u01<R>(w1);
    } break;
    case 54: {
      R nx = f.tx, ny = f.ty;
      if (nx < (R)0.0) nx = nx * P(bent2_x);
      if (ny < (R)0.0) ny = ny * P(bent2_y);
      f.p0 += w * nx; f.p1 += w * ny;
    } break;
    case 55: {
      R x2y2 = f.sumsq, t = x2y2 + (R)1, x2 = (R)2 * f.tx, ps = -PI_2_R * P(bipolar_shift);
      R y = (R)0.5 * m_atan2((R)2.0 * f.ty, x2y2 - (R)1.0) + ps;
      if (y > PI_2_R) y = -PI_2_R + m_fmod(y + PI_2_R, PI_R);
      else if (y < -PI_2_R) y = PI_2_R - m_fmod(PI_2_R - y, PI_R);
      f.p0 += w * (R)0.25 * TWO_PI_R * m_log((t + x2) / (t - x2));
      f.p1 += w * TWO_PI_R * y;
    } break;
    case 56: {
      R roundX = m_rint(f.tx), roundY = m_rint(f.ty), offsetX = f.tx - roundX, offsetY = f.ty - roundY;
      if (u01<R>(w0) >= (R)0.75) {
        f.p0 += w * (offsetX * (R)0.5 + roundX); f.p1 += w * (offsetY * (R)0.5 + roundY);
      } else if (m_fabs(offsetX) >= m_fabs(offsetY)) {
        if (offsetX >= (R)0.0) {
          f.p0 += w * (offsetX * (R)0.5 + roundX + (R)0.25);
          f.p1 += w * (offsetY * (R)0.5 + roundY + (R)0.25 * offsetY / offsetX);
        } else {
          f.p0 += w * (offsetX * (R)0.5 + roundX - (R)0.25);
          f.p1 += w * (offsetY * (R)0.5 + roundY - (R)0.25 * offsetY / offsetX);
        }
      } else {
        if (offsetY >= (R)0.0) {
          f.p1 += w * (offsetY * (R)0.5 + roundY + (R)0.25);
          f.p0 += w * (offsetX * (R)0.5 + roundX + offsetX / offsetY * (R)0.25);
        } else {
          f.p1 += w * (offsetY * (R)0.5 + roundY - (R)0.25);
          f.p0 += w * (offsetX * (R)0.5 + roundX - offsetX / offsetY * (R)0.25);
        }
      }
    } break;
    case 57: {
      R wx = w * (R)1.3029400317411197908970256609023, y2 = f.ty * (R)2.0;
      R r = wx * m_sqrt(m_fabs(f.ty * f.tx) / (EPS_R + f.tx * f.tx + y2 * y2));
      f.p0 += r * f.tx; f.p1 += r * y2;
    } break;
    case 58: {
      R inv = (R)1.0 / P(cell_size);
      int xi = (int)m_floor(f.tx * inv), yi = (int)m_floor(f.ty * inv);
      R dx = f.tx - (R)xi * P(cell_size), dy = f.ty - (R)yi * P(cell_size);
      if (yi >= 0) {
        if (xi >= 0) { yi *= 2; xi *= 2; } else { yi *= 2; xi = -(2 * xi + 1); }
      } else {
        if (xi >= 0) { yi = -(2 * yi + 1); xi *= 2; } else { yi = -(2 * yi + 1); xi = -(2 * xi + 1); }
      }
      f.p0 += w * (dx + (R)xi * P(cell_size)); f.p1 -= w * (dy + (R)yi * P(cell_size));
    } break;
    case 59: {
      R a = f.atan_yx, lnr = (R)0.5 * m_log(f.sumsq), va = (R)2.0 * PI_R / P(cpow_power);
      R vc = P(cpow_r) / P(cpow_power), vd = P(cpow_i) / P(cpow_power);
      R ang = vc * a + vd * lnr + va * m_floor(P(cpow_power) * u01<R>(w0));
      R sa, ca, m = w * m_exp(vc * lnr - vd * a); m_sincos(ang, &sa, &ca);
      f.p0 += m * ca; f.p1 += m * sa;
    } break;
    case 60: {
      R xl = P(curve_xlength) * P(curve_xlength), yl = P(curve_ylength) * P(curve_ylength);
      if (xl < (R)1E-20) xl = (R)1E-20;
      if (yl < (R)1E-20) yl = (R)1E-20;
      f.p0 += w * (f.tx + P(curve_xamp) * m_exp(-f.ty * f.ty / xl));
      f.p1 += w * (f.ty + P(curve_yamp) * m_exp(-f.tx * f.tx / yl));
    } break;
    case 61: {
      R tmp = f.sumsq + (R)1.0, tmp2 = (R)2.0 * f.tx, r1 = m_sqrt(tmp + tmp2), r2 = m_sqrt(tmp - tmp2);
      R xmax = (r1 + r2) * (R)0.5, a1 = m_log(xmax + m_sqrt(xmax - (R)1.0)), a2 = -m_acos(f.tx / xmax);
      R wv = w / (R)11.57034632, snv, csv; m_sincos(a1, &snv, &csv);
      R snhu = m_sinh(a2), cshu = m_cosh(a2);
      if (f.ty > (R)0.0) snv = -snv;
      f.p0 += wv * cshu * csv; f.p1 += wv * snhu * snv;
    } break;
    case 62: {
      R tmp = f.sumsq + (R)1.0, x2 = (R)2.0 * f.tx;
      R xmax = (R)0.5 * (m_sqrt(tmp + x2) + m_sqrt(tmp - x2)), a = f.tx / xmax, b = (R)1.0 - a * a;
      R ssx = xmax - (R)1.0, wv = w / PI_2_R;
      if (b < (R)0) b = (R)0; else b = m_sqrt(b);
      if (ssx < (R)0) ssx = (R)0; else ssx = m_sqrt(ssx);
      f.p0 += wv * m_atan2(a, b);
      if (f.ty > (R)0) f.p1 += wv * m_log(xmax + ssx); else f.p1 -= wv * m_log(xmax + ssx);
    } break;
    case 63: {
      R a = f.atan_yx, lnr = (R)0.5 * m_log(f.sumsq), seb, ceb; m_sincos(P(escher_beta), &seb, &ceb);
      R vc = (R)0.5 * ((R)1.0 + ceb), vd = (R)0.5 * seb;
      R m = w * m_exp(vc * lnr - vd * a), n = vc * a + vd * lnr, sn, cn; m_sincos(n, &sn, &cn);
      f.p0 += m * cn; f.p1 += m * sn;
    } break;
    case 64: {
      R expx = m_exp(f.tx) * (R)0.5, expnx = (R)0.25 / expx, sn, cn; m_sincos(f.ty, &sn, &cn);
      R tmp = w / (expx + expnx - cn);
      f.p0 += tmp * (expx - expnx); f.p1 += tmp * sn;
    } break;
    case 65: {
      R xx = f.tx - P(lazysusan_x), yy = f.ty + P(lazysusan_y), r = m_sqrt(xx * xx + yy * yy), sina, cosa;
      if (r < w) {
        R a = m_atan2(yy, xx) + P(lazysusan_spin) + P(lazysusan_twist) * (w - r);
        m_sincos(a, &sina, &cosa);
        r = w * r;
        f.p0 += r * cosa + P(lazysusan_x); f.p1 += r * sina - P(lazysusan_y);
      } else {
        r = w * ((R)1.0 + P(lazysusan_space) / r);
        f.p0 += r * xx + P(lazysusan_x); f.p1 += r * yy - P(lazysusan_y);
      }
    } break;
    case 66: {
      R r2 = f.sumsq, w2 = w * w;
      if (r2 < w2) { R r = w * m_sqrt(w2 / r2 - (R)1.0); f.p0 += r * f.tx; f.p1 += r * f.ty; }
      else { f.p0 += w * f.tx; f.p1 += w * f.ty; }
    } break;
    case 67: break; /* pre_blur runs before the sum */
    case 68: {
      R mx = P(modulus_x), my = P(modulus_y), xr = (R)2 * mx, yr = (R)2 * my;
      if (f.tx > mx) f.p0 += w * (-mx + m_fmod(f.tx + mx, xr));
      else if (f.tx < -mx) f.p0 += w * (mx - m_fmod(mx - f.tx, xr));
      else f.p0 += w * f.tx;
      if (f.ty > my) f.p1 += w * (-my + m_fmod(f.ty + my, yr));
      else if (f.ty < -my) f.p1 += w * (my - m_fmod(my - f.ty, yr));
      else f.p1 += w * f.ty;
    } break;
    case 69: {
      R tpf = (R)2 * PI_R * P(oscope_frequency), t;
      if (P(oscope_damping) == (R)0.0) t = P(oscope_amplitude) * m_cos(tpf * f.tx) + P(oscope_separation);
      else
        t = P(oscope_amplitude) * m_exp(-m_fabs(f.tx) * P(oscope_damping)) * m_cos(tpf * f.tx) +
            P(oscope_separation);
      if (m_fabs(f.ty) <= t) { f.p0 += w * f.tx; f.p1 -= w * f.ty; }
      else { f.p0 += w * f.tx; f.p1 += w * f.ty; }
    } break;
    case 70: {
      R p2v = w / PI_R;
      f.p0 += p2v * f.atan_xy; f.p1 += p2v / (R)2.0 * m_log(f.sumsq);
    } break;
    case 71:
      f.p0 += w * (f.tx + P(popcorn2_x) * m_sin(m_tan(f.ty * P(popcorn2_c))));
      f.p1 += w * (f.ty + P(popcorn2_y) * m_sin(m_tan(f.tx * P(popcorn2_c))));
      break;
    case 72: {
      R t = f.sumsq, r = (R)1.0 / (f.sqrtv * (t + (R)1.0 / (w + EPS_R)));
      f.p0 += f.tx * r; f.p1 += f.ty * r;
    } break;
    case 73: {
      R sx2 = P(separation_x) * P(separation_x), sy2 = P(separation_y) * P(separation_y);
      if (f.tx > (R)0.0) f.p0 += w * (m_sqrt(f.tx * f.tx + sx2) - f.tx * P(separation_xinside));
      else f.p0 -= w * (m_sqrt(f.tx * f.tx + sx2) + f.tx * P(separation_xinside));
      if (f.ty > (R)0.0) f.p1 += w * (m_sqrt(f.ty * f.ty + sy2) - f.ty * P(separation_yinside));
      else f.p1 -= w * (m_sqrt(f.ty * f.ty + sy2) + f.ty * P(separation_yinside));
    } break;
    case 74:
      if (m_cos(f.tx * P(split_xsize) * PI_R) >= (R)0) f.p1 += w * f.ty; else f.p1 -= w * f.ty;
      if (m_cos(f.ty * P(split_ysize) * PI_R) >= (R)0) f.p0 += w * f.tx; else f.p0 -= w * f.tx;
      break;
    case 75:
      if (f.tx >= (R)0) f.p0 += w * (f.tx + P(splits_x)); else f.p0 += w * (f.tx - P(splits_x));
      if (f.ty >= (R)0) f.p1 += w * (f.ty + P(splits_y)); else f.p1 += w * (f.ty - P(splits_y));
      break;
    case 76: {
      R roundx = m_floor(f.tx + (R)0.5), offsetx = f.tx - roundx;
      f.p0 += w * (offsetx * ((R)1.0 - P(stripes_space)) + roundx);
      f.p1 += w * (f.ty + offsetx * offsetx * P(stripes_warp));
    } break;
    case 77: {
      R r = f.sqrtv, a = f.atan_yx + P(wedge_swirl) * r;
      R c = m_floor((P(wedge_count) * a + PI_R) * ONE_PI_R * (R)0.5);
      R comp_fac = (R)1 - P(wedge_angle) * P(wedge_count) * ONE_PI_R * (R)0.5, sa, ca;
      a = a * comp_fac + c * P(wedge_angle);
      m_sincos(a, &sa, &ca);
      r = w * (r + P(wedge_hole));
      f.p0 += r * ca; f.p1 += r * sa;
    } break;
    case 78: {
      R r = w * m_pow(f.sumsq, P(wedgeJulia_cn));
      int t_rnd = (int)(P(wedgeJulia_rN) * u01<R>(w0));
      R a = (f.atan_yx + (R)2 * PI_R * (R)t_rnd) / P(wedge_julia_power);
      R c = m_floor((P(wedge_julia_count) * a + PI_R) * ONE_PI_R * (R)0.5), sa, ca;
      a = a * P(wedgeJulia_cf) + c * P(wedge_julia_angle);
      m_sincos(a, &sa, &ca);
      f.p0 += r * ca; f.p1 += r * sa;
    } break;
    case 79: {
      R r = (R)1.0 / (f.sqrtv + EPS_R), a = f.atan_yx + P(wedge_sph_swirl) * r;
      R c = m_floor((P(wedge_sph_count) * a + PI_R) * ONE_PI_R * (R)0.5);
      R comp_fac = (R)1 - P(wedge_sph_angle) * P(wedge_sph_count) * ONE_PI_R * (R)0.5, sa, ca;
      a = a * comp_fac + c * P(wedge_sph_angle);
      m_sincos(a, &sa, &ca);
      r = w * (r + P(wedge_sph_hole));
      f.p0 += r * ca; f.p1 += r * sa;
    } break;
    case 80: {
      R r = f.sqrtv, a, sa, ca;
      if (r < w) a = f.atan_yx + P(whorl_inside) / (w - r);
      else a = f.atan_yx + P(whorl_outside) / (w - r);
      m_sincos(a, &sa, &ca);
      f.p0 += w * r * ca; f.p1 += w * r * sa;
    } break;
    case 81:
      f.p0 += w * (f.tx + P(waves2_scalex) * m_sin(f.ty * P(waves2_freqx)));
      f.p1 += w * (f.ty + P(waves2_scaley) * m_sin(f.tx * P(waves2_freqy)));
      break;
    case 82: {
      R e = m_exp(f.tx), c, s; m_sincos(f.ty, &s, &c);
      f.p0 += w * e * c; f.p1 += w * e * s;
    } break;
    case 83: f.p0 += w * (R)0.5 * m_log(f.sumsq); f.p1 += w * f.atan_yx; break;
    case 84: {
      R s, c; m_sincos(f.tx, &s, &c); R sh = m_sinh(f.ty), ch = m_cosh(f.ty);
      f.p0 += w * s * ch; f.p1 += w * c * sh;
    } break;
    case 85: {
      R s, c; m_sincos(f.tx, &s, &c); R sh = m_sinh(f.ty), ch = m_cosh(f.ty);
      f.p0 += w * c * ch; f.p1 -= w * s * sh;
    } break;
    case 86: {
      R s, c; m_sincos((R)2 * f.tx, &s, &c); R sh = m_sinh((R)2.0 * f.ty), ch = m_cosh((R)2.0 * f.ty);
      R den = (R)1.0 / (c + ch);
      f.p0 += w * den * s; f.p1 += w * den * sh;
    } break;
    case 87: {
      R s, c; m_sincos(f.tx, &s, &c); R sh = m_sinh(f.ty), ch = m_cosh(f.ty);
      R den = (R)2.0 / (m_cos((R)2 * f.tx) + m_cosh((R)2 * f.ty));
      f.p0 += w * den * c * ch; f.p1 += w * den * s * sh;
    } break;
    case 88: {
      R s, c; m_sincos(f.tx, &s, &c); R sh = m_sinh(f.ty), ch = m_cosh(f.ty);
      R den = (R)2.0 / (m_cosh((R)2.0 * f.ty) - m_cos((R)2.0 * f.tx));
      f.p0 += w * den * s * ch; f.p1 -= w * den * c * sh;
    } break;
    case 89: {
      R s, c; m_sincos((R)2.0 * f.tx, &s, &c); R sh = m_sinh((R)2.0 * f.ty), ch = m_cosh((R)2.0 * f.ty);
      R den = (R)1.0 / (ch - c);
      f.p0 += w * den * s; f.p1 += w * den * (R)-1 * sh;
    } break;
    case 90: {
      R s, c; m_sincos(f.ty, &s, &c); R sh = m_sinh(f.tx), ch = m_cosh(f.tx);
      f.p0 += w * sh * c; f.p1 += w * ch * s;
    } break;
    case 91: {
      R s, c; m_sincos(f.ty, &s, &c); R sh = m_sinh(f.tx), ch = m_cosh(f.tx);
      f.p0 += w * ch * c; f.p1 += w * sh * s;
    } break;
    case 92: {
      R s, c; m_sincos((R)2.0 * f.ty, &s, &c); R sh = m_sinh((R)2.0 * f.tx), ch = m_cosh((R)2.0 * f.tx);
      R den = (R)1.0 / (c + ch);
      f.p0 += w * den * sh; f.p1 += w * den * s;
    } break;
    case 93: {
      R s, c; m_sincos(f.ty, &s, &c); R sh = m_sinh(f.tx), ch = m_cosh(f.tx);
      R den = (R)2.0 / (m_cos((R)2.0 * f.ty) + m_cosh((R)2.0 * f.tx));
      f.p0 += w * den * c * ch; f.p1 -= w * den * s * sh;
    } break;
    case 94: {
      R s, c; m_sincos(f.ty, &s, &c); R sh = m_sinh(f.tx), ch = m_cosh(f.tx);
      R den = (R)2.0 / (m_cosh((R)2.0 * f.tx) - m_cos((R)2.0 * f.ty));
      f.p0 += w * den * sh * c; f.p1 -= w * den * ch * s;
    } break;
    case 95: {
      R s, c; m_sincos((R)2.0 * f.ty, &s, &c); R sh = m_sinh((R)2.0 * f.tx), ch = m_cosh((R)2.0 * f.tx);
      R den = (R)1.0 / (ch - c);
      f.p0 += w * den * sh; f.p1 += w * den * s;
    } break;
    case 96: {
      R s = m_sin(P(auger_freq) * f.tx), t = m_sin(P(auger_freq) * f.ty);
      R dy = f.ty + P(auger_weight) * (P(auger_scale) * s / (R)2.0 + m_fabs(f.ty) * s);
      R dx = f.tx + P(auger_weight) * (P(auger_scale) * t / (R)2.0 + m_fabs(f.tx) * t);
      f.p0 += w * (f.tx + P(auger_sym) * (dx - f.tx)); f.p1 += w * dy;
    } break;
    case 97: {
      R xpw = f.tx + w, xmw = f.tx - w;
      R avgr = w * ((R)2 + P(flux_spread)) *
               m_sqrt(m_sqrt(f.ty * f.ty + xpw * xpw) / m_sqrt(f.ty * f.ty + xmw * xmw));
      R avga = (m_atan2(f.ty, xmw) - m_atan2(f.ty, xpw)) * (R)0.5;
      f.p0 += avgr * m_cos(avga); f.p1 += avgr * m_sin(avga);
    } break;
    case 98: {
      R re_u = P(mobius_re_a) * f.tx - P(mobius_im_a) * f.ty + P(mobius_re_b);
      R im_u = P(mobius_re_a) * f.ty + P(mobius_im_a) * f.tx + P(mobius_im_b);
      R re_v = P(mobius_re_c) * f.tx - P(mobius_im_c) * f.ty + P(mobius_re_d);
      R im_v = P(mobius_re_c) * f.ty + P(mobius_im_c) * f.tx + P(mobius_im_d);
      R rad_v = w / (re_v * re_v + im_v * im_v);
      f.p0 += rad_v * (re_u * re_v + im_u * im_v); f.p1 += rad_v * (im_u * re_v - re_u * im_v);
    } break;
    default:
      break;
  }
  typename Vec2<R>::T r;
  r.x = f.p0;
  r.y = f.p1;
  return r;
}

/* The fields apply_xform reads first.  In FP32 they come in four vector
 * loads from the 16-byte aligned record in shared memory (c[0..3],
 * c[4..5]; color, color_speed, vis_adjusted, opacity; preblur, flags,
 * var_off, nvars) instead of twelve scalar ones. */
template <typename R> struct XfHead {
  R c0, c1, c2, c3, c4, c5, color, color_speed, vis_adjusted;
  int flags, var_off, nvars;
};
template <typename R> __device__ __forceinline__ void load_head(const XfS<R> &x, XfHead<R> &h) {
  h.c0 = x.c[0]; h.c1 = x.c[1]; h.c2 = x.c[2]; h.c3 = x.c[3]; h.c4 = x.c[4]; h.c5 = x.c[5];
  h.color = x.color; h.color_speed = x.color_speed; h.vis_adjusted = x.vis_adjusted;
  h.flags = x.flags; h.var_off = x.var_off; h.nvars = x.nvars;
}
template <> __device__ __forceinline__ void load_head<float>(const XfS<float> &x, XfHead<float> &h) {
  static_assert(offsetof(XfS<float>, c) == 0 && offsetof(XfS<float>, color) == 48 &&
                    offsetof(XfS<float>, preblur) == 64 && offsetof(XfS<float>, flags) == 68 &&
                    offsetof(XfS<float>, var_off) == 72 && offsetof(XfS<float>, nvars) == 76,
                "XfS<float> layout");
  const float4 a = *reinterpret_cast<const float4 *>(&x.c[0]);
  const float2 b = *reinterpret_cast<const float2 *>(&x.c[4]);
  const float4 m = *reinterpret_cast<const float4 *>(&x.color);
  const int4 q = *reinterpret_cast<const int4 *>(&x.preblur);
  h.c0 = a.x; h.c1 = a.y; h.c2 = a.z; h.c3 = a.w; h.c4 = b.x; h.c5 = b.y;
  h.color = m.x; h.color_speed = m.y; h.vis_adjusted = m.z;
  h.flags = q.y; h.var_off = q.z; h.nvars = q.w;
}
/* the post-transform, as two vector loads in FP32 (post[0..1], post[2..5]) */
template <typename R>
__device__ __forceinline__ void load_post(const XfS<R> &x, R &p0, R &p1, R &p2, R &p3, R &p4, R &p5) {
  p0 = x.post[0]; p1 = x.post[1]; p2 = x.post[2]; p3 = x.post[3]; p4 = x.post[4]; p5 = x.post[5];
}
template <>
__device__ __forceinline__ void load_post<float>(const XfS<float> &x, float &p0, float &p1, float &p2, float &p3,
                                                 float &p4, float &p5) {
  static_assert(offsetof(XfS<float>, post) == 24, "XfS<float> layout");
  const float2 a = *reinterpret_cast<const float2 *>(&x.post[0]);
  const float4 b = *reinterpret_cast<const float4 *>(&x.post[2]);
  p0 = a.x; p1 = a.y; p2 = b.x; p3 = b.y; p4 = b.z; p5 = b.w;
}

/* variations.c:2129-2399.  p = (x, y, color); q receives (x, y, color,
 * opacity).  Returns true when the result was a bad value and was replaced
 * by a random point. */
template <typename R, bool FULL, class G>
__device__ __forceinline__ bool apply_xform(const XfS<R> &x, const uint8_t *var_id, const R *var_w, R px, R py,
                                            R pc, R &qx, R &qy, R &qc, R &qo, G &rng) {
  Helper<R> f;
  XfHead<R> h;
  load_head<R>(x, h);
  R s1 = h.color_speed;
  qc = s1 * h.color + ((R)1.0 - s1) * pc;
  qo = h.vis_adjusted;
  f.tx = h.c0 * px + h.c2 * py + h.c4;
  f.ty = h.c1 * px + h.c3 * py + h.c5;
  if (FULL && (h.flags & F3G_F_PREBLUR)) {
    /* var67_pre_blur (variations.c:1480-1496) */
    R g1 = u01<R>(rng.word()), g2 = u01<R>(rng.word()), g3 = u01<R>(rng.word()), g4 = u01<R>(rng.word());
    R rndG = x.preblur * (g1 + g2 + g3 + g4 - (R)2.0);
    R rndA = u01<R>(rng.word()) * (R)2.0 * PI_R, sA, cA;
    m_sincos(rndA, &sA, &cA);
    f.tx += rndG * cA;
    f.ty += rndG * sA;
  }
  f.sumsq = f.tx * f.tx + f.ty * f.ty;
  f.sqrtv = m_sqrt(f.sumsq);
  f.atan_xy = f.sina = f.cosa = f.atan_yx = (R)0;
  /* with variations 0-19 only (FULL false) and F3G_LAZY_ANGLES, the angle
   * terms are computed by the variations that use them */
  if (FULL || !F3G_LAZY_ANGLES) {
    if (h.flags & F3G_F_ATAN_XY) f.atan_xy = pre_atan_xy<R>(f);
    if (h.flags & F3G_F_ANGLES) pre_angles<R>(f, f.sina, f.cosa);
    if (h.flags & F3G_F_ATAN_YX) f.atan_yx = m_atan2(f.ty, f.tx);
  }
  f.p0 = (R)0;
  f.p1 = (R)0;
  for (int k = 0; k < h.nvars; k++) {
    int v = var_id[h.var_off + k];
    R w = var_w[h.var_off + k];
    if (FULL && v >= 20) {
      /* draw this variation's words first, in its order, then call it */
      const int nd = ext_draws(v);
      uint32_t w0 = 0, w1 = 0, w2 = 0, w3 = 0, w4 = 0;
      if (nd > 0) w0 = rng.word();
      if (nd > 1) w1 = rng.word();
      if (nd > 2) w2 = rng.word();
      if (nd > 3) w3 = rng.word();
      if (nd > 4) w4 = rng.word();
      typename Vec2<R>::T r = var_extended_impl<R>(v, w, f.tx, f.ty, f.sumsq, f.sqrtv, f.atan_xy, f.sina, f.cosa,
                                                   f.atan_yx, f.p0, f.p1, &x, w0, w1, w2, w3, w4);
      f.p0 = r.x;
      f.p1 = r.y;
    } else
      var_basic<R, G, !FULL && F3G_LAZY_ANGLES>(v, w, f, x, rng);
  }
  if (h.flags & F3G_F_POST) {
    R p0, p1, p2, p3, p4, p5;
    load_post<R>(x, p0, p1, p2, p3, p4, p5);
    qx = p0 * f.p0 + p2 * f.p1 + p4;
    qy = p1 * f.p0 + p3 * f.p1 + p5;
  } else {
    qx = f.p0;
    qy = f.p1;
  }
  if (badvalue(qx) || badvalue(qy)) {
    qx = u11<R>(rng.word());
    qy = u11<R>(rng.word());
    return true;
  }
  return false;
}

#undef P

}  // namespace f3g

#endif
