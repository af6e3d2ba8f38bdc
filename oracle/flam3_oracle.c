/*
 * flam3_oracle.c -- TEST ORACLE (see flam3_oracle.h).  Plain C99, FP64.
 *
 * A restatement of the reference flam3 render path, written for this
 * project.  Every function cites the reference file:line it follows.  Only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
 */
#define _GNU_SOURCE
#include "flam3_oracle.h"

#include <limits.h>
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define F3O_EPS 1e-10                 /* private.h:47 */
#define F3O_PREFILTER_WHITE 255       /* private.h:46 */
#define F3O_WHITE_LEVEL 255           /* rect.c:38 */
#define F3O_GRAIN 16384               /* flam3.c:70 */
#define F3O_GRAIN_M1 16383
#define F3O_FUSE_27 15                /* rect.c:36-37 */
#define F3O_FUSE_28 100
#define F3O_DE_THRESH 100             /* filters.h:24 */

/* ======================================================================
 * ISAAC (isaac.c:25-110, isaac.h:49-52).  ub4 is unsigned long; the
 * arithmetic below is masked exactly where the reference masks it, so the
 * 64-bit intermediate values of the seeding mix are preserved.
 * ==================================================================== */
#define F3O_IND(mm, x) ((mm)[((x) >> 2) & (F3_RANDSIZ - 1)])
#define F3O_STEP(mix, a, b, mm, m, m2, r, x)                 \
  do {                                                       \
    x = *m;                                                  \
    a = ((a ^ (mix)) + *(m2++)) & 0xffffffff;                \
    *(m++) = y = (F3O_IND(mm, x) + a + b) & 0xffffffff;      \
    *(r++) = b = (F3O_IND(mm, y >> F3_RANDSIZL) + x) & 0xffffffff; \
  } while (0)

void f3o_isaac(randctx *ctx) {
  unsigned long a, b, x, y, *m, *mm, *m2, *r, *mend;
  mm = ctx->randmem;
  r = ctx->randrsl;
  a = ctx->randa;
  b = (ctx->randb + (++ctx->randc)) & 0xffffffff;
  for (m = mm, mend = m2 = m + (F3_RANDSIZ / 2); m < mend;) {
    F3O_STEP(a << 13, a, b, mm, m, m2, r, x);
    F3O_STEP(a >> 6, a, b, mm, m, m2, r, x);
    F3O_STEP(a << 2, a, b, mm, m, m2, r, x);
    F3O_STEP(a >> 16, a, b, mm, m, m2, r, x);
  }
  for (m2 = mm; m2 < mend;) {
    F3O_STEP(a << 13, a, b, mm, m, m2, r, x);
    F3O_STEP(a >> 6, a, b, mm, m, m2, r, x);
    F3O_STEP(a << 2, a, b, mm, m, m2, r, x);
    F3O_STEP(a >> 16, a, b, mm, m, m2, r, x);
  }
  ctx->randb = b;
  ctx->randa = a;
}

#define F3O_MIX(a, b, c, d, e, f, g, h) \
  do {                                  \
    a ^= b << 11; d += a; b += c;       \
    b ^= c >> 2;  e += b; c += d;       \
    c ^= d << 8;  f += c; d += e;       \
    d ^= e >> 16; g += d; e += f;       \
    e ^= f << 10; h += e; f += g;       \
    f ^= g >> 4;  a += f; g += h;       \
    g ^= h << 8;  b += g; h += a;       \
    h ^= a >> 9;  c += h; a += b;       \
  } while (0)

void f3o_irandinit(randctx *ctx, int flag) {
  int i;
  unsigned long a, b, c, d, e, f, g, h, *m, *r;
  ctx->randa = ctx->randb = ctx->randc = 0;
  m = ctx->randmem;
  r = ctx->randrsl;
  a = b = c = d = e = f = g = h = 0x9e3779b9;
  for (i = 0; i < 4; ++i) F3O_MIX(a, b, c, d, e, f, g, h);
  if (flag) {
    for (i = 0; i < F3_RANDSIZ; i += 8) {
      a += r[i]; b += r[i + 1]; c += r[i + 2]; d += r[i + 3];
      e += r[i + 4]; f += r[i + 5]; g += r[i + 6]; h += r[i + 7];
      F3O_MIX(a, b, c, d, e, f, g, h);
      m[i] = a; m[i + 1] = b; m[i + 2] = c; m[i + 3] = d;
      m[i + 4] = e; m[i + 5] = f; m[i + 6] = g; m[i + 7] = h;
    }
    for (i = 0; i < F3_RANDSIZ; i += 8) {
      a += m[i]; b += m[i + 1]; c += m[i + 2]; d += m[i + 3];
      e += m[i + 4]; f += m[i + 5]; g += m[i + 6]; h += m[i + 7];
      F3O_MIX(a, b, c, d, e, f, g, h);
      m[i] = a; m[i + 1] = b; m[i + 2] = c; m[i + 3] = d;
      m[i + 4] = e; m[i + 5] = f; m[i + 6] = g; m[i + 7] = h;
    }
  } else {
    for (i = 0; i < F3_RANDSIZ; i += 8) {
      F3O_MIX(a, b, c, d, e, f, g, h);
      m[i] = a; m[i + 1] = b; m[i + 2] = c; m[i + 3] = d;
      m[i + 4] = e; m[i + 5] = f; m[i + 6] = g; m[i + 7] = h;
    }
  }
  f3o_isaac(ctx);
  ctx->randcnt = F3_RANDSIZ;
}

/* isaac.h:49-52: results are handed out from the top of randrsl down */
unsigned long f3o_irand(randctx *r) {
  if (!r->randcnt--) {
    f3o_isaac(r);
    r->randcnt = F3_RANDSIZ - 1;
  }
  return r->randrsl[r->randcnt];
}

/* flam3.c:2494-2516 with the isaac_seed string given explicitly
 * (NULL seeds from the clock as the reference does). */
void f3o_init_rc(randctx *r, const char *seed) {
  memset(r->randrsl, 0, sizeof(r->randrsl));
  if (seed == NULL) {
    long s = (long)time(0);
    for (int i = 0; i < F3_RANDSIZ; i++) r->randrsl[i] = (unsigned long)s;
  } else {
    strncpy((char *)r->randrsl, seed, sizeof(r->randrsl));
  }
  f3o_irandinit(r, 1);
}

/* ======================================================================
 * Philox4x32-10 (Salmon et al., SC'11), the counter-based generator of the
 * CUDA path, restated so the oracle can replay its words.
 * ==================================================================== */
void f3o_philox4x32(uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; r++) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c0 = hi1 ^ c1 ^ k0;
    c1 = lo1;
    c2 = hi0 ^ c3 ^ k1;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* ======================================================================
 * Random-word source used by apply_xform / iterate: the reference's ISAAC
 * context, a caller-given word array, or the Philox stream of one chain.
 * Every consumer looks only at the low 32 bits of a draw, as the reference
 * does ((int)irand(...) & mask, (unsigned)irand(...) & mask).
 * ==================================================================== */
typedef struct {
  int kind; /* 0 isaac, 1 words, 2 philox */
  randctx *rc;
  const uint32_t *words;
  int nwords, pos;
  uint32_t key[2], ctr[4], buf[4];
  int bufpos;
} f3o_rng;

static uint32_t rng_word(f3o_rng *r) {
  if (r->kind == 0) return (uint32_t)f3o_irand(r->rc);
  if (r->kind == 1) return r->pos < r->nwords ? r->words[r->pos++] : 0u;
  if (r->bufpos == 4) {
    f3o_philox4x32(r->ctr, r->key, r->buf);
    r->ctr[1]++;
    r->bufpos = 0;
  }
  return r->buf[r->bufpos++];
}

/* flam3.c:2519-2544 */
static double rng_01(f3o_rng *r) { return ((int)rng_word(r) & 0xfffffff) / (double)0xfffffff; }
static double rng_11(f3o_rng *r) {
  return (((int)rng_word(r) & 0xfffffff) - 0x7ffffff) / (double)0x7ffffff;
}
static int rng_bit(f3o_rng *r) { return (int)rng_word(r) & 1; }

/* ======================================================================
 * Genome preparation
 * ==================================================================== */

/* interpolation.c:22-29 */
static double adjust_percentage(double in) {
  if (in == 0.0) return 0.0;
  return pow(10.0, -log(1.0 / in) / log(2));
}

/* interpolation.c:60-68 */
static int id_matrix(double s[3][2]) {
  return (s[0][0] == 1.0) && (s[0][1] == 0.0) && (s[1][0] == 0.0) && (s[1][1] == 1.0) &&
         (s[2][0] == 0.0) && (s[2][1] == 0.0);
}

/* variations.c:2016-2126: per-xform active-variation list and precalc flags */
int f3o_prepare_precalc_flags(flam3_genome *cp) {
  for (int i = 0; i < cp->num_xforms; i++) {
    flam3_xform *x = &cp->xform[i];
    double d = x->density;
    if (d < 0.0) {
      fprintf(stderr, "xform %d weight must be non-negative, not %g.\n", i, d);
      return 1;
    }
    if (i != cp->final_xform_index && d == 0.0) continue;
    int totnum = 0;
    x->vis_adjusted = adjust_percentage(x->opacity);
    x->precalc_angles_flag = 0;
    x->precalc_atan_xy_flag = 0;
    x->precalc_atan_yx_flag = 0;
    x->has_preblur = 0;
    x->has_post = !id_matrix(x->post);
    for (int j = 0; j < flam3_nvariations; j++) {
      if (x->var[j] == 0) continue;
      x->varFunc[totnum] = j;
      x->active_var_weights[totnum] = x->var[j];
      switch (j) {
        /* variations reading precalc_atan (atan2(tx, ty)) */
        case 5: case 6: case 7: case 8: case 12: case 13: case 22: case 25: case 49: case 70:
          x->precalc_atan_xy_flag = 1;
          break;
        /* variations reading precalc_sina / precalc_cosa */
        case 9: case 10: case 11: case 19: case 21: case 26:
          x->precalc_angles_flag = 1;
          break;
        case 23: /* blob reads both */
          x->precalc_atan_xy_flag = 1;
          x->precalc_angles_flag = 1;
          break;
        /* variations reading precalc_atanyx (atan2(ty, tx)) */
        case 32: case 33: case 36: case 38: case 50: case 51: case 52: case 59: case 63:
        case 77: case 78: case 79: case 80: case 83:
          x->precalc_atan_yx_flag = 1;
          break;
        case 67: /* pre_blur runs before the others, weight kept here */
          x->has_preblur = x->var[j];
          break;
        default:
          break;
      }
      totnum++;
    }
    x->num_active_vars = totnum;
  }
  return 0;
}

/* variations.c:1942-2014 */
void f3o_xform_precalc(flam3_genome *cp, int xi) {
  flam3_xform *xf = &cp->xform[xi];
  double ang = xf->perspective_angle * M_PI / 2.0;
  xf->persp_vsin = sin(ang);
  xf->persp_vfcos = xf->perspective_dist * cos(ang);

  xf->julian_rN = fabs(xf->julian_power);
  xf->julian_cn = xf->julian_dist / (double)xf->julian_power / 2.0;

  xf->juliascope_rN = fabs(xf->juliascope_power);
  xf->juliascope_cn = xf->juliascope_dist / (double)xf->juliascope_power / 2.0;

  sincos(xf->radial_blur_angle * M_PI / 2.0, &xf->radialBlur_spinvar, &xf->radialBlur_zoomvar);

  double dx = xf->c[2][0], dy = xf->c[2][1];
  xf->waves_dx2 = 1.0 / (dx * dx + F3O_EPS);
  xf->waves_dy2 = 1.0 / (dy * dy + F3O_EPS);

  double add = xf->disc2_twist, k;
  xf->disc2_timespi = xf->disc2_rot * M_PI;
  sincos(add, &xf->disc2_sinadd, &xf->disc2_cosadd);
  xf->disc2_cosadd -= 1;
  if (add > 2 * M_PI) {
    k = (1 + add - 2 * M_PI);
    xf->disc2_cosadd *= k;
    xf->disc2_sinadd *= k;
  }
  if (add < -2 * M_PI) {
    k = (1 + add + 2 * M_PI);
    xf->disc2_cosadd *= k;
    xf->disc2_sinadd *= k;
  }

  xf->super_shape_pm_4 = xf->super_shape_m / 4.0;
  xf->super_shape_pneg1_n1 = -1.0 / xf->super_shape_n1;

  xf->wedgeJulia_cf = 1.0 - xf->wedge_julia_angle * xf->wedge_julia_count * M_1_PI * 0.5;
  xf->wedgeJulia_rN = fabs(xf->wedge_julia_power);
  xf->wedgeJulia_cn = xf->wedge_julia_dist / xf->wedge_julia_power / 2.0;
}

/* flam3.c:148-163 */
static int check_unity_chaos(flam3_genome *cp) {
  int num_std = cp->num_xforms - (cp->final_xform_index >= 0);
  int unity = 1;
  for (int i = 0; i < num_std; i++)
    for (int j = 0; j < num_std; j++)
      if (fabs(cp->chaos[i][j] - 1.0) > F3O_EPS) unity = 0;
  return unity;
}

/* flam3.c:165-224: one 16384-entry row; xi < 0 is the raw-weight row */
static int create_chaos_distrib(flam3_genome *cp, int xi, unsigned short *row) {
  int num_std = cp->num_xforms - (cp->final_xform_index >= 0);
  double dr = 0.0;
  for (int i = 0; i < num_std; i++) {
    double d = cp->xform[i].density;
    if (xi >= 0) d *= cp->chaos[xi][i];
    if (d < 0.0) {
      fprintf(stderr, "xform weight must be non-negative, not %g.\n", d);
      return 1;
    }
    dr += d;
  }
  if (dr == 0.0) {
    fprintf(stderr, "cannot iterate empty flame.\n");
    return 1;
  }
  dr = dr / F3O_GRAIN;
  int j = 0;
  double t = cp->xform[0].density;
  if (xi >= 0) t *= cp->chaos[xi][0];
  double r = 0.0;
  for (int i = 0; i < F3O_GRAIN; i++) {
    while (r >= t) {
      j++;
      if (xi >= 0) t += cp->xform[j].density * cp->chaos[xi][j];
      else t += cp->xform[j].density;
    }
    row[i] = (unsigned short)j;
    r += dr;
  }
  return 0;
}

/* flam3.c:76-111 */
unsigned short *f3o_create_xform_distrib(flam3_genome *cp) {
  int numrows = cp->num_xforms - (cp->final_xform_index >= 0) + 1;
  unsigned short *xd = (unsigned short *)calloc((size_t)numrows * F3O_GRAIN, sizeof(unsigned short));
  if (create_chaos_distrib(cp, -1, xd)) {
    free(xd);
    return NULL;
  }
  cp->chaos_enable = 1 - check_unity_chaos(cp);
  if (cp->chaos_enable) {
    int dist_row = 0;
    for (int i = 0; i < cp->num_xforms; i++) {
      if (cp->final_xform_index == i) continue;
      dist_row++;
      if (create_chaos_distrib(cp, i, &xd[F3O_GRAIN * dist_row])) {
        free(xd);
        return NULL;
      }
    }
  }
  return xd;
}

/* ======================================================================
 * apply_xform and the 99 variations (variations.c:142-1938, 2129-2399).
 * Each case keeps the reference's operation order; random draws are taken
 * in the order the reference's statements take them.
 * ==================================================================== */
#define BADVALUE(x) (((x) != (x)) || ((x) > 1e10) || ((x) < -1e10))

typedef struct {
  double tx, ty;
  double precalc_atan, precalc_sina, precalc_cosa, precalc_sqrt, precalc_sumsq, precalc_atanyx;
  double p0, p1;
  flam3_xform *xf;
  f3o_rng *rng;
} iter_helper;

static void var_pre_blur(iter_helper *f, double weight) {
  /* variations.c:1480-1496 */
  double g1 = rng_01(f->rng);
  double g2 = rng_01(f->rng);
  double g3 = rng_01(f->rng);
  double g4 = rng_01(f->rng);
  double rndG = weight * (g1 + g2 + g3 + g4 - 2.0);
  double rndA = rng_01(f->rng) * 2.0 * M_PI;
  double sinA, cosA;
  sincos(rndA, &sinA, &cosA);
  f->tx += rndG * cosA;
  f->ty += rndG * sinA;
}

static void apply_variation(iter_helper *f, int v, double weight) {
  flam3_xform *x = f->xf;
  double tx = f->tx, ty = f->ty;
  switch (v) {
    case 0: /* linear 142 */
      f->p0 += weight * f->tx;
      f->p1 += weight * f->ty;
      break;
    case 1: /* sinusoidal 153 */
      f->p0 += weight * sin(f->tx);
      f->p1 += weight * sin(f->ty);
      break;
    case 2: { /* spherical 164 */
      double r2 = weight / (f->precalc_sumsq + F3O_EPS);
      f->p0 += r2 * f->tx;
      f->p1 += r2 * f->ty;
    } break;
    case 3: { /* swirl 178 */
      double r2 = f->precalc_sumsq, c1, c2;
      sincos(r2, &c1, &c2);
      double nx = c1 * f->tx - c2 * f->ty;
      double ny = c2 * f->tx + c1 * f->ty;
      f->p0 += weight * nx;
      f->p1 += weight * ny;
    } break;
    case 4: { /* horseshoe 202 */
      double r = weight / (f->precalc_sqrt + F3O_EPS);
      f->p0 += (f->tx - f->ty) * (f->tx + f->ty) * r;
      f->p1 += 2.0 * f->tx * f->ty * r;
    } break;
    case 5: { /* polar 218 */
      double nx = f->precalc_atan * M_1_PI;
      double ny = f->precalc_sqrt - 1.0;
      f->p0 += weight * nx;
      f->p1 += weight * ny;
    } break;
    case 6: { /* handkerchief 232 */
      double a = f->precalc_atan, r = f->precalc_sqrt;
      f->p0 += weight * r * sin(a + r);
      f->p1 += weight * r * cos(a - r);
    } break;
    case 7: { /* heart 246 */
      double a = f->precalc_sqrt * f->precalc_atan, ca, sa;
      double r = weight * f->precalc_sqrt;
      sincos(a, &sa, &ca);
      f->p0 += r * sa;
      f->p1 += (-r) * ca;
    } break;
    case 8: { /* disc 264 */
      double a = f->precalc_atan * M_1_PI;
      double r = M_PI * f->precalc_sqrt, sr, cr;
      sincos(r, &sr, &cr);
      f->p0 += weight * sr * a;
      f->p1 += weight * cr * a;
    } break;
    case 9: { /* spiral 282 */
      double r = f->precalc_sqrt + F3O_EPS;
      double r1 = weight / r, sr, cr;
      sincos(r, &sr, &cr);
      f->p0 += r1 * (f->precalc_cosa + sr);
      f->p1 += r1 * (f->precalc_sina - cr);
    } break;
    case 10: { /* hyperbolic 298 */
      double r = f->precalc_sqrt + F3O_EPS;
      f->p0 += weight * f->precalc_sina / r;
      f->p1 += weight * f->precalc_cosa * r;
    } break;
    case 11: { /* diamond 311 */
      double r = f->precalc_sqrt, sr, cr;
      sincos(r, &sr, &cr);
      f->p0 += weight * f->precalc_sina * cr;
      f->p1 += weight * f->precalc_cosa * sr;
    } break;
    case 12: { /* ex 326 */
      double a = f->precalc_atan, r = f->precalc_sqrt;
      double n0 = sin(a + r), n1 = cos(a - r);
      double m0 = n0 * n0 * n0 * r, m1 = n1 * n1 * n1 * r;
      f->p0 += weight * (m0 + m1);
      f->p1 += weight * (m0 - m1);
    } break;
    case 13: { /* julia 350 */
      double r, a = 0.5 * f->precalc_atan, sa, ca;
      if (rng_bit(f->rng)) a += M_PI;
      r = weight * sqrt(f->precalc_sqrt);
      sincos(a, &sa, &ca);
      f->p0 += r * ca;
      f->p1 += r * sa;
    } break;
    case 14: { /* bent 375 */
      double nx = f->tx, ny = f->ty;
      if (nx < 0.0) nx = nx * 2.0;
      if (ny < 0.0) ny = ny / 2.0;
      f->p0 += weight * nx;
      f->p1 += weight * ny;
    } break;
    case 15: { /* waves 396 */
      double c10 = x->c[1][0], c11 = x->c[1][1];
      double nx = f->tx + c10 * sin(f->ty * x->waves_dx2);
      double ny = f->ty + c11 * sin(f->tx * x->waves_dy2);
      f->p0 += weight * nx;
      f->p1 += weight * ny;
    } break;
    case 16: { /* fisheye 415 */
      double r = f->precalc_sqrt;
      r = 2 * weight / (r + 1);
      f->p0 += r * f->ty;
      f->p1 += r * f->tx;
    } break;
    case 17: { /* popcorn 433 */
      double dx = tan(3 * f->ty), dy = tan(3 * f->tx);
      double nx = f->tx + x->c[2][0] * sin(dx);
      double ny = f->ty + x->c[2][1] * sin(dy);
      f->p0 += weight * nx;
      f->p1 += weight * ny;
    } break;
    case 18: { /* exponential 452 */
      double dx = weight * exp(f->tx - 1.0), dy = M_PI * f->ty, sdy, cdy;
      sincos(dy, &sdy, &cdy);
      f->p0 += dx * cdy;
      f->p1 += dx * sdy;
    } break;
    case 19: { /* power 472 */
      double r = weight * pow(f->precalc_sqrt, f->precalc_sina);
      f->p0 += r * f->precalc_cosa;
      f->p1 += r * f->precalc_sina;
    } break;
    case 20: { /* cosine 489 */
      double a = f->tx * M_PI, sa, ca;
      sincos(a, &sa, &ca);
      double nx = ca * cosh(f->ty), ny = -sa * sinh(f->ty);
      f->p0 += weight * nx;
      f->p1 += weight * ny;
    } break;
    case 21: { /* rings 508 */
      double dx = x->c[2][0] * x->c[2][0] + F3O_EPS;
      double r = f->precalc_sqrt;
      r = weight * (fmod(r + dx, 2 * dx) - dx + r * (1 - dx));
      f->p0 += r * f->precalc_cosa;
      f->p1 += r * f->precalc_sina;
    } break;
    case 22: { /* fan 528 */
      double dx = M_PI * (x->c[2][0] * x->c[2][0] + F3O_EPS);
      double dy = x->c[2][1], dx2 = 0.5 * dx;
      double a = f->precalc_atan, r = weight * f->precalc_sqrt, sa, ca;
      a += (fmod(a + dy, dx) > dx2) ? -dx2 : dx2;
      sincos(a, &sa, &ca);
      f->p0 += r * ca;
      f->p1 += r * sa;
    } break;
    case 23: { /* blob 557 */
      double r = f->precalc_sqrt, a = f->precalc_atan;
      double bdiff = x->blob_high - x->blob_low;
      r = r * (x->blob_low + bdiff * (0.5 + 0.5 * sin(x->blob_waves * a)));
      f->p0 += weight * f->precalc_sina * r;
      f->p1 += weight * f->precalc_cosa * r;
    } break;
    case 24: { /* pdj 579 */
      double nx1 = cos(x->pdj_b * f->tx), nx2 = sin(x->pdj_c * f->tx);
      double ny1 = sin(x->pdj_a * f->ty), ny2 = cos(x->pdj_d * f->ty);
      f->p0 += weight * (ny1 - nx1);
      f->p1 += weight * (nx2 - ny2);
    } break;
    case 25: { /* fan2 598 */
      double dy = x->fan2_y;
      double dx = M_PI * (x->fan2_x * x->fan2_x + F3O_EPS), dx2 = 0.5 * dx;
      double a = f->precalc_atan, sa, ca, r = weight * f->precalc_sqrt;
      double t = a + dy - dx * (int)((a + dy) / dx);
      if (t > dx2) a = a - dx2;
      else a = a + dx2;
      sincos(a, &sa, &ca);
      f->p0 += r * sa;
      f->p1 += r * ca;
    } break;
    case 26: { /* rings2 640 */
      double r = f->precalc_sqrt;
      double dx = x->rings2_val * x->rings2_val + F3O_EPS;
      r += -2.0 * dx * (int)((r + dx) / (2.0 * dx)) + r * (1.0 - dx);
      f->p0 += weight * f->precalc_sina * r;
      f->p1 += weight * f->precalc_cosa * r;
    } break;
    case 27: { /* eyefish 659 */
      double r = (weight * 2.0) / (f->precalc_sqrt + 1.0);
      f->p0 += r * f->tx;
      f->p1 += r * f->ty;
    } break;
    case 28: { /* bubble 671 */
      double r = weight / (0.25 * (f->precalc_sumsq) + 1);
      f->p0 += r * f->tx;
      f->p1 += r * f->ty;
    } break;
    case 29: /* cylinder 680 */
      f->p0 += weight * sin(f->tx);
      f->p1 += weight * f->ty;
      break;
    case 30: { /* perspective 687 */
      double t = 1.0 / (x->perspective_dist - f->ty * x->persp_vsin);
      f->p0 += weight * x->perspective_dist * f->tx * t;
      f->p1 += weight * x->persp_vfcos * f->ty * t;
    } break;
    case 31: { /* noise 696 */
      double tmpr = rng_01(f->rng) * 2 * M_PI, sinr, cosr;
      sincos(tmpr, &sinr, &cosr);
      double r = weight * rng_01(f->rng);
      f->p0 += f->tx * r * cosr;
      f->p1 += f->ty * r * sinr;
    } break;
    case 32: { /* julian 710 */
      int t_rnd = (int)trunc((x->julian_rN) * rng_01(f->rng));
      double tmpr = (f->precalc_atanyx + 2 * M_PI * t_rnd) / x->julian_power;
      double r = weight * pow(f->precalc_sumsq, x->julian_cn), sina, cosa;
      sincos(tmpr, &sina, &cosa);
      f->p0 += r * cosa;
      f->p1 += r * sina;
    } break;
    case 33: { /* juliascope 725 */
      int t_rnd = (int)trunc((x->juliascope_rN) * rng_01(f->rng));
      double tmpr, r, sina, cosa;
      if ((t_rnd & 1) == 0)
        tmpr = (2 * M_PI * t_rnd + f->precalc_atanyx) / x->juliascope_power;
      else
        tmpr = (2 * M_PI * t_rnd - f->precalc_atanyx) / x->juliascope_power;
      sincos(tmpr, &sina, &cosa);
      r = weight * pow(f->precalc_sumsq, x->juliascope_cn);
      f->p0 += r * cosa;
      f->p1 += r * sina;
    } break;
    case 34: { /* blur 746 */
      double tmpr = rng_01(f->rng) * 2 * M_PI, sinr, cosr;
      sincos(tmpr, &sinr, &cosr);
      double r = weight * rng_01(f->rng);
      f->p0 += r * cosr;
      f->p1 += r * sinr;
    } break;
    case 35: { /* gaussian_blur 760 */
      double ang = rng_01(f->rng) * 2 * M_PI, sina, cosa;
      sincos(ang, &sina, &cosa);
      double g1 = rng_01(f->rng), g2 = rng_01(f->rng), g3 = rng_01(f->rng), g4 = rng_01(f->rng);
      double r = weight * (g1 + g2 + g3 + g4 - 2.0);
      f->p0 += r * cosa;
      f->p1 += r * sina;
    } break;
    case 36: { /* radial_blur 775 */
      double g1 = rng_01(f->rng), g2 = rng_01(f->rng), g3 = rng_01(f->rng), g4 = rng_01(f->rng);
      double rndG = weight * (g1 + g2 + g3 + g4 - 2.0), sa, ca;
      double ra = f->precalc_sqrt;
      double tmpa = f->precalc_atanyx + x->radialBlur_spinvar * rndG;
      sincos(tmpa, &sa, &ca);
      double rz = x->radialBlur_zoomvar * rndG - 1;
      f->p0 += ra * ca + rz * f->tx;
      f->p1 += ra * sa + rz * f->ty;
    } break;
    case 37: { /* pie 795 */
      int sl = (int)(rng_01(f->rng) * x->pie_slices + 0.5);
      double a = x->pie_rotation + 2.0 * M_PI * (sl + rng_01(f->rng) * x->pie_thickness) / x->pie_slices;
      double r = weight * rng_01(f->rng), sa, ca;
      sincos(a, &sa, &ca);
      f->p0 += r * ca;
      f->p1 += r * sa;
    } break;
    case 38: { /* ngon 811 */
      double r_factor = pow(f->precalc_sumsq, x->ngon_power / 2.0);
      double theta = f->precalc_atanyx;
      double b = 2 * M_PI / x->ngon_sides;
      double phi = theta - (b * floor(theta / b));
      if (phi > b / 2) phi -= b;
      double amp = x->ngon_corners * (1.0 / (cos(phi) + F3O_EPS) - 1.0) + x->ngon_circle;
      amp /= (r_factor + F3O_EPS);
      f->p0 += weight * f->tx * amp;
      f->p1 += weight * f->ty * amp;
    } break;
    case 39: { /* curl 832 */
      double re = 1.0 + x->curl_c1 * f->tx + x->curl_c2 * (f->tx * f->tx - f->ty * f->ty);
      double im = x->curl_c1 * f->ty + 2.0 * x->curl_c2 * f->tx * f->ty;
      double r = weight / (re * re + im * im);
      f->p0 += (f->tx * re + f->ty * im) * r;
      f->p1 += (f->ty * re - f->tx * im) * r;
    } break;
    case 40: /* rectangles 843 */
      if (x->rectangles_x == 0) f->p0 += weight * f->tx;
      else f->p0 += weight * ((2 * floor(f->tx / x->rectangles_x) + 1) * x->rectangles_x - f->tx);
      if (x->rectangles_y == 0) f->p1 += weight * f->ty;
      else f->p1 += weight * ((2 * floor(f->ty / x->rectangles_y) + 1) * x->rectangles_y - f->ty);
      break;
    case 41: { /* arch 857 */
      double ang = rng_01(f->rng) * weight * M_PI, sinr, cosr;
      sincos(ang, &sinr, &cosr);
      f->p0 += weight * sinr;
      f->p1 += weight * (sinr * sinr) / cosr;
    } break;
    case 42: /* tangent 885 */
      f->p0 += weight * sin(f->tx) / cos(f->ty);
      f->p1 += weight * tan(f->ty);
      break;
    case 43: { /* square 900 */
      double a = rng_01(f->rng);
      f->p0 += weight * (a - 0.5);
      double b = rng_01(f->rng);
      f->p1 += weight * (b - 0.5);
    } break;
    case 44: { /* rays 915 */
      double ang = weight * rng_01(f->rng) * M_PI;
      double r = weight / (f->precalc_sumsq + F3O_EPS);
      double tanr = weight * tan(ang) * r;
      f->p0 += tanr * cos(f->tx);
      f->p1 += tanr * sin(f->ty);
    } break;
    case 45: { /* blade 946 */
      double r = rng_01(f->rng) * weight * f->precalc_sqrt, sinr, cosr;
      sincos(r, &sinr, &cosr);
      f->p0 += weight * f->tx * (cosr + sinr);
      f->p1 += weight * f->tx * (cosr - sinr);
    } break;
    case 46: { /* secant2 976 */
      double r = weight * f->precalc_sqrt;
      double cr = cos(r), icr = 1.0 / cr;
      f->p0 += weight * f->tx;
      if (cr < 0) f->p1 += weight * (icr + 1);
      else f->p1 += weight * (icr - 1);
    } break;
    case 47: { /* twintrian 998 */
      double r = rng_01(f->rng) * weight * f->precalc_sqrt, sinr, cosr, diff;
      sincos(r, &sinr, &cosr);
      diff = log10(sinr * sinr) + cosr;
      if (BADVALUE(diff)) diff = -30.0;
      f->p0 += weight * f->tx * diff;
      f->p1 += weight * f->tx * (diff - sinr * M_PI);
    } break;
    case 48: { /* cross 1033 */
      double s = f->tx * f->tx - f->ty * f->ty;
      double r = weight * sqrt(1.0 / (s * s + F3O_EPS));
      f->p0 += f->tx * r;
      f->p1 += f->ty * r;
    } break;
    case 49: { /* disc2 1054 */
      double t = x->disc2_timespi * (f->tx + f->ty), sinr, cosr;
      sincos(t, &sinr, &cosr);
      double r = weight * f->precalc_atan / M_PI;
      f->p0 += (sinr + x->disc2_cosadd) * r;
      f->p1 += (cosr + x->disc2_sinadd) * r;
    } break;
    case 50: { /* super_shape 1092 */
      double theta = x->super_shape_pm_4 * f->precalc_atanyx + M_PI_4, st, ct;
      sincos(theta, &st, &ct);
      double t1 = fabs(ct);
      t1 = pow(t1, x->super_shape_n2);
      double t2 = fabs(st);
      t2 = pow(t2, x->super_shape_n3);
      double myrnd = x->super_shape_rnd;
      double r = weight * ((myrnd * rng_01(f->rng) + (1.0 - myrnd) * f->precalc_sqrt) - x->super_shape_holes) *
                 pow(t1 + t2, x->super_shape_pneg1_n1) / f->precalc_sqrt;
      f->p0 += r * f->tx;
      f->p1 += r * f->ty;
    } break;
    case 51: { /* flower 1118 */
      double theta = f->precalc_atanyx;
      double r = weight * (rng_01(f->rng) - x->flower_holes) * cos(x->flower_petals * theta) / f->precalc_sqrt;
      f->p0 += r * f->tx;
      f->p1 += r * f->ty;
    } break;
    case 52: { /* conic 1133 */
      double ct = f->tx / f->precalc_sqrt;
      double r = weight * (rng_01(f->rng) - x->conic_holes) * x->conic_eccentricity /
                 (1 + x->conic_eccentricity * ct) / f->precalc_sqrt;
      f->p0 += r * f->tx;
      f->p1 += r * f->ty;
    } break;
    case 53: { /* parabola 1148 */
      double r = f->precalc_sqrt, sr, cr;
      sincos(r, &sr, &cr);
      f->p0 += x->parabola_height * weight * sr * sr * rng_01(f->rng);
      f->p1 += x->parabola_width * weight * cr * rng_01(f->rng);
    } break;
    case 54: { /* bent2 1164 */
      double nx = f->tx, ny = f->ty;
      if (nx < 0.0) nx = nx * x->bent2_x;
      if (ny < 0.0) ny = ny * x->bent2_y;
      f->p0 += weight * nx;
      f->p1 += weight * ny;
    } break;
    case 55: { /* bipolar 1180 */
      double x2y2 = f->precalc_sumsq, t = x2y2 + 1, x2 = 2 * f->tx;
      double ps = -M_PI_2 * x->bipolar_shift;
      double y = 0.5 * atan2(2.0 * f->ty, x2y2 - 1.0) + ps;
      if (y > M_PI_2) y = -M_PI_2 + fmod(y + M_PI_2, M_PI);
      else if (y < -M_PI_2) y = M_PI_2 - fmod(M_PI_2 - y, M_PI);
      f->p0 += weight * 0.25 * M_2_PI * log((t + x2) / (t - x2));
      f->p1 += weight * M_2_PI * y;
    } break;
    case 56: { /* boarders 1199 */
      double roundX = rint(f->tx), roundY = rint(f->ty);
      double offsetX = f->tx - roundX, offsetY = f->ty - roundY;
      if (rng_01(f->rng) >= 0.75) {
        f->p0 += weight * (offsetX * 0.5 + roundX);
        f->p1 += weight * (offsetY * 0.5 + roundY);
      } else {
        if (fabs(offsetX) >= fabs(offsetY)) {
          if (offsetX >= 0.0) {
            f->p0 += weight * (offsetX * 0.5 + roundX + 0.25);
            f->p1 += weight * (offsetY * 0.5 + roundY + 0.25 * offsetY / offsetX);
          } else {
            f->p0 += weight * (offsetX * 0.5 + roundX - 0.25);
            f->p1 += weight * (offsetY * 0.5 + roundY - 0.25 * offsetY / offsetX);
          }
        } else {
          if (offsetY >= 0.0) {
            f->p1 += weight * (offsetY * 0.5 + roundY + 0.25);
            f->p0 += weight * (offsetX * 0.5 + roundX + offsetX / offsetY * 0.25);
          } else {
            f->p1 += weight * (offsetY * 0.5 + roundY - 0.25);
            f->p0 += weight * (offsetX * 0.5 + roundX - offsetX / offsetY * 0.25);
          }
        }
      }
    } break;
    case 57: { /* butterfly 1238 */
      double wx = weight * 1.3029400317411197908970256609023;
      double y2 = f->ty * 2.0;
      double r = wx * sqrt(fabs(f->ty * f->tx) / (F3O_EPS + f->tx * f->tx + y2 * y2));
      f->p0 += r * f->tx;
      f->p1 += r * y2;
    } break;
    case 58: { /* cell 1253 */
      double inv_cell_size = 1.0 / x->cell_size;
      int xi = (int)floor(f->tx * inv_cell_size);
      int yi = (int)floor(f->ty * inv_cell_size);
      double dx = f->tx - xi * x->cell_size;
      double dy = f->ty - yi * x->cell_size;
      if (yi >= 0) {
        if (xi >= 0) { yi *= 2; xi *= 2; }
        else { yi *= 2; xi = -(2 * xi + 1); }
      } else {
        if (xi >= 0) { yi = -(2 * yi + 1); xi *= 2; }
        else { yi = -(2 * yi + 1); xi = -(2 * xi + 1); }
      }
      f->p0 += weight * (dx + xi * x->cell_size);
      f->p1 -= weight * (dy + yi * x->cell_size);
    } break;
    case 59: { /* cpow 1291 */
      double a = f->precalc_atanyx;
      double lnr = 0.5 * log(f->precalc_sumsq);
      double va = 2.0 * M_PI / x->cpow_power;
      double vc = x->cpow_r / x->cpow_power;
      double vd = x->cpow_i / x->cpow_power;
      double ang = vc * a + vd * lnr + va * floor(x->cpow_power * rng_01(f->rng));
      double sa, ca, m = weight * exp(vc * lnr - vd * a);
      sincos(ang, &sa, &ca);
      f->p0 += m * ca;
      f->p1 += m * sa;
    } break;
    case 60: { /* curve 1312 */
      double pc_xlen = x->curve_xlength * x->curve_xlength;
      double pc_ylen = x->curve_ylength * x->curve_ylength;
      if (pc_xlen < 1E-20) pc_xlen = 1E-20;
      if (pc_ylen < 1E-20) pc_ylen = 1E-20;
      f->p0 += weight * (f->tx + x->curve_xamp * exp(-f->ty * f->ty / pc_xlen));
      f->p1 += weight * (f->ty + x->curve_yamp * exp(-f->tx * f->tx / pc_ylen));
    } break;
    case 61: { /* edisc 1328 */
      double tmp = f->precalc_sumsq + 1.0, tmp2 = 2.0 * f->tx;
      double r1 = sqrt(tmp + tmp2), r2 = sqrt(tmp - tmp2);
      double xmax = (r1 + r2) * 0.5;
      double a1 = log(xmax + sqrt(xmax - 1.0));
      double a2 = -acos(f->tx / xmax);
      double w = weight / 11.57034632, snv, csv, snhu, cshu;
      sincos(a1, &snv, &csv);
      snhu = sinh(a2);
      cshu = cosh(a2);
      if (f->ty > 0.0) snv = -snv;
      f->p0 += w * cshu * csv;
      f->p1 += w * snhu * snv;
    } break;
    case 62: { /* elliptic 1354 */
      double tmp = f->precalc_sumsq + 1.0, x2 = 2.0 * f->tx;
      double xmax = 0.5 * (sqrt(tmp + x2) + sqrt(tmp - x2));
      double a = f->tx / xmax, b = 1.0 - a * a, ssx = xmax - 1.0;
      double w = weight / M_PI_2;
      if (b < 0) b = 0;
      else b = sqrt(b);
      if (ssx < 0) ssx = 0;
      else ssx = sqrt(ssx);
      f->p0 += w * atan2(a, b);
      if (f->ty > 0) f->p1 += w * log(xmax + ssx);
      else f->p1 -= w * log(xmax + ssx);
    } break;
    case 63: { /* escher 1385 */
      double seb, ceb, vc, vd, m, n, sn, cn;
      double a = f->precalc_atanyx;
      double lnr = 0.5 * log(f->precalc_sumsq);
      sincos(x->escher_beta, &seb, &ceb);
      vc = 0.5 * (1.0 + ceb);
      vd = 0.5 * seb;
      m = weight * exp(vc * lnr - vd * a);
      n = vc * a + vd * lnr;
      sincos(n, &sn, &cn);
      f->p0 += m * cn;
      f->p1 += m * sn;
    } break;
    case 64: { /* foci 1412 */
      double expx = exp(f->tx) * 0.5, expnx = 0.25 / expx, sn, cn, tmp;
      sincos(f->ty, &sn, &cn);
      tmp = weight / (expx + expnx - cn);
      f->p0 += tmp * (expx - expnx);
      f->p1 += tmp * sn;
    } break;
    case 65: { /* lazysusan 1428 */
      double xx = f->tx - x->lazysusan_x, yy = f->ty + x->lazysusan_y;
      double r = sqrt(xx * xx + yy * yy), sina, cosa;
      if (r < weight) {
        double a = atan2(yy, xx) + x->lazysusan_spin + x->lazysusan_twist * (weight - r);
        sincos(a, &sina, &cosa);
        r = weight * r;
        f->p0 += r * cosa + x->lazysusan_x;
        f->p1 += r * sina - x->lazysusan_y;
      } else {
        r = weight * (1.0 + x->lazysusan_space / r);
        f->p0 += r * xx + x->lazysusan_x;
        f->p1 += r * yy - x->lazysusan_y;
      }
    } break;
    case 66: { /* loonie 1456 */
      double r2 = f->precalc_sumsq, w2 = weight * weight;
      if (r2 < w2) {
        double r = weight * sqrt(w2 / r2 - 1.0);
        f->p0 += r * f->tx;
        f->p1 += r * f->ty;
      } else {
        f->p0 += weight * f->tx;
        f->p1 += weight * f->ty;
      }
    } break;
    case 67: /* pre_blur is applied before the sum (apply_xform), no-op here */
      break;
    case 68: { /* modulus 1498 */
      double xr = 2 * x->modulus_x, yr = 2 * x->modulus_y;
      if (f->tx > x->modulus_x) f->p0 += weight * (-x->modulus_x + fmod(f->tx + x->modulus_x, xr));
      else if (f->tx < -x->modulus_x) f->p0 += weight * (x->modulus_x - fmod(x->modulus_x - f->tx, xr));
      else f->p0 += weight * f->tx;
      if (f->ty > x->modulus_y) f->p1 += weight * (-x->modulus_y + fmod(f->ty + x->modulus_y, yr));
      else if (f->ty < -x->modulus_y) f->p1 += weight * (x->modulus_y - fmod(x->modulus_y - f->ty, yr));
      else f->p1 += weight * f->ty;
    } break;
    case 69: { /* oscilloscope 1521 */
      double tpf = 2 * M_PI * x->oscope_frequency, t;
      if (x->oscope_damping == 0.0)
        t = x->oscope_amplitude * cos(tpf * f->tx) + x->oscope_separation;
      else
        t = x->oscope_amplitude * exp(-fabs(f->tx) * x->oscope_damping) * cos(tpf * f->tx) +
            x->oscope_separation;
      if (fabs(f->ty) <= t) {
        f->p0 += weight * f->tx;
        f->p1 -= weight * f->ty;
      } else {
        f->p0 += weight * f->tx;
        f->p1 += weight * f->ty;
      }
    } break;
    case 70: { /* polar2 1544 */
      double p2v = weight / M_PI;
      f->p0 += p2v * f->precalc_atan;
      f->p1 += p2v / 2.0 * log(f->precalc_sumsq);
    } break;
    case 71: /* popcorn2 1554 */
      f->p0 += weight * (f->tx + x->popcorn2_x * sin(tan(f->ty * x->popcorn2_c)));
      f->p1 += weight * (f->ty + x->popcorn2_y * sin(tan(f->tx * x->popcorn2_c)));
      break;
    case 72: { /* scry 1563 */
      double t = f->precalc_sumsq;
      double r = 1.0 / (f->precalc_sqrt * (t + 1.0 / (weight + F3O_EPS)));
      f->p0 += f->tx * r;
      f->p1 += f->ty * r;
    } break;
    case 73: { /* separation 1584 */
      double sx2 = x->separation_x * x->separation_x, sy2 = x->separation_y * x->separation_y;
      if (f->tx > 0.0) f->p0 += weight * (sqrt(f->tx * f->tx + sx2) - f->tx * x->separation_xinside);
      else f->p0 -= weight * (sqrt(f->tx * f->tx + sx2) + f->tx * x->separation_xinside);
      if (f->ty > 0.0) f->p1 += weight * (sqrt(f->ty * f->ty + sy2) - f->ty * x->separation_yinside);
      else f->p1 -= weight * (sqrt(f->ty * f->ty + sy2) + f->ty * x->separation_yinside);
    } break;
    case 74: /* split 1603 */
      if (cos(f->tx * x->split_xsize * M_PI) >= 0) f->p1 += weight * f->ty;
      else f->p1 -= weight * f->ty;
      if (cos(f->ty * x->split_ysize * M_PI) >= 0) f->p0 += weight * f->tx;
      else f->p0 -= weight * f->tx;
      break;
    case 75: /* splits 1619 */
      if (f->tx >= 0) f->p0 += weight * (f->tx + x->splits_x);
      else f->p0 += weight * (f->tx - x->splits_x);
      if (f->ty >= 0) f->p1 += weight * (f->ty + x->splits_y);
      else f->p1 += weight * (f->ty - x->splits_y);
      break;
    case 76: { /* stripes 1635 */
      double roundx = floor(f->tx + 0.5), offsetx = f->tx - roundx;
      f->p0 += weight * (offsetx * (1.0 - x->stripes_space) + roundx);
      f->p1 += weight * (f->ty + offsetx * offsetx * x->stripes_warp);
    } break;
    case 77: { /* wedge 1649 */
      double r = f->precalc_sqrt;
      double a = f->precalc_atanyx + x->wedge_swirl * r;
      double c = floor((x->wedge_count * a + M_PI) * M_1_PI * 0.5);
      double comp_fac = 1 - x->wedge_angle * x->wedge_count * M_1_PI * 0.5, sa, ca;
      a = a * comp_fac + c * x->wedge_angle;
      sincos(a, &sa, &ca);
      r = weight * (r + x->wedge_hole);
      f->p0 += r * ca;
      f->p1 += r * sa;
    } break;
    case 78: { /* wedge_julia 1671 */
      double r = weight * pow(f->precalc_sumsq, x->wedgeJulia_cn);
      int t_rnd = (int)((x->wedgeJulia_rN) * rng_01(f->rng));
      double a = (f->precalc_atanyx + 2 * M_PI * t_rnd) / x->wedge_julia_power;
      double c = floor((x->wedge_julia_count * a + M_PI) * M_1_PI * 0.5), sa, ca;
      a = a * x->wedgeJulia_cf + c * x->wedge_julia_angle;
      sincos(a, &sa, &ca);
      f->p0 += r * ca;
      f->p1 += r * sa;
    } break;
    case 79: { /* wedge_sph 1689 */
      double r = 1.0 / (f->precalc_sqrt + F3O_EPS);
      double a = f->precalc_atanyx + x->wedge_sph_swirl * r;
      double c = floor((x->wedge_sph_count * a + M_PI) * M_1_PI * 0.5);
      double comp_fac = 1 - x->wedge_sph_angle * x->wedge_sph_count * M_1_PI * 0.5, sa, ca;
      a = a * comp_fac + c * x->wedge_sph_angle;
      sincos(a, &sa, &ca);
      r = weight * (r + x->wedge_sph_hole);
      f->p0 += r * ca;
      f->p1 += r * sa;
    } break;
    case 80: { /* whorl 1710 */
      double r = f->precalc_sqrt, a, sa, ca;
      if (r < weight) a = f->precalc_atanyx + x->whorl_inside / (weight - r);
      else a = f->precalc_atanyx + x->whorl_outside / (weight - r);
      sincos(a, &sa, &ca);
      f->p0 += weight * r * ca;
      f->p1 += weight * r * sa;
    } break;
    case 81: /* waves2 1735 */
      f->p0 += weight * (f->tx + x->waves2_scalex * sin(f->ty * x->waves2_freqx));
      f->p1 += weight * (f->ty + x->waves2_scaley * sin(f->tx * x->waves2_freqy));
      break;
    case 82: { /* exp 1747 */
      double expe = exp(f->tx), expcos, expsin;
      sincos(f->ty, &expsin, &expcos);
      f->p0 += weight * expe * expcos;
      f->p1 += weight * expe * expsin;
    } break;
    case 83: /* log 1756 */
      f->p0 += weight * 0.5 * log(f->precalc_sumsq);
      f->p1 += weight * f->precalc_atanyx;
      break;
    case 84: { /* sin 1763 */
      double s, c, sh, ch;
      sincos(f->tx, &s, &c);
      sh = sinh(f->ty);
      ch = cosh(f->ty);
      f->p0 += weight * s * ch;
      f->p1 += weight * c * sh;
    } break;
    case 85: { /* cos 1773 */
      double s, c, sh, ch;
      sincos(f->tx, &s, &c);
      sh = sinh(f->ty);
      ch = cosh(f->ty);
      f->p0 += weight * c * ch;
      f->p1 -= weight * s * sh;
    } break;
    case 86: { /* tan 1783 */
      double s, c, sh, ch, den;
      sincos(2 * f->tx, &s, &c);
      sh = sinh(2.0 * f->ty);
      ch = cosh(2.0 * f->ty);
      den = 1.0 / (c + ch);
      f->p0 += weight * den * s;
      f->p1 += weight * den * sh;
    } break;
    case 87: { /* sec 1795 */
      double s, c, sh, ch, den;
      sincos(f->tx, &s, &c);
      sh = sinh(f->ty);
      ch = cosh(f->ty);
      den = 2.0 / (cos(2 * f->tx) + cosh(2 * f->ty));
      f->p0 += weight * den * c * ch;
      f->p1 += weight * den * s * sh;
    } break;
    case 88: { /* csc 1807 */
      double s, c, sh, ch, den;
      sincos(f->tx, &s, &c);
      sh = sinh(f->ty);
      ch = cosh(f->ty);
      den = 2.0 / (cosh(2.0 * f->ty) - cos(2.0 * f->tx));
      f->p0 += weight * den * s * ch;
      f->p1 -= weight * den * c * sh;
    } break;
    case 89: { /* cot 1819 */
      double s, c, sh, ch, den;
      sincos(2.0 * f->tx, &s, &c);
      sh = sinh(2.0 * f->ty);
      ch = cosh(2.0 * f->ty);
      den = 1.0 / (ch - c);
      f->p0 += weight * den * s;
      f->p1 += weight * den * -1 * sh;
    } break;
    case 90: { /* sinh 1831 */
      double s, c, sh, ch;
      sincos(f->ty, &s, &c);
      sh = sinh(f->tx);
      ch = cosh(f->tx);
      f->p0 += weight * sh * c;
      f->p1 += weight * ch * s;
    } break;
    case 91: { /* cosh 1841 */
      double s, c, sh, ch;
      sincos(f->ty, &s, &c);
      sh = sinh(f->tx);
      ch = cosh(f->tx);
      f->p0 += weight * ch * c;
      f->p1 += weight * sh * s;
    } break;
    case 92: { /* tanh 1851 */
      double s, c, sh, ch, den;
      sincos(2.0 * f->ty, &s, &c);
      sh = sinh(2.0 * f->tx);
      ch = cosh(2.0 * f->tx);
      den = 1.0 / (c + ch);
      f->p0 += weight * den * sh;
      f->p1 += weight * den * s;
    } break;
    case 93: { /* sech 1863 */
      double s, c, sh, ch, den;
      sincos(f->ty, &s, &c);
      sh = sinh(f->tx);
      ch = cosh(f->tx);
      den = 2.0 / (cos(2.0 * f->ty) + cosh(2.0 * f->tx));
      f->p0 += weight * den * c * ch;
      f->p1 -= weight * den * s * sh;
    } break;
    case 94: { /* csch 1875 */
      double s, c, sh, ch, den;
      sincos(f->ty, &s, &c);
      sh = sinh(f->tx);
      ch = cosh(f->tx);
      den = 2.0 / (cosh(2.0 * f->tx) - cos(2.0 * f->ty));
      f->p0 += weight * den * sh * c;
      f->p1 -= weight * den * ch * s;
    } break;
    case 95: { /* coth 1887 */
      double s, c, sh, ch, den;
      sincos(2.0 * f->ty, &s, &c);
      sh = sinh(2.0 * f->tx);
      ch = cosh(2.0 * f->tx);
      den = 1.0 / (ch - c);
      f->p0 += weight * den * sh;
      f->p1 += weight * den * s;
    } break;
    case 96: { /* auger 1899 */
      double s = sin(x->auger_freq * f->tx), t = sin(x->auger_freq * f->ty);
      double dy = f->ty + x->auger_weight * (x->auger_scale * s / 2.0 + fabs(f->ty) * s);
      double dx = f->tx + x->auger_weight * (x->auger_scale * t / 2.0 + fabs(f->tx) * t);
      f->p0 += weight * (f->tx + x->auger_sym * (dx - f->tx));
      f->p1 += weight * dy;
    } break;
    case 97: { /* flux 1911 */
      double xpw = f->tx + weight, xmw = f->tx - weight;
      double avgr = weight * (2 + x->flux_spread) *
                    sqrt(sqrt(f->ty * f->ty + xpw * xpw) / sqrt(f->ty * f->ty + xmw * xmw));
      double avga = (atan2(f->ty, xmw) - atan2(f->ty, xpw)) * 0.5;
      f->p0 += avgr * cos(avga);
      f->p1 += avgr * sin(avga);
    } break;
    case 98: { /* mobius 1923 */
      double re_u = x->mobius_re_a * f->tx - x->mobius_im_a * f->ty + x->mobius_re_b;
      double im_u = x->mobius_re_a * f->ty + x->mobius_im_a * f->tx + x->mobius_im_b;
      double re_v = x->mobius_re_c * f->tx - x->mobius_im_c * f->ty + x->mobius_re_d;
      double im_v = x->mobius_re_c * f->ty + x->mobius_im_c * f->tx + x->mobius_im_d;
      double rad_v = weight / (re_v * re_v + im_v * im_v);
      f->p0 += rad_v * (re_u * re_v + im_u * im_v);
      f->p1 += rad_v * (im_u * re_v - re_u * im_v);
    } break;
    default:
      break;
  }
  (void)tx;
  (void)ty;
}

/* variations.c:2129-2399 */
static int apply_xform(flam3_genome *cp, int fn, const double *p, double *q, f3o_rng *rng) {
  iter_helper f;
  flam3_xform *x = &cp->xform[fn];
  f.rng = rng;
  double s1 = x->color_speed;
  q[2] = s1 * x->color + (1.0 - s1) * p[2];
  q[3] = x->vis_adjusted;
  f.tx = x->c[0][0] * p[0] + x->c[1][0] * p[1] + x->c[2][0];
  f.ty = x->c[0][1] * p[0] + x->c[1][1] * p[1] + x->c[2][1];
  if (x->has_preblur != 0.0) var_pre_blur(&f, x->has_preblur);
  f.precalc_sumsq = f.tx * f.tx + f.ty * f.ty;
  f.precalc_sqrt = sqrt(f.precalc_sumsq);
  f.precalc_atan = f.precalc_sina = f.precalc_cosa = f.precalc_atanyx = 0.0;
  if (x->precalc_atan_xy_flag > 0) f.precalc_atan = atan2(f.tx, f.ty);
  if (x->precalc_angles_flag > 0) {
    f.precalc_sina = f.tx / f.precalc_sqrt;
    f.precalc_cosa = f.ty / f.precalc_sqrt;
  }
  if (x->precalc_atan_yx_flag > 0) f.precalc_atanyx = atan2(f.ty, f.tx);
  f.p0 = 0.0;
  f.p1 = 0.0;
  f.xf = x;
  for (int vn = 0; vn < x->num_active_vars; vn++)
    apply_variation(&f, x->varFunc[vn], x->active_var_weights[vn]);
  if (x->has_post) {
    q[0] = x->post[0][0] * f.p0 + x->post[1][0] * f.p1 + x->post[2][0];
    q[1] = x->post[0][1] * f.p0 + x->post[1][1] * f.p1 + x->post[2][1];
  } else {
    q[0] = f.p0;
    q[1] = f.p1;
  }
  if (BADVALUE(q[0]) || BADVALUE(q[1])) {
    q[0] = rng_11(rng);
    q[1] = rng_11(rng);
    return 1;
  }
  return 0;
}

int f3o_apply_xform(flam3_genome *cp, int fn, int n, const double *p_in, const uint32_t *words, int wpp,
                    double *q_out, int *bad_out) {
  if (f3o_prepare_precalc_flags(cp)) return 1;
  for (int i = 0; i < cp->num_xforms; i++) f3o_xform_precalc(cp, i);
  for (int k = 0; k < n; k++) {
    f3o_rng r;
    memset(&r, 0, sizeof(r));
    r.kind = 1;
    r.words = words + (size_t)k * wpp;
    r.nwords = wpp;
    int b = apply_xform(cp, fn, p_in + 4 * k, q_out + 4 * k, &r);
    if (bad_out) bad_out[k] = b;
  }
  return 0;
}

/* flam3.c:232-299 */
static int iterate(flam3_genome *cp, int n, int fuse, double *samples, unsigned short *xform_distrib,
                   f3o_rng *rng) {
  double p[4], q[4];
  int consec = 0, badvals = 0, lastxf = 0, fn;
  p[0] = samples[0];
  p[1] = samples[1];
  p[2] = samples[2];
  p[3] = samples[3];
  for (int i = 0; i < cp->num_xforms; i++) f3o_xform_precalc(cp, i);
  for (int i = -4 * fuse; i < 4 * n; i += 4) {
    if (cp->chaos_enable)
      fn = xform_distrib[lastxf * F3O_GRAIN + (rng_word(rng) & F3O_GRAIN_M1)];
    else
      fn = xform_distrib[rng_word(rng) & F3O_GRAIN_M1];
    if (apply_xform(cp, fn, p, q, rng) > 0) {
      consec++;
      badvals++;
      if (consec < 5) {
        p[0] = q[0]; p[1] = q[1]; p[2] = q[2]; p[3] = q[3];
        i -= 4;
        continue;
      } else
        consec = 0;
    } else
      consec = 0;
    lastxf = fn + 1;
    p[0] = q[0]; p[1] = q[1]; p[2] = q[2]; p[3] = q[3];
    if (cp->final_xform_enable == 1) {
      if (cp->xform[cp->final_xform_index].opacity == 1 ||
          rng_01(rng) < cp->xform[cp->final_xform_index].opacity) {
        apply_xform(cp, cp->final_xform_index, p, q, rng);
        q[3] = p[3];
      }
    }
    if (i >= 0) {
      samples[i] = q[0];
      samples[i + 1] = q[1];
      samples[i + 2] = q[2];
      samples[i + 3] = q[3];
    }
  }
  return badvals;
}


#include "flam3_oracle_render.inc"

/* Chains of flam3_iterate (flam3.c:232-299) driven by the CUDA path's
 * Philox stream: chain c draws from key (seed lo, seed hi), counter
 * (c, block, 0, 0xC4A1) -- the same words the GPU's recorded-chain probe
 * consumes -- so both sides pick the same xforms and random parameters. */
int f3o_iterate_chains(flam3_genome *src, int nchains, int n, int fuse, const double *starts, uint64_t seed,
                       double *samples, long *badvals);

int f3o_iterate_chains(flam3_genome *src, int nchains, int n, int fuse, const double *starts, uint64_t seed,
                       double *samples, long *badvals) {
  flam3_genome cp;
  memset(&cp, 0, sizeof(cp));
  genome_copy(&cp, src);
  long bad = 0;
  int rc = 1;
  double *buf = (double *)malloc(sizeof(double) * 4 * (size_t)(n > 0 ? n : 1));
  unsigned short *xd = NULL;
  if (f3o_prepare_precalc_flags(&cp)) goto out;
  xd = f3o_create_xform_distrib(&cp);
  if (!xd) goto out;
  for (int c = 0; c < nchains; c++) {
    f3o_rng r;
    memset(&r, 0, sizeof(r));
    r.kind = 2;
    r.key[0] = (uint32_t)seed;
    r.key[1] = (uint32_t)(seed >> 32);
    r.ctr[0] = (uint32_t)c;
    r.ctr[1] = 0;
    r.ctr[2] = 0;
    r.ctr[3] = 0xC4A1u;
    r.bufpos = 4;
    memcpy(buf, starts + 4 * (size_t)c, 4 * sizeof(double));
    bad += iterate(&cp, n, fuse, buf, xd, &r);
    memcpy(samples + (size_t)c * n * 4, buf, sizeof(double) * 4 * (size_t)n);
  }
  rc = 0;
out:
  if (badvals) *badvals = bad;
  free(buf);
  free(xd);
  genome_free(&cp);
  return rc;
}
