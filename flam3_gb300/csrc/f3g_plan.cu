/*
 * f3g_plan.cu -- the temporal samples of an animation frame planned on the
 * device: one block per sample blends the genome at the sample's time from
 * the aligned key genomes (flam3_interpolate, flam3.c:717-802, with the
 * blend of interpolation.c:373-709), prepares it (prepare_precalc_flags and
 * xform_precalc, variations.c:1942-2126), builds its xform-choice rows
 * (flam3.c:76-224, stored as breakpoints) and writes the pass the iterate
 * kernel reads: colour map, xforms with their parameters, active-variation
 * lists.  FP64 throughout, the same operations in the same order as the host
 * path (host/interp.c, host/prep.c); CUDA's libm may round the last bit of
 * atan2/exp/log/sin/cos/pow differently from the host's.
 *
 * The host plans only what it needs before the launch (the key segment and
 * weights of each sample, the genome scalars, the chaos rows and the camera)
 * and uploads each pass's header; this kernel fills in the rest.
 *
 * Work per sample: 256 palette entries (two HSV conversions per key), about
 * 230 blended doubles and two matrices per xform, up to 33 choice rows --
 * spread over the block's threads.  A choice row's 16384 dependent FP64 adds
 * are replaced by the exact binade walk of f3g_choice.h.
 */
#include <cuda_runtime.h>
#include <math.h>
#include <stddef.h>
#include <stdint.h>

#include "flam3_gpu.h"
#include "f3g_common.h"
#include "f3g_launch.h"
#include "f3g_choice.h"

#define PL_THREADS 256
#define PL_VBLK 99 /* variation weights per xform */

namespace f3g {

__constant__ size_t c_prm_off[PRM_COUNT] = {
#define F3G_X(n) offsetof(flam3_xform, n),
    F3G_PARAM_LIST(F3G_X)
#undef F3G_X
};

__device__ __forceinline__ double xfield(const flam3_xform *x, size_t off) {
  return *(const double *)((const char *)x + off);
}

__device__ __forceinline__ double clamp01d(double v) { return v < 0 ? 0 : (v > 1 ? 1 : v); }

/* acc + a*b with the product and the sum each rounded, as the host computes
 * them (no fused multiply-add), so the blend repeats the host's sums exactly */
__device__ __forceinline__ double mac(double acc, double a, double b) { return __dadd_rn(acc, __dmul_rn(a, b)); }

/* palettes.c:199-272 (the host's rgb2hsv / hsv2rgb of interp.c) */
__device__ void d_rgb2hsv(const double *rgb, double *hsv) {
  const double r = rgb[0], g = rgb[1], b = rgb[2];
  const double hi = r >= g ? (r >= b ? r : b) : (g >= b ? g : b);
  const double lo = r <= g ? (r <= b ? r : b) : (g <= b ? g : b);
  const double span = hi - lo;
  double h = 0.0;
  const double s = hi != 0.0 ? span / hi : 0.0;
  if (s != 0.0) {
    const double dr = (hi - r) / span, dg = (hi - g) / span, db = (hi - b) / span;
    if (r == hi)
      h = db - dg;
    else if (g == hi)
      h = 2 + dr - db;
    else if (b == hi)
      h = 4 + dg - dr;
    if (h < 0) h += 6;
  }
  hsv[0] = h;
  hsv[1] = s;
  hsv[2] = hi;
}

__device__ void d_hsv2rgb(const double *hsv, double *rgb) {
  double h = hsv[0];
  const double s = hsv[1], v = hsv[2];
  while (h >= 6.0) h -= 6.0;
  while (h < 0.0) h += 6.0;
  const int sector = (int)floor(h);
  const double f = h - sector;
  const double p = v * (1 - s), q = v * __dsub_rn(1, __dmul_rn(s, f)), t = v * __dsub_rn(1, __dmul_rn(s, 1 - f));
  const double val[4] = {v, p, q, t};
  const unsigned char pick[6][3] = {{0, 3, 1}, {2, 0, 1}, {1, 0, 3}, {1, 2, 0}, {3, 1, 0}, {0, 1, 2}};
  const unsigned char *sel = pick[(sector >= 0 && sector < 6) ? sector : 0];
  for (int c = 0; c < 3; c++) rgb[c] = val[sel[c]];
}

__device__ __forceinline__ bool identity6(const double m[3][2]) {
  return m[0][0] == 1.0 && m[0][1] == 0.0 && m[1][0] == 0.0 && m[1][1] == 1.0 && m[2][0] == 0.0 && m[2][1] == 0.0;
}

/* precalc flag of each variation (variations.c:2050-2115) */
__device__ __forceinline__ int d_var_flag(int j) {
  switch (j) {
    case 5: case 6: case 7: case 8: case 12: case 13: case 22: case 25: case 49: case 70:
      return F3G_F_ATAN_XY;
    case 9: case 10: case 11: case 19: case 21: case 26:
      return F3G_F_ANGLES;
    case 23:
      return F3G_F_ATAN_XY | F3G_F_ANGLES;
    case 32: case 33: case 36: case 38: case 50: case 51: case 52: case 59: case 63: case 77: case 78: case 79:
    case 80: case 83:
      return F3G_F_ATAN_YX;
    default:
      return 0;
  }
}

/* one matrix (c when which = 0, post when 1) of xform xf blended over the
 * keys: per column in log-polar form (angle, magnitude, translation) when
 * the keys interpolate log-polar, else entry by entry (interpolation.c:173-323) */
__device__ void blend_matrix(const flam3_xform *X, int nk, int nx, int xf, int which, int log_polar,
                             const double *w, double out[6]) {
  bool posts_identity = true;
  for (int k = 0; k < nk; k++) posts_identity &= identity6(X[k * nx + xf].post);
  if (!log_polar) {
    for (int r = 0; r < 3; r++)
      for (int c = 0; c < 2; c++) {
        double a = 0.0;
        for (int k = 0; k < nk; k++) {
          const flam3_xform *x = &X[k * nx + xf];
          a = mac(a, w[k], which ? x->post[r][c] : x->c[r][c]);
        }
        out[2 * r + c] = a;
      }
    if (which && posts_identity) {
      out[0] = 1.0; out[1] = 0.0; out[2] = 0.0; out[3] = 1.0; out[4] = 0.0; out[5] = 0.0;
    }
    return;
  }
  if (which && posts_identity) {
    out[0] = 1.0; out[1] = 0.0; out[2] = 0.0; out[3] = 1.0; out[4] = 0.0; out[5] = 0.0;
    return;
  }
  double ang[4][2], mag[4][2], trn[4][2];
  for (int k = 0; k < nk; k++) {
    const flam3_xform *x = &X[k * nx + xf];
    const double(*m)[2] = which ? x->post : x->c;
    bool zero[2];
    for (int col = 0; col < 2; col++) {
      const double u = m[col][0], v = m[col][1];
      ang[k][col] = atan2(v, u);
      mag[k][col] = sqrt(__dadd_rn(__dmul_rn(u, u), __dmul_rn(v, v)));
      trn[k][col] = m[2][col];
      zero[col] = mag[k][col] == 0.0;
    }
    if (zero[0] && !zero[1]) ang[k][0] = ang[k][1];
    if (zero[1] && !zero[0]) ang[k][1] = ang[k][0];
  }
  const double turn = 2 * M_PI, eps = 1e-10;
  for (int col = 0; col < 2; col++)
    for (int k = 1; k < nk; k++) {
      const double wind = X[k * nx + xf].wind[col];
      double *a0 = &ang[k - 1][col], *a1 = &ang[k][col];
      if (wind > 0 && which == 0) {
        const double lo = wind - turn;
        while (*a0 < lo) *a0 += turn;
        while (*a0 > lo + turn) *a0 -= turn;
        while (*a1 < lo) *a1 += turn;
        while (*a1 > lo + turn) *a1 -= turn;
      } else {
        const double d = *a1 - *a0;
        if (d > M_PI + eps)
          *a1 -= turn;
        else if (d < -(M_PI - eps))
          *a1 += turn;
      }
    }
  for (int col = 0; col < 2; col++) {
    bool linear_mag = false;
    for (int k = 0; k < nk; k++)
      if (log(mag[k][col]) < -10) linear_mag = true;
    double a = 0.0, mg = 0.0, t = 0.0;
    for (int k = 0; k < nk; k++) {
      a = mac(a, w[k], ang[k][col]);
      mg = mac(mg, w[k], linear_mag ? mag[k][col] : log(mag[k][col]));
      t = mac(t, w[k], trn[k][col]);
    }
    const double r = linear_mag ? mg : exp(mg);
    out[2 * col + 0] = r * cos(a);
    out[2 * col + 1] = r * sin(a);
    out[4 + col] = t;
  }
}

__global__ void __launch_bounds__(PL_THREADS) k_plan(const unsigned char *__restrict__ keys,
                                                     const F3GPlanSample *__restrict__ samples, F3GPass *passes,
                                                     int *err) {
  extern __shared__ double pl_smem[];
  const F3GPlanSample S = samples[blockIdx.x];
  const unsigned char *base = keys + S.keyset;
  const F3GKeySet *ks = (const F3GKeySet *)base;
  const int nk = ks->nk, nx = ks->nx, nstd = ks->nstd, fin = ks->final_index;
  const flam3_genome *G = (const flam3_genome *)(base + ks->off_genome);
  const flam3_xform *X = (const flam3_xform *)(base + ks->off_xform);
  const double *CH = (const double *)(base + ks->off_chaos);
  F3GPass *p = passes + blockIdx.x;
  double *svar = pl_smem;                 /* nx x 99 blended variation weights */
  double *sdens = svar + nx * PL_VBLK;    /* nx densities */
  double *sch = sdens + nx;               /* nstd x nstd chaos */
  int *snv = (int *)(sch + nstd * nstd);  /* nx active-variation counts */
  int *soff = snv + nx;                   /* nx list offsets */
  const int t = threadIdx.x;
  const double *w = S.w;

  /* 1. colour map (interp.c blend_palette, rect.c:778-782) */
  for (int i = t; i < 256; i += PL_THREADS) {
    double col[4];
    const int mode = G[0].palette_interpolation;
    if (mode == 1) {
      const flam3_palette_entry *e = &G[(i < (256 * w[0])) ? 0 : 1].palette[i];
      for (int c = 0; c < 4; c++) col[c] = e->color[c];
    } else {
      const double rgb_part = mode == 2 ? 1.0 : (mode == 3 ? G[0].hsv_rgb_palette_blend : 0.0);
      double hsv[4][3];
      for (int k = 0; k < nk; k++) d_rgb2hsv(G[k].palette[i].color, hsv[k]);
      if (nk == 2 && mode == 3) {
        const double dh = hsv[1][0] - hsv[0][0];
        if (dh > 3.0)
          hsv[0][0] += 6.0;
        else if (dh < -3.0)
          hsv[0][0] -= 6.0;
      }
      double rgb[3] = {0, 0, 0}, h[3] = {0, 0, 0}, alpha = 0, back[3];
      bool opaque = true;
      for (int k = 0; k < nk; k++) {
        const flam3_palette_entry *e = &G[k].palette[i];
        for (int c = 0; c < 3; c++) {
          rgb[c] = mac(rgb[c], w[k], e->color[c]);
          h[c] = mac(h[c], w[k], hsv[k][c]);
        }
        alpha = mac(alpha, w[k], e->color[3]);
        opaque &= e->color[3] == 1.0;
      }
      d_hsv2rgb(h, back);
      for (int c = 0; c < 3; c++) col[c] = clamp01d(__dadd_rn(__dmul_rn(rgb_part, rgb[c]), __dmul_rn(1.0 - rgb_part, back[c])));
      col[3] = clamp01d(opaque ? 1.0 : alpha);
    }
    for (int c = 0; c < 4; c++) p->dmap[i][c] = (float)((col[c] * 255.0) * S.color_scalar);
  }

  /* 2. xform scalars, user parameters and variation weights: per item a
   *    weighted sum over the keys in key order (interp.c x_block) */
  const int per = 5 + PRM_persp_vsin + PL_VBLK;
  for (int it = t; it < nx * per; it += PL_THREADS) {
    const int xf = it / per, f = it % per;
    size_t off;
    if (f < 5)
      off = offsetof(flam3_xform, density) + (size_t)f * sizeof(double);
    else if (f < 5 + PRM_persp_vsin)
      off = c_prm_off[f - 5];
    else
      off = offsetof(flam3_xform, var) + (size_t)(f - 5 - PRM_persp_vsin) * sizeof(double);
    double v = 0.0;
    for (int k = 0; k < nk; k++) v = mac(v, w[k], xfield(&X[k * nx + xf], off));
    F3GXform *d = &p->xf[xf];
    if (f == 0)
      sdens[xf] = v < 0.0 ? 0.0 : v;
    else if (f == 1)
      d->color = clamp01d(v);
    else if (f == 2)
      d->color_speed = clamp01d(v);
    else if (f == 4)
      d->opacity = v;
    else if (f >= 5 && f < 5 + PRM_persp_vsin)
      d->prm[f - 5] = v;
    else if (f >= 5 + PRM_persp_vsin)
      svar[xf * PL_VBLK + (f - 5 - PRM_persp_vsin)] = v;
  }
  /* 3. matrices, one per thread */
  const int log_polar = G[0].interpolation_type == 1;
  for (int it = t; it < 2 * nx; it += PL_THREADS) {
    const int xf = it >> 1, which = it & 1;
    blend_matrix(X, nk, nx, xf, which, log_polar, w, which ? p->xf[xf].post : p->xf[xf].c);
  }
  /* 4. chaos rows */
  for (int it = t; it < nstd * nstd; it += PL_THREADS) {
    double v = 0.0;
    for (int k = 0; k < nk; k++) v = mac(v, w[k], CH[(size_t)k * nstd * nstd + it]);
    sch[it] = v < 0 ? 0 : v;
  }
  __syncthreads();

  /* 5. per xform: prepare_precalc_flags (variations.c:2016-2126) and
   *    xform_precalc (variations.c:1942-2014); xforms of zero weight other
   *    than the final one keep no list, flags or visibility */
  for (int xf = t; xf < nx; xf += PL_THREADS) {
    F3GXform *d = &p->xf[xf];
    const double *var = svar + xf * PL_VBLK;
    const bool used = xf == fin || sdens[xf] != 0.0;
    int flags = 0, nv = 0;
    double preblur = 0.0, vis = 0.0;
    if (used) {
      const double op = d->opacity;
      vis = op == 0.0 ? 0.0 : pow(10.0, -log(1.0 / op) / log(2.0));
      for (int j = 0; j < PL_VBLK; j++) {
        if (var[j] == 0) continue;
        flags |= d_var_flag(j);
        if (j == 67) preblur = var[j];
        nv++;
      }
      double pm[3][2] = {{d->post[0], d->post[1]}, {d->post[2], d->post[3]}, {d->post[4], d->post[5]}};
      if (!identity6(pm)) flags |= F3G_F_POST;
      if (preblur != 0.0) flags |= F3G_F_PREBLUR;
    }
    d->vis_adjusted = vis;
    d->preblur = preblur;
    d->flags = flags;
    d->nvars = nv;
    snv[xf] = nv;
    double *prm = d->prm;
    const double ang = prm[PRM_perspective_angle] * M_PI / 2.0;
    prm[PRM_persp_vsin] = sin(ang);
    prm[PRM_persp_vfcos] = prm[PRM_perspective_dist] * cos(ang);
    prm[PRM_julian_rN] = fabs(prm[PRM_julian_power]);
    prm[PRM_julian_cn] = prm[PRM_julian_dist] / (double)prm[PRM_julian_power] / 2.0;
    prm[PRM_juliascope_rN] = fabs(prm[PRM_juliascope_power]);
    prm[PRM_juliascope_cn] = prm[PRM_juliascope_dist] / (double)prm[PRM_juliascope_power] / 2.0;
    prm[PRM_radialBlur_spinvar] = sin(prm[PRM_radial_blur_angle] * M_PI / 2.0);
    prm[PRM_radialBlur_zoomvar] = cos(prm[PRM_radial_blur_angle] * M_PI / 2.0);
    const double dx = d->c[4], dy = d->c[5];
    prm[PRM_waves_dx2] = 1.0 / __dadd_rn(__dmul_rn(dx, dx), F3G_EPS);
    prm[PRM_waves_dy2] = 1.0 / __dadd_rn(__dmul_rn(dy, dy), F3G_EPS);
    const double add = prm[PRM_disc2_twist];
    prm[PRM_disc2_timespi] = prm[PRM_disc2_rot] * M_PI;
    prm[PRM_disc2_sinadd] = sin(add);
    prm[PRM_disc2_cosadd] = cos(add) - 1;
    if (add > 2 * M_PI) {
      const double kk = (1 + add - 2 * M_PI);
      prm[PRM_disc2_cosadd] *= kk;
      prm[PRM_disc2_sinadd] *= kk;
    }
    if (add < -2 * M_PI) {
      const double kk = (1 + add + 2 * M_PI);
      prm[PRM_disc2_cosadd] *= kk;
      prm[PRM_disc2_sinadd] *= kk;
    }
    prm[PRM_super_shape_pm_4] = prm[PRM_super_shape_m] / 4.0;
    prm[PRM_super_shape_pneg1_n1] = -1.0 / prm[PRM_super_shape_n1];
    prm[PRM_wedgeJulia_cf] =
        __dsub_rn(1.0, __dmul_rn(__dmul_rn(__dmul_rn(prm[PRM_wedge_julia_angle], prm[PRM_wedge_julia_count]), M_1_PI), 0.5));
    prm[PRM_wedgeJulia_rN] = fabs(prm[PRM_wedge_julia_power]);
    prm[PRM_wedgeJulia_cn] = prm[PRM_wedge_julia_dist] / prm[PRM_wedge_julia_power] / 2.0;
  }
  __syncthreads();
  if (t == 0) {
    int off = 0, full = 0;
    for (int xf = 0; xf < nx; xf++) {
      soff[xf] = off;
      off += snv[xf];
      if (p->xf[xf].flags & F3G_F_PREBLUR) full = 1;
    }
    if (off > F3G_MAX_VARLIST) {
      err[blockIdx.x] = 1;
      for (int xf = 0; xf < nx; xf++) snv[xf] = 0;
    }
    p->full_variations = full;
  }
  __syncthreads();
  /* 6. active-variation lists (the pack of host/prep.c) */
  for (int xf = t; xf < nx; xf += PL_THREADS) {
    const double *var = svar + xf * PL_VBLK;
    F3GXform *d = &p->xf[xf];
    d->var_off = soff[xf];
    d->nvars = snv[xf];
    int n = soff[xf], full = 0;
    if (snv[xf])
      for (int j = 0; j < PL_VBLK; j++) {
        if (var[j] == 0) continue;
        p->var_id[n] = (uint8_t)j;
        p->var_w[n] = var[j];
        if (j >= 20) full = 1;
        n++;
      }
    if (full) p->full_variations = 1;
  }
  /* 7. xform-choice rows (flam3.c:165-224) as breakpoints: row 0 from the
   *    weights, row 1+i after xform i when xaos is on */
  const int rows = 1 + (p->chaos_enable ? nstd : 0);
  for (int r = t; r < rows; r += PL_THREADS) {
    const int xi = r - 1;
    double dr = 0.0;
    for (int i = 0; i < nstd; i++) dr = xi >= 0 ? mac(dr, sdens[i], sch[xi * nstd + i]) : __dadd_rn(dr, sdens[i]);
    int nb = 0;
    if (dr > 0.0 &&
        f3g_choice_breakpoints(dr / F3G_GRAIN, sdens, xi >= 0 ? sch + xi * nstd : nullptr, nstd, nx, p->brk[r],
                               F3G_MAX_XFORMS, &nb, nullptr))
      err[blockIdx.x] = 2;
    p->nbrk[r] = (uint16_t)nb;
  }
}

}  // namespace f3g

using namespace f3g;

extern "C" size_t f3g_plan_smem(int nx, int nstd) {
  return (size_t)nx * PL_VBLK * 8 + (size_t)nx * 8 + (size_t)nstd * nstd * 8 + (size_t)nx * 8;
}

extern "C" int f3g_launch_plan(const unsigned char *d_keys, const F3GPlanSample *d_samples, int n, int nx_max,
                               int nstd_max, F3GPass *d_passes, int *d_err, cudaStream_t st) {
  if (n < 1) return 0;
  const size_t smem = f3g_plan_smem(nx_max, nstd_max);
  static volatile int attr_done = 0;
  if (!attr_done) {
    cudaError_t e = cudaFuncSetAttribute(k_plan, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)f3g_plan_smem(F3G_MAX_XFORMS, F3G_MAX_XFORMS));
    if (e != cudaSuccess) return (int)e;
    attr_done = 1;
  }
  k_plan<<<n, PL_THREADS, smem, st>>>(d_keys, d_samples, d_passes, d_err);
  return (int)cudaGetLastError();
}
