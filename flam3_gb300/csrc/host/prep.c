/*
 * prep.c -- host preparation of a genome for the iterate kernel.
 *
 * Follows the reference's per-temporal-sample setup: flam3_copy
 * (flam3.c:1171-1209), prepare_precalc_flags (variations.c:2016-2126),
 * xform_precalc (variations.c:1942-2014), flam3_create_xform_distrib /
 * flam3_create_chaos_distrib (flam3.c:76-224).  The 16384-entry xform-choice
 * rows are built exactly as the reference builds them and then stored as
 * breakpoints (the row is nondecreasing, so "index = number of breakpoints
 * <= v" reproduces every entry).
 */
#define _GNU_SOURCE
#include <math.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "f3g_host.h"
#include "../f3g_choice.h"

void f3g_genome_free(flam3_genome *g) {
  if (g->xform) {
    int ns = g->num_xforms - (g->final_xform_index >= 0);
    if (g->chaos) {
      for (int i = 0; i < ns; i++) free(g->chaos[i]);
      free(g->chaos);
    }
    free(g->xform);
  }
  g->xform = NULL;
  g->chaos = NULL;
  g->num_xforms = 0;
}

/* flam3_copy: standard xforms first, the final xform (if any) last */
void f3g_genome_copy(flam3_genome *dst, const flam3_genome *src) {
  memcpy(dst, src, sizeof(flam3_genome));
  int ns = src->num_xforms - (src->final_xform_index >= 0);
  dst->xform = (flam3_xform *)calloc((size_t)(src->num_xforms > 0 ? src->num_xforms : 1), sizeof(flam3_xform));
  for (int i = 0; i < ns; i++) {
    dst->xform[i] = src->xform[i];
    dst->xform[i].motion = NULL;
    dst->xform[i].num_motion = 0;
  }
  if (src->final_xform_index >= 0) {
    dst->xform[ns] = src->xform[src->final_xform_index];
    dst->xform[ns].motion = NULL;
    dst->xform[ns].num_motion = 0;
    dst->final_xform_index = ns;
  }
  dst->chaos = (double **)calloc((size_t)(ns > 0 ? ns : 1), sizeof(double *));
  for (int i = 0; i < ns; i++) {
    dst->chaos[i] = (double *)malloc((size_t)(ns > 0 ? ns : 1) * sizeof(double));
    for (int j = 0; j < ns; j++) dst->chaos[i][j] = src->chaos ? src->chaos[i][j] : 1.0;
  }
}

/* interpolation.c:22-29 */
static double adjust_percentage(double in) {
  if (in == 0.0) return 0.0;
  return pow(10.0, -log(1.0 / in) / log(2));
}

static int is_identity(double s[3][2]) {
  return s[0][0] == 1.0 && s[0][1] == 0.0 && s[1][0] == 0.0 && s[1][1] == 1.0 && s[2][0] == 0.0 && s[2][1] == 0.0;
}

/* precalc flag of each variation (variations.c:2050-2115) */
static int var_flag(int j) {
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

int f3g_prepare_precalc_flags(flam3_genome *cp) {
  for (int i = 0; i < cp->num_xforms; i++) {
    flam3_xform *x = &cp->xform[i];
    if (x->density < 0.0) {
      f3g_set_error("xform %d weight must be non-negative, not %g.", i, x->density);
      return 1;
    }
    if (i != cp->final_xform_index && x->density == 0.0) continue;
    int tot = 0;
    x->vis_adjusted = adjust_percentage(x->opacity);
    x->precalc_angles_flag = x->precalc_atan_xy_flag = x->precalc_atan_yx_flag = 0;
    x->has_preblur = 0;
    x->has_post = !is_identity(x->post);
    for (int j = 0; j < flam3_nvariations; j++) {
      if (x->var[j] == 0) continue;
      x->varFunc[tot] = j;
      x->active_var_weights[tot] = x->var[j];
      int fl = var_flag(j);
      if (fl & F3G_F_ATAN_XY) x->precalc_atan_xy_flag = 1;
      if (fl & F3G_F_ANGLES) x->precalc_angles_flag = 1;
      if (fl & F3G_F_ATAN_YX) x->precalc_atan_yx_flag = 1;
      if (j == 67) x->has_preblur = x->var[j];
      tot++;
    }
    x->num_active_vars = tot;
  }
  return 0;
}

void f3g_xform_precalc(flam3_genome *cp, int xi) {
  flam3_xform *xf = &cp->xform[xi];
  double ang = xf->perspective_angle * M_PI / 2.0;
  xf->persp_vsin = sin(ang);
  xf->persp_vfcos = xf->perspective_dist * cos(ang);
  xf->julian_rN = fabs(xf->julian_power);
  xf->julian_cn = xf->julian_dist / (double)xf->julian_power / 2.0;
  xf->juliascope_rN = fabs(xf->juliascope_power);
  xf->juliascope_cn = xf->juliascope_dist / (double)xf->juliascope_power / 2.0;
  xf->radialBlur_spinvar = sin(xf->radial_blur_angle * M_PI / 2.0);
  xf->radialBlur_zoomvar = cos(xf->radial_blur_angle * M_PI / 2.0);
  double dx = xf->c[2][0], dy = xf->c[2][1];
  xf->waves_dx2 = 1.0 / (dx * dx + F3G_EPS);
  xf->waves_dy2 = 1.0 / (dy * dy + F3G_EPS);
  double add = xf->disc2_twist;
  xf->disc2_timespi = xf->disc2_rot * M_PI;
  xf->disc2_sinadd = sin(add);
  xf->disc2_cosadd = cos(add) - 1;
  if (add > 2 * M_PI) {
    double k = (1 + add - 2 * M_PI);
    xf->disc2_cosadd *= k;
    xf->disc2_sinadd *= k;
  }
  if (add < -2 * M_PI) {
    double k = (1 + add + 2 * M_PI);
    xf->disc2_cosadd *= k;
    xf->disc2_sinadd *= k;
  }
  xf->super_shape_pm_4 = xf->super_shape_m / 4.0;
  xf->super_shape_pneg1_n1 = -1.0 / xf->super_shape_n1;
  xf->wedgeJulia_cf = 1.0 - xf->wedge_julia_angle * xf->wedge_julia_count * M_1_PI * 0.5;
  xf->wedgeJulia_rN = fabs(xf->wedge_julia_power);
  xf->wedgeJulia_cn = xf->wedge_julia_dist / xf->wedge_julia_power / 2.0;
}

/* the step of a choice row (flam3.c:165-224): the sum of its weights
 * d[i] (times the row's chaos entries c[i]; c NULL for the raw-weight row)
 * over the standard xforms, divided by F3G_GRAIN */
static int choice_step(const double *d, const double *c, int nstd, double *dr) {
  double sum = 0.0;
  for (int i = 0; i < nstd; i++) {
    const double w = c ? d[i] * c[i] : d[i];
    if (w < 0.0) {
      f3g_set_error("xform weight must be non-negative, not %g.", w);
      return 1;
    }
    sum += w;
  }
  if (sum == 0.0) {
    f3g_set_error("cannot iterate empty flame.");
    return 1;
  }
  *dr = sum / F3G_GRAIN;
  return 0;
}

/* one table row (flam3.c:165-224) over the weights d[0..nx) (a chaos row
 * weights the standard xforms by c and the final xform by 0) */
static int choice_row(const double *d, const double *c, int nstd, int nx, unsigned short *row) {
  double dr;
  if (choice_step(d, c, nstd, &dr)) return 1;
  int j = 0;
  double t = c ? d[0] * c[0] : d[0];
  double r = 0.0;
  for (int i = 0; i < F3G_GRAIN; i++) {
    while (r >= t) {
      j++;
      if (j >= nx) { /* the reference would read past the xform array */
        f3g_set_error("xform distribution overran the xform list");
        return 1;
      }
      t += c ? d[j] * (j < nstd ? c[j] : 0.0) : d[j];
    }
    row[i] = (unsigned short)j;
    r += dr;
  }
  return 0;
}

static int row_to_breakpoints(const unsigned short *row, uint16_t *brk, uint16_t *nbrk) {
  int n = 0, cur = 0;
  for (int v = 0; v < F3G_GRAIN; v++) {
    while (cur < row[v]) {
      if (n >= F3G_MAX_XFORMS) return 1;
      brk[n++] = (uint16_t)v;
      cur++;
    }
  }
  *nbrk = (uint16_t)n;
  return 0;
}

/* row xi of the genome's table (xi < 0: the raw-weight row) as breakpoints */
static int chaos_row(flam3_genome *cp, int xi, unsigned short *row, uint16_t *brk, uint16_t *nbrk) {
  const int nstd = cp->num_xforms - (cp->final_xform_index >= 0);
  double d[F3G_MAX_XFORMS];
  if (cp->num_xforms > F3G_MAX_XFORMS) {
    f3g_set_error("genome has %d xforms; the library handles up to %d", cp->num_xforms, F3G_MAX_XFORMS);
    return 1;
  }
  for (int i = 0; i < cp->num_xforms; i++) d[i] = cp->xform[i].density;
  return choice_row(d, xi >= 0 ? cp->chaos[xi] : NULL, nstd, cp->num_xforms, row) ||
         row_to_breakpoints(row, brk, nbrk);
}

int f3g_choice_breakpoints_host(const double *d, const double *c, int nstd, int nx, int walk, uint16_t *brk,
                                int *nbrk, int *moves) {
  if (nx < 1 || nx > F3G_MAX_XFORMS || nstd < 1 || nstd > nx) {
    f3g_set_error("choice row of %d xforms (%d standard)", nx, nstd);
    return 1;
  }
  if (!walk) {
    unsigned short *row = (unsigned short *)malloc(F3G_GRAIN * sizeof(unsigned short));
    uint16_t n = 0;
    const int rc = !row || choice_row(d, c, nstd, nx, row) || row_to_breakpoints(row, brk, &n);
    free(row);
    *nbrk = n;
    if (moves) *moves = F3G_GRAIN;
    return rc;
  }
  double dr;
  if (choice_step(d, c, nstd, &dr)) return 1;
  if (f3g_choice_breakpoints(dr, d, c, nstd, nx, brk, F3G_MAX_XFORMS, nbrk, moves)) {
    f3g_set_error("xform distribution overran the xform list");
    return 1;
  }
  return 0;
}

int f3g_build_distrib(flam3_genome *cp, F3GPass *pass) {
  unsigned short *row = (unsigned short *)malloc(F3G_GRAIN * sizeof(unsigned short));
  int rc = 0;
  memset(pass->nbrk, 0, sizeof(pass->nbrk));
  if (chaos_row(cp, -1, row, pass->brk[0], &pass->nbrk[0])) {
    rc = 1;
    goto out;
  }
  {
    int num_std = cp->num_xforms - (cp->final_xform_index >= 0);
    int unity = 1;
    for (int i = 0; i < num_std; i++)
      for (int j = 0; j < num_std; j++)
        if (fabs(cp->chaos[i][j] - 1.0) > F3G_EPS) unity = 0;
    cp->chaos_enable = 1 - unity;
    pass->chaos_enable = cp->chaos_enable;
    if (cp->chaos_enable) {
      int dist_row = 0;
      for (int i = 0; i < cp->num_xforms; i++) {
        if (cp->final_xform_index == i) continue;
        dist_row++;
        if (chaos_row(cp, i, row, pass->brk[dist_row], &pass->nbrk[dist_row])) {
          rc = 1;
          goto out;
        }
      }
    }
  }
out:
  free(row);
  return rc;
}

int f3g_pack_genome(flam3_genome *cp, F3GPass *pass) {
  if (cp->num_xforms > F3G_MAX_XFORMS) {
    f3g_set_error("genome has %d xforms; the library handles up to %d", cp->num_xforms, F3G_MAX_XFORMS);
    return 1;
  }
  static const size_t prm_off[PRM_COUNT] = {
#define F3G_X(n) offsetof(flam3_xform, n),
      F3G_PARAM_LIST(F3G_X)
#undef F3G_X
  };
  pass->num_xforms = cp->num_xforms;
  pass->num_std = cp->num_xforms - (cp->final_xform_index >= 0);
  pass->final_index = cp->final_xform_index;
  pass->final_enable = cp->final_xform_enable == 1 && cp->final_xform_index >= 0;
  pass->full_variations = 0;
  int nv = 0;
  for (int i = 0; i < cp->num_xforms; i++) {
    flam3_xform *x = &cp->xform[i];
    F3GXform *d = &pass->xf[i];
    memset(d, 0, sizeof(*d));
    for (int k = 0; k < 3; k++) {
      d->c[2 * k] = x->c[k][0];
      d->c[2 * k + 1] = x->c[k][1];
      d->post[2 * k] = x->post[k][0];
      d->post[2 * k + 1] = x->post[k][1];
    }
    d->color = x->color;
    d->color_speed = x->color_speed;
    d->vis_adjusted = x->vis_adjusted;
    d->opacity = x->opacity;
    d->preblur = x->has_preblur;
    /* xforms skipped by prepare_precalc_flags (zero weight) keep whatever
     * flags they had; they can never be picked */
    int used = (i == cp->final_xform_index) || x->density != 0.0;
    d->flags = 0;
    if (used) {
      if (x->precalc_atan_xy_flag > 0) d->flags |= F3G_F_ATAN_XY;
      if (x->precalc_angles_flag > 0) d->flags |= F3G_F_ANGLES;
      if (x->precalc_atan_yx_flag > 0) d->flags |= F3G_F_ATAN_YX;
      if (x->has_post) d->flags |= F3G_F_POST;
      if (x->has_preblur != 0.0) d->flags |= F3G_F_PREBLUR;
    }
    d->var_off = nv;
    d->nvars = used ? x->num_active_vars : 0;
    if (nv + d->nvars > F3G_MAX_VARLIST) {
      f3g_set_error("genome has more than %d active variations in total", F3G_MAX_VARLIST);
      return 1;
    }
    for (int k = 0; k < d->nvars; k++) {
      int v = x->varFunc[k];
      if (v < 0 || v >= F3G_NVARS) {
        f3g_set_error("xform %d has an unknown variation %d", i, v);
        return 1;
      }
      pass->var_id[nv + k] = (uint8_t)v;
      pass->var_w[nv + k] = x->active_var_weights[k];
      if (v >= 20) pass->full_variations = 1;
    }
    if (d->flags & F3G_F_PREBLUR) pass->full_variations = 1;
    nv += d->nvars;
    const char *base = (const char *)x;
    for (int k = 0; k < PRM_COUNT; k++) d->prm[k] = *(const double *)(base + prm_off[k]);
  }
  return 0;
}

/* Genome at `time` (flam3.c:717-802).  One genome: a copy.  Several genomes:
 * see interp.c. */
int f3g_interpolate_n(flam3_genome *cps, int ncps, double time, flam3_genome *result);

int f3g_interpolate(flam3_genome *cps, int ncps, double time, flam3_genome *result) {
  f3g_genome_free(result);
  if (ncps == 1) {
    f3g_genome_copy(result, &cps[0]);
    return 0;
  }
  return f3g_interpolate_n(cps, ncps, time, result);
}
