/*
 * interp.c -- genome interpolation for frames with several control points
 * (animation keys, motion-blur temporal samples), host FP64.
 *
 * Semantics: flam3_interpolate (flam3.c:717-802) -- pick the two (or, for
 * smooth interpolation, four) keys around the time, align them
 * (flam3_align, interpolation.c:768-1033), blend them with linear or
 * Catmull-Rom weights (interpolation.c:326-337, 373-709).
 *
 * Design.  A blend is a weighted sum over the aligned keys, done per data
 * block rather than per named field:
 *   - an xform is three contiguous double vectors in flam3_xform: the
 *     variation weights var[], the scalars density..opacity, and the user
 *     parameter block blob_low..mobius_im_d (the values after it are
 *     xform_precalc's and are recomputed, not blended);
 *   - the genome scalars are one offset table (doubles, and integers that
 *     are rounded after blending);
 *   - affine matrices blend per column in log-polar form (angle, log
 *     magnitude, translation) or linearly;
 *   - palettes blend in RGB and in HSV and are mixed by the genome's RGB
 *     fraction.
 * Every weighted sum starts at 0.0 and adds w[k]*v[k] in key order, which is
 * the reference's order of operations, so with FP contraction off the result
 * is bit-identical to the reference's (tests/test_interp_pin.py).
 *
 * Alignment pads the keys to a common xform count; a padding xform takes
 * parameters from its neighbours and an identity-like variation chosen by a
 * rule table.
 *
 * Exported as flam3gpu_interpolate for standalone callers; a caller that
 * links the reference library can route the render through the reference's
 * own flam3_interpolate with flam3gpu_set_interpolator.
 */
#define _GNU_SOURCE
#include <math.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "f3g_host.h"

#define XO(f) offsetof(flam3_xform, f)
#define GO(f) offsetof(flam3_genome, f)
#define XD(x, off) (*(double *)((char *)(x) + (off)))
#define XDC(x, off) (*(const double *)((const char *)(x) + (off)))

/* the three blended blocks of an xform */
#define VAR_BLOCK_OFF XO(var)
#define VAR_BLOCK_N flam3_nvariations
#define SCALAR_BLOCK_OFF XO(density)
#define SCALAR_BLOCK_N ((XO(vis_adjusted) - XO(density)) / sizeof(double))
#define PARAM_BLOCK_OFF XO(blob_low)
#define PARAM_BLOCK_N ((XO(persp_vsin) - XO(blob_low)) / sizeof(double))

_Static_assert(XO(opacity) - XO(density) == 4 * sizeof(double), "density..opacity must be contiguous doubles");
_Static_assert((XO(persp_vsin) - XO(blob_low)) % sizeof(double) == 0, "parameter block must be doubles");
_Static_assert((XO(persp_vsin) - XO(blob_low)) / sizeof(double) == PRM_persp_vsin,
               "the parameter block must hold exactly the user parameters of F3G_PARAM_LIST");

/* ---- defaults ---------------------------------------------------------- */

/* initialize_xforms (variations.c:2401-2563): the non-zero defaults of a new
 * xform; everything else is zero */
static const struct {
  size_t off;
  double v;
} kXformDefaults[] = {
    {XO(color_speed), 0.5}, {XO(animate), 1.0}, {XO(opacity), 1.0}, {XO(var[0]), 1.0},
    {XO(c[0][0]), 1.0}, {XO(c[1][1]), 1.0}, {XO(post[0][0]), 1.0}, {XO(post[1][1]), 1.0},
    {XO(blob_high), 1.0}, {XO(blob_waves), 1.0}, {XO(bent2_x), 1.0}, {XO(bent2_y), 1.0},
    {XO(cell_size), 1.0}, {XO(cpow_r), 1.0}, {XO(cpow_power), 1.0}, {XO(curve_xlength), 1.0},
    {XO(curve_ylength), 1.0}, {XO(oscope_separation), 1.0}, {XO(oscope_frequency), M_PI},
    {XO(oscope_amplitude), 1.0}, {XO(wedge_count), 1.0}, {XO(wedge_sph_count), 1.0},
    {XO(wedge_julia_power), 1.0}, {XO(wedge_julia_count), 1.0}, {XO(wedgeJulia_cn), 0.5},
    {XO(wedgeJulia_rN), 1.0}, {XO(auger_freq), 1.0}, {XO(auger_weight), 0.5}, {XO(auger_scale), 1.0},
    {XO(julian_power), 1.0}, {XO(julian_dist), 1.0}, {XO(julian_rN), 1.0}, {XO(julian_cn), 0.5},
    {XO(juliascope_power), 1.0}, {XO(juliascope_dist), 1.0}, {XO(juliascope_rN), 1.0},
    {XO(juliascope_cn), 0.5}, {XO(radialBlur_zoomvar), 1.0}, {XO(pie_slices), 6.0},
    {XO(pie_thickness), 0.5}, {XO(ngon_sides), 5.0}, {XO(ngon_power), 3.0}, {XO(ngon_circle), 1.0},
    {XO(ngon_corners), 2.0}, {XO(curl_c1), 1.0}, {XO(rectangles_x), 1.0}, {XO(rectangles_y), 1.0},
    {XO(amw_amp), 1.0}, {XO(super_shape_n1), 1.0}, {XO(super_shape_n2), 1.0}, {XO(super_shape_n3), 1.0},
    {XO(conic_eccentricity), 1.0},
};

static void new_xform(flam3_xform *x, int index, int padding) {
  memset(x, 0, sizeof(*x));
  for (size_t k = 0; k < sizeof(kXformDefaults) / sizeof(kXformDefaults[0]); k++)
    XD(x, kXformDefaults[k].off) = kXformDefaults[k].v;
  x->color = index & 1;
  x->padding = padding;
}

/* clear_cp(cp, flam3_defaults_on) (flam3.c:1270-1337): the fields it sets */
static void genome_defaults(flam3_genome *cp) {
  static const struct {
    size_t off;
    double v;
  } dbl[] = {
      {GO(center[0]), 0.0}, {GO(center[1]), 0.0}, {GO(rot_center[0]), 0.0}, {GO(rot_center[1]), 0.0},
      {GO(gamma), 4.0}, {GO(vibrancy), 1.0}, {GO(contrast), 1.0}, {GO(brightness), 4.0},
      {GO(hue_rotation), 0.0}, {GO(rotate), 0.0}, {GO(pixels_per_unit), 50.0},
      {GO(hsv_rgb_palette_blend), 0.0}, {GO(highlight_power), -1.0}, {GO(background[0]), 0.0},
      {GO(background[1]), 0.0}, {GO(background[2]), 0.0}, {GO(spatial_filter_radius), 0.5},
      {GO(zoom), 0.0}, {GO(sample_density), 1.0}, {GO(estimator), 9.0}, {GO(estimator_minimum), 0.0},
      {GO(estimator_curve), 0.4}, {GO(gam_lin_thresh), 0.01}, {GO(temporal_filter_width), 1.0},
      {GO(temporal_filter_exp), 0.0},
  };
  for (size_t k = 0; k < sizeof(dbl) / sizeof(dbl[0]); k++) *(double *)((char *)cp + dbl[k].off) = dbl[k].v;
  cp->palette_index = -1;
  cp->symmetry = 0;
  cp->interpolation = 0;
  cp->palette_interpolation = 3;
  cp->genome_index = 0;
  memset(cp->parent_fname, 0, sizeof(cp->parent_fname));
  cp->width = cp->height = 100;
  cp->spatial_oversample = 1;
  cp->nbatches = 1;
  cp->ntemporal_samples = 1000;
  cp->spatial_filter_select = 0;
  cp->interpolation_type = 1;
  cp->temporal_filter_type = 0;
  cp->palette_mode = 0;
  cp->final_xform_enable = 0;
  cp->final_xform_index = -1;
}

/* ---- xform storage ------------------------------------------------------ */

static int n_std(const flam3_genome *g) { return g->num_xforms - (g->final_xform_index >= 0); }

static void release(flam3_genome *g) {
  if (g->xform) {
    if (g->chaos) {
      for (int i = 0; i < n_std(g); i++) free(g->chaos[i]);
      free(g->chaos);
    }
    for (int i = 0; i < g->num_xforms; i++)
      if (g->xform[i].num_motion > 0) free(g->xform[i].motion);
    free(g->xform);
  }
  g->xform = NULL;
  g->chaos = NULL;
  g->num_xforms = 0;
  g->final_xform_index = -1;
}

/* Grow a genome by `count` new xforms (flam3_add_xforms, flam3.c:1033-1093):
 * the xform array is rebuilt as [standard xforms, new xforms, final xform],
 * then either the last one becomes the final xform (final_flag) or the chaos
 * matrix grows to the new standard count with unit entries. */
static void grow_xforms(flam3_genome *cp, int count, int padding, int final_flag) {
  const int old_n = cp->num_xforms, old_std = n_std(cp), has_final = cp->final_xform_index >= 0;
  const int n = old_n + count;
  flam3_xform *xs = (flam3_xform *)malloc((size_t)n * sizeof(flam3_xform));
  int w = 0;
  for (int i = 0; i < old_n; i++)
    if (i != cp->final_xform_index) xs[w++] = cp->xform[i];
  for (int i = old_n; i < n; i++) new_xform(&xs[w++], i, padding);
  if (has_final) xs[w++] = cp->xform[cp->final_xform_index];
  free(cp->xform);
  cp->xform = xs;
  cp->num_xforms = n;
  if (has_final) cp->final_xform_index = n - 1;
  if (final_flag) {
    cp->final_xform_enable = 1;
    cp->final_xform_index = n - 1;
    return;
  }
  const int nstd = n_std(cp);
  double **rows = (double **)malloc((size_t)(nstd > 0 ? nstd : 1) * sizeof(double *));
  for (int i = 0; i < nstd; i++) {
    rows[i] = (double *)malloc((size_t)nstd * sizeof(double));
    for (int j = 0; j < nstd; j++) rows[i][j] = (i < old_std && j < old_std && cp->chaos) ? cp->chaos[i][j] : 1.0;
  }
  if (cp->chaos)
    for (int i = 0; i < old_std; i++) free(cp->chaos[i]);
  free(cp->chaos);
  cp->chaos = rows;
}

/* An xform of a key without its motion elements */
static flam3_xform bare(const flam3_xform *s) {
  flam3_xform x = *s;
  x.num_motion = 0;
  x.motion = NULL;
  return x;
}

/* A key padded to nstd standard xforms and, if want_final, a final xform
 * (flam3_copyx, flam3.c:1211-1268); padding xforms carry padding = 1. */
static void padded_copy(flam3_genome *dst, const flam3_genome *src, int nstd, int want_final) {
  memcpy(dst, src, sizeof(flam3_genome));
  dst->num_xforms = 0;
  dst->xform = NULL;
  dst->chaos = NULL;
  dst->final_xform_index = -1;
  grow_xforms(dst, nstd, 1, 0);
  const int sstd = n_std(src);
  for (int i = 0; i < sstd; i++) {
    dst->xform[i] = bare(&src->xform[i]);
    memcpy(dst->chaos[i], src->chaos[i], (size_t)sstd * sizeof(double));
  }
  if (want_final > 0) {
    grow_xforms(dst, want_final, 1, 1);
    flam3_xform *f = &dst->xform[dst->num_xforms - 1];
    if (src->final_xform_enable > 0) {
      *f = bare(&src->xform[src->final_xform_index]);
    } else {
      f->animate = 0.0;
      f->color_speed = 0.0;
    }
  } else {
    dst->final_xform_index = -1;
    dst->final_xform_enable = 0;
  }
}

/* ---- alignment (flam3_align, interpolation.c:768-1033) ------------------- */

/* Parameters that travel with each parametric variation: a key that lacks
 * the variation takes them from a neighbour that has it, so the blend does
 * not pass through the defaults (flam3_copy_params, flam3.c:804-1005; the
 * reference copies flower's petals and never its holes). */
static const struct {
  int var;
  size_t off[8];
} kVariationParams[] = {
    {23, {XO(blob_low), XO(blob_high), XO(blob_waves)}},
    {24, {XO(pdj_a), XO(pdj_b), XO(pdj_c), XO(pdj_d)}},
    {25, {XO(fan2_x), XO(fan2_y)}},
    {26, {XO(rings2_val)}},
    {30, {XO(perspective_angle), XO(perspective_dist), XO(persp_vsin), XO(persp_vfcos)}},
    {32, {XO(julian_power), XO(julian_dist), XO(julian_rN), XO(julian_cn)}},
    {33, {XO(juliascope_power), XO(juliascope_dist), XO(juliascope_rN), XO(juliascope_cn)}},
    {36, {XO(radial_blur_angle)}},
    {37, {XO(pie_slices), XO(pie_rotation), XO(pie_thickness)}},
    {38, {XO(ngon_sides), XO(ngon_power), XO(ngon_corners), XO(ngon_circle)}},
    {39, {XO(curl_c1), XO(curl_c2)}},
    {40, {XO(rectangles_x), XO(rectangles_y)}},
    {49, {XO(disc2_rot), XO(disc2_twist)}},
    {50, {XO(super_shape_rnd), XO(super_shape_m), XO(super_shape_n1), XO(super_shape_n2), XO(super_shape_n3),
          XO(super_shape_holes)}},
    {51, {XO(flower_petals)}},
    {52, {XO(conic_eccentricity), XO(conic_holes)}},
    {53, {XO(parabola_height), XO(parabola_width)}},
    {54, {XO(bent2_x), XO(bent2_y)}},
    {55, {XO(bipolar_shift)}},
    {58, {XO(cell_size)}},
    {59, {XO(cpow_i), XO(cpow_r), XO(cpow_power)}},
    {60, {XO(curve_xamp), XO(curve_yamp), XO(curve_xlength), XO(curve_ylength)}},
    {63, {XO(escher_beta)}},
    {65, {XO(lazysusan_x), XO(lazysusan_y), XO(lazysusan_spin), XO(lazysusan_space), XO(lazysusan_twist)}},
    {68, {XO(modulus_x), XO(modulus_y)}},
    {69, {XO(oscope_separation), XO(oscope_frequency), XO(oscope_amplitude), XO(oscope_damping)}},
    {71, {XO(popcorn2_x), XO(popcorn2_y), XO(popcorn2_c)}},
    {73, {XO(separation_x), XO(separation_y), XO(separation_xinside), XO(separation_yinside)}},
    {74, {XO(split_xsize), XO(split_ysize)}},
    {75, {XO(splits_x), XO(splits_y)}},
    {76, {XO(stripes_space), XO(stripes_warp)}},
    {77, {XO(wedge_angle), XO(wedge_hole), XO(wedge_count), XO(wedge_swirl)}},
    {78, {XO(wedge_julia_angle), XO(wedge_julia_count), XO(wedge_julia_power), XO(wedge_julia_dist),
          XO(wedgeJulia_cf), XO(wedgeJulia_cn), XO(wedgeJulia_rN)}},
    {79, {XO(wedge_sph_angle), XO(wedge_sph_hole), XO(wedge_sph_count), XO(wedge_sph_swirl)}},
    {80, {XO(whorl_inside), XO(whorl_outside)}},
    {81, {XO(waves2_scalex), XO(waves2_scaley), XO(waves2_freqx), XO(waves2_freqy)}},
    {96, {XO(auger_sym), XO(auger_weight), XO(auger_freq), XO(auger_scale)}},
    {97, {XO(flux_spread)}},
    {98, {XO(mobius_re_a), XO(mobius_re_b), XO(mobius_re_c), XO(mobius_re_d), XO(mobius_im_a), XO(mobius_im_b),
          XO(mobius_im_c), XO(mobius_im_d)}},
};
#define N_VARIATION_PARAMS ((int)(sizeof(kVariationParams) / sizeof(kVariationParams[0])))

static void take_params(flam3_xform *d, const flam3_xform *s, int var) {
  for (int r = 0; r < N_VARIATION_PARAMS; r++) {
    if (kVariationParams[r].var != var) continue;
    /* offset 0 is var[0], never a parameter: it ends each list */
    for (int k = 0; k < 8 && kVariationParams[r].off[k]; k++)
      XD(d, kVariationParams[r].off[k]) = XDC(s, kVariationParams[r].off[k]);
    return;
  }
}

/* Identity-like stand-ins for a padding xform, by what its neighbours use.
 * (1) under log-polar matrix blending, a neighbour with a variation that
 *     inverts or wraps the plane: linear -1 with the matrix -I; */
static const int kInvertingVariations[] = {2, 38, 32, 33, 5, 79, 78};
/* (2) otherwise a neighbour's parametric variation at parameters where it
 *     is the identity; */
static const struct {
  int var, n;
  size_t off[5];
  double val[5];
} kIdentityAt[] = {
    {40, 2, {XO(rectangles_x), XO(rectangles_y)}, {0.0, 0.0}},
    {26, 1, {XO(rings2_val)}, {0.0}},
    {25, 2, {XO(fan2_x), XO(fan2_y)}, {0.0, 0.0}},
    {23, 3, {XO(blob_low), XO(blob_high), XO(blob_waves)}, {1.0, 1.0, 1.0}},
    {30, 1, {XO(perspective_angle)}, {0.0}},
    {39, 2, {XO(curl_c1), XO(curl_c2)}, {0.0, 0.0}},
    {50, 5, {XO(super_shape_n1), XO(super_shape_n2), XO(super_shape_n3), XO(super_shape_rnd), XO(super_shape_holes)},
     {2.0, 2.0, 2.0, 0.0, 0.0}},
};
/* (3) otherwise a neighbour's fan or rings, with the axes swapped;
 * (4) otherwise plain linear. */
static const int kSwapVariations[] = {22, 21};

static void set_matrix(double m[3][2], double a, double b, double c, double d) {
  m[0][0] = a;
  m[0][1] = b;
  m[1][0] = c;
  m[1][1] = d;
  m[2][0] = 0.0;
  m[2][1] = 0.0;
}

static void pad_stand_in(flam3_genome *keys, int nkeys, int i, int xf) {
  flam3_xform *x = &keys[i].xform[xf];
  const flam3_xform *nb[2] = {NULL, NULL};
  int nnb = 0;
  for (int side = -1; side <= 1; side += 2) {
    const int k = i + side;
    if (k >= 0 && k < nkeys && keys[k].xform[xf].padding != 1) nb[nnb++] = &keys[k].xform[xf];
  }
  x->var[0] = 0.0;
  const int log_blend = (i == 0) ? keys[0].interpolation_type == 1 : keys[i - 1].interpolation_type == 1;
  if (log_blend) {
    int invert = 0;
    for (int a = 0; a < nnb; a++)
      for (size_t v = 0; v < sizeof(kInvertingVariations) / sizeof(int); v++)
        if (nb[a]->var[kInvertingVariations[v]] > 0) invert = 1;
    if (invert) {
      x->var[0] = -1.0;
      set_matrix(x->c, -1.0, 0.0, 0.0, -1.0);
      return;
    }
  }
  int found = 0;
  for (int a = 0; a < nnb; a++)
    for (size_t r = 0; r < sizeof(kIdentityAt) / sizeof(kIdentityAt[0]); r++)
      if (nb[a]->var[kIdentityAt[r].var] > 0) {
        x->var[kIdentityAt[r].var] = 1.0;
        for (int p = 0; p < kIdentityAt[r].n; p++) XD(x, kIdentityAt[r].off[p]) = kIdentityAt[r].val[p];
        found++;
      }
  if (!found) {
    for (int a = 0; a < nnb; a++)
      for (size_t v = 0; v < sizeof(kSwapVariations) / sizeof(int); v++)
        if (nb[a]->var[kSwapVariations[v]] > 0) {
          x->var[kSwapVariations[v]] = 1.0;
          found++;
        }
    if (found) set_matrix(x->c, 0.0, 1.0, 1.0, 0.0);
  }
  if (!found) {
    x->var[0] = 1.0;
    return;
  }
  double total = 0.0;
  for (int j = 0; j < flam3_nvariations; j++) total += x->var[j];
  for (int j = 0; j < flam3_nvariations; j++) x->var[j] /= total;
}

/* keys[0..nkeys) padded copies of src[0..nkeys) with equal xform counts */
static void align_keys(flam3_genome *keys, const flam3_genome *src, int nkeys) {
  int nstd = n_std(&src[0]), fin = src[0].final_xform_enable, uniform = 1;
  for (int i = 1; i < nkeys; i++) {
    if (n_std(&src[i]) != nstd) uniform = 0;
    if (n_std(&src[i]) > nstd) nstd = n_std(&src[i]);
    if (src[i].final_xform_enable != fin) uniform = 0;
    fin |= src[i].final_xform_enable;
  }
  for (int i = 0; i < nkeys; i++) padded_copy(&keys[i], &src[i], nstd, fin);
  /* the "old" and "older" interpolation types use the keys as they are */
  const int it = keys[nkeys / 2 - 1].interpolation_type;
  if (it == 2 || it == 3) return;
  for (int i = 0; i < nkeys; i++)
    for (int xf = 0; xf < nstd + fin; xf++) {
      /* a variation this key lacks takes its parameters from the previous key
       * (the first key: from the next) when that one uses it */
      const int from = i > 0 ? i - 1 : (nkeys > 1 ? 1 : -1);
      if (from >= 0)
        for (int j = 23; j < flam3_nvariations; j++)
          if (keys[i].xform[xf].var[j] == 0 && keys[from].xform[xf].var[j] != 0)
            take_params(&keys[i].xform[xf], &keys[from].xform[xf], j);
      if (keys[i].xform[xf].padding == 1 && !uniform) pad_stand_in(keys, nkeys, i, xf);
    }
}

/* ---- blending ----------------------------------------------------------- */

typedef struct {
  const flam3_genome *key; /* aligned keys */
  int n;
  const double *w; /* weights */
} blend_t;

/* weighted sum of the double at byte offset `off` of each key's genome */
static double g_sum(const blend_t *b, size_t off) {
  double acc = 0.0;
  for (int k = 0; k < b->n; k++) acc += b->w[k] * *(const double *)((const char *)&b->key[k] + off);
  return acc;
}

static double g_sum_int(const blend_t *b, size_t off) {
  double acc = 0.0;
  for (int k = 0; k < b->n; k++) acc += b->w[k] * *(const int *)((const char *)&b->key[k] + off);
  return acc;
}

/* weighted sums of a block of n doubles at byte offset `off` of xform xf */
static void x_block(const blend_t *b, const double *w, int xf, size_t off, size_t n, flam3_xform *out) {
  double *dst = (double *)((char *)out + off);
  for (size_t j = 0; j < n; j++) dst[j] = 0.0;
  for (size_t j = 0; j < n; j++)
    for (int k = 0; k < b->n; k++) dst[j] += w[k] * XDC(&b->key[k].xform[xf], off + j * sizeof(double));
}

static double clamp01(double v) { return v < 0 ? 0 : (v > 1 ? 1 : v); }

/* Genome scalars blended by weight; integers rounded to nearest. */
static const size_t kGenomeDoubles[] = {
    GO(brightness), GO(contrast), GO(highlight_power), GO(gamma), GO(vibrancy), GO(hue_rotation),
    GO(center[0]), GO(center[1]), GO(rot_center[0]), GO(rot_center[1]), GO(background[0]), GO(background[1]),
    GO(background[2]), GO(pixels_per_unit), GO(spatial_filter_radius), GO(temporal_filter_exp),
    GO(temporal_filter_width), GO(sample_density), GO(zoom), GO(rotate), GO(estimator), GO(estimator_minimum),
    GO(estimator_curve), GO(gam_lin_thresh),
};
static const size_t kGenomeInts[] = {GO(width), GO(height), GO(spatial_oversample), GO(nbatches),
                                     GO(ntemporal_samples)};

/* One column of an affine matrix in log-polar form: angle, magnitude and
 * translation (interpolation.c:173-323). */
typedef struct {
  double ang, mag, trn;
} polar_col;

/* The keys' matrix `which` (0: c, 1: post) of xform xf in polar form, angles
 * unwrapped along the keys (by the xform's winding for c when it has one,
 * else to the nearest turn). */
static void to_polar(const blend_t *b, int xf, int which, polar_col pc[4][2]) {
  for (int k = 0; k < b->n; k++) {
    const flam3_xform *x = &b->key[k].xform[xf];
    const double(*m)[2] = which ? x->post : x->c;
    int zero[2];
    for (int col = 0; col < 2; col++) {
      const double u = m[col][0], v = m[col][1];
      pc[k][col].ang = atan2(v, u);
      pc[k][col].mag = sqrt(u * u + v * v);
      pc[k][col].trn = m[2][col];
      zero[col] = pc[k][col].mag == 0.0;
    }
    /* a vanishing column takes the other column's angle */
    if (zero[0] && !zero[1]) pc[k][0].ang = pc[k][1].ang;
    if (zero[1] && !zero[0]) pc[k][1].ang = pc[k][0].ang;
  }
  const double turn = 2 * M_PI, eps = 1e-10;
  for (int col = 0; col < 2; col++)
    for (int k = 1; k < b->n; k++) {
      const double wind = b->key[k].xform[xf].wind[col];
      double *a0 = &pc[k - 1][col].ang, *a1 = &pc[k][col].ang;
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
}

/* Blend polar columns back to a matrix: angles and translations linearly,
 * magnitudes in log space unless some key's magnitude is below e^-10. */
static void from_polar(const blend_t *b, const double *w, polar_col pc[4][2], double m[3][2]) {
  for (int col = 0; col < 2; col++) {
    int linear_mag = 0;
    for (int k = 0; k < b->n; k++)
      if (log(pc[k][col].mag) < -10) linear_mag = 1;
    double ang = 0.0, mag = 0.0, trn = 0.0;
    for (int k = 0; k < b->n; k++) {
      ang += w[k] * pc[k][col].ang;
      mag += linear_mag ? w[k] * pc[k][col].mag : w[k] * log(pc[k][col].mag);
      trn += w[k] * pc[k][col].trn;
    }
    const double r = linear_mag ? mag : exp(mag);
    m[col][0] = r * cos(ang);
    m[col][1] = r * sin(ang);
    m[2][col] = trn;
  }
}

static int identity_matrix(const double m[3][2]) {
  return m[0][0] == 1.0 && m[0][1] == 0.0 && m[1][0] == 0.0 && m[1][1] == 1.0 && m[2][0] == 0.0 && m[2][1] == 0.0;
}

static void blend_matrices(const blend_t *b, const double *w, int xf, flam3_xform *out) {
  int posts_identity = 1;
  for (int k = 0; k < b->n; k++) posts_identity &= identity_matrix(b->key[k].xform[xf].post);
  if (b->key[0].interpolation_type == 1) {
    polar_col pc[4][2];
    to_polar(b, xf, 0, pc);
    from_polar(b, w, pc, out->c);
    if (posts_identity) {
      set_matrix(out->post, 1.0, 0.0, 0.0, 1.0);
    } else {
      to_polar(b, xf, 1, pc);
      from_polar(b, w, pc, out->post);
    }
    return;
  }
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 2; c++) {
      double a = 0.0, p = 0.0;
      for (int k = 0; k < b->n; k++) {
        a += w[k] * b->key[k].xform[xf].c[r][c];
        p += w[k] * b->key[k].xform[xf].post[r][c];
      }
      out->c[r][c] = a;
      out->post[r][c] = p;
    }
  if (posts_identity) set_matrix(out->post, 1.0, 0.0, 0.0, 1.0);
}

/* ---- colour (palettes.c:199-272) ----------------------------------------- */

static void rgb2hsv(const double *rgb, double *hsv) {
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

static void hsv2rgb(const double *hsv, double *rgb) {
  double h = hsv[0];
  const double s = hsv[1], v = hsv[2];
  while (h >= 6.0) h -= 6.0;
  while (h < 0.0) h += 6.0;
  const int sector = (int)floor(h);
  const double f = h - sector;
  const double p = v * (1 - s), q = v * (1 - (s * f)), t = v * (1 - (s * (1 - f)));
  /* (r, g, b) per sector as indices into {v, p, q, t} */
  static const unsigned char pick[6][3] = {{0, 3, 1}, {2, 0, 1}, {1, 0, 3}, {1, 2, 0}, {3, 1, 0}, {0, 1, 2}};
  const double val[4] = {v, p, q, t};
  const unsigned char *sel = pick[(sector >= 0 && sector < 6) ? sector : 0];
  for (int c = 0; c < 3; c++) rgb[c] = val[sel[c]];
}

/* Palette of the blend (interpolation.c:388-462).  Modes: 0 hsv, 1 sweep
 * (entries below 256*w[0] from the first key, the rest from the second),
 * 2 rgb, 3 hsv_circular (hsv with the first key's hue moved by a turn when
 * that brings it within half a turn of the second key's; two keys only). */
static void blend_palette(const blend_t *b, const double *w, flam3_genome *out) {
  const flam3_genome *k0 = &b->key[0];
  const int mode = k0->palette_interpolation;
  if (mode == 1) {
    for (int i = 0; i < 256; i++) out->palette[i] = b->key[(i < (256 * w[0])) ? 0 : 1].palette[i];
    return;
  }
  const double rgb_part = mode == 2 ? 1.0 : (mode == 3 ? k0->hsv_rgb_palette_blend : 0.0);
  double hsv[4][256][3];
  for (int k = 0; k < b->n; k++)
    for (int i = 0; i < 256; i++) rgb2hsv(b->key[k].palette[i].color, hsv[k][i]);
  if (b->n == 2 && mode == 3)
    for (int i = 0; i < 256; i++) {
      const double dh = hsv[1][i][0] - hsv[0][i][0];
      if (dh > 3.0)
        hsv[0][i][0] += 6.0;
      else if (dh < -3.0)
        hsv[0][i][0] -= 6.0;
    }
  for (int i = 0; i < 256; i++) {
    double rgb[3] = {0, 0, 0}, h[3] = {0, 0, 0}, alpha = 0, index = 0, back[3];
    int opaque = 1;
    for (int k = 0; k < b->n; k++) {
      const flam3_palette_entry *e = &b->key[k].palette[i];
      for (int c = 0; c < 3; c++) {
        rgb[c] += w[k] * e->color[c];
        h[c] += w[k] * hsv[k][i][c];
      }
      alpha += w[k] * e->color[3];
      opaque &= e->color[3] == 1.0;
      index += w[k] * e->index;
    }
    hsv2rgb(h, back);
    flam3_palette_entry *o = &out->palette[i];
    for (int c = 0; c < 3; c++) o->color[c] = rgb_part * rgb[c] + (1.0 - rgb_part) * back[c];
    o->color[3] = opaque ? 1.0 : alpha;
    o->index = index;
    for (int c = 0; c < 4; c++) o->color[c] = clamp01(o->color[c]);
    o->index = o->index < 0.0 ? 0.0 : (o->index > 255.0 ? 255.0 : o->index);
  }
}

/* Weight of the first of two keys for xform x under stagger: xforms start
 * and finish their move one after another, eased by 3t^2-2t^3
 * (interpolation.c:358-371). */
static double staggered(double t, double stagger, int nstd, int x) {
  const double spread = stagger * ((double)(nstd - 1) / nstd);
  const double start = spread * (nstd - 1 - x) / (nstd - 1);
  const double end = start + (1 - spread);
  if (t <= start) return 0;
  if (t >= end) return 1;
  const double u = (t - start) / (1 - spread);
  return 3 * u * u - 2 * u * u * u;
}

static void blend(const blend_t *b, double stagger, flam3_genome *out) {
  const flam3_genome *k0 = &b->key[0];
  blend_palette(b, b->w, out);
  out->palette_index = -1;
  out->symmetry = 0;
  out->spatial_filter_select = k0->spatial_filter_select;
  out->temporal_filter_type = k0->temporal_filter_type;
  out->palette_mode = k0->palette_mode;
  out->interpolation_type = k0->interpolation_type;
  out->palette_interpolation = k0->palette_interpolation;
  out->hsv_rgb_palette_blend = k0->hsv_rgb_palette_blend;
  for (size_t f = 0; f < sizeof(kGenomeDoubles) / sizeof(size_t); f++)
    *(double *)((char *)out + kGenomeDoubles[f]) = g_sum(b, kGenomeDoubles[f]);
  for (size_t f = 0; f < sizeof(kGenomeInts) / sizeof(size_t); f++)
    *(int *)((char *)out + kGenomeInts[f]) = (int)rint(g_sum_int(b, kGenomeInts[f]));
  const int nstd = n_std(k0);
  for (int i = 0; i < nstd; i++)
    for (int j = 0; j < nstd; j++) {
      double v = 0.0;
      for (int k = 0; k < b->n; k++) v += b->w[k] * b->key[k].chaos[i][j];
      out->chaos[i][j] = v < 0 ? 0 : v;
    }
  for (int xf = 0; xf < k0->num_xforms; xf++) {
    double w2[2];
    const double *w = b->w;
    if (b->n == 2 && stagger > 0 && xf != k0->final_xform_index) {
      w2[0] = staggered(b->w[0], stagger, nstd, xf);
      w2[1] = 1.0 - w2[0];
      w = w2;
    }
    flam3_xform *x = &out->xform[xf];
    x_block(b, w, xf, SCALAR_BLOCK_OFF, SCALAR_BLOCK_N, x);
    if (x->density < 0.0) x->density = 0.0;
    x->color = clamp01(x->color);
    x->color_speed = clamp01(x->color_speed);
    x_block(b, w, xf, PARAM_BLOCK_OFF, PARAM_BLOCK_N, x);
    x_block(b, w, xf, VAR_BLOCK_OFF, VAR_BLOCK_N, x);
    blend_matrices(b, w, xf, x);
  }
}

/* ---- flam3_interpolate (flam3.c:717-802) --------------------------------- */

static int interpolate_keys(const flam3_genome *cps, int ncps, double time, double stagger, flam3_genome *result) {
  if (ncps < 2) return 1;
  /* the segment [i1, i1+1] holding the time, clamped to the ends */
  int i1 = 0;
  if (cps[0].time >= time)
    i1 = 0;
  else if (cps[ncps - 1].time <= time)
    i1 = ncps - 2;
  else
    while (cps[i1 + 1].time < time) i1++;
  const int i2 = i1 + 1;
  double lin[2];
  lin[0] = (cps[i2].time - time) / (cps[i2].time - cps[i1].time);
  lin[1] = 1.0 - lin[0];
  flam3_genome keys[4];
  memset(keys, 0, sizeof(keys));
  /* smooth (Catmull-Rom) blending needs a key on each side of the segment;
   * on the first and last segment the reference reads outside the key list,
   * linear blending is used here */
  const int smooth = cps[i1].interpolation != 0 && i1 > 0 && i2 < ncps - 1;
  blend_t b;
  double cr[4];
  if (smooth) {
    align_keys(keys, &cps[i1 - 1], 4);
    const double t = lin[1], t2 = t * t, t3 = t2 * t;
    cr[0] = (2 * t2 - t - t3) / 2;
    cr[1] = (3 * t3 - 5 * t2 + 2) / 2;
    cr[2] = (4 * t2 - 3 * t3 + t) / 2;
    cr[3] = (t3 - t2) / 2;
    b = (blend_t){keys, 4, cr};
    stagger = 0;
  } else {
    align_keys(keys, &cps[i1], 2);
    b = (blend_t){keys, 2, lin};
  }
  memset(result, 0, sizeof(*result));
  genome_defaults(result);
  if (keys[0].final_xform_index >= 0) {
    grow_xforms(result, keys[0].num_xforms - 1, 0, 0);
    grow_xforms(result, 1, 0, 1);
  } else {
    grow_xforms(result, keys[0].num_xforms, 0, 0);
  }
  result->time = time;
  result->interpolation = 0;
  blend(&b, stagger, result);
  for (int k = 0; k < b.n; k++) release(&keys[k]);
  return 0;
}

/* ---- pieces of the blend for the device planner (f3g_plan.cu) ----------- */

/* The keys and weights a temporal sample at `time` blends: the first key of
 * its segment in cps, the key count (2, or 4 for Catmull-Rom) and the
 * weights, exactly as interpolate_keys chooses them (stagger 0). */
int f3g_interp_segment(const flam3_genome *cps, int ncps, double time, int *first, double w[4]) {
  if (ncps < 2) return -1;
  int i1 = 0;
  if (cps[0].time >= time)
    i1 = 0;
  else if (cps[ncps - 1].time <= time)
    i1 = ncps - 2;
  else
    while (cps[i1 + 1].time < time) i1++;
  const int i2 = i1 + 1;
  double lin0 = (cps[i2].time - time) / (cps[i2].time - cps[i1].time);
  double lin1 = 1.0 - lin0;
  if (cps[i1].interpolation != 0 && i1 > 0 && i2 < ncps - 1) {
    const double t = lin1, t2 = t * t, t3 = t2 * t;
    w[0] = (2 * t2 - t - t3) / 2;
    w[1] = (3 * t3 - 5 * t2 + 2) / 2;
    w[2] = (4 * t2 - 3 * t3 + t) / 2;
    w[3] = (t3 - t2) / 2;
    *first = i1 - 1;
    return 4;
  }
  w[0] = lin0;
  w[1] = lin1;
  w[2] = w[3] = 0.0;
  *first = i1;
  return 2;
}

void f3g_align_keys(flam3_genome *keys, const flam3_genome *src, int nkeys) { align_keys(keys, src, nkeys); }

void f3g_release_genome(flam3_genome *g) { release(g); }

/* The blended genome without its xforms' variations, parameters, matrices
 * and palette colours: the scalars, the xforms' densities and opacities, the
 * chaos rows and the palette's alpha -- what the host needs to size and
 * check a temporal sample whose genome the device blends.  Same arithmetic
 * as blend(). */
void f3g_blend_scalars(const flam3_genome *keys, int nk, const double *w, flam3_genome *out) {
  const blend_t b = {keys, nk, w};
  const flam3_genome *k0 = &keys[0];
  memset(out, 0, sizeof(*out));
  genome_defaults(out);
  if (k0->final_xform_index >= 0) {
    grow_xforms(out, k0->num_xforms - 1, 0, 0);
    grow_xforms(out, 1, 0, 1);
  } else {
    grow_xforms(out, k0->num_xforms, 0, 0);
  }
  out->interpolation = 0;
  out->palette_index = -1;
  out->spatial_filter_select = k0->spatial_filter_select;
  out->temporal_filter_type = k0->temporal_filter_type;
  out->palette_mode = k0->palette_mode;
  out->interpolation_type = k0->interpolation_type;
  out->palette_interpolation = k0->palette_interpolation;
  out->hsv_rgb_palette_blend = k0->hsv_rgb_palette_blend;
  for (size_t f = 0; f < sizeof(kGenomeDoubles) / sizeof(size_t); f++)
    *(double *)((char *)out + kGenomeDoubles[f]) = g_sum(&b, kGenomeDoubles[f]);
  for (size_t f = 0; f < sizeof(kGenomeInts) / sizeof(size_t); f++)
    *(int *)((char *)out + kGenomeInts[f]) = (int)rint(g_sum_int(&b, kGenomeInts[f]));
  const int nstd = n_std(k0);
  for (int i = 0; i < nstd; i++)
    for (int j = 0; j < nstd; j++) {
      double v = 0.0;
      for (int k = 0; k < nk; k++) v += w[k] * keys[k].chaos[i][j];
      out->chaos[i][j] = v < 0 ? 0 : v;
    }
  for (int xf = 0; xf < k0->num_xforms; xf++) {
    x_block(&b, w, xf, SCALAR_BLOCK_OFF, SCALAR_BLOCK_N, &out->xform[xf]);
    if (out->xform[xf].density < 0.0) out->xform[xf].density = 0.0;
  }
  for (int i = 0; i < 256; i++) {
    double alpha = 0.0;
    int opaque = 1;
    if (k0->palette_interpolation == 1) {
      out->palette[i].color[3] = keys[(i < (256 * w[0])) ? 0 : 1].palette[i].color[3];
      continue;
    }
    for (int k = 0; k < nk; k++) {
      alpha += w[k] * keys[k].palette[i].color[3];
      opaque &= keys[k].palette[i].color[3] == 1.0;
    }
    out->palette[i].color[3] = clamp01(opaque ? 1.0 : alpha);
  }
}

/* optional override: the reference's flam3_interpolate, when the caller links it */
static void (*g_interp)(flam3_genome *, int, double, double, flam3_genome *) = NULL;

void flam3gpu_set_interpolator(void (*fn)(flam3_genome *, int, double, double, flam3_genome *)) { g_interp = fn; }

int f3g_interp_overridden(void) { return g_interp != NULL; }

int f3g_interpolate_n(flam3_genome *cps, int ncps, double time, flam3_genome *result) {
  if (g_interp) {
    flam3_genome tmp;
    memset(&tmp, 0, sizeof(tmp));
    tmp.final_xform_index = -1;
    g_interp(cps, ncps, time, 0.0, &tmp);
    /* own a copy in this library's allocations */
    f3g_genome_copy(result, &tmp);
    return 0;
  }
  return interpolate_keys(cps, ncps, time, 0.0, result);
}

int flam3gpu_interpolate(flam3_genome *cps, int ncps, double time, double stagger, flam3_genome *result) {
  f3g_clear_error();
  if (ncps < 1) {
    f3g_set_error("no genomes to interpolate");
    return 1;
  }
  if (ncps == 1) {
    f3g_genome_copy(result, &cps[0]);
    return 0;
  }
  return interpolate_keys(cps, ncps, time, stagger, result);
}

void flam3gpu_free_genome(flam3_genome *g) { release(g); }

/* ---- helpers for the genome reader (xml.c) ------------------------------- */

/* clear_cp (flam3.c:1270-1368): defaults (default_flag 1) or the "unset"
 * markers (0); xforms, chaos and motion elements released; the name,
 * palette, time, edits and chaos flag kept */
void f3g_clear_cp(flam3_genome *cp, int default_flag) {
  release(cp);
  const double time = cp->time;
  char name[flam3_name_len + 1];
  memcpy(name, cp->flame_name, sizeof(name));
  flam3_palette pal;
  memcpy(pal, cp->palette, sizeof(pal));
  void *edits = cp->edits;
  const int chaos_enable = cp->chaos_enable;
  genome_defaults(cp);
  if (default_flag != 1) {
    cp->highlight_power = -1.0;
    cp->background[0] = cp->background[1] = cp->background[2] = -1.0;
    cp->zoom = 999999999;
    cp->spatial_oversample = -1;
    cp->spatial_filter_radius = -1;
    cp->width = -1;
    cp->height = -1;
    cp->sample_density = -1;
    cp->estimator = -1;
    cp->estimator_minimum = -1;
    cp->estimator_curve = -1;
    cp->gam_lin_thresh = -1;
    cp->nbatches = 0;
    cp->ntemporal_samples = 0;
    cp->spatial_filter_select = -1;
    cp->interpolation_type = -1;
    cp->temporal_filter_type = -1;
    cp->temporal_filter_width = -1;
    cp->temporal_filter_exp = -999;
    cp->palette_mode = -1;
  }
  cp->time = time;
  memcpy(cp->flame_name, name, sizeof(name));
  memcpy(cp->palette, pal, sizeof(pal));
  cp->edits = edits;
  cp->chaos_enable = chaos_enable;
}

void f3g_add_xforms(flam3_genome *cp, int num_to_add, int interp_padding, int final_flag) {
  grow_xforms(cp, num_to_add, interp_padding, final_flag);
}

void f3g_rgb2hsv(const double *rgb, double *hsv) { rgb2hsv(rgb, hsv); }
void f3g_hsv2rgb(const double *hsv, double *rgb) { hsv2rgb(hsv, rgb); }
