/*
 * interp.c -- genome interpolation for frames with several control points
 * (animation, motion blur).  Restates flam3_interpolate (flam3.c:717-802)
 * with flam3_align (interpolation.c:768-1033), flam3_copyx
 * (flam3.c:1211-1268), flam3_add_xforms (flam3.c:1033-1093),
 * initialize_xforms (variations.c:2401-2563), flam3_copy_params
 * (flam3.c:804-1005), flam3_interpolate_n (interpolation.c:373-709) and
 * interpolate_catmull_rom (interpolation.c:326-337), host FP64.
 *
 * Exported as flam3gpu_interpolate for standalone callers; a caller that
 * links the reference library can route the render through the reference's
 * own flam3_interpolate with flam3gpu_set_interpolator.
 */
#define _GNU_SOURCE
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "f3g_host.h"

#define EPSI 1e-10

/* ---- defaults ---- */

/* initialize_xforms (variations.c:2401-2563) for one xform */
static void init_xform(flam3_xform *x, int i) {
  memset(x, 0, sizeof(*x));
  x->color_speed = 0.5;
  x->animate = 1.0;
  x->color = i & 1;
  x->opacity = 1.0;
  x->var[0] = 1.0;
  x->c[0][0] = 1.0;
  x->c[1][1] = 1.0;
  x->post[0][0] = 1.0;
  x->post[1][1] = 1.0;
  x->blob_high = 1.0;
  x->blob_waves = 1.0;
  x->bent2_x = 1.0;
  x->bent2_y = 1.0;
  x->cell_size = 1.0;
  x->cpow_r = 1.0;
  x->cpow_power = 1.0;
  x->curve_xlength = 1.0;
  x->curve_ylength = 1.0;
  x->oscope_separation = 1.0;
  x->oscope_frequency = M_PI;
  x->oscope_amplitude = 1.0;
  x->wedge_count = 1.0;
  x->wedge_sph_count = 1.0;
  x->wedge_julia_power = 1.0;
  x->wedge_julia_count = 1.0;
  x->wedgeJulia_cn = 0.5;
  x->wedgeJulia_rN = 1.0;
  x->auger_freq = 1.0;
  x->auger_weight = 0.5;
  x->auger_scale = 1.0;
  x->julian_power = 1.0;
  x->julian_dist = 1.0;
  x->julian_rN = 1.0;
  x->julian_cn = 0.5;
  x->juliascope_power = 1.0;
  x->juliascope_dist = 1.0;
  x->juliascope_rN = 1.0;
  x->juliascope_cn = 0.5;
  x->radialBlur_zoomvar = 1.0;
  x->pie_slices = 6.0;
  x->pie_thickness = 0.5;
  x->ngon_sides = 5;
  x->ngon_power = 3;
  x->ngon_circle = 1;
  x->ngon_corners = 2;
  x->curl_c1 = 1.0;
  x->rectangles_x = 1.0;
  x->rectangles_y = 1.0;
  x->amw_amp = 1.0;
  x->super_shape_n1 = 1.0;
  x->super_shape_n2 = 1.0;
  x->super_shape_n3 = 1.0;
  x->conic_eccentricity = 1.0;
}

/* clear_cp(cp, flam3_defaults_on) (flam3.c:1270-1337) on an empty genome */
static void clear_defaults(flam3_genome *cp) {
  cp->palette_index = -1;
  cp->center[0] = cp->center[1] = 0.0;
  cp->rot_center[0] = cp->rot_center[1] = 0.0;
  cp->gamma = 4.0;
  cp->vibrancy = 1.0;
  cp->contrast = 1.0;
  cp->brightness = 4.0;
  cp->symmetry = 0;
  cp->hue_rotation = 0.0;
  cp->rotate = 0.0;
  cp->pixels_per_unit = 50;
  cp->interpolation = 0;
  cp->palette_interpolation = 3;
  cp->hsv_rgb_palette_blend = 0.0;
  cp->genome_index = 0;
  memset(cp->parent_fname, 0, sizeof(cp->parent_fname));
  cp->highlight_power = -1.0;
  cp->background[0] = cp->background[1] = cp->background[2] = 0.0;
  cp->width = 100;
  cp->height = 100;
  cp->spatial_oversample = 1;
  cp->spatial_filter_radius = 0.5;
  cp->zoom = 0.0;
  cp->sample_density = 1;
  cp->estimator = 9.0;
  cp->estimator_minimum = 0.0;
  cp->estimator_curve = 0.4;
  cp->gam_lin_thresh = 0.01;
  cp->nbatches = 1;
  cp->ntemporal_samples = 1000;
  cp->spatial_filter_select = 0;
  cp->interpolation_type = 1;
  cp->temporal_filter_type = 0;
  cp->temporal_filter_width = 1.0;
  cp->temporal_filter_exp = 0.0;
  cp->palette_mode = 0;
  cp->final_xform_enable = 0;
  cp->final_xform_index = -1;
}

/* flam3_add_xforms (flam3.c:1033-1093) */
static void add_xforms(flam3_genome *cp, int num_to_add, int interp_padding, int final_flag) {
  int old_num = cp->num_xforms;
  int oldstd = cp->num_xforms - (cp->final_xform_index >= 0);
  cp->xform = (flam3_xform *)realloc(cp->xform, (size_t)(cp->num_xforms + num_to_add) * sizeof(flam3_xform));
  cp->num_xforms += num_to_add;
  for (int i = old_num; i < cp->num_xforms; i++) {
    init_xform(&cp->xform[i], i);
    if (interp_padding) cp->xform[i].padding = 1;
  }
  if (cp->final_xform_index >= 0 && cp->final_xform_index != cp->num_xforms - 1) {
    flam3_xform tmp = cp->xform[cp->final_xform_index];
    for (int i = cp->final_xform_index; i < cp->num_xforms - 1; i++) cp->xform[i] = cp->xform[i + 1];
    cp->final_xform_index = cp->num_xforms - 1;
    cp->xform[cp->final_xform_index] = tmp;
  }
  if (final_flag) {
    cp->final_xform_enable = 1;
    cp->final_xform_index = cp->num_xforms - 1;
  } else {
    int numstd = cp->num_xforms - (cp->final_xform_index >= 0);
    for (int i = 0; i < oldstd; i++) {
      cp->chaos[i] = (double *)realloc(cp->chaos[i], (size_t)numstd * sizeof(double));
      for (int j = oldstd; j < numstd; j++) cp->chaos[i][j] = 1.0;
    }
    cp->chaos = (double **)realloc(cp->chaos, (size_t)numstd * sizeof(double *));
    for (int i = oldstd; i < numstd; i++) {
      cp->chaos[i] = (double *)malloc((size_t)numstd * sizeof(double));
      for (int j = 0; j < numstd; j++) cp->chaos[i][j] = 1.0;
    }
  }
}

static void free_genome(flam3_genome *g) {
  if (g->xform) {
    int ns = g->num_xforms - (g->final_xform_index >= 0);
    if (g->chaos) {
      for (int i = 0; i < ns; i++) free(g->chaos[i]);
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

static void copy_xform(flam3_xform *d, const flam3_xform *s) {
  *d = *s;
  d->num_motion = 0;
  d->motion = NULL;
}

/* flam3_copyx (flam3.c:1211-1268) */
static void copyx(flam3_genome *dest, const flam3_genome *src, int dest_std, int dest_final) {
  memcpy(dest, src, sizeof(flam3_genome));
  dest->num_xforms = 0;
  dest->xform = NULL;
  dest->chaos = NULL;
  dest->final_xform_index = -1;
  add_xforms(dest, dest_std, 1, 0);
  int numsrcstd = src->num_xforms - (src->final_xform_index >= 0);
  for (int i = 0; i < numsrcstd; i++) {
    copy_xform(&dest->xform[i], &src->xform[i]);
    memcpy(dest->chaos[i], src->chaos[i], (size_t)numsrcstd * sizeof(double));
  }
  if (dest_final > 0) {
    add_xforms(dest, dest_final, 1, 1);
    if (src->final_xform_enable > 0) {
      copy_xform(&dest->xform[dest->num_xforms - 1], &src->xform[src->final_xform_index]);
    } else {
      dest->xform[dest->num_xforms - 1].num_motion = 0;
      dest->xform[dest->num_xforms - 1].motion = NULL;
      dest->xform[dest->num_xforms - 1].animate = 0.0;
      dest->xform[dest->num_xforms - 1].color_speed = 0.0;
    }
  } else {
    dest->final_xform_index = -1;
    dest->final_xform_enable = 0;
  }
}

/* flam3_copy_params (flam3.c:804-1005): parameters of variation varn */
static void copy_params(flam3_xform *d, const flam3_xform *s, int varn) {
#define CP(f) d->f = s->f
  switch (varn) {
    case 23: CP(blob_low); CP(blob_high); CP(blob_waves); break;
    case 24: CP(pdj_a); CP(pdj_b); CP(pdj_c); CP(pdj_d); break;
    case 25: CP(fan2_x); CP(fan2_y); break;
    case 26: CP(rings2_val); break;
    case 30: CP(perspective_angle); CP(perspective_dist); CP(persp_vsin); CP(persp_vfcos); break;
    case 32: CP(julian_power); CP(julian_dist); CP(julian_rN); CP(julian_cn); break;
    case 33: CP(juliascope_power); CP(juliascope_dist); CP(juliascope_rN); CP(juliascope_cn); break;
    case 36: CP(radial_blur_angle); break;
    case 37: CP(pie_slices); CP(pie_rotation); CP(pie_thickness); break;
    case 38: CP(ngon_sides); CP(ngon_power); CP(ngon_corners); CP(ngon_circle); break;
    case 39: CP(curl_c1); CP(curl_c2); break;
    case 40: CP(rectangles_x); CP(rectangles_y); break;
    case 49: CP(disc2_rot); CP(disc2_twist); break;
    case 50:
      CP(super_shape_rnd); CP(super_shape_m); CP(super_shape_n1); CP(super_shape_n2); CP(super_shape_n3);
      CP(super_shape_holes);
      break;
    case 51: CP(flower_petals); break; /* the reference copies petals twice and never holes */
    case 52: CP(conic_eccentricity); CP(conic_holes); break;
    case 53: CP(parabola_height); CP(parabola_width); break;
    case 54: CP(bent2_x); CP(bent2_y); break;
    case 55: CP(bipolar_shift); break;
    case 58: CP(cell_size); break;
    case 59: CP(cpow_i); CP(cpow_r); CP(cpow_power); break;
    case 60: CP(curve_xamp); CP(curve_yamp); CP(curve_xlength); CP(curve_ylength); break;
    case 63: CP(escher_beta); break;
    case 65: CP(lazysusan_x); CP(lazysusan_y); CP(lazysusan_spin); CP(lazysusan_space); CP(lazysusan_twist); break;
    case 68: CP(modulus_x); CP(modulus_y); break;
    case 69: CP(oscope_separation); CP(oscope_frequency); CP(oscope_amplitude); CP(oscope_damping); break;
    case 71: CP(popcorn2_x); CP(popcorn2_y); CP(popcorn2_c); break;
    case 73: CP(separation_x); CP(separation_y); CP(separation_xinside); CP(separation_yinside); break;
    case 74: CP(split_xsize); CP(split_ysize); break;
    case 75: CP(splits_x); CP(splits_y); break;
    case 76: CP(stripes_space); CP(stripes_warp); break;
    case 77: CP(wedge_angle); CP(wedge_hole); CP(wedge_count); CP(wedge_swirl); break;
    case 78:
      CP(wedge_julia_angle); CP(wedge_julia_count); CP(wedge_julia_power); CP(wedge_julia_dist);
      CP(wedgeJulia_cf); CP(wedgeJulia_cn); CP(wedgeJulia_rN);
      break;
    case 79: CP(wedge_sph_angle); CP(wedge_sph_hole); CP(wedge_sph_count); CP(wedge_sph_swirl); break;
    case 80: CP(whorl_inside); CP(whorl_outside); break;
    case 81: CP(waves2_scalex); CP(waves2_scaley); CP(waves2_freqx); CP(waves2_freqy); break;
    case 96: CP(auger_sym); CP(auger_weight); CP(auger_freq); CP(auger_scale); break;
    case 97: CP(flux_spread); break;
    case 98:
      CP(mobius_re_a); CP(mobius_re_b); CP(mobius_re_c); CP(mobius_re_d);
      CP(mobius_im_a); CP(mobius_im_b); CP(mobius_im_c); CP(mobius_im_d);
      break;
    default: break;
  }
#undef CP
}

/* flam3_align (interpolation.c:768-1033) */
static void align(flam3_genome *dst, const flam3_genome *src, int nsrc) {
  int usethisone = (nsrc / 2) - 1;
  int max_nx = src[0].num_xforms - (src[0].final_xform_index >= 0);
  int max_fx = src[0].final_xform_enable, already_aligned = 1;
  for (int i = 1; i < nsrc; i++) {
    int tnx = src[i].num_xforms - (src[i].final_xform_index >= 0);
    if (max_nx != tnx) {
      already_aligned = 0;
      if (tnx > max_nx) max_nx = tnx;
    }
    int tfx = src[i].final_xform_enable;
    if (max_fx != tfx) {
      already_aligned = 0;
      max_fx |= tfx;
    }
  }
  for (int i = 0; i < nsrc; i++) copyx(&dst[i], &src[i], max_nx, max_fx);
  if (dst[usethisone].interpolation_type == 2 || dst[usethisone].interpolation_type == 3) return;
  for (int i = 0; i < nsrc; i++) {
    for (int xf = 0; xf < max_nx + max_fx; xf++) {
      for (int j = 23; j < flam3_nvariations; j++) {
        if (dst[i].xform[xf].var[j] != 0) continue;
        if (i > 0) {
          if (dst[i - 1].xform[xf].var[j] != 0) {
            copy_params(&dst[i].xform[xf], &dst[i - 1].xform[xf], j);
            continue;
          }
        } else if (i < nsrc - 1) {
          if (dst[i + 1].xform[xf].var[j] != 0) {
            copy_params(&dst[i].xform[xf], &dst[i + 1].xform[xf], j);
            continue;
          }
        }
      }
      flam3_xform *x = &dst[i].xform[xf];
      if (x->padding == 1 && !already_aligned) {
        int fnd = 0;
        x->var[0] = 0.0;
        if ((i == 0 && dst[i].interpolation_type == 1) || (i > 0 && dst[i - 1].interpolation_type == 1)) {
          for (int ii = -1; ii <= 1; ii += 2) {
            if (i + ii < 0 || i + ii >= nsrc) continue;
            const flam3_xform *o = &dst[i + ii].xform[xf];
            if (o->padding == 1) continue;
            if (o->var[2] > 0 || o->var[38] > 0 || o->var[32] > 0 || o->var[33] > 0 || o->var[5] > 0 ||
                o->var[79] > 0 || o->var[78] > 0) {
              x->var[0] = -1.0;
              x->c[0][0] = -1.0; x->c[0][1] = 0.0; x->c[1][0] = 0.0;
              x->c[1][1] = -1.0; x->c[2][0] = 0.0; x->c[2][1] = 0.0;
              fnd = -1;
            }
          }
        }
        if (fnd == 0) {
          for (int ii = -1; ii <= 1; ii += 2) {
            if (i + ii < 0 || i + ii >= nsrc) continue;
            const flam3_xform *o = &dst[i + ii].xform[xf];
            if (o->padding == 1) continue;
            if (o->var[40] > 0) { x->var[40] = 1.0; x->rectangles_x = 0.0; x->rectangles_y = 0.0; fnd++; }
            if (o->var[26] > 0) { x->var[26] = 1.0; x->rings2_val = 0.0; fnd++; }
            if (o->var[25] > 0) { x->var[25] = 1.0; x->fan2_x = 0.0; x->fan2_y = 0.0; fnd++; }
            if (o->var[23] > 0) {
              x->var[23] = 1.0; x->blob_low = 1.0; x->blob_high = 1.0; x->blob_waves = 1.0; fnd++;
            }
            if (o->var[30] > 0) { x->var[30] = 1.0; x->perspective_angle = 0.0; fnd++; }
            if (o->var[39] > 0) { x->var[39] = 1.0; x->curl_c1 = 0.0; x->curl_c2 = 0.0; fnd++; }
            if (o->var[50] > 0) {
              x->var[50] = 1.0;
              x->super_shape_n1 = 2.0; x->super_shape_n2 = 2.0; x->super_shape_n3 = 2.0;
              x->super_shape_rnd = 0.0; x->super_shape_holes = 0.0;
              fnd++;
            }
          }
        }
        if (fnd == 0) {
          for (int ii = -1; ii <= 1; ii += 2) {
            if (i + ii < 0 || i + ii >= nsrc) continue;
            const flam3_xform *o = &dst[i + ii].xform[xf];
            if (o->padding == 1) continue;
            if (o->var[22] > 0) { x->var[22] = 1.0; fnd++; }
            if (o->var[21] > 0) { x->var[21] = 1.0; fnd++; }
          }
          if (fnd > 0) {
            x->c[0][0] = 0.0; x->c[0][1] = 1.0; x->c[1][0] = 1.0;
            x->c[1][1] = 0.0; x->c[2][0] = 0.0; x->c[2][1] = 0.0;
          }
        }
        if (fnd == 0)
          x->var[0] = 1.0;
        else if (fnd > 0) {
          double normed = 0.0;
          for (int j = 0; j < flam3_nvariations; j++) normed += x->var[j];
          for (int j = 0; j < flam3_nvariations; j++) x->var[j] /= normed;
        }
      }
    }
  }
}

/* ---- interpolation of matrices (interpolation.c:173-323) ---- */

static int id_matrix(double s[3][2]) {
  return s[0][0] == 1.0 && s[0][1] == 0.0 && s[1][0] == 0.0 && s[1][1] == 1.0 && s[2][0] == 0.0 && s[2][1] == 0.0;
}

static void clear_matrix(double m[3][2]) { memset(m, 0, sizeof(double) * 6); }

static void sum_matrix(double s, double m1[3][2], double m2[3][2]) {
  for (int a = 0; a < 3; a++)
    for (int b = 0; b < 2; b++) m2[a][b] += s * m1[a][b];
}

static void interp_and_convert_back(const double *c, int ncps, double cxang[4][2], double cxmag[4][2],
                                    double cxtrn[4][2], double store[3][2]) {
  double accang[2] = {0, 0}, accmag[2] = {0, 0};
  int accmode[2] = {0, 0};
  for (int col = 0; col < 2; col++)
    for (int i = 0; i < ncps; i++)
      if (log(cxmag[i][col]) < -10) accmode[col] = 1;
  for (int i = 0; i < ncps; i++)
    for (int col = 0; col < 2; col++) {
      accang[col] += c[i] * cxang[i][col];
      if (accmode[col] == 0) accmag[col] += c[i] * log(cxmag[i][col]);
      else accmag[col] += c[i] * (cxmag[i][col]);
      store[2][col] += c[i] * cxtrn[i][col];
    }
  for (int col = 0; col < 2; col++) {
    double expmag = accmode[col] == 0 ? exp(accmag[col]) : accmag[col];
    store[col][0] = expmag * cos(accang[col]);
    store[col][1] = expmag * sin(accang[col]);
  }
}

static void convert_linear_to_polar(flam3_genome *cp, int ncps, int xfi, int cflag, double cxang[4][2],
                                    double cxmag[4][2], double cxtrn[4][2]) {
  double c1[2], d, t, refang;
  for (int k = 0; k < ncps; k++) {
    int zlm[2] = {0, 0};
    for (int col = 0; col < 2; col++) {
      if (cflag == 0) {
        c1[0] = cp[k].xform[xfi].c[col][0];
        c1[1] = cp[k].xform[xfi].c[col][1];
        t = cp[k].xform[xfi].c[2][col];
      } else {
        c1[0] = cp[k].xform[xfi].post[col][0];
        c1[1] = cp[k].xform[xfi].post[col][1];
        t = cp[k].xform[xfi].post[2][col];
      }
      cxang[k][col] = atan2(c1[1], c1[0]);
      cxmag[k][col] = sqrt(c1[0] * c1[0] + c1[1] * c1[1]);
      if (cxmag[k][col] == 0.0) zlm[col] = 1;
      cxtrn[k][col] = t;
    }
    if (zlm[0] == 1 && zlm[1] == 0) cxang[k][0] = cxang[k][1];
    else if (zlm[0] == 0 && zlm[1] == 1) cxang[k][1] = cxang[k][0];
  }
  for (int col = 0; col < 2; col++)
    for (int k = 1; k < ncps; k++) {
      if (cp[k].xform[xfi].wind[col] > 0 && cflag == 0) {
        refang = cp[k].xform[xfi].wind[col] - 2 * M_PI;
        while (cxang[k - 1][col] < refang) cxang[k - 1][col] += 2 * M_PI;
        while (cxang[k - 1][col] > refang + 2 * M_PI) cxang[k - 1][col] -= 2 * M_PI;
        while (cxang[k][col] < refang) cxang[k][col] += 2 * M_PI;
        while (cxang[k][col] > refang + 2 * M_PI) cxang[k][col] -= 2 * M_PI;
      } else {
        d = cxang[k][col] - cxang[k - 1][col];
        if (d > M_PI + EPSI) cxang[k][col] -= 2 * M_PI;
        else if (d < -(M_PI - EPSI)) cxang[k][col] += 2 * M_PI;
      }
    }
}

/* ---- colour (palettes.c:199-272) ---- */

static void rgb2hsv(const double *rgb, double *hsv) {
  double rd = rgb[0], gd = rgb[1], bd = rgb[2], mx, mn, del, h = 0, s, v;
  if (rd >= gd) mx = rd >= bd ? rd : bd;
  else mx = gd >= bd ? gd : bd;
  if (rd <= gd) mn = rd <= bd ? rd : bd;
  else mn = gd <= bd ? gd : bd;
  del = mx - mn;
  v = mx;
  s = mx != 0.0 ? del / mx : 0.0;
  if (s != 0.0) {
    double rc = (mx - rd) / del, gc = (mx - gd) / del, bc = (mx - bd) / del;
    if (rd == mx) h = bc - gc;
    else if (gd == mx) h = 2 + rc - bc;
    else if (bd == mx) h = 4 + gc - rc;
    if (h < 0) h += 6;
  }
  hsv[0] = h;
  hsv[1] = s;
  hsv[2] = v;
}

static void hsv2rgb(const double *hsv, double *rgb) {
  double h = hsv[0], s = hsv[1], v = hsv[2], f, p, q, t;
  while (h >= 6.0) h -= 6.0;
  while (h < 0.0) h += 6.0;
  int j = (int)floor(h);
  f = h - j;
  p = v * (1 - s);
  q = v * (1 - (s * f));
  t = v * (1 - (s * (1 - f)));
  switch (j) {
    case 0: rgb[0] = v; rgb[1] = t; rgb[2] = p; break;
    case 1: rgb[0] = q; rgb[1] = v; rgb[2] = p; break;
    case 2: rgb[0] = p; rgb[1] = v; rgb[2] = t; break;
    case 3: rgb[0] = p; rgb[1] = q; rgb[2] = v; break;
    case 4: rgb[0] = t; rgb[1] = p; rgb[2] = v; break;
    case 5: rgb[0] = v; rgb[1] = p; rgb[2] = q; break;
    default: rgb[0] = v; rgb[1] = t; rgb[2] = p; break;
  }
}

/* interpolation.c:358-371 */
static double smoother(double t) { return 3 * t * t - 2 * t * t * t; }

static double stagger_coef(double t, double stagger_prc, int num_xforms, int this_xform) {
  double max_stag = (double)(num_xforms - 1) / num_xforms;
  double stag_scaled = stagger_prc * max_stag;
  double st = stag_scaled * (num_xforms - 1 - this_xform) / (num_xforms - 1);
  double et = st + (1 - stag_scaled);
  if (t <= st) return 0;
  if (t >= et) return 1;
  return smoother((t - st) / (1 - stag_scaled));
}

#define IP(f)                                              \
  do {                                                     \
    result->f = 0.0;                                       \
    for (int k_ = 0; k_ < ncp; k_++) result->f += c[k_] * cpi[k_].f; \
  } while (0)
#define II(f)                                              \
  do {                                                     \
    double tt_ = 0.0;                                      \
    for (int k_ = 0; k_ < ncp; k_++) tt_ += c[k_] * cpi[k_].f; \
    result->f = (int)rint(tt_);                            \
  } while (0)

/* flam3_interpolate_n (interpolation.c:373-709) */
static void interpolate_n(flam3_genome *result, int ncp, flam3_genome *cpi, double *c, double stagger) {
  if (cpi[0].palette_interpolation != 1) {
    double rgb_fraction = 0.0;
    if (cpi[0].palette_interpolation == 2) rgb_fraction = 1.0;
    else if (cpi[0].palette_interpolation == 3) rgb_fraction = cpi[0].hsv_rgb_palette_blend;
    for (int i = 0; i < 256; i++) {
      double col_rgb[3], col_hsv[3], new_rgb[3] = {0, 0, 0}, new_hsv[3] = {0, 0, 0};
      double new_count = 0, new_index = 0;
      int alpha1 = 1;
      for (int k = 0; k < ncp; k++) {
        rgb2hsv(cpi[k].palette[i].color, col_hsv);
        for (int l = 0; l < 3; l++) col_rgb[l] = cpi[k].palette[i].color[l];
        if (2 == ncp && k == 0 && cpi[0].palette_interpolation == 3) {
          double second[3];
          rgb2hsv(cpi[1].palette[i].color, second);
          if ((second[0] - col_hsv[0]) > 3.0) col_hsv[0] += 6.0;
          else if ((second[0] - col_hsv[0]) < -3.0) col_hsv[0] -= 6.0;
        }
        for (int j = 0; j < 3; j++) {
          new_rgb[j] += c[k] * col_rgb[j];
          new_hsv[j] += c[k] * col_hsv[j];
        }
        new_count += c[k] * cpi[k].palette[i].color[3];
        if (cpi[k].palette[i].color[3] != 1.0) alpha1 = 0;
        new_index += c[k] * cpi[k].palette[i].index;
      }
      if (alpha1 == 1) new_count = 1.0;
      double hr[3];
      hsv2rgb(new_hsv, hr);
      for (int l = 0; l < 3; l++) result->palette[i].color[l] = rgb_fraction * new_rgb[l] + (1.0 - rgb_fraction) * hr[l];
      result->palette[i].color[3] = new_count;
      result->palette[i].index = new_index;
      for (int j = 0; j < 4; j++) {
        if (result->palette[i].color[j] < 0.0) result->palette[i].color[j] = 0.0;
        if (result->palette[i].color[j] > 1.0) result->palette[i].color[j] = 1.0;
      }
      if (result->palette[i].index < 0.0) result->palette[i].index = 0.0;
      if (result->palette[i].index > 255.0) result->palette[i].index = 255.0;
    }
  } else {
    for (int i = 0; i < 256; i++) {
      int j = (i < (256 * c[0])) ? 0 : 1;
      result->palette[i] = cpi[j].palette[i];
    }
  }
  result->palette_index = -1;
  result->symmetry = 0;
  result->spatial_filter_select = cpi[0].spatial_filter_select;
  result->temporal_filter_type = cpi[0].temporal_filter_type;
  result->palette_mode = cpi[0].palette_mode;
  result->interpolation_type = cpi[0].interpolation_type;
  result->palette_interpolation = cpi[0].palette_interpolation;
  result->hsv_rgb_palette_blend = cpi[0].hsv_rgb_palette_blend;
  IP(brightness); IP(contrast); IP(highlight_power); IP(gamma); IP(vibrancy); IP(hue_rotation);
  II(width); II(height); II(spatial_oversample);
  IP(center[0]); IP(center[1]); IP(rot_center[0]); IP(rot_center[1]);
  IP(background[0]); IP(background[1]); IP(background[2]);
  IP(pixels_per_unit); IP(spatial_filter_radius); IP(temporal_filter_exp); IP(temporal_filter_width);
  IP(sample_density); IP(zoom); IP(rotate);
  II(nbatches); II(ntemporal_samples);
  IP(estimator); IP(estimator_minimum); IP(estimator_curve); IP(gam_lin_thresh);
  int numstd = cpi[0].num_xforms - (cpi[0].final_xform_index >= 0);
  for (int i = 0; i < numstd; i++)
    for (int j = 0; j < numstd; j++) {
      IP(chaos[i][j]);
      if (result->chaos[i][j] < 0) result->chaos[i][j] = 0;
    }
  for (int i = 0; i < cpi[0].num_xforms; i++) {
    double csave[2] = {0, 0};
    int nx = cpi[0].num_xforms - (cpi[0].final_xform_index >= 0);
    if (ncp == 2 && stagger > 0 && i != cpi[0].final_xform_index) {
      csave[0] = c[0];
      csave[1] = c[1];
      c[0] = stagger_coef(csave[0], stagger, nx, i);
      c[1] = 1.0 - c[0];
    }
    IP(xform[i].density);
    if (result->xform[i].density < 0.0) result->xform[i].density = 0.0;
    IP(xform[i].color);
    if (result->xform[i].color < 0) result->xform[i].color = 0;
    if (result->xform[i].color > 1) result->xform[i].color = 1;
    IP(xform[i].color_speed);
    if (result->xform[i].color_speed < 0) result->xform[i].color_speed = 0;
    if (result->xform[i].color_speed > 1) result->xform[i].color_speed = 1;
    IP(xform[i].opacity);
    IP(xform[i].animate);
    /* every variation parameter (interpolation.c:545-651) */
    IP(xform[i].blob_low); IP(xform[i].blob_high); IP(xform[i].blob_waves);
    IP(xform[i].pdj_a); IP(xform[i].pdj_b); IP(xform[i].pdj_c); IP(xform[i].pdj_d);
    IP(xform[i].fan2_x); IP(xform[i].fan2_y); IP(xform[i].rings2_val);
    IP(xform[i].perspective_angle); IP(xform[i].perspective_dist);
    IP(xform[i].julian_power); IP(xform[i].julian_dist);
    IP(xform[i].juliascope_power); IP(xform[i].juliascope_dist);
    IP(xform[i].radial_blur_angle);
    IP(xform[i].pie_slices); IP(xform[i].pie_rotation); IP(xform[i].pie_thickness);
    IP(xform[i].ngon_sides); IP(xform[i].ngon_power); IP(xform[i].ngon_circle); IP(xform[i].ngon_corners);
    IP(xform[i].curl_c1); IP(xform[i].curl_c2);
    IP(xform[i].rectangles_x); IP(xform[i].rectangles_y);
    IP(xform[i].amw_amp);
    IP(xform[i].disc2_rot); IP(xform[i].disc2_twist);
    IP(xform[i].super_shape_rnd); IP(xform[i].super_shape_m); IP(xform[i].super_shape_n1);
    IP(xform[i].super_shape_n2); IP(xform[i].super_shape_n3); IP(xform[i].super_shape_holes);
    IP(xform[i].flower_petals); IP(xform[i].flower_holes);
    IP(xform[i].conic_eccentricity); IP(xform[i].conic_holes);
    IP(xform[i].parabola_height); IP(xform[i].parabola_width);
    IP(xform[i].bent2_x); IP(xform[i].bent2_y);
    IP(xform[i].bipolar_shift); IP(xform[i].cell_size);
    IP(xform[i].cpow_r); IP(xform[i].cpow_i); IP(xform[i].cpow_power);
    IP(xform[i].curve_xamp); IP(xform[i].curve_yamp); IP(xform[i].curve_xlength); IP(xform[i].curve_ylength);
    IP(xform[i].escher_beta);
    IP(xform[i].lazysusan_x); IP(xform[i].lazysusan_y); IP(xform[i].lazysusan_twist);
    IP(xform[i].lazysusan_space); IP(xform[i].lazysusan_spin);
    IP(xform[i].modulus_x); IP(xform[i].modulus_y);
    IP(xform[i].oscope_separation); IP(xform[i].oscope_frequency); IP(xform[i].oscope_amplitude);
    IP(xform[i].oscope_damping);
    IP(xform[i].popcorn2_x); IP(xform[i].popcorn2_y); IP(xform[i].popcorn2_c);
    IP(xform[i].separation_x); IP(xform[i].separation_xinside); IP(xform[i].separation_y);
    IP(xform[i].separation_yinside);
    IP(xform[i].split_xsize); IP(xform[i].split_ysize); IP(xform[i].splits_x); IP(xform[i].splits_y);
    IP(xform[i].stripes_space); IP(xform[i].stripes_warp);
    IP(xform[i].wedge_angle); IP(xform[i].wedge_hole); IP(xform[i].wedge_count); IP(xform[i].wedge_swirl);
    IP(xform[i].wedge_julia_angle); IP(xform[i].wedge_julia_count); IP(xform[i].wedge_julia_power);
    IP(xform[i].wedge_julia_dist);
    IP(xform[i].wedge_sph_angle); IP(xform[i].wedge_sph_hole); IP(xform[i].wedge_sph_count);
    IP(xform[i].wedge_sph_swirl);
    IP(xform[i].whorl_inside); IP(xform[i].whorl_outside);
    IP(xform[i].waves2_scalex); IP(xform[i].waves2_scaley); IP(xform[i].waves2_freqx); IP(xform[i].waves2_freqy);
    IP(xform[i].auger_sym); IP(xform[i].auger_weight); IP(xform[i].auger_freq); IP(xform[i].auger_scale);
    IP(xform[i].flux_spread);
    IP(xform[i].mobius_re_a); IP(xform[i].mobius_im_a); IP(xform[i].mobius_re_b); IP(xform[i].mobius_im_b);
    IP(xform[i].mobius_re_c); IP(xform[i].mobius_im_c); IP(xform[i].mobius_re_d); IP(xform[i].mobius_im_d);
    for (int j = 0; j < flam3_nvariations; j++) IP(xform[i].var[j]);
    if (cpi[0].interpolation_type == 1) {
      double cxmag[4][2], cxang[4][2], cxtrn[4][2];
      clear_matrix(result->xform[i].c);
      convert_linear_to_polar(cpi, ncp, i, 0, cxang, cxmag, cxtrn);
      interp_and_convert_back(c, ncp, cxang, cxmag, cxtrn, result->xform[i].c);
      int all_id = 1;
      for (int k = 0; k < ncp; k++) all_id &= id_matrix(cpi[k].xform[i].post);
      clear_matrix(result->xform[i].post);
      if (all_id) {
        result->xform[i].post[0][0] = 1.0;
        result->xform[i].post[1][1] = 1.0;
      } else {
        convert_linear_to_polar(cpi, ncp, i, 1, cxang, cxmag, cxtrn);
        interp_and_convert_back(c, ncp, cxang, cxmag, cxtrn, result->xform[i].post);
      }
    } else {
      clear_matrix(result->xform[i].c);
      clear_matrix(result->xform[i].post);
      int all_id = 1;
      for (int k = 0; k < ncp; k++) {
        sum_matrix(c[k], cpi[k].xform[i].c, result->xform[i].c);
        sum_matrix(c[k], cpi[k].xform[i].post, result->xform[i].post);
        all_id &= id_matrix(cpi[k].xform[i].post);
      }
      if (all_id) {
        clear_matrix(result->xform[i].post);
        result->xform[i].post[0][0] = 1.0;
        result->xform[i].post[1][1] = 1.0;
      }
    }
    if (ncp == 2 && stagger > 0 && i != cpi[0].final_xform_index) {
      c[0] = csave[0];
      c[1] = csave[1];
    }
  }
}

/* flam3_interpolate (flam3.c:717-802) for ncps >= 2 into an empty result */
static int interpolate_frame(flam3_genome *cps, int ncps, double time, double stagger, flam3_genome *result) {
  int i1, i2, smoothflag = 0;
  double c[4];
  flam3_genome cpi[4];
  if (ncps < 2) return 1;
  if (cps[0].time >= time) {
    i1 = 0;
    i2 = 1;
  } else if (cps[ncps - 1].time <= time) {
    i1 = ncps - 2;
    i2 = ncps - 1;
  } else {
    i1 = 0;
    while (cps[i1].time < time) i1++;
    i1--;
    i2 = i1 + 1;
  }
  c[0] = (cps[i2].time - time) / (cps[i2].time - cps[i1].time);
  c[1] = 1.0 - c[0];
  memset(cpi, 0, sizeof(cpi));
  if (cps[i1].interpolation == 0) {
    align(cpi, &cps[i1], 2);
    smoothflag = 0;
  } else {
    if (0 == i1 || ncps - 1 == i2) {
      /* smooth interpolation needs a neighbour on each side: the reference
       * prints an error and aligns linearly first; it then still aligns four
       * genomes from i1-1, reading outside the list.  Linear is used here. */
      align(cpi, &cps[i1], 2);
      smoothflag = 0;
    } else {
      align(cpi, &cps[i1 - 1], 4);
      smoothflag = 1;
    }
  }
  memset(result, 0, sizeof(*result));
  clear_defaults(result);
  if (cpi[0].final_xform_index >= 0) {
    add_xforms(result, cpi[0].num_xforms - 1, 0, 0);
    add_xforms(result, 1, 0, 1);
  } else
    add_xforms(result, cpi[0].num_xforms, 0, 0);
  result->time = time;
  result->interpolation = 0;
  result->interpolation_type = cpi[0].interpolation_type;
  result->palette_interpolation = 3;
  result->hsv_rgb_palette_blend = 0.0;
  if (!smoothflag) {
    interpolate_n(result, 2, cpi, c, stagger);
  } else {
    double t = c[1], t2 = t * t, t3 = t2 * t, cmc[4];
    cmc[0] = (2 * t2 - t - t3) / 2;
    cmc[1] = (3 * t3 - 5 * t2 + 2) / 2;
    cmc[2] = (4 * t2 - 3 * t3 + t) / 2;
    cmc[3] = (t3 - t2) / 2;
    interpolate_n(result, 4, cpi, cmc, 0);
    free_genome(&cpi[2]);
    free_genome(&cpi[3]);
  }
  free_genome(&cpi[0]);
  free_genome(&cpi[1]);
  return 0;
}

/* optional override: the reference's flam3_interpolate, when the caller links it */
static void (*g_interp)(flam3_genome *, int, double, double, flam3_genome *) = NULL;

void flam3gpu_set_interpolator(void (*fn)(flam3_genome *, int, double, double, flam3_genome *)) { g_interp = fn; }

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
  return interpolate_frame(cps, ncps, time, 0.0, result);
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
  return interpolate_frame(cps, ncps, time, stagger, result);
}

void flam3gpu_free_genome(flam3_genome *g) { free_genome(g); }

/* ---- helpers for the genome reader (xml.c) ---- */

/* clear_cp (flam3.c:1270-1368): defaults (default_flag 1) or the
 * "unset" markers (0), xforms, chaos and motion elements released */
void f3g_clear_cp(flam3_genome *cp, int default_flag) {
  free_genome(cp);
  const double time = cp->time;
  char name[flam3_name_len + 1];
  memcpy(name, cp->flame_name, sizeof(name));
  flam3_palette pal;
  memcpy(pal, cp->palette, sizeof(pal));
  void *edits = cp->edits;
  const int chaos_enable = cp->chaos_enable;
  clear_defaults(cp);
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
  /* fields clear_cp does not touch keep their values */
  cp->time = time;
  memcpy(cp->flame_name, name, sizeof(name));
  memcpy(cp->palette, pal, sizeof(pal));
  cp->edits = edits;
  cp->chaos_enable = chaos_enable;
}

void f3g_add_xforms(flam3_genome *cp, int num_to_add, int interp_padding, int final_flag) {
  add_xforms(cp, num_to_add, interp_padding, final_flag);
}

void f3g_rgb2hsv(const double *rgb, double *hsv) { rgb2hsv(rgb, hsv); }
void f3g_hsv2rgb(const double *hsv, double *rgb) { hsv2rgb(hsv, rgb); }
