/*
 * filters.c -- host construction of the spatial, density-estimation and
 * temporal filters (reference filters.c:29-489).  The tables are small and
 * built in FP64 on the host exactly as the reference builds them; the
 * kernels receive FP32 copies.
 */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "f3g_host.h"

/* support of each spatial kernel, indexed like flam3_spatial_filter's knum */
static const double support[14] = {1.5, 1.0, 0.5, 1.0, 1.5, 2.0, 2.0, 1.0, 2.0, 1.0, 1.0, 3.0, 2.0, 1.5};

static double sinc(double x) {
  x *= M_PI;
  return x != 0 ? sin(x) / x : 1.0;
}

static double kernel(int knum, double x) {
  double t = x < 0 ? -x : x, tt;
  switch (knum) {
    case 0: return exp(-2.0 * x * x) * sqrt(2.0 / M_PI);                      /* gaussian */
    case 1: return t < 1.0 ? (2.0 * t - 3.0) * t * t + 1.0 : 0.0;             /* hermite */
    case 2: return (x > -0.5 && x <= 0.5) ? 1.0 : 0.0;                          /* box */
    case 3: return t < 1.0 ? 1.0 - t : 0.0;                                    /* triangle */
    case 4:                                                                    /* bell */
      if (t < .5) return .75 - t * t;
      if (t < 1.5) { t -= 1.5; return .5 * t * t; }
      return 0.0;
    case 5:                                                                    /* b-spline */
      if (t < 1) { tt = t * t; return .5 * tt * t - tt + 2.0 / 3.0; }
      if (t < 2) { t = 2 - t; return (1.0 / 6.0) * t * t * t; }
      return 0.0;
    case 6: { /* mitchell, B = C = 1/3 */
      const double B = 1.0 / 3.0, C = 1.0 / 3.0;
      tt = x * x;
      if (t < 1.0) return ((12.0 - 9.0 * B - 6.0 * C) * (t * tt) + (-18.0 + 12.0 * B + 6.0 * C) * tt + (6.0 - 2 * B)) / 6.0;
      if (t < 2.0)
        return ((-1.0 * B - 6.0 * C) * (t * tt) + (6.0 * B + 30.0 * C) * tt + (-12.0 * B - 48.0 * C) * t +
                (8.0 * B + 24 * C)) / 6.0;
      return 0.0;
    }
    case 7: return sinc(x) * (0.42 + 0.5 * cos(M_PI * x) + 0.08 * cos(2 * M_PI * x)); /* blackman */
    case 8:                                                                    /* catmull-rom */
      if (x < -2.0) return 0.0;
      if (x < -1.0) return 0.5 * (4.0 + x * (8.0 + x * (5.0 + x)));
      if (x < 0.0) return 0.5 * (2.0 + x * x * (-5.0 - 3.0 * x));
      if (x < 1.0) return 0.5 * (2.0 + x * x * (-5.0 + 3.0 * x));
      if (x < 2.0) return 0.5 * (4.0 + x * (-8.0 + x * (5.0 - x)));
      return 0.0;
    case 9: return sinc(x) * (0.5 + 0.5 * cos(M_PI * x));                      /* hanning */
    case 10: return sinc(x) * (0.54 + 0.46 * cos(M_PI * x));                   /* hamming */
    case 11: return (t < 3.0 ? sinc(t) * sinc(t / 3.0) : 0.0) * sinc(x / 3.0); /* lanczos3 */
    case 12: return (t < 2.0 ? sinc(t) * sinc(t / 2.0) : 0.0) * sinc(x / 2.0); /* lanczos2 */
    default:                                                                   /* quadratic */
      if (x < -1.5) return 0.0;
      if (x < -0.5) return 0.5 * (x + 1.5) * (x + 1.5);
      if (x < 0.5) return 0.75 - x * x;
      if (x < 1.5) return 0.5 * (x - 1.5) * (x - 1.5);
      return 0.0;
  }
}

/* filters.c:217-270 */
int f3g_spatial_filter(flam3_frame *spec, int field, double **filter) {
  int knum = spec->genomes[0].spatial_filter_select;
  if (knum < 0 || knum > 13) {
    f3g_set_error("unknown spatial filter %d", knum);
    return -1;
  }
  int ss = spec->genomes[0].spatial_oversample;
  double radius = spec->genomes[0].spatial_filter_radius, aspect = spec->pixel_aspect_ratio;
  double supp = support[knum];
  double fw = 2.0 * supp * ss * radius / aspect, adjust;
  int fwidth = ((int)fw) + 1;
  if ((fwidth ^ ss) & 1) fwidth++;
  adjust = fw > 0.0 ? supp * fwidth / fw : 1.0;
  /* fw x fw filter, then its vertical and horizontal factors */
  double *f = (double *)calloc(F3G_FILTER_FLOATS(fwidth), sizeof(double));
  if (!f) {
    f3g_set_error("out of host memory");
    return -1;
  }
  double *fu = f + (size_t)fwidth * fwidth, *fv = fu + fwidth;
  double sum = 0.0, sum_h = 0.0;
  for (int i = 0; i < fwidth; i++) {
    double ii = ((2.0 * i + 1.0) / (double)fwidth - 1.0) * adjust;
    double jj = ((2.0 * i + 1.0) / (double)fwidth - 1.0) * adjust;
    if (field) jj *= 2.0;
    jj /= aspect;
    fv[i] = kernel(knum, ii);
    fu[i] = kernel(knum, jj);
    sum_h += fv[i];
  }
  for (int i = 0; i < fwidth; i++)
    for (int j = 0; j < fwidth; j++) f[i + j * fwidth] = fv[i] * fu[j];
  for (int i = 0; i < fwidth * fwidth; i++) sum += f[i];
  if (sum == 0.0 || sum_h == 0.0) {
    free(f);
    f3g_set_error("Spatial filter value is too small: %g.", radius);
    return -1;
  }
  sum = 1.0 / sum;
  for (int i = 0; i < fwidth * fwidth; i++) f[i] *= sum;
  /* fu[j] * fv[i] == f[i + j*fw]: the horizontal factor sums to one */
  for (int i = 0; i < fwidth; i++) {
    fu[i] *= sum * sum_h;
    fv[i] /= sum_h;
  }
  *filter = f;
  return fwidth;
}

/* filters.c:272-407 */
static int de_filters_build(double max_rad, double min_rad, double curve, int ss, int *max_filtered_counts,
                            int *max_filter_index, double **widths, double **coefs);

/* The filter bank depends only on (max_rad, min_rad, curve, ss) and costs up
 * to ~2 ms to build for large radii at oversample 2: the last banks built
 * are kept (process-wide) and handed out as copies. */
#define DE_CACHE 32
static struct {
  double max_rad, min_rad, curve;
  int ss, mfc, mfi, ks;
  double *w, *c;
  unsigned long long used;
} de_cache[DE_CACHE];
static unsigned long long de_clock;
static pthread_mutex_t de_mu = PTHREAD_MUTEX_INITIALIZER;

int f3g_de_filters(double max_rad, double min_rad, double curve, int ss, int *max_filtered_counts,
                   int *max_filter_index, double **widths, double **coefs) {
  pthread_mutex_lock(&de_mu);
  for (int i = 0; i < DE_CACHE; i++)
    if (de_cache[i].w && de_cache[i].max_rad == max_rad && de_cache[i].min_rad == min_rad &&
        de_cache[i].curve == curve && de_cache[i].ss == ss) {
      const int n = de_cache[i].mfi + 1, ks = de_cache[i].ks;
      double *w = (double *)malloc((size_t)n * sizeof(double));
      double *c = (double *)malloc((size_t)n * ks * sizeof(double));
      if (!w || !c) {
        free(w);
        free(c);
        break;
      }
      memcpy(w, de_cache[i].w, (size_t)n * sizeof(double));
      memcpy(c, de_cache[i].c, (size_t)n * ks * sizeof(double));
      *widths = w;
      *coefs = c;
      *max_filtered_counts = de_cache[i].mfc;
      *max_filter_index = de_cache[i].mfi;
      de_cache[i].used = ++de_clock;
      pthread_mutex_unlock(&de_mu);
      return ks;
    }
  pthread_mutex_unlock(&de_mu);
  const int ks = de_filters_build(max_rad, min_rad, curve, ss, max_filtered_counts, max_filter_index, widths, coefs);
  if (ks <= 0) return ks;
  const int n = *max_filter_index + 1;
  double *w = (double *)malloc((size_t)n * sizeof(double));
  double *c = (double *)malloc((size_t)n * ks * sizeof(double));
  if (!w || !c) {
    free(w);
    free(c);
    return ks;
  }
  memcpy(w, *widths, (size_t)n * sizeof(double));
  memcpy(c, *coefs, (size_t)n * ks * sizeof(double));
  pthread_mutex_lock(&de_mu);
  int v = 0;
  for (int i = 1; i < DE_CACHE; i++)
    if (!de_cache[i].w || (de_cache[v].w && de_cache[i].used < de_cache[v].used)) v = i;
  free(de_cache[v].w);
  free(de_cache[v].c);
  de_cache[v].max_rad = max_rad;
  de_cache[v].min_rad = min_rad;
  de_cache[v].curve = curve;
  de_cache[v].ss = ss;
  de_cache[v].mfc = *max_filtered_counts;
  de_cache[v].mfi = *max_filter_index;
  de_cache[v].ks = ks;
  de_cache[v].w = w;
  de_cache[v].c = c;
  de_cache[v].used = ++de_clock;
  pthread_mutex_unlock(&de_mu);
  return ks;
}

static int de_filters_build(double max_rad, double min_rad, double curve, int ss, int *max_filtered_counts,
                            int *max_filter_index, double **widths, double **coefs) {
  const int keep = 100;
  if (curve <= 0.0) {
    f3g_set_error("estimator curve must be > 0");
    return -1;
  }
  if (max_rad < min_rad) {
    f3g_set_error("estimator must be larger than estimator_minimum (%f > %f)", max_rad, min_rad);
    return -1;
  }
  double cmax = max_rad * ss + 1, cmin = min_rad * ss + 1;
  double nd = pow(cmax / cmin, 1.0 / curve);
  if (nd > 1e7) {
    f3g_set_error("too many filters required in this configuration (%g)", nd);
    return -1;
  }
  int n = (int)ceil(nd), max_ind;
  if (n > keep) {
    max_ind = (int)ceil(100 + pow(n - 100, curve)) + 1;
    *max_filtered_counts = (int)pow((double)(max_ind - 100), 1.0 / curve) + 100;
  } else {
    max_ind = n;
    *max_filtered_counts = max_ind;
  }
  int row = (int)(2 * ceil(cmax) - 1), half = (row - 1) / 2, ks = (half + 1) * (2 + half) / 2;
  double *c = (double *)calloc((size_t)max_ind * ks, sizeof(double));
  double *w = (double *)calloc((size_t)max_ind, sizeof(double));
  *max_filter_index = 0;
  for (int fl = 0; fl < max_ind; fl++) {
    double h, sum = 0.0;
    if (fl < keep) h = cmax / pow(fl + 1, curve);
    else h = cmax / pow(pow(fl - keep, 1.0 / curve) + keep + 1, curve);
    if (h <= cmin) {
      h = cmin;
      *max_filter_index = fl;
    }
    w[fl] = h;
    for (int a = -half; a <= half; a++)
      for (int b = -half; b <= half; b++) {
        double d = sqrt((double)(a * a + b * b)) / h;
        if (d <= 1.0) sum += kernel(0, support[0] * d);
      }
    int idx = fl * ks;
    for (int a = 0; a <= half; a++)
      for (int b = 0; b <= a; b++, idx++) {
        double d = sqrt((double)(a * a + b * b)) / h;
        c[idx] = d > 1.0 ? 0.0 : kernel(0, support[0] * d) / sum;
      }
    if (*max_filter_index > 0) break;
  }
  if (*max_filter_index == 0) *max_filter_index = max_ind - 1;
  *widths = w;
  *coefs = c;
  return ks;
}

/* filters.c:409-489 */
double f3g_temporal_filter(int n, int type, double fexp, double width, double **tfilter, double **tdeltas) {
  double *d = (double *)malloc((size_t)n * sizeof(double)), *f = (double *)malloc((size_t)n * sizeof(double));
  double maxf = 0.0, sumf = 0.0;
  *tdeltas = d;
  *tfilter = f;
  if (n == 1) {
    d[0] = 0;
    f[0] = 1.0;
    return 1.0;
  }
  for (int i = 0; i < n; i++) d[i] = ((double)i / (double)(n - 1) - 0.5) * width;
  if (type == 2) {
    for (int i = 0; i < n; i++) {
      double s = fexp >= 0 ? ((double)i + 1.0) / n : (double)(n - i) / n;
      f[i] = pow(s, fabs(fexp));
      if (f[i] > maxf) maxf = f[i];
    }
  } else if (type == 1) {
    double half = n / 2.0;
    for (int i = 0; i < n; i++) {
      f[i] = kernel(0, support[0] * fabs(i - half) / half);
      if (f[i] > maxf) maxf = f[i];
    }
  } else {
    for (int i = 0; i < n; i++) f[i] = 1.0;
    maxf = 1.0;
  }
  for (int i = 0; i < n; i++) {
    f[i] /= maxf;
    sumf += f[i];
  }
  return sumf / n;
}
