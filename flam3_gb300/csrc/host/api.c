/*
 * api.c -- error reporting, options, version, and the kernel-level entry
 * points of libflam3gpu (apply_xform, point accumulation, recorded chains).
 */
#define _GNU_SOURCE
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "f3g_host.h"

static __thread char err_buf[512];

void f3g_set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(err_buf, sizeof(err_buf), fmt, ap);
  va_end(ap);
}

void f3g_clear_error(void) { err_buf[0] = 0; }

const char *flam3gpu_last_error(void) { return err_buf; }

const char *flam3gpu_version(void) { return "flam3-gb300 0.1 (sm_103a)"; }

flam3gpu_options f3g_opts = {1, 32, 3, 256, 0, 0, 0, 0, {0}};

void flam3gpu_default_options(flam3gpu_options *o) {
  memset(o, 0, sizeof(*o));
  o->iter_mode = 1;
  o->iter_precision = 32;
  o->shuffle_every = 3;
  o->threads_per_block = 256;
}

int flam3gpu_set_options(const flam3gpu_options *o) {
  if (o->iter_mode != 0 && o->iter_mode != 1) {
    f3g_set_error("iter_mode must be 0 or 1");
    return 1;
  }
  if (o->iter_precision != 32 && o->iter_precision != 64) {
    f3g_set_error("iter_precision must be 32 or 64");
    return 1;
  }
  int t = o->threads_per_block;
  if (t != 0 && (t < 32 || t > 256 || (t & (t - 1)))) {
    f3g_set_error("threads_per_block must be a power of two in [32, 256]");
    return 1;
  }
  if (o->shuffle_every < 0 || o->blocks < 0 || o->chain_samples < 0) {
    f3g_set_error("negative option");
    return 1;
  }
  if (o->de_tile != 0 && (o->de_tile < 4 || o->de_tile > 64)) {
    f3g_set_error("de_tile must be 0 or in [4, 64]");
    return 1;
  }
  f3g_opts = *o;
  return 0;
}

void flam3gpu_get_options(flam3gpu_options *o) { *o = f3g_opts; }

/* Prepare genome cp (a copy) into a single pass in device memory. */
static int prepare_single_pass(f3g_ctx *c, flam3_genome *src, F3GPass **d_pass, flam3_genome *cp) {
  memset(cp, 0, sizeof(*cp));
  f3g_genome_copy(cp, src);
  if (f3g_prepare_precalc_flags(cp)) return 1;
  for (int i = 0; i < cp->num_xforms; i++) f3g_xform_precalc(cp, i);
  if (ensure_host_pass_one(c)) return 1;
  F3GPass *p = c->h_passes;
  memset(p, 0, sizeof(*p));
  if (cp->num_xforms - (cp->final_xform_index >= 0) > 0 && f3g_build_distrib(cp, p)) return 1;
  if (f3g_pack_genome(cp, p)) return 1;
  if (f3g_ensure((void **)&c->d_passes, &c->passes_bytes, sizeof(F3GPass))) return 1;
  *d_pass = c->d_passes;
  return 0;
}

int ensure_host_pass_one(f3g_ctx *c) {
  if (c->h_passes && c->h_passes_bytes >= sizeof(F3GPass)) return 0;
  if (c->h_passes) cudaFreeHost(c->h_passes);
  c->h_passes = NULL;
  if (cudaMallocHost((void **)&c->h_passes, sizeof(F3GPass)) != cudaSuccess) {
    f3g_set_error("cudaMallocHost failed");
    return 1;
  }
  c->h_passes_bytes = sizeof(F3GPass);
  return 0;
}

int flam3gpu_apply_xform(flam3_genome *src, int fn, int n, const double *p_in, const uint32_t *words, int wpp,
                         double *q_out, int *bad_out, int precision) {
  f3g_clear_error();
  f3g_ctx *c = f3g_get_ctx();
  if (!c) {
    f3g_set_error("no CUDA device available");
    return 1;
  }
  if (fn < 0 || fn >= src->num_xforms || n < 0 || wpp < 0) {
    f3g_set_error("bad xform index or sizes");
    return 1;
  }
  flam3_genome cp;
  F3GPass *d_pass = NULL;
  int rc = 1;
  double *d_pin = NULL, *d_q = NULL;
  uint32_t *d_w = NULL;
  int *d_bad = NULL;
  /* the copy moves the final xform last; translate the index */
  int ns = src->num_xforms - (src->final_xform_index >= 0);
  int fnc = fn;
  if (src->final_xform_index >= 0) {
    if (fn == src->final_xform_index) fnc = ns;
    else if (fn > src->final_xform_index) fnc = fn - 1;
  }
  if (prepare_single_pass(c, src, &d_pass, &cp)) goto out;
  if (cudaMemcpy(d_pass, c->h_passes, sizeof(F3GPass), cudaMemcpyHostToDevice) != cudaSuccess) goto out;
  if (n == 0) {
    rc = 0;
    goto out;
  }
  if (cudaMalloc((void **)&d_pin, (size_t)n * 4 * sizeof(double)) != cudaSuccess) goto out;
  if (cudaMalloc((void **)&d_q, (size_t)n * 4 * sizeof(double)) != cudaSuccess) goto out;
  if (cudaMalloc((void **)&d_w, (size_t)n * (wpp > 0 ? wpp : 1) * sizeof(uint32_t)) != cudaSuccess) goto out;
  if (cudaMalloc((void **)&d_bad, (size_t)n * sizeof(int)) != cudaSuccess) goto out;
  cudaMemcpy(d_pin, p_in, (size_t)n * 4 * sizeof(double), cudaMemcpyHostToDevice);
  if (wpp > 0) cudaMemcpy(d_w, words, (size_t)n * wpp * sizeof(uint32_t), cudaMemcpyHostToDevice);
  if (f3g_launch_apply_xform(d_pass, fnc, n, d_pin, d_w, wpp, d_q, d_bad, precision == 64 ? 64 : 32, c->stream)) {
    f3g_set_error("apply_xform launch failed");
    goto out;
  }
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) goto out;
  cudaMemcpy(q_out, d_q, (size_t)n * 4 * sizeof(double), cudaMemcpyDeviceToHost);
  if (bad_out) cudaMemcpy(bad_out, d_bad, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost);
  rc = 0;
out:
  if (rc && !flam3gpu_last_error()[0]) f3g_set_error("CUDA error: %s", cudaGetErrorString(cudaGetLastError()));
  cudaFree(d_pin);
  cudaFree(d_q);
  cudaFree(d_w);
  cudaFree(d_bad);
  f3g_genome_free(&cp);
  return rc;
}

int flam3gpu_iterate_chains(flam3_genome *src, int nchains, int n, int fuse, const double *starts, uint64_t seed,
                            double *samples, long *badvals, int precision) {
  f3g_clear_error();
  f3g_ctx *c = f3g_get_ctx();
  if (!c) {
    f3g_set_error("no CUDA device available");
    return 1;
  }
  if (nchains < 0 || n < 0 || fuse < 0) {
    f3g_set_error("negative sizes");
    return 1;
  }
  flam3_genome cp;
  F3GPass *d_pass = NULL;
  double *d_s = NULL, *d_out = NULL;
  unsigned long long *d_bad = NULL, hbad = 0;
  int rc = 1;
  if (prepare_single_pass(c, src, &d_pass, &cp)) goto out;
  if (cudaMemcpy(d_pass, c->h_passes, sizeof(F3GPass), cudaMemcpyHostToDevice) != cudaSuccess) goto out;
  if (cudaMalloc((void **)&d_s, (size_t)(nchains > 0 ? nchains : 1) * 4 * sizeof(double)) != cudaSuccess) goto out;
  if (cudaMalloc((void **)&d_out, (size_t)(nchains > 0 ? nchains : 1) * (n > 0 ? n : 1) * 4 * sizeof(double)) !=
      cudaSuccess)
    goto out;
  if (cudaMalloc((void **)&d_bad, sizeof(unsigned long long)) != cudaSuccess) goto out;
  cudaMemset(d_bad, 0, sizeof(unsigned long long));
  cudaMemcpy(d_s, starts, (size_t)nchains * 4 * sizeof(double), cudaMemcpyHostToDevice);
  if (nchains > 0 &&
      f3g_launch_iterate_chains(d_pass, nchains, n, fuse, d_s, (uint32_t)seed, (uint32_t)(seed >> 32), d_out, d_bad,
                                precision == 64 ? 64 : 32, c->stream)) {
    f3g_set_error("iterate_chains launch failed");
    goto out;
  }
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) goto out;
  cudaMemcpy(samples, d_out, (size_t)nchains * n * 4 * sizeof(double), cudaMemcpyDeviceToHost);
  cudaMemcpy(&hbad, d_bad, sizeof(hbad), cudaMemcpyDeviceToHost);
  if (badvals) *badvals = (long)hbad;
  rc = 0;
out:
  if (rc && !flam3gpu_last_error()[0]) f3g_set_error("CUDA error: %s", cudaGetErrorString(cudaGetLastError()));
  cudaFree(d_s);
  cudaFree(d_out);
  cudaFree(d_bad);
  f3g_genome_free(&cp);
  return rc;
}

int f3g_accumulate_impl(flam3_frame *f, int field, const double *points, long n, double *hist, int *hist_w,
                        int *hist_h);

int flam3gpu_accumulate_points(flam3_frame *f, int field, const double *points, long n, double *hist, int *hist_w,
                               int *hist_h) {
  f3g_clear_error();
  return f3g_accumulate_impl(f, field, points, n, hist, hist_w, hist_h);
}

/* ---- callers of flam3_iterate (flam3.c:351-391, 3574-3640) on the GPU ----
 * Both draw their chains from the chain kernel (FP32 iteration, fuse 20 as
 * the reference); the start points and the Philox key come from the
 * caller's ISAAC context, which advances by 2 words per chain plus 2. */

/* flam3_random_isaac_11 (flam3.c:2523-2525) */
static double isaac_11(randctx *rc) { return (((int)f3g_irand(rc) & 0xfffffff) - 0x7ffffff) / (double)0x7ffffff; }

static int chains_from_rc(flam3_genome *cp, int nchains, int n, randctx *rc, double *samples, long *bad) {
  double *starts = (double *)malloc((size_t)(nchains > 0 ? nchains : 1) * 4 * sizeof(double));
  if (!starts) {
    f3g_set_error("host memory exhausted");
    return 1;
  }
  for (int c = 0; c < nchains; c++) {
    starts[4 * c] = isaac_11(rc);
    starts[4 * c + 1] = isaac_11(rc);
    starts[4 * c + 2] = 0.0;
    starts[4 * c + 3] = 0.0;
  }
  const uint64_t seed = (uint64_t)(uint32_t)f3g_irand(rc) | ((uint64_t)(uint32_t)f3g_irand(rc) << 32);
  int r = flam3gpu_iterate_chains(cp, nchains, n, 20, starts, seed, samples, bad, 32);
  free(starts);
  return r;
}

/* k-th smallest of v[0..n) (Hoare's selection), v reordered */
static double select_kth(double *v, long n, long k) {
  long lo = 0, hi = n - 1;
  while (lo < hi) {
    const double piv = v[lo + (hi - lo) / 2];
    long i = lo, j = hi;
    while (i <= j) {
      while (v[i] < piv) i++;
      while (v[j] > piv) j--;
      if (i <= j) {
        const double t = v[i];
        v[i] = v[j];
        v[j] = t;
        i++;
        j--;
      }
    }
    if (k <= j) hi = j;
    else if (k >= i) lo = i;
    else return v[k];
  }
  return v[k];
}

int flam3gpu_estimate_bounding_box(flam3_genome *cp, double eps, int nsamples, double *bmin, double *bmax,
                                   randctx *rc) {
  f3g_clear_error();
  if (nsamples <= 0) nsamples = 10000;
  const int per = 1024;
  const int nchains = (nsamples + per - 1) / per;
  const int n = (nsamples + nchains - 1) / nchains;
  const long total = (long)nchains * n;
  double *pts = (double *)malloc((size_t)total * 4 * sizeof(double));
  double *axis = (double *)malloc((size_t)total * sizeof(double));
  long bv = 0;
  int ret = -1;
  if (!pts || !axis) {
    f3g_set_error("host memory exhausted");
    goto out;
  }
  if (chains_from_rc(cp, nchains, n, rc, pts, &bv)) goto out;
  /* flam3.c:3601-3639 */
  if (bv / (double)total > eps) eps = 3 * bv / (double)total;
  if (eps > 0.3) eps = 0.3;
  const long low = (long)(total * eps), high = total - low;
  for (int d = 0; d < 2; d++) {
    if (low == 0) {
      double mn = 1e10, mx = -1e10;
      for (long i = 0; i < total; i++) {
        const double x = pts[4 * i + d];
        if (x < mn) mn = x;
        if (x > mx) mx = x;
      }
      bmin[d] = mn;
      bmax[d] = mx;
    } else {
      for (long i = 0; i < total; i++) axis[i] = pts[4 * i + d];
      bmin[d] = select_kth(axis, total, low);
      bmax[d] = select_kth(axis, total, high);
    }
  }
  ret = (int)bv;
out:
  free(pts);
  free(axis);
  return ret;
}

int flam3gpu_colorhist(flam3_genome *cp, int num_batches, randctx *rc, double *hist) {
  f3g_clear_error();
  const int sbs = 10000;
  memset(hist, 0, 256 * sizeof(double));
  if (num_batches <= 0) return 0;
  double *pts = (double *)malloc((size_t)num_batches * sbs * 4 * sizeof(double));
  if (!pts) {
    f3g_set_error("host memory exhausted");
    return 1;
  }
  long bv = 0;
  if (chains_from_rc(cp, num_batches, sbs, rc, pts, &bv)) {
    free(pts);
    return 1;
  }
  const long total = (long)num_batches * sbs;
  for (long i = 0; i < total; i++) {
    int c = (int)(pts[4 * i + 2] * 256);
    if (c < 0) c = 0;
    if (c > 255) c = 255;
    hist[c] += 1;
  }
  for (int k = 0; k < 256; k++) hist[k] /= (float)total;
  free(pts);
  return 0;
}

