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

size_t flam3gpu_pass_bytes(void) { return sizeof(F3GPass); }

flam3gpu_options f3g_opts = {1, 32, 3, 256, 0, 0, 0, 0, 0, 0, 0, 0, {0}};

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
  if (o->shuffle_every < 0 || o->blocks < 0 || o->chain_samples < 0 || o->tail_chain_samples < -1 ||
      o->tail_wave_pct < 0 || o->tail_wave_pct > 1000) {
    f3g_set_error("negative option");
    return 1;
  }
  if (o->de_kernel != 0 && o->de_kernel != 1) {
    f3g_set_error("de_kernel must be 0 or 1");
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
  if (f3g_ensure_host_pass_one(c)) return 1;
  F3GPass *p = c->h_passes;
  memset(p, 0, sizeof(*p));
  if (cp->num_xforms - (cp->final_xform_index >= 0) > 0 && f3g_build_distrib(cp, p)) return 1;
  if (f3g_pack_genome(cp, p)) return 1;
  if (f3g_ensure((void **)&c->d_passes, &c->passes_bytes, sizeof(F3GPass))) return 1;
  *d_pass = c->d_passes;
  return 0;
}

int f3g_ensure_host_pass_one(f3g_ctx *c) {
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

int flam3gpu_chunk_plan(const long long *samples, int n, int threads, int blocks, int sub_batch_size, int *S,
                        int *S_tail, long long *chunk_tail, long long *nchunks) {
  f3g_clear_error();
  if (!samples || n < 1 || threads < 1 || blocks < 1 || !S || !S_tail || !chunk_tail || !nchunks) {
    f3g_set_error("bad arguments to flam3gpu_chunk_plan");
    return 1;
  }
  F3GPass *p = (F3GPass *)calloc((size_t)n, sizeof(F3GPass));
  if (!p) {
    f3g_set_error("host memory exhausted");
    return 1;
  }
  long long total = 0;
  for (int i = 0; i < n; i++) {
    p[i].samples = samples[i];
    total += samples[i];
  }
  *S = f3g_chunk_samples(NULL, total, threads, blocks, sub_batch_size);
  f3g_chunk_passes(p, n, threads, blocks, *S, NULL);
  *S_tail = p[0].S_tail;
  for (int i = 0; i < n; i++) {
    chunk_tail[i] = p[i].chunk_tail;
    nchunks[i] = p[i].nchunks;
  }
  free(p);
  return 0;
}

int flam3gpu_choice_breakpoints(const double *d, const double *c, int nstd, int nx, int walk, uint16_t *brk,
                                int *nbrk, int *moves) {
  f3g_clear_error();
  *nbrk = 0;
  if (moves) *moves = 0;
  return f3g_choice_breakpoints_host(d, c, nstd, nx, walk, brk, nbrk, moves);
}

int flam3gpu_xform_choice_table(flam3_genome *src, uint16_t *table, int *rows_out) {
  f3g_clear_error();
  f3g_ctx *c = f3g_get_ctx();
  if (!c) {
    f3g_set_error("no CUDA device available");
    return 1;
  }
  const int ns = src->num_xforms - (src->final_xform_index >= 0);
  if (ns < 1) {
    f3g_set_error("the genome has no standard xforms");
    return 1;
  }
  flam3_genome cp;
  F3GPass *d_pass = NULL;
  uint16_t *d_out = NULL;
  int rc = 1;
  if (prepare_single_pass(c, src, &d_pass, &cp)) goto out;
  const int rows = 1 + (c->h_passes->chaos_enable ? ns : 0);
  if (cudaMemcpy(d_pass, c->h_passes, sizeof(F3GPass), cudaMemcpyHostToDevice) != cudaSuccess) goto out;
  if (cudaMalloc((void **)&d_out, (size_t)rows * F3G_GRAIN * sizeof(uint16_t)) != cudaSuccess) goto out;
  if (f3g_launch_xform_choice(d_pass, rows, d_out, c->stream)) {
    f3g_set_error("xform choice launch failed");
    goto out;
  }
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) goto out;
  if (cudaMemcpy(table, d_out, (size_t)rows * F3G_GRAIN * sizeof(uint16_t), cudaMemcpyDeviceToHost) != cudaSuccess)
    goto out;
  if (rows_out) *rows_out = rows;
  rc = 0;
out:
  if (rc && !flam3gpu_last_error()[0]) f3g_set_error("CUDA error: %s", cudaGetErrorString(cudaGetLastError()));
  cudaFree(d_out);
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

/* flam3_dimension (flam3.h:592, flam3.c:3949-4052): the correlation
 * dimension from ntries attractor points (chains of 10000 samples after 20
 * fuse steps, optionally clipped to the camera) and ntries random pairs:
 * 0.434294 * log(n2 / (n1 - 0.5)), n2 / n1 counting pairs closer than
 * 0.004 / 0.00004 of the squared box diagonal.  The reference draws its
 * points from a private ISAAC context seeded with time(0) and the partners
 * from libc random(); here both come from the caller's rc, so the estimate
 * is reproducible.  Returns -1 on failure and NaN when clipping rejects
 * more than 10 * ntries points, as the reference does. */
double flam3gpu_dimension(flam3_genome *cp, int ntries, int clip_to_camera, randctx *rc) {
  f3g_clear_error();
  if (!rc) {
    f3g_set_error("flam3gpu_dimension needs an ISAAC context");
    return -1.0;
  }
  if (ntries < 2) ntries = 3000 * 1000;
  double bmin[2], bmax[2];
  if (clip_to_camera) {
    const double scale = pow(2.0, cp->zoom), ppux = cp->pixels_per_unit * scale;
    const double corner0 = cp->center[0] - cp->width / ppux / 2.0;
    const double corner1 = cp->center[1] - cp->height / ppux / 2.0;
    bmin[0] = corner0;
    bmin[1] = corner1;
    bmax[0] = corner0 + cp->width / ppux;
    bmax[1] = corner1 + cp->height / ppux;
  } else if (flam3gpu_estimate_bounding_box(cp, 0.0, 0, bmin, bmax, rc) < 0)
    return -1.0;
  const double d2max = (bmax[0] - bmin[0]) * (bmax[0] - bmin[0]) + (bmax[1] - bmin[1]) * (bmax[1] - bmin[1]);
  const int sbs = 10000, maxchains = 64;
  double *pts = (double *)malloc((size_t)ntries * 2 * sizeof(double));
  double *buf = (double *)malloc((size_t)maxchains * sbs * 4 * sizeof(double));
  double fd = -1.0;
  if (!pts || !buf) {
    f3g_set_error("host memory exhausted");
    goto out;
  }
  long got = 0, nclipped = 0;
  while (got < ntries) {
    long need = ntries - got;
    int nchains = (int)((need + sbs - 1) / sbs);
    if (nchains > maxchains) nchains = maxchains;
    long bv = 0;
    if (chains_from_rc(cp, nchains, sbs, rc, buf, &bv)) goto out;
    for (long i = 0; i < (long)nchains * sbs && got < ntries; i++) {
      const double x = buf[4 * i], y = buf[4 * i + 1];
      const int clipped = clip_to_camera && (x < bmin[0] || y < bmin[1] || x > bmax[0] || y > bmax[1]);
      if (!clipped) {
        pts[2 * got] = x;
        pts[2 * got + 1] = y;
        got++;
      } else if (++nclipped > 10L * ntries) {
        f3g_set_error("too much clipping, flam3gpu_dimension giving up");
        fd = sqrt(-1.0);
        goto out;
      }
    }
  }
  {
    long n1 = 0, n2 = 0;
    for (long i = 0; i < ntries; i++) {
      long k;
      /* the reference rejects the partner whose double index 2k equals i */
      do {
        k = (long)(f3g_irand(rc) % (unsigned long)ntries);
      } while (2 * k == i);
      const double dx = pts[2 * k] - pts[2 * i], dy = pts[2 * k + 1] - pts[2 * i + 1];
      const double d2 = dx * dx + dy * dy;
      if (d2 < 0.004 * d2max) n2++;
      if (d2 < 0.00004 * d2max) n1++;
    }
    fd = 0.434294 * log(n2 / (n1 - 0.5));
  }
out:
  free(pts);
  free(buf);
  return fd;
}

/* flam3_lyapunov (flam3.h:593, flam3.c:4054-4150): for each try a point is
 * brought onto the attractor (one sample after 20 + (0..9) fuse steps),
 * then one step is taken from it and one from a point eps = 1e-5 away in a
 * random direction, and log(distance / eps) is averaged; the result is
 * sum / (log 2 * ntries).  As in the reference the two steps draw their own
 * random numbers (its ISAAC context advances between them), so they may
 * pick different xforms.  All tries run as GPU chains in FP64; the draws
 * come from the caller's rc (the reference: a private ISAAC context seeded
 * with time(0), and libc random() for the fuse length). */
double flam3gpu_lyapunov(flam3_genome *cp, int ntries, randctx *rc) {
  f3g_clear_error();
  if (!rc) {
    f3g_set_error("flam3gpu_lyapunov needs an ISAAC context");
    return -1.0;
  }
  if (ntries < 1) ntries = 10000;
  const double eps = 1e-5;
  double *st = (double *)malloc((size_t)ntries * 4 * sizeof(double));
  double *on = (double *)malloc((size_t)ntries * 4 * sizeof(double));
  double *s1 = (double *)malloc((size_t)ntries * 4 * sizeof(double));
  double *s2 = (double *)malloc((size_t)ntries * 4 * sizeof(double));
  double *tmp = (double *)malloc((size_t)ntries * 4 * sizeof(double));
  int *fuse = (int *)malloc((size_t)ntries * sizeof(int));
  long *idx = (long *)malloc((size_t)ntries * sizeof(long));
  double res = -1.0;
  long bv = 0;
  if (!st || !on || !s1 || !s2 || !tmp || !fuse || !idx) {
    f3g_set_error("host memory exhausted");
    goto out;
  }
  for (int i = 0; i < ntries; i++) {
    st[4 * i] = isaac_11(rc);
    st[4 * i + 1] = isaac_11(rc);
    st[4 * i + 2] = 0.0;
    st[4 * i + 3] = 0.0;
    fuse[i] = 20 + (int)(f3g_irand(rc) % 10);
  }
  /* onto the attractor: one chain per try, grouped by fuse length */
  for (int f = 20; f < 30; f++) {
    long cnt = 0;
    for (int i = 0; i < ntries; i++)
      if (fuse[i] == f) {
        memcpy(tmp + 4 * cnt, st + 4 * i, 4 * sizeof(double));
        idx[cnt++] = i;
      }
    if (!cnt) continue;
    const uint64_t seed = (uint64_t)(uint32_t)f3g_irand(rc) | ((uint64_t)(uint32_t)f3g_irand(rc) << 32);
    if (flam3gpu_iterate_chains(cp, (int)cnt, 1, f, tmp, seed, s1, &bv, 64)) goto out;
    for (long c = 0; c < cnt; c++) memcpy(on + 4 * idx[c], s1 + 4 * c, 4 * sizeof(double));
  }
  /* one step from the point ... */
  {
    const uint64_t seed = (uint64_t)(uint32_t)f3g_irand(rc) | ((uint64_t)(uint32_t)f3g_irand(rc) << 32);
    if (flam3gpu_iterate_chains(cp, ntries, 1, 0, on, seed, s1, &bv, 64)) goto out;
  }
  /* ... and one from a point eps away (flam3.c:4127-4137) */
  for (int i = 0; i < ntries; i++) {
    double dx, dy, r;
    do {
      dx = isaac_11(rc);
      dy = isaac_11(rc);
      r = sqrt(dx * dx + dy * dy);
    } while (r == 0.0);
    tmp[4 * i] = on[4 * i] + dx / r * eps;
    tmp[4 * i + 1] = on[4 * i + 1] + dy / r * eps;
    tmp[4 * i + 2] = 0.0;
    tmp[4 * i + 3] = on[4 * i + 3];
  }
  {
    const uint64_t seed = (uint64_t)(uint32_t)f3g_irand(rc) | ((uint64_t)(uint32_t)f3g_irand(rc) << 32);
    if (flam3gpu_iterate_chains(cp, ntries, 1, 0, tmp, seed, s2, &bv, 64)) goto out;
  }
  {
    double sum = 0.0;
    for (int i = 0; i < ntries; i++) {
      const double ex = s1[4 * i] - s2[4 * i], ey = s1[4 * i + 1] - s2[4 * i + 1];
      sum += log(sqrt(ex * ex + ey * ey) / eps);
    }
    res = sum / (log(2.0) * ntries);
  }
out:
  free(st);
  free(on);
  free(s1);
  free(s2);
  free(tmp);
  free(fuse);
  free(idx);
  return res;
}


/* ---- strips (flam3-render.c:35-101, 311-345) ---- */

int flam3gpu_calc_nstrips(flam3_frame *f, double budget_bytes) {
  f3g_clear_error();
  if (!f || f->ngenomes < 1) {
    f3g_set_error("no genome");
    return -1;
  }
  double avail = budget_bytes;
  if (avail <= 0) {
    size_t fr = 0, tot = 0;
    if (!f3g_get_ctx() || cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
      f3g_set_error("no CUDA device available");
      return -1;
    }
    avail = 0.8 * (double)fr;
  }
  const double need = flam3gpu_render_memory_required(f);
  if (avail >= need) return 1;
  return (int)ceil(need / avail);
}

int flam3gpu_render_strips(flam3_frame *f, void *out, int nchan, int transp, stat_struct *stats, int nstrips) {
  f3g_clear_error();
  if (!f || f->ngenomes < 1 || !out) {
    f3g_set_error("no genome or output buffer");
    return 1;
  }
  if (nstrips < 1) nstrips = 1;
  const int real_height = f->genomes[0].height, width = f->genomes[0].width;
  if (nstrips > real_height) {
    f3g_set_error("cannot have more strips than rows but %d>%d", nstrips, real_height);
    return 1;
  }
  /* per-strip copies of the genomes: top-level fields only change */
  flam3_genome *orig = f->genomes;
  flam3_genome *g = (flam3_genome *)malloc((size_t)f->ngenomes * sizeof(flam3_genome));
  if (!g) {
    f3g_set_error("host memory exhausted");
    return 1;
  }
  const int strip_h = (int)ceil(real_height / (double)nstrips);
  double *center_base = (double *)malloc((size_t)f->ngenomes * sizeof(double));
  if (!center_base) {
    free(g);
    f3g_set_error("host memory exhausted");
    return 1;
  }
  for (int k = 0; k < f->ngenomes; k++) {
    const double zs = pow(2.0, orig[k].zoom);
    center_base[k] = orig[k].center[1] - ((nstrips - 1) * strip_h) / (2 * orig[k].pixels_per_unit * zs);
  }
  const size_t row = (size_t)nchan * width * (f->bytes_per_channel == 2 ? 2 : 1);
  randctx saved;
  memcpy(&saved, &f->rc, sizeof(randctx));
  stat_struct acc;
  memset(&acc, 0, sizeof(acc));
  int rv = 0;
  for (int strip = 0; strip < nstrips && !rv; strip++) {
    for (int k = 0; k < f->ngenomes; k++) {
      g[k] = orig[k];
      const double zs = pow(2.0, g[k].zoom);
      g[k].sample_density *= nstrips;
      g[k].height = strip_h;
      g[k].center[1] = center_base[k] + strip_h * (double)strip / (g[k].pixels_per_unit * zs);
      if (strip_h * (strip + 1) > real_height) {
        g[k].height = real_height - strip_h * strip;
        g[k].center[1] -= (strip_h - g[k].height) * 0.5 / (g[k].pixels_per_unit * zs);
      }
      g[k].ntemporal_samples = 1;
    }
    memcpy(&f->rc, &saved, sizeof(randctx));
    f->genomes = g;
    stat_struct st;
    memset(&st, 0, sizeof(st));
    rv = flam3gpu_render(f, (unsigned char *)out + (size_t)strip_h * strip * row, 0, nchan, transp, &st);
    f->genomes = orig;
    acc.num_iters += st.num_iters;
    acc.badvals += st.badvals;
    acc.render_seconds += st.render_seconds;
  }
  f->genomes = orig;
  free(g);
  free(center_base);
  if (stats) *stats = acc;
  return rv;
}

/* ---- ceiling probe for the iterate roofline ---- */

int flam3gpu_measure_atomic_rate(long long nbuckets, long long natomics, double *per_second) {
  f3g_clear_error();
  f3g_ctx *c = f3g_get_ctx();
  if (!c || nbuckets <= 0 || natomics <= 0 || !per_second) {
    f3g_set_error(c ? "bad arguments" : "no CUDA device available");
    return 1;
  }
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = (nsm > 0 ? nsm : 1) * 8;
  long long per = natomics / ((long long)blocks * 256);
  if (per < 1) per = 1;
  if (per > (1 << 30)) per = 1 << 30;
  float4 *buf = NULL;
  cudaEvent_t e0 = NULL, e1 = NULL;
  int rv = 1;
  if (cudaMalloc((void **)&buf, (size_t)nbuckets * sizeof(float4)) != cudaSuccess) goto out;
  if (cudaMemsetAsync(buf, 0, (size_t)nbuckets * sizeof(float4), c->stream) != cudaSuccess) goto out;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) goto out;
  /* one warm-up launch, then the timed one */
  if (f3g_launch_atomic_rate(buf, (unsigned long long)nbuckets, blocks, (int)(per / 8 + 1), 1u, c->stream)) goto out;
  cudaEventRecord(e0, c->stream);
  if (f3g_launch_atomic_rate(buf, (unsigned long long)nbuckets, blocks, (int)per, 2u, c->stream)) goto out;
  cudaEventRecord(e1, c->stream);
  if (cudaEventSynchronize(e1) != cudaSuccess) goto out;
  {
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    *per_second = (double)blocks * 256 * per / (ms / 1e3);
  }
  rv = 0;
out:
  if (rv && !flam3gpu_last_error()[0]) f3g_set_error("CUDA error: %s", cudaGetErrorString(cudaGetLastError()));
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(buf);
  return rv;
}
