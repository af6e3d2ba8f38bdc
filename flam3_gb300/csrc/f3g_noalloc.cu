/*
 * f3g_noalloc.cu -- flam3gpu_render_noalloc: a render that allocates no
 * device memory.
 *
 * Some callers cannot call cudaMalloc: plug-in hosts whose memory pool owns
 * every device allocation of the process, and services that fix their
 * device-memory budget at start-up and must not grow it per request.  This
 * entry point takes all of its device scratch -- the histogram (and its
 * count plane), the pass tables, the work counters, the filter tables and the
 * staged output image -- from one file-scope static __device__ array of
 * F3G_NOALLOC_BYTES, which the CUDA loader reserves on every device that
 * loads the library and keeps until the process exits.  It calls no
 * cudaMalloc, cudaFree, cudaMallocHost or other allocating CUDA routine.  Its
 * copies are blocking cudaMemcpy calls on the legacy default stream, and it
 * reads the work counters back to the host between the iteration and the
 * tail, so the call returns only when the image is in the caller's buffer.
 *
 * Each call looks up the array's address on the current device with
 * cudaGetSymbolAddress.
 *
 * Limits: one batch (nbatches == 1), and the render's scratch must fit the
 * array; larger requests are refused with an error naming both sizes.
 * Every call shares the array and leaves its contents behind: the histogram
 * is cleared at the start of each call.  Calls that overlap on the GPU (from
 * several host threads at once) race on the array.
 */
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "f3g_launch.h"
#include "host/f3g_host.h"

/* 48 MiB: a 1.5 M-bucket FP32 histogram (about 1200 x 1200 buckets including
 * the gutter) with its tables and image, or half that many FP64 buckets. */
#define F3G_NOALLOC_BYTES (48u << 20)

static __device__ __align__(256) unsigned char f3g_noalloc_scratch[F3G_NOALLOC_BYTES];

/* The array's device address on the current device, looked up on every
 * call (the lookup is cheap, and a reset device may place the array
 * elsewhere).  In host code `f3g_noalloc_scratch` names a host-side
 * stand-in, not device memory, so only this address is ever passed to
 * kernels. */
static int scratch_address(unsigned char **out) {
  void *p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, f3g_noalloc_scratch);
  if (e != cudaSuccess || !p) {
    f3g_set_error("cudaGetSymbolAddress of the scratch array failed: %s", cudaGetErrorString(e));
    return 1;
  }
  *out = (unsigned char *)p;
  return 0;
}

/* bump allocation inside the scratch array */
struct Carve {
  unsigned char *base;
  size_t used;
  void *take(size_t n) {
    void *p = base ? base + used : nullptr;
    used += (n + 255) & ~(size_t)255;
    return p;
  }
};

extern "C" size_t flam3gpu_noalloc_capacity(void) { return F3G_NOALLOC_BYTES; }

#define NCK(call)                                                                           \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess) {                                                                \
      f3g_set_error("CUDA error %s at %s:%d", cudaGetErrorString(e_), __FILE__, __LINE__); \
      goto done;                                                                            \
    }                                                                                       \
  } while (0)

extern "C" int flam3gpu_render_noalloc(flam3_frame *spec, void *out, int field, int nchan, int transp,
                                       stat_struct *stats) {
  f3g_clear_error();
  int rv = 1;
  double *filter = nullptr, *tfilter = nullptr, *tdeltas = nullptr, *de_w = nullptr, *de_c = nullptr;
  float *fbuf = nullptr;
  F3GPass *passes = nullptr;
  long long *prefix = nullptr;
  F3GItem *items = nullptr;
  flam3_genome cp;
  memset(&cp, 0, sizeof(cp));
  unsigned char *scratch = nullptr;
  const int bits = spec->bits;
  f3g_geom g;
  memset(&g, 0, sizeof(g));
  stats->num_iters = 0;
  stats->badvals = 0;
  if (bits != 32 && bits != 33 && bits != 64) {
    f3g_set_error("flam3: bits must be 32, 33, or 64 not %d.", bits);
    return 1;
  }
  if (nchan != 3 && nchan != 4) {
    f3g_set_error("nchan must be 3 or 4, not %d", nchan);
    return 1;
  }
  if (scratch_address(&scratch)) return 1;
  const char *ap = getenv("apo_palette");
  const int cmap_size = 256 - (ap ? atoi(ap) : 0);
  if (cmap_size < 2 || cmap_size > 256) {
    f3g_set_error("apo_palette gives a colour map of %d entries", cmap_size);
    return 1;
  }
  if (f3g_interpolate(spec->genomes, spec->ngenomes, spec->time, &cp)) return 1;
  {
    const int nbatches = cp.nbatches, ntemporal = cp.ntemporal_samples;
    const double highpow = cp.highlight_power;
    if (nbatches != 1) {
      f3g_set_error("the no-allocation render takes one batch, not %d", nbatches);
      goto done;
    }
    if (cp.spatial_oversample < 1 || ntemporal < 1) {
      f3g_set_error("oversample and temporal samples must be positive");
      goto done;
    }
    if (f3g_geometry(spec, &cp, field, &filter, &g)) goto done;
    const double sumfilt = f3g_temporal_filter(ntemporal, cp.temporal_filter_type, cp.temporal_filter_exp,
                                               cp.temporal_filter_width, &tfilter, &tdeltas);
    const long long nb = (long long)g.W * g.H;
    const int bkind = bits == 64 ? F3G_BK_F64 : F3G_BK_F32;
    const size_t bsz = bkind == F3G_BK_F64 ? 32 : 16, csz = bkind == F3G_BK_F64 ? 8 : 4;
    /* density-estimation tables (rect.c:735-751) */
    int mfc = 0, mfi = 0, ks = 0, R = 0;
    if (f3g_interpolate(spec->genomes, spec->ngenomes, spec->time + tdeltas[0], &cp)) goto done;
    if (cp.estimator < 0.0 || cp.estimator_minimum < 0.0) {
      f3g_set_error("density estimator filter widths must be >= 0");
      goto done;
    }
    if (bits <= 32 && cp.estimator > 0.0) {
      fprintf(stderr, "warning: density estimation disabled with %d bit buffers.\n", bits);
      cp.estimator = 0.0;
    }
    if (cp.estimator > 0.0) {
      ks = f3g_de_filters(cp.estimator, cp.estimator_minimum, cp.estimator_curve, g.oversample, &mfc, &mfi, &de_w,
                          &de_c);
      if (ks < 0) goto done;
      R = (int)ceil(de_w[0]) - 1;
      if (mfi > 0 && f3g_de_fused_smem(g.oversample, g.filter_width, R, mfi + 1) > 220 * 1024) {
        f3g_set_error("density estimation radius %d is beyond the no-allocation render", R);
        goto done;
      }
    }
    const int de_on = mfi > 0;
    int need_count = 0;
    for (int i = 0; i < ntemporal; i++)
      if (tfilter[i] != 1.0) need_count = 1;
    /* carve the scratch array; the first pass only measures */
    const size_t out_bytes = (size_t)g.image_width * g.image_height * nchan * spec->bytes_per_channel;
    Carve cv{nullptr, 0};
    for (int pass = 0; pass < 2; pass++) {
      cv.base = pass ? scratch : nullptr;
      cv.used = 0;
      cv.take((size_t)ntemporal * sizeof(F3GPass));
      cv.take((size_t)(ntemporal + 1) * sizeof(long long));
      cv.take((size_t)ntemporal * sizeof(F3GItem));
      cv.take(sizeof(F3GCounters));
      cv.take(F3G_FILTER_FLOATS(g.filter_width) * sizeof(float));
      cv.take(de_on ? (size_t)(mfi + 1) * 4 * sizeof(float) : 0);
      cv.take((size_t)nb * bsz);
      cv.take(de_on ? (size_t)nb * csz : 0);
      cv.take(out_bytes);
      if (cv.used > F3G_NOALLOC_BYTES) {
        f3g_set_error("render needs %zu bytes of device scratch; flam3gpu_render_noalloc holds at most %u",
                      cv.used, F3G_NOALLOC_BYTES);
        goto done;
      }
    }
    cv.base = scratch;
    cv.used = 0;
    F3GPass *d_passes = (F3GPass *)cv.take((size_t)ntemporal * sizeof(F3GPass));
    long long *d_prefix = (long long *)cv.take((size_t)(ntemporal + 1) * sizeof(long long));
    F3GItem *d_items = (F3GItem *)cv.take((size_t)ntemporal * sizeof(F3GItem));
    F3GCounters *d_ctr = (F3GCounters *)cv.take(sizeof(F3GCounters));
    float *d_filter = (float *)cv.take(F3G_FILTER_FLOATS(g.filter_width) * sizeof(float));
    float *d_de = (float *)cv.take(de_on ? (size_t)(mfi + 1) * 4 * sizeof(float) : 0);
    void *d_hist = cv.take((size_t)nb * bsz);
    void *d_count = cv.take(de_on ? (size_t)nb * csz : 0);
    unsigned char *d_out = (unsigned char *)cv.take(out_bytes);

    /* host tables (host memory only) */
    passes = (F3GPass *)malloc((size_t)ntemporal * sizeof(F3GPass));
    prefix = (long long *)malloc((size_t)(ntemporal + 1) * sizeof(long long));
    items = (F3GItem *)malloc((size_t)ntemporal * sizeof(F3GItem));
    const size_t nf = F3G_FILTER_FLOATS(g.filter_width) + (de_on ? (size_t)(mfi + 1) * 4 : 0);
    fbuf = (float *)malloc(nf * sizeof(float));
    if (!passes || !prefix || !items || !fbuf) {
      f3g_set_error("host memory exhausted");
      goto done;
    }
    double vibrancy = 0, gamma = 0, background[3] = {0, 0, 0}, ppux = 0, ppuy = 0, sample_density = 0;
    long long batch_samples = 0;
    int full = 0, mode = 1;
    for (int ts = 0; ts < ntemporal; ts++) {
      const double color_scalar = tfilter[ts];
      F3GPass *p = &passes[ts];
      memset(p, 0, sizeof(F3GPass));
      if (f3g_interpolate(spec->genomes, spec->ngenomes, spec->time + tdeltas[ts], &cp)) goto done;
      if (f3g_prepare_precalc_flags(&cp) || f3g_build_distrib(&cp, p)) goto done;
      for (int i = 0; i < cp.num_xforms; i++) f3g_xform_precalc(&cp, i);
      if (f3g_pack_genome(&cp, p)) goto done;
      for (int j = 0; j < 256; j++) {
        for (int k = 0; k < 4; k++) p->dmap[j][k] = (float)((cp.palette[j].color[k] * 255.0) * color_scalar);
        if (cp.palette[j].color[3] != 1.0) need_count = 1;
      }
      p->cmap_size = cmap_size;
      p->palette_mode = cp.palette_mode;
      if (f3g_camera(spec, &cp, field, &g, p, &sample_density, &ppux, &ppuy)) goto done;
      const double batch_size = sample_density * g.image_width * g.image_height / ntemporal;
      stats->num_iters += batch_size;
      p->samples = (long long)batch_size;
      p->fuse = spec->earlyclip ? 100 : 15;
      p->iter_mode = f3g_choice_mode(cp.chaos_enable);
      p->bucket_kind = bkind;
      p->trunc_hits = bits <= 33 && !f3g_opts.float_buckets;
      p->buckets = d_hist;
      f3g_pass_key(spec, p->key);
      batch_samples += p->samples;
      full |= p->full_variations;
      if (p->iter_mode == 0) mode = 0;
      vibrancy += cp.vibrancy;
      gamma += cp.gamma;
      for (int k = 0; k < 3; k++) background[k] += cp.background[k];
    }
    const int use_count = de_on && need_count;
    const int threads = f3g_opts.threads_per_block > 0 ? f3g_opts.threads_per_block : 256;
    const int precision = f3g_opts.iter_precision == 64 ? 64 : 32;
    int nsm = 0, dev = 0;
    NCK(cudaGetDevice(&dev));
    NCK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    int occ = f3g_iterate_occupancy(precision, full, mode, threads);
    if (occ < 1) occ = 1;
    const int blocks = f3g_opts.blocks > 0 ? f3g_opts.blocks : nsm * occ;
    const int S = f3g_chunk_samples(nullptr, batch_samples, threads, blocks, spec->sub_batch_size);
    const long long total_chunks = f3g_chunk_passes(passes, ntemporal, threads, blocks, S, prefix);
    for (int ts = 0; ts < ntemporal; ts++) {
      passes[ts].count = use_count ? d_count : nullptr;
      passes[ts].counters = &d_ctr->badvals;
      items[ts].pass = d_passes + ts;
      items[ts].chunk_first = 0;
    }
    for (size_t i = 0; i < F3G_FILTER_FLOATS(g.filter_width); i++) fbuf[i] = (float)filter[i];
    if (de_on) {
      f3g_de_kernel_info(mfi, ks, de_w, de_c, fbuf + F3G_FILTER_FLOATS(g.filter_width));
    }
    F3GCounters ctr;
    memset(&ctr, 0, sizeof(ctr));
    /* the array keeps the last call's contents: clear what must start at zero */
    NCK(cudaMemsetAsync(d_hist, 0, (size_t)nb * bsz, 0));
    if (use_count) NCK(cudaMemsetAsync(d_count, 0, (size_t)nb * csz, 0));
    NCK(cudaMemcpy(d_passes, passes, (size_t)ntemporal * sizeof(F3GPass), cudaMemcpyHostToDevice));
    NCK(cudaMemcpy(d_prefix, prefix, (size_t)(ntemporal + 1) * sizeof(long long), cudaMemcpyHostToDevice));
    NCK(cudaMemcpy(d_items, items, (size_t)ntemporal * sizeof(F3GItem), cudaMemcpyHostToDevice));
    NCK(cudaMemcpy(d_ctr, &ctr, sizeof(ctr), cudaMemcpyHostToDevice));
    NCK(cudaMemcpy(d_filter, fbuf, F3G_FILTER_FLOATS(g.filter_width) * sizeof(float), cudaMemcpyHostToDevice));
    if (de_on)
      NCK(cudaMemcpy(d_de, fbuf + F3G_FILTER_FLOATS(g.filter_width),
                     (size_t)(mfi + 1) * 4 * sizeof(float), cudaMemcpyHostToDevice));
    const int shuffle = f3g_opts.shuffle_every > 0 ? f3g_opts.shuffle_every : 1;
    int e = f3g_launch_iterate(d_items, d_prefix, ntemporal, total_chunks, shuffle, precision, full, mode, threads,
                               blocks, d_ctr, 0);
    if (e) {
      f3g_set_error("iterate launch failed: %s", cudaGetErrorString((cudaError_t)e));
      goto done;
    }
    NCK(cudaMemcpy(&ctr, d_ctr, sizeof(ctr), cudaMemcpyDeviceToHost));
    if (ctr.error) {
      f3g_set_error("iterate kernel: a point-exchange wait timed out");
      goto done;
    }
    stats->badvals = (double)ctr.badvals;
    const double k1 = (cp.contrast * cp.brightness * 255.0 * 268.0) / 256;
    const double area = g.image_width * g.image_height / (ppux * ppuy);
    const double k2 = (g.oversample * g.oversample) / (cp.contrast * area * 255.0 * sample_density * sumfilt);
    F3GTonemap tp;
    const double gm = 1.0 / (gamma / ntemporal);
    tp.g = (float)gm;
    tp.linrange = (float)cp.gam_lin_thresh;
    tp.funcval = (float)pow(cp.gam_lin_thresh, gm);
    tp.vibrancy = (float)(vibrancy / ntemporal);
    tp.highpow = (float)highpow;
    for (int k = 0; k < 3; k++) tp.background[k] = (float)(background[k] / (ntemporal / 256.0));
    tp.nchan = nchan;
    tp.transp = transp;
    tp.bpc = spec->bytes_per_channel;
    tp.trunc_acc = bits == 32 && !f3g_opts.float_buckets;
    if (de_on)
      e = f3g_launch_de_fused(d_hist, bkind, use_count ? d_count : nullptr, g.W, g.H, g.oversample, k1, k2,
                              cp.estimator_curve, mfc, mfi, d_de, R, g.de_offset, d_filter,
                              g.filter_width, g.image_width, g.image_height, d_out, spec->earlyclip, &tp, 0);
    else
      e = f3g_launch_fused_log_filter(d_hist, bkind, g.W, g.H, k1, k2, g.de_offset, g.oversample, d_filter,
                                      g.filter_width, g.image_width, g.image_height, d_out, spec->earlyclip, &tp, 0);
    if (e) {
      f3g_set_error("tail launch failed: %s", cudaGetErrorString((cudaError_t)e));
      goto done;
    }
    const size_t row = (size_t)g.image_width * nchan * spec->bytes_per_channel;
    unsigned char *dst = (unsigned char *)out + (field == flam3_field_odd ? row : 0);
    NCK(cudaMemcpy2D(dst, (size_t)g.out_width * nchan * spec->bytes_per_channel, d_out, row, row,
                     (size_t)g.image_height, cudaMemcpyDeviceToHost));
    rv = 0;
  }
done:
  free(filter);
  free(tfilter);
  free(tdeltas);
  free(de_w);
  free(de_c);
  free(fbuf);
  free(passes);
  free(prefix);
  free(items);
  f3g_genome_free(&cp);
  stats->render_seconds = 0;
  if (rv) fprintf(stderr, "flam3gpu: %s\n", flam3gpu_last_error());
  return rv;
}
