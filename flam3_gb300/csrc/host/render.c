/*
 * render.c -- flam3gpu_render: the GPU body of flam3_render.
 *
 * Follows render_rectangle (rect.c:529-1286) step for step on the host --
 * interpolation, filters, gutter, batches, temporal samples, camera, k1/k2,
 * tonemap constants, consumption of the caller's ISAAC context -- and runs
 * the per-pixel and per-sample work as kernels:
 *
 *   iterate (all temporal samples of a batch in one persistent launch)
 *   -> [one batch, no DE]  fused log-scale + filter + tonemap + pack
 *   -> [otherwise]         log-scale or DE into the accumulator per batch,
 *                          then earlyclip / filter + tonemap + pack
 *
 * Device buffers live in a per-thread context and are reused across calls.
 */
#define _GNU_SOURCE
#include <math.h>
#include <pthread.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>

#include "f3g_host.h"

#define F3G_WHITE 255.0

static __thread f3g_ctx tls_ctx;

/* CUDA call inside flam3gpu_render_ex: record the error and leave through `done` */
#define CK(call)                                                                           \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) {                                                               \
      f3g_set_error("CUDA error %s at %s:%d", cudaGetErrorString(e_), __FILE__, __LINE__); \
      goto done;                                                                           \
    }                                                                                      \
  } while (0)

f3g_ctx *f3g_get_ctx(void) {
  f3g_ctx *c = &tls_ctx;
  if (!c->ready) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return NULL;
    c->device = dev;
    if (cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return NULL;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) return NULL;
    for (int i = 0; i < 8; i++)
      if (cudaEventCreate(&c->ev[i]) != cudaSuccess) return NULL;
    if (cudaMalloc((void **)&c->d_ctr, sizeof(F3GCounters)) != cudaSuccess) return NULL;
    if (cudaMallocHost((void **)&c->h_ctr, sizeof(F3GCounters)) != cudaSuccess) return NULL;
    c->ready = 1;
  }
  return c;
}

int f3g_ensure(void **ptr, size_t *cap, size_t need) {
  if (need <= *cap && *ptr) return 0;
  if (*ptr) cudaFree(*ptr);
  *ptr = NULL;
  *cap = 0;
  size_t alloc = need < 256 ? 256 : need;
  cudaError_t e = cudaMalloc(ptr, alloc);
  if (e != cudaSuccess) {
    f3g_set_error("cudaMalloc of %zu bytes failed: %s", alloc, cudaGetErrorString(e));
    *ptr = NULL;
    return 1;
  }
  *cap = alloc;
  return 0;
}

static int ensure_host_passes(f3g_ctx *c, size_t n) {
  size_t need = n * sizeof(F3GPass);
  if (!(need <= c->h_passes_bytes && c->h_passes)) {
    if (c->h_passes) cudaFreeHost(c->h_passes);
    c->h_passes = NULL;
    c->h_passes_bytes = 0;
    if (cudaMallocHost((void **)&c->h_passes, need) != cudaSuccess) {
      f3g_set_error("cudaMallocHost of %zu bytes failed", need);
      return 1;
    }
    c->h_passes_bytes = need;
  }
  if (!(c->h_prefix && c->prefix_n >= n + 1)) {
    if (c->h_prefix) cudaFreeHost(c->h_prefix);
    c->h_prefix = NULL;
    c->prefix_n = 0;
    if (cudaMallocHost((void **)&c->h_prefix, (n + 1) * sizeof(long long)) != cudaSuccess) {
      f3g_set_error("cudaMallocHost of the chunk prefix failed");
      return 1;
    }
    c->prefix_n = n + 1;
  }
  if (!(c->h_info && c->h_info_n >= n)) {
    free(c->h_info);
    c->h_info = (f3g_pass_info *)calloc(n, sizeof(f3g_pass_info));
    c->h_info_n = c->h_info ? n : 0;
    if (!c->h_info) {
      f3g_set_error("host memory exhausted");
      return 1;
    }
  }
  if (!(c->h_items && c->h_items_n >= n)) {
    if (c->h_items) cudaFreeHost(c->h_items);
    c->h_items = NULL;
    c->h_items_n = 0;
    if (cudaMallocHost((void **)&c->h_items, n * sizeof(F3GItem)) != cudaSuccess) {
      f3g_set_error("cudaMallocHost of the work list failed");
      return 1;
    }
    c->h_items_n = n;
  }
  return 0;
}

int f3g_chunk_samples(const f3g_ctx *c, long long samples, int threads, int blocks, int sub_batch_size) {
  (void)c;
  long long per = samples / ((long long)threads * blocks);
  /* chains of 1024 samples, 2048 in launches of 8 or more waves of those
   * (fewer fuse steps; the short tail chunks keep the end of the launch
   * even): measured on the 1920x1080 still 2 % faster, on 100-sample
   * animation frames (3 waves) 1024 is the better length */
  int cap = f3g_opts.chain_samples > 0 ? f3g_opts.chain_samples : (per >= 8 * 2048 ? 2048 : 1024);
  if (sub_batch_size > 0 && cap > sub_batch_size) cap = sub_batch_size;
  if (per > cap) per = cap;
  if (per < 64) per = 64;
  if (per > cap) per = cap;
  return (int)per;
}

long long f3g_chunk_passes(F3GPass *p, int n, int threads, int blocks, int S, long long *prefix) {
  /* the tail chunks: a quarter of S (at least 64 samples per thread), for
   * the launch's last samples -- half a wave of S chunks, a whole wave for
   * S = 2048 -- so the blocks that took the last long chunks and those
   * still taking short ones finish within a short chunk of each other
   * (measured: 1.3 % on the 1920x1080 still at S = 1024, 2.2 % with
   * S = 2048 and a whole wave, 5.8 % on 1280x720 animation frames) */
  int St = f3g_opts.tail_chain_samples > 0 ? f3g_opts.tail_chain_samples : S / 4;
  if (f3g_opts.tail_chain_samples < 0 || S < 512 || St < 64) St = S;
  if (St > S) St = S;
  const double waves = f3g_opts.tail_wave_pct > 0 ? f3g_opts.tail_wave_pct / 100.0 : (S >= 2048 ? 1.0 : 0.5);
  const long long big = (long long)threads * S, small = (long long)threads * St;
  long long r = St < S ? (long long)(waves * blocks * (double)big) : 0;
  for (int i = n - 1; i >= 0; i--) {
    F3GPass *q = &p[i];
    const long long ns = q->samples;
    q->S = S;
    q->S_tail = St;
    if (r <= 0) {
      q->chunk_tail = (ns + big - 1) / big;
      q->nchunks = q->chunk_tail;
    } else if (r >= ns) {
      q->chunk_tail = 0;
      q->nchunks = (ns + small - 1) / small;
      r -= ns;
    } else {
      q->chunk_tail = (ns - r) / big;
      q->nchunks = q->chunk_tail + (ns - q->chunk_tail * big + small - 1) / small;
      r = 0;
    }
  }
  long long tot = 0;
  for (int i = 0; i < n; i++) {
    p[i].chunk_begin = tot;
    if (prefix) prefix[i] = tot;
    tot += p[i].nchunks;
  }
  if (prefix) prefix[n] = tot;
  return tot;
}

int f3g_choice_mode(int chaos_enable) {
  /* mode 1 shares each step's xform draw within a warp and relies on the
   * exchange between a block's warps to decorrelate the chains: with fewer
   * than 4 warps per block there is too little to exchange with, so those
   * blocks draw per thread (as for genomes with xaos) */
  const int threads = f3g_opts.threads_per_block > 0 ? f3g_opts.threads_per_block : 256;
  return (chaos_enable || f3g_opts.iter_mode == 0 || threads < 128) ? 0 : 1;
}

static int compute_geom(flam3_frame *spec, const flam3_genome *cp, int field, double **filter, f3g_geom *g) {
  g->oversample = cp->spatial_oversample;
  g->image_width = cp->width;
  g->out_width = g->image_width;
  if (field) {
    g->image_height = cp->height / 2;
    g->out_width *= 2;
  } else
    g->image_height = cp->height;
  if (g->image_width < 1 || g->image_height < 1) {
    f3g_set_error("image size must be positive, not %dx%d.", g->image_width, g->image_height);
    return 1;
  }
  double *flt = NULL;
  g->filter_width = f3g_spatial_filter(spec, field, &flt);
  if (g->filter_width < 0) return 1;
  if (filter) *filter = flt;
  else free(flt);
  g->gutter = (g->filter_width - g->oversample) / 2;
  int mx = 0;
  for (int i = 0; i < spec->ngenomes; i++) {
    int w = (int)ceil(spec->genomes[i].estimator) * g->oversample;
    if (w > mx) mx = w;
  }
  if (mx > 0) mx += g->oversample - 1;
  if (mx > g->gutter) {
    g->de_offset = mx - g->gutter;
    g->gutter = mx;
  } else
    g->de_offset = 0;
  g->H = g->oversample * g->image_height + 2 * g->gutter;
  g->W = g->oversample * g->image_width + 2 * g->gutter;
  return 0;
}

/* camera of one temporal sample (rect.c:785-827) */
static int set_camera(flam3_frame *spec, const flam3_genome *cp, int field, const f3g_geom *g, F3GPass *p,
                      double *sample_density, double *ppux_out, double *ppuy_out) {
  if (cp->sample_density <= 0.0) {
    f3g_set_error("sample density (quality) must be greater than zero, not %g.", cp->sample_density);
    return 1;
  }
  double scale = pow(2.0, cp->zoom);
  *sample_density = cp->sample_density * scale * scale;
  double ppux = cp->pixels_per_unit * scale, ppuy = field ? ppux / 2.0 : ppux, shift = 0.0;
  ppux /= spec->pixel_aspect_ratio;
  if (field == flam3_field_even) shift = -0.5;
  else if (field == flam3_field_odd) shift = 0.5;
  shift = shift / ppux;
  double t0 = (double)g->gutter / (g->oversample * ppux), t1 = (double)g->gutter / (g->oversample * ppuy);
  double corner0 = cp->center[0] - g->image_width / ppux / 2.0;
  double corner1 = cp->center[1] - g->image_height / ppuy / 2.0;
  p->bounds[0] = corner0 - t0;
  p->bounds[1] = corner1 - t1 + shift;
  p->bounds[2] = corner0 + g->image_width / ppux + t0;
  p->bounds[3] = corner1 + g->image_height / ppuy + t1 + shift;
  double size0 = 1.0 / (p->bounds[2] - p->bounds[0]), size1 = 1.0 / (p->bounds[3] - p->bounds[1]);
  p->rot[0][0] = cos(cp->rotate * 2 * M_PI / 360.0);
  p->rot[0][1] = -sin(cp->rotate * 2 * M_PI / 360.0);
  p->rot[1][0] = -p->rot[0][1];
  p->rot[1][1] = p->rot[0][0];
  p->rot_center[0] = cp->rot_center[0];
  p->rot_center[1] = cp->rot_center[1];
  p->rotate = cp->rotate != 0.0;
  p->width = g->W;
  p->height = g->H;
  p->ws0 = g->W * size0;
  p->wb0s0 = p->ws0 * p->bounds[0];
  p->hs1 = g->H * size1;
  p->hb1s1 = p->hs1 * p->bounds[1];
  *ppux_out = ppux;
  *ppuy_out = ppuy;
  return 0;
}

static unsigned long irand(randctx *r);

/* Advance the caller's ISAAC context as the reference does for one temporal
 * sample (rect.c:858-865: RANDSIZ words per host thread) and derive the
 * pass's Philox key from the words drawn. */
static void consume_rc(flam3_frame *spec, uint32_t key[2]) {
  int nthreads = spec->nthreads < 1 ? 1 : spec->nthreads;
  uint32_t w[4] = {0, 0, 0, 0};
  for (int t = 0; t < nthreads; t++)
    for (int k = 0; k < F3_RANDSIZ; k++) {
      unsigned long v = irand(&spec->rc);
      if (t == 0 && k < 4) w[k] = (uint32_t)v;
    }
  uint64_t salt = f3g_opts.seed_salt;
  key[0] = w[0] ^ (w[2] << 7 | w[2] >> 25) ^ (uint32_t)salt;
  key[1] = w[1] ^ (w[3] << 13 | w[3] >> 19) ^ (uint32_t)(salt >> 32);
}

/* ISAAC (isaac.c:25-45 with RANDSIZL 4), to advance the caller's context */
static void isaac_gen(randctx *ctx) {
  unsigned long a = ctx->randa, b, x, y, *m, *mm = ctx->randmem, *m2, *r = ctx->randrsl, *mend;
  b = (ctx->randb + (++ctx->randc)) & 0xffffffff;
#define IND(x) (mm[((x) >> 2) & (F3_RANDSIZ - 1)])
#define STEP(mix)                                       \
  do {                                                  \
    x = *m;                                             \
    a = ((a ^ (mix)) + *(m2++)) & 0xffffffff;           \
    *(m++) = y = (IND(x) + a + b) & 0xffffffff;         \
    *(r++) = b = (IND(y >> F3_RANDSIZL) + x) & 0xffffffff; \
  } while (0)
  for (m = mm, mend = m2 = m + F3_RANDSIZ / 2; m < mend;) {
    STEP(a << 13); STEP(a >> 6); STEP(a << 2); STEP(a >> 16);
  }
  for (m2 = mm; m2 < mend;) {
    STEP(a << 13); STEP(a >> 6); STEP(a << 2); STEP(a >> 16);
  }
#undef STEP
#undef IND
  ctx->randb = b;
  ctx->randa = a;
}

static unsigned long irand(randctx *r) {
  if (!r->randcnt--) {
    isaac_gen(r);
    r->randcnt = F3_RANDSIZ - 1;
  }
  return r->randrsl[r->randcnt];
}

/* ---- building the passes of one batch (rect.c:754-827) ----
 * The Philox keys are drawn first, in temporal-sample order, from the
 * caller's ISAAC context (the only ordered step); the genome interpolation,
 * preparation and packing of each temporal sample are independent and run on
 * up to 16 host threads; the per-sample scalars are summed afterwards in
 * order, so the result does not depend on the thread count. */
typedef struct {
  flam3_frame *spec;
  const f3g_geom *g;
  int field, first, ntemporal, nbatches, cmap_size, stride, start;
  const double *tfilter, *tdeltas;
  F3GPass *passes;
  f3g_pass_info *info;
} pass_job;

static void build_one_pass(const pass_job *pj, int ts) {
  F3GPass *p = &pj->passes[ts];
  f3g_pass_info *in = &pj->info[ts];
  flam3_frame *spec = pj->spec;
  flam3_genome cp;
  memset(&cp, 0, sizeof(cp));
  const int gi = pj->first + ts;
  const double color_scalar = pj->tfilter[gi];
  const double tst = spec->time + pj->tdeltas[gi];
  uint32_t key0 = p->key[0], key1 = p->key[1];
  memset(p, 0, offsetof(F3GPass, xf));
  p->key[0] = key0;
  p->key[1] = key1;
  in->err = 1;
  f3g_clear_error();
  if (f3g_interpolate(spec->genomes, spec->ngenomes, tst, &cp) || f3g_prepare_precalc_flags(&cp) ||
      f3g_build_distrib(&cp, p))
    goto fail;
  for (int i = 0; i < cp.num_xforms; i++) f3g_xform_precalc(&cp, i);
  if (f3g_pack_genome(&cp, p)) goto fail;
  in->need_count = 0;
  for (int j = 0; j < 256; j++) {
    for (int k = 0; k < 4; k++) p->dmap[j][k] = (float)((cp.palette[j].color[k] * F3G_WHITE) * color_scalar);
    if (cp.palette[j].color[3] != 1.0) in->need_count = 1;
  }
  p->cmap_size = pj->cmap_size;
  p->palette_mode = cp.palette_mode;
  if (set_camera(spec, &cp, pj->field, pj->g, p, &in->sample_density, &in->ppux, &in->ppuy)) goto fail;
  const double nsamples = in->sample_density * pj->g->image_width * pj->g->image_height;
  in->batch_size = nsamples / (pj->nbatches * pj->ntemporal);
  p->samples = (long long)in->batch_size;
  p->fuse = spec->earlyclip ? 100 : 15;
  p->iter_mode = f3g_choice_mode(cp.chaos_enable);
  in->vibrancy = cp.vibrancy;
  in->gamma = cp.gamma;
  for (int k = 0; k < 3; k++) in->background[k] = cp.background[k];
  in->contrast = cp.contrast;
  in->brightness = cp.brightness;
  in->gam_lin_thresh = cp.gam_lin_thresh;
  in->estimator_curve = cp.estimator_curve;
  in->err = 0;
  f3g_genome_free(&cp);
  return;
fail:
  snprintf(in->errmsg, sizeof(in->errmsg), "%s", flam3gpu_last_error());
  f3g_genome_free(&cp);
}

/* Process-wide planning workers: the temporal samples of every concurrent
 * f3g_build_batch_passes call are handed out one at a time (the calling
 * thread works on its own call too), so no threads are created per frame
 * and uneven samples balance themselves.  Workers start on first use (up to
 * 16, one per online core but the caller's) and live for the process. */
typedef struct plan_batch_s {
  const pass_job *pj;
  int next, done, n;
  struct plan_batch_s *link;
} plan_batch;

static pthread_mutex_t pl_mu = PTHREAD_MUTEX_INITIALIZER;
static pthread_cond_t pl_work = PTHREAD_COND_INITIALIZER, pl_done = PTHREAD_COND_INITIALIZER;
static plan_batch *pl_head = NULL;
static int pl_workers = 0;

static void *plan_worker(void *arg) {
  (void)arg;
  pthread_mutex_lock(&pl_mu);
  for (;;) {
    plan_batch *b = pl_head;
    while (b && b->next >= b->n) b = b->link;
    if (!b) {
      pthread_cond_wait(&pl_work, &pl_mu);
      continue;
    }
    const int ts = b->next++;
    pthread_mutex_unlock(&pl_mu);
    build_one_pass(b->pj, ts);
    pthread_mutex_lock(&pl_mu);
    if (++b->done == b->n) pthread_cond_broadcast(&pl_done);
  }
  return NULL;
}

/* under pl_mu */
static void plan_workers_start(void) {
  long ncpu = sysconf(_SC_NPROCESSORS_ONLN);
  int want = (int)(ncpu > 1 ? ncpu - 1 : 0);
  if (want > 16) want = 16;
  while (pl_workers < want) {
    pthread_t th;
    pthread_attr_t at;
    pthread_attr_init(&at);
    pthread_attr_setdetachstate(&at, PTHREAD_CREATE_DETACHED);
    const int ok = pthread_create(&th, &at, plan_worker, NULL) == 0;
    pthread_attr_destroy(&at);
    if (!ok) break;
    pl_workers++;
  }
}

int f3g_build_batch_passes(flam3_frame *spec, int field, const f3g_geom *g, int batch, int nbatches, int ntemporal,
                           const double *tfilter, const double *tdeltas, int cmap_size, F3GPass *passes,
                           f3g_pass_info *info) {
  /* keys in order: the caller's ISAAC context advances as the reference's */
  for (int ts = 0; ts < ntemporal; ts++) consume_rc(spec, passes[ts].key);
  pass_job pj = {spec, g, field, batch * ntemporal, ntemporal, nbatches, cmap_size, 1, 0, tfilter, tdeltas, passes, info};
  if (ntemporal < 3) {
    for (int ts = 0; ts < ntemporal; ts++) build_one_pass(&pj, ts);
  } else {
    plan_batch b = {&pj, 0, 0, ntemporal, NULL};
    pthread_mutex_lock(&pl_mu);
    plan_workers_start();
    plan_batch **tail = &pl_head;
    while (*tail) tail = &(*tail)->link;
    *tail = &b;
    pthread_cond_broadcast(&pl_work);
    while (b.next < b.n) {
      const int ts = b.next++;
      pthread_mutex_unlock(&pl_mu);
      build_one_pass(&pj, ts);
      pthread_mutex_lock(&pl_mu);
      b.done++;
    }
    while (b.done < b.n) pthread_cond_wait(&pl_done, &pl_mu);
    for (plan_batch **q = &pl_head; *q; q = &(*q)->link)
      if (*q == &b) {
        *q = b.link;
        break;
      }
    pthread_mutex_unlock(&pl_mu);
  }
  for (int ts = 0; ts < ntemporal; ts++)
    if (info[ts].err) {
      f3g_set_error("%s", info[ts].errmsg[0] ? info[ts].errmsg : "pass preparation failed");
      return 1;
    }
  return 0;
}

/* ---- temporal samples planned on the device (f3g_plan.cu) ----
 * For frames with several genomes the host does only what it needs before
 * the launch: each sample's key segment and weights (the keys of a segment
 * aligned once), the genome scalars, xform weights, chaos rows and palette
 * alpha of its blend (camera, sample count, choice mode, checks) and the
 * pass header.  The key sets and one record per sample are staged in pinned
 * memory for the plan kernel, which fills in the colour map, xforms,
 * variation lists and choice rows on the device. */
typedef struct {
  int first, n;
  size_t off;
  flam3_genome keys[4];
} plan_seg;

static size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

static int plan_stage_keys(f3g_ctx *c, size_t need, size_t keep) {
  if (need <= c->h_plan_keys_bytes) return 0;
  size_t cap = need < 65536 ? 65536 : 2 * need;
  unsigned char *nb = NULL;
  if (cudaMallocHost((void **)&nb, cap) != cudaSuccess) {
    f3g_set_error("cudaMallocHost of %zu bytes failed", cap);
    return 1;
  }
  if (c->h_plan_keys) {
    memcpy(nb, c->h_plan_keys, keep);
    cudaFreeHost(c->h_plan_keys);
  }
  c->h_plan_keys = nb;
  c->h_plan_keys_bytes = cap;
  return 0;
}

/* Returns 0 with the batch planned for the device, 1 on error, -1 when the
 * frame needs the host planner (lists beyond the pass's capacity). */
static int build_batch_passes_device(f3g_ctx *c, flam3_frame *spec, int field, const f3g_geom *g, int batch,
                                     int nbatches, int ntemporal, const double *tfilter, const double *tdeltas,
                                     int cmap_size, F3GPass *passes, f3g_pass_info *info, size_t *key_bytes) {
  /* a frame whose keys could make more active variations than a pass holds
   * stays on the host planner (which reports the limit) */
  for (int k = 0; k < spec->ngenomes; k++) {
    const flam3_genome *gk = &spec->genomes[k];
    if (gk->num_xforms > F3G_MAX_XFORMS) return -1;
  }
  {
    int nv = 0, nxm = 0;
    for (int k = 0; k < spec->ngenomes; k++) nxm = spec->genomes[k].num_xforms > nxm ? spec->genomes[k].num_xforms : nxm;
    for (int xf = 0; xf < nxm; xf++)
      for (int j = 0; j < flam3_nvariations; j++) {
        int any = j == 0; /* padding xforms may take linear */
        for (int k = 0; k < spec->ngenomes && !any; k++)
          if (xf < spec->genomes[k].num_xforms && spec->genomes[k].xform[xf].var[j] != 0) any = 1;
        nv += any;
      }
    if (nv + 8 * nxm > F3G_MAX_VARLIST) return -1;
  }
  if (c->h_plan_samples_n < (size_t)ntemporal) {
    if (c->h_plan_samples) cudaFreeHost(c->h_plan_samples);
    c->h_plan_samples = NULL;
    c->h_plan_samples_n = 0;
    if (cudaMallocHost((void **)&c->h_plan_samples, (size_t)ntemporal * sizeof(F3GPlanSample)) != cudaSuccess) {
      f3g_set_error("cudaMallocHost of the plan records failed");
      return 1;
    }
    c->h_plan_samples_n = (size_t)ntemporal;
  }
  /* keys in order: the caller's ISAAC context advances as the reference's */
  for (int ts = 0; ts < ntemporal; ts++) consume_rc(spec, passes[ts].key);
  plan_seg *segs = (plan_seg *)calloc((size_t)ntemporal, sizeof(plan_seg));
  int nseg = 0, rc = 1;
  size_t used = 0;
  flam3_genome sg;
  memset(&sg, 0, sizeof(sg));
  c->plan_nx = c->plan_nstd = 0;
  for (int ts = 0; ts < ntemporal; ts++) {
    const int gi = batch * ntemporal + ts;
    const double tst = spec->time + tdeltas[gi];
    double w[4];
    int first = 0;
    const int n = f3g_interp_segment(spec->genomes, spec->ngenomes, tst, &first, w);
    int si = -1;
    for (int k = 0; k < nseg; k++)
      if (segs[k].first == first && segs[k].n == n) si = k;
    if (si < 0) {
      plan_seg *sp = &segs[nseg];
      sp->first = first;
      sp->n = n;
      f3g_align_keys(sp->keys, &spec->genomes[first], n);
      const int nx = sp->keys[0].num_xforms, nstd = nx - (sp->keys[0].final_xform_index >= 0);
      F3GKeySet ks;
      ks.nk = n;
      ks.nx = nx;
      ks.nstd = nstd;
      ks.final_index = sp->keys[0].final_xform_index;
      ks.off_genome = (long long)align16(sizeof(F3GKeySet));
      ks.off_xform = (long long)align16((size_t)ks.off_genome + (size_t)n * sizeof(flam3_genome));
      ks.off_chaos = (long long)align16((size_t)ks.off_xform + (size_t)n * nx * sizeof(flam3_xform));
      const size_t off = align16(used), total = (size_t)ks.off_chaos + (size_t)n * nstd * nstd * sizeof(double);
      if (plan_stage_keys(c, off + total, used)) goto out;
      unsigned char *b = c->h_plan_keys + off;
      memcpy(b, &ks, sizeof(ks));
      for (int k = 0; k < n; k++) {
        memcpy(b + ks.off_genome + (size_t)k * sizeof(flam3_genome), &sp->keys[k], sizeof(flam3_genome));
        memcpy(b + ks.off_xform + (size_t)k * nx * sizeof(flam3_xform), sp->keys[k].xform, (size_t)nx * sizeof(flam3_xform));
        for (int i = 0; i < nstd; i++)
          memcpy(b + ks.off_chaos + ((size_t)k * nstd + i) * nstd * sizeof(double), sp->keys[k].chaos[i],
                 (size_t)nstd * sizeof(double));
      }
      sp->off = off;
      used = off + total;
      if (nx > c->plan_nx) c->plan_nx = nx;
      if (nstd > c->plan_nstd) c->plan_nstd = nstd;
      si = nseg++;
    }
    plan_seg *sp = &segs[si];
    F3GPlanSample *rec = &c->h_plan_samples[ts];
    rec->keyset = (long long)sp->off;
    for (int k = 0; k < 4; k++) rec->w[k] = w[k];
    rec->color_scalar = tfilter[gi];
    /* the blend's scalars, xform weights, chaos rows and palette alpha */
    f3g_release_genome(&sg);
    f3g_blend_scalars(sp->keys, n, w, &sg);
    const int nx = sg.num_xforms, nstd = nx - (sg.final_xform_index >= 0);
    F3GPass *p = &passes[ts];
    f3g_pass_info *in = &info[ts];
    const uint32_t key0 = p->key[0], key1 = p->key[1];
    memset(p, 0, offsetof(F3GPass, xf));
    p->key[0] = key0;
    p->key[1] = key1;
    memset(in, 0, sizeof(*in));
    int unity = 1;
    for (int i = 0; i < nstd; i++)
      for (int j = 0; j < nstd; j++)
        if (fabs(sg.chaos[i][j] - 1.0) > F3G_EPS) unity = 0;
    /* choice rows of zero total weight (flam3.c:190-196) */
    for (int r = -1; r < (unity ? 0 : nstd); r++) {
      double dr = 0.0;
      for (int i = 0; i < nstd; i++) dr += r >= 0 ? sg.xform[i].density * sg.chaos[r][i] : sg.xform[i].density;
      if (dr == 0.0) {
        f3g_set_error("cannot iterate empty flame.");
        goto out;
      }
    }
    p->num_xforms = nx;
    p->num_std = nstd;
    p->final_index = sg.final_xform_index;
    p->final_enable = sg.final_xform_enable == 1 && sg.final_xform_index >= 0;
    p->chaos_enable = 1 - unity;
    p->cmap_size = cmap_size;
    p->palette_mode = sg.palette_mode;
    /* the iterate kernel's instantiation: extended variations in any key */
    for (int k = 0; k < n && !p->full_variations; k++)
      for (int xf = 0; xf < nx && !p->full_variations; xf++)
        for (int j = 20; j < flam3_nvariations; j++)
          if (sp->keys[k].xform[xf].var[j] != 0) {
            p->full_variations = 1;
            break;
          }
    if (set_camera(spec, &sg, field, g, p, &in->sample_density, &in->ppux, &in->ppuy)) goto out;
    const double nsamples = in->sample_density * g->image_width * g->image_height;
    in->batch_size = nsamples / (nbatches * ntemporal);
    p->samples = (long long)in->batch_size;
    p->fuse = spec->earlyclip ? 100 : 15;
    p->iter_mode = f3g_choice_mode(p->chaos_enable);
    for (int j = 0; j < 256; j++)
      if (sg.palette[j].color[3] != 1.0) in->need_count = 1;
    in->vibrancy = sg.vibrancy;
    in->gamma = sg.gamma;
    for (int k = 0; k < 3; k++) in->background[k] = sg.background[k];
    in->contrast = sg.contrast;
    in->brightness = sg.brightness;
    in->gam_lin_thresh = sg.gam_lin_thresh;
    in->estimator_curve = sg.estimator_curve;
  }
  *key_bytes = used;
  rc = 0;
out:
  f3g_release_genome(&sg);
  for (int k = 0; k < nseg; k++)
    for (int i = 0; i < segs[k].n; i++) f3g_release_genome(&segs[k].keys[i]);
  free(segs);
  return rc;
}

/* Uploads the staged key sets and sample records and launches the plan
 * kernel over the passes (whose headers are already on the device). */
static int launch_device_plan(f3g_ctx *c, int ntemporal, size_t key_bytes) {
  if (f3g_ensure((void **)&c->d_plan_keys, &c->d_plan_keys_bytes, key_bytes) ||
      f3g_ensure((void **)&c->d_plan_samples, &c->d_plan_samples_bytes, (size_t)ntemporal * sizeof(F3GPlanSample)) ||
      f3g_ensure((void **)&c->d_plan_err, &c->d_plan_err_bytes, (size_t)ntemporal * sizeof(int)))
    return 1;
  if (cudaMemcpyAsync(c->d_plan_keys, c->h_plan_keys, key_bytes, cudaMemcpyHostToDevice, c->stream) != cudaSuccess ||
      cudaMemcpyAsync(c->d_plan_samples, c->h_plan_samples, (size_t)ntemporal * sizeof(F3GPlanSample),
                      cudaMemcpyHostToDevice, c->stream) != cudaSuccess ||
      cudaMemsetAsync(c->d_plan_err, 0, (size_t)ntemporal * sizeof(int), c->stream) != cudaSuccess) {
    f3g_set_error("plan upload failed");
    return 1;
  }
  int e = f3g_launch_plan(c->d_plan_keys, c->d_plan_samples, ntemporal, c->plan_nx, c->plan_nstd, c->d_passes,
                          c->d_plan_err, c->stream);
  if (e) {
    f3g_set_error("plan launch failed: %s", cudaGetErrorString((cudaError_t)e));
    return 1;
  }
  return 0;
}

/* Copies n values as floats to a device buffer through the context's pinned
 * staging area at float offset `slot` (so the copy is truly asynchronous);
 * a slot may be reused only after the stream has passed the copy. */
static float *upload_floats(f3g_ctx *c, float **dptr, size_t *cap, const double *src, size_t n, size_t slot) {
  if (slot + n > c->h_stage_n) {
    size_t want = slot + n < 4096 ? 4096 : 2 * (slot + n);
    float *nb = NULL;
    cudaStreamSynchronize(c->stream); /* the old staging area may still be read */
    if (cudaMallocHost((void **)&nb, want * sizeof(float)) != cudaSuccess) {
      f3g_set_error("cudaMallocHost of %zu floats failed", want);
      return NULL;
    }
    if (c->h_stage) cudaFreeHost(c->h_stage);
    c->h_stage = nb;
    c->h_stage_n = want;
  }
  float *tmp = c->h_stage + slot;
  for (size_t i = 0; i < n; i++) tmp[i] = (float)src[i];
  if (f3g_ensure((void **)dptr, cap, n * sizeof(float))) return NULL;
  cudaError_t e = cudaMemcpyAsync(*dptr, tmp, n * sizeof(float), cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) f3g_set_error("filter upload failed: %s", cudaGetErrorString(e));
  return e == cudaSuccess ? *dptr : NULL;
}

int flam3gpu_histogram_dims(flam3_frame *f, int field, int *w, int *h, int *gutter, int *de_offset,
                            int *filter_width) {
  f3g_clear_error();
  flam3_genome cp;
  memset(&cp, 0, sizeof(cp));
  if (f3g_interpolate(f->genomes, f->ngenomes, f->time, &cp)) return 1;
  f3g_geom g;
  int rc = compute_geom(f, &cp, field, NULL, &g);
  f3g_genome_free(&cp);
  if (rc) return 1;
  if (w) *w = g.W;
  if (h) *h = g.H;
  if (gutter) *gutter = g.gutter;
  if (de_offset) *de_offset = g.de_offset;
  if (filter_width) *filter_width = g.filter_width;
  return 0;
}

static double now_s(void) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return t.tv_sec + 1e-9 * t.tv_nsec;
}

int flam3gpu_render_ex(flam3_frame *spec, void *out, int field, int nchan, int transp, stat_struct *stats,
                       flam3gpu_render_io *io) {
  f3g_clear_error();
  double t_iter = 0, t_de = 0, t_tail = 0;
  int launches = 0;
  double h2d = 0, d2h = 0, plotted = 0;
  double wall0 = now_s();
  time_t tstart = time(NULL);
  int bits = spec->bits;
  /* failures before any state exists: message on stderr, return 1 (the
   * reference prints its argument errors, flam3.c:3889-3892) */
  if (bits != 32 && bits != 33 && bits != 64) {
    f3g_set_error("flam3: bits must be 32, 33, or 64 not %d.", bits);
    fprintf(stderr, "flam3gpu: %s\n", flam3gpu_last_error());
    return 1;
  }
  if (nchan != 3 && nchan != 4) {
    f3g_set_error("nchan must be 3 or 4, not %d", nchan);
    fprintf(stderr, "flam3gpu: %s\n", flam3gpu_last_error());
    return 1;
  }
  f3g_ctx *c = f3g_get_ctx();
  if (!c) {
    f3g_set_error("no CUDA device available");
    fprintf(stderr, "flam3gpu: %s\n", flam3gpu_last_error());
    return 1;
  }
  stats->num_iters = 0;
  stats->badvals = 0;
  const char *ap = getenv("apo_palette");
  int cmap_size = 256 - (ap ? atoi(ap) : 0);
  if (cmap_size < 2 || cmap_size > 256) {
    f3g_set_error("apo_palette gives a colour map of %d entries", cmap_size);
    return 1;
  }
  flam3_genome cp;
  memset(&cp, 0, sizeof(cp));
  if (f3g_interpolate(spec->genomes, spec->ngenomes, spec->time, &cp)) return 1;
  int rv = 1;
  double *filter = NULL, *tfilter = NULL, *tdeltas = NULL, *de_w = NULL, *de_c = NULL;
  int nbatches = cp.nbatches, ntemporal = cp.ntemporal_samples;
  double highpow = cp.highlight_power;
  f3g_geom g;
  if (nbatches < 1) {
    f3g_set_error("nbatches must be positive, not %d.", nbatches);
    goto done;
  }
  if (cp.spatial_oversample < 1) {
    f3g_set_error("oversample must be positive, not %d.", cp.spatial_oversample);
    goto done;
  }
  if (ntemporal < 1) {
    f3g_set_error("temporal samples must be positive, not %d.", ntemporal);
    goto done;
  }
  if (compute_geom(spec, &cp, field, &filter, &g)) goto done;
  if (io) {
    io->hist_w = g.W;
    io->hist_h = g.H;
    io->image_w = g.image_width;
    io->image_h = g.image_height;
  }
  if (!out && !(io && io->keep_on_device)) {
    f3g_set_error("no output buffer");
    goto done;
  }
  double sumfilt = f3g_temporal_filter(nbatches * ntemporal, cp.temporal_filter_type, cp.temporal_filter_exp,
                                       cp.temporal_filter_width, &tfilter, &tdeltas);
  const long long nb = (long long)g.W * g.H;
  const int bkind = bits == 64 ? F3G_BK_F64 : F3G_BK_F32;
  const size_t bsz = bkind == F3G_BK_F64 ? 32 : 16;
  const size_t csz = bkind == F3G_BK_F64 ? 8 : 4;
  /* does the fifth (count) channel differ from alpha?  only for palettes
   * with alpha != 1 or temporal filter weights != 1 (rect.c:778-782) */
  int need_count = 0;
  for (int i = 0; i < nbatches * ntemporal; i++)
    if (tfilter[i] != 1.0) need_count = 1;
  const int threads = f3g_opts.threads_per_block > 0 ? f3g_opts.threads_per_block : 256;
  if (f3g_ensure(&c->d_hist, &c->hist_bytes, (size_t)nb * bsz)) goto done;
  if (f3g_ensure(&c->d_acc, &c->acc_bytes, (size_t)nb * bsz)) goto done;
  size_t out_bytes = (size_t)g.image_width * g.image_height * nchan * spec->bytes_per_channel;
  if (f3g_ensure((void **)&c->d_out, &c->out_bytes, out_bytes)) goto done;
  const size_t filter_n = F3G_FILTER_FLOATS(g.filter_width);
  const size_t kinfo_slot = (filter_n + 63) & ~(size_t)63;
  if (!upload_floats(c, &c->d_filter, &c->filter_bytes, filter, filter_n, 0)) goto done;
  h2d += (double)filter_n * sizeof(float);
  int acc_cleared = 0; /* the accumulator is cleared only when a path uses it */
  if (ensure_host_passes(c, (size_t)ntemporal)) goto done;
  if (f3g_ensure((void **)&c->d_passes, &c->passes_bytes, (size_t)ntemporal * sizeof(F3GPass))) goto done;
  if (f3g_ensure((void **)&c->d_prefix, &c->prefix_bytes, (size_t)(ntemporal + 1) * sizeof(long long))) goto done;
  if (f3g_ensure((void **)&c->d_items, &c->d_items_bytes, (size_t)ntemporal * sizeof(F3GItem))) goto done;
  const int precision = f3g_opts.iter_precision == 64 ? 64 : 32;
  const int de_tile = f3g_opts.de_tile > 0 ? f3g_opts.de_tile : 16;
  /* a one-batch render without a progress callback runs uploads, iterate,
   * tail and copy-out back to back and waits once */
  const int deferred_iter = nbatches == 1 && !spec->progress && !(io && (io->hist_out || io->accum_out));
  int pending_ctr = 0;
  double vibrancy = 0.0, gamma = 0.0, background[3] = {0, 0, 0};
  int vib_gam_n = 0;
  double ppux = 0, ppuy = 0, sample_density = 0;
  const int fused_tail = (nbatches == 1) && !(io && io->accum_out);
  int de_used_any = 0;
  /* fused DE tail state (one batch) */
  int fde = 0, fde_mfc = 0, fde_mfi = 0, fde_R = 0, fde_count = 0, bands = 0;
  /* work counters of band DE, when asked for (flam3gpu_options.de_stats) */
  unsigned long long *de_stats = NULL;
  memset(c->de_work, 0, sizeof(c->de_work));
  if (f3g_opts.de_stats) {
    if (f3g_ensure((void **)&c->d_de_stats, &c->de_stats_bytes, 4 * sizeof(unsigned long long))) goto done;
    CK(cudaMemsetAsync(c->d_de_stats, 0, 4 * sizeof(unsigned long long), c->stream));
    de_stats = c->d_de_stats;
  }
  double fde_k1 = 0, fde_k2 = 0, fde_curve = 0;

  for (int batch = 0; batch < nbatches; batch++) {
    double de_time = spec->time + tdeltas[batch * ntemporal];
    int mfc = 0, mfi = 0, ks = 0;
    free(de_w);
    free(de_c);
    de_w = de_c = NULL;
    if (f3g_interpolate(spec->genomes, spec->ngenomes, de_time, &cp)) goto done;
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
    }
    const int de_on = mfi > 0;
    de_used_any |= de_on;
    int use_count = de_on && need_count;
    CK(cudaMemsetAsync(c->d_hist, 0, (size_t)nb * bsz, c->stream));
    if (use_count) {
      if (f3g_ensure(&c->d_count, &c->count_bytes, (size_t)nb * csz)) goto done;
      CK(cudaMemsetAsync(c->d_count, 0, (size_t)nb * csz, c->stream));
    }
    /* ---- passes of this batch: multi-genome frames planned on the device ---- */
    long long total_chunks = 0, batch_samples = 0;
    int dev_plan = 0;
    size_t key_bytes = 0;
    if (spec->ngenomes > 1 && !f3g_opts.host_plan && !f3g_interp_overridden()) {
      if (batch > 0) CK(cudaStreamSynchronize(c->stream)); /* the staging of the previous batch is read */
      const int r = build_batch_passes_device(c, spec, field, &g, batch, nbatches, ntemporal, tfilter, tdeltas,
                                              cmap_size, c->h_passes, c->h_info, &key_bytes);
      if (r > 0) goto done;
      dev_plan = r == 0;
    }
    if (!dev_plan && f3g_build_batch_passes(spec, field, &g, batch, nbatches, ntemporal, tfilter, tdeltas, cmap_size,
                                            c->h_passes, c->h_info))
      goto done;
    for (int ts = 0; ts < ntemporal; ts++) {
      F3GPass *p = &c->h_passes[ts];
      const f3g_pass_info *in = &c->h_info[ts];
      need_count |= in->need_count;
      sample_density = in->sample_density;
      ppux = in->ppux;
      ppuy = in->ppuy;
      stats->num_iters += in->batch_size;
      p->buckets = c->d_hist;
      p->count = use_count ? c->d_count : NULL;
      p->bucket_kind = bkind;
      p->trunc_hits = bits <= 33 && !f3g_opts.float_buckets;
      batch_samples += p->samples;
      vibrancy += in->vibrancy;
      gamma += in->gamma;
      background[0] += in->background[0];
      background[1] += in->background[1];
      background[2] += in->background[2];
      vib_gam_n++;
    }
    /* k1/k2, the DE curve and the tonemap read the last temporal sample's genome */
    cp.contrast = c->h_info[ntemporal - 1].contrast;
    cp.brightness = c->h_info[ntemporal - 1].brightness;
    cp.gam_lin_thresh = c->h_info[ntemporal - 1].gam_lin_thresh;
    cp.estimator_curve = c->h_info[ntemporal - 1].estimator_curve;
    if (use_count == 0 && de_on && need_count) {
      /* palette alpha != 1 found while packing: redo the batch with a count plane */
      use_count = 1;
      if (f3g_ensure(&c->d_count, &c->count_bytes, (size_t)nb * csz)) goto done;
      CK(cudaMemsetAsync(c->d_count, 0, (size_t)nb * csz, c->stream));
      for (int ts = 0; ts < ntemporal; ts++) c->h_passes[ts].count = c->d_count;
    }
    if (!(io && io->hist_in)) {
      int full = 0, mode = 1;
      for (int ts = 0; ts < ntemporal; ts++) {
        full |= c->h_passes[ts].full_variations;
        if (c->h_passes[ts].iter_mode == 0) mode = 0;
      }
      int occ = f3g_iterate_occupancy(precision, full, mode, threads);
      if (occ < 1) occ = 1;
      int blocks = f3g_opts.blocks > 0 ? f3g_opts.blocks : c->nsm * occ;
      int S = f3g_chunk_samples(c, batch_samples, threads, blocks, spec->sub_batch_size);
      unsigned long long *d_counts =
          (unsigned long long *)((char *)c->d_ctr + offsetof(F3GCounters, badvals));
      total_chunks = f3g_chunk_passes(c->h_passes, ntemporal, threads, blocks, S, c->h_prefix);
      for (int ts = 0; ts < ntemporal; ts++) {
        c->h_passes[ts].counters = d_counts;
        c->h_items[ts].pass = c->d_passes + ts;
        c->h_items[ts].chunk_first = 0;
      }
      int nxmax = 0;
      for (int ts = 0; ts < ntemporal; ts++)
        if (c->h_passes[ts].num_xforms > nxmax) nxmax = c->h_passes[ts].num_xforms;
      /* device-planned passes: the headers here, the rest from the plan kernel */
      const size_t pass_bytes = dev_plan ? offsetof(F3GPass, xf) : F3G_PASS_BYTES(nxmax);
      CK(cudaMemcpy2DAsync(c->d_passes, sizeof(F3GPass), c->h_passes, sizeof(F3GPass), pass_bytes,
                           (size_t)ntemporal, cudaMemcpyHostToDevice, c->stream));
      if (dev_plan) {
        if (launch_device_plan(c, ntemporal, key_bytes)) goto done;
        launches++;
        h2d += (double)key_bytes + (double)ntemporal * sizeof(F3GPlanSample);
      }
      h2d += (double)ntemporal * pass_bytes + (double)(ntemporal + 1) * sizeof(long long) +
             (double)ntemporal * sizeof(F3GItem);
      CK(cudaMemcpyAsync(c->d_prefix, c->h_prefix, (size_t)(ntemporal + 1) * sizeof(long long),
                               cudaMemcpyHostToDevice, c->stream));
      CK(cudaMemcpyAsync(c->d_items, c->h_items, (size_t)ntemporal * sizeof(F3GItem), cudaMemcpyHostToDevice,
                         c->stream));
      if (c->plan_only_out) {
        /* plan-only probe: batch 0's passes to the caller, no render */
        const int n = ntemporal < c->plan_only_max ? ntemporal : c->plan_only_max;
        CK(cudaMemcpyAsync(c->plan_only_out, c->d_passes, (size_t)n * sizeof(F3GPass), cudaMemcpyDeviceToHost,
                           c->stream));
        CK(cudaStreamSynchronize(c->stream));
        c->plan_only_n = n;
        rv = 0;
        goto done;
      }
      int shuffle = f3g_opts.shuffle_every > 0 ? f3g_opts.shuffle_every : 1;
      /* rounds: one launch, or ~10 launches with progress callbacks between */
      int nrounds = spec->progress ? 10 : 1;
      long long per_round = (total_chunks + nrounds - 1) / nrounds;
      if (per_round < 1) per_round = 1;
      for (long long lo = 0; lo < total_chunks; lo += per_round) {
        long long hi = lo + per_round < total_chunks ? lo + per_round : total_chunks;
        F3GCounters init;
        memset(&init, 0, sizeof(init));
        init.next_chunk = (unsigned long long)lo;
        init.test_stall = f3g_opts.test_exchange_stall ? (unsigned long long)lo + 1 : 0; /* the launch's first chunk */
        *c->h_ctr = init;
        CK(cudaMemcpyAsync(c->d_ctr, c->h_ctr, sizeof(F3GCounters), cudaMemcpyHostToDevice, c->stream));
        h2d += sizeof(F3GCounters);
        d2h += sizeof(F3GCounters);
        CK(cudaEventRecord(c->ev[0], c->stream));
        int e = f3g_launch_iterate(c->d_items, c->d_prefix, ntemporal, hi, shuffle, precision, full, mode,
                                   threads, blocks, c->d_ctr, c->stream);
        launches++;
        if (e) {
          f3g_set_error("iterate launch failed: %s", cudaGetErrorString((cudaError_t)e));
          goto done;
        }
        CK(cudaEventRecord(c->ev[1], c->stream));
        CK(cudaMemcpyAsync(c->h_ctr, c->d_ctr, sizeof(F3GCounters), cudaMemcpyDeviceToHost, c->stream));
        if (deferred_iter) {
          /* one batch, no progress callback: the tail is queued right behind
           * this launch; the counters are read after the final wait */
          pending_ctr = 1;
          continue;
        }
        CK(cudaStreamSynchronize(c->stream));
        float ms = 0;
        cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]);
        t_iter += ms;
        stats->badvals += (double)c->h_ctr->badvals;
        plotted += (double)c->h_ctr->plotted;
        if (c->h_ctr->error) {
          f3g_set_error("iterate kernel: a point-exchange wait timed out");
          goto done;
        }
        if (spec->progress) {
          double pct = 100.0 * ((double)batch + (double)hi / (double)total_chunks) / nbatches;
          int r = spec->progress(spec->progress_parameter, pct, 0, 0.0);
          while (r == 2) {
            struct timespec ts = {0, 100000000};
            nanosleep(&ts, NULL);
            r = spec->progress(spec->progress_parameter, pct, 0, 0.0);
          }
          if (r == 1) {
            rv = 0;
            goto done; /* abort: return 0 with the output as it stands (rect.c:919-922) */
          }
        }
      }
    } else {
      /* injected histogram (R,G,B,A,count doubles per bucket) */
      size_t n5 = (size_t)nb * 5;
      void *hb = malloc((size_t)nb * bsz);
      void *hc = use_count ? malloc((size_t)nb * csz) : NULL;
      for (size_t b = 0; b < (size_t)nb; b++) {
        const double *s = io->hist_in + 5 * b;
        if (bkind == F3G_BK_F64) {
          memcpy((double *)hb + 4 * b, s, 4 * sizeof(double));
          if (hc) ((double *)hc)[b] = s[4];
        } else {
          for (int k = 0; k < 4; k++) ((float *)hb)[4 * b + k] = (float)s[k];
          if (hc) ((float *)hc)[b] = (float)s[4];
        }
      }
      (void)n5;
      cudaError_t e1 = cudaMemcpy(c->d_hist, hb, (size_t)nb * bsz, cudaMemcpyHostToDevice);
      cudaError_t e2 = hc ? cudaMemcpy(c->d_count, hc, (size_t)nb * csz, cudaMemcpyHostToDevice) : cudaSuccess;
      free(hb);
      free(hc);
      if (e1 != cudaSuccess || e2 != cudaSuccess) {
        f3g_set_error("histogram upload failed");
        goto done;
      }
    }
    if (io && io->hist_out) {
      void *hb = malloc((size_t)nb * bsz);
      void *hc = use_count ? malloc((size_t)nb * csz) : NULL;
      CK(cudaStreamSynchronize(c->stream));
      cudaMemcpy(hb, c->d_hist, (size_t)nb * bsz, cudaMemcpyDeviceToHost);
      if (hc) cudaMemcpy(hc, c->d_count, (size_t)nb * csz, cudaMemcpyDeviceToHost);
      for (size_t b = 0; b < (size_t)nb; b++) {
        double *d = io->hist_out + 5 * b;
        for (int k = 0; k < 4; k++)
          d[k] = bkind == F3G_BK_F64 ? ((double *)hb)[4 * b + k] : (double)((float *)hb)[4 * b + k];
        d[4] = hc ? (bkind == F3G_BK_F64 ? ((double *)hc)[b] : (double)((float *)hc)[b]) : d[3];
      }
      free(hb);
      free(hc);
    }
    /* ---- k1/k2 and density estimation (rect.c:933-1050) ---- */
    double k1 = (cp.contrast * cp.brightness * 255.0 * 268.0 * (1.0 / nbatches)) / 256;
    double area = g.image_width * g.image_height / (ppux * ppuy);
    double k2 = (g.oversample * g.oversample * nbatches) / (cp.contrast * area * F3G_WHITE * sample_density * sumfilt);
    if (fused_tail && !de_on) {
      /* the fused tail below reads the histogram directly */
      goto tail_fused;
    }
    if (de_on) {
      int R = (int)ceil(de_w[0]) - 1;
      if (R > f3g_de_max_reach()) {
        f3g_set_error("density estimation radius %d exceeds the library's limit %d", R, f3g_de_max_reach());
        goto done;
      }
      int nk = mfi + 1;
      {
        float *ki = (float *)malloc((size_t)nk * 4 * sizeof(float));
        double *kid = (double *)malloc((size_t)nk * 4 * sizeof(double));
        f3g_de_kernel_info(mfi, ks, de_w, de_c, ki);
        for (int i = 0; i < 4 * nk; i++) kid[i] = ki[i];
        /* several batches reuse the slot: wait for the previous batch's copy */
        if (batch > 0) cudaStreamSynchronize(c->stream);
        float *ok = upload_floats(c, &c->d_de_w, &c->de_w_bytes, kid, (size_t)nk * 4, kinfo_slot);
        free(ki);
        free(kid);
        if (!ok) goto done;
      }
      h2d += (double)nk * 4 * sizeof(float);
      bands = f3g_opts.de_kernel == 0 && f3g_de_bands_supported(R, mfi);
      if (bands && f3g_ensure((void **)&c->d_fi, &c->fi_bytes, (size_t)nb)) goto done;
      if (fused_tail && (bands || f3g_de_fused_smem_tile(g.oversample, g.filter_width, R, nk, de_tile) <= 220 * 1024)) {
        /* one batch: band DE into the accumulator, then filter + tonemap +
         * pack; or DE, filter, tonemap and pack in one fused kernel */
        fde = bands ? 2 : 1;
        fde_mfc = mfc;
        fde_mfi = mfi;
        fde_R = R;
        fde_k1 = k1;
        fde_k2 = k2;
        fde_curve = cp.estimator_curve;
        fde_count = use_count;
        goto tail_fused;
      }
    }
    if (!acc_cleared) {
      CK(cudaMemsetAsync(c->d_acc, 0, (size_t)nb * bsz, c->stream));
      acc_cleared = 1;
    }
    CK(cudaEventRecord(c->ev[2], c->stream));
    if (de_on) {
      int R = (int)ceil(de_w[0]) - 1;
      int e = bands ? f3g_launch_de_bands(c->d_hist, bkind, use_count ? c->d_count : NULL, g.W, g.H, g.oversample,
                                          k1, k2, cp.estimator_curve, mfc, mfi, c->d_de_w, R, c->d_fi, c->d_acc,
                                          bkind, 1, de_stats, c->stream)
                    : f3g_launch_de(c->d_hist, bkind, use_count ? c->d_count : NULL, g.W, g.H, g.oversample, k1, k2,
                                    cp.estimator_curve, mfc, mfi, c->d_de_w, R, c->d_acc, bkind, c->stream);
      launches += bands ? 2 : 1;
      if (e) {
        f3g_set_error("density estimation launch failed: %s", cudaGetErrorString((cudaError_t)e));
        goto done;
      }
    } else {
      int e = f3g_launch_logscale(c->d_hist, bkind, nb, k1, k2, c->d_acc, bkind, bits == 32 && !f3g_opts.float_buckets,
                                  c->stream);
      launches++;
      if (e) {
        f3g_set_error("log scaling launch failed: %s", cudaGetErrorString((cudaError_t)e));
        goto done;
      }
    }
    CK(cudaEventRecord(c->ev[3], c->stream));
    CK(cudaStreamSynchronize(c->stream));
    {
      float ms = 0;
      cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]);
      t_de += ms;
    }
    if (spec->progress) {
      int r = spec->progress(spec->progress_parameter, 100.0 * (batch + 1) / nbatches, 1, 0.0);
      if (r == 1) {
        rv = 0;
        goto done;
      }
    }
  }

  if (io && io->accum_out) {
    size_t n4 = (size_t)nb * 4;
    void *ha = malloc((size_t)nb * bsz);
    CK(cudaStreamSynchronize(c->stream));
    cudaMemcpy(ha, c->d_acc, (size_t)nb * bsz, cudaMemcpyDeviceToHost);
    for (size_t k = 0; k < n4; k++)
      io->accum_out[k] = bkind == F3G_BK_F64 ? ((double *)ha)[k] : (double)((float *)ha)[k];
    free(ha);
  }

tail_fused:;
  {
    /* ---- filter + tonemap + pack (rect.c:1067-1247) ---- */
    F3GTonemap tp;
    double gm = 1.0 / (gamma / vib_gam_n);
    tp.g = (float)gm;
    tp.linrange = (float)cp.gam_lin_thresh;
    tp.funcval = (float)pow(cp.gam_lin_thresh, gm);
    tp.vibrancy = (float)(vibrancy / vib_gam_n);
    tp.highpow = (float)highpow;
    for (int k = 0; k < 3; k++) tp.background[k] = (float)(background[k] / (vib_gam_n / 256.0));
    tp.nchan = nchan;
    tp.transp = transp;
    tp.bpc = spec->bytes_per_channel;
    tp.trunc_acc = bits == 32 && !f3g_opts.float_buckets;
    CK(cudaEventRecord(c->ev[4], c->stream));
    int e;
    if (fde == 2) {
      e = f3g_launch_de_bands(c->d_hist, bkind, fde_count ? c->d_count : NULL, g.W, g.H, g.oversample, fde_k1, fde_k2,
                              fde_curve, fde_mfc, fde_mfi, c->d_de_w, fde_R, c->d_fi, c->d_acc, F3G_BK_F32, 0,
                              de_stats, c->stream);
      launches += 2;
      if (!e) {
        e = f3g_launch_acc_filter(c->d_acc, g.W, g.H, g.de_offset, g.oversample, c->d_filter, g.filter_width,
                                  g.image_width, g.image_height, c->d_out, spec->earlyclip, &tp, c->stream);
        launches++;
      }
    } else if (fde) {
      e = f3g_launch_de_fused_tile(c->d_hist, bkind, fde_count ? c->d_count : NULL, g.W, g.H, g.oversample, fde_k1,
                              fde_k2, fde_curve, fde_mfc, fde_mfi, c->d_de_w, fde_R, g.de_offset,
                              c->d_filter, g.filter_width, g.image_width, g.image_height, c->d_out, spec->earlyclip,
                              &tp, de_tile, c->stream);
      launches++;
    } else if (fused_tail && !de_used_any) {
      double k1 = (cp.contrast * cp.brightness * 255.0 * 268.0 * 1.0) / 256;
      double area = g.image_width * g.image_height / (ppux * ppuy);
      double k2 = (g.oversample * g.oversample * 1) / (cp.contrast * area * F3G_WHITE * sample_density * sumfilt);
      e = f3g_launch_fused_log_filter(c->d_hist, bkind, g.W, g.H, k1, k2, g.de_offset, g.oversample, c->d_filter,
                                      g.filter_width, g.image_width, g.image_height, c->d_out, spec->earlyclip, &tp,
                                      c->stream);
      launches++;
    } else {
      e = 0;
      if (spec->earlyclip) {
        e = f3g_launch_earlyclip(c->d_acc, bkind, nb, &tp, c->stream);
        launches++;
      }
      if (!e) {
        e = f3g_launch_filter_tonemap(c->d_acc, bkind, g.W, g.de_offset, g.oversample, c->d_filter, g.filter_width,
                                      g.image_width, g.image_height, c->d_out, spec->earlyclip, &tp, c->stream);
        launches++;
      }
    }
    if (e) {
      f3g_set_error("filter/tonemap launch failed: %s", cudaGetErrorString((cudaError_t)e));
      goto done;
    }
    CK(cudaEventRecord(c->ev[5], c->stream));
    if (io && io->keep_on_device) {
      /* the image stays in c->d_out for the caller's next device step */
      float ms = 0;
      CK(cudaEventSynchronize(c->ev[5]));
      cudaEventElapsedTime(&ms, c->ev[4], c->ev[5]);
      t_tail = ms;
      if (pending_ctr) {
        float mi = 0;
        cudaEventElapsedTime(&mi, c->ev[0], c->ev[1]);
        t_iter += mi;
        stats->badvals += (double)c->h_ctr->badvals;
        plotted += (double)c->h_ctr->plotted;
        if (c->h_ctr->error) {
          f3g_set_error("iterate kernel: a point-exchange wait timed out");
          goto done;
        }
      }
      rv = 0;
      goto done;
    }
    size_t row = (size_t)g.image_width * nchan * spec->bytes_per_channel;
    unsigned char *dst = (unsigned char *)out;
    if (field == flam3_field_odd) dst += row;
    size_t dpitch = (size_t)g.out_width * nchan * spec->bytes_per_channel;
    const size_t img_bytes = row * (size_t)g.image_height;
    /* through pinned staging: a DMA at full speed, then one host copy (a
     * direct copy into pageable memory runs at a fraction of the link) */
    if (img_bytes > c->h_img_bytes) {
      if (c->h_img) cudaFreeHost(c->h_img);
      c->h_img = NULL;
      c->h_img_bytes = 0;
      if (cudaMallocHost((void **)&c->h_img, img_bytes) == cudaSuccess) c->h_img_bytes = img_bytes;
    }
    if (c->h_img) {
      CK(cudaMemcpyAsync(c->h_img, c->d_out, img_bytes, cudaMemcpyDeviceToHost, c->stream));
      CK(cudaStreamSynchronize(c->stream));
      if (dpitch == row) memcpy(dst, c->h_img, img_bytes);
      else
        for (int y = 0; y < g.image_height; y++) memcpy(dst + (size_t)y * dpitch, c->h_img + (size_t)y * row, row);
    } else {
      CK(cudaMemcpy2DAsync(dst, dpitch, c->d_out, row, row, (size_t)g.image_height, cudaMemcpyDeviceToHost,
                           c->stream));
      CK(cudaStreamSynchronize(c->stream));
    }
    d2h += (double)img_bytes;
    float ms = 0;
    cudaEventElapsedTime(&ms, c->ev[4], c->ev[5]);
    t_tail = ms;
    if (pending_ctr) {
      float mi = 0;
      cudaEventElapsedTime(&mi, c->ev[0], c->ev[1]);
      t_iter += mi;
      stats->badvals += (double)c->h_ctr->badvals;
      plotted += (double)c->h_ctr->plotted;
      if (c->h_ctr->error) {
        f3g_set_error("iterate kernel: a point-exchange wait timed out");
        goto done;
      }
    }
  }
  rv = 0;
  if (de_stats) {
    unsigned long long w[4];
    if (cudaMemcpy(w, c->d_de_stats, sizeof(w), cudaMemcpyDeviceToHost) == cudaSuccess)
      for (int i = 0; i < 3; i++) c->de_work[i] = (double)w[i];
  }

done:
  c->timings[0] = t_iter;
  c->timings[1] = t_de;
  c->timings[2] = t_tail;
  c->timings[3] = 1e3 * (now_s() - wall0);
  c->timings[4] = launches;
  c->timings[5] = h2d;
  c->timings[6] = d2h;
  c->timings[7] = plotted;
  free(filter);
  free(tfilter);
  free(tdeltas);
  free(de_w);
  free(de_c);
  f3g_genome_free(&cp);
  stats->render_seconds = (int)(time(NULL) - tstart);
  if (rv) fprintf(stderr, "flam3gpu: %s\n", flam3gpu_last_error());
  return rv;
}

int flam3gpu_render(flam3_frame *f, void *out, int field, int nchan, int transp, stat_struct *stats) {
  return flam3gpu_render_ex(f, out, field, nchan, transp, stats, NULL);
}

double flam3gpu_render_memory_required(flam3_frame *f) {
  flam3_genome *cp = &f->genomes[0];
  int bsz = f->bits == 64 ? 32 : 16;
  double nb = (double)cp->spatial_oversample * cp->spatial_oversample * (double)cp->width * cp->height;
  return nb * bsz * 2.0 + (double)cp->width * cp->height * 4 * 2;
}

int flam3gpu_plan_passes(flam3_frame *f, int on_device, void *passes, int max_passes) {
  f3g_ctx *c = f3g_get_ctx();
  if (!c) {
    f3g_set_error("no CUDA device available");
    return -1;
  }
  const flam3gpu_options saved = f3g_opts;
  f3g_opts.host_plan = !on_device;
  c->plan_only_out = passes;
  c->plan_only_max = max_passes;
  c->plan_only_n = 0;
  stat_struct st;
  unsigned char unused; /* the render stops after planning: the image buffer is never written */
  const int r = flam3gpu_render_ex(f, &unused, 0, 3, 0, &st, NULL);
  c->plan_only_out = NULL;
  f3g_opts = saved;
  return r ? -1 : c->plan_only_n;
}

int flam3gpu_last_de_work(double w[3]) {
  f3g_ctx *c = f3g_get_ctx();
  if (!c) return 1;
  for (int i = 0; i < 3; i++) w[i] = c->de_work[i];
  return 0;
}

int flam3gpu_last_timings(double t[8]) {
  f3g_ctx *c = f3g_get_ctx();
  if (!c) return 1;
  for (int i = 0; i < 8; i++) t[i] = c->timings[i];
  return 0;
}

/* GPU bucket accumulation of a given point stream (rect.c:411-516) into a
 * FP64 histogram of the render geometry; the result is added to `hist`
 * (5 doubles per bucket). */
int f3g_accumulate_impl(flam3_frame *f, int field, const double *points, long n, double *hist, int *hist_w,
                        int *hist_h) {
  f3g_ctx *c = f3g_get_ctx();
  if (!c) {
    f3g_set_error("no CUDA device available");
    return 1;
  }
  flam3_genome cp;
  memset(&cp, 0, sizeof(cp));
  int rv = 1;
  double *d_pts = NULL, *h4 = NULL, *hc = NULL;
  void *d_b = NULL, *d_c = NULL;
  size_t cap_b = 0, cap_c = 0;
  if (f3g_interpolate(f->genomes, f->ngenomes, f->time, &cp)) return 1;
  f3g_geom g;
  if (compute_geom(f, &cp, field, NULL, &g)) goto done;
  *hist_w = g.W;
  *hist_h = g.H;
  if (!hist) {
    rv = 0;
    goto done;
  }
  if (f3g_ensure_host_pass_one(c)) goto done;
  F3GPass *p = c->h_passes;
  memset(p, 0, sizeof(*p));
  const char *ap = getenv("apo_palette");
  p->cmap_size = 256 - (ap ? atoi(ap) : 0);
  if (p->cmap_size < 2 || p->cmap_size > 256) {
    f3g_set_error("apo_palette gives a colour map of %d entries", p->cmap_size);
    goto done;
  }
  p->palette_mode = cp.palette_mode;
  for (int j = 0; j < 256; j++)
    for (int k = 0; k < 4; k++) p->dmap[j][k] = (float)(cp.palette[j].color[k] * F3G_WHITE);
  double sd, px, py;
  if (set_camera(f, &cp, field, &g, p, &sd, &px, &py)) goto done;
  long long nb = (long long)g.W * g.H;
  if (f3g_ensure(&d_b, &cap_b, (size_t)nb * 32) || f3g_ensure(&d_c, &cap_c, (size_t)nb * 8)) goto done;
  CK(cudaMemset(d_b, 0, (size_t)nb * 32));
  CK(cudaMemset(d_c, 0, (size_t)nb * 8));
  p->buckets = d_b;
  p->count = d_c;
  p->bucket_kind = F3G_BK_F64;
  if (f3g_ensure((void **)&c->d_passes, &c->passes_bytes, sizeof(F3GPass))) goto done;
  CK(cudaMemcpy(c->d_passes, p, sizeof(F3GPass), cudaMemcpyHostToDevice));
  if (n > 0) {
    CK(cudaMalloc((void **)&d_pts, (size_t)n * 4 * sizeof(double)));
    CK(cudaMemcpy(d_pts, points, (size_t)n * 4 * sizeof(double), cudaMemcpyHostToDevice));
    if (f3g_launch_accumulate(c->d_passes, d_pts, n, c->stream)) {
      f3g_set_error("accumulate launch failed");
      goto done;
    }
    CK(cudaStreamSynchronize(c->stream));
  }
  h4 = (double *)malloc((size_t)nb * 32);
  hc = (double *)malloc((size_t)nb * 8);
  CK(cudaMemcpy(h4, d_b, (size_t)nb * 32, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(hc, d_c, (size_t)nb * 8, cudaMemcpyDeviceToHost));
  for (long long b = 0; b < nb; b++) {
    for (int k = 0; k < 4; k++) hist[5 * b + k] += h4[4 * b + k];
    hist[5 * b + 4] += hc[b];
  }
  rv = 0;
done:
  cudaFree(d_pts);
  cudaFree(d_b);
  cudaFree(d_c);
  free(h4);
  free(hc);
  f3g_genome_free(&cp);
  return rv;
}

/* Thin accessors used by the no-allocation entry point (f3g_noalloc.cu). */
int f3g_geometry(flam3_frame *spec, const flam3_genome *cp, int field, double **filter, f3g_geom *g) {
  return compute_geom(spec, cp, field, filter, g);
}

int f3g_camera(flam3_frame *spec, const flam3_genome *cp, int field, const f3g_geom *g, F3GPass *p,
               double *sample_density, double *ppux, double *ppuy) {
  return set_camera(spec, cp, field, g, p, sample_density, ppux, ppuy);
}

void f3g_pass_key(flam3_frame *spec, uint32_t key[2]) { consume_rc(spec, key); }

/* the ISAAC word stream of a caller's context (isaac.h:49-52), for host
 * entry points that draw from it */
unsigned long f3g_irand(randctx *r) { return irand(r); }

