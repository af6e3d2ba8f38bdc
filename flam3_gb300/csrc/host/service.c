/*
 * service.c -- batched and served rendering (flam3_gpu_service.h).
 *
 * A job is one flam3_render request.  It is planned on the submitting
 * thread exactly as flam3gpu_render plans a render (render.c, after
 * rect.c:529-1286): genome interpolation per temporal sample, pass tables,
 * filters, k1/k2 per batch, tonemap constants, and the caller's ISAAC
 * context advanced as the reference advances it.  The service thread then
 *
 *   admits jobs while their device buffers fit the HBM budget (one
 *     stream-ordered allocation per job from a device memory pool, pass
 *     tables and filters uploaded on an upload stream);
 *   issues rounds: a round takes the next chunks of every admitted job's
 *     current batch, shortest remaining job first, up to a sample budget,
 *     and runs them in one persistent iterate launch per kernel class;
 *     rounds alternate over several low-priority streams so the last
 *     blocks of one round overlap the first blocks of the next;
 *   gives every job whose batch finished in a round its tail (density
 *     estimation, filter, tonemap, copy-out; or the per-batch accumulation
 *     of multi-batch renders) on a high-priority stream, all such jobs of a
 *     round in one CUDA graph with one branch per job;
 *   completes jobs when their tail has run: copies the image to the
 *     caller's buffer and fills the stats.
 *
 * The chunking of a job (samples per chain, chunk count per temporal
 * sample) and its random streams are fixed at planning, so rounds only
 * decide when chunks run, never what they compute.
 */
#define _GNU_SOURCE
#include <math.h>
#include <pthread.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "f3g_host.h"
#include "flam3_gpu_service.h"

#define F3G_WHITE 255.0
#define NRB 4         /* round buffers (at most NRB-1 rounds in flight) */
#define NTAIL 8       /* tail slots */
#define NBRANCH 4     /* parallel branches of a tail graph */
#define NCLASS 4      /* kernel classes: full variations x xform-choice mode */
#define NGRAPH 32     /* cached executable tail graphs */

enum { J_QUEUED = 0, J_ACTIVE, J_DONE, J_FAILED };
enum { P_ITER = 0, P_TAIL, P_WAIT_UP };

typedef struct {
  int de_on, mfc, mfi, R, nk, use_count, full, mode, S, S_tail, blocks;
  double k1, k2, curve;
  size_t kinfo_off; /* floats into the job's kinfo table */
  long long chunks; /* chunks of the batch (all temporal samples) */
} batch_plan;

typedef struct f3g_job {
  uint64_t ticket;
  int state, rv;
  char err[256];
  /* request */
  flam3_frame spec;
  void *out;
  int field, nchan, transp;
  stat_struct stats;
  /* plan */
  f3g_geom g;
  int bkind;
  size_t bsz, csz;
  long long nb;
  int nbatches, ntemporal, threads, precision;
  int fused_de, fused_log, need_acc, count_any, tile, band_de;
  int aborted; /* the progress callback asked to abort: no more rounds, no tail, output untouched */
  double sort_key; /* the round's ordering key (cfg.order 1 and 2) */
  F3GPass *h_passes;      /* nbatches * ntemporal (freed once uploaded) */
  long long *pass_tail;   /* each pass's first short chunk (F3GPass.chunk_tail), kept for round building */
  long long *pass_prefix; /* per batch: ntemporal+1 chunk offsets, concatenated */
  batch_plan *bp;
  float *h_kinfo;
  size_t nkinfo;
  float *h_filter;
  F3GTonemap tp;
  size_t out_bytes, dev_bytes;
  double total_samples, done_samples;
  /* device */
  char *d_base;
  void *d_hist, *d_count, *d_acc;
  uint8_t *d_fi; /* band DE: kernel index per bucket */
  unsigned char *d_out;
  F3GPass *d_passes;
  float *d_filter, *d_kinfo;
  unsigned long long *d_counts;
  /* pinned staging for the result */
  unsigned char *h_out;
  unsigned long long *h_counts;
  /* progress */
  int batch, phase, tail_slot, rounds;
  long long cursor;
  int pass_hint;
  double t_submit, t_admit, t_first, t_done;
  struct f3g_job *next; /* pending queue */
} f3g_job;

typedef struct {
  F3GItem *h_items, *d_items;
  long long *h_prefix, *d_prefix;
  size_t cap; /* items */
  F3GCounters *d_ctr, *h_ctr; /* one per class; pinned copy read when the round completes */
  cudaEvent_t ev, t0, t1; /* completion; timing of the round's launches */
  int in_use;
} round_buf;

typedef struct {
  cudaEvent_t ev, t0; /* completion (timed) and start of the slot's tail work */
  int in_use, njobs;
  f3g_job **jobs;
  int cap;
} tail_slot;

typedef struct {
  char sig[512];
  cudaGraphExec_t exec;
  unsigned long long used;
} graph_entry;

struct flam3gpu_service {
  flam3gpu_service_config cfg;
  int device, nsm;
  cudaStream_t s_up, s_tail, s_iter[8], s_br[NBRANCH];
  cudaEvent_t ev_last[8], ev_fork, ev_join[NBRANCH];
  cudaMemPool_t pool;
  pthread_t thread;
  pthread_mutex_t mu;
  pthread_cond_t cv_work, cv_done;
  int stop, thread_started;
  /* jobs by ticket (ticket - 1) */
  f3g_job **jobs;
  size_t njobs_cap;
  uint64_t next_ticket;
  f3g_job *pend_head, *pend_tail;
  f3g_job **active;
  int nactive, active_cap;
  size_t budget, used, peak;
  round_buf rb[NRB];
  unsigned long long round_no;
  int paused; /* jobs the last round left out because their progress callback paused them */
  char kernel_err[128]; /* set when an iterate launch reported an error: jobs finishing later fail */
  int inflight[NRB];
  tail_slot ts[NTAIL];
  unsigned long long tail_no;
  graph_entry graphs[NGRAPH];
  unsigned long long graph_clock;
  /* counters */
  double c_done, c_failed, c_rounds, c_launches, c_graphs, c_inst, c_plotted, c_h2d, c_d2h;
  double h_admit, h_round, h_tail, h_done, h_wait; /* service-thread seconds by activity */
  double g_iter, g_tail;                           /* device seconds of iterate rounds and of tails */
  double c_samples;                                /* samples issued in iterate rounds */
  double t_first_admit, t_last_done;
};

/* Pinned host staging buffers, kept for reuse by every service of the
 * process (allocating and freeing pinned memory is slow and freeing it
 * synchronizes the device); size classes are powers of two from 64 KiB. */
struct pin_buf {
  void *p;
  struct pin_buf *next;
};
static struct pin_buf *g_pin_free[40];
static pthread_mutex_t g_pin_mu = PTHREAD_MUTEX_INITIALIZER;

static int pin_class(size_t n) {
  int c = 16;
  while (((size_t)1 << c) < n && c < 39) c++;
  return c;
}

static void *pin_get(size_t n) {
  const int c = pin_class(n);
  pthread_mutex_lock(&g_pin_mu);
  struct pin_buf *b = g_pin_free[c];
  if (b) g_pin_free[c] = b->next;
  pthread_mutex_unlock(&g_pin_mu);
  if (b) {
    void *p = b->p;
    free(b);
    return p;
  }
  void *p = NULL;
  if (cudaMallocHost(&p, (size_t)1 << c) != cudaSuccess) return NULL;
  return p;
}

static void pin_put(void *p, size_t n) {
  if (!p) return;
  struct pin_buf *b = (struct pin_buf *)malloc(sizeof(*b));
  if (!b) return; /* leaked rather than freed mid-flight */
  const int c = pin_class(n);
  b->p = p;
  pthread_mutex_lock(&g_pin_mu);
  b->next = g_pin_free[c];
  g_pin_free[c] = b;
  pthread_mutex_unlock(&g_pin_mu);
}

static double now_s(void) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return t.tv_sec + 1e-9 * t.tv_nsec;
}

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

/* the DE "tile" value that selects density estimation by owner bands (the
 * fused tile kernel takes tile edges of 4 and more) */
#define DE_BANDS 1

/* ------------------------------------------------------------------ tuning */

typedef struct {
  char key[96];
  int S, tile;
} tune_entry;

static tune_entry *g_tune = NULL;
static int g_ntune = 0;
static pthread_mutex_t g_tune_mu = PTHREAD_MUTEX_INITIALIZER;

static void tune_key(const f3g_job *j, char *key, size_t n) {
  double spp = j->total_samples / ((double)j->g.image_width * j->g.image_height);
  int qb = (int)floor(log2(spp > 1 ? spp : 1));
  int R = j->bp ? j->bp[0].R : 0;
  snprintf(key, n, "%dx%d/b%d/ss%d/R%d/q%d/nt%d", j->g.image_width, j->g.image_height, j->bkind == F3G_BK_F64 ? 64 : 32,
           j->g.oversample, R, qb, j->ntemporal);
}

static int tune_lookup(const char *key, int *S, int *tile) {
  int found = 0;
  pthread_mutex_lock(&g_tune_mu);
  for (int i = 0; i < g_ntune; i++)
    if (!strcmp(g_tune[i].key, key)) {
      *S = g_tune[i].S;
      *tile = g_tune[i].tile;
      found = 1;
      break;
    }
  pthread_mutex_unlock(&g_tune_mu);
  return found;
}

static void tune_store(const char *key, int S, int tile) {
  pthread_mutex_lock(&g_tune_mu);
  int i;
  for (i = 0; i < g_ntune; i++)
    if (!strcmp(g_tune[i].key, key)) break;
  if (i == g_ntune) {
    tune_entry *t = (tune_entry *)realloc(g_tune, (size_t)(g_ntune + 1) * sizeof(tune_entry));
    if (!t) {
      pthread_mutex_unlock(&g_tune_mu);
      return;
    }
    g_tune = t;
    g_ntune++;
    snprintf(g_tune[i].key, sizeof(g_tune[i].key), "%s", key);
  }
  g_tune[i].S = S;
  g_tune[i].tile = tile;
  pthread_mutex_unlock(&g_tune_mu);
}

/* ---------------------------------------------------------------- planning */

static void job_free_plan(f3g_job *j) {
  free(j->h_passes);
  free(j->pass_tail);
  j->pass_tail = NULL;
  free(j->pass_prefix);
  free(j->bp);
  free(j->h_kinfo);
  free(j->h_filter);
  j->h_passes = NULL;
  j->pass_prefix = NULL;
  j->bp = NULL;
  j->h_kinfo = NULL;
  j->h_filter = NULL;
  if (j->spec.genomes) {
    for (int i = 0; i < j->spec.ngenomes; i++) f3g_genome_free(&j->spec.genomes[i]);
    free(j->spec.genomes);
    j->spec.genomes = NULL;
  }
}

/* The planning of flam3gpu_render_ex (render.c), recorded instead of run.
 * Works on the job's copy of the frame; advances job->spec.rc. */
static int plan_job(f3g_job *j, int nsm, int use_tuning, int force_S, int force_tile) {
  flam3_frame *spec = &j->spec;
  const int bits = spec->bits, field = j->field, nchan = j->nchan;
  if (bits != 32 && bits != 33 && bits != 64) {
    f3g_set_error("flam3: bits must be 32, 33, or 64 not %d.", bits);
    return 1;
  }
  if (nchan != 3 && nchan != 4) {
    f3g_set_error("nchan must be 3 or 4, not %d", nchan);
    return 1;
  }
  if (spec->bytes_per_channel != 1 && spec->bytes_per_channel != 2) {
    f3g_set_error("bytes_per_channel must be 1 or 2, not %d", spec->bytes_per_channel);
    return 1;
  }
  const char *ap = getenv("apo_palette");
  const int cmap_size = 256 - (ap ? atoi(ap) : 0);
  if (cmap_size < 2 || cmap_size > 256) {
    f3g_set_error("apo_palette gives a colour map of %d entries", cmap_size);
    return 1;
  }
  flam3_genome cp;
  memset(&cp, 0, sizeof(cp));
  if (f3g_interpolate(spec->genomes, spec->ngenomes, spec->time, &cp)) return 1;
  int rv = 1;
  double *filter = NULL, *tfilter = NULL, *tdeltas = NULL, *de_w = NULL, *de_c = NULL;
  f3g_pass_info *info = NULL;
  const int nbatches = cp.nbatches, ntemporal = cp.ntemporal_samples;
  const double highpow = cp.highlight_power;
  j->nbatches = nbatches;
  j->ntemporal = ntemporal;
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
  if (f3g_geometry(spec, &cp, field, &filter, &j->g)) goto done;
  const f3g_geom g = j->g;
  const double sumfilt = f3g_temporal_filter(nbatches * ntemporal, cp.temporal_filter_type, cp.temporal_filter_exp,
                                             cp.temporal_filter_width, &tfilter, &tdeltas);
  j->nb = (long long)g.W * g.H;
  j->bkind = bits == 64 ? F3G_BK_F64 : F3G_BK_F32;
  j->bsz = j->bkind == F3G_BK_F64 ? 32 : 16;
  j->csz = j->bkind == F3G_BK_F64 ? 8 : 4;
  int need_count = 0;
  for (int i = 0; i < nbatches * ntemporal; i++)
    if (tfilter[i] != 1.0) need_count = 1;
  j->threads = f3g_opts.threads_per_block > 0 ? f3g_opts.threads_per_block : 256;
  j->precision = f3g_opts.iter_precision == 64 ? 64 : 32;
  const int npass = nbatches * ntemporal;
  j->h_passes = (F3GPass *)calloc((size_t)npass, sizeof(F3GPass));
  j->pass_tail = (long long *)calloc((size_t)npass, sizeof(long long));
  j->pass_prefix = (long long *)calloc((size_t)nbatches * (ntemporal + 1), sizeof(long long));
  j->bp = (batch_plan *)calloc((size_t)nbatches, sizeof(batch_plan));
  j->h_filter = (float *)malloc(F3G_FILTER_FLOATS(g.filter_width) * sizeof(float));
  info = (f3g_pass_info *)calloc((size_t)ntemporal, sizeof(f3g_pass_info));
  if (!j->h_passes || !j->pass_tail || !j->pass_prefix || !j->bp || !j->h_filter || !info) {
    f3g_set_error("host memory exhausted");
    goto done;
  }
  for (size_t i = 0; i < F3G_FILTER_FLOATS(g.filter_width); i++) j->h_filter[i] = (float)filter[i];
  double vibrancy = 0.0, gamma = 0.0, background[3] = {0, 0, 0};
  int vib_gam_n = 0;
  double ppux = 0, ppuy = 0, sample_density = 0;
  j->stats.num_iters = 0;
  j->stats.badvals = 0;
  j->total_samples = 0;
  for (int batch = 0; batch < nbatches; batch++) {
    batch_plan *b = &j->bp[batch];
    const double de_time = spec->time + tdeltas[batch * ntemporal];
    int mfc = 0, mfi = 0, ks = 0;
    free(de_w);
    free(de_c);
    de_w = de_c = NULL;
    if (f3g_interpolate(spec->genomes, spec->ngenomes, de_time, &cp)) goto done;
    if (cp.estimator < 0.0 || cp.estimator_minimum < 0.0) {
      f3g_set_error("density estimator filter widths must be >= 0");
      goto done;
    }
    if (bits <= 32 && cp.estimator > 0.0) cp.estimator = 0.0; /* as render.c: no DE with 32-bit buffers */
    if (cp.estimator > 0.0) {
      ks = f3g_de_filters(cp.estimator, cp.estimator_minimum, cp.estimator_curve, g.oversample, &mfc, &mfi, &de_w,
                          &de_c);
      if (ks < 0) goto done;
    }
    b->de_on = mfi > 0;
    b->mfc = mfc;
    b->mfi = mfi;
    if (b->de_on) {
      b->R = (int)ceil(de_w[0]) - 1;
      if (b->R > f3g_de_max_reach()) {
        f3g_set_error("density estimation radius %d exceeds the library's limit %d", b->R, f3g_de_max_reach());
        goto done;
      }
      b->nk = mfi + 1;
      float *nk = (float *)realloc(j->h_kinfo, (j->nkinfo + (size_t)b->nk * 4) * sizeof(float));
      if (!nk) {
        f3g_set_error("host memory exhausted");
        goto done;
      }
      j->h_kinfo = nk;
      b->kinfo_off = j->nkinfo;
      f3g_de_kernel_info(mfi, ks, de_w, de_c, j->h_kinfo + j->nkinfo);
      j->nkinfo += (size_t)b->nk * 4;
    }
    long long batch_samples = 0;
    int full = 0, mode = 1;
    F3GPass *bpass = &j->h_passes[batch * ntemporal];
    if (f3g_build_batch_passes(spec, field, &g, batch, nbatches, ntemporal, tfilter, tdeltas, cmap_size, bpass, info))
      goto done;
    for (int ts = 0; ts < ntemporal; ts++) {
      F3GPass *p = &bpass[ts];
      const f3g_pass_info *in = &info[ts];
      need_count |= in->need_count;
      sample_density = in->sample_density;
      ppux = in->ppux;
      ppuy = in->ppuy;
      j->stats.num_iters += in->batch_size;
      p->bucket_kind = j->bkind;
      p->trunc_hits = bits <= 33 && !f3g_opts.float_buckets;
      batch_samples += p->samples;
      full |= p->full_variations;
      if (p->iter_mode == 0) mode = 0;
      vibrancy += in->vibrancy;
      gamma += in->gamma;
      background[0] += in->background[0];
      background[1] += in->background[1];
      background[2] += in->background[2];
      vib_gam_n++;
    }
    cp.contrast = info[ntemporal - 1].contrast;
    cp.brightness = info[ntemporal - 1].brightness;
    cp.gam_lin_thresh = info[ntemporal - 1].gam_lin_thresh;
    cp.estimator_curve = info[ntemporal - 1].estimator_curve;
    b->use_count = b->de_on && need_count;
    j->count_any |= b->use_count;
    b->full = full;
    b->mode = mode;
    b->k1 = (cp.contrast * cp.brightness * 255.0 * 268.0 * (1.0 / nbatches)) / 256;
    const double area = g.image_width * g.image_height / (ppux * ppuy);
    b->k2 = (g.oversample * g.oversample * nbatches) / (cp.contrast * area * F3G_WHITE * sample_density * sumfilt);
    b->curve = cp.estimator_curve;
    int occ = f3g_iterate_occupancy(j->precision, full, mode, j->threads);
    if (occ < 1) occ = 1;
    const int blocks = f3g_opts.blocks > 0 ? f3g_opts.blocks : nsm * occ;
    b->S = force_S > 0 ? force_S : f3g_chunk_samples(NULL, batch_samples, j->threads, blocks, spec->sub_batch_size);
    b->blocks = blocks;
    /* the plain render's chunking, so a served job draws the same samples */
    b->chunks = f3g_chunk_passes(&j->h_passes[batch * ntemporal], ntemporal, j->threads, blocks, b->S,
                                 j->pass_prefix + (size_t)batch * (ntemporal + 1));
    j->total_samples += (double)batch_samples;
  }
  /* tonemap constants (render.c tail; rect.c:1069-1081) */
  {
    F3GTonemap *tp = &j->tp;
    const double gm = 1.0 / (gamma / vib_gam_n);
    tp->g = (float)gm;
    tp->linrange = (float)cp.gam_lin_thresh;
    tp->funcval = (float)pow(cp.gam_lin_thresh, gm);
    tp->vibrancy = (float)(vibrancy / vib_gam_n);
    tp->highpow = (float)highpow;
    for (int k = 0; k < 3; k++) tp->background[k] = (float)(background[k] / (vib_gam_n / 256.0));
    tp->nchan = nchan;
    tp->transp = j->transp;
    tp->bpc = spec->bytes_per_channel;
    tp->trunc_acc = bits == 32 && !f3g_opts.float_buckets;
  }
  /* tail shape: one batch -> band DE + filter, or fused kernels; otherwise
   * accumulate per batch */
  j->tile = f3g_opts.de_kernel == 0 ? DE_BANDS : 16;
  int tS = 0, tTile = 0;
  if (use_tuning && force_S <= 0) {
    char key[96];
    tune_key(j, key, sizeof(key));
    if (tune_lookup(key, &tS, &tTile)) {
      if (tTile > 0) j->tile = tTile;
      if (tS > 0) {
        /* re-chunk with the tuned chain length */
        for (int batch = 0; batch < nbatches; batch++) {
          batch_plan *b = &j->bp[batch];
          b->S = tS;
          b->chunks = f3g_chunk_passes(&j->h_passes[batch * ntemporal], ntemporal, j->threads, b->blocks, tS,
                                       j->pass_prefix + (size_t)batch * (ntemporal + 1));
        }
      }
    }
  }
  if (force_tile > 0) j->tile = force_tile;
  /* the chunking the rounds need after the host passes are gone */
  for (int b = 0; b < nbatches; b++) {
    j->bp[b].S_tail = j->h_passes[b * ntemporal].S_tail;
    for (int ts = 0; ts < ntemporal; ts++) j->pass_tail[b * ntemporal + ts] = j->h_passes[b * ntemporal + ts].chunk_tail;
  }
  int de_any = 0, bands_ok = 1;
  for (int b = 0; b < nbatches; b++)
    if (j->bp[b].de_on) {
      de_any = 1;
      bands_ok &= f3g_de_bands_supported(j->bp[b].R, j->bp[b].mfi);
    }
  j->band_de = de_any && bands_ok && j->tile == DE_BANDS;
  if (j->tile == DE_BANDS && !j->band_de) j->tile = 16;
  if (nbatches == 1) {
    if (j->bp[0].de_on && j->band_de) {
      /* band DE into the accumulator, then the filter pass */
    } else if (j->bp[0].de_on) {
      j->fused_de = f3g_de_fused_smem_tile(g.oversample, g.filter_width, j->bp[0].R, j->bp[0].nk, j->tile) <=
                    220 * 1024;
      if (!j->fused_de && j->tile != 16 &&
          f3g_de_fused_smem_tile(g.oversample, g.filter_width, j->bp[0].R, j->bp[0].nk, 16) <= 220 * 1024) {
        j->tile = 16;
        j->fused_de = 1;
      }
    } else
      j->fused_log = 1;
  }
  j->need_acc = !(j->fused_de || j->fused_log);
  j->out_bytes = (size_t)g.image_width * g.image_height * nchan * spec->bytes_per_channel;
  j->dev_bytes = align256((size_t)npass * sizeof(F3GPass)) + align256((size_t)j->nb * j->bsz) +
                 (j->count_any ? align256((size_t)j->nb * j->csz) : 0) +
                 (j->need_acc ? align256((size_t)j->nb * j->bsz) : 0) + (j->band_de ? align256((size_t)j->nb) : 0) +
                 align256(j->out_bytes) +
                 align256(F3G_FILTER_FLOATS(g.filter_width) * sizeof(float)) +
                 align256(j->nkinfo * sizeof(float)) + 256;
  rv = 0;
done:
  free(filter);
  free(tfilter);
  free(tdeltas);
  free(de_w);
  free(de_c);
  free(info);
  f3g_genome_free(&cp);
  return rv;
}

/* ------------------------------------------------------------- the service */

void flam3gpu_service_default_config(flam3gpu_service_config *cfg) {
  memset(cfg, 0, sizeof(*cfg));
  cfg->tail_graphs = 1;
  cfg->streams = 1;
  cfg->use_tuning = 1;
  cfg->max_inflight = 2;
  cfg->tail_branches = 1;
  cfg->order = 1;
}

static void *service_main(void *arg);

static int job_remaining_cmp(const void *a, const void *b) {
  const f3g_job *x = *(f3g_job *const *)a, *y = *(f3g_job *const *)b;
  double rx = x->total_samples - x->done_samples, ry = y->total_samples - y->done_samples;
  if (rx < ry) return -1;
  if (rx > ry) return 1;
  return x->ticket < y->ticket ? -1 : (x->ticket > y->ticket);
}

/* higher sort key first, then arrival order */
static int job_key_cmp(const void *a, const void *b) {
  const f3g_job *x = *(f3g_job *const *)a, *y = *(f3g_job *const *)b;
  if (x->sort_key > y->sort_key) return -1;
  if (x->sort_key < y->sort_key) return 1;
  return x->ticket < y->ticket ? -1 : (x->ticket > y->ticket);
}

/* orders a round's candidate jobs by the service's policy (cfg.order) */
static void order_jobs(flam3gpu_service *s, f3g_job **cand, int nc) {
  if (s->cfg.order == 1) {
    /* response ratio: remaining time from the service's measured sample
     * rate (samples per second of iterate GPU time) */
    const double rate = s->g_iter > 0.05 && s->c_samples > 0 ? s->c_samples / s->g_iter : 4.0e10;
    const double now = now_s();
    for (int i = 0; i < nc; i++) {
      f3g_job *j = cand[i];
      double rem = (j->total_samples - j->done_samples) / rate;
      if (rem < 1e-4) rem = 1e-4;
      j->sort_key = (now - j->t_submit + rem) / rem;
    }
    qsort(cand, (size_t)nc, sizeof(f3g_job *), job_key_cmp);
  } else if (s->cfg.order == 2) {
    for (int i = 0; i < nc; i++) cand[i]->sort_key = -(double)cand[i]->ticket;
    qsort(cand, (size_t)nc, sizeof(f3g_job *), job_key_cmp);
  } else
    qsort(cand, (size_t)nc, sizeof(f3g_job *), job_remaining_cmp);
}

flam3gpu_service *flam3gpu_service_create(const flam3gpu_service_config *cfg_in) {
  f3g_clear_error();
  flam3gpu_service *s = (flam3gpu_service *)calloc(1, sizeof(*s));
  if (!s) {
    f3g_set_error("host memory exhausted");
    return NULL;
  }
  if (cfg_in) s->cfg = *cfg_in;
  else flam3gpu_service_default_config(&s->cfg);
  if (s->cfg.streams < 1) s->cfg.streams = 1;
  if (s->cfg.streams > 8) s->cfg.streams = 8;
  if (s->cfg.max_inflight < 1) s->cfg.max_inflight = 2;
  if (s->cfg.max_inflight > NRB - 1) s->cfg.max_inflight = NRB - 1;
  if (s->cfg.tail_branches < 1) s->cfg.tail_branches = 1;
  if (s->cfg.tail_branches > NBRANCH) s->cfg.tail_branches = NBRANCH;
  if (s->cfg.order < 0 || s->cfg.order > 2) s->cfg.order = 0;
  if (cudaGetDevice(&s->device) != cudaSuccess ||
      cudaDeviceGetAttribute(&s->nsm, cudaDevAttrMultiProcessorCount, s->device) != cudaSuccess) {
    f3g_set_error("no CUDA device available");
    free(s);
    return NULL;
  }
  int lo = 0, hi = 0;
  cudaDeviceGetStreamPriorityRange(&lo, &hi); /* hi is the numerically smaller, higher priority */
  int ok = cudaStreamCreateWithFlags(&s->s_up, cudaStreamNonBlocking) == cudaSuccess &&
           cudaStreamCreateWithPriority(&s->s_tail, cudaStreamNonBlocking, hi) == cudaSuccess &&
           cudaEventCreateWithFlags(&s->ev_fork, cudaEventDisableTiming) == cudaSuccess;
  for (int k = 0; ok && k < s->cfg.streams; k++)
    ok = cudaStreamCreateWithPriority(&s->s_iter[k], cudaStreamNonBlocking, lo) == cudaSuccess &&
         cudaEventCreateWithFlags(&s->ev_last[k], cudaEventDisableTiming) == cudaSuccess;
  for (int k = 0; ok && k < NBRANCH; k++)
    ok = cudaStreamCreateWithPriority(&s->s_br[k], cudaStreamNonBlocking, hi) == cudaSuccess &&
         cudaEventCreateWithFlags(&s->ev_join[k], cudaEventDisableTiming) == cudaSuccess;
  for (int k = 0; ok && k < NRB; k++)
    ok = cudaEventCreateWithFlags(&s->rb[k].ev, cudaEventDisableTiming | cudaEventBlockingSync) == cudaSuccess &&
         cudaEventCreate(&s->rb[k].t0) == cudaSuccess && cudaEventCreate(&s->rb[k].t1) == cudaSuccess &&
         cudaMalloc((void **)&s->rb[k].d_ctr, NCLASS * sizeof(F3GCounters)) == cudaSuccess &&
         cudaMallocHost((void **)&s->rb[k].h_ctr, NCLASS * sizeof(F3GCounters)) == cudaSuccess;
  for (int k = 0; ok && k < NTAIL; k++)
    ok = cudaEventCreateWithFlags(&s->ts[k].ev, cudaEventBlockingSync) == cudaSuccess &&
         cudaEventCreate(&s->ts[k].t0) == cudaSuccess;
  if (ok) ok = cudaDeviceGetDefaultMemPool(&s->pool, s->device) == cudaSuccess;
  if (ok) {
    uint64_t thr = ~(uint64_t)0;
    cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  if (ok) ok = f3g_de_prepare() == 0 && f3g_tail_prepare() == 0;
  if (!ok) {
    f3g_set_error("CUDA setup of the service failed: %s", cudaGetErrorString(cudaGetLastError()));
    flam3gpu_service_destroy(s);
    return NULL;
  }
  size_t freeb = 0, totalb = 0;
  cudaMemGetInfo(&freeb, &totalb);
  double want = s->cfg.hbm_budget_bytes > 0 ? s->cfg.hbm_budget_bytes : 150e9;
  if (want > 0.9 * (double)freeb) want = 0.9 * (double)freeb;
  s->budget = (size_t)want;
  pthread_mutex_init(&s->mu, NULL);
  pthread_cond_init(&s->cv_work, NULL);
  pthread_cond_init(&s->cv_done, NULL);
  if (pthread_create(&s->thread, NULL, service_main, s) != 0) {
    f3g_set_error("could not start the service thread");
    flam3gpu_service_destroy(s);
    return NULL;
  }
  s->thread_started = 1;
  return s;
}

int flam3gpu_service_submit(flam3gpu_service *s, flam3_frame *f, void *out, int field, int nchan, int transp,
                            uint64_t *ticket) {
  f3g_clear_error();
  if (!s || !f || !out || f->ngenomes < 1 || !f->genomes) {
    f3g_set_error("bad arguments to flam3gpu_service_submit");
    return 1;
  }
  f3g_job *j = (f3g_job *)calloc(1, sizeof(f3g_job));
  if (!j) {
    f3g_set_error("host memory exhausted");
    return 1;
  }
  j->t_submit = now_s();
  j->spec = *f; /* keeps the request's progress callback, called between rounds */
  j->spec.genomes = (flam3_genome *)calloc((size_t)f->ngenomes, sizeof(flam3_genome));
  for (int i = 0; i < f->ngenomes; i++) f3g_genome_copy(&j->spec.genomes[i], &f->genomes[i]);
  j->out = out;
  j->field = field;
  j->nchan = nchan;
  j->transp = transp;
  if (plan_job(j, s->nsm, s->cfg.use_tuning, 0, 0)) {
    job_free_plan(j);
    free(j);
    return 1;
  }
  f->rc = j->spec.rc; /* the caller's context advances as flam3_render advances it */
  pthread_mutex_lock(&s->mu);
  if ((size_t)s->next_ticket >= s->njobs_cap) {
    size_t nc = s->njobs_cap ? 2 * s->njobs_cap : 256;
    f3g_job **nj = (f3g_job **)realloc(s->jobs, nc * sizeof(f3g_job *));
    if (!nj) {
      pthread_mutex_unlock(&s->mu);
      job_free_plan(j);
      free(j);
      f3g_set_error("host memory exhausted");
      return 1;
    }
    memset(nj + s->njobs_cap, 0, (nc - s->njobs_cap) * sizeof(f3g_job *));
    s->jobs = nj;
    s->njobs_cap = nc;
  }
  j->ticket = ++s->next_ticket;
  s->jobs[j->ticket - 1] = j;
  j->state = J_QUEUED;
  if (s->pend_tail) s->pend_tail->next = j;
  else s->pend_head = j;
  s->pend_tail = j;
  pthread_cond_broadcast(&s->cv_work);
  pthread_mutex_unlock(&s->mu);
  *ticket = j->ticket;
  return 0;
}

/* device buffers and uploads of an admitted job (service thread) */
static int admit_job(flam3gpu_service *s, f3g_job *j) {
  char *base = NULL;
  cudaError_t e = cudaMallocFromPoolAsync((void **)&base, j->dev_bytes, s->pool, s->s_up);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return 2; /* no room now */
  }
  j->d_base = base;
  size_t off = 0;
#define CARVE(ptr, type, bytes)              \
  do {                                       \
    ptr = (type)(base + off);                \
    off += align256((size_t)(bytes));        \
  } while (0)
  const int npass = j->nbatches * j->ntemporal;
  CARVE(j->d_passes, F3GPass *, (size_t)npass * sizeof(F3GPass));
  CARVE(j->d_hist, void *, (size_t)j->nb * j->bsz);
  if (j->count_any) CARVE(j->d_count, void *, (size_t)j->nb * j->csz);
  if (j->need_acc) CARVE(j->d_acc, void *, (size_t)j->nb * j->bsz);
  if (j->band_de) CARVE(j->d_fi, uint8_t *, (size_t)j->nb);
  CARVE(j->d_out, unsigned char *, j->out_bytes);
  CARVE(j->d_filter, float *, F3G_FILTER_FLOATS(j->g.filter_width) * sizeof(float));
  CARVE(j->d_kinfo, float *, j->nkinfo * sizeof(float));
  CARVE(j->d_counts, unsigned long long *, 2 * sizeof(unsigned long long));
#undef CARVE
  for (int b = 0; b < j->nbatches; b++)
    for (int ts = 0; ts < j->ntemporal; ts++) {
      F3GPass *p = &j->h_passes[b * j->ntemporal + ts];
      p->buckets = j->d_hist;
      p->count = j->bp[b].use_count ? j->d_count : NULL;
      p->counters = j->d_counts;
    }
  int nxmax = 0;
  for (int i = 0; i < npass; i++)
    if (j->h_passes[i].num_xforms > nxmax) nxmax = j->h_passes[i].num_xforms;
  const size_t pass_bytes = F3G_PASS_BYTES(nxmax);
  int ok = cudaMemcpy2DAsync(j->d_passes, sizeof(F3GPass), j->h_passes, sizeof(F3GPass), pass_bytes, (size_t)npass,
                             cudaMemcpyHostToDevice, s->s_up) == cudaSuccess;
  ok = ok && cudaMemcpyAsync(j->d_filter, j->h_filter, F3G_FILTER_FLOATS(j->g.filter_width) * sizeof(float),
                             cudaMemcpyHostToDevice, s->s_up) == cudaSuccess;
  if (j->nkinfo)
    ok = ok && cudaMemcpyAsync(j->d_kinfo, j->h_kinfo, j->nkinfo * sizeof(float), cudaMemcpyHostToDevice,
                               s->s_up) == cudaSuccess;
  ok = ok && cudaMemsetAsync(j->d_hist, 0, (size_t)j->nb * j->bsz, s->s_up) == cudaSuccess;
  if (j->count_any) ok = ok && cudaMemsetAsync(j->d_count, 0, (size_t)j->nb * j->csz, s->s_up) == cudaSuccess;
  if (j->need_acc) ok = ok && cudaMemsetAsync(j->d_acc, 0, (size_t)j->nb * j->bsz, s->s_up) == cudaSuccess;
  ok = ok && cudaMemsetAsync(j->d_counts, 0, 2 * sizeof(unsigned long long), s->s_up) == cudaSuccess;
  if (ok) {
    j->h_out = (unsigned char *)pin_get(align256(j->out_bytes) + 2 * sizeof(unsigned long long));
    if (!j->h_out) ok = 0;
  }
  if (ok) j->h_counts = (unsigned long long *)(j->h_out + align256(j->out_bytes));
  /* rounds on every iterate stream start after the uploads */
  cudaEvent_t ev;
  if (ok && cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) == cudaSuccess) {
    cudaEventRecord(ev, s->s_up);
    for (int k = 0; k < s->cfg.streams; k++) cudaStreamWaitEvent(s->s_iter[k], ev, 0);
    cudaEventDestroy(ev);
  } else
    ok = 0;
  s->c_h2d += (double)npass * pass_bytes + (double)F3G_FILTER_FLOATS(j->g.filter_width) * 4 + j->nkinfo * 4.0;
  if (ok) {
    /* copies from pageable memory return once the data is staged: the host
     * tables are no longer needed */
    free(j->h_passes);
    free(j->h_filter);
    free(j->h_kinfo);
    j->h_passes = NULL;
    j->h_filter = NULL;
    j->h_kinfo = NULL;
  }
  if (!ok) {
    snprintf(j->err, sizeof(j->err), "device setup failed: %s", cudaGetErrorString(cudaGetLastError()));
    return 1;
  }
  j->phase = P_ITER;
  j->batch = 0;
  j->cursor = 0;
  j->pass_hint = 0;
  return 0;
}

static void release_job_device(flam3gpu_service *s, f3g_job *j) {
  if (j->d_base) {
    cudaFreeAsync(j->d_base, s->s_up);
    j->d_base = NULL;
    s->used -= j->dev_bytes;
  }
  if (j->h_out) {
    pin_put(j->h_out, align256(j->out_bytes) + 2 * sizeof(unsigned long long));
    j->h_out = NULL;
    j->h_counts = NULL;
  }
}

static void remove_active(flam3gpu_service *s, f3g_job *j) {
  for (int i = 0; i < s->nactive; i++)
    if (s->active[i] == j) {
      s->active[i] = s->active[--s->nactive];
      return;
    }
}

static void fail_job(flam3gpu_service *s, f3g_job *j, const char *msg) {
  if (msg && !j->err[0]) snprintf(j->err, sizeof(j->err), "%s", msg);
  if (j->d_base) {
    /* work of this job may still be queued: let it drain before the free */
    for (int k = 0; k < s->cfg.streams; k++) cudaStreamSynchronize(s->s_iter[k]);
    cudaStreamSynchronize(s->s_tail);
  }
  release_job_device(s, j);
  job_free_plan(j);
  pthread_mutex_lock(&s->mu);
  j->state = J_FAILED;
  j->rv = 1;
  j->t_done = now_s();
  s->c_failed++;
  pthread_cond_broadcast(&s->cv_done);
  pthread_mutex_unlock(&s->mu);
}

/* the tail of one job's current batch, on stream st */
static int enqueue_tail_ops(flam3gpu_service *s, f3g_job *j, cudaStream_t st, char *sig, size_t sigcap) {
  const batch_plan *b = &j->bp[j->batch];
  const int final = j->batch == j->nbatches - 1;
  const f3g_geom *g = &j->g;
  const flam3_frame *spec = &j->spec;
  int e = 0;
  char tag[32];
  if (j->band_de && j->nbatches == 1) {
    e = f3g_launch_de_bands(j->d_hist, j->bkind, b->use_count ? j->d_count : NULL, g->W, g->H, g->oversample, b->k1,
                            b->k2, b->curve, b->mfc, b->mfi, j->d_kinfo + b->kinfo_off, b->R, j->d_fi, j->d_acc,
                            F3G_BK_F32, 0, NULL, st);
    s->c_launches += 2;
    if (!e) {
      e = f3g_launch_acc_filter(j->d_acc, g->W, g->H, g->de_offset, g->oversample, j->d_filter, g->filter_width,
                                g->image_width, g->image_height, j->d_out, spec->earlyclip, &j->tp, st);
      s->c_launches++;
    }
    snprintf(tag, sizeof(tag), "B");
  } else if (j->fused_de) {
    e = f3g_launch_de_fused_tile(j->d_hist, j->bkind, b->use_count ? j->d_count : NULL, g->W, g->H, g->oversample,
                                 b->k1, b->k2, b->curve, b->mfc, b->mfi, j->d_kinfo + b->kinfo_off, b->R,
                                 g->de_offset, j->d_filter, g->filter_width, g->image_width, g->image_height,
                                 j->d_out, spec->earlyclip, &j->tp, j->tile, st);
    s->c_launches++;
    snprintf(tag, sizeof(tag), "F%d", j->tile);
  } else if (j->fused_log) {
    e = f3g_launch_fused_log_filter(j->d_hist, j->bkind, g->W, g->H, b->k1, b->k2, g->de_offset, g->oversample,
                                    j->d_filter, g->filter_width, g->image_width, g->image_height, j->d_out,
                                    spec->earlyclip, &j->tp, st);
    s->c_launches++;
    snprintf(tag, sizeof(tag), "L");
  } else {
    if (b->de_on && j->band_de)
      e = f3g_launch_de_bands(j->d_hist, j->bkind, b->use_count ? j->d_count : NULL, g->W, g->H, g->oversample, b->k1,
                              b->k2, b->curve, b->mfc, b->mfi, j->d_kinfo + b->kinfo_off, b->R, j->d_fi, j->d_acc,
                              j->bkind, 1, NULL, st);
    else if (b->de_on)
      e = f3g_launch_de(j->d_hist, j->bkind, b->use_count ? j->d_count : NULL, g->W, g->H, g->oversample, b->k1, b->k2,
                        b->curve, b->mfc, b->mfi, j->d_kinfo + b->kinfo_off, b->R, j->d_acc, j->bkind, st);
    else
      e = f3g_launch_logscale(j->d_hist, j->bkind, j->nb, b->k1, b->k2, j->d_acc, j->bkind, j->tp.trunc_acc, st);
    s->c_launches++;
    snprintf(tag, sizeof(tag), "%c", b->de_on ? 'D' : 'S');
    if (!e && !final) {
      if (cudaMemsetAsync(j->d_hist, 0, (size_t)j->nb * j->bsz, st) != cudaSuccess) e = 1;
      if (!e && j->count_any && cudaMemsetAsync(j->d_count, 0, (size_t)j->nb * j->csz, st) != cudaSuccess) e = 1;
      strcat(tag, "M");
    }
    if (!e && final) {
      if (spec->earlyclip) {
        e = f3g_launch_earlyclip(j->d_acc, j->bkind, j->nb, &j->tp, st);
        s->c_launches++;
        strcat(tag, "E");
      }
      if (!e) {
        e = f3g_launch_filter_tonemap(j->d_acc, j->bkind, g->W, g->de_offset, g->oversample, j->d_filter,
                                      g->filter_width, g->image_width, g->image_height, j->d_out, spec->earlyclip,
                                      &j->tp, st);
        s->c_launches++;
        strcat(tag, "T");
      }
    }
  }
  if (!e && final) {
    if (cudaMemcpyAsync(j->h_out, j->d_out, j->out_bytes, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(j->h_counts, j->d_counts, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st) !=
            cudaSuccess)
      e = 1;
    strcat(tag, "C");
    s->c_d2h += (double)j->out_bytes + 16;
  }
  if (sig && strlen(sig) + strlen(tag) + 2 < sigcap) {
    strcat(sig, tag);
    strcat(sig, ",");
  }
  return e;
}

static cudaGraphExec_t graph_for(flam3gpu_service *s, cudaGraph_t graph, const char *sig) {
  graph_entry *hit = NULL, *victim = &s->graphs[0];
  for (int i = 0; i < NGRAPH; i++) {
    graph_entry *g = &s->graphs[i];
    if (g->exec && !strcmp(g->sig, sig)) hit = g;
    if (!g->exec || (victim->exec && g->used < victim->used)) victim = g;
  }
  s->graph_clock++;
  if (hit) {
    cudaGraphExecUpdateResultInfo info;
    if (cudaGraphExecUpdate(hit->exec, graph, &info) == cudaSuccess) {
      hit->used = s->graph_clock;
      return hit->exec;
    }
    cudaGetLastError();
    cudaGraphExecDestroy(hit->exec);
    hit->exec = NULL;
    victim = hit;
  }
  if (victim->exec) cudaGraphExecDestroy(victim->exec);
  victim->exec = NULL;
  if (cudaGraphInstantiate(&victim->exec, graph, 0) != cudaSuccess) {
    cudaGetLastError();
    victim->exec = NULL;
    return NULL;
  }
  s->c_inst++;
  snprintf(victim->sig, sizeof(victim->sig), "%s", sig);
  victim->used = s->graph_clock;
  return victim->exec;
}

static void finish_slot(flam3gpu_service *s, tail_slot *t);

/* tails of the jobs whose current batch finished in the round just issued */
static void enqueue_tails_impl(flam3gpu_service *s, f3g_job **jobs, int n);
static void enqueue_tails(flam3gpu_service *s, f3g_job **jobs, int n) {
  const double t0 = now_s();
  enqueue_tails_impl(s, jobs, n);
  const double dt = now_s() - t0;
  s->h_tail += dt;
  s->h_round -= dt; /* reported apart from round building */
}

static void enqueue_tails_impl(flam3gpu_service *s, f3g_job **jobs, int n) {
  tail_slot *t = &s->ts[s->tail_no % NTAIL];
  if (t->in_use) {
    cudaEventSynchronize(t->ev);
    finish_slot(s, t);
  }
  if (t->cap < n) {
    f3g_job **nj = (f3g_job **)realloc(t->jobs, (size_t)n * sizeof(f3g_job *));
    if (!nj) {
      for (int i = 0; i < n; i++) {
        remove_active(s, jobs[i]);
        fail_job(s, jobs[i], "host memory exhausted");
      }
      return;
    }
    t->jobs = nj;
    t->cap = n;
  }
  for (int k = 0; k < s->cfg.streams; k++) cudaStreamWaitEvent(s->s_tail, s->ev_last[k], 0);
  cudaEventRecord(t->t0, s->s_tail);
  int err = 0, live = 0;
  for (int i = 0; i < n; i++) live += !jobs[i]->aborted;
  if (s->cfg.tail_graphs == 1) {
    /* one graph per job tail, keyed by its shape; the executable graph of a
     * shape is updated in place with the next job's buffers and sizes */
    for (int i = 0; i < n && !err; i++) {
      if (jobs[i]->aborted) continue; /* an aborted job has no tail */
      char sig[128];
      sig[0] = 0;
      cudaGraph_t graph = NULL;
      if (cudaStreamBeginCapture(s->s_tail, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        err = 1;
        break;
      }
      err = enqueue_tail_ops(s, jobs[i], s->s_tail, sig, sizeof(sig));
      if (cudaStreamEndCapture(s->s_tail, &graph) != cudaSuccess) err = 1;
      if (!err) {
        cudaGraphExec_t ex = graph_for(s, graph, sig);
        if (!ex || cudaGraphLaunch(ex, s->s_tail) != cudaSuccess) err = 1;
        s->c_graphs++;
      }
      if (graph) cudaGraphDestroy(graph);
    }
  } else if (s->cfg.tail_graphs == 2 && live) {
    /* one graph per round, one branch per job across tail_branches streams */
    char sig[512];
    sig[0] = 0;
    cudaGraph_t graph = NULL;
    if (cudaStreamBeginCapture(s->s_tail, cudaStreamCaptureModeThreadLocal) != cudaSuccess) err = 1;
    if (!err) {
      cudaEventRecord(s->ev_fork, s->s_tail);
      int used[NBRANCH] = {0};
      for (int i = 0; i < n && !err; i++) {
        if (jobs[i]->aborted) continue;
        const int k = i % s->cfg.tail_branches;
        if (!used[k]) {
          cudaStreamWaitEvent(s->s_br[k], s->ev_fork, 0);
          used[k] = 1;
        }
        char bs[16];
        snprintf(bs, sizeof(bs), "%d:", k);
        if (strlen(sig) + strlen(bs) + 1 < sizeof(sig)) strcat(sig, bs);
        err = enqueue_tail_ops(s, jobs[i], s->s_br[k], sig, sizeof(sig));
      }
      for (int k = 0; k < NBRANCH; k++)
        if (used[k]) {
          cudaEventRecord(s->ev_join[k], s->s_br[k]);
          cudaStreamWaitEvent(s->s_tail, s->ev_join[k], 0);
        }
      if (cudaStreamEndCapture(s->s_tail, &graph) != cudaSuccess) err = 1;
    }
    if (!err) {
      cudaGraphExec_t ex = graph_for(s, graph, sig);
      if (!ex || cudaGraphLaunch(ex, s->s_tail) != cudaSuccess) err = 1;
      s->c_graphs++;
    }
    if (graph) cudaGraphDestroy(graph);
  } else {
    for (int i = 0; i < n && !err; i++)
      if (!jobs[i]->aborted) err = enqueue_tail_ops(s, jobs[i], s->s_tail, NULL, 0);
  }
  if (err) {
    const char *m = cudaGetErrorString(cudaGetLastError());
    for (int i = 0; i < n; i++) {
      remove_active(s, jobs[i]);
      char msg[200];
      snprintf(msg, sizeof(msg), "tail launch failed: %s", m);
      fail_job(s, jobs[i], msg);
    }
    return;
  }
  cudaEventRecord(t->ev, s->s_tail);
  t->in_use = 1;
  t->njobs = n;
  for (int i = 0; i < n; i++) {
    t->jobs[i] = jobs[i];
    jobs[i]->phase = P_TAIL;
  }
  s->tail_no++;
}

/* copies a finished job's staged image to the caller's buffer (rows
 * interleaved for fields) and returns the staging buffer */
static void copy_out(f3g_job *j) {
  if (!j->h_out) return;
  if (j->aborted) { /* the reference leaves the output as it stands (rect.c:919-922) */
    pin_put(j->h_out, align256(j->out_bytes) + 2 * sizeof(unsigned long long));
    j->h_out = NULL;
    j->h_counts = NULL;
    return;
  }
  const f3g_geom *g = &j->g;
  const size_t row = (size_t)g->image_width * j->nchan * j->spec.bytes_per_channel;
  unsigned char *dst = (unsigned char *)j->out;
  if (j->field == flam3_field_odd) dst += row;
  const size_t dpitch = (size_t)g->out_width * j->nchan * j->spec.bytes_per_channel;
  if (dpitch == row) memcpy(dst, j->h_out, row * g->image_height);
  else
    for (int y = 0; y < g->image_height; y++) memcpy(dst + (size_t)y * dpitch, j->h_out + (size_t)y * row, row);
  pin_put(j->h_out, align256(j->out_bytes) + 2 * sizeof(unsigned long long));
  j->h_out = NULL;
  j->h_counts = NULL;
}

/* the job's tail has run: release its device memory and publish it; the
 * waiter copies the image out (off the service thread) */
static void complete_job(flam3gpu_service *s, f3g_job *j) {
  j->stats.badvals = (double)j->h_counts[0];
  s->c_plotted += (double)j->h_counts[1];
  j->stats.render_seconds = (int)(now_s() - j->t_submit);
  unsigned char *keep = j->h_out;
  j->h_out = NULL; /* release_job_device leaves the staging buffer to the waiter */
  release_job_device(s, j);
  j->h_out = keep;
  remove_active(s, j);
  job_free_plan(j);
  pthread_mutex_lock(&s->mu);
  j->state = J_DONE;
  j->rv = 0;
  j->t_done = now_s();
  s->t_last_done = j->t_done;
  s->c_done++;
  pthread_cond_broadcast(&s->cv_done);
  pthread_mutex_unlock(&s->mu);
}

static int rounds_in_flight(flam3gpu_service *s);

static void finish_slot(flam3gpu_service *s, tail_slot *t) {
  float ms = 0;
  if (cudaEventElapsedTime(&ms, t->t0, t->ev) == cudaSuccess) s->g_tail += ms * 1e-3;
  (void)rounds_in_flight(s); /* the rounds before this tail are done: read their error flags */
  for (int i = 0; i < t->njobs; i++) {
    f3g_job *j = t->jobs[i];
    if (s->kernel_err[0]) {
      remove_active(s, j);
      fail_job(s, j, s->kernel_err);
    } else if (j->batch == j->nbatches - 1) complete_job(s, j);
    else {
      j->batch++;
      j->cursor = 0;
      j->pass_hint = 0;
      j->phase = P_ITER;
    }
  }
  t->in_use = 0;
  t->njobs = 0;
}

/* finish every tail slot whose work has completed; returns slots in flight */
static int poll_tails(flam3gpu_service *s) {
  int busy = 0;
  for (unsigned long long k = s->tail_no >= NTAIL ? s->tail_no - NTAIL : 0; k < s->tail_no; k++) {
    tail_slot *t = &s->ts[k % NTAIL];
    if (!t->in_use) continue;
    cudaError_t q = cudaEventQuery(t->ev);
    if (q == cudaSuccess) finish_slot(s, t);
    else if (q == cudaErrorNotReady) busy++;
    else {
      char msg[200];
      snprintf(msg, sizeof(msg), "tail failed: %s", cudaGetErrorString(q));
      for (int i = 0; i < t->njobs; i++) {
        remove_active(s, t->jobs[i]);
        fail_job(s, t->jobs[i], msg);
      }
      t->in_use = 0;
    }
  }
  return busy;
}

static int ensure_round_cap(round_buf *r, size_t n) {
  if (r->cap >= n) return 0;
  size_t cap = r->cap ? r->cap : 1024;
  while (cap < n) cap *= 2;
  if (r->h_items) cudaFreeHost(r->h_items);
  if (r->h_prefix) cudaFreeHost(r->h_prefix);
  if (r->d_items) cudaFree(r->d_items);
  if (r->d_prefix) cudaFree(r->d_prefix);
  r->h_items = NULL;
  r->h_prefix = NULL;
  r->d_items = NULL;
  r->d_prefix = NULL;
  r->cap = 0;
  if (cudaMallocHost((void **)&r->h_items, cap * sizeof(F3GItem)) != cudaSuccess ||
      cudaMallocHost((void **)&r->h_prefix, (cap + NCLASS) * sizeof(long long)) != cudaSuccess ||
      cudaMalloc((void **)&r->d_items, cap * sizeof(F3GItem)) != cudaSuccess ||
      cudaMalloc((void **)&r->d_prefix, (cap + NCLASS) * sizeof(long long)) != cudaSuccess)
    return 1;
  r->cap = cap;
  return 0;
}

typedef struct {
  F3GItem it;
  long long span;
  int cls;
  long long clen; /* samples per chunk of the item's chunks */
} tmp_item;

/* a round's work list: by kernel class, then longest chunks first, so each
 * class's launch ends on short chunks and its blocks finish close together
 * (the jobs of a round complete with the round, so the order within it
 * changes no job's latency) */
static int tmp_item_cmp(const void *a, const void *b) {
  const tmp_item *x = (const tmp_item *)a, *y = (const tmp_item *)b;
  if (x->cls != y->cls) return x->cls - y->cls;
  if (x->clen != y->clen) return x->clen > y->clen ? -1 : 1;
  return 0;
}

static void round_done(flam3gpu_service *s, round_buf *r);

/* one iterate round over the admitted jobs; returns 1 if a round was issued */
static int issue_round(flam3gpu_service *s) {
  const int na = s->nactive;
  f3g_job **cand = (f3g_job **)malloc((size_t)(na + 1) * sizeof(f3g_job *));
  f3g_job **tails = (f3g_job **)malloc((size_t)(na + 1) * sizeof(f3g_job *));
  long long *takes = (long long *)malloc((size_t)(na + 1) * sizeof(long long));
  int nc = 0, ntails = 0;
  s->paused = 0;
  for (int i = 0; i < na; i++) {
    f3g_job *j = s->active[i];
    if (j->phase != P_ITER) continue;
    /* the request's progress callback, between the rounds of its job
     * (rect.c:324-391: 1 aborts, 2 pauses); called on the service thread */
    if (j->spec.progress && !j->aborted) {
      const double pct = j->total_samples > 0 ? 100.0 * j->done_samples / j->total_samples : 0.0;
      const int r = j->spec.progress(j->spec.progress_parameter, pct, 0, 0.0);
      if (r == 1) {
        j->aborted = 1;
        j->batch = j->nbatches - 1;
        j->cursor = j->bp[j->batch].chunks;
        if (j->h_counts) j->h_counts[0] = j->h_counts[1] = 0;
      } else if (r == 2) {
        s->paused++;
        continue;
      }
    }
    if (j->cursor < j->bp[j->batch].chunks) cand[nc++] = j;
    else tails[ntails++] = j; /* a batch without samples (or an aborted job) goes straight to its tail */
  }
  if (!nc) {
    if (ntails) enqueue_tails(s, tails, ntails);
    free(cand);
    free(tails);
    free(takes);
    return ntails > 0;
  }
  order_jobs(s, cand, nc);
  /* jobs in the policy's order (shortest remaining first by default), up to the round's sample budget; the
   * automatic budget gives every resident block at least 4 chunks of the
   * coarsest job, so the round's last wave wastes little */
  double budget;
  if (s->cfg.round_samples < 0) budget = 1e300;
  else if (s->cfg.round_samples > 0) budget = (double)s->cfg.round_samples;
  else {
    double cmax = 0;
    for (int i = 0; i < nc; i++) {
      const double cs = (double)cand[i]->threads * cand[i]->bp[cand[i]->batch].S;
      if (cs > cmax) cmax = cs;
    }
    budget = 4.0 * cmax * s->nsm * 4;
    if (budget < 2.0e8) budget = 2.0e8;
  }
  int np = 0;
  for (int i = 0; i < nc && budget > 0; i++, np++) {
    f3g_job *j = cand[i];
    const batch_plan *b = &j->bp[j->batch];
    const double cs = (double)j->threads * b->S;
    const long long avail = b->chunks - j->cursor;
    long long take = avail;
    if ((double)take * cs > budget) {
      take = (long long)ceil(budget / cs);
      if (take < 1) take = 1;
      if (take > avail) take = avail;
    }
    budget -= (double)take * cs;
    takes[i] = take;
  }
  /* work items: one per (job, temporal sample) range */
  size_t nit = 0, cap = (size_t)np * 2 + 16;
  tmp_item *ti = (tmp_item *)malloc(cap * sizeof(tmp_item));
  for (int i = 0; i < np && ti; i++) {
    f3g_job *j = cand[i];
    const batch_plan *b = &j->bp[j->batch];
    const long long *pre = j->pass_prefix + (size_t)j->batch * (j->ntemporal + 1);
    long long cur = j->cursor;
    const long long end = j->cursor + takes[i];
    int p = j->pass_hint;
    while (pre[p + 1] <= cur) p++;
    while (cur < end) {
      long long stop = pre[p + 1] < end ? pre[p + 1] : end;
      /* items do not straddle the pass's switch to short chunks */
      const long long tail_at = pre[p] + j->pass_tail[(size_t)j->batch * j->ntemporal + p];
      if (b->S_tail > 0 && cur < tail_at && stop > tail_at) stop = tail_at;
      if (stop > cur) {
        if (nit == cap) {
          cap *= 2;
          tmp_item *t2 = (tmp_item *)realloc(ti, cap * sizeof(tmp_item));
          if (!t2) {
            free(ti);
            ti = NULL;
            break;
          }
          ti = t2;
        }
        ti[nit].it.pass = j->d_passes + (size_t)j->batch * j->ntemporal + p;
        ti[nit].it.chunk_first = cur - pre[p];
        ti[nit].span = stop - cur;
        ti[nit].cls = b->full * 2 + b->mode;
        ti[nit].clen = (long long)j->threads * (b->S_tail > 0 && cur >= tail_at ? b->S_tail : b->S);
        nit++;
        cur = stop;
      }
      if (cur >= pre[p + 1]) p++;
    }
    if (!ti) break;
    j->pass_hint = p < j->ntemporal ? p : j->ntemporal - 1;
    j->done_samples += (double)takes[i] * j->threads * b->S;
    s->c_samples += (double)takes[i] * j->threads * b->S;
    j->cursor = end;
    j->rounds++;
    if (j->t_first == 0) j->t_first = now_s();
    if (j->cursor >= b->chunks) tails[ntails++] = j;
  }
  const unsigned long long rno = s->round_no;
  round_buf *r = &s->rb[rno % NRB];
  if (r->in_use) {
    cudaEventSynchronize(r->ev);
    round_done(s, r);
  }
  if (!ti || ensure_round_cap(r, nit + 1)) {
    free(ti);
    for (int i = 0; i < np; i++) {
      remove_active(s, cand[i]);
      fail_job(s, cand[i], "round work list: out of memory");
    }
    free(cand);
    free(tails);
    free(takes);
    return 0;
  }
  qsort(ti, nit, sizeof(tmp_item), tmp_item_cmp);
  /* classes in order; class c's prefix has one extra entry for its end */
  size_t cls_n[NCLASS] = {0}, cls_off[NCLASS + 1];
  long long tot[NCLASS] = {0};
  for (size_t k = 0; k < nit; k++) cls_n[ti[k].cls]++;
  cls_off[0] = 0;
  for (int c = 0; c < NCLASS; c++) cls_off[c + 1] = cls_off[c] + cls_n[c];
  size_t fill[NCLASS];
  for (int c = 0; c < NCLASS; c++) fill[c] = cls_off[c];
  for (size_t k = 0; k < nit; k++) {
    const int c = ti[k].cls;
    const size_t d = fill[c]++;
    r->h_items[d] = ti[k].it;
    r->h_prefix[d + c] = tot[c];
    tot[c] += ti[k].span;
  }
  for (int c = 0; c < NCLASS; c++) r->h_prefix[cls_off[c + 1] + c] = tot[c];
  free(ti);
  const int si = (int)(rno % (unsigned long long)s->cfg.streams);
  cudaStream_t st = s->s_iter[si];
  int err = 0;
  if (cudaMemcpyAsync(r->d_items, r->h_items, nit * sizeof(F3GItem), cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(r->d_prefix, r->h_prefix, (nit + NCLASS) * sizeof(long long), cudaMemcpyHostToDevice, st) !=
          cudaSuccess ||
      cudaMemsetAsync(r->d_ctr, 0, NCLASS * sizeof(F3GCounters), st) != cudaSuccess)
    err = 1;
  s->c_h2d += (double)nit * sizeof(F3GItem) + (double)(nit + NCLASS) * 8;
  const int shuffle = f3g_opts.shuffle_every > 0 ? f3g_opts.shuffle_every : 1;
  const int threads = f3g_opts.threads_per_block > 0 ? f3g_opts.threads_per_block : 256;
  const int precision = f3g_opts.iter_precision == 64 ? 64 : 32;
  cudaEventRecord(r->t0, st);
  for (int c = 0; c < NCLASS && !err; c++) {
    if (!cls_n[c]) continue;
    const int full = c >> 1, mode = c & 1;
    int occ = f3g_iterate_occupancy(precision, full, mode, threads);
    if (occ < 1) occ = 1;
    long long blocks = f3g_opts.blocks > 0 ? f3g_opts.blocks : (long long)s->nsm * occ;
    if (blocks > tot[c]) blocks = tot[c];
    int e = f3g_launch_iterate(r->d_items + cls_off[c], r->d_prefix + cls_off[c] + c, (int)cls_n[c], tot[c], shuffle,
                               precision, full, mode, threads, (int)blocks, r->d_ctr + c, st);
    s->c_launches++;
    if (e) err = 1;
  }
  cudaEventRecord(r->t1, st);
  if (!err && cudaMemcpyAsync(r->h_ctr, r->d_ctr, NCLASS * sizeof(F3GCounters), cudaMemcpyDeviceToHost, st) !=
                  cudaSuccess)
    err = 1;
  cudaEventRecord(r->ev, st);
  cudaEventRecord(s->ev_last[si], st);
  r->in_use = 1;
  s->round_no++;
  s->c_rounds++;
  if (err) {
    char msg[200];
    snprintf(msg, sizeof(msg), "iterate launch failed: %s", cudaGetErrorString(cudaGetLastError()));
    for (int i = 0; i < np; i++) {
      remove_active(s, cand[i]);
      fail_job(s, cand[i], msg);
    }
    ntails = 0;
  }
  if (ntails) enqueue_tails(s, tails, ntails);
  free(cand);
  free(tails);
  free(takes);
  return 1;
}

static void round_done(flam3gpu_service *s, round_buf *r) {
  float ms = 0;
  if (cudaEventElapsedTime(&ms, r->t0, r->t1) == cudaSuccess) s->g_iter += ms * 1e-3;
  for (int c = 0; c < NCLASS; c++)
    if (r->h_ctr[c].error && !s->kernel_err[0])
      snprintf(s->kernel_err, sizeof(s->kernel_err), "iterate kernel: a point-exchange wait timed out");
  r->in_use = 0;
}

static int rounds_in_flight(flam3gpu_service *s) {
  int n = 0;
  for (int k = 0; k < NRB; k++)
    if (s->rb[k].in_use) {
      if (cudaEventQuery(s->rb[k].ev) == cudaSuccess) round_done(s, &s->rb[k]);
      else n++;
    }
  return n;
}

static void wait_oldest_round(flam3gpu_service *s) {
  for (unsigned long long k = s->round_no >= NRB ? s->round_no - NRB : 0; k < s->round_no; k++) {
    round_buf *r = &s->rb[k % NRB];
    if (r->in_use) {
      cudaEventSynchronize(r->ev);
      round_done(s, r);
      return;
    }
  }
}

static void wait_oldest_tail(flam3gpu_service *s) {
  for (unsigned long long k = s->tail_no >= NTAIL ? s->tail_no - NTAIL : 0; k < s->tail_no; k++) {
    tail_slot *t = &s->ts[k % NTAIL];
    if (t->in_use) {
      cudaEventSynchronize(t->ev);
      return;
    }
  }
}

/* admits queued jobs while they fit; called with s->mu held */
static void admit_pending(flam3gpu_service *s) {
  while (s->pend_head) {
    f3g_job *j = s->pend_head;
    if (s->cfg.max_active > 0 && s->nactive >= s->cfg.max_active) return;
    if (j->dev_bytes > s->budget) {
      s->pend_head = j->next;
      if (!s->pend_head) s->pend_tail = NULL;
      pthread_mutex_unlock(&s->mu);
      char msg[200];
      snprintf(msg, sizeof(msg), "job needs %zu device bytes, more than the service budget %zu", j->dev_bytes,
               s->budget);
      fail_job(s, j, msg);
      pthread_mutex_lock(&s->mu);
      continue;
    }
    if (s->used + j->dev_bytes > s->budget) return;
    if (s->nactive >= s->active_cap) {
      int nc2 = s->active_cap ? 2 * s->active_cap : 64;
      f3g_job **na = (f3g_job **)realloc(s->active, (size_t)nc2 * sizeof(f3g_job *));
      if (!na) return;
      s->active = na;
      s->active_cap = nc2;
    }
    s->pend_head = j->next;
    if (!s->pend_head) s->pend_tail = NULL;
    j->next = NULL;
    pthread_mutex_unlock(&s->mu);
    const double ta = now_s();
    const int a = admit_job(s, j);
    s->h_admit += now_s() - ta;
    pthread_mutex_lock(&s->mu);
    if (a == 2) {
      /* the pool has no room yet: back to the queue head until a job ends */
      if (s->nactive == 0) {
        pthread_mutex_unlock(&s->mu);
        fail_job(s, j, "device memory exhausted");
        pthread_mutex_lock(&s->mu);
        continue;
      }
      j->next = s->pend_head;
      s->pend_head = j;
      if (!s->pend_tail) s->pend_tail = j;
      return;
    }
    if (a == 1) {
      pthread_mutex_unlock(&s->mu);
      fail_job(s, j, NULL);
      pthread_mutex_lock(&s->mu);
      continue;
    }
    j->state = J_ACTIVE;
    j->t_admit = now_s();
    if (s->t_first_admit == 0) s->t_first_admit = j->t_admit;
    s->used += j->dev_bytes;
    if (s->used > s->peak) s->peak = s->used;
    s->active[s->nactive++] = j;
  }
}

static void *service_main(void *arg) {
  flam3gpu_service *s = (flam3gpu_service *)arg;
  cudaSetDevice(s->device);
  for (;;) {
    pthread_mutex_lock(&s->mu);
    admit_pending(s);
    pthread_mutex_unlock(&s->mu);
    double t0 = now_s();
    poll_tails(s);
    s->h_done += now_s() - t0;
    if (rounds_in_flight(s) >= s->cfg.max_inflight) {
      t0 = now_s();
      wait_oldest_round(s);
      s->h_wait += now_s() - t0;
    }
    t0 = now_s();
    const int issued = issue_round(s);
    s->h_round += now_s() - t0;
    if (issued) continue;
    const int paused = s->paused;
    /* nothing to issue: wait for the GPU, or for submissions */
    t0 = now_s();
    const int busy = poll_tails(s);
    s->h_done += now_s() - t0;
    if (busy > 0) {
      t0 = now_s();
      wait_oldest_tail(s);
      s->h_wait += now_s() - t0;
      continue;
    }
    if (rounds_in_flight(s)) {
      t0 = now_s();
      wait_oldest_round(s);
      s->h_wait += now_s() - t0;
      continue;
    }
    pthread_mutex_lock(&s->mu);
    if (s->nactive == 0 && !s->pend_head) {
      if (s->stop) {
        pthread_mutex_unlock(&s->mu);
        break;
      }
      pthread_cond_wait(&s->cv_work, &s->mu);
    } else if (s->nactive == 0 || s->pend_head || paused) {
      /* queued work that does not fit yet, a retry after a pool miss, or
       * paused jobs to ask again (every 10 ms) */
      struct timespec dl;
      clock_gettime(CLOCK_REALTIME, &dl);
      dl.tv_nsec += paused ? 10000000 : 1000000;
      if (dl.tv_nsec >= 1000000000) {
        dl.tv_sec++;
        dl.tv_nsec -= 1000000000;
      }
      pthread_cond_timedwait(&s->cv_work, &s->mu, &dl);
    }
    pthread_mutex_unlock(&s->mu);
  }
  return NULL;
}

int flam3gpu_service_wait(flam3gpu_service *s, uint64_t ticket, double timeout_ms, stat_struct *stats,
                          double times_ms[4]) {
  f3g_clear_error();
  if (!s || ticket == 0 || ticket > s->next_ticket) {
    f3g_set_error("unknown ticket %llu", (unsigned long long)ticket);
    return 1;
  }
  pthread_mutex_lock(&s->mu);
  f3g_job *j = s->jobs[ticket - 1];
  if (!j) {
    pthread_mutex_unlock(&s->mu);
    f3g_set_error("ticket %llu was already collected", (unsigned long long)ticket);
    return 1;
  }
  struct timespec dl;
  if (timeout_ms >= 0) {
    clock_gettime(CLOCK_REALTIME, &dl);
    double t = dl.tv_sec + 1e-9 * dl.tv_nsec + timeout_ms * 1e-3;
    dl.tv_sec = (time_t)t;
    dl.tv_nsec = (long)((t - (double)dl.tv_sec) * 1e9);
  }
  while (j->state != J_DONE && j->state != J_FAILED) {
    if (timeout_ms >= 0) {
      if (pthread_cond_timedwait(&s->cv_done, &s->mu, &dl) != 0 && j->state != J_DONE && j->state != J_FAILED) {
        pthread_mutex_unlock(&s->mu);
        return 2;
      }
    } else
      pthread_cond_wait(&s->cv_done, &s->mu);
  }
  s->jobs[ticket - 1] = NULL;
  pthread_mutex_unlock(&s->mu);
  int rv = j->rv;
  if (rv == 0) copy_out(j);
  if (stats) *stats = j->stats;
  if (times_ms) {
    times_ms[0] = j->t_admit > 0 ? 1e3 * (j->t_admit - j->t_submit) : -1;
    times_ms[1] = j->t_first > 0 && j->t_admit > 0 ? 1e3 * (j->t_first - j->t_admit) : -1;
    times_ms[2] = 1e3 * (j->t_done - j->t_submit);
    times_ms[3] = j->rounds;
  }
  if (rv) f3g_set_error("%s", j->err[0] ? j->err : "render failed");
  job_free_plan(j);
  free(j);
  return rv;
}

int flam3gpu_service_drain(flam3gpu_service *s) {
  if (!s) return 1;
  pthread_mutex_lock(&s->mu);
  for (;;) {
    int busy = s->pend_head != NULL;
    for (uint64_t t = 0; !busy && t < s->next_ticket; t++) {
      f3g_job *j = s->jobs[t];
      if (j && j->state != J_DONE && j->state != J_FAILED) busy = 1;
    }
    if (!busy) break;
    pthread_cond_wait(&s->cv_done, &s->mu);
  }
  pthread_mutex_unlock(&s->mu);
  return 0;
}

void flam3gpu_service_counters(flam3gpu_service *s, double out[19]) {
  memset(out, 0, 19 * sizeof(double));
  if (!s) return;
  pthread_mutex_lock(&s->mu);
  out[0] = s->c_done;
  out[1] = s->c_failed;
  out[2] = s->c_rounds;
  out[3] = s->c_launches;
  out[4] = s->c_graphs;
  out[5] = s->c_inst;
  out[6] = s->c_plotted;
  out[7] = (double)s->used;
  out[8] = (double)s->peak;
  out[9] = s->t_last_done > s->t_first_admit ? s->t_last_done - s->t_first_admit : 0;
  out[10] = s->c_h2d;
  out[11] = s->c_d2h;
  out[12] = s->h_admit;
  out[13] = s->h_round;
  out[14] = s->h_tail;
  out[15] = s->h_done;
  out[16] = s->h_wait;
  out[17] = s->g_iter;
  out[18] = s->g_tail;
  pthread_mutex_unlock(&s->mu);
}

void flam3gpu_service_destroy(flam3gpu_service *s) {
  if (!s) return;
  if (s->thread_started) {
    pthread_mutex_lock(&s->mu);
    s->stop = 1;
    pthread_cond_broadcast(&s->cv_work);
    pthread_mutex_unlock(&s->mu);
    pthread_join(s->thread, NULL);
    pthread_mutex_destroy(&s->mu);
    pthread_cond_destroy(&s->cv_work);
    pthread_cond_destroy(&s->cv_done);
  }
  for (uint64_t t = 0; t < s->next_ticket; t++)
    if (s->jobs && s->jobs[t]) {
      if (s->jobs[t]->h_out) pin_put(s->jobs[t]->h_out, align256(s->jobs[t]->out_bytes) + 2 * sizeof(unsigned long long));
      job_free_plan(s->jobs[t]);
      free(s->jobs[t]);
    }
  free(s->jobs);
  free(s->active);
  for (int k = 0; k < NRB; k++) {
    if (s->rb[k].h_items) cudaFreeHost(s->rb[k].h_items);
    if (s->rb[k].h_prefix) cudaFreeHost(s->rb[k].h_prefix);
    if (s->rb[k].d_items) cudaFree(s->rb[k].d_items);
    if (s->rb[k].d_prefix) cudaFree(s->rb[k].d_prefix);
    if (s->rb[k].d_ctr) cudaFree(s->rb[k].d_ctr);
    if (s->rb[k].h_ctr) cudaFreeHost(s->rb[k].h_ctr);
    if (s->rb[k].ev) cudaEventDestroy(s->rb[k].ev);
    if (s->rb[k].t0) cudaEventDestroy(s->rb[k].t0);
    if (s->rb[k].t1) cudaEventDestroy(s->rb[k].t1);
  }
  for (int k = 0; k < NTAIL; k++) {
    if (s->ts[k].ev) cudaEventDestroy(s->ts[k].ev);
    if (s->ts[k].t0) cudaEventDestroy(s->ts[k].t0);
    free(s->ts[k].jobs);
  }
  for (int k = 0; k < NGRAPH; k++)
    if (s->graphs[k].exec) cudaGraphExecDestroy(s->graphs[k].exec);

  for (int k = 0; k < 8; k++) {
    if (s->s_iter[k]) cudaStreamDestroy(s->s_iter[k]);
    if (s->ev_last[k]) cudaEventDestroy(s->ev_last[k]);
  }
  for (int k = 0; k < NBRANCH; k++) {
    if (s->s_br[k]) cudaStreamDestroy(s->s_br[k]);
    if (s->ev_join[k]) cudaEventDestroy(s->ev_join[k]);
  }
  if (s->ev_fork) cudaEventDestroy(s->ev_fork);
  if (s->s_up) cudaStreamDestroy(s->s_up);
  if (s->s_tail) cudaStreamDestroy(s->s_tail);
  free(s);
}

typedef struct {
  flam3gpu_service *s;
  flam3_frame *frames;
  void **outs;
  uint64_t *tk;
  int n, field, nchan, transp, k, stride, rv;
  char err[256];
} submit_arg;

static void *submit_worker(void *p) {
  submit_arg *a = (submit_arg *)p;
  for (int i = a->k; i < a->n; i += a->stride)
    if (flam3gpu_service_submit(a->s, &a->frames[i], a->outs[i], a->field, a->nchan, a->transp, &a->tk[i])) {
      a->tk[i] = 0;
      if (!a->rv) snprintf(a->err, sizeof(a->err), "%s", flam3gpu_last_error());
      a->rv = 1;
    }
  return NULL;
}

/* plans the frames on up to 16 host threads; each is admitted as soon as it
 * is planned, so the device starts on the first while the rest are planned */
int flam3gpu_service_submit_many(flam3gpu_service *s, flam3_frame *frames, int n, void **outs, int field, int nchan,
                                 int transp, uint64_t *tk) {
  f3g_clear_error();
  if (!s || n < 0 || (n > 0 && (!frames || !outs || !tk))) {
    f3g_set_error("bad arguments to flam3gpu_service_submit_many");
    return 1;
  }
  if (n == 0) return 0;
  int nt = n < 16 ? n : 16;
  submit_arg *args = (submit_arg *)calloc((size_t)nt, sizeof(submit_arg));
  pthread_t *th = (pthread_t *)calloc((size_t)nt, sizeof(pthread_t));
  int *started = (int *)calloc((size_t)nt, sizeof(int));
  for (int k = 0; k < nt; k++) {
    args[k] = (submit_arg){s, frames, outs, tk, n, field, nchan, transp, k, nt, 0, ""};
    started[k] = pthread_create(&th[k], NULL, submit_worker, &args[k]) == 0;
    if (!started[k]) submit_worker(&args[k]);
  }
  int rv = 0;
  for (int k = 0; k < nt; k++) {
    if (started[k]) pthread_join(th[k], NULL);
    if (args[k].rv && !rv) f3g_set_error("%s", args[k].err);
    rv |= args[k].rv;
  }
  free(args);
  free(th);
  free(started);
  return rv;
}

int flam3gpu_render_batch(flam3_frame *frames, int n, void **outs, int field, int nchan, int transp,
                          stat_struct *stats, const flam3gpu_service_config *cfg) {
  f3g_clear_error();
  if (n < 1) return 0;
  flam3gpu_service_config c;
  if (cfg) c = *cfg;
  else {
    flam3gpu_service_default_config(&c);
    c.round_samples = -1; /* everything admitted runs in one launch per round */
  }
  flam3gpu_service *s = flam3gpu_service_create(&c);
  if (!s) return 1;
  uint64_t *tk = (uint64_t *)calloc((size_t)n, sizeof(uint64_t));
  int rv = flam3gpu_service_submit_many(s, frames, n, outs, field, nchan, transp, tk);
  char first_err[256] = "";
  for (int i = 0; i < n; i++) {
    if (!tk[i]) continue;
    if (flam3gpu_service_wait(s, tk[i], -1, stats ? &stats[i] : NULL, NULL)) {
      if (!first_err[0]) snprintf(first_err, sizeof(first_err), "%s", flam3gpu_last_error());
      rv = 1;
    }
  }
  free(tk);
  flam3gpu_service_destroy(s);
  if (rv && first_err[0]) f3g_set_error("%s", first_err);
  return rv;
}

/* ------------------------------------------------------------- autotuner */

/* time one job alone through a private service with forced knobs */
static double time_job(flam3_frame *f, int nchan, int S, int tile, double *iter_ms) {
  flam3gpu_service_config c;
  flam3gpu_service_default_config(&c);
  c.round_samples = -1;
  c.use_tuning = 0;
  flam3gpu_service *s = flam3gpu_service_create(&c);
  if (!s) return -1;
  f3g_job *j = (f3g_job *)calloc(1, sizeof(f3g_job));
  j->spec = *f;
  j->spec.progress = NULL;
  j->spec.genomes = (flam3_genome *)calloc((size_t)f->ngenomes, sizeof(flam3_genome));
  for (int i = 0; i < f->ngenomes; i++) f3g_genome_copy(&j->spec.genomes[i], &f->genomes[i]);
  j->nchan = nchan;
  double t = -1;
  if (plan_job(j, s->nsm, 0, S, tile) == 0) {
    void *out = malloc(j->out_bytes);
    j->out = out;
    pthread_mutex_lock(&s->mu);
    j->ticket = ++s->next_ticket;
    s->jobs = (f3g_job **)calloc(1, sizeof(f3g_job *));
    s->njobs_cap = 1;
    s->jobs[0] = j;
    j->t_submit = now_s();
    s->pend_head = s->pend_tail = j;
    pthread_cond_broadcast(&s->cv_work);
    pthread_mutex_unlock(&s->mu);
    double tm[4];
    stat_struct st;
    if (flam3gpu_service_wait(s, 1, -1, &st, tm) == 0) t = tm[2];
    if (iter_ms) *iter_ms = t;
    free(out);
  } else {
    job_free_plan(j);
    free(j);
  }
  flam3gpu_service_destroy(s);
  return t;
}

int flam3gpu_autotune(flam3_frame *frames, int n, double quality_scale) {
  f3g_clear_error();
  int tuned = 0;
  int nsm = 0, dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) {
    f3g_set_error("no CUDA device available");
    return -1;
  }
  static const int S_cand[] = {128, 256, 512, 1024};
  /* DE tail shapes: owner bands, or the fused tile kernel at three edges */
  static const int T_cand[] = {DE_BANDS, 8, 16, 32};
  for (int i = 0; i < n; i++) {
    /* class key of the frame as submitted */
    f3g_job probe;
    memset(&probe, 0, sizeof(probe));
    probe.spec = frames[i];
    probe.spec.genomes = (flam3_genome *)calloc((size_t)frames[i].ngenomes, sizeof(flam3_genome));
    for (int k = 0; k < frames[i].ngenomes; k++) f3g_genome_copy(&probe.spec.genomes[k], &frames[i].genomes[k]);
    probe.nchan = 3;
    if (plan_job(&probe, nsm, 0, 0, 0)) {
      job_free_plan(&probe);
      continue;
    }
    char key[96];
    tune_key(&probe, key, sizeof(key));
    const int has_de = probe.fused_de || probe.band_de;
    job_free_plan(&probe);
    int S0, T0;
    if (tune_lookup(key, &S0, &T0)) continue;
    /* a reduced-quality copy of the frame */
    flam3_frame f = frames[i];
    f.genomes = (flam3_genome *)calloc((size_t)frames[i].ngenomes, sizeof(flam3_genome));
    for (int k = 0; k < frames[i].ngenomes; k++) {
      f3g_genome_copy(&f.genomes[k], &frames[i].genomes[k]);
      if (quality_scale > 0) f.genomes[k].sample_density *= quality_scale;
    }
    double best = 1e300;
    int bestS = 256, bestT = f3g_opts.de_kernel == 0 ? DE_BANDS : 16;
    for (size_t a = 0; a < sizeof(S_cand) / sizeof(S_cand[0]); a++) {
      double t = time_job(&f, 3, S_cand[a], 0, NULL);
      if (t > 0 && t < best) {
        best = t;
        bestS = S_cand[a];
      }
    }
    if (has_de) {
      best = 1e300;
      for (size_t b = 0; b < sizeof(T_cand) / sizeof(T_cand[0]); b++) {
        double t = time_job(&f, 3, bestS, T_cand[b], NULL);
        if (t > 0 && t < best) {
          best = t;
          bestT = T_cand[b];
        }
      }
    }
    for (int k = 0; k < frames[i].ngenomes; k++) f3g_genome_free(&f.genomes[k]);
    free(f.genomes);
    tune_store(key, bestS, bestT);
    tuned++;
  }
  return tuned;
}

int flam3gpu_autotune_save(const char *path) {
  FILE *fp = fopen(path, "w");
  if (!fp) {
    f3g_set_error("cannot write %s", path);
    return 1;
  }
  pthread_mutex_lock(&g_tune_mu);
  for (int i = 0; i < g_ntune; i++) fprintf(fp, "%s %d %d\n", g_tune[i].key, g_tune[i].S, g_tune[i].tile);
  pthread_mutex_unlock(&g_tune_mu);
  fclose(fp);
  return 0;
}

int flam3gpu_autotune_load(const char *path) {
  FILE *fp = fopen(path, "r");
  if (!fp) {
    f3g_set_error("cannot read %s", path);
    return 1;
  }
  char key[96];
  int S, tile;
  while (fscanf(fp, "%95s %d %d", key, &S, &tile) == 3) tune_store(key, S, tile);
  fclose(fp);
  return 0;
}

void flam3gpu_autotune_clear(void) {
  pthread_mutex_lock(&g_tune_mu);
  free(g_tune);
  g_tune = NULL;
  g_ntune = 0;
  pthread_mutex_unlock(&g_tune_mu);
}
