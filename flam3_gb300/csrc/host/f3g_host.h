/*
 * f3g_host.h -- internal interface of the libflam3gpu host driver (C).
 */
#ifndef F3G_HOST_H
#define F3G_HOST_H

#include <cuda_runtime.h>
#include <stdint.h>

#include "flam3_gpu.h"
#include "../f3g_common.h"
#include "../f3g_launch.h"

#ifndef F3_RANDSIZ
#define F3_RANDSIZ RANDSIZ
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* geometry of a render (rect.c:613-687) */
typedef struct {
  int oversample, image_width, image_height, out_width;
  int filter_width, gutter, de_offset, W, H;
} f3g_geom;

int f3g_geometry(flam3_frame *spec, const flam3_genome *cp, int field, double **filter, f3g_geom *g);

/* per temporal sample results of f3g_build_batch_passes */
typedef struct f3g_pass_info_s {
  double vibrancy, gamma, background[3];
  double sample_density, ppux, ppuy, batch_size;
  double contrast, brightness, gam_lin_thresh, estimator_curve;
  int need_count; /* palette alpha != 1 */
  int err;
  char errmsg[256];
} f3g_pass_info;

/* The passes of batch `batch` (its ntemporal temporal samples): keys drawn
 * in order from spec->rc, then each sample's genome interpolated, prepared
 * and packed (host threads); per-sample scalars in info[]. */
int f3g_build_batch_passes(flam3_frame *spec, int field, const f3g_geom *g, int batch, int nbatches, int ntemporal,
                           const double *tfilter, const double *tdeltas, int cmap_size, F3GPass *passes,
                           f3g_pass_info *info);
int f3g_camera(flam3_frame *spec, const flam3_genome *cp, int field, const f3g_geom *g, F3GPass *p,
               double *sample_density, double *ppux, double *ppuy);
void f3g_pass_key(flam3_frame *spec, uint32_t key[2]);
unsigned long f3g_irand(randctx *r);

/* pieces of genome interpolation for the device planner (interp.c) */
int f3g_interp_segment(const flam3_genome *cps, int ncps, double time, int *first, double w[4]);
void f3g_align_keys(flam3_genome *keys, const flam3_genome *src, int nkeys);
void f3g_release_genome(flam3_genome *g);
void f3g_blend_scalars(const flam3_genome *keys, int nk, const double *w, flam3_genome *out);
int f3g_interp_overridden(void);

/* genome helpers (interp.c) for the XML genome reader (xml.c) */
void f3g_clear_cp(flam3_genome *cp, int default_flag);
void f3g_add_xforms(flam3_genome *cp, int num_to_add, int interp_padding, int final_flag);
void f3g_rgb2hsv(const double *rgb, double *hsv);
void f3g_hsv2rgb(const double *hsv, double *rgb);

/* error reporting: message kept per thread, also printed to stderr */
void f3g_set_error(const char *fmt, ...);
void f3g_clear_error(void);

#define F3G_CUDA(call)                                                            \
  do {                                                                            \
    cudaError_t e_ = (call);                                                      \
    if (e_ != cudaSuccess) {                                                      \
      f3g_set_error("CUDA error %s at %s:%d", cudaGetErrorString(e_), __FILE__, __LINE__); \
      return 1;                                                                   \
    }                                                                             \
  } while (0)

/* ---- genome preparation (prep.c) ---- */
void f3g_genome_free(flam3_genome *g);
void f3g_genome_copy(flam3_genome *dst, const flam3_genome *src);
int f3g_interpolate(flam3_genome *cps, int ncps, double time, flam3_genome *result);
int f3g_prepare_precalc_flags(flam3_genome *cp);
void f3g_xform_precalc(flam3_genome *cp, int xi);
/* builds the xform-choice table rows (flam3.c:76-224) and stores them as
 * breakpoints into pass; returns 0 on success */
/* one choice row's breakpoints on the host: the reference's loop (walk 0) or
 * the device planner's binade walk (walk 1) */
int f3g_choice_breakpoints_host(const double *d, const double *c, int nstd, int nx, int walk, uint16_t *brk,
                                int *nbrk, int *moves);
int f3g_build_distrib(flam3_genome *cp, F3GPass *pass);
/* fills the genome part of a pass from a prepared genome */
int f3g_pack_genome(flam3_genome *cp, F3GPass *pass);

/* ---- filters (filters.c) ---- */
int f3g_spatial_filter(flam3_frame *spec, int field, double **filter);
int f3g_de_filters(double max_rad, double min_rad, double curve, int ss, int *max_filtered_counts,
                   int *max_filter_index, double **widths, double **coefs);
double f3g_temporal_filter(int numsteps, int filter_type, double filter_exp, double filter_width, double **tfilter,
                           double **tdeltas);

/* ---- per-thread device context (render.c) ---- */
typedef struct {
  int device, nsm, ready;
  cudaStream_t stream;
  cudaEvent_t ev[8];
  void *d_hist; size_t hist_bytes;
  void *d_count; size_t count_bytes;
  void *d_acc; size_t acc_bytes;
  unsigned char *d_out; size_t out_bytes;
  F3GPass *d_passes; size_t passes_bytes;
  F3GPass *h_passes; size_t h_passes_bytes; /* pinned */
  long long *d_prefix; size_t prefix_bytes; long long *h_prefix; size_t prefix_n;
  F3GItem *d_items; size_t d_items_bytes; F3GItem *h_items; size_t h_items_n; /* pinned */
  struct f3g_pass_info_s *h_info; size_t h_info_n;
  F3GCounters *d_ctr; F3GCounters *h_ctr;
  float *d_filter; size_t filter_bytes;
  float *h_stage; size_t h_stage_n; /* pinned staging of small uploads (floats) */
  unsigned char *h_img; size_t h_img_bytes; /* pinned staging of the image */
  float *d_de_w; size_t de_w_bytes;
  uint8_t *d_fi; size_t fi_bytes; /* DE kernel index per bucket (band DE) */
  unsigned long long *d_de_stats; size_t de_stats_bytes;
  double de_work[3];               /* band DE work of the last render (de_stats) */
  float *d_de_c; size_t de_c_bytes;
  /* device planning of temporal samples: key sets and sample records
   * (pinned host staging and their device copies), error flags */
  unsigned char *h_plan_keys; size_t h_plan_keys_bytes;
  unsigned char *d_plan_keys; size_t d_plan_keys_bytes;
  F3GPlanSample *h_plan_samples; size_t h_plan_samples_n;
  F3GPlanSample *d_plan_samples; size_t d_plan_samples_bytes;
  int *d_plan_err; size_t d_plan_err_bytes;
  int plan_nx, plan_nstd;
  /* plan-only probe (flam3gpu_plan_passes): copy batch 0's passes out, skip the render */
  void *plan_only_out; int plan_only_max, plan_only_n;
  double timings[8];
  /* PNG encoder (png.c): scratch, IDAT chunks, their length, host images */
  void *d_png_work; size_t png_work_bytes;
  void *d_png_idat; size_t png_idat_bytes;
  void *d_png_img; size_t png_img_bytes;
  unsigned long long *d_png_len, *h_png_len; /* pinned */
} f3g_ctx;

f3g_ctx *f3g_get_ctx(void);
int f3g_ensure_host_pass_one(f3g_ctx *c);
int f3g_ensure(void **ptr, size_t *cap, size_t need);
extern flam3gpu_options f3g_opts;
/* samples per thread per chunk for a pass of `samples` samples */
int f3g_chunk_samples(const f3g_ctx *c, long long samples, int threads, int blocks, int sub_batch_size);
/* the xform-choice mode of a pass: 1 (warp-coherent) unless the genome has
 * xaos, the options ask for 0, or blocks hold fewer than 4 warps */
int f3g_choice_mode(int chaos_enable);
/* chunking of one launch's passes (S, S_tail, chunk_tail, nchunks,
 * chunk_begin; prefix[0..n] if not NULL); returns the launch's chunks */
long long f3g_chunk_passes(F3GPass *p, int n, int threads, int blocks, int S, long long *prefix);

#ifdef __cplusplus
}
#endif

#endif
