/*
 * f3g_launch.h -- internal C interface between the host driver and the
 * kernel launch wrappers (all return a cudaError_t value, 0 on success).
 */
#ifndef F3G_LAUNCH_H
#define F3G_LAUNCH_H

#include <cuda_runtime.h>
#include <stddef.h>

#include "f3g_common.h"

#ifdef __cplusplus
extern "C" {
#endif

/* tonemap constants of one render (rect.c:1069-1081) */
typedef struct {
  float g;            /* 1 / mean gamma */
  float linrange;     /* gam_lin_thresh */
  float funcval;      /* linrange^g */
  float vibrancy;     /* mean vibrancy */
  float highpow;      /* highlight_power */
  float background[3];/* mean background * 256 */
  int nchan, transp, bpc;
  int trunc_acc;      /* integer accumulator (bits 32): log-scaled and earlyclip values truncated */
} F3GTonemap;

int f3g_iterate_occupancy(int precision, int full, int mode, int threads);
/* One persistent iterate launch over a work list: item i covers chunk-prefix
 * span [d_prefix[i], d_prefix[i+1]) of the launch, starting at chunk
 * d_items[i].chunk_first of its pass.  d_ctr->next_chunk must hold the first
 * chunk of the launch (normally 0). */
int f3g_launch_iterate(const F3GItem *d_items, const long long *d_prefix, int nitems, long long total_chunks,
                       int shuffle_every, int precision, int full, int mode, int threads, int blocks,
                       F3GCounters *d_ctr, cudaStream_t st);

int f3g_launch_logscale(const void *buckets, int bkind, long long n, double k1, double k2, void *acc, int akind,
                        int trunc, cudaStream_t st);
/* DE kernels take per-kernel constants (4 floats per kernel, see f3g_de.cu) */
void f3g_de_kernel_info(int mfi, int ks, const double *widths, const double *coefs, float *out);
int f3g_launch_de(const void *buckets, int bkind, const void *count, int W, int H, int oversample, double k1,
                  double k2, double curve, int max_filtered_counts, int max_filter_index, const float *kinfo, int R,
                  void *acc, int akind, cudaStream_t st);
int f3g_de_max_reach(void);
size_t f3g_de_fused_smem(int oversample, int fw, int R, int nk);
int f3g_launch_de_fused(const void *buckets, int bkind, const void *count, int W, int H, int oversample, double k1,
                        double k2, double curve, int mfc, int mfi, const float *kinfo, int R, int de_offset,
                        const float *filter, int fw, int image_w, int image_h, unsigned char *out, int earlyclip,
                        const F3GTonemap *tp, cudaStream_t st);
/* the fused DE kernel with a chosen output-tile edge (tile x tile pixels per block) */
size_t f3g_de_fused_smem_tile(int oversample, int fw, int R, int nk, int tile);
int f3g_launch_de_fused_tile(const void *buckets, int bkind, const void *count, int W, int H, int oversample,
                             double k1, double k2, double curve, int mfc, int mfi, const float *kinfo, int R,
                             int de_offset, const float *filter, int fw, int image_w, int image_h,
                             unsigned char *out, int earlyclip, const F3GTonemap *tp, int tile, cudaStream_t st);
/* Density estimation by owner bands (f3g_de_bands.cu): classifies every
 * bucket into fi (W*H bytes) and stores (add = 0) or adds (add = 1) the DE
 * result into acc (akind: F3G_BK_F32 float4 or F3G_BK_F64 double4 per
 * bucket).  stats (NULL in renders): device counters [sources, source-band
 * pairs, taps] the launch adds its work to.  -1 when R or mfi is beyond the
 * kernel's limits. */
int f3g_de_bands_supported(int R, int mfi);
int f3g_de_bands_prepare(void);
int f3g_launch_de_bands(const void *buckets, int bkind, const void *count, int W, int H, int oversample, double k1,
                        double k2, double curve, int mfc, int mfi, const float *kinfo, int R, uint8_t *fi, void *acc,
                        int akind, int add, unsigned long long *stats, cudaStream_t st);
/* filter + tonemap + pack of an FP32 accumulator (the separable strip kernel
 * where an instantiation exists, else earlyclip + the 2-D filter kernel) */
int f3g_launch_acc_filter(void *acc, int W, int H, int de_offset, int oversample, const float *filter, int fw,
                          int image_w, int image_h, unsigned char *out, int earlyclip, const F3GTonemap *tp,
                          cudaStream_t st);
/* raises the tail kernels' shared-memory limits (call before stream capture) */
int f3g_de_prepare(void);
int f3g_tail_prepare(void);
/* ceiling probe: blocks x 256 threads each add per_thread float4s at
 * pseudo-random buckets of buf[nbuckets] (f3g_probe.cu) */
int f3g_launch_atomic_rate(float4 *buf, unsigned long long nbuckets, int blocks, int per_thread, uint32_t salt,
                           cudaStream_t st);
/* separable strip kernels (f3g_strip_{f32,f64}{,e}.cu: FP32/FP64
 * histogram, earlyclip off/on): -2 when no instantiation covers
 * (oversample, fw) */
#define F3G_STRIP_DECL(SUFFIX)                                                                                  \
  int f3g_strip_prepare_##SUFFIX(void);                                                                       \
  int f3g_strip_launch_##SUFFIX(const void *buckets, int W, int H, double k1, double k2, int de_offset,       \
                                int oversample, const float *filter, int fw, int image_w, int image_h,        \
                                unsigned char *out, const F3GTonemap *tp, cudaStream_t st);
F3G_STRIP_DECL(f32)
F3G_STRIP_DECL(f64)
F3G_STRIP_DECL(f32e)
F3G_STRIP_DECL(f64e)
F3G_STRIP_DECL(acc)
F3G_STRIP_DECL(acce)
#undef F3G_STRIP_DECL
int f3g_launch_earlyclip(void *acc, int akind, long long n, const F3GTonemap *tp, cudaStream_t st);
int f3g_launch_filter_tonemap(const void *acc, int akind, int W, int de_offset, int oversample, const float *filter,
                              int fw, int image_w, int image_h, unsigned char *out, int earlyclip,
                              const F3GTonemap *tp, cudaStream_t st);
int f3g_launch_fused_log_filter(const void *buckets, int bkind, int W, int H, double k1, double k2, int de_offset,
                                int oversample, const float *filter, int fw, int image_w, int image_h,
                                unsigned char *out, int earlyclip, const F3GTonemap *tp, cudaStream_t st);

/* Temporal samples planned on the device (f3g_plan.cu).  A key set is the
 * aligned key genomes of one interpolation segment, laid out from its start
 * as: this header, nk flam3_genome structs (their scalars and palettes; the
 * pointers are not used), nk x nx flam3_xform, nk x nstd x nstd chaos
 * doubles.  Each sample names its key set (byte offset in the key buffer),
 * the keys' weights and its colour scalar; the kernel fills in the colour
 * map, xforms, variation lists and choice rows of the sample's pass, whose
 * other fields the host has uploaded.  d_err[i] != 0: sample i overflowed a
 * limit (variation lists, choice rows). */
typedef struct {
  int nk, nx, nstd, final_index;
  long long off_genome, off_xform, off_chaos;
} F3GKeySet;
typedef struct {
  long long keyset;
  double w[4];
  double color_scalar;
} F3GPlanSample;
size_t f3g_plan_smem(int nx, int nstd);
int f3g_launch_plan(const unsigned char *d_keys, const F3GPlanSample *d_samples, int n, int nx_max, int nstd_max,
                    F3GPass *d_passes, int *d_err, cudaStream_t st);

/* parity helpers (f3g_probe.cu) */
int f3g_launch_apply_xform(const F3GPass *d_pass, int fn, int n, const double *d_pin, const uint32_t *d_words,
                           int wpp, double *d_qout, int *d_bad, int precision, cudaStream_t st);
int f3g_launch_accumulate(const F3GPass *d_pass, const double *d_points, long long n, cudaStream_t st);
int f3g_launch_xform_choice(const F3GPass *d_pass, int rows, uint16_t *d_out, cudaStream_t st);
int f3g_launch_iterate_chains(const F3GPass *d_pass, int nchains, int n, int fuse, const double *d_starts,
                              uint32_t key0, uint32_t key1, double *d_samples, unsigned long long *d_bad,
                              int precision, cudaStream_t st);

/* PNG encoder (f3g_png.cu) */
long long f3g_png_filtered_bytes(int w, int h, int nchan, int bpc);
int f3g_png_segments(int w, int h, int nchan, int bpc);
size_t f3g_png_work_bytes(int w, int h, int nchan, int bpc);
size_t f3g_png_idat_bound(int w, int h, int nchan, int bpc);
int f3g_png_encode_idat(const void *d_img, int w, int h, int nchan, int bpc, void *d_work, void *d_idat,
                        unsigned long long *d_len, cudaStream_t st);

#ifdef __cplusplus
}
#endif
#endif
