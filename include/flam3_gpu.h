/*
 * flam3_gpu.h -- C ABI of the GB300 render hot path for flam3.
 *
 * The library (flam3_gb300/libflam3gpu.so) replaces the body of
 * flam3_render(): chaos-game iteration, histogram accumulation, density
 * estimation, the spatial filter and the log-density/gamma tonemap run as
 * CUDA kernels for sm_103a; everything else about the call (arguments,
 * output layout, error returns, consumption of the caller's ISAAC context)
 * follows the reference.
 *
 * Part 1 mirrors the reference's public structs byte for byte so that a
 * flam3_frame built by unmodified flam3 code can be handed straight to
 * flam3gpu_render().  When the real flam3.h has already been included
 * (flam3_included is defined) the mirror is skipped and the reference's own
 * definitions are used.
 *
 * Part 2 is the drop-in entry point and its companions.
 * Part 3 are kernel-level entry points (plain pointers and sizes) used by the
 * parity tests and by callers that manage device memory themselves.
 *
 * All functions return 0 on success and nonzero on failure, with a message
 * retrievable through flam3gpu_last_error(); none of them throws.
 */
#ifndef FLAM3_GPU_H
#define FLAM3_GPU_H

#include <stddef.h>
#include <stdint.h>
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------
 * Part 1: layout mirror of the reference's public structs.
 * Field order, types and names are those of flam3.h and isaac.h; the layout
 * has to be identical for flam3-render/flam3-animate to call this library
 * unchanged.  The oracle build checks every offset against the real header.
 * ---------------------------------------------------------------------- */
#ifndef flam3_included

/* isaac.h:19-31 with isaacs.h:17 (ub4 is unsigned long) */
#define F3_RANDSIZL 4
#define F3_RANDSIZ (1 << F3_RANDSIZL)
typedef struct randctx {
  unsigned long randcnt;
  unsigned long randrsl[F3_RANDSIZ];
  unsigned long randmem[F3_RANDSIZ];
  unsigned long randa, randb, randc;
} randctx;

#define flam3_nvariations 99
#define flam3_name_len 64
#define flam3_parent_fn_len 30

/* flam3.h:49-54 */
typedef struct {
  double index;
  double color[4];
} flam3_palette_entry;
typedef flam3_palette_entry flam3_palette[256];

/* flam3.h:185-191 */
typedef struct {
  double badvals;
  long int num_iters;
  int render_seconds;
} stat_struct;

/* flam3.h:213-448: one xform, variation weights and parameters */
typedef struct xform {
  double var[flam3_nvariations];
  double c[3][2];
  double post[3][2];
  double density, color, color_speed, animate, opacity, vis_adjusted;
  int padding;
  double wind[2];
  int precalc_angles_flag, precalc_atan_xy_flag, precalc_atan_yx_flag;
  double has_preblur;
  int has_post;
  double blob_low, blob_high, blob_waves;
  double pdj_a, pdj_b, pdj_c, pdj_d;
  double fan2_x, fan2_y;
  double rings2_val;
  double perspective_angle, perspective_dist;
  double julian_power, julian_dist;
  double juliascope_power, juliascope_dist;
  double radial_blur_angle;
  double pie_slices, pie_rotation, pie_thickness;
  double ngon_sides, ngon_power, ngon_circle, ngon_corners;
  double curl_c1, curl_c2;
  double rectangles_x, rectangles_y;
  double amw_amp;
  double disc2_rot, disc2_twist;
  double super_shape_rnd, super_shape_m, super_shape_n1, super_shape_n2,
      super_shape_n3, super_shape_holes;
  double flower_petals, flower_holes;
  double conic_eccentricity, conic_holes;
  double parabola_height, parabola_width;
  double bent2_x, bent2_y;
  double bipolar_shift;
  double cell_size;
  double cpow_r, cpow_i, cpow_power;
  double curve_xamp, curve_yamp, curve_xlength, curve_ylength;
  double escher_beta;
  double lazysusan_spin, lazysusan_space, lazysusan_twist, lazysusan_x, lazysusan_y;
  double modulus_x, modulus_y;
  double oscope_separation, oscope_frequency, oscope_amplitude, oscope_damping;
  double popcorn2_x, popcorn2_y, popcorn2_c;
  double separation_x, separation_xinside, separation_y, separation_yinside;
  double split_xsize, split_ysize;
  double splits_x, splits_y;
  double stripes_space, stripes_warp;
  double wedge_angle, wedge_hole, wedge_count, wedge_swirl;
  double wedge_julia_angle, wedge_julia_count, wedge_julia_power, wedge_julia_dist;
  double wedge_sph_angle, wedge_sph_count, wedge_sph_hole, wedge_sph_swirl;
  double whorl_inside, whorl_outside;
  double waves2_freqx, waves2_scalex, waves2_freqy, waves2_scaley;
  double auger_sym, auger_weight, auger_freq, auger_scale;
  double flux_spread;
  double mobius_re_a, mobius_im_a, mobius_re_b, mobius_im_b;
  double mobius_re_c, mobius_im_c, mobius_re_d, mobius_im_d;
  /* values derived by xform_precalc (variations.c:1942-2014) */
  double persp_vsin, persp_vfcos;
  double julian_rN, julian_cn;
  double juliascope_rN, juliascope_cn;
  double wedgeJulia_rN, wedgeJulia_cn, wedgeJulia_cf;
  double radialBlur_spinvar, radialBlur_zoomvar;
  double waves_dx2, waves_dy2;
  double disc2_sinadd, disc2_cosadd, disc2_timespi;
  double super_shape_pm_4, super_shape_pneg1_n1;
  /* active-variation list built by prepare_precalc_flags */
  int num_active_vars;
  double active_var_weights[flam3_nvariations];
  int varFunc[flam3_nvariations];
  int motion_freq, motion_func;
  struct xform *motion;
  int num_motion;
} flam3_xform;

/* flam3.h:450-525: a genome (control point) */
typedef struct {
  char flame_name[flam3_name_len + 1];
  double time;
  int interpolation, interpolation_type, palette_interpolation;
  double hsv_rgb_palette_blend;
  int num_xforms, final_xform_index, final_xform_enable;
  flam3_xform *xform;
  double **chaos;
  int chaos_enable;
  int genome_index;
  char parent_fname[flam3_parent_fn_len];
  int symmetry;
  flam3_palette palette;
  char *input_image;
  int palette_index;
  double brightness, contrast, gamma, highlight_power;
  int width, height;
  int spatial_oversample;
  double center[2], rot_center[2];
  double rotate, vibrancy, hue_rotation;
  double background[3];
  double zoom, pixels_per_unit, spatial_filter_radius;
  int spatial_filter_select;
  double sample_density;
  int nbatches, ntemporal_samples;
  double estimator, estimator_curve, estimator_minimum;
  void *edits; /* xmlDocPtr in the reference */
  double gam_lin_thresh;
  int palette_index0;
  double hue_rotation0;
  int palette_index1;
  double hue_rotation1, palette_blend;
  int temporal_filter_type;
  double temporal_filter_width, temporal_filter_exp;
  int palette_mode;
} flam3_genome;

/* flam3.h:599-614: a render request */
typedef struct {
  double pixel_aspect_ratio;
  flam3_genome *genomes;
  int ngenomes, verbose, bits, bytes_per_channel, earlyclip;
  double time;
  int (*progress)(void *, double, int, double);
  void *progress_parameter;
  randctx rc;
  int nthreads, sub_batch_size;
} flam3_frame;

#define flam3_field_both 0
#define flam3_field_even 1
#define flam3_field_odd 2

#endif /* !flam3_included */

/* ------------------------------------------------------------------------
 * Part 2: drop-in render entry point.
 * ---------------------------------------------------------------------- */

/* Replaces flam3_render (flam3.h:623, flam3.c:3894-3932; body rect.c:529-1286).
 * Same arguments and meaning: `out` is a caller-owned buffer of
 * nchan*bytes_per_channel*width*height bytes; field selects both/even/odd
 * scanlines; stats receives num_iters, badvals and render_seconds.  bits must
 * be 32, 33 or 64 (else returns 1, as bits_error does).  f->rc is advanced
 * exactly as the reference advances it (RANDSIZ draws per host thread per
 * temporal sample), so callers that save and restore it (strips) behave the
 * same.  The progress callback is called from the calling thread between
 * kernel rounds with the reference's (param, percent, stage, eta) contract;
 * a return of 1 aborts (returns 0 with a partial image), 2 pauses.
 * Returns 0 on success, 1 on failure (message on stderr and in
 * flam3gpu_last_error()). */
int flam3gpu_render(flam3_frame *f, void *out, int field, int nchan, int transp, stat_struct *stats);

/* Replaces flam3_render_memory_required (flam3.c:3874-3887): device bytes the
 * render of f->genomes[0] needs (histogram + accumulator + chain state). */
double flam3gpu_render_memory_required(flam3_frame *f);

/* Replaces flam3_parse_xml2 (flam3.h:581, flam3.c:1423-1485, parser.c): reads
 * flam3's XML genome format (every <flame> element, at any depth, in
 * document order) into a malloc'd array of *ncps genomes with the
 * reference's defaults (default_flag 1) or unset markers (0), palettes
 * (inline <color>/<colors>/<palette> data, missing entries interpolated,
 * library palettes by number from the file named by $flam3_palettes),
 * <symmetry>, xforms, final xform, motion elements, xaos and solo xform.
 * xmlfilename's base name goes to parent_fname.  Free each genome with
 * flam3gpu_free_genome, then the array with free().  Returns NULL (and
 * *ncps = 0) on malformed XML or a malformed flame.  <edit> elements are not
 * kept (edits stays NULL). */
flam3_genome *flam3gpu_parse_xml2(char *xmldata, char *xmlfilename, int default_flag, int *ncps);

/* Replaces calc_nstrips (flam3-render.c:35-101) for device memory: the number
 * of horizontal strips the still f needs so that each strip's device bytes
 * (flam3gpu_render_memory_required) fit budget_bytes, or 80 % of the free
 * device memory when budget_bytes <= 0 (the reference: 80 % of physical host
 * memory, or $use_mem).  Returns 1 when the whole image fits, -1 on failure. */
int flam3gpu_calc_nstrips(flam3_frame *f, double budget_bytes);

/* The strip loop of flam3-render (flam3-render.c:311-345) around
 * flam3gpu_render: renders f (all fields, one temporal sample per genome, as
 * flam3-render renders stills) in nstrips horizontal strips of
 * ceil(height / nstrips) rows into the caller's full-size out buffer, each
 * strip with sample_density * nstrips, its own centre and the same saved
 * random context (f->rc is left as the last strip left it).  As in
 * flam3-render, when the height is not a multiple of nstrips the strips are
 * laid out for nstrips * ceil(height / nstrips) rows about the centre, which
 * moves the image down by half the excess.  The caller's genomes are not
 * modified.  stats receives the sums over the strips (each strip iterates
 * the whole frame's samples, so nstrips times the plain render's).
 * Returns 0 on success, 1 on failure (also when nstrips exceeds the height). */
int flam3gpu_render_strips(flam3_frame *f, void *out, int nchan, int transp, stat_struct *stats, int nstrips);

/* ---- PNG output on the device ---- */

/* Comments write_png stores in the PNG (img.h:29-36, the same layout). */
typedef struct {
  char *genome;
  char *badvals;
  char *numiters;
  char *rtime;
} flam3gpu_img_comments;

/* One PNG text chunk: tEXt, or zTXt when `compressed` (NULL or empty text:
 * an empty tEXt chunk, as libpng writes it). */
typedef struct {
  const char *key;
  const char *text;
  int compressed;
} flam3gpu_png_text;

/* Encodes a packed image as a PNG in host memory (the pixel path of
 * write_png, png.c:36-116: per-row PNG filters chosen by the
 * minimum-sum-of-absolute-values rule, deflate, IDAT chunks) with the
 * filtering, deflate, CRC-32 and Adler-32 done on the device.  image is
 * width x height pixels of nchan (3: RGB, 4: RGBA) samples of bpc bytes
 * (16-bit samples in host byte order, as flam3_render writes them), in
 * device memory when image_on_device, else in host memory.  The text chunks
 * follow IHDR in the given order.  *png receives a malloc'd buffer (release
 * it with free) and *png_len its size.  Returns 0, or 1 on failure. */
int flam3gpu_encode_png(const void *image, int image_on_device, int width, int height, int nchan, int bpc,
                        const flam3gpu_png_text *text, int ntext, unsigned char **png, size_t *png_len);

/* Replaces write_png (png.c:36, img.h:40): writes the RGBA image (bpc 1 or
 * 2) to `file` as a PNG with write_png's text chunks (flam3_version,
 * flam3_nickname/url/id from $nick/$url/$id, flam3_error_rate,
 * flam3_samples, flam3_time, and the genome as zTXt; none when
 * $enable_png_comments is not 1).  Returns 0, or 1 after a message on
 * stderr (the reference returns nothing and prints through perror). */
int flam3gpu_write_png(FILE *file, void *image, int width, int height, flam3gpu_img_comments *fpc, int bpc);

/* flam3-render's render-and-write step (flam3-render.c:345-378) without
 * the image leaving the device: renders f as flam3gpu_render(f, out,
 * flam3_field_both, 4, transp, stats) does, then encodes the RGBA image on
 * the device with the comments flam3-render passes to write_png (error rate,
 * samples and seconds from stats; genome_xml, may be NULL, as the genome).
 * *png receives a malloc'd PNG (release it with free).  Returns 0, or 1 on
 * failure. */
int flam3gpu_render_png(flam3_frame *f, int transp, stat_struct *stats, const char *genome_xml,
                        unsigned char **png, size_t *png_len);

/* flam3-animate's frame loop with PNG output (flam3-animate.c:225-310):
 * renders the n frames as RGBA (all fields, as flam3gpu_render(f, out,
 * flam3_field_both, 4, transp, stats) would) through a render service, in
 * chunks of 32 with the next chunk queued before the current one is
 * collected (host memory: two chunks of raw images), and encodes each on
 * the device as soon as it completes, while the rest render.  Each frame's size is its first genome's width x height.
 * pngs[i] receives a malloc'd PNG (release with free), lens[i] its size,
 * stats[i] the frame's statistics; the text chunks carry the statistics
 * (no genome).  Returns 0, or 1 when any frame failed. */
int flam3gpu_render_batch_png(flam3_frame *frames, int n, int transp, stat_struct *stats, unsigned char **pngs,
                              size_t *lens);

/* Kernel time (ms, CUDA events) of the calling thread's last PNG encode. */
int flam3gpu_png_last_ms(double *encode_ms);

/* Last error message of the calling thread ("" if none). */
const char *flam3gpu_last_error(void);

/* Version string of the library build. */
const char *flam3gpu_version(void);

/* Execution options (no counterpart in the reference; defaults are chosen by
 * the library).  iter_mode: 0 = one independent chain per thread, xform picked
 * per thread (the reference's semantics); 1 = warp-coherent xform choice with
 * a point exchange between the block's warps every `shuffle_every` steps
 * (default, every 3 steps: the image error against a 16x-quality render is
 * within 0.2 % of mode 0's).  Genomes with non-unity xaos, and blocks of
 * fewer than 128 threads (too few warps to exchange with), always use mode
 * 0.  iter_precision: 32 or 64 (FP64
 * iteration, slow on GB300; parity work).  threads_per_block, blocks: 0 =
 * automatic.  chain_samples: samples per chain before a restart with a new
 * random point and fuse (at most f->sub_batch_size, like the reference).
 * de_tile: output pixels per tile edge of the fused density-estimation
 * kernel (8 .. 32; 0 = 16).  de_kernel: 0 = density estimation by owner
 * bands (register accumulators, no atomics; default), 1 = the fused tile
 * kernel (DE, filter and tonemap in one pass, shared-memory scatter).
 * de_stats: 1 = band DE runs an instrumented variant that counts its work
 * (sources, source-band pairs, taps), read with flam3gpu_last_de_work.
 * float_buckets: 0 = the reference's integer arithmetic for bits 32 and 33
 * (each hit's channels truncated before the add, and for bits 32 the
 * log-scaled accumulator truncated too, flam3.c:3642-3647, 3688-3703,
 * 3771-3856); 1 = exact FP32 sums (more accurate than the reference).
 * chain_samples 0: 1024, or 2048 when a launch holds at least 8 waves of
 * 2048-sample chains.  tail_chain_samples, tail_wave_pct: the last samples
 * of each iterate launch (half a wave of full chunks, a whole wave with
 * 2048-sample chains) run in chunks a quarter as long, so the blocks finish
 * close together; the chunking is fixed when a render is planned (the same
 * for the plain and the served render of a frame).
 * test_exchange_stall: tests only (failure detection of the point
 * exchange; no fault): see the field.
 * host_plan: 0 = the temporal samples of frames with several genomes
 * (animation, motion blur) are interpolated, prepared and packed on the
 * device, one block per sample; 1 = on host threads (always for one genome,
 * and when a caller interpolator is installed). */
typedef struct {
  int iter_mode;
  int iter_precision;
  int shuffle_every;
  int threads_per_block;
  int blocks;
  int chain_samples;
  uint64_t seed_salt;
  int de_tile;        /* output-tile edge of the fused DE kernel (0 = 16) */
  int de_kernel;      /* 0 owner bands (default), 1 fused tile */
  int de_stats;       /* 1: band DE counts its work (flam3gpu_last_de_work) */
  int float_buckets;  /* 1: bits 32/33 keep exact FP32 sums (no per-hit truncation) */
  int host_plan;      /* 1: plan every temporal sample on host threads (0: multi-genome frames on the device) */
  int tail_chain_samples; /* samples per thread of the launch's last chunks (0: chain length / 4; -1: none) */
  int tail_wave_pct;  /* those chunks hold this percentage of one wave of full chunks (0: 50, 100 for 2048-sample chains) */
  int test_exchange_stall; /* tests only: 1 makes one block of the next iterate launch withhold a point-exchange
                              arrival, so its waits run out (2 s) and the render fails with that error */
} flam3gpu_options;

void flam3gpu_default_options(flam3gpu_options *o);
int flam3gpu_set_options(const flam3gpu_options *o);
void flam3gpu_get_options(flam3gpu_options *o);

/* Measurements of the last flam3gpu_render call on this thread (no
 * counterpart in the reference): [0] iterate+accumulate kernel time, [1]
 * density estimation / log scaling, [2] filter+tonemap+pack (ms, CUDA events
 * on the library's stream), [3] wall time of the whole call (ms), [4] kernel
 * launches, [5] host-to-device bytes, [6] device-to-host bytes, [7] samples
 * plotted by the iterate kernels. */
int flam3gpu_last_timings(double t[8]);

/* Work of the last render's band density estimation on this thread (no
 * counterpart in the reference), counted only while the de_stats option is
 * set: [0] sources (non-empty buckets inside the DE bounds), [1] source x
 * 8-row-band pairs the kernel processed, [2] kernel taps (bucket updates
 * inside the kernels' discs). */
int flam3gpu_last_de_work(double w[3]);

/* Replaces flam3_interpolate (flam3.h:562, flam3.c:717-802): the genome at
 * `time` between control points cps[0..ncps-1] (sorted by time), with the
 * reference's alignment (flam3_align), linear or Catmull-Rom blending,
 * log-polar or linear matrix interpolation, palette blending and xform
 * stagger.  `result` is overwritten (not freed first); release it with
 * flam3gpu_free_genome.  Smooth interpolation on the first or last segment
 * falls back to linear (the reference reads past the control points there).
 * flam3gpu_render uses this function for frames with several genomes unless
 * flam3gpu_set_interpolator installed another one, e.g. the reference's own
 * flam3_interpolate when the caller links it. */
int flam3gpu_interpolate(flam3_genome *cps, int ncps, double time, double stagger, flam3_genome *result);
void flam3gpu_free_genome(flam3_genome *g);
void flam3gpu_set_interpolator(void (*fn)(flam3_genome *cps, int ncps, double time, double stagger,
                                          flam3_genome *result));

#ifdef __cplusplus
}
#endif

#include "flam3_gpu_kernels.h"

#endif /* FLAM3_GPU_H */
