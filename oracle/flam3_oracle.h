/*
 * flam3_oracle.h -- TEST ORACLE, not product code.
 *
 * A plain-C, FP64 restatement of the reference flam3 render path
 * (rect.c render_rectangle, flam3.c flam3_iterate / xform distribution,
 * variations.c apply_xform and var0..var98, filters.c, palettes.c tonemap
 * helpers, isaac.c).  It operates on the same flam3_frame / flam3_genome
 * layout as the reference (mirrored in include/flam3_gpu.h) and is used by
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg to check
 * and time the CUDA path.  The product never links it.
 *
 * Parity status: pinned.  Compiled with IEEE-faithful flags on x86-64 it
 * reproduces the reference (built unmodified from its sources with the same
 * flags, oracle/_ref/libflam3ref_strict.so) bit for bit on whole renders
 * and per-variation vectors; tests/golden/ holds vectors generated from the
 * reference by tests/golden/make_golden.py.
 */
#ifndef FLAM3_ORACLE_H
#define FLAM3_ORACLE_H

#include "flam3_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* isaac.c / isaac.h restated (RANDSIZL 4, ub4 = unsigned long) */
void f3o_isaac(randctx *r);
void f3o_irandinit(randctx *r, int flag);
unsigned long f3o_irand(randctx *r);
/* flam3.c:2494-2516 with a caller-given seed string (isaac_seed) */
void f3o_init_rc(randctx *r, const char *seed);

/* variations.c:2016-2126 and 1942-2014 */
int f3o_prepare_precalc_flags(flam3_genome *cp);
void f3o_xform_precalc(flam3_genome *cp, int xi);

/* flam3.c:76-111: returns a malloc'd (rows x 16384) table, NULL on error */
unsigned short *f3o_create_xform_distrib(flam3_genome *cp);

/* Apply xform `fn` of cp (already prepared) to n points p_in[4n] -> q_out[4n].
 * Random draws come from `words`: point k uses words[k*wpp ...] in order.
 * bad_out[k] = apply_xform's return value (1 when the result was a bad value
 * and was replaced with a random point).  variations.c:2129-2399. */
int f3o_apply_xform(flam3_genome *cp, int fn, int n, const double *p_in,
                    const uint32_t *words, int wpp, double *q_out, int *bad_out);

/* filters.c:217-270 (returns width, -1 on error; *filter malloc'd) */
int f3o_create_spatial_filter(flam3_frame *spec, int field, double **filter);
/* filters.c:272-407; arrays malloc'd; returns kernel_size (-1 on error) */
int f3o_create_de_filters(double max_rad, double min_rad, double curve, int ss,
                          int *max_filtered_counts, int *max_filter_index,
                          double **filter_widths, double **filter_coefs);
/* filters.c:409-489 */
double f3o_create_temporal_filter(int numsteps, int filter_type, double filter_exp,
                                  double filter_width, double **temporal_filter,
                                  double **temporal_deltas);
/* palettes.c:274-290, 292-349 */
double f3o_calc_alpha(double density, double gamma, double linrange);
void f3o_calc_newrgb(double *cbuf, double ls, double highpow, double *newrgb);

/* Optional inputs/outputs of a render, for parity work. */
typedef struct {
  const double *hist_in; /* if set: iteration is skipped and every batch uses
                            this histogram (W_h*H_h*5 doubles, R,G,B,A,count) */
  double *hist_out;      /* if set: the last batch's histogram (same layout) */
  double *accum_out;     /* if set: the accumulator before the spatial filter
                            (W_h*H_h*4 doubles) */
  int hist_w, hist_h;    /* out: histogram dimensions incl. gutter */
  int nthreads_used;     /* out: worker threads used for iteration */
} f3o_render_io;

/* rect.c:529-1286 restated.  Honors f->bits (32/33/64), f->nthreads (ISAAC
 * streams and worker threads), f->sub_batch_size, earlyclip,
 * bytes_per_channel, field, nchan, transp.  Multi-genome frames call the
 * interpolator installed by f3o_set_interpolator (flam3_interpolate's
 * arguments, flam3.c:717; nonzero return on failure) once per temporal sample and per batch, as
 * rect.c:592/726/763 call flam3_interpolate. */
void f3o_set_interpolator(int (*fn)(flam3_genome *, int, double, double, flam3_genome *));
int f3o_render(flam3_frame *f, void *out, int field, int nchan, int transp, stat_struct *stats);
int f3o_render_ex(flam3_frame *f, void *out, int field, int nchan, int transp,
                  stat_struct *stats, f3o_render_io *io);

/* Accumulate a point stream into a FP64 5-channel histogram the way
 * iter_thread does (rect.c:411-516) for genome f->genomes[0] at f->time,
 * temporal sample 0.  hist has W_h*H_h*5 doubles and is added to. */
int f3o_accumulate_points(flam3_frame *f, int field, const double *points, long n,
                          double *hist, int *hist_w, int *hist_h);

/* Chains replaying the CUDA path's Philox stream (see flam3_oracle.c). */
int f3o_iterate_chains(flam3_genome *cp, int nchains, int n, int fuse, const double *starts, uint64_t seed,
                       double *samples, long *badvals);

/* Counter-based stream used by the CUDA path (Philox4x32-10), exposed so the
 * oracle can replay the GPU's random words. */
void f3o_philox4x32(uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

#ifdef __cplusplus
}
#endif
#endif
