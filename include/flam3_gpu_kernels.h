/*
 * flam3_gpu_kernels.h -- kernel-level C ABI of libflam3gpu (plain pointers
 * and sizes).  Included by flam3_gpu.h; see there for the drop-in entry.
 */
#ifndef FLAM3_GPU_KERNELS_H
#define FLAM3_GPU_KERNELS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Optional inputs/outputs of flam3gpu_render_ex.  No counterpart in the
 * reference: they expose the intermediate buffers of render_rectangle
 * (rect.c:685-701) for parity checks.
 *   hist_in  : skip iteration; every batch uses this host histogram
 *              (hist_h rows x hist_w buckets x 5 doubles: R,G,B,A,count).
 *   hist_out : receives the last batch's histogram in the same layout.
 *   accum_out: receives the accumulator before the spatial filter
 *              (hist_h x hist_w x 4 doubles).
 *   hist_w, hist_h: set by the call.
 *   keep_on_device: the packed image stays in the calling thread's device
 *              buffer for a following device step (flam3gpu_render_png);
 *              `out` is not written and may be NULL.
 *   image_w, image_h: the packed image's size, set by the call. */
typedef struct {
  const double *hist_in;
  double *hist_out;
  double *accum_out;
  int hist_w, hist_h;
  int keep_on_device;
  int image_w, image_h;
  int reserved[3];
} flam3gpu_render_io;

/* flam3gpu_render with optional parity inputs/outputs (io may be NULL). */
int flam3gpu_render_ex(flam3_frame *f, void *out, int field, int nchan, int transp,
                       stat_struct *stats, flam3gpu_render_io *io);

/* Histogram geometry that a render of f would use (rect.c:613-687):
 * bucket-array width/height including the gutter, gutter width, DE offset
 * and spatial filter width. */
int flam3gpu_histogram_dims(flam3_frame *f, int field, int *w, int *h, int *gutter,
                            int *de_offset, int *filter_width);

/* GPU apply_xform (variations.c:2129-2399) on n points: xform `fn` of genome
 * cp (prepared on the host exactly as prepare_precalc_flags/xform_precalc
 * do), p_in/q_out are n x 4 doubles (x, y, color, opacity) in host memory,
 * random draws for point k are words[k*wpp ...] consumed in order, bad_out[k]
 * receives apply_xform's return value.  precision 64 computes in FP64,
 * precision 32 in FP32 (inputs rounded to float). */
int flam3gpu_apply_xform(flam3_genome *cp, int fn, int n, const double *p_in,
                         const uint32_t *words, int wpp, double *q_out, int *bad_out,
                         int precision);

/* The GPU's xform choice for every 14-bit random value of every row of the
 * genome's choice table: table[r*16384 + v] is the xform the iterate kernel
 * picks for value v in row r (row 0 from the xform weights, row 1+i after
 * xform i when xaos is on).  Replaces the table flam3_create_xform_distrib
 * builds (flam3.h:575, flam3.c:165-224), which the kernels hold as
 * breakpoints; the caller passes room for (standard xforms + 1) * 16384
 * entries and receives the row count in *rows. */
int flam3gpu_xform_choice_table(flam3_genome *cp, uint16_t *table, int *rows);

/* Host probe of the iterate launch's chunking (no GPU): for passes of
 * samples[0..n) in one launch of `blocks` blocks of `threads`, the chain
 * length S the render picks (f->sub_batch_size as sub_batch_size), the
 * short-chunk length S_tail, and per pass the first short chunk and the chunk
 * count.  Chunk c of pass i holds threads*S samples below chunk_tail[i],
 * threads*S_tail from there (the last one fewer). */
int flam3gpu_chunk_plan(const long long *samples, int n, int threads, int blocks, int sub_batch_size, int *S,
                        int *S_tail, long long *chunk_tail, long long *nchunks);

/* Host probe of one choice row (no GPU): the breakpoints of the row with
 * xform weights d[0..nx) (times the row's chaos entries c[0..nstd), or c NULL
 * for the raw-weight row), built by the reference's 16384-step loop
 * (flam3.c:165-224; walk = 0) or by the binade walk the device planner uses
 * (walk = 1).  brk gets up to 32 entries, *nbrk their count, *moves (if not
 * NULL) the sequential steps taken (16384 for the loop; real steps plus
 * closed-form runs for the walk); returns 1 with the reference's errors
 * (negative or all-zero weights, a walk past the last xform). */
int flam3gpu_choice_breakpoints(const double *d, const double *c, int nstd, int nx, int walk, uint16_t *brk,
                                int *nbrk, int *moves);

/* The passes (per temporal sample: interpolated genome, prepared xforms,
 * choice rows, colour map, camera) that flam3gpu_render would build for the
 * first batch of frame f, planned on the device (on_device = 1) or on host
 * threads (0), copied to `passes` as sizeof(F3GPass) records (at most
 * max_passes); nothing is rendered and f->rc advances as a render's would.
 * No counterpart in the reference: the parity probe of the device planner
 * against the host's restatement of flam3_interpolate (flam3.c:717-802) and
 * rect.c:754-827.  Returns the number of passes, -1 on failure. */
int flam3gpu_plan_passes(flam3_frame *f, int on_device, void *passes, int max_passes);
/* sizeof the pass record flam3gpu_plan_passes writes */
size_t flam3gpu_pass_bytes(void);

/* GPU bucket accumulation (rect.c:411-516) of a host point stream
 * (n x 4 doubles) for genome f->genomes[0] at f->time; adds into a host FP64
 * 5-channel histogram of the render's geometry.  bits selects the device
 * bucket type (33/32: FP32, 64: FP64). */
int flam3gpu_accumulate_points(flam3_frame *f, int field, const double *points, long n,
                               double *hist, int *hist_w, int *hist_h);

/* GPU chaos game for parity work: nchains independent chains of flam3_iterate
 * (flam3.c:232-299) with fuse discarded steps and n stored steps each,
 * starting from starts[4*c..], random words from the counter-based stream
 * keyed by `seed` (chain c uses counter (c, step/4, 0, 0) ...).  samples
 * receives nchains x n x 4 doubles; returns the total bad-value count in
 * *badvals. */
int flam3gpu_iterate_chains(flam3_genome *cp, int nchains, int n, int fuse,
                            const double *starts, uint64_t seed, double *samples,
                            long *badvals, int precision);

/* flam3_estimate_bounding_box (flam3.h:588, flam3.c:3574-3640) on the GPU: same
 * arguments, eps rule and return value (bad values met, -1 on failure); the
 * nsamples points come from chains of 1024 samples after 20 fuse steps
 * (the reference: one chain) drawn with the counter-based stream, so the box
 * matches the reference's statistically, not bit for bit.  Start points and
 * the stream key are drawn from rc. */
int flam3gpu_estimate_bounding_box(flam3_genome *cp, double eps, int nsamples, double *bmin, double *bmax,
                                   randctx *rc);

/* flam3_colorhist (flam3.h:587, flam3.c:351-391) on the GPU: hist[256] is the
 * normalised histogram of the colour coordinate over num_batches chains of
 * 10000 samples after 20 fuse steps.  Returns 0 on success. */
int flam3gpu_colorhist(flam3_genome *cp, int num_batches, randctx *rc, double *hist);

/* flam3_dimension (flam3.h:592, flam3.c:3949-4052) on the GPU: the
 * correlation dimension from ntries attractor points (optionally clipped to
 * the camera) and ntries random pairs; same formula, defaults (ntries < 2:
 * 3 000 000) and failure values (-1; NaN when clipping rejects more than
 * 10 * ntries points).  Points and pair partners are drawn from rc (the
 * reference: a private time-seeded ISAAC context and libc random()), so the
 * estimate matches the reference's statistically. */
double flam3gpu_dimension(flam3_genome *cp, int ntries, int clip_to_camera, randctx *rc);

/* flam3_lyapunov (flam3.h:593, flam3.c:4054-4150) on the GPU: mean
 * log2(distance / 1e-5) after one step from an attractor point and one from a
 * point 1e-5 away, over ntries tries (ntries < 1: 10000), in FP64; draws
 * from rc.  Returns -1 on failure. */
double flam3gpu_lyapunov(flam3_genome *cp, int ntries, randctx *rc);

/* Ceiling probe (no counterpart in the reference): float4 atomic adds per
 * second at pseudo-random buckets of an nbuckets histogram, natomics adds in
 * one timed launch over every SM; the bucket update of the chaos game is one
 * such add per plotted sample.  Returns 0 on success. */
int flam3gpu_measure_atomic_rate(long long nbuckets, long long natomics, double *per_second);

/* flam3gpu_render without device allocation.  No counterpart in the
 * reference: for callers that cannot call cudaMalloc (plug-in hosts whose
 * memory pool owns every device allocation, services with a device-memory
 * budget fixed at start-up).  Same arguments, output and errors as
 * flam3gpu_render, but all device scratch (histogram, pass tables, filter
 * tables, staged image) comes from one static device array of
 * flam3gpu_noalloc_capacity() bytes (48 MiB) that every GPU loading the
 * library holds until exit; it calls no cudaMalloc or cudaFree, and its
 * copies are blocking cudaMemcpy calls on the legacy default stream.  Renders
 * of one batch only, and only those whose scratch fits the array (roughly
 * 1.5 M FP32 or 0.75 M FP64 histogram buckets including the gutter); anything
 * larger returns 1 with an error naming the sizes.  Calls share the array:
 * each clears the histogram first, and calls that overlap on the GPU race.
 * Each call looks up the array's address on the current device
 * (cudaGetSymbolAddress). */
int flam3gpu_render_noalloc(flam3_frame *f, void *out, int field, int nchan, int transp, stat_struct *stats);
size_t flam3gpu_noalloc_capacity(void);

#ifdef __cplusplus
}
#endif
#endif
