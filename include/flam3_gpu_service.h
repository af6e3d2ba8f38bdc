/*
 * flam3_gpu_service.h -- batched and served rendering on one GPU.
 *
 * No counterpart in the reference: flam3_render (flam3.h:623) renders one
 * frame per call on the calling thread.  These entry points keep its
 * arguments and output contract per frame, and run many frames at once:
 *
 *   - a service owns a host scheduling thread, CUDA streams and a device
 *     memory pool; requests (stills, animation frames, any size) are
 *     submitted from any thread and admitted while their device buffers fit
 *     the service's HBM budget;
 *   - the scheduler runs iteration in rounds: each round is one persistent
 *     iterate-and-accumulate launch over slices of every admitted job's
 *     temporal samples (per-job work lists in one chunk queue), shortest
 *     remaining job first; rounds may alternate over several streams;
 *   - jobs whose iteration finished in a round get their density
 *     estimation / filter / tonemap / copy-out as CUDA graphs: one
 *     executable graph per tail shape, updated in place for each job;
 *   - requests that arrive while others run join at the next round
 *     (continuous batching); histograms, pass tables and chunk cursors stay
 *     resident on the device between rounds.
 *
 * A job's samples do not depend on what else runs: chunk k of every
 * temporal sample draws the same random stream alone or in a mix, so a
 * served result equals flam3gpu_render's result for the same frame up to
 * the order of floating-point atomic additions.
 *
 * Each call returns 0 on success and nonzero on failure, with the message in
 * flam3gpu_last_error() of the calling thread.
 */
#ifndef FLAM3_GPU_SERVICE_H
#define FLAM3_GPU_SERVICE_H

#include <stdint.h>

#include "flam3_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct flam3gpu_service flam3gpu_service;

typedef struct {
  double hbm_budget_bytes;  /* device bytes held for job buffers (0: 150 GB or 90% of free memory) */
  long long round_samples;  /* samples per iterate round (0: automatic -- at least 2e8 samples and
                               4 chunks per resident block; -1: one round holds all admitted work) */
  int max_active;           /* admitted jobs at once (0: unlimited) */
  int tail_graphs;          /* 1 (default): each job's tail is a CUDA graph per tail shape, updated in
                               place for the next job of that shape; 2: one graph per round with
                               tail_branches parallel branches; 0: direct launches */
  int streams;              /* iterate streams rounds alternate over (default 1; with 2 the next
                               round's blocks fill the SMs a draining round frees) */
  int use_tuning;           /* 1: apply the autotuned table (flam3gpu_autotune) to new jobs */
  int max_inflight;         /* iterate rounds queued on the device at once (default 2) */
  int tail_branches;        /* parallel branches of a round's tail graph with tail_graphs 2 (default 1) */
  int order;                /* which admitted jobs a round serves first: 1 (default) the highest
                               response ratio, (waiting time + remaining time) / remaining time, so short
                               jobs pass long ones and long jobs gain priority as they wait; 0 the
                               shortest remaining work; 2 arrival order */
  int reserved[5];
} flam3gpu_service_config;

void flam3gpu_service_default_config(flam3gpu_service_config *cfg);

/* Creates a service on the current CUDA device.  NULL on failure. */
flam3gpu_service *flam3gpu_service_create(const flam3gpu_service_config *cfg);

/* Queues one render with flam3_render's arguments.  The frame and its
 * genomes are copied (the caller may reuse them at once) and f->rc is
 * advanced now, exactly as flam3_render would advance it.  `out` must stay
 * valid until the job completes.  *ticket identifies the job.  A frame's
 * progress callback (f->progress, f->progress_parameter) is called on the
 * service thread before each iterate round the job could take part in, with
 * the percentage of its samples done and stage 0: returning 1 aborts the
 * job (no further rounds and no filtering; it completes with 0 and leaves
 * `out` as it stands, as flam3_render's abort does, rect.c:919-922),
 * returning 2 pauses it (it is left out of rounds and asked again about
 * every 10 ms). */
int flam3gpu_service_submit(flam3gpu_service *s, flam3_frame *f, void *out, int field, int nchan, int transp,
                            uint64_t *ticket);

/* Queues n renders at once: they are planned on up to 16 host threads and
 * admitted together, so one round can hold all of them.  tickets[i] is 0
 * for a frame whose planning failed (the call then returns 1). */
int flam3gpu_service_submit_many(flam3gpu_service *s, flam3_frame *frames, int n, void **outs, int field, int nchan,
                                 int transp, uint64_t *tickets);

/* Waits for a job (timeout_ms < 0: no limit).  Returns 0 when it finished
 * successfully (stats filled like flam3_render's), 1 when it failed, 2 on
 * timeout.  times_ms (may be NULL) receives [0] submit -> admitted,
 * [1] admitted -> first iterate round, [2] submit -> done (latency),
 * [3] iterate rounds the job took part in. */
int flam3gpu_service_wait(flam3gpu_service *s, uint64_t ticket, double timeout_ms, stat_struct *stats,
                          double times_ms[4]);

/* Waits for every submitted job. */
int flam3gpu_service_drain(flam3gpu_service *s);

/* Counters since creation: [0] jobs done, [1] jobs failed, [2] iterate rounds,
 * [3] kernel launches, [4] tail graphs launched, [5] tail graphs
 * instantiated, [6] samples plotted, [7] device bytes in use, [8] peak device
 * bytes, [9] busy seconds (first admission to last completion),
 * [10] host-to-device bytes, [11] device-to-host bytes; service-thread
 * seconds spent [12] admitting jobs, [13] building and launching rounds,
 * [14] capturing and launching tails, [15] completing jobs (copy-out),
 * [16] waiting for the GPU; device seconds (CUDA events) of [17] iterate
 * rounds and [18] tails (rounds on different streams overlap, so [17] can
 * exceed the wall time). */
void flam3gpu_service_counters(flam3gpu_service *s, double out[19]);

/* Waits for all jobs and releases the service. */
void flam3gpu_service_destroy(flam3gpu_service *s);

/* Renders n frames through a temporary service (one persistent launch per
 * round over all of them) and waits for all.  outs[i], stats[i] as for
 * flam3_render; field, nchan and transp apply to every frame. */
int flam3gpu_render_batch(flam3_frame *frames, int n, void **outs, int field, int nchan, int transp,
                          stat_struct *stats, const flam3gpu_service_config *cfg);

/* Autotuner.  Renders each frame (at reduced quality) with every candidate
 * of the knobs below, keeps the fastest per frame class (output size, bits,
 * oversample, estimator radius) in the process-wide table, and returns the
 * number of classes tuned:
 *   chains per job  -- samples per chain (the chunk length) S in {128 .. 1024};
 *   DE tile shape   -- density estimation by owner bands (32 x 64 bucket
 *                      tiles) or the fused density-estimation kernel with
 *                      an output-tile edge in {8, 16, 32}.
 * Services created with use_tuning apply the table to new jobs. */
int flam3gpu_autotune(flam3_frame *frames, int n, double quality_scale);
/* Writes / reads the table as text ("key S tile" per line). */
int flam3gpu_autotune_save(const char *path);
int flam3gpu_autotune_load(const char *path);
/* Empties the table. */
void flam3gpu_autotune_clear(void);

#ifdef __cplusplus
}
#endif
#endif
