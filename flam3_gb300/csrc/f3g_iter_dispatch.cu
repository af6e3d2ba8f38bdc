/*
 * f3g_iter_dispatch.cu -- selects the iterate-kernel instantiation for a
 * launch (iteration precision, variation set, xform-choice mode).
 */
#include <cuda_runtime.h>

#include "f3g_launch.h"

#define DECL(tag)                                                                                         \
  extern "C" int f3g_iterate_occ_##tag(int threads);                                                      \
  extern "C" int f3g_iterate_launch_##tag(const F3GItem *, const long long *, int, long long, int, int, int, \
                                          F3GCounters *, cudaStream_t);
DECL(f32b0)
DECL(f32b1)
DECL(f32f0)
DECL(f32f1)
DECL(f64b0)
DECL(f64b1)
DECL(f64f0)
DECL(f64f1)

typedef int (*occ_fn)(int);
typedef int (*launch_fn)(const F3GItem *, const long long *, int, long long, int, int, int, F3GCounters *,
                         cudaStream_t);
/* index: precision64 * 4 + full * 2 + mode */
static const occ_fn occ_tab[8] = {f3g_iterate_occ_f32b0, f3g_iterate_occ_f32b1, f3g_iterate_occ_f32f0,
                                  f3g_iterate_occ_f32f1, f3g_iterate_occ_f64b0, f3g_iterate_occ_f64b1,
                                  f3g_iterate_occ_f64f0, f3g_iterate_occ_f64f1};
static const launch_fn launch_tab[8] = {f3g_iterate_launch_f32b0, f3g_iterate_launch_f32b1, f3g_iterate_launch_f32f0,
                                        f3g_iterate_launch_f32f1, f3g_iterate_launch_f64b0, f3g_iterate_launch_f64b1,
                                        f3g_iterate_launch_f64f0, f3g_iterate_launch_f64f1};

static int idx(int precision, int full, int mode) {
  return (precision == 64 ? 4 : 0) + (full ? 2 : 0) + (mode ? 1 : 0);
}

extern "C" int f3g_iterate_occupancy(int precision, int full, int mode, int threads) {
  return occ_tab[idx(precision, full, mode)](threads);
}

extern "C" int f3g_launch_iterate(const F3GItem *d_items, const long long *d_prefix, int nitems,
                                  long long total_chunks, int shuffle_every, int precision, int full, int mode,
                                  int threads, int blocks, F3GCounters *d_ctr, cudaStream_t st) {
  return launch_tab[idx(precision, full, mode)](d_items, d_prefix, nitems, total_chunks, shuffle_every, threads,
                                                blocks, d_ctr, st);
}
