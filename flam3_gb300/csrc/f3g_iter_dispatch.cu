/*
 * f3g_iter_dispatch.cu -- selects the iterate-kernel instantiation for a
 * launch (iteration precision, variation set).
 */
#include <cuda_runtime.h>

#include "f3g_launch.h"

#define DECL(tag)                                                                                         \
  extern "C" int f3g_iterate_occ_##tag(int threads);                                                      \
  extern "C" int f3g_iterate_launch_##tag(const F3GPass *, const long long *, int, long long, int, int, int, \
                                          int, F3GCounters *, cudaStream_t);
DECL(f32b)
DECL(f32f)
DECL(f64b)
DECL(f64f)

extern "C" int f3g_iterate_occupancy(int precision, int full, int threads) {
  if (precision == 64) return full ? f3g_iterate_occ_f64f(threads) : f3g_iterate_occ_f64b(threads);
  return full ? f3g_iterate_occ_f32f(threads) : f3g_iterate_occ_f32b(threads);
}

extern "C" int f3g_launch_iterate(const F3GPass *d_passes, const long long *d_prefix, int npasses,
                                  long long total_chunks, int S, int shuffle_every, int precision, int full,
                                  int threads, int blocks, F3GCounters *d_ctr, cudaStream_t st) {
  if (precision == 64)
    return full ? f3g_iterate_launch_f64f(d_passes, d_prefix, npasses, total_chunks, S, shuffle_every, threads,
                                          blocks, d_ctr, st)
                : f3g_iterate_launch_f64b(d_passes, d_prefix, npasses, total_chunks, S, shuffle_every, threads,
                                          blocks, d_ctr, st);
  return full ? f3g_iterate_launch_f32f(d_passes, d_prefix, npasses, total_chunks, S, shuffle_every, threads, blocks,
                                        d_ctr, st)
              : f3g_iterate_launch_f32b(d_passes, d_prefix, npasses, total_chunks, S, shuffle_every, threads, blocks,
                                        d_ctr, st);
}
