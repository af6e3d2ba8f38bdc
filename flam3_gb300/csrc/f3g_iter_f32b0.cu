/*
 * f3g_iter_f32b0.cu -- instantiation of the iterate kernel for FP32 iteration, variations 0-19, per-thread xform choice.
 */
#include "f3g_iterate.cuh"

extern "C" int f3g_iterate_occ_f32b0(int threads) {
  int nb = 0;
  size_t smem = f3g::iterate_smem<float>(threads);
  if (cudaFuncSetAttribute(f3g::k_iterate<float, false, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, f3g::k_iterate<float, false, 0>, threads, smem) !=
      cudaSuccess)
    return 0;
  return nb;
}

extern "C" int f3g_iterate_launch_f32b0(const F3GItem *d_items, const long long *d_prefix, int nitems,
                                       long long total_chunks, int shuffle_every, int threads, int blocks,
                                       F3GCounters *d_ctr, cudaStream_t st) {
  return (int)f3g::launch_iterate_t<float, false, 0>(d_items, d_prefix, nitems, total_chunks, shuffle_every, threads,
                                                         blocks, d_ctr, st);
}
