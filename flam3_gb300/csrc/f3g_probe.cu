/*
 * f3g_probe.cu -- launch wrappers of the parity probe kernels
 * (apply_xform on given words, point-stream accumulation, recorded chains).
 */
#include "f3g_iterate.cuh"

extern "C" int f3g_launch_apply_xform(const F3GPass *d_pass, int fn, int n, const double *d_pin,
                                      const uint32_t *d_words, int wpp, double *d_qout, int *d_bad, int precision,
                                      cudaStream_t st) {
  int blocks = (n + 255) / 256;
  if (blocks < 1) blocks = 1;
  cudaError_t e;
  if (precision == 64) {
    size_t smem = sizeof(f3g::PassS<double>);
    cudaFuncSetAttribute(f3g::k_apply_xform<double, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    f3g::k_apply_xform<double, true><<<blocks, 256, smem, st>>>(d_pass, fn, n, d_pin, d_words, wpp, d_qout, d_bad);
  } else {
    size_t smem = sizeof(f3g::PassS<float>);
    cudaFuncSetAttribute(f3g::k_apply_xform<float, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    f3g::k_apply_xform<float, true><<<blocks, 256, smem, st>>>(d_pass, fn, n, d_pin, d_words, wpp, d_qout, d_bad);
  }
  e = cudaGetLastError();
  return (int)e;
}

extern "C" int f3g_launch_accumulate(const F3GPass *d_pass, const double *d_points, long long n, cudaStream_t st) {
  long long b = (n + 255) / 256;
  if (b > 1024) b = 1024;
  if (b < 1) b = 1;
  size_t smem = sizeof(f3g::PassS<double>);
  cudaFuncSetAttribute(f3g::k_accumulate, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  f3g::k_accumulate<<<(int)b, 256, smem, st>>>(d_pass, d_points, n);
  return (int)cudaGetLastError();
}

extern "C" int f3g_launch_iterate_chains(const F3GPass *d_pass, int nchains, int n, int fuse, const double *d_starts,
                                         uint32_t key0, uint32_t key1, double *d_samples, unsigned long long *d_bad,
                                         int precision, cudaStream_t st) {
  int blocks = (nchains + 255) / 256;
  if (blocks < 1) blocks = 1;
  if (precision == 64) {
    size_t smem = sizeof(f3g::PassS<double>);
    cudaFuncSetAttribute(f3g::k_iterate_chains<double, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    f3g::k_iterate_chains<double, true><<<blocks, 256, smem, st>>>(d_pass, nchains, n, fuse, d_starts, key0, key1,
                                                                   d_samples, d_bad);
  } else {
    size_t smem = sizeof(f3g::PassS<float>);
    cudaFuncSetAttribute(f3g::k_iterate_chains<float, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    f3g::k_iterate_chains<float, true><<<blocks, 256, smem, st>>>(d_pass, nchains, n, fuse, d_starts, key0, key1,
                                                                  d_samples, d_bad);
  }
  return (int)cudaGetLastError();
}

extern "C" int f3g_launch_xform_choice(const F3GPass *d_pass, int rows, uint16_t *d_out, cudaStream_t st) {
  const size_t smem = sizeof(f3g::PassS<float>);
  cudaFuncSetAttribute(f3g::k_xform_choice, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const int blocks = (rows * F3G_GRAIN + 255) / 256;
  f3g::k_xform_choice<<<blocks, 256, smem, st>>>(d_pass, rows, d_out);
  return (int)cudaGetLastError();
}

/* ---------------------------------------------------------------------
 * Ceiling probe for the iterate kernel's roofline: float4 atomic adds
 * (red.global.add.v4.f32, the bucket update of plot()) at pseudo-random
 * buckets of a histogram-sized buffer, every lane its own bucket.
 * ------------------------------------------------------------------- */
namespace f3g {
__global__ void __launch_bounds__(256) k_atomic_rate(float4 *buf, unsigned long long nbuckets, int per_thread,
                                                     uint32_t salt) {
  uint32_t h = (blockIdx.x * blockDim.x + threadIdx.x) * 0x9E3779B1u ^ salt;
  const float4 one = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
  for (int i = 0; i < per_thread; i++) {
    /* xorshift32: a new bucket per add */
    h ^= h << 13;
    h ^= h >> 17;
    h ^= h << 5;
    const unsigned long long b = (unsigned long long)h * nbuckets >> 32;
    atomicAdd(buf + b, one);
  }
}
}  // namespace f3g

extern "C" int f3g_launch_atomic_rate(float4 *buf, unsigned long long nbuckets, int blocks, int per_thread,
                                      uint32_t salt, cudaStream_t st) {
  f3g::k_atomic_rate<<<blocks, 256, 0, st>>>(buf, nbuckets, per_thread, salt);
  return (int)cudaGetLastError();
}
