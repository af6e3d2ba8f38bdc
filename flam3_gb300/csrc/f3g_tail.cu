/*
 * f3g_tail.cu -- the render tail: log-density scaling, density estimation,
 * spatial filter, gamma/vibrancy/highlight tonemap and 8/16-bit packing.
 *
 * Replaces rect.c:933-974 (k1/k2 log scaling), rect.c:57-251 (de_thread),
 * rect.c:1067-1247 (earlyclip, filter, tonemap, pack) and the helpers of
 * palettes.c:199-349.  Arithmetic is FP32 (FP64 reads when the histogram is
 * FP64).
 *
 * Kernels (density estimation is in f3g_de.cu):
 *   k_logscale        acc += ls(bucket) * bucket           (no DE)
 *   k_earlyclip       tonemap the accumulator in place     (earlyclip=1)
 *   k_filter_tonemap  spatial filter + tonemap + pack      (one output pixel per thread)
 *   k_fused_log_filter: log scaling + filter + tonemap + pack in one pass over
 *                     the histogram, for one batch without DE
 *   k_log_filter_strip (f3g_strip.cuh): the same pass with the filter
 *                     applied as its two 1-D factors, streaming histogram
 *                     rows through shared memory; used for oversample 1
 *                     with filter widths 1..7 and oversample 2 with 2..16
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "f3g_common.h"
#include "f3g_launch.h"
#include "f3g_tail.cuh"

namespace f3g {

/* ---------------------------------------------------------------------
 * kernels
 * ------------------------------------------------------------------- */
__global__ void k_logscale(const void *__restrict__ buckets, int bkind, long long n, float k1, float k2, void *acc,
                           int akind, int trunc) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float4 c = load_bucket(buckets, bkind, i);
    if (c.w == 0.0f) continue;
    float ls = log_scale(c.w, k1, k2);
    float4 v = make_float4(c.x * ls, c.y * ls, c.z * ls, c.w * ls);
    /* integer accumulator (bits 32): each add is truncated */
    if (trunc) v = make_float4(truncf(v.x), truncf(v.y), truncf(v.z), truncf(v.w));
    if (akind == F3G_BK_F32) {
      float4 *a = (float4 *)acc + i;
      float4 o = *a;
      *a = make_float4(o.x + v.x, o.y + v.y, o.z + v.z, o.w + v.w);
    } else {
      double *d = (double *)acc + 4 * i;
      d[0] += v.x; d[1] += v.y; d[2] += v.z; d[3] += v.w;
    }
  }
}

__global__ void k_earlyclip(void *acc, int akind, long long n, F3GTonemap tp) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float4 a = acc_load(acc, akind, i);
    float t[4] = {a.x, a.y, a.z, a.w};
    tonemap(t, tp);
    if (tp.trunc_acc)
      for (int k = 0; k < 4; k++) t[k] = truncf(t[k]);
    acc_store(acc, akind, i, make_float4(t[0], t[1], t[2], t[3]));
  }
}

__global__ void k_filter_tonemap(const void *__restrict__ acc, int akind, int W, int de_offset, int oversample,
                                 const float *__restrict__ filter, int fw, int image_w, int image_h,
                                 unsigned char *out, int earlyclip, F3GTonemap tp) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= image_w || j >= image_h) return;
  int x = de_offset + i * oversample, y = de_offset + j * oversample;
  float t[4] = {0, 0, 0, 0};
  for (int jj = 0; jj < fw; jj++)
    for (int ii = 0; ii < fw; ii++) {
      float k = __ldg(filter + ii + jj * fw);
      float4 a = acc_load(acc, akind, (long long)(x + ii) + (long long)(y + jj) * W);
      t[0] += k * a.x; t[1] += k * a.y; t[2] += k * a.z; t[3] += k * a.w;
    }
  if (!earlyclip) tonemap(t, tp);
  pack_pixel(out + (size_t)tp.nchan * tp.bpc * ((size_t)i + (size_t)j * image_w), t, tp);
}

/* One batch without DE: read each histogram bucket once, log-scale it into a
 * shared tile, filter and tonemap the output pixels of the tile, pack. */
#define FL_TX 32
#define FL_TY 8
__global__ void __launch_bounds__(256) k_fused_log_filter(const void *__restrict__ buckets, int bkind, int W, int H,
                                                          float k1, float k2, int de_offset, int oversample,
                                                          const float *__restrict__ filter, int fw, int image_w,
                                                          int image_h, unsigned char *out, int earlyclip,
                                                          F3GTonemap tp) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int sw = FL_TX * oversample + fw - oversample, sh = FL_TY * oversample + fw - oversample;
  float4 *tile = (float4 *)smem_raw;
  float *sf = (float *)(tile + sw * sh);
  const int i0 = blockIdx.x * FL_TX, j0 = blockIdx.y * FL_TY;
  const int bx0 = de_offset + i0 * oversample, by0 = de_offset + j0 * oversample;
  const int tid = threadIdx.x + threadIdx.y * blockDim.x, nt = blockDim.x * blockDim.y;
  for (int k = tid; k < fw * fw; k += nt) sf[k] = filter[k];
  for (int k = tid; k < sw * sh; k += nt) {
    int bx = bx0 + k % sw, by = by0 + k / sw;
    float4 v = make_float4(0, 0, 0, 0);
    if (bx < W && by < H) {
      float4 c = load_bucket(buckets, bkind, (long long)bx + (long long)by * W);
      if (c.w != 0.0f) {
        float ls = log_scale(c.w, k1, k2);
        v = make_float4(c.x * ls, c.y * ls, c.z * ls, c.w * ls);
        if (tp.trunc_acc) v = make_float4(truncf(v.x), truncf(v.y), truncf(v.z), truncf(v.w));
        if (earlyclip) {
          float t[4] = {v.x, v.y, v.z, v.w};
          tonemap(t, tp);
          if (tp.trunc_acc)
            for (int k = 0; k < 4; k++) t[k] = truncf(t[k]);
          v = make_float4(t[0], t[1], t[2], t[3]);
        }
      } else if (earlyclip) {
        float t[4] = {0, 0, 0, 0};
        tonemap(t, tp);
        if (tp.trunc_acc)
          for (int k = 0; k < 4; k++) t[k] = truncf(t[k]);
        v = make_float4(t[0], t[1], t[2], t[3]);
      }
    }
    tile[k] = v;
  }
  __syncthreads();
  const int i = i0 + threadIdx.x, j = j0 + threadIdx.y;
  if (i >= image_w || j >= image_h) return;
  const int lx = threadIdx.x * oversample, ly = threadIdx.y * oversample;
  float t[4] = {0, 0, 0, 0};
  for (int jj = 0; jj < fw; jj++)
    for (int ii = 0; ii < fw; ii++) {
      float k = sf[ii + jj * fw];
      float4 a = tile[(lx + ii) + (ly + jj) * sw];
      t[0] += k * a.x; t[1] += k * a.y; t[2] += k * a.z; t[3] += k * a.w;
    }
  if (!earlyclip) tonemap(t, tp);
  pack_pixel(out + (size_t)tp.nchan * tp.bpc * ((size_t)i + (size_t)j * image_w), t, tp);
}


}  // namespace f3g

using namespace f3g;

static int grid_for(long long n, int threads) {
  long long b = (n + threads - 1) / threads;
  if (b > 152 * 32) b = 152 * 32;
  if (b < 1) b = 1;
  return (int)b;
}

extern "C" int f3g_launch_logscale(const void *buckets, int bkind, long long n, double k1, double k2, void *acc,
                                   int akind, int trunc, cudaStream_t st) {
  k_logscale<<<grid_for(n, 256), 256, 0, st>>>(buckets, bkind, n, (float)k1, (float)k2, acc, akind, trunc);
  return (int)cudaGetLastError();
}

extern "C" int f3g_launch_earlyclip(void *acc, int akind, long long n, const F3GTonemap *tp, cudaStream_t st) {
  k_earlyclip<<<grid_for(n, 256), 256, 0, st>>>(acc, akind, n, *tp);
  return (int)cudaGetLastError();
}

extern "C" int f3g_launch_filter_tonemap(const void *acc, int akind, int W, int de_offset, int oversample,
                                         const float *filter, int fw, int image_w, int image_h, unsigned char *out,
                                         int earlyclip, const F3GTonemap *tp, cudaStream_t st) {
  dim3 block(32, 8), grid((image_w + 31) / 32, (image_h + 7) / 8);
  k_filter_tonemap<<<grid, block, 0, st>>>(acc, akind, W, de_offset, oversample, filter, fw, image_w, image_h, out,
                                           earlyclip, *tp);
  return (int)cudaGetLastError();
}

/* The shared-memory limit is raised once, to the largest size a launch asks
 * for, so that launches inside stream capture make no attribute calls. */
static volatile int fused_log_attr_done = 0;

extern "C" int f3g_tail_prepare(void) {
  if (fused_log_attr_done) return 0;
  cudaError_t e = cudaFuncSetAttribute(k_fused_log_filter, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  if (e != cudaSuccess) return (int)e;
  if (f3g_strip_prepare_f32() || f3g_strip_prepare_f64() || f3g_strip_prepare_f32e() || f3g_strip_prepare_f64e() ||
      f3g_strip_prepare_acc() || f3g_strip_prepare_acce())
    return (int)cudaErrorUnknown;
  fused_log_attr_done = 1;
  return 0;
}

extern "C" int f3g_launch_fused_log_filter(const void *buckets, int bkind, int W, int H, double k1, double k2,
                                           int de_offset, int oversample, const float *filter, int fw, int image_w,
                                           int image_h, unsigned char *out, int earlyclip, const F3GTonemap *tp,
                                           cudaStream_t st) {
  int e = f3g_tail_prepare();
  if (e) return e;
  /* the separable strip kernel where an instantiation exists */
  e = (bkind == F3G_BK_F32 ? (earlyclip ? f3g_strip_launch_f32e : f3g_strip_launch_f32)
                            : (earlyclip ? f3g_strip_launch_f64e : f3g_strip_launch_f64))(
      buckets, W, H, k1, k2, de_offset, oversample, filter, fw, image_w, image_h, out, tp, st);
  if (e != -2) return e;
  int sw = FL_TX * oversample + fw - oversample, sh = FL_TY * oversample + fw - oversample;
  size_t smem = (size_t)sw * sh * sizeof(float4) + (size_t)fw * fw * sizeof(float);
  if (smem > 200 * 1024) return -1;
  dim3 block(FL_TX, FL_TY), grid((image_w + FL_TX - 1) / FL_TX, (image_h + FL_TY - 1) / FL_TY);
  k_fused_log_filter<<<grid, block, smem, st>>>(buckets, bkind, W, H, (float)k1, (float)k2, de_offset, oversample,
                                                filter, fw, image_w, image_h, out, earlyclip, *tp);
  return (int)cudaGetLastError();
}

extern "C" int f3g_launch_acc_filter(void *acc, int W, int H, int de_offset, int oversample, const float *filter,
                                     int fw, int image_w, int image_h, unsigned char *out, int earlyclip,
                                     const F3GTonemap *tp, cudaStream_t st) {
  int e = f3g_tail_prepare();
  if (e) return e;
  e = (earlyclip ? f3g_strip_launch_acce : f3g_strip_launch_acc)(acc, W, H, 0.0, 0.0, de_offset, oversample, filter,
                                                                 fw, image_w, image_h, out, tp, st);
  if (e != -2) return e;
  if (earlyclip) {
    e = f3g_launch_earlyclip(acc, F3G_BK_F32, (long long)W * H, tp, st);
    if (e) return e;
  }
  return f3g_launch_filter_tonemap(acc, F3G_BK_F32, W, de_offset, oversample, filter, fw, image_w, image_h, out,
                                   earlyclip, tp, st);
}
