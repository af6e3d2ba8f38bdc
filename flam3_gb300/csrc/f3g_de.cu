/*
 * f3g_de.cu -- density estimation (rect.c:57-251) fused with the spatial
 * filter, tonemap and packing (rect.c:1067-1247).
 *
 * The reference scatters every non-empty bucket with a Gaussian kernel whose
 * width falls with the density around that bucket.  On the GPU each block
 * owns a tile of output pixels and computes everything the tile needs:
 *
 *   1. the accumulator region A x A under the tile's filter footprint;
 *   2. the sources that can reach it: region A + 2R (R = reach of the widest
 *      kernel), whose counts (+ss border, for the density sums) are staged in
 *      shared memory;
 *   3. every non-empty source whose kernel square meets the region scatters
 *      its taps into the shared accumulator (shared-memory atomics); sources
 *      with many taps are queued and spread over the 32 lanes of a warp;
 *   4. the filter + tonemap + pack of the tile's pixels read the shared
 *      accumulator; nothing but the image is written to global memory.
 *
 * A second instantiation adds the DE result of a core tile to a global
 * accumulator instead (several batches, or when the accumulator is asked for).
 * Work per tile is proportional to the taps that land in it, so sparse
 * histograms (most buckets empty) cost little beyond reading the histogram.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "f3g_common.h"
#include "f3g_launch.h"
#include "f3g_tail.cuh"

namespace f3g {

struct DEParams {
  const void *buckets;
  const void *count;
  int bkind, W, H, os, ss, scf;
  float scfact, k1, k2, curve;
  int mfc, mfi, ks, R;
  const float *widths, *coefs;
  /* tile geometry */
  int A;            /* accumulator region edge (buckets) */
  int TO;           /* output pixels per tile edge (fused) or core buckets (accumulate) */
  int de_offset, fw, image_w, image_h, earlyclip;
  const float *filter;
  unsigned char *out;
  void *acc;        /* accumulate mode */
  int akind;
  F3GTonemap tp;
};

/* sources with more taps than this inside the region go to the warp queue */
#define DE_WARP_TAPS 32

template <bool FUSED>
__global__ void __launch_bounds__(256) k_de_tile(DEParams P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int A = P.A, R = P.R, ss = P.ss;
  const int S = A + 2 * R, Cc = S + 2 * ss;
  float *acc = (float *)smem_raw;                 /* 4 planes of A*A */
  float *cnt = acc + 4 * A * A;                   /* Cc*Cc counts / 255 */
  float *filt = cnt + Cc * Cc;                    /* fw*fw (fused) */
  /* queue of wide sources: local index in the S x S region, kernel index */
  uint32_t *queue = (uint32_t *)(filt + P.fw * P.fw);
  __shared__ int qn;
  const int tid = threadIdx.x, nt = blockDim.x;
  /* region origin in bucket coordinates */
  int ax0, ay0;
  if (FUSED) {
    ax0 = P.de_offset + blockIdx.x * P.TO * P.os;
    ay0 = P.de_offset + blockIdx.y * P.TO * P.os;
  } else {
    ax0 = blockIdx.x * A;
    ay0 = blockIdx.y * A;
  }
  const int cx0 = ax0 - R - ss, cy0 = ay0 - R - ss;
  if (tid == 0) qn = 0;
  for (int k = tid; k < 4 * A * A; k += nt) acc[k] = 0.0f;
  if (FUSED)
    for (int k = tid; k < P.fw * P.fw; k += nt) filt[k] = P.filter[k];
  /* counts of the source region (+ss border) */
  for (int k = tid; k < Cc * Cc; k += nt) {
    int bx = cx0 + k % Cc, by = cy0 + k / Cc;
    float c = 0.0f;
    if (bx >= 0 && bx < P.W && by >= 0 && by < P.H)
      c = load_count(P.buckets, P.bkind, P.count, (long long)bx + (long long)by * P.W) / 255.0f;
    cnt[k] = c;
  }
  __syncthreads();
  /* DE loop bounds of the reference (rect.c:79-80) */
  const int istart = P.os - 1, iend = P.W - (P.os - 1);
  const int jstart = P.os - 1, jend = min(P.H, (P.os - 1) + (P.H - 2 * (P.os - 1) + 1));
  for (int k = tid; k < S * S; k += nt) {
    const int lx = k % S, ly = k / S;
    const int sx = ax0 - R + lx, sy = ay0 - R + ly;
    if (sx < istart || sx >= iend || sy < jstart || sy >= jend) continue;
    const float c_self = cnt[(lx + ss) + (ly + ss) * Cc];
    if (c_self == 0.0f) continue;
    float4 v = load_bucket(P.buckets, P.bkind, (long long)sx + (long long)sy * P.W);
    if (v.w == 0.0f) continue;
    float f = 0.0f;
    for (int jj = -ss; jj <= ss; jj++)
      for (int ii = -ss; ii <= ss; ii++) f += cnt[(lx + ss + ii) + (ly + ss + jj) * Cc];
    if (P.scf) f *= P.scfact;
    int fi;
    if (f > (float)P.mfc) fi = P.mfi;
    else if (f <= 100.0f) fi = (int)ceilf(f) - 1;
    else fi = 100 + (int)floorf(powf(f - 100.0f, P.curve));
    fi = min(max(fi, 0), P.mfi);
    const int reach = (int)ceilf(__ldg(P.widths + fi)) - 1;
    /* part of the source's square inside the region */
    const int x_lo = max(sx - reach, ax0), x_hi = min(sx + reach, ax0 + A - 1);
    const int y_lo = max(sy - reach, ay0), y_hi = min(sy + reach, ay0 + A - 1);
    if (x_lo > x_hi || y_lo > y_hi) continue;
    const int ntaps = (x_hi - x_lo + 1) * (y_hi - y_lo + 1);
    if (ntaps > DE_WARP_TAPS) {
      /* every source fits: the queue has room for the whole S x S region */
      queue[atomicAdd(&qn, 1)] = ((uint32_t)k << 16) | (uint32_t)fi;
      continue;
    }
    const float ls = P.k1 * log1pf(v.w * P.k2) / v.w;
    v = make_float4(v.x * ls, v.y * ls, v.z * ls, v.w * ls);
    const float *cf = P.coefs + (long long)fi * P.ks;
    for (int y = y_lo; y <= y_hi; y++) {
      const int ady = abs(y - sy);
      for (int x = x_lo; x <= x_hi; x++) {
        const int adx = abs(x - sx);
        const int hi = max(adx, ady), lo = min(adx, ady);
        const float w = __ldg(cf + hi * (hi + 1) / 2 + lo);
        if (w == 0.0f) continue;
        const int o = (x - ax0) + (y - ay0) * A;
        atomicAdd(acc + o, w * v.x);
        atomicAdd(acc + A * A + o, w * v.y);
        atomicAdd(acc + 2 * A * A + o, w * v.z);
        atomicAdd(acc + 3 * A * A + o, w * v.w);
      }
    }
  }
  __syncthreads();
  /* queued sources with many taps: one warp each, lanes over the taps */
  const int nq = qn;
  const int warp = tid >> 5, lane = tid & 31, nwarps = nt >> 5;
  for (int q = warp; q < nq; q += nwarps) {
    const uint32_t e = queue[q];
    const int kk = (int)(e >> 16), fi = (int)(e & 0xffffu);
    const int sx = ax0 - R + kk % S, sy = ay0 - R + kk / S;
    const int reach = (int)ceilf(__ldg(P.widths + fi)) - 1;
    float4 v = load_bucket(P.buckets, P.bkind, (long long)sx + (long long)sy * P.W);
    const float ls = P.k1 * log1pf(v.w * P.k2) / v.w;
    v = make_float4(v.x * ls, v.y * ls, v.z * ls, v.w * ls);
    const int x_lo = max(sx - reach, ax0), x_hi = min(sx + reach, ax0 + A - 1);
    const int y_lo = max(sy - reach, ay0), y_hi = min(sy + reach, ay0 + A - 1);
    const int wdt = x_hi - x_lo + 1, n = wdt * (y_hi - y_lo + 1);
    const float *cf = P.coefs + (long long)fi * P.ks;
    for (int t = lane; t < n; t += 32) {
      const int x = x_lo + t % wdt, y = y_lo + t / wdt;
      const int adx = abs(x - sx), ady = abs(y - sy);
      const int hi = max(adx, ady), lo = min(adx, ady);
      const float w = __ldg(cf + hi * (hi + 1) / 2 + lo);
      if (w == 0.0f) continue;
      const int o = (x - ax0) + (y - ay0) * A;
      atomicAdd(acc + o, w * v.x);
      atomicAdd(acc + A * A + o, w * v.y);
      atomicAdd(acc + 2 * A * A + o, w * v.z);
      atomicAdd(acc + 3 * A * A + o, w * v.w);
    }
  }
  __syncthreads();
  if (!FUSED) {
    /* add the core tile to the global accumulator (tiles do not overlap) */
    for (int k = tid; k < A * A; k += nt) {
      const int x = ax0 + k % A, y = ay0 + k / A;
      if (x >= P.W || y >= P.H) continue;
      const long long g = (long long)x + (long long)y * P.W;
      float4 o = acc_load(P.acc, P.akind, g);
      acc_store(P.acc, P.akind, g,
                make_float4(o.x + acc[k], o.y + acc[A * A + k], o.z + acc[2 * A * A + k], o.w + acc[3 * A * A + k]));
    }
    return;
  }
  if (P.earlyclip) {
    for (int k = tid; k < A * A; k += nt) {
      float t[4] = {acc[k], acc[A * A + k], acc[2 * A * A + k], acc[3 * A * A + k]};
      tonemap(t, P.tp);
      acc[k] = t[0];
      acc[A * A + k] = t[1];
      acc[2 * A * A + k] = t[2];
      acc[3 * A * A + k] = t[3];
    }
    __syncthreads();
  }
  for (int k = tid; k < P.TO * P.TO; k += nt) {
    const int oi = k % P.TO, oj = k / P.TO;
    const int i = blockIdx.x * P.TO + oi, j = blockIdx.y * P.TO + oj;
    if (i >= P.image_w || j >= P.image_h) continue;
    const int lx = oi * P.os, ly = oj * P.os;
    float t[4] = {0, 0, 0, 0};
    for (int jj = 0; jj < P.fw; jj++)
      for (int ii = 0; ii < P.fw; ii++) {
        const float w = filt[ii + jj * P.fw];
        const int o = (lx + ii) + (ly + jj) * A;
        t[0] += w * acc[o];
        t[1] += w * acc[A * A + o];
        t[2] += w * acc[2 * A * A + o];
        t[3] += w * acc[3 * A * A + o];
      }
    if (!P.earlyclip) tonemap(t, P.tp);
    pack_pixel(P.out + (size_t)P.tp.nchan * P.tp.bpc * ((size_t)i + (size_t)j * P.image_w), t, P.tp);
  }
}

static size_t de_smem(int A, int R, int ss, int fw) {
  const int S = A + 2 * R, Cc = S + 2 * ss;
  return (size_t)4 * A * A * 4 + (size_t)Cc * Cc * 4 + (size_t)fw * fw * 4 + (size_t)S * S * 4;
}

static DEParams base_params(const void *buckets, int bkind, const void *count, int W, int H, int oversample,
                            double k1, double k2, double curve, int mfc, int mfi, int ks, const float *widths,
                            const float *coefs, int R) {
  DEParams P;
  P.buckets = buckets; P.count = count; P.bkind = bkind; P.W = W; P.H = H; P.os = oversample;
  P.ss = oversample / 2; P.scf = !(oversample & 1);
  P.scfact = (float)((oversample / (oversample + 1.0)) * (oversample / (oversample + 1.0)));
  P.k1 = (float)k1; P.k2 = (float)k2; P.curve = (float)curve;
  P.mfc = mfc; P.mfi = mfi; P.ks = ks; P.R = R; P.widths = widths; P.coefs = coefs;
  P.de_offset = 0; P.fw = 0; P.image_w = P.image_h = 0; P.earlyclip = 0; P.filter = nullptr; P.out = nullptr;
  P.acc = nullptr; P.akind = bkind;
  return P;
}

}  // namespace f3g

using namespace f3g;

extern "C" size_t f3g_de_fused_smem(int oversample, int fw, int R) {
  const int TO = 16, A = (TO - 1) * oversample + fw;
  return de_smem(A, R, oversample / 2, fw);
}

extern "C" int f3g_launch_de_fused(const void *buckets, int bkind, const void *count, int W, int H, int oversample,
                                   double k1, double k2, double curve, int mfc, int mfi, int ks, const float *widths,
                                   const float *coefs, int R, int de_offset, const float *filter, int fw,
                                   int image_w, int image_h, unsigned char *out, int earlyclip, const F3GTonemap *tp,
                                   cudaStream_t st) {
  DEParams P = base_params(buckets, bkind, count, W, H, oversample, k1, k2, curve, mfc, mfi, ks, widths, coefs, R);
  P.TO = 16;
  P.A = (P.TO - 1) * oversample + fw;
  P.de_offset = de_offset; P.fw = fw; P.filter = filter; P.image_w = image_w; P.image_h = image_h;
  P.out = out; P.earlyclip = earlyclip; P.tp = *tp;
  size_t smem = de_smem(P.A, R, P.ss, fw);
  if (smem > 220 * 1024) return -1;
  cudaError_t e = cudaFuncSetAttribute(k_de_tile<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  dim3 grid((image_w + P.TO - 1) / P.TO, (image_h + P.TO - 1) / P.TO);
  k_de_tile<true><<<grid, 256, smem, st>>>(P);
  return (int)cudaGetLastError();
}

extern "C" int f3g_launch_de(const void *buckets, int bkind, const void *count, int W, int H, int oversample,
                             double k1, double k2, double curve, int mfc, int mfi, int ks, const float *widths,
                             const float *coefs, int R, void *acc, int akind, cudaStream_t st) {
  DEParams P = base_params(buckets, bkind, count, W, H, oversample, k1, k2, curve, mfc, mfi, ks, widths, coefs, R);
  P.A = 32;
  P.TO = 32;
  P.acc = acc;
  P.akind = akind;
  size_t smem = de_smem(P.A, R, P.ss, 0);
  if (smem > 220 * 1024) return -1;
  cudaError_t e = cudaFuncSetAttribute(k_de_tile<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  dim3 grid((W + P.A - 1) / P.A, (H + P.A - 1) / P.A);
  k_de_tile<false><<<grid, 256, smem, st>>>(P);
  return (int)cudaGetLastError();
}

extern "C" int f3g_de_max_reach(void) { return 40; }
