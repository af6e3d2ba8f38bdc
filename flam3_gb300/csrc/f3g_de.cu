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
 *      its taps into the shared accumulator (shared-memory atomics): sources
 *      with few taps from their own thread, then, in a second pass in which
 *      each warp re-classifies 32 sources at a time, each source with many
 *      taps over the warp's 32 lanes;
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
  int mfc, mfi, R;
  /* per DE kernel k: (c_k, m_k, r2max_k, reach_k) with
   * coef(dx, dy) = c_k * 2^(m_k * (dx^2 + dy^2)) for dx^2 + dy^2 <= r2max_k */
  const float4 *kinfo;
  /* tile geometry */
  int A;            /* accumulator region edge (buckets) */
  int TO;           /* output pixels per tile edge (fused) */
  int de_offset, fw, image_w, image_h, earlyclip;
  const float *filter;
  unsigned char *out;
  void *acc;        /* accumulate mode */
  int akind;
  F3GTonemap tp;
};

/* sources with more taps than this inside the region go to the shared list
 * (one warp per source); fewer are scattered by the classifying thread */
#ifndef DE_SMALL_TAPS
#define DE_SMALL_TAPS 4
#endif

__device__ __forceinline__ float de_coef(float4 ki, int r2) {
  return (float)r2 <= ki.z ? ki.x * exp2f(ki.y * (float)r2) : 0.0f;
}

/* Classifies source k of the tile's S x S source window (rect.c:79-117):
 * returns false when it adds nothing to the region, else its kernel, its
 * clipped tap rectangle inside the region and its bucket coordinates. */
struct DESource {
  int sx, sy, fi, x_lo, x_hi, y_lo, y_hi;
};

__device__ __forceinline__ bool de_classify(const DEParams &P, const float *cnt, const float4 *kin, int k, int S,
                                            int Cc, int ax0, int ay0, int A, int R, int ss, int istart, int iend,
                                            int jstart, int jend, DESource &o) {
  const int lx = k % S, ly = k / S;
  const int sx = ax0 - R + lx, sy = ay0 - R + ly;
  if (sx < istart || sx >= iend || sy < jstart || sy >= jend) return false;
  if (cnt[(lx + ss) + (ly + ss) * Cc] == 0.0f) return false;
  float f = 0.0f;
  for (int jj = -ss; jj <= ss; jj++)
    for (int ii = -ss; ii <= ss; ii++) f += cnt[(lx + ss + ii) + (ly + ss + jj) * Cc];
  if (P.scf) f *= P.scfact;
  int fi;
  if (f > (float)P.mfc) fi = P.mfi;
  else if (f <= 100.0f) fi = (int)ceilf(f) - 1;
  else fi = 100 + (int)floorf(powf(f - 100.0f, P.curve));
  fi = min(max(fi, 0), P.mfi);
  const int reach = (int)kin[fi].w;
  o.sx = sx;
  o.sy = sy;
  o.fi = fi;
  o.x_lo = max(sx - reach, ax0);
  o.x_hi = min(sx + reach, ax0 + A - 1);
  o.y_lo = max(sy - reach, ay0);
  o.y_hi = min(sy + reach, ay0 + A - 1);
  return o.x_lo <= o.x_hi && o.y_lo <= o.y_hi;
}

template <bool FUSED>
__global__ void __launch_bounds__(256) k_de_tile(DEParams P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int A = P.A, R = P.R, ss = P.ss;
  const int S = A + 2 * R, Cc = S + 2 * ss, AA = A * A;
  const int nk = P.mfi + 1;
  float4 *kin = (float4 *)smem_raw;               /* nk kernel constants */
  float *acc = (float *)(kin + nk);               /* 4 planes of A*A */
  float *cnt = acc + 4 * AA;                      /* Cc*Cc counts / 255 */
  float *filt = cnt + Cc * Cc;                    /* fw*fw (fused) */
  const int tid = threadIdx.x, nt = blockDim.x;
  int ax0, ay0;
  if (FUSED) {
    ax0 = P.de_offset + blockIdx.x * P.TO * P.os;
    ay0 = P.de_offset + blockIdx.y * P.TO * P.os;
  } else {
    ax0 = blockIdx.x * A;
    ay0 = blockIdx.y * A;
  }
  const int cx0 = ax0 - R - ss, cy0 = ay0 - R - ss;
  for (int k = tid; k < nk; k += nt) kin[k] = P.kinfo[k];
  for (int k = tid; k < 4 * AA; k += nt) acc[k] = 0.0f;
  if (FUSED)
    for (int k = tid; k < P.fw * P.fw; k += nt) filt[k] = P.filter[k];
  for (int k = tid; k < Cc * Cc; k += nt) {
    const int bx = cx0 + k % Cc, by = cy0 + k / Cc;
    float c = 0.0f;
    if (bx >= 0 && bx < P.W && by >= 0 && by < P.H)
      c = load_count(P.buckets, P.bkind, P.count, (long long)bx + (long long)by * P.W) / 255.0f;
    cnt[k] = c;
  }
  __syncthreads();
  /* DE loop bounds of the reference (rect.c:79-80, 979) */
  const int istart = P.os - 1, iend = P.W - (P.os - 1);
  const int jstart = P.os - 1, jend = min(P.H, (P.os - 1) + (P.H - 2 * (P.os - 1) + 1));
  /* 1. sources with few taps in the region scatter from their thread
   *    (shared-memory atomics) */
  for (int k = tid; k < S * S; k += nt) {
    DESource o;
    if (!de_classify(P, cnt, kin, k, S, Cc, ax0, ay0, A, R, ss, istart, iend, jstart, jend, o)) continue;
    if ((o.x_hi - o.x_lo + 1) * (o.y_hi - o.y_lo + 1) > DE_SMALL_TAPS) continue;
    float4 v = load_bucket(P.buckets, P.bkind, (long long)o.sx + (long long)o.sy * P.W);
    if (v.w == 0.0f) continue;
    const float ls = P.k1 * log1pf(v.w * P.k2) / v.w;
    v = make_float4(v.x * ls, v.y * ls, v.z * ls, v.w * ls);
    const float4 ki = kin[o.fi];
    for (int y = o.y_lo; y <= o.y_hi; y++) {
      const int dy = y - o.sy;
      for (int x = o.x_lo; x <= o.x_hi; x++) {
        const int dx = x - o.sx;
        const float w = de_coef(ki, dx * dx + dy * dy);
        if (w == 0.0f) continue;
        const int off = (x - ax0) + (y - ay0) * A;
        atomicAdd(acc + off, w * v.x);
        atomicAdd(acc + AA + off, w * v.y);
        atomicAdd(acc + 2 * AA + off, w * v.z);
        atomicAdd(acc + 3 * AA + off, w * v.w);
      }
    }
  }
  /* 2. sources with many taps: each warp classifies 32 sources at a time,
   *    then spreads each wide one over its lanes (row-major taps; each lane
   *    advances by 32 taps without dividing) -- no list in shared memory */
  const int warp = tid >> 5, lane = tid & 31, nwarps = nt >> 5;
  for (int base = warp * 32; base < S * S; base += nwarps * 32) {
    DESource o;
    bool wide = false;
    if (base + lane < S * S && de_classify(P, cnt, kin, base + lane, S, Cc, ax0, ay0, A, R, ss, istart, iend, jstart,
                                           jend, o))
      wide = (o.x_hi - o.x_lo + 1) * (o.y_hi - o.y_lo + 1) > DE_SMALL_TAPS;
    unsigned mask = __ballot_sync(0xffffffffu, wide);
    while (mask) {
      const int src = __ffs(mask) - 1;
      mask &= mask - 1;
      const int sx = __shfl_sync(0xffffffffu, o.sx, src), sy = __shfl_sync(0xffffffffu, o.sy, src);
      const int fi = __shfl_sync(0xffffffffu, o.fi, src);
      const int x_lo = __shfl_sync(0xffffffffu, o.x_lo, src), x_hi = __shfl_sync(0xffffffffu, o.x_hi, src);
      const int y_lo = __shfl_sync(0xffffffffu, o.y_lo, src), y_hi = __shfl_sync(0xffffffffu, o.y_hi, src);
      float4 v = load_bucket(P.buckets, P.bkind, (long long)sx + (long long)sy * P.W);
      if (v.w == 0.0f) continue;
      const float ls = P.k1 * log1pf(v.w * P.k2) / v.w;
      v = make_float4(v.x * ls, v.y * ls, v.z * ls, v.w * ls);
      const float4 ki = kin[fi];
      const int wdt = x_hi - x_lo + 1;
      const int step_y = 32 / wdt, step_x = 32 % wdt;
      int cx = lane % wdt, y = y_lo + lane / wdt;
      const int dx0 = x_lo - sx;
      while (y <= y_hi) {
        const int dx = dx0 + cx, dy = y - sy;
        const float w = de_coef(ki, dx * dx + dy * dy);
        if (w != 0.0f) {
          const int off = (x_lo - ax0 + cx) + (y - ay0) * A;
          atomicAdd(acc + off, w * v.x);
          atomicAdd(acc + AA + off, w * v.y);
          atomicAdd(acc + 2 * AA + off, w * v.z);
          atomicAdd(acc + 3 * AA + off, w * v.w);
        }
        cx += step_x;
        y += step_y;
        if (cx >= wdt) {
          cx -= wdt;
          y++;
        }
      }
    }
  }
  __syncthreads();
  if (!FUSED) {
    /* add the core tile to the global accumulator (tiles do not overlap) */
    for (int k = tid; k < AA; k += nt) {
      const int x = ax0 + k % A, y = ay0 + k / A;
      if (x >= P.W || y >= P.H) continue;
      const long long g = (long long)x + (long long)y * P.W;
      float4 o = acc_load(P.acc, P.akind, g);
      acc_store(P.acc, P.akind, g,
                make_float4(o.x + acc[k], o.y + acc[AA + k], o.z + acc[2 * AA + k], o.w + acc[3 * AA + k]));
    }
    return;
  }
  if (P.earlyclip) {
    for (int k = tid; k < AA; k += nt) {
      float t[4] = {acc[k], acc[AA + k], acc[2 * AA + k], acc[3 * AA + k]};
      tonemap(t, P.tp);
      acc[k] = t[0];
      acc[AA + k] = t[1];
      acc[2 * AA + k] = t[2];
      acc[3 * AA + k] = t[3];
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
        t[1] += w * acc[AA + o];
        t[2] += w * acc[2 * AA + o];
        t[3] += w * acc[3 * AA + o];
      }
    if (!P.earlyclip) tonemap(t, P.tp);
    pack_pixel(P.out + (size_t)P.tp.nchan * P.tp.bpc * ((size_t)i + (size_t)j * P.image_w), t, P.tp);
  }
}

static size_t de_smem(int A, int R, int ss, int fw, int nk) {
  const int S = A + 2 * R, Cc = S + 2 * ss;
  (void)S;
  return (size_t)nk * 16 + (size_t)4 * A * A * 4 + (size_t)Cc * Cc * 4 + (size_t)fw * fw * 4;
}

static DEParams base_params(const void *buckets, int bkind, const void *count, int W, int H, int oversample,
                            double k1, double k2, double curve, int mfc, int mfi, const float4 *kinfo, int R) {
  DEParams P;
  P.buckets = buckets; P.count = count; P.bkind = bkind; P.W = W; P.H = H; P.os = oversample;
  P.ss = oversample / 2; P.scf = !(oversample & 1);
  P.scfact = (float)((oversample / (oversample + 1.0)) * (oversample / (oversample + 1.0)));
  P.k1 = (float)k1; P.k2 = (float)k2; P.curve = (float)curve;
  P.mfc = mfc; P.mfi = mfi; P.R = R; P.kinfo = kinfo;
  P.de_offset = 0; P.fw = 0; P.image_w = P.image_h = 0; P.earlyclip = 0; P.filter = nullptr; P.out = nullptr;
  P.acc = nullptr; P.akind = bkind;
  return P;
}

}  // namespace f3g

using namespace f3g;

/* Per-kernel constants from the reference's tables (filters.c:272-407):
 * coefs[k][0] is the kernel's value at distance 0 (its normalisation),
 * widths[k] its radius h_k; the coefficient at squared distance r2 is
 * coefs[k][0] * exp(-4.5 r2 / h_k^2) inside the disc, and the disc is the set
 * of (dx, dy) whose table entry is non-zero. */
extern "C" void f3g_de_kernel_info(int mfi, int ks, const double *widths, const double *coefs, float *out) {
  for (int k = 0; k <= mfi; k++) {
    const double h = widths[k];
    const double *c = coefs + (size_t)k * ks;
    int r2max = -1, idx = 0, half = 0;
    while ((half + 1) * (half + 2) / 2 < ks) half++;
    for (int a = 0; a <= half; a++)
      for (int b = 0; b <= a; b++, idx++)
        if (c[idx] != 0.0 && a * a + b * b > r2max) r2max = a * a + b * b;
    out[4 * k + 0] = (float)c[0];
    out[4 * k + 1] = (float)(-4.5 / (h * h) / log(2.0));
    out[4 * k + 2] = (float)r2max;
    out[4 * k + 3] = (float)(ceil(h) - 1);
  }
}

/* The tail kernels may be launched inside stream capture, where only
 * stream-ordered calls belong: their shared-memory limit is raised once, to
 * the largest size any launch asks for, before the first launch. */
#define DE_SMEM_MAX (220 * 1024)
template <bool FUSED> static cudaError_t de_attr_once() {
  static volatile int done = 0;
  if (done) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(k_de_tile<FUSED>, cudaFuncAttributeMaxDynamicSharedMemorySize, DE_SMEM_MAX);
  if (e == cudaSuccess) done = 1;
  return e;
}

extern "C" int f3g_de_prepare(void) {
  cudaError_t e = de_attr_once<true>();
  if (e == cudaSuccess) e = de_attr_once<false>();
  if (e == cudaSuccess) e = (cudaError_t)f3g_de_bands_prepare();
  return (int)e;
}

extern "C" size_t f3g_de_fused_smem_tile(int oversample, int fw, int R, int nk, int tile) {
  const int A = (tile - 1) * oversample + fw;
  return de_smem(A, R, oversample / 2, fw, nk);
}

extern "C" size_t f3g_de_fused_smem(int oversample, int fw, int R, int nk) {
  return f3g_de_fused_smem_tile(oversample, fw, R, nk, 16);
}

extern "C" int f3g_launch_de_fused_tile(const void *buckets, int bkind, const void *count, int W, int H,
                                        int oversample, double k1, double k2, double curve, int mfc, int mfi,
                                        const float *kinfo, int R, int de_offset, const float *filter, int fw,
                                        int image_w, int image_h, unsigned char *out, int earlyclip,
                                        const F3GTonemap *tp, int tile, cudaStream_t st) {
  DEParams P = base_params(buckets, bkind, count, W, H, oversample, k1, k2, curve, mfc, mfi,
                           (const float4 *)kinfo, R);
  P.TO = tile;
  P.A = (P.TO - 1) * oversample + fw;
  P.de_offset = de_offset; P.fw = fw; P.filter = filter; P.image_w = image_w; P.image_h = image_h;
  P.out = out; P.earlyclip = earlyclip; P.tp = *tp;
  size_t smem = de_smem(P.A, R, P.ss, fw, mfi + 1);
  if (tile < 4 || tile > 64 || smem > DE_SMEM_MAX) return -1;
  cudaError_t e = de_attr_once<true>();
  if (e != cudaSuccess) return (int)e;
  dim3 grid((image_w + P.TO - 1) / P.TO, (image_h + P.TO - 1) / P.TO);
  k_de_tile<true><<<grid, 256, smem, st>>>(P);
  return (int)cudaGetLastError();
}

extern "C" int f3g_launch_de_fused(const void *buckets, int bkind, const void *count, int W, int H, int oversample,
                                   double k1, double k2, double curve, int mfc, int mfi, const float *kinfo, int R,
                                   int de_offset, const float *filter, int fw, int image_w, int image_h,
                                   unsigned char *out, int earlyclip, const F3GTonemap *tp, cudaStream_t st) {
  return f3g_launch_de_fused_tile(buckets, bkind, count, W, H, oversample, k1, k2, curve, mfc, mfi, kinfo, R,
                                  de_offset, filter, fw, image_w, image_h, out, earlyclip, tp, 16, st);
}

extern "C" int f3g_launch_de(const void *buckets, int bkind, const void *count, int W, int H, int oversample,
                             double k1, double k2, double curve, int mfc, int mfi, const float *kinfo, int R,
                             void *acc, int akind, cudaStream_t st) {
  DEParams P = base_params(buckets, bkind, count, W, H, oversample, k1, k2, curve, mfc, mfi,
                           (const float4 *)kinfo, R);
  P.A = 32;
  P.TO = 32;
  P.acc = acc;
  P.akind = akind;
  size_t smem = de_smem(P.A, R, P.ss, 0, mfi + 1);
  if (smem > DE_SMEM_MAX) return -1;
  cudaError_t e = de_attr_once<false>();
  if (e != cudaSuccess) return (int)e;
  dim3 grid((W + P.A - 1) / P.A, (H + P.A - 1) / P.A);
  k_de_tile<false><<<grid, 256, smem, st>>>(P);
  return (int)cudaGetLastError();
}

extern "C" int f3g_de_max_reach(void) { return 40; }
