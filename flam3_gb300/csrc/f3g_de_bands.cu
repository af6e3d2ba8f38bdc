/*
 * f3g_de_bands.cu -- density estimation (rect.c:57-251) as an
 * output-stationary pass with register accumulators.
 *
 * The reference scatters every non-empty bucket over a disc-shaped Gaussian
 * whose width falls with the density around the bucket.  Here:
 *
 *   k_de_classify  one thread per bucket: the density around it (the counts
 *                  of its (2ss+1)^2 neighbourhood, rect.c:79-117) and its
 *                  kernel index, one byte per bucket (0xFF: not a source --
 *                  empty, or outside the reference's DE loop bounds).
 *   k_de_bands     a block owns a 32 x 64 tile of the accumulator; lane l of
 *                  warp w keeps the four channels of buckets
 *                  (x0 + l, y0 + 8w + r), r < 8, in registers.  The block
 *                  walks the tile's source window (the tile grown by the
 *                  widest kernel's reach R on every side) in row chunks: it
 *                  compacts a chunk's sources into a shared list in row-major
 *                  order, each with its log-scaled channels, and every warp
 *                  then adds each listed source that reaches its 8-row band
 *                  with coef(dx, dy) = c_k 2^(m_k dx^2) 2^(m_k dy^2) inside
 *                  the kernel's disc.  Every bucket has one owner, so there
 *                  are no atomics; the list order fixes the order of the
 *                  additions, so a render repeats bit for bit.  The tile is
 *                  then stored to (or added into) the accumulator, which the
 *                  filter + tonemap pass reads.
 *
 * Work is proportional to (sources x the 8-row bands and 32-column tiles
 * their kernels reach): the taps themselves are fused multiply-adds into
 * registers, and the histogram is read once by the classifier plus once per
 * source by the tiles whose window holds it (L2).
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "f3g_common.h"
#include "f3g_launch.h"
#include "f3g_tail.cuh"

#define DEB_TW 32   /* tile columns: one per lane */
#define DEB_ROWS 8  /* rows per warp */
#define DEB_WARPS 8
#define DEB_TH (DEB_ROWS * DEB_WARPS)
#define DEB_THREADS (32 * DEB_WARPS)
#define DEB_LCAP 2048 /* sources of one chunk (a chunk never holds more positions) */
#define DEB_Q (DEB_LCAP / DEB_THREADS)
#define DEB_MAX_REACH 40
#define DEB_WROWS (DEB_TH + 2 * DEB_MAX_REACH) /* rows of the widest source window */
#define DEB_NOSRC 0xFFu

namespace f3g {

struct DEClassify {
  const void *buckets;
  const void *count;
  int bkind, W, H, ss, scf, mfc, mfi;
  float scfact, curve;
  int istart, iend, jstart, jend;
  uint8_t *fi;
  unsigned long long *stats; /* optional work counters: [0] sources */
};

/* rect.c:79-117: kernel index of the bucket at (x, y), or 0xFF */
__global__ void __launch_bounds__(256) k_de_classify(DEClassify P) {
  const long long n = (long long)P.W * P.H;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % P.W), y = (int)(i / P.W);
    unsigned out = DEB_NOSRC;
    if (x >= P.istart && x < P.iend && y >= P.jstart && y < P.jend &&
        load_count(P.buckets, P.bkind, P.count, i) / 255.0f != 0.0f) {
      float f = 0.0f;
      for (int jj = -P.ss; jj <= P.ss; jj++)
        for (int ii = -P.ss; ii <= P.ss; ii++) {
          const int bx = x + ii, by = y + jj;
          if (bx >= 0 && bx < P.W && by >= 0 && by < P.H)
            f += load_count(P.buckets, P.bkind, P.count, (long long)bx + (long long)by * P.W) / 255.0f;
        }
      if (P.scf) f *= P.scfact;
      int k;
      if (f > (float)P.mfc) k = P.mfi;
      else if (f <= 100.0f) k = (int)ceilf(f) - 1;
      else k = 100 + (int)floorf(powf(f - 100.0f, P.curve));
      out = (unsigned)min(max(k, 0), P.mfi);
    }
    P.fi[i] = (uint8_t)out;
    if (P.stats) {
      const unsigned b = __ballot_sync(__activemask(), out != DEB_NOSRC);
      if ((threadIdx.x & 31) == __ffs(__activemask()) - 1 && b) atomicAdd(P.stats, (unsigned long long)__popc(b));
    }
  }
}

struct DEBands {
  const void *buckets;
  int bkind, W, H, R, nk;
  float k1, k2;
  const uint8_t *fi;
  const float4 *kinfo; /* (c_k, m_k, r2max_k, reach_k) */
  void *acc;
  int akind, add;
  unsigned long long *stats; /* STATS: [1] source-band pairs, [2] taps */
};

/* STATS counts the work (source-band pairs that pass the reach test, and
 * taps inside the kernels' discs) for the roofline; the render uses the
 * plain instantiation. */
template <bool STATS>
__global__ void __launch_bounds__(DEB_THREADS, 4) k_de_bands(DEBands P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float4 *sv = (float4 *)smem_raw;                  /* DEB_LCAP log-scaled channels */
  uint32_t *sxyk = (uint32_t *)(sv + DEB_LCAP);     /* column | row << 8 | kernel << 16 | reach << 24 */
  float4 *kin = (float4 *)(sxyk + DEB_LCAP);        /* nk kernels */
  uint8_t *sfi = (uint8_t *)(kin + P.nk);           /* the chunk's kernel bytes */
  int *rowstart = (int *)(sfi + DEB_LCAP);          /* list index of each window row, + total */
  int *rowreach = rowstart + DEB_WROWS + 1;         /* widest reach among each row's sources */
  int *wsum = rowreach + DEB_WROWS + 1;             /* per-warp counts of the scan */
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int R = P.R, X0 = blockIdx.x * DEB_TW, Y0 = blockIdx.y * DEB_TH;
  const int WX0 = X0 - R, WY0 = Y0 - R, WW = DEB_TW + 2 * R, WH = DEB_TH + 2 * R;
  /* chunks are column slices of the window over all its rows, so every
   * chunk feeds every band (row slices would leave the warps of the far
   * bands idle at each chunk's barrier) */
  const int CW = DEB_LCAP / WH;
  const int B0 = Y0 + DEB_ROWS * warp; /* this warp's first row */
  for (int k = tid; k < P.nk; k += DEB_THREADS) kin[k] = P.kinfo[k];
  float acc[DEB_ROWS][4];
#pragma unroll
  for (int r = 0; r < DEB_ROWS; r++) acc[r][0] = acc[r][1] = acc[r][2] = acc[r][3] = 0.0f;
  unsigned long long n_pairs = 0, n_taps = 0;
  /* window rows whose sources can reach this warp's band */
  const int rlo = max(0, B0 - R - WY0), rhi = min(WH - 1, B0 + DEB_ROWS - 1 + R - WY0);

  for (int cc0 = 0; cc0 < WW; cc0 += CW) {
    const int cols = min(CW, WW - cc0), npos = WH * cols;
    /* 1. the chunk's kernel bytes, row-major */
    for (int k = tid; k < WH; k += DEB_THREADS) rowreach[k] = -1;
    for (int k = tid; k < npos; k += DEB_THREADS) {
      const int bx = WX0 + cc0 + k % cols, by = WY0 + k / cols;
      sfi[k] = (bx >= 0 && bx < P.W && by >= 0 && by < P.H) ? P.fi[(long long)by * P.W + bx] : (uint8_t)DEB_NOSRC;
    }
    __syncthreads();
    /* 2. row-major compaction: thread t takes positions [t*DEB_Q, t*DEB_Q + DEB_Q) */
    const int p0 = tid * DEB_Q;
    int mine = 0;
#pragma unroll
    for (int q = 0; q < DEB_Q; q++) mine += (p0 + q < npos && sfi[p0 + q] != DEB_NOSRC);
    int incl = mine;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    int base = incl - mine;
    for (int w = 0; w < warp; w++) base += wsum[w];
    if (tid == DEB_THREADS - 1) {
      int total = 0;
      for (int w = 0; w < DEB_WARPS; w++) total += wsum[w];
      rowstart[WH] = total;
    }
    /* 3. records: position, kernel, reach, log-scaled channels (rect.c:120-123) */
#pragma unroll
    for (int q = 0; q < DEB_Q; q++) {
      const int p = p0 + q;
      if (p >= npos) break;
      const int c = p % cols, r = p / cols;
      if (c == 0) rowstart[r] = base;
      const unsigned k = sfi[p];
      if (k == DEB_NOSRC) continue;
      float4 v = load_bucket(P.buckets, P.bkind, (long long)(WY0 + r) * P.W + (WX0 + cc0 + c));
      const float ls = log_scale_nz(v.w, P.k1, P.k2);
      const unsigned reach = (unsigned)kin[k].w;
      sv[base] = make_float4(v.x * ls, v.y * ls, v.z * ls, v.w * ls);
      sxyk[base] = (uint32_t)(cc0 + c) | ((uint32_t)r << 8) | (k << 16) | (reach << 24);
      atomicMax(rowreach + r, (int)reach);
      base++;
    }
    __syncthreads();
    /* 4. this warp's band takes every listed source whose kernel reaches it:
     *    rows whose widest kernel falls short are skipped whole */
    for (int rr = rlo; rr <= rhi; rr++) {
      const int sy = WY0 + rr;
      const int dyb = sy < B0 ? B0 - sy : (sy > B0 + DEB_ROWS - 1 ? sy - (B0 + DEB_ROWS - 1) : 0);
      if (rowreach[rr] < dyb) continue; /* uniform over the warp */
      const int i1 = rowstart[rr + 1];
      for (int i = rowstart[rr]; i < i1; i++) {
        const uint32_t xyk = sxyk[i];
        const int reach = (int)(xyk >> 24);
        const int sx = WX0 + (int)(xyk & 0xffu);
        if (reach < dyb || sx + reach < X0 || sx - reach > X0 + DEB_TW - 1) continue; /* uniform */
        const float4 ki = kin[(xyk >> 16) & 0xffu];
        const int dy0 = B0 - sy;
        const float4 v = sv[i];
        const int r2max = (int)ki.z;
        if (STATS) n_pairs++;
        /* taps inside the kernel's disc and inside its reach box: the
         * reference visits offsets up to ceil(h)-1 only (rect.c:121-126),
         * though an integer width puts non-zero coefficients at distance h;
         * colf and rowf are zero outside the box */
        const int dx = X0 + lane - sx, dx2 = dx * dx;
        const bool xin = dx2 <= r2max && dx >= -reach && dx <= reach;
        const float colf = xin ? exp2f(ki.y * (float)dx2) : 0.0f;
        const int mdy = dy0 + (lane & (DEB_ROWS - 1));
        const float rf = (mdy >= -reach && mdy <= reach) ? ki.x * exp2f(ki.y * (float)(mdy * mdy)) : 0.0f;
#pragma unroll
        for (int r = 0; r < DEB_ROWS; r++) {
          const int dy = dy0 + r;
          const float rowf = __shfl_sync(0xffffffffu, rf, r);
          const bool disc = dx2 + dy * dy <= r2max;
          const float w = disc ? colf * rowf : 0.0f;
          if (STATS) n_taps += __popc(__ballot_sync(0xffffffffu, disc && xin && dy >= -reach && dy <= reach));
          acc[r][0] = fmaf(w, v.x, acc[r][0]);
          acc[r][1] = fmaf(w, v.y, acc[r][1]);
          acc[r][2] = fmaf(w, v.z, acc[r][2]);
          acc[r][3] = fmaf(w, v.w, acc[r][3]);
        }
      }
    }
    __syncthreads(); /* the list is reused by the next chunk */
  }
  if (STATS && lane == 0) {
    atomicAdd(P.stats + 1, n_pairs);
    atomicAdd(P.stats + 2, n_taps);
  }
  /* 5. the tile to the accumulator */
  const int x = X0 + lane;
  if (x >= P.W) return;
#pragma unroll
  for (int r = 0; r < DEB_ROWS; r++) {
    const int y = B0 + r;
    if (y >= P.H) break;
    const long long g = (long long)y * P.W + x;
    float4 a = make_float4(acc[r][0], acc[r][1], acc[r][2], acc[r][3]);
    if (P.add) {
      const float4 o = acc_load(P.acc, P.akind, g);
      a = make_float4(o.x + a.x, o.y + a.y, o.z + a.z, o.w + a.w);
    }
    acc_store(P.acc, P.akind, g, a);
  }
}

static size_t bands_smem(int nk) {
  return (size_t)DEB_LCAP * (16 + 4) + (size_t)nk * 16 + DEB_LCAP + (2 * (DEB_WROWS + 1) + DEB_WARPS) * 4;
}

}  // namespace f3g

using namespace f3g;

extern "C" int f3g_de_bands_supported(int R, int mfi) { return R >= 0 && R <= DEB_MAX_REACH && mfi >= 0 && mfi < 255; }

/* The shared-memory limit is raised once, before any stream capture
 * (f3g_de_prepare calls this too). */
extern "C" int f3g_de_bands_prepare(void) {
  static volatile int done = 0;
  if (done) return 0;
  cudaError_t e = cudaFuncSetAttribute(k_de_bands<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)bands_smem(255));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_de_bands<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bands_smem(255));
  if (e == cudaSuccess) done = 1;
  return (int)e;
}

extern "C" int f3g_launch_de_bands(const void *buckets, int bkind, const void *count, int W, int H, int oversample,
                                   double k1, double k2, double curve, int mfc, int mfi, const float *kinfo, int R,
                                   uint8_t *fi, void *acc, int akind, int add, unsigned long long *stats,
                                   cudaStream_t st) {
  if (!f3g_de_bands_supported(R, mfi)) return -1;
  cudaError_t e = (cudaError_t)f3g_de_bands_prepare();
  if (e != cudaSuccess) return (int)e;
  DEClassify C;
  C.buckets = buckets;
  C.count = count;
  C.bkind = bkind;
  C.W = W;
  C.H = H;
  C.ss = oversample / 2;
  C.scf = !(oversample & 1);
  C.scfact = (float)((oversample / (oversample + 1.0)) * (oversample / (oversample + 1.0)));
  C.curve = (float)curve;
  C.mfc = mfc;
  C.mfi = mfi;
  /* the reference's DE loop bounds (rect.c:79-80, 979) */
  C.istart = oversample - 1;
  C.iend = W - (oversample - 1);
  C.jstart = oversample - 1;
  C.jend = H < (oversample - 1) + (H - 2 * (oversample - 1) + 1) ? H : (oversample - 1) + (H - 2 * (oversample - 1) + 1);
  C.fi = fi;
  C.stats = stats;
  const long long n = (long long)W * H;
  long long blocks = (n + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  k_de_classify<<<(int)(blocks > 0 ? blocks : 1), 256, 0, st>>>(C);
  DEBands B;
  B.buckets = buckets;
  B.bkind = bkind;
  B.W = W;
  B.H = H;
  B.R = R;
  B.nk = mfi + 1;
  B.k1 = (float)k1;
  B.k2 = (float)k2;
  B.fi = fi;
  B.kinfo = (const float4 *)kinfo;
  B.acc = acc;
  B.akind = akind;
  B.add = add;
  B.stats = stats;
  dim3 grid((W + DEB_TW - 1) / DEB_TW, (H + DEB_TH - 1) / DEB_TH);
  if (stats)
    k_de_bands<true><<<grid, DEB_THREADS, bands_smem(mfi + 1), st>>>(B);
  else
    k_de_bands<false><<<grid, DEB_THREADS, bands_smem(mfi + 1), st>>>(B);
  return (int)cudaGetLastError();
}
