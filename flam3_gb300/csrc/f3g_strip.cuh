/*
 * f3g_strip.cuh -- the separable strip kernel of the render tail: log
 * scaling (rect.c:933-974) + spatial filter + tonemap + pack
 * (rect.c:1067-1247) in one pass over the histogram, for one batch without
 * density estimation.  Instantiated per filter width in f3g_strip_f32.cu,
 * f3g_strip_f64.cu, f3g_strip_f32e.cu and f3g_strip_f64e.cu (FP32 / FP64
 * histograms, earlyclip off / on), which compile in parallel.
 *
 * flam3's spatial filter is separable (filters.c:217-270 builds it as the
 * product of one kernel in x and one in y), so it is applied as its two
 * factors, stored after the fw x fw filter as fu[fw] (vertical) and fv[fw]
 * (horizontal), vertical pass first.  A block of LS_T threads owns SS
 * histogram columns per thread (LS_T*SS consecutive columns: OC = LS_T -
 * (fw-SS)/SS output columns; neighbouring blocks overlap by fw-SS columns)
 * and walks a strip of output rows.  Each thread streams its own columns'
 * histogram rows through a private ring of F3G_STRIP_STAGES shared-memory
 * stages with cp.async (STAGES-1 rows in flight), log-scales each bucket
 * once and adds it with the vertical weights into register accumulators of
 * the NR = fw/SS output rows it touches -- no barrier per histogram row,
 * since a thread reads only what it copied.  A complete output row's
 * vertically filtered values (at histogram resolution) are parked in shared
 * memory; every NR output rows a barrier, and each thread filters its output
 * pixel of each parked row horizontally (fw taps), tonemaps and packs it (the
 * tonemap code exists once, in a rolled loop).  Channel arithmetic runs as packed f32x2
 * operations (two lanes per instruction, each rounded like the scalar
 * operation).
 *
 * Odd strips walk upwards, so the halo rows that two neighbouring strips
 * share are read by both at about the same time (the second read hits L2).
 * The filtered row is stored with column c at (c % SS) * PV + c / SS, so the
 * horizontal taps of a warp read consecutive float4 (no bank conflicts).
 */
#ifndef F3G_STRIP_CUH
#define F3G_STRIP_CUH

#include <cuda_runtime.h>
#include <stdint.h>

#include "f3g_common.h"
#include "f3g_launch.h"
#include "f3g_tail.cuh"

#ifndef LS_T
#define LS_T 128
#endif
#ifndef F3G_STRIP_STAGES
#define F3G_STRIP_STAGES 4
#endif

namespace f3g {

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

/* two FP32 lanes in one 64-bit register */
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 x2_pack(float lo, float hi) {
  f32x2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ void x2_unpack(f32x2 v, float &lo, float &hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f32x2 x2_fma(f32x2 a, f32x2 b, f32x2 c) {
  f32x2 r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}
__device__ __forceinline__ f32x2 x2_mul(f32x2 a, f32x2 b) {
  f32x2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}

#ifndef F3G_STRIP_MINB
#define F3G_STRIP_MINB 6
#endif
/* Register budget: 65536 / (LS_T * F3G_STRIP_MINB) per thread while a bucket
 * touches at most 5 output rows, 128 above.  EARLY: tonemap each bucket
 * before the filter (flam3's earlyclip) instead of each output pixel.  LOG:
 * the input is the histogram, log-scaled here; without it, the input is an
 * accumulator that density estimation has already filled with log-scaled
 * values. */
template <int SS, int FW, bool F64, bool EARLY, bool LOG = true>
__global__ void __launch_bounds__(LS_T, (FW / SS <= 5 ? F3G_STRIP_MINB : 4))
    k_log_filter_strip(const void *__restrict__ buckets, int W, int H, float k1, float k2, int de_offset,
                       const float *__restrict__ filter, int image_w, int image_h, int OC, unsigned char *out,
                       F3GTonemap tp) {
  static_assert(FW % SS == 0, "filter width and oversample have the same parity");
  constexpr int NR = FW / SS, NS = F3G_STRIP_STAGES;
  static_assert((NS & (NS - 1)) == 0, "ring stages: a power of two");
  constexpr int BB = F64 ? 32 : 16;     /* bytes per bucket */
  constexpr int PV = LS_T;              /* filtered-row stride per residue class */
  constexpr int STAGE = LS_T * SS * BB; /* bytes of one ring stage */
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ulonglong2 *vrow = (ulonglong2 *)(smem_raw + NS * STAGE); /* NR x SS*PV: one group's rows */
  f32x2 *fv = (f32x2 *)(vrow + NR * SS * PV);               /* horizontal taps, packed */
  const int t = threadIdx.x;
  /* strips of image_h / gridDim.y rows (the grid is sized to the resident
   * capacity, so every SM gets the same number of rows) */
  const int i0 = blockIdx.x * OC;
  const int j0 = (int)((long long)blockIdx.y * image_h / gridDim.y);
  const int j1 = (int)((long long)(blockIdx.y + 1) * image_h / gridDim.y);
  const bool rev = blockIdx.y & 1;
  const int bx = de_offset + i0 * SS + t * SS; /* first histogram column of this thread */
  const float *fu = filter + FW * FW, *fvg = fu + FW;
  if (t < FW) {
    const float w = __ldg(fvg + t);
    fv[t] = x2_pack(w, w); /* first read after the first row barrier */
  }
  /* Step j adds histogram rows (j + NR - 1)*SS + q (q < SS) of the strip's
   * walking order to output rows j + s (s < NR) with vertical tap
   * (NR-1-s)*SS + q; an upward strip walks the rows and taps mirrored. */
  f32x2 cv[SS][NR];
#pragma unroll
  for (int q = 0; q < SS; q++)
#pragma unroll
    for (int s = 0; s < NR; s++) {
      const int tap = (NR - 1 - s) * SS + q;
      const float w = __ldg(fu + (rev ? FW - 1 - tap : tap));
      cv[q][s] = x2_pack(w, w);
    }
  /* acc[p]: output row j + ((p - x) mod NR) at unrolled position x */
  f32x2 acc[NR][SS][2];
#pragma unroll
  for (int p = 0; p < NR; p++)
#pragma unroll
    for (int e = 0; e < SS; e++) acc[p][e][0] = acc[p][e][1] = 0ull;

  /* rows of the strip: n = 0 .. nrows-1, histogram row by_first + dir*n */
  const int nrows = (j1 - j0) * SS + FW - SS;
  const int dir = rev ? -1 : 1;
  const int by_first = de_offset + (rev ? (j1 - 1) * SS + FW - 1 : j0 * SS);
  /* this thread's next row to copy: g walks by +-W buckets per row */
  const long long gstep = (long long)dir * W * BB;
  const unsigned char *g = (const unsigned char *)buckets + ((long long)by_first * W + bx) * BB;
  int col_bytes[SS]; /* 16 where the column exists, 0 past the histogram's right edge */
#pragma unroll
  for (int e = 0; e < SS; e++) col_bytes[e] = bx + e < W ? 16 : 0;
  const unsigned sbase = (unsigned)__cvta_generic_to_shared(smem_raw) + t * SS * BB;
  /* copies of this thread's buckets of row n into ring slot n mod NS (one
   * commit group, empty past the last row); rows are issued in order */
  auto issue_row = [&](int n) {
    if (n < nrows) {
      const unsigned sd = sbase + (unsigned)(n & (NS - 1)) * STAGE;
      const bool rok = by_first + dir * n < H;
#pragma unroll
      for (int e = 0; e < SS; e++) {
        const int nb = rok ? col_bytes[e] : 0;
        const unsigned char *ge = nb ? g + e * BB : (const unsigned char *)buckets;
#pragma unroll
        for (int h = 0; h < BB; h += 16)
          asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(sd + e * BB + h), "l"(ge + (nb ? h : 0)),
                       "r"(nb)
                       : "memory");
      }
      g += gstep;
    }
    cp_async_commit();
  };
#pragma unroll
  for (int n = 0; n < NS - 1; n++) issue_row(n);
  const unsigned char *mine = smem_raw + t * SS * BB;
  int n = 0; /* next row to consume */
  for (int jb = j0 - NR + 1; jb < j1; jb += NR) {
#pragma unroll
    for (int x = 0; x < NR; x++) {
      const int j = jb + x;
      if (j < j1) { /* uniform over the block */
#pragma unroll
        for (int q = 0; q < SS; q++, n++) {
          cp_async_wait<NS - 2>();
          const unsigned char *src = mine + (n & (NS - 1)) * STAGE;
          f32x2 c01[SS], c23[SS];
#pragma unroll
          for (int e = 0; e < SS; e++) {
            if (!F64) {
              const ulonglong2 c = ((const ulonglong2 *)src)[e];
              c01[e] = c.x;
              c23[e] = c.y;
            } else {
              const double2 d01 = ((const double2 *)src)[2 * e], d23 = ((const double2 *)src)[2 * e + 1];
              c01[e] = x2_pack((float)d01.x, (float)d01.y);
              c23[e] = x2_pack((float)d23.x, (float)d23.y);
            }
          }
          /* the slot of row n-1 is free: this thread has read it */
          issue_row(n + NS - 1);
#pragma unroll
          for (int e = 0; e < SS; e++) {
            f32x2 v01 = c01[e], v23 = c23[e];
            if (LOG) {
              float c2, c3;
              x2_unpack(c23[e], c2, c3);
              const float ls = log_scale_nz(c3, k1, k2);
              const f32x2 ls2 = x2_pack(ls, ls);
              v01 = x2_mul(c01[e], ls2);
              v23 = x2_mul(c23[e], ls2);
              if (tp.trunc_acc) { /* integer accumulator (bits 32) */
                float e4[4];
                x2_unpack(v01, e4[0], e4[1]);
                x2_unpack(v23, e4[2], e4[3]);
                v01 = x2_pack(truncf(e4[0]), truncf(e4[1]));
                v23 = x2_pack(truncf(e4[2]), truncf(e4[3]));
              }
            }
            if (EARLY) {
              float e4[4];
              x2_unpack(v01, e4[0], e4[1]);
              x2_unpack(v23, e4[2], e4[3]);
              tonemap(e4, tp);
              if (tp.trunc_acc)
                for (int k = 0; k < 4; k++) e4[k] = truncf(e4[k]);
              v01 = x2_pack(e4[0], e4[1]);
              v23 = x2_pack(e4[2], e4[3]);
            }
#pragma unroll
            for (int s = 0; s < NR; s++) {
              const int p = (x + s) % NR;
              acc[p][e][0] = x2_fma(cv[q][s], v01, acc[p][e][0]);
              acc[p][e][1] = x2_fma(cv[q][s], v23, acc[p][e][1]);
            }
          }
        }
        const int p0 = x % NR; /* output row j (static once unrolled) */
        if (j >= j0) {         /* output row j is complete: park it for the group's emission */
          ulonglong2 *vb = vrow + x * SS * PV;
#pragma unroll
          for (int e = 0; e < SS; e++) vb[e * PV + t] = make_ulonglong2(acc[p0][e][0], acc[p0][e][1]);
        }
#pragma unroll
        for (int e = 0; e < SS; e++) acc[p0][e][0] = acc[p0][e][1] = 0ull;
      }
    }
    /* emit the group's complete rows: horizontal filter, tonemap, pack */
    __syncthreads();
    const int i = i0 + t;
    if (t < OC && i < image_w) {
      for (int x = 0; x < NR; x++) {
        const int j = jb + x;
        if (j < j0 || j >= j1) continue;
        const ulonglong2 *vb = vrow + x * SS * PV;
        f32x2 h01 = 0ull, h23 = 0ull;
#pragma unroll
        for (int k = 0; k < FW; k++) {
          const f32x2 w2 = fv[k];
          const ulonglong2 a = vb[(k % SS) * PV + t + k / SS];
          h01 = x2_fma(w2, a.x, h01);
          h23 = x2_fma(w2, a.y, h23);
        }
        float tt[4];
        x2_unpack(h01, tt[0], tt[1]);
        x2_unpack(h23, tt[2], tt[3]);
        if (!EARLY) tonemap(tt, tp);
        const int o = rev ? j0 + j1 - 1 - j : j;
        pack_pixel(out + (size_t)tp.nchan * tp.bpc * ((size_t)i + (size_t)o * image_w), tt, tp);
      }
    }
    __syncthreads(); /* the parked rows are read */
  }
  cp_async_wait<0>();
}

}  // namespace f3g

using namespace f3g;

static inline size_t strip_smem(int ss, bool f64, int fw) {
  return (size_t)F3G_STRIP_STAGES * LS_T * ss * (f64 ? 32 : 16) + (size_t)(fw / ss) * ss * LS_T * 16 +
         (size_t)fw * 8;
}

static inline int num_sms(void) {
  static int n = 0;
  if (!n) {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v < 1)
      v = 1;
    n = v;
  }
  return n;
}

/* resident blocks per SM of one instantiation (queried once, outside any
 * stream capture: f3g_tail_prepare asks for every instantiation) */
template <int SS, int FW, bool D, bool E, bool L = true>
static int strip_occupancy(void) {
  static int occ = 0;
  if (!occ) {
    int o = 0;
    cudaFuncSetAttribute(k_log_filter_strip<SS, FW, D, E, L>, cudaFuncAttributePreferredSharedMemoryCarveout,
                         cudaSharedmemCarveoutMaxShared);
    cudaFuncSetAttribute(k_log_filter_strip<SS, FW, D, E, L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)strip_smem(SS, D, FW));
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_log_filter_strip<SS, FW, D, E, L>, LS_T,
                                                      strip_smem(SS, D, FW)) != cudaSuccess ||
        o < 1)
      o = 1;
    occ = o;
  }
  return occ;
}

/* One wave: as many strips as the resident capacity allows for the column
 * blocks (so every SM holds the same number of rows), with strips of 8 to
 * 32 output rows (shorter ones re-read too much vertical halo). */
template <int SS, int FW, bool D, bool E, bool L = true>
static int launch_strip(const void *buckets, int W, int H, double k1, double k2, int de_offset, const float *filter,
                        int image_w, int image_h, unsigned char *out, const F3GTonemap *tp, cudaStream_t st) {
  const int OC = LS_T - (FW - SS) / SS;
  const int gx = (image_w + OC - 1) / OC;
  const int cap = strip_occupancy<SS, FW, D, E, L>() * num_sms();
  int gy = cap / gx;
  const int gmin = (image_h + 31) / 32, gmax = (image_h + 7) / 8;
  if (gy < gmin) gy = gmin;
  if (gy > gmax) gy = gmax;
  if (gy < 1) gy = 1;
  k_log_filter_strip<SS, FW, D, E, L><<<dim3(gx, gy), LS_T, strip_smem(SS, D, FW), st>>>(
      buckets, W, H, (float)k1, (float)k2, de_offset, filter, image_w, image_h, OC, out, *tp);
  return (int)cudaGetLastError();
}

/* the filter widths with a strip instantiation: oversample 1 takes odd
 * widths 1..7, oversample 2 even widths 2..16 */
#define F3G_STRIP_WIDTHS(X) \
  X(1, 1) X(1, 3) X(1, 5) X(1, 7) X(2, 2) X(2, 4) X(2, 6) X(2, 8) X(2, 10) X(2, 12) X(2, 14) X(2, 16)

/* entry points of one histogram precision D and earlyclip mode E
 * (declared in f3g_launch.h) */
#define F3G_STRIP_ENTRIES(SUFFIX, D, E)                                                                           \
  extern "C" int f3g_strip_prepare_##SUFFIX(void) {                                                              \
    num_sms();                                                                                                    \
    F3G_STRIP_WIDTHS(F3G_STRIP_OCC)                                                                               \
    return 0;                                                                                                     \
  }                                                                                                               \
  extern "C" int f3g_strip_launch_##SUFFIX(const void *buckets, int W, int H, double k1, double k2, int de_offset, \
                                           int oversample, const float *filter, int fw, int image_w, int image_h,  \
                                           unsigned char *out, const F3GTonemap *tp, cudaStream_t st) {           \
    F3G_STRIP_WIDTHS(F3G_STRIP_CASE)                                                                              \
    return -2; /* no instantiation: the 2-D kernel runs */                                                        \
  }

#endif
