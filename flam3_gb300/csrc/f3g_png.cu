/*
 * f3g_png.cu -- the PNG encoder's kernels (write_png, png.c:36-116, done on
 * the device): K_filter (one CTA per image row: the five PNG filters, the
 * cheapest by the sum of absolute signed bytes, first on ties), K_deflate
 * (one CTA per 32 KB segment of the filtered stream, see f3g_png.cuh) and
 * K_assemble (IDAT chunks laid end to end with the zlib header and Adler-32
 * trailer chunks, one CTA per segment).
 */
#include <cuda_runtime.h>

#include "f3g_launch.h"
#include "f3g_png.cuh"

using namespace f3gpng;

namespace {

constexpr int FT = 256; /* threads of the filter kernel */

/* the filtered bytes of 4 consecutive stream bytes (x, left a, up b,
 * up-left c as little-endian words) for filter k */
__device__ __forceinline__ uint32_t filter_word(int k, uint32_t x, uint32_t a, uint32_t b, uint32_t c) {
  uint32_t o = 0;
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const int sh = 8 * q;
    o |= (uint32_t)filter_byte(k, (x >> sh) & 255, (a >> sh) & 255, (b >> sh) & 255, (c >> sh) & 255) << sh;
  }
  return o;
}

__device__ __forceinline__ uint32_t cost_word(int k, uint32_t x, uint32_t a, uint32_t b, uint32_t c) {
  uint32_t s = 0;
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const int sh = 8 * q;
    s += filter_cost(filter_byte(k, (x >> sh) & 255, (a >> sh) & 255, (b >> sh) & 255, (c >> sh) & 255));
  }
  return s;
}

/* row r of the image, in PNG byte order (16-bit samples big-endian: the
 * image holds them little-endian, as png_set_swap undoes in png.c:105-107).
 * RGBA rows (4 or 8 bytes per pixel) are read as words: the left neighbour
 * is the previous word (8-bit) or the one before (16-bit, bytes of each
 * sample swapped with a byte permute); RGB rows byte by byte. */
__global__ void __launch_bounds__(FT) k_png_filter(const uint8_t *__restrict__ img, int w, int h, int bpp, int bpc,
                                                   uint8_t *__restrict__ F) {
  const int r = blockIdx.x;
  const long long RB = (long long)w * bpp;
  const uint8_t *row = img + (long long)r * RB;
  const uint8_t *up = r ? row - RB : nullptr;
  const int sw = bpc == 2 ? 1 : 0;
  /* word path: 4-byte aligned rows of whole words with a whole-word left
   * neighbour */
  const bool words = (bpp == 4 || bpp == 8) && ((reinterpret_cast<uintptr_t>(img) & 3) == 0);
  const int lw = bpp / 4; /* left neighbour distance in words */
  const uint32_t *row4 = reinterpret_cast<const uint32_t *>(row);
  const uint32_t *up4 = reinterpret_cast<const uint32_t *>(up);
  const long long nw = RB / 4;
  auto ld = [&](const uint32_t *p, long long i) -> uint32_t {
    const uint32_t v = p[i];
    return sw ? __byte_perm(v, 0, 0x2301) : v;
  };
  uint32_t s[5] = {0, 0, 0, 0, 0};
  if (words) {
    for (long long i = threadIdx.x; i < nw; i += FT) {
      const uint32_t x = ld(row4, i);
      const uint32_t a = i >= lw ? ld(row4, i - lw) : 0;
      const uint32_t b = up ? ld(up4, i) : 0;
      const uint32_t c = (up && i >= lw) ? ld(up4, i - lw) : 0;
#pragma unroll
      for (int k = 0; k < 5; k++) s[k] += cost_word(k, x, a, b, c);
    }
  } else {
    for (long long i = threadIdx.x; i < RB; i += FT) {
      const int x = row[i ^ sw];
      const int a = i >= bpp ? row[(i - bpp) ^ sw] : 0;
      const int b = up ? up[i ^ sw] : 0;
      const int c = (up && i >= bpp) ? up[(i - bpp) ^ sw] : 0;
#pragma unroll
      for (int k = 0; k < 5; k++) s[k] += filter_cost(filter_byte(k, x, a, b, c));
    }
  }
  __shared__ uint32_t red[5][FT / 32];
  __shared__ int best;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 5; k++) {
    uint32_t v = s[k];
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (!lane) red[k][wid] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long bs = ~0ull;
    int bk = 0;
    for (int k = 0; k < 5; k++) {
      unsigned long long t = 0;
      for (int q = 0; q < FT / 32; q++) t += red[k][q];
      if (t < bs) bs = t, bk = k;
    }
    best = bk;
  }
  __syncthreads();
  const int k = best;
  uint8_t *o = F + (long long)r * (RB + 1);
  if (threadIdx.x == 0) o[0] = (uint8_t)k;
  if (words) {
    for (long long i = threadIdx.x; i < nw; i += FT) {
      const uint32_t x = ld(row4, i);
      const uint32_t a = i >= lw ? ld(row4, i - lw) : 0;
      const uint32_t b = up ? ld(up4, i) : 0;
      const uint32_t c = (up && i >= lw) ? ld(up4, i - lw) : 0;
      const uint32_t v = filter_word(k, x, a, b, c);
      uint8_t *d = o + 1 + 4 * i; /* 1 + 4i: not word aligned */
      d[0] = (uint8_t)v, d[1] = (uint8_t)(v >> 8), d[2] = (uint8_t)(v >> 16), d[3] = (uint8_t)(v >> 24);
    }
  } else {
    for (long long i = threadIdx.x; i < RB; i += FT) {
      const int x = row[i ^ sw];
      const int a = i >= bpp ? row[(i - bpp) ^ sw] : 0;
      const int b = up ? up[i ^ sw] : 0;
      const int c = (up && i >= bpp) ? up[(i - bpp) ^ sw] : 0;
      o[1 + i] = (uint8_t)filter_byte(k, x, a, b, c);
    }
  }
}

__global__ void __launch_bounds__(NT) k_png_deflate(SegArgs A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SegShared &S = *reinterpret_cast<SegShared *>(smem_raw);
  const int seg = blockIdx.x, tid = threadIdx.x;
  phase_init(S, A, seg, tid);
  __syncthreads();
  phase_window(S, A, seg, tid);
  __syncthreads();
  phase_parse(S, A, seg, tid);
  __syncthreads();
  phase_trim(S, A, seg, tid);
  __syncthreads();
  phase_keys(S, tid);
  __syncthreads();
  sort_keys(S, tid);
  phase_bounds(S, tid);
  __syncthreads();
  phase_rank(S, tid);
  __syncthreads();
  phase_lengths(S, tid);
  __syncthreads();
  phase_codes(S, tid);
  __syncthreads();
  phase_rle_count(S, tid);
  __syncthreads();
  phase_rle_scan(S, tid);
  __syncthreads();
  phase_rle_write(S, tid);
  __syncthreads();
  phase_cl_code(S, tid);
  __syncthreads();
  phase_hdr_bits(S, tid);
  phase_count(S, A, seg, tid);
  __syncthreads();
  phase_layout(S, A, seg, tid);
  __syncthreads();
  phase_emit(S, A, seg, tid);
  __syncthreads();
  uint32_t q;
  phase_crc_parts(S, tid, q);
  if (tid < 32) {
    /* warp 0: the shifts of the combine levels and of the whole chunk */
    uint32_t x = xpow8_warp(q);
    const uint32_t xn = xpow8_warp(4 + S.nbytes);
    if (tid == 0) {
      S.crc_xn = xn;
      for (int l = 0; l < LOG_NT; l++) {
        S.crc_x[l] = x;
        x = gf2_mult(x, x);
      }
    }
  }
  __syncthreads();
  for (int l = 0; l < LOG_NT; l++) {
    phase_crc_level(S, tid, l, S.crc_x[l]);
    __syncthreads();
  }
  phase_store(S, A, seg, tid);
}

__device__ void put_be32(uint8_t *p, uint32_t v) {
  p[0] = (uint8_t)(v >> 24), p[1] = (uint8_t)(v >> 16), p[2] = (uint8_t)(v >> 8), p[3] = (uint8_t)v;
}

/* CRC-32 of "IDAT" followed by n bytes, bitwise (the few bytes of the zlib
 * header and trailer chunks) */
__device__ uint32_t crc_idat_small(const uint8_t *d, int n) {
  uint32_t c = 0xFFFFFFFFu;
  for (int i = 0; i < 4 + n; i++) {
    c ^= i < 4 ? (uint8_t)("IDAT"[i]) : d[i - 4];
    for (int k = 0; k < 8; k++) c = (c & 1u) ? (c >> 1) ^ CRC_POLY : c >> 1;
  }
  return c ^ 0xFFFFFFFFu;
}

/* one small IDAT chunk: length, type, payload, CRC */
__device__ void small_chunk(uint8_t *o, const uint8_t *d, int n) {
  put_be32(o, (uint32_t)n);
  o[4] = 'I', o[5] = 'D', o[6] = 'A', o[7] = 'T';
  for (int i = 0; i < n; i++) o[8 + i] = d[i];
  put_be32(o + 8 + n, crc_idat_small(d, n));
}

constexpr int HDR_CHUNK = 14, TRL_CHUNK = 16;

__global__ void __launch_bounds__(NT) k_png_assemble(const uint8_t *__restrict__ stage,
                                                     const SegMeta *__restrict__ meta, int nseg, long long total,
                                                     uint8_t *__restrict__ out, unsigned long long *out_len) {
  const int s = blockIdx.x, tid = threadIdx.x;
  __shared__ unsigned long long red[NT], red2[NT];
  unsigned long long acc = 0;
  for (int j = tid; j < s; j += NT) acc += 12ull + meta[j].nbytes;
  red[tid] = acc;
  __syncthreads();
  for (int o = NT / 2; o; o >>= 1) {
    if (tid < o) red[tid] += red[tid + o];
    __syncthreads();
  }
  const unsigned long long off = HDR_CHUNK + red[0];
  const SegMeta m = meta[s];
  uint8_t *o = out + off;
  const uint8_t *src = stage + (size_t)s * STAGE;
  for (uint32_t i = tid; i < m.nbytes; i += NT) o[8 + i] = src[i];
  if (tid == 0) {
    put_be32(o, m.nbytes);
    o[4] = 'I', o[5] = 'D', o[6] = 'A', o[7] = 'T';
    put_be32(o + 8 + m.nbytes, m.crc);
  }
  if (s == 0 && tid == 0) {
    /* CMF 0x78: deflate, 32 KB window; FLG 0x01: check bits, no dictionary */
    const uint8_t zh[2] = {0x78, 0x01};
    small_chunk(out, zh, 2);
  }
  if (s != nseg - 1) return;
  /* Adler-32 of the whole filtered stream from the segments' partial sums:
   * a = 1 + sum s1, b = total + sum (s2 + s1 * bytes after the segment) */
  __syncthreads();
  unsigned long long a = 0, b = 0;
  for (int j = tid; j < nseg; j += NT) {
    const SegMeta mj = meta[j];
    long long end = (long long)(j + 1) * SEG;
    if (end > total) end = total;
    const unsigned long long after = (unsigned long long)(total - end) % ADLER_MOD;
    a += mj.s1;
    b += mj.s2 + ((unsigned long long)mj.s1 * after) % ADLER_MOD;
  }
  red[tid] = a % ADLER_MOD;
  red2[tid] = b % ADLER_MOD;
  __syncthreads();
  for (int w = NT / 2; w; w >>= 1) {
    if (tid < w) red[tid] += red[tid + w], red2[tid] += red2[tid + w];
    __syncthreads();
  }
  if (tid == 0) {
    const uint32_t A = (uint32_t)((1 + red[0]) % ADLER_MOD);
    const uint32_t B = (uint32_t)(((unsigned long long)total % ADLER_MOD + red2[0]) % ADLER_MOD);
    const uint32_t ad = (B << 16) | A;
    const uint8_t tr[4] = {(uint8_t)(ad >> 24), (uint8_t)(ad >> 16), (uint8_t)(ad >> 8), (uint8_t)ad};
    uint8_t *t = o + 12 + m.nbytes;
    small_chunk(t, tr, 4);
    *out_len = (unsigned long long)(t + TRL_CHUNK - out);
  }
}

}  // namespace

extern "C" {

long long f3g_png_filtered_bytes(int w, int h, int nchan, int bpc) {
  return (long long)h * (1 + (long long)w * nchan * bpc);
}

int f3g_png_segments(int w, int h, int nchan, int bpc) {
  return (int)((f3g_png_filtered_bytes(w, h, nchan, bpc) + SEG - 1) / SEG);
}

/* device scratch for one encode: filtered stream, segment staging, metadata */
size_t f3g_png_work_bytes(int w, int h, int nchan, int bpc) {
  const long long fb = f3g_png_filtered_bytes(w, h, nchan, bpc);
  const long long ns = f3g_png_segments(w, h, nchan, bpc);
  return (size_t)(((fb + 255) / 256) * 256 + ns * STAGE + ns * (long long)sizeof(SegMeta) +
                  ns * (long long)TOK_PER_SEG * 2);
}

/* the IDAT chunks' bytes, at most */
size_t f3g_png_idat_bound(int w, int h, int nchan, int bpc) {
  const long long ns = f3g_png_segments(w, h, nchan, bpc);
  return (size_t)(HDR_CHUNK + TRL_CHUNK + ns * (12 + (long long)STAGE));
}

/* Encodes the w x h image (nchan 3 or 4 channels of bpc 1 or 2 bytes,
 * row-major, 16-bit samples little-endian) at d_img into the IDAT chunks of
 * a PNG at d_idat; *d_len receives their byte count.  All on stream st. */
int f3g_png_encode_idat(const void *d_img, int w, int h, int nchan, int bpc, void *d_work, void *d_idat,
                        unsigned long long *d_len, cudaStream_t st) {
  if (w <= 0 || h <= 0 || (nchan != 3 && nchan != 4) || (bpc != 1 && bpc != 2)) return 1;
  const int bpp = nchan * bpc;
  const long long fb = f3g_png_filtered_bytes(w, h, nchan, bpc);
  const int ns = f3g_png_segments(w, h, nchan, bpc);
  uint8_t *F = (uint8_t *)d_work;
  uint8_t *stage = F + ((fb + 255) / 256) * 256;
  SegMeta *meta = (SegMeta *)(stage + (size_t)ns * STAGE);
  uint16_t *tokens = (uint16_t *)(meta + ns);
  const int smem = (int)sizeof(SegShared);
  /* per device and cheap: set on every call */
  if (cudaFuncSetAttribute(k_png_deflate, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess) return 2;
  k_png_filter<<<h, FT, 0, st>>>((const uint8_t *)d_img, w, h, bpp, bpc, F);
  SegArgs A;
  A.F = F;
  A.total = fb;
  A.bpp = bpp;
  A.stride = (int)(1 + (long long)w * bpp > 0x7fffffff ? 0x7fffffff : 1 + (long long)w * bpp);
  A.nseg = ns;
  A.stage = stage;
  A.meta = meta;
  A.tokens = tokens;
  k_png_deflate<<<ns, NT, smem, st>>>(A);
  k_png_assemble<<<ns, NT, 0, st>>>(stage, meta, ns, fb, (uint8_t *)d_idat, d_len);
  return cudaGetLastError() == cudaSuccess ? 0 : 3;
}

}  // extern "C"
