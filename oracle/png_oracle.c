/*
 * png_oracle.c -- TEST ORACLE for the PNG output step.  Plain C99.
 *
 * The reference writes PNGs through libpng (png.c:36-116, write_png), a
 * third-party library that the reference does not carry; its source is not
 * part of the reference tree.  What the reference fixes at its call site:
 * RGBA (PNG colour type 6) at 8 * bpc bits per sample, no interlace, base
 * compression and filter method (png.c:93-98), 16-bit samples swapped from
 * host order to PNG's big-endian order (png.c:105-107), all rows written at
 * once (png.c:109).  libpng then filters each row with the adaptive rule
 * that the PNG specification (ISO/IEC 15948, "Filter selection") recommends
 * for truecolour images: apply each of the five filters and keep the one
 * whose output bytes, read as signed values, have the smallest sum of
 * absolute values.  This file restates that filtering step and its inverse;
 * the deflate step is checked by decoding with zlib.  Only tests/ and
 * bench.py's CPU-baseline leg use it.
 */
#include <stdlib.h>
#include <string.h>

static int paeth(int a, int b, int c) {
  const int p = a + b - c;
  const int pa = abs(p - a), pb = abs(p - b), pc = abs(p - c);
  if (pa <= pb && pa <= pc) return a;
  if (pb <= pc) return b;
  return c;
}

static int predict(int k, int a, int b, int c) {
  switch (k) {
    case 0: return 0;
    case 1: return a;
    case 2: return b;
    case 3: return (a + b) >> 1;
    default: return paeth(a, b, c);
  }
}

/* byte i of row r in PNG order: 16-bit samples big-endian */
static int pbyte(const unsigned char *img, long long RB, int r, long long i, int bpc) {
  return img[(long long)r * RB + (bpc == 2 ? (i ^ 1) : i)];
}

/* The filtered stream write_png's libpng call deflates: h rows of a filter
 * type byte and w*nchan*bpc filtered bytes.  Returns its length. */
long long oracle_png_filter(const unsigned char *img, int w, int h, int nchan, int bpc, unsigned char *F) {
  const long long RB = (long long)w * nchan * bpc;
  const int bpp = nchan * bpc;
  for (int r = 0; r < h; r++) {
    unsigned long long sum[5] = {0, 0, 0, 0, 0};
    for (long long i = 0; i < RB; i++) {
      const int x = pbyte(img, RB, r, i, bpc);
      const int a = i >= bpp ? pbyte(img, RB, r, i - bpp, bpc) : 0;
      const int b = r ? pbyte(img, RB, r - 1, i, bpc) : 0;
      const int c = (r && i >= bpp) ? pbyte(img, RB, r - 1, i - bpp, bpc) : 0;
      for (int k = 0; k < 5; k++) {
        const int v = (x - predict(k, a, b, c)) & 255;
        sum[k] += v < 128 ? v : 256 - v;
      }
    }
    int best = 0;
    for (int k = 1; k < 5; k++)
      if (sum[k] < sum[best]) best = k;
    unsigned char *o = F + (long long)r * (RB + 1);
    o[0] = (unsigned char)best;
    for (long long i = 0; i < RB; i++) {
      const int x = pbyte(img, RB, r, i, bpc);
      const int a = i >= bpp ? pbyte(img, RB, r, i - bpp, bpc) : 0;
      const int b = r ? pbyte(img, RB, r - 1, i, bpc) : 0;
      const int c = (r && i >= bpp) ? pbyte(img, RB, r - 1, i - bpp, bpc) : 0;
      o[1 + i] = (unsigned char)((x - predict(best, a, b, c)) & 255);
    }
  }
  return (long long)h * (RB + 1);
}

/* Inverse of the filtering (a PNG decoder's reconstruction step): the image
 * in host sample order (16-bit little-endian).  Returns 0, or 1 on an
 * unknown filter type. */
int oracle_png_unfilter(const unsigned char *F, int w, int h, int nchan, int bpc, unsigned char *img) {
  const long long RB = (long long)w * nchan * bpc;
  const int bpp = nchan * bpc;
  unsigned char *prev = calloc((size_t)RB + 1, 1), *cur = calloc((size_t)RB + 1, 1);
  if (!prev || !cur) {
    free(prev);
    free(cur);
    return 1;
  }
  int bad = 0;
  for (int r = 0; r < h && !bad; r++) {
    const unsigned char *f = F + (long long)r * (RB + 1);
    const int k = f[0];
    if (k > 4) {
      bad = 1;
      break;
    }
    for (long long i = 0; i < RB; i++) {
      const int a = i >= bpp ? cur[i - bpp] : 0;
      const int b = prev[i];
      const int c = i >= bpp ? prev[i - bpp] : 0;
      cur[i] = (unsigned char)((f[1 + i] + predict(k, a, b, c)) & 255);
    }
    for (long long i = 0; i < RB; i++) img[(long long)r * RB + (bpc == 2 ? (i ^ 1) : i)] = cur[i];
    unsigned char *t = prev;
    prev = cur;
    cur = t;
  }
  free(prev);
  free(cur);
  return bad;
}
