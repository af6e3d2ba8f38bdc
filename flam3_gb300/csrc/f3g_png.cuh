/*
 * f3g_png.cuh -- PNG encoding of a rendered image on the device: the
 * reference hands the packed RGBA image to libpng (png.c:36-116, write_png),
 * which filters each row (PNG filter types 0-4, chosen per row by the
 * minimum-sum-of-absolute-values rule) and deflates the filtered rows into
 * one zlib stream split over IDAT chunks.
 *
 * Here the filtered stream (h rows of 1 + w*bpp bytes) is cut into
 * segments of PNG_SEG bytes and each segment is deflated by one CTA on its
 * own: a greedy LZ77 parse over a few candidate distances that suit images
 * (1, one pixel, two pixels, one row), one dynamic-Huffman block per
 * segment (a stored block where that is smaller), the segment ended on a
 * byte boundary by an empty stored block, so every segment becomes one IDAT
 * chunk whose CRC the CTA computes itself.  Back-references may reach into
 * earlier segments (the decoder holds all of the stream), so cutting costs
 * only the few bytes of each block header.  The zlib header and the Adler-32
 * trailer are two small IDAT chunks of their own.
 *
 * Format constants follow RFC 1950 (zlib), RFC 1951 (deflate) and the PNG
 * specification (chunk layout, CRC-32 polynomial, filter types).
 *
 * The phase functions are plain __host__ __device__ code over one CTA's
 * shared state; the kernel runs them with a barrier between phases.
 */
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define PNG_HD __host__ __device__ __forceinline__
#else
#define PNG_HD inline
#endif

namespace f3gpng {

constexpr int SEG = 32768;          /* filtered bytes per segment (one CTA) */
constexpr int NT = 256;             /* threads per CTA */
constexpr int SUB = SEG / NT;       /* bytes parsed by one thread */
constexpr int MIN_MATCH = 4;        /* shortest match emitted (3 is legal) */
constexpr int MAX_MATCH = 258;
constexpr int WINDOW = 32768;
constexpr int NLIT = 286, NDIST = 30, NCL = 19;
constexpr int MAXD = 4;             /* candidate distances */
constexpr int OUT_BYTES = SEG + 64; /* a segment's deflate output, at most */
constexpr int STAGE = OUT_BYTES;    /* per-segment staging stride (bytes) */
constexpr uint32_t CRC_POLY = 0xEDB88320u;
constexpr uint32_t ADLER_MOD = 65521u;

struct SegMeta {
  uint32_t nbytes;  /* deflate bytes of the segment */
  uint32_t crc;     /* CRC-32 of "IDAT" + those bytes */
  uint32_t s1, s2;  /* Adler-32 partial sums of the segment's input (mod 65521) */
  uint32_t len;     /* input bytes */
  uint32_t mode;    /* 2 dynamic Huffman, 0 stored */
  uint32_t pad[2];
};

PNG_HD int ilog2(uint32_t v) {
#ifdef __CUDA_ARCH__
  return 31 - __clz((int)v);
#else
  return 31 - __builtin_clz(v);
#endif
}

PNG_HD void atomic_add_u32(uint32_t *p, uint32_t v) {
#ifdef __CUDA_ARCH__
  atomicAdd(p, v);
#else
  *p += v;
#endif
}

PNG_HD void atomic_or_u32(uint32_t *p, uint32_t v) {
#ifdef __CUDA_ARCH__
  atomicOr(p, v);
#else
  *p |= v;
#endif
}

PNG_HD uint32_t rev_bits(uint32_t c, int n) {
#ifdef __CUDA_ARCH__
  return __brev(c) >> (32 - n);
#else
  uint32_t r = 0;
  for (int i = 0; i < n; i++) r |= ((c >> i) & 1u) << (n - 1 - i);
  return r;
#endif
}

/* length 3..258 -> literal/length symbol 257..285 and its extra bits (RFC 1951 3.2.5) */
PNG_HD void len_code(int L, int &sym, int &next, int &extra) {
  if (L == 258) {
    sym = 285, next = 0, extra = 0;
    return;
  }
  const int m = L - 3;
  if (m < 8) {
    sym = 257 + m, next = 0, extra = 0;
    return;
  }
  const int n = ilog2((uint32_t)m);
  sym = 257 + 4 * (n - 1) + ((m >> (n - 2)) & 3);
  next = n - 2;
  extra = m & ((1 << (n - 2)) - 1);
}

/* distance 1..32768 -> distance symbol 0..29 and its extra bits */
PNG_HD void dist_code(int d, int &sym, int &next, int &extra) {
  const int m = d - 1;
  if (m < 2) {
    sym = m, next = 0, extra = 0;
    return;
  }
  const int n = ilog2((uint32_t)m);
  sym = 2 * n + ((m >> (n - 1)) & 1);
  next = n - 1;
  extra = m & ((1 << (n - 1)) - 1);
}

/* Greedy parse of F[beg, end): at each position the longest run equal to
 * the bytes at one of the candidate distances (no match reaches past end),
 * a match when it is at least MIN_MATCH long, else a literal. */
template <class Sink>
PNG_HD void parse(const uint8_t *F, long long beg, long long end, const int *dist, int nd, Sink &s) {
  long long p = beg;
  while (p < end) {
    const int maxlen = (int)((end - p) < MAX_MATCH ? (end - p) : MAX_MATCH);
    int bl = 0, bd = 0;
    const uint8_t x0 = F[p];
    for (int k = 0; k < nd; k++) {
      const int d = dist[k];
      if ((long long)d > p) continue;
      const uint8_t *a = F + p, *b = F + p - d;
      if (b[0] != x0) continue;
      int L = 1;
      while (L < maxlen && a[L] == b[L]) L++;
      if (L > bl) bl = L, bd = d;
    }
    if (bl >= MIN_MATCH) {
      s.match(bl, bd);
      p += bl;
    } else {
      s.literal(x0);
      p++;
    }
  }
}

/* ---- shared state of one segment's CTA ---- */

struct HuffScratch {
  uint16_t sorted[NLIT]; /* used symbols, ascending frequency */
  uint32_t wi[NLIT];     /* internal node weights */
  uint16_t par_leaf[NLIT], par_int[NLIT];
  uint8_t depth[NLIT];
  int nused;
};

struct SegShared {
  uint32_t out[OUT_BYTES / 4];
  uint32_t hist_lit[NLIT], hist_dist[NDIST], hist_cl[NCL];
  uint16_t code_lit[NLIT], code_dist[NDIST], code_cl[NCL]; /* bit-reversed */
  uint8_t len_lit[NLIT], len_dist[NDIST], len_cl[NCL];
  uint8_t cl_sym[NLIT + NDIST], cl_extra[NLIT + NDIST];
  HuffScratch hs[2];
  uint32_t crc_table[256];
  uint32_t tbits[NT];           /* per-thread token bits, then their offsets */
  uint32_t crc_part[NT];
  uint32_t crc_x[8];            /* x^(8 q 2^l) mod the CRC polynomial */
  uint32_t a1[NT], a2[NT], alen[NT]; /* Adler-32 partial sums per thread */
  int ncl, hlit, hdist, hclen;
  uint32_t hdr_bits, body_bits, nbytes, mode;
  int dist[MAXD], nd;
};

/* ---- sinks of the parse ---- */

struct HistSink {
  SegShared *S;
  PNG_HD void literal(uint8_t v) { atomic_add_u32(&S->hist_lit[v], 1); }
  PNG_HD void match(int L, int d) {
    int s, n, e;
    len_code(L, s, n, e);
    atomic_add_u32(&S->hist_lit[s], 1);
    dist_code(d, s, n, e);
    atomic_add_u32(&S->hist_dist[s], 1);
  }
};

struct CountSink {
  const SegShared *S;
  uint32_t bits;
  PNG_HD void literal(uint8_t v) { bits += S->len_lit[v]; }
  PNG_HD void match(int L, int d) {
    int s, n, e;
    len_code(L, s, n, e);
    bits += S->len_lit[s] + n;
    dist_code(d, s, n, e);
    bits += S->len_dist[s] + n;
  }
};

/* LSB-first bit writer into the zeroed shared output; words at the edges of
 * a thread's range are shared with its neighbours, hence the OR. */
struct BitWriter {
  uint32_t *buf;
  unsigned long long acc;
  int nacc;
  uint32_t word;
  PNG_HD void start(uint32_t *b, uint32_t bitpos) {
    buf = b;
    word = bitpos >> 5;
    nacc = (int)(bitpos & 31);
    acc = 0;
  }
  PNG_HD void put(uint32_t v, int n) {
    acc |= (unsigned long long)v << nacc;
    nacc += n;
    while (nacc >= 32) {
      atomic_or_u32(&buf[word++], (uint32_t)acc);
      acc >>= 32;
      nacc -= 32;
    }
  }
  PNG_HD void flush() {
    if (nacc > 0) atomic_or_u32(&buf[word], (uint32_t)acc);
    nacc = 0;
    acc = 0;
  }
};

struct EmitSink {
  const SegShared *S;
  BitWriter w;
  PNG_HD void literal(uint8_t v) { w.put(S->code_lit[v], S->len_lit[v]); }
  PNG_HD void match(int L, int d) {
    int s, n, e;
    len_code(L, s, n, e);
    w.put(S->code_lit[s], S->len_lit[s]);
    if (n) w.put((uint32_t)e, n);
    dist_code(d, s, n, e);
    w.put(S->code_dist[s], S->len_dist[s]);
    if (n) w.put((uint32_t)e, n);
  }
};

/* ---- Huffman code lengths ---- */

/* rank of symbol `sym` among the used symbols by (frequency, symbol); run
 * by every thread for its symbols, fills h.sorted */
PNG_HD void rank_symbols(const uint32_t *freq, int n, HuffScratch &h, int tid, int nthreads) {
  for (int s = tid; s < n; s += nthreads) {
    const uint32_t f = freq[s];
    if (!f) continue;
    int r = 0;
    for (int j = 0; j < n; j++) {
      const uint32_t g = freq[j];
      r += (g && (g < f || (g == f && j < s))) ? 1 : 0;
    }
    h.sorted[r] = (uint16_t)s;
  }
}

PNG_HD int count_used(const uint32_t *freq, int n) {
  int m = 0;
  for (int s = 0; s < n; s++) m += freq[s] ? 1 : 0;
  return m;
}

/* Huffman code lengths limited to maxbits, forming a complete code (Kraft
 * sum exactly 1) whenever at least two symbols are used; one used symbol
 * gets length 1.  h.sorted must hold the used symbols in ascending
 * frequency.  One thread. */
PNG_HD void huff_lengths(const uint32_t *freq, int n, int maxbits, HuffScratch &h, uint8_t *len) {
  for (int s = 0; s < n; s++) len[s] = 0;
  const int m = count_used(freq, n);
  h.nused = m;
  if (m == 0) return;
  if (m == 1) {
    len[h.sorted[0]] = 1;
    return;
  }
  /* two-queue construction: leaves in ascending order, internal nodes are
   * created in ascending order too */
  int i = 0, j = 0;
  for (int t = 0; t < m - 1; t++) {
    uint32_t w = 0;
    for (int pick = 0; pick < 2; pick++) {
      if (i < m && (j >= t || freq[h.sorted[i]] <= h.wi[j])) {
        w += freq[h.sorted[i]];
        h.par_leaf[i++] = (uint16_t)t;
      } else {
        w += h.wi[j];
        h.par_int[j++] = (uint16_t)t;
      }
    }
    h.wi[t] = w;
  }
  /* depths: the root is the last internal node */
  uint8_t *dint = h.depth; /* internal node depths, reused */
  dint[m - 2] = 0;
  for (int t = m - 3; t >= 0; t--) dint[t] = (uint8_t)(dint[h.par_int[t]] + 1 < 255 ? dint[h.par_int[t]] + 1 : 255);
  int bl[33];
  for (int b = 0; b <= 32; b++) bl[b] = 0;
  for (int k = 0; k < m; k++) {
    int d = dint[h.par_leaf[k]] + 1;
    if (d > maxbits) d = maxbits;
    bl[d]++;
  }
  /* Kraft sum in units of 2^-maxbits; lengthen codes while it is over one,
   * then shorten the deepest ones while it is under */
  const long long full = 1ll << maxbits;
  long long K = 0;
  for (int b = 1; b <= maxbits; b++) K += (long long)bl[b] << (maxbits - b);
  while (K > full) {
    int b = maxbits - 1;
    while (b > 0 && bl[b] == 0) b--;
    bl[b]--;
    bl[b + 1]++;
    K -= 1ll << (maxbits - b - 1);
  }
  while (K < full) {
    int b = maxbits;
    while (b > 1 && (bl[b] == 0 || (1ll << (maxbits - b)) > full - K)) b--;
    if (b <= 1) break; /* cannot happen: see the multiple-of argument */
    bl[b]--;
    bl[b - 1]++;
    K += 1ll << (maxbits - b);
  }
  /* the least frequent symbols take the longest codes */
  int k = 0;
  for (int b = maxbits; b >= 1; b--)
    for (int c = 0; c < bl[b]; c++) len[h.sorted[k++]] = (uint8_t)b;
}

/* canonical codes (RFC 1951 3.2.2), stored bit-reversed for LSB-first output */
PNG_HD void canonical_codes(const uint8_t *len, int n, uint16_t *code, int tid, int nthreads) {
  for (int s = tid; s < n; s += nthreads) {
    const int L = len[s];
    if (!L) {
      code[s] = 0;
      continue;
    }
    /* first code of length L: codes of all shorter lengths, doubled per step */
    uint32_t c = 0;
    for (int b = 1; b < L; b++) {
      int cnt = 0;
      for (int j = 0; j < n; j++) cnt += len[j] == b ? 1 : 0;
      c = (c + cnt) << 1;
    }
    for (int j = 0; j < s; j++) c += len[j] == L ? 1 : 0;
    code[s] = (uint16_t)rev_bits(c, L);
  }
}

/* ---- CRC-32 (PNG / ISO 3309, reflected) ---- */

PNG_HD uint32_t gf2_mult(uint32_t a, uint32_t b) {
  uint32_t p = 0;
  for (int i = 0; i < 32; i++) {
    if (a & (0x80000000u >> i)) p ^= b;
    b = (b & 1u) ? (b >> 1) ^ CRC_POLY : b >> 1;
  }
  return p;
}

/* x^e modulo the CRC polynomial, reflected */
PNG_HD uint32_t gf2_xpow(unsigned long long e) {
  uint32_t r = 0x80000000u, base = 0x40000000u;
  while (e) {
    if (e & 1) r = gf2_mult(r, base);
    base = gf2_mult(base, base);
    e >>= 1;
  }
  return r;
}

/* transmission order of the code-length code lengths (RFC 1951 3.2.7) */
PNG_HD int cl_order(int k) {
  const uint8_t o[NCL] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
  return o[k];
}

/* ---- phases of one segment ---- */

struct SegArgs {
  const uint8_t *F;
  long long total;    /* bytes of the filtered stream */
  int bpp, stride;    /* bytes per pixel, bytes per filtered row */
  int nseg;
  uint8_t *stage;     /* nseg x STAGE bytes */
  SegMeta *meta;
};

PNG_HD void seg_range(const SegArgs &A, int seg, long long &b, long long &e) {
  b = (long long)seg * SEG;
  e = b + SEG < A.total ? b + SEG : A.total;
}

PNG_HD void sub_range(const SegArgs &A, int seg, int tid, long long &b, long long &e) {
  long long sb, se;
  seg_range(A, seg, sb, se);
  b = sb + (long long)tid * SUB;
  e = b + SUB;
  if (b > se) b = se;
  if (e > se) e = se;
}

/* phase 0: clear, CRC table, candidate distances */
PNG_HD void phase_init(SegShared &S, const SegArgs &A, int tid) {
  for (int i = tid; i < OUT_BYTES / 4; i += NT) S.out[i] = 0;
  for (int i = tid; i < NLIT; i += NT) S.hist_lit[i] = 0;
  for (int i = tid; i < NDIST; i += NT) S.hist_dist[i] = 0;
  for (int i = tid; i < NCL; i += NT) S.hist_cl[i] = 0;
  for (int i = tid; i < 256; i += NT) {
    uint32_t c = (uint32_t)i;
    for (int k = 0; k < 8; k++) c = (c & 1u) ? (c >> 1) ^ CRC_POLY : c >> 1;
    S.crc_table[i] = c;
  }
  if (tid == 0) {
    int nd = 0;
    const int cand[MAXD] = {1, A.bpp, A.stride, 2 * A.bpp};
    for (int k = 0; k < MAXD; k++) {
      const int d = cand[k];
      bool dup = d < 1 || d > WINDOW;
      for (int q = 0; q < nd; q++) dup = dup || S.dist[q] == d;
      if (!dup) S.dist[nd++] = d;
    }
    S.nd = nd;
  }
}

/* phase 1: symbol histogram and Adler-32 partial sums */
PNG_HD void phase_hist(SegShared &S, const SegArgs &A, int seg, int tid) {
  long long b, e;
  sub_range(A, seg, tid, b, e);
  HistSink hsink{&S};
  parse(A.F, b, e, S.dist, S.nd, hsink);
  unsigned long long s1 = 0, s2 = 0;
  for (long long p = b; p < e; p++) {
    s1 += A.F[p];
    s2 += (unsigned long long)(e - p) * A.F[p];
  }
  S.a1[tid] = (uint32_t)s1;
  S.a2[tid] = (uint32_t)s2;
  S.alen[tid] = (uint32_t)(e - b);
  if (tid == 0) atomic_add_u32(&S.hist_lit[256], 1); /* end of block */
}

/* phase 2: order the used symbols of both alphabets */
PNG_HD void phase_rank(SegShared &S, int tid) {
  rank_symbols(S.hist_lit, NLIT, S.hs[0], tid, NT);
  rank_symbols(S.hist_dist, NDIST, S.hs[1], tid, NT);
}

/* phase 3: code lengths (thread 0: literal/length, thread 32: distance) */
PNG_HD void phase_lengths(SegShared &S, int tid) {
  if (tid == 0) huff_lengths(S.hist_lit, NLIT, 15, S.hs[0], S.len_lit);
  if (tid == 32) {
    huff_lengths(S.hist_dist, NDIST, 15, S.hs[1], S.len_dist);
    /* no matches: one distance code of one bit (RFC 1951 3.2.7) */
    if (S.hs[1].nused == 0) S.len_dist[0] = 1;
  }
}

/* phase 4: canonical codes of both alphabets */
PNG_HD void phase_codes(SegShared &S, int tid) {
  canonical_codes(S.len_lit, NLIT, S.code_lit, tid, NT);
  canonical_codes(S.len_dist, NDIST, S.code_dist, tid, NT);
}

/* phase 5 (thread 0): run-length coded code lengths, the code-length code
 * and the header size */
PNG_HD void phase_header(SegShared &S, int tid) {
  if (tid != 0) return;
  int hlit = NLIT;
  while (hlit > 257 && S.len_lit[hlit - 1] == 0) hlit--;
  int hdist = NDIST;
  while (hdist > 1 && S.len_dist[hdist - 1] == 0) hdist--;
  S.hlit = hlit;
  S.hdist = hdist;
  const int total = hlit + hdist;
  auto L = [&](int i) -> int { return i < hlit ? S.len_lit[i] : S.len_dist[i - hlit]; };
  int ncl = 0;
  int i = 0;
  while (i < total) {
    const int v = L(i);
    int run = 1;
    while (i + run < total && L(i + run) == v) run++;
    if (v == 0) {
      int r = run;
      while (r >= 11) {
        const int c = r < 138 ? r : 138;
        S.cl_sym[ncl] = 18, S.cl_extra[ncl++] = (uint8_t)(c - 11);
        r -= c;
      }
      if (r >= 3) {
        S.cl_sym[ncl] = 17, S.cl_extra[ncl++] = (uint8_t)(r - 3);
        r = 0;
      }
      while (r > 0) S.cl_sym[ncl] = 0, S.cl_extra[ncl++] = 0, r--;
    } else {
      S.cl_sym[ncl] = (uint8_t)v, S.cl_extra[ncl++] = 0;
      int r = run - 1;
      while (r >= 3) {
        const int c = r < 6 ? r : 6;
        S.cl_sym[ncl] = 16, S.cl_extra[ncl++] = (uint8_t)(c - 3);
        r -= c;
      }
      while (r > 0) S.cl_sym[ncl] = (uint8_t)v, S.cl_extra[ncl++] = 0, r--;
    }
    i += run;
  }
  S.ncl = ncl;
  for (int k = 0; k < ncl; k++) S.hist_cl[S.cl_sym[k]]++;
  /* a code-length code must be complete: give a lone symbol a partner */
  int used = count_used(S.hist_cl, NCL);
  uint32_t f2[NCL];
  for (int k = 0; k < NCL; k++) f2[k] = S.hist_cl[k];
  if (used < 2)
    for (int k = 0; k < NCL && used < 2; k++)
      if (!f2[k]) f2[k] = 1, used++;
  /* 19 symbols: an insertion sort is enough */
  HuffScratch &h = S.hs[1];
  int m = 0;
  for (int k = 0; k < NCL; k++) {
    if (!f2[k]) continue;
    int q = m++;
    while (q > 0 && (f2[h.sorted[q - 1]] > f2[k])) {
      h.sorted[q] = h.sorted[q - 1];
      q--;
    }
    h.sorted[q] = (uint16_t)k;
  }
  huff_lengths(f2, NCL, 7, h, S.len_cl);
  canonical_codes(S.len_cl, NCL, S.code_cl, 0, 1);
  int hclen = NCL;
  while (hclen > 4 && S.len_cl[cl_order(hclen - 1)] == 0) hclen--;
  S.hclen = hclen;
  uint32_t bits = 3 + 5 + 5 + 4 + 3 * hclen;
  for (int k = 0; k < ncl; k++) {
    const int s = S.cl_sym[k];
    bits += S.len_cl[s] + (s == 16 ? 2 : s == 17 ? 3 : s == 18 ? 7 : 0);
  }
  S.hdr_bits = bits;
}

/* phase 6: bits of each thread's tokens */
PNG_HD void phase_count(SegShared &S, const SegArgs &A, int seg, int tid) {
  long long b, e;
  sub_range(A, seg, tid, b, e);
  CountSink cs{&S, 0};
  parse(A.F, b, e, S.dist, S.nd, cs);
  S.tbits[tid] = cs.bits;
}

/* phase 7 (thread 0): offsets of the threads' tokens, the block's size and
 * the choice between the Huffman block and a stored block */
PNG_HD void phase_layout(SegShared &S, const SegArgs &A, int seg, int tid) {
  if (tid != 0) return;
  uint32_t off = S.hdr_bits;
  for (int t = 0; t < NT; t++) {
    const uint32_t c = S.tbits[t];
    S.tbits[t] = off;
    off += c;
  }
  const uint32_t eob = off;
  const uint32_t end_bits = eob + S.len_lit[256];
  const bool last = seg == A.nseg - 1;
  /* a non-final segment ends with an empty stored block on a byte boundary */
  const uint32_t dyn_bytes = last ? (end_bits + 7) / 8 : (end_bits + 3 + 7) / 8 + 4;
  long long sb, se;
  seg_range(A, seg, sb, se);
  const uint32_t stored_bytes = (uint32_t)(se - sb) + 5;
  S.body_bits = eob;
  if (dyn_bytes < stored_bytes) {
    S.mode = 2;
    S.nbytes = dyn_bytes;
  } else {
    S.mode = 0;
    S.nbytes = stored_bytes;
  }
}

/* phase 8: the block itself */
PNG_HD void phase_emit(SegShared &S, const SegArgs &A, int seg, int tid) {
  const bool last = seg == A.nseg - 1;
  long long sb, se;
  seg_range(A, seg, sb, se);
  if (S.mode == 0) {
    uint8_t *o = (uint8_t *)S.out;
    const uint32_t n = (uint32_t)(se - sb);
    if (tid == 0) {
      o[0] = last ? 1 : 0; /* BFINAL, BTYPE 00, then byte aligned */
      o[1] = (uint8_t)(n & 255), o[2] = (uint8_t)(n >> 8);
      o[3] = (uint8_t)(~n & 255), o[4] = (uint8_t)((~n >> 8) & 255);
    }
    /* bytes 5.. by whole words where each thread owns them */
    for (uint32_t i = (uint32_t)tid; i < n; i += NT) {
      const uint32_t pos = 5 + i;
      atomic_or_u32(&S.out[pos >> 2], (uint32_t)A.F[sb + i] << (8 * (pos & 3)));
    }
    return;
  }
  if (tid == 0) {
    BitWriter w;
    w.start(S.out, 0);
    w.put(last ? 1u : 0u, 1);
    w.put(2u, 2);
    w.put((uint32_t)(S.hlit - 257), 5);
    w.put((uint32_t)(S.hdist - 1), 5);
    w.put((uint32_t)(S.hclen - 4), 4);
    for (int k = 0; k < S.hclen; k++) w.put(S.len_cl[cl_order(k)], 3);
    for (int k = 0; k < S.ncl; k++) {
      const int s = S.cl_sym[k];
      w.put(S.code_cl[s], S.len_cl[s]);
      if (s == 16) w.put(S.cl_extra[k], 2);
      else if (s == 17) w.put(S.cl_extra[k], 3);
      else if (s == 18) w.put(S.cl_extra[k], 7);
    }
    w.flush();
    /* end of block, then the byte-aligning empty stored block */
    w.start(S.out, S.body_bits);
    w.put(S.code_lit[256], S.len_lit[256]);
    if (!last) {
      w.put(0u, 3);
      w.flush();
      const uint32_t bytepos = (S.body_bits + S.len_lit[256] + 3 + 7) / 8;
      atomic_or_u32(&S.out[(bytepos + 2) >> 2], 0xFFu << (8 * ((bytepos + 2) & 3)));
      atomic_or_u32(&S.out[(bytepos + 3) >> 2], 0xFFu << (8 * ((bytepos + 3) & 3)));
    } else {
      w.flush();
    }
  }
  long long b, e;
  sub_range(A, seg, tid, b, e);
  EmitSink es{&S, {}};
  es.w.start(S.out, S.tbits[tid]);
  parse(A.F, b, e, S.dist, S.nd, es);
  es.w.flush();
}

/* phase 9: per-thread CRC of an equal share of the virtual stream
 * [zeros | "IDAT" | data] padded at the front to NT equal parts (leading
 * zeros leave a zero CRC register unchanged) */
PNG_HD void phase_crc_parts(SegShared &S, int tid, uint32_t &q) {
  const uint32_t n = 4 + S.nbytes;
  q = (n + NT - 1) / NT;
  const uint32_t pad = q * NT - n;
  const uint8_t *o = (const uint8_t *)S.out;
  uint32_t c = 0;
  for (uint32_t v = (uint32_t)tid * q; v < (uint32_t)(tid + 1) * q; v++) {
    uint8_t x;
    if (v < pad) continue;
    const uint32_t u = v - pad;
    x = u < 4 ? (uint8_t)("IDAT"[u]) : o[u - 4];
    c = S.crc_table[(c ^ x) & 255u] ^ (c >> 8);
  }
  S.crc_part[tid] = c;
}

/* tree combine of the parts, level `lvl` (run for lvl = 0..7 with a barrier
 * after each): the right neighbour's part is q * 2^lvl bytes long */
PNG_HD void phase_crc_level(SegShared &S, int tid, int lvl, uint32_t xp) {
  const int step = 1 << lvl;
  if ((tid & (2 * step - 1)) == 0) S.crc_part[tid] = gf2_mult(S.crc_part[tid], xp) ^ S.crc_part[tid + step];
}

/* phase 10: the segment's bytes to its staging slot; thread 0 writes the
 * metadata (CRC with the initial register folded in, Adler sums) */
PNG_HD void phase_store(SegShared &S, const SegArgs &A, int seg, int tid) {
  uint32_t *dst = (uint32_t *)(A.stage + (size_t)seg * STAGE);
  const uint32_t nw = (S.nbytes + 3) / 4;
  for (uint32_t i = (uint32_t)tid; i < nw; i += NT) dst[i] = S.out[i];
  if (tid == 0) {
    const uint32_t n = 4 + S.nbytes;
    const uint32_t crc = gf2_mult(0xFFFFFFFFu, gf2_xpow(8ull * n)) ^ S.crc_part[0] ^ 0xFFFFFFFFu;
    unsigned long long s1 = 0, s2 = 0, after = 0;
    for (int t = NT - 1; t >= 0; t--) {
      s1 += S.a1[t];
      s2 += S.a2[t] + (unsigned long long)S.a1[t] * after;
      after += S.alen[t];
      s2 %= ADLER_MOD;
    }
    SegMeta m;
    m.nbytes = S.nbytes;
    m.crc = crc;
    m.s1 = (uint32_t)(s1 % ADLER_MOD);
    m.s2 = (uint32_t)(s2 % ADLER_MOD);
    m.len = (uint32_t)after;
    m.mode = S.mode;
    m.pad[0] = m.pad[1] = 0;
    A.meta[seg] = m;
  }
}

/* ---- row filters (PNG filter types 0-4) ---- */

PNG_HD int paeth(int a, int b, int c) {
  const int p = a + b - c;
  const int pa = p > a ? p - a : a - p, pb = p > b ? p - b : b - p, pc = p > c ? p - c : c - p;
  if (pa <= pb && pa <= pc) return a;
  if (pb <= pc) return b;
  return c;
}

/* filtered byte k (0 none, 1 sub, 2 up, 3 average, 4 paeth) */
PNG_HD int filter_byte(int k, int x, int a, int b, int c) {
  switch (k) {
    case 0: return x;
    case 1: return (x - a) & 255;
    case 2: return (x - b) & 255;
    case 3: return (x - ((a + b) >> 1)) & 255;
    default: return (x - paeth(a, b, c)) & 255;
  }
}

PNG_HD int filter_cost(int v) { return v < 128 ? v : 256 - v; }

} /* namespace f3gpng */
