/*
 * f3g_png.cuh -- PNG encoding of a rendered image on the device: the
 * reference hands the packed RGBA image to libpng (png.c:36-116, write_png),
 * which filters each row (PNG filter types 0-4, chosen per row by the
 * minimum-sum-of-absolute-values rule) and deflates the filtered rows into
 * one zlib stream split over IDAT chunks.
 *
 * Here the filtered stream (h rows of 1 + w*bpp bytes) is cut into
 * segments of SEG (16 KB) bytes and each segment is deflated by one CTA on
 * its own.  The segment and the LOOKBACK bytes before it are staged in
 * shared memory; each thread parses SUB bytes greedily against fixed
 * distances that suit images (neighbouring pixels, the row above and its
 * diagonals, two rows) and a table of the latest 4-byte occurrences in the
 * look-back; the segment becomes one dynamic-Huffman block (a stored block
 * where that is smaller), ended on a byte boundary by an empty stored block,
 * so every segment is one IDAT chunk whose CRC the CTA computes itself.
 * Back-references may reach into earlier segments (the decoder holds all of
 * the stream), so cutting costs only the few bytes of each block header.
 * The zlib header and the Adler-32 trailer are two small IDAT chunks of
 * their own.
 *
 * Format constants follow RFC 1950 (zlib), RFC 1951 (deflate) and the PNG
 * specification (chunk layout, CRC-32 polynomial, filter types).
 *
 * The phase functions are plain __host__ __device__ code over one CTA's
 * shared state; the kernel runs them with a barrier between phases.
 */
#pragma once
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define PNG_HD __host__ __device__ __forceinline__
#else
#define PNG_HD inline
#endif

namespace f3gpng {

constexpr int SEG = 16384;          /* filtered bytes per segment (one CTA) */
constexpr int NT = 256;             /* threads per CTA */
constexpr int LOG_NT = 8;
constexpr int SUB = SEG / NT;       /* bytes parsed by one thread */
constexpr int MIN_MATCH = 4;        /* shortest match emitted (3 is legal) */
constexpr int OVERRUN = 64;         /* how far a thread's last match may run past its share */
constexpr int MAX_MATCH = 258;
constexpr int WINDOW = 32768;       /* deflate's largest distance */
constexpr int LOOKBACK = 16384;     /* bytes before a segment that its matches may reach */
constexpr int NLIT = 286, NDIST = 30, NCL = 19;
constexpr int MAXD = 9;             /* fixed candidate distances */
constexpr int WT_BITS = 11;         /* window table: 4-byte hash -> latest position */
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

PNG_HD void atomic_max_u32(uint32_t *p, uint32_t v) {
#ifdef __CUDA_ARCH__
  atomicMax(p, v);
#else
  if (v > *p) *p = v;
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

/* multiplicative hash of the 4 bytes at p (Knuth's golden-ratio constant) */
PNG_HD uint32_t hash4(const uint8_t *p) {
  const uint32_t v = (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
  return (v * 2654435761u) >> (32 - WT_BITS);
}

/* where a parse looks for matches: fixed distances (neighbouring pixels and
 * rows) and the latest earlier occurrence of the next 4 bytes in the 32 KB
 * before the segment (wtab[h] = position - wbase + 1, 0 = none) */
struct Cands {
  const int *dist;
  int nd;
  const uint32_t *wtab;
  long long wbase, total;
};

/* the 4 bytes at w[pos] as a little-endian word (w 4-byte aligned; may read
 * up to 3 bytes past the valid data, which the caller masks by length) */
PNG_HD uint32_t load32u(const uint8_t *w, int pos) {
#ifdef __CUDA_ARCH__
  const uint32_t *q = reinterpret_cast<const uint32_t *>(w);
  return __funnelshift_r(q[pos >> 2], q[(pos >> 2) + 1], (pos & 3) * 8);
#else
  uint32_t v;
  memcpy(&v, w + pos, 4);
  return v;
#endif
}

PNG_HD int ctz32(uint32_t x) {
#ifdef __CUDA_ARCH__
  return __ffs((int)x) - 1;
#else
  return __builtin_ctz(x);
#endif
}

/* bytes equal at a and a - d, up to maxlen, compared a word at a time */
PNG_HD int match_len(const uint8_t *F, int a, int d, int maxlen) {
  int L = 0;
  while (L < maxlen) {
    const uint32_t x = load32u(F, a + L) ^ load32u(F, a - d + L);
    if (x) {
      L += ctz32(x) >> 3;
      break;
    }
    L += 4;
  }
  return L < maxlen ? L : maxlen;
}

/* longest match at p among the candidates, not reaching past end; the
 * search stops at the first match of the greatest possible length.  Only
 * candidates whose first 4 bytes match can reach MIN_MATCH, so one word
 * compare screens each candidate. */
PNG_HD int best_match(const uint8_t *F, long long p, long long end, const Cands &C, int &bd) {
  const int maxlen = (int)((end - p) < MAX_MATCH ? (end - p) : MAX_MATCH);
  int bl = 0;
  bd = 0;
  if (maxlen < MIN_MATCH) return 0;
  const int ip = (int)p;
  const uint32_t w = load32u(F, ip);
  for (int k = 0; k < C.nd && bl < maxlen; k++) {
    const int d = C.dist[k];
    if (d > ip || load32u(F, ip - d) != w) continue;
    const int L = 4 + match_len(F, ip + 4, d, maxlen - 4);
    if (L > bl) bl = L, bd = d;
  }
  if (bl < maxlen && p + 4 <= C.total) {
    const uint32_t v = C.wtab[hash4(F + ip)];
    if (v) {
      const long long d = p - (C.wbase + (long long)v - 1);
      if (d >= 1 && d <= WINDOW && load32u(F, ip - (int)d) == w) {
        const int L = 4 + match_len(F, ip + 4, (int)d, maxlen - 4);
        if (L > bl) bl = L, bd = (int)d;
      }
    }
  }
  return bl;
}

/* Greedy parse from beg while the position is before end: the longest
 * candidate match at each position (it may run on up to `limit`, past end)
 * when it is at least MIN_MATCH long, else a literal.  Returns the position
 * after the last token.  (One step of lazy evaluation, as zlib does, gains
 * under 1 % on rendered images for twice the search.) */
template <class Sink>
PNG_HD long long parse(const uint8_t *F, long long beg, long long end, long long limit, const Cands &C, Sink &s) {
  long long p = beg;
  while (p < end) {
    int bd;
    const int bl = best_match(F, p, limit, C, bd);
    if (bl >= MIN_MATCH) {
      s.match(bl, bd);
      p += bl;
    } else {
      s.literal(F[p]);
      p++;
    }
  }
  return p;
}

/* ---- shared state of one segment's CTA ---- */

template <int N>
struct HuffScratchT {
  uint16_t sorted[N]; /* used symbols, ascending frequency */
  uint32_t wl[N];     /* their frequencies, in that order */
  uint32_t wi[N];     /* internal node weights */
  uint16_t par_leaf[N], par_int[N];
  uint8_t depth[N];
  uint32_t first[16]; /* first canonical code of each length */
  uint32_t nused;
};
using HuffScratch = HuffScratchT<NLIT>;
using HuffScratchSmall = HuffScratchT<32>; /* distances (30), code lengths (19) */

struct SegShared {
  alignas(16) uint8_t win[LOOKBACK + SEG]; /* F[w0, se): the segment and the bytes before it */
  union {
    uint32_t out[OUT_BYTES / 4];
    unsigned long long keys[1024]; /* symbol sort keys, before the output exists */
  };
  uint32_t hist_lit[NLIT], hist_dist[NDIST], hist_cl[NCL];
  uint16_t code_lit[NLIT], code_dist[NDIST], code_cl[NCL]; /* bit-reversed */
  uint8_t len_lit[NLIT], len_dist[NDIST], len_cl[NCL];
  uint8_t cl_sym[NLIT + NDIST], cl_extra[NLIT + NDIST];
  HuffScratch hs0;      /* literal/length alphabet */
  HuffScratchSmall hs1; /* distance alphabet, then the code-length code */
  uint32_t crc_table[256];
  union {
    uint32_t tbits[NT];         /* per-thread token bits, then their offsets */
    uint32_t crc_part[NT];      /* per-thread CRC registers, after the block is out */
  };
  int ntok[NT];                 /* per-thread token entries */
  int tend[NT];                 /* where each thread's last token ends (relative to w0) */
  uint16_t tstart[NT], tfrom[NT]; /* a thread's first byte, its first uncovered byte */
  uint32_t crc_x[8];            /* x^(8 q 2^l) mod the CRC polynomial */
  uint32_t crc_xn;              /* x^(8 n), n = 4 + the segment's bytes */
  uint32_t a1[NT], a2[NT], alen[NT]; /* Adler-32 partial sums per thread */
  int ncl, hlit, hdist, hclen;
  uint32_t lit_end, dist_end;   /* one past the last nonzero length */
  uint32_t dist_first, dist_last; /* the distance keys' range after the sort */
  uint32_t hdr_bits, body_bits, nbytes, mode;
  int dist[MAXD], nd;
  uint32_t wtab[1 << WT_BITS];
  long long w0;                 /* stream position of win[0] */
  int wlen;                     /* bytes staged in win */
  /* the parse works in positions relative to w0 */
  PNG_HD Cands cands() const { return Cands{dist, nd, wtab, 0, wlen}; }
};

/* ---- sinks of the parse ---- */

/* records a thread's tokens */
struct TokSink {
  uint16_t *tok;
  int n;
  PNG_HD void literal(uint8_t v) { tok[(size_t)(n++) * NT] = v; }
  PNG_HD void match(int L, int d) {
    tok[(size_t)(n++) * NT] = (uint16_t)(256 + L - 3);
    tok[(size_t)(n++) * NT] = (uint16_t)(d - 1);
  }
};

/* adds (or, with inc = 0xFFFFFFFF, removes) tokens' symbols in the histograms */
struct HistSink {
  SegShared *S;
  uint32_t inc;
  PNG_HD void literal(uint8_t v) { atomic_add_u32(&S->hist_lit[v], inc); }
  PNG_HD void match(int L, int d) {
    int s, nx, e;
    len_code(L, s, nx, e);
    atomic_add_u32(&S->hist_lit[s], inc);
    dist_code(d, s, nx, e);
    atomic_add_u32(&S->hist_dist[s], inc);
  }
};

/* records a thread's tokens and counts their symbols */
struct ParseSink {
  TokSink t;
  HistSink h;
  PNG_HD void literal(uint8_t v) { t.literal(v), h.literal(v); }
  PNG_HD void match(int L, int d) { t.match(L, d), h.match(L, d); }
};

/* A thread's final match may run past its share; the bytes it covers are
 * dropped from the following threads' tokens: tokens that end at or before
 * `from` are skipped, a match that straddles it keeps its tail (the same
 * distance still matches there) or, when that is under 3 bytes, turns into
 * literals. */
template <class Sink>
struct TrimSink {
  Sink &inner;
  const uint8_t *F;
  long long pos, from;
  PNG_HD void literal(uint8_t v) {
    if (pos >= from) inner.literal(v);
    pos++;
  }
  PNG_HD void match(int L, int d) {
    const long long e = pos + L;
    if (pos >= from) {
      inner.match(L, d);
    } else if (e > from) {
      const int k = (int)(e - from);
      if (k >= 3) {
        inner.match(k, d);
      } else {
        for (long long q = from; q < e; q++) inner.literal(F[q]);
      }
    }
    pos = e;
  }
};

/* replays a thread's tokens into a sink */
template <class Sink>
PNG_HD void replay(const uint16_t *tok, int n, Sink &s) {
  constexpr int B = 8; /* entries loaded ahead, independent loads */
  int i = 0;
  while (i < n) {
    uint16_t t[B];
    const int m = n - i < B ? n - i : B;
#pragma unroll
    for (int k = 0; k < B; k++) t[k] = k < m ? tok[(size_t)(i + k) * NT] : 0;
    int j = 0;
#pragma unroll
    for (int k = 0; k < B; k++) {
      if (k != j || j >= m) continue;
      const int v = t[k];
      if (v < 256) {
        s.literal((uint8_t)v);
        j = k + 1;
      } else {
        const int d = k + 1 < m ? t[k + 1] : tok[(size_t)(i + k + 1) * NT];
        s.match(v - 253, d + 1);
        j = k + 2;
      }
    }
    i += j;
  }
}

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
/* Huffman code lengths limited to maxbits, forming a complete code (Kraft
 * sum exactly 1) whenever at least two symbols are used; one used symbol
 * gets length 1.  h.sorted / h.wl / h.nused hold the used symbols in
 * ascending frequency (phase_rank); len must be zero on entry.  Also
 * leaves the first canonical code of each length in h.first.  One thread. */
template <class H>
PNG_HD void huff_lengths(int maxbits, H &h, uint8_t *len) {
  const int m = (int)h.nused;
  int bl[16];
  for (int b = 0; b < 16; b++) bl[b] = 0;
  if (m == 1) {
    len[h.sorted[0]] = 1;
    bl[1] = 1;
  } else if (m >= 2) {
    /* two-queue construction: leaves in ascending order, internal nodes
     * are created in ascending order too */
    int i = 0, j = 0;
    uint32_t wleaf = h.wl[0];
    for (int t = 0; t < m - 1; t++) {
      uint32_t w = 0;
      for (int pick = 0; pick < 2; pick++) {
        if (i < m && (j >= t || wleaf <= h.wi[j])) {
          w += wleaf;
          h.par_leaf[i++] = (uint16_t)t;
          wleaf = i < m ? h.wl[i] : 0;
        } else {
          w += h.wi[j];
          h.par_int[j++] = (uint16_t)t;
        }
      }
      h.wi[t] = w;
    }
    /* depths: the root is the last internal node */
    uint8_t *dint = h.depth;
    dint[m - 2] = 0;
    for (int t = m - 3; t >= 0; t--) {
      const int d = dint[h.par_int[t]] + 1;
      dint[t] = (uint8_t)(d < 255 ? d : 255);
    }
    for (int k = 0; k < m; k++) {
      int d = dint[h.par_leaf[k]] + 1;
      if (d > maxbits) d = maxbits;
      bl[d]++;
    }
    /* Kraft sum in units of 2^-maxbits; lengthen codes while it is over
     * one, then shorten the deepest ones while it is under */
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
      if (b <= 1) break; /* cannot happen: K and full are multiples of the deepest step */
      bl[b]--;
      bl[b - 1]++;
      K += 1ll << (maxbits - b);
    }
    /* the least frequent symbols take the longest codes */
    int k = 0;
    for (int b = maxbits; b >= 1; b--)
      for (int c = 0; c < bl[b]; c++) len[h.sorted[k++]] = (uint8_t)b;
  }
  uint32_t code = 0;
  h.first[0] = 0;
  for (int b = 1; b < 16; b++) {
    code = (code + (b > 1 ? bl[b - 1] : 0)) << (b > 1 ? 1 : 0);
    h.first[b] = code;
  }
}

/* canonical codes (RFC 1951 3.2.2), stored bit-reversed for LSB-first
 * output: the first code of the symbol's length plus its rank among the
 * earlier symbols of that length */
PNG_HD void canonical_codes(const uint8_t *len, int n, const uint32_t *first, uint16_t *code, int tid,
                            int nthreads) {
  for (int s = tid; s < n; s += nthreads) {
    const int L = len[s];
    uint32_t c = 0;
    for (int j = 0; j < s; j++) c += len[j] == L ? 1u : 0u;
    code[s] = L ? (uint16_t)rev_bits(first[L] + c, L) : 0;
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

/* x^(8 * 2^k) modulo the CRC polynomial (reflected), k = 0..31: the
 * shift of a CRC register over 2^k zero bytes */
struct X8Table {
  uint32_t v[32];
};

constexpr uint32_t cx_mult(uint32_t a, uint32_t b) {
  uint32_t p = 0;
  for (int i = 0; i < 32; i++) {
    if (a & (0x80000000u >> i)) p ^= b;
    b = (b & 1u) ? (b >> 1) ^ CRC_POLY : b >> 1;
  }
  return p;
}

constexpr X8Table make_x8() {
  X8Table t{};
  uint32_t p = 0x00800000u; /* x^8 */
  for (int k = 0; k < 32; k++) {
    t.v[k] = p;
    p = cx_mult(p, p);
  }
  return t;
}

#ifdef __CUDACC__
__constant__ X8Table c_x8 = make_x8();
#endif

#ifdef __CUDACC__
/* x^(8 n) modulo the CRC polynomial over a whole warp (every lane gets the
 * product): lane k holds the factor of bit k, then a butterfly of products */
__device__ __forceinline__ uint32_t xpow8_warp(uint32_t n) {
  const int lane = threadIdx.x & 31;
  uint32_t f = ((n >> lane) & 1u) ? c_x8.v[lane] : 0x80000000u;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) f = gf2_mult(f, __shfl_xor_sync(0xffffffffu, f, o));
  return f;
}
#endif

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
  uint16_t *tokens;   /* nseg x TOK_PER_SEG parse tokens, interleaved over the threads */
};

/* A thread's parse tokens: a literal is one entry (the byte), a match two
 * (256 + length - 3, then distance - 1).  A match takes at least 4 bytes,
 * but the thread's last one may start at its last byte, so a thread records
 * at most SUB + 1 entries.  Entry k of thread t sits at k * NT + t of the
 * segment's area of TOK_PER_SEG entries. */
constexpr int TOK_PER_THREAD = SUB + 2;
constexpr int TOK_PER_SEG = TOK_PER_THREAD * NT;
PNG_HD uint16_t *thread_tokens(const SegArgs &A, int seg, int tid) {
  return A.tokens + (size_t)seg * TOK_PER_SEG + tid;
}

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
PNG_HD void phase_init(SegShared &S, const SegArgs &A, int seg, int tid) {
  for (int i = tid; i < NLIT; i += NT) S.hist_lit[i] = 0, S.len_lit[i] = 0;
  for (int i = tid; i < NDIST; i += NT) S.hist_dist[i] = 0, S.len_dist[i] = 0;
  for (int i = tid; i < NCL; i += NT) S.hist_cl[i] = 0, S.len_cl[i] = 0;
  for (int i = tid; i < 256; i += NT) {
    uint32_t c = (uint32_t)i;
    for (int k = 0; k < 8; k++) c = (c & 1u) ? (c >> 1) ^ CRC_POLY : c >> 1;
    S.crc_table[i] = c;
  }
  for (int i = tid; i < (1 << WT_BITS); i += NT) S.wtab[i] = 0;
  /* stage F[w0, se) (w0 and F are 16-byte aligned: segments start at
   * multiples of SEG) */
  const long long sb = (long long)seg * SEG;
  const long long se = sb + SEG < A.total ? sb + SEG : A.total;
  const long long w0 = sb - LOOKBACK > 0 ? sb - LOOKBACK : 0;
  const int n = (int)(se - w0);
#ifdef __CUDA_ARCH__
  const uint4 *src = reinterpret_cast<const uint4 *>(A.F + w0);
  uint4 *dst = reinterpret_cast<uint4 *>(S.win);
  for (int i = tid; i < n / 16; i += NT) dst[i] = src[i];
  for (int i = (n / 16) * 16 + tid; i < n; i += NT) S.win[i] = A.F[w0 + i];
#else
  if (tid == 0) memcpy(S.win, A.F + w0, (size_t)n);
#endif
  if (tid == 0) {
    S.w0 = w0;
    S.wlen = n;
    S.hs0.nused = S.hs1.nused = 0;
    S.dist_first = S.dist_last = 0;
    S.lit_end = S.dist_end = 0;
    int nd = 0;
    const int cand[MAXD] = {1,          A.bpp,          A.stride, 2 * A.bpp, A.stride - A.bpp,
                            A.stride + A.bpp, 3 * A.bpp, 4 * A.bpp, 2 * A.stride};
    for (int k = 0; k < MAXD; k++) {
      const int d = cand[k];
      bool dup = d < 1 || d > WINDOW;
      for (int q = 0; q < nd; q++) dup = dup || S.dist[q] == d;
      if (!dup) S.dist[nd++] = d;
    }
    S.nd = nd;
  }
}

/* phase 0b: the window table over the look-back before the segment; the
 * maximum is order-independent, so the table is the same on every run */
PNG_HD void phase_window(SegShared &S, const SegArgs &A, int seg, int tid) {
  long long sb, se;
  seg_range(A, seg, sb, se);
  (void)se;
  const int nb = (int)(sb - S.w0); /* window bytes before the segment */
  for (int q = tid; q < nb && q + 4 <= S.wlen; q += NT) {
    const uint32_t v = (uint32_t)(q + 1);
#ifdef __CUDA_ARCH__
    atomicMax(&S.wtab[hash4(S.win + q)], v);
#else
    uint32_t &t = S.wtab[hash4(S.win + q)];
    if (v > t) t = v;
#endif
  }
}

/* phase 1: the parse (tokens, where the thread's last token ends) and the
 * Adler-32 partial sums */
PNG_HD void phase_parse(SegShared &S, const SegArgs &A, int seg, int tid) {
  long long b, e;
  sub_range(A, seg, tid, b, e);
  ParseSink ps{{thread_tokens(A, seg, tid), 0}, {&S, 1u}};
  const long long rb = b - S.w0, re = e - S.w0;
  const long long lim = re + OVERRUN < (long long)S.wlen ? re + OVERRUN : (long long)S.wlen;
  S.tend[tid] = (int)parse(S.win, rb, re, lim, S.cands(), ps);
  S.ntok[tid] = ps.t.n;
  unsigned long long s1 = 0, s2 = 0;
  for (long long p = rb; p < re; p++) {
    s1 += S.win[p];
    s2 += (unsigned long long)(re - p) * S.win[p];
  }
  S.a1[tid] = (uint32_t)s1;
  S.a2[tid] = (uint32_t)s2;
  S.alen[tid] = (uint32_t)(e - b);
}

/* replays thread tid's tokens, trimmed to the bytes no earlier thread's
 * final match covers (matches are at most 258 bytes, so only the five
 * threads before can reach into this share) */
template <class Sink>
PNG_HD void replay_trimmed(const SegShared &S, const SegArgs &A, int seg, int tid, Sink &s) {
  TrimSink<Sink> t{s, S.win, (long long)S.tstart[tid], (long long)S.tfrom[tid]};
  replay(thread_tokens(A, seg, tid), S.ntok[tid], t);
}

/* phase 1b: each thread's first uncovered byte; the histogram loses the
 * symbols of the tokens (or token heads) that byte drops and gains their
 * replacements -- only the thread's first few tokens are walked */
PNG_HD void phase_trim(SegShared &S, const SegArgs &A, int seg, int tid) {
  long long b, e;
  sub_range(A, seg, tid, b, e);
  (void)e;
  const int start = (int)(b - S.w0);
  int from = start;
  for (int j = tid - 1; j >= 0 && j >= tid - 5; j--) from = S.tend[j] > from ? S.tend[j] : from;
  S.tstart[tid] = start;
  S.tfrom[tid] = from;
  if (tid == 0) atomic_add_u32(&S.hist_lit[256], 1); /* end of block */
  if (from == start) return;
  HistSink sub{&S, 0xFFFFFFFFu}, add{&S, 1u};
  TrimSink<HistSink> keep{add, S.win, (long long)start, (long long)from};
  const uint16_t *tok = thread_tokens(A, seg, tid);
  long long pos = start;
  for (int i = 0; i < S.ntok[tid] && pos < from; i++) {
    const int v = tok[(size_t)i * NT];
    if (v < 256) {
      sub.literal((uint8_t)v);
      keep.literal((uint8_t)v);
      pos++;
    } else {
      const int L = v - 253, d = tok[(size_t)(i + 1) * NT] + 1;
      sub.match(L, d);
      keep.match(L, d);
      pos += L;
      i++;
    }
  }
}

/* phase 2a: sort keys of both alphabets' symbols, (alphabet, frequency,
 * symbol) ascending with unused symbols last */
PNG_HD void phase_keys(SegShared &S, int tid) {
  for (int i = tid; i < 1024; i += NT) {
    unsigned long long k = ~0ull;
    if (i < NLIT && S.hist_lit[i]) k = ((unsigned long long)S.hist_lit[i] << 16) | (unsigned)i;
    if (i >= 512 && i - 512 < NDIST && S.hist_dist[i - 512])
      k = (1ull << 63) | ((unsigned long long)S.hist_dist[i - 512] << 16) | (unsigned)(i - 512);
    S.keys[i] = k;
  }
}

#ifdef __CUDACC__
/* phase 2b on the device: bitonic sort of the 1024 keys by the whole CTA */
__device__ __forceinline__ void sort_keys(SegShared &S, int tid) {
  for (int k = 2; k <= 1024; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = tid; i < 1024; i += NT) {
        const int l = i ^ j;
        if (l > i) {
          const unsigned long long a = S.keys[i], b = S.keys[l];
          const bool up = (i & k) == 0;
          if ((a > b) == up) S.keys[i] = b, S.keys[l] = a;
        }
      }
      __syncthreads();
    }
}
#endif

/* phase 2c: how many symbols each alphabet uses (where the sorted keys
 * change alphabet or become unused) */
PNG_HD void phase_bounds(SegShared &S, int tid) {
  for (int i = tid; i < 1024; i += NT) {
    const unsigned long long k = S.keys[i], n = i + 1 < 1024 ? S.keys[i + 1] : ~0ull;
    const int ka = k == ~0ull ? 2 : (int)(k >> 63), na = n == ~0ull ? 2 : (int)(n >> 63);
    if (i == 0 && ka != 0) S.hs0.nused = 0;
    if (ka == 0 && na != 0) S.hs0.nused = (uint32_t)(i + 1);
    if (ka != 1 && na == 1) S.dist_first = (uint32_t)(i + 1);
    if (i == 0 && ka == 1) S.dist_first = 0;
    if (ka == 1 && na != 1) S.dist_last = (uint32_t)(i + 1);
  }
}

/* phase 2d: the used symbols of each alphabet in ascending order */
PNG_HD void phase_rank(SegShared &S, int tid) {
  if (tid == 0) S.hs1.nused = S.dist_last > S.dist_first ? S.dist_last - S.dist_first : 0;
  for (int i = tid; i < 1024; i += NT) {
    const unsigned long long k = S.keys[i];
    if (k == ~0ull) continue;
    const int a = (int)(k >> 63);
    /* literal/length keys come first: a distance key's rank is i minus them */
    const uint16_t sym = (uint16_t)(k & 0xFFFF);
    const uint32_t f = (uint32_t)((k >> 16) & 0x7FFFFFFFull);
    if (a) {
      const int r = i - (int)S.dist_first;
      S.hs1.sorted[r] = sym, S.hs1.wl[r] = f;
    } else {
      S.hs0.sorted[i] = sym, S.hs0.wl[i] = f;
    }
  }
}

/* phase 3: code lengths (thread 0: literal/length, thread 32: distance) */
PNG_HD void phase_lengths(SegShared &S, int tid) {
  if (tid == 0) huff_lengths(15, S.hs0, S.len_lit);
  if (tid == 32) {
    /* no matches: one distance code of one bit (RFC 1951 3.2.7) */
    if (S.hs1.nused == 0) S.hs1.nused = 1, S.hs1.sorted[0] = 0;
    huff_lengths(15, S.hs1, S.len_dist);
  }
}

/* phase 4: canonical codes of both alphabets, and where each alphabet's
 * nonzero lengths end */
PNG_HD void phase_codes(SegShared &S, int tid) {
  for (int i = tid; i < OUT_BYTES / 4; i += NT) S.out[i] = 0; /* the sort keys are dead */
  canonical_codes(S.len_lit, NLIT, S.hs0.first, S.code_lit, tid, NT);
  canonical_codes(S.len_dist, NDIST, S.hs1.first, S.code_dist, tid, NT);
  for (int i = tid; i < NLIT; i += NT)
    if (S.len_lit[i]) atomic_max_u32(&S.lit_end, (uint32_t)i + 1);
  for (int i = tid; i < NDIST; i += NT)
    if (S.len_dist[i]) atomic_max_u32(&S.dist_end, (uint32_t)i + 1);
}

/* The header's code lengths (RFC 1951 3.2.7): literal/length lengths
 * 0..hlit-1 then distance lengths 0..hdist-1 as one sequence, run-length
 * coded (16: repeat the previous length 3-6 times, 17: 3-10 zeros, 18:
 * 11-138 zeros).  Done per run in parallel: each run start counts its
 * entries, a scan places them, each run writes its own. */
PNG_HD int hdr_len(const SegShared &S, int i) { return i < S.hlit ? S.len_lit[i] : S.len_dist[i - S.hlit]; }

/* entries of the run of `run` copies of v (written at cl + off when cl) */
PNG_HD int rle_run(int v, int run, uint8_t *sym, uint8_t *extra) {
  int n = 0;
  auto put = [&](int s_, int e_) {
    if (sym) sym[n] = (uint8_t)s_, extra[n] = (uint8_t)e_;
    n++;
  };
  if (v == 0) {
    int r = run;
    while (r >= 11) {
      const int c = r < 138 ? r : 138;
      put(18, c - 11);
      r -= c;
    }
    if (r >= 3) {
      put(17, r - 3);
      r = 0;
    }
    while (r > 0) put(0, 0), r--;
  } else {
    put(v, 0);
    int r = run - 1;
    while (r >= 3) {
      const int c = r < 6 ? r : 6;
      put(16, c - 3);
      r -= c;
    }
    while (r > 0) put(v, 0), r--;
  }
  return n;
}

PNG_HD int run_at(const SegShared &S, int i, int total) {
  const int v = hdr_len(S, i);
  int run = 1;
  while (i + run < total && hdr_len(S, i + run) == v) run++;
  return run;
}

PNG_HD bool run_start(const SegShared &S, int i) { return i == 0 || hdr_len(S, i) != hdr_len(S, i - 1); }

/* phase 5a: sizes, and each thread's count of entries over its indices */
PNG_HD void phase_rle_count(SegShared &S, int tid) {
  const int hlit = S.lit_end > 257 ? (int)S.lit_end : 257;
  const int hdist = S.dist_end > 1 ? (int)S.dist_end : 1;
  const int total = hlit + hdist;
  if (tid == 0) S.hlit = hlit, S.hdist = hdist;
  const int ch = (total + NT - 1) / NT;
  int c = 0;
  /* S.hlit is not yet visible to other threads: index with the local sizes */
  for (int i = tid * ch; i < (tid + 1) * ch && i < total; i++) {
    auto L = [&](int k) -> int { return k < hlit ? S.len_lit[k] : S.len_dist[k - hlit]; };
    if (i == 0 || L(i) != L(i - 1)) {
      int run = 1;
      while (i + run < total && L(i + run) == L(i)) run++;
      c += rle_run(L(i), run, nullptr, nullptr);
    }
  }
  S.tbits[tid] = (uint32_t)c;
}

/* phase 5b (thread 0): offsets of the threads' entries */
PNG_HD void phase_rle_scan(SegShared &S, int tid) {
  if (tid != 0) return;
  uint32_t off = 0;
  for (int t = 0; t < NT; t++) {
    const uint32_t c = S.tbits[t];
    S.tbits[t] = off;
    off += c;
  }
  S.ncl = (int)off;
}

/* phase 5c: the entries, and their code-length histogram */
PNG_HD void phase_rle_write(SegShared &S, int tid) {
  const int total = S.hlit + S.hdist;
  const int ch = (total + NT - 1) / NT;
  int off = (int)S.tbits[tid];
  for (int i = tid * ch; i < (tid + 1) * ch && i < total; i++)
    if (run_start(S, i)) {
      const int n = rle_run(hdr_len(S, i), run_at(S, i, total), S.cl_sym + off, S.cl_extra + off);
      for (int k = 0; k < n; k++) atomic_add_u32(&S.hist_cl[S.cl_sym[off + k]], 1);
      off += n;
    }
}

/* phase 5d (thread 0): the code-length code (19 symbols, max 7 bits) */
PNG_HD void phase_cl_code(SegShared &S, int tid) {
  if (tid != 0) return;
  HuffScratchSmall &h = S.hs1;
  /* a code-length code must be complete: give a lone symbol a partner */
  uint32_t f2[NCL];
  int used = 0;
  for (int k = 0; k < NCL; k++) f2[k] = S.hist_cl[k], used += f2[k] ? 1 : 0;
  if (used < 2)
    for (int k = 0; k < NCL && used < 2; k++)
      if (!f2[k]) f2[k] = 1, used++;
  int m = 0;
  for (int k = 0; k < NCL; k++) {
    if (!f2[k]) continue;
    int q = m++;
    while (q > 0 && h.wl[q - 1] > f2[k]) {
      h.sorted[q] = h.sorted[q - 1];
      h.wl[q] = h.wl[q - 1];
      q--;
    }
    h.sorted[q] = (uint16_t)k;
    h.wl[q] = f2[k];
  }
  h.nused = (uint32_t)m;
  huff_lengths(7, h, S.len_cl);
  canonical_codes(S.len_cl, NCL, h.first, S.code_cl, 0, 1);
  int hclen = NCL;
  while (hclen > 4 && S.len_cl[cl_order(hclen - 1)] == 0) hclen--;
  S.hclen = hclen;
  S.hdr_bits = 3 + 5 + 5 + 4 + 3 * hclen;
}

/* phase 5e: the header's size */
PNG_HD void phase_hdr_bits(SegShared &S, int tid) {
  uint32_t bits = 0;
  for (int k = tid; k < S.ncl; k += NT) {
    const int s = S.cl_sym[k];
    bits += S.len_cl[s] + (s == 16 ? 2 : s == 17 ? 3 : s == 18 ? 7 : 0);
  }
  if (bits) atomic_add_u32(&S.hdr_bits, bits);
}

/* phase 6: bits of each thread's tokens */
PNG_HD void phase_count(SegShared &S, const SegArgs &A, int seg, int tid) {
  long long b, e;
  sub_range(A, seg, tid, b, e);
  (void)b, (void)e;
  CountSink cs{&S, 0};
  replay_trimmed(S, A, seg, tid, cs);
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
      atomic_or_u32(&S.out[pos >> 2], (uint32_t)S.win[sb - S.w0 + i] << (8 * (pos & 3)));
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
  (void)b, (void)e;
  replay_trimmed(S, A, seg, tid, es);
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
    (void)n;
    const uint32_t crc = gf2_mult(0xFFFFFFFFu, S.crc_xn) ^ S.crc_part[0] ^ 0xFFFFFFFFu;
    unsigned long long s1 = 0, s2 = 0, after = 0;
    for (int t = NT - 1; t >= 0; t--) {
      s1 += S.a1[t];
      s2 += S.a2[t] + (unsigned long long)S.a1[t] * after;
      after += S.alen[t];
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
