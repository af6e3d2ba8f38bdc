/*
 * f3g_iterate.cuh -- K1: chaos-game iteration + histogram accumulation.
 *
 * Replaces iter_thread (rect.c:253-527), flam3_iterate (flam3.c:232-299) and
 * the bucket accumulation (rect.c:411-516).  One persistent launch processes
 * any number of passes (temporal samples, frames, jobs): work is cut into
 * chunks of blockDim*S samples (blockDim*S_tail from a pass's chunk_tail on:
 * the short chunks that end a launch); a block takes chunk indices from a
 * global counter, stages the chunk's pass (xforms, variation lists,
 * xform-choice breakpoints, colour map, camera) in shared memory, and runs
 * fresh chains: random start point, discarded fuse steps, then its samples.
 *
 * Two ways to pick xforms:
 *   mode 0: every thread draws its own xform per step (the reference's
 *           semantics, and the only mode for genomes with xaos and for
 *           blocks of fewer than 4 warps);
 *   mode 1: one draw per warp per step, so the 32 lanes run the same
 *           variation code; every `shuffle_every` steps the warps exchange
 *           their points through shared memory (lagged by a round, on
 *           mbarriers: F3G_EXCHANGE) so the lanes of a warp hold points
 *           with different histories.  Each point still sees an i.i.d.
 *           xform sequence with the genome's probabilities.
 *
 * Samples are added to float4 buckets with one vector atomic
 * (red.global.add.v4.f32) or to double buckets with four FP64 atomics.
 */
#ifndef F3G_ITERATE_CUH
#define F3G_ITERATE_CUH
#include <cuda_runtime.h>
#include <stdint.h>

#include "f3g_common.h"
#include "f3g_device.cuh"
#include "f3g_launch.h"

namespace f3g {

/* F3G_FINAL_UNROLL: 1 (default) gives the final xform its own apply_xform
 * call site (more code, fewer loop branches: 4 % faster on the 1920x1080
 * still); 0 shares one site */
#ifndef F3G_FINAL_UNROLL
#define F3G_FINAL_UNROLL 1
#endif

/* F3G_PRETRUNC: see stage_pass */
#ifndef F3G_PRETRUNC
#define F3G_PRETRUNC 1
#endif

template <typename R> struct PassS {
  int num_xforms, num_std, final_index, final_enable, chaos_enable, fuse, mode, full;
  int width, height, nbuckets, rotate, cmap_size, palette_mode, bucket_kind, S, S_tail, trunc;
  long long samples, nchunks, chunk_tail;
  unsigned long long *counters;
  uint32_t key0, key1;
  R b0, b1, b2, b3, r00, r01, r10, r11, rcx, rcy, ws0, wb0s0, hs1, hb1s1, cmap_size_r;
  double db0, db1, db2, db3, dws0, dwb0s0, dhs1, dhb1s1;
  void *buckets, *count;
  uint16_t nbrk[F3G_MAX_XFORMS + 1];
  uint16_t brk[F3G_MAX_XFORMS + 1][F3G_MAX_XFORMS];
  /* row 0 by the top 8 of the 14 bits: the xform when no breakpoint falls
   * in the bucket, else 0x8000 | breakpoints below the bucket */
  uint16_t lut[256];
  uint8_t var_id[F3G_MAX_VARLIST];
  R var_w[F3G_MAX_VARLIST];
  float4 dmap[256];
  XfS<R> xf[F3G_MAX_XFORMS];
};

template <typename R> struct ShufPoint { R x, y, c; int consec; };

/* Stage pass `p` into shared memory (all threads participate). */
template <typename R>
__device__ void stage_pass(PassS<R> &s, const F3GPass *__restrict__ p) {
  const int t = threadIdx.x, T = blockDim.x;
#if F3G_PRETRUNC
  /* integer buckets with a step palette where every xform plots at opacity
   * 1: each hit adds a colour-map entry as it stands, so the map is
   * truncated once here instead of at every hit (trunc 2) */
  int vis1 = 1;
  for (int i = t; i < p->num_xforms; i += T) vis1 &= p->xf[i].vis_adjusted == 1.0;
  const bool pretrunc = __syncthreads_and(vis1) && p->trunc_hits && p->palette_mode == 0;
#else
  const bool pretrunc = false;
#endif
  if (t == 0) {
    s.num_xforms = p->num_xforms; s.num_std = p->num_std; s.final_index = p->final_index;
    s.final_enable = p->final_enable; s.chaos_enable = p->chaos_enable; s.fuse = p->fuse;
    s.mode = p->iter_mode; s.full = p->full_variations;
    s.width = p->width; s.height = p->height; s.nbuckets = p->width * p->height;
    s.rotate = p->rotate; s.cmap_size = p->cmap_size; s.cmap_size_r = (R)p->cmap_size;
    s.palette_mode = p->palette_mode; s.bucket_kind = p->bucket_kind;
    s.trunc = p->trunc_hits ? (pretrunc ? 2 : 1) : 0;
    s.samples = p->samples; s.nchunks = p->nchunks; s.key0 = p->key[0]; s.key1 = p->key[1];
    s.b0 = (R)p->bounds[0]; s.b1 = (R)p->bounds[1]; s.b2 = (R)p->bounds[2]; s.b3 = (R)p->bounds[3];
    s.db0 = p->bounds[0]; s.db1 = p->bounds[1]; s.db2 = p->bounds[2]; s.db3 = p->bounds[3];
    s.r00 = (R)p->rot[0][0]; s.r01 = (R)p->rot[0][1]; s.r10 = (R)p->rot[1][0]; s.r11 = (R)p->rot[1][1];
    s.rcx = (R)p->rot_center[0]; s.rcy = (R)p->rot_center[1];
    s.ws0 = (R)p->ws0; s.wb0s0 = (R)p->wb0s0; s.hs1 = (R)p->hs1; s.hb1s1 = (R)p->hb1s1;
    s.dws0 = p->ws0; s.dwb0s0 = p->wb0s0; s.dhs1 = p->hs1; s.dhb1s1 = p->hb1s1;
    s.buckets = p->buckets; s.count = p->count;
    s.S = p->S; s.counters = p->counters;
    s.S_tail = p->S_tail > 0 ? p->S_tail : p->S;
    s.chunk_tail = p->S_tail > 0 ? p->chunk_tail : p->nchunks;
  }
  const int nx = p->num_xforms;
  const int rows = p->num_std + 1;
  for (int i = t; i < rows * F3G_MAX_XFORMS; i += T) {
    int r = i / F3G_MAX_XFORMS, c = i % F3G_MAX_XFORMS;
    s.brk[r][c] = p->brk[r][c];
  }
  for (int i = t; i < rows; i += T) s.nbrk[i] = p->nbrk[i];
  for (int b = t; b < 256; b += T) {
    const int n = p->nbrk[0];
    int lo = 0, hi = 0;
    for (int k = 0; k < n; k++) {
      lo += p->brk[0][k] <= (uint16_t)(b << 6);
      hi += p->brk[0][k] <= (uint16_t)((b << 6) | 63);
    }
    s.lut[b] = (uint16_t)(lo == hi ? lo : (0x8000 | lo));
  }
  for (int i = t; i < F3G_MAX_VARLIST; i += T) {
    s.var_id[i] = p->var_id[i];
    s.var_w[i] = (R)p->var_w[i];
  }
  for (int i = t; i < 256; i += T) {
    float4 d = make_float4(p->dmap[i][0], p->dmap[i][1], p->dmap[i][2], p->dmap[i][3]);
    if (pretrunc) d = make_float4(truncf(d.x), truncf(d.y), truncf(d.z), truncf(d.w));
    s.dmap[i] = d;
  }
  /* xform scalars and parameters */
  const int per = 6 + 6 + 5 + PRM_COUNT;
  for (int i = t; i < nx * per; i += T) {
    int xi = i / per, k = i % per;
    const F3GXform &g = p->xf[xi];
    XfS<R> &d = s.xf[xi];
    if (k < 6) d.c[k] = (R)g.c[k];
    else if (k < 12) d.post[k - 6] = (R)g.post[k - 6];
    else if (k == 12) d.color = (R)g.color;
    else if (k == 13) d.color_speed = (R)g.color_speed;
    else if (k == 14) d.vis_adjusted = (R)g.vis_adjusted;
    else if (k == 15) d.opacity = (R)g.opacity;
    else if (k == 16) {
      d.preblur = (R)g.preblur;
      d.flags = g.flags;
      d.var_off = g.var_off;
      d.nvars = g.nvars;
    } else
      d.prm[k - 17] = (R)g.prm[k - 17];
  }
}

/* xform choice: the number of breakpoints of row `row` that are <= v
 * (row 0 through the 256-entry table, scanning only inside a bucket that
 * holds a breakpoint) */
template <typename R>
__device__ __forceinline__ int pick_xform(const PassS<R> &s, int row, uint32_t v) {
  if (row == 0) {
    const int e = s.lut[v >> 6];
    if (!(e & 0x8000)) return e;
    int fn = e & 0x7fff;
    const int n = s.nbrk[0];
    while (fn < n && s.brk[0][fn] <= v) fn++;
    return fn;
  }
  int n = s.nbrk[row], fn = 0;
  for (int k = 0; k < n; k++) fn += (s.brk[row][k] <= v);
  return fn;
}

/* Bucket of a point (rect.c:411-440): optional rotation about rot_center,
 * the inclusive bounds test, the index; -1 outside the histogram. */
template <typename R>
__device__ __forceinline__ int bucket_of(const PassS<R> &s, R qx, R qy) {
  R p0 = qx, p1 = qy;
  if (s.rotate) {
    R p00 = qx - s.rcx, p11 = qy - s.rcy;
    p0 = p00 * s.r00 + p11 * s.r01 + s.rcx;
    p1 = p00 * s.r10 + p11 * s.r11 + s.rcy;
  }
  if (!(p0 >= s.b0 && p1 >= s.b1 && p0 <= s.b2 && p1 <= s.b3)) return -1;
  int xi, yi;
  if (sizeof(R) == 8) {
    xi = (int)(s.dws0 * (double)p0 - s.dwb0s0);
    yi = (int)(s.dhs1 * (double)p1 - s.dhb1s1);
  } else {
    /* same index as the reference's ws0*p0 - wb0s0, rearranged so FP32 does
     * not cancel against a large wb0s0 */
    xi = (int)(s.ws0 * (p0 - s.b0));
    yi = (int)(s.hs1 * (p1 - s.b1));
  }
  /* inside the bounds xi <= W and yi <= H, so the index fits 32 bits; one
   * unsigned compare tests 0 <= idx < nbuckets */
  const int idx = xi + s.width * yi;
  return (unsigned)idx >= (unsigned)s.nbuckets ? -1 : idx;
}

/* rect.c:411-516 for one sample.  With `agg` (warp-uniform), lanes of the
 * converged group that hit the same bucket are summed through shuffles and
 * added with one atomic by the lowest such lane: attractors concentrated on
 * few buckets otherwise serialise on same-address atomics in L2. */
template <typename R>
__device__ __forceinline__ unsigned plot(const PassS<R> &s, R qx, R qy, R qc, R qo, bool agg = false) {
  const int idx = bucket_of(s, qx, qy);
  if (idx < 0) return 0u;
  if (qo == (R)0) return 0u;
  float4 col;
  const R dbl_index0 = qc * s.cmap_size_r;
  int ci = (int)dbl_index0;
  const int cm1 = s.cmap_size - 1;
  if (s.palette_mode == 1) {
    R frac;
    if (ci < 0) { ci = 0; frac = (R)0; }
    else if (ci >= cm1) { ci = cm1 - 1; frac = (R)1; }
    else frac = dbl_index0 - (R)ci;
    float4 a = s.dmap[ci], b = s.dmap[ci + 1];
    float ff = (float)frac, gg = 1.0f - ff;
    col = make_float4(a.x * gg + b.x * ff, a.y * gg + b.y * ff, a.z * gg + b.z * ff, a.w * gg + b.w * ff);
  } else {
    if (ci < 0) ci = 0;
    else if (ci >= cm1) ci = cm1;
    col = s.dmap[ci];
  }
  float cnt = 255.0f;
  if (qo != (R)1) {
    float o = (float)qo;
    col.x *= o; col.y *= o; col.z *= o; col.w *= o;
    cnt *= o;
  }
  if (s.trunc == 1) {
    /* integer buckets: the reference adds (unsigned)(delta) per hit (trunc
     * 2: the colour map is truncated already and every opacity is 1) */
    col = make_float4(truncf(col.x), truncf(col.y), truncf(col.z), truncf(col.w));
    cnt = truncf(cnt);
  }
  if (agg) {
    const unsigned act = __activemask();
    const unsigned peers = __match_any_sync(act, idx);
    if (peers != (1u << (threadIdx.x & 31))) {
      float4 sum = make_float4(0.f, 0.f, 0.f, 0.f);
      float csum = 0.f;
      for (unsigned m = peers; m; m &= m - 1) {
        const int src = __ffs(m) - 1;
        sum.x += __shfl_sync(peers, col.x, src);
        sum.y += __shfl_sync(peers, col.y, src);
        sum.z += __shfl_sync(peers, col.z, src);
        sum.w += __shfl_sync(peers, col.w, src);
        csum += __shfl_sync(peers, cnt, src);
      }
      if ((int)(threadIdx.x & 31) != __ffs(peers) - 1) return 1u;
      col = sum;
      cnt = csum;
    }
  }
  if (s.bucket_kind == F3G_BK_F32) {
    float4 *b = (float4 *)s.buckets + idx;
    atomicAdd(b, col);
    if (s.count) atomicAdd((float *)s.count + idx, cnt);
  } else {
    double *b = (double *)s.buckets + 4 * idx;
    atomicAdd(b + 0, (double)col.x);
    atomicAdd(b + 1, (double)col.y);
    atomicAdd(b + 2, (double)col.z);
    atomicAdd(b + 3, (double)col.w);
    if (s.count) atomicAdd((double *)s.count + idx, (double)cnt);
  }
  return 1u;
}

/* One chain step (flam3.c:249-296).  Returns true when q is a sample to
 * store (false while retrying a bad value).  The xform and, when enabled,
 * the final xform are the two stages of a loop (unrolled by default, see
 * F3G_FINAL_UNROLL). */
template <typename R, bool FULL, class G>
__device__ __forceinline__ bool chain_step(const PassS<R> &s, int fn, R &px, R &py, R &pc, R &po, int &consec,
                                           int &lastxf, unsigned &bad, R &qx, R &qy, R &qc, R &qo, G &rng) {
  int cur = fn;
  R ix = px, iy = py, ic = pc;
#if F3G_FINAL_UNROLL
#pragma unroll
#else
#pragma unroll 1
#endif
  for (int stage = 0; stage < 2; stage++) {
    R nx, ny, nc, no;
    const bool b = apply_xform<R, FULL, G>(s.xf[cur], s.var_id, s.var_w, ix, iy, ic, nx, ny, nc, no, rng);
    if (stage == 0) {
      if (b) {
        consec++;
        bad++;
        if (consec < 5) {
          px = nx; py = ny; pc = nc; po = no;
          return false;
        }
        consec = 0;
      } else
        consec = 0;
      lastxf = fn + 1;
      px = nx; py = ny; pc = nc; po = no;
      qx = px; qy = py; qc = pc; qo = po;
      if (!s.final_enable) break;
      const R fop = s.xf[s.final_index].opacity;
      if (!(fop == (R)1 || u01<R>(rng.word()) < fop)) break;
      cur = s.final_index;
      ix = px; iy = py; ic = pc;
    } else {
      /* the final xform's result is plotted; the opacity stays the xform's */
      qx = nx; qy = ny; qc = nc;
    }
  }
  return true;
}

/* F3G_LEAN_RNG: where the iterate kernels' random streams keep their state.
 * 0: pass key, counters and words in registers (Rng, WarpWords); 1: the
 * pass key and chunk index in shared memory, read at each refill (ChunkRng,
 * ChunkWarpWords); 2 (default): the words in shared memory too
 * (ChunkRngS, ChunkWarpWordsS), one counter register per stream.  The
 * kernel runs at its 64-register cap, so each register freed is a spill
 * avoided: on the 1920x1080 still 50.7 (0), 51.6 (1) and 52.5 (2) Giter/s.
 * The words are the same at every level. */
#ifndef F3G_LEAN_RNG
#define F3G_LEAN_RNG 2
#endif

/* The random streams of the chunk a block is running: the pass key and the
 * chunk's counter word, set by thread 0 before the chunk starts.  The
 * streams below read them at each refill instead of holding them in
 * registers (the iterate kernel runs at its 64-register cap). */
static __shared__ uint32_t f3g_chunk_ctx[3]; /* key0, key1, chunk */

/* Per-thread word stream of a chunk: Philox blocks of counter (chunk, k,
 * thread, 0x5EED) under the pass key, k = 0, 1, ...; four words per block
 * in order.  Registers: the block's four words and the word count. */
struct ChunkRng {
  uint32_t b0, b1, b2, b3, m;
  __device__ __forceinline__ void init() { m = 0; }
  __device__ __forceinline__ uint32_t word() {
    if ((m & 3u) == 0) {
      const uint4 r = philox_block(f3g_chunk_ctx[2], m >> 2, threadIdx.x, 0x5EEDu, f3g_chunk_ctx[0], f3g_chunk_ctx[1]);
      b0 = r.x; b1 = r.y; b2 = r.z; b3 = r.w;
    }
    const uint32_t c = m & 3u;
    m++;
    return c == 0 ? b0 : c == 1 ? b1 : c == 2 ? b2 : b3;
  }
};

/* Warp-shared stream of xform-choice words: lane L holds words 4L..4L+3 of
 * the current 128-word block, counter (chunk, k, 0xC0DE0000 | warp, L) under
 * the pass key, so one Philox call per lane serves 128 steps of the warp;
 * word n is read from lane (n / 4) % 32 with one shuffle.  The counters are
 * disjoint from the per-thread streams (third word = thread index <
 * 0xC0DE0000).  Warp-uniform: every lane calls word() at the same step. */
struct ChunkWarpWords {
  uint32_t b0, b1, b2, b3, n;
  __device__ __forceinline__ void init() { n = 0; }
  __device__ __forceinline__ uint32_t word() {
    if ((n & 127u) == 0) {
      const uint4 r = philox_block(f3g_chunk_ctx[2], n >> 7, 0xC0DE0000u | (threadIdx.x >> 5), threadIdx.x & 31u,
                                   f3g_chunk_ctx[0], f3g_chunk_ctx[1]);
      b0 = r.x; b1 = r.y; b2 = r.z; b3 = r.w;
    }
    const uint32_t c = n & 3u;
    const uint32_t mine = c == 0 ? b0 : c == 1 ? b1 : c == 2 ? b2 : b3;
    const uint32_t w = __shfl_sync(0xffffffffu, mine, (n >> 2) & 31u);
    n++;
    return w;
  }
};

/* The same two streams with their words in shared memory as well
 * (F3G_LEAN_RNG 2): a thread keeps one word counter.  A thread's four words
 * sit at f3g_thread_words[k][thread] (consecutive threads, consecutive
 * banks); a warp's 128-word block at f3g_warp_words[warp][n], lane L's four
 * words at 4L..4L+3 -- word n of the block is component n % 4 of lane n / 4,
 * as in ChunkWarpWords -- read as a broadcast. */
static __shared__ __align__(16) uint32_t f3g_thread_words[4][256];
static __shared__ __align__(16) uint32_t f3g_warp_words[8][128];

struct ChunkRngS {
  uint32_t m;
  __device__ __forceinline__ void init() { m = 0; }
  __device__ __forceinline__ uint32_t word() {
    const unsigned t = threadIdx.x;
    if ((m & 3u) == 0) {
      const uint4 r = philox_block(f3g_chunk_ctx[2], m >> 2, t, 0x5EEDu, f3g_chunk_ctx[0], f3g_chunk_ctx[1]);
      f3g_thread_words[0][t] = r.x;
      f3g_thread_words[1][t] = r.y;
      f3g_thread_words[2][t] = r.z;
      f3g_thread_words[3][t] = r.w;
    }
    const uint32_t w = f3g_thread_words[m & 3u][t];
    m++;
    return w;
  }
};

struct ChunkWarpWordsS {
  uint32_t n;
  __device__ __forceinline__ void init() { n = 0; }
  /* warp-uniform: every lane calls it at the same step */
  __device__ __forceinline__ uint32_t word() {
    const unsigned warp = threadIdx.x >> 5;
    if ((n & 127u) == 0) {
      const unsigned lane = threadIdx.x & 31u;
      const uint4 r = philox_block(f3g_chunk_ctx[2], n >> 7, 0xC0DE0000u | warp, lane, f3g_chunk_ctx[0],
                                   f3g_chunk_ctx[1]);
      __syncwarp(); /* every lane has read the last block */
      reinterpret_cast<uint4 *>(f3g_warp_words[warp])[lane] = r;
      __syncwarp();
    }
    const uint32_t w = f3g_warp_words[warp][n & 127u];
    n++;
    return w;
  }
};

/* mode 0: independent chains, one per thread */
template <typename R, bool FULL>
__device__ void run_chunk_thread(const PassS<R> &s, long long local_chunk, long long base, long long len,
                                 unsigned &bad_total, unsigned &hits) {
  const int T = blockDim.x, t = threadIdx.x;
  long long n_chunk = s.samples - base;
  if (n_chunk > len) n_chunk = len;
  const int q = (int)(n_chunk / T + ((long long)t < n_chunk % T ? 1 : 0));
#if F3G_LEAN_RNG == 2
  ChunkRngS rng;
  rng.init();
  typedef ChunkRngS RngT;
#elif F3G_LEAN_RNG
  ChunkRng rng;
  rng.init();
  typedef ChunkRng RngT;
#else
  Rng rng;
  rng.init(s.key0, s.key1, (uint32_t)local_chunk, (uint32_t)t, 0x5EEDu);
  typedef Rng RngT;
#endif
  R px = u11<R>(rng.word()), py = u11<R>(rng.word()), pc = u01<R>(rng.word()), po = u01<R>(rng.word());
  int consec = 0, lastxf = 0;
  unsigned bad = 0;
  const int total = s.fuse;
  for (int i = -total; i < q;) {
    int row = s.chaos_enable ? min(lastxf, s.num_std) : 0;
    int fn = pick_xform(s, row, rng.word() & (F3G_GRAIN - 1));
    R qx, qy, qc, qo;
    if (!chain_step<R, FULL, RngT>(s, fn, px, py, pc, po, consec, lastxf, bad, qx, qy, qc, qo, rng)) continue;
    if (i >= 0) hits += plot(s, qx, qy, qc, qo);
    i++;
  }
  bad_total += bad;
}

/* F3G_AGG: 0 never aggregate bucket adds, 1 (default) always for FP64
 * buckets (four atomics per sample) and, for FP32 buckets, per chunk when
 * probes taken right after block shuffles find at least F3G_AGG_LANES of a
 * warp's points sharing buckets, 2 always.  Measured on the 1920x1080 q2000 still /
 * an animation key genome whose attractor covers few buckets: never 45.9 /
 * 10.0 Giter/s, always 38.0 / 41.0, probed after the shuffle with 8 lanes
 * 48.7 / 39.2 (the still's chunks stay direct); FP64 buckets 13.9 without,
 * 20.2 with aggregation. */
#ifndef F3G_AGG
#define F3G_AGG 1
#endif
#ifndef F3G_AGG_LANES
#define F3G_AGG_LANES 8
#endif

/* F3G_SHUF_WARPS: warps per shuffle group (8 = the whole block, default);
 * smaller groups synchronise on named barriers and wait for fewer warps, but
 * mix less: measured on the 1920x1080 still, groups of 4 warps 43.2 Giter/s
 * and 0.4 % more image error than whole-block shuffles at 49.4 */
#ifndef F3G_SHUF_WARPS
#define F3G_SHUF_WARPS 8
#endif

/* named barrier `id` over n threads (PTX bar.sync) */
__device__ __forceinline__ void group_sync(int id, int n) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}
/* named barrier with an OR of `pred` over its n threads (PTX bar.red.or.pred) */
__device__ __forceinline__ int group_or(int id, int n, int pred) {
  int r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\tsetp.ne.s32 q, %1, 0;\n\tbar.red.or.pred p, %2, %3, q;\n\tselp.s32 %0, 1, 0, p;\n\t}"
      : "=r"(r)
      : "r"(pred), "r"(id), "r"(n)
      : "memory");
  return r;
}

/* Warp-shared stream of xform-choice words: lane L holds four words of the
 * current 128-word block of counter (chunk, block, 0xC0DE0000 | warp, L),
 * so one Philox call per lane serves 128 steps of the warp; word k is
 * component k % 4 of lane k / 4 (one shuffle).  The counters are disjoint
 * from the per-thread streams (third word = thread index < 0xC0DE0000). */
struct WarpWords {
  uint4 blk;
  uint32_t c0, next, tag, lane, k0, k1;
  int used;
  __device__ __forceinline__ void init(uint32_t key0, uint32_t key1, uint32_t chunk, uint32_t warp, uint32_t ln) {
    k0 = key0; k1 = key1; c0 = chunk; next = 0; tag = 0xC0DE0000u | warp; lane = ln; used = 128;
  }
  /* warp-uniform: every lane of the warp calls it at the same step */
  __device__ __forceinline__ uint32_t word() {
    if (used == 128) {
      blk = philox_block(c0, next, tag, lane, k0, k1);
      next++;
      used = 0;
    }
    const int c = used & 3;
    const uint32_t mine = c == 0 ? blk.x : c == 1 ? blk.y : c == 2 ? blk.z : blk.w;
    const uint32_t w = __shfl_sync(0xffffffffu, mine, used >> 2);
    used++;
    return w;
  }
};

/* mode 1: warp-coherent xform choice plus block-wide point shuffles */
template <typename R, bool FULL>
__device__ void run_chunk_warp(const PassS<R> &s, ShufPoint<R> *buf, long long local_chunk, long long base,
                               long long len, int shuffle_every, unsigned &bad_total, unsigned &hits) {
  const int T = blockDim.x, t = threadIdx.x, lane = t & 31, nwarps = T >> 5;
  long long n_chunk = s.samples - base;
  if (n_chunk > len) n_chunk = len;
  long long q = n_chunk / T + ((long long)t < n_chunk % T ? 1 : 0);
  R *bx = reinterpret_cast<R *>(buf), *by = bx + T, *bc = by + T;
  int *bq = reinterpret_cast<int *>(bc + T);
#if F3G_SHUF_WARPS < 8
  /* shuffle groups of G warps (named barriers 1.. when G < the block's warps) */
  const int G = nwarps < F3G_SHUF_WARPS ? nwarps : F3G_SHUF_WARPS;
  const int GT = 32 * G, grp = (t >> 5) / G, wl = (t >> 5) % G, gbase = grp * GT;
#else
  const int G = nwarps, GT = T, wl = t >> 5, gbase = 0;
#endif
  Rng rng;
  rng.init(s.key0, s.key1, (uint32_t)local_chunk, (uint32_t)t, 0x5EEDu);
  WarpWords ww;
  ww.init(s.key0, s.key1, (uint32_t)local_chunk, (uint32_t)(t >> 5), (uint32_t)lane);
  R px = u11<R>(rng.word()), py = u11<R>(rng.word()), pc = u01<R>(rng.word()), po = u01<R>(rng.word());
  int consec = 0, lastxf = 0;
  unsigned bad = 0;
  /* fuse, then sample; the block leaves only when every thread is done */
  int fuse_left = s.fuse;
  long long remaining = q;
  uint32_t rot = 0;
  /* warp-aggregated accumulation: always for FP64 buckets; for FP32 it is
   * switched on for the rest of the chunk when probes (after the shuffles of
   * rounds 7, 15, 23, 31) find many of the warp's points sharing buckets in
   * two of four probes */
  bool agg = F3G_AGG == 2 || (F3G_AGG == 1 && s.bucket_kind == F3G_BK_F64);
  int probes = 0, dups = 0;
  for (int round = 0;; round++) {
    for (int k = 0; k < shuffle_every; k++) {
      const uint32_t w = ww.word();
      int fn = pick_xform(s, 0, w & (F3G_GRAIN - 1));
      R qx, qy, qc, qo;
      bool ok = chain_step<R, FULL, Rng>(s, fn, px, py, pc, po, consec, lastxf, bad, qx, qy, qc, qo, rng);
      if (ok) {
        if (fuse_left > 0) fuse_left--;
        else if (remaining > 0) {
          hits += plot(s, qx, qy, qc, qo, agg);
          remaining--;
        }
      }
    }

    rot += 0x9E3779B1u * (uint32_t)(round + 1);
    /* transpose lanes across the warps of the shuffle group, XOR the low five
     * bits and rotate by whole 32-point segments (group-uniform amounts);
     * points are stored structure-of-arrays at swizzled slots
     * i ^ ((i >> 5) & 31), so both the transposed writes and the reads hit
     * 32 distinct banks */
    const int x5 = (int)(rot >> 27), kr = (int)(rot >> 24) % G;
    const int dst = gbase + ((((lane * G + wl) ^ x5) + 32 * kr) & (GT - 1));
    const int wslot = dst ^ ((dst >> 5) & 31), rslot = t ^ ((t >> 5) & 31);
    int more;
#if F3G_SHUF_WARPS < 8
    if (G < nwarps) {
      group_sync(1 + grp, GT);
      bx[wslot] = px; by[wslot] = py; bc[wslot] = pc; bq[wslot] = consec;
      more = group_or(1 + grp, GT, remaining > 0 || fuse_left > 0);
    } else
#endif
    {
      __syncthreads();
      bx[wslot] = px; by[wslot] = py; bc[wslot] = pc; bq[wslot] = consec;
      more = __syncthreads_or(remaining > 0 || fuse_left > 0);
    }
    px = bx[rslot]; py = by[rslot]; pc = bc[rslot]; consec = bq[rslot];
    if (!more) break;
#if F3G_AGG == 1
    /* probe right after the shuffle (block converged), when a warp holds
     * points from every warp: shared buckets then reflect the attractor,
     * not the steps the warp's lanes took together */
    if (!agg && probes < 4 && (round & 7) == 7) {
      const int b = bucket_of(s, px, py);
      const unsigned peers = __match_any_sync(0xffffffffu, b < 0 ? -1 - lane : b);
      const unsigned shared = __ballot_sync(0xffffffffu, __popc(peers) > 1);
      dups += __popc(shared) >= F3G_AGG_LANES;
      if (++probes == 4) agg = dups >= 2;
    }
#endif
  }
  (void)po;
  bad_total += bad;
}

/* F3G_EXCHANGE: how mode 1 moves points between warps.
 *   0: the block shuffle above -- every `shuffle_every` steps all warps
 *      meet at a block barrier, so each round waits for the warp whose
 *      xforms were the most expensive;
 *   1 (default): a lagged exchange through two shared buffers and two
 *      mbarriers -- a warp writes its points to the buffer of round h and
 *      takes its next points from the buffer of round h-1, waiting only
 *      until every warp has finished round h-1, so warps drift up to one
 *      round apart instead of meeting every round. */
#ifndef F3G_EXCHANGE
#define F3G_EXCHANGE 1
#endif

/* shared-memory mbarrier helpers (PTX mbarrier.*; CTA scope) */
__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_addr(bar))
               : "memory");
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
/* waits for the completion of the barrier's phase of parity `ph`; false when
 * it has not completed within about two seconds (a lost arrival) */
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned ph) {
  const unsigned a = smem_addr(bar);
  unsigned long long t0 = 0;
  for (unsigned i = 0; i < (1u << 30); i++) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(a), "r"(ph)
        : "memory");
    if (ok) return true;
    if ((i & 255) == 0) {
      const unsigned long long t = global_ns();
      if (i == 0) t0 = t;
      else if (t - t0 > 2000000000ull) return false;
    }
  }
  return false;
}

/* Block state of the lagged exchange: two mbarriers (one arrival per warp
 * per round), the done-thread counts of rounds h mod 4, an abort flag. */
struct Exchange {
  uint64_t bar[2];
  int done[4];
  int abort;
};

/* mode 1 with the lagged exchange (F3G_EXCHANGE 1).  The block keeps 2T
 * points: T in registers, T in the buffer of the last round.  Round h: a
 * thread runs `shuffle_every` steps on its point, waits for buffer (h-1)&1
 * (every warp has written round h-1), takes the point at its slot there,
 * writes its own point to buffer h&1 at the round's permuted slot and
 * arrives.  A buffer is rewritten only after every thread waited for the
 * other one, which each does after reading, so no read races a write.  A
 * point is advanced every other round, so the thread discards 2 fuse +
 * shuffle_every steps before plotting: every point then has at least `fuse`
 * steps behind it.  Threads add themselves to the round's done count (no
 * samples left) before arriving; when the count of round h-1 is the whole
 * block, every thread sees it after the same wait and all leave together.
 * The count of round h+2 is cleared in round h, after every thread has read
 * it (in round h-1) and before anyone adds to it (in round h+2).  `ph` holds
 * the two barriers' phase parities (kept across chunks); false when a wait
 * timed out. */
template <typename R, bool FULL>
__device__ bool run_chunk_warp_lag(const PassS<R> &s, ShufPoint<R> *buf, Exchange &xc, unsigned &ph,
                                   long long local_chunk, long long base, long long len, int shuffle_every,
                                   int stall, unsigned &bad_total, unsigned &hits) {
  const int T = blockDim.x, t = threadIdx.x, lane = t & 31, G = T >> 5, wl = t >> 5;
  long long n_chunk = s.samples - base;
  if (n_chunk > len) n_chunk = len;
  /* samples of this thread (at most S) */
  int remaining = (int)(n_chunk / T + ((long long)t < n_chunk % T ? 1 : 0));
  /* buffer k: x, y, colour (R) and bad-value count (int) arrays of T each,
   * at xb + k * half */
  unsigned char *const xb = reinterpret_cast<unsigned char *>(buf);
  const unsigned half = (unsigned)(sizeof(ShufPoint<R>) * T);
#if F3G_LEAN_RNG == 2
  ChunkRngS rng;
  rng.init();
  ChunkWarpWordsS ww;
  ww.init();
  typedef ChunkRngS RngT;
#elif F3G_LEAN_RNG
  ChunkRng rng;
  rng.init();
  ChunkWarpWords ww;
  ww.init();
  typedef ChunkRng RngT;
#else
  Rng rng;
  rng.init(s.key0, s.key1, (uint32_t)local_chunk, (uint32_t)t, 0x5EEDu);
  WarpWords ww;
  ww.init(s.key0, s.key1, (uint32_t)local_chunk, (uint32_t)wl, (uint32_t)lane);
  typedef Rng RngT;
#endif
  R px = u11<R>(rng.word()), py = u11<R>(rng.word()), pc = u01<R>(rng.word()), po = u01<R>(rng.word());
  int consec = 0, lastxf = 0;
  unsigned bad = 0;
  const int rslot = t ^ ((t >> 5) & 31);
  /* round -1: the second set of points, at the reading slots of round 0 */
  {
    const R ax = u11<R>(rng.word()), ay = u11<R>(rng.word()), ac = u01<R>(rng.word());
    R *X = reinterpret_cast<R *>(xb + half);
    X[rslot] = ax; X[T + rslot] = ay; X[2 * T + rslot] = ac;
    reinterpret_cast<int *>(X + 3 * T)[rslot] = 0;
    __syncwarp();
    /* the stall test: warp 0 withholds this arrival, so every warp's first
     * wait runs out */
    if (lane == 0 && !(stall && wl == 0)) mbar_arrive(&xc.bar[1]);
  }
  int fuse_left = 2 * s.fuse + shuffle_every;
  uint32_t rot_acc = 0; /* the rounds' rotation, accumulated */
  /* bucket-sharing probes: bits 0-2 probes taken, 3-5 probes with shared
   * buckets, bit 6 aggregation on */
  int agg_state = (F3G_AGG == 2 || (F3G_AGG == 1 && s.bucket_kind == F3G_BK_F64)) ? 64 : 0;
  bool ok_all = true;
  for (int round = 0;; round++) {
    const bool agg = agg_state & 64;
    for (int k = 0; k < shuffle_every; k++) {
      const uint32_t w = ww.word();
      int fn = pick_xform(s, 0, w & (F3G_GRAIN - 1));
      R qx, qy, qc, qo;
      bool ok = chain_step<R, FULL, RngT>(s, fn, px, py, pc, po, consec, lastxf, bad, qx, qy, qc, qo, rng);
      if (ok) {
        if (fuse_left > 0) fuse_left--;
        else if (remaining > 0) {
          hits += plot(s, qx, qy, qc, qo, agg);
          remaining--;
        }
      }
    }
    const int cur = round & 1, prev = cur ^ 1;
    /* the points of round h-1 (the warp decides together, so a wait that
     * ends at the time limit in one lane ends the exchange for all) */
    if (!__all_sync(0xffffffffu, mbar_wait(&xc.bar[prev], (ph >> prev) & 1u))) {
      xc.abort = 1;
      ok_all = false;
      break;
    }
    ph ^= 1u << prev;
    const R *P = reinterpret_cast<const R *>(xb + prev * half);
    const R nx_ = P[rslot], ny_ = P[T + rslot], nc_ = P[2 * T + rslot];
    const int nq_ = reinterpret_cast<const int *>(P + 3 * T)[rslot];
    if (xc.done[(round - 1) & 3] == T) break; /* every thread had finished by round h-1 */
    if (t == 0) xc.done[(round + 2) & 3] = 0;
    /* this round's points to buffer h&1: transpose lanes across warps, XOR
     * the low five bits, rotate by whole 32-point segments (block-uniform
     * amounts), at swizzled slots (32 distinct banks) */
    rot_acc += 0x9E3779B1u * (uint32_t)(round + 1);
    const uint32_t rot = rot_acc;
    const int x5 = (int)(rot >> 27), kr = (int)(rot >> 24) % G;
    const int dst = (((lane * G + wl) ^ x5) + 32 * kr) & (T - 1);
    const int wslot = dst ^ ((dst >> 5) & 31);
    R *W = reinterpret_cast<R *>(xb + cur * half);
    W[wslot] = px; W[T + wslot] = py; W[2 * T + wslot] = pc;
    reinterpret_cast<int *>(W + 3 * T)[wslot] = consec;
    const unsigned ndone = __popc(__ballot_sync(0xffffffffu, remaining == 0 && fuse_left == 0));
    __syncwarp();
    if (lane == 0) {
      if (ndone) atomicAdd(&xc.done[round & 3], (int)ndone);
      mbar_arrive(&xc.bar[cur]);
    }
    px = nx_; py = ny_; pc = nc_; consec = nq_;
#if F3G_AGG == 1
    if (!(agg_state & 64) && (agg_state & 7) < 4 && (round & 7) == 7) {
      const int b = bucket_of(s, px, py);
      const unsigned peers = __match_any_sync(0xffffffffu, b < 0 ? -1 - lane : b);
      const unsigned shared = __ballot_sync(0xffffffffu, __popc(peers) > 1);
      agg_state += 1 + (__popc(shared) >= F3G_AGG_LANES ? 8 : 0);
      if ((agg_state & 7) == 4 && ((agg_state >> 3) & 7) >= 2) agg_state |= 64;
    }
#endif
  }
  (void)po;
  bad_total += bad;
  return ok_all;
}

/* occupancy target: 4 blocks of 256 threads per SM for FP32 iteration (64
 * registers; measured 10 % faster than 3 blocks at 80 registers despite a
 * few spilled bytes), 2 for FP64 */
#ifndef F3G_ITER_MIN_BLOCKS
#define F3G_ITER_MIN_BLOCKS 4
#endif
template <typename R> struct IterMinBlocks { static const int v = F3G_ITER_MIN_BLOCKS; };
template <> struct IterMinBlocks<double> { static const int v = 2; };

/* add this block's bad-value and plotted counts to the pass's counters */
__device__ __forceinline__ void flush_counts(unsigned long long *counters, unsigned &bad, unsigned &hits) {
  unsigned long long b = bad, h = hits;
  for (int o = 16; o > 0; o >>= 1) {
    b += __shfl_down_sync(0xffffffffu, b, o);
    h += __shfl_down_sync(0xffffffffu, h, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (b) atomicAdd(&counters[0], b);
    if (h) atomicAdd(&counters[1], h);
  }
  bad = hits = 0;
}

template <typename R, bool FULL, int MODE>
__global__ void __launch_bounds__(256, IterMinBlocks<R>::v) k_iterate(const F3GItem *__restrict__ items,
                                                 const long long *__restrict__ chunk_prefix, int nitems,
                                                 long long total_chunks, int shuffle_every, F3GCounters *ctr) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  PassS<R> &s = *reinterpret_cast<PassS<R> *>(smem_raw);
  ShufPoint<R> *buf = reinterpret_cast<ShufPoint<R> *>(smem_raw + ((sizeof(PassS<R>) + 15) & ~(size_t)15));
  __shared__ long long sh_chunk;
  __shared__ int sh_item;
#if F3G_EXCHANGE == 1
  __shared__ Exchange xc;
  __shared__ unsigned long long sh_stall; /* the stall test: 1 + the chunk that withholds, or 0 */
  unsigned ph = 0; /* phase parities of xc.bar[0..1] */
  if (MODE == 1 && threadIdx.x == 0) {
    mbar_init(&xc.bar[0], blockDim.x >> 5);
    mbar_init(&xc.bar[1], blockDim.x >> 5);
    xc.abort = 0;
    sh_stall = ctr->test_stall;
  }
#endif
  int cur = -1;
  long long first = 0;
  unsigned bad = 0, hits = 0;
  for (;;) {
    if (threadIdx.x == 0) {
#if F3G_EXCHANGE == 1
      xc.done[0] = xc.done[1] = xc.done[2] = xc.done[3] = 0;
#endif
      long long g = (long long)atomicAdd(&ctr->next_chunk, 1ull);
      int p = cur;
      if (g < total_chunks) {
        if (p < 0 || g < chunk_prefix[p] || g >= chunk_prefix[p + 1]) {
          int lo = 0, hi = nitems - 1;
          while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (chunk_prefix[mid] <= g) lo = mid;
            else hi = mid - 1;
          }
          p = lo;
        }
        /* the chunk's random streams: pass key, chunk index within the pass */
        const F3GPass *ps = items[p].pass;
        f3g_chunk_ctx[0] = ps->key[0];
        f3g_chunk_ctx[1] = ps->key[1];
        f3g_chunk_ctx[2] = (uint32_t)(g - chunk_prefix[p] + items[p].chunk_first);
      }
      sh_chunk = g;
      sh_item = p;
    }
    __syncthreads();
    long long g = sh_chunk;
    int p = sh_item;
    if (g >= total_chunks) break;
    if (p != cur) {
      if (cur >= 0) flush_counts(s.counters, bad, hits);
      __syncthreads();
      stage_pass<R>(s, items[p].pass);
      first = items[p].chunk_first;
      cur = p;
      __syncthreads();
    }
    long long local = g - chunk_prefix[p] + first;
    /* the chunk's samples: blockDim*S each up to chunk_tail, blockDim*S_tail after */
    const long long TT = blockDim.x;
    long long base, len;
    if (local < s.chunk_tail) {
      base = local * TT * s.S;
      len = TT * s.S;
    } else {
      base = s.chunk_tail * TT * s.S + (local - s.chunk_tail) * TT * s.S_tail;
      len = TT * s.S_tail;
    }
#if F3G_EXCHANGE == 1
    if (MODE == 1)
      (void)run_chunk_warp_lag<R, FULL>(s, buf, xc, ph, local, base, len, shuffle_every,
                                        sh_stall != 0 && (unsigned long long)g == sh_stall - 1, bad, hits);
#else
    if (MODE == 1) run_chunk_warp<R, FULL>(s, buf, local, base, len, shuffle_every, bad, hits);
#endif
    else run_chunk_thread<R, FULL>(s, local, base, len, bad, hits);
    __syncthreads();
#if F3G_EXCHANGE == 1
    if (MODE == 1 && xc.abort) {
      /* an exchange wait timed out: report it and stop this block */
      if (threadIdx.x == 0) atomicExch(&ctr->error, 1ull);
      break;
    }
#endif
  }
  if (cur >= 0) flush_counts(s.counters, bad, hits);
}

/* pass + the exchange buffers of mode 1 (two rounds of points) */
template <typename R> static size_t iterate_smem(int threads) {
  return ((sizeof(PassS<R>) + 15) & ~(size_t)15) + 2 * sizeof(ShufPoint<R>) * (size_t)threads;
}

template <typename R, bool FULL, int MODE>
static cudaError_t launch_iterate_t(const F3GItem *d_items, const long long *d_prefix, int nitems,
                                    long long total_chunks, int shuffle_every, int threads, int blocks,
                                    F3GCounters *d_ctr, cudaStream_t st) {
  size_t smem = iterate_smem<R>(threads);
  cudaError_t e =
      cudaFuncSetAttribute(k_iterate<R, FULL, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_iterate<R, FULL, MODE><<<blocks, threads, smem, st>>>(d_items, d_prefix, nitems, total_chunks, shuffle_every,
                                                          d_ctr);
  return cudaGetLastError();
}

}  // namespace f3g

/* ---------------------------------------------------------------------
 * Parity probes: apply_xform on given points/words, accumulation of a given
 * point stream, and chains with recorded output.  One block stages the pass;
 * grids are small (test sizes).
 * ------------------------------------------------------------------- */
namespace f3g {

template <typename R, bool FULL>
__global__ void __launch_bounds__(256) k_apply_xform(const F3GPass *__restrict__ pass, int fn, int n,
                                                     const double *__restrict__ pin,
                                                     const uint32_t *__restrict__ words, int wpp, double *qout,
                                                     int *bad) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  PassS<R> &s = *reinterpret_cast<PassS<R> *>(smem_raw);
  stage_pass<R>(s, pass);
  __syncthreads();
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    ArrayRng rng{words + (size_t)k * wpp, wpp, 0};
    R qx, qy, qc, qo;
    bool b = apply_xform<R, FULL, ArrayRng>(s.xf[fn], s.var_id, s.var_w, (R)pin[4 * k], (R)pin[4 * k + 1],
                                            (R)pin[4 * k + 2], qx, qy, qc, qo, rng);
    qout[4 * k] = (double)qx;
    qout[4 * k + 1] = (double)qy;
    qout[4 * k + 2] = (double)qc;
    qout[4 * k + 3] = (double)qo;
    bad[k] = b ? 1 : 0;
  }
}

/* xform choice of every 14-bit value of every row of a pass's choice table
 * (the iterate kernel's pick_xform), for comparison with the reference's
 * 16384-entry rows (flam3.c:76-111, 165-224) */
static __global__ void __launch_bounds__(256) k_xform_choice(const F3GPass *__restrict__ pass, int rows,
                                                      uint16_t *out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  PassS<float> &s = *reinterpret_cast<PassS<float> *>(smem_raw);
  stage_pass<float>(s, pass);
  __syncthreads();
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < rows * F3G_GRAIN; k += gridDim.x * blockDim.x)
    out[k] = (uint16_t)pick_xform<float>(s, k / F3G_GRAIN, (uint32_t)(k % F3G_GRAIN));
}

static __global__ void __launch_bounds__(256) k_accumulate(const F3GPass *__restrict__ pass, const double *__restrict__ pts,
                                                    long long n) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  PassS<double> &s = *reinterpret_cast<PassS<double> *>(smem_raw);
  stage_pass<double>(s, pass);
  __syncthreads();
  /* warp-aggregated accumulation, so the parity tests cover the shuffle sums */
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    (void)plot<double>(s, pts[4 * k], pts[4 * k + 1], pts[4 * k + 2], pts[4 * k + 3], true);
}

template <typename R, bool FULL>
__global__ void __launch_bounds__(256) k_iterate_chains(const F3GPass *__restrict__ pass, int nchains, int n,
                                                        int fuse, const double *__restrict__ starts, uint32_t key0,
                                                        uint32_t key1, double *samples, unsigned long long *bad_out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  PassS<R> &s = *reinterpret_cast<PassS<R> *>(smem_raw);
  stage_pass<R>(s, pass);
  __syncthreads();
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nchains) return;
  Rng rng;
  rng.init(key0, key1, (uint32_t)c, 0u, 0xC4A1u);
  R px = (R)starts[4 * c], py = (R)starts[4 * c + 1], pc = (R)starts[4 * c + 2], po = (R)starts[4 * c + 3];
  int consec = 0, lastxf = 0;
  unsigned bad = 0;
  for (int i = -fuse; i < n;) {
    int row = s.chaos_enable ? min(lastxf, s.num_std) : 0;
    int fn = pick_xform(s, row, rng.word() & (F3G_GRAIN - 1));
    R qx, qy, qc, qo;
    if (!chain_step<R, FULL, Rng>(s, fn, px, py, pc, po, consec, lastxf, bad, qx, qy, qc, qo, rng)) continue;
    if (i >= 0) {
      double *o = samples + ((size_t)c * n + i) * 4;
      o[0] = (double)qx; o[1] = (double)qy; o[2] = (double)qc; o[3] = (double)qo;
    }
    i++;
  }
  atomicAdd(bad_out, (unsigned long long)bad);
}

}  // namespace f3g


#endif
