/*
 * f3g_choice.h -- the breakpoints of one xform-choice row without its
 * 16384-step loop.
 *
 * The reference builds each row (flam3.c:165-224) by walking r from 0 in
 * F3G_GRAIN steps of r = fl(r + dr) and, at each step i, advancing the xform
 * index j while r >= t_j (t_j the running sum of the weights).  The row is
 * nondecreasing, so it is stored as breakpoints: the first step at which
 * r_i >= t_j, once per j.  The loop is a chain of 16384 dependent FP64 adds,
 * which is slow on a GPU thread; this walk gives the same breakpoints exactly
 * in a few dozen operations.
 *
 * Inside one binade [2^e, 2^(e+1)) every double is an integer multiple R of
 * u = 2^(e-52), so fl(r + dr) = (R + rn(dr/u)) u as long as the exact sum stays
 * below 2^(e+1): each step adds the same number D of ulps (round to nearest;
 * at an exact tie the result is the even neighbour, and from an even R every
 * tie step adds D = m or m + 1, whichever is even).  So the values of a run of
 * K steps are R + k D, K follows from R, D and the binade's end, and the
 * first step of the run that reaches a threshold t (also a multiple of u
 * there) is ceil((t/u - R) / D).  The step that leaves the binade, steps from
 * r = 0 and from an odd R at a tie are taken as real FP64 adds.  Everything
 * else is 64-bit integer arithmetic on the doubles' significands, identical on
 * the host and the device.
 *
 * Used by the device planner; the host planner keeps the reference's loop,
 * and a test compares the two on the host over random and tie-heavy weights.
 */
#ifndef F3G_CHOICE_H
#define F3G_CHOICE_H

#include <stdint.h>

#ifdef __CUDACC__
#define F3G_CH_HD __host__ __device__ __forceinline__
#else
#include <string.h>
#define F3G_CH_HD static inline
#endif

#define F3G_CH_GRAIN 16384

F3G_CH_HD uint64_t f3g_ch_bits(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t b;
  memcpy(&b, &x, sizeof(b));
  return b;
#endif
}

/* a + b and a * b, each rounded once (no contraction into an FMA) */
F3G_CH_HD double f3g_ch_add(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dadd_rn(a, b);
#else
  volatile double s = a + b;
  return s;
#endif
}

F3G_CH_HD double f3g_ch_mul(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dmul_rn(a, b);
#else
  volatile double p = a * b;
  return p;
#endif
}

/* the next threshold t_j = t_(j-1) + d_j (* c_j): the raw-weight row sums
 * every xform's weight, a chaos row weights the standard xforms by the row's
 * chaos entries and the final xform by 0 */
F3G_CH_HD double f3g_ch_next(double t, const double *d, const double *c, int nstd, int j) {
  if (c) return f3g_ch_add(t, f3g_ch_mul(d[j], j < nstd ? c[j] : 0.0));
  return f3g_ch_add(t, d[j]);
}

/* Breakpoints of the row with step dr (> 0) and weights d[0..nx) (times
 * c[0..nstd) for a chaos row, c NULL for the raw row) into brk[0..maxb);
 * *nbrk gets their count, *moves (if not NULL) the number of real steps and
 * runs the walk took.  Returns 0, or 2 if the walk runs past the last xform
 * (the reference would read beyond its xform array). */
F3G_CH_HD int f3g_choice_breakpoints(double dr, const double *d, const double *c, int nstd, int nx, uint16_t *brk,
                                     int maxb, int *nbrk, int *moves) {
  const int64_t TOP = (int64_t)1 << 53; /* 2^(e+1) / u */
  int nb = 0, j = 0;
  double t = c ? f3g_ch_mul(d[0], c[0]) : d[0];
  double r = 0.0;
  int i = 0, nmoves = 0;
  for (;;) {
    /* thresholds reached at step i */
    while (r >= t) {
      if (nb < maxb) brk[nb++] = (uint16_t)i;
      j++;
      if (j >= nx) {
        *nbrk = nb;
        if (moves) *moves = nmoves;
        return 2;
      }
      t = f3g_ch_next(t, d, c, nstd, j);
    }
    if (i == F3G_CH_GRAIN - 1) break;
    /* a run of steps inside r's binade */
    int64_t K = 0, R = 0, D = 0;
    int e = 0;
    if (r > 0.0) {
      const uint64_t rb = f3g_ch_bits(r), db = f3g_ch_bits(dr);
      const int er = (int)((rb >> 52) & 0x7ff), ed = (int)((db >> 52) & 0x7ff);
      if (er > 0 && er < 0x7ff && ed > 0 && ed < er) {
        const int s = er - ed; /* dr = Md 2^(ed-1075), u = 2^(er-1075) */
        R = (int64_t)((rb & (((uint64_t)1 << 52) - 1)) | ((uint64_t)1 << 52));
        const int64_t Md = (int64_t)((db & (((uint64_t)1 << 52) - 1)) | ((uint64_t)1 << 52));
        int64_t m;
        int cmp; /* the fraction of dr/u against one half */
        if (s >= 62) {
          m = 0;
          cmp = -1;
        } else {
          m = Md >> s;
          const int64_t rem = Md & (((int64_t)1 << s) - 1), half = (int64_t)1 << (s - 1);
          cmp = rem < half ? -1 : (rem > half ? 1 : 0);
        }
        if (cmp < 0) D = m;
        else if (cmp > 0) D = m + 1;
        else if ((R & 1) == 0) D = (m & 1) ? m + 1 : m;
        else D = -1; /* a tie from an odd R: one real step */
        if (D >= 0) {
          const int64_t room = TOP - 1 - m - R; /* the sum before each run step stays below 2^(e+1) */
          const int64_t left = F3G_CH_GRAIN - 1 - i;
          if (room >= 0) K = D > 0 ? room / D + 1 : left;
          if (K > left) K = left;
          e = er;
        }
      }
    }
    nmoves++;
    if (K > 0) {
      const int64_t Rend = R + K * D;
      /* thresholds reached inside the run: a threshold in (r, r_end] is a
       * multiple of u in this binade (or 2^(e+1) itself); one at or below r
       * (after a negative weight) is reached at the step that reached the
       * threshold before it, as the loop's while does */
      int64_t kprev = 1;
      for (;;) {
        if (t != t) break; /* a NaN threshold is never reached */
        int64_t k = kprev;
        if (t > r) {
          const uint64_t tb = f3g_ch_bits(t);
          const int et = (int)((tb >> 52) & 0x7ff);
          int64_t T;
          if (et == e) T = (int64_t)((tb & (((uint64_t)1 << 52) - 1)) | ((uint64_t)1 << 52));
          else if (et == e + 1 && (tb & (((uint64_t)1 << 52) - 1)) == 0) T = TOP;
          else break; /* beyond the run */
          if (T > Rend) break;
          const int64_t kt = (T - R + D - 1) / D; /* D > 0 whenever a threshold is inside the run */
          if (kt > k) k = kt;
        }
        kprev = k;
        if (nb < maxb) brk[nb++] = (uint16_t)(i + k);
        j++;
        if (j >= nx) {
          *nbrk = nb;
          if (moves) *moves = nmoves;
          return 2;
        }
        t = f3g_ch_next(t, d, c, nstd, j);
      }
      i += (int)K;
      /* r = Rend u, rebuilt from its bits (Rend <= 2^53) */
      if (Rend == TOP) {
        const uint64_t nbits = (uint64_t)(e + 1) << 52;
#ifdef __CUDA_ARCH__
        r = __longlong_as_double((long long)nbits);
#else
        memcpy(&r, &nbits, sizeof(r));
#endif
      } else {
        const uint64_t nbits = ((uint64_t)e << 52) | ((uint64_t)Rend & (((uint64_t)1 << 52) - 1));
#ifdef __CUDA_ARCH__
        r = __longlong_as_double((long long)nbits);
#else
        memcpy(&r, &nbits, sizeof(r));
#endif
      }
      continue;
    }
    r = f3g_ch_add(r, dr);
    i++;
  }
  *nbrk = nb;
  if (moves) *moves = nmoves;
  return 0;
}

#endif
