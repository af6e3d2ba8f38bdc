/*
 * f3g_common.h -- data layout shared by the host driver (C) and the CUDA
 * kernels of libflam3gpu.
 *
 * A "pass" is one temporal sample of one render batch: the genome
 * interpolated at that time, prepared (active-variation lists, precalc
 * values, xform-choice table), its colour map scaled by the temporal filter
 * weight, the camera, the number of samples and the histogram it adds to.
 * The iterate kernel processes any list of passes (of any number of renders)
 * in one persistent launch: work is split into chunks of blockDim*S samples,
 * a block takes chunks from a global counter and stages the pass it belongs
 * to in shared memory.
 */
#ifndef F3G_COMMON_H
#define F3G_COMMON_H

#include <stddef.h>
#include <stdint.h>

#define F3G_MAX_XFORMS 32      /* standard + final xforms of one genome */
#define F3G_MAX_VARLIST 384    /* active variations summed over a genome's xforms */
#define F3G_NVARS 99
#define F3G_GRAIN 16384        /* flam3.c:70 CHOOSE_XFORM_GRAIN */
#define F3G_EPS 1e-10          /* private.h:47 */

/* Variation parameters and xform_precalc values, in flam3_xform order
 * (flam3.h:240-441).  The host copies them by name; kernels index them. */
#define F3G_PARAM_LIST(X)                                                                          \
  X(blob_low) X(blob_high) X(blob_waves) X(pdj_a) X(pdj_b) X(pdj_c) X(pdj_d) X(fan2_x) X(fan2_y)   \
  X(rings2_val) X(perspective_angle) X(perspective_dist) X(julian_power) X(julian_dist)            \
  X(juliascope_power) X(juliascope_dist) X(radial_blur_angle) X(pie_slices) X(pie_rotation)        \
  X(pie_thickness) X(ngon_sides) X(ngon_power) X(ngon_circle) X(ngon_corners) X(curl_c1)           \
  X(curl_c2) X(rectangles_x) X(rectangles_y) X(amw_amp) X(disc2_rot) X(disc2_twist)               \
  X(super_shape_rnd) X(super_shape_m) X(super_shape_n1) X(super_shape_n2) X(super_shape_n3)        \
  X(super_shape_holes) X(flower_petals) X(flower_holes) X(conic_eccentricity) X(conic_holes)       \
  X(parabola_height) X(parabola_width) X(bent2_x) X(bent2_y) X(bipolar_shift) X(cell_size)         \
  X(cpow_r) X(cpow_i) X(cpow_power) X(curve_xamp) X(curve_yamp) X(curve_xlength) X(curve_ylength)  \
  X(escher_beta) X(lazysusan_spin) X(lazysusan_space) X(lazysusan_twist) X(lazysusan_x)            \
  X(lazysusan_y) X(modulus_x) X(modulus_y) X(oscope_separation) X(oscope_frequency)                \
  X(oscope_amplitude) X(oscope_damping) X(popcorn2_x) X(popcorn2_y) X(popcorn2_c) X(separation_x)  \
  X(separation_xinside) X(separation_y) X(separation_yinside) X(split_xsize) X(split_ysize)        \
  X(splits_x) X(splits_y) X(stripes_space) X(stripes_warp) X(wedge_angle) X(wedge_hole)            \
  X(wedge_count) X(wedge_swirl) X(wedge_julia_angle) X(wedge_julia_count) X(wedge_julia_power)     \
  X(wedge_julia_dist) X(wedge_sph_angle) X(wedge_sph_count) X(wedge_sph_hole) X(wedge_sph_swirl)   \
  X(whorl_inside) X(whorl_outside) X(waves2_freqx) X(waves2_scalex) X(waves2_freqy)                \
  X(waves2_scaley) X(auger_sym) X(auger_weight) X(auger_freq) X(auger_scale) X(flux_spread)        \
  X(mobius_re_a) X(mobius_im_a) X(mobius_re_b) X(mobius_im_b) X(mobius_re_c) X(mobius_im_c)        \
  X(mobius_re_d) X(mobius_im_d) X(persp_vsin) X(persp_vfcos) X(julian_rN) X(julian_cn)             \
  X(juliascope_rN) X(juliascope_cn) X(wedgeJulia_rN) X(wedgeJulia_cn) X(wedgeJulia_cf)             \
  X(radialBlur_spinvar) X(radialBlur_zoomvar) X(waves_dx2) X(waves_dy2) X(disc2_sinadd)            \
  X(disc2_cosadd) X(disc2_timespi) X(super_shape_pm_4) X(super_shape_pneg1_n1)

enum {
#define F3G_X(n) PRM_##n,
  F3G_PARAM_LIST(F3G_X)
#undef F3G_X
  PRM_COUNT
};

/* precalc flags (variations.c:2036-2115) */
#define F3G_F_ATAN_XY 1
#define F3G_F_ANGLES 2
#define F3G_F_ATAN_YX 4
#define F3G_F_POST 8
#define F3G_F_PREBLUR 16

/* One prepared xform (values in FP64 here; kernels stage them in the
 * iteration precision). */
typedef struct {
  double c[6];      /* c[0][0] c[0][1] c[1][0] c[1][1] c[2][0] c[2][1] */
  double post[6];
  double color, color_speed, vis_adjusted, opacity;
  double preblur;   /* has_preblur weight */
  int flags;
  int var_off, nvars; /* into PassDesc.var_id / var_w */
  int pad;
  double prm[PRM_COUNT];
} F3GXform;

/* Bucket layouts on the device (all channel-last, one bucket per pixel):
 *   F3G_BK_F32: float4 (R,G,B,A)               bits 32/33
 *   F3G_BK_F64: double4 (R,G,B,A)              bits 64
 * plus an optional count plane (float or double) holding the reference's
 * fifth channel (255*opacity per hit) when it can differ from A. */
#define F3G_BK_F32 0
#define F3G_BK_F64 1

typedef struct {
  /* --- work ---------------------------------------------------------- */
  int64_t samples;          /* samples this pass adds */
  int64_t chunk_begin;      /* first global chunk index of this pass */
  int64_t nchunks;
  uint32_t key[2];          /* Philox key of the pass */
  int fuse;                 /* 15, or 100 with earlyclip (rect.c:36-37, 266) */
  int iter_mode;            /* 0 per-thread choice, 1 warp-coherent choice */
  /* --- genome -------------------------------------------------------- */
  int num_xforms, num_std, final_index, final_enable, chaos_enable;
  int full_variations;      /* uses variations beyond 0-19 */
  /* xform-choice table compressed to breakpoints: for row r (0 = raw
   * weights, 1+i = after xform i when xaos is on), the xform chosen for a
   * random 14-bit value v is the number of entries in brk[r] that are <= v. */
  uint16_t nbrk[F3G_MAX_XFORMS + 1];
  uint16_t brk[F3G_MAX_XFORMS + 1][F3G_MAX_XFORMS];
  uint8_t var_id[F3G_MAX_VARLIST];
  double var_w[F3G_MAX_VARLIST];
  /* --- colour -------------------------------------------------------- */
  float dmap[256][4];       /* palette * 255 * color_scalar (rect.c:778-782) */
  int cmap_size;            /* 256 - apo_palette */
  int palette_mode;         /* 0 step, 1 linear */
  int trunc_hits;           /* integer buckets (bits 32/33): each hit's channels truncated (flam3.c:3688-3703) */
  /* --- camera (rect.c:785-827) ---------------------------------------- */
  double bounds[4];
  double rot[2][2];
  double rot_center[2];
  int rotate;               /* cp.rotate != 0 */
  int width, height;        /* histogram incl. gutter */
  double ws0, wb0s0, hs1, hb1s1;
  /* --- output -------------------------------------------------------- */
  void *buckets;
  void *count;              /* optional count plane, NULL if A == count */
  int bucket_kind;
  int S;                    /* samples per thread per chunk: a chunk is blockDim*S samples, */
  int S_tail;               /* except chunks chunk_tail.. of the pass, which hold blockDim*S_tail */
  int64_t chunk_tail;       /* (0 < S_tail <= S; S_tail 0: every chunk holds blockDim*S) */
  unsigned long long *counters; /* [0] bad values, [1] samples plotted (device) */
  /* --- xforms last: a pass is uploaded up to its last used xform ------ */
  F3GXform xf[F3G_MAX_XFORMS];
} F3GPass;

/* bytes of a pass that hold data when its genome has nx xforms */
#define F3G_PASS_BYTES(nx) (offsetof(F3GPass, xf) + (size_t)(nx) * sizeof(F3GXform))

/* The spatial filter as uploaded: the fw x fw filter (index i + j*fw, i
 * horizontal) followed by its vertical factor fu[fw] and horizontal factor
 * fv[fw], with filter[i + j*fw] == fu[j] * fv[i]. */
#define F3G_FILTER_FLOATS(fw) ((size_t)(fw) * (size_t)(fw) + 2 * (size_t)(fw))

/* One entry of an iterate launch's work list: chunks [chunk_first,
 * chunk_first + n) of a pass, where n is the entry's span in the launch's
 * chunk prefix.  Chunk k of a pass always draws the same random stream, so a
 * pass may be split over several launches (rounds of a batched or served
 * workload) without changing its samples. */
typedef struct {
  const F3GPass *pass;
  long long chunk_first;
} F3GItem;

/* Device result counters of one iterate launch. */
typedef struct {
  unsigned long long next_chunk;  /* work counter */
  unsigned long long badvals;     /* bad values and samples plotted, when a */
  unsigned long long plotted;     /* pass's counters point here */
  unsigned long long error;       /* nonzero: a kernel refused its input */
  unsigned long long test_stall;  /* input, tests only: 1 + c makes the block that runs chunk c withhold
                                     one exchange arrival, so its waits run out (2 s); 0: off */
} F3GCounters;

#endif
