/*
 * Prints sizeof/offsetof for the public flam3 structs.  Built twice: against
 * the reference header (-DF3_ABI_REFERENCE, oracle/_ref/abi_offsets) and
 * against include/flam3_gpu.h; tests compare the two outputs and the Python
 * mirror in flam3_gb300/abi.py.  Test infrastructure only.
 */
#include <stddef.h>
#include <stdio.h>
#ifdef F3_ABI_REFERENCE
#include "flam3.h"
#else
#include "flam3_gpu.h"
#endif

#define S(t) printf("sizeof %s %zu\n", #t, sizeof(t))
#define O(t, f) printf("offset %s.%s %zu\n", #t, #f, offsetof(t, f))

int main(void) {
  S(randctx); S(flam3_palette_entry); S(stat_struct); S(flam3_xform); S(flam3_genome); S(flam3_frame);
  O(randctx, randrsl); O(randctx, randmem); O(randctx, randc);
  O(stat_struct, num_iters); O(stat_struct, render_seconds);
  O(flam3_xform, c); O(flam3_xform, post); O(flam3_xform, density); O(flam3_xform, vis_adjusted);
  O(flam3_xform, padding); O(flam3_xform, wind); O(flam3_xform, precalc_angles_flag);
  O(flam3_xform, has_preblur); O(flam3_xform, has_post); O(flam3_xform, blob_low);
  O(flam3_xform, amw_amp); O(flam3_xform, super_shape_holes); O(flam3_xform, cpow_power);
  O(flam3_xform, lazysusan_y); O(flam3_xform, wedge_sph_swirl); O(flam3_xform, mobius_im_d);
  O(flam3_xform, persp_vsin); O(flam3_xform, wedgeJulia_cf); O(flam3_xform, super_shape_pneg1_n1);
  O(flam3_xform, num_active_vars); O(flam3_xform, active_var_weights); O(flam3_xform, varFunc);
  O(flam3_xform, motion_freq); O(flam3_xform, motion); O(flam3_xform, num_motion);
  O(flam3_genome, time); O(flam3_genome, interpolation); O(flam3_genome, hsv_rgb_palette_blend);
  O(flam3_genome, num_xforms); O(flam3_genome, xform); O(flam3_genome, chaos); O(flam3_genome, chaos_enable);
  O(flam3_genome, genome_index); O(flam3_genome, parent_fname); O(flam3_genome, symmetry);
  O(flam3_genome, palette); O(flam3_genome, input_image); O(flam3_genome, palette_index);
  O(flam3_genome, brightness); O(flam3_genome, highlight_power); O(flam3_genome, width);
  O(flam3_genome, spatial_oversample); O(flam3_genome, center); O(flam3_genome, rot_center);
  O(flam3_genome, rotate); O(flam3_genome, background); O(flam3_genome, zoom);
  O(flam3_genome, spatial_filter_radius); O(flam3_genome, spatial_filter_select);
  O(flam3_genome, sample_density); O(flam3_genome, nbatches); O(flam3_genome, ntemporal_samples);
  O(flam3_genome, estimator); O(flam3_genome, estimator_minimum); O(flam3_genome, edits);
  O(flam3_genome, gam_lin_thresh); O(flam3_genome, palette_index0); O(flam3_genome, hue_rotation1);
  O(flam3_genome, palette_blend); O(flam3_genome, temporal_filter_type); O(flam3_genome, temporal_filter_exp);
  O(flam3_genome, palette_mode);
  O(flam3_frame, genomes); O(flam3_frame, ngenomes); O(flam3_frame, bits); O(flam3_frame, earlyclip);
  O(flam3_frame, time); O(flam3_frame, progress); O(flam3_frame, progress_parameter); O(flam3_frame, rc);
  O(flam3_frame, nthreads); O(flam3_frame, sub_batch_size);
  return 0;
}
