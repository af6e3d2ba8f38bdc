/*
 * f3g_strip_f64.cu -- separable strip kernels for FP64 histograms, tonemap after the filter.
 */
#include "f3g_strip.cuh"

#define F3G_STRIP_OCC(SSV, FWV) strip_occupancy<SSV, FWV, true, false>();
#define F3G_STRIP_CASE(SSV, FWV)                                                                              \
  if (oversample == SSV && fw == FWV)                                                                         \
    return launch_strip<SSV, FWV, true, false>(buckets, W, H, k1, k2, de_offset, filter, image_w, image_h, out, tp, \
                                        st);

F3G_STRIP_ENTRIES(f64, true, false)
