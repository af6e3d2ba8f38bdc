/*
 * f3g_strip_acc.cu -- separable strip kernels over an FP32 accumulator that
 * density estimation has filled (no log scaling here): filter + tonemap +
 * pack, earlyclip off (suffix acc) and on (acce).
 */
#include "f3g_strip.cuh"

#define F3G_STRIP_OCC(SSV, FWV) strip_occupancy<SSV, FWV, false, false, false>();
#define F3G_STRIP_CASE(SSV, FWV)                                                                              \
  if (oversample == SSV && fw == FWV)                                                                         \
    return launch_strip<SSV, FWV, false, false, false>(buckets, W, H, k1, k2, de_offset, filter, image_w, image_h, \
                                                       out, tp, st);
F3G_STRIP_ENTRIES(acc, false, false)
#undef F3G_STRIP_OCC
#undef F3G_STRIP_CASE

#define F3G_STRIP_OCC(SSV, FWV) strip_occupancy<SSV, FWV, false, true, false>();
#define F3G_STRIP_CASE(SSV, FWV)                                                                              \
  if (oversample == SSV && fw == FWV)                                                                         \
    return launch_strip<SSV, FWV, false, true, false>(buckets, W, H, k1, k2, de_offset, filter, image_w, image_h, \
                                                      out, tp, st);
F3G_STRIP_ENTRIES(acce, false, true)
