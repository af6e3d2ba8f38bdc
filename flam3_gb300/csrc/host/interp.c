/*
 * interp.c -- genome interpolation between several control points
 * (flam3.c:717-802, interpolation.c:373-709).
 */
#include "f3g_host.h"

int f3g_interpolate_n(flam3_genome *cps, int ncps, double time, flam3_genome *result) {
  (void)cps; (void)time; (void)result;
  f3g_set_error("interpolation between %d genomes is not available in this build", ncps);
  return 1;
}
