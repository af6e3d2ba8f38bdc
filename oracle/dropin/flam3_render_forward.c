/*
 * flam3_render_forward.c -- the drop-in binding on the reference's side: a
 * libflam3 whose flam3_render and flam3_render_memory_required
 * (flam3.h:623, 625; flam3.c:3874-3932) hand the call to libflam3gpu.
 *
 * Test infrastructure: `make -C oracle dropin REF=<reference tree>` compiles
 * the reference's library sources unmodified, with its own flam3_render
 * renamed at compile time (-Dflam3_render=flam3_render_cpu), links this file
 * in its place, and links the reference's unmodified flam3-render.c and
 * flam3-animate.c against the result and libflam3gpu.so.  Every
 * flam3_render call of those programs (flam3-render.c:345,
 * flam3-animate.c:234,239,248) then runs on the GPU; the library's other
 * callers (palettes.c:408) take the same route.
 *
 * The structs are the reference's (flam3.h); libflam3gpu's ABI mirror has
 * the same layout, so the pointers pass through unchanged.
 */
#include "flam3.h"

extern int flam3gpu_render(flam3_frame *f, void *out, int field, int nchan, int transp, stat_struct *stats);
extern double flam3gpu_render_memory_required(flam3_frame *f);

int flam3_render(flam3_frame *f, void *out, int field, int nchan, int transp, stat_struct *stats) {
  return flam3gpu_render(f, out, field, nchan, transp, stats);
}

double flam3_render_memory_required(flam3_frame *f) { return flam3gpu_render_memory_required(f); }
