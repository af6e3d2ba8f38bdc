/*
 * Stand-ins for the reference's PNG/JPEG writers and readers (png.c, jpeg.c),
 * whose libpng/libjpeg headers are not installed in this image.  The oracle
 * build of flam3-render/flam3-animate is only ever run with format=ppm, so
 * these report an error if reached.  Test infrastructure only.
 */
#include <stdio.h>
#include <stdlib.h>

typedef struct flam3_img_comments_s flam3_img_comments;

void write_png(FILE *file, void *image, int width, int height, flam3_img_comments *fpc, int bpc) {
  (void)file; (void)image; (void)width; (void)height; (void)fpc; (void)bpc;
  fprintf(stderr, "oracle build: PNG output is not available, use format=ppm\n");
}

void write_jpeg(FILE *file, unsigned char *image, int width, int height, flam3_img_comments *fpc) {
  (void)file; (void)image; (void)width; (void)height; (void)fpc;
  fprintf(stderr, "oracle build: JPEG output is not available, use format=ppm\n");
}

unsigned char *read_png(FILE *file, int *width, int *height) {
  (void)file; (void)width; (void)height;
  return NULL;
}

unsigned char *read_jpeg(FILE *file, int *width, int *height) {
  (void)file; (void)width; (void)height;
  return NULL;
}
