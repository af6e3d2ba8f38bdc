/*
 * png.c -- PNG output on the device (write_png, png.c:36-116 of the
 * reference, which hands the image to libpng).  The pixels are filtered and
 * deflated by the kernels of f3g_png.cu into the IDAT chunks; this file
 * writes what surrounds them: the signature, IHDR (RGBA or RGB, 8 or 16 bits
 * per sample, no interlace), the text chunks write_png adds (png.c:48-78:
 * seven tEXt chunks and the genome as zTXt, all behind the
 * enable_png_comments switch), and IEND.
 *
 * The zTXt genome is a zlib stream of stored blocks: valid for every
 * reader, not compressed.  Text values that are NULL or empty are written
 * as empty tEXt chunks, as libpng does.
 */
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime.h>

#include "f3g_host.h"
#include "f3g_launch.h"
#include "flam3_gpu.h"
#include "flam3_gpu_service.h"

/* ---- chunk writing (host side, a few bytes) ---- */

static uint32_t crc_table[256];
static pthread_once_t crc_once = PTHREAD_ONCE_INIT;

static void crc_fill(void) {
  for (uint32_t i = 0; i < 256; i++) {
    uint32_t c = i;
    for (int k = 0; k < 8; k++) c = (c & 1u) ? (c >> 1) ^ 0xEDB88320u : c >> 1;
    crc_table[i] = c;
  }
}

/* concurrent writers from several host threads fill the table once */
static void crc_init(void) { pthread_once(&crc_once, crc_fill); }

static uint32_t crc_update(uint32_t c, const unsigned char *d, size_t n) {
  for (size_t i = 0; i < n; i++) c = crc_table[(c ^ d[i]) & 255u] ^ (c >> 8);
  return c;
}

typedef struct {
  unsigned char *p;
  size_t n, cap;
  int oom;
} buf_t;

static void buf_put(buf_t *b, const void *d, size_t n) {
  if (b->oom) return;
  if (b->n + n > b->cap) {
    size_t cap = b->cap ? b->cap : 4096;
    while (cap < b->n + n) cap *= 2;
    unsigned char *q = realloc(b->p, cap);
    if (!q) {
      b->oom = 1;
      return;
    }
    b->p = q;
    b->cap = cap;
  }
  if (n) memcpy(b->p + b->n, d, n);
  b->n += n;
}

static void put_be32(unsigned char *p, uint32_t v) {
  p[0] = (unsigned char)(v >> 24), p[1] = (unsigned char)(v >> 16), p[2] = (unsigned char)(v >> 8),
  p[3] = (unsigned char)v;
}

/* one chunk whose data is the concatenation of up to three parts */
static void put_chunk(buf_t *b, const char *type, const void *d1, size_t n1, const void *d2, size_t n2,
                      const void *d3, size_t n3) {
  unsigned char hdr[8];
  put_be32(hdr, (uint32_t)(n1 + n2 + n3));
  memcpy(hdr + 4, type, 4);
  buf_put(b, hdr, 8);
  buf_put(b, d1, n1);
  buf_put(b, d2, n2);
  buf_put(b, d3, n3);
  uint32_t c = crc_update(0xFFFFFFFFu, (const unsigned char *)type, 4);
  c = crc_update(c, d1, n1);
  c = crc_update(c, d2, n2);
  c = crc_update(c, d3, n3);
  unsigned char t[4];
  put_be32(t, c ^ 0xFFFFFFFFu);
  buf_put(b, t, 4);
}

/* zlib stream (RFC 1950) of stored deflate blocks */
static int zlib_stored(const unsigned char *d, size_t n, unsigned char **out, size_t *out_n) {
  const size_t nblk = n ? (n + 65534) / 65535 : 1;
  unsigned char *z = malloc(2 + nblk * 5 + n + 4);
  if (!z) return 1;
  size_t k = 0;
  z[k++] = 0x78, z[k++] = 0x01;
  size_t off = 0;
  for (size_t i = 0; i < nblk; i++) {
    const size_t len = n - off < 65535 ? n - off : 65535;
    z[k++] = (unsigned char)(i + 1 == nblk ? 1 : 0);
    z[k++] = (unsigned char)(len & 255), z[k++] = (unsigned char)(len >> 8);
    z[k++] = (unsigned char)(~len & 255), z[k++] = (unsigned char)((~len >> 8) & 255);
    memcpy(z + k, d + off, len);
    k += len;
    off += len;
  }
  uint32_t a = 1, bb = 0;
  for (size_t i = 0; i < n; i++) {
    a = (a + d[i]) % 65521u;
    bb = (bb + a) % 65521u;
  }
  put_be32(z + k, (bb << 16) | a);
  k += 4;
  *out = z;
  *out_n = k;
  return 0;
}

static void put_text(buf_t *b, const char *key, const char *text, int compressed) {
  static const unsigned char zero = 0;
  const size_t kl = strlen(key);
  const size_t tl = text ? strlen(text) : 0;
  if (!compressed || tl == 0) {
    put_chunk(b, "tEXt", key, kl, &zero, 1, text, tl);
    return;
  }
  unsigned char *z = NULL;
  size_t zn = 0;
  if (zlib_stored((const unsigned char *)text, tl, &z, &zn)) {
    b->oom = 1;
    return;
  }
  static const unsigned char kz[2] = {0, 0}; /* separator, compression method 0 */
  put_chunk(b, "zTXt", key, kl, kz, 2, z, zn);
  free(z);
}

/* ---- the device encode ---- */

static int ensure_png_buffers(f3g_ctx *c, int w, int h, int nchan, int bpc) {
  if (f3g_ensure(&c->d_png_work, &c->png_work_bytes, f3g_png_work_bytes(w, h, nchan, bpc))) return 1;
  if (f3g_ensure(&c->d_png_idat, &c->png_idat_bytes, f3g_png_idat_bound(w, h, nchan, bpc))) return 1;
  if (!c->d_png_len) {
    if (cudaMalloc((void **)&c->d_png_len, sizeof(unsigned long long)) != cudaSuccess) {
      f3g_set_error("cudaMalloc failed");
      return 1;
    }
    if (cudaMallocHost((void **)&c->h_png_len, sizeof(unsigned long long)) != cudaSuccess) {
      f3g_set_error("cudaMallocHost failed");
      return 1;
    }
  }
  return 0;
}

static int grow_pinned(f3g_ctx *c, size_t n) {
  if (n <= c->h_img_bytes && c->h_img) return 0;
  if (c->h_img) cudaFreeHost(c->h_img);
  c->h_img = NULL;
  c->h_img_bytes = 0;
  if (cudaMallocHost((void **)&c->h_img, n) != cudaSuccess) {
    f3g_set_error("cudaMallocHost of %zu bytes failed", n);
    return 1;
  }
  c->h_img_bytes = n;
  return 0;
}

#define CKP(x)                                                           \
  do {                                                                   \
    cudaError_t e_ = (x);                                                \
    if (e_ != cudaSuccess) {                                             \
      f3g_set_error("%s: %s", #x, cudaGetErrorString(e_));               \
      goto fail;                                                         \
    }                                                                    \
  } while (0)

/* Encodes the image at d_img (device) into a complete PNG in host memory. */
static int encode_device_image(f3g_ctx *c, const void *d_img, int w, int h, int nchan, int bpc,
                               const flam3gpu_png_text *text, int ntext, unsigned char **png, size_t *png_len,
                               double *kernel_ms) {
  buf_t b = {0};
  crc_init();
  if (ensure_png_buffers(c, w, h, nchan, bpc)) return 1;
  CKP(cudaEventRecord(c->ev[6], c->stream));
  if (f3g_png_encode_idat(d_img, w, h, nchan, bpc, c->d_png_work, c->d_png_idat, c->d_png_len, c->stream)) {
    f3g_set_error("PNG encode launch failed: %s", cudaGetErrorString(cudaGetLastError()));
    goto fail;
  }
  CKP(cudaEventRecord(c->ev[7], c->stream));
  CKP(cudaMemcpyAsync(c->h_png_len, c->d_png_len, sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->stream));
  /* the header chunks are built while the kernels run */
  static const unsigned char sig[8] = {0x89, 'P', 'N', 'G', 0x0d, 0x0a, 0x1a, 0x0a};
  buf_put(&b, sig, 8);
  unsigned char ihdr[13];
  put_be32(ihdr, (uint32_t)w);
  put_be32(ihdr + 4, (uint32_t)h);
  ihdr[8] = (unsigned char)(8 * bpc);
  ihdr[9] = nchan == 4 ? 6 : 2; /* RGBA / RGB */
  ihdr[10] = ihdr[11] = ihdr[12] = 0;
  put_chunk(&b, "IHDR", ihdr, 13, NULL, 0, NULL, 0);
  for (int i = 0; i < ntext; i++) put_text(&b, text[i].key, text[i].text, text[i].compressed);
  CKP(cudaStreamSynchronize(c->stream));
  const size_t n = (size_t)*c->h_png_len;
  if (n > f3g_png_idat_bound(w, h, nchan, bpc)) {
    f3g_set_error("PNG encode produced %zu bytes, more than its bound", n);
    goto fail;
  }
  if (grow_pinned(c, n)) goto fail;
  CKP(cudaMemcpyAsync(c->h_img, c->d_png_idat, n, cudaMemcpyDeviceToHost, c->stream));
  CKP(cudaStreamSynchronize(c->stream));
  if (kernel_ms) {
    float ms = 0;
    cudaEventElapsedTime(&ms, c->ev[6], c->ev[7]);
    *kernel_ms = ms;
  }
  buf_put(&b, c->h_img, n);
  put_chunk(&b, "IEND", NULL, 0, NULL, 0, NULL, 0);
  if (b.oom) {
    f3g_set_error("out of host memory");
    goto fail;
  }
  *png = b.p;
  *png_len = b.n;
  return 0;
fail:
  free(b.p);
  return 1;
}

static int check_image(int w, int h, int nchan, int bpc) {
  if (w <= 0 || h <= 0) {
    f3g_set_error("image size %d x %d", w, h);
    return 1;
  }
  if (nchan != 3 && nchan != 4) {
    f3g_set_error("nchan must be 3 or 4, not %d", nchan);
    return 1;
  }
  if (bpc != 1 && bpc != 2) {
    f3g_set_error("bytes per channel must be 1 or 2, not %d", bpc);
    return 1;
  }
  return 0;
}

static __thread double png_last_ms = 0; /* the calling thread's last encode, kernels only */

int flam3gpu_encode_png(const void *image, int image_on_device, int width, int height, int nchan, int bpc,
                        const flam3gpu_png_text *text, int ntext, unsigned char **png, size_t *png_len) {
  f3g_clear_error();
  if (!png || !png_len || !image) {
    f3g_set_error("NULL argument");
    return 1;
  }
  *png = NULL;
  *png_len = 0;
  if (check_image(width, height, nchan, bpc)) return 1;
  if (ntext < 0 || (ntext > 0 && !text)) {
    f3g_set_error("bad text chunk list");
    return 1;
  }
  for (int i = 0; i < ntext; i++) {
    const size_t kl = text[i].key ? strlen(text[i].key) : 0;
    if (kl < 1 || kl > 79) { /* PNG keywords are 1-79 bytes */
      f3g_set_error("text chunk %d: keyword must be 1-79 bytes", i);
      return 1;
    }
  }
  f3g_ctx *c = f3g_get_ctx();
  if (!c) {
    f3g_set_error("no CUDA device available");
    return 1;
  }
  const void *d_img = image;
  if (!image_on_device) {
    const size_t nb = (size_t)width * height * nchan * bpc;
    if (f3g_ensure(&c->d_png_img, &c->png_img_bytes, nb)) return 1;
    if (grow_pinned(c, nb)) return 1;
    memcpy(c->h_img, image, nb);
    if (cudaMemcpyAsync(c->d_png_img, c->h_img, nb, cudaMemcpyHostToDevice, c->stream) != cudaSuccess) {
      f3g_set_error("image upload failed");
      return 1;
    }
    d_img = c->d_png_img;
  }
  return encode_device_image(c, d_img, width, height, nchan, bpc, text, ntext, png, png_len, &png_last_ms);
}

/* the text chunks of write_png (png.c:48-78) */
static int comment_texts(const char *genome, const char *badvals, const char *numiters, const char *rtime,
                         flam3gpu_png_text *t) {
  const char *e = getenv("enable_png_comments");
  if (e && atoi(e) != 1) return 0;
  t[0] = (flam3gpu_png_text){"flam3_version", flam3gpu_version(), 0};
  t[1] = (flam3gpu_png_text){"flam3_nickname", getenv("nick"), 0};
  t[2] = (flam3gpu_png_text){"flam3_url", getenv("url"), 0};
  t[3] = (flam3gpu_png_text){"flam3_id", getenv("id"), 0};
  t[4] = (flam3gpu_png_text){"flam3_error_rate", badvals, 0};
  t[5] = (flam3gpu_png_text){"flam3_samples", numiters, 0};
  t[6] = (flam3gpu_png_text){"flam3_time", rtime, 0};
  t[7] = (flam3gpu_png_text){"flam3_genome", genome, 1};
  return 8;
}

int flam3gpu_write_png(FILE *file, void *image, int width, int height, flam3gpu_img_comments *fpc, int bpc) {
  flam3gpu_png_text t[8];
  const int nt = comment_texts(fpc ? fpc->genome : NULL, fpc ? fpc->badvals : NULL, fpc ? fpc->numiters : NULL,
                               fpc ? fpc->rtime : NULL, t);
  unsigned char *png = NULL;
  size_t n = 0;
  if (!file || flam3gpu_encode_png(image, 0, width, height, 4, bpc, t, nt, &png, &n)) {
    fprintf(stderr, "flam3gpu: writing file: %s\n", file ? flam3gpu_last_error() : "no file");
    return 1;
  }
  const int bad = fwrite(png, 1, n, file) != n;
  free(png);
  if (bad) {
    perror("writing file");
    return 1;
  }
  return 0;
}

int flam3gpu_render_png(flam3_frame *f, int transp, stat_struct *stats, const char *genome_xml, unsigned char **png,
                        size_t *png_len) {
  if (!png || !png_len || !stats || !f) {
    f3g_set_error("NULL argument");
    return 1;
  }
  *png = NULL;
  *png_len = 0;
  flam3gpu_render_io io;
  memset(&io, 0, sizeof(io));
  io.keep_on_device = 1;
  if (flam3gpu_render_ex(f, NULL, flam3_field_both, 4, transp, stats, &io)) return 1;
  f3g_ctx *c = f3g_get_ctx();
  /* the strings flam3-render.c:357-365 passes to write_png */
  char badvals[64], numiters[64], rtime[32];
  snprintf(badvals, sizeof(badvals), "%g", stats->badvals / (double)stats->num_iters);
  snprintf(numiters, sizeof(numiters), "%g", (double)stats->num_iters);
  snprintf(rtime, sizeof(rtime), "%d", stats->render_seconds);
  flam3gpu_png_text t[8];
  const int nt = comment_texts(genome_xml, badvals, numiters, rtime, t);
  const int rv = encode_device_image(c, c->d_out, io.image_w, io.image_h, 4, f->bytes_per_channel, t, nt, png,
                                     png_len, &png_last_ms);
  if (rv) fprintf(stderr, "flam3gpu: %s\n", flam3gpu_last_error());
  return rv;
}

int flam3gpu_png_last_ms(double *encode_ms) {
  if (!encode_ms) return 1;
  *encode_ms = png_last_ms;
  return 0;
}


/* flam3-animate's frame loop with PNG output (flam3-animate.c:225-310):
 * the frames render through a render service in chunks of up to BATCH_PNG
 * frames, the next chunk queued before the current one is collected, and
 * each frame is encoded on the device as soon as it completes, on this
 * thread's stream while the service renders the rest.  Host memory holds
 * the raw images of two chunks at most. */
#define BATCH_PNG 32

static int submit_chunk(flam3gpu_service *s, flam3_frame *frames, int n, int transp, void **outs, uint64_t *tk) {
  for (int i = 0; i < n; i++) {
    const flam3_genome *g = &frames[i].genomes[0];
    outs[i] = malloc((size_t)g->width * g->height * 4 * frames[i].bytes_per_channel);
    if (!outs[i]) {
      f3g_set_error("out of host memory");
      return 1;
    }
  }
  return flam3gpu_service_submit_many(s, frames, n, outs, flam3_field_both, 4, transp, tk);
}

int flam3gpu_render_batch_png(flam3_frame *frames, int n, int transp, stat_struct *stats, unsigned char **pngs,
                              size_t *lens) {
  f3g_clear_error();
  if (n < 1) return 0;
  if (!frames || !stats || !pngs || !lens) {
    f3g_set_error("NULL argument");
    return 1;
  }
  for (int i = 0; i < n; i++) pngs[i] = NULL, lens[i] = 0;
  flam3gpu_service_config cfg;
  flam3gpu_service_default_config(&cfg);
  cfg.round_samples = -1;
  void **outs = (void **)calloc((size_t)n, sizeof(void *));
  uint64_t *tk = (uint64_t *)calloc((size_t)n, sizeof(uint64_t));
  if (!outs || !tk) {
    f3g_set_error("out of host memory");
    free(outs);
    free(tk);
    return 1;
  }
  flam3gpu_service *s = flam3gpu_service_create(&cfg);
  int rv = s ? 0 : 1;
  char first_err[256] = "";
  if (s && submit_chunk(s, frames, n < BATCH_PNG ? n : BATCH_PNG, transp, outs, tk)) rv = 1;
  for (int c0 = 0; c0 < n && s; c0 += BATCH_PNG) {
    const int c1 = c0 + BATCH_PNG < n ? c0 + BATCH_PNG : n;
    /* queue the next chunk first, so the device stays busy */
    if (!rv && c1 < n) {
      const int m = c1 + BATCH_PNG < n ? BATCH_PNG : n - c1;
      if (submit_chunk(s, frames + c1, m, transp, outs + c1, tk + c1)) rv = 1;
    }
    for (int i = c0; i < c1; i++) {
      if (!tk[i]) continue;
      if (flam3gpu_service_wait(s, tk[i], -1, &stats[i], NULL)) {
        if (!first_err[0]) snprintf(first_err, sizeof(first_err), "%s", flam3gpu_last_error());
        rv = 1;
      } else {
        char badvals[64], numiters[64], rtime[32];
        snprintf(badvals, sizeof(badvals), "%g", stats[i].badvals / (double)stats[i].num_iters);
        snprintf(numiters, sizeof(numiters), "%g", (double)stats[i].num_iters);
        snprintf(rtime, sizeof(rtime), "%d", stats[i].render_seconds);
        flam3gpu_png_text t[8];
        const int nt = comment_texts(NULL, badvals, numiters, rtime, t);
        const flam3_genome *g = &frames[i].genomes[0];
        if (flam3gpu_encode_png(outs[i], 0, g->width, g->height, 4, frames[i].bytes_per_channel, t, nt, &pngs[i],
                                &lens[i])) {
          if (!first_err[0]) snprintf(first_err, sizeof(first_err), "%s", flam3gpu_last_error());
          rv = 1;
        }
      }
      free(outs[i]);
      outs[i] = NULL;
    }
  }
  if (s) flam3gpu_service_destroy(s);
  for (int i = 0; i < n; i++) free(outs[i]);
  free(outs);
  free(tk);
  if (rv && first_err[0]) f3g_set_error("%s", first_err);
  if (rv) fprintf(stderr, "flam3gpu: %s\n", flam3gpu_last_error());
  return rv;
}
