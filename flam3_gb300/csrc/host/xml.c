/*
 * xml.c -- the flame genome reader: flam3's XML genome format (the input of
 * flam3-render / flam3-animate) into flam3_genome arrays, with the same
 * result as the reference's flam3_parse_xml2 (flam3.h:581, flam3.c:1423-1485,
 * parser.c:220-1257), without libxml2.
 *
 * A small DOM (elements, attributes in document order, text content; entity
 * references; comments, processing instructions, DOCTYPE and CDATA) feeds a
 * table-driven reader of the <flame> elements:
 *   - flame attributes (parser.c:329-498), the <color>, <colors>, <palette>,
 *     <symmetry>, <xform>, <finalxform> (with <motion>) and <edit> children
 *     (parser.c:500-790), solo xform, xaos and final-xform placement
 *     (parser.c:792-828);
 *   - xform attributes (parser.c:833-1257): weight, colour, colour speed,
 *     the deprecated symmetry, animate, motion, var / var1 lists, chaos,
 *     plotmode, opacity, coefs, post, the variation weights by name and
 *     their parameters;
 *   - palettes: hex data (parser.c:83-133), missing entries interpolated
 *     (parser.c:135-218), library palettes by number read from the file named
 *     by $flam3_palettes (palettes.c:89-198; without it, as when the
 *     reference cannot read its library, the palette is white).
 * then the document-level fixes of flam3.c:1477-1512 (smooth interpolation
 * on the first and last segment, rotation continuity).
 * Numbers convert like flam3_atof / flam3_atoi: strtod / strtol in the C
 * locale, a trailing character or a range error fails the flame.
 *
 * Deliberate differences: <edit> elements are not kept (the reference keeps
 * a libxml2 document the render never reads); xaos entries that would write
 * past the xform list (undefined in the reference) are dropped.
 */
#include <ctype.h>
#include <errno.h>
#include <libgen.h>
#include <locale.h>
#include <math.h>
#include <pthread.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "f3g_host.h"

/* ---------------------------------------------------------------------
 * DOM
 * ------------------------------------------------------------------- */
typedef struct xnode {
  char *name;
  int nattr;
  char **an, **av;
  char *text; /* concatenated character data of this element */
  struct xnode *child, *next;
} xnode;

typedef struct {
  const char *p, *end;
  int err;
} xcur;

static void xfree(xnode *n) {
  while (n) {
    xnode *nx = n->next;
    free(n->name);
    for (int i = 0; i < n->nattr; i++) {
      free(n->an[i]);
      free(n->av[i]);
    }
    free(n->an);
    free(n->av);
    free(n->text);
    xfree(n->child);
    free(n);
    n = nx;
  }
}

static void put_utf8(char **o, unsigned long c) {
  unsigned char *u = (unsigned char *)*o;
  if (c < 0x80) *u++ = (unsigned char)c;
  else if (c < 0x800) {
    *u++ = (unsigned char)(0xC0 | (c >> 6));
    *u++ = (unsigned char)(0x80 | (c & 0x3F));
  } else if (c < 0x10000) {
    *u++ = (unsigned char)(0xE0 | (c >> 12));
    *u++ = (unsigned char)(0x80 | ((c >> 6) & 0x3F));
    *u++ = (unsigned char)(0x80 | (c & 0x3F));
  } else {
    *u++ = (unsigned char)(0xF0 | (c >> 18));
    *u++ = (unsigned char)(0x80 | ((c >> 12) & 0x3F));
    *u++ = (unsigned char)(0x80 | ((c >> 6) & 0x3F));
    *u++ = (unsigned char)(0x80 | (c & 0x3F));
  }
  *o = (char *)u;
}

/* copy [a, b) with the five predefined entities and character references
 * resolved */
static char *unescape(const char *a, const char *b, int *err) {
  char *out = (char *)malloc((size_t)(b - a) + 1), *o = out;
  if (!out) {
    *err = 1;
    return NULL;
  }
  while (a < b) {
    if (*a != '&') {
      *o++ = *a++;
      continue;
    }
    const char *semi = memchr(a, ';', (size_t)(b - a));
    if (!semi) {
      *err = 1;
      break;
    }
    const size_t n = (size_t)(semi - a - 1);
    const char *e = a + 1;
    if (n == 2 && !strncmp(e, "lt", 2)) *o++ = '<';
    else if (n == 2 && !strncmp(e, "gt", 2)) *o++ = '>';
    else if (n == 3 && !strncmp(e, "amp", 3)) *o++ = '&';
    else if (n == 4 && !strncmp(e, "quot", 4)) *o++ = '"';
    else if (n == 4 && !strncmp(e, "apos", 4)) *o++ = '\'';
    else if (n > 1 && e[0] == '#') {
      char *ep;
      const unsigned long c = (e[1] == 'x' || e[1] == 'X') ? strtoul(e + 2, &ep, 16) : strtoul(e + 1, &ep, 10);
      if (ep != semi || c == 0 || c > 0x10FFFF) {
        *err = 1;
        break;
      }
      put_utf8(&o, c);
    } else {
      *err = 1;
      break;
    }
    a = semi + 1;
  }
  *o = 0;
  return out;
}

static int starts(const xcur *c, const char *s) {
  const size_t n = strlen(s);
  return (size_t)(c->end - c->p) >= n && !memcmp(c->p, s, n);
}

static void skip_past(xcur *c, const char *s) {
  const size_t n = strlen(s);
  while (c->p + n <= c->end && memcmp(c->p, s, n)) c->p++;
  if (c->p + n > c->end) {
    c->err = 1;
    c->p = c->end;
  } else
    c->p += n;
}

static int name_char(int ch) { return isalnum(ch) || ch == '_' || ch == '-' || ch == '.' || ch == ':' || ch >= 0x80; }

static void append_text(xnode *n, const char *a, const char *b, int raw, int *err) {
  if (b <= a) return;
  char *t = raw ? NULL : unescape(a, b, err);
  if (raw) {
    t = (char *)malloc((size_t)(b - a) + 1);
    if (!t) {
      *err = 1;
      return;
    }
    memcpy(t, a, (size_t)(b - a));
    t[b - a] = 0;
  }
  if (!t) return;
  if (!n->text) {
    n->text = t;
    return;
  }
  const size_t l0 = strlen(n->text), l1 = strlen(t);
  char *m = (char *)realloc(n->text, l0 + l1 + 1);
  if (!m) {
    *err = 1;
    free(t);
    return;
  }
  memcpy(m + l0, t, l1 + 1);
  n->text = m;
  free(t);
}

static xnode *parse_element(xcur *c);

/* children and text of `parent` up to its end tag (or the end of input at
 * the top level, parent == NULL semantics handled by the caller) */
static void parse_content(xcur *c, xnode *parent, xnode **tail) {
  while (c->p < c->end && !c->err) {
    if (*c->p != '<') {
      const char *a = c->p;
      while (c->p < c->end && *c->p != '<') c->p++;
      if (parent) append_text(parent, a, c->p, 0, &c->err);
      continue;
    }
    if (starts(c, "<!--")) {
      skip_past(c, "-->");
    } else if (starts(c, "<![CDATA[")) {
      const char *a = c->p + 9;
      skip_past(c, "]]>");
      if (!c->err && parent) append_text(parent, a, c->p - 3, 1, &c->err);
    } else if (starts(c, "<?")) {
      skip_past(c, "?>");
    } else if (starts(c, "<!")) {
      /* DOCTYPE and friends, with an optional [internal subset] */
      int depth = 0;
      while (c->p < c->end) {
        if (*c->p == '[') depth++;
        else if (*c->p == ']') depth--;
        else if (*c->p == '>' && depth <= 0) break;
        c->p++;
      }
      if (c->p >= c->end) c->err = 1;
      else c->p++;
    } else if (starts(c, "</")) {
      return; /* the caller checks the name */
    } else {
      xnode *n = parse_element(c);
      if (!n) {
        c->err = 1;
        return;
      }
      *tail = n;
      tail = &n->next;
    }
  }
}

static xnode *parse_element(xcur *c) {
  c->p++; /* '<' */
  const char *a = c->p;
  while (c->p < c->end && name_char((unsigned char)*c->p)) c->p++;
  if (c->p == a) return NULL;
  xnode *n = (xnode *)calloc(1, sizeof(xnode));
  if (!n) return NULL;
  n->name = (char *)malloc((size_t)(c->p - a) + 1);
  memcpy(n->name, a, (size_t)(c->p - a));
  n->name[c->p - a] = 0;
  for (;;) {
    while (c->p < c->end && isspace((unsigned char)*c->p)) c->p++;
    if (c->p >= c->end) goto bad;
    if (*c->p == '/') {
      if (c->p + 1 >= c->end || c->p[1] != '>') goto bad;
      c->p += 2;
      return n;
    }
    if (*c->p == '>') {
      c->p++;
      break;
    }
    const char *an = c->p;
    while (c->p < c->end && name_char((unsigned char)*c->p)) c->p++;
    if (c->p == an) goto bad;
    const char *ane = c->p;
    while (c->p < c->end && isspace((unsigned char)*c->p)) c->p++;
    if (c->p >= c->end || *c->p != '=') goto bad;
    c->p++;
    while (c->p < c->end && isspace((unsigned char)*c->p)) c->p++;
    if (c->p >= c->end || (*c->p != '"' && *c->p != '\'')) goto bad;
    const char q = *c->p++;
    const char *av = c->p;
    while (c->p < c->end && *c->p != q) c->p++;
    if (c->p >= c->end) goto bad;
    char **nan = (char **)realloc(n->an, (size_t)(n->nattr + 1) * sizeof(char *));
    if (!nan) goto bad;
    n->an = nan;
    char **nav = (char **)realloc(n->av, (size_t)(n->nattr + 1) * sizeof(char *));
    if (!nav) goto bad;
    n->av = nav;
    n->an[n->nattr] = (char *)malloc((size_t)(ane - an) + 1);
    memcpy(n->an[n->nattr], an, (size_t)(ane - an));
    n->an[n->nattr][ane - an] = 0;
    n->av[n->nattr] = unescape(av, c->p, &c->err);
    n->nattr++;
    c->p++;
    if (c->err) goto bad;
  }
  parse_content(c, n, &n->child);
  if (c->err || !starts(c, "</")) goto bad;
  c->p += 2;
  {
    const size_t ln = strlen(n->name);
    if ((size_t)(c->end - c->p) < ln || memcmp(c->p, n->name, ln)) goto bad;
    c->p += ln;
    while (c->p < c->end && isspace((unsigned char)*c->p)) c->p++;
    if (c->p >= c->end || *c->p != '>') goto bad;
    c->p++;
  }
  return n;
bad:
  xfree(n);
  return NULL;
}

/* the document's root element, or NULL when the text is not well formed */
static xnode *parse_document(const char *s, size_t len) {
  xcur c = {s, s + len, 0};
  xnode *top = NULL;
  parse_content(&c, NULL, &top);
  if (c.err || c.p != c.end || !top) {
    xfree(top);
    return NULL;
  }
  if (top->next) { /* one root element only */
    xfree(top);
    return NULL;
  }
  return top;
}

static const char *attr(const xnode *n, const char *name) {
  for (int i = 0; i < n->nattr; i++)
    if (!strcmp(n->an[i], name)) return n->av[i];
  return NULL;
}

/* ---------------------------------------------------------------------
 * numbers (parser.c:26-72)
 * ------------------------------------------------------------------- */
typedef struct {
  int conv_failed;
} rstate;

static int r_atoi(rstate *r, const char *s) {
  char *e;
  errno = 0;
  const long v = strtol(s, &e, 10);
  if (e != s + strlen(s) || errno) {
    r->conv_failed = 1;
    fprintf(stderr, "flam3gpu: error converting integer '%s'\n", s);
  }
  return (int)v;
}

static double r_atof(rstate *r, const char *s) {
  char *e;
  errno = 0;
  const double v = strtod(s, &e);
  if (e != s + strlen(s) || errno) {
    r->conv_failed = 1;
    fprintf(stderr, "flam3gpu: error converting number '%s'\n", s);
  }
  return v;
}

/* ---------------------------------------------------------------------
 * palettes
 * ------------------------------------------------------------------- */

/* hex colour data (parser.c:83-133): chan 3 "RRGGBB", 4 "RRGGBBAA", -4
 * "00RRGGBB" per entry, whitespace allowed between entries */
static int hex_colors(const char *s, flam3_genome *cp, int ncolors, int chan) {
  int i = 0, n = 0;
  const int skip = abs(chan);
  char tmps[2];
  while (isspace((unsigned char)s[i])) i++;
  do {
    int r, g, b, a = 255, got;
    if (chan == 3) got = sscanf(s + i, "%2x%2x%2x", &r, &g, &b);
    else if (chan == -4) got = sscanf(s + i, "00%2x%2x%2x", &r, &g, &b);
    else got = sscanf(s + i, "%2x%2x%2x%2x", &r, &g, &b, &a);
    if ((chan != 4 && got != 3) || (chan == 4 && got != 4)) {
      fprintf(stderr, "flam3gpu: bad hexadecimal colour data\n");
      return 1;
    }
    i += 2 * skip;
    while (isspace((unsigned char)s[i])) i++;
    if (n < 256) {
      cp->palette[n].color[0] = r / 255.0;
      cp->palette[n].color[1] = g / 255.0;
      cp->palette[n].color[2] = b / 255.0;
      cp->palette[n].color[3] = a / 255.0;
      cp->palette[n].index = n;
    }
    n++;
  } while (n < ncolors);
  if (sscanf(s + i, "%1s", tmps) > 0) {
    fprintf(stderr, "flam3gpu: extra data after hex colour data\n");
    return 1;
  }
  return 0;
}

/* entries with index < 0 interpolated between their set neighbours,
 * wrapping around (parser.c:135-218) */
static void fill_missing_colors(flam3_genome *cp) {
  int minix = -1, maxix = 255;
  for (int i = 0; i < 256; i++)
    if (cp->palette[i].index >= 0) {
      minix = i;
      break;
    }
  if (minix < 0) {
    for (int i = 0; i < 256; i++) cp->palette[i].index = i;
    return;
  }
  for (int i = 255; i >= 0; i--)
    if (cp->palette[i].index >= 0) {
      maxix = i;
      break;
    }
  const int wrapmin = minix + 256, wrapmax = maxix - 256;
  int i = 0;
  while (i < 256) {
    if (cp->palette[i].index >= 0) {
      i++;
      continue;
    }
    const int first = i;
    int last = i, left = i - 1, right = i + 1, cl = left, cr = right;
    while (i < 256 && cp->palette[i].index < 0) {
      last = i;
      right = i + 1;
      cr = right;
      i++;
    }
    if (left == -1) {
      left = wrapmax;
      cl = maxix;
    }
    if (right == 256) {
      right = wrapmin;
      cr = minix;
    }
    for (int j = first; j <= last; j++) {
      const double t = (j - left) / (double)(right - left);
      for (int k = 0; k < 4; k++)
        cp->palette[j].color[k] = cp->palette[cl].color[k] * (1.0 - t) + cp->palette[cr].color[k] * t;
      cp->palette[j].index = j;
    }
    i = cr + 1;
  }
}

/* the palette library ($flam3_palettes; palettes.c:31-139), read once */
typedef struct {
  int number;
  unsigned char rgb[256][3];
} lib_pal;
static lib_pal *g_lib;
static int g_nlib = -1; /* -1: not read yet */

static void lib_scan(const xnode *n) {
  for (; n; n = n->next) {
    if (!strcmp(n->name, "palette")) {
      const char *num = attr(n, "number"), *data = attr(n, "data");
      if (data) {
        lib_pal p;
        memset(&p, 0, sizeof(p));
        int k = 0, ok = 1, cnt = 0;
        while (cnt < 256 && ok) {
          unsigned r, g, b;
          while (isspace((unsigned char)data[k])) k++;
          if (sscanf(data + k, "00%2x%2x%2x", &r, &g, &b) != 3) {
            ok = 0;
            break;
          }
          k += 8;
          p.rgb[cnt][0] = (unsigned char)r;
          p.rgb[cnt][1] = (unsigned char)g;
          p.rgb[cnt][2] = (unsigned char)b;
          cnt++;
        }
        if (ok) {
          p.number = num ? atoi(num) : 0;
          lib_pal *m = (lib_pal *)realloc(g_lib, (size_t)(g_nlib + 1) * sizeof(lib_pal));
          if (m) {
            g_lib = m;
            g_lib[g_nlib++] = p;
          }
        }
      }
    } else
      lib_scan(n->child);
  }
}

static void lib_load(void) {
  if (g_nlib >= 0) return;
  g_nlib = 0;
  const char *fn = getenv("flam3_palettes");
  if (!fn) return;
  FILE *f = fopen(fn, "rb");
  if (!f) return;
  fseek(f, 0, SEEK_END);
  const long len = ftell(f);
  fseek(f, 0, SEEK_SET);
  char *s = len > 0 ? (char *)malloc((size_t)len) : NULL;
  if (s && fread(s, 1, (size_t)len, f) == (size_t)len) {
    xnode *root = parse_document(s, (size_t)len);
    lib_scan(root);
    xfree(root);
  }
  free(s);
  fclose(f);
}

/* flam3_get_palette (palettes.c:141-194): white when the number is unknown */
static int lib_palette(int number, flam3_palette pal, double hue_rotation) {
  static pthread_mutex_t mu = PTHREAD_MUTEX_INITIALIZER;
  for (int i = 0; i < 256; i++) {
    pal[i].index = i;
    for (int k = 0; k < 4; k++) pal[i].color[k] = 1.0;
  }
  pthread_mutex_lock(&mu);
  lib_load();
  pthread_mutex_unlock(&mu);
  if (g_nlib <= 0) {
    fprintf(stderr, "flam3gpu: no palette library ($flam3_palettes), palette %d set to white\n", number);
    return -1;
  }
  if (number == -1) number = g_lib[random() % g_nlib].number;
  for (int p = 0; p < g_nlib; p++) {
    if (g_lib[p].number != number) continue;
    for (int i = 0; i < 256; i++) {
      double rgb[3], hsv[3];
      for (int k = 0; k < 3; k++) rgb[k] = g_lib[p].rgb[i][k] / 255.0;
      f3g_rgb2hsv(rgb, hsv);
      hsv[0] += hue_rotation * 6.0;
      f3g_hsv2rgb(hsv, rgb);
      pal[i].index = i;
      for (int k = 0; k < 3; k++) pal[i].color[k] = rgb[k];
      pal[i].color[3] = 1.0;
    }
    return number;
  }
  fprintf(stderr, "flam3gpu: palette number %d not found, using white\n", number);
  return -1;
}

/* interpolate_cmap (interpolation.c:149-191): two library palettes blended
 * in HSV, hue the short way round */
static void blend_lib_palettes(flam3_palette cmap, double blend, int i0, double h0, int i1, double h1) {
  flam3_palette p0, p1;
  lib_palette(i0, p0, h0);
  lib_palette(i1, p1, h1);
  for (int i = 0; i < 256; i++) {
    double s[5], t[5];
    f3g_rgb2hsv(p0[i].color, s);
    f3g_rgb2hsv(p1[i].color, t);
    s[3] = p0[i].color[3];
    t[3] = p1[i].color[3];
    s[4] = p0[i].index;
    t[4] = p1[i].index;
    if (s[0] - t[0] > 3.0) s[0] -= 6.0;
    if (s[0] - t[0] < -3.0) s[0] += 6.0;
    for (int j = 0; j < 5; j++) t[j] = (1.0 - blend) * s[j] + blend * t[j];
    f3g_hsv2rgb(t, cmap[i].color);
    cmap[i].color[3] = t[3];
    cmap[i].index = t[4];
  }
}

/* ---------------------------------------------------------------------
 * xforms
 * ------------------------------------------------------------------- */

/* variation names in index order (variations.c:35-136, the genome format's
 * attribute names) */
static const char *const VAR_NAMES[flam3_nvariations] = {
    "linear", "sinusoidal", "spherical", "swirl", "horseshoe", "polar", "handkerchief", "heart", "disc", "spiral",
    "hyperbolic", "diamond", "ex", "julia", "bent", "waves", "fisheye", "popcorn", "exponential", "power", "cosine",
    "rings", "fan", "blob", "pdj", "fan2", "rings2", "eyefish", "bubble", "cylinder", "perspective", "noise",
    "julian", "juliascope", "blur", "gaussian_blur", "radial_blur", "pie", "ngon", "curl", "rectangles", "arch",
    "tangent", "square", "rays", "blade", "secant2", "twintrian", "cross", "disc2", "super_shape", "flower", "conic",
    "parabola", "bent2", "bipolar", "boarders", "butterfly", "cell", "cpow", "curve", "edisc", "elliptic", "escher",
    "foci", "lazysusan", "loonie", "pre_blur", "modulus", "oscilloscope", "polar2", "popcorn2", "scry", "separation",
    "split", "splits", "stripes", "wedge", "wedge_julia", "wedge_sph", "whorl", "waves2", "exp", "log", "sin", "cos",
    "tan", "sec", "csc", "cot", "sinh", "cosh", "tanh", "sech", "csch", "coth", "auger", "flux", "mobius"};

/* variation parameters by attribute name (parser.c:1010-1246); aliases map
 * to the same field */
typedef struct {
  const char *name;
  size_t off;
} prm_attr;
#define PA(n) {#n, offsetof(flam3_xform, n)}
static const prm_attr PRM_ATTRS[] = {
    PA(blob_low), PA(blob_high), PA(blob_waves), PA(pdj_a), PA(pdj_b), PA(pdj_c), PA(pdj_d), PA(fan2_x), PA(fan2_y),
    PA(rings2_val), PA(perspective_angle), PA(perspective_dist), PA(julian_power), PA(julian_dist),
    PA(juliascope_power), PA(juliascope_dist), PA(radial_blur_angle), PA(pie_slices), PA(pie_rotation),
    PA(pie_thickness), PA(ngon_sides), PA(ngon_power), PA(ngon_circle), PA(ngon_corners), PA(curl_c1), PA(curl_c2),
    PA(rectangles_x), PA(rectangles_y), PA(amw_amp), PA(disc2_rot), PA(disc2_twist), PA(super_shape_m),
    PA(super_shape_n1), PA(super_shape_n2), PA(super_shape_n3), PA(super_shape_holes), PA(flower_petals),
    PA(flower_holes), PA(conic_eccentricity), PA(conic_holes), PA(parabola_height), PA(parabola_width), PA(bent2_x),
    PA(bent2_y), PA(bipolar_shift), PA(cell_size), PA(cpow_i), PA(cpow_r), PA(cpow_power), PA(curve_xamp),
    PA(curve_yamp), PA(curve_xlength), PA(curve_ylength), PA(escher_beta), PA(lazysusan_x), PA(lazysusan_y),
    PA(lazysusan_spin), PA(lazysusan_space), PA(lazysusan_twist), PA(modulus_x), PA(modulus_y),
    {"oscilloscope_separation", offsetof(flam3_xform, oscope_separation)},
    {"oscilloscope_frequency", offsetof(flam3_xform, oscope_frequency)},
    {"oscilloscope_amplitude", offsetof(flam3_xform, oscope_amplitude)},
    {"oscilloscope_damping", offsetof(flam3_xform, oscope_damping)}, PA(oscope_separation), PA(oscope_frequency),
    PA(oscope_amplitude), PA(oscope_damping), PA(popcorn2_x), PA(popcorn2_y), PA(popcorn2_c), PA(separation_x),
    PA(separation_xinside), PA(separation_y), PA(separation_yinside), PA(split_xsize), PA(split_ysize), PA(splits_x),
    PA(splits_y), PA(stripes_space), PA(stripes_warp), PA(wedge_angle), PA(wedge_hole), PA(wedge_count),
    PA(wedge_swirl), PA(wedge_julia_angle), PA(wedge_julia_count), PA(wedge_julia_power), PA(wedge_julia_dist),
    PA(wedge_sph_angle), PA(wedge_sph_hole), PA(wedge_sph_count), PA(wedge_sph_swirl), PA(whorl_inside),
    PA(whorl_outside), PA(waves2_scalex), PA(waves2_scaley), PA(waves2_freqx), PA(waves2_freqy), PA(auger_freq),
    PA(auger_weight), PA(auger_sym), PA(auger_scale), PA(flux_spread),
    {"Re_A", offsetof(flam3_xform, mobius_re_a)}, {"mobius_re_a", offsetof(flam3_xform, mobius_re_a)},
    {"Re_B", offsetof(flam3_xform, mobius_re_b)}, {"mobius_re_b", offsetof(flam3_xform, mobius_re_b)},
    {"Re_C", offsetof(flam3_xform, mobius_re_c)}, {"mobius_re_c", offsetof(flam3_xform, mobius_re_c)},
    {"Re_D", offsetof(flam3_xform, mobius_re_d)}, {"mobius_re_d", offsetof(flam3_xform, mobius_re_d)},
    {"Im_A", offsetof(flam3_xform, mobius_im_a)}, {"mobius_im_a", offsetof(flam3_xform, mobius_im_a)},
    {"Im_B", offsetof(flam3_xform, mobius_im_b)}, {"mobius_im_b", offsetof(flam3_xform, mobius_im_b)},
    {"Im_C", offsetof(flam3_xform, mobius_im_c)}, {"mobius_im_c", offsetof(flam3_xform, mobius_im_c)},
    {"Im_D", offsetof(flam3_xform, mobius_im_d)}, {"mobius_im_d", offsetof(flam3_xform, mobius_im_d)},
};
#undef PA

typedef struct {
  int from, to;
  double v;
} xaos_e;

/* six numbers of a coefs / post attribute (parser.c:967-1008) */
static int six(const char *s, double m[3][2]) {
  const char *p = s;
  for (int k = 0; k < 3; k++)
    for (int j = 0; j < 2; j++) {
      char *e;
      errno = 0;
      m[k][j] = strtod(p, &e);
      if (errno || e == p) return 1;
      p = e;
    }
  return p != s + strlen(s);
}

/* parse_xform_xml (parser.c:833-1257): motion elements take no chaos or
 * plotmode; chaos entries are collected in *xa */
static int read_xform(rstate *r, const xnode *n, flam3_xform *x, xaos_e **xa, int *nxa, int numstd, int motion) {
  if (n->nattr == 0) {
    fprintf(stderr, "flam3gpu: element without attributes\n");
    return 1;
  }
  for (int a = 0; a < n->nattr; a++) {
    const char *nm = n->an[a], *v = n->av[a];
    char tmps[2];
    if (!strcmp(nm, "weight")) x->density = r_atof(r, v);
    else if (!strcmp(nm, "symmetry")) {
      x->color_speed = (1.0 - r_atof(r, v)) / 2.0;
      x->animate = r_atof(r, v) > 0 ? 0 : 1;
    } else if (!strcmp(nm, "color_speed")) x->color_speed = r_atof(r, v);
    else if (!strcmp(nm, "animate")) x->animate = r_atof(r, v);
    else if (!strcmp(nm, "motion_frequency")) x->motion_freq = r_atoi(r, v);
    else if (!strcmp(nm, "motion_function")) {
      if (!strcmp(v, "sin")) x->motion_func = 1;
      else if (!strcmp(v, "triangle")) x->motion_func = 2;
      else if (!strcmp(v, "hill")) x->motion_func = 3;
      else {
        fprintf(stderr, "flam3gpu: unknown motion function '%s'\n", v);
        return 1;
      }
    } else if (!strcmp(nm, "color")) {
      double second;
      x->color = 0.0;
      if (sscanf(v, "%lf %lf%1s", &x->color, &second, tmps) != 2 && sscanf(v, "%lf%1s", &x->color, tmps) != 1) {
        fprintf(stderr, "flam3gpu: malformed xform color '%s'\n", v);
        return 1;
      }
    } else if (!strcmp(nm, "var1")) {
      for (int j = 0; j < flam3_nvariations; j++) x->var[j] = 0.0;
      const int j = r_atoi(r, v);
      if (j < 0 || j >= flam3_nvariations) {
        fprintf(stderr, "flam3gpu: bad variation %d\n", j);
        return 1;
      }
      x->var[j] = 1.0;
    } else if (!strcmp(nm, "var")) {
      const char *p = v;
      for (int j = 0; j < flam3_nvariations; j++) {
        char *e;
        errno = 0;
        x->var[j] = strtod(p, &e);
        if (errno || e == p) {
          fprintf(stderr, "flam3gpu: bad value in var '%s'\n", v);
          return 1;
        }
        p = e;
      }
      if (p != v + strlen(v)) {
        fprintf(stderr, "flam3gpu: extra characters in var '%s'\n", v);
        return 1;
      }
    } else if (!strcmp(nm, "chaos")) {
      if (motion) {
        fprintf(stderr, "flam3gpu: a motion element cannot have a chaos attribute\n");
        return 1;
      }
      /* space-separated scalars; 1.0 entries are skipped */
      char *cpy = strdup(v), *save = NULL;
      int to = 0;
      for (char *tok = strtok_r(cpy, " ", &save); tok; tok = strtok_r(NULL, " ", &save), to++) {
        const double s = r_atof(r, tok);
        if (s == 1.0) continue;
        xaos_e *m = (xaos_e *)realloc(*xa, (size_t)(*nxa + 1) * sizeof(xaos_e));
        if (!m) {
          free(cpy);
          return 1;
        }
        *xa = m;
        (*xa)[*nxa].from = numstd;
        (*xa)[*nxa].to = to;
        (*xa)[*nxa].v = s;
        (*nxa)++;
      }
      free(cpy);
    } else if (!strcmp(nm, "plotmode")) {
      if (motion) {
        fprintf(stderr, "flam3gpu: a motion element cannot have a plotmode attribute\n");
        return 1;
      }
      if (!strcmp(v, "off")) x->opacity = 0.0;
    } else if (!strcmp(nm, "opacity")) x->opacity = r_atof(r, v);
    else if (!strcmp(nm, "coefs")) {
      if (six(v, x->c)) {
        fprintf(stderr, "flam3gpu: bad coefs '%s'\n", v);
        return 1;
      }
    } else if (!strcmp(nm, "post")) {
      if (six(v, x->post)) {
        fprintf(stderr, "flam3gpu: bad post '%s'\n", v);
        return 1;
      }
    } else if (!strcmp(nm, "super_shape_rnd")) {
      double s = r_atof(r, v);
      x->super_shape_rnd = s < 0 ? 0 : (s > 1 ? 1 : s);
    } else {
      size_t k = 0;
      const size_t np = sizeof(PRM_ATTRS) / sizeof(PRM_ATTRS[0]);
      for (; k < np; k++)
        if (!strcmp(nm, PRM_ATTRS[k].name)) break;
      if (k < np) {
        *(double *)((char *)x + PRM_ATTRS[k].off) = r_atof(r, v);
      } else {
        int vi = -1;
        for (int j = 0; j < flam3_nvariations; j++)
          if (!strcmp(nm, VAR_NAMES[j])) {
            vi = j;
            break;
          }
        if (vi >= 0) x->var[vi] = r_atof(r, v);
        else fprintf(stderr, "flam3gpu: unrecognized variation %s, ignored\n", nm);
      }
    }
  }
  return 0;
}

/* round6 and the symmetry xforms of flam3_add_symmetry (flam3.c:2546-2640) */
static double round6(double x) {
  x *= 1e6;
  if (x < 0) x -= 1.0;
  return 1e-6 * (int)(x + 0.5);
}

static double det2(const double m[3][2]) { return m[0][0] * m[1][1] - m[0][1] * m[1][0]; }

/* compare_xforms (interpolation.c:117-147) */
static int cmp_xforms(const void *av, const void *bv) {
  const flam3_xform *a = (const flam3_xform *)av, *b = (const flam3_xform *)bv;
  double ad = det2(a->c), bd = det2(b->c);
  if (a->color_speed > b->color_speed) return 1;
  if (a->color_speed < b->color_speed) return -1;
  if (a->color_speed != 0.0) {
    if (ad < 0) return -1;
    if (bd < 0) return 1;
    ad = atan2(a->c[0][0], a->c[0][1]);
    bd = atan2(b->c[0][0], b->c[0][1]);
  }
  if (ad < bd) return -1;
  if (ad > bd) return 1;
  return 0;
}

static void symmetry_xform(flam3_genome *cp, int i) {
  flam3_xform *x = &cp->xform[i];
  x->density = 1.0;
  x->color_speed = 0.0;
  x->animate = 0.0;
  x->var[0] = 1.0;
  for (int j = 1; j < flam3_nvariations; j++) x->var[j] = 0;
  x->c[2][0] = 0.0;
  x->c[2][1] = 0.0;
}

static void add_symmetry(flam3_genome *cp, int sym) {
  if (sym == 0) {
    /* random kind, with libc random() as the reference draws it */
    static const int dist[] = {-4, -3, -2, -2, -2, -1, -1, -1, 2, 2, 2, 3, 3, 4, 4};
    if (random() & 1) sym = dist[random() % (long)(sizeof(dist) / sizeof(dist[0]))];
    else if (random() & 31) sym = (int)(random() % 13) - 6;
    else sym = (int)(random() % 51) - 25;
  }
  if (sym == 1 || sym == 0) return;
  cp->symmetry = sym;
  int added = 0;
  if (sym < 0) {
    const int i = cp->num_xforms - (cp->final_xform_enable ? 1 : 0);
    f3g_add_xforms(cp, 1, 0, 0);
    symmetry_xform(cp, i);
    cp->xform[i].color = 1.0;
    cp->xform[i].c[0][0] = -1.0;
    cp->xform[i].c[0][1] = 0.0;
    cp->xform[i].c[1][0] = 0.0;
    cp->xform[i].c[1][1] = 1.0;
    added++;
    sym = -sym;
  }
  const double a = 2 * M_PI / sym;
  for (int k = 1; k < sym; k++) {
    const int i = cp->num_xforms - (cp->final_xform_enable ? 1 : 0);
    f3g_add_xforms(cp, 1, 0, 0);
    symmetry_xform(cp, i);
    cp->xform[i].color = (sym < 3) ? 0.0 : ((k - 1.0) / (sym - 2.0));
    cp->xform[i].c[0][0] = round6(cos(k * a));
    cp->xform[i].c[0][1] = round6(sin(k * a));
    cp->xform[i].c[1][0] = round6(-cp->xform[i].c[0][1]);
    cp->xform[i].c[1][1] = cp->xform[i].c[0][0];
    added++;
  }
  /* the reference sorts the last `added` entries of the list */
  qsort(&cp->xform[cp->num_xforms - added], (size_t)added, sizeof(flam3_xform), cmp_xforms);
}

/* ---------------------------------------------------------------------
 * flame elements (parser.c:288-831)
 * ------------------------------------------------------------------- */
typedef enum { F_D, F_I } ftype;
typedef struct {
  const char *name;
  ftype t;
  size_t off;
} flame_attr;
static const flame_attr FLAME_NUM[] = {
    {"time", F_D, offsetof(flam3_genome, time)},
    {"hsv_rgb_palette_blend", F_D, offsetof(flam3_genome, hsv_rgb_palette_blend)},
    {"palette", F_I, offsetof(flam3_genome, palette_index)},
    {"scale", F_D, offsetof(flam3_genome, pixels_per_unit)},
    {"rotate", F_D, offsetof(flam3_genome, rotate)},
    {"zoom", F_D, offsetof(flam3_genome, zoom)},
    {"oversample", F_I, offsetof(flam3_genome, spatial_oversample)},
    {"supersample", F_I, offsetof(flam3_genome, spatial_oversample)},
    {"filter", F_D, offsetof(flam3_genome, spatial_filter_radius)},
    {"temporal_filter_width", F_D, offsetof(flam3_genome, temporal_filter_width)},
    {"temporal_filter_exp", F_D, offsetof(flam3_genome, temporal_filter_exp)},
    {"quality", F_D, offsetof(flam3_genome, sample_density)},
    {"passes", F_I, offsetof(flam3_genome, nbatches)},
    {"temporal_samples", F_I, offsetof(flam3_genome, ntemporal_samples)},
    {"brightness", F_D, offsetof(flam3_genome, brightness)},
    {"gamma", F_D, offsetof(flam3_genome, gamma)},
    {"vibrancy", F_D, offsetof(flam3_genome, vibrancy)},
    {"estimator_radius", F_D, offsetof(flam3_genome, estimator)},
    {"estimator_minimum", F_D, offsetof(flam3_genome, estimator_minimum)},
    {"estimator_curve", F_D, offsetof(flam3_genome, estimator_curve)},
    {"gamma_threshold", F_D, offsetof(flam3_genome, gam_lin_thresh)},
};

/* keyword attributes: the value's index in the list, or a warning */
static int keyword(const char *v, const char *const *words, int n) {
  for (int i = 0; i < n; i++)
    if (!strcmp(v, words[i])) return i;
  return -1;
}

static int read_flame(rstate *r, const xnode *fl, flam3_genome *cp) {
  int solo = -1, num_std = -1, nxa = 0;
  xaos_e *xa = NULL;
  char tmps[2];
  r->conv_failed = 0;
  for (int i = 0; i < 256; i++) {
    for (int k = 0; k < 4; k++) cp->palette[i].color[k] = 0;
    cp->palette[i].index = -1;
  }
  if (fl->nattr == 0) {
    fprintf(stderr, "flam3gpu: <flame> element has no attributes\n");
    return 1;
  }
  memset(cp->flame_name, 0, sizeof(cp->flame_name));
  for (int a = 0; a < fl->nattr; a++) {
    const char *nm = fl->an[a], *v = fl->av[a];
    size_t k = 0;
    const size_t nnum = sizeof(FLAME_NUM) / sizeof(FLAME_NUM[0]);
    for (; k < nnum; k++)
      if (!strcmp(nm, FLAME_NUM[k].name)) break;
    if (k < nnum) {
      char *dst = (char *)cp + FLAME_NUM[k].off;
      if (FLAME_NUM[k].t == F_D) *(double *)dst = r_atof(r, v);
      else *(int *)dst = r_atoi(r, v);
      continue;
    }
    if (!strcmp(nm, "interpolation")) {
      static const char *const w[] = {"linear", "smooth"};
      const int i = keyword(v, w, 2);
      if (i >= 0) cp->interpolation = i;
      else fprintf(stderr, "flam3gpu: unrecognized interpolation %s\n", v);
    } else if (!strcmp(nm, "palette_interpolation")) {
      /* flam3_palette_interpolation_{hsv, sweep, rgb, hsv_circular} = 0, 1, 2, 3 */
      static const char *const w[] = {"hsv", "sweep", "rgb", "hsv_circular"};
      const int i = keyword(v, w, 4);
      if (i >= 0) cp->palette_interpolation = i;
      else fprintf(stderr, "flam3gpu: unrecognized palette interpolation %s\n", v);
    } else if (!strcmp(nm, "interpolation_space") || !strcmp(nm, "interpolation_type")) {
      static const char *const w[] = {"linear", "log", "old", "older"};
      const int i = keyword(v, w, 4);
      if (i >= 0) cp->interpolation_type = i;
      else fprintf(stderr, "flam3gpu: unrecognized interpolation_type %s\n", v);
    } else if (!strcmp(nm, "name")) {
      strncpy(cp->flame_name, v, flam3_name_len);
      /* whitespace becomes '_', the last character excepted (parser.c:370-374) */
      for (int i = (int)strlen(cp->flame_name) - 2; i >= 0; i--)
        if (isspace((unsigned char)cp->flame_name[i])) cp->flame_name[i] = '_';
    } else if (!strcmp(nm, "size")) {
      if (sscanf(v, "%d %d%1s", &cp->width, &cp->height, tmps) != 2) {
        fprintf(stderr, "flam3gpu: invalid size '%s'\n", v);
        return 1;
      }
    } else if (!strcmp(nm, "center")) {
      if (sscanf(v, "%lf %lf%1s", &cp->center[0], &cp->center[1], tmps) != 2) {
        fprintf(stderr, "flam3gpu: invalid center '%s'\n", v);
        return 1;
      }
      cp->rot_center[0] = cp->center[0];
      cp->rot_center[1] = cp->center[1];
    } else if (!strcmp(nm, "filter_shape")) {
      /* the kernel numbers of filters.c:29-45 */
      static const char *const w[] = {"gaussian", "hermite", "box",     "triangle", "bell",     "bspline", "lanczos3",
                                      "lanczos2", "mitchell", "blackman", "catrom",   "hamming", "hanning", "quadratic"};
      const int i = keyword(v, w, 14);
      if (i >= 0) cp->spatial_filter_select = i;
      else fprintf(stderr, "flam3gpu: unrecognized kernel shape %s, using gaussian\n", v);
    } else if (!strcmp(nm, "temporal_filter_type")) {
      static const char *const w[] = {"box", "gaussian", "exp"};
      const int i = keyword(v, w, 3);
      if (i >= 0) cp->temporal_filter_type = i;
      else fprintf(stderr, "flam3gpu: unrecognized temporal filter %s, using box\n", v);
    } else if (!strcmp(nm, "palette_mode")) {
      static const char *const w[] = {"step", "linear"};
      const int i = keyword(v, w, 2);
      if (i >= 0) cp->palette_mode = i;
      else fprintf(stderr, "flam3gpu: unrecognized palette mode %s, using step\n", v);
    } else if (!strcmp(nm, "background")) {
      if (sscanf(v, "%lf %lf %lf%1s", &cp->background[0], &cp->background[1], &cp->background[2], tmps) != 3) {
        fprintf(stderr, "flam3gpu: invalid background '%s'\n", v);
        return 1;
      }
    } else if (!strcmp(nm, "highlight_power")) {
      cp->highlight_power = atof(v); /* converted without the check, as the reference does */
    } else if (!strcmp(nm, "hue")) {
      cp->hue_rotation = fmod(r_atof(r, v), 1.0);
    } else if (!strcmp(nm, "soloxform")) {
      solo = (int)r_atof(r, v);
    }
    /* other attributes are ignored */
  }

  for (const xnode *ch = fl->child; ch; ch = ch->next) {
    if (!strcmp(ch->name, "color")) {
      int index = -1;
      double cr = 0, cg = 0, cb = 0, ca = 0;
      if (ch->nattr == 0) goto attr_error;
      for (int a = 0; a < ch->nattr; a++) {
        const char *nm = ch->an[a], *v = ch->av[a];
        ca = 255.0; /* reset for every attribute (parser.c:516) */
        if (!strcmp(nm, "index")) index = r_atoi(r, v);
        else if (!strcmp(nm, "rgb")) {
          if (sscanf(v, "%lf %lf %lf%1s", &cr, &cg, &cb, tmps) != 3) goto bad_value;
        } else if (!strcmp(nm, "rgba")) {
          if (sscanf(v, "%lf %lf %lf %lf%1s", &cr, &cg, &cb, &ca, tmps) != 4) goto bad_value;
        } else if (!strcmp(nm, "a")) {
          if (sscanf(v, "%lf%1s", &ca, tmps) != 1) goto bad_value;
        } else
          goto attr_error;
      }
      if (index < 0 || index > 255) {
        fprintf(stderr, "flam3gpu: color element with a bad index (%d)\n", index);
        goto fail;
      }
      cp->palette[index].color[3] = ca / 255.0;
      cp->palette[index].color[0] = cp->palette[index].color[3] * cr / 255.0; /* premultiplied */
      cp->palette[index].color[1] = cp->palette[index].color[3] * cg / 255.0;
      cp->palette[index].color[2] = cp->palette[index].color[3] * cb / 255.0;
      cp->palette[index].index = index;
    } else if (!strcmp(ch->name, "colors")) {
      int count = 0;
      if (ch->nattr == 0) goto attr_error;
      for (int a = 0; a < ch->nattr; a++) {
        if (!strcmp(ch->an[a], "count")) count = r_atoi(r, ch->av[a]);
        else if (!strcmp(ch->an[a], "data")) {
          if (hex_colors(ch->av[a], cp, count, -4)) goto fail;
        } else
          goto attr_error;
      }
    } else if (!strcmp(ch->name, "palette")) {
      int ncol = 0, nbytes = 0, oldf = 0, newf = 0, i0 = -1, i1 = -1;
      double h0 = 0, h1 = 0, blend = 0.5;
      if (ch->nattr == 0) goto attr_error;
      for (int a = 0; a < ch->nattr; a++) {
        const char *nm = ch->an[a], *v = ch->av[a];
        if (!strcmp(nm, "index0")) oldf++, i0 = r_atoi(r, v);
        else if (!strcmp(nm, "index1")) oldf++, i1 = r_atoi(r, v);
        else if (!strcmp(nm, "hue0")) oldf++, h0 = r_atof(r, v);
        else if (!strcmp(nm, "hue1")) oldf++, h1 = r_atof(r, v);
        else if (!strcmp(nm, "blend")) oldf++, blend = r_atof(r, v);
        else if (!strcmp(nm, "count")) newf++, ncol = r_atoi(r, v);
        else if (!strcmp(nm, "format")) {
          newf++;
          if (!strcmp(v, "RGB")) nbytes = 3;
          else if (!strcmp(v, "RGBA")) nbytes = 4;
          else {
            fprintf(stderr, "flam3gpu: unrecognized palette format %s\n", v);
            goto fail;
          }
        } else
          goto attr_error;
      }
      if (newf > 0 && oldf > 0) {
        fprintf(stderr, "flam3gpu: old and new palette syntax mixed\n");
        goto fail;
      }
      if (oldf > 0) blend_lib_palettes(cp->palette, blend, i0, h0, i1, h1);
      else if (hex_colors(ch->text ? ch->text : "", cp, ncol, nbytes))
        goto fail;
    } else if (!strcmp(ch->name, "symmetry")) {
      int kind = 0;
      if (ch->nattr == 0) goto attr_error;
      for (int a = 0; a < ch->nattr; a++) {
        if (!strcmp(ch->an[a], "kind")) kind = r_atoi(r, ch->av[a]);
        else goto attr_error;
      }
      const int before = cp->num_xforms;
      add_symmetry(cp, kind);
      num_std += cp->num_xforms - before;
    } else if (!strcmp(ch->name, "xform") || !strcmp(ch->name, "finalxform")) {
      int xf = cp->num_xforms;
      if (!strcmp(ch->name, "finalxform")) {
        if (cp->final_xform_index >= 0) {
          fprintf(stderr, "flam3gpu: more than one final xform\n");
          goto fail;
        }
        f3g_add_xforms(cp, 1, 0, 1);
        cp->xform[xf].var[0] = 0.0;
        cp->final_xform_index = xf;
        cp->final_xform_enable = 1;
      } else {
        f3g_add_xforms(cp, 1, 0, 0);
        if (cp->final_xform_index >= 0) xf--;
        cp->xform[xf].var[0] = 0.0;
        num_std++;
      }
      if (read_xform(r, ch, &cp->xform[xf], &xa, &nxa, num_std, 0)) goto fail;
      if (cp->final_xform_index == xf && cp->xform[xf].density != 0.0) {
        fprintf(stderr, "flam3gpu: final xforms should not have a weight\n");
        goto fail;
      }
      if (cp->xform[xf].motion_freq != 0 || cp->xform[xf].motion_func != 0) {
        fprintf(stderr, "flam3gpu: motion parameters belong in motion elements\n");
        goto fail;
      }
      for (const xnode *m = ch->child; m; m = m->next) {
        if (strcmp(m->name, "motion")) continue;
        flam3_xform *x = &cp->xform[xf];
        flam3_xform *nm = (flam3_xform *)realloc(x->motion, (size_t)(x->num_motion + 1) * sizeof(flam3_xform));
        if (!nm) goto fail;
        x->motion = nm;
        memset(&x->motion[x->num_motion], 0, sizeof(flam3_xform));
        x->num_motion++;
        if (read_xform(r, m, &x->motion[x->num_motion - 1], NULL, NULL, 0, 1)) goto fail;
      }
    }
    /* <edit> and other children are not kept */
  }
  num_std++;
  for (int i = 0; i < num_std; i++)
    if (solo >= 0 && i != solo) cp->xform[i].opacity = 0.0;
  {
    const int ns = cp->num_xforms - (cp->final_xform_index >= 0);
    for (int i = 0; i < nxa; i++)
      if (xa[i].from >= 0 && xa[i].from < ns && xa[i].to >= 0 && xa[i].to < ns)
        cp->chaos[xa[i].from][xa[i].to] = xa[i].v;
  }
  free(xa);
  xa = NULL;
  if (cp->final_xform_index >= 0 && cp->final_xform_index != cp->num_xforms - 1) {
    const flam3_xform t = cp->xform[cp->final_xform_index];
    for (int i = cp->final_xform_index + 1; i < cp->num_xforms; i++) cp->xform[i - 1] = cp->xform[i];
    cp->xform[cp->num_xforms - 1] = t;
    cp->final_xform_index = cp->num_xforms - 1;
  }
  if (r->conv_failed) {
    fprintf(stderr, "flam3gpu: a number or integer attribute did not convert\n");
    return 1;
  }
  return 0;
bad_value:
  fprintf(stderr, "flam3gpu: invalid color attribute value\n");
  goto fail;
attr_error:
  fprintf(stderr, "flam3gpu: missing or unknown attribute in <%s>\n", fl->name);
fail:
  free(xa);
  return 1;
}

/* deep copy including motion elements (flam3_copy, flam3.c:1171-1209) */
static void copy_genome_motion(flam3_genome *dst, const flam3_genome *src) {
  f3g_genome_copy(dst, src);
  const int ns = src->num_xforms - (src->final_xform_index >= 0);
  for (int i = 0; i < src->num_xforms; i++) {
    const flam3_xform *s = &src->xform[i];
    const int d = (src->final_xform_index == i) ? ns : i;
    if (s->num_motion > 0) {
      dst->xform[d].motion = (flam3_xform *)malloc((size_t)s->num_motion * sizeof(flam3_xform));
      if (dst->xform[d].motion) {
        memcpy(dst->xform[d].motion, s->motion, (size_t)s->num_motion * sizeof(flam3_xform));
        dst->xform[d].num_motion = s->num_motion;
      }
    }
  }
}

/* scan_for_flame_nodes (parser.c:220-286): <flame> elements in document
 * order at any depth (not inside another flame); one working genome is
 * reused, so attributes clear_cp leaves alone (time) carry over */
static int scan(rstate *r, const xnode *n, const char *parent, int default_flag, flam3_genome *work,
                flam3_genome **all, int *nall) {
  for (; n; n = n->next) {
    if (strcmp(n->name, "flame")) {
      if (scan(r, n->child, parent, default_flag, work, all, nall)) return 1;
      continue;
    }
    f3g_clear_cp(work, default_flag);
    if (read_flame(r, n, work)) return 1;
    flam3_genome *m = (flam3_genome *)realloc(*all, (size_t)(*nall + 1) * sizeof(flam3_genome));
    if (!m) return 1;
    *all = m;
    memset(&m[*nall], 0, sizeof(flam3_genome));
    if (work->palette_index != -1) lib_palette(work->palette_index, work->palette, work->hue_rotation);
    fill_missing_colors(work);
    work->genome_index = *nall;
    memset(work->parent_fname, 0, flam3_parent_fn_len);
    strncpy(work->parent_fname, parent, flam3_parent_fn_len - 1);
    copy_genome_motion(&m[*nall], work);
    (*nall)++;
  }
  return 0;
}

flam3_genome *flam3gpu_parse_xml2(char *xmldata, char *xmlfilename, int default_flag, int *ncps) {
  f3g_clear_error();
  *ncps = 0;
  if (!xmldata) {
    f3g_set_error("no XML data");
    return NULL;
  }
  xnode *root = parse_document(xmldata, strlen(xmldata));
  if (!root) {
    f3g_set_error("failed to parse %s", xmlfilename ? xmlfilename : "XML data");
    return NULL;
  }
  /* the C locale for strtod / sscanf, restored afterwards */
  locale_t cloc = newlocale(LC_NUMERIC_MASK, "C", (locale_t)0);
  locale_t old = cloc ? uselocale(cloc) : (locale_t)0;
  char fn[flam3_parent_fn_len + 256];
  snprintf(fn, sizeof(fn), "%s", xmlfilename ? xmlfilename : "");
  const char *base = basename(fn);
  flam3_genome work, *all = NULL;
  memset(&work, 0, sizeof(work));
  work.final_xform_index = -1;
  rstate r = {0};
  int nall = 0;
  const int err = scan(&r, root, base, default_flag, &work, &all, &nall);
  f3g_clear_cp(&work, default_flag);
  if (cloc) {
    uselocale(old);
    freelocale(cloc);
  }
  xfree(root);
  if (err) {
    for (int i = 0; i < nall; i++) flam3gpu_free_genome(&all[i]);
    free(all);
    f3g_set_error("error parsing a flame element of %s", xmlfilename ? xmlfilename : "XML data");
    return NULL;
  }
  /* flam3.c:1477-1512: smooth interpolation is not allowed on the first
   * or the last segment, and consecutive rotations stay within 180 degrees
   * (outside the compat / older interpolation types) */
  if (nall >= 1 && all[0].interpolation == 1) {
    fprintf(stderr, "flam3gpu: smooth interpolation cannot be used for the first segment, switching to linear\n");
    all[0].interpolation = 0;
  }
  if (nall >= 2 && all[nall - 2].interpolation == 1) {
    fprintf(stderr, "flam3gpu: smooth interpolation cannot be used for the last segment, switching to linear\n");
    all[nall - 2].interpolation = 0;
  }
  for (int i = 1; i < nall; i++) {
    if (all[i - 1].interpolation_type == 2 || all[i - 1].interpolation_type == 3) continue;
    while (all[i].rotate < all[i - 1].rotate - 180) all[i].rotate += 360;
    while (all[i].rotate > all[i - 1].rotate + 180) all[i].rotate -= 360;
  }
  *ncps = nall;
  return all;
}
