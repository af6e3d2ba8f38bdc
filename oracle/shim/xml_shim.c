/*
 * A small DOM reader behind the libxml2 API subset declared in
 * shim/libxml/parser.h.  It understands what .flam3 genome files and
 * flam3-palettes.xml contain: a prolog, comments, elements with quoted
 * attributes, self-closing tags, character data and the five predefined
 * entities.  It is test infrastructure for building the reference oracle.
 */
#include "libxml/parser.h"

#include <ctype.h>
#include <stdlib.h>
#include <string.h>

static char *dup_range(const char *s, size_t n) {
  char *d = (char *)malloc(n + 1);
  memcpy(d, s, n);
  d[n] = 0;
  return d;
}

/* Decode the predefined entities and numeric character references in place. */
static void decode_entities(char *s) {
  char *r = s, *w = s;
  while (*r) {
    if (*r == '&') {
      const char *semi = strchr(r, ';');
      if (semi) {
        size_t n = (size_t)(semi - r - 1);
        const char *e = r + 1;
        int ch = -1;
        if (n == 3 && !strncmp(e, "amp", 3)) ch = '&';
        else if (n == 2 && !strncmp(e, "lt", 2)) ch = '<';
        else if (n == 2 && !strncmp(e, "gt", 2)) ch = '>';
        else if (n == 4 && !strncmp(e, "quot", 4)) ch = '"';
        else if (n == 4 && !strncmp(e, "apos", 4)) ch = '\'';
        else if (n > 1 && e[0] == '#') {
          ch = (e[1] == 'x') ? (int)strtol(e + 2, NULL, 16) : atoi(e + 1);
          if (ch > 127) ch = '?';
        }
        if (ch >= 0) {
          *w++ = (char)ch;
          r = semi + 1;
          continue;
        }
      }
    }
    *w++ = *r++;
  }
  *w = 0;
}

typedef struct {
  const char *p, *end;
  int error;
} cursor;

static void skip_ws(cursor *c) {
  while (c->p < c->end && isspace((unsigned char)*c->p)) c->p++;
}

static int starts(cursor *c, const char *lit) {
  size_t n = strlen(lit);
  return (size_t)(c->end - c->p) >= n && !memcmp(c->p, lit, n);
}

static void skip_past(cursor *c, const char *lit) {
  size_t n = strlen(lit);
  while (c->p < c->end && !starts(c, lit)) c->p++;
  if (c->p < c->end) c->p += n;
  else c->error = 1;
}

static xmlNode *new_node(xmlElementType t, const char *name, size_t n) {
  xmlNode *x = (xmlNode *)calloc(1, sizeof(xmlNode));
  x->type = t;
  x->name = (const xmlChar *)dup_range(name, n);
  return x;
}

static void append_child(xmlNode *parent, xmlNode *child, xmlNode **last) {
  child->parent = parent;
  if (*last) (*last)->next = child;
  else parent->children = child;
  *last = child;
}

static xmlNode *parse_element(cursor *c);

/* Parse the children of `parent` up to and including its closing tag. */
static void parse_content(cursor *c, xmlNode *parent) {
  xmlNode *last = NULL;
  while (c->p < c->end && !c->error) {
    if (starts(c, "</")) {
      skip_past(c, ">");
      return;
    } else if (starts(c, "<!--")) {
      skip_past(c, "-->");
    } else if (starts(c, "<?")) {
      skip_past(c, "?>");
    } else if (starts(c, "<![CDATA[")) {
      const char *s = c->p + 9;
      skip_past(c, "]]>");
      xmlNode *t = new_node(XML_TEXT_NODE, "text", 4);
      t->content = (xmlChar *)dup_range(s, (size_t)(c->p - 3 - s));
      append_child(parent, t, &last);
    } else if (*c->p == '<') {
      xmlNode *e = parse_element(c);
      if (!e) return;
      append_child(parent, e, &last);
    } else {
      const char *s = c->p;
      while (c->p < c->end && *c->p != '<') c->p++;
      xmlNode *t = new_node(XML_TEXT_NODE, "text", 4);
      t->content = (xmlChar *)dup_range(s, (size_t)(c->p - s));
      decode_entities((char *)t->content);
      append_child(parent, t, &last);
    }
  }
}

static xmlNode *parse_element(cursor *c) {
  c->p++; /* '<' */
  const char *s = c->p;
  while (c->p < c->end && !isspace((unsigned char)*c->p) && *c->p != '>' && *c->p != '/') c->p++;
  xmlNode *e = new_node(XML_ELEMENT_NODE, s, (size_t)(c->p - s));
  xmlAttr *alast = NULL;
  for (;;) {
    skip_ws(c);
    if (c->p >= c->end) { c->error = 1; return e; }
    if (starts(c, "/>")) { c->p += 2; return e; }
    if (*c->p == '>') { c->p++; parse_content(c, e); return e; }
    const char *an = c->p;
    while (c->p < c->end && *c->p != '=' && !isspace((unsigned char)*c->p) && *c->p != '>' && *c->p != '/') c->p++;
    size_t anl = (size_t)(c->p - an);
    skip_ws(c);
    xmlAttr *a = (xmlAttr *)calloc(1, sizeof(xmlAttr));
    a->name = (const xmlChar *)dup_range(an, anl);
    if (c->p < c->end && *c->p == '=') {
      c->p++;
      skip_ws(c);
      char q = *c->p;
      if (q == '"' || q == '\'') {
        const char *v = ++c->p;
        while (c->p < c->end && *c->p != q) c->p++;
        a->value = (xmlChar *)dup_range(v, (size_t)(c->p - v));
        if (c->p < c->end) c->p++;
      } else {
        const char *v = c->p;
        while (c->p < c->end && !isspace((unsigned char)*c->p) && *c->p != '>') c->p++;
        a->value = (xmlChar *)dup_range(v, (size_t)(c->p - v));
      }
      decode_entities((char *)a->value);
    } else {
      a->value = (xmlChar *)dup_range("", 0);
    }
    if (alast) alast->next = a;
    else e->properties = a;
    alast = a;
  }
}

static void free_node(xmlNode *n) {
  while (n) {
    xmlNode *nx = n->next;
    xmlAttr *a = n->properties;
    while (a) {
      xmlAttr *an = a->next;
      free((void *)a->name);
      free(a->value);
      free(a);
      a = an;
    }
    free_node(n->children);
    free((void *)n->name);
    free(n->content);
    free(n);
    n = nx;
  }
}

int xmlStrcmp(const xmlChar *a, const xmlChar *b) {
  if (a == b) return 0;
  if (!a) return -1;
  if (!b) return 1;
  return strcmp((const char *)a, (const char *)b);
}

xmlChar *xmlGetProp(const xmlNode *node, const xmlChar *name) {
  for (const xmlAttr *a = node ? node->properties : NULL; a; a = a->next)
    if (!xmlStrcmp(a->name, name)) return (xmlChar *)strdup((const char *)a->value);
  return NULL;
}

static void gather_text(const xmlNode *n, char **buf, size_t *len) {
  for (; n; n = n->next) {
    if (n->type == XML_TEXT_NODE && n->content) {
      size_t k = strlen((const char *)n->content);
      *buf = (char *)realloc(*buf, *len + k + 1);
      memcpy(*buf + *len, n->content, k + 1);
      *len += k;
    } else {
      gather_text(n->children, buf, len);
    }
  }
}

xmlChar *xmlNodeGetContent(const xmlNode *node) {
  if (!node) return NULL;
  if (node->type == XML_TEXT_NODE) return (xmlChar *)strdup((const char *)node->content);
  char *buf = (char *)calloc(1, 1);
  size_t len = 0;
  gather_text(node->children, &buf, &len);
  return (xmlChar *)buf;
}

int xmlIsBlankNode(const xmlNode *node) {
  if (!node || node->type != XML_TEXT_NODE || !node->content) return 0;
  for (const xmlChar *p = node->content; *p; p++)
    if (!isspace(*p)) return 0;
  return 1;
}

xmlDocPtr xmlReadMemory(const char *buffer, int size, const char *url, const char *encoding, int options) {
  (void)url; (void)encoding; (void)options;
  cursor c = {buffer, buffer + size, 0};
  xmlNode holder;
  memset(&holder, 0, sizeof(holder));
  parse_content(&c, &holder);
  xmlNode *root = NULL;
  for (xmlNode *n = holder.children; n; n = n->next)
    if (n->type == XML_ELEMENT_NODE) { root = n; break; }
  if (c.error || !root) {
    free_node(holder.children);
    return NULL;
  }
  /* keep only the root element */
  for (xmlNode *n = holder.children, *nx; n; n = nx) {
    nx = n->next;
    if (n != root) { n->next = NULL; free_node(n); }
  }
  root->next = NULL;
  root->parent = NULL;
  xmlDoc *d = (xmlDoc *)calloc(1, sizeof(xmlDoc));
  d->root = root;
  return d;
}

xmlNodePtr xmlDocGetRootElement(const xmlDoc *doc) { return doc ? doc->root : NULL; }

xmlDocPtr xmlNewDoc(const xmlChar *version) {
  (void)version;
  return (xmlDoc *)calloc(1, sizeof(xmlDoc));
}

xmlNodePtr xmlDocSetRootElement(xmlDocPtr doc, xmlNodePtr root) {
  xmlNode *old = doc->root;
  doc->root = root;
  return old;
}

xmlNodePtr xmlCopyNode(xmlNodePtr node, int recursive) {
  if (!node) return NULL;
  xmlNode *c = new_node(node->type, (const char *)node->name, strlen((const char *)node->name));
  if (node->content) c->content = (xmlChar *)strdup((const char *)node->content);
  xmlAttr *alast = NULL;
  for (xmlAttr *a = node->properties; a; a = a->next) {
    xmlAttr *na = (xmlAttr *)calloc(1, sizeof(xmlAttr));
    na->name = (const xmlChar *)strdup((const char *)a->name);
    na->value = (xmlChar *)strdup((const char *)a->value);
    if (alast) alast->next = na;
    else c->properties = na;
    alast = na;
  }
  if (recursive) {
    xmlNode *last = NULL;
    for (xmlNode *k = node->children; k; k = k->next) append_child(c, xmlCopyNode(k, 1), &last);
  }
  return c;
}

void xmlFreeDoc(xmlDocPtr doc) {
  if (!doc) return;
  free_node(doc->root);
  free(doc);
}

void xmlCleanupParser(void) {}

void xmlFree(void *p) { free(p); }
