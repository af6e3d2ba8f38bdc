/*
 * Minimal stand-in for the libxml2 parser API, used only to compile the
 * reference flam3 sources into the test oracle (oracle/_ref).  libxml2 is
 * not installed in this image.  Only the types, fields and functions that
 * flam3.c, parser.c, palettes.c and interpolation.c touch are declared; the
 * implementation (xml_shim.c) is a small DOM reader written for this project.
 *
 * This is test infrastructure: nothing in the product links it.
 */
#ifndef F3_XML_SHIM_PARSER_H
#define F3_XML_SHIM_PARSER_H

#include <stddef.h>

typedef unsigned char xmlChar;

typedef enum {
  XML_ELEMENT_NODE = 1,
  XML_ATTRIBUTE_NODE = 2,
  XML_TEXT_NODE = 3
} xmlElementType;

enum { XML_PARSE_NONET = 1 << 11 };

typedef struct _xmlAttr {
  const xmlChar *name;
  xmlChar *value;
  struct _xmlAttr *next;
} xmlAttr;
typedef xmlAttr *xmlAttrPtr;

typedef struct _xmlNode {
  xmlElementType type;
  const xmlChar *name;      /* element name, or "text" for text nodes */
  xmlChar *content;         /* text nodes only */
  struct _xmlNode *children;
  struct _xmlNode *next;
  struct _xmlNode *parent;
  xmlAttr *properties;
} xmlNode;
typedef xmlNode *xmlNodePtr;

typedef struct _xmlDoc {
  xmlNode *root;
} xmlDoc;
typedef xmlDoc *xmlDocPtr;

int xmlStrcmp(const xmlChar *a, const xmlChar *b);
xmlChar *xmlGetProp(const xmlNode *node, const xmlChar *name);
xmlChar *xmlNodeGetContent(const xmlNode *node);
int xmlIsBlankNode(const xmlNode *node);
xmlDocPtr xmlReadMemory(const char *buffer, int size, const char *url,
                        const char *encoding, int options);
xmlNodePtr xmlDocGetRootElement(const xmlDoc *doc);
xmlDocPtr xmlNewDoc(const xmlChar *version);
xmlNodePtr xmlDocSetRootElement(xmlDocPtr doc, xmlNodePtr root);
xmlNodePtr xmlCopyNode(xmlNodePtr node, int recursive);
void xmlFreeDoc(xmlDocPtr doc);
void xmlCleanupParser(void);
void xmlFree(void *p);

#endif
