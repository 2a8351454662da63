/*
 * charm_yaml.c - the subset of YAML that CHARM_3D's case files use, read into
 * a small node tree (maps, sequences, scalars).
 *
 * Supported: block mappings and block sequences by indentation (spaces),
 * "- key: value" sequence items, flow mappings {k: v, ...} and flow
 * sequences [a, b] (nested), plain, 'single' and "double" quoted scalars,
 * comments (# at the start of a line or after a blank).  Not supported (an
 * error, never a silent misread): tabs in indentation, anchors and aliases,
 * tags, multi-line scalars, multiple documents.
 */
#include "charm_yaml.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    int indent;
    char *text;     /* content after the indentation, comment stripped, right-trimmed */
    int lineno;
} yline_t;

typedef struct {
    yline_t *lines;
    int n;
    char *err;
    size_t errlen;
    int failed;
} yparser_t;

static void yfail(yparser_t *p, int lineno, const char *msg)
{
    if (!p->failed && p->err && p->errlen) snprintf(p->err, p->errlen, "line %d: %s", lineno, msg);
    p->failed = 1;
}

static charm_ynode_t *ynew(int type)
{
    charm_ynode_t *n = (charm_ynode_t *) calloc(1, sizeof(charm_ynode_t));
    if (n) n->type = type;
    return n;
}

static int ypush(charm_ynode_t *n, char *key, charm_ynode_t *val)
{
    if (n->n == n->cap) {
        int cap = n->cap ? 2 * n->cap : 8;
        char **k = (char **) realloc(n->keys, sizeof(char *) * (size_t) cap);
        if (!k) return -1;
        n->keys = k;
        charm_ynode_t **v = (charm_ynode_t **) realloc(n->items, sizeof(charm_ynode_t *) * (size_t) cap);
        if (!v) return -1;
        n->items = v;
        n->cap = cap;
    }
    n->keys[n->n] = key;
    n->items[n->n] = val;
    n->n++;
    return 0;
}

void charm_yaml_free(charm_ynode_t *n)
{
    if (!n) return;
    for (int i = 0; i < n->n; i++) {
        free(n->keys[i]);
        charm_yaml_free(n->items[i]);
    }
    free(n->keys);
    free(n->items);
    free(n->str);
    free(n);
}

static char *ystrndup(const char *s, size_t len)
{
    char *r = (char *) malloc(len + 1);
    if (!r) return NULL;
    memcpy(r, s, len);
    r[len] = 0;
    return r;
}

/* ---- flow context: scalars, {..}, [..] ---------------------------------- */

static const char *skip_ws(const char *s)
{
    while (*s == ' ') s++;
    return s;
}

/* A scalar starting at *ps; in a flow collection it ends at , ] } ; a key
 * ends at ": " (or ':' before a flow terminator).  Quotes are removed. */
static char *yscalar(yparser_t *p, int lineno, const char **ps, int in_flow, int is_key)
{
    const char *s = skip_ws(*ps);
    if (*s == '\'' || *s == '"') {
        const char q = *s++;
        char *out = (char *) malloc(strlen(s) + 1);
        size_t k = 0;
        if (!out) return NULL;
        while (*s && *s != q) {
            if (q == '"' && *s == '\\' && s[1]) {
                s++;
                out[k++] = (*s == 'n') ? '\n' : (*s == 't') ? '\t' : *s;
                s++;
                continue;
            }
            if (q == '\'' && *s == '\'' && s[1] == '\'') { out[k++] = '\''; s += 2; continue; }
            out[k++] = *s++;
        }
        if (*s != q) { free(out); yfail(p, lineno, "unterminated quoted scalar"); return NULL; }
        out[k] = 0;
        *ps = s + 1;
        return out;
    }
    const char *b = s;
    while (*s) {
        if (in_flow && (*s == ',' || *s == ']' || *s == '}')) break;
        if (is_key && *s == ':' && (s[1] == ' ' || s[1] == 0 || (in_flow && (s[1] == ',' || s[1] == '}')))) break;
        s++;
    }
    const char *e = s;
    while (e > b && e[-1] == ' ') e--;
    *ps = s;
    if (e == b) return ystrndup("", 0);
    if (*b == '&' || *b == '*' || *b == '!' || *b == '|' || *b == '>') {
        yfail(p, lineno, "anchors, aliases, tags and block scalars are not supported");
        return NULL;
    }
    return ystrndup(b, (size_t) (e - b));
}

static charm_ynode_t *yflow(yparser_t *p, int lineno, const char **ps);

static charm_ynode_t *yflow_value(yparser_t *p, int lineno, const char **ps)
{
    const char *s = skip_ws(*ps);
    if (*s == '{' || *s == '[') {
        *ps = s;
        return yflow(p, lineno, ps);
    }
    charm_ynode_t *n = ynew(CHARM_Y_SCALAR);
    if (!n) return NULL;
    n->str = yscalar(p, lineno, &s, 1, 0);
    *ps = s;
    if (!n->str) { charm_yaml_free(n); return NULL; }
    return n;
}

/* A flow collection starting at **ps ('{' or '['). */
static charm_ynode_t *yflow(yparser_t *p, int lineno, const char **ps)
{
    const char *s = *ps;
    const int is_map = (*s == '{');
    const char close = is_map ? '}' : ']';
    charm_ynode_t *n = ynew(is_map ? CHARM_Y_MAP : CHARM_Y_SEQ);
    if (!n) return NULL;
    s = skip_ws(s + 1);
    if (*s == close) { *ps = s + 1; return n; }
    for (;;) {
        char *key = NULL;
        if (is_map) {
            key = yscalar(p, lineno, &s, 1, 1);
            if (!key) { charm_yaml_free(n); return NULL; }
            s = skip_ws(s);
            if (*s != ':') { free(key); charm_yaml_free(n); yfail(p, lineno, "expected ':' in a flow mapping"); return NULL; }
            s++;
        }
        charm_ynode_t *v = yflow_value(p, lineno, &s);
        if (!v) { free(key); charm_yaml_free(n); return NULL; }
        if (ypush(n, key, v)) { free(key); charm_yaml_free(v); charm_yaml_free(n); return NULL; }
        s = skip_ws(s);
        if (*s == ',') { s = skip_ws(s + 1); continue; }
        if (*s == close) { *ps = s + 1; return n; }
        charm_yaml_free(n);
        yfail(p, lineno, is_map ? "expected ',' or '}'" : "expected ',' or ']'");
        return NULL;
    }
}

/* The value text of a block line (after "key:" or "- "). */
static charm_ynode_t *yinline(yparser_t *p, int lineno, const char *s)
{
    const char *t = s;
    charm_ynode_t *n = yflow_value(p, lineno, &t);
    if (!n) return NULL;
    t = skip_ws(t);
    if (*t) {
        charm_yaml_free(n);
        yfail(p, lineno, "unexpected text after a value");
        return NULL;
    }
    return n;
}

/* ---- block context -------------------------------------------------------- */

static charm_ynode_t *yblock(yparser_t *p, int *pi, int indent);

static int is_seq_item(const char *t) { return t[0] == '-' && (t[1] == ' ' || t[1] == 0); }

/* Position of the ':' that ends a block mapping key, or NULL. */
static const char *key_colon(const char *t)
{
    if (*t == '"' || *t == '\'') {
        const char q = *t;
        const char *e = strchr(t + 1, q);
        if (!e) return NULL;
        e = skip_ws(e + 1);
        return (*e == ':') ? e : NULL;
    }
    if (*t == '{' || *t == '[') return NULL;
    for (const char *s = t; *s; s++)
        if (*s == ':' && (s[1] == ' ' || s[1] == 0)) return s;
    return NULL;
}

static charm_ynode_t *yblock_seq(yparser_t *p, int *pi, int indent)
{
    charm_ynode_t *n = ynew(CHARM_Y_SEQ);
    if (!n) return NULL;
    while (*pi < p->n && !p->failed) {
        yline_t *L = &p->lines[*pi];
        if (L->indent < indent) break;
        if (L->indent > indent) { yfail(p, L->lineno, "bad indentation in a sequence"); break; }
        if (!is_seq_item(L->text)) break;
        const char *rest = skip_ws(L->text + 1);
        charm_ynode_t *v = NULL;
        if (!*rest) {
            (*pi)++;
            if (*pi < p->n && p->lines[*pi].indent > indent) {
                v = yblock(p, pi, p->lines[*pi].indent);
            } else if ((v = ynew(CHARM_Y_SCALAR))) {
                v->str = ystrndup("", 0);
            }
        } else if (key_colon(rest)) {
            /* "- key: value": a mapping whose first line is this one */
            L->indent = indent + (int) (rest - L->text);
            L->text = (char *) rest;
            v = yblock(p, pi, L->indent);
        } else {
            v = yinline(p, L->lineno, rest);
            (*pi)++;
        }
        if (!v || ypush(n, NULL, v)) { charm_yaml_free(v); charm_yaml_free(n); return NULL; }
    }
    return n;
}

static charm_ynode_t *yblock_map(yparser_t *p, int *pi, int indent)
{
    charm_ynode_t *n = ynew(CHARM_Y_MAP);
    if (!n) return NULL;
    while (*pi < p->n && !p->failed) {
        yline_t *L = &p->lines[*pi];
        if (L->indent < indent) break;
        if (L->indent > indent) { yfail(p, L->lineno, "bad indentation in a mapping"); break; }
        if (is_seq_item(L->text)) { yfail(p, L->lineno, "sequence item where a mapping key was expected"); break; }
        const char *c = key_colon(L->text);
        if (!c) { yfail(p, L->lineno, "expected 'key: value'"); break; }
        const char *ks = L->text;
        char *key = yscalar(p, L->lineno, &ks, 0, 1);
        if (!key) break;
        for (int i = 0; i < n->n; i++)
            if (strcmp(n->keys[i], key) == 0) yfail(p, L->lineno, "duplicate key");
        if (p->failed) { free(key); break; }
        const char *rest = skip_ws(c + 1);
        charm_ynode_t *v = NULL;
        if (!*rest) {
            (*pi)++;
            if (*pi < p->n && (p->lines[*pi].indent > indent ||
                               (p->lines[*pi].indent == indent && is_seq_item(p->lines[*pi].text))))
                v = yblock(p, pi, p->lines[*pi].indent);
            else if ((v = ynew(CHARM_Y_SCALAR)))
                v->str = ystrndup("", 0);
        } else {
            v = yinline(p, L->lineno, rest);
            (*pi)++;
        }
        if (!v || ypush(n, key, v)) { free(key); charm_yaml_free(v); charm_yaml_free(n); return NULL; }
    }
    return n;
}

static charm_ynode_t *yblock(yparser_t *p, int *pi, int indent)
{
    if (*pi >= p->n) return NULL;
    if (is_seq_item(p->lines[*pi].text)) return yblock_seq(p, pi, indent);
    if (key_colon(p->lines[*pi].text)) return yblock_map(p, pi, indent);
    /* a lone scalar or flow collection */
    charm_ynode_t *v = yinline(p, p->lines[*pi].lineno, p->lines[*pi].text);
    (*pi)++;
    return v;
}

charm_ynode_t *charm_yaml_parse(const char *text, char *err, size_t errlen)
{
    yparser_t p;
    memset(&p, 0, sizeof(p));
    p.err = err;
    p.errlen = errlen;
    if (err && errlen) err[0] = 0;
    const char *src = text ? text : "";
    char *buf = ystrndup(src, strlen(src));
    if (!buf) return NULL;
    int cap = 64, lineno = 0;
    p.lines = (yline_t *) malloc(sizeof(yline_t) * (size_t) cap);
    if (!p.lines) { free(buf); return NULL; }
    for (char *s = buf; s && *s;) {
        char *nl = strchr(s, '\n');
        if (nl) *nl = 0;
        lineno++;
        /* strip the comment: '#' at the start or after a blank, outside quotes */
        char q = 0;
        for (char *c = s; *c; c++) {
            if (q) { if (*c == q) q = 0; continue; }
            if (*c == '\'' || *c == '"') { if (c == s || c[-1] == ' ' || c[-1] == '[' || c[-1] == '{' || c[-1] == ',') q = *c; continue; }
            if (*c == '#' && (c == s || c[-1] == ' ' || c[-1] == '\t')) { *c = 0; break; }
        }
        size_t len = strlen(s);
        while (len && (s[len - 1] == ' ' || s[len - 1] == '\r' || s[len - 1] == '\t')) s[--len] = 0;
        int ind = 0;
        while (s[ind] == ' ') ind++;
        if (s[ind] == '\t') { yfail(&p, lineno, "tab in indentation"); break; }
        if (s[ind]) {
            if (strcmp(s + ind, "---") == 0 && p.n == 0) { /* document start */ }
            else if (strcmp(s + ind, "---") == 0 || strcmp(s + ind, "...") == 0) {
                yfail(&p, lineno, "multiple documents are not supported");
                break;
            } else {
                if (p.n == cap) {
                    cap *= 2;
                    yline_t *nlines = (yline_t *) realloc(p.lines, sizeof(yline_t) * (size_t) cap);
                    if (!nlines) { p.failed = 1; break; }
                    p.lines = nlines;
                }
                p.lines[p.n].indent = ind;
                p.lines[p.n].text = s + ind;
                p.lines[p.n].lineno = lineno;
                p.n++;
            }
        }
        s = nl ? nl + 1 : NULL;
    }
    charm_ynode_t *root = NULL;
    if (!p.failed) {
        int i = 0;
        root = (p.n == 0) ? ynew(CHARM_Y_MAP) : yblock(&p, &i, p.lines[0].indent);
        if (!p.failed && i < p.n) yfail(&p, p.lines[i].lineno, "unexpected indentation");
        if (p.failed) { charm_yaml_free(root); root = NULL; }
        else if (!root && err && errlen) snprintf(err, errlen, "out of memory");
    }
    free(p.lines);
    free(buf);
    return root;
}

charm_ynode_t *charm_yaml_load(const char *path, char *err, size_t errlen)
{
    FILE *f = fopen(path, "rb");
    if (!f) {
        if (err && errlen) snprintf(err, errlen, "cannot open '%s'", path);
        return NULL;
    }
    fseek(f, 0, SEEK_END);
    long sz = ftell(f);
    fseek(f, 0, SEEK_SET);
    if (sz < 0 || sz > (64L << 20)) {
        fclose(f);
        if (err && errlen) snprintf(err, errlen, "'%s': bad size", path);
        return NULL;
    }
    char *text = (char *) malloc((size_t) sz + 1);
    if (!text) { fclose(f); return NULL; }
    size_t got = fread(text, 1, (size_t) sz, f);
    fclose(f);
    text[got] = 0;
    charm_ynode_t *n = charm_yaml_parse(text, err, errlen);
    free(text);
    return n;
}

const charm_ynode_t *charm_yaml_get(const charm_ynode_t *map, const char *key)
{
    if (!map || map->type != CHARM_Y_MAP) return NULL;
    for (int i = 0; i < map->n; i++)
        if (strcmp(map->keys[i], key) == 0) return map->items[i];
    return NULL;
}

int charm_yaml_double(const charm_ynode_t *n, double *out)
{
    if (!n || n->type != CHARM_Y_SCALAR || !n->str[0]) return -1;
    char *end = NULL;
    double v = strtod(n->str, &end);
    if (end == n->str) return -1;
    while (*end == ' ') end++;
    if (*end) return -1;
    *out = v;
    return 0;
}

int charm_yaml_int(const charm_ynode_t *n, int *out)
{
    if (!n || n->type != CHARM_Y_SCALAR || !n->str[0]) return -1;
    char *end = NULL;
    long v = strtol(n->str, &end, 10);
    if (end == n->str) return -1;
    while (*end == ' ') end++;
    if (*end || v < -2147483647L || v > 2147483647L) return -1;
    *out = (int) v;
    return 0;
}

const char *charm_yaml_str(const charm_ynode_t *n)
{
    return (n && n->type == CHARM_Y_SCALAR) ? n->str : NULL;
}
