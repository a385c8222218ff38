/*
 * libconfig_min.c -- project-written reader for the libconfig syntax subset
 * used by starrynight.cfg.  See libconfig.h in this directory for the
 * supported grammar and the lookup semantics (which follow the calls made by
 * the reference's load_config(), src/starrynight-config.c:98-182).
 *
 * Recursive-descent parser over the whole file held in memory.  Errors are
 * reported through config_error_text()/config_error_line(), never by exit().
 */
#include "libconfig.h"

#include <ctype.h>
#include <errno.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    const char *s;
    size_t pos;
    size_t len;
    int line;
    config_t *cfg;
    int failed;
} parser;

static config_setting_t *new_setting(int type, int line)
{
    config_setting_t *st = (config_setting_t *)calloc(1, sizeof(*st));
    if (st) {
        st->type = type;
        st->line = line;
    }
    return st;
}

static void free_setting(config_setting_t *st)
{
    int i;
    if (!st) return;
    for (i = 0; i < st->nchild; i++) free_setting(st->child[i]);
    free(st->child);
    free(st->name);
    free(st->sval);
    free(st);
}

static int add_child(config_setting_t *parent, config_setting_t *child)
{
    if (parent->nchild == parent->cap) {
        int ncap = parent->cap ? 2 * parent->cap : 8;
        config_setting_t **nc = (config_setting_t **)realloc(parent->child, sizeof(*nc) * (size_t)ncap);
        if (!nc) return 0;
        parent->child = nc;
        parent->cap = ncap;
    }
    parent->child[parent->nchild++] = child;
    return 1;
}

static void fail(parser *p, const char *msg)
{
    if (p->failed) return;
    p->failed = 1;
    snprintf(p->cfg->error_text, sizeof(p->cfg->error_text), "%s", msg);
    p->cfg->error_line = p->line;
}

static void skip_ws(parser *p)
{
    while (p->pos < p->len) {
        char c = p->s[p->pos];
        if (c == '\n') {
            p->line++;
            p->pos++;
        } else if (isspace((unsigned char)c)) {
            p->pos++;
        } else if (c == '#') {
            while (p->pos < p->len && p->s[p->pos] != '\n') p->pos++;
        } else if (c == '/' && p->pos + 1 < p->len && p->s[p->pos + 1] == '/') {
            while (p->pos < p->len && p->s[p->pos] != '\n') p->pos++;
        } else if (c == '/' && p->pos + 1 < p->len && p->s[p->pos + 1] == '*') {
            p->pos += 2;
            while (p->pos + 1 < p->len && !(p->s[p->pos] == '*' && p->s[p->pos + 1] == '/')) {
                if (p->s[p->pos] == '\n') p->line++;
                p->pos++;
            }
            if (p->pos + 1 >= p->len) {
                fail(p, "unterminated comment");
                p->pos = p->len;
                return;
            }
            p->pos += 2;
        } else {
            return;
        }
    }
}

static int peek(parser *p)
{
    skip_ws(p);
    return p->pos < p->len ? (unsigned char)p->s[p->pos] : -1;
}

static int is_name_start(int c) { return isalpha(c) || c == '*'; }
static int is_name_char(int c) { return isalnum(c) || c == '_' || c == '-' || c == '*'; }

static char *parse_name(parser *p)
{
    size_t start, n;
    char *out;
    skip_ws(p);
    start = p->pos;
    if (p->pos >= p->len || !is_name_start((unsigned char)p->s[p->pos])) {
        fail(p, "syntax error: expected a setting name");
        return NULL;
    }
    while (p->pos < p->len && is_name_char((unsigned char)p->s[p->pos])) p->pos++;
    n = p->pos - start;
    out = (char *)malloc(n + 1);
    if (!out) {
        fail(p, "out of memory");
        return NULL;
    }
    memcpy(out, p->s + start, n);
    out[n] = '\0';
    return out;
}

static config_setting_t *parse_value(parser *p);

static int parse_string_piece(parser *p, char **buf, size_t *blen, size_t *bcap)
{
    p->pos++; /* opening quote */
    while (p->pos < p->len && p->s[p->pos] != '"') {
        char c = p->s[p->pos++];
        if (c == '\n') p->line++;
        if (c == '\\' && p->pos < p->len) {
            char e = p->s[p->pos++];
            switch (e) {
            case 'n': c = '\n'; break;
            case 't': c = '\t'; break;
            case 'r': c = '\r'; break;
            case 'f': c = '\f'; break;
            case '\\': c = '\\'; break;
            case '"': c = '"'; break;
            case 'x': {
                int v = 0, k;
                for (k = 0; k < 2 && p->pos < p->len && isxdigit((unsigned char)p->s[p->pos]); k++) {
                    char h = p->s[p->pos++];
                    v = v * 16 + (isdigit((unsigned char)h) ? h - '0' : (tolower((unsigned char)h) - 'a' + 10));
                }
                c = (char)v;
                break;
            }
            default: c = e; break;
            }
        }
        if (*blen + 2 > *bcap) {
            size_t ncap = *bcap ? 2 * *bcap : 32;
            char *nb = (char *)realloc(*buf, ncap);
            if (!nb) {
                fail(p, "out of memory");
                return 0;
            }
            *buf = nb;
            *bcap = ncap;
        }
        (*buf)[(*blen)++] = c;
    }
    if (p->pos >= p->len) {
        fail(p, "unterminated string");
        return 0;
    }
    p->pos++; /* closing quote */
    return 1;
}

static config_setting_t *parse_scalar(parser *p)
{
    int c = peek(p);
    int line = p->line;
    config_setting_t *st;
    if (c == '"') {
        char *buf = NULL;
        size_t blen = 0, bcap = 0;
        while (peek(p) == '"') {
            if (!parse_string_piece(p, &buf, &blen, &bcap)) {
                free(buf);
                return NULL;
            }
        }
        st = new_setting(CONFIG_TYPE_STRING, line);
        if (!st) {
            free(buf);
            fail(p, "out of memory");
            return NULL;
        }
        if (!buf) buf = (char *)calloc(1, 1);
        else buf[blen] = '\0';
        st->sval = buf;
        return st;
    }
    if (isalpha(c)) {
        size_t start = p->pos;
        char word[16];
        size_t n;
        while (p->pos < p->len && isalpha((unsigned char)p->s[p->pos])) p->pos++;
        n = p->pos - start;
        if (n < sizeof(word)) {
            size_t k;
            for (k = 0; k < n; k++) word[k] = (char)tolower((unsigned char)p->s[start + k]);
            word[n] = '\0';
            if (!strcmp(word, "true") || !strcmp(word, "false")) {
                st = new_setting(CONFIG_TYPE_BOOL, line);
                if (!st) {
                    fail(p, "out of memory");
                    return NULL;
                }
                st->ival = word[0] == 't';
                return st;
            }
        }
        fail(p, "syntax error: unknown literal");
        return NULL;
    }
    if (isdigit(c) || c == '-' || c == '+' || c == '.') {
        const char *start = p->s + p->pos;
        size_t i = p->pos;
        int is_float = 0;
        char tmp[128];
        size_t n;
        if (p->s[i] == '-' || p->s[i] == '+') i++;
        if (i + 1 < p->len && p->s[i] == '0' && (p->s[i + 1] == 'x' || p->s[i + 1] == 'X')) {
            i += 2;
            while (i < p->len && isxdigit((unsigned char)p->s[i])) i++;
        } else {
            while (i < p->len && isdigit((unsigned char)p->s[i])) i++;
            if (i < p->len && p->s[i] == '.') {
                is_float = 1;
                i++;
                while (i < p->len && isdigit((unsigned char)p->s[i])) i++;
            }
            if (i < p->len && (p->s[i] == 'e' || p->s[i] == 'E')) {
                is_float = 1;
                i++;
                if (i < p->len && (p->s[i] == '-' || p->s[i] == '+')) i++;
                while (i < p->len && isdigit((unsigned char)p->s[i])) i++;
            }
        }
        n = i - p->pos;
        if (n == 0 || n >= sizeof(tmp)) {
            fail(p, "syntax error: bad number");
            return NULL;
        }
        memcpy(tmp, start, n);
        tmp[n] = '\0';
        p->pos = i;
        if (is_float) {
            char *end;
            st = new_setting(CONFIG_TYPE_FLOAT, line);
            if (!st) {
                fail(p, "out of memory");
                return NULL;
            }
            st->fval = strtod(tmp, &end);
            if (*end != '\0') {
                free_setting(st);
                fail(p, "syntax error: bad float");
                return NULL;
            }
            return st;
        } else {
            char *end;
            int is64 = 0;
            long long v;
            if (p->pos < p->len && p->s[p->pos] == 'L') {
                is64 = 1;
                p->pos++;
                if (p->pos < p->len && p->s[p->pos] == 'L') p->pos++;
            }
            errno = 0;
            v = strtoll(tmp, &end, 0);
            if (*end != '\0' || errno) {
                fail(p, "syntax error: bad integer");
                return NULL;
            }
            if (!is64 && (v > 2147483647LL || v < -2147483648LL)) is64 = 1;
            st = new_setting(is64 ? CONFIG_TYPE_INT64 : CONFIG_TYPE_INT, line);
            if (!st) {
                fail(p, "out of memory");
                return NULL;
            }
            st->ival = v;
            return st;
        }
    }
    fail(p, "syntax error: expected a value");
    return NULL;
}

static void skip_separator(parser *p)
{
    int c = peek(p);
    if (c == ';' || c == ',') p->pos++;
}

static int parse_settings(parser *p, config_setting_t *group, int closing)
{
    for (;;) {
        int c = peek(p);
        char *name;
        config_setting_t *val;
        int k;
        if (p->failed) return 0;
        if (c == closing) return 1; /* closing == -1 means end of input */
        if (c == -1) {
            fail(p, "syntax error: unexpected end of file");
            return 0;
        }
        name = parse_name(p);
        if (!name) return 0;
        c = peek(p);
        if (c != '=' && c != ':') {
            free(name);
            fail(p, "syntax error: expected '=' or ':'");
            return 0;
        }
        p->pos++;
        val = parse_value(p);
        if (!val) {
            free(name);
            return 0;
        }
        for (k = 0; k < group->nchild; k++) {
            if (group->child[k]->name && !strcmp(group->child[k]->name, name)) {
                free(name);
                free_setting(val);
                fail(p, "duplicate setting name");
                return 0;
            }
        }
        val->name = name;
        if (!add_child(group, val)) {
            free_setting(val);
            fail(p, "out of memory");
            return 0;
        }
        skip_separator(p);
    }
}

static config_setting_t *parse_value(parser *p)
{
    int c = peek(p);
    int line = p->line;
    config_setting_t *st;
    if (c == '{') {
        p->pos++;
        st = new_setting(CONFIG_TYPE_GROUP, line);
        if (!st) {
            fail(p, "out of memory");
            return NULL;
        }
        if (!parse_settings(p, st, '}')) {
            free_setting(st);
            return NULL;
        }
        p->pos++;
        return st;
    }
    if (c == '[' || c == '(') {
        int closing = c == '[' ? ']' : ')';
        p->pos++;
        st = new_setting(c == '[' ? CONFIG_TYPE_ARRAY : CONFIG_TYPE_LIST, line);
        if (!st) {
            fail(p, "out of memory");
            return NULL;
        }
        if (peek(p) == closing) {
            p->pos++;
            return st;
        }
        for (;;) {
            config_setting_t *el = closing == ']' ? parse_scalar(p) : parse_value(p);
            if (!el) {
                free_setting(st);
                return NULL;
            }
            if (closing == ']' && st->nchild > 0 && el->type != st->child[0]->type) {
                free_setting(el);
                free_setting(st);
                fail(p, "mismatched element type in array");
                return NULL;
            }
            if (!add_child(st, el)) {
                free_setting(el);
                free_setting(st);
                fail(p, "out of memory");
                return NULL;
            }
            c = peek(p);
            if (c == ',') {
                p->pos++;
                continue;
            }
            if (c == closing) {
                p->pos++;
                return st;
            }
            free_setting(st);
            fail(p, "syntax error in array or list");
            return NULL;
        }
    }
    return parse_scalar(p);
}

void config_init(config_t *cfg)
{
    memset(cfg, 0, sizeof(*cfg));
}

void config_destroy(config_t *cfg)
{
    free_setting(cfg->root);
    cfg->root = NULL;
}

int config_read_string(config_t *cfg, const char *text)
{
    parser p;
    config_setting_t *root;
    free_setting(cfg->root);
    cfg->root = NULL;
    cfg->error_text[0] = '\0';
    cfg->error_line = 0;
    root = new_setting(CONFIG_TYPE_GROUP, 1);
    if (!root) {
        snprintf(cfg->error_text, sizeof(cfg->error_text), "out of memory");
        return CONFIG_FALSE;
    }
    p.s = text;
    p.pos = 0;
    p.len = strlen(text);
    p.line = 1;
    p.cfg = cfg;
    p.failed = 0;
    if (!parse_settings(&p, root, -1) || p.failed) {
        free_setting(root);
        return CONFIG_FALSE;
    }
    cfg->root = root;
    return CONFIG_TRUE;
}

int config_read_file(config_t *cfg, const char *filename)
{
    FILE *f = fopen(filename, "rb");
    long n;
    char *buf;
    int ok;
    snprintf(cfg->error_file, sizeof(cfg->error_file), "%s", filename ? filename : "(null)");
    if (!f) {
        snprintf(cfg->error_text, sizeof(cfg->error_text), "file I/O error");
        cfg->error_line = 0;
        return CONFIG_FALSE;
    }
    fseek(f, 0, SEEK_END);
    n = ftell(f);
    fseek(f, 0, SEEK_SET);
    if (n < 0) {
        fclose(f);
        snprintf(cfg->error_text, sizeof(cfg->error_text), "file I/O error");
        return CONFIG_FALSE;
    }
    buf = (char *)malloc((size_t)n + 1);
    if (!buf) {
        fclose(f);
        snprintf(cfg->error_text, sizeof(cfg->error_text), "out of memory");
        return CONFIG_FALSE;
    }
    if (fread(buf, 1, (size_t)n, f) != (size_t)n) {
        free(buf);
        fclose(f);
        snprintf(cfg->error_text, sizeof(cfg->error_text), "file I/O error");
        return CONFIG_FALSE;
    }
    buf[n] = '\0';
    fclose(f);
    ok = config_read_string(cfg, buf);
    free(buf);
    return ok;
}

const char *config_error_text(const config_t *cfg) { return cfg->error_text; }
const char *config_error_file(const config_t *cfg) { return cfg->error_file; }
int config_error_line(const config_t *cfg) { return cfg->error_line; }

config_setting_t *config_lookup(const config_t *cfg, const char *path)
{
    config_setting_t *cur = cfg ? cfg->root : NULL;
    const char *seg = path;
    if (!cur || !path) return NULL;
    while (*seg) {
        const char *end = seg;
        size_t n;
        int k, found = 0;
        while (*end && *end != '.' && *end != '/') end++;
        n = (size_t)(end - seg);
        if (cur->type != CONFIG_TYPE_GROUP) return NULL;
        for (k = 0; k < cur->nchild; k++) {
            const char *nm = cur->child[k]->name;
            if (nm && strlen(nm) == n && !strncmp(nm, seg, n)) {
                cur = cur->child[k];
                found = 1;
                break;
            }
        }
        if (!found) return NULL;
        seg = *end ? end + 1 : end;
    }
    return cur;
}

int config_lookup_int(const config_t *cfg, const char *path, int *value)
{
    config_setting_t *st = config_lookup(cfg, path);
    if (!st) return CONFIG_FALSE;
    if (st->type == CONFIG_TYPE_INT || (st->type == CONFIG_TYPE_INT64 && st->ival >= -2147483647LL - 1 && st->ival <= 2147483647LL)) {
        *value = (int)st->ival;
        return CONFIG_TRUE;
    }
    return CONFIG_FALSE;
}

int config_lookup_int64(const config_t *cfg, const char *path, long long *value)
{
    config_setting_t *st = config_lookup(cfg, path);
    if (!st) return CONFIG_FALSE;
    if (st->type == CONFIG_TYPE_INT || st->type == CONFIG_TYPE_INT64) {
        *value = st->ival;
        return CONFIG_TRUE;
    }
    return CONFIG_FALSE;
}

int config_lookup_float(const config_t *cfg, const char *path, double *value)
{
    config_setting_t *st = config_lookup(cfg, path);
    if (!st || st->type != CONFIG_TYPE_FLOAT) return CONFIG_FALSE;
    *value = st->fval;
    return CONFIG_TRUE;
}

int config_lookup_bool(const config_t *cfg, const char *path, int *value)
{
    config_setting_t *st = config_lookup(cfg, path);
    if (!st || st->type != CONFIG_TYPE_BOOL) return CONFIG_FALSE;
    *value = (int)st->ival;
    return CONFIG_TRUE;
}

int config_lookup_string(const config_t *cfg, const char *path, const char **value)
{
    config_setting_t *st = config_lookup(cfg, path);
    if (!st || st->type != CONFIG_TYPE_STRING) return CONFIG_FALSE;
    *value = st->sval;
    return CONFIG_TRUE;
}

int config_setting_length(const config_setting_t *setting)
{
    if (!setting) return 0;
    if (setting->type == CONFIG_TYPE_GROUP || setting->type == CONFIG_TYPE_ARRAY || setting->type == CONFIG_TYPE_LIST)
        return setting->nchild;
    return 0;
}

int config_setting_type(const config_setting_t *setting)
{
    return setting ? setting->type : CONFIG_TYPE_NONE;
}

config_setting_t *config_setting_get_elem(const config_setting_t *setting, unsigned int idx)
{
    if (!setting) return NULL;
    if (setting->type != CONFIG_TYPE_GROUP && setting->type != CONFIG_TYPE_ARRAY && setting->type != CONFIG_TYPE_LIST)
        return NULL;
    if (idx >= (unsigned int)setting->nchild) return NULL;
    return setting->child[idx];
}

double config_setting_get_float_elem(const config_setting_t *setting, int idx)
{
    config_setting_t *el = idx < 0 ? NULL : config_setting_get_elem(setting, (unsigned int)idx);
    if (!el || el->type != CONFIG_TYPE_FLOAT) return 0.0;
    return el->fval;
}

int config_setting_get_int_elem(const config_setting_t *setting, int idx)
{
    config_setting_t *el = idx < 0 ? NULL : config_setting_get_elem(setting, (unsigned int)idx);
    if (!el || (el->type != CONFIG_TYPE_INT && el->type != CONFIG_TYPE_INT64)) return 0;
    return (int)el->ival;
}
