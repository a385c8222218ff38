/*
 * libconfig.h -- a small, project-written reader for the subset of the
 * libconfig file syntax that starrynight.cfg uses.
 *
 * The reference reads its configuration through libconfig
 * (src/starrynight-config.c:98-182, #include at src/starrynight-main.c:16).
 * libconfig itself is not part of this project.  This header exposes the
 * same names and calling conventions that the reference's load_config()
 * uses, so that (a) the GPU host driver reads starrynight.cfg with the same
 * key semantics and (b) the unmodified reference sources compile against it.
 *
 * Supported syntax: settings `name = value` or `name : value`, optionally
 * terminated by `;` or `,`; groups `{ ... }`; arrays `[ ... ]` of scalars;
 * lists `( ... )`; integers (decimal, hex 0x.., optional L suffix); floats;
 * booleans true/false (any case); strings "..." with C escapes, adjacent
 * strings concatenated; comments `#`, `//`, and C block comments.
 *
 * Typed lookups are strict, as libconfig's defaults are: an int lookup does
 * not match a float setting and a float lookup does not match an int
 * setting (libconfig converts only when CONFIG_OPTION_AUTOCONVERT is set,
 * which the reference never does).
 */
#ifndef SN_LIBCONFIG_MIN_H
#define SN_LIBCONFIG_MIN_H

#ifdef __cplusplus
extern "C" {
#endif

#define CONFIG_TRUE  1
#define CONFIG_FALSE 0

#define CONFIG_TYPE_NONE   0
#define CONFIG_TYPE_GROUP  1
#define CONFIG_TYPE_INT    2
#define CONFIG_TYPE_INT64  3
#define CONFIG_TYPE_FLOAT  4
#define CONFIG_TYPE_STRING 5
#define CONFIG_TYPE_BOOL   6
#define CONFIG_TYPE_ARRAY  7
#define CONFIG_TYPE_LIST   8

typedef struct config_setting_t {
    char *name;                       /* NULL for array/list elements */
    int type;
    long long ival;                   /* INT, INT64, BOOL */
    double fval;                      /* FLOAT */
    char *sval;                       /* STRING */
    struct config_setting_t **child;  /* GROUP, ARRAY, LIST */
    int nchild;
    int cap;
    int line;
} config_setting_t;

typedef struct config_t {
    config_setting_t *root;
    char error_text[256];
    char error_file[256];
    int error_line;
} config_t;

void config_init(config_t *cfg);
void config_destroy(config_t *cfg);
int config_read_file(config_t *cfg, const char *filename);
int config_read_string(config_t *cfg, const char *text);

const char *config_error_text(const config_t *cfg);
const char *config_error_file(const config_t *cfg);
int config_error_line(const config_t *cfg);

config_setting_t *config_lookup(const config_t *cfg, const char *path);
int config_lookup_int(const config_t *cfg, const char *path, int *value);
int config_lookup_int64(const config_t *cfg, const char *path, long long *value);
int config_lookup_float(const config_t *cfg, const char *path, double *value);
int config_lookup_bool(const config_t *cfg, const char *path, int *value);
int config_lookup_string(const config_t *cfg, const char *path, const char **value);

int config_setting_length(const config_setting_t *setting);
int config_setting_type(const config_setting_t *setting);
config_setting_t *config_setting_get_elem(const config_setting_t *setting, unsigned int idx);
double config_setting_get_float_elem(const config_setting_t *setting, int idx);
int config_setting_get_int_elem(const config_setting_t *setting, int idx);

#ifdef __cplusplus
}
#endif

#endif
