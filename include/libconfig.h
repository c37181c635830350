/*
 * libconfig.h -- the subset of the libconfig C API that cpic's sources and
 * tests use, implemented by this project (cpic_gb300/csrc/cpic_conf.c).
 *
 * The names, argument meanings and return conventions follow libconfig's
 * public API (CONFIG_TRUE / CONFIG_FALSE, settings addressed by dotted
 * paths) because cpic's code calls them (src/sim.c:46-84, src/config.c,
 * src/specie.c:19-23, src/particle.c:39-120, src/output.c:67-110,
 * src/cpic.c:155-162).  The structure layouts are this project's own:
 * callers only ever hold pointers to settings and pass a config_t by
 * address.
 *
 * Supported syntax: `name = value;` or `name : value`, groups { }, lists
 * ( ), arrays [ ], integers (decimal, hex, L suffix), floats, strings
 * (adjacent literals concatenate), booleans, # // and C comments, and
 * @include "file".  As in libconfig, a float lookup does not accept an
 * integer setting unless auto-conversion is enabled.
 */
#ifndef CPIC_LIBCONFIG_H
#define CPIC_LIBCONFIG_H

#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CONFIG_TRUE 1
#define CONFIG_FALSE 0

#define CONFIG_TYPE_NONE 0
#define CONFIG_TYPE_GROUP 1
#define CONFIG_TYPE_INT 2
#define CONFIG_TYPE_INT64 3
#define CONFIG_TYPE_FLOAT 4
#define CONFIG_TYPE_STRING 5
#define CONFIG_TYPE_BOOL 6
#define CONFIG_TYPE_ARRAY 7
#define CONFIG_TYPE_LIST 8

#define CONFIG_OPTION_AUTOCONVERT 0x01

typedef struct config_setting_t config_setting_t;
typedef struct config_t config_t;

struct config_setting_t {
	char *name;
	short type;
	long long ival;
	double fval;
	char *sval;
	config_setting_t **elems;   /* group members / list or array elements */
	int nelems, cap;
	config_setting_t *parent;
	config_t *config;
	int line;
	const char *file;
};

struct config_t {
	config_setting_t *root;
	int options;
	char *include_dir;
	const char *error_text;
	const char *error_file;
	int error_line;
	char **files;           /* names of parsed files (owned) */
	int nfiles;
	char errbuf[256];
};

void config_init(config_t *config);
void config_destroy(config_t *config);
int config_read(config_t *config, FILE *stream);
int config_read_file(config_t *config, const char *filename);
int config_read_string(config_t *config, const char *str);
void config_set_include_dir(config_t *config, const char *include_dir);
void config_set_auto_convert(config_t *config, int flag);

const char *config_error_text(const config_t *config);
const char *config_error_file(const config_t *config);
int config_error_line(const config_t *config);

config_setting_t *config_root_setting(const config_t *config);
config_setting_t *config_lookup(const config_t *config, const char *path);
int config_lookup_int(const config_t *config, const char *path, int *value);
int config_lookup_int64(const config_t *config, const char *path, long long *value);
int config_lookup_float(const config_t *config, const char *path, double *value);
int config_lookup_bool(const config_t *config, const char *path, int *value);
int config_lookup_string(const config_t *config, const char *path, const char **value);

int config_setting_type(const config_setting_t *setting);
int config_setting_length(const config_setting_t *setting);
const char *config_setting_name(const config_setting_t *setting);
int config_setting_source_line(const config_setting_t *setting);
config_setting_t *config_setting_get_elem(const config_setting_t *setting, unsigned int idx);
config_setting_t *config_setting_get_member(const config_setting_t *setting, const char *name);
config_setting_t *config_setting_lookup(config_setting_t *setting, const char *path);

int config_setting_get_int(const config_setting_t *setting);
long long config_setting_get_int64(const config_setting_t *setting);
double config_setting_get_float(const config_setting_t *setting);
int config_setting_get_bool(const config_setting_t *setting);
const char *config_setting_get_string(const config_setting_t *setting);

int config_setting_get_int_elem(const config_setting_t *setting, int idx);
long long config_setting_get_int64_elem(const config_setting_t *setting, int idx);
double config_setting_get_float_elem(const config_setting_t *setting, int idx);
const char *config_setting_get_string_elem(const config_setting_t *setting, int idx);

int config_setting_lookup_int(const config_setting_t *setting, const char *name, int *value);
int config_setting_lookup_int64(const config_setting_t *setting, const char *name, long long *value);
int config_setting_lookup_float(const config_setting_t *setting, const char *name, double *value);
int config_setting_lookup_bool(const config_setting_t *setting, const char *name, int *value);
int config_setting_lookup_string(const config_setting_t *setting, const char *name, const char **value);

#ifdef __cplusplus
}
#endif

#endif /* CPIC_LIBCONFIG_H */
