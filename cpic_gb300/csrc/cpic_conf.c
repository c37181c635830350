/*
 * cpic_conf.c -- a libconfig-subset parser (include/libconfig.h): the
 * .conf front end of the simulation (the reference reads its settings with
 * libconfig, src/sim.c:46-84) written for this project.
 *
 * Grammar handled: setting := name ('=' | ':') value [';' | ','];
 * value := scalar | '[' scalars ']' | '(' values ')' | '{' settings '}';
 * scalar := integer | float | string+ | true | false.  Comments: '#',
 * '//', C comments.  '@include "file"' splices another file, resolved
 * against the include directory or the including file's directory.
 */
#define _GNU_SOURCE
#include <ctype.h>
#include <errno.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>

#include "../../include/libconfig.h"

#define CONF_API __attribute__((visibility("default")))

/* ------------------------------------------------------------ settings */

static config_setting_t *
setting_new(config_t *cfg, config_setting_t *parent, const char *name, int type, int line,
		const char *file)
{
	config_setting_t *s = calloc(1, sizeof(*s));
	if(!s) return NULL;
	s->name = name ? strdup(name) : NULL;
	s->type = (short) type;
	s->parent = parent;
	s->config = cfg;
	s->line = line;
	s->file = file;
	return s;
}

static int
setting_add(config_setting_t *parent, config_setting_t *child)
{
	if(parent->nelems == parent->cap)
	{
		int ncap = parent->cap ? 2 * parent->cap : 8;
		config_setting_t **e = realloc(parent->elems, sizeof(*e) * (size_t) ncap);
		if(!e) return -1;
		parent->elems = e;
		parent->cap = ncap;
	}
	parent->elems[parent->nelems++] = child;
	return 0;
}

static void
setting_free(config_setting_t *s)
{
	int i;
	if(!s) return;
	for(i = 0; i < s->nelems; i++) setting_free(s->elems[i]);
	free(s->elems);
	free(s->name);
	free(s->sval);
	free(s);
}

/* -------------------------------------------------------------- lexer */

typedef struct {
	const char *p, *end;
	int line;
	const char *file;
	config_t *cfg;
	int depth;
} lexer_t;

static int
fail(lexer_t *lx, const char *msg)
{
	config_t *c = lx->cfg;
	snprintf(c->errbuf, sizeof(c->errbuf), "%s", msg);
	c->error_text = c->errbuf;
	c->error_line = lx->line;
	c->error_file = lx->file;
	return -1;
}

static void
skip_ws(lexer_t *lx)
{
	for(;;)
	{
		while(lx->p < lx->end && isspace((unsigned char) *lx->p))
		{
			if(*lx->p == '\n') lx->line++;
			lx->p++;
		}
		if(lx->p >= lx->end) return;
		if(*lx->p == '#' || (*lx->p == '/' && lx->p + 1 < lx->end && lx->p[1] == '/'))
		{
			while(lx->p < lx->end && *lx->p != '\n') lx->p++;
			continue;
		}
		if(*lx->p == '/' && lx->p + 1 < lx->end && lx->p[1] == '*')
		{
			lx->p += 2;
			while(lx->p + 1 < lx->end && !(lx->p[0] == '*' && lx->p[1] == '/'))
			{
				if(*lx->p == '\n') lx->line++;
				lx->p++;
			}
			lx->p = lx->p + 2 <= lx->end ? lx->p + 2 : lx->end;
			continue;
		}
		return;
	}
}

static int
parse_string(lexer_t *lx, char **out)
{
	size_t cap = 64, len = 0;
	char *buf = malloc(cap);
	if(!buf) return fail(lx, "out of memory");
	/* adjacent string literals concatenate */
	while(lx->p < lx->end && *lx->p == '"')
	{
		lx->p++;
		while(lx->p < lx->end && *lx->p != '"')
		{
			char ch = *lx->p++;
			if(ch == '\\' && lx->p < lx->end)
			{
				char e = *lx->p++;
				ch = e == 'n' ? '\n' : e == 't' ? '\t' : e == 'r' ? '\r' : e == 'f' ? '\f' : e;
			}
			if(ch == '\n') lx->line++;
			if(len + 2 > cap)
			{
				char *nb = realloc(buf, cap *= 2);
				if(!nb) { free(buf); return fail(lx, "out of memory"); }
				buf = nb;
			}
			buf[len++] = ch;
		}
		if(lx->p >= lx->end) { free(buf); return fail(lx, "unterminated string"); }
		lx->p++;
		skip_ws(lx);
	}
	buf[len] = '\0';
	*out = buf;
	return 0;
}

static int parse_settings(lexer_t *lx, config_setting_t *group, char closer);

/* Parse one value into a new child of `parent` named `name`. */
static int
parse_value(lexer_t *lx, config_setting_t *parent, const char *name)
{
	config_setting_t *s;
	int line = lx->line;
	skip_ws(lx);
	if(lx->p >= lx->end) return fail(lx, "unexpected end of input");
	char ch = *lx->p;
	if(ch == '{' || ch == '(' || ch == '[')
	{
		int type = ch == '{' ? CONFIG_TYPE_GROUP : ch == '(' ? CONFIG_TYPE_LIST : CONFIG_TYPE_ARRAY;
		char closer = ch == '{' ? '}' : ch == '(' ? ')' : ']';
		if(++lx->depth > 64) return fail(lx, "nesting too deep");
		s = setting_new(lx->cfg, parent, name, type, line, lx->file);
		if(!s || setting_add(parent, s)) return fail(lx, "out of memory");
		lx->p++;
		if(type == CONFIG_TYPE_GROUP)
		{
			if(parse_settings(lx, s, '}')) return -1;
		}
		else
		{
			skip_ws(lx);
			while(lx->p < lx->end && *lx->p != closer)
			{
				if(parse_value(lx, s, NULL)) return -1;
				skip_ws(lx);
				if(lx->p < lx->end && *lx->p == ',') { lx->p++; skip_ws(lx); }
			}
			if(lx->p >= lx->end) return fail(lx, "unterminated list or array");
			lx->p++;
			if(type == CONFIG_TYPE_ARRAY)
			{
				int i;
				for(i = 0; i < s->nelems; i++)
				{
					int et = s->elems[i]->type;
					if(et == CONFIG_TYPE_GROUP || et == CONFIG_TYPE_LIST || et == CONFIG_TYPE_ARRAY)
						return fail(lx, "arrays hold scalars only");
				}
			}
		}
		lx->depth--;
		return 0;
	}
	s = setting_new(lx->cfg, parent, name, CONFIG_TYPE_NONE, line, lx->file);
	if(!s || setting_add(parent, s)) return fail(lx, "out of memory");
	if(ch == '"')
	{
		s->type = CONFIG_TYPE_STRING;
		return parse_string(lx, &s->sval);
	}
	if(!strncasecmp(lx->p, "true", 4) && !isalnum((unsigned char) (lx->p + 4 < lx->end ? lx->p[4] : ' ')))
	{
		s->type = CONFIG_TYPE_BOOL; s->ival = 1; lx->p += 4; return 0;
	}
	if(!strncasecmp(lx->p, "false", 5) && !isalnum((unsigned char) (lx->p + 5 < lx->end ? lx->p[5] : ' ')))
	{
		s->type = CONFIG_TYPE_BOOL; s->ival = 0; lx->p += 5; return 0;
	}
	/* number */
	{
		const char *q = lx->p;
		int isfloat = 0, ishex = 0;
		if(*q == '+' || *q == '-') q++;
		if(q + 1 < lx->end && q[0] == '0' && (q[1] == 'x' || q[1] == 'X')) ishex = 1;
		const char *r = q;
		while(r < lx->end && (isalnum((unsigned char) *r) || *r == '.' || *r == '+' || *r == '-'))
		{
			if(!ishex && (*r == '.' || *r == 'e' || *r == 'E')) isfloat = 1;
			if((*r == '+' || *r == '-') && !(r[-1] == 'e' || r[-1] == 'E')) break;
			r++;
		}
		if(r == q) return fail(lx, "syntax error");
		char tmp[128];
		size_t len = (size_t) (r - lx->p);
		if(len >= sizeof(tmp)) return fail(lx, "number too long");
		memcpy(tmp, lx->p, len);
		tmp[len] = '\0';
		char *e;
		errno = 0;
		if(isfloat)
		{
			s->type = CONFIG_TYPE_FLOAT;
			s->fval = strtod(tmp, &e);
		}
		else
		{
			int is64 = 0;
			if(len > 0 && (tmp[len - 1] == 'L' || tmp[len - 1] == 'l'))
			{
				tmp[--len] = '\0';
				is64 = 1;
				if(len > 0 && (tmp[len - 1] == 'L' || tmp[len - 1] == 'l')) tmp[--len] = '\0';
			}
			s->ival = strtoll(tmp, &e, ishex ? 16 : 10);
			if(s->ival > 2147483647LL || s->ival < -2147483648LL) is64 = 1;
			s->type = is64 ? CONFIG_TYPE_INT64 : CONFIG_TYPE_INT;
		}
		if(*e != '\0' || errno) return fail(lx, "invalid number");
		lx->p = r;
	}
	return 0;
}

static int parse_file(config_t *cfg, config_setting_t *group, const char *path, int depth);

static int
parse_settings(lexer_t *lx, config_setting_t *group, char closer)
{
	for(;;)
	{
		skip_ws(lx);
		if(lx->p >= lx->end)
		{
			if(closer) return fail(lx, "unterminated group");
			return 0;
		}
		if(closer && *lx->p == closer)
		{
			lx->p++;
			return 0;
		}
		if(*lx->p == '@')
		{
			const char kw[] = "@include";
			if(strncmp(lx->p, kw, sizeof(kw) - 1)) return fail(lx, "unknown directive");
			lx->p += sizeof(kw) - 1;
			skip_ws(lx);
			if(lx->p >= lx->end || *lx->p != '"') return fail(lx, "@include needs a file name");
			char *fn;
			if(parse_string(lx, &fn)) return -1;
			char full[4096];
			if(fn[0] != '/' && lx->cfg->include_dir)
				snprintf(full, sizeof(full), "%s/%s", lx->cfg->include_dir, fn);
			else if(fn[0] != '/' && lx->file && strrchr(lx->file, '/'))
				snprintf(full, sizeof(full), "%.*s/%s", (int) (strrchr(lx->file, '/') - lx->file),
						lx->file, fn);
			else
				snprintf(full, sizeof(full), "%s", fn);
			free(fn);
			if(lx->depth > 16) return fail(lx, "@include nesting too deep");
			if(parse_file(lx->cfg, group, full, lx->depth + 1)) return -1;
			continue;
		}
		if(!(isalpha((unsigned char) *lx->p) || *lx->p == '*'))
			return fail(lx, "syntax error");
		const char *q = lx->p;
		while(lx->p < lx->end && (isalnum((unsigned char) *lx->p) || *lx->p == '_' || *lx->p == '-'
					|| *lx->p == '*'))
			lx->p++;
		char name[256];
		size_t len = (size_t) (lx->p - q);
		if(len >= sizeof(name)) return fail(lx, "name too long");
		memcpy(name, q, len);
		name[len] = '\0';
		skip_ws(lx);
		if(lx->p >= lx->end || (*lx->p != '=' && *lx->p != ':'))
			return fail(lx, "expected '=' or ':'");
		lx->p++;
		/* a later duplicate name is an error in libconfig */
		if(config_setting_get_member(group, name))
			return fail(lx, "duplicate setting name");
		if(parse_value(lx, group, name)) return -1;
		skip_ws(lx);
		if(lx->p < lx->end && (*lx->p == ';' || *lx->p == ','))
			lx->p++;
	}
}

static char *
slurp(FILE *f, size_t *n)
{
	size_t cap = 4096, len = 0;
	char *buf = malloc(cap);
	size_t r;
	if(!buf) return NULL;
	while((r = fread(buf + len, 1, cap - len, f)) > 0)
	{
		len += r;
		if(len == cap)
		{
			char *nb = realloc(buf, cap *= 2);
			if(!nb) { free(buf); return NULL; }
			buf = nb;
		}
	}
	*n = len;
	return buf;
}

static const char *
remember_file(config_t *cfg, const char *path)
{
	char **f = realloc(cfg->files, sizeof(char *) * (size_t) (cfg->nfiles + 1));
	if(!f) return NULL;
	cfg->files = f;
	cfg->files[cfg->nfiles] = strdup(path);
	return cfg->files[cfg->nfiles++];
}

static int
parse_buffer(config_t *cfg, config_setting_t *group, const char *buf, size_t n, const char *file,
		int depth)
{
	lexer_t lx;
	lx.p = buf;
	lx.end = buf + n;
	lx.line = 1;
	lx.file = file;
	lx.cfg = cfg;
	lx.depth = depth;
	return parse_settings(&lx, group, 0);
}

static int
parse_file(config_t *cfg, config_setting_t *group, const char *path, int depth)
{
	FILE *f = fopen(path, "r");
	size_t n;
	char *buf;
	int r;
	if(!f)
	{
		snprintf(cfg->errbuf, sizeof(cfg->errbuf), "cannot open file");
		cfg->error_text = cfg->errbuf;
		cfg->error_file = remember_file(cfg, path);
		cfg->error_line = 0;
		return -1;
	}
	buf = slurp(f, &n);
	fclose(f);
	if(!buf) return -1;
	r = parse_buffer(cfg, group, buf, n, remember_file(cfg, path), depth);
	free(buf);
	return r;
}

/* ------------------------------------------------------------------ API */

CONF_API void
config_init(config_t *c)
{
	memset(c, 0, sizeof(*c));
	c->root = setting_new(c, NULL, NULL, CONFIG_TYPE_GROUP, 0, NULL);
}

CONF_API void
config_destroy(config_t *c)
{
	int i;
	setting_free(c->root);
	c->root = NULL;
	free(c->include_dir);
	c->include_dir = NULL;
	for(i = 0; i < c->nfiles; i++) free(c->files[i]);
	free(c->files);
	c->files = NULL;
	c->nfiles = 0;
}

static void
reset_root(config_t *c)
{
	setting_free(c->root);
	c->root = setting_new(c, NULL, NULL, CONFIG_TYPE_GROUP, 0, NULL);
	c->error_text = NULL;
	c->error_file = NULL;
	c->error_line = 0;
}

CONF_API int
config_read(config_t *c, FILE *stream)
{
	size_t n;
	char *buf;
	int r;
	reset_root(c);
	buf = slurp(stream, &n);
	if(!buf) return CONFIG_FALSE;
	r = parse_buffer(c, c->root, buf, n, NULL, 0);
	free(buf);
	return r ? CONFIG_FALSE : CONFIG_TRUE;
}

CONF_API int
config_read_string(config_t *c, const char *str)
{
	reset_root(c);
	return parse_buffer(c, c->root, str, strlen(str), NULL, 0) ? CONFIG_FALSE : CONFIG_TRUE;
}

CONF_API int
config_read_file(config_t *c, const char *filename)
{
	reset_root(c);
	return parse_file(c, c->root, filename, 0) ? CONFIG_FALSE : CONFIG_TRUE;
}

CONF_API void
config_set_include_dir(config_t *c, const char *dir)
{
	free(c->include_dir);
	c->include_dir = dir ? strdup(dir) : NULL;
}

CONF_API void
config_set_auto_convert(config_t *c, int flag)
{
	if(flag) c->options |= CONFIG_OPTION_AUTOCONVERT;
	else c->options &= ~CONFIG_OPTION_AUTOCONVERT;
}

CONF_API const char *config_error_text(const config_t *c) { return c->error_text; }
CONF_API const char *config_error_file(const config_t *c) { return c->error_file; }
CONF_API int config_error_line(const config_t *c) { return c->error_line; }
CONF_API config_setting_t *config_root_setting(const config_t *c) { return c->root; }

CONF_API config_setting_t *
config_setting_get_member(const config_setting_t *s, const char *name)
{
	int i;
	if(!s || s->type != CONFIG_TYPE_GROUP || !name) return NULL;
	for(i = 0; i < s->nelems; i++)
		if(s->elems[i]->name && !strcmp(s->elems[i]->name, name))
			return s->elems[i];
	return NULL;
}

CONF_API config_setting_t *
config_setting_get_elem(const config_setting_t *s, unsigned int idx)
{
	if(!s || (s->type != CONFIG_TYPE_GROUP && s->type != CONFIG_TYPE_LIST
				&& s->type != CONFIG_TYPE_ARRAY))
		return NULL;
	if(idx >= (unsigned int) s->nelems) return NULL;
	return s->elems[idx];
}

/* Dotted path: names separated by '.', '/' or ':'; "[n]" or a bare
 * number selects an element. */
CONF_API config_setting_t *
config_setting_lookup(config_setting_t *s, const char *path)
{
	char tok[256];
	const char *p = path;
	while(s && *p)
	{
		size_t n = 0;
		while(*p && *p != '.' && *p != '/' && *p != ':' && n + 1 < sizeof(tok))
			tok[n++] = *p++;
		tok[n] = '\0';
		if(*p) p++;
		if(n == 0) continue;
		if(tok[0] == '[' || isdigit((unsigned char) tok[0]))
		{
			char *e;
			long idx = strtol(tok[0] == '[' ? tok + 1 : tok, &e, 10);
			if(idx < 0) return NULL;
			s = config_setting_get_elem(s, (unsigned int) idx);
		}
		else
			s = config_setting_get_member(s, tok);
	}
	return s;
}

CONF_API config_setting_t *
config_lookup(const config_t *c, const char *path)
{
	return config_setting_lookup(c->root, path);
}

CONF_API int config_setting_type(const config_setting_t *s) { return s ? s->type : CONFIG_TYPE_NONE; }
CONF_API const char *config_setting_name(const config_setting_t *s) { return s ? s->name : NULL; }
CONF_API int config_setting_source_line(const config_setting_t *s) { return s ? s->line : 0; }

CONF_API int
config_setting_length(const config_setting_t *s)
{
	if(!s) return 0;
	if(s->type == CONFIG_TYPE_GROUP || s->type == CONFIG_TYPE_LIST || s->type == CONFIG_TYPE_ARRAY)
		return s->nelems;
	return 0;
}

static int
autoconv(const config_setting_t *s)
{
	return s->config && (s->config->options & CONFIG_OPTION_AUTOCONVERT);
}

/* Typed reads: 1 and the value when the setting has (or converts to) the
 * type, 0 otherwise. */
static int
get_int64(const config_setting_t *s, long long *v)
{
	if(!s) return 0;
	if(s->type == CONFIG_TYPE_INT || s->type == CONFIG_TYPE_INT64) { *v = s->ival; return 1; }
	if(s->type == CONFIG_TYPE_FLOAT && autoconv(s)) { *v = (long long) s->fval; return 1; }
	return 0;
}

static int
get_float(const config_setting_t *s, double *v)
{
	if(!s) return 0;
	if(s->type == CONFIG_TYPE_FLOAT) { *v = s->fval; return 1; }
	if((s->type == CONFIG_TYPE_INT || s->type == CONFIG_TYPE_INT64) && autoconv(s))
	{
		*v = (double) s->ival;
		return 1;
	}
	return 0;
}

CONF_API int
config_setting_get_int(const config_setting_t *s)
{
	long long v;
	if(!get_int64(s, &v) || v > 2147483647LL || v < -2147483648LL) return 0;
	return (int) v;
}

CONF_API long long
config_setting_get_int64(const config_setting_t *s)
{
	long long v;
	return get_int64(s, &v) ? v : 0;
}

CONF_API double
config_setting_get_float(const config_setting_t *s)
{
	double v;
	return get_float(s, &v) ? v : 0.0;
}

CONF_API int
config_setting_get_bool(const config_setting_t *s)
{
	return s && s->type == CONFIG_TYPE_BOOL ? (int) s->ival : 0;
}

CONF_API const char *
config_setting_get_string(const config_setting_t *s)
{
	return s && s->type == CONFIG_TYPE_STRING ? s->sval : NULL;
}

CONF_API int
config_setting_get_int_elem(const config_setting_t *s, int idx)
{
	return idx < 0 ? 0 : config_setting_get_int(config_setting_get_elem(s, (unsigned int) idx));
}

CONF_API long long
config_setting_get_int64_elem(const config_setting_t *s, int idx)
{
	return idx < 0 ? 0 : config_setting_get_int64(config_setting_get_elem(s, (unsigned int) idx));
}

CONF_API double
config_setting_get_float_elem(const config_setting_t *s, int idx)
{
	return idx < 0 ? 0.0 : config_setting_get_float(config_setting_get_elem(s, (unsigned int) idx));
}

CONF_API const char *
config_setting_get_string_elem(const config_setting_t *s, int idx)
{
	return idx < 0 ? NULL : config_setting_get_string(config_setting_get_elem(s, (unsigned int) idx));
}

CONF_API int
config_setting_lookup_int64(const config_setting_t *s, const char *name, long long *value)
{
	long long v;
	if(!get_int64(config_setting_get_member(s, name), &v)) return CONFIG_FALSE;
	*value = v;
	return CONFIG_TRUE;
}

CONF_API int
config_setting_lookup_int(const config_setting_t *s, const char *name, int *value)
{
	long long v;
	if(!get_int64(config_setting_get_member(s, name), &v) || v > 2147483647LL || v < -2147483648LL)
		return CONFIG_FALSE;
	*value = (int) v;
	return CONFIG_TRUE;
}

CONF_API int
config_setting_lookup_float(const config_setting_t *s, const char *name, double *value)
{
	double v;
	if(!get_float(config_setting_get_member(s, name), &v)) return CONFIG_FALSE;
	*value = v;
	return CONFIG_TRUE;
}

CONF_API int
config_setting_lookup_bool(const config_setting_t *s, const char *name, int *value)
{
	config_setting_t *m = config_setting_get_member(s, name);
	if(!m || m->type != CONFIG_TYPE_BOOL) return CONFIG_FALSE;
	*value = (int) m->ival;
	return CONFIG_TRUE;
}

CONF_API int
config_setting_lookup_string(const config_setting_t *s, const char *name, const char **value)
{
	config_setting_t *m = config_setting_get_member(s, name);
	if(!m || m->type != CONFIG_TYPE_STRING) return CONFIG_FALSE;
	*value = m->sval;
	return CONFIG_TRUE;
}

CONF_API int
config_lookup_int(const config_t *c, const char *path, int *value)
{
	long long v;
	if(!get_int64(config_lookup(c, path), &v) || v > 2147483647LL || v < -2147483648LL)
		return CONFIG_FALSE;
	*value = (int) v;
	return CONFIG_TRUE;
}

CONF_API int
config_lookup_int64(const config_t *c, const char *path, long long *value)
{
	long long v;
	if(!get_int64(config_lookup(c, path), &v)) return CONFIG_FALSE;
	*value = v;
	return CONFIG_TRUE;
}

CONF_API int
config_lookup_float(const config_t *c, const char *path, double *value)
{
	double v;
	if(!get_float(config_lookup(c, path), &v)) return CONFIG_FALSE;
	*value = v;
	return CONFIG_TRUE;
}

CONF_API int
config_lookup_bool(const config_t *c, const char *path, int *value)
{
	config_setting_t *s = config_lookup(c, path);
	if(!s || s->type != CONFIG_TYPE_BOOL) return CONFIG_FALSE;
	*value = (int) s->ival;
	return CONFIG_TRUE;
}

CONF_API int
config_lookup_string(const config_t *c, const char *path, const char **value)
{
	config_setting_t *s = config_lookup(c, path);
	if(!s || s->type != CONFIG_TYPE_STRING) return CONFIG_FALSE;
	*value = s->sval;
	return CONFIG_TRUE;
}
