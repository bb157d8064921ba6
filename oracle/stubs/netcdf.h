/*
 * ORACLE — test infrastructure only.  No-op stand-in for <netcdf.h> so the
 * reference's NetCdfWriter compiles and links; nothing is written.
 */
#ifndef ORACLE_STUB_NETCDF_H
#define ORACLE_STUB_NETCDF_H

#include <stddef.h>

#define NC_NOERR 0
#define NC_NETCDF4 0x1000
#define NC_UNLIMITED 0L
#define NC_FLOAT 5
#define NC_GLOBAL (-1)

static inline int nc_create(const char *p, int m, int *id) { (void)p; (void)m; *id = 0; return NC_NOERR; }
static inline int nc_def_dim(int id, const char *n, size_t l, int *d) { (void)id; (void)n; (void)l; *d = 0; return NC_NOERR; }
static inline int nc_def_var(int id, const char *n, int t, int nd, const int *d, int *v) { (void)id; (void)n; (void)t; (void)nd; (void)d; *v = 0; return NC_NOERR; }
static inline int nc_put_att_text(int id, int v, const char *n, size_t l, const char *s) { (void)id; (void)v; (void)n; (void)l; (void)s; return NC_NOERR; }
static inline int nc_enddef(int id) { (void)id; return NC_NOERR; }
static inline int nc_put_var1_float(int id, int v, const size_t *i, const float *p) { (void)id; (void)v; (void)i; (void)p; return NC_NOERR; }
static inline int nc_put_vara_float(int id, int v, const size_t *s, const size_t *c, const float *p) { (void)id; (void)v; (void)s; (void)c; (void)p; return NC_NOERR; }
static inline int nc_sync(int id) { (void)id; return NC_NOERR; }
static inline int nc_close(int id) { (void)id; return NC_NOERR; }
static inline const char *nc_strerror(int e) { (void)e; return "stub"; }

#endif
