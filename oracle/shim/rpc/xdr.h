/* Stand-in for SunRPC <rpc/xdr.h>: every XDR call aborts, since the oracle
 * never reads or writes snapshots.  Test infrastructure only. */
#ifndef TSPH_SHIM_RPC_XDR_H
#define TSPH_SHIM_RPC_XDR_H
#include <stdio.h>
#include <stdlib.h>
#include "types.h"
enum xdr_op { XDR_ENCODE = 0, XDR_DECODE = 1, XDR_FREE = 2 };
typedef struct { enum xdr_op x_op; } XDR;
static inline void xdrstdio_create(XDR *x, FILE *f, enum xdr_op op) { (void)x; (void)f; (void)op; abort(); }
static inline bool_t xdr_float(XDR *x, float *v) { (void)x; (void)v; abort(); return 0; }
static inline bool_t xdr_double(XDR *x, double *v) { (void)x; (void)v; abort(); return 0; }
static inline bool_t xdr_int(XDR *x, int *v) { (void)x; (void)v; abort(); return 0; }
static inline bool_t xdr_u_int(XDR *x, unsigned int *v) { (void)x; (void)v; abort(); return 0; }
static inline bool_t xdr_longlong_t(XDR *x, long long *v) { (void)x; (void)v; abort(); return 0; }
#define xdr_destroy(x) ((void)(x))
#endif
