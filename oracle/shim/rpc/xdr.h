/* Stand-in for SunRPC <rpc/xdr.h>, enough for the reference's Tipsy snapshot
 * I/O (pkdReadTipsy / pkdWriteTipsy) to run in the oracle build.  Written
 * from the XDR standard (RFC 4506): every item is a whole number of 4-byte
 * units in big-endian order; int and float take one unit (a float is its
 * IEEE-754 single bits), double and hyper integers take two, most
 * significant unit first.  Only the stdio stream form is provided.
 * Test infrastructure only. */
#ifndef TSPH_SHIM_RPC_XDR_H
#define TSPH_SHIM_RPC_XDR_H
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "types.h"
enum xdr_op { XDR_ENCODE = 0, XDR_DECODE = 1, XDR_FREE = 2 };
typedef struct { enum xdr_op x_op; FILE *fp; } XDR;

static inline void xdrstdio_create(XDR *x, FILE *f, enum xdr_op op) { x->x_op = op; x->fp = f; }

static inline bool_t tsph_xdr_unit(XDR *x, unsigned int *v) {
    unsigned char b[4];
    if (x->x_op == XDR_ENCODE) {
        b[0] = (unsigned char)(*v >> 24); b[1] = (unsigned char)(*v >> 16);
        b[2] = (unsigned char)(*v >> 8);  b[3] = (unsigned char)(*v);
        return fwrite(b, 1, 4, x->fp) == 4;
    }
    if (x->x_op == XDR_DECODE) {
        if (fread(b, 1, 4, x->fp) != 4) return FALSE;
        *v = ((unsigned int)b[0] << 24) | ((unsigned int)b[1] << 16) |
             ((unsigned int)b[2] << 8) | (unsigned int)b[3];
        return TRUE;
    }
    return TRUE;
}
static inline bool_t tsph_xdr_hyper(XDR *x, unsigned long long *v) {
    unsigned int hi = (unsigned int)(*v >> 32), lo = (unsigned int)*v;
    if (!tsph_xdr_unit(x, &hi) || !tsph_xdr_unit(x, &lo)) return FALSE;
    *v = ((unsigned long long)hi << 32) | lo;
    return TRUE;
}
static inline bool_t xdr_u_int(XDR *x, unsigned int *v) { return tsph_xdr_unit(x, v); }
static inline bool_t xdr_int(XDR *x, int *v) {
    unsigned int u; memcpy(&u, v, 4);
    if (!tsph_xdr_unit(x, &u)) return FALSE;
    memcpy(v, &u, 4); return TRUE;
}
static inline bool_t xdr_float(XDR *x, float *v) {
    unsigned int u; memcpy(&u, v, 4);
    if (!tsph_xdr_unit(x, &u)) return FALSE;
    memcpy(v, &u, 4); return TRUE;
}
static inline bool_t xdr_double(XDR *x, double *v) {
    unsigned long long u; memcpy(&u, v, 8);
    if (!tsph_xdr_hyper(x, &u)) return FALSE;
    memcpy(v, &u, 8); return TRUE;
}
/* an 8-byte integer behind any pointer type (quad_t differs between libcs) */
static inline bool_t xdr_longlong_t(XDR *x, void *v) {
    unsigned long long u; memcpy(&u, v, 8);
    if (!tsph_xdr_hyper(x, &u)) return FALSE;
    memcpy(v, &u, 8); return TRUE;
}
#define xdr_destroy(x) ((void)fflush((x)->fp))
#endif
