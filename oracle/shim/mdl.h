/*
 * Single-rank "null" stand-in for the MDL communication layer that the
 * reference's per-rank code (pkd.c, walk.c, smooth.c, ...) includes as
 * "mdl.h".  MDL itself is a separate project that is not part of the
 * reference tree.  With one rank every cache access is local, so the
 * cache calls reduce to pointer arithmetic over the registered array.
 *
 * Test infrastructure only: used to compile the reference sources into
 * oracle/_ref/ for pinning the oracle.  Nothing in the product links it.
 */
#ifndef TSPH_ORACLE_NULL_MDL_H
#define TSPH_ORACLE_NULL_MDL_H
#include <stddef.h>
#include <assert.h>

typedef struct mdlContext {
    int idSelf;
    int nThreads;
    struct { char *base; int stride; int n; } cache[4];
} *MDL;

#define mdlassert(mdl, expr) assert(expr)

int mdlSelf(MDL mdl);
int mdlThreads(MDL mdl);
void *mdlMalloc(MDL mdl, size_t n);
void mdlFree(MDL mdl, void *p);
void mdlROcache(MDL mdl, int cid, void *base, int stride, int n);
void mdlCOcache(MDL mdl, int cid, void *base, int stride, int n,
                void (*init)(void *), void (*comb)(void *, void *));
void mdlFinishCache(MDL mdl, int cid);
void *mdlAquire(MDL mdl, int cid, int i, int id);
void mdlRelease(MDL mdl, int cid, void *p);
void mdlCacheCheck(MDL mdl);
double mdlNumAccess(MDL mdl, int cid);
double mdlMissRatio(MDL mdl, int cid);
double mdlCollRatio(MDL mdl, int cid);
double mdlMinRatio(MDL mdl, int cid);
double mdlCpuTimer(MDL mdl);
void mdlDiag(MDL mdl, char *psz);
int mdlSwap(MDL mdl, int id, size_t nBufBytes, void *vBuf, size_t nOutBytes,
            size_t *pnSndBytes, size_t *pnRcvBytes);
#endif
