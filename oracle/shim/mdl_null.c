/* Single-rank MDL stand-in; see mdl.h.  Test infrastructure only. */
#include <stdlib.h>
#include <time.h>
#include "mdl.h"

int mdlSelf(MDL mdl) { return mdl->idSelf; }
int mdlThreads(MDL mdl) { return mdl->nThreads; }
void *mdlMalloc(MDL mdl, size_t n) { (void)mdl; return malloc(n); }
void mdlFree(MDL mdl, void *p) { (void)mdl; free(p); }
void mdlROcache(MDL mdl, int cid, void *base, int stride, int n) {
    mdl->cache[cid].base = (char *)base;
    mdl->cache[cid].stride = stride;
    mdl->cache[cid].n = n;
}
void mdlCOcache(MDL mdl, int cid, void *base, int stride, int n,
                void (*init)(void *), void (*comb)(void *, void *)) {
    (void)init; (void)comb;
    mdlROcache(mdl, cid, base, stride, n);
}
void mdlFinishCache(MDL mdl, int cid) { (void)mdl; (void)cid; }
void *mdlAquire(MDL mdl, int cid, int i, int id) {
    (void)id;
    return mdl->cache[cid].base + (size_t)i * (size_t)mdl->cache[cid].stride;
}
void mdlRelease(MDL mdl, int cid, void *p) { (void)mdl; (void)cid; (void)p; }
void mdlCacheCheck(MDL mdl) { (void)mdl; }
double mdlNumAccess(MDL mdl, int cid) { (void)mdl; (void)cid; return 0; }
double mdlMissRatio(MDL mdl, int cid) { (void)mdl; (void)cid; return 0; }
double mdlCollRatio(MDL mdl, int cid) { (void)mdl; (void)cid; return 0; }
double mdlMinRatio(MDL mdl, int cid) { (void)mdl; (void)cid; return 0; }
double mdlCpuTimer(MDL mdl) { (void)mdl; return (double)clock() / CLOCKS_PER_SEC; }
void mdlDiag(MDL mdl, char *psz) { (void)mdl; (void)psz; }
int mdlSwap(MDL mdl, int id, size_t nBufBytes, void *vBuf, size_t nOutBytes,
            size_t *pnSndBytes, size_t *pnRcvBytes) {
    (void)mdl; (void)id; (void)nBufBytes; (void)vBuf; (void)nOutBytes;
    *pnSndBytes = 0; *pnRcvBytes = 0;
    abort();
}
