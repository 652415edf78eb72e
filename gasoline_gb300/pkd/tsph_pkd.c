/*
 * tsph_pkd -- the reference-side binding of libtsph (see tsph_pkd.h).
 *
 * Every call hands the PKD's particle store (pkd->pStore, PARTICLE structs,
 * pkd.h:90-225) to libtsph with its layout taken from pkd.h by offsetof,
 * registered once so the GPU reads and writes the fields in place, and
 * maps libtsph's caller index to store entries:
 *   - caller index = iOrder when the iOrders of the store are a permutation
 *     of 0..n-1 with the gas first (as a snapshot loads them).  The store
 *     is permuted by every reference tree build, but iOrder names the same
 *     particle from one call to the next, so libtsph keeps its last tree's
 *     order and the next GPU build starts from it;
 *   - otherwise the store's own order with the gas moved first, which is a
 *     new particle set for libtsph at every call.
 */
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "pkd.h"
#include "smooth.h"
#include "smoothfcn.h"
#include "opentype.h"
#include "tsph.h"
#include "tsph_pkd.h"

#define TSPH_PKD_MAX 64

typedef struct {
    PKD pkd;
    tsph_ctx *ctx;
    int device, precision;
    int nBucket, iOpenType;
    double dCrit;
    void *store;          /* registered extent of pStore */
    size_t storeBytes;
    int *order;           /* store entry of every caller index */
    int nOrder, ngas;
} tsph_pkd_entry;

static tsph_pkd_entry g_tab[TSPH_PKD_MAX];

static void die(const char *where, int rc, tsph_ctx *ctx)
{
    fprintf(stderr, "tsph_pkd: %s: %s%s%s\n", where, tsph_error_string(rc),
            ctx ? " " : "", ctx ? tsph_last_cuda_error(ctx) : "");
    abort();
}

static tsph_pkd_entry *lookup(PKD pkd, int create)
{
    int i, free_slot = -1;
    for (i = 0; i < TSPH_PKD_MAX; ++i) {
        if (g_tab[i].pkd == pkd) return &g_tab[i];
        if (!g_tab[i].pkd && free_slot < 0) free_slot = i;
    }
    if (!create) return NULL;
    if (free_slot < 0) die("side table full (more PKDs than TSPH_PKD_MAX)", TSPH_ERR_ARG, NULL);
    memset(&g_tab[free_slot], 0, sizeof(g_tab[free_slot]));
    g_tab[free_slot].pkd = pkd;
    g_tab[free_slot].precision = TSPH_FP32;
    g_tab[free_slot].nBucket = 8;           /* the reference's default nBucket */
    g_tab[free_slot].iOpenType = OPEN_JOSH;
    g_tab[free_slot].dCrit = 0.7;           /* and opening angle (master.c) */
    return &g_tab[free_slot];
}

static tsph_pkd_entry *context(PKD pkd)
{
    tsph_pkd_entry *e = lookup(pkd, 1);
    if (!e->ctx) {
        int rc = tsph_create(&e->ctx, e->device, NULL);
        if (rc) die("tsph_create", rc, NULL);
    }
    return e;
}

void tsph_pkd_attach(PKD pkd, int device, int precision)
{
    tsph_pkd_entry *e = lookup(pkd, 1);
    if (e->ctx && e->device != device) tsph_pkd_detach(pkd), e = lookup(pkd, 1);
    e->device = device;
    e->precision = precision;
}

void tsph_pkd_detach(PKD pkd)
{
    tsph_pkd_entry *e = lookup(pkd, 0);
    if (!e) return;
    if (e->ctx) {
        if (e->store) tsph_store_unregister(e->ctx, e->store);
        tsph_destroy(e->ctx);
    }
    free(e->order);
    memset(e, 0, sizeof(*e));
}

void tsph_pkd_set_tree_params(PKD pkd, int nBucket, int iOpenType, double dCrit)
{
    tsph_pkd_entry *e = lookup(pkd, 1);
    e->nBucket = nBucket;
    e->iOpenType = iOpenType;
    e->dCrit = dCrit;
}

void tsph_pkdBuildBinary(PKD pkd, int nBucket, int iOpenType, double dCrit, int iOrder,
                         int bTreeActiveOnly, int bGravity, KDN *pRoot)
{
    tsph_pkd_set_tree_params(pkd, nBucket, iOpenType, dCrit);
    pkdBuildBinary(pkd, nBucket, iOpenType, dCrit, iOrder, bTreeActiveOnly, bGravity, pRoot);
}

/* The PARTICLE layout of this build of the reference. */
static tsph_store_layout layout(void)
{
    tsph_store_layout L;
    memset(&L, 0, sizeof(L));
    L.stride = (long long)sizeof(PARTICLE);
    L.r = (int)offsetof(PARTICLE, r);
    L.fMass = (int)offsetof(PARTICLE, fMass);
    L.fSoft = (int)offsetof(PARTICLE, fSoft);
    L.v = (int)offsetof(PARTICLE, v);
    L.a = (int)offsetof(PARTICLE, a);
    L.fPot = (int)offsetof(PARTICLE, fPot);
    L.dtGrav = (int)offsetof(PARTICLE, dtGrav);
    L.fBall2 = (int)offsetof(PARTICLE, fBall2);
    L.fDensity = (int)offsetof(PARTICLE, fDensity);
    L.dtNew = (int)offsetof(PARTICLE, dtNew);
#ifdef GASOLINE
    L.vPred = (int)offsetof(PARTICLE, vPred);
    L.u = (int)offsetof(PARTICLE, u);
    L.uPred = (int)offsetof(PARTICLE, uPred);
    L.divv = (int)offsetof(PARTICLE, divv);
    L.curlv = (int)offsetof(PARTICLE, curlv);
    L.dvds = (int)offsetof(PARTICLE, dvds);
    L.BalsaraSwitch = (int)offsetof(PARTICLE, BalsaraSwitch);
    L.diff = (int)offsetof(PARTICLE, diff);
    L.PoverRho2 = (int)offsetof(PARTICLE, PoverRho2);
    L.c = (int)offsetof(PARTICLE, c);
    L.uDotPdV = (int)offsetof(PARTICLE, uDotPdV);
    L.uDotAV = (int)offsetof(PARTICLE, uDotAV);
    L.mumax = (int)offsetof(PARTICLE, mumax);
#else
    L.vPred = L.u = L.uPred = L.divv = L.curlv = L.dvds = L.BalsaraSwitch = L.diff = -1;
    L.PoverRho2 = L.c = L.uDotPdV = L.uDotAV = L.mumax = -1;
#endif
    L.iActive = (int)offsetof(PARTICLE, iActive);
    L.activeBit = TYPE_ACTIVE;
    return L;
}

/* Caller index -> store entry (see the file comment) and the gas count. */
static void map_store(tsph_pkd_entry *e, PKD pkd)
{
    const int n = pkdLocal(pkd);
    PARTICLE *p = pkd->pStore;
    int i, ngas = 0, byIOrder = 1;
    if (e->nOrder < n) {
        free(e->order);
        e->order = malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
        if (!e->order) die("map_store", TSPH_ERR_NOMEM, NULL);
        e->nOrder = n;
    }
    for (i = 0; i < n; ++i) ngas += (p[i].iActive & TYPE_GAS) != 0;
    for (i = 0; i < n; ++i) e->order[i] = -1;
    for (i = 0; i < n && byIOrder; ++i) {
        const int k = p[i].iOrder;
        const int gas = (p[i].iActive & TYPE_GAS) != 0;
        if (k < 0 || k >= n || e->order[k] >= 0 || gas != (k < ngas)) byIOrder = 0;
        else e->order[k] = i;
    }
    if (!byIOrder) {
        int g = 0, d = ngas;
        for (i = 0; i < n; ++i) {
            if (p[i].iActive & TYPE_GAS) e->order[g++] = i;
            else e->order[d++] = i;
        }
    }
    e->ngas = ngas;
}

/* Register the store with CUDA (once, and again when it moved or grew) and
 * load it into the context. */
static void load(tsph_pkd_entry *e, PKD pkd, const tsph_store_layout *L)
{
    const int n = pkdLocal(pkd);
    const size_t bytes = sizeof(PARTICLE) * (size_t)(n > 0 ? n : 1);
    int rc;
    if (e->store != (void *)pkd->pStore || e->storeBytes < bytes) {
        if (e->store) tsph_store_unregister(e->ctx, e->store);
        e->store = NULL;
        rc = tsph_store_register(e->ctx, pkd->pStore, bytes);
        if (rc) die("tsph_store_register", rc, e->ctx);
        e->store = pkd->pStore;
        e->storeBytes = bytes;
    }
    map_store(e, pkd);
    rc = tsph_store_load(e->ctx, n, pkd->pStore, L, e->order, e->ngas);
    if (rc) die("tsph_store_load", rc, e->ctx);
}

void tsph_pkdGravAll(PKD pkd, int nReps, int bPeriodic, int iOrder, int bEwald, int iEwOrder,
                     double fEwCut, double fEwhCut, int bComove, double dRhoFac, int bDoSun,
                     double dSunSoft, double *aSun, int *nActive, double *pdPartSum,
                     double *pdCellSum, double *pdSoftSum, CASTAT *pcs, double *pdFlop)
{
    tsph_pkd_entry *e = context(pkd);
    const tsph_store_layout L = layout();
    tsph_grav_params gp;
    tsph_grav_out out;
    int rc;
    (void)dRhoFac;
    (void)dSunSoft;
    (void)aSun;
    if (bComove || bDoSun) die("comoving and Sun-indirect terms", TSPH_ERR_UNSUPPORTED, NULL);
    if (e->iOpenType != OPEN_JOSH) die("opening criterion other than OPEN_JOSH", TSPH_ERR_UNSUPPORTED, NULL);
    load(e, pkd, &L);
    memset(&gp, 0, sizeof(gp));
    gp.nBucket = e->nBucket;
    gp.iOrder = iOrder;
    gp.bPeriodic = bPeriodic;
    gp.bEwald = bEwald;
    gp.iEwOrder = iEwOrder;
    gp.nReps = nReps;
    gp.dTheta = e->dCrit;
    gp.dPeriod = bPeriodic ? pkd->fPeriod[0] : 1.0;
    gp.fEwCut = fEwCut;
    gp.fEwhCut = fEwhCut;
    gp.precision = e->precision;
    rc = tsph_grav_all(e->ctx, &gp, &out);
    if (rc) die("tsph_grav_all", rc, e->ctx);
    rc = tsph_store_put_gravity(e->ctx, pkd->pStore, &L, e->order);
    if (rc) die("tsph_store_put_gravity", rc, e->ctx);
    *nActive = out.nActive;
    *pdPartSum = out.dPartSum;
    *pdCellSum = out.dCellSum;
    *pdSoftSum = out.dSoftSum;
    *pdFlop = out.dFlop;
    if (pcs) memset(pcs, 0, sizeof(*pcs));   /* no MDL cache traffic on this path */
}

static void sph_params(const SMX smx, const SMF *smf, const tsph_pkd_entry *e, tsph_sph_params *sp)
{
    memset(sp, 0, sizeof(*sp));
    sp->nSmooth = smx->nSmooth;
    sp->bPeriodic = smx->bPeriodic;
    sp->dPeriod = smx->bPeriodic ? smx->lx : 1.0;
    sp->alpha = smf->alpha;
    sp->beta = smf->beta;
    sp->gamma = smf->gamma;
    /* dtFacCourant = dEtaCourant * a * 2/1.6 (pkdDtFacCourant, pkd.c:5893) */
    sp->dEtaCourant = smf->dtFacCourant * 1.6 / (2.0 * (smf->a > 0 ? smf->a : 1.0));
    sp->iViscosityLimiter = smf->iViscosityLimiter;
    sp->precision = e->precision;
}

void tsph_smSmooth(SMX smx, SMF *smf)
{
    PKD pkd = smx->pkd;
    tsph_pkd_entry *e = context(pkd);
    const tsph_store_layout L = layout();
    tsph_sph_params sp;
    tsph_smooth_out out;
    int type, rc;
    if (smx->fcnSmooth == DenDVDX) type = TSPH_SMX_DENDVDX;
    else if (smx->fcnSmooth == Density) type = TSPH_SMX_DENSITY;
    else die("smooth type", TSPH_ERR_UNSUPPORTED, NULL);
    if (smf->H != 0.0 || (smf->a != 1.0 && smf->a != 0.0))
        die("comoving smooth parameters", TSPH_ERR_UNSUPPORTED, NULL);
    load(e, pkd, &L);
    sph_params(smx, smf, e, &sp);
    rc = tsph_smooth(e->ctx, type, &sp, &out);
    if (rc) die("tsph_smooth", rc, e->ctx);
    rc = tsph_store_put_sph(e->ctx, type, pkd->pStore, &L, e->order);
    if (rc) die("tsph_store_put_sph", rc, e->ctx);
    smf->nSmoothed = out.nSmoothed;
}

/* The pressure pass runs on the particles its tsph_smSmooth loaded: msrSph
 * calls smSmooth, pkdGasPressure and smReSmooth back to back on unchanged
 * particles (master.c:9258-9362).  libtsph evaluates the gas pressure
 * itself as part of this pass. */
void tsph_smReSmooth(SMX smx, SMF *smf)
{
    PKD pkd = smx->pkd;
    tsph_pkd_entry *e = context(pkd);
    const tsph_store_layout L = layout();
    tsph_sph_params sp;
    tsph_smooth_out out;
    int rc;
    if (smx->fcnSmooth != SphPressureTermsSym) die("re-smooth type", TSPH_ERR_UNSUPPORTED, NULL);
    if (!e->order) die("tsph_smReSmooth before tsph_smSmooth", TSPH_ERR_STATE, NULL);
    sph_params(smx, smf, e, &sp);
    rc = tsph_smooth(e->ctx, TSPH_SMX_SPHPRESSURETERMS, &sp, &out);
    if (rc) die("tsph_smooth", rc, e->ctx);
    rc = tsph_store_put_sph(e->ctx, TSPH_SMX_SPHPRESSURETERMS, pkd->pStore, &L, e->order);
    if (rc) die("tsph_store_put_sph", rc, e->ctx);
    smf->nSmoothed = out.nSmoothed;
}
