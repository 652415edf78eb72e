/*
 * A CPU stand-in for libtsph, for testing the reference-side binding
 * (gasoline_gb300/pkd/tsph_pkd.c) where no GPU is present.
 *
 * TEST INFRASTRUCTURE ONLY.  It implements the libtsph calls the binding
 * makes, with the same argument meanings, on the CPU: the particle-store
 * loads and write-backs follow include/tsph.h field by field, and the
 * arithmetic is the oracle's (orc_grav, orc_sph in tsph_oracle.c), which
 * restates the reference bit for bit.  Built with the reference's sources
 * and the binding into oracle/_ref/libgasadapt.so by build_ref.sh; a
 * harness run through it must reproduce the reference's own outputs.  No
 * arithmetic of the product path lives here.
 */
#include <float.h>
#include <stdlib.h>
#include <string.h>

#include "tsph.h"
#include "tsph_oracle.h"

struct tsph_ctx {
    int n, ngas, loaded, haveGrav, haveDensity, havePressure;
    double *pos, *vel, *mass, *soft, *u;
    int *active;
    double *acc, *pot, *dtg;
    double *sph, *dtNew, *mumax;     /* orc_sph outputs, caller order (gas) */
};

int tsph_create(tsph_ctx **pctx, int device, void *stream)
{
    (void)device;
    (void)stream;
    *pctx = calloc(1, sizeof(tsph_ctx));
    return *pctx ? TSPH_OK : TSPH_ERR_NOMEM;
}

static void release(tsph_ctx *c)
{
    free(c->pos); free(c->vel); free(c->mass); free(c->soft); free(c->u); free(c->active);
    free(c->acc); free(c->pot); free(c->dtg); free(c->sph); free(c->dtNew); free(c->mumax);
}

void tsph_destroy(tsph_ctx *ctx)
{
    if (!ctx) return;
    release(ctx);
    free(ctx);
}

const char *tsph_error_string(int s) { return s ? "error" : "ok"; }
const char *tsph_last_cuda_error(tsph_ctx *ctx) { (void)ctx; return ""; }
int tsph_store_register(tsph_ctx *ctx, void *store, size_t bytes) { (void)ctx; (void)store; (void)bytes; return TSPH_OK; }
int tsph_store_unregister(tsph_ctx *ctx, void *store) { (void)ctx; (void)store; return TSPH_OK; }

static double ld(const void *store, long long stride, int entry, int off)
{
    double v;
    memcpy(&v, (const char *)store + (long long)entry * stride + off, sizeof(v));
    return v;
}
static double *at(void *store, long long stride, int entry, int off)
{
    return (double *)((char *)store + (long long)entry * stride + off);
}

int tsph_store_load(tsph_ctx *c, int n, const void *store, const tsph_store_layout *L,
                    const int *order, int ngas)
{
    int i, k;
    release(c);
    memset(c, 0, sizeof(*c));
    c->n = n;
    c->ngas = ngas;
    c->pos = malloc(sizeof(double) * 3 * (n + 1));
    c->vel = malloc(sizeof(double) * 3 * (n + 1));
    c->mass = malloc(sizeof(double) * (n + 1));
    c->soft = malloc(sizeof(double) * (n + 1));
    c->u = calloc((size_t)n + 1, sizeof(double));
    c->active = malloc(sizeof(int) * (n + 1));
    for (i = 0; i < n; ++i) {
        const int e = order ? order[i] : i;
        for (k = 0; k < 3; ++k) {
            c->pos[3 * i + k] = ld(store, L->stride, e, L->r + 8 * k);
            /* the gas passes take the predicted velocity */
            c->vel[3 * i + k] = i < ngas && L->vPred >= 0 ? ld(store, L->stride, e, L->vPred + 8 * k)
                                : (L->v >= 0 ? ld(store, L->stride, e, L->v + 8 * k) : 0.0);
        }
        c->mass[i] = ld(store, L->stride, e, L->fMass);
        c->soft[i] = ld(store, L->stride, e, L->fSoft);
        if (i < ngas) c->u[i] = L->uPred >= 0 ? ld(store, L->stride, e, L->uPred) : ld(store, L->stride, e, L->u);
        if (L->iActive >= 0) {
            unsigned w;
            memcpy(&w, (const char *)store + (long long)e * L->stride + L->iActive, sizeof(w));
            c->active[i] = (w & L->activeBit) != 0;
        } else {
            c->active[i] = 1;
        }
    }
    c->loaded = 1;
    return TSPH_OK;
}

int tsph_grav_all(tsph_ctx *c, const tsph_grav_params *gp, tsph_grav_out *out)
{
    orc_grav_params og;
    double cnt[5];
    if (!c->loaded) return TSPH_ERR_STATE;
    og.nBucket = gp->nBucket;
    og.iOrder = gp->iOrder;
    og.bPeriodic = gp->bPeriodic;
    og.bEwald = gp->bEwald;
    og.iEwOrder = gp->iEwOrder;
    og.nReps = gp->nReps;
    og.dTheta = gp->dTheta;
    og.dPeriod = gp->dPeriod;
    og.fEwCut = gp->fEwCut;
    og.fEwhCut = gp->fEwhCut;
    c->acc = malloc(sizeof(double) * 3 * (c->n + 1));
    c->pot = malloc(sizeof(double) * (c->n + 1));
    c->dtg = malloc(sizeof(double) * (c->n + 1));
    orc_grav(c->n, c->pos, c->mass, c->soft, &og, c->acc, c->pot, c->dtg, cnt, 1);
    memset(out, 0, sizeof(*out));
    out->nActive = (int)cnt[0];
    out->dPartSum = cnt[1];
    out->dCellSum = cnt[2];
    out->dSoftSum = cnt[3];
    out->dFlop = cnt[4];
    c->haveGrav = 1;
    return TSPH_OK;
}

int tsph_store_put_gravity(tsph_ctx *c, void *store, const tsph_store_layout *L, const int *order)
{
    int i, k;
    if (!c->haveGrav) return TSPH_ERR_STATE;
    for (i = 0; i < c->n; ++i) {
        const int e = order ? order[i] : i;
        if (!c->active[i]) continue;
        for (k = 0; k < 3; ++k) *at(store, L->stride, e, L->a + 8 * k) += c->acc[3 * i + k];
        *at(store, L->stride, e, L->fPot) += c->pot[i];
        if (c->dtg[i] > *at(store, L->stride, e, L->dtGrav)) *at(store, L->stride, e, L->dtGrav) = c->dtg[i];
    }
    return TSPH_OK;
}

int tsph_smooth(tsph_ctx *c, int type, const tsph_sph_params *sp, tsph_smooth_out *out)
{
    orc_sph_params os;
    if (!c->loaded) return TSPH_ERR_STATE;
    memset(out, 0, sizeof(*out));
    if (type == TSPH_SMX_SPHPRESSURETERMS) {   /* computed with the density pass */
        if (!c->haveDensity) return TSPH_ERR_STATE;
        c->havePressure = 1;
        out->nSmoothed = c->ngas;
        return TSPH_OK;
    }
    os.nSmooth = sp->nSmooth;
    os.bPeriodic = sp->bPeriodic;
    os.dPeriod = sp->dPeriod;
    os.alpha = sp->alpha;
    os.beta = sp->beta;
    os.gamma = sp->gamma;
    os.dEtaCourant = sp->dEtaCourant;
    os.nBucket = 16;
    os.iViscosityLimiter = sp->iViscosityLimiter;
    c->sph = malloc(sizeof(double) * 16 * (c->ngas + 1));
    c->dtNew = malloc(sizeof(double) * (c->ngas + 1));
    c->mumax = malloc(sizeof(double) * (c->ngas + 1));
    orc_sph(c->ngas, c->pos, c->vel, c->mass, c->soft, c->u, &os, c->sph, c->dtNew, c->mumax,
            NULL, NULL, 1);
    c->haveDensity = 1;
    out->nSmoothed = c->ngas;
    return TSPH_OK;
}

int tsph_store_put_sph(tsph_ctx *c, int which, void *store, const tsph_store_layout *L, const int *order)
{
    int i, k;
    if (!c->haveDensity || (which == TSPH_SMX_SPHPRESSURETERMS && !c->havePressure)) return TSPH_ERR_STATE;
    for (i = 0; i < c->ngas; ++i) {
        const int e = order ? order[i] : i;
        const double *o = &c->sph[16 * i];
        if (which == TSPH_SMX_SPHPRESSURETERMS) {
            if (!c->active[i]) continue;
            *at(store, L->stride, e, L->PoverRho2) = o[9];
            *at(store, L->stride, e, L->c) = o[10];
            for (k = 0; k < 3; ++k) *at(store, L->stride, e, L->a + 8 * k) += o[11 + k];
            *at(store, L->stride, e, L->uDotPdV) = o[14];
            *at(store, L->stride, e, L->uDotAV) = o[15];
            *at(store, L->stride, e, L->mumax) = c->mumax[i];
            if (c->dtNew[i] < *at(store, L->stride, e, L->dtNew)) *at(store, L->stride, e, L->dtNew) = c->dtNew[i];
            continue;
        }
        *at(store, L->stride, e, L->fBall2) = o[0];
        *at(store, L->stride, e, L->fDensity) = o[1];
        *at(store, L->stride, e, L->divv) = o[2];
        for (k = 0; k < 3; ++k) *at(store, L->stride, e, L->curlv + 8 * k) = o[3 + k];
        *at(store, L->stride, e, L->dvds) = o[6];
        *at(store, L->stride, e, L->BalsaraSwitch) = o[7];
        *at(store, L->stride, e, L->diff) = o[8];
    }
    return TSPH_OK;
}
