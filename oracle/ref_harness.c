/*
 * Harness around the UNMODIFIED reference sources (gasoline pkd.c, walk.c,
 * grav.c, ewald.c, v_sqrt1.c, smooth.c, smoothfcn.c), compiled from where
 * they lie by oracle/build_ref.sh into oracle/_ref/libgasref.so.
 *
 * TEST INFRASTRUCTURE ONLY.  It is used in this container to pin the C
 * restatement in oracle/tsph_oracle.c and to write golden fixtures under
 * tests/golden/.  Nothing in the product links or calls it.
 *
 * It reproduces, for a single rank, what the reference's master/PST layers
 * do around the per-rank kernels:
 *   msrBuildTree (master.c:4249-4308): pkdBuildBinary, a one-cell top tree
 *     (pstColCells pst.c:3924-3929 with pLower = rank id 0), pkdCalcRoot +
 *     pkdDistribRoot for Ewald;
 *   msrGravity -> pstGravity -> pkdGravAll (pst.c:3310-3315);
 *   msrSph (master.c:9258-9362): pkdBuildLocal, smSmooth(SMX_DENDVDX),
 *     pkdGasPressure, smReSmooth(SMX_SPHPRESSURETERMS).
 * Inputs and outputs are SoA arrays indexed by iOrder (input order).
 *
 * Built with -DTSPH_ADAPTER (oracle/_ref/libgasadapt.so), ref_grav and
 * ref_sph run the same sequence through the reference-side binding of
 * libtsph instead (gasoline_gb300/pkd/tsph_pkd.c: tsph_pkdBuildBinary,
 * tsph_pkdGravAll, tsph_smSmooth, tsph_smReSmooth at the call sites of
 * pstBuildTree, pstGravity, pstSmooth and pstReSmooth), linked against the
 * CPU stand-in of libtsph in adapter_fake_tsph.c.
 */
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <float.h>
#include "pkd.h"
#include "walk.h"
#include "grav.h"
#include "ewald.h"
#include "smooth.h"
#include "smoothfcn.h"
#include "opentype.h"
#ifdef TSPH_ADAPTER
#include "tsph_pkd.h"
#define BUILD_BINARY tsph_pkdBuildBinary
#define GRAV_ALL tsph_pkdGravAll
#define SM_SMOOTH tsph_smSmooth
#define SM_RESMOOTH tsph_smReSmooth
#else
#define BUILD_BINARY pkdBuildBinary
#define GRAV_ALL pkdGravAll
#define SM_SMOOTH smSmooth
#define SM_RESMOOTH smReSmooth
#endif

typedef struct {
    int nBucket;
    int iOrder;        /* multipole order of cell interactions (2 = quadrupole) */
    int bPeriodic;
    int bEwald;
    int iEwOrder;
    int nReps;
    double dTheta;
    double dPeriod;
    double fEwCut;
    double fEwhCut;
} ref_grav_params;

static struct mdlContext g_mdl;

static PKD make_pkd(int n, const double *pos, const double *mass,
                    const double *soft, int bPeriodic, double dPeriod,
                    int iOrder, int bGas)
{
    PKD pkd;
    FLOAT fPeriod[3];
    int i, j;
    memset(&g_mdl, 0, sizeof(g_mdl));
    g_mdl.idSelf = 0;
    g_mdl.nThreads = 1;
    for (j = 0; j < 3; ++j) fPeriod[j] = bPeriodic ? dPeriod : FLOAT_MAXVAL;
    pkdInitialize(&pkd, &g_mdl, iOrder, n, 0, fPeriod, 0.0, 0.0,
                  bGas ? 0 : n, bGas ? n : 0, 0);
    pkd->nLocal = n;
    pkd->nActive = n;
    pkd->nTreeActive = n;
    pkd->nSmoothActive = n;
    for (i = 0; i < n; ++i) {
        PARTICLE *p = &pkd->pStore[i];
        memset(p, 0, sizeof(*p));
        p->iOrder = i;
        p->iActive = TYPE_ACTIVE | TYPE_TREEACTIVE | TYPE_SMOOTHACTIVE |
                     (bGas ? TYPE_GAS : TYPE_DARK);
        p->fMass = mass[i];
        p->fSoft = soft[i];
        p->fSoft0 = soft[i];
        for (j = 0; j < 3; ++j) p->r[j] = pos[3 * i + j];
        p->fBall2 = 0.0;
        p->fBallMax = 0.0;
        p->dt = FLT_MAX;
        p->dtGrav = 0.0;
    }
    return pkd;
}

/* One-rank top tree: kdTop[ROOT] is the local root with pLower = rank 0. */
static void make_top(PKD pkd, KDN *pRoot)
{
    pkd->kdTop = malloc(2 * sizeof(KDN));
    pkd->piLeaf = malloc(sizeof(int));
    memset(pkd->kdTop, 0, 2 * sizeof(KDN));
    pkd->kdTop[ROOT] = *pRoot;
    pkd->kdTop[ROOT].pLower = 0;
    if (pkd->kdTop[ROOT].pUpper < 0) pkd->kdTop[ROOT].pUpper = -1;
    pkd->kdTop[ROOT].iLower = -1;
    pkd->kdTop[ROOT].iUpper = -1;
    pkd->piLeaf[0] = ROOT;
}

static void build_grav_tree(PKD pkd, const ref_grav_params *gp)
{
    KDN root;
    struct ilCellNewt rootmom;
    int iOrderTree = gp->iOrder;
    if (gp->bPeriodic && gp->bEwald && gp->iEwOrder > iOrderTree)
        iOrderTree = gp->iEwOrder;
    BUILD_BINARY(pkd, gp->nBucket, OPEN_JOSH, gp->dTheta, iOrderTree,
                 0, 1, &root);
    make_top(pkd, &root);
    pkdCalcRoot(pkd, &rootmom);
    pkdDistribRoot(pkd, &rootmom);
}

/*
 * Gravity: one pkdGravAll over all particles.  Outputs a[3n], pot[n],
 * dtGrav[n] (by iOrder), counters[5] = nActive, dPartSum, dCellSum,
 * dSoftSum, dFlop.  Returns the number of tree nodes.
 */
int ref_grav(int n, const double *pos, const double *mass, const double *soft,
             const ref_grav_params *gp, double *acc, double *pot,
             double *dtGrav, double *counters)
{
    PKD pkd = make_pkd(n, pos, mass, soft, gp->bPeriodic, gp->dPeriod,
                       gp->iOrder, 0);
    int nActive = 0, i, j, nNodes;
    double dPartSum, dCellSum, dSoftSum, dFlop;
    CASTAT cs;
    double aSun[3] = {0, 0, 0};
    build_grav_tree(pkd, gp);
    for (i = 0; i < n; ++i) {
        PARTICLE *p = &pkd->pStore[i];
        for (j = 0; j < 3; ++j) p->a[j] = 0.0;
        p->fPot = 0.0;
        p->dtGrav = 0.0;
    }
    GRAV_ALL(pkd, gp->bPeriodic ? gp->nReps : 0, gp->bPeriodic, gp->iOrder,
               gp->bEwald, gp->iEwOrder, gp->fEwCut, gp->fEwhCut, 0, 0.0, 0,
               0.0, aSun, &nActive, &dPartSum, &dCellSum, &dSoftSum, &cs,
               &dFlop);
    for (i = 0; i < n; ++i) {
        PARTICLE *p = &pkd->pStore[i];
        int k = p->iOrder;
        for (j = 0; j < 3; ++j) acc[3 * k + j] = p->a[j];
        pot[k] = p->fPot;
        dtGrav[k] = p->dtGrav;
    }
    counters[0] = nActive;
    counters[1] = dPartSum;
    counters[2] = dCellSum;
    counters[3] = dSoftSum;
    counters[4] = dFlop;
    nNodes = pkd->nNodes;
#ifdef TSPH_ADAPTER
    tsph_pkd_detach(pkd);
#endif
    pkdFinish(pkd);
    return nNodes;
}

/*
 * Tree export for cell-membership parity.  Writes, for every node in the
 * reference's own node order (depth-first, pkd.c:2452-2453):
 *   inode[6*i+..] = pLower, pUpper, iDim, iLower, iUpper (threaded), 0
 *   dnode[16*i+..] = fSplit, bnd.fMin[3], bnd.fMax[3], fMass, fSoft, r[3],
 *                    fOpen2, Bmax, Qxx, Qyy
 * and perm[pos] = iOrder of the particle at storage position pos.
 * Returns the node count (call with inode == NULL to size buffers).
 */
int ref_tree(int n, const double *pos, const double *mass, const double *soft,
             const ref_grav_params *gp, int *inode, double *dnode, int *perm)
{
    PKD pkd = make_pkd(n, pos, mass, soft, gp->bPeriodic, gp->dPeriod,
                       gp->iOrder, 0);
    int i, j, nNodes;
    build_grav_tree(pkd, gp);
    nNodes = pkd->nNodes;
    if (inode) {
        for (i = 0; i < nNodes; ++i) {
            KDN *c = &pkd->kdNodes[i];
            inode[6 * i + 0] = c->pLower;
            inode[6 * i + 1] = c->pUpper;
            inode[6 * i + 2] = c->iDim;
            inode[6 * i + 3] = c->iLower;
            inode[6 * i + 4] = c->iUpper;
            inode[6 * i + 5] = 0;
            dnode[16 * i + 0] = c->fSplit;
            for (j = 0; j < 3; ++j) {
                dnode[16 * i + 1 + j] = c->bnd.fMin[j];
                dnode[16 * i + 4 + j] = c->bnd.fMax[j];
                dnode[16 * i + 9 + j] = c->r[j];
            }
            dnode[16 * i + 7] = c->fMass;
            dnode[16 * i + 8] = c->fSoft;
            dnode[16 * i + 12] = c->fOpen2;
            dnode[16 * i + 13] = c->mom.Bmax;
            dnode[16 * i + 14] = c->mom.Qxx;
            dnode[16 * i + 15] = c->mom.Qyy;
        }
        for (i = 0; i < n; ++i) perm[i] = pkd->pStore[i].iOrder;
    }
    pkdFinish(pkd);
    return nNodes;
}

/*
 * Interaction-list lengths per bucket, walked exactly as pkdGravAll does
 * (active-bound swap pkd.c:2917-2944, then pkdBucketWalk).  For each
 * bucket b in threaded-walk order: blist[4*b+..] = node index, nPart,
 * nCellSoft, nCellNewt.  Returns the number of buckets.
 */
int ref_lists(int n, const double *pos, const double *mass, const double *soft,
              const ref_grav_params *gp, int *blist)
{
    PKD pkd = make_pkd(n, pos, mass, soft, gp->bPeriodic, gp->dPeriod,
                       gp->iOrder, 0);
    KDN *c;
    int iCell, nb = 0, i, j;
    build_grav_tree(pkd, gp);
    c = pkd->kdNodes;
    iCell = pkd->iRoot;
    while (iCell != -1) {
        BND bndActive, bndTmp;
        if (c[iCell].iLower != -1) { iCell = c[iCell].iLower; continue; }
        for (j = 0; j < 3; ++j) {
            bndActive.fMin[j] = FLOAT_MAXVAL;
            bndActive.fMax[j] = -FLOAT_MAXVAL;
        }
        for (i = c[iCell].pLower; i <= c[iCell].pUpper; ++i)
            for (j = 0; j < 3; ++j) {
                if (pkd->pStore[i].r[j] < bndActive.fMin[j]) bndActive.fMin[j] = pkd->pStore[i].r[j];
                if (pkd->pStore[i].r[j] > bndActive.fMax[j]) bndActive.fMax[j] = pkd->pStore[i].r[j];
            }
        bndTmp = c[iCell].bnd;
        c[iCell].bnd = bndActive;
        pkdBucketWalk(pkd, iCell, gp->bPeriodic ? gp->nReps : 0, gp->iOrder);
        c[iCell].bnd = bndTmp;
        if (blist) {
            blist[4 * nb + 0] = iCell;
            blist[4 * nb + 1] = pkd->nPart;
            blist[4 * nb + 2] = pkd->nCellSoft;
            blist[4 * nb + 3] = pkd->nCellNewt;
        }
        ++nb;
        iCell = c[iCell].iUpper;
    }
    pkdFinish(pkd);
    return nb;
}

typedef struct {
    int nSmooth;
    int bPeriodic;
    double dPeriod;
    double alpha;
    double beta;
    double gamma;
    double dEtaCourant;
    int nBucket;
    int iViscosityLimiter;
} ref_sph_params;

/*
 * SPH force pass as in msrSph for the all-active case (master.c:9308-9353):
 * density tree, smSmooth(SMX_DENDVDX, symmetric), pkdGasPressure,
 * smReSmooth(SMX_SPHPRESSURETERMS, symmetric).  Inputs: pos, vel (=vPred),
 * mass, soft, u (=uPred).  Outputs (by iOrder):
 *   out[16*i+..] = fBall2, fDensity, divv, curlv[3], dvds, BalsaraSwitch,
 *                  diff, PoverRho2, c, a_hydro[3], uDotPdV, uDotAV
 *   dtNew[i], mumax[i].
 */
/* The reference's own kNN sets: smSmooth (SMX_DENDVDX set-up, density
 * tree as in ref_sph) with its smooth callback replaced by one that records,
 * per particle, how many entries nnList holds and a hash of their input
 * indices -- the same order-independent hash (sum over the set of a 64-bit
 * mix of iOrder + 1) that the oracle and the CUDA path report -- and the
 * fBall2 smSmooth set.  The post-pass callback is dropped too: nothing was
 * accumulated for it to normalise. */
static unsigned long long *g_knn_hash;
static int *g_knn_cnt;

static void knn_hash_fcn(PARTICLE *p, int nSmooth, NN *nnList, SMF *smf)
{
    unsigned long long h = 0;
    int i;
    (void)smf;
    for (i = 0; i < nSmooth; ++i) {
        unsigned long long x = (unsigned long long)(nnList[i].pPart->iOrder + 1);
        x *= 0x9E3779B97F4A7C15ULL;
        x ^= x >> 29;
        x *= 0xBF58476D1CE4E5B9ULL;
        x ^= x >> 32;
        h += x;
    }
    g_knn_hash[p->iOrder] = h;
    g_knn_cnt[p->iOrder] = nSmooth;
}

int ref_knn_sets(int n, const double *pos, const double *mass, const double *soft,
                 const ref_sph_params *sp, unsigned long long *hash, int *cnt, double *fBall2)
{
    PKD pkd = make_pkd(n, pos, mass, soft, sp->bPeriodic, sp->dPeriod, 2, 1);
    KDN root;
    SMX smx;
    SMF smf;
    CASTAT cs;
    int i;
    memset(&smf, 0, sizeof(smf));
    smf.a = 1.0;
    smf.bCannonical = 1;
    g_knn_hash = hash;
    g_knn_cnt = cnt;
    pkdBuildLocal(pkd, sp->nBucket, OPEN_JOSH, 0.7, 2, 1, 0, &root);
    make_top(pkd, &root);
    smInitialize(&smx, pkd, &smf, sp->nSmooth, sp->bPeriodic, 1, SMX_DENDVDX, 1, 0.0);
    smx->fcnSmooth = knn_hash_fcn;
    smx->fcnPost = NULL;
    smSmooth(smx, &smf);
    smFinish(smx, &smf, &cs);
    for (i = 0; i < n; ++i) fBall2[pkd->pStore[i].iOrder] = pkd->pStore[i].fBall2;
    pkdFinish(pkd);
    g_knn_hash = NULL;
    g_knn_cnt = NULL;
    return 0;
}

int ref_sph(int n, const double *pos, const double *vel, const double *mass,
            const double *soft, const double *u, const ref_sph_params *sp,
            double *out, double *dtNew, double *mumax)
{
    PKD pkd = make_pkd(n, pos, mass, soft, sp->bPeriodic, sp->dPeriod, 2, 1);
    KDN root;
    SMX smx;
    SMF smf;
    CASTAT cs;
    struct GasPressureContext gpc;
    int i, j;
    for (i = 0; i < n; ++i) {
        PARTICLE *p = &pkd->pStore[i];
        for (j = 0; j < 3; ++j) {
            p->v[j] = vel[3 * i + j];
            p->vPred[j] = vel[3 * i + j];
        }
        p->u = u[i];
        p->uPred = u[i];
    }
    memset(&smf, 0, sizeof(smf));
    smf.H = 0.0;
    smf.a = 1.0;
    smf.alpha = sp->alpha;
    smf.beta = sp->beta;
    smf.gamma = sp->gamma;
    smf.algam = smf.alpha * sqrt(smf.gamma * (smf.gamma - 1));
    smf.iViscosityLimiter = sp->iViscosityLimiter;
    smf.dtFacCourant = pkdDtFacCourant(sp->dEtaCourant, smf.a);
    smf.dtFacDiffusion = 2 * 0.1;
    smf.bCannonical = 1;
    smf.dtMin = FLOAT_MAXVAL;
    smf.bStepZero = 1;

    /* density tree: msrBuildTree(bTreeActiveOnly=1, bSmooth=1) */
    pkdBuildLocal(pkd, sp->nBucket, OPEN_JOSH, 0.7, 2, 1, 0, &root);
    make_top(pkd, &root);
    smInitialize(&smx, pkd, &smf, sp->nSmooth, sp->bPeriodic, 1, SMX_DENDVDX, 1, 0.0);
    SM_SMOOTH(smx, &smf);
    smFinish(smx, &smf, &cs);

    memset(&gpc, 0, sizeof(gpc));
    gpc.iGasModel = GASMODEL_ADIABATIC;
    gpc.gamma = sp->gamma;
    gpc.gammam1 = sp->gamma - 1;
    gpc.dResolveJeans = 0.0;
    gpc.dCosmoFac = 1.0;
    gpc.dtFacCourant = smf.dtFacCourant;
    pkdGasPressure(pkd, &gpc);

    for (i = 0; i < n; ++i) {
        PARTICLE *p = &pkd->pStore[i];
        for (j = 0; j < 3; ++j) p->a[j] = 0.0;
    }
    smInitialize(&smx, pkd, &smf, sp->nSmooth, sp->bPeriodic, 1, SMX_SPHPRESSURETERMS, 0, 0.0);
    SM_RESMOOTH(smx, &smf);
    smFinish(smx, &smf, &cs);

    for (i = 0; i < n; ++i) {
        PARTICLE *p = &pkd->pStore[i];
        int k = p->iOrder;
        double *o = &out[16 * k];
        o[0] = p->fBall2;
        o[1] = p->fDensity;
        o[2] = p->divv;
        o[3] = p->curlv[0];
        o[4] = p->curlv[1];
        o[5] = p->curlv[2];
        o[6] = p->dvds;
        o[7] = p->BalsaraSwitch;
        o[8] = p->diff;
        o[9] = p->PoverRho2;
        o[10] = p->c;
        o[11] = p->a[0];
        o[12] = p->a[1];
        o[13] = p->a[2];
        o[14] = p->uDotPdV;
        o[15] = p->uDotAV;
        dtNew[k] = p->dtNew;
        mumax[k] = p->mumax;
    }
#ifdef TSPH_ADAPTER
    tsph_pkd_detach(pkd);
#endif
    pkdFinish(pkd);
    return 0;
}

/* The PARTICLE layout of this build (sizeof and byte offsets, in the order
 * of tsph_store_layout's fields), for the store-layout fixture the GPU tests
 * use where the reference's headers are absent. */
void ref_particle_layout(long long *o)
{
    o[0] = (long long)sizeof(PARTICLE);
    o[1] = offsetof(PARTICLE, r);
    o[2] = offsetof(PARTICLE, fMass);
    o[3] = offsetof(PARTICLE, fSoft);
    o[4] = offsetof(PARTICLE, v);
    o[5] = offsetof(PARTICLE, vPred);
    o[6] = offsetof(PARTICLE, u);
    o[7] = offsetof(PARTICLE, uPred);
    o[8] = offsetof(PARTICLE, a);
    o[9] = offsetof(PARTICLE, fPot);
    o[10] = offsetof(PARTICLE, dtGrav);
    o[11] = offsetof(PARTICLE, fBall2);
    o[12] = offsetof(PARTICLE, fDensity);
    o[13] = offsetof(PARTICLE, divv);
    o[14] = offsetof(PARTICLE, curlv);
    o[15] = offsetof(PARTICLE, dvds);
    o[16] = offsetof(PARTICLE, BalsaraSwitch);
    o[17] = offsetof(PARTICLE, diff);
    o[18] = offsetof(PARTICLE, PoverRho2);
    o[19] = offsetof(PARTICLE, c);
    o[20] = offsetof(PARTICLE, uDotPdV);
    o[21] = offsetof(PARTICLE, uDotAV);
    o[22] = offsetof(PARTICLE, mumax);
    o[23] = offsetof(PARTICLE, dtNew);
    o[24] = offsetof(PARTICLE, iActive);
    o[25] = TYPE_ACTIVE;
    o[26] = offsetof(PARTICLE, iOrder);
    o[27] = TYPE_GAS;
}

/* The reference's approximate 1/sqrt (v_sqrt1.c:11), exported for tests. */
void v_sqrt1(int, double *, double *);
void ref_v_sqrt1(int n, double *r2, double *a) { v_sqrt1(n, r2, a); }

/*
 * Tipsy snapshot I/O through the reference's own pkdReadTipsy (pkd.c:297-686)
 * and pkdWriteTipsy (pkd.c:1628-1798), with the stdio XDR stand-in in
 * shim/rpc/xdr.h for the standard (big-endian) form.  The 32-byte header
 * is written the way msrWriteTipsy does (master.c:3999-4013): xdrHeader's
 * field order (master.c:3563-3575) for the standard form, the struct dump
 * of tipsydefs.h as it lies in memory for the native form.
 * Per-particle arrays are in file order (gas, dark, star):
 *   f[9*i + ..] = mass, soft (eps), u, rho, metals, tform, phi, 0, 0
 * pos/vel are [3n].  Returns 0, or -1 when a file cannot be opened.
 */
#include <rpc/types.h>
#include <rpc/xdr.h>
#include "tipsydefs.h"

static int tipsy_type_of(int i, int nGas, int nDark)
{
    return i < nGas ? TYPE_GAS : (i < nGas + nDark ? TYPE_DARK : TYPE_STAR);
}

int ref_tipsy_write(const char *fname, int bStandard, double time, int nGas,
                    int nDark, int nStar, double dvFac, double duTFac,
                    const double *pos, const double *vel, const double *f)
{
    int n = nGas + nDark + nStar, i, j;
    struct dump h;
    FILE *fp = fopen(fname, "wb");
    PKD pkd;
    FLOAT fPeriod[3] = {FLOAT_MAXVAL, FLOAT_MAXVAL, FLOAT_MAXVAL};
    if (!fp) return -1;
    memset(&h, 0, sizeof(h));
    h.time = time; h.nbodies = n; h.ndim = 3;
    h.nsph = nGas; h.ndark = nDark; h.nstar = nStar;
    if (bStandard) {
        XDR xdrs;
        int pad = 0;
        xdrstdio_create(&xdrs, fp, XDR_ENCODE);
        xdr_double(&xdrs, &h.time);
        xdr_int(&xdrs, &h.nbodies); xdr_int(&xdrs, &h.ndim);
        xdr_int(&xdrs, &h.nsph); xdr_int(&xdrs, &h.ndark);
        xdr_int(&xdrs, &h.nstar); xdr_int(&xdrs, &pad);
        xdr_destroy(&xdrs);
    } else {
        fwrite(&h, sizeof(struct dump), 1, fp);
    }
    fclose(fp);
    memset(&g_mdl, 0, sizeof(g_mdl));
    g_mdl.nThreads = 1;
    pkdInitialize(&pkd, &g_mdl, 2, n > 0 ? n : 1, 0, fPeriod, 0.0, 0.0, nDark, nGas, nStar);
    pkd->nLocal = n;
    for (i = 0; i < n; ++i) {
        PARTICLE *p = &pkd->pStore[i];
        const double *q = &f[9 * i];
        memset(p, 0, sizeof(*p));
        p->iOrder = i;
        p->iActive = tipsy_type_of(i, nGas, nDark);
        for (j = 0; j < 3; ++j) { p->r[j] = pos[3 * i + j]; p->v[j] = vel[3 * i + j]; }
        p->fMass = q[0]; p->fSoft = p->fSoft0 = q[1]; p->u = q[2];
        p->fDensity = q[3]; p->fMetals = q[4]; p->fTimeForm = q[5]; p->fPot = q[6];
    }
    pkdWriteTipsy(pkd, (char *)fname, 0, bStandard, dvFac, duTFac, GASMODEL_ADIABATIC);
    pkdFinish(pkd);
    return 0;
}

int ref_tipsy_read(const char *fname, int bStandard, int nGas, int nDark, int nStar,
                   double dvFac, double dTuFac, double *pos, double *vel, double *f)
{
    int n = nGas + nDark + nStar, i, j;
    PKD pkd;
    FLOAT fPeriod[3] = {FLOAT_MAXVAL, FLOAT_MAXVAL, FLOAT_MAXVAL};
    FILE *fp = fopen(fname, "rb");
    if (!fp) return -1;
    fclose(fp);
    memset(&g_mdl, 0, sizeof(g_mdl));
    g_mdl.nThreads = 1;
    pkdInitialize(&pkd, &g_mdl, 2, n > 0 ? n : 1, 0, fPeriod, 0.0, 0.0, nDark, nGas, nStar);
    pkdReadTipsy(pkd, (char *)fname, 0, n, bStandard, 0, dvFac, dTuFac);
    for (i = 0; i < n; ++i) {
        PARTICLE *p = &pkd->pStore[i];
        double *q = &f[9 * i];
        for (j = 0; j < 3; ++j) { pos[3 * i + j] = p->r[j]; vel[3 * i + j] = p->v[j]; }
        q[0] = p->fMass; q[1] = p->fSoft; q[2] = p->u; q[3] = p->fDensity;
        q[4] = p->fMetals; q[5] = p->fTimeForm; q[6] = p->fPot; q[7] = q[8] = 0.0;
    }
    pkdFinish(pkd);
    return 0;
}

/*
 * Adaptive multistepping (rungs) as msrTopStepKDK drives it
 * (master.c:8242-8465), restated for one rank around the reference's own
 * pkd-level functions: pkdKick / pkdDrift / pkdKickVpred (master.c:6306-6741
 * supply their factors for a non-comoving, canonical run: dvFacOne = 1,
 * dvFacTwo = dt), pkdInitAccel, pkdGravAll over the active rungs,
 * the non-FastGas msrSph (master.c:9258-9362), pkdInitDt, pkdGravStep,
 * pkdAccelStep, pkdSphStep, pkdDtToRung (msrDtToRung master.c:7980-8004,
 * nTruncateRung 0) and pkdEmergencyAdjust (msrEmergencyAdjust
 * master.c:6742-6763).  Initial forces as main.c:360-386 and msrInitSph
 * (all particles active, rungs 0).  The first ngas particles are gas.
 *
 * Outputs by iOrder: pos, vel, vPred [3n]; a [3n] (total); f[12*i + ..] =
 * u, uPred, fPot, dtGrav, dt, dtNew, mumax, fDensity, fBall2, uDotPdV,
 * uDotAV, rung; per top step maxRung[s] (iCurrMaxRung after it) and
 * counts[0] = force passes, counts[1] = sum of active particles over the
 * gravity passes.
 */
typedef struct {
    int nSteps;
    int iMaxRung;
    double dDelta;
    double dEta;
    int bGravStep;
    int bEpsAccStep;
    int bSqrtPhiStep;
    double dEtauDot;
    double duMinDt;
} ref_step_params;

typedef struct {
    PKD pkd;
    const ref_grav_params *gp;
    const ref_sph_params *sp;
    const ref_step_params *st;
    int ngas;
    int iCurrMaxRung;
    double counts[2];
} MSH;

static void msh_smf(SMF *smf, const ref_sph_params *sp)
{
    memset(smf, 0, sizeof(*smf));
    smf->H = 0.0;
    smf->a = 1.0;
    smf->alpha = sp->alpha;
    smf->beta = sp->beta;
    smf->gamma = sp->gamma;
    smf->algam = smf->alpha * sqrt(smf->gamma * (smf->gamma - 1));
    smf->iViscosityLimiter = sp->iViscosityLimiter;
    smf->dtFacCourant = pkdDtFacCourant(sp->dEtaCourant, smf->a);
    smf->dtFacDiffusion = 2 * 0.1;
    smf->bCannonical = 1;
    smf->dtMin = FLOAT_MAXVAL;
}

static UHC msh_uhc(void)
{
    UHC u;
    memset(&u, 0, sizeof(u));
    return u;
}

/* msrActiveRung + msrKickKDKOpen / msrKickKDKClose (master.c:6540-6741) */
static void msh_kick(MSH *m, int iRung, double dDelta, int bClose)
{
    pkdActiveRung(m->pkd, iRung, 0);
    pkdKick(m->pkd, 1.0, dDelta, 1.0, bClose ? dDelta : 0.0, dDelta, bClose ? dDelta : 0.0,
            GASMODEL_ADIABATIC, 0.0, 0.0, 0.0, msh_uhc());
}

/* msrDrift (master.c:6306-6437): pkdDrift then pkdKickVpred */
static void msh_drift(MSH *m, double dDelta)
{
    FLOAT fCenter[3] = {0, 0, 0};
    pkdDrift(m->pkd, dDelta, fCenter, m->gp->bPeriodic, 0, 0, 0.0, 0.0);
    if (dDelta != 0.0)
        pkdKickVpred(m->pkd, 1.0, dDelta, dDelta, GASMODEL_ADIABATIC, 0.0, 0.0, 0.0, msh_uhc());
}

/* msrSph for the non-FastGas branch (master.c:9258-9362) */
static void msh_sph(MSH *m, int iKickRung)
{
    PKD pkd = m->pkd;
    KDN root;
    SMX smx;
    SMF smf;
    CASTAT cs;
    struct GasPressureContext gpc;
    msh_smf(&smf, m->sp);
    pkdActiveTypeRung(pkd, TYPE_GAS, TYPE_ACTIVE, iKickRung, 1);
    pkdActiveType(pkd, TYPE_GAS, TYPE_TREEACTIVE | TYPE_SMOOTHACTIVE);
    pkdBuildLocal(pkd, m->sp->nBucket, OPEN_JOSH, 0.7, 2, 1, 0, &root);
    free(pkd->kdTop); free(pkd->piLeaf);
    make_top(pkd, &root);
    pkdActiveTypeRung(pkd, TYPE_GAS, TYPE_ACTIVE, iKickRung, 1);
    pkdResetType(pkd, TYPE_GAS, TYPE_SMOOTHDONE | TYPE_NbrOfACTIVE);
    pkdActiveType(pkd, TYPE_ACTIVE, TYPE_SMOOTHACTIVE | TYPE_DensACTIVE);
    pkdActiveType(pkd, TYPE_GAS, TYPE_SMOOTHACTIVE);
    smInitialize(&smx, pkd, &smf, m->sp->nSmooth, m->sp->bPeriodic, 1, SMX_DENDVDX, 1, 0.0);
    smSmooth(smx, &smf);
    smFinish(smx, &smf, &cs);
    pkdActiveType(pkd, TYPE_NbrOfACTIVE, TYPE_SMOOTHACTIVE);
    memset(&gpc, 0, sizeof(gpc));
    gpc.iGasModel = GASMODEL_ADIABATIC;
    gpc.gamma = m->sp->gamma;
    gpc.gammam1 = m->sp->gamma - 1;
    gpc.dResolveJeans = 0.0;
    gpc.dCosmoFac = 1.0;
    gpc.dtFacCourant = smf.dtFacCourant;
    pkdGasPressure(pkd, &gpc);
    smInitialize(&smx, pkd, &smf, m->sp->nSmooth, m->sp->bPeriodic, 1, SMX_SPHPRESSURETERMS, 0, 0.0);
    smReSmooth(smx, &smf);
    smFinish(smx, &smf, &cs);
}

/* the force pass of msrTopStepKDK (master.c:8397-8436) */
static void msh_forces(MSH *m, int iKickRung)
{
    PKD pkd = m->pkd;
    const ref_grav_params *gp = m->gp;
    int nActive = 0, i;
    double dPartSum, dCellSum, dSoftSum, dFlop;
    double aSun[3] = {0, 0, 0};
    CASTAT cs;
    if (pkdActiveMaskRung(pkd, TYPE_ACTIVE, iKickRung, 1) == 0) return;
    pkdInitAccel(pkd);
    pkdActiveRung(pkd, iKickRung, 1);
    pkdActiveType(pkd, TYPE_ALL, TYPE_TREEACTIVE);
    free(pkd->kdTop); free(pkd->piLeaf);
    build_grav_tree(pkd, gp);
    pkdGravAll(pkd, gp->bPeriodic ? gp->nReps : 0, gp->bPeriodic, gp->iOrder, gp->bEwald,
               gp->iEwOrder, gp->fEwCut, gp->fEwhCut, 0, 0.0, 0, 0.0, aSun, &nActive,
               &dPartSum, &dCellSum, &dSoftSum, &cs, &dFlop);
    m->counts[0] += 1;
    m->counts[1] += nActive;
    int bGasActive = 0;
    for (i = 0; i < pkd->nLocal; ++i) {
        PARTICLE *p = &pkd->pStore[i];
        if (TYPETest(p, TYPE_GAS) && p->iRung >= iKickRung) bGasActive = 1;
    }
    if (bGasActive) msh_sph(m, iKickRung);
}

/* the Adjust block of msrTopStepKDK (master.c:8264-8317) */
static void msh_adjust(MSH *m, int iRung, double dDelta)
{
    PKD pkd = m->pkd;
    const ref_step_params *st = m->st;
    double dtMinGas;
    int nMaxRung, iMaxRungIdeal;
    pkdActiveRung(pkd, iRung, 1);
    pkdInitDt(pkd, st->dDelta);
    if (st->bGravStep) pkdGravStep(pkd, st->dEta);
    if (st->bEpsAccStep || st->bSqrtPhiStep)
        pkdAccelStep(pkd, st->dEta, 1.0, 1.0, 1, st->bEpsAccStep, st->bSqrtPhiStep, 0.0);
    pkdSphStep(pkd, 1.0, m->sp->dEtaCourant, st->dEtauDot, st->duMinDt, 0.0, 0.1, 0.0, 0,
               &dtMinGas);
    m->iCurrMaxRung = pkdDtToRung(pkd, iRung, dDelta, st->iMaxRung, 1, 1, &nMaxRung,
                                  &iMaxRungIdeal);
}

static void msh_top_step(MSH *m, double dTime, double dDelta, int iRung, int iKickRung,
                         int iAdjust)
{
    PKD pkd = m->pkd;
    if (iAdjust) {
        int nUn, iIdeal, nMax, iOut;
        pkdActiveRung(pkd, iRung, 1);
        pkdEmergencyAdjust(pkd, iRung, m->st->iMaxRung, dDelta, dDelta * 0.5, &nUn, &iIdeal,
                           &nMax, &iOut);
        if (nUn && iOut > m->iCurrMaxRung) m->iCurrMaxRung = iOut;
    }
    if (iAdjust && iRung < m->st->iMaxRung - 1) msh_adjust(m, iRung, dDelta);
    msh_kick(m, iRung, 0.5 * dDelta, 0);
    if (m->iCurrMaxRung > iRung) {
        msh_top_step(m, dTime, 0.5 * dDelta, iRung + 1, iRung + 1, 0);
        dTime += 0.5 * dDelta;
        msh_top_step(m, dTime, 0.5 * dDelta, iRung + 1, iKickRung, 1);
    } else {
        msh_drift(m, 0.5 * dDelta);
        dTime += 0.5 * dDelta;
        msh_drift(m, 0.5 * dDelta);
        dTime += 0.5 * dDelta;
        msh_forces(m, iKickRung);
        dTime -= 0.5 * dDelta;
    }
    msh_kick(m, iRung, 0.5 * dDelta, 1);
}

int ref_multistep(int n, int ngas, const double *pos, const double *vel, const double *mass,
                  const double *soft, const double *u, const ref_grav_params *gp,
                  const ref_sph_params *sp, const ref_step_params *st, double *opos,
                  double *ovel, double *ovpred, double *oacc, double *f, int *maxRung,
                  double *counts)
{
    MSH m;
    PKD pkd = make_pkd(n, pos, mass, soft, gp->bPeriodic, gp->dPeriod, gp->iOrder, 0);
    int i, j, s;
    double dTime = 0.0;
    pkd->nGas = ngas;
    pkd->nDark = n - ngas;
    for (i = 0; i < n; ++i) {
        PARTICLE *p = &pkd->pStore[i];
        p->iActive = TYPE_ACTIVE | TYPE_TREEACTIVE | (i < ngas ? TYPE_GAS : TYPE_DARK);
        for (j = 0; j < 3; ++j) p->v[j] = p->vPred[j] = vel[3 * i + j];
        if (i < ngas) p->u = p->uPred = u[i];
        p->iRung = 0;
        p->dt = FLT_MAX;
        p->dtNew = FLT_MAX;
    }
    memset(&m, 0, sizeof(m));
    m.pkd = pkd; m.gp = gp; m.sp = sp; m.st = st; m.ngas = ngas;
    /* initial forces (main.c:360-386, msrInitSph master.c:9060-9100) */
    build_grav_tree(pkd, gp);
    pkdActiveType(pkd, TYPE_ALL, TYPE_ACTIVE);
    msh_forces(&m, 0);
    for (s = 0; s < st->nSteps; ++s) {
        msh_top_step(&m, dTime, st->dDelta, 0, 0, 1);
        dTime += st->dDelta;
        maxRung[s] = m.iCurrMaxRung;
    }
    for (i = 0; i < n; ++i) {
        PARTICLE *p = &pkd->pStore[i];
        int k = p->iOrder;
        double *q = &f[12 * k];
        for (j = 0; j < 3; ++j) {
            opos[3 * k + j] = p->r[j];
            ovel[3 * k + j] = p->v[j];
            ovpred[3 * k + j] = p->vPred[j];
            oacc[3 * k + j] = p->a[j];
        }
        q[0] = p->u; q[1] = p->uPred; q[2] = p->fPot; q[3] = p->dtGrav; q[4] = p->dt;
        q[5] = p->dtNew; q[6] = p->mumax; q[7] = p->fDensity; q[8] = p->fBall2;
        q[9] = p->uDotPdV; q[10] = p->uDotAV; q[11] = p->iRung;
    }
    counts[0] = m.counts[0];
    counts[1] = m.counts[1];
    pkdFinish(pkd);
    return 0;
}

/*
 * Force passes over an active subset, as one step of msrTopStepKDK runs
 * them: particles with rung >= iRung are active (msrActiveRung(iRung, 1)).
 * Gravity: pkdInitAccel, tree of all particles, pkdGravAll.  SPH (all
 * particles gas): the non-FastGas msrSph above.  Outputs by iOrder;
 * inactive particles keep a = 0, fPot = 0 (gravity) or their initial
 * dt = dtNew = FLT_MAX, mumax = 0 (SPH).
 *   grav: acc[3n], pot[n], dtGrav[n], counters[5] as ref_grav
 *   sph:  acc[3n] (hydro), f[6*i + ..] = uDotPdV, uDotAV, dtNew, mumax,
 *         dt, fDensity
 */
int ref_grav_active(int n, const double *pos, const double *mass, const double *soft,
                    const int *rung, int iRung, const ref_grav_params *gp, double *acc,
                    double *pot, double *dtGrav, double *counters)
{
    PKD pkd = make_pkd(n, pos, mass, soft, gp->bPeriodic, gp->dPeriod, gp->iOrder, 0);
    int nActive = 0, i, j;
    double dPartSum, dCellSum, dSoftSum, dFlop;
    CASTAT cs;
    double aSun[3] = {0, 0, 0};
    for (i = 0; i < n; ++i) pkd->pStore[i].iRung = rung[i];
    pkdActiveRung(pkd, iRung, 1);
    pkdInitAccel(pkd);
    build_grav_tree(pkd, gp);
    pkdGravAll(pkd, gp->bPeriodic ? gp->nReps : 0, gp->bPeriodic, gp->iOrder, gp->bEwald,
               gp->iEwOrder, gp->fEwCut, gp->fEwhCut, 0, 0.0, 0, 0.0, aSun, &nActive,
               &dPartSum, &dCellSum, &dSoftSum, &cs, &dFlop);
    for (i = 0; i < n; ++i) {
        PARTICLE *p = &pkd->pStore[i];
        int k = p->iOrder;
        for (j = 0; j < 3; ++j) acc[3 * k + j] = p->a[j];
        pot[k] = p->fPot;
        dtGrav[k] = p->dtGrav;
    }
    counters[0] = nActive; counters[1] = dPartSum; counters[2] = dCellSum;
    counters[3] = dSoftSum; counters[4] = dFlop;
    pkdFinish(pkd);
    return 0;
}

int ref_sph_active(int n, const double *pos, const double *vel, const double *mass,
                   const double *soft, const double *u, const int *rung, int iRung,
                   const ref_sph_params *sp, double *acc, double *f)
{
    ref_grav_params gp;
    MSH m;
    PKD pkd = make_pkd(n, pos, mass, soft, sp->bPeriodic, sp->dPeriod, 2, 1);
    int i, j;
    memset(&gp, 0, sizeof(gp));
    gp.bPeriodic = sp->bPeriodic;
    gp.dPeriod = sp->dPeriod;
    for (i = 0; i < n; ++i) {
        PARTICLE *p = &pkd->pStore[i];
        for (j = 0; j < 3; ++j) p->v[j] = p->vPred[j] = vel[3 * i + j];
        p->u = p->uPred = u[i];
        p->iRung = rung[i];
        p->dt = FLT_MAX;
        p->dtNew = FLT_MAX;
        p->mumax = 0.0;
    }
    memset(&m, 0, sizeof(m));
    m.pkd = pkd; m.gp = &gp; m.sp = sp; m.ngas = n;
    pkd->kdTop = NULL; pkd->piLeaf = NULL;
    msh_sph(&m, iRung);
    for (i = 0; i < n; ++i) {
        PARTICLE *p = &pkd->pStore[i];
        int k = p->iOrder;
        double *q = &f[6 * k];
        for (j = 0; j < 3; ++j) acc[3 * k + j] = p->a[j];
        q[0] = p->uDotPdV; q[1] = p->uDotAV; q[2] = p->dtNew; q[3] = p->mumax; q[4] = p->dt;
        q[5] = p->fDensity;
    }
    pkdFinish(pkd);
    return 0;
}

/*
 * A TSC frame through the reference's own dfRenderParticles
 * (dumpframe.c:1394-1470) and dfRenderParticleTSC (dumpframe.c:1125-1230),
 * with the frame set up as dfSetupFrame does (xlim, ylim, hmul,
 * dumpframe.c:259-261).  Particles: the first ngas gas, the last nstar
 * stars, the rest dark; rgb receives nxPix*nyPix*3 floats.
 */
#include "dumpframe.h"
#include "tsph.h"

typedef struct {
    double r[3];
    double fMass, fSoft, fBall2;
    unsigned int iActive;
    double fDensity, fTimeForm;
} RPART;

int ref_render_tsc(int n, int ngas, int nstar, const double *pos, const double *mass,
                   const double *soft, const double *fBall2, const double *fDensity,
                   const tsph_render_params *rp, float *rgb)
{
    struct inDumpFrame in;
    RPART *p = (RPART *)calloc(n > 0 ? n : 1, sizeof(RPART));
    DFIMAGE *img = (DFIMAGE *)calloc((size_t)rp->nxPix * rp->nyPix, sizeof(DFIMAGE));
    int i, j;
    memset(&in, 0, sizeof(in));
    in.nxPix = rp->nxPix; in.nyPix = rp->nyPix;
    for (j = 0; j < 3; ++j) {
        in.r[j] = rp->r[j]; in.x[j] = rp->x[j]; in.y[j] = rp->y[j]; in.z[j] = rp->z[j];
    }
    in.zEye = rp->zEye; in.zClipNear = rp->zClipNear; in.zClipFar = rp->zClipFar;
    in.iProject = rp->iProject == 2 ? DF_PROJECT_PERSPECTIVE : DF_PROJECT_ORTHO;
    in.dGasSoftMul = rp->dGasSoftMul; in.dDarkSoftMul = rp->dDarkSoftMul;
    in.dStarSoftMul = rp->dStarSoftMul;
    in.bGasSph = rp->bGasSph;
    in.dMassGasMin = rp->dMassGasMin; in.dMassGasMax = rp->dMassGasMax;
    in.dMassDarkMin = rp->dMassDarkMin; in.dMassDarkMax = rp->dMassDarkMax;
    in.dMassStarMin = rp->dMassStarMin; in.dMassStarMax = rp->dMassStarMax;
    in.bColMassWeight = rp->bColMassWeight; in.bColLogInterp = rp->bColLogInterp;
    in.nColGas = rp->nColGas; in.nColDark = rp->nColDark; in.nColStar = rp->nColStar;
    for (i = 0; i < 10; ++i) {
        in.dColGas[i] = rp->dColGas[i]; in.dColDark[i] = rp->dColDark[i];
        in.dColStar[i] = rp->dColStar[i];
        in.ColGas[i].r = rp->colGas[i][0]; in.ColGas[i].g = rp->colGas[i][1]; in.ColGas[i].b = rp->colGas[i][2];
        in.ColDark[i].r = rp->colDark[i][0]; in.ColDark[i].g = rp->colDark[i][1]; in.ColDark[i].b = rp->colDark[i][2];
        in.ColStar[i].r = rp->colStar[i][0]; in.ColStar[i].g = rp->colStar[i][1]; in.ColStar[i].b = rp->colStar[i][2];
    }
    in.iColStarAge = DF_STAR_AGE_BASIC;
    in.iRender = DF_RENDER_TSC;
    in.dTime = 0.0;
    in.dYearUnit = 1.0;
    in.xlim = (in.nxPix - 1) * .5;
    in.ylim = (in.nyPix - 1) * .5;
    in.hmul = 4 * sqrt(in.x[0] * in.x[0] + in.x[1] * in.x[1] + in.x[2] * in.x[2]);
    for (i = 0; i < n; ++i) {
        for (j = 0; j < 3; ++j) p[i].r[j] = pos[3 * i + j];
        p[i].fMass = mass[i];
        p[i].fSoft = soft[i];
        p[i].fBall2 = fBall2[i];
        p[i].fDensity = fDensity[i];
        p[i].iActive = i < ngas ? TYPE_GAS : (i < n - nstar ? TYPE_DARK : TYPE_STAR);
    }
    dfRenderParticlesInit(&in, TYPE_GAS, TYPE_DARK, TYPE_STAR, &p[0].r[0], &p[0].fMass,
                          &p[0].fSoft, &p[0].fBall2, &p[0].iActive, &p[0].fDensity,
                          &p[0].fTimeForm, p, sizeof(RPART));
    dfRenderParticles(&in, img, p, n);
    for (i = 0; i < rp->nxPix * rp->nyPix; ++i) {
        rgb[3 * i] = img[i].r; rgb[3 * i + 1] = img[i].g; rgb[3 * i + 2] = img[i].b;
    }
    free(p);
    free(img);
    return 0;
}
