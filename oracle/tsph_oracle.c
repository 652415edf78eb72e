/*
 * CPU oracle for the TreeSPH force path -- a plain-C restatement of the
 * reference's algorithm, written for this project.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path and the timed CPU
 * baseline.  The product library (libtsph) never links or calls it.
 *
 * Gravity follows the reference operation by operation so that, on the same
 * machine and compiled with -ffp-contract=off, its trees, interaction lists
 * and accelerations are bit-identical to the reference's own pkdGravAll:
 *   tree build      pkd.c:1109-1157 (pkdUpperPart), :2373-2587
 *                   (NumBinaryNodes/BuildBinary), :2590-2620 (pkdThreadTree)
 *   moments         pkd.c:2018-2135 (pkdCalcCell), :2228-2264 (pkdCalcOpen)
 *   root/Ewald      pkd.c:4395-4493 (pkdCalcRoot/pkdDistribRoot),
 *                   ewald.c:182-248 (pkdEwaldInit), ewald.c:15-178
 *   walk            walk.c:10-178 (SETILIST, pkdLocalWalk), :306-439,
 *                   walk.h:12-31 (INTERSECTNP)
 *   interactions    grav.c:23-249, grav.h:17-101, qeval.h:21-64,
 *                   meval.h:21-81, v_sqrt1.c:11-113
 *   driver          pkd.c:2869-3060 (pkdGravAll)
 * SPH follows smooth.c / smoothfcn.c / SphPressureTerms.h / pkd.c:5690-5785
 * with an exact kNN and a two-sided gather in place of the reference's
 * priority queue and scatter-add cache; results agree to rounding (the
 * summation order differs) and the neighbour sets are identical.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "tsph_oracle.h"

#define ORC_FLOAT_MAX DBL_MAX

/* ------------------------------------------------------------------ */
/* particles in storage order                                          */
/* ------------------------------------------------------------------ */
typedef struct {
    int n;
    double *r;      /* 3n */
    double *m;
    double *h;
    int *iord;
} orc_parts;

static void parts_init(orc_parts *P, int n, const double *pos,
                       const double *mass, const double *soft) {
    int i;
    P->n = n;
    P->r = malloc(sizeof(double) * 3 * (size_t)(n > 0 ? n : 1));
    P->m = malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    P->h = malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    P->iord = malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    memcpy(P->r, pos, sizeof(double) * 3 * (size_t)n);
    memcpy(P->m, mass, sizeof(double) * (size_t)n);
    if (soft) memcpy(P->h, soft, sizeof(double) * (size_t)n);
    else memset(P->h, 0, sizeof(double) * (size_t)n);
    for (i = 0; i < n; ++i) P->iord[i] = i;
}

static void parts_free(orc_parts *P) {
    free(P->r); free(P->m); free(P->h); free(P->iord);
}

static void parts_swap(orc_parts *P, int i, int j) {
    double t;
    int k, ti;
    for (k = 0; k < 3; ++k) {
        t = P->r[3 * i + k]; P->r[3 * i + k] = P->r[3 * j + k]; P->r[3 * j + k] = t;
    }
    t = P->m[i]; P->m[i] = P->m[j]; P->m[j] = t;
    t = P->h[i]; P->h[i] = P->h[j]; P->h[j] = t;
    ti = P->iord[i]; P->iord[i] = P->iord[j]; P->iord[j] = ti;
}

/* ------------------------------------------------------------------ */
/* tree                                                                */
/* ------------------------------------------------------------------ */
typedef struct {
    int pLower, pUpper, iDim, iLower, iUpper;
    double fSplit;
    double bmin[3], bmax[3];
    double fMass, fSoft, r[3];
    double fOpen2;
    /* moments about the centre of mass, pkdCalcCellStruct order */
    double Qxx, Qyy, Qzz, Qxy, Qxz, Qyz;
    double Oxxx, Oxyy, Oxxy, Oyyy, Oxxz, Oyyz, Oxyz, Oxzz, Oyzz, Ozzz;
    double Hxxxx, Hxyyy, Hxxxy, Hyyyy, Hxxxz, Hyyyz, Hxxyy, Hxxyz, Hxyyz;
    double Hxxzz, Hxyzz, Hxzzz, Hyyzz, Hyzzz, Hzzzz;
    double Bmax, B2, B3, B4, B5, B6;
} orc_node;

typedef struct {
    orc_node *c;
    int nNodes;
    int nMax;
} orc_tree_t;

/* Partition [i,j] so that r[d] < fSplit come first; same pairing of
 * misplaced elements as pkdUpperPart (pkd.c:1109-1157). Returns the first
 * index of the upper part. */
static int upper_part(orc_parts *P, int d, double fSplit, int i, int j) {
    const double *r = P->r;
    if (i > j) return i;
    i--;
    j++;
    while (++i < j && r[3 * i + d] < fSplit);
    while (i < --j && r[3 * j + d] >= fSplit);
    if (i >= j) return i;
    parts_swap(P, i, j);
    for (;;) {
        while (P->r[3 * (++i) + d] < fSplit);
        while (P->r[3 * (--j) + d] >= fSplit);
        if (i > j) return i;
        parts_swap(P, i, j);
    }
}

/* Moments about rcm: pkdCalcCell (pkd.c:2018-2135), same operation order. */
static void calc_cell(const orc_parts *P, orc_node *c, const double *rcm, int iOrder) {
    int pj;
    double m, dx, dy, dz, d2, d1;
    c->Hxxxx = c->Hxyyy = c->Hxxxy = c->Hyyyy = c->Hxxxz = c->Hyyyz = 0.0;
    c->Hxxyy = c->Hxxyz = c->Hxyyz = c->Hxxzz = c->Hxyzz = c->Hxzzz = 0.0;
    c->Hyyzz = c->Hyzzz = c->Hzzzz = 0.0;
    c->Oxxx = c->Oxyy = c->Oxxy = c->Oyyy = c->Oxxz = c->Oyyz = c->Oxyz = 0.0;
    c->Oxzz = c->Oyzz = c->Ozzz = 0.0;
    c->Qxx = c->Qyy = c->Qzz = c->Qxy = c->Qxz = c->Qyz = 0.0;
    c->B2 = c->B3 = c->B4 = c->B5 = c->B6 = 0.0;
    c->Bmax = 0.0;
    for (pj = c->pLower; pj <= c->pUpper; ++pj) {
        m = P->m[pj];
        dx = P->r[3 * pj + 0] - rcm[0];
        dy = P->r[3 * pj + 1] - rcm[1];
        dz = P->r[3 * pj + 2] - rcm[2];
        d2 = dx * dx + dy * dy + dz * dz;
        d1 = sqrt(d2);
        if (d1 > c->Bmax) c->Bmax = d1;
        c->B2 += m * d2;
        c->B3 += m * d2 * d1;
        c->B4 += m * d2 * d2;
        c->B5 += m * d2 * d2 * d1;
        c->B6 += m * d2 * d2 * d2;
        if (iOrder >= 4) {
            c->Hxxxx += m * (dx * dx * dx * dx - 6.0 / 7.0 * d2 * (dx * dx - 0.1 * d2));
            c->Hxyyy += m * (dx * dy * dy * dy - 3.0 / 7.0 * d2 * dx * dy);
            c->Hxxxy += m * (dx * dx * dx * dy - 3.0 / 7.0 * d2 * dx * dy);
            c->Hyyyy += m * (dy * dy * dy * dy - 6.0 / 7.0 * d2 * (dy * dy - 0.1 * d2));
            c->Hxxxz += m * (dx * dx * dx * dz - 3.0 / 7.0 * d2 * dx * dz);
            c->Hyyyz += m * (dy * dy * dy * dz - 3.0 / 7.0 * d2 * dy * dz);
            c->Hxxyy += m * (dx * dx * dy * dy - 1.0 / 7.0 * d2 * (dx * dx + dy * dy - 0.2 * d2));
            c->Hxxyz += m * (dx * dx * dy * dz - 1.0 / 7.0 * d2 * dy * dz);
            c->Hxyyz += m * (dx * dy * dy * dz - 1.0 / 7.0 * d2 * dx * dz);
            c->Hxxzz += m * (dx * dx * dz * dz - 1.0 / 7.0 * d2 * (dx * dx + dz * dz - 0.2 * d2));
            c->Hxyzz += m * (dx * dy * dz * dz - 1.0 / 7.0 * d2 * dx * dy);
            c->Hxzzz += m * (dx * dz * dz * dz - 3.0 / 7.0 * d2 * dx * dz);
            c->Hyyzz += m * (dy * dy * dz * dz - 1.0 / 7.0 * d2 * (dy * dy + dz * dz - 0.2 * d2));
            c->Hyzzz += m * (dy * dz * dz * dz - 3.0 / 7.0 * d2 * dy * dz);
            c->Hzzzz += m * (dz * dz * dz * dz - 6.0 / 7.0 * d2 * (dz * dz - 0.1 * d2));
        }
        if (iOrder >= 3) {
            c->Oxxx += m * (dx * dx * dx - 0.6 * d2 * dx);
            c->Oxyy += m * (dx * dy * dy - 0.2 * d2 * dx);
            c->Oxxy += m * (dx * dx * dy - 0.2 * d2 * dy);
            c->Oyyy += m * (dy * dy * dy - 0.6 * d2 * dy);
            c->Oxxz += m * (dx * dx * dz - 0.2 * d2 * dz);
            c->Oyyz += m * (dy * dy * dz - 0.2 * d2 * dz);
            c->Oxyz += m * dx * dy * dz;
            c->Oxzz += m * (dx * dz * dz - 0.2 * d2 * dx);
            c->Oyzz += m * (dy * dz * dz - 0.2 * d2 * dy);
            c->Ozzz += m * (dz * dz * dz - 0.6 * d2 * dz);
        }
        c->Qxx += m * dx * dx;
        c->Qyy += m * dy * dy;
        c->Qzz += m * dz * dz;
        c->Qxy += m * dx * dy;
        c->Qxz += m * dx * dz;
        c->Qyz += m * dy * dz;
    }
}

/* OPEN_JOSH opening radius (pkd.c:2245-2253). */
static double calc_open(const orc_node *c, double dCrit) {
    double dOpen = 2 / sqrt(3.0) * c->Bmax / dCrit;
    if (dOpen < c->Bmax) dOpen = c->Bmax;
    return dOpen;
}

static int build_rec(orc_parts *P, orc_tree_t *T, int nBucket, int pLower,
                     int pUpper, double dCrit, int iOrder) {
    orc_node *c;
    int i, j, m, d, ic;
    int bGood;
    double bmin[3], bmax[3];
    if (pLower > pUpper) return -1;
    if (T->nNodes == T->nMax) {
        T->nMax = T->nMax * 2 + 16;
        T->c = realloc(T->c, sizeof(orc_node) * (size_t)T->nMax);
    }
    ic = T->nNodes++;
    for (j = 0; j < 3; ++j) {
        bmin[j] = P->r[3 * pLower + j];
        bmax[j] = P->r[3 * pLower + j];
    }
    for (i = pLower + 1; i <= pUpper; ++i) {
        for (j = 0; j < 3; ++j) {
            double x = P->r[3 * i + j];
            if (x < bmin[j]) bmin[j] = x;
            else if (x > bmax[j]) bmax[j] = x;
        }
    }
    bGood = 0;
    for (j = 0; j < 3; ++j) if (bmax[j] > bmin[j]) bGood = 1;
    c = &T->c[ic];
    memset(c, 0, sizeof(*c));
    c->pLower = pLower;
    c->pUpper = pUpper;
    for (j = 0; j < 3; ++j) { c->bmin[j] = bmin[j]; c->bmax[j] = bmax[j]; }
    if ((pUpper - pLower + 1 > nBucket) && bGood) {
        int il, iu;
        double fm, fMass = 0.0, fSoft = 0.0, r[3] = {0.0, 0.0, 0.0};
        d = 0;
        for (j = 1; j < 3; ++j)
            if (bmax[j] - bmin[j] > bmax[d] - bmin[d]) d = j;
        c->iDim = d;
        c->fSplit = 0.5 * (bmin[d] + bmax[d]);
        m = upper_part(P, d, c->fSplit, pLower, pUpper);
        il = build_rec(P, T, nBucket, pLower, m - 1, dCrit, iOrder);
        iu = build_rec(P, T, nBucket, m, pUpper, dCrit, iOrder);
        c = &T->c[ic];
        c->iLower = il;
        c->iUpper = iu;
        /* children combination, BuildBinary pkd.c:2522-2547 */
        fm = T->c[il].fMass;
        fMass += fm;
        fSoft += fm * T->c[il].fSoft;
        for (j = 0; j < 3; ++j) r[j] += fm * T->c[il].r[j];
        fm = T->c[iu].fMass;
        fMass += fm;
        fSoft += fm * T->c[iu].fSoft;
        for (j = 0; j < 3; ++j) r[j] += fm * T->c[iu].r[j];
        if (fMass > 0) {
            fSoft /= fMass;
            for (j = 0; j < 3; ++j) r[j] /= fMass;
        }
        c->fMass = fMass;
        c->fSoft = fSoft;
        for (j = 0; j < 3; ++j) c->r[j] = r[j];
    } else {
        double fm, fMass = 0.0, fSoft = 0.0, r[3] = {0.0, 0.0, 0.0};
        c->iDim = -1;
        c->fSplit = 0.0;
        c->iLower = -1;
        c->iUpper = -1;
        for (i = pLower; i <= pUpper; ++i) {
            fm = P->m[i];
            fMass += fm;
            fSoft += fm * P->h[i];
            for (j = 0; j < 3; ++j) r[j] += fm * P->r[3 * i + j];
        }
        if (fMass > 0) {
            fSoft /= fMass;
            for (j = 0; j < 3; ++j) r[j] /= fMass;
        }
        c->fMass = fMass;
        c->fSoft = fSoft;
        for (j = 0; j < 3; ++j) c->r[j] = r[j];
    }
    calc_cell(P, c, c->r, iOrder);
    {
        double dOpen = calc_open(c, dCrit);
        c->fOpen2 = dOpen * dOpen;
    }
    return ic;
}

/* pkdThreadTree (pkd.c:2590-2620): iLower = first child, iUpper = next. */
static void thread_tree(orc_tree_t *T, int ic, int iNext) {
    orc_node *c;
    if (ic == -1) return;
    c = &T->c[ic];
    if (c->iDim != -1) {
        int l = c->iLower, u = c->iUpper;
        thread_tree(T, l, u);
        thread_tree(T, u, iNext);
        T->c[ic].iUpper = iNext;
    } else {
        c->iLower = -1;
        c->iUpper = iNext;
    }
}

static void build_tree(orc_parts *P, orc_tree_t *T, int nBucket, double dCrit, int iOrder) {
    T->c = NULL;
    T->nNodes = 0;
    T->nMax = 0;
    if (P->n == 0) {
        T->nMax = 1;
        T->c = calloc(1, sizeof(orc_node));
        T->nNodes = 1;
        T->c[0].pLower = 0;
        T->c[0].pUpper = -1;
        T->c[0].iDim = -1;
        T->c[0].iLower = -1;
        T->c[0].iUpper = -1;
        return;
    }
    build_rec(P, T, nBucket, 0, P->n - 1, dCrit, iOrder);
    thread_tree(T, 0, -1);
}

/* ------------------------------------------------------------------ */
/* v_sqrt1 restated: Chebyshev fit of 1/sqrt on [1,2) + one Newton step */
/* ------------------------------------------------------------------ */
static double g_vs_u[2048], g_vs_t[2048];
static double g_vs_g[6];
static int g_vs_init = 0;

static void vs_init(void) {
    double xi, c[6], f[201], z[201];
    double d0, d1, d2, d3, d4, d5;
    int i, j, k;
    const int NCH = 200;
    if (g_vs_init) return;
    xi = 1.0;
    g_vs_t[1023] = 1.0;
    g_vs_u[1023] = 1.0;
    for (i = 1; i < 1024; ++i) {
        xi *= 0.5;
        g_vs_t[1023 + i] = sqrt(xi);
        if (xi != 0.0) g_vs_t[1023 - i] = 1.0 / g_vs_t[1023 + i];
        g_vs_u[1023 + i] = xi;
        if (xi != 0.0) g_vs_u[1023 - i] = 1.0 / xi;
    }
    for (k = 1; k <= NCH; ++k) {
        double zero;
        z[k] = (M_PI * (k - 0.5)) / NCH;
        zero = cos(z[k]);
        f[k] = pow(1.5 + 0.5 * zero, -0.5);
    }
    for (j = 0; j < 6; ++j) {
        double sum = 0.0;
        for (k = 1; k <= NCH; ++k) sum += f[k] * cos(z[k] * j);
        c[j] = (2.0 / NCH) * sum;
    }
    d0 = 0.5 * c[0] - c[2] + c[4];
    d1 = c[1] - 3 * c[3] + 5 * c[5];
    d2 = 2 * c[2] - 8 * c[4];
    d3 = 4 * c[3] - 20 * c[5];
    d4 = 8 * c[4];
    d5 = 16 * c[5];
    g_vs_g[0] = d0 - 3 * d1 + 9 * d2 - 27 * d3 + 81 * d4 - 243 * d5;
    g_vs_g[1] = 2 * d1 - 12 * d2 + 54 * d3 - 216 * d4 + 810 * d5;
    g_vs_g[2] = 4 * d2 - 36 * d3 + 216 * d4 - 1080 * d5;
    g_vs_g[3] = 8 * d3 - 96 * d4 + 720 * d5;
    g_vs_g[4] = 16 * d4 - 240 * d5;
    g_vs_g[5] = 32 * d5;
    g_vs_init = 1;
}

/* When set, 1/sqrt is taken as 1.0/sqrt(r2) instead of the reference's
 * v_sqrt1 approximation (used to separate the reference's own 2e-10 1/sqrt
 * error from other differences). */
static int g_exact_rsqrt = 0;
void orc_set_exact_rsqrt(int on) { g_exact_rsqrt = on; }

static inline double vs_one(double r2) {
    if (g_exact_rsqrt) return 1.0 / sqrt(r2);
    uint64_t bits;
    int it;
    double x, s;
    memcpy(&bits, &r2, sizeof(bits));
    it = (int)((int32_t)(uint32_t)(bits >> 32) >> 20);
    x = r2 * g_vs_u[it];
    s = g_vs_g[0] + x * (g_vs_g[1] + x * (g_vs_g[2] + x * (g_vs_g[3] + x * (g_vs_g[4] + x * g_vs_g[5]))));
    s *= 1.5 - 0.5 * x * s * s;
    return s * g_vs_t[it];
}

void orc_v_sqrt1(int n, const double *r2, double *a) {
    int i;
    vs_init();
    for (i = 0; i < n; ++i) a[i] = vs_one(r2[i]);
}

/* ------------------------------------------------------------------ */
/* interaction lists                                                   */
/* ------------------------------------------------------------------ */
typedef struct { double m, h, x, y, z; } orc_ilp;
typedef struct { double m, h, x, y, z, xx, yy, zz, xy, xz, yz; } orc_ilcs;
typedef struct {
    double m, x, y, z;
    double xx, yy, xy, xz, yz, zz;
    double xxx, xyy, xxy, yyy, xxz, yyz, xyz, xzz, yzz, zzz;
    double xxxx, xyyy, xxxy, yyyy, xxxz, yyyz, xxyy, xxyz, xyyz;
    double xxzz, xyzz, xzzz, yyzz, yzzz, zzzz;
} orc_ilcn;

typedef struct {
    orc_ilp *ilp; int nPart, nMaxPart;
    orc_ilcs *ilcs; int nCellSoft, nMaxCellSoft;
    orc_ilcn *ilcn; int nCellNewt, nMaxCellNewt;
    double *d2a, *sq; int nSq;
} orc_lists_t;

static void lists_init(orc_lists_t *L) {
    memset(L, 0, sizeof(*L));
}
static void lists_free(orc_lists_t *L) {
    free(L->ilp); free(L->ilcs); free(L->ilcn); free(L->d2a); free(L->sq);
}
static void lists_sq(orc_lists_t *L, int n) {
    if (n > L->nSq) {
        L->nSq = n * 2;
        L->d2a = realloc(L->d2a, sizeof(double) * (size_t)L->nSq);
        L->sq = realloc(L->sq, sizeof(double) * (size_t)L->nSq);
    }
}

/* INTERSECTNP (walk.h:12-31) */
static inline int intersect_np(const double *bmin, const double *bmax,
                               double fBall2, double x, double y, double z) {
    double dx, dy, dz, dx1, dy1, dz1, fDist2;
    dx = bmin[0] - x;
    dx1 = x - bmax[0];
    dy = bmin[1] - y;
    dy1 = y - bmax[1];
    dz = bmin[2] - z;
    dz1 = z - bmax[2];
    if (dx > 0.0) fDist2 = dx * dx;
    else if (dx1 > 0.0) fDist2 = dx1 * dx1;
    else fDist2 = 0.0;
    if (dy > 0.0) fDist2 += dy * dy;
    else if (dy1 > 0.0) fDist2 += dy1 * dy1;
    if (dz > 0.0) fDist2 += dz * dz;
    else if (dz1 > 0.0) fDist2 += dz1 * dz1;
    return fDist2 <= fBall2;
}

/* SETILIST (walk.c:10-56) */
static void set_ilist(int iOrder, orc_ilcn *l, const orc_node *c, double x, double y, double z) {
    if (iOrder >= 4) {
        l->xxxx = c->Hxxxx; l->xyyy = c->Hxyyy; l->xxxy = c->Hxxxy; l->yyyy = c->Hyyyy;
        l->xxxz = c->Hxxxz; l->yyyz = c->Hyyyz; l->xxyy = c->Hxxyy; l->xxyz = c->Hxxyz;
        l->xyyz = c->Hxyyz; l->xxzz = c->Hxxzz; l->xyzz = c->Hxyzz; l->xzzz = c->Hxzzz;
        l->yyzz = c->Hyyzz; l->yzzz = c->Hyzzz; l->zzzz = c->Hzzzz;
    }
    if (iOrder >= 3) {
        l->xxx = c->Oxxx; l->xyy = c->Oxyy; l->xxy = c->Oxxy; l->yyy = c->Oyyy;
        l->xxz = c->Oxxz; l->yyz = c->Oyyz; l->xyz = c->Oxyz; l->xzz = c->Oxzz;
        l->yzz = c->Oyzz; l->zzz = c->Ozzz;
    }
    if (iOrder >= 2) {
        double tr = c->Qxx + c->Qyy + c->Qzz;
        l->xx = c->Qxx - tr / 3.0;
        l->yy = c->Qyy - tr / 3.0;
        l->zz = c->Qzz - tr / 3.0;
        l->xy = c->Qxy;
        l->xz = c->Qxz;
        l->yz = c->Qyz;
    }
    l->m = c->fMass;
    l->x = x;
    l->y = y;
    l->z = z;
}

/* pkdLocalWalk (walk.c:58-178) for one replica offset. */
static void local_walk(const orc_parts *P, const orc_tree_t *T, int iBucket,
                       const double *bbmin, const double *bbmax, double fSoftMax,
                       int bRep, const double *rOffset, int iOrder, orc_lists_t *L) {
    int iCell = 0;
    while (iCell != -1) {
        const orc_node *c = &T->c[iCell];
        double x = c->r[0] + rOffset[0];
        double y = c->r[1] + rOffset[1];
        double z = c->r[2] + rOffset[2];
        int bInt = intersect_np(bbmin, bbmax, c->fOpen2, x, y, z);
        if (c->pUpper - c->pLower < 3) bInt = 1;
        if (bInt) {
            if (c->iLower != -1) {
                iCell = c->iLower;
            } else {
                if (iCell != iBucket || bRep) {
                    int pj, n = c->pUpper - c->pLower + 1;
                    if (L->nPart + n > L->nMaxPart) {
                        L->nMaxPart += L->nMaxPart + n;
                        L->ilp = realloc(L->ilp, sizeof(orc_ilp) * (size_t)L->nMaxPart);
                    }
                    for (pj = c->pLower; pj <= c->pUpper; ++pj, ++L->nPart) {
                        orc_ilp *q = &L->ilp[L->nPart];
                        q->x = P->r[3 * pj + 0] + rOffset[0];
                        q->y = P->r[3 * pj + 1] + rOffset[1];
                        q->z = P->r[3 * pj + 2] + rOffset[2];
                        q->m = P->m[pj];
                        q->h = P->h[pj];
                    }
                }
                iCell = c->iUpper;
            }
        } else {
            double twoh2 = c->fSoft + fSoftMax;
            twoh2 *= twoh2;
            if (twoh2 < c->fOpen2) bInt = 0;
            else bInt = intersect_np(bbmin, bbmax, twoh2, x, y, z);
            if (bInt) {
                orc_ilcs *q;
                if (L->nCellSoft == L->nMaxCellSoft) {
                    L->nMaxCellSoft = L->nMaxCellSoft * 2 + 64;
                    L->ilcs = realloc(L->ilcs, sizeof(orc_ilcs) * (size_t)L->nMaxCellSoft);
                }
                q = &L->ilcs[L->nCellSoft++];
                q->m = c->fMass; q->h = c->fSoft;
                q->x = x; q->y = y; q->z = z;
                q->xx = c->Qxx; q->yy = c->Qyy; q->zz = c->Qzz;
                q->xy = c->Qxy; q->xz = c->Qxz; q->yz = c->Qyz;
            } else {
                if (L->nCellNewt == L->nMaxCellNewt) {
                    L->nMaxCellNewt = L->nMaxCellNewt * 2 + 64;
                    L->ilcn = realloc(L->ilcn, sizeof(orc_ilcn) * (size_t)L->nMaxCellNewt);
                }
                set_ilist(iOrder, &L->ilcn[L->nCellNewt++], c, x, y, z);
            }
            iCell = c->iUpper;
        }
    }
}

/* pkdBucketWalk (walk.c:306-439), single rank: the top tree is the root. */
static void bucket_walk(const orc_parts *P, const orc_tree_t *T, int iBucket,
                        const double *bbmin, const double *bbmax, int nReps,
                        const double *fPeriod, int iOrder, orc_lists_t *L) {
    const orc_node *b = &T->c[iBucket];
    double fSoftMax = 0.0, rOffset[3];
    int pj, ix, iy, iz;
    L->nPart = L->nCellSoft = L->nCellNewt = 0;
    for (pj = b->pLower; pj <= b->pUpper; ++pj)
        if (P->h[pj] > fSoftMax) fSoftMax = P->h[pj];
    for (ix = -nReps; ix <= nReps; ++ix) {
        if (ix && fPeriod[0] >= ORC_FLOAT_MAX) continue;
        rOffset[0] = ix * fPeriod[0];
        for (iy = -nReps; iy <= nReps; ++iy) {
            if (iy && fPeriod[1] >= ORC_FLOAT_MAX) continue;
            rOffset[1] = iy * fPeriod[1];
            for (iz = -nReps; iz <= nReps; ++iz) {
                if (iz && fPeriod[2] >= ORC_FLOAT_MAX) continue;
                rOffset[2] = iz * fPeriod[2];
                local_walk(P, T, iBucket, bbmin, bbmax, fSoftMax,
                           ix || iy || iz, rOffset, iOrder, L);
            }
        }
    }
}

/* ------------------------------------------------------------------ */
/* spline softening (grav.h:17-101) and multipole evaluation           */
/* ------------------------------------------------------------------ */
static inline void splinem(double dir, double r2, double twoh, double *pa, double *pb) {
    double u, dih, a, b;
    if (r2 < twoh * twoh) {
        dih = 2.0 / twoh;
        u = dih / dir;
        if (u < 1.0) {
            a = dih * (7.0 / 5.0 - 2.0 / 3.0 * u * u + 3.0 / 10.0 * u * u * u * u
                       - 1.0 / 10.0 * u * u * u * u * u);
            b = dih * dih * dih * (4.0 / 3.0 - 6.0 / 5.0 * u * u + 1.0 / 2.0 * u * u * u);
        } else {
            a = -1.0 / 15.0 * dir + dih * (8.0 / 5.0 - 4.0 / 3.0 * u * u + u * u * u
                                           - 3.0 / 10.0 * u * u * u * u + 1.0 / 30.0 * u * u * u * u * u);
            b = -1.0 / 15.0 * dir * dir * dir + dih * dih * dih * (8.0 / 3.0 - 3.0 * u + 6.0 / 5.0 * u * u - 1.0 / 6.0 * u * u * u);
        }
    } else {
        a = dir;
        b = a * a * a;
    }
    *pa = a;
    *pb = b;
}

static inline void splineq(double dir, double r2, double twoh, double *pa,
                           double *pb, double *pc, double *pd) {
    double u, dih, a, b, c, d;
    if (r2 < twoh * twoh) {
        dih = 2.0 / twoh;
        u = dih / dir;
        if (u < 1.0) {
            a = dih * (7.0 / 5.0 - 2.0 / 3.0 * u * u + 3.0 / 10.0 * u * u * u * u
                       - 1.0 / 10.0 * u * u * u * u * u);
            b = dih * dih * dih * (4.0 / 3.0 - 6.0 / 5.0 * u * u + 1.0 / 2.0 * u * u * u);
            c = dih * dih * dih * dih * dih * (12.0 / 5.0 - 3.0 / 2.0 * u);
            d = 3.0 / 2.0 * dih * dih * dih * dih * dih * dih * dir;
        } else {
            a = -1.0 / 15.0 * dir + dih * (8.0 / 5.0 - 4.0 / 3.0 * u * u + u * u * u
                                           - 3.0 / 10.0 * u * u * u * u + 1.0 / 30.0 * u * u * u * u * u);
            b = -1.0 / 15.0 * dir * dir * dir + dih * dih * dih * (8.0 / 3.0 - 3.0 * u + 6.0 / 5.0 * u * u - 1.0 / 6.0 * u * u * u);
            c = -1.0 / 5.0 * dir * dir * dir * dir * dir + 3.0 * dih * dih * dih * dih * dir
                + dih * dih * dih * dih * dih * (-12.0 / 5.0 + 1.0 / 2.0 * u);
            d = -dir * dir * dir * dir * dir * dir * dir
                + 3.0 * dih * dih * dih * dih * dir * dir * dir
                - 1.0 / 2.0 * dih * dih * dih * dih * dih * dih * dir;
        }
    } else {
        a = dir;
        b = a * a * a;
        c = 3.0 * b * a * a;
        d = 5.0 * c * a * a;
    }
    *pa = a; *pb = b; *pc = c; *pd = d;
}

static inline void spline(double r2, double twoh, double *pa, double *pb) {
    double r, u, dih, dir, a, b;
    r = sqrt(r2);
    if (r < twoh) {
        dih = 2.0 / twoh;
        u = r * dih;
        if (u < 1.0) {
            a = dih * (7.0 / 5.0 - 2.0 / 3.0 * u * u + 3.0 / 10.0 * u * u * u * u
                       - 1.0 / 10.0 * u * u * u * u * u);
            b = dih * dih * dih * (4.0 / 3.0 - 6.0 / 5.0 * u * u + 1.0 / 2.0 * u * u * u);
        } else {
            dir = 1.0 / r;
            a = -1.0 / 15.0 * dir + dih * (8.0 / 5.0 - 4.0 / 3.0 * u * u + u * u * u
                                           - 3.0 / 10.0 * u * u * u * u + 1.0 / 30.0 * u * u * u * u * u);
            b = -1.0 / 15.0 * dir * dir * dir + dih * dih * dih * (8.0 / 3.0 - 3.0 * u + 6.0 / 5.0 * u * u - 1.0 / 6.0 * u * u * u);
        }
    } else {
        a = 1.0 / r;
        b = a * a * a;
    }
    *pa = a;
    *pb = b;
}

/* Reduced multipole evaluation, QEVAL (qeval.h:21-64). */
static inline void qeval(int iOrder, const orc_ilcn *mom, const double *gam,
                         double dx, double dy, double dz, double *ax,
                         double *ay, double *az, double *fPot) {
    double Qmirx, Qmiry, Qmirz, Qmir, Qta = 0.0;
    if (iOrder >= 4) {
        Qmirx = (1.0 / 6.0) * (mom->xzzz * dz * dz * dz + 3 * mom->xyzz * dy * dz * dz + 3 * mom->xyyz * dy * dy * dz + mom->xyyy * dy * dy * dy + 3 * mom->xxzz * dx * dz * dz + 6 * mom->xxyz * dx * dy * dz + 3 * mom->xxyy * dx * dy * dy + 3 * mom->xxxz * dx * dx * dz + 3 * mom->xxxy * dx * dx * dy + mom->xxxx * dx * dx * dx);
        Qmiry = (1.0 / 6.0) * (mom->yzzz * dz * dz * dz + 3 * mom->xyzz * dx * dz * dz + 3 * mom->xxyz * dx * dx * dz + mom->xxxy * dx * dx * dx + 3 * mom->yyzz * dy * dz * dz + 6 * mom->xyyz * dx * dy * dz + 3 * mom->xxyy * dx * dx * dy + 3 * mom->yyyz * dy * dy * dz + 3 * mom->xyyy * dx * dy * dy + mom->yyyy * dy * dy * dy);
        Qmirz = (1.0 / 6.0) * (mom->yyyz * dy * dy * dy + 3 * mom->xyyz * dx * dy * dy + 3 * mom->xxyz * dx * dx * dy + mom->xxxz * dx * dx * dx + 3 * mom->yyzz * dy * dy * dz + 6 * mom->xyzz * dx * dy * dz + 3 * mom->xxzz * dx * dx * dz + 3 * mom->yzzz * dy * dz * dz + 3 * mom->xzzz * dx * dz * dz + mom->zzzz * dz * dz * dz);
        Qmir = (1.0 / 4.0) * (Qmirx * dx + Qmiry * dy + Qmirz * dz);
        *fPot -= gam[4] * Qmir;
        Qta += gam[5] * Qmir;
        *ax += gam[4] * Qmirx;
        *ay += gam[4] * Qmiry;
        *az += gam[4] * Qmirz;
    }
    if (iOrder >= 3) {
        Qmirx = (1.0 / 2.0) * (mom->xzz * dz * dz + 2 * mom->xyz * dy * dz + mom->xyy * dy * dy + 2 * mom->xxz * dx * dz + 2 * mom->xxy * dx * dy + mom->xxx * dx * dx);
        Qmiry = (1.0 / 2.0) * (mom->yzz * dz * dz + 2 * mom->xyz * dx * dz + mom->xxy * dx * dx + 2 * mom->yyz * dy * dz + 2 * mom->xyy * dx * dy + mom->yyy * dy * dy);
        Qmirz = (1.0 / 2.0) * (mom->yyz * dy * dy + 2 * mom->xyz * dx * dy + mom->xxz * dx * dx + 2 * mom->yzz * dy * dz + 2 * mom->xzz * dx * dz + mom->zzz * dz * dz);
        Qmir = (1.0 / 3.0) * (Qmirx * dx + Qmiry * dy + Qmirz * dz);
        *fPot -= gam[3] * Qmir;
        Qta += gam[4] * Qmir;
        *ax += gam[3] * Qmirx;
        *ay += gam[3] * Qmiry;
        *az += gam[3] * Qmirz;
    }
    if (iOrder >= 2) {
        Qmirx = (1.0 / 1.0) * (mom->xz * dz + mom->xy * dy + mom->xx * dx);
        Qmiry = (1.0 / 1.0) * (mom->yz * dz + mom->xy * dx + mom->yy * dy);
        Qmirz = (1.0 / 1.0) * (mom->yz * dy + mom->xz * dx + mom->zz * dz);
        Qmir = (1.0 / 2.0) * (Qmirx * dx + Qmiry * dy + Qmirz * dz);
        *fPot -= gam[2] * Qmir;
        Qta += gam[3] * Qmir;
        *ax += gam[2] * Qmirx;
        *ay += gam[2] * Qmiry;
        *az += gam[2] * Qmirz;
    }
    *fPot -= gam[0] * mom->m;
    Qta += gam[1] * mom->m;
    *ax -= dx * Qta;
    *ay -= dy * Qta;
    *az -= dz * Qta;
}

/* Complete multipole evaluation, MEVAL (meval.h:21-81). */
static inline void meval(int iOrder, const orc_ilcn *mom, const double *gam,
                         double dx, double dy, double dz, double *ax,
                         double *ay, double *az, double *fPot) {
    double Qmirx, Qmiry, Qmirz, Qmir, Qta = 0.0;
    double Qxx, Qyy, Qzz, Qxy, Qxz, Qyz, Qx, Qy, Qz, Qtr, Qhx, Qhy, Qhz, Qh;
    if (iOrder >= 4) {
        Qmirx = (1.0 / 6.0) * (mom->xzzz * dz * dz * dz + 3 * mom->xyzz * dy * dz * dz + 3 * mom->xyyz * dy * dy * dz + mom->xyyy * dy * dy * dy + 3 * mom->xxzz * dx * dz * dz + 6 * mom->xxyz * dx * dy * dz + 3 * mom->xxyy * dx * dy * dy + 3 * mom->xxxz * dx * dx * dz + 3 * mom->xxxy * dx * dx * dy + mom->xxxx * dx * dx * dx);
        Qmiry = (1.0 / 6.0) * (mom->yzzz * dz * dz * dz + 3 * mom->xyzz * dx * dz * dz + 3 * mom->xxyz * dx * dx * dz + mom->xxxy * dx * dx * dx + 3 * mom->yyzz * dy * dz * dz + 6 * mom->xyyz * dx * dy * dz + 3 * mom->xxyy * dx * dx * dy + 3 * mom->yyyz * dy * dy * dz + 3 * mom->xyyy * dx * dy * dy + mom->yyyy * dy * dy * dy);
        Qmirz = (1.0 / 6.0) * (mom->yyyz * dy * dy * dy + 3 * mom->xyyz * dx * dy * dy + 3 * mom->xxyz * dx * dx * dy + mom->xxxz * dx * dx * dx + 3 * mom->yyzz * dy * dy * dz + 6 * mom->xyzz * dx * dy * dz + 3 * mom->xxzz * dx * dx * dz + 3 * mom->yzzz * dy * dz * dz + 3 * mom->xzzz * dx * dz * dz + mom->zzzz * dz * dz * dz);
        Qmir = (1.0 / 4.0) * (Qmirx * dx + Qmiry * dy + Qmirz * dz);
        Qxx = mom->xxxx + mom->xxyy + mom->xxzz;
        Qxy = mom->xxxy + mom->xyyy + mom->xyzz;
        Qxz = mom->xxxz + mom->xyyz + mom->xzzz;
        Qyy = mom->xxyy + mom->yyyy + mom->yyzz;
        Qyz = mom->xxyz + mom->yyyz + mom->yzzz;
        Qzz = mom->xxzz + mom->yyzz + mom->zzzz;
        Qtr = (1.0 / 8.0) * (Qxx + Qyy + Qzz);
        Qhx = 0.5 * (Qxx * dx + Qxy * dy + Qxz * dz);
        Qhy = 0.5 * (Qxy * dx + Qyy * dy + Qyz * dz);
        Qhz = 0.5 * (Qxz * dx + Qyz * dy + Qzz * dz);
        Qh = 0.5 * (Qhx * dx + Qhy * dy + Qhz * dz);
        *fPot -= gam[4] * Qmir - gam[3] * Qh + gam[2] * Qtr;
        Qta += gam[5] * Qmir - gam[4] * Qh + gam[3] * Qtr;
        *ax += gam[4] * Qmirx - gam[3] * Qhx;
        *ay += gam[4] * Qmiry - gam[3] * Qhy;
        *az += gam[4] * Qmirz - gam[3] * Qhz;
    }
    if (iOrder >= 3) {
        Qmirx = (1.0 / 2.0) * (mom->xzz * dz * dz + 2 * mom->xyz * dy * dz + mom->xyy * dy * dy + 2 * mom->xxz * dx * dz + 2 * mom->xxy * dx * dy + mom->xxx * dx * dx);
        Qmiry = (1.0 / 2.0) * (mom->yzz * dz * dz + 2 * mom->xyz * dx * dz + mom->xxy * dx * dx + 2 * mom->yyz * dy * dz + 2 * mom->xyy * dx * dy + mom->yyy * dy * dy);
        Qmirz = (1.0 / 2.0) * (mom->yyz * dy * dy + 2 * mom->xyz * dx * dy + mom->xxz * dx * dx + 2 * mom->yzz * dy * dz + 2 * mom->xzz * dx * dz + mom->zzz * dz * dz);
        Qmir = (1.0 / 3.0) * (Qmirx * dx + Qmiry * dy + Qmirz * dz);
        Qx = 0.5 * (mom->xxx + mom->xyy + mom->xzz);
        Qy = 0.5 * (mom->xxy + mom->yyy + mom->yzz);
        Qz = 0.5 * (mom->xxz + mom->yyz + mom->zzz);
        Qtr = Qx * dx + Qy * dy + Qz * dz;
        *fPot -= gam[3] * Qmir - gam[2] * Qtr;
        Qta += gam[4] * Qmir - gam[3] * Qtr;
        *ax += gam[3] * Qmirx - gam[2] * Qx;
        *ay += gam[3] * Qmiry - gam[2] * Qy;
        *az += gam[3] * Qmirz - gam[2] * Qz;
    }
    if (iOrder >= 2) {
        Qmirx = (1.0 / 1.0) * (mom->xz * dz + mom->xy * dy + mom->xx * dx);
        Qmiry = (1.0 / 1.0) * (mom->yz * dz + mom->xy * dx + mom->yy * dy);
        Qmirz = (1.0 / 1.0) * (mom->yz * dy + mom->xz * dx + mom->zz * dz);
        Qmir = (1.0 / 2.0) * (Qmirx * dx + Qmiry * dy + Qmirz * dz);
        Qtr = 0.5 * (mom->xx + mom->yy + mom->zz);
        *fPot -= gam[2] * Qmir - gam[1] * Qtr;
        Qta += gam[3] * Qmir - gam[2] * Qtr;
        *ax += gam[2] * Qmirx;
        *ay += gam[2] * Qmiry;
        *az += gam[2] * Qmirz;
    }
    *fPot -= gam[0] * mom->m;
    Qta += gam[1] * mom->m;
    *ax -= dx * Qta;
    *ay -= dy * Qta;
    *az -= dz * Qta;
}

/* pkdBucketInteract (grav.c:23-249).  Particle arrays in storage order. */
static double bucket_interact(const orc_parts *P, const orc_node *b, int iOrder,
                              orc_lists_t *L, double *acc, double *pot, double *dtg) {
    static const int qflop[5] = {10, 10, 41, 120, 277};
    int n = b->pUpper - b->pLower + 1;
    int i, j, nActive = 0;
    int nPart = L->nPart, nCellSoft = L->nCellSoft, nCellNewt = L->nCellNewt;
    int nmax = nPart;
    if (nCellSoft > nmax) nmax = nCellSoft;
    if (nCellNewt > nmax) nmax = nCellNewt;
    lists_sq(L, nmax + 1);
    for (i = 0; i < n; ++i) {
        int pi = b->pLower + i;
        double ax = 0.0, ay = 0.0, az = 0.0, fPot = 0.0;
        double x = P->r[3 * pi + 0], y = P->r[3 * pi + 1], z = P->r[3 * pi + 2];
        double h = P->h[pi], pm = P->m[pi];
        double dtGrav = dtg[pi];
        ++nActive;
        for (j = 0; j < nPart; ++j) {
            double dx = x - L->ilp[j].x, dy = y - L->ilp[j].y, dz = z - L->ilp[j].z;
            L->d2a[j] = dx * dx + dy * dy + dz * dz;
        }
        for (j = 0; j < nPart; ++j) L->sq[j] = vs_one(L->d2a[j]);
        for (j = 0; j < nPart; ++j) {
            double a, bb, idt2;
            double dx = x - L->ilp[j].x, dy = y - L->ilp[j].y, dz = z - L->ilp[j].z;
            double twoh = h + L->ilp[j].h;
            splinem(L->sq[j], L->d2a[j], twoh, &a, &bb);
            idt2 = (pm + L->ilp[j].m) * bb;
            if (idt2 > dtGrav) dtGrav = idt2;
            a *= L->ilp[j].m;
            bb *= L->ilp[j].m;
            fPot -= a;
            ax -= dx * bb;
            ay -= dy * bb;
            az -= dz * bb;
        }
        for (j = 0; j < nCellSoft; ++j) {
            double dx = x - L->ilcs[j].x, dy = y - L->ilcs[j].y, dz = z - L->ilcs[j].z;
            L->d2a[j] = dx * dx + dy * dy + dz * dz;
        }
        for (j = 0; j < nCellSoft; ++j) L->sq[j] = vs_one(L->d2a[j]);
        for (j = 0; j < nCellSoft; ++j) {
            const orc_ilcs *q = &L->ilcs[j];
            double a, bb, c, d, qirx, qiry, qirz, qir, tr, qir3, idt2;
            double dx = x - q->x, dy = y - q->y, dz = z - q->z;
            double twoh = h + q->h;
            splineq(L->sq[j], L->d2a[j], twoh, &a, &bb, &c, &d);
            qirx = q->xx * dx + q->xy * dy + q->xz * dz;
            qiry = q->xy * dx + q->yy * dy + q->yz * dz;
            qirz = q->xz * dx + q->yz * dy + q->zz * dz;
            qir = 0.5 * (qirx * dx + qiry * dy + qirz * dz);
            tr = 0.5 * (q->xx + q->yy + q->zz);
            qir3 = bb * q->m + d * qir - c * tr;
            fPot -= a * q->m + c * qir - bb * tr;
            ax -= qir3 * dx - c * qirx;
            ay -= qir3 * dy - c * qiry;
            az -= qir3 * dz - c * qirz;
            idt2 = (pm + q->m) * bb;
            if (idt2 > dtGrav) dtGrav = idt2;
        }
        for (j = 0; j < nCellNewt; ++j) {
            double dx = x - L->ilcn[j].x, dy = y - L->ilcn[j].y, dz = z - L->ilcn[j].z;
            L->d2a[j] = dx * dx + dy * dy + dz * dz;
        }
        for (j = 0; j < nCellNewt; ++j) L->sq[j] = vs_one(L->d2a[j]);
        for (j = 0; j < nCellNewt; ++j) {
            double gam[6], dir2, idt2;
            double dx = x - L->ilcn[j].x, dy = y - L->ilcn[j].y, dz = z - L->ilcn[j].z;
            gam[0] = L->sq[j];
            dir2 = gam[0] * gam[0];
            gam[1] = gam[0] * dir2;
            gam[2] = 3 * gam[1] * dir2;
            gam[3] = 5 * gam[2] * dir2;
            gam[4] = 7 * gam[3] * dir2;
            gam[5] = 9 * gam[4] * dir2;
            qeval(iOrder, &L->ilcn[j], gam, dx, dy, dz, &ax, &ay, &az, &fPot);
            idt2 = (pm + L->ilcn[j].m) * gam[1];
            if (idt2 > dtGrav) dtGrav = idt2;
        }
        pot[pi] += fPot;
        acc[3 * pi + 0] += ax;
        acc[3 * pi + 1] += ay;
        acc[3 * pi + 2] += az;
        dtg[pi] = dtGrav;
    }
    /* intra-bucket pairs */
    for (i = 0; i < n - 1; ++i) {
        for (j = i + 1; j < n; ++j) {
            int pi = b->pLower + i, pj = b->pLower + j;
            double a, bb, idt2, twoh;
            double dx = P->r[3 * pj + 0] - P->r[3 * pi + 0];
            double dy = P->r[3 * pj + 1] - P->r[3 * pi + 1];
            double dz = P->r[3 * pj + 2] - P->r[3 * pi + 2];
            double d2 = dx * dx + dy * dy + dz * dz;
            twoh = P->h[pi] + P->h[pj];
            spline(d2, twoh, &a, &bb);
            idt2 = (P->m[pi] + P->m[pj]) * bb;
            pot[pj] -= a * P->m[pi];
            acc[3 * pj + 0] -= dx * bb * P->m[pi];
            acc[3 * pj + 1] -= dy * bb * P->m[pi];
            acc[3 * pj + 2] -= dz * bb * P->m[pi];
            if (idt2 > dtg[pj]) dtg[pj] = idt2;
            pot[pi] -= a * P->m[pj];
            acc[3 * pi + 0] += dx * bb * P->m[pj];
            acc[3 * pi + 1] += dy * bb * P->m[pj];
            acc[3 * pi + 2] += dz * bb * P->m[pj];
            if (idt2 > dtg[pi]) dtg[pi] = idt2;
        }
    }
    return (double)nActive * ((double)(nPart + n) * 38 + nCellSoft * 82.0 +
                              nCellNewt * (35.0 + qflop[iOrder]));
}

/* ------------------------------------------------------------------ */
/* Ewald                                                               */
/* ------------------------------------------------------------------ */
typedef struct { double hx, hy, hz, hCfac, hSfac; } orc_ewt;

/* pkdCalcRoot + pkdDistribRoot (pkd.c:4395-4493): complete moments. */
static void calc_root(const orc_parts *P, const orc_tree_t *T, orc_ilcn *R) {
    const orc_node *c = &T->c[0];
    int pj;
    double tr = 0.0;
    memset(R, 0, sizeof(*R));
    for (pj = c->pLower; pj <= c->pUpper; ++pj) {
        double m = P->m[pj];
        double dx = P->r[3 * pj + 0] - c->r[0];
        double dy = P->r[3 * pj + 1] - c->r[1];
        double dz = P->r[3 * pj + 2] - c->r[2];
        double d2 = 0.0;
        R->xxxx += m * (dx * dx * dx * dx - 6.0 / 7.0 * d2 * (dx * dx - 0.1 * d2));
        R->xyyy += m * (dx * dy * dy * dy - 3.0 / 7.0 * d2 * dx * dy);
        R->xxxy += m * (dx * dx * dx * dy - 3.0 / 7.0 * d2 * dx * dy);
        R->yyyy += m * (dy * dy * dy * dy - 6.0 / 7.0 * d2 * (dy * dy - 0.1 * d2));
        R->xxxz += m * (dx * dx * dx * dz - 3.0 / 7.0 * d2 * dx * dz);
        R->yyyz += m * (dy * dy * dy * dz - 3.0 / 7.0 * d2 * dy * dz);
        R->xxyy += m * (dx * dx * dy * dy - 1.0 / 7.0 * d2 * (dx * dx + dy * dy - 0.2 * d2));
        R->xxyz += m * (dx * dx * dy * dz - 1.0 / 7.0 * d2 * dy * dz);
        R->xyyz += m * (dx * dy * dy * dz - 1.0 / 7.0 * d2 * dx * dz);
        R->xxzz += m * (dx * dx * dz * dz - 1.0 / 7.0 * d2 * (dx * dx + dz * dz - 0.2 * d2));
        R->xyzz += m * (dx * dy * dz * dz - 1.0 / 7.0 * d2 * dx * dy);
        R->xzzz += m * (dx * dz * dz * dz - 3.0 / 7.0 * d2 * dx * dz);
        R->yyzz += m * (dy * dy * dz * dz - 1.0 / 7.0 * d2 * (dy * dy + dz * dz - 0.2 * d2));
        R->yzzz += m * (dy * dz * dz * dz - 3.0 / 7.0 * d2 * dy * dz);
        R->zzzz += m * (dz * dz * dz * dz - 6.0 / 7.0 * d2 * (dz * dz - 0.1 * d2));
        R->xxx += m * (dx * dx * dx - 0.6 * d2 * dx);
        R->xyy += m * (dx * dy * dy - 0.2 * d2 * dx);
        R->xxy += m * (dx * dx * dy - 0.2 * d2 * dy);
        R->yyy += m * (dy * dy * dy - 0.6 * d2 * dy);
        R->xxz += m * (dx * dx * dz - 0.2 * d2 * dz);
        R->yyz += m * (dy * dy * dz - 0.2 * d2 * dz);
        R->xyz += m * dx * dy * dz;
        R->xzz += m * (dx * dz * dz - 0.2 * d2 * dx);
        R->yzz += m * (dy * dz * dz - 0.2 * d2 * dy);
        R->zzz += m * (dz * dz * dz - 0.6 * d2 * dz);
    }
    R->m = c->fMass;
    R->x = c->r[0];
    R->y = c->r[1];
    R->z = c->r[2];
    R->xx = c->Qxx - tr / 3.0;
    R->xy = c->Qxy;
    R->xz = c->Qxz;
    R->yy = c->Qyy - tr / 3.0;
    R->yz = c->Qyz;
    R->zz = c->Qzz - tr / 3.0;
}

/* pkdEwaldInit (ewald.c:182-248). Returns the table length. */
static int ewald_init(const orc_ilcn *mom, double L, double fhCut, int iOrder, orc_ewt **pewt) {
    int hReps = (int)ceil(fhCut), hx, hy, hz, i = 0, nMax = 128;
    double alpha = 2.0 / L;
    double k4 = M_PI * M_PI / (alpha * alpha * L * L);
    orc_ewt *ewt = malloc(sizeof(orc_ewt) * (size_t)nMax);
    for (hx = -hReps; hx <= hReps; ++hx)
        for (hy = -hReps; hy <= hReps; ++hy)
            for (hz = -hReps; hz <= hReps; ++hz) {
                double gam[6], ax, ay, az, mfacc, mfacs;
                int h2 = hx * hx + hy * hy + hz * hz;
                if (h2 == 0) continue;
                if (h2 > fhCut * fhCut) continue;
                if (i == nMax) {
                    nMax *= 2;
                    ewt = realloc(ewt, sizeof(orc_ewt) * (size_t)nMax);
                }
                gam[0] = exp(-k4 * h2) / (M_PI * h2 * L);
                gam[1] = 2 * M_PI / L * gam[0];
                gam[2] = -2 * M_PI / L * gam[1];
                gam[3] = 2 * M_PI / L * gam[2];
                gam[4] = -2 * M_PI / L * gam[3];
                gam[5] = 2 * M_PI / L * gam[4];
                gam[1] = 0.0; gam[3] = 0.0; gam[5] = 0.0;
                ax = ay = az = 0.0;
                mfacc = 0.0;
                qeval(iOrder, mom, gam, (double)hx, (double)hy, (double)hz, &ax, &ay, &az, &mfacc);
                gam[0] = exp(-k4 * h2) / (M_PI * h2 * L);
                gam[1] = 2 * M_PI / L * gam[0];
                gam[2] = -2 * M_PI / L * gam[1];
                gam[3] = 2 * M_PI / L * gam[2];
                gam[4] = -2 * M_PI / L * gam[3];
                gam[5] = 2 * M_PI / L * gam[4];
                gam[0] = 0.0; gam[2] = 0.0; gam[4] = 0.0;
                ax = ay = az = 0.0;
                mfacs = 0.0;
                qeval(iOrder, mom, gam, (double)hx, (double)hy, (double)hz, &ax, &ay, &az, &mfacs);
                ewt[i].hx = 2 * M_PI / L * hx;
                ewt[i].hy = 2 * M_PI / L * hy;
                ewt[i].hz = 2 * M_PI / L * hz;
                ewt[i].hCfac = mfacc;
                ewt[i].hSfac = mfacs;
                ++i;
            }
    *pewt = ewt;
    return i;
}

/* pkdBucketEwald (ewald.c:15-178). */
static double bucket_ewald(const orc_parts *P, const orc_node *b, int nReps,
                           double fEwCut, int iOrder, const orc_ilcn *mom,
                           double L, const orc_ewt *ewt, int nEwh,
                           double *acc, double *pot) {
    static const int mflop[5] = {10, 10, 48, 151, 343};
    int nEwReps, j, ix, iy, iz, nLoop = 0, nActive = 0;
    double alpha, alpha2, k1, ka, fEwCut2;
    if (!iOrder) return 0;
    nEwReps = (int)ceil(fEwCut);
    fEwCut2 = fEwCut * fEwCut * L * L;
    nEwReps = nEwReps > nReps ? nEwReps : nReps;
    alpha = 2.0 / L;
    alpha2 = alpha * alpha;
    k1 = M_PI / (alpha2 * L * L * L);
    ka = 2.0 * alpha / sqrt(M_PI);
    for (j = b->pLower; j <= b->pUpper; ++j) {
        double fPot = mom->m * k1, ax = 0.0, ay = 0.0, az = 0.0;
        double dx = P->r[3 * j + 0] - mom->x;
        double dy = P->r[3 * j + 1] - mom->y;
        double dz = P->r[3 * j + 2] - mom->z;
        int i;
        for (ix = -nEwReps; ix <= nEwReps; ++ix) {
            int bInHolex = (ix >= -nReps && ix <= nReps);
            double dxo = dx + ix * L;
            for (iy = -nEwReps; iy <= nEwReps; ++iy) {
                int bInHolexy = (bInHolex && iy >= -nReps && iy <= nReps);
                double dyo = dy + iy * L;
                for (iz = -nEwReps; iz <= nEwReps; ++iz) {
                    int bInHole = (bInHolexy && iz >= -nReps && iz <= nReps);
                    double dzo = dz + iz * L;
                    double r2 = dxo * dxo + dyo * dyo + dzo * dzo;
                    double gam[6], alphan;
                    if (r2 > fEwCut2 && !bInHole) continue;
                    if (r2 < 3.0e-3 * L * L) {
                        alphan = ka;
                        r2 *= alpha2;
                        gam[0] = alphan * (r2 / 3 - 1);
                        alphan *= 2 * alpha2;
                        gam[1] = alphan * (r2 / 5 - 1.0 / 3.0);
                        alphan *= 2 * alpha2;
                        gam[2] = alphan * (r2 / 7 - 1.0 / 5.0);
                        alphan *= 2 * alpha2;
                        gam[3] = alphan * (r2 / 9 - 1.0 / 7.0);
                        alphan *= 2 * alpha2;
                        gam[4] = alphan * (r2 / 11 - 1.0 / 9.0);
                        alphan *= 2 * alpha2;
                        gam[5] = alphan * (r2 / 13 - 1.0 / 11.0);
                    } else {
                        double r = sqrt(r2), dir, dir2, a;
                        dir = 1 / r;
                        dir2 = dir * dir;
                        a = exp(-r2 * alpha2);
                        a *= ka * dir2;
                        if (bInHole) gam[0] = -erf(alpha * r);
                        else gam[0] = erfc(alpha * r);
                        gam[0] *= dir;
                        gam[1] = gam[0] * dir2 + a;
                        alphan = 2 * alpha2;
                        gam[2] = 3 * gam[1] * dir2 + alphan * a;
                        alphan *= 2 * alpha2;
                        gam[3] = 5 * gam[2] * dir2 + alphan * a;
                        alphan *= 2 * alpha2;
                        gam[4] = 7 * gam[3] * dir2 + alphan * a;
                        alphan *= 2 * alpha2;
                        gam[5] = 9 * gam[4] * dir2 + alphan * a;
                    }
                    meval(iOrder, mom, gam, dxo, dyo, dzo, &ax, &ay, &az, &fPot);
                    ++nLoop;
                }
            }
        }
        for (i = 0; i < nEwh; ++i) {
            double hdotx = ewt[i].hx * dx + ewt[i].hy * dy + ewt[i].hz * dz;
            double c = cos(hdotx), s = sin(hdotx);
            fPot += ewt[i].hCfac * c + ewt[i].hSfac * s;
            ax += ewt[i].hx * (ewt[i].hCfac * s - ewt[i].hSfac * c);
            ay += ewt[i].hy * (ewt[i].hCfac * s - ewt[i].hSfac * c);
            az += ewt[i].hz * (ewt[i].hCfac * s - ewt[i].hSfac * c);
        }
        pot[j] += fPot;
        acc[3 * j + 0] += ax;
        acc[3 * j + 1] += ay;
        acc[3 * j + 2] += az;
        ++nActive;
    }
    return nLoop * (104.0 + mflop[iOrder]) + (double)nActive * nEwh * 58.0;
}

/* ------------------------------------------------------------------ */
/* gravity driver                                                      */
/* ------------------------------------------------------------------ */
static void setup_grav(orc_parts *P, orc_tree_t *T, const orc_grav_params *gp) {
    int iOrderTree = gp->iOrder;
    if (gp->bPeriodic && gp->bEwald && gp->iEwOrder > iOrderTree) iOrderTree = gp->iEwOrder;
    build_tree(P, T, gp->nBucket, gp->dTheta, iOrderTree);
}

static void active_bounds(const orc_parts *P, const orc_node *b, double *bmin, double *bmax) {
    int i, j;
    for (j = 0; j < 3; ++j) { bmin[j] = ORC_FLOAT_MAX; bmax[j] = -ORC_FLOAT_MAX; }
    for (i = b->pLower; i <= b->pUpper; ++i)
        for (j = 0; j < 3; ++j) {
            double x = P->r[3 * i + j];
            if (x < bmin[j]) bmin[j] = x;
            if (x > bmax[j]) bmax[j] = x;
        }
}

int orc_grav(int n, const double *pos, const double *mass, const double *soft,
             const orc_grav_params *gp, double *acc, double *pot,
             double *dtGrav, double *counters, int nthreads) {
    orc_parts P;
    orc_tree_t T;
    orc_ilcn root;
    orc_ewt *ewt = NULL;
    int nEwh = 0, nb = 0, i, k, *leaf;
    double fPeriod[3], *a, *pt, *dg;
    double cnt[5] = {0, 0, 0, 0, 0};
    int bEw = gp->bPeriodic && gp->bEwald;
    int nReps = gp->bPeriodic ? gp->nReps : 0;
    vs_init();
    parts_init(&P, n, pos, mass, soft);
    setup_grav(&P, &T, gp);
    for (k = 0; k < 3; ++k) fPeriod[k] = gp->bPeriodic ? gp->dPeriod : ORC_FLOAT_MAX;
    if (bEw) {
        calc_root(&P, &T, &root);
        nEwh = ewald_init(&root, fPeriod[0], gp->fEwhCut, gp->iEwOrder, &ewt);
    }
    a = calloc((size_t)3 * (n > 0 ? n : 1), sizeof(double));
    pt = calloc((size_t)(n > 0 ? n : 1), sizeof(double));
    dg = calloc((size_t)(n > 0 ? n : 1), sizeof(double));
    leaf = malloc(sizeof(int) * (size_t)T.nNodes);
    for (i = 0; i < T.nNodes; ++i)
        if (T.c[i].iLower == -1 && T.c[i].pLower <= T.c[i].pUpper) leaf[nb++] = i;
#ifdef _OPENMP
    if (nthreads > 1) omp_set_num_threads(nthreads);
#pragma omp parallel if (nthreads > 1)
#endif
    {
        orc_lists_t L;
        double c1 = 0, c2 = 0, c3 = 0, c4 = 0, c0 = 0;
        int ib;
        lists_init(&L);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
        for (ib = 0; ib < nb; ++ib) {
            const orc_node *b = &T.c[leaf[ib]];
            double bbmin[3], bbmax[3], fl;
            int nn = b->pUpper - b->pLower + 1;
            active_bounds(&P, b, bbmin, bbmax);
            bucket_walk(&P, &T, leaf[ib], bbmin, bbmax, nReps, fPeriod, gp->iOrder, &L);
            c0 += nn;
            c1 += (double)nn * L.nPart + (double)nn * (2 * (b->pUpper - b->pLower) - nn + 1) / 2;
            c2 += (double)nn * L.nCellNewt;
            c3 += (double)nn * L.nCellSoft;
            fl = bucket_interact(&P, b, gp->iOrder, &L, a, pt, dg);
            if (bEw)
                fl += bucket_ewald(&P, b, nReps, gp->fEwCut, gp->iEwOrder, &root,
                                   fPeriod[0], ewt, nEwh, a, pt);
            c4 += fl;
        }
#ifdef _OPENMP
#pragma omp critical
#endif
        {
            cnt[0] += c0; cnt[1] += c1; cnt[2] += c2; cnt[3] += c3; cnt[4] += c4;
        }
        lists_free(&L);
    }
    for (i = 0; i < n; ++i) {
        int o = P.iord[i];
        for (k = 0; k < 3; ++k) acc[3 * o + k] = a[3 * i + k];
        pot[o] = pt[i];
        dtGrav[o] = dg[i];
    }
    if (counters) for (k = 0; k < 5; ++k) counters[k] = cnt[k];
    free(a); free(pt); free(dg); free(leaf); free(ewt);
    free(T.c);
    parts_free(&P);
    return nb;
}

int orc_tree(int n, const double *pos, const double *mass, const double *soft,
             const orc_grav_params *gp, int *inode, double *dnode, int *perm) {
    orc_parts P;
    orc_tree_t T;
    int i, j, nn;
    parts_init(&P, n, pos, mass, soft);
    setup_grav(&P, &T, gp);
    nn = T.nNodes;
    if (inode) {
        for (i = 0; i < nn; ++i) {
            const orc_node *c = &T.c[i];
            inode[6 * i + 0] = c->pLower;
            inode[6 * i + 1] = c->pUpper;
            inode[6 * i + 2] = c->iDim;
            inode[6 * i + 3] = c->iLower;
            inode[6 * i + 4] = c->iUpper;
            inode[6 * i + 5] = 0;
            dnode[16 * i + 0] = c->fSplit;
            for (j = 0; j < 3; ++j) {
                dnode[16 * i + 1 + j] = c->bmin[j];
                dnode[16 * i + 4 + j] = c->bmax[j];
                dnode[16 * i + 9 + j] = c->r[j];
            }
            dnode[16 * i + 7] = c->fMass;
            dnode[16 * i + 8] = c->fSoft;
            dnode[16 * i + 12] = c->fOpen2;
            dnode[16 * i + 13] = c->Bmax;
            dnode[16 * i + 14] = c->Qxx;
            dnode[16 * i + 15] = c->Qyy;
        }
        for (i = 0; i < n; ++i) perm[i] = P.iord[i];
    }
    free(T.c);
    parts_free(&P);
    return nn;
}

int orc_lists(int n, const double *pos, const double *mass, const double *soft,
              const orc_grav_params *gp, int *blist) {
    orc_parts P;
    orc_tree_t T;
    orc_lists_t L;
    double fPeriod[3];
    int i, k, nb = 0;
    parts_init(&P, n, pos, mass, soft);
    setup_grav(&P, &T, gp);
    lists_init(&L);
    for (k = 0; k < 3; ++k) fPeriod[k] = gp->bPeriodic ? gp->dPeriod : ORC_FLOAT_MAX;
    for (i = 0; i < T.nNodes; ++i) {
        const orc_node *b = &T.c[i];
        double bbmin[3], bbmax[3];
        if (b->iLower != -1 || b->pLower > b->pUpper) continue;
        active_bounds(&P, b, bbmin, bbmax);
        bucket_walk(&P, &T, i, bbmin, bbmax, gp->bPeriodic ? gp->nReps : 0,
                    fPeriod, gp->iOrder, &L);
        if (blist) {
            blist[4 * nb + 0] = i;
            blist[4 * nb + 1] = L.nPart;
            blist[4 * nb + 2] = L.nCellSoft;
            blist[4 * nb + 3] = L.nCellNewt;
        }
        ++nb;
    }
    lists_free(&L);
    free(T.c);
    parts_free(&P);
    return nb;
}

/* ------------------------------------------------------------------ */
/* SPH                                                                 */
/* ------------------------------------------------------------------ */
/* M4 kernel and derivative (smoothfcn.c KERNEL/DKERNEL, M4 branch). */
static inline double kern_m4(double ar2) {
    double ak = 2.0 - sqrt(ar2);
    if (ar2 < 1.0) ak = (1.0 - 0.75 * ak * ar2);
    else ak = 0.25 * ak * ak * ak;
    return ak;
}
static inline double dkern_m4(double ar2) {
    double adk = sqrt(ar2);
    if (ar2 < 1.0) adk = -3 + 2.25 * adk;
    else adk = -0.75 * (2.0 - adk) * (2.0 - adk) / adk;
    return adk;
}

typedef struct { double d2; int j; double dx, dy, dz; } orc_nb;

/* image of query x chosen for particle coordinate q: the nearer of x, x+L,
 * x-L, computed as x+s like the periodic INTERSECT (smooth.h:291-390). */
static inline double img(double x, double q, double L, int bPer) {
    double d0, dp, dm;
    if (!bPer) return x;
    d0 = fabs(x - q);
    dp = fabs((x + L) - q);
    dm = fabs((x - L) - q);
    if (dp < d0 && dp <= dm) return x + L;
    if (dm < d0 && dm < dp) return x - L;
    return x;
}

static inline double box_d2(const orc_node *c, double x, double y, double z, double L, int bPer) {
    double q[3] = {x, y, z}, d2 = 0.0;
    int k;
    for (k = 0; k < 3; ++k) {
        double lo = c->bmin[k] - q[k], hi = q[k] - c->bmax[k], d = 0.0;
        if (lo > 0.0) d = lo;
        else if (hi > 0.0) d = hi;
        if (bPer) {
            double lo2 = c->bmin[k] - (q[k] + L), hi2 = (q[k] + L) - c->bmax[k];
            double lo3 = c->bmin[k] - (q[k] - L), hi3 = (q[k] - L) - c->bmax[k];
            double d2a = lo2 > 0 ? lo2 : (hi2 > 0 ? hi2 : 0.0);
            double d3a = lo3 > 0 ? lo3 : (hi3 > 0 ? hi3 : 0.0);
            if (d2a < d) d = d2a;
            if (d3a < d) d = d3a;
        }
        d2 += d * d;
    }
    return d2;
}

/* max-heap on d2 of size k */
static void heap_push(orc_nb *h, int *nh, int k, orc_nb e) {
    int i;
    if (*nh < k) {
        i = (*nh)++;
        while (i > 0) {
            int p = (i - 1) / 2;
            if (h[p].d2 >= e.d2) break;
            h[i] = h[p];
            i = p;
        }
        h[i] = e;
    } else if (e.d2 < h[0].d2) {
        int n = *nh;
        i = 0;
        for (;;) {
            int l = 2 * i + 1, r = l + 1, m = i;
            double dm = e.d2;
            if (l < n && h[l].d2 > dm) { m = l; dm = h[l].d2; }
            if (r < n && h[r].d2 > dm) { m = r; }
            if (m == i) break;
            h[i] = h[m];
            i = m;
        }
        h[i] = e;
    }
}

static int knn_one(const orc_parts *P, const orc_tree_t *T, int pi, int k, double L,
                   int bPer, orc_nb *heap, int *stack) {
    int nh = 0, sp = 0;
    double x = P->r[3 * pi], y = P->r[3 * pi + 1], z = P->r[3 * pi + 2];
    stack[sp++] = 0;
    while (sp > 0) {
        int ic = stack[--sp];
        const orc_node *c = &T->c[ic];
        if (nh == k && box_d2(c, x, y, z, L, bPer) > heap[0].d2) continue;
        if (c->iDim == -1) {
            int pj;
            for (pj = c->pLower; pj <= c->pUpper; ++pj) {
                orc_nb e;
                double sx = img(x, P->r[3 * pj], L, bPer);
                double sy = img(y, P->r[3 * pj + 1], L, bPer);
                double sz = img(z, P->r[3 * pj + 2], L, bPer);
                e.dx = sx - P->r[3 * pj];
                e.dy = sy - P->r[3 * pj + 1];
                e.dz = sz - P->r[3 * pj + 2];
                e.d2 = e.dx * e.dx + e.dy * e.dy + e.dz * e.dz;
                e.j = pj;
                heap_push(heap, &nh, k, e);
            }
        } else {
            /* children are ic+1 (lower) and the other; push farther first */
            int lo = ic + 1;
            int up = -1;
            /* upper child index: first node after the lower subtree */
            {
                const orc_node *cl = &T->c[lo];
                up = (cl->iUpper);  /* threaded next of the lower child */
            }
            {
                double dl = box_d2(&T->c[lo], x, y, z, L, bPer);
                double du = box_d2(&T->c[up], x, y, z, L, bPer);
                if (dl <= du) { stack[sp++] = up; stack[sp++] = lo; }
                else { stack[sp++] = lo; stack[sp++] = up; }
            }
        }
    }
    return nh;
}

static int cmp_nb(const void *a, const void *b) {
    const orc_nb *x = a, *y = b;
    if (x->d2 < y->d2) return -1;
    if (x->d2 > y->d2) return 1;
    return x->j - y->j;
}

int orc_knn(int n, const double *pos, int nSmooth, int bPeriodic,
            double dPeriod, double *fBall2, int nthreads) {
    orc_parts P;
    orc_tree_t T;
    double *ones = malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    int i, k = nSmooth < n ? nSmooth : n;
    for (i = 0; i < n; ++i) ones[i] = 1.0;
    parts_init(&P, n, pos, ones, NULL);
    build_tree(&P, &T, 8, 0.7, 2);
#ifdef _OPENMP
    if (nthreads > 1) omp_set_num_threads(nthreads);
#pragma omp parallel if (nthreads > 1)
#endif
    {
        orc_nb *heap = malloc(sizeof(orc_nb) * (size_t)(k + 1));
        int *stack = malloc(sizeof(int) * 4096);
        int ii;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 256)
#endif
        for (ii = 0; ii < n; ++ii) {
            knn_one(&P, &T, ii, k, dPeriod, bPeriodic, heap, stack);
            fBall2[P.iord[ii]] = heap[0].d2;
        }
        free(heap);
        free(stack);
    }
    free(T.c);
    parts_free(&P);
    free(ones);
    return 0;
}

int orc_sph(int n, const double *pos, const double *vel, const double *mass,
            const double *soft, const double *u, const orc_sph_params *sp,
            double *out, double *dtNew, double *mumax, int *nbr_count,
            unsigned long long *nbr_hash, int nthreads) {
    orc_parts P;
    orc_tree_t T;
    int i, k = sp->nSmooth < n ? sp->nSmooth : n;
    double L = sp->dPeriod;
    int bPer = sp->bPeriodic;
    double gamma = sp->gamma, gammam1 = sp->gamma - 1;
    double dtFacCourant = sp->dEtaCourant * 1.0 * 2 / 1.6;   /* pkd.c:5893-5895 */
    double H = 0.0, aFac = 1.0, vFac = 1.0;
    /* storage-order copies */
    double *v, *uu, *fBall2, *rho, *divv, *curl, *dvds, *bal, *diffc, *pr2, *cs, *dtp;
    double *ah, *updv, *uav, *dtn, *mum;
    int *nn_off, *nn_idx, *rv_off, *rv_idx, *rv_fill;
    parts_init(&P, n, pos, mass, soft);
    build_tree(&P, &T, sp->nBucket > 0 ? sp->nBucket : 8, 0.7, 2);
#define ALLOCD(p_, m_) p_ = calloc((size_t)(m_) * (size_t)(n > 0 ? n : 1), sizeof(double))
    ALLOCD(v, 3); ALLOCD(uu, 1); ALLOCD(fBall2, 1); ALLOCD(rho, 1); ALLOCD(divv, 1);
    ALLOCD(curl, 3); ALLOCD(dvds, 1); ALLOCD(bal, 1); ALLOCD(diffc, 1); ALLOCD(pr2, 1);
    ALLOCD(cs, 1); ALLOCD(dtp, 1); ALLOCD(ah, 3); ALLOCD(updv, 1); ALLOCD(uav, 1);
    ALLOCD(dtn, 1); ALLOCD(mum, 1);
#undef ALLOCD
    for (i = 0; i < n; ++i) {
        int o = P.iord[i], j;
        for (j = 0; j < 3; ++j) v[3 * i + j] = vel[3 * o + j];
        uu[i] = u[o];
    }
    /* pass 1: kNN (smSmooth semantics: fBall2 = k-th smallest d^2, self
     * included) and DenDVDX over the k neighbours. */
    nn_off = malloc(sizeof(int) * (size_t)(n + 1));
#ifdef _OPENMP
    if (nthreads > 1) omp_set_num_threads(nthreads);
#pragma omp parallel if (nthreads > 1)
#endif
    {
        orc_nb *heap = malloc(sizeof(orc_nb) * (size_t)(k + 1));
        int *stack = malloc(sizeof(int) * 4096);
        int pi;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 64)
#endif
        for (pi = 0; pi < n; ++pi) {
            int nh = knn_one(&P, &T, pi, k, L, bPer, heap, stack), ii;
            double ih2, ih, fNorm, fNorm1, fDensity = 0.0;
            double dvxdx = 0, dvxdy = 0, dvxdz = 0, dvydx = 0, dvydy = 0, dvydz = 0;
            double dvzdx = 0, dvzdy = 0, dvzdz = 0, grx = 0, gry = 0, grz = 0;
            double divvnorm = 0, trace, gnorm, dvdr, Hcorr;
            qsort(heap, (size_t)nh, sizeof(orc_nb), cmp_nb);
            fBall2[pi] = heap[nh - 1].d2;
            ih2 = 4.0 / fBall2[pi];
            ih = sqrt(ih2);
            fNorm = M_1_PI * ih2 * ih;
            fNorm1 = fNorm * ih2;
            (void)fNorm1;
            for (ii = 0; ii < nh; ++ii) {
                int q = heap[ii].j;
                double r2 = heap[ii].d2 * ih2, rs, rs1, dx, dy, dz, dvx, dvy, dvz;
                rs = kern_m4(r2);
                fDensity += rs * P.m[q];
                rs1 = dkern_m4(r2);
                rs1 *= P.m[q];
                dx = heap[ii].dx; dy = heap[ii].dy; dz = heap[ii].dz;
                dvx = (-v[3 * pi + 0] + v[3 * q + 0]) * vFac;
                dvy = (-v[3 * pi + 1] + v[3 * q + 1]) * vFac;
                dvz = (-v[3 * pi + 2] + v[3 * q + 2]) * vFac;
                dvxdx += dvx * dx * rs1; dvxdy += dvx * dy * rs1; dvxdz += dvx * dz * rs1;
                dvydx += dvy * dx * rs1; dvydy += dvy * dy * rs1; dvydz += dvy * dz * rs1;
                dvzdx += dvz * dx * rs1; dvzdy += dvz * dy * rs1; dvzdz += dvz * dz * rs1;
                divvnorm += (dx * dx + dy * dy + dz * dz) * rs1;
                grx += (uu[q]) * dx * rs1;
                gry += (uu[q]) * dy * rs1;
                grz += (uu[q]) * dz * rs1;
            }
            fDensity *= fNorm;
            rho[pi] = fDensity;
            trace = dvxdx + dvydy + dvzdz;
            fNorm1 = (divvnorm != 0 ? 3 / fabs(divvnorm) : 0);
            divv[pi] = fNorm1 * trace + 3 * H;
            curl[3 * pi + 0] = fNorm1 * (dvzdy - dvydz);
            curl[3 * pi + 1] = fNorm1 * (dvxdz - dvzdx);
            curl[3 * pi + 2] = fNorm1 * (dvydx - dvxdy);
            Hcorr = (fNorm1 != 0 ? H / fNorm1 : 0);
            gnorm = (grx * grx + gry * gry + grz * grz);
            if (gnorm > 0) gnorm = 1 / sqrt(gnorm);
            grx *= gnorm; gry *= gnorm; grz *= gnorm;
            dvdr = (((dvxdx + Hcorr) * grx + dvxdy * gry + dvxdz * grz) * grx
                    + (dvydx * grx + (dvydy + Hcorr) * gry + dvydz * grz) * gry
                    + (dvzdx * grx + dvzdy * gry + (dvzdz + Hcorr) * grz) * grz) * fNorm1;
            dvds[pi] = (divv[pi] < 0 ? 1.5 * (dvdr - (1. / 3.) * divv[pi]) : dvdr);
            if (sp->iViscosityLimiter == 1) {
                if (divv[pi] != 0.0)
                    bal[pi] = fabs(divv[pi]) / (fabs(divv[pi]) + sqrt(curl[3 * pi] * curl[3 * pi] +
                                                                      curl[3 * pi + 1] * curl[3 * pi + 1] +
                                                                      curl[3 * pi + 2] * curl[3 * pi + 2]));
                else bal[pi] = 0;
            } else {
                bal[pi] = 1;
            }
            {
                double onethirdtrace = (1. / 3.) * trace;
                double sxx = dvxdx - onethirdtrace, syy = dvydy - onethirdtrace, szz = dvzdz - onethirdtrace;
                double sxy = 0.5 * (dvxdy + dvydx), sxz = 0.5 * (dvxdz + dvzdx), syz = 0.5 * (dvydz + dvzdy);
                double S2 = fNorm1 * fNorm1 * (sxx * sxx + syy * syy + szz * szz + 2 * (sxy * sxy + sxz * sxz + syz * syz));
                diffc[pi] = 0.25 * fBall2[pi] * sqrt(2 * S2);
            }
        }
        free(heap);
        free(stack);
    }
    /* gas pressure (pkdGasPressure, adiabatic, no Jeans floor) */
    for (i = 0; i < n; ++i) {
        double PoverRhoGas = gammam1 * uu[i];
        double cGas = sqrt(gamma * PoverRhoGas);
        double PoverRho = PoverRhoGas + 0.0;
        double dt;
        pr2[i] = PoverRho / rho[i];
        cs[i] = sqrt(cGas * cGas + (5. / 3.) * 0.0 + 2.0 * 0.0);
        dt = dtFacCourant * sqrt(fBall2[i] * 0.25) / (2 * (cs[i]));
        dtp[i] = FLT_MAX;
        if (dt < dtp[i]) dtp[i] = dt;
    }
    /* pass 2: ball gather lists N(i) = {j : d2 <= fBall2_i} and the
     * reverse lists {j : i in N(j)}. */
    {
        int *cnt = calloc((size_t)(n > 0 ? n : 1), sizeof(int));
        int **lists = malloc(sizeof(int *) * (size_t)(n > 0 ? n : 1));
#ifdef _OPENMP
#pragma omp parallel if (nthreads > 1)
#endif
        {
            int *stack = malloc(sizeof(int) * 4096);
            int *buf = malloc(sizeof(int) * 1024);
            int cap = 1024, pi;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 64)
#endif
            for (pi = 0; pi < n; ++pi) {
                double x = P.r[3 * pi], y = P.r[3 * pi + 1], z = P.r[3 * pi + 2];
                int spn = 0, nc = 0;
                stack[spn++] = 0;
                while (spn > 0) {
                    int ic = stack[--spn];
                    const orc_node *c = &T.c[ic];
                    if (box_d2(c, x, y, z, L, bPer) > fBall2[pi]) continue;
                    if (c->iDim == -1) {
                        int pj;
                        for (pj = c->pLower; pj <= c->pUpper; ++pj) {
                            double sx = img(x, P.r[3 * pj], L, bPer);
                            double sy = img(y, P.r[3 * pj + 1], L, bPer);
                            double sz = img(z, P.r[3 * pj + 2], L, bPer);
                            double dx = sx - P.r[3 * pj], dy = sy - P.r[3 * pj + 1], dz = sz - P.r[3 * pj + 2];
                            double d2 = dx * dx + dy * dy + dz * dz;
                            if (d2 <= fBall2[pi]) {
                                if (nc == cap) { cap *= 2; buf = realloc(buf, sizeof(int) * (size_t)cap); }
                                buf[nc++] = pj;
                            }
                        }
                    } else {
                        stack[spn++] = T.c[ic + 1].iUpper;
                        stack[spn++] = ic + 1;
                    }
                }
                cnt[pi] = nc;
                lists[pi] = malloc(sizeof(int) * (size_t)(nc > 0 ? nc : 1));
                memcpy(lists[pi], buf, sizeof(int) * (size_t)nc);
            }
            free(stack);
            free(buf);
        }
        nn_off[0] = 0;
        for (i = 0; i < n; ++i) nn_off[i + 1] = nn_off[i] + cnt[i];
        nn_idx = malloc(sizeof(int) * (size_t)(nn_off[n] > 0 ? nn_off[n] : 1));
        for (i = 0; i < n; ++i) {
            /* sort each list by particle index for a deterministic order */
            int a2, b2;
            for (a2 = 1; a2 < cnt[i]; ++a2) {
                int key = lists[i][a2];
                b2 = a2 - 1;
                while (b2 >= 0 && lists[i][b2] > key) { lists[i][b2 + 1] = lists[i][b2]; --b2; }
                lists[i][b2 + 1] = key;
            }
            memcpy(&nn_idx[nn_off[i]], lists[i], sizeof(int) * (size_t)cnt[i]);
            free(lists[i]);
        }
        free(lists);
        rv_off = calloc((size_t)n + 1, sizeof(int));
        for (i = 0; i < nn_off[n]; ++i) rv_off[nn_idx[i] + 1]++;
        for (i = 0; i < n; ++i) rv_off[i + 1] += rv_off[i];
        rv_idx = malloc(sizeof(int) * (size_t)(nn_off[n] > 0 ? nn_off[n] : 1));
        rv_fill = calloc((size_t)(n > 0 ? n : 1), sizeof(int));
        for (i = 0; i < n; ++i) {
            int e;
            for (e = nn_off[i]; e < nn_off[i + 1]; ++e) {
                int j = nn_idx[e];
                rv_idx[rv_off[j] + rv_fill[j]++] = i;
            }
        }
        free(cnt);
    }
    /* pass 3: SphPressureTermsSym as a two-sided gather.  For particle i:
     * pairs (p=i, q=j in N(i)) in the p role, pairs (p=j, q=i) for i in
     * N(j) in the q role (smoothfcn.c:2276-2385, SphPressureTerms.h). */
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64) if (nthreads > 1)
#endif
    for (i = 0; i < n; ++i) {
        double ax = 0, ay = 0, az = 0, uPdV = 0, uAV = 0, mu = 0.0, dtN = FLT_MAX;
        int role, e;
        for (role = 0; role < 2; ++role) {
            int e0 = role == 0 ? nn_off[i] : rv_off[i];
            int e1 = role == 0 ? nn_off[i + 1] : rv_off[i + 1];
            for (e = e0; e < e1; ++e) {
                int p = role == 0 ? i : rv_idx[e];
                int q = role == 0 ? nn_idx[e] : i;
                double pc = cs[p], pMass = P.m[p], pDensity = rho[p];
                double pPoverRho2 = pr2[p], pd2 = rho[p] * rho[p];
                double pPoverRho2f = (pPoverRho2 * pd2 + 0) / pd2;
                double ph = sqrt(0.25 * fBall2[p]);
                double ih2 = 4.0 / fBall2[p];
                double fNorm = 0.5 * M_1_PI * ih2 / ph;
                double fNorm1 = fNorm * ih2;
                double sx = img(P.r[3 * p], P.r[3 * q], L, bPer);
                double sy = img(P.r[3 * p + 1], P.r[3 * q + 1], L, bPer);
                double sz = img(P.r[3 * p + 2], P.r[3 * q + 2], L, bPer);
                double dx = sx - P.r[3 * q], dy = sy - P.r[3 * q + 1], dz = sz - P.r[3 * q + 2];
                double fDist2 = dx * dx + dy * dy + dz * dz;
                double r2 = fDist2 * ih2, rs1, rp, rq, dvx, dvy, dvz, dvdotdr;
                double qPoverRho2, qd2, qPoverRho2f, Acc, dt, visc, absmu;
                rs1 = dkern_m4(r2);
                rs1 *= fNorm1;
                rs1 *= 1.0;
                rp = rs1 * pMass;
                rq = rs1 * P.m[q];
                dvx = v[3 * p + 0] - v[3 * q + 0];
                dvy = v[3 * p + 1] - v[3 * q + 1];
                dvz = v[3 * p + 2] - v[3 * q + 2];
                dvdotdr = vFac * (dvx * dx + dvy * dy + dvz * dz) + fDist2 * H;
                qPoverRho2 = pr2[q];
                qd2 = rho[q] * rho[q];
                qPoverRho2f = (qPoverRho2 * qd2 + 0) / qd2;
                if (role == 0) {
                    uPdV += rq * pPoverRho2 * dvdotdr;
                    Acc = (pPoverRho2f + qPoverRho2f);
                } else {
                    uPdV += rp * qPoverRho2 * dvdotdr;
                    Acc = (qPoverRho2f + pPoverRho2f);
                }
                if (dvdotdr >= 0.0) {
                    dt = dtFacCourant * ph / (2 * (pc > cs[q] ? pc : cs[q]));
                } else {
                    absmu = -dvdotdr * aFac / sqrt(fDist2);
                    if (absmu > mu) mu = absmu;
                    visc = (sp->alpha * (pc + cs[q]) + sp->beta * 1.5 * absmu);
                    dt = dtFacCourant * ph / (0.625 * (pc + cs[q]) + 0.375 * visc);
                    visc = (0.5 * (bal[p] + bal[q])) * visc * absmu / (pDensity + rho[q]);
                    if (role == 0) uAV += rq * (0.5 * visc) * dvdotdr;
                    else uAV += rp * (0.5 * visc) * dvdotdr;
                    Acc += visc;
                }
                if (role == 0) {
                    Acc *= rq * aFac;
                    ax -= Acc * dx; ay -= Acc * dy; az -= Acc * dz;
                    if (dt < dtN) dtN = dt;
                    if (4 * dtp[q] < dtN) dtN = 4 * dtp[q];
                } else {
                    Acc *= rp * aFac;
                    ax += Acc * dx; ay += Acc * dy; az += Acc * dz;
                    if (dt < dtN) dtN = dt;
                    if (4 * dtp[p] < dtN) dtN = 4 * dtp[p];
                }
            }
        }
        ah[3 * i + 0] = ax; ah[3 * i + 1] = ay; ah[3 * i + 2] = az;
        updv[i] = uPdV; uav[i] = uAV; mum[i] = mu; dtn[i] = dtN;
    }
    for (i = 0; i < n; ++i) {
        int o = P.iord[i];
        double *w = &out[16 * o];
        w[0] = fBall2[i]; w[1] = rho[i]; w[2] = divv[i];
        w[3] = curl[3 * i]; w[4] = curl[3 * i + 1]; w[5] = curl[3 * i + 2];
        w[6] = dvds[i]; w[7] = bal[i]; w[8] = diffc[i]; w[9] = pr2[i]; w[10] = cs[i];
        w[11] = ah[3 * i]; w[12] = ah[3 * i + 1]; w[13] = ah[3 * i + 2];
        w[14] = updv[i]; w[15] = uav[i];
        if (dtNew) dtNew[o] = dtn[i];
        if (mumax) mumax[o] = mum[i];
        if (nbr_count) nbr_count[o] = nn_off[i + 1] - nn_off[i];
        if (nbr_hash) {
            unsigned long long hsh = 0;
            int e;
            for (e = nn_off[i]; e < nn_off[i + 1]; ++e) {
                unsigned long long x = (unsigned long long)(P.iord[nn_idx[e]] + 1);
                x *= 0x9E3779B97F4A7C15ULL;
                x ^= x >> 29;
                x *= 0xBF58476D1CE4E5B9ULL;
                x ^= x >> 32;
                hsh += x;
            }
            nbr_hash[o] = hsh;
        }
    }
    free(v); free(uu); free(fBall2); free(rho); free(divv); free(curl); free(dvds);
    free(bal); free(diffc); free(pr2); free(cs); free(dtp); free(ah); free(updv);
    free(uav); free(dtn); free(mum);
    free(nn_off); free(nn_idx); free(rv_off); free(rv_idx); free(rv_fill);
    free(T.c);
    parts_free(&P);
    return 0;
}

/* ------------------------------------------------------------------ */
/* kick-drift-kick                                                     */
/* ------------------------------------------------------------------ */
void orc_kdk(int n, int which, double dt, int bPeriodic, double dPeriod,
             double *pos, double *vel, const double *acc, int ngas,
             double *u, const double *udot, double *vpred, double *upred) {
    int i, j;
    double h = 0.5 * dt;
    for (i = 0; i < n; ++i) {
        int bGas = i < ngas;
        for (j = 0; j < 3; ++j) {
            if (bGas && vpred) vpred[3 * i + j] = vel[3 * i + j] + acc[3 * i + j] * h;
            vel[3 * i + j] = vel[3 * i + j] + acc[3 * i + j] * h;
        }
        if (bGas && u) {
            if (upred) upred[i] = u[i] + udot[i] * h;
            u[i] = u[i] + udot[i] * h;
            if (upred && upred[i] < 0) upred[i] = 0;
            if (u[i] < 0) u[i] = 0;
        }
        if (which == 0) {
            for (j = 0; j < 3; ++j) {
                pos[3 * i + j] += dt * vel[3 * i + j];
                if (bPeriodic) {
                    if (pos[3 * i + j] >= 0.5 * dPeriod) pos[3 * i + j] -= dPeriod;
                    if (pos[3 * i + j] < -0.5 * dPeriod) pos[3 * i + j] += dPeriod;
                }
            }
        }
    }
}

/* ------------------------------------------------------------------ */
/* FP64 direct summation: the exact force the tree approximates       */
/* ------------------------------------------------------------------ */
/* For each target t = qidx[k]: a = -sum_j m_j b(r, h_t + h_j) (r_t - r_j),
 * pot = -sum_j m_j a(r, h_t + h_j), j != t, with the reference's spline
 * softening SPLINE (grav.h:74-101) as in the intra-bucket sum
 * (grav.c:211-242).  Test infrastructure for the batched systems. */
void orc_direct(int n, const double *pos, const double *mass, const double *soft, int nq,
                const int *qidx, double *acc, double *pot, int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 4)
#endif
    for (int k = 0; k < nq; ++k) {
        int t = qidx[k];
        double ax = 0, ay = 0, az = 0, p = 0;
        for (int j = 0; j < n; ++j) {
            if (j == t) continue;
            double dx = pos[3 * t] - pos[3 * j], dy = pos[3 * t + 1] - pos[3 * j + 1],
                   dz = pos[3 * t + 2] - pos[3 * j + 2];
            double r2 = dx * dx + dy * dy + dz * dz;
            double a, b;
            spline(r2, soft[t] + soft[j], &a, &b);
            p -= mass[j] * a;
            ax -= mass[j] * b * dx;
            ay -= mass[j] * b * dy;
            az -= mass[j] * b * dz;
        }
        acc[3 * k] = ax;
        acc[3 * k + 1] = ay;
        acc[3 * k + 2] = az;
        pot[k] = p;
    }
}

/* Exact periodic accelerations by pairwise Ewald summation (not the
 * reference's method: an independent check of the tree + Ewald result).
 * For targets qidx[k], the force of every other particle j and all its
 * images in a cube of side L: real space sum over images with
 * alpha r < 6, erfc(alpha r)/r^2 + 2 alpha/sqrt(pi) e^-(alpha r)^2 / r
 * radial profile, k space sum over k = 2 pi h / L, 0 < |h| <= hmax, with
 * (4 pi / V) e^(-k^2 / 4 alpha^2) / k^2; the nearest image's Newtonian part
 * is replaced by the reference's spline softening inside 2h (SPLINE,
 * grav.h:74-101).  Test infrastructure for the periodic box. */
void orc_ewald_direct(int n, const double *pos, const double *mass, const double *soft, double L,
                      int nq, const int *qidx, double *acc, int nthreads) {
    const double alpha = 2.0 / L, V = L * L * L;
    const int nr = 4, hmax = 6;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int k = 0; k < nq; ++k) {
        const int t = qidx[k];
        double ax = 0, ay = 0, az = 0;
        for (int j = 0; j < n; ++j) {
            if (j == t) continue;
            double d[3];
            for (int c = 0; c < 3; ++c) {
                double x = pos[3 * t + c] - pos[3 * j + c];
                x -= L * floor(x / L + 0.5);          /* nearest image */
                d[c] = x;
            }
            double fx = 0, fy = 0, fz = 0;
            for (int ix = -nr; ix <= nr; ++ix)
                for (int iy = -nr; iy <= nr; ++iy)
                    for (int iz = -nr; iz <= nr; ++iz) {
                        double rx = d[0] + ix * L, ry = d[1] + iy * L, rz = d[2] + iz * L;
                        double r2 = rx * rx + ry * ry + rz * rz, r = sqrt(r2);
                        if (alpha * r > 6.0) continue;
                        double g = (erfc(alpha * r) + 2.0 * alpha * r / sqrt(M_PI) *
                                    exp(-alpha * alpha * r2)) / (r2 * r);
                        if (ix == 0 && iy == 0 && iz == 0) {
                            double a, b;
                            spline(r2, soft[t] + soft[j], &a, &b);
                            g += b - 1.0 / (r2 * r);        /* softened nearest image */
                        }
                        fx -= g * rx; fy -= g * ry; fz -= g * rz;
                    }
            for (int hx = -hmax; hx <= hmax; ++hx)
                for (int hy = -hmax; hy <= hmax; ++hy)
                    for (int hz = -hmax; hz <= hmax; ++hz) {
                        int h2 = hx * hx + hy * hy + hz * hz;
                        if (h2 == 0 || h2 > hmax * hmax) continue;
                        double kx = 2 * M_PI * hx / L, ky = 2 * M_PI * hy / L, kz = 2 * M_PI * hz / L;
                        double k2 = kx * kx + ky * ky + kz * kz;
                        double c = 4.0 * M_PI / V * exp(-k2 / (4.0 * alpha * alpha)) / k2 *
                                   sin(kx * d[0] + ky * d[1] + kz * d[2]);
                        fx -= c * kx; fy -= c * ky; fz -= c * kz;
                    }
            ax += mass[j] * fx;
            ay += mass[j] * fy;
            az += mass[j] * fz;
        }
        acc[3 * k] = ax;
        acc[3 * k + 1] = ay;
        acc[3 * k + 2] = az;
    }
}
