/*
 * tsph_pkd -- the reference-side binding of libtsph.
 *
 * Compiled together with the reference's own sources (it includes pkd.h,
 * smooth.h and smoothfcn.h, with the same -D flags as the rest of the
 * build, e.g. -DGASOLINE) and linked against libtsph.  Each entry point has
 * the signature of the reference function it stands in for, so a call site
 * changes only its function name:
 *
 *   pstBuildTree  (pst.c:2957)  pkdBuildBinary -> tsph_pkdBuildBinary
 *   pstGravity    (pst.c:3310)  pkdGravAll     -> tsph_pkdGravAll
 *   pstSmooth     (pst.c:3019)  smSmooth       -> tsph_smSmooth
 *   pstReSmooth   (pst.c:3176)  smReSmooth     -> tsph_smReSmooth
 *
 * tsph_pkdBuildBinary still builds the reference's own tree (the rest of the
 * reference reads it: the top tree, the Ewald root moments, domain
 * bookkeeping) and records nBucket and the opening angle dCrit for the GPU,
 * which builds its own exact copy of that tree in tsph_pkdGravAll.  A run in
 * which nothing else reads the reference's local tree can call
 * tsph_pkd_set_tree_params in its place.
 *
 * Per-PKD state (the libtsph context, the tree parameters, the registered
 * particle store) lives in a side table keyed by the PKD pointer; the PKD
 * struct is not changed.  Like the reference's kernels these calls are not
 * re-entrant for one PKD.  Errors abort with a message, as the reference's
 * assert()s do in the same places.
 */
#ifndef TSPH_PKD_H
#define TSPH_PKD_H

#include "pkd.h"
#include "smooth.h"

/* Optional: the device and precision (TSPH_FP32 / TSPH_FP64) for this PKD's
 * evaluations; without it the first call attaches device 0 in FP32. */
void tsph_pkd_attach(PKD pkd, int device, int precision);
/* Release the PKD's context and unregister its particle store. */
void tsph_pkd_detach(PKD pkd);
/* The tree parameters pkdBuildBinary takes (nBucket, the OPEN_JOSH opening
 * angle dCrit) for the next tsph_pkdGravAll. */
void tsph_pkd_set_tree_params(PKD pkd, int nBucket, int iOpenType, double dCrit);

void tsph_pkdBuildBinary(PKD pkd, int nBucket, int iOpenType, double dCrit, int iOrder,
                         int bTreeActiveOnly, int bGravity, KDN *pRoot);
void tsph_pkdGravAll(PKD pkd, int nReps, int bPeriodic, int iOrder, int bEwald, int iEwOrder,
                     double fEwCut, double fEwhCut, int bComove, double dRhoFac, int bDoSun,
                     double dSunSoft, double *aSun, int *nActive, double *pdPartSum,
                     double *pdCellSum, double *pdSoftSum, CASTAT *pcs, double *pdFlop);
void tsph_smSmooth(SMX smx, SMF *smf);
void tsph_smReSmooth(SMX smx, SMF *smf);

#endif
