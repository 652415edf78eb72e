/*
 * CPU oracle for the TreeSPH force path: a plain-C restatement of the
 * reference's algorithm (gasoline pkd.c / walk.c / grav.c / ewald.c /
 * v_sqrt1.c / smooth.c / smoothfcn.c / SphPressureTerms.h).
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py call it, as the checker; the product path
 * (libtsph) never links or calls it.
 *
 * All arrays are SoA, indexed by the caller's particle order (iOrder).
 */
#ifndef TSPH_ORACLE_H
#define TSPH_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

/* Same field order as the reference harness's parameter block. */
typedef struct {
    int nBucket;
    int iOrder;     /* multipole order of cell interactions (1..4) */
    int bPeriodic;
    int bEwald;
    int iEwOrder;
    int nReps;
    double dTheta;
    double dPeriod;
    double fEwCut;
    double fEwhCut;
} orc_grav_params;

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
} orc_sph_params;

/* Full gravity evaluation (pkdBuildBinary + pkdGravAll).  counters[5] =
 * nActive, dPartSum, dCellSum, dSoftSum, dFlop.  nthreads <= 1: serial. */
int orc_grav(int n, const double *pos, const double *mass, const double *soft,
             const orc_grav_params *gp, double *acc, double *pot,
             double *dtGrav, double *counters, int nthreads);

/* Tree export, same layout as the reference harness's ref_tree. */
int orc_tree(int n, const double *pos, const double *mass, const double *soft,
             const orc_grav_params *gp, int *inode, double *dnode, int *perm);

/* Per-bucket list lengths, same layout as ref_lists. */
int orc_lists(int n, const double *pos, const double *mass, const double *soft,
              const orc_grav_params *gp, int *blist);

/* SPH: kNN smoothing lengths, DenDVDX, gas pressure, symmetric pressure
 * terms.  out[16*i..] as in ref_sph.  nbr_count[i] = |N(i)| (ball gather
 * with fBall2); nbr_hash[i] = order-independent hash of N(i)'s iOrders. */
int orc_sph(int n, const double *pos, const double *vel, const double *mass,
            const double *soft, const double *u, const orc_sph_params *sp,
            double *out, double *dtNew, double *mumax, int *nbr_count,
            unsigned long long *nbr_hash, int nthreads);

/* Exact kNN only: fBall2[i] = nSmooth-th smallest d^2 (self included). */
int orc_knn(int n, const double *pos, int nSmooth, int bPeriodic,
            double dPeriod, double *fBall2, int nthreads);

/* Kick-drift-kick update of one step for all-active particles, in the
 * reference's single-rung order (master.c:8242-8465, NOCOOLING):
 *   kick(dt/2): v += a dt/2, gas u += uDot dt/2 (uPred/vPred predicted),
 *   drift(dt): r += v dt (periodic wrap into [-L/2, L/2)).
 * which = 0: opening kick + drift; which = 1: closing kick only. */
void orc_kdk(int n, int which, double dt, int bPeriodic, double dPeriod,
             double *pos, double *vel, const double *acc, int ngas,
             double *u, const double *udot, double *vpred, double *upred);

/* Use 1.0/sqrt(r2) in place of v_sqrt1 for the interaction 1/r (off by
 * default, which restates the reference exactly). */
void orc_set_exact_rsqrt(int on);

/* v_sqrt1 restated (reference v_sqrt1.c:11-113). */
void orc_v_sqrt1(int n, const double *r2, double *a);

/* FP64 direct sum with the reference's SPLINE softening (grav.h:74-101)
 * for the targets qidx[0..nq) over all n particles: acc[3 nq], pot[nq]. */
void orc_direct(int n, const double *pos, const double *mass, const double *soft, int nq,
                const int *qidx, double *acc, double *pot, int nthreads);

/* Exact periodic accelerations (pairwise Ewald sum, box side L) of the
 * targets qidx[0..nq): an independent check of tree + Ewald. */
void orc_ewald_direct(int n, const double *pos, const double *mass, const double *soft, double L,
                      int nq, const int *qidx, double *acc, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
