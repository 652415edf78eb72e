/*
 * libtsph -- GB300-native TreeSPH force path behind a C ABI.
 *
 * The entry points replace the per-rank kernels of the reference (gasoline)
 * that its processor-set tree calls on every rank:
 *   tsph_grav_all   <- pkdGravAll           (pkd.h:797-801, pkd.c:2868-3060)
 *                      with the tree build it needs, pkdBuildBinary
 *                      (pkd.c:2627-2723), pkdCalcRoot/pkdDistribRoot
 *                      (pkd.c:4395-4493) and pkdEwaldInit (ewald.c:182-248)
 *   tsph_smooth     <- smInitialize + smSmooth / smReSmooth + smFinish
 *                      (smooth.h:616-638, smooth.c:54-542,1439-1749) for the
 *                      smooth types SMX_DENDVDX and SMX_SPHPRESSURETERMS
 *                      (smoothfcn.h:147-199), with pkdGasPressure
 *                      (pkd.c:5750-5785) run between the two
 *   tsph_kick/drift <- pkdKick (pkd.c:3780-3969), pkdDrift (pkd.c:3686-3778)
 *
 * Arguments are plain pointers and sizes.  Arrays are in the caller's
 * particle order (the reference's iOrder); positions, velocities and
 * accelerations are interleaved xyz (3 doubles per particle), like the
 * r[3]/v[3]/a[3] members of the reference's PARTICLE (pkd.h:90-225).
 * Gas particles are the first ngas particles.
 *
 * Every call returns TSPH_OK (0) or a positive TSPH_ERR_* code; device-side
 * failures (list overflow, kNN not converging, non-finite input) come back
 * as codes rather than traps, and the context stays usable.  The reference
 * aborts through assert() in the same situations.
 *
 * A context owns one GPU's device buffers and a CUDA stream; it is not
 * thread-safe (like the reference's PKD, one context per host thread).
 */
#ifndef TSPH_H
#define TSPH_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct tsph_ctx tsph_ctx;

enum tsph_status {
    TSPH_OK = 0,
    TSPH_ERR_ARG = 1,             /* bad argument (NULL, n < 0, ...) */
    TSPH_ERR_CUDA = 2,            /* CUDA runtime error; see tsph_last_cuda_error */
    TSPH_ERR_STACK_OVERFLOW = 3,  /* walk stack exceeded its capacity */
    TSPH_ERR_LIST_OVERFLOW = 4,   /* neighbour list exceeded its capacity */
    TSPH_ERR_KNN_NO_CONVERGE = 5, /* kNN radius search hit its iteration cap */
    TSPH_ERR_NONFINITE = 6,       /* NaN or Inf in the particle data */
    TSPH_ERR_UNSUPPORTED = 7,     /* smooth type or option not implemented */
    TSPH_ERR_STATE = 8,           /* call order (e.g. no particles loaded) */
    TSPH_ERR_TREE_DEPTH = 9,      /* tree deeper than the build's level cap */
    TSPH_ERR_NOMEM = 10,          /* device allocation failed */
    TSPH_ERR_BOUNDS = 11,         /* a particle left the coordinate bound a
                                     captured step graph was built for */
    TSPH_ERR_IO = 12              /* snapshot file: cannot be opened, is
                                     short, or its header or masses are
                                     inconsistent */
};

enum tsph_precision {
    TSPH_FP64 = 0,   /* all pairwise and multipole arithmetic in FP64 */
    TSPH_FP32 = 1    /* FP32 on bucket-relative offsets, compensated sums */
};

/* Smooth types, numbered as the reference's enum smx_smoothtype
 * (smoothfcn.h:147-199). */
enum tsph_smx {
    TSPH_SMX_DENSITY = 1,
    TSPH_SMX_SPHPRESSURETERMS = 22,
    TSPH_SMX_DENDVDX = 23
};

/*
 * Gravity parameters: the arguments of pkdGravAll (nReps, bPeriodic,
 * iOrder, bEwald, iEwOrder, fEwCut, fEwhCut; pkd.h:797) plus those of the
 * tree build it depends on (nBucket, dTheta with OPEN_JOSH opening,
 * master.c:1897-1934; the period fPeriod of pkdInitialize) and the
 * arithmetic precision.  Comoving and Sun-indirect terms (bComove,
 * bDoSun) are not part of this path.
 */
#define TSPH_MAX_BUCKET 32   /* largest nBucket: one warp walks one bucket */

typedef struct {
    int nBucket;      /* max particles per leaf, 1..TSPH_MAX_BUCKET (reference
                         default 8; larger returns TSPH_ERR_UNSUPPORTED) */
    int iOrder;       /* cell multipole order, 1..4: 2 = quadrupole, 3 octopole,
                         4 hexadecapole (the reference's default) */
    int bPeriodic;
    int bEwald;
    int iEwOrder;     /* Ewald multipole order, 1..4 */
    int nReps;        /* periodic replicas per side (1 when periodic) */
    double dTheta;    /* opening angle */
    double dPeriod;   /* box length L (cube) */
    double fEwCut;    /* real-space cut in units of L (2.6) */
    double fEwhCut;   /* k-space cut (2.8) */
    int precision;    /* enum tsph_precision */
    int reserved;
} tsph_grav_params;

/* pkdGravAll's out-parameters (nActive, pdPartSum, pdCellSum, pdSoftSum,
 * pdFlop), same definitions (pkd.c:2946-2962, grav.c:246-247,
 * ewald.c:175-176), plus the fraction of opening tests settled in FP64
 * and the number of opening tests the walk made. */
typedef struct {
    int nActive;
    int nBuckets;
    double dPartSum;
    double dCellSum;
    double dSoftSum;
    double dFlop;
    double dFlopEwald;
    double dExactFrac;
    double dTests;       /* opening tests of cells with >= 4 particles */
    double dVisits;      /* (cell, replica) entries examined by the walk */
} tsph_grav_out;

/* SPH parameters: the SMF fields the two passes read (smoothfcn.h:22-130,
 * filled by msrSmoothFcnParam master.c:5548-5669) for a non-comoving run
 * (a = 1, H = 0), adiabatic gas without cooling. */
typedef struct {
    int nSmooth;
    int bPeriodic;
    double dPeriod;
    double alpha;         /* dConstAlpha */
    double beta;          /* dConstBeta */
    double gamma;         /* dConstGamma */
    double dEtaCourant;   /* dtFacCourant = dEtaCourant*2/1.6 (pkd.c:5893) */
    int iViscosityLimiter;/* 0 none, 1 Balsara (reference default) */
    int precision;        /* enum tsph_precision for the gathers */
    int bLearnedH;        /* seed the kNN with the h-network's prediction */
    int reserved;
} tsph_sph_params;

typedef struct {
    int nSmoothed;        /* SMF.nSmoothed */
    int nFallback;        /* ball radii grown because a ball held < nSmooth */
    double dPairs;        /* neighbour pairs gathered */
    double dCandidates;   /* particles inside the gathered balls (kNN cost) */
    int bSeeded;          /* 1 when the learned-h prediction seeded the balls */
    int reserved;
} tsph_smooth_out;

/* --- context --------------------------------------------------------- */

/* Create a context on `device`.  `stream` is a cudaStream_t to run on, or
 * NULL for a stream the context creates and owns. */
int tsph_create(tsph_ctx **pctx, int device, void *stream);
void tsph_destroy(tsph_ctx *ctx);
const char *tsph_error_string(int status);
/* The last CUDA error message seen by this context ("" if none). */
const char *tsph_last_cuda_error(tsph_ctx *ctx);

/* Load particles (host arrays, caller order): pos[3n], mass[n], soft[n]
 * (spline softening length, the reference's fSoft).  Replaces the previous
 * set.  Device memory grows as needed and is kept between calls. */
int tsph_set_particles(tsph_ctx *ctx, int n, const double *pos,
                       const double *mass, const double *soft);
/* New positions, masses and softenings for the n particles already
 * loaded (same caller indices).  Everything else stays, including the
 * particle order the last tree build left, as the reference's particle
 * store keeps its order between steps; the next build starts from it.
 * With a different n it is tsph_set_particles. */
int tsph_update_particles(tsph_ctx *ctx, int n, const double *pos,
                          const double *mass, const double *soft);
/* Velocities vel[3n] (all particles) and, for the first ngas particles,
 * specific thermal energy u[ngas] (the reference's u; uPred = u, vPred = v
 * at load).  ngas may be 0. */
int tsph_set_velocities(tsph_ctx *ctx, const double *vel, int ngas,
                        const double *u);

/* Independent systems in one context (a forest of trees).  sysOf[i] in
 * [0, nSys) is the system of caller particle i (call after
 * tsph_set_particles, and after tsph_set_velocities when there is gas; a
 * later tsph_set_velocities keeps the assignment, tsph_set_particles
 * clears it).  Every system gets its own gravity tree and, for its gas,
 * its own gas tree: forces and SPH neighbours never cross systems, and
 * each system's tree, lists and forces equal those of that system loaded
 * alone.  Non-periodic only (periodic calls return TSPH_ERR_UNSUPPORTED
 * when nSys > 1).  This is the batched form of one pkdGravAll per system;
 * the reference runs such systems as separate jobs. */
int tsph_set_systems(tsph_ctx *ctx, int nSys, const int *sysOf);

/* --- the reference's particle store ----------------------------------------
 * The reference keeps its particles in one array of PARTICLE structs
 * (pkd.h:90-225, pkd->pStore) and its kernels read and write their fields
 * in place.  These calls do the same from the store's layout: its stride
 * and the byte offsets of the fields, as offsetof(PARTICLE, ...) gives them
 * in code compiled against the reference's pkd.h (gasoline_gb300/pkd/
 * tsph_pkd.c does so).  Doubles on 8-byte boundaries; an offset < 0 marks a
 * field the store does not have.  Caller particle i is store entry order[i]
 * (order NULL: entry i); order must name each of the entries 0..n-1 once,
 * and the first ngas of that order are the gas.
 * A store registered with tsph_store_register (pinned and mapped) is read
 * and written in place by the GPU, field by field; otherwise the load
 * copies the n entries to the device in one block and the results are
 * written back by the host. */
typedef struct {
    long long stride;          /* bytes per entry: sizeof(PARTICLE) */
    /* inputs (doubles): positions r[3], fMass, fSoft, and for gas loads
     * v[3], vPred[3], u, uPred (a store without vPred/uPred predicts them
     * as v/u, as tsph_set_velocities does) */
    int r, fMass, fSoft, v, vPred, u, uPred;
    /* gravity outputs: a[3] +=, fPot +=, dtGrav = max (pkdGravAll) */
    int a, fPot, dtGrav;
    /* density-pass outputs (set): fBall2, fDensity, divv, curlv[3], dvds,
     * BalsaraSwitch, diff (DenDVDX) */
    int fBall2, fDensity, divv, curlv, dvds, BalsaraSwitch, diff;
    /* pressure-pass outputs: PoverRho2, c, uDotPdV, uDotAV, mumax (set),
     * a[3] += hydro acceleration, dtNew = min (pkdGasPressure +
     * SphPressureTermsSym) */
    int PoverRho2, c, uDotPdV, uDotAV, mumax, dtNew;
    /* unsigned int activity word; entries with (word & activeBit) set are
     * active (the reference's iActive & TYPE_ACTIVE); < 0: all active */
    int iActive;
    unsigned int activeBit;
    int reserved[6];
} tsph_store_layout;

/* Pin and map `bytes` of host memory holding a store (cudaHostRegister)
 * so the GPU reads and writes it in place; once per store, before the
 * loads.  tsph_store_unregister undoes it. */
int tsph_store_register(tsph_ctx *ctx, void *store, size_t bytes);
int tsph_store_unregister(tsph_ctx *ctx, void *store);
/* Load n particles from the store: positions, masses, softenings, and when
 * layout->v >= 0 velocities and the first ngas particles' gas fields;
 * active particles (activity word) are the ones the force passes act on.
 * A load of the same store with the same n and ngas as the last one is an
 * update of the same particles (caller index i names the same particle,
 * wherever order puts it in the store now) and keeps the particle order of
 * the last tree, as tsph_update_particles does; any other is a new particle
 * set, as tsph_set_particles + tsph_set_velocities make it. */
int tsph_store_load(tsph_ctx *ctx, int n, const void *store,
                    const tsph_store_layout *layout, const int *order, int ngas);
/* The last tsph_grav_all's results into the store, as pkdGravAll leaves
 * them (active particles: a[3] += acc, fPot += pot, dtGrav = max). */
int tsph_store_put_gravity(tsph_ctx *ctx, void *store, const tsph_store_layout *layout,
                           const int *order);
/* The last tsph_smooth pass's results into the store's gas entries: which
 * = TSPH_SMX_DENDVDX (or TSPH_SMX_DENSITY) writes the density-pass fields,
 * TSPH_SMX_SPHPRESSURETERMS the pressure-pass fields of the active gas. */
int tsph_store_put_sph(tsph_ctx *ctx, int which, void *store, const tsph_store_layout *layout,
                       const int *order);

/* --- gravity (pkdGravAll) -------------------------------------------- */

/* Build the gravity tree over the loaded particles and compute every
 * particle's acceleration, potential and dtGrav (the reference's
 * 1/dt^2 estimate), overwriting them (the reference accumulates into
 * a[] after msrInitAccel zeroes it).  Results stay on the device. */
int tsph_grav_all(tsph_ctx *ctx, const tsph_grav_params *gp,
                  tsph_grav_out *out);
/* Copy gravity results to the host in caller order; NULL skips a field. */
int tsph_get_gravity(tsph_ctx *ctx, double *acc, double *pot, double *dtGrav);

/* Tree export for parity checks, in the reference's node order.  Writes
 * inode[6*i] = pLower, pUpper, iDim, iLower, iUpper (threaded), 0 and
 * dnode[16*i] = fSplit, bnd.fMin[3], bnd.fMax[3], fMass, fSoft, r[3],
 * fOpen2, Bmax, Qxx, Qyy; perm[pos] = caller index at tree position pos.
 * With inode == NULL only returns the node count in *nNodes. */
int tsph_get_tree(tsph_ctx *ctx, int *nNodes, int *inode, double *dnode,
                  int *perm);
/* Per-bucket interaction-list lengths of the last tsph_grav_all (in
 * depth-first bucket order): blist[4*b] = node, nPart, nCellSoft,
 * nCellNewt.  With blist == NULL returns the bucket count. */
int tsph_get_lists(tsph_ctx *ctx, int *nBuckets, int *blist);

/* --- SPH (smSmooth / smReSmooth) -------------------------------------- */

/* Run one smooth pass over the gas particles:
 *   TSPH_SMX_DENDVDX: exact kNN smoothing lengths (fBall2 = nSmooth-th
 *     smallest squared distance, self included) and the DenDVDX gather;
 *   TSPH_SMX_DENSITY: the same kNN and density (Density,
 *     smoothfcn.c:239-256; the gradient fields come along);
 *   TSPH_SMX_SPHPRESSURETERMS: gas pressure (pkdGasPressure) and the
 *     symmetric pressure / artificial-viscosity terms over every pair with
 *     d^2 <= fBall2 of either particle.
 * Other types return TSPH_ERR_UNSUPPORTED. */
int tsph_smooth(tsph_ctx *ctx, int smx_type, const tsph_sph_params *sp,
                tsph_smooth_out *out);
/* SPH results in caller order for the gas particles: out[16*i] = fBall2,
 * fDensity, divv, curlv[3], dvds, BalsaraSwitch, diff, PoverRho2, c,
 * a_hydro[3], uDotPdV, uDotAV; dtNew[i]; mumax[i]. NULL skips.  Fields of
 * the pressure pass (PoverRho2 .. uDotAV, dtNew, mumax) are zero until it
 * has run. */
int tsph_get_sph(tsph_ctx *ctx, double *out16, double *dtNew, double *mumax);
/* Neighbour-set fingerprint per gas particle: |N(i)| and an
 * order-independent hash of the caller indices in N(i). */
int tsph_get_neighbour_hash(tsph_ctx *ctx, int *count,
                            unsigned long long *hash);

/* --- learned smoothing length (no counterpart in the reference) --------
 * A 3 -> 32 -> 32 -> 1 tanh network (FP32) predicts each gas particle's
 * log(fBall2) from the last pass's fBall2 and divv and the
 * density of the deepest gas-tree cell holding >= nSmooth particles.  With
 * sph.bLearnedH the prediction (widened by `margin` in log radius) seeds the
 * DENDVDX ball gather; balls holding < nSmooth grow and retry, so fBall2
 * and the neighbour sets are those of the exact kNN.  Training runs on the
 * GPU (Adam) over samples collected from earlier passes. */
int tsph_hnet_num_params(void);
int tsph_hnet_init(tsph_ctx *ctx, unsigned long long seed);
int tsph_hnet_set_params(tsph_ctx *ctx, const float *params, int n);
int tsph_hnet_get_params(tsph_ctx *ctx, float *params, int n);
/* 0.5*mean((net(x)-y)^2) and its gradient over given normalised samples
 * x[3n], y[n] (for gradient checks). */
int tsph_hnet_loss_grad(tsph_ctx *ctx, int n, const float *x3, const float *y,
                        float *grad, double *loss);
/* collect: append each DENDVDX pass's (features, target) samples;
 * predict: allow seeding (needs a trained network). */
int tsph_hnet_mode(tsph_ctx *ctx, int collect, int predict, double margin);
/* `steps` Adam steps on random batches of the collected samples; *loss is
 * the final loss over all samples (normalised units). */
int tsph_hnet_train(tsph_ctx *ctx, int steps, int batch, double lr, double *loss);
int tsph_hnet_info(tsph_ctx *ctx, long long *nSamples, float *stats8);

/* Loss and gradient of the h-network without allocating device memory.  No
 * counterpart in the reference.  For callers that cannot allocate where they
 * need the gradient: a host code that reserves all its device memory up
 * front and updates the network inside its step loop, where a cudaMalloc
 * would synchronise the device and stall its other streams, or exceed a
 * fixed memory budget.  Every argument is a device pointer: params[
 * tsph_hnet_num_params()], normalised samples x3[3n] and y[n]; outputs
 * grad[tsph_hnet_num_params()] and loss[1] (0.5*mean((net(x)-y)^2)).  Runs
 * on `stream` (a cudaStream_t, NULL = default) of the current device and
 * returns without synchronising.  Scratch lives in one fixed device array
 * of ~2.5 MB that the library holds on every GPU that loads it until exit;
 * n above TSPH_HNET_NOALLOC_MAX_SAMPLES returns TSPH_ERR_ARG.  Every call
 * looks up that array's address in the calling thread's current context;
 * the first call on a device also loads the library's device code there,
 * so make it before any stream capture.  Calls share the array: calls that
 * overlap on the GPU race and must be serialised by the caller. */
#define TSPH_HNET_NOALLOC_MAX_SAMPLES 16384
int tsph_hnet_loss_grad_noalloc(const float *params, int n, const float *x3,
                                const float *y, float *grad, float *loss,
                                void *stream);

/* --- kick-drift-kick (pkdKick / pkdDrift) ------------------------------ */

/* Every particle: v += a*dt (a = gravity + hydro); gas: vPred = v + a*dt,
 * u += uDot*dt and uPred = u + uDot*dt with uDot = uDotPdV + uDotAV
 * (NOCOOLING, pkd.c:3936-3939) -- the closing kick of a KDK step. */
int tsph_kick(tsph_ctx *ctx, double dt);
/* r += v*dt, wrapped into [-L/2, L/2) when periodic (pkdDrift
 * pkd.c:3726-3756); for gas also vPred += a*dt and uPred += uDot*dt
 * (pkdKickVpred pkd.c:6489-6552), as msrDrift runs them. */
int tsph_drift(tsph_ctx *ctx, double dt, int bPeriodic, double dPeriod);
/* pkdKick (pkd.c:3780-3969) for the particles on rung iRung (all when
 * iRung < 0): v += a*dt and, for gas, u += uDot*dt.  bClose = 0 is the
 * opening kick of a KDK step (vPred, uPred keep the values from before
 * it, msrKickKDKOpen master.c:6540); bClose = 1 the closing kick (vPred,
 * uPred predicted to its end, msrKickKDKClose master.c:6644).
 * tsph_kick(ctx, dt) is tsph_kick_rung(ctx, -1, dt, 1). */
int tsph_kick_rung(tsph_ctx *ctx, int iRung, double dt, int bClose);
/* Copy state to the host in caller order; NULL skips a field. */
int tsph_get_state(tsph_ctx *ctx, double *pos, double *vel, double *u);

/* --- adaptive timesteps (rungs) -----------------------------------------
 * Particle i steps with dDelta / 2^rung[i].  tsph_top_step_kdk advances
 * every particle by one base step dDelta as msrTopStepKDK does
 * (master.c:8242-8465): timestep criteria and new rungs at each level
 * (pkdInitDt, pkdGravStep, pkdAccelStep, pkdSphStep, pkdDtToRung),
 * emergency moves of gas whose dtNew fell below half a step
 * (pkdEmergencyAdjust), opening and closing kicks per rung, drifts of
 * every particle, and force passes over the particles of the kicked rungs
 * (gravity for them on a tree of all particles with each bucket's box
 * shrunk to its active particles, as pkdGravAll does; SPH densities of all
 * gas and pressure forces for the active gas).  Call it after forces on
 * every particle (tsph_grav_all and, with gas, both tsph_smooth passes),
 * which is the reference's start-up.  Defaults are the reference's
 * (master.c:572-623). */
typedef struct {
    int iMaxRung;        /* rungs 0..iMaxRung-1 (1 to 29) */
    double dEta;         /* 0.1: acceleration criteria */
    int bGravStep;       /* 0: dt <= dEta/sqrt(dtGrav) */
    int bEpsAccStep;     /* 1: dt <= dEta*sqrt(eps/|a|), eps = h for gas */
    int bSqrtPhiStep;    /* 0: dt <= 3.5*dEta*sqrt(|phi|)/|a| */
    double dEtauDot;     /* 0.25: gas dt <= dEtauDot*u/|uDotPdV| when cooling adiabatically */
    double duMinDt;      /* 0: floor of u in that criterion */
} tsph_step_params;     /* the Courant factor is tsph_sph_params.dEtaCourant */

typedef struct {
    int iCurrMaxRung;       /* highest rung of any particle after the step */
    int nForcePasses;       /* force evaluations (one per smallest substep) */
    long long nActiveSum;   /* particles that received forces, summed over the passes */
    int nEmergency;         /* emergency rung moves */
} tsph_step_out;

int tsph_top_step_kdk(tsph_ctx *ctx, double dTime, double dDelta,
                      const tsph_grav_params *gp, const tsph_sph_params *sp,
                      const tsph_step_params *st, tsph_step_out *out);
/* Force passes (tsph_grav_all, tsph_smooth) act on the particles with
 * rung >= iRung only (msrActiveRung(iRung, 1)); 0, the default, is all. */
int tsph_set_active_rung(tsph_ctx *ctx, int iRung);
int tsph_set_rungs(tsph_ctx *ctx, const int *rung);
/* rung, the timestep dt, dtNew and mumax of every particle (caller order;
 * NULL skips a field).  dt and dtNew start at FLT_MAX as in the reference's
 * reader. */
int tsph_get_rungs(tsph_ctx *ctx, int *rung, double *dt, double *dtNew, double *mumax);

/* --- Tipsy snapshots (pkdReadTipsy pkd.c:297, pkdWriteTipsy pkd.c:1628) --
 * The reference's particle file (tipsydefs.h:9-45): a 32-byte header, then
 * the gas, dark and star records, 4-byte floats; bStandard = 1 is the XDR
 * (big-endian) form, 0 the host-order form.  Gas comes first in the file,
 * as the library's convention wants. */
typedef struct {
    double time;     /* expansion factor when comoving, else time */
    int nbodies, ndim, nsph, ndark, nstar;
} tsph_tipsy_header;

/* The header of a snapshot (msrReadTipsy's read, master.c:3612-3622). */
int tsph_tipsy_read_header(const char *path, int bStandard, tsph_tipsy_header *h);
/* Load a snapshot into the context, replacing its particles as
 * tsph_set_particles + tsph_set_velocities would: v = dvFac*vel,
 * u = uPred = dTuFac*temp for the nsph gas particles, softening = eps,
 * potential = phi; rho, metals and tform are kept for tsph_write_tipsy.
 * dvFac and dTuFac are the caller's unit factors (master.c:3742-3775).
 * h (may be NULL) receives the header.  TSPH_ERR_IO for a missing, short
 * or inconsistent file, or a mass the reference rejects (standard-form gas
 * mass <= 0, any other mass < 0), and the context then holds no particles. */
int tsph_read_tipsy(tsph_ctx *ctx, const char *path, int bStandard, double dvFac,
                    double dTuFac, tsph_tipsy_header *h);
/* Write the context's particles as a snapshot at `time`: the first ngas are
 * gas, the last nStar stars, the rest dark; vel*dvFac and u*duTFac rounded
 * to float (pkdWriteTipsy with the adiabatic gas model).  rho is the
 * density of the last SPH density pass, else the value read in; metals and
 * tform are those read in (0 for particles loaded by tsph_set_particles);
 * phi is the potential of the last gravity evaluation, else the value read
 * in. */
int tsph_write_tipsy(tsph_ctx *ctx, const char *path, int bStandard, double time,
                     int nStar, double dvFac, double duTFac);
/* Per-particle fields of the loaded set in caller order; NULL skips one:
 * mass, softening and potential (double; the potential read in or of the
 * last gravity evaluation), and the snapshot's rho, metals and tform
 * (float; zeros when the particles did not come from a snapshot). */
int tsph_get_snapshot_fields(tsph_ctx *ctx, double *mass, double *soft, double *pot,
                             float *rho, float *metals, float *tform);
/* Set the fields a snapshot carries beside the particles (caller order;
 * NULL keeps a field): the potential, and rho, metals and tform as stored
 * in the file.  For writing particles loaded with tsph_set_particles. */
int tsph_set_snapshot_fields(tsph_ctx *ctx, const double *pot, const float *rho,
                             const float *metals, const float *tform);

/* --- rendering (dfRenderParticleTSC dumpframe.c:1125-1230) ---------------
 * A frame of the loaded particles splatted with the reference's TSC
 * kernel into a headless RGB float image (the reference's DFIMAGE,
 * row-major, y = 0 the top row).  Sizes: gas from its ball (bGasSph) or
 * softening, dark and stars from their softening, each times its
 * multiplier; colours interpolated in the density from per-type tables
 * (dfColInterp dumpframe.c:1096-1122; star colour by age is not
 * supported: stars use their table).  The gas density is that of the last
 * SPH density pass, else the snapshot's; other particles use 0.  The first
 * ngas particles are gas and the last nStar stars.  xlim, ylim and hmul
 * follow dfSetupFrame (dumpframe.c:259-261). */
typedef struct {
    int nxPix, nyPix;
    double r[3];                 /* centre */
    double x[3], y[3], z[3];     /* projection vectors (pixels per length unit) */
    double zEye, zClipNear, zClipFar;
    int iProject;                /* 1 orthographic, 2 perspective */
    double dGasSoftMul, dDarkSoftMul, dStarSoftMul;
    int bGasSph;
    double dMassGasMin, dMassGasMax, dMassDarkMin, dMassDarkMax, dMassStarMin, dMassStarMax;
    int bColMassWeight, bColLogInterp;
    int nColGas, nColDark, nColStar;         /* table lengths, 0..10 */
    float dColGas[10], dColDark[10], dColStar[10];
    float colGas[10][3], colDark[10][3], colStar[10][3];
} tsph_render_params;

/* rgb receives nxPix*nyPix*3 floats (host memory). */
int tsph_render_tsc(tsph_ctx *ctx, const tsph_render_params *rp, int nStar, float *rgb);

/* --- tuning --------------------------------------------------------------
 * Launch-shape knobs of the CUDA path (no reference counterpart; the
 * reference's equivalents are compile-time constants and nBucket).  None
 * changes the tree or an interaction list.  taskSize and walkBlocksPerSM
 * change no result at all; walkGroup changes the order in which a
 * particle's interactions are summed, so forces move by rounding only.
 * Zero selects the default. */
typedef struct {
    int taskSize;         /* largest tree node one CTA builds whole (>= 1024; default 1536) */
    int walkBlocksPerSM;  /* walk blocks per SM (default 5 for FP32, 4 for FP64) */
    int walkGroup;        /* particles per walk group, 32..4096; -1 = no groups; default
                             128 when there are at least 256 particles per walk warp, else
                             none.  The buckets of a group (the largest subtree with at
                             most this many particles) share one walk for the cells that
                             every bucket of it opens or accepts, and each bucket walks
                             only the rest */
    int walkLists;        /* 1: the walk in two passes -- a list pass stores every bucket's
                             interaction list (the tree walk alone, at high occupancy), then
                             the evaluation pass reads them; 32..65536: the same with that
                             many list entries per bucket (default 1024, grown when buckets
                             overflow; a bucket that overflows is walked by the evaluation
                             pass); -1 and the default: one fused pass.  Walk groups take
                             precedence.  Same lists, same order: results are
                             bit-identical either way */
    int reserved[4];
} tsph_tuning;
int tsph_set_tuning(tsph_ctx *ctx, const tsph_tuning *t);
int tsph_get_tuning(tsph_ctx *ctx, tsph_tuning *t);

/* --- whole steps ----------------------------------------------------------
 * One kick-drift-kick step of the single-rung msrTopStepKDK
 * (master.c:8242-8465): kick dt/2, drift dt, gravity (+ for gas the density
 * pass, gas pressure and the pressure pass), kick dt/2.  sp may be NULL
 * (gravity only).  Returns when the work is queued on the context stream.
 * With TSPH_STEP_GRAPH the step's launches are captured once into a CUDA
 * graph (recaptured when the parameters or the particle set change; the
 * graph reads dt from device memory, so a new dt replays the same graph)
 * and each call replays it with one launch.  Graph mode takes isolated and
 * periodic (Ewald) systems and a density pass seeded by the h-network; it
 * returns TSPH_ERR_UNSUPPORTED while the h-network collects samples.  The
 * capture evaluates the forces once outside the graph and keeps the
 * accelerations the step's opening kick reads, so graph steps equal direct
 * ones bit for bit.  No reference counterpart for the graph: the reference
 * drives the same sequence from its host loop.
 * dt may be any finite value, negative included (the leapfrog is
 * time-reversible: a step of -dt undoes one of dt up to rounding).
 * tsph_step_status waits for the queued steps and returns the first error
 * any of them raised (TSPH_OK if none); TSPH_ERR_BOUNDS means a particle
 * moved beyond twice the extent the graph was captured for, and the next
 * tsph_step recaptures. */
#define TSPH_STEP_GRAPH 1
int tsph_step(tsph_ctx *ctx, double dt, const tsph_grav_params *gp,
              const tsph_sph_params *sp, int flags);
int tsph_step_status(tsph_ctx *ctx);

/* Timing of the last call's kernels on the context stream (ms), by phase:
 * t[0] tree build, t[1] moments, t[2] walk+interactions, t[3] Ewald,
 * t[4] kNN, t[5] density, t[6] pressure, t[7] total. */
int tsph_get_timings(tsph_ctx *ctx, float *t8);
/* Number of libtsph kernel launches issued since context creation. */
long long tsph_launch_count(tsph_ctx *ctx);
/* Measured FMA throughput of this GPU in TFLOP/s (precision FP32 or FP64),
 * the denominator of the force kernels' roofline fraction. */
int tsph_fma_peak(tsph_ctx *ctx, int precision, double *tflops);

#ifdef __cplusplus
}
#endif
#endif
