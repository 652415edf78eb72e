// Host-side context of libtsph: device buffers, stream, error state.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "tsph_internal.cuh"

// Device-side control block of one tree build.
struct TsphBuildCtl {
    int taskCount;    // subtree tasks queued
    int taskNext;     // next task to claim
    int nTop;         // temp nodes made by the level-wise top phase
    int status;       // TSPH_ERR_* bits raised on the device
    int nNodes;       // nodes of the finished forest
    int pad[3];
    int levF[TSPH_MAX_LEVELS + 2];      // top phase: frontier size of each level
    int levStart[TSPH_MAX_LEVELS + 2];  // top phase: first temp id of each level
};

struct TsphBuildBufs {
    int cap;          // particle capacity
    int topCap;       // temp ids [0, topCap): roots and top-phase nodes
    int tcap;         // topCap + 2*cap: task slots follow, 2 per particle
    int *seg;         // temp id of the frontier node of each particle (-1 = done)
    int *lt;          // r[d] < fSplit flag
    int *scan;        // inclusive scan of lt
    int *scanTmp;     // block sums for the scan
    int *f_node[2];   // top-phase frontier (temp ids), double-buffered
    int *f_split, *f_rank;
    int *tasks;       // subtree task roots (temp ids)
    int *chunkScan;   // top phase: inclusive scan of the frontier nodes' chunk counts
    int *ctot, *coff; // top phase: flags per chunk and their inclusive scan
    int *chunkNode;   // top phase: frontier index of each chunk
    // temporary nodes: roots, then the top phase breadth first, then the
    // subtree slots of every task (a task over particles [lo, hi] owns
    // slots topCap + 2*lo ... topCap + 2*hi + 1)
    int *t_lo, *t_hi, *t_dim, *t_child, *t_size, *t_pre, *t_root, *t_loc;
    double *t_split;
    double *t_bnd;    // 6 per node; holds order-preserving keys while bounds accumulate
    unsigned long long *maxd2;   // per final node: max squared distance to COM
    int *visit;                  // per final node: children finished (bottom-up moments)
    int nodeScratchCap;
    int *leafFlag, *leafScan;
    TsphBuildCtl *ctl;           // device
    int *hostCount;              // pinned
    int topLevels;               // top-phase levels of the last build
};

// SPH arrays, in gas-tree order (G.iord maps to the caller index)
struct TsphSphBufs {
    int cap;
    double *vx, *vy, *vz, *u;    // vPred, uPred gathered from the state
    float4 *vh, *vl;             // vPred split into FP32 hi and lo parts (FP32 passes)
    double *fBall2, *rho, *divv, *curl, *dvds, *bal, *diff, *pr2, *cs, *dtp;
    double *hax, *hay, *haz, *uPdV, *uAV, *dtNew, *mumax;
    double *seed;                // optional fBall2 seed per particle (learned h)
    int *nnCount;
    unsigned long long *nnHash;
    unsigned long long *nodeBall2;   // per gas-tree node: max fBall2 (bits)
    // neighbour lists of the last density pass: N(i) = {j : d2 <= fBall2_i}
    // in ascending gas-tree index (nbrCap per particle), and the reverse
    // lists R(i) = {j : i in N(j)}, also ascending
    int nbrCap;
    int *nbrList;
    int *rcnt, *roff, *rcur, *rlist;
    int *listFlag;               // device: [0] = a list did not fit (use the tree walk)
    double *ph, *ih2, *fn1, *pr2f;   // per-particle kernel invariants of the pressure pass
    float4 *pfa, *pfb, *pfc;         // FP32 copies: (ph, ih2, fn1, pr2f), (c, rho, bal, dtp), (pr2)
    int nFallback;
    bool haveDensity, havePressure, haveSeed;
    tsph_sph_params last;
    // passes over active rungs: which gas particles this pass computed
    // (need, tree order), the active ones and the rest as index lists,
    // their counts (device, [0] active, [1] rest), per-particle bound on
    // the squared ball radius since their last density (rb2)
    int *need, *list, *list2, *listN;
    double *rb2;
    bool subset;
    int nComputed;
};

// Learned smoothing-length network (3 -> 32 -> 32 -> 1, tanh, FP32).
#define HNET_H 32
#define HNET_NP (HNET_H * 3 + HNET_H + HNET_H * HNET_H + HNET_H + HNET_H + 1)
struct TsphHnet {
    float *W;            // parameters, layout W1[32x3] b1[32] W2[32x32] b2[32] W3[32] b3
    float *grad;         // full gradient
    float *m1, *m2;      // Adam moments
    float *partial;      // per-warp partial gradients
    float *loss;         // per-warp partial losses
    float *feat;         // features of the current density pass (gas-tree order), 3 per particle
    long long featCap;   // particles feat holds
    float *samples;      // training samples: 4 floats (x0,x1,x2,target) each
    long long nSamples, capSamples;
    float stats[8];      // mean/std of the three features and the target
    bool init, statsReady, trained, collect, predict, havePrev;
    double margin;       // log-radius safety margin of the seed
    long long adamStep;
};

struct tsph_ctx {
    int device;
    cudaStream_t stream;
    bool ownStream;
    int smCount;
    char cudaErr[256];
    long long launches;

    int n, ngas;
    int cap;
    TsphDevState C;              // caller order
    TsphDevParts P;              // gravity tree order
    TsphDevTree T;               // gravity tree
    TsphDevParts G;              // gas tree order
    TsphDevTree TG;              // gas tree
    TsphBuildBufs B;
    TsphSphBufs S;
    TsphDevCounters *dCnt;       // device counters
    TsphDevCounters *hCnt;       // pinned mirror
    int *dBucketLists;           // 4 ints per bucket
    int bucketListCap;

    // Ewald
    double *dRoot;               // 35 doubles: root complete moments
    void *dEw;                   // the Ewald constants, built on the device (EwConst)
    cudaEvent_t evGather;        // the gather's status and coordinate scale are on the host
    cudaStream_t side;           // work beside the moments: FP32 particle records, bucket
                                 // geometry, Ewald constants
    cudaEvent_t evBuilt, evParts, evMoments, evPrep, evEwald;   // its branches and merges
    bool bucketPrepQueued;       // the walk's bucket geometry is queued on the side stream
    int nEwt;                    // k-space vectors kept (a function of fEwhCut only)

    // input staging (caller order)
    double *dStage;
    size_t stageBytes;

    // Tipsy snapshot I/O: two chunks of pinned host and device staging, and
    // the per-particle fields a snapshot carries that the path does not use
    // (caller order; valid after tsph_read_tipsy until the next load)
    void *hPin;
    unsigned int *dSnapRaw;
    size_t snapChunkBytes;
    float *snapRho, *snapMetals, *snapTform;
    int snapCap;
    bool snapValid;
    int snapNStar;               // star count of the last snapshot read

    // adaptive timesteps: force passes act on particles with rung >= actRung
    // (the reference's TYPE_ACTIVE after msrActiveRung(actRung, 1))
    int actRung;
    unsigned int *dSnapStatus;
    cudaEvent_t snapEv[2];

    bool haveParts, haveVel, haveTree, haveGrav;
    tsph_grav_params lastGrav;
    double dPeriodTree;
    double coordScale;           // largest |coordinate| of the particles (or a captured bound)

    TsphHnet hnet;

    unsigned long long *dAux;    // device scratch: [0] gas max |coordinate| bits, [1] capture
                                 // extent, [2..] the rung statistics of the multistep driver
    double *hTmp;                // host staging of tsph_get_sph
    size_t hTmpN;
    double gasScale;             // last measured gas max |coordinate|
    // systems (forest): caller-order system id of every particle
    int nSys;
    int *hSys;

    // tree build tuning and mode
    int taskSize;                // largest node one CTA builds whole (0 = automatic)
    int subtreeBlocks[4];        // resident CTAs of the subtree kernel ...
    size_t subtreeSmem[4];       // ... for each dynamic shared memory size seen
    bool subtreeAttr;            // its shared-memory limit raised
    int walkBlocksPerSM;         // resident walk blocks per SM (0 = default)
    int walkGroup;               // particles per walk group (0 = default, -1 = off)
    int walkLists;               // two-pass walk (1 or a slot size: on; 0, -1: off)
    double *dKeep;               // accelerations kept across a step capture's preparation
    size_t keepCap;
    int *dWalkListPP;            // the list pass's P-P particles, walkListSlot per bucket
    int *dWalkListCell;          // its Newtonian cells, walkListSlot per bucket
    int *dWalkListSoft;          // its softened cells, walkListSlot / 4 per bucket
    int4 *dWalkListInfo;         // list lengths per bucket (w = -1: left to a fused walk)
    int *dWalkListFallback;      // the buckets left to a fused walk
    long long walkListBuckets;   // buckets the arrays hold
    size_t walkListEntries;      // entries dWalkListPP and dWalkListCell hold
    int walkListSlot;            // entries per bucket
    long long lastListNeed;      // longest list a bucket of the last evaluation did not fit
    int *dGroupFlag, *dGroupScan;  // per bucket: starts a group, and the inclusive scan
    int *dGroupFirst;            // first bucket of every group, then the bucket count
    int *dGroupCount;            // device: number of groups
    int groupCap;                // buckets the group arrays hold
    int *dGroupScratch;          // per walk warp: the lists its group walk leaves
    int groupScratchWarps;
    bool capturing;              // inside a CUDA graph capture: no host reads
    double capLimit;             // |coordinate| bound of the captured step (0 = none)
    unsigned int *dStepStatus;   // device: status bits accumulated over a step
    // captured kick-drift-kick step (tsph_step)
    cudaGraphExec_t graphExec;
    double *dStepDt;             // the step's dt, read by a captured step's kicks and drifts
    const double *stepDtDev;     // dStepDt while a step is captured, else null
    tsph_grav_params graphGrav;
    tsph_sph_params graphSph;
    int graphN, graphNgas, graphHasSph;
    long long graphKernels;      // kernel launches recorded in the graph
    long long graphSysVersion;
    long long sysVersion;        // bumped by every particle / system change
    // the reference-layout particle store (store.cu)
    unsigned long long storeKey; // store, n and order of the last tsph_store_load
    char *dStore;                // device copy of an unregistered store
    size_t storeCap;
    int *dStoreOrder;            // store entry of every caller index

    cudaEvent_t ev[10];
    float timings[8];
};

// error helpers -----------------------------------------------------------
int tsph_cuda_fail(tsph_ctx *ctx, cudaError_t e, const char *where);
#define TSPH_CK(call)                                                  \
    do {                                                               \
        cudaError_t e_ = (call);                                       \
        if (e_ != cudaSuccess) return tsph_cuda_fail(ctx, e_, #call);  \
    } while (0)
#define TSPH_LAUNCH_CK(where)                                          \
    do {                                                               \
        ctx->launches++;                                               \
        cudaError_t e_ = cudaGetLastError();                           \
        if (e_ != cudaSuccess) return tsph_cuda_fail(ctx, e_, where);  \
    } while (0)

template <typename T>
static int tsph_grow(tsph_ctx *ctx, T **p, size_t count) {
    if (*p) cudaFree(*p);
    *p = nullptr;
    cudaError_t e = cudaMalloc((void **)p, sizeof(T) * (count > 0 ? count : 1));
    if (e != cudaSuccess) { *p = nullptr; return tsph_cuda_fail(ctx, e, "cudaMalloc"); }
    return TSPH_OK;
}

static inline int tsph_blocks(long long n, int bs) {
    long long b = (n + bs - 1) / bs;
    return (int)(b > 0 ? b : 1);
}

// internal entry points implemented across the .cu files
int tsph_scan_inclusive(tsph_ctx *ctx, const int *in, int *out, int n);
int tsph_build_tree(tsph_ctx *ctx, TsphDevParts &P, TsphDevTree &T, int n, int nBucket);
int tsph_set_ranges(tsph_ctx *ctx, TsphDevParts &P, TsphDevTree &T, int n, int nR, const int *counts);
int tsph_tree_moments(tsph_ctx *ctx, TsphDevParts &P, TsphDevTree &T, int n, double dTheta,
                      int order, int fp32);
void tsph_free_build(TsphBuildBufs &B);
int tsph_apply_gas_systems(tsph_ctx *ctx);
int tsph_load_begin(tsph_ctx *ctx, int n);
int tsph_kick_launch(tsph_ctx *ctx, int iRung, double dt, int bClose);
int tsph_drift_launch(tsph_ctx *ctx, double dt, int bPeriodic, double dPeriod);
int tsph_load_gas(tsph_ctx *ctx, int ngas);
int tsph_load_state_from_stage(tsph_ctx *ctx, int n);
void tsph_free_snapshot(tsph_ctx *ctx);
int tsph_fold_status(tsph_ctx *ctx);
int tsph_copy_out(tsph_ctx *ctx, const double *a0, const double *a1, const double *a2, int comp,
                  double *host);
int tsph_copy_out_n(tsph_ctx *ctx, int n, const double *a0, const double *a1, const double *a2,
                    int comp, double *host);
void tsph_free_tree(TsphDevTree &T);
int tsph_walk_interact(tsph_ctx *ctx, const tsph_grav_params *gp);
int tsph_bucket_prep(tsph_ctx *ctx, cudaStream_t s);
int tsph_walk_finish_f32(tsph_ctx *ctx);
int tsph_ewald_roots(tsph_ctx *ctx, const tsph_grav_params *gp, cudaStream_t s);
int tsph_ewald(tsph_ctx *ctx, const tsph_grav_params *gp);
int tsph_ensure_particles(tsph_ctx *ctx, int n);
int tsph_sph_density(tsph_ctx *ctx, const tsph_sph_params *sp, tsph_smooth_out *out);
// h-network hooks used by the density pass (mlp.cu)
int tsph_hnet_features(tsph_ctx *ctx, int k);
int tsph_hnet_seed(tsph_ctx *ctx);
int tsph_hnet_append(tsph_ctx *ctx);
void tsph_hnet_free(tsph_ctx *ctx);
int tsph_sph_pressure(tsph_ctx *ctx, const tsph_sph_params *sp, tsph_smooth_out *out);
