// Internal device-side data layout and helpers for libtsph.
//
// Particles live in HBM as structure-of-arrays in *tree order* (the order the
// reference's pkdBuildBinary leaves pStore in, pkd.c:2627-2723), with the
// caller's index kept in `iord`.  Tree nodes are stored in the reference's
// own depth-first numbering (BuildBinary allocates a node, then its lower
// subtree, then its upper subtree: pkd.c:2452-2453), so node i's lower child
// is i+1 and the node after its subtree is i + size(i).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/tsph.h"

#define TSPH_WARP 32
#define TSPH_MAX_LEVELS 128
#define TSPH_NBR_CAP 64      // stored neighbours per gas particle (ties beyond: tree-walk pressure)
#define TSPH_RCAP 1024       // longest reverse list sorted in shared memory

// FP64 helpers that never contract into FMA: the reference's tree and walk
// decisions are reproduced bit for bit, so every rounding step must match
// the C source's separate multiply and add.
__device__ __forceinline__ double xmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double xadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double xsub(double a, double b) { return __dsub_rn(a, b); }

// Monotone 64-bit key of a double: key order == numeric order (no NaN).
__device__ __forceinline__ unsigned long long dkey(double x) {
    unsigned long long b = (unsigned long long)__double_as_longlong(x);
    return (b & 0x8000000000000000ULL) ? ~b : (b | 0x8000000000000000ULL);
}
// A key that orders finite doubles as < does, -0 equal to +0: a partition
// test r < fSplit in integer instructions (GB300 issues FP64 compares at
// the FP64 rate, 1/64 of FP32).
__device__ __forceinline__ unsigned long long dlt_key(double x) {
    unsigned long long b = (unsigned long long)__double_as_longlong(x);
    if (b == 0x8000000000000000ULL) b = 0ULL;
    return (b & 0x8000000000000000ULL) ? ~b : (b | 0x8000000000000000ULL);
}
__device__ __forceinline__ double dunkey(unsigned long long k) {
    unsigned long long b = (k & 0x8000000000000000ULL) ? (k & 0x7FFFFFFFFFFFFFFFULL) : ~k;
    return __longlong_as_double((long long)b);
}

// Largest |x|, |y|, |z| over n particles, as the bits of a non-negative
// double (which order like the values) max-reduced into *out.
__device__ __forceinline__ void warp_max_abs(double a, unsigned long long *out) {
    unsigned long long key = (unsigned long long)__double_as_longlong(a);
    unsigned hiw = (unsigned)(key >> 32), low = (unsigned)key;
    unsigned mh = __reduce_max_sync(0xffffffffu, hiw);
    unsigned ml = __reduce_max_sync(0xffffffffu, hiw == mh ? low : 0u);
    if ((threadIdx.x & 31) == 0) atomicMax(out, ((unsigned long long)mh << 32) | ml);
}

// Split a double into float hi + float lo with hi + lo == x to ~2^-48.
__host__ __device__ __forceinline__ void split2f(double x, float &hi, float &lo) {
    hi = (float)x;
    lo = (float)(x - (double)hi);
}

struct TsphDevTree {
    int nNodes;
    int nLeaves;
    int cap;          // allocated node capacity
    // node arrays, depth-first (reference) order
    int *pLower, *pUpper, *iDim;
    int *upper;       // upper child index, -1 for a leaf
    int2 *dlink;      // (upper child, its first particle): one load a level of a descent
    int *skip;        // node after this subtree, -1 at the end (threaded "next")
    double *fSplit;
    double *bnd;      // 6 per node: min xyz, max xyz
    double *fMass, *fSoft;
    double *r;        // 3 per node, centre of mass
    double *fOpen2, *Bmax;
    double *Q;        // 6 per node: xx yy zz xy xz yz (complete, about the COM)
    // walk copies in FP32
    float4 *wcomh;    // com hi xyz + fOpen2 (float)
    float4 *wcoml;    // com lo xyz + fSoft (float)
    int4 *wlink;      // pLower, count, upper (-1 leaf), 0
    float4 *wmom0;    // m, Qxx, Qyy, Qzz
    float4 *wmom1;    // Qxy, Qxz, Qyz, fSoft
    // octopole and hexadecapole cells (iOrder >= 3; sized on first use)
    double *M3, *M4;  // complete 3rd (10) and 4th (15) moments about the COM
    double *OH;       // reduced octopole (10) + hexadecapole (15) per node,
                      // pkdCalcCell's O* and H* in its field order
    float *wOH;       // FP32 copies of OH, 25 per node
    int highCap;      // nodes M3/M4/OH/wOH hold
    int *leaves;      // leaf node ids in depth-first order (the buckets)
    int *parent;      // parent node, -1 at a root
    // forest of independent trees over contiguous particle ranges (one
    // range = one system; a single system is a forest of one)
    int nR;           // trees
    int maxRange;     // particles in the largest tree (host)
    int *rLo, *rHi;   // device: particle range of each tree
    int *hLo, *hHi;   // host copies
    int *sysRoot;     // device: root node of each tree
    int *rEnd;        // device: one past the last node of each tree
    int *dcnt;        // device: nNodes, nLeaves
    int rCap;
    int lastTopLevels; // top-phase levels of the last host-paced build
    float4 *brec;     // per bucket: centre hi + soft max, centre lo + extent
                      // (negative: no active particle), box min - centre
                      // (+ active count), box max - centre (FP32)
    double *bact;     // per bucket: bounds of its active particles, min xyz,
                      // max xyz (pkdGravAll's bndActive, pkd.c:2917-2935)
};

struct TsphDevParts {
    int n;
    int ngas;
    double *x, *y, *z, *m, *h;   // tree order
    int *iord;                   // caller index of each tree-order slot
    int *rid;                    // tree (range) of each tree-order slot
    int *act;                    // 1 if the slot's particle is active (rung >= the active rung)
    float4 *ph;                  // hi xyz + mass (float)
    float4 *pl;                  // lo xyz + soft (float)
    // outputs in tree order
    double *ax, *ay, *az, *pot, *dtGrav;
    // FP32 walk results as compensated pairs (sum, negated low part) of
    // (ax, ay, az, pot), combined in FP64 with the Ewald term
    float4 *wsum, *wcmp;
    float *wdt;
};

// Particle state in the caller's order (the reference's iOrder): what the
// kick/drift update and the host see.  The gravity tree and the gas tree
// each keep their own tree-ordered copies (TsphDevParts) mapped back by iord.
struct TsphDevState {
    double *x, *y, *z, *vx, *vy, *vz, *m, *h, *u;
    double *vpx, *vpy, *vpz, *upred;     // predicted (time-centred) v and u
    double *ax, *ay, *az, *pot, *dtGrav; // gravity
    double *hax, *hay, *haz, *udot;      // SPH (gas only): hydro accel, uDotPdV+uDotAV
    double *fb2prev, *divvprev;          // last density pass: fBall2, divv (h-network inputs)
    // adaptive timesteps: the reference's p->iRung, p->dt, p->dtNew, p->mumax
    // and p->uDotPdV, kept across passes (an inactive particle keeps its own)
    int *rung;
    double *dt, *dtNew, *mumax, *updv;
    double *cs;                          // gas sound speed of the last pressure pass (p->c)
    double *disp;                        // gas: bound on the distance drifted since the last
                                         // density pass over all gas
};

// Counters accumulated by the walk (integers: deterministic).
struct TsphDevCounters {
    unsigned long long nActive;
    unsigned long long nPartPP;      // sum over buckets of n * nPart
    unsigned long long nIntra;       // sum over buckets of n*(n-1)/2
    unsigned long long nBucketSq;    // sum over buckets of n*n
    unsigned long long nCellNewt;    // sum of n * nCellNewt
    unsigned long long nCellSoft;    // sum of n * nCellSoft
    unsigned long long nEwLoop;      // Ewald real-space terms evaluated
    unsigned long long nExactTests;  // opening tests settled in FP64
    unsigned long long nTests;       // opening tests in total
    unsigned long long nVisits;      // (cell, replica) entries the walk examined
    unsigned long long maxAbs;       // bits of max |coordinate| (non-negative double)
    unsigned int status;             // TSPH_ERR_* raised on device
    unsigned int pad;                // work counter of the walk's evaluation pass
    unsigned int listWork;           // work counter of the walk's list pass
    unsigned int evalWork;           // work counter of its evaluation pass
    unsigned int nListFallback;      // buckets the list pass left to a fused walk
    unsigned int listNeed;           // longest list of such a bucket (slot entries)
};
