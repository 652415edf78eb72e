// C ABI of libtsph: context management, host<->device transfer in the
// caller's particle order, and the pkdGravAll-equivalent driver.
#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "tsph_ctx.cuh"

int tsph_cuda_fail(tsph_ctx *ctx, cudaError_t e, const char *where) {
    if (ctx) snprintf(ctx->cudaErr, sizeof(ctx->cudaErr), "%s: %s", where, cudaGetErrorString(e));
    if (e == cudaErrorMemoryAllocation) return TSPH_ERR_NOMEM;
    return TSPH_ERR_CUDA;
}

extern "C" const char *tsph_error_string(int s) {
    switch (s) {
    case TSPH_OK: return "ok";
    case TSPH_ERR_ARG: return "invalid argument";
    case TSPH_ERR_CUDA: return "CUDA runtime error";
    case TSPH_ERR_STACK_OVERFLOW: return "tree-walk stack overflow";
    case TSPH_ERR_LIST_OVERFLOW: return "neighbour list overflow";
    case TSPH_ERR_KNN_NO_CONVERGE: return "kNN search did not converge";
    case TSPH_ERR_NONFINITE: return "non-finite particle data";
    case TSPH_ERR_UNSUPPORTED: return "unsupported option or smooth type";
    case TSPH_ERR_STATE: return "call out of order";
    case TSPH_ERR_TREE_DEPTH: return "tree deeper than the level cap";
    case TSPH_ERR_NOMEM: return "device allocation failed";
    case TSPH_ERR_BOUNDS: return "particle outside the captured coordinate bound";
    case TSPH_ERR_IO: return "snapshot file missing, short or inconsistent";
    default: return "unknown status";
    }
}

extern "C" const char *tsph_last_cuda_error(tsph_ctx *ctx) { return ctx ? ctx->cudaErr : ""; }

extern "C" int tsph_create(tsph_ctx **pctx, int device, void *stream) {
    if (!pctx) return TSPH_ERR_ARG;
    *pctx = nullptr;
    tsph_ctx *ctx = (tsph_ctx *)calloc(1, sizeof(tsph_ctx));
    if (!ctx) return TSPH_ERR_NOMEM;
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) { int rc = tsph_cuda_fail(ctx, e, "cudaSetDevice"); free(ctx); return rc; }
    if (stream) {
        ctx->stream = (cudaStream_t)stream;
        ctx->ownStream = false;
    } else {
        e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) { int rc = tsph_cuda_fail(ctx, e, "cudaStreamCreate"); free(ctx); return rc; }
        ctx->ownStream = true;
    }
    cudaDeviceGetAttribute(&ctx->smCount, cudaDevAttrMultiProcessorCount, device);
    if (cudaMalloc((void **)&ctx->dCnt, sizeof(TsphDevCounters)) != cudaSuccess ||
        cudaMallocHost((void **)&ctx->hCnt, sizeof(TsphDevCounters)) != cudaSuccess ||
        cudaMallocHost((void **)&ctx->B.hostCount, sizeof(int) * (TSPH_MAX_LEVELS + 16)) != cudaSuccess ||
        cudaMalloc((void **)&ctx->dRoot, sizeof(double) * (64 + 256 * 32)) != cudaSuccess ||
        cudaMalloc((void **)&ctx->dAux, sizeof(unsigned long long) * 64) != cudaSuccess ||
        cudaMalloc((void **)&ctx->dStepStatus, sizeof(unsigned int)) != cudaSuccess ||
        cudaMemset(ctx->dStepStatus, 0, sizeof(unsigned int)) != cudaSuccess) {
        tsph_destroy(ctx);
        return TSPH_ERR_NOMEM;
    }
    for (int k = 0; k < 10; ++k) cudaEventCreate(&ctx->ev[k]);
    if (cudaEventCreateWithFlags(&ctx->evGather, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->evBuilt, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->evParts, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->evMoments, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->evPrep, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->evEwald, cudaEventDisableTiming) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking) != cudaSuccess) {
        tsph_destroy(ctx);
        return TSPH_ERR_NOMEM;
    }
    *pctx = ctx;
    return TSPH_OK;
}

#define FREE(p) do { if (p) cudaFree(p); (p) = nullptr; } while (0)

extern "C" void tsph_destroy(tsph_ctx *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->side) cudaStreamSynchronize(ctx->side);
    TsphDevState &C = ctx->C;
    FREE(C.x); FREE(C.y); FREE(C.z); FREE(C.vx); FREE(C.vy); FREE(C.vz); FREE(C.m); FREE(C.h);
    FREE(C.u); FREE(C.vpx); FREE(C.vpy); FREE(C.vpz); FREE(C.upred); FREE(C.ax); FREE(C.ay);
    FREE(C.az); FREE(C.pot); FREE(C.dtGrav); FREE(C.hax); FREE(C.hay); FREE(C.haz); FREE(C.udot);
    FREE(C.fb2prev); FREE(C.divvprev);
    FREE(C.rung); FREE(C.dt); FREE(C.dtNew); FREE(C.mumax); FREE(C.updv); FREE(C.cs);
    FREE(C.disp);
    tsph_hnet_free(ctx);
    TsphDevParts *PP[2] = {&ctx->P, &ctx->G};
    for (int k = 0; k < 2; ++k) {
        TsphDevParts &P = *PP[k];
        FREE(P.x); FREE(P.y); FREE(P.z); FREE(P.m); FREE(P.h); FREE(P.iord); FREE(P.rid);
        FREE(P.act);
        FREE(P.ph); FREE(P.pl); FREE(P.ax); FREE(P.ay); FREE(P.az); FREE(P.pot); FREE(P.dtGrav);
        FREE(P.wsum); FREE(P.wcmp); FREE(P.wdt);
    }
    tsph_free_tree(ctx->T);
    tsph_free_tree(ctx->TG);
    TsphBuildBufs &B = ctx->B;
    FREE(B.seg); FREE(B.lt); FREE(B.scan); FREE(B.scanTmp);
    tsph_free_build(B);
    TsphSphBufs &S = ctx->S;
    FREE(S.vx); FREE(S.vy); FREE(S.vz); FREE(S.u); FREE(S.fBall2); FREE(S.rho); FREE(S.divv);
    FREE(S.curl); FREE(S.dvds); FREE(S.bal); FREE(S.diff); FREE(S.pr2); FREE(S.cs); FREE(S.dtp);
    FREE(S.hax); FREE(S.hay); FREE(S.haz); FREE(S.uPdV); FREE(S.uAV); FREE(S.dtNew); FREE(S.mumax);
    FREE(S.seed); FREE(S.nnCount); FREE(S.nnHash); FREE(S.nodeBall2);
    FREE(S.nbrList); FREE(S.rcnt); FREE(S.roff); FREE(S.rcur); FREE(S.rlist); FREE(S.listFlag);
    FREE(S.ph); FREE(S.ih2); FREE(S.fn1); FREE(S.pr2f); FREE(S.pfa); FREE(S.pfb); FREE(S.pfc);
    FREE(S.need); FREE(S.list); FREE(S.list2); FREE(S.listN); FREE(S.rb2); FREE(S.vh); FREE(S.vl);
    FREE(ctx->dCnt); FREE(ctx->dBucketLists); FREE(ctx->dRoot); FREE(ctx->dEw); FREE(ctx->dStage);
    FREE(ctx->dAux); FREE(ctx->dStepStatus);
    FREE(ctx->dGroupFlag); FREE(ctx->dGroupScan); FREE(ctx->dGroupFirst); FREE(ctx->dGroupCount);
    FREE(ctx->dGroupScratch);
    FREE(ctx->dStore); FREE(ctx->dStoreOrder);
    FREE(ctx->dWalkListPP); FREE(ctx->dWalkListCell); FREE(ctx->dWalkListSoft);
    FREE(ctx->dWalkListInfo); FREE(ctx->dWalkListFallback); FREE(ctx->dKeep);
    FREE(ctx->dStepDt);
    tsph_free_snapshot(ctx);
    free(ctx->hSys);
    free(ctx->hTmp);
    if (ctx->graphExec) cudaGraphExecDestroy(ctx->graphExec);
    if (ctx->hCnt) cudaFreeHost(ctx->hCnt);
    if (ctx->B.hostCount) cudaFreeHost(ctx->B.hostCount);
    for (int k = 0; k < 10; ++k) if (ctx->ev[k]) cudaEventDestroy(ctx->ev[k]);
    if (ctx->evGather) cudaEventDestroy(ctx->evGather);
    cudaEvent_t *evs[5] = {&ctx->evBuilt, &ctx->evParts, &ctx->evMoments, &ctx->evPrep, &ctx->evEwald};
    for (cudaEvent_t *e : evs) if (*e) cudaEventDestroy(*e);
    if (ctx->side) cudaStreamDestroy(ctx->side);
    if (ctx->ownStream && ctx->stream) cudaStreamDestroy(ctx->stream);
    free(ctx);
}

int tsph_ensure_particles(tsph_ctx *ctx, int n) {
    if (n <= ctx->cap && ctx->P.x) return TSPH_OK;
    int cap = n + n / 8 + 1024;
    int rc = 0;
    TsphDevParts &P = ctx->P;
    rc |= tsph_grow(ctx, &P.x, cap); rc |= tsph_grow(ctx, &P.y, cap); rc |= tsph_grow(ctx, &P.z, cap);
    rc |= tsph_grow(ctx, &P.m, cap); rc |= tsph_grow(ctx, &P.h, cap); rc |= tsph_grow(ctx, &P.iord, cap);
    rc |= tsph_grow(ctx, &P.ph, cap); rc |= tsph_grow(ctx, &P.pl, cap);
    rc |= tsph_grow(ctx, &P.ax, cap); rc |= tsph_grow(ctx, &P.ay, cap); rc |= tsph_grow(ctx, &P.az, cap);
    rc |= tsph_grow(ctx, &P.pot, cap); rc |= tsph_grow(ctx, &P.dtGrav, cap);
    rc |= tsph_grow(ctx, &P.wsum, cap); rc |= tsph_grow(ctx, &P.wcmp, cap);
    rc |= tsph_grow(ctx, &P.wdt, cap);
    TsphDevParts &G = ctx->G;
    rc |= tsph_grow(ctx, &G.x, cap); rc |= tsph_grow(ctx, &G.y, cap); rc |= tsph_grow(ctx, &G.z, cap);
    rc |= tsph_grow(ctx, &G.m, cap); rc |= tsph_grow(ctx, &G.h, cap); rc |= tsph_grow(ctx, &G.iord, cap);
    rc |= tsph_grow(ctx, &G.ph, cap); rc |= tsph_grow(ctx, &G.pl, cap);
    TsphDevState &C = ctx->C;
    double **cs[] = {&C.x, &C.y, &C.z, &C.vx, &C.vy, &C.vz, &C.m, &C.h, &C.u, &C.vpx, &C.vpy,
                     &C.vpz, &C.upred, &C.ax, &C.ay, &C.az, &C.pot, &C.dtGrav, &C.hax, &C.hay,
                     &C.haz, &C.udot, &C.fb2prev, &C.divvprev, &C.dt, &C.dtNew, &C.mumax,
                     &C.updv, &C.cs, &C.disp};
    for (auto pp : cs) rc |= tsph_grow(ctx, pp, cap);
    rc |= tsph_grow(ctx, &C.rung, cap);
    rc |= tsph_grow(ctx, &P.act, cap);
    rc |= tsph_grow(ctx, &G.act, cap);
    TsphSphBufs &S = ctx->S;
    double **ss[] = {&S.vx, &S.vy, &S.vz, &S.u, &S.fBall2, &S.rho, &S.divv, &S.dvds, &S.bal,
                     &S.diff, &S.pr2, &S.cs, &S.dtp, &S.hax, &S.hay, &S.haz, &S.uPdV, &S.uAV,
                     &S.dtNew, &S.mumax, &S.seed};
    for (auto pp : ss) rc |= tsph_grow(ctx, pp, cap);
    rc |= tsph_grow(ctx, &S.curl, (size_t)3 * cap);
    rc |= tsph_grow(ctx, &S.nnCount, cap);
    rc |= tsph_grow(ctx, &S.nnHash, cap);
    rc |= tsph_grow(ctx, &S.nodeBall2, (size_t)2 * cap + 64);
    S.nbrCap = TSPH_NBR_CAP;
    rc |= tsph_grow(ctx, &S.nbrList, (size_t)S.nbrCap * cap);
    rc |= tsph_grow(ctx, &S.rlist, (size_t)S.nbrCap * cap);
    rc |= tsph_grow(ctx, &S.rcnt, cap); rc |= tsph_grow(ctx, &S.roff, cap);
    rc |= tsph_grow(ctx, &S.rcur, cap); rc |= tsph_grow(ctx, &S.listFlag, 4);
    rc |= tsph_grow(ctx, &S.ph, cap); rc |= tsph_grow(ctx, &S.ih2, cap);
    rc |= tsph_grow(ctx, &S.fn1, cap); rc |= tsph_grow(ctx, &S.pr2f, cap);
    rc |= tsph_grow(ctx, &S.pfa, cap); rc |= tsph_grow(ctx, &S.pfb, cap); rc |= tsph_grow(ctx, &S.pfc, cap);
    rc |= tsph_grow(ctx, &S.vh, cap); rc |= tsph_grow(ctx, &S.vl, cap);
    rc |= tsph_grow(ctx, &S.need, cap); rc |= tsph_grow(ctx, &S.list, cap);
    rc |= tsph_grow(ctx, &S.list2, cap); rc |= tsph_grow(ctx, &S.listN, 4);
    rc |= tsph_grow(ctx, &S.rb2, cap);
    S.cap = cap;
    TsphBuildBufs &B = ctx->B;
    rc |= tsph_grow(ctx, &B.seg, cap); rc |= tsph_grow(ctx, &B.lt, cap); rc |= tsph_grow(ctx, &B.scan, cap);
    rc |= tsph_grow(ctx, &B.scanTmp, cap / 1024 + 4096);
    rc |= tsph_grow(ctx, &P.rid, cap);
    rc |= tsph_grow(ctx, &G.rid, cap);
    rc |= tsph_grow(ctx, &ctx->dStage, (size_t)3 * cap);
    if (rc) return TSPH_ERR_NOMEM;
    B.cap = cap;
    ctx->cap = cap;
    return TSPH_OK;
}

__global__ void k_load_state(int n, const double *__restrict__ pos3, TsphDevState C, int *piord,
                             int *giord) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    C.x[i] = pos3[3 * i];
    C.y[i] = pos3[3 * i + 1];
    C.z[i] = pos3[3 * i + 2];
    C.vx[i] = C.vy[i] = C.vz[i] = 0.0;
    C.vpx[i] = C.vpy[i] = C.vpz[i] = 0.0;
    C.u[i] = C.upred[i] = C.udot[i] = 0.0;
    C.hax[i] = C.hay[i] = C.haz[i] = 0.0;
    C.ax[i] = C.ay[i] = C.az[i] = C.pot[i] = C.dtGrav[i] = 0.0;
    C.fb2prev[i] = C.divvprev[i] = 0.0;
    // timestep state as the reference's reader leaves it (pkd.c:318-331)
    C.rung[i] = 0;
    C.dt[i] = C.dtNew[i] = FLT_MAX;
    C.mumax[i] = C.updv[i] = C.cs[i] = C.disp[i] = 0.0;
    piord[i] = i;
    giord[i] = i;
}

// The caller-order state gathered into the last tree order (the reference
// keeps pStore in tree order between steps), checked on the way: non-finite
// input, the coordinate scale of the walk's rounding bound, and (for a
// captured step) particles beyond the bound the graph was built for.
__global__ void k_gather_tree(int n, TsphDevState C, TsphDevParts P, TsphDevCounters *cnt,
                              double limit) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double a = 0.0;
    if (i < n) {
        int o = P.iord[i];
        const double x = C.x[o], y = C.y[o], z = C.z[o];   // masses and softenings after the build
        P.x[i] = x;
        P.y[i] = y;
        P.z[i] = z;
        // the checks on the bits of |x|, |y|, |z| (they order like the
        // values): integer instructions, not the FP64 pipe
        const unsigned long long M = 0x7FFFFFFFFFFFFFFFULL;
        unsigned long long b = (unsigned long long)__double_as_longlong(x) & M;
        const unsigned long long by = (unsigned long long)__double_as_longlong(y) & M;
        const unsigned long long bz = (unsigned long long)__double_as_longlong(z) & M;
        b = b > by ? b : by;
        b = b > bz ? b : bz;
        if (b >= 0x7FF0000000000000ULL) atomicOr(&cnt->status, 1u << TSPH_ERR_NONFINITE);
        else if (b > (unsigned long long)__double_as_longlong(limit))
            atomicOr(&cnt->status, 1u << TSPH_ERR_BOUNDS);
        a = __longlong_as_double((long long)b);
    }
    warp_max_abs(a, &cnt->maxAbs);
}

// gravity results of the active particles; the others keep theirs
// (pkdInitAccel zeroes only active particles, pkd.c:5443-5456)
__global__ void k_scatter_grav(int n, TsphDevParts P, TsphDevState C) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !P.act[i]) return;
    int o = P.iord[i];
    C.ax[o] = P.ax[i];
    C.ay[o] = P.ay[i];
    C.az[o] = P.az[i];
    C.pot[o] = P.pot[i];
    C.dtGrav[o] = P.dtGrav[i];
}

// A new particle set of n: buffers, one system, every derived state stale.
// The caller then fills the caller-order state on the stream.
int tsph_load_begin(tsph_ctx *ctx, int n) {
    if (n < 0 || n >= (1 << 27)) return TSPH_ERR_ARG;   // 27-bit particle indices in the walk entries
    int rc = tsph_ensure_particles(ctx, n > 0 ? n : 1);
    if (rc) return rc;
    ctx->n = n;
    ctx->ngas = 0;
    ctx->haveParts = ctx->haveTree = ctx->haveGrav = ctx->haveVel = false;
    ctx->S.haveDensity = false;
    ctx->snapValid = false;
    ctx->P.n = n;
    ctx->G.n = 0;
    ctx->sysVersion++;
    ctx->nSys = 1;
    ctx->T.lastTopLevels = ctx->TG.lastTopLevels = 0;   // a new particle set: no depth known
    if (n == 0) return TSPH_OK;
    return tsph_set_ranges(ctx, ctx->P, ctx->T, n, 1, &n);
}

// The caller-order state of a new particle set from interleaved positions
// already in the staging buffer (k_load_state); masses, softenings and the
// rest are the caller's to fill.
int tsph_load_state_from_stage(tsph_ctx *ctx, int n) {
    if (n <= 0) return TSPH_OK;
    k_load_state<<<tsph_blocks(n, 256), 256, 0, ctx->stream>>>(n, ctx->dStage, ctx->C, ctx->P.iord,
                                                               ctx->G.iord);
    TSPH_LAUNCH_CK("k_load_state");
    return TSPH_OK;
}

extern "C" int tsph_set_particles(tsph_ctx *ctx, int n, const double *pos, const double *mass,
                                  const double *soft) {
    if (!ctx || n < 0 || (n > 0 && (!pos || !mass || !soft))) return TSPH_ERR_ARG;
    cudaSetDevice(ctx->device);
    int rc = tsph_load_begin(ctx, n);
    if (rc) return rc;
    if (n == 0) { ctx->haveParts = true; return TSPH_OK; }
    TSPH_CK(cudaMemcpyAsync(ctx->dStage, pos, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
    k_load_state<<<tsph_blocks(n, 256), 256, 0, ctx->stream>>>(n, ctx->dStage, ctx->C, ctx->P.iord,
                                                               ctx->G.iord);
    TSPH_LAUNCH_CK("k_load_state");
    TSPH_CK(cudaMemcpyAsync(ctx->C.m, mass, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    TSPH_CK(cudaMemcpyAsync(ctx->C.h, soft, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    // the caller may reuse its (possibly pinned) buffers once this returns
    TSPH_CK(cudaStreamSynchronize(ctx->stream));
    ctx->haveParts = true;
    return TSPH_OK;
}

__global__ void k_update_pos(int n, const double *__restrict__ pos3, TsphDevState C) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    C.x[i] = pos3[3 * i];
    C.y[i] = pos3[3 * i + 1];
    C.z[i] = pos3[3 * i + 2];
}

// New positions, masses and softenings of the particles already loaded
// (same count, same caller indices): everything else, including the
// particle order the last tree left, is kept, as the reference's particle
// store keeps its order from one step to the next.
extern "C" int tsph_update_particles(tsph_ctx *ctx, int n, const double *pos, const double *mass,
                                     const double *soft) {
    if (!ctx || n < 0 || (n > 0 && (!pos || !mass || !soft))) return TSPH_ERR_ARG;
    if (!ctx->haveParts || n != ctx->n) return tsph_set_particles(ctx, n, pos, mass, soft);
    if (ctx->capturing) return TSPH_ERR_STATE;
    cudaSetDevice(ctx->device);
    ctx->haveTree = ctx->haveGrav = false;
    ctx->S.haveDensity = ctx->S.havePressure = false;
    ctx->sysVersion++;
    if (n == 0) return TSPH_OK;
    TSPH_CK(cudaMemcpyAsync(ctx->dStage, pos, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
    k_update_pos<<<tsph_blocks(n, 256), 256, 0, ctx->stream>>>(n, ctx->dStage, ctx->C);
    TSPH_LAUNCH_CK("k_update_pos");
    TSPH_CK(cudaMemcpyAsync(ctx->C.m, mass, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    TSPH_CK(cudaMemcpyAsync(ctx->C.h, soft, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    TSPH_CK(cudaStreamSynchronize(ctx->stream));   // host buffers reusable on return
    return TSPH_OK;
}

// Tree order grouped by system: a stable counting sort of the caller
// indices [0, n) by sys[], the sizes of the non-empty systems in order.
static int order_by_system(const int *sys, int n, int nSys, int *order, int *counts, int *nR) {
    int *start = (int *)calloc((size_t)nSys + 1, sizeof(int));
    if (!start) return TSPH_ERR_NOMEM;
    for (int i = 0; i < n; ++i) start[sys[i] + 1]++;
    int r = 0;
    for (int s = 0; s < nSys; ++s) {
        if (start[s + 1] > 0) counts[r++] = start[s + 1];
        start[s + 1] += start[s];
    }
    for (int i = 0; i < n; ++i) order[start[sys[i]]++] = i;
    free(start);
    *nR = r;
    return TSPH_OK;
}

static int apply_systems_one(tsph_ctx *ctx, TsphDevParts &P, TsphDevTree &T, int n) {
    if (n == 0) return TSPH_OK;
    int *order = (int *)malloc(sizeof(int) * (size_t)n);
    int *counts = (int *)malloc(sizeof(int) * (size_t)(ctx->nSys > n ? n : ctx->nSys));
    if (!order || !counts) { free(order); free(counts); return TSPH_ERR_NOMEM; }
    int nR = 0;
    int rc = order_by_system(ctx->hSys, n, ctx->nSys, order, counts, &nR);
    if (!rc) {
        cudaError_t e = cudaMemcpy(P.iord, order, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice);
        rc = e == cudaSuccess ? tsph_set_ranges(ctx, P, T, n, nR, counts) : tsph_cuda_fail(ctx, e, "iord");
    }
    free(order);
    free(counts);
    return rc;
}

// Gas tree order grouped by system (the gas particles are the first ngas).
int tsph_apply_gas_systems(tsph_ctx *ctx) {
    if (ctx->nSys <= 1 || !ctx->hSys) {
        int ng = ctx->ngas;
        return ng > 0 ? tsph_set_ranges(ctx, ctx->G, ctx->TG, ng, 1, &ng) : TSPH_OK;
    }
    return apply_systems_one(ctx, ctx->G, ctx->TG, ctx->ngas);
}

extern "C" int tsph_set_systems(tsph_ctx *ctx, int nSys, const int *sysOf) {
    if (!ctx || nSys < 1) return TSPH_ERR_ARG;
    if (!ctx->haveParts) return TSPH_ERR_STATE;
    const int n = ctx->n;
    if (n > 0 && !sysOf) return TSPH_ERR_ARG;
    for (int i = 0; i < n; ++i)
        if (sysOf[i] < 0 || sysOf[i] >= nSys) return TSPH_ERR_ARG;
    cudaSetDevice(ctx->device);
    TSPH_CK(cudaStreamSynchronize(ctx->stream));
    free(ctx->hSys);
    ctx->hSys = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    if (!ctx->hSys) return TSPH_ERR_NOMEM;
    if (n > 0) memcpy(ctx->hSys, sysOf, sizeof(int) * (size_t)n);
    ctx->nSys = nSys;
    int rc = apply_systems_one(ctx, ctx->P, ctx->T, n);
    if (rc) return rc;
    rc = tsph_apply_gas_systems(ctx);
    if (rc) return rc;
    ctx->haveTree = ctx->haveGrav = false;
    ctx->S.haveDensity = ctx->S.havePressure = false;
    ctx->sysVersion++;
    return TSPH_OK;
}

__global__ void k_fold_status(const TsphDevCounters *cnt, unsigned int *acc) {
    if (threadIdx.x == 0 && cnt->status) atomicOr(acc, cnt->status);
}

// Keep a pass's device status bits in the step's status word before the
// next pass clears the counters.
int tsph_fold_status(tsph_ctx *ctx) {
    k_fold_status<<<1, 32, 0, ctx->stream>>>(ctx->dCnt, ctx->dStepStatus);
    TSPH_LAUNCH_CK("k_fold_status");
    return TSPH_OK;
}

static int read_status(tsph_ctx *ctx) {
    TSPH_CK(cudaMemcpyAsync(ctx->hCnt, ctx->dCnt, sizeof(TsphDevCounters), cudaMemcpyDeviceToHost,
                            ctx->stream));
    TSPH_CK(cudaStreamSynchronize(ctx->stream));
    unsigned st = ctx->hCnt->status;
    if (st) {
        for (int k = 1; k < 32; ++k)
            if (st & (1u << k)) return k;
    }
    return TSPH_OK;
}

extern "C" int tsph_grav_all(tsph_ctx *ctx, const tsph_grav_params *gp, tsph_grav_out *out) {
    if (!ctx || !gp) return TSPH_ERR_ARG;
    if (!ctx->haveParts) return TSPH_ERR_STATE;
    if (gp->nBucket < 1 || gp->dTheta <= 0 || gp->iOrder < 1 || gp->iOrder > 4) return TSPH_ERR_ARG;
    // one warp walks one bucket, a lane per (particle, entry slot): at most 32 particles
    if (gp->nBucket > TSPH_MAX_BUCKET) return TSPH_ERR_UNSUPPORTED;
    if (gp->bPeriodic && !(gp->dPeriod > 0)) return TSPH_ERR_ARG;
    if (gp->bPeriodic && ctx->T.nR > 1) return TSPH_ERR_UNSUPPORTED;   // isolated systems only
    if (gp->precision != TSPH_FP32 && gp->precision != TSPH_FP64) return TSPH_ERR_ARG;
    cudaSetDevice(ctx->device);
    const int n = ctx->n;
    // Inside a graph capture (tsph_step) nothing here may wait for the
    // device: no status reads, no timing events, scales fixed beforehand.
    const bool cap = ctx->capturing;
    // a direct call re-uploads constants a captured step relies on
    if (!cap) ctx->sysVersion++;
    TSPH_CK(cudaMemsetAsync(ctx->dCnt, 0, sizeof(TsphDevCounters), ctx->stream));
    if (!cap) cudaEventRecord(ctx->ev[0], ctx->stream);
    if (n > 0) {
        k_gather_tree<<<tsph_blocks(n, 256), 256, 0, ctx->stream>>>(
            n, ctx->C, ctx->P, ctx->dCnt, ctx->capLimit > 0 ? ctx->capLimit : INFINITY);
        TSPH_LAUNCH_CK("k_gather_tree");
    }
    // The gather's status and largest |coordinate| reach the host behind an
    // event and are read once the tree build is queued: nothing in the
    // build needs them (the moments' rounding floor and the walk's
    // constants do), so the stream does not drain here.
    if (!cap) {
        TSPH_CK(cudaMemcpyAsync(ctx->hCnt, ctx->dCnt, sizeof(TsphDevCounters), cudaMemcpyDeviceToHost,
                                ctx->stream));
        TSPH_CK(cudaEventRecord(ctx->evGather, ctx->stream));
    }
    ctx->dPeriodTree = gp->bPeriodic ? gp->dPeriod : 0.0;
    int rc = tsph_build_tree(ctx, ctx->P, ctx->T, n, gp->nBucket);
    if (!cap) {
        TSPH_CK(cudaEventSynchronize(ctx->evGather));
        const unsigned st = ctx->hCnt->status;   // bad input reported before a build error
        for (int k = 1; k < 32 && st; ++k)
            if (st & (1u << k)) return k;
    }
    if (rc) return rc;
    {
        double r;
        memcpy(&r, &ctx->hCnt->maxAbs, sizeof(r));
        ctx->coordScale = ctx->capLimit > 0 ? ctx->capLimit : r;
    }
    if (!cap) cudaEventRecord(ctx->ev[1], ctx->stream);
    rc = tsph_tree_moments(ctx, ctx->P, ctx->T, n, gp->dTheta, gp->iOrder, gp->precision == TSPH_FP32);
    if (rc) return rc;
    const bool ewald = n > 0 && gp->bPeriodic && gp->bEwald && gp->iEwOrder >= 1;
    // from the moments' completion a second stream prepares the walk's
    // bucket geometry and (periodic) the root multipoles and Ewald
    // constants, beside the Bmax and opening passes; the walk and the
    // Ewald pass wait for them
    if (n > 0 && ctx->T.nLeaves > 0) {
        TSPH_CK(cudaStreamWaitEvent(ctx->side, ctx->evMoments, 0));
        rc = tsph_bucket_prep(ctx, ctx->side);
        TSPH_CK(cudaEventRecord(ctx->evPrep, ctx->side));
        if (rc) {
            TSPH_CK(cudaStreamWaitEvent(ctx->stream, ctx->evPrep, 0));
            return rc;
        }
        ctx->bucketPrepQueued = true;
    }
    if (ewald) {
        TSPH_CK(cudaStreamWaitEvent(ctx->side, ctx->evMoments, 0));
        rc = tsph_ewald_roots(ctx, gp, ctx->side);
        TSPH_CK(cudaEventRecord(ctx->evEwald, ctx->side));   // the merge, error or not
        if (rc) {
            TSPH_CK(cudaStreamWaitEvent(ctx->stream, ctx->evEwald, 0));
            if (ctx->bucketPrepQueued) TSPH_CK(cudaStreamWaitEvent(ctx->stream, ctx->evPrep, 0));
            ctx->bucketPrepQueued = false;
            return rc;
        }
    }
    if (!cap) cudaEventRecord(ctx->ev[2], ctx->stream);
    ctx->haveTree = true;
    if (!gp->bPeriodic) {
        // coordinate scale for the rounding floor: the largest |coordinate|
        // (for a captured step, the bound its particles are checked against)
        double r;
        memcpy(&r, &ctx->hCnt->maxAbs, sizeof(r));
        if (ctx->capLimit > 0) r = ctx->capLimit;
        ctx->dPeriodTree = 2.0 * r;
    } else {
        ctx->dPeriodTree = 2.0 * gp->dPeriod;
    }
    if (n > 0 && ctx->T.nLeaves > 0) {
        rc = tsph_walk_interact(ctx, gp);
        ctx->bucketPrepQueued = false;
        if (rc) return rc;
    }
    if (!cap) cudaEventRecord(ctx->ev[3], ctx->stream);
    if (ewald) TSPH_CK(cudaStreamWaitEvent(ctx->stream, ctx->evEwald, 0));
    if (n > 0) {
        if (ewald) rc = tsph_ewald(ctx, gp);
        else if (gp->precision == TSPH_FP32 && ctx->T.nLeaves > 0) rc = tsph_walk_finish_f32(ctx);
        if (rc) return rc;
    }
    if (n > 0) {
        k_scatter_grav<<<tsph_blocks(n, 256), 256, 0, ctx->stream>>>(n, ctx->P, ctx->C);
        TSPH_LAUNCH_CK("k_scatter_grav");
    }
    if (cap) {
        ctx->haveGrav = true;
        return tsph_fold_status(ctx);
    }
    cudaEventRecord(ctx->ev[4], ctx->stream);
    rc = read_status(ctx);
    if (rc) return rc;
    ctx->lastListNeed = ctx->hCnt->listNeed;
    cudaEventElapsedTime(&ctx->timings[0], ctx->ev[0], ctx->ev[1]);
    cudaEventElapsedTime(&ctx->timings[1], ctx->ev[1], ctx->ev[2]);
    cudaEventElapsedTime(&ctx->timings[2], ctx->ev[2], ctx->ev[3]);
    cudaEventElapsedTime(&ctx->timings[3], ctx->ev[3], ctx->ev[4]);
    cudaEventElapsedTime(&ctx->timings[7], ctx->ev[0], ctx->ev[4]);
    ctx->lastGrav = *gp;
    ctx->haveGrav = true;
    if (out) {
        static const int qflop[5] = {10, 10, 41, 120, 277};
        static const int mflop[5] = {10, 10, 48, 151, 343};
        const TsphDevCounters &c = *ctx->hCnt;
        memset(out, 0, sizeof(*out));
        out->nActive = (int)c.nActive;
        out->nBuckets = ctx->T.nLeaves;
        out->dPartSum = (double)c.nPartPP + (double)c.nIntra;
        out->dCellSum = (double)c.nCellNewt;
        out->dSoftSum = (double)c.nCellSoft;
        double fg = 38.0 * ((double)c.nPartPP + (double)c.nBucketSq) + 82.0 * (double)c.nCellSoft +
                    (35.0 + qflop[gp->iOrder]) * (double)c.nCellNewt;
        double fe = 0.0;
        if (gp->bPeriodic && gp->bEwald && gp->iEwOrder >= 1)
            fe = (double)c.nEwLoop * (104.0 + mflop[gp->iEwOrder]) + (double)c.nActive * ctx->nEwt * 58.0;
        out->dFlop = fg + fe;
        out->dFlopEwald = fe;
        out->dExactFrac = c.nTests ? (double)c.nExactTests / (double)c.nTests : 0.0;
        out->dTests = (double)c.nTests;
        out->dVisits = (double)c.nVisits;
    }
    return TSPH_OK;
}

// interleave up to three caller-order arrays for one host copy
__global__ void k_interleave(int n, const double *__restrict__ a0, const double *__restrict__ a1,
                             const double *__restrict__ a2, int comp, double *dst) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    dst[comp * i] = a0[i];
    if (comp > 1) dst[comp * i + 1] = a1[i];
    if (comp > 2) dst[comp * i + 2] = a2[i];
}

// caller-order device arrays (n entries) -> host, interleaved by comp
int tsph_copy_out_n(tsph_ctx *ctx, int n, const double *a0, const double *a1, const double *a2,
                    int comp, double *host) {
    if (n == 0 || !host) return TSPH_OK;
    if (comp == 1) {
        TSPH_CK(cudaMemcpyAsync(host, a0, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
        TSPH_CK(cudaStreamSynchronize(ctx->stream));
        return TSPH_OK;
    }
    k_interleave<<<tsph_blocks(n, 256), 256, 0, ctx->stream>>>(n, a0, a1, a2, comp, ctx->dStage);
    TSPH_LAUNCH_CK("k_interleave");
    TSPH_CK(cudaMemcpyAsync(host, ctx->dStage, sizeof(double) * comp * n, cudaMemcpyDeviceToHost,
                            ctx->stream));
    TSPH_CK(cudaStreamSynchronize(ctx->stream));
    return TSPH_OK;
}

int tsph_copy_out(tsph_ctx *ctx, const double *a0, const double *a1, const double *a2, int comp,
                  double *host) {
    return tsph_copy_out_n(ctx, ctx->n, a0, a1, a2, comp, host);
}

extern "C" int tsph_get_gravity(tsph_ctx *ctx, double *acc, double *pot, double *dtGrav) {
    if (!ctx) return TSPH_ERR_ARG;
    if (!ctx->haveGrav) return TSPH_ERR_STATE;
    cudaSetDevice(ctx->device);
    int rc = tsph_copy_out(ctx, ctx->C.ax, ctx->C.ay, ctx->C.az, 3, acc);
    if (!rc) rc = tsph_copy_out(ctx, ctx->C.pot, nullptr, nullptr, 1, pot);
    if (!rc) rc = tsph_copy_out(ctx, ctx->C.dtGrav, nullptr, nullptr, 1, dtGrav);
    return rc;
}

extern "C" int tsph_get_tree(tsph_ctx *ctx, int *nNodes, int *inode, double *dnode, int *perm) {
    if (!ctx || !nNodes) return TSPH_ERR_ARG;
    if (!ctx->haveTree) return TSPH_ERR_STATE;
    cudaSetDevice(ctx->device);
    TSPH_CK(cudaStreamSynchronize(ctx->stream));
    const TsphDevTree &T = ctx->T;
    int nn = T.nNodes;
    *nNodes = nn;
    if (!inode) return TSPH_OK;
    size_t N = (size_t)nn;
    int *hi = (int *)malloc(sizeof(int) * N * 5);
    double *hd = (double *)malloc(sizeof(double) * N * 19);
    if (!hi || !hd) { free(hi); free(hd); return TSPH_ERR_NOMEM; }
    int *pLo = hi, *pUp = hi + N, *dim = hi + 2 * N, *up = hi + 3 * N, *skip = hi + 4 * N;
    double *fs = hd, *bnd = hd + N, *fm = hd + 7 * N, *so = hd + 8 * N, *r = hd + 9 * N;
    double *fo = hd + 12 * N, *bm = hd + 13 * N, *q = hd + 14 * N;   // q needs 6N: ends at 20N
    double *qbuf = (double *)malloc(sizeof(double) * N * 6);
    if (!qbuf) { free(hi); free(hd); return TSPH_ERR_NOMEM; }
    q = qbuf;
    int rc = TSPH_OK;
#define CPY(dst, src, cnt) \
    if (!rc && cudaMemcpy(dst, src, cnt, cudaMemcpyDeviceToHost) != cudaSuccess) rc = TSPH_ERR_CUDA
    CPY(pLo, T.pLower, sizeof(int) * N);
    CPY(pUp, T.pUpper, sizeof(int) * N);
    CPY(dim, T.iDim, sizeof(int) * N);
    CPY(up, T.upper, sizeof(int) * N);
    CPY(skip, T.skip, sizeof(int) * N);
    CPY(fs, T.fSplit, sizeof(double) * N);
    CPY(bnd, T.bnd, sizeof(double) * 6 * N);
    CPY(fm, T.fMass, sizeof(double) * N);
    CPY(so, T.fSoft, sizeof(double) * N);
    CPY(r, T.r, sizeof(double) * 3 * N);
    CPY(fo, T.fOpen2, sizeof(double) * N);
    CPY(bm, T.Bmax, sizeof(double) * N);
    CPY(q, T.Q, sizeof(double) * 6 * N);
    if (perm && ctx->n > 0) CPY(perm, ctx->P.iord, sizeof(int) * ctx->n);
#undef CPY
    if (!rc) {
        for (size_t i = 0; i < N; ++i) {
            bool leaf = up[i] < 0;
            inode[6 * i + 0] = pLo[i];
            inode[6 * i + 1] = pUp[i];
            inode[6 * i + 2] = dim[i];
            inode[6 * i + 3] = leaf ? -1 : (int)i + 1;   // threaded: first child
            inode[6 * i + 4] = skip[i];                  // threaded: next
            inode[6 * i + 5] = 0;
            dnode[16 * i + 0] = fs[i];
            for (int k = 0; k < 3; ++k) {
                dnode[16 * i + 1 + k] = bnd[6 * i + k];
                dnode[16 * i + 4 + k] = bnd[6 * i + 3 + k];
                dnode[16 * i + 9 + k] = r[3 * i + k];
            }
            dnode[16 * i + 7] = fm[i];
            dnode[16 * i + 8] = so[i];
            dnode[16 * i + 12] = fo[i];
            dnode[16 * i + 13] = bm[i];
            dnode[16 * i + 14] = q[6 * i + 0];
            dnode[16 * i + 15] = q[6 * i + 1];
        }
    }
    free(hi);
    free(hd);
    free(qbuf);
    return rc;
}

extern "C" int tsph_get_lists(tsph_ctx *ctx, int *nBuckets, int *blist) {
    if (!ctx || !nBuckets) return TSPH_ERR_ARG;
    if (!ctx->haveGrav) return TSPH_ERR_STATE;
    *nBuckets = ctx->T.nLeaves;
    if (!blist || ctx->T.nLeaves == 0) return TSPH_OK;
    cudaSetDevice(ctx->device);
    TSPH_CK(cudaStreamSynchronize(ctx->stream));
    TSPH_CK(cudaMemcpy(blist, ctx->dBucketLists, sizeof(int) * 4 * ctx->T.nLeaves,
                       cudaMemcpyDeviceToHost));
    return TSPH_OK;
}

extern "C" int tsph_get_timings(tsph_ctx *ctx, float *t8) {
    if (!ctx || !t8) return TSPH_ERR_ARG;
    memcpy(t8, ctx->timings, sizeof(float) * 8);
    return TSPH_OK;
}

extern "C" long long tsph_launch_count(tsph_ctx *ctx) { return ctx ? ctx->launches : 0; }

extern "C" int tsph_set_tuning(tsph_ctx *ctx, const tsph_tuning *t) {
    if (!ctx || !t) return TSPH_ERR_ARG;
    if (t->taskSize < 0 || (t->taskSize > 0 && t->taskSize < 1024)) return TSPH_ERR_ARG;
    if (t->walkBlocksPerSM < 0 || t->walkBlocksPerSM > 32) return TSPH_ERR_ARG;
    if (t->walkGroup < -1 || (t->walkGroup > 0 && (t->walkGroup < 32 || t->walkGroup > 4096)))
        return TSPH_ERR_ARG;
    if (t->walkLists < -1 || (t->walkLists > 1 && (t->walkLists < 32 || t->walkLists > 65536)))
        return TSPH_ERR_ARG;
    // a captured step keeps the knobs it was captured with: a change recaptures
    if (t->taskSize != ctx->taskSize || t->walkBlocksPerSM != ctx->walkBlocksPerSM ||
        t->walkGroup != ctx->walkGroup || t->walkLists != ctx->walkLists)
        ctx->sysVersion++;
    ctx->taskSize = t->taskSize;
    ctx->walkBlocksPerSM = t->walkBlocksPerSM;
    ctx->walkGroup = t->walkGroup;
    // a new list mode starts its slots afresh; the same mode keeps the
    // slots it has grown to
    if (t->walkLists != ctx->walkLists) ctx->walkListSlot = t->walkLists > 1 ? t->walkLists : 0;
    ctx->walkLists = t->walkLists;
    return TSPH_OK;
}

extern "C" int tsph_get_tuning(tsph_ctx *ctx, tsph_tuning *t) {
    if (!ctx || !t) return TSPH_ERR_ARG;
    memset(t, 0, sizeof(*t));
    t->taskSize = ctx->taskSize;
    t->walkBlocksPerSM = ctx->walkBlocksPerSM;
    t->walkGroup = ctx->walkGroup;
    t->walkLists = ctx->walkLists;
    return TSPH_OK;
}
