// One kick-drift-kick step as a single stream of kernels, optionally
// captured once as a CUDA graph and replayed.
//
// The step follows the reference's single-rung msrTopStepKDK
// (master.c:8242-8465): opening kick by dt/2 (msrKickKDKOpen), two drifts
// by dt/2 (msrDrift: pkdDrift + pkdKickVpred), forces at the new positions
// for every particle (pkdGravAll, then for the gas smSmooth(SMX_DENDVDX),
// pkdGasPressure, smReSmooth(SMX_SPHPRESSURETERMS)), closing kick by dt/2
// (msrKickKDKClose).  In graph mode every launch of that sequence is
// recorded once and the whole step replays as one graph launch: no host
// round trip, no per-kernel launch cost, which is what many small systems
// in one context need.  The graph's kicks and drifts read dt from device
// memory, set by a one-thread kernel before each replay, so a new dt needs
// no recapture.  A captured build runs a fixed number of top-phase levels
// (its preparation's depth + 2; deeper nodes become subtree tasks) and has
// fixed coordinate bounds; a particle leaving them raises TSPH_ERR_BOUNDS
// and the next call recaptures.  dt may be negative: the leapfrog is
// time-reversible, so a step of -dt undoes a step of dt up to rounding.
#include <math.h>
#include <string.h>

#include "tsph_ctx.cuh"

__global__ void k_coord_maxabs(int n, TsphDevState C, unsigned long long *out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double a = 0.0;
    if (i < n) a = fmax(fabs(C.x[i]), fmax(fabs(C.y[i]), fabs(C.z[i])));
    warp_max_abs(a, out);
}

__global__ void k_set_step_dt(double *d, double dt) { *d = dt; }

static int step_body(tsph_ctx *ctx, double dt, const tsph_grav_params *gp,
                     const tsph_sph_params *sp) {
    const int actRung = ctx->actRung;
    ctx->actRung = 0;   // one rung: every particle is active
    int rc = tsph_kick_rung(ctx, -1, 0.5 * dt, 0);
    if (!rc) rc = tsph_drift(ctx, 0.5 * dt, gp->bPeriodic, gp->dPeriod);
    if (!rc) rc = tsph_drift(ctx, 0.5 * dt, gp->bPeriodic, gp->dPeriod);
    if (!rc) rc = tsph_grav_all(ctx, gp, nullptr);
    if (!rc && sp && ctx->ngas > 0) {
        rc = tsph_smooth(ctx, TSPH_SMX_DENDVDX, sp, nullptr);
        if (!rc) rc = tsph_smooth(ctx, TSPH_SMX_SPHPRESSURETERMS, sp, nullptr);
    }
    if (!rc) rc = tsph_kick_rung(ctx, -1, 0.5 * dt, 1);
    ctx->actRung = actRung;
    return rc;
}

static void drop_graph(tsph_ctx *ctx) {
    if (ctx->graphExec) cudaGraphExecDestroy(ctx->graphExec);
    ctx->graphExec = nullptr;
}

// A captured step reads dt from device memory, so one graph serves every dt.
static bool graph_matches(const tsph_ctx *ctx, const tsph_grav_params *gp, const tsph_sph_params *sp) {
    if (!ctx->graphExec || ctx->graphN != ctx->n || ctx->graphNgas != ctx->ngas ||
        ctx->graphSysVersion != ctx->sysVersion)
        return false;
    if (memcmp(&ctx->graphGrav, gp, sizeof(*gp)) != 0) return false;
    if ((sp != nullptr) != (ctx->graphHasSph != 0)) return false;
    return !sp || memcmp(&ctx->graphSph, sp, sizeof(*sp)) == 0;
}

// Record the step: forces are first evaluated once on the current state
// (allocating everything, uploading constants; the accelerations the
// previous step left are kept), then the step is captured with the
// coordinate bound fixed at twice the current extent.
static int capture_step(tsph_ctx *ctx, const tsph_grav_params *gp, const tsph_sph_params *sp) {
    drop_graph(ctx);
    const int n = ctx->n;
    TSPH_CK(cudaMemsetAsync(ctx->dAux + 1, 0, sizeof(unsigned long long), ctx->stream));
    k_coord_maxabs<<<tsph_blocks(n, 256), 256, 0, ctx->stream>>>(n, ctx->C, ctx->dAux + 1);
    TSPH_LAUNCH_CK("k_coord_maxabs");
    unsigned long long bits = 0;
    TSPH_CK(cudaMemcpyAsync(&bits, ctx->dAux + 1, sizeof(bits), cudaMemcpyDeviceToHost, ctx->stream));
    TSPH_CK(cudaStreamSynchronize(ctx->stream));
    double ext;
    memcpy(&ext, &bits, sizeof(ext));
    ctx->capLimit = 2.0 * ext + 1e-300;
    // The preparation must leave the accelerations the step's opening kick
    // reads as they are: the gas's pressure accelerations and uDot depend on
    // vPred and uPred, which the last closing kick moved on, so evaluating
    // them again here would change them.  Keep them and put them back.
    const int ng = sp ? ctx->ngas : 0;
    const size_t nKeep = 3 * (size_t)n + 4 * (size_t)ng;
    if (ctx->keepCap < nKeep) {
        int rc = tsph_grow(ctx, &ctx->dKeep, nKeep);
        if (rc) { ctx->keepCap = 0; ctx->capLimit = 0; return rc; }
        ctx->keepCap = nKeep;
    }
    double *const keep[7] = {ctx->C.ax, ctx->C.ay, ctx->C.az, ctx->C.hax, ctx->C.hay, ctx->C.haz,
                             ctx->C.udot};
    size_t len[7], off[7];
    size_t o = 0;
    for (int k = 0; k < 7; ++k) {
        len[k] = k < 3 ? (size_t)n : (size_t)ng;
        off[k] = o;
        o += len[k];
    }
    for (int k = 0; k < 7; ++k)
        if (len[k]) TSPH_CK(cudaMemcpyAsync(ctx->dKeep + off[k], keep[k], sizeof(double) * len[k],
                                            cudaMemcpyDeviceToDevice, ctx->stream));
    int rc = tsph_grav_all(ctx, gp, nullptr);
    if (!rc && sp && ctx->ngas > 0) {
        rc = tsph_smooth(ctx, TSPH_SMX_DENDVDX, sp, nullptr);
        if (!rc) rc = tsph_smooth(ctx, TSPH_SMX_SPHPRESSURETERMS, sp, nullptr);
    }
    if (rc) { ctx->capLimit = 0; return rc; }
    for (int k = 0; k < 7; ++k)
        if (len[k]) TSPH_CK(cudaMemcpyAsync(keep[k], ctx->dKeep + off[k], sizeof(double) * len[k],
                                            cudaMemcpyDeviceToDevice, ctx->stream));
    TSPH_CK(cudaStreamSynchronize(ctx->stream));
    if (!ctx->dStepDt && cudaMalloc((void **)&ctx->dStepDt, sizeof(double)) != cudaSuccess) {
        ctx->capLimit = 0;
        return TSPH_ERR_NOMEM;
    }
    cudaGraph_t graph = nullptr;
    TSPH_CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    ctx->capturing = true;
    ctx->stepDtDev = ctx->dStepDt;   // kicks and drifts scale a unit step by the dt there
    const long long before = ctx->launches;
    rc = step_body(ctx, 1.0, gp, sp);
    ctx->graphKernels = ctx->launches - before;
    ctx->launches = before;
    ctx->stepDtDev = nullptr;
    ctx->capturing = false;
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
    if (!rc && e != cudaSuccess) rc = tsph_cuda_fail(ctx, e, "cudaStreamEndCapture");
    if (!rc) {
        e = cudaGraphInstantiate(&ctx->graphExec, graph, 0);
        if (e != cudaSuccess) rc = tsph_cuda_fail(ctx, e, "cudaGraphInstantiate");
    }
    if (graph) cudaGraphDestroy(graph);
    ctx->capLimit = 0;   // the graph keeps its own copy; direct calls measure afresh
    if (rc) {
        drop_graph(ctx);
        cudaGetLastError();
        return rc;
    }
    ctx->graphN = n;
    ctx->graphNgas = ctx->ngas;
    ctx->graphSysVersion = ctx->sysVersion;
    ctx->graphGrav = *gp;
    ctx->graphHasSph = sp != nullptr;
    if (sp) ctx->graphSph = *sp;
    return TSPH_OK;
}

extern "C" int tsph_step(tsph_ctx *ctx, double dt, const tsph_grav_params *gp,
                         const tsph_sph_params *sp, int flags) {
    if (!ctx || !gp || !isfinite(dt)) return TSPH_ERR_ARG;
    if (!ctx->haveParts || !ctx->haveVel) return TSPH_ERR_STATE;
    cudaSetDevice(ctx->device);
    if (!(flags & TSPH_STEP_GRAPH)) return step_body(ctx, dt, gp, sp);
    // a captured density pass can seed from the h-network, not collect for it
    if (sp && sp->bLearnedH && ctx->hnet.collect) return TSPH_ERR_UNSUPPORTED;
    if (ctx->n == 0) return TSPH_OK;
    if (!graph_matches(ctx, gp, sp)) {
        int rc = capture_step(ctx, gp, sp);
        if (rc) return rc;
    }
    k_set_step_dt<<<1, 1, 0, ctx->stream>>>(ctx->dStepDt, dt);
    TSPH_LAUNCH_CK("k_set_step_dt");
    TSPH_CK(cudaGraphLaunch(ctx->graphExec, ctx->stream));
    ctx->launches += ctx->graphKernels;   // kernels the replay runs
    return TSPH_OK;
}

extern "C" int tsph_step_status(tsph_ctx *ctx) {
    if (!ctx) return TSPH_ERR_ARG;
    cudaSetDevice(ctx->device);
    unsigned int st = 0;
    TSPH_CK(cudaMemcpyAsync(&st, ctx->dStepStatus, sizeof(st), cudaMemcpyDeviceToHost, ctx->stream));
    TSPH_CK(cudaMemsetAsync(ctx->dStepStatus, 0, sizeof(st), ctx->stream));
    TSPH_CK(cudaStreamSynchronize(ctx->stream));
    for (int k = 1; k < 32; ++k)
        if (st & (1u << k)) {
            if (k == TSPH_ERR_BOUNDS) drop_graph(ctx);   // recapture on the next step
            return k;
        }
    return TSPH_OK;
}
