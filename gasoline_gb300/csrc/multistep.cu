// Adaptive timesteps: particles on rungs 0..iMaxRung-1 take steps of
// dDelta / 2^rung, driven by the recursion of the reference's
// msrTopStepKDK (master.c:8242-8465).
//
// The recursion is host code (as the reference's master is); everything it
// does to particles runs on the device:
//   k_rung_adjust    the timestep criteria of the particles on rung >= iRung
//                    (pkdInitDt pkd.c:4818, pkdGravStep pkd.c:4609,
//                    pkdAccelStep pkd.c:4625, pkdSphStep pkd.c:5901) and
//                    their new rung (pkdDtToRung pkd.c:4715-4815)
//   k_rung_emergency gas on a lower rung whose dtNew fell below half the
//                    current step moves up (pkdEmergencyAdjust pkd.c:3971)
//   k_rung_hist      rung histograms (all, gas) the host branches on
//   k_kick_rung, k_drift (sph.cu) and the force passes over the active
//                    rungs (tsph_grav_all / tsph_smooth with ctx->actRung).
// All arithmetic of the criteria follows the reference's operation order
// without contraction, so rungs agree bit for bit with the reference given
// the same accelerations.
#include <float.h>
#include <math.h>
#include <string.h>

#include "tsph_ctx.cuh"

namespace {

constexpr int RUNG_MAX = 30;   // the reference allows at most 29 rungs

// pkdOneParticleDtToRung (pkd.c:4693-4713)
__device__ int one_particle_dt_to_rung(int iRung, double dDelta, double dt) {
    const double dSteps = dDelta / dt;
    int iSteps = (int)floor(dSteps);
    if (fmod(dDelta, dt) == 0.0) iSteps--;   // an exact multiple goes to the lower rung
    int r = iRung;
    if (iSteps < 0) iSteps = 0;
    while (iSteps) {
        ++r;
        iSteps >>= 1;
    }
    return r;
}

struct AdjustArgs {
    int n, ngas, iRung, iMaxRung;
    double dDeltaBase;   // msrInitDt: the base step (master.c:7970-7977)
    double dDelta;       // the step of rung iRung
    double dEta;
    int bGravStep, bEpsAccStep, bSqrtPhiStep, bSph;
    double dtFacCourant, dEtauDot, duMinDt;
};

__global__ void k_rung_adjust(AdjustArgs A, TsphDevState C, unsigned int *status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n || C.rung[i] < A.iRung) return;
    const bool gas = i < A.ngas;
    double dt = A.dDeltaBase;                                    // pkdInitDt
    if (A.bGravStep) {                                           // pkdGravStep
        const double g = C.dtGrav[i];
        if (g > 0.0) {
            const double d = A.dEta / sqrt(g);
            if (d < dt) dt = d;
        } else {
            atomicOr(status, 1u << TSPH_ERR_NONFINITE);   // the reference asserts dtGrav > 0
        }
    }
    if (A.bEpsAccStep || A.bSqrtPhiStep) {                       // pkdAccelStep, dVelFac = dAccFac = 1
        double a[3] = {C.ax[i], C.ay[i], C.az[i]};
        if (gas) { a[0] = xadd(a[0], C.hax[i]); a[1] = xadd(a[1], C.hay[i]); a[2] = xadd(a[2], C.haz[i]); }
        double acc = 0.0;
#pragma unroll
        for (int k = 0; k < 3; ++k) acc = xadd(acc, xmul(a[k], a[k]));
        acc = xmul(sqrt(acc), 1.0);
        double dT = DBL_MAX;
        if (A.bEpsAccStep && acc > 0) {
            if (gas) dT = xmul(A.dEta, sqrt(sqrt(xmul(0.25, C.fb2prev[i])) / acc));
            else dT = xmul(A.dEta, sqrt(C.h[i] / acc));
        }
        if (A.bSqrtPhiStep && acc > 0) {
            const double d = xmul(xmul(A.dEta, 3.5), sqrt(xmul(1.0, fabs(C.pot[i])))) / acc;
            if (d < dT) dT = d;
        }
        if (dT < dt) dt = dT;
    }
    if (gas && A.bSph) {                                         // pkdSphStep (its last criterion)
        double dT = C.dtNew[i];
        C.dtNew[i] = FLT_MAX;
        const double uTotDot = C.udot[i];
        if (uTotDot > 0) {
            const double c = C.cs[i];
            const double dtExtrap = xmul(A.dtFacCourant,
                sqrt(xmul(C.fb2prev[i], 0.25) /
                     xmul(4.0, xadd(xmul(c, c), xmul(xmul(5. / 3., uTotDot), dt)))));
            if (dtExtrap < dT) dT = dtExtrap;
        }
        const double updv = C.updv[i];
        if (A.dEtauDot > 0.0 && updv < 0.0) {
            double uEff = xadd(xadd(0.0, 0.0 / (2.0 - 1)), C.u[i]);   // PONRHOFLOOR + Jeans floor (0) + u
            if (uEff < A.duMinDt) uEff = A.duMinDt;
            const double dTu = xmul(A.dEtauDot, uEff) / fabs(updv);
            if (dTu < dT) dT = dTu;
        }
        if (dT < dt) dt = dT;
    }
    C.dt[i] = dt;
    int r = one_particle_dt_to_rung(A.iRung, A.dDelta, dt);      // pkdDtToRung, bAll = 1
    if (r >= A.iMaxRung) r = A.iMaxRung - 1;
    C.rung[i] = r;
}

__global__ void k_rung_emergency(int ngas, int iRung, int iMaxRung, double dDelta, double thresh,
                                 TsphDevState C, int *stat) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ngas) return;
    if (!(C.rung[i] < iRung && C.dtNew[i] < thresh)) return;
    const double dt = C.dtNew[i];
    C.dt[i] = dt;
    int r = one_particle_dt_to_rung(iRung, dDelta, dt);
    if (r >= iMaxRung) r = iMaxRung - 1;
    C.rung[i] = r;
    // unkick: back to the predicted velocity (NOCOOLING keeps u)
    C.vx[i] = C.vpx[i];
    C.vy[i] = C.vpy[i];
    C.vz[i] = C.vpz[i];
    atomicAdd(&stat[0], 1);
    atomicMax(&stat[1], r);
}

// hist[r] = particles on rung r, hist[RUNG_MAX + r] = gas particles on it
__global__ void k_rung_hist(int n, int ngas, const int *__restrict__ rung, int *hist) {
    __shared__ int sh[2 * RUNG_MAX];
    for (int k = threadIdx.x; k < 2 * RUNG_MAX; k += blockDim.x) sh[k] = 0;
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        int r = rung[i];
        r = r < 0 ? 0 : (r >= RUNG_MAX ? RUNG_MAX - 1 : r);
        atomicAdd(&sh[r], 1);
        if (i < ngas) atomicAdd(&sh[RUNG_MAX + r], 1);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 2 * RUNG_MAX; k += blockDim.x)
        if (sh[k]) atomicAdd(&hist[k], sh[k]);
}

struct TopStep {
    tsph_ctx *ctx;
    const tsph_grav_params *gp;
    const tsph_sph_params *sp;
    const tsph_step_params *st;
    double dDeltaBase;
    int iCurrMaxRung;
    int hist[2 * RUNG_MAX];
    tsph_step_out out;
};

int *stat_buf(tsph_ctx *ctx) { return reinterpret_cast<int *>(ctx->dAux + 2); }

// histograms of the current rungs on the host (one round trip)
int refresh_hist(TopStep &T) {
    tsph_ctx *ctx = T.ctx;
    int *d = stat_buf(ctx) + 4;
    TSPH_CK(cudaMemsetAsync(d, 0, sizeof(int) * 2 * RUNG_MAX, ctx->stream));
    if (ctx->n > 0) {
        k_rung_hist<<<tsph_blocks(ctx->n, 256), 256, 0, ctx->stream>>>(ctx->n, ctx->ngas, ctx->C.rung, d);
        TSPH_LAUNCH_CK("k_rung_hist");
    }
    TSPH_CK(cudaMemcpyAsync(T.hist, d, sizeof(int) * 2 * RUNG_MAX, cudaMemcpyDeviceToHost, ctx->stream));
    TSPH_CK(cudaStreamSynchronize(ctx->stream));
    return TSPH_OK;
}

int count_from(const TopStep &T, int iRung, bool gasOnly) {
    int c = 0;
    for (int r = iRung < 0 ? 0 : iRung; r < RUNG_MAX; ++r) c += T.hist[(gasOnly ? RUNG_MAX : 0) + r];
    return c;
}

int max_rung(const TopStep &T) {
    for (int r = RUNG_MAX - 1; r > 0; --r)
        if (T.hist[r]) return r;
    return 0;
}

// msrEmergencyAdjust (master.c:6742-6763)
int emergency(TopStep &T, int iRung, double dDelta) {
    tsph_ctx *ctx = T.ctx;
    if (ctx->ngas == 0) return TSPH_OK;
    int *d = stat_buf(ctx);
    TSPH_CK(cudaMemsetAsync(d, 0, 2 * sizeof(int), ctx->stream));
    k_rung_emergency<<<tsph_blocks(ctx->ngas, 256), 256, 0, ctx->stream>>>(
        ctx->ngas, iRung, T.st->iMaxRung, dDelta, dDelta * 0.5, ctx->C, d);
    TSPH_LAUNCH_CK("k_rung_emergency");
    int h[2];
    TSPH_CK(cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    TSPH_CK(cudaStreamSynchronize(ctx->stream));
    if (h[0]) {
        T.out.nEmergency += h[0];
        if (h[1] > T.iCurrMaxRung) T.iCurrMaxRung = h[1];
        return refresh_hist(T);
    }
    return TSPH_OK;
}

// the Adjust block of msrTopStepKDK (master.c:8264-8317)
int adjust(TopStep &T, int iRung, double dDelta) {
    tsph_ctx *ctx = T.ctx;
    AdjustArgs A;
    memset(&A, 0, sizeof(A));
    A.n = ctx->n;
    A.ngas = ctx->ngas;
    A.iRung = iRung;
    A.iMaxRung = T.st->iMaxRung;
    A.dDeltaBase = T.dDeltaBase;
    A.dDelta = dDelta;
    A.dEta = T.st->dEta;
    A.bGravStep = T.st->bGravStep;
    A.bEpsAccStep = T.st->bEpsAccStep;
    A.bSqrtPhiStep = T.st->bSqrtPhiStep;
    A.bSph = T.sp != nullptr;
    A.dtFacCourant = T.sp ? T.sp->dEtaCourant * 1.0 * 2 / 1.6 : 0.0;   // pkdDtFacCourant, a = 1
    A.dEtauDot = T.st->dEtauDot;
    A.duMinDt = T.st->duMinDt;
    unsigned int *st = reinterpret_cast<unsigned int *>(stat_buf(ctx) + 3);
    TSPH_CK(cudaMemsetAsync(st, 0, sizeof(unsigned int), ctx->stream));
    if (ctx->n > 0) {
        k_rung_adjust<<<tsph_blocks(ctx->n, 256), 256, 0, ctx->stream>>>(A, ctx->C, st);
        TSPH_LAUNCH_CK("k_rung_adjust");
    }
    unsigned int hst = 0;
    TSPH_CK(cudaMemcpyAsync(&hst, st, sizeof(hst), cudaMemcpyDeviceToHost, ctx->stream));
    int rc = refresh_hist(T);   // synchronises
    if (rc) return rc;
    if (hst) for (int k = 1; k < 32; ++k) if (hst & (1u << k)) return k;
    T.iCurrMaxRung = max_rung(T);   // msrDtToRung: the highest rung of any particle
    return TSPH_OK;
}

// the force pass of msrTopStepKDK (master.c:8397-8436): gravity on the
// particles of rung >= iKickRung, SPH when any gas is among them
int forces(TopStep &T, int iKickRung) {
    tsph_ctx *ctx = T.ctx;
    const int nAct = count_from(T, iKickRung, false);
    if (nAct == 0) return TSPH_OK;
    ctx->actRung = iKickRung;
    int rc = tsph_grav_all(ctx, T.gp, nullptr);
    if (!rc && T.sp && count_from(T, iKickRung, true) > 0) {
        rc = tsph_smooth(ctx, TSPH_SMX_DENDVDX, T.sp, nullptr);
        if (!rc) rc = tsph_smooth(ctx, TSPH_SMX_SPHPRESSURETERMS, T.sp, nullptr);
    }
    ctx->actRung = 0;
    if (rc) return rc;
    T.out.nForcePasses += 1;
    T.out.nActiveSum += nAct;
    return TSPH_OK;
}

int top_step(TopStep &T, double dTime, double dDelta, int iRung, int iKickRung, int iAdjust) {
    tsph_ctx *ctx = T.ctx;
    int rc;
    if (iAdjust) {
        rc = emergency(T, iRung, dDelta);
        if (rc) return rc;
    }
    if (iAdjust && iRung < T.st->iMaxRung - 1) {
        rc = adjust(T, iRung, dDelta);
        if (rc) return rc;
    }
    rc = tsph_kick_launch(ctx, iRung, 0.5 * dDelta, 0);
    if (rc) return rc;
    if (T.iCurrMaxRung > iRung) {
        rc = top_step(T, dTime, 0.5 * dDelta, iRung + 1, iRung + 1, 0);
        if (rc) return rc;
        dTime += 0.5 * dDelta;
        rc = top_step(T, dTime, 0.5 * dDelta, iRung + 1, iKickRung, 1);
        if (rc) return rc;
    } else {
        rc = tsph_drift(ctx, 0.5 * dDelta, T.gp->bPeriodic, T.gp->dPeriod);
        if (!rc) rc = tsph_drift(ctx, 0.5 * dDelta, T.gp->bPeriodic, T.gp->dPeriod);
        if (!rc) rc = forces(T, iKickRung);
        if (rc) return rc;
    }
    return tsph_kick_launch(ctx, iRung, 0.5 * dDelta, 1);
}

}  // namespace

extern "C" int tsph_top_step_kdk(tsph_ctx *ctx, double dTime, double dDelta,
                                 const tsph_grav_params *gp, const tsph_sph_params *sp,
                                 const tsph_step_params *st, tsph_step_out *out) {
    if (!ctx || !gp || !st || !(dDelta > 0)) return TSPH_ERR_ARG;
    if (st->iMaxRung < 1 || st->iMaxRung > 29) return TSPH_ERR_ARG;
    if (!ctx->haveParts || !ctx->haveVel) return TSPH_ERR_STATE;
    if (ctx->capturing) return TSPH_ERR_STATE;
    cudaSetDevice(ctx->device);
    TopStep T;
    memset(&T, 0, sizeof(T));
    T.ctx = ctx;
    T.gp = gp;
    T.sp = (sp && ctx->ngas > 0) ? sp : nullptr;
    T.st = st;
    T.dDeltaBase = dDelta;
    int rc = refresh_hist(T);
    if (rc) return rc;
    T.iCurrMaxRung = max_rung(T);
    rc = top_step(T, dTime, dDelta, 0, 0, 1);
    ctx->actRung = 0;
    if (rc) return rc;
    TSPH_CK(cudaStreamSynchronize(ctx->stream));
    T.out.iCurrMaxRung = T.iCurrMaxRung;
    if (out) *out = T.out;
    return TSPH_OK;
}

extern "C" int tsph_set_active_rung(tsph_ctx *ctx, int iRung) {
    if (!ctx || iRung < 0) return TSPH_ERR_ARG;
    ctx->actRung = iRung;
    return TSPH_OK;
}

extern "C" int tsph_set_rungs(tsph_ctx *ctx, const int *rung) {
    if (!ctx || !rung) return TSPH_ERR_ARG;
    if (!ctx->haveParts) return TSPH_ERR_STATE;
    for (int i = 0; i < ctx->n; ++i)
        if (rung[i] < 0 || rung[i] >= 29) return TSPH_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->n == 0) return TSPH_OK;
    TSPH_CK(cudaMemcpyAsync(ctx->C.rung, rung, sizeof(int) * ctx->n, cudaMemcpyHostToDevice, ctx->stream));
    TSPH_CK(cudaStreamSynchronize(ctx->stream));
    return TSPH_OK;
}

extern "C" int tsph_get_rungs(tsph_ctx *ctx, int *rung, double *dt, double *dtNew, double *mumax) {
    if (!ctx) return TSPH_ERR_ARG;
    if (!ctx->haveParts) return TSPH_ERR_STATE;
    cudaSetDevice(ctx->device);
    const int n = ctx->n;
    if (n == 0) return TSPH_OK;
    if (rung) TSPH_CK(cudaMemcpyAsync(rung, ctx->C.rung, sizeof(int) * n, cudaMemcpyDeviceToHost, ctx->stream));
    if (dt) TSPH_CK(cudaMemcpyAsync(dt, ctx->C.dt, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    if (dtNew) TSPH_CK(cudaMemcpyAsync(dtNew, ctx->C.dtNew, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    if (mumax) TSPH_CK(cudaMemcpyAsync(mumax, ctx->C.mumax, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    TSPH_CK(cudaStreamSynchronize(ctx->stream));
    return TSPH_OK;
}
