// Frames: the reference's TSC particle splat (dfRenderParticleTSC,
// dumpframe.c:1125-1230) as one thread per particle adding its footprint
// into a device image.  Contributions accumulate in FP64 (the reference
// adds them into a float image in particle order; FP64 makes the result
// independent of the order the atomics land in, to the float it is stored
// as) and the frame is converted to the reference's float RGB at the end.
#include <math.h>
#include <string.h>

#include "tsph_ctx.cuh"

namespace {

struct RenderArgs {
    int n, ngas, nStar;
    tsph_render_params p;
    double xlim, ylim, hmul;
};

struct Col3 { float r, g, b; };

// dfColInterp (dumpframe.c:1096-1122), float arithmetic as there
__device__ Col3 col_interp(int nCol, const float *dCol, const float (*Col)[3], double fVar,
                           int bLog) {
    Col3 c0 = {Col[0][0], Col[0][1], Col[0][2]};
    if (!nCol) return c0;
    if (bLog) fVar = log10(fVar);
    if (fVar <= dCol[0]) return c0;
    Col3 cl = {Col[nCol - 1][0], Col[nCol - 1][1], Col[nCol - 1][2]};
    if (fVar >= dCol[nCol - 1]) return cl;
    int i = 1;
    for (;;) {
        if (fVar <= dCol[i]) break;
        i++;
        if (i >= nCol) return cl;
    }
    const float x = (float)((fVar - dCol[i - 1]) / (dCol[i] - dCol[i - 1]));
    Col3 c;
    c.r = __fadd_rn(__fmul_rn(x, Col[i][0]), __fmul_rn(1 - x, Col[i - 1][0]));
    c.g = __fadd_rn(__fmul_rn(x, Col[i][1]), __fmul_rn(1 - x, Col[i - 1][1]));
    c.b = __fadd_rn(__fmul_rn(x, Col[i][2]), __fmul_rn(1 - x, Col[i - 1][2]));
    return c;
}

__global__ void k_render_tsc(RenderArgs A, TsphDevState C, const double *__restrict__ rho,
                             double *img) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n) return;
    const tsph_render_params &P = A.p;
    const double m = C.m[i];
    double h;
    Col3 col;
    if (i < A.ngas) {
        if (m < P.dMassGasMin || m > P.dMassGasMax) return;
        h = P.bGasSph ? sqrt(C.fb2prev[i]) * 0.5 * P.dGasSoftMul : C.h[i] * P.dGasSoftMul;
        col = col_interp(P.nColGas, P.dColGas, P.colGas, rho ? rho[i] : 0.0, P.bColLogInterp);
    } else if (i < A.n - A.nStar) {
        if (m < P.dMassDarkMin || m > P.dMassDarkMax) return;
        h = C.h[i] * P.dDarkSoftMul;
        col = col_interp(P.nColDark, P.dColDark, P.colDark, 0.0, P.bColLogInterp);
    } else {
        if (m < P.dMassStarMin || m > P.dMassStarMax) return;
        h = C.h[i] * P.dStarSoftMul;
        col = col_interp(P.nColStar, P.dColStar, P.colStar, 0.0, P.bColLogInterp);
    }
    double br0 = 1;
    if (P.bColMassWeight) br0 *= m;
    const double dr[3] = {C.x[i] - P.r[0], C.y[i] - P.r[1], C.z[i] - P.r[2]};
    const double z = dr[0] * P.z[0] + dr[1] * P.z[1] + dr[2] * P.z[2] + P.zEye;
    if (!(z >= P.zClipNear && z <= P.zClipFar)) return;
    const bool persp = P.iProject == 2;
    h = persp ? h * A.hmul / z : h * A.hmul;
    const int hint = (int)h;
    double x = dr[0] * P.x[0] + dr[1] * P.x[1] + dr[2] * P.x[2];
    if (persp) x /= z;
    if (!(fabs(x) < A.xlim + hint)) return;
    double y = dr[0] * P.y[0] + dr[1] * P.y[1] + dr[2] * P.y[2];
    if (persp) y /= z;
    if (!(fabs(y) < A.ylim + hint)) return;
    x = x + A.xlim;
    const int xp = (int)x;
    y = A.ylim - y;   // screen convention
    const int yp = (int)y;
    const int nx = P.nxPix, ny = P.nyPix;
    if (hint < 1) {
        if (xp < 0 || xp >= nx || yp < 0 || yp >= ny) return;
        double *q = img + 3 * ((size_t)yp * nx + xp);
        atomicAdd(q, br0 * col.r);
        atomicAdd(q + 1, br0 * col.g);
        atomicAdd(q + 2, br0 * col.b);
        return;
    }
    const double ih2 = 1. / (h * h);
    const double br1 = br0 * (6 / (2.0 * 3.1412)) * ih2;   // the reference's constant
    const int xmin = xp - hint < 0 ? 0 : xp - hint, xmax = xp + hint >= nx ? nx - 1 : xp + hint;
    const int ymin = yp - hint < 0 ? 0 : yp - hint, ymax = yp + hint >= ny ? ny - 1 : yp + hint;
    for (int iy = ymin; iy <= ymax; ++iy) {
        for (int ix = xmin; ix <= xmax; ++ix) {
            const double r2 = ((ix - x) * (ix - x) + (iy - y) * (iy - y)) * ih2;
            if (r2 > 1) continue;
            const double br = br1 * (1.0 - sqrt(r2));
            double *q = img + 3 * ((size_t)iy * nx + ix);
            atomicAdd(q, br * col.r);
            atomicAdd(q + 1, br * col.g);
            atomicAdd(q + 2, br * col.b);
        }
    }
}

__global__ void k_image_to_float(size_t n, const double *__restrict__ img, float *out) {
    size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) out[k] = (float)img[k];
}

// the gas density of the last SPH pass in caller order
__global__ void k_rho_caller(int ng, const int *__restrict__ iord, const double *__restrict__ rho,
                             double *out) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < ng) out[iord[k]] = rho[k];
}

__global__ void k_rho_snap(int ng, const float *__restrict__ rho, double *out) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < ng) out[k] = rho[k];
}

}  // namespace

extern "C" int tsph_render_tsc(tsph_ctx *ctx, const tsph_render_params *rp, int nStar, float *rgb) {
    if (!ctx || !rp || !rgb) return TSPH_ERR_ARG;
    if (rp->nxPix < 1 || rp->nyPix < 1 || rp->nxPix > 16384 || rp->nyPix > 16384) return TSPH_ERR_ARG;
    if (rp->nColGas < 0 || rp->nColGas > 10 || rp->nColDark < 0 || rp->nColDark > 10 ||
        rp->nColStar < 0 || rp->nColStar > 10 || (rp->iProject != 1 && rp->iProject != 2))
        return TSPH_ERR_ARG;
    if (!ctx->haveParts) return TSPH_ERR_STATE;
    if (ctx->capturing) return TSPH_ERR_STATE;
    if (nStar < 0 || nStar > ctx->n - ctx->ngas) return TSPH_ERR_ARG;
    cudaSetDevice(ctx->device);
    const size_t npix = (size_t)rp->nxPix * rp->nyPix * 3;
    double *img = nullptr, *rho = nullptr;
    float *out = nullptr;
    int rc = TSPH_OK;
    if (cudaMalloc((void **)&img, npix * sizeof(double)) != cudaSuccess ||
        cudaMalloc((void **)&out, npix * sizeof(float)) != cudaSuccess ||
        cudaMalloc((void **)&rho, sizeof(double) * (ctx->ngas > 0 ? ctx->ngas : 1)) != cudaSuccess) {
        rc = TSPH_ERR_NOMEM;
    }
    const int ng = ctx->ngas;
    if (!rc && cudaMemsetAsync(img, 0, npix * sizeof(double), ctx->stream) != cudaSuccess) rc = TSPH_ERR_CUDA;
    if (!rc && ng > 0) {
        if (cudaMemsetAsync(rho, 0, sizeof(double) * ng, ctx->stream) != cudaSuccess) rc = TSPH_ERR_CUDA;
        else if (ctx->S.haveDensity)
            k_rho_caller<<<tsph_blocks(ng, 256), 256, 0, ctx->stream>>>(ng, ctx->G.iord, ctx->S.rho, rho);
        else if (ctx->snapValid)
            k_rho_snap<<<tsph_blocks(ng, 256), 256, 0, ctx->stream>>>(ng, ctx->snapRho, rho);
    }
    if (!rc && ctx->n > 0) {
        RenderArgs A;
        A.n = ctx->n;
        A.ngas = ng;
        A.nStar = nStar;
        A.p = *rp;
        A.xlim = (rp->nxPix - 1) * .5;   // dfSetupFrame (dumpframe.c:259-261)
        A.ylim = (rp->nyPix - 1) * .5;
        A.hmul = 4 * sqrt(rp->x[0] * rp->x[0] + rp->x[1] * rp->x[1] + rp->x[2] * rp->x[2]);
        k_render_tsc<<<tsph_blocks(ctx->n, 128), 128, 0, ctx->stream>>>(A, ctx->C, ng > 0 ? rho : nullptr,
                                                                         img);
        if (cudaGetLastError() != cudaSuccess) rc = TSPH_ERR_CUDA;
        ctx->launches++;
    }
    if (!rc) {
        k_image_to_float<<<tsph_blocks((long long)npix, 256), 256, 0, ctx->stream>>>(npix, img, out);
        if (cudaMemcpyAsync(rgb, out, npix * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
            cudaStreamSynchronize(ctx->stream) != cudaSuccess)
            rc = TSPH_ERR_CUDA;
    }
    cudaStreamSynchronize(ctx->stream);
    if (img) cudaFree(img);
    if (out) cudaFree(out);
    if (rho) cudaFree(rho);
    return rc;
}
