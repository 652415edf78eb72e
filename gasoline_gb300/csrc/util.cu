// Measured arithmetic peaks of this GPU: a dependent-chain FMA
// microbenchmark (8 independent chains per thread on every SM) that gives
// the FP32 / FP64 FMA throughput the force kernels are compared against.
#include "tsph_ctx.cuh"

#define FMA_ITERS 2048
#define FMA_CHAINS 8

template <typename Real>
__global__ void k_fma(Real *out, Real a, Real b) {
    Real v[FMA_CHAINS];
#pragma unroll
    for (int c = 0; c < FMA_CHAINS; ++c) v[c] = (Real)(threadIdx.x + c);
    for (int it = 0; it < FMA_ITERS; ++it) {
#pragma unroll
        for (int c = 0; c < FMA_CHAINS; ++c) v[c] = v[c] * a + b;
    }
    Real s = 0;
#pragma unroll
    for (int c = 0; c < FMA_CHAINS; ++c) s += v[c];
    if (s == (Real)-1.2345) out[0] = s;   // keeps the chains live
}

extern "C" int tsph_fma_peak(tsph_ctx *ctx, int precision, double *tflops) {
    if (!ctx || !tflops) return TSPH_ERR_ARG;
    cudaSetDevice(ctx->device);
    const int threads = 256;
    const int blocks = ctx->smCount * 8;
    double best = 0.0;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(ctx->ev[0], ctx->stream);
        if (precision == TSPH_FP64)
            k_fma<double><<<blocks, threads, 0, ctx->stream>>>((double *)ctx->dRoot, 0.999999, 1e-7);
        else
            k_fma<float><<<blocks, threads, 0, ctx->stream>>>((float *)ctx->dRoot, 0.999999f, 1e-7f);
        TSPH_LAUNCH_CK("k_fma");
        cudaEventRecord(ctx->ev[1], ctx->stream);
        TSPH_CK(cudaEventSynchronize(ctx->ev[1]));
        float ms = 0;
        cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
        double flop = 2.0 * FMA_CHAINS * FMA_ITERS * (double)threads * blocks;
        double tf = flop / (ms * 1e-3) / 1e12;
        if (rep > 0 && tf > best) best = tf;
    }
    *tflops = best;
    return TSPH_OK;
}
