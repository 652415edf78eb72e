// Allocation-free loss/gradient of the learned smoothing-length network.
//
// Some callers cannot allocate device memory at the point where they need
// the h-network gradient: a host code that reserves all of its device
// memory up front (as the reference does through its own allocator) and
// updates the network inside its time-step loop, where a cudaMalloc would
// synchronise the whole device and stall the other streams of the step, or
// fail against a fixed per-process memory budget.  tsph_hnet_loss_grad_noalloc
// serves them: it takes device pointers for every input and output and keeps
// its per-warp scratch in one file-scope device array of fixed size.
//
// The scratch array (HNA_MAX_WARPS partial gradients + partial losses,
// about 2.5 MB) is created with the library and held by every GPU that
// loads it until the process exits.  All calls share it: each call
// overwrites every partial it later reads (the partials of warps 0..nwarps-1,
// whatever a larger earlier call left beyond them), so nothing needs
// clearing, but calls that overlap on the GPU (two streams, or two host
// threads) race on it and must be serialised by the caller.
#include <stdio.h>

#include "tsph_ctx.cuh"

#define HNA_H HNET_H
#define HNA_SAMPLES_PER_WARP 32
#define HNA_MAX_WARPS 512
#define HNA_MAX_SAMPLES (HNA_MAX_WARPS * HNA_SAMPLES_PER_WARP)

static_assert(HNA_MAX_SAMPLES == TSPH_HNET_NOALLOC_MAX_SAMPLES, "header limit");

// partial gradients of up to HNA_MAX_WARPS warps, then their partial losses
static __device__ __align__(256) float g_hna_scratch[HNA_MAX_WARPS * HNET_NP + HNA_MAX_WARPS];


// One sample, one warp: lane j owns hidden unit j of both layers.  Same
// network and loss (0.5 (out - y)^2) as the allocating path.
struct HnaGrad {
    float w1[3], b1, w2[HNA_H], b2, w3, b3;
};

__device__ __forceinline__ float hna_sample(const float *__restrict__ W, const float *x, float y,
                                            int j, HnaGrad &g) {
    const unsigned FULL = 0xffffffffu;
    const int oB1 = HNA_H * 3, oW2 = oB1 + HNA_H, oB2 = oW2 + HNA_H * HNA_H, oW3 = oB2 + HNA_H,
              oB3 = oW3 + HNA_H;
    float h1 = tanhf(W[oB1 + j] + W[3 * j] * x[0] + W[3 * j + 1] * x[1] + W[3 * j + 2] * x[2]);
    float z2 = W[oB2 + j];
#pragma unroll
    for (int k = 0; k < HNA_H; ++k) z2 += W[oW2 + HNA_H * j + k] * __shfl_sync(FULL, h1, k);
    float h2 = tanhf(z2);
    float o = W[oW3 + j] * h2;
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) o += __shfl_xor_sync(FULL, o, s);
    o += W[oB3];
    float d = o - y;
    g.w3 += d * h2;
    if (j == 0) g.b3 += d;
    float dz2 = d * W[oW3 + j] * (1.0f - h2 * h2);
    g.b2 += dz2;
#pragma unroll
    for (int k = 0; k < HNA_H; ++k) g.w2[k] += dz2 * __shfl_sync(FULL, h1, k);
    float dh1 = 0.0f;
#pragma unroll
    for (int i = 0; i < HNA_H; ++i) dh1 += W[oW2 + HNA_H * i + j] * __shfl_sync(FULL, dz2, i);
    float dz1 = dh1 * (1.0f - h1 * h1);
    g.b1 += dz1;
    g.w1[0] += dz1 * x[0];
    g.w1[1] += dz1 * x[1];
    g.w1[2] += dz1 * x[2];
    return 0.5f * d * d;
}

// per-warp partial gradient and loss into the scratch array
__global__ void __launch_bounds__(256) k_hna_partial(const float *__restrict__ W,
                                                     const float *__restrict__ x3,
                                                     const float *__restrict__ y, int n, int nwarps,
                                                     float *scratch) {
    __shared__ float Ws[HNET_NP];
    for (int k = threadIdx.x; k < HNET_NP; k += blockDim.x) Ws[k] = W[k];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (warp >= nwarps) return;
    HnaGrad g;
    memset(&g, 0, sizeof(g));
    float loss = 0.0f;
    for (int s = warp; s < n; s += nwarps) {
        float x[3] = {x3[3 * s], x3[3 * s + 1], x3[3 * s + 2]};
        loss += hna_sample(Ws, x, y[s], lane, g);
    }
    const int oB1 = HNA_H * 3, oW2 = oB1 + HNA_H, oB2 = oW2 + HNA_H * HNA_H, oW3 = oB2 + HNA_H,
              oB3 = oW3 + HNA_H;
    float *P = scratch + (size_t)warp * HNET_NP;
    P[3 * lane] = g.w1[0];
    P[3 * lane + 1] = g.w1[1];
    P[3 * lane + 2] = g.w1[2];
    P[oB1 + lane] = g.b1;
#pragma unroll
    for (int k = 0; k < HNA_H; ++k) P[oW2 + HNA_H * lane + k] = g.w2[k];
    P[oB2 + lane] = g.b2;
    P[oW3 + lane] = g.w3;
    if (lane == 0) {
        P[oB3] = g.b3;
        scratch[(size_t)HNA_MAX_WARPS * HNET_NP + warp] = loss;
    }
}

// fixed-order sum of the partials into the caller's outputs, scaled by 1/n
__global__ void k_hna_reduce(const float *__restrict__ scratch, int nwarps, float scale,
                             float *grad, float *lossOut) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < HNET_NP) {
        float s = 0.0f;
        for (int w = 0; w < nwarps; ++w) s += scratch[(size_t)w * HNET_NP + k];
        grad[k] = s * scale;
    }
    if (k == HNET_NP) {
        float s = 0.0f;
        for (int w = 0; w < nwarps; ++w) s += scratch[(size_t)HNA_MAX_WARPS * HNET_NP + w];
        lossOut[0] = s * scale;
    }
}

// The scratch array's device address in the calling thread's current
// context.  The symbol's name is only a host stand-in; its device address
// comes from cudaGetSymbolAddress with the device current.  It is looked up
// on every call rather than cached per device ordinal: the address belongs
// to one context, and a device reset or a caller-made context on the same
// device places the array elsewhere.  The lookup is host-side and does not
// touch the stream; the first one on a device loads the library's device
// code there, which is why that first call must come before any stream
// capture.
static int hna_scratch_address(float **ptr) {
    float *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void **)&p, g_hna_scratch);
    if (e != cudaSuccess || !p) return TSPH_ERR_CUDA;
    *ptr = p;
    return TSPH_OK;
}

extern "C" int tsph_hnet_loss_grad_noalloc(const float *params, int n, const float *x3,
                                           const float *y, float *grad, float *loss,
                                           void *stream) {
    if (!params || !x3 || !y || !grad || !loss || n <= 0) return TSPH_ERR_ARG;
    if (n > HNA_MAX_SAMPLES) return TSPH_ERR_ARG;   // more samples than the fixed scratch holds
    float *scratch = nullptr;
    int rc = hna_scratch_address(&scratch);
    if (rc) return rc;
    // an error left by earlier, unrelated work (not a sticky one, which
    // would fail the launches below as well) is cleared here, so the checks
    // after the launches report this call's own
    (void)cudaGetLastError();
    cudaStream_t s = (cudaStream_t)stream;
    int nwarps = (n + HNA_SAMPLES_PER_WARP - 1) / HNA_SAMPLES_PER_WARP;
    int blocks = (nwarps * 32 + 255) / 256;
    k_hna_partial<<<blocks, 256, 0, s>>>(params, x3, y, n, nwarps, scratch);
    if (cudaGetLastError() != cudaSuccess) return TSPH_ERR_CUDA;
    k_hna_reduce<<<(HNET_NP + 1 + 127) / 128, 128, 0, s>>>(scratch, nwarps, 1.0f / (float)n, grad,
                                                            loss);
    if (cudaGetLastError() != cudaSuccess) return TSPH_ERR_CUDA;
    return TSPH_OK;
}
