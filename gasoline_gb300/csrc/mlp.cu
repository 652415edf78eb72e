// K11: learned smoothing length (no counterpart in the reference).
//
// A 3 -> 32 -> 32 -> 1 tanh network, FP32, predicts for every gas particle
// t = log(fBall2_now) from
//   f0 = log(fBall2_prev)                       (last density pass)
//   f1 = (2/3) log(V_A / n_A)                   (deepest gas-tree cell A
//                                                holding >= nSmooth particles)
//   f2 = divv_prev                              (last density pass)
// The prediction, widened by a safety margin, seeds the kNN ball gather;
// a ball holding fewer than nSmooth particles grows and retries, so the
// neighbour set stays exact and the network only changes the speed.
//
// Training runs on the GPU with these kernels: one warp per sample, lane j
// owning hidden unit j of both layers (dot products through shuffles),
// per-warp gradient partials summed in a fixed order (deterministic), Adam.
// Inference (k_hnet_predict) runs one thread per particle.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include "tsph_ctx.cuh"

#define H HNET_H
#define OFF_W1 0
#define OFF_B1 (H * 3)
#define OFF_W2 (OFF_B1 + H)
#define OFF_B2 (OFF_W2 + H * H)
#define OFF_W3 (OFF_B2 + H)
#define OFF_B3 (OFF_W3 + H)
#define TRAIN_WARPS 1024

// forward + backward of one sample for this lane's hidden unit j;
// accumulates this lane's slice of the gradient into g (registers)
struct LaneGrad {
    float w1[3], b1, w2[H], b2, w3;
    float b3;   // lane 0 only
};

// W2T is W2 transposed (W2T[k*H + j] = W2[j*H + k]): lane j reads its row
// of W2 as a column of W2T, one bank per lane.
__device__ __forceinline__ float sample_fwd_bwd(const float *__restrict__ W,
                                                const float *__restrict__ W2T, const float *x,
                                                float y, int j, LaneGrad &g, bool backward) {
    const unsigned FULL = 0xffffffffu;
    // layer 1
    float z1 = W[OFF_B1 + j] + W[OFF_W1 + 3 * j] * x[0] + W[OFF_W1 + 3 * j + 1] * x[1] +
               W[OFF_W1 + 3 * j + 2] * x[2];
    float h1 = tanhf(z1);
    // layer 2: z2_j = b2_j + sum_k W2[j,k] h1_k
    float z2 = W[OFF_B2 + j];
#pragma unroll
    for (int k = 0; k < H; ++k) z2 += W2T[H * k + j] * __shfl_sync(FULL, h1, k);
    float h2 = tanhf(z2);
    // output
    float o = W[OFF_W3 + j] * h2;
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) o += __shfl_xor_sync(FULL, o, s);
    o += W[OFF_B3];
    float d = o - y;
    if (!backward) return o;
    // loss 0.5 d^2
    g.w3 += d * h2;
    if (j == 0) g.b3 += d;
    float dz2 = d * W[OFF_W3 + j] * (1.0f - h2 * h2);
    g.b2 += dz2;
#pragma unroll
    for (int k = 0; k < H; ++k) g.w2[k] += dz2 * __shfl_sync(FULL, h1, k);
    // dh1_j = sum_i W2[i,j] dz2_i
    float dh1 = 0.0f;
#pragma unroll
    for (int i = 0; i < H; ++i) dh1 += W[OFF_W2 + H * i + j] * __shfl_sync(FULL, dz2, i);
    float dz1 = dh1 * (1.0f - h1 * h1);
    g.b1 += dz1;
    g.w1[0] += dz1 * x[0];
    g.w1[1] += dz1 * x[1];
    g.w1[2] += dz1 * x[2];
    return o;
}

// per-warp partial gradients over samples [base, base+count) strided by warps
__global__ void __launch_bounds__(256) k_hnet_grad(const float *__restrict__ W,
                                                   const float *__restrict__ samples,
                                                   const long long *__restrict__ idx, long long n,
                                                   const float *__restrict__ st, float *partial,
                                                   float *lossp) {
    __shared__ float Ws[HNET_NP];
    __shared__ float W2T[H * H];
    for (int k = threadIdx.x; k < HNET_NP; k += blockDim.x) Ws[k] = W[k];
    for (int k = threadIdx.x; k < H * H; k += blockDim.x) W2T[(k % H) * H + k / H] = W[OFF_W2 + k];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    LaneGrad g;
    memset(&g, 0, sizeof(g));
    float loss = 0.0f;
    for (long long s = warp; s < n; s += nwarps) {
        long long r = idx ? idx[s] : s;
        const float *smp = samples + 4 * r;
        float x[3];
        x[0] = st ? (smp[0] - st[0]) / st[1] : smp[0];
        x[1] = st ? (smp[1] - st[2]) / st[3] : smp[1];
        x[2] = st ? (smp[2] - st[4]) / st[5] : smp[2];
        float y = st ? (smp[3] - st[6]) / st[7] : smp[3];
        float o = sample_fwd_bwd(Ws, W2T, x, y, lane, g, true);
        loss += 0.5f * (o - y) * (o - y);
    }
    float *P = partial + (size_t)warp * HNET_NP;
    P[OFF_W1 + 3 * lane] = g.w1[0];
    P[OFF_W1 + 3 * lane + 1] = g.w1[1];
    P[OFF_W1 + 3 * lane + 2] = g.w1[2];
    P[OFF_B1 + lane] = g.b1;
#pragma unroll
    for (int k = 0; k < H; ++k) P[OFF_W2 + H * lane + k] = g.w2[k];
    P[OFF_B2 + lane] = g.b2;
    P[OFF_W3 + lane] = g.w3;
    if (lane == 0) {
        P[OFF_B3] = g.b3;
        lossp[warp] = loss;
    }
}

// fixed-order sum of the per-warp partials, scaled by 1/n
__global__ void k_hnet_reduce(const float *__restrict__ partial, int nwarps, float scale,
                              float *grad, const float *__restrict__ lossp, float *lossOut) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < HNET_NP) {
        float s = 0.0f;
        for (int w = 0; w < nwarps; ++w) s += partial[(size_t)w * HNET_NP + k];
        grad[k] = s * scale;
    }
    if (k == HNET_NP) {
        float s = 0.0f;
        for (int w = 0; w < nwarps; ++w) s += lossp[w];
        lossOut[0] = s * scale;
    }
}

__global__ void k_adam(float *W, const float *__restrict__ grad, float *m1, float *m2, float lr,
                       float b1t, float b2t) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= HNET_NP) return;
    const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
    float gk = grad[k];
    float a = beta1 * m1[k] + (1 - beta1) * gk;
    float b = beta2 * m2[k] + (1 - beta2) * gk * gk;
    m1[k] = a;
    m2[k] = b;
    float ah = a / (1 - b1t), bh = b / (1 - b2t);
    W[k] -= lr * ah / (sqrtf(bh) + eps);
}

// Features of every gas particle of the current density pass (gas-tree
// order): f0, f1, f2 as described at the top of this file.
__global__ void k_hnet_features(int ng, int k, TsphDevTree T, const int *__restrict__ iord,
                                const int *__restrict__ rid, const double *__restrict__ fb2prev,
                                const double *__restrict__ divvprev, float *feat) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ng) return;
    int node = T.sysRoot[rid[i]];
    for (;;) {
        int up = T.upper[node];
        if (up < 0) break;
        int child = (i >= T.pLower[up]) ? up : node + 1;
        if (T.pUpper[child] - T.pLower[child] + 1 < k) break;
        node = child;
    }
    const double *b = &T.bnd[6 * node];
    double vol = 1.0;
    for (int a = 0; a < 3; ++a) vol *= fmax(b[3 + a] - b[a], 1e-12);
    double nA = T.pUpper[node] - T.pLower[node] + 1;
    int o = iord[i];
    double f0 = fb2prev[o] > 0 ? log(fb2prev[o]) : 0.0;
    feat[3 * i] = (float)f0;
    feat[3 * i + 1] = (float)((2.0 / 3.0) * log(vol / nA));
    feat[3 * i + 2] = (float)divvprev[o];
}

// seed fBall2 = exp(t_pred + 2*margin) for the kNN ball gather.
// Inference runs one thread per particle: every thread reads the same
// weight at the same time, a shared-memory broadcast (the warp-per-sample
// form of training reads a row of W2 per lane, which conflicts).
__global__ void __launch_bounds__(256) k_hnet_predict(int ng, const float *__restrict__ W,
                                                      const float *__restrict__ feat,
                                                      const float *__restrict__ st, double margin,
                                                      double *seed) {
    __shared__ float Ws[HNET_NP];
    for (int k = threadIdx.x; k < HNET_NP; k += blockDim.x) Ws[k] = W[k];
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ng; i += gridDim.x * blockDim.x) {
        const float *f = feat + 3 * i;
        const float x0 = (f[0] - st[0]) / st[1];
        const float x1 = (f[1] - st[2]) / st[3];
        const float x2 = (f[2] - st[4]) / st[5];
        float h1[H];
#pragma unroll
        for (int j = 0; j < H; ++j)
            h1[j] = tanhf(Ws[OFF_B1 + j] + Ws[OFF_W1 + 3 * j] * x0 + Ws[OFF_W1 + 3 * j + 1] * x1 +
                          Ws[OFF_W1 + 3 * j + 2] * x2);
        float o = 0.0f;
#pragma unroll 4
        for (int j = 0; j < H; ++j) {
            float z2 = Ws[OFF_B2 + j];
#pragma unroll
            for (int k = 0; k < H; ++k) z2 += Ws[OFF_W2 + H * j + k] * h1[k];
            o += Ws[OFF_W3 + j] * tanhf(z2);
        }
        o += Ws[OFF_B3];
        const double t = (double)o * st[7] + st[6];
        seed[i] = exp(t + 2.0 * margin);
    }
}

// append (features, target) of this pass to the sample buffer
__global__ void k_hnet_append(int ng, const float *__restrict__ feat, const double *__restrict__ fBall2,
                              float *samples, long long base) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ng) return;
    float *s = samples + 4 * (base + i);
    s[0] = feat[3 * i];
    s[1] = feat[3 * i + 1];
    s[2] = feat[3 * i + 2];
    s[3] = (float)log(fBall2[i]);
}

// mean and std of the 4 sample columns (fixed-order reduction, one block)
__global__ void k_hnet_stats(const float *__restrict__ samples, long long n, float *st) {
    __shared__ double acc[8][256];
    double s[4] = {0, 0, 0, 0}, q[4] = {0, 0, 0, 0};
    for (long long r = threadIdx.x; r < n; r += blockDim.x)
        for (int c = 0; c < 4; ++c) {
            double v = samples[4 * r + c];
            s[c] += v;
            q[c] += v * v;
        }
    for (int c = 0; c < 4; ++c) { acc[c][threadIdx.x] = s[c]; acc[4 + c][threadIdx.x] = q[c]; }
    __syncthreads();
    if (threadIdx.x < 8) {
        double t = 0;
        for (int k = 0; k < 256; ++k) t += acc[threadIdx.x][k];
        acc[threadIdx.x][0] = t;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        int c = threadIdx.x;
        double mean = acc[c][0] / (double)n;
        double var = acc[4 + c][0] / (double)n - mean * mean;
        st[2 * c] = (float)mean;
        st[2 * c + 1] = (float)sqrt(var > 1e-12 ? var : 1e-12);
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static int hnet_alloc(tsph_ctx *ctx) {
    TsphHnet &Hn = ctx->hnet;
    if (Hn.W) return TSPH_OK;
    int rc = 0;
    rc |= tsph_grow(ctx, &Hn.W, HNET_NP);
    rc |= tsph_grow(ctx, &Hn.grad, HNET_NP);
    rc |= tsph_grow(ctx, &Hn.m1, HNET_NP);
    rc |= tsph_grow(ctx, &Hn.m2, HNET_NP);
    rc |= tsph_grow(ctx, &Hn.partial, (size_t)TRAIN_WARPS * HNET_NP);
    rc |= tsph_grow(ctx, &Hn.loss, TRAIN_WARPS + 8 + 16);
    return rc ? TSPH_ERR_NOMEM : TSPH_OK;
}

void tsph_hnet_free(tsph_ctx *ctx) {
    TsphHnet &Hn = ctx->hnet;
    float **ps[] = {&Hn.W, &Hn.grad, &Hn.m1, &Hn.m2, &Hn.partial, &Hn.loss, &Hn.feat, &Hn.samples};
    for (auto p : ps) {
        if (*p) cudaFree(*p);
        *p = nullptr;
    }
}

extern "C" int tsph_hnet_init(tsph_ctx *ctx, unsigned long long seed) {
    if (!ctx) return TSPH_ERR_ARG;
    cudaSetDevice(ctx->device);
    int rc = hnet_alloc(ctx);
    if (rc) return rc;
    // Xavier-uniform initialisation from a splitmix64 stream
    float h[HNET_NP];
    unsigned long long st = seed * 0x9E3779B97F4A7C15ULL + 1;
    auto uni = [&st]() {
        st += 0x9E3779B97F4A7C15ULL;
        unsigned long long z = st;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0);
    };
    for (int k = 0; k < HNET_NP; ++k) h[k] = 0.0f;
    double a1 = sqrt(6.0 / (3 + H)), a2 = sqrt(6.0 / (H + H)), a3 = sqrt(6.0 / (H + 1));
    for (int k = 0; k < 3 * H; ++k) h[OFF_W1 + k] = (float)((2 * uni() - 1) * a1);
    for (int k = 0; k < H * H; ++k) h[OFF_W2 + k] = (float)((2 * uni() - 1) * a2);
    for (int k = 0; k < H; ++k) h[OFF_W3 + k] = (float)((2 * uni() - 1) * a3);
    TSPH_CK(cudaMemcpy(ctx->hnet.W, h, sizeof(h), cudaMemcpyHostToDevice));
    TSPH_CK(cudaMemset(ctx->hnet.m1, 0, sizeof(float) * HNET_NP));
    TSPH_CK(cudaMemset(ctx->hnet.m2, 0, sizeof(float) * HNET_NP));
    ctx->hnet.init = true;
    ctx->hnet.trained = false;
    ctx->hnet.adamStep = 0;
    return TSPH_OK;
}

extern "C" int tsph_hnet_num_params(void) { return HNET_NP; }

extern "C" int tsph_hnet_set_params(tsph_ctx *ctx, const float *params, int n) {
    if (!ctx || !params || n != HNET_NP) return TSPH_ERR_ARG;
    cudaSetDevice(ctx->device);
    int rc = hnet_alloc(ctx);
    if (rc) return rc;
    TSPH_CK(cudaMemcpy(ctx->hnet.W, params, sizeof(float) * HNET_NP, cudaMemcpyHostToDevice));
    ctx->hnet.init = true;
    return TSPH_OK;
}

extern "C" int tsph_hnet_get_params(tsph_ctx *ctx, float *params, int n) {
    if (!ctx || !params || n != HNET_NP) return TSPH_ERR_ARG;
    if (!ctx->hnet.init) return TSPH_ERR_STATE;
    cudaSetDevice(ctx->device);
    TSPH_CK(cudaMemcpy(params, ctx->hnet.W, sizeof(float) * HNET_NP, cudaMemcpyDeviceToHost));
    return TSPH_OK;
}

static int grad_on(tsph_ctx *ctx, const float *samples, const long long *idx, long long n,
                   const float *st, float *lossHost) {
    TsphHnet &Hn = ctx->hnet;
    const int threads = 256, blocks = TRAIN_WARPS * 32 / threads;
    k_hnet_grad<<<blocks, threads, 0, ctx->stream>>>(Hn.W, samples, idx, n, st, Hn.partial, Hn.loss);
    TSPH_LAUNCH_CK("k_hnet_grad");
    k_hnet_reduce<<<tsph_blocks(HNET_NP + 1, 128), 128, 0, ctx->stream>>>(
        Hn.partial, TRAIN_WARPS, 1.0f / (float)n, Hn.grad, Hn.loss, Hn.loss + TRAIN_WARPS);
    TSPH_LAUNCH_CK("k_hnet_reduce");
    if (lossHost) {
        TSPH_CK(cudaMemcpyAsync(lossHost, Hn.loss + TRAIN_WARPS, sizeof(float), cudaMemcpyDeviceToHost,
                                ctx->stream));
        TSPH_CK(cudaStreamSynchronize(ctx->stream));
    }
    return TSPH_OK;
}

// Loss 0.5 mean((net(x) - y)^2) and its gradient on caller-provided
// (already normalised) samples: x[3n], y[n].  For gradient checks.
extern "C" int tsph_hnet_loss_grad(tsph_ctx *ctx, int n, const float *x3, const float *y,
                                   float *grad, double *loss) {
    if (!ctx || n <= 0 || !x3 || !y || !grad) return TSPH_ERR_ARG;
    if (!ctx->hnet.init) return TSPH_ERR_STATE;
    cudaSetDevice(ctx->device);
    float *buf = nullptr;
    if (cudaMalloc((void **)&buf, sizeof(float) * 4 * (size_t)n) != cudaSuccess) return TSPH_ERR_NOMEM;
    float *hs = (float *)malloc(sizeof(float) * 4 * (size_t)n);
    for (int i = 0; i < n; ++i) {
        hs[4 * i] = x3[3 * i];
        hs[4 * i + 1] = x3[3 * i + 1];
        hs[4 * i + 2] = x3[3 * i + 2];
        hs[4 * i + 3] = y[i];
    }
    int rc = TSPH_OK;
    if (cudaMemcpy(buf, hs, sizeof(float) * 4 * n, cudaMemcpyHostToDevice) != cudaSuccess) rc = TSPH_ERR_CUDA;
    float l = 0;
    if (!rc) rc = grad_on(ctx, buf, nullptr, n, nullptr, &l);
    if (!rc && cudaMemcpy(grad, ctx->hnet.grad, sizeof(float) * HNET_NP, cudaMemcpyDeviceToHost) != cudaSuccess)
        rc = TSPH_ERR_CUDA;
    if (loss) *loss = l;
    cudaFree(buf);
    free(hs);
    return rc;
}

// collect: append this pass's samples; predict: seed the next passes
extern "C" int tsph_hnet_mode(tsph_ctx *ctx, int collect, int predict, double margin) {
    if (!ctx) return TSPH_ERR_ARG;
    if (predict && !ctx->hnet.trained) return TSPH_ERR_STATE;
    ctx->hnet.collect = collect != 0;
    ctx->hnet.predict = predict != 0;
    ctx->hnet.margin = margin;
    ctx->sysVersion++;   // a captured step graph seeds (or not) as the mode was
    return TSPH_OK;
}

int tsph_hnet_features(tsph_ctx *ctx, int k) {
    TsphHnet &Hn = ctx->hnet;
    const int ng = ctx->ngas;
    if (!(Hn.collect || Hn.predict) || !Hn.havePrev || ng == 0) return TSPH_OK;
    if (!Hn.feat || (size_t)ng > (size_t)Hn.featCap) {
        if (ctx->capturing) return TSPH_ERR_STATE;   // no allocation inside a capture
        int rc = tsph_grow(ctx, &Hn.feat, (size_t)3 * ctx->S.cap);
        if (rc) { Hn.featCap = 0; return rc; }
        Hn.featCap = ctx->S.cap;
    }
    k_hnet_features<<<tsph_blocks(ng, 256), 256, 0, ctx->stream>>>(ng, k, ctx->TG, ctx->G.iord,
                                                                  ctx->G.rid, ctx->C.fb2prev,
                                                                  ctx->C.divvprev, Hn.feat);
    TSPH_LAUNCH_CK("k_hnet_features");
    return TSPH_OK;
}

int tsph_hnet_seed(tsph_ctx *ctx) {
    TsphHnet &Hn = ctx->hnet;
    const int ng = ctx->ngas;
    ctx->S.haveSeed = false;
    if (!Hn.predict || !Hn.trained || !Hn.havePrev || ng == 0) return TSPH_OK;
    float *st = Hn.loss + TRAIN_WARPS + 8;   // device copy of the stats
    k_hnet_predict<<<ctx->smCount * 4, 256, 0, ctx->stream>>>(ng, Hn.W, Hn.feat, st, Hn.margin,
                                                             ctx->S.seed);
    TSPH_LAUNCH_CK("k_hnet_predict");
    ctx->S.haveSeed = true;
    return TSPH_OK;
}

int tsph_hnet_append(tsph_ctx *ctx) {
    TsphHnet &Hn = ctx->hnet;
    const int ng = ctx->ngas;
    if (!Hn.collect || !Hn.havePrev || ng == 0) return TSPH_OK;
    if (Hn.nSamples + ng > Hn.capSamples) {
        long long cap = (Hn.nSamples + ng) * 2 + 1024;
        float *nb = nullptr;
        if (cudaMalloc((void **)&nb, sizeof(float) * 4 * (size_t)cap) != cudaSuccess) return TSPH_ERR_NOMEM;
        if (Hn.samples) {
            TSPH_CK(cudaMemcpyAsync(nb, Hn.samples, sizeof(float) * 4 * (size_t)Hn.nSamples,
                                    cudaMemcpyDeviceToDevice, ctx->stream));
            TSPH_CK(cudaStreamSynchronize(ctx->stream));
            cudaFree(Hn.samples);
        }
        Hn.samples = nb;
        Hn.capSamples = cap;
    }
    k_hnet_append<<<tsph_blocks(ng, 256), 256, 0, ctx->stream>>>(ng, Hn.feat, ctx->S.fBall2,
                                                                Hn.samples, Hn.nSamples);
    TSPH_LAUNCH_CK("k_hnet_append");
    Hn.nSamples += ng;
    return TSPH_OK;
}

__global__ void k_perm_batch(long long n, long long off, int b, unsigned long long seed,
                             long long *idx) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= b) return;
    unsigned long long z = seed + (unsigned long long)(off + t) * 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    idx[t] = (long long)(z % (unsigned long long)n);
}

// Train on the collected samples: `steps` Adam steps of `batch` random
// samples each (with replacement).  Returns the final full-data loss.
extern "C" int tsph_hnet_train(tsph_ctx *ctx, int steps, int batch, double lr, double *loss) {
    if (!ctx || steps < 0 || batch <= 0) return TSPH_ERR_ARG;
    TsphHnet &Hn = ctx->hnet;
    if (!Hn.init || Hn.nSamples < 16) return TSPH_ERR_STATE;
    cudaSetDevice(ctx->device);
    float *st = Hn.loss + TRAIN_WARPS + 8;
    if (!Hn.statsReady) {
        k_hnet_stats<<<1, 256, 0, ctx->stream>>>(Hn.samples, Hn.nSamples, st);
        TSPH_LAUNCH_CK("k_hnet_stats");
        TSPH_CK(cudaMemcpyAsync(Hn.stats, st, sizeof(float) * 8, cudaMemcpyDeviceToHost, ctx->stream));
        TSPH_CK(cudaStreamSynchronize(ctx->stream));
        Hn.statsReady = true;
    }
    long long *idx = nullptr;
    if (cudaMalloc((void **)&idx, sizeof(long long) * (size_t)batch) != cudaSuccess) return TSPH_ERR_NOMEM;
    int rc = TSPH_OK;
    for (int s = 0; s < steps && !rc; ++s) {
        k_perm_batch<<<tsph_blocks(batch, 256), 256, 0, ctx->stream>>>(
            Hn.nSamples, (long long)Hn.adamStep * batch, batch, 0x1234567ULL, idx);
        ctx->launches++;
        rc = grad_on(ctx, Hn.samples, idx, batch, st, nullptr);
        if (rc) break;
        Hn.adamStep++;
        float b1t = (float)pow(0.9, (double)Hn.adamStep), b2t = (float)pow(0.999, (double)Hn.adamStep);
        k_adam<<<tsph_blocks(HNET_NP, 256), 256, 0, ctx->stream>>>(Hn.W, Hn.grad, Hn.m1, Hn.m2,
                                                                  (float)lr, b1t, b2t);
        ctx->launches++;
    }
    cudaFree(idx);
    if (rc) return rc;
    float l = 0;
    rc = grad_on(ctx, Hn.samples, nullptr, Hn.nSamples, st, &l);
    if (loss) *loss = l;
    Hn.trained = true;
    return rc;
}

extern "C" int tsph_hnet_info(tsph_ctx *ctx, long long *nSamples, float *stats8) {
    if (!ctx) return TSPH_ERR_ARG;
    if (nSamples) *nSamples = ctx->hnet.nSamples;
    if (stats8) memcpy(stats8, ctx->hnet.stats, sizeof(float) * 8);
    return TSPH_OK;
}
