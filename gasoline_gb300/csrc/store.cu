// The reference's particle store read and written where it lies.
//
// The reference keeps its particles as one array of PARTICLE structs
// (pkd.h:90-225, pkd->pStore) and its per-rank kernels read and write their
// fields in place: pkdGravAll adds a[], fPot and the dtGrav maximum of the
// active particles (grav.c:101-239, ewald.c:165), the DenDVDX pass sets
// fBall2, fDensity and the velocity-gradient fields (smoothfcn.c:3390-3627),
// pkdGasPressure sets PoverRho2 and c (pkd.c:5690-5785), and the pressure
// pass adds the hydro acceleration into a[] and sets uDotPdV, uDotAV, mumax
// and lowers dtNew (smoothfcn.c:2276-2385).  These entry points do the same
// from a caller-described layout (stride and byte offsets), so a binding
// compiled against the reference's pkd.h needs no packing loop of its own.
//
// GB300 mapping: a store the caller registered with CUDA (pinned and
// mapped; on Grace the GPU reaches it coherently over NVLink-C2C) is read
// and written in place by the unpack and write-back kernels, one particle
// per thread, only the fields named.  An unregistered store is copied to
// the device in one block for the unpack, and results are added into it by
// a host loop over the compact arrays.
#include <stdlib.h>
#include <string.h>

#include "tsph_ctx.cuh"

__device__ __forceinline__ double st_ld(const char *b, int off) {
    return *reinterpret_cast<const double *>(b + off);
}
__device__ __forceinline__ double *st_at(char *b, int off) {
    return reinterpret_cast<double *>(b + off);
}

// Positions into the interleaved staging array (for k_load_state) or
// straight into the caller-order state (update of a loaded set).
__global__ void k_store_pos(int n, const char *__restrict__ store, long long stride, int offR,
                            const int *__restrict__ order, double *pos3, TsphDevState C, int update) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const char *b = store + (long long)(order ? order[i] : i) * stride;
    const double x = st_ld(b, offR), y = st_ld(b, offR + 8), z = st_ld(b, offR + 16);
    if (update) {
        C.x[i] = x;
        C.y[i] = y;
        C.z[i] = z;
    } else {
        pos3[3 * i] = x;
        pos3[3 * i + 1] = y;
        pos3[3 * i + 2] = z;
    }
}

// Mass, softening, velocities, gas energies and the active flag.  A store
// without vPred (or uPred) predicts them as v (u), as tsph_set_velocities
// does.  Active particles go to rung 1, the others to rung 0.
__global__ void k_store_rest(int n, int ngas, const char *__restrict__ store, long long stride,
                             tsph_store_layout L, const int *__restrict__ order, TsphDevState C,
                             int loadVel) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const char *b = store + (long long)(order ? order[i] : i) * stride;
    C.m[i] = st_ld(b, L.fMass);
    C.h[i] = st_ld(b, L.fSoft);
    if (loadVel) {
        const double vx = st_ld(b, L.v), vy = st_ld(b, L.v + 8), vz = st_ld(b, L.v + 16);
        C.vx[i] = vx;
        C.vy[i] = vy;
        C.vz[i] = vz;
        const bool vp = i < ngas && L.vPred >= 0;
        C.vpx[i] = vp ? st_ld(b, L.vPred) : vx;
        C.vpy[i] = vp ? st_ld(b, L.vPred + 8) : vy;
        C.vpz[i] = vp ? st_ld(b, L.vPred + 16) : vz;
        if (i < ngas) {
            const double u = L.u >= 0 ? st_ld(b, L.u) : 0.0;
            C.u[i] = u;
            C.upred[i] = L.uPred >= 0 ? st_ld(b, L.uPred) : u;
        }
    }
    if (L.iActive >= 0) {
        const unsigned a = *reinterpret_cast<const unsigned *>(b + L.iActive);
        C.rung[i] = (a & L.activeBit) ? 1 : 0;
    }
}

// pkdGravAll's accumulation into the store for the active particles.
__global__ void k_store_put_grav(int n, char *store, long long stride, tsph_store_layout L,
                                 const int *__restrict__ order, TsphDevState C, int actRung) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || C.rung[i] < actRung) return;
    char *b = store + (long long)(order ? order[i] : i) * stride;
    if (L.a >= 0) {
        *st_at(b, L.a) += C.ax[i];
        *st_at(b, L.a + 8) += C.ay[i];
        *st_at(b, L.a + 16) += C.az[i];
    }
    if (L.fPot >= 0) *st_at(b, L.fPot) += C.pot[i];
    if (L.dtGrav >= 0) {
        double *d = st_at(b, L.dtGrav);
        if (C.dtGrav[i] > *d) *d = C.dtGrav[i];
    }
}

struct StoreSph {
    const double *fBall2, *rho, *divv, *curl, *dvds, *bal, *diff;    // density pass
    const double *pr2, *cs, *hax, *hay, *haz, *uPdV, *uAV, *dtNew, *mumax;   // pressure pass
};

// SPH results (gas-tree slot g holds caller particle G.iord[g]) into the
// store: the density fields, or the pressure pass's (hydro acceleration
// added into a[], dtNew lowered, the rest set) for the active particles.
__global__ void k_store_put_sph(int ng, char *store, long long stride, tsph_store_layout L,
                                const int *__restrict__ order, const int *__restrict__ giord,
                                StoreSph S, TsphDevState C, int which, int actRung) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ng) return;
    const int c = giord[g];
    char *b = store + (long long)(order ? order[c] : c) * stride;
    if (which == TSPH_SMX_SPHPRESSURETERMS) {
        if (C.rung[c] < actRung) return;
        if (L.PoverRho2 >= 0) *st_at(b, L.PoverRho2) = S.pr2[g];
        if (L.c >= 0) *st_at(b, L.c) = S.cs[g];
        if (L.a >= 0) {
            *st_at(b, L.a) += S.hax[g];
            *st_at(b, L.a + 8) += S.hay[g];
            *st_at(b, L.a + 16) += S.haz[g];
        }
        if (L.uDotPdV >= 0) *st_at(b, L.uDotPdV) = S.uPdV[g];
        if (L.uDotAV >= 0) *st_at(b, L.uDotAV) = S.uAV[g];
        if (L.mumax >= 0) *st_at(b, L.mumax) = S.mumax[g];
        if (L.dtNew >= 0) {
            double *d = st_at(b, L.dtNew);
            if (S.dtNew[g] < *d) *d = S.dtNew[g];
        }
        return;
    }
    if (L.fBall2 >= 0) *st_at(b, L.fBall2) = S.fBall2[g];
    if (L.fDensity >= 0) *st_at(b, L.fDensity) = S.rho[g];
    if (L.divv >= 0) *st_at(b, L.divv) = S.divv[g];
    if (L.curlv >= 0) {
        *st_at(b, L.curlv) = S.curl[3 * g];
        *st_at(b, L.curlv + 8) = S.curl[3 * g + 1];
        *st_at(b, L.curlv + 16) = S.curl[3 * g + 2];
    }
    if (L.dvds >= 0) *st_at(b, L.dvds) = S.dvds[g];
    if (L.BalsaraSwitch >= 0) *st_at(b, L.BalsaraSwitch) = S.bal[g];
    if (L.diff >= 0) *st_at(b, L.diff) = S.diff[g];
}

// Every field inside the stride, doubles on 8-byte boundaries (the kernels
// load them as doubles), the active word on a 4-byte one.
static bool layout_ok(const tsph_store_layout *L) {
    if (!L || L->stride < 8 || L->stride % 8) return false;
    const int need[3] = {L->r, L->fMass, L->fSoft};
    for (int k = 0; k < 3; ++k)
        if (need[k] < 0 || need[k] % 8 || need[k] + 8 > L->stride) return false;
    if (L->r + 24 > L->stride) return false;
    const int opt[] = {L->v, L->vPred, L->u, L->uPred, L->a, L->fPot, L->dtGrav, L->fBall2,
                       L->fDensity, L->divv, L->curlv, L->dvds, L->BalsaraSwitch, L->diff,
                       L->PoverRho2, L->c, L->uDotPdV, L->uDotAV, L->mumax, L->dtNew};
    const int width[] = {24, 24, 8, 8, 24, 8, 8, 8, 8, 8, 24, 8, 8, 8, 8, 8, 8, 8, 8, 8};
    for (size_t k = 0; k < sizeof(opt) / sizeof(opt[0]); ++k)
        if (opt[k] >= 0 && (opt[k] % 8 || opt[k] + width[k] > L->stride)) return false;
    if (L->iActive >= 0 && (L->iActive % 4 || L->iActive + 4 > L->stride)) return false;
    return true;
}

static bool aligned(const void *p) { return ((size_t)p & 7) == 0; }

// A device-readable address of the store: in place when the caller
// registered it (pinned and mapped), else null.
static const char *mapped(const void *store) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, store) != cudaSuccess) {
        (void)cudaGetLastError();   // pageable memory on older runtimes
        return nullptr;
    }
    if (at.type != cudaMemoryTypeHost || !at.devicePointer) return nullptr;
    return reinterpret_cast<const char *>(at.devicePointer);
}

// A load is an update of the loaded particles when the store, n and ngas
// are those of the last load: caller index c names the same particle, even
// though the store's own order may have changed (the reference permutes its
// store at every tree build; the order array follows it).
static unsigned long long store_key(int n, int ngas, const void *store) {
    unsigned long long h = 1469598103934665603ULL ^ (unsigned long long)(size_t)store;
    h = (h ^ (unsigned long long)(unsigned)n) * 1099511628211ULL;
    return (h ^ (unsigned long long)(unsigned)ngas) * 1099511628211ULL;
}

extern "C" int tsph_store_register(tsph_ctx *ctx, void *store, size_t bytes) {
    if (!ctx || !store || bytes == 0) return TSPH_ERR_ARG;
    cudaSetDevice(ctx->device);
    TSPH_CK(cudaHostRegister(store, bytes, cudaHostRegisterMapped));
    return TSPH_OK;
}

extern "C" int tsph_store_unregister(tsph_ctx *ctx, void *store) {
    if (!ctx || !store) return TSPH_ERR_ARG;
    cudaSetDevice(ctx->device);
    TSPH_CK(cudaStreamSynchronize(ctx->stream));
    TSPH_CK(cudaHostUnregister(store));
    return TSPH_OK;
}

extern "C" int tsph_store_load(tsph_ctx *ctx, int n, const void *store, const tsph_store_layout *L,
                               const int *order, int ngas) {
    if (!ctx || n < 0 || (n > 0 && !store) || !layout_ok(L) || ngas < 0 || ngas > n ||
        !aligned(store))
        return TSPH_ERR_ARG;
    if (ctx->capturing) return TSPH_ERR_STATE;
    if (order)   // store entries 0..n-1, each named once by the caller
        for (int i = 0; i < n; ++i)
            if (order[i] < 0 || order[i] >= n) return TSPH_ERR_ARG;
    const bool loadVel = L->v >= 0;
    if (ngas > 0 && !loadVel) return TSPH_ERR_ARG;   // gas needs velocities
    cudaSetDevice(ctx->device);
    // the particles of the last load again: keep the last tree's order
    // (tsph_update_particles), else a new particle set
    const unsigned long long key = store_key(n, ngas, store);
    const bool update = ctx->haveParts && ctx->n == n && ctx->storeKey == key && ctx->ngas == ngas &&
                        ctx->nSys <= 1 && n > 0;
    int rc = TSPH_OK;
    if (!update) {
        rc = tsph_load_begin(ctx, n);
        if (rc) return rc;
    }
    if (n == 0) {
        ctx->haveParts = true;
        ctx->storeKey = key;
        return TSPH_OK;
    }
    const char *src = mapped(store);
    if (!src) {   // not registered: one block copy to the device
        const size_t bytes = (size_t)n * (size_t)L->stride;
        if (ctx->storeCap < bytes) {
            if (ctx->dStore) cudaFree(ctx->dStore);
            ctx->dStore = nullptr;
            ctx->storeCap = 0;
            TSPH_CK(cudaMalloc((void **)&ctx->dStore, bytes));
            ctx->storeCap = bytes;
        }
        TSPH_CK(cudaMemcpyAsync(ctx->dStore, store, bytes, cudaMemcpyHostToDevice, ctx->stream));
        src = ctx->dStore;
    }
    int *dOrder = nullptr;
    if (order) {
        rc = tsph_grow(ctx, &ctx->dStoreOrder, (size_t)n);
        if (rc) return rc;
        TSPH_CK(cudaMemcpyAsync(ctx->dStoreOrder, order, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice,
                                ctx->stream));
        dOrder = ctx->dStoreOrder;
    }
    k_store_pos<<<tsph_blocks(n, 256), 256, 0, ctx->stream>>>(n, src, L->stride, L->r, dOrder,
                                                              ctx->dStage, ctx->C, update ? 1 : 0);
    TSPH_LAUNCH_CK("k_store_pos");
    if (!update) {
        rc = tsph_load_state_from_stage(ctx, n);
        if (rc) return rc;
    }
    k_store_rest<<<tsph_blocks(n, 256), 256, 0, ctx->stream>>>(n, ngas, src, L->stride, *L, dOrder, ctx->C,
                                                               loadVel ? 1 : 0);
    TSPH_LAUNCH_CK("k_store_rest");
    ctx->actRung = L->iActive >= 0 ? 1 : 0;
    ctx->storeKey = key;
    if (update) {
        // new values for the loaded particles: derived state is stale, the
        // gravity and gas trees keep their order
        ctx->haveTree = ctx->haveGrav = false;
        ctx->S.haveDensity = ctx->S.havePressure = false;
        ctx->sysVersion++;
        TSPH_CK(cudaStreamSynchronize(ctx->stream));
        ctx->haveVel = ctx->haveVel || loadVel;
        return TSPH_OK;
    }
    ctx->haveParts = true;
    if (!loadVel) {
        TSPH_CK(cudaStreamSynchronize(ctx->stream));
        return TSPH_OK;
    }
    return tsph_load_gas(ctx, ngas);   // gas tree order, flags; synchronises
}

// Results of one pass into an unregistered store, by the host: fetch the
// compact caller-order arrays and apply them entry by entry.
static int fetch(tsph_ctx *ctx, const double *dev, int n, double *host) {
    TSPH_CK(cudaMemcpyAsync(host, dev, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream));
    return TSPH_OK;
}

extern "C" int tsph_store_put_gravity(tsph_ctx *ctx, void *store, const tsph_store_layout *L,
                                      const int *order) {
    if (!ctx || !layout_ok(L)) return TSPH_ERR_ARG;
    if (!ctx->haveGrav) return TSPH_ERR_STATE;
    const int n = ctx->n;
    if (n == 0) return TSPH_OK;
    if (!store || !aligned(store)) return TSPH_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (order)
        for (int i = 0; i < n; ++i)
            if (order[i] < 0 || order[i] >= n) return TSPH_ERR_ARG;
    const char *dst = mapped(store);
    if (dst) {
        int *dOrder = nullptr;
        if (order) {
            int rc = tsph_grow(ctx, &ctx->dStoreOrder, (size_t)n);
            if (rc) return rc;
            TSPH_CK(cudaMemcpyAsync(ctx->dStoreOrder, order, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice,
                                    ctx->stream));
            dOrder = ctx->dStoreOrder;
        }
        k_store_put_grav<<<tsph_blocks(n, 256), 256, 0, ctx->stream>>>(n, const_cast<char *>(dst), L->stride,
                                                                       *L, dOrder, ctx->C, ctx->actRung);
        TSPH_LAUNCH_CK("k_store_put_grav");
        TSPH_CK(cudaStreamSynchronize(ctx->stream));
        return TSPH_OK;
    }
    double *h = (double *)malloc(sizeof(double) * 5 * (size_t)n);
    int *rung = (int *)malloc(sizeof(int) * (size_t)n);
    if (!h || !rung) { free(h); free(rung); return TSPH_ERR_NOMEM; }
    const double *src[5] = {ctx->C.ax, ctx->C.ay, ctx->C.az, ctx->C.pot, ctx->C.dtGrav};
    int rc = TSPH_OK;
    for (int k = 0; k < 5 && !rc; ++k) rc = fetch(ctx, src[k], n, h + (size_t)k * n);
    if (!rc && cudaMemcpyAsync(rung, ctx->C.rung, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost,
                               ctx->stream) != cudaSuccess)
        rc = TSPH_ERR_CUDA;
    if (!rc && cudaStreamSynchronize(ctx->stream) != cudaSuccess) rc = TSPH_ERR_CUDA;
    if (!rc) {
        for (int i = 0; i < n; ++i) {
            if (rung[i] < ctx->actRung) continue;
            char *b = (char *)store + (long long)(order ? order[i] : i) * L->stride;
            double *f;
            if (L->a >= 0) {
                f = (double *)(b + L->a);
                f[0] += h[i];
                f[1] += h[(size_t)n + i];
                f[2] += h[2 * (size_t)n + i];
            }
            if (L->fPot >= 0) *(double *)(b + L->fPot) += h[3 * (size_t)n + i];
            if (L->dtGrav >= 0) {
                f = (double *)(b + L->dtGrav);
                if (h[4 * (size_t)n + i] > *f) *f = h[4 * (size_t)n + i];
            }
        }
    }
    free(h);
    free(rung);
    return rc;
}

extern "C" int tsph_store_put_sph(tsph_ctx *ctx, int which, void *store, const tsph_store_layout *L,
                                  const int *order) {
    if (!ctx || !layout_ok(L)) return TSPH_ERR_ARG;
    if (which != TSPH_SMX_DENDVDX && which != TSPH_SMX_DENSITY && which != TSPH_SMX_SPHPRESSURETERMS)
        return TSPH_ERR_ARG;
    const TsphSphBufs &S = ctx->S;
    if (!S.haveDensity || (which == TSPH_SMX_SPHPRESSURETERMS && !S.havePressure)) return TSPH_ERR_STATE;
    const int ng = ctx->ngas;
    if (ng == 0) return TSPH_OK;
    if (!store || !aligned(store)) return TSPH_ERR_ARG;
    cudaSetDevice(ctx->device);
    const StoreSph D{S.fBall2, S.rho, S.divv, S.curl, S.dvds, S.bal, S.diff,
                     S.pr2, S.cs, S.hax, S.hay, S.haz, S.uPdV, S.uAV, S.dtNew, S.mumax};
    if (order)   // store entries 0..n-1
        for (int i = 0; i < ctx->n; ++i)
            if (order[i] < 0 || order[i] >= ctx->n) return TSPH_ERR_ARG;
    const char *dst = mapped(store);
    int *dOrder = nullptr;
    if (order) {
        int rc = tsph_grow(ctx, &ctx->dStoreOrder, (size_t)ctx->n);
        if (rc) return rc;
        TSPH_CK(cudaMemcpyAsync(ctx->dStoreOrder, order, sizeof(int) * (size_t)ctx->n, cudaMemcpyHostToDevice,
                                ctx->stream));
        dOrder = ctx->dStoreOrder;
    }
    if (dst) {
        k_store_put_sph<<<tsph_blocks(ng, 256), 256, 0, ctx->stream>>>(ng, const_cast<char *>(dst), L->stride,
                                                                      *L, dOrder, ctx->G.iord, D, ctx->C,
                                                                      which, ctx->actRung);
        TSPH_LAUNCH_CK("k_store_put_sph");
        TSPH_CK(cudaStreamSynchronize(ctx->stream));
        return TSPH_OK;
    }
    // unregistered: write the fields into a device copy of the gas entries'
    // store block, then apply them on the host field by field
    const size_t bytes = (size_t)ctx->n * (size_t)L->stride;
    if (ctx->storeCap < bytes) {
        if (ctx->dStore) cudaFree(ctx->dStore);
        ctx->dStore = nullptr;
        ctx->storeCap = 0;
        TSPH_CK(cudaMalloc((void **)&ctx->dStore, bytes));
        ctx->storeCap = bytes;
    }
    // the copy starts from the store as it is, so accumulated and lowered
    // fields (a[], dtNew) combine with the store's current values
    TSPH_CK(cudaMemcpyAsync(ctx->dStore, store, bytes, cudaMemcpyHostToDevice, ctx->stream));
    k_store_put_sph<<<tsph_blocks(ng, 256), 256, 0, ctx->stream>>>(ng, ctx->dStore, L->stride, *L, dOrder,
                                                                  ctx->G.iord, D, ctx->C, which, ctx->actRung);
    TSPH_LAUNCH_CK("k_store_put_sph");
    char *tmp = (char *)malloc(bytes);
    if (!tmp) return TSPH_ERR_NOMEM;
    if (cudaMemcpyAsync(tmp, ctx->dStore, bytes, cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
        free(tmp);
        return TSPH_ERR_CUDA;
    }
    const int fld[] = {L->fBall2, L->fDensity, L->divv, L->curlv, L->dvds, L->BalsaraSwitch, L->diff,
                       L->PoverRho2, L->c, L->a, L->uDotPdV, L->uDotAV, L->mumax, L->dtNew};
    const int width[] = {8, 8, 8, 24, 8, 8, 8, 8, 8, 24, 8, 8, 8, 8};
    for (int i = 0; i < ctx->n; ++i) {
        const size_t o = (size_t)(order ? order[i] : i) * (size_t)L->stride;
        for (size_t k = 0; k < sizeof(fld) / sizeof(fld[0]); ++k)
            if (fld[k] >= 0) memcpy((char *)store + o + fld[k], tmp + o + fld[k], (size_t)width[k]);
    }
    free(tmp);
    return TSPH_OK;
}
