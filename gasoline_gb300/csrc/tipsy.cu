// Tipsy snapshot I/O: the on-disk particle format of the reference
// (tipsydefs.h:9-45), read into and written from the context's device state.
//
// Format.  A 32-byte header (time as a double; nbodies, ndim, nsph, ndark,
// nstar as ints; 4 bytes of padding), then every gas record, every dark
// record and every star record, each a run of 4-byte floats:
//   gas  (12): mass, pos[3], vel[3], rho, temp, eps, metals, phi
//   dark  (9): mass, pos[3], vel[3], eps, phi
//   star (11): mass, pos[3], vel[3], metals, tform, eps, phi
// The standard form (bStandard, the reference's XDR encoding) stores every
// item big-endian; the native form stores the same bytes in host order.
// Header field order: xdrHeader master.c:3563-3575; record offsets:
// pkdSeek pkd.c:253-285.
//
// Reading (pkdReadTipsy pkd.c:297-686) converts each float to double, with
// v = dvFac*vel and u = uPred = dTuFac*temp for gas; eps becomes the
// softening and phi the potential.  Writing (pkdWriteTipsy pkd.c:1628-1798)
// rounds the doubles to float after vel*dvFac and u*duTFac (the adiabatic
// gas model's conversion).  Both run as a pipeline of fixed-size chunks:
// file <-> pinned host buffer <-> device buffer <-> a decode/encode kernel
// that byte-swaps and scatters one record per thread, with the file I/O of
// one chunk overlapping the copy and kernel of the next.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>
#include <sys/stat.h>

#include "tsph_ctx.cuh"

namespace {

constexpr int TIPSY_HEADER = 32;
constexpr int TIPSY_CHUNK = 1 << 19;            // particles per pipeline chunk
constexpr int TIPSY_WORDS_MAX = 12;             // longest record (gas), in words
constexpr int TIPSY_BS = 256;
constexpr int TIPSY_WARPS = TIPSY_BS / 32;

// byte offset of record i after the header
__host__ __device__ inline long long tipsy_offset(long long i, int nGas, int nDark) {
    if (i <= nGas) return 48LL * i;
    if (i <= (long long)nGas + nDark) return 48LL * nGas + 36LL * (i - nGas);
    return 48LL * nGas + 36LL * nDark + 44LL * (i - nGas - nDark);
}

__device__ inline unsigned int bswap32(unsigned int w) { return __byte_perm(w, 0u, 0x0123); }

struct SnapFields {
    float *rho, *metals, *tform;
};

// One warp stages the contiguous words of its 32 records in shared memory
// with coalesced loads, then each lane decodes its own record.
__global__ void __launch_bounds__(TIPSY_BS)
k_tipsy_decode(int i0, int i1, const unsigned int *__restrict__ raw, int swap, int nGas,
               int nDark, int bStandard, double dvFac, double dTuFac, TsphDevState C,
               SnapFields F, int *piord, int *giord, unsigned int *status) {
    __shared__ unsigned int sw[TIPSY_WARPS][32 * TIPSY_WORDS_MAX];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long wbase = (long long)blockIdx.x * TIPSY_BS + warp * 32 + i0;   // warp's first record
    if (wbase >= i1) return;
    const long long wend = wbase + 32 < i1 ? wbase + 32 : i1;
    const long long base0 = tipsy_offset(i0, nGas, nDark);
    const long long b0 = (tipsy_offset(wbase, nGas, nDark) - base0) >> 2;
    const long long b1 = (tipsy_offset(wend, nGas, nDark) - base0) >> 2;
    unsigned int *s = sw[warp];
    for (long long k = b0 + lane; k < b1; k += 32) {
        unsigned int w = __ldg(raw + k);
        s[k - b0] = swap ? bswap32(w) : w;
    }
    __syncwarp();
    const long long i = wbase + lane;
    if (i >= wend) return;
    const float *r = reinterpret_cast<const float *>(s) + ((tipsy_offset(i, nGas, nDark) - base0) >> 2) - b0;
    const int type = i < nGas ? 0 : (i < (long long)nGas + nDark ? 1 : 2);
    const double m = (double)r[0];
    // the reference asserts fMass > 0 for standard-form gas, >= 0 otherwise
    const bool badMass = (type == 0 && bStandard) ? !(m > 0.0) : !(m >= 0.0);
    if (badMass) atomicOr(status, 1u);
    double eps, phi, u = 0.0;
    float rho = 0.0f, metals = 0.0f, tform = 0.0f;
    if (type == 0) {
        rho = r[7]; u = dTuFac * (double)r[8]; eps = r[9]; metals = r[10]; phi = r[11];
    } else if (type == 1) {
        eps = r[7]; phi = r[8];
    } else {
        metals = r[7]; tform = r[8]; eps = r[9]; phi = r[10];
    }
    C.m[i] = m;
    C.x[i] = (double)r[1]; C.y[i] = (double)r[2]; C.z[i] = (double)r[3];
    const double vx = dvFac * (double)r[4], vy = dvFac * (double)r[5], vz = dvFac * (double)r[6];
    C.vx[i] = C.vpx[i] = vx; C.vy[i] = C.vpy[i] = vy; C.vz[i] = C.vpz[i] = vz;
    C.h[i] = eps;
    C.pot[i] = phi;
    C.u[i] = C.upred[i] = u;
    C.udot[i] = 0.0;
    C.hax[i] = C.hay[i] = C.haz[i] = 0.0;
    C.ax[i] = C.ay[i] = C.az[i] = C.dtGrav[i] = 0.0;
    C.fb2prev[i] = C.divvprev[i] = 0.0;
    C.rung[i] = 0;
    C.dt[i] = C.dtNew[i] = FLT_MAX;
    C.mumax[i] = C.updv[i] = C.cs[i] = C.disp[i] = 0.0;
    F.rho[i] = rho; F.metals[i] = metals; F.tform[i] = tform;
    piord[i] = (int)i;
    giord[i] = (int)i;
}

// Each lane builds its record in shared memory; the warp then stores the
// contiguous words with coalesced writes.
__global__ void __launch_bounds__(TIPSY_BS)
k_tipsy_encode(int i0, int i1, unsigned int *__restrict__ raw, int swap, int nGas, int nDark,
               double dvFac, double duTFac, TsphDevState C, SnapFields F, int haveSnap) {
    __shared__ unsigned int sw[TIPSY_WARPS][32 * TIPSY_WORDS_MAX];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long wbase = (long long)blockIdx.x * TIPSY_BS + warp * 32 + i0;
    if (wbase >= i1) return;
    const long long wend = wbase + 32 < i1 ? wbase + 32 : i1;
    const long long base0 = tipsy_offset(i0, nGas, nDark);
    const long long b0 = (tipsy_offset(wbase, nGas, nDark) - base0) >> 2;
    const long long b1 = (tipsy_offset(wend, nGas, nDark) - base0) >> 2;
    unsigned int *s = sw[warp];
    const long long i = wbase + lane;
    if (i < wend) {
        float *r = reinterpret_cast<float *>(s) + ((tipsy_offset(i, nGas, nDark) - base0) >> 2) - b0;
        const int type = i < nGas ? 0 : (i < (long long)nGas + nDark ? 1 : 2);
        r[0] = (float)C.m[i];
        r[1] = (float)C.x[i]; r[2] = (float)C.y[i]; r[3] = (float)C.z[i];
        r[4] = (float)(dvFac * C.vx[i]); r[5] = (float)(dvFac * C.vy[i]);
        r[6] = (float)(dvFac * C.vz[i]);
        const float eps = (float)C.h[i], phi = (float)C.pot[i];
        const float metals = haveSnap ? F.metals[i] : 0.0f;
        if (type == 0) {
            r[7] = haveSnap ? F.rho[i] : 0.0f;
            r[8] = (float)(duTFac * C.u[i]);
            r[9] = eps; r[10] = metals; r[11] = phi;
        } else if (type == 1) {
            r[7] = eps; r[8] = phi;
        } else {
            r[7] = metals; r[8] = haveSnap ? F.tform[i] : 0.0f; r[9] = eps; r[10] = phi;
        }
    }
    __syncwarp();
    for (long long k = b0 + lane; k < b1; k += 32) {
        unsigned int w = s[k - b0];
        raw[k] = swap ? bswap32(w) : w;
    }
}

// the SPH density of the last DenDVDX pass, in caller order, as the float
// the snapshot stores (the reference writes p->fDensity)
__global__ void k_rho_to_snap(int ng, const int *__restrict__ iord, const double *__restrict__ rho,
                              float *out) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < ng) out[iord[k]] = (float)rho[k];
}

bool host_little_endian() {
    const unsigned int one = 1;
    unsigned char b;
    memcpy(&b, &one, 1);
    return b == 1;
}

unsigned int load_be32(const unsigned char *p) {
    return ((unsigned int)p[0] << 24) | ((unsigned int)p[1] << 16) | ((unsigned int)p[2] << 8) |
           (unsigned int)p[3];
}

void store_be32(unsigned char *p, unsigned int v) {
    p[0] = (unsigned char)(v >> 24); p[1] = (unsigned char)(v >> 16);
    p[2] = (unsigned char)(v >> 8); p[3] = (unsigned char)v;
}

// header bytes -> fields; the native form is struct dump as laid out in
// memory (double at 0, five ints at 8..27, padding to 32)
void parse_header(const unsigned char *b, int bStandard, tsph_tipsy_header *h) {
    int v[5];
    if (bStandard) {
        unsigned long long t = ((unsigned long long)load_be32(b) << 32) | load_be32(b + 4);
        memcpy(&h->time, &t, 8);
        for (int k = 0; k < 5; ++k) {
            unsigned int w = load_be32(b + 8 + 4 * k);
            memcpy(&v[k], &w, 4);
        }
    } else {
        memcpy(&h->time, b, 8);
        memcpy(v, b + 8, 20);
    }
    h->nbodies = v[0]; h->ndim = v[1]; h->nsph = v[2]; h->ndark = v[3]; h->nstar = v[4];
}

void format_header(unsigned char *b, int bStandard, const tsph_tipsy_header *h) {
    memset(b, 0, TIPSY_HEADER);
    int v[5] = {h->nbodies, h->ndim, h->nsph, h->ndark, h->nstar};
    if (bStandard) {
        unsigned long long t;
        memcpy(&t, &h->time, 8);
        store_be32(b, (unsigned int)(t >> 32));
        store_be32(b + 4, (unsigned int)t);
        for (int k = 0; k < 5; ++k) {
            unsigned int w;
            memcpy(&w, &v[k], 4);
            store_be32(b + 8 + 4 * k, w);
        }
    } else {
        memcpy(b, &h->time, 8);
        memcpy(b + 8, v, 20);
    }
}

int header_valid(const tsph_tipsy_header *h) {
    if (h->nbodies < 0 || h->nsph < 0 || h->ndark < 0 || h->nstar < 0) return TSPH_ERR_IO;
    if ((long long)h->nsph + h->ndark + h->nstar != h->nbodies) return TSPH_ERR_IO;
    if (h->nbodies >= (1 << 27)) return TSPH_ERR_ARG;   // the library's particle-index limit
    return TSPH_OK;
}

int read_header_file(FILE *fp, int bStandard, tsph_tipsy_header *h) {
    unsigned char b[TIPSY_HEADER];
    if (fread(b, 1, TIPSY_HEADER, fp) != (size_t)TIPSY_HEADER) return TSPH_ERR_IO;
    parse_header(b, bStandard, h);
    return header_valid(h);
}

int ensure_snapshot(tsph_ctx *ctx) {
    const size_t chunk = (size_t)48 * TIPSY_CHUNK;
    if (!ctx->hPin) {
        cudaError_t e = cudaMallocHost(&ctx->hPin, 2 * chunk + 64);
        if (e != cudaSuccess) { ctx->hPin = nullptr; return tsph_cuda_fail(ctx, e, "cudaMallocHost"); }
        int rc = tsph_grow(ctx, &ctx->dSnapRaw, 2 * chunk / sizeof(unsigned int));
        if (!rc) rc = tsph_grow(ctx, &ctx->dSnapStatus, 1);
        if (rc) return rc;
        for (int k = 0; k < 2; ++k) TSPH_CK(cudaEventCreateWithFlags(&ctx->snapEv[k], cudaEventDisableTiming));
        ctx->snapChunkBytes = chunk;
    }
    if (ctx->snapCap < ctx->cap) {
        int rc = tsph_grow(ctx, &ctx->snapRho, ctx->cap);
        if (!rc) rc = tsph_grow(ctx, &ctx->snapMetals, ctx->cap);
        if (!rc) rc = tsph_grow(ctx, &ctx->snapTform, ctx->cap);
        if (rc) return rc;
        ctx->snapCap = ctx->cap;
        ctx->snapValid = false;
    }
    return TSPH_OK;
}

bool host_swaps(int bStandard) { return bStandard && host_little_endian(); }

}  // namespace

void tsph_free_snapshot(tsph_ctx *ctx) {
    if (ctx->hPin) cudaFreeHost(ctx->hPin);
    ctx->hPin = nullptr;
    for (int k = 0; k < 2; ++k)
        if (ctx->snapEv[k]) { cudaEventDestroy(ctx->snapEv[k]); ctx->snapEv[k] = nullptr; }
    void *d[] = {ctx->dSnapRaw, ctx->snapRho, ctx->snapMetals, ctx->snapTform, ctx->dSnapStatus};
    for (void *p : d) if (p) cudaFree(p);
    ctx->dSnapRaw = nullptr; ctx->snapRho = ctx->snapMetals = ctx->snapTform = nullptr;
    ctx->dSnapStatus = nullptr;
    ctx->snapCap = 0;
    ctx->snapValid = false;
}

extern "C" int tsph_tipsy_read_header(const char *path, int bStandard, tsph_tipsy_header *h) {
    if (!path || !h) return TSPH_ERR_ARG;
    FILE *fp = fopen(path, "rb");
    if (!fp) return TSPH_ERR_IO;
    int rc = read_header_file(fp, bStandard, h);
    fclose(fp);
    return rc;
}

// file body -> device state, chunk by chunk; fp is past the header
static int read_body(tsph_ctx *ctx, FILE *fp, const tsph_tipsy_header &h, int bStandard,
                     double dvFac, double dTuFac) {
    const int n = h.nbodies;
    unsigned int *hStatus = (unsigned int *)((unsigned char *)ctx->hPin + 2 * ctx->snapChunkBytes);
    TSPH_CK(cudaMemsetAsync(ctx->dSnapStatus, 0, sizeof(unsigned int), ctx->stream));
    const int swap = host_swaps(bStandard);
    const SnapFields F{ctx->snapRho, ctx->snapMetals, ctx->snapTform};
    unsigned char *hbuf[2] = {(unsigned char *)ctx->hPin, (unsigned char *)ctx->hPin + ctx->snapChunkBytes};
    unsigned int *dbuf[2] = {ctx->dSnapRaw, ctx->dSnapRaw + ctx->snapChunkBytes / 4};
    const int nChunks = (n + TIPSY_CHUNK - 1) / TIPSY_CHUNK;
    for (int c = 0; c < nChunks; ++c) {
        const int b = c & 1;
        const int i0 = c * TIPSY_CHUNK, i1 = i0 + TIPSY_CHUNK < n ? i0 + TIPSY_CHUNK : n;
        const size_t bytes = (size_t)(tipsy_offset(i1, h.nsph, h.ndark) - tipsy_offset(i0, h.nsph, h.ndark));
        // the copy that last read this host buffer (chunk c-2) must be done
        if (c >= 2) TSPH_CK(cudaEventSynchronize(ctx->snapEv[b]));
        if (fread(hbuf[b], 1, bytes, fp) != bytes) {
            cudaStreamSynchronize(ctx->stream);
            return TSPH_ERR_IO;
        }
        TSPH_CK(cudaMemcpyAsync(dbuf[b], hbuf[b], bytes, cudaMemcpyHostToDevice, ctx->stream));
        TSPH_CK(cudaEventRecord(ctx->snapEv[b], ctx->stream));
        k_tipsy_decode<<<tsph_blocks(i1 - i0, TIPSY_BS), TIPSY_BS, 0, ctx->stream>>>(
            i0, i1, dbuf[b], swap, h.nsph, h.ndark, bStandard, dvFac, dTuFac, ctx->C, F,
            ctx->P.iord, ctx->G.iord, ctx->dSnapStatus);
        TSPH_LAUNCH_CK("k_tipsy_decode");
    }
    TSPH_CK(cudaMemcpyAsync(hStatus, ctx->dSnapStatus, sizeof(unsigned int), cudaMemcpyDeviceToHost,
                            ctx->stream));
    TSPH_CK(cudaStreamSynchronize(ctx->stream));
    return *hStatus ? TSPH_ERR_IO : TSPH_OK;
}

extern "C" int tsph_read_tipsy(tsph_ctx *ctx, const char *path, int bStandard, double dvFac,
                               double dTuFac, tsph_tipsy_header *hout) {
    if (!ctx || !path) return TSPH_ERR_ARG;
    if (ctx->capturing) return TSPH_ERR_STATE;
    FILE *fp = fopen(path, "rb");
    if (!fp) return TSPH_ERR_IO;
    tsph_tipsy_header h;
    int rc = read_header_file(fp, bStandard, &h);
    struct stat st;
    if (!rc && (fstat(fileno(fp), &st) != 0 ||
                (long long)st.st_size < TIPSY_HEADER + tipsy_offset(h.nbodies, h.nsph, h.ndark)))
        rc = TSPH_ERR_IO;
    if (!rc) {
        cudaSetDevice(ctx->device);
        // the load replaces the particles as tsph_set_particles + tsph_set_velocities do
        rc = tsph_load_begin(ctx, h.nbodies);
        if (!rc) rc = ensure_snapshot(ctx);
        if (!rc && h.nbodies > 0) rc = read_body(ctx, fp, h, bStandard, dvFac, dTuFac);
    }
    fclose(fp);
    if (rc) {   // leave no half-loaded state behind
        ctx->haveParts = ctx->haveVel = false;
        ctx->snapValid = false;
        return rc;
    }
    ctx->snapValid = true;
    ctx->snapNStar = h.nstar;
    rc = tsph_load_gas(ctx, h.nsph);
    if (rc) return rc;
    if (hout) *hout = h;
    return TSPH_OK;
}

// device state -> file body, chunk by chunk; fp is past the header
static int write_body(tsph_ctx *ctx, FILE *fp, const tsph_tipsy_header &h, int bStandard,
                      double dvFac, double duTFac) {
    const int n = h.nbodies, nGas = h.nsph;
    const int swap = host_swaps(bStandard);
    const SnapFields F{ctx->snapRho, ctx->snapMetals, ctx->snapTform};
    unsigned char *hbuf[2] = {(unsigned char *)ctx->hPin, (unsigned char *)ctx->hPin + ctx->snapChunkBytes};
    unsigned int *dbuf[2] = {ctx->dSnapRaw, ctx->dSnapRaw + ctx->snapChunkBytes / 4};
    const int nChunks = (n + TIPSY_CHUNK - 1) / TIPSY_CHUNK;
    size_t pending = 0;   // bytes of chunk c-1 waiting in its host buffer
    for (int c = 0; c <= nChunks; ++c) {
        if (c < nChunks) {   // buffer c&1 was last written out in iteration c-1
            const int b = c & 1;
            const int i0 = c * TIPSY_CHUNK, i1 = i0 + TIPSY_CHUNK < n ? i0 + TIPSY_CHUNK : n;
            k_tipsy_encode<<<tsph_blocks(i1 - i0, TIPSY_BS), TIPSY_BS, 0, ctx->stream>>>(
                i0, i1, dbuf[b], swap, nGas, h.ndark, dvFac, duTFac, ctx->C, F, ctx->snapValid ? 1 : 0);
            TSPH_LAUNCH_CK("k_tipsy_encode");
            const size_t bytes = (size_t)(tipsy_offset(i1, nGas, h.ndark) - tipsy_offset(i0, nGas, h.ndark));
            TSPH_CK(cudaMemcpyAsync(hbuf[b], dbuf[b], bytes, cudaMemcpyDeviceToHost, ctx->stream));
            TSPH_CK(cudaEventRecord(ctx->snapEv[b], ctx->stream));
        }
        if (c > 0) {   // write chunk c-1 while chunk c is encoded and copied
            const int pb = (c - 1) & 1;
            TSPH_CK(cudaEventSynchronize(ctx->snapEv[pb]));
            if (fwrite(hbuf[pb], 1, pending, fp) != pending) {
                cudaStreamSynchronize(ctx->stream);
                return TSPH_ERR_IO;
            }
        }
        if (c < nChunks) {
            const int i0 = c * TIPSY_CHUNK, i1 = i0 + TIPSY_CHUNK < n ? i0 + TIPSY_CHUNK : n;
            pending = (size_t)(tipsy_offset(i1, nGas, h.ndark) - tipsy_offset(i0, nGas, h.ndark));
        }
    }
    return TSPH_OK;
}

extern "C" int tsph_write_tipsy(tsph_ctx *ctx, const char *path, int bStandard, double time,
                                int nStar, double dvFac, double duTFac) {
    if (!ctx || !path) return TSPH_ERR_ARG;
    if (ctx->capturing) return TSPH_ERR_STATE;
    if (!ctx->haveParts || !ctx->haveVel) return TSPH_ERR_STATE;
    const int n = ctx->n, nGas = ctx->ngas;
    if (nStar < 0 || nStar > n - nGas) return TSPH_ERR_ARG;
    tsph_tipsy_header h;
    h.time = time; h.nbodies = n; h.ndim = 3; h.nsph = nGas; h.ndark = n - nGas - nStar; h.nstar = nStar;
    cudaSetDevice(ctx->device);
    int rc = ensure_snapshot(ctx);
    if (rc) return rc;
    // the density of the last SPH pass replaces the density read in
    if (ctx->S.haveDensity && nGas > 0) {
        if (!ctx->snapValid) {
            TSPH_CK(cudaMemsetAsync(ctx->snapRho, 0, sizeof(float) * n, ctx->stream));
            TSPH_CK(cudaMemsetAsync(ctx->snapMetals, 0, sizeof(float) * n, ctx->stream));
            TSPH_CK(cudaMemsetAsync(ctx->snapTform, 0, sizeof(float) * n, ctx->stream));
            ctx->snapValid = true;
        }
        k_rho_to_snap<<<tsph_blocks(nGas, 256), 256, 0, ctx->stream>>>(nGas, ctx->G.iord, ctx->S.rho,
                                                                      ctx->snapRho);
        TSPH_LAUNCH_CK("k_rho_to_snap");
    }
    FILE *fp = fopen(path, "wb");
    if (!fp) return TSPH_ERR_IO;
    unsigned char hb[TIPSY_HEADER];
    format_header(hb, bStandard, &h);
    rc = fwrite(hb, 1, TIPSY_HEADER, fp) == (size_t)TIPSY_HEADER ? TSPH_OK : TSPH_ERR_IO;
    if (!rc && n > 0) rc = write_body(ctx, fp, h, bStandard, dvFac, duTFac);
    if (fclose(fp) != 0 && !rc) rc = TSPH_ERR_IO;
    return rc;
}

extern "C" int tsph_get_snapshot_fields(tsph_ctx *ctx, double *mass, double *soft, double *pot,
                                        float *rho, float *metals, float *tform) {
    if (!ctx) return TSPH_ERR_ARG;
    if (!ctx->haveParts) return TSPH_ERR_STATE;
    const int n = ctx->n;
    if (n == 0) return TSPH_OK;
    cudaSetDevice(ctx->device);
    if (mass) TSPH_CK(cudaMemcpyAsync(mass, ctx->C.m, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    if (soft) TSPH_CK(cudaMemcpyAsync(soft, ctx->C.h, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    if (pot) TSPH_CK(cudaMemcpyAsync(pot, ctx->C.pot, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    float *src[3] = {ctx->snapRho, ctx->snapMetals, ctx->snapTform};
    float *dst[3] = {rho, metals, tform};
    for (int k = 0; k < 3; ++k) {
        if (!dst[k]) continue;
        if (ctx->snapValid) {
            TSPH_CK(cudaMemcpyAsync(dst[k], src[k], sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream));
        } else {
            memset(dst[k], 0, sizeof(float) * n);
        }
    }
    TSPH_CK(cudaStreamSynchronize(ctx->stream));
    return TSPH_OK;
}

extern "C" int tsph_set_snapshot_fields(tsph_ctx *ctx, const double *pot, const float *rho,
                                        const float *metals, const float *tform) {
    if (!ctx) return TSPH_ERR_ARG;
    if (ctx->capturing) return TSPH_ERR_STATE;
    if (!ctx->haveParts) return TSPH_ERR_STATE;
    const int n = ctx->n;
    cudaSetDevice(ctx->device);
    int rc = ensure_snapshot(ctx);
    if (rc) return rc;
    if (n == 0) { ctx->snapValid = true; return TSPH_OK; }
    if (pot) TSPH_CK(cudaMemcpyAsync(ctx->C.pot, pot, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    const float *src[3] = {rho, metals, tform};
    float *dst[3] = {ctx->snapRho, ctx->snapMetals, ctx->snapTform};
    for (int k = 0; k < 3; ++k) {
        if (src[k]) {
            TSPH_CK(cudaMemcpyAsync(dst[k], src[k], sizeof(float) * n, cudaMemcpyHostToDevice, ctx->stream));
        } else if (!ctx->snapValid) {
            TSPH_CK(cudaMemsetAsync(dst[k], 0, sizeof(float) * n, ctx->stream));
        }
    }
    TSPH_CK(cudaStreamSynchronize(ctx->stream));   // host buffers reusable on return
    ctx->snapValid = true;
    return TSPH_OK;
}
