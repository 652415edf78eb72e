// K1/K2: gravity kd-tree build and cell moments on the device.
//
// The tree is the reference's binary tree (pkdBuildBinary, pkd.c:2627-2723):
// squeezed bounds, split at the midpoint of the longest axis, r[d] < fSplit
// goes low, a leaf when n <= nBucket or the bounds have zero extent.  It is
// built level by level over all nodes of a depth at once.  The particle
// permutation reproduces the reference's Hoare partition (pkdUpperPart,
// pkd.c:1109-1157) exactly: that scan swaps the k-th element >= fSplit from
// the left end with the k-th element < fSplit from the right end, so each
// such "misplaced" pair is found by its rank from a prefix sum and swapped
// independently.  Leaf particle order, node numbering, bounds, centres of
// mass, softening and opening radii therefore match the reference bit for
// bit, which keeps every walk decision identical.
#include <float.h>
#include <math.h>

#include "tsph_ctx.cuh"

// ---------------------------------------------------------------------------
// inclusive scan of int (three-phase: block scan, scan of block sums, add)
// ---------------------------------------------------------------------------
#define SCAN_BS 512
#define SCAN_IPT 8
#define SCAN_TILE (SCAN_BS * SCAN_IPT)

__global__ void k_scan_tile(const int *__restrict__ in, int *__restrict__ out,
                            int *__restrict__ sums, int n) {
    __shared__ int warpSums[SCAN_BS / 32];
    int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_IPT;
    int v[SCAN_IPT];
    int acc = 0;
#pragma unroll
    for (int k = 0; k < SCAN_IPT; ++k) {
        int i = base + k;
        acc += (i < n) ? in[i] : 0;
        v[k] = acc;
    }
    // warp inclusive scan of per-thread totals
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int t = acc;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= o) t += y;
    }
    if (lane == 31) warpSums[w] = t;
    __syncthreads();
    if (w == 0) {
        int s = (lane < SCAN_BS / 32) ? warpSums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < SCAN_BS / 32) warpSums[lane] = s;
    }
    __syncthreads();
    int prefix = t - acc + (w > 0 ? warpSums[w - 1] : 0);
#pragma unroll
    for (int k = 0; k < SCAN_IPT; ++k) {
        int i = base + k;
        if (i < n) out[i] = v[k] + prefix;
    }
    if (threadIdx.x == SCAN_BS - 1) sums[blockIdx.x] = prefix + acc;
}

__global__ void k_scan_add(int *__restrict__ out, const int *__restrict__ sums, int n) {
    if (blockIdx.x == 0) return;
    int add = sums[blockIdx.x - 1];
    int base = blockIdx.x * SCAN_TILE;
    for (int k = threadIdx.x; k < SCAN_TILE; k += SCAN_BS) {
        int i = base + k;
        if (i < n) out[i] += add;
    }
}

// scratch for the block sums lives in B.scanTmp (sized for the recursion)
static int scan_rec(tsph_ctx *ctx, const int *in, int *out, int n, int *tmp) {
    int nb = tsph_blocks(n, SCAN_TILE);
    k_scan_tile<<<nb, SCAN_BS, 0, ctx->stream>>>(in, out, tmp, n);
    TSPH_LAUNCH_CK("k_scan_tile");
    if (nb > 1) {
        int rc = scan_rec(ctx, tmp, tmp, nb, tmp + nb);
        if (rc) return rc;
        k_scan_add<<<nb, SCAN_BS, 0, ctx->stream>>>(out, tmp, n);
        TSPH_LAUNCH_CK("k_scan_add");
    }
    return TSPH_OK;
}

int tsph_scan_inclusive(tsph_ctx *ctx, const int *in, int *out, int n) {
    if (n <= 0) return TSPH_OK;
    return scan_rec(ctx, in, out, n, ctx->B.scanTmp);
}

// ---------------------------------------------------------------------------
// top phase: level-wise over all nodes larger than the task size
// ---------------------------------------------------------------------------
__device__ __forceinline__ void key_init(double *t_bnd, int v) {
    unsigned long long *k = reinterpret_cast<unsigned long long *>(t_bnd + 6 * v);
    k[0] = k[1] = k[2] = ~0ULL;
    k[3] = k[4] = k[5] = 0ULL;
}

__device__ __forceinline__ void key_atomics(double *t_bnd, int s, const unsigned long long *mn,
                                            const unsigned long long *mx) {
    unsigned long long *k = reinterpret_cast<unsigned long long *>(t_bnd + 6 * s);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        atomicMin(&k[d], mn[d]);
        atomicMax(&k[3 + d], mx[d]);
    }
}

// Roots of the forest: temp ids 0..nR-1.  Roots larger than S start the top
// phase's frontier; the others are subtree tasks straight away.
__global__ void k_roots(int nR, const int *__restrict__ rLo, const int *__restrict__ rHi, int S,
                        int *t_lo, int *t_hi, double *t_bnd, int *front, int *tasks,
                        TsphBuildCtl *ctl) {
    __shared__ int ws[2][32];
    __shared__ int carry[2];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (threadIdx.x < 2) carry[threadIdx.x] = 0;
    __syncthreads();
    for (int base = 0; base < nR; base += blockDim.x) {
        int r = base + threadIdx.x;
        bool live = r < nR;
        int lo = live ? rLo[r] : 0, hi = live ? rHi[r] : -1;
        bool big = live && (hi - lo + 1 > S);
        bool small = live && !big;
        unsigned bb = __ballot_sync(0xffffffffu, big), bs = __ballot_sync(0xffffffffu, small);
        if (lane == 0) { ws[0][w] = __popc(bb); ws[1][w] = __popc(bs); }
        __syncthreads();
        int ob = carry[0], os = carry[1], tb = 0, ts = 0;
        for (int k = 0; k < nw; ++k) {
            if (k < w) { ob += ws[0][k]; os += ws[1][k]; }
            tb += ws[0][k];
            ts += ws[1][k];
        }
        unsigned lt = (1u << lane) - 1u;
        if (live) {
            t_lo[r] = lo;
            t_hi[r] = hi;
            key_init(t_bnd, r);
            if (big) front[ob + __popc(bb & lt)] = r;
            else tasks[os + __popc(bs & lt)] = r;
        }
        __syncthreads();
        if (threadIdx.x == 0) { carry[0] += tb; carry[1] += ts; }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        ctl->taskCount = carry[1];
        ctl->taskNext = 0;
        ctl->nTop = nR;
        ctl->status = 0;
        ctl->nNodes = 0;
        ctl->levF[0] = carry[0];
        ctl->levStart[0] = 0;
        ctl->levStart[1] = nR;
    }
}

// Top-phase bounds over fixed chunks of each frontier node's particle range:
// a block reduces one chunk of one node and issues one set of atomics, so
// a node of N particles costs N / TB_CHUNK atomics instead of one per warp.
#define TB_CHUNK 4096
#define TB_BS 256
// Top-phase kernels run over Fb >= F frontier slots (a host-side bound);
// the frontier size F of level L lives on the device (ctl->levF[L]), so the
// host launches levels without waiting for each one.
// Chunks of frontier node v: none for a node of at most S particles (it
// becomes a subtree task, which finds its own bounds).
__device__ __forceinline__ int node_chunks(int size, int S) {
    return size > S ? (size + TB_CHUNK - 1) / TB_CHUNK : 0;
}

__global__ void k_chunk_count(int Fb, int L, int S, const TsphBuildCtl *__restrict__ ctl,
                              const int *__restrict__ f_node, const int *__restrict__ t_lo,
                              const int *__restrict__ t_hi, int *cc) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= Fb) return;
    if (k >= ctl->levF[L]) { cc[k] = 0; return; }
    int v = f_node[k];
    cc[k] = node_chunks(t_hi[v] - t_lo[v] + 1, S);
}

// The frontier index of every chunk (cs = inclusive scan of the chunk
// counts), so that a chunk's block finds its node with one load.
__global__ void k_chunk_map(int Fb, const int *__restrict__ cs, int *chunkNode) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cs[Fb - 1]) return;
    int a = 0, e = Fb - 1;   // first k with cs[k] > c
    while (a < e) {
        int m = (a + e) >> 1;
        if (cs[m] > c) e = m; else a = m + 1;
    }
    chunkNode[c] = a;
}

__device__ __forceinline__ unsigned long long umin64(unsigned long long a, unsigned long long b) {
    return a < b ? a : b;
}
__device__ __forceinline__ unsigned long long umax64(unsigned long long a, unsigned long long b) {
    return a > b ? a : b;
}

__global__ void __launch_bounds__(TB_BS) k_bounds_chunks(int F, const int *__restrict__ f_node,
                                                         const int *__restrict__ cs,
                                                         const int *__restrict__ chunkNode,
                                                         const int *__restrict__ t_lo,
                                                         const int *__restrict__ t_hi,
                                                         const double *__restrict__ x,
                                                         const double *__restrict__ y,
                                                         const double *__restrict__ z, double *t_bnd) {
    __shared__ unsigned long long red[TB_BS / 32][6];
    const int b = blockIdx.x;
    if (b >= cs[F - 1]) return;          // F here is the slot bound; unused slots count 0
    const int a = chunkNode[b];
    const int v = f_node[a];
    const int j = b - (a > 0 ? cs[a - 1] : 0);
    const int p0 = t_lo[v] + j * TB_CHUNK;
    const int p1 = min(p0 + TB_CHUNK, t_hi[v] + 1);
    unsigned long long mn[3] = {~0ULL, ~0ULL, ~0ULL}, mx[3] = {0ULL, 0ULL, 0ULL};
    for (int p = p0 + threadIdx.x; p < p1; p += TB_BS) {
        unsigned long long kx = dkey(x[p]), ky = dkey(y[p]), kz = dkey(z[p]);
        mn[0] = umin64(mn[0], kx); mx[0] = umax64(mx[0], kx);
        mn[1] = umin64(mn[1], ky); mx[1] = umax64(mx[1], ky);
        mn[2] = umin64(mn[2], kz); mx[2] = umax64(mx[2], kz);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            mn[d] = umin64(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], o));
            mx[d] = umax64(mx[d], __shfl_xor_sync(0xffffffffu, mx[d], o));
        }
    }
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
#pragma unroll
        for (int d = 0; d < 3; ++d) { red[w][d] = mn[d]; red[w][3 + d] = mx[d]; }
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int d = threadIdx.x;
        unsigned long long r = red[0][d];
        for (int k = 1; k < TB_BS / 32; ++k) r = d < 3 ? umin64(r, red[k][d]) : umax64(r, red[k][d]);
        unsigned long long *key = reinterpret_cast<unsigned long long *>(t_bnd + 6 * v);
        if (d < 3) atomicMin(&key[d], r); else atomicMax(&key[d], r);
    }
}

// Bounds keys -> doubles, and the split decision of a node
// (BuildBinary pkd.c:2460-2506): split at the midpoint of the longest axis
// unless the node holds at most nBucket particles or has zero extent.
__device__ __forceinline__ bool decide_node(int v, int nBucket, int *t_lo, int *t_hi, int *t_dim,
                                            int *t_child, double *t_split, double *t_bnd) {
    // the keys were accumulated by atomics in L2: read them past L1
    const unsigned long long *k = reinterpret_cast<const unsigned long long *>(t_bnd + 6 * v);
    double bmin[3], bmax[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        bmin[d] = dunkey(__ldcg(k + d));
        bmax[d] = dunkey(__ldcg(k + 3 + d));
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        t_bnd[6 * v + d] = bmin[d];
        t_bnd[6 * v + 3 + d] = bmax[d];
    }
    int good = 0;
#pragma unroll
    for (int d = 0; d < 3; ++d)
        if (bmax[d] > bmin[d]) good = 1;
    if ((t_hi[v] - t_lo[v] + 1 > nBucket) && good) {
        int d = 0;
        for (int j = 1; j < 3; ++j)
            if (xsub(bmax[j], bmin[j]) > xsub(bmax[d], bmin[d])) d = j;
        t_dim[v] = d;
        t_split[v] = xmul(0.5, xadd(bmin[d], bmax[d]));
        return true;
    }
    t_dim[v] = -1;
    t_split[v] = 0.0;
    t_child[v] = -1;
    return false;
}

// Top-phase frontier: nodes of at most S particles become subtree tasks,
// the others split here (or end as zero-extent leaves).
__global__ void k_top_split(int Fb, int L, const int *__restrict__ f_node, int S, int nBucket,
                            int *t_lo, int *t_hi, int *t_dim, int *t_child, int *t_size,
                            double *t_split, double *t_bnd, int *f_split, int *tasks,
                            TsphBuildCtl *ctl) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= Fb) return;
    if (k >= ctl->levF[L]) { f_split[k] = 0; return; }
    int v = f_node[k];
    if (t_hi[v] - t_lo[v] + 1 <= S) {
        t_dim[v] = -2;                       // handed to a subtree task
        f_split[k] = 0;
        key_init(t_bnd, v);
        tasks[atomicAdd(&ctl->taskCount, 1)] = v;
        return;
    }
    bool sp = decide_node(v, nBucket, t_lo, t_hi, t_dim, t_child, t_split, t_bnd);
    if (!sp) t_size[v] = 1;
    f_split[k] = sp ? 1 : 0;
}

// Smallest q in [a, b] with S[q] >= target (S non-decreasing).
__device__ __forceinline__ int lower_bound_scan(const int *__restrict__ S, int a, int b, int target) {
    while (a < b) {
        int c = (a + b) >> 1;
        if (S[c] >= target) b = c; else a = c + 1;
    }
    return a;
}

// The build moves positions and caller indices only; masses and
// softenings follow by one gather at its end (k_gather_mass).
__device__ __forceinline__ void swap_particles(double *x, double *y, double *z, int *iord, int p, int q) {
    double t0;
    t0 = x[p]; x[p] = x[q]; x[q] = t0;
    t0 = y[p]; y[p] = y[q]; y[q] = t0;
    t0 = z[p]; z[p] = z[q]; z[q] = t0;
    int ti = iord[p]; iord[p] = iord[q]; iord[q] = ti;
}

// Partition flags (r[d] < fSplit) of one chunk of a split frontier node and
// their in-chunk inclusive scan; ctot[b] = the chunk's count.  Warps take
// contiguous runs and count with ballots, kept in registers for the scan.
// The pass also gathers the bounds of the node's two children (their keys were
// initialised when the node was split), so the next level needs no pass of
// its own for them.
__global__ void __launch_bounds__(TB_BS, 3) k_flag_chunks(int Fb, int L, int nChunkSlots,
                                                       const int *__restrict__ f_node,
                                                       const int *__restrict__ cs,
                                                       const int *__restrict__ chunkNode,
                                                       const int *__restrict__ t_lo,
                                                       const int *__restrict__ t_hi,
                                                       const int *__restrict__ t_dim,
                                                       const double *__restrict__ t_split,
                                                       const double *__restrict__ x,
                                                       const double *__restrict__ y,
                                                       const double *__restrict__ z, int *scan,
                                                       int *ctot, const TsphBuildCtl *__restrict__ ctl,
                                                       const int *__restrict__ f_rank, int topCap,
                                                       double *t_bnd) {
    __shared__ int wt[TB_BS / 32];
    __shared__ unsigned long long kred[TB_BS / 32][12];
    const int b = blockIdx.x;
    if (b >= nChunkSlots) return;
    if (b >= cs[Fb - 1]) {
        if (threadIdx.x == 0) ctot[b] = 0;
        return;
    }
    const int k = chunkNode[b];
    const int v = f_node[k];
    const int d = t_dim[v];
    if (d < 0) {                          // a task or a leaf: nothing moves
        if (threadIdx.x == 0) ctot[b] = 0;
        return;
    }
    const int j = b - (k > 0 ? cs[k - 1] : 0);
    const int p0 = t_lo[v] + j * TB_CHUNK, p1 = min(p0 + TB_CHUNK, t_hi[v] + 1);
    const unsigned long long kfs = dlt_key(t_split[v]);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int CW = TB_CHUNK / (TB_BS / 32);
    const int w0 = p0 + w * CW, w1 = min(w0 + CW, p1);
    // first pass: the flags' count, and the bounds keys of the two
    // children (flagged: the lower child, the others: the upper one), which
    // the partition only moves about
    unsigned long long mn[2][3], mx[2][3];
#pragma unroll
    for (int c = 0; c < 2; ++c)
#pragma unroll
        for (int e = 0; e < 3; ++e) { mn[c][e] = ~0ULL; mx[c][e] = 0ULL; }
    // the warp's rows of 32 (CW / 32 of them): their flag ballots stay in
    // registers for the second pass
    constexpr int NR = CW / 32;
    unsigned bal[NR];
    int cnt = 0;
#pragma unroll
    for (int r0 = 0; r0 < NR; r0 += 4) {   // four rows' loads in flight at once
        double r[4][3];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int p = w0 + 32 * (r0 + u) + lane;
            r[u][0] = p < w1 ? x[p] : 0.0;
            r[u][1] = p < w1 ? y[p] : 0.0;
            r[u][2] = p < w1 ? z[p] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int p = w0 + 32 * (r0 + u) + lane;
            bool f = false;
            if (p < w1) {
                f = dlt_key(d == 0 ? r[u][0] : (d == 1 ? r[u][1] : r[u][2])) < kfs;
#pragma unroll
                for (int e = 0; e < 3; ++e) {
                    const unsigned long long kk = dkey(r[u][e]);
                    if (f) { mn[0][e] = umin64(mn[0][e], kk); mx[0][e] = umax64(mx[0][e], kk); }
                    else { mn[1][e] = umin64(mn[1][e], kk); mx[1][e] = umax64(mx[1][e], kk); }
                }
            }
            bal[r0 + u] = __ballot_sync(0xffffffffu, f);
            cnt += __popc(bal[r0 + u]);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int c = 0; c < 2; ++c)
#pragma unroll
            for (int e = 0; e < 3; ++e) {
                mn[c][e] = umin64(mn[c][e], __shfl_xor_sync(0xffffffffu, mn[c][e], o));
                mx[c][e] = umax64(mx[c][e], __shfl_xor_sync(0xffffffffu, mx[c][e], o));
            }
    }
    if (lane == 0) {
        wt[w] = cnt;
#pragma unroll
        for (int c = 0; c < 2; ++c)
#pragma unroll
            for (int e = 0; e < 3; ++e) { kred[w][6 * c + e] = mn[c][e]; kred[w][6 * c + 3 + e] = mx[c][e]; }
    }
    __syncthreads();
    if (threadIdx.x < 12) {
        // the children are numbered by the node's split rank (k_top_children)
        const int q = threadIdx.x % 6, c0 = ctl->levStart[L + 1] + 2 * (f_rank[k] - 1);
        const int c = c0 + threadIdx.x / 6;
        unsigned long long r = kred[0][threadIdx.x];
        for (int u = 1; u < TB_BS / 32; ++u)
            r = q < 3 ? umin64(r, kred[u][threadIdx.x]) : umax64(r, kred[u][threadIdx.x]);
        unsigned long long *key = reinterpret_cast<unsigned long long *>(t_bnd + 6 * (size_t)c) + q;
        if (c0 + 1 < topCap && (q < 3 ? r != ~0ULL : r != 0ULL)) {   // else k_top_children fails
            if (q < 3) atomicMin(key, r); else atomicMax(key, r);
        }
    }
    int run = 0, tot = 0;
#pragma unroll
    for (int q = 0; q < TB_BS / 32; ++q) {
        if (q < w) run += wt[q];
        tot += wt[q];
    }
    const unsigned le = (lane == 31) ? 0xffffffffu : ((2u << lane) - 1u);
#pragma unroll
    for (int q = 0; q < NR; ++q) {
        const int p = w0 + 32 * q + lane;
        if (p < w1) scan[p] = run + __popc(bal[q] & le);
        run += __popc(bal[q]);
    }
    if (threadIdx.x == 0) ctot[b] = tot;
}

// Node-local inclusive count of flags up to particle q of node v, from the
// in-chunk scans and the inclusive scan coff of the chunk counts.
__device__ __forceinline__ int node_scan(const int *__restrict__ scan, const int *__restrict__ coff,
                                         int first, int base, int lo, int q) {
    const int c = first + (q - lo) / TB_CHUNK;
    return scan[q] + (c > 0 ? coff[c - 1] : 0) - base;
}

// Hoare-partition swaps without searching: the left element of rank t
// (t-th element >= fSplit in [lo, mid)) swaps with the right element of
// rank t (t-th element < fSplit counted from hi downwards in [mid, hi]).
// k_mark_chunks scatters both into rank-indexed lists (slot lo + t of mL
// and mR), k_pair_chunks swaps list entry t of each.
__global__ void __launch_bounds__(TB_BS) k_mark_chunks(int Fb, const int *__restrict__ f_node,
                                                       const int *__restrict__ cs,
                                                       const int *__restrict__ chunkNode,
                                                       const int *__restrict__ coff,
                                                       const int *__restrict__ t_lo,
                                                       const int *__restrict__ t_hi,
                                                       const int *__restrict__ t_dim,
                                                       const int *__restrict__ scan, int *mL,
                                                       int *mR) {
    const int b = blockIdx.x;
    if (b >= cs[Fb - 1]) return;
    const int k = chunkNode[b];
    const int v = f_node[k];
    if (t_dim[v] < 0) return;
    const int first = k > 0 ? cs[k - 1] : 0, last = cs[k] - 1;
    const int base = first > 0 ? coff[first - 1] : 0;
    const int lo = t_lo[v], hi = t_hi[v];
    const int total = coff[last] - base;          // flags in the whole node
    const int mid = lo + total;                    // first index of the upper part
    const int j = b - first;
    const int p0 = lo + j * TB_CHUNK, p1 = min(p0 + TB_CHUNK, hi + 1);
    const int cbase = (b > 0 ? coff[b - 1] : 0) - base;   // flags before this chunk
    // four strides' loads in flight at once
    for (int q = p0 + threadIdx.x; q < p1; q += 4 * TB_BS) {
        int sv[4], pv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int p = q + u * TB_BS;
            sv[u] = p < p1 ? scan[p] : 0;
            pv[u] = p < p1 && p > p0 ? scan[p - 1] : 0;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int p = q + u * TB_BS;
            if (p >= p1) break;
            const int s = sv[u] + cbase;               // node-local inclusive count
            const int sp = p == p0 ? cbase : pv[u] + cbase;
            const bool flag = s != sp;                 // r < fSplit
            if (p < mid) {
                if (!flag) mL[lo + (p - lo) - sp] = p;          // misplaced left, rank (p-lo) - sp
            } else if (flag) {
                mR[lo + total - s] = p;                          // misplaced right, rank from hi
            }
        }
    }
}

__global__ void __launch_bounds__(TB_BS) k_pair_chunks(int Fb, const int *__restrict__ f_node,
                                                       const int *__restrict__ cs,
                                                       const int *__restrict__ chunkNode,
                                                       const int *__restrict__ coff,
                                                       const int *__restrict__ t_lo,
                                                       const int *__restrict__ t_dim,
                                                       const int *__restrict__ scan,
                                                       const int *__restrict__ mL,
                                                       const int *__restrict__ mR, double *x,
                                                       double *y, double *z, int *iord) {
    const int b = blockIdx.x;
    if (b >= cs[Fb - 1]) return;
    const int k = chunkNode[b];
    const int v = f_node[k];
    if (t_dim[v] < 0) return;
    const int first = k > 0 ? cs[k - 1] : 0, last = cs[k] - 1;
    const int base = first > 0 ? coff[first - 1] : 0;
    const int lo = t_lo[v];
    const int total = coff[last] - base;
    // misplaced pairs: the elements >= fSplit among the first `total`
    const int nMis = total > 0 ? total - node_scan(scan, coff, first, base, lo, lo + total - 1) : 0;
    // the node's swaps are dealt out over all of its chunk blocks
    const int j = b - first, nc = last - first + 1;
    for (int t = j * TB_BS + threadIdx.x; t < nMis; t += nc * TB_BS)
        swap_particles(x, y, z, iord, mL[lo + t], mR[lo + t]);
}

// ---- single-block forms of the per-level frontier work (one launch
// instead of a kernel plus a multi-kernel scan when the frontier is small)
#define LB_BS 1024
#define LB_ITEMS 4
#define LB_MAX (LB_BS * LB_ITEMS)

// Inclusive scan of v[0, count) (count <= LB_MAX) by one 1024-thread block;
// each thread owns LB_ITEMS consecutive items.
__device__ void block_scan_items(int *v, int count) {
    __shared__ int ws[LB_BS / 32];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    int a[LB_ITEMS], run = 0;
#pragma unroll
    for (int q = 0; q < LB_ITEMS; ++q) {
        int i = t * LB_ITEMS + q;
        run += i < count ? v[i] : 0;
        a[q] = run;
    }
    int incl = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) ws[w] = incl;
    __syncthreads();
    if (w == 0) {
        int x = ws[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        ws[lane] = x;
    }
    __syncthreads();
    const int off = incl - run + (w > 0 ? ws[w - 1] : 0);
#pragma unroll
    for (int q = 0; q < LB_ITEMS; ++q) {
        int i = t * LB_ITEMS + q;
        if (i < count) v[i] = a[q] + off;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(LB_BS) k_scan_small(int count, const int *__restrict__ in, int *out) {
    for (int i = threadIdx.x; i < count; i += LB_BS) out[i] = in[i];
    __syncthreads();
    block_scan_items(out, count);
}

// chunk counts of the frontier nodes, their inclusive scan and the
// frontier index of every chunk (Fb <= LB_MAX)
__global__ void __launch_bounds__(LB_BS) k_level_chunks(int Fb, int L, int S,
                                                        const TsphBuildCtl *__restrict__ ctl,
                                                        const int *__restrict__ f_node,
                                                        const int *__restrict__ t_lo,
                                                        const int *__restrict__ t_hi, int *cs,
                                                        int *chunkNode) {
    __shared__ int scs[LB_MAX];
    const int F = ctl->levF[L];
    for (int k = threadIdx.x; k < Fb; k += LB_BS) {
        int c = 0;
        if (k < F) {
            int v = f_node[k];
            c = node_chunks(t_hi[v] - t_lo[v] + 1, S);
        }
        scs[k] = c;
    }
    __syncthreads();
    block_scan_items(scs, Fb);
    for (int k = threadIdx.x; k < Fb; k += LB_BS) cs[k] = scs[k];
    const int total = Fb > 0 ? scs[Fb - 1] : 0;
    for (int c = threadIdx.x; c < total; c += LB_BS) {
        int a = 0, e = Fb - 1;   // first k with scs[k] > c
        while (a < e) {
            int m = (a + e) >> 1;
            if (scs[m] > c) e = m; else a = m + 1;
        }
        chunkNode[c] = a;
    }
}

// One level's frontier work in one block (Fb <= LB_MAX): the split
// decisions (as k_top_split, from the bounds the parent's flag pass
// gathered), the split ranks, the chunks of the nodes above the task size
// with their scan and node map (k_level_chunks), and the bounds keys of
// the children, which this level's flag pass accumulates.
__global__ void __launch_bounds__(LB_BS) k_level_prep(int Fb, int L, const int *__restrict__ f_node,
                                                      int S, int nBucket, int *t_lo, int *t_hi,
                                                      int *t_dim, int *t_child, int *t_size,
                                                      double *t_split, double *t_bnd, int *f_split,
                                                      int *f_rank, int *tasks, TsphBuildCtl *ctl,
                                                      int *cs, int *chunkNode, int topCap) {
    __shared__ int scs[LB_MAX];
    const int F = ctl->levF[L];
    for (int k = threadIdx.x; k < Fb; k += LB_BS) {
        int sp = 0, nc = 0;
        if (k < F) {
            int v = f_node[k];
            const int size = t_hi[v] - t_lo[v] + 1;
            if (size <= S) {
                t_dim[v] = -2;                   // handed to a subtree task
                key_init(t_bnd, v);
                tasks[atomicAdd(&ctl->taskCount, 1)] = v;
            } else {
                sp = decide_node(v, nBucket, t_lo, t_hi, t_dim, t_child, t_split, t_bnd) ? 1 : 0;
                if (!sp) t_size[v] = 1;
                nc = node_chunks(size, S);
            }
        }
        f_split[k] = sp;
        f_rank[k] = sp;
        scs[k] = nc;
    }
    __syncthreads();
    block_scan_items(f_rank, Fb);
    block_scan_items(scs, Fb);
    const int nTop = ctl->levStart[L + 1];
    for (int k = threadIdx.x; k < Fb; k += LB_BS) {
        cs[k] = scs[k];
        if (f_split[k]) {
            const int c = nTop + 2 * (f_rank[k] - 1);
            if (c + 1 < topCap) {
                key_init(t_bnd, c);
                key_init(t_bnd, c + 1);
            }
        }
    }
    const int total = Fb > 0 ? scs[Fb - 1] : 0;
    for (int c = threadIdx.x; c < total; c += LB_BS) {
        int a = 0, e = Fb - 1;   // first k with scs[k] > c
        while (a < e) {
            int m = (a + e) >> 1;
            if (scs[m] > c) e = m; else a = m + 1;
        }
        chunkNode[c] = a;
    }
}

// The children's bounds keys when the frontier is too large for one block.
__global__ void k_child_keys(int Fb, int L, const int *__restrict__ f_split,
                             const int *__restrict__ f_rank, const TsphBuildCtl *__restrict__ ctl,
                             int topCap, double *t_bnd) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= Fb || k >= ctl->levF[L] || !f_split[k]) return;
    const int c = ctl->levStart[L + 1] + 2 * (f_rank[k] - 1);
    if (c + 1 < topCap) {
        key_init(t_bnd, c);
        key_init(t_bnd, c + 1);
    }
}

__global__ void k_top_children(int Fb, int L, const int *__restrict__ f_node,
                               const int *__restrict__ f_split, const int *__restrict__ f_rank,
                               const int *__restrict__ cs, const int *__restrict__ coff,
                               int topCap, int *t_lo, int *t_hi, int *t_child, double *t_bnd,
                               int *nf_node, TsphBuildCtl *ctl) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int nTop = ctl->levStart[L + 1];      // this level's children start here
    if (k == 0) {
        int nt = nTop + 2 * f_rank[Fb - 1];
        if (nt > topCap) {
            atomicOr(&ctl->status, 1 << TSPH_ERR_TREE_DEPTH);
            nt = nTop;
        }
        ctl->levF[L + 1] = nt - nTop;
        ctl->levStart[L + 2] = nt;
        ctl->nTop = nt;
    }
    if (k >= Fb || k >= ctl->levF[L] || !f_split[k]) return;
    int v = f_node[k];
    int lo = t_lo[v], hi = t_hi[v];
    const int first = k > 0 ? cs[k - 1] : 0, last = cs[k] - 1;
    const int mid = lo + coff[last] - (first > 0 ? coff[first - 1] : 0);
    int r = f_rank[k] - 1;
    int c = nTop + 2 * r;
    if (c + 1 >= topCap) return;
    t_child[v] = c;
    t_lo[c] = lo;
    t_hi[c] = mid - 1;
    t_lo[c + 1] = mid;
    t_hi[c + 1] = hi;
    nf_node[2 * r] = c;
    nf_node[2 * r + 1] = c + 1;
}

// ---------------------------------------------------------------------------
// subtree phase: one CTA builds the whole subtree of a task, level by level
// ---------------------------------------------------------------------------
#define ST_BS 256
#define ST_W (ST_BS / 32)
#define ST_MAXLEV 96

struct BuildArgs {
    double *x, *y, *z, *m, *h;
    int *iord;
    int *seg, *lt, *scan;
    int *t_lo, *t_hi, *t_dim, *t_child, *t_size, *t_root, *t_loc;
    double *t_split, *t_bnd;
    const int *tasks;
    TsphBuildCtl *ctl;
    int topCap, nBucket;
    int scap;             // tasks up to this size are staged in shared memory
};

__device__ __forceinline__ unsigned lanemask_lt_b() {
    unsigned r;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(r));
    return r;
}

// Exclusive offset of this warp's total within the block, and the block
// total.  Two barriers.
__device__ __forceinline__ int st_warp_offset(int wtot, int *ws, int &total) {
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) ws[w] = wtot;
    __syncthreads();
    int off = 0, tot = 0;
#pragma unroll
    for (int k = 0; k < ST_W; ++k) {
        int v = ws[k];
        if (k < w) off += v;
        tot += v;
    }
    __syncthreads();
    total = tot;
    return off;
}

// Particle arrays a task works on: the global arrays, or (for a task of at
// most ST_SCAP particles) shared-memory copies of the positions plus the
// permutation, written back once the subtree is done.  Pointers are offset
// so that both are indexed by the global particle index.
struct TaskView {
    double *x, *y, *z;
    int *seg, *scan;
    int *lt;              // flags (global path only; the staged path re-derives them)
    short *perm;          // staged path: original local index of each slot
    bool staged;
};

// Bounds of every node of the current level: each warp reduces a
// contiguous chunk of the task's particles, carrying the open run of one
// node from step to step so a node costs about one atomic per warp.
__device__ void st_bounds(const BuildArgs &A, const TaskView &V, int lo, int hi) {
    const unsigned FULL = 0xffffffffu;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m = hi - lo + 1;
    const int C = ((m + ST_BS - 1) / ST_BS) * 32;
    const int b0 = lo + w * C;
    const int b1 = min(b0 + C, hi + 1);
    int cs = -1;
    unsigned long long cmn[3] = {~0ULL, ~0ULL, ~0ULL}, cmx[3] = {0ULL, 0ULL, 0ULL};
    for (int base = b0; base < b1; base += 32) {
        int p = base + lane;
        int s = p < b1 ? V.seg[p] : -1;
        unsigned long long mn[3], mx[3];
        if (s >= 0) {
            mn[0] = mx[0] = dkey(V.x[p]);
            mn[1] = mx[1] = dkey(V.y[p]);
            mn[2] = mx[2] = dkey(V.z[p]);
            if (lane == 0 && s == cs) {
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    mn[k] = cmn[k] < mn[k] ? cmn[k] : mn[k];
                    mx[k] = cmx[k] > mx[k] ? cmx[k] : mx[k];
                }
            }
        } else {
            mn[0] = mn[1] = mn[2] = ~0ULL;
            mx[0] = mx[1] = mx[2] = 0ULL;
        }
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int so = __shfl_down_sync(FULL, s, o);
            bool same = (lane + o < 32) && (so == s);
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                unsigned long long a = __shfl_down_sync(FULL, mn[k], o);
                unsigned long long b = __shfl_down_sync(FULL, mx[k], o);
                if (same) {
                    mn[k] = a < mn[k] ? a : mn[k];
                    mx[k] = b > mx[k] ? b : mx[k];
                }
            }
        }
        const int s0 = __shfl_sync(FULL, s, 0);
        const int s31 = __shfl_sync(FULL, s, 31);
        if (cs >= 0 && s0 != cs && lane == 0) key_atomics(A.t_bnd, cs, cmn, cmx);
        unsigned lastMask = __ballot_sync(FULL, s31 >= 0 && s == s31);
        int hl = lastMask ? __ffs(lastMask) - 1 : -1;
        int sp = __shfl_up_sync(FULL, s, 1);
        bool head = lane == 0 || sp != s;
        if (s >= 0 && head && lane != hl) key_atomics(A.t_bnd, s, mn, mx);
        if (hl >= 0) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                cmn[k] = __shfl_sync(FULL, mn[k], hl);
                cmx[k] = __shfl_sync(FULL, mx[k], hl);
            }
            cs = s31;
        } else {
            cs = -1;
        }
    }
    if (cs >= 0 && lane == 0) key_atomics(A.t_bnd, cs, cmn, cmx);
}

__device__ __forceinline__ int st_flag(const BuildArgs &A, const TaskView &V, int p) {
    int s = V.seg[p];
    if (s < 0) return 0;
    int d = A.t_dim[s];
    if (d < 0) return 0;
    double r = d == 0 ? V.x[p] : (d == 1 ? V.y[p] : V.z[p]);
    return r < A.t_split[s] ? 1 : 0;
}

#define ST_SCAP 3072      // largest task staged in shared memory
#define ST_DEFAULT_TASK 1536   // default task size: ~52 KB of staging, 4 CTAs per SM
#define ST_BYTES_PER (3 * sizeof(double) + 2 * sizeof(int) + sizeof(short))

__global__ void __launch_bounds__(ST_BS, 4) k_subtree(BuildArgs A) {
    extern __shared__ __align__(16) unsigned char stsm[];
    __shared__ int ws[ST_W];
    __shared__ int lvStart[ST_MAXLEV], lvCnt[ST_MAXLEV];
    __shared__ int sTask;
    const unsigned FULL = 0xffffffffu;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double *sx = reinterpret_cast<double *>(stsm);
    const int scap = A.scap;            // staging capacity of this launch
    double *sy = sx + scap, *sz = sy + scap;
    int *sseg = reinterpret_cast<int *>(sz + scap);
    int *sscan = sseg + scap;
    short *sperm = reinterpret_cast<short *>(sscan + scap);
    for (;;) {
        if (threadIdx.x == 0) {
            int t = atomicAdd(&A.ctl->taskNext, 1);
            sTask = t < A.ctl->taskCount ? A.tasks[t] : -1;
        }
        __syncthreads();
        const int root = sTask;
        if (root < 0) break;
        const int lo = A.t_lo[root], hi = A.t_hi[root];
        const int m = hi - lo + 1;
        const int slot0 = A.topCap + 2 * lo, slotEnd = slot0 + 2 * m;
        const int C = ((m + ST_BS - 1) / ST_BS) * 32;
        const int b0 = lo + w * C, b1 = min(b0 + C, hi + 1);
        TaskView V;
        V.staged = m <= scap;
        if (V.staged) {
            V.x = sx - lo; V.y = sy - lo; V.z = sz - lo;
            V.seg = sseg - lo; V.scan = sscan - lo; V.lt = nullptr; V.perm = sperm - lo;
            for (int p = lo + threadIdx.x; p <= hi; p += ST_BS) {
                V.x[p] = A.x[p];
                V.y[p] = A.y[p];
                V.z[p] = A.z[p];
                V.perm[p] = (short)(p - lo);
            }
        } else {
            V.x = A.x; V.y = A.y; V.z = A.z;
            V.seg = A.seg; V.scan = A.scan; V.lt = A.lt; V.perm = nullptr;
        }
        for (int p = lo + threadIdx.x; p <= hi; p += ST_BS) V.seg[p] = root;
        if (threadIdx.x == 0) {
            key_init(A.t_bnd, root);
            lvStart[0] = root;
            lvCnt[0] = 1;
        }
        __syncthreads();
        int L = 0;
        bool failed = false;
        for (;;) {
            const int start = lvStart[L], cnt = lvCnt[L];
            // 1. bounds of this level's nodes
            st_bounds(A, V, lo, hi);
            __syncthreads();
            // 2. split decisions
            for (int k = threadIdx.x; k < cnt; k += ST_BS)
                decide_node(start + k, A.nBucket, A.t_lo, A.t_hi, A.t_dim, A.t_child, A.t_split,
                            A.t_bnd);
            __syncthreads();
            // 3. partition flags and their scan over the task's particles
            int wtot = 0;
            for (int base = b0; base < b1; base += 32) {
                int p = base + lane;
                int f = p < b1 ? st_flag(A, V, p) : 0;
                if (!V.staged && p < b1) V.lt[p] = f;
                wtot += __popc(__ballot_sync(FULL, f));
            }
            int tot;
            int run = st_warp_offset(wtot, ws, tot);
            for (int base = b0; base < b1; base += 32) {
                int p = base + lane;
                int f = p < b1 ? (V.staged ? st_flag(A, V, p) : V.lt[p]) : 0;
                unsigned bal = __ballot_sync(FULL, f);
                if (p < b1) V.scan[p] = run + __popc(bal & (lanemask_lt_b() | (1u << lane)));
                run += __popc(bal);
            }
            __syncthreads();
            // 4. Hoare-partition swaps (scan is task-local: S(lo - 1) = 0)
            for (int p = lo + threadIdx.x; p <= hi; p += ST_BS) {
                int s = V.seg[p];
                if (s < 0 || A.t_dim[s] < 0) continue;
                const int Sp1 = p > lo ? V.scan[p - 1] : 0;
                if (V.scan[p] - Sp1) continue;            // r < fSplit: stays
                int vlo = A.t_lo[s], vhi = A.t_hi[s];
                int Slo = vlo > lo ? V.scan[vlo - 1] : 0;
                int Shi = V.scan[vhi];
                int mid = vlo + (Shi - Slo);
                if (p >= mid) continue;
                int t = (p - vlo) - (Sp1 - Slo);
                int q = lower_bound_scan(V.scan, mid, vhi, Shi - t);
                if (V.staged) {
                    double t0;
                    t0 = V.x[p]; V.x[p] = V.x[q]; V.x[q] = t0;
                    t0 = V.y[p]; V.y[p] = V.y[q]; V.y[q] = t0;
                    t0 = V.z[p]; V.z[p] = V.z[q]; V.z[q] = t0;
                    short ti = V.perm[p]; V.perm[p] = V.perm[q]; V.perm[q] = ti;
                } else {
                    swap_particles(A.x, A.y, A.z, A.iord, p, q);
                }
            }
            __syncthreads();
            // 5. children of the split nodes, numbered by split rank
            const int next = (L == 0) ? slot0 : start + cnt;
            const int NC = ((cnt + ST_BS - 1) / ST_BS) * 32;
            const int k0 = w * NC, k1 = min(k0 + NC, cnt);
            int ntot = 0;
            for (int kb = k0; kb < k1; kb += 32) {
                int k = kb + lane;
                bool f = k < k1 && A.t_dim[start + k] >= 0;
                ntot += __popc(__ballot_sync(FULL, f));
            }
            int nsplit;
            int rank = st_warp_offset(ntot, ws, nsplit);
            for (int kb = k0; kb < k1; kb += 32) {
                int k = kb + lane;
                bool f = k < k1 && A.t_dim[start + k] >= 0;
                unsigned bal = __ballot_sync(FULL, f);
                if (f) {
                    int v = start + k;
                    int c = next + 2 * (rank + __popc(bal & lanemask_lt_b()));
                    if (c + 1 >= slotEnd) {
                        atomicOr(&A.ctl->status, 1 << TSPH_ERR_ARG);
                    } else {
                        int vlo = A.t_lo[v], vhi = A.t_hi[v];
                        int Slo = vlo > lo ? V.scan[vlo - 1] : 0;
                        int mid = vlo + (V.scan[vhi] - Slo);
                        A.t_child[v] = c;
                        A.t_lo[c] = vlo;
                        A.t_hi[c] = mid - 1;
                        A.t_lo[c + 1] = mid;
                        A.t_hi[c + 1] = vhi;
                        key_init(A.t_bnd, c);
                        key_init(A.t_bnd, c + 1);
                        A.t_root[c] = root;
                        A.t_root[c + 1] = root;
                    }
                }
                rank += __popc(bal);
            }
            __syncthreads();
            // 6. particles follow their node into a child, or finish in a leaf
            for (int p = lo + threadIdx.x; p <= hi; p += ST_BS) {
                int s = V.seg[p];
                if (s < 0) continue;
                if (A.t_dim[s] >= 0) {
                    int c = A.t_child[s];
                    V.seg[p] = p < A.t_lo[c + 1] ? c : c + 1;
                } else {
                    V.seg[p] = -1;
                }
            }
            if (nsplit == 0) break;
            if (L + 1 >= ST_MAXLEV) {
                if (threadIdx.x == 0) atomicOr(&A.ctl->status, 1 << TSPH_ERR_TREE_DEPTH);
                failed = true;
                break;
            }
            if (threadIdx.x == 0) {
                lvStart[L + 1] = next;
                lvCnt[L + 1] = 2 * nsplit;
            }
            __syncthreads();
            ++L;
        }
        __syncthreads();
        if (V.staged) {
            // the final order back to the global arrays: positions first,
            // then the caller index gathered through the freed shared memory
            for (int p = lo + threadIdx.x; p <= hi; p += ST_BS) {
                A.x[p] = V.x[p];
                A.y[p] = V.y[p];
                A.z[p] = V.z[p];
            }
            __syncthreads();
            int *gi = reinterpret_cast<int *>(sx) - lo;
            for (int p = lo + threadIdx.x; p <= hi; p += ST_BS) gi[p] = A.iord[lo + V.perm[p]];
            __syncthreads();
            for (int p = lo + threadIdx.x; p <= hi; p += ST_BS) A.iord[p] = gi[p];
        }
        if (!failed) {
            // subtree sizes bottom-up, then depth-first offsets from the root
            for (int l = L; l >= 0; --l) {
                const int start = lvStart[l], cnt = lvCnt[l];
                for (int k = threadIdx.x; k < cnt; k += ST_BS) {
                    int v = start + k;
                    int c = A.t_child[v];
                    A.t_size[v] = 1 + (c >= 0 ? A.t_size[c] + A.t_size[c + 1] : 0);
                }
                __syncthreads();
            }
            if (threadIdx.x == 0) A.t_loc[root] = 0;
            __syncthreads();
            for (int l = 0; l < L; ++l) {
                const int start = lvStart[l], cnt = lvCnt[l];
                for (int k = threadIdx.x; k < cnt; k += ST_BS) {
                    int v = start + k;
                    int c = A.t_child[v];
                    if (c < 0) continue;
                    int lv = A.t_loc[v];
                    A.t_loc[c] = lv + 1;
                    A.t_loc[c + 1] = lv + 1 + A.t_size[c];
                }
                __syncthreads();
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// depth-first numbering and the final node arrays
// ---------------------------------------------------------------------------
// subtree sizes, bottom-up over one top level [a, b)
__global__ void k_size(int a, int b, const int *__restrict__ t_child, int *t_size) {
    int v = a + blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= b) return;
    int c = t_child[v];
    t_size[v] = 1 + (c >= 0 ? t_size[c] + t_size[c + 1] : 0);
}

// the same over a top level whose range lives on the device (a captured
// build does not know its levels on the host)
__global__ void k_size_dev(int l, const TsphBuildCtl *__restrict__ ctl,
                           const int *__restrict__ t_child, int *t_size) {
    const int a = ctl->levStart[l], b = ctl->levStart[l + 1];
    for (int v = a + blockIdx.x * blockDim.x + threadIdx.x; v < b; v += gridDim.x * blockDim.x) {
        int c = t_child[v];
        t_size[v] = 1 + (c >= 0 ? t_size[c] + t_size[c + 1] : 0);
    }
}

__global__ void k_pre_dev(int l, const TsphBuildCtl *__restrict__ ctl, const int *__restrict__ t_child,
                          const int *__restrict__ t_size, int *t_pre) {
    const int a = ctl->levStart[l], b = ctl->levStart[l + 1];
    for (int v = a + blockIdx.x * blockDim.x + threadIdx.x; v < b; v += gridDim.x * blockDim.x) {
        int c = t_child[v];
        if (c < 0) continue;
        int pv = t_pre[v];
        t_pre[c] = pv + 1;
        t_pre[c + 1] = pv + 1 + t_size[c];
    }
}

// Frontier nodes still unsplit when the top phase stops become subtree tasks.
__global__ void k_frontier_to_tasks(int Fb, int L, const int *__restrict__ f_node, int *t_dim,
                                    int *tasks, TsphBuildCtl *ctl) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= Fb || k >= ctl->levF[L]) return;
    int v = f_node[k];
    t_dim[v] = -2;
    tasks[atomicAdd(&ctl->taskCount, 1)] = v;
}

// roots: trees are stored one after another in range order
__global__ void k_root_pre(int nR, const int *__restrict__ t_size, int *t_pre, int *sysRoot,
                           int *rEnd, TsphBuildCtl *ctl) {
    __shared__ int ws[32];
    __shared__ int carry;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nR; base += blockDim.x) {
        int r = base + threadIdx.x;
        int v = r < nR ? t_size[r] : 0;
        int t = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane == 31) ws[w] = t;
        __syncthreads();
        int off = carry, tot = 0;
        for (int k = 0; k < nw; ++k) {
            if (k < w) off += ws[k];
            tot += ws[k];
        }
        if (r < nR) {
            int e = off + t - v;
            t_pre[r] = e;
            sysRoot[r] = e;
            rEnd[r] = e + v;
        }
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) ctl->nNodes = carry;
}

// depth-first (reference) index, top-down over one top level [a, b)
__global__ void k_pre(int a, int b, const int *__restrict__ t_child,
                      const int *__restrict__ t_size, int *t_pre) {
    int v = a + blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= b) return;
    int c = t_child[v];
    if (c < 0) return;
    int pv = t_pre[v];
    t_pre[c] = pv + 1;
    t_pre[c + 1] = pv + 1 + t_size[c];
}

__global__ void k_slot_pre(int topCap, int nSlots, const int *__restrict__ t_root,
                           const int *__restrict__ t_loc, int *t_pre) {
    int w = topCap + blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= topCap + nSlots) return;
    int r = t_root[w];
    if (r >= 0) t_pre[w] = t_pre[r] + t_loc[w];
}

__global__ void k_scatter_nodes(int topCap, int tcap, const TsphBuildCtl *__restrict__ ctl,
                                const int *__restrict__ t_lo, const int *__restrict__ t_hi,
                                const int *__restrict__ t_dim, const int *__restrict__ t_child,
                                const int *__restrict__ t_size, const int *__restrict__ t_pre,
                                const int *__restrict__ t_root, const double *__restrict__ t_split,
                                const double *__restrict__ t_bnd, const int *__restrict__ rid,
                                int nR, TsphDevTree T, int *leafFlag) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= tcap) return;
    if (v < topCap ? v >= ctl->nTop : t_root[v] < 0) return;
    int i = t_pre[v];
    int c = t_child[v];
    T.pLower[i] = t_lo[v];
    T.pUpper[i] = t_hi[v];
    T.iDim[i] = t_dim[v] >= 0 ? t_dim[v] : -1;
    T.fSplit[i] = t_split[v];
#pragma unroll
    for (int k = 0; k < 6; ++k) T.bnd[6 * i + k] = t_bnd[6 * v + k];
    T.upper[i] = c >= 0 ? t_pre[c + 1] : -1;
    T.dlink[i] = c >= 0 ? make_int2(t_pre[c + 1], t_lo[c + 1]) : make_int2(-1, 0);
    int nx = i + t_size[v];
    T.skip[i] = nx < T.rEnd[rid[t_lo[v]]] ? nx : -1;
    leafFlag[i] = c < 0 ? 1 : 0;
    if (c >= 0) {
        T.parent[t_pre[c]] = i;
        T.parent[t_pre[c + 1]] = i;
    }
    if (v < nR) T.parent[i] = -1;
}

__global__ void k_leaf_list(const TsphBuildCtl *__restrict__ ctl, const int *__restrict__ leafFlag,
                            const int *__restrict__ leafScan, int *leaves, int *dcnt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int nNodes = ctl->nNodes;
    if (i == 0) {
        dcnt[0] = nNodes;
        dcnt[1] = nNodes > 0 ? leafScan[nNodes - 1] : 0;
    }
    if (i >= nNodes || !leafFlag[i]) return;
    leaves[leafScan[i] - 1] = i;
}

// ---------------------------------------------------------------------------
// moments
// ---------------------------------------------------------------------------
// FP32 hi/lo copy of a node's centre of mass (w lanes are filled by k_open)
__device__ __forceinline__ void store_com32(TsphDevTree &T, int i, double x, double y, double z) {
    float hx, lx, hy, ly, hz, lz;
    split2f(x, hx, lx);
    split2f(y, hy, ly);
    split2f(z, hz, lz);
    T.wcomh[i] = make_float4(hx, hy, hz, 0.0f);
    T.wcoml[i] = make_float4(lx, ly, lz, 0.0f);
}

// Mass, softening and centre of mass of an interior node from its two
// children in the reference's order (pkd.c:2522-2547); the quadrupole by the
// parallel-axis theorem (equal to the reference's direct sum up to
// rounding).  Children may have been written by other SMs: read past L1.
// --- octopole and hexadecapole cells (iOrder >= 3) ------------------------
// Complete moments about each node's centre of mass, M3_abc = sum m d_a d_b
// d_c (10) and M4_abcd (15), in the field order of the reference's reduced
// moments (pkd.h:441-451): xxx xyy xxy yyy xxz yyz xyz xzz yzz zzz and
// xxxx xyyy xxxy yyyy xxxz yyyz xxyy xxyz xyyz xxzz xyzz xzzz yyzz yzzz zzzz.
// Leaves sum them over their particles; a parent adds its children's moments
// shifted to its own centre by the binomial expansion of (d' + D)^k, as the
// quadrupole is combined.  The reduced (trace-free) moments pkdCalcCell
// sums per particle (pkd.c:2076-2128) follow from the complete ones by
// linear identities (k_open).
__host__ __device__ constexpr int q_index(int a, int b) {
    return a == b ? a : (a + b == 1 ? 3 : (a + b == 2 ? 4 : 5));   // xx yy zz xy xz yz
}
__host__ __device__ constexpr int m3_index(int a, int b, int c) {
    // sort a <= b <= c
    int t = 0;
    if (a > b) { t = a; a = b; b = t; }
    if (b > c) { t = b; b = c; c = t; }
    if (a > b) { t = a; a = b; b = t; }
    const int code = a * 9 + b * 3 + c;
    return code == 0 ? 0 : code == 4 ? 1 : code == 1 ? 2 : code == 13 ? 3 : code == 2 ? 4 :
           code == 14 ? 5 : code == 5 ? 6 : code == 8 ? 7 : code == 17 ? 8 : 9;
}

// A particle's complete third and fourth moments about the leaf's centre
// of mass, added to m3 (xxx xyy xxy yyy xxz yyz xyz xzz yzz zzz) and m4
// (xxxx xyyy xxxy yyyy xxxz yyyz xxyy xxyz xyyz xxzz xyzz xzzz yyzz yzzz
// zzzz): fused multiply-adds on shared products, 37 FP64 operations (they
// are checked to rounding, as the parents' binomial shifts are).
template <typename R>
__device__ __forceinline__ void leaf_high(const R *d, R m, R *m3, R *m4) {
    const R x = d[0], y = d[1], z = d[2];
    const R xx = x * x, yy = y * y, zz = z * z, xy = x * y, xz = x * z, yz = y * z;
    const R mx = m * x, my = m * y, mz = m * z;
    m3[0] = fma(mx, xx, m3[0]);
    m3[1] = fma(mx, yy, m3[1]);
    m3[2] = fma(my, xx, m3[2]);
    m3[3] = fma(my, yy, m3[3]);
    m3[4] = fma(mz, xx, m3[4]);
    m3[5] = fma(mz, yy, m3[5]);
    m3[6] = fma(mx, yz, m3[6]);
    m3[7] = fma(mx, zz, m3[7]);
    m3[8] = fma(my, zz, m3[8]);
    m3[9] = fma(mz, zz, m3[9]);
    const R mxx = m * xx, myy = m * yy, mzz = m * zz;
    m4[0] = fma(mxx, xx, m4[0]);
    m4[1] = fma(myy, xy, m4[1]);
    m4[2] = fma(mxx, xy, m4[2]);
    m4[3] = fma(myy, yy, m4[3]);
    m4[4] = fma(mxx, xz, m4[4]);
    m4[5] = fma(myy, yz, m4[5]);
    m4[6] = fma(mxx, yy, m4[6]);
    m4[7] = fma(mxx, yz, m4[7]);
    m4[8] = fma(myy, xz, m4[8]);
    m4[9] = fma(mxx, zz, m4[9]);
    m4[10] = fma(mzz, xy, m4[10]);
    m4[11] = fma(mzz, xz, m4[11]);
    m4[12] = fma(myy, zz, m4[12]);
    m4[13] = fma(mzz, yz, m4[13]);
    m4[14] = fma(mzz, zz, m4[14]);
}

// Child moments (mass m, complete Q, M3, M4 about its own centre) shifted
// by d = child centre - parent centre, added into the parent's M3, M4.
template <typename R>
__device__ __forceinline__ void shift_high(const R *d, R m, const R *q, const R *c3, const R *c4, R *m3,
                                           R *m4) {
    constexpr unsigned char I3[10][3] = {{0, 0, 0}, {0, 1, 1}, {0, 0, 1}, {1, 1, 1}, {0, 0, 2},
                                         {1, 1, 2}, {0, 1, 2}, {0, 2, 2}, {1, 2, 2}, {2, 2, 2}};
    constexpr unsigned char I4[15][4] = {{0, 0, 0, 0}, {0, 1, 1, 1}, {0, 0, 0, 1}, {1, 1, 1, 1},
                                         {0, 0, 0, 2}, {1, 1, 1, 2}, {0, 0, 1, 1}, {0, 0, 1, 2},
                                         {0, 1, 1, 2}, {0, 0, 2, 2}, {0, 1, 2, 2}, {0, 2, 2, 2},
                                         {1, 1, 2, 2}, {1, 2, 2, 2}, {2, 2, 2, 2}};
#pragma unroll
    for (int k = 0; k < 10; ++k) {
        const int a = I3[k][0], b = I3[k][1], c = I3[k][2];
        m3[k] += c3[k] + q[q_index(a, b)] * d[c] + q[q_index(a, c)] * d[b] + q[q_index(b, c)] * d[a] +
                 m * d[a] * d[b] * d[c];
    }
#pragma unroll
    for (int k = 0; k < 15; ++k) {
        const int a = I4[k][0], b = I4[k][1], c = I4[k][2], e = I4[k][3];
        m4[k] += c4[k] + c3[m3_index(b, c, e)] * d[a] + c3[m3_index(a, c, e)] * d[b] +
                 c3[m3_index(a, b, e)] * d[c] + c3[m3_index(a, b, c)] * d[e] +
                 q[q_index(c, e)] * d[a] * d[b] + q[q_index(b, e)] * d[a] * d[c] +
                 q[q_index(b, c)] * d[a] * d[e] + q[q_index(a, e)] * d[b] * d[c] +
                 q[q_index(a, c)] * d[b] * d[e] + q[q_index(a, b)] * d[c] * d[e] +
                 m * d[a] * d[b] * d[c] * d[e];
    }
}

// A parent's complete M3, M4 from its children's (cc), shifted to its
// centre r, in R: FP64 (M3, M4 as allocated) for the FP64 walk, FP32 for
// the FP32 walk, whose cells only use FP32 copies of the reduced moments
// (the arrays then hold FP32 moments in their first half).  The child
// offsets are FP64 differences of the FP64 centres.
template <typename R>
__device__ __forceinline__ void combine_high(const TsphDevTree &T, int i, const double *r, const int *cc,
                                             R *M3, R *M4) {
    R m3[10], m4[15];
#pragma unroll
    for (int k = 0; k < 10; ++k) m3[k] = R(0);
#pragma unroll
    for (int k = 0; k < 15; ++k) m4[k] = R(0);
#pragma unroll
    for (int s = 0; s < 2; ++s) {
        const int ch = cc[s];
        const R mc = (R)__ldcg(&T.fMass[ch]);
        const R d[3] = {(R)(__ldcg(&T.r[3 * ch]) - r[0]), (R)(__ldcg(&T.r[3 * ch + 1]) - r[1]),
                        (R)(__ldcg(&T.r[3 * ch + 2]) - r[2])};
        R qc[6], c3[10], c4[15];
#pragma unroll
        for (int k = 0; k < 6; ++k) qc[k] = (R)__ldcg(&T.Q[6 * ch + k]);
#pragma unroll
        for (int k = 0; k < 10; ++k) c3[k] = __ldcg(&M3[10 * (size_t)ch + k]);
#pragma unroll
        for (int k = 0; k < 15; ++k) c4[k] = __ldcg(&M4[15 * (size_t)ch + k]);
        shift_high<R>(d, mc, qc, c3, c4, m3, m4);
    }
#pragma unroll
    for (int k = 0; k < 10; ++k) M3[10 * (size_t)i + k] = m3[k];
#pragma unroll
    for (int k = 0; k < 15; ++k) M4[15 * (size_t)i + k] = m4[k];
}

// A leaf's complete M3, M4 about its centre (r0, r1, r2) from its
// particles [lo, hi], in R as combine_high.
template <typename R>
__device__ __forceinline__ void leaf_moments_high(int i, int lo, int hi, const double *__restrict__ x,
                                                  const double *__restrict__ y, const double *__restrict__ z,
                                                  const double *__restrict__ m, double r0, double r1,
                                                  double r2, R *M3, R *M4) {
    R m3[10], m4[15];
#pragma unroll
    for (int k = 0; k < 10; ++k) m3[k] = R(0);
#pragma unroll
    for (int k = 0; k < 15; ++k) m4[k] = R(0);
    for (int p = lo; p <= hi; ++p) {
        const R d[3] = {(R)xsub(x[p], r0), (R)xsub(y[p], r1), (R)xsub(z[p], r2)};
        leaf_high<R>(d, (R)m[p], m3, m4);
    }
#pragma unroll
    for (int k = 0; k < 10; ++k) M3[10 * (size_t)i + k] = m3[k];
#pragma unroll
    for (int k = 0; k < 15; ++k) M4[15 * (size_t)i + k] = m4[k];
}

__device__ void combine_node(TsphDevTree &T, int i, int high) {
    const int l = i + 1, u = T.upper[i];
    double fMass = 0.0, fSoft = 0.0, r[3] = {0.0, 0.0, 0.0};
    double fm = __ldcg(&T.fMass[l]);
    fMass = xadd(fMass, fm);
    fSoft = xadd(fSoft, xmul(fm, __ldcg(&T.fSoft[l])));
#pragma unroll
    for (int j = 0; j < 3; ++j) r[j] = xadd(r[j], xmul(fm, __ldcg(&T.r[3 * l + j])));
    fm = __ldcg(&T.fMass[u]);
    fMass = xadd(fMass, fm);
    fSoft = xadd(fSoft, xmul(fm, __ldcg(&T.fSoft[u])));
#pragma unroll
    for (int j = 0; j < 3; ++j) r[j] = xadd(r[j], xmul(fm, __ldcg(&T.r[3 * u + j])));
    if (fMass > 0) {
        fSoft = __ddiv_rn(fSoft, fMass);
#pragma unroll
        for (int j = 0; j < 3; ++j) r[j] = __ddiv_rn(r[j], fMass);
    }
    T.fMass[i] = fMass;
    T.fSoft[i] = fSoft;
#pragma unroll
    for (int j = 0; j < 3; ++j) T.r[3 * i + j] = r[j];
    store_com32(T, i, r[0], r[1], r[2]);
    double q[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) q[k] = __ldcg(&T.Q[6 * l + k]) + __ldcg(&T.Q[6 * u + k]);
    int cc[2] = {l, u};
#pragma unroll
    for (int s = 0; s < 2; ++s) {
        int ch = cc[s];
        double mc = __ldcg(&T.fMass[ch]);
        double dx = __ldcg(&T.r[3 * ch]) - r[0], dy = __ldcg(&T.r[3 * ch + 1]) - r[1],
               dz = __ldcg(&T.r[3 * ch + 2]) - r[2];
        q[0] += mc * dx * dx;
        q[1] += mc * dy * dy;
        q[2] += mc * dz * dz;
        q[3] += mc * dx * dy;
        q[4] += mc * dx * dz;
        q[5] += mc * dy * dz;
    }
    // complete M3, M4 from the children's, before q is final
    if (high == 1) combine_high<double>(T, i, r, cc, T.M3, T.M4);
    else if (high == 2) combine_high<float>(T, i, r, cc, reinterpret_cast<float *>(T.M3),
                                            reinterpret_cast<float *>(T.M4));
#pragma unroll
    for (int k = 0; k < 6; ++k) T.Q[6 * i + k] = q[k];
}

// Leaf mass, softening and centre of mass summed in tree order exactly as
// BuildBinary (pkd.c:2559-2574); quadrupole summed as pkdCalcCell
// (pkd.c:2094-2130).  k_moments then climbs: at each parent the second
// child to finish (counted by an atomic) combines it, so every interior
// node is formed once, after both children, with no per-level launches.
__device__ __forceinline__ void leaf_node(TsphDevTree &T, int i, const double *__restrict__ x,
                                          const double *__restrict__ y, const double *__restrict__ z,
                                          const double *__restrict__ m, const double *__restrict__ h,
                                          int high) {
    int lo = T.pLower[i], hi = T.pUpper[i];
    double fMass = 0.0, fSoft = 0.0, r0 = 0.0, r1 = 0.0, r2 = 0.0;
    for (int p = lo; p <= hi; ++p) {
        double fm = m[p];
        fMass = xadd(fMass, fm);
        fSoft = xadd(fSoft, xmul(fm, h[p]));
        r0 = xadd(r0, xmul(fm, x[p]));
        r1 = xadd(r1, xmul(fm, y[p]));
        r2 = xadd(r2, xmul(fm, z[p]));
    }
    if (fMass > 0) {
        fSoft = __ddiv_rn(fSoft, fMass);
        r0 = __ddiv_rn(r0, fMass);
        r1 = __ddiv_rn(r1, fMass);
        r2 = __ddiv_rn(r2, fMass);
    }
    T.fMass[i] = fMass;
    T.fSoft[i] = fSoft;
    T.r[3 * i + 0] = r0;
    T.r[3 * i + 1] = r1;
    T.r[3 * i + 2] = r2;
    store_com32(T, i, r0, r1, r2);
    // the quadrupole with fused multiply-adds on m d (9 FP64 operations a
    // particle instead of 18: GB300 runs FP64 at 1/64 of the FP32 rate);
    // it matches the reference's sums to rounding, as the parent's
    // parallel-axis combination does, while mass, centre of mass and
    // softening above keep the reference's operations bit for bit
    double q[6] = {0, 0, 0, 0, 0, 0};
    for (int p = lo; p <= hi; ++p) {
        const double fm = m[p];
        const double dx = xsub(x[p], r0), dy = xsub(y[p], r1), dz = xsub(z[p], r2);
        const double mx = fm * dx, my = fm * dy, mz = fm * dz;
        q[0] = fma(mx, dx, q[0]);
        q[1] = fma(my, dy, q[1]);
        q[2] = fma(mz, dz, q[2]);
        q[3] = fma(mx, dy, q[3]);
        q[4] = fma(mx, dz, q[4]);
        q[5] = fma(my, dz, q[5]);
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) T.Q[6 * i + k] = q[k];
    if (high == 1)
        leaf_moments_high<double>(i, lo, hi, x, y, z, m, r0, r1, r2, T.M3, T.M4);
    else if (high == 2)
        leaf_moments_high<float>(i, lo, hi, x, y, z, m, r0, r1, r2, reinterpret_cast<float *>(T.M3),
                                 reinterpret_cast<float *>(T.M4));
}

// The arrival at i's parent once i is complete: the parent if i was its
// second child to finish (its combination is then due), else -1.
__device__ __forceinline__ int arrive(const TsphDevTree &T, int *visit, int i) {
    __threadfence();
    const int par = T.parent[i];
    if (par < 0) return -1;
    if (atomicAdd(&visit[par], 1) == 0) return -1;   // the sibling is not done yet
    __threadfence();
    return par;
}

#define MOM_BS 128

__global__ void __launch_bounds__(MOM_BS) k_moments(TsphDevTree T, const double *__restrict__ x,
                                                    const double *__restrict__ y, const double *__restrict__ z,
                                                    const double *__restrict__ m, const double *__restrict__ h,
                                                    int *visit, int high) {
    __shared__ int queue[MOM_BS];
    __shared__ int wcount[MOM_BS / 32];
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int next = -1;
    if (b < T.dcnt[1]) {
        const int i = T.leaves[b];
        leaf_node(T, i, x, y, z, m, h, high);
        next = arrive(T, visit, i);
    }
    // The climb: the parents that this block's threads completed are packed
    // into the first threads of the block and combined there, level after
    // level, so a warp's FP64 instructions serve up to 32 nodes however
    // few of the block's threads are still climbing.
    for (;;) {
        const unsigned bal = __ballot_sync(0xffffffffu, next >= 0);
        if (lane == 0) wcount[w] = __popc(bal);
        __syncthreads();
        int off = 0, tot = 0;
#pragma unroll
        for (int k = 0; k < MOM_BS / 32; ++k) {
            const int c = wcount[k];
            off += k < w ? c : 0;
            tot += c;
        }
        if (next >= 0) queue[off + __popc(bal & ((1u << lane) - 1u))] = next;
        __syncthreads();
        if (tot == 0) break;
        next = -1;
        if ((int)threadIdx.x < tot) {
            const int node = queue[threadIdx.x];
            __threadfence();
            combine_node(T, node, high);
            next = arrive(T, visit, node);
        }
    }
}

__global__ void k_zero_u64(unsigned long long *a, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = 0ULL;
}

// Bmax in two FP32 descents and few FP64 distances.  The squared distance
// of particle p to the COM of node i is bracketed in FP32 from the hi/lo
// splits ([lo, hi], per-axis error erel |d| + eabs); pass A takes each
// node's max of lo, a lower bound of its Bmax^2; pass B computes the exact
// FP64 distance (the reference's operations) only for particles whose hi
// reaches that bound, the only ones that can attain the maximum.
__device__ __forceinline__ void com_d2_interval(float4 ph, float4 pl, float4 ch, float4 cl, float eabs,
                                                float &lo, float &hi) {
    const float u = 5.9604645e-08f;
    const float d[3] = {(ph.x - ch.x) + (pl.x - cl.x), (ph.y - ch.y) + (pl.y - cl.y),
                        (ph.z - ch.z) + (pl.z - cl.z)};
    lo = 0.0f;
    hi = 0.0f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float ad = fabsf(d[a]), e = 4.0f * u * ad + eabs;
        const float l = fmaxf(ad - e, 0.0f), h = ad + e;
        lo += l * l;
        hi += h * h;
    }
    lo *= 1.0f - 4.0f * u;
    hi *= 1.0f + 4.0f * u;
}

__global__ void k_bmax_lo(int n, TsphDevTree T, const float4 *__restrict__ ph,
                          const float4 *__restrict__ pl, const int *__restrict__ rid, float eabs,
                          unsigned int *maxLo) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    bool live = p < n;
    int i = live ? T.sysRoot[rid[p]] : 0;
    const float4 a = live ? ph[p] : make_float4(0, 0, 0, 0), b = live ? pl[p] : make_float4(0, 0, 0, 0);
    unsigned mask = __ballot_sync(0xffffffffu, live);
    while (mask) {
        if (live) {
            float lo, hi;
            com_d2_interval(a, b, T.wcomh[i], T.wcoml[i], eabs, lo, hi);
            unsigned grp = __match_any_sync(mask, i);
            unsigned m = __reduce_max_sync(grp, __float_as_uint(lo));
            if ((int)(threadIdx.x & 31) == __ffs(grp) - 1) atomicMax(&maxLo[i], m);
            const int2 dl = T.dlink[i];
            if (dl.x < 0) live = false;
            else i = (p >= dl.y) ? dl.x : i + 1;
        }
        mask = __ballot_sync(0xffffffffu, live);
    }
}

__global__ void k_bmax_exact(int n, TsphDevTree T, const double *__restrict__ x,
                             const double *__restrict__ y, const double *__restrict__ z,
                             const float4 *__restrict__ ph, const float4 *__restrict__ pl,
                             const int *__restrict__ rid, float eabs,
                             const unsigned int *__restrict__ maxLo, unsigned long long *maxd2) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    int i = T.sysRoot[rid[p]];
    const float4 a = ph[p], b = pl[p];
    for (;;) {
        float lo, hi;
        com_d2_interval(a, b, T.wcomh[i], T.wcoml[i], eabs, lo, hi);
        if (hi >= __uint_as_float(maxLo[i])) {
            double dx = xsub(x[p], T.r[3 * i]);
            double dy = xsub(y[p], T.r[3 * i + 1]);
            double dz = xsub(z[p], T.r[3 * i + 2]);
            double d2 = xadd(xadd(xmul(dx, dx), xmul(dy, dy)), xmul(dz, dz));
            atomicMax(&maxd2[i], (unsigned long long)__double_as_longlong(d2));
        }
        const int2 dl = T.dlink[i];
        if (dl.x < 0) break;
        i = (p >= dl.y) ? dl.x : i + 1;
    }
}

// Opening radius, OPEN_JOSH (pkd.c:2245-2253); walk copies in FP32.
// Reduced octopole and hexadecapole (pkdCalcCell pkd.c:2076-2128) from the
// complete moments: sum m (d_a d_b d_c - 0.2 d^2 (...)) etc. are linear in
// the complete moments, with sum m d^2 d_a = T_a and sum m d^2 d_a d_b =
// S_ab, sum m d^4 = S_xx + S_yy + S_zz.
template <typename R>
__device__ __forceinline__ void reduce_high(const R *M, const R *H4, R *o, R *h) {
    const R Tx = M[0] + M[1] + M[7], Ty = M[2] + M[3] + M[8], Tz = M[4] + M[5] + M[9];
    o[0] = M[0] - R(0.6) * Tx;   // xxx
    o[1] = M[1] - R(0.2) * Tx;   // xyy
    o[2] = M[2] - R(0.2) * Ty;   // xxy
    o[3] = M[3] - R(0.6) * Ty;   // yyy
    o[4] = M[4] - R(0.2) * Tz;   // xxz
    o[5] = M[5] - R(0.2) * Tz;   // yyz
    o[6] = M[6];              // xyz
    o[7] = M[7] - R(0.2) * Tx;   // xzz
    o[8] = M[8] - R(0.2) * Ty;   // yzz
    o[9] = M[9] - R(0.6) * Tz;   // zzz
    const R Sxx = H4[0] + H4[6] + H4[9], Syy = H4[6] + H4[3] + H4[12], Szz = H4[9] + H4[12] + H4[14];
    const R Sxy = H4[2] + H4[1] + H4[10], Sxz = H4[4] + H4[8] + H4[11], Syz = H4[7] + H4[5] + H4[13];
    const R S4 = Sxx + Syy + Szz;
    h[0] = H4[0] - R(6.0 / 7.0) * Sxx + R(0.6 / 7.0) * S4;            // xxxx
    h[1] = H4[1] - R(3.0 / 7.0) * Sxy;                             // xyyy
    h[2] = H4[2] - R(3.0 / 7.0) * Sxy;                             // xxxy
    h[3] = H4[3] - R(6.0 / 7.0) * Syy + R(0.6 / 7.0) * S4;            // yyyy
    h[4] = H4[4] - R(3.0 / 7.0) * Sxz;                             // xxxz
    h[5] = H4[5] - R(3.0 / 7.0) * Syz;                             // yyyz
    h[6] = H4[6] - R(1.0 / 7.0) * (Sxx + Syy) + R(0.2 / 7.0) * S4;    // xxyy
    h[7] = H4[7] - R(1.0 / 7.0) * Syz;                             // xxyz
    h[8] = H4[8] - R(1.0 / 7.0) * Sxz;                             // xyyz
    h[9] = H4[9] - R(1.0 / 7.0) * (Sxx + Szz) + R(0.2 / 7.0) * S4;    // xxzz
    h[10] = H4[10] - R(1.0 / 7.0) * Sxy;                           // xyzz
    h[11] = H4[11] - R(3.0 / 7.0) * Sxz;                           // xzzz
    h[12] = H4[12] - R(1.0 / 7.0) * (Syy + Szz) + R(0.2 / 7.0) * S4;  // yyzz
    h[13] = H4[13] - R(3.0 / 7.0) * Syz;                           // yzzz
    h[14] = H4[14] - R(6.0 / 7.0) * Szz + R(0.6 / 7.0) * S4;          // zzzz
}

__global__ void k_open(TsphDevTree T, const unsigned long long *__restrict__ maxd2,
                       double twoOverSqrt3, double dCrit, int high) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= T.dcnt[0]) return;
    double Bmax = sqrt(__longlong_as_double((long long)maxd2[i]));
    double dOpen = __ddiv_rn(xmul(twoOverSqrt3, Bmax), dCrit);
    if (dOpen < Bmax) dOpen = Bmax;
    double fOpen2 = xmul(dOpen, dOpen);
    if (T.pUpper[i] < T.pLower[i]) { Bmax = 0.0; fOpen2 = 0.0; }
    T.Bmax[i] = Bmax;
    T.fOpen2[i] = fOpen2;
    float hx, lx, hy, ly, hz, lz;
    split2f(T.r[3 * i], hx, lx);
    split2f(T.r[3 * i + 1], hy, ly);
    split2f(T.r[3 * i + 2], hz, lz);
    T.wcomh[i] = make_float4(hx, hy, hz, (float)fOpen2);
    T.wcoml[i] = make_float4(lx, ly, lz, (float)T.fSoft[i]);
    T.wlink[i] = make_int4(T.pLower[i], T.pUpper[i] - T.pLower[i] + 1, T.upper[i], 0);
    const double *q = &T.Q[6 * i];
    T.wmom0[i] = make_float4((float)T.fMass[i], (float)q[0], (float)q[1], (float)q[2]);
    T.wmom1[i] = make_float4((float)q[3], (float)q[4], (float)q[5], (float)T.fSoft[i]);
    if (high == 2) {   // FP32 moments: the FP32 copies only
        const float *M3f = reinterpret_cast<const float *>(T.M3);
        const float *M4f = reinterpret_cast<const float *>(T.M4);
        float M[10], H4[15], oh[25];
#pragma unroll
        for (int k = 0; k < 10; ++k) M[k] = M3f[10 * (size_t)i + k];
#pragma unroll
        for (int k = 0; k < 15; ++k) H4[k] = M4f[15 * (size_t)i + k];
        reduce_high<float>(M, H4, oh, oh + 10);
        const bool empty = T.pUpper[i] < T.pLower[i];
#pragma unroll
        for (int k = 0; k < 25; ++k) T.wOH[25 * (size_t)i + k] = empty ? 0.0f : oh[k];
    } else if (high) {
        double M[10], H4[15], oh[25];
#pragma unroll
        for (int k = 0; k < 10; ++k) M[k] = T.M3[10 * (size_t)i + k];
#pragma unroll
        for (int k = 0; k < 15; ++k) H4[k] = T.M4[15 * (size_t)i + k];
        reduce_high<double>(M, H4, oh, oh + 10);
        if (T.pUpper[i] < T.pLower[i])
            for (int k = 0; k < 25; ++k) oh[k] = 0.0;
#pragma unroll
        for (int k = 0; k < 25; ++k) {
            T.OH[25 * (size_t)i + k] = oh[k];
            T.wOH[25 * (size_t)i + k] = (float)oh[k];
        }
    }
}

__global__ void k_parts32(int n, const double *__restrict__ x, const double *__restrict__ y,
                          const double *__restrict__ z, const double *__restrict__ m,
                          const double *__restrict__ h, float4 *ph, float4 *pl) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    float hx, lx, hy, ly, hz, lz;
    split2f(x[p], hx, lx);
    split2f(y[p], hy, ly);
    split2f(z[p], hz, lz);
    ph[p] = make_float4(hx, hy, hz, (float)m[p]);
    pl[p] = make_float4(lx, ly, lz, (float)h[p]);
}

// ---------------------------------------------------------------------------
// host driver
// ---------------------------------------------------------------------------
#define TFREE(p) do { if (p) cudaFree(p); (p) = nullptr; } while (0)
void tsph_free_tree(TsphDevTree &T) {
    TFREE(T.pLower); TFREE(T.pUpper); TFREE(T.iDim); TFREE(T.upper); TFREE(T.dlink); TFREE(T.skip);
    TFREE(T.fSplit); TFREE(T.bnd); TFREE(T.fMass); TFREE(T.fSoft); TFREE(T.r);
    TFREE(T.fOpen2); TFREE(T.Bmax); TFREE(T.Q); TFREE(T.wcomh); TFREE(T.wcoml);
    TFREE(T.wlink); TFREE(T.wmom0); TFREE(T.wmom1); TFREE(T.leaves); TFREE(T.parent);
    TFREE(T.M3); TFREE(T.M4); TFREE(T.OH); TFREE(T.wOH);
    T.highCap = 0;
    TFREE(T.rLo); TFREE(T.rHi); TFREE(T.sysRoot); TFREE(T.rEnd); TFREE(T.dcnt);
    if (T.brec) cudaFree(T.brec);
    T.brec = nullptr;
    TFREE(T.bact);
    free(T.hLo);
    free(T.hHi);
    T.hLo = T.hHi = nullptr;
    T.cap = 0;
    T.rCap = 0;
}

void tsph_free_build(TsphBuildBufs &B) {
    TFREE(B.f_node[0]); TFREE(B.f_node[1]); TFREE(B.f_split); TFREE(B.f_rank); TFREE(B.tasks);
    TFREE(B.chunkScan); TFREE(B.ctot); TFREE(B.coff); TFREE(B.chunkNode);
    TFREE(B.t_lo); TFREE(B.t_hi); TFREE(B.t_dim); TFREE(B.t_child); TFREE(B.t_size);
    TFREE(B.t_pre); TFREE(B.t_root); TFREE(B.t_loc); TFREE(B.t_split); TFREE(B.t_bnd);
    TFREE(B.maxd2); TFREE(B.visit); TFREE(B.leafFlag); TFREE(B.leafScan); TFREE(B.ctl);
    B.tcap = B.topCap = B.nodeScratchCap = 0;
}

// Final node arrays: a forest over n particles in nR trees has at most
// 2n - nR nodes.
static int ensure_nodes(tsph_ctx *ctx, TsphDevTree &T, int nNodes) {
    TsphBuildBufs &B = ctx->B;
    int rc = 0;
    if (ctx->capturing && (nNodes > T.cap || !T.pLower || B.nodeScratchCap < nNodes))
        return TSPH_ERR_STATE;   // no allocation inside a capture
    if (nNodes > T.cap || !T.pLower) {
        int cap = nNodes + 64;
        rc |= tsph_grow(ctx, &T.pLower, cap);
        rc |= tsph_grow(ctx, &T.pUpper, cap);
        rc |= tsph_grow(ctx, &T.iDim, cap);
        rc |= tsph_grow(ctx, &T.upper, cap);
        rc |= tsph_grow(ctx, &T.dlink, cap);
        rc |= tsph_grow(ctx, &T.skip, cap);
        rc |= tsph_grow(ctx, &T.parent, cap);
        rc |= tsph_grow(ctx, &T.fSplit, cap);
        rc |= tsph_grow(ctx, &T.bnd, (size_t)6 * cap);
        rc |= tsph_grow(ctx, &T.fMass, cap);
        rc |= tsph_grow(ctx, &T.fSoft, cap);
        rc |= tsph_grow(ctx, &T.r, (size_t)3 * cap);
        rc |= tsph_grow(ctx, &T.fOpen2, cap);
        rc |= tsph_grow(ctx, &T.Bmax, cap);
        rc |= tsph_grow(ctx, &T.Q, (size_t)6 * cap);
        rc |= tsph_grow(ctx, &T.wcomh, cap);
        rc |= tsph_grow(ctx, &T.wcoml, cap);
        rc |= tsph_grow(ctx, &T.wlink, cap);
        rc |= tsph_grow(ctx, &T.wmom0, cap);
        rc |= tsph_grow(ctx, &T.wmom1, cap);
        rc |= tsph_grow(ctx, &T.leaves, cap);
        rc |= tsph_grow(ctx, &T.brec, (size_t)4 * cap);
        rc |= tsph_grow(ctx, &T.bact, (size_t)6 * cap);
        if (rc) return TSPH_ERR_NOMEM;
        T.cap = cap;
    }
    // per-node scratch shared by both trees (sized to the larger)
    if (B.nodeScratchCap < T.cap) {
        rc |= tsph_grow(ctx, &B.maxd2, T.cap);
        rc |= tsph_grow(ctx, &B.visit, T.cap);
        rc |= tsph_grow(ctx, &B.leafFlag, T.cap);
        rc |= tsph_grow(ctx, &B.leafScan, T.cap);
        if (rc) return TSPH_ERR_NOMEM;
        B.nodeScratchCap = T.cap;
    }
    return TSPH_OK;
}

// Temporary nodes: top-phase nodes all hold more than the task size (at
// least 1024 particles), so a level has at most n/1024 of them.
static int ensure_temp(tsph_ctx *ctx, int n, int nR) {
    TsphBuildBufs &B = ctx->B;
    int topCap = nR + 2 * (n / 1024 + 1) * TSPH_MAX_LEVELS + 512;
    int tcap = topCap + 2 * n;
    if (B.ctl && topCap <= B.topCap && tcap <= B.tcap) return TSPH_OK;
    if (ctx->capturing) return TSPH_ERR_STATE;   // no allocation inside a capture
    topCap += topCap / 8;
    tcap = topCap + 2 * (n + n / 8 + 64);
    int rc = 0;
    rc |= tsph_grow(ctx, &B.f_node[0], topCap);
    rc |= tsph_grow(ctx, &B.f_node[1], topCap);
    rc |= tsph_grow(ctx, &B.f_split, topCap);
    rc |= tsph_grow(ctx, &B.f_rank, topCap);
    rc |= tsph_grow(ctx, &B.tasks, topCap);
    rc |= tsph_grow(ctx, &B.chunkScan, topCap);
    rc |= tsph_grow(ctx, &B.ctot, n / TB_CHUNK + topCap + 2);
    rc |= tsph_grow(ctx, &B.coff, n / TB_CHUNK + topCap + 2);
    rc |= tsph_grow(ctx, &B.chunkNode, n / TB_CHUNK + topCap + 2);
    rc |= tsph_grow(ctx, &B.t_lo, tcap);
    rc |= tsph_grow(ctx, &B.t_hi, tcap);
    rc |= tsph_grow(ctx, &B.t_dim, tcap);
    rc |= tsph_grow(ctx, &B.t_child, tcap);
    rc |= tsph_grow(ctx, &B.t_size, tcap);
    rc |= tsph_grow(ctx, &B.t_pre, tcap);
    rc |= tsph_grow(ctx, &B.t_root, tcap);
    rc |= tsph_grow(ctx, &B.t_loc, tcap);
    rc |= tsph_grow(ctx, &B.t_split, tcap);
    rc |= tsph_grow(ctx, &B.t_bnd, (size_t)6 * tcap);
    if (!B.ctl) rc |= tsph_grow(ctx, &B.ctl, 1);
    if (rc) return TSPH_ERR_NOMEM;
    B.topCap = topCap;
    B.tcap = tcap;
    return TSPH_OK;
}

// System (range) of every tree-order slot: the last range starting at or
// before it.
__global__ void k_fill_rid(int n, int nR, const int *__restrict__ rLo, int *rid) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    int a = 0, b = nR - 1;
    while (a < b) {
        int c = (a + b + 1) >> 1;
        if (rLo[c] <= p) a = c; else b = c - 1;
    }
    rid[p] = a;
}

// The forest's trees: nR consecutive particle ranges of the given sizes
// (each at least 1), in tree order.  A single system is one range.
int tsph_set_ranges(tsph_ctx *ctx, TsphDevParts &P, TsphDevTree &T, int n, int nR,
                    const int *counts) {
    if (nR < 1) return TSPH_ERR_ARG;
    int rc = 0;
    if (T.rCap < nR || !T.rLo) {
        rc |= tsph_grow(ctx, &T.rLo, nR);
        rc |= tsph_grow(ctx, &T.rHi, nR);
        rc |= tsph_grow(ctx, &T.sysRoot, nR);
        rc |= tsph_grow(ctx, &T.rEnd, nR);
        if (!T.dcnt) rc |= tsph_grow(ctx, &T.dcnt, 2);
        if (rc) return TSPH_ERR_NOMEM;
        free(T.hLo);
        free(T.hHi);
        T.hLo = (int *)malloc(sizeof(int) * nR);
        T.hHi = (int *)malloc(sizeof(int) * nR);
        if (!T.hLo || !T.hHi) return TSPH_ERR_NOMEM;
        T.rCap = nR;
    }
    if (!P.rid || ctx->B.cap < n) return TSPH_ERR_STATE;
    int lo = 0, mx = 0;
    for (int r = 0; r < nR; ++r) {
        if (counts[r] < 1 || lo + counts[r] > n) return TSPH_ERR_ARG;
        T.hLo[r] = lo;
        T.hHi[r] = lo + counts[r] - 1;
        mx = counts[r] > mx ? counts[r] : mx;
        lo += counts[r];
    }
    if (lo != n) return TSPH_ERR_ARG;
    T.nR = nR;
    T.maxRange = mx;
    // the small range tables from the host, the per-slot system on the device
    TSPH_CK(cudaMemcpyAsync(T.rLo, T.hLo, sizeof(int) * nR, cudaMemcpyHostToDevice, ctx->stream));
    TSPH_CK(cudaMemcpyAsync(T.rHi, T.hHi, sizeof(int) * nR, cudaMemcpyHostToDevice, ctx->stream));
    if (n > 0) {
        if (nR == 1) {
            TSPH_CK(cudaMemsetAsync(P.rid, 0, sizeof(int) * (size_t)n, ctx->stream));
        } else {
            k_fill_rid<<<tsph_blocks(n, 256), 256, 0, ctx->stream>>>(n, nR, T.rLo, P.rid);
            TSPH_LAUNCH_CK("k_fill_rid");
        }
    }
    return TSPH_OK;
}

// Task size: the largest node handed whole to one CTA.
// By default, the shared-memory limit, lowered for small particle sets so
// that there are tasks for every SM (about two per SM).
static int task_size(tsph_ctx *ctx, const TsphDevTree &T, int n) {
    int S = ctx->taskSize;
    if (S <= 0) {
        S = n / (4 * ctx->smCount);
        if (S > ST_DEFAULT_TASK) S = ST_DEFAULT_TASK;
    }
    if (S < 1024) S = 1024;
    return S;
}

// Activity of every tree slot in the final particle order: rung >= the
// context's active rung (msrActiveRung(actRung, 1)).
__global__ void k_tree_act(int n, const int *__restrict__ iord, const int *__restrict__ rung,
                           int actRung, int *act) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) act[i] = rung[iord[i]] >= actRung;
}

static int build_tree_body(tsph_ctx *ctx, TsphDevParts &P, TsphDevTree &T, int n, int nBucket);

// Masses and softenings of the particles in the order a build left them,
// from the caller-order state.
__global__ void k_gather_mass(int n, const double *__restrict__ cm, const double *__restrict__ ch,
                              TsphDevParts P, unsigned int *status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int o = P.iord[i];
    const double m = cm[o], h = ch[o];
    P.m[i] = m;
    P.h[i] = h;
    if (status && !isfinite(m + h)) atomicOr(status, 1u << TSPH_ERR_NONFINITE);
}

int tsph_build_tree(tsph_ctx *ctx, TsphDevParts &P, TsphDevTree &T, int n, int nBucket) {
    int rc = build_tree_body(ctx, P, T, n, nBucket);
    if (rc || n == 0) return rc;
    k_tree_act<<<tsph_blocks(n, 256), 256, 0, ctx->stream>>>(n, P.iord, ctx->C.rung, ctx->actRung, P.act);
    TSPH_LAUNCH_CK("k_tree_act");
    return TSPH_OK;
}

static int build_tree_body(tsph_ctx *ctx, TsphDevParts &P, TsphDevTree &T, int n, int nBucket) {
    TsphBuildBufs &B = ctx->B;
    const int BS = 256;
    if (nBucket < 1) return TSPH_ERR_ARG;
    if (n == 0) {
        // an empty bucket (pkdBuildBinary's bEmpty branch, pkd.c:2686-2714)
        int rc = ensure_nodes(ctx, T, 1);
        if (rc) return rc;
        static const int h6[4] = {0, -1, 1, 0};
        TSPH_CK(cudaMemcpyAsync(T.pLower, &h6[0], sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
        TSPH_CK(cudaMemcpyAsync(T.pUpper, &h6[1], sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
        if (T.dcnt)
            TSPH_CK(cudaMemcpyAsync(T.dcnt, &h6[2], 2 * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
        TSPH_CK(cudaStreamSynchronize(ctx->stream));
        T.nNodes = 1;
        T.nLeaves = 0;
        return TSPH_OK;
    }
    if (T.nR < 1 || T.hHi[T.nR - 1] != n - 1) return TSPH_ERR_STATE;
    const int nR = T.nR;
    int rc = ensure_temp(ctx, n, nR);
    if (rc) return rc;
    const int nodeNeed = 2 * n;
    rc = ensure_nodes(ctx, T, nodeNeed);
    if (rc) return rc;
    const int S = task_size(ctx, T, n);
    int F = 0;
    for (int r = 0; r < nR; ++r)
        if (T.hHi[r] - T.hLo[r] + 1 > S) ++F;
    k_roots<<<1, 1024, 0, ctx->stream>>>(nR, T.rLo, T.rHi, S, B.t_lo, B.t_hi, B.t_bnd, B.f_node[0],
                                         B.tasks, B.ctl);
    TSPH_LAUNCH_CK("k_roots");
    TSPH_CK(cudaMemsetAsync(B.t_root + B.topCap, 0xff, sizeof(int) * 2 * (size_t)n, ctx->stream));
    // top phase: levels are launched in batches; the frontier of each level
    // is known on the device only, the host bounds it (every split node of
    // a level holds more than S particles, so a level has at most 2n/S
    // children) and looks at the true size now and then
    const int TOP_BATCH = 4;
    int levelStart[TSPH_MAX_LEVELS + 2];
    int cur = 0, level = 0;
    const int Fcap = 2 * (n / S) + 2;
    int Fb = F;
    // a captured build runs a fixed number of levels (its preparation's
    // depth + 1: one spare level) with no host look; what is left becomes
    // subtree tasks
    const bool cap = ctx->capturing;
    const int Lmax = cap ? (T.lastTopLevels + 1 < TSPH_MAX_LEVELS - 2 ? T.lastTopLevels + 1
                                                                      : TSPH_MAX_LEVELS - 2)
                         : TSPH_MAX_LEVELS - 2;
    // the first look comes at the last build's depth (the same particles
    // rebuilt give the same depth), then every TOP_BATCH levels
    const int look0 = (!cap && T.lastTopLevels > 0) ? T.lastTopLevels : TOP_BATCH;
    // level 0: the bounds of the roots; every later frontier node gets its
    // bounds from its parent's flag pass
    if (Fb > 0) {
        const int slots = n / TB_CHUNK + Fb + 1;
        if (Fb <= LB_MAX) {
            k_level_chunks<<<1, LB_BS, 0, ctx->stream>>>(Fb, 0, S, B.ctl, B.f_node[0], B.t_lo,
                                                         B.t_hi, B.chunkScan, B.chunkNode);
            TSPH_LAUNCH_CK("k_level_chunks");
        } else {
            k_chunk_count<<<tsph_blocks(Fb, BS), BS, 0, ctx->stream>>>(Fb, 0, S, B.ctl, B.f_node[0],
                                                                        B.t_lo, B.t_hi, B.ctot);
            TSPH_LAUNCH_CK("k_chunk_count");
            rc = tsph_scan_inclusive(ctx, B.ctot, B.chunkScan, Fb);
            if (rc) return rc;
            k_chunk_map<<<tsph_blocks(slots, BS), BS, 0, ctx->stream>>>(Fb, B.chunkScan, B.chunkNode);
            TSPH_LAUNCH_CK("k_chunk_map");
        }
        k_bounds_chunks<<<slots, TB_BS, 0, ctx->stream>>>(Fb, B.f_node[0], B.chunkScan, B.chunkNode,
                                                          B.t_lo, B.t_hi, P.x, P.y, P.z, B.t_bnd);
        TSPH_LAUNCH_CK("k_bounds_chunks");
    }
    while (Fb > 0 && level < Lmax) {
        if (!cap && level + 2 >= TSPH_MAX_LEVELS) return TSPH_ERR_TREE_DEPTH;
        const int slots = n / TB_CHUNK + Fb + 1;     // >= chunks of any frontier
        const bool small = Fb <= LB_MAX;              // frontier work in single blocks
        if (small) {
            k_level_prep<<<1, LB_BS, 0, ctx->stream>>>(
                Fb, level, B.f_node[cur], S, nBucket, B.t_lo, B.t_hi, B.t_dim, B.t_child, B.t_size,
                B.t_split, B.t_bnd, B.f_split, B.f_rank, B.tasks, B.ctl, B.chunkScan, B.chunkNode,
                B.topCap);
            TSPH_LAUNCH_CK("k_level_prep");
        } else {
            k_top_split<<<tsph_blocks(Fb, BS), BS, 0, ctx->stream>>>(
                Fb, level, B.f_node[cur], S, nBucket, B.t_lo, B.t_hi, B.t_dim, B.t_child,
                B.t_size, B.t_split, B.t_bnd, B.f_split, B.tasks, B.ctl);
            TSPH_LAUNCH_CK("k_top_split");
            rc = tsph_scan_inclusive(ctx, B.f_split, B.f_rank, Fb);
            if (rc) return rc;
            k_child_keys<<<tsph_blocks(Fb, BS), BS, 0, ctx->stream>>>(Fb, level, B.f_split, B.f_rank,
                                                                       B.ctl, B.topCap, B.t_bnd);
            TSPH_LAUNCH_CK("k_child_keys");
            k_chunk_count<<<tsph_blocks(Fb, BS), BS, 0, ctx->stream>>>(Fb, level, S, B.ctl,
                                                                        B.f_node[cur], B.t_lo,
                                                                        B.t_hi, B.ctot);
            TSPH_LAUNCH_CK("k_chunk_count");
            rc = tsph_scan_inclusive(ctx, B.ctot, B.chunkScan, Fb);
            if (rc) return rc;
            k_chunk_map<<<tsph_blocks(slots, BS), BS, 0, ctx->stream>>>(Fb, B.chunkScan, B.chunkNode);
            TSPH_LAUNCH_CK("k_chunk_map");
        }
        k_flag_chunks<<<slots, TB_BS, 0, ctx->stream>>>(Fb, level, slots, B.f_node[cur], B.chunkScan,
                                                        B.chunkNode, B.t_lo, B.t_hi, B.t_dim, B.t_split, P.x,
                                                        P.y, P.z, B.scan, B.ctot, B.ctl, B.f_rank,
                                                        B.topCap, B.t_bnd);
        TSPH_LAUNCH_CK("k_flag_chunks");
        if (slots <= LB_MAX) {
            k_scan_small<<<1, LB_BS, 0, ctx->stream>>>(slots, B.ctot, B.coff);
            TSPH_LAUNCH_CK("k_scan_small");
        } else {
            rc = tsph_scan_inclusive(ctx, B.ctot, B.coff, slots);
            if (rc) return rc;
        }
        k_mark_chunks<<<slots, TB_BS, 0, ctx->stream>>>(Fb, B.f_node[cur], B.chunkScan, B.chunkNode, B.coff,
                                                        B.t_lo, B.t_hi, B.t_dim, B.scan, B.lt,
                                                        B.seg);
        TSPH_LAUNCH_CK("k_mark_chunks");
        k_pair_chunks<<<slots, TB_BS, 0, ctx->stream>>>(Fb, B.f_node[cur], B.chunkScan, B.chunkNode, B.coff,
                                                        B.t_lo, B.t_dim, B.scan, B.lt, B.seg, P.x,
                                                        P.y, P.z, P.iord);
        TSPH_LAUNCH_CK("k_pair_chunks");
        k_top_children<<<tsph_blocks(Fb, BS), BS, 0, ctx->stream>>>(
            Fb, level, B.f_node[cur], B.f_split, B.f_rank, B.chunkScan, B.coff, B.topCap, B.t_lo,
            B.t_hi, B.t_child, B.t_bnd, B.f_node[1 - cur], B.ctl);
        TSPH_LAUNCH_CK("k_top_children");
        cur = 1 - cur;
        ++level;
        Fb = 2 * Fb < Fcap ? 2 * Fb : Fcap;
        if (!cap && level >= look0 && (level - look0) % TOP_BATCH == 0) {
            TSPH_CK(cudaMemcpyAsync(B.hostCount, &B.ctl->levF[level], sizeof(int),
                                    cudaMemcpyDeviceToHost, ctx->stream));
            TSPH_CK(cudaStreamSynchronize(ctx->stream));
            if (B.hostCount[0] == 0) break;
        }
    }
    if (level > 0) {
        k_frontier_to_tasks<<<tsph_blocks(Fb, BS), BS, 0, ctx->stream>>>(Fb, level, B.f_node[cur],
                                                                         B.t_dim, B.tasks, B.ctl);
        TSPH_LAUNCH_CK("k_frontier_to_tasks");
    }
    // the true level table (levels after the last split launched empty)
    int levF[TSPH_MAX_LEVELS + 2];
    int topLevels = 1;
    levelStart[0] = 0;
    levelStart[1] = nR;
    if (cap) {
        topLevels = level + 1;               // ranges stay on the device
    } else if (level > 0) {
        TSPH_CK(cudaMemcpyAsync(levF, B.ctl->levF, sizeof(int) * (level + 1),
                                cudaMemcpyDeviceToHost, ctx->stream));
        TSPH_CK(cudaMemcpyAsync(levelStart, B.ctl->levStart, sizeof(int) * (level + 2),
                                cudaMemcpyDeviceToHost, ctx->stream));
        TSPH_CK(cudaStreamSynchronize(ctx->stream));
        // level 0 holds the roots; level L >= 1 exists while levF[L] > 0
        while (topLevels < level && levF[topLevels] > 0) ++topLevels;
        if (topLevels == level && levF[level] > 0) return TSPH_ERR_TREE_DEPTH;
    }
    if (!cap) T.lastTopLevels = topLevels;
    B.topLevels = topLevels;
    // subtree phase
    BuildArgs A;
    A.x = P.x; A.y = P.y; A.z = P.z; A.m = P.m; A.h = P.h; A.iord = P.iord;
    A.seg = B.seg; A.lt = B.lt; A.scan = B.scan;
    A.t_lo = B.t_lo; A.t_hi = B.t_hi; A.t_dim = B.t_dim; A.t_child = B.t_child;
    A.t_size = B.t_size; A.t_root = B.t_root; A.t_loc = B.t_loc;
    A.t_split = B.t_split; A.t_bnd = B.t_bnd;
    A.tasks = B.tasks; A.ctl = B.ctl;
    A.topCap = B.topCap; A.nBucket = nBucket;
    // shared memory sized to the task size (positions, flags, scan, order)
    A.scap = S < ST_SCAP ? S : ST_SCAP;
    const size_t smem = ((size_t)A.scap * ST_BYTES_PER + 15) & ~(size_t)15;
    // resident CTAs per shared-memory size (the gravity and gas trees of one
    // step may use different task sizes; a capture finds both cached)
    int slot = -1;
    for (int k = 0; k < 4 && slot < 0; ++k)
        if (ctx->subtreeBlocks[k] > 0 && ctx->subtreeSmem[k] == smem) slot = k;
    if (slot < 0) {
        if (ctx->capturing) return TSPH_ERR_STATE;
        if (!ctx->subtreeAttr) {
            TSPH_CK(cudaFuncSetAttribute(k_subtree, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(ST_SCAP * ST_BYTES_PER)));
            ctx->subtreeAttr = true;
        }
        int per = 0;
        TSPH_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_subtree, ST_BS, smem));
        for (slot = 0; slot < 4 && ctx->subtreeBlocks[slot] > 0; ++slot) {}
        if (slot == 4) {   // full: keep the newest three
            for (int k = 0; k < 3; ++k) {
                ctx->subtreeBlocks[k] = ctx->subtreeBlocks[k + 1];
                ctx->subtreeSmem[k] = ctx->subtreeSmem[k + 1];
            }
            slot = 3;
        }
        ctx->subtreeBlocks[slot] = (per > 0 ? per : 1) * ctx->smCount;
        ctx->subtreeSmem[slot] = smem;
    }
    k_subtree<<<ctx->subtreeBlocks[slot], ST_BS, smem, ctx->stream>>>(A);
    TSPH_LAUNCH_CK("k_subtree");
    // masses and softenings in the final order (the build moved only the
    // positions and caller indices); a non-finite one is bad input
    k_gather_mass<<<tsph_blocks(n, BS), BS, 0, ctx->stream>>>(
        n, ctx->C.m, ctx->C.h, P, &P == &ctx->P ? &ctx->dCnt->status : nullptr);
    TSPH_LAUNCH_CK("k_gather_mass");
    // numbering
    const int levBound = nR > Fcap ? nR : Fcap;
    for (int l = topLevels - 1; l >= 0; --l) {
        if (cap) {
            k_size_dev<<<tsph_blocks(levBound, BS), BS, 0, ctx->stream>>>(l, B.ctl, B.t_child,
                                                                         B.t_size);
        } else {
            int a = levelStart[l], b = levelStart[l + 1];
            k_size<<<tsph_blocks(b - a, BS), BS, 0, ctx->stream>>>(a, b, B.t_child, B.t_size);
        }
        TSPH_LAUNCH_CK("k_size");
    }
    k_root_pre<<<1, 1024, 0, ctx->stream>>>(nR, B.t_size, B.t_pre, T.sysRoot, T.rEnd, B.ctl);
    TSPH_LAUNCH_CK("k_root_pre");
    for (int l = 0; l < topLevels; ++l) {
        if (cap) {
            k_pre_dev<<<tsph_blocks(levBound, BS), BS, 0, ctx->stream>>>(l, B.ctl, B.t_child,
                                                                        B.t_size, B.t_pre);
        } else {
            int a = levelStart[l], b = levelStart[l + 1];
            k_pre<<<tsph_blocks(b - a, BS), BS, 0, ctx->stream>>>(a, b, B.t_child, B.t_size,
                                                                  B.t_pre);
        }
        TSPH_LAUNCH_CK("k_pre");
    }
    k_slot_pre<<<tsph_blocks(2 * (long long)n, BS), BS, 0, ctx->stream>>>(B.topCap, 2 * n, B.t_root,
                                                                          B.t_loc, B.t_pre);
    TSPH_LAUNCH_CK("k_slot_pre");
    TSPH_CK(cudaMemsetAsync(B.leafFlag, 0, sizeof(int) * (size_t)nodeNeed, ctx->stream));
    const int scatN = B.topCap + 2 * n;
    k_scatter_nodes<<<tsph_blocks(scatN, BS), BS, 0, ctx->stream>>>(
        B.topCap, scatN, B.ctl, B.t_lo, B.t_hi, B.t_dim, B.t_child, B.t_size, B.t_pre, B.t_root,
        B.t_split, B.t_bnd, P.rid, nR, T, B.leafFlag);
    TSPH_LAUNCH_CK("k_scatter_nodes");
    rc = tsph_scan_inclusive(ctx, B.leafFlag, B.leafScan, nodeNeed);
    if (rc) return rc;
    k_leaf_list<<<tsph_blocks(nodeNeed, BS), BS, 0, ctx->stream>>>(B.ctl, B.leafFlag, B.leafScan,
                                                                   T.leaves, T.dcnt);
    TSPH_LAUNCH_CK("k_leaf_list");
    if (!ctx->capturing) {
        TSPH_CK(cudaMemcpyAsync(B.hostCount, T.dcnt, 2 * sizeof(int), cudaMemcpyDeviceToHost,
                                ctx->stream));
        TSPH_CK(cudaMemcpyAsync(B.hostCount + 2, &B.ctl->status, sizeof(int), cudaMemcpyDeviceToHost,
                                ctx->stream));
        TSPH_CK(cudaStreamSynchronize(ctx->stream));
        int st = B.hostCount[2];
        for (int k = 1; k < 32; ++k)
            if (st & (1 << k)) return k;
        T.nNodes = B.hostCount[0];
        T.nLeaves = B.hostCount[1];
    } else {
        T.nNodes = nodeNeed;     // upper bounds; the device holds the counts
        T.nLeaves = n;
    }
    return TSPH_OK;
}

int tsph_tree_moments(tsph_ctx *ctx, TsphDevParts &P, TsphDevTree &T, int n, double dTheta, int order,
                      int fp32) {
    TsphBuildBufs &B = ctx->B;
    const int BS = 256;
    if (n == 0) return TSPH_OK;
    const int nodeNeed = 2 * n;
    // octopole/hexadecapole moments: FP64 for the FP64 walk (1), FP32 for
    // the FP32 walk (2), whose cells read FP32 copies of them only
    const int high = order >= 3 ? (fp32 ? 2 : 1) : 0;
    if (high && T.highCap < T.cap) {   // octopole/hexadecapole storage, on first use
        if (ctx->capturing) return TSPH_ERR_STATE;
        int rc = tsph_grow(ctx, &T.M3, (size_t)10 * T.cap);
        rc |= tsph_grow(ctx, &T.M4, (size_t)15 * T.cap);
        rc |= tsph_grow(ctx, &T.OH, (size_t)25 * T.cap);
        rc |= tsph_grow(ctx, &T.wOH, (size_t)25 * T.cap);
        if (rc) return TSPH_ERR_NOMEM;
        T.highCap = T.cap;
    }
    // the FP32 particle records on the side stream beside k_moments (FP64
    // bound at low issue); the Bmax passes wait for them
    TSPH_CK(cudaEventRecord(ctx->evBuilt, ctx->stream));
    TSPH_CK(cudaStreamWaitEvent(ctx->side, ctx->evBuilt, 0));
    k_parts32<<<tsph_blocks(n, BS), BS, 0, ctx->side>>>(n, P.x, P.y, P.z, P.m, P.h, P.ph, P.pl);
    TSPH_LAUNCH_CK("k_parts32");
    TSPH_CK(cudaEventRecord(ctx->evParts, ctx->side));
    TSPH_CK(cudaMemsetAsync(B.visit, 0, sizeof(int) * (size_t)nodeNeed, ctx->stream));
    k_moments<<<tsph_blocks(n, MOM_BS), MOM_BS, 0, ctx->stream>>>(T, P.x, P.y, P.z, P.m, P.h, B.visit, high);
    TSPH_LAUNCH_CK("k_moments");
    TSPH_CK(cudaEventRecord(ctx->evMoments, ctx->stream));   // the root cell is final
    TSPH_CK(cudaStreamWaitEvent(ctx->stream, ctx->evParts, 0));
    k_zero_u64<<<tsph_blocks(nodeNeed, BS), BS, 0, ctx->stream>>>(B.maxd2, nodeNeed);
    TSPH_LAUNCH_CK("k_zero_u64");
    // the per-node arrival counters of k_moments are free again: max of lo
    TSPH_CK(cudaMemsetAsync(B.visit, 0, sizeof(int) * (size_t)nodeNeed, ctx->stream));
    const float eabs = (float)(ldexp(1.0, -43) * (ctx->coordScale > 0 ? ctx->coordScale : 1.0)) + 1e-30f;
    unsigned int *maxLo = reinterpret_cast<unsigned int *>(B.visit);
    k_bmax_lo<<<tsph_blocks(n, BS), BS, 0, ctx->stream>>>(n, T, P.ph, P.pl, P.rid, eabs, maxLo);
    TSPH_LAUNCH_CK("k_bmax_lo");
    k_bmax_exact<<<tsph_blocks(n, BS), BS, 0, ctx->stream>>>(n, T, P.x, P.y, P.z, P.ph, P.pl, P.rid,
                                                             eabs, maxLo, B.maxd2);
    TSPH_LAUNCH_CK("k_bmax_exact");
    const double twoOverSqrt3 = 2 / sqrt(3.0);
    k_open<<<tsph_blocks(nodeNeed, BS), BS, 0, ctx->stream>>>(T, B.maxd2, twoOverSqrt3, dTheta, high);
    TSPH_LAUNCH_CK("k_open");
    return TSPH_OK;
}
