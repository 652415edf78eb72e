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
// level kernels
// ---------------------------------------------------------------------------
__global__ void k_init_build(int *seg, int n, int *f_lo, int *f_hi, int *f_node) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) seg[p] = 0;
    if (p == 0) { f_lo[0] = 0; f_hi[0] = n - 1; f_node[0] = 0; }
}

__global__ void k_fbnd_init(unsigned long long *f_bnd, int F) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= F) return;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        f_bnd[6 * s + k] = ~0ULL;      // min
        f_bnd[6 * s + 3 + k] = 0ULL;   // max
    }
}

// Segmented min/max of positions per frontier node.  Particles of one node
// are contiguous, so runs inside a warp are reduced with shuffles and the
// run head issues the atomics.
__global__ void k_bounds(const double *__restrict__ x, const double *__restrict__ y,
                         const double *__restrict__ z, const int *__restrict__ seg,
                         unsigned long long *f_bnd, int n) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    int lane = threadIdx.x & 31;
    int s = (p < n) ? seg[p] : -1;
    unsigned long long mn[3], mx[3];
    if (s >= 0) {
        mn[0] = mx[0] = dkey(x[p]);
        mn[1] = mx[1] = dkey(y[p]);
        mn[2] = mx[2] = dkey(z[p]);
    } else {
        mn[0] = mn[1] = mn[2] = ~0ULL;
        mx[0] = mx[1] = mx[2] = 0ULL;
    }
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int so = __shfl_down_sync(0xffffffffu, s, o);
        bool same = (lane + o < 32) && (so == s);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            unsigned long long a = __shfl_down_sync(0xffffffffu, mn[k], o);
            unsigned long long b = __shfl_down_sync(0xffffffffu, mx[k], o);
            if (same) {
                mn[k] = a < mn[k] ? a : mn[k];
                mx[k] = b > mx[k] ? b : mx[k];
            }
        }
    }
    int sp = __shfl_up_sync(0xffffffffu, s, 1);
    bool head = (lane == 0) || (sp != s);
    if (s >= 0 && head) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            atomicMin(&f_bnd[6 * s + k], mn[k]);
            atomicMax(&f_bnd[6 * s + 3 + k], mx[k]);
        }
    }
}

// Decide leaf/split for every frontier node (BuildBinary pkd.c:2460-2506).
__global__ void k_split(int F, const int *__restrict__ f_lo, const int *__restrict__ f_hi,
                        const int *__restrict__ f_node, const unsigned long long *__restrict__ f_bnd,
                        int nBucket, int *f_split, int *f_dim, double *f_fs,
                        int *t_lo, int *t_hi, int *t_dim, int *t_child, double *t_split,
                        double *t_bnd, int *t_level, int level) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= F) return;
    double bmin[3], bmax[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        bmin[k] = dunkey(f_bnd[6 * s + k]);
        bmax[k] = dunkey(f_bnd[6 * s + 3 + k]);
    }
    int lo = f_lo[s], hi = f_hi[s], node = f_node[s];
    int good = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k)
        if (bmax[k] > bmin[k]) good = 1;
    t_lo[node] = lo;
    t_hi[node] = hi;
    t_level[node] = level;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        t_bnd[6 * node + k] = bmin[k];
        t_bnd[6 * node + 3 + k] = bmax[k];
    }
    t_child[node] = -1;
    if ((hi - lo + 1 > nBucket) && good) {
        int d = 0;
        for (int j = 1; j < 3; ++j)
            if (xsub(bmax[j], bmin[j]) > xsub(bmax[d], bmin[d])) d = j;
        double fs = xmul(0.5, xadd(bmin[d], bmax[d]));
        f_split[s] = 1;
        f_dim[s] = d;
        f_fs[s] = fs;
        t_dim[node] = d;
        t_split[node] = fs;
    } else {
        f_split[s] = 0;
        f_dim[s] = -1;
        f_fs[s] = 0.0;
        t_dim[node] = -1;
        t_split[node] = 0.0;
    }
}

__global__ void k_flag(const double *__restrict__ x, const double *__restrict__ y,
                       const double *__restrict__ z, const int *__restrict__ seg,
                       const int *__restrict__ f_split, const int *__restrict__ f_dim,
                       const double *__restrict__ f_fs, int *lt, int n) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    int s = seg[p];
    int v = 0;
    if (s >= 0 && f_split[s]) {
        int d = f_dim[s];
        double r = d == 0 ? x[p] : (d == 1 ? y[p] : z[p]);
        v = r < f_fs[s] ? 1 : 0;
    }
    lt[p] = v;
}

// Swap each misplaced pair of the Hoare partition: the left element of rank
// t (t-th element >= fSplit in [lo, m)) with the right element of rank t
// (t-th element < fSplit counted from hi downwards in [m, hi]).
__global__ void k_swap(double *x, double *y, double *z, double *m, double *h, int *iord,
                       const int *__restrict__ seg, const int *__restrict__ f_split,
                       const int *__restrict__ f_lo, const int *__restrict__ f_hi,
                       const int *__restrict__ lt, const int *__restrict__ S, int n) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    int s = seg[p];
    if (s < 0 || !f_split[s] || lt[p]) return;
    int lo = f_lo[s], hi = f_hi[s];
    int Slo = lo > 0 ? S[lo - 1] : 0;
    int mid = lo + (S[hi] - Slo);          // first index of the upper part
    if (p >= mid) return;                  // already in place
    int ltBefore = (p > 0 ? S[p - 1] : 0) - Slo;
    int t = (p - lo) - ltBefore;           // rank among misplaced-left
    int target = S[hi] - t;                // S[q] value at the partner
    // smallest q in [mid, hi] with S[q] >= target
    int a = mid, b = hi;
    while (a < b) {
        int c = (a + b) >> 1;
        if (S[c] >= target) b = c; else a = c + 1;
    }
    int q = a;
    double t0;
    t0 = x[p]; x[p] = x[q]; x[q] = t0;
    t0 = y[p]; y[p] = y[q]; y[q] = t0;
    t0 = z[p]; z[p] = z[q]; z[q] = t0;
    t0 = m[p]; m[p] = m[q]; m[q] = t0;
    t0 = h[p]; h[p] = h[q]; h[q] = t0;
    int ti = iord[p]; iord[p] = iord[q]; iord[q] = ti;
}

__global__ void k_children(int F, const int *__restrict__ f_lo, const int *__restrict__ f_hi,
                           const int *__restrict__ f_node, const int *__restrict__ f_split,
                           const int *__restrict__ f_rank, const int *__restrict__ S,
                           int nTemp, int *f_m, int *t_child, int *nf_lo, int *nf_hi, int *nf_node) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= F || !f_split[s]) return;
    int lo = f_lo[s], hi = f_hi[s];
    int Slo = lo > 0 ? S[lo - 1] : 0;
    int mid = lo + (S[hi] - Slo);
    int r = f_rank[s] - 1;
    int c = nTemp + 2 * r;
    f_m[s] = mid;
    t_child[f_node[s]] = c;
    nf_lo[2 * r] = lo;
    nf_hi[2 * r] = mid - 1;
    nf_node[2 * r] = c;
    nf_lo[2 * r + 1] = mid;
    nf_hi[2 * r + 1] = hi;
    nf_node[2 * r + 1] = c + 1;
}

__global__ void k_seg(int *seg, const int *__restrict__ f_split, const int *__restrict__ f_rank,
                      const int *__restrict__ f_m, int n) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    int s = seg[p];
    if (s < 0) return;
    if (f_split[s]) seg[p] = 2 * (f_rank[s] - 1) + (p >= f_m[s] ? 1 : 0);
    else seg[p] = -1;
}

// subtree sizes, bottom-up over one BFS level [a, b)
__global__ void k_size(int a, int b, const int *__restrict__ t_child, int *t_size) {
    int v = a + blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= b) return;
    int c = t_child[v];
    t_size[v] = 1 + (c >= 0 ? t_size[c] + t_size[c + 1] : 0);
}

// depth-first (reference) index, top-down over one BFS level [a, b)
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

__global__ void k_scatter_nodes(int nTemp, const int *__restrict__ t_lo, const int *__restrict__ t_hi,
                                const int *__restrict__ t_dim, const int *__restrict__ t_child,
                                const int *__restrict__ t_size, const int *__restrict__ t_pre,
                                const double *__restrict__ t_split, const double *__restrict__ t_bnd,
                                TsphDevTree T, int *leafFlag) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nTemp) return;
    int i = t_pre[v];
    int c = t_child[v];
    T.pLower[i] = t_lo[v];
    T.pUpper[i] = t_hi[v];
    T.iDim[i] = t_dim[v];
    T.fSplit[i] = t_split[v];
#pragma unroll
    for (int k = 0; k < 6; ++k) T.bnd[6 * i + k] = t_bnd[6 * v + k];
    T.upper[i] = c >= 0 ? t_pre[c + 1] : -1;
    int nx = i + t_size[v];
    T.skip[i] = nx < nTemp ? nx : -1;
    leafFlag[i] = c < 0 ? 1 : 0;
}

__global__ void k_leaf_list(int nNodes, const int *__restrict__ leafFlag,
                            const int *__restrict__ leafScan, int *leaves) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nNodes || !leafFlag[i]) return;
    leaves[leafScan[i] - 1] = i;
}

// ---------------------------------------------------------------------------
// moments
// ---------------------------------------------------------------------------
// Leaf mass, softening and centre of mass summed in tree order exactly as
// BuildBinary (pkd.c:2559-2574); quadrupole summed as pkdCalcCell
// (pkd.c:2094-2130).
__global__ void k_leaf_moments(int nLeaves, const int *__restrict__ leaves, TsphDevTree T,
                               const double *__restrict__ x, const double *__restrict__ y,
                               const double *__restrict__ z, const double *__restrict__ m,
                               const double *__restrict__ h) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nLeaves) return;
    int i = leaves[b];
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
    double q[6] = {0, 0, 0, 0, 0, 0};
    for (int p = lo; p <= hi; ++p) {
        double fm = m[p];
        double dx = xsub(x[p], r0), dy = xsub(y[p], r1), dz = xsub(z[p], r2);
        q[0] = xadd(q[0], xmul(xmul(fm, dx), dx));
        q[1] = xadd(q[1], xmul(xmul(fm, dy), dy));
        q[2] = xadd(q[2], xmul(xmul(fm, dz), dz));
        q[3] = xadd(q[3], xmul(xmul(fm, dx), dy));
        q[4] = xadd(q[4], xmul(xmul(fm, dx), dz));
        q[5] = xadd(q[5], xmul(xmul(fm, dy), dz));
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) T.Q[6 * i + k] = q[k];
}

// Interior nodes of one BFS level: combine the two children in the
// reference's order (pkd.c:2522-2547); the quadrupole by the parallel-axis
// theorem (equal to the reference's direct sum up to rounding).
__global__ void k_combine(int a, int b, const int *__restrict__ t_child,
                          const int *__restrict__ t_pre, TsphDevTree T) {
    int v = a + blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= b) return;
    int c = t_child[v];
    if (c < 0) return;
    int i = t_pre[v], l = t_pre[c], u = t_pre[c + 1];
    double fMass = 0.0, fSoft = 0.0, r[3] = {0.0, 0.0, 0.0};
    double fm = T.fMass[l];
    fMass = xadd(fMass, fm);
    fSoft = xadd(fSoft, xmul(fm, T.fSoft[l]));
#pragma unroll
    for (int j = 0; j < 3; ++j) r[j] = xadd(r[j], xmul(fm, T.r[3 * l + j]));
    fm = T.fMass[u];
    fMass = xadd(fMass, fm);
    fSoft = xadd(fSoft, xmul(fm, T.fSoft[u]));
#pragma unroll
    for (int j = 0; j < 3; ++j) r[j] = xadd(r[j], xmul(fm, T.r[3 * u + j]));
    if (fMass > 0) {
        fSoft = __ddiv_rn(fSoft, fMass);
#pragma unroll
        for (int j = 0; j < 3; ++j) r[j] = __ddiv_rn(r[j], fMass);
    }
    T.fMass[i] = fMass;
    T.fSoft[i] = fSoft;
#pragma unroll
    for (int j = 0; j < 3; ++j) T.r[3 * i + j] = r[j];
    double q[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) q[k] = T.Q[6 * l + k] + T.Q[6 * u + k];
    int cc[2] = {l, u};
#pragma unroll
    for (int s = 0; s < 2; ++s) {
        int ch = cc[s];
        double mc = T.fMass[ch];
        double dx = T.r[3 * ch] - r[0], dy = T.r[3 * ch + 1] - r[1], dz = T.r[3 * ch + 2] - r[2];
        q[0] += mc * dx * dx;
        q[1] += mc * dy * dy;
        q[2] += mc * dz * dz;
        q[3] += mc * dx * dy;
        q[4] += mc * dx * dz;
        q[5] += mc * dy * dz;
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) T.Q[6 * i + k] = q[k];
}

__global__ void k_zero_u64(unsigned long long *a, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = 0ULL;
}

// Bmax of every node = max over its particles of |r - COM| (pkd.c:2086-2092).
// Each particle descends from the root to its leaf; max of d^2 is taken on
// the raw bits (non-negative doubles order like their bit patterns) and the
// square root taken once: sqrt is monotone, so this equals the max of the
// per-particle square roots the reference takes.
__global__ void k_bmax(int n, TsphDevTree T, const double *__restrict__ x,
                       const double *__restrict__ y, const double *__restrict__ z,
                       unsigned long long *maxd2) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    bool live = p < n;
    int i = 0;
    double px = live ? x[p] : 0.0, py = live ? y[p] : 0.0, pz = live ? z[p] : 0.0;
    unsigned mask = __ballot_sync(0xffffffffu, live);
    while (mask) {
        if (live) {
            double dx = xsub(px, T.r[3 * i]);
            double dy = xsub(py, T.r[3 * i + 1]);
            double dz = xsub(pz, T.r[3 * i + 2]);
            double d2 = xadd(xadd(xmul(dx, dx), xmul(dy, dy)), xmul(dz, dz));
            unsigned long long key = (unsigned long long)__double_as_longlong(d2);
            unsigned grp = __match_any_sync(mask, i);
            unsigned hiw = (unsigned)(key >> 32), low = (unsigned)key;
            unsigned mh = __reduce_max_sync(grp, hiw);
            unsigned ml = __reduce_max_sync(grp, hiw == mh ? low : 0u);
            int leader = __ffs(grp) - 1;
            if ((threadIdx.x & 31) == leader)
                atomicMax(&maxd2[i], ((unsigned long long)mh << 32) | ml);
            int up = T.upper[i];
            if (up < 0) live = false;
            else i = (p >= T.pLower[up]) ? up : i + 1;
        }
        mask = __ballot_sync(0xffffffffu, live);
    }
}

// Opening radius, OPEN_JOSH (pkd.c:2245-2253); walk copies in FP32.
__global__ void k_open(int nNodes, TsphDevTree T, const unsigned long long *__restrict__ maxd2,
                       double twoOverSqrt3, double dCrit) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nNodes) return;
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
    TFREE(T.pLower); TFREE(T.pUpper); TFREE(T.iDim); TFREE(T.upper); TFREE(T.skip);
    TFREE(T.fSplit); TFREE(T.bnd); TFREE(T.fMass); TFREE(T.fSoft); TFREE(T.r);
    TFREE(T.fOpen2); TFREE(T.Bmax); TFREE(T.Q); TFREE(T.wcomh); TFREE(T.wcoml);
    TFREE(T.wlink); TFREE(T.wmom0); TFREE(T.wmom1); TFREE(T.leaves);
    if (T.brec) cudaFree(T.brec);
    T.brec = nullptr;
    T.cap = 0;
}

static int ensure_nodes(tsph_ctx *ctx, TsphDevTree &T, int nNodes) {
    TsphBuildBufs &B = ctx->B;
    if (nNodes <= T.cap && T.pLower && nNodes <= B.nodeCap) return TSPH_OK;
    int cap = nNodes + nNodes / 4 + 64;
    int rc = 0;
    rc |= tsph_grow(ctx, &T.pLower, cap);
    rc |= tsph_grow(ctx, &T.pUpper, cap);
    rc |= tsph_grow(ctx, &T.iDim, cap);
    rc |= tsph_grow(ctx, &T.upper, cap);
    rc |= tsph_grow(ctx, &T.skip, cap);
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
    if (rc) return TSPH_ERR_NOMEM;
    T.cap = cap;
    // per-node scratch shared by both trees (sized to the larger)
    if (B.maxd2Cap < cap) {
        rc |= tsph_grow(ctx, &B.maxd2, cap);
        rc |= tsph_grow(ctx, &B.leafFlag, cap);
        rc |= tsph_grow(ctx, &B.leafScan, cap);
        if (rc) return TSPH_ERR_NOMEM;
        B.maxd2Cap = cap;
    }
    return TSPH_OK;
}

int tsph_build_tree(tsph_ctx *ctx, TsphDevParts &P, TsphDevTree &T, int n, int nBucket) {
    TsphBuildBufs &B = ctx->B;
    const int BS = 256;
    if (nBucket < 1) return TSPH_ERR_ARG;
    if (n == 0) {
        // an empty bucket (pkdBuildBinary's bEmpty branch, pkd.c:2686-2714)
        int rc = ensure_nodes(ctx, T, 1);
        if (rc) return rc;
        int h6[6] = {0, -1, -1, -1, -1, 0};
        TSPH_CK(cudaMemcpyAsync(T.pLower, &h6[0], sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
        TSPH_CK(cudaMemcpyAsync(T.pUpper, &h6[1], sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
        TSPH_CK(cudaStreamSynchronize(ctx->stream));
        T.nNodes = 1;
        T.nLeaves = 0;
        return TSPH_OK;
    }
    k_init_build<<<tsph_blocks(n, BS), BS, 0, ctx->stream>>>(B.seg, n, B.f_lo[0], B.f_hi[0], B.f_node[0]);
    TSPH_LAUNCH_CK("k_init_build");
    int F = 1, cur = 0, nTemp = 1, level = 0;
    int levelStart[TSPH_MAX_LEVELS + 2];
    levelStart[0] = 0;
    while (F > 0) {
        if (level >= TSPH_MAX_LEVELS) return TSPH_ERR_TREE_DEPTH;
        levelStart[level + 1] = nTemp;   // provisional; fixed below
        k_fbnd_init<<<tsph_blocks(F, BS), BS, 0, ctx->stream>>>(B.f_bnd, F);
        TSPH_LAUNCH_CK("k_fbnd_init");
        k_bounds<<<tsph_blocks(n, BS), BS, 0, ctx->stream>>>(P.x, P.y, P.z, B.seg, B.f_bnd, n);
        TSPH_LAUNCH_CK("k_bounds");
        k_split<<<tsph_blocks(F, BS), BS, 0, ctx->stream>>>(
            F, B.f_lo[cur], B.f_hi[cur], B.f_node[cur], B.f_bnd, nBucket, B.f_split, B.f_dim,
            B.f_fs, B.t_lo, B.t_hi, B.t_dim, B.t_child, B.t_split, B.t_bnd, B.t_level, level);
        TSPH_LAUNCH_CK("k_split");
        k_flag<<<tsph_blocks(n, BS), BS, 0, ctx->stream>>>(P.x, P.y, P.z, B.seg, B.f_split, B.f_dim,
                                                           B.f_fs, B.lt, n);
        TSPH_LAUNCH_CK("k_flag");
        int rc = tsph_scan_inclusive(ctx, B.lt, B.scan, n);
        if (rc) return rc;
        k_swap<<<tsph_blocks(n, BS), BS, 0, ctx->stream>>>(P.x, P.y, P.z, P.m, P.h, P.iord, B.seg,
                                                           B.f_split, B.f_lo[cur], B.f_hi[cur],
                                                           B.lt, B.scan, n);
        TSPH_LAUNCH_CK("k_swap");
        rc = tsph_scan_inclusive(ctx, B.f_split, B.f_rank, F);
        if (rc) return rc;
        k_children<<<tsph_blocks(F, BS), BS, 0, ctx->stream>>>(
            F, B.f_lo[cur], B.f_hi[cur], B.f_node[cur], B.f_split, B.f_rank, B.scan, nTemp, B.f_m,
            B.t_child, B.f_lo[1 - cur], B.f_hi[1 - cur], B.f_node[1 - cur]);
        TSPH_LAUNCH_CK("k_children");
        k_seg<<<tsph_blocks(n, BS), BS, 0, ctx->stream>>>(B.seg, B.f_split, B.f_rank, B.f_m, n);
        TSPH_LAUNCH_CK("k_seg");
        TSPH_CK(cudaMemcpyAsync(B.hostCount, B.f_rank + (F - 1), sizeof(int), cudaMemcpyDeviceToHost,
                                ctx->stream));
        TSPH_CK(cudaStreamSynchronize(ctx->stream));
        int nSplit = B.hostCount[0];
        levelStart[level + 1] = nTemp;
        nTemp += 2 * nSplit;
        F = 2 * nSplit;
        if (nTemp > B.nodeCap - 2 && F > 0) return TSPH_ERR_ARG;   // cannot happen: nodes <= 2n-1
        cur = 1 - cur;
        level++;
    }
    int nLevels = level;
    levelStart[nLevels] = nTemp;
    int rc = ensure_nodes(ctx, T, nTemp);
    if (rc) return rc;
    // subtree sizes bottom-up, depth-first numbering top-down
    for (int l = nLevels - 1; l >= 0; --l) {
        int a = levelStart[l], b = levelStart[l + 1];
        k_size<<<tsph_blocks(b - a, BS), BS, 0, ctx->stream>>>(a, b, B.t_child, B.t_size);
        TSPH_LAUNCH_CK("k_size");
    }
    TSPH_CK(cudaMemsetAsync(B.t_pre, 0, sizeof(int), ctx->stream));
    for (int l = 0; l < nLevels; ++l) {
        int a = levelStart[l], b = levelStart[l + 1];
        k_pre<<<tsph_blocks(b - a, BS), BS, 0, ctx->stream>>>(a, b, B.t_child, B.t_size, B.t_pre);
        TSPH_LAUNCH_CK("k_pre");
    }
    k_scatter_nodes<<<tsph_blocks(nTemp, BS), BS, 0, ctx->stream>>>(
        nTemp, B.t_lo, B.t_hi, B.t_dim, B.t_child, B.t_size, B.t_pre, B.t_split, B.t_bnd, T,
        B.leafFlag);
    TSPH_LAUNCH_CK("k_scatter_nodes");
    rc = tsph_scan_inclusive(ctx, B.leafFlag, B.leafScan, nTemp);
    if (rc) return rc;
    k_leaf_list<<<tsph_blocks(nTemp, BS), BS, 0, ctx->stream>>>(nTemp, B.leafFlag, B.leafScan,
                                                                T.leaves);
    TSPH_LAUNCH_CK("k_leaf_list");
    TSPH_CK(cudaMemcpyAsync(B.hostCount, B.leafScan + (nTemp - 1), sizeof(int),
                            cudaMemcpyDeviceToHost, ctx->stream));
    TSPH_CK(cudaStreamSynchronize(ctx->stream));
    T.nNodes = nTemp;
    T.nLeaves = B.hostCount[0];
    // keep the level table for the moment pass
    memcpy(ctx->B.hostCount + 1, levelStart, sizeof(int) * (nLevels + 1));
    ctx->B.hostCount[TSPH_MAX_LEVELS + 4] = nLevels;
    return TSPH_OK;
}

int tsph_tree_moments(tsph_ctx *ctx, TsphDevParts &P, TsphDevTree &T, int n, double dTheta) {
    TsphBuildBufs &B = ctx->B;
    const int BS = 256;
    if (n == 0) return TSPH_OK;
    int nLevels = B.hostCount[TSPH_MAX_LEVELS + 4];
    const int *levelStart = B.hostCount + 1;
    k_leaf_moments<<<tsph_blocks(T.nLeaves, BS), BS, 0, ctx->stream>>>(T.nLeaves, T.leaves, T, P.x,
                                                                      P.y, P.z, P.m, P.h);
    TSPH_LAUNCH_CK("k_leaf_moments");
    for (int l = nLevels - 1; l >= 0; --l) {
        int a = levelStart[l], b = levelStart[l + 1];
        k_combine<<<tsph_blocks(b - a, BS), BS, 0, ctx->stream>>>(a, b, B.t_child, B.t_pre, T);
        TSPH_LAUNCH_CK("k_combine");
    }
    k_zero_u64<<<tsph_blocks(T.nNodes, BS), BS, 0, ctx->stream>>>(B.maxd2, T.nNodes);
    TSPH_LAUNCH_CK("k_zero_u64");
    k_bmax<<<tsph_blocks(n, BS), BS, 0, ctx->stream>>>(n, T, P.x, P.y, P.z, B.maxd2);
    TSPH_LAUNCH_CK("k_bmax");
    const double twoOverSqrt3 = 2 / sqrt(3.0);
    k_open<<<tsph_blocks(T.nNodes, BS), BS, 0, ctx->stream>>>(T.nNodes, T, B.maxd2, twoOverSqrt3,
                                                              dTheta);
    TSPH_LAUNCH_CK("k_open");
    k_parts32<<<tsph_blocks(n, BS), BS, 0, ctx->stream>>>(n, P.x, P.y, P.z, P.m, P.h, P.ph, P.pl);
    TSPH_LAUNCH_CK("k_parts32");
    return TSPH_OK;
}
