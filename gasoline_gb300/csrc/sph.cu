// K6-K10: SPH smoothing lengths, density/velocity-gradient gather, gas
// pressure, symmetric pressure/viscosity gather, kick and drift.
//
// Reference semantics:
//   smSmooth (smooth.c:1439-1713): fBall2 = the nSmooth-th smallest squared
//     distance, self included, distances dx = x - q.r, d2 = dx*dx+dy*dy+dz*dz
//     (smooth.c:639-642), periodic images chosen per axis (smooth.h:291-390);
//   DenDVDX (smoothfcn.c:3390-3627) with the M4 kernel (smoothfcn.c:200-214);
//   pkdGasPressure (pkd.c:5750-5785), adiabatic, no Jeans floor;
//   SphPressureTermsSym (smoothfcn.c:2276-2385, SphPressureTerms.h) over
//     every pair with d2 <= fBall2 of either particle, summed from both sides.
//
// GB300 mapping: a gas-only kd-tree (the same device builder as gravity) and
// one warp per gas particle.  The kNN is a ball gather around a seed radius
// (the learned-h prediction when present, else the box of the deepest tree
// cell holding >= nSmooth particles) followed by an exact radix select of
// the nSmooth-th squared distance over the candidates' FP64 bit patterns;
// a ball holding fewer than nSmooth grows and retries (the fallback), so
// the neighbour set and fBall2 equal the exact kNN's.  Squared distances
// are FP64 without FMA contraction, exactly as the reference rounds them.
// The pressure pass gathers both roles of every pair (i in N(j) found via
// a per-node max fBall2 bound), so no scatter-adds and no atomics: results
// are deterministic run to run.
#include <float.h>
#include <math.h>

#include "tsph_ctx.cuh"

#define SW 4          // warps per block
#define SSTK 1024     // walk stack per warp
#define SCAP 384      // kNN candidate capacity per warp (more: the ball shrinks)
#define SMAXIT 48     // radius iterations before giving up

struct SphConst {
    int ngas, k;
    int bPeriodic;
    double L;
    double alpha, beta, gamma, gammam1, dtFacCourant;
    int limiter;
    float margin;     // absolute slack for FP32 box-distance pruning
    float erel, eabs; // FP32 relative-coordinate error bound: erel |dx| + eabs
    float Lf, alphaf, betaf, dtFacCourantf;   // FP32 copies for the FP32 kernels
};
__constant__ SphConst cS;

__device__ __forceinline__ unsigned lane_lt_s() {
    unsigned r;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(r));
    return r;
}

// query coordinate shifted to the image of q nearest to it (x, x+L or x-L)
__device__ __forceinline__ double img_q(double x, double q) {
    if (!cS.bPeriodic) return x;
    double d0 = fabs(x - q), dp = fabs((x + cS.L) - q), dm = fabs((x - cS.L) - q);
    if (dp < d0 && dp <= dm) return x + cS.L;
    if (dm < d0 && dm < dp) return x - cS.L;
    return x;
}

// exact squared distance as the reference computes it, with dx = sx - q
__device__ __forceinline__ double dist2_exact(double x, double y, double z, double qx, double qy,
                                              double qz, double &dx, double &dy, double &dz) {
    double sx = img_q(x, qx), sy = img_q(y, qy), sz = img_q(z, qz);
    dx = xsub(sx, qx);
    dy = xsub(sy, qy);
    dz = xsub(sz, qz);
    return xadd(xadd(xmul(dx, dx), xmul(dy, dy)), xmul(dz, dz));
}

// conservative FP32 squared distance from a point to a node box
__device__ __forceinline__ float box_d2f(float x, float y, float z, float4 lo, float4 hi) {
    float p[3] = {x, y, z}, a[3] = {lo.x, lo.y, lo.z}, b[3] = {hi.x, hi.y, hi.z};
    float d2 = 0.0f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float d = fmaxf(fmaxf(a[k] - p[k], p[k] - b[k]), 0.0f);
        if (cS.bPeriodic) {
            float L = cS.Lf;
            float d1 = fmaxf(fmaxf(a[k] - (p[k] + L), (p[k] + L) - b[k]), 0.0f);
            float d2b = fmaxf(fmaxf(a[k] - (p[k] - L), (p[k] - L) - b[k]), 0.0f);
            d = fminf(d, fminf(d1, d2b));
        }
        d = fmaxf(d - cS.margin, 0.0f);
        d2 += d * d;
    }
    return d2;
}

__device__ __forceinline__ double dkern_m4(double ar2) {
    double adk = sqrt(ar2);
    if (ar2 < 1.0) adk = -3 + 2.25 * adk;
    else adk = -0.75 * (2.0 - adk) * (2.0 - adk) / adk;
    return adk;
}

__device__ __forceinline__ double wsum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

struct SphArgs {
    TsphDevTree T;          // gas tree: wcomh = box min, wcoml = box max (float)
    TsphDevParts G;
    TsphSphBufs S;
    TsphDevCounters *cnt;
    int *work;
    const double *seed;     // optional fBall2 seeds (tree order) or null
    TsphDevState C;         // caller-order state (the inactive particles' dtNew, mumax)
    const int *list;        // density pass over these gas-tree indices only (or null: all)
    const int *nList;       // device count of list
    int bucketGather = 0;   // seeded pass over all gas: one candidate gather per gas bucket
};

// The pressure pass acts on active particles (G.act); an inactive one
// takes part only in pairs with an active partner, and from those only its
// dtNew and mumax change (SphPressureTerms.h:97-110: SETDTNEW_PQ and the
// viscous mu update both sides; initSphPressureTermsParticle resets only
// active particles, smoothfcn.c:2204-2221; pairs of two inactive
// particles are skipped, smoothfcn.c:2331).  Final per-particle write:
__device__ __forceinline__ void pressure_store(const SphArgs &A, int i, bool ai, double ax,
                                               double ay, double az, double uPdV, double uAV,
                                               double mu, double dtN) {
    const TsphSphBufs &S = A.S;
    if (ai) {
        S.hax[i] = ax; S.hay[i] = ay; S.haz[i] = az;
        S.uPdV[i] = uPdV; S.uAV[i] = uAV; S.mumax[i] = mu; S.dtNew[i] = dtN;
    } else {
        const int o = A.G.iord[i];
        const double m0 = A.C.mumax[o], d0 = A.C.dtNew[o];
        S.mumax[i] = mu > m0 ? mu : m0;
        S.dtNew[i] = dtN < d0 ? dtN : d0;
    }
}

#define SNBR 192      // neighbours summed in canonical (index) order
#define KSTK 896      // ball-gather walk stack per warp (the size of the sum transpose)
#define KB 16         // finished particles per lane-parallel epilogue
#define BCAP 512      // candidates of one gas bucket's union ball (more: per particle)

struct KnnSmem {
    union {
        int stack[KSTK];          // ball-gather walk stack
        double red[14][32];       // then: transpose of the 14 DenDVDX partial sums
    } u;
    float2 lh[SCAP];              // candidate squared-distance interval [lo, hi]; a
                                  // straddling candidate's exact FP64 d2 overlays it
    int idx[SCAP];                // candidate index (bit 31: exact value in lh)
    int nbr[SNBR];                // N(i), then sorted
};

// Finished particles of a warp awaiting the lane-parallel DenDVDX epilogue.
struct KnnBatch {
    double s[14][KB];
    double fb2[KB];
    unsigned long long hsh[KB];
    int id[KB];
    int nn[KB];
};

// Sort nbr[0, cnt) ascending (bitonic network over the next power of two,
// padded with INT_MAX), one warp.
__device__ void warp_sort_idx(int *nbr, int cnt, int lane) {
    int P = 1;
    while (P < cnt) P <<= 1;
    for (int e = cnt + lane; e < P; e += 32) nbr[e] = 0x7fffffff;
    __syncwarp();
    for (int k = 2; k <= P; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = lane; i < P; i += 32) {
                int l = i ^ j;
                if (l > i) {
                    int a = nbr[i], b = nbr[l];
                    bool up = (i & k) == 0;
                    if ((a > b) == up) { nbr[i] = b; nbr[l] = a; }
                }
            }
            __syncwarp();
        }
    }
}

// M4 kernel W and its derivative from one square root (KERNEL/DKERNEL,
// smoothfcn.c:64-224): identical values to the two separate evaluations.
__device__ __forceinline__ void kern_dkern_m4(double ar2, double &w, double &dw) {
    const double r = sqrt(ar2);
    double ak = 2.0 - r;
    if (ar2 < 1.0) {
        w = 1.0 - 0.75 * ak * ar2;
        dw = -3 + 2.25 * r;
    } else {
        w = 0.25 * ak * ak * ak;
        dw = -0.75 * (2.0 - r) * (2.0 - r) / r;
    }
}

// Squared-distance interval of candidate j around particle i from the FP32
// hi/lo split coordinates: |dx_true - dx32| <= erel |dx32| + eabs per axis.
// A periodic separation close to half the box (where the FP32 and FP64
// image choices could differ) gets the whole range.
// Velocity difference p - q from the FP32 hi/lo parts (no FP64 arithmetic).
__device__ __forceinline__ void split_dv(const TsphSphBufs &S, int p, int q, float &dvx, float &dvy,
                                         float &dvz) {
    const float4 hp = S.vh[p], lp = S.vl[p], hq = S.vh[q], lq = S.vl[q];
    dvx = (hp.x - hq.x) + (lp.x - lq.x);
    dvy = (hp.y - hq.y) + (lp.y - lq.y);
    dvz = (hp.z - hq.z) + (lp.z - lq.z);
}

__device__ __forceinline__ float2 d2_interval(float4 hi_i, float4 lo_i, float4 hj, float4 lj) {
    const float u = 5.9604645e-08f;
    float d[3] = {(hj.x - hi_i.x) + (lj.x - lo_i.x), (hj.y - hi_i.y) + (lj.y - lo_i.y),
                  (hj.z - hi_i.z) + (lj.z - lo_i.z)};
    float lo = 0.0f, hi = 0.0f;
    bool wide = false;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float ad = fabsf(d[a]);
        if (cS.bPeriodic) {
            const float L = cS.Lf;
            if (ad > 0.5f * L) ad = L - ad;
            if (fabsf(ad - 0.5f * L) < 1e-4f * L) wide = true;
        }
        const float e = cS.erel * ad + cS.eabs;
        const float l = fmaxf(ad - e, 0.0f), h = ad + e;
        lo += l * l;
        hi += h * h;
    }
    if (wide) return make_float2(0.0f, FLT_MAX);
    return make_float2(lo * (1.0f - 4.0f * u), hi * (1.0f + 4.0f * u));
}

// Ball gather around particle i: every gas particle whose squared-distance
// interval may reach r2 (lo <= r2) becomes a candidate.  Returns the count
// (-1 when it exceeds SCAP or the stack overflows) and in nSure those
// certainly inside (hi <= r2).
__device__ int ball_gather(KnnSmem &W, const SphArgs &A, int lane, int root, float xf, float yf,
                           float zf, float4 hi_i, float4 lo_i, float r2, int &nSure) {
    const unsigned FULL = 0xffffffffu;
    int sp = 1, nc = 0, ns = 0;
    if (lane == 0) W.u.stack[0] = root;
    __syncwarp();
    const float r2box = r2 * 1.00001f;
    bool bad = false;
    while (sp > 0) {
        int take = sp < 32 ? sp : 32;
        int node = lane < take ? W.u.stack[sp - take + lane] : -1;
        __syncwarp();
        sp -= take;
        bool open = false, leaf = false;
        int4 lk = make_int4(0, 0, -1, 0);
        if (node >= 0) {
            lk = A.T.wlink[node];
            float d2 = box_d2f(xf, yf, zf, A.T.wcomh[node], A.T.wcoml[node]);
            if (d2 <= r2box) {
                if (lk.z >= 0) open = true;
                else leaf = true;
            }
        }
        unsigned bo = __ballot_sync(FULL, open);
        if (sp + 2 * __popc(bo) > KSTK) { bad = true; break; }
        if (open) {
            int pos = sp + 2 * __popc(bo & lane_lt_s());
            W.u.stack[pos] = lk.z;
            W.u.stack[pos + 1] = node + 1;
        }
        sp += 2 * __popc(bo);
        // leaf particles, every lane one (leaf, particle) pair per step over
        // all the leaves this round reached, in a fixed order (leaf-lane
        // major, particle minor): the round's t-th particle belongs to the
        // first lane whose inclusive count exceeds t
        const int cnt = leaf ? lk.y : 0;
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += y;
        }
        const int tot = __shfl_sync(FULL, incl, 31);
        const int base = lk.x - (incl - cnt);   // this lane's t-th particle: base + t
        for (int t0 = 0; t0 < tot; t0 += 32) {
            const int t = t0 + lane;
            int own = 0;
#pragma unroll
            for (int st = 16; st > 0; st >>= 1) {
                const int v = __shfl_sync(FULL, incl, own + st - 1);
                if (v <= t) own += st;
            }
            const int j = __shfl_sync(FULL, base, own & 31) + t;
            float2 iv = make_float2(FLT_MAX, FLT_MAX);
            if (t < tot) iv = d2_interval(hi_i, lo_i, A.G.ph[j], A.G.pl[j]);
            const bool in = iv.x <= r2;
            unsigned bi = __ballot_sync(FULL, in);
            ns += __popc(__ballot_sync(FULL, iv.y <= r2));
            if (nc + __popc(bi) > SCAP) { bad = true; }
            else if (in) {
                int pos = nc + __popc(bi & lane_lt_s());
                W.lh[pos] = iv;
                W.idx[pos] = j;
            }
            nc += __popc(bi);
        }
        __syncwarp();
        if (bad) break;
    }
    __syncwarp();
    nSure = ns;
    return bad ? -1 : nc;
}

// Radix select (4 bits per pass, MSB first) of the need-th smallest key
// among the candidates that `take` accepts; counts kept per lane in 16-bit
// fields of four registers and summed over the warp.
template <int BITS, typename KeyOf>
__device__ unsigned long long radix_select(int nc, int need, int lane, KeyOf keyOf) {
    unsigned long long prefix = 0ULL;
    for (int shift = BITS - 4; shift >= 0; shift -= 4) {
        unsigned long long c[4] = {0ULL, 0ULL, 0ULL, 0ULL};
        const unsigned long long hiMask = (shift + 4 >= 64) ? 0ULL : (~0ULL << (shift + 4));
        for (int e = lane; e < nc; e += 32) {
            unsigned long long key;
            if (!keyOf(e, key)) continue;
            if ((key & hiMask) != prefix) continue;
            unsigned d = (unsigned)(key >> shift) & 15u;
            unsigned long long inc = 1ULL << (16 * (d & 3u));
            c[0] += (d >> 2) == 0 ? inc : 0ULL;
            c[1] += (d >> 2) == 1 ? inc : 0ULL;
            c[2] += (d >> 2) == 2 ? inc : 0ULL;
            c[3] += (d >> 2) == 3 ? inc : 0ULL;
        }
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) c[q] += __shfl_xor_sync(0xffffffffu, c[q], o);
        int d = 0;
        for (; d < 15; ++d) {
            int cd = (int)((c[d >> 2] >> (16 * (d & 3))) & 0xffffULL);
            if (need <= cd) break;
            need -= cd;
        }
        prefix |= (unsigned long long)d << shift;
    }
    return prefix;
}

// The k-th smallest (1-based) of up to 64 keys held two per lane (v0 for
// element lane, v1 for element 32 + lane; pad with the type's maximum) by a
// warp bitonic sort in registers: the same value as the radix select of the
// same keys, in far fewer instructions for the short candidate lists of a
// kNN ball.  T is float (the distance-interval bounds) or unsigned long long
// (the bit patterns of non-negative FP64 squared distances, ordered as the
// doubles are).
template <typename T>
__device__ __forceinline__ T warp_kth64(T v0, T v1, int k, int lane) {
    const unsigned FULL = 0xffffffffu;
    T v[2] = {v0, v1};
#pragma unroll
    for (int kk = 2; kk <= 64; kk <<= 1) {
#pragma unroll
        for (int j = kk >> 1; j > 0; j >>= 1) {
            if (j == 32) {   // partner in the same lane: ascending for kk = 64
                const T lo = v[0] < v[1] ? v[0] : v[1], hi = v[0] < v[1] ? v[1] : v[0];
                v[0] = lo;
                v[1] = hi;
            } else {
#pragma unroll
                for (int s = 0; s < 2; ++s) {
                    const int i = 32 * s + lane;
                    const T p = __shfl_xor_sync(FULL, v[s], j);
                    const bool up = (i & kk) == 0, lower = (i & j) == 0;
                    const T mn = v[s] < p ? v[s] : p, mx = v[s] < p ? p : v[s];
                    v[s] = (lower == up) ? mn : mx;
                }
            }
        }
    }
    const int e = k - 1;
    return __shfl_sync(FULL, e < 32 ? v[0] : v[1], e & 31);
}

// The lane-parallel DenDVDX epilogue (smoothfcn.c:3390-3627) of up to KB
// finished particles: lane l finishes batch entry l.
__device__ void density_epilogue(const SphArgs &A, KnnBatch &Bt, int cnt, int lane) {
    __syncwarp();
    if (lane < cnt) {
        const int i = Bt.id[lane];
        const double fBall2 = Bt.fb2[lane];
        double sm[14];
#pragma unroll
        for (int q = 0; q < 14; ++q) sm[q] = Bt.s[q][lane];
        const double H = 0.0;
        double ih2 = 4.0 / fBall2, ih = sqrt(ih2);
        double fNorm = M_1_PI * ih2 * ih;
        double fDensity = sm[0] * fNorm;
        double dvxdx = sm[1], dvxdy = sm[2], dvxdz = sm[3], dvydx = sm[4], dvydy = sm[5],
               dvydz = sm[6], dvzdx = sm[7], dvzdy = sm[8], dvzdz = sm[9];
        double divvnorm = sm[10], grx = sm[11], gry = sm[12], grz = sm[13];
        double trace = dvxdx + dvydy + dvzdz;
        double fNorm1 = (divvnorm != 0 ? 3 / fabs(divvnorm) : 0);
        double divv = fNorm1 * trace + 3 * H;
        double cx = fNorm1 * (dvzdy - dvydz), cy = fNorm1 * (dvxdz - dvzdx),
               cz = fNorm1 * (dvydx - dvxdy);
        double Hcorr = (fNorm1 != 0 ? H / fNorm1 : 0);
        double gnorm = grx * grx + gry * gry + grz * grz;
        if (gnorm > 0) gnorm = 1 / sqrt(gnorm);
        grx *= gnorm; gry *= gnorm; grz *= gnorm;
        double dvdr = (((dvxdx + Hcorr) * grx + dvxdy * gry + dvxdz * grz) * grx +
                       (dvydx * grx + (dvydy + Hcorr) * gry + dvydz * grz) * gry +
                       (dvzdx * grx + dvzdy * gry + (dvzdz + Hcorr) * grz) * grz) * fNorm1;
        double dvds = (divv < 0 ? 1.5 * (dvdr - (1. / 3.) * divv) : dvdr);
        double bal;
        if (cS.limiter == 1) {
            bal = divv != 0.0 ? fabs(divv) / (fabs(divv) + sqrt(cx * cx + cy * cy + cz * cz)) : 0.0;
        } else {
            bal = 1.0;
        }
        double ot = (1. / 3.) * trace;
        double sxx = dvxdx - ot, syy = dvydy - ot, szz = dvzdz - ot;
        double sxy = 0.5 * (dvxdy + dvydx), sxz = 0.5 * (dvxdz + dvzdx), syz = 0.5 * (dvydz + dvzdy);
        double S2 = fNorm1 * fNorm1 * (sxx * sxx + syy * syy + szz * szz +
                                       2 * (sxy * sxy + sxz * sxz + syz * syz));
        A.S.fBall2[i] = fBall2;
        A.S.rho[i] = fDensity;
        A.S.divv[i] = divv;
        A.S.curl[3 * i] = cx;
        A.S.curl[3 * i + 1] = cy;
        A.S.curl[3 * i + 2] = cz;
        A.S.dvds[i] = dvds;
        A.S.bal[i] = bal;
        A.S.diff[i] = 0.25 * fBall2 * sqrt(2 * S2);
        A.S.nnCount[i] = Bt.nn[lane];
        A.S.nnHash[i] = Bt.hsh[lane];
    }
    __syncwarp();
}

// kNN + DenDVDX, one warp per gas particle.  The set N(i) and fBall2 are the
// exact FP64 ones: candidates carry FP32 distance intervals, the k-th
// distance is bracketed from them, and only candidates whose interval
// straddles the bracket get their FP64 distance.  The neighbour sums run
// over N(i) in ascending index (FP64), so they depend on the set only.
// Squared distance from a box to a box in FP32, each axis the nearest
// periodic image, less the coordinate rounding margin of both boxes: never
// more than the true distance.
__device__ __forceinline__ float box_box_d2f(float4 alo, float4 ahi, float4 blo, float4 bhi) {
    const float a0[3] = {alo.x, alo.y, alo.z}, a1[3] = {ahi.x, ahi.y, ahi.z};
    const float b0[3] = {blo.x, blo.y, blo.z}, b1[3] = {bhi.x, bhi.y, bhi.z};
    float d2 = 0.0f;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        float d = fmaxf(fmaxf(a0[q] - b1[q], b0[q] - a1[q]), 0.0f);
        if (cS.bPeriodic) {
            const float L = cS.Lf;
            const float dp = fmaxf(fmaxf(a0[q] - (b1[q] + L), (b0[q] + L) - a1[q]), 0.0f);
            const float dm = fmaxf(fmaxf(a0[q] - (b1[q] - L), (b0[q] - L) - a1[q]), 0.0f);
            d = fminf(d, fminf(dp, dm));
        }
        d = fmaxf(d - 2.0f * cS.margin, 0.0f);
        d2 += d * d;
    }
    return d2;
}

// Every gas particle whose distance from the bucket box [blo, bhi] may be
// within sqrt(R2) (the box test of ball_gather, made against a box): a
// superset of the candidates ball_gather finds for any particle of the
// bucket at any radius^2 up to R2.  Stored in bc in walk order; returns
// their number, or -1 when they exceed BCAP or the stack overflows.
__device__ int bucket_gather(KnnSmem &W, int *bc, const SphArgs &A, int lane, int root, float4 blo,
                             float4 bhi, float R2) {
    const unsigned FULL = 0xffffffffu;
    int sp = 1, nc = 0;
    if (lane == 0) W.u.stack[0] = root;
    __syncwarp();
    bool bad = false;
    while (sp > 0) {
        const int take = sp < 32 ? sp : 32;
        const int node = lane < take ? W.u.stack[sp - take + lane] : -1;
        __syncwarp();
        sp -= take;
        bool open = false, leaf = false;
        int4 lk = make_int4(0, 0, -1, 0);
        if (node >= 0) {
            lk = A.T.wlink[node];
            if (box_box_d2f(A.T.wcomh[node], A.T.wcoml[node], blo, bhi) <= R2) {
                if (lk.z >= 0) open = true;
                else leaf = true;
            }
        }
        const unsigned bo = __ballot_sync(FULL, open);
        if (sp + 2 * __popc(bo) > KSTK) { bad = true; break; }
        if (open) {
            const int pos = sp + 2 * __popc(bo & lane_lt_s());
            W.u.stack[pos] = lk.z;
            W.u.stack[pos + 1] = node + 1;
        }
        sp += 2 * __popc(bo);
        // the particles of this round's leaves, a lane per particle (leaf-lane
        // major, particle minor, as ball_gather takes them)
        const int cnt = leaf ? lk.y : 0;
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += y;
        }
        const int tot = __shfl_sync(FULL, incl, 31);
        const int base = lk.x - (incl - cnt);
        for (int t0 = 0; t0 < tot; t0 += 32) {
            const int t = t0 + lane;
            int own = 0;
#pragma unroll
            for (int st = 16; st > 0; st >>= 1) {
                const int v = __shfl_sync(FULL, incl, own + st - 1);
                if (v <= t) own += st;
            }
            const int j = __shfl_sync(FULL, base, own & 31) + t;
            bool in = false;
            if (t < tot) {
                const float4 hj = A.G.ph[j];
                in = box_d2f(hj.x, hj.y, hj.z, blo, bhi) <= R2;
            }
            const unsigned bi = __ballot_sync(FULL, in);
            if (nc + __popc(bi) > BCAP) { bad = true; break; }
            if (in) bc[nc + __popc(bi & lane_lt_s())] = j;
            nc += __popc(bi);
        }
        __syncwarp();
        if (bad) break;
    }
    __syncwarp();
    return bad ? -1 : nc;
}

// ball_gather's result for particle i at radius^2 r2, taken from a bucket's
// gathered list bc[0, nbc) (which holds every candidate at any r2 up to
// the gather's radius): the same candidates in the list's order, their
// intervals in W.lh, and the number surely inside in nSure; -1 when they
// exceed SCAP.
__device__ int bucket_filter(KnnSmem &W, const int *bc, int nbc, int lane, const SphArgs &A,
                             float4 hi_i, float4 lo_i, float r2, int &nSure) {
    const unsigned FULL = 0xffffffffu;
    int nc = 0, ns = 0;
    for (int e0 = 0; e0 < nbc; e0 += 32) {
        const int e = e0 + lane;
        float2 iv = make_float2(FLT_MAX, FLT_MAX);
        int j = 0;
        if (e < nbc) {
            j = bc[e];
            iv = d2_interval(hi_i, lo_i, A.G.ph[j], A.G.pl[j]);
        }
        const bool in = iv.x <= r2;
        const unsigned bi = __ballot_sync(FULL, in);
        ns += __popc(__ballot_sync(FULL, iv.y <= r2));
        if (nc + __popc(bi) > SCAP) {
            __syncwarp();
            return -1;
        }
        if (in) {
            const int pos = nc + __popc(bi & lane_lt_s());
            W.lh[pos] = iv;
            W.idx[pos] = j;
        }
        nc += __popc(bi);
    }
    __syncwarp();
    nSure = ns;
    return nc;
}

// Particle i's starting kNN radius^2: the learned seed when there is one,
// else from the smallest tree node around i that holds k particles (any
// positive value works: a short ball grows, a large one shrinks; the seed
// only sets the cost).
__device__ __forceinline__ float seed_r2(const SphArgs &A, int i, int k) {
    const float4 hi_i = A.G.ph[i];
    const float xf = hi_i.x, yf = hi_i.y, zf = hi_i.z;
    const int root = A.T.sysRoot[A.G.rid[i]];
    float r2;
    if (A.seed && A.seed[i] > 0.0) {
        r2 = (float)A.seed[i];
    } else {
        int node = root;
        for (;;) {
            int up = A.T.upper[node];
            if (up < 0) break;
            int child = (i >= A.T.pLower[up]) ? up : node + 1;
            if (A.T.pUpper[child] - A.T.pLower[child] + 1 < k) break;
            node = child;
        }
        // farthest box corner (surely k particles), or the radius holding
        // twice the volume k particles need at the node's mean density
        const float4 bl = A.T.wcomh[node], bh = A.T.wcoml[node];
        const float p[3] = {xf, yf, zf}, a[3] = {bl.x, bl.y, bl.z}, c[3] = {bh.x, bh.y, bh.z};
        float rc = 0.0f, vol = 1.0f;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            float d = fmaxf(fabsf(p[q] - a[q]), fabsf(p[q] - c[q]));
            rc += d * d;
            vol *= c[q] - a[q];
        }
        r2 = rc * 1.0001f + 1e-30f;
        const int nNode = A.T.pUpper[node] - A.T.pLower[node] + 1;
        if (vol > 0.0f) {
            float rd = cbrtf(2.0f * 3.0f * k * vol / (4.0f * 3.14159265f * nNode));
            if (rd * rd < r2) r2 = rd * rd;
        }
    }
    return r2;
}

template <bool F32>
__global__ void __launch_bounds__(SW * 32, 5) k_knn_density(SphArgs A) {
    extern __shared__ __align__(16) unsigned char smraw[];
    KnnSmem &W = reinterpret_cast<KnnSmem *>(smraw)[threadIdx.x >> 5];
    KnnBatch &Bt = reinterpret_cast<KnnBatch *>(smraw + sizeof(KnnSmem) * SW)[threadIdx.x >> 5];
    // a bucket launch's candidate lists follow the batches (the other
    // launches do not allocate them: their occupancy stays a block higher)
    int *bcw = reinterpret_cast<int *>(smraw + (sizeof(KnnSmem) + sizeof(KnnBatch)) * SW) +
               (threadIdx.x >> 5) * BCAP;
    const int lane = threadIdx.x & 31;
    const unsigned FULL = 0xffffffffu;
    const int ng = cS.ngas, k = cS.k;
    unsigned long long nFall = 0, nPairs = 0, nCand = 0;
    int nb = 0;                              // particles waiting in the batch
    // Particle i's kNN and DenDVDX sums, its search starting at radius^2 r2.
    // With bc non-null the candidates of any ball of radius^2 <= bcR2
    // around i come from the bucket's gathered list bc[0, nbc).
    auto one = [&](int i, float r2, const int *bc, int nbc, float bcR2) {
        const double xi = A.G.x[i], yi = A.G.y[i], zi = A.G.z[i];
        const float4 hi_i = A.G.ph[i], lo_i = A.G.pl[i];
        const float xf = hi_i.x, yf = hi_i.y, zf = hi_i.z;
        const int root = A.T.sysRoot[A.G.rid[i]];   // this particle's system
        float lo2 = 0.0f, hi2 = 0.0f;   // radii known too small / too large
        int nc = -1, nSure = 0, it = 0;
        for (; it < SMAXIT; ++it) {
            nc = (bc && r2 <= bcR2) ? bucket_filter(W, bc, nbc, lane, A, hi_i, lo_i, r2, nSure)
                                    : ball_gather(W, A, lane, root, xf, yf, zf, hi_i, lo_i, r2, nSure);
            if (nc < 0) {                       // too many candidates: shrink
                hi2 = r2;
                r2 = lo2 > 0.0f ? sqrtf(lo2 * hi2) : 0.5f * r2;
            } else if (nSure < k) {             // k not surely inside: grow
                lo2 = r2;
                r2 = hi2 > 0.0f ? sqrtf(lo2 * hi2) : 2.25f * r2;
                ++nFall;
            } else {
                break;
            }
            if (hi2 > 0.0f && lo2 > 0.0f && hi2 <= lo2 * 1.0001f) { it = SMAXIT; break; }
        }
        if (it == SMAXIT) {
            if (lane == 0) atomicOr(&A.cnt->status, 1u << TSPH_ERR_KNN_NO_CONVERGE);
            return;
        }
        nCand += nc;
        // bracket the k-th distance: Tlo <= fBall2 <= Thi (a register sort
        // for the usual short lists, a radix select for long ones)
        float Tlo, Thi;
        if (nc <= 64) {
            const float2 a = lane < nc ? W.lh[lane] : make_float2(FLT_MAX, FLT_MAX);
            const float2 b = lane + 32 < nc ? W.lh[lane + 32] : make_float2(FLT_MAX, FLT_MAX);
            Tlo = warp_kth64<float>(a.x, b.x, k, lane);
            Thi = warp_kth64<float>(a.y, b.y, k, lane);
        } else {
            Tlo = __uint_as_float((unsigned)radix_select<32>(nc, k, lane,
                [&](int e, unsigned long long &key) { key = __float_as_uint(W.lh[e].x); return true; }));
            Thi = __uint_as_float((unsigned)radix_select<32>(nc, k, lane,
                [&](int e, unsigned long long &key) { key = __float_as_uint(W.lh[e].y); return true; }));
        }
        // certainly inside (hi < Tlo), straddling (exact FP64 now), outside
        int nIn = 0;
        for (int e = lane; e < nc; e += 32) {
            const float2 iv = W.lh[e];
            if (iv.y < Tlo) {
                ++nIn;
            } else if (iv.x <= Thi) {
                const int j = W.idx[e];
                double dx, dy, dz;
                double d2 = dist2_exact(xi, yi, zi, A.G.x[j], A.G.y[j], A.G.z[j], dx, dy, dz);
                *reinterpret_cast<double *>(&W.lh[e]) = d2;
                W.idx[e] = j | (int)0x80000000;
            }
        }
        nIn = __reduce_add_sync(FULL, (unsigned)nIn);
        __syncwarp();
        // the (k - nIn)-th exact distance among the straddling candidates:
        // gathered into registers (at most 64) and sorted, else radix select
        int nStr = 0;
        for (int e = lane; e < nc; e += 32) nStr += W.idx[e] < 0;
        nStr = __reduce_add_sync(FULL, (unsigned)nStr);
        double fBall2;
        if (nStr <= 64) {
            // compacted into the neighbour buffer, free until N(i) is chosen
            // (192 ints hold 96 keys; 8-byte aligned within the warp's area)
            unsigned long long *sk = reinterpret_cast<unsigned long long *>(W.nbr);
            int got = 0;
            for (int e0 = 0; e0 < nc; e0 += 32) {
                const int e = e0 + lane;
                const bool str = e < nc && W.idx[e] < 0;
                const unsigned bs = __ballot_sync(FULL, str);
                if (str)
                    sk[got + __popc(bs & lane_lt_s())] =
                        (unsigned long long)__double_as_longlong(*reinterpret_cast<const double *>(&W.lh[e]));
                got += __popc(bs);
            }
            __syncwarp();
            unsigned long long s2[2];
            s2[0] = lane < nStr ? sk[lane] : ~0ULL;
            s2[1] = lane + 32 < nStr ? sk[lane + 32] : ~0ULL;
            __syncwarp();
            fBall2 = __longlong_as_double((long long)warp_kth64<unsigned long long>(s2[0], s2[1],
                                                                                     k - nIn, lane));
        } else {
            fBall2 = __longlong_as_double((long long)radix_select<64>(
                nc, k - nIn, lane, [&](int e, unsigned long long &key) {
                    if (W.idx[e] >= 0) return false;
                    key = (unsigned long long)__double_as_longlong(*reinterpret_cast<const double *>(&W.lh[e]));
                    return true;
                }));
        }
        // N(i) in ascending particle order, so the sums below depend only on
        // the neighbour set, not on the order the ball gather found them
        int nsel = 0;
        for (int e0 = 0; e0 < nc; e0 += 32) {
            int e = e0 + lane;
            bool in = false;
            int j = 0;
            if (e < nc) {
                const int t = W.idx[e];
                if (t < 0) {
                    j = t & 0x7fffffff;
                    in = *reinterpret_cast<const double *>(&W.lh[e]) <= fBall2;
                } else {
                    j = t;
                    in = W.lh[e].y < Tlo;
                }
            }
            unsigned bi = __ballot_sync(FULL, in);
            if (in && nsel + __popc(bi & lane_lt_s()) < SNBR) W.nbr[nsel + __popc(bi & lane_lt_s())] = j;
            nsel += __popc(bi);
        }
        __syncwarp();
        if (nsel > SNBR) {                   // more than SNBR exact ties
            if (lane == 0) atomicOr(&A.cnt->status, 1u << TSPH_ERR_LIST_OVERFLOW);
            return;
        }
        warp_sort_idx(W.nbr, nsel, lane);
        if (nsel <= A.S.nbrCap) {
            int *dst = A.S.nbrList + (size_t)i * A.S.nbrCap;
            for (int e = lane; e < nsel; e += 32) dst[e] = W.nbr[e];
        } else if (lane == 0) {
            A.S.listFlag[0] = 1;
        }
        // DenDVDX neighbour sums (smoothfcn.c:3390-3627) over N(i)
        const double vxi = A.S.vx[i], vyi = A.S.vy[i], vzi = A.S.vz[i];
        const double ih2 = 4.0 / fBall2;
        unsigned long long hsh = 0ULL;
        for (int e = lane; e < nsel; e += 32) {
            unsigned long long hx = (unsigned long long)(A.G.iord[W.nbr[e]] + 1);
            hx *= 0x9E3779B97F4A7C15ULL;
            hx ^= hx >> 29;
            hx *= 0xBF58476D1CE4E5B9ULL;
            hx ^= hx >> 32;
            hsh += hx;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) hsh += __shfl_xor_sync(FULL, hsh, o);
        if constexpr (!F32) {
            double sm[14];
#pragma unroll
            for (int q = 0; q < 14; ++q) sm[q] = 0.0;
            for (int e = lane; e < nsel; e += 32) {
                const int j = W.nbr[e];
                double dx, dy, dz;
                const double d2 = dist2_exact(xi, yi, zi, A.G.x[j], A.G.y[j], A.G.z[j], dx, dy, dz);
                double rs, rs1;
                kern_dkern_m4(d2 * ih2, rs, rs1);
                const double mj = A.G.m[j];
                sm[0] += rs * mj;
                rs1 *= mj;
                double dvx = (-vxi + A.S.vx[j]), dvy = (-vyi + A.S.vy[j]), dvz = (-vzi + A.S.vz[j]);
                sm[1] += dvx * dx * rs1; sm[2] += dvx * dy * rs1; sm[3] += dvx * dz * rs1;
                sm[4] += dvy * dx * rs1; sm[5] += dvy * dy * rs1; sm[6] += dvy * dz * rs1;
                sm[7] += dvz * dx * rs1; sm[8] += dvz * dy * rs1; sm[9] += dvz * dz * rs1;
                sm[10] += (dx * dx + dy * dy + dz * dz) * rs1;
                const double uj = A.S.u[j];
                sm[11] += uj * dx * rs1;
                sm[12] += uj * dy * rs1;
                sm[13] += uj * dz * rs1;
            }
            // fixed-order sums: the 14 x 32 partials transposed through
            // shared memory, lane q adds quantity q's 32 partials in order
#pragma unroll
            for (int q = 0; q < 14; ++q) W.u.red[q][lane] = sm[q];
            __syncwarp();
            if (lane < 14) {
                double t = 0.0;
                for (int l = 0; l < 32; ++l) t += W.u.red[lane][l];
                Bt.s[lane][nb] = t;
            }
        } else {
            // FP32 neighbour terms on split relative coordinates and split
            // velocities (the hi/lo differences keep a bulk flow from
            // swamping them); a fixed-order FP32 warp sum, widened for the
            // FP64 epilogue
            const float ih2f = (float)ih2;
            float sm[14];
#pragma unroll
            for (int q = 0; q < 14; ++q) sm[q] = 0.0f;
            for (int e = lane; e < nsel; e += 32) {
                const int j = W.nbr[e];
                const float4 hj = A.G.ph[j], lj = A.G.pl[j];
                float dx = (hi_i.x - hj.x) + (lo_i.x - lj.x);
                float dy = (hi_i.y - hj.y) + (lo_i.y - lj.y);
                float dz = (hi_i.z - hj.z) + (lo_i.z - lj.z);
                if (cS.bPeriodic) {
                    const float L = cS.Lf, h = 0.5f * L;
                    dx = dx > h ? dx - L : (dx < -h ? dx + L : dx);
                    dy = dy > h ? dy - L : (dy < -h ? dy + L : dy);
                    dz = dz > h ? dz - L : (dz < -h ? dz + L : dz);
                }
                const float d2 = dx * dx + dy * dy + dz * dz;
                const float ar2 = d2 * ih2f, r = sqrtf(ar2);
                float rs, rs1;
                if (ar2 < 1.0f) {
                    rs = 1.0f - 0.75f * (2.0f - r) * ar2;
                    rs1 = -3.0f + 2.25f * r;
                } else {
                    const float t = 2.0f - r;
                    rs = 0.25f * t * t * t;
                    rs1 = -0.75f * t * t / r;
                }
                const float mj = hj.w;
                sm[0] += rs * mj;
                rs1 *= mj;
                float dvx, dvy, dvz;
                split_dv(A.S, j, i, dvx, dvy, dvz);
                sm[1] += dvx * dx * rs1; sm[2] += dvx * dy * rs1; sm[3] += dvx * dz * rs1;
                sm[4] += dvy * dx * rs1; sm[5] += dvy * dy * rs1; sm[6] += dvy * dz * rs1;
                sm[7] += dvz * dx * rs1; sm[8] += dvz * dy * rs1; sm[9] += dvz * dz * rs1;
                sm[10] += d2 * rs1;
                const float uj = lj.w;
                sm[11] += uj * dx * rs1;
                sm[12] += uj * dy * rs1;
                sm[13] += uj * dz * rs1;
            }
#pragma unroll
            for (int q = 0; q < 14; ++q) {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) sm[q] += __shfl_xor_sync(FULL, sm[q], o);
            }
            if (lane == 0) {
#pragma unroll
                for (int q = 0; q < 14; ++q) Bt.s[q][nb] = (double)sm[q];
            }
        }
        if (lane == 0) {
            Bt.fb2[nb] = fBall2;
            Bt.hsh[nb] = hsh;
            Bt.id[nb] = i;
            Bt.nn[nb] = nsel;
        }
        nPairs += nsel;
        ++nb;
        if (nb == KB) {
            density_epilogue(A, Bt, nb, lane);
            nb = 0;
        }
    };
    // the work: particles from the list, or (a pass over all gas) gas
    // buckets, each gathered once when that pays, or single particles; one
    // call site for the per-particle work keeps the kernel's code compact
    int curLo = 0, curN = 0, curT = 0, nbc = -1;
    float r2l = 0.0f, R2 = 0.0f;
    for (;;) {
        if (curT >= curN) {
            int u = 0;
            if (lane == 0) u = atomicAdd(A.work, 1);
            u = __shfl_sync(FULL, u, 0);
            curT = 0;
            nbc = -1;
            if (A.list) {
                if (u >= *A.nList) break;
                curLo = A.list[u];
                curN = 1;
                r2l = seed_r2(A, curLo, k);
            } else if (A.bucketGather) {
                // a gas bucket: one tree walk gathers every candidate of its
                // particles' balls (the largest seed around the bucket's
                // box), then each particle takes its own from that list
                if (u >= A.T.dcnt[1]) break;
                const int node = A.T.leaves[u];
                curLo = A.T.pLower[node];
                curN = A.T.pUpper[node] - curLo + 1;
                r2l = lane < curN ? seed_r2(A, curLo + lane, k) : 0.0f;
                R2 = r2l;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) R2 = fmaxf(R2, __shfl_xor_sync(FULL, R2, o));
                nbc = bucket_gather(W, bcw, A, lane, A.T.sysRoot[A.G.rid[curLo]], A.T.wcomh[node],
                                    A.T.wcoml[node], R2 * 1.001f);
            } else {
                if (u >= ng) break;
                curLo = u;
                curN = 1;
                r2l = seed_r2(A, u, k);
            }
        }
        const int t = curT++;
        const float r2t = A.bucketGather && !A.list ? __shfl_sync(FULL, r2l, t) : r2l;
        one(curLo + t, r2t, nbc >= 0 ? bcw : nullptr, nbc, R2);
        __syncwarp();
    }
    if (nb > 0) density_epilogue(A, Bt, nb, lane);
    if (lane == 0) {
        if (nFall) atomicAdd(&A.cnt->nExactTests, nFall);
        if (nPairs) atomicAdd(&A.cnt->nPartPP, nPairs);
        if (nCand) atomicAdd(&A.cnt->nCellNewt, nCand);
    }
}

// FP32 hi/lo split of the gas positions (tree order) for the kNN intervals.
__global__ void k_gas_split(int ng, TsphDevParts G, const double *__restrict__ u) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ng) return;
    float hx, lx, hy, ly, hz, lz;
    split2f(G.x[i], hx, lx);
    split2f(G.y[i], hy, ly);
    split2f(G.z[i], hz, lz);
    G.ph[i] = make_float4(hx, hy, hz, (float)G.m[i]);
    G.pl[i] = make_float4(lx, ly, lz, (float)u[i]);
}

// pkdGasPressure (pkd.c:5750-5785) for the adiabatic gas model.  Every gas
// particle's timestep p->dt (caller order, kept across passes) drops to
// its Courant time "to scare the neighbours" (pkd.c:5779-5781).
__global__ void k_gas_pressure(int ng, TsphSphBufs S, const int *__restrict__ iord, TsphDevState C) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ng) return;
    const int o = iord[i];
    if (!S.need[i]) {
        // not computed this pass: its sound speed and timestep from its
        // current uPred and its last ball (what the reference's FastGas
        // branch leaves a particle outside the active neighbourhood with)
        const double cGas = sqrt(cS.gamma * (cS.gammam1 * S.u[i]));
        const double c = sqrt(cGas * cGas + (5. / 3.) * 0.0 + 2.0 * 0.0);
        const double fb = C.fb2prev[o], uTotDot = C.udot[o];
        double dtp = C.dt[o], dt;
        if (uTotDot > 0)
            dt = cS.dtFacCourant * sqrt(fb * 0.25 / (4 * (c * c + (5. / 3.) * uTotDot * dtp)));
        else
            dt = cS.dtFacCourant * sqrt(fb * 0.25) / (2 * c);
        if (dt < dtp) C.dt[o] = dt;
        C.cs[o] = c;
        return;
    }
    double PoverRhoGas = cS.gammam1 * S.u[i];
    double cGas = sqrt(cS.gamma * PoverRhoGas);
    double PoverRho = PoverRhoGas + 0.0;
    S.pr2[i] = PoverRho / S.rho[i];
    double c = sqrt(cGas * cGas + (5. / 3.) * 0.0 + 2.0 * 0.0);
    S.cs[i] = c;
    double dtp = C.dt[o];
    const double uTotDot = C.udot[o];
    double dt;
    if (uTotDot > 0)
        dt = cS.dtFacCourant * sqrt(S.fBall2[i] * 0.25 / (4 * (c * c + (5. / 3.) * uTotDot * dtp)));
    else
        dt = cS.dtFacCourant * sqrt(S.fBall2[i] * 0.25) / (2 * c);
    if (dt < dtp) dtp = dt;
    S.dtp[i] = dtp;
    C.dt[o] = dtp;
    C.cs[o] = c;
    // the pair terms' per-particle factors (SphPressureTerms.h:1-40)
    double fb = S.fBall2[i], rho = S.rho[i], d2 = rho * rho;
    double ph = sqrt(0.25 * fb);
    double ih2 = 4.0 / fb;
    double fNorm = 0.5 * M_1_PI * ih2 / ph;
    S.ph[i] = ph;
    S.ih2[i] = ih2;
    S.fn1[i] = fNorm * ih2;
    S.pr2f[i] = (S.pr2[i] * d2 + 0) / d2;
    // FP32 copies for the FP32 pressure pass
    S.pfa[i] = make_float4((float)ph, (float)ih2, (float)(fNorm * ih2), (float)S.pr2f[i]);
    S.pfb[i] = make_float4((float)c, (float)rho, (float)S.bal[i], (float)dtp);
    S.pfc[i] = make_float4((float)S.pr2[i], 0.0f, 0.0f, 0.0f);
}

// Reverse neighbour lists: count, fill, sort (ascending index).
__global__ void k_rev_count(int ng, TsphSphBufs S) {
    if (S.listFlag[0]) return;           // incomplete lists: not used
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int i = (int)(t / S.nbrCap), e = (int)(t % S.nbrCap);
    if (i >= ng || !S.need[i] || e >= S.nnCount[i]) return;
    atomicAdd(&S.rcnt[S.nbrList[(size_t)i * S.nbrCap + e]], 1);
}

__global__ void k_rev_fill(int ng, TsphSphBufs S) {
    if (S.listFlag[0]) return;
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int i = (int)(t / S.nbrCap), e = (int)(t % S.nbrCap);
    if (i >= ng || !S.need[i] || e >= S.nnCount[i]) return;
    int j = S.nbrList[(size_t)i * S.nbrCap + e];
    int slot = atomicAdd(&S.rcur[j], 1);
    S.rlist[(j > 0 ? S.roff[j - 1] : 0) + slot] = i;
}

__global__ void __launch_bounds__(SW * 32) k_rev_sort(int ng, TsphSphBufs S, int *work) {
    __shared__ int buf[SW][TSPH_RCAP];
    const int lane = threadIdx.x & 31;
    int *b = buf[threadIdx.x >> 5];
    if (S.listFlag[0]) return;
    for (;;) {
        int j = 0;
        if (lane == 0) j = atomicAdd(work, 1);
        j = __shfl_sync(0xffffffffu, j, 0);
        if (j >= ng) break;
        const int o = j > 0 ? S.roff[j - 1] : 0, len = S.roff[j] - o;
        if (len > TSPH_RCAP) {
            if (lane == 0) S.listFlag[0] = 1;
            continue;
        }
        for (int e = lane; e < len; e += 32) b[e] = S.rlist[o + e];
        __syncwarp();
        warp_sort_idx(b, len, lane);
        for (int e = lane; e < len; e += 32) S.rlist[o + e] = b[e];
        __syncwarp();
    }
}

// per gas-tree node: max fBall2 of its particles (atomicMax on the bits)
__global__ void k_node_ball(int ng, TsphDevTree T, const int *__restrict__ rid,
                            const double *__restrict__ fBall2, const int *listFlag,
                            unsigned long long *nodeBall2, const int *__restrict__ need, int always) {
    if (!always && !*listFlag) return;   // only the tree-walk fallback needs node balls
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    bool live = p < ng;
    unsigned long long key =
        (live && (!need || need[p])) ? (unsigned long long)__double_as_longlong(fBall2[p]) : 0ULL;
    int i = live ? T.sysRoot[rid[p]] : 0;
    unsigned mask = __ballot_sync(0xffffffffu, live);
    while (mask) {
        if (live) {
            unsigned grp = __match_any_sync(mask, i);
            unsigned hiw = (unsigned)(key >> 32), low = (unsigned)key;
            unsigned mh = __reduce_max_sync(grp, hiw);
            unsigned ml = __reduce_max_sync(grp, hiw == mh ? low : 0u);
            if ((int)(threadIdx.x & 31) == __ffs(grp) - 1)
                atomicMax(&nodeBall2[i], ((unsigned long long)mh << 32) | ml);
            int up = T.upper[i];
            if (up < 0) live = false;
            else i = (p >= T.pLower[up]) ? up : i + 1;
        }
        mask = __ballot_sync(0xffffffffu, live);
    }
}

// One pair of SphPressureTermsSym (smoothfcn.c:2276-2385 with
// SphPressureTerms.h:1-152) as it acts on particle i: own = true when the
// ball is i's (p = i, q = j), false when it is j's (p = j, q = i).  dx is
// r_p - r_q (nearest image), fDist2 = |dx|^2.
__device__ __forceinline__ void sph_pair(const TsphSphBufs &S, const double *__restrict__ m, int p,
                                         int q, double dx, double dy, double dz, double fDist2,
                                         bool own, double &ax, double &ay, double &az,
                                         double &uPdV, double &uAV, double &mu, double &dtN) {
    const double aFac = 1.0, vFac = 1.0, H = 0.0;
    const double pc = S.cs[p], qc = S.cs[q];
    const double ph = S.ph[p];
    const double r2 = fDist2 * S.ih2[p];
    const double rs1 = dkern_m4(r2) * S.fn1[p];
    const double rp = rs1 * m[p], rq = rs1 * m[q];
    const double dvx = S.vx[p] - S.vx[q], dvy = S.vy[p] - S.vy[q], dvz = S.vz[p] - S.vz[q];
    const double dvdotdr = vFac * (dvx * dx + dvy * dy + dvz * dz) + fDist2 * H;
    double Acc, dt;
    if (own) {
        uPdV += rq * S.pr2[p] * dvdotdr;
        Acc = S.pr2f[p] + S.pr2f[q];
    } else {
        uPdV += rp * S.pr2[q] * dvdotdr;
        Acc = S.pr2f[q] + S.pr2f[p];
    }
    if (dvdotdr >= 0.0) {
        dt = cS.dtFacCourant * ph / (2 * (pc > qc ? pc : qc));
    } else {
        double absmu = -dvdotdr * aFac / sqrt(fDist2);
        if (absmu > mu) mu = absmu;
        double visc = (cS.alpha * (pc + qc) + cS.beta * 1.5 * absmu);
        dt = cS.dtFacCourant * ph / (0.625 * (pc + qc) + 0.375 * visc);
        visc = (0.5 * (S.bal[p] + S.bal[q])) * visc * absmu / (S.rho[p] + S.rho[q]);
        if (own) uAV += rq * (0.5 * visc) * dvdotdr;
        else uAV += rp * (0.5 * visc) * dvdotdr;
        Acc += visc;
    }
    if (own) {
        Acc *= rq * aFac;
        ax -= Acc * dx; ay -= Acc * dy; az -= Acc * dz;
        if (dt < dtN) dtN = dt;
        if (4 * S.dtp[q] < dtN) dtN = 4 * S.dtp[q];
    } else {
        Acc *= rp * aFac;
        ax += Acc * dx; ay += Acc * dy; az += Acc * dz;
        if (dt < dtN) dtN = dt;
        if (4 * S.dtp[p] < dtN) dtN = 4 * S.dtp[p];
    }
}

// sph_pair in FP32 (same terms and order); m_p, m_q come with the split
// positions, dv is an FP64 difference rounded once.
__device__ __forceinline__ void sph_pair_f(const TsphSphBufs &S, const TsphDevParts &G, int p, int q,
                                           float dx, float dy, float dz, float fDist2, bool own,
                                           float &ax, float &ay, float &az, float &uPdV,
                                           float &uAV, float &mu, float &dtN) {
    const float4 ap = S.pfa[p], bp = S.pfb[p], aq = S.pfa[q], bq = S.pfb[q];
    const float pc = bp.x, qc = bq.x, ph = ap.x;
    const float r2 = fDist2 * ap.y;
    const float r = sqrtf(r2);
    const float dk = r2 < 1.0f ? -3.0f + 2.25f * r : -0.75f * (2.0f - r) * (2.0f - r) / r;
    const float rs1 = dk * ap.z;
    const float rp = rs1 * G.ph[p].w, rq = rs1 * G.ph[q].w;
    float dvx, dvy, dvz;
    split_dv(S, p, q, dvx, dvy, dvz);
    const float dvdotdr = dvx * dx + dvy * dy + dvz * dz;
    float Acc, dt;
    if (own) {
        uPdV += rq * S.pfc[p].x * dvdotdr;
        Acc = ap.w + aq.w;
    } else {
        uPdV += rp * S.pfc[q].x * dvdotdr;
        Acc = aq.w + ap.w;
    }
    const float fac = cS.dtFacCourantf;
    if (dvdotdr >= 0.0f) {
        dt = fac * ph / (2 * fmaxf(pc, qc));
    } else {
        float absmu = -dvdotdr / sqrtf(fDist2);
        if (absmu > mu) mu = absmu;
        float visc = (cS.alphaf * (pc + qc) + cS.betaf * 1.5f * absmu);
        dt = fac * ph / (0.625f * (pc + qc) + 0.375f * visc);
        visc = (0.5f * (bp.z + bq.z)) * visc * absmu / (bp.y + bq.y);
        uAV += (own ? rq : rp) * (0.5f * visc) * dvdotdr;
        Acc += visc;
    }
    if (own) {
        Acc *= rq;
        ax -= Acc * dx; ay -= Acc * dy; az -= Acc * dz;
        dtN = fminf(dtN, fminf(dt, 4 * bq.w));
    } else {
        Acc *= rp;
        ax += Acc * dx; ay += Acc * dy; az += Acc * dz;
        dtN = fminf(dtN, fminf(dt, 4 * bp.w));
    }
}

__device__ __forceinline__ void split_dx(float4 hi, float4 lo, float4 hj, float4 lj, float &dx,
                                         float &dy, float &dz) {
    dx = (hi.x - hj.x) + (lo.x - lj.x);
    dy = (hi.y - hj.y) + (lo.y - lj.y);
    dz = (hi.z - hj.z) + (lo.z - lj.z);
    if (cS.bPeriodic) {
        const float L = cS.Lf, h = 0.5f * L;
        dx = dx > h ? dx - L : (dx < -h ? dx + L : dx);
        dy = dy > h ? dy - L : (dy < -h ? dy + L : dy);
        dz = dz > h ? dz - L : (dz < -h ? dz + L : dz);
    }
}

// SphPressureTermsSym from the stored lists: particle i sums its own-ball
// pairs N(i) and the pairs R(i) whose ball holds i, each list in ascending
// index, lane-strided, then a fixed-order warp sum.  No tree walk.
template <bool F32>
__global__ void __launch_bounds__(SW * 32) k_pressure_lists(SphArgs A) {
    const int lane = threadIdx.x & 31;
    const unsigned FULL = 0xffffffffu;
    const int ng = cS.ngas;
    const TsphSphBufs &S = A.S;
    if (S.listFlag[0]) return;           // a list overflowed: the tree walk runs instead
    for (;;) {
        int i = 0;
        if (lane == 0) i = atomicAdd(A.work, 1);
        i = __shfl_sync(FULL, i, 0);
        if (i >= ng) break;
        if (!S.need[i]) continue;        // not computed this pass: no pair with an active particle
        const bool ai = A.G.act[i] != 0;
        if constexpr (F32) {
            const float4 hi = A.G.ph[i], lo = A.G.pl[i];
            float ax = 0, ay = 0, az = 0, uPdV = 0, uAV = 0, mu = 0.0f, dtN = FLT_MAX;
            const int *own = S.nbrList + (size_t)i * S.nbrCap;
            const int nOwn = S.nnCount[i];
            for (int e = lane; e < nOwn; e += 32) {
                int j = own[e];
                if (!ai && !A.G.act[j]) continue;
                float dx, dy, dz;
                split_dx(hi, lo, A.G.ph[j], A.G.pl[j], dx, dy, dz);
                sph_pair_f(S, A.G, i, j, dx, dy, dz, dx * dx + dy * dy + dz * dz, true, ax, ay, az,
                           uPdV, uAV, mu, dtN);
            }
            const int ro = i > 0 ? S.roff[i - 1] : 0, nRev = S.roff[i] - ro;
            for (int e = lane; e < nRev; e += 32) {
                int j = S.rlist[ro + e];
                if (!ai && !A.G.act[j]) continue;
                float dx, dy, dz;
                split_dx(A.G.ph[j], A.G.pl[j], hi, lo, dx, dy, dz);
                sph_pair_f(S, A.G, j, i, dx, dy, dz, dx * dx + dy * dy + dz * dz, false, ax, ay, az,
                           uPdV, uAV, mu, dtN);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                ax += __shfl_xor_sync(FULL, ax, o);
                ay += __shfl_xor_sync(FULL, ay, o);
                az += __shfl_xor_sync(FULL, az, o);
                uPdV += __shfl_xor_sync(FULL, uPdV, o);
                uAV += __shfl_xor_sync(FULL, uAV, o);
                mu = fmaxf(mu, __shfl_xor_sync(FULL, mu, o));
                dtN = fminf(dtN, __shfl_xor_sync(FULL, dtN, o));
            }
            if (lane == 0)
                pressure_store(A, i, ai, ax, ay, az, uPdV, uAV, mu,
                               dtN == FLT_MAX ? (double)FLT_MAX : (double)dtN);
            continue;
        }
        const double xi = A.G.x[i], yi = A.G.y[i], zi = A.G.z[i];
        double ax = 0, ay = 0, az = 0, uPdV = 0, uAV = 0, mu = 0.0, dtN = FLT_MAX;
        const int *own = S.nbrList + (size_t)i * S.nbrCap;
        const int nOwn = S.nnCount[i];
        for (int e = lane; e < nOwn; e += 32) {
            int j = own[e];
            if (!ai && !A.G.act[j]) continue;
            double dx, dy, dz;
            double d2 = dist2_exact(xi, yi, zi, A.G.x[j], A.G.y[j], A.G.z[j], dx, dy, dz);
            sph_pair(S, A.G.m, i, j, dx, dy, dz, d2, true, ax, ay, az, uPdV, uAV, mu, dtN);
        }
        const int ro = i > 0 ? S.roff[i - 1] : 0, nRev = S.roff[i] - ro;
        for (int e = lane; e < nRev; e += 32) {
            int j = S.rlist[ro + e];
            if (!ai && !A.G.act[j]) continue;
            double dx, dy, dz;
            double d2 = dist2_exact(A.G.x[j], A.G.y[j], A.G.z[j], xi, yi, zi, dx, dy, dz);
            sph_pair(S, A.G.m, j, i, dx, dy, dz, d2, false, ax, ay, az, uPdV, uAV, mu, dtN);
        }
        ax = wsum(ax); ay = wsum(ay); az = wsum(az); uPdV = wsum(uPdV); uAV = wsum(uAV);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            double a = __shfl_xor_sync(FULL, mu, o);
            double b = __shfl_xor_sync(FULL, dtN, o);
            mu = a > mu ? a : mu;
            dtN = b < dtN ? b : dtN;
        }
        if (lane == 0) pressure_store(A, i, ai, ax, ay, az, uPdV, uAV, mu, dtN);
    }
}

// SphPressureTermsSym as a gather over both roles of every pair.
__global__ void __launch_bounds__(SW * 32) k_pressure(SphArgs A) {
    __shared__ int stackAll[SW][SSTK];
    int *stack = stackAll[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const unsigned FULL = 0xffffffffu;
    const int ng = cS.ngas;
    const double aFac = 1.0, vFac = 1.0, H = 0.0;
    if (!A.S.listFlag[0]) return;        // the list kernel did the work
    for (;;) {
        int i = 0;
        if (lane == 0) i = atomicAdd(A.work, 1);
        i = __shfl_sync(FULL, i, 0);
        if (i >= ng) break;
        const double xi = A.G.x[i], yi = A.G.y[i], zi = A.G.z[i];
        const float xf = (float)xi, yf = (float)yi, zf = (float)zi;
        if (!A.S.need[i]) continue;
        const double fbi = A.S.fBall2[i];
        const TsphSphBufs &S = A.S;
        const bool ai = A.G.act[i] != 0;
        double ax = 0, ay = 0, az = 0, uPdV = 0, uAV = 0, mu = 0.0, dtN = FLT_MAX;
        int sp = 1;
        if (lane == 0) stack[0] = A.T.sysRoot[A.G.rid[i]];
        __syncwarp();
        bool bad = false;
        while (sp > 0) {
            int take = sp < 32 ? sp : 32;
            int node = lane < take ? stack[sp - take + lane] : -1;
            __syncwarp();
            sp -= take;
            bool open = false, leaf = false;
            int4 lk = make_int4(0, 0, -1, 0);
            if (node >= 0) {
                lk = A.T.wlink[node];
                double nb = __longlong_as_double((long long)S.nodeBall2[node]);
                float bound = (float)(nb > fbi ? nb : fbi) * 1.00001f;
                float d2 = box_d2f(xf, yf, zf, A.T.wcomh[node], A.T.wcoml[node]);
                if (d2 <= bound) {
                    if (lk.z >= 0) open = true;
                    else leaf = true;
                }
            }
            unsigned bo = __ballot_sync(FULL, open);
            if (sp + 2 * __popc(bo) > SSTK) { bad = true; break; }
            if (open) {
                int pos = sp + 2 * __popc(bo & lane_lt_s());
                stack[pos] = lk.z;
                stack[pos + 1] = node + 1;
            }
            sp += 2 * __popc(bo);
            int cnt = leaf ? lk.y : 0;
            for (int kk = 0; kk < cnt; ++kk) {
                int j = lk.x + kk;
                if (!S.need[j] || (!ai && !A.G.act[j])) continue;
                double xj = A.G.x[j], yj = A.G.y[j], zj = A.G.z[j];
                double dxi, dyi, dzi, dxj, dyj, dzj;
                double d2i = dist2_exact(xi, yi, zi, xj, yj, zj, dxi, dyi, dzi);
                double d2j = dist2_exact(xj, yj, zj, xi, yi, zi, dxj, dyj, dzj);
                double fbj = S.fBall2[j];
                bool inI = d2i <= fbi, inJ = d2j <= fbj;
                if (!inI && !inJ) continue;
                for (int role = 0; role < 2; ++role) {
                    if (role == 0 && !inI) continue;
                    if (role == 1 && !inJ) continue;
                    // p = owner of the ball, q = the other particle
                    int p = role == 0 ? i : j, q = role == 0 ? j : i;
                    double dx = role == 0 ? dxi : dxj, dy = role == 0 ? dyi : dyj,
                           dz = role == 0 ? dzi : dzj;
                    double fDist2 = role == 0 ? d2i : d2j;
                    double fbp = S.fBall2[p];
                    double pc = S.cs[p], pMass = A.G.m[p], pDensity = S.rho[p];
                    double pPoverRho2 = S.pr2[p], pd2 = pDensity * pDensity;
                    double pPoverRho2f = (pPoverRho2 * pd2 + 0) / pd2;
                    double ph = sqrt(0.25 * fbp);
                    double ih2 = 4.0 / fbp;
                    double fNorm = 0.5 * M_1_PI * ih2 / ph;
                    double fNorm1 = fNorm * ih2;
                    double r2 = fDist2 * ih2;
                    double rs1 = dkern_m4(r2) * fNorm1;
                    double rp = rs1 * pMass, rq = rs1 * A.G.m[q];
                    double dvx = S.vx[p] - S.vx[q], dvy = S.vy[p] - S.vy[q], dvz = S.vz[p] - S.vz[q];
                    double dvdotdr = vFac * (dvx * dx + dvy * dy + dvz * dz) + fDist2 * H;
                    double qPoverRho2 = S.pr2[q], qd2 = S.rho[q] * S.rho[q];
                    double qPoverRho2f = (qPoverRho2 * qd2 + 0) / qd2;
                    double qc = S.cs[q];
                    double Acc, dt;
                    if (role == 0) {
                        uPdV += rq * pPoverRho2 * dvdotdr;
                        Acc = pPoverRho2f + qPoverRho2f;
                    } else {
                        uPdV += rp * qPoverRho2 * dvdotdr;
                        Acc = qPoverRho2f + pPoverRho2f;
                    }
                    if (dvdotdr >= 0.0) {
                        dt = cS.dtFacCourant * ph / (2 * (pc > qc ? pc : qc));
                    } else {
                        double absmu = -dvdotdr * aFac / sqrt(fDist2);
                        if (absmu > mu) mu = absmu;
                        double visc = (cS.alpha * (pc + qc) + cS.beta * 1.5 * absmu);
                        dt = cS.dtFacCourant * ph / (0.625 * (pc + qc) + 0.375 * visc);
                        visc = (0.5 * (S.bal[p] + S.bal[q])) * visc * absmu / (pDensity + S.rho[q]);
                        if (role == 0) uAV += rq * (0.5 * visc) * dvdotdr;
                        else uAV += rp * (0.5 * visc) * dvdotdr;
                        Acc += visc;
                    }
                    if (role == 0) {
                        Acc *= rq * aFac;
                        ax -= Acc * dx; ay -= Acc * dy; az -= Acc * dz;
                        if (dt < dtN) dtN = dt;
                        if (4 * S.dtp[q] < dtN) dtN = 4 * S.dtp[q];
                    } else {
                        Acc *= rp * aFac;
                        ax += Acc * dx; ay += Acc * dy; az += Acc * dz;
                        if (dt < dtN) dtN = dt;
                        if (4 * S.dtp[p] < dtN) dtN = 4 * S.dtp[p];
                    }
                }
            }
            __syncwarp();
        }
        if (bad) {
            if (lane == 0) atomicOr(&A.cnt->status, 1u << TSPH_ERR_STACK_OVERFLOW);
            continue;
        }
        ax = wsum(ax); ay = wsum(ay); az = wsum(az); uPdV = wsum(uPdV); uAV = wsum(uAV);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            double a = __shfl_xor_sync(FULL, mu, o);
            double b = __shfl_xor_sync(FULL, dtN, o);
            mu = a > mu ? a : mu;
            dtN = b < dtN ? b : dtN;
        }
        if (lane == 0) pressure_store(A, i, ai, ax, ay, az, uPdV, uAV, mu, dtN);
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// gathers/scatters between caller order and gas-tree order
// ---------------------------------------------------------------------------
__global__ void k_gas_identity(int ng, int *iord) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ng) iord[i] = i;
}

__global__ void k_gas_gather_pos(int ng, TsphDevState C, TsphDevParts G) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ng) return;
    int o = G.iord[i];
    G.x[i] = C.x[o]; G.y[i] = C.y[o]; G.z[i] = C.z[o];   // masses and softenings after the build
}

// ---------------------------------------------------------------------------
// Density passes over active rungs.  Every particle an active one pairs
// with must have its density, ball and lists of this pass: the active
// particles, their gather neighbours N(i), and the particles j whose ball
// holds an active i.  j's ball radius cannot exceed its radius at its last
// density plus twice the largest distance any gas particle drifted since
// the last pass over all gas (the k particles inside the old ball moved at
// most that far, and so did j), so every j with an active particle inside
// that bound is computed too.  The active particles' results then equal
// those of a pass over all gas; the reference's FastGas branch
// (master.c:9270-9298) serves the same purpose with marking passes.
// ---------------------------------------------------------------------------
__global__ void k_act_list(int ng, const int *__restrict__ act, int *need, int *list, int *listN) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ng) return;
    const int a = act[i] != 0;
    need[i] = a;
    if (a) list[atomicAdd(&listN[0], 1)] = i;
}

__global__ void k_mark_gather(int na, const int *__restrict__ list, TsphSphBufs S) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int a = (int)(t / S.nbrCap), e = (int)(t % S.nbrCap);
    if (a >= na) return;
    const int i = list[a];
    if (e >= S.nnCount[i]) return;
    S.need[S.nbrList[(size_t)i * S.nbrCap + e]] = 1;
}

__global__ void k_disp_max(int ng, const double *__restrict__ disp, unsigned long long *out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    warp_max_abs(i < ng ? disp[i] : 0.0, out);
}

__global__ void k_rbound(int ng, const int *__restrict__ iord, const double *__restrict__ fb2prev,
                         const unsigned long long *dmax, double *rb2) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ng) return;
    double dm;
    memcpy(&dm, dmax, sizeof(dm));
    const double r = (sqrt(fb2prev[iord[i]]) + 2.0 * dm) * (1.0 + 1e-9);
    rb2[i] = r * r * (1.0 + 1e-9);
}

__global__ void __launch_bounds__(SW * 32) k_mark_scatter(SphArgs A, const unsigned long long *nodeB) {
    __shared__ int stackAll[SW][SSTK];
    int *stack = stackAll[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const unsigned FULL = 0xffffffffu;
    const TsphSphBufs &S = A.S;
    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(A.work, 1);
        t = __shfl_sync(FULL, t, 0);
        if (t >= *A.nList) break;
        const int i = A.list[t];
        const double xi = A.G.x[i], yi = A.G.y[i], zi = A.G.z[i];
        const float xf = (float)xi, yf = (float)yi, zf = (float)zi;
        int sp = 1;
        if (lane == 0) stack[0] = A.T.sysRoot[A.G.rid[i]];
        __syncwarp();
        bool bad = false;
        while (sp > 0) {
            int take = sp < 32 ? sp : 32;
            int node = lane < take ? stack[sp - take + lane] : -1;
            __syncwarp();
            sp -= take;
            bool open = false, leaf = false;
            int4 lk = make_int4(0, 0, -1, 0);
            if (node >= 0) {
                lk = A.T.wlink[node];
                const double nb = __longlong_as_double((long long)nodeB[node]);
                const float d2 = box_d2f(xf, yf, zf, A.T.wcomh[node], A.T.wcoml[node]);
                if (d2 <= (float)nb * 1.00001f) {
                    if (lk.z >= 0) open = true;
                    else leaf = true;
                }
            }
            unsigned bo = __ballot_sync(FULL, open);
            if (sp + 2 * __popc(bo) > SSTK) { bad = true; break; }
            if (open) {
                int pos = sp + 2 * __popc(bo & lane_lt_s());
                stack[pos] = lk.z;
                stack[pos + 1] = node + 1;
            }
            sp += 2 * __popc(bo);
            const int cnt = leaf ? lk.y : 0;
            for (int kk = 0; kk < cnt; ++kk) {
                const int j = lk.x + kk;
                double dx, dy, dz;
                if (dist2_exact(xi, yi, zi, A.G.x[j], A.G.y[j], A.G.z[j], dx, dy, dz) <= S.rb2[j])
                    S.need[j] = 1;
            }
            __syncwarp();
        }
        if (bad && lane == 0) atomicOr(&A.cnt->status, 1u << TSPH_ERR_STACK_OVERFLOW);
        __syncwarp();
    }
}

__global__ void k_need_list(int ng, const int *__restrict__ act, const int *__restrict__ need,
                            int *list2, int *listN) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ng) return;
    if (need[i] && !act[i]) list2[atomicAdd(&listN[1], 1)] = i;
}

__global__ void k_gas_maxabs(int ng, TsphDevParts G, unsigned long long *out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double a = 0.0;
    if (i < ng) a = fmax(fabs(G.x[i]), fmax(fabs(G.y[i]), fabs(G.z[i])));
    warp_max_abs(a, out);
}

__global__ void k_gas_gather_vel(int ng, TsphDevState C, const int *__restrict__ iord, TsphSphBufs S) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ng) return;
    int o = iord[i];
    const double vx = C.vpx[o], vy = C.vpy[o], vz = C.vpz[o];
    S.vx[i] = vx; S.vy[i] = vy; S.vz[i] = vz;
    S.u[i] = C.upred[o];
    // FP32 hi/lo parts: (hj - hi) + (lj - li) is the velocity difference to
    // FP32 rounding however large a bulk flow both share
    float hx, lx, hy, ly, hz, lz;
    split2f(vx, hx, lx);
    split2f(vy, hy, ly);
    split2f(vz, hz, lz);
    S.vh[i] = make_float4(hx, hy, hz, 0.0f);
    S.vl[i] = make_float4(lx, ly, lz, 0.0f);
}


// FP32 node boxes for the gas walks (stored in wcomh/wcoml of the gas tree)
__global__ void k_gas_nodes(TsphDevTree T) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= T.dcnt[0]) return;
    const double *b = &T.bnd[6 * i];
    T.wcomh[i] = make_float4((float)b[0], (float)b[1], (float)b[2], 0.0f);
    T.wcoml[i] = make_float4((float)b[3], (float)b[4], (float)b[5], 0.0f);
    T.wlink[i] = make_int4(T.pLower[i], T.pUpper[i] - T.pLower[i] + 1, T.upper[i], 0);
}

// pressure-pass results to caller order: forces and energy rates of the
// active particles, dtNew and mumax of every gas particle
__global__ void k_scatter_hydro(int ng, TsphDevParts G, TsphSphBufs S, TsphDevState C) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ng || !S.need[i]) return;
    int o = G.iord[i];
    C.dtNew[o] = S.dtNew[i];
    C.mumax[o] = S.mumax[i];
    if (!G.act[i]) return;
    C.hax[o] = S.hax[i]; C.hay[o] = S.hay[i]; C.haz[o] = S.haz[i];
    C.udot[o] = S.uPdV[i] + S.uAV[i];
    C.updv[o] = S.uPdV[i];
}

__global__ void k_to_caller1(int ng, const int *__restrict__ iord, const double *__restrict__ a,
                             int stride, int off, double *dst, int dstride, int doff) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ng) return;
    dst[dstride * iord[i] + doff] = a[stride * i + off];
}

__global__ void k_save_prev(int ng, const int *__restrict__ iord, const double *__restrict__ fb2,
                            const double *__restrict__ divv, double *fb2prev, double *divvprev,
                            const int *__restrict__ need) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ng || !need[i]) return;
    fb2prev[iord[i]] = fb2[i];
    divvprev[iord[i]] = divv[i];
}

__global__ void k_load_vel(int n, const double *__restrict__ v3, TsphDevState C) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    C.vx[i] = C.vpx[i] = v3[3 * i];
    C.vy[i] = C.vpy[i] = v3[3 * i + 1];
    C.vz[i] = C.vpz[i] = v3[3 * i + 2];
}

__global__ void k_load_u(int ng, TsphDevState C) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ng) return;
    C.upred[i] = C.u[i];
    C.udot[i] = 0.0;
}

static void set_sph_const(tsph_ctx *ctx, const tsph_sph_params *sp) {
    SphConst c;
    memset(&c, 0, sizeof(c));
    c.ngas = ctx->ngas;
    c.k = sp->nSmooth < ctx->ngas ? sp->nSmooth : ctx->ngas;
    c.bPeriodic = sp->bPeriodic;
    c.L = sp->dPeriod;
    c.alpha = sp->alpha;
    c.beta = sp->beta;
    c.gamma = sp->gamma;
    c.gammam1 = sp->gamma - 1;
    c.dtFacCourant = sp->dEtaCourant * 1.0 * 2 / 1.6;   // pkdDtFacCourant, a = 1
    c.Lf = (float)c.L;
    c.alphaf = (float)c.alpha;
    c.betaf = (float)c.beta;
    c.dtFacCourantf = (float)c.dtFacCourant;
    c.limiter = sp->iViscosityLimiter;
    // FP32 box tests: pad by a few ulps of the largest |coordinate| (of all
    // systems), measured by k_gas_maxabs
    double r = ctx->gasScale;
    if (!ctx->capturing) {
        unsigned long long bits = 0;
        cudaMemcpy(&bits, ctx->dAux, sizeof(bits), cudaMemcpyDeviceToHost);
        memcpy(&r, &bits, sizeof(r));
        ctx->gasScale = r;
    }
    if (ctx->capLimit > r) r = ctx->capLimit;   // a captured step's coordinate bound
    c.erel = 4.0f * 5.9604645e-08f;
    c.eabs = (float)(ldexp(1.0, -44) * r + (sp->bPeriodic ? 8.0 * 5.960464477539063e-08 * sp->dPeriod : 0.0)) + 1e-30f;
    if (sp->bPeriodic) r += sp->dPeriod;
    c.margin = (float)(8.0 * 5.960464477539063e-08 * r) + 1e-30f;
    cudaMemcpyToSymbolAsync(cS, &c, sizeof(c), 0, cudaMemcpyHostToDevice, ctx->stream);
}

extern "C" int tsph_set_velocities(tsph_ctx *ctx, const double *vel, int ngas, const double *u) {
    if (!ctx || !vel || ngas < 0) return TSPH_ERR_ARG;
    if (!ctx->haveParts) return TSPH_ERR_STATE;
    if (ngas > ctx->n || (ngas > 0 && !u)) return TSPH_ERR_ARG;
    cudaSetDevice(ctx->device);
    const int n = ctx->n;
    ctx->ngas = ngas;
    ctx->G.n = ngas;
    ctx->sysVersion++;
    ctx->S.haveDensity = ctx->S.havePressure = false;
    ctx->hnet.havePrev = false;
    if (n == 0) { ctx->haveVel = true; return TSPH_OK; }
    TSPH_CK(cudaMemcpyAsync(ctx->dStage, vel, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
    k_load_vel<<<tsph_blocks(n, 256), 256, 0, ctx->stream>>>(n, ctx->dStage, ctx->C);
    TSPH_LAUNCH_CK("k_load_vel");
    if (ngas > 0) {
        TSPH_CK(cudaMemcpyAsync(ctx->C.u, u, sizeof(double) * ngas, cudaMemcpyHostToDevice, ctx->stream));
        k_load_u<<<tsph_blocks(ngas, 256), 256, 0, ctx->stream>>>(ngas, ctx->C);
        TSPH_LAUNCH_CK("k_load_u");
        k_gas_identity<<<tsph_blocks(ngas, 256), 256, 0, ctx->stream>>>(ngas, ctx->G.iord);
        TSPH_LAUNCH_CK("k_gas_identity");
        int rc = tsph_apply_gas_systems(ctx);
        if (rc) return rc;
    }
    TSPH_CK(cudaStreamSynchronize(ctx->stream));   // host buffers reusable on return
    ctx->haveVel = true;
    return TSPH_OK;
}

// The gas of a particle set whose caller-order state (u, uPred, vPred and
// the gas tree's identity order) is already on the device: the first ngas
// particles become gas, as tsph_set_velocities makes them.
int tsph_load_gas(tsph_ctx *ctx, int ngas) {
    if (ngas < 0 || ngas > ctx->n) return TSPH_ERR_ARG;
    ctx->ngas = ngas;
    ctx->G.n = ngas;
    ctx->sysVersion++;
    ctx->S.haveDensity = ctx->S.havePressure = false;
    ctx->hnet.havePrev = false;
    if (ngas > 0) {
        int rc = tsph_apply_gas_systems(ctx);
        if (rc) return rc;
    }
    TSPH_CK(cudaStreamSynchronize(ctx->stream));
    ctx->haveParts = ctx->haveVel = true;
    return TSPH_OK;
}

static int launch_knn(tsph_ctx *ctx, const tsph_sph_params *sp, const SphArgs &A) {
    const bool cap = ctx->capturing;
    // the buckets' candidate lists only in a bucket launch; the attribute
    // allows the larger size for every launch (a capture sets none)
    const size_t smMax = (sizeof(KnnSmem) + sizeof(KnnBatch) + sizeof(int) * BCAP) * SW;
    const size_t sm = A.bucketGather ? smMax : (sizeof(KnnSmem) + sizeof(KnnBatch)) * SW;
    if (sp->precision == TSPH_FP32) {
        if (!cap)
            TSPH_CK(cudaFuncSetAttribute(k_knn_density<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smMax));
        k_knn_density<true><<<ctx->smCount * 6, SW * 32, sm, ctx->stream>>>(A);
        TSPH_LAUNCH_CK("k_knn_density<f32>");
    } else {
        if (!cap)
            TSPH_CK(cudaFuncSetAttribute(k_knn_density<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smMax));
        k_knn_density<false><<<ctx->smCount * 6, SW * 32, sm, ctx->stream>>>(A);
        TSPH_LAUNCH_CK("k_knn_density<f64>");
    }
    return TSPH_OK;
}

// The density pass over only the particles the active ones need (see
// k_act_list ... k_need_list).  Returns in *nComputed the particles done.
static int run_density_subset(tsph_ctx *ctx, const tsph_sph_params *sp, SphArgs A, int na) {
    const int ng = ctx->ngas;
    TsphSphBufs &S = ctx->S;
    int *work = A.work;
    // the active particles
    A.list = S.list;
    A.nList = S.listN;
    int rc = launch_knn(ctx, sp, A);
    if (rc) return rc;
    // their gather neighbours
    k_mark_gather<<<tsph_blocks((long long)na * S.nbrCap, 256), 256, 0, ctx->stream>>>(na, S.list, S);
    TSPH_LAUNCH_CK("k_mark_gather");
    // particles whose ball can hold an active one
    unsigned long long *dmax = ctx->dAux + 40;
    TSPH_CK(cudaMemsetAsync(dmax, 0, sizeof(unsigned long long), ctx->stream));
    k_disp_max<<<tsph_blocks(ng, 256), 256, 0, ctx->stream>>>(ng, ctx->C.disp, dmax);
    TSPH_LAUNCH_CK("k_disp_max");
    k_rbound<<<tsph_blocks(ng, 256), 256, 0, ctx->stream>>>(ng, ctx->G.iord, ctx->C.fb2prev, dmax, S.rb2);
    TSPH_LAUNCH_CK("k_rbound");
    TSPH_CK(cudaMemsetAsync(S.nodeBall2, 0, sizeof(unsigned long long) * ctx->TG.nNodes, ctx->stream));
    k_node_ball<<<tsph_blocks(ng, 256), 256, 0, ctx->stream>>>(ng, ctx->TG, ctx->G.rid, S.rb2, S.listFlag,
                                                              S.nodeBall2, nullptr, 1);
    TSPH_LAUNCH_CK("k_node_ball");
    TSPH_CK(cudaMemsetAsync(work, 0, sizeof(int), ctx->stream));
    k_mark_scatter<<<ctx->smCount * 4, SW * 32, 0, ctx->stream>>>(A, S.nodeBall2);
    TSPH_LAUNCH_CK("k_mark_scatter");
    k_need_list<<<tsph_blocks(ng, 256), 256, 0, ctx->stream>>>(ng, ctx->G.act, S.need, S.list2, S.listN);
    TSPH_LAUNCH_CK("k_need_list");
    // and the rest of them
    A.list = S.list2;
    A.nList = S.listN + 1;
    TSPH_CK(cudaMemsetAsync(work, 0, sizeof(int), ctx->stream));
    return launch_knn(ctx, sp, A);
}

static int run_density(tsph_ctx *ctx, const tsph_sph_params *sp, tsph_smooth_out *out) {
    const int ng = ctx->ngas;
    TsphSphBufs &S = ctx->S;
    const bool cap = ctx->capturing;
    // a captured pass may seed from the h-network but not collect samples
    // (their count is host state that a replay would not advance)
    if (cap && sp->bLearnedH && ctx->hnet.collect) return TSPH_ERR_UNSUPPORTED;
    if (cap && ctx->actRung > 0) return TSPH_ERR_UNSUPPORTED;
    if (!cap) cudaEventRecord(ctx->ev[5], ctx->stream);
    k_gas_gather_pos<<<tsph_blocks(ng, 256), 256, 0, ctx->stream>>>(ng, ctx->C, ctx->G);
    TSPH_LAUNCH_CK("k_gas_gather_pos");
    if (!ctx->capturing) {
        TSPH_CK(cudaMemsetAsync(ctx->dAux, 0, sizeof(unsigned long long), ctx->stream));
        k_gas_maxabs<<<tsph_blocks(ng, 256), 256, 0, ctx->stream>>>(ng, ctx->G, ctx->dAux);
        TSPH_LAUNCH_CK("k_gas_maxabs");
    }
    int rc = tsph_build_tree(ctx, ctx->G, ctx->TG, ng, 16);
    if (rc) return rc;
    k_gas_nodes<<<tsph_blocks(ctx->TG.nNodes, 256), 256, 0, ctx->stream>>>(ctx->TG);
    TSPH_LAUNCH_CK("k_gas_nodes");
    k_gas_gather_vel<<<tsph_blocks(ng, 256), 256, 0, ctx->stream>>>(ng, ctx->C, ctx->G.iord, S);
    TSPH_LAUNCH_CK("k_gas_gather_vel");
    k_gas_split<<<tsph_blocks(ng, 256), 256, 0, ctx->stream>>>(ng, ctx->G, S.u);
    TSPH_LAUNCH_CK("k_gas_split");
    if (!cap) set_sph_const(ctx, sp);
    const int kk = sp->nSmooth < ng ? sp->nSmooth : ng;
    rc = tsph_hnet_features(ctx, kk);
    if (rc) return rc;
    if (sp->bLearnedH) {
        rc = tsph_hnet_seed(ctx);
        if (rc) return rc;
    } else {
        S.haveSeed = false;
    }
    SphArgs A;
    A.T = ctx->TG;
    A.G = ctx->G;
    A.S = S;
    A.cnt = ctx->dCnt;
    A.work = (int *)&ctx->dCnt->pad;
    A.seed = (sp->bLearnedH && S.haveSeed) ? S.seed : nullptr;
    A.C = ctx->C;
    A.list = nullptr;
    A.nList = nullptr;
    TSPH_CK(cudaMemsetAsync(ctx->dCnt, 0, sizeof(TsphDevCounters), ctx->stream));
    TSPH_CK(cudaMemsetAsync(S.listFlag, 0, sizeof(int), ctx->stream));
    // a pass over active rungs computes only the particles the active ones
    // need when they are a minority of the gas
    int na = ng;
    S.subset = false;
    if (ctx->actRung > 0) {
        TSPH_CK(cudaMemsetAsync(S.listN, 0, 4 * sizeof(int), ctx->stream));
        k_act_list<<<tsph_blocks(ng, 256), 256, 0, ctx->stream>>>(ng, ctx->G.act, S.need, S.list, S.listN);
        TSPH_LAUNCH_CK("k_act_list");
        TSPH_CK(cudaMemcpyAsync(&na, S.listN, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        TSPH_CK(cudaStreamSynchronize(ctx->stream));
        S.subset = 2 * na < ng;
    }
    if (!cap) cudaEventRecord(ctx->ev[6], ctx->stream);
    if (S.subset) {
        rc = run_density_subset(ctx, sp, A, na);
    } else {
        TSPH_CK(cudaMemsetAsync(S.need, 0x01, sizeof(int) * ng, ctx->stream));   // every particle
        // one gather per gas bucket pays with the h-network's tight seeds;
        // with the tree's coarse ones the buckets' union balls grow too large
        // (measured: 1/r collapse 2.01 -> 1.77 ms with learned seeds; 128
        // Plummer/Hernquist systems 3.70 -> 5.36 ms with tree seeds)
        A.bucketGather = A.seed != nullptr;
        rc = launch_knn(ctx, sp, A);
    }
    if (rc) return rc;
    if (cap) {
        rc = tsph_fold_status(ctx);
        if (rc) return rc;
        TSPH_CK(cudaMemsetAsync(ctx->C.disp, 0, sizeof(double) * ng, ctx->stream));
        k_save_prev<<<tsph_blocks(ng, 256), 256, 0, ctx->stream>>>(ng, ctx->G.iord, S.fBall2, S.divv,
                                                                  ctx->C.fb2prev, ctx->C.divvprev, S.need);
        TSPH_LAUNCH_CK("k_save_prev");
        S.haveDensity = true;
        S.havePressure = false;
        S.last = *sp;
        return TSPH_OK;
    }
    cudaEventRecord(ctx->ev[7], ctx->stream);
    TSPH_CK(cudaMemcpyAsync(ctx->hCnt, ctx->dCnt, sizeof(TsphDevCounters), cudaMemcpyDeviceToHost,
                            ctx->stream));
    TSPH_CK(cudaStreamSynchronize(ctx->stream));
    cudaEventElapsedTime(&ctx->timings[4], ctx->ev[5], ctx->ev[6]);
    cudaEventElapsedTime(&ctx->timings[5], ctx->ev[6], ctx->ev[7]);
    unsigned st = ctx->hCnt->status;
    if (st) for (int k = 1; k < 32; ++k) if (st & (1u << k)) return k;
    S.nComputed = ng;
    if (S.subset) {
        int nl[2];
        TSPH_CK(cudaMemcpy(nl, S.listN, sizeof(nl), cudaMemcpyDeviceToHost));
        S.nComputed = nl[0] + nl[1];
    } else {
        // a pass over all gas starts the drift bound afresh
        TSPH_CK(cudaMemsetAsync(ctx->C.disp, 0, sizeof(double) * ng, ctx->stream));
        // h-network: samples of this pass, then this pass becomes "previous"
        rc = tsph_hnet_append(ctx);
        if (rc) return rc;
    }
    k_save_prev<<<tsph_blocks(ng, 256), 256, 0, ctx->stream>>>(ng, ctx->G.iord, S.fBall2, S.divv,
                                                              ctx->C.fb2prev, ctx->C.divvprev, S.need);
    TSPH_LAUNCH_CK("k_save_prev");
    ctx->hnet.havePrev = true;
    S.nFallback = (int)ctx->hCnt->nExactTests;
    S.haveDensity = true;
    S.havePressure = false;
    S.last = *sp;
    if (out) {
        out->nSmoothed = S.nComputed;
        out->nFallback = S.nFallback;
        out->dPairs = (double)ctx->hCnt->nPartPP;
        out->dCandidates = (double)ctx->hCnt->nCellNewt;
        out->bSeeded = S.haveSeed ? 1 : 0;
    }
    return TSPH_OK;
}

static int run_pressure(tsph_ctx *ctx, const tsph_sph_params *sp, tsph_smooth_out *out) {
    const int ng = ctx->ngas;
    TsphSphBufs &S = ctx->S;
    const bool cap = ctx->capturing;
    if (!cap) {
        set_sph_const(ctx, sp);
        cudaEventRecord(ctx->ev[8], ctx->stream);
    }
    k_gas_pressure<<<tsph_blocks(ng, 256), 256, 0, ctx->stream>>>(ng, S, ctx->G.iord, ctx->C);
    TSPH_LAUNCH_CK("k_gas_pressure");
    // reverse neighbour lists (the kernels stand down when a list overflowed)
    TSPH_CK(cudaMemsetAsync(S.rcnt, 0, sizeof(int) * ng, ctx->stream));
    TSPH_CK(cudaMemsetAsync(S.rcur, 0, sizeof(int) * ng, ctx->stream));
    TSPH_CK(cudaMemsetAsync(S.listFlag + 1, 0, 3 * sizeof(int), ctx->stream));
    const long long pairSlots = (long long)ng * S.nbrCap;
    k_rev_count<<<tsph_blocks(pairSlots, 256), 256, 0, ctx->stream>>>(ng, S);
    TSPH_LAUNCH_CK("k_rev_count");
    int rc = tsph_scan_inclusive(ctx, S.rcnt, S.roff, ng);
    if (rc) return rc;
    k_rev_fill<<<tsph_blocks(pairSlots, 256), 256, 0, ctx->stream>>>(ng, S);
    TSPH_LAUNCH_CK("k_rev_fill");
    k_rev_sort<<<ctx->smCount * 4, SW * 32, 0, ctx->stream>>>(ng, S, S.listFlag + 1);
    TSPH_LAUNCH_CK("k_rev_sort");
    TSPH_CK(cudaMemsetAsync(S.nodeBall2, 0, sizeof(unsigned long long) * ctx->TG.nNodes, ctx->stream));
    k_node_ball<<<tsph_blocks(ng, 256), 256, 0, ctx->stream>>>(ng, ctx->TG, ctx->G.rid, S.fBall2,
                                                              S.listFlag, S.nodeBall2, S.need, 0);
    TSPH_LAUNCH_CK("k_node_ball");
    SphArgs A;
    A.T = ctx->TG;
    A.G = ctx->G;
    A.S = S;
    A.cnt = ctx->dCnt;
    A.work = (int *)&ctx->dCnt->pad;
    A.seed = nullptr;
    A.C = ctx->C;
    TSPH_CK(cudaMemsetAsync(ctx->dCnt, 0, sizeof(TsphDevCounters), ctx->stream));
    SphArgs AL = A;
    AL.work = S.listFlag + 2;
    if (sp->precision == TSPH_FP32) {
        k_pressure_lists<true><<<ctx->smCount * 8, SW * 32, 0, ctx->stream>>>(AL);
        TSPH_LAUNCH_CK("k_pressure_lists<f32>");
    } else {
        k_pressure_lists<false><<<ctx->smCount * 8, SW * 32, 0, ctx->stream>>>(AL);
        TSPH_LAUNCH_CK("k_pressure_lists<f64>");
    }
    k_pressure<<<ctx->smCount * 4, SW * 32, 0, ctx->stream>>>(A);
    TSPH_LAUNCH_CK("k_pressure");
    k_scatter_hydro<<<tsph_blocks(ng, 256), 256, 0, ctx->stream>>>(ng, ctx->G, S, ctx->C);
    TSPH_LAUNCH_CK("k_scatter_hydro");
    if (cap) {
        S.havePressure = true;
        return tsph_fold_status(ctx);
    }
    cudaEventRecord(ctx->ev[9], ctx->stream);
    TSPH_CK(cudaMemcpyAsync(ctx->hCnt, ctx->dCnt, sizeof(TsphDevCounters), cudaMemcpyDeviceToHost,
                            ctx->stream));
    TSPH_CK(cudaStreamSynchronize(ctx->stream));
    cudaEventElapsedTime(&ctx->timings[6], ctx->ev[8], ctx->ev[9]);
    unsigned st = ctx->hCnt->status;
    if (st) for (int k = 1; k < 32; ++k) if (st & (1u << k)) return k;
    S.havePressure = true;
    if (out) {
        memset(out, 0, sizeof(*out));
        out->nSmoothed = ng;
    }
    return TSPH_OK;
}

extern "C" int tsph_smooth(tsph_ctx *ctx, int smx_type, const tsph_sph_params *sp,
                           tsph_smooth_out *out) {
    if (!ctx || !sp) return TSPH_ERR_ARG;
    if (smx_type != TSPH_SMX_DENDVDX && smx_type != TSPH_SMX_SPHPRESSURETERMS &&
        smx_type != TSPH_SMX_DENSITY)
        return TSPH_ERR_UNSUPPORTED;
    if (!ctx->haveParts || !ctx->haveVel) return TSPH_ERR_STATE;
    if (sp->nSmooth < 1 || sp->gamma <= 1.0) return TSPH_ERR_ARG;
    if (sp->bPeriodic && !(sp->dPeriod > 0)) return TSPH_ERR_ARG;
    if (sp->precision != TSPH_FP64 && sp->precision != TSPH_FP32) return TSPH_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->ngas == 0) {
        if (out) memset(out, 0, sizeof(*out));
        return TSPH_OK;
    }
    if (ctx->TG.nR > 1) {
        // several systems: isolated, and each needs nSmooth gas particles
        if (sp->bPeriodic) return TSPH_ERR_UNSUPPORTED;
        for (int r = 0; r < ctx->TG.nR; ++r)
            if (ctx->TG.hHi[r] - ctx->TG.hLo[r] + 1 < sp->nSmooth) return TSPH_ERR_ARG;
    }
    if (!ctx->capturing) ctx->sysVersion++;   // constants change: recapture a step graph
    // SMX_DENSITY (Density, smoothfcn.c:239-256) is the density part of the
    // same pass: the kNN fBall2 and fDensity = 1/pi ih^3 sum m_j W (the
    // velocity-gradient fields come along)
    if (smx_type == TSPH_SMX_DENDVDX || smx_type == TSPH_SMX_DENSITY) return run_density(ctx, sp, out);
    if (!ctx->S.haveDensity) return TSPH_ERR_STATE;
    return run_pressure(ctx, sp, out);
}

extern "C" int tsph_get_sph(tsph_ctx *ctx, double *out16, double *dtNew, double *mumax) {
    if (!ctx) return TSPH_ERR_ARG;
    if (!ctx->S.haveDensity) return TSPH_ERR_STATE;
    cudaSetDevice(ctx->device);
    const int ng = ctx->ngas;
    TsphSphBufs &S = ctx->S;
    const int *iord = ctx->G.iord;
    if (out16 && ng > 0) {
        const double *src[16] = {S.fBall2, S.rho, S.divv, S.curl, S.curl, S.curl, S.dvds, S.bal,
                                 S.diff, S.pr2, S.cs, S.hax, S.hay, S.haz, S.uPdV, S.uAV};
        int strd[16] = {1, 1, 1, 3, 3, 3, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1};
        int off[16] = {0, 0, 0, 0, 1, 2, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
        TSPH_CK(cudaMemsetAsync(ctx->dStage, 0, sizeof(double) * 3 * ng, ctx->stream));
        // 16 fields interleaved: stage holds 3*cap doubles, so copy in groups of 3
        for (int f0 = 0; f0 < 16; f0 += 3) {
            int nf = 16 - f0 < 3 ? 16 - f0 : 3;
            for (int f = 0; f < nf; ++f) {
                bool ready = (f0 + f) < 9 || S.havePressure;
                if (!ready) continue;
                k_to_caller1<<<tsph_blocks(ng, 256), 256, 0, ctx->stream>>>(
                    ng, iord, src[f0 + f], strd[f0 + f], off[f0 + f], ctx->dStage, 3, f);
                TSPH_LAUNCH_CK("k_to_caller1");
            }
            if (ctx->hTmpN < (size_t)3 * ng) {
                free(ctx->hTmp);
                ctx->hTmp = (double *)malloc(sizeof(double) * 3 * ng);
                ctx->hTmpN = ctx->hTmp ? (size_t)3 * ng : 0;
                if (!ctx->hTmp) return TSPH_ERR_NOMEM;
            }
            double *tmp = ctx->hTmp;
            TSPH_CK(cudaMemcpyAsync(tmp, ctx->dStage, sizeof(double) * 3 * ng, cudaMemcpyDeviceToHost,
                                    ctx->stream));
            TSPH_CK(cudaStreamSynchronize(ctx->stream));
            for (int i = 0; i < ng; ++i)
                for (int f = 0; f < nf; ++f) out16[16 * i + f0 + f] = tmp[3 * i + f];
        }
    }
    double *arr[2] = {dtNew, mumax};
    const double *srcs[2] = {S.dtNew, S.mumax};
    for (int k = 0; k < 2; ++k) {
        if (!arr[k] || ng == 0) continue;
        if (!S.havePressure) {               // set by the pressure pass; zero before it
            memset(arr[k], 0, sizeof(double) * ng);
            continue;
        }
        k_to_caller1<<<tsph_blocks(ng, 256), 256, 0, ctx->stream>>>(ng, iord, srcs[k], 1, 0,
                                                                    ctx->dStage, 1, 0);
        TSPH_LAUNCH_CK("k_to_caller1");
        TSPH_CK(cudaMemcpyAsync(arr[k], ctx->dStage, sizeof(double) * ng, cudaMemcpyDeviceToHost,
                                ctx->stream));
        TSPH_CK(cudaStreamSynchronize(ctx->stream));
    }
    return TSPH_OK;
}

__global__ void k_hash_to_caller(int ng, const int *__restrict__ iord, const int *__restrict__ cnt,
                                 const unsigned long long *__restrict__ hsh, int *ocnt,
                                 unsigned long long *ohsh) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ng) return;
    ocnt[iord[i]] = cnt[i];
    ohsh[iord[i]] = hsh[i];
}

extern "C" int tsph_get_neighbour_hash(tsph_ctx *ctx, int *count, unsigned long long *hash) {
    if (!ctx || !count || !hash) return TSPH_ERR_ARG;
    if (!ctx->S.haveDensity) return TSPH_ERR_STATE;
    cudaSetDevice(ctx->device);
    const int ng = ctx->ngas;
    if (ng == 0) return TSPH_OK;
    int *dc = (int *)ctx->dStage;
    unsigned long long *dh = (unsigned long long *)(ctx->dStage + ng);
    k_hash_to_caller<<<tsph_blocks(ng, 256), 256, 0, ctx->stream>>>(ng, ctx->G.iord, ctx->S.nnCount,
                                                                   ctx->S.nnHash, dc, dh);
    TSPH_LAUNCH_CK("k_hash_to_caller");
    TSPH_CK(cudaMemcpyAsync(count, dc, sizeof(int) * ng, cudaMemcpyDeviceToHost, ctx->stream));
    TSPH_CK(cudaMemcpyAsync(hash, dh, sizeof(unsigned long long) * ng, cudaMemcpyDeviceToHost,
                            ctx->stream));
    TSPH_CK(cudaStreamSynchronize(ctx->stream));
    return TSPH_OK;
}

// ---------------------------------------------------------------------------
// kick and drift (pkdKick pkd.c:3780-3969, pkdDrift pkd.c:3686-3778)
// ---------------------------------------------------------------------------
// pkdKick (pkd.c:3780-3969) for a non-comoving canonical run with
// NOCOOLING (dvFacOne = dvPredFacOne = 1, dvFacTwo = duDelta = dt): the
// particles on rung iRung (every particle when iRung < 0).  The opening
// kick of a KDK step leaves vPred = v and uPred = u from before it
// (dvPredFacTwo = duPredDelta = 0, msrKickKDKOpen master.c:6540-6639); the
// closing kick predicts them to its end (msrKickKDKClose master.c:6644-6741).
// a is gravity plus, for gas, the hydrodynamic acceleration.
__global__ void k_kick_rung(int n, int ngas, int iRung, double dt, const double *dtp, int bClose,
                            TsphDevState C) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (dtp) dt *= *dtp;   // a captured step: dt is a fraction of the step in device memory
    if (iRung >= 0 && C.rung[i] != iRung) return;
    const bool gas = i < ngas;
    double a[3] = {C.ax[i], C.ay[i], C.az[i]};
    if (gas) { a[0] = xadd(a[0], C.hax[i]); a[1] = xadd(a[1], C.hay[i]); a[2] = xadd(a[2], C.haz[i]); }
    double *v[3] = {C.vx, C.vy, C.vz};
    double *vp[3] = {C.vpx, C.vpy, C.vpz};
    const double predFac = bClose ? dt : 0.0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {   // no contraction: the reference's rounding
        const double vk = v[k][i];
        if (gas) vp[k][i] = xadd(vk, xmul(a[k], predFac));
        v[k][i] = xadd(vk, xmul(a[k], dt));
    }
    if (gas) {
        const double u = C.u[i], udot = C.udot[i];
        C.upred[i] = xadd(u, xmul(udot, predFac));
        C.u[i] = xadd(u, xmul(udot, dt));
    }
}

// pkdDrift (pkd.c:3686-3778) and, for gas, pkdKickVpred (pkd.c:6489-6552)
// as msrDrift runs them (master.c:6306-6437): r += v dt with the periodic
// wrap, then vPred += a dt and uPred += uDot dt.
__global__ void k_drift(int n, int ngas, double dt, const double *dtp, int bPeriodic, double L,
                        TsphDevState C) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (dtp) dt *= *dtp;   // a captured step: dt is a fraction of the step in device memory
    double *r[3] = {C.x, C.y, C.z};
    const double *v[3] = {C.vx, C.vy, C.vz};
    // the wrap tests x >= L/2 and x < -L/2 on integer order keys (the FP64
    // pipe is left the arithmetic)
    const unsigned long long kHi = dlt_key(0.5 * L), kLo = dlt_key(-0.5 * L);
#pragma unroll
    for (int k = 0; k < 3; ++k) {   // no contraction: the reference's rounding
        double x = xadd(r[k][i], xmul(dt, v[k][i]));
        if (bPeriodic) {
            if (!(dlt_key(x) < kHi)) x = xsub(x, L);
            if (dlt_key(x) < kLo) x = xadd(x, L);
        }
        r[k][i] = x;
    }
    if (i < ngas && dt != 0.0) {
        // distance bound for passes over active rungs (|r| moved by |v| dt)
        const double vx = C.vx[i], vy = C.vy[i], vz = C.vz[i];
        C.disp[i] += sqrt(vx * vx + vy * vy + vz * vz) * fabs(dt) * (1.0 + 1e-12);
        C.vpx[i] = xadd(C.vpx[i], xmul(xadd(C.ax[i], C.hax[i]), dt));
        C.vpy[i] = xadd(C.vpy[i], xmul(xadd(C.ay[i], C.hay[i]), dt));
        C.vpz[i] = xadd(C.vpz[i], xmul(xadd(C.az[i], C.haz[i]), dt));
        C.upred[i] = xadd(C.upred[i], xmul(C.udot[i], dt));
    }
}

int tsph_kick_launch(tsph_ctx *ctx, int iRung, double dt, int bClose) {
    k_kick_rung<<<tsph_blocks(ctx->n, 256), 256, 0, ctx->stream>>>(ctx->n, ctx->ngas, iRung, dt,
                                                                     ctx->stepDtDev, bClose, ctx->C);
    TSPH_LAUNCH_CK("k_kick_rung");
    return TSPH_OK;
}

int tsph_drift_launch(tsph_ctx *ctx, double dt, int bPeriodic, double dPeriod) {
    k_drift<<<tsph_blocks(ctx->n, 256), 256, 0, ctx->stream>>>(ctx->n, ctx->ngas, dt, ctx->stepDtDev,
                                                                 bPeriodic, dPeriod, ctx->C);
    TSPH_LAUNCH_CK("k_drift");
    return TSPH_OK;
}

extern "C" int tsph_kick_rung(tsph_ctx *ctx, int iRung, double dt, int bClose) {
    if (!ctx) return TSPH_ERR_ARG;
    if (!ctx->haveParts || !ctx->haveVel) return TSPH_ERR_STATE;
    cudaSetDevice(ctx->device);
    if (ctx->n == 0) return TSPH_OK;
    int rc = tsph_kick_launch(ctx, iRung, dt, bClose);
    if (rc) return rc;
    if (!ctx->capturing) TSPH_CK(cudaStreamSynchronize(ctx->stream));
    return TSPH_OK;
}

extern "C" int tsph_kick(tsph_ctx *ctx, double dt) { return tsph_kick_rung(ctx, -1, dt, 1); }

extern "C" int tsph_drift(tsph_ctx *ctx, double dt, int bPeriodic, double dPeriod) {
    if (!ctx) return TSPH_ERR_ARG;
    if (!ctx->haveParts || !ctx->haveVel) return TSPH_ERR_STATE;
    if (bPeriodic && !(dPeriod > 0)) return TSPH_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->n == 0) return TSPH_OK;
    int rc = tsph_drift_launch(ctx, dt, bPeriodic, dPeriod);
    if (rc) return rc;
    if (!ctx->capturing) TSPH_CK(cudaStreamSynchronize(ctx->stream));
    ctx->S.haveDensity = ctx->S.havePressure = false;
    ctx->haveGrav = false;
    return TSPH_OK;
}

extern "C" int tsph_get_state(tsph_ctx *ctx, double *pos, double *vel, double *u) {
    if (!ctx) return TSPH_ERR_ARG;
    if (!ctx->haveParts) return TSPH_ERR_STATE;
    cudaSetDevice(ctx->device);
    int rc = tsph_copy_out(ctx, ctx->C.x, ctx->C.y, ctx->C.z, 3, pos);
    if (!rc) rc = tsph_copy_out(ctx, ctx->C.vx, ctx->C.vy, ctx->C.vz, 3, vel);
    if (!rc && u && ctx->ngas > 0) rc = tsph_copy_out_n(ctx, ctx->ngas, ctx->C.u, nullptr, nullptr, 1, u);
    return rc;
}
