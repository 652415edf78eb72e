// K3+K4: bucket walk fused with the particle-particle and particle-cell
// interactions.
//
// Semantics follow the reference's pkdGravAll bucket loop (pkd.c:2911-3001),
// pkdBucketWalk / pkdLocalWalk (walk.c:58-178, 306-439) and
// pkdBucketInteract (grav.c:23-249):
//   * a cell is opened when the bucket box lies within sqrt(fOpen2) of the
//     cell's centre of mass (INTERSECTNP, walk.h:12-31) or it holds fewer
//     than 4 particles (walk.c:81); an opened leaf contributes its particles
//     (P-P), except the bucket itself in the unshifted replica (walk.c:93);
//   * an accepted cell is "softened" when twoh2 = (cellSoft + maxSoft)^2 is
//     not below fOpen2 and the bucket box lies within twoh (walk.c:122-127),
//     otherwise Newtonian with the trace-free quadrupole (SETILIST);
//   * P-P uses spline softening with twoh = h_i + h_j (SPLINEM), softened
//     cells SPLINEQ, Newtonian cells QEVAL; intra-bucket pairs SPLINE.
//
// GB300 mapping: one warp per bucket.  The walk is a warp-cooperative
// depth-first traversal with an explicit stack in shared memory: each step
// pops up to 32 (cell, replica) entries, one per lane.  Opening tests run in
// FP32 on hi/lo split coordinates relative to the bucket centre with a
// rigorous rounding bound; only tests inside that bound are redone in FP64
// with the reference's own operation order, so every decision equals the
// reference's FP64 decision while FP64 work (1/64 rate on this part) stays
// rare.  Accepted interactions are staged in shared-memory tiles and
// evaluated with lanes = (bucket particle, entry slot), FP32 with tile
// partial sums merged by compensated (Kahan) addition, or FP64.
#include <float.h>
#include <math.h>

#include "tsph_ctx.cuh"

// NBT (template): largest bucket one warp handles, 8, 16 or 32; lanes are
// (bucket particle, entry slot) pairs with 32 / NBT slots per particle.
#define WPB 4                   // warps per block
#define STK 768                 // walk stack entries per warp (a batch-of-32 descent
                                // holds ~100 at most on clustered 4M-particle trees)
#define PPF 128                 // P-P tile size
#define CNF 64                  // cell tile size
#define CNB (CNF + 32)

#define ACT_NONE 0
#define ACT_OPEN 1
#define ACT_LEAF 2
#define ACT_NEWT 3
#define ACT_SOFT 4

struct WalkConst {
    int nRep;
    int selfRep;
    double off[27][3];
    float offh[27][3];
    float offl[27][3];
    float offmax;      // max |offset| component
    float E0;          // absolute error floor of the hi/lo relative coordinates
    double L;          // period (0 when not periodic)
    float Lh, Ll;      // its hi/lo FP32 split
};
__constant__ WalkConst cW;

// Replica offsets from the replica index r = (ix+1)*9 + (iy+1)*3 + (iz+1)
// (at most one replica each way): i*L, and its FP32 hi/lo parts i*Lh and
// i*Ll, exact for i in {-1, 0, 1}.  Computed instead of read from a
// constant table, whose reads would serialise on the warp's distinct
// replicas.
__device__ __forceinline__ void rep_idx(int r, float &ix, float &iy, float &iz) {
    ix = (float)(r / 9 - 1);
    iy = (float)((r / 3) % 3 - 1);
    iz = (float)(r % 3 - 1);
}
__device__ __forceinline__ void rep_off32(int r, float &hx, float &hy, float &hz, float &lx, float &ly,
                                          float &lz) {
    float ix, iy, iz;
    rep_idx(r, ix, iy, iz);
    hx = ix * cW.Lh; hy = iy * cW.Lh; hz = iz * cW.Lh;
    lx = ix * cW.Ll; ly = iy * cW.Ll; lz = iz * cW.Ll;
}
__device__ __forceinline__ void rep_off64(int r, double *o) {
    float ix, iy, iz;
    rep_idx(r, ix, iy, iz);
    o[0] = (double)ix * cW.L; o[1] = (double)iy * cW.L; o[2] = (double)iz * cW.L;
}

// Staged tile data.  FP64: P-P uses x,y,z,m,h and cells x,y,z,m,q0..q5,h,
// one array per field.  FP32: entries are stored in pairs (2p, 2p+1), each
// field of a pair side by side, so one 128-bit load gives two fields of
// both entries and every packed f32x2 instruction of the evaluation works
// on the two entries at once:  xy = (x0, x1, y0, y1), zm = (z0, z1, m0, m1),
// q01 = (xx0, xx1, yy0, yy1), q23 = (zz0, zz1, xy0, xy1),
// q45 = (xz0, xz1, yz0, yz1), h = (h0, h1).
// HIGH (octopole and hexadecapole cells, iOrder >= 3): cell tiles of 32,
// with the 25 reduced moments of every entry in oh[k][entry] (FP32: the
// octopole scaled by -15/2 and the hexadecapole by 35/2, the factors of
// the packed evaluation).
template <bool HIGH>
__host__ __device__ constexpr int cell_tile() { return HIGH ? 32 : CNF; }

template <typename Real, bool HIGH>
struct TileData {
    Real ex[PPF], ey[PPF], ez[PPF], em[PPF], eh[PPF];
    Real q[6][cell_tile<HIGH>()];
    Real oh[HIGH ? 25 : 1][HIGH ? cell_tile<HIGH>() : 1];
};
template <bool HIGH>
struct TileData<float, HIGH> {
    static constexpr int C = cell_tile<HIGH>();
    union {
        struct {
            float4 xy[PPF / 2], zm[PPF / 2];
            float2 h[PPF / 2];
        } pp;
        struct {
            float4 xy[C / 2], zm[C / 2], q01[C / 2], q23[C / 2], q45[C / 2];
            float2 h[C / 2];
            float oh[HIGH ? 25 : 1][HIGH ? C : 1];
        } cn;
    };
};

template <typename Real, int NBT, bool HIGH>
struct WalkSmem {
    int stack[STK];
    int pp[PPF + 32 * NBT + NBT];
    int cn[CNB];
    int cs[CNB];
    TileData<Real, HIGH> D;
    Real px[NBT], py[NBT], pz[NBT], pm[NBT], ph[NBT];
    // the warp's tallies of pkdGravAll's sums (lane 0 only)
    unsigned long long tAct, tPP, tNewt, tSoft, tBsq, tIntra;
    int gU, gNA;   // sizes of the lists the last group walk left
};

// The evaluation pass's per-warp shared memory: tiles and the bucket's
// particles only (no walk stack or list buffers).
template <typename Real, int NBT, bool HIGH>
struct EvalSmem {
    TileData<Real, HIGH> D;
    Real px[NBT], py[NBT], pz[NBT], pm[NBT], ph[NBT];
    unsigned long long tAct, tPP, tNewt, tSoft, tBsq, tIntra;
};

struct WalkArgs {
    TsphDevTree T;
    TsphDevParts P;
    TsphDevCounters *cnt;
    int *bucketLists;      // optional, 4 ints per bucket
    const int *nBuckets;   // device: the tree's leaf count
    int *workCounter;
    int iOrder;
    // walk groups (groupFirst null: one bucket per work unit)
    const int *groupFirst;   // first bucket of every group, then the bucket count
    const int *nGroups;      // device: number of groups
    int *groupScratch;       // GRP_SCRATCH ints per warp of the launch
    int groupMax;            // particles per group at most
    // two-pass walk (listInfo null: one fused pass): the list pass stores
    // bucket b's P-P particles at listPP + b * listCap (its own first),
    // Newtonian cells at listCell + b * listCap and softened cells at
    // listSoft + b * (listCap / 4), their numbers in listInfo[b] (w = -1: a
    // list did not fit; the evaluation pass walks the bucket itself)
    int *listPP, *listCell, *listSoft;
    int4 *listInfo;
    int listCap;
    // the buckets marked w = -1, walked by a fused launch after the
    // evaluation pass (their number in cnt->nListFallback); null otherwise
    int *fallback;
};

__device__ __forceinline__ unsigned lane_lt() {
    unsigned r;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(r));
    return r;
}

// INTERSECTNP (walk.h:12-31) in FP64 with the reference's rounding.
__device__ __forceinline__ bool intersect_exact(const double *bmin, const double *bmax,
                                                double fBall2, double x, double y, double z) {
    double dx = xsub(bmin[0], x), dx1 = xsub(x, bmax[0]);
    double dy = xsub(bmin[1], y), dy1 = xsub(y, bmax[1]);
    double dz = xsub(bmin[2], z), dz1 = xsub(z, bmax[2]);
    double d2;
    if (dx > 0.0) d2 = xmul(dx, dx);
    else if (dx1 > 0.0) d2 = xmul(dx1, dx1);
    else d2 = 0.0;
    if (dy > 0.0) d2 = xadd(d2, xmul(dy, dy));
    else if (dy1 > 0.0) d2 = xadd(d2, xmul(dy1, dy1));
    if (dz > 0.0) d2 = xadd(d2, xmul(dz, dz));
    else if (dz1 > 0.0) d2 = xadd(d2, xmul(dz1, dz1));
    return d2 <= fBall2;
}

// The reference's FP64 decisions for one (bucket, cell, replica), used only
// when the FP32 filter cannot settle them.  Returns 0 = not opened
// (Newtonian), 1 = opened, 2 = not opened (softened) when !openTestOnly.
// The bucket box is the bounds of its active particles (T.bact).
__device__ __noinline__ int exact_decision(const TsphDevTree &T, const TsphDevParts &P, int b,
                                           int lo, int n, int cell, const double *off,
                                           bool openTestOnly) {
    double bmn[3], bmx[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        bmn[k] = T.bact[6 * b + k];
        bmx[k] = T.bact[6 * b + 3 + k];
    }
    double x = xadd(T.r[3 * cell], off[0]);
    double y = xadd(T.r[3 * cell + 1], off[1]);
    double z = xadd(T.r[3 * cell + 2], off[2]);
    if (openTestOnly) return intersect_exact(bmn, bmx, T.fOpen2[cell], x, y, z) ? 1 : 0;
    double fSoftMax = 0.0;
    for (int p = lo; p < lo + n; ++p) fSoftMax = fmax(fSoftMax, P.h[p]);
    double twoh2 = xadd(T.fSoft[cell], fSoftMax);
    twoh2 = xmul(twoh2, twoh2);
    if (twoh2 < T.fOpen2[cell]) return 0;
    return intersect_exact(bmn, bmx, twoh2, x, y, z) ? 2 : 0;
}

// Three-way FP32 filter: +1 certainly D2 > F, -1 certainly D2 <= F, 0 unsure.
__device__ __forceinline__ int filt(float D2, float M, float F, float relF) {
    if (D2 - M > F * (1.0f + relF)) return 1;
    if (D2 + M < F * (1.0f - relF)) return -1;
    return 0;
}

__device__ __forceinline__ void kahan_add(float &s, float &c, float v) {
    float y = v - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
}
__device__ __forceinline__ void kahan_add(double &s, double &c, double v) { s += v; (void)c; }

// Error-free sum of two compensated pairs (used in the warp reduction).
__device__ __forceinline__ void two_sum_merge(float &s, float &c, float s2, float c2) {
    float t = s + s2;
    float bp = t - s;
    float err = (s - (t - bp)) + (s2 - bp);
    s = t;
    c = c + c2 - err;   // c holds the negated low part (Kahan convention)
}
__device__ __forceinline__ void two_sum_merge(double &s, double &c, double s2, double c2) {
    s += s2;
    c += c2;
}

template <typename Real>
__device__ __forceinline__ Real rsq(Real x);
template <>
__device__ __forceinline__ float rsq<float>(float x) { return rsqrtf(x); }
template <>
__device__ __forceinline__ double rsq<double>(double x) { return rsqrt(x); }

// SPLINEM (grav.h:53-72) given dir = 1/r.
template <typename Real>
__device__ __forceinline__ void spline_m(Real dir, Real r2, Real twoh, Real &a, Real &b) {
    if (r2 < twoh * twoh) {
        Real dih = Real(2.0) / twoh;
        Real u = dih / dir;
        if (u < Real(1.0)) {
            a = dih * (Real(7.0 / 5.0) - Real(2.0 / 3.0) * u * u + Real(3.0 / 10.0) * u * u * u * u -
                       Real(1.0 / 10.0) * u * u * u * u * u);
            b = dih * dih * dih * (Real(4.0 / 3.0) - Real(6.0 / 5.0) * u * u + Real(0.5) * u * u * u);
        } else {
            a = Real(-1.0 / 15.0) * dir +
                dih * (Real(8.0 / 5.0) - Real(4.0 / 3.0) * u * u + u * u * u -
                       Real(3.0 / 10.0) * u * u * u * u + Real(1.0 / 30.0) * u * u * u * u * u);
            b = Real(-1.0 / 15.0) * dir * dir * dir +
                dih * dih * dih * (Real(8.0 / 3.0) - Real(3.0) * u + Real(6.0 / 5.0) * u * u -
                                   Real(1.0 / 6.0) * u * u * u);
        }
    } else {
        a = dir;
        b = a * a * a;
    }
}

// SPLINEQ (grav.h:17-51) given dir = 1/r.
template <typename Real>
__device__ __forceinline__ void spline_q(Real dir, Real r2, Real twoh, Real &a, Real &b, Real &c,
                                         Real &d) {
    if (r2 < twoh * twoh) {
        Real dih = Real(2.0) / twoh;
        Real u = dih / dir;
        Real dih2 = dih * dih, dih3 = dih2 * dih, dih4 = dih2 * dih2, dih5 = dih4 * dih;
        if (u < Real(1.0)) {
            a = dih * (Real(7.0 / 5.0) - Real(2.0 / 3.0) * u * u + Real(3.0 / 10.0) * u * u * u * u -
                       Real(1.0 / 10.0) * u * u * u * u * u);
            b = dih3 * (Real(4.0 / 3.0) - Real(6.0 / 5.0) * u * u + Real(0.5) * u * u * u);
            c = dih5 * (Real(12.0 / 5.0) - Real(1.5) * u);
            d = Real(1.5) * dih5 * dih * dir;
        } else {
            Real dir2 = dir * dir, dir3 = dir2 * dir;
            a = Real(-1.0 / 15.0) * dir +
                dih * (Real(8.0 / 5.0) - Real(4.0 / 3.0) * u * u + u * u * u -
                       Real(3.0 / 10.0) * u * u * u * u + Real(1.0 / 30.0) * u * u * u * u * u);
            b = Real(-1.0 / 15.0) * dir3 +
                dih3 * (Real(8.0 / 3.0) - Real(3.0) * u + Real(6.0 / 5.0) * u * u -
                        Real(1.0 / 6.0) * u * u * u);
            c = Real(-1.0 / 5.0) * dir3 * dir2 + Real(3.0) * dih4 * dir +
                dih5 * (Real(-12.0 / 5.0) + Real(0.5) * u);
            d = -dir3 * dir3 * dir + Real(3.0) * dih4 * dir3 - Real(0.5) * dih5 * dih * dir;
        }
    } else {
        a = dir;
        b = a * a * a;
        c = Real(3.0) * b * a * a;
        d = Real(5.0) * c * a * a;
    }
}

template <typename Real>
struct Acc {
    Real s[4], c[4];     // ax, ay, az, pot (sum and compensation)
    Real t[4];           // current tile partial (FP64 path)
    Real dt;             // max (m_i + m_j) * b
};

// ---- packed FP32 pair arithmetic (sm_100 family f32x2: one instruction,
// two lanes' worth of FP32 work, each rounded as the scalar operation) ----
__device__ __forceinline__ float2 p_add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 p_mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 p_fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 p_sub(float2 a, float2 b) {
    unsigned long long r;
    asm("sub.rn.f32x2 %0, %1, %2;"
        : "=l"(r)
        : "l"(*reinterpret_cast<const unsigned long long *>(&a)),
          "l"(*reinterpret_cast<const unsigned long long *>(&b)));
    return *reinterpret_cast<const float2 *>(&r);
}
__device__ __forceinline__ float2 p_rsqrt(float2 a) { return make_float2(rsqrtf(a.x), rsqrtf(a.y)); }
__device__ __forceinline__ float2 p_splat(float a) { return make_float2(a, a); }

// The partner of an odd-length tile's last entry: far away and massless,
// so each of its terms is exactly zero (1/r^3 underflows, m = 0).
#define FAR_ENTRY 1.0e18f

// A packed tile partial folded into a compensated sum.
__device__ __forceinline__ void kahan_add2(float &s, float &c, float2 v) {
    kahan_add(s, c, v.x);
    kahan_add(s, c, v.y);
}

// Relative FP32 position of an entry (particle or cell COM, hi/lo split)
// in replica r about the bucket centre (hi/lo split).
__device__ __forceinline__ void rel_pos(float4 h, float4 l, int r, float bchx, float bchy, float bchz,
                                        float bclx, float bcly, float bclz, float &x, float &y,
                                        float &z) {
    float ohx, ohy, ohz, olx, oly, olz;
    rep_off32(r, ohx, ohy, ohz, olx, oly, olz);
    x = ((h.x - bchx) + ohx) + ((l.x - bclx) + olx);
    y = ((h.y - bchy) + ohy) + ((l.y - bcly) + oly);
    z = ((h.z - bchz) + ohz) + ((l.z - bclz) + olz);
}

// Stage P-P entries [0, cnt) of buf (the warp's buffer in shared memory, or
// a stored list) into shared memory.
template <typename Real, int NBT, bool HIGH, class Smem>
__device__ __forceinline__ void stage_pp(Smem &S, const TsphDevParts &P, const int *buf,
                                         int cnt, int lane, float bchx, float bchy, float bchz,
                                         float bclx, float bcly, float bclz) {
    if constexpr (sizeof(Real) == 4) {
        const int np = (cnt + 1) >> 1;
        for (int p = lane; p < np; p += 32) {
            float x[2], y[2], z[2], m[2], h[2];
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                const int e = 2 * p + k;
                if (e < cnt) {
                    const int ent = buf[e];
                    const int idx = ent >> 5, rep = ent & 31;
                    const float4 a = P.ph[idx], b = P.pl[idx];
                    rel_pos(a, b, rep == 31 ? cW.selfRep : rep, bchx, bchy, bchz, bclx, bcly, bclz,
                            x[k], y[k], z[k]);
                    m[k] = a.w;
                    h[k] = b.w;
                } else {
                    x[k] = y[k] = z[k] = FAR_ENTRY;
                    m[k] = h[k] = 0.0f;
                }
            }
            S.D.pp.xy[p] = make_float4(x[0], x[1], y[0], y[1]);
            S.D.pp.zm[p] = make_float4(z[0], z[1], m[0], m[1]);
            S.D.pp.h[p] = make_float2(h[0], h[1]);
        }
    } else {
        for (int e = lane; e < cnt; e += 32) {
            const int ent = buf[e];
            const int idx = ent >> 5, rep = ent & 31;
            const int r = rep == 31 ? cW.selfRep : rep;
            double o[3];
            rep_off64(r, o);
            S.D.ex[e] = (Real)(P.x[idx] + o[0]);
            S.D.ey[e] = (Real)(P.y[idx] + o[1]);
            S.D.ez[e] = (Real)(P.z[idx] + o[2]);
            S.D.em[e] = (Real)P.m[idx];
            S.D.eh[e] = (Real)P.h[idx];
        }
    }
}

// Evaluate staged P-P entries for this lane's particle i.  SELF: the tile
// holds the bucket's own particles (the first tile of every bucket, where
// the own particles are entries 0..n-1), so the particle's pair with itself
// is left out.
template <typename Real, int NBT, bool HIGH, bool SELF, class Smem>
__device__ __forceinline__ void eval_pp(Smem &S, int cnt, int i, int slot, Acc<Real> &A) {
    if constexpr (sizeof(Real) == 4) {
        const float2 X = p_splat(S.px[i]), Y = p_splat(S.py[i]), Z = p_splat(S.pz[i]);
        const float2 H = p_splat(S.ph[i]), M = p_splat(S.pm[i]);
        float2 tx = p_splat(0.0f), ty = tx, tz = tx, tp = tx;   // tp: minus the potential
        float dt = A.dt;
        const int np = (cnt + 1) >> 1;
#pragma unroll 1
        for (int p = slot; p < np; p += 32 / NBT) {
            const float4 a = S.D.pp.xy[p], b = S.D.pp.zm[p];
            const float2 he = S.D.pp.h[p];
            float2 ex = make_float2(a.x, a.y), ey = make_float2(a.z, a.w);
            float2 ez = make_float2(b.x, b.y), me = make_float2(b.z, b.w);
            if constexpr (SELF) {
                if (p == (i >> 1)) {   // entry i is the particle itself
                    if (i & 1) { ex.y = ey.y = ez.y = FAR_ENTRY; me.y = 0.0f; }
                    else { ex.x = ey.x = ez.x = FAR_ENTRY; me.x = 0.0f; }
                }
            }
            // entry minus particle: the reference's dx with the sign flipped
            const float2 dx = p_sub(ex, X), dy = p_sub(ey, Y), dz = p_sub(ez, Z);
            const float2 d2 = p_fma(dz, dz, p_fma(dy, dy, p_mul(dx, dx)));
            const float2 twoh = p_add(H, he);
            const float2 dir = p_rsqrt(d2);
            const float2 t2 = p_mul(twoh, twoh);
            float2 av, bv;
            if (d2.x < t2.x || d2.y < t2.y) {   // inside a softening length: SPLINEM
                spline_m<float>(dir.x, d2.x, twoh.x, av.x, bv.x);
                spline_m<float>(dir.y, d2.y, twoh.y, av.y, bv.y);
            } else {
                av = dir;
                bv = p_mul(p_mul(dir, dir), dir);
            }
            const float2 idt2 = p_mul(p_add(M, me), bv);
            dt = fmaxf(dt, fmaxf(idt2.x, idt2.y));
            tp = p_fma(av, me, tp);
            const float2 bm = p_mul(bv, me);
            tx = p_fma(dx, bm, tx);
            ty = p_fma(dy, bm, ty);
            tz = p_fma(dz, bm, tz);
        }
        A.dt = dt;
        kahan_add2(A.s[0], A.c[0], tx);
        kahan_add2(A.s[1], A.c[1], ty);
        kahan_add2(A.s[2], A.c[2], tz);
        kahan_add2(A.s[3], A.c[3], make_float2(-tp.x, -tp.y));
    } else {
        const Real xi = S.px[i], yi = S.py[i], zi = S.pz[i], hi = S.ph[i], mi = S.pm[i];
        for (int e = slot; e < cnt; e += 32 / NBT) {
            if constexpr (SELF) {
                if (e == i) continue;   // self
            }
            const Real ex = S.D.ex[e], ey = S.D.ey[e], ez = S.D.ez[e], me = S.D.em[e], he = S.D.eh[e];
            Real dx = xi - ex, dy = yi - ey, dz = zi - ez;
            Real d2 = dx * dx + dy * dy + dz * dz;
            Real twoh = hi + he;
            Real dir = rsq<Real>(d2);
            Real a, b;
            spline_m<Real>(dir, d2, twoh, a, b);
            Real idt2 = (mi + me) * b;
            A.dt = idt2 > A.dt ? idt2 : A.dt;
            a *= me;
            b *= me;
            A.t[3] -= a;
            A.t[0] -= dx * b;
            A.t[1] -= dy * b;
            A.t[2] -= dz * b;
        }
    }
}

// One cell entry's FP32 record: relative COM, mass, quadrupole (trace
// removed for Newtonian cells, SETILIST walk.c:41-48) and softening.
__device__ __forceinline__ void cell_record(const TsphDevTree &T, int ent, bool soft, float bchx,
                                            float bchy, float bchz, float bclx, float bcly, float bclz,
                                            float *f) {
    const int c = ent >> 5, r = ent & 31;
    const float4 h4 = T.wcomh[c], l4 = T.wcoml[c];
    const float4 m0 = T.wmom0[c], m1 = T.wmom1[c];
    rel_pos(h4, l4, r, bchx, bchy, bchz, bclx, bcly, bclz, f[0], f[1], f[2]);
    f[3] = m0.x;
    float q[6] = {m0.y, m0.z, m0.w, m1.x, m1.y, m1.z};
    if (!soft) {
        const float tr = q[0] + q[1] + q[2];
        q[0] -= tr / 3.0f;
        q[1] -= tr / 3.0f;
        q[2] -= tr / 3.0f;
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) f[4 + k] = q[k];
    f[10] = m1.w;
}

// Stage cell entries (Newtonian when soft == 0, else softened).
template <typename Real, int NBT, bool HIGH, class Smem>
__device__ __forceinline__ void stage_cells(Smem &S, const int *buf, const TsphDevTree &T,
                                            int cnt, int lane, bool soft, float bchx, float bchy,
                                            float bchz, float bclx, float bcly, float bclz) {
    if constexpr (sizeof(Real) == 4) {
        const int np = (cnt + 1) >> 1;
        for (int p = lane; p < np; p += 32) {
            float f0[11], f1[11];
            cell_record(T, buf[2 * p], soft, bchx, bchy, bchz, bclx, bcly, bclz, f0);
            if (2 * p + 1 < cnt) {
                cell_record(T, buf[2 * p + 1], soft, bchx, bchy, bchz, bclx, bcly, bclz, f1);
            } else {
#pragma unroll
                for (int k = 0; k < 11; ++k) f1[k] = k < 3 ? FAR_ENTRY : 0.0f;
            }
            S.D.cn.xy[p] = make_float4(f0[0], f1[0], f0[1], f1[1]);
            S.D.cn.zm[p] = make_float4(f0[2], f1[2], f0[3], f1[3]);
            S.D.cn.q01[p] = make_float4(f0[4], f1[4], f0[5], f1[5]);
            S.D.cn.q23[p] = make_float4(f0[6], f1[6], f0[7], f1[7]);
            S.D.cn.q45[p] = make_float4(f0[8], f1[8], f0[9], f1[9]);
            S.D.cn.h[p] = make_float2(f0[10], f1[10]);
            if constexpr (HIGH) {
                if (!soft) {   // reduced octopole (x -15/2) and hexadecapole (x 35/2) of both entries
                    const float *o0 = T.wOH + 25 * (size_t)(buf[2 * p] >> 5);
                    const bool two = 2 * p + 1 < cnt;
                    const float *o1 = T.wOH + 25 * (size_t)(two ? buf[2 * p + 1] >> 5 : 0);
#pragma unroll
                    for (int k = 0; k < 25; ++k) {
                        const float sc = k < 10 ? -7.5f : 17.5f;
                        S.D.cn.oh[k][2 * p] = sc * o0[k];
                        S.D.cn.oh[k][2 * p + 1] = two ? sc * o1[k] : 0.0f;
                    }
                }
            }
        }
    } else {
        for (int e = lane; e < cnt; e += 32) {
            const int ent = buf[e];
            const int c = ent >> 5, r = ent & 31;
            double o[3];
            rep_off64(r, o);
            Real q[6];
#pragma unroll
            for (int k = 0; k < 6; ++k) q[k] = (Real)T.Q[6 * c + k];
            if (!soft) {   // reduced (trace-free) quadrupole, SETILIST walk.c:41-48
                Real tr = q[0] + q[1] + q[2];
                q[0] -= tr / Real(3.0);
                q[1] -= tr / Real(3.0);
                q[2] -= tr / Real(3.0);
            }
            S.D.ex[e] = (Real)(T.r[3 * c] + o[0]);
            S.D.ey[e] = (Real)(T.r[3 * c + 1] + o[1]);
            S.D.ez[e] = (Real)(T.r[3 * c + 2] + o[2]);
            S.D.em[e] = (Real)T.fMass[c];
            S.D.eh[e] = (Real)T.fSoft[c];
#pragma unroll
            for (int k = 0; k < 6; ++k) S.D.q[k][e] = q[k];
            if constexpr (HIGH) {
                if (!soft)
#pragma unroll
                    for (int k = 0; k < 25; ++k) S.D.oh[k][e] = (Real)T.OH[25 * (size_t)c + k];
            }
        }
    }
}

// QEVAL (qeval.h:21-64) at orders 1 to 4 for one cell: reduced moments m,
// q (xx yy zz xy xz yz), o (pkdCalcCell's O*: xxx xyy xxy yyy xxz yyz xyz
// xzz yzz zzz), h (H*: xxxx xyyy xxxy yyyy xxxz yyyz xxyy xxyz xyyz xxzz
// xyzz xzzz yyzz yzzz zzzz); (dx, dy, dz) = particle - cell, gam[0..5] the
// reference's gamma series; accumulates into a and pot like the macro.
template <typename Real>
__device__ __forceinline__ void qeval_cell(int iOrder, Real m, const Real *q, const Real *o, const Real *h,
                                           const Real *gam, Real dx, Real dy, Real dz, Real &ax, Real &ay,
                                           Real &az, Real &pot) {
    Real Qmirx, Qmiry, Qmirz, Qmir, Qta = 0;
    if (iOrder >= 4) {
        Qmirx = Real(1.0 / 6.0) * (h[11] * dz * dz * dz + 3 * h[10] * dy * dz * dz + 3 * h[8] * dy * dy * dz +
                                    h[1] * dy * dy * dy + 3 * h[9] * dx * dz * dz + 6 * h[7] * dx * dy * dz +
                                    3 * h[6] * dx * dy * dy + 3 * h[4] * dx * dx * dz + 3 * h[2] * dx * dx * dy +
                                    h[0] * dx * dx * dx);
        Qmiry = Real(1.0 / 6.0) * (h[13] * dz * dz * dz + 3 * h[10] * dx * dz * dz + 3 * h[7] * dx * dx * dz +
                                    h[2] * dx * dx * dx + 3 * h[12] * dy * dz * dz + 6 * h[8] * dx * dy * dz +
                                    3 * h[6] * dx * dx * dy + 3 * h[5] * dy * dy * dz + 3 * h[1] * dx * dy * dy +
                                    h[3] * dy * dy * dy);
        Qmirz = Real(1.0 / 6.0) * (h[5] * dy * dy * dy + 3 * h[8] * dx * dy * dy + 3 * h[7] * dx * dx * dy +
                                    h[4] * dx * dx * dx + 3 * h[12] * dy * dy * dz + 6 * h[10] * dx * dy * dz +
                                    3 * h[9] * dx * dx * dz + 3 * h[13] * dy * dz * dz + 3 * h[11] * dx * dz * dz +
                                    h[14] * dz * dz * dz);
        Qmir = Real(1.0 / 4.0) * (Qmirx * dx + Qmiry * dy + Qmirz * dz);
        pot -= gam[4] * Qmir;
        Qta += gam[5] * Qmir;
        ax += gam[4] * Qmirx;
        ay += gam[4] * Qmiry;
        az += gam[4] * Qmirz;
    }
    if (iOrder >= 3) {
        Qmirx = Real(1.0 / 2.0) * (o[7] * dz * dz + 2 * o[6] * dy * dz + o[1] * dy * dy + 2 * o[4] * dx * dz +
                                    2 * o[2] * dx * dy + o[0] * dx * dx);
        Qmiry = Real(1.0 / 2.0) * (o[8] * dz * dz + 2 * o[6] * dx * dz + o[2] * dx * dx + 2 * o[5] * dy * dz +
                                    2 * o[1] * dx * dy + o[3] * dy * dy);
        Qmirz = Real(1.0 / 2.0) * (o[5] * dy * dy + 2 * o[6] * dx * dy + o[4] * dx * dx + 2 * o[8] * dy * dz +
                                    2 * o[7] * dx * dz + o[9] * dz * dz);
        Qmir = Real(1.0 / 3.0) * (Qmirx * dx + Qmiry * dy + Qmirz * dz);
        pot -= gam[3] * Qmir;
        Qta += gam[4] * Qmir;
        ax += gam[3] * Qmirx;
        ay += gam[3] * Qmiry;
        az += gam[3] * Qmirz;
    }
    if (iOrder >= 2) {
        Qmirx = q[4] * dz + q[3] * dy + q[0] * dx;
        Qmiry = q[5] * dz + q[3] * dx + q[1] * dy;
        Qmirz = q[5] * dy + q[4] * dx + q[2] * dz;
        Qmir = Real(0.5) * (Qmirx * dx + Qmiry * dy + Qmirz * dz);
        pot -= gam[2] * Qmir;
        Qta += gam[3] * Qmir;
        ax += gam[2] * Qmirx;
        ay += gam[2] * Qmiry;
        az += gam[2] * Qmirz;
    }
    pot -= gam[0] * m;
    Qta += gam[1] * m;
    ax -= dx * Qta;
    ay -= dy * Qta;
    az -= dz * Qta;
}

// FP64 Newtonian cells of a HIGH tile (iOrder >= 3), one cell per lane
// step, by QEVAL in the reference's form.
template <typename Real, int NBT, bool HIGH, class Smem>
__device__ __forceinline__ void eval_newt_high(Smem &S, int cnt, int i, int slot,
                                               int iOrder, Acc<Real> &A) {
    const Real xi = S.px[i], yi = S.py[i], zi = S.pz[i], mi = S.pm[i];
    for (int e = slot; e < cnt; e += 32 / NBT) {
        Real q[6], o[10], h[15];
        const Real cx = S.D.ex[e], cy = S.D.ey[e], cz = S.D.ez[e], m = S.D.em[e];
#pragma unroll
        for (int k = 0; k < 6; ++k) q[k] = S.D.q[k][e];
#pragma unroll
        for (int k = 0; k < 10; ++k) o[k] = S.D.oh[k][e];
#pragma unroll
        for (int k = 0; k < 15; ++k) h[k] = S.D.oh[10 + k][e];
        const Real dx = xi - cx, dy = yi - cy, dz = zi - cz;
        const Real d2 = dx * dx + dy * dy + dz * dz;
        Real gam[6];
        gam[0] = rsq<Real>(d2);
        const Real dir2 = gam[0] * gam[0];
        gam[1] = gam[0] * dir2;
        gam[2] = Real(3) * gam[1] * dir2;
        gam[3] = Real(5) * gam[2] * dir2;
        gam[4] = Real(7) * gam[3] * dir2;
        gam[5] = Real(9) * gam[4] * dir2;
        Real ax = 0, ay = 0, az = 0, pot = 0;
        qeval_cell<Real>(iOrder, m, q, o, h, gam, dx, dy, dz, ax, ay, az, pot);
        kahan_add(A.s[0], A.c[0], ax);
        kahan_add(A.s[1], A.c[1], ay);
        kahan_add(A.s[2], A.c[2], az);
        A.t[3] += pot;
        const Real idt2 = (mi + m) * gam[1];
        A.dt = idt2 > A.dt ? idt2 : A.dt;
    }
}

// FP32 Newtonian cells of a HIGH tile for particle i, two cells per packed
// instruction: QEVAL (qeval.h:21-64) at order 3, or with HEX at order 4,
// restated on the unit vector n = d / r (d = cell - particle, the
// reference's dx with the sign flipped; ir = 1/r), so that no power of r
// is formed unscaled:
//   W2 = 3 Q.n,  W3 = -15/2 O:nn,  W4 = 35/2 H:nnn,  p_k = W_k . n,
//   E  = (W2 - 5/2 p2 n) + ir ((W3 - 7/3 p3 n) + ir (W4 - 9/4 p4 n)),
//   a += m ir^2 n - ir^4 E,
//   -pot = m ir + ir^3 (p2 / 2 + ir (p3 / 3 + ir p4 / 4)),
// which is the reference's gamma series (g_k = (2k-1)!! / r^(2k+1)) with
// its Qmir vectors and scalars regrouped by powers of 1/r.  The factors
// -15/2 and 35/2 are applied to O and H when the tile is staged; the
// monomials carry the multiplicities of the symmetric contractions (2 for
// xy, 3 for xxy, 6 for xyz).  The odd tile's massless partner (FAR_ENTRY,
// zero moments) adds exactly zero: its n is finite and ir^3 underflows.
template <int NBT, bool HEX, class Smem>
__device__ __forceinline__ void newt_tile_f32_high(Smem &S, int cnt, int i, int slot, Acc<float> &A) {
    const float2 X = p_splat(S.px[i]), Y = p_splat(S.py[i]), Z = p_splat(S.pz[i]);
    const float2 M = p_splat(S.pm[i]);
    const float2 c3 = p_splat(3.0f), cm52 = p_splat(-2.5f), cm73 = p_splat(-7.0f / 3.0f);
    const float2 cm94 = p_splat(-2.25f), ch = p_splat(0.5f), c13 = p_splat(1.0f / 3.0f);
    const float2 c14 = p_splat(0.25f);
    float2 tx = p_splat(0.0f), ty = tx, tz = tx;   // monopole: m ir^2 n
    float2 ux = tx, uy = tx, uz = tx;              // ir^4 E
    float2 tp = tx;                                // minus the potential
    float dt = A.dt;
    constexpr int RS = cell_tile<true>() / 2;      // float2 pairs per moment row
    const float2 *oh = reinterpret_cast<const float2 *>(&S.D.cn.oh[0][0]);
    const int np = (cnt + 1) >> 1;
#pragma unroll 1
    for (int p = slot; p < np; p += 32 / NBT) {
        const float4 a = S.D.cn.xy[p], b = S.D.cn.zm[p];
        const float2 dx = p_sub(make_float2(a.x, a.y), X);
        const float2 dy = p_sub(make_float2(a.z, a.w), Y);
        const float2 dz = p_sub(make_float2(b.x, b.y), Z);
        const float2 m = make_float2(b.z, b.w);
        const float2 d2 = p_fma(dz, dz, p_fma(dy, dy, p_mul(dx, dx)));
        const float2 ir = p_rsqrt(d2);
        const float2 ir2 = p_mul(ir, ir);
        const float2 nx = p_mul(dx, ir), ny = p_mul(dy, ir), nz = p_mul(dz, ir);
        const float2 n3x = p_mul(c3, nx), n3y = p_mul(c3, ny), n3z = p_mul(c3, nz);
        // W2 = 3 Q.n (Q: xx yy zz xy xz yz)
        const float4 q01 = S.D.cn.q01[p], q23 = S.D.cn.q23[p], q45 = S.D.cn.q45[p];
        const float2 qxx = make_float2(q01.x, q01.y), qyy = make_float2(q01.z, q01.w);
        const float2 qzz = make_float2(q23.x, q23.y), qxy = make_float2(q23.z, q23.w);
        const float2 qxz = make_float2(q45.x, q45.y), qyz = make_float2(q45.z, q45.w);
        const float2 w2x = p_fma(qxx, n3x, p_fma(qxy, n3y, p_mul(qxz, n3z)));
        const float2 w2y = p_fma(qyy, n3y, p_fma(qxy, n3x, p_mul(qyz, n3z)));
        const float2 w2z = p_fma(qzz, n3z, p_fma(qxz, n3x, p_mul(qyz, n3y)));
        const float2 p2 = p_fma(w2z, nz, p_fma(w2y, ny, p_mul(w2x, nx)));
        // W3 = -15/2 O:nn (O: xxx xyy xxy yyy xxz yyz xyz xzz yzz zzz)
        const float2 xx = p_mul(nx, nx), yy = p_mul(ny, ny), zz = p_mul(nz, nz);
        const float2 n2x = p_add(nx, nx), n2y = p_add(ny, ny);
        const float2 xy2 = p_mul(n2x, ny), xz2 = p_mul(n2x, nz), yz2 = p_mul(n2y, nz);
#define OHR(k) oh[(k) * RS + p]
        const float2 w3x = p_fma(OHR(0), xx, p_fma(OHR(2), xy2, p_fma(OHR(4), xz2,
                           p_fma(OHR(1), yy, p_fma(OHR(6), yz2, p_mul(OHR(7), zz))))));
        const float2 w3y = p_fma(OHR(2), xx, p_fma(OHR(1), xy2, p_fma(OHR(6), xz2,
                           p_fma(OHR(3), yy, p_fma(OHR(5), yz2, p_mul(OHR(8), zz))))));
        const float2 w3z = p_fma(OHR(4), xx, p_fma(OHR(6), xy2, p_fma(OHR(7), xz2,
                           p_fma(OHR(5), yy, p_fma(OHR(8), yz2, p_mul(OHR(9), zz))))));
        const float2 p3 = p_fma(w3z, nz, p_fma(w3y, ny, p_mul(w3x, nx)));
        const float2 c3p = p_mul(cm73, p3);
        float2 fx = p_fma(c3p, nx, w3x), fy = p_fma(c3p, ny, w3y), fz = p_fma(c3p, nz, w3z);
        float2 pin = p_mul(c13, p3);
        if constexpr (HEX) {
            // W4 = 35/2 H:nnn (H: xxxx xyyy xxxy yyyy xxxz yyyz xxyy xxyz xyyz
            // xxzz xyzz xzzz yyzz yzzz zzzz, rows 10..24)
            const float2 mxxx = p_mul(xx, nx), myyy = p_mul(yy, ny), mzzz = p_mul(zz, nz);
            const float2 mxxy = p_mul(xx, n3y), mxxz = p_mul(xx, n3z), mxyy = p_mul(yy, n3x);
            const float2 myyz = p_mul(yy, n3z), mxzz = p_mul(zz, n3x), myzz = p_mul(zz, n3y);
            const float2 mxyz = p_mul(xy2, n3z);
#define HR(k) OHR(10 + (k))
            const float2 w4x = p_fma(HR(0), mxxx, p_fma(HR(2), mxxy, p_fma(HR(4), mxxz, p_fma(HR(6), mxyy,
                               p_fma(HR(7), mxyz, p_fma(HR(9), mxzz, p_fma(HR(1), myyy, p_fma(HR(8), myyz,
                               p_fma(HR(10), myzz, p_mul(HR(11), mzzz))))))))));
            const float2 w4y = p_fma(HR(2), mxxx, p_fma(HR(6), mxxy, p_fma(HR(7), mxxz, p_fma(HR(1), mxyy,
                               p_fma(HR(8), mxyz, p_fma(HR(10), mxzz, p_fma(HR(3), myyy, p_fma(HR(5), myyz,
                               p_fma(HR(12), myzz, p_mul(HR(13), mzzz))))))))));
            const float2 w4z = p_fma(HR(4), mxxx, p_fma(HR(7), mxxy, p_fma(HR(9), mxxz, p_fma(HR(8), mxyy,
                               p_fma(HR(10), mxyz, p_fma(HR(11), mxzz, p_fma(HR(5), myyy, p_fma(HR(12), myyz,
                               p_fma(HR(13), myzz, p_mul(HR(14), mzzz))))))))));
#undef HR
            const float2 p4 = p_fma(w4z, nz, p_fma(w4y, ny, p_mul(w4x, nx)));
            const float2 c4p = p_mul(cm94, p4);
            fx = p_fma(ir, p_fma(c4p, nx, w4x), fx);
            fy = p_fma(ir, p_fma(c4p, ny, w4y), fy);
            fz = p_fma(ir, p_fma(c4p, nz, w4z), fz);
            pin = p_fma(p_mul(c14, ir), p4, pin);
        }
#undef OHR
        const float2 c2p = p_mul(cm52, p2);
        const float2 ex = p_fma(ir, fx, p_fma(c2p, nx, w2x));
        const float2 ey = p_fma(ir, fy, p_fma(c2p, ny, w2y));
        const float2 ez = p_fma(ir, fz, p_fma(c2p, nz, w2z));
        const float2 ir4 = p_mul(ir2, ir2);
        ux = p_fma(ir4, ex, ux);
        uy = p_fma(ir4, ey, uy);
        uz = p_fma(ir4, ez, uz);
        const float2 mir2 = p_mul(m, ir2);
        tx = p_fma(mir2, nx, tx);
        ty = p_fma(mir2, ny, ty);
        tz = p_fma(mir2, nz, tz);
        const float2 ir3 = p_mul(ir2, ir);
        tp = p_fma(ir3, p_fma(ir, pin, p_mul(ch, p2)), p_fma(m, ir, tp));
        const float2 idt2 = p_mul(p_add(M, m), ir3);
        dt = fmaxf(dt, fmaxf(idt2.x, idt2.y));
    }
    A.dt = dt;
    kahan_add2(A.s[0], A.c[0], p_sub(tx, ux));
    kahan_add2(A.s[1], A.c[1], p_sub(ty, uy));
    kahan_add2(A.s[2], A.c[2], p_sub(tz, uz));
    kahan_add2(A.s[3], A.c[3], make_float2(-tp.x, -tp.y));
}

// FP32 Newtonian cell tile for particle i, two cells per packed
// instruction: monopole, and with QUAD the trace-free quadrupole.  With
// s = 1/r^5 and u = d.Q.d (d = cell - particle), QEVAL's quadrupole terms
// (qeval.h:53-64) are pot -= 1.5 s u, a += 3 s Q.d - 7.5 s u d / r^2 (the
// reference's g2 = 3 s, g3 = 15 s / r^2 and Qmir = u / 2 folded together).
template <int NBT, bool QUAD, class Smem>
__device__ __forceinline__ void newt_tile_f32(Smem &S, int cnt, int i, int slot, Acc<float> &A) {
    const float2 X = p_splat(S.px[i]), Y = p_splat(S.py[i]), Z = p_splat(S.pz[i]);
    const float2 M = p_splat(S.pm[i]);
    const float2 c15 = p_splat(1.5f), c75 = p_splat(7.5f), cm3 = p_splat(-3.0f);
    float2 tx = p_splat(0.0f), ty = tx, tz = tx, tp = tx;   // tp: minus the potential
    float dt = A.dt;
    const int np = (cnt + 1) >> 1;
#pragma unroll 1
    for (int p = slot; p < np; p += 32 / NBT) {
        const float4 a = S.D.cn.xy[p], b = S.D.cn.zm[p];
        // entry minus particle: the reference's dx with the sign flipped
        const float2 dx = p_sub(make_float2(a.x, a.y), X);
        const float2 dy = p_sub(make_float2(a.z, a.w), Y);
        const float2 dz = p_sub(make_float2(b.x, b.y), Z);
        const float2 m = make_float2(b.z, b.w);
        const float2 d2 = p_fma(dz, dz, p_fma(dy, dy, p_mul(dx, dx)));
        const float2 g0 = p_rsqrt(d2);
        const float2 dir2 = p_mul(g0, g0);
        const float2 g1 = p_mul(g0, dir2);
        float2 Qta = p_mul(g1, m);
        tp = p_fma(g0, m, tp);
        if constexpr (QUAD) {
            const float4 q01 = S.D.cn.q01[p], q23 = S.D.cn.q23[p], q45 = S.D.cn.q45[p];
            const float2 xx = make_float2(q01.x, q01.y), yy = make_float2(q01.z, q01.w);
            const float2 zz = make_float2(q23.x, q23.y), xy = make_float2(q23.z, q23.w);
            const float2 xz = make_float2(q45.x, q45.y), yz = make_float2(q45.z, q45.w);
            // Q.d with the flipped dx: minus the reference's Qmir vector
            const float2 qx = p_fma(xx, dx, p_fma(xy, dy, p_mul(xz, dz)));
            const float2 qy = p_fma(yy, dy, p_fma(xy, dx, p_mul(yz, dz)));
            const float2 qz = p_fma(zz, dz, p_fma(xz, dx, p_mul(yz, dy)));
            const float2 u = p_fma(qz, dz, p_fma(qy, dy, p_mul(qx, dx)));
            const float2 s5 = p_mul(g1, dir2);
            const float2 w = p_mul(s5, u);
            tp = p_fma(c15, w, tp);
            Qta = p_fma(c75, p_mul(w, dir2), Qta);
            const float2 ns3 = p_mul(cm3, s5);
            tx = p_fma(ns3, qx, tx);
            ty = p_fma(ns3, qy, ty);
            tz = p_fma(ns3, qz, tz);
        }
        tx = p_fma(dx, Qta, tx);
        ty = p_fma(dy, Qta, ty);
        tz = p_fma(dz, Qta, tz);
        const float2 idt2 = p_mul(p_add(M, m), g1);
        dt = fmaxf(dt, fmaxf(idt2.x, idt2.y));
    }
    A.dt = dt;
    kahan_add2(A.s[0], A.c[0], tx);
    kahan_add2(A.s[1], A.c[1], ty);
    kahan_add2(A.s[2], A.c[2], tz);
    kahan_add2(A.s[3], A.c[3], make_float2(-tp.x, -tp.y));
}

// Newtonian cells, QEVAL (qeval.h:21-64), for the particle i:
// acceleration, potential, and (m_i + m) / r^3 for the timestep.  FP32
// evaluates two cells per packed instruction into tile partials that are
// folded into the compensated sums once per tile, at every order.
template <typename Real, int NBT, bool HIGH, class Smem>
__device__ __forceinline__ void eval_newt(Smem &S, int cnt, int i, int slot, int iOrder,
                                          Acc<Real> &A) {
    if constexpr (HIGH && sizeof(Real) == 4) {
        if (iOrder >= 4) newt_tile_f32_high<NBT, true>(S, cnt, i, slot, A);
        else newt_tile_f32_high<NBT, false>(S, cnt, i, slot, A);
    } else if constexpr (HIGH) {
        eval_newt_high<Real, NBT, HIGH>(S, cnt, i, slot, iOrder, A);
    } else if constexpr (sizeof(Real) == 4) {
        if (iOrder >= 2) newt_tile_f32<NBT, true>(S, cnt, i, slot, A);
        else newt_tile_f32<NBT, false>(S, cnt, i, slot, A);
    } else {
        const Real xi = S.px[i], yi = S.py[i], zi = S.pz[i], mi = S.pm[i];
        for (int e = slot; e < cnt; e += 32 / NBT) {
            const Real cx = S.D.ex[e], cy = S.D.ey[e], cz = S.D.ez[e], m = S.D.em[e];
            const Real xx = S.D.q[0][e], yy = S.D.q[1][e], zz = S.D.q[2][e];
            const Real xy = S.D.q[3][e], xz = S.D.q[4][e], yz = S.D.q[5][e];
            Real dx = xi - cx, dy = yi - cy, dz = zi - cz;
            Real d2 = dx * dx + dy * dy + dz * dz;
            Real g0 = rsq<Real>(d2);
            Real dir2 = g0 * g0;
            Real g1 = g0 * dir2;
            Real g2 = Real(3) * g1 * dir2;
            Real g3 = Real(5) * g2 * dir2;
            Real Qta = 0, pot = 0, ax = 0, ay = 0, az = 0;
            if (iOrder >= 2) {
                Real Qmirx = xz * dz + xy * dy + xx * dx;
                Real Qmiry = yz * dz + xy * dx + yy * dy;
                Real Qmirz = yz * dy + xz * dx + zz * dz;
                Real Qmir = Real(0.5) * (Qmirx * dx + Qmiry * dy + Qmirz * dz);
                pot -= g2 * Qmir;
                Qta += g3 * Qmir;
                ax += g2 * Qmirx;
                ay += g2 * Qmiry;
                az += g2 * Qmirz;
            }
            pot -= g0 * m;
            Qta += g1 * m;
            ax -= dx * Qta;
            ay -= dy * Qta;
            az -= dz * Qta;
            A.s[0] += ax;
            A.s[1] += ay;
            A.s[2] += az;
            A.t[3] += pot;
            const Real idt2 = (mi + m) * g1;
            A.dt = idt2 > A.dt ? idt2 : A.dt;
        }
    }
}

// Softened cells with the full quadrupole (grav.c:126-150): one term of
// the particle at (xi, yi, zi) from cell (c, m, q, hc).
template <typename Real>
__device__ __forceinline__ void soft_term(Real xi, Real yi, Real zi, Real hi, Real mi, Real cx, Real cy,
                                          Real cz, Real m, Real xx, Real yy, Real zz, Real xy, Real xz,
                                          Real yz, Real hc, Real &ax, Real &ay, Real &az, Real &pot,
                                          Real &idt2) {
    Real dx = xi - cx, dy = yi - cy, dz = zi - cz;
    Real d2 = dx * dx + dy * dy + dz * dz;
    Real twoh = hi + hc;
    Real dir = rsq<Real>(d2);
    Real a, b, c, d;
    spline_q<Real>(dir, d2, twoh, a, b, c, d);
    Real qirx = xx * dx + xy * dy + xz * dz;
    Real qiry = xy * dx + yy * dy + yz * dz;
    Real qirz = xz * dx + yz * dy + zz * dz;
    Real qir = Real(0.5) * (qirx * dx + qiry * dy + qirz * dz);
    Real tr = Real(0.5) * (xx + yy + zz);
    Real qir3 = b * m + d * qir - c * tr;
    pot = -(a * m + c * qir - b * tr);
    ax = -(qir3 * dx - c * qirx);
    ay = -(qir3 * dy - c * qiry);
    az = -(qir3 * dz - c * qirz);
    idt2 = (mi + m) * b;
}

template <typename Real, int NBT, bool HIGH, class Smem>
__device__ __forceinline__ void eval_soft(Smem &S, int cnt, int i, int slot, Acc<Real> &A) {
    const Real xi = S.px[i], yi = S.py[i], zi = S.pz[i], hi = S.ph[i], mi = S.pm[i];
    if constexpr (sizeof(Real) == 4) {
        const int np = (cnt + 1) >> 1;
        for (int p = slot; p < np; p += 32 / NBT) {
            const float4 a = S.D.cn.xy[p], b = S.D.cn.zm[p];
            const float4 q01 = S.D.cn.q01[p], q23 = S.D.cn.q23[p], q45 = S.D.cn.q45[p];
            const float2 h = S.D.cn.h[p];
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                float ax, ay, az, pot, idt2;
                soft_term<float>(xi, yi, zi, hi, mi, k ? a.y : a.x, k ? a.w : a.z, k ? b.y : b.x,
                                 k ? b.w : b.z, k ? q01.y : q01.x, k ? q01.w : q01.z,
                                 k ? q23.y : q23.x, k ? q23.w : q23.z, k ? q45.y : q45.x,
                                 k ? q45.w : q45.z, k ? h.y : h.x, ax, ay, az, pot, idt2);
                kahan_add(A.s[0], A.c[0], ax);
                kahan_add(A.s[1], A.c[1], ay);
                kahan_add(A.s[2], A.c[2], az);
                kahan_add(A.s[3], A.c[3], pot);
                A.dt = fmaxf(A.dt, idt2);
            }
        }
    } else {
        for (int e = slot; e < cnt; e += 32 / NBT) {
            Real ax, ay, az, pot, idt2;
            soft_term<Real>(xi, yi, zi, hi, mi, S.D.ex[e], S.D.ey[e], S.D.ez[e], S.D.em[e],
                            S.D.q[0][e], S.D.q[1][e], S.D.q[2][e], S.D.q[3][e], S.D.q[4][e],
                            S.D.q[5][e], S.D.eh[e], ax, ay, az, pot, idt2);
            A.s[0] += ax;
            A.s[1] += ay;
            A.s[2] += az;
            A.t[3] += pot;
            A.dt = idt2 > A.dt ? idt2 : A.dt;
        }
    }
}

// FP64: add the tile partial to the running sums.  FP32 tiles fold their
// packed partials themselves.
template <typename Real>
__device__ __forceinline__ void flush_tile(Acc<Real> &A) {
    if constexpr (sizeof(Real) == 8) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            A.s[k] += A.t[k];
            A.t[k] = 0;
        }
    }
}

// Per-lane tallies of the opening tests, summed when the warp exits.
struct WalkTally {
    unsigned visit, tests, exact;
};

// A group walk leaves in its warp's scratch, for the bucket walks of the
// group, the (cell, replica) entries every bucket must still test (U, from
// the scratch's start) and the cells every bucket accepts as Newtonian
// (NA, from GRP_U on); their sizes are in the warp's shared memory.  U
// seeds a bucket walk's stack, so it stays well below STK.
#define GRP_U 384
#define GRP_NA 1024
#define GRP_SCRATCH (GRP_U + GRP_NA)

#define GW_NONE 0
#define GW_PUSH 1
#define GW_U 2
#define GW_NA 3

// One bucket's walk and interactions.  With valid group lists the group's
// NA cells are evaluated first, as Newtonian cells, and the walk starts
// from the group's U entries; otherwise it starts from the root in every
// replica.  Either way the lists are the reference's.
// A bucket's FP32 walk geometry (k_bucket_prep): centre (hi/lo), box
// corners about the centre, box extent (negative: no active particle),
// largest softening and active count.
struct BucketGeom {
    float bch[3], bcl[3], fbmn[3], fbmx[3], bext, fSoftMaxF;
    int nAct;
};

__device__ __forceinline__ BucketGeom bucket_geom(const TsphDevTree &T, int b) {
    BucketGeom g;
    const float4 r0 = T.brec[4 * b], r1 = T.brec[4 * b + 1];
    const float4 r2 = T.brec[4 * b + 2], r3 = T.brec[4 * b + 3];
    g.bch[0] = r0.x; g.bch[1] = r0.y; g.bch[2] = r0.z; g.fSoftMaxF = r0.w;
    g.bcl[0] = r1.x; g.bcl[1] = r1.y; g.bcl[2] = r1.z; g.bext = r1.w;
    g.fbmn[0] = r2.x; g.fbmn[1] = r2.y; g.fbmn[2] = r2.z; g.nAct = (int)r2.w;
    g.fbmx[0] = r3.x; g.fbmx[1] = r3.y; g.fbmx[2] = r3.z;
    return g;
}

// One walk entry (cell, replica) against bucket b (node `node`, particles
// [lo, lo + n)): the reference's decisions of pkdBucketWalk (walk.c:58-178)
// -- opened (interior: ACT_OPEN, leaf: ACT_LEAF; the bucket's own leaf in
// the home replica is left out), or accepted as a Newtonian (ACT_NEWT) or
// softened (ACT_SOFT) cell.  The FP32 tests carry a bound on their own
// rounding; what they cannot settle is decided in FP64 exactly as the
// reference does (exact_decision).  classify_loaded takes the cell's walk
// records (particle count cnt, child link up, COM hi/lo with fOpen2 and
// softening in .w) already loaded; classify_entry loads them and returns
// the child link and the leaf's particle range through up / plo / cnt.
__device__ __forceinline__ int classify_loaded(const TsphDevTree &T, const TsphDevParts &P, int b, int node,
                                               int lo, int n, const BucketGeom &G, int cell, int rep,
                                               int up, int cnt, float4 ch, float4 cl, WalkTally &K) {
    const float u32 = 5.9604645e-08f;   // 2^-24
    const float relF = 4.0f * u32;
    float ohx, ohy, ohz, olx, oly, olz;
    rep_off32(rep, ohx, ohy, ohz, olx, oly, olz);
    const float rx = ((ch.x - G.bch[0]) + ohx) + ((cl.x - G.bcl[0]) + olx);
    const float ry = ((ch.y - G.bch[1]) + ohy) + ((cl.y - G.bcl[1]) + oly);
    const float rz = ((ch.z - G.bch[2]) + ohz) + ((cl.z - G.bcl[2]) + olz);
    const float dx = fmaxf(fmaxf(G.fbmn[0] - rx, rx - G.fbmx[0]), 0.0f);
    const float dy = fmaxf(fmaxf(G.fbmn[1] - ry, ry - G.fbmx[1]), 0.0f);
    const float dz = fmaxf(fmaxf(G.fbmn[2] - rz, rz - G.fbmx[2]), 0.0f);
    const float D2 = dx * dx + dy * dy + dz * dz;
    const float Sx = fmaxf(fmaxf(fabsf(rx), fabsf(ry)), fabsf(rz)) + G.bext + cW.offmax;
    const float e = 6.0f * u32 * Sx + cW.E0;
    const float M = 2.0f * e * (dx + dy + dz + 2.0f * e) + 3.0f * e * e + 4.0f * u32 * D2;
    bool open;
    if (cnt < 4) {
        open = true;
    } else {
        ++K.tests;
        const int fo = filt(D2, M, ch.w, relF);
        if (fo == 0) {
            ++K.exact;
            double o[3];
            rep_off64(rep, o);
            open = exact_decision(T, P, b, lo, n, cell, o, true) == 1;
        } else {
            open = fo < 0;
        }
    }
    if (open) {
        if (up >= 0) return ACT_OPEN;
        return (cell == node && rep == cW.selfRep) ? ACT_NONE : ACT_LEAF;
    }
    // softened or Newtonian (walk.c:122-127)
    const float a32 = cl.w + G.fSoftMaxF;
    const float t2 = a32 * a32;
    const int fs = filt(t2, 8.0f * u32 * t2, ch.w, relF);   // t2 vs fOpen2
    bool newt = false;
    bool exactNeeded = (fs == 0);
    if (!exactNeeded) {
        if (fs < 0) newt = true;   // twoh2 < fOpen2 (certain)
        else {
            const int fi = filt(D2, M + 8.0f * u32 * t2, t2, relF);
            if (fi == 0) exactNeeded = true;
            else newt = fi > 0;
        }
    }
    if (exactNeeded) {
        ++K.exact;
        double o[3];
        rep_off64(rep, o);
        newt = exact_decision(T, P, b, lo, n, cell, o, false) == 0;
    }
    return newt ? ACT_NEWT : ACT_SOFT;
}

__device__ __forceinline__ int classify_entry(const TsphDevTree &T, const TsphDevParts &P, int b, int node,
                                              int lo, int n, const BucketGeom &G, int cell, int rep,
                                              int &up, int &plo, int &cnt, WalkTally &K) {
    ++K.visit;
    const int4 lk = T.wlink[cell];
    plo = lk.x;
    cnt = lk.y;
    up = lk.z;
    return classify_loaded(T, P, b, node, lo, n, G, cell, rep, up, cnt, T.wcomh[cell], T.wcoml[cell], K);
}

// A bucket's start, shared by the fused walk and the list evaluation: its
// node and particles; a bucket holding more than NBT coincident particles
// raises TSPH_ERR_UNSUPPORTED and one with no active particle is not
// walked (pkd.c:2932) -- both return false.  Otherwise the bucket's
// particles are in S.px.. (FP32: relative to the bucket centre).
template <typename Real, int NBT, bool HIGH, class Smem>
__device__ __forceinline__ bool bucket_begin(const WalkArgs &W, Smem &S, int b, int lane,
                                             int &node, int &lo, int &n, BucketGeom &G) {
    const TsphDevTree &T = W.T;
    const TsphDevParts &P = W.P;
    node = T.leaves[b];
    lo = T.pLower[node];
    n = T.pUpper[node] - lo + 1;
    if (n > NBT) {
        // a zero-extent leaf holding more than NBT coincident particles
        if (lane == 0) atomicOr(&W.cnt->status, 1u << TSPH_ERR_UNSUPPORTED);
        return false;
    }
    // bucket geometry: FP32 records prepared once per bucket (k_bucket_prep)
    G = bucket_geom(T, b);
    if (G.bext < 0.0f) {   // no active particle: not walked (pkd.c:2932)
        if (lane == 0 && W.bucketLists) {
            W.bucketLists[4 * b + 0] = node;
            W.bucketLists[4 * b + 1] = W.bucketLists[4 * b + 2] = W.bucketLists[4 * b + 3] = -1;
        }
        return false;
    }
    // bucket particles
    if (lane < NBT) {
        int p = lo + (lane < n ? lane : 0);
        if constexpr (sizeof(Real) == 4) {
            float4 a = P.ph[p], c = P.pl[p];
            S.px[lane] = ((a.x - G.bch[0]) + (c.x - G.bcl[0]));
            S.py[lane] = ((a.y - G.bch[1]) + (c.y - G.bcl[1]));
            S.pz[lane] = ((a.z - G.bch[2]) + (c.z - G.bcl[2]));
            S.pm[lane] = a.w;
            S.ph[lane] = c.w;
        } else {
            S.px[lane] = (Real)P.x[p];
            S.py[lane] = (Real)P.y[p];
            S.pz[lane] = (Real)P.z[p];
            S.pm[lane] = (Real)P.m[p];
            S.ph[lane] = (Real)P.h[p];
        }
    }
    return true;
}

// A bucket's end: the 32 / NBT partial accumulators of each particle
// reduced, the results written, and pkdGravAll's sums tallied.
template <typename Real, int NBT, bool HIGH, class Smem>
__device__ __forceinline__ void bucket_end(const WalkArgs &W, Smem &S, int b, int node,
                                           int lo, int n, int nAct, Acc<Real> &A, int nPart, int nNewt,
                                           int nSoft, int lane) {
    const TsphDevParts &P = W.P;
    const unsigned FULL = 0xffffffffu;
#pragma unroll
    for (int o = NBT; o < 32; o <<= 1) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            Real s2 = __shfl_xor_sync(FULL, A.s[k], o);
            Real c2 = __shfl_xor_sync(FULL, A.c[k], o);
            two_sum_merge(A.s[k], A.c[k], s2, c2);
        }
        Real d2 = __shfl_xor_sync(FULL, A.dt, o);
        A.dt = d2 > A.dt ? d2 : A.dt;
    }
    if (lane < n) {
        int p = lo + lane;
        if constexpr (sizeof(Real) == 4) {
            P.wsum[p] = make_float4(A.s[0], A.s[1], A.s[2], A.s[3]);
            P.wcmp[p] = make_float4(A.c[0], A.c[1], A.c[2], A.c[3]);
            P.wdt[p] = A.dt;
        } else {
            P.ax[p] = (double)A.s[0];
            P.ay[p] = (double)A.s[1];
            P.az[p] = (double)A.s[2];
            P.pot[p] = (double)A.s[3];
            P.dtGrav[p] = (double)A.dt;
        }
    }
    if (lane == 0) {
        // pkdGravAll's sums over the active particles (pkd.c:2945-2950)
        S.tAct += nAct;
        S.tPP += (unsigned long long)nAct * nPart;
        S.tNewt += (unsigned long long)nAct * nNewt;
        S.tSoft += (unsigned long long)nAct * nSoft;
        S.tBsq += (unsigned long long)nAct * n;
        S.tIntra += (unsigned long long)nAct * (2 * (n - 1) - nAct + 1) / 2;
        if (W.bucketLists) {
            W.bucketLists[4 * b + 0] = node;
            W.bucketLists[4 * b + 1] = nPart;
            W.bucketLists[4 * b + 2] = nSoft;
            W.bucketLists[4 * b + 3] = nNewt;
        }
    }
    __syncwarp();
}

template <typename Real, int NBT, bool HIGH>
__device__ __forceinline__ void walk_bucket(const WalkArgs &W, WalkSmem<Real, NBT, HIGH> &S, int b,
                                            const int *gl, WalkTally &K, int lane) {
    const TsphDevTree &T = W.T;
    const TsphDevParts &P = W.P;
    constexpr int CT = cell_tile<HIGH>();   // cells per tile
    const unsigned FULL = 0xffffffffu;
    int node, lo, n;
    BucketGeom G;
    if (!bucket_begin<Real, NBT, HIGH>(W, S, b, lane, node, lo, n, G)) return;
    const int nAct = G.nAct;
    // accumulators: lane = (particle i, slot)
    const int i = lane % NBT, slot = lane / NBT;
    Acc<Real> A;
#pragma unroll
    for (int k = 0; k < 4; ++k) { A.s[k] = 0; A.c[k] = 0; A.t[k] = 0; }
    A.dt = 0;
    // initial stack: the group's U entries (after its NA cells, evaluated
    // here tile by tile), or the root in every replica; P-P buffer: the
    // bucket's own particles for the intra-bucket pairs (replica tag 31)
    int sp = 0, ppn = 0, cnn = 0, csn = 0, nPart = 0, nNewt = 0, nSoft = 0;
    if (gl) {
        const int nU = S.gU, nNA = S.gNA;
        __syncwarp();
        for (int k0 = 0; k0 < nNA; k0 += CT) {
            const int c = nNA - k0 < CT ? nNA - k0 : CT;
            for (int e = lane; e < c; e += 32) S.cn[e] = gl[GRP_U + k0 + e];
            __syncwarp();
            stage_cells<Real, NBT, HIGH>(S, S.cn, T, c, lane, false, G.bch[0], G.bch[1], G.bch[2], G.bcl[0], G.bcl[1], G.bcl[2]);
            __syncwarp();
            if (i < n) eval_newt<Real, NBT, HIGH>(S, c, i, slot, W.iOrder, A);
            flush_tile(A);
            __syncwarp();
        }
        nNewt = nNA;
        for (int k = lane; k < nU; k += 32) S.stack[k] = gl[k];
        sp = nU;
    } else {
        const int root = T.sysRoot[P.rid[lo]];   // the bucket's own system
        for (int r = lane; r < cW.nRep; r += 32) S.stack[r] = (root << 5) | r;
        sp = cW.nRep;
    }
    if (lane < n) S.pp[lane] = ((lo + lane) << 5) | 31;
    ppn = n;
    bool ppSelf = true;   // the own particles sit in the first P-P tile
    bool overflow = false;
    __syncwarp();

    while (sp > 0) {
        int act = ACT_NONE, cell = 0, rep = 0, cnt = 0, plo = 0;
        {
            const int take = sp < 32 ? sp : 32;
            const int ent = lane < take ? S.stack[sp - take + lane] : -1;
            __syncwarp();
            sp -= take;
            int up = -1;
            if (ent >= 0) {
                cell = ent >> 5;
                rep = ent & 31;
                act = classify_entry(T, P, b, node, lo, n, G, cell, rep, up, plo, cnt, K);
            }
            // children (upper first so the lower child is popped first)
            const unsigned bo = __ballot_sync(FULL, act == ACT_OPEN);
            if (sp + 2 * __popc(bo) > STK) { overflow = true; break; }
            if (act == ACT_OPEN) {
                const int pos = sp + 2 * __popc(bo & lane_lt());
                S.stack[pos] = (up << 5) | rep;
                S.stack[pos + 1] = ((cell + 1) << 5) | rep;
            }
            sp += 2 * __popc(bo);
        }
        // leaf particles
        if (act == ACT_LEAF && cnt > NBT) {
            atomicOr(&W.cnt->status, 1u << TSPH_ERR_UNSUPPORTED);
            act = ACT_NONE;
        }
        int c0 = act == ACT_LEAF ? cnt : 0;
        int incl = c0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += y;
        }
        int tot = __shfl_sync(FULL, incl, 31);
        for (int k = 0; k < c0; ++k) S.pp[ppn + incl - c0 + k] = ((plo + k) << 5) | rep;
        ppn += tot;
        nPart += tot;
        unsigned bn = __ballot_sync(FULL, act == ACT_NEWT);
        if (act == ACT_NEWT) S.cn[cnn + __popc(bn & lane_lt())] = (cell << 5) | rep;
        cnn += __popc(bn);
        nNewt += __popc(bn);
        unsigned bs = __ballot_sync(FULL, act == ACT_SOFT);
        if (act == ACT_SOFT) S.cs[csn + __popc(bs & lane_lt())] = (cell << 5) | rep;
        csn += __popc(bs);
        nSoft += __popc(bs);
        __syncwarp();
        // evaluate full tiles
        while (ppn >= PPF) {
            stage_pp<Real, NBT, HIGH>(S, P, S.pp, PPF, lane, G.bch[0], G.bch[1], G.bch[2], G.bcl[0], G.bcl[1], G.bcl[2]);
            __syncwarp();
            if (i < n) {
                if (ppSelf) eval_pp<Real, NBT, HIGH, true>(S, PPF, i, slot, A);
                else eval_pp<Real, NBT, HIGH, false>(S, PPF, i, slot, A);
            }
            ppSelf = false;
            flush_tile(A);
            __syncwarp();
            for (int e = lane; e < ppn - PPF; e += 32) S.pp[e] = S.pp[PPF + e];
            ppn -= PPF;
            __syncwarp();
        }
        while (cnn >= CT) {
            stage_cells<Real, NBT, HIGH>(S, S.cn, T, CT, lane, false, G.bch[0], G.bch[1], G.bch[2], G.bcl[0], G.bcl[1], G.bcl[2]);
            __syncwarp();
            if (i < n) eval_newt<Real, NBT, HIGH>(S, CT, i, slot, W.iOrder, A);
            flush_tile(A);
            __syncwarp();
            for (int e = lane; e < cnn - CT; e += 32) S.cn[e] = S.cn[CT + e];
            cnn -= CT;
            __syncwarp();
        }
        while (csn >= CT) {
            stage_cells<Real, NBT, HIGH>(S, S.cs, T, CT, lane, true, G.bch[0], G.bch[1], G.bch[2], G.bcl[0], G.bcl[1], G.bcl[2]);
            __syncwarp();
            if (i < n) eval_soft<Real, NBT, HIGH>(S, CT, i, slot, A);
            flush_tile(A);
            __syncwarp();
            for (int e = lane; e < csn - CT; e += 32) S.cs[e] = S.cs[CT + e];
            csn -= CT;
            __syncwarp();
        }
    }
    if (overflow) {
        if (lane == 0) atomicOr(&W.cnt->status, 1u << TSPH_ERR_STACK_OVERFLOW);
        __syncwarp();
        return;
    }
    // remaining partial tiles
    if (ppn > 0) {
        stage_pp<Real, NBT, HIGH>(S, P, S.pp, ppn, lane, G.bch[0], G.bch[1], G.bch[2], G.bcl[0], G.bcl[1], G.bcl[2]);
        __syncwarp();
        if (i < n) {
            if (ppSelf) eval_pp<Real, NBT, HIGH, true>(S, ppn, i, slot, A);
            else eval_pp<Real, NBT, HIGH, false>(S, ppn, i, slot, A);
        }
        flush_tile(A);
        __syncwarp();
    }
    if (cnn > 0) {
        stage_cells<Real, NBT, HIGH>(S, S.cn, T, cnn, lane, false, G.bch[0], G.bch[1], G.bch[2], G.bcl[0], G.bcl[1], G.bcl[2]);
        __syncwarp();
        if (i < n) eval_newt<Real, NBT, HIGH>(S, cnn, i, slot, W.iOrder, A);
        flush_tile(A);
        __syncwarp();
    }
    if (csn > 0) {
        stage_cells<Real, NBT, HIGH>(S, S.cs, T, csn, lane, true, G.bch[0], G.bch[1], G.bch[2], G.bcl[0], G.bcl[1], G.bcl[2]);
        __syncwarp();
        if (i < n) eval_soft<Real, NBT, HIGH>(S, csn, i, slot, A);
        flush_tile(A);
        __syncwarp();
    }
    bucket_end<Real, NBT, HIGH>(W, S, b, node, lo, n, nAct, A, nPart, nNewt, nSoft, lane);
}

// The evaluation pass of the two-pass walk for bucket b: its stored lists
// (k_walk_lists) streamed tile by tile -- P-P particles (the bucket's own
// first: the first tile leaves out each particle's pair with itself), then
// Newtonian cells, then softened cells.  The tiles are the fused walk's,
// fed from memory with no walk state: the terms are the same, summed in
// list order.
template <typename Real, int NBT, bool HIGH, class Smem>
__device__ __forceinline__ void eval_bucket_lists(const WalkArgs &W, Smem &S, int b,
                                                  int4 info, int lane) {
    const TsphDevTree &T = W.T;
    const TsphDevParts &P = W.P;
    constexpr int CT = cell_tile<HIGH>();   // cells per tile
    int node, lo, n;
    BucketGeom G;
    if (!bucket_begin<Real, NBT, HIGH>(W, S, b, lane, node, lo, n, G)) return;
    const int i = lane % NBT, slot = lane / NBT;
    Acc<Real> A;
#pragma unroll
    for (int k = 0; k < 4; ++k) { A.s[k] = 0; A.c[k] = 0; A.t[k] = 0; }
    A.dt = 0;
    const size_t base = (size_t)b * W.listCap;
    const int *lp = W.listPP + base, *lc = W.listCell + base;
    const int *ls = W.listSoft + (size_t)b * (W.listCap / 4);
    __syncwarp();
    for (int t0 = 0; t0 < info.x; t0 += PPF) {
        const int c = info.x - t0 < PPF ? info.x - t0 : PPF;
        stage_pp<Real, NBT, HIGH>(S, P, lp + t0, c, lane, G.bch[0], G.bch[1], G.bch[2], G.bcl[0], G.bcl[1], G.bcl[2]);
        __syncwarp();
        if (i < n) {
            if (t0 == 0) eval_pp<Real, NBT, HIGH, true>(S, c, i, slot, A);
            else eval_pp<Real, NBT, HIGH, false>(S, c, i, slot, A);
        }
        flush_tile(A);
        __syncwarp();
    }
    for (int t0 = 0; t0 < info.y; t0 += CT) {
        const int c = info.y - t0 < CT ? info.y - t0 : CT;
        stage_cells<Real, NBT, HIGH>(S, lc + t0, T, c, lane, false, G.bch[0], G.bch[1], G.bch[2], G.bcl[0], G.bcl[1], G.bcl[2]);
        __syncwarp();
        if (i < n) eval_newt<Real, NBT, HIGH>(S, c, i, slot, W.iOrder, A);
        flush_tile(A);
        __syncwarp();
    }
    for (int t0 = 0; t0 < info.z; t0 += CT) {
        const int c = info.z - t0 < CT ? info.z - t0 : CT;
        stage_cells<Real, NBT, HIGH>(S, ls + t0, T, c, lane, true, G.bch[0], G.bch[1], G.bch[2], G.bcl[0], G.bcl[1], G.bcl[2]);
        __syncwarp();
        if (i < n) eval_soft<Real, NBT, HIGH>(S, c, i, slot, A);
        flush_tile(A);
        __syncwarp();
    }
    bucket_end<Real, NBT, HIGH>(W, S, b, node, lo, n, G.nAct, A, info.x - n, info.y, info.z, lane);
}

// The walk of a group of buckets (the subtree node g, buckets b0..b1-1),
// made once with the group's box, which holds every bucket's box.  A cell
// goes to NA when it is certainly not opened and certainly Newtonian for
// any box inside the group's (its distance from the group box exceeds
// sqrt(fOpen2), and (cellSoft + group max softening)^2 is below fOpen2 or
// below that distance); an interior cell is opened here when the whole
// group box lies within sqrt(fOpen2) of it (or it holds fewer than 4
// particles); every other cell, leaves included, goes to U.
// The FP32 tests carry the bucket walk's rounding bound, so every such
// decision is the one each bucket's FP64 test would reach.  Returns false
// when a list or the stack overflows (the buckets then walk from the root).
template <typename Real, int NBT, bool HIGH>
__device__ __noinline__ bool walk_group(const WalkArgs &W, WalkSmem<Real, NBT, HIGH> &S, int g, int b0,
                                        int b1, int *gl, WalkTally &K, int lane) {
    const TsphDevTree &T = W.T;
    const unsigned FULL = 0xffffffffu;
    const float u32 = 5.9604645e-08f;   // 2^-24
    const float relF = 4.0f * u32;
    // group box (the node's bounds) about its centre in FP32, by one lane
    float v[13];
    if (lane == 0) {
        float ext = 0.0f;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const double mn = T.bnd[6 * g + k], mx = T.bnd[6 * g + 3 + k];
            const double c = 0.5 * (mn + mx);
            split2f(c, v[k], v[3 + k]);
            v[6 + k] = (float)(mn - c);
            v[9 + k] = (float)(mx - c);
            ext = fmaxf(ext, fmaxf(fabsf(v[6 + k]), fabsf(v[9 + k])));
        }
        v[12] = ext;
    }
#pragma unroll
    for (int k = 0; k < 13; ++k) v[k] = __shfl_sync(FULL, v[k], 0);
    const float gch[3] = {v[0], v[1], v[2]}, gcl[3] = {v[3], v[4], v[5]};
    const float gmn[3] = {v[6], v[7], v[8]}, gmx[3] = {v[9], v[10], v[11]};
    const float gext = v[12];
    // largest softening of the group (each bucket's FP32 maximum)
    float gsoft = 0.0f;
    for (int b = b0 + lane; b < b1; b += 32) gsoft = fmaxf(gsoft, T.brec[4 * b].w);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) gsoft = fmaxf(gsoft, __shfl_xor_sync(FULL, gsoft, o));

    int *gu = gl, *gna = gl + GRP_U;
    const int root = T.sysRoot[W.P.rid[T.pLower[g]]];
    for (int r = lane; r < cW.nRep; r += 32) S.stack[r] = (root << 5) | r;
    int sp = cW.nRep, nU = 0, nNA = 0;
    bool ok = true;
    __syncwarp();
    while (sp > 0) {
        const int take = sp < 32 ? sp : 32;
        const int ent = lane < take ? S.stack[sp - take + lane] : -1;
        __syncwarp();
        sp -= take;
        int cls = GW_NONE, cell = 0, rep = 0, up = -1;
        if (ent >= 0) {
            ++K.visit;
            cell = ent >> 5;
            rep = ent & 31;
            const int4 lk = T.wlink[cell];
            const int cnt = lk.y;
            up = lk.z;
            const float4 ch = T.wcomh[cell], cl = T.wcoml[cell];
            float ohx, ohy, ohz, olx, oly, olz;
            rep_off32(rep, ohx, ohy, ohz, olx, oly, olz);
            const float rx = ((ch.x - gch[0]) + ohx) + ((cl.x - gcl[0]) + olx);
            const float ry = ((ch.y - gch[1]) + ohy) + ((cl.y - gcl[1]) + oly);
            const float rz = ((ch.z - gch[2]) + ohz) + ((cl.z - gcl[2]) + olz);
            // nearest and farthest point of the group box
            const float dx = fmaxf(fmaxf(gmn[0] - rx, rx - gmx[0]), 0.0f);
            const float dy = fmaxf(fmaxf(gmn[1] - ry, ry - gmx[1]), 0.0f);
            const float dz = fmaxf(fmaxf(gmn[2] - rz, rz - gmx[2]), 0.0f);
            const float fx = fmaxf(rx - gmn[0], gmx[0] - rx);
            const float fy = fmaxf(ry - gmn[1], gmx[1] - ry);
            const float fz = fmaxf(rz - gmn[2], gmx[2] - rz);
            const float D2 = dx * dx + dy * dy + dz * dz;
            const float F2 = fx * fx + fy * fy + fz * fz;
            const float Sx = fmaxf(fmaxf(fabsf(rx), fabsf(ry)), fabsf(rz)) + gext + cW.offmax;
            const float e = 6.0f * u32 * Sx + cW.E0;
            const float M = 2.0f * e * (dx + dy + dz + 2.0f * e) + 3.0f * e * e + 4.0f * u32 * D2;
            const float MF = 2.0f * e * (fx + fy + fz + 2.0f * e) + 3.0f * e * e + 4.0f * u32 * F2;
            if (cnt < 4) {
                cls = up >= 0 ? GW_PUSH : GW_U;
            } else {
                ++K.tests;
                if (filt(F2, MF, ch.w, relF) < 0) {
                    cls = up >= 0 ? GW_PUSH : GW_U;
                } else if (filt(D2, M, ch.w, relF) > 0) {
                    const float a32 = cl.w + gsoft;
                    const float t2 = a32 * a32;
                    const bool newt = filt(t2, 8.0f * u32 * t2, ch.w, relF) < 0 ||
                                      filt(D2, M + 8.0f * u32 * t2, t2, relF) > 0;
                    cls = newt ? GW_NA : GW_U;
                } else {
                    cls = GW_U;
                }
            }
        }
        const unsigned bo = __ballot_sync(FULL, cls == GW_PUSH);
        const unsigned bu = __ballot_sync(FULL, cls == GW_U);
        const unsigned bn = __ballot_sync(FULL, cls == GW_NA);
        if (sp + 2 * __popc(bo) > STK || nU + __popc(bu) > GRP_U || nNA + __popc(bn) > GRP_NA) {
            ok = false;
            break;
        }
        const unsigned lt = lane_lt();
        if (cls == GW_PUSH) {
            const int pos = sp + 2 * __popc(bo & lt);
            S.stack[pos] = (up << 5) | rep;
            S.stack[pos + 1] = ((cell + 1) << 5) | rep;
        } else if (cls == GW_U) {
            gu[nU + __popc(bu & lt)] = ent;
        } else if (cls == GW_NA) {
            gna[nNA + __popc(bn & lt)] = ent;
        }
        sp += 2 * __popc(bo);
        nU += __popc(bu);
        nNA += __popc(bn);
        __syncwarp();
    }
    if (lane == 0) {
        S.gU = nU;
        S.gNA = nNA;
    }
    __syncwarp();   // the lists are read back by other lanes of this warp
    return ok;
}

// FP32: five resident blocks per SM (96 registers, 40 KB of shared memory
// per block), three with octopole/hexadecapole cells; FP64: limited by its
// larger tiles.
template <typename Real, int NBT, bool HIGH>
__global__ void __launch_bounds__(WPB * 32, sizeof(Real) == 4 ? (HIGH ? 3 : 5) : 1) k_walk(WalkArgs W) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    WalkSmem<Real, NBT, HIGH> &S = reinterpret_cast<WalkSmem<Real, NBT, HIGH> *>(smraw)[wib];
    const unsigned FULL = 0xffffffffu;
    WalkTally K = {0u, 0u, 0u};
    if (lane == 0) S.tAct = S.tPP = S.tNewt = S.tSoft = S.tBsq = S.tIntra = 0ull;
    __syncwarp();

    for (;;) {
        int u = 0;
        if (lane == 0) u = atomicAdd(W.workCounter, 1);
        u = __shfl_sync(FULL, u, 0);
        if (W.groupFirst) {
            if (u >= *W.nGroups) break;
            const int b0 = W.groupFirst[u], b1 = W.groupFirst[u + 1];
            // a group walk pays off once two of its buckets walk
            int na = 0;
            for (int b = b0 + lane; b < b1; b += 32) na += W.T.brec[4 * b + 1].w >= 0.0f;
            na = __reduce_add_sync(FULL, na);
            int *gl = W.groupScratch + (size_t)(blockIdx.x * WPB + wib) * GRP_SCRATCH;
            bool grp = false;
            if (na >= 2) {
                // the group's node: the highest ancestor of its first bucket
                // holding at most groupMax particles
                int g = W.T.leaves[b0];
                if (lane == 0)
                    for (;;) {
                        const int p = W.T.parent[g];
                        if (p < 0 || W.T.pUpper[p] - W.T.pLower[p] + 1 > W.groupMax) break;
                        g = p;
                    }
                g = __shfl_sync(FULL, g, 0);
                grp = walk_group<Real, NBT, HIGH>(W, S, g, b0, b1, gl, K, lane);
            }
            for (int b = b0; b < b1; ++b) walk_bucket<Real, NBT, HIGH>(W, S, b, grp ? gl : nullptr, K, lane);
        } else if (W.fallback) {   // the buckets the list pass left over
            if (u >= (int)W.cnt->nListFallback) break;
            walk_bucket<Real, NBT, HIGH>(W, S, W.fallback[u], nullptr, K, lane);
        } else {
            if (u >= *W.nBuckets) break;
            walk_bucket<Real, NBT, HIGH>(W, S, u, nullptr, K, lane);
        }
    }
    // counters: tests and visits per lane, the rest from the warp's tallies
    unsigned long long tests = K.tests, visit = K.visit, exact = K.exact;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        tests += __shfl_xor_sync(FULL, tests, o);
        visit += __shfl_xor_sync(FULL, visit, o);
        exact += __shfl_xor_sync(FULL, exact, o);
    }
    if (lane == 0) {
        atomicAdd(&W.cnt->nActive, S.tAct);
        atomicAdd(&W.cnt->nPartPP, S.tPP);
        atomicAdd(&W.cnt->nCellNewt, S.tNewt);
        atomicAdd(&W.cnt->nCellSoft, S.tSoft);
        atomicAdd(&W.cnt->nBucketSq, S.tBsq);
        atomicAdd(&W.cnt->nIntra, S.tIntra);
        atomicAdd(&W.cnt->nTests, tests);
        atomicAdd(&W.cnt->nVisits, visit);
        atomicAdd(&W.cnt->nExactTests, exact);
    }
}

// The list pass of the two-pass walk.  Each warp takes buckets from a work
// counter and walks them exactly as walk_bucket does (classify_entry, the
// same stack discipline), but stores what it finds instead of evaluating:
// the bucket's own particles and then the particles of every opened leaf
// (P-P list), the Newtonian cells and the softened cells, each as
// (index << 5) | replica, in walk order.  This mirrors the reference's own
// split into pkdBucketWalk (walk.c:58-178), which builds the lists, and
// pkdBucketInteract (grav.c:23-249), which evaluates them.  Without the
// evaluation's registers and tiles a warp needs a stack only, so many
// warps fit on an SM and the walk's dependent L2 loads overlap.  A bucket
// whose lists do not fit their slots is marked (w = -1) and walked by a
// fused launch; its walk is still counted to the end, so the longest list
// any bucket needed sizes the slots of the next call.  Buckets the
// evaluation pass skips (no active particle, more than NBT coincident
// particles) are not walked here.  (Walking units of 2 or 4 neighbouring
// buckets together, one stack entry per cell of their union walk with a
// mask of the buckets it concerns, measured slower: the per-bucket
// decisions and appends, not the shared loads, carry the cost.)
#define LWPB 8   // warps per block
#define LBPS 5   // blocks per SM: 40 warps, 48 registers a thread
template <int NBT>
__global__ void __launch_bounds__(LWPB * 32, LBPS) k_walk_lists(WalkArgs W) {
    __shared__ int stk[LWPB][STK];
    const int lane = threadIdx.x & 31;
    int *stack = stk[threadIdx.x >> 5];
    const unsigned FULL = 0xffffffffu;
    const TsphDevTree &T = W.T;
    const TsphDevParts &P = W.P;
    WalkTally K = {0u, 0u, 0u};
    int *work = reinterpret_cast<int *>(&W.cnt->listWork);
    const int cap = W.listCap, capS = W.listCap / 4;
    for (;;) {
        int b = 0;
        if (lane == 0) b = atomicAdd(work, 1);
        b = __shfl_sync(FULL, b, 0);
        if (b >= *W.nBuckets) break;
        const int node = T.leaves[b];
        const int lo = T.pLower[node];
        const int n = T.pUpper[node] - lo + 1;
        const BucketGeom G = bucket_geom(T, b);
        if (n > NBT || G.bext < 0.0f) {
            if (lane == 0) W.listInfo[b] = make_int4(0, 0, 0, 0);
            continue;
        }
        int *lp = W.listPP + (size_t)b * cap;
        int *lc = W.listCell + (size_t)b * cap;
        int *ls = W.listSoft + (size_t)b * capS;
        if (lane < n) lp[lane] = ((lo + lane) << 5) | 31;   // own particles, replica tag 31
        const int root = T.sysRoot[P.rid[lo]];               // the bucket's own system
        for (int r = lane; r < cW.nRep; r += 32) stack[r] = (root << 5) | r;
        int sp = cW.nRep, nP = n, nC = 0, nS = 0;
        bool spill = false, overflow = false;
        __syncwarp();
        while (sp > 0) {
            const int take = sp < 32 ? sp : 32;
            const int ent = lane < take ? stack[sp - take + lane] : -1;
            __syncwarp();
            sp -= take;
            int act = ACT_NONE, cell = 0, rep = 0, up = -1, plo = 0, cnt = 0;
            if (ent >= 0) {
                cell = ent >> 5;
                rep = ent & 31;
                act = classify_entry(T, P, b, node, lo, n, G, cell, rep, up, plo, cnt, K);
            }
            if (act == ACT_LEAF && cnt > NBT) {
                atomicOr(&W.cnt->status, 1u << TSPH_ERR_UNSUPPORTED);
                act = ACT_NONE;
            }
            const unsigned bo = __ballot_sync(FULL, act == ACT_OPEN);
            if (sp + 2 * __popc(bo) > STK) {
                overflow = true;
                break;
            }
            const unsigned bl = __ballot_sync(FULL, act == ACT_LEAF);
            const unsigned bn = __ballot_sync(FULL, act == ACT_NEWT);
            const unsigned bs = __ballot_sync(FULL, act == ACT_SOFT);
            const int leafParts = __reduce_add_sync(FULL, act == ACT_LEAF ? cnt : 0);
            // past a full slot the lists are only counted
            spill = spill || nP + leafParts > cap || nC + __popc(bn) > cap || nS + __popc(bs) > capS;
            const unsigned lt = lane_lt();
            if (act == ACT_OPEN) {
                const int pos = sp + 2 * __popc(bo & lt);
                stack[pos] = (up << 5) | rep;
                stack[pos + 1] = ((cell + 1) << 5) | rep;
            } else if (!spill && act == ACT_NEWT) {
                lc[nC + __popc(bn & lt)] = (cell << 5) | rep;
            } else if (!spill && act == ACT_SOFT) {
                ls[nS + __popc(bs & lt)] = (cell << 5) | rep;
            }
            if (!spill) {   // opened leaves: their particles, one leaf at a time across the warp
                int at = nP;
                for (unsigned m = bl; m; m &= m - 1u) {
                    const int src = __ffs(m) - 1;
                    const int c = __shfl_sync(FULL, cnt, src);
                    const int p0 = __shfl_sync(FULL, plo, src);
                    const int r0 = __shfl_sync(FULL, rep, src);
                    if (lane < c) lp[at + lane] = ((p0 + lane) << 5) | r0;
                    at += c;
                }
            }
            sp += 2 * __popc(bo);
            nP += leafParts;
            nC += __popc(bn);
            nS += __popc(bs);
            __syncwarp();
        }
        if (lane == 0) {
            const bool left = spill || overflow;
            W.listInfo[b] = left ? make_int4(0, 0, 0, -1) : make_int4(nP, nC, nS, 0);
            if (left) W.fallback[atomicAdd(&W.cnt->nListFallback, 1u)] = b;
            if (spill && !overflow) {
                const int need = nP > nC ? (nP > 4 * nS ? nP : 4 * nS) : (nC > 4 * nS ? nC : 4 * nS);
                atomicMax(&W.cnt->listNeed, (unsigned)need);
            }
        }
        __syncwarp();
    }
    unsigned long long tests = K.tests, visit = K.visit, exact = K.exact;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        tests += __shfl_xor_sync(FULL, tests, o);
        visit += __shfl_xor_sync(FULL, visit, o);
        exact += __shfl_xor_sync(FULL, exact, o);
    }
    if (lane == 0) {
        atomicAdd(&W.cnt->nTests, tests);
        atomicAdd(&W.cnt->nVisits, visit);
        atomicAdd(&W.cnt->nExactTests, exact);
    }
}

// The evaluation pass of the two-pass walk: every bucket with stored lists
// (eval_bucket_lists), a warp per bucket from a work counter.  Its shared
// memory holds tiles only, so registers alone set its occupancy.
#define EVAL_BPS(Real, HIGH) (sizeof(Real) == 4 ? (HIGH ? 4 : 8) : 2)
template <typename Real, int NBT, bool HIGH>
__global__ void __launch_bounds__(WPB * 32, EVAL_BPS(Real, HIGH)) k_walk_eval(WalkArgs W) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const int lane = threadIdx.x & 31;
    EvalSmem<Real, NBT, HIGH> &S = reinterpret_cast<EvalSmem<Real, NBT, HIGH> *>(smraw)[threadIdx.x >> 5];
    const unsigned FULL = 0xffffffffu;
    if (lane == 0) S.tAct = S.tPP = S.tNewt = S.tSoft = S.tBsq = S.tIntra = 0ull;
    __syncwarp();
    int *work = reinterpret_cast<int *>(&W.cnt->evalWork);
    for (;;) {
        int b = 0;
        if (lane == 0) b = atomicAdd(work, 1);
        b = __shfl_sync(FULL, b, 0);
        if (b >= *W.nBuckets) break;
        const int4 info = W.listInfo[b];
        if (info.w >= 0) eval_bucket_lists<Real, NBT, HIGH>(W, S, b, info, lane);
    }
    if (lane == 0) {
        atomicAdd(&W.cnt->nActive, S.tAct);
        atomicAdd(&W.cnt->nPartPP, S.tPP);
        atomicAdd(&W.cnt->nCellNewt, S.tNewt);
        atomicAdd(&W.cnt->nCellSoft, S.tSoft);
        atomicAdd(&W.cnt->nBucketSq, S.tBsq);
        atomicAdd(&W.cnt->nIntra, S.tIntra);
    }
}

// FP32 geometry of every bucket: centre (hi/lo), max softening, box
// extent, box corners relative to the centre.  The FP64 work happens here
// once per bucket, by one thread, instead of redundantly on every lane of
// the walk (FP64 issues at 1/64 of the FP32 rate on this part).
//
// As pkdGravAll does (pkd.c:2917-2944), the box a bucket walks with is the
// bounds of its active particles; with every particle active that is the
// node's own box.  A bucket with no active particle gets a negative extent
// and is skipped.  The softening maximum runs over all its particles
// (pkdBucketWalk walk.c:319-324).
__global__ void k_bucket_prep(TsphDevTree T, TsphDevParts P) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= T.dcnt[1]) return;
    int node = T.leaves[b];
    int lo = T.pLower[node], hi = T.pUpper[node];
    double amn[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, amx[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
    double sm = 0.0;
    int nAct = 0;
    for (int p = lo; p <= hi; ++p) {
        sm = fmax(sm, P.h[p]);
        if (!P.act[p]) continue;
        ++nAct;
        const double r[3] = {P.x[p], P.y[p], P.z[p]};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            amn[k] = fmin(amn[k], r[k]);
            amx[k] = fmax(amx[k], r[k]);
        }
    }
    if (nAct == 0) {
#pragma unroll
        for (int k = 0; k < 3; ++k) amn[k] = amx[k] = T.r[3 * node + k];
    }
    double bc[3];
    float bh[3], bl[3], mn[3], mx[3];
    float ext = 0.0f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        T.bact[6 * b + k] = amn[k];
        T.bact[6 * b + 3 + k] = amx[k];
        bc[k] = 0.5 * (amn[k] + amx[k]);
        split2f(bc[k], bh[k], bl[k]);
        mn[k] = (float)(amn[k] - bc[k]);
        mx[k] = (float)(amx[k] - bc[k]);
        ext = fmaxf(ext, fmaxf(fabsf(mn[k]), fabsf(mx[k])));
    }
    T.brec[4 * b] = make_float4(bh[0], bh[1], bh[2], (float)sm);
    T.brec[4 * b + 1] = make_float4(bl[0], bl[1], bl[2], nAct > 0 ? ext : -1.0f);
    T.brec[4 * b + 2] = make_float4(mn[0], mn[1], mn[2], (float)nAct);
    T.brec[4 * b + 3] = make_float4(mx[0], mx[1], mx[2], 0.0f);
}

// FP32 walk without an Ewald pass: fold the compensated pairs into FP64
__global__ void k_finish_f32(int n, TsphDevParts P) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    float4 s = P.wsum[p], c = P.wcmp[p];
    P.ax[p] = (double)s.x - (double)c.x;
    P.ay[p] = (double)s.y - (double)c.y;
    P.az[p] = (double)s.z - (double)c.z;
    P.pot[p] = (double)s.w - (double)c.w;
    P.dtGrav[p] = (double)P.wdt[p];
}

int tsph_walk_finish_f32(tsph_ctx *ctx) {
    k_finish_f32<<<tsph_blocks(ctx->n, 256), 256, 0, ctx->stream>>>(ctx->n, ctx->P);
    TSPH_LAUNCH_CK("k_finish_f32");
    return TSPH_OK;
}

// Walk groups: the largest subtrees holding at most G particles.  Bucket b
// starts a group when the group's node begins at the bucket's first
// particle (the buckets of a subtree are consecutive in depth-first order).
__global__ void k_group_mark(TsphDevTree T, int G, int cap, int *flag) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= cap) return;
    int f = 0;
    if (b < T.dcnt[1]) {
        const int leaf = T.leaves[b];
        int c = leaf;
        for (;;) {
            const int p = T.parent[c];
            if (p < 0 || T.pUpper[p] - T.pLower[p] + 1 > G) break;
            c = p;
        }
        f = T.pLower[c] == T.pLower[leaf];
    }
    flag[b] = f;
}

__global__ void k_group_list(TsphDevTree T, int cap, const int *flag, const int *scan, int *first,
                             int *count) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= cap) return;
    const int nb = T.dcnt[1];
    if (b < nb && flag[b]) first[scan[b] - 1] = b;
    if (b == (nb > 0 ? nb - 1 : 0)) {
        const int ng = nb > 0 ? scan[nb - 1] : 0;
        *count = ng;
        first[ng] = nb;
    }
}

// Group arrays and the per-warp list scratch; outside a capture they grow
// to the particle count (a bound on the buckets of any later captured
// step).  A.groupFirst stays null when groups are off or (in a capture)
// not sized.
// By default groups hold up to 128 particles, and are used when there are
// at least 256 particles per walk warp: a group is one work unit, and with
// fewer the last units leave most warps idle.
static int prepare_groups(tsph_ctx *ctx, WalkArgs &A, int nbHost, int warps) {
    const int G = ctx->walkGroup == 0 ? 128 : ctx->walkGroup;
    if (ctx->walkGroup == 0 && (long long)ctx->n < 256LL * warps) return TSPH_OK;
    if (G <= 0 || nbHost <= 0) return TSPH_OK;
    if (!ctx->capturing) {
        const int cap = nbHost > ctx->n ? nbHost : ctx->n;
        if (ctx->groupCap < cap) {
            int rc = tsph_grow(ctx, &ctx->dGroupFlag, (size_t)cap);
            if (!rc) rc = tsph_grow(ctx, &ctx->dGroupScan, (size_t)cap);
            if (!rc) rc = tsph_grow(ctx, &ctx->dGroupFirst, (size_t)cap + 2);
            if (!rc && !ctx->dGroupCount) rc = tsph_grow(ctx, &ctx->dGroupCount, 1);
            if (rc) { ctx->groupCap = 0; return rc; }
            ctx->groupCap = cap;
        }
        if (ctx->groupScratchWarps < warps) {
            int rc = tsph_grow(ctx, &ctx->dGroupScratch, (size_t)warps * GRP_SCRATCH);
            if (rc) { ctx->groupScratchWarps = 0; return rc; }
            ctx->groupScratchWarps = warps;
        }
    }
    if (ctx->groupCap < nbHost || ctx->groupScratchWarps < warps) return TSPH_OK;
    k_group_mark<<<tsph_blocks(nbHost, 256), 256, 0, ctx->stream>>>(ctx->T, G, nbHost, ctx->dGroupFlag);
    TSPH_LAUNCH_CK("k_group_mark");
    int rc = tsph_scan_inclusive(ctx, ctx->dGroupFlag, ctx->dGroupScan, nbHost);
    if (rc) return rc;
    k_group_list<<<tsph_blocks(nbHost, 256), 256, 0, ctx->stream>>>(ctx->T, nbHost, ctx->dGroupFlag,
                                                                     ctx->dGroupScan, ctx->dGroupFirst,
                                                                     ctx->dGroupCount);
    TSPH_LAUNCH_CK("k_group_list");
    A.groupFirst = ctx->dGroupFirst;
    A.nGroups = ctx->dGroupCount;
    A.groupScratch = ctx->dGroupScratch;
    A.groupMax = G;
    return TSPH_OK;
}

// The two-pass walk (k_walk_lists, then k_walk_eval over the stored
// lists), when there are no walk groups and the tuning asks for it
// (walkLists 1, or >= 32: that many P-P and cell entries per bucket; 0 and
// -1: one fused pass).  By default a bucket's slots start at 512 entries
// and grow, for the next call, to the power of two that holds the longest
// list a bucket of the last call needed, as long as all slots stay within
// 16 GB; a bucket that does not fit is walked by a fused launch.  Outside a
// capture the arrays grow to twice the buckets; a capture uses what is
// there (and walks fused when that is too little).
static int prepare_lists(tsph_ctx *ctx, WalkArgs &A, int nbHost, int nbt) {
    A.listPP = A.listCell = A.listSoft = nullptr;
    A.listInfo = nullptr;
    A.listCap = 0;
    A.fallback = nullptr;
    if (ctx->walkLists <= 0 || A.groupFirst || nbHost <= 0) return TSPH_OK;
    if (ctx->n >= (1 << 26) || ctx->T.nNodes >= (1 << 26)) return TSPH_OK;   // (index << 5) entries
    if (!ctx->capturing) {
        // room for twice the buckets (a captured step's trees may hold more)
        const long long cap = 2LL * nbHost > 1024 ? 2LL * nbHost : 1024;
        if (ctx->walkListSlot == 0) ctx->walkListSlot = 512;
        if (ctx->walkLists == 1) {
            // P-P and cell slots, a quarter for softened cells: 9 bytes per entry
            const long long maxSlot = (16LL << 30) / (9LL * cap);
            while ((long long)ctx->walkListSlot < ctx->lastListNeed && 2LL * ctx->walkListSlot <= maxSlot)
                ctx->walkListSlot *= 2;
        }
        const size_t need = (size_t)cap * ctx->walkListSlot;
        if (ctx->walkListBuckets < cap || ctx->walkListEntries < need) {
            int rc = tsph_grow(ctx, &ctx->dWalkListPP, need);
            if (!rc) rc = tsph_grow(ctx, &ctx->dWalkListCell, need);
            if (!rc) rc = tsph_grow(ctx, &ctx->dWalkListSoft, need / 4);
            if (!rc) rc = tsph_grow(ctx, &ctx->dWalkListInfo, (size_t)cap);
            if (!rc) rc = tsph_grow(ctx, &ctx->dWalkListFallback, (size_t)cap);
            if (rc) { ctx->walkListBuckets = 0; ctx->walkListEntries = 0; return rc; }
            ctx->walkListBuckets = cap;
            ctx->walkListEntries = need;
        }
    }
    if (ctx->walkListBuckets < nbHost || !ctx->walkListSlot ||
        ctx->walkListEntries < (size_t)nbHost * ctx->walkListSlot)
        return TSPH_OK;
    A.listPP = ctx->dWalkListPP;
    A.listCell = ctx->dWalkListCell;
    A.listSoft = ctx->dWalkListSoft;
    A.listInfo = ctx->dWalkListInfo;
    A.listCap = ctx->walkListSlot;
    A.fallback = ctx->dWalkListFallback;
    // list and evaluation work counters, and the left-over count
    TSPH_CK(cudaMemsetAsync(&ctx->dCnt->listWork, 0, 3 * sizeof(unsigned int), ctx->stream));
    const int blocks = ctx->smCount * LBPS;
    if (nbt == 8) k_walk_lists<8><<<blocks, LWPB * 32, 0, ctx->stream>>>(A);
    else if (nbt == 16) k_walk_lists<16><<<blocks, LWPB * 32, 0, ctx->stream>>>(A);
    else k_walk_lists<32><<<blocks, LWPB * 32, 0, ctx->stream>>>(A);
    TSPH_LAUNCH_CK("k_walk_lists");
    return TSPH_OK;
}

template <typename Real, int NBT, bool HIGH>
static int launch_walk(tsph_ctx *ctx, const WalkArgs &A, int blocks, const char *name) {
    size_t sm = sizeof(WalkSmem<Real, NBT, HIGH>) * WPB;
    if (!ctx->capturing)
        TSPH_CK(cudaFuncSetAttribute(k_walk<Real, NBT, HIGH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)sm));
    if (A.listInfo) {
        // evaluation pass over the stored lists, then the fused walk of the
        // buckets whose lists did not fit
        const size_t se = sizeof(EvalSmem<Real, NBT, HIGH>) * WPB;
        if (!ctx->capturing)
            TSPH_CK(cudaFuncSetAttribute(k_walk_eval<Real, NBT, HIGH>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)se));
        k_walk_eval<Real, NBT, HIGH><<<ctx->smCount * EVAL_BPS(Real, HIGH), WPB * 32, se, ctx->stream>>>(A);
        TSPH_LAUNCH_CK("k_walk_eval");
    }
    k_walk<Real, NBT, HIGH><<<blocks, WPB * 32, sm, ctx->stream>>>(A);
    TSPH_LAUNCH_CK(name);
    return TSPH_OK;
}

// The walk's per-bucket geometry (k_bucket_prep) on stream s.
int tsph_bucket_prep(tsph_ctx *ctx, cudaStream_t s) {
    k_bucket_prep<<<tsph_blocks(ctx->T.nLeaves, 128), 128, 0, s>>>(ctx->T, ctx->P);
    TSPH_LAUNCH_CK("k_bucket_prep");
    return TSPH_OK;
}

int tsph_walk_interact(tsph_ctx *ctx, const tsph_grav_params *gp) {
    if (gp->iOrder < 1 || gp->iOrder > 4) return TSPH_ERR_ARG;
    if (gp->bPeriodic && gp->nReps > 1) return TSPH_ERR_UNSUPPORTED;
    if (gp->nBucket > 32) return TSPH_ERR_UNSUPPORTED;
    WalkConst wc;
    memset(&wc, 0, sizeof(wc));
    int nR = gp->bPeriodic ? gp->nReps : 0;
    int side = 2 * nR + 1;
    wc.nRep = side * side * side;
    wc.selfRep = wc.nRep / 2;
    double L = gp->bPeriodic ? gp->dPeriod : 0.0;
    float offmax = 0.0f;
    double rabs = 0.0;
    for (int ix = -nR, r = 0; ix <= nR; ++ix)
        for (int iy = -nR; iy <= nR; ++iy)
            for (int iz = -nR; iz <= nR; ++iz, ++r) {
                int id[3] = {ix, iy, iz};
                for (int k = 0; k < 3; ++k) {
                    wc.off[r][k] = id[k] * L;
                    wc.offh[r][k] = (float)wc.off[r][k];
                    wc.offl[r][k] = (float)(wc.off[r][k] - (double)wc.offh[r][k]);
                    offmax = fmaxf(offmax, fabsf(wc.offh[r][k]));
                }
            }
    wc.offmax = offmax;
    wc.L = L;
    wc.Lh = (float)L;
    wc.Ll = (float)(L - (double)wc.Lh);
    // absolute error floor of hi/lo coordinates: a few ulp^2 of the largest
    // absolute coordinate (positions + offsets)
    rabs = ctx->dPeriodTree + offmax;
    wc.E0 = (float)(16.0 * 3.552713678800501e-15 * rabs) + 1e-30f;
    // constants are uploaded outside graph capture (a captured step reuses
    // the ones its preparation set)
    if (!ctx->capturing)
        TSPH_CK(cudaMemcpyToSymbolAsync(cW, &wc, sizeof(wc), 0, cudaMemcpyHostToDevice, ctx->stream));

    WalkArgs A;
    A.T = ctx->T;
    A.P = ctx->P;
    A.cnt = ctx->dCnt;
    A.nBuckets = ctx->T.dcnt + 1;
    A.iOrder = gp->iOrder;
    int rc = TSPH_OK;
    const int nbHost = ctx->T.nLeaves;   // exact, or an upper bound while capturing
    A.bucketLists = nullptr;
    if (!ctx->capturing) {
        if (ctx->bucketListCap < nbHost) {
            rc = tsph_grow(ctx, &ctx->dBucketLists, (size_t)4 * nbHost + 64);
            if (rc) return rc;
            ctx->bucketListCap = nbHost;
        }
        A.bucketLists = ctx->dBucketLists;
    }
    // work counter lives in the counters block's pad area
    A.workCounter = (int *)&ctx->dCnt->pad;
    TSPH_CK(cudaMemsetAsync(A.workCounter, 0, sizeof(int), ctx->stream));
    if (ctx->bucketPrepQueued) {   // prepared on the side stream beside the moments
        TSPH_CK(cudaStreamWaitEvent(ctx->stream, ctx->evPrep, 0));
    } else {
        rc = tsph_bucket_prep(ctx, ctx->stream);
        if (rc) return rc;
    }
    const int wbDefault = gp->precision == TSPH_FP32 ? (gp->iOrder >= 3 ? 3 : 5) : 4;
    int blocks = ctx->smCount * (ctx->walkBlocksPerSM > 0 ? ctx->walkBlocksPerSM : wbDefault);
    A.groupFirst = nullptr;
    A.nGroups = nullptr;
    A.groupScratch = nullptr;
    A.groupMax = 0;
    rc = prepare_groups(ctx, A, nbHost, blocks * WPB);
    if (rc) return rc;
    const int nbt = gp->nBucket <= 8 ? 8 : (gp->nBucket <= 16 ? 16 : 32);
    rc = prepare_lists(ctx, A, nbHost, nbt);
    if (rc) return rc;
    if (gp->iOrder >= 3) {   // octopole / hexadecapole cells
        if (gp->precision == TSPH_FP32) {
            if (nbt == 8) rc = launch_walk<float, 8, true>(ctx, A, blocks, "k_walk<float,8,high>");
            else if (nbt == 16) rc = launch_walk<float, 16, true>(ctx, A, blocks, "k_walk<float,16,high>");
            else rc = launch_walk<float, 32, true>(ctx, A, blocks, "k_walk<float,32,high>");
        } else {
            if (nbt == 8) rc = launch_walk<double, 8, true>(ctx, A, blocks, "k_walk<double,8,high>");
            else if (nbt == 16) rc = launch_walk<double, 16, true>(ctx, A, blocks, "k_walk<double,16,high>");
            else rc = launch_walk<double, 32, true>(ctx, A, blocks, "k_walk<double,32,high>");
        }
    } else if (gp->precision == TSPH_FP32) {
        if (nbt == 8) rc = launch_walk<float, 8, false>(ctx, A, blocks, "k_walk<float,8>");
        else if (nbt == 16) rc = launch_walk<float, 16, false>(ctx, A, blocks, "k_walk<float,16>");
        else rc = launch_walk<float, 32, false>(ctx, A, blocks, "k_walk<float,32>");
    } else {
        if (nbt == 8) rc = launch_walk<double, 8, false>(ctx, A, blocks, "k_walk<double,8>");
        else if (nbt == 16) rc = launch_walk<double, 16, false>(ctx, A, blocks, "k_walk<double,16>");
        else rc = launch_walk<double, 32, false>(ctx, A, blocks, "k_walk<double,32>");
    }
    if (rc) return rc;
    return TSPH_OK;
}
