// K5: Ewald periodic correction.
//
// Follows pkdBucketEwald (ewald.c:15-178): for every particle a real-space
// sum over the images (ix,iy,iz) in [-ceil(fEwCut), ceil(fEwCut)]^3 kept when
// r <= fEwCut*L or inside the replica "hole" (the -erf branch, ewald.c:85-125),
// with the small-r series below r^2 < 3e-3 L^2, then a k-space sum over the
// table built by pkdEwaldInit (ewald.c:182-248), all with the complete root
// multipoles of pkdCalcRoot/pkdDistribRoot (pkd.c:4395-4493) evaluated by
// MEVAL (meval.h:21-81).  The table is built on the device in FP64 from
// root moments reduced in a fixed order (deterministic), with no host round
// trip, so periodic evaluations can be captured in a CUDA graph.
// erf/erfc/exp/sin/cos are CUDA's own functions.
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "tsph_ctx.cuh"

#define EW_MAXH 512

// The FP32 kernel's real-space sum stops at alpha r = EW_XCUT_F32 when that
// is nearer than fEwCut L.  An image there contributes at most
// M alpha^2 (erfc(x)/x^2 + 2/sqrt(pi) e^(-x^2)/x) = 1.6e-9 M alpha^2 at
// x = 4.5 (less for the higher moments), falling by 10^2 per 0.5 in x,
// while the hole images add terms of order M alpha^2 / 4 whose FP32
// rounding (2^-24 of each) is of the size of all the left-out terms
// together.  The FP32 error against the FP64 path is measured on the box
// (bench.py) and held to the FP32 bars of the tests.  The FP64 kernel
// keeps the reference's cut, fEwCut, and both count pkdGravAll's Ewald
// flops over the terms within it, as the reference does.
#define EW_XCUT_F32 4.5

// complete root multipoles in the reference's ILCN member order
struct EwMom {
    double m, x, y, z;
    double xx, yy, xy, xz, yz, zz;
    double xxx, xyy, xxy, yyy, xxz, yyz, xyz, xzz, yzz, zzz;
    double xxxx, xyyy, xxxy, yyyy, xxxz, yyyz, xxyy, xxyz, xyyz;
    double xxzz, xyzz, xzzz, yyzz, yzzz, zzzz;
};

#define EW_MAXIMG 343   // (2*3+1)^3 images at fEwCut <= 3

struct EwConst {
    EwMom mom;
    float momf[35];
    double L, alpha, alpha2, k1, ka, fEwCut2, smallR2;
    float fEwCut2f;      // the FP32 kernel's real-space cut (see EW_XCUT_F32)
    // FP32 copies of L, alpha, alpha^2, ka, fEwCut2, smallR2, 2 pi / L and
    // the potential's constant term m k1, converted once here rather than
    // by every thread of the FP32 kernel
    float fL, fAlpha, fAlpha2, fKa, fCut2, fSmallR2, fTwoPiL, fPot0;
    int nEwReps, nReps, nEwh, iOrder;
    int hMax;            // largest |component| of a k-space vector
    int hCut2;           // floor(fEwhCut^2): the integer |h|^2 kept (ewald.c:205-211)
    double hx[EW_MAXH], hy[EW_MAXH], hz[EW_MAXH], hC[EW_MAXH], hS[EW_MAXH];
    // FP32 copies of the k-space table for the FP32 kernel
    float hxf[EW_MAXH], hyf[EW_MAXH], hzf[EW_MAXH], hCf[EW_MAXH], hSf[EW_MAXH];
    // the real-space images (ix, iy, iz, hole) that can pass the cut for
    // some particle of the box: the nHole images of the replica "hole"
    // first, then the others, each in the reference's loop order
    int nImg, nHole;
    char4 img[EW_MAXIMG];
    // FP32 MEVAL coefficients: the moments pre-combined per monomial
    // (c4: hexadecapole mirror over dx^3 .. dz^3, c3: octopole mirror over
    // dx^2 .. dz^2, with MEVAL's 1/6, 1/2 and multiplicities folded in)
    float c4[3][10], hQ[6], qtr4;
    float c3[3][6], q3[3];
    float q2[6], qtr2, m;
};
__constant__ EwConst cE;

// --------------------------------------------------------------------------
// root moments: block partial sums in a fixed order, then a fixed-order sum
// --------------------------------------------------------------------------
#define RM_BS 256
#define RM_NV 25

// Acc = double for the FP64 path; float for the FP32 path, whose kernel
// uses the moments in FP32 anyway (offsets from the COM in FP64, then FP32
// products and sums, FP64 per-block partials).
template <typename Acc>
__global__ void k_root_partial(int n, const double *__restrict__ x, const double *__restrict__ y,
                               const double *__restrict__ z, const double *__restrict__ m,
                               const double *__restrict__ rc, double *partial) {
    __shared__ Acc sh[RM_NV][RM_BS / 32];
    Acc acc[RM_NV];
#pragma unroll
    for (int k = 0; k < RM_NV; ++k) acc[k] = 0;
    double cx = rc[0], cy = rc[1], cz = rc[2];
    for (int p = blockIdx.x * RM_BS + threadIdx.x; p < n; p += gridDim.x * RM_BS) {
        Acc mm = (Acc)m[p], dx = (Acc)(x[p] - cx), dy = (Acc)(y[p] - cy), dz = (Acc)(z[p] - cz);
        Acc dx2 = dx * dx, dy2 = dy * dy, dz2 = dz * dz;
        // hexadecapole (complete): xxxx xyyy xxxy yyyy xxxz yyyz xxyy xxyz xyyz xxzz xyzz xzzz yyzz yzzz zzzz
        acc[0] += mm * dx2 * dx2;
        acc[1] += mm * dx * dy2 * dy;
        acc[2] += mm * dx2 * dx * dy;
        acc[3] += mm * dy2 * dy2;
        acc[4] += mm * dx2 * dx * dz;
        acc[5] += mm * dy2 * dy * dz;
        acc[6] += mm * dx2 * dy2;
        acc[7] += mm * dx2 * dy * dz;
        acc[8] += mm * dx * dy2 * dz;
        acc[9] += mm * dx2 * dz2;
        acc[10] += mm * dx * dy * dz2;
        acc[11] += mm * dx * dz2 * dz;
        acc[12] += mm * dy2 * dz2;
        acc[13] += mm * dy * dz2 * dz;
        acc[14] += mm * dz2 * dz2;
        // octopole (complete): xxx xyy xxy yyy xxz yyz xyz xzz yzz zzz
        acc[15] += mm * dx2 * dx;
        acc[16] += mm * dx * dy2;
        acc[17] += mm * dx2 * dy;
        acc[18] += mm * dy2 * dy;
        acc[19] += mm * dx2 * dz;
        acc[20] += mm * dy2 * dz;
        acc[21] += mm * dx * dy * dz;
        acc[22] += mm * dx * dz2;
        acc[23] += mm * dy * dz2;
        acc[24] += mm * dz2 * dz;
    }
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < RM_NV; ++k) {
        Acc v = acc[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) sh[k][w] = v;
    }
    __syncthreads();
    if (threadIdx.x < RM_NV) {
        double v = 0.0;
        for (int j = 0; j < RM_BS / 32; ++j) v += (double)sh[threadIdx.x][j];
        partial[blockIdx.x * RM_NV + threadIdx.x] = v;
    }
}

__global__ void k_root_final(int nb, const double *__restrict__ partial, double *out) {
    int k = threadIdx.x;
    if (k >= RM_NV) return;
    double v = 0.0;
    for (int b = 0; b < nb; ++b) v += partial[b * RM_NV + k];
    out[k] = v;
}

// --------------------------------------------------------------------------
// MEVAL and the per-particle Ewald kernel
// --------------------------------------------------------------------------
template <typename Real>
struct MomR {
    Real m, xx, yy, xy, xz, yz, zz;
    Real xxx, xyy, xxy, yyy, xxz, yyz, xyz, xzz, yzz, zzz;
    Real xxxx, xyyy, xxxy, yyyy, xxxz, yyyz, xxyy, xxyz, xyyz, xxzz, xyzz, xzzz, yyzz, yzzz, zzzz;
};

template <typename Real>
__device__ __forceinline__ void load_mom(MomR<Real> &M) {
    if (sizeof(Real) == 8) {
        const EwMom &e = cE.mom;
        M.m = e.m; M.xx = e.xx; M.yy = e.yy; M.xy = e.xy; M.xz = e.xz; M.yz = e.yz; M.zz = e.zz;
        M.xxx = e.xxx; M.xyy = e.xyy; M.xxy = e.xxy; M.yyy = e.yyy; M.xxz = e.xxz; M.yyz = e.yyz;
        M.xyz = e.xyz; M.xzz = e.xzz; M.yzz = e.yzz; M.zzz = e.zzz;
        M.xxxx = e.xxxx; M.xyyy = e.xyyy; M.xxxy = e.xxxy; M.yyyy = e.yyyy; M.xxxz = e.xxxz;
        M.yyyz = e.yyyz; M.xxyy = e.xxyy; M.xxyz = e.xxyz; M.xyyz = e.xyyz; M.xxzz = e.xxzz;
        M.xyzz = e.xyzz; M.xzzz = e.xzzz; M.yyzz = e.yyzz; M.yzzz = e.yzzz; M.zzzz = e.zzzz;
    } else {
        const float *f = cE.momf;
        M.m = f[0]; M.xx = f[4]; M.yy = f[5]; M.xy = f[6]; M.xz = f[7]; M.yz = f[8]; M.zz = f[9];
        M.xxx = f[10]; M.xyy = f[11]; M.xxy = f[12]; M.yyy = f[13]; M.xxz = f[14]; M.yyz = f[15];
        M.xyz = f[16]; M.xzz = f[17]; M.yzz = f[18]; M.zzz = f[19];
        M.xxxx = f[20]; M.xyyy = f[21]; M.xxxy = f[22]; M.yyyy = f[23]; M.xxxz = f[24];
        M.yyyz = f[25]; M.xxyy = f[26]; M.xxyz = f[27]; M.xyyz = f[28]; M.xxzz = f[29];
        M.xyzz = f[30]; M.xzzz = f[31]; M.yyzz = f[32]; M.yzzz = f[33]; M.zzzz = f[34];
    }
}

template <typename Real>
__device__ __forceinline__ void meval(int iOrder, const MomR<Real> &mom, const Real *gam, Real dx,
                                      Real dy, Real dz, Real &ax, Real &ay, Real &az, Real &fPot) {
    Real Qmirx, Qmiry, Qmirz, Qmir, Qta = 0;
    if (iOrder >= 4) {
        Qmirx = Real(1.0 / 6.0) * (mom.xzzz * dz * dz * dz + 3 * mom.xyzz * dy * dz * dz + 3 * mom.xyyz * dy * dy * dz + mom.xyyy * dy * dy * dy + 3 * mom.xxzz * dx * dz * dz + 6 * mom.xxyz * dx * dy * dz + 3 * mom.xxyy * dx * dy * dy + 3 * mom.xxxz * dx * dx * dz + 3 * mom.xxxy * dx * dx * dy + mom.xxxx * dx * dx * dx);
        Qmiry = Real(1.0 / 6.0) * (mom.yzzz * dz * dz * dz + 3 * mom.xyzz * dx * dz * dz + 3 * mom.xxyz * dx * dx * dz + mom.xxxy * dx * dx * dx + 3 * mom.yyzz * dy * dz * dz + 6 * mom.xyyz * dx * dy * dz + 3 * mom.xxyy * dx * dx * dy + 3 * mom.yyyz * dy * dy * dz + 3 * mom.xyyy * dx * dy * dy + mom.yyyy * dy * dy * dy);
        Qmirz = Real(1.0 / 6.0) * (mom.yyyz * dy * dy * dy + 3 * mom.xyyz * dx * dy * dy + 3 * mom.xxyz * dx * dx * dy + mom.xxxz * dx * dx * dx + 3 * mom.yyzz * dy * dy * dz + 6 * mom.xyzz * dx * dy * dz + 3 * mom.xxzz * dx * dx * dz + 3 * mom.yzzz * dy * dz * dz + 3 * mom.xzzz * dx * dz * dz + mom.zzzz * dz * dz * dz);
        Qmir = Real(0.25) * (Qmirx * dx + Qmiry * dy + Qmirz * dz);
        Real Qxx = mom.xxxx + mom.xxyy + mom.xxzz;
        Real Qxy = mom.xxxy + mom.xyyy + mom.xyzz;
        Real Qxz = mom.xxxz + mom.xyyz + mom.xzzz;
        Real Qyy = mom.xxyy + mom.yyyy + mom.yyzz;
        Real Qyz = mom.xxyz + mom.yyyz + mom.yzzz;
        Real Qzz = mom.xxzz + mom.yyzz + mom.zzzz;
        Real Qtr = Real(0.125) * (Qxx + Qyy + Qzz);
        Real Qhx = Real(0.5) * (Qxx * dx + Qxy * dy + Qxz * dz);
        Real Qhy = Real(0.5) * (Qxy * dx + Qyy * dy + Qyz * dz);
        Real Qhz = Real(0.5) * (Qxz * dx + Qyz * dy + Qzz * dz);
        Real Qh = Real(0.5) * (Qhx * dx + Qhy * dy + Qhz * dz);
        fPot -= gam[4] * Qmir - gam[3] * Qh + gam[2] * Qtr;
        Qta += gam[5] * Qmir - gam[4] * Qh + gam[3] * Qtr;
        ax += gam[4] * Qmirx - gam[3] * Qhx;
        ay += gam[4] * Qmiry - gam[3] * Qhy;
        az += gam[4] * Qmirz - gam[3] * Qhz;
    }
    if (iOrder >= 3) {
        Qmirx = Real(0.5) * (mom.xzz * dz * dz + 2 * mom.xyz * dy * dz + mom.xyy * dy * dy + 2 * mom.xxz * dx * dz + 2 * mom.xxy * dx * dy + mom.xxx * dx * dx);
        Qmiry = Real(0.5) * (mom.yzz * dz * dz + 2 * mom.xyz * dx * dz + mom.xxy * dx * dx + 2 * mom.yyz * dy * dz + 2 * mom.xyy * dx * dy + mom.yyy * dy * dy);
        Qmirz = Real(0.5) * (mom.yyz * dy * dy + 2 * mom.xyz * dx * dy + mom.xxz * dx * dx + 2 * mom.yzz * dy * dz + 2 * mom.xzz * dx * dz + mom.zzz * dz * dz);
        Qmir = Real(1.0 / 3.0) * (Qmirx * dx + Qmiry * dy + Qmirz * dz);
        Real Qx = Real(0.5) * (mom.xxx + mom.xyy + mom.xzz);
        Real Qy = Real(0.5) * (mom.xxy + mom.yyy + mom.yzz);
        Real Qz = Real(0.5) * (mom.xxz + mom.yyz + mom.zzz);
        Real Qtr = Qx * dx + Qy * dy + Qz * dz;
        fPot -= gam[3] * Qmir - gam[2] * Qtr;
        Qta += gam[4] * Qmir - gam[3] * Qtr;
        ax += gam[3] * Qmirx - gam[2] * Qx;
        ay += gam[3] * Qmiry - gam[2] * Qy;
        az += gam[3] * Qmirz - gam[2] * Qz;
    }
    if (iOrder >= 2) {
        Qmirx = mom.xz * dz + mom.xy * dy + mom.xx * dx;
        Qmiry = mom.yz * dz + mom.xy * dx + mom.yy * dy;
        Qmirz = mom.yz * dy + mom.xz * dx + mom.zz * dz;
        Qmir = Real(0.5) * (Qmirx * dx + Qmiry * dy + Qmirz * dz);
        Real Qtr = Real(0.5) * (mom.xx + mom.yy + mom.zz);
        fPot -= gam[2] * Qmir - gam[1] * Qtr;
        Qta += gam[3] * Qmir - gam[2] * Qtr;
        ax += gam[2] * Qmirx;
        ay += gam[2] * Qmiry;
        az += gam[2] * Qmirz;
    }
    fPot -= gam[0] * mom.m;
    Qta += gam[1] * mom.m;
    ax -= dx * Qta;
    ay -= dy * Qta;
    az -= dz * Qta;
}

// MEVAL (meval.h:21-81) in FP32 from the pre-combined coefficients: the
// same terms, each multipole's mirror a dot product over the monomials of
// (dx, dy, dz) formed once.
__device__ __forceinline__ void meval_f32(int iOrder, const float *gam, float dx, float dy, float dz,
                                          float &ax, float &ay, float &az, float &fPot) {
    float Qta = 0.0f;
    const float xx2 = dx * dx, xy2 = dx * dy, xz2 = dx * dz, yy2 = dy * dy, yz2 = dy * dz,
                zz2 = dz * dz;
    if (iOrder >= 4) {
        const float m3[10] = {xx2 * dx, xx2 * dy, xx2 * dz, yy2 * dx, xy2 * dz,
                              zz2 * dx, yy2 * dy, yy2 * dz, zz2 * dy, zz2 * dz};
        float Qmx = 0.0f, Qmy = 0.0f, Qmz = 0.0f;
#pragma unroll
        for (int k = 0; k < 10; ++k) {
            Qmx += cE.c4[0][k] * m3[k];
            Qmy += cE.c4[1][k] * m3[k];
            Qmz += cE.c4[2][k] * m3[k];
        }
        const float Qmir = 0.25f * (Qmx * dx + Qmy * dy + Qmz * dz);
        const float Qhx = cE.hQ[0] * dx + cE.hQ[1] * dy + cE.hQ[2] * dz;
        const float Qhy = cE.hQ[1] * dx + cE.hQ[3] * dy + cE.hQ[4] * dz;
        const float Qhz = cE.hQ[2] * dx + cE.hQ[4] * dy + cE.hQ[5] * dz;
        const float Qh = 0.5f * (Qhx * dx + Qhy * dy + Qhz * dz);
        fPot -= gam[4] * Qmir - gam[3] * Qh + gam[2] * cE.qtr4;
        Qta += gam[5] * Qmir - gam[4] * Qh + gam[3] * cE.qtr4;
        ax += gam[4] * Qmx - gam[3] * Qhx;
        ay += gam[4] * Qmy - gam[3] * Qhy;
        az += gam[4] * Qmz - gam[3] * Qhz;
    }
    if (iOrder >= 3) {
        const float m2[6] = {xx2, xy2, xz2, yy2, yz2, zz2};
        float Qmx = 0.0f, Qmy = 0.0f, Qmz = 0.0f;
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            Qmx += cE.c3[0][k] * m2[k];
            Qmy += cE.c3[1][k] * m2[k];
            Qmz += cE.c3[2][k] * m2[k];
        }
        const float Qmir = (1.0f / 3.0f) * (Qmx * dx + Qmy * dy + Qmz * dz);
        const float Qtr = cE.q3[0] * dx + cE.q3[1] * dy + cE.q3[2] * dz;
        fPot -= gam[3] * Qmir - gam[2] * Qtr;
        Qta += gam[4] * Qmir - gam[3] * Qtr;
        ax += gam[3] * Qmx - gam[2] * cE.q3[0];
        ay += gam[3] * Qmy - gam[2] * cE.q3[1];
        az += gam[3] * Qmz - gam[2] * cE.q3[2];
    }
    if (iOrder >= 2) {
        const float *q = cE.q2;            // xx yy zz xy xz yz
        const float Qmx = q[4] * dz + q[3] * dy + q[0] * dx;
        const float Qmy = q[5] * dz + q[3] * dx + q[1] * dy;
        const float Qmz = q[5] * dy + q[4] * dx + q[2] * dz;
        const float Qmir = 0.5f * (Qmx * dx + Qmy * dy + Qmz * dz);
        fPot -= gam[2] * Qmir - gam[1] * cE.qtr2;
        Qta += gam[3] * Qmir - gam[2] * cE.qtr2;
        ax += gam[2] * Qmx;
        ay += gam[2] * Qmy;
        az += gam[2] * Qmz;
    }
    fPot -= gam[0] * cE.m;
    Qta += gam[1] * cE.m;
    ax -= dx * Qta;
    ay -= dy * Qta;
    az -= dz * Qta;
}

__device__ __forceinline__ float erf_r(float x) { return erff(x); }
__device__ __forceinline__ double erf_r(double x) { return erf(x); }
__device__ __forceinline__ float erfc_r(float x) { return erfcf(x); }
__device__ __forceinline__ double erfc_r(double x) { return erfc(x); }
__device__ __forceinline__ float exp_r(float x) { return expf(x); }
__device__ __forceinline__ double exp_r(double x) { return exp(x); }
__device__ __forceinline__ float sqrt_r(float x) { return sqrtf(x); }
__device__ __forceinline__ double sqrt_r(double x) { return sqrt(x); }
__device__ __forceinline__ void sincos_r(float x, float *s, float *c) { sincosf(x, s, c); }
__device__ __forceinline__ void sincos_r(double x, double *s, double *c) { sincos(x, s, c); }

// Kahan addition in FP32 (the Ewald terms are O(1) and cancel against the
// replica part of the tree walk); plain addition in FP64.
__device__ __forceinline__ void kadd(float &s, float &c, float v) {
    float y = v - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
}
__device__ __forceinline__ void kadd(double &s, double &c, double v) { s += v; (void)c; }

// gam_0..5 of one real-space image at squared distance r2 (the g_n of
// pkdBucketEwald, ewald.c:85-125): images of the replica "hole" carry
// -erf(alpha r), the others erfc(alpha r).
template <typename Real, bool HOLE>
__device__ __forceinline__ void ewald_gam(Real r2, Real alpha, Real alpha2, Real ka, Real smallR2,
                                          Real *gam) {
    if (sizeof(Real) == 4 && HOLE && r2 * alpha2 < Real(4.0)) {
        // FP32: the recurrence below cancels catastrophically for a
        // hole image at small alpha*r.  With u = alpha^2 r^2,
        //   gam_n = -ka (2 alpha^2)^n S_n(u),
        //   S_n(u) = sum_j (-u)^j/(j!(2j+2n+1)) = int_0^1 t^2n e^(-u t^2) dt
        //          = e^-u T_n(u),  T_n = sum_j (2u)^j / prod_{i<=j}(2n+2i+1),
        // a series of positive terms; T_5 is summed directly and the
        // stable downward recurrence T_n = (2u T_{n+1} + 1)/(2n+1)
        // gives the rest (max rel. error ~2e-7 for u < 4).
        // The reference's small-r branch is the first two terms of S_n.
        Real u = r2 * alpha2, tu = 2 * u;
        Real t = Real(1.0 / 11.0), T5 = t;
#pragma unroll
        for (int j = 1; j < 14; ++j) {
            t *= tu * Real(1.0 / (11 + 2 * j));   // constant reciprocals: no divisions
            T5 += t;
        }
        Real T[6];
        T[5] = T5;
#pragma unroll
        for (int q = 4; q >= 0; --q) T[q] = (tu * T[q + 1] + 1) * Real(1.0 / (2 * q + 1));
        Real pre = -ka * exp_r(-u);
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            gam[q] = pre * T[q];
            pre *= 2 * alpha2;
        }
    } else if (r2 < smallR2) {
        Real alphan = ka;
        Real s = r2 * alpha2;
        gam[0] = alphan * (s / 3 - 1);
        alphan *= 2 * alpha2;
        gam[1] = alphan * (s / 5 - Real(1.0 / 3.0));
        alphan *= 2 * alpha2;
        gam[2] = alphan * (s / 7 - Real(1.0 / 5.0));
        alphan *= 2 * alpha2;
        gam[3] = alphan * (s / 9 - Real(1.0 / 7.0));
        alphan *= 2 * alpha2;
        gam[4] = alphan * (s / 11 - Real(1.0 / 9.0));
        alphan *= 2 * alpha2;
        gam[5] = alphan * (s / 13 - Real(1.0 / 11.0));
    } else {
        Real r, dir;
        if constexpr (sizeof(Real) == 4) {
            // FP32: 1/r from the hardware reciprocal square root (a few ulp,
            // far inside the FP32 path's error)
            dir = rsqrtf(r2);
            r = r2 * dir;
        } else {
            r = sqrt_r(r2);
            dir = Real(1) / r;
        }
        Real dir2 = dir * dir;
        Real a = exp_r(-r2 * alpha2);
        a *= ka * dir2;
        gam[0] = HOLE ? -erf_r(alpha * r) : erfc_r(alpha * r);
        gam[0] *= dir;
        gam[1] = gam[0] * dir2 + a;
        Real alphan = 2 * alpha2;
        gam[2] = 3 * gam[1] * dir2 + alphan * a;
        alphan *= 2 * alpha2;
        gam[3] = 5 * gam[2] * dir2 + alphan * a;
        alphan *= 2 * alpha2;
        gam[4] = 7 * gam[3] * dir2 + alphan * a;
        alphan *= 2 * alpha2;
        gam[5] = 9 * gam[4] * dir2 + alphan * a;
    }
}

template <typename Real>
__global__ void __launch_bounds__(128) k_ewald(TsphDevParts P, TsphDevCounters *cnt) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long nLoop = 0;
    if (p < P.n && P.act[p]) {   // active particles only (pkdBucketEwald, ewald.c:53)
        MomR<Real> mom;
        load_mom<Real>(mom);
        constexpr bool F32 = sizeof(Real) == 4;
        const Real L = F32 ? (Real)cE.fL : (Real)cE.L;
        const Real alpha2 = F32 ? (Real)cE.fAlpha2 : (Real)cE.alpha2;
        const Real alpha = F32 ? (Real)cE.fAlpha : (Real)cE.alpha;
        const Real ka = F32 ? (Real)cE.fKa : (Real)cE.ka;
        const Real fEwCut2 = F32 ? (Real)cE.fCut2 : (Real)cE.fEwCut2;
        const Real smallR2 = F32 ? (Real)cE.fSmallR2 : (Real)cE.smallR2;
        const Real evalCut2 = F32 ? (Real)cE.fEwCut2f : fEwCut2;
        const int iOrder = cE.iOrder;
        Real fPot = F32 ? (Real)cE.fPot0 : (Real)(cE.mom.m * cE.k1), ax = 0, ay = 0, az = 0;
        Real cpot = 0, cax = 0, cay = 0, caz = 0;   // compensations (FP32 only)
        Real dx = (Real)(P.x[p] - cE.mom.x);
        Real dy = (Real)(P.y[p] - cE.mom.y);
        Real dz = (Real)(P.z[p] - cE.mom.z);
        // the hole images (always kept), then the others within the cut
        for (int q = 0; q < cE.nHole; ++q) {
            const char4 im = cE.img[q];
            const Real dxo = dx + im.x * L, dyo = dy + im.y * L, dzo = dz + im.z * L;
            const Real r2 = dxo * dxo + dyo * dyo + dzo * dzo;
            Real gam[6];
            ewald_gam<Real, true>(r2, alpha, alpha2, ka, smallR2, gam);
            Real tx = 0, ty = 0, tz = 0, tp = 0;
            if constexpr (sizeof(Real) == 4) meval_f32(iOrder, gam, dxo, dyo, dzo, tx, ty, tz, tp);
            else meval<Real>(iOrder, mom, gam, dxo, dyo, dzo, tx, ty, tz, tp);
            kadd(ax, cax, tx);
            kadd(ay, cay, ty);
            kadd(az, caz, tz);
            kadd(fPot, cpot, tp);
            ++nLoop;
        }
        for (int q = cE.nHole; q < cE.nImg; ++q) {
            const char4 im = cE.img[q];
            const Real dxo = dx + im.x * L, dyo = dy + im.y * L, dzo = dz + im.z * L;
            const Real r2 = dxo * dxo + dyo * dyo + dzo * dzo;
            if (r2 > fEwCut2) continue;
            ++nLoop;   // pkdGravAll's flop count follows the reference's cut
            if (r2 > evalCut2) continue;
            Real gam[6];
            ewald_gam<Real, false>(r2, alpha, alpha2, ka, smallR2, gam);
            Real tx = 0, ty = 0, tz = 0, tp = 0;
            if constexpr (sizeof(Real) == 4) meval_f32(iOrder, gam, dxo, dyo, dzo, tx, ty, tz, tp);
            else meval<Real>(iOrder, mom, gam, dxo, dyo, dzo, tx, ty, tz, tp);
            kadd(ax, cax, tx);
            kadd(ay, cay, ty);
            kadd(az, caz, tz);
            kadd(fPot, cpot, tp);
        }
        if (sizeof(Real) == 4 && cE.hMax <= 3) {
            // FP32: e^{i h.x} of every kept k-space vector from the three
            // phase factors e^{i 2 pi x/L}, e^{i 2 pi y/L}, e^{i 2 pi z/L} by
            // complex products, in the table's order (hx, hy, hz ascending) --
            // three sincos per particle instead of one per vector.  The z
            // factors e^{i k 2 pi z/L}, |k| <= 3, are tabulated; a row (hx, hy)
            // outside the cut is skipped and a row inside it visits only its
            // kept hz.
            const float tp = cE.fTwoPiL;
            float c1[3], s1[3];
            sincosf(tp * (float)dx, &s1[0], &c1[0]);
            sincosf(tp * (float)dy, &s1[1], &c1[1]);
            sincosf(tp * (float)dz, &s1[2], &c1[2]);
            const int R = cE.hMax;
            float czt[7], szt[7];   // e^{i k theta_z} at index k + 3
            czt[3] = 1.0f;
            szt[3] = 0.0f;
#pragma unroll
            for (int k = 1; k <= 3; ++k) {
                czt[3 + k] = czt[2 + k] * c1[2] - szt[2 + k] * s1[2];
                szt[3 + k] = czt[2 + k] * s1[2] + szt[2 + k] * c1[2];
                czt[3 - k] = czt[3 + k];
                szt[3 - k] = -szt[3 + k];
            }
            // e^{-i R theta} for x and y
            float cs0[2], sn0[2];
#pragma unroll
            for (int a = 0; a < 2; ++a) {
                float c = 1.0f, s = 0.0f;
                for (int k = 0; k < R; ++k) {
                    const float t = c * c1[a] + s * s1[a];   // times e^{-i theta}
                    s = s * c1[a] - c * s1[a];
                    c = t;
                }
                cs0[a] = c;
                sn0[a] = s;
            }
            const int cut2 = cE.hCut2;
            int i = 0;
            float cx = cs0[0], sx = sn0[0];
            for (int ix = -R; ix <= R; ++ix) {
                float cy = cs0[1], sy = sn0[1];
                for (int iy = -R; iy <= R; ++iy) {
                    const int rem = cut2 - ix * ix - iy * iy;
                    if (rem >= 0) {
                        const float cxy = cx * cy - sx * sy, sxy = cx * sy + sx * cy;
#pragma unroll
                        for (int iz = -3; iz <= 3; ++iz) {
                            if (iz >= -R && iz <= R && iz * iz <= rem && (ix | iy | iz) != 0) {
                                const float c = cxy * czt[3 + iz] - sxy * szt[3 + iz];
                                const float s = cxy * szt[3 + iz] + sxy * czt[3 + iz];
                                const float hC = cE.hCf[i], hS = cE.hSf[i];
                                kadd(fPot, cpot, (Real)(hC * c + hS * s));
                                const float t = hC * s - hS * c;
                                kadd(ax, cax, (Real)(cE.hxf[i] * t));
                                kadd(ay, cay, (Real)(cE.hyf[i] * t));
                                kadd(az, caz, (Real)(cE.hzf[i] * t));
                                ++i;
                            }
                        }
                    }
                    const float t = cy * c1[1] - sy * s1[1];
                    sy = cy * s1[1] + sy * c1[1];
                    cy = t;
                }
                const float t = cx * c1[0] - sx * s1[0];
                sx = cx * s1[0] + sx * c1[0];
                cx = t;
            }
        } else {
            for (int i = 0; i < cE.nEwh; ++i) {
                Real hx, hy, hz, hC, hS;
                if constexpr (sizeof(Real) == 4) {
                    hx = cE.hxf[i]; hy = cE.hyf[i]; hz = cE.hzf[i]; hC = cE.hCf[i]; hS = cE.hSf[i];
                } else {
                    hx = cE.hx[i]; hy = cE.hy[i]; hz = cE.hz[i]; hC = cE.hC[i]; hS = cE.hS[i];
                }
                Real hdotx = hx * dx + hy * dy + hz * dz;
                Real s, c;
                sincos_r(hdotx, &s, &c);
                kadd(fPot, cpot, hC * c + hS * s);
                Real t = hC * s - hS * c;
                kadd(ax, cax, hx * t);
                kadd(ay, cay, hy * t);
                kadd(az, caz, hz * t);
            }
        }
        if constexpr (sizeof(Real) == 4) {
            // walk (compensated FP32 pair) + Ewald (compensated FP32 pair), in FP64
            float4 ws = P.wsum[p], wc = P.wcmp[p];
            P.ax[p] = ((double)ws.x - (double)wc.x) + ((double)ax - (double)cax);
            P.ay[p] = ((double)ws.y - (double)wc.y) + ((double)ay - (double)cay);
            P.az[p] = ((double)ws.z - (double)wc.z) + ((double)az - (double)caz);
            P.pot[p] = ((double)ws.w - (double)wc.w) + ((double)fPot - (double)cpot);
            P.dtGrav[p] = (double)P.wdt[p];
        } else {
            P.pot[p] += (double)fPot;
            P.ax[p] += (double)ax;
            P.ay[p] += (double)ay;
            P.az[p] += (double)az;
        }
    }
    // count real-space terms
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) nLoop += __shfl_xor_sync(0xffffffffu, nLoop, o);
    if ((threadIdx.x & 31) == 0 && nLoop) atomicAdd(&cnt->nEwLoop, nLoop);
}

// --------------------------------------------------------------------------
// The constants on the device: QEVAL for the k-space table (qeval.h:21-64),
// the arithmetic of the reference's pkdEwaldInit (ewald.c:182-248)
// --------------------------------------------------------------------------
__device__ void qeval_h(int iOrder, const EwMom &mom, const double *gam, double dx, double dy,
                        double dz, double *fPot) {
    double Qmirx, Qmiry, Qmirz, Qmir;
    if (iOrder >= 4) {
        Qmirx = (1.0 / 6.0) * (mom.xzzz * dz * dz * dz + 3 * mom.xyzz * dy * dz * dz + 3 * mom.xyyz * dy * dy * dz + mom.xyyy * dy * dy * dy + 3 * mom.xxzz * dx * dz * dz + 6 * mom.xxyz * dx * dy * dz + 3 * mom.xxyy * dx * dy * dy + 3 * mom.xxxz * dx * dx * dz + 3 * mom.xxxy * dx * dx * dy + mom.xxxx * dx * dx * dx);
        Qmiry = (1.0 / 6.0) * (mom.yzzz * dz * dz * dz + 3 * mom.xyzz * dx * dz * dz + 3 * mom.xxyz * dx * dx * dz + mom.xxxy * dx * dx * dx + 3 * mom.yyzz * dy * dz * dz + 6 * mom.xyyz * dx * dy * dz + 3 * mom.xxyy * dx * dx * dy + 3 * mom.yyyz * dy * dy * dz + 3 * mom.xyyy * dx * dy * dy + mom.yyyy * dy * dy * dy);
        Qmirz = (1.0 / 6.0) * (mom.yyyz * dy * dy * dy + 3 * mom.xyyz * dx * dy * dy + 3 * mom.xxyz * dx * dx * dy + mom.xxxz * dx * dx * dx + 3 * mom.yyzz * dy * dy * dz + 6 * mom.xyzz * dx * dy * dz + 3 * mom.xxzz * dx * dx * dz + 3 * mom.yzzz * dy * dz * dz + 3 * mom.xzzz * dx * dz * dz + mom.zzzz * dz * dz * dz);
        Qmir = (1.0 / 4.0) * (Qmirx * dx + Qmiry * dy + Qmirz * dz);
        *fPot -= gam[4] * Qmir;
    }
    if (iOrder >= 3) {
        Qmirx = (1.0 / 2.0) * (mom.xzz * dz * dz + 2 * mom.xyz * dy * dz + mom.xyy * dy * dy + 2 * mom.xxz * dx * dz + 2 * mom.xxy * dx * dy + mom.xxx * dx * dx);
        Qmiry = (1.0 / 2.0) * (mom.yzz * dz * dz + 2 * mom.xyz * dx * dz + mom.xxy * dx * dx + 2 * mom.yyz * dy * dz + 2 * mom.xyy * dx * dy + mom.yyy * dy * dy);
        Qmirz = (1.0 / 2.0) * (mom.yyz * dy * dy + 2 * mom.xyz * dx * dy + mom.xxz * dx * dx + 2 * mom.yzz * dy * dz + 2 * mom.xzz * dx * dz + mom.zzz * dz * dz);
        Qmir = (1.0 / 3.0) * (Qmirx * dx + Qmiry * dy + Qmirz * dz);
        *fPot -= gam[3] * Qmir;
    }
    if (iOrder >= 2) {
        Qmirx = (1.0 / 1.0) * (mom.xz * dz + mom.xy * dy + mom.xx * dx);
        Qmiry = (1.0 / 1.0) * (mom.yz * dz + mom.xy * dx + mom.yy * dy);
        Qmirz = (1.0 / 1.0) * (mom.yz * dy + mom.xz * dx + mom.zz * dz);
        Qmir = (1.0 / 2.0) * (Qmirx * dx + Qmiry * dy + Qmirz * dz);
        *fPot -= gam[2] * Qmir;
    }
    *fPot -= gam[0] * mom.m;
}

// parameters of one Ewald evaluation (the caller's tsph_grav_params)
struct EwParams {
    double L, fEwCut, fEwhCut;
    int nReps, nEwReps, iOrder, hReps;
};

#define EWC_BS 512

// The exclusive rank of this thread's `keep` among the block's threads in
// thread order, and the block's total; every thread of the block calls it.
__device__ __forceinline__ int block_rank(bool keep, int *shw, int *total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned b = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) shw[w] = __popc(b);
    __syncthreads();
    int off = 0, tot = 0;
    for (int k = 0; k < EWC_BS / 32; ++k) {
        const int v = shw[k];
        off += k < w ? v : 0;
        tot += v;
    }
    __syncthreads();
    *total = tot;
    return off + __popc(b & ((1u << lane) - 1u));
}

// One block builds every Ewald constant from the root moments left by
// k_root_final (octopole, hexadecapole), the root cell (mass, centre of
// mass, complete quadrupole; pkdDistribRoot, pkd.c:4472-4493) and the
// particles' largest |coordinate| (the gather's, in cnt): the MEVAL
// coefficients, the k-space table in the reference's loop order, and the
// real-space images.  Nothing goes through the host, so a periodic
// evaluation can be captured in a CUDA graph.  The host has checked that
// the table and the image list fit (tsph_ewald_roots).
__global__ void __launch_bounds__(EWC_BS) k_ewald_const(EwParams p, const double *__restrict__ root,
                                                        TsphDevTree T, const TsphDevCounters *cnt,
                                                        EwConst *out) {
    __shared__ EwMom M;
    __shared__ int shw[EWC_BS / 32];
    __shared__ double ext;
    EwConst &E = *out;
    {   // clear the block: unused table entries read as zeros
        unsigned *w = reinterpret_cast<unsigned *>(out);
        for (size_t i = threadIdx.x; i < sizeof(EwConst) / sizeof(unsigned); i += EWC_BS) w[i] = 0u;
    }
    if (threadIdx.x == 0) {
        const double *h = root;   // xxxx xyyy xxxy yyyy xxxz yyyz xxyy xxyz xyyz xxzz xyzz xzzz yyzz yzzz zzzz, xxx ... zzz
        M.xxxx = h[0]; M.xyyy = h[1]; M.xxxy = h[2]; M.yyyy = h[3]; M.xxxz = h[4]; M.yyyz = h[5];
        M.xxyy = h[6]; M.xxyz = h[7]; M.xyyz = h[8]; M.xxzz = h[9]; M.xyzz = h[10]; M.xzzz = h[11];
        M.yyzz = h[12]; M.yzzz = h[13]; M.zzzz = h[14];
        M.xxx = h[15]; M.xyy = h[16]; M.xxy = h[17]; M.yyy = h[18]; M.xxz = h[19]; M.yyz = h[20];
        M.xyz = h[21]; M.xzz = h[22]; M.yzz = h[23]; M.zzz = h[24];
        M.m = T.fMass[0];
        M.x = T.r[0]; M.y = T.r[1]; M.z = T.r[2];
        M.xx = T.Q[0]; M.yy = T.Q[1]; M.zz = T.Q[2];
        M.xy = T.Q[3]; M.xz = T.Q[4]; M.yz = T.Q[5];
        double e = __longlong_as_double((long long)cnt->maxAbs);
        ext = e < 0.5 * p.L ? 0.5 * p.L : e;
    }
    __syncthreads();
    const double L = p.L;
    if (threadIdx.x == 0) {
        E.mom = M;
        const double *mv = &M.m;
        for (int k = 0; k < 35; ++k) E.momf[k] = (float)mv[k];
        // FP32 MEVAL coefficients (monomials dx3 dx2dy dx2dz dxdy2 dxdydz dxdz2 dy3 dy2dz dydz2 dz3)
        const double s6 = 1.0 / 6.0;
        const double c4[3][10] = {
            {M.xxxx, 3 * M.xxxy, 3 * M.xxxz, 3 * M.xxyy, 6 * M.xxyz, 3 * M.xxzz, M.xyyy, 3 * M.xyyz, 3 * M.xyzz, M.xzzz},
            {M.xxxy, 3 * M.xxyy, 3 * M.xxyz, 3 * M.xyyy, 6 * M.xyyz, 3 * M.xyzz, M.yyyy, 3 * M.yyyz, 3 * M.yyzz, M.yzzz},
            {M.xxxz, 3 * M.xxyz, 3 * M.xxzz, 3 * M.xyyz, 6 * M.xyzz, 3 * M.xzzz, M.yyyz, 3 * M.yyzz, 3 * M.yzzz, M.zzzz}};
        for (int a = 0; a < 3; ++a)
            for (int k = 0; k < 10; ++k) E.c4[a][k] = (float)(s6 * c4[a][k]);
        const double Qxx = M.xxxx + M.xxyy + M.xxzz, Qxy = M.xxxy + M.xyyy + M.xyzz,
                     Qxz = M.xxxz + M.xyyz + M.xzzz, Qyy = M.xxyy + M.yyyy + M.yyzz,
                     Qyz = M.xxyz + M.yyyz + M.yzzz, Qzz = M.xxzz + M.yyzz + M.zzzz;
        const double hq[6] = {Qxx, Qxy, Qxz, Qyy, Qyz, Qzz};
        for (int k = 0; k < 6; ++k) E.hQ[k] = (float)(0.5 * hq[k]);
        E.qtr4 = (float)(0.125 * (Qxx + Qyy + Qzz));
        // octopole (monomials dx2 dxdy dxdz dy2 dydz dz2)
        const double c3[3][6] = {{M.xxx, 2 * M.xxy, 2 * M.xxz, M.xyy, 2 * M.xyz, M.xzz},
                                 {M.xxy, 2 * M.xyy, 2 * M.xyz, M.yyy, 2 * M.yyz, M.yzz},
                                 {M.xxz, 2 * M.xyz, 2 * M.xzz, M.yyz, 2 * M.yzz, M.zzz}};
        for (int a = 0; a < 3; ++a)
            for (int k = 0; k < 6; ++k) E.c3[a][k] = (float)(0.5 * c3[a][k]);
        E.q3[0] = (float)(0.5 * (M.xxx + M.xyy + M.xzz));
        E.q3[1] = (float)(0.5 * (M.xxy + M.yyy + M.yzz));
        E.q3[2] = (float)(0.5 * (M.xxz + M.yyz + M.zzz));
        const double q2[6] = {M.xx, M.yy, M.zz, M.xy, M.xz, M.yz};
        for (int k = 0; k < 6; ++k) E.q2[k] = (float)q2[k];
        E.qtr2 = (float)(0.5 * (M.xx + M.yy + M.zz));
        E.m = (float)M.m;
        E.L = L;
        E.alpha = 2.0 / L;
        E.alpha2 = E.alpha * E.alpha;
        E.k1 = M_PI / (E.alpha2 * L * L * L);
        E.ka = 2.0 * E.alpha / sqrt(M_PI);
        E.fEwCut2 = p.fEwCut * p.fEwCut * L * L;
        const double xc = EW_XCUT_F32 / E.alpha;
        E.fEwCut2f = (float)(xc * xc < E.fEwCut2 ? xc * xc : E.fEwCut2);
        E.smallR2 = 3.0e-3 * L * L;
        E.fL = (float)E.L;
        E.fAlpha = (float)E.alpha;
        E.fAlpha2 = (float)E.alpha2;
        E.fKa = (float)E.ka;
        E.fCut2 = (float)E.fEwCut2;
        E.fSmallR2 = (float)E.smallR2;
        E.fTwoPiL = (float)(2.0 * M_PI / E.L);
        E.fPot0 = (float)(M.m * E.k1);
        E.nReps = p.nReps;
        E.nEwReps = p.nEwReps;
        E.iOrder = p.iOrder;
        const double hc2 = p.fEwhCut * p.fEwhCut;
        E.hCut2 = hc2 < 1e6 ? (int)floor(hc2) : 1000000;
        E.hMax = 0;
        for (int h = p.hReps; h >= 1; --h)
            if (h * h <= hc2) { E.hMax = h; break; }
    }
    // k-space table: (hx, hy, hz) over [-hReps, hReps]^3 in the reference's
    // loop order (hz fastest), h = 0 and |h| > fEwhCut left out
    const double alpha = 2.0 / L;
    const double k4 = M_PI * M_PI / (alpha * alpha * L * L);
    const double hc2 = p.fEwhCut * p.fEwhCut;
    const int side = 2 * p.hReps + 1, nCand = side * side * side;
    int base = 0;
    for (int c0 = 0; c0 < nCand; c0 += EWC_BS) {
        const int c = c0 + threadIdx.x;
        const int hx = c / (side * side) - p.hReps, hy = (c / side) % side - p.hReps, hz = c % side - p.hReps;
        const int h2 = hx * hx + hy * hy + hz * hz;
        const bool keep = c < nCand && h2 != 0 && !(h2 > hc2);
        int tot;
        const int ih = base + block_rank(keep, shw, &tot);
        if (keep && ih < EW_MAXH) {
            double gam[6], mfacc = 0.0, mfacs = 0.0;
            gam[0] = exp(-k4 * h2) / (M_PI * h2 * L);
            gam[1] = 2 * M_PI / L * gam[0];
            gam[2] = -2 * M_PI / L * gam[1];
            gam[3] = 2 * M_PI / L * gam[2];
            gam[4] = -2 * M_PI / L * gam[3];
            gam[5] = 2 * M_PI / L * gam[4];
            const double g1 = gam[1], g3 = gam[3], g5 = gam[5];
            gam[1] = 0.0; gam[3] = 0.0; gam[5] = 0.0;
            qeval_h(p.iOrder, M, gam, hx, hy, hz, &mfacc);
            gam[1] = g1; gam[3] = g3; gam[5] = g5;
            gam[0] = 0.0; gam[2] = 0.0; gam[4] = 0.0;
            qeval_h(p.iOrder, M, gam, hx, hy, hz, &mfacs);
            E.hx[ih] = 2 * M_PI / L * hx;
            E.hy[ih] = 2 * M_PI / L * hy;
            E.hz[ih] = 2 * M_PI / L * hz;
            E.hC[ih] = mfacc;
            E.hS[ih] = mfacs;
            E.hxf[ih] = (float)E.hx[ih];
            E.hyf[ih] = (float)E.hy[ih];
            E.hzf[ih] = (float)E.hz[ih];
            E.hCf[ih] = (float)mfacc;
            E.hSf[ih] = (float)mfacs;
        }
        base += tot;
    }
    if (threadIdx.x == 0) E.nEwh = base < EW_MAXH ? base : EW_MAXH;
    // real-space images: a particle's offset from the root COM lies within
    // max|coordinate| + |COM| per axis, so an image whose nearest point of
    // that box is beyond fEwCut*L is never kept; the rest keep the
    // reference's loop order, the replica "hole" first
    const int R = p.nEwReps, s2 = 2 * R + 1, nImg = s2 * s2 * s2;
    const double com[3] = {M.x, M.y, M.z};
    const double fEwCut2 = p.fEwCut * p.fEwCut * L * L;
    int ni = 0;
    for (int pass = 0; pass < 2; ++pass) {
        for (int c0 = 0; c0 < nImg; c0 += EWC_BS) {
            const int c = c0 + threadIdx.x;
            const int ix = c / (s2 * s2) - R, iy = (c / s2) % s2 - R, iz = c % s2 - R;
            const int id[3] = {ix, iy, iz};
            double d2 = 0.0;
            for (int k = 0; k < 3; ++k) {
                const double s = ext + fabs(com[k]) + 1e-9 * L;
                const double d = fabs(id[k] * L) - s;
                if (d > 0) d2 += d * d;
            }
            const bool hole = abs(ix) <= p.nReps && abs(iy) <= p.nReps && abs(iz) <= p.nReps;
            const bool keep = c < nImg && hole == (pass == 0) && (hole || !(d2 > fEwCut2 * (1.0 + 1e-9)));
            int tot;
            const int k = ni + block_rank(keep, shw, &tot);
            if (keep && k < EW_MAXIMG)
                E.img[k] = make_char4((signed char)ix, (signed char)iy, (signed char)iz, hole ? 1 : 0);
            ni += tot;
        }
        if (pass == 0 && threadIdx.x == 0) E.nHole = ni;
    }
    if (threadIdx.x == 0) E.nImg = ni < EW_MAXIMG ? ni : EW_MAXIMG;
}

// The k-space vectors pkdEwaldInit keeps for fEwhCut: the count depends on
// the cut alone, so the host checks the table's capacity without the moments.
static int ewald_table_size(double fEwhCut) {
    const int hReps = (int)ceil(fEwhCut);
    int ih = 0;
    for (int hx = -hReps; hx <= hReps; ++hx)
        for (int hy = -hReps; hy <= hReps; ++hy)
            for (int hz = -hReps; hz <= hReps; ++hz) {
                const int h2 = hx * hx + hy * hy + hz * hz;
                if (h2 != 0 && !(h2 > fEwhCut * fEwhCut)) ++ih;
            }
    return ih;
}

// Root moments (pkdCalcRoot) and then every Ewald constant, on the device
// right after the cell moments; the constants land in the constant bank by
// a device-to-device copy, so no step of the evaluation waits for the host.
int tsph_ewald_roots(tsph_ctx *ctx, const tsph_grav_params *gp, cudaStream_t s) {
    if (!(gp->bPeriodic && gp->bEwald) || gp->iEwOrder < 1) return TSPH_OK;
    if (gp->iEwOrder > 4) return TSPH_ERR_ARG;
    const int n = ctx->n;
    if (n == 0) return TSPH_OK;
    if (!(gp->fEwhCut >= 0 && gp->fEwhCut < 32) || !(gp->fEwCut >= 0)) return TSPH_ERR_ARG;
    EwParams p;
    p.L = gp->dPeriod;
    p.fEwCut = gp->fEwCut;
    p.fEwhCut = gp->fEwhCut;
    p.nReps = gp->nReps;
    const int nEwReps = (int)ceil(gp->fEwCut);
    p.nEwReps = nEwReps > gp->nReps ? nEwReps : gp->nReps;
    p.iOrder = gp->iEwOrder;
    p.hReps = (int)ceil(gp->fEwhCut);
    if (p.nEwReps > 3) return TSPH_ERR_UNSUPPORTED;   // the image table holds (2*3+1)^3
    const int nh = ewald_table_size(gp->fEwhCut);
    if (nh > EW_MAXH) return TSPH_ERR_UNSUPPORTED;
    ctx->nEwt = nh;
    if (!ctx->dEw) {
        if (ctx->capturing) return TSPH_ERR_STATE;   // no allocation inside a capture
        if (cudaMalloc(&ctx->dEw, sizeof(EwConst)) != cudaSuccess) return TSPH_ERR_NOMEM;
    }
    int nb = 256;
    double *partial = ctx->dRoot + 64;
    if (gp->precision == TSPH_FP32) {
        k_root_partial<float><<<nb, RM_BS, 0, s>>>(n, ctx->P.x, ctx->P.y, ctx->P.z,
                                                             ctx->P.m, ctx->T.r, partial);
        TSPH_LAUNCH_CK("k_root_partial<f32>");
    } else {
        k_root_partial<double><<<nb, RM_BS, 0, s>>>(n, ctx->P.x, ctx->P.y, ctx->P.z,
                                                              ctx->P.m, ctx->T.r, partial);
        TSPH_LAUNCH_CK("k_root_partial<f64>");
    }
    k_root_final<<<1, 32, 0, s>>>(nb, partial, ctx->dRoot);
    TSPH_LAUNCH_CK("k_root_final");
    EwConst *dE = static_cast<EwConst *>(ctx->dEw);
    k_ewald_const<<<1, EWC_BS, 0, s>>>(p, ctx->dRoot, ctx->T, ctx->dCnt, dE);
    TSPH_LAUNCH_CK("k_ewald_const");
    TSPH_CK(cudaMemcpyToSymbolAsync(cE, dE, sizeof(EwConst), 0, cudaMemcpyDeviceToDevice, s));
    return TSPH_OK;
}

// The per-particle pass, queued behind the walk.
int tsph_ewald(tsph_ctx *ctx, const tsph_grav_params *gp) {
    if (!(gp->bPeriodic && gp->bEwald) || gp->iEwOrder < 1) return TSPH_OK;
    if (gp->iEwOrder > 4) return TSPH_ERR_ARG;
    const int n = ctx->n;
    if (n == 0) return TSPH_OK;
    const int BS = 128;
    if (gp->precision == TSPH_FP32) {
        k_ewald<float><<<tsph_blocks(n, BS), BS, 0, ctx->stream>>>(ctx->P, ctx->dCnt);
        TSPH_LAUNCH_CK("k_ewald<float>");
    } else {
        k_ewald<double><<<tsph_blocks(n, BS), BS, 0, ctx->stream>>>(ctx->P, ctx->dCnt);
        TSPH_LAUNCH_CK("k_ewald<double>");
    }
    return TSPH_OK;
}
