// Mixed-precision (FP32 + double-float) evaluation of one (target, element) pair,
// shared by the mixed assembly kernel and the on-the-fly operator kernels.
//
// Element record layout: MixedLayout in bie_internal.h.  The pair set-up forms
// D = c_e - t and r0 = |D| in double-float and reduces k r0 modulo 2 pi there;
// the quadrature loop then evaluates, per point x_q = c_e + o,
//   r = |D + o|,  phase = k r0 + k (r - r0),  r - r0 = (2 D.o + |o|^2) / (r + r0),
//   G_q = e^{i phase} jw / (4 pi r)
//   F_q = e^{i phase} (i k r - 1) (x_q - t).n jw / (4 pi r^3)
//   C_q = -(x_q - t).n jw / (4 pi r^3)
// (greens3d!, freens3d!, freens3dk0! of src/3d/kernels.jl:13-55 times the
// jacobian-weight product of src/3d/assembly_collocation.jl:213-252).
#pragma once

#include "bie_device.cuh"

namespace bie {
namespace mixed {

using dev::df;

constexpr float kTwoPiA = 6.28125f;                 // 2 pi = A + B + C (A has 8 bits)
constexpr float kTwoPiB = 1.9353071795864769e-3f;
constexpr float kTwoPiC = 1.0253376606e-11f;        // (2 pi - A) - B, rounded
constexpr float kInv2Pi = 0.15915494309189535f;

template <int NP>
struct PhiPad {
    static constexpr int value = NP <= 4 ? 4 : 8;   // Phi rows padded for 16-byte loads
};

// sqrt of a positive double-float: float estimate from rsqrt, one correction
__device__ __forceinline__ df df_sqrt_fast(df a) {
    const float ri = rsqrtf(a.hi);
    const float y = a.hi * ri;
    const float e = __fadd_rn(__fmaf_rn(-y, y, a.hi), a.lo);
    return dev::fast_two_sum(y, e * (0.5f * ri));
}

struct Target {
    df x, y, z;
};

struct PairSetup {
    int c;            // rule = nearest physics node
    bool deferred;    // near pair or nearest-node near-tie: integrate in FP64
    float Dx, Dy, Dz; // c_e - t (FP32)
    df Dxd, Dyd, Dzd; // c_e - t (double-float)
};

// Nearest physics node in FP32 with near / near-tie detection.
template <int NP>
__device__ __forceinline__ PairSetup pair_setup(const float *r, const Target &T) {
    PairSetup P;
    const float4 h0 = *reinterpret_cast<const float4 *>(r);       // c_hi xyz, c_lo x
    const float4 h1 = *reinterpret_cast<const float4 *>(r + 4);   // c_lo yz, near2, -
    P.Dxd = dev::df_sub({h0.x, h0.w}, T.x);
    P.Dyd = dev::df_sub({h0.y, h1.x}, T.y);
    P.Dzd = dev::df_sub({h0.z, h1.y}, T.z);
    P.Dx = P.Dxd.hi;
    P.Dy = P.Dyd.hi;
    P.Dz = P.Dzd.hi;
    float d2[NP];
#pragma unroll
    for (int a = 0; a < NP; ++a) {
        const float ax = P.Dx + r[8 + 3 * a], ay = P.Dy + r[9 + 3 * a], az = P.Dz + r[10 + 3 * a];
        d2[a] = ax * ax + ay * ay + az * az;
    }
    int c = 0;
    float b = d2[0];
#pragma unroll
    for (int a = 1; a < NP; ++a)
        if (d2[a] < b) {
            b = d2[a];
            c = a;
        }
    const float lim = b * (1.0f + 1e-5f);
    bool tie = false;
#pragma unroll
    for (int a = 0; a < NP; ++a) tie |= (a != c) && (d2[a] <= lim);
    const float r0f2 = P.Dx * P.Dx + P.Dy * P.Dy + P.Dz * P.Dz;
    const float near2 = h1.z;
    P.c = c;
    P.deferred = tie || r0f2 < near2 || 4.0f * b < near2;
    return P;
}

struct Phase {
    float th0;   // k r0 mod 2 pi
    float r0;
};

__device__ __forceinline__ Phase pair_phase(const PairSetup &P, df K) {
    const df r0sq = dev::df_add(dev::df_add(dev::df_sqr(P.Dxd), dev::df_sqr(P.Dyd)), dev::df_sqr(P.Dzd));
    const df r0 = df_sqrt_fast(r0sq);
    const df kr0 = dev::df_mul(K, r0);
    const float nrev = rintf(kr0.hi * kInv2Pi);
    float th0 = __fmaf_rn(-nrev, kTwoPiA, kr0.hi);
    th0 = __fmaf_rn(-nrev, kTwoPiB, th0);
    th0 = __fmaf_rn(-nrev, kTwoPiC, th0);
    th0 += kr0.lo;
    return {th0, r0.hi};
}

// Kernel values at quadrature point q of the chosen rule.
struct QpeValues {
    float Fr, Fi, Gr, Gi, tq;   // tq = (x - t).n jw / (4 pi r^3); C_q = -tq
};

template <bool CPLX_K>
__device__ __forceinline__ QpeValues qpe(const float4 A, const float4 B, const PairSetup &P,
                                         const Phase &ph, float kf, float kimf) {
    const float dx = P.Dx + A.x, dy = P.Dy + A.y, dz = P.Dz + A.z;   // x_q - t
    const float r2 = dx * dx + dy * dy + dz * dz;
    const float rinv = rsqrtf(r2);
    const float rr = r2 * rinv;
    // r - r0 = (2 D.o + |o|^2) / (r + r0), free of cancellation
    const float num = __fmaf_rn(2.0f, P.Dx * A.x + P.Dy * A.y + P.Dz * A.z, B.w);
    const float dr = __fdividef(num, rr + ph.r0);
    float sn, cs;
    dev::sincos_f32(__fmaf_rn(kf, dr, ph.th0), &sn, &cs);
    if (CPLX_K) {
        const float damp = __expf(-kimf * rr);
        sn *= damp;
        cs *= damp;
    }
    const float dn = B.x * dx + B.y * dy + B.z * dz;
    const float wg = rinv * A.w;                      // jw / (4 pi r)
    QpeValues v;
    v.Gr = cs * wg;
    v.Gi = sn * wg;
    v.tq = dn * (rinv * rinv) * wg;                   // (x-t).n jw / (4 pi r^3)
    const float ar = CPLX_K ? (-1.0f - kimf * rr) : -1.0f;
    const float ai = kf * rr;
    v.Fr = (cs * ar - sn * ai) * v.tq;
    v.Fi = (cs * ai + sn * ar) * v.tq;
    return v;
}

// C row sum in double-float: acc += x
__device__ __forceinline__ void df_accum(df &acc, float x) {
    const df t = dev::two_sum(acc.hi, x);
    acc = dev::fast_two_sum(t.hi, __fadd_rn(t.lo, acc.lo));
}

}  // namespace mixed
}  // namespace bie
