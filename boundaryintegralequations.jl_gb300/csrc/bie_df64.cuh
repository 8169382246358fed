// Double-float (pairs of floats, ~48-bit significand) helpers of the
// FP64-grade kernels (BIE_PREC_DF64): Taylor coefficient tables, a four-part
// pi/2, sine/cosine with quadrant reduction, reciprocal, square root,
// compensated sums, and the kernel values of one quadrature point.
#pragma once

#include "bie_device.cuh"
#include "bie_mixed.cuh"

#include <cmath>

namespace bie {
namespace df64 {
namespace {

// The coefficients (-1)^j/(2j)!, (-1)^j/(2j+1)!, 1/j! as hi + lo floats
// (computed with 200-bit arithmetic, ~2^-49 relative).
__constant__ float2 kDfCos[13] = {
    {0x1.0000000000000p+0f, 0x0.0p+0f}, {-0x1.0000000000000p-1f, 0x0.0p+0f},
    {0x1.5555560000000p-5f, -0x1.5555560000000p-30f}, {-0x1.6c16c20000000p-10f, 0x1.27d27e0000000p-35f},
    {0x1.a01a020000000p-16f, -0x1.7f97fa0000000p-42f}, {-0x1.27e4fc0000000p-22f, 0x1.10ec140000000p-47f},
    {0x1.1eed8e0000000p-29f, 0x1.ff1b120000000p-54f}, {-0x1.93974a0000000p-37f, -0x1.180f940000000p-62f},
    {0x1.ae7f3e0000000p-45f, 0x1.ccee080000000p-71f}, {-0x1.6827860000000p-53f, -0x1.dcbecc0000000p-80f},
    {0x1.e542ba0000000p-62f, 0x1.00808a0000000p-88f}, {-0x1.0ce3960000000p-70f, -0x1.b6ff0a0000000p-95f},
    {0x1.f2cf020000000p-80f, -0x1.a342a20000000p-106f},
};
__constant__ float2 kDfSin[13] = {
    {0x1.0000000000000p+0f, 0x0.0p+0f}, {-0x1.5555560000000p-3f, 0x1.5555560000000p-28f},
    {0x1.1111120000000p-7f, -0x1.ddddde0000000p-32f}, {-0x1.a01a020000000p-13f, 0x1.7f97fa0000000p-39f},
    {0x1.71de3a0000000p-19f, 0x1.55b1cc0000000p-45f}, {-0x1.ae64560000000p-26f, -0x1.fd51380000000p-52f},
    {0x1.6124620000000p-33f, -0x1.8af25e0000000p-58f}, {-0x1.ae7f3e0000000p-41f, -0x1.ccee080000000p-67f},
    {0x1.952c780000000p-49f, -0x1.f9ea560000000p-74f}, {-0x1.2f49b40000000p-57f, -0x1.a050560000000p-83f},
    {0x1.71b8f00000000p-66f, -0x1.2461520000000p-91f}, {-0x1.761b420000000p-75f, 0x1.9d38fc0000000p-100f},
    {0x1.3f3cce0000000p-84f, -0x1.74d02c0000000p-111f},
};
__constant__ float2 kDfExp[25] = {
    {0x1.0000000000000p+0f, 0x0.0p+0f}, {0x1.0000000000000p+0f, 0x0.0p+0f},
    {0x1.0000000000000p-1f, 0x0.0p+0f}, {0x1.5555560000000p-3f, -0x1.5555560000000p-28f},
    {0x1.5555560000000p-5f, -0x1.5555560000000p-30f}, {0x1.1111120000000p-7f, -0x1.ddddde0000000p-32f},
    {0x1.6c16c20000000p-10f, -0x1.27d27e0000000p-35f}, {0x1.a01a020000000p-13f, -0x1.7f97fa0000000p-39f},
    {0x1.a01a020000000p-16f, -0x1.7f97fa0000000p-42f}, {0x1.71de3a0000000p-19f, 0x1.55b1cc0000000p-45f},
    {0x1.27e4fc0000000p-22f, -0x1.10ec140000000p-47f}, {0x1.ae64560000000p-26f, 0x1.fd51380000000p-52f},
    {0x1.1eed8e0000000p-29f, 0x1.ff1b120000000p-54f}, {0x1.6124620000000p-33f, -0x1.8af25e0000000p-58f},
    {0x1.93974a0000000p-37f, 0x1.180f940000000p-62f}, {0x1.ae7f3e0000000p-41f, 0x1.ccee080000000p-67f},
    {0x1.ae7f3e0000000p-45f, 0x1.ccee080000000p-71f}, {0x1.952c780000000p-49f, -0x1.f9ea560000000p-74f},
    {0x1.6827860000000p-53f, 0x1.dcbecc0000000p-80f}, {0x1.2f49b40000000p-57f, 0x1.a050560000000p-83f},
    {0x1.e542ba0000000p-62f, 0x1.00808a0000000p-88f}, {0x1.71b8f00000000p-66f, -0x1.2461520000000p-91f},
    {0x1.0ce3960000000p-70f, 0x1.b6ff0a0000000p-95f}, {0x1.761b420000000p-75f, -0x1.9d38fc0000000p-100f},
    {0x1.f2cf020000000p-80f, -0x1.a342a20000000p-106f},
};
constexpr int kDfMaxTrig = 12;   // highest coefficient index of kDfCos / kDfSin
constexpr int kDfMaxExp = 24;    // of kDfExp

// pi/2 = P1 + P2 + P3 + P4 (P1, P2 with 12 significant bits: n * P1 and
// n * P2 are exact for |n| < 2^12; the sum is pi/2 to ~2e-25)
constexpr float kPio2P1 = 0x1.922p+0f;
constexpr float kPio2P2 = -0x1.2aep-18f;
constexpr float kPio2P3 = -0x1.de973ep-31f;
constexpr float kPio2P4 = 0x1.a62634p-58f;
constexpr float kTwoOverPi = 0x1.45f306p-1f;
constexpr float kDfMaxPhase = 4000.0f;    // beyond: pair deferred to FP64

namespace dd {
using dev::df;

__device__ __forceinline__ df add_f(df a, float b) {
    df s = dev::two_sum(a.hi, b);
    s.lo = __fadd_rn(s.lo, a.lo);
    return dev::fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df neg(df a) { return {-a.hi, -a.lo}; }
// 1 / a: correctly rounded float reciprocal plus one correction, which
// squares its error (relative error ~2^-47)
__device__ __forceinline__ df rcp(df a) {
    const float q1 = __frcp_rn(a.hi);
    float r = __fmaf_rn(-a.hi, q1, 1.0f);
    r = __fmaf_rn(-a.lo, q1, r);
    return dev::fast_two_sum(q1, __fmul_rn(q1, r));
}
// sqrt(a), a > 0: correctly rounded float square root plus one Newton
// correction whose 1/(2 y) only needs float accuracy (relative error ~2^-46)
__device__ __forceinline__ df sqrt_df(df a) {
    const float y = __fsqrt_rn(a.hi);
    const float e = __fadd_rn(__fmaf_rn(-y, y, a.hi), a.lo);
    return dev::fast_two_sum(y, __fmul_rn(e, 0.5f * rsqrtf(a.hi)));
}
// a * b with the product left unnormalised (hi, lo): for sums that
// renormalise later
__device__ __forceinline__ df mul_raw(df a, df b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return {p, e};
}
__device__ __forceinline__ df coef(const float2 *c, int j) {
    const float2 v = c[j];
    return {v.x, v.y};
}
// sum_{j <= J} c_j z^j by Horner's rule
__device__ __forceinline__ df poly(const float2 *c, int J, df z) {
    df acc = coef(c, J);
    for (int j = J - 1; j >= 0; --j) acc = dev::df_add(dev::df_mul(acc, z), coef(c, j));
    return acc;
}
// sin and cos of x (|x| < kDfMaxPhase): x - n pi/2 in double-float, then the
// Taylor series to x^17 / x^16 on |y| <= pi/4 (truncation below 1e-17)
__device__ __forceinline__ void sincos_df(df x, df &s, df &c) {
    const float n = rintf(__fmul_rn(x.hi, kTwoOverPi));
    df y = add_f(x, -__fmul_rn(n, kPio2P1));
    y = add_f(y, -__fmul_rn(n, kPio2P2));
    const float p = __fmul_rn(n, kPio2P3);
    y = dev::df_sub(y, df{p, __fmaf_rn(n, kPio2P3, -p)});
    y = add_f(y, -__fmul_rn(n, kPio2P4));
    const df z = dev::df_sqr(y);
    const df sn = dev::df_mul(y, poly(kDfSin, 8, z));
    const df cs = poly(kDfCos, 8, z);
    const int q = ((int)n) & 3;
    if (q == 0) { s = sn; c = cs; }
    else if (q == 1) { s = cs; c = neg(sn); }
    else if (q == 2) { s = neg(sn); c = neg(cs); }
    else { s = neg(cs); c = sn; }
}
}  // namespace dd

// sin and cos of an FP64 phase through sincos_df on the FP32 pipes (relative
// error ~2^-46, well inside the FP64-grade and mixed-precision budgets), FP64
// sincos beyond its range.  For the FP64 element integrals of the deferred
// (near) pairs of the mixed and double-float paths: the FP64 sine and cosine
// are most of their FP64-pipe work, and this GPU's FP64 pipe runs at 1/64 of
// the FP32 rate.
struct TrigDf {
    static __device__ __forceinline__ void sincos_of(double x, double *s, double *c) {
        if (!(fabs(x) < (double)kDfMaxPhase)) {
            sincos(x, s, c);
            return;
        }
        dev::df sd, cd;
        dd::sincos_df(dev::df_from_double(x), sd, cd);
        *s = dev::f2d(sd.hi) + dev::f2d(sd.lo);
        *c = dev::f2d(cd.hi) + dev::f2d(cd.lo);
    }
};

namespace dd {

// running sum of double-float terms with the error term carried in float
// (renormalised once at the end of a pair)
struct Acc {
    float hi, lo;
};
__device__ __forceinline__ void acc_add(Acc &s, df p) {
    const df t = dev::two_sum(s.hi, p.hi);
    s.hi = t.hi;
    s.lo = __fadd_rn(s.lo, __fadd_rn(t.lo, p.lo));
}
__device__ __forceinline__ double acc_value(const Acc &s) {
    return dev::f2d(s.hi) + dev::f2d(s.lo);
}
__device__ __forceinline__ df to_df(double x) { return dev::df_from_double(x); }
}  // namespace dd

// e^{i j h}, h = 2^-7, j = -kPhaseTabHalf..kPhaseTabHalf as (cos hi, cos lo,
// sin hi, sin lo): the per-point rotation e^{i theta} is the table entry at
// the nearest j h times a short Taylor series of the remainder (|.| <= 2^-8)
constexpr int kPhaseTabHalf = 512;
constexpr float kPhaseTabStep = 0x1p-7f;

struct DfDegrees {
    int Jc, Js, Je;        // Taylor degrees (coefficient counts - 1) of cos, sin, exp
    const float4 *tab;     // device phase table (2 kPhaseTabHalf + 1 entries)
};

// Taylor degrees for |k (r - r0)| <= theta (and |Im k (r - r0)| <= kappa):
// the first omitted term below 2^-53; false if a table is too short
inline bool df_degrees(double theta, double kappa, DfDegrees &d) {
    if (!(theta < 0.9 * kPhaseTabHalf * (double)kPhaseTabStep)) return false;   // table range
    auto need = [](double x, int first, int step, int jmax, int &J) {
        // term index n = first + step * j; stop once x^n / n! < 2^-53
        for (int j = 0; j <= jmax; ++j) {
            const int n = first + step * (j + 1);
            double t = 1.0;
            for (int m = 1; m <= n; ++m) t *= x / m;
            if (t < 0x1p-53) {
                J = j;
                return true;
            }
        }
        return false;
    };
    return need(theta, 0, 2, kDfMaxTrig, d.Jc) && need(theta, 1, 2, kDfMaxTrig, d.Js) &&
           need(kappa, 0, 1, kDfMaxExp, d.Je);
}


// Kernel values at one quadrature point of a regular pair in double-float
// (greens3d!, freens3d!, freens3dk0! of src/3d/kernels.jl:13-55 times the
// jacobian-weight product): D = c_e - t, record point (A, B: o and jw/4pi as
// hi/lo; Cn, Dn: the unit normal as hi/lo), r0 = |D|, E0 = e^{i k r0}
// (times e^{-Im k r0}).  Returns F_q, G_q and t_q (C_q = -t_q).
template <bool CPLX_K>
__device__ __forceinline__ void qpe_df64(const float4 A, const float4 B, const float4 Cn, const float4 Dn,
                                         const mixed::PairSetup &P, dev::df r0, dev::df E0r, dev::df E0i,
                                         dev::df K, dev::df Ki, const DfDegrees deg, dev::df &Fr, dev::df &Fi,
                                         dev::df &Gr, dev::df &Gi, dev::df &tq) {
    using dev::df;
    const df dx = dev::df_add(P.Dxd, df{A.x, B.x});
    const df dy = dev::df_add(P.Dyd, df{A.y, B.y});
    const df dz = dev::df_add(P.Dzd, df{A.z, B.z});
    const df rr = dd::sqrt_df(dev::df_add(dev::df_add(dev::df_sqr(dx), dev::df_sqr(dy)), dev::df_sqr(dz)));
    const df ri_ = dd::rcp(rr);
    // e^{i k (r - r0)} = e^{i j h} e^{i (theta - j h)}, |theta| < kPhaseTabHalf h
    const df th = dev::df_mul(K, dev::df_sub(rr, r0));
    const float jf = rintf(__fmul_rn(th.hi, 1.0f / kPhaseTabStep));
    const df dl = dd::add_f(th, -__fmul_rn(jf, kPhaseTabStep));    // exact product
    const df z = dev::df_sqr(dl);
    const df cd = dd::poly(kDfCos, 2, z);                            // to dl^4: dl^6/6! < 5e-18
    const df sd = dev::df_mul(dl, dd::poly(kDfSin, 2, z));
    // (|jf| <= 0.9 kPhaseTabHalf by the host's bound on |k| x element radius;
    // clamped so that no value can index outside the table)
    const int jt = min(kPhaseTabHalf, max(-kPhaseTabHalf, __float2int_rn(jf)));
    const float4 T = __ldg(deg.tab + kPhaseTabHalf + jt);
    const df Tc{T.x, T.y}, Ts{T.z, T.w};
    df ct = dev::df_sub(dev::df_mul(Tc, cd), dev::df_mul(Ts, sd));
    df st = dev::df_add(dev::df_mul(Ts, cd), dev::df_mul(Tc, sd));
    if (CPLX_K) {
        const df damp = dd::poly(kDfExp, deg.Je, dd::neg(dev::df_mul(Ki, dev::df_sub(rr, r0))));
        ct = dev::df_mul(ct, damp);
        st = dev::df_mul(st, damp);
    }
    const df er = dev::df_sub(dev::df_mul(E0r, ct), dev::df_mul(E0i, st));
    const df ei = dev::df_add(dev::df_mul(E0r, st), dev::df_mul(E0i, ct));
    // G = e jw / (4 pi r); t = (x - y).n jw / (4 pi r^3); F = e (i k r - 1) t
    const df sw = dev::df_mul(df{A.w, B.w}, ri_);
    Gr = dev::df_mul(er, sw);
    Gi = dev::df_mul(ei, sw);
    const df dn = dev::df_add(dev::df_add(dev::df_mul(dx, df{Cn.x, Dn.x}), dev::df_mul(dy, df{Cn.y, Dn.y})),
                              dev::df_mul(dz, df{Cn.z, Dn.z}));
    tq = dev::df_mul(dev::df_mul(dn, sw), dev::df_sqr(ri_));
    const df kr = dev::df_mul(K, rr);
    df ar = {-1.0f, 0.0f};
    if (CPLX_K) ar = dev::df_sub(ar, dev::df_mul(Ki, rr));
    Fr = dev::df_mul(dev::df_sub(dev::df_mul(er, ar), dev::df_mul(ei, kr)), tq);
    Fi = dev::df_mul(dev::df_add(dev::df_mul(er, kr), dev::df_mul(ei, ar)), tq);
}

// e^{i k r0} (times e^{-Im k r0}) of one pair
template <bool CPLX_K>
__device__ __forceinline__ void pair_phase_df64(dev::df kr0, dev::df r0, double kim, dev::df &E0r, dev::df &E0i) {
    dd::sincos_df(kr0, E0i, E0r);
    if (CPLX_K) {
        const dev::df damp = dd::to_df(exp(-kim * (dev::f2d(r0.hi) + dev::f2d(r0.lo))));
        E0r = dev::df_mul(E0r, damp);
        E0i = dev::df_mul(E0i, damp);
    }
}

}  // namespace
}  // namespace df64
}  // namespace bie
