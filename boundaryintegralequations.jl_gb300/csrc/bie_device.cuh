// Device helpers shared by the assembly and operator kernels.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace bie {
namespace dev {

constexpr double kInv4Pi = 0.07957747154594767;   // 1 / (4 pi)

struct RuleInfo {
    int Q[6];
    int off[6];
};

// Julia's 3-argument hypot (maximum-abs scaling, IEEE-rounded division and
// square root, ((a^2 + b^2) + c^2) summation), evaluated bit-exactly.
__device__ __forceinline__ double julia_hypot3(double x, double y, double z) {
    const double m = fmax(fmax(fabs(x), fabs(y)), fabs(z));
    if (m == 0.0) return 0.0;
    const double a = __ddiv_rn(x, m), b = __ddiv_rn(y, m), c = __ddiv_rn(z, m);
    const double s = __dadd_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)), __dmul_rn(c, c));
    return __dmul_rn(m, __dsqrt_rn(s));
}

// find_closest_corner (src/3d/assembly_collocation.jl:102-115): index of the
// physics node nearest to the target, strict '<' so the first of equal
// distances wins.  Squared distances decide whenever the runner-up is more
// than 1e-12 (relative) farther; only near-ties are re-decided with the exact
// Julia hypot so the choice is the reference's in every case.
// `P` holds the NP node coordinates, a-major (x, y, z).
template <int NP>
__device__ __forceinline__ int nearest_node(const double *P, double tx, double ty, double tz) {
    double d2[NP];
#pragma unroll
    for (int a = 0; a < NP; ++a) {
        const double dx = P[3 * a + 0] - tx, dy = P[3 * a + 1] - ty, dz = P[3 * a + 2] - tz;
        d2[a] = dx * dx + dy * dy + dz * dz;
    }
    int c = 0;
    double b = d2[0];
#pragma unroll
    for (int a = 1; a < NP; ++a)
        if (d2[a] < b) {
            b = d2[a];
            c = a;
        }
    const double lim = b * (1.0 + 1e-12);
    bool tie = false;
#pragma unroll
    for (int a = 0; a < NP; ++a) tie |= (a != c) && (d2[a] <= lim);
    if (tie) {
        double best = __longlong_as_double(0x7ff0000000000000LL);
        c = 0;
#pragma unroll
        for (int a = 0; a < NP; ++a) {
            const double h = julia_hypot3(__dsub_rn(P[3 * a + 0], tx), __dsub_rn(P[3 * a + 1], ty),
                                          __dsub_rn(P[3 * a + 2], tz));
            if (h < best) {
                best = h;
                c = a;
            }
        }
    }
    return c;
}

// sin and cos of the phase k r in FP64: the plain FP64 kernels keep the
// reference's arithmetic (Julia's sincos of a Float64)
struct TrigFp64 {
    static __device__ __forceinline__ void sincos_of(double x, double *s, double *c) { sincos(x, s, c); }
};

// FP64 integration of one element for one target with the rule clustered at
// node c: computing_integrals! (src/3d/assembly_collocation.jl:213-252).
// g: rule data x[Q] y[Q] z[Q] nx[Q] ny[Q] nz[Q] jw[Q]; ph: Phi[q][a].
// Accumulates F, G per node and returns the C contribution.  Trig: how the
// sine and cosine of k r are formed (TrigFp64, or df64::TrigDf).
template <int NP, bool CPLX_K, class Trig = TrigFp64>
__device__ __forceinline__ double element_fp64(const double *g, int Q, const double *ph, double tx,
                                               double ty, double tz, double kre, double kim,
                                               double *fr, double *fi, double *gr, double *gi,
                                               int tm = -1) {
    // tm >= 0: tm-th derivative with respect to k (taylor_greens3d!,
    // taylor_freens3d!, src/3d/kernels.jl:94-118): both kernels times (i r)^tm,
    // and F's factor (i k r - 1) becomes (i k r - 1 + tm).
#pragma unroll
    for (int a = 0; a < NP; ++a) fr[a] = fi[a] = gr[a] = gi[a] = 0.0;
    double ce = 0.0;
    for (int q = 0; q < Q; ++q) {
        const double dx = g[q] - tx;
        const double dy = g[Q + q] - ty;
        const double dz = g[2 * Q + q] - tz;
        const double r2 = dx * dx + dy * dy + dz * dz;
        const double rinv = rsqrt(r2);
        const double rr = r2 * rinv;
        const double jw = g[6 * Q + q];
        const double dn = g[3 * Q + q] * dx + g[4 * Q + q] * dy + g[5 * Q + q] * dz;
        double sn, cs;
        Trig::sincos_of(kre * rr, &sn, &cs);
        if (CPLX_K) {
            const double damp = exp(-kim * rr);
            sn *= damp;
            cs *= damp;
        }
        // G: e^{ikr} / (4 pi r) * jw
        const double wg = rinv * kInv4Pi * jw;
        double Gr = cs * wg, Gi = sn * wg;
        // C: -(x - y).n / (4 pi r^3) * jw ; F: e^{ikr} (ikr - 1) (x - y).n / (4 pi r^3) * jw
        const double tq = dn * (rinv * rinv * rinv) * kInv4Pi * jw;
        ce -= tq;
        double ar = CPLX_K ? (-1.0 - kim * rr) : -1.0;
        const double ai = kre * rr;
        if (tm > 0) ar += (double)tm;
        double Fr = (cs * ar - sn * ai) * tq;
        double Fi = (cs * ai + sn * ar) * tq;
        if (tm > 0) {
            double rm = rr;
            for (int t = 1; t < tm; ++t) rm *= rr;
            // (i r)^tm = i^tm r^tm
            const int q4 = tm & 3;
            const double pr = q4 == 0 ? rm : (q4 == 2 ? -rm : 0.0);
            const double pi = q4 == 1 ? rm : (q4 == 3 ? -rm : 0.0);
            double t0 = Gr * pr - Gi * pi;
            Gi = Gr * pi + Gi * pr;
            Gr = t0;
            t0 = Fr * pr - Fi * pi;
            Fi = Fr * pi + Fi * pr;
            Fr = t0;
        }
        const double *pq = ph + q * NP;
#pragma unroll
        for (int a = 0; a < NP; ++a) {
            const double p = pq[a];
            fr[a] += Fr * p;
            fi[a] += Fi * p;
            gr[a] += Gr * p;
            gi[a] += Gi * p;
        }
    }
    return ce;
}

// ---------------------------------------------------------------------------
// Double-float (unevaluated sum of two floats) arithmetic, ~48-bit significand.
// Error-free transformations after Knuth (TwoSum) and Dekker (FastTwoSum,
// TwoProduct with an FMA).
// ---------------------------------------------------------------------------
struct df {
    float hi, lo;
};

__device__ __forceinline__ df two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}
__device__ __forceinline__ df fast_two_sum(float a, float b) {   // |a| >= |b|
    const float s = __fadd_rn(a, b);
    const float e = __fsub_rn(b, __fsub_rn(s, a));
    return {s, e};
}
__device__ __forceinline__ df df_sub(df a, df b) {
    df s = two_sum(a.hi, -b.hi);
    s.lo = __fadd_rn(s.lo, __fsub_rn(a.lo, b.lo));
    return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df df_add(df a, df b) {
    df s = two_sum(a.hi, b.hi);
    s.lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
    return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df df_sqr(df a) {
    const float p = __fmul_rn(a.hi, a.hi);
    float e = __fmaf_rn(a.hi, a.hi, -p);
    e = __fmaf_rn(2.0f * a.hi, a.lo, e);
    return fast_two_sum(p, e);
}
__device__ __forceinline__ df df_mul(df a, df b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return fast_two_sum(p, e);
}
// sqrt(a) for a > 0: one Newton correction of the float square root
__device__ __forceinline__ df df_sqrt(df a) {
    const float y = __fsqrt_rn(a.hi);
    const float e = __fadd_rn(__fmaf_rn(-y, y, a.hi), a.lo);
    return fast_two_sum(y, __fdiv_rn(e, 2.0f * y));
}
__device__ __forceinline__ df df_from_double(double x) {
    const float hi = __double2float_rn(x);
    return {hi, __double2float_rn(x - (double)hi)};
}

// sin and cos of a float angle of moderate size (|x| < 1e4): quadrant
// reduction by pi/2 in two FMA steps (Cody-Waite with an 8-bit leading
// constant), then the Taylor series of sin to x^9 and of cos to x^10 on
// |x| <= pi/4 (truncation below 2e-9).
__device__ __forceinline__ void sincos_f32(float x, float *s, float *c) {
    const float kPio2Hi = 1.5703125f;                     // 8 significant bits
    const float kPio2Lo = 4.83826794897e-4f;              // pi/2 - kPio2Hi
    const float j = rintf(x * 0.63661977236758134f);      // 2 / pi
    float f = __fmaf_rn(-j, kPio2Hi, x);
    f = __fmaf_rn(-j, kPio2Lo, f);
    const float f2 = f * f;
    float ps = __fmaf_rn(f2, 2.7557319e-6f, -1.9841270e-4f);   // 1/9!, -1/7!
    ps = __fmaf_rn(f2, ps, 8.3333333e-3f);                       // 1/5!
    ps = __fmaf_rn(f2, ps, -1.6666667e-1f);                      // -1/3!
    const float sn = __fmaf_rn(f * f2, ps, f);
    float pc = __fmaf_rn(f2, -2.7557319e-7f, 2.4801587e-5f);    // -1/10!, 1/8!
    pc = __fmaf_rn(f2, pc, -1.3888889e-3f);                      // -1/6!
    pc = __fmaf_rn(f2, pc, 4.1666667e-2f);                       // 1/4!
    pc = __fmaf_rn(f2, pc, -0.5f);                               // -1/2!
    const float cs = __fmaf_rn(f2, pc, 1.0f);
    const int q = ((int)j) & 3;
    const float a = (q & 1) ? cs : sn;
    const float b = (q & 1) ? sn : cs;
    *s = (q & 2) ? -a : a;
    *c = ((q + 1) & 2) ? -b : b;
}

// float -> double by moving bits with integer instructions only (GB300's
// conversion instruction runs on the narrow FP64 pipe).  Normal numbers take a
// five-instruction path (exponent rebias by adding 896 << 20 to the shifted
// bits); zero, subnormals, infinities and NaNs take the general path, which
// normalises subnormals with a leading-zero count.  Exact for every input.
static __device__ __noinline__ double f2d_special(uint32_t u) {
    const uint32_t sign = u & 0x80000000u;
    const uint32_t ex = (u >> 23) & 0xffu;
    const uint32_t man = u & 0x7fffffu;
    if (ex == 0xffu)   // infinity or NaN (payload kept nonzero)
        return __hiloint2double((int)(sign | 0x7ff00000u | (man >> 3) | ((man != 0u && (man >> 3) == 0u) ? 1u : 0u)),
                                (int)(man << 29));
    if (man == 0u) return __hiloint2double((int)sign, 0);   // signed zero
    // subnormal: value man 2^-149, leading one moved to bit 23
    const uint32_t lz = (uint32_t)__clz((int)man);          // 9..31
    const uint32_t mn = (man << (lz - 8u)) & 0x7fffffu;
    return __hiloint2double((int)(sign | ((905u - lz) << 20) | (mn >> 3)), (int)(mn << 29));
}

__device__ __forceinline__ double f2d(float f) {
    const uint32_t u = __float_as_uint(f);
    const uint32_t a = u & 0x7fffffffu;
    if (a - 0x00800000u < 0x7f000000u)   // normal: exponent field 1..254
        return __hiloint2double((int)((u & 0x80000000u) | ((a >> 3) + 0x38000000u)), (int)(u << 29));
    return f2d_special(u);
}

}  // namespace dev
}  // namespace bie
