// K2: mixed-precision dense collocation assembly (BIE_PREC_MIXED).
//
// Same result as K1 (assemble_parallel!, src/3d/assembly_collocation.jl:270-479)
// to a stated relative error, with the regular (target, element) pairs on the
// FP32 pipe and the pairs that need FP64 moved to a sparse FP64 correction:
//
//   * regular pairs: quadrature points stored relative to the element centroid
//     c_e in FP32.  Per pair, D = c_e - t and r0 = |D| are formed in
//     double-float arithmetic and the phase k r0 is reduced modulo 2 pi there,
//     so the per-point phase  k r0 + k (r - r0)  with
//     r - r0 = (2 D.o + |o|^2) / (r + r0)  (o = x_q - c_e) stays accurate to
//     ~1e-7 even for k r ~ 20.  sin/cos are evaluated with a quadrant reduction
//     and Taylor polynomials on the FMA pipe.  Per-node sums are FP32 over the
//     <= 8 points of one element.  Each (row, node) entry is written by the
//     thread that owns the row, in the element slice the node belongs to: the
//     node's first element in the slice stores its FP32 sums, later elements
//     add to them in place, the last one converts the sum to complex128 and
//     stores it (or keeps complex64 when the caller asks for complex64
//     matrices).  The F and G partial sums travel together as one float4 in
//     the F entry's 16 bytes, so no memset, no atomics and no widening pass
//     touch the matrices.  Nodes touched by several slices sum their slice's
//     contributions in a side slot; a fix-up pass adds the slots and writes
//     those columns.
//   * near pairs (target within one element size of the centroid, or within half
//     an element size of a physics node: the singular and near-singular
//     elements, which include every element containing the target node) and
//     pairs whose nearest physics node is a near-tie (runner-up within 1e-5)
//     are not integrated in FP32: they are appended to a list and integrated in
//     FP64 by a correction kernel with the exact reference rule choice, then
//     added to F, G and C.  If the list is full the pair is integrated in FP64
//     in place (slower, same result).
//   * C (free term): per-pair FP32 sums accumulated in double-float per row,
//     the near pairs in FP64.
#include "bie_internal.h"
#include "bie_device.cuh"
#include "bie_mixed.cuh"
#include "bie_df64.cuh"

#include <algorithm>
#include <cmath>
#include <type_traits>

namespace bie {

namespace {

using dev::df;
using dev::RuleInfo;
constexpr int kThreads = 128;
using mixed::PhiPad;

struct Fp64View {
    const double *rec;
    int stride;
    int nidx_off;
    const double *phi;   // global, R x qmax x NP
    int qmax;
    RuleInfo ri;
};

// Per-node sums of one pair, returned by value from the out-of-line FP64 path
// so that the caller's register arrays never have their address taken (an
// address passed to a non-inlined call would keep them in local memory for
// the whole element loop).
template <int NP>
struct PairSums {
    float fr[NP], fi[NP], gr[NP], gi[NP];
    double ce;
};

// FP64 integration of one deferred pair (exact rule choice), used in place when
// the deferred list is full.
template <int NP, bool CPLX>
__device__ __noinline__ PairSums<NP> pair_fp64_inplace(const Fp64View &v, int64_t p, double tx, double ty,
                                                       double tz, double kre, double kim) {
    const double *r = v.rec + (size_t)p * v.stride;
    const int c = dev::nearest_node<NP>(r, tx, ty, tz);
    double dfr[NP], dfi[NP], dgr[NP], dgi[NP];
    PairSums<NP> out;
    out.ce = dev::element_fp64<NP, CPLX, df64::TrigDf>(r + v.ri.off[c], v.ri.Q[c], v.phi + (size_t)c * v.qmax * NP,
                                         tx, ty, tz, kre, kim, dfr, dfi, dgr, dgi);
#pragma unroll
    for (int a = 0; a < NP; ++a) {
        out.fr[a] = (float)dfr[a];
        out.fi[a] = (float)dfi[a];
        out.gr[a] = (float)dgr[a];
        out.gi[a] = (float)dgi[a];
    }
    return out;
}

// Quadrature loop of one regular pair: per-node sums of F, G and the C term.
// QN > 0: the rule size is known at compile time (4-point corner and 8-point
// midpoint rules of n = m = 2), the loop is unrolled and the independent
// points interleave; QN == 0: runtime size Q.
template <int NP, bool CPLX_K, int QN>
__device__ __forceinline__ void quad_loop(const float4 *g4, const float *phc, int Q, const mixed::PairSetup &P,
                                          const mixed::Phase &ph, float kf, float kimf, float (&fr)[NP],
                                          float (&fi)[NP], float (&gr)[NP], float (&gi)[NP], float &ce) {
    constexpr int NPP = PhiPad<NP>::value;
    const int nq = QN > 0 ? QN : Q;
#pragma unroll
    for (int q = 0; q < (QN > 0 ? QN : 1); ++q) {
        if (QN == 0) break;
        const mixed::QpeValues v = mixed::qpe<CPLX_K>(g4[2 * q], g4[2 * q + 1], P, ph, kf, kimf);
        ce += v.tq;
        float p[NPP];
        *reinterpret_cast<float4 *>(p) = *reinterpret_cast<const float4 *>(phc + q * NPP);
        if (NPP == 8) *reinterpret_cast<float4 *>(p + 4) = *reinterpret_cast<const float4 *>(phc + q * NPP + 4);
#pragma unroll
        for (int a = 0; a < NP; ++a) {
            fr[a] = __fmaf_rn(v.Fr, p[a], fr[a]);
            fi[a] = __fmaf_rn(v.Fi, p[a], fi[a]);
            gr[a] = __fmaf_rn(v.Gr, p[a], gr[a]);
            gi[a] = __fmaf_rn(v.Gi, p[a], gi[a]);
        }
    }
    if (QN == 0) {
        for (int q = 0; q < nq; ++q) {
            const mixed::QpeValues v = mixed::qpe<CPLX_K>(g4[2 * q], g4[2 * q + 1], P, ph, kf, kimf);
            ce += v.tq;
            float p[NPP];
            *reinterpret_cast<float4 *>(p) = *reinterpret_cast<const float4 *>(phc + q * NPP);
            if (NPP == 8)
                *reinterpret_cast<float4 *>(p + 4) = *reinterpret_cast<const float4 *>(phc + q * NPP + 4);
#pragma unroll
            for (int a = 0; a < NP; ++a) {
                fr[a] = __fmaf_rn(v.Fr, p[a], fr[a]);
                fi[a] = __fmaf_rn(v.Fi, p[a], fi[a]);
                gr[a] = __fmaf_rn(v.Gr, p[a], gr[a]);
                gi[a] = __fmaf_rn(v.Gi, p[a], gi[a]);
            }
        }
    }
}

#ifndef BIE_K2_MIN_BLOCKS
#define BIE_K2_MIN_BLOCKS 4   // resident 128-thread blocks per SM (register budget)
#endif

// float -> double of an entry, two ways with the same (exact) result: integer
// bit moves (dev::f2d) for the streaming passes, whose FP64 pipe would be their
// bottleneck, and the conversion instruction for the assembly kernel, which
// is bound by instruction issue and leaves its FP64 pipe idle (2.30 vs 2.48 ms
// per assembly kernel at 11562 nodes with the integer form there)
__device__ __forceinline__ double2 widen2(float re, float im) { return make_double2(dev::f2d(re), dev::f2d(im)); }
__device__ __forceinline__ double2 widen2_cvt(float re, float im) { return make_double2((double)re, (double)im); }

// fire-and-forget vector FP32 reductions (red.global.add.v4 / .v2)
__device__ __forceinline__ void red4(float4 *p, float4 v) { atomicAdd(p, v); }
__device__ __forceinline__ void red2(float2 *p, float2 v) { atomicAdd(p, v); }

// Output of one pair's per-node sums to node a of its element under the write
// protocol (flag word fw: first / last / shared / ring bits of the element's
// nodes; slot: the node's side slot or ring slot).  Ring nodes sum in the
// thread's shared-memory slot (stride TPB float4s) and are written as final
// complex128 entries at their last contribution; other entries with several
// contributions keep float partial sums until the widening pass
// (k2_widen_kernel).
template <bool C64, int TPB>
__device__ __forceinline__ void k2_write(int a, uint32_t fw, int32_t slot, size_t off, int64_t i, int64_t M,
                                         bool doF, bool doG, float fr, float fi, float gr, float gi,
                                         void *__restrict__ Fo, void *__restrict__ Go, float4 *__restrict__ side,
                                         float4 *ring) {
    const bool first = (fw >> a) & 1u;
    if ((fw >> (16 + a)) & 1u) {   // shared node: this slice's sum in its side slot
        float4 *q = side + (size_t)slot * (size_t)M + (size_t)i;
        const float4 v = make_float4(fr, fi, gr, gi);
        if (first) *q = v;
        else red4(q, v);
        return;
    }
    if (!C64 && ((fw >> (24 + a)) & 1u)) {   // ring node: partial sums in shared memory
        float4 *q = ring + slot * TPB;
        float4 v = make_float4(fr, fi, gr, gi);
        if (!first) {
            const float4 o = *q;
            v.x = o.x + v.x;
            v.y = o.y + v.y;
            v.z = o.z + v.z;
            v.w = o.w + v.w;
        }
        if ((fw >> (8 + a)) & 1u) {
            double2 *pf = static_cast<double2 *>(Fo) + off, *pg = static_cast<double2 *>(Go) + off;
            if (doF) __stcs(pf, widen2_cvt(v.x, v.y));
            if (doG) __stcs(pg, widen2_cvt(v.z, v.w));
        } else {
            *q = v;
        }
        return;
    }
    if (C64) {   // complex64 matrices: the entry accumulates its own sum
        float2 *pf = static_cast<float2 *>(Fo) + off, *pg = static_cast<float2 *>(Go) + off;
        if (doF) {
            if (first) *pf = make_float2(fr, fi);
            else red2(pf, make_float2(fr, fi));
        }
        if (doG) {
            if (first) *pg = make_float2(gr, gi);
            else red2(pg, make_float2(gr, gi));
        }
        return;
    }
    double2 *pf = static_cast<double2 *>(Fo) + off, *pg = static_cast<double2 *>(Go) + off;
    if (first && ((fw >> (8 + a)) & 1u)) {   // the only contribution: final value at once
        if (doF) __stcs(pf, widen2_cvt(fr, fi));
        if (doG) __stcs(pg, widen2_cvt(gr, gi));
        return;
    }
    // partial sums (F re, F im, G re, G im) in the 16 bytes of one entry
    float4 *q = reinterpret_cast<float4 *>(doF ? pf : pg);
    const float4 v = make_float4(fr, fi, gr, gi);
    if (first) *q = v;
    else red4(q, v);
}

template <int NP, bool CPLX_K, bool C64, int TPB>
__global__ void __launch_bounds__(TPB, BIE_K2_MIN_BLOCKS * 128 / TPB)
assemble_mixed_kernel(const float *__restrict__ rec, int stride, int nidx_off, int64_t E, int S,
                      const float *__restrict__ phi, int nphi, int qmax, const __grid_constant__ RuleInfo ri,
                      const double *__restrict__ tgt, int64_t M, double kre, double kim, int flags,
                      void *__restrict__ Fo, void *__restrict__ Go, float4 *__restrict__ side,
                      const uint32_t *__restrict__ kflags, const int32_t *__restrict__ kside,
                      double *__restrict__ Cpart, int chunk, int2 *__restrict__ defer,
                      unsigned int *__restrict__ defer_count, unsigned int defer_cap,
                      const __grid_constant__ Fp64View v64, unsigned long long *__restrict__ qpe_count,
                      const double *__restrict__ kdev) {
    if (kdev) {   // wavenumber read from device memory (recorded sweeps)
        kre = kdev[0];
        kim = kdev[1];
    }
    constexpr int NPP = PhiPad<NP>::value;
    constexpr int kRing = C64 ? 0 : kK2RingSlots;
    extern __shared__ __align__(16) float smemf[];
    float *s_phi = smemf;                                   // nphi floats (padded to 4)
    float4 *s_ring = reinterpret_cast<float4 *>(smemf + ((nphi + 3) & ~3));   // kRing x TPB
    float *s_rec = reinterpret_cast<float *>(s_ring + kRing * TPB);            // chunk * stride floats
    uint32_t *s_flags = reinterpret_cast<uint32_t *>(s_rec + (size_t)chunk * stride);   // chunk
    int32_t *s_slot = reinterpret_cast<int32_t *>(s_flags + chunk);                     // chunk * NP

    const int s = blockIdx.y;
    const int64_t e0 = (int64_t)s * E / S;
    const int64_t e1 = (int64_t)(s + 1) * E / S;
    const int64_t i = (int64_t)blockIdx.x * TPB + threadIdx.x;
    const bool active = i < M;
    const bool doF = flags & BIE_F, doG = flags & BIE_G, doC = flags & BIE_C;
    const bool doFG = doF || doG;

    double tx = 0, ty = 0, tz = 0;
    if (active) {
        tx = tgt[3 * i + 0];
        ty = tgt[3 * i + 1];
        tz = tgt[3 * i + 2];
    }
    const mixed::Target T{dev::df_from_double(tx), dev::df_from_double(ty), dev::df_from_double(tz)};
    const df K = dev::df_from_double(kre);
    const float kf = K.hi;
    const float kimf = (float)kim;
    for (int t = threadIdx.x; t < nphi; t += TPB) s_phi[t] = phi[t];
    // the rule table in shared memory: indexed by each thread's nearest node,
    // it would otherwise be copied to local memory (divergent dynamic index)
    __shared__ RuleInfo s_ri;
    if (threadIdx.x == 0) s_ri = ri;

    df cacc = {0.f, 0.f};
    unsigned long long nqpe = 0;
    for (int64_t cb = e0; cb < e1; cb += chunk) {
        const int n = (int)min((int64_t)chunk, e1 - cb);
        __syncthreads();
        {
            const float4 *src = reinterpret_cast<const float4 *>(rec + cb * stride);
            float4 *dst = reinterpret_cast<float4 *>(s_rec);
            const int n4 = n * stride / 4;
            for (int t = threadIdx.x; t < n4; t += TPB) dst[t] = src[t];
            for (int t = threadIdx.x; t < n; t += TPB) s_flags[t] = kflags[cb + t];
            for (int t = threadIdx.x; t < n * NP; t += TPB) s_slot[t] = kside[cb * NP + t];
        }
        __syncthreads();
        if (!active) continue;

        for (int el = 0; el < n; ++el) {
            const float *r = s_rec + (size_t)el * stride;
            const int64_t p = cb + el;
            const mixed::PairSetup P = mixed::pair_setup<NP>(r, T);
            float fr[NP], fi[NP], gr[NP], gi[NP];
            float ce = 0.f;
            bool listed = false;   // integrated later by the FP64 correction kernel
#pragma unroll
            for (int a = 0; a < NP; ++a) fr[a] = fi[a] = gr[a] = gi[a] = 0.f;
            if (P.deferred) {
                const unsigned int slot = atomicAdd(defer_count, 1u);
                if (slot < defer_cap) {
                    defer[slot] = make_int2((int)i, (int)p);
                    listed = true;
                } else {
                    const PairSums<NP> ps = pair_fp64_inplace<NP, CPLX_K>(v64, p, tx, ty, tz, kre, kim);
#pragma unroll
                    for (int a = 0; a < NP; ++a) {
                        fr[a] = ps.fr[a];
                        fi[a] = ps.fi[a];
                        gr[a] = ps.gr[a];
                        gi[a] = ps.gi[a];
                    }
                    ce = (float)(-ps.ce);   // stored with the sign of the FP32 path below
                }
            } else {
                const mixed::Phase ph = mixed::pair_phase(P, K);
                const int c = P.c;
                const int Q = s_ri.Q[c];
                nqpe += Q;
                const float4 *g4 = reinterpret_cast<const float4 *>(r + s_ri.off[c]);
                const float *phc = s_phi + (size_t)c * qmax * NPP;
                // blocks of four points (one unrolled body for the 4- and
                // 8-point rules keeps the kernel's code small), then the rest
                int q = 0;
                for (; q + 4 <= Q; q += 4)
                    quad_loop<NP, CPLX_K, 4>(g4 + 2 * q, phc + q * NPP, 4, P, ph, kf, kimf, fr, fi, gr, gi, ce);
                if (q < Q)
                    quad_loop<NP, CPLX_K, 0>(g4 + 2 * q, phc + q * NPP, Q - q, P, ph, kf, kimf, fr, fi, gr, gi, ce);
            }
            if (!listed) mixed::df_accum(cacc, -ce);   // C = -sum tq
            if (!doFG) continue;
            const uint32_t fw = s_flags[el];
            const int32_t *nid = reinterpret_cast<const int32_t *>(r + nidx_off);
#pragma unroll
            for (int a = 0; a < NP; ++a) {
                // a listed pair adds nothing: only its first stores (zero) and
                // a ring node's last contribution (the final write) remain
                if (listed && !((fw >> a) & 1u) && !(kRing && ((fw >> (24 + a)) & (fw >> (8 + a)) & 1u)))
                    continue;
                k2_write<C64, TPB>(a, fw, s_slot[el * NP + a], (size_t)nid[a] * (size_t)M + (size_t)i, i, M, doF,
                                   doG, fr[a], fi[a], gr[a], gi[a], Fo, Go, side, s_ring + threadIdx.x);
            }
        }
    }
    if (active && doC) Cpart[(int64_t)s * M + i] = dev::f2d(cacc.hi) + dev::f2d(cacc.lo);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) nqpe += __shfl_down_sync(0xffffffffu, nqpe, o);
    if ((threadIdx.x & 31) == 0 && nqpe) atomicAdd(qpe_count, nqpe);
}

// Entries of the nodes with several contributions in their one slice: the
// float4 partial sums (F re, F im, G re, G im) in the first 16 bytes of each
// entry become the complex128 F and G entries, in place.
__global__ void k2_widen_kernel(int64_t M, const int32_t *__restrict__ wnode, int64_t nw, int flags,
                                double2 *__restrict__ F, double2 *__restrict__ G) {
    const bool doF = flags & BIE_F, doG = flags & BIE_G;
    const int64_t total = nw * M;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t n = t / M;
        const size_t off = (size_t)wnode[n] * (size_t)M + (size_t)(t - n * M);
        const float4 v = __ldcs(reinterpret_cast<const float4 *>((doF ? F : G) + off));
        if (doF) __stcs(F + off, widen2(v.x, v.y));
        if (doG) __stcs(G + off, widen2(v.z, v.w));
    }
}

// Columns of the nodes shared between slices: sum of the slices' side slots
// (nodes touched by no element: zero), written as complex128 or complex64.
template <bool C64>
__global__ void k2_fixup_kernel(const float4 *__restrict__ side, int64_t M, const int32_t *__restrict__ fnode,
                                const int32_t *__restrict__ fptr, const int32_t *__restrict__ fslot, int64_t nfix,
                                int flags, void *__restrict__ Fo, void *__restrict__ Go) {
    const bool doF = flags & BIE_F, doG = flags & BIE_G;
    const int64_t total = nfix * M;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t n = t / M;
        const int64_t i = t - n * M;
        float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int32_t q = fptr[n]; q < fptr[n + 1]; ++q) {
            const float4 v = __ldcs(side + (size_t)fslot[q] * (size_t)M + (size_t)i);
            acc.x += v.x;
            acc.y += v.y;
            acc.z += v.z;
            acc.w += v.w;
        }
        const size_t off = (size_t)fnode[n] * (size_t)M + (size_t)i;
        if (C64) {
            if (doF) static_cast<float2 *>(Fo)[off] = make_float2(acc.x, acc.y);
            if (doG) static_cast<float2 *>(Go)[off] = make_float2(acc.z, acc.w);
        } else {
            if (doF) static_cast<double2 *>(Fo)[off] = widen2(acc.x, acc.y);
            if (doG) static_cast<double2 *>(Go)[off] = widen2(acc.z, acc.w);
        }
    }
}

__device__ __forceinline__ void add_entry(double2 *p, double re, double im) {
    atomicAdd(&p->x, re);
    atomicAdd(&p->y, im);
}
__device__ __forceinline__ void add_entry(float2 *p, double re, double im) {
    atomicAdd(p, make_float2((float)re, (float)im));
}

// FP64 integration of the deferred pairs; results added atomically to the
// complex128 output (or to the complex64 accumulators when the caller keeps
// complex64 matrices).
template <int NP, bool CPLX_K, typename T2>
__global__ void __launch_bounds__(128)
correct_fp64_kernel(const int2 *__restrict__ defer, const unsigned int *__restrict__ defer_count,
                    unsigned int defer_cap, const __grid_constant__ Fp64View v, const double *__restrict__ tgt,
                    int64_t M,
                    double kre, double kim, int flags, T2 *__restrict__ F,
                    T2 *__restrict__ G, double *__restrict__ Cnear,
                    unsigned long long *__restrict__ qpe_count, const double *__restrict__ kdev,
                    const double2 *__restrict__ gweight = nullptr) {
    if (kdev) {
        kre = kdev[0];
        kim = kdev[1];
    }
    const unsigned int n = min(*defer_count, defer_cap);
    const bool doF = flags & BIE_F, doG = flags & BIE_G, doC = flags & BIE_C;
    unsigned long long nqpe = 0;
    for (unsigned int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const int2 pr = defer[j];
        const int64_t i = pr.x;
        const double *r = v.rec + (size_t)pr.y * v.stride;
        const double tx = tgt[3 * i], ty = tgt[3 * i + 1], tz = tgt[3 * i + 2];
        const int c = dev::nearest_node<NP>(r, tx, ty, tz);
        nqpe += v.ri.Q[c];
        double fr[NP], fi[NP], gr[NP], gi[NP];
        const double ce = dev::element_fp64<NP, CPLX_K, df64::TrigDf>(r + v.ri.off[c], v.ri.Q[c],
                                                        v.phi + (size_t)c * v.qmax * NP, tx, ty, tz,
                                                        kre, kim, fr, fi, gr, gi);
        if (gweight && doG) {   // element factor on the single layer
            const double2 w = gweight[pr.y];
#pragma unroll
            for (int a = 0; a < NP; ++a) {
                const double t = gr[a] * w.x - gi[a] * w.y;
                gi[a] = gr[a] * w.y + gi[a] * w.x;
                gr[a] = t;
            }
        }
        const int32_t *nid = reinterpret_cast<const int32_t *>(r + v.nidx_off);
#pragma unroll
        for (int a = 0; a < NP; ++a) {
            const size_t off = (size_t)nid[a] * (size_t)M + (size_t)i;
            if (doF) add_entry(F + off, fr[a], fi[a]);
            if (doG) add_entry(G + off, gr[a], gi[a]);
        }
        if (doC) atomicAdd(&Cnear[i], ce);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) nqpe += __shfl_down_sync(0xffffffffu, nqpe, o);
    if ((threadIdx.x & 31) == 0 && nqpe) atomicAdd(qpe_count, nqpe);
}

template <int NP, bool CPLX, bool C64>
void launch_np(Ctx &c, const AssembleArgs &a, int level, size_t smem, int chunk, int tpb, float4 *side,
               double *Cpart, int2 *defer, unsigned int *dcount, unsigned int dcap, double *Cnear) {
    const RecordLayout &L = c.lay;
    const MixedLayout &X = c.mlay;
    const int S = 1 << level;
    RuleInfo ri{}, ri64{};
    for (int r = 0; r < L.R; ++r) {
        ri.Q[r] = L.Q[r];
        ri.off[r] = X.rule_off[r];
        ri64.Q[r] = L.Q[r];
        ri64.off[r] = L.rule_off[r];
    }
    Fp64View v{c.d_records, L.stride, L.nidx_off, c.d_phi, L.qmax, ri64};
    auto kern = tpb == 256 ? assemble_mixed_kernel<NP, CPLX, C64, 256> : assemble_mixed_kernel<NP, CPLX, C64, 128>;
    BIE_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grid((unsigned)((a.M + tpb - 1) / tpb), (unsigned)S);
    const int64_t E = c.n_elements;
    cudaEvent_t t0 = c.timer_begin();
    kern<<<grid, tpb, smem, c.stream>>>(
        c.d_mrecords, X.stride, X.nidx_off, E, S, c.d_mphi, L.R * L.qmax * PhiPad<NP>::value, L.qmax, ri,
        a.targets, a.M, a.k_re, a.k_im, a.flags, a.F, a.G, side, c.d_k2_flags + (size_t)level * E,
        c.d_k2_side + (size_t)level * E * NP, Cpart, chunk, defer, dcount, dcap, v, c.d_qpe, a.k_dev);
    BIE_CUDA(cudaGetLastError());
    c.timer_end(t0);
    ++c.kernel_launches;

    const int64_t nfix = c.k2_nfix[level];
    if (nfix > 0 && (a.flags & (BIE_F | BIE_G))) {
        const int32_t *fnode = c.d_k2_fix + c.k2_fix_off[level];
        const int32_t *fptr = fnode + nfix;
        const int32_t *fslot = fptr + nfix + 1;
        const int64_t total = nfix * a.M;
        const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 16LL * c.num_sms));
        k2_fixup_kernel<C64><<<g, 256, 0, c.stream>>>(side, a.M, fnode, fptr, fslot, nfix, a.flags, a.F, a.G);
        BIE_CUDA(cudaGetLastError());
        ++c.kernel_launches;
    }
    const int64_t nw = c.k2_nwiden[level];
    if (!C64 && nw > 0 && (a.flags & (BIE_F | BIE_G))) {
        const int64_t total = nw * a.M;
        const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 16LL * c.num_sms));
        k2_widen_kernel<<<g, 256, 0, c.stream>>>(a.M, c.d_k2_fix + c.k2_widen_off[level], nw, a.flags,
                                                 reinterpret_cast<double2 *>(a.F), reinterpret_cast<double2 *>(a.G));
        BIE_CUDA(cudaGetLastError());
        ++c.kernel_launches;
    }
    // FP64 corrections of the deferred pairs, added to the finished entries
    using T2 = typename std::conditional<C64, float2, double2>::type;
    correct_fp64_kernel<NP, CPLX, T2><<<(unsigned)(4 * c.num_sms), 128, 0, c.stream>>>(
        defer, dcount, dcap, v, a.targets, a.M, a.k_re, a.k_im, a.flags, reinterpret_cast<T2 *>(a.F),
        reinterpret_cast<T2 *>(a.G), Cnear, c.d_qpe, a.k_dev);
    BIE_CUDA(cudaGetLastError());
    ++c.kernel_launches;
}

}  // namespace

void build_df64_records(Ctx &c, const std::vector<double> &rec64, const std::vector<float> &mrec);

void build_mixed_records(Ctx &c, const std::vector<double> &rec64) {
    const RecordLayout &L = c.lay;
    MixedLayout &X = c.mlay;
    X = MixedLayout{};
    const int NP = L.NP;
    const int NPP = NP <= 4 ? 4 : 8;
    int off = (8 + 3 * NP + 3) & ~3;
    for (int r = 0; r < L.R; ++r) {
        X.rule_off[r] = off;
        off += 8 * L.Q[r];
    }
    X.nidx_off = off;
    off += NP;
    X.stride = (off + 3) & ~3;
    const int64_t E = c.n_elements;
    std::vector<float> rec((size_t)E * X.stride, 0.f);
    for (int64_t p = 0; p < E; ++p) {
        const int64_t e = c.order[p];
        const double *R0 = &rec64[(size_t)p * L.stride];
        float *W = &rec[(size_t)p * X.stride];
        double cen[3] = {0, 0, 0}, hmax = 0;
        for (int a = 0; a < 3; ++a)
            for (int k = 0; k < 3; ++k) cen[k] += c.coords[3 * (int64_t)c.topo[c.NS * e + a] + k] / 3.0;
        for (int a = 0; a < 3; ++a) {
            const double *A = &c.coords[3 * (int64_t)c.topo[c.NS * e + a]];
            const double *B = &c.coords[3 * (int64_t)c.topo[c.NS * e + (a + 1) % 3]];
            hmax = std::max(hmax, std::sqrt((A[0] - B[0]) * (A[0] - B[0]) + (A[1] - B[1]) * (A[1] - B[1]) +
                                            (A[2] - B[2]) * (A[2] - B[2])));
        }
        // header: c_hi x y z, c_lo x | c_lo y z, near radius^2, 0
        for (int k = 0; k < 3; ++k) W[k] = (float)cen[k];
        W[3] = (float)(cen[0] - (double)W[0]);
        W[4] = (float)(cen[1] - (double)W[1]);
        W[5] = (float)(cen[2] - (double)W[2]);
        W[6] = (float)(hmax * hmax);   // near: centroid within one element size
        for (int a = 0; a < NP; ++a)
            for (int k = 0; k < 3; ++k) W[8 + 3 * a + k] = (float)(R0[3 * a + k] - cen[k]);
        for (int r = 0; r < L.R; ++r) {
            const int Q = L.Q[r];
            const double *g = R0 + L.rule_off[r];
            float *w = W + X.rule_off[r];
            for (int q = 0; q < Q; ++q) {
                const float ox = (float)(g[q] - cen[0]), oy = (float)(g[Q + q] - cen[1]),
                            oz = (float)(g[2 * Q + q] - cen[2]);
                float *P = w + 8 * q;
                P[0] = ox;
                P[1] = oy;
                P[2] = oz;
                P[3] = (float)(g[6 * Q + q] * 0.07957747154594767);    // jw / (4 pi)
                P[4] = (float)g[3 * Q + q];
                P[5] = (float)g[4 * Q + q];
                P[6] = (float)g[5 * Q + q];
                // |o|^2 of the rounded offsets, so that 2 D.o + |o|^2 = |D + o|^2 - |D|^2
                P[7] = (float)((double)ox * ox + (double)oy * oy + (double)oz * oz);
            }
        }
        int32_t *nid = reinterpret_cast<int32_t *>(W + X.nidx_off);
        for (int a = 0; a < NP; ++a) nid[a] = c.ptopo[NP * e + a];
    }
    // Phi[r][q][a] padded to NPP columns
    std::vector<float> phi32((size_t)L.R * L.qmax * NPP, 0.f);
    for (int r = 0; r < L.R; ++r)
        for (int q = 0; q < L.qmax; ++q)
            for (int a = 0; a < NP; ++a)
                phi32[((size_t)r * L.qmax + q) * NPP + a] = (float)c.phi[((size_t)r * L.qmax + q) * NP + a];
    BIE_CUDA(cudaMalloc(&c.d_mrecords, rec.size() * sizeof(float)));
    BIE_CUDA(cudaMalloc(&c.d_mphi, phi32.size() * sizeof(float)));
    BIE_CUDA(cudaMemcpy(c.d_mrecords, rec.data(), rec.size() * sizeof(float), cudaMemcpyHostToDevice));
    BIE_CUDA(cudaMemcpy(c.d_mphi, phi32.data(), phi32.size() * sizeof(float), cudaMemcpyHostToDevice));
    build_df64_records(c, rec64, rec);
}

void launch_assemble_mixed(Ctx &c, const AssembleArgs &a) {
    const RecordLayout &L = c.lay;
    if (!(a.flags & (BIE_F | BIE_G | BIE_C))) return;

    // deferred-pair list: M x 64 entries + counter + near C (M doubles)
    const unsigned int dcap = (unsigned int)std::min<int64_t>(a.M * 64 + 4096, (int64_t)1 << 30);
    const size_t dbytes = (size_t)dcap * sizeof(int2);
    char *dbuf = static_cast<char *>(c.scratch(kScratchDefer, dbytes + 256 + (size_t)a.M * 8));
    int2 *defer = reinterpret_cast<int2 *>(dbuf);
    unsigned int *dcount = reinterpret_cast<unsigned int *>(dbuf + dbytes);
    double *Cnear = reinterpret_cast<double *>(dbuf + dbytes + 256);
    BIE_CUDA(cudaMemsetAsync(dbuf + dbytes, 0, 256 + (size_t)a.M * 8, c.stream));

    const int NPP = L.NP <= 4 ? 4 : 8;
    const size_t rec_bytes = (size_t)c.mlay.stride * sizeof(float);
    const size_t phi_f = (size_t)((L.R * L.qmax * NPP + 3) & ~3);
    // per element: record, flag word, NP slot indices; the ring of partial
    // sums (complex128 outputs only) takes kK2RingSlots float4s per thread
    const size_t el_bytes = rec_bytes + 4 + 4 * (size_t)L.NP;
    const size_t ring128 = a.c64_out ? 0 : (size_t)kK2RingSlots * 128 * 16;
    // four 128-thread blocks per SM: 228 KB of shared memory less 1 KB per block
    const size_t blk_budget = (228u << 10) / 4 - (1u << 10);
    const size_t fit = blk_budget > phi_f * 4 + ring128 ? (blk_budget - phi_f * 4 - ring128) / el_bytes : 1;
    const int chunk0 = (int)std::max<size_t>(1, std::min<size_t>({64, (24u << 10) / rec_bytes, fit}));
    const bool cplx = a.k_im != 0.0;
    const bool fg = (a.flags & (BIE_F | BIE_G)) != 0;
    auto run = [&](const LaunchShape &sh) {
        const int level = sh.level, chunk = sh.chunk, tpb = sh.tpb;
        const size_t ring = a.c64_out ? 0 : (size_t)kK2RingSlots * tpb * 16;
        const size_t smem = phi_f * sizeof(float) + ring + (size_t)chunk * el_bytes;
        if (smem > (227u << 10))
            fail(BIE_ERR_INVALID, "mixed assembly shape (chunk " + std::to_string(chunk) + ", " +
                                      std::to_string(tpb) + " threads) needs " + std::to_string(smem) +
                                      " bytes of shared memory per block, more than 232448");
        const int S = 1 << level;
        double *Cpart = static_cast<double *>(c.scratch(kScratchCpart, (size_t)S * a.M * sizeof(double)));
        float4 *side = fg ? static_cast<float4 *>(c.scratch(kScratchK2Side, (size_t)c.k2_nside[level] * a.M * 16))
                          : nullptr;
#define BIE_K2_LAUNCH(NP_)                                                                                      \
    do {                                                                                                        \
        if (a.c64_out) {                                                                                        \
            if (cplx) launch_np<NP_, true, true>(c, a, level, smem, chunk, tpb, side, Cpart, defer, dcount, dcap, Cnear); \
            else launch_np<NP_, false, true>(c, a, level, smem, chunk, tpb, side, Cpart, defer, dcount, dcap, Cnear);    \
        } else {                                                                                                \
            if (cplx) launch_np<NP_, true, false>(c, a, level, smem, chunk, tpb, side, Cpart, defer, dcount, dcap, Cnear); \
            else launch_np<NP_, false, false>(c, a, level, smem, chunk, tpb, side, Cpart, defer, dcount, dcap, Cnear);    \
        }                                                                                                       \
    } while (0)
        if (L.NP == 1) BIE_K2_LAUNCH(1);
        else if (L.NP == 3) BIE_K2_LAUNCH(3);
        else BIE_K2_LAUNCH(6);
#undef BIE_K2_LAUNCH
        if (a.flags & BIE_C) launch_reduce_c(c, Cpart, S, Cnear, a.M, a.C);
    };
    auto reset = [&] {   // fresh deferred list (every entry of F, G is overwritten)
        BIE_CUDA(cudaMemsetAsync(dbuf + dbytes, 0, 256 + (size_t)a.M * 8, c.stream));
    };
    // launch shape: the heuristic one, the autotuner's choice for this M, or
    // one a caller forced (bie_ctx_set_shape)
    const LaunchShape base{wave_slice_level(c, a.M, kThreads), chunk0, kThreads};
    ShapeAxes ax;
    for (int l = base.level - 1; l <= base.level + 1; ++l)
        if (l >= 0 && l < kMaxLevels && (int64_t(1) << l) <= c.n_elements) ax.levels.push_back(l);
    ax.chunks = {std::max(1, chunk0 / 2), chunk0, std::min(64, 2 * chunk0)};
    ax.tpbs = {128, 256};
    const LaunchShape sh = resolve_shape(c, kShapeK2, a.M, base, ax, run, reset);
    run(sh);
}

// ===========================================================================
// K9: FP64-grade assembly in double-float arithmetic (BIE_PREC_DF64).
//
// GB300 runs FP32 FMAs at ~73x its FP64 rate.  K9 keeps K2's structure
// (thread per target, element records staged in shared memory, near pairs and
// nearest-node near-ties deferred to the FP64 correction kernel) but evaluates
// every regular quadrature point in double-float arithmetic (pairs of floats,
// ~48-bit significand) instead of FP32, so F, G and C agree with the FP64
// assembly to ~1e-14 relative rather than ~1e-7:
//   * per pair: D = c_e - t and r0 = |D| in double-float; e^{i k r0} from a
//     double-float sine/cosine with a quadrant reduction by a four-part pi/2;
//   * per point: r = |D + o| (o = x_q - c_e stored in double-float), the
//     phase rotation e^{i k (r - r0)} from Taylor polynomials whose degree the
//     host picks from k and the largest |o| of the mesh, the kernels of
//     greens3d! / freens3d! / freens3dk0! (src/3d/kernels.jl:13-55) and the
//     per-node sums (mygemm_vec!, src/2d/assembly_collocation.jl:142-150)
//     all in double-float;
//   * F, G are written as complex128 (the owning thread's read-modify-write,
//     or FP64 atomics on nodes shared between element slices), C per slice.
// The Taylor coefficients (-1)^j/(2j)!, (-1)^j/(2j+1)!, 1/j! are stored as
// hi + lo float pairs (to ~2^-49 relative).
// ===========================================================================
namespace {

using namespace df64;

// entry (re, im) kept as double-float pairs: += (a, b)
__device__ __forceinline__ void dd_rmw(float4 *p, const dd::Acc &a, const dd::Acc &b) {
    float4 w = *p;
    const dev::df re = dev::df_add(dev::df{w.x, w.y}, dev::fast_two_sum(a.hi, a.lo));
    const dev::df im = dev::df_add(dev::df{w.z, w.w}, dev::fast_two_sum(b.hi, b.lo));
    w.x = re.hi;
    w.y = re.lo;
    w.z = im.hi;
    w.w = im.lo;
    *p = w;
}

// complex128 entries of the nodes not shared between element slices held
// (re_hi, re_lo, im_hi, im_lo) floats during the assembly: widen them in
// place (entry (i, j) at j M + i; shared nodes already hold doubles)
__global__ void df_widen_kernel(double2 *__restrict__ F, int64_t M, int64_t N,
                                const uint8_t *__restrict__ node_shared) {
    const int64_t total = M * N;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += stride) {
        const int64_t j = t / M;
        if (node_shared[j]) continue;
        const float4 w = reinterpret_cast<const float4 *>(F)[t];
        F[t] = make_double2(dev::f2d(w.x) + dev::f2d(w.y), dev::f2d(w.z) + dev::f2d(w.w));
    }
}

#ifndef BIE_K9_MIN_BLOCKS
#define BIE_K9_MIN_BLOCKS 2   // resident 128-thread blocks per SM (register budget)
#endif
#ifndef BIE_K9_UNROLL
#define BIE_K9_UNROLL 1       // quadrature points interleaved per iteration
#endif
constexpr int kK9Unroll = BIE_K9_UNROLL;

// FP64 integration of one pair of the double-float assembly whose deferred
// list is full, with its writes; returns the pair's C term.  Out of line so
// that this rare path does not sit in the middle of the kernel's hot loop
// (instruction fetch).
template <int NP, bool CPLX_K>
__device__ __noinline__ double k9_pair_inplace(const Fp64View &v64, int64_t p, double tx, double ty, double tz,
                                               double kre, double kim, const double2 *__restrict__ gweight,
                                               bool doF, bool doG, int64_t M, int64_t i, double2 *__restrict__ F,
                                               double2 *__restrict__ G, uint32_t m) {
    const double *r64 = v64.rec + (size_t)p * v64.stride;
    const int cn = dev::nearest_node<NP>(r64, tx, ty, tz);
    double fr[NP], fi[NP], gr[NP], gi[NP];
    const double ce = dev::element_fp64<NP, CPLX_K, df64::TrigDf>(r64 + v64.ri.off[cn], v64.ri.Q[cn],
                                                                  v64.phi + (size_t)cn * v64.qmax * NP, tx, ty, tz,
                                                                  kre, kim, fr, fi, gr, gi);
    if (gweight && doG) {
        const double2 w = gweight[p];
#pragma unroll
        for (int a = 0; a < NP; ++a) {
            const double t = gr[a] * w.x - gi[a] * w.y;
            gi[a] = gr[a] * w.y + gi[a] * w.x;
            gr[a] = t;
        }
    }
    const int32_t *nid = reinterpret_cast<const int32_t *>(r64 + v64.nidx_off);
    auto acc_of = [](double x) {
        const dev::df t = dd::to_df(x);
        return dd::Acc{t.hi, t.lo};
    };
#pragma unroll
    for (int a = 0; a < NP; ++a) {
        const size_t off = (size_t)nid[a] * (size_t)M + (size_t)i;
        if ((m >> a) & 1u) {
            if (doF) add_entry(F + off, fr[a], fi[a]);
            if (doG) add_entry(G + off, gr[a], gi[a]);
        } else {   // float-pair entry (see the kernel)
            if (doF) dd_rmw(reinterpret_cast<float4 *>(F + off), acc_of(fr[a]), acc_of(fi[a]));
            if (doG) dd_rmw(reinterpret_cast<float4 *>(G + off), acc_of(gr[a]), acc_of(gi[a]));
        }
    }
    return ce;
}

template <int NP, bool CPLX_K>
__global__ void __launch_bounds__(kThreads, BIE_K9_MIN_BLOCKS)
assemble_df64_kernel(const float *__restrict__ rec, int stride, int nidx_off, int64_t E, int S,
                     const uint32_t *__restrict__ smask, const float2 *__restrict__ phi, int nphi, int qmax,
                     RuleInfo ri, const double *__restrict__ tgt, int64_t M, double kre, double kim,
                     int flags, double2 *__restrict__ F, double2 *__restrict__ G,
                     double *__restrict__ Cpart, int chunk, int2 *__restrict__ defer,
                     unsigned int *__restrict__ defer_count, unsigned int defer_cap,
                     const __grid_constant__ Fp64View v64, DfDegrees deg, unsigned long long *__restrict__ qpe_count, const double *__restrict__ kdev,
                     const double2 *__restrict__ gweight) {
    using dev::df;
    if (kdev) {   // wavenumber read from device memory (recorded sweeps)
        kre = kdev[0];
        kim = kdev[1];
    }
    extern __shared__ __align__(16) float smemf[];
    float2 *s_phi = reinterpret_cast<float2 *>(smemf);             // nphi (hi, lo) pairs
    float *s_rec = smemf + ((2 * nphi + 3) & ~3);                     // chunk * stride floats
    uint32_t *s_mask = reinterpret_cast<uint32_t *>(s_rec + (size_t)chunk * stride);

    const int s = blockIdx.y;
    const int64_t e0 = (int64_t)s * E / S;
    const int64_t e1 = (int64_t)(s + 1) * E / S;
    const int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x;
    const bool active = i < M;
    const bool doF = flags & BIE_F, doG = flags & BIE_G, doC = flags & BIE_C;

    double tx = 0, ty = 0, tz = 0;
    if (active) {
        tx = tgt[3 * i + 0];
        ty = tgt[3 * i + 1];
        tz = tgt[3 * i + 2];
    }
    const mixed::Target T{dev::df_from_double(tx), dev::df_from_double(ty), dev::df_from_double(tz)};
    const df K = dd::to_df(kre);
    const df Ki = dd::to_df(kim);
    for (int t = threadIdx.x; t < nphi; t += kThreads) s_phi[t] = phi[t];
    __shared__ RuleInfo s_ri;   // indexed by each thread's nearest node (see the mixed kernel)
    if (threadIdx.x == 0) s_ri = ri;

    dd::Acc cacc{0.f, 0.f};
    unsigned long long nqpe = 0;
    for (int64_t cb = e0; cb < e1; cb += chunk) {
        const int n = (int)min((int64_t)chunk, e1 - cb);
        __syncthreads();
        {
            const float4 *src = reinterpret_cast<const float4 *>(rec + cb * stride);
            float4 *dst = reinterpret_cast<float4 *>(s_rec);
            const int n4 = n * stride / 4;
            for (int t = threadIdx.x; t < n4; t += kThreads) dst[t] = src[t];
            for (int t = threadIdx.x; t < n; t += kThreads) s_mask[t] = smask[cb + t];
        }
        __syncthreads();
        if (!active) continue;

        for (int el = 0; el < n; ++el) {
            const float *r = s_rec + (size_t)el * stride;
            const mixed::PairSetup P = mixed::pair_setup<NP>(r, T);
            // r0 = |c_e - t| and the phase k r0 in double-float
            const df r0 = dd::sqrt_df(dev::df_add(dev::df_add(dev::df_sqr(P.Dxd), dev::df_sqr(P.Dyd)),
                                                  dev::df_sqr(P.Dzd)));
            const df kr0 = dev::df_mul(K, r0);
            if (P.deferred || !(fabsf(kr0.hi) < kDfMaxPhase)) {
                const unsigned int slot = atomicAdd(defer_count, 1u);
                if (slot < defer_cap) {
                    defer[slot] = make_int2((int)i, (int)(cb + el));
                    continue;
                }
                // list full: the pair in FP64 here (slower, same result)
                const double ce = k9_pair_inplace<NP, CPLX_K>(v64, cb + el, tx, ty, tz, kre, kim, gweight, doF, doG,
                                                              M, i, F, G, s_mask[el]);
                dd::acc_add(cacc, dd::to_df(ce));
                continue;
            }
            df E0r, E0i;
            pair_phase_df64<CPLX_K>(kr0, r0, kim, E0r, E0i);
            const int c = P.c;
            const int Q = s_ri.Q[c];
            nqpe += Q;
            const float4 *g4 = reinterpret_cast<const float4 *>(r + s_ri.off[c]);
            const float2 *phc = s_phi + (size_t)c * qmax * NP;
            dd::Acc fr[NP], fi[NP], gr[NP], gi[NP];
#pragma unroll
            for (int a = 0; a < NP; ++a) fr[a] = fi[a] = gr[a] = gi[a] = dd::Acc{0.f, 0.f};
            dd::Acc ce{0.f, 0.f};
#pragma unroll(kK9Unroll)
            for (int q = 0; q < Q; ++q) {
                df Fr, Fi, Gr, Gi, tq;
                qpe_df64<CPLX_K>(g4[4 * q], g4[4 * q + 1], g4[4 * q + 2], g4[4 * q + 3], P, r0, E0r, E0i, K, Ki,
                                 deg, Fr, Fi, Gr, Gi, tq);
                dd::acc_add(ce, tq);
                const float2 *pq = phc + q * NP;
#pragma unroll
                for (int a = 0; a < NP; ++a) {
                    const float2 pv = pq[a];
                    const df ph{pv.x, pv.y};
                    dd::acc_add(fr[a], dd::mul_raw(Fr, ph));
                    dd::acc_add(fi[a], dd::mul_raw(Fi, ph));
                    dd::acc_add(gr[a], dd::mul_raw(Gr, ph));
                    dd::acc_add(gi[a], dd::mul_raw(Gi, ph));
                }
            }
            // C = -sum t
            dd::acc_add(cacc, dd::neg(dev::fast_two_sum(ce.hi, ce.lo)));
            if (gweight && doG) {   // element factor on the single layer, in double-float
                const double2 w = gweight[cb + el];
                const df wr = dd::to_df(w.x), wi = dd::to_df(w.y);
#pragma unroll
                for (int a = 0; a < NP; ++a) {
                    const df xr = dev::fast_two_sum(gr[a].hi, gr[a].lo), xi = dev::fast_two_sum(gi[a].hi, gi[a].lo);
                    const df yr = dev::df_sub(dev::df_mul(xr, wr), dev::df_mul(xi, wi));
                    const df yi = dev::df_add(dev::df_mul(xr, wi), dev::df_mul(xi, wr));
                    gr[a] = dd::Acc{yr.hi, yr.lo};
                    gi[a] = dd::Acc{yi.hi, yi.lo};
                }
            }
            const int32_t *nid = reinterpret_cast<const int32_t *>(r + nidx_off);
            const uint32_t m = s_mask[el];
#pragma unroll
            for (int a = 0; a < NP; ++a) {
                const size_t off = (size_t)nid[a] * (size_t)M + (size_t)i;
                if ((m >> a) & 1u) {
                    // node shared with another element slice: FP64 atomics into
                    // the complex128 entry
                    if (doF) add_entry(F + off, dd::acc_value(fr[a]), dd::acc_value(fi[a]));
                    if (doG) add_entry(G + off, dd::acc_value(gr[a]), dd::acc_value(gi[a]));
                } else {
                    // owned by this thread: the entry holds (re_hi, re_lo, im_hi,
                    // im_lo) floats until df_widen_kernel, no FP64 instruction here
                    if (doF) dd_rmw(reinterpret_cast<float4 *>(F + off), fr[a], fi[a]);
                    if (doG) dd_rmw(reinterpret_cast<float4 *>(G + off), gr[a], gi[a]);
                }
            }
        }
    }
    if (active && doC) Cpart[(int64_t)s * M + i] = dd::acc_value(cacc);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) nqpe += __shfl_down_sync(0xffffffffu, nqpe, o);
    if ((threadIdx.x & 31) == 0 && nqpe) atomicAdd(qpe_count, nqpe);
}

template <int NP, bool CPLX>
void launch_df64_np(Ctx &c, const AssembleArgs &a, int S, int level, size_t smem, int chunk, double *Cpart,
                    int2 *defer, unsigned int *dcount, unsigned int dcap, double *Cnear, DfDegrees deg) {
    const RecordLayout &L = c.lay;
    const Df64Layout &X = c.dlay;
    RuleInfo ri{}, ri64{};
    for (int r = 0; r < L.R; ++r) {
        ri.Q[r] = L.Q[r];
        ri.off[r] = X.rule_off[r];
        ri64.Q[r] = L.Q[r];
        ri64.off[r] = L.rule_off[r];
    }
    Fp64View v{c.d_records, L.stride, L.nidx_off, c.d_phi, L.qmax, ri64};
    auto kern = assemble_df64_kernel<NP, CPLX>;
    BIE_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grid((unsigned)((a.M + kThreads - 1) / kThreads), (unsigned)S);
    cudaEvent_t t0 = c.timer_begin();
    kern<<<grid, kThreads, smem, c.stream>>>(
        c.d_drecords, X.stride, X.nidx_off, c.n_elements, S, c.d_shared_mask + (size_t)level * c.n_elements,
        reinterpret_cast<const float2 *>(c.d_dphi), L.R * L.qmax * NP, L.qmax, ri, a.targets, a.M, a.k_re,
        a.k_im, a.flags, reinterpret_cast<double2 *>(a.F), reinterpret_cast<double2 *>(a.G), Cpart, chunk, defer,
        dcount, dcap, v, deg, c.d_qpe, a.k_dev, reinterpret_cast<const double2 *>(a.g_weight));
    BIE_CUDA(cudaGetLastError());
    c.timer_end(t0);
    ++c.kernel_launches;
    const uint8_t *nsh = c.d_node_shared + (size_t)level * c.n_sources;
    const unsigned wgrid = (unsigned)std::min<int64_t>((a.M * c.n_sources + 255) / 256, 16LL * c.num_sms);
    for (double *X : {a.F, a.G}) {
        if (!X) continue;
        df_widen_kernel<<<std::max(1u, wgrid), 256, 0, c.stream>>>(reinterpret_cast<double2 *>(X), a.M,
                                                                    c.n_sources, nsh);
        BIE_CUDA(cudaGetLastError());
        ++c.kernel_launches;
    }
    correct_fp64_kernel<NP, CPLX, double2><<<(unsigned)(4 * c.num_sms), 128, 0, c.stream>>>(
        defer, dcount, dcap, v, a.targets, a.M, a.k_re, a.k_im, a.flags,
        reinterpret_cast<double2 *>(a.F), reinterpret_cast<double2 *>(a.G), Cnear, c.d_qpe, a.k_dev,
        reinterpret_cast<const double2 *>(a.g_weight));
    BIE_CUDA(cudaGetLastError());
    ++c.kernel_launches;
}

}  // namespace

void build_df64_records(Ctx &c, const std::vector<double> &rec64, const std::vector<float> &mrec) {
    const RecordLayout &L = c.lay;
    Df64Layout &X = c.dlay;
    X = Df64Layout{};
    const int NP = L.NP;
    // header as the mixed records (centroid hi/lo, near radius^2, node offsets)
    int off = (8 + 3 * NP + 3) & ~3;
    for (int r = 0; r < L.R; ++r) {
        X.rule_off[r] = off;
        off += 16 * L.Q[r];
    }
    X.nidx_off = off;
    off += NP;
    X.stride = (off + 3) & ~3;
    const int64_t E = c.n_elements;
    std::vector<float> rec((size_t)E * X.stride, 0.f);
    auto split = [](double x, float &hi, float &lo) {
        hi = (float)x;
        lo = (float)(x - (double)hi);
    };
    double rho = 0.0;
    for (int64_t p = 0; p < E; ++p) {
        const float *M0 = &mrec[(size_t)p * c.mlay.stride];
        const double *R0 = &rec64[(size_t)p * L.stride];
        float *W = &rec[(size_t)p * X.stride];
        std::copy(M0, M0 + 8 + 3 * NP, W);
        const double cen[3] = {(double)M0[0] + (double)M0[3], (double)M0[1] + (double)M0[4],
                               (double)M0[2] + (double)M0[5]};
        for (int r = 0; r < L.R; ++r) {
            const int Q = L.Q[r];
            const double *g = R0 + L.rule_off[r];
            float *w = W + X.rule_off[r];
            for (int q = 0; q < Q; ++q) {
                float *P = w + 16 * q;
                const double o[3] = {g[q] - cen[0], g[Q + q] - cen[1], g[2 * Q + q] - cen[2]};
                rho = std::max(rho, std::sqrt(o[0] * o[0] + o[1] * o[1] + o[2] * o[2]));
                // (ox oy oz jw/4pi)_hi, (...)_lo, (nx ny nz 0)_hi, (...)_lo
                split(o[0], P[0], P[4]);
                split(o[1], P[1], P[5]);
                split(o[2], P[2], P[6]);
                split(g[6 * Q + q] * 0.079577471545947667884, P[3], P[7]);
                split(g[3 * Q + q], P[8], P[12]);
                split(g[4 * Q + q], P[9], P[13]);
                split(g[5 * Q + q], P[10], P[14]);
            }
        }
        std::copy(M0 + c.mlay.nidx_off, M0 + c.mlay.nidx_off + NP, W + X.nidx_off);
    }
    c.df_rho_max = rho;
    std::vector<float> phi((size_t)L.R * L.qmax * NP * 2, 0.f);
    for (size_t j = 0; j < (size_t)L.R * L.qmax * NP; ++j) split(c.phi[j], phi[2 * j], phi[2 * j + 1]);
    // phase table e^{i j h}: cos and sin in FP64 (correctly rounded to ~1 ulp), split
    std::vector<float> tab((size_t)4 * (2 * df64::kPhaseTabHalf + 1));
    for (int j = -df64::kPhaseTabHalf; j <= df64::kPhaseTabHalf; ++j) {
        const double th = (double)j * (double)df64::kPhaseTabStep;
        float *t = &tab[(size_t)4 * (j + df64::kPhaseTabHalf)];
        split(std::cos(th), t[0], t[1]);
        split(std::sin(th), t[2], t[3]);
    }
    BIE_CUDA(cudaMalloc(&c.d_phase_tab, tab.size() * sizeof(float)));
    BIE_CUDA(cudaMemcpy(c.d_phase_tab, tab.data(), tab.size() * sizeof(float), cudaMemcpyHostToDevice));
    BIE_CUDA(cudaMalloc(&c.d_drecords, rec.size() * sizeof(float)));
    BIE_CUDA(cudaMalloc(&c.d_dphi, phi.size() * sizeof(float)));
    BIE_CUDA(cudaMemcpy(c.d_drecords, rec.data(), rec.size() * sizeof(float), cudaMemcpyHostToDevice));
    BIE_CUDA(cudaMemcpy(c.d_dphi, phi.data(), phi.size() * sizeof(float), cudaMemcpyHostToDevice));
}

bool launch_assemble_df64(Ctx &c, const AssembleArgs &a) {
    const RecordLayout &L = c.lay;
    if (a.taylor_m >= 0 || (a.k_dev && !(a.k_abs_max > 0))) return false;
    df64::DfDegrees deg{};
    const double kabs = std::max(std::hypot(a.k_re, a.k_im), a.k_dev ? a.k_abs_max : 0.0);
    const double kimb = a.k_dev ? kabs : std::fabs(a.k_im);
    if (!df64::df_degrees(kabs * c.df_rho_max, kimb * c.df_rho_max, deg)) return false;
    deg.tab = reinterpret_cast<const float4 *>(c.d_phase_tab);
    const int64_t N = c.n_sources;
    if (!(a.flags & (BIE_F | BIE_G | BIE_C))) return true;

    const unsigned int dcap = (unsigned int)std::min<int64_t>(a.M * 64 + 4096, (int64_t)1 << 30);
    const size_t dbytes = (size_t)dcap * sizeof(int2);
    char *dbuf = static_cast<char *>(c.scratch(kScratchDefer, dbytes + 256 + (size_t)a.M * 8));
    int2 *defer = reinterpret_cast<int2 *>(dbuf);
    unsigned int *dcount = reinterpret_cast<unsigned int *>(dbuf + dbytes);
    double *Cnear = reinterpret_cast<double *>(dbuf + dbytes + 256);
    auto reset = [&] {   // zeroed outputs (entries accumulate in place) and deferred list
        if (a.flags & BIE_F) BIE_CUDA(cudaMemsetAsync(a.F, 0, (size_t)a.M * N * 16, c.stream));
        if (a.flags & BIE_G) BIE_CUDA(cudaMemsetAsync(a.G, 0, (size_t)a.M * N * 16, c.stream));
        BIE_CUDA(cudaMemsetAsync(dbuf + dbytes, 0, 256 + (size_t)a.M * 8, c.stream));
    };
    reset();

    const size_t rec_bytes = (size_t)c.dlay.stride * sizeof(float);
    const int chunk0 = (int)std::max<size_t>(1, std::min<size_t>(32, (32u << 10) / rec_bytes));
    const size_t phi_f = (size_t)((2 * L.R * L.qmax * L.NP + 3) & ~3);
    const bool cplx = a.k_im != 0.0;
    auto run = [&](const LaunchShape &sh) {
        const int level = sh.level, chunk = sh.chunk;
        const int S = 1 << level;
        const size_t smem = phi_f * sizeof(float) + (size_t)chunk * rec_bytes + (size_t)chunk * 4;
        double *Cpart = static_cast<double *>(c.scratch(kScratchCpart, (size_t)S * a.M * sizeof(double)));
        if (L.NP == 1) {
            if (cplx) launch_df64_np<1, true>(c, a, S, level, smem, chunk, Cpart, defer, dcount, dcap, Cnear, deg);
            else launch_df64_np<1, false>(c, a, S, level, smem, chunk, Cpart, defer, dcount, dcap, Cnear, deg);
        } else if (L.NP == 3) {
            if (cplx) launch_df64_np<3, true>(c, a, S, level, smem, chunk, Cpart, defer, dcount, dcap, Cnear, deg);
            else launch_df64_np<3, false>(c, a, S, level, smem, chunk, Cpart, defer, dcount, dcap, Cnear, deg);
        } else {
            if (cplx) launch_df64_np<6, true>(c, a, S, level, smem, chunk, Cpart, defer, dcount, dcap, Cnear, deg);
            else launch_df64_np<6, false>(c, a, S, level, smem, chunk, Cpart, defer, dcount, dcap, Cnear, deg);
        }
        if (a.flags & BIE_C) launch_reduce_c(c, Cpart, S, Cnear, a.M, a.C);
    };
    const LaunchShape base{wave_slice_level(c, a.M, kThreads), chunk0, kThreads};
    ShapeAxes ax;
    for (int l = base.level - 1; l <= base.level + 1; ++l)
        if (l >= 0 && l < kMaxLevels && (int64_t(1) << l) <= c.n_elements) ax.levels.push_back(l);
    ax.chunks = {std::max(1, chunk0 / 2), chunk0, std::min(64, 2 * chunk0)};
    LaunchShape sh = resolve_shape(c, kShapeK9, a.M, base, ax, run, reset);
    sh.tpb = kThreads;   // the double-float kernel has one block size
    run(sh);
    return true;
}

}  // namespace bie
