// K3: matrix-free operator application  yF = F x,  yG = G v  (F, G as assembled
// by assemble_parallel!, src/3d/assembly_collocation.jl:270-479, never stored).
//
// This is the GPU counterpart of the LinearMaps operators fed to gmres
// (FMMFOperator / FMMGOperator._unsafe_mul!, src/3d/fast_multipole_method.jl:
// 238-247, 392-404): each product recomputes the kernel values on the fly, so
// an N = 40k operator needs O(N) memory instead of a 26 GB matrix.
//
// Mixed precision (BIE_PREC_MIXED):
//   1. interp: xi[e, r, q] = sum_a Phi_r[q][a] x[node_a(e)] for every element,
//      rule and quadrature point (complex64), likewise for v.
//   2. one thread per target row (x element slices for occupancy) evaluates the
//      regular pairs with the shared mixed-precision pair code and accumulates
//      yF += F_q xiF_q, yG += G_q xiG_q: FP32 per element, double-float across
//      elements (compensated), written once per (row, slice).
//   3. near pairs and nearest-node near-ties are integrated in FP64 by a
//      correction kernel (same rule as the assembly) and added atomically.
//   4. y = sum over slices + correction.
// FP64 (BIE_PREC_FP64): the FP64 element integrals of the assembly kernel,
// dotted with x and v per element, accumulated in FP64.
#include "bie_internal.h"
#include "bie_device.cuh"
#include "bie_mixed.cuh"
#include "bie_df64.cuh"

#include <algorithm>

namespace bie {

namespace {

using dev::df;
using dev::RuleInfo;
constexpr int kThreads = 128;

// xi[p][slot] for slot in [0, QT): rule r covers [xoff[r], xoff[r] + Q_r)
__global__ void interp_kernel(const double *__restrict__ rec64, int stride64, int nidx_off,
                              const double *__restrict__ phi, int qmax, int NP, int R, RuleInfo ri,
                              int QT, int QTp, int64_t E, const double2 *__restrict__ x,
                              const double2 *__restrict__ v, float2 *__restrict__ xiF,
                              float2 *__restrict__ xiG) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= E * QT) return;
    const int64_t p = j / QT;
    int slot = (int)(j - p * QT);
    int r = 0;
    while (r + 1 < R && slot >= ri.Q[r]) {
        slot -= ri.Q[r];
        ++r;
    }
    const int q = slot;
    const int32_t *nid = reinterpret_cast<const int32_t *>(rec64 + (size_t)p * stride64 + nidx_off);
    const double *ph = phi + ((size_t)r * qmax + q) * NP;
    double fr = 0, fi = 0, gr = 0, gi = 0;
    for (int a = 0; a < NP; ++a) {
        const double w = ph[a];
        if (x) {
            const double2 xa = x[nid[a]];
            fr += w * xa.x;
            fi += w * xa.y;
        }
        if (v) {
            const double2 va = v[nid[a]];
            gr += w * va.x;
            gi += w * va.y;
        }
    }
    const int64_t o = p * QTp + (j - p * QT);
    if (xiF) xiF[o] = make_float2((float)fr, (float)fi);
    if (xiG) xiG[o] = make_float2((float)gr, (float)gi);
}

struct Fp64Rec {
    const double *rec;
    int stride;
    int nidx_off;
    const double *phi;   // global, R x qmax x NP
    int qmax;
    RuleInfo ri;
};

// FP64 element integral of one pair dotted with x (f) and v (g), returned by
// value: a pointer into the caller's registers would keep them in local memory
struct PairDot {
    double2 f, g;
};

// FP64 element integral of one pair dotted with x and v (deferred-list overflow)
template <int NP, bool CPLX>
__device__ __noinline__ PairDot pair_fp64_dot(const Fp64Rec &v, int64_t p, double tx, double ty,
                                              double tz, double kre, double kim,
                                              const double2 *x, const double2 *vin) {
    const double *r = v.rec + (size_t)p * v.stride;
    const int c = dev::nearest_node<NP>(r, tx, ty, tz);
    double fr[NP], fi[NP], gr[NP], gi[NP];
    dev::element_fp64<NP, CPLX, df64::TrigDf>(r + v.ri.off[c], v.ri.Q[c], v.phi + (size_t)c * v.qmax * NP, tx,
                                ty, tz, kre, kim, fr, fi, gr, gi);
    const int32_t *nid = reinterpret_cast<const int32_t *>(r + v.nidx_off);
    double a0 = 0, a1 = 0, b0 = 0, b1 = 0;
    for (int a = 0; a < NP; ++a) {
        if (x) {
            const double2 xa = x[nid[a]];
            a0 += fr[a] * xa.x - fi[a] * xa.y;
            a1 += fr[a] * xa.y + fi[a] * xa.x;
        }
        if (vin) {
            const double2 va = vin[nid[a]];
            b0 += gr[a] * va.x - gi[a] * va.y;
            b1 += gr[a] * va.y + gi[a] * va.x;
        }
    }
    return PairDot{make_double2(a0, a1), make_double2(b0, b1)};
}

template <int NP, bool CPLX_K>
__global__ void __launch_bounds__(kThreads, 4)
matvec_mixed_kernel(const float *__restrict__ rec, int stride, int64_t E, int S, RuleInfo ri,
                    RuleInfo rxi, int QTp, const float2 *__restrict__ xiF,
                    const float2 *__restrict__ xiG, const double *__restrict__ tgt, int64_t M,
                    double kre, double kim, double2 *__restrict__ yFpart,
                    double2 *__restrict__ yGpart, int chunk, int2 *__restrict__ defer,
                    unsigned int *__restrict__ defer_count, unsigned int defer_cap,
                    const __grid_constant__ Fp64Rec v64, const double2 *__restrict__ x64,
                    const double2 *__restrict__ v64in, unsigned long long *__restrict__ qpe_count) {
    extern __shared__ __align__(16) float smemf[];
    float *s_rec = smemf;                                               // chunk * stride
    float2 *s_xiF = reinterpret_cast<float2 *>(s_rec + (size_t)chunk * stride);
    float2 *s_xiG = s_xiF + (xiF ? (size_t)chunk * QTp : 0);

    const int s = blockIdx.y;
    const int64_t e0 = (int64_t)s * E / S;
    const int64_t e1 = (int64_t)(s + 1) * E / S;
    const int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x;
    const bool active = i < M;
    const bool doF = xiF != nullptr, doG = xiG != nullptr;
    // rule tables in shared memory: indexed by each thread's nearest node, they
    // would otherwise be copied to local memory (divergent dynamic index)
    __shared__ RuleInfo s_ri, s_rxi;
    if (threadIdx.x == 0) {
        s_ri = ri;
        s_rxi = rxi;
    }

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

    df yFr = {0.f, 0.f}, yFi = {0.f, 0.f}, yGr = {0.f, 0.f}, yGi = {0.f, 0.f};
    unsigned long long nqpe = 0;
    for (int64_t cb = e0; cb < e1; cb += chunk) {
        const int n = (int)min((int64_t)chunk, e1 - cb);
        __syncthreads();
        {
            const float4 *src = reinterpret_cast<const float4 *>(rec + cb * stride);
            float4 *dst = reinterpret_cast<float4 *>(s_rec);
            const int n4 = n * stride / 4;
            for (int t = threadIdx.x; t < n4; t += kThreads) dst[t] = src[t];
            const int nx = n * QTp;
            if (doF)
                for (int t = threadIdx.x; t < nx; t += kThreads) s_xiF[t] = xiF[cb * QTp + t];
            if (doG)
                for (int t = threadIdx.x; t < nx; t += kThreads) s_xiG[t] = xiG[cb * QTp + t];
        }
        __syncthreads();
        if (!active) continue;

        for (int el = 0; el < n; ++el) {
            const float *r = s_rec + (size_t)el * stride;
            const mixed::PairSetup P = mixed::pair_setup<NP>(r, T);
            if (P.deferred) {
                const unsigned int slot = atomicAdd(defer_count, 1u);
                if (slot < defer_cap) {
                    defer[slot] = make_int2((int)i, (int)(cb + el));
                } else {   // list full: integrate this pair in FP64 in place
                    const PairDot pd = pair_fp64_dot<NP, CPLX_K>(v64, cb + el, tx, ty, tz, kre, kim, x64, v64in);
                    const double2 pf = pd.f, pg = pd.g;
                    // both float parts of each FP64 value, so that the pair
                    // keeps double-float accuracy in the row sums
                    if (doF) {
                        mixed::df_accum(yFr, (float)pf.x);
                        mixed::df_accum(yFr, (float)(pf.x - (double)(float)pf.x));
                        mixed::df_accum(yFi, (float)pf.y);
                        mixed::df_accum(yFi, (float)(pf.y - (double)(float)pf.y));
                    }
                    if (doG) {
                        mixed::df_accum(yGr, (float)pg.x);
                        mixed::df_accum(yGr, (float)(pg.x - (double)(float)pg.x));
                        mixed::df_accum(yGi, (float)pg.y);
                        mixed::df_accum(yGi, (float)(pg.y - (double)(float)pg.y));
                    }
                }
                continue;
            }
            const mixed::Phase ph = mixed::pair_phase(P, K);
            const int c = P.c;
            const int Q = s_ri.Q[c];
            nqpe += Q;
            const float4 *g4 = reinterpret_cast<const float4 *>(r + s_ri.off[c]);
            const float2 *xf = s_xiF + (size_t)el * QTp + s_rxi.off[c];
            const float2 *xg = s_xiG + (size_t)el * QTp + s_rxi.off[c];
            float afr = 0.f, afi = 0.f, agr = 0.f, agi = 0.f;
            for (int q = 0; q < Q; ++q) {
                const mixed::QpeValues w = mixed::qpe<CPLX_K>(g4[2 * q], g4[2 * q + 1], P, ph, kf, kimf);
                if (doF) {
                    const float2 a = xf[q];
                    afr = __fmaf_rn(w.Fr, a.x, __fmaf_rn(-w.Fi, a.y, afr));
                    afi = __fmaf_rn(w.Fr, a.y, __fmaf_rn(w.Fi, a.x, afi));
                }
                if (doG) {
                    const float2 a = xg[q];
                    agr = __fmaf_rn(w.Gr, a.x, __fmaf_rn(-w.Gi, a.y, agr));
                    agi = __fmaf_rn(w.Gr, a.y, __fmaf_rn(w.Gi, a.x, agi));
                }
            }
            if (doF) {
                mixed::df_accum(yFr, afr);
                mixed::df_accum(yFi, afi);
            }
            if (doG) {
                mixed::df_accum(yGr, agr);
                mixed::df_accum(yGi, agi);
            }
        }
    }
    if (active) {
        if (doF) yFpart[(int64_t)s * M + i] = make_double2(dev::f2d(yFr.hi) + dev::f2d(yFr.lo),
                                                           dev::f2d(yFi.hi) + dev::f2d(yFi.lo));
        if (doG) yGpart[(int64_t)s * M + i] = make_double2(dev::f2d(yGr.hi) + dev::f2d(yGr.lo),
                                                           dev::f2d(yGi.hi) + dev::f2d(yGi.lo));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) nqpe += __shfl_down_sync(0xffffffffu, nqpe, o);
    if ((threadIdx.x & 31) == 0 && nqpe) atomicAdd(qpe_count, nqpe);
}

// FP64 matrix-free product: per (row, element) the FP64 element integrals of
// the assembly, dotted with x / v.
template <int NP, bool CPLX_K>
__global__ void __launch_bounds__(kThreads)
matvec_fp64_kernel(const double *__restrict__ rec, int stride, int nidx_off, int64_t E, int S,
                   const double *__restrict__ phi, int nphi, int qmax, RuleInfo ri,
                   const double2 *__restrict__ x, const double2 *__restrict__ v,
                   const double *__restrict__ tgt, int64_t M, double kre, double kim,
                   double2 *__restrict__ yFpart, double2 *__restrict__ yGpart, int chunk,
                   unsigned long long *__restrict__ qpe_count) {
    extern __shared__ __align__(16) double smem[];
    double *s_phi = smem;
    double *s_rec = smem + ((nphi + 1) & ~1);
    const int s = blockIdx.y;
    const int64_t e0 = (int64_t)s * E / S;
    const int64_t e1 = (int64_t)(s + 1) * E / S;
    const int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x;
    const bool active = i < M;
    double tx = 0, ty = 0, tz = 0;
    if (active) {
        tx = tgt[3 * i + 0];
        ty = tgt[3 * i + 1];
        tz = tgt[3 * i + 2];
    }
    for (int t = threadIdx.x; t < nphi; t += kThreads) s_phi[t] = phi[t];
    __shared__ RuleInfo s_ri;   // indexed by each thread's nearest node
    if (threadIdx.x == 0) s_ri = ri;
    double yfr = 0, yfi = 0, ygr = 0, ygi = 0;
    unsigned long long nqpe = 0;
    for (int64_t cb = e0; cb < e1; cb += chunk) {
        const int n = (int)min((int64_t)chunk, e1 - cb);
        __syncthreads();
        {
            const double2 *src = reinterpret_cast<const double2 *>(rec + cb * stride);
            double2 *dst = reinterpret_cast<double2 *>(s_rec);
            const int n2 = n * stride / 2;
            for (int t = threadIdx.x; t < n2; t += kThreads) dst[t] = src[t];
        }
        __syncthreads();
        if (!active) continue;
        for (int el = 0; el < n; ++el) {
            const double *r = s_rec + (size_t)el * stride;
            const int c = dev::nearest_node<NP>(r, tx, ty, tz);
            nqpe += s_ri.Q[c];
            double fr[NP], fi[NP], gr[NP], gi[NP];
            dev::element_fp64<NP, CPLX_K>(r + s_ri.off[c], s_ri.Q[c], s_phi + (size_t)c * qmax * NP, tx,
                                          ty, tz, kre, kim, fr, fi, gr, gi);
            const int32_t *nid = reinterpret_cast<const int32_t *>(r + nidx_off);
#pragma unroll
            for (int a = 0; a < NP; ++a) {
                if (x) {
                    const double2 xa = x[nid[a]];
                    yfr += fr[a] * xa.x - fi[a] * xa.y;
                    yfi += fr[a] * xa.y + fi[a] * xa.x;
                }
                if (v) {
                    const double2 va = v[nid[a]];
                    ygr += gr[a] * va.x - gi[a] * va.y;
                    ygi += gr[a] * va.y + gi[a] * va.x;
                }
            }
        }
    }
    if (active) {
        if (x) yFpart[(int64_t)s * M + i] = make_double2(yfr, yfi);
        if (v) yGpart[(int64_t)s * M + i] = make_double2(ygr, ygi);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) nqpe += __shfl_down_sync(0xffffffffu, nqpe, o);
    if ((threadIdx.x & 31) == 0 && nqpe) atomicAdd(qpe_count, nqpe);
}

// FP64 correction for the deferred pairs of the mixed product.
template <int NP, bool CPLX_K>
__global__ void __launch_bounds__(128)
matvec_correct_kernel(const int2 *__restrict__ defer, const unsigned int *__restrict__ defer_count,
                      unsigned int defer_cap, const double *__restrict__ rec, int stride,
                      int nidx_off, const double *__restrict__ phi, int qmax, const __grid_constant__ RuleInfo ri,
                      const double2 *__restrict__ x, const double2 *__restrict__ v,
                      const double *__restrict__ tgt, double kre, double kim,
                      double2 *__restrict__ yFn, double2 *__restrict__ yGn,
                      unsigned long long *__restrict__ qpe_count) {
    const unsigned int n = min(*defer_count, defer_cap);
    unsigned long long nqpe = 0;
    for (unsigned int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const int2 pr = defer[j];
        const int64_t i = pr.x;
        const double *r = rec + (size_t)pr.y * stride;
        const double tx = tgt[3 * i], ty = tgt[3 * i + 1], tz = tgt[3 * i + 2];
        const int c = dev::nearest_node<NP>(r, tx, ty, tz);
        nqpe += ri.Q[c];
        double fr[NP], fi[NP], gr[NP], gi[NP];
        dev::element_fp64<NP, CPLX_K, df64::TrigDf>(r + ri.off[c], ri.Q[c], phi + (size_t)c * qmax * NP, tx, ty,
                                      tz, kre, kim, fr, fi, gr, gi);
        const int32_t *nid = reinterpret_cast<const int32_t *>(r + nidx_off);
        double yfr = 0, yfi = 0, ygr = 0, ygi = 0;
#pragma unroll
        for (int a = 0; a < NP; ++a) {
            if (x) {
                const double2 xa = x[nid[a]];
                yfr += fr[a] * xa.x - fi[a] * xa.y;
                yfi += fr[a] * xa.y + fi[a] * xa.x;
            }
            if (v) {
                const double2 va = v[nid[a]];
                ygr += gr[a] * va.x - gi[a] * va.y;
                ygi += gr[a] * va.y + gi[a] * va.x;
            }
        }
        if (x) {
            atomicAdd(&yFn[i].x, yfr);
            atomicAdd(&yFn[i].y, yfi);
        }
        if (v) {
            atomicAdd(&yGn[i].x, ygr);
            atomicAdd(&yGn[i].y, ygi);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) nqpe += __shfl_down_sync(0xffffffffu, nqpe, o);
    if ((threadIdx.x & 31) == 0 && nqpe) atomicAdd(qpe_count, nqpe);
}

// y = sum_s part[s] (+ extra)
__global__ void reduce_y_kernel(const double2 *__restrict__ part, int S,
                                const double2 *__restrict__ extra, int64_t M,
                                double2 *__restrict__ y) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M) return;
    double re = 0, im = 0;
    for (int s = 0; s < S; ++s) {
        const double2 p = part[(int64_t)s * M + i];
        re += p.x;
        im += p.y;
    }
    if (extra) {
        re += extra[i].x;
        im += extra[i].y;
    }
    y[i] = make_double2(re, im);
}

template <int NP, bool CPLX>
void run_mixed(Ctx &c, const MatvecArgs &a) {
    const RecordLayout &L = c.lay;
    const MixedLayout &X = c.mlay;
    RuleInfo ri{}, ri64{}, rxi{};
    int QT = 0;
    for (int r = 0; r < L.R; ++r) {
        ri.Q[r] = ri64.Q[r] = rxi.Q[r] = L.Q[r];
        ri.off[r] = X.rule_off[r];
        ri64.off[r] = L.rule_off[r];
        rxi.off[r] = QT;
        QT += L.Q[r];
    }
    const int QTp = (QT + 1) & ~1;
    const int64_t E = c.n_elements, M = a.M;
    const bool doF = a.x != nullptr, doG = a.v != nullptr;

    // scratch: xiF, xiG | yFpart, yGpart | defer list, counter, yFn, yGn
    const size_t xi_bytes = (size_t)E * QTp * sizeof(float2);
    char *xb = static_cast<char *>(c.scratch(kScratchMatvecXi, 2 * xi_bytes));
    float2 *xiF = doF ? reinterpret_cast<float2 *>(xb) : nullptr;
    float2 *xiG = doG ? reinterpret_cast<float2 *>(xb + xi_bytes) : nullptr;
    const unsigned int dcap = (unsigned int)std::min<int64_t>(M * 64 + 4096, (int64_t)1 << 30);
    const size_t dbytes = (size_t)dcap * sizeof(int2);
    char *db = static_cast<char *>(c.scratch(kScratchDefer, dbytes + 256 + 2 * (size_t)M * 16));
    int2 *defer = reinterpret_cast<int2 *>(db);
    unsigned int *dcount = reinterpret_cast<unsigned int *>(db + dbytes);
    double2 *yFn = reinterpret_cast<double2 *>(db + dbytes + 256);
    double2 *yGn = yFn + M;

    const int64_t nslots = E * QT;
    interp_kernel<<<(unsigned)((nslots + 255) / 256), 256, 0, c.stream>>>(
        c.d_records, L.stride, L.nidx_off, c.d_phi, L.qmax, L.NP, L.R, ri64, QT, QTp, E,
        reinterpret_cast<const double2 *>(a.x), reinterpret_cast<const double2 *>(a.v), xiF, xiG);
    BIE_CUDA(cudaGetLastError());
    ++c.kernel_launches;

    const size_t rec_bytes = (size_t)X.stride * sizeof(float);
    const size_t per_el = rec_bytes + (size_t)(doF + doG) * QTp * sizeof(float2);
    const int chunk0 = (int)std::max<size_t>(1, std::min<size_t>(64, (24u << 10) / per_el));
    const Fp64Rec v64{c.d_records, L.stride, L.nidx_off, c.d_phi, L.qmax, ri64};
    // one complete product (slice partials, deferred pairs, reductions) for a launch shape
    auto run = [&](const LaunchShape &sh) {
        const int S = 1 << sh.level, chunk = sh.chunk;
        const size_t part_bytes = (size_t)S * M * sizeof(double2);
        char *pb = static_cast<char *>(c.scratch(kScratchMatvecPart, 2 * part_bytes));
        double2 *yFpart = reinterpret_cast<double2 *>(pb);
        double2 *yGpart = reinterpret_cast<double2 *>(pb + part_bytes);
        BIE_CUDA(cudaMemsetAsync(db + dbytes, 0, 256 + 2 * (size_t)M * 16, c.stream));
        const size_t smem = (size_t)chunk * per_el;
        auto kern = matvec_mixed_kernel<NP, CPLX>;
        BIE_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        dim3 grid((unsigned)((M + kThreads - 1) / kThreads), (unsigned)S);
        cudaEvent_t t0 = c.timer_begin();
        kern<<<grid, kThreads, smem, c.stream>>>(c.d_mrecords, X.stride, E, S, ri, rxi, QTp, xiF, xiG,
                                                 a.targets, M, a.k_re, a.k_im, yFpart, yGpart, chunk,
                                                 defer, dcount, dcap, v64,
                                                 reinterpret_cast<const double2 *>(a.x),
                                                 reinterpret_cast<const double2 *>(a.v), c.d_qpe);
        BIE_CUDA(cudaGetLastError());
        c.timer_end(t0);
        ++c.kernel_launches;
        matvec_correct_kernel<NP, CPLX><<<(unsigned)(4 * c.num_sms), 128, 0, c.stream>>>(
            defer, dcount, dcap, c.d_records, L.stride, L.nidx_off, c.d_phi, L.qmax, ri64,
            reinterpret_cast<const double2 *>(a.x), reinterpret_cast<const double2 *>(a.v), a.targets,
            a.k_re, a.k_im, yFn, yGn, c.d_qpe);
        BIE_CUDA(cudaGetLastError());
        ++c.kernel_launches;
        if (doF) {
            reduce_y_kernel<<<(unsigned)((M + 255) / 256), 256, 0, c.stream>>>(
                yFpart, S, yFn, M, reinterpret_cast<double2 *>(a.yF));
            BIE_CUDA(cudaGetLastError());
            ++c.kernel_launches;
        }
        if (doG) {
            reduce_y_kernel<<<(unsigned)((M + 255) / 256), 256, 0, c.stream>>>(
                yGpart, S, yGn, M, reinterpret_cast<double2 *>(a.yG));
            BIE_CUDA(cudaGetLastError());
            ++c.kernel_launches;
        }
    };
    const LaunchShape base{wave_slice_level(c, M, kThreads), chunk0, kThreads};
    ShapeAxes ax;
    for (int l = base.level - 1; l <= base.level + 1; ++l)
        if (l >= 0 && l < kMaxLevels && (int64_t(1) << l) <= c.n_elements) ax.levels.push_back(l);
    ax.chunks = {std::max(1, chunk0 / 2), chunk0, std::min(64, 2 * chunk0)};
    LaunchShape sh = resolve_shape(c, kShapeK3, M, base, ax, run, [] {});
    sh.tpb = kThreads;
    run(sh);
}

template <int NP, bool CPLX>
void run_fp64(Ctx &c, const MatvecArgs &a) {
    const RecordLayout &L = c.lay;
    RuleInfo ri{};
    for (int r = 0; r < L.R; ++r) {
        ri.Q[r] = L.Q[r];
        ri.off[r] = L.rule_off[r];
    }
    const int64_t M = a.M;
    const int level = choose_slice_level(c, M, kThreads);
    const int S = 1 << level;
    const size_t part_bytes = (size_t)S * M * sizeof(double2);
    char *pb = static_cast<char *>(c.scratch(kScratchMatvecPart, 2 * part_bytes));
    double2 *yFpart = reinterpret_cast<double2 *>(pb);
    double2 *yGpart = reinterpret_cast<double2 *>(pb + part_bytes);
    const size_t rec_bytes = (size_t)L.stride * sizeof(double);
    const int chunk = (int)std::max<size_t>(1, std::min<size_t>(64, (40u << 10) / rec_bytes));
    const int nphi = L.R * L.qmax * L.NP;
    const size_t smem = (size_t)((nphi + 1) & ~1) * sizeof(double) + (size_t)chunk * rec_bytes;
    auto kern = matvec_fp64_kernel<NP, CPLX>;
    BIE_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grid((unsigned)((M + kThreads - 1) / kThreads), (unsigned)S);
    cudaEvent_t t0 = c.timer_begin();
    kern<<<grid, kThreads, smem, c.stream>>>(
        c.d_records, L.stride, L.nidx_off, c.n_elements, S, c.d_phi, nphi, L.qmax, ri,
        reinterpret_cast<const double2 *>(a.x), reinterpret_cast<const double2 *>(a.v), a.targets, M,
        a.k_re, a.k_im, yFpart, yGpart, chunk, c.d_qpe);
    BIE_CUDA(cudaGetLastError());
    c.timer_end(t0);
    ++c.kernel_launches;
    if (a.x) {
        reduce_y_kernel<<<(unsigned)((M + 255) / 256), 256, 0, c.stream>>>(
            yFpart, S, nullptr, M, reinterpret_cast<double2 *>(a.yF));
        BIE_CUDA(cudaGetLastError());
        ++c.kernel_launches;
    }
    if (a.v) {
        reduce_y_kernel<<<(unsigned)((M + 255) / 256), 256, 0, c.stream>>>(
            yGpart, S, nullptr, M, reinterpret_cast<double2 *>(a.yG));
        BIE_CUDA(cudaGetLastError());
        ++c.kernel_launches;
    }
}

// ---------------------------------------------------------------------------
// Allocation-free variant of the mixed-precision product.
//
// Some callers cannot let a library call cudaMalloc: a Julia session whose
// CUDA.jl memory pool (or a Python process whose PyTorch caching allocator)
// has already reserved most of the device, real-time loops that must not
// synchronise the device, or code that runs between the set-up and the
// capture of a CUDA graph.  For them bie_matvec_device_noalloc keeps every
// temporary of the product (interpolated densities, per-slice partial sums,
// the list of pairs integrated in FP64) in one file-scope device array of
// kNoAllocScratchBytes.
//
// The array belongs to this file's module, which the CUDA runtime may load
// lazily; loading it commits the array's device memory.  prepare_noalloc runs
// when a context is created: it looks the array's device address up with
// cudaGetSymbolAddress (with the context's device current; the host-side name
// of the array is only a stand-in for the device symbol), keeps it in the
// context, and launches the product's kernels once on empty work, so that the
// module, the kernels and their stack reservation are in place before the
// first product.  From the first context on a device until the process exits
// that device holds the array.  All calls share it: the parts that must start
// at zero are cleared on every call, and calls whose executions overlap on the
// GPU (different streams or contexts of the same device) race on it.
// ---------------------------------------------------------------------------
constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;   // 32 MiB
// the last 256 bytes hold a zero word for the priming launches, outside the
// part a product carves up, so that creating a context never disturbs a
// product in flight on the same device
constexpr size_t kNoAllocUsable = kNoAllocScratchBytes - 256;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

template <int NP, bool CPLX>
void prime_noalloc_kernels(Ctx &c, unsigned int *zero_word) {
    // empty work: E = 0 elements and M = 0 targets, so no thread reads or
    // writes anything but the zeroed counter
    RuleInfo ri{};
    const Fp64Rec v64{c.d_records, c.lay.stride, c.lay.nidx_off, c.d_phi, c.lay.qmax, ri};
    matvec_mixed_kernel<NP, CPLX><<<dim3(1, 1), kThreads, 0, c.stream>>>(
        c.d_mrecords, c.mlay.stride, 0, 1, ri, ri, 2, nullptr, nullptr, c.d_sources, 0, 0.0, 0.0,
        nullptr, nullptr, 1, nullptr, zero_word, 0, v64, nullptr, nullptr, c.d_qpe);
    BIE_CUDA(cudaGetLastError());
    matvec_correct_kernel<NP, CPLX><<<1, 128, 0, c.stream>>>(
        nullptr, zero_word, 0, c.d_records, c.lay.stride, c.lay.nidx_off, c.d_phi, c.lay.qmax, ri,
        nullptr, nullptr, c.d_sources, 0.0, 0.0, nullptr, nullptr, c.d_qpe);
    BIE_CUDA(cudaGetLastError());
}

}  // namespace

void prepare_noalloc(Ctx &c) {
    void *p = nullptr;
    BIE_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    c.noalloc_base = static_cast<char *>(p);
    unsigned int *zero_word = reinterpret_cast<unsigned int *>(c.noalloc_base + kNoAllocUsable);
    BIE_CUDA(cudaMemsetAsync(zero_word, 0, 256, c.stream));
    RuleInfo ri{};
    interp_kernel<<<1, 256, 0, c.stream>>>(c.d_records, c.lay.stride, c.lay.nidx_off, c.d_phi, c.lay.qmax,
                                           c.lay.NP, 1, ri, 1, 2, 0, nullptr, nullptr, nullptr, nullptr);
    BIE_CUDA(cudaGetLastError());
    reduce_y_kernel<<<1, 256, 0, c.stream>>>(nullptr, 0, nullptr, 0, nullptr);
    BIE_CUDA(cudaGetLastError());
    if (c.lay.NP == 1) {
        prime_noalloc_kernels<1, false>(c, zero_word);
        prime_noalloc_kernels<1, true>(c, zero_word);
    } else if (c.lay.NP == 3) {
        prime_noalloc_kernels<3, false>(c, zero_word);
        prime_noalloc_kernels<3, true>(c, zero_word);
    } else {
        prime_noalloc_kernels<6, false>(c, zero_word);
        prime_noalloc_kernels<6, true>(c, zero_word);
    }
    BIE_CUDA(cudaStreamSynchronize(c.stream));
}

namespace {

inline size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

template <int NP, bool CPLX>
void run_mixed_noalloc(Ctx &c, const MatvecArgs &a) {
    const RecordLayout &L = c.lay;
    const MixedLayout &X = c.mlay;
    RuleInfo ri{}, ri64{}, rxi{};
    int QT = 0;
    for (int r = 0; r < L.R; ++r) {
        ri.Q[r] = ri64.Q[r] = rxi.Q[r] = L.Q[r];
        ri.off[r] = X.rule_off[r];
        ri64.off[r] = L.rule_off[r];
        rxi.off[r] = QT;
        QT += L.Q[r];
    }
    const int QTp = (QT + 1) & ~1;
    const int64_t E = c.n_elements, M = a.M;
    const bool doF = a.x != nullptr, doG = a.v != nullptr;
    const int level = choose_slice_level(c, M, kThreads);
    const int S = 1 << level;

    // carve the static array: xiF | xiG | yFpart | yGpart | defer list | counter | yFn, yGn
    const size_t xi_bytes = align256((size_t)E * QTp * sizeof(float2));
    const size_t part_bytes = align256((size_t)S * M * sizeof(double2));
    // deferred-pair list: the capacity of bie_matvec_device (M*64 + 4096
    // pairs) where it fits, shrunk for large meshes down to M*16 + 1024; a pair
    // beyond the capacity is integrated in FP64 inside the product kernel
    // (slower, equally accurate)
    const size_t near_bytes = align256(256 + 2 * (size_t)M * sizeof(double2));
    const size_t fixed = (doF ? xi_bytes : 0) + (doG ? xi_bytes : 0) + (doF ? part_bytes : 0) +
                         (doG ? part_bytes : 0) + near_bytes;
    const int64_t cap_full = std::min<int64_t>(M * 64 + 4096, (int64_t)1 << 30);
    const int64_t cap_min = M * 16 + 1024;
    const int64_t cap_fit =
        fixed + 256 < kNoAllocUsable ? (int64_t)((kNoAllocUsable - fixed - 256) / sizeof(int2)) : 0;
    const unsigned int dcap = (unsigned int)std::min(cap_full, cap_fit);
    const size_t dbytes = align256((size_t)dcap * sizeof(int2));
    const size_t need = fixed + align256((size_t)std::max<int64_t>(dcap, cap_min) * sizeof(int2));
    if ((int64_t)dcap < cap_min || need > kNoAllocUsable)
        fail(BIE_ERR_INVALID, "bie_matvec_device_noalloc: this mesh needs " + std::to_string(need) +
                                  " bytes of scratch, more than the fixed " +
                                  std::to_string(kNoAllocUsable) +
                                  "; use bie_matvec_device");
    if (!c.noalloc_base) fail(BIE_ERR_CUDA, "allocation-free scratch was not set up for this context");
    char *base = c.noalloc_base;
    size_t off = 0;
    float2 *xiF = nullptr, *xiG = nullptr;
    double2 *yFpart = nullptr, *yGpart = nullptr;
    if (doF) { xiF = reinterpret_cast<float2 *>(base + off); off += xi_bytes; }
    if (doG) { xiG = reinterpret_cast<float2 *>(base + off); off += xi_bytes; }
    if (doF) { yFpart = reinterpret_cast<double2 *>(base + off); off += part_bytes; }
    if (doG) { yGpart = reinterpret_cast<double2 *>(base + off); off += part_bytes; }
    int2 *defer = reinterpret_cast<int2 *>(base + off);
    off += dbytes;
    unsigned int *dcount = reinterpret_cast<unsigned int *>(base + off);
    double2 *yFn = reinterpret_cast<double2 *>(base + off + 256);
    double2 *yGn = yFn + M;
    // the counter and the FP64 correction sums start at zero on every call
    BIE_CUDA(cudaMemsetAsync(base + off, 0, 256 + 2 * (size_t)M * sizeof(double2), c.stream));

    const int64_t nslots = E * QT;
    interp_kernel<<<(unsigned)((nslots + 255) / 256), 256, 0, c.stream>>>(
        c.d_records, L.stride, L.nidx_off, c.d_phi, L.qmax, L.NP, L.R, ri64, QT, QTp, E,
        reinterpret_cast<const double2 *>(a.x), reinterpret_cast<const double2 *>(a.v), xiF, xiG);
    BIE_CUDA(cudaGetLastError());

    const size_t rec_bytes = (size_t)X.stride * sizeof(float);
    const size_t per_el = rec_bytes + (size_t)(doF + doG) * QTp * sizeof(float2);
    const int chunk = (int)std::max<size_t>(1, std::min<size_t>(64, (24u << 10) / per_el));
    const size_t smem = (size_t)chunk * per_el;
    auto kern = matvec_mixed_kernel<NP, CPLX>;
    BIE_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grid((unsigned)((M + kThreads - 1) / kThreads), (unsigned)S);
    const Fp64Rec v64{c.d_records, L.stride, L.nidx_off, c.d_phi, L.qmax, ri64};
    kern<<<grid, kThreads, smem, c.stream>>>(c.d_mrecords, X.stride, E, S, ri, rxi, QTp, xiF, xiG,
                                             a.targets, M, a.k_re, a.k_im, yFpart, yGpart, chunk,
                                             defer, dcount, dcap, v64,
                                             reinterpret_cast<const double2 *>(a.x),
                                             reinterpret_cast<const double2 *>(a.v), c.d_qpe);
    BIE_CUDA(cudaGetLastError());
    matvec_correct_kernel<NP, CPLX><<<(unsigned)(4 * c.num_sms), 128, 0, c.stream>>>(
        defer, dcount, dcap, c.d_records, L.stride, L.nidx_off, c.d_phi, L.qmax, ri64,
        reinterpret_cast<const double2 *>(a.x), reinterpret_cast<const double2 *>(a.v), a.targets,
        a.k_re, a.k_im, yFn, yGn, c.d_qpe);
    BIE_CUDA(cudaGetLastError());
    if (doF) {
        reduce_y_kernel<<<(unsigned)((M + 255) / 256), 256, 0, c.stream>>>(
            yFpart, S, yFn, M, reinterpret_cast<double2 *>(a.yF));
        BIE_CUDA(cudaGetLastError());
    }
    if (doG) {
        reduce_y_kernel<<<(unsigned)((M + 255) / 256), 256, 0, c.stream>>>(
            yGpart, S, yGn, M, reinterpret_cast<double2 *>(a.yG));
        BIE_CUDA(cudaGetLastError());
    }
    c.kernel_launches += 3 + (doF ? 1 : 0) + (doG ? 1 : 0);
}

}  // namespace

// ---------------------------------------------------------------------------
// FP64-grade product in double-float arithmetic (BIE_PREC_DF64): x and v are
// interpolated to the quadrature points in FP64 and stored as (re_hi, re_lo,
// im_hi, im_lo); each regular pair then costs the double-float kernel values
// of its points and one complex product-sum per point; near pairs, near-ties
// and very large phases go to the FP64 correction.
// ---------------------------------------------------------------------------
namespace {
using namespace df64;

__global__ void interp_df_kernel(const double *__restrict__ rec64, int stride64, int nidx_off,
                                 const double *__restrict__ phi, int qmax, int NP, int R, RuleInfo ri, int QT,
                                 int QTp, int64_t E, const double2 *__restrict__ x, const double2 *__restrict__ v,
                                 float4 *__restrict__ xiF, float4 *__restrict__ xiG) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= E * QT) return;
    const int64_t p = j / QT;
    int slot = (int)(j - p * QT);
    int r = 0;
    while (r + 1 < R && slot >= ri.Q[r]) {
        slot -= ri.Q[r];
        ++r;
    }
    const int q = slot;
    const int32_t *nid = reinterpret_cast<const int32_t *>(rec64 + (size_t)p * stride64 + nidx_off);
    const double *ph = phi + ((size_t)r * qmax + q) * NP;
    double fr = 0, fi = 0, gr = 0, gi = 0;
    for (int a = 0; a < NP; ++a) {
        const double w = ph[a];
        if (x) {
            const double2 xa = x[nid[a]];
            fr += w * xa.x;
            fi += w * xa.y;
        }
        if (v) {
            const double2 va = v[nid[a]];
            gr += w * va.x;
            gi += w * va.y;
        }
    }
    const int64_t o = p * QTp + (j - p * QT);
    auto pack = [](double re, double im) {
        const df a = dd::to_df(re), b = dd::to_df(im);
        return make_float4(a.hi, a.lo, b.hi, b.lo);
    };
    if (xiF) xiF[o] = pack(fr, fi);
    if (xiG) xiG[o] = pack(gr, gi);
}

// y += (ar + i ai) (b.x + b.y i ...) with b = (re_hi, re_lo, im_hi, im_lo)
__device__ __forceinline__ void cmul_acc(dd::Acc &yr, dd::Acc &yi, df ar, df ai, const float4 b) {
    const df br{b.x, b.y}, bi{b.z, b.w};
    dd::acc_add(yr, dd::mul_raw(ar, br));
    dd::acc_add(yr, dd::mul_raw(dd::neg(ai), bi));
    dd::acc_add(yi, dd::mul_raw(ar, bi));
    dd::acc_add(yi, dd::mul_raw(ai, br));
}

template <int NP, bool CPLX_K>
__global__ void __launch_bounds__(kThreads, 3)
matvec_df64_kernel(const float *__restrict__ rec, int stride, int64_t E, int S, RuleInfo ri, RuleInfo rxi,
                   int QTp, const float4 *__restrict__ xiF, const float4 *__restrict__ xiG,
                   const double *__restrict__ tgt, int64_t M, double kre, double kim,
                   double2 *__restrict__ yFpart, double2 *__restrict__ yGpart, int chunk,
                   int2 *__restrict__ defer, unsigned int *__restrict__ defer_count, unsigned int defer_cap,
                   const __grid_constant__ Fp64Rec v64, const double2 *__restrict__ x64,
                   const double2 *__restrict__ v64in, DfDegrees deg, unsigned long long *__restrict__ qpe_count) {
    extern __shared__ __align__(16) float smemf[];
    float *s_rec = smemf;                                                   // chunk * stride
    float4 *s_xiF = reinterpret_cast<float4 *>(s_rec + (size_t)chunk * stride);
    float4 *s_xiG = s_xiF + (xiF ? (size_t)chunk * QTp : 0);

    const int s = blockIdx.y;
    const int64_t e0 = (int64_t)s * E / S;
    const int64_t e1 = (int64_t)(s + 1) * E / S;
    const int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x;
    const bool active = i < M;
    const bool doF = xiF != nullptr, doG = xiG != nullptr;
    // rule tables in shared memory: indexed by each thread's nearest node, they
    // would otherwise be copied to local memory (divergent dynamic index)
    __shared__ RuleInfo s_ri, s_rxi;
    if (threadIdx.x == 0) {
        s_ri = ri;
        s_rxi = rxi;
    }

    double tx = 0, ty = 0, tz = 0;
    if (active) {
        tx = tgt[3 * i + 0];
        ty = tgt[3 * i + 1];
        tz = tgt[3 * i + 2];
    }
    const mixed::Target T{dev::df_from_double(tx), dev::df_from_double(ty), dev::df_from_double(tz)};
    const df K = dd::to_df(kre), Ki = dd::to_df(kim);

    dd::Acc yFr{0.f, 0.f}, yFi{0.f, 0.f}, yGr{0.f, 0.f}, yGi{0.f, 0.f};
    unsigned long long nqpe = 0;
    for (int64_t cb = e0; cb < e1; cb += chunk) {
        const int n = (int)min((int64_t)chunk, e1 - cb);
        __syncthreads();
        {
            const float4 *src = reinterpret_cast<const float4 *>(rec + cb * stride);
            float4 *dst = reinterpret_cast<float4 *>(s_rec);
            const int n4 = n * stride / 4;
            for (int t = threadIdx.x; t < n4; t += kThreads) dst[t] = src[t];
            const int nx = n * QTp;
            if (doF)
                for (int t = threadIdx.x; t < nx; t += kThreads) s_xiF[t] = xiF[cb * QTp + t];
            if (doG)
                for (int t = threadIdx.x; t < nx; t += kThreads) s_xiG[t] = xiG[cb * QTp + t];
        }
        __syncthreads();
        if (!active) continue;

        for (int el = 0; el < n; ++el) {
            const float *r = s_rec + (size_t)el * stride;
            const mixed::PairSetup P = mixed::pair_setup<NP>(r, T);
            const df r0 = dd::sqrt_df(dev::df_add(dev::df_add(dev::df_sqr(P.Dxd), dev::df_sqr(P.Dyd)),
                                                  dev::df_sqr(P.Dzd)));
            const df kr0 = dev::df_mul(K, r0);
            if (P.deferred || !(fabsf(kr0.hi) < kDfMaxPhase)) {
                const unsigned int slot = atomicAdd(defer_count, 1u);
                if (slot < defer_cap) {
                    defer[slot] = make_int2((int)i, (int)(cb + el));
                } else {   // list full: this pair in FP64 in place
                    const PairDot pd = pair_fp64_dot<NP, CPLX_K>(v64, cb + el, tx, ty, tz, kre, kim, x64, v64in);
                    const double2 pf = pd.f, pg = pd.g;
                    if (doF) {
                        dd::acc_add(yFr, dd::to_df(pf.x));
                        dd::acc_add(yFi, dd::to_df(pf.y));
                    }
                    if (doG) {
                        dd::acc_add(yGr, dd::to_df(pg.x));
                        dd::acc_add(yGi, dd::to_df(pg.y));
                    }
                }
                continue;
            }
            df E0r, E0i;
            pair_phase_df64<CPLX_K>(kr0, r0, kim, E0r, E0i);
            const int c = P.c;
            const int Q = s_ri.Q[c];
            nqpe += Q;
            const float4 *g4 = reinterpret_cast<const float4 *>(r + s_ri.off[c]);
            const float4 *xf = s_xiF + (size_t)el * QTp + s_rxi.off[c];
            const float4 *xg = s_xiG + (size_t)el * QTp + s_rxi.off[c];
            for (int q = 0; q < Q; ++q) {
                df Fr, Fi, Gr, Gi, tq;
                qpe_df64<CPLX_K>(g4[4 * q], g4[4 * q + 1], g4[4 * q + 2], g4[4 * q + 3], P, r0, E0r, E0i, K, Ki,
                                 deg, Fr, Fi, Gr, Gi, tq);
                if (doF) cmul_acc(yFr, yFi, Fr, Fi, xf[q]);
                if (doG) cmul_acc(yGr, yGi, Gr, Gi, xg[q]);
            }
        }
    }
    if (active) {
        if (doF) yFpart[(int64_t)s * M + i] = make_double2(dd::acc_value(yFr), dd::acc_value(yFi));
        if (doG) yGpart[(int64_t)s * M + i] = make_double2(dd::acc_value(yGr), dd::acc_value(yGi));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) nqpe += __shfl_down_sync(0xffffffffu, nqpe, o);
    if ((threadIdx.x & 31) == 0 && nqpe) atomicAdd(qpe_count, nqpe);
}

template <int NP, bool CPLX>
void run_df64(Ctx &c, const MatvecArgs &a, DfDegrees deg) {
    const RecordLayout &L = c.lay;
    const Df64Layout &X = c.dlay;
    RuleInfo ri{}, ri64{}, rxi{};
    int QT = 0;
    for (int r = 0; r < L.R; ++r) {
        ri.Q[r] = ri64.Q[r] = rxi.Q[r] = L.Q[r];
        ri.off[r] = X.rule_off[r];
        ri64.off[r] = L.rule_off[r];
        rxi.off[r] = QT;
        QT += L.Q[r];
    }
    const int QTp = (QT + 1) & ~1;
    const int64_t E = c.n_elements, M = a.M;
    const bool doF = a.x != nullptr, doG = a.v != nullptr;

    const int level = wave_slice_level(c, M, kThreads);
    const int S = 1 << level;
    const size_t xi_bytes = (size_t)E * QTp * sizeof(float4);
    char *xb = static_cast<char *>(c.scratch(kScratchMatvecXi, 2 * xi_bytes));
    float4 *xiF = doF ? reinterpret_cast<float4 *>(xb) : nullptr;
    float4 *xiG = doG ? reinterpret_cast<float4 *>(xb + xi_bytes) : nullptr;
    const size_t part_bytes = (size_t)S * M * sizeof(double2);
    char *pb = static_cast<char *>(c.scratch(kScratchMatvecPart, 2 * part_bytes));
    double2 *yFpart = reinterpret_cast<double2 *>(pb);
    double2 *yGpart = reinterpret_cast<double2 *>(pb + part_bytes);
    const unsigned int dcap = (unsigned int)std::min<int64_t>(M * 64 + 4096, (int64_t)1 << 30);
    const size_t dbytes = (size_t)dcap * sizeof(int2);
    char *db = static_cast<char *>(c.scratch(kScratchDefer, dbytes + 256 + 2 * (size_t)M * 16));
    int2 *defer = reinterpret_cast<int2 *>(db);
    unsigned int *dcount = reinterpret_cast<unsigned int *>(db + dbytes);
    double2 *yFn = reinterpret_cast<double2 *>(db + dbytes + 256);
    double2 *yGn = yFn + M;
    BIE_CUDA(cudaMemsetAsync(db + dbytes, 0, 256 + 2 * (size_t)M * 16, c.stream));

    const int64_t nslots = E * QT;
    interp_df_kernel<<<(unsigned)((nslots + 255) / 256), 256, 0, c.stream>>>(
        c.d_records, L.stride, L.nidx_off, c.d_phi, L.qmax, L.NP, L.R, ri64, QT, QTp, E,
        reinterpret_cast<const double2 *>(a.x), reinterpret_cast<const double2 *>(a.v), xiF, xiG);
    BIE_CUDA(cudaGetLastError());
    ++c.kernel_launches;

    const size_t rec_bytes = (size_t)X.stride * sizeof(float);
    const size_t per_el = rec_bytes + (size_t)(doF + doG) * QTp * sizeof(float4);
    const int chunk = (int)std::max<size_t>(1, std::min<size_t>(32, (32u << 10) / per_el));
    const size_t smem = (size_t)chunk * per_el;
    auto kern = matvec_df64_kernel<NP, CPLX>;
    BIE_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grid((unsigned)((M + kThreads - 1) / kThreads), (unsigned)S);
    cudaEvent_t t0 = c.timer_begin();
    const Fp64Rec v64{c.d_records, L.stride, L.nidx_off, c.d_phi, L.qmax, ri64};
    kern<<<grid, kThreads, smem, c.stream>>>(c.d_drecords, X.stride, E, S, ri, rxi, QTp, xiF, xiG, a.targets, M,
                                             a.k_re, a.k_im, yFpart, yGpart, chunk, defer, dcount, dcap, v64,
                                             reinterpret_cast<const double2 *>(a.x),
                                             reinterpret_cast<const double2 *>(a.v), deg, c.d_qpe);
    BIE_CUDA(cudaGetLastError());
    c.timer_end(t0);
    ++c.kernel_launches;

    matvec_correct_kernel<NP, CPLX><<<(unsigned)(4 * c.num_sms), 128, 0, c.stream>>>(
        defer, dcount, dcap, c.d_records, L.stride, L.nidx_off, c.d_phi, L.qmax, ri64,
        reinterpret_cast<const double2 *>(a.x), reinterpret_cast<const double2 *>(a.v), a.targets,
        a.k_re, a.k_im, yFn, yGn, c.d_qpe);
    BIE_CUDA(cudaGetLastError());
    ++c.kernel_launches;
    if (doF) {
        reduce_y_kernel<<<(unsigned)((M + 255) / 256), 256, 0, c.stream>>>(
            yFpart, S, yFn, M, reinterpret_cast<double2 *>(a.yF));
        BIE_CUDA(cudaGetLastError());
        ++c.kernel_launches;
    }
    if (doG) {
        reduce_y_kernel<<<(unsigned)((M + 255) / 256), 256, 0, c.stream>>>(
            yGpart, S, yGn, M, reinterpret_cast<double2 *>(a.yG));
        BIE_CUDA(cudaGetLastError());
        ++c.kernel_launches;
    }
}

}  // namespace

void launch_matvec_noalloc(Ctx &c, const MatvecArgs &a) {
    if (!a.x && !a.v) return;
    const bool cplx = a.k_im != 0.0;
    if (c.lay.NP == 1) {
        if (cplx) run_mixed_noalloc<1, true>(c, a);
        else run_mixed_noalloc<1, false>(c, a);
    } else if (c.lay.NP == 3) {
        if (cplx) run_mixed_noalloc<3, true>(c, a);
        else run_mixed_noalloc<3, false>(c, a);
    } else {
        if (cplx) run_mixed_noalloc<6, true>(c, a);
        else run_mixed_noalloc<6, false>(c, a);
    }
}

void launch_matvec(Ctx &c, const MatvecArgs &a) {
    if (!a.x && !a.v) return;
    const bool cplx = a.k_im != 0.0;
    if (a.precision == BIE_PREC_DF64) {
        df64::DfDegrees deg{};
        if (df64::df_degrees(std::hypot(a.k_re, a.k_im) * c.df_rho_max, std::fabs(a.k_im) * c.df_rho_max, deg)) {
            deg.tab = reinterpret_cast<const float4 *>(c.d_phase_tab);
            if (c.lay.NP == 1) {
                if (cplx) run_df64<1, true>(c, a, deg);
                else run_df64<1, false>(c, a, deg);
            } else if (c.lay.NP == 3) {
                if (cplx) run_df64<3, true>(c, a, deg);
                else run_df64<3, false>(c, a, deg);
            } else {
                if (cplx) run_df64<6, true>(c, a, deg);
                else run_df64<6, false>(c, a, deg);
            }
            return;
        }
        // phase rotations beyond the Taylor tables: the FP64 product
    }
    if (a.precision == BIE_PREC_MIXED) {
        if (c.lay.NP == 1) {
            if (cplx) run_mixed<1, true>(c, a);
            else run_mixed<1, false>(c, a);
        } else if (c.lay.NP == 3) {
            if (cplx) run_mixed<3, true>(c, a);
            else run_mixed<3, false>(c, a);
        } else {
            if (cplx) run_mixed<6, true>(c, a);
            else run_mixed<6, false>(c, a);
        }
    } else {
        if (c.lay.NP == 1) {
            if (cplx) run_fp64<1, true>(c, a);
            else run_fp64<1, false>(c, a);
        } else if (c.lay.NP == 3) {
            if (cplx) run_fp64<3, true>(c, a);
            else run_fp64<3, false>(c, a);
        } else {
            if (cplx) run_fp64<6, true>(c, a);
            else run_fp64<6, false>(c, a);
        }
    }
}

}  // namespace bie
