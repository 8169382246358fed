// K1: dense FP64 collocation assembly of F (double layer), G (single layer) and
// C (k = 0 double-layer row sums) for 3- and 6-node triangles.
//
// Replaces the hot loop of assemble_parallel! (src/3d/assembly_collocation.jl:
// 314-349 and 424-476) with computing_integrals! (:213-252), the kernels
// greens3d!, freens3d!, freens3dk0! (src/3d/kernels.jl:13-55), the nearest
// physics node rule choice find_closest_corner (:102-115) and the
// accumulation mygemm_vec! (src/2d/assembly_collocation.jl:142-150).
//
// Work decomposition (one GPU):
//   grid.x  tiles of 128 target rows, one thread per row i
//   grid.y  S element slices (contiguous ranges of the bisection-ordered element
//           records), so that even a few thousand rows fill all 152 SMs
// Each block stages a chunk of element records (quadrature points, normals,
// jacobian x weight for every clustered rule, the physics-node coordinates and
// indices) in shared memory; every thread walks the chunk for its own row.
// F and G are column-major M x N complex128 (the layout of Julia's
// Matrix{ComplexF64}); a warp's 32 consecutive rows give one coalesced 512-byte
// access per node.  A (row, node) entry whose node is touched by one slice only
// is updated with a plain read-modify-write by the one thread that owns the row;
// nodes shared between slices are updated with FP64 atomics.  C is accumulated
// per slice and reduced by a second kernel.
#include "bie_internal.h"
#include "bie_device.cuh"

#include <algorithm>

namespace bie {

namespace {

using dev::RuleInfo;
constexpr int kThreads = 128;

template <int NP, bool CPLX_K>
__global__ void __launch_bounds__(kThreads)
assemble_fp64_kernel(const double *__restrict__ rec, int stride, int nidx_off,
                     int64_t E, int S, const uint32_t *__restrict__ smask,
                     const double *__restrict__ phi, int nphi, int qmax, RuleInfo ri,
                     const double *__restrict__ tgt, int64_t M, double kre, double kim,
                     int flags, double2 *__restrict__ F, double2 *__restrict__ G,
                     double *__restrict__ Cpart, int chunk,
                     unsigned long long *__restrict__ qpe_count,
                     const double2 *__restrict__ gweight, int tm, const double *__restrict__ kdev) {
    if (kdev) {   // wavenumber read from device memory (recorded sweeps)
        kre = kdev[0];
        kim = kdev[1];
    }
    extern __shared__ __align__(16) double smem[];
    double *s_phi = smem;                                   // nphi doubles (padded even)
    double *s_rec = smem + ((nphi + 1) & ~1);               // chunk * stride doubles
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
    for (int t = threadIdx.x; t < nphi; t += kThreads) s_phi[t] = phi[t];

    double cacc = 0.0;
    unsigned long long nqpe = 0;
    for (int64_t cb = e0; cb < e1; cb += chunk) {
        const int n = (int)min((int64_t)chunk, e1 - cb);
        __syncthreads();   // previous chunk fully consumed
        {
            const double2 *src = reinterpret_cast<const double2 *>(rec + cb * stride);
            double2 *dst = reinterpret_cast<double2 *>(s_rec);
            const int n2 = n * stride / 2;
            for (int t = threadIdx.x; t < n2; t += kThreads) dst[t] = src[t];
            for (int t = threadIdx.x; t < n; t += kThreads) s_mask[t] = smask[cb + t];
        }
        __syncthreads();
        if (!active) continue;

        for (int el = 0; el < n; ++el) {
            const double *r = s_rec + (size_t)el * stride;
            // k-derivative assembly uses the three corner rules only, nodes 4-6
            // falling to the third (taylor_assemble!, src/3d/rosebem.jl:114-127)
            const int cn = dev::nearest_node<NP>(r, tx, ty, tz);
            const int c = (tm >= 0 && cn > 2) ? 2 : cn;
            const int Q = ri.Q[c];
            nqpe += Q;
            double fr[NP], fi[NP], gr[NP], gi[NP];
            cacc += dev::element_fp64<NP, CPLX_K>(r + ri.off[c], Q, s_phi + (size_t)c * qmax * NP,
                                                  tx, ty, tz, kre, kim, fr, fi, gr, gi, tm);

            if (gweight && doG) {   // element factor on the single layer
                const double2 wgt = gweight[cb + el];
#pragma unroll
                for (int a = 0; a < NP; ++a) {
                    const double t = gr[a] * wgt.x - gi[a] * wgt.y;
                    gi[a] = gr[a] * wgt.y + gi[a] * wgt.x;
                    gr[a] = t;
                }
            }
            const int32_t *nid = reinterpret_cast<const int32_t *>(r + nidx_off);
            const uint32_t m = s_mask[el];
#pragma unroll
            for (int a = 0; a < NP; ++a) {
                const size_t off = (size_t)nid[a] * (size_t)M + (size_t)i;
                if ((m >> a) & 1u) {
                    if (doF) {
                        atomicAdd(&F[off].x, fr[a]);
                        atomicAdd(&F[off].y, fi[a]);
                    }
                    if (doG) {
                        atomicAdd(&G[off].x, gr[a]);
                        atomicAdd(&G[off].y, gi[a]);
                    }
                } else {
                    if (doF) {
                        double2 v = F[off];
                        v.x += fr[a];
                        v.y += fi[a];
                        F[off] = v;
                    }
                    if (doG) {
                        double2 v = G[off];
                        v.x += gr[a];
                        v.y += gi[a];
                        G[off] = v;
                    }
                }
            }
        }
    }
    if (active && doC) Cpart[(int64_t)s * M + i] = cacc;
    // one atomic per warp for the evaluation counter
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) nqpe += __shfl_down_sync(0xffffffffu, nqpe, o);
    if ((threadIdx.x & 31) == 0 && nqpe) atomicAdd(qpe_count, nqpe);
}

template <int NP, bool CPLX>
void launch_np(Ctx &c, const AssembleArgs &a, int S, int level, size_t smem, int chunk,
               double *Cpart) {
    const RecordLayout &L = c.lay;
    RuleInfo ri{};
    for (int r = 0; r < L.R; ++r) {
        ri.Q[r] = L.Q[r];
        ri.off[r] = L.rule_off[r];
    }
    auto kern = assemble_fp64_kernel<NP, CPLX>;
    BIE_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grid((unsigned)((a.M + kThreads - 1) / kThreads), (unsigned)S);
    cudaEvent_t t0 = c.timer_begin();
    kern<<<grid, kThreads, smem, c.stream>>>(
        c.d_records, L.stride, L.nidx_off, c.n_elements, S,
        c.d_shared_mask + (size_t)level * c.n_elements, c.d_phi, L.R * L.qmax * L.NP, L.qmax,
        ri, a.targets, a.M, a.k_re, a.k_im, a.flags, reinterpret_cast<double2 *>(a.F),
        reinterpret_cast<double2 *>(a.G), Cpart, chunk, c.d_qpe,
        reinterpret_cast<const double2 *>(a.g_weight), a.taylor_m, a.k_dev);
    BIE_CUDA(cudaGetLastError());
    c.timer_end(t0);
    ++c.kernel_launches;
}

}  // namespace

int choose_slice_level(const Ctx &c, int64_t M, int threads_per_row_tile) {
    const int64_t row_tiles = (M + threads_per_row_tile - 1) / threads_per_row_tile;
    int level = 0;
    while (level + 1 < kMaxLevels && row_tiles * (int64_t(1) << level) < 8LL * c.num_sms &&
           (int64_t(2) << level) <= c.n_elements)
        ++level;
    return level;
}

// Element slicing for the FP32-issue-bound kernels (mixed and double-float
// assembly, mixed and double-float products): at least 32 blocks per SM, so
// that the last partial wave of resident blocks is a small part of the launch,
// but at least 64 elements per slice where the mesh allows it (finer slices
// add partial sums, and for the mixed assembly nodes shared between slices),
// and never coarser than choose_slice_level.  Rigid-sphere P2 (11562 rows,
// 5780 elements): level 6 instead of 4; mixed assembly 2.31 -> 2.08 ms,
// double-float assembly 16.9 -> 15.6 ms, mixed product 2.05 -> 1.80 ms.
int wave_slice_level(const Ctx &c, int64_t M, int threads_per_row_tile) {
    const int64_t row_tiles = (M + threads_per_row_tile - 1) / threads_per_row_tile;
    const int64_t want = 32LL * c.num_sms;
    int level = 0;
    while (level + 1 < kMaxLevels && row_tiles * (int64_t(1) << level) < want &&
           (c.n_elements >> (level + 1)) >= 64)
        ++level;
    return std::max(level, choose_slice_level(c, M, threads_per_row_tile));
}

void launch_reduce_c(Ctx &c, const double *Cpart, int S, const double *Cextra, int64_t M,
                     double *C);

LaunchShape resolve_shape(Ctx &c, int kernel, int64_t M, const LaunchShape &base, const ShapeAxes &ax,
                          const std::function<void(const LaunchShape &)> &run, const std::function<void()> &reset) {
    for (const int64_t key : {M, int64_t(0)}) {
        const auto f = c.forced_shapes.find({kernel, key});
        if (f != c.forced_shapes.end()) {
            LaunchShape sh = f->second;
            if (sh.level < 0 || sh.level >= kMaxLevels) sh.level = base.level;
            if (sh.chunk <= 0) sh.chunk = base.chunk;
            if (sh.tpb != 128 && sh.tpb != 256) sh.tpb = base.tpb;
            return sh;
        }
    }
    const auto it = c.tuned_shapes.find({kernel, M});
    if (it != c.tuned_shapes.end()) return it->second;
    if (!c.autotune || c.capturing) return base;   // (timing needs host synchronisation)
    cudaEvent_t e0, e1;
    BIE_CUDA(cudaEventCreate(&e0));
    BIE_CUDA(cudaEventCreate(&e1));
    LaunchShape best = base;
    float best_ms = 3.4e38f;
    auto time_one = [&](const LaunchShape &sh) {
        reset();
        BIE_CUDA(cudaEventRecord(e0, c.stream));
        run(sh);
        BIE_CUDA(cudaEventRecord(e1, c.stream));
        BIE_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        BIE_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best_ms) {
            best_ms = ms;
            best = sh;
        }
    };
    try {
        time_one(base);
        const LaunchShape b0 = best;
        for (int l : ax.levels)
            if (l != b0.level) time_one(LaunchShape{l, b0.chunk, b0.tpb});
        const LaunchShape b1 = best;
        for (int ch : ax.chunks)
            if (ch != b1.chunk) time_one(LaunchShape{b1.level, ch, b1.tpb});
        const LaunchShape b2 = best;
        for (int t : ax.tpbs)
            if (t != b2.tpb) time_one(LaunchShape{b2.level, b2.chunk, t});
    } catch (...) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    c.tuned_shapes[{kernel, M}] = best;
    reset();
    return best;
}

void launch_assemble_fp64(Ctx &c, const AssembleArgs &a) {
    const RecordLayout &L = c.lay;
    const int64_t N = c.n_sources;
    if (a.flags & BIE_F) BIE_CUDA(cudaMemsetAsync(a.F, 0, (size_t)a.M * N * 16, c.stream));
    if (a.flags & BIE_G) BIE_CUDA(cudaMemsetAsync(a.G, 0, (size_t)a.M * N * 16, c.stream));
    if (!(a.flags & (BIE_F | BIE_G | BIE_C))) return;

    // slices: enough blocks for ~8 per SM, power of two, at most one per element
    const int level = choose_slice_level(c, a.M, kThreads);
    const int S = 1 << level;

    // element chunk: ~40 KB of records per block
    const size_t rec_bytes = (size_t)L.stride * sizeof(double);
    int chunk = (int)std::max<size_t>(1, std::min<size_t>(64, (40u << 10) / rec_bytes));
    const size_t phi_d = (size_t)((L.R * L.qmax * L.NP + 1) & ~1);
    const size_t smem = phi_d * sizeof(double) + (size_t)chunk * rec_bytes + (size_t)chunk * 4;

    double *Cpart = static_cast<double *>(c.scratch(kScratchCpart, (size_t)S * a.M * sizeof(double)));
    const bool cplx = a.k_im != 0.0;
    if (L.NP == 1) {
        if (cplx) launch_np<1, true>(c, a, S, level, smem, chunk, Cpart);
        else launch_np<1, false>(c, a, S, level, smem, chunk, Cpart);
    } else if (L.NP == 3) {
        if (cplx) launch_np<3, true>(c, a, S, level, smem, chunk, Cpart);
        else launch_np<3, false>(c, a, S, level, smem, chunk, Cpart);
    } else {
        if (cplx) launch_np<6, true>(c, a, S, level, smem, chunk, Cpart);
        else launch_np<6, false>(c, a, S, level, smem, chunk, Cpart);
    }
    if (a.flags & BIE_C) launch_reduce_c(c, Cpart, S, nullptr, a.M, a.C);
}

// ---------------------------------------------------------------------------
// C = sum over slices of the partial row sums (+ optional extra term)
// ---------------------------------------------------------------------------
namespace {
__global__ void reduce_c_kernel(const double *__restrict__ Cpart, int S,
                                const double *__restrict__ Cextra, int64_t M,
                                double2 *__restrict__ C) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M) return;
    double acc = 0.0;
    for (int s = 0; s < S; ++s) acc += Cpart[(int64_t)s * M + i];
    if (Cextra) acc += Cextra[i];
    C[i] = make_double2(acc, 0.0);
}
}  // namespace

void launch_reduce_c(Ctx &c, const double *Cpart, int S, const double *Cextra, int64_t M,
                     double *C) {
    reduce_c_kernel<<<(unsigned)((M + 255) / 256), 256, 0, c.stream>>>(
        Cpart, S, Cextra, M, reinterpret_cast<double2 *>(C));
    BIE_CUDA(cudaGetLastError());
    ++c.kernel_launches;
}

}  // namespace bie
