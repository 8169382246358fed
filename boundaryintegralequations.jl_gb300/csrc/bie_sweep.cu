// K6: batched frequency sweep over meshes of uneven size (bie_sweep).
//
// Work queue: every (mesh, k) item runs on the mesh context's stream:
//   1. dense assembly of F, G, C (mixed or FP64 kernels of this library),
//   2. diag = 1 - C, b = G w (the library's dense product),
//   3. GMRES on (F + Diagonal(1 - C)) p = b.  Mixed precision keeps F and G
//      in complex64 end to end (the assembly's FP32 accumulators with the FP64
//      near-pair corrections added in place; half the HBM bytes of
//      complex128); with refinement the Arnoldi iterations use the fast FP32
//      product (HBM-bound, ~1e-7) and the outer residuals and the right-hand
//      side the exact one (double-float sums, ~1e-14); FP64 uses complex128
//      matrices and FP64 products,
//   4. p copied into the caller's host array (pinned or not).
// Each mesh's device buffers are allocated once for its whole frequency list;
// frequencies of a mesh reuse them (assemble -> solve -> overwrite), so a
// 64-frequency sweep holds one mesh's matrices at a time.
// The reference has no batched form (a user loop per frequency:
// examples/sweep_meta.jl:219-233, src/3d/rosebem.jl:235-262).
#include "bie_internal.h"

#include <algorithm>
#include <vector>

namespace bie {

namespace {

__global__ void one_minus_kernel(const double2 *__restrict__ C, double2 *__restrict__ d, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) d[i] = make_double2(1.0 - C[i].x, -C[i].y);
}

struct DevBuf {
    void *p = nullptr;
    explicit DevBuf(size_t bytes) { BIE_CUDA(cudaMalloc(&p, bytes)); }
    ~DevBuf() { cudaFree(p); }
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    template <class T>
    T *as() const { return static_cast<T *>(p); }
};

}  // namespace

void run_sweep(Ctx *const *ctxs, int nmesh, const double *ks, int nk, const double *const *w,
               double *const *p, const bie_sweep_opts &o, bie_sweep_info &info, int32_t *iters) {
    info = bie_sweep_info{};
    for (int m = 0; m < nmesh; ++m) {
        Ctx &c = *ctxs[m];
        std::lock_guard<std::mutex> lock(c.mu);
        BIE_CUDA(cudaSetDevice(c.device));
        c.autotune = true;   // the first wavenumber of a mesh picks its slicing
        const int64_t N = c.n_sources;
        // mixed: complex64 matrices end to end (assembly accumulators with the FP64
        // corrections added in place, complex64 products with double-float sums);
        // FP64: complex128 matrices and FP64 products
        const bool mixed = o.precision == BIE_PREC_MIXED;
        const size_t mat = (size_t)N * N * (mixed ? 8 : 16);
        DevBuf F(mat), G(mat), vec(6 * (size_t)N * 16);
        double2 *Cv = vec.as<double2>(), *dg = Cv + N, *b = dg + N, *x = b + N, *wd = x + N;
        BIE_CUDA(cudaMemcpyAsync(wd, w[m], (size_t)N * 16, cudaMemcpyHostToDevice, c.stream));
        cudaEvent_t e0, e1, e2;
        BIE_CUDA(cudaEventCreate(&e0));
        BIE_CUDA(cudaEventCreate(&e1));
        BIE_CUDA(cudaEventCreate(&e2));
        for (int j = 0; j < nk; ++j) {
            const double kr = ks[2 * j], ki = ks[2 * j + 1];
            BIE_CUDA(cudaEventRecord(e0, c.stream));
            AssembleArgs a{kr, ki, c.d_sources, N, BIE_F | BIE_G | BIE_C, F.as<double>(), G.as<double>(),
                           reinterpret_cast<double *>(Cv)};
            a.c64_out = mixed;
            if (mixed) launch_assemble_mixed(c, a);
            else launch_assemble_fp64(c, a);
            BIE_CUDA(cudaEventRecord(e1, c.stream));
            one_minus_kernel<<<(unsigned)((N + 255) / 256), 256, 0, c.stream>>>(Cv, dg, N);
            BIE_CUDA(cudaGetLastError());
            ++c.kernel_launches;
            // b = G w
            bie_operator gop{};
            gop.kind = BIE_OP_DENSE;
            if (mixed) gop.A32 = G.as<float>();
            else gop.A = G.as<double>();
            gop.scale_re = 1.0;
            // (the exact complex64 product in the mixed path)
            apply_operator(c, gop, BIE_PREC_FP64, reinterpret_cast<const double *>(wd),
                           reinterpret_cast<double *>(b));
            // (F + Diagonal(1 - C)) p = b
            bie_operator op{};
            op.kind = BIE_OP_DENSE;
            if (mixed) op.A32 = F.as<float>();
            else op.A = F.as<double>();
            op.scale_re = 1.0;
            op.diag = reinterpret_cast<const double *>(dg);
            // mixed + refine: iterations with the fast complex64 product (~1e-7),
            // refined with residuals from the exact complex64 product; mixed
            // without refine: the exact complex64 product throughout; plain:
            // FP64 GMRES on complex128 matrices
            bie_gmres_opts go = o.gmres;
            go.refine = (mixed && o.refine) ? 1 : 0;
            go.precision = go.refine ? BIE_PREC_MIXED : BIE_PREC_FP64;
            if (go.refine && !(go.inner_reltol > 0)) go.inner_reltol = 1e-6;
            go.initially_nonzero = 0;
            bie_gmres_info gi{};
            run_gmres(c, op, reinterpret_cast<const double *>(b), reinterpret_cast<double *>(x), go, gi);
            BIE_CUDA(cudaEventRecord(e2, c.stream));
            BIE_CUDA(cudaMemcpyAsync(p[m] + (size_t)j * N * 2, x, (size_t)N * 16, cudaMemcpyDeviceToHost,
                                     c.stream));
            BIE_CUDA(cudaStreamSynchronize(c.stream));
            float ta = 0, ts = 0;
            BIE_CUDA(cudaEventElapsedTime(&ta, e0, e1));
            BIE_CUDA(cudaEventElapsedTime(&ts, e1, e2));
            info.assemble_ms += ta;
            info.solve_ms += ts;
            info.solves += 1;
            info.converged += gi.converged ? 1 : 0;
            info.iterations += gi.iterations;
            if (iters) iters[(size_t)m * nk + j] = gi.iterations;
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaEventDestroy(e2);
    }
}

}  // namespace bie
