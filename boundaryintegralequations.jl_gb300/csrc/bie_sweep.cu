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
//   4. p written into a device array of all nk solutions, copied to the
//      caller's host array once per mesh.
// Each mesh's device buffers are allocated once for its whole frequency list;
// frequencies of a mesh reuse them (assemble -> solve -> overwrite), so a
// 64-frequency sweep holds one mesh's matrices at a time.
//
// The first wavenumber of a mesh runs launch by launch: it sizes every scratch
// buffer and lets the autotuner pick the assembly's slicing.  Then the GMRES
// solve over the mesh's fixed buffers is recorded once by stream capture as a
// CUDA graph whose refinement, restart and Arnoldi loops are conditional nodes
// driven by device state (capture_gmres), and every later wavenumber is its
// assembly launches (k as kernel arguments) followed by one launch of that
// graph.  The host enqueues the whole rest of the mesh's sweep without
// synchronising and reads the results once.  (Recording every wavenumber into
// one graph was measured too: ~280 nodes per solve made recording and
// instantiation cost more than the replays saved.)
// The reference has no batched form (a user loop per frequency:
// examples/sweep_meta.jl:219-233, src/3d/rosebem.jl:235-262).
#include "bie_internal.h"

#include <algorithm>
#include <chrono>
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

// Events, body streams and graph objects of one mesh's recorded sweep; ends an
// unfinished capture and restores the context flags if an error unwinds.
struct GraphScope {
    Ctx &c;
    std::vector<cudaEvent_t> ev;
    cudaStream_t body[4] = {};
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool capturing = false;
    bool timing_saved;
    GraphScope(Ctx &ctx, int nev, bool streams) : c(ctx), ev(nev, nullptr), timing_saved(ctx.timing) {
        for (auto &e : ev) BIE_CUDA(cudaEventCreate(&e));
        if (streams)
            for (auto &s : body) BIE_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    }
    void begin() {
        c.timing = false;   // no host-side event timers inside a recorded graph
        c.capturing = true;
        BIE_CUDA(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeRelaxed));
        capturing = true;
    }
    void end() {
        capturing = false;
        c.capturing = false;
        c.timing = timing_saved;
        BIE_CUDA(cudaStreamEndCapture(c.stream, &graph));
    }
    ~GraphScope() {
        if (capturing) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(c.stream, &g);
            if (g) cudaGraphDestroy(g);
            c.capturing = false;
            c.timing = timing_saved;
        }
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        for (auto &s : body)
            if (s) cudaStreamDestroy(s);
        for (auto &e : ev)
            if (e) cudaEventDestroy(e);
    }
    GraphScope(const GraphScope &) = delete;
    GraphScope &operator=(const GraphScope &) = delete;
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
        DevBuf F(mat), G(mat), vec(4 * (size_t)N * 16), P((size_t)(nk + 1) * N * 16),
            dinfo((size_t)nk * sizeof(bie_gmres_info));
        double2 *Cv = vec.as<double2>(), *dg = Cv + N, *b = dg + N, *wd = b + N;
        double2 *X = P.as<double2>();
        bie_gmres_info *dgi = dinfo.as<bie_gmres_info>();
        BIE_CUDA(cudaMemcpyAsync(wd, w[m], (size_t)N * 16, cudaMemcpyHostToDevice, c.stream));

        // (F + Diagonal(1 - C)) p = b: mixed + refine: iterations with the fast
        // complex64 product (~1e-7), refined with residuals from the exact
        // complex64 product; mixed without refine: the exact complex64 product
        // throughout; plain: FP64 GMRES on complex128 matrices
        bie_gmres_opts go = o.gmres;
        go.refine = (mixed && o.refine) ? 1 : 0;
        go.precision = go.refine ? BIE_PREC_MIXED : BIE_PREC_FP64;
        if (go.refine && !(go.inner_reltol > 0)) go.inner_reltol = 1e-6;
        go.initially_nonzero = 0;
        bie_operator op{};
        op.kind = BIE_OP_DENSE;
        if (mixed) op.A32 = F.as<float>();
        else op.A = F.as<double>();
        op.scale_re = 1.0;
        op.diag = reinterpret_cast<const double *>(dg);
        bie_operator gop{};
        gop.kind = BIE_OP_DENSE;
        if (mixed) gop.A32 = G.as<float>();
        else gop.A = G.as<double>();
        gop.scale_re = 1.0;

        // assembly and right-hand side of wavenumber j (event e_a before the
        // assembly, e_b after it)
        auto assemble_rhs = [&](int j, cudaEvent_t e_a, cudaEvent_t e_b, unsigned ev_flags) {
            BIE_CUDA(cudaEventRecordWithFlags(e_a, c.stream, ev_flags));
            AssembleArgs a{ks[2 * j], ks[2 * j + 1], c.d_sources, N, BIE_F | BIE_G | BIE_C, F.as<double>(),
                           G.as<double>(), reinterpret_cast<double *>(Cv)};
            a.c64_out = mixed;
            if (mixed) launch_assemble_mixed(c, a);
            else launch_assemble_fp64(c, a);
            BIE_CUDA(cudaEventRecordWithFlags(e_b, c.stream, ev_flags));
            one_minus_kernel<<<(unsigned)((N + 255) / 256), 256, 0, c.stream>>>(Cv, dg, N);
            BIE_CUDA(cudaGetLastError());
            ++c.kernel_launches;
            // b = G w (the exact complex64 product in the mixed path)
            apply_operator(c, gop, BIE_PREC_FP64, reinterpret_cast<const double *>(wd),
                           reinterpret_cast<double *>(b));
        };

        const int restart = (int)std::max<int64_t>(1, std::min<int64_t>(go.restart > 0 ? go.restart : 20, N));
        const bool graph = !o.eager && nk > 1 && restart <= kGraphMaxRestart;
        const int j_eager = graph ? 1 : nk;   // wavenumbers solved by host-driven GMRES
        GraphScope gs(c, graph ? 3 * nk : 3, graph);
        std::vector<bie_gmres_info> hinfo(nk);
        double asm_ms = 0, sol_ms = 0;
        for (int j = 0; j < j_eager; ++j) {
            const int e = graph ? 3 * j : 0;
            assemble_rhs(j, gs.ev[e], gs.ev[e + 1], cudaEventRecordDefault);
            run_gmres(c, op, reinterpret_cast<const double *>(b), reinterpret_cast<double *>(X + (size_t)j * N),
                      go, hinfo[j]);
            BIE_CUDA(cudaEventRecord(gs.ev[e + 2], c.stream));
            BIE_CUDA(cudaStreamSynchronize(c.stream));
            float ta = 0, ts = 0;
            BIE_CUDA(cudaEventElapsedTime(&ta, gs.ev[e], gs.ev[e + 1]));
            BIE_CUDA(cudaEventElapsedTime(&ts, gs.ev[e + 1], gs.ev[e + 2]));
            asm_ms += ta;
            sol_ms += ts;
        }
        if (graph) {
            // the solve of (F + Diagonal(1 - C)) p = b over the mesh's fixed
            // buffers, recorded once and replayed for every later wavenumber; its
            // solution and statistics land in the extra column X[nk] / dgi[0]
            double2 *xs = X + (size_t)nk * N;
            const auto t0 = std::chrono::steady_clock::now();
            gs.begin();
            capture_gmres(c, op, reinterpret_cast<const double *>(b), reinterpret_cast<double *>(xs), go, dgi,
                          gs.body);
            gs.end();
            BIE_CUDA(cudaGraphInstantiate(&gs.exec, gs.graph, 0));
            info.record_ms +=
                std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            // the host enqueues the remaining wavenumbers without waiting
            for (int j = 1; j < nk; ++j) {
                assemble_rhs(j, gs.ev[3 * j], gs.ev[3 * j + 1], cudaEventRecordDefault);
                BIE_CUDA(cudaGraphLaunch(gs.exec, c.stream));
                ++info.graph_launches;
                BIE_CUDA(cudaMemcpyAsync(X + (size_t)j * N, xs, (size_t)N * 16, cudaMemcpyDeviceToDevice,
                                         c.stream));
                BIE_CUDA(cudaMemcpyAsync(dgi + j, dgi, sizeof(bie_gmres_info), cudaMemcpyDeviceToDevice,
                                         c.stream));
                BIE_CUDA(cudaEventRecord(gs.ev[3 * j + 2], c.stream));
            }
            BIE_CUDA(cudaMemcpyAsync(hinfo.data() + 1, dgi + 1, (size_t)(nk - 1) * sizeof(bie_gmres_info),
                                     cudaMemcpyDeviceToHost, c.stream));
            BIE_CUDA(cudaStreamSynchronize(c.stream));
            for (int j = 1; j < nk; ++j) {
                float ta = 0, ts = 0;
                BIE_CUDA(cudaEventElapsedTime(&ta, gs.ev[3 * j], gs.ev[3 * j + 1]));
                BIE_CUDA(cudaEventElapsedTime(&ts, gs.ev[3 * j + 1], gs.ev[3 * j + 2]));
                asm_ms += ta;
                sol_ms += ts;
            }
        }
        BIE_CUDA(cudaMemcpyAsync(p[m], X, (size_t)nk * N * 16, cudaMemcpyDeviceToHost, c.stream));
        BIE_CUDA(cudaStreamSynchronize(c.stream));
        info.assemble_ms += asm_ms;
        info.solve_ms += sol_ms;
        for (int j = 0; j < nk; ++j) {
            info.solves += 1;
            info.converged += hinfo[j].converged ? 1 : 0;
            info.iterations += hinfo[j].iterations;
            if (iters) iters[(size_t)m * nk + j] = hinfo[j].iterations;
        }
    }
}

}  // namespace bie
