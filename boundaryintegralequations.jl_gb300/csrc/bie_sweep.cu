// K6: batched frequency sweep over meshes of uneven size (bie_sweep).
//
// Work per (mesh, k) item, on the mesh context's stream:
//   1. dense assembly of F, G, C (mixed or FP64 kernels of this library),
//   2. diag = 1 - C, b = G w (the library's dense product),
//   3. GMRES on (F + Diagonal(1 - C)) p = b.  Mixed precision keeps F and G
//      in complex64 end to end (the assembly's FP32 accumulators with the FP64
//      near-pair corrections added in place; half the HBM bytes of
//      complex128); with refinement the Arnoldi iterations use the fast FP32
//      product (HBM-bound, ~1e-7) and the outer residuals and the right-hand
//      side the exact one (double-float sums, ~1e-14); FP64 uses complex128
//      matrices and FP64 products,
//   4. p written into a device array of the mesh's nk solutions, copied to the
//      caller's host array at the end.
// Each mesh's device buffers are allocated once for its whole frequency list;
// its frequencies reuse them (assemble -> solve -> overwrite).
//
// The first wavenumber of every mesh runs launch by launch: it sizes every
// scratch buffer and lets the autotuner pick the assembly's slicing.  All the
// remaining work of the sweep is then ONE launch of a recorded CUDA graph: per
// mesh, a WHILE node over the wavenumbers whose body reads k_j from device
// memory, assembles F, G, C (the kernels take k from there), forms b, runs the
// GMRES solve whose refinement, restart and Arnoldi loops are nested
// conditional nodes (capture_gmres), stores p_j and advances j; the meshes'
// loops follow one another in the graph.  Each body is recorded once (~280
// nodes) whatever the number of wavenumbers; device timestamps (%globaltimer)
// split assembly and solve times per wavenumber.  (Recording every wavenumber
// unrolled was measured first: its record + instantiate time grew with nk and
// cancelled the gain.)  Contexts on different devices, restart > 64 or
// opts.eager fall back to launch-by-launch solves, one mesh at a time.
// The reference has no batched form (a user loop per frequency:
// examples/sweep_meta.jl:219-233, src/3d/rosebem.jl:235-262).
#include "bie_internal.h"

#include <algorithm>
#include <chrono>
#include <memory>
#include <vector>

namespace bie {

namespace {

// Relative surface-pressure error of a mixed solve per unit of sensitivity
// (the FP32 rounding of the assembly and of the complex64 matrices), the scale
// of the sensitivity estimate in the re-solve test: the largest ratio of error
// to estimate measured over the 3-mesh x 64-wavenumber sweep workload against
// double-float solutions (median 7e-8, largest 5.07e-7).
constexpr double kMixedSweepError = 5e-7;

__global__ void one_minus_kernel(const double2 *__restrict__ C, double2 *__restrict__ d, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) d[i] = make_double2(1.0 - C[i].x, -C[i].y);
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// j = j0; enter the wavenumber loop if j0 < nk
__global__ void sweep_begin_kernel(int *j, int j0, int nk, cudaGraphConditionalHandle h) {
    *j = j0;
    cudaGraphSetConditional(h, j0 < nk ? 1u : 0u);
}

// kcur = k_j; timestamp 0 of wavenumber j
__global__ void sweep_k_kernel(const double *__restrict__ ks, const int *__restrict__ j, double *__restrict__ kcur,
                               unsigned long long *__restrict__ ts) {
    const int jj = *j;
    kcur[0] = ks[2 * jj];
    kcur[1] = ks[2 * jj + 1];
    ts[3 * jj] = global_ns();
}

__global__ void sweep_stamp_kernel(const int *__restrict__ j, unsigned long long *__restrict__ ts, int slot) {
    ts[3 * *j + slot] = global_ns();
}

// column j of X = xs, statistics of wavenumber j = *info0
__global__ void sweep_store_kernel(const double2 *__restrict__ xs, double2 *__restrict__ X, int64_t n,
                                   const int *__restrict__ j, const bie_gmres_info *info0,
                                   bie_gmres_info *info) {
    const int64_t jj = *j;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        X[jj * n + i] = xs[i];
    if (blockIdx.x == 0 && threadIdx.x == 0) info[jj] = *info0;
}

// timestamp 2 of wavenumber j, then j + 1 and the loop condition (j + 1 < nk:
// the loop runs at most nk times whatever the data)
__global__ void sweep_next_kernel(int *j, int nk, unsigned long long *__restrict__ ts, cudaGraphConditionalHandle h) {
    const int jj = *j;
    ts[3 * jj + 2] = global_ns();
    *j = jj + 1;
    cudaGraphSetConditional(h, jj + 1 < nk ? 1u : 0u);
}

// Sensitivity estimate of a mixed solve (no reference counterpart): with z a
// fixed pseudo-random vector, y ~ A^{-1} z (a short GMRES solve with the
// complex64 matrix) and wz = A z,  amp = |A z| |y| / |z|^2  estimates how much
// the solve magnifies a relative perturbation of A or b that is spread over
// all singular directions, as the FP32 rounding of the mixed assembly is
// (about 1 away from the mesh's interior resonances, large near them).
__global__ void sweep_probe_init_kernel(double2 *__restrict__ z, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        // (+-1 +- i) / sqrt 2 from a 64-bit hash of the index
        uint64_t h = (uint64_t)i * 0x9E3779B97F4A7C15ull;
        h ^= h >> 31;
        h *= 0xBF58476D1CE4E5B9ull;
        h ^= h >> 29;
        const double a = 0.7071067811865476;
        z[i] = make_double2((h & 1u) ? a : -a, (h & 2u) ? a : -a);
    }
}

__global__ void sweep_amp_kernel(const double2 *__restrict__ wz, const double2 *__restrict__ y,
                                 const double2 *__restrict__ z, int64_t n, const int *__restrict__ jd, int jhost,
                                 double *__restrict__ amp) {
    __shared__ double s[3][32];
    double a = 0, b = 0, c = 0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        a += wz[i].x * wz[i].x + wz[i].y * wz[i].y;
        b += y[i].x * y[i].x + y[i].y * y[i].y;
        c += z[i].x * z[i].x + z[i].y * z[i].y;
    }
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
        c += __shfl_down_sync(0xffffffffu, c, o);
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) {
        s[0][w] = a;
        s[1][w] = b;
        s[2][w] = c;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        a = b = c = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
            a += s[0][k];
            b += s[1][k];
            c += s[2][k];
        }
        amp[jd ? *jd : jhost] = c > 0 ? sqrt(a * b) / c : 0.0;
    }
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

// One mesh of the sweep: its buffers, operators and results.
struct MeshRun {
    Ctx &c;
    int64_t N;
    int nk;
    bool mixed;
    bool df64;        // FP64-grade assembly in double-float arithmetic
    double kmax = 0;  // largest |k| of the sweep (the double-float phase tables' bound)
    DevBuf F, G, vec, P, dinfo, kb, ctl, tsb;
    double2 *Cv, *dg, *b, *wd, *X;
    double2 *pz = nullptr, *py = nullptr, *pw = nullptr;   // sensitivity probe: z, y ~ A^-1 z, A z
    double *amp = nullptr;                                 // nk sensitivity estimates (device)
    bool probe = false;
    bie_gmres_opts gp{};                                   // the probe's short solve
    bie_gmres_info *dgi_probe = nullptr;
    bie_gmres_info *dgi;
    double *ks_d, *kcur;
    int *jd;
    unsigned long long *ts;
    bie_gmres_opts go{};
    bie_operator op{}, gop{};
    std::vector<bie_gmres_info> hinfo;
    double asm_ms = 0, sol_ms = 0;

    MeshRun(Ctx &ctx, int nk_, const double *ks, const double *w, const bie_sweep_opts &o)
        : c(ctx), N(ctx.n_sources), nk(nk_), mixed(o.precision == BIE_PREC_MIXED),
          df64(o.precision == BIE_PREC_DF64),
          F((size_t)N * N * (mixed ? 8 : 16)), G((size_t)N * N * (mixed ? 8 : 16)),
          vec(7 * (size_t)N * 16 + (size_t)nk * 8),
          P((size_t)(nk + 1) * N * 16), dinfo((size_t)(nk + 1) * sizeof(bie_gmres_info)),
          kb(((size_t)2 * nk + 2) * sizeof(double)), ctl(256), tsb((size_t)3 * nk * 8), hinfo(nk) {
        Cv = vec.as<double2>();
        dg = Cv + N;
        b = dg + N;
        wd = b + N;
        pz = wd + N;
        py = pz + N;
        pw = py + N;
        amp = reinterpret_cast<double *>(pw + N);
        X = P.as<double2>();
        dgi = dinfo.as<bie_gmres_info>();
        dgi_probe = dgi + nk;
        probe = mixed && o.target_error > 0;
        if (probe) {
            BIE_CUDA(cudaMemsetAsync(amp, 0, (size_t)nk * 8, c.stream));
            sweep_probe_init_kernel<<<(unsigned)std::min<int64_t>((N + 255) / 256, 4LL * c.num_sms), 256, 0,
                                      c.stream>>>(pz, N);
            BIE_CUDA(cudaGetLastError());
            ++c.kernel_launches;
            // a few Arnoldi cycles to 1e-4: enough to resolve the near-null
            // direction, whose share of a random z is about 1 / sqrt(N)
            gp.restart = 20;
            gp.maxiter = 40;
            gp.reltol = 1e-4;
            gp.precision = BIE_PREC_MIXED;
        }
        ks_d = kb.as<double>();
        kcur = ks_d + 2 * nk;
        jd = ctl.as<int>();
        ts = tsb.as<unsigned long long>();
        BIE_CUDA(cudaMemcpyAsync(wd, w, (size_t)N * 16, cudaMemcpyHostToDevice, c.stream));
        BIE_CUDA(cudaMemcpyAsync(ks_d, ks, (size_t)2 * nk * sizeof(double), cudaMemcpyHostToDevice, c.stream));
        BIE_CUDA(cudaMemsetAsync(tsb.p, 0, (size_t)3 * nk * 8, c.stream));
        // (F + Diagonal(1 - C)) p = b: mixed + refine: iterations with the fast
        // complex64 product (~1e-7), refined with residuals from the exact
        // complex64 product; mixed without refine: the exact complex64 product
        // throughout; plain: FP64 GMRES on complex128 matrices
        go = o.gmres;
        go.refine = (mixed && o.refine) ? 1 : 0;
        go.precision = go.refine ? BIE_PREC_MIXED : BIE_PREC_FP64;
        if (go.refine && !(go.inner_reltol > 0)) go.inner_reltol = 1e-6;
        go.initially_nonzero = 0;
        op.kind = BIE_OP_DENSE;
        if (mixed) op.A32 = F.as<float>();
        else op.A = F.as<double>();
        op.scale_re = 1.0;
        op.diag = reinterpret_cast<const double *>(dg);
        gop.kind = BIE_OP_DENSE;
        if (mixed) gop.A32 = G.as<float>();
        else gop.A = G.as<double>();
        gop.scale_re = 1.0;
    }

    int restart() const { return (int)std::max<int64_t>(1, std::min<int64_t>(go.restart > 0 ? go.restart : 20, N)); }

    // assembly of one wavenumber (k_re, k_im; or from device memory kd, with k_im
    // only selecting the complex-k code path)
    void assemble(double kr, double ki, const double *kd) {
        AssembleArgs a{kr, ki, c.d_sources, N, BIE_F | BIE_G | BIE_C, F.as<double>(), G.as<double>(),
                       reinterpret_cast<double *>(Cv)};
        a.c64_out = mixed;
        a.k_dev = kd;
        a.k_abs_max = kmax;
        if (mixed) launch_assemble_mixed(c, a);
        else if (!(df64 && launch_assemble_df64(c, a))) launch_assemble_fp64(c, a);
    }
    // diag = 1 - C, b = G w (the exact complex64 product in the mixed path)
    void rhs() {
        one_minus_kernel<<<(unsigned)((N + 255) / 256), 256, 0, c.stream>>>(Cv, dg, N);
        BIE_CUDA(cudaGetLastError());
        ++c.kernel_launches;
        apply_operator(c, gop, BIE_PREC_FP64, reinterpret_cast<const double *>(wd), reinterpret_cast<double *>(b));
    }
    // wavenumber j launch by launch, timed by events e[0..2]
    void eager(int j, const double *ks, const cudaEvent_t *e) {
        BIE_CUDA(cudaEventRecord(e[0], c.stream));
        assemble(ks[2 * j], ks[2 * j + 1], nullptr);
        BIE_CUDA(cudaEventRecord(e[1], c.stream));
        rhs();
        run_gmres(c, op, reinterpret_cast<const double *>(b), reinterpret_cast<double *>(X + (size_t)j * N), go,
                  hinfo[j]);
        if (probe) {
            bie_gmres_info pi{};
            run_gmres(c, op, reinterpret_cast<const double *>(pz), reinterpret_cast<double *>(py), gp, pi);
            finish_probe(nullptr, j);
        }
        BIE_CUDA(cudaEventRecord(e[2], c.stream));
        BIE_CUDA(cudaStreamSynchronize(c.stream));
        float ta = 0, tsv = 0;
        BIE_CUDA(cudaEventElapsedTime(&ta, e[0], e[1]));
        BIE_CUDA(cudaEventElapsedTime(&tsv, e[1], e[2]));
        asm_ms += ta;
        sol_ms += tsv;
    }
    // amp[j] from y and A z
    void finish_probe(const int *jdev, int jhost) {
        apply_operator(c, op, BIE_PREC_MIXED, reinterpret_cast<const double *>(pz), reinterpret_cast<double *>(pw));
        sweep_amp_kernel<<<1, 1024, 0, c.stream>>>(pw, py, pz, N, jdev, jhost, amp);
        BIE_CUDA(cudaGetLastError());
        ++c.kernel_launches;
    }
    // record wavenumbers 1 .. nk-1 as a WHILE node appended on `top`; the loop
    // body is captured on the context stream, the GMRES bodies on body[0..3]
    void record(cudaStream_t top, const cudaStream_t *body, bool cplx) {
        const cudaGraphConditionalHandle h = graph_new_handle(top);
        sweep_begin_kernel<<<1, 1, 0, top>>>(jd, 1, nk, h);
        BIE_CUDA(cudaGetLastError());
        cudaGraph_t loop_body;
        graph_add_conditional(top, h, cudaGraphCondTypeWhile, 1, &loop_body);
        BodyCapture bc(c.stream, loop_body);
        sweep_k_kernel<<<1, 1, 0, c.stream>>>(ks_d, jd, kcur, ts);
        BIE_CUDA(cudaGetLastError());
        assemble(0.0, cplx ? 1.0 : 0.0, kcur);
        sweep_stamp_kernel<<<1, 1, 0, c.stream>>>(jd, ts, 1);
        BIE_CUDA(cudaGetLastError());
        rhs();
        // the solve writes the extra column X[nk] and dgi[0]; the store moves them
        double2 *xs = X + (size_t)nk * N;
        capture_gmres(c, op, reinterpret_cast<const double *>(b), reinterpret_cast<double *>(xs), go, dgi, body);
        if (probe) {
            capture_gmres(c, op, reinterpret_cast<const double *>(pz), reinterpret_cast<double *>(py), gp, dgi_probe,
                          body);
            finish_probe(jd, 0);
        }
        sweep_store_kernel<<<(unsigned)std::min<int64_t>((N + 255) / 256, 4LL * c.num_sms), 256, 0, c.stream>>>(
            xs, X, N, jd, dgi, dgi);
        BIE_CUDA(cudaGetLastError());
        sweep_next_kernel<<<1, 1, 0, c.stream>>>(jd, nk, ts, h);
        BIE_CUDA(cudaGetLastError());
        c.kernel_launches += 5;
        bc.end();
    }
    // statistics and timestamps of the recorded wavenumbers (after the launch)
    void collect() {
        std::vector<unsigned long long> hts((size_t)3 * nk);
        BIE_CUDA(cudaMemcpyAsync(hinfo.data() + 1, dgi + 1, (size_t)(nk - 1) * sizeof(bie_gmres_info),
                                 cudaMemcpyDeviceToHost, c.stream));
        BIE_CUDA(cudaMemcpyAsync(hts.data(), ts, hts.size() * 8, cudaMemcpyDeviceToHost, c.stream));
        BIE_CUDA(cudaStreamSynchronize(c.stream));
        for (int j = 1; j < nk; ++j) {
            asm_ms += 1e-6 * (double)(hts[3 * j + 1] - hts[3 * j]);
            sol_ms += 1e-6 * (double)(hts[3 * j + 2] - hts[3 * j + 1]);
        }
    }
    // Solves whose sensitivity estimate times the mixed path's typical error
    // exceeds opts.target_error are solved again at FP64 grade: double-float
    // assembly of complex128 F, G, C and FP64 GMRES, launch by launch.
    void accurate_pass(int m, const double *ks, const double *w, const bie_sweep_opts &o, bie_sweep_info &info,
                       const cudaEvent_t *e) {
        if (!probe) return;
        std::vector<double> amph((size_t)nk);
        BIE_CUDA(cudaMemcpyAsync(amph.data(), amp, (size_t)nk * 8, cudaMemcpyDeviceToHost, c.stream));
        BIE_CUDA(cudaStreamSynchronize(c.stream));
        if (o.sensitivity)
            for (int j = 0; j < nk; ++j) o.sensitivity[(size_t)m * nk + j] = amph[j];
        std::vector<int> flag;
        for (int j = 0; j < nk; ++j)
            if (!(amph[j] * kMixedSweepError <= o.target_error)) flag.push_back(j);   // NaN: re-solve too
        if (flag.empty()) return;
        const int nf = (int)flag.size();
        std::vector<double> kf((size_t)2 * nf);
        for (int t = 0; t < nf; ++t) {
            kf[2 * t] = ks[2 * flag[t]];
            kf[2 * t + 1] = ks[2 * flag[t] + 1];
        }
        bie_sweep_opts od = o;
        od.precision = BIE_PREC_DF64;
        od.refine = 0;
        od.target_error = 0;
        od.eager = 1;
        MeshRun rd(c, nf, kf.data(), w, od);
        for (int t = 0; t < nf; ++t) {
            rd.eager(t, kf.data(), e);
            BIE_CUDA(cudaMemcpyAsync(X + (size_t)flag[t] * N, rd.X + (size_t)t * N, (size_t)N * 16,
                                     cudaMemcpyDeviceToDevice, c.stream));
            hinfo[flag[t]] = rd.hinfo[t];
        }
        asm_ms += rd.asm_ms;
        sol_ms += rd.sol_ms;
        info.accurate_solves += nf;
    }
    void finish(double *p_host, int m, bie_sweep_info &info, int32_t *iters) {
        BIE_CUDA(cudaMemcpyAsync(p_host, X, (size_t)nk * N * 16, cudaMemcpyDeviceToHost, c.stream));
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
};

// Capture streams and graph objects of the recorded sweep; ends an unfinished
// capture and restores the contexts' flags if an error unwinds.  The
// top-level graph is captured on `top`.
struct GraphScope {
    std::vector<Ctx *> cs;
    std::vector<bool> timing_saved;
    cudaStream_t top = nullptr;
    cudaStream_t body[4] = {};
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool capturing = false;
    explicit GraphScope(const std::vector<Ctx *> &ctxs) : cs(ctxs) {
        for (Ctx *c : cs) timing_saved.push_back(c->timing);
        BIE_CUDA(cudaStreamCreateWithFlags(&top, cudaStreamNonBlocking));
        for (auto &s : body) BIE_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    }
    void flags(bool on) {
        for (size_t i = 0; i < cs.size(); ++i) {
            cs[i]->timing = on ? false : timing_saved[i];   // no host-side event timers in a graph
            cs[i]->capturing = on;
        }
    }
    void begin() {
        flags(true);
        BIE_CUDA(cudaStreamBeginCapture(top, cudaStreamCaptureModeRelaxed));
        capturing = true;
    }
    void end() {
        capturing = false;
        flags(false);
        BIE_CUDA(cudaStreamEndCapture(top, &graph));
    }
    ~GraphScope() {
        if (capturing) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(top, &g);
            if (g) cudaGraphDestroy(g);
            flags(false);
        }
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (top) cudaStreamDestroy(top);
        for (auto &s : body)
            if (s) cudaStreamDestroy(s);
    }
    GraphScope(const GraphScope &) = delete;
    GraphScope &operator=(const GraphScope &) = delete;
};

struct Events {
    cudaEvent_t e[3] = {};
    Events() {
        for (auto &x : e) BIE_CUDA(cudaEventCreate(&x));
    }
    ~Events() {
        for (auto x : e)
            if (x) cudaEventDestroy(x);
    }
};

}  // namespace

void run_sweep(Ctx *const *ctxs, int nmesh, const double *ks, int nk, const double *const *w,
               double *const *p, const bie_sweep_opts &o, bie_sweep_info &info, int32_t *iters) {
    info = bie_sweep_info{};
    // every distinct context locked once, in address order
    std::vector<Ctx *> uniq(ctxs, ctxs + nmesh);
    std::sort(uniq.begin(), uniq.end());
    uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
    std::vector<std::unique_lock<std::mutex>> locks;
    for (Ctx *c : uniq) locks.emplace_back(c->mu);

    bool graph = !o.eager && nk > 1;
    for (int m = 0; m < nmesh; ++m) {
        const int64_t N = ctxs[m]->n_sources;
        const int64_t restart = std::max<int64_t>(1, std::min<int64_t>(o.gmres.restart > 0 ? o.gmres.restart : 20, N));
        if (restart > kGraphMaxRestart || ctxs[m]->device != ctxs[0]->device) graph = false;
    }
    bool cplx = false;   // any complex k: the complex-k kernels serve every recorded wavenumber
    for (int j = 1; j < nk; ++j) cplx = cplx || ks[2 * j + 1] != 0.0;
    Events ev;

    if (!graph) {   // launch by launch, one mesh (and its matrices) at a time
        for (int m = 0; m < nmesh; ++m) {
            Ctx &c = *ctxs[m];
            BIE_CUDA(cudaSetDevice(c.device));
            c.autotune = true;   // the first wavenumber of a mesh picks its slicing
            MeshRun r(c, nk, ks, w[m], o);
            for (int j = 0; j < nk; ++j) r.eager(j, ks, ev.e);
            r.accurate_pass(m, ks, w[m], o, info, ev.e);
            r.finish(p[m], m, info, iters);
        }
        return;
    }

    BIE_CUDA(cudaSetDevice(ctxs[0]->device));
    std::vector<std::unique_ptr<MeshRun>> runs;
    for (int m = 0; m < nmesh; ++m) {
        Ctx &c = *ctxs[m];
        c.autotune = true;
        runs.push_back(std::make_unique<MeshRun>(c, nk, ks, w[m], o));
        for (int j = 0; j < nk; ++j) runs.back()->kmax = std::max(runs.back()->kmax, std::hypot(ks[2 * j], ks[2 * j + 1]));
        runs.back()->eager(0, ks, ev.e);   // sizes the scratch, tunes the slicing
    }
    GraphScope gs(uniq);
    const auto t0 = std::chrono::steady_clock::now();
    gs.begin();
    for (auto &r : runs) r->record(gs.top, gs.body, cplx);
    gs.end();
    BIE_CUDA(cudaGraphInstantiate(&gs.exec, gs.graph, 0));
    info.record_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    BIE_CUDA(cudaGraphLaunch(gs.exec, gs.top));
    ++info.graph_launches;
    BIE_CUDA(cudaStreamSynchronize(gs.top));
    for (int m = 0; m < nmesh; ++m) {
        runs[m]->collect();
        runs[m]->accurate_pass(m, ks, w[m], o, info, ev.e);
        runs[m]->finish(p[m], m, info, iters);
    }
}

}  // namespace bie
