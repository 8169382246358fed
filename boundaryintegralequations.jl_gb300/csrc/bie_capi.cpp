// C-ABI entry points of libbiegpu.so (declared in include/biegpu.h).
// Each wrapper validates its arguments, runs under the context mutex, converts
// every bie::Error / std::exception into a status code and a thread-local
// message, and never lets an exception cross the boundary.
#include "bie_internal.h"

#include <cmath>
#include <exception>
#include <new>

namespace {

thread_local std::string g_last_error;

template <class Fn>
int guarded(Fn &&fn) {
    try {
        g_last_error.clear();
        fn();
        return BIE_OK;
    } catch (const bie::Error &e) {
        g_last_error = e.msg;
        return e.code;
    } catch (const std::bad_alloc &) {
        g_last_error = "host allocation failed";
        return BIE_ERR_NOMEM;
    } catch (const std::exception &e) {
        g_last_error = e.what();
        return BIE_ERR_INVALID;
    } catch (...) {
        g_last_error = "unknown error";
        return BIE_ERR_INVALID;
    }
}

bie::Ctx *as_ctx(bie_ctx *p) {
    if (!p) bie::fail(BIE_ERR_INVALID, "context is NULL");
    return reinterpret_cast<bie::Ctx *>(p);
}

void check_assemble_args(bie::Ctx &c, double kr, double ki, int64_t M, int flags, int precision,
                         const void *F, const void *G, const void *C) {
    if (!std::isfinite(kr) || !std::isfinite(ki)) bie::fail(BIE_ERR_INVALID, "k must be finite");
    if (M <= 0) bie::fail(BIE_ERR_INVALID, "number of targets must be positive");
    if (flags & ~(BIE_F | BIE_G | BIE_C)) bie::fail(BIE_ERR_INVALID, "unknown flag bits");
    if (precision != BIE_PREC_FP64 && precision != BIE_PREC_MIXED)
        bie::fail(BIE_ERR_INVALID, "unknown precision");
    if ((flags & BIE_F) && !F) bie::fail(BIE_ERR_INVALID, "F requested but NULL");
    if ((flags & BIE_G) && !G) bie::fail(BIE_ERR_INVALID, "G requested but NULL");
    if ((flags & BIE_C) && !C) bie::fail(BIE_ERR_INVALID, "C requested but NULL");
    // M * N * 16 bytes must not overflow
    if (M > (int64_t)(INT64_MAX / 16) / c.n_sources)
        bie::fail(BIE_ERR_INVALID, "M x N output too large");
}

void run_assemble(bie::Ctx &c, const bie::AssembleArgs &a, int precision) {
    if (precision == BIE_PREC_MIXED) bie::launch_assemble_mixed(c, a);
    else bie::launch_assemble_fp64(c, a);
}

}  // namespace

extern "C" {

const char *bie_version(void) { return "biegpu 0.1.0 sm_103a"; }

const char *bie_last_error(void) { return g_last_error.c_str(); }

int bie_quadrature_rule(int n, int m, int node, double *u, double *v, double *w, int capacity,
                        int *count) {
    return guarded([&] {
        if (!count) bie::fail(BIE_ERR_INVALID, "count must not be NULL");
        if (n < 1 || m < 1 || n > 32 || m > 32) bie::fail(BIE_ERR_INVALID, "n, m must be in 1..32");
        if (node < 1 || node > 6) bie::fail(BIE_ERR_INVALID, "node must be in 1..6");
        bie::Rule r = node <= 3 ? bie::duffy_corner_rule(n, m, node) : bie::duffy_midpoint_rule(n, m, node);
        *count = r.size();
        if (r.size() > capacity) bie::fail(BIE_ERR_INVALID, "capacity too small for the rule");
        if (!u || !v || !w) bie::fail(BIE_ERR_INVALID, "u, v, w must not be NULL");
        for (int q = 0; q < r.size(); ++q) {
            u[q] = r.u[q];
            v[q] = r.v[q];
            w[q] = r.w[q];
        }
    });
}

int bie_ctx_create(bie_ctx **out, const bie_mesh_desc *desc, int device) {
    return guarded([&] {
        if (!out || !desc) bie::fail(BIE_ERR_INVALID, "out and desc must not be NULL");
        *out = nullptr;
        auto *c = new bie::Ctx();
        try {
            bie::build_context(*c, *desc, device);
        } catch (...) {
            bie::destroy_context(*c);
            delete c;
            throw;
        }
        *out = reinterpret_cast<bie_ctx *>(c);
    });
}

int bie_ctx_destroy(bie_ctx *ctx) {
    return guarded([&] {
        if (!ctx) return;
        auto *c = reinterpret_cast<bie::Ctx *>(ctx);
        bie::destroy_context(*c);
        delete c;
    });
}

int bie_ctx_stream(bie_ctx *ctx, void **stream) {
    return guarded([&] {
        bie::Ctx &c = *as_ctx(ctx);
        if (!stream) bie::fail(BIE_ERR_INVALID, "stream out-pointer is NULL");
        *stream = (void *)c.stream;
    });
}

int bie_measure_peaks(int device, bie_peaks *out) {
    return guarded([&] {
        if (!out) bie::fail(BIE_ERR_INVALID, "out must not be NULL");
        bie::measure_peaks(device, *out);
    });
}

int bie_ctx_set_timing(bie_ctx *ctx, int on) {
    return guarded([&] {
        bie::Ctx &c = *as_ctx(ctx);
        std::lock_guard<std::mutex> lock(c.mu);
        c.timing = on != 0;
    });
}

int bie_ctx_stats(bie_ctx *ctx, bie_stats *out, int reset) {
    return guarded([&] {
        bie::Ctx &c = *as_ctx(ctx);
        if (!out) bie::fail(BIE_ERR_INVALID, "stats out-pointer is NULL");
        std::lock_guard<std::mutex> lock(c.mu);
        BIE_CUDA(cudaSetDevice(c.device));
        c.collect_timers();
        unsigned long long q = 0;
        BIE_CUDA(cudaMemcpy(&q, c.d_qpe, sizeof(q), cudaMemcpyDeviceToHost));
        out->kernel_launches = c.kernel_launches;
        out->timed_launches = c.timed_launches;
        out->timed_ms = c.timed_ms;
        out->quadrature_evals = (int64_t)q;
        out->algorithmic_flops = (double)q * (32.0 + 8.0 * c.lay.NP);
        if (reset) {
            c.kernel_launches = 0;
            c.timed_launches = 0;
            c.timed_ms = 0.0;
            BIE_CUDA(cudaMemset(c.d_qpe, 0, sizeof(unsigned long long)));
        }
    });
}

int bie_assemble(bie_ctx *ctx, double k_re, double k_im, const double *targets, int64_t n_targets,
                 int flags, int precision, double *F, double *G, double *C) {
    return guarded([&] {
        bie::Ctx &c = *as_ctx(ctx);
        std::lock_guard<std::mutex> lock(c.mu);
        const int64_t M = targets ? n_targets : c.n_sources;
        check_assemble_args(c, k_re, k_im, M, flags, precision, F, G, C);
        BIE_CUDA(cudaSetDevice(c.device));
        const double *d_t = c.d_sources;
        if (targets) {
            for (int64_t i = 0; i < 3 * M; ++i)
                if (!std::isfinite(targets[i])) bie::fail(BIE_ERR_INVALID, "non-finite target");
            double *dt = static_cast<double *>(c.scratch(bie::kScratchTargets, (size_t)M * 24));
            BIE_CUDA(cudaMemcpyAsync(dt, targets, (size_t)M * 24, cudaMemcpyHostToDevice, c.stream));
            d_t = dt;
        }
        const size_t mat = (size_t)M * (size_t)c.n_sources * 16;
        bie::AssembleArgs a{k_re, k_im, d_t, M, flags, nullptr, nullptr, nullptr};
        if (flags & BIE_F) a.F = static_cast<double *>(c.scratch(bie::kScratchF, mat));
        if (flags & BIE_G) a.G = static_cast<double *>(c.scratch(bie::kScratchG, mat));
        if (flags & BIE_C) a.C = static_cast<double *>(c.scratch(bie::kScratchC, (size_t)M * 16));
        run_assemble(c, a, precision);
        if (flags & BIE_F) BIE_CUDA(cudaMemcpyAsync(F, a.F, mat, cudaMemcpyDeviceToHost, c.stream));
        if (flags & BIE_G) BIE_CUDA(cudaMemcpyAsync(G, a.G, mat, cudaMemcpyDeviceToHost, c.stream));
        if (flags & BIE_C)
            BIE_CUDA(cudaMemcpyAsync(C, a.C, (size_t)M * 16, cudaMemcpyDeviceToHost, c.stream));
        BIE_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int bie_assemble_device(bie_ctx *ctx, double k_re, double k_im, const double *d_targets,
                        int64_t n_targets, int flags, int precision, double *d_F, double *d_G,
                        double *d_C) {
    return guarded([&] {
        bie::Ctx &c = *as_ctx(ctx);
        std::lock_guard<std::mutex> lock(c.mu);
        const int64_t M = d_targets ? n_targets : c.n_sources;
        check_assemble_args(c, k_re, k_im, M, flags, precision, d_F, d_G, d_C);
        BIE_CUDA(cudaSetDevice(c.device));
        bie::AssembleArgs a{k_re, k_im, d_targets ? d_targets : c.d_sources, M, flags,
                            d_F, d_G, d_C};
        run_assemble(c, a, precision);
    });
}

}  // extern "C"
