// C-ABI entry points of libbiegpu.so (declared in include/biegpu.h).
// Each wrapper validates its arguments, runs under the context mutex, converts
// every bie::Error / std::exception into a status code and a thread-local
// message, and never lets an exception cross the boundary.
#include "bie_internal.h"

#include <algorithm>
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

bie::FastOp &as_fastop(bie_fastop *op) {
    if (!op) bie::fail(BIE_ERR_INVALID, "operator is NULL");
    return *reinterpret_cast<bie::FastOp *>(op);
}

void check_prec2(int precision) {
    if (precision != BIE_PREC_FP64 && precision != BIE_PREC_MIXED && precision != BIE_PREC_DF64)
        bie::fail(BIE_ERR_INVALID, "precision must be BIE_PREC_FP64, BIE_PREC_MIXED or BIE_PREC_DF64");
}

void check_assemble_args(bie::Ctx &c, double kr, double ki, int64_t M, int flags, int precision,
                         const void *F, const void *G, const void *C) {
    if (!std::isfinite(kr) || !std::isfinite(ki)) bie::fail(BIE_ERR_INVALID, "k must be finite");
    if (M <= 0) bie::fail(BIE_ERR_INVALID, "number of targets must be positive");
    if (flags & ~(BIE_F | BIE_G | BIE_C)) bie::fail(BIE_ERR_INVALID, "unknown flag bits");
    if (precision != BIE_PREC_FP64 && precision != BIE_PREC_MIXED && precision != BIE_PREC_DF64)
        bie::fail(BIE_ERR_INVALID, "unknown precision");
    if ((flags & BIE_F) && !F) bie::fail(BIE_ERR_INVALID, "F requested but NULL");
    if ((flags & BIE_G) && !G) bie::fail(BIE_ERR_INVALID, "G requested but NULL");
    if ((flags & BIE_C) && !C) bie::fail(BIE_ERR_INVALID, "C requested but NULL");
    // M * N * 16 bytes must not overflow
    if (M > (int64_t)(INT64_MAX / 16) / c.n_sources)
        bie::fail(BIE_ERR_INVALID, "M x N output too large");
}

void check_matvec_args(bie::Ctx &c, double kr, double ki, int64_t M, int precision, const void *x,
                       const void *v, const void *yF, const void *yG) {
    (void)c;
    if (!std::isfinite(kr) || !std::isfinite(ki)) bie::fail(BIE_ERR_INVALID, "k must be finite");
    if (M <= 0) bie::fail(BIE_ERR_INVALID, "number of targets must be positive");
    if (precision != BIE_PREC_FP64 && precision != BIE_PREC_MIXED && precision != BIE_PREC_DF64)
        bie::fail(BIE_ERR_INVALID, "unknown precision");
    if (!x && !v) bie::fail(BIE_ERR_INVALID, "neither x nor v given");
    if (x && !yF) bie::fail(BIE_ERR_INVALID, "x given without yF");
    if (v && !yG) bie::fail(BIE_ERR_INVALID, "v given without yG");
}

void run_assemble(bie::Ctx &c, const bie::AssembleArgs &a, int precision) {
    if (precision == BIE_PREC_MIXED) bie::launch_assemble_mixed(c, a);
    else if (precision == BIE_PREC_DF64 && bie::launch_assemble_df64(c, a)) return;
    else bie::launch_assemble_fp64(c, a);
}

bie::LossyOp &as_lossy(bie_lossy *L) {
    if (!L) bie::fail(BIE_ERR_INVALID, "lossy system is NULL");
    return *reinterpret_cast<bie::LossyOp *>(L);
}

void check_block(int block) {
    if (block < BIE_LOSSY_OUTER || block > BIE_LOSSY_INNER) bie::fail(BIE_ERR_INVALID, "unknown lossy block");
}

void check_solve_opts(const bie_gmres_opts &o) {
    if (!(o.reltol >= 0) || !(o.abstol >= 0)) bie::fail(BIE_ERR_INVALID, "tolerances must be >= 0");
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

int bie_basis(int kind, double beta, int64_t n, const double *u, const double *v, double *N, double *dNu,
              double *dNv) {
    return guarded([&] {
        const int NP = bie::n_nodes_of_kind(kind);
        if (n < 0 || (n > 0 && (!u || !v))) bie::fail(BIE_ERR_INVALID, "u and v must hold n >= 0 points");
        if (bie::is_discontinuous(kind) && kind != BIE_TRI_DISC_CONSTANT && !(beta > 0.0 && beta < 1.0 / 3.0))
            bie::fail(BIE_ERR_INVALID, "beta of discontinuous physics must lie in (0, 1/3)");
        double nv[6], du[6], dv[6];
        for (int64_t q = 0; q < n; ++q) {
            bie::physics_values(kind, beta, u[q], v[q], nv);
            bie::physics_derivs(kind, beta, u[q], v[q], du, dv);
            for (int a = 0; a < NP; ++a) {
                if (N) N[q * NP + a] = nv[a];
                if (dNu) dNu[q * NP + a] = du[a];
                if (dNv) dNv[q * NP + a] = dv[a];
            }
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

int bie_ctx_create_rules(bie_ctx **out, const bie_mesh_desc *desc, const bie_rule_table *rules, int n_rules,
                         int device) {
    return guarded([&] {
        if (!out || !desc || !rules) bie::fail(BIE_ERR_INVALID, "out, desc and rules must not be NULL");
        *out = nullptr;
        if (n_rules < 1 || n_rules > 6) bie::fail(BIE_ERR_INVALID, "n_rules must be in 1..6");
        std::vector<bie::Rule> tables((size_t)n_rules);
        for (int r = 0; r < n_rules; ++r) {
            const bie_rule_table &t = rules[r];
            if (t.n_points < 1 || t.n_points > bie::kMaxQ)
                bie::fail(BIE_ERR_INVALID, "rule table " + std::to_string(r) + " must hold 1.." +
                                               std::to_string(bie::kMaxQ) + " points");
            if (!t.u || !t.v || !t.w)
                bie::fail(BIE_ERR_INVALID, "rule table " + std::to_string(r) + " has a NULL array");
            tables[r].u.assign(t.u, t.u + t.n_points);
            tables[r].v.assign(t.v, t.v + t.n_points);
            tables[r].w.assign(t.w, t.w + t.n_points);
        }
        auto *c = new bie::Ctx();
        try {
            bie::build_context(*c, *desc, device, 0, &tables);
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

int bie_ctx_set_autotune(bie_ctx *ctx, int on) {
    return guarded([&] {
        bie::Ctx &c = *as_ctx(ctx);
        std::lock_guard<std::mutex> lock(c.mu);
        c.autotune = on != 0;
    });
}

int bie_ctx_get_shape(bie_ctx *ctx, int kernel, int64_t M, int *found, int *level, int *chunk, int *tpb) {
    return guarded([&] {
        bie::Ctx &c = *as_ctx(ctx);
        std::lock_guard<std::mutex> lock(c.mu);
        if (!found) bie::fail(BIE_ERR_INVALID, "found must not be NULL");
        if (kernel < 0 || kernel >= bie::kShapeCount) bie::fail(BIE_ERR_INVALID, "unknown kernel id");
        *found = 0;
        const bie::LaunchShape *sh = nullptr;
        for (const int64_t key : {M, int64_t(0)}) {
            const auto f = c.forced_shapes.find({kernel, key});
            if (f != c.forced_shapes.end()) {
                sh = &f->second;
                break;
            }
        }
        if (!sh) {
            const auto t = c.tuned_shapes.find({kernel, M});
            if (t != c.tuned_shapes.end()) sh = &t->second;
        }
        if (!sh) return;
        *found = 1;
        if (level) *level = sh->level;
        if (chunk) *chunk = sh->chunk;
        if (tpb) *tpb = sh->tpb;
    });
}

int bie_ctx_set_shape(bie_ctx *ctx, int kernel, int64_t M, int level, int chunk, int tpb) {
    return guarded([&] {
        bie::Ctx &c = *as_ctx(ctx);
        std::lock_guard<std::mutex> lock(c.mu);
        if (kernel < 0 || kernel >= bie::kShapeCount) bie::fail(BIE_ERR_INVALID, "unknown kernel id");
        if (M < 0) bie::fail(BIE_ERR_INVALID, "M must be >= 0");
        if (level < 0) {
            c.forced_shapes.erase({kernel, M});
            return;
        }
        if (level >= bie::kMaxLevels || (int64_t(1) << level) > c.n_elements)
            bie::fail(BIE_ERR_INVALID, "level must be in 0.." + std::to_string(bie::kMaxLevels - 1) +
                                           " with at most one slice per element");
        if (chunk > 64) bie::fail(BIE_ERR_INVALID, "chunk must be at most 64 records");
        c.forced_shapes[{kernel, M}] = bie::LaunchShape{level, chunk, tpb};
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
        out->tensor_launches = c.tensor_launches;
        out->tensor_ms = c.tensor_ms;
        out->tensor_flops = c.tensor_flops;
        out->tensor_flops_executed = c.tensor_flops_executed;
        if (reset) {
            c.kernel_launches = 0;
            c.timed_launches = 0;
            c.timed_ms = 0.0;
            c.tensor_launches = 0;
            c.tensor_ms = 0.0;
            c.tensor_flops = 0.0;
            c.tensor_flops_executed = 0.0;
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
        const int64_t N = c.n_sources;
        const size_t mat = (size_t)M * (size_t)N * 16;
        const int nmat = ((flags & BIE_F) ? 1 : 0) + ((flags & BIE_G) ? 1 : 0);
        // Outputs of 256 MB and more: row blocks assembled on the context stream
        // while the previous block is copied to the host on a second stream, so
        // the assembly hides behind the device-to-host transfer (which bounds
        // this call).  Each block is its own assembly over targets [i0, i1); a
        // block's rows are a strided 2D copy whose row segments are kept >= 45 KB
        // (narrower segments slow the copy engines: measured 193 GB/s at 46 KB,
        // 171 GB/s at 20 KB on GB300), so nb <= 8 and M >= 2 * 2880.
        const int nb = (mat * nmat >= (size_t(256) << 20)) ? (int)std::min<int64_t>(8, M * 16 / 46080) : 1;
        if (nb < 2) {
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
            return;
        }
        const int64_t mb = (M + nb - 1) / nb;   // rows per block
        const size_t blk = (size_t)mb * (size_t)N * 16;
        double *dF = (flags & BIE_F) ? static_cast<double *>(c.scratch(bie::kScratchF, 2 * blk)) : nullptr;
        double *dG = (flags & BIE_G) ? static_cast<double *>(c.scratch(bie::kScratchG, 2 * blk)) : nullptr;
        double *dC = (flags & BIE_C) ? static_cast<double *>(c.scratch(bie::kScratchC, 2 * (size_t)mb * 16)) : nullptr;
        if (!c.copy_stream) BIE_CUDA(cudaStreamCreateWithFlags(&c.copy_stream, cudaStreamNonBlocking));
        struct Events {
            cudaStream_t s0, s1;
            cudaEvent_t e[4] = {};
            ~Events() {   // (also on an error: no copy into the caller's arrays outlives the call)
                cudaStreamSynchronize(s1);
                cudaStreamSynchronize(s0);
                for (auto x : e)
                    if (x) cudaEventDestroy(x);
            }
        } ev{c.stream, c.copy_stream};   // ready[2] (block assembled), copied[2] (slot free again)
        for (auto &x : ev.e) BIE_CUDA(cudaEventCreateWithFlags(&x, cudaEventDisableTiming));
        const int nblocks = (int)((M + mb - 1) / mb);
        auto compute = [&](int b) {
            const int slot = b & 1;
            const int64_t i0 = (int64_t)b * mb, m = std::min<int64_t>(mb, M - i0);
            if (b >= 2) BIE_CUDA(cudaStreamWaitEvent(c.stream, ev.e[2 + slot], 0));
            bie::AssembleArgs a{k_re, k_im, d_t + 3 * i0, m, flags,
                                dF ? dF + slot * (blk / 8) : nullptr, dG ? dG + slot * (blk / 8) : nullptr,
                                dC ? dC + slot * 2 * mb : nullptr};
            run_assemble(c, a, precision);
            BIE_CUDA(cudaEventRecord(ev.e[slot], c.stream));
        };
        auto copy = [&](int b) {
            const int slot = b & 1;
            const int64_t i0 = (int64_t)b * mb, m = std::min<int64_t>(mb, M - i0);
            cudaStream_t s = c.copy_stream;
            BIE_CUDA(cudaStreamWaitEvent(s, ev.e[slot], 0));
            if (dF)
                BIE_CUDA(cudaMemcpy2DAsync(F + 2 * i0, (size_t)M * 16, dF + slot * (blk / 8), (size_t)m * 16,
                                           (size_t)m * 16, (size_t)N, cudaMemcpyDeviceToHost, s));
            if (dG)
                BIE_CUDA(cudaMemcpy2DAsync(G + 2 * i0, (size_t)M * 16, dG + slot * (blk / 8), (size_t)m * 16,
                                           (size_t)m * 16, (size_t)N, cudaMemcpyDeviceToHost, s));
            if (dC)
                BIE_CUDA(cudaMemcpyAsync(C + 2 * i0, dC + slot * 2 * mb, (size_t)m * 16, cudaMemcpyDeviceToHost, s));
            BIE_CUDA(cudaEventRecord(ev.e[2 + slot], s));
        };
        // the next block is enqueued before this block's copy, so that the
        // assembly overlaps the copy even when a pageable host copy blocks
        compute(0);
        for (int b = 0; b < nblocks; ++b) {
            if (b + 1 < nblocks) compute(b + 1);
            copy(b);
        }
        BIE_CUDA(cudaStreamSynchronize(c.copy_stream));
        BIE_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int bie_taylor_assemble(bie_ctx *ctx, double k0_re, double k0_im, const double *targets, int64_t n_targets,
                        int flags, int order, double *F, double *G, double *C) {
    return guarded([&] {
        bie::Ctx &c = *as_ctx(ctx);
        std::lock_guard<std::mutex> lock(c.mu);
        const int64_t M = targets ? n_targets : c.n_sources;
        check_assemble_args(c, k0_re, k0_im, M, flags, BIE_PREC_FP64, F, G, C);
        if (order < 0 || order > 64) bie::fail(BIE_ERR_INVALID, "order must be in 0..64");
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
        const size_t ent = (size_t)M * (size_t)c.n_sources * 2;   // doubles per matrix
        for (int m = 0; m <= order; ++m) {
            const int fl = (flags & (BIE_F | BIE_G)) | (m == 0 ? (flags & BIE_C) : 0);
            bie::AssembleArgs a{k0_re, k0_im, d_t, M, fl, nullptr, nullptr, nullptr};
            a.taylor_m = m;
            if (fl & BIE_F) a.F = static_cast<double *>(c.scratch(bie::kScratchF, mat));
            if (fl & BIE_G) a.G = static_cast<double *>(c.scratch(bie::kScratchG, mat));
            if (fl & BIE_C) a.C = static_cast<double *>(c.scratch(bie::kScratchC, (size_t)M * 16));
            bie::launch_assemble_fp64(c, a);
            if (fl & BIE_F) BIE_CUDA(cudaMemcpyAsync(F + m * ent, a.F, mat, cudaMemcpyDeviceToHost, c.stream));
            if (fl & BIE_G) BIE_CUDA(cudaMemcpyAsync(G + m * ent, a.G, mat, cudaMemcpyDeviceToHost, c.stream));
            if (fl & BIE_C) BIE_CUDA(cudaMemcpyAsync(C, a.C, (size_t)M * 16, cudaMemcpyDeviceToHost, c.stream));
            BIE_CUDA(cudaStreamSynchronize(c.stream));
        }
    });
}

int bie_matvec(bie_ctx *ctx, double k_re, double k_im, const double *targets, int64_t n_targets,
               const double *x, const double *v, double *yF, double *yG, int precision) {
    return guarded([&] {
        bie::Ctx &c = *as_ctx(ctx);
        std::lock_guard<std::mutex> lock(c.mu);
        const int64_t M = targets ? n_targets : c.n_sources;
        check_matvec_args(c, k_re, k_im, M, precision, x, v, yF, yG);
        BIE_CUDA(cudaSetDevice(c.device));
        const int64_t N = c.n_sources;
        // device staging: targets | x | v | yF | yG  (solver workspace slot is not used here)
        const size_t tb = targets ? (size_t)M * 24 : 0;
        char *buf = static_cast<char *>(c.scratch(bie::kScratchTargets, tb + 2 * (size_t)N * 16 +
                                                                               2 * (size_t)M * 16 + 64));
        double *dt = targets ? reinterpret_cast<double *>(buf) : c.d_sources;
        double *dx = reinterpret_cast<double *>(buf + ((tb + 15) & ~size_t(15)));
        double *dv = dx + 2 * N;
        double *dyF = dv + 2 * N;
        double *dyG = dyF + 2 * M;
        if (targets) {
            for (int64_t i = 0; i < 3 * M; ++i)
                if (!std::isfinite(targets[i])) bie::fail(BIE_ERR_INVALID, "non-finite target");
            BIE_CUDA(cudaMemcpyAsync(dt, targets, tb, cudaMemcpyHostToDevice, c.stream));
        }
        if (x) BIE_CUDA(cudaMemcpyAsync(dx, x, (size_t)N * 16, cudaMemcpyHostToDevice, c.stream));
        if (v) BIE_CUDA(cudaMemcpyAsync(dv, v, (size_t)N * 16, cudaMemcpyHostToDevice, c.stream));
        bie::MatvecArgs a{k_re, k_im, dt, M, x ? dx : nullptr, v ? dv : nullptr, dyF, dyG, precision};
        bie::launch_matvec(c, a);
        if (x) BIE_CUDA(cudaMemcpyAsync(yF, dyF, (size_t)M * 16, cudaMemcpyDeviceToHost, c.stream));
        if (v) BIE_CUDA(cudaMemcpyAsync(yG, dyG, (size_t)M * 16, cudaMemcpyDeviceToHost, c.stream));
        BIE_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int bie_matvec_device(bie_ctx *ctx, double k_re, double k_im, const double *d_targets,
                      int64_t n_targets, const double *d_x, const double *d_v, double *d_yF,
                      double *d_yG, int precision) {
    return guarded([&] {
        bie::Ctx &c = *as_ctx(ctx);
        std::lock_guard<std::mutex> lock(c.mu);
        const int64_t M = d_targets ? n_targets : c.n_sources;
        check_matvec_args(c, k_re, k_im, M, precision, d_x, d_v, d_yF, d_yG);
        BIE_CUDA(cudaSetDevice(c.device));
        bie::MatvecArgs a{k_re, k_im, d_targets ? d_targets : c.d_sources, M, d_x, d_v, d_yF, d_yG,
                          precision};
        bie::launch_matvec(c, a);
    });
}

int bie_matvec_device_noalloc(bie_ctx *ctx, double k_re, double k_im, const double *d_targets,
                              int64_t n_targets, const double *d_x, const double *d_v,
                              double *d_yF, double *d_yG) {
    return guarded([&] {
        bie::Ctx &c = *as_ctx(ctx);
        std::lock_guard<std::mutex> lock(c.mu);
        const int64_t M = d_targets ? n_targets : c.n_sources;
        check_matvec_args(c, k_re, k_im, M, BIE_PREC_MIXED, d_x, d_v, d_yF, d_yG);
        BIE_CUDA(cudaSetDevice(c.device));
        bie::MatvecArgs a{k_re, k_im, d_targets ? d_targets : c.d_sources, M, d_x, d_v, d_yF, d_yG,
                          BIE_PREC_MIXED};
        bie::launch_matvec_noalloc(c, a);
    });
}

int bie_matvec_multi_device(bie_ctx *ctx, double k_re, double k_im, int64_t nrhs, const double *d_X,
                            const double *d_V, double *d_YF, double *d_YG, int precision,
                            int64_t scratch_bytes) {
    return guarded([&] {
        bie::Ctx &c = *as_ctx(ctx);
        std::lock_guard<std::mutex> lock(c.mu);
        if (!std::isfinite(k_re) || !std::isfinite(k_im)) bie::fail(BIE_ERR_INVALID, "k must be finite");
        if (nrhs <= 0) bie::fail(BIE_ERR_INVALID, "nrhs must be positive");
        if (precision < BIE_PREC_FP64 || precision > BIE_PREC_BF16_SPLIT)
            bie::fail(BIE_ERR_INVALID, "unknown precision");
        if (!d_X && !d_V) bie::fail(BIE_ERR_INVALID, "neither X nor V given");
        if (d_X && !d_YF) bie::fail(BIE_ERR_INVALID, "X given without YF");
        if (d_V && !d_YG) bie::fail(BIE_ERR_INVALID, "V given without YG");
        if (scratch_bytes < 0) bie::fail(BIE_ERR_INVALID, "scratch_bytes must be >= 0");
        BIE_CUDA(cudaSetDevice(c.device));
        bie::MultiArgs a{k_re, k_im, nrhs, d_X, d_V, d_YF, d_YG, precision, scratch_bytes};
        bie::run_matvec_multi(c, a);
    });
}

int bie_matvec_multi(bie_ctx *ctx, double k_re, double k_im, int64_t nrhs, const double *X, const double *V,
                     double *YF, double *YG, int precision, int64_t scratch_bytes) {
    return guarded([&] {
        bie::Ctx &c = *as_ctx(ctx);
        if (nrhs <= 0) bie::fail(BIE_ERR_INVALID, "nrhs must be positive");
        if (!X && !V) bie::fail(BIE_ERR_INVALID, "neither X nor V given");
        if ((X && !YF) || (V && !YG)) bie::fail(BIE_ERR_INVALID, "an input is given without its output");
        void *d = nullptr;
        const size_t bytes = (size_t)c.n_sources * (size_t)nrhs * 16;
        const int nbuf = (X ? 2 : 0) + (V ? 2 : 0);
        {
            std::lock_guard<std::mutex> lock(c.mu);
            BIE_CUDA(cudaSetDevice(c.device));
            BIE_CUDA(cudaMalloc(&d, bytes * nbuf));
        }
        struct Free {
            void *p;
            ~Free() { cudaFree(p); }
        } guard{d};
        double *dX = X ? static_cast<double *>(d) : nullptr;
        double *dYF = X ? dX + 2 * c.n_sources * nrhs : nullptr;
        double *dV = V ? static_cast<double *>(d) + (X ? 4 * c.n_sources * nrhs : 0) : nullptr;
        double *dYG = V ? dV + 2 * c.n_sources * nrhs : nullptr;
        {
            std::lock_guard<std::mutex> lock(c.mu);
            if (X) BIE_CUDA(cudaMemcpyAsync(dX, X, bytes, cudaMemcpyHostToDevice, c.stream));
            if (V) BIE_CUDA(cudaMemcpyAsync(dV, V, bytes, cudaMemcpyHostToDevice, c.stream));
        }
        const int st = bie_matvec_multi_device(ctx, k_re, k_im, nrhs, dX, dV, dYF, dYG, precision, scratch_bytes);
        if (st != BIE_OK) bie::fail(st, bie_last_error());
        std::lock_guard<std::mutex> lock(c.mu);
        if (X) BIE_CUDA(cudaMemcpyAsync(YF, dYF, bytes, cudaMemcpyDeviceToHost, c.stream));
        if (V) BIE_CUDA(cudaMemcpyAsync(YG, dYG, bytes, cudaMemcpyDeviceToHost, c.stream));
        BIE_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int bie_lowp_gemm_device(bie_ctx *ctx, int precision, int64_t M, int64_t N, int64_t K, const float *d_A,
                         const float *d_B, double *d_C) {
    return guarded([&] {
        bie::Ctx &c = *as_ctx(ctx);
        std::lock_guard<std::mutex> lock(c.mu);
        if (!d_A || !d_B || !d_C) bie::fail(BIE_ERR_INVALID, "A, B and C must not be NULL");
        if (precision < BIE_PREC_FP16 || precision > BIE_PREC_BF16_SPLIT)
            bie::fail(BIE_ERR_INVALID, "precision must be one of the 16-bit tensor-core forms");
        BIE_CUDA(cudaSetDevice(c.device));
        bie::run_lowp_gemm(c, precision, M, N, K, d_A, d_B, d_C);
    });
}

int bie_solve_multi_device(bie_ctx *ctx, double k_re, double k_im, int64_t nrhs, const double *d_B, double *d_X,
                           const bie_multisolve_opts *opts, bie_multisolve_info *info) {
    return guarded([&] {
        bie::Ctx &c = *as_ctx(ctx);
        std::lock_guard<std::mutex> lock(c.mu);
        if (!std::isfinite(k_re) || !std::isfinite(k_im)) bie::fail(BIE_ERR_INVALID, "k must be finite");
        if (nrhs < 1 || nrhs > 65535) bie::fail(BIE_ERR_INVALID, "nrhs must be in 1..65535");
        if (!d_B || !d_X) bie::fail(BIE_ERR_INVALID, "B and X must not be NULL");
        BIE_CUDA(cudaSetDevice(c.device));
        bie_multisolve_opts o{};
        if (opts) o = *opts;
        bie_multisolve_info inf{};
        bie::run_solve_multi(c, k_re, k_im, nrhs, d_B, d_X, o, inf);
        if (info) *info = inf;
    });
}

int bie_solve_multi(bie_ctx *ctx, double k_re, double k_im, int64_t nrhs, const double *B, double *X,
                    const bie_multisolve_opts *opts, bie_multisolve_info *info) {
    return guarded([&] {
        bie::Ctx &c = *as_ctx(ctx);
        if (nrhs < 1 || nrhs > 65535) bie::fail(BIE_ERR_INVALID, "nrhs must be in 1..65535");
        if (!B || !X) bie::fail(BIE_ERR_INVALID, "B and X must not be NULL");
        const size_t bytes = (size_t)c.n_sources * (size_t)nrhs * 16;
        char *d = nullptr;
        {
            std::lock_guard<std::mutex> lock(c.mu);
            BIE_CUDA(cudaSetDevice(c.device));
            BIE_CUDA(cudaMalloc(&d, 2 * bytes));
        }
        struct Free {
            void *p;
            ~Free() { cudaFree(p); }
        } guard{d};
        double *dB = reinterpret_cast<double *>(d), *dX = reinterpret_cast<double *>(d + bytes);
        BIE_CUDA(cudaMemcpy(dB, B, bytes, cudaMemcpyHostToDevice));
        const int st = bie_solve_multi_device(ctx, k_re, k_im, nrhs, dB, dX, opts, info);
        if (st != BIE_OK) bie::fail(st, bie_last_error());
        BIE_CUDA(cudaMemcpy(X, dX, bytes, cudaMemcpyDeviceToHost));
    });
}

int bie_ctx_set_gemm_wait(bie_ctx *ctx, int64_t cycles, int stall) {
    return guarded([&] {
        bie::Ctx &c = *as_ctx(ctx);
        std::lock_guard<std::mutex> lock(c.mu);
        c.gemm_wait_cycles = cycles < 0 ? -1 : cycles;
        c.gemm_stall = stall != 0;
    });
}

int bie_singular_rule(int node, double offset, double *u, double *v, double *w, int capacity,
                      int *count) {
    return guarded([&] {
        if (!count) bie::fail(BIE_ERR_INVALID, "count must not be NULL");
        if (!(offset >= 0.0) || offset > 1.0) bie::fail(BIE_ERR_INVALID, "offset must be in [0, 1]");
        const bie::Rule r = bie::singular_rule(node, offset);
        *count = r.size();
        if (r.size() > capacity) bie::fail(BIE_ERR_INVALID, "capacity too small for the rule");
        if (!u || !v || !w) bie::fail(BIE_ERR_INVALID, "u, v, w must not be NULL");
        std::copy(r.u.begin(), r.u.end(), u);
        std::copy(r.v.begin(), r.v.end(), v);
        std::copy(r.w.begin(), r.w.end(), w);
    });
}

int bie_nearfield_pattern(bie_ctx *ctx, int depth, int64_t *nnz, int64_t *row_ptr, int64_t *cols) {
    return guarded([&] {
        bie::Ctx &c = *as_ctx(ctx);
        if (!nnz) bie::fail(BIE_ERR_INVALID, "nnz must not be NULL");
        std::lock_guard<std::mutex> lock(c.mu);
        BIE_CUDA(cudaSetDevice(c.device));
        const bie::NearField &nf = bie::get_nearfield(c, depth, 0.0, 3);
        *nnz = (int64_t)nf.cols.size();
        if (row_ptr) std::copy(nf.row_ptr.begin(), nf.row_ptr.end(), row_ptr);
        if (cols)
            for (size_t j = 0; j < nf.cols.size(); ++j) cols[j] = nf.cols[j];
    });
}

int bie_nearfield_assemble(bie_ctx *ctx, double k_re, double k_im, int depth, double offset,
                           int flags, int coarse, int n_gauss, double *F, double *G) {
    return guarded([&] {
        bie::Ctx &c = *as_ctx(ctx);
        if (!std::isfinite(k_re) || !std::isfinite(k_im)) bie::fail(BIE_ERR_INVALID, "k must be finite");
        if (flags & ~(BIE_F | BIE_G)) bie::fail(BIE_ERR_INVALID, "flags: only BIE_F | BIE_G");
        if ((flags & BIE_F) && !F) bie::fail(BIE_ERR_INVALID, "F requested but NULL");
        if ((flags & BIE_G) && !G) bie::fail(BIE_ERR_INVALID, "G requested but NULL");
        if (coarse) bie::triangle_gauss_rule(n_gauss);   // validates n_gauss
        std::lock_guard<std::mutex> lock(c.mu);
        BIE_CUDA(cudaSetDevice(c.device));
        const double off = offset < 0 ? 0.0 : offset;
        const bie::NearField &nf = bie::get_nearfield(c, depth, off, coarse ? n_gauss : 3);
        const size_t bytes = nf.cols.size() * 16;
        double *dF = (flags & BIE_F) ? static_cast<double *>(c.scratch(bie::kScratchF, bytes)) : nullptr;
        double *dG = (flags & BIE_G) ? static_cast<double *>(c.scratch(bie::kScratchG, bytes)) : nullptr;
        if (dF) BIE_CUDA(cudaMemsetAsync(dF, 0, bytes, c.stream));
        if (dG) BIE_CUDA(cudaMemsetAsync(dG, 0, bytes, c.stream));
        bie::launch_nearfield(c, nf, k_re, k_im, flags, coarse != 0, 1.0, dF, dG);
        if (dF) BIE_CUDA(cudaMemcpyAsync(F, dF, bytes, cudaMemcpyDeviceToHost, c.stream));
        if (dG) BIE_CUDA(cudaMemcpyAsync(G, dG, bytes, cudaMemcpyDeviceToHost, c.stream));
        BIE_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int bie_fastop_create(bie_ctx *ctx, double k_re, double k_im, int which, int n_gauss, int nearfield,
                      double offset, int depth, bie_fastop **out) {
    return guarded([&] {
        bie::Ctx &c = *as_ctx(ctx);
        if (!out) bie::fail(BIE_ERR_INVALID, "out must not be NULL");
        *out = nullptr;
        if (!std::isfinite(k_re) || !std::isfinite(k_im)) bie::fail(BIE_ERR_INVALID, "k must be finite");
        if (which != BIE_F && which != BIE_G) bie::fail(BIE_ERR_INVALID, "which must be BIE_F or BIE_G");
        if (depth != 1 && depth != 2) bie::fail(BIE_ERR_INVALID, "depth must be 1 or 2");
        if (!(offset >= 0.0) || offset > 1.0) bie::fail(BIE_ERR_INVALID, "offset must be in [0, 1]");
        std::lock_guard<std::mutex> lock(c.mu);
        BIE_CUDA(cudaSetDevice(c.device));
        auto op = bie::create_fastop(c, k_re, k_im, which, n_gauss, nearfield != 0, offset, depth);
        *out = reinterpret_cast<bie_fastop *>(op.release());
    });
}

int bie_fastop_destroy(bie_fastop *op) {
    return guarded([&] {
        if (!op) return;
        auto *f = reinterpret_cast<bie::FastOp *>(op);
        std::lock_guard<std::mutex> lock(f->base->mu);
        BIE_CUDA(cudaSetDevice(f->base->device));
        BIE_CUDA(cudaStreamSynchronize(f->base->stream));
        delete f;
    });
}

int bie_fastop_apply_device(bie_fastop *op, const double *d_x, double *d_y, int precision) {
    return guarded([&] {
        bie::FastOp &f = as_fastop(op);
        if (!d_x || !d_y) bie::fail(BIE_ERR_INVALID, "x and y must not be NULL");
        check_prec2(precision);
        std::lock_guard<std::mutex> lock(f.base->mu);
        BIE_CUDA(cudaSetDevice(f.base->device));
        bie::apply_fastop(f, d_x, d_y, precision, nullptr, 0);
    });
}

int bie_fastop_apply(bie_fastop *op, const double *x, double *y, int precision) {
    return guarded([&] {
        bie::FastOp &f = as_fastop(op);
        if (!x || !y) bie::fail(BIE_ERR_INVALID, "x and y must not be NULL");
        check_prec2(precision);
        std::lock_guard<std::mutex> lock(f.base->mu);
        bie::Ctx &c = *f.base;
        BIE_CUDA(cudaSetDevice(c.device));
        const int64_t N = c.n_sources;
        double *d = static_cast<double *>(c.scratch(bie::kScratchTargets, (size_t)N * 32 + 64));
        BIE_CUDA(cudaMemcpyAsync(d, x, (size_t)N * 16, cudaMemcpyHostToDevice, c.stream));
        bie::apply_fastop(f, d, d + 2 * N, precision, nullptr, 0);
        BIE_CUDA(cudaMemcpyAsync(y, d + 2 * N, (size_t)N * 16, cudaMemcpyDeviceToHost, c.stream));
        BIE_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int bie_fastop_evaluate_targets(bie_fastop *op, const double *targets, int64_t n_targets, const double *x,
                                double *y, int precision) {
    return guarded([&] {
        bie::FastOp &f = as_fastop(op);
        if (!targets || !x || !y) bie::fail(BIE_ERR_INVALID, "targets, x and y must not be NULL");
        if (n_targets <= 0) bie::fail(BIE_ERR_INVALID, "n_targets must be positive");
        check_prec2(precision);
        for (int64_t i = 0; i < 3 * n_targets; ++i)
            if (!std::isfinite(targets[i])) bie::fail(BIE_ERR_INVALID, "non-finite target");
        std::lock_guard<std::mutex> lock(f.base->mu);
        bie::Ctx &c = *f.base;
        BIE_CUDA(cudaSetDevice(c.device));
        const int64_t N = c.n_sources, M = n_targets;
        const size_t tb = ((size_t)M * 24 + 15) & ~size_t(15);
        char *buf = static_cast<char *>(c.scratch(bie::kScratchTargets, tb + (size_t)N * 16 + (size_t)M * 16 + 64));
        double *dt = reinterpret_cast<double *>(buf);
        double *dx = reinterpret_cast<double *>(buf + tb);
        double *dy = dx + 2 * N;
        BIE_CUDA(cudaMemcpyAsync(dt, targets, (size_t)M * 24, cudaMemcpyHostToDevice, c.stream));
        BIE_CUDA(cudaMemcpyAsync(dx, x, (size_t)N * 16, cudaMemcpyHostToDevice, c.stream));
        bie::apply_fastop(f, dx, dy, precision, dt, M);
        BIE_CUDA(cudaMemcpyAsync(y, dy, (size_t)M * 16, cudaMemcpyDeviceToHost, c.stream));
        BIE_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int bie_gmres_device(bie_ctx *ctx, const bie_operator *op, const double *d_b, double *d_x,
                     const bie_gmres_opts *opts, bie_gmres_info *info) {
    int converged = 1;
    const int st = guarded([&] {
        bie::Ctx &c = *as_ctx(ctx);
        if (!op || !d_b || !d_x) bie::fail(BIE_ERR_INVALID, "op, b and x must not be NULL");
        if (op->kind != BIE_OP_DENSE && op->kind != BIE_OP_MATRIX_FREE && op->kind != BIE_OP_FAST)
            bie::fail(BIE_ERR_INVALID, "unknown operator kind");
        if (op->kind == BIE_OP_DENSE && !op->A) bie::fail(BIE_ERR_INVALID, "dense operator without A");
        if (op->kind == BIE_OP_FAST &&
            (!op->fast || reinterpret_cast<const bie::FastOp *>(op->fast)->base != &c))
            bie::fail(BIE_ERR_INVALID, "fast operator missing or made from another context");
        if (!std::isfinite(op->k_re) || !std::isfinite(op->k_im) || !std::isfinite(op->scale_re) ||
            !std::isfinite(op->scale_im))
            bie::fail(BIE_ERR_INVALID, "k and scale must be finite");
        bie_gmres_opts o{};
        if (opts) o = *opts;
        if (o.precision != BIE_PREC_FP64 && o.precision != BIE_PREC_MIXED && o.precision != BIE_PREC_DF64)
            bie::fail(BIE_ERR_INVALID, "unknown precision");
        if (!(o.reltol >= 0) || !(o.abstol >= 0)) bie::fail(BIE_ERR_INVALID, "tolerances must be >= 0");
        std::lock_guard<std::mutex> lock(c.mu);
        BIE_CUDA(cudaSetDevice(c.device));
        bie_gmres_info inf{};
        bie::run_gmres(c, *op, d_b, d_x, o, inf);
        if (info) *info = inf;
        converged = inf.converged;
    });
    if (st == BIE_OK && !converged) {
        g_last_error = "GMRES reached maxiter before the tolerance";
        return BIE_ERR_NOT_CONVERGED;
    }
    return st;
}

int bie_gmres(bie_ctx *ctx, const bie_operator *op, const double *b, double *x, const bie_gmres_opts *opts,
              bie_gmres_info *info) {
    int converged = 1;
    const int st = guarded([&] {
        bie::Ctx &c = *as_ctx(ctx);
        if (!op || !b || !x) bie::fail(BIE_ERR_INVALID, "op, b and x must not be NULL");
        if (op->kind != BIE_OP_DENSE && op->kind != BIE_OP_MATRIX_FREE && op->kind != BIE_OP_FAST)
            bie::fail(BIE_ERR_INVALID, "unknown operator kind");
        if (op->kind == BIE_OP_DENSE && !op->A) bie::fail(BIE_ERR_INVALID, "dense operator without A");
        if (op->kind == BIE_OP_FAST &&
            (!op->fast || reinterpret_cast<const bie::FastOp *>(op->fast)->base != &c))
            bie::fail(BIE_ERR_INVALID, "fast operator missing or made from another context");
        if (!std::isfinite(op->k_re) || !std::isfinite(op->k_im) || !std::isfinite(op->scale_re) ||
            !std::isfinite(op->scale_im))
            bie::fail(BIE_ERR_INVALID, "k and scale must be finite");
        bie_gmres_opts o{};
        if (opts) o = *opts;
        if (o.precision != BIE_PREC_FP64 && o.precision != BIE_PREC_MIXED && o.precision != BIE_PREC_DF64)
            bie::fail(BIE_ERR_INVALID, "unknown precision");
        if (!(o.reltol >= 0) || !(o.abstol >= 0)) bie::fail(BIE_ERR_INVALID, "tolerances must be >= 0");
        // one device block: [A (16 N^2)] [A32 (8 N^2)] [diag (16 N)] b (16 N) x (16 N),
        // every part starting on a 256-byte boundary (8 N^2 is not a multiple
        // of 16 for odd N)
        const size_t N = (size_t)c.n_sources;
        const bool dense = op->kind == BIE_OP_DENSE;
        const bool low = dense && (op->A32 || o.refine || o.precision == BIE_PREC_MIXED);
        auto up = [](size_t b) { return (b + 255) & ~size_t(255); };
        const size_t a_bytes = dense ? 16 * N * N : 0, a32_bytes = low ? 8 * N * N : 0;
        const size_t d_bytes = op->diag ? 16 * N : 0, v_bytes = 16 * N;
        const size_t o_a32 = up(a_bytes), o_diag = o_a32 + up(a32_bytes), o_b = o_diag + up(d_bytes);
        const size_t o_x = o_b + up(v_bytes);
        std::lock_guard<std::mutex> lock(c.mu);
        BIE_CUDA(cudaSetDevice(c.device));
        char *d = nullptr;
        BIE_CUDA(cudaMalloc(&d, o_x + up(v_bytes)));
        struct Free {
            void *p;
            ~Free() { cudaFree(p); }
        } guard{d};
        double *dA = dense ? reinterpret_cast<double *>(d) : nullptr;
        float *dA32 = low ? reinterpret_cast<float *>(d + o_a32) : nullptr;
        double *ddiag = op->diag ? reinterpret_cast<double *>(d + o_diag) : nullptr;
        double *db = reinterpret_cast<double *>(d + o_b);
        double *dx = reinterpret_cast<double *>(d + o_x);
        if (dense) BIE_CUDA(cudaMemcpyAsync(dA, op->A, a_bytes, cudaMemcpyHostToDevice, c.stream));
        if (low) {
            if (op->A32)
                BIE_CUDA(cudaMemcpyAsync(dA32, op->A32, a32_bytes, cudaMemcpyHostToDevice, c.stream));
            else
                bie::round_to_c64(c, dA, dA32, (int64_t)(N * N));
        }
        if (ddiag) BIE_CUDA(cudaMemcpyAsync(ddiag, op->diag, d_bytes, cudaMemcpyHostToDevice, c.stream));
        BIE_CUDA(cudaMemcpyAsync(db, b, v_bytes, cudaMemcpyHostToDevice, c.stream));
        if (o.initially_nonzero)
            BIE_CUDA(cudaMemcpyAsync(dx, x, v_bytes, cudaMemcpyHostToDevice, c.stream));
        else
            BIE_CUDA(cudaMemsetAsync(dx, 0, v_bytes, c.stream));
        bie_operator dop = *op;
        dop.A = dA;
        dop.A32 = dA32;
        dop.diag = ddiag;
        bie_gmres_info inf{};
        bie::run_gmres(c, dop, db, dx, o, inf);
        BIE_CUDA(cudaMemcpyAsync(x, dx, v_bytes, cudaMemcpyDeviceToHost, c.stream));
        BIE_CUDA(cudaStreamSynchronize(c.stream));
        if (info) *info = inf;
        converged = inf.converged;
    });
    if (st == BIE_OK && !converged) {
        g_last_error = "GMRES reached maxiter before the tolerance";
        return BIE_ERR_NOT_CONVERGED;
    }
    return st;
}

int bie_sweep(bie_ctx *const *ctxs, int nmesh, const double *ks, int nk, const double *const *w,
              double *const *p, const bie_sweep_opts *opts, bie_sweep_info *info, int32_t *iters) {
    return guarded([&] {
        if (!ctxs || nmesh <= 0 || !ks || nk <= 0 || !w || !p)
            bie::fail(BIE_ERR_INVALID, "ctxs, ks, w, p must be given with positive counts");
        std::vector<bie::Ctx *> cs(nmesh);
        for (int m = 0; m < nmesh; ++m) {
            cs[m] = as_ctx(ctxs[m]);
            if (!w[m] || !p[m]) bie::fail(BIE_ERR_INVALID, "w[m] and p[m] must not be NULL");
        }
        for (int j = 0; j < 2 * nk; ++j)
            if (!std::isfinite(ks[j])) bie::fail(BIE_ERR_INVALID, "wavenumbers must be finite");
        bie_sweep_opts o{};
        o.precision = BIE_PREC_MIXED;
        o.refine = 1;
        if (opts) o = *opts;
        if (o.precision != BIE_PREC_FP64 && o.precision != BIE_PREC_MIXED && o.precision != BIE_PREC_DF64)
            bie::fail(BIE_ERR_INVALID, "unknown precision");
        bie_sweep_info inf{};
        bie::run_sweep(cs.data(), nmesh, ks, nk, w, p, o, inf, iters);
        if (info) *info = inf;
    });
}

int bie_adjoint(bie_ctx *ctx, double k_re, double k_im, const double *Z, const double *field,
                int64_t n_field, const bie_adjoint_opts *opts, double *J, double *pf, double *dX,
                double *dZ, bie_adjoint_info *info) {
    return guarded([&] {
        bie::Ctx &c = *as_ctx(ctx);
        if (!Z || !field || n_field <= 0 || !opts || !J)
            bie::fail(BIE_ERR_INVALID, "Z, field, opts and J must be given (n_field > 0)");
        if (!std::isfinite(k_re) || !std::isfinite(k_im) || !(opts->rho_c > 0))
            bie::fail(BIE_ERR_INVALID, "k must be finite and rho_c positive");
        const double dn = std::sqrt(opts->dir[0] * opts->dir[0] + opts->dir[1] * opts->dir[1] +
                                    opts->dir[2] * opts->dir[2]);
        if (!(std::fabs(dn - 1.0) < 1e-12)) bie::fail(BIE_ERR_INVALID, "dir must be a unit vector");
        for (int64_t e = 0; e < 2 * c.n_elements; e += 2)
            if (!std::isfinite(Z[e]) || !std::isfinite(Z[e + 1]) || (Z[e] == 0 && Z[e + 1] == 0))
                bie::fail(BIE_ERR_INVALID, "impedances must be finite and non-zero");
        for (int64_t i = 0; i < 3 * n_field; ++i)
            if (!std::isfinite(field[i])) bie::fail(BIE_ERR_INVALID, "non-finite field point");
        std::lock_guard<std::mutex> lock(c.mu);
        BIE_CUDA(cudaSetDevice(c.device));
        bie::AdjointArgs a{k_re, k_im, opts->rho_c, Z, {opts->dir[0], opts->dir[1], opts->dir[2]},
                           field, n_field, opts->reltol, pf, dX, dZ};
        if (opts->precision != BIE_PREC_FP64 && opts->precision != BIE_PREC_DF64)
            bie::fail(BIE_ERR_INVALID, "adjoint precision must be BIE_PREC_FP64 or BIE_PREC_DF64");
        a.precision = opts->precision;
        bie::AdjointOut o;
        bie::run_adjoint(c, a, o);
        *J = o.J;
        if (info) {
            info->forward_iterations = o.forward_iterations;
            info->forward_converged = o.forward_converged;
            info->adjoint_iterations = o.adjoint_iterations;
            info->adjoint_converged = o.adjoint_converged;
        }
    });
}

int bie_round_c64_device(bie_ctx *ctx, const double *d_in, float *d_out, int64_t n) {
    return guarded([&] {
        bie::Ctx &c = *as_ctx(ctx);
        if (!d_in || !d_out || n < 0) bie::fail(BIE_ERR_INVALID, "bad arguments");
        std::lock_guard<std::mutex> lock(c.mu);
        BIE_CUDA(cudaSetDevice(c.device));
        if (n > 0) bie::round_to_c64(c, d_in, d_out, n);
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

// ---- mesh input ------------------------------------------------------------------
int bie_read_comsol(const char *path, int64_t *n_coordinates, int64_t *n_elements, int32_t *nodes_per_element,
                    int64_t *n_entities, double *coordinates, int64_t *topology, int64_t *entities) {
    return guarded([&] {
        if (!path || !n_coordinates || !n_elements || !nodes_per_element || !n_entities)
            bie::fail(BIE_ERR_INVALID, "path and the size outputs must not be NULL");
        std::vector<double> co;
        std::vector<int64_t> to, en;
        int npe = 0;
        bie::read_comsol(path, co, to, npe, en);
        *n_coordinates = (int64_t)co.size() / 3;
        *nodes_per_element = npe;
        *n_elements = (int64_t)to.size() / npe;
        *n_entities = (int64_t)en.size();
        if (!coordinates) return;
        if (!topology) bie::fail(BIE_ERR_INVALID, "topology must not be NULL");
        std::copy(co.begin(), co.end(), coordinates);
        std::copy(to.begin(), to.end(), topology);
        if (entities) std::copy(en.begin(), en.end(), entities);
    });
}

// ---- visco-thermal system ----------------------------------------------------
int bie_ambient_to_properties(double f, double ps, double t, double H, double out[10]) {
    return guarded([&] {
        if (!out) bie::fail(BIE_ERR_INVALID, "out must not be NULL");
        if (!std::isfinite(f) || !std::isfinite(ps) || !std::isfinite(t) || !std::isfinite(H) || !(ps > 0) ||
            !(t > -273.15) || H < 0)
            bie::fail(BIE_ERR_INVALID, "need finite f, ps > 0, t > -273.15 C, H >= 0");
        bie::ambient_to_properties(f, ps, t, H, out);
    });
}

int bie_visco_thermal_constants(double freq, double S, double pa, double t, double Hr, bie_lossy_constants *out) {
    return guarded([&] {
        if (!out) bie::fail(BIE_ERR_INVALID, "out must not be NULL");
        if (!(freq > 0) || !std::isfinite(freq) || !std::isfinite(S) || S == 0.0)
            bie::fail(BIE_ERR_INVALID, "need freq > 0 and a nonzero finite S");
        if (!std::isfinite(pa) || !(pa > 0) || !std::isfinite(t) || !(t > -273.15) || !std::isfinite(Hr) || Hr < 0)
            bie::fail(BIE_ERR_INVALID, "need pa > 0, t > -273.15 C, Hr >= 0");
        *out = bie::visco_thermal_constants(freq, S, pa, t, Hr);
    });
}

int bie_tangential_derivatives(const bie_mesh_desc *d, int64_t *nnz, int64_t *row_ptr, int64_t *cols, double *Dx,
                               double *Dy, double *Dz) {
    return guarded([&] {
        if (!d || !nnz) bie::fail(BIE_ERR_INVALID, "mesh and nnz must not be NULL");
        if (d->n_coordinates <= 0 || d->n_elements <= 0 || d->n_sources <= 0 || !d->coordinates || !d->topology ||
            !d->physics_topology)
            bie::fail(BIE_ERR_INVALID, "mesh sizes must be positive and its arrays given");
        if (d->n_coordinates > INT32_MAX || d->n_sources > INT32_MAX || d->n_elements > INT32_MAX)
            bie::fail(BIE_ERR_INVALID, "mesh too large for 32-bit node indices");
        const int NS = bie::n_nodes_of_kind(d->shape_kind), NP = bie::n_nodes_of_kind(d->physics_kind);
        const int64_t E = d->n_elements, N = d->n_sources;
        std::vector<int32_t> topo((size_t)NS * E), ptopo((size_t)NP * E);
        for (int64_t i = 0; i < NS * E; ++i) {
            const int64_t v = d->topology[i];
            if (v < 1 || v > d->n_coordinates) bie::fail(BIE_ERR_INVALID, "topology index out of range");
            topo[(size_t)i] = (int32_t)(v - 1);
        }
        for (int64_t i = 0; i < NP * E; ++i) {
            const int64_t v = d->physics_topology[i];
            if (v < 1 || v > N) bie::fail(BIE_ERR_INVALID, "physics_topology index out of range");
            ptopo[(size_t)i] = (int32_t)(v - 1);
        }
        for (int64_t i = 0; i < 3 * d->n_coordinates; ++i)
            if (!std::isfinite(d->coordinates[i])) bie::fail(BIE_ERR_INVALID, "non-finite coordinate");
        std::vector<int64_t> rp;
        std::vector<int32_t> cl;
        std::vector<double> dx, dy, dz;
        bie::tangential_derivatives(d->shape_kind, d->physics_kind, d->coordinates, E, topo.data(), ptopo.data(), N,
                                    rp, cl, dx, dy, dz);
        *nnz = (int64_t)cl.size();
        if (!row_ptr) return;
        if (!cols || !Dx || !Dy || !Dz) bie::fail(BIE_ERR_INVALID, "cols, Dx, Dy, Dz must not be NULL");
        std::copy(rp.begin(), rp.end(), row_ptr);
        std::copy(cl.begin(), cl.end(), cols);
        std::copy(dx.begin(), dx.end(), Dx);
        std::copy(dy.begin(), dy.end(), Dy);
        std::copy(dz.begin(), dz.end(), Dz);
    });
}

int bie_element_slicing(const bie_mesh_desc *d, int level, int32_t *order, int64_t *counts, uint32_t *flags,
                        int32_t *slots) {
    return guarded([&] {
        if (!d) bie::fail(BIE_ERR_INVALID, "mesh must not be NULL");
        if (d->n_coordinates <= 0 || d->n_elements <= 0 || d->n_sources <= 0 || !d->coordinates || !d->topology ||
            !d->physics_topology)
            bie::fail(BIE_ERR_INVALID, "mesh sizes must be positive and its arrays given");
        if (d->n_coordinates > INT32_MAX || d->n_sources > INT32_MAX || d->n_elements > INT32_MAX)
            bie::fail(BIE_ERR_INVALID, "mesh too large for 32-bit node indices");
        if (d->shape_kind != BIE_TRI_LINEAR && d->shape_kind != BIE_TRI_QUADRATIC)
            bie::fail(BIE_ERR_UNSUPPORTED, "geometry must be 3- or 6-node triangles");
        if (level < 0 || level >= bie::kMaxLevels)
            bie::fail(BIE_ERR_INVALID, "level must be in 0.." + std::to_string(bie::kMaxLevels - 1));
        const int NS = bie::n_nodes_of_kind(d->shape_kind), NP = bie::n_nodes_of_kind(d->physics_kind);
        const int64_t E = d->n_elements, N = d->n_sources;
        std::vector<int32_t> topo((size_t)NS * E), ptopo((size_t)NP * E);
        for (int64_t i = 0; i < NS * E; ++i) {
            const int64_t v = d->topology[i];
            if (v < 1 || v > d->n_coordinates) bie::fail(BIE_ERR_INVALID, "topology index out of range");
            topo[(size_t)i] = (int32_t)(v - 1);
        }
        for (int64_t i = 0; i < NP * E; ++i) {
            const int64_t v = d->physics_topology[i];
            if (v < 1 || v > N) bie::fail(BIE_ERR_INVALID, "physics_topology index out of range");
            ptopo[(size_t)i] = (int32_t)(v - 1);
        }
        for (int64_t i = 0; i < 3 * d->n_coordinates; ++i)
            if (!std::isfinite(d->coordinates[i])) bie::fail(BIE_ERR_INVALID, "non-finite coordinate");
        const std::vector<int32_t> ord = bie::bisection_order(d->coordinates, d->n_coordinates, topo.data(), NS, E);
        if (order)
            for (int64_t p = 0; p < E; ++p) order[p] = ord[(size_t)p] + 1;
        if (counts || flags || slots) {
            bie::WriteProtocol w;
            bie::build_write_protocol(ord.data(), E, ptopo.data(), NP, N, w);
            if (counts) {
                counts[0] = w.nshared[level];
                counts[1] = w.nside[level];
                counts[2] = w.nring[level];
                counts[3] = w.nwiden[level];
                counts[4] = w.nsingle[level];
                counts[5] = w.nuntouched[level];
            }
            if (flags) std::copy_n(w.k2_flags.begin() + (size_t)level * E, E, flags);
            if (slots) std::copy_n(w.k2_side.begin() + (size_t)level * E * NP, E * NP, slots);
        }
    });
}

int bie_lossy_create(bie_ctx *ctx, double freq, const bie_lossy_opts *opts, bie_lossy **out) {
    return guarded([&] {
        bie::Ctx &c = *as_ctx(ctx);
        if (!opts || !out) bie::fail(BIE_ERR_INVALID, "opts and out must not be NULL");
        *out = nullptr;
        const bie_lossy_opts &o = *opts;
        if (!(freq > 0) || !std::isfinite(freq)) bie::fail(BIE_ERR_INVALID, "freq must be positive");
        if (!o.normals) bie::fail(BIE_ERR_INVALID, "normals (3 x N) must be given");
        if (!std::isfinite(o.S)) bie::fail(BIE_ERR_INVALID, "S must be finite");
        if (o.custom_air && (!(o.pa > 0) || !std::isfinite(o.pa) || !(o.t > -273.15) || !std::isfinite(o.t) ||
                             !(o.Hr >= 0) || !std::isfinite(o.Hr)))
            bie::fail(BIE_ERR_INVALID, "need pa > 0, t > -273.15 C, Hr >= 0");
        if (o.depth != 0 && o.depth != 1 && o.depth != 2) bie::fail(BIE_ERR_INVALID, "depth must be 1 or 2");
        if (o.fmm_on && o.fmm_offset > 1.0) bie::fail(BIE_ERR_INVALID, "fmm_offset must be <= 1");
        check_solve_opts(o.solve);
        for (int64_t i = 0; i < 3 * c.n_sources; ++i)
            if (!std::isfinite(o.normals[i])) bie::fail(BIE_ERR_INVALID, "non-finite normal");
        std::lock_guard<std::mutex> lock(c.mu);
        BIE_CUDA(cudaSetDevice(c.device));
        *out = reinterpret_cast<bie_lossy *>(bie::create_lossy(c, freq, o));
    });
}

int bie_lossy_destroy(bie_lossy *L) {
    return guarded([&] {
        if (!L) return;
        bie::LossyOp *p = reinterpret_cast<bie::LossyOp *>(L);
        bie::Ctx &c = bie::lossy_context(*p);
        std::lock_guard<std::mutex> lock(c.mu);
        BIE_CUDA(cudaSetDevice(c.device));
        BIE_CUDA(cudaStreamSynchronize(c.stream));
        bie::destroy_lossy(p);
    });
}

int bie_lossy_constants_of(const bie_lossy *L, bie_lossy_constants *out) {
    return guarded([&] {
        if (!out) bie::fail(BIE_ERR_INVALID, "out must not be NULL");
        *out = bie::lossy_constants(as_lossy(const_cast<bie_lossy *>(L)));
    });
}

int bie_lossy_apply_device(bie_lossy *L, int block, const double *d_x, double *d_y) {
    return guarded([&] {
        bie::LossyOp &op = as_lossy(L);
        check_block(block);
        if (!d_x || !d_y) bie::fail(BIE_ERR_INVALID, "x and y must not be NULL");
        if (d_x == d_y) bie::fail(BIE_ERR_INVALID, "x and y must not alias");
        bie::Ctx &c = bie::lossy_context(op);
        std::lock_guard<std::mutex> lock(c.mu);
        BIE_CUDA(cudaSetDevice(c.device));
        bie::lossy_apply(op, block, d_x, d_y);
    });
}

int bie_lossy_solve_device(bie_lossy *L, int block, const double *d_b, double *d_x, const bie_gmres_opts *opts,
                           bie_gmres_info *info) {
    int converged = 1;
    const int st = guarded([&] {
        bie::LossyOp &op = as_lossy(L);
        check_block(block);
        if (!d_b || !d_x) bie::fail(BIE_ERR_INVALID, "b and x must not be NULL");
        if (d_b == d_x) bie::fail(BIE_ERR_INVALID, "b and x must not alias");
        bie_gmres_opts o{};
        if (opts) o = *opts;
        check_solve_opts(o);
        bie::Ctx &c = bie::lossy_context(op);
        std::lock_guard<std::mutex> lock(c.mu);
        BIE_CUDA(cudaSetDevice(c.device));
        bie_gmres_info inf{};
        bie::lossy_solve(op, block, d_b, d_x, o, inf);
        if (info) *info = inf;
        converged = inf.converged;
    });
    if (st == BIE_OK && !converged) {
        g_last_error = "GMRES reached maxiter before the tolerance";
        return BIE_ERR_NOT_CONVERGED;
    }
    return st;
}

int bie_lossy_apply(bie_lossy *L, int block, const double *x, double *y) {
    return guarded([&] {
        bie::LossyOp &op = as_lossy(L);
        check_block(block);
        if (!x || !y) bie::fail(BIE_ERR_INVALID, "x and y must not be NULL");
        bie::Ctx &c = bie::lossy_context(op);
        std::lock_guard<std::mutex> lock(c.mu);
        BIE_CUDA(cudaSetDevice(c.device));
        const int64_t N = c.n_sources;
        const int64_t ni = bie::lossy_block_len(block, true, N), no = bie::lossy_block_len(block, false, N);
        double *d = static_cast<double *>(c.scratch(bie::kScratchTargets, (size_t)(ni + no) * 16));
        BIE_CUDA(cudaMemcpyAsync(d, x, (size_t)ni * 16, cudaMemcpyHostToDevice, c.stream));
        bie::lossy_apply(op, block, d, d + 2 * ni);
        BIE_CUDA(cudaMemcpyAsync(y, d + 2 * ni, (size_t)no * 16, cudaMemcpyDeviceToHost, c.stream));
        BIE_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int bie_lossy_solve(bie_lossy *L, int block, const double *b, double *x, const bie_gmres_opts *opts,
                    bie_gmres_info *info) {
    int converged = 1;
    const int st = guarded([&] {
        bie::LossyOp &op = as_lossy(L);
        check_block(block);
        if (!b || !x) bie::fail(BIE_ERR_INVALID, "b and x must not be NULL");
        bie_gmres_opts o{};
        if (opts) o = *opts;
        check_solve_opts(o);
        bie::Ctx &c = bie::lossy_context(op);
        std::lock_guard<std::mutex> lock(c.mu);
        BIE_CUDA(cudaSetDevice(c.device));
        const int64_t n = bie::lossy_block_len(block, true, c.n_sources);
        double *d = static_cast<double *>(c.scratch(bie::kScratchTargets, (size_t)n * 32));
        BIE_CUDA(cudaMemcpyAsync(d, b, (size_t)n * 16, cudaMemcpyHostToDevice, c.stream));
        bie_gmres_info inf{};
        bie::lossy_solve(op, block, d, d + 2 * n, o, inf);
        BIE_CUDA(cudaMemcpyAsync(x, d + 2 * n, (size_t)n * 16, cudaMemcpyDeviceToHost, c.stream));
        BIE_CUDA(cudaStreamSynchronize(c.stream));
        if (info) *info = inf;
        converged = inf.converged;
    });
    if (st == BIE_OK && !converged) {
        g_last_error = "GMRES reached maxiter before the tolerance";
        return BIE_ERR_NOT_CONVERGED;
    }
    return st;
}

int bie_lossy_stats(bie_lossy *L, int64_t *nested_solves, int64_t *nested_iterations, int reset) {
    return guarded([&] {
        bie::LossyOp &op = as_lossy(L);
        bie::Ctx &c = bie::lossy_context(op);
        std::lock_guard<std::mutex> lock(c.mu);
        bie::lossy_stats(op, nested_solves, nested_iterations, reset != 0);
    });
}

int bie_lossy_set_one_launch(bie_lossy *L, int mode) {
    return guarded([&] {
        bie::LossyOp &op = as_lossy(L);
        std::lock_guard<std::mutex> lock(bie::lossy_context(op).mu);
        bie::lossy_set_one_launch(op, mode);
    });
}

}  // extern "C"
