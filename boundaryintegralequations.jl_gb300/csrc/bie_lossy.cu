// K8: the visco-thermal ("lossy") system resident on the device
// (LossyGlobalOuter / LossyGlobalInner of src/3d/LossyGlobalMatrix.jl).
//
// Construction (LossyGlobalMatrix.jl:76-172):
//   constants   visco_thermal_constants(freq, S) (bie_lossy.cpp)
//   acoustic    Ha = F(ka) + Diagonal(C), Ga = G(ka): dense complex128 from the
//               FP64 assembly (fmm_on = false; interior: -F + Diagonal(1 - C)),
//               or the fast operators (fmm_on = true, Ha = F_fast + I / 2)
//   thermal     Hh = F(kh) + C0, Gh = G(kh): near-field CSR of the adaptive
//               near-field rules (sparse_assemble_parallel!, depth, offset 0)
//   viscous     Av = F(kv) + C0, Bv = G(kv) the same way; Hv, Gv = blockdiag x 3
//   derivatives Dx, Dy, Dz (bie_lossy.cpp), Nd = -[diag nx; diag ny; diag nz]
// Product (LossyGlobalMatrix.jl:179-197, :26-37):
//   y = -phi_a Ha x + Ga (mu_h gmres(Gh, Hh x)
//                        + mu_a gmres(inner, Dr Dc x - Nd' gmres(Gv, Hv Dc x)))
//   inner z = Dr Nd z - Nd' gmres(Gv, Hv Nd z)
// Every gmres is this library's device GMRES (run_gmres_devop) with the
// reference's defaults; the solves nest two deep (a Gv solve inside the inner
// operator inside the outer product), each level on its own workspace.
// The sparse and derivative kernels are HBM/latency bound, one row per thread.
#include "bie_internal.h"

#include <algorithm>
#include <vector>

namespace bie {

namespace {

inline unsigned nblocks(int64_t n) { return (unsigned)((n + 255) / 256); }

// y = V x + d .* x   (V complex CSR; d optional)
__global__ void csr_apply_kernel(const int64_t *__restrict__ rp, const int32_t *__restrict__ cols,
                                 const double2 *__restrict__ v, const double2 *__restrict__ d,
                                 const double2 *__restrict__ x, double2 *__restrict__ y, int64_t n,
                                 const int *__restrict__ stop) {
    if (stop && *stop) return;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double re = 0.0, im = 0.0;
    for (int64_t p = rp[i]; p < rp[i + 1]; ++p) {
        const double2 a = v[p], b = x[cols[p]];
        re += a.x * b.x - a.y * b.y;
        im += a.x * b.y + a.y * b.x;
    }
    if (d) {
        const double2 a = d[i], b = x[i];
        re += a.x * b.x - a.y * b.y;
        im += a.x * b.y + a.y * b.x;
    }
    y[i] = make_double2(re, im);
}

// q_k = D_k x for k = x, y, z  (real CSR values on one pattern)
__global__ void dc_kernel(const int64_t *__restrict__ rp, const int32_t *__restrict__ cols,
                          const double *__restrict__ Dx, const double *__restrict__ Dy,
                          const double *__restrict__ Dz, const double2 *__restrict__ x, double2 *__restrict__ q,
                          int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double2 a = {0, 0}, b = {0, 0}, c = {0, 0};
    for (int64_t p = rp[i]; p < rp[i + 1]; ++p) {
        const double2 xv = x[cols[p]];
        a.x += Dx[p] * xv.x;
        a.y += Dx[p] * xv.y;
        b.x += Dy[p] * xv.x;
        b.y += Dy[p] * xv.y;
        c.x += Dz[p] * xv.x;
        c.y += Dz[p] * xv.y;
    }
    q[i] = a;
    q[n + i] = b;
    q[2 * n + i] = c;
}

// y = Dx q_0 + Dy q_1 + Dz q_2 + s (nx g_0 + ny g_1 + nz g_2)   (q, g optional).
// Since Nd' g = -(nx g_0 + ny g_1 + nz g_2): s = 1 gives Dr q - Nd' g, and
// q = null, s = -1 gives Nd' g.
__global__ void dr_ndt_kernel(const int64_t *__restrict__ rp, const int32_t *__restrict__ cols,
                              const double *__restrict__ Dx, const double *__restrict__ Dy,
                              const double *__restrict__ Dz, const double2 *__restrict__ q,
                              const double *__restrict__ nrm, const double2 *__restrict__ g, double s,
                              double2 *__restrict__ y, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double re = 0.0, im = 0.0;
    if (q) {
        for (int64_t p = rp[i]; p < rp[i + 1]; ++p) {
            const int64_t j = cols[p];
            const double2 a = q[j], b = q[n + j], c = q[2 * n + j];
            re += Dx[p] * a.x + Dy[p] * b.x + Dz[p] * c.x;
            im += Dx[p] * a.y + Dy[p] * b.y + Dz[p] * c.y;
        }
    }
    if (g) {
        const double nx = nrm[3 * i], ny = nrm[3 * i + 1], nz = nrm[3 * i + 2];
        const double2 a = g[i], b = g[n + i], c = g[2 * n + i];
        re += s * (nx * a.x + ny * b.x + nz * c.x);
        im += s * (nx * a.y + ny * b.y + nz * c.y);
    }
    y[i] = make_double2(re, im);
}

// p = Nd z = -[nx z; ny z; nz z]
__global__ void nd_kernel(const double *__restrict__ nrm, const double2 *__restrict__ z, double2 *__restrict__ p,
                          int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double2 v = z[i];
    for (int k = 0; k < 3; ++k) {
        const double c = -nrm[3 * i + k];
        p[k * n + i] = make_double2(c * v.x, c * v.y);
    }
}

// y = a y + b x  (complex a, b)
__global__ void axpby_kernel(double2 a, double2 *__restrict__ y, double2 b, const double2 *__restrict__ x,
                             int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double2 yv = y[i], xv = x[i];
    y[i] = make_double2(a.x * yv.x - a.y * yv.y + b.x * xv.x - b.y * xv.y,
                        a.x * yv.y + a.y * yv.x + b.x * xv.y + b.y * xv.x);
}

// v = s v (real s)
__global__ void scale_kernel(double2 *__restrict__ v, double s, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = make_double2(s * v[i].x, s * v[i].y);
}

// d = a + b c  (complex a, b; c may be null: d = a)
__global__ void diag_kernel(double2 a, double2 b, const double2 *__restrict__ c, double2 *__restrict__ d,
                            int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double2 v = a;
    if (c) {
        v.x += b.x * c[i].x - b.y * c[i].y;
        v.y += b.x * c[i].y + b.y * c[i].x;
    }
    d[i] = v;
}

template <class T>
T *dev_alloc(size_t count) {
    T *p = nullptr;
    BIE_CUDA(cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)));
    return p;
}

template <class T>
T *dev_upload(const std::vector<T> &h, cudaStream_t s) {
    T *p = dev_alloc<T>(h.size());
    if (!h.empty()) BIE_CUDA(cudaMemcpyAsync(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    return p;
}

inline double2 cx(const double *v) { return make_double2(v[0], v[1]); }

}  // namespace

struct LossyOp {
    Ctx *c = nullptr;
    int64_t N = 0;
    bie_lossy_constants k{};
    bool fmm = false;
    double sgn = 1.0;                 // +1 exterior, -1 interior (sign of the F blocks)
    bie_gmres_opts nested{};          // options of the nested gmres calls
    // acoustic
    double2 *Fa = nullptr, *Ga = nullptr;        // dense N x N (fmm_on = false)
    std::unique_ptr<FastOp> fa, ga;              // fast operators (fmm_on = true)
    double2 *C0 = nullptr;                       // integral-free terms (N)
    // thermal / viscous near field
    int64_t *nf_rp = nullptr;
    int32_t *nf_cols = nullptr;
    double2 *Fh = nullptr, *Gh = nullptr, *Fv = nullptr, *Gv = nullptr;
    // derivatives
    int64_t *d_rp = nullptr;
    int32_t *d_cols = nullptr;
    double *Dx = nullptr, *Dy = nullptr, *Dz = nullptr;
    double *nrm = nullptr;                       // 3 x N
    // work vectors
    double2 *work = nullptr;
    double2 *o_t, *o_sh, *o_q, *o_hq, *o_sv, *o_r, *o_si, *o_w, *i_p, *i_hp, *i_g, *s_t;
    // solve nesting and statistics (host-counted solves, plus the one-launch
    // sparse solves counted on the device in d_acc = {solves, iterations})
    int active = -1;
    int64_t nested_solves = 0, nested_iterations = 0;
    int one_launch = 1;                 // sparse solves as one launch where they fit (0: off; 1: auto;
                                        // 2: cluster form only; 3: grid form only)
    unsigned long long *d_acc = nullptr;
    bie_gmres_info *d_info = nullptr;
    int *d_err = nullptr;               // set by a one-launch solve whose grid barrier gave up

    ~LossyOp() {
        cudaFree(Fa);
        cudaFree(Ga);
        cudaFree(C0);
        cudaFree(nf_rp);
        cudaFree(nf_cols);
        cudaFree(Fh);
        cudaFree(Gh);
        cudaFree(Fv);
        cudaFree(Gv);
        cudaFree(d_rp);
        cudaFree(d_cols);
        cudaFree(Dx);
        cudaFree(Dy);
        cudaFree(Dz);
        cudaFree(nrm);
        cudaFree(work);
        cudaFree(d_acc);
        cudaFree(d_info);
        cudaFree(d_err);
    }

    cudaStream_t stream() const { return c->stream; }
    void launched() { ++c->kernel_launches; }

    // ---- blocks --------------------------------------------------------------
    void Ha(const double2 *x, double2 *y) {
        if (fmm) {
            apply_fastop(*fa, reinterpret_cast<const double *>(x), reinterpret_cast<double *>(y), BIE_PREC_FP64,
                         nullptr, 0);
            axpby_kernel<<<nblocks(N), 256, 0, stream()>>>(make_double2(1, 0), y, make_double2(0.5, 0), x, N);
            BIE_CUDA(cudaGetLastError());
            launched();
        } else {
            bie_operator op{};
            op.kind = BIE_OP_DENSE;
            op.A = reinterpret_cast<const double *>(Fa);
            op.scale_re = sgn;
            op.diag = reinterpret_cast<const double *>(C0);
            apply_operator(*c, op, BIE_PREC_FP64, reinterpret_cast<const double *>(x), reinterpret_cast<double *>(y));
        }
    }
    void Ga_(const double2 *x, double2 *y) {
        if (fmm) {
            apply_fastop(*ga, reinterpret_cast<const double *>(x), reinterpret_cast<double *>(y), BIE_PREC_FP64,
                         nullptr, 0);
        } else {
            bie_operator op{};
            op.kind = BIE_OP_DENSE;
            op.A = reinterpret_cast<const double *>(Ga);
            op.scale_re = 1.0;
            apply_operator(*c, op, BIE_PREC_FP64, reinterpret_cast<const double *>(x), reinterpret_cast<double *>(y));
        }
    }
    // y = V x + d .* x on `nb` consecutive blocks of N
    void csr(const double2 *v, const double2 *d, const double2 *x, double2 *y, int nb, const int *stop = nullptr) {
        for (int b = 0; b < nb; ++b) {
            csr_apply_kernel<<<nblocks(N), 256, 0, stream()>>>(nf_rp, nf_cols, v, d, x + b * N, y + b * N, N, stop);
            BIE_CUDA(cudaGetLastError());
            launched();
        }
    }
    void Dc(const double2 *x, double2 *q) {
        dc_kernel<<<nblocks(N), 256, 0, stream()>>>(d_rp, d_cols, Dx, Dy, Dz, x, q, N);
        BIE_CUDA(cudaGetLastError());
        launched();
    }
    // y = Dr q - Nd' g  (q or g may be null)
    void Dr_minus_NdT(const double2 *q, const double2 *g, double2 *y) {
        dr_ndt_kernel<<<nblocks(N), 256, 0, stream()>>>(d_rp, d_cols, Dx, Dy, Dz, q, nrm, g, 1.0, y, N);
        BIE_CUDA(cudaGetLastError());
        launched();
    }
    void Nd(const double2 *z, double2 *p) {
        nd_kernel<<<nblocks(N), 256, 0, stream()>>>(nrm, z, p, N);
        BIE_CUDA(cudaGetLastError());
        launched();
    }

    void solve(DevOp &op, const double2 *b, double2 *x, const bie_gmres_opts &o, bie_gmres_info &info,
               bool count) {
        const int lvl = active + 1;
        if (lvl > kMaxSolveLevel) fail(BIE_ERR_INVALID, "lossy system: GMRES nested deeper than two levels");
        ++active;
        try {
            run_gmres_devop(*c, op, reinterpret_cast<const double *>(b), reinterpret_cast<double *>(x), o, info,
                            lvl);
        } catch (...) {
            --active;
            throw;
        }
        --active;
        if (count) {
            ++nested_solves;
            nested_iterations += info.iterations;
        }
    }

    // After a synchronisation: fail if a one-launch solve's barrier gave up
    // (the word is cleared, so the operator stays usable)
    void check_error() {
        int e = 0;
        BIE_CUDA(cudaMemcpyAsync(&e, d_err, sizeof(int), cudaMemcpyDeviceToHost, stream()));
        BIE_CUDA(cudaStreamSynchronize(stream()));
        if (e) {
            BIE_CUDA(cudaMemsetAsync(d_err, 0, sizeof(int), stream()));
            BIE_CUDA(cudaStreamSynchronize(stream()));
            fail(BIE_ERR_TIMEOUT, "lossy system: a one-launch GMRES barrier wait ran out");
        }
    }

    // gmres(V + Diagonal(d), b) on nb blocks of the near-field pattern: one
    // launch with the statistics kept on the device when it fits, else the
    // launch-per-operation GMRES
    void solve_csr(const double2 *v, const double2 *d, int nb, const double2 *b, double2 *x,
                   const bie_gmres_opts &o, bie_gmres_info &info, bool count);

    // inner z = Dr Nd z - Nd' gmres(Gv, Hv Nd z)
    void inner(const double2 *z, double2 *y);
    // the LossyGlobalOuter product
    void outer(const double2 *x, double2 *y);
};

namespace {

struct CsrOp : DevOp {
    LossyOp &L;
    const double2 *v, *d;
    int nb;
    CsrOp(LossyOp &l, const double2 *v_, const double2 *d_, int nb_) : L(l), v(v_), d(d_), nb(nb_) {}
    int64_t size() const override { return nb * L.N; }
    void apply(const double2 *x, double2 *y, const int *stop) override { L.csr(v, d, x, y, nb, stop); }
    bool honours_stop() const override { return true; }
};

struct BlockOp : DevOp {   // Ha, Ga, inner or outer
    LossyOp &L;
    int block;
    BlockOp(LossyOp &l, int b) : L(l), block(b) {}
    int64_t size() const override { return L.N; }
    void apply(const double2 *x, double2 *y, const int *) override {
        switch (block) {
        case BIE_LOSSY_HA: L.Ha(x, y); break;
        case BIE_LOSSY_GA: L.Ga_(x, y); break;
        case BIE_LOSSY_INNER: L.inner(x, y); break;
        default: L.outer(x, y); break;
        }
    }
};

}  // namespace

void LossyOp::solve_csr(const double2 *v, const double2 *d, int nb, const double2 *b, double2 *x,
                        const bie_gmres_opts &o, bie_gmres_info &info, bool count) {
    const int lvl = active + 1;
    if (lvl > kMaxSolveLevel) fail(BIE_ERR_INVALID, "lossy system: GMRES nested deeper than two levels");
    if (one_launch) {
        const CsrSystem A{nf_rp, nf_cols, v, d, N, nb};
        const int forms = one_launch == 2 ? kOneLaunchCluster : one_launch == 3 ? kOneLaunchGrid : kOneLaunchAuto;
        if (csr_gmres_one_launch(*c, A, b, x, o, lvl, count ? nullptr : d_info, count ? d_acc : nullptr, d_err,
                                 forms)) {
            if (!count) {
                BIE_CUDA(cudaMemcpyAsync(&info, d_info, sizeof(info), cudaMemcpyDeviceToHost, stream()));
                BIE_CUDA(cudaStreamSynchronize(stream()));
                check_error();
            }
            return;
        }
    }
    CsrOp op(*this, v, d, nb);
    solve(op, b, x, o, info, count);
}

void LossyOp::inner(const double2 *z, double2 *y) {
    Nd(z, i_p);
    csr(Fv, C0, i_p, i_hp, 3);
    bie_gmres_info gi{};
    solve_csr(Gv, nullptr, 3, i_hp, i_g, nested, gi, true);
    // y = Dr p - Nd' g with p = Nd z
    Dr_minus_NdT(i_p, i_g, y);
}

void LossyOp::outer(const double2 *x, double2 *y) {
    const double2 phi_a = cx(k.phi_a), mu_a = cx(k.mu_a), mu_h = cx(k.mu_h);
    // y = -phi_a Ha x
    Ha(x, y);
    axpby_kernel<<<nblocks(N), 256, 0, stream()>>>(make_double2(-phi_a.x, -phi_a.y), y, make_double2(0, 0), y, N);
    BIE_CUDA(cudaGetLastError());
    launched();
    // sh = gmres(Gh, Hh x)
    csr(Fh, C0, x, o_t, 1);
    bie_gmres_info gi{};
    solve_csr(Gh, nullptr, 1, o_t, o_sh, nested, gi, true);
    // r = Dr Dc x - Nd' gmres(Gv, Hv Dc x)
    Dc(x, o_q);
    csr(Fv, C0, o_q, o_hq, 3);
    solve_csr(Gv, nullptr, 3, o_hq, o_sv, nested, gi, true);
    Dr_minus_NdT(o_q, o_sv, o_r);
    // si = gmres(inner, r)
    BlockOp in(*this, BIE_LOSSY_INNER);
    solve(in, o_r, o_si, nested, gi, true);
    // y += Ga (mu_h sh + mu_a si)
    BIE_CUDA(cudaMemcpyAsync(o_w, o_sh, (size_t)N * 16, cudaMemcpyDeviceToDevice, stream()));
    axpby_kernel<<<nblocks(N), 256, 0, stream()>>>(mu_h, o_w, mu_a, o_si, N);
    BIE_CUDA(cudaGetLastError());
    launched();
    Ga_(o_w, s_t);
    axpby_kernel<<<nblocks(N), 256, 0, stream()>>>(make_double2(1, 0), y, make_double2(1, 0), s_t, N);
    BIE_CUDA(cudaGetLastError());
    launched();
}

LossyOp *create_lossy(Ctx &c, double freq, const bie_lossy_opts &o) {
    if (is_discontinuous(c.physics_kind))
        fail(BIE_ERR_UNSUPPORTED, "the lossy system takes continuous physics only");
    auto L = std::make_unique<LossyOp>();
    L->c = &c;
    const int64_t N = c.n_sources, E = c.n_elements;
    L->N = N;
    const double S = o.S != 0.0 ? o.S : 1.0;
    const double pa = o.custom_air ? o.pa : 101325.0, t = o.custom_air ? o.t : 20.0,
                 Hr = o.custom_air ? o.Hr : 50.0;
    L->k = visco_thermal_constants(freq, S, pa, t, Hr);
    L->fmm = o.fmm_on != 0;
    L->sgn = o.interior ? -1.0 : 1.0;
    L->nested = o.solve;
    L->nested.refine = 0;
    L->nested.initially_nonzero = 0;
    const int depth = o.depth > 0 ? o.depth : 1;
    cudaStream_t s = c.stream;
    const bie_lossy_constants &k = L->k;

    // acoustic operators and the integral-free terms C0
    L->C0 = dev_alloc<double2>(N);
    if (L->fmm) {
        const int ng = o.n_gauss > 0 ? o.n_gauss : 3;
        const double off = o.fmm_offset >= 0 ? o.fmm_offset : 0.2;
        L->fa = create_fastop(c, k.ka[0], k.ka[1], BIE_F, ng, true, off, depth);
        L->ga = create_fastop(c, k.ka[0], k.ka[1], BIE_G, ng, true, off, depth);
        diag_kernel<<<nblocks(N), 256, 0, s>>>(make_double2(0.5, 0), make_double2(0, 0), nullptr, L->C0, N);
    } else {
        L->Fa = dev_alloc<double2>((size_t)N * N);
        L->Ga = dev_alloc<double2>((size_t)N * N);
        AssembleArgs a{k.ka[0], k.ka[1], c.d_sources, N, BIE_F | BIE_G | BIE_C, reinterpret_cast<double *>(L->Fa),
                       reinterpret_cast<double *>(L->Ga), reinterpret_cast<double *>(L->C0)};
        launch_assemble_fp64(c, a);
        if (o.interior)   // Diagonal(1 - C)
            diag_kernel<<<nblocks(N), 256, 0, s>>>(make_double2(1, 0), make_double2(-1, 0), L->C0, L->C0, N);
    }
    BIE_CUDA(cudaGetLastError());

    // thermal and viscous near field on the depth pattern (offset 0: continuous physics)
    const NearField &nf = get_nearfield(c, depth, 0.0, 3);
    const size_t nnz = nf.cols.size();
    L->nf_rp = dev_upload(nf.row_ptr, s);
    L->nf_cols = dev_upload(nf.cols, s);
    double2 **bufs[4] = {&L->Fh, &L->Gh, &L->Fv, &L->Gv};
    for (auto b : bufs) {
        *b = dev_alloc<double2>(nnz);
        BIE_CUDA(cudaMemsetAsync(*b, 0, std::max<size_t>(nnz, 1) * 16, s));
    }
    launch_nearfield(c, nf, k.kh[0], k.kh[1], BIE_F | BIE_G, false, 1.0, reinterpret_cast<double *>(L->Fh),
                     reinterpret_cast<double *>(L->Gh));
    launch_nearfield(c, nf, k.kv[0], k.kv[1], BIE_F | BIE_G, false, 1.0, reinterpret_cast<double *>(L->Fv),
                     reinterpret_cast<double *>(L->Gv));
    if (o.interior) {
        scale_kernel<<<nblocks((int64_t)nnz), 256, 0, s>>>(L->Fh, -1.0, (int64_t)nnz);
        scale_kernel<<<nblocks((int64_t)nnz), 256, 0, s>>>(L->Fv, -1.0, (int64_t)nnz);
        BIE_CUDA(cudaGetLastError());
    }

    // tangential derivatives and normals
    std::vector<int64_t> drp;
    std::vector<int32_t> dcols;
    std::vector<double> dx, dy, dz;
    tangential_derivatives(c.shape_kind, c.physics_kind, c.coords.data(), E, c.topo.data(), c.ptopo.data(), N,
                           drp, dcols, dx, dy, dz);
    L->d_rp = dev_upload(drp, s);
    L->d_cols = dev_upload(dcols, s);
    L->Dx = dev_upload(dx, s);
    L->Dy = dev_upload(dy, s);
    L->Dz = dev_upload(dz, s);
    std::vector<double> nv(o.normals, o.normals + 3 * N);
    L->nrm = dev_upload(nv, s);

    // work vectors: outer t, sh, q (3N), hq (3N), sv (3N), r, si, w; inner p, hp, g
    // (3N each); one more for the acoustic G product
    const int64_t words = 5 + 3 * 3 + 3 * 3 + 1;
    L->work = dev_alloc<double2>((size_t)words * N);
    double2 *p = L->work;
    auto take = [&](int n_vec) {
        double2 *r = p;
        p += (size_t)n_vec * N;
        return r;
    };
    L->o_t = take(1);
    L->o_sh = take(1);
    L->o_q = take(3);
    L->o_hq = take(3);
    L->o_sv = take(3);
    L->o_r = take(1);
    L->o_si = take(1);
    L->o_w = take(1);
    L->i_p = take(3);
    L->i_hp = take(3);
    L->i_g = take(3);
    L->s_t = take(1);
    L->d_acc = dev_alloc<unsigned long long>(2);
    L->d_info = dev_alloc<bie_gmres_info>(1);
    L->d_err = dev_alloc<int>(1);
    BIE_CUDA(cudaMemsetAsync(L->d_acc, 0, 2 * sizeof(unsigned long long), s));
    BIE_CUDA(cudaMemsetAsync(L->d_err, 0, sizeof(int), s));
    BIE_CUDA(cudaStreamSynchronize(s));   // host vectors above are released on return
    return L.release();
}

void destroy_lossy(LossyOp *L) { delete L; }

Ctx &lossy_context(const LossyOp &L) { return *L.c; }

const bie_lossy_constants &lossy_constants(const LossyOp &L) { return L.k; }

int64_t lossy_block_len(int block, bool input, int64_t N) {
    switch (block) {
    case BIE_LOSSY_HV:
    case BIE_LOSSY_GV: return 3 * N;
    case BIE_LOSSY_DC: return input ? N : 3 * N;
    case BIE_LOSSY_ND: return input ? N : 3 * N;
    case BIE_LOSSY_DR:
    case BIE_LOSSY_NDT: return input ? 3 * N : N;
    default: return N;
    }
}

void lossy_apply(LossyOp &L, int block, const double *x_, double *y_) {
    const double2 *x = reinterpret_cast<const double2 *>(x_);
    double2 *y = reinterpret_cast<double2 *>(y_);
    switch (block) {
    case BIE_LOSSY_OUTER: L.outer(x, y); break;
    case BIE_LOSSY_HA: L.Ha(x, y); break;
    case BIE_LOSSY_GA: L.Ga_(x, y); break;
    case BIE_LOSSY_HH: L.csr(L.Fh, L.C0, x, y, 1); break;
    case BIE_LOSSY_GH: L.csr(L.Gh, nullptr, x, y, 1); break;
    case BIE_LOSSY_HV: L.csr(L.Fv, L.C0, x, y, 3); break;
    case BIE_LOSSY_GV: L.csr(L.Gv, nullptr, x, y, 3); break;
    case BIE_LOSSY_DC: L.Dc(x, y); break;
    case BIE_LOSSY_DR: L.Dr_minus_NdT(x, nullptr, y); break;
    case BIE_LOSSY_ND: L.Nd(x, y); break;
    case BIE_LOSSY_NDT:   // Nd' g = -(nx g_0 + ny g_1 + nz g_2)
        dr_ndt_kernel<<<nblocks(L.N), 256, 0, L.stream()>>>(L.d_rp, L.d_cols, L.Dx, L.Dy, L.Dz, nullptr, L.nrm, x,
                                                             -1.0, y, L.N);
        BIE_CUDA(cudaGetLastError());
        L.launched();
        break;
    case BIE_LOSSY_INNER: L.inner(x, y); break;
    default: fail(BIE_ERR_INVALID, "unknown lossy block");
    }
    BIE_CUDA(cudaStreamSynchronize(L.stream()));
    L.check_error();
}

void lossy_solve(LossyOp &L, int block, const double *b, double *x, const bie_gmres_opts &o, bie_gmres_info &info) {
    const double2 *bb = reinterpret_cast<const double2 *>(b);
    double2 *xx = reinterpret_cast<double2 *>(x);
    bie_gmres_opts go = o;
    go.refine = 0;
    go.initially_nonzero = 0;
    switch (block) {
    case BIE_LOSSY_HH: L.solve_csr(L.Fh, L.C0, 1, bb, xx, go, info, false); break;
    case BIE_LOSSY_GH: L.solve_csr(L.Gh, nullptr, 1, bb, xx, go, info, false); break;
    case BIE_LOSSY_HV: L.solve_csr(L.Fv, L.C0, 3, bb, xx, go, info, false); break;
    case BIE_LOSSY_GV: L.solve_csr(L.Gv, nullptr, 3, bb, xx, go, info, false); break;
    case BIE_LOSSY_OUTER:
    case BIE_LOSSY_HA:
    case BIE_LOSSY_GA:
    case BIE_LOSSY_INNER: {
        BlockOp op(L, block);
        L.solve(op, bb, xx, go, info, false);
        break;
    }
    default: fail(BIE_ERR_INVALID, "lossy block is not square");
    }
    BIE_CUDA(cudaStreamSynchronize(L.stream()));
    L.check_error();
}

void lossy_stats(LossyOp &L, int64_t *solves, int64_t *iterations, bool reset) {
    unsigned long long acc[2] = {0, 0};
    BIE_CUDA(cudaMemcpyAsync(acc, L.d_acc, sizeof(acc), cudaMemcpyDeviceToHost, L.stream()));
    BIE_CUDA(cudaStreamSynchronize(L.stream()));
    if (solves) *solves = L.nested_solves + (int64_t)acc[0];
    if (iterations) *iterations = L.nested_iterations + (int64_t)acc[1];
    if (reset) {
        L.nested_solves = L.nested_iterations = 0;
        BIE_CUDA(cudaMemsetAsync(L.d_acc, 0, sizeof(acc), L.stream()));
        BIE_CUDA(cudaStreamSynchronize(L.stream()));
    }
}

void lossy_set_one_launch(LossyOp &L, int mode) {
    if (mode < 0 || mode > 3) fail(BIE_ERR_INVALID, "one-launch mode must be 0, 1, 2 or 3");
    L.one_launch = mode;
}

}  // namespace bie
