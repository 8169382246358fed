// Multi-right-hand-side solve (bie_solve_multi_device):
//     (F + Diagonal(1 - C)) X = B,   B, X: N x R complex,
// the exterior collocation system of test/3d/assembly_test.jl:37-38 for many
// right-hand sides at once.  The reference solves one column at a time
// (IterativeSolvers.gmres per right-hand side; its fast operators take matrix
// arguments in batches of 32 columns, src/3d/fast_multipole_method.jl:249-287).
//
// Here R GMRES solves run in lockstep, so every Arnoldi step applies the
// operator to all R Krylov vectors with one tcgen05 tensor-core product:
//   1. F (mixed assembly, complex64) and C are assembled once; F is quantised
//      once to resident 16-bit tiles (FP16 split by default, ~1e-5 relative
//      product error);
//   2. iterative refinement: the residual B - A X of every column is formed
//      with the exact product of the complex64 matrix (double-float sums, the
//      refinement residual of the frequency sweep), and the correction solves
//      A D = R run as lockstep restarted GMRES on the tensor-core operator to
//      a loose inner tolerance;
//   3. per column the Gram-Schmidt coefficients, the Hessenberg column, the
//      Givens rotations and the residual estimate stay on the device (one
//      thread per column); the host reads one count per step (columns not yet
//      converged).
// Each pass reduces the error by about the inner tolerance, so a few passes
// reach sqrt(eps) relative residual with respect to the complex64 matrix; the
// solution then differs from the FP64 one by the mixed assembly's error times
// the system's sensitivity.
#include "bie_internal.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

namespace bie {

namespace {

constexpr int kIB = 4;   // basis vectors per block of the batched dot products

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cmulc(double2 a, double2 b) {   // conj(a) b
    return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}

// out[i * R + r] = V_i[:, r]^H W[:, r] for i in [i0, i0 + kIB) below nb, with
// V_i = V + i * vstride; all blocks N x R column-major.  grid (R, ceil(nb / kIB))
__global__ void __launch_bounds__(256) bdot_kernel(const double2 *__restrict__ V, int64_t vstride, int nb,
                                                   const double2 *__restrict__ W, int64_t N, int64_t R,
                                                   double2 *__restrict__ out) {
    const int64_t r = blockIdx.x;
    const int i0 = blockIdx.y * kIB;
    double2 acc[kIB];
#pragma unroll
    for (int b = 0; b < kIB; ++b) acc[b] = make_double2(0.0, 0.0);
    const double2 *w = W + r * N;
    for (int64_t n = threadIdx.x; n < N; n += blockDim.x) {
        const double2 wv = w[n];
#pragma unroll
        for (int b = 0; b < kIB; ++b) {
            if (i0 + b < nb) {
                const double2 p = cmulc(V[(int64_t)(i0 + b) * vstride + r * N + n], wv);
                acc[b].x += p.x;
                acc[b].y += p.y;
            }
        }
    }
    __shared__ double2 sm[kIB][8];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int b = 0; b < kIB; ++b) {
        double x = acc[b].x, y = acc[b].y;
        for (int o = 16; o > 0; o >>= 1) {
            x += __shfl_down_sync(0xffffffffu, x, o);
            y += __shfl_down_sync(0xffffffffu, y, o);
        }
        if (lane == 0) sm[b][wid] = make_double2(x, y);
    }
    __syncthreads();
    if (threadIdx.x < kIB && i0 + (int)threadIdx.x < nb) {
        double x = 0, y = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
            x += sm[threadIdx.x][k].x;
            y += sm[threadIdx.x][k].y;
        }
        out[(int64_t)(i0 + threadIdx.x) * R + r] = make_double2(x, y);
    }
}

// W[:, r] -= sum_i V_i[:, r] h[i * R + r]
__global__ void bupdate_kernel(double2 *__restrict__ W, const double2 *__restrict__ V, int64_t vstride, int nb,
                               const double2 *__restrict__ h, int64_t N, int64_t R) {
    const int64_t total = N * R;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = idx / N;
        double2 w = W[idx];
        for (int i = 0; i < nb; ++i) {
            const double2 p = cmul(V[(int64_t)i * vstride + idx], h[(int64_t)i * R + r]);
            w.x -= p.x;
            w.y -= p.y;
        }
        W[idx] = w;
    }
}

// W += d .* V (the diagonal 1 - C)
__global__ void bdiag_kernel(double2 *__restrict__ W, const double2 *__restrict__ V, const double2 *__restrict__ d,
                             int64_t N, int64_t R) {
    const int64_t total = N * R;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const double2 p = cmul(d[idx % N], V[idx]);
        W[idx].x += p.x;
        W[idx].y += p.y;
    }
}

// out = a - b  (out may alias a or b)
__global__ void bsub_kernel(const double2 *a, const double2 *b, double2 *out, int64_t total) {
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const double2 x = a[idx], y = b[idx];
        out[idx] = make_double2(x.x - y.x, x.y - y.y);
    }
}

// X += D
__global__ void badd_kernel(double2 *__restrict__ X, const double2 *__restrict__ D, int64_t total) {
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        X[idx].x += D[idx].x;
        X[idx].y += D[idx].y;
    }
}

// V0[:, r] = W[:, r] / beta_r with beta_r^2 = nrm2[r].x
__global__ void bstart_kernel(double2 *__restrict__ V0, const double2 *__restrict__ W,
                              const double2 *__restrict__ nrm2, int64_t N, int64_t R) {
    const int64_t total = N * R;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const double beta = sqrt(fmax(nrm2[idx / N].x, 0.0));
        const double s = beta > 0 ? 1.0 / beta : 0.0;
        V0[idx] = make_double2(W[idx].x * s, W[idx].y * s);
    }
}

// g_r = (beta_r, 0, ..., 0), one thread per column
__global__ void bginit_kernel(const double2 *__restrict__ nrm2, int64_t R, int m, double2 *__restrict__ g) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
    const double beta = sqrt(fmax(nrm2[r].x, 0.0));
    for (int i = 0; i <= m; ++i) g[r * (m + 1) + i] = make_double2(i == 0 ? beta : 0.0, 0.0);
}

// Arnoldi step j of every column: Hessenberg column from the two Gram-Schmidt
// passes and |w|, previous rotations applied, new rotation, residual estimate
// |g_{j+1}|.  One thread per column; rotation i is [c s; -conj(s) c], c real.
__global__ void bgivens_kernel(int j, int m, int64_t R, const double2 *__restrict__ h1,
                               const double2 *__restrict__ h2, const double2 *__restrict__ nrm2,
                               double2 *__restrict__ H, double2 *__restrict__ g, double *__restrict__ cs,
                               double2 *__restrict__ sn, double *__restrict__ res, double *__restrict__ inv_hn) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
    double2 *Hc = H + (r * m + j) * (int64_t)(m + 1);   // column j of column r's Hessenberg matrix
    for (int i = 0; i <= j; ++i) {
        const double2 a = h1[(int64_t)i * R + r], b = h2[(int64_t)i * R + r];
        Hc[i] = make_double2(a.x + b.x, a.y + b.y);
    }
    const double hn = sqrt(fmax(nrm2[r].x, 0.0));
    inv_hn[r] = hn > 0 ? 1.0 / hn : 0.0;
    double *csr = cs + r * m;
    double2 *snr = sn + r * m;
    for (int i = 0; i < j; ++i) {
        const double2 a = Hc[i], b = Hc[i + 1];
        const double c = csr[i];
        const double2 s = snr[i];
        const double2 sb = cmul(s, b);
        const double2 sa = cmulc(s, a);
        Hc[i] = make_double2(c * a.x + sb.x, c * a.y + sb.y);
        Hc[i + 1] = make_double2(-sa.x + c * b.x, -sa.y + c * b.y);
    }
    const double2 a = Hc[j];
    const double aa = hypot(a.x, a.y);
    double c;
    double2 s;
    if (hn == 0.0) {
        c = 1.0;
        s = make_double2(0.0, 0.0);
    } else if (aa == 0.0) {
        c = 0.0;
        s = make_double2(1.0, 0.0);
    } else {
        const double t = hypot(aa, hn);
        c = aa / t;
        s = make_double2(a.x / aa * (hn / t), a.y / aa * (hn / t));   // (a / |a|) hn / t
    }
    csr[j] = c;
    snr[j] = s;
    Hc[j] = make_double2(c * a.x + s.x * hn, c * a.y + s.y * hn);
    double2 *gr = g + r * (m + 1);
    const double2 gj = gr[j];
    const double2 sg = cmulc(s, gj);
    gr[j] = make_double2(c * gj.x, c * gj.y);
    gr[j + 1] = make_double2(-sg.x, -sg.y);
    res[r] = hypot(gr[j + 1].x, gr[j + 1].y);
}

// V_{j+1}[:, r] = W[:, r] / |w_r|
__global__ void bscale_kernel(double2 *__restrict__ Vn, const double2 *__restrict__ W,
                              const double *__restrict__ inv, int64_t N, int64_t R) {
    const int64_t total = N * R;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const double s = inv[idx / N];
        Vn[idx] = make_double2(W[idx].x * s, W[idx].y * s);
    }
}

// columns whose residual estimate is above their tolerance (NaN counts)
__global__ void bcount_kernel(const double *__restrict__ res, const double *__restrict__ tol, int64_t R,
                              int *__restrict__ count) {
    __shared__ int s;
    if (threadIdx.x == 0) s = 0;
    __syncthreads();
    int k = 0;
    for (int64_t r = threadIdx.x; r < R; r += blockDim.x) k += !(res[r] <= tol[r]);
    atomicAdd(&s, k);
    __syncthreads();
    if (threadIdx.x == 0) *count = s;
}

// y_r = R_r^{-1} g_r over the first jd columns (back substitution), per column
__global__ void btrisolve_kernel(int jd, int m, int64_t R, const double2 *__restrict__ H,
                                 const double2 *__restrict__ g, double2 *__restrict__ y) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
    const double2 *Hr = H + r * m * (int64_t)(m + 1);
    double2 *yr = y + r * m;
    for (int i = jd - 1; i >= 0; --i) {
        double2 t = g[r * (m + 1) + i];
        for (int k = i + 1; k < jd; ++k) {
            const double2 p = cmul(Hr[(int64_t)k * (m + 1) + i], yr[k]);
            t.x -= p.x;
            t.y -= p.y;
        }
        const double2 d = Hr[(int64_t)i * (m + 1) + i];
        const double dd = d.x * d.x + d.y * d.y;
        yr[i] = dd > 0 ? make_double2((t.x * d.x + t.y * d.y) / dd, (t.y * d.x - t.x * d.y) / dd)
                       : make_double2(0.0, 0.0);
    }
}

// D[:, r] += sum_{i < jd} V_i[:, r] y_r[i]
__global__ void bcombo_kernel(double2 *__restrict__ D, const double2 *__restrict__ V, int64_t vstride, int jd, int m,
                              const double2 *__restrict__ y, int64_t N, int64_t R) {
    const int64_t total = N * R;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = idx / N;
        double2 acc = D[idx];
        for (int i = 0; i < jd; ++i) {
            const double2 p = cmul(V[(int64_t)i * vstride + idx], y[r * m + i]);
            acc.x += p.x;
            acc.y += p.y;
        }
        D[idx] = acc;
    }
}

__global__ void one_minus_c_kernel(const double2 *__restrict__ C, double2 *__restrict__ d, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) d[i] = make_double2(1.0 - C[i].x, -C[i].y);
}

struct Buf {
    void *p = nullptr;
    explicit Buf(size_t bytes) { BIE_CUDA(cudaMalloc(&p, std::max<size_t>(bytes, 16))); }
    ~Buf() { cudaFree(p); }
    Buf(const Buf &) = delete;
    Buf &operator=(const Buf &) = delete;
    template <class T> T *as() const { return static_cast<T *>(p); }
};

struct LowpGuard {
    LowpMatrix *m;
    ~LowpGuard() { lowp_matrix_destroy(m); }
};

inline unsigned g1(const Ctx &c, int64_t n) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 16LL * c.num_sms));
}
inline unsigned gcols(int64_t R) { return (unsigned)((R + 127) / 128); }

}  // namespace

void run_solve_multi(Ctx &c, double k_re, double k_im, int64_t R, const double *B_, double *X_,
                     const bie_multisolve_opts &o, bie_multisolve_info &info) {
    // BIE_TRACE=1: stage markers on stderr (locating failures on a GPU machine)
    static const bool trace = [] {
        const char *e = std::getenv("BIE_TRACE");
        return e && *e == '1';
    }();
    auto mark = [&](const char *what) {
        if (!trace) return;
        const cudaError_t e = cudaStreamSynchronize(c.stream);
        std::fprintf(stderr, "[solve_multi] %s (%s)\n", what, cudaGetErrorString(e));
        std::fflush(stderr);
    };
    info = bie_multisolve_info{};
    const int64_t N = c.n_sources;
    const int prec = o.precision > 0 ? o.precision : BIE_PREC_FP16_SPLIT;
    if (prec < BIE_PREC_FP16 || prec > BIE_PREC_BF16_SPLIT)
        fail(BIE_ERR_INVALID, "precision must be one of the 16-bit tensor-core forms");
    const int m =
        (int)std::max<int64_t>(1, std::min<int64_t>(o.restart > 0 ? o.restart : 20, std::min<int64_t>(N, 64)));
    const int maxiter = o.maxiter > 0 ? o.maxiter : 200;
    const int max_refine = o.max_refine > 0 ? o.max_refine : 10;
    const double reltol = o.reltol > 0 ? o.reltol : std::sqrt(2.220446049250313e-16);
    const double inner_rel = o.inner_reltol > 0 ? o.inner_reltol : 1e-4;
    const double2 *B = reinterpret_cast<const double2 *>(B_);
    double2 *X = reinterpret_cast<double2 *>(X_);
    const int64_t NR = N * R;
    using clk = std::chrono::steady_clock;
    auto ms_since = [](clk::time_point t) {
        return std::chrono::duration<double, std::milli>(clk::now() - t).count();
    };
    mark("start");

    // 1. F (complex64) and C by the mixed assembly; diag = 1 - C; resident tiles of F
    const auto t0 = clk::now();
    Buf F32((size_t)N * N * 8), Cv((size_t)N * 16), dg((size_t)N * 16);
    AssembleArgs a{k_re, k_im, c.d_sources, N, BIE_F | BIE_C, F32.as<double>(), nullptr, Cv.as<double>()};
    a.c64_out = true;
    launch_assemble_mixed(c, a);
    one_minus_c_kernel<<<(unsigned)((N + 255) / 256), 256, 0, c.stream>>>(Cv.as<double2>(), dg.as<double2>(), N);
    BIE_CUDA(cudaGetLastError());
    ++c.kernel_launches;
    mark("assembled");
    LowpGuard lg{lowp_matrix_create(c, F32.as<float>(), N, prec)};
    BIE_CUDA(cudaStreamSynchronize(c.stream));
    mark("quantised");
    info.setup_ms = ms_since(t0);

    // 2. workspace: Krylov blocks V_0..V_m, W, the residual, the correction, and
    // per-column arrays (each on a 256-byte boundary, sizes as taken below)
    const int64_t vstride = NR;
    Buf Vb((size_t)(m + 1) * NR * 16), Wb((size_t)NR * 16), Rb((size_t)NR * 16), Db((size_t)NR * 16);
    auto up = [](size_t b) { return (b + 255) & ~size_t(255); };
    const size_t small = up((size_t)R * m * (m + 1) * 16) + 3 * up((size_t)R * (m + 1) * 16) +
                         2 * up((size_t)R * m * 16) + 2 * up((size_t)R * 16) + up((size_t)R * m * 8) +
                         4 * up((size_t)R * 8) + up(16);
    Buf Sb(small);
    double2 *V = Vb.as<double2>(), *W = Wb.as<double2>(), *Rr = Rb.as<double2>(), *D = Db.as<double2>();
    char *sp = Sb.as<char>();
    char *const sp_end = sp + small;
    auto take = [&](size_t bytes) {
        char *p = sp;
        sp += up(bytes);
        if (sp > sp_end) fail(BIE_ERR_INVALID, "multi-RHS solve: workspace carve overrun");
        return p;
    };
    double2 *H = reinterpret_cast<double2 *>(take((size_t)R * m * (m + 1) * 16));
    double2 *g = reinterpret_cast<double2 *>(take((size_t)R * (m + 1) * 16));
    double2 *h1 = reinterpret_cast<double2 *>(take((size_t)R * (m + 1) * 16));
    double2 *h2 = reinterpret_cast<double2 *>(take((size_t)R * (m + 1) * 16));
    double2 *sn = reinterpret_cast<double2 *>(take((size_t)R * m * 16));
    double2 *y = reinterpret_cast<double2 *>(take((size_t)R * m * 16));
    double2 *nrm = reinterpret_cast<double2 *>(take((size_t)R * 16));
    double2 *bnrm = reinterpret_cast<double2 *>(take((size_t)R * 16));
    double *cs = reinterpret_cast<double *>(take((size_t)R * m * 8));
    double *res = reinterpret_cast<double *>(take((size_t)R * 8));
    double *inv = reinterpret_cast<double *>(take((size_t)R * 8));
    double *tol = reinterpret_cast<double *>(take((size_t)R * 8));
    double *spare = reinterpret_cast<double *>(take((size_t)R * 8));
    int *count = reinterpret_cast<int *>(take(16));
    (void)spare;
    std::vector<double2> nh((size_t)R), bh((size_t)R);
    std::vector<double> th((size_t)R);

    auto dot = [&](const double2 *Vs, int nb, const double2 *w, double2 *out) {
        dim3 grid((unsigned)R, (unsigned)((nb + kIB - 1) / kIB));
        bdot_kernel<<<grid, 256, 0, c.stream>>>(Vs, vstride, nb, w, N, R, out);
        BIE_CUDA(cudaGetLastError());
        ++c.kernel_launches;
    };
    // tensor-core operator: Wout = F Vin + d .* Vin
    auto apply_tc = [&](const double2 *Vin, double2 *Wout) {
        const auto ta = clk::now();
        lowp_matrix_apply(c, *lg.m, reinterpret_cast<const double *>(Vin), R, reinterpret_cast<double *>(Wout));
        bdiag_kernel<<<g1(c, NR), 256, 0, c.stream>>>(Wout, Vin, dg.as<double2>(), N, R);
        BIE_CUDA(cudaGetLastError());
        ++c.kernel_launches;
        ++info.tensor_products;
        info.tensor_ms += ms_since(ta);
        mark("tensor product");
    };
    // exact product of the complex64 matrix, column by column: Wout = F Xin + d .* Xin
    bie_operator exact{};
    exact.kind = BIE_OP_DENSE;
    exact.A32 = F32.as<float>();
    exact.scale_re = 1.0;
    exact.diag = dg.as<double>();
    auto apply_exact = [&](const double2 *Xin, double2 *Wout) {
        const auto ta = clk::now();
        for (int64_t r = 0; r < R; ++r)
            apply_operator(c, exact, BIE_PREC_FP64, reinterpret_cast<const double *>(Xin + r * N),
                           reinterpret_cast<double *>(Wout + r * N));
        BIE_CUDA(cudaStreamSynchronize(c.stream));
        ++info.exact_products;
        info.exact_ms += ms_since(ta);
        mark("exact product");
    };
    auto read_count = [&]() {
        bcount_kernel<<<1, 256, 0, c.stream>>>(res, tol, R, count);
        BIE_CUDA(cudaGetLastError());
        ++c.kernel_launches;
        int h = 0;
        BIE_CUDA(cudaMemcpyAsync(&h, count, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
        BIE_CUDA(cudaStreamSynchronize(c.stream));
        return h;
    };
    auto norms_to_host = [&](const double2 *dev, std::vector<double2> &host) {
        BIE_CUDA(cudaMemcpyAsync(host.data(), dev, (size_t)R * 16, cudaMemcpyDeviceToHost, c.stream));
        BIE_CUDA(cudaStreamSynchronize(c.stream));
    };

    // 3. refinement passes
    dot(B, 1, B, bnrm);
    norms_to_host(bnrm, bh);
    BIE_CUDA(cudaMemsetAsync(X, 0, (size_t)NR * 16, c.stream));
    BIE_CUDA(cudaMemcpyAsync(Rr, B, (size_t)NR * 16, cudaMemcpyDeviceToDevice, c.stream));   // R = B - A 0
    mark("workspace");
    for (int pass = 0;; ++pass) {
        if (pass > 0) {
            apply_exact(X, W);
            bsub_kernel<<<g1(c, NR), 256, 0, c.stream>>>(B, W, Rr, NR);
            BIE_CUDA(cudaGetLastError());
            ++c.kernel_launches;
        }
        // relative residuals ||R_r|| / ||B_r||
        dot(Rr, 1, Rr, nrm);
        norms_to_host(nrm, nh);
        info.max_relres = 0.0;
        int64_t conv = 0;
        for (int64_t r = 0; r < R; ++r) {
            const double bn = std::sqrt(std::max(bh[r].x, 0.0));
            const double rn = std::sqrt(std::max(nh[r].x, 0.0));
            const double v = bn > 0 ? rn / bn : rn;
            info.max_relres = std::max(info.max_relres, std::isnan(v) ? INFINITY : v);
            conv += v <= reltol;
            th[r] = inner_rel * rn;   // tolerance of this pass's inner solve
        }
        info.converged = (int32_t)conv;
        if (conv == R || pass >= max_refine) break;
        ++info.passes;
        BIE_CUDA(cudaMemcpyAsync(tol, th.data(), (size_t)R * 8, cudaMemcpyHostToDevice, c.stream));

        // inner lockstep restarted GMRES on A D = R with the tensor-core operator
        BIE_CUDA(cudaMemsetAsync(D, 0, (size_t)NR * 16, c.stream));
        int steps = 0;
        for (int cycle = 0; steps < maxiter; ++cycle) {
            const double2 *rhs = Rr;
            if (cycle > 0) {   // the inner residual R - A D
                apply_tc(D, W);
                bsub_kernel<<<g1(c, NR), 256, 0, c.stream>>>(Rr, W, W, NR);
                BIE_CUDA(cudaGetLastError());
                ++c.kernel_launches;
                rhs = W;
            }
            dot(rhs, 1, rhs, nrm);
            bstart_kernel<<<g1(c, NR), 256, 0, c.stream>>>(V, rhs, nrm, N, R);
            bginit_kernel<<<gcols(R), 128, 0, c.stream>>>(nrm, R, m, g);
            BIE_CUDA(cudaGetLastError());
            c.kernel_launches += 2;
            int jd = 0;
            bool done = false;
            for (int j = 0; j < m && steps < maxiter; ++j) {
                apply_tc(V + (int64_t)j * vstride, W);
                dot(V, j + 1, W, h1);
                bupdate_kernel<<<g1(c, NR), 256, 0, c.stream>>>(W, V, vstride, j + 1, h1, N, R);
                dot(V, j + 1, W, h2);
                bupdate_kernel<<<g1(c, NR), 256, 0, c.stream>>>(W, V, vstride, j + 1, h2, N, R);
                dot(W, 1, W, nrm);
                bgivens_kernel<<<gcols(R), 128, 0, c.stream>>>(j, m, R, h1, h2, nrm, H, g, cs, sn, res, inv);
                bscale_kernel<<<g1(c, NR), 256, 0, c.stream>>>(V + (int64_t)(j + 1) * vstride, W, inv, N, R);
                BIE_CUDA(cudaGetLastError());
                c.kernel_launches += 4;
                ++steps;
                jd = j + 1;
                if (read_count() == 0) {
                    done = true;
                    break;
                }
            }
            btrisolve_kernel<<<gcols(R), 128, 0, c.stream>>>(jd, m, R, H, g, y);
            bcombo_kernel<<<g1(c, NR), 256, 0, c.stream>>>(D, V, vstride, jd, m, y, N, R);
            BIE_CUDA(cudaGetLastError());
            c.kernel_launches += 2;
            if (done) break;
        }
        info.inner_steps += steps;
        badd_kernel<<<g1(c, NR), 256, 0, c.stream>>>(X, D, NR);
        BIE_CUDA(cudaGetLastError());
        ++c.kernel_launches;
        mark("pass done");
    }
    BIE_CUDA(cudaStreamSynchronize(c.stream));
}

}  // namespace bie
