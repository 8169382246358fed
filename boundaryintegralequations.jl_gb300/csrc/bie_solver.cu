// K5: restarted GMRES on the device for  A x = b  with
//     A x = s (K x) + d .* x,
// K either a stored dense matrix (complex128 or complex64, column-major, the
// output of the assembly) or the matrix-free double-layer operator F.
// This replaces IterativeSolvers.gmres (v0.9) as called by the reference
// (test/3d/assembly_test.jl:38, examples/3d_pulsating_sphere.jl:44-50):
// same defaults (restart = min(20, N), reltol = sqrt(eps(Float64)), abstol 0,
// maxiter = N, x0 = 0) and the same stopping test ||r|| <= max(reltol ||b||,
// abstol) on the Arnoldi residual estimate.
//
// Arnoldi uses classical Gram-Schmidt with one reorthogonalisation pass
// (CGS2, the same numerical role as IterativeSolvers' default DGKS
// orthogonalisation); the small Hessenberg least-squares problem is solved on
// the host with Givens rotations (FP64).  Mixed-precision iterative refinement
// (opts->refine) runs the inner GMRES on the cheaper operator (complex64 dense
// copy or mixed matrix-free product) and forms the outer residual b - A x with
// the FP64 operator.
#include "bie_internal.h"
#include "bie_device.cuh"

#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

namespace bie {

namespace {

using cplx = std::complex<double>;
constexpr int kT = 256;

// y[i] = s * sum_j A[i + j*lda] x[j] for the column slice of blockIdx.y
template <typename T2>
__global__ void __launch_bounds__(kT)
dense_gemv_kernel(const T2 *__restrict__ A, int64_t n, const double2 *__restrict__ x,
                  double2 *__restrict__ part, int S, const int *__restrict__ stop) {
    if (stop && *stop) return;
    const int64_t i = (int64_t)blockIdx.x * kT + threadIdx.x;
    const int s = blockIdx.y;
    const int64_t j0 = (int64_t)s * n / S, j1 = (int64_t)(s + 1) * n / S;
    __shared__ double2 xs[kT];
    double re = 0, im = 0;
    for (int64_t jb = j0; jb < j1; jb += kT) {
        const int nb = (int)min((int64_t)kT, j1 - jb);
        __syncthreads();
        if (threadIdx.x < nb) xs[threadIdx.x] = x[jb + threadIdx.x];
        __syncthreads();
        if (i < n) {
            const T2 *col = A + jb * n + i;
#pragma unroll 4
            for (int j = 0; j < nb; ++j) {
                const T2 a = col[(int64_t)j * n];
                const double ar = (double)a.x, ai = (double)a.y;
                const double2 xv = xs[j];
                re += ar * xv.x - ai * xv.y;
                im += ar * xv.y + ai * xv.x;
            }
        }
    }
    if (i < n) part[(int64_t)s * n + i] = make_double2(re, im);
}

// Complex64 matrix times complex128 vector on the FP32 pipe, for the column
// slice of blockIdx.y.  On GB300 the FP64 pipe cannot keep up with HBM even for
// a matrix-vector product, so the products run in FP32: the vector is rounded
// to FP32, every block of kFold columns is summed with plain FP32 FMAs and the
// block sums are carried in double-float (TwoSum).  The product then has a
// relative error of a few FP32 roundings (~1e-7) — the size of the complex64
// rounding of the stored matrix itself — at 8 FMAs per 16-byte load, which
// keeps the kernel on the HBM roofline.  Each thread handles two consecutive
// rows (one 16-byte load per column).
constexpr int kFold = 16;

__device__ __forceinline__ void df_fold(dev::df &acc, float s) {
    const dev::df t = dev::two_sum(acc.hi, s);
    acc = dev::fast_two_sum(t.hi, __fadd_rn(t.lo, acc.lo));
}

// The same product to ~1e-14 relative (the residuals of refinement and the
// right-hand sides): the vector is split into double-float (x = hi + lo),
// a * hi is formed exactly (TwoProduct), a * lo is added to its error term and
// every sum is carried in double-float (TwoSum).  About 14 instructions per
// real multiply-add, so issue-bound at roughly half the HBM rate.
__global__ void __launch_bounds__(kT)
dense_gemv_c64_exact_kernel(const float4 *__restrict__ A2, int64_t n, const double2 *__restrict__ x,
                            double2 *__restrict__ part, int S, const int *__restrict__ stop) {
    if (stop && *stop) return;
    const int64_t r2 = (int64_t)blockIdx.x * kT + threadIdx.x;   // row pair index
    const int64_t i0 = 2 * r2;
    const int s = blockIdx.y;
    const int64_t j0 = (int64_t)s * n / S, j1 = (int64_t)(s + 1) * n / S;
    __shared__ float4 xs[kT];   // (re hi, re lo, im hi, im lo)
    dev::df yr0 = {0.f, 0.f}, yi0 = {0.f, 0.f}, yr1 = {0.f, 0.f}, yi1 = {0.f, 0.f};
    const int64_t ld2 = n / 2;  // float4 per column (n even)
    auto mac = [](dev::df &acc, float av, float xh, float xl) {
        const float p = av * xh;
        float e = __fmaf_rn(av, xh, -p);
        e = __fmaf_rn(av, xl, e);
        const dev::df t = dev::two_sum(acc.hi, p);
        acc = dev::fast_two_sum(t.hi, __fadd_rn(__fadd_rn(t.lo, e), acc.lo));
    };
    for (int64_t jb = j0; jb < j1; jb += kT) {
        const int nb = (int)min((int64_t)kT, j1 - jb);
        __syncthreads();
        if (threadIdx.x < nb) {
            const double2 v = x[jb + threadIdx.x];
            const dev::df re = dev::df_from_double(v.x), im = dev::df_from_double(v.y);
            xs[threadIdx.x] = make_float4(re.hi, re.lo, im.hi, im.lo);
        }
        __syncthreads();
        if (i0 < n) {
            const float4 *col = A2 + jb * ld2 + r2;
#pragma unroll 4
            for (int j = 0; j < nb; ++j) {
                const float4 a = col[(int64_t)j * ld2];   // (re0, im0, re1, im1)
                const float4 xv = xs[j];
                mac(yr0, a.x, xv.x, xv.y);
                mac(yr0, -a.y, xv.z, xv.w);
                mac(yi0, a.x, xv.z, xv.w);
                mac(yi0, a.y, xv.x, xv.y);
                mac(yr1, a.z, xv.x, xv.y);
                mac(yr1, -a.w, xv.z, xv.w);
                mac(yi1, a.z, xv.z, xv.w);
                mac(yi1, a.w, xv.x, xv.y);
            }
        }
    }
    if (i0 < n) {
        part[(int64_t)s * n + i0] = make_double2(dev::f2d(yr0.hi) + dev::f2d(yr0.lo),
                                                 dev::f2d(yi0.hi) + dev::f2d(yi0.lo));
        if (i0 + 1 < n)
            part[(int64_t)s * n + i0 + 1] = make_double2(dev::f2d(yr1.hi) + dev::f2d(yr1.lo),
                                                         dev::f2d(yi1.hi) + dev::f2d(yi1.lo));
    }
}

// Odd n, exact form: one row per thread, 8-byte loads.
__global__ void __launch_bounds__(kT)
dense_gemv_c64_rows_exact_kernel(const float2 *__restrict__ A, int64_t n, const double2 *__restrict__ x,
                                 double2 *__restrict__ part, int S, const int *__restrict__ stop) {
    if (stop && *stop) return;
    const int64_t i = (int64_t)blockIdx.x * kT + threadIdx.x;
    const int s = blockIdx.y;
    const int64_t j0 = (int64_t)s * n / S, j1 = (int64_t)(s + 1) * n / S;
    __shared__ float4 xs[kT];
    dev::df yr = {0.f, 0.f}, yi = {0.f, 0.f};
    auto mac = [](dev::df &acc, float av, float xh, float xl) {
        const float p = av * xh;
        float e = __fmaf_rn(av, xh, -p);
        e = __fmaf_rn(av, xl, e);
        const dev::df t = dev::two_sum(acc.hi, p);
        acc = dev::fast_two_sum(t.hi, __fadd_rn(__fadd_rn(t.lo, e), acc.lo));
    };
    for (int64_t jb = j0; jb < j1; jb += kT) {
        const int nb = (int)min((int64_t)kT, j1 - jb);
        __syncthreads();
        if (threadIdx.x < nb) {
            const double2 v = x[jb + threadIdx.x];
            const dev::df re = dev::df_from_double(v.x), im = dev::df_from_double(v.y);
            xs[threadIdx.x] = make_float4(re.hi, re.lo, im.hi, im.lo);
        }
        __syncthreads();
        if (i < n) {
            const float2 *col = A + jb * n + i;
            for (int j = 0; j < nb; ++j) {
                const float2 a = col[(int64_t)j * n];
                const float4 xv = xs[j];
                mac(yr, a.x, xv.x, xv.y);
                mac(yr, -a.y, xv.z, xv.w);
                mac(yi, a.x, xv.z, xv.w);
                mac(yi, a.y, xv.x, xv.y);
            }
        }
    }
    if (i < n)
        part[(int64_t)s * n + i] = make_double2(dev::f2d(yr.hi) + dev::f2d(yr.lo),
                                                dev::f2d(yi.hi) + dev::f2d(yi.lo));
}

__global__ void __launch_bounds__(kT)
dense_gemv_c64_kernel(const float4 *__restrict__ A2, int64_t n, const double2 *__restrict__ x,
                      double2 *__restrict__ part, int S, const int *__restrict__ stop) {
    if (stop && *stop) return;
    const int64_t r2 = (int64_t)blockIdx.x * kT + threadIdx.x;   // row pair index
    const int64_t i0 = 2 * r2;
    const int s = blockIdx.y;
    const int64_t j0 = (int64_t)s * n / S, j1 = (int64_t)(s + 1) * n / S;
    __shared__ float2 xs[kT];
    dev::df yr0 = {0.f, 0.f}, yi0 = {0.f, 0.f}, yr1 = {0.f, 0.f}, yi1 = {0.f, 0.f};
    const int64_t ld2 = n / 2;  // float4 per column (n even)
    for (int64_t jb = j0; jb < j1; jb += kT) {
        const int nb = (int)min((int64_t)kT, j1 - jb);
        __syncthreads();
        if (threadIdx.x < nb) {
            const double2 v = x[jb + threadIdx.x];
            xs[threadIdx.x] = make_float2((float)v.x, (float)v.y);
        }
        __syncthreads();
        if (i0 < n) {
            const float4 *col = A2 + jb * ld2 + r2;
            for (int jf = 0; jf < nb; jf += kFold) {
                const int ne = min(kFold, nb - jf);
                float sr0 = 0.f, si0 = 0.f, sr1 = 0.f, si1 = 0.f;
                if (ne == kFold) {
#pragma unroll
                    for (int j = 0; j < kFold; ++j) {
                        const float4 a = col[(int64_t)(jf + j) * ld2];   // (re0, im0, re1, im1)
                        const float2 xv = xs[jf + j];
                        sr0 = __fmaf_rn(a.x, xv.x, sr0);
                        sr0 = __fmaf_rn(-a.y, xv.y, sr0);
                        si0 = __fmaf_rn(a.x, xv.y, si0);
                        si0 = __fmaf_rn(a.y, xv.x, si0);
                        sr1 = __fmaf_rn(a.z, xv.x, sr1);
                        sr1 = __fmaf_rn(-a.w, xv.y, sr1);
                        si1 = __fmaf_rn(a.z, xv.y, si1);
                        si1 = __fmaf_rn(a.w, xv.x, si1);
                    }
                } else {
                    for (int j = 0; j < ne; ++j) {
                        const float4 a = col[(int64_t)(jf + j) * ld2];
                        const float2 xv = xs[jf + j];
                        sr0 = __fmaf_rn(a.x, xv.x, sr0);
                        sr0 = __fmaf_rn(-a.y, xv.y, sr0);
                        si0 = __fmaf_rn(a.x, xv.y, si0);
                        si0 = __fmaf_rn(a.y, xv.x, si0);
                        sr1 = __fmaf_rn(a.z, xv.x, sr1);
                        sr1 = __fmaf_rn(-a.w, xv.y, sr1);
                        si1 = __fmaf_rn(a.z, xv.y, si1);
                        si1 = __fmaf_rn(a.w, xv.x, si1);
                    }
                }
                df_fold(yr0, sr0);
                df_fold(yi0, si0);
                df_fold(yr1, sr1);
                df_fold(yi1, si1);
            }
        }
    }
    if (i0 < n) {
        part[(int64_t)s * n + i0] = make_double2(dev::f2d(yr0.hi) + dev::f2d(yr0.lo),
                                                 dev::f2d(yi0.hi) + dev::f2d(yi0.lo));
        if (i0 + 1 < n)
            part[(int64_t)s * n + i0 + 1] = make_double2(dev::f2d(yr1.hi) + dev::f2d(yr1.lo),
                                                         dev::f2d(yi1.hi) + dev::f2d(yi1.lo));
    }
}

// Same product for odd n: one row per thread, 8-byte loads.
__global__ void __launch_bounds__(kT)
dense_gemv_c64_rows_kernel(const float2 *__restrict__ A, int64_t n, const double2 *__restrict__ x,
                           double2 *__restrict__ part, int S, const int *__restrict__ stop) {
    if (stop && *stop) return;
    const int64_t i = (int64_t)blockIdx.x * kT + threadIdx.x;
    const int s = blockIdx.y;
    const int64_t j0 = (int64_t)s * n / S, j1 = (int64_t)(s + 1) * n / S;
    __shared__ float2 xs[kT];
    dev::df yr = {0.f, 0.f}, yi = {0.f, 0.f};
    for (int64_t jb = j0; jb < j1; jb += kT) {
        const int nb = (int)min((int64_t)kT, j1 - jb);
        __syncthreads();
        if (threadIdx.x < nb) {
            const double2 v = x[jb + threadIdx.x];
            xs[threadIdx.x] = make_float2((float)v.x, (float)v.y);
        }
        __syncthreads();
        if (i < n) {
            const float2 *col = A + jb * n + i;
            for (int jf = 0; jf < nb; jf += kFold) {
                const int ne = min(kFold, nb - jf);
                float sr = 0.f, si = 0.f;
                for (int j = 0; j < ne; ++j) {
                    const float2 a = col[(int64_t)(jf + j) * n];
                    const float2 xv = xs[jf + j];
                    sr = __fmaf_rn(a.x, xv.x, sr);
                    sr = __fmaf_rn(-a.y, xv.y, sr);
                    si = __fmaf_rn(a.x, xv.y, si);
                    si = __fmaf_rn(a.y, xv.x, si);
                }
                df_fold(yr, sr);
                df_fold(yi, si);
            }
        }
    }
    if (i < n)
        part[(int64_t)s * n + i] = make_double2(dev::f2d(yr.hi) + dev::f2d(yr.lo),
                                                dev::f2d(yi.hi) + dev::f2d(yi.lo));
}

// y = s * sum_slices(part) + d .* x   (d may be null)
__global__ void combine_kernel(const double2 *__restrict__ part, int S, int64_t n, double2 sc,
                               const double2 *__restrict__ d, const double2 *__restrict__ x,
                               double2 *__restrict__ y, const int *__restrict__ stop) {
    if (stop && *stop) return;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double re = 0, im = 0;
    for (int s = 0; s < S; ++s) {
        const double2 p = part[(int64_t)s * n + i];
        re += p.x;
        im += p.y;
    }
    double yr = sc.x * re - sc.y * im, yi = sc.x * im + sc.y * re;
    if (d) {
        const double2 dv = d[i], xv = x[i];
        yr += dv.x * xv.x - dv.y * xv.y;
        yi += dv.x * xv.y + dv.y * xv.x;
    }
    y[i] = make_double2(yr, yi);
}

// partial[col * nb + block] = sum over the block's rows of conj(V[:, col]) . w
__global__ void __launch_bounds__(kT)
multidot_kernel(const double2 *__restrict__ V, int64_t ldv, const double2 *__restrict__ w,
                int64_t n, double2 *__restrict__ partial, const int *__restrict__ stop) {
    if (stop && *stop) return;
    const int col = blockIdx.y;
    const double2 *v = V + (int64_t)col * ldv;
    double re = 0, im = 0;
    for (int64_t i = (int64_t)blockIdx.x * kT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kT) {
        const double2 a = v[i], b = w[i];
        re += a.x * b.x + a.y * b.y;
        im += a.x * b.y - a.y * b.x;
    }
    __shared__ double sr[kT], si[kT];
    sr[threadIdx.x] = re;
    si[threadIdx.x] = im;
    __syncthreads();
    for (int o = kT / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            sr[threadIdx.x] += sr[threadIdx.x + o];
            si[threadIdx.x] += si[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[(int64_t)col * gridDim.x + blockIdx.x] = make_double2(sr[0], si[0]);
}

__global__ void sum_partials_kernel(const double2 *__restrict__ partial, int nb, int ncol,
                                    double2 *__restrict__ out, const int *__restrict__ stop) {
    if (stop && *stop) return;
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= ncol) return;
    double re = 0, im = 0;
    for (int b = 0; b < nb; ++b) {
        re += partial[(int64_t)col * nb + b].x;
        im += partial[(int64_t)col * nb + b].y;
    }
    out[col] = make_double2(re, im);
}

// w -= V[:, 0..ncol) h
__global__ void gs_update_kernel(const double2 *__restrict__ V, int64_t ldv, int ncol,
                                 const double2 *__restrict__ h, double2 *__restrict__ w, int64_t n,
                                 const int *__restrict__ stop) {
    if (stop && *stop) return;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double re = w[i].x, im = w[i].y;
    for (int c = 0; c < ncol; ++c) {
        const double2 v = V[(int64_t)c * ldv + i], hc = h[c];
        re -= v.x * hc.x - v.y * hc.y;
        im -= v.x * hc.y + v.y * hc.x;
    }
    w[i] = make_double2(re, im);
}

// y = a - b
__global__ void sub_kernel(const double2 *__restrict__ a, const double2 *__restrict__ b,
                           double2 *__restrict__ y, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = make_double2(a[i].x - b[i].x, a[i].y - b[i].y);
}

// x += sum_c V[:, c] yc  (yc in constant-size device array)
__global__ void combo_add_kernel(const double2 *__restrict__ V, int64_t ldv, int ncol,
                                 const double2 *__restrict__ yc, double2 *__restrict__ x, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double re = x[i].x, im = x[i].y;
    for (int c = 0; c < ncol; ++c) {
        const double2 v = V[(int64_t)c * ldv + i], y = yc[c];
        re += v.x * y.x - v.y * y.y;
        im += v.x * y.y + v.y * y.x;
    }
    x[i] = make_double2(re, im);
}

// ---- device-resident Arnoldi state (one GMRES cycle without host round trips)
// Layout in one device block: H (m+1) x m, g (m+1), sn (m), h1 (m+1), h2 (m+1),
// y (m) complex; cs (m) real; scalars.
struct GmScalars {
    double2 nrm2;      // output of the last norm reduction (|w|^2 in .x)
    double beta;       // residual norm at the start of the cycle
    double inv_beta;
    double inv_hn;     // 1 / h_{j+1,j} of the last step
    double res;        // |g_{j+1}| after the last step
    double tol;
    int done;          // 1: converged (or breakdown); later kernels of the cycle skip
    int start_ok;      // 1: the starting residual already met the tolerance
    int jdone;         // Arnoldi steps completed in this cycle
    int pad;
};
struct GmState {
    double2 *H, *g, *sn, *h1, *h2, *y;
    double *cs;
    GmScalars *s;
    int m;
};

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double cabs2(double2 a) { return hypot(a.x, a.y); }

// start of a cycle: beta = |w|, g = (beta, 0, ...), done = beta <= tol
__global__ void gm_init_kernel(GmState st, double tol) {
    GmScalars &s = *st.s;
    s.tol = tol;
    const double beta = sqrt(fmax(s.nrm2.x, 0.0));
    s.beta = beta;
    s.res = beta;
    s.jdone = 0;
    s.start_ok = beta <= s.tol ? 1 : 0;
    s.done = s.start_ok;
    s.inv_beta = beta > 0.0 ? 1.0 / beta : 0.0;
    for (int k = 0; k <= st.m; ++k) st.g[k] = make_double2(0.0, 0.0);
    st.g[0] = make_double2(beta, 0.0);
}

// Arnoldi step j: column j of H from the two Gram-Schmidt passes and |w|,
// previous rotations applied, new rotation, residual estimate, stop test.
// The rotation follows the host form used before (cs real, sn complex).
__global__ void gm_givens_kernel(GmState st, int j) {
    GmScalars &s = *st.s;
    if (s.done) return;
    const int ld = st.m + 1;
    double2 *col = st.H + (int64_t)j * ld;
    for (int k = 0; k <= j; ++k) col[k] = make_double2(st.h1[k].x + st.h2[k].x, st.h1[k].y + st.h2[k].y);
    const double hn = sqrt(fmax(s.nrm2.x, 0.0));
    col[j + 1] = make_double2(hn, 0.0);
    s.inv_hn = hn > 0.0 ? 1.0 / hn : 0.0;
    for (int k = 0; k < j; ++k) {
        const double c = st.cs[k];
        const double2 sn = st.sn[k];
        const double2 a = col[k], b = col[k + 1];
        const double2 t = make_double2(c * a.x + cmul(sn, b).x, c * a.y + cmul(sn, b).y);
        const double2 u = cmul(cconj(sn), a);
        col[k + 1] = make_double2(-u.x + c * b.x, -u.y + c * b.y);
        col[k] = t;
    }
    // rotation zeroing col[j + 1]
    const double2 a = col[j], b = col[j + 1];
    const double na = cabs2(a), nb = cabs2(b);
    double c;
    double2 sn, r;
    if (nb == 0.0) {
        c = 1.0;
        sn = make_double2(0.0, 0.0);
        r = a;
    } else if (na == 0.0) {
        c = 0.0;
        sn = make_double2(b.x / nb, -b.y / nb);
        r = make_double2(nb, 0.0);
    } else {
        const double nrm = hypot(na, nb);
        const double2 alpha = make_double2(a.x / na, a.y / na);
        c = na / nrm;
        const double2 t = cmul(alpha, cconj(b));
        sn = make_double2(t.x / nrm, t.y / nrm);
        r = make_double2(alpha.x * nrm, alpha.y * nrm);
    }
    st.cs[j] = c;
    st.sn[j] = sn;
    col[j] = r;
    col[j + 1] = make_double2(0.0, 0.0);
    const double2 gj = st.g[j], gj1 = st.g[j + 1];
    const double2 sg = cmul(sn, gj1);
    const double2 ug = cmul(cconj(sn), gj);
    st.g[j] = make_double2(c * gj.x + sg.x, c * gj.y + sg.y);
    st.g[j + 1] = make_double2(-ug.x + c * gj1.x, -ug.y + c * gj1.y);
    s.res = cabs2(st.g[j + 1]);
    s.jdone = j + 1;
    if (s.res <= s.tol || hn == 0.0) s.done = 1;
}

// y = R^{-1} g over the jdone columns (back substitution)
__global__ void gm_trisolve_kernel(GmState st) {
    const int j = st.s->jdone;
    const int ld = st.m + 1;
    for (int k = j - 1; k >= 0; --k) {
        double2 acc = st.g[k];
        for (int l = k + 1; l < j; ++l) {
            const double2 t = cmul(st.H[(int64_t)l * ld + k], st.y[l]);
            acc.x -= t.x;
            acc.y -= t.y;
        }
        const double2 d = st.H[(int64_t)k * ld + k];
        const double den = d.x * d.x + d.y * d.y;
        st.y[k] = make_double2((acc.x * d.x + acc.y * d.y) / den, (acc.y * d.x - acc.x * d.y) / den);
    }
}

// y = x * (*alpha) (alpha real, on the device)
__global__ void scale_dev_kernel(const double2 *__restrict__ x, const double *__restrict__ alpha,
                                 double2 *__restrict__ y, int64_t n, const int *__restrict__ stop) {
    if (stop && *stop) return;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const double a = *alpha;
    if (i < n) y[i] = make_double2(a * x[i].x, a * x[i].y);
}

// x += V[:, 0..*ncol) yc  (column count on the device)
__global__ void combo_add_dev_kernel(const double2 *__restrict__ V, int64_t ldv, const int *__restrict__ ncol,
                                     const double2 *__restrict__ yc, double2 *__restrict__ x, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int nc = *ncol;
    double re = x[i].x, im = x[i].y;
    for (int c = 0; c < nc; ++c) {
        const double2 v = V[(int64_t)c * ldv + i], y = yc[c];
        re += v.x * y.x - v.y * y.y;
        im += v.x * y.y + v.y * y.x;
    }
    x[i] = make_double2(re, im);
}

// ---- graph form: the whole (refined) solve as conditional graph nodes --------
// Control flow lives in device memory (RfState) and in conditional handles that
// single-thread kernels set; every loop has a counter bound, so each WHILE node
// ends even for NaN residuals.
struct RfState {
    double bnorm, tol;     // |b| and the absolute tolerance max(reltol |b|, abstol)
    double res;            // last outer residual |b - A x| (exact product)
    double inner_tol;      // absolute tolerance of the current inner solve
    double last_beta;      // residual norm at the start of the last cycle
    long long matvecs;
    int iters, restarts, refinements;
    int outer_zero;        // x == 0: the outer residual is b (its product skipped)
    int inner_zero;        // dx == 0: the cycle residual is the right-hand side
    int jmax;              // Arnoldi steps allowed in the current cycle
    int steps, cycles;     // loop counters (bounds of the WHILE nodes)
    int pad;
};

// out = *zero ? r : r - w   (out may be w)
__global__ void resid_flag_kernel(const double2 *__restrict__ r, const double2 *w, double2 *out, int64_t n,
                                  const int *__restrict__ zero) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double2 a = r[i];
    if (*zero) {
        out[i] = a;
    } else {
        const double2 b = w[i];
        out[i] = make_double2(a.x - b.x, a.y - b.y);
    }
}

// x += d
__global__ void axpy1_kernel(const double2 *__restrict__ d, double2 *__restrict__ x, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = make_double2(x[i].x + d[i].x, x[i].y + d[i].y);
}

// |b| from the norm reduction, tolerance, counters; enter the outer loop
__global__ void rf_start_kernel(GmState st, RfState *rf, double reltol, double abstol,
                                cudaGraphConditionalHandle h_outer) {
    RfState &r = *rf;
    const double bn = sqrt(fmax(st.s->nrm2.x, 0.0));
    r = RfState{};
    r.bnorm = bn;
    r.tol = fmax(reltol * bn, abstol);
    r.res = bn;
    r.last_beta = bn;
    r.outer_zero = 1;
    cudaGraphSetConditional(h_outer, 1u);
}

// Top of an outer pass.  Refinement: the outer residual |b - A x| decides
// whether another inner solve runs (the host loop of run_gmres); plain GMRES:
// one pass whose inner solve is the whole solve.
__global__ void rf_check_kernel(GmState st, RfState *rf, int refine, int maxiter, int max_outer,
                                double inner_rel, cudaGraphConditionalHandle h_outer,
                                cudaGraphConditionalHandle h_cycle) {
    RfState &r = *rf;
    if (refine) {
        if (!r.outer_zero) r.matvecs += 1;
        r.outer_zero = 0;
        const double res = sqrt(fmax(st.s->nrm2.x, 0.0));
        r.res = res;
        if (res <= r.tol || r.iters >= maxiter || r.refinements >= max_outer) {
            cudaGraphSetConditional(h_outer, 0u);
            cudaGraphSetConditional(h_cycle, 0u);
            return;
        }
        r.refinements += 1;
        r.inner_tol = fmax(inner_rel * res, r.tol * 0.5);
    } else {
        r.inner_tol = r.tol;
        cudaGraphSetConditional(h_outer, 0u);
    }
    r.inner_zero = 1;
    r.cycles = 0;
    cudaGraphSetConditional(h_cycle, 1u);
}

// Start of a restart cycle (gm_init_kernel with the inner tolerance read from
// the device); opens the Arnoldi loop unless the true residual already meets it.
__global__ void gm_cycle_init_kernel(GmState st, RfState *rf, int maxiter, int restart,
                                     cudaGraphConditionalHandle h_step, cudaGraphConditionalHandle h_sel) {
    GmScalars &s = *st.s;
    RfState &r = *rf;
    s.tol = r.inner_tol;
    const double beta = sqrt(fmax(s.nrm2.x, 0.0));
    s.beta = beta;
    s.res = beta;
    s.jdone = 0;
    s.start_ok = beta <= s.tol ? 1 : 0;
    s.done = s.start_ok;
    s.inv_beta = beta > 0.0 ? 1.0 / beta : 0.0;
    for (int k = 0; k <= st.m; ++k) st.g[k] = make_double2(0.0, 0.0);
    st.g[0] = make_double2(beta, 0.0);
    if (!r.inner_zero) r.matvecs += 1;
    r.inner_zero = 0;
    r.last_beta = beta;
    r.jmax = min(restart, max(0, maxiter - r.iters));
    r.steps = 0;
    cudaGraphSetConditional(h_step, (!s.start_ok && r.jmax > 0) ? 1u : 0u);
    cudaGraphSetConditional(h_sel, 0u);
}

// After each Arnoldi step: the next step index, and whether it runs (not
// converged, steps left in the cycle; at most `restart` passes)
__global__ void gm_step_guard_kernel(GmState st, RfState *rf, int restart, cudaGraphConditionalHandle h_step,
                                     cudaGraphConditionalHandle h_sel) {
    const GmScalars &s = *st.s;
    RfState &r = *rf;
    r.steps += 1;
    const int jd = s.jdone;
    cudaGraphSetConditional(h_step, (!s.done && jd < r.jmax && r.steps < restart) ? 1u : 0u);
    cudaGraphSetConditional(h_sel, (unsigned)jd);
}

// End of a cycle: tallies; another cycle (whose first action re-checks the true
// residual) follows any cycle that took steps
__global__ void gm_cycle_end_kernel(GmState st, RfState *rf, int maxiter, cudaGraphConditionalHandle h_cycle) {
    RfState &r = *rf;
    const int jd = st.s->jdone;
    r.iters += jd;
    r.matvecs += jd;
    if (jd > 0) r.restarts += 1;
    r.cycles += 1;
    cudaGraphSetConditional(h_cycle, (jd > 0 && r.cycles <= maxiter) ? 1u : 0u);
}

__global__ void rf_final_kernel(const RfState *rf, int refine, bie_gmres_info *out) {
    const RfState &r = *rf;
    bie_gmres_info o{};
    o.iterations = r.iters;
    o.restarts = r.restarts;
    o.refinements = refine ? r.refinements : 0;
    o.matvecs = r.matvecs;
    o.residual_norm = refine ? r.res : r.last_beta;
    o.rhs_norm = r.bnorm;
    o.converged = o.residual_norm <= r.tol ? 1 : 0;
    *out = o;
}

__global__ void round_c64_kernel(const double2 *__restrict__ in, float2 *__restrict__ out, int64_t n) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        out[i] = make_float2((float)in[i].x, (float)in[i].y);
}

inline unsigned blocks(int64_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

// Column slices of a dense product: as many as make one resident wave of
// blocks (the kernel's occupancy x the SMs) over the row tiles, so that no
// partial second wave trails the product (7842-node complex64 matrix: 5.1 ->
// 6.1 TB/s against a fixed 8 blocks per SM).
constexpr int kMaxSlices = 64;
inline int gemv_slices(const void *kern, int64_t rows, int num_sms) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kT, 0) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    const int64_t tiles = (rows + kT - 1) / kT;
    return (int)std::max<int64_t>(1, std::min<int64_t>(kMaxSlices, (int64_t)per_sm * num_sms / tiles));
}

// ---------------------------------------------------------------------------
// Operator application and BLAS-1 helpers bound to a context
// ---------------------------------------------------------------------------
struct Solver {
    Ctx &c;
    int64_t n;
    int m;                        // restart length
    double2 *part = nullptr;      // gemv slices / multidot partials
    int nbdot = 1;
    double2 *hdev = nullptr;      // device scratch for dot results (>= restart + 2)
    std::vector<double2> hhost;
    GmState st{};                 // device-resident Arnoldi state
    RfState *rf = nullptr;        // device-resident refinement state (graph form)
    const int *stop = nullptr;    // device stop flag honoured by the launches below
    cudaStream_t stream;          // launch stream (a capture stream while recording a graph)
    DevOp *devop = nullptr;       // operator applied through DevOp::apply (else bie_operator)

    // level > 0: the workspace of a solve nested inside another solve's product
    Solver(Ctx &ctx, int64_t n_, int restart, int level = 0)
        : c(ctx), n(n_), m(restart), stream(ctx.stream) {
        const int part_slot = level == 0 ? kScratchSolverPart : kScratchSolverNested + 2 * (level - 1) + 1;
        // dot-product blocks per column; vectors up to 4096 entries take one
        // block per column, which writes its result directly (no second launch)
        nbdot = n <= 4096 ? 1 : (int)std::min<int64_t>(std::max<int64_t>(1, (n + kT * 8 - 1) / (kT * 8)), 256);
        const size_t part_bytes = (size_t)std::max<int64_t>(kMaxSlices * n, (int64_t)(restart + 2) * nbdot) * 16;
        const size_t hbytes = (size_t)(restart + 2) * 16;
        const size_t nc = (size_t)(restart + 1) * restart + 4 * (size_t)(restart + 1) + restart;
        const size_t st_bytes = nc * 16 + (size_t)restart * 8 + sizeof(GmScalars) + sizeof(RfState) + 96;
        char *base = static_cast<char *>(c.scratch(part_slot, part_bytes + hbytes + st_bytes));
        part = reinterpret_cast<double2 *>(base);
        hdev = reinterpret_cast<double2 *>(base + part_bytes);
        double2 *z = reinterpret_cast<double2 *>(base + part_bytes + hbytes);
        st.m = restart;
        st.H = z;
        z += (size_t)(restart + 1) * restart;
        st.g = z;
        z += restart + 1;
        st.sn = z;
        z += restart;
        st.h1 = z;
        z += restart + 1;
        st.h2 = z;
        z += restart + 1;
        st.y = z;
        z += restart + 1;
        st.cs = reinterpret_cast<double *>(z);
        st.s = reinterpret_cast<GmScalars *>(reinterpret_cast<char *>(st.cs) + (((size_t)restart * 8 + 15) & ~size_t(15)));
        rf = reinterpret_cast<RfState *>(reinterpret_cast<char *>(st.s) + ((sizeof(GmScalars) + 15) & ~size_t(15)));
        hhost.resize(restart + 2);
    }

    void launched() { ++c.kernel_launches; }

    // y = s (K x) + d .* x   (dense kernels skip when *stop is set)
    void apply(const bie_operator &op, int precision, const double2 *x, double2 *y) {
        if (devop) {
            devop->apply(x, y, stop);
            return;
        }
        const double2 sc = make_double2(op.scale_re, op.scale_im);
        const double2 *d = reinterpret_cast<const double2 *>(op.diag);
        if (op.kind == BIE_OP_DENSE) {
            cudaEvent_t t0 = c.timer_begin();
            int S = 1;
            if (op.A32 && (precision == BIE_PREC_MIXED || !op.A)) {
                // complex64 operator: the fast product for mixed iterations, the
                // exact one where FP64 arithmetic was asked for (residuals of
                // refinement, right-hand sides) and no complex128 matrix exists
                const bool exact = precision != BIE_PREC_MIXED;
                if (n % 2 == 0) {
                    if (exact) {
                        S = gemv_slices((const void *)dense_gemv_c64_exact_kernel, n / 2, c.num_sms);
                        dense_gemv_c64_exact_kernel<<<dim3(blocks(n / 2, kT), (unsigned)S), kT, 0, stream>>>(
                            reinterpret_cast<const float4 *>(op.A32), n, x, part, S, stop);
                    } else {
                        S = gemv_slices((const void *)dense_gemv_c64_kernel, n / 2, c.num_sms);
                        dense_gemv_c64_kernel<<<dim3(blocks(n / 2, kT), (unsigned)S), kT, 0, stream>>>(
                            reinterpret_cast<const float4 *>(op.A32), n, x, part, S, stop);
                    }
                } else {
                    if (exact) {
                        S = gemv_slices((const void *)dense_gemv_c64_rows_exact_kernel, n, c.num_sms);
                        dense_gemv_c64_rows_exact_kernel<<<dim3(blocks(n, kT), (unsigned)S), kT, 0, stream>>>(
                            reinterpret_cast<const float2 *>(op.A32), n, x, part, S, stop);
                    } else {
                        S = gemv_slices((const void *)dense_gemv_c64_rows_kernel, n, c.num_sms);
                        dense_gemv_c64_rows_kernel<<<dim3(blocks(n, kT), (unsigned)S), kT, 0, stream>>>(
                            reinterpret_cast<const float2 *>(op.A32), n, x, part, S, stop);
                    }
                }
            } else {
                S = gemv_slices((const void *)dense_gemv_kernel<double2>, n, c.num_sms);
                dense_gemv_kernel<double2><<<dim3(blocks(n, kT), (unsigned)S), kT, 0, stream>>>(
                    reinterpret_cast<const double2 *>(op.A), n, x, part, S, stop);
            }
            BIE_CUDA(cudaGetLastError());
            c.timer_end(t0);
            launched();
            combine_kernel<<<blocks(n), 256, 0, stream>>>(part, S, n, sc, d, x, y, stop);
            BIE_CUDA(cudaGetLastError());
            launched();
        } else {
            // matrix-free F x (or the fast operator) into y, then y = s y + d .* x
            // (these products do not look at the stop flag: the caller checks it
            // on the host after every step)
            if (op.kind == BIE_OP_FAST) {
                FastOp &f = *const_cast<FastOp *>(reinterpret_cast<const FastOp *>(op.fast));
                apply_fastop(f, reinterpret_cast<const double *>(x), reinterpret_cast<double *>(y), precision,
                             nullptr, 0);
            } else {
                MatvecArgs mv{op.k_re, op.k_im, c.d_sources, n, reinterpret_cast<const double *>(x),
                              nullptr, reinterpret_cast<double *>(y), nullptr, precision};
                launch_matvec(c, mv);
            }
            combine_kernel<<<blocks(n), 256, 0, c.stream>>>(y, 1, n, sc, d, x, y, stop);
            BIE_CUDA(cudaGetLastError());
            launched();
        }
    }

    // out[0..ncol) = V[:, 0..ncol)^H w on the device (no host copy)
    void multidot_dev(const double2 *V, int64_t ldv, int ncol, const double2 *w, double2 *out) {
        dim3 grid((unsigned)nbdot, (unsigned)ncol);
        multidot_kernel<<<grid, kT, 0, stream>>>(V, ldv, w, n, nbdot == 1 ? out : part, stop);
        BIE_CUDA(cudaGetLastError());
        launched();
        if (nbdot == 1) return;   // partial[col] is the sum already
        sum_partials_kernel<<<blocks(ncol, 64), 64, 0, stream>>>(part, nbdot, ncol, out, stop);
        BIE_CUDA(cudaGetLastError());
        launched();
    }

    // out[0..ncol) = V[:, 0..ncol)^H w  (copied to host)
    void multidot(const double2 *V, int64_t ldv, int ncol, const double2 *w, std::vector<cplx> &out) {
        multidot_dev(V, ldv, ncol, w, hdev);
        BIE_CUDA(cudaMemcpyAsync(hhost.data(), hdev, ncol * sizeof(double2), cudaMemcpyDeviceToHost, c.stream));
        BIE_CUDA(cudaStreamSynchronize(c.stream));
        out.resize(ncol);
        for (int k = 0; k < ncol; ++k) out[k] = cplx(hhost[k].x, hhost[k].y);
    }

    double norm(const double2 *w) {
        std::vector<cplx> o;
        multidot(w, n, 1, w, o);
        return std::sqrt(std::max(o[0].real(), 0.0));
    }

    void upload_coeffs(const std::vector<cplx> &h) {
        for (size_t k = 0; k < h.size(); ++k) hhost[k] = make_double2(h[k].real(), h[k].imag());
        BIE_CUDA(cudaMemcpyAsync(hdev, hhost.data(), h.size() * sizeof(double2), cudaMemcpyHostToDevice,
                                 c.stream));
    }

    // w -= V[:, 0..ncol) h  with h on the device
    void gs_update_dev(const double2 *V, int64_t ldv, int ncol, double2 *w, const double2 *h) {
        gs_update_kernel<<<blocks(n), 256, 0, stream>>>(V, ldv, ncol, h, w, n, stop);
        BIE_CUDA(cudaGetLastError());
        launched();
    }

    void combo_add(const double2 *V, int64_t ldv, int ncol, const std::vector<cplx> &y, double2 *x) {
        upload_coeffs(y);
        combo_add_kernel<<<blocks(n), 256, 0, c.stream>>>(V, ldv, ncol, hdev, x, n);
        BIE_CUDA(cudaGetLastError());
        launched();
    }

    void scale_dev(const double2 *x, const double *a, double2 *y) {
        scale_dev_kernel<<<blocks(n), 256, 0, stream>>>(x, a, y, n, stop);
        BIE_CUDA(cudaGetLastError());
        launched();
    }

    void sub(const double2 *a, const double2 *b, double2 *y) {
        sub_kernel<<<blocks(n), 256, 0, stream>>>(a, b, y, n);
        BIE_CUDA(cudaGetLastError());
        launched();
    }
};

// One GMRES solve of A x = b from the initial x (device), operator precision
// `prec`; returns the number of iterations; `tol` is an absolute tolerance on
// the residual norm.  V: (restart + 1) x n workspace.
//
// Each restart cycle runs on the device without host round trips: the
// Gram-Schmidt coefficients, the Hessenberg column, the Givens rotations and
// the residual estimate stay in device memory (GmState), a single-thread
// kernel decides convergence and raises a stop flag, and every later kernel of
// the cycle returns at once when it sees the flag.  The host reads the state
// once per cycle (dense operators) or once per step (matrix-free and fast
// operators, whose products do not look at the flag).
int gmres_core(Solver &S, const bie_operator &op, int prec, const double2 *b, double2 *x,
               bool x_zero, double2 *V, double2 *w, int restart, int maxiter, double tol,
               double *res_out, int *restarts_out, int64_t *matvecs) {
    const int64_t n = S.n;
    const bool dense = S.devop ? S.devop->honours_stop() : op.kind == BIE_OP_DENSE;
    const GmState st = S.st;
    const int *stop_flag = &st.s->done;
    cudaStream_t stream = S.stream;
    int it = 0, restarts = 0;
    double beta = 0.0;
    bool first = true;
    GmScalars hs{};
    while (true) {
        // r = b - A x  (r = b for a zero start), beta = |r|
        S.stop = nullptr;
        if (first && x_zero) {
            BIE_CUDA(cudaMemcpyAsync(w, b, (size_t)n * 16, cudaMemcpyDeviceToDevice, stream));
        } else {
            S.apply(op, prec, x, w);
            ++*matvecs;
            S.sub(b, w, w);
        }
        first = false;
        S.multidot_dev(w, n, 1, w, &st.s->nrm2);
        gm_init_kernel<<<1, 1, 0, stream>>>(st, tol);
        BIE_CUDA(cudaGetLastError());
        S.launched();
        const int jmax = std::min(restart, std::max(0, maxiter - it));
        BIE_CUDA(cudaMemcpyAsync(&hs, st.s, sizeof(GmScalars), cudaMemcpyDeviceToHost, stream));
        BIE_CUDA(cudaStreamSynchronize(stream));
        if (hs.start_ok || jmax == 0) {
            beta = hs.beta;
            break;
        }
        S.stop = stop_flag;
        S.scale_dev(w, &st.s->inv_beta, V);
        for (int j = 0; j < jmax; ++j) {
            const double2 *vj = V + (int64_t)j * n;
            double2 *vn = V + (int64_t)(j + 1) * n;
            S.apply(op, prec, vj, w);
            // CGS2
            S.multidot_dev(V, n, j + 1, w, st.h1);
            S.gs_update_dev(V, n, j + 1, w, st.h1);
            S.multidot_dev(V, n, j + 1, w, st.h2);
            S.gs_update_dev(V, n, j + 1, w, st.h2);
            S.multidot_dev(w, n, 1, w, &st.s->nrm2);
            gm_givens_kernel<<<1, 1, 0, stream>>>(st, j);
            BIE_CUDA(cudaGetLastError());
            S.launched();
            S.scale_dev(w, &st.s->inv_hn, vn);
            // the host looks at the stop flag after every step for operators whose
            // products ignore it, every kCheck steps for dense ones (at most
            // kCheck - 1 skipped steps are queued after convergence)
            constexpr int kCheck = 4;
            if (!dense || j % kCheck == kCheck - 1) {
                int done = 0;
                BIE_CUDA(cudaMemcpyAsync(&done, stop_flag, sizeof(int), cudaMemcpyDeviceToHost, stream));
                BIE_CUDA(cudaStreamSynchronize(stream));
                if (done) break;
            }
        }
        // x += V y,  R y = g
        S.stop = nullptr;
        gm_trisolve_kernel<<<1, 1, 0, stream>>>(st);
        BIE_CUDA(cudaGetLastError());
        combo_add_dev_kernel<<<blocks(n), 256, 0, stream>>>(V, n, &st.s->jdone, st.y, x, n);
        BIE_CUDA(cudaGetLastError());
        S.launched();
        S.launched();
        BIE_CUDA(cudaMemcpyAsync(&hs, st.s, sizeof(GmScalars), cudaMemcpyDeviceToHost, stream));
        BIE_CUDA(cudaStreamSynchronize(stream));
        it += hs.jdone;
        *matvecs += hs.jdone;
        ++restarts;
    }
    *res_out = beta;
    *restarts_out = restarts;
    return it;
}

}  // namespace

// A conditional handle of the graph being captured on `s`.
cudaGraphConditionalHandle graph_new_handle(cudaStream_t s) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaGraph_t g = nullptr;
    BIE_CUDA(cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, nullptr, nullptr, nullptr));
    if (cs != cudaStreamCaptureStatusActive) fail(BIE_ERR_INVALID, "graph GMRES: the stream is not capturing");
    cudaGraphConditionalHandle h;
    BIE_CUDA(cudaGraphConditionalHandleCreate(&h, g, 0, 0));
    return h;
}

// Appends a conditional node after the capture's current dependencies; its body
// graphs are returned for capture on other streams.
void graph_add_conditional(cudaStream_t s, cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type,
                           unsigned size, cudaGraph_t *bodies) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    size_t nd = 0;
    BIE_CUDA(cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, &deps, nullptr, &nd));
    if (cs != cudaStreamCaptureStatusActive) fail(BIE_ERR_INVALID, "graph GMRES: the stream is not capturing");
    cudaGraphNodeParams p{};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = type;
    p.conditional.size = size;
    cudaGraphNode_t node;
    BIE_CUDA(cudaGraphAddNode(&node, g, deps, nullptr, nd, &p));
    BIE_CUDA(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    for (unsigned i = 0; i < size; ++i) bodies[i] = p.conditional.phGraph_out[i];
}

void capture_gmres(Ctx &c, const bie_operator &op, const double *b_, double *x_, const bie_gmres_opts &o,
                   bie_gmres_info *d_info, const cudaStream_t *body) {
    if (op.kind != BIE_OP_DENSE) fail(BIE_ERR_UNSUPPORTED, "graph GMRES needs a dense operator");
    if (o.initially_nonzero) fail(BIE_ERR_UNSUPPORTED, "graph GMRES starts from x = 0");
    const int64_t n = c.n_sources;
    const int restart = (int)std::max<int64_t>(1, std::min<int64_t>(o.restart > 0 ? o.restart : 20, n));
    if (restart > kGraphMaxRestart) fail(BIE_ERR_UNSUPPORTED, "graph GMRES: restart above 64");
    const int maxiter = o.maxiter > 0 ? o.maxiter : (int)std::min<int64_t>(n, INT32_MAX);
    const double reltol = o.reltol > 0 ? o.reltol : std::sqrt(2.220446049250313e-16);
    const double abstol = std::max(0.0, o.abstol);
    const bool refine = o.refine != 0;
    const int prec = refine ? BIE_PREC_MIXED : o.precision;
    const double inner_rel = o.inner_reltol > 0 ? o.inner_reltol : 1e-4;
    const int max_outer = o.max_refine > 0 ? o.max_refine : 10;
    const double2 *b = reinterpret_cast<const double2 *>(b_);
    double2 *x = reinterpret_cast<double2 *>(x_);

    char *ws = static_cast<char *>(c.scratch(kScratchSolver, (size_t)(restart + 4) * n * 16));
    double2 *V = reinterpret_cast<double2 *>(ws);
    double2 *w = V + (int64_t)(restart + 1) * n;
    double2 *rr = w + n;
    double2 *dx = rr + n;
    Solver S(c, n, restart);
    const GmState st = S.st;
    RfState *rf = S.rf;
    cudaStream_t s0 = c.stream;

    BIE_CUDA(cudaMemsetAsync(x, 0, (size_t)n * 16, s0));
    S.multidot_dev(b, n, 1, b, &st.s->nrm2);
    const cudaGraphConditionalHandle h_outer = graph_new_handle(s0);
    rf_start_kernel<<<1, 1, 0, s0>>>(st, rf, reltol, abstol, h_outer);
    BIE_CUDA(cudaGetLastError());
    S.launched();
    cudaGraph_t g_outer;
    graph_add_conditional(s0, h_outer, cudaGraphCondTypeWhile, 1, &g_outer);
    {
        // outer pass: refinement residual rr = b - A x (exact product), then the
        // inner restarted GMRES on A dx = rr
        BodyCapture bc1(body[0], g_outer);
        S.stream = body[0];
        if (refine) {
            S.stop = &rf->outer_zero;
            S.apply(op, o.precision == BIE_PREC_DF64 ? BIE_PREC_DF64 : BIE_PREC_FP64, x, w);
            S.stop = nullptr;
            resid_flag_kernel<<<blocks(n), 256, 0, S.stream>>>(b, w, rr, n, &rf->outer_zero);
            BIE_CUDA(cudaGetLastError());
            S.launched();
            S.multidot_dev(rr, n, 1, rr, &st.s->nrm2);
            BIE_CUDA(cudaMemsetAsync(dx, 0, (size_t)n * 16, S.stream));
        }
        const double2 *rhs = refine ? rr : b;
        double2 *sol = refine ? dx : x;
        const cudaGraphConditionalHandle h_cycle = graph_new_handle(S.stream);
        rf_check_kernel<<<1, 1, 0, S.stream>>>(st, rf, refine ? 1 : 0, maxiter, max_outer, inner_rel, h_outer,
                                                h_cycle);
        BIE_CUDA(cudaGetLastError());
        S.launched();
        cudaGraph_t g_cycle;
        graph_add_conditional(S.stream, h_cycle, cudaGraphCondTypeWhile, 1, &g_cycle);
        {
            // restart cycle: w = rhs - A sol (rhs itself on the first cycle), beta,
            // then up to `restart` Arnoldi steps
            BodyCapture bc2(body[1], g_cycle);
            S.stream = body[1];
            S.stop = &rf->inner_zero;
            S.apply(op, prec, sol, w);
            S.stop = nullptr;
            resid_flag_kernel<<<blocks(n), 256, 0, S.stream>>>(rhs, w, w, n, &rf->inner_zero);
            BIE_CUDA(cudaGetLastError());
            S.launched();
            S.multidot_dev(w, n, 1, w, &st.s->nrm2);
            const cudaGraphConditionalHandle h_step = graph_new_handle(S.stream);
            const cudaGraphConditionalHandle h_sel = graph_new_handle(S.stream);
            gm_cycle_init_kernel<<<1, 1, 0, S.stream>>>(st, rf, maxiter, restart, h_step, h_sel);
            BIE_CUDA(cudaGetLastError());
            S.launched();
            S.scale_dev(w, &st.s->inv_beta, V);
            cudaGraph_t g_step;
            graph_add_conditional(S.stream, h_step, cudaGraphCondTypeWhile, 1, &g_step);
            {
                // one Arnoldi step per pass: a switch over the step index j runs
                // the body recorded for that j (CGS2 over j + 1 basis vectors)
                BodyCapture bc3(body[2], g_step);
                S.stream = body[2];
                std::vector<cudaGraph_t> branch(restart);
                graph_add_conditional(S.stream, h_sel, cudaGraphCondTypeSwitch, (unsigned)restart, branch.data());
                gm_step_guard_kernel<<<1, 1, 0, S.stream>>>(st, rf, restart, h_step, h_sel);
                BIE_CUDA(cudaGetLastError());
                S.launched();
                for (int j = 0; j < restart; ++j) {
                    BodyCapture bc4(body[3], branch[j]);
                    S.stream = body[3];
                    const double2 *vj = V + (int64_t)j * n;
                    double2 *vn = V + (int64_t)(j + 1) * n;
                    S.apply(op, prec, vj, w);
                    S.multidot_dev(V, n, j + 1, w, st.h1);
                    S.gs_update_dev(V, n, j + 1, w, st.h1);
                    S.multidot_dev(V, n, j + 1, w, st.h2);
                    S.gs_update_dev(V, n, j + 1, w, st.h2);
                    S.multidot_dev(w, n, 1, w, &st.s->nrm2);
                    gm_givens_kernel<<<1, 1, 0, S.stream>>>(st, j);
                    BIE_CUDA(cudaGetLastError());
                    S.launched();
                    S.scale_dev(w, &st.s->inv_hn, vn);
                    bc4.end();
                }
                bc3.end();
            }
            S.stream = body[1];
            gm_trisolve_kernel<<<1, 1, 0, S.stream>>>(st);
            BIE_CUDA(cudaGetLastError());
            combo_add_dev_kernel<<<blocks(n), 256, 0, S.stream>>>(V, n, &st.s->jdone, st.y, sol, n);
            BIE_CUDA(cudaGetLastError());
            gm_cycle_end_kernel<<<1, 1, 0, S.stream>>>(st, rf, maxiter, h_cycle);
            BIE_CUDA(cudaGetLastError());
            S.launched();
            S.launched();
            S.launched();
            bc2.end();
        }
        S.stream = body[0];
        if (refine) {
            axpy1_kernel<<<blocks(n), 256, 0, S.stream>>>(dx, x, n);
            BIE_CUDA(cudaGetLastError());
            S.launched();
        }
        bc1.end();
    }
    S.stream = s0;
    rf_final_kernel<<<1, 1, 0, s0>>>(rf, refine ? 1 : 0, d_info);
    BIE_CUDA(cudaGetLastError());
    S.launched();
}

namespace {

// The restarted (optionally refined) GMRES behind run_gmres and run_gmres_devop.
void gmres_solve(Ctx &c, const bie_operator &op, DevOp *devop, int64_t n, int level, const double *b_,
                 double *x_, const bie_gmres_opts &o, bie_gmres_info &info) {
    if (level < 0 || level > kMaxSolveLevel) fail(BIE_ERR_INVALID, "GMRES nesting deeper than two levels");
    const int restart = (int)std::max<int64_t>(1, std::min<int64_t>(o.restart > 0 ? o.restart : 20, n));
    const int maxiter = o.maxiter > 0 ? o.maxiter : (int)std::min<int64_t>(n, INT32_MAX);
    const double reltol = o.reltol > 0 ? o.reltol : std::sqrt(2.220446049250313e-16);
    const double abstol = std::max(0.0, o.abstol);
    const double2 *b = reinterpret_cast<const double2 *>(b_);
    double2 *x = reinterpret_cast<double2 *>(x_);

    // workspace: V (restart + 1) x n, w, r, dx
    const int ws_slot = level == 0 ? kScratchSolver : kScratchSolverNested + 2 * (level - 1);
    char *ws = static_cast<char *>(c.scratch(ws_slot, (size_t)(restart + 4) * n * 16));
    double2 *V = reinterpret_cast<double2 *>(ws);
    double2 *w = V + (int64_t)(restart + 1) * n;
    double2 *rr = w + n;
    double2 *dx = rr + n;
    Solver S(c, n, restart, level);
    S.devop = devop;
    const double bnorm = S.norm(b);
    const double tol = std::max(reltol * bnorm, abstol);
    if (!o.initially_nonzero) BIE_CUDA(cudaMemsetAsync(x, 0, (size_t)n * 16, c.stream));
    int64_t matvecs = 0;
    int iters = 0, restarts = 0;
    double res = 0;
    int outer = 0;
    if (!o.refine) {
        const int prec = o.precision;
        iters = gmres_core(S, op, prec, b, x, !o.initially_nonzero, V, w, restart, maxiter, tol, &res,
                           &restarts, &matvecs);
    } else {
        // iterative refinement: r = b - A x in FP64; inner solve A_low dx = r
        const double inner_rel = o.inner_reltol > 0 ? o.inner_reltol : 1e-4;
        const int max_outer = o.max_refine > 0 ? o.max_refine : 10;
        bie_operator low = op;
        for (outer = 0; outer < max_outer; ++outer) {
            S.apply(op, o.precision == BIE_PREC_DF64 ? BIE_PREC_DF64 : BIE_PREC_FP64, x, w);
            ++matvecs;
            S.sub(b, w, rr);
            res = S.norm(rr);
            if (res <= tol || iters >= maxiter) break;
            BIE_CUDA(cudaMemsetAsync(dx, 0, (size_t)n * 16, c.stream));
            double ires = 0;
            int irs = 0;
            iters += gmres_core(S, low, BIE_PREC_MIXED, rr, dx, true, V, w, restart, maxiter - iters,
                                std::max(inner_rel * res, tol * 0.5), &ires, &irs, &matvecs);
            restarts += irs;
            // x += dx
            std::vector<cplx> one{cplx(1.0, 0.0)};
            S.combo_add(dx, n, 1, one, x);
        }
    }
    BIE_CUDA(cudaStreamSynchronize(c.stream));
    info.iterations = iters;
    info.restarts = restarts;
    info.refinements = outer;
    info.matvecs = matvecs;
    info.residual_norm = res;
    info.rhs_norm = bnorm;
    info.converged = res <= tol ? 1 : 0;
}

}  // namespace

void run_gmres(Ctx &c, const bie_operator &op, const double *b, double *x, const bie_gmres_opts &o,
               bie_gmres_info &info) {
    gmres_solve(c, op, nullptr, c.n_sources, 0, b, x, o, info);
}

void run_gmres_devop(Ctx &c, DevOp &op, const double *b, double *x, const bie_gmres_opts &o,
                     bie_gmres_info &info, int level) {
    bie_gmres_opts plain = o;
    plain.refine = 0;   // one arithmetic: the operator's own
    bie_operator none{};
    none.kind = -1;
    gmres_solve(c, none, &op, op.size(), level, b, x, plain, info);
}

void apply_operator(Ctx &c, const bie_operator &op, int precision, const double *x, double *y) {
    Solver S(c, c.n_sources, 1);
    S.apply(op, precision, reinterpret_cast<const double2 *>(x), reinterpret_cast<double2 *>(y));
}

void round_to_c64(Ctx &c, const double *in, float *out, int64_t n) {
    round_c64_kernel<<<(unsigned)std::min<int64_t>((n + 255) / 256, 64LL * c.num_sms), 256, 0, c.stream>>>(
        reinterpret_cast<const double2 *>(in), reinterpret_cast<float2 *>(out), n);
    BIE_CUDA(cudaGetLastError());
    ++c.kernel_launches;
}

}  // namespace bie
