// K7: adjoint gradient of a far-field objective with respect to vertex
// positions and per-element boundary impedance (bie_adjoint).
//
// Forward model (3-node triangles with nodal physics on the vertices, the
// configuration of the shape/impedance study):
//   A p = p_I,   A = F + Diagonal(1 - C) - i rho c k G_Y,
//   G_Y[i, a] = sum_e Y_e G^(e)[i, a],  Y_e = 1 / Z_e  (element admittance),
// i.e. the boundary integral equation of README.md:10-18 with the impedance
// condition v_n = p / Z on each element, F, G, C as assembled by
// assemble_parallel! (src/3d/assembly_collocation.jl:270-353) and the
// exterior collocation form of test/3d/assembly_test.jl:37.  The reference's
// closest impedance form is nodal (examples/3d_cube_wave_anechoic.jl:62-68);
// the per-element admittance is defined here.
//   p_f = p_I(x_f) + B p,   B = -F_x + i rho c k G_{x,Y}   (field points x_f),
//   J = sum_j |p_f(x_j)|^2,  p_I(x) = exp(-i k d.x)  (incoming_wave,
//   src/analytical/3d_scattering.jl:4-12).
// Adjoint: A^H lambda = B^H p_f, then
//   dJ = 2 Re[ p_f^H dB p - lambda^H dA p + lambda^H dp_I ].
// The reverse pass recomputes the quadrature of every (row, element) pair
// with the forward rule choice (the nearest-node rule is piecewise constant
// in the geometry) and accumulates analytic derivatives of the integrands
// with respect to the element vertices, the collocation point and Y_e.
// FP64 throughout.
#include "bie_internal.h"
#include "bie_device.cuh"
#include "bie_df64.cuh"

#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

namespace bie {

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr int kT = 128;

struct cd {
    double re, im;
};
__device__ __forceinline__ cd cmul(cd a, cd b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__device__ __forceinline__ cd cadd(cd a, cd b) { return {a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ cd cscale(cd a, double s) { return {a.re * s, a.im * s}; }
__device__ __forceinline__ cd cconj(cd a) { return {a.re, -a.im}; }

// ---------------------------------------------------------------------------
// small kernels of the driver
// ---------------------------------------------------------------------------
__global__ void admittance_kernel(const double2 *__restrict__ Z, const int32_t *__restrict__ order,
                                  int64_t E, double2 *__restrict__ Y) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= E) return;
    const double2 z = Z[order[p]];
    const double den = z.x * z.x + z.y * z.y;
    Y[p] = make_double2(z.x / den, -z.y / den);
}

// A = F + a G (in place in F), A_ii += 1 - C_i  (diag only when C != null)
__global__ void combine_system_kernel(double2 *__restrict__ F, const double2 *__restrict__ G,
                                      double2 a, const double2 *__restrict__ C, int64_t M,
                                      int64_t N) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < M * N; t += stride) {
        const double2 f = F[t], g = G[t];
        double re = f.x + a.x * g.x - a.y * g.y, im = f.y + a.x * g.y + a.y * g.x;
        if (C) {
            const int64_t i = t % M, j = t / M;
            if (i == j) {
                re += 1.0 - C[i].x;
                im += -C[i].y;
            }
        }
        F[t] = make_double2(re, im);
    }
}

// p_I(x) = exp(-i k d.x) at n points (3 x n)
__global__ void incident_kernel(const double *__restrict__ X, int64_t n, double kre, double kim,
                                double dx, double dy, double dz, double2 *__restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double s = dx * X[3 * i] + dy * X[3 * i + 1] + dz * X[3 * i + 2];
    // -i k s = kim s - i kre s
    const double mag = exp(kim * s);
    double sn, cs;
    sincos(-kre * s, &sn, &cs);
    out[i] = make_double2(mag * cs, mag * sn);
}

// y[i] = b0[i] + sum_j B[i + j M] p[j]   (M small), one warp per row
__global__ void small_gemv_kernel(const double2 *__restrict__ B, int64_t M, int64_t N,
                                  const double2 *__restrict__ p, const double2 *__restrict__ b0,
                                  double2 *__restrict__ y) {
    const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= M) return;
    double re = 0, im = 0;
    for (int64_t j = lane; j < N; j += 32) {
        const double2 b = B[row + j * M], v = p[j];
        re += b.x * v.x - b.y * v.y;
        im += b.x * v.y + b.y * v.x;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        re += __shfl_xor_sync(0xffffffffu, re, o);
        im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    if (lane == 0) y[row] = make_double2(b0[row].x + re, b0[row].y + im);
}

// r[j] = sum_i conj(B[i + j M]) pf[i]   (B^H pf), one thread per column
__global__ void adjoint_rhs_kernel(const double2 *__restrict__ B, int64_t M, int64_t N,
                                   const double2 *__restrict__ pf, double2 *__restrict__ r) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N) return;
    double re = 0, im = 0;
    for (int64_t i = 0; i < M; ++i) {
        const double2 b = B[i + j * M], v = pf[i];
        re += b.x * v.x + b.y * v.y;
        im += b.x * v.y - b.y * v.x;
    }
    r[j] = make_double2(re, im);
}

// At = A^H (N x N column-major), 32 x 32 tiles through shared memory
__global__ void conj_transpose_kernel(const double2 *__restrict__ A, double2 *__restrict__ At, int64_t N) {
    __shared__ double2 tile[32][33];
    const int64_t bx = (int64_t)blockIdx.x * 32, by = (int64_t)blockIdx.y * 32;
    for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
        const int64_t i = bx + threadIdx.x, j = by + yy;   // A[i, j]
        if (i < N && j < N) tile[yy][threadIdx.x] = A[i + j * N];
    }
    __syncthreads();
    for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
        const int64_t i = by + threadIdx.x, j = bx + yy;   // At[i, j] = conj(A[j, i])
        if (i < N && j < N) {
            const double2 v = tile[threadIdx.x][yy];
            At[i + j * N] = make_double2(v.x, -v.y);
        }
    }
}

// ---------------------------------------------------------------------------
// Reverse pass.  Rows: [0, N) collocation rows of A (target = node i, weight
// w_i = -lambda_i, alpha_F = 1, alpha_G = -i rho c k, C term), [N, N + M)
// field rows of B (weight p_f, alpha_F = -1, alpha_G = +i rho c k).
// For L = Re sum_rows conj(w) [row . p] the kernel accumulates dL/dX for the
// vertices (atomics), and s_e = dL_complex/dY_e per element.
// ---------------------------------------------------------------------------
struct RuleTab {
    int Q[3];
    int off[3];   // first point of rule r in the table (4 doubles per point: N1 N2 N3 w)
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <bool CPLX_K>
__global__ void __launch_bounds__(kT)
adjoint_grad_kernel(int64_t N, int64_t M, const double *__restrict__ src, const double *__restrict__ fpts,
                    const double2 *__restrict__ w, const double2 *__restrict__ p,
                    const double *__restrict__ coords, const int32_t *__restrict__ topo,
                    const int32_t *__restrict__ order, const double2 *__restrict__ Y, int64_t E, int S,
                    const double *__restrict__ tab, RuleTab rt, double kre, double kim, double rhock,
                    double *__restrict__ dX, double2 *__restrict__ sY) {
    const int64_t row = (int64_t)blockIdx.x * kT + threadIdx.x;
    const bool active = row < N + M;
    const bool arow = row < N;
    const int s = blockIdx.y;
    const int64_t e0 = (int64_t)s * E / S, e1 = (int64_t)(s + 1) * E / S;
    double tx = 0, ty = 0, tz = 0;
    cd cw = {0, 0}, pi = {0, 0};
    if (active) {
        const double *T = arow ? src + 3 * row : fpts + 3 * (row - N);
        tx = T[0];
        ty = T[1];
        tz = T[2];
        const double2 wv = w[row];
        cw = {wv.x, -wv.y};   // conj(w)
        if (arow) pi = {p[row].x, p[row].y};
    }
    // alpha_F, alpha_G per row kind
    const double aF = arow ? 1.0 : -1.0;
    const cd aG = arow ? cd{0.0, -rhock} : cd{0.0, rhock};
    const cd ik = {-kim, kre};
    const double inv4pi = 1.0 / (4.0 * kPi);
    double gtx = 0, gty = 0, gtz = 0;   // d L / d target (collocation node)

    for (int64_t pe = e0; pe < e1; ++pe) {
        const int64_t e = order[pe];
        const int32_t n0 = topo[3 * e], n1 = topo[3 * e + 1], n2 = topo[3 * e + 2];
        double X[9];
        X[0] = coords[3 * n0]; X[1] = coords[3 * n0 + 1]; X[2] = coords[3 * n0 + 2];
        X[3] = coords[3 * n1]; X[4] = coords[3 * n1 + 1]; X[5] = coords[3 * n1 + 2];
        X[6] = coords[3 * n2]; X[7] = coords[3 * n2 + 1]; X[8] = coords[3 * n2 + 2];
        const double2 yv = Y[pe];
        const cd Ye = {yv.x, yv.y};
        const cd p0 = {p[n0].x, p[n0].y}, p1 = {p[n1].x, p[n1].y}, p2 = {p[n2].x, p[n2].y};
        // element vectors
        const double ux = X[3] - X[0], uy = X[4] - X[1], uz = X[5] - X[2];
        const double vx = X[6] - X[0], vy = X[7] - X[1], vz = X[8] - X[2];
        const double nx = uy * vz - uz * vy, ny = uz * vx - ux * vz, nz = ux * vy - uy * vx;
        const double jac = sqrt(nx * nx + ny * ny + nz * nz);
        double g1x = 0, g1y = 0, g1z = 0, g2x = 0, g2y = 0, g2z = 0, g3x = 0, g3y = 0, g3z = 0;
        double Gnx = 0, Gny = 0, Gnz = 0;
        cd se = {0, 0};
        if (active) {
            const int c = dev::nearest_node<3>(X, tx, ty, tz);
            const double *P = tab + 4 * (int64_t)rt.off[c];
            const int Q = rt.Q[c];
            for (int q = 0; q < Q; ++q) {
                const double N1 = P[4 * q], N2 = P[4 * q + 1], N3 = P[4 * q + 2], wq = P[4 * q + 3];
                const double yx = N1 * X[0] + N2 * X[3] + N3 * X[6];
                const double yy = N1 * X[1] + N2 * X[4] + N3 * X[7];
                const double yz = N1 * X[2] + N2 * X[5] + N3 * X[8];
                const double dx = yx - tx, dy = yy - ty, dz = yz - tz;
                const double r2 = dx * dx + dy * dy + dz * dz;
                const double rinv = rsqrt(r2);
                const double r = r2 * rinv;
                double sn, cs;
                // on the FP32 pipes in double-float (~2^-46 relative): the FP64
                // sine and cosine would be a quarter of this loop's FP64 work
                df64::TrigDf::sincos_of(kre * r, &sn, &cs);
                if (CPLX_K) {
                    const double dmp = exp(-kim * r);
                    sn *= dmp;
                    cs *= dmp;
                }
                const cd E1 = {cs, sn};                       // e^{ikr}
                const cd ikr = cscale(ik, r);
                const cd ikr1 = {ikr.re - 1.0, ikr.im};
                const double ri2 = rinv * rinv, ri3 = ri2 * rinv, ri4 = ri2 * ri2;
                // phi_F = -e^{ikr}(ikr-1)/(4 pi r^3), phi_F' = e^{ikr}(k^2/r^2 + 3(ikr-1)/r^4)/(4 pi)
                const cd phiF = cscale(cmul(E1, ikr1), -inv4pi * ri3);
                const cd k2 = cmul(ik, ik);                   // (ik)^2 = -k^2
                const cd dphiF = cscale(cmul(E1, cadd(cscale(k2, -ri2), cscale(ikr1, 3.0 * ri4))), inv4pi);
                // phi_G = e^{ikr}/(4 pi r), phi_G' = e^{ikr}(ikr - 1)/(4 pi r^2)
                const cd phiG = cscale(E1, inv4pi * rinv);
                const cd dphiG = cscale(cmul(E1, ikr1), inv4pi * ri2);
                // phi_C = -1/(4 pi r^3), phi_C' = 3/(4 pi r^4)
                const double phiC = -inv4pi * ri3, dphiC = 3.0 * inv4pi * ri4;
                const cd Ph = cadd(cadd(cscale(p0, N1), cscale(p1, N2)), cscale(p2, N3));
                const cd base = cscale(cmul(cw, Ph), wq);     // conj(w) Ph w_q
                const cd SF = cscale(base, aF);
                const cd SG = cmul(cmul(base, aG), Ye);
                const cd SC = arow ? cscale(cmul(cw, pi), wq) : cd{0, 0};
                const double dn = dx * nx + dy * ny + dz * nz;
                const double coef_r = cmul(SF, dphiF).re * dn + cmul(SG, dphiG).re * jac + SC.re * dphiC * dn;
                const double coef_n = cmul(SF, phiF).re + SC.re * phiC;
                const double coef_j = cmul(SG, phiG).re / jac;
                const double gdx = coef_r * dx * rinv + coef_n * nx;
                const double gdy = coef_r * dy * rinv + coef_n * ny;
                const double gdz = coef_r * dz * rinv + coef_n * nz;
                Gnx += coef_n * dx + coef_j * nx;
                Gny += coef_n * dy + coef_j * ny;
                Gnz += coef_n * dz + coef_j * nz;
                g1x += N1 * gdx; g1y += N1 * gdy; g1z += N1 * gdz;
                g2x += N2 * gdx; g2y += N2 * gdy; g2z += N2 * gdz;
                g3x += N3 * gdx; g3y += N3 * gdy; g3z += N3 * gdz;
                gtx -= gdx; gty -= gdy; gtz -= gdz;
                se = cadd(se, cmul(cmul(base, aG), cscale(phiG, jac)));
            }
            // nn = u x v: dL/du = v x Gn, dL/dv = Gn x u
            const double aux = vy * Gnz - vz * Gny, auy = vz * Gnx - vx * Gnz, auz = vx * Gny - vy * Gnx;
            const double avx = Gny * uz - Gnz * uy, avy = Gnz * ux - Gnx * uz, avz = Gnx * uy - Gny * ux;
            g2x += aux; g2y += auy; g2z += auz;
            g3x += avx; g3y += avy; g3z += avz;
            g1x -= aux + avx; g1y -= auy + avy; g1z -= auz + avz;
        }
        // reduce over the warp's rows, one set of atomics per warp and element
        g1x = warp_sum(g1x); g1y = warp_sum(g1y); g1z = warp_sum(g1z);
        g2x = warp_sum(g2x); g2y = warp_sum(g2y); g2z = warp_sum(g2z);
        g3x = warp_sum(g3x); g3y = warp_sum(g3y); g3z = warp_sum(g3z);
        se.re = warp_sum(se.re);
        se.im = warp_sum(se.im);
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(&dX[3 * n0], g1x); atomicAdd(&dX[3 * n0 + 1], g1y); atomicAdd(&dX[3 * n0 + 2], g1z);
            atomicAdd(&dX[3 * n1], g2x); atomicAdd(&dX[3 * n1 + 1], g2y); atomicAdd(&dX[3 * n1 + 2], g2z);
            atomicAdd(&dX[3 * n2], g3x); atomicAdd(&dX[3 * n2 + 1], g3y); atomicAdd(&dX[3 * n2 + 2], g3z);
            atomicAdd(&sY[e].x, se.re);
            atomicAdd(&sY[e].y, se.im);
        }
    }
    if (active && arow) {   // the collocation point is vertex `row`
        atomicAdd(&dX[3 * row], gtx);
        atomicAdd(&dX[3 * row + 1], gty);
        atomicAdd(&dX[3 * row + 2], gtz);
    }
}

inline unsigned nblocks(int64_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

}  // namespace

void run_adjoint(Ctx &c, const AdjointArgs &a, AdjointOut &out) {
    if (c.shape_kind != BIE_TRI_LINEAR || c.physics_kind != BIE_TRI_LINEAR)
        fail(BIE_ERR_UNSUPPORTED, "the adjoint supports 3-node triangles with vertex physics");
    if (c.n_sources != c.n_coords || c.sources != c.coords || c.ptopo != c.topo)
        fail(BIE_ERR_UNSUPPORTED, "the adjoint needs collocation nodes identical to the vertices");
    const int64_t N = c.n_sources, E = c.n_elements, M = a.n_field;
    if (a.k_im != 0.0) fail(BIE_ERR_UNSUPPORTED, "the adjoint supports real wavenumbers");
    // device buffers (allocated per call; the adjoint runs once per design step)
    struct Buf {
        void *p = nullptr;
        explicit Buf(size_t b) { BIE_CUDA(cudaMalloc(&p, std::max<size_t>(b, 16))); }
        ~Buf() { cudaFree(p); }
        double2 *d2() const { return static_cast<double2 *>(p); }
        double *d() const { return static_cast<double *>(p); }
        int32_t *i32() const { return static_cast<int32_t *>(p); }
    };
    Buf A((size_t)N * N * 16), G((size_t)N * N * 16), B((size_t)M * N * 16), Gx((size_t)M * N * 16);
    Buf Cv(N * 16), Y(E * 16), Zd(E * 16), ord(E * 4), fp(M * 24), pI(N * 16), pIf(M * 16);
    Buf p(N * 16), pf(M * 16), rhs(N * 16), lam(N * 16), w((N + M) * 16), dX(3 * N * 8), sY(E * 16);
    Buf tab(4 * 3 * 64 * 8);
    cudaStream_t st = c.stream;
    BIE_CUDA(cudaMemcpyAsync(Zd.p, a.Z, E * 16, cudaMemcpyHostToDevice, st));
    BIE_CUDA(cudaMemcpyAsync(ord.p, c.order.data(), E * 4, cudaMemcpyHostToDevice, st));
    BIE_CUDA(cudaMemcpyAsync(fp.p, a.field, M * 24, cudaMemcpyHostToDevice, st));
    admittance_kernel<<<nblocks(E), 256, 0, st>>>(Zd.d2(), ord.i32(), E, Y.d2());
    BIE_CUDA(cudaGetLastError());
    if (!c.d_coords) {
        BIE_CUDA(cudaMalloc(&c.d_coords, c.coords.size() * sizeof(double)));
        BIE_CUDA(cudaMemcpy(c.d_coords, c.coords.data(), c.coords.size() * sizeof(double), cudaMemcpyHostToDevice));
        BIE_CUDA(cudaMalloc(&c.d_topo, c.topo.size() * sizeof(int32_t)));
        BIE_CUDA(cudaMemcpy(c.d_topo, c.topo.data(), c.topo.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    }
    // -i rho c k and +i rho c k (k real)
    const double2 aAc = make_double2(0.0, -a.rho_c * a.k_re);
    const double2 aBc = make_double2(0.0, a.rho_c * a.k_re);
    // ---- forward: A, B ----------------------------------------------------------
    {
        AssembleArgs s{a.k_re, a.k_im, c.d_sources, N, BIE_F | BIE_G | BIE_C, A.d(), G.d(), Cv.d()};
        s.g_weight = Y.d();
        if (!(a.precision == BIE_PREC_DF64 && launch_assemble_df64(c, s))) launch_assemble_fp64(c, s);
        combine_system_kernel<<<std::min<unsigned>(nblocks(N * N), 65535u), 256, 0, st>>>(
            A.d2(), G.d2(), aAc, Cv.d2(), N, N);
        BIE_CUDA(cudaGetLastError());
        AssembleArgs f{a.k_re, a.k_im, fp.d(), M, BIE_F | BIE_G, B.d(), Gx.d(), nullptr};
        f.g_weight = Y.d();
        if (!(a.precision == BIE_PREC_DF64 && launch_assemble_df64(c, f))) launch_assemble_fp64(c, f);
        // stored: F_x - i rho c k G_x  (= -B)
        combine_system_kernel<<<std::min<unsigned>(nblocks(M * N), 65535u), 256, 0, st>>>(
            B.d2(), Gx.d2(), make_double2(-aBc.x, -aBc.y), nullptr, M, N);
        BIE_CUDA(cudaGetLastError());
    }
    incident_kernel<<<nblocks(N), 256, 0, st>>>(c.d_sources, N, a.k_re, a.k_im, a.dir[0], a.dir[1],
                                                 a.dir[2], pI.d2());
    incident_kernel<<<nblocks(M), 256, 0, st>>>(fp.d(), M, a.k_re, a.k_im, a.dir[0], a.dir[1], a.dir[2],
                                                 pIf.d2());
    BIE_CUDA(cudaGetLastError());
    bie_gmres_opts go{};
    go.reltol = a.reltol > 0 ? a.reltol : 1e-13;
    go.restart = 60;
    go.maxiter = (int)std::min<int64_t>(N, 5000);
    go.precision = BIE_PREC_FP64;
    bie_gmres_info gi{};
    bie_operator op{};
    op.kind = BIE_OP_DENSE;
    op.A = A.d();
    op.scale_re = 1.0;
    run_gmres(c, op, pI.d(), p.d(), go, gi);
    out.forward_iterations = gi.iterations;
    out.forward_converged = gi.converged;
    // The B buffer holds F_x - i rho c k G_x = -B, so p_f = p_I(x_f) - (stored) p.
    {
        Buf tmp(M * 16), zero(M * 16);
        BIE_CUDA(cudaMemsetAsync(zero.p, 0, M * 16, st));
        small_gemv_kernel<<<nblocks(M * 32), 256, 0, st>>>(B.d2(), M, N, p.d2(), zero.d2(), tmp.d2());
        BIE_CUDA(cudaGetLastError());
        std::vector<std::complex<double>> ht(M), hi(M);
        BIE_CUDA(cudaMemcpyAsync(ht.data(), tmp.p, M * 16, cudaMemcpyDeviceToHost, st));
        BIE_CUDA(cudaMemcpyAsync(hi.data(), pIf.p, M * 16, cudaMemcpyDeviceToHost, st));
        BIE_CUDA(cudaStreamSynchronize(st));
        double J = 0;
        std::vector<std::complex<double>> hpf(M);
        for (int64_t j = 0; j < M; ++j) {
            hpf[j] = hi[j] - ht[j];
            J += std::norm(hpf[j]);
        }
        out.J = J;
        if (a.pf) std::copy(hpf.begin(), hpf.end(), reinterpret_cast<std::complex<double> *>(a.pf));
        BIE_CUDA(cudaMemcpyAsync(pf.p, hpf.data(), M * 16, cudaMemcpyHostToDevice, st));
        BIE_CUDA(cudaStreamSynchronize(st));
    }
    if (!a.dX && !a.dZ) return;
    // ---- adjoint: A^H lambda = B^H p_f  (B^H p_f = -(stored)^H p_f) ---------------
    adjoint_rhs_kernel<<<nblocks(N), 256, 0, st>>>(B.d2(), M, N, pf.d2(), rhs.d2());
    BIE_CUDA(cudaGetLastError());
    {
        std::vector<std::complex<double>> hr(N);
        BIE_CUDA(cudaMemcpyAsync(hr.data(), rhs.p, N * 16, cudaMemcpyDeviceToHost, st));
        BIE_CUDA(cudaStreamSynchronize(st));
        for (auto &v : hr) v = -v;
        BIE_CUDA(cudaMemcpyAsync(rhs.p, hr.data(), N * 16, cudaMemcpyHostToDevice, st));
        BIE_CUDA(cudaStreamSynchronize(st));
    }
    conj_transpose_kernel<<<dim3((unsigned)((N + 31) / 32), (unsigned)((N + 31) / 32)), dim3(32, 8), 0, st>>>(
        A.d2(), G.d2(), N);   // G buffer reused for A^H
    BIE_CUDA(cudaGetLastError());
    op.A = G.d();
    run_gmres(c, op, rhs.d(), lam.d(), go, gi);
    out.adjoint_iterations = gi.iterations;
    out.adjoint_converged = gi.converged;
    // ---- reverse pass ----------------------------------------------------------------
    {
        std::vector<std::complex<double>> hl(N), hw(N + M), hp(M);
        BIE_CUDA(cudaMemcpyAsync(hl.data(), lam.p, N * 16, cudaMemcpyDeviceToHost, st));
        BIE_CUDA(cudaMemcpyAsync(hp.data(), pf.p, M * 16, cudaMemcpyDeviceToHost, st));
        BIE_CUDA(cudaStreamSynchronize(st));
        for (int64_t i = 0; i < N; ++i) hw[i] = -hl[i];
        for (int64_t j = 0; j < M; ++j) hw[N + j] = hp[j];
        BIE_CUDA(cudaMemcpyAsync(w.p, hw.data(), (N + M) * 16, cudaMemcpyHostToDevice, st));
        // rule table: 3 corner rules, 4 doubles per point (N1 N2 N3 w)
        std::vector<double> ht;
        RuleTab rt{};
        for (int r = 0; r < 3; ++r) {
            rt.off[r] = (int)(ht.size() / 4);
            rt.Q[r] = c.rules[r].size();
            for (int q = 0; q < rt.Q[r]; ++q) {
                double Nv[3];
                shape_values(BIE_TRI_LINEAR, c.rules[r].u[q], c.rules[r].v[q], Nv);
                ht.push_back(Nv[0]);
                ht.push_back(Nv[1]);
                ht.push_back(Nv[2]);
                ht.push_back(c.rules[r].w[q]);
            }
        }
        BIE_CUDA(cudaMemcpyAsync(tab.p, ht.data(), ht.size() * 8, cudaMemcpyHostToDevice, st));
        BIE_CUDA(cudaMemsetAsync(dX.p, 0, 3 * N * 8, st));
        BIE_CUDA(cudaMemsetAsync(sY.p, 0, E * 16, st));
        int S = 1;
        const int64_t tiles = (N + M + kT - 1) / kT;
        while (tiles * S < 8LL * c.num_sms && S < 256 && S * 2 <= E) S *= 2;
        const double rhock_re = a.rho_c * a.k_re;
        dim3 grid((unsigned)tiles, (unsigned)S);
        adjoint_grad_kernel<false><<<grid, kT, 0, st>>>(N, M, c.d_sources, fp.d(), w.d2(), p.d2(),
                                                        c.d_coords, c.d_topo, ord.i32(), Y.d2(), E, S,
                                                        tab.d(), rt, a.k_re, a.k_im, rhock_re, dX.d(),
                                                        sY.d2());
        BIE_CUDA(cudaGetLastError());
        std::vector<double> hdX(3 * N);
        std::vector<std::complex<double>> hs(E), hpI(N);
        BIE_CUDA(cudaMemcpyAsync(hdX.data(), dX.p, 3 * N * 8, cudaMemcpyDeviceToHost, st));
        BIE_CUDA(cudaMemcpyAsync(hs.data(), sY.p, E * 16, cudaMemcpyDeviceToHost, st));
        BIE_CUDA(cudaMemcpyAsync(hpI.data(), pI.p, N * 16, cudaMemcpyDeviceToHost, st));
        BIE_CUDA(cudaStreamSynchronize(st));
        if (a.dX) {
            const std::complex<double> ik(-a.k_im, a.k_re);
            for (int64_t i = 0; i < N; ++i) {
                // 2 Re[conj(lambda_i) d p_I / d x_i],  d p_I / d x = -i k d p_I
                const std::complex<double> s = std::conj(hl[i]) * (-ik) * hpI[i];
                for (int k = 0; k < 3; ++k) a.dX[3 * i + k] = 2.0 * hdX[3 * i + k] + 2.0 * s.real() * a.dir[k];
            }
        }
        if (a.dZ) {
            const std::complex<double> *Z = reinterpret_cast<const std::complex<double> *>(a.Z);
            std::complex<double> *dZ = reinterpret_cast<std::complex<double> *>(a.dZ);
            for (int64_t e = 0; e < E; ++e) dZ[e] = -2.0 * std::conj(hs[e] / (Z[e] * Z[e]));
        }
    }
}

}  // namespace bie
