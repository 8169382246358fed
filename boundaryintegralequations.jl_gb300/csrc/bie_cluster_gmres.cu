// One-launch restarted GMRES for the sparse near-field systems of the
// visco-thermal operator (the gmres(Gh, .) and gmres(Gv, .) calls of
// LossyGlobalOuter / LossyGlobalInner, src/3d/LossyGlobalMatrix.jl:26-37 and
// :179-197).
//
// Those systems are small (N or 3N rows, N = mesh nodes, a few to a few tens of
// non-zeros per row) and converge in a handful of Arnoldi steps, so the
// launch-per-operation form of the device GMRES (dot products, Gram-Schmidt
// updates, Givens steps, host checks) spends its time in launch latency.  Here
// a single thread-block cluster (16 CTAs where the GPU schedules them, else 8)
// runs the whole solve:
//   * the rows are split into one contiguous range per CTA; the working vector
//     w of the CTA's rows lives in its shared memory, the Krylov basis V and
//     the iterate x in global memory (L2-resident at these sizes);
//   * every reduction (Gram-Schmidt coefficients, norms) is a per-warp pass
//     over the CTA's rows, a cluster barrier, and a sum of the CTAs' partials
//     read through distributed shared memory in rank order, so every CTA holds
//     bit-identical coefficients and takes the same branches;
//   * the Hessenberg column, Givens rotations, residual estimate and back
//     substitution run on one thread of each CTA on its own copy of the state.
// The algorithm is the device GMRES of bie_solver.cu (gmres_core): zero start,
// classical Gram-Schmidt with one re-orthogonalisation, complex Givens
// rotations (real cosine), restart after `restart` steps with the true
// residual, stop when |r| <= max(reltol |b|, abstol) or after maxiter steps.
// Every loop has a bound, and every CTA runs the same sequence of cluster
// barriers, so the kernel cannot wait forever.
#include "bie_internal.h"

#include <cooperative_groups.h>

#include <algorithm>
#include <map>
#include <mutex>

namespace cg = cooperative_groups;

namespace bie {

namespace {

constexpr int kCT = 512;              // threads per CTA
constexpr int kCW = kCT / 32;         // warps per CTA
constexpr int kMaxRestart = 48;       // longest restart cycle of the one-launch path
constexpr size_t kMaxSmem = 200 * 1024;

struct CgArgs {
    const int64_t *rp;
    const int32_t *cols;
    const double2 *val;
    const double2 *diag;   // may be null
    int64_t N;             // rows of one block
    int64_t n;             // nb * N
    const double2 *b;
    double2 *x;
    double2 *V;            // (m + 1) x n
    int64_t rows_per;      // rows per CTA
    int m, maxiter;
    double reltol, abstol;
    bie_gmres_info *info;          // may be null
    unsigned long long *acc;       // [0] += 1 solve, [1] += iterations (may be null)
};

struct CgScalars {
    double res;     // |g_{j+1}| after the last step
    double hn;      // h_{j+1,j} of the last step
    int done;       // converged or breakdown in this cycle
    int jdone;      // steps completed in this cycle
};

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// (A s)[i] for global row i; s was written by other CTAs of the cluster before
// the last cluster barrier, so it is read through L2 (ld.global.cg).
__device__ __forceinline__ double2 csr_row(const CgArgs &a, const double2 *s, int64_t i) {
    const int64_t blk = i / a.N;
    const int64_t r = i - blk * a.N;
    const double2 *sb = s + blk * a.N;
    const int64_t p0 = __ldg(a.rp + r), p1 = __ldg(a.rp + r + 1);
    double re = 0.0, im = 0.0;
    int64_t p = p0;
    for (; p + 4 <= p1; p += 4) {
        const int c0 = __ldg(a.cols + p), c1 = __ldg(a.cols + p + 1), c2 = __ldg(a.cols + p + 2),
                  c3 = __ldg(a.cols + p + 3);
        const double2 v0 = __ldg(a.val + p), v1 = __ldg(a.val + p + 1), v2 = __ldg(a.val + p + 2),
                      v3 = __ldg(a.val + p + 3);
        const double2 x0 = __ldcg(sb + c0), x1 = __ldcg(sb + c1), x2 = __ldcg(sb + c2), x3 = __ldcg(sb + c3);
        re += v0.x * x0.x - v0.y * x0.y;
        im += v0.x * x0.y + v0.y * x0.x;
        re += v1.x * x1.x - v1.y * x1.y;
        im += v1.x * x1.y + v1.y * x1.x;
        re += v2.x * x2.x - v2.y * x2.y;
        im += v2.x * x2.y + v2.y * x2.x;
        re += v3.x * x3.x - v3.y * x3.y;
        im += v3.x * x3.y + v3.y * x3.x;
    }
    for (; p < p1; ++p) {
        const double2 v = __ldg(a.val + p), xv = __ldcg(sb + __ldg(a.cols + p));
        re += v.x * xv.x - v.y * xv.y;
        im += v.x * xv.y + v.y * xv.x;
    }
    if (a.diag) {
        const double2 d = __ldg(a.diag + r), xv = __ldcg(s + i);
        re += d.x * xv.x - d.y * xv.y;
        im += d.x * xv.y + d.y * xv.x;
    }
    return make_double2(re, im);
}

// out[0..nc) = sum over the cluster's CTAs of part[0..nc); the caller has
// written this CTA's part.  One warp per column, lane r reading CTA r's
// partial through distributed shared memory, then the same butterfly sum in
// every CTA (bit-identical results).  Ends with the CTA synchronised.
__device__ __forceinline__ void cluster_sum(cg::cluster_group &cl, double2 *part, int nc, double2 *out) {
    cl.sync();
    const unsigned C = cl.num_blocks();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int c = warp; c < nc; c += kCW) {
        double2 v = make_double2(0.0, 0.0);
        if ((unsigned)lane < C) v = cl.map_shared_rank(part, (unsigned)lane)[c];
        const double re = warp_sum(v.x), im = warp_sum(v.y);
        if (lane == 0) out[c] = make_double2(re, im);
    }
    __syncthreads();
}

// part[c] = V[:, c]^H w over this CTA's rows, c < nc (one warp per column)
__device__ __forceinline__ void local_multidot(const double2 *V, int64_t n, int64_t lo, int cnt, int nc,
                                               const double2 *w_s, double2 *part) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int c = warp; c < nc; c += kCW) {
        const double2 *vc = V + (int64_t)c * n + lo;
        double re = 0.0, im = 0.0;
        for (int i = lane; i < cnt; i += 32) {
            const double2 a = vc[i], w = w_s[i];
            re += a.x * w.x + a.y * w.y;
            im += a.x * w.y - a.y * w.x;
        }
        re = warp_sum(re);
        im = warp_sum(im);
        if (lane == 0) part[c] = make_double2(re, im);
    }
}

// part[0] = |w|^2 over this CTA's rows
__device__ __forceinline__ void local_norm2(int cnt, const double2 *w_s, double2 *part, double *wred) {
    double s = 0.0;
    for (int i = threadIdx.x; i < cnt; i += kCT) s += w_s[i].x * w_s[i].x + w_s[i].y * w_s[i].y;
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) wred[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < kCW; ++k) t += wred[k];
        part[0] = make_double2(t, 0.0);
    }
}

__global__ void __launch_bounds__(kCT, 1) csr_gmres_cluster_kernel(CgArgs a) {
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    const int m = a.m;
    const int64_t n = a.n;
    const int64_t lo0 = (int64_t)rank * a.rows_per;
    const int64_t lo = lo0 < n ? lo0 : n;
    const int64_t hi = lo + a.rows_per < n ? lo + a.rows_per : n;
    const int cnt = (int)(hi - lo);

    // shared memory: w (rows_per), three partial slots (m + 2 each), h1, h2, y
    // (m + 2 each), H ((m + 1) x m), g (m + 1), sn (m), cs (m), warp partials,
    // scalars
    extern __shared__ double2 smem[];
    double2 *w_s = smem;
    double2 *part = w_s + a.rows_per;
    const int ps = m + 2;
    double2 *h1 = part + 3 * ps;
    double2 *h2 = h1 + ps;
    double2 *y = h2 + ps;
    double2 *H = y + ps;
    double2 *g = H + (int64_t)(m + 1) * m;
    double2 *sn = g + (m + 1);
    double *cs = reinterpret_cast<double *>(sn + m);
    double *wred = cs + m;
    CgScalars *sc = reinterpret_cast<CgScalars *>(wred + kCW);
    int slot = 0;
    auto next_part = [&]() {
        double2 *p = part + slot * ps;
        slot = slot == 2 ? 0 : slot + 1;
        return p;
    };

    // |b|, x = 0, w = b
    for (int i = threadIdx.x; i < cnt; i += kCT) {
        w_s[i] = a.b[lo + i];
        a.x[lo + i] = make_double2(0.0, 0.0);
    }
    __syncthreads();
    {
        double2 *p = next_part();
        local_norm2(cnt, w_s, p, wred);
        cluster_sum(cl, p, 1, h1);
    }
    const double bnorm = sqrt(fmax(h1[0].x, 0.0));
    const double tol = fmax(a.reltol * bnorm, a.abstol);
    double beta = bnorm;
    int it = 0, restarts = 0;
    long long matvecs = 0;

    for (int cycle = 0; cycle <= a.maxiter; ++cycle) {
        if (cycle > 0) {
            // w = b - A x with the x of every CTA
            cl.sync();
            for (int i = threadIdx.x; i < cnt; i += kCT) {
                const double2 ax = csr_row(a, a.x, lo + i), bv = a.b[lo + i];
                w_s[i] = make_double2(bv.x - ax.x, bv.y - ax.y);
            }
            ++matvecs;
            __syncthreads();
            double2 *p = next_part();
            local_norm2(cnt, w_s, p, wred);
            cluster_sum(cl, p, 1, h1);
            beta = sqrt(fmax(h1[0].x, 0.0));
        }
        const int jmax = min(m, max(0, a.maxiter - it));
        if (beta <= tol || jmax == 0) break;

        // v_0 = w / beta; g = (beta, 0, ...)
        const double inv_beta = 1.0 / beta;
        for (int i = threadIdx.x; i < cnt; i += kCT)
            a.V[lo + i] = make_double2(w_s[i].x * inv_beta, w_s[i].y * inv_beta);
        if (threadIdx.x == 0) {
            for (int k = 0; k <= m; ++k) g[k] = make_double2(0.0, 0.0);
            g[0] = make_double2(beta, 0.0);
            sc->done = 0;
            sc->jdone = 0;
        }
        for (int j = 0; j < jmax; ++j) {
            cl.sync();   // v_j of every CTA is in global memory
            const double2 *vj = a.V + (int64_t)j * n;
            for (int i = threadIdx.x; i < cnt; i += kCT) w_s[i] = csr_row(a, vj, lo + i);
            __syncthreads();
            // classical Gram-Schmidt, two passes
            for (int pass = 0; pass < 2; ++pass) {
                double2 *h = pass == 0 ? h1 : h2;
                double2 *p = next_part();
                local_multidot(a.V, n, lo, cnt, j + 1, w_s, p);
                cluster_sum(cl, p, j + 1, h);
                for (int i = threadIdx.x; i < cnt; i += kCT) {
                    double re = w_s[i].x, im = w_s[i].y;
                    for (int c = 0; c <= j; ++c) {
                        const double2 v = a.V[(int64_t)c * n + lo + i], hc = h[c];
                        re -= v.x * hc.x - v.y * hc.y;
                        im -= v.x * hc.y + v.y * hc.x;
                    }
                    w_s[i] = make_double2(re, im);
                }
                __syncthreads();
            }
            {
                double2 *p = next_part();
                local_norm2(cnt, w_s, p, wred);
                cluster_sum(cl, p, 1, y);
            }
            if (threadIdx.x == 0) {
                // Hessenberg column j, earlier rotations, the new rotation
                const int ld = m + 1;
                double2 *col = H + (int64_t)j * ld;
                for (int k = 0; k <= j; ++k) col[k] = make_double2(h1[k].x + h2[k].x, h1[k].y + h2[k].y);
                const double hn = sqrt(fmax(y[0].x, 0.0));
                col[j + 1] = make_double2(hn, 0.0);
                for (int k = 0; k < j; ++k) {
                    const double c = cs[k];
                    const double2 s = sn[k];
                    const double2 u = col[k], v = col[k + 1];
                    const double2 sv = cmul(s, v), su = cmul(cconj(s), u);
                    col[k] = make_double2(c * u.x + sv.x, c * u.y + sv.y);
                    col[k + 1] = make_double2(-su.x + c * v.x, -su.y + c * v.y);
                }
                const double2 u = col[j], v = col[j + 1];
                const double nu = hypot(u.x, u.y), nv = hypot(v.x, v.y);
                double c;
                double2 s, r;
                if (nv == 0.0) {
                    c = 1.0;
                    s = make_double2(0.0, 0.0);
                    r = u;
                } else if (nu == 0.0) {
                    c = 0.0;
                    s = make_double2(v.x / nv, -v.y / nv);
                    r = make_double2(nv, 0.0);
                } else {
                    const double nrm = hypot(nu, nv);
                    const double2 al = make_double2(u.x / nu, u.y / nu);
                    c = nu / nrm;
                    const double2 t = cmul(al, cconj(v));
                    s = make_double2(t.x / nrm, t.y / nrm);
                    r = make_double2(al.x * nrm, al.y * nrm);
                }
                cs[j] = c;
                sn[j] = s;
                col[j] = r;
                col[j + 1] = make_double2(0.0, 0.0);
                const double2 gj = g[j], gj1 = g[j + 1];
                const double2 sg = cmul(s, gj1), ug = cmul(cconj(s), gj);
                g[j] = make_double2(c * gj.x + sg.x, c * gj.y + sg.y);
                g[j + 1] = make_double2(-ug.x + c * gj1.x, -ug.y + c * gj1.y);
                sc->res = hypot(g[j + 1].x, g[j + 1].y);
                sc->hn = hn;
                sc->jdone = j + 1;
                sc->done = (sc->res <= tol || hn == 0.0) ? 1 : 0;
            }
            __syncthreads();
            // v_{j+1} = w / h_{j+1,j}
            const double hn = sc->hn;
            const double inv_hn = hn > 0.0 ? 1.0 / hn : 0.0;
            double2 *vn = a.V + (int64_t)(j + 1) * n;
            for (int i = threadIdx.x; i < cnt; i += kCT)
                vn[lo + i] = make_double2(w_s[i].x * inv_hn, w_s[i].y * inv_hn);
            if (sc->done) break;
        }
        // y = R^{-1} g; x += V y (this CTA's rows)
        const int jd = sc->jdone;
        if (threadIdx.x == 0) {
            const int ld = m + 1;
            for (int k = jd - 1; k >= 0; --k) {
                double2 acc = g[k];
                for (int l = k + 1; l < jd; ++l) {
                    const double2 t = cmul(H[(int64_t)l * ld + k], y[l]);
                    acc.x -= t.x;
                    acc.y -= t.y;
                }
                const double2 d = H[(int64_t)k * ld + k];
                const double den = d.x * d.x + d.y * d.y;
                y[k] = make_double2((acc.x * d.x + acc.y * d.y) / den, (acc.y * d.x - acc.x * d.y) / den);
            }
        }
        __syncthreads();
        for (int i = threadIdx.x; i < cnt; i += kCT) {
            double2 xv = a.x[lo + i];
            for (int c = 0; c < jd; ++c) {
                const double2 v = a.V[(int64_t)c * n + lo + i], yc = y[c];
                xv.x += v.x * yc.x - v.y * yc.y;
                xv.y += v.x * yc.y + v.y * yc.x;
            }
            a.x[lo + i] = xv;
        }
        it += jd;
        matvecs += jd;
        ++restarts;
    }
    if (rank == 0 && threadIdx.x == 0) {
        if (a.info) {
            bie_gmres_info o{};
            o.iterations = it;
            o.restarts = restarts;
            o.refinements = 0;
            o.converged = beta <= tol ? 1 : 0;
            o.matvecs = matvecs;
            o.residual_norm = beta;
            o.rhs_norm = bnorm;
            *a.info = o;
        }
        if (a.acc) {
            atomicAdd(a.acc, 1ull);
            atomicAdd(a.acc + 1, (unsigned long long)it);
        }
    }
    cl.sync();   // no CTA leaves while another may still read its shared memory
}

size_t smem_bytes(int64_t rows_per, int m) {
    const size_t c2 = (size_t)rows_per + 3 * (m + 2) + 3 * (m + 2) + (size_t)(m + 1) * m + (m + 1) + m;
    return c2 * 16 + (size_t)m * 8 + kCW * 8 + sizeof(CgScalars) + 16;
}

// Largest cluster (16, else 8) the GPU co-schedules with `smem` bytes per CTA;
// 0 if none.  Cached per (device, smem).  The kernel's dynamic shared-memory
// limit is raised once per device to the largest size this path launches
// with (kMaxSmem), so every cached answer stays launchable.
int cluster_size_for(int device, size_t smem) {
    static std::mutex mu;
    static std::map<std::pair<int, size_t>, int> cache;
    static std::map<int, bool> attrs_ok;
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find({device, smem});
    if (it != cache.end()) return it->second;
    auto at_it = attrs_ok.find(device);
    if (at_it == attrs_ok.end()) {
        const bool ok = cudaFuncSetAttribute(csr_gmres_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)kMaxSmem) == cudaSuccess &&
                        cudaFuncSetAttribute(csr_gmres_cluster_kernel,
                                             cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess;
        at_it = attrs_ok.emplace(device, ok).first;
    }
    int best = 0;
    if (at_it->second) {
        for (int C : {16, 8}) {
            cudaLaunchConfig_t cfg{};
            cfg.gridDim = dim3(C);
            cfg.blockDim = dim3(kCT);
            cfg.dynamicSmemBytes = smem;
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = C;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            int nclusters = 0;
            if (cudaOccupancyMaxActiveClusters(&nclusters, csr_gmres_cluster_kernel, &cfg) == cudaSuccess &&
                nclusters > 0) {
                best = C;
                break;
            }
        }
    }
    cudaGetLastError();
    cache[{device, smem}] = best;
    return best;
}

}  // namespace

bool csr_gmres_one_launch(Ctx &c, const CsrSystem &A, const double2 *b, double2 *x, const bie_gmres_opts &o,
                          int level, bie_gmres_info *d_info, unsigned long long *d_acc) {
    const int64_t n = A.N * A.nb;
    if (n <= 0 || c.capturing) return false;
    const int m = (int)std::max<int64_t>(1, std::min<int64_t>(o.restart > 0 ? o.restart : 20, n));
    if (m > kMaxRestart) return false;
    const int maxiter = o.maxiter > 0 ? o.maxiter : (int)std::min<int64_t>(n, INT32_MAX);
    // rows per CTA for the largest cluster that could take them
    int C = 16;
    int64_t rows_per = (n + C - 1) / C;
    size_t smem = smem_bytes(rows_per, m);
    if (smem > kMaxSmem) return false;
    C = cluster_size_for(c.device, smem);
    if (C == 0) return false;
    if (C != 16) {
        rows_per = (n + C - 1) / C;
        smem = smem_bytes(rows_per, m);
        if (smem > kMaxSmem || cluster_size_for(c.device, smem) < C) return false;
    }
    const int ws_slot = level == 0 ? kScratchSolver : kScratchSolverNested + 2 * (level - 1);
    double2 *V = static_cast<double2 *>(c.scratch(ws_slot, (size_t)(m + 1) * n * 16));

    CgArgs a{};
    a.rp = A.rp;
    a.cols = A.cols;
    a.val = A.val;
    a.diag = A.diag;
    a.N = A.N;
    a.n = n;
    a.b = b;
    a.x = x;
    a.V = V;
    a.rows_per = rows_per;
    a.m = m;
    a.maxiter = maxiter;
    a.reltol = o.reltol > 0 ? o.reltol : std::sqrt(2.220446049250313e-16);
    a.abstol = std::max(0.0, o.abstol);
    a.info = d_info;
    a.acc = d_acc;

    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(C);
    cfg.blockDim = dim3(kCT);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = c.stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    BIE_CUDA(cudaLaunchKernelEx(&cfg, csr_gmres_cluster_kernel, a));
    ++c.kernel_launches;
    return true;
}

}  // namespace bie
