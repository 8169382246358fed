// One-launch restarted GMRES for the sparse near-field systems of the
// visco-thermal operator (the gmres(Gh, .) and gmres(Gv, .) calls of
// LossyGlobalOuter / LossyGlobalInner, src/3d/LossyGlobalMatrix.jl:26-37 and
// :179-197).
//
// Those systems are small (N or 3N rows, N = mesh nodes, a few to a few tens of
// non-zeros per row) and converge in a handful of Arnoldi steps, so the
// launch-per-operation form of the device GMRES (dot products, Gram-Schmidt
// updates, Givens steps, host checks) spends its time in launch latency.  Here
// one launch runs the whole solve:
//   * the rows are split into one contiguous range per CTA; the working vector
//     w and, where it fits, the Krylov basis V of the CTA's rows live in its
//     shared memory; the newest basis vector is also written to a global
//     vector, from which the sparse product gathers it; the iterate x is in
//     global memory (V too when it does not fit; all L2-resident here);
//   * every reduction (Gram-Schmidt coefficients, norms) is a per-warp pass
//     over the CTA's rows, a barrier, and a sum of the CTAs' partials in a
//     fixed order, so every CTA holds bit-identical coefficients and takes the
//     same branches;
//   * the Hessenberg column, Givens rotations, residual estimate and back
//     substitution run on one thread of each CTA on its own copy of the state.
// Two synchronisation forms:
//   * grid (large systems): one CTA per SM, partials in global memory, a
//     grid barrier of this file (one monotonic arrival counter: barrier b
//     completes when it reaches (b + 1) x CTAs; release add, acquire polls)
//     whose waits are bounded: a wait that runs out sets an error word, which
//     makes every later barrier return at once, and the host reports the
//     error.  The launch is cooperative, so all CTAs are resident.  The
//     arithmetic is FP64 and this GPU's FP64 pipe is narrow, so the rows are
//     spread over all SMs;
//   * cluster (small systems): a 16-CTA (else 8-CTA) thread-block cluster,
//     partials read through distributed shared memory after hardware cluster
//     barriers, which every CTA reaches the same number of times.
// The algorithm is the device GMRES of bie_solver.cu (gmres_core): zero start,
// classical Gram-Schmidt with one re-orthogonalisation, complex Givens
// rotations (real cosine), restart after `restart` steps with the true
// residual, stop when |r| <= max(reltol |b|, abstol) or after maxiter steps.
// Every loop has a bound.
#include "bie_internal.h"

#include <cooperative_groups.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>

namespace cg = cooperative_groups;

namespace bie {

namespace {

constexpr int kMaxRestart = 48;        // longest restart cycle of the one-launch path
constexpr size_t kMaxSmem = 224 * 1024;
constexpr int kClusterThreads = 512;
constexpr int kGridThreads = 256;
constexpr long long kSpinLimit = 1LL << 23;   // grid-barrier polls (about a second)

struct CgArgs {
    const int64_t *rp;
    const int32_t *cols;
    const double2 *val;
    const double2 *diag;   // may be null
    int64_t N;             // rows of one block
    int64_t n;             // nb * N
    const double2 *b;
    double2 *x;
    double2 *V;            // VS: the newest basis vector (n); else the basis, (m + 1) x n
    double2 *gpart;        // grid form: partials, 3 slots x (m + 2) columns x CTAs
    unsigned *bar;         // grid form: arrival counter (zero at launch)
    int *err;              // grid form: set when a barrier wait runs out
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

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void red_add_release(unsigned *p, unsigned v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_relaxed(const int *p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Synchronisation over a thread-block cluster: partials in shared memory,
// read by the other CTAs through distributed shared memory.
template <int NT>
struct ClusterSync {
    static constexpr int kThreads = NT;
    cg::cluster_group cl;
    double2 *spart;   // shared: 3 slots x ps
    int ps;
    __device__ ClusterSync(const CgArgs &, double2 *spart_, int ps_) : cl(cg::this_cluster()), spart(spart_), ps(ps_) {}
    __device__ unsigned rank() const { return cl.block_rank(); }
    __device__ void sync() { cl.sync(); }
    // where this CTA writes column c of slot s (stride between columns)
    __device__ double2 *mine(int s) const { return spart + s * ps; }
    __device__ int stride() const { return 1; }
    // out[c] = sum over CTAs of their slot-s partial of column c (after sync)
    __device__ void gather(int s, int nc, double2 *out) {
        const unsigned C = cl.num_blocks();
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        for (int c = warp; c < nc; c += NT / 32) {
            double2 v = make_double2(0.0, 0.0);
            if ((unsigned)lane < C) v = cl.map_shared_rank(spart + s * ps, (unsigned)lane)[c];
            const double re = warp_sum(v.x), im = warp_sum(v.y);
            if (lane == 0) out[c] = make_double2(re, im);
        }
    }
    __device__ void finish() { cl.sync(); }   // no CTA leaves while another reads its shared memory
};

// Synchronisation over a cooperative grid: partials in global memory, a
// bounded counting barrier.  The CTA barrier before the release add makes the
// CTA's writes visible with it; the acquire poll and the CTA barrier after it
// order the CTA's later reads.
template <int NT>
struct GridSync {
    static constexpr int kThreads = NT;
    double2 *gpart;
    unsigned *count;
    int *err;
    int ps;
    unsigned nb, r, target;
    __device__ GridSync(const CgArgs &a, double2 *, int ps_)
        : gpart(a.gpart), count(a.bar), err(a.err), ps(ps_), nb(gridDim.x), r(blockIdx.x), target(0) {}
    __device__ unsigned rank() const { return r; }
    __device__ void sync() {
        target += nb;
        __syncthreads();
        if (threadIdx.x == 0 && ld_relaxed(err) == 0) {
            red_add_release(count, 1u);
            long long spins = 0;
            while ((int)(ld_acquire(count) - target) < 0) {
                if (++spins > kSpinLimit || ld_relaxed(err) != 0) {
                    atomicExch(err, 1);
                    break;
                }
            }
            asm volatile("fence.acq_rel.gpu;" ::: "memory");
        }
        __syncthreads();
    }
    __device__ double2 *mine(int s) const { return gpart + (size_t)s * ps * nb + r; }
    __device__ int stride() const { return (int)nb; }
    __device__ void gather(int s, int nc, double2 *out) {
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        const double2 *base = gpart + (size_t)s * ps * nb;
        for (int c = warp; c < nc; c += NT / 32) {
            double re = 0.0, im = 0.0;
            for (unsigned q0 = 0; q0 < nb; q0 += 128) {   // four independent loads per lane in flight
                double2 v[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const unsigned q = q0 + 32 * u + lane;
                    v[u] = q < nb ? __ldcg(base + (size_t)c * nb + q) : make_double2(0.0, 0.0);
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    re += v[u].x;
                    im += v[u].y;
                }
            }
            re = warp_sum(re);
            im = warp_sum(im);
            if (lane == 0) out[c] = make_double2(re, im);
        }
    }
    __device__ void finish() {}
};

// (A s)[i] for global row i; s was written by other CTAs before the last
// barrier, so it is read through L2 (ld.global.cg).
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

// part[c * ps] = V[:, c]^H w over this CTA's rows, c < nc (one warp per
// column); column c of the CTA's rows starts at Vl + c * ld
template <int NT>
__device__ __forceinline__ void local_multidot(const double2 *Vl, int64_t ld, int cnt, int nc, const double2 *w_s,
                                               double2 *part, int pst) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int c = warp; c < nc; c += NT / 32) {
        const double2 *vc = Vl + (int64_t)c * ld;
        double re = 0.0, im = 0.0;
        for (int i = lane; i < cnt; i += 32) {
            const double2 a = vc[i], w = w_s[i];
            re += a.x * w.x + a.y * w.y;
            im += a.x * w.y - a.y * w.x;
        }
        re = warp_sum(re);
        im = warp_sum(im);
        if (lane == 0) part[(int64_t)c * pst] = make_double2(re, im);
    }
}

// part[0] = |w|^2 over this CTA's rows
template <int NT>
__device__ __forceinline__ void local_norm2(int cnt, const double2 *w_s, double2 *part, double *wred) {
    double s = 0.0;
    for (int i = threadIdx.x; i < cnt; i += NT) s += w_s[i].x * w_s[i].x + w_s[i].y * w_s[i].y;
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) wred[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < NT / 32; ++k) t += wred[k];
        part[0] = make_double2(t, 0.0);
    }
}

template <class Sync, bool VS>
__global__ void __launch_bounds__(Sync::kThreads, 1) csr_gmres_one_kernel(CgArgs a) {
    constexpr int NT = Sync::kThreads;
    const int m = a.m;
    const int64_t n = a.n;
    const int ps = m + 2;

    // shared memory: [VS: basis (m + 1) x rows_per], w (rows_per), three
    // partial slots (m + 2 each; cluster form), h1, h2, y (m + 2 each),
    // H ((m + 1) x m), g (m + 1), sn (m), cs (m), warp partials, scalars
    extern __shared__ double2 smem[];
    double2 *V_s = smem;
    double2 *w_s = VS ? smem + (int64_t)(m + 1) * a.rows_per : smem;
    double2 *spart = w_s + a.rows_per;
    double2 *h1 = spart + 3 * ps;
    double2 *h2 = h1 + ps;
    double2 *y = h2 + ps;
    double2 *H = y + ps;
    double2 *g = H + (int64_t)(m + 1) * m;
    double2 *sn = g + (m + 1);
    double *cs = reinterpret_cast<double *>(sn + m);
    double *wred = cs + m;
    CgScalars *sc = reinterpret_cast<CgScalars *>(wred + NT / 32);

    Sync S(a, spart, ps);
    const int rank = (int)S.rank();
    const int64_t lo0 = (int64_t)rank * a.rows_per;
    const int64_t lo = lo0 < n ? lo0 : n;
    const int64_t hi = lo + a.rows_per < n ? lo + a.rows_per : n;
    const int cnt = (int)(hi - lo);
    // this CTA's rows of basis column c: Vl + c * ldv
    double2 *Vl = VS ? V_s : a.V + lo;
    const int64_t ldv = VS ? a.rows_per : n;

    int slot = 0;
    // reduction into out[0..nc): this CTA's partials are in slot `s` already
    auto reduce = [&](int s, int nc, double2 *out) {
        S.sync();
        S.gather(s, nc, out);
        __syncthreads();
    };
    auto next_slot = [&]() {
        const int s = slot;
        slot = slot == 2 ? 0 : slot + 1;
        return s;
    };

    // |b|, x = 0, w = b
    for (int i = threadIdx.x; i < cnt; i += NT) {
        w_s[i] = a.b[lo + i];
        a.x[lo + i] = make_double2(0.0, 0.0);
    }
    __syncthreads();
    {
        const int s = next_slot();
        local_norm2<NT>(cnt, w_s, S.mine(s), wred);
        reduce(s, 1, h1);
    }
    const double bnorm = sqrt(fmax(h1[0].x, 0.0));
    const double tol = fmax(a.reltol * bnorm, a.abstol);
    double beta = bnorm;
    int it = 0, restarts = 0;
    long long matvecs = 0;

    for (int cycle = 0; cycle <= a.maxiter; ++cycle) {
        if (cycle > 0) {
            // w = b - A x with the x of every CTA
            S.sync();
            for (int i = threadIdx.x; i < cnt; i += NT) {
                const double2 ax = csr_row(a, a.x, lo + i), bv = a.b[lo + i];
                w_s[i] = make_double2(bv.x - ax.x, bv.y - ax.y);
            }
            ++matvecs;
            __syncthreads();
            const int s = next_slot();
            local_norm2<NT>(cnt, w_s, S.mine(s), wred);
            reduce(s, 1, h1);
            beta = sqrt(fmax(h1[0].x, 0.0));
        }
        const int jmax = min(m, max(0, a.maxiter - it));
        if (beta <= tol || jmax == 0) break;

        // v_0 = w / beta; g = (beta, 0, ...)
        const double inv_beta = 1.0 / beta;
        for (int i = threadIdx.x; i < cnt; i += NT) {
            const double2 v = make_double2(w_s[i].x * inv_beta, w_s[i].y * inv_beta);
            Vl[i] = v;
            if (VS) a.V[lo + i] = v;
        }
        if (threadIdx.x == 0) {
            for (int k = 0; k <= m; ++k) g[k] = make_double2(0.0, 0.0);
            g[0] = make_double2(beta, 0.0);
            sc->done = 0;
            sc->jdone = 0;
        }
        for (int j = 0; j < jmax; ++j) {
            S.sync();   // v_j of every CTA is in global memory
            const double2 *vj = VS ? a.V : a.V + (int64_t)j * n;
            for (int i = threadIdx.x; i < cnt; i += NT) w_s[i] = csr_row(a, vj, lo + i);
            __syncthreads();
            // classical Gram-Schmidt, two passes
            for (int pass = 0; pass < 2; ++pass) {
                double2 *h = pass == 0 ? h1 : h2;
                const int s = next_slot();
                local_multidot<NT>(Vl, ldv, cnt, j + 1, w_s, S.mine(s), S.stride());
                reduce(s, j + 1, h);
                for (int i = threadIdx.x; i < cnt; i += NT) {
                    double re = w_s[i].x, im = w_s[i].y;
                    for (int c = 0; c <= j; ++c) {
                        const double2 v = Vl[(int64_t)c * ldv + i], hc = h[c];
                        re -= v.x * hc.x - v.y * hc.y;
                        im -= v.x * hc.y + v.y * hc.x;
                    }
                    w_s[i] = make_double2(re, im);
                }
                __syncthreads();
            }
            {
                const int s = next_slot();
                local_norm2<NT>(cnt, w_s, S.mine(s), wred);
                reduce(s, 1, y);
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
            double2 *vn = Vl + (int64_t)(j + 1) * ldv;
            for (int i = threadIdx.x; i < cnt; i += NT) {
                const double2 v = make_double2(w_s[i].x * inv_hn, w_s[i].y * inv_hn);
                vn[i] = v;
                // the global copy of v_j was last read by the products before
                // this step's first reduction barrier
                if (VS) a.V[lo + i] = v;
            }
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
        for (int i = threadIdx.x; i < cnt; i += NT) {
            double2 xv = a.x[lo + i];
            for (int c = 0; c < jd; ++c) {
                const double2 v = Vl[(int64_t)c * ldv + i], yc = y[c];
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
    S.finish();
}

size_t smem_bytes(int64_t rows_per, int m, bool vs, int threads) {
    const size_t c2 = (size_t)rows_per * (vs ? m + 2 : 1) + 3 * (m + 2) + 3 * (m + 2) + (size_t)(m + 1) * m +
                      (m + 1) + m;
    return c2 * 16 + (size_t)m * 8 + (size_t)(threads / 32) * 8 + sizeof(CgScalars) + 16;
}

// Whether kernel `kern` launches with `blocks` CTAs of `threads` threads and
// `smem` bytes each: as a cluster of `blocks` CTAs (cluster form), or all
// resident at once (grid form).  Cached per (kernel, device, smem, blocks).
// The kernel's dynamic shared-memory limit is raised once per device to the
// largest size this path launches with (kMaxSmem), so every cached answer
// stays launchable.
bool launch_fits(const void *kern, bool cluster, int device, int num_sms, size_t smem, int blocks, int threads) {
    static std::mutex mu;
    static std::map<std::tuple<const void *, int, size_t, int>, bool> cache;
    static std::map<std::pair<const void *, int>, bool> attrs_ok;
    std::lock_guard<std::mutex> lk(mu);
    const auto key = std::make_tuple(kern, device, smem, blocks);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    auto at_it = attrs_ok.find({kern, device});
    if (at_it == attrs_ok.end()) {
        bool ok = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem) == cudaSuccess;
        if (cluster)
            ok = ok && cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess;
        at_it = attrs_ok.emplace(std::make_pair(kern, device), ok).first;
    }
    bool fits = false;
    if (at_it->second) {
        if (cluster) {
            cudaLaunchConfig_t cfg{};
            cfg.gridDim = dim3(blocks);
            cfg.blockDim = dim3(threads);
            cfg.dynamicSmemBytes = smem;
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = blocks;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            int nclusters = 0;
            fits = cudaOccupancyMaxActiveClusters(&nclusters, kern, &cfg) == cudaSuccess && nclusters > 0;
        } else {
            int per_sm = 0;
            fits = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem) == cudaSuccess &&
                   (int64_t)per_sm * num_sms >= blocks;
        }
    }
    cudaGetLastError();
    cache[key] = fits;
    return fits;
}

struct Form {
    const void *kern;
    bool cluster, vs;
    int threads;
};

}  // namespace

bool csr_gmres_one_launch(Ctx &c, const CsrSystem &A, const double2 *b, double2 *x, const bie_gmres_opts &o,
                          int level, bie_gmres_info *d_info, unsigned long long *d_acc, int *d_err, int forms) {
    const int64_t n = A.N * A.nb;
    if (n <= 0 || c.capturing) return false;
    const int m = (int)std::max<int64_t>(1, std::min<int64_t>(o.restart > 0 ? o.restart : 20, n));
    if (m > kMaxRestart) return false;
    const int maxiter = o.maxiter > 0 ? o.maxiter : (int)std::min<int64_t>(n, INT32_MAX);
    // Launch forms in order of preference.  Systems of more than 2048 rows go
    // to the grid form (the FP64 work spread over up to one CTA per SM, 32 rows
    // or more per CTA), smaller ones to a cluster; the basis in shared memory
    // where it fits.  `forms` may restrict the choice to one of the two.
    const Form grid_vs{reinterpret_cast<const void *>(csr_gmres_one_kernel<GridSync<kGridThreads>, true>), false,
                       true, kGridThreads};
    const Form grid_g{reinterpret_cast<const void *>(csr_gmres_one_kernel<GridSync<kGridThreads>, false>), false,
                      false, kGridThreads};
    const Form cl_vs{reinterpret_cast<const void *>(csr_gmres_one_kernel<ClusterSync<kClusterThreads>, true>),
                     true, true, kClusterThreads};
    const Form cl_g{reinterpret_cast<const void *>(csr_gmres_one_kernel<ClusterSync<kClusterThreads>, false>),
                    true, false, kClusterThreads};
    std::vector<std::pair<Form, int>> cands;
    const bool grid_ok = d_err && forms != kOneLaunchCluster;
    if (grid_ok && (n > 2048 || forms == kOneLaunchGrid)) {
        const int P = (int)std::max<int64_t>(1, std::min<int64_t>(c.num_sms, (n + 31) / 32));
        cands = {{grid_vs, P}, {grid_g, P}};
    }
    if (forms != kOneLaunchGrid)
        for (const Form &f : {cl_vs, cl_g})
            for (const int cs : {16, 8}) cands.push_back({f, cs});
    Form form{};
    int P = 0;
    int64_t rows_per = 0;
    size_t smem = 0;
    for (const auto &cd : cands) {
        const int64_t rp = (n + cd.second - 1) / cd.second;
        const size_t sm = smem_bytes(rp, m, cd.first.vs, cd.first.threads);
        if (sm > kMaxSmem || !launch_fits(cd.first.kern, cd.first.cluster, c.device, c.num_sms, sm, cd.second,
                                          cd.first.threads))
            continue;
        form = cd.first;
        P = cd.second;
        rows_per = rp;
        smem = sm;
        break;
    }
    if (P == 0) return false;

    // workspace: basis (or its newest vector), grid partials, barrier words
    const int ws_slot = level == 0 ? kScratchSolver : kScratchSolverNested + 2 * (level - 1);
    const size_t vbytes = (size_t)(form.vs ? 1 : m + 1) * n * 16;
    const size_t pbytes = form.cluster ? 0 : (size_t)3 * (m + 2) * P * 16;
    char *ws = static_cast<char *>(c.scratch(ws_slot, vbytes + pbytes + 16));
    unsigned *bar = reinterpret_cast<unsigned *>(ws + vbytes + pbytes);
    if (!form.cluster) BIE_CUDA(cudaMemsetAsync(bar, 0, 8, c.stream));

    CgArgs a{};
    a.rp = A.rp;
    a.cols = A.cols;
    a.val = A.val;
    a.diag = A.diag;
    a.N = A.N;
    a.n = n;
    a.b = b;
    a.x = x;
    a.V = reinterpret_cast<double2 *>(ws);
    a.gpart = reinterpret_cast<double2 *>(ws + vbytes);
    a.bar = bar;
    a.err = d_err;
    a.rows_per = rows_per;
    a.m = m;
    a.maxiter = maxiter;
    a.reltol = o.reltol > 0 ? o.reltol : std::sqrt(2.220446049250313e-16);
    a.abstol = std::max(0.0, o.abstol);
    a.info = d_info;
    a.acc = d_acc;

    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(P);
    cfg.blockDim = dim3(form.threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = c.stream;
    cudaLaunchAttribute at[1];
    if (form.cluster) {
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = P;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
    } else {
        at[0].id = cudaLaunchAttributeCooperative;
        at[0].val.cooperative = 1;
    }
    cfg.attrs = at;
    cfg.numAttrs = 1;
    void *args[] = {&a};
    BIE_CUDA(cudaLaunchKernelExC(&cfg, form.kern, args));
    ++c.kernel_launches;
    return true;
}

}  // namespace bie
