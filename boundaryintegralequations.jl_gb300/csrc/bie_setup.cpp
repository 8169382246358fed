// Host-side set-up of a libbiegpu context: quadrature rules, shape functions,
// per-element quadrature geometry, element ordering and slicing.
//
// Reference behaviour followed (BoundaryIntegralEquations.jl):
//   Gauss-Legendre on [0,1]           src/2d/quadrature.jl:5-11
//   Duffy rules clustered at nodes    src/3d/quadrature.jl:70-113
//   midpoint (two half-Duffy) rules   src/3d/quadrature.jl:116-144
//   triangle shape functions          src/3d/surface_functions.jl:191-236
//   rule per closest node, tables     src/3d/assembly_collocation.jl:122-136, 284-305, 369-413
//   element interpolation + jacobian  src/3d/assembly_collocation.jl:27-66, src/3d/jacobian.jl:78-87
#include "bie_internal.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <utility>

namespace bie {

[[noreturn]] void fail(int code, const std::string &msg) { throw Error{code, msg}; }

void cuda_check(cudaError_t e, const char *what) {
    if (e != cudaSuccess) {
        int code = (e == cudaErrorMemoryAllocation) ? BIE_ERR_NOMEM : BIE_ERR_CUDA;
        fail(code, std::string(what) + ": " + cudaGetErrorString(e));
    }
}

// ---------------------------------------------------------------------------
// Gauss-Legendre: Newton iteration on the three-term Legendre recurrence, run in
// long double and rounded once, so the nodes/weights are correctly rounded to
// within an ulp of the exact values (the reference takes them from
// FastGaussQuadrature.gausslegendre, which is accurate to the same level).
// ---------------------------------------------------------------------------
void gauss_legendre(int n, std::vector<double> &x, std::vector<double> &w) {
    if (n < 1) fail(BIE_ERR_INVALID, "gauss_legendre: n must be >= 1");
    x.assign(n, 0.0);
    w.assign(n, 0.0);
    const long double pi = 3.141592653589793238462643383279502884L;
    for (int i = 0; i < (n + 1) / 2; ++i) {
        // initial guess for the (i+1)-th largest root
        long double z = std::cos(pi * (i + 0.75L) / (n + 0.5L));
        long double pn = 0, dpn = 1;
        for (int it = 0; it < 100; ++it) {
            long double p0 = 1, p1 = z;
            for (int j = 2; j <= n; ++j) {
                long double p2 = ((2 * j - 1) * z * p1 - (j - 1) * p0) / j;
                p0 = p1;
                p1 = p2;
            }
            pn = (n == 1) ? z : p1;
            long double pm = (n == 1) ? 1.0L : p0;
            dpn = n * (z * pn - pm) / (z * z - 1.0L);
            long double dz = pn / dpn;
            z -= dz;
            if (std::fabs((double)dz) < 1e-19) break;
        }
        // re-evaluate the derivative at the converged root for the weight
        {
            long double p0 = 1, p1 = z;
            for (int j = 2; j <= n; ++j) {
                long double p2 = ((2 * j - 1) * z * p1 - (j - 1) * p0) / j;
                p0 = p1;
                p1 = p2;
            }
            long double pm = (n == 1) ? 1.0L : p0;
            long double pnn = (n == 1) ? z : p1;
            dpn = n * (z * pnn - pm) / (z * z - 1.0L);
        }
        long double wi = 2.0L / ((1.0L - z * z) * dpn * dpn);
        // ascending order: the largest root goes last
        x[n - 1 - i] = (double)z;
        x[i] = (double)(-z);
        w[n - 1 - i] = (double)wi;
        w[i] = (double)wi;
    }
    if (n % 2 == 1) x[n / 2] = 0.0;
}

// nodes/weights mapped to [0, 1]
static void gl01(int n, std::vector<double> &x, std::vector<double> &w) {
    gauss_legendre(n, x, w);
    for (int i = 0; i < n; ++i) {
        w[i] = 0.5 * w[i];
        x[i] = 0.5 * (x[i] + 1.0);
    }
}

// tensor grid with the u index fastest: point j*n + i has (x_i, y_j, wy_j*wx_i)
static void tensor01(int n, int m, std::vector<double> &u, std::vector<double> &v,
                     std::vector<double> &w) {
    std::vector<double> xn, wn, xm, wm;
    gl01(n, xn, wn);
    gl01(m, xm, wm);
    u.resize(n * m);
    v.resize(n * m);
    w.resize(n * m);
    for (int j = 0; j < m; ++j)
        for (int i = 0; i < n; ++i) {
            u[j * n + i] = xn[i];
            v[j * n + i] = xm[j];
            w[j * n + i] = wm[j] * wn[i];
        }
}

Rule duffy_corner_rule(int n, int m, int corner) {
    if (corner < 1 || corner > 3) fail(BIE_ERR_INVALID, "duffy_corner_rule: corner must be 1..3");
    std::vector<double> u, v, w;
    tensor01(n, m, u, v, w);
    Rule r;
    const int Q = n * m;
    r.u.resize(Q);
    r.v.resize(Q);
    r.w.resize(Q);
    for (int q = 0; q < Q; ++q) {
        double xi, eta, wt;
        if (corner == 1) {          // collapsed towards node 1
            xi = u[q] * v[q];
            eta = (1.0 - u[q]) * v[q];
            wt = w[q] * v[q];
        } else {                    // collapsed towards node 3 (plain Duffy)
            xi = u[q];
            eta = v[q] * (1.0 - u[q]);
            wt = w[q] * std::fabs(1.0 - u[q]);
        }
        if (corner == 3) std::swap(xi, eta);   // mirror: clusters at node 3
        r.u[q] = xi;
        r.v[q] = eta;
        r.w[q] = wt;
    }
    return r;
}

Rule duffy_midpoint_rule(int n, int m, int vertex) {
    if (vertex < 4 || vertex > 6) fail(BIE_ERR_INVALID, "duffy_midpoint_rule: vertex must be 4..6");
    const int me = ((m + 1) / 2) * 2;
    std::vector<double> u, v, w;
    tensor01(n, me, u, v, w);
    const int H = n * me;
    std::vector<double> X(2 * H), Y(2 * H), W(2 * H);
    for (int q = 0; q < H; ++q) {
        X[q] = 0.5 * u[q];
        Y[q] = v[q] * (1.0 - u[q]);
        W[q] = w[q] * (0.5 * (1.0 - u[q]));
        X[H + q] = (u[q] - 0.5) * v[q] + 0.5;
        Y[H + q] = v[q] * (1.0 - u[q]);
        W[H + q] = w[q] * (0.5 * v[q]);
    }
    Rule r;
    r.w = W;
    r.u.resize(2 * H);
    r.v.resize(2 * H);
    for (int q = 0; q < 2 * H; ++q) {
        if (vertex == 4) {
            r.u[q] = X[q];
            r.v[q] = Y[q];
        } else if (vertex == 5) {
            r.u[q] = (1.0 - X[q]) - Y[q];
            r.v[q] = X[q];
        } else {
            r.u[q] = Y[q];
            r.v[q] = (1.0 - X[q]) - Y[q];
        }
    }
    return r;
}

Rule triangle_gauss_rule(int n) {
    // Symmetric rules on the unit triangle (weights sum to 1/2).  These are the
    // standard published Strang-Fix / Dunavant tables, in the same point order as
    // gauss_points_triangle (src/3d/adaptive_integration.jl:13-64).
    static const double r1[] = {1.0 / 3, 1.0 / 3, 0.5};
    static const double r3[] = {1.0 / 6, 1.0 / 6, 1.0 / 6, 2.0 / 3, 1.0 / 6, 1.0 / 6,
                                1.0 / 6, 2.0 / 3, 1.0 / 6};
    static const double r4[] = {1.0 / 3, 1.0 / 3, -9.0 / 32, 0.2, 0.6, 25.0 / 96,
                                0.2, 0.2, 25.0 / 96, 0.6, 0.2, 25.0 / 96};
    static const double r7[] = {
        1.0 / 3, 1.0 / 3, 0.1125,
        0.797426985353087, 0.101286507323456, 0.0629695902724135,
        0.101286507323456, 0.797426985353087, 0.0629695902724135,
        0.101286507323456, 0.101286507323456, 0.0629695902724135,
        0.059715871789770, 0.470142064105115, 0.066197076394253,
        0.470142064105115, 0.059715871789770, 0.066197076394253,
        0.470142064105115, 0.470142064105115, 0.066197076394253};
    static const double r12[] = {
        0.873821971016996, 0.063089014491502, 0.0254224531851035,
        0.063089014491502, 0.873821971016996, 0.0254224531851035,
        0.063089014491502, 0.063089014491502, 0.0254224531851035,
        0.501426509658279, 0.249286745170910, 0.0583931378631895,
        0.249286745170910, 0.501426509658279, 0.0583931378631895,
        0.249286745170910, 0.249286745170910, 0.0583931378631895,
        0.636502499121399, 0.310352451033785, 0.041425537809187,
        0.636502499121399, 0.053145049844816, 0.041425537809187,
        0.310352451033785, 0.636502499121399, 0.041425537809187,
        0.310352451033785, 0.053145049844816, 0.041425537809187,
        0.053145049844816, 0.636502499121399, 0.041425537809187,
        0.053145049844816, 0.310352451033785, 0.041425537809187};
    static const double r13[] = {
        1.0 / 3, 1.0 / 3, -0.074785022233835,
        0.479308067841923, 0.260345966079038, 0.087807628716602,
        0.260345966079038, 0.479308067841923, 0.087807628716602,
        0.260345966079038, 0.260345966079038, 0.087807628716602,
        0.869739794195568, 0.065130102902216, 0.0266736178044195,
        0.065130102902216, 0.869739794195568, 0.0266736178044195,
        0.065130102902216, 0.065130102902216, 0.0266736178044195,
        0.638444188569809, 0.312865496004875, 0.0385568804451285,
        0.638444188569809, 0.048690315425316, 0.0385568804451285,
        0.312865496004875, 0.638444188569809, 0.0385568804451285,
        0.312865496004875, 0.048690315425316, 0.0385568804451285,
        0.048690315425316, 0.638444188569809, 0.0385568804451285,
        0.048690315425316, 0.312865496004875, 0.0385568804451285};
    const double *t = nullptr;
    switch (n) {
        case 1: t = r1; break;
        case 3: t = r3; break;
        case 4: t = r4; break;
        case 7: t = r7; break;
        case 12: t = r12; break;
        case 13: t = r13; break;
        default: fail(BIE_ERR_UNSUPPORTED, "triangle rule with n=" + std::to_string(n) +
                                              " points (supported: 1,3,4,7,12,13)");
    }
    Rule r;
    for (int i = 0; i < n; ++i) {
        r.u.push_back(t[3 * i]);
        r.v.push_back(t[3 * i + 1]);
        r.w.push_back(t[3 * i + 2]);
    }
    return r;
}

int n_nodes_of_kind(int kind) {
    if (kind == BIE_TRI_LINEAR || kind == BIE_TRI_DISC_LINEAR) return 3;
    if (kind == BIE_TRI_QUADRATIC || kind == BIE_TRI_DISC_QUADRATIC) return 6;
    if (kind == BIE_TRI_DISC_CONSTANT) return 1;
    fail(BIE_ERR_UNSUPPORTED, "unknown element kind " + std::to_string(kind));
}

bool is_discontinuous(int kind) {
    return kind == BIE_TRI_DISC_CONSTANT || kind == BIE_TRI_DISC_LINEAR || kind == BIE_TRI_DISC_QUADRATIC;
}

void physics_values(int kind, double beta, double u, double v, double *N) {
    // discontinuous triangles (src/3d/surface_functions.jl:236-318): the
    // continuous bases in psi(s) = (s - beta) / (1 - 3 beta) of the
    // barycentric coordinates
    if (kind == BIE_TRI_DISC_CONSTANT) {
        N[0] = 1.0;
        return;
    }
    if (kind != BIE_TRI_DISC_LINEAR && kind != BIE_TRI_DISC_QUADRATIC) {
        shape_values(kind, u, v, N);
        return;
    }
    const double den = 1.0 - 3.0 * beta;
    const double p3 = (((1.0 - u) - v) - beta) / den, pu = (u - beta) / den, pv = (v - beta) / den;
    if (kind == BIE_TRI_DISC_LINEAR) {
        N[0] = p3;
        N[1] = pu;
        N[2] = pv;
    } else {
        N[0] = p3 * (2.0 * p3 - 1.0);
        N[1] = pu * (2.0 * pu - 1.0);
        N[2] = pv * (2.0 * pv - 1.0);
        N[3] = 4.0 * pu * p3;
        N[4] = 4.0 * pu * pv;
        N[5] = 4.0 * pv * p3;
    }
}

void shape_values(int kind, double u, double v, double *N) {
    if (kind == BIE_TRI_LINEAR) {
        N[0] = (1.0 - u) - v;
        N[1] = u;
        N[2] = v;
    } else {
        const double l = (1.0 - v) - u;
        N[0] = l * ((1.0 - 2.0 * v) - 2.0 * u);
        N[1] = u * (2.0 * u - 1.0);
        N[2] = v * (2.0 * v - 1.0);
        N[3] = 4.0 * u * l;
        N[4] = 4.0 * u * v;
        N[5] = 4.0 * v * l;
    }
}

void physics_derivs(int kind, double beta, double u, double v, double *dNu, double *dNv) {
    // d psi / ds = 1 / (1 - 3 beta) (src/3d/surface_functions.jl:262-318)
    if (kind == BIE_TRI_DISC_CONSTANT) {
        dNu[0] = dNv[0] = 0.0;
        return;
    }
    if (kind != BIE_TRI_DISC_LINEAR && kind != BIE_TRI_DISC_QUADRATIC) {
        shape_derivs(kind, u, v, dNu, dNv);
        return;
    }
    const double den = 1.0 - 3.0 * beta, d = 1.0 / den;
    if (kind == BIE_TRI_DISC_LINEAR) {
        dNu[0] = -d; dNu[1] = d; dNu[2] = 0.0;
        dNv[0] = -d; dNv[1] = 0.0; dNv[2] = d;
        return;
    }
    const double p3 = (((1.0 - u) - v) - beta) / den, pu = (u - beta) / den, pv = (v - beta) / den;
    const double a3 = -(4.0 * p3 - 1.0) * d;
    dNu[0] = a3; dNu[1] = (4.0 * pu - 1.0) * d; dNu[2] = 0.0;
    dNu[3] = 4.0 * d * p3 - 4.0 * pu * d; dNu[4] = 4.0 * d * pv; dNu[5] = -4.0 * pv * d;
    dNv[0] = a3; dNv[1] = 0.0; dNv[2] = (4.0 * pv - 1.0) * d;
    dNv[3] = -4.0 * pu * d; dNv[4] = 4.0 * pu * d; dNv[5] = 4.0 * d * p3 - 4.0 * pv * d;
}

void shape_derivs(int kind, double u, double v, double *dNu, double *dNv) {
    if (kind == BIE_TRI_LINEAR) {
        dNu[0] = -1; dNu[1] = 1; dNu[2] = 0;
        dNv[0] = -1; dNv[1] = 0; dNv[2] = 1;
    } else {
        const double l = (1.0 - v) - u;
        const double d1 = -(2.0 * l - 1.0) - 2.0 * l;
        dNu[0] = d1; dNu[1] = 4.0 * u - 1.0; dNu[2] = 0.0;
        dNu[3] = 4.0 * l - 4.0 * u; dNu[4] = 4.0 * v; dNu[5] = -4.0 * v;
        dNv[0] = d1; dNv[1] = 0.0; dNv[2] = 4.0 * v - 1.0;
        dNv[3] = -4.0 * u; dNv[4] = 4.0 * u; dNv[5] = 4.0 * l - 4.0 * v;
    }
}

// ---------------------------------------------------------------------------
// Morton code of a point in the unit cube (10 bits per axis)
// ---------------------------------------------------------------------------
static uint32_t spread10(uint32_t x) {
    x &= 0x3ff;
    x = (x | (x << 16)) & 0x030000ff;
    x = (x | (x << 8)) & 0x0300f00f;
    x = (x | (x << 4)) & 0x030c30c3;
    x = (x | (x << 2)) & 0x09249249;
    return x;
}

void *Ctx::scratch(int slot, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (scratch_bytes[slot] < bytes) {
        if (capturing) fail(BIE_ERR_INVALID, "device scratch would grow while a CUDA graph is recorded");
        if (d_scratch[slot]) BIE_CUDA(cudaFree(d_scratch[slot]));
        d_scratch[slot] = nullptr;
        scratch_bytes[slot] = 0;
        BIE_CUDA(cudaMalloc(&d_scratch[slot], bytes));
        scratch_bytes[slot] = bytes;
    }
    return d_scratch[slot];
}

cudaEvent_t Ctx::take_event() {
    if (!ev_free.empty()) {
        cudaEvent_t e = ev_free.back();
        ev_free.pop_back();
        return e;
    }
    cudaEvent_t e;
    BIE_CUDA(cudaEventCreate(&e));
    return e;
}

cudaEvent_t Ctx::timer_begin() {
    if (!timing) return nullptr;
    cudaEvent_t a = take_event();
    BIE_CUDA(cudaEventRecord(a, stream));
    return a;
}

void Ctx::timer_end(cudaEvent_t a) {
    if (!timing || !a) return;
    cudaEvent_t b = take_event();
    BIE_CUDA(cudaEventRecord(b, stream));
    ev_pending.emplace_back(a, b);
    ++timed_launches;
}

void Ctx::tensor_timer_end(cudaEvent_t a, double flops, double flops_executed) {
    if (!timing || !a) return;
    cudaEvent_t b = take_event();
    BIE_CUDA(cudaEventRecord(b, stream));
    ev_tensor.emplace_back(a, b);
    ++tensor_launches;
    tensor_flops += flops;
    tensor_flops_executed += flops_executed;
}

void Ctx::collect_timers() {
    BIE_CUDA(cudaStreamSynchronize(stream));
    for (auto &p : ev_pending) {
        float ms = 0.f;
        BIE_CUDA(cudaEventElapsedTime(&ms, p.first, p.second));
        timed_ms += ms;
        ev_free.push_back(p.first);
        ev_free.push_back(p.second);
    }
    ev_pending.clear();
    for (auto &p : ev_tensor) {
        float ms = 0.f;
        BIE_CUDA(cudaEventElapsedTime(&ms, p.first, p.second));
        tensor_ms += ms;
        ev_free.push_back(p.first);
        ev_free.push_back(p.second);
    }
    ev_tensor.clear();
}

// Element order of the assembly kernels: recursive coordinate bisection of
// the element centroids (topo: 0-based geometry nodes, NS per element).
std::vector<int32_t> bisection_order(const double *coords, int64_t n_coords, const int32_t *topo, int NS,
                                     int64_t E) {
    std::vector<int32_t> order;
    // The range of slice s at level l, [s*E/2^l, (s+1)*E/2^l), is split at
    // the boundary of its two level-(l+1) halves across the longest side of
    // its centroids' bounding box, so every slicing 2^l is a set of compact
    // patches of equal size with short borders (fewer nodes shared between
    // slices than a space-filling-curve order gives).  Ties break on the
    // element index, and the elements of a range of at most two go in Morton
    // order of their centroids, so the order is the same on every host.
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int64_t i = 0; i < n_coords; ++i)
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], coords[3 * i + k]);
            hi[k] = std::max(hi[k], coords[3 * i + k]);
        }
    std::vector<double> cen((size_t)3 * E);
    std::vector<uint32_t> key(E);
    for (int64_t e = 0; e < E; ++e) {
        uint32_t code = 0;
        for (int k = 0; k < 3; ++k) {
            double s = 0;
            for (int a = 0; a < 3; ++a) s += coords[3 * (int64_t)topo[NS * e + a] + k];
            s /= 3.0;
            cen[3 * e + k] = s;
            double span = hi[k] - lo[k];
            double t = span > 0 ? (s - lo[k]) / span : 0.0;
            uint32_t qk = (uint32_t)std::min(1023.0, std::max(0.0, t * 1023.0));
            code |= spread10(qk) << k;
        }
        key[e] = code;
    }
    order.resize(E);
    std::iota(order.begin(), order.end(), 0);
    {
        struct Range { int64_t p0, p1, num, den; };   // [p0, p1) = [num*E/den, (num+1)*E/den)
        std::vector<Range> pending{{0, E, 0, 1}};
        while (!pending.empty()) {
            const Range r = pending.back();
            pending.pop_back();
            auto b = order.begin();
            if (r.p1 - r.p0 <= 2 || r.den > (int64_t(1) << 40)) {
                std::sort(b + r.p0, b + r.p1, [&](int32_t x, int32_t y) {
                    return key[x] != key[y] ? key[x] < key[y] : x < y;
                });
                continue;
            }
            double blo[3] = {1e300, 1e300, 1e300}, bhi[3] = {-1e300, -1e300, -1e300};
            for (int64_t p = r.p0; p < r.p1; ++p)
                for (int k = 0; k < 3; ++k) {
                    blo[k] = std::min(blo[k], cen[3 * (int64_t)order[p] + k]);
                    bhi[k] = std::max(bhi[k], cen[3 * (int64_t)order[p] + k]);
                }
            int ax = 0;
            for (int k = 1; k < 3; ++k)
                if (bhi[k] - blo[k] > bhi[ax] - blo[ax]) ax = k;
            const int64_t den = 2 * r.den, left = 2 * r.num;
            const int64_t mid = (int64_t)((__int128)(left + 1) * E / den);
            std::nth_element(b + r.p0, b + mid, b + r.p1, [&](int32_t x, int32_t y) {
                const double cx = cen[3 * (int64_t)x + ax], cy = cen[3 * (int64_t)y + ax];
                return cx != cy ? cx < cy : x < y;
            });
            pending.push_back({mid, r.p1, left + 1, den});
            pending.push_back({r.p0, mid, left, den});
        }
    }
    return order;
}

// Write protocol of the assembly kernels for every slicing level (order: the
// element order, ptopo: 0-based physics nodes, NP per element, Nn nodes).
void build_write_protocol(const int32_t *order, int64_t E, const int32_t *ptopo, int NP, int64_t Nn,
                          WriteProtocol &w) {
    // ---- shared-node masks for the element slicings S = 2^l ------------------
    // Slice s of S covers sorted positions [s*E/S, (s+1)*E/S).  A node is shared
    // at level l when elements of two different slices touch it; writes to a
    // shared node use atomics, all other writes are plain read-modify-writes by
    // the single thread that owns the (row, node) entry.
    std::vector<uint32_t> &masks = w.masks;
    masks.assign((size_t)kMaxLevels * E, 0u);
    std::vector<int32_t> first(Nn);
    std::vector<uint8_t> shared(Nn);
    std::vector<uint8_t> &node_shared = w.node_shared;
    node_shared.assign((size_t)kMaxLevels * Nn, 0);
    for (int l = 0; l < kMaxLevels; ++l) {
        const int64_t S = int64_t(1) << l;
        std::fill(first.begin(), first.end(), -1);
        std::fill(shared.begin(), shared.end(), 0);
        for (int64_t s = 0; s < S; ++s) {
            const int64_t p0 = s * E / S, p1 = (s + 1) * E / S;
            for (int64_t p = p0; p < p1; ++p) {
                const int64_t e = order[p];
                for (int a = 0; a < NP; ++a) {
                    int32_t nd = ptopo[NP * e + a];
                    if (first[nd] < 0) first[nd] = (int32_t)s;
                    else if (first[nd] != (int32_t)s) shared[nd] = 1;
                }
            }
        }
        for (int64_t p = 0; p < E; ++p) {
            const int64_t e = order[p];
            uint32_t m = 0;
            for (int a = 0; a < NP; ++a)
                if (shared[ptopo[NP * e + a]]) m |= 1u << a;
            masks[(size_t)l * E + p] = m;
        }
        std::copy(shared.begin(), shared.end(), node_shared.begin() + (size_t)l * Nn);
    }

    // ---- write protocol of the mixed assembly per slicing level --------------
    // Each (row, node) entry is written by the one thread that owns its row in
    // the node's slice: its first contribution stores, later ones add, the last
    // one converts; nodes shared between slices go through side slots.
    std::vector<uint32_t> &k2_flags = w.k2_flags;
    k2_flags.assign((size_t)kMaxLevels * E, 0u);
    std::vector<int32_t> &k2_side = w.k2_side;
    k2_side.assign((size_t)kMaxLevels * E * NP, -1);
    std::vector<int32_t> &k2_fix = w.k2_fix;
    k2_fix.clear();
    {
        std::vector<int64_t> stamp(Nn), fpos(Nn), lpos(Nn);
        std::vector<int32_t> slot_of(Nn), ring_of(Nn);
        std::vector<std::vector<int32_t>> node_slots(Nn);
        std::vector<uint8_t> touched(Nn);
        std::vector<int32_t> opened;
        std::vector<std::pair<int64_t, int32_t>> spans;
        for (int l = 0; l < kMaxLevels; ++l) {
            const int64_t S = int64_t(1) << l;
            const uint8_t *sh = node_shared.data() + (size_t)l * Nn;
            std::fill(stamp.begin(), stamp.end(), -1);
            std::fill(touched.begin(), touched.end(), 0);
            std::fill(ring_of.begin(), ring_of.end(), -1);
            for (auto &v : node_slots) v.clear();
            int64_t nside = 0;
            for (int64_t s = 0; s < S; ++s) {
                const int64_t p0 = s * E / S, p1 = (s + 1) * E / S;
                opened.clear();
                for (int64_t p = p0; p < p1; ++p) {
                    const int64_t e = order[p];
                    for (int a = 0; a < NP; ++a) {
                        const int32_t nd = ptopo[NP * e + a];
                        touched[nd] = 1;
                        if (stamp[nd] != s) {
                            stamp[nd] = s;
                            fpos[nd] = p;
                            if (sh[nd]) {
                                if (nside >= INT32_MAX) fail(BIE_ERR_INVALID, "mesh too large for the slot index");
                                slot_of[nd] = (int32_t)nside;
                                node_slots[nd].push_back((int32_t)nside);
                                ++nside;
                            } else {
                                opened.push_back(nd);
                            }
                        }
                        lpos[nd] = p;
                    }
                }
                // ring slots for the slice's own nodes with several
                // contributions: spans [fpos, lpos] in order of their last
                // position, each to the slot that became free latest before
                // the span opens (the most spans of any assignment)
                spans.clear();
                for (int32_t nd : opened)
                    if (fpos[nd] != lpos[nd]) spans.push_back({lpos[nd], nd});
                std::sort(spans.begin(), spans.end());
                int64_t slot_end[kK2RingSlots];
                std::fill(slot_end, slot_end + kK2RingSlots, int64_t(-1));
                for (const auto &sp : spans) {
                    const int32_t nd = sp.second;
                    int best = -1;
                    for (int k = 0; k < kK2RingSlots; ++k)
                        if (slot_end[k] < fpos[nd] && (best < 0 || slot_end[k] > slot_end[best])) best = k;
                    if (best < 0) continue;
                    slot_end[best] = lpos[nd];
                    ring_of[nd] = best;
                }
                for (int64_t p = p0; p < p1; ++p) {
                    const int64_t e = order[p];
                    uint32_t w = 0;
                    for (int a = 0; a < NP; ++a) {
                        const int32_t nd = ptopo[NP * e + a];
                        if (fpos[nd] == p) w |= 1u << a;
                        if (lpos[nd] == p) w |= 1u << (8 + a);
                        if (sh[nd]) {
                            w |= 1u << (16 + a);
                            k2_side[((size_t)l * E + p) * NP + a] = slot_of[nd];
                        } else if (ring_of[nd] >= 0) {
                            w |= 1u << (24 + a);
                            k2_side[((size_t)l * E + p) * NP + a] = ring_of[nd];
                        }
                    }
                    k2_flags[(size_t)l * E + p] = w;
                }
            }
            // fix-up list: shared nodes with their slots, untouched nodes with
            // none; widening list: nodes of one slice with several contributions
            // and no ring slot (their entries hold float partial sums until the
            // widening pass)
            std::vector<int32_t> nodes, ptr{0}, slots, widen;
            int64_t nshared = 0, nring = 0, nsingle = 0;
            for (int64_t nd = 0; nd < Nn; ++nd) {
                if (touched[nd] && !sh[nd]) {
                    if (fpos[nd] == lpos[nd]) ++nsingle;
                    else if (ring_of[nd] >= 0) ++nring;
                    else widen.push_back((int32_t)nd);
                    continue;
                }
                if (sh[nd]) ++nshared;
                nodes.push_back((int32_t)nd);
                for (int32_t k : node_slots[nd]) slots.push_back(k);
                ptr.push_back((int32_t)slots.size());
            }
            w.fix_off[l] = (int64_t)k2_fix.size();
            w.nfix[l] = (int64_t)nodes.size();
            w.nside[l] = nside;
            w.nwiden[l] = (int64_t)widen.size();
            w.nshared[l] = nshared;
            w.nring[l] = nring;
            w.nsingle[l] = nsingle;
            w.nuntouched[l] = (int64_t)nodes.size() - nshared;
            k2_fix.insert(k2_fix.end(), nodes.begin(), nodes.end());
            k2_fix.insert(k2_fix.end(), ptr.begin(), ptr.end());
            k2_fix.insert(k2_fix.end(), slots.begin(), slots.end());
            w.widen_off[l] = (int64_t)k2_fix.size();
            k2_fix.insert(k2_fix.end(), widen.begin(), widen.end());
        }
    }
}

void build_context(Ctx &c, const bie_mesh_desc &d, int device, int gauss_rule,
                   const std::vector<Rule> *explicit_rules) {
    // ---- validation -------------------------------------------------------
    if (d.n_coordinates <= 0 || d.n_elements <= 0 || d.n_sources <= 0)
        fail(BIE_ERR_INVALID, "mesh sizes must be positive");
    if (!d.coordinates || !d.topology || !d.physics_topology || !d.sources)
        fail(BIE_ERR_INVALID, "mesh arrays must not be NULL");
    if (d.n_coordinates > INT32_MAX || d.n_sources > INT32_MAX || d.n_elements > INT32_MAX)
        fail(BIE_ERR_INVALID, "mesh too large for 32-bit node indices");
    if (d.shape_kind != BIE_TRI_LINEAR && d.shape_kind != BIE_TRI_QUADRATIC)
        fail(BIE_ERR_UNSUPPORTED, "geometry must be 3- or 6-node triangles (kind " +
                                      std::to_string(d.shape_kind) + ")");
    const int NS = n_nodes_of_kind(d.shape_kind);
    const int NP = n_nodes_of_kind(d.physics_kind);
    if (d.shape_kind == BIE_TRI_LINEAR && d.physics_kind == BIE_TRI_QUADRATIC)
        fail(BIE_ERR_UNSUPPORTED, "quadratic physics on linear geometry is not supported");
    const bool disc = is_discontinuous(d.physics_kind);
    if (disc && d.physics_kind != BIE_TRI_DISC_CONSTANT &&
        !(d.physics_beta > 0.0 && d.physics_beta < 1.0 / 3.0))
        fail(BIE_ERR_INVALID, "physics_beta of discontinuous physics must lie in (0, 1/3)");
    const bool own_rules = gauss_rule <= 0 && !explicit_rules;
    if (own_rules && (d.quad_n < 1 || d.quad_m < 1 || d.quad_n > 32 || d.quad_m > 32))
        fail(BIE_ERR_INVALID, "quad_n and quad_m must be in 1..32");
    // one rule per physics node; linear geometry has the three corner rules
    // only, so its nodes 4-6 (6-node discontinuous physics) take corner 3's
    const int R = NP;
    const int n_tables = (d.shape_kind == BIE_TRI_LINEAR) ? std::min(NP, 3) : NP;
    if (explicit_rules) {
        if ((int)explicit_rules->size() != n_tables)
            fail(BIE_ERR_INVALID, "expected " + std::to_string(n_tables) +
                                      " rule tables for this element kind, got " +
                                      std::to_string(explicit_rules->size()));
        for (int r = 0; r < n_tables; ++r) {
            const Rule &t = (*explicit_rules)[r];
            if (t.size() < 1 || t.size() > kMaxQ || (int)t.u.size() != t.size() || (int)t.v.size() != t.size())
                fail(BIE_ERR_INVALID, "rule table " + std::to_string(r) + " must hold 1.." +
                                          std::to_string(kMaxQ) + " points");
            for (int q = 0; q < t.size(); ++q) {
                const double u = t.u[q], v = t.v[q], w = t.w[q];
                if (!std::isfinite(u) || !std::isfinite(v) || !std::isfinite(w))
                    fail(BIE_ERR_INVALID, "non-finite value in rule table " + std::to_string(r));
                if (u < 0.0 || v < 0.0 || u + v > 1.0 + 1e-12)
                    fail(BIE_ERR_INVALID, "rule table " + std::to_string(r) + " point " + std::to_string(q) +
                                              " lies outside the reference triangle");
            }
        }
    }
    c.shape_kind = d.shape_kind;
    c.physics_kind = d.physics_kind;
    c.physics_beta = disc ? d.physics_beta : 0.0;
    c.n_coords = d.n_coordinates;
    c.n_elements = d.n_elements;
    c.n_sources = d.n_sources;
    c.NS = NS;
    c.quad_n = own_rules ? d.quad_n : 0;   // 0: the rules did not come from (n, m)
    c.quad_m = own_rules ? d.quad_m : 0;
    const int64_t E = d.n_elements;

    c.coords.assign(d.coordinates, d.coordinates + 3 * d.n_coordinates);
    c.sources.assign(d.sources, d.sources + 3 * d.n_sources);
    for (double x : c.coords)
        if (!std::isfinite(x)) fail(BIE_ERR_INVALID, "non-finite mesh coordinate");
    for (double x : c.sources)
        if (!std::isfinite(x)) fail(BIE_ERR_INVALID, "non-finite source coordinate");
    c.topo.resize((size_t)NS * E);
    c.ptopo.resize((size_t)NP * E);
    for (int64_t i = 0; i < NS * E; ++i) {
        int64_t t = d.topology[i];
        if (t < 1 || t > d.n_coordinates)
            fail(BIE_ERR_INVALID, "topology index out of range at entry " + std::to_string(i));
        c.topo[i] = (int32_t)(t - 1);
    }
    for (int64_t i = 0; i < NP * E; ++i) {
        int64_t t = d.physics_topology[i];
        if (t < 1 || t > d.n_sources)
            fail(BIE_ERR_INVALID, "physics_topology index out of range at entry " + std::to_string(i));
        c.ptopo[i] = (int32_t)(t - 1);
    }

    // ---- clustered rules ---------------------------------------------------
    // Linear geometry: three rules clustered at the corners.  Quadratic geometry:
    // one rule per physics node (corners, then edge midpoints 4-6).
    // gauss_rule > 0: every rule is the symmetric gauss_rule-point triangle rule
    // (the far-field rule of the fast operators, setup_fast_operator,
    // src/3d/fast_multipole_method.jl:163-170), whatever the nearest node.
    c.rules.clear();
    for (int r = 0; r < R; ++r) {
        const int t = std::min(r, n_tables - 1);
        if (explicit_rules) c.rules.push_back((*explicit_rules)[t]);
        else if (gauss_rule > 0) c.rules.push_back(triangle_gauss_rule(gauss_rule));
        else
            c.rules.push_back(t < 3 ? duffy_corner_rule(d.quad_n, d.quad_m, t + 1)
                                    : duffy_midpoint_rule(d.quad_n, d.quad_m, t + 1));
    }
    RecordLayout &L = c.lay;
    L = RecordLayout{};
    L.NP = NP;
    L.R = R;
    int off = 3 * NP;
    for (int r = 0; r < R; ++r) {
        L.Q[r] = c.rules[r].size();
        if (L.Q[r] > kMaxQ)
            fail(BIE_ERR_INVALID, "quadrature rule has more than 64 points; reduce quad_n/quad_m");
        L.qmax = std::max(L.qmax, L.Q[r]);
        L.rule_off[r] = off;
        off += 7 * L.Q[r];
    }
    L.nidx_off = off;
    off += (NP + 1) / 2;
    L.stride = (off + 1) & ~1;

    // physics interpolation at each rule's points: Phi[r][q][a]
    c.phi.assign((size_t)R * L.qmax * NP, 0.0);
    for (int r = 0; r < R; ++r)
        for (int q = 0; q < L.Q[r]; ++q)
            physics_values(d.physics_kind, c.physics_beta, c.rules[r].u[q], c.rules[r].v[q],
                         &c.phi[((size_t)r * L.qmax + q) * NP]);

    // ---- element order -------------------------------------------------------
    c.order = bisection_order(c.coords.data(), d.n_coordinates, c.topo.data(), NS, E);

    // ---- element records (quadrature geometry per rule) ---------------------
    std::vector<double> rec((size_t)E * L.stride, 0.0);
    std::vector<double> N(NS), dNu(NS), dNv(NS);
    for (int64_t p = 0; p < E; ++p) {
        const int64_t e = c.order[p];
        double *R0 = &rec[(size_t)p * L.stride];
        for (int a = 0; a < NP; ++a)
            for (int k = 0; k < 3; ++k)
                R0[3 * a + k] = c.sources[3 * (int64_t)c.ptopo[NP * e + a] + k];
        for (int r = 0; r < R; ++r) {
            const int Q = L.Q[r];
            double *g = R0 + L.rule_off[r];
            for (int q = 0; q < Q; ++q) {
                const double u = c.rules[r].u[q], v = c.rules[r].v[q];
                shape_values(d.shape_kind, u, v, N.data());
                shape_derivs(d.shape_kind, u, v, dNu.data(), dNv.data());
                double x[3] = {0, 0, 0}, t[3] = {0, 0, 0}, s[3] = {0, 0, 0};
                for (int a = 0; a < NS; ++a) {
                    const double *X = &c.coords[3 * (int64_t)c.topo[NS * e + a]];
                    for (int k = 0; k < 3; ++k) {
                        x[k] += X[k] * N[a];
                        t[k] += X[k] * dNu[a];
                        s[k] += X[k] * dNv[a];
                    }
                }
                double nrm[3] = {t[1] * s[2] - t[2] * s[1], t[2] * s[0] - t[0] * s[2],
                                 t[0] * s[1] - t[1] * s[0]};
                double jac = std::hypot(std::hypot(nrm[0], nrm[1]), nrm[2]);
                if (!(jac > 0)) fail(BIE_ERR_INVALID, "degenerate element " + std::to_string(e + 1));
                g[0 * Q + q] = x[0];
                g[1 * Q + q] = x[1];
                g[2 * Q + q] = x[2];
                g[3 * Q + q] = -nrm[0] / jac;
                g[4 * Q + q] = -nrm[1] / jac;
                g[5 * Q + q] = -nrm[2] / jac;
                g[6 * Q + q] = jac * c.rules[r].w[q];
            }
        }
        int32_t *nid = reinterpret_cast<int32_t *>(R0 + L.nidx_off);
        for (int a = 0; a < NP; ++a) nid[a] = c.ptopo[NP * e + a];
    }

    // ---- shared-node masks and the write protocol per slicing level ----------
    WriteProtocol wp;
    build_write_protocol(c.order.data(), E, c.ptopo.data(), NP, d.n_sources, wp);
    for (int l = 0; l < kMaxLevels; ++l) {
        c.k2_fix_off[l] = wp.fix_off[l];
        c.k2_nfix[l] = wp.nfix[l];
        c.k2_nside[l] = wp.nside[l];
        c.k2_widen_off[l] = wp.widen_off[l];
        c.k2_nwiden[l] = wp.nwiden[l];
    }
    const std::vector<uint32_t> &masks = wp.masks;
    const std::vector<uint8_t> &node_shared = wp.node_shared;
    const std::vector<uint32_t> &k2_flags = wp.k2_flags;
    const std::vector<int32_t> &k2_side = wp.k2_side;
    const std::vector<int32_t> &k2_fix = wp.k2_fix;

    // ---- device upload --------------------------------------------------------
    int ndev = 0;
    BIE_CUDA(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev)
        fail(BIE_ERR_INVALID, "device " + std::to_string(device) + " not present (" +
                                  std::to_string(ndev) + " visible)");
    c.device = device;
    BIE_CUDA(cudaSetDevice(device));
    BIE_CUDA(cudaDeviceGetAttribute(&c.num_sms, cudaDevAttrMultiProcessorCount, device));
    BIE_CUDA(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
    BIE_CUDA(cudaMalloc(&c.d_records, rec.size() * sizeof(double)));
    BIE_CUDA(cudaMalloc(&c.d_phi, c.phi.size() * sizeof(double)));
    BIE_CUDA(cudaMalloc(&c.d_sources, c.sources.size() * sizeof(double)));
    BIE_CUDA(cudaMalloc(&c.d_shared_mask, masks.size() * sizeof(uint32_t)));
    BIE_CUDA(cudaMalloc(&c.d_node_shared, node_shared.size()));
    BIE_CUDA(cudaMemcpy(c.d_node_shared, node_shared.data(), node_shared.size(), cudaMemcpyHostToDevice));
    BIE_CUDA(cudaMalloc(&c.d_qpe, sizeof(unsigned long long)));
    BIE_CUDA(cudaMemset(c.d_qpe, 0, sizeof(unsigned long long)));
    BIE_CUDA(cudaMemcpy(c.d_records, rec.data(), rec.size() * sizeof(double), cudaMemcpyHostToDevice));
    BIE_CUDA(cudaMemcpy(c.d_phi, c.phi.data(), c.phi.size() * sizeof(double), cudaMemcpyHostToDevice));
    BIE_CUDA(cudaMemcpy(c.d_sources, c.sources.data(), c.sources.size() * sizeof(double),
                        cudaMemcpyHostToDevice));
    BIE_CUDA(cudaMemcpy(c.d_shared_mask, masks.data(), masks.size() * sizeof(uint32_t),
                        cudaMemcpyHostToDevice));
    BIE_CUDA(cudaMalloc(&c.d_k2_flags, k2_flags.size() * sizeof(uint32_t)));
    BIE_CUDA(cudaMalloc(&c.d_k2_side, k2_side.size() * sizeof(int32_t)));
    BIE_CUDA(cudaMalloc(&c.d_k2_fix, std::max<size_t>(1, k2_fix.size()) * sizeof(int32_t)));
    BIE_CUDA(cudaMemcpy(c.d_k2_flags, k2_flags.data(), k2_flags.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    BIE_CUDA(cudaMemcpy(c.d_k2_side, k2_side.data(), k2_side.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    if (!k2_fix.empty())
        BIE_CUDA(cudaMemcpy(c.d_k2_fix, k2_fix.data(), k2_fix.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    build_mixed_records(c, rec);
    prepare_noalloc(c);
}

void destroy_context(Ctx &c) {
    if (c.device >= 0) cudaSetDevice(c.device);
    if (c.stream) cudaStreamSynchronize(c.stream);
    cudaFree(c.d_records);
    cudaFree(c.d_phi);
    cudaFree(c.d_sources);
    cudaFree(c.d_shared_mask);
    cudaFree(c.d_node_shared);
    c.d_node_shared = nullptr;
    cudaFree(c.d_k2_flags);
    cudaFree(c.d_k2_side);
    cudaFree(c.d_k2_fix);
    c.d_k2_flags = nullptr;
    c.d_k2_side = nullptr;
    c.d_k2_fix = nullptr;
    cudaFree(c.d_mrecords);
    cudaFree(c.d_mphi);
    c.d_mrecords = nullptr;
    c.d_mphi = nullptr;
    cudaFree(c.d_drecords);
    cudaFree(c.d_dphi);
    cudaFree(c.d_phase_tab);
    c.d_phase_tab = nullptr;
    c.d_drecords = nullptr;
    c.d_dphi = nullptr;
    for (auto &nf : c.nearfields) free_nearfield(*nf);
    c.nearfields.clear();
    cudaFree(c.d_coords);
    cudaFree(c.d_topo);
    c.d_coords = nullptr;
    c.d_topo = nullptr;
    cudaFree(c.d_qpe);
    for (int i = 0; i < kScratchCount; ++i) cudaFree(c.d_scratch[i]);
    for (auto &p : c.ev_pending) {
        cudaEventDestroy(p.first);
        cudaEventDestroy(p.second);
    }
    for (auto &p : c.ev_tensor) {
        cudaEventDestroy(p.first);
        cudaEventDestroy(p.second);
    }
    for (auto e : c.ev_free) cudaEventDestroy(e);
    c.ev_pending.clear();
    c.ev_tensor.clear();
    c.ev_free.clear();
    c.d_qpe = nullptr;
    if (c.copy_stream) {
        cudaStreamSynchronize(c.copy_stream);
        cudaStreamDestroy(c.copy_stream);
        c.copy_stream = nullptr;
    }
    if (c.stream && c.owns_stream) cudaStreamDestroy(c.stream);
    c.d_records = nullptr;
    c.d_phi = nullptr;
    c.d_sources = nullptr;
    c.d_shared_mask = nullptr;
    c.stream = nullptr;
}

}  // namespace bie
