// Host set-up of the near-field (sparse) assembly:
//   * connected_sources (src/3d/assembly_collocation_losses.jl:98-132): for every
//     collocation node the elements that contain it (depth 1) or contain one of
//     its neighbours (depth 2), and the physics nodes of those elements;
//   * the adaptive singular rules of sparse_assemble_parallel!
//     (src/3d/assembly_collocation_losses.jl:200-254) built by subdivide_triangle /
//     singular_triangle_integration (src/3d/adaptive_integration.jl:172-246):
//     the reference triangle is split into four recursively towards the
//     barycentric point of element node c (shifted by `offset`), and a scaled
//     copy of the 3-point rule is placed in every kept sub-triangle;
//   * the coarse rule of partial_assemble_parallel!
//     (src/3d/fast_multipole_method.jl:11-81): gauss_points_triangle(n_gauss).
// All of it is mesh geometry only; the k-dependent integration runs on the GPU
// (bie_nearfield.cu).
#include "bie_internal.h"

#include <algorithm>
#include <cmath>

namespace bie {

namespace {

struct P2 {
    double u, v;
};

// barycentric image (N1, N2, N3) = (1 - u - v, u, v) of a point of the
// reference triangle (the linear basis used by the subdivision)
inline void bary(const P2 &p, double *out) {
    out[0] = (1.0 - p.u) - p.v;
    out[1] = p.u;
    out[2] = p.v;
}

inline double dist3(const double *a, const double *b) {
    const double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    return std::sqrt((dx * dx + dy * dy) + dz * dz);
}

// subdivide_triangle: depth-first, kept triangles appended in order
void subdivide(const P2 &P1, const P2 &P2_, const P2 &P3, const double *src, double esize,
               double tol, std::vector<P2> &out) {
    const P2 P12{(P1.u + P2_.u) / 2, (P1.v + P2_.v) / 2};
    const P2 P23{(P2_.u + P3.u) / 2, (P2_.v + P3.v) / 2};
    const P2 P31{(P3.u + P1.u) / 2, (P3.v + P1.v) / 2};
    const P2 C{(P1.u + P2_.u + P3.u) / 3.0, (P1.v + P2_.v + P3.v) / 3.0};
    double pc[3], p1[3], p2[3], p3[3];
    bary(C, pc);
    bary(P1, p1);
    bary(P2_, p2);
    bary(P3, p3);
    const double dist = std::min(std::min(dist3(pc, src), dist3(p1, src)),
                                 std::min(dist3(p2, src), dist3(p3, src)));
    double size = std::max(std::max(dist3(p2, p1), dist3(p3, p2)), dist3(p1, p3));
    if (size < esize * tol) size = 0;
    if (size > dist / 4) {
        subdivide(P1, P12, P31, src, esize, tol, out);
        subdivide(P12, P2_, P23, src, esize, tol, out);
        subdivide(P31, P23, P3, src, esize, tol, out);
        subdivide(P12, P23, P31, src, esize, tol, out);
    } else {
        out.push_back(P1);
        out.push_back(P2_);
        out.push_back(P3);
    }
}

}  // namespace

// singular_triangle_integration(shape, 3, source, Diagonal(ones(3)), 1e-6) for the
// barycentric source of element node `node` (1..6) with offset `off`.
Rule singular_rule(int node, double off) {
    double src[3];
    switch (node) {
        case 1: src[0] = 1.0; src[1] = off; src[2] = off; break;
        case 2: src[0] = off; src[1] = 1.0; src[2] = off; break;
        case 3: src[0] = off; src[1] = off; src[2] = 1.0; break;
        case 4: src[0] = 0.5; src[1] = 0.5; src[2] = off; break;
        case 5: src[0] = off; src[1] = 0.5; src[2] = 0.5; break;
        case 6: src[0] = 0.5; src[1] = off; src[2] = 0.5; break;
        default: fail(BIE_ERR_INVALID, "singular_rule: node must be 1..6");
    }
    const double esize = std::sqrt(2.0);   // maximum side length of the identity "element"
    std::vector<P2> tri;
    subdivide({0.0, 0.0}, {1.0, 0.0}, {0.0, 1.0}, src, esize, 1e-6, tri);
    const Rule g = triangle_gauss_rule(3);
    const double third = 1.0 / 3.0;
    Rule r;
    const size_t nt = tri.size() / 3;
    r.u.reserve(nt * 3);
    for (size_t t = 0; t < nt; ++t) {
        const P2 &a = tri[3 * t], &b = tri[3 * t + 1], &c = tri[3 * t + 2];
        auto side = [](const P2 &p, const P2 &q) {
            const double du = q.u - p.u, dv = q.v - p.v;
            return std::sqrt(du * du + dv * dv);
        };
        const double dim = std::min(std::min(side(a, b), side(b, c)), side(c, a));
        const double cu = ((a.u + b.u) + c.u) / 3, cv = ((a.v + b.v) + c.v) / 3;
        for (int q = 0; q < g.size(); ++q) {
            r.u.push_back((g.u[q] - third) * dim + cu);
            r.v.push_back((g.v[q] - third) * dim + cv);
            r.w.push_back(g.w[q] * (dim * dim));
        }
    }
    return r;
}

void build_nearfield(Ctx &c, NearField &nf, int depth, double offset, int n_gauss) {
    if (depth != 1 && depth != 2) fail(BIE_ERR_INVALID, "depth must be 1 or 2");
    if (!(offset >= 0.0) || offset > 1.0) fail(BIE_ERR_INVALID, "offset must be in [0, 1]");
    nf.depth = depth;
    nf.offset = offset;
    nf.n_gauss = n_gauss;
    const int NP = c.lay.NP, NS = c.NS;
    const int64_t N = c.n_sources, E = c.n_elements;

    // ---- connected_sources (continuous physics) ----------------------------
    std::vector<std::vector<int32_t>> econ(N), scon(N);
    for (int64_t e = 0; e < E; ++e)
        for (int a = 0; a < NP; ++a) {
            const int32_t nd = c.ptopo[NP * e + a];
            econ[nd].push_back((int32_t)e);
            for (int b = 0; b < NP; ++b) scon[nd].push_back(c.ptopo[NP * e + b]);
        }
    auto uniq = [](std::vector<int32_t> &v) {
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
    };
    if (depth == 2) {
        std::vector<std::vector<int32_t>> e2(N), s2(N);
        for (int64_t i = 0; i < N; ++i) {
            for (int32_t j : scon[i]) {
                e2[i].insert(e2[i].end(), econ[j].begin(), econ[j].end());
                s2[i].insert(s2[i].end(), scon[j].begin(), scon[j].end());
            }
        }
        econ.swap(e2);
        scon.swap(s2);
    }
    for (int64_t i = 0; i < N; ++i) {
        uniq(econ[i]);
        uniq(scon[i]);
    }
    // ---- CSR pattern and pair table ----------------------------------------
    nf.row_ptr.assign(N + 1, 0);
    for (int64_t i = 0; i < N; ++i) nf.row_ptr[i + 1] = nf.row_ptr[i] + (int64_t)scon[i].size();
    nf.cols.resize(nf.row_ptr[N]);
    for (int64_t i = 0; i < N; ++i)
        std::copy(scon[i].begin(), scon[i].end(), nf.cols.begin() + nf.row_ptr[i]);
    nf.pair_stride = 2 + NP;
    nf.pairs.clear();
    for (int64_t i = 0; i < N; ++i)
        for (int32_t e : econ[i]) {
            nf.pairs.push_back((int32_t)i);
            nf.pairs.push_back(e);
            for (int a = 0; a < NP; ++a) {
                const int32_t nd = c.ptopo[NP * (int64_t)e + a];
                const auto it = std::lower_bound(scon[i].begin(), scon[i].end(), nd);
                nf.pairs.push_back((int32_t)(nf.row_ptr[i] + (it - scon[i].begin())));
            }
        }
    nf.npairs = (int64_t)nf.pairs.size() / nf.pair_stride;

    // ---- rule tables: per point N[NS] dNu[NS] dNv[NS] Phi[NP] w ----------------
    const int R = (NS == 3) ? 3 : 6;   // closest geometry node picks the rule
    nf.point_stride = 3 * NS + NP + 1;
    std::vector<double> tab;
    auto append_rule = [&](const Rule &rule) {
        double N_[6], du[6], dv[6], ph[6];
        for (int q = 0; q < rule.size(); ++q) {
            shape_values(c.shape_kind, rule.u[q], rule.v[q], N_);
            shape_derivs(c.shape_kind, rule.u[q], rule.v[q], du, dv);
            shape_values(c.physics_kind, rule.u[q], rule.v[q], ph);
            for (int a = 0; a < NS; ++a) tab.push_back(N_[a]);
            for (int a = 0; a < NS; ++a) tab.push_back(du[a]);
            for (int a = 0; a < NS; ++a) tab.push_back(dv[a]);
            for (int a = 0; a < NP; ++a) tab.push_back(ph[a]);
            tab.push_back(rule.w[q]);
        }
    };
    nf.nrules = R;
    for (int r = 0; r < R; ++r) {
        const Rule rule = singular_rule(r + 1, offset);
        nf.rule_off[r] = (int64_t)tab.size() / nf.point_stride;
        nf.rule_q[r] = rule.size();
        append_rule(rule);
    }
    const Rule coarse = triangle_gauss_rule(n_gauss);
    nf.coarse_off = (int64_t)tab.size() / nf.point_stride;
    nf.coarse_q = coarse.size();
    append_rule(coarse);
    nf.table = std::move(tab);

    // ---- device copies -------------------------------------------------------
    BIE_CUDA(cudaMalloc(&nf.d_pairs, nf.pairs.size() * sizeof(int32_t)));
    BIE_CUDA(cudaMalloc(&nf.d_table, nf.table.size() * sizeof(double)));
    BIE_CUDA(cudaMemcpy(nf.d_pairs, nf.pairs.data(), nf.pairs.size() * sizeof(int32_t),
                        cudaMemcpyHostToDevice));
    BIE_CUDA(cudaMemcpy(nf.d_table, nf.table.data(), nf.table.size() * sizeof(double),
                        cudaMemcpyHostToDevice));
    if (!c.d_coords) {
        BIE_CUDA(cudaMalloc(&c.d_coords, c.coords.size() * sizeof(double)));
        BIE_CUDA(cudaMemcpy(c.d_coords, c.coords.data(), c.coords.size() * sizeof(double),
                            cudaMemcpyHostToDevice));
        BIE_CUDA(cudaMalloc(&c.d_topo, c.topo.size() * sizeof(int32_t)));
        BIE_CUDA(cudaMemcpy(c.d_topo, c.topo.data(), c.topo.size() * sizeof(int32_t),
                            cudaMemcpyHostToDevice));
    }
    nf.ready = true;
}

void free_nearfield(NearField &nf) {
    cudaFree(nf.d_pairs);
    cudaFree(nf.d_table);
    nf.d_pairs = nullptr;
    nf.d_table = nullptr;
    nf.ready = false;
}

NearField &get_nearfield(Ctx &c, int depth, double offset, int n_gauss) {
    // the reference integrates discontinuous physics near the source with
    // polar rules (assembly_collocation_losses.jl:409-447), not restated here
    if (is_discontinuous(c.physics_kind))
        fail(BIE_ERR_UNSUPPORTED, "the near field takes continuous physics only");
    for (auto &p : c.nearfields)
        if (p->depth == depth && p->offset == offset && p->n_gauss == n_gauss) return *p;
    c.nearfields.emplace_back(new NearField());
    NearField &nf = *c.nearfields.back();
    build_nearfield(c, nf, depth, offset, n_gauss);
    return nf;
}

}  // namespace bie
