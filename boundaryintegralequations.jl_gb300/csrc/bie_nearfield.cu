// Near-field (sparse) FP64 assembly: the GPU counterpart of
// sparse_assemble_parallel! (src/3d/assembly_collocation_losses.jl:200-405, with
// sparse_computing_integrals! :158-186) and of the coarse partial assembly
// partial_assemble_parallel! (src/3d/fast_multipole_method.jl:11-81).
//
// One warp per (collocation node, connected element) pair: the warp picks the
// rule of the geometry node nearest to the target (find_closest_corner on the
// element's geometry nodes, Julia hypot semantics) — or the coarse Gauss rule —
// and its lanes stride over the rule's points (3711 points for a corner rule,
// 10623 for an edge-midpoint rule at offset 0).  Per point the geometry is
// interpolated from the element's nodes (tabulated shape functions and
// derivatives), the jacobian and negated unit normal formed as in jacobian!
// (src/3d/jacobian.jl:78-87), and the F and G integrands of kernels.jl:13-37
// accumulated per physics node.  A warp-shuffle reduction gives the element's
// contributions, which lane 0 adds (FP64 atomics) to the pair's CSR slots.
// FP64 throughout: these are the singular and near-singular integrals.
#include "bie_internal.h"
#include "bie_device.cuh"

namespace bie {

namespace {

constexpr double kInv4Pi = 0.07957747154594767;

struct RuleSet {
    int64_t off[kMaxRules];
    int q[kMaxRules];
    int64_t coarse_off;
    int coarse_q;
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <int NS, int NP, bool CPLX_K>
__global__ void __launch_bounds__(256)
nearfield_kernel(const int32_t *__restrict__ pairs, int pstride, int64_t npairs,
                 const double *__restrict__ table, int tstride, RuleSet rs, bool coarse,
                 const double *__restrict__ coords, const int32_t *__restrict__ topo,
                 const double *__restrict__ tgt, double kre, double kim, int flags, double sign,
                 double2 *__restrict__ Fv, double2 *__restrict__ Gv) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const bool doF = flags & BIE_F, doG = flags & BIE_G;
    for (int64_t p = warp; p < npairs; p += nwarps) {
        const int32_t *pr = pairs + p * pstride;
        const int64_t i = pr[0];
        const int64_t e = pr[1];
        double X[3 * NS];
#pragma unroll
        for (int a = 0; a < NS; ++a) {
            const double *xa = coords + 3 * (int64_t)topo[(int64_t)NS * e + a];
            X[3 * a] = xa[0];
            X[3 * a + 1] = xa[1];
            X[3 * a + 2] = xa[2];
        }
        const double tx = tgt[3 * i], ty = tgt[3 * i + 1], tz = tgt[3 * i + 2];
        int64_t base;
        int Q;
        if (coarse) {
            base = rs.coarse_off;
            Q = rs.coarse_q;
        } else {
            const int c = dev::nearest_node<NS>(X, tx, ty, tz);
            base = rs.off[c];
            Q = rs.q[c];
        }
        double fr[NP], fi[NP], gr[NP], gi[NP];
#pragma unroll
        for (int a = 0; a < NP; ++a) fr[a] = fi[a] = gr[a] = gi[a] = 0.0;
        for (int q = lane; q < Q; q += 32) {
            // The subdivided rules put points within 1e-6 element sizes of the
            // singular node, where x_q - t and n.(x_q - t) cancel: the geometry
            // is therefore evaluated with separately rounded products and sums
            // in the reference's order (interpolation, cross product, Julia
            // hypot for the jacobian and the distance, IEEE division for the
            // normal), so the result does not depend on FMA contraction.
            const double *P = table + (base + q) * tstride;
            double x[3] = {0, 0, 0}, tu[3] = {0, 0, 0}, tv[3] = {0, 0, 0};
#pragma unroll
            for (int a = 0; a < NS; ++a) {
                const double Na = P[a], Ua = P[NS + a], Va = P[2 * NS + a];
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    x[k] = __dadd_rn(x[k], __dmul_rn(X[3 * a + k], Na));
                    tu[k] = __dadd_rn(tu[k], __dmul_rn(X[3 * a + k], Ua));
                    tv[k] = __dadd_rn(tv[k], __dmul_rn(X[3 * a + k], Va));
                }
            }
            const double n0 = __dsub_rn(__dmul_rn(tu[1], tv[2]), __dmul_rn(tu[2], tv[1]));
            const double n1 = __dsub_rn(__dmul_rn(tu[2], tv[0]), __dmul_rn(tu[0], tv[2]));
            const double n2 = __dsub_rn(__dmul_rn(tu[0], tv[1]), __dmul_rn(tu[1], tv[0]));
            const double jac = dev::julia_hypot3(n0, n1, n2);
            const double jw = __dmul_rn(jac, P[3 * NS + NP]);
            const double nx = __ddiv_rn(-n0, jac), ny = __ddiv_rn(-n1, jac), nz = __ddiv_rn(-n2, jac);
            const double dx = __dsub_rn(x[0], tx), dy = __dsub_rn(x[1], ty), dz = __dsub_rn(x[2], tz);
            const double rr = dev::julia_hypot3(dx, dy, dz);
            const double rinv = __ddiv_rn(1.0, rr);
            double sn, cs;
            sincos(kre * rr, &sn, &cs);
            if (CPLX_K) {
                const double damp = exp(-kim * rr);
                sn *= damp;
                cs *= damp;
            }
            const double wg = rinv * kInv4Pi * jw;
            const double Gr = cs * wg, Gi = sn * wg;
            const double dn = __dadd_rn(__dadd_rn(__dmul_rn(nx, dx), __dmul_rn(ny, dy)), __dmul_rn(nz, dz));
            const double tq = dn * (rinv * rinv * rinv) * kInv4Pi * jw;
            const double ar = CPLX_K ? (-1.0 - kim * rr) : -1.0;
            const double ai = kre * rr;
            const double Fr = (cs * ar - sn * ai) * tq;
            const double Fi = (cs * ai + sn * ar) * tq;
            const double *ph = P + 3 * NS;
#pragma unroll
            for (int a = 0; a < NP; ++a) {
                fr[a] += Fr * ph[a];
                fi[a] += Fi * ph[a];
                gr[a] += Gr * ph[a];
                gi[a] += Gi * ph[a];
            }
        }
#pragma unroll
        for (int a = 0; a < NP; ++a) {
            if (doF) {
                fr[a] = warp_sum(fr[a]);
                fi[a] = warp_sum(fi[a]);
            }
            if (doG) {
                gr[a] = warp_sum(gr[a]);
                gi[a] = warp_sum(gi[a]);
            }
        }
        if (lane == 0) {
#pragma unroll
            for (int a = 0; a < NP; ++a) {
                const int64_t slot = pr[2 + a];
                if (doF) {
                    atomicAdd(&Fv[slot].x, sign * fr[a]);
                    atomicAdd(&Fv[slot].y, sign * fi[a]);
                }
                if (doG) {
                    atomicAdd(&Gv[slot].x, sign * gr[a]);
                    atomicAdd(&Gv[slot].y, sign * gi[a]);
                }
            }
        }
    }
}

template <int NS, int NP>
void launch_ns_np(Ctx &c, const NearField &nf, double kre, double kim, int flags, bool coarse,
                  double sign, double *Fv, double *Gv) {
    RuleSet rs{};
    for (int r = 0; r < nf.nrules; ++r) {
        rs.off[r] = nf.rule_off[r];
        rs.q[r] = nf.rule_q[r];
    }
    rs.coarse_off = nf.coarse_off;
    rs.coarse_q = nf.coarse_q;
    const int64_t warps = std::min<int64_t>(nf.npairs, (int64_t)c.num_sms * 64);
    const unsigned blocks = (unsigned)std::max<int64_t>(1, (warps * 32 + 255) / 256);
    const bool cplx = kim != 0.0;
    cudaEvent_t t0 = c.timer_begin();
    if (cplx)
        nearfield_kernel<NS, NP, true><<<blocks, 256, 0, c.stream>>>(
            nf.d_pairs, nf.pair_stride, nf.npairs, nf.d_table, nf.point_stride, rs, coarse,
            c.d_coords, c.d_topo, c.d_sources, kre, kim, flags, sign,
            reinterpret_cast<double2 *>(Fv), reinterpret_cast<double2 *>(Gv));
    else
        nearfield_kernel<NS, NP, false><<<blocks, 256, 0, c.stream>>>(
            nf.d_pairs, nf.pair_stride, nf.npairs, nf.d_table, nf.point_stride, rs, coarse,
            c.d_coords, c.d_topo, c.d_sources, kre, kim, flags, sign,
            reinterpret_cast<double2 *>(Fv), reinterpret_cast<double2 *>(Gv));
    BIE_CUDA(cudaGetLastError());
    c.timer_end(t0);
    ++c.kernel_launches;
}

}  // namespace

void launch_nearfield(Ctx &c, const NearField &nf, double k_re, double k_im, int flags, bool coarse,
                      double sign, double *Fv, double *Gv) {
    if (nf.npairs == 0 || !(flags & (BIE_F | BIE_G))) return;
    if (c.NS == 3 && c.lay.NP == 3) launch_ns_np<3, 3>(c, nf, k_re, k_im, flags, coarse, sign, Fv, Gv);
    else if (c.NS == 6 && c.lay.NP == 6) launch_ns_np<6, 6>(c, nf, k_re, k_im, flags, coarse, sign, Fv, Gv);
    else if (c.NS == 6 && c.lay.NP == 3) launch_ns_np<6, 3>(c, nf, k_re, k_im, flags, coarse, sign, Fv, Gv);
    else fail(BIE_ERR_UNSUPPORTED, "near-field assembly for this element combination");
}

}  // namespace bie
