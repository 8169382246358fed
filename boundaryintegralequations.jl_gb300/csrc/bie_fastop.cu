// Fast operators: the algorithm of FMMFOperator / FMMGOperator
// (src/3d/fast_multipole_method.jl:163-194, 220-324, 347-490) with the
// FMM3D far-field sum replaced by an exact direct sum on the GPU.
//
//   y = K_gauss x + (S - C_coarse) x
//
// K_gauss: every (collocation node, element) pair integrated with the
//   symmetric n_gauss-point triangle rule (setup_fast_operator's
//   `set_interpolation_nodes!(shape_function, gauss_points_triangle(n_gauss)...)`
//   and C_map = jacobian x weight x physics interpolation, create_coefficient_map
//   :120-137); the reference evaluates the sum with hfmm3d (charges for G,
//   dipoles n x coefficient for F) to tolerance `tol`; here it is the
//   matrix-free product of a context whose every rule is that Gauss rule
//   (FP64 exact, or mixed precision).
// S - C_coarse: nearfield_correction on the connected_sources pattern (depth):
//   accurate near field (sparse_assemble_parallel!, adaptive rules, `offset`)
//   minus the same pairs with the Gauss rule (partial_assemble_parallel!).
#include "bie_internal.h"

#include <algorithm>
#include <memory>
#include <vector>

namespace bie {

namespace {

// y[i] += sum_{p in row i} v[p] x[col[p]]   (complex128 CSR, one thread per row)
__global__ void csr_spmv_add_kernel(const int64_t *__restrict__ row_ptr, const int32_t *__restrict__ cols,
                                    const double2 *__restrict__ v, const double2 *__restrict__ x, int64_t n,
                                    double2 *__restrict__ y) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double re = 0.0, im = 0.0;
    for (int64_t p = row_ptr[i]; p < row_ptr[i + 1]; ++p) {
        const double2 a = v[p], b = x[cols[p]];
        re += a.x * b.x - a.y * b.y;
        im += a.x * b.y + a.y * b.x;
    }
    const double2 yo = y[i];
    y[i] = make_double2(yo.x + re, yo.y + im);
}

}  // namespace

FastOp::~FastOp() {
    if (g) destroy_context(*g);
    cudaFree(d_row_ptr);
    cudaFree(d_cols);
    cudaFree(d_vals);
}

std::unique_ptr<FastOp> create_fastop(Ctx &c, double k_re, double k_im, int which, int n_gauss, bool nearfield,
                                      double offset, int depth) {
    if (is_discontinuous(c.physics_kind))
        fail(BIE_ERR_UNSUPPORTED, "fast operators take continuous physics only");
    triangle_gauss_rule(n_gauss);   // validates n_gauss
    auto op = std::make_unique<FastOp>();
    op->base = &c;
    op->which = which;
    op->k_re = k_re;
    op->k_im = k_im;
    op->n_gauss = n_gauss;
    // Gauss-rule context over the same mesh, on the base context's stream
    std::vector<int64_t> topo(c.topo.size()), ptopo(c.ptopo.size());
    for (size_t i = 0; i < topo.size(); ++i) topo[i] = (int64_t)c.topo[i] + 1;
    for (size_t i = 0; i < ptopo.size(); ++i) ptopo[i] = (int64_t)c.ptopo[i] + 1;
    bie_mesh_desc d{};
    d.n_coordinates = c.n_coords;
    d.coordinates = c.coords.data();
    d.n_elements = c.n_elements;
    d.shape_kind = c.shape_kind;
    d.physics_kind = c.physics_kind;
    d.topology = topo.data();
    d.physics_topology = ptopo.data();
    d.n_sources = c.n_sources;
    d.sources = c.sources.data();
    d.quad_n = c.quad_n;
    d.quad_m = c.quad_m;
    d.physics_beta = c.physics_beta;
    op->g = std::make_unique<Ctx>();
    try {
        build_context(*op->g, d, c.device, n_gauss);
    } catch (...) {
        destroy_context(*op->g);
        op->g.reset();
        throw;
    }
    BIE_CUDA(cudaStreamSynchronize(op->g->stream));
    BIE_CUDA(cudaStreamDestroy(op->g->stream));
    op->g->stream = c.stream;
    op->g->owns_stream = false;
    // near-field correction S - C_coarse on the base context's pattern
    if (nearfield) {
        NearField &nf = get_nearfield(c, depth, offset, n_gauss);
        const int64_t nnz = (int64_t)nf.cols.size();
        op->nnz = nnz;
        BIE_CUDA(cudaMalloc(&op->d_row_ptr, nf.row_ptr.size() * sizeof(int64_t)));
        BIE_CUDA(cudaMalloc(&op->d_cols, std::max<int64_t>(nnz, 1) * sizeof(int32_t)));
        BIE_CUDA(cudaMalloc(&op->d_vals, std::max<int64_t>(nnz, 1) * sizeof(double2)));
        BIE_CUDA(cudaMemcpyAsync(op->d_row_ptr, nf.row_ptr.data(), nf.row_ptr.size() * sizeof(int64_t),
                                 cudaMemcpyHostToDevice, c.stream));
        BIE_CUDA(cudaMemcpyAsync(op->d_cols, nf.cols.data(), nnz * sizeof(int32_t), cudaMemcpyHostToDevice,
                                 c.stream));
        BIE_CUDA(cudaMemsetAsync(op->d_vals, 0, std::max<int64_t>(nnz, 1) * sizeof(double2), c.stream));
        double *v = reinterpret_cast<double *>(op->d_vals);
        const int flags = which;
        launch_nearfield(c, nf, k_re, k_im, flags, false, 1.0, which == BIE_F ? v : nullptr,
                         which == BIE_G ? v : nullptr);
        launch_nearfield(c, nf, k_re, k_im, flags, true, -1.0, which == BIE_F ? v : nullptr,
                         which == BIE_G ? v : nullptr);
        BIE_CUDA(cudaStreamSynchronize(c.stream));   // host pattern copies complete
    }
    return op;
}

void apply_fastop(FastOp &op, const double *x, double *y, int precision, const double *targets, int64_t M) {
    Ctx &g = *op.g;
    const bool at_nodes = targets == nullptr;
    MatvecArgs m{op.k_re, op.k_im, at_nodes ? g.d_sources : targets, at_nodes ? g.n_sources : M,
                 op.which == BIE_F ? x : nullptr, op.which == BIE_G ? x : nullptr,
                 op.which == BIE_F ? y : nullptr, op.which == BIE_G ? y : nullptr, precision};
    launch_matvec(g, m);
    if (at_nodes && op.nnz > 0) {
        const int64_t n = g.n_sources;
        csr_spmv_add_kernel<<<(unsigned)((n + 255) / 256), 256, 0, g.stream>>>(
            op.d_row_ptr, op.d_cols, op.d_vals, reinterpret_cast<const double2 *>(x), n,
            reinterpret_cast<double2 *>(y));
        BIE_CUDA(cudaGetLastError());
        ++g.kernel_launches;
    }
}

}  // namespace bie
