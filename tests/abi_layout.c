/* Prints the memory layout of the public structs of include/biegpu.h: one line
 * per struct, "name sizeof offset:size ..." over its leaf fields in declaration
 * order (nested structs and arrays flattened).  tests/test_abi_layout.py
 * compiles it with the system C compiler and checks the Python (ctypes) and
 * Julia (julia/src/BIEGPU.jl) mirrors of these structs against its output. */
#include <stddef.h>
#include <stdio.h>

#include "biegpu.h"

#define LEAF(T, f) printf(" %zu:%zu", offsetof(T, f), sizeof(((T *)0)->f))
#define LEAFA(T, f, n)                                                             \
    for (int i_ = 0; i_ < (n); ++i_)                                               \
    printf(" %zu:%zu", offsetof(T, f) + i_ * sizeof(((T *)0)->f[0]), sizeof(((T *)0)->f[0]))
#define BEGIN(T) printf(#T " %zu", sizeof(T))
#define END() printf("\n")

static void gmres_leaves(size_t base) {
    const size_t o[] = {offsetof(bie_gmres_opts, restart), offsetof(bie_gmres_opts, maxiter),
                        offsetof(bie_gmres_opts, reltol), offsetof(bie_gmres_opts, abstol),
                        offsetof(bie_gmres_opts, precision), offsetof(bie_gmres_opts, refine),
                        offsetof(bie_gmres_opts, inner_reltol), offsetof(bie_gmres_opts, max_refine),
                        offsetof(bie_gmres_opts, initially_nonzero)};
    const size_t s[] = {4, 4, 8, 8, 4, 4, 8, 4, 4};
    for (int i = 0; i < 9; ++i) printf(" %zu:%zu", base + o[i], s[i]);
}

int main(void) {
    BEGIN(bie_mesh_desc);
    LEAF(bie_mesh_desc, n_coordinates); LEAF(bie_mesh_desc, coordinates); LEAF(bie_mesh_desc, n_elements);
    LEAF(bie_mesh_desc, shape_kind); LEAF(bie_mesh_desc, physics_kind); LEAF(bie_mesh_desc, topology);
    LEAF(bie_mesh_desc, physics_topology); LEAF(bie_mesh_desc, n_sources); LEAF(bie_mesh_desc, sources);
    LEAF(bie_mesh_desc, quad_n); LEAF(bie_mesh_desc, quad_m); LEAF(bie_mesh_desc, physics_beta);
    END();
    BEGIN(bie_rule_table);
    LEAF(bie_rule_table, n_points); LEAF(bie_rule_table, u); LEAF(bie_rule_table, v); LEAF(bie_rule_table, w);
    END();
    BEGIN(bie_stats);
    LEAF(bie_stats, kernel_launches); LEAF(bie_stats, timed_launches); LEAF(bie_stats, timed_ms);
    LEAF(bie_stats, algorithmic_flops); LEAF(bie_stats, quadrature_evals); LEAF(bie_stats, tensor_launches);
    LEAF(bie_stats, tensor_ms); LEAF(bie_stats, tensor_flops); LEAF(bie_stats, tensor_flops_executed);
    END();
    BEGIN(bie_peaks);
    LEAF(bie_peaks, fp64_flops); LEAF(bie_peaks, fp32_flops);
    END();
    BEGIN(bie_operator);
    LEAF(bie_operator, kind); LEAF(bie_operator, A); LEAF(bie_operator, A32); LEAF(bie_operator, k_re);
    LEAF(bie_operator, k_im); LEAF(bie_operator, scale_re); LEAF(bie_operator, scale_im); LEAF(bie_operator, diag);
    LEAF(bie_operator, fast);
    END();
    BEGIN(bie_gmres_opts);
    gmres_leaves(0);
    END();
    BEGIN(bie_gmres_info);
    LEAF(bie_gmres_info, iterations); LEAF(bie_gmres_info, restarts); LEAF(bie_gmres_info, refinements);
    LEAF(bie_gmres_info, converged); LEAF(bie_gmres_info, matvecs); LEAF(bie_gmres_info, residual_norm);
    LEAF(bie_gmres_info, rhs_norm);
    END();
    BEGIN(bie_sweep_opts);
    LEAF(bie_sweep_opts, precision); LEAF(bie_sweep_opts, refine);
    gmres_leaves(offsetof(bie_sweep_opts, gmres));
    LEAF(bie_sweep_opts, eager); LEAF(bie_sweep_opts, target_error); LEAF(bie_sweep_opts, sensitivity);
    END();
    BEGIN(bie_sweep_info);
    LEAF(bie_sweep_info, solves); LEAF(bie_sweep_info, converged); LEAF(bie_sweep_info, iterations);
    LEAF(bie_sweep_info, assemble_ms); LEAF(bie_sweep_info, solve_ms); LEAF(bie_sweep_info, record_ms);
    LEAF(bie_sweep_info, graph_launches); LEAF(bie_sweep_info, accurate_solves);
    END();
    BEGIN(bie_adjoint_opts);
    LEAF(bie_adjoint_opts, rho_c); LEAFA(bie_adjoint_opts, dir, 3); LEAF(bie_adjoint_opts, reltol);
    LEAF(bie_adjoint_opts, precision);
    END();
    BEGIN(bie_adjoint_info);
    LEAF(bie_adjoint_info, forward_iterations); LEAF(bie_adjoint_info, forward_converged);
    LEAF(bie_adjoint_info, adjoint_iterations); LEAF(bie_adjoint_info, adjoint_converged);
    END();
    BEGIN(bie_lossy_constants);
    LEAF(bie_lossy_constants, rho); LEAF(bie_lossy_constants, c); LEAF(bie_lossy_constants, kp);
    LEAFA(bie_lossy_constants, ka, 2); LEAFA(bie_lossy_constants, kh, 2); LEAFA(bie_lossy_constants, kv, 2);
    LEAFA(bie_lossy_constants, tau_a, 2); LEAFA(bie_lossy_constants, tau_h, 2);
    LEAFA(bie_lossy_constants, phi_a, 2); LEAFA(bie_lossy_constants, phi_h, 2);
    LEAF(bie_lossy_constants, eta); LEAF(bie_lossy_constants, mu);
    LEAFA(bie_lossy_constants, mu_a, 2); LEAFA(bie_lossy_constants, mu_h, 2);
    END();
    BEGIN(bie_lossy_opts);
    LEAF(bie_lossy_opts, S); LEAF(bie_lossy_opts, custom_air); LEAF(bie_lossy_opts, pa); LEAF(bie_lossy_opts, t);
    LEAF(bie_lossy_opts, Hr); LEAF(bie_lossy_opts, depth); LEAF(bie_lossy_opts, interior);
    LEAF(bie_lossy_opts, fmm_on); LEAF(bie_lossy_opts, n_gauss); LEAF(bie_lossy_opts, fmm_offset);
    LEAF(bie_lossy_opts, normals);
    gmres_leaves(offsetof(bie_lossy_opts, solve));
    END();
    BEGIN(bie_multisolve_opts);
    LEAF(bie_multisolve_opts, precision); LEAF(bie_multisolve_opts, restart); LEAF(bie_multisolve_opts, maxiter);
    LEAF(bie_multisolve_opts, max_refine); LEAF(bie_multisolve_opts, reltol); LEAF(bie_multisolve_opts, inner_reltol);
    END();
    BEGIN(bie_multisolve_info);
    LEAF(bie_multisolve_info, passes); LEAF(bie_multisolve_info, inner_steps); LEAF(bie_multisolve_info, converged);
    LEAF(bie_multisolve_info, tensor_products); LEAF(bie_multisolve_info, exact_products);
    LEAF(bie_multisolve_info, reserved); LEAF(bie_multisolve_info, max_relres); LEAF(bie_multisolve_info, setup_ms);
    LEAF(bie_multisolve_info, tensor_ms); LEAF(bie_multisolve_info, exact_ms);
    END();
    return 0;
}
