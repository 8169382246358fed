/*
 * biegpu.h - C ABI of libbiegpu.so, the GB300 (sm_103a) collocation-BEM hot path.
 *
 * The library replaces the dense collocation assembly and the operator
 * application of BoundaryIntegralEquations.jl (3D, triangular elements).
 * Every entry point is `extern "C"`, takes plain pointers and sizes, returns an
 * int status (BIE_OK == 0, negative on failure) and never lets a C++ exception
 * cross the boundary.  `bie_last_error()` gives a thread-local message for the
 * last failing call made by the calling thread.
 *
 * Array conventions (identical to Julia's column-major storage, so a Julia
 * caller passes `pointer(A)` directly):
 *   - point sets are 3 x n column-major doubles: x0 y0 z0 x1 y1 z1 ...
 *   - connectivities are n_per_element x E column-major int64, 1-based
 *     (Julia's `mesh.topology`, `mesh.physics_topology`); they are checked and
 *     converted to 0-based on upload.
 *   - complex outputs are interleaved (re, im) doubles, the memory layout of
 *     Julia's ComplexF64; matrices are column-major M x N with leading
 *     dimension M.
 *
 * Threading: each context owns one CUDA stream; calls on one context are
 * serialised by a mutex inside the library.  Different contexts may be used
 * from different host threads.
 */
#ifndef BIEGPU_H
#define BIEGPU_H

#include <stdint.h>

#if defined(__GNUC__)
#define BIE_API __attribute__((visibility("default")))
#else
#define BIE_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define BIE_OK                 0
#define BIE_ERR_INVALID       -1  /* bad argument: sizes, indices, NaN, NULL */
#define BIE_ERR_CUDA          -2  /* a CUDA runtime call failed             */
#define BIE_ERR_NOT_CONVERGED -3  /* iterative solver hit maxiter           */
#define BIE_ERR_TIMEOUT       -4  /* a bounded device wait gave up          */
#define BIE_ERR_NOMEM         -5  /* device or host allocation failed       */
#define BIE_ERR_UNSUPPORTED   -6  /* element kind / option not implemented  */

/* ---- element kinds (Julia: TriangularLinear, TriangularQuadratic) ----- */
#define BIE_TRI_LINEAR    1   /* 3-node triangle, N = [1-u-v, u, v]            */
#define BIE_TRI_QUADRATIC 2   /* 6-node triangle, nodes 1 2 3 corners, 4 5 6 mid */
/* Discontinuous physics (physics_kind only; Julia: DiscontinuousTriangular-
 * Constant / -Linear / -Quadratic, src/3d/SurfaceFunction.jl:81-105,430-439,
 * src/3d/surface_functions.jl:236-318).  With b = physics_beta and
 * psi(s) = (s - b) / (1 - 3 b): constant N = [1] (node at (1/3, 1/3));
 * linear N = [psi(1-u-v), psi(u), psi(v)] (nodes (b,b), (1-2b,b), (b,1-2b));
 * quadratic N = the 6-node quadratic basis in those psi (edge nodes
 * ((1-b)/2, b), ((1-b)/2, (1-b)/2), (b, (1-b)/2)).  The collocation nodes
 * (`sources`) are the physics nodes of every element, as compute_sources
 * places them (src/3d/mesh.jl:115-145).                                    */
#define BIE_TRI_DISC_CONSTANT  3
#define BIE_TRI_DISC_LINEAR    4
#define BIE_TRI_DISC_QUADRATIC 5

/* ---- assembly selection flags (Julia keywords fOn, gOn, cOn) ---------- */
#define BIE_F 1   /* double-layer matrix F  */
#define BIE_G 2   /* single-layer matrix G  */
#define BIE_C 4   /* free-term row sums C   */

/* ---- arithmetic of an assembly or operator application ---------------- */
#define BIE_PREC_FP64  0  /* plain FP64 throughout (the reference's arithmetic) */
#define BIE_PREC_MIXED 1  /* FP32 regular pairs, FP64 near-singular pairs and C  */
/* Multi-right-hand-side products only (bie_matvec_multi_device): matrix tiles
 * generated in mixed precision, then multiplied on the tensor cores with
 * 16-bit operands scaled by powers of two per matrix row and per right-hand
 * side, FP32 accumulation.  The _SPLIT forms carry every operand as hi + lo
 * 16-bit parts and add three products (hi.hi + hi.lo + lo.hi).             */
#define BIE_PREC_FP16       2   /* ~5e-4 relative product error */
#define BIE_PREC_BF16       3   /* ~4e-3                        */
#define BIE_PREC_FP16_SPLIT 4   /* ~1e-6                        */
#define BIE_PREC_BF16_SPLIT 5   /* ~2e-5                        */
/* Assembly, matrix-free products and GMRES operator arithmetic (bie_assemble*,
 * bie_matvec*, bie_gmres*; with `refine`, the residuals of refinement):
 * FP64-grade results with the regular pairs in double-float arithmetic (pairs
 * of floats, ~48-bit significand) on the FP32 pipes, the near pairs in FP64 and
 * every sum compensated; assembled entries ~1e-14 from BIE_PREC_FP64.  Falls
 * back to the FP64 kernels where the phase rotation k (r - r0) over one
 * element exceeds the Taylor tables (|k| x element radius > ~2.5).          */
#define BIE_PREC_DF64       6

typedef struct bie_ctx bie_ctx;

/*
 * Mesh description.  Mirrors the fields of `Mesh3d` that the collocation
 * assembly reads (src/utils/mesh.jl:23-34): `coordinates`, `topology`,
 * `sources`, `physics_topology` and the element kinds of `shape_function` and
 * `physics_function`.  `quad_n`, `quad_m` are the `n`, `m` keywords of
 * `assemble_parallel!` (src/3d/assembly_collocation.jl:259-260).
 * The rule used for a (target, element) pair is the one clustered at the
 * element's physics node nearest to the target (find_closest_corner); for
 * linear geometry nodes 4-6 of 6-node physics use the rule of corner 3, as
 * the reference's linear-geometry method does (:330-346).
 * Dense assembly, operator products, GMRES and sweeps take every kind; the
 * near-field, fast-operator near-field, lossy, tangential-derivative and
 * adjoint paths take continuous physics only (BIE_ERR_UNSUPPORTED).
 * The library copies everything it needs; the caller keeps ownership.
 */
typedef struct bie_mesh_desc {
    int64_t        n_coordinates;     /* N_c                                    */
    const double  *coordinates;       /* 3 x N_c                                */
    int64_t        n_elements;        /* E                                      */
    int32_t        shape_kind;        /* BIE_TRI_LINEAR | BIE_TRI_QUADRATIC     */
    int32_t        physics_kind;      /* BIE_TRI_LINEAR | BIE_TRI_QUADRATIC     */
    const int64_t *topology;          /* n_shape x E, 1-based into coordinates  */
    const int64_t *physics_topology;  /* n_phys x E, 1-based into sources       */
    int64_t        n_sources;         /* N (collocation nodes = matrix columns) */
    const double  *sources;           /* 3 x N                                  */
    int32_t        quad_n;            /* Gauss-Legendre points along u (>= 1)   */
    int32_t        quad_m;            /* Gauss-Legendre points along v (>= 1)   */
    double         physics_beta;      /* node offset b of discontinuous physics
                                         (0 < b < 1/3); ignored otherwise      */
} bie_mesh_desc;

/* Library version string, e.g. "biegpu 0.1.0 sm_103a". */
BIE_API const char *bie_version(void);

/* Message of the last failing call on this host thread ("" if none). */
BIE_API const char *bie_last_error(void);

/*
 * Quadrature rule on the reference triangle clustered at element node `node`
 * (1, 2, 3: Duffy rules collapsed at that corner, from an n x m Gauss grid;
 * 4, 5, 6: two half-Duffy triangles split at that edge midpoint, m rounded up
 * to even).  Host-only (needs no GPU).  Writes at most `capacity` points to
 * u, v, w and the rule size to *count.
 * Replaces rotated_triangular_quadpoints / triangularQuadpoints /
 * rotated_midpoint_triangular_quadpoints as chosen by create_rotated_element
 * (src/3d/quadrature.jl:70-144; src/3d/assembly_collocation.jl:122-136, 384-389).
 */
BIE_API int bie_quadrature_rule(int n, int m, int node, double *u, double *v, double *w,
                                int capacity, int *count);

/*
 * Basis functions of element kind `kind` (BIE_TRI_* including the
 * discontinuous kinds, node offset `beta`) and their u- and v-derivatives at
 * n points: N, dNu, dNv are n_nodes x n column-major (NULL to skip), the
 * layout of basisFunction / basisFunctionDerivative
 * (src/3d/surface_functions.jl:191-318).  Host-only (needs no GPU); these are
 * the values the assembly tabulates at its quadrature points.
 */
BIE_API int bie_basis(int kind, double beta, int64_t n, const double *u, const double *v, double *N,
                      double *dNu, double *dNv);

/*
 * Create a context on CUDA device `device`: validates and uploads the mesh,
 * builds the Duffy rules clustered at each element node and the per-element
 * quadrature geometry (points, unit normals, jacobian x weight).
 * Replaces the set-up half of `assemble_parallel!` for triangles:
 * create_rotated_element / rotated_midpoint_triangular_quadpoints and
 * interpolate_elements (src/3d/assembly_collocation.jl:122-136, 27-66,
 * 284-305, 369-413; src/3d/quadrature.jl:70-144; src/3d/jacobian.jl:78-87).
 */
BIE_API int bie_ctx_create(bie_ctx **out, const bie_mesh_desc *desc, int device);

/* One clustered quadrature rule on the reference triangle: `n_points` points
 * (u, v) with weights w (a full-triangle rule has weights summing to 1/2). */
typedef struct bie_rule_table {
    int64_t       n_points;           /* 1..64                                  */
    const double *u;                  /* n_points                               */
    const double *v;                  /* n_points                               */
    const double *w;                  /* n_points                               */
} bie_rule_table;

/*
 * bie_ctx_create with the caller's own rule tables instead of the rules built
 * from (quad_n, quad_m), which are then ignored: `rules[r]` is the rule used
 * when element node r+1 is the nearest physics node to the collocation point
 * (n_rules = min(NP, 3) for linear geometry and NP for quadratic geometry,
 * NP = physics nodes per element; with linear geometry and NP = 6, nodes 4-6
 * use table 3), points summed in table order.  Passing the
 * `gauss_u`, `gauss_v`, `weights` of the shape functions that
 * create_rotated_element returns (src/3d/assembly_collocation.jl:122-136,
 * 284-305, 369-413) reproduces the reference's quadrature bit for bit.
 * Every point must satisfy u >= 0, v >= 0, u + v <= 1 and all values must be
 * finite; the tables are copied.
 */
BIE_API int bie_ctx_create_rules(bie_ctx **out, const bie_mesh_desc *desc,
                                 const bie_rule_table *rules, int n_rules, int device);

/* Release every device and host resource of a context. NULL is a no-op. */
BIE_API int bie_ctx_destroy(bie_ctx *ctx);

/* The context's CUDA stream (a cudaStream_t), for callers that enqueue
 * their own work or record events around the device entry points. */
BIE_API int bie_ctx_stream(bie_ctx *ctx, void **stream);

/*
 * Launch statistics of a context, for profiling.  `kernel_launches` counts every
 * kernel libbiegpu enqueued on the context; with timing on, the dominant
 * compute kernel of each call (assembly or operator application) is bracketed
 * by CUDA events on the context stream and `timed_ms` sums their durations
 * over `timed_launches` launches.  Not part of the reference API (its only
 * instrumentation is ProgressMeter and @time in examples).
 */
typedef struct bie_stats {
    int64_t kernel_launches;
    int64_t timed_launches;
    double  timed_ms;
    double  algorithmic_flops;   /* flops of the timed launches, counted as
                                    32 + 8 n_phys per quadrature-point evaluation */
    int64_t quadrature_evals;    /* (target, quadrature point) evaluations */
    /* tensor-core GEMM launches of bie_matvec_multi_device / bie_lowp_gemm_device,
       timed on their own while timing is on */
    int64_t tensor_launches;
    double  tensor_ms;
    double  tensor_flops;            /* algorithmic: 8 M N R per complex product, 2 M N K real */
    double  tensor_flops_executed;   /* issued MMA flops (padding, 3 products when split)     */
} bie_stats;

/*
 * Measured FMA throughput of a device (dependency-free FMA chains on every SM,
 * ~0.1 s): the denominators of the FP64 / FP32 pipe rooflines of the assembly
 * and operator kernels.  Values in FLOP/s (an FMA counts 2).
 */
typedef struct bie_peaks {
    double fp64_flops;
    double fp32_flops;
} bie_peaks;
BIE_API int bie_measure_peaks(int device, bie_peaks *out);

BIE_API int bie_ctx_set_timing(bie_ctx *ctx, int on);

/*
 * Autotuning of launch shapes (no reference counterpart: the reference has no
 * GPU launch shapes).  While on, the first call of the context for a given
 * number of targets M of the mixed assembly (BIE_SHAPE_MIXED_ASSEMBLY), the
 * double-float assembly (BIE_SHAPE_DF64_ASSEMBLY) and the mixed matrix-free
 * product (BIE_SHAPE_MIXED_PRODUCT) searches the launch shape coordinate by
 * coordinate: element slicing (2^level slices, the default level and its two
 * neighbours), element records per shared-memory chunk (half, default,
 * double) and, for the mixed assembly, threads per block (128, 256); each
 * candidate is timed as a complete call with CUDA events on the context stream
 * (about seven calls for the first M), and the fastest is kept per (kernel, M)
 * for later calls.  Results of different shapes differ only by rounding order.
 * bie_sweep turns it on for the contexts it is given.
 */
#define BIE_SHAPE_MIXED_ASSEMBLY 0
#define BIE_SHAPE_DF64_ASSEMBLY  1
#define BIE_SHAPE_MIXED_PRODUCT  2
BIE_API int bie_ctx_set_autotune(bie_ctx *ctx, int on);
/* The shape in use for (kernel, M): *found = 1 and the shape if one was tuned
 * or forced, else *found = 0. */
BIE_API int bie_ctx_get_shape(bie_ctx *ctx, int kernel, int64_t M, int *found, int *level, int *chunk, int *tpb);
/* Force a shape for (kernel, M) (M = 0: every M) until cleared with level < 0;
 * chunk <= 0 or tpb other than 128 / 256 keep the default of that axis.  For
 * tests and measurements of individual shapes. */
BIE_API int bie_ctx_set_shape(bie_ctx *ctx, int kernel, int64_t M, int level, int chunk, int tpb);
/* Synchronises the context stream, then fills *out; `reset` != 0 zeroes the counters. */
BIE_API int bie_ctx_stats(bie_ctx *ctx, bie_stats *out, int reset);

/*
 * Dense collocation assembly into HOST buffers.
 * Replaces `assemble_parallel!(mesh, k, targets; fOn, gOn, cOn, m, n)`
 * (src/3d/assembly_collocation.jl:259-268, triangle methods :270-353 and
 * :355-479) returning (F, G, C).
 *   k = k_re + i k_im (the reference accepts real or complex k).
 *   targets: 3 x M collocation / field points; NULL means the mesh sources.
 *   flags: BIE_F | BIE_G | BIE_C.  precision: BIE_PREC_*.
 *   F, G: M x N complex (interleaved doubles), C: M complex.  A buffer whose
 *   flag is off may be NULL and is not touched.
 * Outputs are fully overwritten (the reference starts from zeros).
 * Blocks until the results are in the host buffers.
 */
BIE_API int bie_assemble(bie_ctx *ctx, double k_re, double k_im,
                 const double *targets, int64_t n_targets,
                 int flags, int precision,
                 double *F, double *G, double *C);

/*
 * Same as bie_assemble with DEVICE pointers for targets (3 x M doubles, may be
 * NULL for the mesh sources) and outputs.  Enqueued on the context stream and
 * returns without synchronising.
 */
BIE_API int bie_assemble_device(bie_ctx *ctx, double k_re, double k_im,
                        const double *d_targets, int64_t n_targets,
                        int flags, int precision,
                        double *d_F, double *d_G, double *d_C);

/*
 * Matrix-free operator application with HOST buffers:
 *   yF = F x,  yG = G v
 * with F, G exactly the matrices bie_assemble would return for the same
 * targets (same rules, same arithmetic class), recomputed on the fly and never
 * stored.  Either product may be skipped by passing NULL for its input and
 * output.  targets: 3 x M (NULL = mesh sources; then M is ignored).
 * Replaces the operator products fed to gmres: FMMFOperator / FMMGOperator
 * `LinearMaps._unsafe_mul!` (src/3d/fast_multipole_method.jl:238-247, 392-404)
 * and the field-point products `Fp*p + Gp*v` of examples/3d_pulsating_sphere.jl:60-63.
 */
BIE_API int bie_matvec(bie_ctx *ctx, double k_re, double k_im,
                       const double *targets, int64_t n_targets,
                       const double *x, const double *v, double *yF, double *yG,
                       int precision);

/* Same with DEVICE pointers; enqueued on the context stream, asynchronous. */
BIE_API int bie_matvec_device(bie_ctx *ctx, double k_re, double k_im,
                              const double *d_targets, int64_t n_targets,
                              const double *d_x, const double *d_v, double *d_yF, double *d_yG,
                              int precision);

/*
 * Allocation-free variant of bie_matvec_device (mixed precision only).
 * This entry point has no counterpart in the reference; it exists for callers
 * that must not have a library allocate device memory behind their back: a
 * Julia session whose CUDA.jl pool (or a Python process whose PyTorch caching
 * allocator) already holds most of the GPU, or a loop that may not
 * synchronise the device.  Such a caller creates the context once at set-up,
 * then calls this function as often as it likes; it performs no cudaMalloc or
 * cudaFree.  All temporaries live in one fixed 32 MiB device array inside the
 * library (32 MiB - 256 bytes usable); a mesh whose product needs more returns
 * BIE_ERR_INVALID with the size in the message.  The array is committed when
 * the first context on a device is created (bie_ctx_create and
 * bie_ctx_create_rules load the module holding it, look its device address up
 * into the context and launch its kernels once on empty work) and stays held
 * by that device until the process exits.  The address is kept per context, so
 * a context must not be used across a reset of its device (cudaDeviceReset,
 * CUDA.jl's device_reset!).  Every call reuses the same array: calls whose
 * executions overlap on the GPU race and must be serialised by the caller.
 * Inputs and outputs are device pointers as in bie_matvec_device; the call is
 * asynchronous on the context stream.  Results agree with bie_matvec_device
 * to the mixed-precision tolerance: near pairs go to the FP64 correction
 * kernel up to the same capacity (M*64+4096 pairs) where the array has room
 * for it, shrunk for large meshes down to M*16+1024 pairs; pairs beyond it are
 * integrated in FP64 inside the product kernel (slower, with both halves of
 * each FP64 value added to the double-float row sums).
 */
BIE_API int bie_matvec_device_noalloc(bie_ctx *ctx, double k_re, double k_im,
                                      const double *d_targets, int64_t n_targets,
                                      const double *d_x, const double *d_v,
                                      double *d_yF, double *d_yG);

/*
 * Products with many right-hand sides at the collocation nodes:
 *     YF = F X,  YG = G V     (X, V, YF, YG: N x nrhs complex, column-major)
 * the matrix form of the operator products (the reference's FMMFOperator /
 * FMMGOperator `_unsafe_mul!` on a matrix, src/3d/fast_multipole_method.jl:
 * 249-287, 427-471, which loop batches of 32 columns).  precision:
 *   BIE_PREC_FP64 / BIE_PREC_MIXED: one matrix-free product per column
 *     (exactly bie_matvec_device per column);
 *   BIE_PREC_FP16 ... BIE_PREC_BF16_SPLIT: row strips of F and G are generated
 *     in mixed precision into device scratch (complex64), quantised to 16-bit
 *     tiles, and multiplied by all right-hand sides at once with tcgen05
 *     tensor-core GEMMs; the matrices never exist whole.
 * Either product may be skipped (NULL input and output).  Device pointers;
 * asynchronous on the context stream.  `scratch_bytes` caps the strip scratch
 * (0: 8 GiB); the right-hand-side operands and partial sums come on top.
 */
BIE_API int bie_matvec_multi_device(bie_ctx *ctx, double k_re, double k_im, int64_t nrhs,
                                    const double *d_X, const double *d_V, double *d_YF,
                                    double *d_YG, int precision, int64_t scratch_bytes);

/* Same with HOST buffers (copied to and from the device inside the call;
 * blocking), the form a Julia `Matrix{ComplexF64}` caller uses. */
BIE_API int bie_matvec_multi(bie_ctx *ctx, double k_re, double k_im, int64_t nrhs,
                             const double *X, const double *V, double *YF, double *YG,
                             int precision, int64_t scratch_bytes);

/*
 * The tensor-core building block of bie_matvec_multi_device on its own
 * (no reference counterpart): C = A B^T for real FP32 A (M x K) and B (N x K),
 * both row-major, C (M x N, row-major) in FP64, through the same 16-bit
 * quantisation (power-of-two scale per row of A and of B) and the same tcgen05
 * GEMM kernel.  precision: BIE_PREC_FP16 ... BIE_PREC_BF16_SPLIT.  Device
 * pointers; runs on the context stream.
 */
BIE_API int bie_lowp_gemm_device(bie_ctx *ctx, int precision, int64_t M, int64_t N, int64_t K,
                                 const float *d_A, const float *d_B, double *d_C);

/*
 * Solve of many right-hand sides at once,
 *     (F + Diagonal(1 - C)) X = B,   B, X: N x nrhs complex (device, column-major),
 * the exterior collocation system of test/3d/assembly_test.jl:37-38, which the
 * reference solves one column at a time (IterativeSolvers.gmres per
 * right-hand side; its operators accept matrices in batches of 32 columns,
 * src/3d/fast_multipole_method.jl:249-287).  F and C come from the mixed
 * assembly (complex64 F); the nrhs GMRES solves run in lockstep so that every
 * Arnoldi step is one tcgen05 tensor-core product of F (quantised once to
 * 16-bit tiles) with all Krylov vectors; the outer iterative refinement forms
 * each column's residual B - A X with the exact product of the complex64
 * matrix (double-float sums).  A column has converged when that residual is
 * at most reltol times ||b||.  X is overwritten.  Synchronous.
 */
typedef struct bie_multisolve_opts {
    int32_t precision;      /* tensor-core form of the inner products: BIE_PREC_FP16 ..
                               BIE_PREC_BF16_SPLIT (<= 0: BIE_PREC_FP16_SPLIT)            */
    int32_t restart;        /* inner GMRES restart (<= 0: 20, at most 64)                  */
    int32_t maxiter;        /* inner Arnoldi steps per refinement pass (<= 0: 200)         */
    int32_t max_refine;     /* refinement passes (<= 0: 10)                                */
    double  reltol;         /* <= 0: sqrt(eps(Float64)), IterativeSolvers' default         */
    double  inner_reltol;   /* inner solves, relative to the pass's residual (<= 0: 1e-4)  */
} bie_multisolve_opts;

typedef struct bie_multisolve_info {
    int32_t passes;          /* refinement passes that ran an inner solve                 */
    int32_t inner_steps;     /* lockstep Arnoldi steps, summed over passes                */
    int32_t converged;       /* columns with ||b - A x|| <= reltol ||b||                  */
    int32_t tensor_products; /* tensor-core products of all columns                       */
    int32_t exact_products;  /* exact residual products of all columns                    */
    int32_t reserved;
    double  max_relres;      /* largest ||b - A x|| / ||b|| (exact product)               */
    double  setup_ms;        /* assembly + quantisation of F (host wall time)             */
    double  tensor_ms;       /* tensor-core products (host wall time)                     */
    double  exact_ms;        /* exact residual products (host wall time)                  */
} bie_multisolve_info;

BIE_API int bie_solve_multi_device(bie_ctx *ctx, double k_re, double k_im, int64_t nrhs, const double *d_B,
                                   double *d_X, const bie_multisolve_opts *opts, bie_multisolve_info *info);
/* The same with host matrices (N x nrhs complex, column-major): B and X are
 * copied to and from device memory the call allocates and frees. */
BIE_API int bie_solve_multi(bie_ctx *ctx, double k_re, double k_im, int64_t nrhs, const double *B, double *X,
                            const bie_multisolve_opts *opts, bie_multisolve_info *info);

/*
 * Failure detection of the tensor-core GEMM (no reference counterpart; the
 * reference has no device code).  Every mbarrier wait of the GEMM kernel gives
 * up after a clock-cycle budget, sets a bit in a device error word and lets
 * the CTA wait for its own MMAs and copies, free its tensor memory and exit;
 * the call then returns BIE_ERR_TIMEOUT and the context stays usable.
 * `cycles` sets the budget of the pipeline waits of this context's later GEMMs
 * (negative: the default, about 2 s at 2 GHz); `stall` != 0 makes their MMA
 * issuer first wait on a barrier that nothing completes, so that the wait runs
 * out (for tests of this path).  The clean-up waits keep the default budget.
 */
BIE_API int bie_ctx_set_gemm_wait(bie_ctx *ctx, int64_t cycles, int stall);

/* ---- near field (sparse) --------------------------------------------- */
/*
 * Adaptive singular rule towards element node `node` (1..6) with `offset`:
 * singular_triangle_integration(shape, 3, source, Diagonal(ones(3)), 1e-6) as
 * set up by sparse_assemble_parallel! (src/3d/adaptive_integration.jl:217-246,
 * src/3d/assembly_collocation_losses.jl:208-220).  Host-only.  *count gets the
 * rule size; at most `capacity` points are written.
 */
BIE_API int bie_singular_rule(int node, double offset, double *u, double *v, double *w,
                              int capacity, int *count);

/*
 * CSR pattern of the near-field matrices: row i holds the physics nodes of
 * the elements connected to collocation node i (depth 1: elements containing
 * node i; depth 2: elements containing one of its neighbours), sorted.
 * Replaces connected_sources (src/3d/assembly_collocation_losses.jl:98-132).
 * Call with row_ptr = cols = NULL to get *nnz, then with row_ptr (N + 1
 * entries) and cols (nnz entries); indices are 0-based.
 */
BIE_API int bie_nearfield_pattern(bie_ctx *ctx, int depth, int64_t *nnz, int64_t *row_ptr,
                                  int64_t *cols);

/*
 * Near-field values of F and G in the CSR order of bie_nearfield_pattern
 * (HOST buffers of nnz complex each; a buffer whose flag is off may be NULL).
 * coarse == 0: the accurate adaptive-subdivision rules of
 *   assemble_parallel!(mesh, k, mesh.sources; sparse=true, depth, offset)
 *   = sparse_assemble_parallel! (src/3d/assembly_collocation_losses.jl:200-405,
 *   src/3d/adaptive_integration.jl:172-246); offset < 0 means the reference's
 *   default for continuous elements (0).
 * coarse == 1: the n_gauss-point triangle rule of partial_assemble_parallel!
 *   (src/3d/fast_multipole_method.jl:11-81), n_gauss in {1, 3, 4, 7, 12, 13}.
 * FP64 arithmetic.  Blocks until the values are in the host buffers.
 */
BIE_API int bie_nearfield_assemble(bie_ctx *ctx, double k_re, double k_im, int depth,
                                   double offset, int flags, int coarse, int n_gauss,
                                   double *F, double *G);

/*
 * Derivatives of F and G with respect to the wavenumber at k0, for Taylor
 * expansions in k (ROSEBEM): taylor_assemble!(mesh, k0, targets,
 * shape_function; M = order, fOn, gOn, cOn, n, m) with U = I
 * (src/3d/rosebem.jl:56-157; kernels taylor_greens3d! / taylor_freens3d!,
 * src/3d/kernels.jl:94-118):
 *   G^(m) = (i r)^m e^{i k0 r} / (4 pi r),
 *   F^(m) = e^{i k0 r} (i r)^m (1 - i k0 r - m) n.(x - y) / (4 pi r^3),
 * integrated with the clustered corner rules of the context (physics nodes
 * 4-6 of quadratic elements use the third corner rule, as the reference
 * does).  F, G: M x N x (order + 1) complex column-major (matrix m at offset
 * m M N), C: M complex (from the same rules).  FP64.  Host buffers, blocking.
 * The expansion itself, sum_m (k - k0)^m / m! A^(m), is a host operation
 * (apply_taylor_expansion, src/3d/rosebem.jl:164-176).
 */
BIE_API int bie_taylor_assemble(bie_ctx *ctx, double k0_re, double k0_im, const double *targets,
                                int64_t n_targets, int flags, int order, double *F, double *G, double *C);

/* ---- fast operators (FMMFOperator / FMMGOperator) ----------------------- */
typedef struct bie_fastop bie_fastop;

/*
 * The operator of FMMFOperator(mesh, k; n_gauss, nearfield, offset, depth)
 * (which = BIE_F) or FMMGOperator (which = BIE_G)
 * (src/3d/fast_multipole_method.jl:163-194 setup_fast_operator, :306-324,
 * :473-490): every element integrated with the symmetric n_gauss-point
 * triangle rule for all collocation nodes, plus nearfield_correction = the
 * accurate near field (adaptive rules, `offset`) minus its Gauss-rule part on
 * the connected_sources(depth) pattern.  The reference sums the far field with
 * FMM3D to `tol`; here the sum is exact (direct, on the GPU), so results agree
 * with the reference to its FMM tolerance.  The correction is computed here,
 * once, for the given k.  The operator keeps a pointer to `ctx` and runs on
 * its stream; destroy it before the context.
 */
BIE_API int bie_fastop_create(bie_ctx *ctx, double k_re, double k_im, int which, int n_gauss, int nearfield,
                              double offset, int depth, bie_fastop **out);
BIE_API int bie_fastop_destroy(bie_fastop *op);
/* y = A x at the collocation nodes (LinearMaps._unsafe_mul!, :238-247, :392-404).
 * precision: BIE_PREC_FP64 (exact sum), BIE_PREC_DF64 (the same in
 * double-float arithmetic) or BIE_PREC_MIXED.  Device pointers, asynchronous
 * on the context stream. */
BIE_API int bie_fastop_apply_device(bie_fastop *op, const double *d_x, double *d_y, int precision);
/* Same with host buffers (blocking). */
BIE_API int bie_fastop_apply(bie_fastop *op, const double *x, double *y, int precision);
/* The far-field sum at other points (evaluate_targets, :326-344, :497-519):
 * no near-field correction, as in the reference.  Host buffers (blocking). */
BIE_API int bie_fastop_evaluate_targets(bie_fastop *op, const double *targets, int64_t n_targets,
                                        const double *x, double *y, int precision);

/* ---- linear systems A x = b,  A x = s (K x) + diag .* x ---------------- */
#define BIE_OP_DENSE       0  /* K = stored dense N x N matrix (device)       */
#define BIE_OP_MATRIX_FREE 1  /* K = F of the context at wavenumber k         */
#define BIE_OP_FAST        2  /* K = a fast operator (FMMFOperator algorithm)  */

typedef struct bie_operator {
    int32_t       kind;        /* BIE_OP_DENSE | BIE_OP_MATRIX_FREE                 */
    const double *A;           /* dense: device N x N complex128, column-major      */
    const float  *A32;         /* dense: optional complex64 copy for the mixed inner
                                  iterations (NULL: the complex128 matrix is used)   */
    double        k_re, k_im;  /* matrix-free: wavenumber                           */
    double        scale_re, scale_im;   /* s                                         */
    const double *diag;        /* device N complex, or NULL for zero                */
    const struct bie_fastop *fast;      /* BIE_OP_FAST: a fast operator of the same
                                           context (bie_fastop_create)              */
} bie_operator;

typedef struct bie_gmres_opts {
    int32_t restart;           /* <= 0: min(20, N)                 (IterativeSolvers) */
    int32_t maxiter;           /* <= 0: N                                             */
    double  reltol;            /* <= 0: sqrt(eps(Float64))                            */
    double  abstol;            /* >= 0, default 0                                     */
    int32_t precision;         /* operator arithmetic without refinement (BIE_PREC_*) */
    int32_t refine;            /* 1: mixed inner GMRES + FP64 residual refinement     */
    double  inner_reltol;      /* refinement: inner relative tolerance (<= 0: 1e-4)   */
    int32_t max_refine;        /* refinement: outer steps (<= 0: 10)                  */
    int32_t initially_nonzero; /* 1: start from the given x instead of zero           */
} bie_gmres_opts;

typedef struct bie_gmres_info {
    int32_t iterations;        /* Arnoldi steps (inner steps summed under refinement) */
    int32_t restarts;
    int32_t refinements;
    int32_t converged;         /* ||b - A x|| <= max(reltol ||b||, abstol)            */
    int64_t matvecs;
    double  residual_norm;     /* final ||b - A x|| (FP64 operator under refinement)  */
    double  rhs_norm;
} bie_gmres_info;

/*
 * Restarted GMRES on the device (vectors of length N = n_sources, device
 * pointers).  Replaces IterativeSolvers.gmres as used by the reference
 * (test/3d/assembly_test.jl:38; examples/3d_pulsating_sphere.jl:44-50) with
 * its defaults.  Returns BIE_ERR_NOT_CONVERGED (x still written, info filled)
 * when maxiter is reached before the tolerance.
 */
BIE_API int bie_gmres_device(bie_ctx *ctx, const bie_operator *op, const double *d_b,
                             double *d_x, const bie_gmres_opts *opts, bie_gmres_info *info);

/*
 * bie_gmres_device with host buffers (blocking): b, x (N complex128) and the
 * operator's A (N x N complex128, column-major), A32 and diag are host arrays,
 * copied to temporary device memory; x is written back.  With a dense operator
 * and `refine` or BIE_PREC_MIXED, a NULL A32 is formed on the device by
 * rounding A to complex64.  The call `gmres(H, b)` of the reference on a
 * matrix returned by bie_assemble (test/3d/assembly_test.jl:37-38;
 * examples/3d_pulsating_sphere.jl:44) becomes one call here.
 */
BIE_API int bie_gmres(bie_ctx *ctx, const bie_operator *op, const double *b, double *x,
                      const bie_gmres_opts *opts, bie_gmres_info *info);

/* ---- frequency sweeps -------------------------------------------------- */
typedef struct bie_sweep_opts {
    int32_t precision;         /* assembly arithmetic: BIE_PREC_MIXED | BIE_PREC_FP64   */
    int32_t refine;            /* mixed: complex64 inner GMRES + complex128 residual     */
    bie_gmres_opts gmres;      /* restart, maxiter, reltol, abstol (zeros: defaults)     */
    int32_t eager;             /* 0 (default): after the first wavenumber of each mesh,
                                  the rest of the sweep is one launch of a recorded CUDA
                                  graph (every mesh's matrices resident at once);
                                  1: launch by launch, one mesh's matrices at a time     */
    double  target_error;      /* mixed only; > 0: after each solve a short GMRES solve
                                  with a fixed pseudo-random right-hand side estimates the
                                  system's sensitivity s (about 1 away from interior
                                  resonances, large near them); solves whose predicted
                                  error 5e-7 s exceeds target_error are solved again at
                                  FP64 grade (double-float assembly + FP64 GMRES).
                                  0: off                                                 */
    double *sensitivity;       /* optional host output, nmesh x nk: the estimates s     */
} bie_sweep_opts;

typedef struct bie_sweep_info {
    int64_t solves;            /* (mesh, k) systems solved                                */
    int64_t converged;         /* of which converged                                      */
    int64_t iterations;        /* GMRES iterations summed                                 */
    double  assemble_ms;       /* device time of the assemblies (CUDA events)            */
    double  solve_ms;          /* device time of right-hand sides + GMRES                */
    double  record_ms;         /* host time spent recording + instantiating graphs       */
    int64_t graph_launches;    /* CUDA graph launches (1 per sweep unless eager)         */
    int64_t accurate_solves;   /* solves redone at FP64 grade (opts.target_error)        */
} bie_sweep_info;

/*
 * Batched frequency sweep over meshes of uneven size: for every context m and
 * wavenumber k_j, assemble F, G, C on the device, form
 *     (F + Diagonal(1 - C)) p = G w_m
 * (the reference's boundary integral equation, README.md:10-18, with the
 * exterior collocation form of test/3d/assembly_test.jl:37) and solve it with
 * GMRES, all on the device.  The reference has no batched form: users loop
 * assemble_parallel! + gmres per frequency (examples/sweep_meta.jl:219-233,
 * src/3d/rosebem.jl:235-262).  ks: nk complex (interleaved), w[m]: N_m complex
 * host vectors, p[m]: nk x N_m complex host outputs (column j = k_j).
 * iters (optional): nmesh x nk GMRES iteration counts.
 * Unless opts->eager is set, the first wavenumber of each mesh runs launch by
 * launch (it sizes the device scratch and, through the autotuner, picks the
 * assembly's slicing); then everything else is ONE launch of a recorded CUDA
 * graph: per mesh a loop over the wavenumbers (k read from device memory)
 * whose GMRES refinement, restart and Arnoldi loops are nested conditional
 * nodes driven by device state (restart <= 64; contexts on one device).  Both
 * forms give the same results up to the rounding order of the assemblies'
 * atomic sums.
 */
BIE_API int bie_sweep(bie_ctx *const *ctxs, int nmesh, const double *ks, int nk,
                      const double *const *w, double *const *p, const bie_sweep_opts *opts,
                      bie_sweep_info *info, int32_t *iters);

/* ---- adjoint shape / impedance gradient ------------------------------- */
typedef struct bie_adjoint_opts {
    double rho_c;        /* characteristic impedance rho0 c of the fluid (e.g. 1.21 * 343) */
    double dir[3];       /* incident plane-wave direction (unit vector)                  */
    double reltol;       /* GMRES tolerance of the forward and adjoint solves (<= 0: 1e-13) */
    int32_t precision;   /* forward-model assembly: BIE_PREC_FP64 (0) or BIE_PREC_DF64       */
} bie_adjoint_opts;

typedef struct bie_adjoint_info {
    int32_t forward_iterations, forward_converged;
    int32_t adjoint_iterations, adjoint_converged;
} bie_adjoint_info;

/*
 * Far-field objective and its gradient (3-node triangles, nodal physics on the
 * vertices, real k).  Forward model: (F + Diagonal(1 - C) - i rho c k G_Y) p =
 * p_I with G_Y the single layer weighted by the element admittances 1 / Z_e
 * (impedance condition v_n = p / Z on each element), p_I = exp(-i k dir.x)
 * (incoming_wave, src/analytical/3d_scattering.jl:4-12); field pressures
 * p_f = p_I + (-F_x + i rho c k G_{x,Y}) p at the M field points; J = sum |p_f|^2.
 * The reference has no gradient code (its only prior art is finite differences
 * in 2D, examples/2d_optimization.jl:187-219; nodal impedance form
 * examples/3d_cube_wave_anechoic.jl:62-68).  Gradients by the adjoint method
 * with a reverse pass that recomputes the quadrature (FP64):
 *   dX: 3 x N_c, dJ/d(vertex coordinates);  dZ: E complex, dJ/dRe Z_e + i dJ/dIm Z_e.
 * Z: E complex impedances in the element order of the mesh.  Outputs may be
 * NULL (J alone costs one forward solve).  Host buffers; blocking.
 */
BIE_API int bie_adjoint(bie_ctx *ctx, double k_re, double k_im, const double *Z,
                        const double *field, int64_t n_field, const bie_adjoint_opts *opts,
                        double *J, double *pf, double *dX, double *dZ, bie_adjoint_info *info);

/* out[i] = (complex64) in[i] for n complex entries (device), e.g. to build
 * bie_operator.A32 from an assembled matrix. */
BIE_API int bie_round_c64_device(bie_ctx *ctx, const double *d_in, float *d_out, int64_t n);

/* ---- mesh input ----------------------------------------------------------- */
/* COMSOL text mesh, read_comsol_mesh(mesh_file) of src/3d/read_comsol.jl:9-54:
 * the vertex coordinates (3 x Nc, column-major), the triangles (npe x E with
 * npe = 3 or 6, 1-based, rows 5 and 6 of 6-node triangles swapped into the
 * library's node order) and the geometric entity indices.  ".mphtxt" is
 * appended to `path` when missing.  Call with coordinates == NULL to get the
 * sizes, then again with coordinates[3 Nc], topology[npe E], entities[n_ent]
 * (entities may be NULL).  Host only. */
BIE_API int bie_read_comsol(const char *path, int64_t *n_coordinates, int64_t *n_elements,
                            int32_t *nodes_per_element, int64_t *n_entities, double *coordinates,
                            int64_t *topology, int64_t *entities);

/* ---- visco-thermal ("lossy") system ------------------------------------ */
/* Physical properties of air (Rasmussen 1997, annex A), as
 * ambient_to_properties(f, ps, t, H) of src/utils/ambient_to_properties.jl:1-134:
 * out = rho, c0, cf, CpCv, eta, alfa, Cp, Cv, landa, beta.  Host only. */
BIE_API int bie_ambient_to_properties(double f, double ps, double t, double H, double out[10]);

typedef struct bie_lossy_constants {
    double rho, c, kp;           /* density, zero-frequency speed of sound, 2 pi f / c      */
    double ka[2], kh[2], kv[2];  /* acoustic, thermal, viscous wavenumbers (re, im)         */
    double tau_a[2], tau_h[2];   /* isothermal-condition constants                         */
    double phi_a[2], phi_h[2];   /* no-slip-condition constants                            */
    double eta, mu;              /* bulk (0.6 mu) and shear viscosity                       */
    double mu_a[2], mu_h[2];     /* phi_a - tau_a phi_h / tau_h  and  tau_a phi_h / tau_h   */
} bie_lossy_constants;

/* visco_thermal_constants(; freq, S, pa, t, Hr) of src/utils/lossy_constants.jl:1-34
 * (the reference's defaults: S = -1, pa = 101325, t = 20, Hr = 50; LossyGlobalOuter
 * uses S = 1).  Host only. */
BIE_API int bie_visco_thermal_constants(double freq, double S, double pa, double t, double Hr,
                                        bie_lossy_constants *out);

/* Tangential derivative matrices Dx, Dy, Dz of the physics interpolation,
 * interpolation_function_derivatives(mesh) of
 * src/3d/interpolation_function_derivatives.jl:36-118: at every node, the
 * surface gradient of each element's basis functions, averaged over the
 * elements of the node.  CSR on the depth-1 node pattern (0-based, sorted
 * columns).  Call with row_ptr == NULL to get *nnz; then row_ptr[N + 1],
 * cols[nnz], Dx/Dy/Dz[nnz].  Host only (no context, no GPU). */
BIE_API int bie_tangential_derivatives(const bie_mesh_desc *mesh, int64_t *nnz, int64_t *row_ptr,
                                       int64_t *cols, double *Dx, double *Dy, double *Dz);

/* Element slicing of the assembly kernels, on the host (no GPU, no context).
 * The kernels process the elements in the order of a recursive coordinate
 * bisection of their centroids and split that order into 2^l slices of
 * consecutive elements (bie_ctx_get_shape reports the level l in use); the
 * mixed assembly writes each node's entries by the rule of its kind below.
 * order: E 1-based element numbers in processing order, or NULL.
 * counts: 6 node counts for `level` (0..7), or NULL:
 *   [0] nodes touched by elements of two or more slices (summed in side slots
 *       and added by a fix-up pass),
 *   [1] side slots: (slice, shared node) pairs,
 *   [2] nodes of one slice with several contributions, summed in the
 *       per-block shared-memory ring and written once,
 *   [3] nodes of one slice with several contributions and no free ring slot
 *       (float partial sums, then the widening pass),
 *   [4] nodes with exactly one contribution,
 *   [5] nodes touched by no element (written as zero).
 * flags: E words, or NULL: for the element at position p of the order and
 *   its local node a: bit a = p is the node's first position in its slice,
 *   bit 8+a = its last, bit 16+a = the node is shared, bit 24+a = it has a
 *   ring slot.
 * slots: E x n_phys indices, or NULL: the node's side slot (shared nodes,
 *   numbered over all slices), its ring slot (0..15), else -1.
 * Replaces nothing in the reference: its assembly loops over collocation
 * points (src/3d/assembly_collocation.jl:270-353) and has no element order. */
BIE_API int bie_element_slicing(const bie_mesh_desc *mesh, int level, int32_t *order, int64_t *counts,
                                uint32_t *flags, int32_t *slots);

typedef struct bie_lossy_opts {
    double  S;              /* sign convention of the constants (0: 1, as LossyGlobalOuter)    */
    int32_t custom_air;     /* 0: 101325 Pa, 20 C, 50 % humidity; 1: pa, t, Hr below          */
    double  pa, t, Hr;      /* ambient pressure (Pa), temperature (Celsius), humidity (%)      */
    int32_t depth;          /* near-field pattern of the thermal and viscous operators (1, 2)  */
    int32_t interior;       /* 0: exterior problem (default); 1: interior                      */
    int32_t fmm_on;         /* 1: acoustic H, G by the fast-operator algorithm                 */
    int32_t n_gauss;        /* fast operators: Gauss rule (<= 0: 3)                            */
    double  fmm_offset;     /* fast operators: near-field offset (< 0: 0.2)                    */
    const double *normals;  /* 3 x N nodal normals (mesh.normals), host, required              */
    bie_gmres_opts solve;   /* the nested gmres calls (zeros: IterativeSolvers defaults)       */
} bie_lossy_opts;

/* Blocks of the system (x, y lengths: N, or 3N where stated) */
#define BIE_LOSSY_OUTER  0  /* LossyGlobalOuter product (N -> N)                         */
#define BIE_LOSSY_HA     1  /* acoustic H with its integral-free term (N -> N)           */
#define BIE_LOSSY_GA     2  /* acoustic G (N -> N)                                       */
#define BIE_LOSSY_HH     3  /* thermal H, near field + integral-free term (N -> N)       */
#define BIE_LOSSY_GH     4  /* thermal G, near field (N -> N)                            */
#define BIE_LOSSY_HV     5  /* blockdiag(Av, Av, Av), viscous H (3N -> 3N)               */
#define BIE_LOSSY_GV     6  /* blockdiag(Bv, Bv, Bv), viscous G (3N -> 3N)               */
#define BIE_LOSSY_DC     7  /* [Dx; Dy; Dz] (N -> 3N)                                    */
#define BIE_LOSSY_DR     8  /* [Dx Dy Dz] (3N -> N)                                      */
#define BIE_LOSSY_ND     9  /* Nd = -[diag(nx); diag(ny); diag(nz)] (N -> 3N)            */
#define BIE_LOSSY_NDT   10  /* Nd' (3N -> N)                                             */
#define BIE_LOSSY_INNER 11  /* LossyGlobalInner: Dr Nd z - Nd' gmres(Gv, Hv Nd z) (N)    */

typedef struct bie_lossy bie_lossy;

/*
 * LossyGlobalOuter(mesh, freq; depth, exterior, fmm_on, n = quadrature of the
 * context) of src/3d/LossyGlobalMatrix.jl:76-172, resident on the device:
 * acoustic H, G (dense complex128 from this library's FP64 assembly, or fast
 * operators), thermal and viscous H, G as near-field CSR matrices (the
 * library's adaptive near-field rules, sparse_assemble_parallel!), Dx, Dy, Dz
 * and the normals.  The reference's LossyGlobalOuter passes n = m = 3 to the
 * acoustic assembly: create the context with quad_n = quad_m = 3 for the same
 * matrices.  The product (LossyGlobalMatrix.jl:179-197)
 *     y = -phi_a Ha x + Ga (mu_h gmres(Gh, Hh x)
 *                          + mu_a gmres(inner, Dr Dc x - Nd' gmres(Gv, Hv Dc x)))
 * runs its nested GMRES solves on the device (two levels deep inside the
 * inner operator), each as the reference's gmres call with opts->solve.
 */
BIE_API int bie_lossy_create(bie_ctx *ctx, double freq, const bie_lossy_opts *opts, bie_lossy **out);
/* Frees the system's device memory; call it before bie_ctx_destroy of its context. */
BIE_API int bie_lossy_destroy(bie_lossy *L);
BIE_API int bie_lossy_constants_of(const bie_lossy *L, bie_lossy_constants *out);
/* y = block x (device vectors, complex interleaved); blocking */
BIE_API int bie_lossy_apply_device(bie_lossy *L, int block, const double *d_x, double *d_y);
/* x = gmres(block, b) from x = 0 for the square blocks OUTER, HA, GA, HH, GH,
 * HV, GV, INNER (device vectors); info optional; BIE_ERR_NOT_CONVERGED with
 * x written when maxiter is reached. */
BIE_API int bie_lossy_solve_device(bie_lossy *L, int block, const double *d_b, double *d_x,
                                   const bie_gmres_opts *opts, bie_gmres_info *info);
/* The same with host vectors. */
BIE_API int bie_lossy_apply(bie_lossy *L, int block, const double *x, double *y);
BIE_API int bie_lossy_solve(bie_lossy *L, int block, const double *b, double *x,
                            const bie_gmres_opts *opts, bie_gmres_info *info);
/* Nested GMRES solves and their iterations since creation (or the last reset). */
BIE_API int bie_lossy_stats(bie_lossy *L, int64_t *nested_solves, int64_t *nested_iterations, int reset);
/* The sparse thermal / viscous solves (gmres(Gh, .), gmres(Gv, .) and solves
 * of the HH, GH, HV, GV blocks).  mode 1 (default): one launch each where the
 * system fits, a cooperative grid over the SMs for more than 2048 rows, else
 * a thread-block cluster; 2: the cluster form only; 3: the grid form only;
 * 0: the launch-per-operation device GMRES.  Same algorithm and tolerances.
 * A grid barrier wait that runs out makes the call return BIE_ERR_TIMEOUT. */
BIE_API int bie_lossy_set_one_launch(bie_lossy *L, int mode);

#ifdef __cplusplus
}
#endif

#endif /* BIEGPU_H */
