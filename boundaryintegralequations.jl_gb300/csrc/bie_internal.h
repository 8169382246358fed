// Internal declarations shared by the host set-up code and the CUDA kernels of
// libbiegpu.so.  Nothing here crosses the C ABI.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <memory>
#include <functional>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/biegpu.h"

namespace bie {

// ----------------------------------------------------------------------------
// Errors: every internal failure throws bie::Error; the C-ABI wrappers catch it,
// store the message in a thread-local string and return the code.
// ----------------------------------------------------------------------------
struct Error {
    int code;
    std::string msg;
};
[[noreturn]] void fail(int code, const std::string &msg);
void cuda_check(cudaError_t e, const char *what);
#define BIE_CUDA(call) ::bie::cuda_check((call), #call)

// ----------------------------------------------------------------------------
// Quadrature rules on the reference triangle (u, v >= 0, u + v <= 1).
// ----------------------------------------------------------------------------
struct Rule {
    std::vector<double> u, v, w;
    int size() const { return (int)w.size(); }
};

// Gauss-Legendre nodes/weights on [-1, 1], ascending nodes.
void gauss_legendre(int n, std::vector<double> &x, std::vector<double> &w);
// Duffy rule clustered at element node `corner` (1, 2, 3) built from an n x m
// tensor Gauss grid; node 1 = rotated rule, node 2 = plain Duffy rule, node 3 =
// plain Duffy with u and v swapped.  src/3d/quadrature.jl:70-113.
Rule duffy_corner_rule(int n, int m, int corner);
// Two half-Duffy triangles split at edge midpoint `vertex` (4, 5, 6), m rounded
// up to even.  src/3d/quadrature.jl:116-144.
Rule duffy_midpoint_rule(int n, int m, int vertex);
// Symmetric triangle rules with n in {1, 3, 4, 7, 12, 13} points
// (src/3d/adaptive_integration.jl:13-64).
Rule triangle_gauss_rule(int n);

// Shape functions of the 3- and 6-node triangles (src/3d/surface_functions.jl:191-236).
int  n_nodes_of_kind(int kind);
bool is_discontinuous(int kind);
// physics basis: shape_values for continuous kinds, the discontinuous
// triangle bases (node offset beta) otherwise
void physics_values(int kind, double beta, double u, double v, double *N);
void physics_derivs(int kind, double beta, double u, double v, double *dNu, double *dNv);
void shape_values(int kind, double u, double v, double *N);
void shape_derivs(int kind, double u, double v, double *dNu, double *dNv);

// ----------------------------------------------------------------------------
// Per-element record consumed by the assembly kernels (doubles, element-major).
//   [0, 3*NP)                       physics-node coordinates, a-major (x, y, z)
//   rule r at rule_off[r]:          x[Q_r] y[Q_r] z[Q_r] nx[Q_r] ny[Q_r] nz[Q_r] jw[Q_r]
//   nidx_off:                       NP int32 physics-node indices (0-based)
// The stride is even so every record starts on a 16-byte boundary.
// ----------------------------------------------------------------------------
constexpr int kMaxRules = 6;
constexpr int kMaxNP = 6;
constexpr int kMaxQ = 64;
constexpr int kMaxLevels = 8;   // element slicings 1, 2, 4, ..., 128
constexpr int kK2RingSlots = 16; // shared-memory partial-sum slots per thread in K2

struct RecordLayout {
    int NP = 0;                 // physics nodes per element (3 or 6)
    int R = 0;                  // number of clustered rules (3 or 6)
    int Q[kMaxRules] = {};      // points per rule
    int rule_off[kMaxRules] = {};
    int nidx_off = 0;
    int stride = 0;             // doubles per record
    int qmax = 0;
};

// Launch shape of the assembly / product kernels the autotuner chooses:
// element-slicing level (S = 2^level slices), element records per shared-
// memory chunk, threads per block (one target row per thread).
struct LaunchShape {
    int level = 0;
    int chunk = 1;
    int tpb = 128;
};
enum ShapeKernel { kShapeK2 = 0, kShapeK9 = 1, kShapeK3 = 2, kShapeCount = 3 };

enum ScratchSlot {
    kScratchTargets = 0,   // uploaded target points (host entry points)
    kScratchF = 1,         // device F (host entry points)
    kScratchG = 2,         // device G (host entry points)
    kScratchCpart = 3,     // per-slice partial C row sums
    kScratchC = 4,         // device C (host entry points)
    kScratchF32 = 5,       // complex64 F accumulator (mixed precision)
    kScratchG32 = 6,       // complex64 G accumulator (mixed precision)
    kScratchDefer = 7,     // deferred (target, element) pairs + counter + near C
    kScratchMatvecXi = 8,  // interpolated densities of the matrix-free products
    kScratchMatvecPart = 9,// per-slice partial products
    kScratchSolver = 10,   // GMRES workspace
    kScratchSolverPart = 11,  // GMRES reduction partials and small coefficient vectors
    kScratchLowp = 12,     // multi-RHS products: strips, 16-bit tiles, partial sums
    kScratchSolverNested = 13,  // GMRES workspace + partials of nested solves, two slots
                                // per level 1, 2 (solves inside another solve's product)
    kScratchK2Side = 17,   // mixed assembly: per-slice partial sums of nodes shared between slices
    kScratchCount = 18
};

// Mixed-precision element record (32-bit words, same element order as the FP64
// records):
//   [0,3) centroid hi, [3,6) centroid lo (double-float), [6] near radius^2
//   [8, 8+3*NP)                      physics-node offsets from the centroid
//   rule r at rule_off[r]:           dx[Q] dy[Q] dz[Q] nx[Q] ny[Q] nz[Q] jw/4pi[Q] |d|^2[Q]
//                                    (quadrature points relative to the centroid)
//   nidx_off:                        NP int32 physics-node indices
// The stride is a multiple of 4 words (16 bytes).
struct MixedLayout {
    int rule_off[kMaxRules] = {};
    int nidx_off = 0;
    int stride = 0;
};

// Double-float element records (K9, BIE_PREC_DF64): the mixed header (centroid
// hi/lo, near radius^2, FP32 node offsets), then per rule and point 16 floats
// (o = x_q - c_e and jw / 4 pi as hi, lo; the unit normal as hi, lo), then the
// physics node indices.
struct Df64Layout {
    int rule_off[kMaxRules] = {};
    int nidx_off = 0;
    int stride = 0;
};

// Near-field (sparse) structure for one (depth, offset, n_gauss): CSR pattern of
// connected nodes per collocation node, the (row, element, CSR slots) pairs and
// the rule tables (adaptive singular rules per element node + the coarse
// Gauss rule).  Built on first use (bie_nearfield.cpp).
struct NearField {
    bool ready = false;
    int depth = 1;
    double offset = 0.0;
    int n_gauss = 3;
    std::vector<int64_t> row_ptr;        // N + 1
    std::vector<int32_t> cols;           // nnz (0-based node indices)
    std::vector<int32_t> pairs;          // npairs x pair_stride: row, element, slot[NP]
    int pair_stride = 0;
    int64_t npairs = 0;
    std::vector<double> table;           // points x point_stride
    int point_stride = 0;                // N[NS] dNu[NS] dNv[NS] Phi[NP] w
    int nrules = 0;
    int64_t rule_off[kMaxRules] = {};    // first point of rule r
    int rule_q[kMaxRules] = {};
    int64_t coarse_off = 0;
    int coarse_q = 0;
    int32_t *d_pairs = nullptr;
    double *d_table = nullptr;
};

struct Ctx {
    std::mutex mu;
    int device = 0;
    cudaStream_t stream = nullptr;
    bool owns_stream = true;             // false: the stream belongs to another context
    cudaStream_t copy_stream = nullptr;  // device-to-host copies overlapped with the assembly
                                         // (bie_assemble with host buffers), made on first use
    int num_sms = 0;

    // mesh (host copies, 0-based)
    int shape_kind = 0, physics_kind = 0;
    double physics_beta = 0.0;
    int64_t n_coords = 0, n_elements = 0, n_sources = 0;
    int NS = 0;                          // geometry nodes per element
    std::vector<double> coords;          // 3 x Nc
    std::vector<int32_t> topo;           // NS x E
    std::vector<int32_t> ptopo;          // NP x E
    std::vector<double> sources;         // 3 x N
    int quad_n = 0, quad_m = 0;

    // clustered rules and physics interpolation tables Phi[r][q][a]
    RecordLayout lay;
    std::vector<Rule> rules;
    std::vector<double> phi;             // R x qmax x NP

    // element order (recursive coordinate bisection of centroids); records follow this order
    std::vector<int32_t> order;

    // device data
    double *d_records = nullptr;         // E x stride, element order
    double *d_phi = nullptr;             // R x qmax x NP
    double *d_sources = nullptr;         // 3 x N (AoS)
    uint32_t *d_shared_mask = nullptr;   // kMaxLevels x E: bit a set -> node a is
                                         // touched by elements of another slice
    uint8_t *d_node_shared = nullptr;    // kMaxLevels x N: the same per node
    // Write protocol of the mixed assembly (K2), per slicing level l, slice s
    // covering sorted positions [s*E/S, (s+1)*E/S): for the element at
    // position p and its local node a (node j),
    //   bit a      : p is the first position of slice s whose element has j,
    //   bit 8 + a  : p is the last such position,
    //   bit 16 + a : j is touched by elements of other slices too (shared);
    // the slice then sums its contributions to j in its side slot
    // d_k2_side[l][p][a] (one slot per (slice, shared node)), and a fix-up pass
    // adds the slots of every shared node (d_k2_fix[l]: nodes | CSR pointers |
    // slots; nodes touched by no element get no slot and are written as zero);
    //   bit 24 + a : j has several contributions, all in slice s, and its
    // partial sums live in ring slot d_k2_side[l][p][a] (< kK2RingSlots) of the
    // block's shared memory from its first to its last position, where the
    // sums become the final entries (slots are reused once a node closes; the
    // host assigns them by earliest last position, which covers the most
    // nodes).  The other nodes of one slice with several contributions keep
    // float partial sums in their entries and are widened by a streaming pass
    // (their list follows at k2_widen_off[l]).
    uint32_t *d_k2_flags = nullptr;      // kMaxLevels x E
    int32_t *d_k2_side = nullptr;        // kMaxLevels x E x NP (side or ring slot, -1: neither)
    int32_t *d_k2_fix = nullptr;         // per level: nfix nodes, nfix + 1 pointers, slots
    int64_t k2_fix_off[kMaxLevels] = {};
    int64_t k2_nfix[kMaxLevels] = {};
    int64_t k2_nside[kMaxLevels] = {};
    int64_t k2_widen_off[kMaxLevels] = {};   // d_k2_fix offset of the widening list
    int64_t k2_nwiden[kMaxLevels] = {};      // nodes of one slice with several contributions
    MixedLayout mlay;
    float *d_mrecords = nullptr;         // E x mlay.stride words, element order
    float *d_mphi = nullptr;             // R x qmax x NP (FP32)
    Df64Layout dlay;
    float *d_drecords = nullptr;         // E x dlay.stride words, element order
    float *d_dphi = nullptr;             // R x qmax x NP (hi, lo) pairs
    double df_rho_max = 0.0;             // largest |x_q - c_e| over the mesh
    float *d_phase_tab = nullptr;        // e^{i j h} as (cos hi, lo, sin hi, lo), double-float kernels
    double *d_coords = nullptr;          // 3 x Nc geometry nodes (near-field kernels)
    int32_t *d_topo = nullptr;           // NS x E, 0-based
    std::vector<std::unique_ptr<NearField>> nearfields;

    // grow-only device scratch, indexed by the kScratch* slots below
    void *d_scratch[kScratchCount] = {};
    size_t scratch_bytes[kScratchCount] = {};
    void *scratch(int slot, size_t bytes);
    // set while the context stream records a CUDA graph: scratch must not grow
    // then (a reallocation would leave the graph pointing at freed memory)
    bool capturing = false;

    // autotuning of the mixed assembly's element slicing: on the first call for
    // a target count M the neighbouring slicing levels are timed and the
    // fastest is kept (bie_ctx_set_autotune; bie_sweep turns it on)
    bool autotune = false;

    // tensor-core GEMM pipeline waits: clock-cycle budget (negative: ~2 s) and
    // the failure-detection test switch (bie_ctx_set_gemm_wait)
    int64_t gemm_wait_cycles = -1;
    bool gemm_stall = false;

    // device address of the allocation-free product's static scratch array
    // (bie_matvec_device_noalloc), looked up when the context is created
    char *noalloc_base = nullptr;

    // launch statistics (bie_ctx_stats)
    std::map<std::pair<int, int64_t>, LaunchShape> tuned_shapes;   // (kernel, M) -> tuned shape
    std::map<std::pair<int, int64_t>, LaunchShape> forced_shapes;  // bie_ctx_set_shape (M = 0: any M)
    bool timing = false;
    int64_t kernel_launches = 0;
    int64_t timed_launches = 0;
    double timed_ms = 0.0;
    unsigned long long *d_qpe = nullptr;     // device counter of quadrature evaluations
    std::vector<cudaEvent_t> ev_free;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_pending;
    cudaEvent_t take_event();
    // Bracket the dominant kernel of a call: timer_begin() before its launch,
    // timer_end() after; both are no-ops while timing is off.
    cudaEvent_t timer_begin();
    void timer_end(cudaEvent_t a);
    // Tensor-core GEMM launches of the multi-RHS products are timed on their
    // own (tensor_*), with their algorithmic and executed flop counts.
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_tensor;
    int64_t tensor_launches = 0;
    double tensor_ms = 0.0, tensor_flops = 0.0, tensor_flops_executed = 0.0;
    void tensor_timer_end(cudaEvent_t a, double flops, double flops_executed);
    void collect_timers();   // synchronises the stream
};

// Host set-up (bie_setup.cpp)
// gauss_rule > 0 replaces the clustered Duffy rules by the symmetric Gauss
// rule of that many points (fast-operator far field); explicit_rules != NULL
// replaces them by the caller's tables (one per nearest element node).
void build_context(Ctx &c, const bie_mesh_desc &d, int device, int gauss_rule = 0,
                   const std::vector<Rule> *explicit_rules = nullptr);
void destroy_context(Ctx &c);

// Kernel launchers (bie_assemble.cu)
struct AssembleArgs {
    double k_re, k_im;
    const double *targets;   // device, 3 x M AoS
    int64_t M;
    int flags;
    double *F, *G, *C;       // device outputs (interleaved complex), may be null
    bool c64_out = false;    // mixed only: F, G are complex64 (float2) buffers, not widened
    const double *g_weight = nullptr;   // FP64 only: per-element complex factor on G
                                        // (record order), e.g. an element admittance
    int taylor_m = -1;                  // FP64 only: >= 0 assembles the taylor_m-th
                                        // k-derivative (corner rules only)
    const double *k_dev = nullptr;      // device (re, im): the kernels read k here instead
                                        // of k_re, k_im (which then only select the real-
                                        // or complex-k code path: k_im != 0)
    double k_abs_max = 0.0;             // double-float kernel with k_dev: a bound on |k|
                                        // (its phase polynomials' degrees)
};
void launch_assemble_fp64(Ctx &c, const AssembleArgs &a);
int choose_slice_level(const Ctx &c, int64_t M, int threads_per_row_tile);
int wave_slice_level(const Ctx &c, int64_t M, int threads_per_row_tile);
// Candidate values per axis of the shape search.
struct ShapeAxes {
    std::vector<int> levels, chunks, tpbs;
};
// The shape for (kernel, M): a forced one (bie_ctx_set_shape), else the cached
// tuned one, else -- with autotuning on and no graph being recorded -- a
// coordinate search (slicing level, then records per chunk, then block size,
// each candidate timed as a complete operation by CUDA events on the context
// stream after `reset`), cached per (kernel, M); else `base`.
LaunchShape resolve_shape(Ctx &c, int kernel, int64_t M, const LaunchShape &base, const ShapeAxes &ax,
                          const std::function<void(const LaunchShape &)> &run, const std::function<void()> &reset);
void launch_reduce_c(Ctx &c, const double *Cpart, int S, const double *Cextra, int64_t M,
                     double *C);

// Matrix-free products yF = F x, yG = G v (bie_matvec.cu); all pointers device
struct MatvecArgs {
    double k_re, k_im;
    const double *targets;   // 3 x M AoS
    int64_t M;
    const double *x;         // N complex, input of F (null: skip F)
    const double *v;         // N complex, input of G (null: skip G)
    double *yF, *yG;         // M complex outputs
    int precision;
};
void launch_matvec(Ctx &c, const MatvecArgs &a);
// Mixed-precision product whose temporaries live in a fixed static device array
// (no device allocation by the library); rejects meshes that do not fit.
void launch_matvec_noalloc(Ctx &c, const MatvecArgs &a);
// At context creation: load the module holding the allocation-free product's
// static scratch array and kernels, store the array's device address in
// c.noalloc_base and launch those kernels once on empty work, so that a later
// bie_matvec_device_noalloc call needs no module load and no stack growth.
void prepare_noalloc(Ctx &c);

// Host-side tables of the element slicings (no GPU): the element order and,
// per slicing level l (S = 2^l slices of the ordered elements), the
// shared-node masks of K1/K9 and the write protocol of K2 (flags, side or
// ring slots, fix-up and widening lists; layout in Ctx::d_k2_flags) with
// counts of each kind of node.
struct WriteProtocol {
    std::vector<uint32_t> masks;          // kMaxLevels x E
    std::vector<uint8_t> node_shared;     // kMaxLevels x N
    std::vector<uint32_t> k2_flags;       // kMaxLevels x E
    std::vector<int32_t> k2_side;         // kMaxLevels x E x NP
    std::vector<int32_t> k2_fix;          // per level: fix-up nodes | pointers | slots | widening nodes
    int64_t fix_off[kMaxLevels] = {}, nfix[kMaxLevels] = {}, nside[kMaxLevels] = {};
    int64_t widen_off[kMaxLevels] = {}, nwiden[kMaxLevels] = {};
    int64_t nshared[kMaxLevels] = {};     // nodes touched by two or more slices
    int64_t nring[kMaxLevels] = {};       // one slice, several contributions, a ring slot
    int64_t nsingle[kMaxLevels] = {};     // exactly one contribution
    int64_t nuntouched[kMaxLevels] = {};  // touched by no element
};
std::vector<int32_t> bisection_order(const double *coords, int64_t n_coords, const int32_t *topo, int NS,
                                     int64_t E);
void build_write_protocol(const int32_t *order, int64_t E, const int32_t *ptopo, int NP, int64_t Nn,
                          WriteProtocol &w);

// GMRES (bie_solver.cu); b, x device, N = n_sources
void run_gmres(Ctx &c, const bie_operator &op, const double *b, double *x, const bie_gmres_opts &o,
               bie_gmres_info &info);
// The same solve (dense operator, x = 0 start) recorded into the graph being
// captured on c.stream: the refinement, restart and Arnoldi loops become
// conditional WHILE nodes and the step index a SWITCH node, all driven by
// device-side state, so a replay needs no host round trip.  body[0..3]: four
// idle streams for the nested body captures.  *d_info (device) receives the
// solve's statistics when the graph runs.
constexpr int kGraphMaxRestart = 64;
// Stream-capture helpers for conditional graph nodes (bie_solver.cu): a handle
// of the graph being captured on `s`; a conditional node appended after the
// capture's current dependencies, its body graphs returned.
cudaGraphConditionalHandle graph_new_handle(cudaStream_t s);
void graph_add_conditional(cudaStream_t s, cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type,
                           unsigned size, cudaGraph_t *bodies);
// Records onto stream `s` into the body graph `g` until end() (or destruction,
// which ends an unfinished capture after an error).
struct BodyCapture {
    cudaStream_t s;
    bool on = false;
    BodyCapture(cudaStream_t s_, cudaGraph_t g) : s(s_) {
        cuda_check(cudaStreamBeginCaptureToGraph(s, g, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed),
                   "cudaStreamBeginCaptureToGraph");
        on = true;
    }
    void end() {
        on = false;
        cudaGraph_t out = nullptr;
        cuda_check(cudaStreamEndCapture(s, &out), "cudaStreamEndCapture");
    }
    ~BodyCapture() {
        if (on) {
            cudaGraph_t out = nullptr;
            cudaStreamEndCapture(s, &out);
        }
    }
    BodyCapture(const BodyCapture &) = delete;
    BodyCapture &operator=(const BodyCapture &) = delete;
};

// COMSOL text mesh (bie_mesh_io.cpp): coords 3 x Nc, topo npe x E (1-based)
void read_comsol(const std::string &path, std::vector<double> &coords, std::vector<int64_t> &topo, int &npe,
                 std::vector<int64_t> &entities);

// Visco-thermal system, host part (bie_lossy.cpp)
void ambient_to_properties(double f, double ps, double t, double H, double out[10]);
bie_lossy_constants visco_thermal_constants(double freq, double S, double pa, double t, double Hr);
// per node the sorted physics nodes of its elements (connected_sources, depth 1)
void node_pattern(int64_t N, int64_t E, int NP, const int32_t *ptopo, std::vector<int64_t> &row_ptr,
                  std::vector<int32_t> &cols);
// Dx, Dy, Dz on node_pattern; topo NS x E, ptopo NP x E, 0-based
void tangential_derivatives(int shape_kind, int physics_kind, const double *coords, int64_t E,
                            const int32_t *topo, const int32_t *ptopo, int64_t N, std::vector<int64_t> &row_ptr,
                            std::vector<int32_t> &cols, std::vector<double> &Dx, std::vector<double> &Dy,
                            std::vector<double> &Dz);

// Visco-thermal system, device part (bie_lossy.cu); calls hold the context mutex
struct LossyOp;
LossyOp *create_lossy(Ctx &c, double freq, const bie_lossy_opts &o);
void destroy_lossy(LossyOp *L);
Ctx &lossy_context(const LossyOp &L);
const bie_lossy_constants &lossy_constants(const LossyOp &L);
int64_t lossy_block_len(int block, bool input, int64_t N);   // vector lengths of a block
void lossy_apply(LossyOp &L, int block, const double *x, double *y);   // device vectors
void lossy_solve(LossyOp &L, int block, const double *b, double *x, const bie_gmres_opts &o,
                 bie_gmres_info &info);
void lossy_stats(LossyOp &L, int64_t *solves, int64_t *iterations, bool reset);
void lossy_set_one_launch(LossyOp &L, int mode);

// An operator that the library's GMRES applies through a virtual call (the
// visco-thermal composite and its sparse blocks).  apply: y = A x on the
// context stream; operators whose kernels return at once while *stop is set
// say so (honours_stop), so GMRES may queue several steps between host checks.
struct DevOp {
    virtual ~DevOp() = default;
    virtual int64_t size() const = 0;
    virtual void apply(const double2 *x, double2 *y, const int *stop) = 0;
    virtual bool honours_stop() const { return false; }
};
// run_gmres on a DevOp of size n; `level` 0, 1 or 2 selects the workspace, so a
// solve may run inside the product of a solve one level up.
constexpr int kMaxSolveLevel = 2;
void run_gmres_devop(Ctx &c, DevOp &op, const double *b, double *x, const bie_gmres_opts &o,
                     bie_gmres_info &info, int level);
void capture_gmres(Ctx &c, const bie_operator &op, const double *b, double *x, const bie_gmres_opts &o,
                   bie_gmres_info *d_info, const cudaStream_t *body);
// (V + Diagonal(diag)) on nb diagonal blocks of N rows that share one CSR
// pattern and value array (the thermal and viscous near-field blocks); diag
// may be null.
struct CsrSystem {
    const int64_t *rp;
    const int32_t *cols;
    const double2 *val;
    const double2 *diag;
    int64_t N;
    int nb;
};
// The restarted GMRES of run_gmres_devop (zero start) on a CsrSystem as one
// launch on the context stream (bie_cluster_gmres.cu): a cooperative grid of
// up to one CTA per SM with a bounded grid barrier, or a thread-block cluster.
// Writes the info to d_info and adds (1, iterations) to d_acc[0..1] on the
// device (either may be null); a grid barrier that gives up sets *d_err (the
// grid form needs d_err).  `forms`: kOneLaunchAuto, kOneLaunchCluster or
// kOneLaunchGrid.  Returns false, launching nothing, when the system or
// restart length fits none of the allowed forms.
constexpr int kOneLaunchAuto = 0, kOneLaunchCluster = 1, kOneLaunchGrid = 2;
bool csr_gmres_one_launch(Ctx &c, const CsrSystem &A, const double2 *b, double2 *x, const bie_gmres_opts &o,
                          int level, bie_gmres_info *d_info, unsigned long long *d_acc, int *d_err, int forms);
void round_to_c64(Ctx &c, const double *in, float *out, int64_t n);
// Frequency sweep (bie_sweep.cu); locks each context while it runs.
void run_sweep(Ctx *const *ctxs, int nmesh, const double *ks, int nk, const double *const *w,
               double *const *p, const bie_sweep_opts &o, bie_sweep_info &info, int32_t *iters);
// Adjoint shape / impedance gradient (bie_adjoint.cu); host pointers
struct AdjointArgs {
    double k_re, k_im, rho_c;
    const double *Z;         // E complex element impedances (original element order)
    double dir[3];           // incident direction (unit)
    const double *field;     // 3 x n_field
    int64_t n_field;
    double reltol;           // GMRES tolerance of the forward and adjoint solves
    double *pf;              // out: n_field complex field pressures (may be null)
    double *dX;              // out: 3 x N vertex gradient (may be null)
    double *dZ;              // out: E complex (dJ/dRe Z, dJ/dIm Z) (may be null)
    int precision = BIE_PREC_FP64;   // forward-model assembly (BIE_PREC_FP64 | BIE_PREC_DF64)
};
struct AdjointOut {
    double J = 0;
    int forward_iterations = 0, forward_converged = 0;
    int adjoint_iterations = 0, adjoint_converged = 0;
};
void run_adjoint(Ctx &c, const AdjointArgs &a, AdjointOut &out);

// K4: products with many right-hand sides (bie_lowp.cu)
struct MultiArgs {
    double k_re, k_im;
    int64_t nrhs;
    const double *X, *V;     // N x nrhs complex (device), null: skip that product
    double *YF, *YG;         // N x nrhs complex outputs
    int precision;           // BIE_PREC_*
    int64_t scratch_bytes;   // cap of the strip scratch (<= 0: default)
};
void run_matvec_multi(Ctx &c, const MultiArgs &a);
// A complex64 N x N matrix (device, column-major) quantised once to resident
// 16-bit tensor-core tiles (precision BIE_PREC_FP16 ... BF16_SPLIT), applied to
// blocks of right-hand sides: Y = A X, X and Y N x R complex128 (device).  The
// apply synchronises the context stream (it reads the GEMM's error word).
struct LowpMatrix;
LowpMatrix *lowp_matrix_create(Ctx &c, const float *A, int64_t n, int precision);
void lowp_matrix_apply(Ctx &c, LowpMatrix &m, const double *X, int64_t R, double *Y);
void lowp_matrix_destroy(LowpMatrix *m);
// Multi-right-hand-side solve (bie_multisolve.cu)
void run_solve_multi(Ctx &c, double k_re, double k_im, int64_t R, const double *B, double *X,
                     const bie_multisolve_opts &o, bie_multisolve_info &info);
void run_lowp_gemm(Ctx &c, int precision, int64_t M, int64_t N, int64_t K, const float *A, const float *B,
                   double *C);

// Fast operators (bie_fastop.cu): Gauss-rule far field + near-field correction
struct FastOp {
    Ctx *base = nullptr;            // context the operator was made from (its stream)
    std::unique_ptr<Ctx> g;         // same mesh, every rule the n_gauss Gauss rule
    int which = BIE_F;              // BIE_F or BIE_G
    double k_re = 0, k_im = 0;
    int n_gauss = 3;
    int64_t nnz = 0;                // near-field correction S - C_coarse (CSR, device)
    int64_t *d_row_ptr = nullptr;
    int32_t *d_cols = nullptr;
    double2 *d_vals = nullptr;
    ~FastOp();
};
std::unique_ptr<FastOp> create_fastop(Ctx &c, double k_re, double k_im, int which, int n_gauss, bool nearfield,
                                      double offset, int depth);
// y = K_gauss x (+ correction at the nodes); targets: device 3 x M or null
void apply_fastop(FastOp &op, const double *x, double *y, int precision, const double *targets, int64_t M);

// y = s (K x) + diag .* x on the context stream (device vectors of length N)
void apply_operator(Ctx &c, const bie_operator &op, int precision, const double *x, double *y);

// Near field (bie_nearfield.cpp / bie_nearfield.cu)
Rule singular_rule(int node, double offset);
NearField &get_nearfield(Ctx &c, int depth, double offset, int n_gauss);
void free_nearfield(NearField &nf);
// Fv, Gv: device, nnz complex each (may be null when the flag is off); values
// are ADDED with sign `sign` (accurate rule) or computed with the coarse rule.
void launch_nearfield(Ctx &c, const NearField &nf, double k_re, double k_im, int flags, bool coarse,
                      double sign, double *Fv, double *Gv);

// Mixed-precision assembly (bie_assemble_mixed.cu)
// host: builds d_mrecords / d_mphi from the FP64 records (E x lay.stride) and uploads them
void build_mixed_records(Ctx &c, const std::vector<double> &rec64);
void launch_assemble_mixed(Ctx &c, const AssembleArgs &a);
// Double-float assembly (K9); false when the arguments need the FP64 kernel
// (element factors, k-derivatives, device-resident k, or phase rotations
// beyond the Taylor tables)
bool launch_assemble_df64(Ctx &c, const AssembleArgs &a);

// FMA throughput probe (bie_peaks.cu)
void measure_peaks(int device, bie_peaks &out);

}  // namespace bie
