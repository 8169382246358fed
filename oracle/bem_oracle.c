/*
 * ORACLE - test infrastructure only, never part of the product path.
 *
 * Plain-C (C99 + OpenMP) restatement of the dense collocation assembly of
 * BoundaryIntegralEquations.jl for 3- and 6-node triangles, used as the checker
 * for libbiegpu.so.  It follows the reference loop structure one to one:
 *
 *   Gauss-Legendre on [0,1]            src/2d/quadrature.jl:5-11
 *   triangularQuadpoints / rotated     src/3d/quadrature.jl:70-113
 *   rotated_midpoint_triangular_...    src/3d/quadrature.jl:116-144
 *   shape functions                    src/3d/surface_functions.jl:191-236
 *   discontinuous triangle physics     src/3d/surface_functions.jl:236-318,
 *                                      src/3d/SurfaceFunction.jl:430-439
 *   create_rotated_element             src/3d/assembly_collocation.jl:122-136
 *   interpolate_elements, jacobian!    src/3d/assembly_collocation.jl:27-66, src/3d/jacobian.jl:78-87
 *   find_closest_corner                src/3d/assembly_collocation.jl:102-115
 *   computing_integrals!               src/3d/assembly_collocation.jl:213-252
 *   greens3d!, freens3d!, freens3dk0!  src/3d/kernels.jl:13-55
 *   mygemm_vec!                        src/2d/assembly_collocation.jl:142-150
 *   assemble_parallel! (triangles)     src/3d/assembly_collocation.jl:270-353, 355-479
 *
 * Parity status: pinned against the reference's own solution-level tests
 * (rigid-sphere error table test/3d/assembly_test.jl:22-23, sphere area
 * test/3d/fmm_test.jl:11-28, rule weight sums test/3d/surface_functions_test.jl)
 * because the Julia reference cannot run in this environment.
 *
 * Julia's 3-argument hypot (maximum-abs scaling, used for distances and the
 * nearest-node choice) is restated in julia_hypot3 below.
 *
 * Build: oracle.build() in oracle/__init__.py (gcc -O2 -fopenmp -ffp-contract=off -shared).
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_LINEAR 1
#define OR_QUADRATIC 2
#define OR_DISC_CONSTANT 3    /* physics only: one node at the centroid            */
#define OR_DISC_LINEAR 4      /* physics only: psi_k = (s_k - beta) / (1 - 3 beta) */
#define OR_DISC_QUADRATIC 5   /* physics only: quadratic in the psi_k              */
#define OR_F 1
#define OR_G 2
#define OR_C 4

static const double PI = 3.14159265358979323846;

/* Julia Base 3-argument hypot: maxabs * sqrt(sum(abs2(x / maxabs))) */
static double julia_hypot3(double x, double y, double z) {
    double ax = fabs(x), ay = fabs(y), az = fabs(z);
    double m = ax;
    if (ay > m) m = ay;
    if (az > m) m = az;
    if (isnan(m) && (isinf(x) || isinf(y) || isinf(z))) return INFINITY;
    if (m == 0.0 || isinf(m)) return m;
    double a = x / m, b = y / m, c = z / m;
    return m * sqrt((a * a + b * b) + c * c);
}

/* ---------------- Gauss-Legendre (Newton on the Legendre recurrence) -------- */
static void legendre_eval(int n, double x, double *p, double *dp) {
    double p0 = 1.0, p1 = x;
    if (n == 0) { *p = 1.0; *dp = 0.0; return; }
    for (int k = 2; k <= n; ++k) {
        double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
    }
    *p = p1;
    *dp = n * (x * p1 - p0) / (x * x - 1.0);
}

/* nodes ascending in [-1,1] */
static void gauss_legendre(int n, double *x, double *w) {
    for (int i = 0; i < n; ++i) {
        /* Tricomi-type initial guess for the i-th smallest root */
        double t = PI * (4.0 * (n - i) - 1.0) / (4.0 * n + 2.0);
        double z = cos(t);
        for (int it = 0; it < 50; ++it) {
            double p, dp;
            legendre_eval(n, z, &p, &dp);
            double dz = p / dp;
            z -= dz;
            if (fabs(dz) <= 1e-17) break;
        }
        double p, dp;
        legendre_eval(n, z, &p, &dp);
        x[i] = z;
        w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
    if (n % 2 == 1) x[n / 2] = 0.0;
    /* symmetrise */
    for (int i = 0; i < n / 2; ++i) {
        double xs = 0.5 * (x[n - 1 - i] - x[i]);
        double ws = 0.5 * (w[n - 1 - i] + w[i]);
        x[i] = -xs; x[n - 1 - i] = xs;
        w[i] = ws;  w[n - 1 - i] = ws;
    }
}

/* curveLinearQuadpoints: nodes/weights on [0,1] */
static void curve_linear(int n, double *x, double *w) {
    gauss_legendre(n, x, w);
    for (int i = 0; i < n; ++i) {
        w[i] = 0.5 * w[i];
        x[i] = 0.5 * (x[i] + 1.0);
    }
}

/* kron(ones(m), nodex), kron(nodey, ones(n)), kron(wy, wx) */
static void tensor_grid(int n, int m, double *u, double *v, double *w) {
    double xn[64], wn[64], xm[64], wm[64];
    curve_linear(n, xn, wn);
    curve_linear(m, xm, wm);
    for (int j = 0; j < m; ++j)
        for (int i = 0; i < n; ++i) {
            u[j * n + i] = xn[i];
            v[j * n + i] = xm[j];
            w[j * n + i] = wm[j] * wn[i];
        }
}

/* Rule clustered at element node c (1..6) for the collocation assembly.
 * Returns number of points; u, v, w must hold 2*n*(m+1) entries. */
int oracle_rule(int n, int m, int c, double *U, double *V, double *W) {
    if (c >= 1 && c <= 3) {
        double u[4096], v[4096], w[4096];
        int Q = n * m;
        tensor_grid(n, m, u, v, w);
        for (int q = 0; q < Q; ++q) {
            double xi, eta, wt;
            if (c == 1) {            /* rotated_triangular_quadpoints */
                xi = u[q] * v[q];
                eta = (1.0 - u[q]) * v[q];
                wt = w[q] * v[q];
            } else {                 /* triangularQuadpoints (duffy) */
                xi = u[q];
                eta = v[q] * (1.0 - u[q]);
                wt = w[q] * fabs(1.0 - u[q]);
            }
            if (c == 3) { U[q] = eta; V[q] = xi; }   /* nodes_v, nodes_u = ... */
            else { U[q] = xi; V[q] = eta; }
            W[q] = wt;
        }
        return Q;
    } else {
        int me = (int)ceil(m / 2.0) * 2;
        double u[4096], v[4096], w[4096];
        int H = n * me;
        tensor_grid(n, me, u, v, w);
        for (int q = 0; q < H; ++q) {
            double X1 = 0.5 * u[q], Y1 = v[q] * (1.0 - u[q]);
            double X2 = (u[q] - 0.5) * v[q] + 0.5, Y2 = v[q] * (1.0 - u[q]);
            double W1 = w[q] * (0.5 * (1.0 - u[q])), W2 = w[q] * (0.5 * v[q]);
            double X[2] = {X1, X2}, Y[2] = {Y1, Y2}, Wt[2] = {W1, W2};
            for (int h = 0; h < 2; ++h) {
                int idx = h * H + q;
                if (c == 4) { U[idx] = X[h]; V[idx] = Y[h]; }
                else if (c == 5) { U[idx] = (1.0 - X[h]) - Y[h]; V[idx] = X[h]; }
                else { U[idx] = Y[h]; V[idx] = (1.0 - X[h]) - Y[h]; }
                W[idx] = Wt[h];
            }
        }
        return 2 * H;
    }
}

/* plain Duffy rule triangularQuadpoints(n, m) */
int oracle_duffy_rule(int n, int m, double *U, double *V, double *W) {
    return oracle_rule(n, m, 2, U, V, W);
}

static int nnodes(int kind) {
    if (kind == OR_DISC_CONSTANT) return 1;
    return (kind == OR_LINEAR || kind == OR_DISC_LINEAR) ? 3 : 6;
}

/* node offset beta of the discontinuous kinds (set by the caller per mesh) */
static double g_beta = 0.0;
void oracle_set_beta(double beta) { g_beta = beta; }

static double psik(double s) { return (s - g_beta) / (1.0 - 3.0 * g_beta); }

static void basis(int kind, double u, double v, double *N) {
    if (kind == OR_DISC_CONSTANT) {
        N[0] = 1.0;
    } else if (kind == OR_DISC_LINEAR || kind == OR_DISC_QUADRATIC) {
        const double p3 = psik(1.0 - u - v), pu = psik(u), pv = psik(v);
        if (kind == OR_DISC_LINEAR) {
            N[0] = p3; N[1] = pu; N[2] = pv;
        } else {
            N[0] = p3 * (2.0 * p3 - 1.0);
            N[1] = pu * (2.0 * pu - 1.0);
            N[2] = pv * (2.0 * pv - 1.0);
            N[3] = 4.0 * pu * p3;
            N[4] = 4.0 * pu * pv;
            N[5] = 4.0 * pv * p3;
        }
    } else if (kind == OR_LINEAR) {
        N[0] = (1.0 - u) - v; N[1] = u; N[2] = v;
    } else {
        N[0] = ((1.0 - v) - u) * ((1.0 - 2.0 * v) - 2.0 * u);
        N[1] = u * (2.0 * u - 1.0);
        N[2] = v * (2.0 * v - 1.0);
        N[3] = 4.0 * u * ((1.0 - v) - u);
        N[4] = 4.0 * u * v;
        N[5] = 4.0 * v * ((1.0 - v) - u);
    }
}

/* basis values of `kind` at n points (N: nnodes x n, column-major) */
void oracle_basis(int kind, double beta, int64_t n, const double *u, const double *v, double *N) {
    const double saved = g_beta;
    g_beta = beta;
    for (int64_t q = 0; q < n; ++q) basis(kind, u[q], v[q], N + (size_t)q * nnodes(kind));
    g_beta = saved;
}

static void basis_deriv(int kind, double u, double v, double *du, double *dv) {
    if (kind == OR_LINEAR) {
        du[0] = -1; du[1] = 1; du[2] = 0;
        dv[0] = -1; dv[1] = 0; dv[2] = 1;
    } else {
        double l = (1.0 - v) - u;
        du[0] = -(2.0 * l - 1.0) - 2.0 * l; du[1] = 4.0 * u - 1.0; du[2] = 0.0;
        du[3] = 4.0 * l - 4.0 * u; du[4] = 4.0 * v; du[5] = -4.0 * v;
        dv[0] = -(2.0 * l - 1.0) - 2.0 * l; dv[1] = 0.0; dv[2] = 4.0 * v - 1.0;
        dv[3] = -4.0 * u; dv[4] = 4.0 * u; dv[5] = 4.0 * l - 4.0 * v;
    }
}

/* SurfaceElement for one element and one rule: x_q (3xQ), n_q (3xQ), jac*w (Q) */
typedef struct {
    double *x, *n, *jw;
} elem_interp;

static void interpolate_element(int skind, const double *coords, const int64_t *topo, int64_t e,
                                int Q, const double *U, const double *V, const double *W,
                                double *x, double *nrm, double *jw) {
    int NS = nnodes(skind);
    double N[6], du[6], dv[6];
    for (int q = 0; q < Q; ++q) {
        basis(skind, U[q], V[q], N);
        basis_deriv(skind, U[q], V[q], du, dv);
        double X[3] = {0, 0, 0}, T[3] = {0, 0, 0}, S[3] = {0, 0, 0};
        for (int a = 0; a < NS; ++a) {
            const double *c = coords + 3 * (topo[NS * e + a] - 1);
            for (int k = 0; k < 3; ++k) {
                X[k] += c[k] * N[a];
                T[k] += c[k] * du[a];
                S[k] += c[k] * dv[a];
            }
        }
        double nn[3] = {T[1] * S[2] - T[2] * S[1], T[2] * S[0] - T[0] * S[2], T[0] * S[1] - T[1] * S[0]};
        double jac = julia_hypot3(nn[0], nn[1], nn[2]);
        for (int k = 0; k < 3; ++k) {
            x[3 * q + k] = X[k];
            nrm[3 * q + k] = -nn[k] / jac;
        }
        jw[q] = jac * W[q];
    }
}

/* Sum over all elements of jacobian x weight of a rule (the sphere-area test,
 * test/3d/fmm_test.jl:11-28 with interpolate_elements(mesh; n, m)). */
double oracle_total_weight(const double *coords, const int64_t *topo, int skind, int64_t E,
                           int n, int m) {
    double U[4096], V[4096], W[4096], x[3 * 4096], nr[3 * 4096], jw[4096];
    int Q = oracle_rule(m, n, 2, U, V, W);  /* getQuadpoints(shape, m, n) */
    double s = 0.0;
    for (int64_t e = 0; e < E; ++e) {
        interpolate_element(skind, coords, topo, e, Q, U, V, W, x, nr, jw);
        for (int q = 0; q < Q; ++q) s += jw[q];
    }
    return s;
}

/*
 * Dense assembly.  coords 3xNc, topo NSxE (1-based), ptopo NPxE (1-based),
 * sources 3xN (mesh.sources: physics-node coordinates), targets 3xM.
 * F, G: M x N complex column-major (interleaved doubles), C: M complex.
 */
int oracle_assemble_w(const double *coords, int64_t Nc, const int64_t *topo, int skind,
                      const int64_t *ptopo, int pkind, int64_t E, const double *sources, int64_t N,
                      const double *targets, int64_t M, int n, int m, double kre, double kim,
                      int flags, double *F, double *G, double *C, int nthreads, const double *gw);

int oracle_assemble(const double *coords, int64_t Nc, const int64_t *topo, int skind,
                    const int64_t *ptopo, int pkind, int64_t E, const double *sources, int64_t N,
                    const double *targets, int64_t M, int n, int m, double kre, double kim,
                    int flags, double *F, double *G, double *C, int nthreads) {
    return oracle_assemble_w(coords, Nc, topo, skind, ptopo, pkind, E, sources, N, targets, M, n, m,
                             kre, kim, flags, F, G, C, nthreads, NULL);
}

static int gauss_triangle(int n, double *u, double *v, double *w);

/* Same assembly with an optional per-element complex factor gw[e] (E complex)
 * on the single-layer contributions (element admittance weighting).
 * n < 0: every rule is the symmetric (-n)-point triangle rule (the far-field
 * rule of setup_fast_operator, src/3d/fast_multipole_method.jl:163-170). */
static int assemble_impl(const double *coords, int64_t Nc, const int64_t *topo, int skind,
                         const int64_t *ptopo, int pkind, int64_t E, const double *sources, int64_t N,
                         const double *targets, int64_t M, int n, int m, double kre, double kim,
                         int flags, double *F, double *G, double *C, int nthreads, const double *gw,
                         int tm);

int oracle_assemble_w(const double *coords, int64_t Nc, const int64_t *topo, int skind,
                      const int64_t *ptopo, int pkind, int64_t E, const double *sources, int64_t N,
                      const double *targets, int64_t M, int n, int m, double kre, double kim,
                      int flags, double *F, double *G, double *C, int nthreads, const double *gw) {
    return assemble_impl(coords, Nc, topo, skind, ptopo, pkind, E, sources, N, targets, M, n, m, kre, kim,
                         flags, F, G, C, nthreads, gw, -1);
}

/* taylor_assemble! (src/3d/rosebem.jl:56-157) with U = I: matrices m = 0..order
 * of the k-derivatives (taylor_greens3d!, taylor_freens3d!, src/3d/kernels.jl:
 * 94-118), F and G stacked as M x N x (order + 1); C from the same rules. */
int oracle_taylor_assemble(const double *coords, int64_t Nc, const int64_t *topo, int skind,
                           const int64_t *ptopo, int pkind, int64_t E, const double *sources, int64_t N,
                           const double *targets, int64_t M, int n, int m, double kre, double kim,
                           int flags, int order, double *F, double *G, double *C, int nthreads) {
    for (int t = 0; t <= order; ++t) {
        const int fl = (flags & (OR_F | OR_G)) | (t == 0 ? (flags & OR_C) : 0);
        const int st = assemble_impl(coords, Nc, topo, skind, ptopo, pkind, E, sources, N, targets, M, n, m,
                                     kre, kim, fl, F ? F + (size_t)2 * t * M * N : NULL,
                                     G ? G + (size_t)2 * t * M * N : NULL, C, nthreads, NULL, t);
        if (st) return st;
    }
    return 0;
}

static int assemble_impl(const double *coords, int64_t Nc, const int64_t *topo, int skind,
                         const int64_t *ptopo, int pkind, int64_t E, const double *sources, int64_t N,
                         const double *targets, int64_t M, int n, int m, double kre, double kim,
                         int flags, double *F, double *G, double *C, int nthreads, const double *gw,
                         int tm) {
    (void)Nc;
    if (n < 0) {
        double tu[16], tv[16], tw[16];
        if (-n > 16 || gauss_triangle(-n, tu, tv, tw) <= 0) return -1;
    }
    const int NP = nnodes(pkind);
    /* linear geometry: the three corner rules; quadratic geometry: one rule
     * per physics node up to 6 (assembly_collocation.jl:287-289, 372-387) */
    const int R = (skind == OR_LINEAR || NP < 6) ? 3 : 6;
    int Q[6];
    double *U[6], *V[6], *W[6], *PHI[6];
    double *X[6], *NR[6], *JW[6];
    for (int r = 0; r < R; ++r) {
        U[r] = malloc(4096 * sizeof(double));
        V[r] = malloc(4096 * sizeof(double));
        W[r] = malloc(4096 * sizeof(double));
        Q[r] = n < 0 ? gauss_triangle(-n, U[r], V[r], W[r]) : oracle_rule(n, m, r + 1, U[r], V[r], W[r]);
        /* physics interpolation transposed: Q x NP */
        PHI[r] = malloc((size_t)Q[r] * NP * sizeof(double));
        for (int q = 0; q < Q[r]; ++q) {
            double Nv[6];
            basis(pkind, U[r][q], V[r][q], Nv);
            for (int a = 0; a < NP; ++a) PHI[r][q * NP + a] = Nv[a];
        }
        X[r] = malloc((size_t)E * 3 * Q[r] * sizeof(double));
        NR[r] = malloc((size_t)E * 3 * Q[r] * sizeof(double));
        JW[r] = malloc((size_t)E * Q[r] * sizeof(double));
        for (int64_t e = 0; e < E; ++e)
            interpolate_element(skind, coords, topo, e, Q[r], U[r], V[r], W[r],
                                X[r] + (size_t)e * 3 * Q[r], NR[r] + (size_t)e * 3 * Q[r],
                                JW[r] + (size_t)e * Q[r]);
    }
    if (flags & OR_F) memset(F, 0, (size_t)M * N * 2 * sizeof(double));
    if (flags & OR_G) memset(G, 0, (size_t)M * N * 2 * sizeof(double));
    if (flags & OR_C) memset(C, 0, (size_t)M * 2 * sizeof(double));
    const double complex k = kre + I * kim;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static)
#endif
    for (int64_t i = 0; i < M; ++i) {
        const double *s = targets + 3 * i;
        double complex integrand[4096];
        double rr[4096];
        double cacc = 0.0;
        for (int64_t e = 0; e < E; ++e) {
            const int64_t *pn = ptopo + (size_t)NP * e;
            /* find_closest_corner over the physics nodes (mesh.sources) */
            double best = INFINITY;
            int c = 0;
            for (int a = 0; a < NP; ++a) {
                const double *P = sources + 3 * (pn[a] - 1);
                double d = julia_hypot3(P[0] - s[0], P[1] - s[1], P[2] - s[2]);
                if (d < best) { best = d; c = a; }
            }
            /* the linear-geometry method's if/elseif/else: nodes 4-6 -> rule 3
             * (assembly_collocation.jl:330-346); the k-derivative assembly uses
             * the corner rules the same way (taylor_assemble!, src/3d/rosebem.jl:114-127) */
            if ((tm >= 0 || skind == OR_LINEAR) && c > 2) c = 2;
            const int Qr = Q[c];
            const double *x = X[c] + (size_t)e * 3 * Qr;
            const double *nr = NR[c] + (size_t)e * 3 * Qr;
            const double *jw = JW[c] + (size_t)e * Qr;
            const double *phi = PHI[c];
            /* compute_distances! */
            for (int q = 0; q < Qr; ++q)
                rr[q] = julia_hypot3(x[3 * q] - s[0], x[3 * q + 1] - s[1], x[3 * q + 2] - s[2]);
            if (flags & OR_G) {
                for (int q = 0; q < Qr; ++q)
                    integrand[q] = cexp(I * k * rr[q]) / (4.0 * PI * rr[q]);      /* greens3d! */
                if (tm >= 0)                                                        /* taylor_greens3d! */
                    for (int q = 0; q < Qr; ++q) integrand[q] *= cpow(I * rr[q], tm);
                for (int q = 0; q < Qr; ++q) integrand[q] = integrand[q] * jw[q];  /* integrand_mul! */
                for (int a = 0; a < NP; ++a) {                                      /* mygemm_vec! */
                    double complex acc = 0.0;
                    for (int q = 0; q < Qr; ++q) acc += integrand[q] * phi[q * NP + a];
                    if (gw) acc *= gw[2 * e] + I * gw[2 * e + 1];
                    double *g = G + 2 * ((size_t)(pn[a] - 1) * M + i);
                    g[0] += creal(acc);
                    g[1] += cimag(acc);
                }
            }
            if (flags & OR_C) {
                double ci = 0.0;
                for (int q = 0; q < Qr; ++q) {                                      /* freens3dk0! */
                    double dn = nr[3 * q] * (x[3 * q] - s[0]) + nr[3 * q + 1] * (x[3 * q + 1] - s[1]) +
                                nr[3 * q + 2] * (x[3 * q + 2] - s[2]);
                    double val = -dn / (4.0 * PI * rr[q] * rr[q] * rr[q]);
                    ci += val * jw[q];                                              /* sum_to_c! */
                }
                cacc += ci;
            }
            if (flags & OR_F) {
                for (int q = 0; q < Qr; ++q) {                                      /* freens3d! */
                    double dn = nr[3 * q] * (x[3 * q] - s[0]) + nr[3 * q + 1] * (x[3 * q + 1] - s[1]) +
                                nr[3 * q + 2] * (x[3 * q + 2] - s[2]);
                    if (tm >= 0)                                                    /* taylor_freens3d! */
                        integrand[q] = cexp(I * k * rr[q]) * cpow(I * rr[q], tm) *
                                       (1.0 - I * k * rr[q] - tm) * (-dn) /
                                       (4.0 * PI * rr[q] * rr[q] * rr[q]);
                    else
                        integrand[q] = cexp(I * k * rr[q]) * (I * k * rr[q] - 1.0) * dn /
                                       (4.0 * PI * rr[q] * rr[q] * rr[q]);
                    integrand[q] = integrand[q] * jw[q];
                }
                for (int a = 0; a < NP; ++a) {
                    double complex acc = 0.0;
                    for (int q = 0; q < Qr; ++q) acc += integrand[q] * phi[q * NP + a];
                    double *f = F + 2 * ((size_t)(pn[a] - 1) * M + i);
                    f[0] += creal(acc);
                    f[1] += cimag(acc);
                }
            }
        }
        if (flags & OR_C) {
            C[2 * i] = cacc;
            C[2 * i + 1] = 0.0;
        }
    }
    for (int r = 0; r < R; ++r) {
        free(U[r]); free(V[r]); free(W[r]); free(PHI[r]);
        free(X[r]); free(NR[r]); free(JW[r]);
    }
    return 0;
}

/* ======================================================================== *
 * Near field: sparse_assemble_parallel! (src/3d/assembly_collocation_losses.jl:
 * 200-405), its adaptive rules (src/3d/adaptive_integration.jl:172-246) and the
 * coarse partial_assemble_parallel! (src/3d/fast_multipole_method.jl:11-81).
 * ======================================================================== */

/* gauss_points_triangle (src/3d/adaptive_integration.jl:13-64) */
static int gauss_triangle(int n, double *u, double *v, double *w) {
    static const double t1[] = {1.0 / 3, 1.0 / 3, 0.5};
    static const double t3[] = {1.0 / 6, 1.0 / 6, 1.0 / 6, 2.0 / 3, 1.0 / 6, 1.0 / 6, 1.0 / 6, 2.0 / 3, 1.0 / 6};
    static const double t4[] = {1.0 / 3, 1.0 / 3, -9.0 / 32, 0.2, 0.6, 25.0 / 96, 0.2, 0.2, 25.0 / 96,
                                0.6, 0.2, 25.0 / 96};
    static const double t7[] = {1.0 / 3, 1.0 / 3, 0.1125,
                                0.797426985353087, 0.101286507323456, 0.0629695902724135,
                                0.101286507323456, 0.797426985353087, 0.0629695902724135,
                                0.101286507323456, 0.101286507323456, 0.0629695902724135,
                                0.059715871789770, 0.470142064105115, 0.066197076394253,
                                0.470142064105115, 0.059715871789770, 0.066197076394253,
                                0.470142064105115, 0.470142064105115, 0.066197076394253};
    const double *t;
    switch (n) {
        case 1: t = t1; break;
        case 3: t = t3; break;
        case 4: t = t4; break;
        case 7: t = t7; break;
        default: return -1;
    }
    for (int i = 0; i < n; ++i) { u[i] = t[3 * i]; v[i] = t[3 * i + 1]; w[i] = t[3 * i + 2]; }
    return n;
}

static double d3(const double *a, const double *b) {
    double x = a[0] - b[0], y = a[1] - b[1], z = a[2] - b[2];
    return sqrt((x * x + y * y) + z * z);
}

typedef struct { double *t; int n, cap; } tri_list;   /* 6 doubles per kept triangle */

static void subdivide_triangle(const double *P1, const double *P2, const double *P3,
                               const double *src, double esize, double tol, tri_list *out) {
    double P12[2] = {(P1[0] + P2[0]) / 2, (P1[1] + P2[1]) / 2};
    double P23[2] = {(P2[0] + P3[0]) / 2, (P2[1] + P3[1]) / 2};
    double P31[2] = {(P3[0] + P1[0]) / 2, (P3[1] + P1[1]) / 2};
    double C[2] = {(P1[0] + P2[0] + P3[0]) / 3.0, (P1[1] + P2[1] + P3[1]) / 3.0};
    /* subelement = Diagonal(ones(3)) * N(u, v), N = [1-u-v, u, v] */
    double c[3] = {(1.0 - C[0]) - C[1], C[0], C[1]};
    double a[3] = {(1.0 - P1[0]) - P1[1], P1[0], P1[1]};
    double b[3] = {(1.0 - P2[0]) - P2[1], P2[0], P2[1]};
    double d[3] = {(1.0 - P3[0]) - P3[1], P3[0], P3[1]};
    double dist = d3(c, src);
    if (d3(a, src) < dist) dist = d3(a, src);
    if (d3(b, src) < dist) dist = d3(b, src);
    if (d3(d, src) < dist) dist = d3(d, src);
    double size = d3(b, a);
    if (d3(d, b) > size) size = d3(d, b);
    if (d3(a, d) > size) size = d3(a, d);
    if (size < esize * tol) size = 0;
    if (size > dist / 4) {
        subdivide_triangle(P1, P12, P31, src, esize, tol, out);
        subdivide_triangle(P12, P2, P23, src, esize, tol, out);
        subdivide_triangle(P31, P23, P3, src, esize, tol, out);
        subdivide_triangle(P12, P23, P31, src, esize, tol, out);
    } else {
        if (out->n + 1 > out->cap) {
            out->cap = out->cap ? 2 * out->cap : 1024;
            out->t = realloc(out->t, (size_t)out->cap * 6 * sizeof(double));
        }
        double *t = out->t + 6 * (size_t)out->n;
        t[0] = P1[0]; t[1] = P1[1]; t[2] = P2[0]; t[3] = P2[1]; t[4] = P3[0]; t[5] = P3[1];
        out->n++;
    }
}

/* singular_triangle_integration(shape, 3, source, I, 1e-6) for element node c
 * (1..6) with offset `off`; returns the number of points (<= cap). */
int oracle_singular_rule(int c, double off, double *U, double *V, double *W, int cap) {
    double src[3];
    switch (c) {
        case 1: src[0] = 1.0; src[1] = off; src[2] = off; break;
        case 2: src[0] = off; src[1] = 1.0; src[2] = off; break;
        case 3: src[0] = off; src[1] = off; src[2] = 1.0; break;
        case 4: src[0] = 0.5; src[1] = 0.5; src[2] = off; break;
        case 5: src[0] = off; src[1] = 0.5; src[2] = 0.5; break;
        default: src[0] = 0.5; src[1] = off; src[2] = 0.5; break;
    }
    const double e1[3] = {1, 0, 0}, e2[3] = {0, 1, 0}, e3[3] = {0, 0, 1};
    double esize = d3(e2, e1);
    if (d3(e3, e2) > esize) esize = d3(e3, e2);
    if (d3(e1, e3) > esize) esize = d3(e1, e3);
    tri_list L = {NULL, 0, 0};
    const double A[2] = {0, 0}, B[2] = {1, 0}, Cc[2] = {0, 1};
    subdivide_triangle(A, B, Cc, src, esize, 1e-6, &L);
    double gu[3], gv[3], gw[3];
    gauss_triangle(3, gu, gv, gw);
    int q = 0;
    for (int i = 0; i < L.n; ++i) {
        const double *t = L.t + 6 * (size_t)i;
        double s1 = sqrt((t[2] - t[0]) * (t[2] - t[0]) + (t[3] - t[1]) * (t[3] - t[1]));
        double s2 = sqrt((t[4] - t[2]) * (t[4] - t[2]) + (t[5] - t[3]) * (t[5] - t[3]));
        double s3 = sqrt((t[0] - t[4]) * (t[0] - t[4]) + (t[1] - t[5]) * (t[1] - t[5]));
        double dim = s1 < s2 ? s1 : s2;
        if (s3 < dim) dim = s3;
        double cu = ((t[0] + t[2]) + t[4]) / 3, cv = ((t[1] + t[3]) + t[5]) / 3;
        for (int g = 0; g < 3; ++g) {
            if (q < cap) {
                U[q] = (gu[g] - 1.0 / 3.0) * dim + cu;
                V[q] = (gv[g] - 1.0 / 3.0) * dim + cv;
                W[q] = gw[g] * (dim * dim);
            }
            ++q;
        }
    }
    free(L.t);
    return q;
}

/*
 * Near-field F, G in CSR order.  pairs: npairs x (2 + NP) = (row, element,
 * CSR slot of each physics node), built from connected_sources by the caller.
 * coarse = 0: adaptive rules chosen by the nearest GEOMETRY node; 1: the
 * n_gauss triangle rule.  F, G: nnz complex (zeroed here).
 */
int oracle_nearfield(const double *coords, const int64_t *topo, int skind, const int64_t *ptopo,
                     int pkind, const double *sources, const int64_t *pairs, int64_t npairs,
                     int64_t nnz, double offset, int coarse, int n_gauss, double kre, double kim,
                     int flags, double *F, double *G, int nthreads) {
    const int NS = nnodes(skind), NP = nnodes(pkind);
    const int R = coarse ? 1 : NS;
    int Q[6];
    double *U[6], *V[6], *W[6];
    for (int r = 0; r < R; ++r) {
        int cap = 32768;
        U[r] = malloc(cap * sizeof(double)); V[r] = malloc(cap * sizeof(double)); W[r] = malloc(cap * sizeof(double));
        Q[r] = coarse ? gauss_triangle(n_gauss, U[r], V[r], W[r]) : oracle_singular_rule(r + 1, offset, U[r], V[r], W[r], cap);
        if (Q[r] < 0 || Q[r] > cap) return -1;
    }
    if (flags & OR_F) memset(F, 0, (size_t)nnz * 16);
    if (flags & OR_G) memset(G, 0, (size_t)nnz * 16);
    const double complex k = kre + I * kim;
    const int ps = 2 + NP;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
    omp_lock_t lock;
    omp_init_lock(&lock);
#pragma omp parallel for schedule(dynamic, 16)
#endif
    for (int64_t p = 0; p < npairs; ++p) {
        const int64_t *pr = pairs + p * ps;
        const int64_t i = pr[0], e = pr[1];
        const double *s = sources + 3 * i;
        int r = 0;
        if (!coarse) {   /* find_closest_corner on the element's geometry nodes */
            double best = INFINITY;
            for (int a = 0; a < NS; ++a) {
                const double *X = coords + 3 * (topo[NS * e + a] - 1);
                double dd = julia_hypot3(X[0] - s[0], X[1] - s[1], X[2] - s[2]);
                if (dd < best) { best = dd; r = a; }
            }
        }
        double *x = malloc((size_t)Q[r] * 3 * sizeof(double));
        double *nr = malloc((size_t)Q[r] * 3 * sizeof(double));
        double *jw = malloc((size_t)Q[r] * sizeof(double));
        interpolate_element(skind, coords, topo, e, Q[r], U[r], V[r], W[r], x, nr, jw);
        double complex fa[6] = {0}, ga[6] = {0};
        for (int q = 0; q < Q[r]; ++q) {
            double rr = julia_hypot3(x[3 * q] - s[0], x[3 * q + 1] - s[1], x[3 * q + 2] - s[2]);
            double Nv[6];
            basis(pkind, U[r][q], V[r][q], Nv);
            double dn = nr[3 * q] * (x[3 * q] - s[0]) + nr[3 * q + 1] * (x[3 * q + 1] - s[1]) +
                        nr[3 * q + 2] * (x[3 * q + 2] - s[2]);
            double complex fv = cexp(I * k * rr) * (I * k * rr - 1.0) * dn / (4.0 * PI * rr * rr * rr) * jw[q];
            double complex gv = cexp(I * k * rr) / (4.0 * PI * rr) * jw[q];
            for (int a = 0; a < NP; ++a) { fa[a] += fv * Nv[a]; ga[a] += gv * Nv[a]; }
        }
        free(x); free(nr); free(jw);
#ifdef _OPENMP
        omp_set_lock(&lock);
#endif
        for (int a = 0; a < NP; ++a) {
            const int64_t slot = pr[2 + a];
            if (flags & OR_F) { F[2 * slot] += creal(fa[a]); F[2 * slot + 1] += cimag(fa[a]); }
            if (flags & OR_G) { G[2 * slot] += creal(ga[a]); G[2 * slot + 1] += cimag(ga[a]); }
        }
#ifdef _OPENMP
        omp_unset_lock(&lock);
#endif
    }
#ifdef _OPENMP
    omp_destroy_lock(&lock);
#endif
    for (int r = 0; r < R; ++r) { free(U[r]); free(V[r]); free(W[r]); }
    return 0;
}
