// Host part of the visco-thermal system: air properties, the three wavenumbers
// and boundary-condition constants, and the tangential derivative matrices.
//
//   ambient_to_properties    src/utils/ambient_to_properties.jl:1-134 (Rasmussen,
//                            DTU report PL-11b, 1997, annex A, table A.1)
//   visco_thermal_constants  src/utils/lossy_constants.jl:1-34
//   tangential_derivatives   src/3d/interpolation_function_derivatives.jl:10-18, 36-118
#include "bie_internal.h"

#include <algorithm>
#include <cmath>
#include <complex>

namespace bie {

namespace {

using cplx = std::complex<double>;

// Rasmussen's table A.1, one coefficient list per property
constexpr double kEnhance[3] = {1.00062, 3.14e-8, 5.6e-7};
constexpr double kZ[9] = {1.58123e-6, -2.9331e-8, 1.1043e-10, 5.707e-6, -2.051e-8,
                          1.9898e-4,  -2.376e-6,  1.83e-11,   -0.765e-8};
constexpr double kSound[16] = {331.5024,  0.603055,  -0.000528, 51.471935, 0.1495874, -0.000782,
                               -1.82e-7,  3.73e-8,   -2.93e-10, -85.20931, -0.228525, 5.91e-5,
                               -2.835149, -2.15e-13, 29.179762, 0.000486};
constexpr double kGamma[16] = {1.400822,   -1.75e-5,   -1.73e-7,   -0.0873629, -0.0001665, -3.26e-6,
                               2.047e-8,   -1.26e-10,  5.939e-14,  -0.1199717, -0.0008693, 1.979e-6,
                               -0.01104,   -3.478e-16, 0.0450616,  1.82e-6};
constexpr double kVisc[6] = {84.986, 7.0, 113.157, -1.0, -3.7501e-3, -100.015};
constexpr double kCond[3] = {60.054, 1.846, 2.06e-6};
constexpr double kCp[10] = {0.251625, -9.2525e-5, 2.1334e-7, -1.0043e-10, 0.12477,
                            -2.283e-5, 1.267e-7,  0.01116,   4.61e-6,     1.74e-8};

// the 16-term form of the speed of sound and the ratio of specific heats
double poly16(const double *a, double t, double xw, double ps, double xc) {
    return a[0] + a[1] * t + a[2] * t * t + (a[3] + a[4] * t + a[5] * t * t) * xw +
           (a[6] + a[7] * t + a[8] * t * t) * ps + (a[9] + a[10] * t + a[11] * t * t) * xc +
           a[12] * xw * xw + a[13] * ps * ps + a[14] * xc * xc + a[15] * xw * ps * xc;
}

void put(double *d, cplx z) {
    d[0] = z.real();
    d[1] = z.imag();
}

}  // namespace

void ambient_to_properties(double f, double ps, double t, double H, double out[10]) {
    constexpr double T0 = 273.15, T20 = 293.15, psr = 101325.0, pi = 3.14159265358979323846;
    const double T = T0 + t;
    const double psv = psr * std::pow(10.0, 4.6151 - 6.8346 * std::pow((T0 + 0.01) / T, 1.261));
    const double fpst = kEnhance[0] + kEnhance[1] * ps + kEnhance[2] * t * t;
    const double xw = H * psv * fpst / (100.0 * ps);
    const double Z = 1.0 -
                     ps / T * (kZ[0] + kZ[1] * t + kZ[2] * t * t + (kZ[3] + kZ[4]) * xw + (kZ[5] + kZ[6]) * xw * xw) +
                     (ps / T) * (ps / T) * (kZ[7] + kZ[8] * xw * xw);
    const double xc = 0.0004;
    const double rho = (3.48349 + 1.44 * (xc - 0.0004)) * 1e-3 * ps / (Z * T) * (1.0 - 0.3780 * xw);
    const double c0 = poly16(kSound, t, xw, ps, xc);
    const double gamma = poly16(kGamma, t, xw, ps, xc);
    const double eta =
        (kVisc[0] + kVisc[1] * T + (kVisc[2] + kVisc[3] * T) * xw + kVisc[4] * T * T + kVisc[5] * xw * xw) * 1e-8;
    // as in the reference, the humidity terms of the conductivity use the
    // viscosity coefficients 4 and 5
    double landa = (kCond[0] + kCond[1] * T + kCond[2] * T * T + (kVisc[3] + kVisc[4] * T) * xw) * 1e-8;
    double Cp = kCp[0] + kCp[1] * T + kCp[2] * T * T + kCp[3] * T * T * T +
                (kCp[4] + kCp[5] * T + kCp[6] * T * T) * xw + (kCp[7] + kCp[8] * T + kCp[9] * T * T) * xw * xw;
    const double frO = ps / psr * (24.0 + 4.04e6 * xw * (0.2 + 1e3 * xw) / (3.91 + 1e3 * xw));
    const double frN = ps / psr * std::pow(T / T20, -0.5) *
                       (9.0 + 28.0e3 * xw * std::exp(-4.170 * (std::pow(T / T20, -1.0 / 3.0) - 1.0)));
    const double aO = 0.01275 * f * f * std::exp(-2239.1 / T) / (frO + f * f / frO) * std::pow(T20 / T, 2.5);
    const double aN = 0.1068 * f * f * std::exp(-3352.0 / T) / (frN + f * f / frN) * std::pow(T20 / T, 2.5);
    const double cf = 1.0 / (1.0 / c0 - aO / (2 * pi * frO) - aN / (2 * pi * frN));
    const double alfa = 18.4e-12 * f * f / (ps / psr) * std::sqrt(T / T20) + aO + aN;
    Cp *= 4.1868 * 1000.0;
    landa *= 4.1868 * 1000.0;
    const double Cv = Cp / gamma;
    const double beta = rho * (Cp - Cv);
    const double v[10] = {rho, c0, cf, gamma, eta, alfa, Cp, Cv, landa, beta};
    std::copy(v, v + 10, out);
}

bie_lossy_constants visco_thermal_constants(double freq, double S, double pa, double t, double Hr) {
    constexpr double pi = 3.14159265358979323846;
    double a[10];
    ambient_to_properties(freq, pa, t, Hr, a);
    const double rho = a[0], c = a[1], cpcv = a[3], mu = a[4], Cp = a[6], landa = a[8], beta = a[9];
    const double eta = 0.6 * mu;
    // characteristic lengths
    const double lh = landa / (rho * Cp * c);
    const double lv = (eta + 4.0 * mu / 3.0) / (rho * c);
    const double lvp = mu / (rho * c);
    const double lvh = lv + (cpcv - 1.0) * lh;
    const double lvhp = (cpcv - 1.0) * (lh - lv);
    const double kp = 2 * pi * freq / c;
    const cplx Si(0.0, S);   // S i
    const cplx ka2 = kp * kp / (1.0 - Si * kp * lvh - kp * kp * lh * lvhp);
    const cplx kh2 = Si * kp / (lh * (1.0 + Si * kp * lvhp));
    const cplx kv2 = Si * kp / lvp;
    const cplx tau_a = (cpcv - 1.0) / (beta * cpcv * (1.0 + Si * lh * ka2 / kp));
    const cplx tau_h = (cpcv - 1.0) / (beta * cpcv * (1.0 + Si * lh * kh2 / kp));
    const cplx phi_a = -Si / (rho * 2.0 * pi * freq * (1.0 + Si * lv * ka2 / kp));
    const cplx phi_h = -Si / (rho * 2.0 * pi * freq * (1.0 + Si * lv * kh2 / kp));
    bie_lossy_constants k{};
    k.rho = rho;
    k.c = c;
    k.kp = kp;
    put(k.ka, std::sqrt(ka2));
    put(k.kh, std::sqrt(kh2));
    put(k.kv, std::sqrt(kv2));
    put(k.tau_a, tau_a);
    put(k.tau_h, tau_h);
    put(k.phi_a, phi_a);
    put(k.phi_h, phi_h);
    k.eta = eta;
    k.mu = mu;
    put(k.mu_a, phi_a - tau_a * phi_h / tau_h);
    put(k.mu_h, tau_a * phi_h / tau_h);
    return k;
}

void node_pattern(int64_t N, int64_t E, int NP, const int32_t *ptopo, std::vector<int64_t> &row_ptr,
                  std::vector<int32_t> &cols) {
    std::vector<std::vector<int32_t>> rows((size_t)N);
    for (int64_t e = 0; e < E; ++e)
        for (int a = 0; a < NP; ++a) {
            auto &r = rows[(size_t)ptopo[NP * e + a]];
            for (int b = 0; b < NP; ++b) r.push_back(ptopo[NP * e + b]);
        }
    row_ptr.assign((size_t)N + 1, 0);
    cols.clear();
    for (int64_t i = 0; i < N; ++i) {
        auto &r = rows[(size_t)i];
        std::sort(r.begin(), r.end());
        r.erase(std::unique(r.begin(), r.end()), r.end());
        cols.insert(cols.end(), r.begin(), r.end());
        row_ptr[(size_t)i + 1] = (int64_t)cols.size();
    }
}

void tangential_derivatives(int shape_kind, int physics_kind, const double *coords, int64_t E,
                            const int32_t *topo, const int32_t *ptopo, int64_t N, std::vector<int64_t> &row_ptr,
                            std::vector<int32_t> &cols, std::vector<double> &Dx, std::vector<double> &Dy,
                            std::vector<double> &Dz) {
    if (is_discontinuous(physics_kind))
        fail(BIE_ERR_UNSUPPORTED, "tangential derivatives take continuous physics only");
    const int NS = n_nodes_of_kind(shape_kind), NP = n_nodes_of_kind(physics_kind);
    node_pattern(N, E, NP, ptopo, row_ptr, cols);
    Dx.assign(cols.size(), 0.0);
    Dy.assign(cols.size(), 0.0);
    Dz.assign(cols.size(), 0.0);
    std::vector<int> count((size_t)N, 0);
    for (int64_t i = 0; i < E * NP; ++i) ++count[(size_t)ptopo[i]];
    // nodal (u, v) of the physics nodes (corners, then edge midpoints 1-2, 2-3, 3-1)
    static const double nodal_u[6] = {0.0, 1.0, 0.0, 0.5, 0.5, 0.0};
    static const double nodal_v[6] = {0.0, 0.0, 1.0, 0.0, 0.5, 0.5};
    double su[6], sv[6], pu[6], pv[6];
    for (int64_t e = 0; e < E; ++e) {
        for (int a = 0; a < NP; ++a) {
            shape_derivs(shape_kind, nodal_u[a], nodal_v[a], su, sv);
            shape_derivs(physics_kind, nodal_u[a], nodal_v[a], pu, pv);
            double tu[3] = {0, 0, 0}, tv[3] = {0, 0, 0};
            for (int s = 0; s < NS; ++s) {
                const double *X = coords + 3 * (int64_t)topo[NS * e + s];
                for (int k = 0; k < 3; ++k) {
                    tu[k] += X[k] * su[s];
                    tv[k] += X[k] * sv[s];
                }
            }
            const double nz[3] = {tu[1] * tv[2] - tu[2] * tv[1], tu[2] * tv[0] - tu[0] * tv[2],
                                  tu[0] * tv[1] - tu[1] * tv[0]};
            // M g = l with rows tu, tv, nz: g = M^-1 l by the adjugate; l = (dN/du, dN/dv, 0)
            const double M[3][3] = {{tu[0], tu[1], tu[2]}, {tv[0], tv[1], tv[2]}, {nz[0], nz[1], nz[2]}};
            double inv[3][3];
            inv[0][0] = M[1][1] * M[2][2] - M[1][2] * M[2][1];
            inv[0][1] = M[0][2] * M[2][1] - M[0][1] * M[2][2];
            inv[0][2] = M[0][1] * M[1][2] - M[0][2] * M[1][1];
            inv[1][0] = M[1][2] * M[2][0] - M[1][0] * M[2][2];
            inv[1][1] = M[0][0] * M[2][2] - M[0][2] * M[2][0];
            inv[1][2] = M[0][2] * M[1][0] - M[0][0] * M[1][2];
            inv[2][0] = M[1][0] * M[2][1] - M[1][1] * M[2][0];
            inv[2][1] = M[0][1] * M[2][0] - M[0][0] * M[2][1];
            inv[2][2] = M[0][0] * M[1][1] - M[0][1] * M[1][0];
            const double det = M[0][0] * inv[0][0] + M[0][1] * inv[1][0] + M[0][2] * inv[2][0];
            if (!(std::fabs(det) > 0.0)) fail(BIE_ERR_INVALID, "degenerate element in the derivative matrices");
            const int32_t row = ptopo[NP * e + a];
            const double w = 1.0 / (det * count[(size_t)row]);
            const int32_t *rb = cols.data() + row_ptr[(size_t)row];
            const int32_t *re = cols.data() + row_ptr[(size_t)row + 1];
            for (int b = 0; b < NP; ++b) {
                const int32_t col = ptopo[NP * e + b];
                const int64_t p = row_ptr[(size_t)row] + (std::lower_bound(rb, re, col) - rb);
                // g_k = sum_j inv[k][j] l_j with l = (pu[b], pv[b], 0)
                Dx[(size_t)p] += (inv[0][0] * pu[b] + inv[0][1] * pv[b]) * w;
                Dy[(size_t)p] += (inv[1][0] * pu[b] + inv[1][1] * pv[b]) * w;
                Dz[(size_t)p] += (inv[2][0] * pu[b] + inv[2][1] * pv[b]) * w;
            }
        }
    }
}

}  // namespace bie
