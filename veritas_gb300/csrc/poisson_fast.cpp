// Host set-up of the scan-based Poisson solve (the device part, poisson_scan.cu,
// documents the algorithm): the Woodbury columns
// Y = (1/c) G^{-T} G^{-1} [e_0 e_1 e_{m-1}] and the 3x3 factor K = (I + C U^T Y)^{-1} C,
// where C holds the top-left correction of T - c G G^T and the corner coupling of B.
#include <cmath>
#include <stdexcept>
#include <string>

#include "engine.hpp"

namespace vx {

namespace {

// (1/c) G^{-T} G^{-1} v, G = (I - S)(I - rho S), in place.
void apply_m0(std::vector<double> &v, double rho, double c_inv) {
    const size_t m = v.size();
    double acc = 0.0;
    for (size_t i = 0; i < m; i++) v[i] = acc = v[i] + acc;
    acc = 0.0;
    for (size_t i = 0; i < m; i++) v[i] = acc = v[i] + rho * acc;
    acc = 0.0;
    for (size_t i = m; i-- > 0;) v[i] = acc = v[i] + rho * acc;
    acc = 0.0;
    for (size_t i = m; i-- > 0;) v[i] = acc = v[i] + acc;
    for (auto &x : v) x *= c_inv;
}

}  // namespace

void Run::build_poisson_fast() {
    const double w1 = -16.0 / 30.0 / 0.4, w2 = 1.0 / 30.0 / 0.4;  // EMSolver.cpp:28
    const int m = n - 1;
    if (m < 4) throw std::invalid_argument("grid too small for the fast Poisson solve");
    if (m > kPsMaxUnknowns)
        throw std::invalid_argument("grid too large for the scan Poisson solve (n - 1 > " +
                                    std::to_string(kPsMaxUnknowns) + ")");
    const double rho = 7.0 - 4.0 * std::sqrt(3.0);
    const double c = w2 / rho;
    const double g1 = -(1.0 + rho);
    // T - c G G^T is c * [[(1+rho)^2 + rho^2, rho g1], [rho g1, rho^2]] at the top left
    double C[3][3] = {{c * (g1 * g1 + rho * rho), c * rho * g1, w2}, {c * rho * g1, c * rho * rho, 0.0}, {w2, 0.0, 0.0}};
    const int U[3] = {0, 1, m - 1};
    pf_Y.assign((size_t)3 * m, 0.0);
    double UY[3][3];
    for (int col = 0; col < 3; col++) {
        std::vector<double> e(m, 0.0);
        e[U[col]] = 1.0;
        apply_m0(e, rho, 1.0 / c);
        for (int k = 0; k < m; k++) pf_Y[(size_t)3 * k + col] = e[k];
        for (int r = 0; r < 3; r++) UY[r][col] = e[U[r]];
    }
    // A = I + C UY, K = A^{-1} C (Gaussian elimination with partial pivoting, 3x3)
    double A[3][6];
    for (int r = 0; r < 3; r++)
        for (int q = 0; q < 3; q++) {
            double v = (r == q) ? 1.0 : 0.0;
            for (int t = 0; t < 3; t++) v += C[r][t] * UY[t][q];
            A[r][q] = v;
            A[r][3 + q] = C[r][q];
        }
    for (int col = 0; col < 3; col++) {
        int piv = col;
        for (int r = col + 1; r < 3; r++)
            if (std::fabs(A[r][col]) > std::fabs(A[piv][col])) piv = r;
        if (A[piv][col] == 0.0) throw std::runtime_error("fast Poisson capacitance matrix is singular");
        if (piv != col)
            for (int q = 0; q < 6; q++) std::swap(A[piv][q], A[col][q]);
        for (int r = 0; r < 3; r++) {
            if (r == col) continue;
            const double f = A[r][col] / A[col][col];
            for (int q = 0; q < 6; q++) A[r][q] -= f * A[col][q];
        }
    }
    for (int r = 0; r < 3; r++)
        for (int q = 0; q < 3; q++) pfdev.K[3 * r + q] = A[r][3 + q] / A[r][r];
    dpf_Y = upload(pf_Y, eng->stream);
    eng->sync();
    pfdev.Y = dpf_Y.as<double>();
    pfdev.rho = rho;
    pfdev.c_inv = 1.0 / c;
    pfdev.w1 = w1;
    pfdev.w2 = w2;
}

}  // namespace vx
