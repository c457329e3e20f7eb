// ORACLE / TEST INFRASTRUCTURE — implementations behind shim/mkl.h (see that header).
#include "mkl.h"
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <map>
#include "../lu_exact.hpp"

namespace {
// Factors keyed by the matrix pointer handed to dgetrf; the reference factorises once
// (EMSolver.cpp:75) and solves with the same pointer every RK stage (EMSolver.cpp:177).
std::map<const double *, vxo::SparseLU> g_factors;
}

lapack_int LAPACKE_dgetrf(int layout, lapack_int m, lapack_int n, double *a, lapack_int lda, lapack_int *ipiv) {
    if (layout != LAPACK_COL_MAJOR || m != n || lda != n) {
        std::fprintf(stderr, "mkl shim: unsupported dgetrf call\n");
        std::abort();
    }
    vxo::SparseLU lu;
    const int N = (int)n;
    int info = lu.factor(N, [&](int r, int c) { return a[(size_t)c * N + r]; });
    // Write the factors back in LAPACK's packed column-major form.
    for (size_t i = 0; i < (size_t)N * N; i++) a[i] = 0.0;
    for (int i = 0; i < N; i++) {
        for (auto &e : lu.Lrows[i]) a[(size_t)e.first * N + i] = e.second;
        for (auto &e : lu.Urows[i]) a[(size_t)e.first * N + i] = e.second;
        a[(size_t)i * N + i] = lu.udiag[i];
        ipiv[i] = lu.ipiv[i] + 1;
    }
    g_factors[a] = std::move(lu);
    return info;
}

lapack_int LAPACKE_dgetrs(int layout, char trans, lapack_int n, lapack_int nrhs, const double *a, lapack_int lda,
                          const lapack_int *ipiv, double *b, lapack_int ldb) {
    (void)ipiv;
    if (layout != LAPACK_COL_MAJOR || trans != 'N' || nrhs != 1 || lda != n || ldb != n) {
        std::fprintf(stderr, "mkl shim: unsupported dgetrs call\n");
        std::abort();
    }
    auto it = g_factors.find(a);
    if (it == g_factors.end()) {
        std::fprintf(stderr, "mkl shim: dgetrs on a matrix not factorised by the shim\n");
        std::abort();
    }
    it->second.solve(b);
    return 0;
}

void vdLn(lapack_int n, const double *a, double *r) {
    for (lapack_int i = 0; i < n; i++) r[i] = std::log(a[i]);
}

void vdExp(lapack_int n, const double *a, double *r) {
    for (lapack_int i = 0; i < n; i++) r[i] = std::exp(a[i]);
}
