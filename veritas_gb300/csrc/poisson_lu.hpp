// Host set-up of the Poisson operator (EMFieldSolver::EMFieldSolver, EMSolver.cpp:28-88).
//
// The reference assembles a dense n x n column-major matrix (n = finest x size) and
// factorises it once with LAPACK dgetrf; every RK stage then calls dgetrs.  The matrix
// is a periodic 4th-order Laplacian stencil with row/column 0 replaced by a gauge
// condition, so its LU factors with partial pivoting have O(n) nonzeros.  PoissonLU
// builds only the nonzeros and runs the unblocked right-looking factorisation with
// partial pivoting (first maximal |pivot|, full-row swaps, multipliers by division),
// skipping only exact-zero operands — the same values the dense algorithm stores.  The
// factors are uploaded once per run; the device applies the column-oriented triangular
// solves in the same order (fields64.cu: k_poisson).
#pragma once
#include <utility>
#include <vector>

namespace vx {

struct PoissonLU {
    int n = 0;
    std::vector<int> ipiv;                             // pivot row of step k (0-based)
    std::vector<int> perm;                             // composed interchanges: b'[k] = b[perm[k]]
    std::vector<int> lptr, lcol, uptr, ucol;           // CSR rows: L ascending, U descending
    std::vector<double> lval, uval, udiag, urdiag;  // urdiag = RN(1/u_ii)
    std::vector<double> urdiag_lo;                  // 1/u_ii - urdiag to double precision
    // Factorise the Veritas Poisson matrix of size n (n >= 5).  Returns 0 or k+1 for a
    // zero pivot at step k.
    int build(int n);
    // Host reference solve with the same operation order as the device (tests only).
    void solve(double *b) const;
    // Band form of the factors for the device (four columns either side of the
    // diagonal, the rest as "far" entries in summation order).
    struct Band {
        std::vector<double> band, diag, rdiag, rdiag_lo, fval;
        std::vector<int> fptr, fcol;
        // Lower factor: the far terms of every row are accumulated by up to kMaxSlots
        // dedicated lanes.  At step i (when x_{i-1} has just been produced) slot s
        // subtracts slot_coef[s*n + i] * x_{i-1}; slot_load[s*n + i] >= 0 names the row
        // whose right-hand side the slot takes up at the start of step i; take[i] is the
        // slot holding row i+4's finished sum at step i (-1: that row has no far terms).
        // nslots = -1 when the rows cannot be scheduled on the lanes.
        static constexpr int kMaxSlots = 4;
        int nslots = 0;
        std::vector<double> slot_coef;
        std::vector<int> slot_load, take;
        // Upper factor: rows below far_pre_row have all their far columns at or above
        // far_pre_col, so their far terms can be subtracted in one parallel pass once the
        // solution is known from far_pre_col up (-1: not possible).
        int far_pre_col = -1;
    };
    Band lower_band() const;
    Band upper_band() const;
    // For each row k, the first chunk of rows_per_chunk steps of the device's forward sweep
    // (fields64.cu, pois_fwd_fast) that reads x[k]: the band lanes read rows 0..3 before
    // the first step and row i+5 at step i, the accumulator lanes the row they take up one
    // step ahead.  Empty when the sweep runs in its other form (nslots < 0).
    std::vector<int> first_read_chunk(const Band &Lb, int rows_per_chunk) const;
};

}  // namespace vx
