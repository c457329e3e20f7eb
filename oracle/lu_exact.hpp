// ORACLE / TEST INFRASTRUCTURE — not part of the product.
//
// Fill-aware LU with partial pivoting that has the *exact* arithmetic of a dense,
// unblocked, right-looking Doolittle factorisation (LAPACK dgetf2 semantics):
//
//   for k = 0..n-1:
//     p = first row i >= k with the largest |a_ik|          (idamax tie rule)
//     swap full rows k and p;  ipiv[k] = p
//     for i > k:  l_ik = a_ik / a_kk                        (division, not reciprocal)
//                 a_ij = a_ij - l_ik * u_kj   for j > k      (k ascending)
//
// and of the column-oriented triangular solves used by dgetrs:
//   b <- P b (swaps in k order);  y_i = b_i - sum_{k<i, ascending} l_ik y_k;
//   x_i = (y_i - sum_{j>i, descending} u_ij x_j) / u_ii.
//
// Work is skipped only where an operand is an exact zero, which leaves every
// stored value bit-identical to the dense algorithm (x - 0*y == x, 0 - l*u == -(l*u)).
// This is how the Veritas Poisson operator (EMSolver.cpp:28-88, dense dgetrf once;
// EMSolver.cpp:156-192, dgetrs per RK stage) is factorised on the oracle side: the
// reference build links it through its MKL header shim, and the oracle port calls it
// directly, so both sides share bit-identical factors.  LAPACK itself is a third-party
// dependency of the reference (CMakeLists.txt:29-35, EMSolver.hpp:5-6); this file
// restates the published textbook algorithm instead of linking a particular LAPACK.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <utility>
#include <vector>

namespace vxo {

struct SparseLU {
    int n = 0;
    // Row-wise factors.  Lrows[i]: (col, l_ij) for j < i, ascending col.
    // Urows[i]: (col, u_ij) for j > i, descending col.  udiag[i] = u_ii.
    std::vector<std::vector<std::pair<int, double>>> Lrows, Urows;
    std::vector<double> udiag;
    std::vector<int> ipiv;  // 0-based pivot row chosen at step k

    // a(r, c) supplied through a callback so that both dense column-major input
    // (reference shim) and explicit triplets (port) can be used.
    template <class Get>
    int factor(int n_, Get get) {
        n = n_;
        // Working rows: sorted (col, val) vectors.
        std::vector<std::vector<std::pair<int, double>>> rows(n);
        for (int r = 0; r < n; r++) {
            for (int c = 0; c < n; c++) {
                double v = get(r, c);
                if (v != 0.0) rows[r].push_back({c, v});
            }
        }
        return factor_rows(std::move(rows));
    }

    int factor_rows(std::vector<std::vector<std::pair<int, double>>> rows) {
        n = (int)rows.size();
        // colset[c]: rows that currently hold an entry in column c (may contain
        // stale entries; verified against the row on use).
        std::vector<std::vector<int>> colset(n);
        for (int r = 0; r < n; r++)
            for (auto &e : rows[r]) colset[e.first].push_back(r);
        ipiv.assign(n, 0);
        Lrows.assign(n, {});
        Urows.assign(n, {});
        udiag.assign(n, 0.0);
        // Multipliers stored separately as they are produced (row identity follows swaps).
        std::vector<std::vector<std::pair<int, double>>> lstore(n);
        int info = 0;
        auto find_in_row = [&](const std::vector<std::pair<int, double>> &row, int c) -> const double * {
            auto it = std::lower_bound(row.begin(), row.end(), std::make_pair(c, -INFINITY),
                                       [](const std::pair<int, double> &a, const std::pair<int, double> &b) {
                                           return a.first < b.first;
                                       });
            if (it != row.end() && it->first == c) return &it->second;
            return nullptr;
        };
        for (int k = 0; k < n; k++) {
            // Candidate rows >= k with an entry in column k, ascending.
            std::vector<int> cand;
            for (int r : colset[k])
                if (r >= k) cand.push_back(r);
            std::sort(cand.begin(), cand.end());
            cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
            int p = k;
            double best = -1.0;
            // idamax over rows k..n-1 in ascending order; rows with no entry are zeros.
            // A zero row can only win when every candidate is zero.
            {
                const double *dk = find_in_row(rows[k], k);
                best = dk ? std::fabs(*dk) : 0.0;
                p = k;
                for (int r : cand) {
                    if (r == k) continue;
                    const double *v = find_in_row(rows[r], k);
                    if (!v) continue;
                    double a = std::fabs(*v);
                    if (a > best) {  // strictly greater keeps the first maximum
                        best = a;
                        p = r;
                    }
                }
            }
            ipiv[k] = p;
            if (p != k) {
                std::swap(rows[k], rows[p]);
                std::swap(lstore[k], lstore[p]);
                for (auto &e : rows[k]) colset[e.first].push_back(k);
                for (auto &e : rows[p]) colset[e.first].push_back(p);
            }
            const double *pk = find_in_row(rows[k], k);
            double akk = pk ? *pk : 0.0;
            if (akk == 0.0) {
                if (info == 0) info = k + 1;
                continue;
            }
            // U row k: entries j > k of row k (ascending in storage).
            std::vector<std::pair<int, double>> urow;
            for (auto &e : rows[k])
                if (e.first > k) urow.push_back(e);
            // Re-derive candidate rows after a possible swap.
            std::vector<int> elim;
            for (int r : colset[k])
                if (r > k) elim.push_back(r);
            std::sort(elim.begin(), elim.end());
            elim.erase(std::unique(elim.begin(), elim.end()), elim.end());
            for (int i : elim) {
                auto &row = rows[i];
                const double *v = find_in_row(row, k);
                if (!v) continue;
                double aik = *v;
                if (aik == 0.0) continue;
                double l = aik / akk;
                lstore[i].push_back({k, l});
                // Remove column k from the working row (it becomes L).
                std::vector<std::pair<int, double>> merged;
                merged.reserve(row.size() + urow.size());
                size_t a = 0, b = 0;
                while (a < row.size() || b < urow.size()) {
                    if (a < row.size() && row[a].first <= k) {
                        if (row[a].first < k) merged.push_back(row[a]);  // columns < k cannot occur
                        a++;
                        continue;
                    }
                    if (b >= urow.size() || (a < row.size() && row[a].first < urow[b].first)) {
                        merged.push_back(row[a]);
                        a++;
                    } else if (a >= row.size() || urow[b].first < row[a].first) {
                        // fill-in: 0 - l*u
                        merged.push_back({urow[b].first, 0.0 - l * urow[b].second});
                        colset[urow[b].first].push_back(i);
                        b++;
                    } else {
                        merged.push_back({row[a].first, row[a].second - l * urow[b].second});
                        a++;
                        b++;
                    }
                }
                row.swap(merged);
            }
            udiag[k] = akk;
            std::vector<std::pair<int, double>> ud(urow.rbegin(), urow.rend());
            Urows[k] = std::move(ud);
        }
        for (int i = 0; i < n; i++) Lrows[i] = lstore[i];
        return info;
    }

    void solve(double *b) const {
        for (int k = 0; k < n; k++)
            if (ipiv[k] != k) std::swap(b[k], b[ipiv[k]]);
        for (int i = 0; i < n; i++) {
            double s = b[i];
            for (auto &e : Lrows[i]) s = s - b[e.first] * e.second;
            b[i] = s;
        }
        for (int i = n - 1; i >= 0; i--) {
            double s = b[i];
            for (auto &e : Urows[i]) s = s - b[e.first] * e.second;
            b[i] = s / udiag[i];
        }
    }
};

}  // namespace vxo
