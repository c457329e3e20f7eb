#include "poisson_lu.hpp"

#include <algorithm>
#include <cmath>
#include <map>
#include <stdexcept>

namespace vx {

namespace {
using Row = std::vector<std::pair<int, double>>;  // (column, value), ascending column

double *row_find(Row &r, int c) {
    auto it = std::lower_bound(r.begin(), r.end(), c, [](const std::pair<int, double> &e, int v) { return e.first < v; });
    return (it != r.end() && it->first == c) ? &it->second : nullptr;
}
}  // namespace

int PoissonLU::build(int N) {
    if (N < 5) throw std::invalid_argument("Poisson operator needs at least 5 finest cells");
    n = N;
    // Matrix entries A(r, c) = pM[c*n + r] of EMSolver.cpp:41-67.
    const double w1 = -16.0 / 30.0 / 0.4, w2 = 1.0 / 30.0 / 0.4, w3 = 1 / 0.4;
    std::vector<std::map<int, double>> acc(n);
    auto put = [&](int col, int row, double v) { acc[row][col] = v; };  // later writes win, as in the dense fill
    for (int i = 2; i < n - 2; i++) {
        put(i, i, w3);
        put(i, i + 1, w1);
        put(i, i - 1, w1);
        put(i, i + 2, w2);
        put(i, i - 2, w2);
    }
    put(0, 0, 1.0);
    put(1, 1, w3);
    put(1, 2, w1);
    put(1, 0, w1);
    put(1, 3, w2);
    put(1, n - 1, w2);
    put(n - 2, n - 2, w3);
    put(n - 2, n - 1, w1);
    put(n - 2, n - 3, w1);
    put(n - 2, 0, w2);
    put(n - 2, n - 4, w2);
    put(n - 1, n - 1, w3);
    put(n - 1, 0, w1);
    put(n - 1, n - 2, w1);
    put(n - 1, 1, w2);
    put(n - 1, n - 3, w2);
    std::vector<Row> rows(n);
    for (int r = 0; r < n; r++)
        for (auto &kv : acc[r])
            if (kv.second != 0.0) rows[r].push_back({kv.first, kv.second});

    // Which rows hold column c (may be stale; checked on use).
    std::vector<std::vector<int>> holders(n);
    for (int r = 0; r < n; r++)
        for (auto &e : rows[r]) holders[e.first].push_back(r);
    std::vector<Row> lrows(n), urows(n);
    udiag.assign(n, 0.0);
    ipiv.assign(n, 0);
    int info = 0;
    for (int k = 0; k < n; k++) {
        std::vector<int> &h = holders[k];
        std::sort(h.begin(), h.end());
        h.erase(std::unique(h.begin(), h.end()), h.end());
        int p = k;
        double *dk = row_find(rows[k], k);
        double best = dk ? std::fabs(*dk) : 0.0;
        for (int r : h) {
            if (r <= k) continue;
            double *v = row_find(rows[r], k);
            if (v && std::fabs(*v) > best) {
                best = std::fabs(*v);
                p = r;
            }
        }
        ipiv[k] = p;
        if (p != k) {
            std::swap(rows[k], rows[p]);
            std::swap(lrows[k], lrows[p]);
            for (auto &e : rows[k]) holders[e.first].push_back(k);
            for (auto &e : rows[p]) holders[e.first].push_back(p);
        }
        double *pk = row_find(rows[k], k);
        double akk = pk ? *pk : 0.0;
        if (akk == 0.0) {
            if (!info) info = k + 1;
            continue;
        }
        Row urow;
        for (auto &e : rows[k])
            if (e.first > k) urow.push_back(e);
        std::vector<int> targets;
        for (int r : holders[k])
            if (r > k) targets.push_back(r);
        std::sort(targets.begin(), targets.end());
        targets.erase(std::unique(targets.begin(), targets.end()), targets.end());
        for (int r : targets) {
            Row &row = rows[r];
            double *v = row_find(row, k);
            if (!v || *v == 0.0) continue;
            double l = *v / akk;
            lrows[r].push_back({k, l});
            Row out;
            out.reserve(row.size() + urow.size());
            size_t a = 0, b = 0;
            while (a < row.size() && row[a].first <= k) a++;
            while (a < row.size() || b < urow.size()) {
                if (b == urow.size() || (a < row.size() && row[a].first < urow[b].first)) {
                    out.push_back(row[a++]);
                } else if (a == row.size() || urow[b].first < row[a].first) {
                    out.push_back({urow[b].first, 0.0 - l * urow[b].second});
                    holders[urow[b].first].push_back(r);
                    b++;
                } else {
                    out.push_back({row[a].first, row[a].second - l * urow[b].second});
                    a++;
                    b++;
                }
            }
            row.swap(out);
        }
        udiag[k] = akk;
        std::reverse(urow.begin(), urow.end());
        urows[k] = std::move(urow);
    }
    urdiag.resize(n);
    urdiag_lo.resize(n);
    for (int i = 0; i < n; i++) {
        urdiag[i] = 1.0 / udiag[i];
        // low part of 1/u: (1 - u*y) is exact by FMA, scaled by y
        urdiag_lo[i] = std::fma(-udiag[i], urdiag[i], 1.0) * urdiag[i];
    }
    perm.resize(n);
    for (int i = 0; i < n; i++) perm[i] = i;
    for (int k = 0; k < n; k++)
        if (ipiv[k] != k) std::swap(perm[k], perm[ipiv[k]]);
    lptr.assign(1, 0);
    uptr.assign(1, 0);
    lcol.clear();
    lval.clear();
    ucol.clear();
    uval.clear();
    for (int i = 0; i < n; i++) {
        for (auto &e : lrows[i]) {
            lcol.push_back(e.first);
            lval.push_back(e.second);
        }
        lptr.push_back((int)lcol.size());
        for (auto &e : urows[i]) {
            ucol.push_back(e.first);
            uval.push_back(e.second);
        }
        uptr.push_back((int)ucol.size());
    }
    return info;
}

PoissonLU::Band PoissonLU::lower_band() const {
    Band B;
    B.band.assign((size_t)4 * n, 0.0);
    B.fptr.push_back(0);
    for (int i = 0; i < n; i++) {
        for (int e = lptr[i]; e < lptr[i + 1]; e++) {  // ascending columns
            int d = i - lcol[e];
            if (d >= 1 && d <= 4) {
                B.band[4 * i + d - 1] = lval[e];
            } else {
                B.fcol.push_back(lcol[e]);
                B.fval.push_back(lval[e]);
            }
        }
        B.fptr.push_back((int)B.fcol.size());
    }
    // Schedule every row with far terms on an accumulator lane: row r occupies a slot from
    // step (first far column + 1) to step r - 4, when lane 3 takes its sum.
    struct Iv {
        int open, close, row;
    };
    std::vector<Iv> ivs;
    for (int i = 0; i < n; i++)
        if (B.fptr[i + 1] > B.fptr[i]) ivs.push_back({B.fcol[B.fptr[i]] + 1, i - 4, i});
    std::sort(ivs.begin(), ivs.end(), [](const Iv &x, const Iv &y) { return x.open < y.open; });
    std::vector<int> slot_of(ivs.size(), -1), busy_until(Band::kMaxSlots, -1);
    int used = 0;
    bool ok = true;
    for (size_t k = 0; k < ivs.size() && ok; k++) {
        int s = -1;
        for (int q = 0; q < Band::kMaxSlots; q++)
            if (busy_until[q] < ivs[k].open) {
                s = q;
                break;
            }
        if (s < 0 || ivs[k].close < ivs[k].open) ok = false;
        else {
            slot_of[k] = s;
            busy_until[s] = ivs[k].close;
            used = std::max(used, s + 1);
        }
    }
    if (!ok) {
        B.nslots = -1;
        return B;
    }
    B.nslots = used;
    B.slot_coef.assign((size_t)Band::kMaxSlots * n, 0.0);
    B.slot_load.assign((size_t)Band::kMaxSlots * n, -1);
    B.take.assign(n, -1);
    for (size_t k = 0; k < ivs.size(); k++) {
        const int s = slot_of[k], r = ivs[k].row;
        B.slot_load[(size_t)s * n + ivs[k].open] = r;
        for (int e = B.fptr[r]; e < B.fptr[r + 1]; e++) B.slot_coef[(size_t)s * n + B.fcol[e] + 1] = B.fval[e];
        B.take[r - 4] = s;
    }
    return B;
}

PoissonLU::Band PoissonLU::upper_band() const {
    Band B;
    B.band.assign((size_t)4 * n, 0.0);
    B.diag = udiag;
    B.rdiag = urdiag;
    B.rdiag_lo = urdiag_lo;
    B.fptr.push_back(0);
    for (int i = 0; i < n; i++) {
        for (int e = uptr[i]; e < uptr[i + 1]; e++) {  // descending columns
            int d = ucol[e] - i;
            if (d >= 1 && d <= 4) {
                B.band[4 * i + d - 1] = uval[e];
            } else {
                B.fcol.push_back(ucol[e]);
                B.fval.push_back(uval[e]);
            }
        }
        B.fptr.push_back((int)B.fcol.size());
    }
    // Far terms of the rows below the last 256-row chunk can be precomputed in parallel
    // after that chunk when every such row's far columns lie inside it.
    const int R = 256;
    const int last = ((n + R - 1) / R - 1) * R;
    bool ok = last > 4;
    for (int i = 0; ok && i < last - 4; i++)
        for (int e = B.fptr[i]; e < B.fptr[i + 1]; e++)
            if (B.fcol[e] < last) ok = false;
    B.far_pre_col = ok ? last : -1;
    return B;
}

std::vector<int> PoissonLU::first_read_chunk(const Band &Lb, int rows_per_chunk) const {
    std::vector<int> fc;
    if (Lb.nslots < 0 || n < 5 || rows_per_chunk <= 0) return fc;  // the device sweep's other form
    const int R = rows_per_chunk;
    fc.assign(n, -1);
    auto mark = [&](int k, int c) {
        if (k >= 0 && k < n && (fc[k] < 0 || c < fc[k])) fc[k] = c;
    };
    const int nch = (n + R - 1) / R;
    for (int c = 0; c < nch; c++) {
        const int r0 = c * R, cnt = std::min(R, n - r0);
        if (c == 0)
            for (int k = 0; k < 4; k++) mark(k, 0);  // the four band lanes' first rows
        // the band's last lane: x[i + 4] at the chunk's start, x[i + 5] one row ahead
        for (int k = r0 + 4; k <= r0 + cnt + 4; k++) mark(k, c);
        // the accumulator lanes: the row taken up at step i, read one step ahead
        for (int s = 0; s < Lb.nslots; s++)
            for (int i = r0; i <= r0 + cnt && i < n; i++) mark(Lb.slot_load[(size_t)s * n + i], c);
    }
    for (int k = 0; k < n; k++)
        if (fc[k] < 0) return {};
    return fc;
}

void PoissonLU::solve(double *b) const {
    for (int k = 0; k < n; k++)
        if (ipiv[k] != k) std::swap(b[k], b[ipiv[k]]);
    for (int i = 0; i < n; i++) {
        double s = b[i];
        for (int e = lptr[i]; e < lptr[i + 1]; e++) s = s - b[lcol[e]] * lval[e];
        b[i] = s;
    }
    for (int i = n - 1; i >= 0; i--) {
        double s = b[i];
        for (int e = uptr[i]; e < uptr[i + 1]; e++) s = s - b[ucol[e]] * uval[e];
        b[i] = s / udiag[i];
    }
}

}  // namespace vx
