// Host side of the AMR machinery: connectivity between patches and the op lists of the
// ghost fills, the coarse/fine interface fluxes and the limiter coefficient exchange.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <chrono>
#include <cstdio>
#include <cstdlib>

#include "engine.hpp"

namespace vx {

namespace {

bool on_line(int x, int y1, int y2) { return ((x - y1) > -1) && ((y2 - x) > -1); }

// Rectangle::CalculateConnectivityFromFiner (Rectangle.cpp:768-864): `cur` is the coarse
// patch, `rf` a patch one level finer.
void conn_from_finer(Rect &cur, Rect &rf, int r) {
    const int x2 = rf.x_pos / r - cur.x_pos, p2 = rf.p_pos / r - cur.p_pos;
    const int nx2 = rf.n_x / r, np2 = rf.n_p / r;
    const int lower_x = std::max(0, x2), upper_x = std::min(cur.n_x, x2 + nx2);
    const int lower_p = std::max(0, p2), upper_p = std::min(cur.n_p, p2 + np2);
    for (int i = lower_x; i < upper_x; i++)
        for (int j = lower_p; j < upper_p; j++) {
            cur.nested[cur.ns(i, j)] = 1;
            cur.finer[cur.ns(i, j)] = rf.id;
        }
    const int last = (int)rf.xp.size() - 1;
    if ((x2 + nx2) < (cur.n_x + 1) && (x2 + nx2) > -1)
        for (int i = lower_p; i < upper_p; i++) {
            cur.finer_x[cur.ns(x2 + nx2, i)] = rf.id;
            cur.ifx[cur.ns(x2 + nx2, i)] = 1;
        }
    if ((x2 + nx2) < cur.n_x && (x2 + nx2) > -1) {
        for (int i = lower_p; i < upper_p; i++) {
            rf.xp[i - p2 + 1] = cur.id;
            rf.sxp[i - p2 + 1] = 0;
        }
        if (on_line(p2 - 1, 0, cur.n_p - 1)) rf.xp[0] = cur.id, rf.sxp[0] = 0;
        if (on_line(p2 + np2, 0, cur.n_p - 1)) rf.xp[last] = cur.id, rf.sxp[last] = 0;
    }
    if (x2 < (cur.n_x + 1) && x2 > -1)
        for (int i = lower_p; i < upper_p; i++) {
            cur.finer_x[cur.ns(x2, i)] = rf.id;
            cur.ifx[cur.ns(x2, i)] = 1;
        }
    if (x2 < (cur.n_x + 1) && x2 > 0) {
        for (int i = lower_p; i < upper_p; i++) {
            rf.xm[i - p2 + 1] = cur.id;
            rf.sxm[i - p2 + 1] = 0;
        }
        if (on_line(p2 - 1, 0, cur.n_p - 1)) rf.xm[0] = cur.id, rf.sxm[0] = 0;
        if (on_line(p2 + np2, 0, cur.n_p - 1)) rf.xm[last] = cur.id, rf.sxm[last] = 0;
    }
    if ((p2 + np2) < (cur.n_p + 1) && (p2 + np2) > -1)
        for (int i = lower_x; i < upper_x; i++) {
            cur.finer_p[cur.ns(i, p2 + np2)] = rf.id;
            cur.ifp[cur.ns(i, p2 + np2)] = 1;
        }
    if ((p2 + np2) < cur.n_p && (p2 + np2) > -1)
        for (int i = lower_x; i < upper_x; i++) {
            rf.pp[i - x2] = cur.id;
            rf.spp[i - x2] = 0;
        }
    if (p2 < (cur.n_p + 1) && p2 > -1)
        for (int i = lower_x; i < upper_x; i++) {
            cur.finer_p[cur.ns(i, p2)] = rf.id;
            cur.ifp[cur.ns(i, p2)] = 1;
        }
    if (p2 < (cur.n_p + 1) && p2 > 0)
        for (int i = lower_x; i < upper_x; i++) {
            rf.pm[i - x2] = cur.id;
            rf.spm[i - x2] = 0;
        }
}

// Rectangle::CalculateConnectivitySame (Rectangle.cpp:671-766): `b` is another patch of
// the same level as `a`.
void conn_same(Rect &a, const Rect &b, int r) {
    const int nx2 = b.n_x, np2 = b.n_p;
    const int xr = b.x_pos - a.x_pos, pr = b.p_pos - a.p_pos;
    const int lx = (int)a.xm.size() - 1;
    if (xr == a.n_x) {
        int lower = std::max(b.p_pos, a.p_pos), upper = std::min(a.p_pos + a.n_p, b.p_pos + np2);
        if (on_line(-1, pr, pr + np2 - 1)) a.xp[0] = b.id, a.sxp[0] = 1;
        if (on_line(a.n_p, pr, pr + np2 - 1)) a.xp[lx] = b.id, a.sxp[lx] = 1;
        for (; lower < upper; lower += r) {
            int i1 = (lower - a.p_pos) / r + 1;
            a.xp.at(i1) = b.id;
            a.sxp.at(i1) = 1;
        }
    }
    if (xr == -nx2) {
        int lower = std::max(b.p_pos, a.p_pos), upper = std::min(a.p_pos + a.n_p, b.p_pos + np2);
        if (on_line(-1, pr, pr + np2 - 1)) a.xm[0] = b.id, a.sxm[0] = 1;
        if (on_line(a.n_p, pr, pr + np2 - 1)) a.xm[lx] = b.id, a.sxm[lx] = 1;
        for (; lower < upper; lower += r) {
            int i1 = (lower - a.p_pos) / r + 1;
            a.xm.at(i1) = b.id;
            a.sxm.at(i1) = 1;
        }
    }
    if (pr == a.n_p) {
        int lower = std::max(b.x_pos, a.x_pos), upper = std::min(a.x_pos + a.n_x, b.x_pos + nx2);
        if (on_line(-1, xr, xr + nx2 - 1)) a.xm[lx] = b.id, a.sxm[lx] = 1;
        if (on_line(a.n_x, xr, xr + nx2 - 1)) a.xp[lx] = b.id, a.sxp[lx] = 1;
        for (; lower < upper; lower += r) {
            int i1 = (lower - a.x_pos) / r;
            a.pp.at(i1) = b.id;
            a.spp.at(i1) = 1;
        }
    }
    if (pr == -np2) {
        int lower = std::max(b.x_pos, a.x_pos), upper = std::min(a.x_pos + a.n_x, b.x_pos + nx2);
        if (on_line(-1, xr, xr + nx2 - 1)) a.xm[0] = b.id, a.sxm[0] = 1;
        if (on_line(a.n_x, xr, xr + nx2 - 1)) a.xp[0] = b.id, a.sxp[0] = 1;
        for (; lower < upper; lower += r) {
            int i1 = (lower - a.x_pos) / r;
            a.pm.at(i1) = b.id;
            a.spm.at(i1) = 1;
        }
    }
}

constexpr int kMaxRatio = 8;  // refinement ratios above it are refused (build_amr)
constexpr int kMaxBatches = 255;  // op batches per list (the fills and exchanges take a few)

// Assigns each op of an ordered list the smallest batch that keeps the list's read /
// write orders (RAW, WAR, WAW) on the cells it touches, with the last write / read batch
// of each cell kept in dense per-patch byte planes (batch + 1, 0 for none; allocated when
// a patch is first touched): the restriction ops of large nested regions number in the
// millions.
struct PlaneScheduler {
    explicit PlaneScheduler(const std::vector<Rect *> &patches) : flat(patches), last_w(patches.size()), last_r(patches.size()) {}
    const std::vector<Rect *> &flat;
    std::vector<std::vector<uint8_t>> last_w, last_r;  // batch + 1, 0 = none
    std::vector<int> batch;
    int nbatches = 0;
    size_t slot(int patch, int i, int j) {
        if (patch < 0 || patch >= (int)flat.size()) throw std::invalid_argument("AMR layout: ghost op on no patch");
        const Rect &R = *flat[patch];
        if (i < -2 || i >= R.n_x + 2 || j < -2 || j >= R.n_p + 2)
            throw std::invalid_argument("AMR layout: ghost op cell outside its patch");
        if (last_w[patch].empty()) {
            const size_t cells = (size_t)(R.n_x + 4) * (R.n_p + 4);
            last_w[patch].assign(cells, 0);
            last_r[patch].assign(cells, 0);
        }
        return (size_t)(i + 2) * (R.n_p + 4) + (j + 2);
    }
    // cells as (patch, i, j) triples
    void add(const int (*reads)[3], int nr, const int (*writes)[3], int nw) {
        int b = 0;
        for (int q = 0; q < nr; q++) {
            const size_t c = slot(reads[q][0], reads[q][1], reads[q][2]);
            b = std::max<int>(b, last_w[reads[q][0]][c]);
        }
        for (int q = 0; q < nw; q++) {
            const size_t c = slot(writes[q][0], writes[q][1], writes[q][2]);
            b = std::max<int>(b, last_w[writes[q][0]][c]);
            b = std::max<int>(b, last_r[writes[q][0]][c]);
        }
        if (b >= kMaxBatches) throw std::runtime_error("AMR op schedule too deep");
        for (int q = 0; q < nr; q++) {
            uint8_t &v = last_r[reads[q][0]][slot(reads[q][0], reads[q][1], reads[q][2])];
            v = (uint8_t)std::max<int>(v, b + 1);
        }
        for (int q = 0; q < nw; q++) last_w[writes[q][0]][slot(writes[q][0], writes[q][1], writes[q][2])] = (uint8_t)(b + 1);
        batch.push_back(b);
        nbatches = std::max(nbatches, b + 1);
    }
    // Restrictions of `len` consecutive cells (di, dj + k) of patch dst from the r x r
    // blocks at (si, sj + r k) of patch src, scheduled as one unit: every cell takes the
    // largest batch any of them needs, which keeps each cell's read / write orders (a
    // later batch than a cell's own minimum never runs before an op it must follow, and
    // the ops emitted after see the batch in the planes).  Bounds are checked once for
    // the row; one batch entry per cell op.
    void add_restrict_row(int dst, int di, int dj, int src, int si, int sj, int r, int len) {
        slot(src, si, sj);
        slot(src, si + r - 1, sj + r * len - 1);  // bounds of the row's blocks
        slot(dst, di, dj);
        const size_t cw = slot(dst, di, dj + len - 1) - (size_t)(len - 1);
        const int wp = flat[src]->n_p + 4;
        const size_t s0 = slot(src, si, sj);
        const uint8_t *lw = last_w[src].data();
        const uint8_t *dw = last_w[dst].data() + cw, *dr = last_r[dst].data() + cw;
        int b = 0;
        for (int a = 0; a < r; a++) {
            const uint8_t *row = lw + s0 + (size_t)a * wp;
            for (int q = 0; q < r * len; q++) b = std::max<int>(b, row[q]);
        }
        for (int k = 0; k < len; k++) b = std::max<int>(b, std::max(dw[k], dr[k]));
        if (b >= kMaxBatches) throw std::runtime_error("AMR op schedule too deep");
        uint8_t *lr = last_r[src].data();
        for (int a = 0; a < r; a++) {
            uint8_t *row = lr + s0 + (size_t)a * wp;
            for (int q = 0; q < r * len; q++) row[q] = std::max<uint8_t>(row[q], (uint8_t)(b + 1));
        }
        uint8_t *dwm = last_w[dst].data() + cw;
        for (int k = 0; k < len; k++) dwm[k] = (uint8_t)(b + 1);
        batch.insert(batch.end(), (size_t)len, b);
        nbatches = std::max(nbatches, b + 1);
    }
};

// Stable counting sort of the ops by batch; out.ptr gets the batch offsets.
template <class Op>
void sort_by_batch(std::vector<Op> &ops, const std::vector<int> &batch, int nb, Batched &out) {
    out.ptr.assign((size_t)nb + 1, 0);
    for (size_t k = 0; k < ops.size(); k++) out.ptr[batch[k] + 1]++;
    for (int b = 0; b < nb; b++) out.ptr[b + 1] += out.ptr[b];
    std::vector<int> fill(out.ptr.begin(), out.ptr.end() - 1);
    std::vector<Op> sorted(ops.size());
    for (size_t k = 0; k < ops.size(); k++) sorted[fill[batch[k]]++] = ops[k];
    ops.swap(sorted);
}

}  // namespace

// Every cell an op reads or writes must lie inside its patch's padded plane
// [-2, n + 2) x [-2, n + 2); a layout that breaks this is rejected before any launch.
void Run::validate_ops() const {
    const int r = S->refinementRatio;
    auto in = [&](int id, int i, int j) {
        if (id < 0 || id >= (int)flat.size()) return false;
        const Rect &R = *flat[id];
        return i >= -2 && i < R.n_x + 2 && j >= -2 && j < R.n_p + 2;
    };
    auto need = [](bool ok, const char *what) {
        if (!ok) throw std::invalid_argument(std::string("AMR layout: ") + what + " outside its patch");
    };
    for (const GhostOp &op : ghost_ops) {
        need(in(op.dst, op.di, op.dj), "ghost target");
        if (op.kind == kGhostCopy) need(in(op.src, op.si, op.sj), "ghost source");
        if (op.kind == kGhostRestrict)
            need(in(op.src, op.si, op.sj) && in(op.src, op.si + r - 1, op.sj + r - 1), "restriction source");
        if (op.kind == kGhostInterp) {
            need(in(op.src, op.si - 2, op.sj - 2) && in(op.src, op.si + 2, op.sj + 2), "interpolation stencil");
            need(op.sub >= 0 && op.sub < r * r, "interpolation entry");
        }
    }
    for (const IfaceOp &op : iface_ops) {
        need(in(op.coarse, op.ci, op.cj), "interface face");
        // r fine faces and the upwind neighbour of each
        if (op.dir == 0) need(in(op.fine, op.fi - 1, op.fj) && in(op.fine, op.fi, op.fj + r - 1), "fine x faces");
        else need(in(op.fine, op.fi, op.fj - 1) && in(op.fine, op.fi + r - 1, op.fj), "fine p faces");
    }
    for (const CSyncOp &op : csync_ops) {
        const bool xf = op.t < 2;
        need(in(op.nb, op.ni, op.nj) && in(op.nb, op.ni - (xf ? 1 : 0), op.nj - (xf ? 0 : 1)), "limiter face");
        const int span = op.kind == kCDiff ? r - 1 : 0;
        need(in(op.caller, op.ci - (xf ? 1 : 0), op.cj - (xf ? 0 : 1)) &&
                 in(op.caller, op.ci + (xf ? 0 : span), op.cj + (xf ? span : 0)),
             "limiter faces");
    }
    if (r > 8) throw std::invalid_argument("refinement ratio above 8 is not supported");
}

void Run::build_amr() {
    const int r = S->refinementRatio;
    const int L = S->maxDepth + 1;
    static const bool trace = std::getenv("VX_TRACE_INIT") != nullptr;
    auto t0 = std::chrono::steady_clock::now();
    auto lap = [&](const char *what) {
        if (!trace) return;
        auto t1 = std::chrono::steady_clock::now();
        std::fprintf(stderr, "vx amr %-15s %8.2f ms\n", what, std::chrono::duration<double, std::milli>(t1 - t0).count());
        t0 = t1;
    };
    flat.clear();
    int nrect = 0;
    for (auto &sp : rects)
        for (auto &lvl : sp)
            for (auto &rp : lvl) {
                Rect &R = *rp;
                R.id = nrect++;
                flat.push_back(&R);
                const size_t cells = (size_t)(R.n_x + 4) * (R.n_p + 4);
                R.xm.assign(R.n_p / r + 2, -1);
                R.xp.assign(R.n_p / r + 2, -1);
                R.pm.assign(R.n_x / r, -1);
                R.pp.assign(R.n_x / r, -1);
                R.sxm.assign(R.n_p / r + 2, 1);
                R.sxp.assign(R.n_p / r + 2, 1);
                R.spm.assign(R.n_x / r, 1);
                R.spp.assign(R.n_x / r, 1);
                R.finer.assign(cells, -1);
                R.finer_x.assign(cells, -1);
                R.finer_p.assign(cells, -1);
                R.nested.assign(cells, 0);
                R.ifx.assign(cells, 0);
                R.ifp.assign(cells, 0);
            }
    multi_patch = nrect > (int)rects.size();
    lap("cell arrays");
    // Mesh::promoteHierarchyToMesh (Mesh.cpp:839-859): finer links first, then same level.
    for (auto &sp : rects) {
        for (int l = 0; l < L; l++)
            for (auto &rl : sp[l])
                if (l > 0)
                    for (auto &rf : sp[l - 1]) conn_from_finer(*rl, *rf, r);
        for (int l = 0; l < L; l++)
            for (auto &rl : sp[l])
                for (auto &rr : sp[l])
                    if (rl != rr) conn_same(*rl, *rr, r);
    }

    lap("links");
    // ------------------------------------------------------------ ghost fills
    ghost_ops.clear();
    PlaneScheduler gs(flat);
    auto emit = [&](const GhostOp &op) {
        int reads[64][3], writes[1][3] = {{op.dst, op.di, op.dj}};  // r <= 8: at most 64 reads
        int nr = 0;
        if (op.kind == kGhostCopy) {
            reads[nr][0] = op.src, reads[nr][1] = op.si, reads[nr][2] = op.sj, nr++;
        } else if (op.kind == kGhostRestrict) {
            for (int a = 0; a < r; a++)
                for (int b = 0; b < r; b++) reads[nr][0] = op.src, reads[nr][1] = op.si + a, reads[nr][2] = op.sj + b, nr++;
        } else if (op.kind == kGhostInterp) {
            for (int a = -2; a <= 2; a++)
                for (int b = -2; b <= 2; b++) reads[nr][0] = op.src, reads[nr][1] = op.si + a, reads[nr][2] = op.sj + b, nr++;
        }
        gs.add(reads, nr, writes, 1);
        ghost_ops.push_back(op);
    };
    // value of global cell (gx, gp) of same-level patch `id` (BoundaryCondition: zero)
    auto copy_from = [&](int dst, int di, int dj, int id, int gx, int gp) {
        if (id < 0) emit({kGhostZero, dst, di, dj, -1, 0, 0, 0});
        else emit({kGhostCopy, dst, di, dj, id, gx - flat[id]->x_pos, gp - flat[id]->p_pos, 0});
    };
    // coarse interpolation (Rectangle::GetWenoValueFromCoarseLevel) of fine-global cell
    // (gi, gj) on coarse patch `id`; entry (kx, kp) of the r x r interpolants
    auto interp_from = [&](int dst, int di, int dj, int id, int gi, int gj, int kx, int kp) {
        const Rect &C = *flat[id];
        emit({kGhostInterp, dst, di, dj, id, gi / r - C.x_pos, gj / r - C.p_pos, kx * r + kp});
    };
    auto corners = [&](Rect &R) {  // Rectangle::UpdateCornerPoints (Rectangle.cpp:1130-1214)
        const int last = (int)R.xm.size() - 1;
        {   // below-left, i = -1
            const int i = -1;
            const int spt = R.xm[0];
            for (int j = r - 2; j < r; j++) {
                if (spt >= 0 && !R.sxm[0]) {
                    interp_from(R.id, -1, i * r + j, spt, R.x_pos - 1, R.p_pos + i * r, r - 1, j);
                    interp_from(R.id, -2, i * r + j, spt, R.x_pos - 1, R.p_pos + i * r, r - 2, j);
                } else {
                    copy_from(R.id, -1, i * r + j, spt, R.x_pos - 1, R.p_pos + i * r + j);
                    copy_from(R.id, -2, i * r + j, spt, R.x_pos - 2, R.p_pos + i * r + j);
                }
            }
        }
        {   // above-left, i = n_p / r
            const int i = last - 1;
            const int spt = R.xm[last];
            for (int j = 0; j < 2; j++) {
                if (spt >= 0 && !R.sxm[last]) {
                    interp_from(R.id, -1, i * r + j, spt, R.x_pos - 1, R.p_pos + i * r, r - 1, j);
                    interp_from(R.id, -2, i * r + j, spt, R.x_pos - 1, R.p_pos + i * r, r - 2, j);
                } else {
                    copy_from(R.id, -1, i * r + j, spt, R.x_pos - 1, R.p_pos + i * r + j);
                    copy_from(R.id, -2, i * r + j, spt, R.x_pos - 2, R.p_pos + i * r + j);
                }
            }
        }
        {   // below-right
            const int i = -1;
            const int spt = R.xp[0];
            for (int j = r - 2; j < r; j++) {
                if (spt >= 0 && !R.sxp[0]) {
                    interp_from(R.id, R.n_x, i * r + j, spt, R.x_pos + R.n_x, R.p_pos + i * r, 0, j);
                    interp_from(R.id, R.n_x + 1, i * r + j, spt, R.x_pos + R.n_x, R.p_pos + i * r, 1, j);
                } else {
                    copy_from(R.id, R.n_x, i * r + j, spt, R.x_pos + R.n_x, R.p_pos + i * r + j);
                    copy_from(R.id, R.n_x + 1, i * r + j, spt, R.x_pos + R.n_x + 1, R.p_pos + i * r + j);
                }
            }
        }
        {   // above-right
            const int i = last - 1;
            const int spt = R.xp[last];
            for (int j = 0; j < 2; j++) {
                if (spt >= 0 && !R.sxp[last]) {
                    interp_from(R.id, R.n_x, i * r + j, spt, R.x_pos + R.n_x, R.p_pos + i * r, 0, j);
                    interp_from(R.id, R.n_x + 1, i * r + j, spt, R.x_pos + R.n_x, R.p_pos + i * r, 1, j);
                } else {
                    copy_from(R.id, R.n_x, i * r + j, spt, R.x_pos + R.n_x, R.p_pos + i * r + j);
                    copy_from(R.id, R.n_x + 1, i * r + j, spt, R.x_pos + R.n_x + 1, R.p_pos + i * r + j);
                }
            }
        }
    };
    auto type0 = [&](std::vector<std::unique_ptr<Rect>> &lvl) {  // UpdateInterriorPoints
        for (auto &rp : lvl) {
            Rect &R = *rp;
            for (int i = 0; i < R.n_x; i++)
                for (int j = 0; j < R.n_p;) {
                    if (!R.nested[R.ns(i, j)]) {  // skip to the row's next nested cell
                        const uint8_t *row = &R.nested[R.ns(i, 0)];
                        const void *hit = std::memchr(row + j, 1, (size_t)(R.n_p - j));
                        if (!hit) break;
                        j = (int)((const uint8_t *)hit - row);
                    }
                    // a run of nested cells over the same finer patch, in the loop's order
                    const int fid = R.finer[R.ns(i, j)];
                    int j1 = j + 1;
                    while (j1 < R.n_p && R.nested[R.ns(i, j1)] && R.finer[R.ns(i, j1)] == fid) j1++;
                    const Rect &F = *flat[fid];
                    const int si = (R.x_pos + i) * r - F.x_pos;
                    gs.add_restrict_row(R.id, i, j, F.id, si, (R.p_pos + j) * r - F.p_pos, r, j1 - j);
                    for (int k = j; k < j1; k++)
                        ghost_ops.push_back({kGhostRestrict, R.id, i, k, F.id, si, (R.p_pos + k) * r - F.p_pos, 0});
                    j = j1;
                }
        }
    };
    auto type1 = [&](std::vector<std::unique_ptr<Rect>> &lvl) {  // UpdateSameLevelBoundaries
        for (auto &rp : lvl) {
            Rect &R = *rp;
            for (size_t e = 1; e + 1 < R.xm.size(); e++)
                if (R.sxm[e]) {
                    const int i = (int)e - 1;
                    for (int j = 0; j < r; j++) {
                        copy_from(R.id, -1, i * r + j, R.xm[e], R.x_pos - 1, R.p_pos + i * r + j);
                        copy_from(R.id, -2, i * r + j, R.xm[e], R.x_pos - 2, R.p_pos + i * r + j);
                    }
                }
            for (size_t e = 1; e + 1 < R.xp.size(); e++)
                if (R.sxp[e]) {
                    const int i = (int)e - 1;
                    for (int j = 0; j < r; j++) {
                        copy_from(R.id, R.n_x, i * r + j, R.xp[e], R.x_pos + R.n_x, R.p_pos + i * r + j);
                        copy_from(R.id, R.n_x + 1, i * r + j, R.xp[e], R.x_pos + R.n_x + 1, R.p_pos + i * r + j);
                    }
                }
            for (size_t e = 0; e < R.pm.size(); e++)
                if (R.spm[e]) {
                    const int i = (int)e;
                    for (int j = 0; j < r; j++) {
                        copy_from(R.id, i * r + j, -1, R.pm[e], R.x_pos + i * r + j, R.p_pos - 1);
                        copy_from(R.id, i * r + j, -2, R.pm[e], R.x_pos + i * r + j, R.p_pos - 2);
                    }
                }
            for (size_t e = 0; e < R.pp.size(); e++)
                if (R.spp[e]) {
                    const int i = (int)e;
                    for (int j = 0; j < r; j++) {
                        copy_from(R.id, i * r + j, R.n_p, R.pp[e], R.x_pos + i * r + j, R.p_pos + R.n_p);
                        copy_from(R.id, i * r + j, R.n_p + 1, R.pp[e], R.x_pos + i * r + j, R.p_pos + R.n_p + 1);
                    }
                }
        }
    };
    auto type2 = [&](std::vector<std::unique_ptr<Rect>> &lvl) {  // UpdateDifferentLevelBoundaries
        for (auto &rp : lvl) {
            Rect &R = *rp;
            for (size_t e = 1; e + 1 < R.xm.size(); e++)
                if (!R.sxm[e] && R.xm[e] >= 0) {
                    const int i = (int)e - 1;
                    for (int j = 0; j < r; j++) {
                        interp_from(R.id, -1, i * r + j, R.xm[e], R.x_pos - 1, R.p_pos + i * r, r - 1, j);
                        interp_from(R.id, -2, i * r + j, R.xm[e], R.x_pos - 1, R.p_pos + i * r, r - 2, j);
                    }
                }
            for (size_t e = 1; e + 1 < R.xp.size(); e++)
                if (!R.sxp[e] && R.xp[e] >= 0) {
                    const int i = (int)e - 1;
                    for (int j = 0; j < r; j++) {
                        interp_from(R.id, R.n_x, i * r + j, R.xp[e], R.x_pos + R.n_x, R.p_pos + i * r, 0, j);
                        interp_from(R.id, R.n_x + 1, i * r + j, R.xp[e], R.x_pos + R.n_x, R.p_pos + i * r, 1, j);
                    }
                }
            for (size_t e = 0; e < R.pm.size(); e++)
                if (!R.spm[e] && R.pm[e] >= 0) {
                    const int i = (int)e;
                    for (int j = 0; j < r; j++) {
                        interp_from(R.id, i * r + j, -1, R.pm[e], R.x_pos + i * r, R.p_pos - 1, j, r - 1);
                        interp_from(R.id, i * r + j, -2, R.pm[e], R.x_pos + i * r, R.p_pos - 1, j, r - 2);
                    }
                }
            for (size_t e = 0; e < R.pp.size(); e++)
                if (!R.spp[e] && R.pp[e] >= 0) {
                    const int i = (int)e;
                    for (int j = 0; j < r; j++) {
                        interp_from(R.id, i * r + j, R.n_p, R.pp[e], R.x_pos + i * r, R.p_pos + R.n_p, j, 0);
                        interp_from(R.id, i * r + j, R.n_p + 1, R.pp[e], R.x_pos + i * r, R.p_pos + R.n_p, j, 1);
                    }
                }
            corners(R);
        }
    };
    // Mesh::PushData (Mesh.cpp:91-106) for every species
    for (auto &sp : rects) {
        type1(sp[0]);
        for (int i = 1; i < L; i++) {
            type0(sp[i]);
            type1(sp[i]);
        }
        for (auto &rp : sp[L - 1]) corners(*rp);
        for (int i = L - 1; i > 0; i--) type2(sp[i - 1]);
    }
    sort_by_batch(ghost_ops, gs.batch, gs.nbatches, ghost_b);
    lap("ghost ops");

    // ------------------------------------------------------------ interface fluxes
    iface_ops.clear();
    std::vector<int> ib;
    int inb = 0;
    for (auto &sp : rects)
        for (int l = 1; l < L; l++)
            for (auto &rp : sp[l]) {
                Rect &R = *rp;
                for (int i = -2; i < R.n_x + 2; i++)
                    for (int j = -2; j < R.n_p + 2; j++) {
                        if (R.ifx[R.ns(i, j)]) {
                            const Rect &F = *flat[R.finer_x[R.ns(i, j)]];
                            iface_ops.push_back({0, R.id, i, j, F.id, (R.x_pos + i) * r - F.x_pos, (R.p_pos + j) * r - F.p_pos});
                            ib.push_back(l - 1);
                        }
                        if (R.ifp[R.ns(i, j)]) {
                            const Rect &F = *flat[R.finer_p[R.ns(i, j)]];
                            iface_ops.push_back({1, R.id, i, j, F.id, (R.x_pos + i) * r - F.x_pos, (R.p_pos + j) * r - F.p_pos});
                            ib.push_back(l - 1);
                        }
                        inb = std::max(inb, l);
                    }
            }
    sort_by_batch(iface_ops, ib, inb, iface_b);
    lap("iface ops");

    // ------------------------------------------------------------ limiter C exchange
    csync_ops.clear();
    // the Cx and Cp planes of every patch as 2 x flat scheduler planes (Cp of patch k at k + nflat)
    std::vector<Rect *> cplanes(flat);
    cplanes.insert(cplanes.end(), flat.begin(), flat.end());
    const int nflat = (int)flat.size();
    PlaneScheduler cs(cplanes);
    auto emit_c = [&](const CSyncOp &op) {
        const int off = op.t < 2 ? 0 : nflat;
        int reads[2][3], writes[2 + kMaxRatio][3];
        int nr = 0, nw = 0;
        auto cell = [&](int (*a)[3], int &n, int patch, int i, int j) {
            a[n][0] = patch + off, a[n][1] = i, a[n][2] = j, n++;
        };
        if (op.kind == kCSame) {
            cell(writes, nw, op.nb, op.ni, op.nj);
            cell(writes, nw, op.caller, op.ci, op.cj);
        } else if (op.kind == kCUpdate) {
            cell(reads, nr, op.nb, op.ni, op.nj);
            cell(reads, nr, op.caller, op.ci, op.cj);
            cell(writes, nw, op.nb, op.ni, op.nj);
            cell(writes, nw, op.caller, op.ci, op.cj);
        } else {
            cell(reads, nr, op.nb, op.ni, op.nj);
            cell(writes, nw, op.nb, op.ni, op.nj);
            for (int k = 0; k < r; k++) {
                if (off == 0) cell(writes, nw, op.caller, op.ci, op.cj + k);
                else cell(writes, nw, op.caller, op.ci + k, op.cj);
            }
        }
        cs.add(reads, nr, writes, nw);
        csync_ops.push_back(op);
    };
    // same-level exchange on every face of every patch edge; the domain boundary's
    // BoundaryCondition object has a zero refinement ratio, so its calls do nothing
    auto same_calls = [&](Rect &R, int kind) {
        auto one = [&](int nbid, int gi, int gj, int t) {
            if (nbid < 0) return;
            const Rect &N = *flat[nbid];
            for (int k = 0; k < r; k++) {
                const int dk = t < 2 ? 0 : k, pk = t < 2 ? k : 0;
                emit_c({kind, t, nbid, gi - N.x_pos + dk, gj - N.p_pos + pk, R.id, gi - R.x_pos + dk, gj - R.p_pos + pk});
            }
        };
        for (size_t e = 1; e + 1 < R.xm.size(); e++)
            if (R.sxm[e]) one(R.xm[e], R.x_pos, R.p_pos + ((int)e - 1) * r, 0);
        for (size_t e = 1; e + 1 < R.xp.size(); e++)
            if (R.sxp[e]) one(R.xp[e], R.x_pos + R.n_x, R.p_pos + ((int)e - 1) * r, 1);
        for (size_t e = 0; e < R.pm.size(); e++)
            if (R.spm[e]) one(R.pm[e], R.x_pos + (int)e * r, R.p_pos, 2);
        for (size_t e = 0; e < R.pp.size(); e++)
            if (R.spp[e]) one(R.pp[e], R.x_pos + (int)e * r, R.p_pos + R.n_p, 3);
    };
    auto diff_calls = [&](Rect &R) {
        auto one = [&](int nbid, int gi, int gj, int t) {
            const Rect &C = *flat[nbid];
            emit_c({kCDiff, t, nbid, gi / r - C.x_pos, gj / r - C.p_pos, R.id, gi - R.x_pos, gj - R.p_pos});
        };
        for (size_t e = 1; e + 1 < R.xm.size(); e++)
            if (!R.sxm[e] && R.xm[e] >= 0) one(R.xm[e], R.x_pos, R.p_pos + r * ((int)e - 1), 0);
        for (size_t e = 1; e + 1 < R.xp.size(); e++)
            if (!R.sxp[e] && R.xp[e] >= 0) one(R.xp[e], R.x_pos + R.n_x, R.p_pos + r * ((int)e - 1), 1);
        for (size_t e = 0; e < R.pm.size(); e++)
            if (!R.spm[e] && R.pm[e] >= 0) one(R.pm[e], R.x_pos + r * (int)e, R.p_pos, 2);
        for (size_t e = 0; e < R.pp.size(); e++)
            if (!R.spp[e] && R.pp[e] >= 0) one(R.pp[e], R.x_pos + r * (int)e, R.p_pos + R.n_p, 3);
    };
    for (auto &sp : rects) {
        for (int l = 0; l < L; l++)
            for (auto &rp : sp[l]) same_calls(*rp, kCSame);
        for (int l = 0; l < L; l++)
            for (auto &rp : sp[l]) diff_calls(*rp);
        for (int l = 0; l < L; l++)
            for (auto &rp : sp[l]) same_calls(*rp, kCUpdate);
    }
    sort_by_batch(csync_ops, cs.batch, cs.nbatches, csync_b);
    lap("csync ops");
    validate_ops();
    lap("validate");
    dghost_ops = upload(ghost_ops, eng->stream);
    diface_ops = upload(iface_ops, eng->stream);
    dcsync_ops = upload(csync_ops, eng->stream);
    lap("op upload");

    // ------------------------------------------------------------ device masks, weights
    for (Rect *R : flat) {
        const size_t pe = R->plane_elems();
        std::vector<uint8_t> m(3 * pe, 0);
        // rows of (n_p + 4) cells in the reference's index order become pitched rows
        const size_t w = (size_t)R->n_p + 4;
        for (int i = -2; i < R->n_x + 2; i++) {
            const size_t d = (size_t)pidx(i, -2, R->pitch), q = (size_t)R->ns(i, -2);
            std::memcpy(&m[d], &R->nested[q], w);
            std::memcpy(&m[pe + d], &R->ifx[q], w);
            std::memcpy(&m[2 * pe + d], &R->ifp[q], w);
        }
        R->masks = DevBuf(m.size(), DevBuf::Uninit{});  // the blocking copy below fills it
        VX_CUDA(cudaMemcpy(R->masks.p, m.data(), m.size(), cudaMemcpyHostToDevice));
    }
    lap("masks");
    std::vector<double> w;
    relc_off.assign(L, 0);
    for (int d = 0; d < L; d++) {
        relc_off[d] = (int)w.size();
        const int rtb = (int)std::pow(r, d);
        const double rb = std::pow(r, d);
        for (int i = 0; i < rtb; i++) {  // Rectangle.cpp:103-110
            double tl = -0.5 + i / rb;
            double tr = -0.5 + (i + 1.0) / rb;
            w.push_back((tl + tr) * 0.5);
            w.push_back((tl * tl + tl * tr + tr * tr) / 3.0 - (1.0 / 12));
            w.push_back((tl * tl * tl + tl * tl * tr + tl * tr * tr + tr * tr * tr) * 0.25);
        }
    }
    drelc = DevBuf(w.size() * sizeof(double));
    VX_CUDA(cudaMemcpy(drelc.p, w.data(), w.size() * sizeof(double), cudaMemcpyHostToDevice));
    std::vector<float> w32;
    relc32_off.assign(L, 0);
    for (int d = 0; d < L; d++) {
        relc32_off[d] = (int)w32.size();
        const int rtb = (int)std::pow(r, d);
        double sum[3] = {0, 0, 0};
        for (int q = 0; q < 3 * rtb; q++) {
            w32.push_back((float)w[relc_off[d] + q]);
            sum[q % 3] += w[relc_off[d] + q];
        }
        for (double v : sum) w32.push_back((float)v);
    }
    drelc32 = DevBuf(w32.size() * sizeof(float));
    VX_CUDA(cudaMemcpy(drelc32.p, w32.data(), w32.size() * sizeof(float), cudaMemcpyHostToDevice));
}

}  // namespace vx
