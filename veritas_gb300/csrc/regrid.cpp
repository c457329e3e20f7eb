// Hierarchy construction and regridding (Mesh::Mesh, Mesh::updateHierarchy and
// Mesh::promoteHierarchyToMesh, Mesh.cpp:8-50, 132-208, 792-880).
//
// The error flags are computed on the device (one launch over every patch); the
// clustering of flagged cells into rectangles is integer work on the host, restating the
// reference's signature / inflection splitter step for step so that the same rectangles
// come out; the data transfer from the old hierarchy and the ghost fills run on the
// device as region ops in the reference's call order.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <functional>
#include <iterator>
#include <tuple>

#include <chrono>
#include <cstdio>
#include <cstdlib>

#include "engine.hpp"

namespace vx {

namespace {

using Coord = std::pair<int, int>;
using Box = std::pair<Coord, Coord>;  // ((x0, p0), (x1, p1)); inclusive while clustering
using Boxes = std::vector<Box>;

int sgn(int x) { return (x > 0) ? 1 : ((x < 0) ? -1 : 0); }

// Mesh::countCells (Mesh.cpp:367-370)
int count_cells(const Box &b) { return (b.second.first - b.first.first + 1) * (b.second.second - b.first.second + 1); }

struct Signatures {
    std::vector<int> sx, dsx, sp, dsp;
};

// Mesh::computeSignatures (Mesh.cpp:388-447): flagged counts per column / row of the
// box and their discrete Laplacians (only for extents of at least 2).
Signatures signatures(const Box &b, const std::vector<Coord> &flagged) {
    Signatures s;
    const int lx = b.second.first - b.first.first, lp = b.second.second - b.first.second;
    s.sx.assign(lx + 1, 0);
    s.sp.assign(lp + 1, 0);
    for (const Coord &c : flagged) {
        s.sx.at(c.first - b.first.first)++;
        s.sp.at(c.second - b.first.second)++;
    }
    auto lap = [](const std::vector<int> &v, std::vector<int> &out) {
        out.resize(v.size() - 2);
        for (size_t h = 1; h + 1 < v.size(); h++) out[h - 1] = v[h - 1] + v[h + 1] - 2 * v[h];
    };
    if (lx >= 2) lap(s.sx, s.dsx);
    if (lp >= 2) lap(s.sp, s.dsp);
    return s;
}

// One direction of Mesh::identifyInflection (Mesh.cpp:449-580): sign changes of the
// Laplacian between non-zero neighbours; a single one is taken, several resolve to the
// largest jump or, when the largest jump is tied, to the change nearest the middle.
struct Inflection {
    int index = 0, size = 0;
    bool bisect = false;
};

Inflection inflection(const std::vector<int> &d, int range0) {
    Inflection r;
    const int n = (int)d.size();
    if (n <= 2) return r;
    std::vector<int> idx, mag;
    for (int i = 0; i + 1 < n; i++)
        if (d[i] != 0 && d[i + 1] != 0 && sgn(d[i]) != sgn(d[i + 1])) {
            idx.push_back(i);
            mag.push_back(std::abs(d[i + 1] - d[i]));
        }
    if (idx.empty()) {
        r.bisect = true;
        return r;
    }
    if (idx.size() == 1) {
        r.index = idx[0];
        r.size = mag[0];
        return r;
    }
    const auto big = std::max_element(mag.begin(), mag.end());
    const int ties = (int)std::count(mag.begin(), mag.end(), *big);
    int chosen = (int)(big - mag.begin());
    if (ties > 1) {
        const int centre = n / 2;
        int best = range0;
        chosen = 0;
        for (size_t i = 0; i < idx.size(); i++)
            if (best > std::abs(idx[i] - centre)) {
                best = std::abs(idx[i] - centre);
                chosen = (int)i;
            }
    }
    r.index = idx[chosen];
    r.size = mag[chosen];
    return r;
}

// Mesh::hasHole (Mesh.cpp:582-611): the first run of empty columns, as the last
// non-empty index before it and the first non-empty index after it.
std::tuple<bool, int, int> find_hole(const std::vector<int> &sig) {
    auto it = std::find(sig.begin(), sig.end(), 0);
    if (it == sig.end()) return std::make_tuple(false, 0, 0);
    const int start = (it == sig.begin()) ? 0 : (int)(it - sig.begin()) - 1;
    auto it2 = std::find_if(it, sig.end(), [](int v) { return v != 0; });
    const int finish = (it2 == sig.end()) ? (int)(it2 - sig.begin()) - 1 : (int)(it2 - sig.begin());
    return std::make_tuple(true, start, finish);
}

// Mesh::splitRectangle (Mesh.cpp:630-790).
Boxes split(const Box &b, const std::vector<Coord> &flagged, double min_eff) {
    const double eff = flagged.size() / double(count_cells(b));
    if (eff > min_eff) return {b};
    Signatures s = signatures(b, flagged);
    bool hx, hp;
    int sx0, sx1, sp0, sp1;
    std::tie(hx, sx0, sx1) = find_hole(s.sx);
    std::tie(hp, sp0, sp1) = find_hole(s.sp);
    sx0 += b.first.first;
    sx1 += b.first.first;
    sp0 += b.first.second;
    sp1 += b.first.second;
    Box one, two;
    auto cut_x = [&](int end_one, int start_two) {
        one = Box(b.first, Coord(end_one, b.second.second));
        two = Box(Coord(start_two, b.first.second), b.second);
    };
    auto cut_p = [&](int end_one, int start_two) {
        one = Box(b.first, Coord(b.second.first, end_one));
        two = Box(Coord(b.first.first, start_two), b.second);
    };
    if (hx && hp) {
        if (std::abs(sx1 - sx0) > std::abs(sp1 - sp0)) cut_x(sx0, sx1);
        else cut_p(sp0, sp1);
    } else if (hx) {
        cut_x(sx0, sx1);
    } else if (hp) {
        cut_p(sp0, sp1);
    } else {
        Inflection ix = inflection(s.dsx, INT_MAX);
        Inflection ip = inflection(s.dsp, 32767);
        const int nx = (int)s.dsx.size(), np = (int)s.dsp.size();
        if (ix.bisect && ip.bisect) {
            const double lx = b.second.first - b.first.first, lp = b.second.second - b.first.second;
            if (lx > lp) {
                const int c = (int)std::floor((lx / 2) + b.first.first);
                cut_x(c, c + 1);
            } else {
                const int c = (int)std::floor((lp / 2) + b.first.second);
                cut_p(c, c + 1);
            }
        } else if ((nx <= 2 && np <= 2) || (ix.size == 0 && ip.size == 0)) {
            return {b};
        } else if (ix.size > ip.size) {
            const int c = ix.index + b.first.first + 1;
            cut_x(c, c + 1);
        } else {
            const int c = ip.index + b.first.second + 1;
            cut_p(c, c + 1);
        }
    }
    std::vector<Coord> f1, f2;
    for (const Coord &c : flagged) {
        const bool in = c.first >= one.first.first && c.first <= one.second.first && c.second >= one.first.second &&
                        c.second <= one.second.second;
        (in ? f1 : f2).push_back(c);
    }
    Boxes out;
    if (!f1.empty()) out = split(one, f1, min_eff);
    if (!f2.empty()) {
        Boxes o2 = split(two, f2, min_eff);
        out.insert(out.end(), o2.begin(), o2.end());
    }
    return out;
}

// Mesh::getExtrema (Mesh.cpp:613-628)
Box extrema(const std::vector<Coord> &flagged) {
    int x0 = INT_MAX, x1 = INT_MIN, p0 = INT_MAX, p1 = INT_MIN;
    for (const Coord &c : flagged) {
        x0 = std::min(x0, c.first);
        x1 = std::max(x1, c.first);
        p0 = std::min(p0, c.second);
        p1 = std::max(p1, c.second);
    }
    return Box(Coord(x0, p0), Coord(x1, p1));
}

}  // namespace

// Mesh::interpRectanglesUp (Mesh.cpp:297-312): inclusive level-l boxes to half-open
// boxes in level l+1 cells.
static void boxes_up(const Settings &s, Boxes &bs, int l, int sp) {
    const int nmax = s.GetXSize(s.maxDepth - l), pmax = s.GetPSize(s.maxDepth - l, sp);
    const int nmax1 = s.GetXSize(s.maxDepth - (l + 1)), pmax1 = s.GetPSize(s.maxDepth - (l + 1), sp);
    for (Box &b : bs) {
        b.second.first += 1;
        b.second.second += 1;
        b.first.first = (int)(b.first.first * (nmax1 / double(nmax)));
        b.first.second = (int)(b.first.second * (pmax1 / double(pmax)));
        b.second.first = (int)(b.second.first * (nmax1 / double(nmax)));
        b.second.second = (int)(b.second.second * (pmax1 / double(pmax)));
    }
}

// Mesh::mergeDownFlaggedData (Mesh.cpp:314-340): level-l cells under (and around) a
// level l+2 box, sorted and unique.
static std::vector<Coord> merge_down(const Settings &s, int l, const Box &b, int sp) {
    const int R = (int)s.refinementRatio;
    const int nmax = s.GetXSize(s.maxDepth - l), pmax = s.GetPSize(s.maxDepth - l, sp);
    const int nmax2 = s.GetXSize(s.maxDepth - (l + 2)), pmax2 = s.GetPSize(s.maxDepth - (l + 2), sp);
    std::vector<Coord> out;
    for (int i = b.first.first - 2 * R; i <= b.second.first + 2 * R + 1; i++)
        for (int j = b.first.second - 2 * R; j <= b.second.second + 2 * R; j++) {
            const int ic = (int)(i * (nmax / double(nmax2)));
            const int jc = (int)(j * (pmax / double(pmax2)));
            if (ic > -1 && ic < nmax && jc > -1 && jc < pmax) out.push_back(Coord(ic, jc));
        }
    std::sort(out.begin(), out.end());
    out.erase(std::unique(out.begin(), out.end()), out.end());
    return out;
}

// Rectangle error weights (Rectangle.cpp:68-74).
void error_weights(const Settings &s, int depth, int sp, double *w) {
    const int r = (int)s.refinementRatio;
    const double fm = s.GetfMax(sp);
    w[0] = 0.5 / fm * std::pow(r, -0.5 * depth);
    w[1] = 0.5 / fm * std::pow(r, -0.5 * depth);
    w[2] = 0.5 / fm * std::pow(r, -2.0 * depth);
    w[3] = 0.5 / fm * std::pow(r, -2.0 * depth);
    w[4] = s.sizeWeight / fm * std::pow(r, -s.maxDepth + depth);
}

// Flagged cells of every patch (Rectangle::getError, Rectangle.cpp:866-890), computed in
// one launch; per patch, the cells in the reference's loop order.
std::vector<std::vector<std::pair<int, int>>> Run::flag_cells() {
    const Settings &s = *S;
    std::vector<FlagPatch> fp;
    size_t total = 0;
    for (Rect *R : flat) {
        FlagPatch f{};
        f.patch = (int)fp.size();
        int offset = 0;
        for (int i = 0; i <= s.maxDepth - R->depth; i++) offset += (int)std::pow(s.refinementRatio, i);
        offset *= 3;
        f.i0 = std::max(R->x_pos, offset) - R->x_pos;
        f.i1 = std::min(R->x_pos + R->n_x, s.GetXSize(R->depth) - offset) - R->x_pos;
        f.j0 = std::max(R->p_pos, offset) - R->p_pos;
        f.j1 = std::min(R->p_pos + R->n_p, s.GetPSize(R->depth, R->species) - offset) - R->p_pos;
        f.out_off = (long long)total;
        error_weights(s, R->depth, R->species, f.w);
        // FP32 form: f is stored times fnorm, so the weights (which carry 1/fMax) are
        // divided by it and the criterion stays as it is
        for (double &wq : f.w) wq /= fnorm[R->species];
        f.crit = s.refinementCriteria;
        total += (size_t)R->n_x * R->n_p;
        fp.push_back(f);
    }
    std::vector<uint8_t> flags(total, 0);
    if (total) {
        std::vector<PatchT<double>> descs;
        for (Rect *R : flat) descs.push_back(R->desc);
        DevBuf dd = upload(descs, eng->stream);
        DevBuf dfp = upload(fp, eng->stream);
        DevBuf dout(total);
        launch_flags(dd.p, dfp.as<FlagPatch>(), (int)fp.size(), dout.as<uint8_t>(), precision, eng->stream);
        VX_CUDA(cudaMemcpyAsync(flags.data(), dout.p, total, cudaMemcpyDeviceToHost, eng->stream));
        eng->sync();
    }
    std::vector<std::vector<std::pair<int, int>>> out(flat.size());
    for (size_t k = 0; k < flat.size(); k++) {
        const Rect &R = *flat[k];
        const FlagPatch &f = fp[k];
        const uint8_t *fl = flags.data() + f.out_off;
        const double dx = s.GetDx(R.depth), dp = s.GetDp(R.depth, R.species);
        const bool hook = s.problem->HasRefinementOverride();
        for (int i = f.i0; i < f.i1; i++)
            for (int j = f.j0; j < f.j1; j++) {
                bool flag = fl[(size_t)i * R.n_p + j] != 0;
                if (!flag && hook)
                    flag = s.RefinementOverride((i + R.x_pos + 0.5) * dx, s.pmin[R.species] + dp * (j + R.p_pos),
                                                R.depth, R.species);
                if (flag) out[k].push_back({i + R.x_pos, j + R.p_pos});
            }
    }
    return out;
}

// Mesh::updateHierarchy (Mesh.cpp:132-208) without its final promotion: `H` is the
// current hierarchy of one species (entry k: the boxes of depth maxDepth - k, half-open,
// from the base level up to the first empty level) and level_flags(l) returns the
// flagged cells of hierarchy level l in the reference's order.  Host only.
std::vector<Run::BoxList> update_hierarchy(const Settings &s, int sp, std::vector<Run::BoxList> H,
                                           const std::function<std::vector<std::pair<int, int>>(int)> &level_flags) {
    const int lloop = (int)H.size() - 1;
    for (int l = lloop; l > -1; l--) {
        std::vector<Coord> flagged;
        if (l < (int)H.size() - 2) {
            std::vector<Coord> l1 = level_flags(l), l2;
            if (H.size() > 2)
                for (const Box &b : H.at(l + 2)) {
                    auto m = merge_down(s, l, b, sp);
                    l2.insert(l2.end(), m.begin(), m.end());
                }
            // the l+2 lists are concatenated unsorted, as the reference does before its
            // set_union; the same library call gives the same cells
            std::sort(l1.begin(), l1.end());
            std::set_union(l1.begin(), l1.end(), l2.begin(), l2.end(), std::back_inserter(flagged));
        } else {
            flagged = level_flags(l);
        }
        if (!flagged.empty()) {
            Boxes found = split(extrema(flagged), flagged, s.minEfficiency);
            boxes_up(s, found, l, sp);
            if (l == lloop) {
                if (l < s.maxDepth) H.push_back(found);
            } else {
                H.at(l + 1) = found;
            }
        } else if (l < lloop) {
            H.erase(H.begin() + l + 1);
        }
    }
    return H;
}

// Patch geometry of a hierarchy as Mesh::promoteHierarchyToMesh (Mesh.cpp:792-826)
// creates it, in level order (depth ascending).  The boundary flags compare with the
// size of level N - lvl, not of the box's own level, exactly as the reference does, so
// a hierarchy with fewer than maxDepth + 1 levels gets open upper/right edges.
std::vector<PatchGeom> promote_geometry(const Settings &s, int sp, const std::vector<Run::BoxList> &H) {
    const int N = (int)H.size() - 1;
    const int empty = s.maxDepth - N;
    std::vector<PatchGeom> out;
    for (int lvl = N; lvl >= 0; lvl--) {
        const int xmax = s.GetXSize(N - lvl), pmax = s.GetPSize(N - lvl, sp);
        for (const auto &b : H.at(lvl)) {
            PatchGeom g;
            g.depth = N - lvl + empty;
            g.x_pos = b.first.first;
            g.p_pos = b.first.second;
            g.n_x = b.second.first - b.first.first;
            g.n_p = b.second.second - b.first.second;
            g.up = b.second.second == pmax;
            g.down = b.first.second == 0;
            g.left = b.first.first == 0;
            g.right = b.second.first == xmax;
            out.push_back(g);
        }
    }
    return out;
}

std::vector<Run::BoxList> Run::hierarchy_of(int sp) const {
    std::vector<BoxList> H;
    for (int d = S->maxDepth; d >= 0; d--) {
        if (rects[sp][d].empty()) break;
        BoxList b;
        for (auto &r : rects[sp][d]) b.push_back(Box(Coord(r->x_pos, r->p_pos), Coord(r->x_pos + r->n_x, r->p_pos + r->n_p)));
        H.push_back(b);
    }
    return H;
}

// SolverManager::reGrid / Mesh::updateHierarchy for every species, then the promotion.
void Run::regrid(bool init) {
    const Settings &s = *S;
    if (s.maxDepth == 0) return;
    static const bool trace = std::getenv("VX_TRACE_INIT") != nullptr;
    auto t0 = std::chrono::steady_clock::now();
    auto lap = [&](const char *what) {
        if (!trace) return;
        auto t1 = std::chrono::steady_clock::now();
        std::fprintf(stderr, "vx regrid %-12s %8.2f ms\n", what, std::chrono::duration<double, std::milli>(t1 - t0).count());
        t0 = t1;
    };
    auto flags = flag_cells();
    lap("flags");
    std::vector<std::vector<BoxList>> hier(rects.size());
    for (size_t sp = 0; sp < rects.size(); sp++) {
        auto level_flags = [&](int l) {  // Mesh::getError(l, false)
            std::vector<Coord> out;
            for (auto &r : rects[sp][s.maxDepth - l]) {
                const auto &f = flags[r->id];
                out.insert(out.end(), f.begin(), f.end());
            }
            return out;
        };
        hier[sp] = update_hierarchy(s, (int)sp, hierarchy_of((int)sp), level_flags);
    }
    lap("clustering");
    bool kept = !init;
    for (size_t sp = 0; kept && sp < rects.size(); sp++) kept = hier[sp] == hierarchy_of((int)sp);
    if (kept) {
        // The clustering returned the current boxes in the current order: the promotion
        // would build the same patches (fresh storage, all zero), the same tables, copy
        // every f1 value across unchanged, refill the slot-1 ghosts and set f0 = f1.  Its
        // result, in place: every plane but f0 and f1 (and the moment columns) zeroed, the
        // ghosts refilled from the same values, f0 = f1.  The layout version stays, so the
        // launch sets and graphs that hold this run stay valid.
        for (Rect *R : flat) {
            const size_t keep = 2 * R->plane_bytes();  // f0 and f1 lead the slab
            VX_CUDA(cudaMemsetAsync(R->slab.as<char>() + keep, 0, R->slab.bytes - keep, eng->stream));
            VX_CUDA(cudaMemsetAsync(R->cols.p, 0, R->cols.bytes, eng->stream));
        }
        push_data(1);
        copy_slot(1, 0);
        lap("kept layout");
        return;
    }
    promote(hier, init);
    lap("promote");
}

// Mesh::promoteHierarchyToMesh (Mesh.cpp:792-880) for all species at once (the species
// are independent): new patches, f from the quadrature (init) or from the old
// hierarchy (Mesh::InterMeshDataTransfer, Mesh.cpp:116-130), connectivity, ghost fill
// and f0 = f1.
void Run::promote(const std::vector<std::vector<BoxList>> &hier, bool init) {
    const Settings &s = *S;
    static const bool trace = std::getenv("VX_TRACE_INIT") != nullptr;
    auto t0 = std::chrono::steady_clock::now();
    auto lap = [&](const char *what) {
        if (!trace) return;
        eng->sync();
        auto t1 = std::chrono::steady_clock::now();
        std::fprintf(stderr, "vx promote %-11s %8.2f ms\n", what, std::chrono::duration<double, std::milli>(t1 - t0).count());
        t0 = t1;
    };
    auto old = std::move(rects);
    rects.clear();
    rects.resize(old.size());
    for (size_t sp = 0; sp < old.size(); sp++) {
        rects[sp].resize(s.maxDepth + 1);
        for (const PatchGeom &g : promote_geometry(s, (int)sp, hier[sp])) {
            auto r = std::make_unique<Rect>();
            r->n_x = g.n_x;
            r->n_p = g.n_p;
            r->x_pos = g.x_pos;
            r->p_pos = g.p_pos;
            r->depth = g.depth;
            r->up = g.up;
            r->down = g.down;
            r->left = g.left;
            r->right = g.right;
            r->species = (int)sp;
            if (r->n_x <= 0 || r->n_p <= 0) throw std::runtime_error("regrid produced an empty patch");
            if (r->n_x % (int)s.refinementRatio || r->n_p % (int)s.refinementRatio)
                throw std::runtime_error("regrid produced a patch not divisible by the refinement ratio");
            allocate_rect(*r);
            rects[sp][g.depth].push_back(std::move(r));
        }
    }
    lap("allocate");
    build_amr();
    lap("connectivity");
    for (Rect *R : flat) upload_rect_desc(*R, 0);
    if (init) {
        for (Rect *R : flat) init_rect_distribution(*R);
    } else {
        transfer_from(old);
    }
    lap(init ? "quadrature" : "transfer");
    push_data(1);
    copy_slot(1, 0);
    lap("ghosts");
    layout_version++;
}

// Mesh::InterMeshDataTransfer (Mesh.cpp:116-130) with Rectangle::GetDataFromCoarseLevel-
// Rectangle, GetDataFromSameLevelRectangle and GetDataFromCoarseNewLevelRectangle
// (Rectangle.cpp:892-1128) as region ops; one launch per call of the level loop.
void Run::transfer_from(std::vector<std::vector<std::vector<std::unique_ptr<Rect>>>> &old) {
    const Settings &s = *S;
    const int r = (int)s.refinementRatio;
    const int L = s.maxDepth + 1;
    // descriptor table: new patches (flat order) then old patches
    std::vector<PatchT<double>> descs;
    for (Rect *R : flat) descs.push_back(R->desc);
    std::vector<Rect *> oflat;
    for (auto &sp : old)
        for (auto &lvl : sp)
            for (auto &rp : lvl) {
                upload_rect_desc(*rp, 0);
                descs.push_back(rp->desc);
                oflat.push_back(rp.get());
            }
    const int nnew = (int)flat.size();
    auto old_id = [&](const Rect *R) { return nnew + (int)(std::find(oflat.begin(), oflat.end(), R) - oflat.begin()); };
    // is_interpolated masks of the new patches
    std::vector<long long> moff;
    long long mtotal = 0;
    for (Rect *R : flat) {
        moff.push_back(mtotal);
        mtotal += (long long)(R->n_x + 4) * (R->n_p + 4);
    }
    DevBuf dmask((size_t)std::max<long long>(mtotal, 1));
    VX_CUDA(cudaMemsetAsync(dmask.p, 0, dmask.bytes, eng->stream));
    DevBuf dd = upload(descs, eng->stream);

    auto bounds = [&](const Rect &R, int i, int j) { return i >= -2 && i < R.n_x + 2 && j >= -2 && j < R.n_p + 2; };
    auto need = [](bool ok) {
        if (!ok) throw std::invalid_argument("AMR transfer: region outside its patch");
    };
    // old coarse `C` (this) into new fine `F` (rectangle): Rectangle.cpp:892-916 / 1100-1128
    auto interp_op = [&](std::vector<XferOp> &ops, int kind, const Rect &C, int cid, const Rect &F, int fid) {
        const int x2 = F.x_pos / r, p2 = F.p_pos / r, nx2 = F.n_x / r, np2 = F.n_p / r;
        XferOp op{};
        op.kind = kind;
        op.dst = fid;
        op.src = cid;
        op.i0 = std::max(C.x_pos, x2 - 1);
        op.i1 = std::min(C.x_pos + C.n_x, x2 + nx2 + 1);
        op.j0 = std::max(C.p_pos, p2 - 1);
        op.j1 = std::min(C.p_pos + C.n_p, p2 + np2 + 1);
        op.x2 = x2;
        op.p2 = p2;
        op.mask_off = moff[F.id];
        if (op.i0 >= op.i1 || op.j0 >= op.j1) return;
        need(bounds(F, (op.i0 - x2) * r, (op.j0 - p2) * r) && bounds(F, (op.i1 - 1 - x2) * r + r - 1, (op.j1 - 1 - p2) * r + r - 1));
        need(bounds(C, op.i0 - C.x_pos - 2, op.j0 - C.p_pos - 2) && bounds(C, op.i1 - 1 - C.x_pos + 2, op.j1 - 1 - C.p_pos + 2));
        ops.push_back(op);
    };
    // old same-level `O` (this) into new `F` (rectangle): Rectangle.cpp:918-941
    auto copy_op = [&](std::vector<XferOp> &ops, const Rect &O, int oid, const Rect &F, int fid) {
        XferOp op{};
        op.kind = kXferCopy;
        op.dst = fid;
        op.src = oid;
        op.i0 = std::max(O.x_pos, F.x_pos - 2);
        op.i1 = std::min(O.x_pos + O.n_x, F.x_pos + F.n_x + 2);
        op.j0 = std::max(O.p_pos, F.p_pos - 2);
        op.j1 = std::min(O.p_pos + O.n_p, F.p_pos + F.n_p + 2);
        op.x2 = F.x_pos;
        op.p2 = F.p_pos;
        op.mask_off = moff[F.id];
        if (op.i0 >= op.i1 || op.j0 >= op.j1) return;
        need(bounds(F, op.i0 - F.x_pos, op.j0 - F.p_pos) && bounds(F, op.i1 - 1 - F.x_pos, op.j1 - 1 - F.p_pos));
        need(bounds(O, op.i0 - O.x_pos, op.j0 - O.p_pos) && bounds(O, op.i1 - 1 - O.x_pos, op.j1 - 1 - O.p_pos));
        ops.push_back(op);
    };
    auto run_ops = [&](const std::vector<XferOp> &ops) {
        if (ops.empty()) return;
        DevBuf d = upload(ops, eng->stream);
        launch_xfer(dd.p, d.as<XferOp>(), (int)ops.size(), dmask.as<uint8_t>(), precision, eng->stream);
        eng->sync();
    };
    for (size_t sp = 0; sp < old.size(); sp++) {
        auto &nl = rects[sp];
        auto &ol = old[sp];
        // Level::GetDataFromCoarserLevel / GetDataFromSameLevel (Level.cpp:127-141): the
        // argument level's patches call into this level's patches
        for (int i = 0; i + 1 < L; i++) {
            std::vector<XferOp> a, b;
            for (auto &C : ol[i + 1])
                for (auto &F : nl[i]) interp_op(a, kXferInterp, *C, old_id(C.get()), *F, F->id);
            run_ops(a);
            for (auto &O : ol[i])
                for (auto &F : nl[i]) copy_op(b, *O, old_id(O.get()), *F, F->id);
            run_ops(b);
        }
        if (L > 1) {
            std::vector<XferOp> b;
            for (auto &O : ol[L - 1])
                for (auto &F : nl[L - 1]) copy_op(b, *O, old_id(O.get()), *F, F->id);
            run_ops(b);
        }
        for (int i = L - 1; i > 0; i--) {  // Level::GetDataFromCoarseNewLevel (Level.cpp:143-149)
            std::vector<XferOp> c;
            for (auto &C : nl[i])
                for (auto &F : nl[i - 1]) interp_op(c, kXferInterpMissing, *C, C->id, *F, F->id);
            run_ops(c);
        }
    }
}

// Run-local descriptor table in flat order (the ids of the op lists).
DevBuf Run::flat_descs() {
    std::vector<PatchT<double>> descs;
    for (Rect *R : flat) descs.push_back(R->desc);
    return upload(descs, eng->stream);
}

// Mesh::PushData(val) (Mesh.cpp:91-106) for this run alone.
void Run::push_data(int slot) {
    DevBuf dd = flat_descs();
    DevBuf dops = upload(ghost_ops, eng->stream);
    for (size_t b = 0; b + 1 < ghost_b.ptr.size(); b++)
        launch_ghost(dd.p, dops.as<GhostOp>() + ghost_b.ptr[b], ghost_b.ptr[b + 1] - ghost_b.ptr[b], slot, precision,
                     eng->stream);
    eng->sync();
}

// FCTTimeStep sub-step 3 (Rectangle.cpp:1614-1621) over every patch: f[to] = f[from].
void Run::copy_slot(int from, int to) {
    for (Rect *R : flat) {
        const double *src = from == 0 ? R->desc.f0 : (from == 1 ? R->desc.f1 : R->desc.f2);
        double *dst = to == 0 ? R->desc.f0 : (to == 1 ? R->desc.f1 : R->desc.f2);
        VX_CUDA(cudaMemcpyAsync(dst, src, R->plane_bytes(), cudaMemcpyDeviceToDevice, eng->stream));
    }
    eng->sync();
}

}  // namespace vx
